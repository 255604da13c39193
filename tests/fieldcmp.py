"""Per-field comparison of a film's state against a reference state (shared
by the config-size GPU tests and tests/report_precision.py).

Fields: h, the flow h - h0 over the run, m, strata_h, per-cell pigment volume
(sum over strata of thickness x slot, slots 0-12), mu, tau_y and the linear
RGB colour.  For each: max |error|, RMS error and relative L2
(||error|| / ||reference||)."""
import numpy as np

import parity


def fields_gpu(f, h0=None):
    s = f.read_state()
    out = {"h": s["h"], "m": s["m"], "strata_h": s["strata_h"],
           "pigment volume": parity.pig_volume(s["strata_h"], s["strata_pig"]),
           "mu": f.plane("mu"), "tau_y": f.plane("tau"), "colour rgb": f.color()[:, :3]}
    if h0 is not None:
        out["flow h - h0"] = np.asarray(s["h"], np.float64) - np.asarray(h0, np.float64)
    return out


def fields_oracle(o, h0=None):
    rheo = o.buf("rheo").reshape(o.n, -1)
    h = o.buf("h")
    out = {"h": h, "m": o.buf("m"), "strata_h": o.buf("strata_h"),
           "pigment volume": parity.pig_volume(o.buf("strata_h"), o.buf("strata_pig")),
           "mu": rheo[:, 0], "tau_y": rheo[:, 1], "colour rgb": o.buf("color").reshape(o.n, 4)[:, :3]}
    if h0 is not None:
        out["flow h - h0"] = np.asarray(h, np.float64) - np.asarray(h0, np.float64)
    return out


def compare(got, want):
    """{field: (max abs, RMS, rel L2)} over the fields both sides have."""
    out = {}
    for k in want:
        if k not in got:
            continue
        a, b = np.asarray(got[k], np.float64).ravel(), np.asarray(want[k], np.float64).ravel()
        d = a - b
        out[k] = (float(np.abs(d).max()), float(np.sqrt(np.mean(d * d))), parity.rel_l2(a, b))
    return out


def table(rows, title):
    lines = ["", "### %s" % title, "", "| field | max abs error | RMS error | rel L2 |", "|---|---|---|---|"]
    for name, (mx, rms, rl2) in rows.items():
        lines.append("| %s | %.3e | %.3e | %.3e |" % (name, mx, rms, rl2))
    text = "\n".join(lines)
    print(text)
    return text
