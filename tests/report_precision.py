"""Per-field error report of the CUDA film against the FP64 oracle (GPU).

Prints a markdown report (commit it as a profile summary):
  1. the 512 x 512 FP32 blob field (K, S over 8 bands), fixed dt 1e-3 s,
     200 steps: the CUDA film and the oracle's own FP32 mirror, each against
     the FP64 oracle;
  2. the blob field over a cured ground at 512 x 512 (the 4096 x 4096
     field's generator at 1/8 side): FP32 and BF16 storage against FP64;
  3. the 4096 x 4096 field, 1000 steps: BF16 storage against the
     FP32-everywhere film (both on the GPU);
  4. the 2048 x 2048 tilted drip field, 1000 adaptive steps: FP64 mass drift.
Per field: max |error|, RMS error and relative L2 (||error|| / ||reference||).

Usage: python tests/report_precision.py [--steps0 200] [--steps2 1000]
"""
import argparse
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
for p in (ROOT, ROOT / "paint-sim-3d_gb300", ROOT / "oracle", ROOT / "tests"):
    sys.path.insert(0, str(p))

import parity  # noqa: E402
import pyoracle as po  # noqa: E402
from canvaz_film import capi, synth  # noqa: E402


def film_for(cv, prec):
    from canvaz_film.film import Film
    f = Film(capi.Settings.default(**cv.settings), cv.w, cv.h, prec)
    f.set_tables(cv.pigtab, cv.cmf)
    f.write_state(cv.planes, pig_format=capi.CF_PIG_F32)
    return f


def fields_gpu(f):
    s = f.read_state()
    return {"h": s["h"], "m": s["m"], "strata_h": s["strata_h"],
            "pigment volume": parity.pig_volume(s["strata_h"], s["strata_pig"]),
            "mu": s["rheo"][:, 0], "tau_y": s["rheo"][:, 1], "colour rgb": f.color()[:, :3]}


def fields_oracle(o):
    rheo = o.buf("rheo").reshape(o.n, -1)
    return {"h": o.buf("h"), "m": o.buf("m"), "strata_h": o.buf("strata_h"),
            "pigment volume": parity.pig_volume(o.buf("strata_h"), o.buf("strata_pig")),
            "mu": rheo[:, 0], "tau_y": rheo[:, 1], "colour rgb": o.buf("color").reshape(o.n, 4)[:, :3]}


def table(rows, title):
    print("\n### %s\n" % title)
    print("| field | max abs error | RMS error | rel L2 |")
    print("|---|---|---|---|")
    for name, (mx, rms, rl2) in rows:
        print("| %s | %.3e | %.3e | %.3e |" % (name, mx, rms, rl2))


def compare(got, want):
    out = []
    for k in want:
        a, b = np.asarray(got[k], np.float64).ravel(), np.asarray(want[k], np.float64).ravel()
        d = a - b
        out.append((k, (float(np.abs(d).max()), float(np.sqrt(np.mean(d * d))), parity.rel_l2(a, b))))
    return out


def run_oracle(cv, steps, bits):
    o = po.Oracle(cv.w, cv.h, po.make_settings(cv.settings), capi.CF_PIG_F32, bits)
    o.set_tables(cv.pigtab, cv.cmf)
    o.write_state(cv.planes)
    o.update_params(1e-3, 1)
    for _ in range(steps):
        o.encode_frame(1)
    return o


def run_gpu(cv, prec, steps):
    f = film_for(cv, prec)
    f.update_params(1e-3, 1)
    for _ in range(steps):
        f.encode_frame(1)
    f.sync()
    return f


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps0", type=int, default=200)
    ap.add_argument("--steps2", type=int, default=1000)
    args = ap.parse_args()
    import __graft_entry__ as g
    g.build()
    t0 = time.time()
    print("# Per-field error of the CUDA film against the FP64 oracle\n")
    print("Command: `python tests/report_precision.py --steps0 %d --steps2 %d` (GB300)." % (args.steps0, args.steps2))
    print("Fixed dt 1e-3 s, one substep per step, every tile active.")

    cv = synth.config(0, 0)
    cv.settings["all_active"] = 1
    ref = fields_oracle(run_oracle(cv, args.steps0, 64))
    table(compare(fields_gpu(run_gpu(cv, capi.CF_PREC_FP32, args.steps0)), ref),
          "512x512 blob field, %d steps: CUDA FP32 vs FP64 oracle" % args.steps0)
    table(compare(fields_oracle(run_oracle(cv, args.steps0, 32)), ref),
          "512x512 blob field, %d steps: the oracle's FP32 CPU mirror vs FP64 oracle (for scale)" % args.steps0)

    cv = synth.config(2, 0, scale=8)
    cv.settings["all_active"] = 1
    ref = fields_oracle(run_oracle(cv, args.steps0, 64))
    for prec, name in ((capi.CF_PREC_FP32, "FP32"), (capi.CF_PREC_BF16, "BF16 pigments + rheology")):
        table(compare(fields_gpu(run_gpu(cv, prec, args.steps0)), ref),
              "512x512 cured-ground blob field (4096^2 generator at 1/8 side), %d steps: CUDA %s vs FP64 oracle"
              % (args.steps0, name))

    cv = synth.config(2, 0)
    cv.settings["all_active"] = 1
    a = fields_gpu(run_gpu(cv, capi.CF_PREC_FP32, args.steps2))
    b = fields_gpu(run_gpu(cv, capi.CF_PREC_BF16, args.steps2))
    table(compare(b, a), "4096x4096 cured-ground blob field, %d steps: CUDA BF16 vs CUDA FP32-everywhere" % args.steps2)

    cv = synth.config(1, 0)
    cv.settings["all_active"] = 1
    f = film_for(cv, capi.CF_PREC_FP32)
    s0 = f.stats()
    for _ in range(1000):
        f.step_adaptive(1.0 / 60.0)
    s1 = f.stats()
    m0, m1 = s0["wet_volume"] + s0["relief_volume"], s1["wet_volume"] + s1["relief_volume"]
    print("\n### 2048x2048 tilted drips, 1000 adaptive steps (FP32)\n")
    print("FP64 mass sum(h + m) dx^2: %.9e -> %.9e, relative drift %.3e; last dt %.3e s; non-finite cells %d"
          % (m0, m1, abs(m1 - m0) / m0, s1["last_dt"], s1["nan_cells"]))
    print("\n(report took %.0f s)" % (time.time() - t0))


if __name__ == "__main__":
    main()
