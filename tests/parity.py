"""Parity metrics shared by the CPU and GPU tests.

An FP32 run of the step (the CUDA kernels, or the oracle's FP32 mirror) is
compared with the FP64 reference through quantities that do not depend on the
discrete branches of the strata stack (merge / push thresholds flip under
rounding and reorder a stack without changing its contents):
  - the film height h: relative L2 error (the benchmark spec's bound is 1e-5) and
    the largest absolute error;
  - per-cell pigment volume V[c, q] = sum_k strata_h[c, k] * pig[c, k, q]
    for the 12 pigments and the thinner, relative L2;
  - colour: the fraction of cells whose linear RGB differs by more than 1e-2;
  - mass: sum(h) + sum(m) over the canvas, relative.
"""
import numpy as np

H_REL_L2 = 1e-5        # height, relative L2 against FP64
PIGVOL_REL_L2 = 2e-3   # per-cell pigment volume, relative L2
COLOR_BAD_FRAC = 0.01  # cells with |drgb| > 1e-2
MASS_REL = 1e-6


def pig_volume(strata_h, strata_pig):
    th = np.asarray(strata_h, np.float64).reshape(-1, 4)
    pg = np.asarray(strata_pig, np.float64).reshape(-1, 4, 16)[:, :, :13]
    return np.einsum("ck,ckq->cq", th, pg)


def rel_l2(a, b):
    a, b = np.asarray(a, np.float64).ravel(), np.asarray(b, np.float64).ravel()
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def metrics(got, want):
    """got/want: dicts with h, m, strata_h, strata_pig, color (oracle layout)."""
    out = {}
    h, hw = np.asarray(got["h"], np.float64), np.asarray(want["h"], np.float64)
    out["h_rel_l2"] = rel_l2(h, hw)
    out["h_max_abs"] = float(np.abs(h - hw).max())
    out["h_scale"] = float(np.abs(hw).max())
    out["pigvol_rel_l2"] = rel_l2(pig_volume(got["strata_h"], got["strata_pig"]),
                                  pig_volume(want["strata_h"], want["strata_pig"]))
    c, cw = np.asarray(got["color"], np.float64).reshape(-1, 4), np.asarray(want["color"], np.float64).reshape(-1, 4)
    out["color_bad_frac"] = float((np.abs(c[:, :3] - cw[:, :3]).max(axis=1) > 1e-2).mean())
    mg = h.sum() + np.asarray(got["m"], np.float64).sum()
    mw = hw.sum() + np.asarray(want["m"], np.float64).sum()
    out["mass_rel"] = float(abs(mg - mw) / max(abs(mw), 1e-300))
    return out


def check(m, h_rel=H_REL_L2):
    """Asserts the bounds; a nearly dry canvas (cure commits) uses the absolute
    height bound instead of the relative one."""
    if m["h_scale"] > 0 and m["h_max_abs"] > 1e-3 * m["h_scale"] + 1e-9:
        raise AssertionError("height max abs error %.3e (scale %.3e)" % (m["h_max_abs"], m["h_scale"]))
    wet_case = m["h_rel_l2"] < 1.0
    if wet_case:
        assert m["h_rel_l2"] <= h_rel, m
    assert m["pigvol_rel_l2"] <= PIGVOL_REL_L2, m
    assert m["color_bad_frac"] <= COLOR_BAD_FRAC, m
