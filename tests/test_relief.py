"""The relief / colour sampling and shadow-march restatement
(oracle/relief_ref.py) against the reference's own render.wgsl functions
(tests/golden/relief_samples.npz, written by their mechanical translation in
FP64)."""
from pathlib import Path

import numpy as np

import relief_ref as rr

FIX = Path(__file__).resolve().parent / "golden" / "relief_samples.npz"


def load():
    d = np.load(FIX)
    R = rr.Relief(int(d["w"]), int(d["h"]), float(d["width_m"]), float(d["height_m"]), d["h_plane"], d["m_plane"],
                  d["color_f16"].view(np.float16).astype(np.float64))
    return d, R


def test_restatement_equals_the_reference_functions():
    d, R = load()
    got, want = R.sample(d["points"]), d["out"]
    scale = np.maximum(np.abs(want).max(0), 1e-30)
    assert (np.abs(got - want).max(0) / scale).max() <= 1e-12


def test_fixture_covers_the_edge_blend_and_the_outside():
    d, R = load()
    pts = d["points"].astype(np.float64)
    px, py = pts[:, 0], pts[:, 1]
    i, j, tx, ty = R._grid(px, py)
    hw = np.stack([R.wet_at(i, j), R.wet_at(i + 1, j), R.wet_at(i, j + 1), R.wet_at(i + 1, j + 1)])
    hmax, hmin = hw.max(0), hw.min(0)
    with np.errstate(divide="ignore", invalid="ignore"):
        edge = R.smoothstep(rr.f(0.3), rr.f(0.6), 1.0 - hmin / hmax)
    sharpened = (hmax > rr.f(1e-6)) & (edge > 0)
    assert sharpened.sum() > 200
    assert R.outside(px, py).sum() > 50
    assert (d["out"][R.outside(px, py), 0] == 0).all()  # no relief outside the canvas


def test_shadow_restatement_equals_the_reference_march():
    d, R = load()
    for li, want in zip(d["shadow_lights"], d["shadow_out"]):
        got = R.shadow(d["points"], d["shadow_z0"], li, d["shadow_top"])
        assert np.abs(got[:, 0] - want[:, 0]).max() <= 1e-12 * max(np.abs(want[:, 0]).max(), 1e-30)
        assert np.abs(got[:, 1] - want[:, 1]).max() <= 1e-12


def test_shadow_fixture_has_shadowed_points():
    d, _ = load()
    shadowed = [(o[:, 1] < 1).sum() for o in d["shadow_out"]]
    assert sum(shadowed) > 50 and max(shadowed) > 40
    assert (d["shadow_out"][:, :, 1] >= 0).all() and (d["shadow_out"][:, :, 1] <= 1).all()


def test_shadow_restatement_at_other_tops():
    """The march's early stop (the ray above cam.canvas.w) against the
    translated shader itself, where oracle/_ref was built (next to a
    reference checkout); skipped elsewhere."""
    import ctypes as C
    lib = Path(__file__).resolve().parents[1] / "oracle" / "_ref" / "librenderref.so"
    if not lib.exists():
        import pytest
        pytest.skip("oracle/_ref/librenderref.so not built")
    d, R = load()
    L = C.CDLL(str(lib))
    fp = C.POINTER(C.c_float)
    dp = C.POINTER(C.c_double)
    L.wgrr_set.argtypes = [C.c_uint32, C.c_uint32, C.c_float, C.c_float, C.c_float, fp, fp, fp]
    L.wgrr_set_top.argtypes = [C.c_float]
    L.wgrr_shadow.argtypes = [dp, C.c_uint32, dp, dp]
    w, h = int(d["w"]), int(d["h"])
    hp = np.ascontiguousarray(d["h_plane"], np.float32)
    mp = np.ascontiguousarray(d["m_plane"], np.float32)
    col = np.ascontiguousarray(d["color_f16"].view(np.float16).astype(np.float32))
    dx = np.float32(d["width_m"]) / np.float32(w)
    L.wgrr_set(w, h, float(d["width_m"]), float(d["height_m"]), float(dx), hp.ctypes.data_as(fp),
               mp.ctypes.data_as(fp), col.ctypes.data_as(fp))
    pts = np.zeros((len(d["points"]), 3))
    pts[:, :2] = d["points"]
    pts[:, 2] = d["shadow_z0"]
    light = np.ascontiguousarray(d["shadow_lights"][2], np.float64)
    for top in (np.float32(float(np.max(hp + mp)) * 0.5), np.float32(float(np.max(hp + mp)) + 2e-4)):
        L.wgrr_set_top(float(top))
        want = np.zeros((len(pts), 2))
        L.wgrr_shadow(np.ascontiguousarray(pts).ctypes.data_as(dp), len(pts), light.ctypes.data_as(dp),
                      want.ctypes.data_as(dp))
        got = R.shadow(d["points"], d["shadow_z0"], light, top)
        assert np.abs(got[:, 1] - want[:, 1]).max() <= 1e-12
