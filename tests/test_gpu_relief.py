"""The render pass's reading of the film on the GPU (cf_sample_relief,
cf_relief_shadow, cf_render_relief) against the reference's render.wgsl
functions (tests/golden/relief_samples.npz, FP64)."""
from pathlib import Path

import numpy as np
import pytest

from canvaz_film import capi

pytestmark = pytest.mark.gpu

FIX = Path(__file__).resolve().parent / "golden" / "relief_samples.npz"


@pytest.fixture(scope="module")
def built():
    import __graft_entry__ as g
    g.build()
    return True


def fixture_film():
    from canvaz_film.film import Film
    d = np.load(FIX)
    w, h = int(d["w"]), int(d["h"])
    s = capi.Settings.default(width_m=float(d["width_m"]), height_m=float(d["height_m"]))
    f = Film(s, w, h, capi.CF_PREC_FP32)
    n = w * h
    f.write_state({"h": d["h_plane"], "m": d["m_plane"], "rheo": np.tile([1.0, 0.0], (n, 1)).astype(np.float32),
                   "strata_h": np.zeros((n, 4), np.float32), "strata_cure": np.zeros((n, 4), np.float32),
                   "strata_pig": np.zeros((n, 64), np.float32), "sub_refl": np.full((n, 16), 0.5, np.float32),
                   "lay": np.zeros(n, np.uint32)})
    f.set_plane("color", d["color_f16"].view(np.float16).reshape(-1))  # the colour plane the renderer reads
    return d, f


def test_samples_match_the_reference(built):
    import torch
    d, f = fixture_film()
    pts = torch.from_numpy(np.ascontiguousarray(d["points"])).cuda()
    out = torch.empty((len(pts), 8), dtype=torch.float32, device="cuda")
    f.sample_relief(pts.data_ptr(), len(pts), out.data_ptr())
    torch.cuda.synchronize()
    got, want = out.cpu().numpy().astype(np.float64), d["out"]
    scale = np.maximum(np.abs(want).max(0), 1e-30)
    err = np.abs(got - want) / scale
    # f32 against FP64: heights and colours to 1e-5 of their range; the
    # colour sharpening's smoothsteps may flip a few points at their edges
    assert (err[:, [0, 7]] > 1e-5).mean() == 0, err[:, [0, 7]].max(0)
    assert (err[:, 3:7] > 1e-4).mean() <= 2e-3, err[:, 3:7].max(0)
    assert (err[:, 1:3] > 1e-3).mean() <= 2e-3, err[:, 1:3].max(0)


def test_render_is_the_shaded_samples(built):
    import torch
    d, f = fixture_film()
    W, H, x0, y0, pm = 96, 64, -1e-3, -2e-3, 0.45e-3
    img = torch.zeros(W * H * 4, dtype=torch.uint8, device="cuda")
    light, amb = (0.3, 0.5, 0.8), 0.35
    f.render_relief(img.data_ptr(), x0, y0, pm, W, H, light=light, ambient=amb)
    yy, xx = np.mgrid[0:H, 0:W]
    pts = np.stack([x0 + (xx.ravel() + 0.5) * pm, y0 + (yy.ravel() + 0.5) * pm], 1).astype(np.float32)
    tp = torch.from_numpy(pts).cuda()
    out = torch.empty((len(pts), 8), dtype=torch.float32, device="cuda")
    f.sample_relief(tp.data_ptr(), len(pts), out.data_ptr())
    torch.cuda.synchronize()
    s = out.cpu().numpy().astype(np.float64)
    l = np.array(light) / np.linalg.norm(light)
    nx, ny = -s[:, 1], -s[:, 2]
    diff = np.maximum((nx * l[0] + ny * l[1] + l[2]) / np.sqrt(nx * nx + ny * ny + 1), 0)
    k = amb + (1 - amb) * diff
    lin = np.clip(s[:, 3:6] * k[:, None], 0, 1)
    srgb = np.where(lin <= 0.0031308, 12.92 * lin, 1.055 * lin ** (1 / 2.4) - 0.055)
    want = np.round(np.clip(srgb, 0, 1) * 255)
    got = img.cpu().numpy().reshape(-1, 4)
    assert np.abs(got[:, :3].astype(np.int32) - want).max() <= 1
    assert (got[:, 3] == 255).all()


def test_errors(built):
    d, f = fixture_film()
    L = capi.load_library()
    assert L.cf_sample_relief(f.p, None, 3, None, None) == capi.CF_ERR_INVALID_ARG
    assert L.cf_sample_relief(f.p, None, 0, None, None) == capi.CF_OK
    v = capi.ReliefView(x0=0, y0=0, pixel_m=0.0, width=4, height=4, ambient=0.3)
    import ctypes as C
    assert L.cf_render_relief(f.p, C.byref(v), C.c_void_p(16), None) == capi.CF_ERR_INVALID_ARG


def test_shadow_march_matches_the_reference(built):
    """cf_relief_shadow against the reference's shadow_at (FP64), for a high,
    a low and a grazing light; and no shadow for a light at or below the
    shader's 0.05 cut."""
    import torch
    d, f = fixture_film()
    n = len(d["points"])
    p3 = np.zeros((n, 3), np.float32)
    p3[:, :2] = d["points"]
    p3[:, 2] = d["shadow_z0"]
    pts = torch.from_numpy(p3).cuda()
    out = torch.empty((n, 2), dtype=torch.float32, device="cuda")
    top = float(d["shadow_top"])
    for li, want in zip(d["shadow_lights"], d["shadow_out"]):
        f.relief_shadow(pts.data_ptr(), n, [float(v) for v in li], top, out.data_ptr())
        torch.cuda.synchronize()
        got = out.cpu().numpy().astype(np.float64)
        # f32 against FP64: the height to 1e-5 of its range; the shadow factor
        # (a min of clamped ratios) to 1e-4, a floor() at a sample's cell
        # boundary may move a few points further
        assert np.abs(got[:, 0] - want[:, 0]).max() <= 1e-5 * np.abs(want[:, 0]).max()
        err = np.abs(got[:, 1] - want[:, 1])
        assert (err > 1e-4).mean() <= 1e-3, err.max()
        assert ((got[:, 1] < 1) == (want[:, 1] < 1)).mean() >= 0.999
    f.relief_shadow(pts.data_ptr(), n, [0.99, 0.0, 0.05], top, out.data_ptr())
    torch.cuda.synchronize()
    assert (out[:, 1] == 1).all()


def test_misaligned_buffers_are_refused(built):
    """Buffers valid byte by byte but not aligned to the vectors the kernels
    use return CF_ERR_INVALID_ARG before any launch (nothing is written)."""
    import torch
    from canvaz_film.capi import FilmError
    d, f = fixture_film()
    buf = torch.zeros(4096, dtype=torch.uint8, device="cuda")
    base = buf.data_ptr()
    assert base % 256 == 0
    with pytest.raises(FilmError):
        f.sample_relief(base + 4, 8, base + 1024)      # points not 8-byte aligned
    with pytest.raises(FilmError):
        f.sample_relief(base, 8, base + 1026)          # out not 4-byte aligned
    with pytest.raises(FilmError):
        f.relief_shadow(base + 2, 8, (0.3, 0.5, 0.8), 1e-3, base + 1024)  # points not 4-byte aligned
    with pytest.raises(FilmError):
        f.relief_shadow(base, 8, (0.3, 0.5, 0.8), 1e-3, base + 1028)      # out not 8-byte aligned
    with pytest.raises(FilmError):
        f.render_relief(base + 2, 0.0, 0.0, 1e-3, 8, 8)                    # rgba8 not 4-byte aligned
    torch.cuda.synchronize()
    assert torch.count_nonzero(buf).item() == 0
    f.sample_relief(base, 8, base + 1024)  # aligned: runs
    torch.cuda.synchronize()
