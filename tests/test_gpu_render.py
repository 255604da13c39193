"""The renderer's fragment shader over the film (cf_render_lit) against the
reference's own fragment shader (GPU).

tests/golden/render_lit.npz holds, for a 40 x 32 film (h, m, the rgba16f
colour, the rgba16f detail texels with brush, knife and roller strokes, the
tile flags) and four cameras (top-down orthographic, oblique perspective, a
thin lens, the beauty mode), the rgba of every pixel of a 48 x 36 target as
shaders/render.wgsl's fs computes it, translated by oracle/wgsl_ref and
evaluated in f32 with one rounding per operation (tests/golden/
make_render_lit.py).  The kernel follows the same f32 arithmetic without
contraction, so pixels differ only where the last bits of a transcendental
function (exp, pow, sin, cos, tanh, atan2) differ between CUDA and the host
library: the bounds below allow that, and a wrong term anywhere in the
shading moves far more pixels by far more.
"""
from pathlib import Path

import numpy as np
import pytest

from canvaz_film import capi

pytestmark = pytest.mark.gpu

FIX = Path(__file__).resolve().parent / "golden" / "render_lit.npz"


@pytest.fixture(scope="module")
def built():
    import __graft_entry__ as g
    g.build()
    return True


def film_from_fixture(d):
    from canvaz_film.film import Film
    w, h = int(d["w"]), int(d["h"])
    st = capi.Settings.default(width_m=float(d["width_m"]), height_m=float(d["height_m"]))
    f = Film(st, w, h, capi.CF_PREC_FP32)
    f.set_plane("h", d["h_plane"])
    f.set_plane("m", d["m_plane"])
    f.set_plane("color", d["color_f16"].view(np.float16).astype(np.float64))
    f.set_plane("detail", d["detail_f16"].view(np.float16).astype(np.float64))
    f.set_plane("tile_flags", d["tile_flags"])
    return f


def render(f, cam_words, iw, ih):
    import torch
    out = torch.zeros((ih * iw * 4,), dtype=torch.float32, device="cuda")
    u8 = torch.zeros((ih * iw,), dtype=torch.int32, device="cuda")
    f.render_lit(cam_words, iw, ih, out.data_ptr(), u8.data_ptr())
    torch.cuda.synchronize()
    rgba = out.cpu().numpy().reshape(-1, 4).astype(np.float64)
    b = u8.cpu().numpy().view(np.uint8).reshape(-1, 4)
    return rgba, b


def test_render_lit_matches_the_reference_fragment(built):
    d = np.load(FIX)
    f = film_from_fixture(d)
    iw, ih = int(d["img_w"]), int(d["img_h"])
    for k, kind in enumerate(d["kinds"]):
        rgba, b = render(f, d["cams"][k], iw, ih)
        want = d["out"][k]
        err = np.abs(rgba - want).max(1)
        off = err > 2e-3
        print("%-6s max |d| %.3e, median %.3e, pixels off by more than 2e-3: %d of %d"
              % (kind, err.max(), np.median(err), int(off.sum()), len(err)))
        assert np.isfinite(rgba).all()
        assert np.median(err) < 1e-5, kind
        assert off.mean() <= 0.02, kind
        # RGBA8: the floats rounded to the nearest 8-bit step, in f32 as the kernel rounds
        r32 = rgba.astype(np.float32)
        q = np.clip(np.floor(r32 * np.float32(255.0) + np.float32(0.5)), 0, 255).astype(np.uint8)
        assert np.array_equal(b, q), kind
    f.close()


def test_render_lit_rejects_bad_arguments(built):
    import torch
    d = np.load(FIX)
    f = film_from_fixture(d)
    out = torch.zeros((64,), dtype=torch.float32, device="cuda")
    cam = capi.RenderCam.from_words(d["cams"][0])
    cam.size[0] = cam.size[0] + 1  # not the film's size
    with pytest.raises(capi.FilmError):
        f.render_lit(cam, 4, 4, out.data_ptr())
    with pytest.raises(capi.FilmError):  # no output
        f.render_lit(d["cams"][0], 4, 4)
    with pytest.raises(capi.FilmError):  # misaligned float output
        f.render_lit(d["cams"][0], 2, 2, out.data_ptr() + 4)
    f.close()
