"""The display epilogue (cf_resolve) on the GPU: against the reference's own
fragment shader (tests/golden/resolve_samples.npz, resolve.wgsl's fs
translated mechanically and run in f32) on the fixture's HDR image, and
against the CPU restatement of shaders/resolve.wgsl on a shaded film's colour
plane: AgX and ACES, with and without bloom, sharpen, vignette and grain.
8-bit outputs agree to one step."""
import numpy as np
import pytest

import resolve_ref
from canvaz_film import synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def shaded_film():
    import __graft_entry__ as g
    g.build()
    from canvaz_film.film import Film
    import pyoracle as po
    cv = synth.blob_canvas(72, 56, 4, n_blobs=5, sigma=(3, 10))
    f = Film(po.make_settings(cv.settings), cv.w, cv.h)
    f.set_tables(cv.pigtab, cv.cmf)
    f.write_state(cv.planes)
    return f


CASES = [dict(agx=1), dict(agx=0, exposure_ev=1.0), dict(agx=1, bloom=0.8, scale=3.0),
         dict(agx=1, sharpen=0.6, vignette=0.4, grain=0.3), dict(agx=0, bloom=0.5, sharpen=0.3, scale=4.0)]


@pytest.mark.parametrize("params", CASES, ids=[str(i) for i in range(len(CASES))])
def test_resolve_matches_restatement(shaded_film, params):
    import torch
    f = shaded_film
    out = torch.zeros((f.h, f.w, 4), dtype=torch.uint8, device="cuda")
    f.resolve(out.data_ptr(), **params)
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    rgb = f.color()[:, :3].reshape(f.h, f.w, 3)
    kw = {k: v for k, v in params.items() if k != "agx"}
    want = resolve_ref.resolve(rgb, agx_on=bool(params.get("agx", 1)), **kw)
    diff = np.abs(got.astype(int) - want.astype(int))
    assert diff.max() <= 1, (diff.max(), np.argwhere(diff > 1)[:5])
    assert (diff > 0).mean() < 0.05


def test_resolve_matches_the_translated_shader(shaded_film):
    """cf_resolve of the fixture's image (set as a film's colour plane) against
    the reference shader's own outputs, every case of the fixture."""
    import torch
    from pathlib import Path
    from canvaz_film import capi
    from canvaz_film.film import Film
    d = np.load(Path(__file__).resolve().parent / "golden" / "resolve_samples.npz")
    w, h = int(d["w"]), int(d["h"])
    f = Film(capi.Settings.default(width_m=w * 1e-3, height_m=h * 1e-3), w, h, capi.CF_PREC_FP32)
    f.set_plane("color", d["image_f16"].view(np.float16).reshape(-1))
    out = torch.zeros((h, w, 4), dtype=torch.uint8, device="cuda")
    for case, ref in zip(d["cases"], d["out"]):
        scale, ev, bloom, grain, vig, sharpen, agx = (float(x) for x in case)
        f.resolve(out.data_ptr(), scale=scale, exposure_ev=ev, bloom=bloom, grain=grain, vignette=vig,
                  sharpen=sharpen, agx=int(agx >= 0.5))
        torch.cuda.synchronize()
        got = out.cpu().numpy().astype(int)
        want = np.rint(np.clip(ref[..., :3], 0.0, 1.0) * 255.0).astype(int)
        diff = np.abs(got[..., :3] - want)
        assert diff.max() <= 1, (case, diff.max(), np.argwhere(diff > 1)[:5])
        assert (diff > 0).mean() < 0.02, (case, (diff > 0).mean())
        assert (got[..., 3] == 255).all()
    f.close()
