"""The display epilogue (cf_resolve) against the CPU restatement of
shaders/resolve.wgsl (GPU): AgX and ACES, with and without bloom, sharpen,
vignette and grain, on a film's colour plane.  8-bit outputs agree to one
step (the CUDA side runs in f32, the restatement in f64)."""
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
