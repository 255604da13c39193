"""The resolve restatement (oracle/resolve_ref.py) against the reference's
own display fragment shader (tests/golden/resolve_samples.npz: resolve.wgsl's
fs translated mechanically and evaluated in f32 by make_resolve.py), for AgX
and ACES with exposure, bloom, sharpen, vignette and grain.  8-bit outputs
(the surface's unorm8) agree to one step."""
from pathlib import Path

import numpy as np

import resolve_ref

FIX = Path(__file__).resolve().parent / "golden" / "resolve_samples.npz"


def fixture_cases():
    d = np.load(FIX)
    img = d["image_f16"].view(np.float16).astype(np.float64)
    for case, out in zip(d["cases"], d["out"]):
        scale, ev, bloom, grain, vig, sharpen, agx = (float(x) for x in case)
        kw = dict(scale=scale, exposure_ev=ev, bloom=bloom, grain=grain, vignette=vig, sharpen=sharpen)
        want8 = np.rint(np.clip(out[..., :3], 0.0, 1.0) * 255.0).astype(int)
        yield img, kw, agx >= 0.5, want8, out


def test_restatement_matches_the_translated_shader():
    for img, kw, agx, want8, out in fixture_cases():
        got = resolve_ref.resolve(img[..., :3], agx_on=agx, **kw)
        diff = np.abs(got[..., :3].astype(int) - want8)
        assert diff.max() <= 1, (kw, agx, diff.max())
        assert (diff > 0).mean() < 0.02, (kw, agx, (diff > 0).mean())
        assert np.all(out[..., 3] == 1.0)


def test_fixture_exercises_every_branch():
    d = np.load(FIX)
    cases = d["cases"]
    assert set(cases[:, 6]) == {0.0, 1.0}                 # AgX and ACES
    assert (cases[:, 2] > 0).any() and (cases[:, 3] > 0).any() and (cases[:, 5] > 0).any()
    img = d["image_f16"].view(np.float16).astype(np.float64)
    lum = img[..., :3] @ np.array([0.2126, 0.7152, 0.0722])
    assert (lum * cases[:, 0].max() > 1.6).any()          # the bloom threshold is crossed
