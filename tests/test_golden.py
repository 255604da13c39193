"""The oracle against the golden fixtures.

tests/golden/*.npz hold seeded inputs and the final planes of the reference's
own WGSL (mechanically translated to C++ and run in FP64 by
tests/golden/make_golden.py).  The FP64 oracle must reproduce them; the
comparison is exact up to a relative 1e-12 (libm differences between hosts)."""
import json
from pathlib import Path

import numpy as np
import pytest

import deposit_ref as dr
import pyoracle as po

# the frame fixtures (relief_samples.npz, resolve_samples.npz and render_lit.npz hold render and
# display samples: tests/test_relief.py, tests/test_resolve_fixture.py)
GOLDEN = sorted(p for p in (Path(__file__).resolve().parent / "golden").glob("*.npz") if p.stem not in ("relief_samples", "resolve_samples", "render_lit"))
FIELDS = ["h", "m", "strata_h", "strata_pig", "strata_cure", "sub_refl", "delta", "fnorm", "color", "acc",
          "tile_flags", "pres", "flux", "alpha", "tmp", "acc_s", "alpha_s"]


def replay(d, bits=64):
    w, h = int(d["w"]), int(d["h"])
    st = po.make_settings(json.loads(str(d["settings"])))
    o = po.Oracle(w, h, st, 0, bits)
    o.set_tables(d["pigtab"], d["cmf"])
    planes = {k[3:]: d[k] for k in d.files if k.startswith("in_")}
    o.write_state(planes)
    for f, ((fdt, n), praw) in enumerate(zip(d["schedule"], d["params"])):
        if "deposits_%d" % f in d.files:  # upload_deposits before choose_substeps (src/main.rs:1881-1892)
            o.upload_deposits(d["deposits_%d" % f].reshape(-1).view(dr.DEPOSIT_DTYPE))
        o.update_params(float(fdt), int(n))
        assert bytes(o.params()) == praw.tobytes(), "update_params drifted from the fixture"
        o.encode_frame(int(n))
    return o


@pytest.mark.parametrize("path", GOLDEN, ids=[p.stem for p in GOLDEN])
def test_oracle_matches_reference_fixture(path):
    d = np.load(path)
    o = replay(d)
    for f in FIELDS:
        got, want = o.buf(f), d["out_" + f]
        if f in ("delta", "tile_flags"):
            assert np.array_equal(got.astype(np.uint64), want.astype(np.uint64)), f
            continue
        scale = max(float(np.abs(want).max()), 1e-30)
        err = float(np.abs(got - want).max()) / scale
        assert err <= 1e-12, (f, err)
    if "out_lay" in d.files:
        assert np.array_equal(o.buf("lay").astype(np.uint64), d["out_lay"].astype(np.uint64))
    rheo = o.buf("rheo").reshape(-1, 3)[:, :2].reshape(-1)
    want = d["out_rheo"].reshape(-1, 3)[:, :2].reshape(-1)
    assert np.allclose(rheo, want, rtol=1e-12, atol=0)


def test_fixtures_exist():
    assert len(GOLDEN) >= 8
    assert any("deposits_0" in np.load(p).files for p in GOLDEN)


@pytest.mark.parametrize("path", GOLDEN[:3], ids=[p.stem for p in GOLDEN[:3]])
def test_fp32_mirror_tracks_fp64(path):
    """The FP32 mirror (the CPU baseline) stays close to the FP64 reference."""
    d = np.load(path)
    o = replay(d, bits=32)
    h, want = o.buf("h"), d["out_h"]
    # FP32 leaves ~1e-10 m residues where FP64 drains a committed cell to 0,
    # so the bound is absolute, scaled by the thickest film.
    err = float(np.abs(h - want).max())
    assert err <= 1e-3 * float(np.abs(want).max()) + 1e-9, err
