"""The committed colour tables (canvaz_film/data/reference_tables.npz).

 - The reference's own colour test, canvas_reflectance_reproduces_colour
   (src/color/mod.rs:377-393), on the committed CMF x D65 table: six canvas
   colours go to a 16-band reflectance (reflectance_of), back to XYZ through
   the table and to sRGB, and land within 0.03 of where they started.  This
   pins the table and the XYZ -> sRGB matrix the shade uses.
 - The pigment table's K and S rows are K = (1 - r)^2 / (2 r) * scatter,
   S = scatter (pigment_table, src/color/mod.rs:243-258): so each band's
   Kubelka-Munk infinite-layer reflectance 1 + K/S - sqrt((K/S)^2 + 2 K/S)
   gives back the pigment's clamped reflectance r in [0.01, 0.98].
 - Where the reference checkout is present, the tables are derived again
   from its sources and must equal the committed ones bit for bit.
"""
import os
import sys
from pathlib import Path

import numpy as np
import pytest

import color_ref
from canvaz_film import synth  # noqa: F401  (package path)

ROOT = Path(__file__).resolve().parents[1]
NPZ = ROOT / "paint-sim-3d_gb300" / "canvaz_film" / "data" / "reference_tables.npz"
CANVAS_COLOURS = [[0.94, 0.93, 0.90], [0.74, 0.56, 0.33], [0.64, 0.37, 0.26], [0.50, 0.56, 0.62],
                  [0.56, 0.56, 0.55], [0.30, 0.45, 0.25]]


def tables():
    d = np.load(NPZ)
    return d["cmf"].astype(np.float32), d["pigtab"].astype(np.float32)


def test_canvas_reflectance_reproduces_colour():
    cmf, _ = tables()
    assert cmf.shape == (48,)
    for rgb in CANVAS_COLOURS:
        refl = color_ref.reflectance_of(rgb, cmf)
        xyz = [np.float32(0)] * 3
        for b in range(16):
            for i in range(3):
                xyz[i] = np.float32(xyz[i] + np.float32(refl[b] * cmf[b * 3 + i]))
        got = color_ref.xyz_to_srgb(xyz)
        assert np.all(np.abs(got - np.float32(rgb)) < 0.03), (rgb, got)


def test_cmf_table_is_normalised_to_unit_y():
    cmf, _ = tables()
    # cmf_table divides every entry by the sum of the Y column
    assert abs(float(cmf.reshape(16, 3)[:, 1].astype(np.float64).sum()) - 1.0) < 1e-6


def test_pigment_rows_give_back_their_reflectance():
    _, pig = tables()
    t = pig.reshape(12, 40).astype(np.float64)
    K, S = t[:, 0:16], t[:, 16:32]
    assert (S > 0).all() and (K > 0).all()
    assert np.all(S == S[:, :1])  # scatter is one value per pigment
    ks = K / S
    r_inf = 1.0 + ks - np.sqrt(ks * ks + 2.0 * ks)
    assert r_inf.min() >= 0.01 - 1e-6 and r_inf.max() <= 0.98 + 1e-6
    # K / S = (1 - r)^2 / (2 r) inverts exactly to r (f32 rounding of K only)
    r = r_inf
    np.testing.assert_allclose((1 - r) ** 2 / (2 * r), ks, rtol=1e-5)
    # viscosity, yield stress and tint columns are positive / non-negative
    assert (t[:, 32] > 0).all() and (t[:, 33] >= 0).all() and (t[:, 34] > 0).all()


def test_tables_rederive_from_the_reference_sources():
    sys.path.insert(0, str(ROOT / "oracle" / "wgsl_ref"))
    import build_ref
    ref = build_ref.reference_root()
    if not (ref / "src" / "color" / "mod.rs").exists():
        pytest.skip("the reference checkout is not present here")
    sys.path.insert(0, str(NPZ.parent))
    import make_tables
    cmf, pig = tables()
    np.testing.assert_array_equal(make_tables.cmf_table(ref), cmf)
    p2, _ = make_tables.pigment_table(ref)
    np.testing.assert_array_equal(p2, pig)
