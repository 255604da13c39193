"""The fused flow kernel (laplacian + plug + fluxes of one substep, one tile
per block, planes staged in shared memory) against the three separate
dispatches on the same state (GPU).

The frame runs the fused kernel; the per-dispatch parity tests check the
separate ones against the oracle.  Here both run from one state and must give
the same face fluxes and plug mobilities, to rounding: each value is the same
expression, but the two compiled copies may contract multiply-adds
differently.  Cases cover a tilted canvas (the plug window is evaluated), flat
ones (it is not), every storage precision, sleeping tiles, and grids whose row
pitch takes the tensor-load path (width a multiple of 8, at least 32) or the
plain-load path (other widths)."""
import importlib.util
from pathlib import Path

import numpy as np
import pytest

import pyoracle as po
from canvaz_film import capi, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gp():
    import __graft_entry__ as g
    g.build()
    spec = importlib.util.spec_from_file_location("gp", Path(__file__).parent / "test_gpu_parity.py")
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def cases(gp):
    yield "drip96x80", gp.make_case("drip")
    yield "blob80x64", gp.make_case("blob")
    yield "mixed", gp.make_case("mixed")
    # widths whose row pitch is not a multiple of 16 bytes: plain loads
    yield "drip90x70", (synth.drip_canvas(90, 70, 8, n_lines=7, per_cell_n=True), (2e-4, 1, 3))
    # a last tile column half outside the grid (tensor loads fill it with 0)
    yield "blob36x28", (synth.blob_canvas(36, 28, 4, n_blobs=3, sigma=(2, 6), per_cell_n=True), (1e-3, 1, 2))


def close(a, b, name):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    scale = max(float(np.abs(b).max()), 1e-30)
    bad = np.abs(a - b) > 1e-5 * np.abs(b) + 1e-7 * scale
    assert not bad.any(), (name, int(bad.sum()), float((np.abs(a - b) / scale).max()))
    return int((a != b).sum())


@pytest.mark.parametrize("prec", [capi.CF_PREC_REFERENCE, capi.CF_PREC_FP32, capi.CF_PREC_BF16])
def test_flow_equals_separate_dispatches(gp, prec):
    from canvaz_film.film import Film
    for name, (cv, sched) in cases(gp):
        o = gp.oracle_state(cv, sched)
        f = Film(po.make_settings(cv.settings), cv.w, cv.h, prec)
        f.set_tables(cv.pigtab, cv.cmf)
        gp.transfer(o, f)
        f.run("flow")
        flux_f, tmp_f = f.plane("flux"), f.plane("tmp")
        gp.transfer(o, f)
        for k in ("laplacian", "plug", "fluxes"):
            f.run(k)
        flux_s, tmp_s = f.plane("flux"), f.plane("tmp")
        nflux = close(flux_f, flux_s, name + " flux")
        ntmp = close(tmp_f, tmp_s, name + " tmp")
        print("%s prec %d: fluxes %d of %d differ in the last bits, tmp %d" % (name, prec, nflux, flux_f.size, ntmp))
        assert np.abs(flux_s).max() > 0.0
        f.close()


@pytest.mark.parametrize("prec", [capi.CF_PREC_REFERENCE, capi.CF_PREC_FP32, capi.CF_PREC_BF16])
def test_limit_apply_equals_separate_dispatches(gp, prec):
    """The fused limiter + apply (alpha in shared memory, the new heights in
    h_next) against the limiter and apply dispatches from the same state: the
    heights, acc, back-filled strata and rheology to rounding, the moved
    tiles and the nose's delta snapshot exactly."""
    from canvaz_film.film import Film
    for name, (cv, sched) in cases(gp):
        o = gp.oracle_state(cv, sched)
        f = Film(po.make_settings(cv.settings), cv.w, cv.h, prec)
        f.set_tables(cv.pigtab, cv.cmf)
        gp.transfer(o, f)
        f.set_plane("tile_moved", np.zeros(f.plane("tile_moved").size))
        f.run("limit_apply")
        fused = {"h": f.plane("h_next")}
        for k in ("acc", "mu", "tau", "nn", "strata_h", "strata_cure", "strata_pig", "tile_moved", "delta_old"):
            fused[k] = f.plane(k)
        gp.transfer(o, f)
        f.set_plane("tile_moved", np.zeros(f.plane("tile_moved").size))
        f.run("limiter")
        f.run("apply")
        sep = {k: f.plane(k) for k in fused}
        for k in ("tile_moved", "delta_old"):
            np.testing.assert_array_equal(fused[k], sep[k], err_msg="%s %s" % (name, k))
        diffs = {k: close(fused[k], sep[k], "%s %s" % (name, k)) for k in ("h", "acc", "mu", "tau", "nn", "strata_h",
                                                                        "strata_cure", "strata_pig")}
        moved = np.count_nonzero(sep["h"] != o.buf("h"))  # the transferred state holds f32-rounded heights
        print("%s prec %d: values differing in the last bits %s; cells whose height changed %d"
              % (name, prec, diffs, moved))
        assert moved > 0
        f.close()
