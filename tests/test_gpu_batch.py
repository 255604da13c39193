"""Batches of films (cf_batch_*) against films stepped alone (GPU).

A batch steps every film with one launch per dispatch over a table of all
their tiles (the same kernel bodies as a film alone), so each film's planes
and colour after a batched run must equal, bit for bit, those of the same
film stepped alone.  The cases mix precision modes (separate packed groups),
sizes that are not multiples of the 16x16 tile, fixed and adaptive dt, direct
launches and graph replays (with a remainder of frames), and films joining
and leaving between steps.
"""
import numpy as np
import pytest

import pyoracle as po
from canvaz_film import capi, synth

pytestmark = pytest.mark.gpu

FRAMES = 5


@pytest.fixture(scope="module")
def built():
    import __graft_entry__ as g
    g.build()
    return True


def cases():
    blob = synth.blob_canvas(80, 64, 13, n_blobs=6, sigma=(3, 9), tau=(0, 0.5), mu=(0.05, 0.3), peak_mm=(1.0, 3.0))
    blob.settings.update(rho=1000.0)
    drip = synth.drip_canvas(96, 80, 5, n_lines=8)
    small = synth.blob_canvas(40, 36, 3, n_blobs=4, sigma=(3, 8), tau=(0, 2.0), mu=(0.1, 1.0), peak_mm=(0.5, 2.0))
    wide = synth.blob_canvas(72, 50, 21, n_blobs=5, sigma=(3, 9), tau=(0, 1.0), mu=(0.05, 0.5), peak_mm=(1.0, 2.5))
    return [(blob, capi.CF_PREC_FP32, 1 / 60), (drip, capi.CF_PREC_FP32, 2e-4), (small, capi.CF_PREC_REFERENCE, 1 / 60),
            (wide, capi.CF_PREC_BF16, 1 / 60)]


def make_film(cv, prec):
    from canvaz_film.film import Film
    f = Film(po.make_settings(cv.settings), cv.w, cv.h, prec)
    f.set_tables(cv.pigtab, cv.cmf)
    f.write_state(cv.planes)
    return f


def snapshot(f):
    st = f.read_state()
    st["color"] = f.color()
    return st


def assert_same(a, b, what):
    for k in a:
        assert np.array_equal(a[k], b[k], equal_nan=True), "%s: plane %s differs" % (what, k)


def solo(cv, prec, fdt, substeps, frames, dt_max=0.0):
    f = make_film(cv, prec)
    if dt_max > 0:
        for _ in range(frames):
            f.step_adaptive(dt_max)
    else:
        f.update_params(fdt, substeps)
        for _ in range(frames):
            f.encode_frame(substeps)
    return snapshot(f)


TUNINGS = [
    {"use_graph": 0, "frames_per_graph": 1, "list_blocks_per_sm": 8, "tiles_per_block": 1},
    {"use_graph": 1, "frames_per_graph": 1, "list_blocks_per_sm": 8, "tiles_per_block": 1},
    {"use_graph": 1, "frames_per_graph": 2, "list_blocks_per_sm": 4, "tiles_per_block": 1},
    # launch tiles of 32x16 and 64x16 cells, and a walk of 37 tiles per block
    # (runs crossing tile rows and films)
    {"use_graph": 0, "frames_per_graph": 1, "list_blocks_per_sm": 8, "tiles_per_block": 2},
    {"use_graph": 1, "frames_per_graph": 1, "list_blocks_per_sm": 8, "tiles_per_block": 4},
    {"use_graph": 1, "frames_per_graph": 2, "list_blocks_per_sm": 8, "tiles_per_block": 37},
]


@pytest.mark.parametrize("tuning", TUNINGS, ids=["direct", "graph1", "graph2", "tiles2", "tiles4-graph", "walk37"])
def test_batch_equals_films_alone_fixed_dt(built, tuning):
    from canvaz_film.film import Batch
    cs = cases()
    substeps = 2
    want = [solo(cv, prec, fdt, substeps, FRAMES) for cv, prec, fdt in cs]
    films = [make_film(cv, prec) for cv, prec, _ in cs]
    b = Batch()
    b.tuning = tuning
    for f, (_, _, fdt) in zip(films, cs):
        f.update_params(fdt, substeps)
        b.add(f)
    b.step(FRAMES, substeps)
    for k, f in enumerate(films):
        assert_same(snapshot(f), want[k], "film %d" % k)
    info = b.info()
    assert info["films"] == len(cs) and info["launches"] > 0
    assert all(f.stats()["frames"] == FRAMES for f in films)
    b.close()


def test_batch_equals_films_alone_adaptive(built):
    from canvaz_film.film import Batch
    cs = cases()
    dt_max = 1 / 60
    want = [solo(cv, prec, fdt, 1, FRAMES, dt_max) for cv, prec, fdt in cs]
    films = [make_film(cv, prec) for cv, prec, _ in cs]
    b = Batch()
    b.tuning = {"use_graph": 1, "frames_per_graph": 2}
    for f in films:
        b.add(f)
    b.step(FRAMES, 1, dt_max)
    for k, f in enumerate(films):
        assert_same(snapshot(f), want[k], "film %d" % k)
    b.close()


def test_films_join_and_leave(built):
    from canvaz_film.film import Batch
    (cx, px, fx), (cy, py, fy) = cases()[0], cases()[3]
    want_x = solo(cx, px, fx, 1, 5)
    want_y = solo(cy, py, fy, 1, 4)
    x, y = make_film(cx, px), make_film(cy, py)
    x.update_params(fx, 1)
    y.update_params(fy, 1)
    b = Batch()
    b.add(x)
    b.step(2)
    b.add(y)
    b.step(3)
    b.remove(x)
    b.step(1)
    assert_same(snapshot(x), want_x, "film x")
    assert_same(snapshot(y), want_y, "film y")
    b.close()


def test_autotune_picks_a_candidate(built):
    from canvaz_film.film import Batch
    films = [make_film(cv, prec) for cv, prec, _ in cases()]
    b = Batch()
    for f, (_, _, fdt) in zip(films, cases()):
        f.update_params(fdt, 1)
        b.add(f)
    tuning, ms = b.autotune(frames_per_trial=2)
    assert ms > 0
    assert tuning["list_blocks_per_sm"] in (4, 8, 16)
    assert (tuning["use_graph"], tuning["frames_per_graph"]) in ((1, 1), (0, 1), (1, 2), (1, 4))
    assert 1 <= tuning["tiles_per_block"] <= 4096
    b.step(3)  # keeps stepping with the chosen tuning
    b.close()


def test_batch_errors_are_status_codes(built):
    from canvaz_film.film import Batch
    from canvaz_film.capi import FilmError
    cv, prec, fdt = cases()[2]
    f = make_film(cv, prec)
    b1, b2 = Batch(), Batch()
    b1.add(f)
    with pytest.raises(FilmError) as e:
        b2.add(f)
    assert e.value.status == capi.CF_ERR_INVALID_ARG
    with pytest.raises(FilmError):
        b2.remove(f)
    with pytest.raises(FilmError):
        b1.tuning = {"frames_per_graph": 0}
    b1.close()
    b2.add(f)  # free again once its batch is gone
    b2.close()
