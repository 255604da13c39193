"""cf_cfl_stats_noalloc against the film's own statistics (GPU).

The allocation-free entry point reads caller-owned device planes h and mu and
keeps its per-tile partials in a fixed device array shared by every call.  It
is checked against cf_get_stats (the film's tile reduction) on the same state,
on calls in a row over canvases of different tile counts, so that partials
left by one call cannot leak into the next, and against a plain numpy max /
min over the same planes (independent of any GPU reduction).  This file is
collected last and also runs alone: its fixture builds the library itself.
"""
import ctypes as C

import numpy as np
import pytest

import pyoracle as po
from canvaz_film import capi, synth

pytestmark = pytest.mark.gpu

RTOL = 1e-6  # both sides take the max / min of the same FP32 values


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__ as g
    g.build()
    return capi.load_library()


def film_case(cv, prec, steps, dt_max):
    """State of a CUDA film after `steps` adaptive steps, with its own stats."""
    from canvaz_film.film import Film
    f = Film(po.make_settings(cv.settings), cv.w, cv.h, prec)
    f.set_tables(cv.pigtab, cv.cmf)
    f.write_state(cv.planes)
    for _ in range(steps):
        f.step_adaptive(dt_max)
    f.sync()
    s = f.stats()
    st = f.read_state()
    h_min = f.params().ein[3]
    return st["h"].copy(), st["rheo"][:, 0].copy(), h_min, (s["h_max"], s["mu_min"])


def noalloc(lib, h, mu, w, hgt, h_min):
    import torch
    dh = torch.from_numpy(np.ascontiguousarray(h, np.float32)).cuda()
    dmu = torch.from_numpy(np.ascontiguousarray(mu, np.float32)).cuda()
    out = torch.full((2,), -7.0, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    st = lib.cf_cfl_stats_noalloc(dh.data_ptr(), dmu.data_ptr(), w, hgt, C.c_float(h_min), out.data_ptr(), stream)
    assert st == capi.CF_OK
    torch.cuda.synchronize()
    return out.cpu().numpy()


def numpy_stats(h, mu, h_min):
    """h_max / mu_min over the cells with h > 4 h_min (mu_min 1 when none),
    in plain numpy on the same FP32 values."""
    h = np.asarray(h, np.float32)
    sel = h > np.float32(4.0) * np.float32(h_min)
    if not sel.any():
        return np.array([0.0, 1.0], np.float32)
    return np.array([h[sel].max(), np.asarray(mu, np.float32)[sel].min()], np.float32)


def test_noalloc_matches_film_stats_on_calls_in_a_row(lib):
    drip = synth.drip_canvas(300, 260, 3, n_lines=12)
    blob = synth.blob_canvas(128, 96, 7, n_blobs=5, sigma=(4, 12))
    cases = [(drip, film_case(drip, capi.CF_PREC_FP32, 2, 2e-3)),
             (blob, film_case(blob, capi.CF_PREC_REFERENCE, 1, 1e-3))]
    # the larger grid first, then the smaller one (its partials lie inside the
    # first call's), then the first again
    for cv, (h, mu, h_min, want) in cases + cases[:1]:
        got = noalloc(lib, h, mu, cv.w, cv.h, h_min)
        assert want[0] > 0.0
        np.testing.assert_allclose(got, np.array(want, np.float32), rtol=RTOL, atol=0)
        np.testing.assert_array_equal(got, numpy_stats(h, mu, h_min))


def test_noalloc_exact_tile_multiples(lib):
    """128 x 64 cells: two whole 64 x 64 tiles, no partial tile edge."""
    cv = synth.blob_canvas(128, 64, 11, n_blobs=4, sigma=(4, 10))
    h, mu, h_min, want = film_case(cv, capi.CF_PREC_FP32, 2, 1e-3)
    got = noalloc(lib, h, mu, cv.w, cv.h, h_min)
    np.testing.assert_allclose(got, np.array(want, np.float32), rtol=RTOL, atol=0)
    np.testing.assert_array_equal(got, numpy_stats(h, mu, h_min))


def test_noalloc_follows_the_callers_stream(lib):
    """On a fresh non-default stream the planes are written on that stream just
    before the call, with no synchronisation in between: the call must see
    them (stream order), then a second call on new values must see those."""
    import torch
    rng = np.random.default_rng(5)
    w, hgt, h_min = 200, 136, 1.5e-5
    s = torch.cuda.Stream()
    dh = torch.zeros(w * hgt, dtype=torch.float32, device="cuda")
    dmu = torch.zeros(w * hgt, dtype=torch.float32, device="cuda")
    out = torch.full((2,), -7.0, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    for k in range(2):
        h = np.where(rng.random(w * hgt) < 0.3, rng.uniform(0, 3e-3, w * hgt), 0.0).astype(np.float32)
        mu = rng.uniform(0.5, 50.0, w * hgt).astype(np.float32)
        hp = torch.from_numpy(h).pin_memory()
        mp = torch.from_numpy(mu).pin_memory()
        with torch.cuda.stream(s):
            dh.copy_(hp, non_blocking=True)
            dmu.copy_(mp, non_blocking=True)
        st = lib.cf_cfl_stats_noalloc(dh.data_ptr(), dmu.data_ptr(), w, hgt, C.c_float(h_min), out.data_ptr(),
                                      s.cuda_stream)
        assert st == capi.CF_OK
        with torch.cuda.stream(s):
            got = out.to("cpu", non_blocking=True)
        s.synchronize()
        np.testing.assert_array_equal(got.numpy(), numpy_stats(h, mu, h_min))


def test_noalloc_one_tile_wide_tall_grid(lib):
    """A grid one 64-cell tile wide and 65,536 tiles tall is inside the
    scratch's limit and must run (40 x 4,194,304 cells)."""
    import torch
    w, hgt, h_min = 40, 64 * 65536, 1.5e-5
    n = w * hgt
    dh = torch.zeros(n, dtype=torch.float32, device="cuda")
    dmu = torch.full((n,), 3.0, dtype=torch.float32, device="cuda")
    dh[n - 7] = 2e-3  # in the last tile
    dmu[n - 7] = 0.75
    dh[5 * w + 3] = 1e-3
    out = torch.full((2,), -7.0, dtype=torch.float32, device="cuda")
    st = lib.cf_cfl_stats_noalloc(dh.data_ptr(), dmu.data_ptr(), w, hgt, C.c_float(h_min), out.data_ptr(),
                                  torch.cuda.current_stream().cuda_stream)
    assert st == capi.CF_OK
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out.cpu().numpy(), np.array([2e-3, 0.75], np.float32))


def test_noalloc_dry_canvas(lib):
    cv = synth.blob_canvas(96, 70, 2, n_blobs=3)
    for k in ("h", "strata_h"):
        cv.planes[k][:] = 0.0
    h, mu, h_min, want = film_case(cv, capi.CF_PREC_FP32, 0, 1e-3)
    got = noalloc(lib, h, mu, cv.w, cv.h, h_min)
    np.testing.assert_allclose(got, np.array(want, np.float32), rtol=RTOL, atol=0)
    assert got[0] == 0.0 and got[1] == 1.0


def test_noalloc_rejects_bad_sizes(lib):
    import torch
    buf = torch.zeros(4, dtype=torch.float32, device="cuda")
    p = buf.data_ptr()
    # 16448 x 16384 is 257 x 256 tiles, one row of tiles past the scratch
    assert lib.cf_cfl_stats_noalloc(p, p, 16448, 16384, C.c_float(1e-5), p, None) == capi.CF_ERR_INVALID_ARG
    assert lib.cf_cfl_stats_noalloc(p, p, 0, 8, C.c_float(1e-5), p, None) == capi.CF_ERR_INVALID_ARG
    assert lib.cf_cfl_stats_noalloc(None, p, 8, 8, C.c_float(1e-5), p, None) == capi.CF_ERR_INVALID_ARG
    torch.cuda.synchronize()
    assert torch.count_nonzero(buf).item() == 0
