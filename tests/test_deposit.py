"""Deposit records: the library's host constructors against the oracle (CPU).

The constructors (cf_deposit_ribbon / capsule / stroke), the profile height
and the lattice volume are host code of the CUDA library, so these tests call
them without a GPU.  They restate the reference's own tests of the same
functions (src/film/mod.rs:1520-1571):
  - lattice_volume_matches_reference: 300 seeded strokes; the lattice volume
    and 50 profile heights each equal, bit for bit, a straight restatement of
    the profile (here the oracle's numpy float32 one);
  - ribbon_segments_hold_their_volume: six ribbons/capsules/strokes hold their
    volume within 3 % on a fine grid;
and check every record field bit for bit against the oracle's constructors.
"""
import numpy as np
import pytest

import deposit_ref as dr
from canvaz_film import deposit as dep

f32 = np.float32


def lcg(seed=12345):
    """The reference test's generator: 64-bit LCG, top 24 bits as f32."""
    state = [seed]

    def rnd():
        state[0] = (state[0] * 6364136223846793005 + 1442695040888963407) & (2 ** 64 - 1)
        return f32(state[0] >> 40) / f32(1 << 24)
    return rnd


def same_record(a, b):
    return np.asarray(a, dep.DEPOSIT_DTYPE).tobytes() == np.asarray(b, dr.DEPOSIT_DTYPE).tobytes()


def test_layout_matches_the_reference():
    assert dep.DEPOSIT_DTYPE.itemsize == 96 == dr.DEPOSIT_DTYPE.itemsize
    assert dep.DEPOSIT_DTYPE.descr == dr.DEPOSIT_DTYPE.descr


def test_lattice_volume_matches_reference():
    pig = np.zeros(8, np.uint32)
    dx = f32(3.9e-4)
    rnd = lcg()
    for _ in range(300):
        p0 = (f32(0.1) + f32(0.05) * rnd(), f32(0.1) + f32(0.05) * rnd())
        p1 = (p0[0] + f32(4e-3) * (rnd() - f32(0.5)), p0[1] + f32(4e-3) * (rnd() - f32(0.5)))
        r = f32(2e-4) + f32(2e-3) * rnd()
        d = dep.stroke(p0, p1, r, 1e-9, pig, dx)
        assert same_record(d, dr.stroke(p0, p1, r, 1e-9, pig, dx))
        lattice = f32(0.25) * dx
        want = dr.sampled_volume(d, lattice)
        got = dep.sampled_volume(d, lattice)
        assert got.view(np.uint32) == want.view(np.uint32), (got, want)
        for _ in range(50):
            p = (p0[0] + f32(6e-3) * (rnd() - f32(0.5)), p0[1] + f32(6e-3) * (rnd() - f32(0.5)))
            want = dr.profile(d, np.array([p[0]], f32), np.array([p[1]], f32))[0]
            got = dep.height_at(d, p)
            assert got.view(np.uint32) == want.view(np.uint32), (p, got, want)


def grid_volume(d):
    """The reference test's fine-grid volume (src/film/mod.rs:1467-1485)."""
    r = max(f32(d["r0"]), f32(d["r1"]))
    step = r / f32(40)
    p0, p1 = np.asarray(d["p0"], f32), np.asarray(d["p1"], f32)
    lo = (min(p0[0], p1[0]) - f32(2) * r, min(p0[1], p1[1]) - f32(2) * r)
    hi = (max(p0[0], p1[0]) + f32(2) * r, max(p0[1], p1[1]) + f32(2) * r)

    def axis(a, b):
        v, out = f32(a), []
        while v < b:
            out.append(v)
            v = f32(v + step)
        return np.array(out, f32)
    xs, ys = axis(lo[0], hi[0]), axis(lo[1], hi[1])
    px, py = np.meshgrid(xs, ys, indexing="ij")
    return dr.lattice_sum(dr.profile(d, px.ravel(), py.ravel())) * step * step


def test_ribbon_segments_hold_their_volume():
    pig = np.zeros(8, np.uint32)
    c, s = f32(np.cos(f32(0.3))), f32(np.sin(f32(0.3)))
    dx = f32(3.9e-4)
    cases = [
        dep.ribbon((0, 0), (1e-3, 0), (1, 0), (1, 0), 4e-4, 6e-4, 0, 1e-9, pig, dx),
        dep.ribbon((0, 0), (1e-3, 0), (c, -s), (c, s), 4e-4, 6e-4, 0, 1e-9, pig, dx),
        dep.ribbon((0, 0), (3e-4, 0), (c, s), (c, -s), 8e-4, 8e-4, 0, 1e-9, pig, dx),
        dep.capsule((0, 0), (2e-3, 1e-3), 5e-4, 1e-9, pig, dx),
        dep.capsule((0, 0), (0, 0), 5e-4, 1e-9, pig, dx),
        dep.stroke((0, 0), (4e-3, 0), 5e-4, 1e-9, pig, dx),
    ]
    for i, d in enumerate(cases):
        v = float(grid_volume(d))
        assert abs(v - float(d["vol"])) < 0.03 * float(d["vol"]), (i, v, float(d["vol"]))


def test_constructor_fields_match_the_oracle():
    """Short strokes become capsules, tiny ribbons collapse to a dot at the
    midpoint, radii are floored at 0.8 dx; every field equals the oracle's."""
    rng = np.random.default_rng(7)
    dx = f32(1e-3)
    for _ in range(60):
        pig = rng.integers(0, 2 ** 32, 8, dtype=np.uint64).astype(np.uint32)
        p0 = tuple(f32(v) for v in rng.uniform(0, 0.05, 2))
        p1 = tuple(f32(v + d) for v, d in zip(p0, rng.normal(0, 3e-3, 2)))
        r0, r1 = (f32(v) for v in rng.uniform(1e-4, 4e-3, 2))
        n0, n1 = (tuple(f32(x) for x in (np.cos(a), np.sin(a))) for a in rng.uniform(-0.5, 0.5, 2))
        vol = f32(rng.uniform(1e-10, 1e-8))
        caps = int(rng.integers(0, 8))
        assert same_record(dep.ribbon(p0, p1, n0, n1, r0, r1, caps, vol, pig, dx),
                           dr.ribbon(p0, p1, n0, n1, r0, r1, caps, vol, pig, dx))
        assert same_record(dep.capsule(p0, p1, r0, vol, pig, dx), dr.capsule(p0, p1, r0, vol, pig, dx))
        assert same_record(dep.stroke(p0, p1, r0, vol, pig, dx), dr.stroke(p0, p1, r0, vol, pig, dx))
    d = dep.stroke((0.01, 0.01), (0.0102, 0.01), 2e-3, 1e-9, np.zeros(8, np.uint32), dx)
    assert d["kind"] == dr.CAP_START | dr.CAP_END  # shorter than its radius: a capsule
    d = dep.ribbon((0.01, 0.01), (0.0101, 0.01), (1, 0), (1, 0), 1e-4, 1e-4, 0, 1e-9, np.zeros(8, np.uint32), dx)
    assert d["p0"][0] == d["p1"][0] and d["r0"] == d["r1"] == f32(0.8) * dx


def test_sampled_volume_sum_is_sequential_f32():
    """lattice_sum accumulates like Rust's `sum += h` (one f32 rounding per add)."""
    rng = np.random.default_rng(1)
    v = rng.uniform(0, 1e-4, 999).astype(f32)
    s = f32(0)
    for x in v:
        s = f32(s + x)
    assert dr.lattice_sum(v) == s


def test_binning_follows_upload_deposits():
    """Tile tables of upload_deposits: a deposit lands in every 64x64-cell
    tile its bounding box touches; ones entirely off the canvas are skipped;
    recycled ones do not count toward the deposited total."""
    dx = f32(1e-3)
    w = h = 200  # 4 x 4 tiles of 64 cells
    pig = np.zeros(8, np.uint32)
    deps = np.array([
        dr.capsule((0.030, 0.030), (0.030, 0.030), 2e-3, 1e-9, pig, dx),    # tile 0
        dr.stroke((0.060, 0.010), (0.070, 0.010), 2e-3, 1e-9, pig, dx),     # tiles 0, 1
        dr.capsule((-0.05, 0.1), (-0.04, 0.1), 1e-3, 1e-9, pig, dx),        # off the canvas
        dr.stroke((0.15, 0.15), (0.199, 0.15), 2e-3, 1e-9, pig, dx),        # tiles 10, 11 (x clamped)
    ])
    deps[3]["kind"] |= dr.RECYCLED
    sent, start, cnt, items, total, hp = dr.bin_deposits(deps, w, h, f32(0.2), f32(0.2))
    assert sent == 4
    lists = {t: list(items[start[t]:start[t] + cnt[t]]) for t in range(16) if cnt[t]}
    assert lists == {0: [0, 1], 1: [1], 10: [3], 11: [3]}
    assert total == pytest.approx(2e-9, rel=1e-6)
    assert hp == pytest.approx(max(float(dr.max_height(d)) for d in deps), rel=1e-6)
