"""CPU restatement of the reference's deposit records (TEST INFRASTRUCTURE).

Only tests/, smoke() and bench.py's CPU baseline use this module, as the
checker.  It restates, in numpy float32 with one rounding per operation (the
reference computes these on the host in Rust f32, which never contracts):
  - Deposit::ribbon / capsule / stroke          src/film/mod.rs:63-93
  - Deposit::profile                            src/film/mod.rs:150-185
  - Deposit::sampled_volume(_in)                src/film/mod.rs:113-131
  - Deposit::inside_fraction                    src/film/mod.rs:133-146
  - Film::upload_deposits (binning, totals)     src/film/mod.rs:1175-1224
Records use the reference's 96-byte Deposit layout (src/film/mod.rs:25-39).
Parity is pinned by the reference's own tests of these functions
(lattice_volume_matches_reference and ribbon_segments_hold_their_volume,
src/film/mod.rs:1520-1571), restated in tests/test_deposit.py.
"""
import numpy as np

f32 = np.float32

RECYCLED, CAP_START, CAP_END, METHOD_SHIFT = 1, 2, 4, 8
MAX_DEPOSITS = 1 << 16

DEPOSIT_DTYPE = np.dtype([("p0", "<f4", 2), ("p1", "<f4", 2), ("n0", "<f4", 2), ("n1", "<f4", 2),
                          ("r0", "<f4"), ("r1", "<f4"), ("h0", "<f4"), ("vol", "<f4"),
                          ("kind", "<u4"), ("pad", "<u4", 3), ("pig", "<u4", 8)])
assert DEPOSIT_DTYPE.itemsize == 96


def record(p0, p1, n0, n1, r0, r1, h0, vol, kind, pig):
    d = np.zeros((), DEPOSIT_DTYPE)
    d["p0"], d["p1"], d["n0"], d["n1"] = p0, p1, n0, n1
    d["r0"], d["r1"], d["h0"], d["vol"] = r0, r1, h0, vol
    d["kind"] = kind
    d["pig"] = pig
    return d


def segment_dir(p0, p1):  # src/film/mod.rs:56-60
    d0, d1 = f32(p1[0]) - f32(p0[0]), f32(p1[1]) - f32(p0[1])
    l = np.sqrt(d0 * d0 + d1 * d1)
    if l > 0:
        return (d0 / l, d1 / l), l
    return (f32(1), f32(0)), f32(0)


def max_radius(d):
    return max(f32(d["r0"]), f32(d["r1"]))


def max_height(d):
    return f32(d["h0"]) * max_radius(d) / f32(d["r0"])


def profile(d, px, py):
    """Height of the deposit's profile at the points (px, py), float32 arrays."""
    px = np.asarray(px, f32)
    py = np.asarray(py, f32)
    p0, p1, n0, n1 = [np.asarray(d[k], f32) for k in ("p0", "p1", "n0", "n1")]
    r0, r1, h0 = f32(d["r0"]), f32(d["r1"]), f32(d["h0"])
    (dx, dy), l = segment_dir(p0, p1)
    kind = int(d["kind"])
    cap_start, cap_end = (kind & CAP_START) != 0, (kind & CAP_END) != 0
    q0x, q0y = px - p0[0], py - p0[1]
    q1x, q1y = px - p1[0], py - p1[1]
    with np.errstate(divide="ignore", invalid="ignore"):
        if l <= 0:
            x = np.sqrt(q0x * q0x + q0y * q0y) / r0
            return np.where(x < 1, h0 * (f32(1) - x * x), f32(0)).astype(f32)
        zero = np.zeros(px.shape, bool)
        if not cap_start:
            zero |= (q0x * n0[0] + q0y * n0[1]) < 0
        if not cap_end:
            zero |= (q1x * n1[0] + q1y * n1[1]) >= 0
        u = q0x * dx + q0y * dy
        zero |= (u < -r0) | (u > l + r1)
        dist = np.abs(q0x * dy - q0y * dx)
        if cap_start:
            dist = np.where(u < 0, np.sqrt(q0x * q0x + q0y * q0y), dist)
        if cap_end:
            dist = np.where(u > l, np.sqrt(q1x * q1x + q1y * q1y), dist)
        rt = r0 + (r1 - r0) * np.minimum(np.maximum(u / l, f32(0)), f32(1))
        x = dist / rt
        h = np.where(x < 1, h0 * (rt / r0) * (f32(1) - x * x), f32(0))
    return np.where(zero, f32(0), h).astype(f32)


def lattice_sum(heights):
    """The sequential float32 sum of Rust's `sum += h` loop."""
    if heights.size == 0:
        return f32(0)
    return np.cumsum(heights.astype(f32), dtype=f32)[-1]


def sampled_volume_in(d, lattice, lo, hi):  # src/film/mod.rs:117-131
    lattice = f32(lattice)
    p0, p1 = np.asarray(d["p0"], f32), np.asarray(d["p1"], f32)
    rm = max_radius(d) + lattice
    x0 = int(np.floor(max(min(p0[0], p1[0]) - rm, f32(lo[0])) / lattice))
    x1 = int(np.ceil(min(max(p0[0], p1[0]) + rm, f32(hi[0])) / lattice))
    y0 = int(np.floor(max(min(p0[1], p1[1]) - rm, f32(lo[1])) / lattice))
    y1 = int(np.ceil(min(max(p0[1], p1[1]) + rm, f32(hi[1])) / lattice))
    if x1 <= x0 or y1 <= y0:
        return f32(0) * lattice * lattice
    xs = (np.arange(x0, x1).astype(f32) + f32(0.5)) * lattice
    ys = (np.arange(y0, y1).astype(f32) + f32(0.5)) * lattice
    px, py = np.meshgrid(xs, ys, indexing="ij")  # i outer, j inner
    return lattice_sum(profile(d, px.ravel(), py.ravel())) * lattice * lattice


def sampled_volume(d, lattice):
    return sampled_volume_in(d, lattice, (-np.inf, -np.inf), (np.inf, np.inf))


def inside_fraction(d, w, h):  # src/film/mod.rs:133-146
    w, h = f32(w), f32(h)
    rb = max_radius(d)
    p0, p1 = np.asarray(d["p0"], f32), np.asarray(d["p1"], f32)
    full = (min(p0[0], p1[0]) - rb >= 0 and min(p0[1], p1[1]) - rb >= 0 and max(p0[0], p1[0]) + rb <= w
            and max(p0[1], p1[1]) + rb <= h)
    if full:
        return f32(1)
    lattice = f32(0.25) * max(min(f32(d["r0"]), f32(d["r1"])), f32(1e-4))
    a = sampled_volume(d, lattice)
    if a <= 0:
        return f32(0)
    return min(max(sampled_volume_in(d, lattice, (0, 0), (w, h)) / a, f32(0)), f32(1))


def ribbon(p0, p1, n0, n1, r0, r1, caps, volume, pig, dx):  # src/film/mod.rs:63-80
    dx, volume = f32(dx), f32(volume)
    min_r = f32(0.8) * dx
    a, b = max(f32(r0), min_r), max(f32(r1), min_r)
    d = record(p0, p1, n0, n1, a, b, a, volume, caps, pig)
    lattice = f32(0.25) * dx
    sampled = sampled_volume(d, lattice)
    rm = max(a, b)
    disc = f32(np.pi) * rm * rm * rm / f32(2)
    if sampled < f32(0.25) * disc:
        p0, p1 = np.asarray(p0, f32), np.asarray(p1, f32)
        mid = (f32(0.5) * (p0[0] + p1[0]), f32(0.5) * (p0[1] + p1[1]))
        d = record(mid, mid, n0, n1, rm, rm, rm, volume, caps, pig)
        d["h0"] = volume / sampled_volume(d, lattice) * rm
        return d
    d["h0"] = volume / sampled * a
    return d


def capsule(p0, p1, r, volume, pig, dx):  # src/film/mod.rs:82-85
    dd, _ = segment_dir(p0, p1)
    return ribbon(p0, p1, dd, dd, r, r, CAP_START | CAP_END, volume, pig, dx)


def stroke(p0, p1, r, volume, pig, dx):  # src/film/mod.rs:87-93
    dd, l = segment_dir(p0, p1)
    if l < max(f32(r), f32(0.8) * f32(dx)):
        return capsule(p0, p1, r, volume, pig, dx)
    return ribbon(p0, p1, dd, dd, r, r, 0, volume, pig, dx)


def bin_deposits(deps, w, h, width_m, height_m, h_max=0.0, h_max_pending=0.0, total=0.0):
    """Film::upload_deposits (src/film/mod.rs:1175-1224) for a w x h film.

    Returns (sent, start, count, items, total_deposited, h_max_pending) with
    the tile tables over 64x64-cell tiles."""
    deps = np.asarray(deps, DEPOSIT_DTYPE).reshape(-1)
    count = min(len(deps), MAX_DEPOSITS)
    dx = f32(width_m) / f32(w)
    tile_m = f32(64) * dx
    tw, th = (w + 63) // 64, (h + 63) // 64
    lists = [[] for _ in range(tw * th)]
    wm, hm = f32(width_m), f32(height_m)
    hp = f32(h_max_pending)
    for di in range(count):
        d = deps[di]
        hp = max(hp, max_height(d) + f32(h_max))
        rb = max_radius(d)
        p0, p1 = np.asarray(d["p0"], f32), np.asarray(d["p1"], f32)
        minx, maxx = min(p0[0], p1[0]) - rb, max(p0[0], p1[0]) + rb
        miny, maxy = min(p0[1], p1[1]) - rb, max(p0[1], p1[1]) + rb
        if not (maxx > 0 and maxy > 0 and minx < wm and miny < hm):
            continue
        if int(d["kind"]) & RECYCLED == 0:
            total += float(d["vol"]) * float(inside_fraction(d, wm, hm))
        if maxx < 0 or maxy < 0:
            continue

        def tix(v, n):
            return min(int(max(np.floor(v / tile_m), f32(0))), n - 1)
        tx0, tx1, ty0, ty1 = tix(minx, tw), tix(maxx, tw), tix(miny, th), tix(maxy, th)
        for ty in range(ty0, ty1 + 1):
            for tx in range(tx0, tx1 + 1):
                lists[ty * tw + tx].append(di)
    start = np.zeros(tw * th, np.uint32)
    cnt = np.zeros(tw * th, np.uint32)
    items = []
    cap = MAX_DEPOSITS * 16
    for t in range(tw * th):
        take = min(len(lists[t]), cap - len(items))
        start[t] = len(items)
        cnt[t] = take
        items.extend(lists[t][:take])
    return count, start, cnt, np.asarray(items, np.uint32), total, float(hp)


def pack_pig(values):
    """16 pigment slots -> 8 u32 words of f16 pairs (pack2x16float)."""
    v = np.asarray(values, np.float16).reshape(8, 2).view(np.uint16).astype(np.uint32)
    return (v[:, 0] | (v[:, 1] << 16)).astype(np.uint32)
