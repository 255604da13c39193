"""Seeded synthetic canvases in the reference's per-cell state layout.

No public dataset or benchmark is involved: every canvas is generated here
from a numpy PCG64 seed, so the same call gives the same bytes on any host.
Each generator returns a `Canvas`: the eight persistent planes of
Film::state_buffers (src/film/mod.rs:1277-1279), the colour tables
(pigment_table / cmf_table layout, src/color/mod.rs:150-171, 243-258) and the
FilmSettings overrides of the workload.

Pigment slots per stratum (strata.wgsl:37-59, cure.wgsl:3-48): 0-11 pigment
fractions, 12 thinner, 13 yield stress (Pa), 14 ln(mu)+10 (0 = use the
pigment table's viscosity), 15 power-law index n (0 = the global n).

Units: dx = 1 mm.  K and S are drawn per millimetre and stored per metre
(x 1e3), the unit of the reference's tables (thickness in metres, km.wgsl:1-11).
"""
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

DATA = Path(__file__).resolve().parent / "data" / "reference_tables.npz"


@dataclass
class Canvas:
    w: int
    h: int
    planes: dict          # name -> numpy array in the oracle layout (see below)
    pigtab: np.ndarray    # float32[480]
    cmf: np.ndarray       # float32[48]
    settings: dict = field(default_factory=dict)
    name: str = ""

    @property
    def n(self):
        return self.w * self.h


def reference_tables():
    """cmf_table and pigment_table of the reference (derived by data/make_tables.py)."""
    d = np.load(DATA)
    return d["pigtab"].astype(np.float32), d["cmf"].astype(np.float32)


def random_tables(rng, nband=16, ks_lo=0.01, ks_hi=10.0):
    """Per-pigment K, S uniform in [ks_lo, ks_hi] per mm (stored per m), tint 1.
    With nband < 16 only the first nband band columns are drawn; the rest are 0."""
    t = np.zeros(12 * 40, dtype=np.float32)
    for i in range(12):
        k = rng.uniform(ks_lo, ks_hi, nband) * 1e3
        s = rng.uniform(ks_lo, ks_hi, nband) * 1e3
        t[i * 40: i * 40 + nband] = k
        t[i * 40 + 16: i * 40 + 16 + nband] = s
        t[i * 40 + 32] = np.exp(rng.uniform(np.log(0.5), np.log(50.0)))
        t[i * 40 + 33] = rng.uniform(0.0, 20.0)
        t[i * 40 + 34] = 1.0
    return t


def substrate(raw=True, nband=16):
    """substrate_refl bands (src/film/mod.rs:188-210)."""
    t = np.arange(16, dtype=np.float32) / np.float32(15.0)
    v = (np.float32(0.50) + np.float32(0.16) * t) if raw else (np.float32(0.84) + np.float32(0.04) * t)
    return v.astype(np.float32)


def _empty_planes(n):
    return {
        "h": np.zeros(n, np.float32),
        "m": np.zeros(n, np.float32),
        "rheo": np.zeros((n, 2), np.float32),
        "strata_h": np.zeros((n, 4), np.float32),
        "strata_pig": np.zeros((n, 64), np.float32),
        "strata_cure": np.zeros((n, 4), np.float32),
        "sub_refl": np.zeros((n, 16), np.float32),
        "lay": np.zeros(n, np.uint32),
    }


def _fill_strata(planes, h, pig_num, wsum, rheo_of, per_cell_n):
    """One stratum per wet cell: h-weighted pigment mix, dominant-source rheology."""
    n = h.size
    wet = h > 0
    planes["h"][:] = h
    planes["strata_h"][:, 0] = h
    with np.errstate(invalid="ignore", divide="ignore"):
        mix = np.where(wsum[:, None] > 0, pig_num / np.maximum(wsum[:, None], 1e-30), 0.0)
    pig = np.zeros((n, 16), np.float32)
    pig[:, :12] = mix
    tau, mu, nn = rheo_of
    pig[:, 13] = tau
    pig[:, 14] = np.log(mu) + 10.0
    pig[:, 15] = nn if per_cell_n else 0.0
    pig[~wet] = 0.0
    planes["strata_pig"][:, :16] = pig
    planes["rheo"][:, 0] = np.where(wet, mu, 1.0)
    planes["rheo"][:, 1] = np.where(wet, tau, 0.0)
    planes["strata_h"][~wet] = 0.0


def blob_canvas(w, h, seed, n_blobs=20, sigma=(5.0, 40.0), peak_mm=(0.1, 2.0), h_min=1.5e-5,
                ground=0.0, per_cell_n=True, tables="random", nband=16, raw=True,
                tau=(0.0, 20.0), mu=(0.5, 50.0), nrange=(0.6, 1.0)):
    """Sum of Gaussian blobs (centres uniform, sigma in cells, peak in mm), each
    with a Dirichlet(0.5) 12-pigment vector and its own rheology: tau_y U[0,20] Pa,
    mu log-U[0.5,50] Pa s, n U[0.6,1.0].  Cells below h_min are dry."""
    rng = np.random.Generator(np.random.PCG64(seed))
    n = w * h
    hh = np.zeros((h, w), np.float64)
    num = np.zeros((h, w, 12), np.float64)
    best = np.zeros((h, w), np.float64)
    arg = np.full((h, w), -1, np.int64)
    cx = rng.uniform(0, w, n_blobs)
    cy = rng.uniform(0, h, n_blobs)
    sg = rng.uniform(sigma[0], sigma[1], n_blobs)
    pk = rng.uniform(peak_mm[0], peak_mm[1], n_blobs) * 1e-3
    pigs = rng.dirichlet(np.full(12, 0.5), n_blobs)
    tau = rng.uniform(tau[0], tau[1], n_blobs)
    mu = np.exp(rng.uniform(np.log(mu[0]), np.log(mu[1]), n_blobs))
    nidx = rng.uniform(nrange[0], nrange[1], n_blobs)
    for b in range(n_blobs):
        r = 4.0 * sg[b]
        x0, x1 = max(int(cx[b] - r), 0), min(int(cx[b] + r) + 1, w)
        y0, y1 = max(int(cy[b] - r), 0), min(int(cy[b] + r) + 1, h)
        if x0 >= x1 or y0 >= y1:
            continue
        xs = np.arange(x0, x1) + 0.5
        ys = np.arange(y0, y1) + 0.5
        g = pk[b] * np.exp(-((xs[None, :] - cx[b]) ** 2 + (ys[:, None] - cy[b]) ** 2) / (2 * sg[b] ** 2))
        hh[y0:y1, x0:x1] += g
        num[y0:y1, x0:x1] += g[:, :, None] * pigs[b][None, None, :]
        sub = best[y0:y1, x0:x1]
        take = g > sub
        sub[take] = g[take]
        arg[y0:y1, x0:x1][take] = b
    hv = np.where(hh >= h_min, hh, 0.0).astype(np.float32).reshape(n)
    planes = _empty_planes(n)
    a = arg.reshape(n)
    a0 = np.maximum(a, 0)
    _fill_strata(planes, hv, num.reshape(n, 12), hh.reshape(n), (tau[a0], mu[a0], nidx[a0]), per_cell_n)
    planes["m"][:] = ground
    planes["sub_refl"][:] = substrate(raw)[None, :]
    if tables == "random":
        pigtab = random_tables(rng, nband)
        _, cmf = reference_tables()
    else:
        pigtab, cmf = reference_tables()
    settings = dict(width_m=w * 1e-3, height_m=h * 1e-3, rho=1300.0, sigma=0.03, weave_um=0.0,
                    implicit_hydro=0, min_substeps=1, raw_canvas=int(raw))
    return Canvas(w, h, planes, pigtab, cmf, settings, "blobs%d_s%d" % (n_blobs, seed))


def _seg_dist(px, py, ax, ay, bx, by):
    vx, vy = bx - ax, by - ay
    l2 = vx * vx + vy * vy
    t = np.clip(((px - ax) * vx + (py - ay) * vy) / max(l2, 1e-30), 0.0, 1.0)
    dx, dy = px - (ax + t * vx), py - (ay + t * vy)
    return np.sqrt(dx * dx + dy * dy)


def drip_canvas(w, h, seed, n_lines=200, segs=(2, 6), width_cells=(2, 8), height_mm=(0.2, 3.0),
                per_cell_n=True, h_min=1.5e-5, tilt_deg=60.0, nband=16):
    """Random drip polylines: 2-6 segments each, width 2-8 cells, height 0.2-3 mm,
    rasterised with the parabolic ribbon cross-section h0 (1 - (d/r)^2) of
    deposit.wgsl:6-29 on a 4x4 supersampled lattice (deposit.wgsl:52-57).
    Within one polyline the segments join by max; polylines add."""
    rng = np.random.Generator(np.random.PCG64(seed))
    n = w * h
    hh = np.zeros((h, w), np.float64)
    num = np.zeros((h, w, 12), np.float64)
    best = np.zeros((h, w), np.float64)
    arg = np.full((h, w), -1, np.int64)
    pigs = rng.dirichlet(np.full(12, 0.5), n_lines)
    tau = rng.uniform(0.0, 20.0, n_lines)
    mu = np.exp(rng.uniform(np.log(0.5), np.log(50.0), n_lines))
    nidx = rng.uniform(0.6, 1.0, n_lines)
    sub = (np.arange(4) - 1.5) * 0.25
    for L in range(n_lines):
        ns = int(rng.integers(segs[0], segs[1] + 1))
        r = rng.uniform(width_cells[0], width_cells[1]) * 0.5
        h0 = rng.uniform(height_mm[0], height_mm[1]) * 1e-3
        pts = [rng.uniform([0, 0], [w, h])]
        for _ in range(ns):
            ang = rng.uniform(0, 2 * np.pi)
            ln = rng.uniform(10, 120)
            pts.append(pts[-1] + ln * np.array([np.cos(ang), np.sin(ang)]))
        pts = np.array(pts)
        x0 = max(int(pts[:, 0].min() - r - 1), 0)
        x1 = min(int(pts[:, 0].max() + r + 2), w)
        y0 = max(int(pts[:, 1].min() - r - 1), 0)
        y1 = min(int(pts[:, 1].max() + r + 2), h)
        if x0 >= x1 or y0 >= y1:
            continue
        xs = np.arange(x0, x1) + 0.5
        ys = np.arange(y0, y1) + 0.5
        prof = np.zeros((y1 - y0, x1 - x0))
        for sy in sub:
            for sx in sub:
                px = xs[None, :] + sx
                py = ys[:, None] + sy
                d = np.full(prof.shape, np.inf)
                for s in range(ns):
                    d = np.minimum(d, _seg_dist(px, py, *pts[s], *pts[s + 1]))
                x = d / r
                prof += 0.0625 * np.where(x < 1.0, h0 * (1.0 - x * x), 0.0)
        hh[y0:y1, x0:x1] += prof
        num[y0:y1, x0:x1] += prof[:, :, None] * pigs[L][None, None, :]
        bsub = best[y0:y1, x0:x1]
        take = prof > bsub
        bsub[take] = prof[take]
        arg[y0:y1, x0:x1][take] = L
    hv = np.where(hh >= h_min, hh, 0.0).astype(np.float32).reshape(n)
    planes = _empty_planes(n)
    a0 = np.maximum(arg.reshape(n), 0)
    _fill_strata(planes, hv, num.reshape(n, 12), hh.reshape(n), (tau[a0], mu[a0], nidx[a0]), per_cell_n)
    planes["sub_refl"][:] = substrate(True)[None, :]
    pigtab = random_tables(rng, nband)
    _, cmf = reference_tables()
    settings = dict(width_m=w * 1e-3, height_m=h * 1e-3, rho=1300.0, sigma=0.03, weave_um=0.0,
                    implicit_hydro=0, min_substeps=1, tilt_deg=tilt_deg, tilt_dir_deg=90.0)
    return Canvas(w, h, planes, pigtab, cmf, settings, "drips%d_s%d" % (n_lines, seed))


def pour_canvas(w, h, seed, n_blobs=300):
    """Thick, runny pours (3-5 mm, mu 0.05-0.2 Pa s, tau_y <= 0.3 Pa) with the
    reference's implicit hydrostatic step on, as its defaults have it: the
    frames take 1-4 implicit CG steps."""
    cv = blob_canvas(w, h, seed, n_blobs=n_blobs, sigma=(8.0, 40.0), per_cell_n=False, tables="reference",
                     tau=(0.0, 0.3), mu=(0.05, 0.2), peak_mm=(3.0, 5.0))
    cv.settings.update(implicit_hydro=1)
    return cv


def config(k, seed=0, scale=1):
    """The workloads: 0 = 512^2 blobs (K, S over 8 bands), 1 = 2048^2 tilted
    drips, 2 = 4096^2 blobs over a cured ground, 5 = 2048^2 thick pours with
    the implicit hydrostatic step.  `scale` divides the side."""
    if k == 0:
        s = 512 // scale
        return blob_canvas(s, s, seed, n_blobs=20, nband=8)
    if k == 1:
        s = 2048 // scale
        return drip_canvas(s, s, seed, n_lines=max(200 // (scale * scale), 4))
    if k == 2:
        s = 4096 // scale
        return blob_canvas(s, s, seed, n_blobs=max(500 // (scale * scale), 8), ground=5e-5, raw=False)
    if k == 5:
        s = 2048 // scale
        return pour_canvas(s, s, seed, n_blobs=max(300 // (scale * scale), 4))
    raise ValueError(k)
