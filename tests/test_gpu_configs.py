"""The named workloads at their own sizes, against the FP64 oracle (GPU).

Each check prints max |error|, RMS error and relative L2 per field (h, the
flow h - h0, m, strata thicknesses, per-cell pigment volume, mu, tau_y,
colour) and asserts the height bound of the target (relative L2 <= 1e-5
against FP64) with the branch-robust pigment / colour bounds of
tests/parity.py:
 - the 512 x 512 FP32 blob field (20 Gaussian blobs, sigma 5-40 cells, peak
   0.1-2 mm, per-blob Bingham / power-law rheology, Dirichlet(0.5) pigments,
   K and S over 8 bands), fixed dt 1e-3 s, the stated 200 steps;
 - the 2048 x 2048 tilted drip field (200 polylines), adaptive steps (a
   bounded number here; the 1000-step mass drift is its own test);
 - the 4096 x 4096 field of 500 blobs over a cured ground: the FP32 film and
   the BF16-storage film against FP64, and BF16 against the FP32-everywhere
   film, a few steps at full size (the field sits near its yield stress; the
   cells that flow are checked to exist, and the flow h - h0 is compared, so
   the comparison covers the flux).
The oracle runs on the host's cores (OpenMP).
"""
import os

import numpy as np
import pytest

import fieldcmp
import parity
import pyoracle as po
from canvaz_film import capi, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def built():
    import __graft_entry__ as g
    g.build()
    return True


def film_for(cv, prec):
    from canvaz_film.film import Film
    f = Film(capi.Settings.default(**cv.settings), cv.w, cv.h, prec)
    f.set_tables(cv.pigtab, cv.cmf)
    f.write_state(cv.planes, pig_format=capi.CF_PIG_F32)
    return f


def oracle_for(cv, bits=64):
    o = po.Oracle(cv.w, cv.h, po.make_settings(cv.settings), capi.CF_PIG_F32, bits)
    o.set_tables(cv.pigtab, cv.cmf)
    o.write_state(cv.planes)
    return o


def parity_metrics(f, o):
    s = f.read_state()
    got = {"h": s["h"], "m": s["m"], "strata_h": s["strata_h"], "strata_pig": s["strata_pig"], "color": f.color()}
    return parity.metrics(got, {k: o.buf(k) for k in ("h", "m", "strata_h", "strata_pig", "color")})


def fixed_dt(cv, steps, films, oracle):
    for f in films:
        f.update_params(1e-3, 1)
    oracle.update_params(1e-3, 1)
    for _ in range(steps):
        for f in films:
            f.encode_frame(1)
        oracle.encode_frame(1)
    for f in films:
        f.sync()


def host_memory_bytes():
    """Memory this process may use: the smaller of physical memory and the
    cgroup limit, where one is set."""
    mem = os.sysconf("SC_PAGE_SIZE") * os.sysconf("SC_PHYS_PAGES")
    for p in ("/sys/fs/cgroup/memory.max", "/sys/fs/cgroup/memory/memory.limit_in_bytes"):
        try:
            v = open(p).read().strip()
            if v.isdigit():
                mem = min(mem, int(v))
        except OSError:
            pass
    return mem


def flow_bound(mirror_rows):
    """The flow h - h0 of a few steps is a few f32 steps of h per cell, so its
    error is set by storing h in f32: the CUDA film's flow error is bounded by
    twice the oracle's own FP32 mirror's (plus 1e-6)."""
    return 2.0 * mirror_rows["flow h - h0"][2] + 1e-6


def test_blobs512_fp32_200_steps_vs_fp64(built):
    cv = synth.config(0, 0)
    cv.settings["all_active"] = 1
    h0 = cv.planes["h"].copy()
    o = oracle_for(cv)
    o32 = oracle_for(cv, 32)
    f = film_for(cv, capi.CF_PREC_FP32)
    fixed_dt(cv, 200, [f], o)
    fixed_dt(cv, 200, [], o32)
    ref = fieldcmp.fields_oracle(o, h0)
    rows = fieldcmp.compare(fieldcmp.fields_gpu(f, h0), ref)
    mrows = fieldcmp.compare(fieldcmp.fields_oracle(o32, h0), ref)
    fieldcmp.table(rows, "512x512 blobs, FP32, 200 steps of dt 1e-3 s: CUDA vs FP64 oracle")
    fieldcmp.table(mrows, "512x512 blobs, FP32, 200 steps: the oracle's FP32 mirror vs FP64 oracle (for scale)")
    assert rows["h"][2] <= parity.H_REL_L2
    assert rows["flow h - h0"][2] <= flow_bound(mrows)
    parity.check(parity_metrics(f, o))


def test_drips2048_adaptive_vs_fp64(built):
    cv = synth.config(1, 0)
    cv.settings["all_active"] = 1
    h0 = cv.planes["h"].copy()
    o = oracle_for(cv)
    f = film_for(cv, capi.CF_PREC_FP32)
    dts = []
    for _ in range(8):
        f.step_adaptive(1.0 / 60.0)
        dts.append(o.step_adaptive(1.0 / 60.0))
    f.sync()
    rows = fieldcmp.compare(fieldcmp.fields_gpu(f, h0), fieldcmp.fields_oracle(o, h0))
    fieldcmp.table(rows, "2048x2048 tilted drips, FP32, 8 adaptive steps (dt %.3e .. %.3e s): CUDA vs FP64 oracle"
                   % (min(dts), max(dts)))
    assert abs(f.stats()["last_dt"] - dts[-1]) <= 1e-6 * dts[-1]
    assert rows["h"][2] <= parity.H_REL_L2
    parity.check(parity_metrics(f, o))


def test_blobs4096_fp32_and_bf16_vs_fp64(built):
    # the FP64 oracle holds about 1.7 kB per cell on the host (28 GB at
    # 4096^2) and its FP32 mirror about half that
    scale = 1 if host_memory_bytes() > 100e9 else 2
    cv = synth.config(2, 0, scale=scale)
    cv.settings["all_active"] = 1
    h0 = cv.planes["h"].copy()
    o = oracle_for(cv)
    o32 = oracle_for(cv, 32)
    a = film_for(cv, capi.CF_PREC_FP32)
    b = film_for(cv, capi.CF_PREC_BF16)
    steps = 3
    fixed_dt(cv, steps, [a, b], o)
    fixed_dt(cv, steps, [], o32)
    ref = fieldcmp.fields_oracle(o, h0)
    fa, fb = fieldcmp.fields_gpu(a, h0), fieldcmp.fields_gpu(b, h0)
    side = "%dx%d" % (cv.w, cv.h)
    ra = fieldcmp.compare(fa, ref)
    rb = fieldcmp.compare(fb, ref)
    rab = fieldcmp.compare(fb, fa)
    mrows = fieldcmp.compare(fieldcmp.fields_oracle(o32, h0), ref)
    del o32
    fieldcmp.table(ra, "%s cured-ground blobs, %d steps: CUDA FP32 vs FP64 oracle" % (side, steps))
    fieldcmp.table(mrows, "%s cured-ground blobs, %d steps: the oracle's FP32 mirror vs FP64 oracle (for scale)"
                   % (side, steps))
    fieldcmp.table(rb, "%s cured-ground blobs, %d steps: CUDA BF16 pigments + rheology vs FP64 oracle"
                   % (side, steps))
    fieldcmp.table(rab, "%s cured-ground blobs, %d steps: CUDA BF16 vs CUDA FP32-everywhere" % (side, steps))
    # the blobs sit at their yield stress: a few thousand cells move in a few
    # steps, and their flow is compared through "flow h - h0"
    flowing = np.count_nonzero(np.abs(ref["flow h - h0"]) > 1e-9)
    print("cells whose height moved by more than 1 nm: %d of %d" % (flowing, cv.w * cv.h))
    assert flowing >= 1000
    assert ra["h"][2] <= parity.H_REL_L2
    assert ra["flow h - h0"][2] <= flow_bound(mrows)
    assert rb["h"][2] <= parity.H_REL_L2
    assert rb["mu"][2] <= 4e-3          # mu stored in bfloat16 (slot 14 as mu)
    parity.check(parity_metrics(a, o))


def test_drips2048_mass_drift_1000_adaptive_steps(built):
    cv = synth.config(1, 0)
    cv.settings["all_active"] = 1
    f = film_for(cv, capi.CF_PREC_FP32)
    s0 = f.stats()
    for _ in range(1000):
        f.step_adaptive(1.0 / 60.0)
    s1 = f.stats()
    m0 = s0["wet_volume"] + s0["relief_volume"]
    m1 = s1["wet_volume"] + s1["relief_volume"]
    drift = abs(m1 - m0) / m0
    print("2048^2 drips, 1000 adaptive steps: mass drift %.3e, nan cells %d" % (drift, s1["nan_cells"]))
    assert s1["nan_cells"] == 0
    assert drift <= 1e-6


def test_blobs4096_bf16_tracks_fp32_1000_steps(built):
    cv = synth.config(2, 0)
    cv.settings["all_active"] = 1
    a = film_for(cv, capi.CF_PREC_FP32)
    b = film_for(cv, capi.CF_PREC_BF16)
    for f in (a, b):
        f.update_params(1e-3, 1)
        for _ in range(1000):
            f.encode_frame(1)
        f.sync()
    rows = fieldcmp.compare(fieldcmp.fields_gpu(b), fieldcmp.fields_gpu(a))
    fieldcmp.table(rows, "4096x4096 cured-ground blobs, 1000 steps: CUDA BF16 vs CUDA FP32-everywhere")
    assert rows["h"][2] < 1e-5
    assert rows["mu"][2] < 4e-3
    assert rows["pigment volume"][2] < 1e-2
