"""The implicit hydrostatic steps (film.wgsl:895-1302) on the GPU.

The frames of thick, runny paint (implicit_hydro on, so update_params picks
1-4 CG steps per frame) against the FP64 oracle, whose CG restatement equals
the translated shaders exactly (tests/golden/implicit_pour.npz); a batch
against the same films stepped alone; the adaptive step; the CG's mass
rescale; the clone guard.
"""
import numpy as np
import pytest

import parity
import pyoracle as po
from canvaz_film import capi, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def built():
    import __graft_entry__ as g
    g.build()
    return True


def pour(w=96, h=80, seed=29):
    cv = synth.blob_canvas(w, h, seed, n_blobs=6, sigma=(4, 10), per_cell_n=False, tables="reference",
                           tau=(0.0, 0.3), mu=(0.05, 0.2), peak_mm=(3.0, 5.0))
    cv.settings.update(implicit_hydro=1)
    return cv


def planes_of(x):
    return {k: x.buf(k) for k in ("h", "m", "strata_h", "strata_pig", "color")}


def state_of(f):
    s = f.read_state()
    return {"h": s["h"], "m": s["m"], "strata_h": s["strata_h"], "strata_pig": s["strata_pig"], "color": f.color()}


@pytest.mark.parametrize("prec,size", [(capi.CF_PREC_REFERENCE, (96, 80)), (capi.CF_PREC_FP32, (96, 80)),
                                       (capi.CF_PREC_FP32, (70, 45))])
def test_implicit_frames_vs_fp64_oracle(built, prec, size):
    """Bound on h: 1e-5, or 1.5x the FP32 mirror's own distance from FP64.
    70 x 45 leaves partial tiles on the right and top edges."""
    from canvaz_film.film import Film
    cv = pour(*size)
    st = po.make_settings(cv.settings)
    pig_mode = capi.PREC_TO_PIG[prec]
    o = po.Oracle(cv.w, cv.h, st, pig_mode, 64)
    o32 = po.Oracle(cv.w, cv.h, st, pig_mode, 32)
    f = Film(st, cv.w, cv.h, prec)
    for x in (o, o32, f):
        x.set_tables(cv.pigtab, cv.cmf)
        x.write_state(cv.planes)
    steps = []
    for fr in range(4):
        n = o.choose_substeps(1 / 60)
        for x in (o, o32, f):
            x.update_params(1 / 60, n)
        steps.append(o.implicit_steps())
        for x in (o, o32, f):
            x.encode_frame(n)
        f.sync()
    assert max(steps) > 0, steps  # the CG ran
    m = parity.metrics(state_of(f), planes_of(o))
    m32 = parity.metrics(planes_of(o32), planes_of(o))
    print(prec, steps, m, "fp32 mirror", m32)
    parity.check(m, h_rel=max(parity.H_REL_L2, 1.5 * m32["h_rel_l2"]))
    assert m["mass_rel"] <= parity.MASS_REL


def test_implicit_changes_the_frame(built):
    """The same frames with implicit_hydro off differ (the CG does work)."""
    from canvaz_film.film import Film
    cv = pour(64, 48, 7)
    out = []
    for imp in (1, 0):
        cv.settings.update(implicit_hydro=imp)
        f = Film(po.make_settings(cv.settings), cv.w, cv.h, capi.CF_PREC_FP32)
        f.set_tables(cv.pigtab, cv.cmf)
        f.write_state(cv.planes)
        for _ in range(2):
            f.update_params(1 / 60, 16)
            f.encode_frame(16)
        f.sync()
        out.append(f.read_state()["h"].astype(np.float64))
    assert parity.rel_l2(out[0], out[1]) > 1e-3


@pytest.mark.parametrize("graph", [0, 1])
def test_implicit_batch_equals_alone(built, graph):
    from canvaz_film.film import Batch, Film
    cvs = [pour(64, 48, 3), pour(80, 64, 4)]
    cvs.append(synth.blob_canvas(48, 48, 5, n_blobs=4, tables="reference"))  # implicit off in the same batch
    alone, batched = [], []
    for cv in cvs:
        for lst in (alone, batched):
            f = Film(po.make_settings(cv.settings), cv.w, cv.h, capi.CF_PREC_FP32)
            f.set_tables(cv.pigtab, cv.cmf)
            f.write_state(cv.planes)
            f.update_params(1 / 60, 8)
            lst.append(f)
    b = Batch()
    for f in batched:
        b.add(f)
    b.tuning = {"list_blocks_per_sm": 8, "use_graph": graph, "frames_per_graph": 1}
    for _ in range(3):
        for f in alone:
            f.encode_frame(8)
        b.step(1, 8)
    for fa, fb in zip(alone, batched):
        fa.sync()
        fb.sync()
        sa, sb = fa.read_state(), fb.read_state()
        for k in sa:
            assert np.array_equal(np.asarray(sa[k]).view(np.uint8), np.asarray(sb[k]).view(np.uint8)), k


def test_implicit_adaptive_batch_equals_alone(built):
    """dt chosen on the device: the launches cover 4 implicit steps and each
    film skips the ones it does not take; batched equals alone, bit for bit."""
    from canvaz_film.film import Batch, Film
    cvs = [pour(64, 48, 21), pour(50, 37, 22)]
    alone, batched = [], []
    for cv in cvs:
        for lst in (alone, batched):
            f = Film(po.make_settings(cv.settings), cv.w, cv.h, capi.CF_PREC_FP32)
            f.set_tables(cv.pigtab, cv.cmf)
            f.write_state(cv.planes)
            lst.append(f)
    b = Batch()
    for f in batched:
        b.add(f)
    b.tuning = {"list_blocks_per_sm": 8, "use_graph": 1, "frames_per_graph": 2}
    for _ in range(3):
        for f in alone:
            f.step_adaptive(1 / 60)
            f.step_adaptive(1 / 60)
        b.step(2, 1, 1 / 60)
    for fa, fb in zip(alone, batched):
        fa.sync()
        fb.sync()
        sa, sb = fa.read_state(), fb.read_state()
        for k in sa:
            assert np.array_equal(np.asarray(sa[k]).view(np.uint8), np.asarray(sb[k]).view(np.uint8)), k


def test_implicit_adaptive_vs_oracle(built):
    from canvaz_film.film import Film
    cv = pour(64, 64, 11)
    st = po.make_settings(cv.settings)
    o = po.Oracle(cv.w, cv.h, st, 0, 64)
    o32 = po.Oracle(cv.w, cv.h, st, 0, 32)
    f = Film(st, cv.w, cv.h, capi.CF_PREC_REFERENCE)
    for x in (o, o32, f):
        x.set_tables(cv.pigtab, cv.cmf)
        x.write_state(cv.planes)
    for _ in range(20):
        for x in (o, o32):
            x.step_adaptive(1 / 60)
        f.step_adaptive(1 / 60)
    f.sync()
    m = parity.metrics(state_of(f), planes_of(o))
    m32 = parity.metrics(planes_of(o32), planes_of(o))
    print(m, "fp32 mirror", m32)
    parity.check(m, h_rel=max(parity.H_REL_L2, 1.5 * m32["h_rel_l2"]))


def test_implicit_mass_and_clone_guard(built):
    from canvaz_film.film import Film
    cv = pour(64, 64, 13)
    st = po.make_settings(cv.settings)
    f = Film(st, cv.w, cv.h, capi.CF_PREC_FP32)
    f.set_tables(cv.pigtab, cv.cmf)
    f.write_state(cv.planes)
    s0 = f.stats()
    for _ in range(5):
        f.update_params(1 / 60, 16)
        f.encode_frame(16)
    s1 = f.stats()
    m0 = s0["wet_volume"] + s0["relief_volume"]
    m1 = s1["wet_volume"] + s1["relief_volume"]
    assert abs(m1 - m0) / m0 < 1e-5, (m0, m1)
    cv.settings.update(implicit_hydro=0)
    g = Film(po.make_settings(cv.settings), cv.w, cv.h, capi.CF_PREC_FP32)
    with pytest.raises(capi.FilmError):
        g.clone_from(f)
