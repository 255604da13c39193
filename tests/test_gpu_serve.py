"""The continuous-batching serving loop (GPU).

Jobs arrive, join the batch as memory allows, step together and leave.  Each
job's final state in the mix must equal, bit for bit, the same job stepped
alone (the batch runs the same compiled kernels as a film alone), and
admission must keep the resident bytes within the budget.
"""
import numpy as np
import pytest

from canvaz_film import capi, serve

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def built():
    import __graft_entry__ as g
    g.build()
    return True


@pytest.fixture(scope="module")
def pool(built):
    p = serve.TemplatePool([48, 64, 80], seed=3)
    yield p
    p.close()


def alone(pool, job):
    from canvaz_film.film import Film
    src = pool.film(job.template, job.precision)
    f = Film(src.settings, src.w, src.h, job.precision)
    f.clone_from(src)
    for _ in range(job.steps):
        f.encode_frame(1)
    st = f.read_state()
    st["color"] = f.color()
    f.close()
    return st


def test_results_equal_alone_and_in_the_mix(pool):
    jobs = serve.poisson_jobs(0.05, 400.0, pool, steps=(3, 9), seed=5)
    assert len(jobs) >= 8
    keep = [j.jid for j in jobs[:5]]
    srv = serve.Server(pool, 1e12, keep=keep)
    rep = srv.run(jobs)
    srv.close()
    assert rep["jobs_done"] == len(jobs)
    assert rep["peak_resident_jobs"] >= 2
    assert rep["step_ms_p99"] >= rep["step_ms_p50"] > 0
    for j in jobs[:5]:
        want = alone(pool, j)
        got = srv.results[j.jid]
        for k in want:
            assert np.array_equal(got[k], want[k], equal_nan=True), "job %d plane %s" % (j.jid, k)


def test_admission_keeps_within_budget(pool):
    jobs = serve.poisson_jobs(0.05, 400.0, pool, steps=(2, 5), seed=9)
    big = max(capi.film_bytes(j.side, j.side, j.precision) for j in jobs)
    budget = int(2.5 * big)
    srv = serve.Server(pool, budget)
    rep = srv.run(jobs)
    srv.close()
    assert rep["jobs_done"] == len(jobs)
    assert rep["peak_bytes"] <= budget
    assert rep["queue_wait_s_p99"] >= 0
