"""Continuous-batching serving loop for thin-film simulation jobs.

Jobs (a canvas, a step count, a precision) arrive open-loop by a Poisson
process.  Each tick of the loop:
  1. admits arrived jobs in arrival order while their device bytes
     (cf_film_bytes) fit the HBM budget: the job's film is created and its
     initial state cloned on the device from a resident template canvas
     (cf_clone_state, no host round trip);
  2. steps every resident job by one frame in one batch (cf_batch_step: one
     launch per dispatch over all their tiles, replayed from a CUDA graph
     while the mix is unchanged);
  3. retires jobs that reached their step count (state kept resident until
     then; the batch is rebuilt when the mix changes).
Reported: per-step latency p50/p99 (each job's step times), queue wait
p50/p99, and aggregate Gcell-updates/s; `plain_sequential` runs the same jobs
one at a time with single-film launches for the comparison.

Step definition: a fixed dt of 1e-3 s with one substep per frame (the
fixed-dt canvases of the film pass, all tiles active).
"""
import argparse
import dataclasses
import json
import math
import time
from collections import deque

import numpy as np

from . import capi, synth
from .film import Batch, Film

DT = 1e-3


@dataclasses.dataclass
class Job:
    jid: int
    side: int
    steps: int
    precision: int
    template: int        # index into the template pool
    arrival: float       # seconds after the start
    admit: float = math.nan
    finish: float = math.nan
    steps_done: int = 0
    nbytes: int = 0
    film: object = None
    step_ms: list = dataclasses.field(default_factory=list)


def template_canvas(side, seed):
    """A seeded blob field (centres uniform, sigma 5-40 cells, peak 0.1-2 mm,
    Dirichlet(0.5) pigments, per-blob rheology), 20 blobs per 512^2."""
    n_blobs = int(min(max(round(20 * (side / 512.0) ** 2), 4), 500))
    cv = synth.blob_canvas(side, side, seed, n_blobs=n_blobs)
    cv.settings["all_active"] = 1
    return cv


def make_settings(cv):
    return capi.Settings.default(**cv.settings)


class TemplatePool:
    """Resident template films, one per (side, precision): admission clones
    them.  Their bytes are outside the serving budget."""

    def __init__(self, sides, seed=0):
        self.sides = list(sides)
        self.canvases = [template_canvas(s, seed + k) for k, s in enumerate(self.sides)]
        self.films = {}

    def film(self, k, precision):
        key = (k, precision)
        if key not in self.films:
            cv = self.canvases[k]
            f = Film(make_settings(cv), cv.w, cv.h, precision)
            f.set_tables(cv.pigtab, cv.cmf)
            f.write_state(cv.planes)
            f.update_params(DT, 1)
            self.films[key] = f
        return self.films[key]

    def close(self):
        for f in self.films.values():
            f.close()
        self.films = {}


def poisson_jobs(duration_s, rate, pool, steps=(100, 3000), seed=1, steps_scale=1.0,
                 precisions=(capi.CF_PREC_FP32, capi.CF_PREC_BF16)):
    """Arrivals of a Poisson process of `rate` jobs/s over `duration_s`: side
    from the pool (log-spaced), steps uniform, precision 50/50."""
    rng = np.random.Generator(np.random.PCG64(seed))
    jobs, t = [], 0.0
    while True:
        t += rng.exponential(1.0 / rate)
        if t > duration_s:
            break
        k = int(rng.integers(0, len(pool.sides)))
        n = int(rng.integers(steps[0], steps[1] + 1))
        n = max(1, int(round(n * steps_scale)))
        prec = precisions[int(rng.integers(0, len(precisions)))]
        jobs.append(Job(len(jobs), pool.sides[k], n, prec, k, t))
    return jobs


def _pct(xs, q):
    return float(np.percentile(np.asarray(xs, np.float64), q)) if len(xs) else math.nan


class Server:
    """Films of retired jobs are kept per (side, precision) and reused by the
    next job of that shape: admission is then a device-side clone into an
    existing arena.  Idle films count against the budget and are freed when a
    job of another shape needs the room."""

    def __init__(self, pool, budget_bytes, tuning=None, keep=None):
        self.pool = pool
        self.budget = int(budget_bytes)
        self.batch = Batch()
        if tuning:
            self.batch.tuning = tuning
        self.keep = set(keep or ())   # job ids whose final state is read back
        self.results = {}
        self.idle = {}                # (side, precision) -> [Film]
        self.idle_bytes = 0

    def fits(self, job, used):
        """Whether the job can be admitted now (freeing idle films if needed)."""
        key = (job.side, job.precision)
        if self.idle.get(key):
            return True
        while used + self.idle_bytes + job.nbytes > self.budget and self.idle_bytes > 0:
            k = max((k for k in self.idle if self.idle[k]), key=lambda k: capi.film_bytes(k[0], k[0], k[1]))
            self.idle[k].pop().close()
            self.idle_bytes -= capi.film_bytes(k[0], k[0], k[1])
        return used + self.idle_bytes + job.nbytes <= self.budget

    def admit(self, job, now):
        src = self.pool.film(job.template, job.precision)
        key = (job.side, job.precision)
        if self.idle.get(key):
            f = self.idle[key].pop()
            self.idle_bytes -= job.nbytes
        else:
            f = Film(src.settings, src.w, src.h, job.precision)
        f.clone_from(src)
        job.film = f
        job.admit = now
        self.batch.add(f)

    def retire(self, job, now):
        job.finish = now
        if job.jid in self.keep:
            st = job.film.read_state()
            st["color"] = job.film.color()
            self.results[job.jid] = st
        self.batch.remove(job.film)
        self.idle.setdefault((job.side, job.precision), []).append(job.film)
        self.idle_bytes += job.nbytes
        job.film = None

    def run(self, jobs, max_wall_s=None):
        """Serves `jobs` (sorted by arrival) in real time; returns a report."""
        pending = deque(sorted(jobs, key=lambda j: j.arrival))
        for j in pending:
            j.nbytes = capi.film_bytes(j.side, j.side, j.precision)
        pending = deque(j for j in pending if j.nbytes <= self.budget)
        resident, done = [], []
        used = peak_used = peak_resident = 0
        admit_s = 0.0
        cell_steps = 0
        t0 = time.perf_counter()
        while pending or resident:
            now = time.perf_counter() - t0
            if max_wall_s is not None and now > max_wall_s:
                break
            ta = time.perf_counter()
            while pending and pending[0].arrival <= now and self.fits(pending[0], used):
                j = pending.popleft()
                self.admit(j, now)
                resident.append(j)
                used += j.nbytes
            admit_s += time.perf_counter() - ta
            peak_used = max(peak_used, used + self.idle_bytes)
            peak_resident = max(peak_resident, len(resident))
            if not resident:
                if pending:
                    time.sleep(max(0.0, min(pending[0].arrival - now, 0.01)))
                continue
            ts = time.perf_counter()
            self.batch.step(1, 1)
            resident[0].film.sync()
            step_ms = (time.perf_counter() - ts) * 1e3
            now = time.perf_counter() - t0
            still = []
            for j in resident:
                j.step_ms.append(step_ms)
                j.steps_done += 1
                cell_steps += j.side * j.side
                if j.steps_done >= j.steps:
                    self.retire(j, now)
                    used -= j.nbytes
                    done.append(j)
                else:
                    still.append(j)
            resident = still
        wall = time.perf_counter() - t0
        for j in resident:  # cut off by max_wall_s
            self.retire(j, wall)
        served = done + resident
        steps = [x for j in served for x in j.step_ms]
        waits = [j.admit - j.arrival for j in served if not math.isnan(j.admit)]
        return {
            "jobs_arrived": len(jobs), "jobs_done": len(done), "jobs_admitted": len(served),
            "step_ms_p50": _pct(steps, 50), "step_ms_p99": _pct(steps, 99),
            "queue_wait_s_p50": _pct(waits, 50), "queue_wait_s_p99": _pct(waits, 99),
            "gcell_updates_per_s": cell_steps / wall / 1e9, "cell_steps": cell_steps, "wall_s": wall,
            "admission_s": admit_s, "peak_resident_jobs": peak_resident, "peak_bytes": peak_used,
            "budget_bytes": self.budget,
        }

    def close(self):
        self.batch.close()
        for fs in self.idle.values():
            for f in fs:
                f.close()
        self.idle, self.idle_bytes = {}, 0


def plain_sequential(jobs, pool, budget_s=None):
    """The same jobs one at a time in arrival order, each with single-film
    launches (cf_encode_frame per step); Gcell-updates/s over the stepping.
    With budget_s, stops once that much stepping time is spent (the last job
    may be cut short)."""
    cell_steps, busy, njobs = 0, 0.0, 0
    for j in sorted(jobs, key=lambda j: j.arrival):
        src = pool.film(j.template, j.precision)
        f = Film(src.settings, src.w, src.h, j.precision)
        f.clone_from(src)
        f.sync()
        t = time.perf_counter()
        done = 0
        while done < j.steps:
            k = min(16, j.steps - done)
            for _ in range(k):
                f.encode_frame(1)
            done += k
            if budget_s is not None and busy + time.perf_counter() - t > budget_s:
                break
        f.sync()
        busy += time.perf_counter() - t
        cell_steps += j.side * j.side * done
        njobs += 1
        f.close()
        if budget_s is not None and busy > budget_s:
            break
    return {"gcell_updates_per_s": cell_steps / max(busy, 1e-12) / 1e9, "cell_steps": cell_steps, "busy_s": busy,
            "jobs": njobs}


def main():
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--duration", type=float, default=60.0, help="arrival window (s)")
    ap.add_argument("--rate", type=float, default=20.0, help="arrivals per second")
    ap.add_argument("--budget-gb", type=float, default=150.0)
    ap.add_argument("--steps-scale", type=float, default=1.0, help="scales the 100-3000 step range")
    ap.add_argument("--sides", default="256,368,528,768,1104,1584,2048")
    ap.add_argument("--max-wall", type=float, default=None)
    ap.add_argument("--sequential-seconds", type=float, default=30.0)
    args = ap.parse_args()
    pool = TemplatePool([int(s) for s in args.sides.split(",")])
    jobs = poisson_jobs(args.duration, args.rate, pool, steps_scale=args.steps_scale)
    srv = Server(pool, args.budget_gb * 1e9)
    rep = srv.run(jobs, args.max_wall)
    srv.close()
    seq = plain_sequential(jobs, pool, args.sequential_seconds)
    rep["plain_sequential_gcell_updates_per_s"] = seq["gcell_updates_per_s"]
    pool.close()
    print(json.dumps(rep))


if __name__ == "__main__":
    main()
