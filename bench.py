#!/usr/bin/env python
"""Benchmark of the GB300 thin-film step (one JSON line on rank 0).

Workload (default): a 4096 x 4096 FP32 canvas (1 mm cells) seeded with 500
Gaussian paint blobs (sigma 5-40 cells, peak 0.1-2 mm, per-blob
Herschel-Bulkley rheology and Dirichlet(0.5) pigments) over a 0.05 mm cured
ground layer, stepped at a fixed dt of 1e-3 s (one substep per frame).  One
step = one frame of film + strata/pigment transport + cure + KM shade
(cf_encode_frame), every 16x16 tile active.  The state (13.7 GB) is far larger
than L2, so no flush is needed between steps.  The same canvas with BF16
pigment and rheology storage is timed too and reported inside the line
("bf16").

Arms:
  --impl gb300 (default): the CUDA library through its C ABI.  `value` is
      device throughput with the state resident in HBM (CUDA events on the
      stream the kernels run on); `e2e` goes through the same C ABI with host
      buffers: every timed step uploads the full state from pinned host
      memory (cf_write_state_async), steps, and reads back h and the colour
      image; two films alternate on two streams, so one film's upload over
      the host link overlaps the other's step.
  --impl reference: the reference path on the host cores (the reference's
      own WGSL translated to C++ when oracle/_ref is built here, else the
      oracle's FP32 restatement), OpenMP over rows on all cores.
Multi-GPU: one replica canvas per rank (independent canvases; no collective
on the data path), `value` = all ranks' cell-updates / max time.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
for _p in (ROOT / "paint-sim-3d_gb300", ROOT / "oracle"):
    if str(_p) not in sys.path:
        sys.path.insert(0, str(_p))

from canvaz_film import capi, synth  # noqa: E402

WORKLOADS = {
    # name: (generator, precision, dt_max, adaptive)
    "drips2048_tilt60_fp32": (lambda seed: synth.config(1, seed), capi.CF_PREC_FP32, 1.0 / 60.0, True),
    # the same field at half the side (50 lines): small case for kernel captures
    "drips1024_tilt60_fp32": (lambda seed: synth.config(1, seed, scale=2), capi.CF_PREC_FP32, 1.0 / 60.0, True),
    "blobs512_dt1e-3_fp32": (lambda seed: synth.config(0, seed), capi.CF_PREC_FP32, 1e-3, False),
    "blobs4096_dt1e-3_bf16": (lambda seed: synth.config(2, seed), capi.CF_PREC_BF16, 1e-3, False),
    "blobs4096_dt1e-3_fp32": (lambda seed: synth.config(2, seed), capi.CF_PREC_FP32, 1e-3, False),
    # the same field at a quarter of the side (31 blobs): small case for kernel captures
    "blobs1024_dt1e-3_fp32": (lambda seed: synth.config(2, seed, scale=4), capi.CF_PREC_FP32, 1e-3, False),
    # at half the side: DRAM-traffic captures whose writes do not stay in L2
    "blobs2048_dt1e-3_fp32": (lambda seed: synth.config(2, seed, scale=2), capi.CF_PREC_FP32, 1e-3, False),
    # thick pours with the implicit hydrostatic CG steps (the reference's default), adaptive
    "pour2048_implicit_fp32": (lambda seed: synth.config(5, seed), capi.CF_PREC_FP32, 1.0 / 60.0, True),
    "pour512_implicit_fp32": (lambda seed: synth.config(5, seed, scale=4), capi.CF_PREC_FP32, 1.0 / 60.0, True),
}
DEFAULT_WORKLOAD = "blobs4096_dt1e-3_fp32"
# the storage variant timed beside a single-canvas workload in the same run
BF16_TWIN = {"blobs4096_dt1e-3_fp32": "blobs4096_dt1e-3_bf16"}

# Compulsory persistent-state bytes per cell-step (read once + write once):
# h 4R+4W, m 4R, rheo 3 fields R+W, delta 4R+4W, strata_h 16R+16W,
# strata_cure 16R+16W, strata_pig 64 slots R+W, sub_refl 16 f16 R, colour 8W.
ALG_BYTES_PER_CELL = {capi.CF_PREC_FP32: 660, capi.CF_PREC_REFERENCE: 404, capi.CF_PREC_BF16: 392}
PREC_NAME = {capi.CF_PREC_FP32: "f32", capi.CF_PREC_REFERENCE: "f32+f16pig", capi.CF_PREC_BF16: "f32+bf16pig"}


# Workloads with their own arm (not a single canvas): config 3, 64 uneven
# canvases stepped as one batch against 64 sequential single-film launches,
# and config 4, the Poisson-served stream.
BATCH_WORKLOAD = "batch64_dt1e-3_fp32"
SERVE_WORKLOAD = "serve_poisson20_fp32bf16"
# The deposit rasteriser alone: 4096 strokes per step onto a 4096^2 FP32 film
# (and the same density at 2048^2, the small case for kernel captures).
DEPOSIT_WORKLOADS = {"deposit4096_strokes4096_fp32": (4096, 4096), "deposit2048_strokes1024_fp32": (2048, 1024)}
DEPOSIT_WORKLOAD = "deposit4096_strokes4096_fp32"
# Compulsory bytes per cell that receives paint (FP32 storage): reads h, m,
# strata_h, strata_cure, 64 f32 pigment slots, 16 f16 substrate bands;
# writes h, strata_h, strata_cure, pigments, lay, the dry bit and the
# composition aggregates.
DEPOSIT_BYTES_PER_CELL = (4 + 4 + 16 + 16 + 256 + 32) + (4 + 16 + 16 + 256 + 4 + 1 + 16)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD,
                    choices=sorted(WORKLOADS) + [BATCH_WORKLOAD, SERVE_WORKLOAD, RELIEF_WORKLOAD, SNAPSHOT_WORKLOAD,
                                                 LIT_WORKLOAD]
                    + sorted(DEPOSIT_WORKLOADS))
    ap.add_argument("--serve-seconds", type=float, default=20.0, help="arrival window of the served workload")
    ap.add_argument("--serve-wall", type=float, default=60.0, help="wall-clock cut-off of the served run")
    ap.add_argument("--serve-steps-scale", type=float, default=1.0, help="scales the served 100-3000 step range")
    ap.add_argument("--e2e-steps", type=int, default=8)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=20.0, help="budget of the CPU baseline sample")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def step_traffic(workload):
    """DRAM bytes per cell-step of `workload` from the committed ncu summary
    (a line `dram_bytes_per_cell_step[<workload>]=<bytes>`), or None."""
    p = ROOT / "profiles" / "step_traffic.txt"
    if not p.exists():
        return None
    key = "dram_bytes_per_cell_step[%s]=" % workload
    for line in p.read_text().splitlines():
        if line.startswith(key):
            return float(line.split("=", 1)[1].split()[0])
    return None


class _Nvml:
    """Read-only NVML queries through ctypes (the driver's libnvidia-ml):
    SM clock, its maximum, power and the active clock-event reasons."""
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown",
               0x80: "hw_power_brake_slowdown"}

    def __init__(self, cuda_index):
        import ctypes as C
        self.C = C
        self.lib = C.CDLL("libnvidia-ml.so.1")
        if self.lib.nvmlInit_v2() != 0:
            raise OSError("nvmlInit failed")
        self.h = C.c_void_p()
        bus = None
        try:
            import torch
            pr = torch.cuda.get_device_properties(cuda_index)
            bus = ("%08x:%02x:%02x.0" % (pr.pci_domain_id, pr.pci_bus_id, pr.pci_device_id)).encode()
        except Exception:
            bus = None
        ok = bus is not None and self.lib.nvmlDeviceGetHandleByPciBusId_v2(bus, C.byref(self.h)) == 0
        if not ok and self.lib.nvmlDeviceGetHandleByIndex_v2(C.c_uint(cuda_index), C.byref(self.h)) != 0:
            raise OSError("no NVML handle")
        fn = getattr(self.lib, "nvmlDeviceGetCurrentClocksEventReasons", None)
        self.reasons_fn = fn if fn is not None else self.lib.nvmlDeviceGetCurrentClocksThrottleReasons

    def sample(self):
        C = self.C
        sm, mx, pw, rs = C.c_uint(), C.c_uint(), C.c_uint(), C.c_ulonglong()
        self.lib.nvmlDeviceGetClockInfo(self.h, 1, C.byref(sm))
        self.lib.nvmlDeviceGetMaxClockInfo(self.h, 1, C.byref(mx))
        self.lib.nvmlDeviceGetPowerUsage(self.h, C.byref(pw))
        self.reasons_fn(self.h, C.byref(rs))
        return float(sm.value), float(mx.value), pw.value / 1000.0, int(rs.value)


class Clocks:
    """Samples SM clocks and throttle reasons during a region: NVML every
    5 ms from a thread (read-only queries) where the driver library loads,
    else nvidia-smi every 200 ms.  mark(True) / mark(False) bracket the timed
    region; the summary keeps the samples inside it."""

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.nvml = None
        self.rows = []  # (t, sm, max, power_w, reasons set)
        self.t0 = self.t1 = None
        self.file = None
        try:
            self.nvml = _Nvml(gpu_index)
        except Exception:
            self.nvml = None

    def _run(self):
        while not self._stop.is_set():
            try:
                sm, mx, pw, rs = self.nvml.sample()
                self.rows.append((time.perf_counter(), sm, mx, pw,
                                  {n for b, n in _Nvml.REASONS.items() if rs & b}))
            except Exception:
                pass
            self._stop.wait(0.005)

    def __enter__(self):
        if self.nvml is not None:
            self._stop = threading.Event()
            self._th = threading.Thread(target=self._run, daemon=True)
            self._th.start()
            time.sleep(0.05)
            return self
        self.file = tempfile.NamedTemporaryFile(prefix="clocks_", suffix=".csv", delete=False)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.file, stderr=subprocess.DEVNULL)
        except FileNotFoundError:
            self.proc = None
        time.sleep(0.3)
        return self

    def mark(self, start):
        if start:
            self.t0 = time.perf_counter()
        else:
            self.t1 = time.perf_counter()

    def __exit__(self, *a):
        if self.nvml is not None:
            self._stop.set()
            self._th.join(2)
            return
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.nvml is not None:
            rows = self.rows
            if self.t0 is not None and self.t1 is not None:
                inside = [r for r in rows if self.t0 <= r[0] <= self.t1]
                rows = inside if inside else rows
            if not rows:
                return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
            reasons = set()
            for r in rows:
                reasons |= r[4]
            return {"sm_mhz": statistics.median(r[1] for r in rows), "sm_max_mhz": rows[0][2],
                    "reasons": sorted(reasons), "samples": len(rows), "source": "nvml 5 ms",
                    "power_w_median": statistics.median(r[3] for r in rows),
                    "timed_region_s": None if self.t0 is None or self.t1 is None else self.t1 - self.t0}
        rows = []
        if self.file is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        try:
            for line in Path(self.file.name).read_text().splitlines():
                f = [x.strip() for x in line.split(",")]
                if len(f) >= 9:
                    rows.append(f)
        finally:
            os.unlink(self.file.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for k, n in enumerate(names):
                if r[5 + k].lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": float(rows[0][2]) if rows else None,
                "reasons": sorted(reasons), "samples": len(rows), "source": "nvidia-smi 200 ms"}


def settings_for(cv):
    s = dict(cv.settings)
    s["all_active"] = 1
    return capi.Settings.default(**s)


def cpu_baseline(cv, workload, budget_s, steps_hint=3):
    """The oracle's FP32 restatement of the reference path on all host cores,
    on a bounded sample: the same canvas, as many whole steps as fit the
    budget (at least one)."""
    import pyoracle as po
    po.build()
    gen, prec, dt_max, adaptive = WORKLOADS[workload]
    pig = capi.PREC_TO_PIG[prec]
    o = po.Oracle(cv.w, cv.h, settings_for(cv), pig, 32)
    o.set_tables(cv.pigtab, cv.cmf)
    o.write_state(cv.planes)
    t0 = time.perf_counter()
    n = 0
    while True:
        if adaptive:
            o.step_adaptive(dt_max)
        else:
            o.update_params(dt_max, 1)
            o.encode_frame(1)
        n += 1
        el = time.perf_counter() - t0
        if n >= steps_hint or el > budget_s or (el / n) * (n + 1) > budget_s:
            break
    el = time.perf_counter() - t0
    return {"value": cv.w * cv.h * n / el / 1e9, "unit": "Gcell-updates/s", "cores": os.cpu_count(),
            "kind": "port", "sample": "%d whole step(s) of the %dx%d workload, FP32 oracle restatement, OpenMP %d threads, %.1f s"
            % (n, cv.w, cv.h, os.cpu_count(), el)}


def deposit_strokes(n, side_m, dx, seed):
    """n strokes / capsules (radius 1.5-6 cells, length 0-40 cells, random
    pigments and laying method) built by the library's Deposit constructors."""
    from canvaz_film import deposit as dep
    rng = np.random.default_rng(seed)
    a = rng.uniform(0.01, 0.99, (n, 2)) * side_m
    ang = rng.uniform(0, 2 * np.pi, n)
    ln = rng.uniform(0, 40, n) * dx
    b = a + ln[:, None] * np.stack([np.cos(ang), np.sin(ang)], 1)
    r = rng.uniform(1.5, 6.0, n) * dx
    pig = np.zeros((n, 16))
    pig[:, :12] = rng.dirichlet(np.full(12, 0.5), n)
    pig[:, 13] = rng.uniform(0.5, 2.0, n)
    method = rng.integers(1, 7, n)
    out = np.zeros(n, dep.DEPOSIT_DTYPE)
    for k in range(n):
        vol = float(np.pi * r[k] * r[k] * (ln[k] + r[k]) * 0.3)
        ctor = dep.capsule if k % 3 == 0 else dep.stroke
        d = ctor(a[k], b[k], float(r[k]), vol, dep.pack_pig(pig[k]), float(dx))
        d["kind"] |= int(method[k]) << dep.METHOD_SHIFT
        out[k] = d
    return out


def tiles_touched(deps, side, dx):
    """Entries of the 64x64-cell tile lists a set of deposits makes (each
    deposit is listed in every tile its bounding box touches)."""
    rb = np.maximum(deps["r0"], deps["r1"])
    tile = 64 * float(dx)
    lo = np.floor((np.minimum(deps["p0"], deps["p1"]) - rb[:, None]) / tile).clip(0, side // 64 - 1)
    hi = np.floor((np.maximum(deps["p0"], deps["p1"]) + rb[:, None]) / tile).clip(0, side // 64 - 1)
    return int(np.prod(hi - lo + 1, axis=1).sum())


RELIEF_WORKLOAD = "relief2048_view3840x2160_fp32"


SNAPSHOT_WORKLOAD = "snapshot2048_fp32"
# the renderer's fragment shader over the film (cf_render_lit): a 1920 x 1080
# perspective view of the default drip canvas, the camera orbiting a little
# every frame
LIT_WORKLOAD = "lit2048_persp1920x1080_fp32"


def snapshot_arm(args):
    """Painting files of the default 2048^2 drip canvas after 5 adaptive steps:
    every step saves the film (cf_snapshot_save: read_state, 32 MiB chunks
    LZ4-compressed on all host threads) and loads the file into a second film
    (cf_snapshot_load).  `value` = GB/s of the 8 read_state planes (212 B per
    cell) saved and loaded; the CPU baseline decodes the same file's chunks
    with oracle/lz4_ref.py (pure Python, one core) on a bounded sample."""
    import torch
    from canvaz_film.film import Film
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if not capi.LIB_PATH.exists():
        import __graft_entry__ as g
        g.build()
    cv = synth.config(1, 0)
    st = settings_for(cv)
    films = []
    for _ in range(2):
        f = Film(st, cv.w, cv.h, capi.CF_PREC_REFERENCE)
        f.set_tables(cv.pigtab, cv.cmf)
        films.append(f)
    films[0].write_state(cv.planes)
    for _ in range(5):
        films[0].step_adaptive(1.0 / 60.0)
    raw = 212 * cv.w * cv.h
    for _ in range(args.warmup):
        films[1].load_snapshot(films[0].save_snapshot())
    with Clocks(local) as clk:
        t0 = time.perf_counter()
        size = 0
        for _ in range(args.steps):
            data = films[0].save_snapshot()
            films[1].load_snapshot(data)
            size = len(data)
        t = time.perf_counter() - t0
    cb = None
    if not args.no_cpu_baseline:
        import lz4_ref
        import struct
        t1 = time.perf_counter()
        done = 0
        off = 48  # header (44 B) and the part count
        plen, nch = struct.unpack_from("<QI", data, off)
        off += 12
        csz = struct.unpack_from("<Q", data, off)[0]
        chunk = data[off + 8: off + 8 + csz]
        while done == 0 or time.perf_counter() - t1 < min(args.cpu_seconds, 20.0):
            done += len(lz4_ref.decompress_size_prepended(chunk))
        el = time.perf_counter() - t1
        cb = {"value": done / el / 1e9, "unit": "GB/s", "cores": 1, "kind": "port",
              "sample": "decode of the file's first chunk (%d B raw) by oracle/lz4_ref.py, repeated for %.1f s"
                        % (done, el)}
    line = {"metric": "GB/s", "value": 2 * raw * args.steps / t / 1e9, "unit": "GB/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8",
            "data": "synthetic (the default drip canvas)",
            "config": {"workload": SNAPSHOT_WORKLOAD, "film": [cv.w, cv.h], "raw_bytes": raw, "file_bytes": size,
                       "ratio": raw / max(size, 1), "host_threads": os.cpu_count()},
            "roofline": None, "gpu_launches": None, "clocks": clk.summary(),
            "e2e": {"value": 2 * raw * args.steps / t / 1e9, "unit": "GB/s", "h2d_bytes_per_step": raw,
                    "d2h_bytes_per_step": raw, "steps": args.steps,
                    "path": "cf_snapshot_save + cf_snapshot_load (host coder, the film's planes over the link)"},
            "cpu_baseline": cb}
    print(json.dumps(line), flush=True)


def relief_cpu(film, cv, st, budget_s):
    """oracle/relief_ref.py (numpy, float64, one core) sampling the film (or,
    without a device, the canvas as generated) at random canvas points, as
    many batches of 200k as fit the budget."""
    import relief_ref as rr
    if film is not None:
        fs = film.read_state()
        hp, mp, col = fs["h"], fs["m"], film.color()
    else:  # no device: the canvas as generated, a flat grey (the sampling cost does not depend on it)
        hp, mp, col = cv.planes["h"], cv.planes["m"], np.full((cv.w * cv.h, 4), 0.5)
    R = rr.Relief(cv.w, cv.h, float(st.width_m), float(st.height_m), hp, mp, col)
    rng = np.random.default_rng(0)
    pts = np.stack([rng.uniform(0, float(st.width_m), 200000), rng.uniform(0, float(st.height_m), 200000)], 1)
    t0 = time.perf_counter()
    n = 0
    while n == 0 or time.perf_counter() - t0 < budget_s:
        R.sample(pts)
        n += len(pts)
    el = time.perf_counter() - t0
    return {"value": n / el / 1e6, "unit": "Mpixel/s", "cores": 1, "kind": "port",
            "sample": "%d points of the film through oracle/relief_ref.py (numpy, float64), %.1f s" % (n, el)}


def relief_arm(args):
    """The render pass's reading of the film: cf_render_relief of a 3840 x 2160
    top-down view of the default 2048^2 drip canvas (after 5 adaptive steps),
    4 pixels per 3 cells, the view panned every step.  `value` = output
    Mpixel/s of device time; `e2e` adds the read-back of each image."""
    import torch
    from canvaz_film.film import Film
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if not capi.LIB_PATH.exists():
        import __graft_entry__ as g
        g.build()
    cv = synth.config(1, 0)
    st = settings_for(cv)
    film = Film(st, cv.w, cv.h, capi.CF_PREC_FP32)
    film.set_tables(cv.pigtab, cv.cmf)
    film.write_state(cv.planes)
    for _ in range(5):
        film.step_adaptive(1.0 / 60.0)
    W, H = 3840, 2160
    pm = 0.75 * float(st.width_m) / cv.w
    img = torch.empty(W * H * 4, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.Stream()
    sh = stream.cuda_stream

    def view(k):
        return 0.02 * (k % 7) * float(st.width_m), 0.03 * (k % 5) * float(st.height_m)

    for k in range(args.warmup):
        film.render_relief(img.data_ptr(), *view(k), pm, W, H, stream=sh)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(local) as clk:
        clk.mark(True)
        e0.record(stream)
        for k in range(args.steps):
            film.render_relief(img.data_ptr(), *view(k), pm, W, H, stream=sh)
        e1.record(stream)
        torch.cuda.synchronize()
        clk.mark(False)
    t = e0.elapsed_time(e1) / 1e3
    value = W * H * args.steps / t / 1e6
    host = torch.empty(W * H * 4, dtype=torch.uint8).pin_memory()
    t0 = time.perf_counter()
    for k in range(max(args.e2e_steps, 1)):
        film.render_relief(img.data_ptr(), *view(k), pm, W, H, stream=sh)
        with torch.cuda.stream(stream):
            host.copy_(img, non_blocking=True)
        stream.synchronize()
    te = time.perf_counter() - t0
    peak, peak_kind = peaks()
    # compulsory bytes per output pixel: the 4 colour texels and 4 x 4 relief
    # cells it reads are shared by about 0.56 pixels per cell (4/3 px per
    # cell), so per pixel about (8 B colour + 8 B h, m) x 0.5625 read + 4 B written
    alg = 16 * 0.5625 + 4
    cb = None if args.no_cpu_baseline else relief_cpu(film, cv, st, min(args.cpu_seconds, 20.0))
    line = {"metric": "Mpixel/s", "value": value, "unit": "Mpixel/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (the default drip canvas)",
            "config": {"workload": RELIEF_WORKLOAD, "view": [W, H], "film": [cv.w, cv.h],
                       "pixel_m": pm, "l2": "the film's h, m and colour planes (67 MB) fit in L2"},
            "roofline": {"bound": "hbm", "achieved": alg * W * H * args.steps / t / 1e9, "peak": peak,
                         "unit": "GB/s", "frac": alg * W * H * args.steps / t / 1e9 / peak,
                         "peak_source": peak_kind, "alg_bytes_per_pixel": alg, "scope": "k_render_relief",
                         "traffic": None},
            "gpu_launches": args.steps, "clocks": clk.summary(),
            "e2e": {"value": W * H * max(args.e2e_steps, 1) / te / 1e6, "unit": "Mpixel/s", "h2d_bytes_per_step": 64,
                    "d2h_bytes_per_step": W * H * 4, "steps": max(args.e2e_steps, 1),
                    "path": "cf_render_relief + read back of the RGBA8 image"},
            "cpu_baseline": cb}
    print(json.dumps(line), flush=True)


def lit_film():
    """The default drip canvas after 5 adaptive steps, and the top of its relief."""
    from canvaz_film.film import Film
    cv = synth.config(1, 0)
    st = settings_for(cv)
    film = Film(st, cv.w, cv.h, capi.CF_PREC_FP32)
    film.set_tables(cv.pigtab, cv.cmf)
    film.write_state(cv.planes)
    for _ in range(5):
        film.step_adaptive(1.0 / 60.0)
    state = film.read_state()
    top = float(np.max(np.asarray(state["h"], np.float64) + np.asarray(state["m"], np.float64))) + 0.5e-3
    return cv, st, film, top


def lit_arm(args):
    """cf_render_lit of a 1920 x 1080 perspective view of the default 2048^2
    drip canvas, the orbit camera turning 0.02 rad a frame.  `value` = output
    Mpixel/s of device time; `e2e` adds the read-back of each RGBA8 image."""
    import torch
    from canvaz_film import camera
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if not capi.LIB_PATH.exists():
        import __graft_entry__ as g
        g.build()
    cv, st, film, top = lit_film()
    W, H = 1920, 1080
    cams = [camera.render_cam(cv.w, cv.h, float(st.width_m), float(st.height_m), top, yaw=0.6 + 0.02 * k,
                              aspect=W / H) for k in range(16)]
    img = torch.empty(W * H * 4, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.Stream()
    sh = stream.cuda_stream
    for k in range(args.warmup):
        film.render_lit(cams[k % 16], W, H, None, img.data_ptr(), stream=sh)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(local) as clk:
        clk.mark(True)
        e0.record(stream)
        for k in range(args.steps):
            film.render_lit(cams[k % 16], W, H, None, img.data_ptr(), stream=sh)
        e1.record(stream)
        torch.cuda.synchronize()
        clk.mark(False)
    t = e0.elapsed_time(e1) / 1e3
    value = W * H * args.steps / t / 1e6
    host = torch.empty(W * H * 4, dtype=torch.uint8).pin_memory()
    t0 = time.perf_counter()
    for k in range(max(args.e2e_steps, 1)):
        film.render_lit(cams[k % 16], W, H, None, img.data_ptr(), stream=sh)
        with torch.cuda.stream(stream):
            host.copy_(img, non_blocking=True)
        stream.synchronize()
    te = time.perf_counter() - t0
    peak, peak_kind = peaks()
    alg = 4.0  # the RGBA8 pixel written; the film's planes it samples (157 MB) are re-read from L2
    line = {"metric": "Mpixel/s", "value": value, "unit": "Mpixel/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (the default drip canvas)",
            "config": {"workload": LIT_WORKLOAD, "view": [W, H], "film": [cv.w, cv.h],
                       "l2": "the film's h, m, colour and detail planes (101 MB) fit in L2"},
            "roofline": {"bound": "hbm", "achieved": alg * W * H * args.steps / t / 1e9, "peak": peak,
                         "unit": "GB/s", "frac": alg * W * H * args.steps / t / 1e9 / peak,
                         "peak_source": peak_kind, "alg_bytes_per_pixel": alg, "scope": "k_render_lit",
                         "note": "bound by instruction issue (the march, micro-relief, shadow, occlusion and "
                                 "lobes per pixel), not by memory", "traffic": None},
            "gpu_launches": args.steps, "clocks": clk.summary(),
            "e2e": {"value": W * H * max(args.e2e_steps, 1) / te / 1e6, "unit": "Mpixel/s", "h2d_bytes_per_step": 304,
                    "d2h_bytes_per_step": W * H * 4, "steps": max(args.e2e_steps, 1),
                    "path": "cf_render_lit + read back of the RGBA8 image"},
            "cpu_baseline": None}
    print(json.dumps(line), flush=True)


DEPOSIT_SETS = 4
DEPOSIT_CPU_SIDE = 1024  # CPU sample: the same stroke density on a 1024^2 film


def deposit_cpu(workload, budget_s):
    """The oracle's FP32 deposit pass (run_deposit, OpenMP over rows) on a
    1024^2 film with the workload's stroke density (256 strokes per launch)."""
    side_w, count_w = DEPOSIT_WORKLOADS[workload]
    import pyoracle as po
    po.build()
    side = DEPOSIT_CPU_SIDE
    st = capi.Settings.default(width_m=side * 1e-3, height_m=side * 1e-3)
    cv = synth.blob_canvas(16, 16, 1, n_blobs=1, tables="reference")
    o = po.Oracle(side, side, st, capi.CF_PIG_F32, 32)
    o.set_tables(cv.pigtab, cv.cmf)
    n = count_w * side * side // (side_w * side_w)
    sets = [deposit_strokes(n, side * 1e-3, np.float32(1e-3), 100 + k) for k in range(2)]
    el, launches = 0.0, 0
    while True:
        o.upload_deposits(sets[launches % 2])
        t0 = time.perf_counter()
        o.run("deposit")
        el += time.perf_counter() - t0
        launches += 1
        if el > budget_s or launches >= 200:
            break
    return {"value": n * launches / el / 1e6, "unit": "Mdeposits/s", "cores": os.cpu_count(), "kind": "port",
            "sample": "%d launches of %d strokes on a %dx%d FP32 film (the %dx%d workload's stroke density), "
                      "oracle run_deposit, OpenMP %d threads, %.1f s" % (launches, n, side, side, side_w,
                                                                          side_w, os.cpu_count(), el)}


def deposit_arm(args):
    """The deposit rasteriser on one GPU: every step uploads one set of
    strokes (cf_upload_deposits: host binning + copies) and lays it
    (cf_lay_deposits).  `value` = strokes per second of device time (CUDA
    events around each launch); `e2e` = strokes per second of the whole
    upload + lay + cf_get_stats (device -> host) loop."""
    import torch
    from canvaz_film.film import Film
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if not capi.LIB_PATH.exists():
        import __graft_entry__ as g
        g.build()
    side, count = DEPOSIT_WORKLOADS[args.workload]
    dx = np.float32(1e-3)
    st = capi.Settings.default(width_m=side * 1e-3, height_m=side * 1e-3)
    cv = synth.blob_canvas(16, 16, 1, n_blobs=1, tables="reference")
    film = Film(st, side, side, capi.CF_PREC_FP32)
    film.set_tables(cv.pigtab, cv.cmf)
    sets = [deposit_strokes(count, side * 1e-3, dx, 10 * rank + k) for k in range(DEPOSIT_SETS)]
    stream = torch.cuda.Stream()
    sh = stream.cuda_stream
    # cells one launch paints (first set on the bare film)
    film.upload_deposits(sets[0])
    film.lay_deposits(sh)
    torch.cuda.synchronize()
    covered = int(np.count_nonzero(film.plane("h")))
    for k in range(args.warmup):
        film.upload_deposits(sets[k % DEPOSIT_SETS])
        film.lay_deposits(sh)
    torch.cuda.synchronize()
    l0 = film.stats()["launches"]
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with Clocks(local) as clk:
        for k in range(args.steps):
            film.upload_deposits(sets[k % DEPOSIT_SETS])
            evs[k][0].record(stream)
            film.lay_deposits(sh)
            evs[k][1].record(stream)
        torch.cuda.synchronize()
    t = sum(a.elapsed_time(b) for a, b in evs) / 1e3
    launches = film.stats()["launches"] - l0
    value = count * args.steps / t / 1e6
    peak, peak_kind = peaks()
    achieved = DEPOSIT_BYTES_PER_CELL * covered * args.steps / t / 1e9
    e2e = None
    if args.e2e_steps > 0:
        pinned = [torch.from_numpy(s.view(np.uint8)).pin_memory().numpy().view(s.dtype) for s in sets]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for k in range(args.e2e_steps):
            film.upload_deposits(pinned[k % DEPOSIT_SETS])
            film.lay_deposits(sh)
            film.stats()
        te = time.perf_counter() - t0
        items = float(np.mean([tiles_touched(s_, side, dx) for s_ in sets]))
        e2e = {"value": count * args.e2e_steps / te / 1e6, "unit": "Mdeposits/s",
               "h2d_bytes_per_step": int(96 * count + 8 * (side // 64) ** 2 + 4 * items),
               "d2h_bytes_per_step": int(ctypes.sizeof(capi.Stats)),
               "steps": args.e2e_steps, "path": "cf_upload_deposits(host records) + cf_lay_deposits + cf_get_stats"}
    cb = None if args.no_cpu_baseline else deposit_cpu(args.workload, args.cpu_seconds)
    line = {
        "metric": "Mdeposits/s", "value": value, "unit": "Mdeposits/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded strokes and capsules)",
        "config": {"workload": args.workload, "w": side, "h": side, "strokes_per_step": count,
                   "cells_painted_per_step": covered, "precision": "f32",
                   "l2": "each step paints new cells of a %d^2 film (%.1f GB of state): no flush"
                         % (side, film_bytes(side * side, capi.CF_PREC_FP32) / 1e9)},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_kind, "alg_bytes_per_painted_cell": DEPOSIT_BYTES_PER_CELL,
                     "scope": "k_deposit", "traffic": None},
        "gpu_launches": int(launches), "clocks": clk.summary(), "e2e": e2e, "cpu_baseline": cb,
    }
    print(json.dumps(line), flush=True)


def reference_arm(args):
    """CPU reference path, same workload / metric / unit / config; rank 0 only."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    if args.workload == RELIEF_WORKLOAD:  # the CPU path needs a film state: the default canvas as written
        cv = synth.config(1, 0)
        st = settings_for(cv)
        cb = relief_cpu(None, cv, st, min(150.0, 5.0 * (args.steps + args.warmup)))
        print(json.dumps({"impl": "reference", "metric": "Mpixel/s", "value": cb["value"], "unit": "Mpixel/s",
                          "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
                          "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                          "config": {"workload": args.workload}, "cpu_baseline": cb,
                          "e2e": {"value": cb["value"], "unit": "Mpixel/s", "h2d_bytes_per_step": 0,
                                  "d2h_bytes_per_step": 0}}), flush=True)
        return
    if args.workload == LIT_WORKLOAD:  # the reference's fragment exists on the host only as its translation
        print(json.dumps({"impl": "reference", "unavailable": "the renderer's fragment shader runs only through wgpu "
                          "(no graphics stack on this box); its CPU translation is test infrastructure built from "
                          "the reference sources where they exist"}), flush=True)
        return
    if args.workload in DEPOSIT_WORKLOADS:
        cb = deposit_cpu(args.workload, min(150.0, 10.0 * (args.steps + args.warmup)))
        print(json.dumps({"impl": "reference", "metric": "Mdeposits/s", "value": cb["value"], "unit": "Mdeposits/s",
                          "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
                          "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                          "config": {"workload": args.workload}, "cpu_baseline": cb,
                          "e2e": {"value": cb["value"], "unit": "Mdeposits/s", "h2d_bytes_per_step": 0,
                                  "d2h_bytes_per_step": 0}}), flush=True)
        return
    if args.workload == BATCH_WORKLOAD:
        reference_batch(args)
        return
    if args.workload == SERVE_WORKLOAD:
        reference_serve(args)
        return
    gen, prec, dt_max, adaptive = WORKLOADS[args.workload]
    cv = gen(0)
    per_step_budget = 150.0 / max(args.steps + args.warmup, 1)
    cb = cpu_baseline(cv, args.workload, per_step_budget * (args.steps + args.warmup), steps_hint=args.steps + args.warmup)
    line = {"impl": "reference", "metric": "Gcell-updates/s", "value": cb["value"], "unit": "Gcell-updates/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": PREC_NAME[prec],
            "data": "synthetic (seeded drip polylines / Gaussian blobs; no public dataset)",
            "config": single_config(args.workload, cv, prec, adaptive, dt_max, world),
            "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": "Gcell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def cpu_step_canvases(canvases, prec, dt, budget_s):
    """The oracle's FP32 restatement stepping each canvas one fixed-dt frame
    in turn (all host cores), round after round while the budget lasts (at
    least one round).  One canvas's oracle is held at a time (set up outside
    the timing), so host memory stays at one canvas's worth.  Returns
    (cell-updates, timed seconds, rounds)."""
    import pyoracle as po
    po.build()
    pig = capi.PREC_TO_PIG[prec]
    el, cells, rounds = 0.0, 0, 0
    while rounds == 0 or el < budget_s:
        for cv in canvases:
            o = po.Oracle(cv.w, cv.h, settings_for(cv), pig, 32)
            o.set_tables(cv.pigtab, cv.cmf)
            o.write_state(cv.planes)
            o.update_params(dt, 1)
            t0 = time.perf_counter()
            o.encode_frame(1)
            el += time.perf_counter() - t0
            cells += cv.w * cv.h
            del o
        rounds += 1
    return cells, el, rounds


def reference_batch(args):
    """Config 3 on the host cores: the same 64 canvases as the GPU arm (rank 0's
    seed), each stepped one frame after the other, rounds while the budget lasts."""
    canv = list(batch64_canvases(seed=0))
    cells, el, rounds = cpu_step_canvases(canv, capi.CF_PREC_FP32, 1e-3, min(150.0, 5.0 * (args.steps + args.warmup)))
    v = cells / el / 1e9
    cb = {"value": v, "unit": "Gcell-updates/s", "cores": os.cpu_count(), "kind": "port",
          "sample": "%d round(s) of one frame of each of the %d batch canvases (%d cells a round), FP32 oracle "
                    "restatement, OpenMP %d threads, %.1f s" % (rounds, len(canv), cells // rounds, os.cpu_count(), el)}
    print(json.dumps({"impl": "reference", "metric": "Gcell-updates/s", "value": v, "unit": "Gcell-updates/s",
                      "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
                      "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                      "data": "synthetic (seeded Gaussian blob fields; no public dataset)",
                      "config": batch_config(canv), "cpu_baseline": cb,
                      "e2e": {"value": v, "unit": "Gcell-updates/s", "h2d_bytes_per_step": 0,
                              "d2h_bytes_per_step": 0}}), flush=True)


def reference_serve(args):
    """Config 4 on the host cores: the served stream's template canvases (every
    side, FP32 and BF16 storage) stepped one frame each, one job at a time,
    rounds while the budget lasts."""
    from canvaz_film import serve
    pool = serve.TemplatePool(SERVE_SIDES, seed=0)
    budget = min(150.0, 5.0 * (args.steps + args.warmup))
    c32, e32, r32 = cpu_step_canvases(pool.canvases, capi.CF_PREC_FP32, serve.DT, budget / 2)
    c16, e16, r16 = cpu_step_canvases(pool.canvases, capi.CF_PREC_BF16, serve.DT, budget / 2)
    v = (c32 + c16) / (e32 + e16) / 1e9
    cb = {"value": v, "unit": "Gcell-updates/s", "cores": os.cpu_count(), "kind": "port",
          "sample": "one frame of each served template canvas (sides %s), %d FP32 and %d BF16 round(s), FP32 oracle "
                    "restatement, OpenMP %d threads, %.1f s" % (SERVE_SIDES, r32, r16, os.cpu_count(), e32 + e16)}
    print(json.dumps({"impl": "reference", "metric": "served Gcell-updates/s", "value": v,
                      "unit": "Gcell-updates/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
                      "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                      "dtype": "f32+f32pig|f32+bf16pig", "data": "synthetic (seeded Gaussian blob fields)",
                      "config": serve_config(args), "cpu_baseline": cb,
                      "e2e": {"value": v, "unit": "Gcell-updates/s", "h2d_bytes_per_step": 0,
                              "d2h_bytes_per_step": 0}}), flush=True)


def single_config(workload, cv, prec, adaptive, dt_max, world):
    """The `config` of a single-canvas line: the GPU arm and the reference arm
    build it with this one function, so both carry the same keys and values."""
    cells = cv.w * cv.h
    try:
        l2 = "working set %.1f GB > L2 (129 MB): no flush needed" % (film_bytes(cells, prec) / 1e9)
    except Exception:  # the library is not built (reference arm on a host without it)
        l2 = "working set > L2 (129 MB): no flush needed"
    return {"workload": workload, "w": cv.w, "h": cv.h, "cells_per_gpu": cells, "precision": PREC_NAME[prec],
            "adaptive_dt": adaptive, "dt_max": dt_max, "all_tiles_active": True,
            "parallelism": "replicas" if world > 1 else "single", "seed": "rank", "l2": l2}


def timed_film(workload, rank, steps, warmup, stream, clk=None):
    """A film of `workload` (seeded by rank) with its state resident, `warmup`
    untimed steps, then `steps` steps timed with CUDA events on `stream`."""
    import torch
    from canvaz_film.film import Film
    gen, prec, dt_max, adaptive = WORKLOADS[workload]
    cv = gen(rank)  # one replica canvas per rank, own seed
    st = settings_for(cv)
    film = Film(st, cv.w, cv.h, prec)
    film.set_tables(cv.pigtab, cv.cmf)
    film.write_state(cv.planes)
    s0 = film.stats()
    sh = stream.cuda_stream

    def step():
        if adaptive:
            film.step_adaptive(dt_max, sh)
        else:
            film.encode_frame(1, sh)

    if not adaptive:
        film.update_params(dt_max, 1)
    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    l0 = film.stats()["launches"]
    if torch.distributed.is_available() and torch.distributed.is_initialized():
        torch.distributed.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if clk is not None:
        clk.mark(True)
    e0.record(stream)
    for _ in range(steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    if clk is not None:
        clk.mark(False)
    if torch.distributed.is_available() and torch.distributed.is_initialized():
        torch.distributed.barrier()
    t = e0.elapsed_time(e1) / 1e3
    s1 = film.stats()
    return film, cv, st, t, s1["launches"] - l0, s0, s1


def gpu_arm(args):
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from canvaz_film.film import Film
    if not capi.LIB_PATH.exists():
        import __graft_entry__ as g
        g.build()
    gen, prec, dt_max, adaptive = WORKLOADS[args.workload]
    stream = torch.cuda.Stream()
    with Clocks(local) as clk:
        film, cv, st, t, launches, s0, s1 = timed_film(args.workload, rank, args.steps, args.warmup, stream, clk)
    if world > 1:
        tt = torch.tensor([t], device="cuda")
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        t = float(tt.item())
    cells = cv.w * cv.h
    value = world * cells * args.steps / t / 1e9
    alg = ALG_BYTES_PER_CELL[prec]
    peak, peak_kind = peaks()
    achieved = alg * cells * args.steps / t / 1e9
    traffic_pc = step_traffic(args.workload)
    mass0 = s0["wet_volume"] + s0["relief_volume"]
    mass1 = s1["wet_volume"] + s1["relief_volume"]

    # end to end through the C ABI with host buffers (pinned)
    e2e = None
    film_b = pair = outs = None
    if args.e2e_steps > 0:
        # the state in the reference's own layout (write_state's planes: f16
        # pigment slots, or BF16 where the film stores BF16)
        pig_fmt = capi.PREC_TO_PIG[prec] if prec != capi.CF_PREC_FP32 else capi.CF_PIG_F16
        state = film.read_state(pig_format=pig_fmt)
        pinned = {}
        for k, v in state.items():
            tv = torch.from_numpy(np.ascontiguousarray(v))
            pinned[k] = tv.pin_memory().numpy()
        h_out = torch.empty(cells, dtype=torch.float32).pin_memory()
        col_out = torch.empty(cells * 4, dtype=torch.int16).pin_memory()
        import ctypes as C
        L = capi.load_library()
        v = capi.StateView(pig_format=pig_fmt, device=0)
        for k in ("h", "m", "rheo", "strata_h", "strata_cure", "lay"):
            setattr(v, k, pinned[k].ctypes.data)
        sub = np.ascontiguousarray(state["sub_refl"].astype(np.float16))
        subp = torch.from_numpy(sub).pin_memory().numpy()
        v.sub_refl = subp.ctypes.data
        pig = state["strata_pig"]
        if pig_fmt == capi.CF_PIG_F16:
            pig = pig.astype(np.float16)
        elif pig_fmt == capi.CF_PIG_BF16:
            from canvaz_film.film import _pig_to_bf16
            pig = _pig_to_bf16(pig)
        pigp = torch.from_numpy(np.ascontiguousarray(pig)).pin_memory().numpy()
        v.strata_pig = pigp.ctypes.data
        h2d = sum(pinned[k].nbytes for k in ("h", "m", "rheo", "strata_h", "strata_cure", "lay")) + subp.nbytes + pigp.nbytes
        d2h = h_out.numel() * 4 + col_out.numel() * 2
        # two films on two streams: one film's upload over the host link
        # overlaps the other's step; every step still uploads its whole state
        # from pinned host memory and reads h and the colour image back
        film_b = Film(st, cv.w, cv.h, prec)
        film_b.set_tables(cv.pigtab, cv.cmf)
        film_b.clone_from(film)
        pair = [(film, stream), (film_b, torch.cuda.Stream())]
        outs = []
        for _ in range(2):
            ho = torch.empty(cells, dtype=torch.float32).pin_memory()
            co = torch.empty(cells * 4, dtype=torch.int16).pin_memory()
            outs.append((capi.StateView(pig_format=pig_fmt, device=0, h=ho.data_ptr()), ho,
                         C.cast(co.data_ptr(), C.POINTER(C.c_uint16)), co))
        if not adaptive:
            film_b.update_params(dt_max, 1)

        def e2e_step(k):
            fl, s = pair[k % 2]
            hv, _, cp, _ = outs[k % 2]
            assert L.cf_write_state_async(fl.p, C.byref(v), s.cuda_stream) == 0
            if adaptive:
                fl.step_adaptive(dt_max, s.cuda_stream)
            else:
                fl.encode_frame(1, s.cuda_stream)
            assert L.cf_read_state_async(fl.p, C.byref(hv), s.cuda_stream) == 0
            assert L.cf_read_color_async(fl.p, cp, s.cuda_stream) == 0

        # a probe of the host link on this machine (three torch copies of the
        # pigment plane, pinned host -> device), reported beside the e2e figure
        dev_buf = torch.empty(pigp.nbytes, dtype=torch.uint8, device="cuda")
        src_buf = torch.from_numpy(pigp.view(np.uint8).reshape(-1))
        torch.cuda.synchronize()
        tl = time.perf_counter()
        for _ in range(3):
            dev_buf.copy_(src_buf, non_blocking=True)
        torch.cuda.synchronize()
        link_gbs = 3 * pigp.nbytes / (time.perf_counter() - tl) / 1e9
        del dev_buf, src_buf
        e2e_step(0)
        e2e_step(1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for k in range(args.e2e_steps):
            e2e_step(k)
        torch.cuda.synchronize()
        te = time.perf_counter() - t0
        if world > 1:
            tt = torch.tensor([te], device="cuda")
            torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
            te = float(tt.item())
        e2e = {"value": world * cells * args.e2e_steps / te / 1e9, "unit": "Gcell-updates/s",
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h), "steps": args.e2e_steps,
               "host_link_probe_gbs": link_gbs,
               "path": "per step: cf_write_state_async(whole state in the reference layout, f16 or BF16 "
                       "pigment slots, pinned host) + step + cf_read_state_async(h) "
                       "+ cf_read_color_async; two films alternate on two streams, uploads one after the "
                       "other on the host link while the other film steps; wall time over the steps"}

    # the same canvas with BF16 pigment / rheology storage, timed the same way
    bf16 = None
    twin = BF16_TWIN.get(args.workload)
    if twin is not None:
        torch.cuda.synchronize()
        if film_b is not None:
            film_b.close()
        pair = outs = film_b = None
        film.close()
        film = None
        fb, cvb, _, tb, lb, _, _ = timed_film(twin, rank, args.steps, args.warmup, stream)
        if world > 1:
            tt = torch.tensor([tb], device="cuda")
            torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
            tb = float(tt.item())
        pb = WORKLOADS[twin][1]
        ab = ALG_BYTES_PER_CELL[pb] * cells * args.steps / tb / 1e9
        bf16 = {"workload": twin, "value": world * cells * args.steps / tb / 1e9, "unit": "Gcell-updates/s",
                "ms_per_step": 1e3 * tb / args.steps, "dtype": PREC_NAME[pb], "gpu_launches": int(lb),
                "roofline": {"bound": "hbm", "achieved": ab, "peak": peak, "unit": "GB/s", "frac": ab / peak,
                             "peak_source": peak_kind, "alg_bytes_per_cell": ALG_BYTES_PER_CELL[pb],
                             "scope": "whole step (all kernels of cf_encode_frame)"}}
        fb.close()
    cb = None
    if rank == 0 and not args.no_cpu_baseline:
        cb = cpu_baseline(cv, args.workload, args.cpu_seconds)
    clocks = clk.summary()
    if rank == 0:
        line = {
            "metric": "Gcell-updates/s", "value": value, "unit": "Gcell-updates/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": PREC_NAME[prec],
            "data": "synthetic (seeded drip polylines / Gaussian blobs; no public dataset)",
            "config": single_config(args.workload, cv, prec, adaptive, dt_max, world),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": peak_kind,
                         "alg_bytes_per_cell": alg,
                         "scope": "whole step (all kernels of %s)" % ("cf_step_adaptive" if adaptive
                                                                      else "cf_encode_frame"),
                         "traffic": None if traffic_pc is None else traffic_pc * cells},
            "gpu_launches": int(launches),
            "clocks": clocks,
            "e2e": e2e,
            "cpu_baseline": cb,
            "mass_drift_rel": abs(mass1 - mass0) / max(mass0, 1e-300),
            "last_dt": s1["last_dt"],
            "bf16": bf16,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def film_bytes(cells, prec):
    side = int(round(cells ** 0.5))
    return capi.film_bytes(side, max(cells // max(side, 1), 1), prec)


def batch64_canvases(count=64, seed=0):
    """64 canvases: side log-uniform 256-1536 rounded to 16, own seed, blob
    count uniform 10-200, rheology and pigments as the 512^2 blob field."""
    import math
    rng = np.random.Generator(np.random.PCG64(seed))
    for k in range(count):
        side = int(round(math.exp(rng.uniform(math.log(256), math.log(1536))) / 16.0)) * 16
        yield synth.blob_canvas(side, side, 1000 + k, n_blobs=int(rng.integers(10, 201)))


def batch_config(canvases):
    """`config` of the batch workload (the GPU and reference arms share it)."""
    sides = [cv.w for cv in canvases]
    return {"workload": BATCH_WORKLOAD, "canvases": len(canvases), "cells": sum(cv.w * cv.h for cv in canvases),
            "side_min": min(sides), "side_max": max(sides), "dt": 1e-3, "substeps": 1, "precision": "f32",
            "all_tiles_active": True,
            "l2": "working set > L2 (129 MB, %d canvases of %d-%d cells a side): no flush needed"
                  % (len(sides), min(sides), max(sides))}


def batch_arm(args):
    """Config 3: the batch (one launch per dispatch over all canvases' tiles,
    graph replay, autotuned) against the same canvases stepped one after the
    other with single-film launches, fixed dt 1e-3 s, one substep."""
    import torch
    from canvaz_film.film import Batch, Film
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if not capi.LIB_PATH.exists():
        import __graft_entry__ as g
        g.build()
    films, cells, sides = [], 0, []
    canvases = list(batch64_canvases(seed=rank))
    for cv in canvases:
        f = Film(settings_for(cv), cv.w, cv.h, capi.CF_PREC_FP32)
        f.set_tables(cv.pigtab, cv.cmf)
        f.write_state(cv.planes)
        f.update_params(1e-3, 1)
        films.append(f)
        cells += cv.w * cv.h
        sides.append(cv.w)
    b = Batch()
    for f in films:
        b.add(f)
    stream = torch.cuda.Stream()
    sh = stream.cuda_stream
    tuning, tune_ms = b.autotune(frames_per_trial=4, stream=sh)
    b.step(max(args.warmup, 3), 1, 0.0, sh)
    torch.cuda.synchronize()
    l0 = b.info()["launches"]
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(local) as clk:
        clk.mark(True)
        e0.record(stream)
        b.step(args.steps, 1, 0.0, sh)
        e1.record(stream)
        torch.cuda.synchronize()
        clk.mark(False)
    tb = e0.elapsed_time(e1) / 1e3
    launches = b.info()["launches"] - l0
    b.close()
    # the same films, one after the other per step, single-film launches
    seq_steps = max(min(args.steps // 4, 25), 3)
    for f in films:
        f.encode_frame(1, sh)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(seq_steps):
        for f in films:
            f.encode_frame(1, sh)
    e1.record(stream)
    torch.cuda.synchronize()
    ts = e0.elapsed_time(e1) / 1e3
    value = cells * args.steps / tb / 1e9
    seq = cells * seq_steps / ts / 1e9
    peak, peak_kind = peaks()
    achieved = ALG_BYTES_PER_CELL[capi.CF_PREC_FP32] * cells * args.steps / tb / 1e9
    clocks = clk.summary()
    if rank == 0:
        print(json.dumps({
            "metric": "Gcell-updates/s", "value": value, "unit": "Gcell-updates/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tb / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded Gaussian blob fields; no public dataset)",
            "config": batch_config(canvases),
            "tuning": tuning, "autotune_ms_per_frame": tune_ms,
            "sequential": {"value": seq, "unit": "Gcell-updates/s", "steps": seq_steps,
                           "form": "64 films one after another per step, single-film launches"},
            "speedup_vs_sequential": value / seq,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": peak_kind,
                         "alg_bytes_per_cell": ALG_BYTES_PER_CELL[capi.CF_PREC_FP32],
                         "scope": "whole batched step", "traffic": None},
            "gpu_launches": int(launches), "clocks": clocks,
        }), flush=True)
    for f in films:
        f.close()


SERVE_SIDES = [256, 368, 528, 768, 1104, 1584, 2048]


def serve_config(args):
    """`config` of the served workload (the GPU and reference arms share it)."""
    return {"workload": SERVE_WORKLOAD, "arrival_rate_per_s": 20.0, "window_s": args.serve_seconds,
            "wall_cutoff_s": args.serve_wall,
            "steps_range": [max(1, round(100 * args.serve_steps_scale)), round(3000 * args.serve_steps_scale)],
            "sides": SERVE_SIDES, "budget_bytes": 150e9, "dt": 1e-3}


def serve_arm(args):
    """Config 4: Poisson arrivals at 20/s, side log-spaced 256-2048, steps
    uniform 100-3000 (scaled), FP32 / BF16 pigments 50/50, 150 GB budget."""
    from canvaz_film import serve
    rank, world, local = dist_env()
    if not capi.LIB_PATH.exists():
        import __graft_entry__ as g
        g.build()
    pool = serve.TemplatePool(SERVE_SIDES, seed=rank)
    jobs = serve.poisson_jobs(args.serve_seconds, 20.0, pool, steps_scale=args.serve_steps_scale, seed=1 + rank)
    for s_ in pool.sides:  # templates resident before the clock starts
        for p_ in (capi.CF_PREC_FP32, capi.CF_PREC_BF16):
            pool.film(pool.sides.index(s_), p_)
    srv = serve.Server(pool, 150e9)
    with Clocks(local) as clk:
        rep = srv.run(jobs, args.serve_wall)
    srv.close()
    seq = serve.plain_sequential(jobs, pool, budget_s=30.0)
    pool.close()
    if rank == 0:
        print(json.dumps({
            "metric": "served Gcell-updates/s", "value": rep["gcell_updates_per_s"], "unit": "Gcell-updates/s",
            "n_gpus": world, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32+f32pig|f32+bf16pig", "data": "synthetic (seeded Gaussian blob fields)",
            "config": serve_config(args),
            "step_ms_p50": rep["step_ms_p50"], "step_ms_p99": rep["step_ms_p99"],
            "queue_wait_s_p50": rep["queue_wait_s_p50"], "queue_wait_s_p99": rep["queue_wait_s_p99"],
            "jobs": {"arrived": rep["jobs_arrived"], "done": rep["jobs_done"], "peak_resident": rep["peak_resident_jobs"]},
            "peak_bytes": rep["peak_bytes"], "admission_s": rep["admission_s"], "wall_s": rep["wall_s"],
            "plain_sequential": {"value": seq["gcell_updates_per_s"], "unit": "Gcell-updates/s", "jobs": seq["jobs"],
                                 "busy_s": seq["busy_s"], "form": "jobs one at a time in arrival order, single-film launches"},
            "speedup_vs_sequential": rep["gcell_updates_per_s"] / seq["gcell_updates_per_s"],
            "clocks": clk.summary(),
        }), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        reference_arm(args)
    elif args.workload == BATCH_WORKLOAD:
        batch_arm(args)
    elif args.workload == SERVE_WORKLOAD:
        serve_arm(args)
    elif args.workload in DEPOSIT_WORKLOADS:
        deposit_arm(args)
    elif args.workload == RELIEF_WORKLOAD:
        relief_arm(args)
    elif args.workload == LIT_WORKLOAD:
        lit_arm(args)
    elif args.workload == SNAPSHOT_WORKLOAD:
        snapshot_arm(args)
    else:
        gpu_arm(args)


if __name__ == "__main__":
    main()
