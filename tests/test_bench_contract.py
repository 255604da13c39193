"""The JSON line of `bench.py --impl reference` on the host cores: one bounded
step of the 512^2 blob workload through the FP32 oracle restatement, with
every key the reference arm promises; and a rank other than 0 under a
multi-rank launch printing nothing and exiting 0."""
import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def run_bench(args, env_extra=None, timeout=600):
    env = dict(os.environ)
    env.update(env_extra or {})
    return subprocess.run([sys.executable, str(ROOT / "bench.py"), *args], cwd=ROOT, env=env, capture_output=True,
                          text=True, timeout=timeout)


def test_reference_arm_line():
    r = run_bench(["--impl", "reference", "--workload", "blobs512_dt1e-3_fp32", "--steps", "1", "--warmup", "0"])
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == d["unit"] == "Gcell-updates/s"
    assert d["value"] > 0 and d["higher_is_better"] is True
    assert d["n_gpus"] == 1 and d["steps"] == 1 and d["warmup"] == 0
    assert d["config"]["workload"] == "blobs512_dt1e-3_fp32"
    # the same config object the GPU arm prints for this workload
    sys.path.insert(0, str(ROOT))
    import bench
    gen, prec, dt_max, adaptive = bench.WORKLOADS["blobs512_dt1e-3_fp32"]
    want = bench.single_config("blobs512_dt1e-3_fp32", gen(0), prec, adaptive, dt_max, 1)
    assert d["config"] == json.loads(json.dumps(want))
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["unit"] == d["unit"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_other_ranks_do_no_work():
    r = run_bench(["--impl", "reference", "--workload", "blobs512_dt1e-3_fp32", "--steps", "1", "--warmup", "0",
                   "--gpus", "2"],
                  {"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1", "MASTER_ADDR": "127.0.0.1",
                   "MASTER_PORT": "29571"}, timeout=120)
    assert r.returncode == 0, r.stderr[-2000:]
    assert not [ln for ln in r.stdout.splitlines() if ln.startswith("{")]


if __name__ == "__main__":
    sys.exit(pytest.main([__file__, "-q"]))
