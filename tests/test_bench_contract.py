"""bench.py's CPU reference arm (`--impl reference`): one JSON line with the keys of the benchmark
contract, printed by rank 0 alone under a two-rank launch (gloo, CPU). Small sizes keep it to a
few seconds; the GPU arms are exercised on a GPU only."""
import json
import os
import subprocess
import sys

from conftest import ROOT

ARGS = ["--impl", "reference", "--workload", "single", "--bodies", "2000", "--free", "200", "--steps", "3",
        "--warmup", "3", "--reference-seconds", "2"]
ARGS_BATCHED = ["--impl", "reference", "--systems", "6", "--min-bodies", "40", "--max-bodies", "80", "--steps", "3",
                "--warmup", "3", "--reference-seconds", "2"]


def _lines(out):
    return [json.loads(l) for l in out.splitlines() if l.startswith("{")]


def _check(d):
    assert d["impl"] == "reference" and d["unit"] == "body-steps/s" and d["value"] > 0
    for k in ("metric", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling", "vs_baseline",
              "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["steps"] == 3 and d["warmup"] == 3 and d["higher_is_better"] is True
    assert d["config"]["bodies"] == 2000 and "2,000 rigid bodies" in d["config"]["workload"]
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0


def test_reference_arm_prints_the_contract_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *ARGS], capture_output=True, text=True,
                       timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _lines(r.stdout)
    assert len(lines) == 1
    _check(lines[0])


def test_reference_arm_under_two_ranks_prints_once():
    env = dict(os.environ, MASTER_ADDR="127.0.0.1")
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
                        "--master-addr", "127.0.0.1", "--master-port", "29517", os.path.join(ROOT, "bench.py"),
                        "--gpus", "2", *ARGS], capture_output=True, text=True, timeout=300, cwd=ROOT, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _lines(r.stdout)
    assert len(lines) == 1
    _check(lines[0])
    assert lines[0]["n_gpus"] == 2


def test_batched_reference_arm_uses_the_gpu_arms_config():
    """The default workload (batched replicas): the reference arm's `config` is the dict the GPU arm
    prints (bench.batched_config), so the two lines describe the same workload."""
    import argparse
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *ARGS_BATCHED], capture_output=True,
                       text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _lines(r.stdout)
    assert len(lines) == 1
    d = lines[0]
    assert d["impl"] == "reference" and d["value"] > 0 and d["cpu_baseline"]["value"] == d["value"]
    sys.path.insert(0, ROOT)
    import bench
    args = argparse.Namespace(systems=6, min_bodies=40, max_bodies=80, steps=3)
    assert d["config"] == bench.batched_config(args, 1)
