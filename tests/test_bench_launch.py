"""bench.py's own launcher for `--gpus N` (one process per GPU when no launcher
set WORLD_SIZE): the reference arm runs on rank 0 while the other ranks exit
without work, and the GPU arm refuses more GPUs than are visible."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(args, env_extra=None):
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK")}
    env.update(env_extra or {})
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py")] + args, capture_output=True, text=True,
                          env=env, timeout=600)


def test_reference_arm_starts_two_ranks():
    r = _run(["--impl", "reference", "--gpus", "2", "--workload", "small", "--steps", "1", "--warmup", "1"])
    assert r.returncode == 0, r.stderr
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1  # rank 0 alone prints
    out = json.loads(lines[0])
    assert out["impl"] == "reference" and out["n_ranks"] == 2
    assert out["config"]["workload"] == "small" and out["value"] > 0
    assert "rank 1/2 exits without work" in r.stderr


def test_gpu_arm_refuses_more_gpus_than_visible():
    r = _run(["--gpus", "9", "--steps", "1", "--warmup", "1"], {"CUDA_VISIBLE_DEVICES": "0"})
    assert r.returncode == 2
    assert "--gpus 9" in r.stderr and "visible" in r.stderr
