"""bench.py --gpus N outside torchrun starts the N ranks itself.

The ranks meet through a gloo process group (barriers, max over ranks), as
under torchrun; rank 0 prints the one JSON line and its n_gpus is N.  Run on
the CPU through the reference arm, which needs no GPU: rank 0 times one
bounded CPU sample of the workload, the other rank waits at the barrier."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(args, timeout=600):
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK", "MASTER_ADDR",
                                                             "MASTER_PORT")}
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], capture_output=True, text=True,
                          cwd=ROOT, env=env, timeout=timeout)


def test_spawned_ranks_report_n_gpus():
    r = _run(["--gpus", "2", "--impl", "reference", "--steps", "1", "--warmup", "0"])
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout  # rank 0 alone prints
    line = json.loads(lines[0])
    assert line["impl"] == "reference"
    assert line["n_gpus"] == 2
    assert line["value"] > 0 and line["cpu_baseline"]["cores"] >= 1


def test_world_size_mismatch_is_an_error():
    env_args = ["--gpus", "2", "--impl", "reference", "--steps", "1", "--warmup", "0"]
    env = dict(os.environ, WORLD_SIZE="1", RANK="0", LOCAL_RANK="0")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *env_args], capture_output=True, text=True,
                       cwd=ROOT, env=env, timeout=300)
    assert r.returncode != 0
    assert "WORLD_SIZE" in r.stderr


def test_rank_without_a_gpu_is_an_error():
    """Our arm on a machine with fewer GPUs than ranks (here: none) stops
    with a message instead of failing inside CUDA."""
    r = _run(["--gpus", "1", "--steps", "1", "--warmup", "3"], timeout=300)
    assert r.returncode == 2, r.stderr[-2000:]
    assert "needs GPU 0" in r.stderr
