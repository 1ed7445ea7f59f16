"""CPU: the reference arm of bench.py prints one JSON line with the keys and
units of the GPU arm (the CPU restatement of the reference's algorithm, timed
on the host's cores), on one process and as rank 0 of two torchrun ranks
(the other rank exits 0 without work).  Small 2D radial workload."""
import json
import os
import subprocess
import sys

from conftest import ROOT

ARGS = ["bench.py", "--impl", "reference", "--workload", "radial2d", "--steps", "2", "--warmup", "1"]


def _lines(out):
    return [json.loads(l) for l in out.splitlines() if l.startswith("{")]


def _check(d, n_gpus):
    assert d["impl"] == "reference"
    assert d["value"] > 0 and d["unit"] == "Msamples/s" and d["higher_is_better"] is True
    assert d["n_gpus"] == n_gpus and d["steps"] == 2 and d["warmup"] == 1 and d["ms_per_step"] > 0
    assert d["config"]["workload"] and d["config"]["coils"] == 8
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert cb["sample"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0


def test_reference_arm_one_process():
    r = subprocess.run([sys.executable] + ARGS, cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _lines(r.stdout)
    assert len(lines) == 1
    _check(lines[0], 1)


def test_reference_arm_under_torchrun_two_ranks():
    env = dict(os.environ, OMP_NUM_THREADS="2")
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
                        "--master-addr", "127.0.0.1", "--master-port", "29613"] + ARGS + ["--gpus", "2"],
                       cwd=ROOT, capture_output=True, text=True, timeout=300, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _lines(r.stdout)
    assert len(lines) == 1  # rank 0 alone
    _check(lines[0], 2)


def test_gpu_arm_has_no_cpu_fallback():
    """Without a GPU the measured arm exits non-zero and prints no result
    line: nothing is timed on a CPU stand-in."""
    import pytest
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    r = subprocess.run([sys.executable, "bench.py", "--workload", "radial2d", "--steps", "1", "--warmup", "0"],
                       cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode != 0
    assert not _lines(r.stdout)
