"""The N > 1 host path of bench.py on CPU: two gloo ranks under torchrun (127.0.0.1).

Each rank of the GPU bench advances its own channel (replicas, no exchange), so what runs
across ranks is only the barrier, the max over ranks of the timed region, and rank 0
alone printing.  The reference arm under two ranks prints one line, from rank 0."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def torchrun(args, timeout=240):
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port())] + args
    env = dict(os.environ, OMP_NUM_THREADS="1", CUDA_VISIBLE_DEVICES="")
    return subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=timeout)


def json_lines(out):
    return [json.loads(l) for l in out.splitlines() if l.startswith("{")]


def test_two_gloo_ranks_agree_on_max(tmp_path):
    r = torchrun([os.path.join("tests", "dist_worker.py"), str(tmp_path)])
    assert r.returncode == 0, r.stderr[-2000:]
    lines = []
    for q in (0, 1):
        with open(tmp_path / f"rank{q}.json") as f:
            lines.append(json.load(f))
    assert [d["rank"] for d in lines] == [0, 1]
    assert all(d["world"] == 2 and d["backend"] == "gloo" for d in lines)
    assert all(d["max"] == 2.5 for d in lines)


def test_reference_arm_two_ranks_prints_once(port):
    port.build(port=True, ref=False)
    r = torchrun(["bench.py", "--impl", "reference", "--gpus", "2", "--grid", "12", "8", "6",
                  "--steps", "3", "--warmup", "3"])
    assert r.returncode == 0, r.stderr[-2000:]
    lines = json_lines(r.stdout)
    assert len(lines) == 1
    d = lines[0]
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["e2e"]["h2d_bytes_per_step"] == 0
