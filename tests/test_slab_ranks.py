"""The z-slab decomposition's host side on CPU: the plan partitions the planes, and under
torchrun with gloo ranks (127.0.0.1) the halo schedule refills every ghost plane as the
single-domain ghost fill does and the reductions over ranks equal the whole domain's
(tests/slab_rank_worker.py).  The device side, one GPU stepping a group of slabs bit for bit
like one context, is tests/test_gpu_slabs.py."""
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


def test_plan_partitions_the_planes(ark):
    """Every split of every small C3: the slabs cover 1..C3 in order without gaps or overlap, sizes
    differ by at most one, and the neighbours form a ring (periodic) or a line (bounded)."""
    for C3 in range(1, 40):
        for n in range(1, C3 + 1):
            for periodic in (True, False):
                plans = [ark.slab_plan(C3, n, s, periodic) for s in range(n)]
                assert plans[0][0] == 1 and plans[-1][1] == C3
                sizes = [b - a + 1 for a, b, _, _ in plans]
                assert max(sizes) - min(sizes) <= 1 and min(sizes) >= 1
                for s in range(n - 1):
                    assert plans[s][1] + 1 == plans[s + 1][0]
                for s, (_, _, below, above) in enumerate(plans):
                    assert below == (s - 1 if s > 0 else (n - 1 if periodic else -1))
                    assert above == (s + 1 if s < n - 1 else (0 if periodic else -1))
    with pytest.raises(ark.ArkError):
        ark.slab_plan(4, 5, 0)


@pytest.mark.parametrize("world,periodic", [(2, 1), (3, 1), (3, 0)])
def test_gloo_ranks_exchange_halos_by_the_schedule(ark, tmp_path, world, periodic):
    ark.lib()  # built by the fixture before the ranks load it
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", str(world),
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()),
           os.path.join("tests", "slab_rank_worker.py"), str(tmp_path), str(periodic)]
    env = dict(os.environ, OMP_NUM_THREADS="1", CUDA_VISIBLE_DEVICES="")
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=240)
    assert r.returncode == 0, r.stderr[-3000:]
    ks = []
    for q in range(world):
        with open(tmp_path / f"rank{q}.json") as f:
            d = json.load(f)
        assert d["world"] == world and d["ok"], d["problems"]
        ks.append(d["k"])
    assert ks[0][0] == 1 and ks[-1][1] == 11
