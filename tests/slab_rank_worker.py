"""One rank of the CPU (gloo) check of the z-slab decomposition's plan and halo schedule;
started by torchrun from tests/test_slab_ranks.py with the world size as the number of slabs.

Every rank builds the same seeded whole-domain arrays, keeps its slab (the library's
ark_slab_plan), clears its ghost planes, and refills them by the library's schedule
(ark_slab_halo_planes): the planes its neighbours need are sent to them over gloo, a bounded end
copies its own zero-gradient plane.  The refilled ghosts must equal the whole domain's ghosts as
the single-domain ghost fill sets them (periodic wrap or zero-gradient copy), and the scalar
reductions of the step (max |u| as FP64 bit patterns, the 2^-32 fixed-point u1 sum) taken as
MAX and SUM over the ranks must equal the whole domain's.  Writes rank<r>.json into the folder
given as the first argument; the second argument is 1 for a periodic z, 0 for a bounded one."""
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "ark-cpp-mpi_gb300"))

import arkgpu  # noqa: E402

C1, C2, C3 = 6, 5, 11


def domain_arrays(seed=4):
    rng = np.random.default_rng(seed)
    cells = [rng.uniform(-1.0, 1.0, (C3 + 2, C2 + 2, C1 + 2)) for _ in range(3)]
    faces = [rng.uniform(-1.0, 1.0, (C3 + 3, C2 + 3, C1 + 3)) for _ in range(2)]
    return cells, faces


def ghost_fill(a, face, periodic):
    """The single-domain z ghost fill (k_wrap): cells ghost 0 <- C3 (periodic) or 1, ghost C3+1
    <- 1 or C3; faces halo 0 <- C3 or 1, halo C3+2 <- 2 or C3+1; interior (i, j) only."""
    a = a.copy()
    I, J = slice(1, C1 + 1), slice(1, C2 + 1)
    if not face:
        a[0, J, I] = a[C3 if periodic else 1, J, I]
        a[C3 + 1, J, I] = a[1 if periodic else C3, J, I]
    else:
        a[0, J, I] = a[C3 if periodic else 1, J, I]
        a[C3 + 2, J, I] = a[2 if periodic else C3 + 1, J, I]
    return a


def fixed32(v):
    return int(np.rint(np.clip(v, -2.0 ** 30, 2.0 ** 30) * 2.0 ** 32))


def main():
    import torch
    import torch.distributed as dist

    out_dir, periodic = sys.argv[1], sys.argv[2] == "1"
    dist.init_process_group("gloo")
    rank, world = dist.get_rank(), dist.get_world_size()
    k0, k1, below, above = arkgpu.slab_plan(C3, world, rank, periodic)
    c3 = k1 - k0 + 1
    plans = [arkgpu.slab_plan(C3, world, r, periodic) for r in range(world)]
    cells, faces = domain_arrays()
    I, J = slice(1, C1 + 1), slice(1, C2 + 1)
    ok, problems = True, []
    for face, arrays in ((0, cells), (1, faces)):
        for q, g in enumerate(arrays):
            local = g[k0 - 1:k1 + 2 + face].copy()
            ghosts = (0, c3 + 1 + face)
            for p in ghosts:
                local[p] = 0.0
            # the planes the neighbours need from this slab, then the planes it needs from them
            reqs = []
            for side, nb in ((0, above), (1, below)):  # the slab above fills its side-0 ghost from this one
                if nb < 0:
                    continue
                c3_nb = plans[nb][1] - plans[nb][0] + 1
                _, src = arkgpu.slab_halo_planes(face, side, c3_nb, c3, False)
                buf = torch.from_numpy(np.ascontiguousarray(local[src, J, I]))
                reqs.append(dist.isend(buf, nb, tag=10 * q + side))
            recvs = []
            for side, nb in ((0, below), (1, above)):
                if nb < 0:
                    dst, src = arkgpu.slab_halo_planes(face, side, c3, c3, True)
                    local[dst, J, I] = local[src, J, I]
                    continue
                c3_nb = plans[nb][1] - plans[nb][0] + 1
                dst, _ = arkgpu.slab_halo_planes(face, side, c3, c3_nb, False)
                buf = torch.empty((C2, C1), dtype=torch.float64)
                recvs.append((dist.irecv(buf, nb, tag=10 * q + side), dst, buf))
            for r in reqs:
                r.wait()
            for r, dst, buf in recvs:
                r.wait()
                local[dst, J, I] = buf.numpy()
            want = ghost_fill(g, face, periodic)[k0 - 1:k1 + 2 + face]
            for p in ghosts:
                if not np.array_equal(local[p, J, I], want[p, J, I]):
                    ok = False
                    problems.append(f"face={face} array={q} ghost plane {p}")
    # the step's reductions over the ranks
    u = cells[0]
    mine = u[k0:k1 + 1, J, I]
    mx = torch.tensor([int(np.abs(mine).max().view(np.int64))], dtype=torch.int64)
    sm = torch.tensor([sum(fixed32(v) for v in mine.ravel())], dtype=torch.int64)
    dist.all_reduce(mx, op=dist.ReduceOp.MAX)
    dist.all_reduce(sm, op=dist.ReduceOp.SUM)
    whole = u[1:C3 + 1, J, I]
    want_mx = int(np.abs(whole).max().view(np.int64))
    want_sm = sum(fixed32(v) for v in whole.ravel())
    if int(mx.item()) != want_mx or int(sm.item()) != want_sm:
        ok = False
        problems.append("reductions")
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
        json.dump({"rank": rank, "world": world, "k": [k0, k1], "below": below, "above": above, "ok": ok,
                   "problems": problems}, f)
    dist.barrier()
    dist.destroy_process_group()


if __name__ == "__main__":
    main()
