"""One rank of the CPU (gloo) check of bench.py's replica helpers; started by torchrun from
tests/test_dist_replicas.py.  Each rank writes rank<r>.json into the folder given as the
first argument (two ranks printing at once could interleave their lines)."""
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def main():
    world, rank, local, dist = bench.dist_setup()
    bench.barrier(dist)
    # each rank's "time" differs; every rank must see the maximum
    got = bench.max_over_ranks(dist, 1.5 + rank)
    bench.barrier(dist)
    with open(os.path.join(sys.argv[1], f"rank{rank}.json"), "w") as f:
        json.dump({"rank": rank, "world": world, "local": local, "max": got,
                   "backend": dist.get_backend() if dist else None}, f)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
