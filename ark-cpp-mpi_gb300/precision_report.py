"""Error of the FP32 path against the FP64 path, on the channel's mean profile
and its wall shear.

    python ark-cpp-mpi_gb300/precision_report.py [--grid 512 256 256] [--steps 2000] [--re 5600]

Both paths start from the same seeded channel state and run the same number of steps.  The
FP64 path is bit-for-bit the reference's arithmetic (it is checked against the reference's
own outputs), so it stands in for the FP64 oracle at sizes where the CPU oracle would take
minutes per step.  Reported, as one JSON line:
  field relative L2 errors of rho - ro0, u1, u2, u3 over interior cells;
  the mean u1(y) profile: max absolute error, and relative to the bulk velocity;
  the wall shear stress 2*VIS*U(wall)/dy at both walls: relative error;
  the time per step of both paths.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import arkgpu  # noqa: E402


def rel_l2(a, b):
    n = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (n if n > 0 else 1.0))


def run(C, re_b, steps, seed=12345, amp=0.1, device=0):
    out = {}
    st0 = None
    for name, prec in (("fp64", arkgpu.FP64), ("fp32", arkgpu.FP32)):
        p = arkgpu.make_params(*C, re_b=re_b, precision=prec, device=device)
        if st0 is None:
            st0 = arkgpu.channel_init(p, seed=seed, amp=amp)
        with arkgpu.Context(p) as ctx:
            ctx.upload(st0)
            ctx.sync()
            t0 = time.perf_counter()
            ctx.step(steps)
            ctx.sync()
            secs = time.perf_counter() - t0
            prof, ws = ctx.mean_profile()
            fields = ctx.download(["ronCon", "u1nCon", "u2nCon", "u3nCon"])
            sc = ctx.scalars()
        out[name] = {"fields": {n: a[1:-1, 1:-1, 1:-1].copy() for n, a in fields.items()}, "profile": prof,
                     "wall_shear": ws, "ms_per_step": 1e3 * secs / steps, "time": sc.time, "ub": sc.bulk_velocity}
        del fields
    a, b = out["fp32"], out["fp64"]
    ro0 = 1.0
    err = {
        "rho_dev_rel_l2": rel_l2(a["fields"]["ronCon"] - ro0, b["fields"]["ronCon"] - ro0),
        "u1_rel_l2": rel_l2(a["fields"]["u1nCon"], b["fields"]["u1nCon"]),
        "u2_rel_l2": rel_l2(a["fields"]["u2nCon"], b["fields"]["u2nCon"]),
        "u3_rel_l2": rel_l2(a["fields"]["u3nCon"], b["fields"]["u3nCon"]),
        "profile_max_abs": float(np.abs(a["profile"] - b["profile"]).max()),
        "profile_max_rel_to_ub": float(np.abs(a["profile"] - b["profile"]).max() / max(abs(b["ub"]), 1e-300)),
        "wall_shear_rel": [float(abs(a["wall_shear"][q] - b["wall_shear"][q]) / abs(b["wall_shear"][q]))
                           for q in range(2)],
    }
    return {"grid": list(C), "re_b": re_b, "steps": steps, "errors": err,
            "ms_per_step": {"fp64": round(b["ms_per_step"], 4), "fp32": round(a["ms_per_step"], 4)},
            "wall_shear_fp64": [float(x) for x in b["wall_shear"]], "time": b["time"]}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--grid", type=int, nargs=3, default=(512, 256, 256))
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--re", type=float, default=5600.0)
    ap.add_argument("--seed", type=int, default=12345)
    a = ap.parse_args()
    print(json.dumps(run(tuple(a.grid), a.re, a.steps, seed=a.seed)))


if __name__ == "__main__":
    main()
