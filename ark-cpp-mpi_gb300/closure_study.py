"""The learned-closure study: fine-grid training data, training, and the coarse-grid test.

    python ark-cpp-mpi_gb300/closure_study.py [--fine 256 128 128] [--coarse 64 48 48]
        [--spin 300000] [--train-steps 100000] [--snapshots 400] [--coarse-steps 5000]
        [--epochs 20] [--batch 65536] [--out report.json]

1. A fine FP32 channel (Re_b 5600, c = 10, CFL 0.2, bulk forcing) starts from the seeded
   channel state plus a streak perturbation (which makes it turbulent within tens of time
   units) and is spun up; its wall shear is recorded along the way.
2. Training data: `snapshots` states of the next `train-steps` steps, each 3 x 3 x 3
   box-filtered on the device, sampled on a 4 x 4 lattice in x and z (every y); y+ uses the
   friction velocity measured at the end of the spin-up.  The last tenth of the snapshots is
   held out.
3. The network is trained on the device (ark_mlp_train) and scored on the held-out samples
   against no closure (nu_t = 0) and the best constant eddy viscosity.
4. The assessment: the fine state at the start of a window, volume-averaged onto the coarse grid,
   runs `coarse-steps` coarse steps twice, without and with the closure; the fine run covers
   the same physical time.  Plane statistics (means over x, z and time of u and of the
   products u_i u_j) of the coarse runs are compared with those of the box-filtered fine
   field: mean profile U(y) and Reynolds shear stress <u'v'>(y), interpolated to the coarse
   cell centres.  GPU time: CUDA-event time of the steps of each run.
The report (JSON) is printed and written to --out.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import arkgpu  # noqa: E402

RE_B = 5600.0  # the study's Reynolds number (--re changes it)


def params(C, precision=arkgpu.FP32):
    return arkgpu.make_params(*C, re_b=RE_B, sound=10.0, rho0=1.0, cfl=0.2, precision=precision)


def streaks(p, st):
    """A large-scale streak and roll perturbation (project choice, to trigger transition)."""
    C1, C2, C3 = p.n1_cells, p.n2_cells, p.n3_cells
    x = (np.arange(C1 + 2) - 0.5) * (p.lx / C1)
    y = -0.5 * p.ly + (np.arange(C2 + 2) - 0.5) * (p.ly / C2)
    z = (np.arange(C3 + 2) - 0.5) * (p.lz / C3)
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    env = np.clip(1 - Y * Y, 0, None)
    du1 = 0.3 * env * np.sin(4 * np.pi * Z / p.lz) * (1 + 0.3 * np.sin(2 * np.pi * X / p.lx))
    du2 = 0.2 * env * env * np.cos(4 * np.pi * Z / p.lz) * (1 + 0.3 * np.cos(2 * np.pi * X / p.lx))
    for lvl in ("", "n"):
        st[f"u1{lvl}Con"][1:-1, 1:-1, 1:-1] += du1[1:-1, 1:-1, 1:-1]
        st[f"u2{lvl}Con"][1:-1, 1:-1, 1:-1] += du2[1:-1, 1:-1, 1:-1]
    return st


def overlap(nf, nc):
    """(nc, nf) volume fractions of fine cells in coarse cells on one uniform axis."""
    M = np.zeros((nc, nf))
    hf, hc = 1.0 / nf, 1.0 / nc
    for J in range(nc):
        a, b = J * hc, (J + 1) * hc
        j0, j1 = int(math.floor(a / hf)), min(nf, int(math.ceil(b / hf)))
        for j in range(j0, j1):
            M[J, j] = max(0.0, min(b, (j + 1) * hf) - max(a, j * hf)) / hc
    return M


def restrict(a, Cc):
    """Volume average of an interior array [k, j, i] onto Cc = (C1, C2, C3)."""
    Mz, My, Mx = overlap(a.shape[0], Cc[2]), overlap(a.shape[1], Cc[1]), overlap(a.shape[2], Cc[0])
    return np.einsum("Kk,Jj,Ii,kji->KJI", Mz, My, Mx, a, optimize=True)


def state_from_cells(p, ro, u):
    """A complete host state from interior cell fields (both levels alike): periodic ghosts in
    x and z, solid rows at the walls, faces the means of their two cells (walls at rest),
    face pressure c^2 (rho - ro0)."""
    st = arkgpu.empty_state(p, alloc=np.zeros)
    C1, C2, C3 = p.n1_cells, p.n2_cells, p.n3_cells
    fields = [ro] + list(u)
    full = []
    for a in fields:
        b = np.zeros((C3 + 2, C2 + 2, C1 + 2))
        b[1:-1, 1:-1, 1:-1] = a
        b[1:-1, 1:-1, 0] = a[:, :, -1]
        b[1:-1, 1:-1, -1] = a[:, :, 0]
        b[0] = b[C3]
        b[C3 + 1] = b[1]
        full.append(b)
    rof, uf = full[0], full[1:]
    for lvl in ("", "n"):
        st[f"ro{lvl}Con"][:] = rof
        for m in range(3):
            st[f"u{m + 1}{lvl}Con"][:] = uf[m]
    cond = st["condition"]
    cond[:] = 0.0
    cond[:, 0, :] = 1.0
    cond[:, C2 + 1, :] = 1.0
    c2 = p.sound * p.sound
    # faces normal to x1 (i = 1..C1+1), x2 (j = 2..C2; walls j = 1, C2+1 at rest), x3
    for d, (sl_lo, sl_hi, fsl) in enumerate((
            ((slice(1, C3 + 1), slice(1, C2 + 1), slice(0, C1 + 1)), (slice(1, C3 + 1), slice(1, C2 + 1), slice(1, C1 + 2)),
             (slice(1, C3 + 1), slice(1, C2 + 1), slice(1, C1 + 2))),
            ((slice(1, C3 + 1), slice(1, C2), slice(1, C1 + 1)), (slice(1, C3 + 1), slice(2, C2 + 1), slice(1, C1 + 1)),
             (slice(1, C3 + 1), slice(2, C2 + 1), slice(1, C1 + 1))),
            ((slice(0, C3 + 1), slice(1, C2 + 1), slice(1, C1 + 1)), (slice(1, C3 + 2), slice(1, C2 + 1), slice(1, C1 + 1)),
             (slice(1, C3 + 2), slice(1, C2 + 1), slice(1, C1 + 1))))):
        n = "123"[d]
        rface = 0.5 * (rof[sl_lo] + rof[sl_hi])
        st[f"ro{n}"][:] = p.ro0
        st[f"ro{n}"][fsl] = rface
        st[f"p{n}"][fsl] = c2 * (rface - p.ro0)
        for m in range(3):
            st[f"u{m + 1}{n}"][fsl] = 0.5 * (uf[m][sl_lo] + uf[m][sl_hi])
    return st


class Stats:
    """Time average of plane statistics (9 per plane)."""

    def __init__(self):
        self.s, self.n = None, 0

    def add(self, a):
        self.s = a.copy() if self.s is None else self.s + a
        self.n += 1

    def result(self, ly):
        a = self.s / self.n
        C2 = a.shape[0]
        y = -0.5 * ly + (np.arange(C2) + 0.5) * (ly / C2)
        U, V = a[:, 0], a[:, 1]
        return {"y": y, "U": U, "uv": a[:, 6] - U * V, "uu": a[:, 3] - U * U, "vv": a[:, 4] - V * V,
                "ww": a[:, 5] - a[:, 2] ** 2, "samples": self.n}


def compare(coarse, fine):
    """Errors of coarse statistics against fine ones interpolated to the coarse cell centres."""
    out = {}
    for q in ("U", "uv", "uu"):
        f = np.interp(coarse["y"], fine["y"], fine[q])
        c = coarse[q]
        ref = np.max(np.abs(f))
        out[q] = {"rel_l2": float(np.linalg.norm(c - f) / np.linalg.norm(f)), "max_rel": float(np.max(np.abs(c - f)) / ref)}
    return out


def main():
    global RE_B
    ap = argparse.ArgumentParser()
    ap.add_argument("--fine", type=int, nargs=3, default=(256, 128, 128))
    ap.add_argument("--coarse", type=int, nargs=3, default=(64, 48, 48))
    ap.add_argument("--spin", type=int, default=300000)
    ap.add_argument("--train-steps", type=int, default=100000)
    ap.add_argument("--snapshots", type=int, default=400)
    ap.add_argument("--coarse-steps", type=int, default=5000)
    ap.add_argument("--epochs", type=int, default=20)
    ap.add_argument("--batch", type=int, default=65536)
    ap.add_argument("--lattice", type=int, default=4)
    ap.add_argument("--seed", type=int, default=11)
    ap.add_argument("--out", default=None)
    ap.add_argument("--re", type=float, default=RE_B, help="bulk Reynolds number U_b h / nu (default 5600)")
    a = ap.parse_args()
    RE_B = a.re
    rep = {"config": vars(a).copy(), "re_b": RE_B}
    t_start = time.time()

    pf = params(tuple(a.fine))
    fine = arkgpu.Context(pf)
    st0 = streaks(pf, arkgpu.channel_init(pf, seed=a.seed, amp=0.1))
    fine.upload(st0)
    rep["fine_shapes"] = fine.autotune(3)  # then start again from the initial state
    fine.upload(st0)
    del st0
    hist = []
    chunk = max(1, a.spin // 30)
    done = 0
    while done < a.spin:
        n = min(chunk, a.spin - done)
        fine.step(n)
        done += n
        fine.sync()
        _, ws = fine.mean_profile()
        sc = fine.scalars()
        hist.append([int(sc.nstep), round(sc.time, 3), float(ws[0]), float(ws[1])])
    rep["spin_wall_shear"] = hist
    _, ws = fine.mean_profile()
    u_tau = math.sqrt(0.5 * (ws[0] + ws[1]))
    rep["u_tau"] = u_tau
    rep["re_tau"] = u_tau / pf.vis

    # training data (the last tenth of the snapshots held out)
    L = a.lattice
    per_snap = ((a.fine[0] + L - 1) // L) * a.fine[1] * ((a.fine[2] + L - 1) // L)
    held = max(1, a.snapshots // 10)
    train = arkgpu.ClosureData(per_snap * (a.snapshots - held) + 16)
    heldd = arkgpu.ClosureData(per_snap * held + 16)
    every = max(1, a.train_steps // a.snapshots)
    for s in range(a.snapshots):
        fine.step(every)
        fine.closure_sample(train if s < a.snapshots - held else heldd, sx=L, sz=L, ox=s % L, oz=(s // L) % L,
                            u_tau=u_tau)
    rep["samples"] = {"train": len(train), "held_out": len(heldd), "per_snapshot": per_snap}

    net = arkgpu.Mlp(seed=a.seed)
    net.fit_normalization(train)
    t0 = time.time()
    losses = []
    for ep in range(a.epochs):
        lr = 2e-3 if ep < a.epochs // 2 else (5e-4 if ep < (3 * a.epochs) // 4 else 1.5e-4)
        losses.append(net.train(train, epochs=1, batch=min(a.batch, len(train)), lr=lr))
    _, ttr = train.get()
    rep["training"] = {"epochs": a.epochs, "loss_per_epoch": losses, "seconds": round(time.time() - t0, 2),
                       "target_mean": float(np.mean(ttr)), "target_var": float(np.var(ttr))}
    _, tho = heldd.get()
    pred = net.predict(heldd)
    rep["a_priori_held_out"] = {"mse_network": float(np.mean((pred - tho) ** 2)), "mse_no_closure": float(np.mean(tho ** 2)),
                                "mse_best_constant": float(np.mean((np.mean(ttr) - tho) ** 2)),
                                "corr_network": float(np.corrcoef(pred, tho)[0, 1])}
    train.close()
    heldd.close()
    del ttr

    # the assessment window
    names = ["ronCon", "u1nCon", "u2nCon", "u3nCon"]
    st = fine.download(names)
    t_window = fine.scalars().time
    Cc = tuple(a.coarse)
    ro = restrict(st["ronCon"][1:-1, 1:-1, 1:-1], Cc)
    uc = [restrict(st[n][1:-1, 1:-1, 1:-1], Cc) for n in names[1:]]
    del st
    pc = params(Cc)
    coarse = {}
    stc = state_from_cells(pc, ro, uc)
    for mode in ("plain", "closure"):
        with arkgpu.Context(pc) as c:
            if mode == "closure":
                c.set_closure(net, u_tau=u_tau)
            c.upload(stc)
            rep[f"coarse_shapes_{mode}"] = c.autotune(20)
            c.upload(stc)
            c.step(2)
            c.sync()
            stats = Stats()
            every_c = max(1, a.coarse_steps // 400)
            ms = 0.0
            t_c0 = c.scalars().time
            for q in range(0, a.coarse_steps, every_c):
                ms += c.time_steps(min(every_c, a.coarse_steps - q))
                stats.add(c.plane_stats())
            coarse[mode] = {"stats": stats.result(pc.ly), "gpu_ms": ms, "time": c.scalars().time - t_c0}
            if mode == "closure":
                # the eddy viscosity the network gives in the coarse run's last state
                nut = c.get("nut")[1:-1, 1:-1, 1:-1] / pc.vis
                prof = nut.mean(axis=(0, 2))
                coarse[mode]["nut_over_nu"] = {"mean": float(nut.mean()), "max": float(nut.max()),
                                               "mean_by_y": prof.tolist()}
    t_phys = coarse["plain"]["time"]

    # the fine run over the same physical time, filtered statistics ~400 times
    fstats = Stats()
    scratch = arkgpu.ClosureData(a.fine[1] * 4)
    dt_f = fine.scalars().dt
    est = max(1, int(t_phys / dt_f))
    every_f = max(1, est // 400)
    ms_f = 0.0
    steps_f = 0
    while fine.scalars().time < t_window + t_phys:
        ms_f += fine.time_steps(every_f)
        steps_f += every_f
        scratch.clear()
        fine.closure_sample(scratch, sx=a.fine[0], sz=a.fine[2], u_tau=u_tau)
        fstats.add(scratch.filtered_stats())
    scratch.close()
    fres = fstats.result(pf.ly)
    rep["assessment"] = {"window_start_time": t_window, "physical_time": t_phys, "fine_steps": steps_f,
                    "fine_gpu_ms": ms_f, "coarse_steps": a.coarse_steps}
    for mode in ("plain", "closure"):
        e = compare(coarse[mode]["stats"], fres)
        rep["assessment"][mode] = {"errors": e, "gpu_ms": coarse[mode]["gpu_ms"],
                              "gpu_time_ratio_fine_over_coarse": ms_f / coarse[mode]["gpu_ms"]}
    rep["assessment"]["closure"]["nut_over_nu"] = coarse["closure"]["nut_over_nu"]
    rep["assessment"]["profiles"] = {
        "y_coarse": coarse["plain"]["stats"]["y"].tolist(),
        "U_fine_filtered": np.interp(coarse["plain"]["stats"]["y"], fres["y"], fres["U"]).tolist(),
        "U_plain": coarse["plain"]["stats"]["U"].tolist(), "U_closure": coarse["closure"]["stats"]["U"].tolist(),
        "uv_fine_filtered": np.interp(coarse["plain"]["stats"]["y"], fres["y"], fres["uv"]).tolist(),
        "uv_plain": coarse["plain"]["stats"]["uv"].tolist(), "uv_closure": coarse["closure"]["stats"]["uv"].tolist(),
        "uu_fine_filtered": np.interp(coarse["plain"]["stats"]["y"], fres["y"], fres["uu"]).tolist(),
        "uu_plain": coarse["plain"]["stats"]["uu"].tolist(), "uu_closure": coarse["closure"]["stats"]["uu"].tolist()}
    params_out, mu, sd = net.get()
    rep["network"] = {"params": params_out.tolist(), "mu": mu.tolist(), "sd": sd.tolist()}
    rep["wall_seconds"] = round(time.time() - t_start, 1)
    fine.close()
    net.close()
    txt = json.dumps(rep)
    if a.out:
        with open(a.out, "w") as f:
            f.write(txt)
    short = {k: v for k, v in rep.items() if k not in ("network",)}
    short["assessment"] = {k: v for k, v in rep["assessment"].items() if k != "profiles"}
    print(json.dumps(short, indent=1))


if __name__ == "__main__":
    main()
