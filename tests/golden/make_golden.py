"""Generate the golden fixtures from the REFERENCE ITSELF (compiled in place).

    make -C oracle ref         # builds oracle/_ref/libark_ref.so from the reference sources
    python tests/golden/make_golden.py

The reference (ark-cpp-mpi) ships no tests, fixtures or known-answer vectors, so these
fixtures are outputs of its own source/main.cpp solver functions (TimeStepSize, Phase1,
StressTensor, UseForces, Phase2), driven by oracle/ref_harness.cpp on seeded channel
states.  They pin the C restatement (oracle/ark_oracle.c) on any machine, including the
GPU machine where the reference sources are absent.

Files:
  small_run.npz      12x8x6 cells, 20 full steps with bulk forcing: interior arrays
  small_bounded.npz  14x6x6 cells, 10 steps, bounded x (inflow/outflow) and z edges
  phases.npz         10x6x8 cells: one call of each step piece on a perturbed state
  digests.json       sha256 of every interior array after longer runs (64x32x32 x 100
                     steps at Re_b 2800, 33x17x9 x 50 steps), plus dt, TIME, U_b
  stock_case.npz     the reference's own case, set up by its Input() and InitializeData()
                     (200x60x1 backward-facing step): the initial state and the interior
                     arrays after 40 steps
  boundary.npz       the reference's BoundaryConditions class (alongX1/2/3) on the "nCon" level
                     of a 9x6x5 grid with random values everywhere (ghosts included), for
                     every combination of x2/x3 periodicity; the values are FP32-exact so
                     FP32 contexts can be compared bit for bit too
  writers.npz        the files of the reference's writers (WriteDataParaView's out_5.vtk,
                     WriteAverageValues' average.vtk, WriteEnergy's energy.txt) and its
                     averageU arrays after 5 steps with AverageValues after each, for a 3-D
                     10x6x4 grid and a 2-D 9x5x1 grid

    python tests/golden/make_golden.py writers   # only writers.npz
    python tests/golden/make_golden.py boundary  # only boundary.npz
"""
from __future__ import annotations

import hashlib
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402

CHECK = ["roCon", "u1Con", "u2Con", "u3Con", "ronCon", "u1nCon", "u2nCon", "u3nCon"] + list(oracle.FACE_NAMES)


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def interior_dump(m) -> dict:
    return {n: oracle.interior(n, m.get(n)) for n in CHECK}


def perturbed_state(p, seed):
    """A channel state whose faces and pressure are also perturbed, so every branch of the
    face update and the limiter is exercised by single calls."""
    st = oracle.channel_state(p)
    draws = [0]

    def noise(shape):  # splitmix64 uniforms in [-1, 1), a fresh stream per array
        draws[0] += 1
        n = int(np.prod(shape))
        return (2.0 * oracle.uniform01(seed * 1000 + draws[0], n) - 1.0).reshape(shape)

    for d in (1, 2, 3):
        for v in ("u1", "u2", "u3"):
            n = f"{v}{d}"
            st[n] = st[n] + 0.05 * noise(st[n].shape)
        st[f"p{d}"] = 0.2 * noise(st[f"p{d}"].shape)
    for lvl in ("", "n"):
        st[f"ro{lvl}Con"] = st[f"ro{lvl}Con"] + 0.002 * noise(st[f"ro{lvl}Con"].shape)
    st["u1Con"] = st["u1nCon"] + 0.01 * noise(st["u1nCon"].shape)
    return st


def writers():
    """Section 6: the reference's writers on two grids (C3 > 1 shows its row offsets without
    a k term; C3 = 1 is its own 2-D case)."""
    out = {}
    for tag, C, seed in (("3d", (10, 6, 4), 21), ("2d", (9, 5, 1), 22)):
        p = oracle.channel_params(*C, seed=seed)
        ref = oracle.Reference(p)
        ref.load(oracle.channel_state(p))
        for _ in range(5):
            ref.run(1)
            ref.average_values()
        d = tempfile.mkdtemp(prefix="ark_golden_") + "/"
        ref.write_paraview(d)
        ref.write_average(d, 0.0)
        ref.write_energy(d)
        out[f"{tag}/params"] = json.dumps(p)
        for name, fn in (("paraview", "out_5.vtk"), ("average", "average.vtk"), ("energy", "energy.txt")):
            with open(d + fn, "rb") as f:
                out[f"{tag}/{name}"] = np.frombuffer(f.read(), dtype=np.uint8)
            os.remove(d + fn)
        os.rmdir(d)
        for m in (1, 2, 3):
            out[f"{tag}/averageU{m}"] = ref.get_average(m)
        out[f"{tag}/time"] = ref.time
    np.savez_compressed(os.path.join(HERE, "writers.npz"), steps=5, **out)


BOUNDARY_LEVEL = ("ronCon", "u1nCon", "u2nCon", "u3nCon")


def boundary_state(p, seed):
    """Random "nCon" cell arrays over every element (ghosts included), FP32-exact: u in
    [-1, 1) rounded to FP32, rho = rho0 + an FP32 deviation below 1e-2 (exact in FP64, and
    rho - rho0 is that FP32 value again)."""
    shape = (p["C3"] + 2, p["C2"] + 2, p["C1"] + 2)
    n = int(np.prod(shape))
    out = {}
    for q, name in enumerate(BOUNDARY_LEVEL):
        r = (2.0 * oracle.uniform01(seed * 100 + q, n) - 1.0).reshape(shape)
        if name == "ronCon":
            out[name] = p["rho0"] + (0.01 * r).astype(np.float32).astype(np.float64)
        else:
            out[name] = r.astype(np.float32).astype(np.float64)
    return out


def boundary():
    """Section 7: BoundaryConditions(u1nCon, u2nCon, u3nCon, ronCon, tnCon, x1Period, x2Period,
    x3Period, n1, n2, n3, t0).alongX1/2/3 (source/BoundaryConditions.cpp:7-83), each axis from
    the same start, for every combination of x2/x3 periodicity (x1Period, which the class never
    reads, set equal to x2Period)."""
    p = oracle.channel_params(9, 6, 5, seed=31)
    st = boundary_state(p, 31)
    out = {"params": json.dumps(p), "state_seed": 31}
    for name in BOUNDARY_LEVEL:
        out[f"state/{name}"] = st[name]
    for x2p in (0, 1):
        for x3p in (0, 1):
            for axis in (1, 2, 3):
                ref = oracle.Reference(p, forcing=False)
                ref.load(st)
                ref.boundary_conditions(axis, x2p, x2p, x3p)
                for name in BOUNDARY_LEVEL:
                    out[f"ax{axis}_p{x2p}{x3p}/{name}"] = ref.get(name)
    np.savez_compressed(os.path.join(HERE, "boundary.npz"), **out)


def main():
    assert oracle.Reference.available(), "build oracle/_ref first: make -C oracle ref"
    if sys.argv[1:] == ["writers"]:
        writers()
        print("writers.npz written to", HERE)
        return
    if sys.argv[1:] == ["boundary"]:
        boundary()
        print("boundary.npz written to", HERE)
        return
    out = {}

    # 1. short forced run, full interior arrays
    p = oracle.channel_params(12, 8, 6, seed=7)
    ref = oracle.Reference(p)
    ref.load(oracle.channel_state(p))
    ref.run(20)
    d = interior_dump(ref)
    np.savez_compressed(os.path.join(HERE, "small_run.npz"), params=json.dumps(p), steps=20,
                        dt=ref.dt, time=ref.time, ub=ref.last_ub, G=ref.last_g, **d)

    # 2. bounded x (inflow R=1 / outflow Q=5/6, main.cpp:1731-1745) and bounded z
    p2 = oracle.channel_params(14, 6, 6, seed=11)
    ref = oracle.Reference(p2, periodic_x=False, periodic_z=False)
    ref.load(oracle.channel_state(p2))
    ref.run(10)
    d = interior_dump(ref)
    np.savez_compressed(os.path.join(HERE, "small_bounded.npz"), params=json.dumps(p2), steps=10,
                        dt=ref.dt, time=ref.time, **d)

    # 3. single calls of each step piece (forcing off: pieces exactly as the reference has them)
    p3 = oracle.channel_params(10, 6, 8, seed=3)
    st = perturbed_state(p3, 5)
    ph = {}
    ref = oracle.Reference(p3, forcing=False)
    ref.load(st)
    ref.time_step_size()
    ph["dt"] = ref.dt
    ref.phase1()
    for n in ("roCon", "u1Con", "u2Con", "u3Con", "ronCon", "u1nCon", "u2nCon", "u3nCon"):
        ph[f"phase1/{n}"] = oracle.interior(n, ref.get(n))
    ref.stress_tensor()
    for n in ("f1", "f2", "f3"):
        ph[f"stress/{n}"] = oracle.interior(n, ref.get(n))
    for m in "123":
        for dd in "123":
            ph[f"stress/sigm{m}{dd}"] = ref.get(f"sigm{m}{dd}")
    ref.use_forces()
    for n in ("u1nCon", "u2nCon", "u3nCon"):
        ph[f"forces/{n}"] = oracle.interior(n, ref.get(n))
    ref.phase2()
    for n in oracle.FACE_NAMES:
        ph[f"phase2/{n}"] = oracle.interior(n, ref.get(n))
    np.savez_compressed(os.path.join(HERE, "phases.npz"), params=json.dumps(p3), state_seed=5, **ph)

    # 4. the reference's own stock case (its Input() and InitializeData())
    ref, ps = oracle.Reference.stock()
    init = {n: ref.get(n) for n in oracle.STATE_NAMES}
    ref.run(40)
    d = interior_dump(ref)
    np.savez_compressed(os.path.join(HERE, "stock_case.npz"), params=json.dumps(ps), steps=40, dt=ref.dt,
                        time=ref.time, **{f"init/{n}": a for n, a in init.items()}, **d)

    # 5. digests of longer runs
    dig = {}
    for (C, steps, re_b, seed) in (((64, 32, 32), 100, 2800.0, 12345), ((33, 17, 9), 50, 2800.0, 99)):
        pp = oracle.channel_params(*C, re_b=re_b, seed=seed)
        ref = oracle.Reference(pp)
        ref.load(oracle.channel_state(pp))
        ref.run(steps)
        key = f"{C[0]}x{C[1]}x{C[2]}_{steps}"
        dig[key] = {"params": pp, "steps": steps, "dt": ref.dt, "time": ref.time, "ub": ref.last_ub,
                    "sha256": {n: digest(oracle.interior(n, ref.get(n))) for n in CHECK},
                    "l2": {n: float(np.linalg.norm(oracle.interior(n, ref.get(n)))) for n in CHECK}}
    with open(os.path.join(HERE, "digests.json"), "w") as f:
        json.dump(dig, f, indent=1, sort_keys=True)

    # 6. the writers
    writers()

    # 7. the BoundaryConditions class
    boundary()
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
