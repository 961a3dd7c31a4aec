"""Slab groups on one GPU: a channel split along z into slab contexts with the reference's two
halo exchanges per step (main.cpp:601-801 before the stress, main.cpp:1049-1631 before Phase2)
and the dt / bulk-flow reductions over all slabs (main.cpp:412) gives the single-domain result
bit for bit -- which for FP64 is the reference's own output (tests/golden/digests.json)."""
import hashlib
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CELLS = ["roCon", "u1Con", "u2Con", "u3Con", "ronCon", "u1nCon", "u2nCon", "u3nCon"]
FACES = ["p1", "ro1", "u11", "u21", "u31", "p2", "ro2", "u12", "u22", "u32", "p3", "ro3", "u13", "u23", "u33"]


def bits_equal(a, b):
    return np.array_equal(np.ascontiguousarray(a).view(np.uint64), np.ascontiguousarray(b).view(np.uint64))


def params_from(ark, p, **kw):
    return ark.make_params(p["C1"], p["C2"], p["C3"], re_b=1.0 / p["nu"], sound=p["sound"], rho0=p["rho0"],
                           cfl=p["cfl"], lx=p["lx"], ly=p["ly"], lz=p["lz"], ub=p["ub"], **kw)


@pytest.mark.parametrize("nslabs", [2, 3, 5])
def test_slabs_match_reference_digest(ark, port, nslabs):
    """64x32x32, Re_b 2800, 100 steps split into 2, 3 or 5 slabs (even and uneven): every interior
    array has the sha256 of the reference's own output, and dt, TIME and U_b are the reference's."""
    with open(os.path.join(GOLD, "digests.json")) as f:
        d = json.load(f)["64x32x32_100"]
    p = d["params"]
    with ark.Slabs(params_from(ark, p), nslabs) as G:
        G.upload(port.channel_state(p))
        G.step(d["steps"])
        G.sync()
        sc = G.scalars()
        assert sc.dt == d["dt"] and sc.time == d["time"] and sc.bulk_velocity == d["ub"]
        st = G.download(CELLS + FACES)
    for n in CELLS + FACES:
        a = port.interior(n, st[n])
        assert hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest() == d["sha256"][n], n


@pytest.mark.parametrize("prec,pz,nslabs", [("fp64", 0, 3), ("fp32", 1, 4), ("fp32", 0, 2), ("fp64", 1, 1)])
def test_slabs_equal_single_context(ark, port, prec, pz, nslabs):
    """Periodic and bounded z, both precisions, ragged slabs: the group's whole-domain state (ghost
    planes included) and conservation sums equal one context's after 12 steps."""
    p = port.channel_params(40, 20, 23, seed=41)
    st0 = port.channel_state(p)
    P = params_from(ark, p, precision=ark.FP64 if prec == "fp64" else ark.FP32)
    P.periodic_z = pz
    with ark.Context(P) as c:
        c.upload(st0)
        c.step(12)
        c.sync()
        want = c.download(CELLS + FACES)
        want_sums = c.sums()
        want_sc = c.scalars()
    with ark.Slabs(P, nslabs) as G:
        G.upload(st0)
        G.step(5)
        G.step(7)
        G.sync()
        got = G.download(CELLS + FACES)
        sums = G.sums()
        sc = G.scalars()
    for n in CELLS + FACES:
        assert bits_equal(port.interior(n, got[n]), port.interior(n, want[n])), n
    for f in ("mass", "momentum1", "momentum2", "momentum3", "kinetic", "cells"):
        assert getattr(sums, f) == getattr(want_sums, f), f
    assert sc.dt == want_sc.dt and sc.nstep == want_sc.nstep == 12 and sc.bulk_force == want_sc.bulk_force


def test_slabs_bounded_z_match_oracle(ark, port):
    """Bounded z (zero-gradient ends of the group) against the C restatement, 3 slabs, 10 steps."""
    p = port.channel_params(48, 20, 24, seed=13)
    st0 = port.channel_state(p)
    o = port.Port(p, periodic_x=True, periodic_z=False)
    o.load(st0)
    o.run(10)
    P = params_from(ark, p)
    P.periodic_z = 0
    with ark.Slabs(P, 3) as G:
        G.upload(st0)
        G.step(10)
        G.sync()
        st = G.download(CELLS + FACES)
    for n in CELLS + FACES:
        assert bits_equal(port.interior(n, st[n]), port.interior(n, o.get(n))), n
