"""The oracle (C restatement of the reference step) against the reference's own outputs.

The golden fixtures under tests/golden were produced by the reference's source/main.cpp
compiled in place (tests/golden/make_golden.py); the live comparison runs only where the
reference sources exist.  Everything here is CPU-only.
"""
import hashlib
import json
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CELLS = ["roCon", "u1Con", "u2Con", "u3Con", "ronCon", "u1nCon", "u2nCon", "u3nCon"]


def bits_equal(a, b):
    return np.array_equal(np.ascontiguousarray(a).view(np.uint64), np.ascontiguousarray(b).view(np.uint64))


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def test_port_matches_golden_small_run(port):
    g = np.load(os.path.join(GOLD, "small_run.npz"))
    p = json.loads(str(g["params"]))
    o = port.Port(p)
    o.load(port.channel_state(p))
    o.run(int(g["steps"]))
    assert o.dt == float(g["dt"]) and o.time == float(g["time"]) and o.last_ub == float(g["ub"])
    for n in CELLS + list(port.FACE_NAMES):
        assert bits_equal(port.interior(n, o.get(n)), g[n]), n


def test_port_matches_golden_bounded_edges(port):
    """Bounded x (inflow/outflow invariants, main.cpp:1731-1745) and zero-gradient z."""
    g = np.load(os.path.join(GOLD, "small_bounded.npz"))
    p = json.loads(str(g["params"]))
    o = port.Port(p, periodic_x=False, periodic_z=False)
    o.load(port.channel_state(p))
    o.run(int(g["steps"]))
    assert o.dt == float(g["dt"])
    for n in CELLS + list(port.FACE_NAMES):
        assert bits_equal(port.interior(n, o.get(n)), g[n]), n


def test_port_matches_golden_step_pieces(port):
    from make_golden import perturbed_state

    g = np.load(os.path.join(GOLD, "phases.npz"))
    p = json.loads(str(g["params"]))
    o = port.Port(p, forcing=False)
    o.load(perturbed_state(p, int(g["state_seed"])))
    o.time_step_size()
    assert o.dt == float(g["dt"])
    o.phase1()
    for n in CELLS:
        assert bits_equal(port.interior(n, o.get(n)), g[f"phase1/{n}"]), n
    o.stress_tensor()
    for n in ("f1", "f2", "f3"):
        assert bits_equal(port.interior(n, o.get(n)), g[f"stress/{n}"]), n
    for m in "123":
        for d in "123":
            assert bits_equal(o.get(f"sigm{m}{d}"), g[f"stress/sigm{m}{d}"]), (m, d)
    o.use_forces()
    for n in ("u1nCon", "u2nCon", "u3nCon"):
        assert bits_equal(port.interior(n, o.get(n)), g[f"forces/{n}"]), n
    o.phase2()
    for n in port.FACE_NAMES:
        assert bits_equal(port.interior(n, o.get(n)), g[f"phase2/{n}"]), n


@pytest.mark.parametrize("key", ["33x17x9_50", "64x32x32_100"])
def test_port_matches_golden_digests(port, key):
    with open(os.path.join(GOLD, "digests.json")) as f:
        d = json.load(f)[key]
    p = d["params"]
    o = port.Port(p)
    o.load(port.channel_state(p))
    o.run(d["steps"])
    assert o.dt == d["dt"] and o.time == d["time"] and o.last_ub == d["ub"]
    for n, h in d["sha256"].items():
        assert sha(port.interior(n, o.get(n))) == h, n


def test_port_thread_count_invariance(port):
    """Only order-independent reductions: 1 thread and many threads agree bit for bit."""
    p = port.channel_params(20, 12, 10, seed=4)
    st = port.channel_state(p)
    a = port.Port(p, threads=1)
    a.load(st)
    a.run(6)
    ra = {n: a.get(n) for n in CELLS}
    b = port.Port(p, threads=4)
    b.load(st)
    b.run(6)
    for n in CELLS:
        assert bits_equal(port.interior(n, b.get(n)), port.interior(n, ra[n])), n
    port.Port.lib().aor_set_threads(os.cpu_count() or 1)


def test_port_conserves_mass(port):
    p = port.channel_params(24, 16, 8, seed=9)
    o = port.Port(p)
    o.load(port.channel_state(p))
    m0 = port.interior("ronCon", o.get("ronCon")).sum()
    o.run(30)
    m1 = port.interior("ronCon", o.get("ronCon")).sum()
    assert abs(m1 - m0) / m0 < 1e-13


def test_port_periodic_faces_consistent(port):
    """With periodic x and z, face 1 and face C+1 carry identical values."""
    p = port.channel_params(16, 8, 12, seed=2)
    o = port.Port(p)
    o.load(port.channel_state(p))
    o.run(10)
    u11 = o.get("u11")
    assert bits_equal(u11[1:-2, 1:-2, 1], u11[1:-2, 1:-2, p["C1"] + 1])
    u13 = o.get("u13")
    assert bits_equal(u13[1, 1:-2, 1:-2], u13[p["C3"] + 1, 1:-2, 1:-2])


def test_port_matches_live_reference(port):
    """Where the reference sources exist, the compiled reference and the port agree on a
    fresh configuration (odd sizes, forcing on)."""
    port.build(port=False)
    if not port.Reference.available():
        pytest.skip("reference sources not present on this machine")
    p = port.channel_params(13, 7, 5, re_b=1500.0, seed=31, amp=0.13)
    st = port.channel_state(p)
    r = port.Reference(p)
    r.load(st)
    r.run(12)
    o = port.Port(p)
    o.load(st)
    o.run(12)
    assert r.dt == o.dt
    for n in CELLS + list(port.FACE_NAMES):
        assert bits_equal(port.interior(n, r.get(n)), port.interior(n, o.get(n))), n


def _boundary_cases():
    for x2p in (0, 1):
        for x3p in (0, 1):
            for axis in (1, 2, 3):
                yield axis, x2p, x3p


def test_boundary_conditions_restated_match_reference_class(port):
    """The numpy restatement of BoundaryConditions::alongX1/2/3 against the reference class's
    own outputs (tests/golden/boundary.npz): every element of every array, ghosts included,
    for each axis and each x2/x3 periodicity."""
    g = np.load(os.path.join(GOLD, "boundary.npz"))
    level = {n[6:]: g[n] for n in g.files if n.startswith("state/")}
    assert sorted(level) == ["ronCon", "u1nCon", "u2nCon", "u3nCon"]
    for axis, x2p, x3p in _boundary_cases():
        got = port.boundary_conditions(level, axis, bool(x2p), bool(x3p))
        for n in level:
            assert bits_equal(got[n], g[f"ax{axis}_p{x2p}{x3p}/{n}"]), (axis, x2p, x3p, n)


def test_boundary_conditions_live_reference(port):
    """Where the reference sources exist: the class on a fresh random level of another grid
    against the restatement."""
    port.build(port=False)
    if not port.Reference.available():
        pytest.skip("reference sources not present on this machine")
    from make_golden import boundary_state

    p = port.channel_params(6, 9, 4, seed=5)
    level = boundary_state(p, 5)
    for axis, x2p, x3p in _boundary_cases():
        r = port.Reference(p, forcing=False)
        r.load(level)
        r.boundary_conditions(axis, 1 - x2p, x2p, x3p)
        want = port.boundary_conditions(level, axis, bool(x2p), bool(x3p))
        for n in level:
            assert bits_equal(r.get(n), want[n]), (axis, x2p, x3p, n)


def test_channel_init_matches_library(port, ark):
    """The numpy channel init (oracle side) and ark_channel_init (library side) agree."""
    p = ark.make_params(9, 6, 5)
    st = ark.channel_init(p, seed=77, amp=0.12)
    ref = port.channel_state(port.channel_params(9, 6, 5, seed=77, amp=0.12))
    for n in ark.STATE_FIELDS:
        assert bits_equal(st[n], ref[n]), n


def test_splitmix64_known_values(port):
    # splitmix64 seeded with 0: published first outputs of the generator
    v = port.splitmix64(0, 3)
    assert [int(x) for x in v] == [0xE220A8397B1DCDAF, 0x6E789E6AA1B965F4, 0x06C45D188009454F]


def test_port_matches_reference_stock_case(port):
    """The reference's own case (its Input() and InitializeData(): 200x60x1 backward-facing
    step, bounded in x and z, solid block x <= 5, y <= 1), 40 steps, bit for bit."""
    g = np.load(os.path.join(GOLD, "stock_case.npz"))
    p = json.loads(str(g["params"]))
    st = {n[5:]: g[n] for n in g.files if n.startswith("init/")}
    o = port.Port(p, periodic_x=False, periodic_z=False, forcing=False)
    o.load(st)
    o.run(int(g["steps"]))
    assert o.dt == float(g["dt"])
    for n in CELLS + list(port.FACE_NAMES):
        assert bits_equal(port.interior(n, o.get(n)), g[n]), n


@pytest.mark.parametrize("tag", ["3d", "2d"])
def test_writers_restated_match_reference_files(port, tag):
    """The numpy restatement of WriteDataParaView / AverageValues / WriteAverageValues /
    WriteEnergy against the files the reference wrote (tests/golden/writers.npz).  In 3-D the
    reference's file keeps only the last k plane (its row offsets have no k term); in 2-D the
    full layout and the reference's coincide."""
    g = np.load(os.path.join(GOLD, "writers.npz"))
    p = json.loads(str(g[f"{tag}/params"]))
    o = port.Port(p)
    o.load(port.channel_state(p))
    avg = [np.zeros((p["C3"] + 2, p["C2"] + 3, p["C1"] + 2)) for _ in range(3)]
    for _ in range(int(g["steps"])):
        o.run(1)
        port.average_add(avg, {n: o.get(n) for n in ("u1nCon", "u2nCon", "u3nCon")}, o.dt)
    assert o.time == float(g[f"{tag}/time"])
    for m in range(3):
        assert bits_equal(avg[m], g[f"{tag}/averageU{m + 1}"]), m
    st = {n: o.get(n) for n in ["u1nCon", "u2nCon", "u3nCon", "ronCon"] + list(port.FACE_NAMES)}
    ref_vtk = g[f"{tag}/paraview"].tobytes()
    assert port.paraview_bytes(p, st, "reference") == ref_vtk
    assert port.average_bytes(p, avg, o.time, 0.0, "reference") == g[f"{tag}/average"].tobytes()
    full = port.paraview_bytes(p, st, "full")
    assert (full == ref_vtk) == (p["C3"] == 1)
    assert len(full) >= len(ref_vtk)
    text = "(%f; %f) " % (o.time, port.kinetic_energy(p, st))
    assert text.encode() == g[f"{tag}/energy"].tobytes()


def test_closure_oracle_gradient_is_the_derivative():
    """The numpy network's analytic gradient against central finite differences (FP64)."""
    import oracle.closure as oc

    rng = np.random.default_rng(5)
    theta = rng.normal(0, 0.3, oc.NPARAM)
    mu, sd = rng.normal(0, 1, oc.NIN), rng.uniform(0.5, 2.0, oc.NIN)
    X = rng.normal(0, 1, (40, oc.NIN)) * sd + mu
    t = rng.uniform(0, 3, 40)
    loss, g = oc.loss_and_grad(theta, mu, sd, X, t)
    idx = rng.choice(oc.NPARAM, 60, replace=False)
    for p in idx:
        e = np.zeros(oc.NPARAM)
        e[p] = 1e-6
        num = (oc.loss_and_grad(theta + e, mu, sd, X, t)[0] - oc.loss_and_grad(theta - e, mu, sd, X, t)[0]) / 2e-6
        assert abs(num - g[p]) <= 1e-6 + 1e-5 * abs(g[p]), (p, num, g[p])
    assert abs(loss - np.mean((oc.forward(theta, mu, sd, X) - t) ** 2)) < 1e-12


def test_closure_oracle_filter_and_target_properties():
    """The box filter keeps a constant interior field away from walls and the least-squares
    target is zero for a uniform flow."""
    import oracle.closure as oc

    u = np.ones((6, 8, 10))
    b = oc.box_filter(u, 1.0)
    assert np.allclose(b, 1.0)
    bv = oc.box_filter(u, -1.0)  # velocities reflect at the walls
    assert np.allclose(bv[:, 2:-2, :], 1.0) and np.all(bv[:, 0, :] < 1.0)
    nut, _ = oc.target([u, 0 * u, 0 * u], (0.1, 0.2, 0.3), 1e-3)
    assert np.all(nut[:, 2:-2, :] == 0.0)
