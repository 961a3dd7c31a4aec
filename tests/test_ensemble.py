"""Ensembles: independent FP32 channels of different sizes and parameters, one launch per
phase.  Every member must equal the same channel advanced alone in an FP32 ark_ctx, bit for
bit, whatever kernel shapes the autotuner picks."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CELLS = ["roCon", "u1Con", "u2Con", "u3Con", "ronCon", "u1nCon", "u2nCon", "u3nCon"]
FACES = ["p1", "ro1", "u11", "u21", "u31", "p2", "ro2", "u12", "u22", "u32", "p3", "ro3", "u13", "u23", "u33"]


def bits_equal(a, b):
    return np.array_equal(np.ascontiguousarray(a).view(np.uint64), np.ascontiguousarray(b).view(np.uint64))


def members(ark):
    spec = [((32, 16, 16), 2000.0, 0.05, 1, 1), ((40, 24, 20), 3500.0, 0.10, 1, 1),
            ((24, 12, 30), 6000.0, 0.15, 0, 1), ((17, 9, 11), 2800.0, 0.08, 1, 0), ((70, 6, 5), 4000.0, 0.1, 0, 0)]
    out = []
    for q, (C, re, amp, px, pz) in enumerate(spec):
        p = ark.make_params(*C, re_b=re, precision=ark.FP32)
        p.periodic_x, p.periodic_z = px, pz
        out.append((p, ark.channel_init(p, seed=100 + q, amp=amp)))
    return out


def singles(ark, mem, steps):
    res = []
    for p, st in mem:
        with ark.Context(p) as c:
            c.upload(st)
            c.step(steps)
            c.sync()
            res.append((c.download(CELLS + FACES), c.scalars().dt))
    return res


def test_ensemble_matches_single_contexts(ark, port):
    mem = members(ark)
    want = singles(ark, mem, 9)
    with ark.Ensemble([p for p, _ in mem]) as E:
        for q, (_, st) in enumerate(mem):
            E.upload(q, st)
        E.step(9)
        E.sync()
        for q in range(len(mem)):
            got = E.download(q, CELLS + FACES)
            assert E.scalars(q).dt == want[q][1]
            for n in CELLS + FACES:
                assert bits_equal(port.interior(n, got[n]), port.interior(n, want[q][0][n])), (q, n)


@pytest.mark.parametrize("shape", [(2, 2, 32), (2, 0, 16), (0, 2, 64), (1, 2, 32), (4, 4, 32), (4, 2, 16), (1, 4, 64),
                                   (5, 5, 32), (5, 4, 16), (7, 5, 32), (6, 4, 16), (7, 0, 64), (9, 5, 32), (8, 4, 16),
                                   (9, 2, 64)])
def test_ensemble_shapes_match_single_contexts(ark, port, shape):
    """Every Phase1 shape (one cell per thread, marching, planes staged in shared memory with
    cp.async or TMA tensor copies, 64 x 4 tiles or 32 x 8 for the members whose width is an odd
    multiple of 32: a persistent kernel over every member's tiles; with the x3 sweep folded into
    Phase1 + stress, shapes 6 and 7, or the x1 and x3 sweeps, 8 and 9, and their seam faces by
    their own persistent kernels) gives each member the single-context bits."""
    mem = members(ark)
    want = singles(ark, mem, 5)
    with ark.Ensemble([p for p, _ in mem]) as E:
        E.set_shape(*shape)
        for q, (_, st) in enumerate(mem):
            E.upload(q, st)
        E.step(5)
        E.sync()
        for q in range(len(mem)):
            got = E.download(q, CELLS + FACES)
            for n in CELLS + FACES:
                assert bits_equal(port.interior(n, got[n]), port.interior(n, want[q][0][n])), (shape, q, n)


def test_ensemble_autotune_keeps_results(ark, port):
    """The autotuner advances the live state while it times the candidate shapes; the
    result is the same as plain steps."""
    mem = members(ark)
    with ark.Ensemble([p for p, _ in mem]) as E:
        for q, (_, st) in enumerate(mem):
            E.upload(q, st)
        E.step(2)
        choice = E.autotune(1)
        assert choice["segment"] in (16, 32, 64)
        kt = E.kernel_times(2)
        a = choice["march_phase1_stress"]
        p1 = "phase1_stress_sweep_x1_x3" if a in (8, 9) else "phase1_stress_sweep_x3" if a in (6, 7) else "phase1_stress_forces"
        assert [n for n, _ in kt] == ["finalize_dt", "wrap_con", p1, "sweep_x1_seams" if a in (8, 9) else "sweep_x1", "sweep_x2",
                                      "sweep_x3_seams" if a in (6, 7, 8, 9) else "sweep_x3", "phase1_forces"]
        assert all(ms > 0 for _, ms in kt)
        done = E.scalars(0).nstep
        E.sync()
        want = singles(ark, mem, done)
        for q in range(len(mem)):
            got = E.download(q, CELLS + FACES)
            for n in CELLS + FACES:
                assert bits_equal(port.interior(n, got[n]), port.interior(n, want[q][0][n])), (q, n)
        prof, ws = E.mean_profile(1)
        assert prof.shape == (24,) and np.isfinite(ws).all()


def test_ensemble_rejects_fp64_members(ark):
    p = ark.make_params(16, 8, 8)
    with pytest.raises(ark.ArkError):
        ark.Ensemble([p])
