"""ark_conservation_sums_noalloc: conservation sums over caller-owned device arrays with no
device allocation (static scratch), for callers whose device memory is already spoken for --
a grid that fills the GPU, or arrays handed out by another framework's caching allocator,
where a cudaMalloc/cudaFree per call would synchronize the device or fail.

It must give what ark_conservation_sums gives for the same level of the same state.  Both sum
exact fixed-point terms, so the comparison is exact (well inside any tolerance).  Two calls in
a row on different states check that the shared scratch carries nothing from one call into
the next; a grid of more than 65,536 cells, not a multiple of it, makes the second kernel add
several rows of partial sums.  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

FIELDS = ("ronCon", "u1nCon", "u2nCon", "u3nCon", "condition")


def _device_copy(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda")


@pytest.mark.gpu
@pytest.mark.parametrize("C", [(48, 24, 20), (72, 40, 30)])
def test_noalloc_sums_match_context_sums(ark, port, C):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    p = port.channel_params(*C, seed=17)
    gp = ark.make_params(*C, re_b=1.0 / p["nu"])
    L = ark.lib()
    with ark.Context(gp) as ctx:
        ctx.upload(port.channel_state(p))
        for call, steps in enumerate((3, 4)):
            ctx.step(steps)
            ctx.sync()
            want = ctx.sums()
            st = ctx.download(list(FIELDS))
            dev = [_device_copy(torch, st[n]) for n in FIELDS]
            torch.cuda.synchronize()
            got = ark.Sums()
            rc = L.ark_conservation_sums_noalloc(ctypes.byref(gp), *[t.data_ptr() for t in dev], ctypes.byref(got))
            assert rc == 0, (call, rc, L.ark_last_error())
            assert got.cells == want.cells == C[0] * C[1] * C[2]
            for f in ("mass", "momentum1", "momentum2", "momentum3", "kinetic"):
                assert getattr(got, f) == getattr(want, f), (call, f, getattr(got, f), getattr(want, f))


def test_noalloc_rejects_oversized_grid(ark):
    """One cell beyond the scratch's 67,108,864-cell limit is refused before any GPU work, with
    the reason in ark_last_error(); NULL arrays are refused the same way."""
    L = ark.lib()
    got = ark.Sums()
    one = ctypes.c_void_p(1)
    gp = ark.make_params(5, 1, 13421773)  # 67,108,865 cells
    assert L.ark_conservation_sums_noalloc(ctypes.byref(gp), one, one, one, one, one, ctypes.byref(got)) == 1
    assert b"67,108,864" in L.ark_last_error()
    assert L.ark_conservation_sums_noalloc(ctypes.byref(gp), None, one, one, one, one, ctypes.byref(got)) == 1
    assert b"NULL" in L.ark_last_error()


def test_noalloc_accepts_the_limit_without_a_gpu(ark):
    """Exactly 67,108,864 cells passes the size check: without a GPU the call gets as far as the
    device query and reports a CUDA error instead of a parameter error.  Skipped where a GPU is
    visible (the placeholder pointers must never reach a kernel)."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    L = ark.lib()
    got = ark.Sums()
    one = ctypes.c_void_p(1)
    gp = ark.make_params(1024, 256, 256)  # 67,108,864 cells
    assert L.ark_conservation_sums_noalloc(ctypes.byref(gp), one, one, one, one, one, ctypes.byref(got)) == 2
