"""ark_conservation_sums_noalloc: conservation sums over caller-owned device arrays with no
device allocation (static scratch), for callers whose device memory is already spoken for.

It must give what ark_conservation_sums gives for the same level of the same state.  Both sum
exact fixed-point terms, so the comparison is exact (well inside any tolerance).  Two calls in
a row on different states check that the shared scratch carries nothing from one call into
the next.  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _device_copy(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda")


def test_noalloc_sums_match_context_sums(ark, port):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    p = port.channel_params(48, 24, 20, seed=17)
    gp = ark.make_params(48, 24, 20, re_b=1.0 / p["nu"])
    L = ark.lib()
    with ark.Context(gp) as ctx:
        ctx.upload(port.channel_state(p))
        for call, steps in enumerate((3, 4)):
            ctx.step(steps)
            ctx.sync()
            want = ctx.sums()
            st = ctx.download(["ronCon", "u1nCon", "u2nCon", "u3nCon", "condition"])
            dev = [_device_copy(torch, st[n]) for n in ("ronCon", "u1nCon", "u2nCon", "u3nCon", "condition")]
            torch.cuda.synchronize()
            got = ark.Sums()
            rc = L.ark_conservation_sums_noalloc(ctypes.byref(gp), *[t.data_ptr() for t in dev], ctypes.byref(got))
            assert rc == 0, (call, rc)
            assert got.cells == want.cells == 48 * 24 * 20
            for f in ("mass", "momentum1", "momentum2", "momentum3", "kinetic"):
                assert getattr(got, f) == getattr(want, f), (call, f, getattr(got, f), getattr(want, f))


def test_noalloc_rejects_oversized_grid(ark):
    """Grids beyond the scratch's 67,108,864-cell limit are refused before any GPU work."""
    gp = ark.make_params(1024, 512, 256)
    got = ark.Sums()
    one = ctypes.c_void_p(1)
    assert ark.lib().ark_conservation_sums_noalloc(ctypes.byref(gp), one, one, one, one, one, ctypes.byref(got)) == 1
