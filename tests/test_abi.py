"""The C-ABI library without a GPU: it loads, exports every declared symbol, and rejects bad
input before touching the device."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    with open(os.path.join(ROOT, "include", "ark_gpu.h")) as f:
        text = f.read()
    return sorted(set(re.findall(r"\b(ark_[a-z0-9_]+)\s*\(", text)))


def test_exports_every_declared_symbol(ark):
    names = declared_functions()
    assert len(names) >= 20
    L = ark.lib()
    for n in names:
        assert hasattr(L, n), n
    assert sorted(ark.EXPORTS) == names


def test_status_strings(ark):
    L = ark.lib()
    for s in range(8):
        assert L.ark_status_string(s)
    assert L.ark_status_string(0) == b"ok"


def test_counts(ark):
    p = ark.make_params(8, 5, 3)
    assert ark.lib().ark_cell_count(ctypes.byref(p)) == 10 * 7 * 5
    assert ark.lib().ark_face_count(ctypes.byref(p)) == 11 * 8 * 6


@pytest.mark.parametrize("field,value,status", [
    ("n1_cells", 0, 1), ("n3_cells", 0, 1), ("n2_cells", -3, 1), ("sound", 0.0, 1), ("cfl", -1.0, 1), ("vis", -1.0, 1),
    ("ly", 0.0, 1), ("precision", 7, 1), ("n1_cells", 2000, 1)])
def test_create_rejects_bad_params(ark, field, value, status):
    p = ark.make_params(8, 6, 4) if field != "n1_cells" or value != 2000 else ark.make_params(8, 1300, 1300)
    setattr(p, field, value)
    rc = ctypes.c_int(-1)
    h = ark.lib().ark_create(ctypes.byref(p), ctypes.byref(rc))
    assert not h
    assert rc.value == status
    assert ark.lib().ark_last_error()


def test_null_arguments(ark):
    L = ark.lib()
    assert L.ark_upload(None, None) == 1
    assert L.ark_step(None, 1) == 1
    assert L.ark_sync(None) == 1
    assert L.ark_destroy(None) == 0
    rc = ctypes.c_int(-1)
    assert not L.ark_create(None, ctypes.byref(rc)) and rc.value == 1


def test_channel_init_layout(ark):
    """ark_channel_init: y ghost rows solid, walls at rest, faces are cell means."""
    p = ark.make_params(6, 4, 5)
    st = ark.channel_init(p, seed=1, amp=0.1)
    c = st["condition"]
    assert (c[:, 0, :] == 1).all() and (c[:, 5, :] == 1).all() and (c[:, 1:5, :] == 0).all()
    assert (st["u12"][1:6, 1, 1:7] == 0).all() and (st["u22"][1:6, 5, 1:7] == 0).all()
    u = st["u1nCon"]
    np.testing.assert_array_equal(st["u11"][1:6, 1:5, 2], 0.5 * (u[1:6, 1:5, 1] + u[1:6, 1:5, 2]))
    assert np.array_equal(st["u1Con"], st["u1nCon"])
    assert (st["p1"] == 0).all()


def test_channel_init_rejects_null(ark):
    p = ark.make_params(6, 4, 5)
    h = ark.HostState()
    assert ark.lib().ark_channel_init(ctypes.byref(p), 1, 0.1, ctypes.byref(h)) == 1


def test_no_gpu_means_error_not_crash(ark):
    """Without a usable device ark_create reports ARK_ERR_CUDA (on a GPU machine it succeeds)."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    p = ark.make_params(8, 6, 4)
    rc = ctypes.c_int(-1)
    assert not ark.lib().ark_create(ctypes.byref(p), ctypes.byref(rc))
    assert rc.value == 2


@pytest.mark.parametrize("C", [(1, 1, 1), (5, 3, 2), (64, 4, 32), (65, 5, 33), (130, 9, 70), (200, 7, 31),
                               (63, 12, 64), (17, 3, 1), (512, 8, 33), (96, 64, 64),
                               # the benchmark ensemble's member grids (the ensemble runs the same plan)
                               (32, 32, 32), (64, 32, 32), (64, 48, 48), (128, 64, 64)])
@pytest.mark.parametrize("kch", [0, 8, 32])
def test_staged_phase1_copy_plan(ark, C, kch):
    """The staged FP32 Phase1 copies row segments into shared memory 16 bytes at a time;
    before it runs anywhere its copy plan is checked on the host: every copy inside its array
    and stage and aligned, no byte copied twice, and every shared-memory read of every thread
    mapped to the element the one-cell kernel reads (and the same for the one-kernel Phase2 +
    second Phase1)."""
    n, msg = ark.staging_selftest(*C, planes_per_block=kch)
    assert n == 0, msg
