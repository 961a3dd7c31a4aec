"""The bounds-checked build (-DARK_CHECK, ark-cpp-mpi_gb300/lib_check/): the kernels compare the
indices of their global-memory accesses and the cell coordinates their blocks decode with the
extents they must stay inside and record any violation (nothing traps).  compute-sanitizer is not
available everywhere this library runs, so this is the memory check of the small-grid suite.

The CPU tests check that the checked library loads, registers its translation units' records and
answers through ark_bounds_check (the ordinary one refuses).  The GPU test runs the small-grid
parity tests -- the reference's goldens, every Phase1 shape and Phase2 form, bounded axes, slab
groups, ensembles, the closure -- in a child process on the checked library; conftest.py makes
each of them also assert that no index went out of range."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "ark-cpp-mpi_gb300")


def checked_lib():
    import ark_build

    return ark_build.build(check=True)


def run_child(code, lib):
    env = dict(os.environ, ARK_GPU_LIB=lib)
    return subprocess.run([sys.executable, "-c", code], cwd=ROOT, env=env, capture_output=True, text=True, timeout=300)


PROBE = """
import sys
sys.path.insert(0, {pkg!r})
import arkgpu
try:
    arkgpu.bounds_check()
    print("status 0")
except arkgpu.ArkError as e:
    print("status", e.status)
"""


def test_ordinary_build_refuses_bounds_check(ark):
    r = run_child(PROBE.format(pkg=PKG), ark.LIB_PATH)
    assert r.returncode == 0, r.stderr
    assert r.stdout.split() == ["status", "6"]


def test_checked_build_answers_bounds_check():
    """Without a GPU the checked library gets as far as the device (CUDA error, not 'unsupported');
    with one, a fresh process has no violations."""
    r = run_child(PROBE.format(pkg=PKG), checked_lib())
    assert r.returncode == 0, r.stderr
    assert r.stdout.split() in (["status", "2"], ["status", "0"])


SMALL_GRID_TESTS = [
    "tests/test_gpu_parity.py::test_step_pieces_match_reference_bitwise",
    "tests/test_gpu_parity.py::test_fused_step_matches_reference_small",
    "tests/test_gpu_parity.py::test_fused_step_matches_reference_digests",
    "tests/test_gpu_parity.py::test_per_phase_api_equals_fused_step",
    "tests/test_gpu_parity.py::test_boundary_conditions_match_reference_class",
    "tests/test_gpu_parity.py::test_fp32_per_phase_equals_fused",
    "tests/test_gpu_parity.py::test_fp32_steps_and_pieces_interleaved_in_both_phase2_forms",
    "tests/test_gpu_parity.py::test_phase1_kernel_shapes_agree",
    "tests/test_gpu_parity.py::test_bounded_edges_match_reference",
    "tests/test_gpu_parity.py::test_reference_stock_case_on_gpu",
    "tests/test_gpu_parity.py::test_bounded_axes_match_oracle",
    "tests/test_gpu_parity.py::test_fused_phase2_agrees",
    "tests/test_gpu_parity.py::test_phase2_phase1_kernel_agrees",
    "tests/test_gpu_parity.py::test_x1_sweep_folded_into_phase1_agrees",
    "tests/test_gpu_parity.py::test_x1_sweep_folded_with_solids",
    "tests/test_gpu_parity.py::test_folded_sweeps_around_a_solid_block",
    "tests/test_gpu_parity.py::test_folded_x1_sweep_with_distinct_periodic_end_faces",
    "tests/test_gpu_slabs.py",
    "tests/test_ensemble.py",
    "tests/test_gpu_closure.py",
]


@pytest.mark.gpu
def test_small_grid_suite_under_the_checked_build():
    lib = checked_lib()
    env = dict(os.environ, ARK_GPU_LIB=lib)
    r = subprocess.run([sys.executable, "-m", "pytest", "-q", "-m", "gpu", "-p", "no:cacheprovider"] + SMALL_GRID_TESTS,
                       cwd=ROOT, env=env, capture_output=True, text=True, timeout=1800)
    print(r.stdout[-3000:])
    assert r.returncode == 0, r.stdout[-4000:] + r.stderr[-2000:]
    assert " passed" in r.stdout and "failed" not in r.stdout
