"""Output and statistics on the GPU: the VTK files of WriteDataParaView / WriteAverageValues,
AverageValues' time averages and WriteEnergy's kinetic energy, against the files the reference
itself wrote (tests/golden/writers.npz) and the oracle's restatement of the writers."""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
NEEDED = ["u1nCon", "u2nCon", "u3nCon", "ronCon", "p1", "ro1", "u11", "u21", "u31", "p2", "ro2", "u12", "u22",
          "u32", "p3", "ro3", "u13", "u23", "u33"]


def bits_equal(a, b):
    return np.array_equal(np.ascontiguousarray(a).view(np.uint64), np.ascontiguousarray(b).view(np.uint64))


def ctx_from(ark, port, p, precision=None, **kw):
    q = ark.make_params(p["C1"], p["C2"], p["C3"], vis=p["nu"], sound=p["sound"], rho0=p["rho0"], cfl=p["cfl"],
                        lx=p["lx"], ly=p["ly"], lz=p["lz"], ub=p["ub"],
                        precision=ark.FP64 if precision is None else precision, **kw)
    c = ark.Context(q)
    c.upload(port.channel_state(p))
    return c


def read(path):
    with open(path, "rb") as f:
        return f.read()


@pytest.mark.parametrize("tag", ["3d", "2d"])
def test_writers_match_reference_files(ark, port, tmp_path, tag):
    g = np.load(os.path.join(GOLD, "writers.npz"))
    p = json.loads(str(g[f"{tag}/params"]))
    with ctx_from(ark, port, p) as c:
        c.set_averaging(True)
        c.step(int(g["steps"]))
        c.sync()
        assert c.scalars().time == float(g[f"{tag}/time"])
        for m in (1, 2, 3):
            assert bits_equal(c.get(f"averageU{m}"), g[f"{tag}/averageU{m}"]), m
        c.write_vtk(str(tmp_path / "ref.vtk"), layout="reference")
        assert read(tmp_path / "ref.vtk") == g[f"{tag}/paraview"].tobytes()
        c.write_average_vtk(str(tmp_path / "avg.vtk"), 0.0, layout="reference")
        assert read(tmp_path / "avg.vtk") == g[f"{tag}/average"].tobytes()
        c.write_energy(str(tmp_path / "energy.txt"))
        assert read(tmp_path / "energy.txt") == g[f"{tag}/energy"].tobytes()
        # the full layout against the restatement, on the downloaded state
        st = c.download(NEEDED)
        c.write_vtk(str(tmp_path / "full.vtk"))
        assert read(tmp_path / "full.vtk") == port.paraview_bytes(p, st, "full")


def test_average_values_call_equals_averaging_in_step(ark, port):
    p = port.channel_params(12, 8, 6, seed=5)
    with ctx_from(ark, port, p) as a, ctx_from(ark, port, p) as b:
        a.set_averaging(True)
        a.step(4)
        for _ in range(4):
            b.step(1)
            b.average_values()
        a.sync()
        b.sync()
        for m in (1, 2, 3):
            assert bits_equal(a.get(f"averageU{m}"), b.get(f"averageU{m}")), m
        # switching off leaves the averages as they are
        a.set_averaging(False)
        a.step(2)
        assert bits_equal(a.get("averageU1"), b.get("averageU1"))


def test_fp32_averages_in_both_phase2_forms(ark, port, monkeypatch):
    """FP32: the averaging kernel at the end of the step reads the new level, which the one-kernel
    Phase2 + second Phase1 writes into the spare level; averages, and the step, equal the
    separate kernels' bit for bit, and the per-step calls equal the in-step averaging."""
    p = port.channel_params(40, 12, 10, seed=5)
    got = []
    for form in ("0", "2"):
        monkeypatch.setenv("ARK_PHASE2_FUSED", form)
        with ctx_from(ark, port, p, precision=ark.FP32) as a, ctx_from(ark, port, p, precision=ark.FP32) as b:
            a.set_averaging(True)
            a.step(5)
            for _ in range(5):
                b.step(1)
                b.average_values()
            a.sync()
            b.sync()
            for m in (1, 2, 3):
                assert bits_equal(a.get(f"averageU{m}"), b.get(f"averageU{m}")), (form, m)
            # the averages whole; the level's interior cells (ghost cells are each form's scratch)
            got.append([a.get(f"averageU{m}") for m in (1, 2, 3)] + [port.interior("u1nCon", a.get("u1nCon"))])
    for x, y in zip(got[0], got[1]):
        assert bits_equal(x, y)


@pytest.mark.parametrize("C,prec", [((64, 32, 32), "fp64"), ((128, 96, 96), "fp64"), ((40, 24, 20), "fp32")])
def test_vtk_full_and_vorticity_match_restatement(ark, port, tmp_path, C, prec):
    """128x96x96 is streamed in two slabs of k planes (double-buffered); FP32 contexts write
    the same bytes as the restatement does from their downloaded (double) state."""
    p = port.channel_params(*C, re_b=5600.0, seed=17)
    with ctx_from(ark, port, p, precision=ark.FP32 if prec == "fp32" else ark.FP64) as c:
        c.step(6)
        c.sync()
        st = c.download(NEEDED)
        c.write_vtk(str(tmp_path / "o.vtk"))
        assert read(tmp_path / "o.vtk") == port.paraview_bytes(p, st, "full")
        assert bits_equal(c.vorticity(), port.vorticity(p, st))
        e = c.kinetic_energy()
        want = port.kinetic_energy(p, st)
        assert abs(e - want) <= 1e-13 * abs(want)


def test_write_errors(ark, port, tmp_path):
    p = port.channel_params(8, 6, 4, seed=1)
    with ctx_from(ark, port, p) as c:
        with pytest.raises(ark.ArkError) as e:
            c.write_vtk(str(tmp_path / "no_such_dir" / "x.vtk"))
        assert e.value.status == 7
        with pytest.raises(ark.ArkError) as e:
            c._call("ark_write_vtk", str(tmp_path / "y.vtk").encode(), 5)  # no such layout
        assert e.value.status == 1
        with pytest.raises(ark.ArkError) as e:
            c.write_average_vtk(str(tmp_path / "no_such_dir" / "a.vtk"), 0.0)
        assert e.value.status == 7
