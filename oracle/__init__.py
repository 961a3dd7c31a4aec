"""Oracle for the CABARET time step -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg may use
this package, and only as the checker / the timed CPU baseline.  The product library never
imports, links or calls anything here.

Three pieces:

* :func:`channel_state` -- the seeded channel-flow initial state (a project definition:
  Poiseuille profile plus splitmix64 perturbations), as numpy arrays in the reference's
  Arr3d layout (``source/Arr3d.cpp:19-21``: i fastest; cell arrays (C+2) per axis, face
  arrays (C+3) per axis, ``source/main.cpp:198-251``).
* :class:`Port` -- ctypes binding of ``ark_oracle.c``, the plain-C restatement of the
  reference step (runs anywhere; built by ``make -C oracle port``).
* :class:`Reference` -- ctypes binding of ``oracle/_ref/libark_ref.so``, the reference's
  own ``source/main.cpp`` compiled in place against a single-rank MPI shim (only where the
  reference sources are present; built by ``make -C oracle ref``).
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "_build", "libark_oracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libark_ref.so")
# The reference checkout: $REF_DIR, else a checkout named "reference" beside this repository.
REF_DIR_DEFAULT = os.path.normpath(os.path.join(HERE, "..", "..", "reference"))

CELL_NAMES = ("roCon", "u1Con", "u2Con", "u3Con", "ronCon", "u1nCon", "u2nCon", "u3nCon",
              "f1", "f2", "f3", "condition")
FACE_NAMES = (
    "p1", "ro1", "u11", "u21", "u31",
    "p2", "ro2", "u12", "u22", "u32",
    "p3", "ro3", "u13", "u23", "u33")
STATE_NAMES = ("roCon", "u1Con", "u2Con", "u3Con", "ronCon", "u1nCon", "u2nCon", "u3nCon",
               "condition") + FACE_NAMES

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed: int, count: int) -> np.ndarray:
    """Outputs 1..count of Vigna's splitmix64 generator started at ``seed``."""
    idx = np.arange(1, count + 1, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = np.uint64(seed) + idx * _GOLDEN
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
    return z ^ (z >> np.uint64(31))


def uniform01(seed: int, count: int) -> np.ndarray:
    """Doubles in [0, 1): the top 53 bits of each splitmix64 output times 2^-53."""
    return (splitmix64(seed, count) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def channel_params(C1, C2, C3, re_b=2800.0, sound=10.0, rho0=1.0, cfl=0.2, lx=2 * math.pi,
                   ly=2.0, lz=math.pi, ub=1.0, amp=0.1, seed=12345):
    return dict(C1=C1, C2=C2, C3=C3, nu=1.0 / re_b, sound=sound, rho0=rho0, cfl=cfl, lx=lx, ly=ly,
                lz=lz, ub=ub, amp=amp, seed=seed)


def channel_state(p: dict) -> dict:
    """Seeded channel initial state (project definition, identical to ark_channel_init).

    Interior cell (i,j,k), visited k-major / i-fastest, draws three uniforms r1,r2,r3:
    u1 = 1.5*ub*(1 - y*y) + amp*(2*r1 - 1), u2 = amp*(2*r2 - 1), u3 = amp*(2*r3 - 1),
    rho = rho0, y = -ly/2 + (j - 0.5)*dy.  Ghost cells are periodic copies in x and z.
    Face values are the mean 0.5*(a + b) of the two adjacent cells; faces normal to y on
    the walls are 0; pressure is 0 and face density rho0 everywhere.  The "Con" level
    starts equal to "nCon".
    """
    C1, C2, C3 = p["C1"], p["C2"], p["C3"]
    ub, amp, rho0 = p["ub"], p["amp"], p["rho0"]
    cshape = (C3 + 2, C2 + 2, C1 + 2)
    fshape = (C3 + 3, C2 + 3, C1 + 3)
    dy = (0.5 * p["ly"] - -0.5 * p["ly"]) / C2
    r = uniform01(p["seed"], 3 * C1 * C2 * C3).reshape(C3, C2, C1, 3)
    j = np.arange(1, C2 + 1, dtype=np.float64)
    y = -0.5 * p["ly"] + (j - 0.5) * dy
    base = 1.5 * ub * (1.0 - y * y)
    u = [np.zeros(cshape) for _ in range(3)]
    u[0][1:-1, 1:-1, 1:-1] = base[None, :, None] + amp * (2.0 * r[..., 0] - 1.0)
    u[1][1:-1, 1:-1, 1:-1] = amp * (2.0 * r[..., 1] - 1.0)
    u[2][1:-1, 1:-1, 1:-1] = amp * (2.0 * r[..., 2] - 1.0)
    ro = np.full(cshape, rho0)
    for a in u + [ro]:
        a[1:-1, 1:-1, 0] = a[1:-1, 1:-1, C1]
        a[1:-1, 1:-1, C1 + 1] = a[1:-1, 1:-1, 1]
        a[0, 1:-1, 1:-1] = a[C3, 1:-1, 1:-1]
        a[C3 + 1, 1:-1, 1:-1] = a[1, 1:-1, 1:-1]
    cond = np.zeros(cshape)
    cond[:, 0, :] = 1.0
    cond[:, C2 + 1, :] = 1.0
    st = {}
    for lvl in ("", "n"):
        st[f"ro{lvl}Con"] = ro.copy()
        for m in range(3):
            st[f"u{m + 1}{lvl}Con"] = u[m].copy()
    st["condition"] = cond
    for d in range(3):
        st[f"p{d + 1}"] = np.zeros(fshape)
        rof = np.zeros(fshape)
        if d == 0:
            rof[1:C3 + 1, 1:C2 + 1, 1:C1 + 2] = rho0
        elif d == 1:
            rof[1:C3 + 1, 1:C2 + 2, 1:C1 + 1] = rho0
        else:
            rof[1:C3 + 2, 1:C2 + 1, 1:C1 + 1] = rho0
        st[f"ro{d + 1}"] = rof
        for m in range(3):
            f = np.zeros(fshape)
            c = u[m]
            if d == 0:   # faces i = 1..C1+1 between cells i-1 and i
                f[1:C3 + 1, 1:C2 + 1, 1:C1 + 2] = 0.5 * (c[1:-1, 1:-1, 0:C1 + 1] + c[1:-1, 1:-1, 1:C1 + 2])
            elif d == 1:  # faces j = 2..C2 interior; j = 1 and C2+1 are walls (0)
                f[1:C3 + 1, 2:C2 + 1, 1:C1 + 1] = 0.5 * (c[1:-1, 1:C2, 1:-1] + c[1:-1, 2:C2 + 1, 1:-1])
            else:
                f[1:C3 + 2, 1:C2 + 1, 1:C1 + 1] = 0.5 * (c[0:C3 + 1, 1:-1, 1:-1] + c[1:C3 + 2, 1:-1, 1:-1])
            st[f"u{m + 1}{d + 1}"] = f
    return st


def interior(name: str, a: np.ndarray) -> np.ndarray:
    """The part of an array the step defines: interior cells, or the computed faces."""
    if name in CELL_NAMES or name.endswith("Con"):
        return a[1:-1, 1:-1, 1:-1]
    d = int(name[-1])
    if d == 1:
        return a[1:-2, 1:-2, 1:-1]
    if d == 2:
        return a[1:-2, 1:-1, 1:-2]
    return a[1:-1, 1:-2, 1:-2]


def build(port=True, ref=None, ref_dir=None):
    """Compile the oracle C code (and the in-place reference build when its sources exist)."""
    ref_dir = ref_dir or os.environ.get("REF_DIR", REF_DIR_DEFAULT)
    targets = ["port"] if port else []
    if ref is None:
        ref = os.path.isfile(os.path.join(ref_dir, "source", "main.cpp"))
    if ref:
        targets.append("ref")
    if targets:
        subprocess.run(["make", "-s", "-C", HERE, f"REF_DIR={ref_dir}"] + targets, check=True)


_dbl_p = ctypes.POINTER(ctypes.c_double)


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_dbl_p)


class Port:
    """ctypes binding of the C restatement (ark_oracle.c)."""

    _lib = None

    @classmethod
    def lib(cls):
        if cls._lib is None:
            if not os.path.isfile(PORT_LIB):
                build(port=True, ref=False)
            L = ctypes.CDLL(PORT_LIB)
            L.aor_create.restype = ctypes.c_void_p
            L.aor_create.argtypes = [ctypes.c_int] * 3 + [ctypes.c_double] * 7 + [ctypes.c_int] * 2
            for fn in ("aor_destroy", "aor_time_step_size", "aor_phase1", "aor_stress_tensor",
                       "aor_use_forces", "aor_phase2"):
                getattr(L, fn).argtypes = [ctypes.c_void_p]
                getattr(L, fn).restype = None
            L.aor_len.restype = ctypes.c_size_t
            L.aor_len.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
            L.aor_put.argtypes = [ctypes.c_void_p, ctypes.c_char_p, _dbl_p]
            L.aor_get.argtypes = [ctypes.c_void_p, ctypes.c_char_p, _dbl_p]
            L.aor_set_forcing.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_double]
            L.aor_set_dt.argtypes = [ctypes.c_void_p, ctypes.c_double]
            for fn in ("aor_dt", "aor_time", "aor_last_ub", "aor_last_g", "aor_bulk_velocity"):
                getattr(L, fn).restype = ctypes.c_double
                getattr(L, fn).argtypes = [ctypes.c_void_p]
            L.aor_nstep.argtypes = [ctypes.c_void_p]
            L.aor_run.argtypes = [ctypes.c_void_p, ctypes.c_int]
            L.aor_set_threads.argtypes = [ctypes.c_int]
            cls._lib = L
        return cls._lib

    def __init__(self, p: dict, periodic_x=True, periodic_z=True, forcing=True, threads=None):
        L = self.lib()
        if threads:
            L.aor_set_threads(int(threads))
        self.p = p
        self.h = L.aor_create(p["C1"], p["C2"], p["C3"], p["lx"], p["ly"], p["lz"], p["nu"],
                              p["sound"], p["rho0"], p["cfl"], int(periodic_x), int(periodic_z))
        L.aor_set_forcing(self.h, int(forcing), p["ub"])
        self.cshape = (p["C3"] + 2, p["C2"] + 2, p["C1"] + 2)
        self.fshape = (p["C3"] + 3, p["C2"] + 3, p["C1"] + 3)

    def __del__(self):
        if getattr(self, "h", None):
            self.lib().aor_destroy(self.h)
            self.h = None

    def put(self, name, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        n = self.lib().aor_len(self.h, name.encode())
        assert n == a.size, (name, n, a.size)
        assert self.lib().aor_put(self.h, name.encode(), _ptr(a)) == 0

    def get(self, name):
        n = self.lib().aor_len(self.h, name.encode())
        shape = self.cshape if n == int(np.prod(self.cshape)) else self.fshape
        out = np.empty(shape)
        assert self.lib().aor_get(self.h, name.encode(), _ptr(out)) == 0
        return out

    def load(self, st: dict):
        for k, v in st.items():
            self.put(k, v)

    def run(self, n):
        self.lib().aor_run(self.h, int(n))

    def phase1(self):
        self.lib().aor_phase1(self.h)

    def phase2(self):
        self.lib().aor_phase2(self.h)

    def stress_tensor(self):
        self.lib().aor_stress_tensor(self.h)

    def use_forces(self):
        self.lib().aor_use_forces(self.h)

    def time_step_size(self):
        self.lib().aor_time_step_size(self.h)

    def set_dt(self, v):
        self.lib().aor_set_dt(self.h, float(v))

    @property
    def dt(self):
        return self.lib().aor_dt(self.h)

    @property
    def time(self):
        return self.lib().aor_time(self.h)

    @property
    def last_ub(self):
        return self.lib().aor_last_ub(self.h)

    @property
    def last_g(self):
        return self.lib().aor_last_g(self.h)

    def bulk_velocity(self):
        return self.lib().aor_bulk_velocity(self.h)


class Reference:
    """ctypes binding of the reference solver compiled in place (one live grid per process)."""

    _lib = None

    @classmethod
    def available(cls):
        return os.path.isfile(REF_LIB)

    @classmethod
    def lib(cls):
        if cls._lib is None:
            L = ctypes.CDLL(REF_LIB)
            L.ref_setup.argtypes = [ctypes.c_int] * 3 + [ctypes.c_double] * 8 + [ctypes.c_int] * 2
            L.ref_array_len.restype = ctypes.c_size_t
            L.ref_array_len.argtypes = [ctypes.c_char_p]
            L.ref_put.argtypes = [ctypes.c_char_p, _dbl_p]
            L.ref_get.argtypes = [ctypes.c_char_p, _dbl_p]
            L.ref_set_forcing.argtypes = [ctypes.c_int, ctypes.c_double]
            L.ref_set_dt.argtypes = [ctypes.c_double]
            for fn in ("ref_get_dt", "ref_get_time", "ref_last_ub", "ref_last_g"):
                getattr(L, fn).restype = ctypes.c_double
            L.ref_run.argtypes = [ctypes.c_int]
            L.ref_write_paraview.argtypes = [ctypes.c_char_p]
            L.ref_write_average.argtypes = [ctypes.c_char_p, ctypes.c_double]
            L.ref_write_energy.argtypes = [ctypes.c_char_p]
            L.ref_average_len.restype = ctypes.c_size_t
            L.ref_get_average.argtypes = [ctypes.c_int, _dbl_p]
            L.ref_boundary_conditions.argtypes = [ctypes.c_int] * 4 + [ctypes.c_double]
            cls._lib = L
        return cls._lib

    def __init__(self, p: dict, periodic_x=True, periodic_z=True, forcing=True, temp0=1.0):
        L = self.lib()
        L.ref_teardown()
        assert L.ref_setup(p["C1"], p["C2"], p["C3"], p["lx"], p["ly"], p["lz"], p["nu"], p["sound"],
                           p["rho0"], p["cfl"], temp0, int(periodic_x), int(periodic_z)) == 0
        L.ref_set_forcing(int(forcing), p["ub"])
        self.p = p
        self.cshape = (p["C3"] + 2, p["C2"] + 2, p["C1"] + 2)
        self.fshape = (p["C3"] + 3, p["C2"] + 3, p["C1"] + 3)
        # the passive temperature is carried by the reference; start it uniform
        for nm in ("tCon", "tnCon"):
            self.put(nm, np.full(self.cshape, temp0))
        for nm in ("t1", "t2", "t3"):
            self.put(nm, np.full(self.fshape, temp0))

    @classmethod
    def stock(cls):
        """The reference's own stock case, set up by its Input() and InitializeData()
        (200x60x1 backward-facing step, bounded in every direction, no forcing).  Returns the
        Reference and the matching parameter dict."""
        L = cls.lib()
        L.ref_teardown()
        assert L.ref_stock_setup() == 0
        cells = (ctypes.c_int * 3)()
        vals = (ctypes.c_double * 10)()
        L.ref_stock_params(cells, vals)
        p = dict(C1=cells[0], C2=cells[1], C3=cells[2], nu=vals[3], sound=vals[4], rho0=vals[5], cfl=vals[6],
                 lx=vals[7], ly=vals[8], lz=vals[9], ub=1.0, amp=0.0, seed=0)
        self = cls.__new__(cls)
        self.p = p
        self.cshape = (p["C3"] + 2, p["C2"] + 2, p["C1"] + 2)
        self.fshape = (p["C3"] + 3, p["C2"] + 3, p["C1"] + 3)
        return self, p

    def put(self, name, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        n = self.lib().ref_array_len(name.encode())
        assert n == a.size, (name, n, a.size)
        assert self.lib().ref_put(name.encode(), _ptr(a)) == 0

    def get(self, name):
        n = self.lib().ref_array_len(name.encode())
        shape = self.cshape if n == int(np.prod(self.cshape)) else self.fshape
        out = np.empty(shape)
        assert self.lib().ref_get(name.encode(), _ptr(out)) == 0
        return out

    def load(self, st: dict):
        for k, v in st.items():
            self.put(k, v)

    def run(self, n):
        self.lib().ref_run(int(n))

    def phase1(self):
        self.lib().ref_phase1()

    def phase2(self):
        self.lib().ref_phase2()

    def stress_tensor(self):
        self.lib().ref_stress_tensor()

    def use_forces(self):
        self.lib().ref_use_forces()

    def time_step_size(self):
        self.lib().ref_time_step_size()

    def set_dt(self, v):
        self.lib().ref_set_dt(float(v))

    @property
    def dt(self):
        return self.lib().ref_get_dt()

    @property
    def time(self):
        return self.lib().ref_get_time()

    @property
    def last_ub(self):
        return self.lib().ref_last_ub()

    @property
    def last_g(self):
        return self.lib().ref_last_g()

    def boundary_conditions(self, axis, x1_period, x2_period, x3_period, t0=1.0):
        """BoundaryConditions(u1nCon, u2nCon, u3nCon, ronCon, tnCon, x1Period, x2Period, x3Period,
        n1, n2, n3, t0).alongX<axis>() (source/BoundaryConditions.cpp:7-83)."""
        assert self.lib().ref_boundary_conditions(int(axis), int(x1_period), int(x2_period), int(x3_period),
                                                  float(t0)) == 0

    # the reference's writers and statistics (dir must end in '/')
    def write_paraview(self, dir_):
        assert self.lib().ref_write_paraview(dir_.encode()) == 0

    def average_values(self):
        assert self.lib().ref_average_values() == 0

    def write_average(self, dir_, start_time):
        assert self.lib().ref_write_average(dir_.encode(), float(start_time)) == 0

    def write_energy(self, dir_):
        assert self.lib().ref_write_energy(dir_.encode()) == 0

    def get_average(self, m):
        out = np.empty((self.p["C3"] + 2, self.p["C2"] + 3, self.p["C1"] + 2))
        assert self.lib().ref_get_average(int(m), _ptr(out)) == 0
        return out


def boundary_conditions(level: dict, axis: int, x2_period: bool, x3_period: bool) -> dict:
    """BoundaryConditions::alongX1/2/3 (source/BoundaryConditions.cpp:22-83) restated on a
    level {"ronCon", "u1nCon", "u2nCon", "u3nCon"} of [k, j, i] arrays; returns new arrays.
    On the interior of the other two axes: axis 1 copies the zero-gradient ghosts (the class
    never reads x1Period); axes 2 and 3 copy the periodic images, or set u = 0 and copy rho
    zero-gradient (no-slip).  The temperature lines are not restated (t is not carried)."""
    out = {n: a.copy() for n, a in level.items()}
    us = [out[n] for n in ("u1nCon", "u2nCon", "u3nCon")]
    ro = out["ronCon"]
    I, J, K = slice(1, -1), slice(1, -1), slice(1, -1)
    if axis == 1:
        for a in us + [ro]:
            a[K, J, -1] = a[K, J, -2]
            a[K, J, 0] = a[K, J, 1]
    elif axis == 2:
        for a in us:
            a[K, -1, I] = a[K, 1, I] if x2_period else 0.0
            a[K, 0, I] = a[K, -2, I] if x2_period else 0.0
        ro[K, -1, I] = ro[K, 1, I] if x2_period else ro[K, -2, I]
        ro[K, 0, I] = ro[K, -2, I] if x2_period else ro[K, 1, I]
    else:
        for a in us:
            a[-1, J, I] = a[1, J, I] if x3_period else 0.0
            a[0, J, I] = a[-2, J, I] if x3_period else 0.0
        ro[-1, J, I] = ro[1, J, I] if x3_period else ro[-2, J, I]
        ro[0, J, I] = ro[-2, J, I] if x3_period else ro[1, J, I]
    return out


# ---- writers and statistics, restated (numpy; host arrays in Arr3d layout [k, j, i]) ----

def _vtk_head(p):
    """Headers and coordinate blocks of WriteDataParaView / WriteAverageValues
    (main.cpp:2585-2645, 2755-2812): node counts n_g = C + 1, coordinates (i-1)*dx."""
    ng = (p["C1"] + 1, p["C2"] + 1, p["C3"] + 1)
    dx = (p["lx"] / p["C1"], (0.5 * p["ly"] - (-0.5 * p["ly"])) / p["C2"], p["lz"] / p["C3"])
    out = [b"# vtk DataFile Version 3.0\nvtk output\nBINARY\n",
           f"DATASET RECTILINEAR_GRID\nDIMENSIONS {ng[0]} {ng[1]} {ng[2]}".encode()]
    for name, n, d in zip("XYZ", ng, dx):
        out.append(f"\n{name}_COORDINATES {n} double\n".encode())
        out.append((np.arange(n, dtype=np.float64) * d).astype(">f8").tobytes())
    cells = p["C1"] * p["C2"] * p["C3"]
    out.append(f"\nCELL_DATA {cells}\nVECTORS U double\n".encode())
    return b"".join(out)


def _interior(a):
    return a[1:-1, 1:-1, 1:-1]


def vorticity(p, st):
    """The R vectors of WriteDataParaView (main.cpp:2716-2733) from the face arrays:
    shape (C3, C2, C1, 3)."""
    C1, C2, C3 = p["C1"], p["C2"], p["C3"]
    dx1, dx2, dx3 = p["lx"] / C1, (0.5 * p["ly"] - (-0.5 * p["ly"])) / C2, p["lz"] / C3
    I = np.s_[1:C3 + 1, 1:C2 + 1, 1:C1 + 1]
    Jp = np.s_[1:C3 + 1, 2:C2 + 2, 1:C1 + 1]
    Kp = np.s_[2:C3 + 2, 1:C2 + 1, 1:C1 + 1]
    Ip = np.s_[1:C3 + 1, 1:C2 + 1, 2:C1 + 2]
    d2u3 = (st["u32"][Jp] - st["u32"][I]) / dx2
    d3u2 = (st["u23"][Kp] - st["u23"][I]) / dx3
    d3u1 = (st["u13"][Kp] - st["u13"][I]) / dx3
    d1u3 = (st["u31"][Ip] - st["u31"][I]) / dx1
    d1u2 = (st["u21"][Ip] - st["u21"][I]) / dx1
    d2u1 = (st["u12"][Jp] - st["u12"][I]) / dx2
    return np.stack([d2u3 - d3u2, d3u1 - d1u3, d1u2 - d2u1], axis=-1)


def _place(parts, length):
    buf = bytearray(length)
    for off, b in parts:
        buf[off:off + len(b)] = b
    return bytes(buf)


def _blocks(p, blocks, layout):
    """Lay out a VTK file: the head, then for each (header, per-cell values of shape
    (C3, C2, C1, m)) its header and its big-endian block.  layout "full": every k plane at
    its place.  layout "reference": the reference's row offsets (main.cpp:2670-2671, 2693-2694,
    2737-2738, 2843-2844) have no k term, so each k plane overwrites the first plane's slot and
    only the last plane (k = C3) is in the file, at the start of its block; the rest of the
    block is a hole (zero bytes) and the file ends after the last block's first plane."""
    head = _vtk_head(p)
    parts, off = [(0, head)], len(head)
    end = off
    for hdr, v in blocks:
        if hdr:
            parts.append((off, hdr))
            off += len(hdr)
        data = v.astype(">f8")
        b = data.tobytes() if layout == "full" else data[-1].tobytes()
        parts.append((off, b))
        end = off + len(b)
        off += data.nbytes
    return _place(parts, end)


def paraview_bytes(p, st, layout="full"):
    """The bytes of WriteDataParaView's out_<nStep>.vtk (main.cpp:2577-2745) for the state
    st (u?nCon, ronCon and the face arrays): big-endian doubles (needSwap, main.cpp:120)."""
    u = np.stack([_interior(st[n]) for n in ("u1nCon", "u2nCon", "u3nCon")], axis=-1)
    return _blocks(p, [(b"", u), (b"\nscalars PC double\nLOOKUP_TABLE default\n", _interior(st["ronCon"])[..., None]),
                       (b"\nVECTORS R double\n", vorticity(p, st))], layout)


def average_add(avg, st, dt):
    """AverageValues (main.cpp:2878-2891): averageU_m += u_m nCon * dt over interior cells.
    avg: three arrays in the averageU layout (C3+2, C2+3, C1+2)."""
    for m, n in enumerate(("u1nCon", "u2nCon", "u3nCon")):
        a = st[n]
        avg[m][1:a.shape[0] - 1, 1:a.shape[1] - 1, 1:a.shape[2] - 1] += _interior(a) * dt


def average_bytes(p, avg, time_now, start_time, layout="full"):
    """The bytes of WriteAverageValues(start_time)'s average.vtk (main.cpp:2747-2849)."""
    C1, C2, C3 = p["C1"], p["C2"], p["C3"]
    v = np.stack([a[1:C3 + 1, 1:C2 + 1, 1:C1 + 1] / (time_now - start_time) for a in avg], axis=-1)
    return _blocks(p, [(b"", v)], layout)


def kinetic_energy_terms(st):
    """The per-cell terms of WriteEnergy (main.cpp:2853-2860), in the reference's loop order
    (i outer, then j, then k): (u1^2 + u2^2 + u3^2)/2 of the nCon level."""
    u1, u2, u3 = (_interior(st[n]) for n in ("u1nCon", "u2nCon", "u3nCon"))
    t = (u1 * u1 + u2 * u2 + u3 * u3) / 2
    return np.transpose(t, (2, 1, 0)).ravel()


def kinetic_energy(p, st):
    """WriteEnergy's value: the terms summed in the reference's order, times the domain volume
    (x3_t - x3_b) * (x2_n - x2_s) * (x1_e - x1_w) (main.cpp:2870)."""
    e = 0.0
    for t in kinetic_energy_terms(st).tolist():
        e += t
    return e * (p["lz"] * (0.5 * p["ly"] - (-0.5 * p["ly"])) * p["lx"])
