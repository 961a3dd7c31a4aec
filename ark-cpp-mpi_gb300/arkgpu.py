"""ctypes binding of libark_gb300.so (include/ark_gpu.h) for Python callers and tests.

This is a thin mirror of the C ABI: every method is one C call and raises ArkError on a
non-zero status.  There is no CPU fallback: if the shared library is missing, loading
raises.  Host arrays are numpy float64 arrays in the reference's Arr3d layout
(C-order shape (C3+2, C2+2, C1+2) for cells, (C3+3, C2+3, C1+3) for faces).
"""
from __future__ import annotations

import ctypes
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# ARK_GPU_LIB selects another build of the library (the bounds-checked one in lib_check/)
LIB_PATH = os.environ.get("ARK_GPU_LIB") or os.path.join(HERE, "lib", "libark_gb300.so")

FP64, FP32 = 0, 1

CELL_FIELDS = ("roCon", "u1Con", "u2Con", "u3Con", "ronCon", "u1nCon", "u2nCon", "u3nCon", "condition")
FACE_FIELDS = ("p1", "ro1", "u11", "u21", "u31", "p2", "ro2", "u12", "u22", "u32",
               "p3", "ro3", "u13", "u23", "u33")
STATE_FIELDS = CELL_FIELDS + FACE_FIELDS

# Every symbol include/ark_gpu.h declares.
EXPORTS = ("ark_create", "ark_destroy", "ark_last_error", "ark_status_string", "ark_cell_count",
           "ark_face_count", "ark_upload", "ark_download", "ark_get_array", "ark_put_array",
           "ark_time_step_size", "ark_phase1", "ark_stress_tensor", "ark_use_forces", "ark_phase2",
           "ark_boundary_fill", "ark_boundary_conditions", "ark_set_dt", "ark_step", "ark_sync", "ark_time_steps",
           "ark_get_scalars", "ark_set_scalars", "ark_conservation_sums", "ark_channel_init",
           "ark_kernel_times", "ark_kernel_name", "ark_step_kernel_name", "ark_alloc_host_state", "ark_free_host_state",
           "ark_conservation_sums_noalloc", "ark_mean_profile", "ark_selftest_division", "ark_selftest_staging_timeout",
           "ark_ensemble_create", "ark_ensemble_destroy", "ark_ensemble_last_error", "ark_ensemble_size",
           "ark_ensemble_upload", "ark_ensemble_download", "ark_ensemble_step", "ark_ensemble_sync",
           "ark_ensemble_time_steps", "ark_ensemble_get_scalars", "ark_ensemble_mean_profile",
           "ark_ensemble_autotune", "ark_ensemble_set_shape", "ark_ensemble_kernel_times", "ark_ensemble_kernel_name",
           "ark_ensemble_step_kernel_name",
           "ark_write_vtk", "ark_average_values", "ark_set_averaging", "ark_write_average_vtk",
           "ark_kinetic_energy", "ark_write_energy", "ark_vorticity", "ark_selftest_staging",
           "ark_closure_last_error", "ark_closure_data_create", "ark_closure_data_destroy", "ark_closure_data_size",
           "ark_closure_data_clear", "ark_closure_data_get", "ark_closure_data_append", "ark_closure_sample",
           "ark_mlp_create", "ark_mlp_destroy", "ark_mlp_set", "ark_mlp_get", "ark_mlp_fit_normalization",
           "ark_mlp_gradient", "ark_mlp_train", "ark_mlp_predict", "ark_set_closure",
           "ark_closure_data_filtered_stats", "ark_plane_stats", "ark_autotune", "ark_mlp_predict_tc",
           "ark_slabs_create", "ark_slabs_destroy", "ark_slabs_count", "ark_slabs_upload", "ark_slabs_download",
           "ark_slabs_step", "ark_slabs_sync", "ark_slabs_time_steps", "ark_slabs_get_scalars",
           "ark_slabs_conservation_sums", "ark_slab_plan", "ark_slab_halo_planes", "ark_bounds_check")


VTK_LAYOUTS = {"full": 0, "reference": 1}


def staging_selftest(C1, C2, C3, planes_per_block=0):
    """(problems, first message) of the staged Phase1's copy plan for a grid (host only)."""
    buf = ctypes.create_string_buffer(512)
    n = lib().ark_selftest_staging(int(C1), int(C2), int(C3), int(planes_per_block), buf, 512)
    return n, buf.value.decode()


class ArkError(RuntimeError):
    def __init__(self, fn, status, text):
        super().__init__(f"{fn} -> {status}: {text}")
        self.status = status


class Params(ctypes.Structure):
    _fields_ = [("n1_cells", ctypes.c_int), ("n2_cells", ctypes.c_int), ("n3_cells", ctypes.c_int),
                ("lx", ctypes.c_double), ("ly", ctypes.c_double), ("lz", ctypes.c_double),
                ("vis", ctypes.c_double), ("sound", ctypes.c_double), ("ro0", ctypes.c_double),
                ("cfl", ctypes.c_double), ("periodic_x", ctypes.c_int), ("periodic_z", ctypes.c_int),
                ("precision", ctypes.c_int), ("forcing", ctypes.c_int), ("u_target", ctypes.c_double),
                ("keep_stress", ctypes.c_int), ("device", ctypes.c_int)]


_DP = ctypes.POINTER(ctypes.c_double)


class HostState(ctypes.Structure):
    _fields_ = [(n, _DP) for n in STATE_FIELDS]


class Scalars(ctypes.Structure):
    _fields_ = [("dt", ctypes.c_double), ("time", ctypes.c_double), ("nstep", ctypes.c_longlong),
                ("bulk_velocity", ctypes.c_double), ("bulk_force", ctypes.c_double)]


class Sums(ctypes.Structure):
    _fields_ = [("mass", ctypes.c_double), ("momentum1", ctypes.c_double), ("momentum2", ctypes.c_double),
                ("momentum3", ctypes.c_double), ("kinetic", ctypes.c_double), ("cells", ctypes.c_longlong)]


_lib = None


def lib():
    """Load libark_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.isfile(LIB_PATH):
            raise FileNotFoundError(f"{LIB_PATH} missing: run ark-cpp-mpi_gb300/ark_build.py")
        L = ctypes.CDLL(LIB_PATH)
        vp, ip = ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)
        L.ark_create.restype = vp
        L.ark_create.argtypes = [ctypes.POINTER(Params), ip]
        L.ark_destroy.argtypes = [vp]
        L.ark_last_error.restype = ctypes.c_char_p
        L.ark_status_string.restype = ctypes.c_char_p
        L.ark_status_string.argtypes = [ctypes.c_int]
        L.ark_cell_count.restype = ctypes.c_size_t
        L.ark_cell_count.argtypes = [ctypes.POINTER(Params)]
        L.ark_face_count.restype = ctypes.c_size_t
        L.ark_face_count.argtypes = [ctypes.POINTER(Params)]
        L.ark_upload.argtypes = [vp, ctypes.POINTER(HostState)]
        L.ark_download.argtypes = [vp, ctypes.POINTER(HostState)]
        L.ark_get_array.argtypes = [vp, ctypes.c_char_p, _DP]
        L.ark_put_array.argtypes = [vp, ctypes.c_char_p, _DP]
        for fn in ("ark_time_step_size", "ark_phase1", "ark_stress_tensor", "ark_use_forces", "ark_phase2",
                   "ark_sync", "ark_selftest_staging_timeout"):
            getattr(L, fn).argtypes = [vp]
        L.ark_boundary_fill.argtypes = [vp, ctypes.c_int]
        L.ark_boundary_conditions.argtypes = [vp] + [ctypes.c_int] * 4
        L.ark_set_dt.argtypes = [vp, ctypes.c_double]
        L.ark_step.argtypes = [vp, ctypes.c_int]
        L.ark_time_steps.argtypes = [vp, ctypes.c_int, _DP]
        L.ark_get_scalars.argtypes = [vp, ctypes.POINTER(Scalars)]
        L.ark_set_scalars.argtypes = [vp, ctypes.POINTER(Scalars)]
        L.ark_conservation_sums.argtypes = [vp, ctypes.POINTER(Sums)]
        L.ark_channel_init.argtypes = [ctypes.POINTER(Params), ctypes.c_uint64, ctypes.c_double,
                                       ctypes.POINTER(HostState)]
        L.ark_kernel_times.argtypes = [vp, ctypes.c_int, _DP, ctypes.c_int, ip]
        L.ark_kernel_name.restype = ctypes.c_char_p
        L.ark_kernel_name.argtypes = [ctypes.c_int]
        L.ark_step_kernel_name.restype = ctypes.c_char_p
        L.ark_step_kernel_name.argtypes = [vp, ctypes.c_int]
        L.ark_alloc_host_state.argtypes = [ctypes.POINTER(Params), ctypes.POINTER(HostState)]
        L.ark_free_host_state.argtypes = [ctypes.POINTER(HostState)]
        L.ark_mean_profile.argtypes = [vp, _DP, _DP]
        L.ark_write_vtk.argtypes = [vp, ctypes.c_char_p, ctypes.c_int]
        L.ark_average_values.argtypes = [vp]
        L.ark_set_averaging.argtypes = [vp, ctypes.c_int]
        L.ark_write_average_vtk.argtypes = [vp, ctypes.c_char_p, ctypes.c_double, ctypes.c_int]
        L.ark_kinetic_energy.argtypes = [vp, _DP]
        L.ark_write_energy.argtypes = [vp, ctypes.c_char_p]
        L.ark_vorticity.argtypes = [vp, _DP]
        L.ark_selftest_staging.argtypes = [ctypes.c_int] * 4 + [ctypes.c_char_p, ctypes.c_int]
        ll, FP = ctypes.c_longlong, ctypes.POINTER(ctypes.c_float)
        L.ark_closure_last_error.restype = ctypes.c_char_p
        L.ark_closure_data_create.restype = vp
        L.ark_closure_data_create.argtypes = [ll, ctypes.c_int, ip]
        L.ark_closure_data_destroy.argtypes = [vp]
        L.ark_closure_data_size.restype = ll
        L.ark_closure_data_size.argtypes = [vp]
        L.ark_closure_data_clear.argtypes = [vp]
        L.ark_closure_data_get.argtypes = [vp, ll, ll, FP, FP]
        L.ark_closure_data_append.argtypes = [vp, ll, FP, FP]
        L.ark_closure_sample.argtypes = [vp, vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double]
        L.ark_mlp_create.restype = vp
        L.ark_mlp_create.argtypes = [ctypes.c_ulonglong, ctypes.c_int, ip]
        L.ark_mlp_destroy.argtypes = [vp]
        L.ark_mlp_set.argtypes = [vp, _DP, _DP, _DP]
        L.ark_mlp_get.argtypes = [vp, _DP, _DP, _DP]
        L.ark_mlp_fit_normalization.argtypes = [vp, vp]
        L.ark_mlp_gradient.argtypes = [vp, vp, ll, ll, _DP, _DP]
        L.ark_mlp_train.argtypes = [vp, vp, ctypes.c_int, ll, ctypes.c_double, _DP]
        L.ark_mlp_predict.argtypes = [vp, vp, ll, ll, FP]
        L.ark_mlp_predict_tc.argtypes = [vp, vp, ll, ll, FP]
        L.ark_set_closure.argtypes = [vp, vp, ctypes.c_double]
        L.ark_closure_data_filtered_stats.argtypes = [vp, _DP]
        L.ark_plane_stats.argtypes = [vp, _DP]
        L.ark_autotune.argtypes = [vp, ctypes.c_int, ip]
        L.ark_slabs_create.restype = vp
        L.ark_slabs_create.argtypes = [ctypes.POINTER(Params), ctypes.c_int, ip]
        for fn in ("ark_slabs_destroy", "ark_slabs_sync", "ark_slabs_count"):
            getattr(L, fn).argtypes = [vp]
        L.ark_slabs_upload.argtypes = [vp, ctypes.POINTER(HostState)]
        L.ark_slabs_download.argtypes = [vp, ctypes.POINTER(HostState)]
        L.ark_slabs_step.argtypes = [vp, ctypes.c_int]
        L.ark_slabs_time_steps.argtypes = [vp, ctypes.c_int, _DP]
        L.ark_slabs_get_scalars.argtypes = [vp, ctypes.POINTER(Scalars)]
        L.ark_slabs_conservation_sums.argtypes = [vp, ctypes.POINTER(Sums)]
        L.ark_slab_plan.argtypes = [ctypes.c_int] * 4 + [ip] * 4
        L.ark_bounds_check.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_longlong)]
        L.ark_slab_halo_planes.argtypes = [ctypes.c_int] * 5 + [ip] * 2
        L.ark_ensemble_create.restype = vp
        L.ark_ensemble_create.argtypes = [ctypes.POINTER(Params), ctypes.c_int, ip]
        L.ark_ensemble_last_error.restype = ctypes.c_char_p
        for fn in ("ark_ensemble_destroy", "ark_ensemble_sync"):
            getattr(L, fn).argtypes = [vp]
        L.ark_ensemble_size.argtypes = [vp]
        L.ark_ensemble_upload.argtypes = [vp, ctypes.c_int, ctypes.POINTER(HostState)]
        L.ark_ensemble_download.argtypes = [vp, ctypes.c_int, ctypes.POINTER(HostState)]
        L.ark_ensemble_step.argtypes = [vp, ctypes.c_int]
        L.ark_ensemble_time_steps.argtypes = [vp, ctypes.c_int, _DP]
        L.ark_ensemble_kernel_times.argtypes = [vp, ctypes.c_int, _DP, ctypes.c_int, ip]
        L.ark_ensemble_kernel_name.restype = ctypes.c_char_p
        L.ark_ensemble_kernel_name.argtypes = [ctypes.c_int]
        L.ark_ensemble_step_kernel_name.restype = ctypes.c_char_p
        L.ark_ensemble_step_kernel_name.argtypes = [vp, ctypes.c_int]
        L.ark_ensemble_get_scalars.argtypes = [vp, ctypes.c_int, ctypes.POINTER(Scalars)]
        L.ark_ensemble_mean_profile.argtypes = [vp, ctypes.c_int, _DP, _DP]
        L.ark_ensemble_autotune.argtypes = [vp, ctypes.c_int, ip]
        L.ark_ensemble_set_shape.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.ark_selftest_division.argtypes = [ctypes.c_longlong, ctypes.c_ulonglong, ctypes.POINTER(ctypes.c_longlong)]
        L.ark_conservation_sums_noalloc.argtypes = [ctypes.POINTER(Params)] + [ctypes.c_void_p] * 5 + [
            ctypes.POINTER(Sums)]
        _lib = L
    return _lib


def make_params(C1, C2, C3, re_b=2800.0, sound=10.0, rho0=1.0, cfl=0.2, lx=2 * math.pi, ly=2.0,
                lz=math.pi, ub=1.0, precision=FP64, forcing=True, keep_stress=False, device=0, vis=None):
    p = Params()
    p.n1_cells, p.n2_cells, p.n3_cells = C1, C2, C3
    p.lx, p.ly, p.lz = lx, ly, lz
    p.vis = (1.0 / re_b) if vis is None else vis
    p.sound, p.ro0, p.cfl = sound, rho0, cfl
    p.periodic_x = p.periodic_z = 1
    p.precision = precision
    p.forcing = int(bool(forcing))
    p.u_target = ub
    p.keep_stress = int(bool(keep_stress))
    p.device = device
    return p


def shapes(p: Params):
    return (p.n3_cells + 2, p.n2_cells + 2, p.n1_cells + 2), (p.n3_cells + 3, p.n2_cells + 3, p.n1_cells + 3)


def empty_state(p: Params, alloc=np.empty) -> dict:
    cs, fs = shapes(p)
    st = {n: alloc(cs) for n in CELL_FIELDS}
    st.update({n: alloc(fs) for n in FACE_FIELDS})
    return st


def host_struct(st: dict) -> HostState:
    h = HostState()
    for n in STATE_FIELDS:
        a = st.get(n)
        if a is not None:
            assert a.dtype == np.float64 and a.flags.c_contiguous, n
            setattr(h, n, a.ctypes.data_as(_DP))
    return h


def _check(fn, rc):
    if rc != 0:
        raise ArkError(fn, rc, lib().ark_last_error().decode(errors="replace"))


def channel_init(p: Params, seed=12345, amp=0.1) -> dict:
    st = empty_state(p)
    _check("ark_channel_init", lib().ark_channel_init(ctypes.byref(p), seed, amp, ctypes.byref(host_struct(st))))
    return st


class PinnedState:
    """A host state whose arrays live in page-locked memory (ark_alloc_host_state)."""

    def __init__(self, p: Params):
        self.h = HostState()
        _check("ark_alloc_host_state", lib().ark_alloc_host_state(ctypes.byref(p), ctypes.byref(self.h)))
        cs, fs = shapes(p)
        self.arrays = {}
        for n in STATE_FIELDS:
            shape = cs if n in CELL_FIELDS else fs
            ptr = getattr(self.h, n)
            self.arrays[n] = np.ctypeslib.as_array(ptr, shape=shape)

    def fill(self, st: dict):
        for n, a in st.items():
            self.arrays[n][...] = a

    def struct(self, with_condition=True) -> HostState:
        h = HostState()
        for n in STATE_FIELDS:
            if n == "condition" and not with_condition:
                continue
            setattr(h, n, getattr(self.h, n))
        return h

    def nbytes(self, with_condition=True):
        return sum(a.nbytes for n, a in self.arrays.items() if with_condition or n != "condition")

    def close(self):
        if getattr(self, "h", None) is not None:
            self.arrays = {}
            lib().ark_free_host_state(ctypes.byref(self.h))
            self.h = None

    def __del__(self):
        self.close()


class Context:
    """One ark_ctx (one CUDA stream on one device)."""

    def __init__(self, p: Params):
        self.p = p
        rc = ctypes.c_int(0)
        self.h = lib().ark_create(ctypes.byref(p), ctypes.byref(rc))
        if not self.h:
            _check("ark_create", rc.value or 2)
        self.cshape, self.fshape = shapes(p)

    def close(self):
        if getattr(self, "h", None):
            lib().ark_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _call(self, fn, *args):
        _check(fn, getattr(lib(), fn)(self.h, *args))

    def upload(self, st: dict):
        self._call("ark_upload", ctypes.byref(host_struct(st)))

    def download(self, names=STATE_FIELDS) -> dict:
        st = {}
        for n in names:
            st[n] = np.empty(self.cshape if n in CELL_FIELDS else self.fshape)
        self._call("ark_download", ctypes.byref(host_struct(st)))
        return st

    def download_into(self, st: dict):
        self._call("ark_download", ctypes.byref(host_struct(st)))

    def get(self, name, face=None):
        if name.startswith("averageU"):
            out = np.empty((self.p.n3_cells + 2, self.p.n2_cells + 3, self.p.n1_cells + 2))
            self._call("ark_get_array", name.encode(), out.ctypes.data_as(_DP))
            return out
        if face is None:
            face = not (name in CELL_FIELDS or name in ("f1", "f2", "f3", "nut"))
        out = np.empty(self.fshape if face else self.cshape)
        self._call("ark_get_array", name.encode(), out.ctypes.data_as(_DP))
        return out

    def put(self, name, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        self._call("ark_put_array", name.encode(), a.ctypes.data_as(_DP))

    def time_step_size(self):
        self._call("ark_time_step_size")

    def phase1(self):
        self._call("ark_phase1")

    def stress_tensor(self):
        self._call("ark_stress_tensor")

    def use_forces(self):
        self._call("ark_use_forces")

    def phase2(self):
        self._call("ark_phase2")

    def boundary_fill(self, axis):
        self._call("ark_boundary_fill", int(axis))

    def boundary_conditions(self, axis, x1_period, x2_period, x3_period):
        """BoundaryConditions(..., x1Period, x2Period, x3Period, ...).alongX<axis>() on "nCon"."""
        self._call("ark_boundary_conditions", int(axis), int(x1_period), int(x2_period), int(x3_period))

    def set_dt(self, dt):
        self._call("ark_set_dt", float(dt))

    def step(self, n=1):
        self._call("ark_step", int(n))

    def sync(self):
        self._call("ark_sync")

    def time_steps(self, n):
        ms = ctypes.c_double(0.0)
        self._call("ark_time_steps", int(n), ctypes.byref(ms))
        return ms.value

    def kernel_times(self, nsteps):
        """Mean device ms of each launch of the fused step: list of (name, ms)."""
        ms = (ctypes.c_double * 32)()
        cnt = ctypes.c_int(0)
        self._call("ark_kernel_times", int(nsteps), ms, 32, ctypes.byref(cnt))
        return [(lib().ark_step_kernel_name(self.h, q).decode(), ms[q]) for q in range(cnt.value)]

    def upload_struct(self, h: HostState):
        self._call("ark_upload", ctypes.byref(h))

    def download_struct(self, h: HostState):
        self._call("ark_download", ctypes.byref(h))

    def scalars(self) -> Scalars:
        s = Scalars()
        self._call("ark_get_scalars", ctypes.byref(s))
        return s

    def set_scalars(self, s: Scalars):
        self._call("ark_set_scalars", ctypes.byref(s))

    def mean_profile(self):
        """(mean u1 per y plane, (wall shear at y = -ly/2, at y = +ly/2))."""
        prof = np.empty(self.p.n2_cells)
        ws = np.empty(2)
        self._call("ark_mean_profile", prof.ctypes.data_as(_DP), ws.ctypes.data_as(_DP))
        return prof, ws

    def sums(self) -> Sums:
        s = Sums()
        self._call("ark_conservation_sums", ctypes.byref(s))
        return s

    # output and statistics (WriteDataParaView, AverageValues, WriteAverageValues, WriteEnergy)
    def write_vtk(self, path, layout="full"):
        self._call("ark_write_vtk", os.fsencode(path), VTK_LAYOUTS[layout])

    def average_values(self):
        self._call("ark_average_values")

    def set_averaging(self, on=True):
        self._call("ark_set_averaging", int(bool(on)))

    def write_average_vtk(self, path, start_time, layout="full"):
        self._call("ark_write_average_vtk", os.fsencode(path), float(start_time), VTK_LAYOUTS[layout])

    def kinetic_energy(self):
        e = ctypes.c_double(0.0)
        self._call("ark_kinetic_energy", ctypes.byref(e))
        return e.value

    def write_energy(self, path):
        self._call("ark_write_energy", os.fsencode(path))

    def autotune(self, steps_per_candidate=3):
        """Pick the fastest kernel shapes on the live state (which advances)."""
        c = (ctypes.c_int * 5)()
        self._call("ark_autotune", int(steps_per_candidate), c)
        # phase2_form: 0 three sweep kernels, 1 one sweep kernel, 2 sweeps + second Phase1 in one kernel
        # (3: the same with TMA copies), 4 the x1 sweep folded into Phase1 + stress
        return {"phase1_stress": c[0], "phase1": c[1], "segment": c[2], "us_per_step": c[3], "phase2_form": c[4]}

    def set_closure(self, mlp, u_tau=0.0):
        """Turn the learned closure on (mlp: an Mlp) or off (None) for ark_step."""
        self._call("ark_set_closure", mlp.h if mlp is not None else None, float(u_tau))

    def closure_sample(self, data, sx=4, sz=4, ox=0, oz=0, u_tau=1.0):
        self._call("ark_closure_sample", data.h, int(sx), int(sz), int(ox), int(oz), float(u_tau))
        data._last_c2 = self.p.n2_cells

    def plane_stats(self):
        """(n2_cells, 9): per y plane the means of u1, u2, u3, u1^2, u2^2, u3^2, u1u2, u1u3, u2u3."""
        out = np.empty((self.p.n2_cells, 9))
        self._call("ark_plane_stats", out.ctypes.data_as(_DP))
        return out

    def vorticity(self):
        """(n3_cells, n2_cells, n1_cells, 3) array of the vorticity R of WriteDataParaView."""
        out = np.empty((self.p.n3_cells, self.p.n2_cells, self.p.n1_cells, 3))
        self._call("ark_vorticity", out.ctypes.data_as(_DP))
        return out


def slab_plan(n3_cells, nslabs, slab, periodic_z=True):
    """(k_first, k_last, below, above) of one slab of a z split (host only)."""
    v = [ctypes.c_int(0) for _ in range(4)]
    rc = lib().ark_slab_plan(int(n3_cells), int(nslabs), int(slab), int(periodic_z), *[ctypes.byref(x) for x in v])
    if rc != 0:
        raise ArkError("ark_slab_plan", rc, lib().ark_last_error().decode())
    return tuple(x.value for x in v)


def slab_halo_planes(face, side, c3, c3_src, bounded):
    """(ghost plane written, source plane read) of one side of a slab's z halo (host only)."""
    d, s_ = ctypes.c_int(0), ctypes.c_int(0)
    rc = lib().ark_slab_halo_planes(int(face), int(side), int(c3), int(c3_src), int(bounded), ctypes.byref(d),
                                    ctypes.byref(s_))
    if rc != 0:
        raise ArkError("ark_slab_halo_planes", rc, lib().ark_last_error().decode())
    return d.value, s_.value


def bounds_check(reset=False):
    """Bounds-checked builds (ARK_GPU_LIB=.../lib_check/libark_gb300.so): (violations, first
    value, its bound, source line) recorded by the kernels so far; ArkError elsewhere."""
    out = (ctypes.c_longlong * 4)()
    rc = lib().ark_bounds_check(int(reset), out)
    if rc != 0:
        raise ArkError("ark_bounds_check", rc, lib().ark_last_error().decode())
    return tuple(int(x) for x in out)


class Slabs:
    """An ark_slabs group: one channel split along z into nslabs slab contexts on one device,
    with the z halo exchanges and shared reductions; host states are whole-domain."""

    def __init__(self, params: Params, nslabs: int):
        L = lib()
        self.params = params
        rc = ctypes.c_int(0)
        self.h = L.ark_slabs_create(ctypes.byref(params), int(nslabs), ctypes.byref(rc))
        if not self.h:
            raise ArkError("ark_slabs_create", rc.value or 2, L.ark_last_error().decode())

    def _call(self, fn, *args):
        rc = getattr(lib(), fn)(self.h, *args)
        if rc != 0:
            raise ArkError(fn, rc, lib().ark_last_error().decode(errors="replace"))

    def close(self):
        if getattr(self, "h", None):
            lib().ark_slabs_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def upload(self, st: dict):
        self._call("ark_slabs_upload", ctypes.byref(host_struct(st)))

    def download(self, names=STATE_FIELDS) -> dict:
        cs, fs = shapes(self.params)
        st = {n: np.empty(cs if n in CELL_FIELDS else fs) for n in names}
        self._call("ark_slabs_download", ctypes.byref(host_struct(st)))
        return st

    def step(self, n=1):
        self._call("ark_slabs_step", int(n))

    def sync(self):
        self._call("ark_slabs_sync")

    def time_steps(self, n):
        ms = ctypes.c_double(0.0)
        self._call("ark_slabs_time_steps", int(n), ctypes.byref(ms))
        return ms.value

    def scalars(self) -> Scalars:
        s = Scalars()
        self._call("ark_slabs_get_scalars", ctypes.byref(s))
        return s

    def sums(self) -> Sums:
        s = Sums()
        self._call("ark_slabs_conservation_sums", ctypes.byref(s))
        return s


class Ensemble:
    """An ark_ensemble: independent FP32 channels advanced together, one launch per phase."""

    def __init__(self, params: list):
        L = lib()
        self.params = list(params)
        arr = (Params * len(params))(*params)
        rc = ctypes.c_int(0)
        self.h = L.ark_ensemble_create(arr, len(params), ctypes.byref(rc))
        if not self.h:
            raise ArkError("ark_ensemble_create", rc.value or 2, L.ark_ensemble_last_error().decode())

    def _call(self, fn, *args):
        rc = getattr(lib(), fn)(self.h, *args)
        if rc != 0:
            raise ArkError(fn, rc, lib().ark_ensemble_last_error().decode(errors="replace"))

    def close(self):
        if getattr(self, "h", None):
            lib().ark_ensemble_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def upload(self, member, st: dict):
        self._call("ark_ensemble_upload", int(member), ctypes.byref(host_struct(st)))

    def download(self, member, names=STATE_FIELDS) -> dict:
        cs, fs = shapes(self.params[member])
        st = {n: np.empty(cs if n in CELL_FIELDS else fs) for n in names}
        self._call("ark_ensemble_download", int(member), ctypes.byref(host_struct(st)))
        return st

    def step(self, n=1):
        self._call("ark_ensemble_step", int(n))

    def sync(self):
        self._call("ark_ensemble_sync")

    def time_steps(self, n):
        ms = ctypes.c_double(0.0)
        self._call("ark_ensemble_time_steps", int(n), ctypes.byref(ms))
        return ms.value

    def kernel_times(self, nsteps):
        """Mean device ms of each launch of the ensemble step: list of (name, ms)."""
        ms = (ctypes.c_double * 32)()
        cnt = ctypes.c_int(0)
        self._call("ark_ensemble_kernel_times", int(nsteps), ms, 32, ctypes.byref(cnt))
        return [(lib().ark_ensemble_step_kernel_name(self.h, q).decode(), ms[q]) for q in range(cnt.value)]

    def scalars(self, member) -> Scalars:
        s = Scalars()
        self._call("ark_ensemble_get_scalars", int(member), ctypes.byref(s))
        return s

    def mean_profile(self, member):
        prof = np.empty(self.params[member].n2_cells)
        ws = np.empty(2)
        self._call("ark_ensemble_mean_profile", int(member), prof.ctypes.data_as(_DP), ws.ctypes.data_as(_DP))
        return prof, ws

    def autotune(self, steps_per_candidate=3):
        c = (ctypes.c_int * 4)()
        self._call("ark_ensemble_autotune", int(steps_per_candidate), c)
        return {"march_phase1_stress": c[0], "march_phase1": c[1], "segment": c[2], "us_per_step": c[3]}

    def set_shape(self, march_a, march_b, segment):
        self._call("ark_ensemble_set_shape", int(march_a), int(march_b), int(segment))


# ---- learned closure ------------------------------------------------------------------------

NIN, NH = 10, 32
NPARAM = NH * NIN + NH + NH * NH + NH + NH + 1


def _cl_check(fn, rc):
    if rc != 0:
        raise ArkError(fn, rc, lib().ark_closure_last_error().decode(errors="replace"))


class ClosureData:
    """Training samples (10 features, 1 target per row) on the device."""

    def __init__(self, capacity, device=0):
        rc = ctypes.c_int(0)
        self.h = lib().ark_closure_data_create(int(capacity), int(device), ctypes.byref(rc))
        if not self.h:
            raise ArkError("ark_closure_data_create", rc.value or 2, lib().ark_closure_last_error().decode())

    def close(self):
        if getattr(self, "h", None):
            lib().ark_closure_data_destroy(self.h)
            self.h = None

    __del__ = close

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __len__(self):
        return int(lib().ark_closure_data_size(self.h))

    def clear(self):
        _cl_check("ark_closure_data_clear", lib().ark_closure_data_clear(self.h))

    def get(self, first=0, count=None):
        count = len(self) - first if count is None else count
        f = np.empty((count, NIN), np.float32)
        t = np.empty(count, np.float32)
        _cl_check("ark_closure_data_get", lib().ark_closure_data_get(
            self.h, int(first), int(count), f.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
            t.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))
        return f, t

    def filtered_stats(self):
        """(n2_cells, 9) plane statistics of the field filtered by the last closure_sample."""
        out = np.empty((self._last_c2, 9))
        _cl_check("ark_closure_data_filtered_stats", lib().ark_closure_data_filtered_stats(self.h, out.ctypes.data_as(_DP)))
        return out

    def append(self, features, targets):
        f = np.ascontiguousarray(features, np.float32)
        t = np.ascontiguousarray(targets, np.float32)
        assert f.shape == (t.size, NIN)
        _cl_check("ark_closure_data_append", lib().ark_closure_data_append(
            self.h, int(t.size), f.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
            t.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))


class Mlp:
    """The closure network: BF16 working weights, FP32 master weights and Adam state."""

    def __init__(self, seed=1, device=0):
        rc = ctypes.c_int(0)
        self.h = lib().ark_mlp_create(int(seed), int(device), ctypes.byref(rc))
        if not self.h:
            raise ArkError("ark_mlp_create", rc.value or 2, lib().ark_closure_last_error().decode())

    def close(self):
        if getattr(self, "h", None):
            lib().ark_mlp_destroy(self.h)
            self.h = None

    __del__ = close

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set(self, params, mu, sd):
        p = np.ascontiguousarray(params, np.float64)
        m = np.ascontiguousarray(mu, np.float64)
        s = np.ascontiguousarray(sd, np.float64)
        assert p.size == NPARAM and m.size == NIN and s.size == NIN
        _cl_check("ark_mlp_set", lib().ark_mlp_set(self.h, p.ctypes.data_as(_DP), m.ctypes.data_as(_DP),
                                                    s.ctypes.data_as(_DP)))

    def get(self):
        p, m, s = np.empty(NPARAM), np.empty(NIN), np.empty(NIN)
        _cl_check("ark_mlp_get", lib().ark_mlp_get(self.h, p.ctypes.data_as(_DP), m.ctypes.data_as(_DP),
                                                    s.ctypes.data_as(_DP)))
        return p, m, s

    def fit_normalization(self, data):
        _cl_check("ark_mlp_fit_normalization", lib().ark_mlp_fit_normalization(self.h, data.h))

    def gradient(self, data, first=0, count=None):
        count = len(data) - first if count is None else count
        g = np.empty(NPARAM)
        loss = ctypes.c_double(0.0)
        _cl_check("ark_mlp_gradient", lib().ark_mlp_gradient(self.h, data.h, int(first), int(count),
                                                              g.ctypes.data_as(_DP), ctypes.byref(loss)))
        return loss.value, g

    def train(self, data, epochs=1, batch=4096, lr=1e-3):
        loss = ctypes.c_double(0.0)
        _cl_check("ark_mlp_train", lib().ark_mlp_train(self.h, data.h, int(epochs), int(batch), float(lr),
                                                        ctypes.byref(loss)))
        return loss.value

    def predict(self, data, first=0, count=None, tensor_cores=False):
        count = len(data) - first if count is None else count
        out = np.empty(count, np.float32)
        fn = "ark_mlp_predict_tc" if tensor_cores else "ark_mlp_predict"
        _cl_check(fn, getattr(lib(), fn)(self.h, data.h, int(first), int(count),
                                         out.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))
        return out
