"""ctypes binding of libpcgb300.so (declarations in include/pcgb300.h).

Loading the library never falls back to anything else: if it is missing or
does not load, :func:`load` raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .build import LIB as _LIB
from .build import LIB_SGL as _LIB_SGL
from .build import build as _do_build

NSLOT = 10
(S_DT1MAX, S_U2SUM, S_U2MAX, S_B2SUM, S_B2MAX, S_EKINSUM, S_RHOSUM, S_DIVB2SUM, S_J2SUM,
 S_ABSUM) = range(NSLOT)
DT_FIXED, DT_LAGGED, DT_CURRENT = 0, 1, 2
# boundary condition codes of pcgb_params.bc (boundcond.f90 bcx/bcy/bcz)
BC_CODES = {"p": 0, "s": 1, "a": 2, "a2": 3}


class Params(C.Structure):
    """Mirror of ``pcgb_params`` (include/pcgb300.h)."""
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("lentropy", C.c_int), ("precision", C.c_int), ("comp", C.c_int),
        ("xyz0", C.c_double * 3), ("Lxyz", C.c_double * 3),
        ("gamma", C.c_double), ("cs0", C.c_double), ("rho0", C.c_double), ("cp", C.c_double),
        ("nu", C.c_double), ("eta", C.c_double), ("chi", C.c_double), ("mu0", C.c_double),
        ("lforcing_cont", C.c_int),
        ("ampl_ff", C.c_double), ("kf", C.c_double), ("relhel", C.c_double),
        ("abc_a", C.c_double), ("abc_b", C.c_double), ("abc_c", C.c_double),
        ("ampl_fcont_uu", C.c_double),
        ("b_ext", C.c_double * 3),
        ("lohmic_heat", C.c_int), ("lviscosity_heat", C.c_int),
        ("cdt", C.c_double), ("cdtv", C.c_double),
        ("dt", C.c_double), ("dt_mode", C.c_int), ("diag_every", C.c_int),
        ("tile", C.c_int), ("zdepth", C.c_int), ("dfloat", C.c_int),
        ("lforcing_hel", C.c_int), ("seed_ff", C.c_int), ("force_hel", C.c_double),
        ("lupw_uu", C.c_int), ("lupw_lnrho", C.c_int), ("lmagnetic_forcing", C.c_int), ("pad_", C.c_int),
        ("bc", ((C.c_int * 2) * 8) * 3),
    ]

    def update(self, **kw) -> "Params":
        """Set fields by name; bcx/bcy/bcz take one entry per field in f-array order,
        each a code name ('p', 's', 'a', 'a2'), 'lower:upper', or a (lower, upper) pair."""
        for k, v in kw.items():
            if k in ("xyz0", "Lxyz", "b_ext"):
                getattr(self, k)[:] = list(v)
            elif k in ("bcx", "bcy", "bcz"):
                self.set_bc("xyz".index(k[-1]), v)
            elif k == "bc":   # the whole [3][8][2] table
                for d in range(3):
                    for f in range(8):
                        self.bc[d][f][0], self.bc[d][f][1] = int(v[d][f][0]), int(v[d][f][1])
            else:
                setattr(self, k, v)
        return self

    def set_bc(self, direction: int, entries) -> "Params":
        for f in range(8):
            self.bc[direction][f][0] = self.bc[direction][f][1] = 0
        for f, e in enumerate(entries):
            if isinstance(e, str):
                lo, _, hi = e.strip().partition(":")
                pair = (BC_CODES[lo.strip()], BC_CODES[(hi or lo).strip()])
            elif isinstance(e, int):
                pair = (e, e)
            else:
                pair = (int(e[0]), int(e[1]))
            self.bc[direction][f][0], self.bc[direction][f][1] = pair
        return self

    def periodic(self, direction: int) -> bool:
        nf = 8 if self.lentropy else 7
        return all(self.bc[direction][f][s] == 0 for f in range(nf) for s in (0, 1))

    def spacing(self, direction: int) -> float:
        """grid.f90:123-151: L/n on a periodic axis, L/(n-1) otherwise."""
        n = (self.nx, self.ny, self.nz)[direction]
        return self.Lxyz[direction] / (n if self.periodic(direction) else n - 1)

    def axis(self, direction: int) -> np.ndarray:
        """Grid points of one axis with ghosts: x0 + (i - 3 + o) dx, o = 1/2 periodic, 0 otherwise."""
        n = (self.nx, self.ny, self.nz)[direction]
        o = 0.5 if self.periodic(direction) else 0.0
        return self.xyz0[direction] + (np.arange(n + 6) - 3 + o) * self.spacing(direction)

    def as_dict(self) -> dict:
        def plain(v):
            return [plain(e) for e in v] if hasattr(v, "__len__") else v
        return {name: plain(getattr(self, name)) for name, _ in self._fields_}


_lib = None

# Every entry point the header declares (checked by the CPU tests).
EXPORTS = [
    "pcgb_default_params", "pcgb_set_params", "pcgb_last_error", "pcgb_error_string", "pcgb_clear_error",
    "pcgb_set_stream", "pcgb_get_stream",
    "registerGPU", "initializeGPU", "finalizeGPU", "getFArrayIn", "substepGPU", "beforeBoundaryGPU",
    "afterSubStepGPU", "radTransfer", "copyFarray", "loadFarray", "reloadConfig", "updateInConfigArr",
    "updateInConfigArrName", "updateInConfigScal", "updateInConfigScalName", "updateInConfigVec",
    "updateInConfigVecName", "prepareForFirstSubstep", "random_initial_condition", "getGPUReducedVars",
    "testBCs", "splitUpdate", "copyVBApointers",
    "tf_save_checkpoint_c_api", "tf_save_model_c_api", "tf_load_model_c_api",
    "tf_load_model_checkpoint_c_api", "tf_create_model_c_api", "tf_train_c_api", "tf_infer_c_api",
    "print_debug",
    "initialize_gpu_c_", "register_gpu_c_", "finalize_gpu_c_", "get_farray_ptr_gpu_c_",
    "before_boundary_gpu_c_", "update_after_substep_gpu_c_", "rhs_gpu_c_", "copy_farray_c_",
    "load_farray_c_", "reload_gpu_config_c_", "update_on_gpu_scal_by_ind_c_",
    "update_on_gpu_vec_by_ind_c_", "update_on_gpu_arr_by_ind_c_", "update_on_gpu_scal_by_name_c_",
    "update_on_gpu_vec_by_name_c_", "update_on_gpu_arr_by_name_c_", "gpu_prepare_for_first_substep_c_",
    "radtransfer_gpu_c_", "get_gpu_reduced_vars_c_", "test_bcs_c_", "split_update_gpu_c_",
    "tf_train_c_", "tf_infer_c_", "tf_create_model_c_", "print_snapshot_c_", "tf_load_model_c_",
    "tf_load_model_checkpoint_c_", "tf_save_model_c_", "tf_save_checkpoint_c_",
    "pcgb_box_set_kvectors", "pcgb_set_kvectors",
    "pcgb_get_dt", "pcgb_get_time", "pcgb_request_diagnostics", "pcgb_time_step",
    "pcgb_box_create", "pcgb_box_destroy", "pcgb_box_load", "pcgb_box_store", "pcgb_box_load_f32",
    "pcgb_box_store_f32", "pcgb_box_init_field", "pcgb_box_steps",
    "pcgb_box_sync", "pcgb_box_diag", "pcgb_box_time", "pcgb_box_set_dt", "pcgb_box_bytes",
    "pcgb_box_info", "pcgb_batch_create", "pcgb_batch_destroy", "pcgb_batch_steps", "pcgb_autotune",
    "pcgb_launch_count", "pcgb_version", "pcgb_substep_noalloc", "pcgb_params_bytes", "pcgb_set_wait_limit", "pcgb_inject_wait_failure",
    "pcgb_server_create", "pcgb_server_submit", "pcgb_server_poll", "pcgb_server_drain", "pcgb_server_stats",
    "pcgb_server_destroy",
]


def lib_path() -> str:
    return _LIB


def load(build_if_missing: bool = True) -> C.CDLL:
    """Load libpcgb300.so (building it first if asked and absent)."""
    global _lib
    if _lib is None:
        _lib = _open(lib_path(), C.c_double, build_if_missing)
    return _lib


def load_sgl(build_if_missing: bool = True) -> C.CDLL:
    """Load libpcgb300_sgl.so: the plug-in entry points with REAL = float, for
    the reference's single-precision build (a library of its own, with its own
    engine state, as the reference links libastaroth_sgl.so)."""
    global _lib_sgl
    if _lib_sgl is None:
        _lib_sgl = _open(_LIB_SGL, C.c_float, build_if_missing)
    return _lib_sgl


_lib_sgl = None


def _open(path: str, real, build_if_missing: bool) -> C.CDLL:
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"{path} is missing; run build() first")
        _do_build()
    L = C.CDLL(path)
    P = C.POINTER(Params)
    vp = C.c_void_p
    dptr = C.POINTER(C.c_double)
    fptr = C.POINTER(C.c_float)
    rptr = C.POINTER(real)   # the Fortran build's REAL
    sig = {
        "pcgb_default_params": (None, [P]),
        "pcgb_set_params": (C.c_int, [P]),
        "pcgb_last_error": (C.c_int, []),
        "pcgb_error_string": (C.c_char_p, [C.c_int]),
        "pcgb_clear_error": (None, []),
        "pcgb_set_stream": (None, [vp]),
        "pcgb_get_stream": (vp, []),
        "initializeGPU": (None, [rptr, C.c_int, C.c_double, C.c_int, C.c_int, C.c_int, C.c_int]),
        "substepGPU": (None, [C.c_int, C.c_double]),
        "beforeBoundaryGPU": (None, [C.c_bool, C.c_int, C.c_double, C.c_bool]),
        "afterSubStepGPU": (None, []),
        "registerGPU": (None, []),
        "copyFarray": (None, [rptr]),
        "loadFarray": (None, []),
        "finalizeGPU": (None, []),
        "reloadConfig": (None, []),
        "prepareForFirstSubstep": (None, [C.c_double]),
        "getGPUReducedVars": (None, [rptr]),
        "copyVBApointers": (None, [C.POINTER(vp), C.POINTER(vp)]),
        "updateInConfigScalName": (C.c_int, [C.c_char_p, real]),
        "updateInConfigVecName": (C.c_int, [C.c_char_p, rptr]),
        "testBCs": (None, []),
        "pcgb_get_dt": (C.c_double, []),
        "pcgb_get_time": (C.c_double, []),
        "pcgb_request_diagnostics": (None, []),
        "pcgb_time_step": (C.c_int, [C.c_int]),
        "pcgb_box_create": (vp, [P]),
        "pcgb_box_destroy": (None, [vp]),
        "pcgb_box_load": (C.c_int, [vp, dptr, C.c_double]),
        "pcgb_box_store": (C.c_int, [vp, dptr]),
        "pcgb_box_load_f32": (C.c_int, [vp, fptr, C.c_double]),
        "pcgb_box_store_f32": (C.c_int, [vp, fptr]),
        "pcgb_box_init_field": (C.c_int, [vp, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                          C.c_double, C.c_ulonglong]),
        "pcgb_box_steps": (C.c_int, [vp, C.c_int]),
        "pcgb_box_sync": (C.c_int, [vp]),
        "pcgb_box_diag": (C.c_int, [vp, dptr, C.c_int]),
        "pcgb_box_time": (C.c_int, [vp, dptr, dptr, C.POINTER(C.c_longlong)]),
        "pcgb_box_set_dt": (C.c_int, [vp, C.c_double]),
        "pcgb_box_set_kvectors": (C.c_int, [vp, dptr, C.c_int, C.c_double]),
        "pcgb_set_kvectors": (C.c_int, [dptr, C.c_int, C.c_double]),
        "pcgb_box_bytes": (C.c_size_t, [vp]),
        "pcgb_box_info": (C.c_int, [vp, C.POINTER(C.c_int), C.c_int]),
        "pcgb_batch_create": (vp, [C.POINTER(vp), C.c_int, C.c_int]),
        "pcgb_batch_destroy": (None, [vp]),
        "pcgb_batch_steps": (C.c_int, [vp, C.c_int, C.c_int, C.c_int]),
        "pcgb_autotune": (C.c_int, [P, C.POINTER(C.c_int), C.POINTER(C.c_int), dptr]),
        "pcgb_substep_noalloc": (C.c_int, [P, C.c_int, C.c_double, vp, vp, vp, dptr, vp]),
        "pcgb_params_bytes": (C.c_size_t, [P]),
        "pcgb_set_wait_limit": (None, [C.c_uint]),
        "pcgb_inject_wait_failure": (None, [C.c_int]),
        "pcgb_server_create": (vp, [C.c_size_t, C.c_int, C.c_int]),
        "pcgb_server_submit": (C.c_longlong, [vp, P, C.c_int, C.c_ulonglong, C.c_double, C.c_double, vp]),
        "pcgb_server_poll": (C.c_int, [vp, C.c_longlong, dptr, dptr]),
        "pcgb_server_drain": (C.c_int, [vp, C.c_double]),
        "pcgb_server_stats": (C.c_int, [vp, dptr, C.c_int]),
        "pcgb_server_destroy": (None, [vp]),
        "pcgb_launch_count": (C.c_longlong, []),
        "pcgb_version": (C.c_char_p, []),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    return L


class PcgbError(RuntimeError):
    pass


def check(rc: int) -> None:
    """Raise for a failed call; the sticky library error is cleared once raised."""
    if rc:
        L = load()
        msg = L.pcgb_error_string(rc).decode()
        L.pcgb_clear_error()
        raise PcgbError(f"pcgb error {rc}: {msg}")


def last_error() -> tuple[int, str]:
    """The sticky library error (code, message), cleared by reading it."""
    L = load()
    rc = L.pcgb_last_error()
    msg = L.pcgb_error_string(rc).decode()
    L.pcgb_clear_error()
    return rc, msg


def default_params(**kw) -> Params:
    p = Params()
    load().pcgb_default_params(C.byref(p))
    return p.update(**kw)


def _dptr(a: np.ndarray):
    assert a.dtype == np.float64
    return a.ctypes.data_as(C.POINTER(C.c_double))


def nfields(p: Params) -> int:
    return 8 if p.lentropy else 7


def host_shape(p: Params) -> tuple:
    return (p.nx + 6, p.ny + 6, p.nz + 6, nfields(p))


class Box:
    """One periodic MHD domain resident on the GPU (``pcgb_box``)."""

    def __init__(self, p: Params):
        L = load()
        self.p = p
        self.h = L.pcgb_box_create(C.byref(p))
        if not self.h:
            rc, msg = last_error()
            raise PcgbError(f"pcgb_box_create failed ({rc}): {msg}")

    def close(self):
        if self.h:
            load().pcgb_box_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def load(self, f: np.ndarray, t: float = 0.0):
        f = np.asarray(f, dtype=np.float64, order="F")
        if f.shape != host_shape(self.p):
            raise ValueError(f"f has shape {f.shape}, expected {host_shape(self.p)}")
        if not f.flags.f_contiguous:
            f = np.asfortranarray(f)
        check(load().pcgb_box_load(self.h, _dptr(f), t))

    def store(self, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.zeros(host_shape(self.p), order="F")
        check(load().pcgb_box_store(self.h, _dptr(out)))
        return out

    def steps(self, n: int):
        check(load().pcgb_box_steps(self.h, n))

    def init_field(self, field: int, kind: str, ampl: float = 0.0, abc=(1.0, 1.0, 1.0), k: float = 1.0,
                   seed: int = 0):
        """Device-side seeded initial condition: kind 'zero', 'noise' or 'abc'."""
        kk = {"zero": 0, "noise": 1, "abc": 2}[kind]
        check(load().pcgb_box_init_field(self.h, field, kk, ampl, abc[0], abc[1], abc[2], k, seed))

    def sync(self):
        check(load().pcgb_box_sync(self.h))

    def diag_raw(self) -> np.ndarray:
        out = np.zeros(NSLOT + 3)
        check(load().pcgb_box_diag(self.h, _dptr(out), NSLOT + 3))
        return out

    def time(self):
        t, dt, ns = C.c_double(), C.c_double(), C.c_longlong()
        check(load().pcgb_box_time(self.h, C.byref(t), C.byref(dt), C.byref(ns)))
        return t.value, dt.value, ns.value

    def set_dt(self, dt: float):
        check(load().pcgb_box_set_dt(self.h, dt))

    def set_kvectors(self, kvec: np.ndarray, kav: float):
        """Helical forcing wavevectors, (3, nk) as in the reference's k.dat."""
        kv = np.ascontiguousarray(kvec, dtype=np.float64)
        check(load().pcgb_box_set_kvectors(self.h, _dptr(kv), kv.shape[1], kav))

    def nbytes(self) -> int:
        return int(load().pcgb_box_bytes(self.h))

    def info(self) -> dict:
        v = (C.c_int * 12)()
        check(load().pcgb_box_info(self.h, v, 12))
        keys = ["nx", "ny", "nz", "nf", "bytes_per_value", "tile", "zdepth", "tiles", "px", "xoff", "pairs", "dfloat"]
        return dict(zip(keys, list(v)))


class Batch:
    """Boxes of one class advanced together by persistent launches (``pcgb_batch``)."""

    def __init__(self, boxes: list[Box], persistent: bool = True):
        L = load()
        self.boxes = boxes
        arr = (C.c_void_p * len(boxes))(*[b.h for b in boxes])
        self.h = L.pcgb_batch_create(arr, len(boxes), int(persistent))
        if not self.h:
            rc, msg = last_error()
            raise PcgbError(f"pcgb_batch_create failed ({rc}): {msg}")

    def steps(self, n: int, use_graph: bool = True, graph_steps: int = 10):
        check(load().pcgb_batch_steps(self.h, n, int(use_graph), graph_steps))

    def close(self):
        if self.h:
            load().pcgb_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def diag_summary(raw: np.ndarray, ncells: int) -> dict:
    """Volume averages in the reference's print.in units (diagnostics.f90:274)."""
    return dict(urms=np.sqrt(raw[S_U2SUM] / ncells), umax=np.sqrt(raw[S_U2MAX]),
                brms=np.sqrt(raw[S_B2SUM] / ncells), bmax=np.sqrt(raw[S_B2MAX]),
                ekin=raw[S_EKINSUM] / ncells, rhom=raw[S_RHOSUM] / ncells,
                divbrms=np.sqrt(raw[S_DIVB2SUM] / ncells), jrms=np.sqrt(raw[S_J2SUM] / ncells),
                abm=raw[S_ABSUM] / ncells)


def autotune(p: Params):
    t, z, ms = C.c_int(), C.c_int(), C.c_double()
    check(load().pcgb_autotune(C.byref(p), C.byref(t), C.byref(z), C.byref(ms)))
    return t.value, z.value, ms.value


def launch_count() -> int:
    return int(load().pcgb_launch_count())
