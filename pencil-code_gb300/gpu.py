"""Mirror of the reference's Fortran module ``GPU`` (src/gpu_astaroth.f90).

Same routine names, argument meaning and call order as the public list of
src/gpu.h:1-13, implemented over the C ABI of libpcgb300.so, so that a test
written against the reference's GPU interface reads the same here.  The
Fortran module variables the reference passes by address (pushpars2c) are
the :class:`Params` block given to :func:`initialize_gpu`.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .lib import NSLOT, Params, PcgbError, check, last_error, load

n_gpu_reduced_vars = 20   # gpu_astaroth.f90:14

_f_host: np.ndarray | None = None


def _raise_if_error():
    rc, msg = last_error()
    if rc:
        load().pcgb_clear_error()
        raise PcgbError(f"pcgb error {rc}: {msg}")


def register_gpu():
    """register_GPU, gpu_astaroth.f90:346."""
    load().registerGPU()


def initialize_gpu(f: np.ndarray, p: Params, t: float = 0.0, nt: int = 1,
                   lcpu_timestep_on_gpu: bool = False, lac_sparse_autotuning: bool = False):
    """initialize_GPU, gpu_astaroth.f90:192: bind f, allocate, load f when nt > 0."""
    global _f_host
    L = load()
    if f.dtype != np.float64 or not f.flags.f_contiguous:
        raise ValueError("f must be a Fortran-ordered float64 array f(mx,my,mz,mvar)")
    check(L.pcgb_set_params(C.byref(p)))
    _f_host = f
    L.initializeGPU(f.ctypes.data_as(C.POINTER(C.c_double)), 0, float(t), int(nt), 0,
                    int(lcpu_timestep_on_gpu), int(lac_sparse_autotuning))
    _raise_if_error()


def finalize_gpu():
    global _f_host
    load().finalizeGPU()
    _f_host = None


def get_farray_ptr_gpu():
    """get_farray_ptr_gpu, gpu_astaroth.f90:360: device pointers (in, out)."""
    a, b = C.c_void_p(), C.c_void_p()
    load().copyVBApointers(C.byref(a), C.byref(b))
    return a.value, b.value


def rhs_gpu(isubstep: int, t: float = 0.0):
    """rhs_GPU, gpu_astaroth.f90:285: one complete RK substep on the device."""
    load().substepGPU(int(isubstep), float(t))
    _raise_if_error()


def before_boundary_gpu(lrmv: bool, isubstep: int, t: float):
    load().beforeBoundaryGPU(bool(lrmv), int(isubstep), float(t), False)


def update_after_substep_gpu():
    load().afterSubStepGPU()


def copy_farray_from_gpu(f: np.ndarray | None = None) -> np.ndarray:
    """copy_farray_from_GPU: device f -> host f (the bound array by default)."""
    f = _f_host if f is None else f
    load().copyFarray(f.ctypes.data_as(C.POINTER(C.c_double)))
    _raise_if_error()
    return f


def load_farray_to_gpu():
    """load_farray_to_GPU: bound host f -> device, ghosts refreshed."""
    load().loadFarray()
    _raise_if_error()


def reload_gpu_config(p: Params):
    check(load().pcgb_set_params(C.byref(p)))
    load().reloadConfig()
    _raise_if_error()


def update_on_gpu(name: str, value):
    """update_on_gpu by name, scalar or 3-vector."""
    L = load()
    if np.ndim(value) == 0:
        rc = L.updateInConfigScalName(name.encode(), float(value))
    else:
        v = np.ascontiguousarray(value, dtype=np.float64)
        rc = L.updateInConfigVecName(name.encode(), v.ctypes.data_as(C.POINTER(C.c_double)))
    if rc != 0:
        raise PcgbError(f"unknown GPU parameter {name!r}")
    _raise_if_error()


def gpu_prepare_for_first_substep(t: float = 0.0):
    load().prepareForFirstSubstep(float(t))
    _raise_if_error()


def get_gpu_reduced_vars() -> dict:
    """urms, umax, brms, bmax, ekin, rhom, divbrms, jrms, abm, dt, t, step."""
    out = np.zeros(n_gpu_reduced_vars)
    load().getGPUReducedVars(out.ctypes.data_as(C.POINTER(C.c_double)))
    _raise_if_error()
    keys = ["urms", "umax", "brms", "bmax", "ekin", "rhom", "divbrms", "jrms", "abm", "dt", "t", "step"]
    return dict(zip(keys, out[:len(keys)]))


def request_diagnostics():
    load().pcgb_request_diagnostics()


def test_gpu_bcs():
    load().testBCs()


def get_dt() -> float:
    return load().pcgb_get_dt()


def get_time() -> float:
    return load().pcgb_get_time()


def time_step(nsteps: int = 1):
    """Timestep.time_step with lgpu=T (timestep.f90:206): rhs_GPU for itsub=1..3."""
    check(load().pcgb_time_step(int(nsteps)))


__all__ = [n for n in dir() if not n.startswith("_")] + ["NSLOT"]
