"""ctypes binding of the FP64 parity oracle (oracle/pc_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
and by the CPU-baseline leg of ``bench.py``, always as the checker.  The
product library never imports or links this module.

Arrays are numpy float64 in the reference f-array layout f(mx,my,mz,nf),
Fortran order (x fastest), ghosts included.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
NGHOST = 3

(D_U2SUM, D_U2MAX, D_B2SUM, D_B2MAX, D_EKINSUM, D_RHOSUM, D_DIVB2SUM, D_J2SUM, D_ABSUM, D_JBSUM, D_EPSKSUM,
 D_N) = range(12)


class OrcParams(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("lentropy", C.c_int),
        ("x0", C.c_double), ("y0", C.c_double), ("z0", C.c_double),
        ("Lx", C.c_double), ("Ly", C.c_double), ("Lz", C.c_double),
        ("gamma", C.c_double), ("cs0", C.c_double), ("rho0", C.c_double), ("cp", C.c_double),
        ("nu", C.c_double), ("eta", C.c_double), ("chi", C.c_double), ("mu0", C.c_double),
        ("lforcing_cont", C.c_int),
        ("ampl_ff", C.c_double), ("kf", C.c_double), ("relhel", C.c_double),
        ("abc_a", C.c_double), ("abc_b", C.c_double), ("abc_c", C.c_double),
        ("ampl_fcont_uu", C.c_double),
        ("b_ext", C.c_double * 3),
        ("lohmic_heat", C.c_int), ("lviscosity_heat", C.c_int),
        ("cdt", C.c_double), ("cdtv", C.c_double),
        ("lupw_uu", C.c_int), ("lupw_lnrho", C.c_int),
        ("bc", ((C.c_int * 2) * 8) * 3),
    ]


def _elf_machine_ok(path: str) -> bool:
    want = {"x86_64": 62, "aarch64": 183, "arm64": 183}.get(os.uname().machine)
    try:
        with open(path, "rb") as fh:
            head = fh.read(20)
    except OSError:
        return False
    return len(head) == 20 and head[:4] == b"\x7fELF" and int.from_bytes(head[18:20], "little") == want


def build() -> str:
    """Compile the oracle with its Makefile (gcc, no GPU needed)."""
    if os.path.exists(_LIB_PATH) and not _elf_machine_ok(_LIB_PATH):
        os.remove(_LIB_PATH)
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = C.CDLL(_LIB_PATH)
        dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="F_CONTIGUOUS")
        dpc = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
        P = C.POINTER(OrcParams)
        L.orc_boundconds.argtypes = [P, dp, C.c_int]
        L.orc_stencil_field.argtypes = [P, dp, C.c_int, C.c_int, C.c_int, C.c_int, dp]
        L.orc_pde.argtypes = [P, dp, dp, C.c_double, C.c_int, C.POINTER(C.c_double), C.c_void_p, C.c_int]
        L.orc_time_step.argtypes = [P, dp, dp, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_int,
                                    C.c_void_p, C.c_int]
        L.orc_ran0.argtypes = [C.POINTER(C.c_int)]
        L.orc_ran0.restype = C.c_double
        L.orc_gaunoise_vect.argtypes = [P, C.c_double, dp, C.c_int, C.c_int, C.POINTER(C.c_int)]
        L.orc_gaunoise_volume.argtypes = [P, C.c_double, dp, C.c_int, C.c_int, C.POINTER(C.c_int)]
        L.orc_grid.argtypes = [P, dpc, dpc, dpc]
        L.orc_helical_coefs.argtypes = [P, C.c_double, dpc, dpc, dpc, C.c_int, C.c_double, C.POINTER(C.c_int),
                                        C.POINTER(HelRec)]
        L.orc_add_helical.argtypes = [P, dp, C.POINTER(HelRec), C.c_double, C.c_int]
        _lib = L
    return _lib


def make_params(**kw) -> OrcParams:
    """Parameter block with the reference defaults of the MHD hot path
    (cdata.f90:211,235,239; eos_idealgas.f90:47; forcing.f90:37,129;
    hydro.f90:283; magnetic.f90:247; entropy.f90:139)."""
    d = dict(nx=32, ny=32, nz=32, lentropy=0,
             x0=-np.pi, y0=-np.pi, z0=-np.pi, Lx=2 * np.pi, Ly=2 * np.pi, Lz=2 * np.pi,
             gamma=1.0, cs0=1.0, rho0=1.0, cp=1.0, nu=0.0, eta=0.0, chi=0.0, mu0=1.0,
             lforcing_cont=0, ampl_ff=0.0, kf=1.0, relhel=1.0, abc_a=1.0, abc_b=1.0, abc_c=1.0,
             ampl_fcont_uu=1.0, b_ext=(0.0, 0.0, 0.0), lohmic_heat=1, lviscosity_heat=1,
             cdt=0.9, cdtv=0.25, lupw_uu=0, lupw_lnrho=0)
    d.update(kw)
    p = OrcParams()
    for k, v in d.items():
        if k == "b_ext":
            p.b_ext[:] = list(v)
        elif k == "bc":
            for a in range(3):
                for f in range(8):
                    p.bc[a][f][0], p.bc[a][f][1] = v[a][f][0], v[a][f][1]
        else:
            setattr(p, k, v)
    return p


def nfields(p: OrcParams) -> int:
    return 8 if p.lentropy else 7


def empty_f(p: OrcParams, nf: int | None = None) -> np.ndarray:
    nf = nfields(p) if nf is None else nf
    return np.zeros((p.nx + 2 * NGHOST, p.ny + 2 * NGHOST, p.nz + 2 * NGHOST, nf), order="F")


def grid(p: OrcParams):
    x = np.zeros(p.nx + 2 * NGHOST); y = np.zeros(p.ny + 2 * NGHOST); z = np.zeros(p.nz + 2 * NGHOST)
    lib().orc_grid(C.byref(p), x, y, z)
    return x, y, z


def ghosts(p: OrcParams, f: np.ndarray) -> None:
    lib().orc_boundconds(C.byref(p), f, f.shape[3])


def stencil(p: OrcParams, f: np.ndarray, k: int, kind: int, i: int, j: int = 0) -> np.ndarray:
    out = np.zeros((p.nx, p.ny, p.nz), order="F")
    lib().orc_stencil_field(C.byref(p), f, k, kind, i, j, out)
    return out


def pde(p: OrcParams, f: np.ndarray, df: np.ndarray, alpha: float, want_dt=False, diag=False, nthreads=1):
    dt1 = C.c_double(0.0)
    dg = np.zeros(D_N) if diag else None
    lib().orc_pde(C.byref(p), f, df, alpha, int(want_dt), C.byref(dt1),
                  dg.ctypes.data if dg is not None else None, nthreads)
    return dt1.value, dg


def time_step(p: OrcParams, f: np.ndarray, df: np.ndarray, t: float, dt: float, ldt: bool,
              diag: bool = False, nthreads: int = 1):
    """One RK3 step in place; returns (t, dt, diag-or-None)."""
    tt = C.c_double(t); dd = C.c_double(dt)
    dg = np.zeros(D_N) if diag else None
    lib().orc_time_step(C.byref(p), f, df, C.byref(tt), C.byref(dd), int(ldt),
                        dg.ctypes.data if dg is not None else None, nthreads)
    return tt.value, dd.value, dg


class HelRec(C.Structure):
    """orc_helrec: one time step's random helical forcing record."""
    _fields_ = [("kk", C.c_double * 3), ("phase", C.c_double), ("coef1", C.c_double * 3),
                ("coef2", C.c_double * 3), ("fact0", C.c_double)]


def helical_coefs(p: OrcParams, force: float, kvec: np.ndarray, kav: float, state: int):
    """fconst_coefs_hel with the ran0 stream: returns (record, new state); kvec is (3, nk)."""
    kv = np.ascontiguousarray(kvec, dtype=np.float64)
    s = C.c_int(state)
    rec = HelRec()
    lib().orc_helical_coefs(C.byref(p), force, kv[0], kv[1], kv[2], kv.shape[1], kav, C.byref(s), C.byref(rec))
    return rec, s.value


def add_helical(p: OrcParams, f: np.ndarray, rec: HelRec, dt: float, target: int = 0) -> None:
    """forcing_hel: f(uu) (target 0) or f(aa) (target 1) += the step's helical
    forcing (interior; refresh ghosts after)."""
    lib().orc_add_helical(C.byref(p), f, C.byref(rec), dt, target)


def read_kdat(path: str):
    """k.dat of the reference (forcing.f90:888-900): 'nk kav', then kkx, kky, kkz."""
    with open(path) as fh:
        vals = fh.read().split()
    nk, kav = int(vals[0]), float(vals[1])
    k = np.array([float(v) for v in vals[2:2 + 3 * nk]]).reshape(3, nk)
    return k, kav


def gaunoise_vect(p: OrcParams, ampl: float, f: np.ndarray, i1: int, i2: int, state: int) -> int:
    s = C.c_int(state)
    lib().orc_gaunoise_vect(C.byref(p), ampl, f, i1, i2, C.byref(s))
    return s.value


def gaunoise_volume(p: OrcParams, ampl: float, f: np.ndarray, i1: int, i2: int, state: int) -> int:
    """gaunoise_vect's draws over whole (mx,my,mz) arrays in random_number_wrapper_3's
    order (z fastest): the realisation of samples/MHD-ABCforcing/reference.out."""
    s = C.c_int(state)
    lib().orc_gaunoise_volume(C.byref(p), ampl, f, i1, i2, C.byref(s))
    return s.value


def diag_summary(p: OrcParams, dg: np.ndarray) -> dict:
    """Volume averages as the reference prints them (diagnostics.f90:274,
    hydro.f90:4709,4743, magnetic.f90:6879,6894)."""
    nw = p.nx * p.ny * p.nz
    return dict(urms=np.sqrt(dg[D_U2SUM] / nw), umax=np.sqrt(dg[D_U2MAX]),
                brms=np.sqrt(dg[D_B2SUM] / nw), bmax=np.sqrt(dg[D_B2MAX]),
                ekin=dg[D_EKINSUM] / nw, rhom=dg[D_RHOSUM] / nw,
                divbrms=np.sqrt(dg[D_DIVB2SUM] / nw), jrms=np.sqrt(dg[D_J2SUM] / nw),
                abm=dg[D_ABSUM] / nw, jbm=dg[D_JBSUM] / nw, epsK=dg[D_EPSKSUM] / nw,
                epsM=p.eta * p.mu0 * dg[D_J2SUM] / nw)
