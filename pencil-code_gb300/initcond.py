"""Seeded initial conditions written into the reference f-array layout.

The reference's start.x sets these with init_uu / init_aa
(hydro.f90:2214-2220 'ABC', initcond.f90:5005 gaussian noise); here they are
produced on the host with numpy's PCG64 so that both codes read the same
var.dat.  Arrays are f(mx,my,mz,nf), Fortran order, ghosts included (ghosts
are left zero: both codes refresh them from the interior).
"""
from __future__ import annotations

import numpy as np

from .lib import Params, host_shape

IUX, IUY, IUZ, ILNRHO = 0, 1, 2, 3


def field_index(p: Params, name: str) -> int:
    iax = 5 if p.lentropy else 4
    return {"ux": 0, "uy": 1, "uz": 2, "lnrho": 3, "ss": 4, "ax": iax, "ay": iax + 1, "az": iax + 2}[name]


def grid(p: Params):
    """The grid with ghosts, grid.f90:123-151: cell centres on a periodic axis,
    points on both boundaries otherwise."""
    return [p.axis(i) for i in range(3)]


def zeros(p: Params) -> np.ndarray:
    return np.zeros(host_shape(p), order="F")


def gaussian_noise(f: np.ndarray, p: Params, names, ampl: float, seed: int) -> np.ndarray:
    """i.i.d. N(0, ampl^2) in the interior of the named fields (one PCG64 stream)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    for nm in names:
        k = field_index(p, nm)
        f[3:3 + p.nx, 3:3 + p.ny, 3:3 + p.nz, k] += ampl * rng.standard_normal((p.nx, p.ny, p.nz)).transpose(0, 1, 2)
    return f


def abc_flow(f: np.ndarray, p: Params, ampl: float = 1.0, A: float = 1.0, B: float = 1.0, C: float = 1.0,
             k: float = 1.0) -> np.ndarray:
    """inituu='ABC', hydro.f90:2214-2220."""
    x, y, z = grid(p)
    X, Y, Z = np.meshgrid(x[3:-3], y[3:-3], z[3:-3], indexing="ij")
    sl = (slice(3, 3 + p.nx), slice(3, 3 + p.ny), slice(3, 3 + p.nz))
    f[sl + (IUX,)] += ampl * (A * np.sin(k * Z) + C * np.cos(k * Y))
    f[sl + (IUY,)] += ampl * (B * np.sin(k * X) + A * np.cos(k * Z))
    f[sl + (IUZ,)] += ampl * (C * np.sin(k * Y) + B * np.cos(k * X))
    return f


def fill_ghosts(f: np.ndarray) -> np.ndarray:
    """Periodic ghosts on the host (boundcond.f90:2387-2531), in place."""
    for ax in range(3):
        n = f.shape[ax] - 6
        idx = [slice(None)] * 4
        src = [slice(None)] * 4
        idx[ax] = slice(0, 3); src[ax] = slice(n, n + 3)
        f[tuple(idx)] = f[tuple(src)]
        idx[ax] = slice(n + 3, n + 6); src[ax] = slice(3, 6)
        f[tuple(idx)] = f[tuple(src)]
    return f
