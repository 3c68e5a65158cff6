"""A run driver with the shape of the reference's run.x time loop (src/run.f90):
read start.in / run.in, set up the initial condition, advance nt steps on the
GPU, write the time series every it1 steps (data/time_series.dat, the state at
the start of that step, as the reference prints it) and var.dat snapshots every
dsnap in time (data/proc0/VARn, then data/proc0/var.dat at the end), with the
reference's dim.dat.

Boundary conditions and the grid follow lperi / bcx / bcy / bcz (periodic, or 's', 'a',
'a2' per field and side).  Initial conditions of this path: zero fields, &magnetic_init_pars
initaa='gaussian-noise' with amplaa (an N(0, amplaa^2) field from a seeded
PCG64 stream; the reference's realisation comes from its own generator), and
&hydro_init_pars inituu='ABC' with ampluu.  Anything else is refused.
"""
from __future__ import annotations

import math
import os

import numpy as np

from . import initcond as ic_mod
from .lib import Box, diag_summary, nfields
from .namelist import params_from_namelists
from .vardat import write_box_snapshot

SERIES_COLUMNS = ("it", "t", "dt", "urms", "umax", "brms", "bmax", "jrms", "divbrms", "rhom")


def initial_state(p, ic: dict, seed: int = 1) -> np.ndarray:
    """f of the start: the initial conditions named in start.in."""
    f = ic_mod.zeros(p)
    initaa = str(ic.get("initaa", "zero")).strip().lower()
    if initaa in ("gaussian-noise", "gaussian_noise"):
        ic_mod.gaussian_noise(f, p, ["ax", "ay", "az"], float(ic.get("amplaa", 0.0)), seed)
    elif initaa not in ("zero", "nothing"):
        raise ValueError(f"initaa={initaa!r} is not an initial condition of this path")
    inituu = str(ic.get("hydro.inituu", "zero")).strip().lower()
    if inituu == "abc":
        ic_mod.abc_flow(f, p, ampl=float(ic.get("hydro.ampluu", 1.0)))
    elif inituu not in ("zero", "nothing"):
        raise ValueError(f"inituu={inituu!r} is not an initial condition of this path")
    return ic_mod.fill_ghosts(f)


def write_dim(path: str, p) -> None:
    """dim.dat: mx my mz mvar maux mglobal / precision / nghost / processor layout."""
    with open(path, "w") as fh:
        fh.write("%7d%7d%7d%7d%7d%7d\n" % (p.nx + 6, p.ny + 6, p.nz + 6, nfields(p), 0, 0))
        fh.write("D\n")
        fh.write("%5d%5d%5d\n" % (3, 3, 3))
        fh.write("%5d%5d%5d%5d\n" % (1, 1, 1, 1))


def format_series_row(row: dict) -> str:
    return "%5d %10.4f %10.3e " % (row["it"], row["t"], row["dt"]) + " ".join(
        "%10.3e" % row[c] for c in SERIES_COLUMNS[3:])


def run(start_text: str, run_text: str, n, outdir: str, kdat=None, precision: int = 8, dfloat: int = 0,
        nt: int | None = None, seed: int = 1, tile: int = -1) -> dict:
    """Run a box from namelist text; returns the time-series rows and the files written.

    n: grid (nx, ny, nz); kdat: (kvec (3, nk), kav) for iforce='helical'; nt overrides run.in."""
    p, ic, extra = params_from_namelists(start_text, run_text, n=tuple(n), precision=precision)
    p.dfloat = dfloat
    p.tile = tile
    it1 = max(int(ic.get("it1") or 10), 1)
    p.diag_every = it1
    nsteps = int(nt if nt is not None else (ic.get("nt") or 0))
    dsnap = float(ic.get("dsnap") or 0.0)
    data = os.path.join(outdir, "data")
    proc = os.path.join(data, "proc0")
    os.makedirs(proc, exist_ok=True)
    write_dim(os.path.join(data, "dim.dat"), p)
    f = initial_state(p, ic, seed)
    box = Box(p)
    if p.lforcing_hel:
        if kdat is None:
            raise ValueError("iforce='helical' needs the wavevector list (k.dat)")
        box.set_kvectors(*kdat)
    box.load(f)
    # VAR0 after update_ghosts (snapshot.f90:363): the device store fills the ghosts of
    # non-periodic directions from their boundary conditions
    write_box_snapshot(os.path.join(proc, "VAR0"), p, box.store() if not all(p.periodic(d) for d in range(3)) else f,
                       0.0)
    rows, files = [], [os.path.join(proc, "VAR0")]
    ncells = p.nx * p.ny * p.nz
    tsnap, isnap = (dsnap if dsnap > 0 else math.inf), 0
    series = open(os.path.join(data, "time_series.dat"), "w")
    series.write("#" + "".join("%-11s" % c for c in SERIES_COLUMNS) + "\n")
    try:
        for it in range(nsteps):
            t0, _, _ = box.time()
            box.steps(1)
            t, _, _ = box.time()
            if it % it1 == 0:
                raw = box.diag_raw()
                d = diag_summary(raw, ncells)
                row = dict(it=it, t=t0, dt=t - t0, **{c: float(d[c]) for c in SERIES_COLUMNS[3:]})
                rows.append(row)
                series.write(format_series_row(row) + "\n")
                series.flush()
            if t >= tsnap:   # wsnap (snapshot.f90:265): one snapshot per crossing of a multiple of dsnap
                isnap += 1
                path = os.path.join(proc, f"VAR{isnap}")
                write_box_snapshot(path, p, box.store(), t)
                files.append(path)
                tsnap += dsnap
        path = os.path.join(proc, "var.dat")
        t, _, _ = box.time()
        write_box_snapshot(path, p, box.store(), t)
        files.append(path)
    finally:
        series.close()
        box.close()
    return {"rows": rows, "files": files, "params": p, "unapplied": extra}
