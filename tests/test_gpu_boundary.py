"""Non-periodic boundary conditions ('s', 'a', 'a2' per field and side) on the
GPU against the oracle's restatement of boundconds_x/y/z (boundcond.f90
bc_sym_x/y/z), with the non-periodic grid of grid.f90 (dx = L/(n-1), points on
both boundaries).

The device fills the ghost zones of the non-periodic directions before every
pass that reads f (the CFL pass and each substep, as pde does before the RHS)
and before a store (update_ghosts before a snapshot), so the stored f,
ghosts included, is compared with the oracle's f after its own boundconds.
Bars as in the other parity tests: FP64 and double-float 1e-11 per field,
FP32 1e-5 (lnrho and ss against max(|field|, 1)).
"""
import importlib

import numpy as np
import pytest

from conftest import LOG7, LOG8, oracle_params, rel_err

pytestmark = pytest.mark.gpu

BCZ7 = ["s", "s", "a", "a2", "s:a2", "a", "a2:s"]          # ux uy uz lnrho ax ay az
BCX7 = ["a", "s", "s", "a2", "s", "a", "a"]
BCY7 = ["s", "a", "s", "s:a2", "a", "s", "a"]
BCZ8 = ["s", "s", "a", "a2", "s", "s", "a", "a2"]         # ux uy uz lnrho ss ax ay az

MODES = {
    "f64": dict(precision=8),
    "dfloat": dict(precision=8, dfloat=1, tile=3),
    "dfloat_pair": dict(precision=8, dfloat=1, tile=5),
    "f32pair": dict(precision=4, comp=1, tile=6),
    "f32pair7": dict(precision=4, comp=1, tile=7),   # the 12-warp tensor-memory tile
    "f32": dict(precision=4, comp=1, tile=0),
}


def _params(pc, n=(24, 20, 16), lentropy=0, **kw):
    p = pc.default_params(nx=n[0], ny=n[1], nz=n[2], lentropy=lentropy, gamma=(5.0 / 3.0 if lentropy else 1.0),
                          nu=4e-3, eta=5e-3, chi=(3e-3 if lentropy else 0.0), dt=2e-3, lforcing_cont=1,
                          ampl_ff=0.05, kf=1.0, b_ext=(0.0, 0.05, 0.02))
    return p.update(**kw)


def _initial(pc, ic, p, seed):
    f = ic.zeros(p)
    rng = np.random.Generator(np.random.PCG64(seed))
    f[3:-3, 3:-3, 3:-3, :] = 0.03 * rng.standard_normal((p.nx, p.ny, p.nz, f.shape[3]))
    return f


def _oracle(orc, p, f0, nsteps, ldt=False):
    op = oracle_params(orc, p)
    f = np.array(f0, order="F", copy=True)
    df = np.zeros_like(f)
    t, dt = 0.0, (0.0 if ldt else p.dt)
    for _ in range(nsteps):
        t, dt, _ = orc.time_step(op, f, df, t, dt, ldt, nthreads=8)
    orc.ghosts(op, f)   # update_ghosts before the snapshot
    return f, t, dt


def _check(g, ref, p, mode=""):
    log = LOG8 if p.lentropy else LOG7
    tol = 1e-5 if p.precision == 4 else 1e-11
    err = rel_err(g, ref, log)
    assert np.all(err <= tol), (mode, err)
    # ghosts included: the whole array against the interior scale of each field
    for k in range(g.shape[3]):
        scale = np.max(np.abs(ref[3:-3, 3:-3, 3:-3, k]))
        if k in log:
            scale = max(scale, 1.0)
        assert np.max(np.abs(g[..., k] - ref[..., k])) <= tol * max(scale, 1e-30) * 4, (mode, k)


@pytest.mark.parametrize("mode", list(MODES))
def test_z_boundaries_match_oracle(pc, ic, orc, mode):
    p = _params(pc, bcz=BCZ7, **MODES[mode])
    assert not p.periodic(2) and p.periodic(0)
    f0 = _initial(pc, ic, p, 3)
    box = pc.Box(p)
    box.load(f0)
    box.steps(10)
    g = box.store()
    ref, t_ref, _ = _oracle(orc, p, f0, 10)
    _check(g, ref, p, mode)
    # the antisymmetric fields are zero on the boundary planes
    assert np.all(g[:, :, 3, 2] == 0.0) and np.all(g[:, :, -4, 2] == 0.0)
    assert abs(box.time()[0] - t_ref) <= 1e-12 * t_ref


@pytest.mark.parametrize("mode", ["f64", "f32pair", "f32pair7"])
def test_x_and_y_boundaries_edges_and_corners(pc, ic, orc, mode):
    """x and y non-periodic, z periodic: boundconds_x before _y, so the corner
    ghosts are the y condition applied to x-filled rows."""
    p = _params(pc, n=(20, 18, 12), bcx=BCX7, bcy=BCY7, **MODES[mode])
    f0 = _initial(pc, ic, p, 5)
    box = pc.Box(p)
    box.load(f0)
    box.steps(8)
    ref, _, _ = _oracle(orc, p, f0, 8)
    _check(box.store(), ref, p, mode)


@pytest.mark.parametrize("mode", ["f64", "dfloat_pair", "f32pair"])
def test_all_directions_entropy_cfl_current(pc, ic, orc, mode):
    """Every direction non-periodic, 8 fields, dt from the CFL condition of the current
    state (the CFL pass reads the ghosts the boundary pass wrote)."""
    kw = dict(MODES[mode])
    if mode == "f64":
        kw["tile"] = 2
    if mode == "f32pair":
        kw["tile"] = 4
    p = _params(pc, n=(16, 14, 18), lentropy=1, bcx=BCZ8, bcy=BCZ8[::-1], bcz=BCZ8, dt=0.0, dt_mode=2, cdt=0.4,
                **kw)
    f0 = _initial(pc, ic, p, 7)
    f0[..., 4] *= 0.2
    box = pc.Box(p)
    box.load(f0)
    box.steps(6)
    ref, t_ref, dt_ref = _oracle(orc, p, f0, 6, ldt=True)
    _check(box.store(), ref, p, mode)
    t, dt, _ = box.time()
    assert abs(t - t_ref) <= (1e-6 if p.precision == 4 else 1e-12) * t_ref


@pytest.mark.parametrize("mode", ["f64", "f32pair"])
def test_boundaries_with_upwinding_and_helical_forcing(pc, ic, orc, mode):
    nl = importlib.import_module("pencil-code_gb300.namelist")
    kvec, kav = nl.kvector_shell(5, 6)
    p = _params(pc, n=(16, 16, 16), bcz=BCZ7, lupw_uu=1, lupw_lnrho=1, lforcing_hel=1, force_hel=0.05,
                lmagnetic_forcing=1, seed_ff=1812, lforcing_cont=0, **MODES[mode])
    f0 = _initial(pc, ic, p, 9)
    box = pc.Box(p)
    box.set_kvectors(kvec, kav)
    box.load(f0)
    box.steps(5)
    op = oracle_params(orc, p)
    f = np.array(f0, order="F", copy=True)
    df = np.zeros_like(f)
    t, dt, state = 0.0, p.dt, p.seed_ff
    for _ in range(5):
        rec, state = orc.helical_coefs(op, p.force_hel, kvec, kav, state)
        _, state = orc.helical_coefs(op, p.force_hel, kvec, kav, state)
        t, dt, _ = orc.time_step(op, f, df, t, dt, False, nthreads=8)
        orc.add_helical(op, f, rec, dt, 1)
    orc.ghosts(op, f)
    _check(box.store(), f, p, mode)


def test_boundary_refusals(pc):
    # a direction cannot mix periodic and non-periodic codes
    p = _params(pc, bcz=["s"] * 6 + ["p"])
    with pytest.raises(pc.PcgbError):
        pc.Box(p)
    # boxes with non-periodic boundaries step through the box API, not in a batch
    q = _params(pc, bcz=BCZ7)
    b = pc.Box(q)
    with pytest.raises(pc.PcgbError):
        pc.Batch([b])
    b.close()
