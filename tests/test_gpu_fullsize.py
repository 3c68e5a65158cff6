"""Parity with the FP64 oracle at the full sizes of the two large fixed-dt
configurations, the shape of the reference's own GPU self-test
(`test_rhs_gpu`, src/equ.f90:1974-2143: max relative error per field).

- 256^3 entropy MHD (8 fields, gamma=5/3, nu=eta=chi=2e-3), uu = ABC flow at
  k=1 with A=B=C=0.1, aa noise 1e-4, dt=1e-3, 200 steps;
- 512^3 isothermal MHD with the steady helical ABC body force at k=2
  (ampl 0.02), nu=eta=5e-4, aa noise 1e-5 from the device initial condition,
  dt=2e-4, 25 steps (5 warm-up + 20 timed of the throughput run).

One oracle run per configuration (OpenMP on all host cores, a few minutes),
then every state mode against it: native FP64 and double-float within 1e-11,
FP32 compensated within 1e-5 (lnrho and ss measured against max(|field|, 1)).
The FP64-class diagnostics of the final state (urms, brms, energies) are
compared at 1e-12 and div B is checked at round-off.
"""
import os

import numpy as np
import pytest

from conftest import LOG7, LOG8, oracle_params, rel_err

pytestmark = pytest.mark.gpu

TOL64 = 1e-11
TOLDIAG = 1e-12
TOL32 = 1e-5
MODES = (("f64", dict(precision=8), TOL64), ("dfloat", dict(precision=8, dfloat=1), TOL64),
         ("f32", dict(precision=4, comp=1), TOL32))


def _oracle_run(orc, p, f0, nsteps):
    op = oracle_params(orc, p)
    f = np.array(f0, order="F", copy=True)
    df = np.zeros_like(f)
    t = 0.0
    for _ in range(nsteps):
        t, _, _ = orc.time_step(op, f, df, t, p.dt, False, nthreads=os.cpu_count() or 1)
    del df
    orc.ghosts(op, f)
    _, dg = orc.pde(op, f, np.zeros_like(f), 0.0, diag=True, nthreads=os.cpu_count() or 1)
    return f, t, dg


def _diag_check(pc, orc, kw, g, dg, tol):
    """Diagnostics of the final GPU state (the FP64 diagnostic evaluation of one
    more substep on it) against the oracle's on its own final state."""
    box = pc.Box(pc.default_params(**kw, precision=8, diag_every=1))
    box.load(g)
    box.steps(1)
    raw = box.diag_raw()
    box.close()
    for k in (orc.D_U2SUM, orc.D_U2MAX, orc.D_B2SUM, orc.D_B2MAX, orc.D_EKINSUM, orc.D_RHOSUM, orc.D_J2SUM):
        assert abs(raw[k + 1] - dg[k]) <= tol * abs(dg[k]), (k, raw[k + 1], dg[k])
    assert raw[orc.D_DIVB2SUM + 1] <= 1e-20 * dg[orc.D_J2SUM]


def _modes_against(pc, ic, orc, kw, f0, nsteps, log_fields):
    ref, t_ref, dg = _oracle_run(orc, pc.default_params(precision=8, **kw), f0, nsteps)
    report = {}
    for name, extra, tol in MODES:
        box = pc.Box(pc.default_params(**kw, **extra))
        box.load(f0)
        box.steps(nsteps)
        g = box.store()
        t, _, nsub = box.time()
        box.close()
        err = rel_err(g, ref, log_fields)
        report[name] = err
        assert np.all(err <= tol), (name, err)
        assert nsub == 3 * nsteps and abs(t - t_ref) <= 1e-12 * t_ref
        assert np.array_equal(ic.fill_ghosts(g.copy()), g)
        if tol == TOL64:
            _diag_check(pc, orc, kw, g, dg, TOLDIAG)
        del g
    print({k: [f"{e:.2e}" for e in v] for k, v in report.items()})


def test_entropy_256_against_oracle(pc, ic, orc):
    """256^3 entropy MHD, 200 steps of dt=1e-3: every state mode against one oracle run."""
    kw = dict(nx=256, ny=256, nz=256, lentropy=1, gamma=5.0 / 3.0, nu=2e-3, eta=2e-3, chi=2e-3, dt=1e-3)
    p64 = pc.default_params(precision=8, **kw)
    f0 = ic.zeros(p64)
    ic.abc_flow(f0, p64, ampl=1.0, A=0.1, B=0.1, C=0.1, k=1.0)
    ic.gaussian_noise(f0, p64, ["ax", "ay", "az"], 1e-4, 7)
    _modes_against(pc, ic, orc, kw, f0, 200, LOG8)


def test_headline_physics_512_against_oracle(pc, ic, orc):
    """512^3 isothermal MHD with the helical ABC body force, 25 steps of dt=2e-4,
    from the seeded device initial condition: every state mode against one oracle run."""
    n = 512
    kw = dict(nx=n, ny=n, nz=n, gamma=1.0, nu=5e-4, eta=5e-4, dt=2e-4, lforcing_cont=1, ampl_ff=0.02,
              kf=2.0, relhel=1.0)
    box = pc.Box(pc.default_params(precision=8, **kw))
    for k in range(7):
        box.init_field(k, "zero")
    for k in range(3):
        box.init_field(4 + k, "noise", ampl=1e-5, seed=20260 + k)
    f0 = box.store()
    box.close()
    _modes_against(pc, ic, orc, kw, f0, 25, LOG7)
