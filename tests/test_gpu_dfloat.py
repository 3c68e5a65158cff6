"""Double-float state (precision 8, dfloat=1): FP64-class results on the FP32 pipes.

The same parity bar as the native FP64 state against the FP64 oracle:
1e-11 on fields after the run, 1e-12 on diagnostics and dt.  In the entropy
case lnrho and ss stay within 1e-5 of zero, so their errors are measured
against max(|field|, 1), the relative error of rho and of exp(ss/cp): the
double-float round-off of div u (about 2^-48 |u| / dx per substep) leaves an
absolute error near 1e-16 in lnrho, which is 1e-10 of a field of size 6e-6.
"""
import numpy as np
import pytest

from conftest import LOG8, oracle_params, rel_err
from test_gpu_parity import TOL64, TOLDIAG, iso_params, iso_state, run_oracle

pytestmark = pytest.mark.gpu


def test_dfloat_isothermal_100_steps(pc, ic, orc):
    p = iso_params(pc, dfloat=1)
    f0 = iso_state(pc, ic, p)
    box = pc.Box(p)
    assert box.info()["dfloat"] == 1
    box.load(f0)
    box.steps(100)
    g = box.store()
    ref, t_ref, _ = run_oracle(orc, p, f0, 100)
    err = rel_err(g, ref)
    assert np.all(err <= TOL64), err
    t, _, nsub = box.time()
    assert nsub == 300 and abs(t - t_ref) <= 1e-12 * t_ref
    gg = ic.fill_ghosts(g.copy())
    assert np.array_equal(gg, g)


def test_dfloat_entropy_abc(pc, ic, orc):
    p = pc.default_params(nx=32, ny=32, nz=32, lentropy=1, gamma=5.0 / 3.0, nu=2e-3, eta=2e-3, chi=2e-3,
                          dt=1e-3, precision=8, dfloat=1)
    f0 = ic.zeros(p)
    ic.abc_flow(f0, p, ampl=1.0, A=0.1, B=0.1, C=0.1, k=1.0)
    ic.gaussian_noise(f0, p, ["ax", "ay", "az"], 1e-4, 7)
    box = pc.Box(p)
    box.load(f0)
    box.steps(20)
    g = box.store()
    ref, _, _ = run_oracle(orc, p, f0, 20)
    err = rel_err(g, ref, LOG8)
    assert np.all(err <= TOL64), err


def test_dfloat_forcing_bext_polytropic(pc, ic, orc):
    p = pc.default_params(nx=48, ny=32, nz=40, gamma=1.4, nu=1e-2, eta=2e-2, dt=2e-3, precision=8, dfloat=1,
                          lforcing_cont=1, ampl_ff=0.05, kf=2.0, relhel=0.5, abc_a=1.0, abc_b=0.7, abc_c=0.3,
                          b_ext=(0.0, 0.1, 0.05))
    p.update(Lxyz=(2 * np.pi, 1.5 * np.pi, 2.5 * np.pi))
    f0 = iso_state(pc, ic, p, ampl=1e-2, seed=3)
    ic.gaussian_noise(f0, p, ["lnrho"], 1e-3, 4)
    box = pc.Box(p)
    box.load(f0)
    box.steps(10)
    g = box.store()
    ref, _, _ = run_oracle(orc, p, f0, 10)
    assert np.all(rel_err(g, ref) <= TOL64)


def test_dfloat_cfl_current(pc, ic, orc):
    p = iso_params(pc, dt=0.0, dt_mode=2, cdt=0.4, b_ext=(0.0, 0.1, 0.0), nu=0.05, eta=0.05, dfloat=1)
    f0 = iso_state(pc, ic, p, ampl=1e-2, seed=5)
    box = pc.Box(p)
    box.load(f0)
    box.steps(10)
    g = box.store()
    t, dt, _ = box.time()
    ref, t_ref, dt_ref = run_oracle(orc, p, f0, 10, ldt=True, dt=0.0)
    assert np.all(rel_err(g, ref) <= TOL64)
    assert abs(dt - dt_ref) <= TOLDIAG * dt_ref and abs(t - t_ref) <= TOLDIAG * t_ref


def test_dfloat_diagnostics(pc, ic, orc):
    p = iso_params(pc, diag_every=1, b_ext=(0.0, 0.1, 0.0), dfloat=1)
    f0 = iso_state(pc, ic, p, ampl=1e-2, seed=8)
    box = pc.Box(p)
    box.load(f0)
    box.steps(1)
    raw = box.diag_raw()
    op = oracle_params(orc, p)
    f = np.array(f0, order="F", copy=True)
    orc.ghosts(op, f)
    _, dg = orc.pde(op, f, np.zeros_like(f), 0.0, diag=True)
    for k in range(9):
        ref, got = dg[k], raw[k + 1]
        if k == orc.D_DIVB2SUM:
            assert got <= 1e-24 * dg[orc.D_J2SUM] and ref <= 1e-24 * dg[orc.D_J2SUM]
            continue
        assert abs(got - ref) <= TOLDIAG * max(abs(ref), 1e-300), (k, got, ref)


def test_dfloat_tiles_agree_and_track_native_fp64(pc, ic):
    """Every tile variant gives the same bits; the state stays within the
    representation error of a double-float of the native FP64 result."""
    p64 = iso_params(pc, n=32)
    f0 = iso_state(pc, ic, p64, seed=11)
    b64 = pc.Box(p64)
    b64.load(f0)
    b64.steps(3)
    g64 = b64.store()
    base = None
    for tile, zd in ((0, 0), (1, 8), (2, 0), (3, 16)):
        p = iso_params(pc, n=32, tile=tile, zdepth=zd, dfloat=1)
        box = pc.Box(p)
        box.load(f0)
        box.steps(3)
        g = box.store()
        if base is None:
            base = g
            assert np.all(rel_err(g, g64) <= 1e-13)
        else:
            assert np.array_equal(g, base), (tile, zd)


@pytest.mark.parametrize("lentropy", [0, 1])
def test_dfloat_pair_tiles_equal_field_major(pc, ic, lentropy):
    """The packed double-float pair layout (tiles 4-7) computes lane by lane the
    same operations as the field-major double-float tiles: same field bits."""
    kw = dict(nx=40, ny=24, nz=20, lentropy=lentropy, gamma=5.0 / 3.0 if lentropy else 1.0, nu=5e-3, eta=5e-3,
              chi=5e-3 if lentropy else 0.0, dt=2e-3, precision=8, dfloat=1, lforcing_cont=1, ampl_ff=0.02, kf=1.0,
              diag_every=1)
    p0 = pc.default_params(tile=0, **kw)
    f0 = iso_state(pc, ic, p0, ampl=1e-2, seed=31)
    if lentropy:
        ic.gaussian_noise(f0, p0, ["lnrho", "ss"], 1e-3, 32)
    base = pc.Box(p0)
    base.load(f0)
    base.steps(3)
    g0, d0 = base.store(), base.diag_raw()
    for tile in (4, 5, 6, 7):
        box = pc.Box(pc.default_params(tile=tile, **kw))
        assert box.info()["pairs"] == 1 and box.info()["tile"] == tile
        box.load(f0)
        box.steps(3)
        assert np.array_equal(box.store(), g0), tile
        # FP64 reductions over a different tile decomposition: same sums up to order
        np.testing.assert_allclose(box.diag_raw(), d0, rtol=1e-12, atol=1e-24)


def test_dfloat_pair_oracle_and_device_init(pc, ic, orc):
    """Pair-tile double-float state against the FP64 oracle after 100 steps, and
    the device initial condition writes the same state into both layouts."""
    p = iso_params(pc, dfloat=1, tile=4)
    f0 = iso_state(pc, ic, p)
    box = pc.Box(p)
    box.load(f0)
    box.steps(100)
    ref, _, _ = run_oracle(orc, p, f0, 100)
    assert np.all(rel_err(box.store(), ref) <= TOL64)
    outs = []
    for tile in (0, 4):
        b = pc.Box(iso_params(pc, dfloat=1, tile=tile))
        for k in range(7):
            b.init_field(k, "zero")
        b.init_field(0, "abc", ampl=0.1, abc=(1.0, 0.5, 0.25), k=1.0)
        for k in (4, 5, 6):
            b.init_field(k, "noise", ampl=1e-3, seed=40 + k)
        outs.append(b.store())
    assert np.array_equal(outs[0], outs[1])
