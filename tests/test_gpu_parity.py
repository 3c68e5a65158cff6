"""Parity of the CUDA substep kernel (through the C ABI) with the FP64 oracle.

Tolerances (max |gpu - oracle| / max |oracle| per field):
  FP64 state: 1e-11 on fields after the run, 1e-12 on diagnostics;
  FP32 compensated state: 1e-5 on fields, where lnrho and ss are measured
  against max(max|field|, 1) (an absolute error in ln rho is the relative
  error of rho).
div B is zero up to round-off in both codes; it is checked against the
current density scale instead of relatively.
"""
import numpy as np
import pytest

from conftest import LOG7, LOG8, oracle_params, rel_err

pytestmark = pytest.mark.gpu

TOL64 = 1e-11
TOLDIAG = 1e-12
TOL32 = 1e-5


def iso_params(pc, n=32, **kw):
    p = pc.default_params(nx=n, ny=n, nz=n, gamma=1.0, nu=5e-3, eta=5e-3, dt=5e-3, precision=8)
    return p.update(**kw)


def iso_state(pc, ic, p, ampl=1e-3, seed=1):
    f = ic.zeros(p)
    ic.gaussian_noise(f, p, ["ux", "uy", "uz", "ax", "ay", "az"], ampl, seed)
    return f


def run_oracle(orc, p, f0, nsteps, ldt=False, dt=None):
    op = oracle_params(orc, p)
    f = np.array(f0, order="F", copy=True)
    df = np.zeros_like(f)
    t, d = 0.0, (p.dt if dt is None else dt)
    for _ in range(nsteps):
        t, d, _ = orc.time_step(op, f, df, t, d, ldt, nthreads=8)
    orc.ghosts(op, f)
    return f, t, d


def test_isothermal_fp64_100_steps(pc, ic, orc):
    """32^3 isothermal MHD, FP64, fixed dt=5e-3, 100 steps (the 32^3 FP64 parity case)."""
    p = iso_params(pc)
    f0 = iso_state(pc, ic, p)
    box = pc.Box(p)
    box.load(f0)
    box.steps(100)
    g = box.store()
    ref, t_ref, _ = run_oracle(orc, p, f0, 100)
    err = rel_err(g, ref)
    assert np.all(err <= TOL64), err
    t, dt, nsub = box.time()
    assert nsub % 3 == 0 and abs(t - t_ref) <= 1e-12 * t_ref
    # ghosts of the stored f are the exact periodic images
    gg = ic.fill_ghosts(g.copy())
    assert np.array_equal(gg, g)


def test_entropy_fp64_abc(pc, ic, orc):
    """8 fields with entropy, ABC initial flow, Ohmic/viscous heating, chi-const conduction."""
    p = pc.default_params(nx=32, ny=32, nz=32, lentropy=1, gamma=5.0 / 3.0, nu=2e-3, eta=2e-3, chi=2e-3,
                          dt=1e-3, precision=8)
    f0 = ic.zeros(p)
    ic.abc_flow(f0, p, ampl=1.0, A=0.1, B=0.1, C=0.1, k=1.0)
    ic.gaussian_noise(f0, p, ["ax", "ay", "az"], 1e-4, 7)
    box = pc.Box(p)
    box.load(f0)
    box.steps(20)
    g = box.store()
    ref, _, _ = run_oracle(orc, p, f0, 20)
    err = rel_err(g, ref)
    assert np.all(err <= TOL64), err


def test_forcing_bext_polytropic(pc, ic, orc):
    """ABC continuous forcing, imposed B_ext, polytropic (gamma != 1 without entropy), non-cubic grid."""
    p = pc.default_params(nx=48, ny=32, nz=40, gamma=1.4, nu=1e-2, eta=2e-2, dt=2e-3, precision=8,
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


def test_cfl_current_semantics(pc, ic, orc):
    """dt from the CFL condition of the current f (CPU semantics, lcpu_timestep_on_gpu)."""
    p = iso_params(pc, dt=0.0, dt_mode=2, cdt=0.4, b_ext=(0.0, 0.1, 0.0), nu=0.05, eta=0.05)
    f0 = iso_state(pc, ic, p, ampl=1e-2, seed=5)
    box = pc.Box(p)
    box.load(f0)
    box.steps(10)
    g = box.store()
    t, dt, _ = box.time()
    ref, t_ref, dt_ref = run_oracle(orc, p, f0, 10, ldt=True, dt=0.0)
    assert np.all(rel_err(g, ref) <= TOL64)
    assert abs(dt - dt_ref) <= 1e-13 * dt_ref and abs(t - t_ref) <= 1e-13 * t_ref


def test_cfl_lagged_semantics(pc, ic, orc):
    """Reference GPU default: dt of step n is the CFL of f at the start of step n-1
    (the first step uses the CFL of the initial f)."""
    p = iso_params(pc, dt=0.0, dt_mode=1, cdt=0.4, nu=0.05, eta=0.05)
    f0 = iso_state(pc, ic, p, ampl=1e-2, seed=6)
    box = pc.Box(p)
    box.load(f0)
    box.steps(6)
    g = box.store()
    op = oracle_params(orc, p)
    f = np.array(f0, order="F", copy=True)
    df = np.zeros_like(f)
    orc.ghosts(op, f)
    dt1, _ = orc.pde(op, f, np.zeros_like(f), 0.0, want_dt=True)
    dt_use = 1.0 / dt1
    t = 0.0
    for _ in range(6):
        orc.ghosts(op, f)
        d1, _ = orc.pde(op, f, np.zeros_like(f), 0.0, want_dt=True)
        t, _, _ = orc.time_step(op, f, df, t, dt_use, False, nthreads=8)
        dt_use = 1.0 / d1
    orc.ghosts(op, f)
    assert np.all(rel_err(g, f) <= TOL64)


def test_diagnostics_fp64(pc, ic, orc):
    p = iso_params(pc, diag_every=1, b_ext=(0.0, 0.1, 0.0))
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
        ref = dg[k]
        got = raw[k + 1]
        if k == orc.D_DIVB2SUM:
            # round-off only: |div B| <= 1e-12 |J| in both codes
            assert got <= 1e-24 * dg[orc.D_J2SUM] and ref <= 1e-24 * dg[orc.D_J2SUM]
            continue
        assert abs(got - ref) <= TOLDIAG * max(abs(ref), 1e-300), (k, got, ref)


@pytest.mark.parametrize("mode", ["f64", "dfloat", "f32pair"])
def test_isothermal_diagnostic_series_100_steps(pc, ic, orc, mode):
    """The 32^3 isothermal case (noise 1e-3 from a seed, nu=eta=5e-3, dt=5e-3) with the
    diagnostics of every step over the 100-step run -- urms, umax, brms, bmax, ekin, rhom,
    jrms, abm, evaluated on the pre-update f of substep 1 (diagnostics.f90:274) -- against
    the oracle's series: 1e-12 relative for the FP64-class states, 1e-5 for FP32 (abm,
    which changes sign, relative to rms(A) brms)."""
    kw = dict(f64=dict(precision=8), dfloat=dict(precision=8, dfloat=1),
              f32pair=dict(precision=4, comp=1, tile=5))[mode]
    tol = 1e-5 if mode == "f32pair" else TOLDIAG
    p = iso_params(pc, diag_every=1, **kw)
    f0 = iso_state(pc, ic, p)
    box = pc.Box(p)
    box.load(f0)
    op = oracle_params(orc, p)
    f = np.array(f0, order="F", copy=True)
    df = np.zeros_like(f)
    t = 0.0
    nw = p.nx * p.ny * p.nz
    worst = {}
    for it in range(100):
        box.steps(1)
        got = pc.diag_summary(box.diag_raw(), nw)
        orc.ghosts(op, f)
        arms = np.sqrt(np.mean(f[3:-3, 3:-3, 3:-3, 4:7] ** 2) * 3)
        t, _, dg = orc.time_step(op, f, df, t, p.dt, False, diag=True, nthreads=8)
        ref = orc.diag_summary(op, dg)
        for key in ("urms", "umax", "brms", "bmax", "ekin", "rhom", "jrms", "abm"):
            # <A.B> changes sign; its sum's round-off scales with arms * brms
            scale = arms * ref["brms"] if key == "abm" else abs(ref[key])
            e = abs(got[key] - ref[key]) / scale
            worst[key] = max(worst.get(key, 0.0), e)
            assert e <= tol, (it, key, got[key], ref[key])
        # div B is round-off in both codes: compare it with the current density
        assert got["divbrms"] <= (1e-5 if mode == "f32pair" else 1e-12) * ref["jrms"]
        assert ref["divbrms"] <= 1e-12 * ref["jrms"]
    print(mode, {k: f"{v:.1e}" for k, v in worst.items()})


def _printed_unit(text):
    mant, _, exp = text.upper().partition("E")
    return 10.0 ** (int(exp or 0) - (len(mant.split(".")[1]) if "." in mant else 0))


@pytest.mark.parametrize("mode", ["f64", "dfloat", "f32pair"])
def test_mhd_abcforcing_sample_known_answer(pc, orc, mode):
    """samples/MHD-ABCforcing run on the GPU: 32^3 isothermal MHD, ABC forcing of uu
    (ampl 1e-4, k=1), B_ext=(0,0.1,0), nu=eta=0.1, CFL dt of the current state with
    cdt=0.4, 51 steps from the sample's Gaussian noise realisation (seed -10). Every
    printed row of t, dt, urms, umax, brms, abm and epsM in the sample's reference.out
    is met at 1.5 units of its last printed digit, in every state mode."""
    import json
    import os
    ref = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "mhd_abcforcing_ref.json")))
    prm = ref["params"]
    kw = dict(f64=dict(precision=8), dfloat=dict(precision=8, dfloat=1),
              f32pair=dict(precision=4, comp=1, tile=5))[mode]
    p = pc.default_params(nx=32, ny=32, nz=32, gamma=1.0, nu=prm["nu"], eta=prm["eta"], lforcing_cont=1,
                          ampl_ff=prm["ampl_ff"], kf=prm["k1_ff"], b_ext=tuple(prm["b_ext"]), cdt=prm["cdt"],
                          dt=0.0, dt_mode=2, diag_every=1, **kw)
    op = oracle_params(orc, p)
    f0 = orc.empty_f(op)
    orc.gaunoise_volume(op, prm["amplaa"], f0, 4, 6, -10)   # seed(1) = -10, start.f90:388
    box = pc.Box(p)
    box.load(f0)
    rows = {int(r["it"]): r for r in ref["printed"]}
    t0 = 0.0
    for it in range(prm["nt"]):
        box.steps(1)
        if it in rows:
            s = pc.diag_summary(box.diag_raw(), 32 ** 3)
            t, dt, _ = box.time()
            got = dict(s, t=t0, dt=dt, epsM=prm["eta"] * s["jrms"] ** 2)
            for c in ("t", "dt", "urms", "umax", "brms", "abm", "epsM"):
                r = rows[it][c]
                assert abs(got[c] - float(r)) <= 1.5 * _printed_unit(r), (mode, it, c, got[c], r)
        t0 = box.time()[0]


@pytest.mark.parametrize("tile", [0, 4, 5, 6, 7])
def test_isothermal_fp32_compensated(pc, ic, orc, tile):
    """FP32 state with the compensated 2N accumulation, within 1e-5 of the FP64 oracle,
    in the field-major layout (tile 0) and the packed field-pair layout (tiles 4-7)."""
    p = iso_params(pc, precision=4, comp=1, tile=tile)
    p.update(nu=5e-3, eta=5e-3)
    f0 = iso_state(pc, ic, p)
    ic.abc_flow(f0, p, ampl=0.1)
    box = pc.Box(p)
    box.load(f0)
    box.steps(100)
    g = box.store()
    ref, _, _ = run_oracle(orc, p, f0, 100)
    err = rel_err(g, ref, LOG7)
    assert np.all(err <= TOL32), err


@pytest.mark.parametrize("tile", [0, 4, 5, 7])
def test_entropy_fp32(pc, ic, orc, tile):
    p = pc.default_params(nx=32, ny=32, nz=32, lentropy=1, gamma=5.0 / 3.0, nu=2e-3, eta=2e-3, chi=2e-3,
                          dt=1e-3, precision=4, comp=1, tile=tile)
    f0 = ic.zeros(p)
    ic.abc_flow(f0, p, ampl=1.0, A=0.1, B=0.1, C=0.1, k=1.0)
    ic.gaussian_noise(f0, p, ["ax", "ay", "az"], 1e-4, 7)
    box = pc.Box(p)
    box.load(f0)
    box.steps(20)
    g = box.store()
    ref, _, _ = run_oracle(orc, p, f0, 20)
    err = rel_err(g, ref, LOG8)
    assert np.all(err <= TOL32), err


@pytest.mark.parametrize("tile", [0, 1, 2, 3])
def test_tile_variants_agree(pc, ic, tile):
    """Every tile variant and z-depth gives bitwise the same FP64 result."""
    base = None
    for zd in (0, 8):
        p = iso_params(pc, n=32, tile=tile, zdepth=zd)
        f0 = iso_state(pc, ic, p, seed=11)
        box = pc.Box(p)
        box.load(f0)
        box.steps(3)
        g = box.store()
        if base is None:
            base = g
        assert np.array_equal(g, base)   # z-depth never changes the arithmetic


def test_tiles_cross_agree(pc, ic):
    """Different tile shapes agree to round-off (FMA contraction may differ per variant)."""
    outs = []
    for tile in range(4):
        p = iso_params(pc, n=32, tile=tile)
        f0 = iso_state(pc, ic, p, seed=12)
        box = pc.Box(p)
        box.load(f0)
        box.steps(3)
        outs.append(box.store())
    for g in outs[1:]:
        assert np.all(rel_err(g, outs[0]) <= 1e-14)


@pytest.mark.parametrize("tile", [4, 5, 7])
def test_fp32_pair_layout_diagnostics_and_cfl(pc, ic, orc, tile):
    """Packed-pair FP32 kernel (tiles 5 and 7: z-direction data in tensor memory, 8 and 12 warps): diagnostics (FP64
    sums of FP32 cell values) and the lagged CFL dt agree with the FP64 oracle to FP32 round-off."""
    p = iso_params(pc, precision=4, comp=1, tile=tile, dt=0.0, dt_mode=2, cdt=0.4, diag_every=1,
                   b_ext=(0.0, 0.1, 0.0), lforcing_cont=1, ampl_ff=0.05, kf=2.0)
    f0 = iso_state(pc, ic, p, ampl=1e-2, seed=41)
    box = pc.Box(p)
    box.load(f0)
    box.steps(1)
    raw = box.diag_raw()
    t, dt, _ = box.time()
    op = oracle_params(orc, p)
    f = np.array(f0, order="F", copy=True)
    orc.ghosts(op, f)
    dt1, dg = orc.pde(op, f, np.zeros_like(f), 0.0, want_dt=True, diag=True)
    assert abs(dt * dt1 - 1.0) <= 1e-6
    for k in (orc.D_U2SUM, orc.D_B2SUM, orc.D_EKINSUM, orc.D_RHOSUM, orc.D_J2SUM):
        assert abs(raw[k + 1] - dg[k]) <= 1e-5 * abs(dg[k]), k


@pytest.mark.parametrize("n", [(37, 19, 11), (6, 6, 6), (6, 40, 7)])
@pytest.mark.parametrize("mode", ["f64", "dfloat", "f32pair", "f32"])
def test_ragged_and_minimal_grids(pc, ic, orc, n, mode):
    """Grids that are not multiples of any tile, and the smallest grid the
    periodic ghost images allow (6 cells per axis), in every state mode."""
    kw = dict(f64=dict(precision=8), dfloat=dict(precision=8, dfloat=1),
              f32pair=dict(precision=4, comp=1, tile=5), f32=dict(precision=4, comp=1, tile=0))[mode]
    p = pc.default_params(nx=n[0], ny=n[1], nz=n[2], gamma=1.0, nu=1e-2, eta=1e-2, dt=2e-3,
                          lforcing_cont=1, ampl_ff=0.02, kf=1.0, b_ext=(0.0, 0.05, 0.0), **kw)
    p.update(Lxyz=(0.37 * np.pi, 0.19 * np.pi, 0.11 * np.pi) if n[0] == 37 else (2 * np.pi,) * 3)
    f0 = iso_state(pc, ic, p, ampl=1e-2, seed=21)
    box = pc.Box(p)
    box.load(f0)
    box.steps(5)
    g = box.store()
    ref, _, _ = run_oracle(orc, p, f0, 5)
    tol = TOL32 if mode.startswith("f32") else TOL64
    err = rel_err(g, ref, LOG7 if mode.startswith("f32") else ())
    assert np.all(err <= tol), err
    assert np.array_equal(ic.fill_ghosts(g.copy()), g)


@pytest.mark.parametrize("n,lentropy,tile", [((37, 19, 11), 0, 6), ((64, 40, 70), 0, 5), ((24, 16, 40), 1, 4)])
def test_fp32_pair_cfl_pass(pc, ic, orc, n, lentropy, tile):
    """The FP32 pair layout's own CFL pass (dt from the current f) against the
    oracle's set_dt1_max on the same state, on ragged grids and with entropy."""
    kw = dict(lentropy=1, gamma=5.0 / 3.0, chi=0.02) if lentropy else {}
    p = iso_params(pc, precision=4, comp=1, tile=tile, dt=0.0, dt_mode=2, cdt=0.4, b_ext=(0.05, 0.0, 0.1),
                   nu=0.02, eta=0.03, **kw).update(nx=n[0], ny=n[1], nz=n[2])
    f0 = ic.zeros(p)
    ic.gaussian_noise(f0, p, ["ux", "uy", "uz", "ax", "ay", "az", "lnrho"] + (["ss"] if lentropy else []), 5e-2, 43)
    ic.fill_ghosts(f0)
    box = pc.Box(p)
    box.load(f0)
    box.steps(1)
    t, dt, _ = box.time()
    op = oracle_params(orc, p)
    f = np.array(f0, order="F", copy=True)
    orc.ghosts(op, f)
    dt1, _ = orc.pde(op, f, np.zeros_like(f), 0.0, want_dt=True)
    assert abs(dt * dt1 - 1.0) <= 2e-6
    assert abs(t - dt) <= 1e-15 * dt


def test_fp32_pair_cfl_pass_flags_nan(pc, ic):
    L = pc.load()
    p = iso_params(pc, precision=4, comp=1, tile=5, dt=0.0, dt_mode=2)
    f = ic.zeros(p)
    ic.gaussian_noise(f, p, ["ux", "uy", "uz"], 1e-2, 3)
    f[7, 9, 11, 5] = np.nan   # A_y: reaches dt only through B
    box = pc.Box(p)
    box.load(f)
    box.steps(1)
    with pytest.raises(pc.PcgbError, match="non-finite"):
        box.sync()
    L.pcgb_clear_error()
