"""Full-size cases, where the FP64 oracle would take too long: the state modes
checked against each other through size-independent properties.

- 256^3 entropy MHD, ABC flow, 200 steps (the 256^3 parity configuration):
  double-float within 1e-11 of native FP64, FP32 within 1e-5 (lnrho and ss
  measured against max(|field|, 1)); div B of the stored state at round-off.
- 512^3 isothermal forced MHD from the device initial condition, 25 steps
  (the headline physics): the same bars.
Native FP64 is pinned to the oracle at 32^3 (test_gpu_parity.py); here it is
the reference for the other two modes at the full sizes.
"""
import numpy as np
import pytest

from conftest import LOG7, LOG8, rel_err

pytestmark = pytest.mark.gpu

TOL_DD = 1e-11
TOL32 = 1e-5


def _divb_rel(pc, p, f):
    """max |div B| / max |J|-scale of the stored f, 6th-order central differences."""
    iax = 5 if p.lentropy else 4
    dx = [p.Lxyz[i] / n for i, n in enumerate((p.nx, p.ny, p.nz))]

    def d(a, ax, h):
        return (45 * (np.roll(a, -1, ax) - np.roll(a, 1, ax)) - 9 * (np.roll(a, -2, ax) - np.roll(a, 2, ax))
                + (np.roll(a, -3, ax) - np.roll(a, 3, ax))) / (60 * h)

    A = [f[3:-3, 3:-3, 3:-3, iax + k] for k in range(3)]
    bx = d(A[2], 1, dx[1]) - d(A[1], 2, dx[2])
    by = d(A[0], 2, dx[2]) - d(A[2], 0, dx[0])
    bz = d(A[1], 0, dx[0]) - d(A[0], 1, dx[1])
    divb = d(bx, 0, dx[0]) + d(by, 1, dx[1]) + d(bz, 2, dx[2])
    scale = max(np.abs(d(bx, 0, dx[0])).max(), np.abs(d(by, 1, dx[1])).max(), 1e-300)
    return float(np.abs(divb).max() / scale)


def test_entropy_256_three_modes(pc, ic):
    kw = dict(nx=256, ny=256, nz=256, lentropy=1, gamma=5.0 / 3.0, nu=2e-3, eta=2e-3, chi=2e-3, dt=1e-3)
    p64 = pc.default_params(precision=8, **kw)
    f0 = ic.zeros(p64)
    ic.abc_flow(f0, p64, ampl=1.0, A=0.1, B=0.1, C=0.1, k=1.0)
    ic.gaussian_noise(f0, p64, ["ax", "ay", "az"], 1e-4, 7)
    out = {}
    for name, extra in (("f64", dict(precision=8)), ("dd", dict(precision=8, dfloat=1)),
                        ("f32", dict(precision=4, comp=1))):
        box = pc.Box(pc.default_params(**{**kw, **extra}))
        box.load(f0)
        box.steps(200)
        out[name] = box.store()
        box.close()
    err_dd = rel_err(out["dd"], out["f64"], LOG8)
    err_32 = rel_err(out["f32"], out["f64"], LOG8)
    assert np.all(err_dd <= TOL_DD), err_dd
    assert np.all(err_32 <= TOL32), err_32
    assert _divb_rel(pc, p64, out["f64"]) <= 1e-9
    assert np.array_equal(ic.fill_ghosts(out["dd"].copy()), out["dd"])


def test_headline_physics_512_three_modes(pc):
    n = 512
    out = {}
    for name, extra in (("f64", dict(precision=8)), ("dd", dict(precision=8, dfloat=1)),
                        ("f32", dict(precision=4, comp=1))):
        p = pc.default_params(nx=n, ny=n, nz=n, gamma=1.0, nu=5e-4, eta=5e-4, dt=2e-4, lforcing_cont=1,
                              ampl_ff=0.02, kf=2.0, relhel=1.0, **extra)
        box = pc.Box(p)
        for k in range(7):
            box.init_field(k, "zero")
        for k in range(3):
            box.init_field(4 + k, "noise", ampl=1e-5, seed=20260 + k)
        box.steps(25)
        out[name] = box.store()
        box.close()
    err_dd = rel_err(out["dd"], out["f64"], LOG7)
    err_32 = rel_err(out["f32"], out["f64"], LOG7)
    assert np.all(err_dd <= TOL_DD), err_dd
    assert np.all(err_32 <= TOL32), err_32
