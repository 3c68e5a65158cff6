"""The oracle's upwinded advection (lupw_uu, lupw_lnrho) on a known answer.

The reference's upwind correction of u.grad f is sum_j |u_j| D6_j f with
D6_j the 6th difference times dx_1/60 (deriv.f90 der6_main, upwind=T;
sub.f90:7491-7574).  On a single Fourier mode f = sin(k x) the stencil
(-20, 15, -6, 1) has the closed form -(2 sin(k dx / 2))^6 sin(k x), so with a
uniform velocity U along x the upwinded right-hand side differs from the
plain one by exactly |U| (dx_1/60) (-(2 sin(k dx/2))^6) sin(k x) in the
advected field.  No GPU.
"""
import numpy as np
import pytest


@pytest.mark.parametrize("which", ["lnrho", "uu"])
def test_upwind_correction_on_fourier_mode(orc, which):
    n, k, U = 32, 3.0, -0.3
    kw = dict(nx=n, ny=8, nz=8)
    plain = orc.make_params(**kw)
    upw = orc.make_params(lupw_lnrho=int(which == "lnrho"), lupw_uu=int(which == "uu"), **kw)
    x, _, _ = orc.grid(plain)
    f = orc.empty_f(plain)
    f[..., 0] = U
    mode = 0.01 * np.sin(k * x)
    field = 3 if which == "lnrho" else 1   # lnrho, or uy advected by ux
    f[..., field] = mode[:, None, None]
    orc.ghosts(plain, f)
    df0 = np.zeros_like(f)
    df1 = np.zeros_like(f)
    orc.pde(plain, f, df0, 0.0)
    orc.pde(upw, f, df1, 0.0)
    dx = 2 * np.pi / n
    theta = k * dx
    expect = abs(U) * (1.0 / 60.0) / dx * (-(2 * np.sin(theta / 2)) ** 6) * mode[3:-3]
    diff = (df1 - df0)[3:-3, 3:-3, 3:-3, field]
    assert np.max(np.abs(diff - expect[:, None, None])) <= 1e-15 + 1e-12 * np.max(np.abs(expect))
    # the other fields change by round-off at most (the 6th difference of the
    # uniform ux is zero up to the rounding of its weighted sum)
    others = [i for i in range(f.shape[3]) if i != field]
    assert np.max(np.abs(df1[3:-3, 3:-3, 3:-3][..., others] - df0[3:-3, 3:-3, 3:-3][..., others])) <= 1e-15


def test_upwind_is_zero_for_polynomials_of_degree_five(orc):
    """The 6th difference annihilates polynomials up to degree 5: upwinding of a
    smooth quadratic profile changes nothing but round-off."""
    kw = dict(nx=16, ny=16, nz=16)
    plain = orc.make_params(**kw)
    upw = orc.make_params(lupw_lnrho=1, lupw_uu=1, **kw)
    f = orc.empty_f(plain)
    ii = np.arange(f.shape[0], dtype=float)[:, None, None]
    f[..., 0] = 0.2
    f[..., 3] = 1e-3 * (ii - 10.0) ** 2
    df0 = np.zeros_like(f)
    df1 = np.zeros_like(f)
    orc.pde(plain, f, df0, 0.0)
    orc.pde(upw, f, df1, 0.0)
    assert np.max(np.abs(df1 - df0)) <= 1e-13
