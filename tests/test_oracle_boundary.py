"""The oracle's boundary conditions and non-periodic grid (no GPU).

bc_sym_x/y/z (boundcond.f90:2637-2677, 3483-3530, 3842-3900) on random fields:
's' mirrors, 'a' mirrors with a sign change and zeroes the boundary value,
'a2' reflects about the boundary value (2 f(n1) - f(n1+i); on the upper z side
f(n2) + (f(n2) - f(n2-i)), as the reference writes it).  boundconds_x runs
before _y and _z, so corner ghosts are the later direction's condition applied
to ghosts the earlier one filled.  grid.f90:123-151: a non-periodic axis has
dx = L/(n-1) with points on both boundaries.
"""
import importlib

import numpy as np
import pytest

NG = 3


def _bc(nf=7, **per_dir):
    bc = [[[0, 0] for _ in range(8)] for _ in range(3)]
    codes = {"p": 0, "s": 1, "a": 2, "a2": 3}
    for d, key in enumerate(("x", "y", "z")):
        for k, e in enumerate(per_dir.get(key, [])):
            lo, _, hi = e.partition(":")
            bc[d][k] = [codes[lo], codes[hi or lo]]
    return bc


def test_grid_of_non_periodic_axis(orc):
    p = orc.make_params(nx=10, ny=8, nz=12, bc=_bc(z=["s"] * 7))
    x, y, z = orc.grid(p)
    dz = 2 * np.pi / 11
    assert z[NG] == -np.pi and abs(z[NG + 11] - np.pi) <= 1e-15
    np.testing.assert_allclose(np.diff(z), dz, rtol=1e-14)
    np.testing.assert_allclose(x[NG:NG + 10], -np.pi + (np.arange(10) + 0.5) * 2 * np.pi / 10, rtol=0, atol=1e-15)


@pytest.mark.parametrize("d", [0, 1, 2])
def test_symmetric_conditions_along_each_axis(orc, d):
    codes = ["s", "a", "a2", "s:a", "a:a2", "a2:s", "a2"]
    p = orc.make_params(nx=9, ny=10, nz=11, bc=_bc(**{"xyz"[d]: codes}))
    rng = np.random.Generator(np.random.PCG64(d))
    f = np.asfortranarray(rng.standard_normal((15, 16, 17, 7)))
    g = f.copy(order="F")
    orc.ghosts(p, g)
    n = (9, 10, 11)[d]
    n1, n2 = NG, NG + n - 1

    def line(a, i):   # f along axis d at index i (all other indices)
        return np.take(a, i, axis=d)

    other = [a for a in range(3) if a != d]
    interior = [slice(NG, -NG)] * 2   # interior of the other axes (their ghosts follow later passes)

    def inner(a):
        idx = [slice(None)] * 3
        idx[other[0]] = interior[0]
        idx[other[1]] = interior[1]
        del idx[d]
        return a[tuple(idx)]

    for k, c in enumerate(codes):
        lo, _, hi = c.partition(":")
        hi = hi or lo
        for i in range(1, NG + 1):
            fi, f0 = line(f[..., k], n1 + i), line(f[..., k], n1)
            want = {"s": fi, "a": -fi, "a2": 2.0 * f0 - fi}[lo]
            assert np.array_equal(inner(line(g[..., k], n1 - i)), inner(want)), (k, "lower", i)
            fi, f0 = line(f[..., k], n2 - i), line(f[..., k], n2)
            if hi == "a2" and d == 2:
                want = f0 + (f0 - fi)
            else:
                want = {"s": fi, "a": -fi, "a2": 2.0 * f0 - fi}[hi]
            assert np.array_equal(inner(line(g[..., k], n2 + i)), inner(want)), (k, "upper", i)
        if lo == "a":
            assert np.all(line(g[..., k], n1) == 0.0)
        if hi == "a":
            assert np.all(line(g[..., k], n2) == 0.0)


def test_corner_ghosts_follow_direction_order(orc):
    """x 'a', y 's': a corner ghost (x ghost, y ghost) is the y mirror of the x-filled row."""
    p = orc.make_params(nx=8, ny=9, nz=7, bc=_bc(x=["a"] * 7, y=["s"] * 7))
    f = np.asfortranarray(np.random.Generator(np.random.PCG64(5)).standard_normal((14, 15, 13, 7)))
    orc.ghosts(p, f)
    # corner (l = n1-1, m = m1-2): y mirror of row m1+2 at l = n1-1, which is -f(n1+1, m1+2)
    assert np.array_equal(f[NG - 1, NG - 2, NG:-NG, 0], f[NG - 1, NG + 2, NG:-NG, 0])
    assert np.array_equal(f[NG - 1, NG + 2, NG:-NG, 0], -f[NG + 1, NG + 2, NG:-NG, 0])
    # z stays periodic
    assert np.array_equal(f[:, :, 0, 3], f[:, :, 7, 3])


def test_periodic_codes_reproduce_the_periodic_fill(orc, ic):
    p = orc.make_params(nx=8, ny=7, nz=6)
    f = np.asfortranarray(np.random.Generator(np.random.PCG64(2)).standard_normal((14, 13, 12, 7)))
    g = f.copy(order="F")
    orc.ghosts(p, g)
    assert np.array_equal(g, ic.fill_ghosts(f.copy(order="F")))


def test_namelist_boundary_conditions():
    nl = importlib.import_module("pencil-code_gb300.namelist")
    start = "&init_pars lperi=T,T,F, bcz='a2','a2','a','a2','s:a2','s','a' /"
    p, _, _ = nl.params_from_namelists(start, "", n=(16, 16, 16))
    assert p.periodic(0) and p.periodic(1) and not p.periodic(2)
    assert [list(p.bc[2][k]) for k in range(7)] == [[3, 3], [3, 3], [2, 2], [3, 3], [1, 3], [1, 1], [2, 2]]
    # run.in's list overrides start.in's; codes outside this path are refused
    with pytest.raises(ValueError, match="bcz"):
        nl.params_from_namelists(start, "&run_pars bcz='g:s','s','a','a2','s','s','a' /", n=(16, 16, 16))
    with pytest.raises(ValueError, match="lperi"):
        nl.params_from_namelists("&init_pars bcx='s' /", "", n=(16, 16, 16))
