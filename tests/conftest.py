"""Shared test setup: the `gpu` marker, import paths, and helpers that build
matching parameter blocks for the CUDA library and the FP64 oracle."""
import importlib
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU and the CUDA library")


@pytest.fixture(scope="session")
def pc():
    return importlib.import_module("pencil-code_gb300")


@pytest.fixture(scope="session")
def ic():
    return importlib.import_module("pencil-code_gb300.initcond")


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.build()
    return oracle


def oracle_params(orc, p):
    """Oracle parameter block equal to a library Params block."""
    return orc.make_params(
        nx=p.nx, ny=p.ny, nz=p.nz, lentropy=p.lentropy,
        x0=p.xyz0[0], y0=p.xyz0[1], z0=p.xyz0[2], Lx=p.Lxyz[0], Ly=p.Lxyz[1], Lz=p.Lxyz[2],
        gamma=p.gamma, cs0=p.cs0, rho0=p.rho0, cp=p.cp, nu=p.nu, eta=p.eta, chi=p.chi, mu0=p.mu0,
        lforcing_cont=p.lforcing_cont, ampl_ff=p.ampl_ff, kf=p.kf, relhel=p.relhel,
        abc_a=p.abc_a, abc_b=p.abc_b, abc_c=p.abc_c, ampl_fcont_uu=p.ampl_fcont_uu,
        b_ext=tuple(p.b_ext), lohmic_heat=p.lohmic_heat, lviscosity_heat=p.lviscosity_heat,
        cdt=p.cdt, cdtv=p.cdtv, lupw_uu=p.lupw_uu, lupw_lnrho=p.lupw_lnrho,
        bc=[[[p.bc[a][f][0], p.bc[a][f][1]] for f in range(8)] for a in range(3)])


def rel_err(a, b, log_fields=()):
    """Per-field max |a-b| / scale over the interior, scale = max |b|.

    For the logarithmic variables (lnrho, ss; indices in log_fields) the scale
    is max(max |b|, 1): an absolute error in ln(rho) is the relative error of
    rho, and ss is in units of cp = 1."""
    out = []
    for k in range(a.shape[3]):
        A = a[3:-3, 3:-3, 3:-3, k]
        B = b[3:-3, 3:-3, 3:-3, k]
        scale = np.max(np.abs(B))
        if k in log_fields:
            scale = max(scale, 1.0)
        out.append(np.max(np.abs(A - B)) / scale if scale > 0 else np.max(np.abs(A - B)))
    return np.array(out)


LOG7 = (3,)       # lnrho in the 7-field (isothermal) f-array
LOG8 = (3, 4)     # lnrho, ss in the 8-field (entropy) f-array
