"""The reference plug-in entry points (gpu_astaroth_ansi.c set) driven the way
the Fortran GPU module drives them (gpu_astaroth.f90, timestep.f90 with lgpu=T),
checked against the FP64 oracle and against the Box API."""
import importlib

import numpy as np
import pytest

from conftest import oracle_params, rel_err

pytestmark = pytest.mark.gpu


def test_plugin_time_step_matches_oracle(pc, ic, orc):
    gpu = importlib.import_module("pencil-code_gb300.gpu")
    p = pc.default_params(nx=32, ny=32, nz=32, gamma=1.0, nu=5e-3, eta=5e-3, dt=5e-3, precision=8,
                          lforcing_cont=1, ampl_ff=1e-2, kf=1.0)
    f = ic.zeros(p)
    ic.gaussian_noise(f, p, ["ux", "uy", "uz", "ax", "ay", "az"], 1e-3, 21)
    f0 = f.copy(order="F")
    gpu.register_gpu()
    gpu.initialize_gpu(f, p, t=0.0, nt=10)          # loads f (nt > 0)
    for it in range(10):                             # timestep.f90:77 advance_substeps, lgpu=T
        gpu.gpu_prepare_for_first_substep(0.0)
        for itsub in (1, 2, 3):
            gpu.before_boundary_gpu(False, itsub, 0.0)
            gpu.rhs_gpu(itsub, 0.0)
            gpu.update_after_substep_gpu()
    gpu.copy_farray_from_gpu(f)
    t = gpu.get_time()
    gpu.finalize_gpu()
    op = oracle_params(orc, p)
    ref = f0.copy(order="F")
    df = np.zeros_like(ref)
    tr = 0.0
    for _ in range(10):
        tr, _, _ = orc.time_step(op, ref, df, tr, 5e-3, False, nthreads=8)
    orc.ghosts(op, ref)
    assert np.all(rel_err(f, ref) <= 1e-11)
    assert abs(t - tr) <= 1e-13


def test_plugin_substep_sequence_enforced(pc, ic):
    gpu = importlib.import_module("pencil-code_gb300.gpu")
    p = pc.default_params(nx=16, ny=16, nz=16, gamma=1.0, dt=1e-3, precision=8)
    f = ic.zeros(p)
    gpu.initialize_gpu(f, p, nt=1)
    with pytest.raises(pc.PcgbError):
        gpu.rhs_gpu(2, 0.0)      # substep 2 before substep 1
    gpu.rhs_gpu(1, 0.0)
    gpu.finalize_gpu()


def test_plugin_reduced_vars_and_update(pc, ic, orc):
    gpu = importlib.import_module("pencil-code_gb300.gpu")
    p = pc.default_params(nx=32, ny=32, nz=32, gamma=1.0, nu=5e-3, eta=5e-3, dt=5e-3, precision=8,
                          b_ext=(0.0, 0.1, 0.0))
    f = ic.zeros(p)
    ic.gaussian_noise(f, p, ["ux", "uy", "uz", "ax", "ay", "az"], 1e-2, 22)
    f0 = f.copy(order="F")
    gpu.initialize_gpu(f, p, nt=1)
    gpu.update_on_gpu("nu", 1e-2)                 # updateInConfigScalName
    gpu.update_on_gpu("b_ext", [0.0, 0.2, 0.0])   # updateInConfigVecName
    with pytest.raises(pc.PcgbError):
        gpu.update_on_gpu("no_such_parameter", 1.0)
    gpu.request_diagnostics()
    gpu.time_step(1)
    red = gpu.get_gpu_reduced_vars()
    gpu.finalize_gpu()
    q = p.update(nu=1e-2, b_ext=(0.0, 0.2, 0.0))
    op = oracle_params(orc, q)
    ref = f0.copy(order="F")
    orc.ghosts(op, ref)
    _, dg = orc.pde(op, ref, np.zeros_like(ref), 0.0, diag=True)
    s = orc.diag_summary(op, dg)
    for k in ("urms", "umax", "brms", "bmax", "ekin", "rhom", "jrms", "abm"):
        assert abs(red[k] - s[k]) <= 1e-12 * abs(s[k]), (k, red[k], s[k])
    assert red["step"] == 0 and abs(red["dt"] - 5e-3) < 1e-18


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tile", [(8, -1), (4, 4), (4, 0)])
def test_pinned_and_pageable_host_arrays_agree(pc, ic, precision, tile):
    """Page-locked host arrays are read and written by the layout kernels directly;
    pageable ones go through the staging buffers.  Both give the same bits."""
    torch = pytest.importorskip("torch")
    p = pc.default_params(nx=40, ny=24, nz=16, gamma=1.0, nu=5e-3, eta=5e-3, dt=1e-3, precision=precision, tile=tile,
                          comp=1 if precision == 4 else 0)
    f0 = ic.zeros(p)
    ic.gaussian_noise(f0, p, ["ux", "uy", "uz", "ax", "ay", "az", "lnrho"], 1e-2, 3)
    shape = pc.host_shape(p)
    pinned_in = torch.zeros(int(np.prod(shape)), dtype=torch.float64, pin_memory=True)
    pinned_out = torch.zeros(int(np.prod(shape)), dtype=torch.float64, pin_memory=True)
    fin = pinned_in.numpy().reshape(shape, order="F")
    fout = pinned_out.numpy().reshape(shape, order="F")
    fin[...] = f0
    a = pc.Box(p)
    a.load(f0)
    a.steps(2)
    ra = a.store()
    b = pc.Box(p)
    b.load(fin)
    b.steps(2)
    b.store(fout)
    assert np.array_equal(ra, fout)
    a.close(); b.close()
