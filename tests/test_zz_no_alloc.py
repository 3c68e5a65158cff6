"""pcgb_substep_noalloc: the allocation-free substep.

It exists for callers that cannot allocate device memory when they step the
solver (their memory belongs to another allocator, or their time loop must not
pay the device-wide synchronisation of cudaMalloc/cudaFree).  The test owns
the buffers (allocated here with torch), calls the entry point twice in a row
(substep 1 then substep 2, the second reading the first's output), and checks
each result against the library's existing path: the reference plug-in calls
substepGPU / copyFarray / getGPUReducedVars on the same initial state.
Tolerance: the FP64 parity tolerance of the other GPU tests (1e-11).
"""
import ctypes as C
import importlib

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

TOL64 = 1e-11


def to_device_layout(f, xoff, px):
    """Host f(mx,my,mz,nf) (Fortran order) -> device layout [nf][mz][my][px]."""
    mx, my, mz, nf = f.shape
    d = np.zeros((nf, mz, my, px))
    d[:, :, :, xoff - 3:xoff - 3 + mx] = np.transpose(f, (3, 2, 1, 0))
    return d


def from_device_layout(d, xoff, mx):
    return np.asfortranarray(np.transpose(d[:, :, :, xoff - 3:xoff - 3 + mx], (3, 2, 1, 0)))


def test_noalloc_two_substeps_match_plugin(pc, ic):
    torch = pytest.importorskip("torch")
    gpu = importlib.import_module("pencil-code_gb300.gpu")
    L = pc.load()
    n = (40, 32, 48)
    p = pc.default_params(nx=n[0], ny=n[1], nz=n[2], gamma=1.0, nu=8e-3, eta=1e-2, dt=3e-3, precision=8,
                          lforcing_cont=1, ampl_ff=0.03, kf=2.0, b_ext=(0.0, 0.05, 0.0), tile=0)
    f0 = ic.zeros(p)
    ic.gaussian_noise(f0, p, ["ux", "uy", "uz", "ax", "ay", "az"], 1e-2, 31)
    ic.gaussian_noise(f0, p, ["lnrho"], 1e-3, 32)
    ic.fill_ghosts(f0)

    # existing entry points: the plug-in path, copying f back after each substep
    f = f0.copy(order="F")
    gpu.initialize_gpu(f, p, nt=1)
    gpu.request_diagnostics()
    gpu.rhs_gpu(1, 0.0)
    ref1 = gpu.copy_farray_from_gpu(np.zeros_like(f0, order="F")).copy(order="F")
    red_ref = gpu.get_gpu_reduced_vars()
    gpu.rhs_gpu(2, 0.0)
    ref2 = gpu.copy_farray_from_gpu(np.zeros_like(f0, order="F")).copy(order="F")
    gpu.finalize_gpu()

    # layout as the library reports it
    box = pc.Box(p)
    info = box.info()
    box.close()
    xoff = 128 // 8
    px = xoff + ((p.nx + 8 + xoff - 1) // xoff) * xoff
    assert (info["xoff"], info["px"]) == (xoff, px)

    mx = p.nx + 6
    a = torch.from_numpy(to_device_layout(f0, xoff, px)).cuda()
    b = torch.zeros_like(a)
    df = torch.zeros_like(a)
    red = np.zeros(10)
    rp = red.ctypes.data_as(C.POINTER(C.c_double))
    torch.cuda.synchronize()

    rc = L.pcgb_substep_noalloc(C.byref(p), 1, 3e-3, C.c_void_p(a.data_ptr()), C.c_void_p(b.data_ptr()),
                                C.c_void_p(df.data_ptr()), rp, None)
    assert rc == 0
    torch.cuda.synchronize()
    out1 = from_device_layout(b.cpu().numpy(), xoff, mx)
    assert np.all(rel_err(out1, ref1) <= TOL64)
    # ghosts written by the kernel are the periodic images
    assert np.array_equal(ic.fill_ghosts(out1.copy()), out1)
    ncell = p.nx * p.ny * p.nz
    got = pc.diag_summary(np.concatenate([red, np.zeros(3)]), ncell)
    for k in ("urms", "umax", "brms", "bmax", "ekin", "rhom", "jrms", "abm"):
        assert abs(got[k] - red_ref[k]) <= 1e-12 * abs(red_ref[k]), k
    assert red[0] > 0   # CFL inverse timestep of substep 1

    # second call in a row: substep 2 reads the first call's f_out and df
    rc = L.pcgb_substep_noalloc(C.byref(p), 2, 3e-3, C.c_void_p(b.data_ptr()), C.c_void_p(a.data_ptr()),
                                C.c_void_p(df.data_ptr()), None, None)
    assert rc == 0
    torch.cuda.synchronize()
    out2 = from_device_layout(a.cpu().numpy(), xoff, mx)
    assert np.all(rel_err(out2, ref2) <= TOL64)


def test_noalloc_rejects_oversize(pc):
    L = pc.load()
    p = pc.default_params(nx=8192, ny=16, nz=16, precision=8, dt=1e-3)
    dummy = C.c_void_p(16)
    assert L.pcgb_substep_noalloc(C.byref(p), 1, 1e-3, dummy, dummy, dummy, None, None) == 7
    p = pc.default_params(nx=32, ny=32, nz=32, precision=8, dt=1e-3)
    assert L.pcgb_substep_noalloc(C.byref(p), 4, 1e-3, dummy, dummy, dummy, None, None) == 2


def test_noalloc_fp32_plain_2n_against_oracle(pc, ic, orc):
    """FP32 state through the allocation-free entry: it runs the plain 2N update
    (the compensated carry would need state kept between calls), so its error is
    stated against the FP64 oracle: 20 RK3 steps of the 32^3 isothermal case
    (noise 1e-3 plus an ABC flow of 0.1) within 1e-5 per field, lnrho measured
    against max(|lnrho|, 1).  Calls after the first allocate no device memory:
    the device's free memory and torch's allocation count do not change."""
    torch = pytest.importorskip("torch")
    from conftest import LOG7, oracle_params
    L = pc.load()
    n, steps, dt = 32, 20, 5e-3
    p = pc.default_params(nx=n, ny=n, nz=n, gamma=1.0, nu=5e-3, eta=5e-3, dt=dt, precision=4, comp=0, tile=0)
    f0 = ic.zeros(p)
    ic.gaussian_noise(f0, p, ["ux", "uy", "uz", "ax", "ay", "az"], 1e-3, 1)
    ic.abc_flow(f0, p, ampl=0.1)
    ic.fill_ghosts(f0)
    xoff = 128 // 4
    px = xoff + ((p.nx + 8 + xoff - 1) // xoff) * xoff
    mx = p.nx + 6
    a = torch.from_numpy(to_device_layout(f0, xoff, px).astype(np.float32)).cuda()
    b = torch.zeros_like(a)
    df = torch.zeros_like(a)
    bufs = [a, b]
    torch.cuda.synchronize()
    rc = L.pcgb_substep_noalloc(C.byref(p), 1, dt, C.c_void_p(a.data_ptr()), C.c_void_p(b.data_ptr()),
                                C.c_void_p(df.data_ptr()), None, None)
    assert rc == 0
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    allocs0 = torch.cuda.memory_stats().get("allocation.all.allocated", 0)
    k = 1   # the first substep above wrote bufs[1]
    for it in range(3 * steps - 1):
        s = (it + 1) % 3 + 1
        src, dst = bufs[k], bufs[k ^ 1]
        rc = L.pcgb_substep_noalloc(C.byref(p), s, dt, C.c_void_p(src.data_ptr()), C.c_void_p(dst.data_ptr()),
                                    C.c_void_p(df.data_ptr()), None, None)
        assert rc == 0
        k ^= 1
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    assert torch.cuda.memory_stats().get("allocation.all.allocated", 0) == allocs0
    g = from_device_layout(bufs[k].cpu().numpy().astype(np.float64), xoff, mx)
    op = oracle_params(orc, p)
    ref = np.array(f0, order="F", copy=True)
    dref = np.zeros_like(ref)
    t = 0.0
    for _ in range(steps):
        t, _, _ = orc.time_step(op, ref, dref, t, dt, False, nthreads=8)
    orc.ghosts(op, ref)
    err = rel_err(g, ref, LOG7)
    print("noalloc FP32 plain 2N, 20 steps:", [f"{e:.2e}" for e in err])
    assert np.all(err <= 1e-5), err
