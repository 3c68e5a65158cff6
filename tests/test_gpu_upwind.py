"""Upwinded advection (lupw_uu, lupw_lnrho) and random helical forcing of the
vector potential (lmagnetic_forcing) on the GPU against the oracle.

Upwinding subtracts sum_j |u_j| D6_j f (the 6th difference times dx_1/60,
deriv.f90 der6_main with upwind=T) from u.grad u and u.grad lnrho
(hydro.f90:3662, density.f90:2772, sub.f90:7491-7574).  The kernels carrying
it are separate variants of the default tiles.  Bars as in the other parity
tests: FP64 and double-float 1e-11 per field, FP32 1e-5 (lnrho and ss against
max(|field|, 1)).
"""
import ctypes as C
import importlib

import numpy as np
import pytest

from conftest import LOG7, LOG8, oracle_params, rel_err

pytestmark = pytest.mark.gpu

MODES = {
    "f64": dict(precision=8),
    "f64_tile1": dict(precision=8, tile=1),
    "dfloat": dict(precision=8, dfloat=1, tile=3),
    "dfloat_tile2": dict(precision=8, dfloat=1, tile=2),
    "dfloat_pair": dict(precision=8, dfloat=1),
    "dfloat_pair6": dict(precision=8, dfloat=1, tile=6),
    "f32pair": dict(precision=4, comp=1),
    "f32pair5": dict(precision=4, comp=1, tile=5),
    "f32": dict(precision=4, comp=1, tile=1),
}


def _params(pc, lentropy=0, n=(24, 20, 16), **kw):
    p = pc.default_params(nx=n[0], ny=n[1], nz=n[2], lentropy=lentropy, gamma=(5.0 / 3.0 if lentropy else 1.0),
                          nu=2e-3, eta=2e-3, chi=(2e-3 if lentropy else 0.0), dt=2e-3, lupw_uu=1, lupw_lnrho=1)
    return p.update(**kw)


def _initial(pc, ic, p, seed=3):
    """Grid-scale noise in every field, so the 6th differences are large."""
    f = ic.zeros(p)
    rng = np.random.Generator(np.random.PCG64(seed))
    nf = f.shape[3]
    f[3:-3, 3:-3, 3:-3, :] = 0.05 * rng.standard_normal((p.nx, p.ny, p.nz, nf))
    return ic.fill_ghosts(f)


def _oracle(orc, p, f0, nsteps, kvec=None, kav=None):
    op = oracle_params(orc, p)
    f = np.array(f0, order="F", copy=True)
    df = np.zeros_like(f)
    t, dt, state = 0.0, p.dt, p.seed_ff
    for _ in range(nsteps):
        if p.lforcing_hel:
            rec, state = orc.helical_coefs(op, p.force_hel, kvec, kav, state)
            if p.lmagnetic_forcing:   # the secondary record of lmhd_forcing is drawn, its force is zero
                _, state = orc.helical_coefs(op, p.force_hel, kvec, kav, state)
        t, dt, _ = orc.time_step(op, f, df, t, dt, False, nthreads=8)
        if p.lforcing_hel:
            orc.add_helical(op, f, rec, dt, 1 if p.lmagnetic_forcing else 0)
            orc.ghosts(op, f)
    orc.ghosts(op, f)
    return f, t


def _check(g, ref, p, mode):
    log = LOG8 if p.lentropy else LOG7
    err = rel_err(g, ref, log)
    tol = 1e-5 if p.precision == 4 else 1e-11
    assert np.all(err <= tol), (mode, err)


@pytest.mark.parametrize("mode", list(MODES))
def test_upwinding_matches_oracle(pc, ic, orc, mode):
    p = _params(pc, **MODES[mode])
    f0 = _initial(pc, ic, p)
    box = pc.Box(p)
    box.load(f0)
    box.steps(10)
    g = box.store()
    ref, t_ref = _oracle(orc, p, f0, 10)
    _check(g, ref, p, mode)
    assert abs(box.time()[0] - t_ref) <= 1e-12 * t_ref


@pytest.mark.parametrize("mode", ["f64", "dfloat_pair", "f32pair"])
def test_upwinding_entropy(pc, ic, orc, mode):
    kw = dict(MODES[mode])
    if mode == "f64":
        kw["tile"] = 2   # the 8-field FP64 default
    p = _params(pc, lentropy=1, **kw)
    f0 = _initial(pc, ic, p, seed=5)
    f0[..., 4] *= 0.1   # ss
    box = pc.Box(p)
    box.load(f0)
    box.steps(6)
    ref, _ = _oracle(orc, p, f0, 6)
    _check(box.store(), ref, p, mode)


@pytest.mark.parametrize("flags", [(1, 0), (0, 1)])
def test_upwinding_flags_separately(pc, ic, orc, flags):
    p = _params(pc, lupw_uu=flags[0], lupw_lnrho=flags[1])
    f0 = _initial(pc, ic, p, seed=9)
    box = pc.Box(p)
    box.load(f0)
    box.steps(5)
    ref, _ = _oracle(orc, p, f0, 5)
    _check(box.store(), ref, p, "f64")
    # and the correction is not negligible: the run without it differs
    q = _params(pc, lupw_uu=0, lupw_lnrho=0)
    plain, _ = _oracle(orc, q, f0, 5)
    k = 0 if flags[0] else 3
    assert np.max(np.abs(plain[..., k] - ref[..., k])) > 1e-6


def test_upwinding_without_variant_is_refused(pc):
    p = _params(pc, precision=4, comp=1, tile=0)   # FP32 field-major (32,4): no upwinding variant
    with pytest.raises(pc.PcgbError):
        pc.Box(p)


def test_reload_switches_kernel_variant(pc, ic, orc):
    """reloadConfig turning upwinding on changes the kernel, not only the parameters."""
    gpu = importlib.import_module("pencil-code_gb300.gpu")
    p0 = _params(pc, lupw_uu=0, lupw_lnrho=0)
    f0 = _initial(pc, ic, p0, seed=11)
    f = np.array(f0, order="F", copy=True)
    gpu.initialize_gpu(f, p0, t=0.0, nt=1)
    p1 = _params(pc)
    gpu.reload_gpu_config(p1)
    gpu.time_step(3)
    gpu.copy_farray_from_gpu(f)
    gpu.finalize_gpu()
    ref, _ = _oracle(orc, p1, f0, 3)
    _check(f, ref, p1, "f64")


def test_reload_switches_default_fp32_tile(pc, ic, orc):
    """An FP32 box large enough for the default 12-warp tile (which has no upwinding variant),
    created without upwinding: reloadConfig turning upwinding on moves it to the default tile
    of the new physics, and the steps match the oracle."""
    gpu = importlib.import_module("pencil-code_gb300.gpu")
    n = (512, 80, 8)   # 16 x 10 column tiles of (32,8): the default FP32 tile is then tile 7
    p0 = _params(pc, n=n, precision=4, comp=1, lupw_uu=0, lupw_lnrho=0)
    f0 = 0.01 * _initial(pc, ic, p0, seed=12)   # grid noise of 5e-4, so that B = curl A stays O(0.1) at dx = 2 pi / 512
    f = np.array(f0, order="F", copy=True)   # the REAL=double library; the device state is FP32
    gpu.initialize_gpu(f, p0, t=0.0, nt=1)
    p1 = _params(pc, n=n, precision=4, comp=1)
    gpu.reload_gpu_config(p1)
    gpu.time_step(3)
    gpu.copy_farray_from_gpu(f)
    gpu.finalize_gpu()
    ref, _ = _oracle(orc, p1, f0, 3)
    _check(f, ref, p1, "f32pair")


def _timing_kvectors():
    """A small shell of the forcing wavevectors (|k|^2 in [5, 6]), ordered as k.dat lists them."""
    nl = importlib.import_module("pencil-code_gb300.namelist")
    return nl.kvector_shell(5, 6)


@pytest.mark.parametrize("mode", ["f64", "dfloat_pair", "f32pair", "f32"])
def test_magnetic_helical_forcing_with_upwinding(pc, ic, orc, mode):
    """The doc/timings physics (lupw_uu, lupw_lnrho, iforce='helical' with
    lmagnetic_forcing, relhel=1) on a small box: the force goes into aa, the
    stream advances two records per step."""
    kvec, kav = _timing_kvectors()
    p = _params(pc, n=(16, 16, 16), nu=2e-5, eta=2e-5, lforcing_hel=1, force_hel=0.05, relhel=1.0,
                lmagnetic_forcing=1, seed_ff=1812, **MODES[mode])
    # noise of amplitude 1e-2 in every field: from zero fields the velocity would
    # only be the Lorentz force's, orders of magnitude below aa, and an FP32
    # relative bar on it would measure the rounding of aa's derivatives instead
    f0 = _initial(pc, ic, p, seed=17)
    f0 *= 0.2
    box = pc.Box(p)
    box.set_kvectors(kvec, kav)
    box.load(f0)
    box.steps(8)
    g = box.store()
    ref, _ = _oracle(orc, p, f0, 8, kvec, kav)
    q = type(p).from_buffer_copy(p).update(lforcing_hel=0, lmagnetic_forcing=0)
    unforced, _ = _oracle(orc, q, f0, 8)
    assert np.max(np.abs(ref[..., 4:7] - unforced[..., 4:7])) > 1e-3   # aa forced
    _check(g, ref, p, mode)


def test_upwinding_through_noalloc_entry(pc, ic, orc):
    """pcgb_substep_noalloc takes the upwinding variant of its tile: three
    substeps in a row against one oracle step."""
    torch = pytest.importorskip("torch")
    from test_zz_no_alloc import from_device_layout, to_device_layout
    L = pc.load()
    p = _params(pc)
    f0 = _initial(pc, ic, p, seed=13)
    xoff = 128 // 8
    px = xoff + ((p.nx + 8 + xoff - 1) // xoff) * xoff
    a = torch.from_numpy(to_device_layout(f0, xoff, px)).cuda()
    b = torch.zeros_like(a)
    df = torch.zeros_like(a)
    bufs = [a, b]
    for s in range(3):
        src, dst = bufs[s % 2], bufs[(s + 1) % 2]
        rc = L.pcgb_substep_noalloc(C.byref(p), s + 1, p.dt, C.c_void_p(src.data_ptr()), C.c_void_p(dst.data_ptr()),
                                    C.c_void_p(df.data_ptr()), None, None)
        assert rc == 0
    torch.cuda.synchronize()
    g = from_device_layout(bufs[1].cpu().numpy(), xoff, p.nx + 6)
    ref, _ = _oracle(orc, p, f0, 1)
    _check(g, ref, p, "f64")


@pytest.mark.parametrize("prec", [4, 8])
def test_upwinding_batch_equals_single(pc, ic, prec):
    """Boxes with upwinding in one persistent batched launch give each box's result alone."""
    sizes = [(24, 20, 16), (16, 16, 16), (32, 24, 8)]
    kw = dict(precision=prec, comp=1) if prec == 4 else dict(precision=8)
    alone, boxes = [], []
    for i, n in enumerate(sizes):
        p = _params(pc, n=n, nu=2e-3 * (i + 1), **kw)
        f0 = _initial(pc, ic, p, seed=30 + i)
        b = pc.Box(p)
        b.load(f0)
        b.steps(4)
        alone.append(b.store())
        b.close()
        b = pc.Box(p)
        b.load(f0)
        boxes.append(b)
    batch = pc.Batch(boxes)
    batch.steps(4, use_graph=True, graph_steps=2)
    for b, ref in zip(boxes, alone):
        assert np.array_equal(b.store(), ref)
    batch.close()
