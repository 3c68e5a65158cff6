"""Random helical forcing (iforce='helical') on the GPU against the oracle.

The device applies, after every step, the force of the record the host drew
for that step (same ran0 stream and fconst_coefs_hel restatement as the
oracle), scaled by the device's dt of the step.  Parity bars as elsewhere:
FP64 and double-float 1e-11, FP32 1e-5 (lnrho against max(|lnrho|, 1)).
"""
import ctypes as C
import importlib
import json
import os

import numpy as np
import pytest

from conftest import LOG7, oracle_params, rel_err

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def _fixture():
    with open(os.path.join(HERE, "golden", "helical_mhdturb_ref.json")) as fh:
        d = json.load(fh)
    kd = d["kdat"]
    return d, np.array(kd["kxyz"]).reshape(3, kd["nk"]), kd["kav"]


def _params(pc, d, **kw):
    prm = d["params"]
    n = prm["n"]
    p = pc.default_params(nx=n, ny=n, nz=n, gamma=prm["gamma"], nu=prm["nu"], eta=prm["eta"], relhel=prm["relhel"],
                          kf=1.0, cdt=prm["cdt"], cdtv=prm["cdtv"], dt=prm["dt"], lforcing_hel=1,
                          force_hel=prm["force"], seed_ff=1812, precision=8)
    return p.update(**kw)


def _initial(pc, p):
    f = np.zeros(pc.host_shape(p), order="F")
    n = p.nx
    f[3:-3, 3:-3, 3:-3, 4:7] = 1e-4 * np.random.Generator(np.random.PCG64(1)).standard_normal((n, n, n, 3))
    return f


def _oracle_run(orc, p, f0, kvec, kav, nsteps, ldt=False):
    op = oracle_params(orc, p)
    f = np.array(f0, order="F", copy=True)
    orc.ghosts(op, f)
    df = np.zeros_like(f)
    state, t, dt = p.seed_ff, 0.0, (0.0 if ldt else p.dt)
    for _ in range(nsteps):
        rec, state = orc.helical_coefs(op, p.force_hel, kvec, kav, state)
        t, dt, _ = orc.time_step(op, f, df, t, dt, ldt, nthreads=8)
        orc.add_helical(op, f, rec, dt)
        orc.ghosts(op, f)
    return f, t


@pytest.mark.parametrize("mode", ["f64", "dfloat", "dfloat_pair", "f32pair", "f32pair7", "f32"])
def test_helical_forcing_matches_oracle(pc, orc, mode):
    d, kvec, kav = _fixture()
    kw = dict(f64=dict(), dfloat=dict(dfloat=1, tile=0), dfloat_pair=dict(dfloat=1, tile=5),
              f32pair=dict(precision=4, comp=1, tile=5), f32pair7=dict(precision=4, comp=1, tile=7),
              f32=dict(precision=4, comp=1, tile=0))[mode]
    p = _params(pc, d, **kw)
    f0 = _initial(pc, p)
    box = pc.Box(p)
    box.set_kvectors(kvec, kav)
    box.load(f0)
    box.steps(10)
    g = box.store()
    ref, t_ref = _oracle_run(orc, p, f0, kvec, kav, 10)
    if mode.startswith("f32"):
        assert np.all(rel_err(g, ref, LOG7) <= 1e-5)
    else:
        assert np.all(rel_err(g, ref) <= 1e-11)
    assert abs(box.time()[0] - t_ref) <= 1e-12
    assert np.array_equal(g, _ghosted(pc, g))


def _ghosted(pc, g):
    ic = importlib.import_module("pencil-code_gb300.initcond")
    return ic.fill_ghosts(g.copy())


def test_helical_forcing_urms_against_reference_series(pc):
    """urms after 2 and 4 steps of samples/helical-MHDturb (one normalised mode per step)."""
    d, kvec, kav = _fixture()
    p = _params(pc, d)
    box = pc.Box(p)
    box.set_kvectors(kvec, kav)
    box.load(_initial(pc, p))
    ref = {r["it"]: r for r in d["series"]}
    for it in (2, 4):
        box.steps(2)
        u = box.store()[3:-3, 3:-3, 3:-3, 0:3]
        urms = np.sqrt((u ** 2).sum(-1).mean())
        assert abs(urms - ref[it]["urms"]) <= 5e-4 * ref[it]["urms"] + 1e-5, (it, urms)


def test_helical_forcing_with_cfl_dt(pc, orc):
    """The force scales with the dt of the step it closes (CFL dt of the current f)."""
    d, kvec, kav = _fixture()
    p = _params(pc, d, dt=0.0, dt_mode=2)
    f0 = _initial(pc, p)
    box = pc.Box(p)
    box.set_kvectors(kvec, kav)
    box.load(f0)
    box.steps(6)
    ref, t_ref = _oracle_run(orc, p, f0, kvec, kav, 6, ldt=True)
    assert np.all(rel_err(box.store(), ref) <= 1e-11)
    assert abs(box.time()[0] - t_ref) <= 1e-12 * t_ref


def test_helical_forcing_plugin_and_refusals(pc, orc):
    d, kvec, kav = _fixture()
    p = _params(pc, d)
    L = pc.load()
    gpu = importlib.import_module("pencil-code_gb300.gpu")
    f0 = _initial(pc, p)
    kv = np.ascontiguousarray(kvec)
    assert L.pcgb_set_kvectors(kv.ctypes.data_as(C.POINTER(C.c_double)), kv.shape[1], kav) == 0
    f = np.array(f0, order="F", copy=True)
    gpu.initialize_gpu(f, p, t=0.0, nt=1)
    gpu.time_step(3)
    gpu.copy_farray_from_gpu(f)
    gpu.finalize_gpu()
    ref, _ = _oracle_run(orc, p, f0, kvec, kav, 3)
    assert np.all(rel_err(f, ref) <= 1e-11)
    # a box without wavevectors cannot step; a batch does not take helical boxes
    box = pc.Box(p)
    box.load(f0)
    with pytest.raises(pc.PcgbError):
        box.steps(1)
    box2 = pc.Box(p)
    box2.set_kvectors(kvec, kav)
    with pytest.raises(pc.PcgbError):
        pc.Batch([box2])
