"""Continuous-batching server: every request's result is the same served in
a mix of uneven requests as computed alone (bitwise: a box's arithmetic does
not depend on what else shares the launch), and admission respects the
device-memory budget."""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _req(pc, n, prec, ent, seed, nu, k):
    """prec: 4 FP32, 8 FP64, 9 FP64-class double-float."""
    p = pc.default_params(nx=n, ny=n, nz=n, lentropy=int(ent), gamma=5.0 / 3.0 if ent else 1.0,
                          precision=4 if prec == 4 else 8, dfloat=int(prec == 9),
                          comp=1, nu=nu, eta=1.3 * nu, chi=nu if ent else 0.0, lforcing_cont=1, ampl_ff=0.03, kf=k,
                          dt=0.0, dt_mode=1, cdt=0.4)
    return p


def _request_tiling(q):
    """The server's tiling of a request that names none (request_tiling in csrc/server.cu)."""
    if q.precision == 4:
        px = 16 + (q.nx + 8 + 15) // 16 * 16
        ps = px * (q.ny + 6)
        big = ((q.nx + 31) // 32) * ((q.ny + 7) // 8) >= 152 and not (q.lupw_uu or q.lupw_lnrho)
        q.tile = 7 if big and 2 * ps * (q.nz + 6) + 8 * ps < (1 << 32) else 6
    else:
        q.tile = 5 if q.dfloat else 1
    q.zdepth = min(64, max(16, q.nz // 4))


def _alone(pc, ens, p, steps, seed):
    q = pc.default_params()
    q.update(**p.as_dict())
    _request_tiling(q)
    b = pc.Box(q)
    ens.init_box(b, q, seed)
    b.steps(steps)
    return b.store()


def test_mix_equals_alone(pc):
    serve = importlib.import_module("pencil-code_gb300.serve")
    ens = importlib.import_module("pencil-code_gb300.ensemble")
    specs = [(32, 4, False, 11, 2e-3, 1.0, 7), (48, 8, False, 12, 5e-3, 2.0, 5), (32, 4, True, 13, 3e-3, 3.0, 9),
             (64, 4, False, 14, 1e-3, 2.0, 4), (16, 8, True, 15, 8e-3, 1.0, 6), (40, 4, False, 16, 4e-3, 1.0, 8),
             (32, 9, False, 17, 2e-3, 2.0, 5), (24, 9, True, 18, 6e-3, 1.0, 7)]
    srv = serve.Server(budget_bytes=20e9, round_steps=3)
    outs, ids = [], []
    for n, prec, ent, seed, nu, k, steps in specs:
        p = _req(pc, n, prec, ent, seed, nu, k)
        f = np.zeros(pc.host_shape(p), order="F")
        outs.append(f)
        ids.append(srv.submit(p, steps, seed, noise=1e-5, f_out=f))
    assert srv.drain(600)
    st = srv.stats()
    for rid in ids:
        rc, times, _ = srv.poll(rid)
        assert rc == 1 and times[0] <= times[1] <= times[2]
    srv.close()
    assert st["peak_active"] >= 2
    for (n, prec, ent, seed, nu, k, steps), f in zip(specs, outs):
        ref = _alone(pc, ens, _req(pc, n, prec, ent, seed, nu, k), steps, seed)
        assert np.array_equal(f, ref), (n, prec, ent)


def test_compensated_and_plain_fp32_in_the_mix(pc):
    """FP32 requests with and without the compensated state (each its own class: the
    compensated one runs kernels compiled per substep) served together: every result
    equals the box alone, bitwise."""
    serve = importlib.import_module("pencil-code_gb300.serve")
    ens = importlib.import_module("pencil-code_gb300.ensemble")
    specs = [(32, 31, 2e-3, 1.0, 6, 1), (32, 32, 3e-3, 2.0, 6, 0), (24, 33, 5e-3, 1.0, 5, 0), (40, 34, 2e-3, 3.0, 4, 1)]
    srv = serve.Server(budget_bytes=20e9, round_steps=2)
    outs, ids = [], []
    for n, seed, nu, k, steps, comp in specs:
        p = _req(pc, n, 4, False, seed, nu, k).update(comp=comp)
        f = np.zeros(pc.host_shape(p), order="F")
        outs.append(f)
        ids.append(srv.submit(p, steps, seed, noise=1e-5, f_out=f))
    assert srv.drain(600)
    assert all(srv.poll(i)[0] == 1 for i in ids)
    srv.close()
    for (n, seed, nu, k, steps, comp), f in zip(specs, outs):
        ref = _alone(pc, ens, _req(pc, n, 4, False, seed, nu, k).update(comp=comp), steps, seed)
        assert np.array_equal(f, ref), (n, comp)


def test_admission_budget_and_fifo(pc):
    serve = importlib.import_module("pencil-code_gb300.serve")
    L = pc.load()
    reqs = [_req(pc, 32, 4, False, s, 2e-3, 1.0) for s in range(4)]
    one = L.pcgb_params_bytes(__import__("ctypes").byref(reqs[0]))
    for max_active, budget, lo, hi in ((1 << 20, 1.5 * one, 1, 1), (1, 100 * one, 1, 1), (1 << 20, 100 * one, 2, 4)):
        srv = serve.Server(budget_bytes=budget, max_active=max_active, round_steps=2)
        ids = [srv.submit(p, 40, 100 + i) for i, p in enumerate(reqs)]
        assert srv.drain(300)
        assert all(srv.poll(i)[0] == 1 for i in ids)
        st = srv.stats()
        srv.close()
        # requests that arrive while a round runs join at the next round boundary
        assert lo <= st["peak_active"] <= hi and st["peak_bytes"] <= budget


def test_upwinding_requests_in_the_mix(pc):
    """Requests with upwinded advection (their own kernel variant, so their own class in
    the batched launch) served together with plain ones: each result equals the box alone.
    Requests the batched launch cannot take (helical forcing, non-periodic boundaries)
    are refused at submission."""
    serve = importlib.import_module("pencil-code_gb300.serve")
    ens = importlib.import_module("pencil-code_gb300.ensemble")
    specs = [(32, 4, False, 21, 2e-3, 1.0, 6, 1), (32, 4, False, 22, 3e-3, 2.0, 6, 0), (24, 8, False, 23, 5e-3, 1.0, 5, 1),
             (24, 8, True, 24, 4e-3, 2.0, 5, 1), (16, 9, False, 25, 6e-3, 1.0, 7, 1), (40, 4, True, 26, 2e-3, 1.0, 4, 1)]

    def req(n, prec, ent, seed, nu, k, upw):
        return _req(pc, n, prec, ent, seed, nu, k).update(lupw_uu=upw, lupw_lnrho=upw)

    srv = serve.Server(budget_bytes=20e9, round_steps=2)
    outs, ids = [], []
    for n, prec, ent, seed, nu, k, steps, upw in specs:
        p = req(n, prec, ent, seed, nu, k, upw)
        f = np.zeros(pc.host_shape(p), order="F")
        outs.append(f)
        ids.append(srv.submit(p, steps, seed, noise=1e-5, f_out=f))
    with pytest.raises(pc.PcgbError):
        srv.submit(req(16, 4, False, 30, 2e-3, 1.0, 0).update(lforcing_hel=1, force_hel=0.05), 3, 30)
    with pytest.raises(pc.PcgbError):
        srv.submit(req(16, 4, False, 31, 2e-3, 1.0, 0).update(bcz=["s"] * 7), 3, 31)
    assert srv.drain(600)
    assert all(srv.poll(rid)[0] == 1 for rid in ids)
    srv.close()
    for (n, prec, ent, seed, nu, k, steps, upw), f in zip(specs, outs):
        ref = _alone(pc, ens, req(n, prec, ent, seed, nu, k, upw), steps, seed)
        assert np.array_equal(f, ref), (n, prec, ent, upw)


def test_failing_request_fails_alone(pc):
    """A request whose state turns non-finite (initial noise of infinite amplitude) fails on
    its own: the requests batched with it in the same class and rounds complete with the
    results they give alone."""
    serve = importlib.import_module("pencil-code_gb300.serve")
    ens = importlib.import_module("pencil-code_gb300.ensemble")
    specs = [(32, 4, False, 21, 2e-3, 1.0, 9), (32, 4, False, 22, 3e-3, 2.0, 9), (24, 4, False, 23, 4e-3, 1.0, 9)]
    srv = serve.Server(budget_bytes=20e9, round_steps=3)
    outs, ids = [], []
    for i, (n, prec, ent, seed, nu, k, steps) in enumerate(specs):
        p = _req(pc, n, prec, ent, seed, nu, k)
        f = np.zeros(pc.host_shape(p), order="F")
        outs.append(f)
        ids.append(srv.submit(p, steps, seed, noise=float("inf") if i == 1 else 1e-5, f_out=f))
    assert srv.drain(600)
    rcs = [srv.poll(rid)[0] for rid in ids]
    srv.close()
    assert rcs == [1, -1, 1], rcs
    for i in (0, 2):
        n, prec, ent, seed, nu, k, steps = specs[i]
        ref = _alone(pc, ens, _req(pc, n, prec, ent, seed, nu, k), steps, seed)
        assert np.array_equal(outs[i], ref)
