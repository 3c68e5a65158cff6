"""Batched persistent launches: each box gives bitwise the same result alone
and inside a batch of uneven boxes, with and without CUDA-graph replay."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def make(pc, ic, n, seed, prec=4, nu=3e-3, amp=0.03, k=2.0, dt=2e-3):
    p = pc.default_params(nx=n, ny=n, nz=n, gamma=1.0, nu=nu, eta=1.5 * nu, dt=dt, precision=prec, comp=1,
                          lforcing_cont=1, ampl_ff=amp, kf=k, tile=2 if prec == 4 else 1, zdepth=16)
    f = ic.zeros(p)
    ic.gaussian_noise(f, p, ["ax", "ay", "az"], 1e-5, seed)
    return p, f


@pytest.mark.parametrize("prec", [4, 8])
def test_batch_equals_single(pc, ic, prec):
    sizes = [32, 48, 64, 16, 32]
    singles = []
    for i, n in enumerate(sizes):
        p, f = make(pc, ic, n, 100 + i, prec, nu=1e-3 * (i + 1), amp=0.01 * (i + 1), k=1 + i % 3)
        b = pc.Box(p)
        b.load(f)
        b.steps(7)
        singles.append(b.store())
        b.close()
    boxes = []
    for i, n in enumerate(sizes):
        p, f = make(pc, ic, n, 100 + i, prec, nu=1e-3 * (i + 1), amp=0.01 * (i + 1), k=1 + i % 3)
        b = pc.Box(p)
        b.load(f)
        boxes.append(b)
    batch = pc.Batch(boxes, persistent=True)
    batch.steps(7, use_graph=True, graph_steps=3)    # 2 graph replays + 1 eager step
    for b, ref in zip(boxes, singles):
        assert np.array_equal(b.store(), ref)
        t, dt, nsub = b.time()
        assert nsub == 21


def test_batch_cfl_per_box(pc, ic):
    """Per-box CFL dt (lagged) inside one batch equals each box's own run."""
    res = []
    for mode in ("single", "batch"):
        boxes = []
        for i, n in enumerate([32, 16, 48]):
            p = pc.default_params(nx=n, ny=n, nz=n, gamma=1.0, nu=2e-3 * (i + 1), eta=2e-3, dt=0.0, dt_mode=1,
                                  cdt=0.4, precision=4, tile=2, zdepth=16)
            f = ic.zeros(p)
            ic.gaussian_noise(f, p, ["ux", "uy", "uz", "ax", "ay", "az"], 1e-2, 7 + i)
            b = pc.Box(p)
            b.load(f)
            boxes.append(b)
        if mode == "single":
            for b in boxes:
                b.steps(5)
        else:
            pc.Batch(boxes).steps(5, use_graph=False)
        res.append([(b.store(), b.time()) for b in boxes])
    for (fa, ta), (fb, tb) in zip(*res):
        assert np.array_equal(fa, fb) and ta == tb


@pytest.mark.parametrize("tile", [5, 7])
def test_tensor_memory_tile_batch_with_zdepth_per_box(pc, ic, tile):
    """FP32 pair tiles 5 and 7 (z data in tensor memory) in one persistent launch over boxes of
    uneven sizes, each with its own z-sweep depth and a ragged tiling (a CTA primes the
    tensor-memory ring at the start of every tile it pulls): bitwise the same as each box
    stepped alone with the same depth, with lagged CFL dt and diagnostics; the fields are
    also bitwise those of the box's default depth (the per-tile diagnostic partial sums
    then group differently, so the diagnostics agree to FP64 round-off)."""
    shapes = [(32, 32, 32, 16), (48, 40, 24, 8), (37, 19, 11, 0), (64, 16, 40, 40), (24, 24, 24, 24)]

    def mk(i, n, zd):
        p = pc.default_params(nx=n[0], ny=n[1], nz=n[2], gamma=1.0, nu=2e-3 * (i + 1), eta=3e-3, dt=0.0,
                              dt_mode=1, cdt=0.4, precision=4, comp=1, lforcing_cont=1, ampl_ff=0.02, kf=1.0 + i % 2,
                              diag_every=2, tile=tile, zdepth=zd)
        f = ic.zeros(p)
        ic.gaussian_noise(f, p, ["ux", "uy", "uz", "ax", "ay", "az"], 1e-2, 50 + i)
        return p, f

    singles, defaults = [], []
    for i, s in enumerate(shapes):
        for zd, out in ((s[3], singles), (0, defaults)):
            p, f = mk(i, s[:3], zd)
            b = pc.Box(p)
            b.load(f)
            b.steps(6)
            out.append((b.store(), b.time(), b.diag_raw()))
            b.close()
    boxes = []
    for i, s in enumerate(shapes):
        p, f = mk(i, s[:3], s[3])
        b = pc.Box(p)
        b.load(f)
        boxes.append(b)
    batch = pc.Batch(boxes, persistent=True)
    batch.steps(6, use_graph=True, graph_steps=2)
    for b, (fs, ts, ds), (fd, td, dd) in zip(boxes, singles, defaults):
        g = b.store()
        assert np.array_equal(g, fs) and np.array_equal(g, fd)
        assert b.time() == ts == td
        assert np.array_equal(b.diag_raw(), ds)
        keep = np.arange(ds.size) != 7          # slot 7: sum of (div B)^2, pure round-off
        assert np.allclose(ds[keep], dd[keep], rtol=1e-12, atol=0.0)
        assert dd[7] <= 1e-10 * dd[8]
