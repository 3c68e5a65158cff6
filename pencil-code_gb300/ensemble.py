"""Batched ensembles of independent boxes (uneven sizes and parameters).

``make_ensemble`` draws the ensemble workload: box sizes uniform from
{32,48,64,96,128}^3, nu and eta log-uniform in [1e-3, 1e-2], continuous ABC
forcing with amplitude uniform in [0.01, 0.05] at k in {1,2,3}, aa noise 1e-5,
uu = lnrho = 0, per-box CFL timestep with cdt = 0.4, FP32 state with FP64
reductions.  ``run_batched`` advances all boxes in persistent launches with
the substep loop captured in a CUDA graph; ``run_plain`` advances them one box
at a time with the single-box kernel.
"""
from __future__ import annotations

import numpy as np

from .lib import Batch, Box, default_params, load

SIZES = (32, 48, 64, 96, 128)


def make_ensemble(nboxes: int = 192, seed: int = 0, precision: int = 4, tile: int = -1, zdepth: int = 0):
    rng = np.random.Generator(np.random.PCG64(seed))
    specs = []
    for i in range(nboxes):
        n = int(rng.choice(SIZES))
        nu = float(np.exp(rng.uniform(np.log(1e-3), np.log(1e-2))))
        eta = float(np.exp(rng.uniform(np.log(1e-3), np.log(1e-2))))
        amp = float(rng.uniform(0.01, 0.05))
        k = float(rng.choice([1, 2, 3]))
        p = default_params(nx=n, ny=n, nz=n, gamma=1.0, precision=precision, comp=1, nu=nu, eta=eta,
                           lforcing_cont=1, ampl_ff=amp, kf=k, dt=0.0, dt_mode=1, cdt=0.4, tile=tile, zdepth=zdepth)
        specs.append((p, 1000 + i))
    return specs


def init_box(box: Box, p, seed: int, noise: float = 1e-5):
    iax = 5 if p.lentropy else 4
    for k in range(iax + 3):
        box.init_field(k, "zero")
    for k in range(3):
        box.init_field(iax + k, "noise", ampl=noise, seed=seed * 8 + k)


def build_boxes(specs):
    boxes = []
    for p, seed in specs:
        b = Box(p)
        init_box(b, p, seed)
        boxes.append(b)
    return boxes


def run_batched(boxes, steps: int, graph_steps: int = 10):
    batch = Batch(boxes, persistent=True)
    batch.steps(steps, use_graph=True, graph_steps=graph_steps)
    boxes[0].sync()
    return batch


def run_plain(boxes, steps: int):
    for b in boxes:
        b.steps(steps)
    boxes[0].sync()


def _time_batch(specs, tile, zd_of, steps):
    """ms per RK3 step of the given boxes in one persistent batched launch per substep."""
    import torch
    boxes = []
    for p, seed in specs:
        q = default_params()
        q.update(**p.as_dict())
        q.tile, q.zdepth = tile, zd_of(q.nx)
        b = Box(q)
        init_box(b, q, seed)
        boxes.append(b)
    batch = Batch(boxes, persistent=True)
    batch.steps(1, use_graph=False)
    torch.cuda.synchronize()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    stream = torch.cuda.ExternalStream(load().pcgb_get_stream())
    t0.record(stream)
    batch.steps(steps, use_graph=False)
    t1.record(stream)
    torch.cuda.synchronize()
    batch.close()
    for b in boxes:
        b.close()
    return t0.elapsed_time(t1) / steps


def autotune_batch(specs, tiles=(4, 5, 6, 7), zdepths=(16, 32, 64), steps: int = 3, sample: int = 24,
                   per_size_zdepths=(8, 16, 32, 64, 128), per_size_sample: int = 8):
    """Pick the tile variant of the batched launch and the z-sweep depth of every box size.

    Stage 1 times the tile variants (with one z-depth for all boxes) on a sample of the
    ensemble that holds every size; stage 2 keeps the best tile and times, size by size,
    batches of that size's boxes at each z-depth up to the box height.  A launch carries
    one tile shape (the kernel is compiled per shape); z-depths are per box.
    Returns (tile, {size: zdepth}, table of ms per step)."""
    by_size = {}
    for p, seed in specs:
        by_size.setdefault(p.nx, []).append((p, seed))
    pick = []
    i = 0
    while len(pick) < min(sample, len(specs)):
        for n in sorted(by_size):
            lst = by_size[n]
            if i < len(lst) and len(pick) < sample:
                pick.append(lst[i])
        i += 1
    table = {}
    for tile in tiles:
        for zd in zdepths:
            table[(tile, zd)] = _time_batch(pick, tile, lambda n, zd=zd: zd, steps)
    best_tile, best_zd = min(table, key=table.get)
    zd_by_size = {}
    for n, lst in sorted(by_size.items()):
        group = lst[:per_size_sample]
        cands = [z for z in per_size_zdepths if z <= n] or [n]
        times = {z: _time_batch(group, best_tile, lambda m, z=z: z, steps) for z in cands}
        for z, ms in times.items():
            table[(best_tile, f"{n}^3 zd {z}")] = ms
        zd_by_size[n] = min(times, key=times.get)
    return best_tile, zd_by_size, table


def with_tiling(specs, tile: int, zdepth):
    """Copies of specs with the tile variant and the z-depth (an int, or {size: zdepth})."""
    out = []
    for p, seed in specs:
        q = default_params()
        q.update(**p.as_dict())
        q.tile = tile
        q.zdepth = zdepth.get(q.nx, 0) if isinstance(zdepth, dict) else zdepth
        out.append((q, seed))
    return out
