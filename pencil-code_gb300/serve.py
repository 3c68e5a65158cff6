"""Serving: a Poisson request stream against the native continuous-batching
server (pcgb_server_*), and the same stream served FIFO one at a time.

Request mix: box size from {32,64,128,256}^3 with weights 0.4/0.3/0.2/0.1,
isothermal (7 fields) or entropy (8 fields) with p = 0.5, FP32 or FP64 flag,
steps uniform in [100, 2000] (times ``steps_scale``), nu/eta/forcing drawn as
in the ensemble workload, seeded initial noise; device-memory admission budget
150 GB by default.  FP64 requests run with the double-float state by default
(``fp64_dfloat``): the same parity bar against the FP64 oracle as native FP64
at about twice its rate on this GPU.
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np

from .lib import NSLOT, PcgbError, default_params, load

SIZES = (32, 64, 128, 256)
WEIGHTS = (0.4, 0.3, 0.2, 0.1)


def draw_requests(n: int, seed: int = 0, steps_scale: float = 1.0, fp64_fraction: float = 0.5,
                  sizes=SIZES, weights=WEIGHTS, fp64_dfloat: bool = True):
    rng = np.random.Generator(np.random.PCG64(seed))
    reqs = []
    for i in range(n):
        size = int(rng.choice(sizes, p=weights))
        ent = bool(rng.random() < 0.5)
        prec = 8 if rng.random() < fp64_fraction else 4
        steps = max(1, int(round(rng.integers(100, 2001) * steps_scale)))
        nu = float(np.exp(rng.uniform(np.log(1e-3), np.log(1e-2))))
        eta = float(np.exp(rng.uniform(np.log(1e-3), np.log(1e-2))))
        amp = float(rng.uniform(0.01, 0.05))
        k = float(rng.choice([1, 2, 3]))
        p = default_params(nx=size, ny=size, nz=size, lentropy=int(ent), gamma=5.0 / 3.0 if ent else 1.0,
                           precision=prec, comp=1, nu=nu, eta=eta, chi=nu if ent else 0.0, lforcing_cont=1,
                           ampl_ff=amp, kf=k, dt=0.0, dt_mode=1, cdt=0.4,
                           dfloat=int(prec == 8 and fp64_dfloat))
        reqs.append(dict(p=p, steps=steps, seed=5000 + i))
    return reqs


class Server:
    def __init__(self, budget_bytes: float = 150e9, max_active: int = 1 << 20, round_steps: int = 10):
        self.L = load()
        self.h = self.L.pcgb_server_create(C.c_size_t(int(budget_bytes)), int(max_active), int(round_steps))
        if not self.h:
            raise PcgbError("pcgb_server_create failed")

    def submit(self, p, steps: int, seed: int, noise: float = 1e-5, abc: float = 0.0, f_out=None) -> int:
        ptr = None if f_out is None else f_out.ctypes.data_as(C.c_void_p)
        rid = self.L.pcgb_server_submit(self.h, C.byref(p), int(steps), int(seed), noise, abc, ptr)
        if rid < 0:
            raise PcgbError("pcgb_server_submit rejected the request")
        return rid

    def poll(self, rid: int):
        times = np.zeros(3)
        diag = np.zeros(NSLOT + 3)
        rc = self.L.pcgb_server_poll(self.h, rid, times.ctypes.data_as(C.POINTER(C.c_double)),
                                     diag.ctypes.data_as(C.POINTER(C.c_double)))
        return rc, times, diag

    def drain(self, timeout: float = 3600.0) -> bool:
        return self.L.pcgb_server_drain(self.h, timeout) == 0

    def stats(self) -> dict:
        st = np.zeros(6)
        self.L.pcgb_server_stats(self.h, st.ctypes.data_as(C.POINTER(C.c_double)), 6)
        return dict(zip(["submitted", "completed", "active", "peak_active", "peak_bytes", "rounds"], st.tolist()))

    def close(self):
        if self.h:
            self.L.pcgb_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def run_stream(reqs, rate: float, seed: int = 0, max_active: int = 1 << 20, budget: float = 150e9,
               round_steps: int = 10, timeout: float = 3600.0) -> dict:
    """Submit reqs at Poisson arrival times (rate per second); return latency statistics."""
    rng = np.random.Generator(np.random.PCG64(seed + 17))
    gaps = rng.exponential(1.0 / rate, size=len(reqs))
    srv = Server(budget, max_active, round_steps)
    t0 = time.perf_counter()
    arrive = np.cumsum(gaps) - gaps[0]
    ids = []
    for r, ta in zip(reqs, arrive):
        dt = ta - (time.perf_counter() - t0)
        if dt > 0:
            time.sleep(dt)
        ids.append(srv.submit(r["p"], r["steps"], r["seed"]))
    ok = srv.drain(timeout)
    wall = time.perf_counter() - t0
    lat, failed = [], 0
    first_submit, last_finish = None, None
    for rid in ids:
        rc, times, _ = srv.poll(rid)
        if rc == 1:
            lat.append(times[2] - times[0])
            first_submit = times[0] if first_submit is None else min(first_submit, times[0])
            last_finish = times[2] if last_finish is None else max(last_finish, times[2])
        else:
            failed += 1
    st = srv.stats()
    srv.close()
    lat = np.array(lat)
    span = (last_finish - first_submit) if lat.size else float("nan")
    return dict(requests=len(reqs), completed=int(lat.size), failed=failed, drained=ok, rate=rate,
                solves_per_s=lat.size / span if lat.size else 0.0,
                p50_s=float(np.percentile(lat, 50)) if lat.size else None,
                p99_s=float(np.percentile(lat, 99)) if lat.size else None,
                mean_s=float(lat.mean()) if lat.size else None, makespan_s=span, wall_s=wall,
                peak_active=st["peak_active"], peak_gb=st["peak_bytes"] / 1e9, rounds=st["rounds"])
