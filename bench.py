#!/usr/bin/env python3
"""Benchmark of the GB300 MHD timestep (Gcell-updates/s per RK substep).

Default workload (N=1): isothermal compressible MHD, 7 fields, 1024^3
periodic box L=2*pi, FP32 state with compensated 2N accumulation,
nu=eta=5e-4, steady helical ABC forcing at k=2 with amplitude 0.02, uu=0,
lnrho=0, aa Gaussian noise 1e-5 (seeded, generated on the device), fixed
dt=2e-4.  A step is one full RK3 step (3 substep kernel launches).

  value      whole-job Gcell-updates/s per substep, device-resident state,
             CUDA events on the launching stream around exactly K steps;
  e2e        the same metric through the reference plug-in C ABI
             (initializeGPU/loadFarray, substepGPU x3 + getGPUReducedVars per
             step, copyFarray) with pinned host buffers, copies inside the
             timed region;
  roofline   algorithmic HBM bytes per launch / mean launch duration of the
             substep kernel against the measured copy bandwidth;
  cpu_baseline  the FP64 oracle (C restatement of the reference Fortran) on
             all host cores over a bounded sample.

--workload timings runs the physics of the reference's own timing run
(doc/timings/N4096_32x32x32: isothermal MHD, upwinded u.grad u and
u.grad lnrho, random helical forcing of the vector potential at |k| = 60 with
force 5e-4, nu = eta = 2e-5, CFL dt with cdt = 0.9 from the current state),
single precision as that run was, zero initial fields, on an n^3 box (1024^3
by default); its us_per_pt_step is the reference's timing unit.

--impl reference runs that CPU implementation alone on the same metric.
Under torchrun with N>1 every rank advances its own replica (weak scaling).
"""
from __future__ import annotations

import argparse
import ctypes as C
import importlib
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

FALLBACK_HBM_GBS = 6800.0


def measured_peak_hbm():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def bytes_per_cell_substep(nf: int, precision: int) -> float:
    """Algorithmic HBM bytes per interior cell and substep, the roofline basis: read f,
    write f, read df, write df on every substep except the first, where alpha = 0 and df
    need not be read -- 3 nf s on substep 1 and 4 nf s on substeps 2 and 3, mean 11/3 nf s
    (s = 4 for FP32, 8 for FP64; a double-float state is FP64-sized).  Compensation carries,
    ghost re-reads and reductions are overhead, not algorithmic bytes."""
    return 11.0 / 3.0 * nf * precision


def bytes_moved_per_cell_substep(nf: int, precision: int, comp: bool) -> float:
    """What the kernel must move at least, overhead included: the FP32 compensated state
    reads and writes its df/carry slot on every substep (4 nf s); FP64 substep 3 does not
    write the dead df (mean 10/3 nf s)."""
    if precision == 4 and comp:
        return 4.0 * nf * 4
    return 10.0 / 3.0 * nf * precision


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def headline_params(pc, n: int, precision: int, lentropy: int = 0, dfloat: int = 0):
    p = pc.default_params(nx=n, ny=n, nz=n, lentropy=lentropy, precision=precision, comp=1, dfloat=dfloat,
                          gamma=1.0 if not lentropy else 5.0 / 3.0, nu=5e-4, eta=5e-4, chi=5e-4 if lentropy else 0.0,
                          dt=2e-4, lforcing_cont=1, ampl_ff=0.02, kf=2.0, relhel=1.0)
    return p


# doc/timings/N4096_32x32x32: k.dat is the shell 3577 <= |k|^2 <= 3624 (17550
# vectors) with kav = 60.0044 as that file gives it
TIMINGS_K2 = (3577, 3624)
TIMINGS_KAV = 60.0044
# the reference's published times per point and step for 1024^3 and 2048^3
# (doc/manual.tex:9527, :9537), single precision, Triolith
TIMINGS_PUBLISHED = [
    {"us_per_pt_step": 3.6e-4, "grid": 1024, "procs": 4096, "system": "Triolith", "source": "doc/manual.tex:9527"},
    {"us_per_pt_step": 1.475e-4, "grid": 2048, "procs": 8192, "system": "Triolith (kf=60 run)",
     "source": "doc/manual.tex:9537"},
]


def timings_params(pc, n: int, precision: int = 4):
    """The run parameters of doc/timings/N4096_32x32x32 (start.in, run.in) on an n^3 box."""
    return pc.default_params(nx=n, ny=n, nz=n, precision=precision, comp=1, gamma=1.0, nu=2e-5, eta=2e-5,
                             cdt=0.9, dt=0.0, dt_mode=2, lupw_uu=1, lupw_lnrho=1, lforcing_hel=1, force_hel=5e-4,
                             relhel=1.0, lmagnetic_forcing=1, seed_ff=1812)


def timings_kvectors():
    nl = importlib.import_module("pencil-code_gb300.namelist")
    kvec, _ = nl.kvector_shell(*TIMINGS_K2)
    return np.ascontiguousarray(kvec), TIMINGS_KAV


def init_headline(box, p):
    iax = 5 if p.lentropy else 4
    for k in range(iax):
        box.init_field(k, "zero")
    for k in range(3):
        box.init_field(iax + k, "zero")
        box.init_field(iax + k, "noise", ampl=1e-5, seed=20260 + k)


def time_box_steps(pc, torch, box, stream, steps: int) -> tuple[float, int]:
    L = pc.load()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    n0 = L.pcgb_launch_count()
    e0.record(stream)
    box.steps(steps)
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1), int(L.pcgb_launch_count() - n0)


def cpu_oracle_rate(n: int, steps: int, threads: int, lentropy: int = 0,
                    workload: str = "headline") -> tuple[float, float, dict]:
    """Gcell-updates/s per substep of the FP64 oracle on an n^3 sample of the workload's physics."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build()
    timings = workload == "timings"
    if timings:
        op = O.make_params(nx=n, ny=n, nz=n, gamma=1.0, nu=2e-5, eta=2e-5, cdt=0.9, lupw_uu=1, lupw_lnrho=1)
    else:
        op = O.make_params(nx=n, ny=n, nz=n, lentropy=lentropy, gamma=1.0 if not lentropy else 5.0 / 3.0,
                           nu=5e-4, eta=5e-4, chi=5e-4 if lentropy else 0.0, lforcing_cont=1, ampl_ff=0.02,
                           kf=2.0)
    f = O.empty_f(op)
    df = O.empty_f(op)
    rng = np.random.Generator(np.random.PCG64(1))
    iax = 5 if lentropy else 4
    f[3:-3, 3:-3, 3:-3, iax:iax + 3] = 1e-5 * rng.standard_normal((n, n, n, 3))
    kvec, kav = timings_kvectors() if timings else (None, None)
    state = 1812

    def step(t, dt):
        nonlocal state
        if not timings:
            t, dt, _ = O.time_step(op, f, df, t, dt, False, nthreads=threads)
            return t, dt
        rec, state = O.helical_coefs(op, 5e-4, kvec, kav, state)
        _, state = O.helical_coefs(op, 5e-4, kvec, kav, state)   # secondary record of lmhd_forcing
        t, dt, _ = O.time_step(op, f, df, t, 0.0, True, nthreads=threads)
        O.add_helical(op, f, rec, dt, 1)
        O.ghosts(op, f)
        return t, dt

    t, dt = 0.0, 2e-4
    t, dt = step(t, dt)   # warm-up (page-in, thread spin-up)
    t0 = time.perf_counter()
    for _ in range(steps):
        t, dt = step(t, dt)
    el = time.perf_counter() - t0
    return n ** 3 * 3 * steps / el / 1e9, el, {"n": n, "steps": steps}


def max_over_ranks(ms: float, device=None) -> float:
    """Slowest rank's time (the timed region ends when every replica is done)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return ms
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_value(cells_per_rank: float, steps: int, world: int, ms: float) -> float:
    """Gcell-updates/s per substep summed over all ranks (weak scaling: every rank owns a replica)."""
    return world * cells_per_rank * 3 * steps / (ms / 1e3) / 1e9


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def run_reference(args):
    ws, rank, _ = dist_setup()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    n = args.cpu_sample_n
    per = []
    for i in range(args.warmup + args.steps):
        rate, el, _ = cpu_oracle_rate(n, 1, threads, workload=args.workload)
        if i >= args.warmup:
            per.append((rate, el))
    total_cells = n ** 3 * 3 * len(per)
    total_t = sum(e for _, e in per)
    value = total_cells / total_t / 1e9
    line = {
        "impl": "reference", "metric": "Gcell-updates/s per RK substep", "value": value,
        "unit": "Gcell-updates/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total_t / len(per), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"isothermal MHD {args.n}^3 "
                               f"{'timing-run' if args.workload == 'timings' else 'headline'} physics, "
                               f"CPU sample {n}^3 per step",
                   "sample_n": n},
        "cpu_baseline": {"value": value, "unit": "Gcell-updates/s", "cores": threads, "kind": "port",
                         "sample": f"{n}^3 box, 1 RK3 step per timed step, FP64 oracle, OpenMP {threads} threads"},
        "e2e": {"value": value, "unit": "Gcell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args):
    import torch
    ws, rank, local = dist_setup()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    pc = importlib.import_module("pencil-code_gb300")
    gpu = importlib.import_module("pencil-code_gb300.gpu")
    L = pc.load()
    stream = torch.cuda.Stream()
    L.pcgb_set_stream(C.c_void_p(stream.cuda_stream))

    n, prec = args.n, args.precision
    timings = args.workload == "timings"
    if timings:
        p = timings_params(pc, n, prec)
        kvec, kav = timings_kvectors()
    else:
        p = headline_params(pc, n, prec, args.lentropy, args.dfloat)
    if args.tile >= 0:
        p.tile = args.tile
    if args.zdepth > 0:
        p.zdepth = args.zdepth
    if not timings and args.dt_mode:   # the CFL timestep instead of the fixed dt (1 lagged, 2 current)
        p.update(dt=0.0, dt_mode=args.dt_mode, cdt=0.4)
    if not timings and args.diag_every:
        p.diag_every = args.diag_every
    nf = 8 if args.lentropy else 7
    box = pc.Box(p)
    if timings:
        box.set_kvectors(kvec, kav)
        for k in range(nf):
            box.init_field(k, "zero")   # the timing run starts from zero fields (start.in)
    else:
        init_headline(box, p)
    info = box.info()
    box.steps(args.warmup)
    box.sync()

    sampler = ClockSampler(local)
    if ws > 1:
        torch.distributed.barrier()
    sampler.start()
    ms, launches = time_box_steps(pc, torch, box, stream, args.steps)
    clocks = sampler.stop()
    box.sync()
    ms = max_over_ranks(ms, device="cuda")
    cells = float(n) ** 3
    value = whole_job_value(cells, args.steps, ws, ms)
    # time per substep kernel: with the headline physics every launch is a substep;
    # the timing-run physics adds a CFL pass and the two forcing kernels per step,
    # charged here to the substeps (a lower bound on the substep kernel's rate)
    per_launch_ms = ms / (3 * args.steps)
    bpc = bytes_per_cell_substep(nf, prec)
    achieved = bpc * cells / (per_launch_ms / 1e3) / 1e9
    peak, peak_kind = measured_peak_hbm()
    traffic, traffic_note = None, None
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath):
        try:
            tj = json.load(open(tpath))
            key = f"f{8 * prec}_{nf}{'_dd' if args.dfloat else ''}"
            if key in tj and not timings:
                traffic = tj[key]["bytes_per_cell_substep"] * cells
                traffic_note = (f"dram bytes of one ncu capture ({tj[key]['file']}) scaled per cell to "
                                f"this launch's {n}^3 cells")
        except Exception:
            traffic = None
    box.close()
    del box

    # ---- FP64-class companions of the headline (512^3, same physics) ----
    fp64_class = None
    if not timings and not args.no_fp64_class and rank == 0 and ws == 1:
        fp64_class = run_fp64_class(args, pc, torch, stream, peak, peak_kind)

    # ---- ensemble and serving companions (rank 0, N=1) ----
    ensemble = serving = None
    if not timings and rank == 0 and ws == 1 and not args.no_ensemble:
        ensemble = ensemble_measure(pc, torch, stream, 192, 5, 3, 5, 500, args.seed, quick=True)
        L.pcgb_set_stream(C.c_void_p(stream.cuda_stream))
    if not timings and rank == 0 and ws == 1 and not args.no_serve:
        serving = serve_measure(pc, 24, [5.0, 50.0], 0.1, 0.5, False, 150.0, 10, args.seed)
        L.pcgb_set_stream(C.c_void_p(stream.cuda_stream))

    # ---- e2e through the plug-in C ABI with pinned host buffers ----
    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(args, pc, gpu, torch, stream, p, nf, ws, kvec=(kvec, kav) if timings else None)

    # ---- CPU baseline (rank 0, N=1 only) ----
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        rate, el, smp = cpu_oracle_rate(args.cpu_sample_n, args.cpu_sample_steps, threads, args.lentropy,
                                        args.workload)
        cpu = {"value": rate, "unit": "Gcell-updates/s", "cores": threads, "kind": "port",
               "sample": f"{smp['n']}^3 box, {smp['steps']} RK3 steps of the same physics, FP64 oracle "
                         f"(C restatement of the reference Fortran), OpenMP {threads} threads, {el:.1f} s"}

    if rank == 0:
        line = {
            "metric": "Gcell-updates/s per RK substep", "value": value, "unit": "Gcell-updates/s",
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            # the reference's own unit (run.f90:740): microseconds per grid point per RK step
            "us_per_pt_step": 1e3 * (ms / args.steps) / (cells * ws),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32" if prec == 4 else ("f32x2 (double-float)" if args.dfloat else "f64"),
            "data": "synthetic (seeded on device)",
            "config": {"workload": (f"timing-run physics (doc/timings/N4096_32x32x32: lupw_uu, lupw_lnrho, "
                                    f"helical forcing of aa at |k|=60, force 5e-4, nu=eta=2e-5, CFL dt cdt=0.9 "
                                    f"from the current state) on {n}^3, 7 fields, "
                                    f"{'FP32 compensated' if prec == 4 else 'FP64'}") if timings else
                                   (f"{'entropy' if args.lentropy else 'isothermal'} MHD {n}^3, {nf} fields, "
                                    f"{'FP32 compensated' if prec == 4 else ('FP64-class double-float' if args.dfloat else 'FP64')}"
                                    f", nu=eta=5e-4, ABC k=2 ampl 0.02, "
                                    + (f"CFL dt cdt=0.4 ({'lagged' if args.dt_mode == 1 else 'current'})"
                                       if args.dt_mode else "dt=2e-4")
                                    + (f", diagnostics every {args.diag_every} steps" if args.diag_every else "")),
                       "grid": n, "fields": nf,
                       "tile": info["tile"], "zdepth": info["zdepth"],
                       "l2": "inputs larger than L2 (state %.1f GB)" % (3 * nf * cells * prec / 1e9),
                       "parallelism": f"replicas x{ws}"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                         "bytes_per_cell_substep": bpc,
                         "bytes_moved_per_cell_substep": bytes_moved_per_cell_substep(nf, prec, True),
                         "traffic_basis": traffic_note},
            "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches, "clocks": clocks,
        }
        if fp64_class is not None:
            line["fp64_class"] = fp64_class
        if ensemble is not None:
            line["ensemble"] = ensemble
        if serving is not None:
            line["serving"] = serving
        if timings:
            line["published_reference"] = TIMINGS_PUBLISHED
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


def run_fp64_class(args, pc, torch, stream, peak, peak_kind) -> dict:
    """The FP64-parity states on the 512^3 headline physics, each timed alone on the
    device (CUDA events around K steps after W warm-up steps): the double-float state
    (FP64-class results on the FP32 pipes) and native FP64.  HBM fraction on the
    11/3 nf s basis with s = 8; the pipe fractions are those of the ncu captures named."""
    pipes = {}
    ppath = os.path.join(ROOT, "profiles", "pipes.json")
    if os.path.exists(ppath):
        try:
            pipes = json.load(open(ppath))
        except Exception:
            pipes = {}
    n, nf = 512, 7
    cells = float(n) ** 3
    steps = max(1, min(args.steps, 5))
    out = {"workload": f"isothermal MHD {n}^3, 7 fields, headline physics, {steps} RK3 steps after "
                       f"{args.warmup} warm-up, state {3 * nf * cells * 8 / 1e9:.1f} GB (larger than L2)"}
    for name, dfl in (("double_float", 1), ("native_fp64", 0)):
        p = headline_params(pc, n, 8, 0, dfl)
        box = pc.Box(p)
        init_headline(box, p)
        box.steps(args.warmup)
        box.sync()
        ms, launches = time_box_steps(pc, torch, box, stream, steps)
        box.sync()
        info = box.info()
        box.close()
        rate = cells * 3 * steps / (ms / 1e3) / 1e9
        achieved = bytes_per_cell_substep(nf, 8) * cells / (ms / (3 * steps) / 1e3) / 1e9
        rec = {"value": rate, "unit": "Gcell-updates/s", "ms_per_step": ms / steps, "tile": info["tile"],
               "hbm": {"achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                       "peak_kind": peak_kind, "bytes_per_cell_substep": bytes_per_cell_substep(nf, 8)},
               "gpu_launches": launches}
        if name in pipes:
            rec["compute"] = dict(pipes[name])
            ops = pipes[name].get("fp32_lane_ops_per_cell")
            if ops:   # compute roofline: FP32 lane operations against 128 FP32 lanes per SM at 2070 MHz
                nsm = torch.cuda.get_device_properties(0).multi_processor_count
                peak_ops = nsm * 128 * 2070e6
                rec["compute"].update({"achieved_fp32_lane_ops_per_s": ops * rate * 1e9,
                                       "peak_fp32_lane_ops_per_s": peak_ops,
                                       "frac_of_fp32_peak": ops * rate * 1e9 / peak_ops,
                                       "peak_basis": f"{nsm} SMs x 128 FP32 lanes x 2070 MHz (the SM clock under load)"})
        out[name] = rec
        torch.cuda.empty_cache()
    return out


def _ck(L, rc: int) -> None:
    """Raise for a non-zero status of library L (the double or the single-precision build)."""
    if rc:
        msg = L.pcgb_error_string(rc).decode()
        L.pcgb_clear_error()
        raise RuntimeError(f"pcgb error {rc}: {msg}")


def run_e2e(args, pc, gpu, torch, stream, p, nf, ws: int = 1, kvec=None):
    """The metric through the reference plug-in ABI with a page-locked host f-array of the
    Fortran build's REAL: float for an FP32 device state (libpcgb300_sgl.so, the
    single-precision build), double otherwise (libpcgb300.so)."""
    lib = importlib.import_module("pencil-code_gb300.lib")
    single = p.precision == 4
    L = lib.load_sgl() if single else pc.load()
    real, hbytes = (C.c_float, 4) if single else (C.c_double, 8)
    rptr = C.POINTER(real)
    n = p.nx
    shape = (n + 6, n + 6, n + 6, nf)
    nbytes = int(np.prod(shape)) * hbytes
    try:
        avail = os.sysconf("SC_AVPHYS_PAGES") * os.sysconf("SC_PAGE_SIZE")
    except Exception:
        avail = 0
    # every rank of the node pins its own host f-array at the same time; all ranks
    # take the same decision (a collective follows)
    fits = not (avail and nbytes > 0.45 * avail / max(ws, 1))
    if ws > 1:
        flag = torch.tensor([1 if fits else 0], dtype=torch.int32, device="cuda")
        torch.distributed.all_reduce(flag, op=torch.distributed.ReduceOp.MIN)
        fits = bool(flag.item())
    if not fits:
        return {"value": None, "unit": "Gcell-updates/s", "h2d_bytes_per_step": None, "d2h_bytes_per_step": None,
                "note": f"host f-array of {nbytes / 1e9:.1f} GB x {ws} ranks exceeds the host memory budget"}
    ht = torch.zeros(int(np.prod(shape)), dtype=torch.float32 if single else torch.float64, pin_memory=True)
    fh = ht.numpy().reshape(shape, order="F")
    iax = 5 if p.lentropy else 4
    rng = np.random.Generator(np.random.PCG64(7))
    for k in range(3):
        fh[3:-3, 3:-3, 3:-3, iax + k] = 1e-5 * rng.standard_normal((n, n, n))
    L.pcgb_set_stream(C.c_void_p(stream.cuda_stream))
    if kvec is not None:
        kv = np.ascontiguousarray(kvec[0])
        _ck(L, L.pcgb_set_kvectors(kv.ctypes.data_as(C.POINTER(C.c_double)), kv.shape[1], kvec[1]))
    _ck(L, L.pcgb_set_params(C.byref(p)))
    fptr = fh.ctypes.data_as(rptr)
    L.initializeGPU(fptr, 0, 0.0, 0, 0, 0, 0)
    _ck(L, L.pcgb_last_error())
    red = np.zeros(gpu.n_gpu_reduced_vars, dtype=np.float32 if single else np.float64)
    rp = red.ctypes.data_as(rptr)
    # warm-up through the same calls
    L.loadFarray()
    for _ in range(args.warmup):
        for s in (1, 2, 3):
            L.substepGPU(s, 0.0)
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    L.loadFarray()
    for _ in range(args.steps):
        for s in (1, 2, 3):
            L.substepGPU(s, 0.0)
        L.getGPUReducedVars(rp)
    L.copyFarray(fptr)
    torch.cuda.synchronize()
    el = max_over_ranks(time.perf_counter() - t0, device="cuda")
    _ck(L, L.pcgb_last_error())
    L.finalizeGPU()
    cells = float(n) ** 3
    # whole job: every rank advances its own replica through its own host array
    return {"value": ws * cells * 3 * args.steps / el / 1e9, "unit": "Gcell-updates/s",
            "h2d_bytes_per_step": ws * nbytes / args.steps,
            "d2h_bytes_per_step": ws * (nbytes / args.steps + red.nbytes),
            "what": "loadFarray + K x (substepGPU x3 + getGPUReducedVars) + copyFarray, pinned host f-array "
                    f"(REAL={'float, libpcgb300_sgl.so' if single else 'double, libpcgb300.so'}), wall clock",
            "amortisation": f"one host-to-device load and one device-to-host copy of the whole f-array "
                            f"({nbytes / 1e9:.1f} GB each) per {args.steps} steps, as the plug-in moves f only "
                            f"at start-up, diagnostics and snapshots (equ.f90:307-312); the reduced "
                            f"diagnostics come back every step"}


def ensemble_measure(pc, torch, stream, boxes_n: int, steps: int, warmup: int, graph_steps: int, solve_steps: int,
                     seed: int = 0, quick: bool = False) -> dict:
    """Ensemble workload: boxes_n boxes of uneven sizes and parameters, `steps` RK3 steps each,
    batched persistent launches under CUDA-graph replay (tile from the batched autotuner, z-depth
    per box size) against the single-box kernel looping over the boxes with its defaults.  Both
    legs advance every box by the same number of steps; solves/s scales the timed steps to a
    solve of solve_steps steps."""
    ens = importlib.import_module("pencil-code_gb300.ensemble")
    L = pc.load()
    specs = ens.make_ensemble(boxes_n, seed=seed)
    cells = sum(p.nx * p.ny * p.nz for p, _ in specs)
    kw = dict(tiles=(5, 6, 7), zdepths=(32, 64), per_size_zdepths=(8, 16, 32, 64, 128), sample=12,
              per_size_sample=8) if quick else {}
    t_tile, t_zd, table = ens.autotune_batch(specs, **kw)
    tuned = ens.with_tiling(specs, t_tile, t_zd)
    out = {}
    for leg in ("batched", "plain"):
        boxes = ens.build_boxes(tuned if leg == "batched" else specs)
        torch.cuda.synchronize()
        if leg == "batched":
            batch = pc.Batch(boxes, persistent=True)
            batch.steps(warmup, use_graph=False)
        else:
            for b in boxes:
                b.steps(warmup)
        torch.cuda.synchronize()
        n0 = L.pcgb_launch_count()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        if leg == "batched":
            batch.steps(steps, use_graph=True, graph_steps=graph_steps)
        else:
            for b in boxes:
                b.steps(steps)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        for b in boxes:
            b.sync()
        out[leg] = {"ms": ms, "solves_per_s": len(boxes) * steps / solve_steps / (ms / 1e3),
                    "gcell_per_s": cells * 3 * steps / (ms / 1e3) / 1e9,
                    "launches": int(L.pcgb_launch_count() - n0)}
        if leg == "batched":
            batch.close()
        for b in boxes:
            b.close()
        torch.cuda.empty_cache()
    return {"metric": "ensemble solves/s", "value": out["batched"]["solves_per_s"], "unit": "solves/s",
            "workload": f"{boxes_n} isothermal MHD boxes, sizes from {{32,48,64,96,128}}^3, nu,eta log-uniform "
                        f"[1e-3,1e-2], ABC ampl U[0.01,0.05] k in {{1,2,3}}, CFL dt cdt=0.4 (lagged), FP32 "
                        f"compensated state, FP64 reductions; {steps} RK3 steps of every box timed after {warmup}, "
                        f"scaled to solves of {solve_steps} steps",
            "graph_steps": graph_steps,
            "autotuned": {"tile": t_tile, "zdepth_by_size": {str(k): v for k, v in t_zd.items()},
                          "ms_per_step": {f"{k[0]}/{k[1]}": round(v, 3) for k, v in table.items()}},
            "batched": out["batched"], "plain": out["plain"],
            "speedup_vs_plain": out["batched"]["solves_per_s"] / out["plain"]["solves_per_s"],
            "target_speedup": 4.0}


def run_ensemble(args):
    import torch
    pc = importlib.import_module("pencil-code_gb300")
    L = pc.load()
    stream = torch.cuda.Stream()
    L.pcgb_set_stream(C.c_void_p(stream.cuda_stream))
    res = ensemble_measure(pc, torch, stream, args.boxes, args.steps, args.warmup, args.graph_steps,
                           args.solve_steps, args.seed)
    line = {"metric": res["metric"], "value": res["value"], "unit": res["unit"], "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "dtype": "f32", "data": "synthetic (seeded on device)",
            "config": {"workload": res["workload"], "graph_steps": args.graph_steps, "autotuned": res["autotuned"]},
            "batched": res["batched"], "plain": res["plain"], "speedup_vs_plain": res["speedup_vs_plain"]}
    print(json.dumps(line), flush=True)
    return 0


def serve_measure(pc, requests: int, rates, steps_scale: float, fp64_fraction: float, fp64_native: bool,
                  budget_gb: float, round_steps: int, seed: int = 0) -> dict:
    """The request stream served by the continuous-batching server and FIFO one at a time."""
    serve = importlib.import_module("pencil-code_gb300.serve")
    pc.load()
    res = []
    for rate in rates:
        reqs = serve.draw_requests(requests, seed=seed, steps_scale=steps_scale, fp64_fraction=fp64_fraction,
                                   fp64_dfloat=not fp64_native)
        row = {"rate": rate}
        for mode, maxa in (("batched", 1 << 20), ("fifo", 1)):
            row[mode] = serve.run_stream(reqs, rate, seed=seed, max_active=maxa, budget=budget_gb * 1e9,
                                         round_steps=round_steps)
        row["p99_batched_over_fifo"] = (row["batched"]["p99_s"] / row["fifo"]["p99_s"]
                                        if row["fifo"]["p99_s"] else None)
        row["solves_batched_over_fifo"] = (row["batched"]["solves_per_s"] / row["fifo"]["solves_per_s"]
                                           if row["fifo"]["solves_per_s"] else None)
        res.append(row)
    return {"metric": "serving solves/s and latency", "unit": "solves/s, s",
            "config": {"requests": requests, "sizes": "{32,64,128,256}^3 weights .4/.3/.2/.1",
                       "physics": "isothermal or entropy p=0.5", "fp64_fraction": fp64_fraction,
                       "fp64_state": "native FP64" if fp64_native else "double-float (FP64 parity bar)",
                       "steps": f"U[100,2000] x {steps_scale}", "budget_gb": budget_gb, "round_steps": round_steps,
                       "scale": (f"step counts x {steps_scale} at the arrival rates as written: every request "
                                 f"needs {steps_scale}x the work, so the offered load is {steps_scale}x config 5's")
                       if steps_scale != 1.0 else "as written"},
            "results": res}


def run_serve(args):
    pc = importlib.import_module("pencil-code_gb300")
    line = serve_measure(pc, args.requests, args.rates, args.steps_scale, args.fp64_fraction, args.fp64_native,
                         args.budget_gb, args.round_steps, args.seed)
    line.update({"n_gpus": 1, "data": "synthetic Poisson request stream"})
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=1024)
    ap.add_argument("--precision", type=int, default=4, choices=[4, 8])
    ap.add_argument("--lentropy", type=int, default=0)
    ap.add_argument("--dfloat", type=int, default=0, choices=[0, 1],
                    help="with --precision 8: double-float state and arithmetic on the FP32 pipes")
    ap.add_argument("--tile", type=int, default=-1)
    ap.add_argument("--zdepth", type=int, default=0)
    ap.add_argument("--dt-mode", type=int, default=0, choices=[0, 1, 2],
                    help="headline physics with the CFL dt: 1 lagged by a step (the GPU path's default), 2 current")
    ap.add_argument("--diag-every", type=int, default=0, help="device diagnostics every N steps")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fp64-class", action="store_true",
                    help="skip the 512^3 double-float and native FP64 companions of the headline line")
    ap.add_argument("--no-ensemble", action="store_true", help="skip the ensemble companion of the headline line")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving companion of the headline line")
    ap.add_argument("--cpu-sample-n", type=int, default=160)
    ap.add_argument("--cpu-sample-steps", type=int, default=60)
    ap.add_argument("--workload", default="headline", choices=["headline", "timings", "ensemble", "serve"])
    ap.add_argument("--boxes", type=int, default=192)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--graph-steps", type=int, default=10)
    ap.add_argument("--solve-steps", type=int, default=500)
    ap.add_argument("--requests", type=int, default=40)
    ap.add_argument("--rates", type=float, nargs="+", default=[5.0, 20.0, 50.0, 200.0])
    ap.add_argument("--steps-scale", type=float, default=0.1)
    ap.add_argument("--fp64-fraction", type=float, default=0.5)
    ap.add_argument("--fp64-native", action="store_true", help="serve FP64 requests with native FP64 state")
    ap.add_argument("--budget-gb", type=float, default=150.0)
    ap.add_argument("--round-steps", type=int, default=10)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "ensemble":
        return run_ensemble(args)
    if args.workload == "serve":
        return run_serve(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
