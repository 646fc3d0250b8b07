"""Benchmark of the explicit finite-volume time step on GB300.

Workload (default): the 2D cylinder aeroacoustics case -- stretched O-grid of
768 azimuthal x 512 radial quads (393,216 cells), M = 0.2, Re = 150, M1 scheme
with minmod on, rkOrder 5, constant dt at acoustic CFL 0.5 -- synthetic mesh and
free-stream initial field generated in memory. A "step" is one time step (5 RK
stages over all cells). The metric is cell-RK-stage updates per second.

The headline is the plain FP64 method, the arithmetic of the reference:

  value  -- device throughput with the state resident in HBM; every timed step
            is preceded (outside its timing) by a 512 MB write that evicts L2.
  e2e    -- the same metric through the C ABI with host buffers: each step
            lfm_solver_advance copies the state from pinned host memory to the
            device, advances one time step and copies the state back, timed on
            the host clock.

Beside it, in the same line: ``fp32_bulk`` -- the FP32-bulk form (FP32 fluxes,
limiter, residual sums and RK increment register on perturbations from the
free stream; FP64 accumulation of the conserved state, ghost states and
geometry) with its own value, e2e, roofline and speed-up over FP64;
``accuracy`` -- the acoustic-pressure error of the FP32-bulk state against the
FP64 state after --accuracy-steps time steps (all cells and 72 probes at
r = 50 D); ``wake3d`` -- the 3D cylinder wake (384x256x96, 9.4M hex cells)
device-timed in both precisions, the HBM-bound case; ``batch64`` -- the
64-case batched sweep (15.5M cells, one persistent kernel per RK stage) with
its roofline, e2e and the plain FP64 path on the same cases; ``serve`` -- a
30-second Poisson stream of solve requests into the request server (p50 /
p99, throughput, against the same stream served one request at a time on the
FP64 path); ``fp64_pipe`` --
the FP64 instruction roofline that bounds the plain method on GB300.

--impl reference times the reference's CPU implementation of the same
workload on the host cores (the oracle port, set up by its own code: one
process per core, each on the full mesh, aggregate throughput, FP64).

Launch: python bench.py [--gpus N] [--steps K] [--warmup W] [--precision fp64|fp32]
Under torchrun each rank runs its own replica (weak scaling); rank 0 prints.
"""
from __future__ import annotations

import argparse
import json
import math
import multiprocessing as mp
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "cell-RK-stage updates/s"
UNIT = "cell-stage/s"
PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")
FP64_PEAK_TFLOPS = 1.195  # DFMA rate measured on GB300 with a dependent-chain-free FMA loop


def workload(name: str):
    from lfm_public_gb300 import cases
    if name == "cylinder2d":
        return cases.cylinder_case(n_theta=768, n_r=512, solver=0, minmod=True)
    if name == "cylinder2d_m2":
        return cases.cylinder_case(n_theta=768, n_r=512, solver=1, minmod=True)
    if name == "cylinder2d_fine":
        return cases.cylinder_case(n_theta=1536, n_r=1024, first=0.004, solver=0, minmod=True)
    if name == "vortex2d":
        return cases.vortex_case(n=256, solver=0)
    if name == "cylinder2d_shuffled":
        # the 768x512 O-grid with its cells numbered at random, as an
        # unstructured mesh generator may leave them (renumbering test)
        import numpy as np
        c = cases.cylinder_case(n_theta=768, n_r=512, solver=0, minmod=True)
        return cases.renumber_cells(c, np.random.default_rng(768512).permutation(c.n_cells))
    if name == "cylinder3d":
        return cases.cylinder_case(n_theta=384, n_r=256, n_span=96, solver=1, reynolds=3900.0, noise=0.01, seed=3900,
                                   minmod=False)
    if name == "cylinder3d_small":
        return cases.cylinder_case(n_theta=192, n_r=128, n_span=48, solver=1, reynolds=3900.0, noise=0.01, seed=3900,
                                   minmod=False)
    raise ValueError(f"unknown workload {name}")


WORKLOAD_DESC = {
    "cylinder2d": dict(workload="2D cylinder O-grid 768x512, M1, minmod on, rkOrder 5, CFL 0.5", cells=393216,
                       dim=2, scheme="M1", faces_per_cell=4, viscous=True),
    "cylinder2d_m2": dict(workload="2D cylinder O-grid 768x512, M2, minmod on, rkOrder 5, CFL 0.5", cells=393216,
                          dim=2, scheme="M2", faces_per_cell=4, viscous=True),
    "cylinder2d_fine": dict(workload="2D cylinder O-grid 1536x1024 (first cell 0.004 D), M1, minmod on, rkOrder 5, CFL 0.5",
                            cells=1572864, dim=2, scheme="M1", faces_per_cell=4, viscous=True),
    "cylinder2d_shuffled": dict(workload="2D cylinder O-grid 768x512 with randomly numbered cells, M1, minmod on, "
                                "rkOrder 5, CFL 0.5", cells=393216, dim=2, scheme="M1", faces_per_cell=4, viscous=True),
    "vortex2d": dict(workload="2D isentropic vortex 256x256, M1, rkOrder 5, CFL 0.5", cells=65536, dim=2,
                     scheme="M1", faces_per_cell=4, viscous=False),
    "cylinder3d": dict(workload="3D cylinder wake 384x256x96, M2, cyclic span, rkOrder 5", cells=9437184, dim=3,
                       scheme="M2", faces_per_cell=6, viscous=True),
    # the same wake at an eighth of the cells (working set ~0.9 GB, still
    # beyond L2): the size the 3D kernels are profiled at
    "cylinder3d_small": dict(workload="3D cylinder wake 192x128x48, M2, cyclic span, rkOrder 5", cells=1179648,
                             dim=3, scheme="M2", faces_per_cell=6, viscous=True),
}


# DRAM bytes (read + write) of one launch of the dominant kernel, from one ncu
# capture of this bench's own command (cold L2: ncu flushes the caches before
# each captured launch). Keyed by (workload, precision, kernel).
DRAM_TRAFFIC = {
    ("cylinder2d", "fp32", "k_update"): 42937856 + 190976,
    ("cylinder2d", "fp32", "k_flux"): 48100000 + 670000,
    # the 384x256x96 wake is too large for a full capture: its figure is the
    # 192x128x48 capture
    # scaled by the cells (x8), the traffic being at the algorithmic bytes,
    # which grow in proportion
    ("cylinder3d_small", "fp32", "k_flux"): 270532096 + 54157824,
    ("cylinder3d", "fp32", "k_flux"): 8 * (270532096 + 54157824),
    ("cylinder2d", "fp64", "k_flux"): 95838720 + 8762112,
}

# FP64 pipe thread-instructions per cell of one launch of each kernel of the
# plain FP64 path (DFMA, DMUL, DADD and the FP64 parts of divisions and square
# roots), counted by ncu (sm__thread_inst_executed_pipe_fp64_pred_on.sum /
# cells) on the 768x512 cylinder, M1, viscous; the update also derives the next
# stage's primitives and boundary ghosts (no preparation kernel).
FP64_INST_PER_CELL = {
    "cylinder2d": {"k_prep": 0.0, "k_grad": 0.0, "k_vis": 45.00, "k_flux": 156.22, "k_update": 42.67},
}
# FP64 pipe instruction rate: the measured DFMA rate (FP64_PEAK_TFLOPS counts
# an FMA as two operations) in instructions per second.
FP64_PIPE_PEAK_GINST = FP64_PEAK_TFLOPS * 1e3 / 2.0


def fp64_pipe_roofline(workload: str, cells: int, stages: int, ms_per_step: float, kernels_ms_per_step: dict):
    """The plain FP64 path is bound by GB300's FP64 pipe, not by HBM: FP64
    instructions executed per second against the measured DFMA rate, for the
    whole step and for its dominant kernel."""
    per = FP64_INST_PER_CELL.get(workload)
    if per is None:
        return None
    step_inst = sum(per.values()) * cells * stages
    dom = max(kernels_ms_per_step, key=kernels_ms_per_step.get)
    dom_ginst = per[dom] * cells * stages / (kernels_ms_per_step[dom] * 1e-3) / 1e9
    achieved = step_inst / (ms_per_step * 1e-3) / 1e9
    return {"bound": "fp64-pipe", "achieved": achieved, "peak": FP64_PIPE_PEAK_GINST, "unit": "G FP64 inst/s",
            "frac": achieved / FP64_PIPE_PEAK_GINST, "kernel": dom, "kernel_achieved": dom_ginst,
            "kernel_frac": dom_ginst / FP64_PIPE_PEAK_GINST, "fp64_inst_per_cell_stage": sum(per.values()),
            "peak_source": "measured DFMA rate"}


def kernel_bytes(dim: int, faces_per_cell: int, fp32: bool, scheme: str, viscous: bool):
    """Algorithmic bytes per cell of one launch of each kernel: every array
    element the kernel must touch, once (face arrays once per face, cell arrays
    once per cell, neighbour re-reads served by cache). ``faces_per_cell`` is
    the faces around a cell; each face is shared by two cells."""
    nq = dim + 2
    fpc = faces_per_cell / 2.0            # faces per cell
    w = 4 if fp32 else 8                  # bulk word (prim, V, grad, flux, geometry)
    prim = (2 * dim + 3) if fp32 else (dim + 3)
    nv = dim * dim + 2 * dim              # dudx, dTdx, sigmaU
    ng = 2 * dim + dim * dim              # rho, p, U gradients
    csr = 4 + 4 * faces_per_cell          # cell -> face offsets and list
    face_basic = 8 + (dim + 1) * w        # fP, fN, S, w
    b = {}
    # the update writes the next stage's primitives of its cell and of its
    # boundary ghosts, so the preparation pass only covers processor halos
    # (none in a single-partition case)
    b["k_prep"] = 0.0
    b["k_grad"] = (prim * w + fpc * face_basic + csr + ng * w) if scheme == "M2AUSM" else 0.0
    b["k_vis"] = ((dim + 1) * w + fpc * face_basic + csr + nv * w) if (viscous or scheme == "M2AUSM") else 0.0
    flux_cell = (prim - 1) * w + (0 if fp32 else nq * 8)   # FP64 also reads q
    if viscous or scheme == "M2AUSM":
        flux_cell += nv * w
    if scheme == "M2AUSM":
        flux_cell += ng * w + w
    flux_face = face_basic + 1 + nq * w + ((dim + 1) * w if viscous else 0) + (dim * w if scheme == "M2AUSM" else 0)
    b["k_flux"] = flux_cell + fpc * flux_face
    if fp32:   # q' read + written (FP64), dq read + written (FP32), 1/V, sigma, primitives out
        b["k_update"] = csr + fpc * nq * w + 2 * nq * 8 + 2 * nq * 4 + 8 + prim * 4
    else:      # q and dq read + written, 1/V, sigma, primitives out (the sound speed for M2AUSM only)
        b["k_update"] = csr + fpc * nq * w + 4 * nq * 8 + 16 + (prim - (0 if scheme == "M2AUSM" else 1)) * 8
    if fp32:
        # the fused tile stage does the work of the gradient, viscous, flux and
        # update kernels: the same algorithmic bytes (its intermediate arrays
        # stay in shared memory, so its traffic is below them)
        b["k_tile_stage"] = b["k_grad"] + b["k_vis"] + b["k_flux"] + b["k_update"]
        # the fused flux + update: both kernels' bytes without the face rhs,
        # which it never writes or reads back
        b["k_flux_update"] = b["k_flux"] + b["k_update"] - 2 * fpc * nq * w
    return b


class _Nvml:
    """Read-only NVML queries through ctypes (the driver's libnvidia-ml):
    SM clock, its maximum and the clock event (throttle) reasons."""

    SM = 1   # NVML_CLOCK_SM
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown",
               0x80: "hw_power_brake_slowdown"}

    def __init__(self, index: int):
        import ctypes as C
        self.C = C
        self.lib = C.CDLL("libnvidia-ml.so.1")
        if self.lib.nvmlInit_v2() != 0:
            raise RuntimeError("nvmlInit failed")
        self.h = C.c_void_p()
        if self.lib.nvmlDeviceGetHandleByIndex_v2(C.c_uint(index), C.byref(self.h)) != 0:
            raise RuntimeError("no NVML device")
        self.reasons_fn = getattr(self.lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            self.lib.nvmlDeviceGetCurrentClocksThrottleReasons

    def sample(self):
        C = self.C
        sm, mx, r = C.c_uint(), C.c_uint(), C.c_ulonglong()
        self.lib.nvmlDeviceGetClockInfo(self.h, self.SM, C.byref(sm))
        self.lib.nvmlDeviceGetMaxClockInfo(self.h, self.SM, C.byref(mx))
        self.reasons_fn(self.h, C.byref(r))
        return float(sm.value), float(mx.value), int(r.value)


class ClockSampler:
    """SM clocks and throttle reasons sampled every few milliseconds through
    NVML while the timed regions run (mark() opens and closes a timed region);
    nvidia-smi every 0.2 s where NVML cannot be loaded."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.samples = []     # (timed, sm_mhz, max_mhz, set of reasons)
        self.timed = False
        self._stop = threading.Event()
        self._t = None
        self.source = "nvml"

    def mark(self):
        self.timed = not self.timed

    def _smi(self):
        out = subprocess.run(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                              "--format=csv,noheader,nounits"], capture_output=True, text=True,
                             timeout=5).stdout.strip()
        if not out:
            return None
        f = [x.strip() for x in out.split(",")]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        num = lambda x: float(x) if x.replace(".", "").isdigit() else None   # noqa: E731
        return num(f[1]), num(f[2]), {n for k, n in enumerate(names) if len(f) > 5 + k and
                                      f[5 + k].lower().startswith("active")}

    def __enter__(self):
        def run():
            nv = None
            try:
                nv = _Nvml(self.device)
            except Exception:
                self.source = "nvidia-smi"
            while not self._stop.is_set():
                timed = self.timed
                try:
                    if nv is not None:
                        sm, mx, r = nv.sample()
                        rec = (sm, mx, {n for b, n in _Nvml.REASONS.items() if r & b})
                    else:
                        rec = self._smi()
                    if rec:
                        self.samples.append((timed,) + rec)
                except Exception:
                    pass
                self._stop.wait(0.002 if nv is not None else 0.2)
        self._t = threading.Thread(target=run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)

    def summary(self):
        sel = [x for x in self.samples if x[0]] or self.samples
        if not sel:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        sm = sorted(x[1] for x in sel if x[1] is not None)
        mx = max((x[2] for x in sel if x[2] is not None), default=None)
        reasons = set()
        for x in sel:
            reasons |= x[3]
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sel), "samples_in_timed_regions": sum(1 for x in self.samples if x[0]),
                "source": self.source}


# ---------------------------------------------------------------------------
# CPU baseline: the oracle port, one process per core. Each process sets its
# case up with the oracle's own code (oracle/port), so the reference arm maps
# nothing of the device library.
# ---------------------------------------------------------------------------
def _port_worker(name, steps, repeats, barrier, out):
    sys.path.insert(0, ROOT)
    import oracle.port as P
    case = workload(name)
    pc = P.PortCase.from_case(case)
    q0 = pc.q0()
    for _ in range(repeats):
        barrier.wait()
        t0 = time.time()
        P.run(pc, q0, steps, case.delta_t)
        t1 = time.time()
        out.put((pc.desc.n_cells * pc.desc.rk_order * steps, t0, t1))


def cpu_baseline(name: str, steps_per_proc: int, procs: int, repeats: int = 1):
    """Aggregate throughput of `procs` oracle processes, each advancing the full
    mesh by `steps_per_proc` time steps, started together `repeats` times.
    Returns a list of (rate, seconds, updates), one per repeat."""
    ctx = mp.get_context("spawn")
    barrier = ctx.Barrier(procs)
    out = ctx.Queue()
    ps = [ctx.Process(target=_port_worker, args=(name, steps_per_proc, repeats, barrier, out)) for _ in range(procs)]
    for p in ps:
        p.start()
    res = [out.get() for _ in range(procs * repeats)]
    for p in ps:
        p.join()
    res.sort(key=lambda r: r[1])
    rounds = []
    for k in range(repeats):
        grp = res[k * procs:(k + 1) * procs]
        upd = sum(r[0] for r in grp)
        t = max(r[2] for r in grp) - min(r[1] for r in grp)
        rounds.append((upd / t, t, upd))
    return rounds


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo", init_method="env://")
        pg = dist
    return ws, rank, local, pg


def _allmax(pg, v: float) -> float:
    if pg is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def run_reference(args):
    """The reference's CPU time step on the host cores: the oracle port (set
    up by its own code), one process per core, each on the full mesh, FP64."""
    ws, rank, _, pg = _dist()
    if rank != 0:
        return 0
    procs = os.cpu_count() or 1
    steps_per_proc = 1
    rounds = cpu_baseline(args.workload, steps_per_proc, procs, repeats=args.warmup + max(1, args.steps))
    timed = rounds[args.warmup:] or rounds
    value = sum(r[2] for r in timed) / sum(r[1] for r in timed)
    desc = WORKLOAD_DESC[args.workload]
    sample = (f"{procs} processes x {steps_per_proc} time step(s) of the full {desc['cells']}-cell mesh per bench "
              f"step; aggregate cell-stage updates / wall time")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * desc["cells"] * 5 / value,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": desc["workload"], "cells": desc["cells"], "rk_stages": 5, "precision": "fp64"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": procs, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def _peaks():
    peaks = json.load(open(PEAKS_FILE)) if os.path.exists(PEAKS_FILE) else {}
    return peaks.get("hbm_gbs", 6800.0), ("measured" if "hbm_gbs" in peaks else "fallback")


def _time_leg(N, ch, precision, dt, steps, warmup, local, pg, clk=None):
    """Device throughput of one solver: W warm-up steps, then K steps timed
    with CUDA events, each preceded by a 512 MB write that evicts L2; then the
    per-kernel times (prefix differences, lfm_solver_profile_step). Returns
    (solver, total ms of the K steps (max over ranks), kernel ms per step,
    launches per step)."""
    s = N.Solver(ch, precision=precision, device=local)
    tune = None
    if precision == N.LFM_FP32_BULK:
        # flux kernel (face, cell-centred, staged at each staging depth): the
        # fastest on this case, by lfm_solver_autotune (all give the same bits)
        tried = []
        t = s.autotune(dt, trial_steps=3, tried=tried)
        tune = {"chosen": t.as_dict(), "tried": [x.as_dict() for x in tried]}
    for _ in range(warmup):
        s.step(1, dt)
    s.sync()
    if pg:
        pg.barrier()
    if clk is not None:
        clk.mark()
    times = s.bench(steps, dt, 512 << 20)
    s.sync()
    if clk is not None:
        clk.mark()
    if pg:
        pg.barrier()
    total_ms = _allmax(pg, float(times.sum()))
    prof = s.profile_step(dt)
    s.sync()
    return s, total_ms, prof, s.launches_per_step(), tune


def _e2e(s, nq, nc, dt, steps, pg):
    """The metric end to end through lfm_solver_advance: every step the state
    in from pinned host memory, one time step, the state out (host clock)."""
    import torch
    host = torch.empty((nq, nc), dtype=torch.float64, pin_memory=True).numpy()
    s.get_state(out=host)
    for _ in range(2):
        s.advance(host, 1, dt, host)
    t0 = time.perf_counter()
    for _ in range(steps):   # lfm_solver_advance: state in, one step, state out
        s.advance(host, 1, dt, host)
    s.sync()
    return _allmax(pg, time.perf_counter() - t0)


def _hbm_roofline(desc, fp32, prof, nc, stages, workload, precision, hbm, peak_src, extra=None):
    """HBM roofline of the dominant kernel: algorithmic bytes per launch over
    its time per launch (from the prefix-difference profile)."""
    kb = kernel_bytes(desc["dim"], desc["faces_per_cell"], fp32, desc["scheme"], desc["viscous"])
    dominant = max(prof, key=prof.get)
    per_launch_ms = prof[dominant] / stages
    achieved = kb[dominant] * nc / (per_launch_ms * 1e-3) / 1e9
    step_bytes = sum(v for k, v in kb.items() if k in prof)
    r = {"bound": "hbm", "kernel": dominant, "achieved": achieved, "peak": hbm, "unit": "GB/s",
         "frac": achieved / hbm, "peak_source": peak_src, "traffic": DRAM_TRAFFIC.get((workload, precision, dominant)),
         "algorithmic_bytes_per_cell": kb[dominant], "cells_per_launch": nc,
         "kernel_ms_per_launch": per_launch_ms, "step_algorithmic_bytes_per_cell_stage": step_bytes}
    if extra:
        r.update(extra)
    return r, step_bytes


def _leg_record(N, ch, precision, dt, args, ws, local, pg, desc, workload, hbm, peak_src, clk=None, e2e=True):
    """Device-timed value, per-kernel times, HBM roofline and (optionally)
    e2e of one precision on one case."""
    nc, nq, stages = ch.desc.n_cells, ch.desc.nq, ch.desc.rk_order
    fp32 = precision == N.LFM_FP32_BULK
    s, total_ms, prof, launches, tune = _time_leg(N, ch, precision, dt, args.steps, args.warmup, local, pg, clk)
    value = ws * nc * stages * args.steps / (total_ms / 1000.0)
    ms_step = total_ms / args.steps
    roof, step_bytes = _hbm_roofline(desc, fp32, prof, nc, stages, workload, "fp32" if fp32 else "fp64", hbm,
                                     peak_src)
    roof["step_achieved"] = step_bytes * nc * stages / (ms_step * 1e-3) / 1e9
    roof["step_frac"] = roof["step_achieved"] / hbm
    rec = {"value": value, "unit": UNIT, "ms_per_step": ms_step, "kernels_ms_per_step": prof,
           "kernels_sum_ms": sum(prof.values()), "roofline": roof, "launches_per_step": launches}
    if tune is not None:
        rec["flux_tuning"] = tune
    if e2e:
        e2e_steps = max(1, args.steps)
        e2e_s = _e2e(s, nq, nc, dt, e2e_steps, pg)
        rec["e2e"] = {"value": ws * nc * stages * e2e_steps / e2e_s, "unit": UNIT,
                      "h2d_bytes_per_step": nq * nc * 8, "d2h_bytes_per_step": nq * nc * 8}
    s.close()
    return rec


RING_RADII = (5.0, 10.0, 20.0, 50.0)


def _accuracy(N, acoustics, case, ch, dt, checkpoints, local, rings):
    """Acoustic-pressure error of the FP32-bulk state against the FP64 state
    at each checkpoint (time steps from the initial state): all cells and the
    72-probe rings. A ring whose FP64 p' is exactly zero has not been reached
    by any disturbance yet (rel_l2 null there)."""
    import numpy as np
    sol = [N.Solver(ch, precision=p, device=local) for p in (N.LFM_FP64, N.LFM_FP32_BULK)]
    g, d = ch.desc.gamma, case.dim
    ring_cells = {r: acoustics.probe_ring(case.cell_centres, ch.cell_ids(), r) for r in rings}
    out, done = [], 0
    for n in checkpoints:
        for s in sol:
            s.step(n - done, dt)
        done = n
        qs = []
        for s in sol:
            s.sync()
            qs.append(s.get_state())
        rec = {"steps": n, "acoustic_p_rel_l2": acoustics.acoustic_rel_l2(qs[1], qs[0], g, d, case.p_inf)}
        ring_recs = []
        for r, cells in ring_cells.items():
            p64 = acoustics.pressure(qs[0], g, d)[cells] - case.p_inf
            rms = float(np.sqrt(np.mean(p64 ** 2)))
            ring_recs.append({"radius": r, "probes": len(cells), "p_rms_ref": rms,
                              "rel_l2": acoustics.acoustic_rel_l2(qs[1], qs[0], g, d, case.p_inf, cells)
                              if rms > 0 else None})
        rec["probe_rings"] = ring_recs
        out.append(rec)
    for s in sol:
        s.close()
    acc = dict(out[0])
    acc["against"] = "FP64 device path (itself within 1e-12 of the oracle), same case and steps"
    if len(out) > 1:
        acc["longer"] = out[1:]
    acc["probe_ring"] = ring_at_longest(out, 50.0)
    return acc


def ring_at_longest(checkpoints, radius):
    """The probe ring of `radius` at the longest checkpoint its FP64 p' has
    reached (a ring the start-up pulse has not reached yet has p' = 0 and no
    error), with that checkpoint's step count; the first checkpoint's ring
    when none has been reached."""
    best = None
    for rec in checkpoints:
        ring = next((x for x in rec["probe_rings"] if x["radius"] == radius), None)
        if ring is not None and (best is None or ring["rel_l2"] is not None):
            best = dict(ring, steps=rec["steps"])
    return best


def _guarded(fn, *a):
    """A sub-record of the default line; a failure there is reported in the
    line (the headline stands) instead of ending the run."""
    try:
        return fn(*a)
    except Exception as e:
        return {"error": repr(e)}


def _wake_record(N, built, args, local, hbm, peak_src):
    """Device-timed sub-record of the 3D cylinder wake (384x256x96, 9.4M hex
    cells, working set far beyond L2): FP32-bulk and FP64, no CPU leg."""
    case, ch = built
    dt = case.delta_t
    desc = WORKLOAD_DESC["cylinder3d"]
    sub = argparse.Namespace(steps=args.wake_steps, warmup=3)
    r32 = _leg_record(N, ch, N.LFM_FP32_BULK, dt, sub, 1, local, None, desc, "cylinder3d", hbm, peak_src, e2e=False)
    r32["roofline"]["traffic_note"] = ("DRAM bytes of one k_flux launch of the 192x128x48 wake scaled by the cells "
                                       "(x8); the traffic sits at the algorithmic bytes, which grow in proportion")
    r64 = _leg_record(N, ch, N.LFM_FP64, dt, argparse.Namespace(steps=max(2, args.wake_steps // 2), warmup=2), 1,
                      local, None, desc, "cylinder3d", hbm, peak_src, e2e=False)
    return {"workload": desc["workload"], "cells": ch.desc.n_cells, "steps": args.wake_steps,
            "l2": "512 MB write between timed steps (working set ~7 GB FP32-bulk, beyond L2)",
            "fp32_bulk": r32, "fp64": r64, "speedup_fp32_bulk_vs_fp64": r32["value"] / r64["value"]}


def run_gpu(args):
    ws, rank, local, pg = _dist()
    from lfm_public_gb300 import _native as N, acoustics
    desc = WORKLOAD_DESC[args.workload]
    fp32_head = args.precision == "fp32"

    base = None
    if rank == 0 and not args.no_cpu_baseline:
        # before any GPU call in this process (the pool uses spawn)
        procs = 1
        r, t, u = cpu_baseline(args.workload, 1, procs)[0]
        base = {"value": r, "unit": UNIT, "cores": procs, "kind": "port",
                "sample": f"1 time step (5 RK stages) of the full {desc['cells']}-cell mesh, single thread, {t:.1f} s"}

    case = workload(args.workload)
    ch = N.CaseHandle.from_case(case, renumber={"none": 0, "rcm": 1, "hilbert": 2, "hpath": 3}[args.renumber])
    nc, stages = ch.desc.n_cells, ch.desc.rk_order
    dt = case.delta_t
    hbm, peak_src = _peaks()

    # the plain FP64 method and the FP32-bulk form, each device-timed, with
    # its per-kernel times, roofline and end-to-end rate
    with ClockSampler(local) as clk:
        time.sleep(0.3)
        legs = {}
        for name, prec in (("fp64", N.LFM_FP64), ("fp32", N.LFM_FP32_BULK)):
            legs[name] = _leg_record(N, ch, prec, dt, args, ws, local, pg, desc, args.workload, hbm, peak_src,
                                     clk=clk)
    head, other = (legs["fp32"], legs["fp64"]) if fp32_head else (legs["fp64"], legs["fp32"])
    pipe64 = fp64_pipe_roofline(args.workload, nc, stages, legs["fp64"]["ms_per_step"],
                                legs["fp64"]["kernels_ms_per_step"])

    # the 3D wake case is set up on a host thread while the long accuracy run
    # keeps the GPU busy
    wake_built, wake_err = [None], [None]

    def build_wake():
        try:
            c3 = workload("cylinder3d")
            wake_built[0] = (c3, N.CaseHandle.from_case(c3))
        except Exception as e:   # reported in the line
            wake_err[0] = repr(e)

    wake_thread = None
    # the accuracy runs and the sub-records are reported by rank 0 alone, and
    # only rank 0 runs them (under torchrun the other ranks would only repeat
    # them, each holding the large cases in host memory)
    extras = rank == 0
    if extras and args.wake and args.workload.startswith("cylinder2d"):
        wake_thread = threading.Thread(target=build_wake, daemon=True)
        wake_thread.start()
    # and so are the 64 cases of the batched sweep
    sweep_built, sweep_err = [None], [None]

    def build_sweep():
        try:
            sweep_built[0] = _build_sweep(64, 20261203)
        except Exception as e:   # reported in the line
            sweep_err[0] = repr(e)

    sweep_thread = None
    if extras and args.batch and args.workload.startswith("cylinder2d"):
        sweep_thread = threading.Thread(target=build_sweep, daemon=True)
        sweep_thread.start()
    # and so is the serving library
    lib_built, lib_err = [None], [None]

    def build_lib():
        try:
            lib_built[0] = _serve_library(args.serve_library, local)
        except Exception as e:   # reported in the line
            lib_err[0] = repr(e)

    lib_thread = None
    if extras and args.serve and args.workload.startswith("cylinder2d"):
        lib_thread = threading.Thread(target=build_lib, daemon=True)
        lib_thread.start()
    accuracy = None
    if extras and args.accuracy_steps:
        accuracy = _accuracy(N, acoustics, case, ch, dt, args.accuracy_steps, local,
                             RING_RADII if args.workload.startswith("cylinder") else ())
    wake = None
    if wake_thread is not None:
        wake_thread.join()
        wake = (_guarded(_wake_record, N, wake_built[0], args, local, hbm, peak_src) if wake_built[0]
                else {"error": wake_err[0]})
        wake_built[0] = None
    batch = None
    if sweep_thread is not None:
        sweep_thread.join()
        if sweep_built[0]:
            spec, built = sweep_built[0]
            batch = _guarded(_batch_record, N, built, spec, local, None, 1, args.batch_steps, 3)
        else:
            batch = {"error": sweep_err[0]}
        sweep_built[0] = None
    serve = None
    if lib_thread is not None:
        lib_thread.join()
        if lib_built[0]:
            lib = lib_built[0]
            def serve_record():
                fp64 = _fp64_times(lib, local)
                rate = float(args.serve_default_rate)
                return dict(_serve_config(args, lib, args.serve_default_window, str(rate)),
                            **_serve_rate(N, args, lib, fp64, rate, args.serve_default_window, 77, local))

            serve = _guarded(serve_record)
        else:
            serve = {"error": lib_err[0]}
        lib_built[0] = None

    if rank != 0:
        return 0
    fp32_rec = dict(legs["fp32"])
    fp32_rec["speedup_vs_fp64"] = legs["fp32"]["value"] / legs["fp64"]["value"]
    fp32_rec["e2e_speedup_vs_fp64"] = legs["fp32"]["e2e"]["value"] / legs["fp64"]["e2e"]["value"]
    fp32_rec["accuracy"] = accuracy
    fp32_rec["dtype"] = "f32-flux/f64-rk"
    line = {
        "metric": METRIC, "value": head["value"], "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": head["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32-flux/f64-rk" if fp32_head else "f64",
        "data": "synthetic (generated mesh and initial field)",
        "config": {"workload": desc["workload"], "cells": nc, "rk_stages": stages,
                   "precision": "fp32-bulk" if fp32_head else "fp64", "l2": "512 MB write between timed steps",
                   "renumber": args.renumber, "parallelism": f"replicas x{ws}"},
        "roofline": dict(head["roofline"], **({} if fp32_head else {
            "limiter": "fp64-pipe (see fp64_pipe: GB300 issues about two FP64 instructions per clock per SM)"})),
        "fp64_pipe": pipe64,
        "kernels_ms_per_step": head["kernels_ms_per_step"], "kernels_sum_ms": head["kernels_sum_ms"],
        "dominant_kernel": head["roofline"]["kernel"],
        "e2e": head["e2e"],
        "fp32_bulk": fp32_rec if not fp32_head else None,
        "plain_fp64": dict(other, speedup=head["value"] / other["value"]) if fp32_head else None,
        "accuracy": accuracy,
        "wake3d": wake,
        "batch64": batch,
        "serve": serve,
        "cpu_baseline": base,
        "gpu_launches": head["launches_per_step"] * args.steps,
        "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)
    return 0


BATCH_DESC = ("64-case batched sweep: quad grids and jittered triangulations of [-10,10]^2, cells log-uniform "
              "16k-1M, isentropic vortex beta U(1,5), M U(0.1,0.6), M1/M2 at random, rkOrder 5, seed 20261203; "
              "FP32-bulk, one persistent kernel per RK stage")


def _build_sweep(n_cases: int, seed: int):
    """Cases and handles of the batched sweep, set up in parallel threads (the
    C++ set-up runs outside the GIL)."""
    from concurrent.futures import ThreadPoolExecutor
    from lfm_public_gb300 import _native as N, cases
    spec = cases.sweep_spec(n_cases=n_cases, seed=seed)

    def one(sp):
        c = cases.sweep_case(sp)
        return c, N.CaseHandle.from_case(c)

    with ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        out = list(ex.map(one, spec))
    return spec, out


def _batch_record(N, built, spec, local, pg, ws, steps, warmup, tuning_arg=None, clk=None):
    """The batched form on the sweep's cases: autotuned (or given) launch
    shape, device-timed steps from the initial states, the HBM roofline of
    the stage kernel, e2e through lfm_batch_advance, and the plain FP64 path
    on the same cases one solver at a time."""
    cells = sum(ch.desc.n_cells for _, ch in built)
    need = sum(N.Batch.case_bytes(ch) for _, ch in built)
    b = N.Batch(device=local, arena_bytes=need + (64 << 20), max_cases=len(built))
    slots = [b.add(ch, c.delta_t) for c, ch in built]
    if tuning_arg:
        v = [int(x) for x in tuning_arg.split(",")]
        b.set_tuning(v[0], v[1], v[2], phased=v[3] if len(v) > 3 else 0)
        tuning = b.tuning()
    else:
        tuning = b.autotune(trial_steps=2)
    for _ in range(warmup):
        b.step(1)
    # timed steps start from the initial states (the reference's central
    # schemes diverge on some jittered triangulations after a few hundred steps)
    for (c, ch), s in zip(built, slots):
        b.set_state(s, ch.q0())
    if pg:
        pg.barrier()
    if clk is not None:
        time.sleep(0.3)
        clk.mark()
    times = b.bench(steps, 512 << 20)
    if clk is not None:
        clk.mark()
    nonfinite = [k for k, s in enumerate(slots) if b.case_status(s) != N.LFM_OK]
    if pg:
        pg.barrier()
    total_ms = _allmax(pg, float(times.sum()))
    stages = 5
    value = ws * cells * stages * steps / (total_ms / 1000.0)

    # end to end through the C ABI: every case's state in from pinned host
    # memory, one step of the batch, every state back out, each step
    import torch
    hosts = [torch.empty((ch.desc.nq, ch.desc.n_cells), dtype=torch.float64, pin_memory=True).numpy()
             for _, ch in built]
    for (c, ch), h in zip(built, hosts):
        h[:] = ch.q0()
    e2e_steps = max(1, min(steps, 20))
    t0 = time.perf_counter()
    for _ in range(e2e_steps):   # lfm_batch_advance: every state in, one step, every state out
        b.advance(slots, hosts, 1, hosts)
    e2e_s = _allmax(pg, time.perf_counter() - t0)
    e2e_value = ws * cells * stages * e2e_steps / e2e_s
    io_bytes = sum(h.nbytes for h in hosts)
    launches = b.launches_per_step()
    b.close()

    # the plain FP64 path on the same cases, one solver per case in turn
    k64 = max(1, min(steps, 20))
    ms64 = 0.0
    for c, ch in built:
        s = N.Solver(ch, precision=N.LFM_FP64, device=local)
        s.step(2, c.delta_t)
        ms64 += float(s.bench(k64, c.delta_t, 0).sum())
        s.close()
    v64 = cells * stages * k64 / (ms64 / 1000.0)

    hbm, peak_src = _peaks()
    step_bytes = 0.0
    for sp, (c, ch) in zip(spec, built):
        kb = kernel_bytes(2, 4 if sp["kind"] == "quad" else 3, True, "M1" if sp["solver"] == 0 else "M2", False)
        step_bytes += sum(v for k, v in kb.items() if k not in ("k_tile_stage", "k_flux_update")) * ch.desc.n_cells
    stage_ms = total_ms / ws / steps / stages
    achieved = step_bytes / (stage_ms * 1e-3) / 1e9
    return {
        "workload": BATCH_DESC, "cases": len(built), "cells": cells, "value": value, "unit": UNIT,
        "steps": steps, "ms_per_step": total_ms / steps, "tuning": tuning, "nonfinite_after_timed_steps": nonfinite,
        "roofline": {"bound": "hbm", "kernel": "k_batch_stage", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "peak_source": peak_src, "traffic": None,
                     "algorithmic_bytes_per_stage": step_bytes, "cells_per_launch": cells},
        "plain_fp64": {"value": v64, "unit": UNIT, "steps_per_case": k64, "speedup": value / v64,
                       "how": "one FP64 solver per case, cases in turn, CUDA-event time summed"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": io_bytes, "d2h_bytes_per_step": io_bytes},
        "launches_per_step": launches,
    }


def run_batch(args):
    """The batched form: all sweep cases in one batch, autotuned launch shape."""
    ws, rank, local, pg = _dist()
    import numpy as np
    from lfm_public_gb300 import _native as N, acoustics
    n_cases = args.batch_cases
    spec, built = _build_sweep(n_cases, 20261203)
    with ClockSampler(local) as clk:
        rec = _batch_record(N, built, spec, local, pg, ws, args.steps, args.warmup, args.tuning, clk)
    need = sum(N.Batch.case_bytes(ch) for _, ch in built)

    # each case against its own FP64 run
    accuracy = None
    if args.accuracy_steps:
        n_acc = args.accuracy_steps[-1]
        ba = N.Batch(device=local, arena_bytes=need + (64 << 20), max_cases=n_cases)
        sa = [ba.add(ch, c.delta_t) for c, ch in built]
        ba.step(n_acc)
        errs, diverged64, diverged32, per_case = [], [], [], []
        for k, ((c, ch), s) in enumerate(zip(built, sa)):
            s64 = N.Solver(ch, precision=N.LFM_FP64, device=local)
            s64.step(n_acc, c.delta_t)
            q64 = s64.get_state()
            s64.close()
            q32 = ba.get_state(s)
            f64, f32 = bool(np.all(np.isfinite(q64))), bool(np.all(np.isfinite(q32)))
            if not f64:
                diverged64.append(k)
            if not f32:
                diverged32.append(k)
            if f64 and f32:
                errs.append(acoustics.acoustic_rel_l2(q32, q64, ch.desc.gamma, c.dim, c.p_inf))
                # growth of the FP64 run's p' rms over the steps: a case on its
                # way to the divergence above amplifies every difference
                p0 = acoustics.pressure(ch.q0(), ch.desc.gamma, c.dim) - c.p_inf
                p1 = acoustics.pressure(q64, ch.desc.gamma, c.dim) - c.p_inf
                growth = float(np.sqrt(np.mean(p1 ** 2)) / max(np.sqrt(np.mean(p0 ** 2)), 1e-300))
                per_case.append({"case": k, "kind": spec[k]["kind"], "cells": ch.desc.n_cells,
                                 "scheme": "M1" if spec[k]["solver"] == 0 else "M2", "p_rel_l2": errs[-1],
                                 "p_rms_growth": growth})
        ba.close()
        accuracy = {"acoustic_p_rel_l2_max": max(errs) if errs else None,
                    "acoustic_p_rel_l2_median": float(np.median(errs)) if errs else None,
                    "cases_within_1e-3": int(sum(e <= 1e-3 for e in errs)),
                    "steps": n_acc, "cases_compared": len(errs),
                    "diverged_fp64": diverged64, "diverged_fp32_bulk": diverged32, "per_case": per_case,
                    "against": "each case's own FP64 device run (within 1e-12 of the oracle), same steps"}

    if rank != 0:
        return 0
    line = {
        "metric": METRIC, "value": rec["value"], "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": rec["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32-flux/f64-rk", "data": "synthetic (generated meshes and initial fields)",
        "config": {"workload": BATCH_DESC, "cases": rec["cases"], "cells": rec["cells"], "rk_stages": 5,
                   "precision": "fp32-bulk", "l2": "512 MB write between timed steps",
                   "parallelism": f"replicas x{ws}", "tuning": rec["tuning"],
                   "nonfinite_after_timed_steps": rec["nonfinite_after_timed_steps"]},
        "roofline": rec["roofline"],
        "plain_fp64": rec["plain_fp64"],
        "accuracy": accuracy,
        "cpu_baseline": None,
        "e2e": rec["e2e"],
        "gpu_launches": rec["launches_per_step"] * args.steps,
        "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)
    return 0


SERVE_DESC = ("Poisson request stream over a fixed window per rate: each request one of a library of cases (2D "
              "vortex grids, 2D cylinder O-grids, 3D cylinder sections, sweep quad/triangle cases; equal odds; cells "
              "log-uniform 10k-4M; seed 5150) with its own step count U(200,5000); FP32-bulk continuous batching "
              "with admission by arena footprint; a client queue bound sheds arrivals beyond it")


def serve_spec(n: int, seed: int, step_scale: float):
    """Cases of the request library: (kind, cells, steps, mach, solver, sub-seed)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        kind = ["vortex", "cylinder2d", "cylinder3d", "sweep"][int(rng.integers(0, 4))]
        cells = math.exp(rng.uniform(math.log(1e4), math.log(4e6)))
        steps = max(1, int(round(rng.uniform(200, 5000) * step_scale)))
        out.append(dict(kind=kind, cells=cells, steps=steps, mach=float(rng.uniform(0.1, 0.6)),
                        beta=float(rng.uniform(1, 5)), solver=int(rng.integers(0, 2)),
                        seed=int(rng.integers(0, 2 ** 31 - 1))))
    return out


def serve_case(sp: dict):
    from lfm_public_gb300 import cases
    cells = sp["cells"]
    if sp["kind"] == "vortex":
        return cases.vortex_case(n=max(16, int(round(math.sqrt(cells)))), mach=sp["mach"], beta=sp["beta"],
                                 solver=sp["solver"])
    if sp["kind"] == "cylinder2d":
        nr = max(12, int(round(math.sqrt(cells / 1.5))))
        return cases.cylinder_case(n_theta=int(1.5 * nr), n_r=nr, solver=sp["solver"], minmod=True)
    if sp["kind"] == "cylinder3d":
        s = (cells / (384 * 256 * 96)) ** (1.0 / 3.0)
        return cases.cylinder_case(n_theta=max(16, int(384 * s)), n_r=max(12, int(256 * s)),
                                   n_span=max(4, int(96 * s)), solver=1, reynolds=3900.0, noise=0.01,
                                   seed=sp["seed"] % 100000, minmod=False)
    sw = dict(kind="quad" if sp["seed"] % 2 == 0 else "tri", mach=sp["mach"], beta=sp["beta"],
              solver=sp["solver"], seed=sp["seed"])
    sw["n"] = max(8, int(round(math.sqrt(cells if sw["kind"] == "quad" else cells / 2))))
    return cases.sweep_case(sw)


def serve_stream(rate: float, window: float, n_lib: int, step_scale: float, seed: int):
    """Arrivals of one rate within the window: (time, library case, steps)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    out, t = [], 0.0
    while True:
        t += float(rng.exponential(1.0 / rate))
        if t >= window:
            return out
        out.append((t, int(rng.integers(0, n_lib)), max(1, int(round(rng.uniform(200, 5000) * step_scale)))))


def _serve_library(n: int, local: int):
    """The request library (cases and handles, set up in parallel threads) and
    each case's plain FP64 set-up, step and read-back times."""
    from concurrent.futures import ThreadPoolExecutor
    from lfm_public_gb300 import _native as N
    spec = serve_spec(n, 5150, 1.0)

    def one(sp):
        c = serve_case(sp)
        return c, N.CaseHandle.from_case(c)

    with ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        lib = list(ex.map(one, spec))
    return lib


def _fp64_times(lib, local):
    from lfm_public_gb300 import _native as N
    fp64 = []
    for c, ch in lib:
        t0 = time.perf_counter()
        s = N.Solver(ch, precision=N.LFM_FP64, device=local)
        s.sync()
        t1 = time.perf_counter()
        s.step(2, c.delta_t)
        s.sync()
        k = 10
        t2 = time.perf_counter()
        s.step(k, c.delta_t)
        s.sync()
        t3 = time.perf_counter()
        s.get_state()
        t4 = time.perf_counter()
        s.close()
        fp64.append((t1 - t0, (t3 - t2) / k, t4 - t3))
    return fp64


def _serve_rate(N, args, lib, fp64, rate, window, seed, local):
    """One Poisson stream of `rate` requests per second over `window` seconds
    into a server, and the same stream replayed on the FP64 server."""
    import numpy as np
    from concurrent.futures import ThreadPoolExecutor
    cells = [ch.desc.n_cells for _, ch in lib]
    arena = int(args.serve_arena_gb * (1 << 30))
    stream = serve_stream(rate, window, len(lib), args.serve_step_scale, seed)
    tuning = tuple(int(x) for x in args.serve_tuning.split(",")) if args.serve_tuning else None
    srv = N.Server(device=local, arena_bytes=arena, chunk_steps=args.serve_chunk, max_cases=args.serve_slots,
                   tuning=tuning, solo_cells=args.serve_solo_cells, max_solo=args.serve_max_solo)
    ids, shed, depth = {}, [], []
    t_start = time.perf_counter() + 0.2
    # times of the server clock (seconds since its creation) are read
    # from the request infos; the window ends `window` after the start
    t0_srv = srv.stats()["t_now"] + 0.2

    def submitter(part):
        for k in part:
            t, li, steps = stream[k]
            time.sleep(max(0.0, t_start + t - time.perf_counter()))
            if srv.stats()["queued"] >= args.serve_queue:
                shed.append(k)
                continue
            c, ch = lib[li]
            ids[k] = srv.submit(ch, c.delta_t, steps)

    nthreads = 8
    parts = [list(range(i, len(stream), nthreads)) for i in range(nthreads)]
    with ThreadPoolExecutor(max_workers=nthreads) as ex:
        futs = [ex.submit(submitter, p) for p in parts]
        st0 = srv.stats()
        while time.perf_counter() < t_start + window:
            st = srv.stats()
            depth.append(st["queued"] + st["running"])
            time.sleep(0.05)
        st_end = srv.stats()   # the device work of the window, finished requests or not
        for f in futs:
            f.result()
    t_end_srv = t0_srv + window
    lat, work_done = [], 0
    for k, rid in ids.items():
        info = srv.info(rid)
        if info["state"] == 2 and info["status"] == N.LFM_OK and info["t_done"] <= t_end_srv:
            lat.append(info["t_done"] - info["t_submit"])
            _, li, steps = stream[k]
            work_done += cells[li] * 5 * steps
    srv.close()
    # the FP64 server: first come, first served, one request at a time,
    # the same queue bound
    fin, lat64, work64, shed64, waiting = 0.0, [], 0, 0, []
    for t, li, steps in stream:
        waiting = [w for w in waiting if w > t]          # start times still ahead
        if len(waiting) >= args.serve_queue:
            shed64 += 1
            continue
        start = max(t, fin)
        fin = start + fp64[li][0] + steps * fp64[li][1] + fp64[li][2]
        waiting.append(start)
        if fin <= window:
            lat64.append(fin - t)
            work64 += cells[li] * 5 * steps
    return {
        "rate_per_s": rate, "window_s": window, "arrivals": len(stream), "shed": len(shed),
        "completed": len(lat), "throughput": work_done / window,
        "p50_s": float(np.percentile(lat, 50)) if lat else None,
        "p99_s": float(np.percentile(lat, 99)) if lat else None,
        "queue_depth_max": int(max(depth) if depth else 0),
        "queue_depth_mean": float(np.mean(depth)) if depth else 0.0,
        "device_busy_fraction": (st_end["busy_s"] - st0["busy_s"]) / window,
        "cell_stage_rate_in_window": (st_end["cell_stages"] - st0["cell_stages"]) / window,
        "cell_stage_rate_while_busy": ((st_end["cell_stages"] - st0["cell_stages"]) /
                                       max(st_end["busy_s"] - st0["busy_s"], 1e-9)),
        "fp64_serial": {"completed": len(lat64), "shed": shed64, "throughput": work64 / window,
                        "p50_s": float(np.percentile(lat64, 50)) if lat64 else None,
                        "p99_s": float(np.percentile(lat64, 99)) if lat64 else None},
    }


def _serve_config(args, lib, window, rates):
    return {"workload": SERVE_DESC, "library_cases": len(lib),
            "library_cells": int(sum(ch.desc.n_cells for _, ch in lib)), "step_scale": args.serve_step_scale,
            "arena_gb": args.serve_arena_gb, "chunk_steps": args.serve_chunk, "slots": args.serve_slots,
            "rates": rates, "tuning": args.serve_tuning or "batch default", "solo_cells": args.serve_solo_cells,
            "max_solo": args.serve_max_solo, "window_s": window, "client_queue_bound": args.serve_queue}


def run_serve(args):
    """Continuous batching of a Poisson request stream at several rates, each
    for a fixed window of wall time, against the same streams served one
    request at a time on the plain FP64 path.

    Every listed rate asks for more work than a GPU does (a request averages
    about 9e9 cell-stage updates), so both servers are saturated: the client
    sheds an arrival while --serve-queue requests already wait (both servers
    the same bound), and a request counts when it completes inside the window.
    Reported per rate: arrivals, shed, completed, throughput (cell-stage
    updates of the completed requests per second of window), p50 / p99 time
    to completion, queue depth, the server's busy fraction and the work it
    advanced in the window. The FP64 server's timeline is replayed from each
    library case's measured FP64 set-up, step and read-back times."""
    ws, rank, local, pg = _dist()
    from lfm_public_gb300 import _native as N
    lib = _serve_library(args.serve_library, local)
    fp64 = _fp64_times(lib, local)
    window = args.serve_window
    with ClockSampler(local) as clk:
        per_rate = []
        for ri, rate in enumerate(float(x) for x in args.serve_rates.split(",")):
            clk.mark()
            per_rate.append(_serve_rate(N, args, lib, fp64, rate, window, 77 + ri, local))
            clk.mark()
    if rank != 0:
        return 0
    best = max(per_rate, key=lambda r: r["throughput"])
    line = {
        "metric": METRIC, "value": best["throughput"], "unit": UNIT, "n_gpus": ws, "steps": None,
        "warmup": 0, "ms_per_step": None, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32-flux/f64-rk", "data": "synthetic (generated meshes and initial fields)",
        "config": _serve_config(args, lib, window, args.serve_rates),
        "serving": per_rate,
        "clocks": clk.summary(),
        "fp64_serial_note": "FP64 server: the same streams first come first served, one request at a time, the "
                            "same queue bound, timeline replayed from each library case's measured FP64 set-up, "
                            "step and read-back times",
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="cylinder2d", choices=sorted(WORKLOAD_DESC) + ["batch64", "serve"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp32"],
                    help="precision of the headline value (the other is reported beside it)")
    ap.add_argument("--accuracy-steps", default=None,
                    help="steps of the FP32-bulk vs FP64 comparison, comma-separated checkpoints (default: "
                         "20000,80000 for the 2D cylinder -- the configured run length, then long enough for the "
                         "start-up pulse to reach the r = 50 D ring; 1000 otherwise; 2000 for batch64; 0: none)")
    ap.add_argument("--no-wake", dest="wake", action="store_false",
                    help="skip the 3D wake sub-record of the 2D cylinder workloads")
    ap.add_argument("--wake-steps", type=int, default=10)
    ap.add_argument("--no-batch", dest="batch", action="store_false",
                    help="leave the 64-case batched sweep out of the default line")
    ap.add_argument("--batch-steps", type=int, default=20, help="timed steps of the batched sweep in the default line")
    ap.add_argument("--batch-cases", type=int, default=64)
    ap.add_argument("--tuning", default=None, help="batch launch shape block,items_per_thread,blocks_per_sm[,phased] "
                                                   "(default: autotuned)")
    ap.add_argument("--serve-rates", default="5,20,50,100,200", help="request arrival rates (1/s) of the serving stream")
    ap.add_argument("--serve-window", type=float, default=60.0, help="seconds of stream per rate")
    ap.add_argument("--serve-library", type=int, default=24, help="distinct cases the requests are drawn from")
    ap.add_argument("--serve-queue", type=int, default=16, help="client queue bound: arrivals beyond it are shed")
    ap.add_argument("--serve-step-scale", type=float, default=1.0, help="scales the U(200,5000) step counts")
    ap.add_argument("--serve-arena-gb", type=float, default=32.0)
    ap.add_argument("--serve-chunk", type=int, default=50)
    ap.add_argument("--serve-slots", type=int, default=8,
                    help="requests on the GPU at once (the server admits by arena footprint up to this many)")
    ap.add_argument("--no-serve", dest="serve", action="store_false",
                    help="leave the serving stream out of the default line")
    ap.add_argument("--serve-default-rate", type=float, default=20.0,
                    help="arrival rate (1/s) of the default line's serving stream")
    ap.add_argument("--serve-default-window", type=float, default=30.0,
                    help="seconds of the default line's serving stream")
    ap.add_argument("--serve-solo-cells", type=int, default=100000,
                    help="requests of at least this many cells run on their own single-case solver (0: none)")
    ap.add_argument("--serve-max-solo", type=int, default=4, help="solo requests on the GPU at once")
    ap.add_argument("--serve-tuning", default=None,
                    help="batch launch shape of the server block,items_per_thread,blocks_per_sm[,cooperative]")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--renumber", default="none", choices=["none", "rcm", "hilbert", "hpath"],
                    help="solver order of the cells (single-case workloads)")
    args = ap.parse_args()
    if args.accuracy_steps is None:
        args.accuracy_steps = {"batch64": "2000", "cylinder2d": "20000,80000",
                               "cylinder2d_m2": "20000,80000"}.get(args.workload, "1000")
    args.accuracy_steps = [int(x) for x in str(args.accuracy_steps).split(",") if int(x) > 0]
    if args.impl == "reference":
        if args.workload in ("batch64", "serve"):
            print(json.dumps({"impl": "reference", "unavailable": "the reference has no batched form; its CPU path is "
                              "timed per case with --workload cylinder2d / vortex2d"}), flush=True)
            return 0
        return run_reference(args)
    if args.workload == "batch64":
        return run_batch(args)
    if args.workload == "serve":
        return run_serve(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
