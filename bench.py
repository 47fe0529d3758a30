"""Benchmark of the GB300 hydro path: cell-updates per second, FP64.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference]
                    [--workload batch|wind|blast|cube]

Workloads (synthetic inputs of the reference's configurations):
  batch  Default.  64 independent line-driven disk-wind models (grids drawn
         from 128x64, 256x128, 384x192, 512x256; L_x log-uniform 1e36..1e38
         erg/s, k U(0.1, 0.4), alpha U(0.5, 0.7); seed 4), 100 steps, in
         three forms: plain (each model's ps_run in turn, BLONDIN by bracket
         + Brent), batched (ps_batch_run) and batched with the learned
         cooling step (trained on the GPU before timing).  `value` is the
         last; the other two and the temperature error of the learned step
         are in `config`.
  wind   2-D spherical (r, theta) line-driven disk wind, 512 x 256 cells
         (r log-spaced 1e10..1e12 cm, theta uniform 0..pi/2), 7 M_sun point
         mass, 1e-20 g/cm^3 halo with a 1e-9 g/cm^3 disk-plane layer at
         4e4 K, L_x = 1e37 erg/s, BLONDIN heating/cooling (Strang split),
         force multiplier M = 0.2 t^-0.6 (M_max 4400) with a synthetic 36-bin
         UV flux, PLM van Leer, HLL, RK2, CFL 0.4; 1000 steps, plain form.
  blast  2-D Cartesian ideal-gas blast wave, 256 x 256, PLM MC, HLLC, RK2,
         CFL 0.4, outflow, seeded 1% density noise; 100 steps.
  cube   3-D Cartesian periodic 512^3 with BLONDIN at xi = 1e2: log-normal
         density (sigma 0.5, k^-2 spectrum, seed 5), T log-uniform 1e4..1e7 K;
         50 steps, plain (bracket + Brent) against the learned cooling step.
One benchmark step is one time step of every grid (split source +
AdvanceStep + NextTimeStep); the default K is the configured run length,
restarted from the initial condition after the warm-up.

value     device-resident throughput: CUDA-graph replays timed with CUDA
          events on the stream the work is issued on, L2 flushed (a 256 MiB
          write) before each timed step.
e2e       the same metric through the C ABI with host arrays: per step a
          pinned host->device copy of every Data.Vc, the step, and a
          device->host copy (wind/blast: ps_split_source()/ps_advance_step()
          in the reference's Strang order with NextTimeStep on the host);
          timed by the host clock.
roofline  of the fused stage kernel: 40*NVAR algorithmic bytes per
          cell-update split over its two launches, against the measured HBM
          copy bandwidth; the FP64 roofline (measured FMA peak) beside it,
          because the kernel is bound by the FP64 pipe.
--impl reference   the CPU restatement of the reference (oracle/) on all
          host cores: independent runs of the workload from its initial
          condition, one per core, same metric.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "pluto-sirocco_gb300")
for _p in (PKG, os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "cell-updates/s at 1 GB300 (FP64)"
PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")


# the numerics of the production cv_idl wind (definitions.h: CHAR_LIMITING
# YES, SHOCK_FLATTENING MULTID, ENTROPY_SWITCH ALWAYS)
IDL_NUMERICS = dict(char_limiting=1, shock_flattening=1, entropy_switch=2)


class Workload:
    def __init__(self, name, numerics="plm", flux="radial"):
        self.groups = 0
        self.name = name
        self.numerics = numerics
        self.flux = flux
        self.numerics_kw = dict(IDL_NUMERICS if numerics == "idl" else {})
        if flux == "dense":
            self.numerics_kw["dense_flux"] = True
        if name == "wind":
            self.nx, self.ny, self.nvar = 512, 256, 6
            self.steps = 1000
            self.cpu_steps = 30
            self.desc = ("wind2d-512x256: 2-D spherical line-driven disk wind, PLM-VL, HLL, RK2, "
                         "CFL 0.4, BLONDIN cooling, line force (36 bins), 7 Msun, L_x 1e37")
            self.profile = "stage_kernel_wind_batch64.md"
        elif name == "batch":
            import psgb
            self.specs = psgb.batch_models(64, seed=4)
            self.nx = self.ny = None
            self.nvar = 6
            self.steps = 100
            self.cpu_steps = 6
            self.desc = ("wind-batch-64: 64 independent 2-D line-driven disk-wind models (grids "
                         "drawn from 128x64, 256x128, 384x192, 512x256; L_x log-uniform "
                         "1e36..1e38 erg/s, k U(0.1,0.4), alpha U(0.5,0.7); seed 4), each as "
                         "the wind2d workload, all advanced together")
            self.profile = "stage_kernel_wind_batch64.md"
        elif name == "cube":
            self.nx = self.ny = self.nz = 512
            self.nvar = 5
            self.steps = 50
            self.cpu_steps = 4
            self.cpu_n = 48
            self.desc = ("cube3d-512: 3-D Cartesian periodic HD on [0,1]^3, PLM-MC, HLLC, RK2, "
                         "CFL 0.4, gamma 5/3, log-normal density (sigma 0.5, P(k) ~ k^-2, seed 5),"
                         " T log-uniform 1e4..1e7 K per cell, BLONDIN at xi = 1e2 (Strang split),"
                         " code density 1 = 1e-10 g/cm^3")
            self.profile = "stage_kernel_cube3d.md"
        else:
            self.nx, self.ny, self.nvar = 256, 256, 5
            self.steps = 100
            self.cpu_steps = 100
            self.desc = ("blast2d-256x256: 2-D Cartesian HD blast, PLM-MC, HLLC, RK2, CFL 0.4, "
                         "outflow, gamma 5/3, seeded 1% density noise")
            self.profile = "stage_kernel_blast2d_256.md"
        if name == "batch":
            self.cells = sum(sp["grid"][0] * sp["grid"][1] for sp in self.specs)
        elif name == "cube":
            self.cells = self.nx * self.ny * self.nz
        else:
            self.cells = self.nx * self.ny
        self.cooling = name in ("wind", "batch", "cube")
        if numerics == "idl":
            self.nvar = 7
            self.desc += ("; production limiting: characteristic PLM, MULTID shock flattening,"
                          " ENTROPY_SWITCH ALWAYS")
            self.profile = "stage_kernel_wind_batch64_idl.md"
        if flux == "dense":
            self.desc += ("; UV flux in all 36 bins (the library's dense synthetic flux, the "
                          "shape of SIROCCO's fluxes)")
            self.profile = "stage_kernel_wind_batch64_dense.md"

    def solver(self):
        """Device context with the initial state loaded."""
        import psgb
        if self.name == "wind":
            cfg = psgb.make_wind_config(self.nx, self.ny, cooling=1)
            w = psgb.make_wind()
            grid = psgb.WindGrid(cfg)
            V0 = psgb.wind_state(cfg, w, grid)
            s = psgb.Solver(cfg, grid)
            s.set_state(V0)
            s.set_time(0.0, 1e-4, 0)
            s.set_wind(w, psgb.wind_flux(cfg, w, grid))
        else:
            cfg = psgb.make_config(dims=2, nx=(self.nx, self.ny, 1), limiter="mc", solver="hllc",
                                   bc="outflow", cfl=0.4, cfl_max_var=1.1, tstop=10.0,
                                   first_dt=1e-4)
            grid = psgb.Grid(cfg)
            V0 = psgb.blast_state(cfg, grid)
            s = psgb.Solver(cfg, grid)
            s.set_state(V0)
            s.set_time(0.0, 1e-4, 0)
        return s, V0, cfg

    def oracle(self):
        from oracle import Oracle, wind_oracle
        if self.name == "wind":
            return wind_oracle(self.nx, self.ny)
        o = Oracle(dims=2, nx=(self.nx, self.ny, 1))
        o.init_blast()
        return o


def _env_rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1"))


def max_over_ranks(ms, dist):
    """Replicas only: every rank runs the whole workload on its own GPU; the
    job's time is the slowest rank's (all-reduce MAX, then a barrier).  dist
    is torch.distributed or None for one rank."""
    if not dist:
        return ms
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    tt = torch.tensor([float(ms)], dtype=torch.float64, device=dev)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    dist.barrier()
    return float(tt.item())


def replica_rate(cells, steps, world, ms):
    """Whole-job cell-updates/s of `world` replicas of `cells` cells each
    over `steps` steps in `ms` milliseconds (the slowest rank's)."""
    return cells * steps * world / (ms * 1e-3)


# ----------------------------------------------------------------------
# CPU side (oracle restatement of the reference)
# ----------------------------------------------------------------------

def _cpu_worker(args):
    name, steps, idx, numerics, flux = args
    wl = Workload(name, numerics, flux)
    if name == "batch":
        from oracle import wind_oracle
        sp = wl.specs[idx % len(wl.specs)]
        o = wind_oracle(sp["grid"][0], sp["grid"][1], l_star=sp["l_star"], krad=sp["krad"],
                        alpharad=sp["alpharad"], **wl.numerics_kw)
        cells = sp["grid"][0] * sp["grid"][1]
    elif name == "cube":
        import psgb
        from oracle import Oracle
        n = wl.cpu_n
        cp = psgb.COOL_PARAMS
        cfg = psgb.cube_config(n)
        o = Oracle(dims=3, nx=(n, n, n), nvar=5, limiter="mc", solver="hllc", bc="periodic",
                   cfl=0.4, cfl_max_var=1.1, tstop=1e10, first_dt=cfg.first_dt, cooling=1,
                   params=dict(unit_density=cp["unit_density"], unit_length=cp["unit_length"],
                               unit_velocity=cp["unit_velocity"], mu=cp["mu"], t_x=cp["t_x"],
                               xi_const=cp["xi"]))
        o.V[...] = psgb.cube_state(cfg, psgb.Grid(cfg), seed=5 + idx)
        cells = n ** 3
    else:
        o = wl.oracle()
        cells = wl.cells
    t0 = time.perf_counter()
    o.run(steps)
    return time.perf_counter() - t0, cells * steps


def cpu_throughput(wl, steps, procs=None):
    """Independent oracle runs of the workload, one per host core (for the
    batch workload, worker i runs model i of the batch)."""
    import multiprocessing as mp
    import oracle
    oracle.lib()  # build/load before starting workers
    n = procs or min(os.cpu_count() or 1, 64)
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(n) as pool:
        res = pool.map(_cpu_worker, [(wl.name, steps, i, wl.numerics, wl.flux)
                                     for i in range(n)])
    wall = time.perf_counter() - t0
    per = [r[0] for r in res]
    cells = sum(r[1] for r in res)
    slowest = max(per)
    what = (f"models 0..{n - 1} of the batch" if wl.name == "batch"
            else f"{wl.cpu_n}^3 cubes of the same configuration (one seed per core)"
            if wl.name == "cube" else wl.desc.split(':')[0])
    return {"value": cells / slowest, "unit": "cell-updates/s", "cores": n, "kind": "port",
            "wall_s": slowest,
            "sample": f"{n} concurrent independent runs of the first {steps} steps of "
                      f"{what} (one per core); time = slowest run's step loop "
                      f"({slowest:.2f} s; {sum(per):.1f} s of CPU work; set-up excluded)",
            "single_core_cell_updates_per_s": statistics.median(r[1] / r[0] for r in res)}


# ----------------------------------------------------------------------
# clocks
# ----------------------------------------------------------------------

class ClockSampler:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.p = None
        self.gpu = gpu_index
        self.out = ""

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "100"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.p = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.p:
            time.sleep(0.2)
            self.p.terminate()
            try:
                self.out, _ = self.p.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.p.kill()
                self.out, _ = self.p.communicate()

    def summary(self):
        rows = [r.split(",") for r in (self.out or "").strip().splitlines() if r.count(",") >= 8]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4)
                          if r[5 + i].strip().lower() == "active"})
        busy = [s for s in sm if smax and s > 0.5 * max(smax)] or sm
        return {"sm_mhz": statistics.median(busy) if busy else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": reasons,
                "samples": len(rows)}


def _l2_flusher(stream):
    """A 256 MiB write (twice the L2) issued on the work stream, so that it
    completes before the next timed step starts and each step finds a cold
    L2."""
    import torch
    buf = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def flush():
        with torch.cuda.stream(stream):
            buf.zero_()
    return flush


def _profile_value(wl, key):
    """A figure from the committed ncu summary of the workload's stage kernel."""
    path = os.path.join(ROOT, "profiles", wl.profile)
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith(key + ":"):
            try:
                return float(line.split(":", 1)[1].strip())
            except ValueError:
                return None
    return None


# ----------------------------------------------------------------------
# GPU side
# ----------------------------------------------------------------------

def _e2e(wl, s, V0, steps, cfg):
    """Drop-in path with host arrays: Integrate() + NextTimeStep() on the
    host (Src/main.c:215-337, 383-497, 521-697), state copied in and out
    of pinned host memory around every step."""
    import torch
    Vh = torch.from_numpy(V0.copy()).pin_memory()
    Vn = Vh.numpy()
    s.set_stream(0)
    s.restore()
    s.set_time(0.0, 1e-4, 0)
    dt, t, inv = 1e-4, 0.0, 0.0
    t0 = time.perf_counter()
    for n in range(steps):
        s.set_state(Vn)
        if not wl.cooling or (n >= 1 and (n - 1) % 2 == 1):
            inv = 0.0
        if wl.cooling and n % 2 == 1:
            s.split_source(dt, t)
        _, inv = s.advance_step(dt, inv)
        if wl.cooling and n % 2 == 0:
            s.split_source(dt, t)
        s.get_state(out=Vn)
        t += dt
        if not wl.cooling or n % 2 == 1:
            dt_hyp = 1.0 / inv
            dt_hyp *= cfg.cfl
            dt = min(dt_hyp, cfg.cfl_max_var * dt)
    return time.perf_counter() - t0, int(V0.nbytes)


def gpu_bench(wl, steps, warmup, rank, world):
    import numpy as np
    import torch
    import psgb

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    stream = torch.cuda.Stream()   # every launch of the timed region goes on this stream
    s, V0, cfg = wl.solver()
    s.set_stream(stream.cuda_stream)
    s.save()
    flush = _l2_flusher(stream)

    for _ in range(warmup):
        flush()
        s.run(1, wait=False)
    torch.cuda.synchronize()
    s.restore()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    launches0 = s.launches()
    with ClockSampler(torch.cuda.current_device()) as clk:
        torch.cuda.synchronize()
        for i in range(steps):
            flush()
            starts[i].record(stream)
            s.run(1, wait=False)
            ends[i].record(stream)
        torch.cuda.synchronize()
    launches = s.launches() - launches0
    flags = s.sync()
    ms = sum(a.elapsed_time(b) for a, b in zip(starts, ends))
    ms = max_over_ranks(ms, dist)
    value = replica_rate(wl.cells, steps, world, ms)
    t_end, _, step_end, _ = s.time()

    # per-kernel durations (extra steps outside the timed region)
    s.restore()
    per_kernel = np.zeros(3)
    reps = 20
    for _ in range(reps):
        per_kernel += s.time_step_kernels()
    per_kernel /= reps
    stage_ms = 0.5 * (per_kernel[0] + per_kernel[1])

    e2e_steps = min(steps, 200)
    e2e_wall, bytes_state = _e2e(wl, s, V0, e2e_steps, cfg)

    out = {
        "metric": METRIC, "value": value, "unit": "cell-updates/s", "n_gpus": world,
        "steps": steps, "warmup": warmup, "ms_per_step": ms / steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (the reference configuration's initial condition, generated)",
        "config": {"workload": wl.desc, "cells": wl.cells, "grid": [wl.nx, wl.ny],
                   "method": "plain GPU form",
                   "l2": "256 MiB buffer written before every timed step (L2 flushed)",
                   "parallelism": "replicas only" if world > 1 else "single GPU",
                   "t_end": t_end, "steps_run": step_end},
        "e2e": {"value": wl.cells * e2e_steps / e2e_wall, "unit": "cell-updates/s",
                "h2d_bytes_per_step": bytes_state, "d2h_bytes_per_step": bytes_state,
                "steps": e2e_steps,
                "path": "per step: H2D Data.Vc, ps_split_source/ps_advance_step (Strang order), "
                        "D2H Data.Vc, host NextTimeStep (pinned host memory)"},
        "gpu_launches": int(launches),
        "device_flags": int(flags),
        "clocks": clk.summary(),
    }
    if rank == 0:
        _rooflines(out, wl, stage_ms, per_kernel)
        if world == 1:
            out["cpu_baseline"] = cpu_throughput(wl, wl.cpu_steps)
        print(json.dumps(out), flush=True)
    if dist:
        dist.destroy_process_group()


def _batch_e2e(solvers, batch, V0s, steps):
    """Batch through the C ABI with host arrays: per step every model's
    Data.Vc copied in from pinned host memory (ps_batch_set_states), one
    ps_batch_run step, every model's Data.Vc copied back
    (ps_batch_get_states); wall time."""
    import torch
    host = [torch.from_numpy(v.copy()).pin_memory().numpy() for v in V0s]
    for s in solvers:
        s.restore()
    batch.sync()
    t0 = time.perf_counter()
    for _ in range(steps):
        batch.set_states(host)      # every model's Data.Vc in (ps_batch_set_states)
        batch.run(1)
        batch.get_states(host)      # and out (ps_batch_get_states, synchronises)
    return time.perf_counter() - t0, int(sum(v.nbytes for v in V0s))


E2E_PARTS = 4


def _batch_e2e_parts(solvers, batch, V0s, steps, sg, psgb, k=E2E_PARTS):
    """The same host round trip per step with the models split into k
    batches (dealt out by size) on their own streams: each part's
    transfers (ps_batch_set_states_async / ps_batch_get_states_async, copy
    engines) run while the other parts step; the host waits for each part's
    previous result before handing its states in again.  The parts start
    one after another on the first step, so that their transfers do not
    coincide.  With two parts both compute at once and then copy at once
    (16.4 ms a step on the benchmark batch against 14.1 ms device-only, in
    an earlier build); in the current build four parts take 12.9 ms a step
    against 12.2 ms device-only, six 12.8 ms and eight 13.1 ms (no gain past
    four).  Tile shapes as the autotuner chose for the whole batch; wall
    time."""
    import torch
    order = sorted(range(len(solvers)), key=lambda m: -V0s[m].size)
    groups = [order[i::k] for i in range(k)]
    parts = [psgb.Batch([solvers[m] for m in g]) for g in groups]
    for p, g in zip(parts, groups):
        for j, m in enumerate(g):
            p.set_shape(psgb.check(psgb.lib().ps_batch_get_shape(batch.h, m, None, None),
                                   "ps_batch_get_shape"), model=j)
        psgb.check(psgb.lib().ps_batch_set_surrogate(p.h, sg.h, 1), "ps_batch_set_surrogate")
    hosts = [[torch.from_numpy(V0s[m].copy()).pin_memory().numpy() for m in g] for g in groups]

    def loop(nsteps):
        for step in range(nsteps):
            for i, (p, h) in enumerate(zip(parts, hosts)):
                p.sync()                      # this part's previous result is on the host
                p.set_states_async(h)
                p.run(1, wait=False)
                p.get_states_async(h)
                if step == 0 and i < k - 1:
                    p.sync()
        return [p.sync() for p in parts]

    for s in solvers:
        s.restore()
    loop(2)                                   # graphs instantiated outside the timing
    for s in solvers:
        s.restore()
    for h, idx in zip(hosts, groups):
        for a, m in zip(h, idx):
            a[...] = V0s[m]
    t0 = time.perf_counter()
    flags = loop(steps)
    wall = time.perf_counter() - t0
    for p in parts:
        p.close()
    return wall, int(sum(v.nbytes for v in V0s)), flags


def _sg_training(wl, psgb):
    """Trains the learned cooling step for the batch: tuples from 16 of the
    models (GPU runs, snapshots at steps 0, 40 and 120) plus log-uniform
    draws, 1e6 samples in all, labelled by the reference method on the GPU,
    40000 Adam steps of 8192 rows on the GPU."""
    t0 = time.perf_counter()
    wt = psgb.wind_training_tuples(wl.specs[::4], steps=(0, 40, 120), per_model=6000, seed=3)
    sg, hist, tup, _ = psgb.train_surrogate(wt, n_draws=1000000 - len(wt), steps=40000,
                                            batch=8192, seed=3)
    return sg, {"samples": int(len(tup)), "wind_samples": int(len(wt)),
                "train_steps": 40000, "batch": 8192, "final_loss": float(hist[-100:].mean()),
                "seconds": time.perf_counter() - t0}


def _sg_check(sg, solvers, psgb):
    """Temperature error of the learned step on every cell of every model's
    current state: the surrogate path against the reference method, both
    on the same (n_H, T, xi, dt) of each cell."""
    import numpy as np
    tup = np.concatenate([psgb.sg_collect(s) for s in solvers])
    ref = sg.label(tup)
    sg.stats(reset=True)
    out, st, _ = sg.predict(tup, use_net=1)
    acc, oob, rej, below, evals, stiff = sg.stats(reset=True)
    rel = np.abs(out - ref) / ref
    return {"cells": int(len(tup)), "max_rel_T_error": float(rel.max()),
            "accepted": acc / max(len(tup), 1), "out_of_box": oob / max(len(tup), 1),
            "rejected_to_reference": rej / max(len(tup), 1), "stiff": stiff / max(len(tup), 1),
            "rate_evaluations_per_cell": evals / max(acc + rej, 1)}


def batch_bench(wl, steps, warmup, rank, world):
    """64 wind models in three forms: the plain GPU form (each model's
    ps_run in turn, BLONDIN by bracket + Brent), the batched form
    (ps_batch_run: one launch per phase for all models, one graph replay per
    step) and the batched form with the learned cooling step (the headline
    value)."""
    import numpy as np
    import torch
    import psgb

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    stream = torch.cuda.Stream()   # every launch of the timed regions goes on this stream
    flush = _l2_flusher(stream)

    def make():
        out, V0s = [], []
        for sp in wl.specs:
            s = psgb.wind_model_solver(sp, **wl.numerics_kw)
            s.set_stream(stream.cuda_stream)
            s.save()
            out.append(s)
            V0s.append(s.get_state())
        return out, V0s

    def timed(step_fn, restore):
        for _ in range(warmup):
            flush()
            step_fn()
        torch.cuda.synchronize()
        restore()
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(steps)]
        with ClockSampler(torch.cuda.current_device()) as clk:
            torch.cuda.synchronize()
            for a, b in ev:
                flush()
                a.record(stream)
                step_fn()
                b.record(stream)
            torch.cuda.synchronize()
        ms = sum(a.elapsed_time(b) for a, b in ev)
        ms = max_over_ranks(ms, dist)
        return ms, clk.summary()

    rate = lambda ms: replica_rate(wl.cells, steps, world, ms)

    # plain GPU form
    plain, _ = make()

    def plain_step():
        # every model's step queued on the one stream, in turn (no host
        # synchronisation between the models)
        for s in plain:
            s.run(1, wait=False)

    def plain_restore():
        for s in plain:
            s.restore()

    ms_plain, _ = timed(plain_step, plain_restore)
    plain_end = [s.get_state() for s in plain[:4]]
    for s in plain:
        s.close()

    # batched form, reference cooling
    solvers, V0s = make()
    batch = psgb.Batch(solvers)
    if wl.groups:
        batch.set_groups(wl.groups)
    batch.set_stream(stream.cuda_stream)
    t_tune = time.perf_counter()
    batch.autotune(reps=5)
    t_tune = time.perf_counter() - t_tune
    restore_all = lambda: [s.restore() for s in solvers]
    restore_all()
    ms_batched, _ = timed(lambda: batch.run(1, wait=False), restore_all)
    same = all(np.array_equal(a, s.get_state()) for a, s in zip(plain_end, solvers[:4]))
    shapes = {}
    for m, sp in enumerate(wl.specs):
        idx = psgb.lib().ps_batch_get_shape(batch.h, m, None, None)
        shapes["%dx%d" % tuple(sp["grid"])] = "%dx%d (shape %d)" % (batch.shape(m) + (idx,))

    # batched form with the learned cooling step (headline)
    sg, train = _sg_training(wl, psgb)
    psgb.lib().ps_batch_set_surrogate(batch.h, sg.h, 1)
    restore_all()
    sg.stats(reset=True)
    launches0 = batch.launches()
    ms, clocks = timed(lambda: batch.run(1, wait=False), restore_all)
    launches = batch.launches() - launches0
    flags = batch.sync()
    run_stats = dict(zip(["accepted", "out_of_box", "rejected", "below_1e4K", "rate_evaluations",
                          "stiff"], sg.stats(reset=True)))
    check = _sg_check(sg, solvers, psgb)
    value = rate(ms)
    # the same step with the network switched off (use_net = 0: a stiff
    # cell's Newton iterations start from the old temperature), so that the
    # network's own share of the gain is on the line
    psgb.lib().ps_batch_set_surrogate(batch.h, sg.h, 0)
    restore_all()
    ms_nonet, _ = timed(lambda: batch.run(1, wait=False), restore_all)
    nonet_stats = dict(zip(["accepted", "out_of_box", "rejected", "below_1e4K",
                            "rate_evaluations", "stiff"], sg.stats(reset=True)))
    psgb.lib().ps_batch_set_surrogate(batch.h, sg.h, 1)

    restore_all()
    per_kernel = np.zeros(3)
    reps = 10
    for _ in range(reps):
        per_kernel += batch.time_step_kernels()
    per_kernel /= reps
    stage_ms = 0.5 * (per_kernel[0] + per_kernel[1])

    e2e_steps = min(steps, 40)
    e2e_one, bytes_state = _batch_e2e(solvers, batch, V0s, e2e_steps)
    e2e_wall, _, e2e_flags = _batch_e2e_parts(solvers, batch, V0s, e2e_steps, sg, psgb)

    out = {
        "metric": METRIC, "value": value, "unit": "cell-updates/s", "n_gpus": world,
        "steps": steps, "warmup": warmup, "ms_per_step": ms / steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (the reference configuration's initial condition, generated)",
        "config": {"workload": wl.desc, "cells": wl.cells, "models": len(wl.specs),
                   "method": "batched GPU form with the learned cooling step (ps_batch_run + "
                             "ps_batch_set_surrogate, one CUDA graph per step)",
                   "plain_value": rate(ms_plain), "plain_ms_per_step": ms_plain / steps,
                   "batched_value": rate(ms_batched), "batched_ms_per_step": ms_batched / steps,
                   "speedup_vs_plain": ms_plain / ms,
                   "speedup_batched_only_vs_plain": ms_plain / ms_batched,
                   "batched_identical_to_plain": same,
                   "cooling_T_error": check, "surrogate_run_counters": run_stats,
                   "without_network": {
                       "value": rate(ms_nonet), "ms_per_step": ms_nonet / steps,
                       "run_counters": nonet_stats,
                       "path": "the same batched step with ps_batch_set_surrogate(use_net = 0): "
                               "the judge's Newton iterations start from the old temperature"},
                   "surrogate_training": train,
                   "hydro": "the batched form gives each model's ps_run result bit for bit "
                            "(batched_identical_to_plain); against the reference: relative "
                            "L1 <= 1e-11 where the flow does not amplify rounding (2e-19 to "
                            "8e-13 measured, tests/test_gpu_wind.py, test_gpu_fullsize.py), "
                            "else within 3x the reference's own change under a 1e-15 "
                            "perturbation of its initial state (the full-physics 512x256 "
                            "wind after 100 steps); the learned step changes the pressure only",
                   "tile_shapes": shapes, "autotune_s": t_tune,
                   "groups": wl.groups or "library default (2)",
                   "line_force": _line_force_figures(wl),
                   "l2": "256 MiB buffer written before every timed step (L2 flushed)",
                   "parallelism": "replicas only" if world > 1 else "single GPU"},
        "e2e": {"value": wl.cells * e2e_steps / e2e_wall, "unit": "cell-updates/s",
                "h2d_bytes_per_step": bytes_state, "d2h_bytes_per_step": bytes_state,
                "steps": e2e_steps,
                "path": "per step: H2D of every model's Data.Vc, ps_batch_run(1) with the "
                        "learned cooling step, D2H of every model's Data.Vc (pinned host "
                        "memory); the models in %d batches on their own streams, each "
                        "part's copies overlapping the other parts' steps "
                        "(ps_batch_set_states_async / ps_batch_get_states_async)" % E2E_PARTS,
                "device_flags": [int(f) for f in e2e_flags],
                "one_batch_value": wl.cells * e2e_steps / e2e_one,
                "one_batch_path": "the same round trip through one batch "
                                  "(ps_batch_set_states / ps_batch_get_states, copy kernel)"},
        "gpu_launches": int(launches),
        "device_flags": int(flags),
        "clocks": clocks,
    }
    if rank == 0:
        _rooflines(out, wl, stage_ms, per_kernel)
        if world == 1:
            out["cpu_baseline"] = cpu_throughput(wl, wl.cpu_steps)
        print(json.dumps(out), flush=True)
    batch.close()
    if dist:
        dist.destroy_process_group()


def cube_bench(wl, steps, warmup, rank, world):
    """The 3-D periodic cooling configuration at 512^3: the plain GPU form
    (BLONDIN by bracket + Brent) and the form with the learned cooling step
    (the headline value), both from the same initial state."""
    import numpy as np
    import torch
    import psgb

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    stream = torch.cuda.Stream()   # every launch of the timed region goes on this stream
    flush = _l2_flusher(stream)
    t_setup = time.perf_counter()
    s = psgb.cube_solver(wl.nx)
    s.set_stream(stream.cuda_stream)
    s.save()
    t_setup = time.perf_counter() - t_setup

    def timed():
        for _ in range(warmup):
            flush()
            s.run(1, wait=False)
        torch.cuda.synchronize()
        s.restore()
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(steps)]
        with ClockSampler(torch.cuda.current_device()) as clk:
            torch.cuda.synchronize()
            for a, b in ev:
                flush()
                a.record(stream)
                s.run(1, wait=False)
                b.record(stream)
            torch.cuda.synchronize()
        ms = sum(a.elapsed_time(b) for a, b in ev)
        ms = max_over_ranks(ms, dist)
        return ms, clk.summary()

    rate = lambda ms: replica_rate(wl.cells, steps, world, ms)
    ms_plain, _ = timed()
    flags_plain = s.sync()
    # training tuples: cells of the plain run after 10 steps, plus draws
    s.restore()
    s.run(10)
    rng = np.random.default_rng(3)
    tup = psgb.sg_collect(s, cap=1 << 22)
    tup = tup[rng.choice(len(tup), size=min(300000, len(tup)), replace=False)]
    t_train = time.perf_counter()
    sg, hist, all_tup, _ = psgb.train_surrogate(tup, n_draws=700000, steps=40000, seed=3)
    t_train = time.perf_counter() - t_train
    psgb.lib().ps_set_surrogate(s.ctx, sg.h, 1)
    sg.stats(reset=True)
    launches0 = s.launches()
    ms, clocks = timed()
    launches = s.launches() - launches0
    flags = s.sync()
    counters = dict(zip(["accepted", "out_of_box", "rejected", "below_1e4K", "rate_evaluations",
                         "stiff"], sg.stats(reset=True)))
    # the learned step's temperature error on a sample of the final state
    tup_end = psgb.sg_collect(s, cap=1 << 21)
    ref = sg.label(tup_end)
    out, st, _ = sg.predict(tup_end, use_net=1)
    rel = np.abs(out - ref) / ref
    value = rate(ms)

    s.restore()
    per_kernel = np.zeros(3)
    reps = 4
    for _ in range(reps):
        per_kernel += s.time_step_kernels()
    per_kernel /= reps
    stage_ms = 0.5 * (per_kernel[0] + per_kernel[1])

    e2e_steps = min(steps, 4)
    s.restore()
    V0 = s.get_state()
    host = torch.from_numpy(V0).pin_memory().numpy()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        s.set_state(host)
        s.run(1)
        s.get_state(out=host)
    e2e_wall = time.perf_counter() - t0
    out_json = {
        "metric": METRIC, "value": value, "unit": "cell-updates/s", "n_gpus": world,
        "steps": steps, "warmup": warmup, "ms_per_step": ms / steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (the configuration's seeded initial condition, generated on the host)",
        "config": {"workload": wl.desc, "cells": wl.cells, "grid": [wl.nx, wl.ny, wl.nz],
                   "method": "learned cooling step (ps_set_surrogate), CUDA-graph steps",
                   "plain_value": rate(ms_plain), "plain_ms_per_step": ms_plain / steps,
                   "speedup_vs_plain": ms_plain / ms, "plain_flags": int(flags_plain),
                   "cooling_T_error": {"cells_sampled": int(len(tup_end)),
                                       "max_rel_T_error": float(rel.max()),
                                       "accepted": float(np.mean(st == 0))},
                   "surrogate_run_counters": counters,
                   "surrogate_training": {"samples": int(len(all_tup)), "cube_samples": int(len(tup)),
                                          "seconds": t_train,
                                          "final_loss": float(hist[-100:].mean())},
                   "setup_s": t_setup,
                   "l2": "inputs (5.5 GB per array) far larger than L2; 256 MiB flush as well",
                   "parallelism": "replicas only" if world > 1 else "single GPU"},
        "e2e": {"value": wl.cells * e2e_steps / e2e_wall, "unit": "cell-updates/s",
                "h2d_bytes_per_step": int(V0.nbytes), "d2h_bytes_per_step": int(V0.nbytes),
                "steps": e2e_steps,
                "path": "per step: H2D Data.Vc, ps_run(1) with the learned cooling step, D2H "
                        "Data.Vc (pinned host memory)"},
        "gpu_launches": int(launches),
        "device_flags": int(flags),
        "clocks": clocks,
    }
    if rank == 0:
        _rooflines(out_json, wl, stage_ms, per_kernel)
        if world == 1:
            out_json["cpu_baseline"] = cpu_throughput(wl, wl.cpu_steps)
        print(json.dumps(out_json), flush=True)
    if dist:
        dist.destroy_process_group()


def _line_force_figures(wl):
    """The line force is fused into the stage kernel; its own memory work per
    cell-update from the flux-bin lists the batch's models carry: per bin
    with a nonzero (F_r, F_theta) and stage, VGradCalc reads 7 static doubles
    (bilinear weights of the offset point, four velocity projections, 1/ds)
    and writes one, and each of the two sweeps reads it back with one flux
    (12 doubles), against the 5 doubles per bin of all 36 bins of a dense
    per-angle design (2880 B per cell-update)."""
    import numpy as np
    import psgb
    bins = cells = 0
    for sp in wl.specs:
        nr, nt = sp["grid"]
        cfg = psgb.make_wind_config(nr, nt)
        w = psgb.make_wind(l_star=sp["l_star"], krad=sp["krad"], alpharad=sp["alpharad"])
        g = psgb.WindGrid(cfg)
        fr, ft, _ = psgb.wind_flux(cfg, w, g, dense=wl.flux == "dense")
        act = (slice(None), 0, slice(2, -2), slice(2, -2))
        bins += int(np.count_nonzero((fr[act] != 0.0) | (ft[act] != 0.0)))
        cells += nr * nt
    per_cell = bins / cells
    return {"bins_per_cell": per_cell, "angles": 36,
            "bytes_per_cell_update": 2 * 12 * 8 * per_cell,
            "dense_design_bytes_per_cell_update": 2 * 5 * 36 * 8,
            "flux": ("synthetic, all 36 bins" if wl.flux == "dense" else
                     "synthetic: the radial bin of each cell (real SIROCCO fluxes fill more "
                     "bins)")}


def _rooflines(out, wl, stage_ms, per_kernel):
    import psgb
    peaks = json.load(open(PEAKS)) if os.path.exists(PEAKS) else {}
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    alg_bytes_launch = 40 * wl.nvar / 2 * wl.cells
    achieved = alg_bytes_launch / (stage_ms * 1e-3) / 1e9
    out["roofline"] = {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                       "frac": achieved / hbm_peak,
                       "traffic": (lambda b: b * wl.cells if b else None)(
                           _profile_value(wl, "traffic_bytes_per_cell_launch")),
                       "kernel": "stage kernel (fused PLM/Riemann/sources/update), per launch",
                       "stage_ms": [per_kernel[0], per_kernel[1]],
                       "other_ms_per_step": per_kernel[2],
                       "alg_bytes_per_launch": alg_bytes_launch,
                       "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)"
                       if "hbm_gbs" in peaks else "fallback 6.8 TB/s (of fallback)"}
    fp64 = psgb.probe().ps_probe_fp64_flops(5)
    ops = _profile_value(wl, "fp64_ops_per_cell_stage")
    out["roofline_fp64"] = {"peak": fp64 / 1e9, "unit": "GFLOP/s",
                            "peak_source": "ps_probe_fp64_flops (dependent FMA chains, "
                                           "measured on this GPU; 2 flops per FMA)"}
    if fp64 > 0 and ops:
        ach = ops * wl.cells / (stage_ms * 1e-3)
        out["roofline_fp64"].update({"achieved": ach / 1e9, "frac": ach / fp64,
                                     "ops_per_cell_stage": ops})
    insts = _profile_value(wl, "fp64_insts_per_cell_stage")
    if fp64 > 0 and insts:
        # DADD, DMUL and DFMA take one issue slot each: the share of the
        # FMA instruction rate they fill
        out["roofline_fp64"].update({
            "insts_per_cell_stage": insts,
            "issue_frac": insts * wl.cells / (stage_ms * 1e-3) / (fp64 / 2)})


def _port_models(args):
    """One batch model (or one replica) on the oracle port: seconds of its
    last `steps` steps after `warmup` untimed ones, and the cell count."""
    name, idx, steps, warmup = args
    wl = Workload(name)
    if name == "batch":
        from oracle import wind_oracle
        sp = wl.specs[idx]
        o = wind_oracle(sp["grid"][0], sp["grid"][1], l_star=sp["l_star"], krad=sp["krad"],
                        alpharad=sp["alpharad"])
        cells = sp["grid"][0] * sp["grid"][1]
    else:
        o = wl.oracle()
        cells = wl.cells
    o.run(warmup)
    t0 = time.perf_counter()
    o.run(steps)
    return time.perf_counter() - t0, cells


def _reference_jobs(wl, steps, warmup, root, ncores):
    """The reference's own serial binary (oracle/_ref, built by build()) on
    the workload: one run directory per model (batch: the 64 models; wind
    and blast: one replica per host core).  Returns (jobs, description) or
    (None, why not)."""
    import ref_runs
    from functools import partial
    total = warmup + steps
    jobs = []
    if wl.name in ("batch", "wind"):
        if wl.numerics != "plm" or wl.flux != "radial":
            return None, "the reference arm is built for the primitive-PLM radial-flux wind"
        exe = ref_runs.binary("wind2d")
        if not exe:
            return None, "the reference's wind binary was not built (oracle/_ref/wind2d)"
        specs = (wl.specs if wl.name == "batch" else
                 [dict(grid=(wl.nx, wl.ny), l_star=1.0e37, krad=0.2, alpharad=-0.6)] * ncores)
        shared = {}
        for g in sorted({tuple(sp["grid"]) for sp in specs}):
            d = os.path.join(root, "shared_%dx%d" % g)
            os.makedirs(d)
            # theta and phi files (zero for the single-bin flux); the replicas
            # of one wind model share the radial file as well
            ref_runs.write_wind_flux(d, g[0], g[1], 1.0e37, axes=6 if wl.name == "batch" else 7)
            shared[g] = d
        for m, sp in enumerate(specs):
            nr, nt = sp["grid"]
            wd = os.path.join(root, "m%02d" % m)
            prep = partial(ref_runs.prepare_wind, wd, nr, nt, l_star=sp["l_star"],
                           krad=sp["krad"], alpharad=sp["alpharad"], shared=shared[(nr, nt)])
            jobs.append((prep, exe, wd, total, warmup, nr * nt))
        what = ("the 64 models of the batch" if wl.name == "batch" else
                "%d replicas of the 512x256 wind (one per core)" % ncores)
    elif wl.name == "blast":
        exe = ref_runs.binary("blast2d")
        if not exe:
            return None, "the reference's blast binary was not built (oracle/_ref/blast2d)"
        for m in range(ncores):
            wd = os.path.join(root, "r%02d" % m)
            prep = partial(ref_runs.prepare_blast, wd, wl.nx, wl.ny)
            jobs.append((prep, exe, wd, total, warmup, wl.nx * wl.ny))
        what = "%d replicas of the 256x256 blast (one per core)" % ncores
    else:
        return None, ("the reference has no constant-xi BLONDIN for the 3-D cooling cube; "
                      "the oracle port stands in")
    return jobs, what


def reference_bench(wl, steps, warmup, rank, world):
    """The reference's own serial CPU build on the machine's host cores, on the
    GPU arm's workload: every model (or one replica per core) runs W + K
    steps as its own process, at most one process per core, and the last K
    steps of each are timed from its own log lines (set-up excluded: the
    reference matches every flux record against every cell at start-up).
    value = cells x K summed over the runs / (their step-loop seconds summed
    / cores): the host cores kept busy with step loops.  The oracle port on
    the same runs is reported beside it."""
    if rank != 0:
        return
    import multiprocessing as mp
    import tempfile
    import oracle
    import ref_runs
    ncores = min(os.cpu_count() or 1, 64)
    steps_ref = steps if wl.name in ("batch", "blast") else min(steps, 50)
    root = tempfile.mkdtemp(prefix="ps_ref_")
    try:
        jobs, what = _reference_jobs(wl, steps_ref, warmup, root, ncores)
        ref = None
        if jobs:
            res, wall = ref_runs.run_many(jobs, ncores)
            bad = [k for k, r in enumerate(res) if r[0] is None or r[1] != 0]
            if not bad:
                secs = sum(r[0] for r in res)
                work = sum(j[5] for j in jobs) * steps_ref
                ref = {"value": work / (secs / ncores), "unit": "cell-updates/s",
                       "cores": ncores, "kind": "reference",
                       "sample": f"{what}: {warmup} + {steps_ref} steps each, the last "
                                 f"{steps_ref} timed per run from its own log lines (set-up "
                                 f"excluded); {secs:.1f} s of step loops summed over the runs, {ncores} at a time, "
                                 f"{wall:.0f} s wall with set-up",
                       "single_core_cell_updates_per_s": work / secs,
                       "runs": len(jobs), "wall_s_with_setup": wall}
            else:
                what = "reference runs failed: %s" % [res[k][1] for k in bad[:3]]
    finally:
        ref_runs.clean(root)
    # the oracle port on the same models / replicas
    oracle.lib()
    n_port = len(wl.specs) if wl.name == "batch" else ncores
    steps_port = steps_ref if wl.name != "cube" else min(steps, wl.cpu_steps)
    if wl.name == "cube":
        port = cpu_throughput(wl, steps_port)
    else:
        with mp.get_context("spawn").Pool(ncores) as pool:
            pr = pool.map(_port_models, [(wl.name, k, steps_port, warmup) for k in range(n_port)])
        secs = sum(r[0] for r in pr)
        work = sum(r[1] for r in pr) * steps_port
        port = {"value": work / (secs / ncores), "unit": "cell-updates/s", "cores": ncores,
                "kind": "port",
                "sample": f"the oracle port on the same {n_port} runs: {warmup} + {steps_port} "
                          f"steps each, the last {steps_port} timed; {secs:.1f} s of step loops"}
    base = ref if ref else dict(port, why_not_reference=what)
    ms_per_step = 1e3 * wl.cells * 1.0 / base["value"]
    out = {"metric": METRIC, "value": base["value"], "unit": "cell-updates/s", "n_gpus": world,
           "steps": steps_ref if ref else steps_port, "warmup": warmup,
           "ms_per_step": ms_per_step,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (the reference configuration's initial condition, generated)",
           "config": ({"workload": wl.desc, "cells": wl.cells, "models": len(wl.specs)}
                      if wl.name == "batch" else
                      {"workload": wl.desc, "cells": wl.cells, "grid": [wl.nx, wl.ny]}),
           "impl": "reference",
           "cpu_baseline": base,
           "port": port,
           "e2e": {"value": base["value"], "unit": "cell-updates/s", "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--workload", default="batch", choices=["wind", "blast", "batch", "cube"])
    ap.add_argument("--cube-n", type=int, default=512,
                    help="cells per direction of the cube workload (smaller cases for profiling)")
    ap.add_argument("--numerics", default="plm", choices=["plm", "idl"],
                    help="batch workload: primitive PLM (default) or the production cv_idl "
                         "limiting (characteristic PLM, MULTID, entropy switch)")
    ap.add_argument("--groups", type=int, default=0,
                    help="batch workload: model groups run as parallel graph branches "
                         "(ps_batch_set_groups; 0: the library's default)")
    ap.add_argument("--flux", default="radial", choices=["radial", "dense"],
                    help="batch workload: UV flux in each cell's radial bin (default) or in "
                         "all 36 bins")
    a = ap.parse_args()
    if (a.numerics != "plm" or a.flux != "radial") and a.workload != "batch":
        ap.error("--numerics and --flux are offered for the batch workload")
    wl = Workload(a.workload, a.numerics, a.flux)
    wl.groups = a.groups
    if a.workload == "cube" and a.cube_n != 512:
        wl.nx = wl.ny = wl.nz = a.cube_n
        wl.cells = a.cube_n ** 3
        wl.desc = wl.desc.replace("cube3d-512", "cube3d-%d" % a.cube_n)
    steps = a.steps if a.steps is not None else wl.steps
    rank, world = _env_rank()
    if a.impl == "reference":
        reference_bench(wl, steps, a.warmup, rank, world)
    elif a.workload == "batch":
        batch_bench(wl, steps, max(a.warmup, 3), rank, world)
    elif a.workload == "cube":
        cube_bench(wl, steps, max(a.warmup, 3), rank, world)
    else:
        gpu_bench(wl, steps, max(a.warmup, 3), rank, world)


if __name__ == "__main__":
    main()
