"""Benchmark of the GB300 hydro path: cell-updates per second, FP64.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference]

Workload: the 2-D Cartesian ideal-gas blast wave (256 x 256 on [0,1]^2,
gamma 5/3, PLM + MC limiter, HLLC, RK2, CFL 0.4, outflow, seeded +-1%
density noise, p = 10 inside r < 0.1) -- the reference's own CPU-runnable
configuration.  One benchmark step is one RK2 time step of the whole grid
(AdvanceStep + NextTimeStep); the default K = 100 steps is exactly the
configured run, restarted from the initial condition after the warm-up.

value     device-resident throughput: ps_run() replaying the captured graph,
          timed with CUDA events on the library's stream, L2 flushed (a
          256 MiB write) before each timed step.
e2e       the same metric through the drop-in AdvanceStep entry point with
          host arrays: per step a pinned host->device copy of Data.Vc,
          ps_advance_step(), a device->host copy, and NextTimeStep on the
          host, timed by the host clock.
roofline  of the fused stage kernel: algorithmic bytes 40*NVAR per
          cell-update split over its two launches, against the measured
          HBM copy bandwidth; the FP64 issue rate against a measured FP64
          FMA peak is reported beside it because the kernel is FP64-bound.
--impl reference   the CPU restatement of the reference (oracle/) on all
          host cores (independent runs, one per core), same metric.
"""
import argparse
import json
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

NX = 256
NVAR = 5
METRIC = "cell-updates/s (FP64 hydro step, 1 GB300)"
WORKLOAD = ("blast2d-256x256: 2-D Cartesian HD blast, PLM-MC, HLLC, RK2, CFL 0.4, outflow, "
            "gamma 5/3, seeded 1% density noise")
ALG_BYTES_PER_CELL_UPDATE = 40 * NVAR  # V^n read, V* write; V*, V^n read, V^{n+1} write
PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")


def _env_rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1"))


# ----------------------------------------------------------------------
# CPU side (oracle restatement of the reference)
# ----------------------------------------------------------------------

def _cpu_worker(args):
    nx, steps = args
    from oracle import Oracle
    o = Oracle(dims=2, nx=(nx, nx, 1))
    o.init_blast()
    t0 = time.perf_counter()
    o.run(steps)
    return time.perf_counter() - t0


def cpu_throughput(steps, procs=None):
    """Independent oracle runs of the workload, one per host core."""
    import multiprocessing as mp
    import oracle
    oracle.lib()  # build/load before forking workers
    n = procs or min(os.cpu_count() or 1, 64)
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(n) as pool:
        per = pool.map(_cpu_worker, [(NX, steps)] * n)
    wall = time.perf_counter() - t0
    cells = NX * NX * steps * n
    return {"value": cells / wall, "unit": "cell-updates/s", "cores": n, "kind": "port",
            "wall_s": wall,
            "sample": f"{n} independent runs of {steps} steps of the {NX}x{NX} blast "
                      f"(one per core), {sum(per):.1f} s of CPU work, wall {wall:.2f} s",
            "single_core_cell_updates_per_s": NX * NX * steps / statistics.median(per)}


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
        self.out = ""
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


def _read_traffic():
    """Per-launch DRAM bytes of the stage kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "stage_kernel_blast2d_256.md")
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].strip())
            except ValueError:
                return None
    return None


# ----------------------------------------------------------------------
# GPU side
# ----------------------------------------------------------------------

def gpu_bench(steps, warmup, rank, world):
    import numpy as np
    import torch
    import psgb

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    stream = torch.cuda.current_stream()
    cfg = psgb.make_config(dims=2, nx=(NX, NX, 1), limiter="mc", solver="hllc", bc="outflow",
                           cfl=0.4, cfl_max_var=1.1, tstop=10.0, first_dt=1e-4)
    grid = psgb.Grid(cfg)
    V0 = psgb.blast_state(cfg, grid)
    s = psgb.Solver(cfg, grid)
    s.set_stream(stream.cuda_stream)
    s.set_state(V0)
    s.set_time(0.0, 1e-4, 0)
    s.save()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    # warm-up steps, then restart from the initial condition
    for _ in range(warmup):
        flush.zero_()
        s.run(1)
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
            flush.zero_()
            starts[i].record(stream)
            s.run(1)
            ends[i].record(stream)
        torch.cuda.synchronize()
    launches = s.launches() - launches0
    flags = s.sync()
    ms = sum(a.elapsed_time(b) for a, b in zip(starts, ends))
    if dist:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
        dist.barrier()
    cells = NX * NX
    value = cells * steps * world / (ms * 1e-3)

    # kernel durations (one extra step, outside the timed region)
    s.restore()
    per_kernel = np.zeros(3)
    reps = 20
    for _ in range(reps):
        per_kernel += s.time_step_kernels()
    per_kernel /= reps
    stage_ms = 0.5 * (per_kernel[0] + per_kernel[1])

    # end-to-end through the drop-in entry point with pinned host buffers
    Vh = torch.from_numpy(V0.copy()).pin_memory()
    Vn = Vh.numpy()
    s.set_stream(0)
    s.set_time(0.0, 1e-4, 0)
    e2e_steps = steps
    t0 = time.perf_counter()
    dt, inv = 1e-4, 0.0
    for _ in range(e2e_steps):
        s.set_state(Vn)
        flags_e, inv = s.advance_step(dt, 0.0)
        s.get_state(out=Vn)
        dt_hyp = 1.0 / inv
        dt_hyp *= 0.4
        dt = min(dt_hyp, 1.1 * dt)
    e2e_wall = time.perf_counter() - t0
    bytes_state = int(V0.nbytes)

    out = {
        "metric": METRIC, "value": value, "unit": "cell-updates/s", "n_gpus": world,
        "steps": steps, "warmup": warmup, "ms_per_step": ms / steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded blast-wave initial condition of the reference config)",
        "config": {"workload": WORKLOAD, "cells": cells, "grid": [NX, NX],
                   "hydro_steps_per_bench_step": 1,
                   "l2": "256 MiB buffer written before every timed step (L2 flushed)",
                   "parallelism": "replicas only" if world > 1 else "single GPU"},
        "e2e": {"value": cells * e2e_steps / e2e_wall, "unit": "cell-updates/s",
                "h2d_bytes_per_step": bytes_state, "d2h_bytes_per_step": bytes_state,
                "path": "ps_set_state + ps_advance_step + ps_get_state per step (pinned host)"},
        "gpu_launches": int(launches),
        "device_flags": int(flags),
        "clocks": clk.summary(),
    }
    if rank == 0:
        peaks = json.load(open(PEAKS)) if os.path.exists(PEAKS) else {}
        hbm_peak = peaks.get("hbm_gbs", 6800.0)
        alg_bytes_launch = ALG_BYTES_PER_CELL_UPDATE / 2 * cells
        achieved = alg_bytes_launch / (stage_ms * 1e-3) / 1e9
        traffic = _read_traffic()
        out["roofline"] = {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                           "frac": achieved / hbm_peak, "traffic": traffic,
                           "kernel": "k_stage (fused PLM/Riemann/update, per stage launch)",
                           "stage_ms": [per_kernel[0], per_kernel[1]],
                           "finish_ms": per_kernel[2],
                           "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)"
                           if "hbm_gbs" in peaks else "fallback 6.8 TB/s (of fallback)"}
        fp64 = psgb.lib().ps_probe_fp64_flops(5)
        flops_cell_stage = _fp64_ops_per_cell_stage()
        out["roofline_fp64"] = {"peak": fp64 / 1e9, "unit": "GFLOP/s",
                                "peak_source": "ps_probe_fp64_flops (dependent FMA chains, "
                                               "measured on this GPU; 2 flops per FMA)"}
        if fp64 > 0 and flops_cell_stage:
            ach = flops_cell_stage * cells / (stage_ms * 1e-3)
            out["roofline_fp64"].update({"achieved": ach / 1e9, "frac": ach / fp64,
                                         "ops_per_cell_stage": flops_cell_stage})
        if world == 1:
            out["cpu_baseline"] = cpu_throughput(100)
        print(json.dumps(out), flush=True)
    if dist:
        dist.destroy_process_group()


def _fp64_ops_per_cell_stage():
    """Algorithmic FP64 operations per cell per stage, counted from the
    kernel source, or None if no count has been committed yet."""
    path = os.path.join(ROOT, "profiles", "stage_kernel_blast2d_256.md")
    if os.path.exists(path):
        for line in open(path):
            if line.startswith("fp64_ops_per_cell_stage:"):
                try:
                    return float(line.split(":", 1)[1].strip())
                except ValueError:
                    return None
    return None


def reference_bench(steps, warmup, rank, world):
    if rank != 0:
        return
    # bounded sample: every host core runs `steps` steps of the workload
    for _ in range(max(0, min(warmup, 1))):
        cpu_throughput(2)
    base = cpu_throughput(steps)
    out = {"metric": METRIC, "value": base["value"], "unit": "cell-updates/s", "n_gpus": world,
           "steps": steps, "warmup": warmup,
           "ms_per_step": base["wall_s"] / steps * 1e3,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (seeded blast-wave initial condition of the reference config)",
           "config": {"workload": WORKLOAD, "cells": NX * NX, "grid": [NX, NX]},
           "impl": "reference",
           "cpu_baseline": base,
           "e2e": {"value": base["value"], "unit": "cell-updates/s", "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    a = ap.parse_args()
    rank, world = _env_rank()
    if a.impl == "reference":
        reference_bench(a.steps, a.warmup, rank, world)
    else:
        gpu_bench(a.steps, max(a.warmup, 3), rank, world)


if __name__ == "__main__":
    main()
