#!/usr/bin/env python
"""Benchmark: Gcell-updates/s of the TMz FDTD step on the 8192^2 production shot.

Workload (one GPU): 8192 x 8192 grid, dx = dy = 0.25 mm, Courant 0.99, 32-cell
CPML, 16-element phased array on x = 64 (pitch 5 cells) at 50 GHz steered to
15 degrees with a 2 ns raised-cosine ramp, tanh plasma 1.5e19 (1 + tanh((x -
5000)/600)) m^-3 times (1 + 0.05 g), g a seeded Gaussian random field
(correlation length 40 cells, seed 1001), nu = 2e9 1/s, 16 co-located Ez
detectors with a 50 GHz FP64 running DFT.  Synthetic inputs of that shape.

A bench "step" is a block of --block FDTD time steps of that shot (default
100).  `value` is device-timed (CUDA events on the shot's stream) with the
fields resident in HBM; the working set (2.4 GB touched per time step) is far
larger than L2, so no flush is needed between blocks.  `e2e` runs whole
shots of --e2e-steps time steps through the C ABI from host buffers:
fdtd2d_create (uploads maps/tables), fdtd2d_run, fdtd2d_read_traces and
fdtd2d_read_dft (downloads results), fdtd2d_destroy.

--impl reference times the reference's algorithm on the host cores (the
FP32 CPU restatement in oracle/, all threads) on the same shot, one time step
per bench step.

Under torchrun with N ranks every rank advances its own replica of the shot
(the path has no data-path exchange: replicas only); value = all ranks'
cell updates / the slowest rank's time.
"""
from __future__ import annotations

import argparse
import csv
import io
import json
import os
import re
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

BYTES_PER_CELL = 36  # read+write Ez, Hx, Hy, Jz (32 B) + plasma drive (4 B)
METRIC = "Gcell-updates/s"
UNIT = "Gcell/s"


def dist_setup(n_gpus: int):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist

        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
        return world, rank, local, dist
    return 1, 0, 0, None


def barrier(dist):
    if dist is not None:
        dist.barrier()


def allreduce_max(dist, x: float) -> float:
    if dist is None:
        return x
    import torch

    dev = "cuda" if torch.cuda.is_available() and dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def allreduce_sum(dist, x: float) -> float:
    if dist is None:
        return x
    import torch

    dev = "cuda" if torch.cuda.is_available() and dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.tmp = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.tmp, stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.tmp.flush()
        self.tmp.seek(0)
        rows = [r for r in csv.reader(io.StringIO(self.tmp.read())) if len(r) >= 9]
        sm, smax, power = [], [], []
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
                power.append(float(r[3]))
            except ValueError:
                continue
            for k, name in enumerate(names):
                if "Active" in r[5 + k] and "Not" not in r[5 + k]:
                    reasons.add(name)
        out = {"sm_mhz": statistics.median(sm) if sm else None,
               "sm_max_mhz": max(smax) if smax else None,
               "reasons": sorted(reasons), "samples": len(sm)}
        if power:
            out["power_w_max"] = max(power)
        return out


def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except Exception:
            pass
    return {}


def profile_traffic() -> float | None:
    """DRAM bytes per launch of the step kernel on this workload, from the
    committed ncu summary (scaled to the full launch as stated there)."""
    f = ROOT / "profiles" / "step_tma_8192_production.md"
    if not f.exists():
        return None
    m = re.search(r"traffic_bytes_per_launch:\s*([0-9.eE+]+)", f.read_text())
    return float(m.group(1)) if m else None


def workload_config(args) -> dict:
    return {"workload": f"{args.size}x{args.size} TMz phased-array reflectometry shot: 32-cell CPML, "
                        "tanh x GRF plasma, nu 2e9/s, 16 elements at 50 GHz steered 15 deg, 16 Ez "
                        "detectors + FP64 DFT",
            "nx": args.size, "ny": args.size, "npml": 32, "shot_steps": 20000, "block_steps": args.block,
            "dx_mm": 0.25, "courant": 0.99, "bytes_per_cell_update": BYTES_PER_CELL,
            "l2": "no flush: 2.4 GB touched per time step >> 129 MB L2",
            "parallelism": f"replicas x{args.gpus}"}


def make_problem(n_steps: int, size: int):
    import fdtd_2d_gb300 as F

    kw = {}
    if size != 8192:
        kw = dict(nx=size, ny=size, x_center=size * 5000 / 8192, src_j=size // 2 - 37, det_j=size // 2 - 37)
    return F.Problem.from_spec(F.production_spec(n_steps=n_steps, **kw))


def cpu_baseline(prob, seconds: float, threads: int | None = None) -> dict:
    """FP32 oracle restatement on the host cores, bounded to ~`seconds`."""
    import oracle as O

    if threads:
        O.set_threads(threads)
    cores = O.threads()
    o = O.Oracle(prob.setup_ptr, fp32=True)
    cells = prob.nx * prob.ny
    o.run(1, 1)  # warm-up
    t = time.perf_counter()
    o.run(2, 2)
    per = max(time.perf_counter() - t, 1e-6)
    n = max(2, min(int(seconds / per), prob.n_steps - 3))
    t = time.perf_counter()
    o.run(3, 2 + n)
    dt = time.perf_counter() - t
    o.close()
    return {"value": cells * n / dt / 1e9, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{n} time steps of the {prob.nx}x{prob.ny} shot (FP32 restatement, OpenMP)"}


def run_reference(args, world, rank, dist) -> None:
    if rank != 0:
        return
    import oracle as O

    prob = make_problem(max(args.steps + args.warmup + 2, 10), args.size)
    cores = O.threads()
    o = O.Oracle(prob.setup_ptr, fp32=True)
    cells = prob.nx * prob.ny
    o.run(1, args.warmup)
    t = time.perf_counter()
    o.run(args.warmup + 1, args.warmup + args.steps)
    dt = time.perf_counter() - t
    value = cells * args.steps / dt / 1e9
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "impl": "reference", "config": dict(workload_config(args), block_steps=1),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{args.steps} time steps of the {prob.nx}x{prob.ny} shot per run "
                                       "(one time step per bench step), FP32 restatement of the "
                                       "reference update equations, OpenMP over rows"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args, world, rank, local, dist) -> None:
    import fdtd_2d_gb300 as F

    S, K, W = args.block, args.steps, args.warmup
    total_steps = (W + K) * S
    prob = make_problem(max(20000, total_steps), args.size)
    cells = prob.nx * prob.ny
    shot = F.Shot(prob, device=local)
    shot.run(1, W * S)
    shot.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    barrier(dist)
    shot.synchronize()
    launches0 = shot.launches()
    kernel = shot.kernel_name()
    ms = shot.run_timed(W * S + 1, W * S + K * S)  # one event pair around the K blocks
    shot.synchronize()
    barrier(dist)
    launches = shot.launches() - launches0
    clk = clocks.stop()
    ok = shot.check_finite()
    shot.close()
    t_max = allreduce_max(dist, ms / 1e3)
    units = allreduce_sum(dist, float(cells) * S * K)
    value = units / t_max / 1e9

    # roofline of the step kernel (one launch per time step on this workload)
    per_launch_s = (ms / 1e3) / (K * S)
    achieved = BYTES_PER_CELL * cells / per_launch_s / 1e9
    peaks = measured_peaks()
    peak = peaks.get("hbm_gbs")
    peak_src = "measured"
    if not peak:
        peak, peak_src = 6800.0, "fallback"
    traffic = profile_traffic()

    # end to end through the C ABI with host buffers
    e2e = None
    if args.e2e_steps > 0:
        eprob = make_problem(args.e2e_steps, args.size)
        s = eprob.setup
        h2d = cells * 4 + 16 * 4 * s.npml + 4 * 2 * (s.nx + s.ny) + 4 * (s.n_steps + 1) + 8 * s.n_src
        d2h = 4 * s.n_steps * s.n_det + 16 * s.n_det
        times = []
        for r in range(1 + args.e2e_runs):
            barrier(dist)
            t = time.perf_counter()
            sh = F.Shot(eprob, device=local)
            sh.run(1, s.n_steps)
            tr = sh.traces()
            d = sh.dft()
            sh.close()
            dt_e = time.perf_counter() - t
            if r > 0:
                times.append(dt_e)
        te = allreduce_max(dist, sum(times) / len(times))
        e_units = allreduce_sum(dist, float(cells) * s.n_steps)
        e2e = {"value": e_units / te / 1e9, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h),
               "note": f"whole {s.n_steps}-step shots: create (upload) + run + read traces/DFT + destroy, "
                       "pageable host buffers"}
        del tr, d

    cpu = None
    if rank == 0 and world == 1 and args.cpu_seconds > 0:
        cpu = cpu_baseline(prob, args.cpu_seconds)

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
                "ms_per_step": t_max * 1e3 / K, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": workload_config(args),
                "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": achieved / peak, "traffic": traffic,
                             "peak_source": peak_src, "kernel": kernel,
                             "algorithmic_bytes_per_launch": BYTES_PER_CELL * cells},
                "e2e": e2e, "cpu_baseline": cpu, "gpu_launches": int(launches), "clocks": clk,
                "finite": ok}
        print(json.dumps(line), flush=True)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--block", type=int, default=100, help="FDTD time steps per bench step")
    ap.add_argument("--e2e-steps", type=int, default=1000)
    ap.add_argument("--e2e-runs", type=int, default=2)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--size", type=int, default=8192, help="grid side (8192 = the production shot)")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    world, rank, local, dist = dist_setup(args.gpus)
    args.gpus = world
    if args.impl == "reference":
        run_reference(args, world, rank, dist)
    else:
        run_ours(args, world, rank, local, dist)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
