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

import numpy as np

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


def replica_throughput(dist, units: float, seconds: float) -> tuple[float, float]:
    """Whole-job rate of N replicas: all ranks' units / the slowest rank's
    time.  Returns (units per second, slowest time)."""
    t_max = allreduce_max(dist, seconds)
    total = allreduce_sum(dist, units)
    return total / t_max, t_max


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


def profile_traffic(kernel: str, cells: int) -> float | None:
    """DRAM bytes per launch of the interior step kernel on this workload,
    from the committed ncu summary of that kernel family: its bytes per cell
    of the launch's region (the region depends on the CPML-band shape the
    autotuner keeps; traffic grows with it in proportion) times `cells`, or
    the per-launch figure when the summary has no per-cell one."""
    name = ("step_tmat2_8192_production.md" if kernel.startswith("step_tmat2") else
            "step_tmat_8192_production.md" if kernel.startswith("step_tmat") else "step_tma_8192_production.md")
    f = ROOT / "profiles" / name
    if not f.exists():
        return None
    text = f.read_text()
    m = re.search(r"traffic_bytes_per_cell:\s*([0-9.eE+]+)", text)
    if m:
        return float(m.group(1)) * cells
    m = re.search(r"traffic_bytes_per_launch:\s*([0-9.eE+]+)", text)
    return float(m.group(1)) if m else None


def workload_config(args) -> dict:
    bpc = BYTES_PER_CELL if getattr(args, "storage", "f32") == "f32" else 18
    touched = bpc * args.size * args.size   # bytes one time step reads and writes
    l2 = (f"no flush: {touched / 1e9:.2g} GB touched per time step >> 129 MB L2" if touched > 4 * 129e6 else
          f"no flush: {touched / 1e6:.3g} MB touched per time step, L2-resident (a small-grid case, not the "
          "HBM-bound workload)")
    return {"workload": f"{args.size}x{args.size} TMz phased-array reflectometry shot: 32-cell CPML, "
                        "tanh x GRF plasma, nu 2e9/s, 16 elements at 50 GHz steered 15 deg, 16 Ez "
                        "detectors + FP64 DFT",
            "nx": args.size, "ny": args.size, "npml": 32, "shot_steps": 20000, "block_steps": args.block,
            "dx_mm": 0.25, "courant": 0.99,
            "bytes_per_cell_update": bpc,
            "storage": getattr(args, "storage", "f32"),
            "l2": l2,
            "parallelism": f"replicas x{args.gpus}"}


def make_problem(n_steps: int, size: int, storage: int = 0):
    import fdtd_2d_gb300 as F

    kw = {}
    if size != 8192:
        kw = dict(nx=size, ny=size, x_center=size * 5000 / 8192, src_j=size // 2 - 37, det_j=size // 2 - 37)
    return F.Problem.from_spec(F.production_spec(n_steps=n_steps, storage=storage, **kw))


C0 = 299792458.0


def mixed_shot_spec(rng, side_lo: float, side_hi: float, f_lo: float, f_hi: float, step_scale: float,
                    seed: int, aspect: bool = True, freq: float | None = None) -> dict:
    """One uneven reflectometry shot: side log-uniform in [side_lo, side_hi]
    (aspect 1:1..1:3 on a random axis), CPML 16..32, dx = lambda/20 at the
    probe frequency, 4..16 elements (pitch 5) with co-located detectors and an
    FP64 DFT at the probe frequency, tanh plasma with peak in [5e18, 5e19] and
    centre in [0.4, 0.8] nx, width 600 * (0.25 mm / dx) cells, 5 % GRF,
    nu = 2e9, 8000..16000 steps times step_scale.  The Courant number is the
    largest <= 0.99 that keeps the Drude leapfrog stable at the peak density."""
    L = float(np.exp(rng.uniform(np.log(side_lo), np.log(side_hi))))
    a = float(rng.uniform(1, 3)) if aspect else 1.0
    S = max(384.0, L / a)
    nx, ny = (int(L), int(S)) if rng.uniform() < 0.5 else (int(S), int(L))
    P = int(rng.integers(16, 33))
    f = float(rng.uniform(f_lo, f_hi)) if freq is None else freq
    dx = C0 / f / 20
    peak = float(rng.uniform(5e18, 5e19))
    xc = float(rng.uniform(0.4, 0.8)) * nx
    wp = 56.4 * np.sqrt(peak * 1.25)            # GRF headroom on the peak
    g = wp * dx / (2 * C0 * np.sqrt(2))         # (omega_p dt / 2) per unit Courant number
    cour = float(min(0.99, 0.985 / np.sqrt(1 + g * g)))
    n_elem = int(rng.integers(4, 17))
    steps = max(16, int(int(rng.integers(8000, 16001)) * step_scale))
    j0 = ny // 2 - 5 * n_elem // 2
    return dict(nx=nx, ny=ny, npml=P, n_steps=steps, dx=dx, dy=dx, courant=cour, profile=3, ne_peak=peak,
                x_center=xc, width=600 * (0.25e-3 / dx), grf_rms=0.05, grf_corr=40, seed=seed, nu=2e9,
                n_elem=n_elem, src_i=P + 32, src_j=j0, src_di=0, src_dj=5, freq=f, steer_deg=15, pulse=1,
                pulse_width=2e-9, n_det=n_elem, det_i=P + 32, det_j=j0, det_di=0, det_dj=5, dft_freq=f)


def run_batched(args, local: int) -> tuple[dict, float]:
    """64 uneven shots (seed 1002) end to end: one at a time through the
    single-shot ABI vs all admitted to one batch, at --batch-step-scale of
    their 8000..16000 steps.  The kernel choice of every size class is timed
    once before the timed passes (a create per shot), so both passes run
    with the choices kept.  With --batch-storage f16 the batch also runs the
    same shots with F16 storage, reported with its DFT phase error against
    the plain FP32 pass.  Returns the JSON object and the batch's throughput
    in cell updates per second."""
    import fdtd_2d_gb300 as F

    rng = np.random.default_rng(1002)
    specs = [mixed_shot_spec(rng, 1024, 6144, 20e9, 75e9, args.batch_step_scale, 1002 + k)
             for k in range(args.batch_shots)]
    probs = [F.Problem.from_spec(**sp) for sp in specs]
    cells = sum(p.nx * p.ny * p.n_steps for p in probs)
    n = len(probs)

    t = time.perf_counter()
    for p in probs:
        with F.Shot(p, local):
            pass
    t_tune = time.perf_counter() - t

    def plain_pass():
        t = time.perf_counter()
        out = []
        for p in probs:
            with F.Shot(p, local) as s:
                s.run(1, p.n_steps)
                s.traces()
                out.append(s.dft())
        return time.perf_counter() - t, out

    def batch_pass(ps):
        t = time.perf_counter()
        with F.Batch(local) as b:
            ids = [b.add(p) for p in ps]
            if any(i is None for i in ids):
                raise RuntimeError("batch budget too small for the mixed-shot sample")
            while not all(b.finished(i) for i in ids):
                b.run(256)
            b.synchronize()
            dft = []
            for i in ids:
                sh = b.shot(i)
                sh.traces()
                dft.append(sh.dft())
            name = b.kernel_name()
            launches = b.launches()
            solo = sum(1 for i in ids if b.shot(i).kernel_name().startswith("step_tmat"))
        return time.perf_counter() - t, dft, name, launches, solo

    tw, plain_dft = plain_pass()
    tb, batch_dft, name, launches, solo = batch_pass(probs)
    same = all(np.array_equal(x, y) for x, y in zip(plain_dft, batch_dft))
    out = {"shots": n, "sample": f"{n} shots, seed 1002, sides log-uniform 1024..6144 (aspect 1..3), CPML 16..32, "
                                 f"20..75 GHz at dx = lambda/20, 4..16 elements, 8000..16000 steps x "
                                 f"{args.batch_step_scale} ({sum(p.n_steps for p in probs)} steps in all)",
           "cell_updates": cells, "plain_shots_per_s": n / tw, "batched_shots_per_s": n / tb,
           "speedup": tw / tb, "plain_gcells": cells / tw / 1e9, "batched_gcells": cells / tb / 1e9,
           "kernel_choice_timing_s": t_tune,
           "kernel": name, "tensor_path_members": solo, "gpu_launches": int(launches),
           "dft_equal_to_plain": bool(same),
           "note": "end to end from host setups: create/upload, all steps, traces + DFT read back; kernel "
                   "choices of every size class timed once before both passes. plain: one shot at a time "
                   "through the single-shot ABI; batch: grids of >= 2^21 cells as solo members (own "
                   "streams, two-step tensor path, at most 8 stepping at a time), the rest in one "
                   "persistent launch per step in CUDA-graph blocks of 16"}
    if args.batch_storage != "f32":
        store = {"f16": F.STORE_F16, "bf16": F.STORE_BF16}[args.batch_storage]
        probs16 = [F.Problem.from_spec(**sp, storage=store) for sp in specs]
        for p in probs16:
            with F.Shot(p, local):
                pass
        t16, dft16, _, _, _ = batch_pass(probs16)
        ph = max(float(np.max(np.abs(np.angle(a * np.conj(b))))) for a, b in zip(dft16, plain_dft))
        out[f"batched_{args.batch_storage}"] = {
            "shots_per_s": n / t16, "gcells": cells / t16 / 1e9, "speedup_vs_plain_f32": tw / t16,
            "dft_phase_err_vs_plain_f32_rad": ph, "phase_within_1e-4_rad": ph <= 1e-4,
            "note": f"the same shots with {args.batch_storage.upper()} field storage (every shot a solo member); "
                    "phase error: largest over shots and detectors"}
    return out, cells / tb


def run_serving(args, local: int, capacity: float) -> dict:
    """Poisson request stream (seed 1004) at 0.8 x the measured batched
    capacity: each request a 4..12-shot frequency sweep over 10..75 GHz on one
    grid size, tanh plasma profiles as the mixed-shot sample's (seeded peak
    and position, no random field); served by the continuous-batching loop
    vs one request at a time through the single-shot ABI.  A request's
    setups are built when it arrives (inside its latency, for both) and
    released when it completes, so the host holds only the requests in
    flight."""
    import fdtd_2d_gb300 as F

    rng = np.random.default_rng(1004)
    reqs = []
    for r in range(args.serve_requests):
        n_shots = int(rng.integers(4, 13))
        freqs = np.sort(rng.uniform(10e9, 75e9, n_shots))
        side = float(np.exp(rng.uniform(np.log(512), np.log(args.serve_max_side))))
        shots = []
        for k, f in enumerate(freqs):
            sub = np.random.default_rng([1004, r, k])
            sp = mixed_shot_spec(sub, side, side, f, f, args.serve_step_scale, 5000 + 100 * r + k, aspect=False,
                                 freq=float(f))
            sp.update(profile=2, grf_rms=0.0)
            shots.append(sp)
        reqs.append(shots)
    work = [sum(sp["nx"] * sp["ny"] * sp["n_steps"] for sp in q) for q in reqs]
    rate = 0.8 * capacity / (sum(work) / len(work))      # requests per second
    gaps = rng.exponential(1.0 / rate, len(reqs))
    arrive = np.cumsum(gaps) - gaps[0]

    def pct(lat):
        return {"p50": float(np.percentile(lat, 50)), "p95": float(np.percentile(lat, 95)),
                "p99": float(np.percentile(lat, 99)), "max": float(np.max(lat))}

    # continuous batching
    t0 = time.perf_counter()
    done_at = {}
    left = {r: len(q) for r, q in enumerate(reqs)}
    nxt = 0
    with F.Server(local, block_steps=64) as srv:
        while len(done_at) < len(reqs):
            now = time.perf_counter() - t0
            while nxt < len(reqs) and arrive[nxt] <= now:
                for k, sp in enumerate(reqs[nxt]):
                    srv.submit(F.Problem.from_spec(**sp), nxt * 1000 + k)
                nxt += 1
            q, running, fin = srv.counts()
            if q == 0 and running == 0 and fin == 0 and nxt < len(reqs):
                time.sleep(max(0.0, arrive[nxt] - (time.perf_counter() - t0)))
                continue
            srv.step()
            while (res := srv.pop()) is not None:
                r = res["tag"] // 1000
                left[r] -= 1
                if left[r] == 0:
                    done_at[r] = time.perf_counter() - t0
        kernel = srv.batch_kernel_name()
    t_batch = max(done_at.values())
    lat_b = [done_at[r] - arrive[r] for r in range(len(reqs))]

    # one request at a time, in arrival order
    t0 = time.perf_counter()
    lat_p = []
    for r, q in enumerate(reqs):
        now = time.perf_counter() - t0
        if now < arrive[r]:
            time.sleep(arrive[r] - now)
        for sp in q:
            p = F.Problem.from_spec(**sp)
            with F.Shot(p, local) as s:
                s.run(1, p.n_steps)
                s.traces()
                s.dft()
            p.close()
        lat_p.append(time.perf_counter() - t0 - arrive[r])
    t_plain = time.perf_counter() - t0
    n_shots = sum(len(q) for q in reqs)
    return {"requests": len(reqs), "shots": n_shots,
            "sample": f"{len(reqs)} Poisson requests (seed 1004) of 4..12-shot sweeps over 10..75 GHz, square "
                      f"grids log-uniform 512..{args.serve_max_side}, tanh profiles with seeded peak and position "
                      f"as the mixed-shot sample, 8000..16000 steps x {args.serve_step_scale} "
                      f"({sum(work):.3g} cell updates); offered load 0.8 x the batched capacity",
           "rate_req_per_s": rate, "shots_per_s": n_shots / t_batch, "latency_s": pct(lat_b),
           "plain_shots_per_s": n_shots / t_plain, "plain_latency_s": pct(lat_p), "kernel": kernel,
           "gcells": sum(work) / t_batch / 1e9, "plain_gcells": sum(work) / t_plain / 1e9,
           "note": "latency = completion of a request's last shot - its arrival (setups built at arrival); "
                   "plain = requests one at a time through the single-shot ABI"}


def run_precision(args, local: int) -> dict:
    """Reduced field storage on the production shot: F16 (per-array 2^k
    scales) and BF16 storage, FP32 arithmetic, FP64 DFT.  Errors are against
    the FP32 GPU run of the same shot over --prec-steps time steps (default
    20000: the whole shot), and against the FP64 oracle on a small shot of the
    same physics (384 x 320, 8 elements, 1500 steps).  Throughput is
    device-timed like `value`; the interior kernel's rate is its launches'
    bytes over their event-timed duration."""
    import fdtd_2d_gb300 as F
    import oracle as O

    def phase_err(a, b):
        return float(np.max(np.abs(np.angle(a * np.conj(b)))))

    def rel(a, b):
        return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-300))

    out = {}
    S, K = args.block, max(3, args.steps // 3)
    n_err = args.prec_steps
    peak = measured_peaks().get("hbm_gbs") or 6800.0
    ref32 = None
    for name, store in (("f32", F.STORE_F32), ("f16", F.STORE_F16), ("bf16", F.STORE_BF16)):
        prob = make_problem(n_err + K * S, args.size, storage=store)
        cells = prob.nx * prob.ny
        with F.Shot(prob, local) as shot:
            t = time.perf_counter()
            shot.run(1, n_err)
            shot.synchronize()
            wall = time.perf_counter() - t
            ez = shot.read_field("ez").astype(np.float64)
            tr = shot.traces(1, n_err)["det_ez"].astype(np.float64)
            dft = shot.dft()
            entry = {"kernel": shot.kernel_name(), "shot_seconds": wall}
            if store != F.STORE_F32:
                shot.time_step_kernel(True)
                ms = shot.run_timed(n_err + 1, n_err + K * S)
                kt = shot.step_kernel_time()
                shot.time_step_kernel(False)
                val = cells * K * S / (ms / 1e3) / 1e9
                two = kt["steps"] == 2
                # 16-bit Ez, Hx, Hy, Jz read and written and the drive read once
                # per launch: 18 B per cell of the launch's region, for the one
                # or two time steps the launch advances
                per_launch = kt["ms"] / 1e3 / max(kt["launches"], 1)
                kgbs = 18 * kt["cells"] / per_launch / 1e9
                entry.update({"value": val, "unit": UNIT, "bytes_per_cell_update": 9 if two else 18,
                              "step_rate_gbs": (9 if two else 18) * val,
                              "interior_kernel": {"achieved_gbs": kgbs, "frac": kgbs / peak,
                                                  "bytes_per_cell_per_launch": 18, "steps_per_launch": kt["steps"],
                                                  "mean_launch_us": per_launch * 1e6},
                              "ok_finite": shot.check_finite()})
        if store == F.STORE_F32:
            ref32 = (ez, tr, dft)
            out["f32"] = entry
            continue
        perr = phase_err(dft, ref32[2])
        entry.update({"ez_rel_l2_vs_f32": rel(ez, ref32[0]), "trace_rel_l2_vs_f32": rel(tr, ref32[1]),
                      "dft_phase_err_vs_f32_rad": perr, "dft_amp_rel_err_vs_f32":
                          float(np.max(np.abs(np.abs(dft) / np.abs(ref32[2]) - 1))),
                      "phase_within_1e-4_rad": perr <= 1e-4, "steps_compared": n_err})
        out[name] = entry
    # against the FP64 oracle on a small shot of the same physics
    small = dict(nx=384, ny=320, npml=16, n_steps=1500, dx=0.25e-3, dy=0.25e-3, courant=0.99, profile=3,
                 ne_peak=3e19, x_center=250, width=40, grf_rms=0.05, grf_corr=10, seed=7, nu=2e9, n_elem=8,
                 src_i=40, src_j=140, src_dj=5, src_di=0, freq=50e9, steer_deg=15, pulse=1, pulse_width=0.2e-9,
                 n_det=8, det_i=40, det_j=140, det_dj=5, det_di=0, dft_freq=50e9)
    p64 = F.Problem.from_spec(**small)
    o = O.Oracle(p64.setup_ptr)
    o.run(1, small["n_steps"])
    o_f = {w: o.read_field(F.FIELD_NAMES[w]) for w in ("ez", "hx", "hy", "jz")}
    o_tr = o.traces(1, small["n_steps"])["det_ez"]
    o_dft = o.dft()
    for name, store in (("f32", F.STORE_F32), ("f16", F.STORE_F16), ("bf16", F.STORE_BF16)):
        p = F.Problem.from_spec(**small, storage=store)
        with F.Shot(p, local) as shot:
            shot.run(1, small["n_steps"])
            e = {w: rel(shot.read_field(w), o_f[w]) for w in o_f}
            res = {"field_rel_l2": e, "trace_rel_l2": rel(shot.traces()["det_ez"], o_tr),
                   "dft_phase_err_rad": phase_err(shot.dft(), o_dft)}
        out.setdefault(name, {})["vs_fp64_oracle_384x320_1500_steps"] = res
    out["note"] = ("F16: Ez, Hx, Hy, Jz and the drive map stored as FP16 with a power-of-two scale per array; "
                   "BF16 the same without scales; 18 B per cell-update per pass (FP32: 36), 9 (18) when a pass "
                   "advances two time steps; arithmetic FP32, DFT FP64; errors vs FP32 over the whole "
                   f"{n_err}-step shot")
    return out


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
    """The reference's step on the host cores: the oracle's FP32 restatement
    of the reference update equations, all threads, on the same shot built by
    oracle/workload.py with numpy (the product library is never loaded in
    this process)."""
    if rank != 0:
        return
    import oracle as O
    from oracle import workload

    wl = workload.production_setup(max(args.steps + args.warmup + 2, 10), args.size)
    cores = O.threads()
    o = O.Oracle(wl.setup_ptr, fp32=True)
    cells = wl.setup.nx * wl.setup.ny
    o.run(1, args.warmup)
    t = time.perf_counter()
    o.run(args.warmup + 1, args.warmup + args.steps)
    dt = time.perf_counter() - t
    o.close()
    value = cells * args.steps / dt / 1e9
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "impl": "reference", "config": dict(workload_config(args), block_steps=1),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{args.steps} time steps of the {wl.setup.nx}x{wl.setup.ny} shot per run "
                                       "(one time step per bench step), FP32 restatement of the "
                                       "reference update equations, OpenMP over rows; setup built with numpy "
                                       "(oracle/workload.py), no product library loaded"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args, world, rank, local, dist) -> None:
    import fdtd_2d_gb300 as F

    S, K, W = args.block, args.steps, args.warmup
    total_steps = (W + K) * S
    store = {"f32": 0, "f16": 1, "bf16": 2}[args.storage]
    bpc = BYTES_PER_CELL if store == 0 else 18   # 16-bit Ez, Hx, Hy, Jz and drive
    prob = make_problem(max(20000, total_steps), args.size, storage=store)
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
    shot.time_step_kernel(True)   # event pair around each interior-kernel launch
    ms = shot.run_timed(W * S + 1, W * S + K * S)  # one event pair around the K blocks
    shot.synchronize()
    kt = shot.step_kernel_time()
    shot.time_step_kernel(False)
    barrier(dist)
    launches = shot.launches() - launches0
    clk = clocks.stop()
    ok = shot.check_finite()
    shot.close()
    rate, t_max = replica_throughput(dist, float(cells) * S * K, ms / 1e3)
    value = rate / 1e9

    # roofline of the interior step kernel: algorithmic bytes of one launch
    # (bpc per cell of its region: each field read and written once per
    # pass, whether a pass advances them one time step or two; the
    # persistent kernel's launch makes one pass per step) over its mean
    # event-timed launch duration
    per_launch_s = kt["ms"] / 1e3 / max(kt["launches"], 1)
    passes = kt["steps"] if kernel.startswith("step_persist") else 1
    alg_bytes = bpc * kt["cells"] * passes
    achieved = alg_bytes / per_launch_s / 1e9
    step_gbs = bpc * cells / ((ms / 1e3) / (K * S)) / 1e9   # bpc per cell-update at the whole-step rate
    peaks = measured_peaks()
    peak = peaks.get("hbm_gbs")
    peak_src = "measured"
    if not peak:
        peak, peak_src = 6800.0, "fallback"
    traffic = profile_traffic(kernel, kt["cells"]) if (store == 0 and args.size == 8192) else None

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
        # a bench step is S time steps: a shot of s.n_steps time steps is
        # s.n_steps / S bench steps, and its copies are spread over them
        per_shot_steps = s.n_steps / S
        e2e = {"value": e_units / te / 1e9, "unit": UNIT, "h2d_bytes_per_step": int(h2d / per_shot_steps),
               "d2h_bytes_per_step": int(d2h / per_shot_steps),
               "h2d_bytes_per_shot": int(h2d), "d2h_bytes_per_shot": int(d2h),
               "bench_steps_per_shot": per_shot_steps,
               "note": f"whole {s.n_steps}-step shots ({per_shot_steps:g} bench steps of {S} time steps): create "
                       "(uploads the drive map, tables, source envelope) + run + read traces/DFT + destroy, "
                       "pageable host buffers; bytes per step = bytes per shot / bench steps per shot"}
        del tr, d

    cpu = None
    if rank == 0 and world == 1 and args.cpu_seconds > 0:
        cpu = cpu_baseline(prob, args.cpu_seconds)
    del shot
    batched = serving = precision = None

    def leg(fn, *a):
        # an extra leg that fails is reported in its own key; the main
        # measurement above stands
        try:
            return fn(*a)
        except Exception as e:  # noqa: BLE001
            return {"error": f"{type(e).__name__}: {e}"}

    if args.prec_steps > 0 and world == 1:
        precision = leg(run_precision, args, local)
    if args.batch_shots > 0:
        barrier(dist)
        res = leg(run_batched, args, local)
        batched, capacity = (res, None) if "error" in res else res
        if args.serve_requests > 0 and capacity:
            serving = leg(run_serving, args, local, capacity)

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
                "ms_per_step": t_max * 1e3 / K, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32" if store == 0 else f"f32 arithmetic, {args.storage} storage",
                "data": "synthetic", "config": workload_config(args),
                "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": achieved / peak, "traffic": traffic,
                             "peak_source": peak_src, "kernel": kernel,
                             "algorithmic_bytes_per_launch": alg_bytes,
                             "cells_per_launch": kt["cells"], "steps_per_launch": kt["steps"],
                             "launches_timed": kt["launches"], "mean_launch_us": per_launch_s * 1e6,
                             "step_rate_gbs_at_36_b_per_cell_update": step_gbs,
                             "note": "achieved: the interior kernel alone (event-timed on its stream); "
                                     "step_rate: whole steps at bpc per cell-update, above the copy peak "
                                     "when a launch advances its cells two steps"},
                "e2e": e2e, "cpu_baseline": cpu, "gpu_launches": int(launches), "clocks": clk,
                "finite": ok, "precision": precision, "batched": batched, "serving": serving}
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
    ap.add_argument("--batch-shots", type=int, default=64, help="mixed-shot sample size (0: skip batched/serving)")
    ap.add_argument("--batch-step-scale", type=float, default=1.0,
                    help="fraction of the 8000..16000 steps each mixed shot runs")
    ap.add_argument("--batch-storage", choices=["f32", "f16", "bf16"], default="f16",
                    help="also run the batch with this field storage (f32: no second run)")
    ap.add_argument("--serve-requests", type=int, default=50, help="requests in the serving sample (0: skip)")
    ap.add_argument("--serve-max-side", type=int, default=8192)
    ap.add_argument("--serve-step-scale", type=float, default=0.1,
                    help="fraction of the 8000..16000 steps each serving shot runs")
    ap.add_argument("--storage", choices=["f32", "f16", "bf16"], default="f32",
                    help="field storage of the main measurement (arithmetic is FP32 in all)")
    ap.add_argument("--prec-steps", type=int, default=20000,
                    help="steps of the F16/BF16 vs FP32 comparison on the production shot (0: skip)")
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
