#!/usr/bin/env python3
"""Benchmark of the per-step agent hot path on GB300: agent-steps/s.

Workload (default, ``--workload large``): the single large run -- icosahedral
grid n=256 (655,362 cells), altitude-derived K, 20M agents placed with
probability proportional to K, ages U[0,60); GetOld, Fertility, RandomPair,
VerhulstVarK, OldAgeDeath (onset U[60,70)), WeightedMove (p=0.2).  Synthetic,
seeded inputs of the configuration's shapes and distributions.

One line of JSON on rank 0 (the contract's keys plus ``roofline``,
``cpu_baseline``, ``e2e``, ``clocks``, ``gpu_launches``).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

``--impl reference`` times the CPU implementation of the path on this host's
cores: the C port of the reference algorithm (oracle/qhg_oracle.c), because
the reference itself cannot be compiled on the GPU host (its sources are not
there).  With several GPUs (torchrun), every rank runs an independent replica
of the workload on its own GPU (the path has no data exchange between runs);
``value`` sums the agent-steps of all ranks over the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from qhg4_gb300 import configs  # noqa: E402
from qhg4_gb300.spec import config1_actions  # noqa: E402

METRIC = "agent-steps/s"

# name: workload factory (seed -> configs.Workload)
WORKLOADS = {
    "large": lambda seed: configs.single_large_run(seed),
    # a smaller case of the same actions for profiler captures (hot table > L2)
    "medium": lambda seed: configs.single_large_run(seed, n=192, agents=8_000_000),
    "plain": lambda seed: configs.plain_method(seed),
    "genetics": lambda seed: configs.genetics_run(seed),
    # a smaller case of the genetics run's actions for profiler captures
    "genetics_small": lambda seed: configs.genetics_run(seed, agents=1_000_000, n=64),
}
AGENT_BYTES = 60   # one read and one write of the 30-byte hot record per agent-step
BIRTH_BYTES = 3 * 1024   # genetics: two parent genomes read, one child genome written (2 x 4,096 loci)
# kernels launched per step of a single run: the action kernel and the
# scatter in each of the three forms (two of each return at once) and the
# cell scan; the genome kernel with genetics
LAUNCHES_PER_STEP = 7
# untimed first steps of every ensemble run, batched and plain alike
ENSEMBLE_WARM = 5
# speed of the C port relative to the reference's own OpenMP code, measured
# where the reference sources are (both on 8 cores of the build container,
# the plain method and the large run's actions at 2M agents)
PORT_VS_REFERENCE = ("at 1.15x (plain method), 0.85x (large run's actions, 2M agents) and 0.98x (genetics, "
                     "400k agents) the speed of")


def build_workload(name: str, seed: int = 42):
    return WORKLOADS[name](seed)


def workload_config(w, world: int):
    """The line's `config` (identical for this implementation and the CPU reference arm)."""
    return {"workload": w.name, "detail": w.desc, "agents": len(w.agents), "cells": w.grid.num_cells,
            "parallelism": f"replicas x{world}",
            "l2": "inputs larger than L2 (hot table ~21 B x agents > 129 MB)"}


class NvmlSampler:
    """Samples the SM clock, power and clock-event reasons through NVML
    (read-only queries, ctypes into libnvidia-ml) every ~2 ms from a thread,
    so that even a timed region of a few milliseconds holds samples.  The
    GPU is found by the PCI bus ID the CUDA runtime gives for `device`."""

    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
               0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown"}

    def __init__(self, device: int):
        import ctypes as ct
        self.ct = ct
        self.nv = ct.CDLL("libnvidia-ml.so.1")
        if self.nv.nvmlInit_v2() != 0:
            raise OSError("nvmlInit failed")
        bus = ct.create_string_buffer(64)
        rt = None
        for name in ("libcudart.so", "libcudart.so.13", "libcudart.so.12"):
            try:
                rt = ct.CDLL(name)
                break
            except OSError:
                continue
        self.h = ct.c_void_p()
        rc = -1
        if rt is not None and rt.cudaDeviceGetPCIBusId(bus, 64, int(device)) == 0:
            rc = self.nv.nvmlDeviceGetHandleByPciBusId_v2(bus, ct.byref(self.h))
        if rc != 0:
            rc = self.nv.nvmlDeviceGetHandleByIndex_v2(int(device), ct.byref(self.h))
        if rc != 0:
            raise OSError("no NVML handle for the device")
        fn = getattr(self.nv, "nvmlDeviceGetCurrentClocksEventReasons", None)
        self.reasons_fn = fn if fn is not None else self.nv.nvmlDeviceGetCurrentClocksThrottleReasons
        mx = ct.c_uint()
        self.max_mhz = float(mx.value) if self.nv.nvmlDeviceGetMaxClockInfo(self.h, 1, ct.byref(mx)) == 0 else None
        self.samples = []
        self.stop_flag = False
        self.thread = None

    def _sample(self):
        ct = self.ct
        mhz, rs, mw = ct.c_uint(), ct.c_ulonglong(), ct.c_uint()
        while not self.stop_flag:
            t = time.perf_counter()
            if self.nv.nvmlDeviceGetClockInfo(self.h, 1, ct.byref(mhz)) == 0 and \
                    self.reasons_fn(self.h, ct.byref(rs)) == 0:
                self.nv.nvmlDeviceGetPowerUsage(self.h, ct.byref(mw))
                self.samples.append((t, float(mhz.value), int(rs.value), mw.value / 1000.0))
            time.sleep(0.002)

    def start(self):
        self.thread = threading.Thread(target=self._sample, daemon=True)
        self.thread.start()

    def wait_first(self, timeout: float = 5.0) -> None:
        t0 = time.perf_counter()
        while not self.samples and time.perf_counter() - t0 < timeout:
            time.sleep(0.005)

    def mark(self) -> float:
        return time.perf_counter()

    def stop(self, t_from: float = None, t_to: float = None):
        self.stop_flag = True
        if self.thread:
            self.thread.join(timeout=2)
        inside = [x for x in self.samples if t_from is not None and t_from <= x[0] <= t_to]
        window = bool(inside)
        use = inside if inside else self.samples
        reasons = sorted({nm for _, _, r, _ in use for bit, nm in self.REASONS.items() if r & bit})
        sm = [m for _, m, _, _ in use]
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": self.max_mhz, "reasons": reasons,
                "samples": len(use), "power_w_max": max((p for *_, p in use), default=None),
                "source": "NVML every ~2 ms",
                "window": "timed region" if window else "whole measurement (no sample inside the timed region)"}


def clock_sampler(device: int):
    """NVML sampler where NVML loads, else nvidia-smi."""
    try:
        return NvmlSampler(device)
    except (OSError, AttributeError):
        return ClockSampler(device)


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi while running."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap,utilization.gpu")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.perf_counter(), line.strip()))

    def wait_first(self, timeout: float = 5.0) -> None:
        """Waits until nvidia-smi has delivered a sample (it starts slowly)."""
        t0 = time.perf_counter()
        while self.proc is not None and not self.lines and time.perf_counter() - t0 < timeout:
            time.sleep(0.02)

    def mark(self) -> float:
        return time.perf_counter()

    def stop(self, t_from: float = None, t_to: float = None):
        """Clocks of the samples taken between t_from and t_to (all samples
        if that window holds none)."""
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons, busy = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        lines = [ln for t, ln in self.lines if t_from is not None and t_from <= t <= t_to]
        window = bool(lines)
        if not lines:
            lines = [ln for _, ln in self.lines]
        for ln in lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 10:
                continue
            try:
                s, m = float(f[1]), float(f[2])
                util = float(f[9])
            except ValueError:
                continue
            sm.append(s)
            smax.append(m)
            if util > 0:
                busy.append(s)
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        load = busy if busy else sm
        return {"sm_mhz": float(np.median(load)) if load else None,
                "sm_max_mhz": float(max(smax)) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm), "samples_busy": len(busy),
                "window": "timed region" if window else "whole measurement (no sample inside the timed region)"}


def read_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def read_traffic(workload: str):
    """DRAM bytes per agent-step of one step's kernels, from the committed ncu
    summary (profiles/step_traffic_<workload>.txt), or None."""
    p = os.path.join(ROOT, "profiles", f"step_traffic_{workload}.txt")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        for ln in f:
            m = re.match(r"\s*dram_bytes_per_agent_step\s*[:=]\s*([0-9.eE+]+)", ln)
            if m:
                return float(m.group(1))
    return None


def cpu_leg(w, steps, warmup):
    """The C port of the reference algorithm on all host threads (OpenMP)."""
    from oracle import port
    threads = os.cpu_count() or 1
    port.set_threads(threads)
    r = port.OracleRun(w.grid, w.actions, w.seed, w.genetics, log_births=False)
    r.load(w.agents)
    if warmup > 0:
        r.step(warmup)
    n0 = r.num_agents()
    t0 = time.perf_counter()
    st = r.step(steps)
    dt = time.perf_counter() - t0
    agent_steps = n0 + int(st[:-1, 0].sum()) if steps > 0 else 0
    r.close()
    return agent_steps, dt, threads


def init_dist(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return world, rank, local, dist


def gather_max(dist, x: float) -> float:
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gather_sum(dist, x: float) -> float:
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def run_reference(args, world, rank, dist):
    """The reference arm: the CPU implementation of the path on this host's
    cores (the C port, OpenMP on every core), on the same workload, config,
    warm-up and timed steps as this implementation's line."""
    if rank != 0:
        return 0
    w = build_workload(args.workload, args.seed)
    steps = max(1, args.steps)
    warm = args.warmup
    n_as, dt, thr = cpu_leg(w, steps, warm)
    v = n_as / dt
    sample = (f"all {steps} timed step(s) after {warm} warm-up step(s) of the full {w.name} workload "
              f"({len(w.agents)} initial agents) on the C port of the reference algorithm "
              f"(oracle/qhg_oracle.c, OpenMP, {thr} threads); the port runs {PORT_VS_REFERENCE} "
              f"the reference's own OpenMP code built from its sources")
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "agent-steps/s", "n_gpus": args.gpus,
        "steps": steps, "warmup": warm, "ms_per_step": 1000.0 * dt / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32/f32/f64",
        "data": "synthetic (seeded; shapes and distributions of the configuration)",
        "config": workload_config(w, world),
        "cpu_baseline": {"value": v, "unit": "agent-steps/s", "cores": thr, "kind": "port", "sample": sample},
        "e2e": {"value": v, "unit": "agent-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def step_roofline(w, kms, prof_agents, births_per_step):
    """Roofline of one step: its algorithmic bytes over the summed event
    time of its kernels; the same for the genome kernel alone."""
    kmean = kms.mean(axis=0)
    names = ["k_actions", "k_cell_scan", "k_scatter", "k_genomes"]
    nk = 4 if w.genetics.genome_size > 0 else 3
    step_ms = float(kmean[:nk].sum())
    kshare = {names[i]: {"ms": float(kmean[i]), "share": float(kmean[i] / step_ms) if step_ms > 0 else 0.0}
              for i in range(nk)}
    dominant = max(range(nk), key=lambda i: kmean[i])
    C = w.grid.num_cells
    alg_bytes = AGENT_BYTES * prof_agents + w.cell_bytes * C + (BIRTH_BYTES * births_per_step if nk == 4 else 0.0)
    peak, peak_kind = read_peaks()
    achieved = alg_bytes / (step_ms / 1000.0) / 1e9 if step_ms > 0 else 0.0
    tpa = read_traffic(w.name)
    roof = {"bound": "hbm", "kernel": "one step: " + " + ".join(names[:nk]) + f" (dominant: {names[dominant]})",
            "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else "fallback",
            "traffic": (tpa * prof_agents) if tpa is not None else None,
            "algorithmic_bytes": alg_bytes,
            "algorithmic_formula": f"{AGENT_BYTES} B x agents + {w.cell_bytes} B x cells"
                                   + (f" + {BIRTH_BYTES} B x births" if nk == 4 else ""),
            "per_kernel": kshare}
    if nk == 4:
        gb = BIRTH_BYTES * births_per_step
        gms = float(kmean[3])
        ga = gb / (gms / 1000.0) / 1e9 if gms > 0 else 0.0
        roof["k_genomes"] = {"achieved": ga, "frac": ga / peak, "ms": gms, "births_per_step": births_per_step,
                             "algorithmic_bytes": gb, "unit": "GB/s"}
    return roof, step_ms


def profile_steps(run, n_prof_start, prof_steps):
    """Per-kernel device times of prof_steps steps (each kernel launched alone
    between CUDA events on the run's stream), the mean agents at their start
    and the mean births per step."""
    kms = run.step_profiled(prof_steps)
    pst = run.stats(prof_steps)
    prof_agents = (n_prof_start + int(pst[:-1, 0].sum())) / prof_steps
    births = float(pst[:, 1].mean())
    return kms, prof_agents, births


def measure_genetics(seed: int, device: int, steps: int, warmup: int, prof_steps: int):
    """The genetics run beside the default workload: agent-steps/s of the
    step with genomes and the genome kernel's roofline (3 x 1 KiB per birth)."""
    from qhg4_gb300.gpu import GpuRun
    w = build_workload("genetics", seed)
    run = GpuRun(w.grid, w.actions, w.seed, w.genetics, capacity=int(len(w.agents) * 1.6) + 65536, device=device)
    run.load(w.agents)
    run.step(warmup)
    run.sync()
    n_start = run.num_agents()
    ms = run.step_timed(steps)
    st = run.stats(steps)
    agent_steps = n_start + int(st[:-1, 0].sum())
    kms, prof_agents, births = profile_steps(run, int(st[-1, 0]), prof_steps)
    roof, step_ms = step_roofline(w, kms, prof_agents, births)
    run.close()
    return {"value": agent_steps / (ms / 1000.0), "unit": "agent-steps/s", "steps": steps, "warmup": warmup,
            "ms_per_step": ms / steps, "agents_at_timed_start": n_start, "config": workload_config(w, 1),
            "births_per_step": births, "roofline": roof}


def run_ours(args, world, rank, local, dist):
    from qhg4_gb300.gpu import GpuRun
    device = local if world > 1 else args.device
    w = build_workload(args.workload, args.seed + rank)
    grid, agents, actions = w.grid, w.agents, w.actions
    N0 = len(agents)
    C = grid.num_cells
    cap = int(N0 * (1.6 if w.genetics.genome_size > 0 else 2.5)) + 65536
    run = GpuRun(grid, actions, w.seed, w.genetics, capacity=cap, device=device)
    run.load(agents)
    if args.warmup > 0:
        run.step(args.warmup)
    run.sync()
    n_start = run.num_agents()
    sampler = clock_sampler(device)
    sampler.start()
    sampler.wait_first()
    if dist is not None:
        dist.barrier()
    t_on = sampler.mark()
    ms = run.step_timed(args.steps)
    t_off = sampler.mark()
    if dist is not None:
        dist.barrier()
    st = run.stats(args.steps) if args.steps > 0 else np.zeros((0, 4), np.uint64)
    agent_steps = n_start + int(st[:-1, 0].sum()) if args.steps > 0 else 0
    # per-kernel device times (each kernel launched alone between events)
    prof_steps = max(1, args.profile_steps)
    kms, prof_agents, births = profile_steps(run, int(st[-1, 0]) if args.steps > 0 else n_start, prof_steps)
    if os.environ.get("QHG_BENCH_DEBUG"):
        sys.stderr.write(f"timed stats tail {st[-3:].tolist()} kms {kms.tolist()}\n")
    clocks = sampler.stop(t_on, t_off)
    t_max = gather_max(dist, ms / 1000.0)
    total = gather_sum(dist, float(agent_steps))
    value = total / t_max if t_max > 0 else 0.0
    roofline, step_ms = step_roofline(w, kms, prof_agents, births)
    run.close()

    # end to end through the public API, as a user runs a job: the grid and
    # the agent table uploaded from page-locked host memory, the configured
    # job length with each step's statistics copied back to the host as the
    # step ends (queued, no wait per step), the final table downloaded into
    # page-locked host memory; wall clock over all of it
    e2e = None
    if not args.skip_e2e:
        from qhg4_gb300.gpu import HostBuffer, pinned_agents
        job_steps = w.steps if args.e2e_steps <= 0 else args.e2e_steps
        gw = 2 * w.genetics.num_blocks if w.genetics.genome_size > 0 else 0
        inp, inbufs = pinned_agents(N0, gw)          # the user's input table, page-locked
        for k in ("id", "cell", "birth", "age", "lastb", "gender", "state"):
            getattr(inp, k)[:] = getattr(agents, k)
        if gw:
            inp.genome[:] = agents.genome
        outp, outbufs = pinned_agents(cap, gw)       # room for the result
        sbuf = HostBuffer((job_steps, 4), np.uint64)
        t0 = time.perf_counter()
        run2 = GpuRun(grid, actions, w.seed, w.genetics, capacity=cap, device=device)
        t_grid = time.perf_counter()
        run2.load(inp)
        run2.sync()
        t_load = time.perf_counter()
        for s_ in range(job_steps):
            run2.step(1)
            run2.stats_async(sbuf.array[s_])
        run2.sync()
        t_steps = time.perf_counter()
        final = run2.agents(sort_by_id=False, out=outp)
        dt = time.perf_counter() - t0
        t_down = t0 + dt
        run2.close()
        live = sbuf.array[:, 0].astype(np.int64)
        e_as = N0 + int(live[:-1].sum())
        rec = 8 + 4 + 4 + 4 + 4 + 1 + 1 + 8 * gw
        e2e_t = gather_max(dist, dt)
        e2e_as = gather_sum(dist, float(e_as))
        e2e = {"value": e2e_as / e2e_t, "unit": "agent-steps/s",
               "h2d_bytes_per_step": int(N0 * rec / job_steps + (C * 6 * 4 + C + C * 8) / job_steps),
               "d2h_bytes_per_step": int(32 + len(final) * rec / job_steps),
               "steps": job_steps, "seconds": dt,
               "phases_s": {"create_and_grid": t_grid - t0, "agents_upload": t_load - t_grid,
                            "steps": t_steps - t_load, "download": t_down - t_steps},
               "detail": "qhg_gpu_create + qhg_gpu_upload_grid + qhg_gpu_upload_agents from page-locked host arrays, "
               "per step qhg_gpu_step(1) + qhg_gpu_stats_async into page-locked memory, qhg_gpu_sync, "
               "qhg_gpu_download into page-locked arrays; wall clock"}
        for bb in inbufs + outbufs + [sbuf]:
            bb.free()

    genetics = None
    if not args.skip_genetics and w.genetics.genome_size == 0:
        genetics = measure_genetics(args.seed + rank, device, args.genetics_steps, 3, prof_steps)
    # the batched ensemble beside the single large run (256 runs, 500 steps each)
    batched = None
    if not args.skip_batched:
        batched = measure_ensemble(args.ensemble_runs, args.ensemble_steps, device, args.plain_runs,
                                   seed=2024 + rank)
        batched["workload"] = ("batched ensemble: runs with grid n in {32,64,128}, agents log-uniform "
                               "[1e4,2e6], per-run b0, d0, p and seed (= run index); plain method's actions")
    served = None
    if not args.skip_served:
        served = measure_served(args.served_jobs, args.served_rate, device, args.hbm_budget_gb * 1e9, seed=7 + rank)
        served["workload"] = ("served stream: Poisson arrivals; grid n in {32,64,128,256}, agents log-uniform "
                              "[1e4,1e7], steps U[50,1000]; HBM-footprint admission; snapshots every 100 steps")
    cpu = None
    if rank == 0 and not args.skip_cpu:
        cs = max(1, args.cpu_steps)
        n_as, dt, thr = cpu_leg(w, cs, 0)
        cpu = {"value": n_as / dt, "unit": "agent-steps/s", "cores": thr, "kind": "port",
               "sample": f"first {cs} step(s) of the same workload on the C port of the reference algorithm "
                         f"(oracle/qhg_oracle.c, OpenMP, {thr} threads); the port runs "
                         f"{PORT_VS_REFERENCE} the reference's own OpenMP code built from its sources"}
    if rank == 0:
        cfg = workload_config(w, world)
        cfg["agents_at_timed_start"] = n_start
        line = {
            "metric": METRIC, "value": value, "unit": "agent-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / max(1, args.steps),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32/f32/f64",
            "data": "synthetic (seeded; shapes and distributions of the configuration)",
            "config": cfg,
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks, "genetics": genetics,
            "batched": batched, "served": served,
            "gpu_launches": (LAUNCHES_PER_STEP + (1 if w.genetics.genome_size > 0 else 0)) * args.steps * world,
            "gpu_launches_per_step": LAUNCHES_PER_STEP + (1 if w.genetics.genome_size > 0 else 0),
        }
        print(json.dumps(line), flush=True)
    return 0


def measure_ensemble(n_runs: int, steps: int, device: int, plain_runs: int, seed: int = 2024):
    """Batched ensemble (many independent runs in one batch) against the
    plain path running the same runs one at a time.  Both time only the
    stepping on the device (CUDA events); admission/upload and graph
    building are outside, the e2e figures include them."""
    from qhg4_gb300.batch import Autotuner, GpuBatch
    from qhg4_gb300.ensemble import ensemble_specs
    from qhg4_gb300.gpu import GpuRun
    t_gen = time.perf_counter()
    specs = ensemble_specs(n_runs=n_runs, steps=steps, seed=seed)
    t_gen = time.perf_counter() - t_gen
    n0 = sum(len(s.agents) for s in specs)
    cells = sum(s.grid.num_cells for s in specs)
    # ---- batched
    t_job = time.perf_counter()
    # room for every run at twice its start or at 40 agents per cell (K = 30), whichever is larger
    cap = sum(max(2 * len(s.agents), 40 * s.grid.num_cells) for s in specs) + 65536
    b = GpuBatch(config1_actions(), agent_capacity=cap, cell_capacity=cells, max_runs=n_runs,
                 stage_capacity=n0, device=device)
    ids = [b.add_run(s.grid, s.actions, s.seed, s.agents) for s in specs]
    # the runs' agents enter the table; the first steps (few births while the
    # runs' first mothers wait out the interbirth time) run untimed before
    # the first tuning, like the plain runs' first steps
    b.step(1 + ENSEMBLE_WARM)
    # the autotuner (re)tunes whenever the batch enters another size bucket
    # (the ensemble shrinks); its timed trial steps are simulation steps and
    # count in the batched figure; steps that capture a new launch's graphs
    # are not timed
    tuner = Autotuner(trial_steps=2, span=2)
    ms_b, as_b, timed_steps = 0.0, 0, 0
    last = None
    while True:
        left = steps - b.steps_done(ids[0])
        if left <= 0:
            break
        launch = tuner.tune(b)
        left = steps - b.steps_done(ids[0])
        if launch != last:
            b.step(min(2, left))   # graphs of both table parities
            last = launch
            continue
        k = min(left, 50)
        n_start = b.num_agents()
        ms_b += b.step_timed(k)
        live = b.live_history(k)
        as_b += n_start + int(live[:-1].sum())
        timed_steps += k
    ms_b += tuner.trial_ms
    as_b += tuner.trial_agent_steps
    timed_steps += tuner.trial_steps_done
    finals = [len(b.agents(r, sort_by_id=False)) for r in ids]
    hist = b.live_history(steps + 1)
    b.close()
    t_job = time.perf_counter() - t_job
    as_job = int(hist[:-1].sum())   # agents at the start of every step of every run
    # ---- plain, one run at a time (the first plain_runs runs)
    ms_p, as_p, wall_p, as_p_all = 0.0, 0, 0.0, 0
    np_runs = min(plain_runs, n_runs)
    for s in specs[:np_runs]:
        t0 = time.perf_counter()
        r = GpuRun(s.grid, s.actions, s.seed, capacity=max(2 * len(s.agents), 40 * s.grid.num_cells) + 65536,
                   device=device)
        r.load(s.agents)
        r.step(1 + ENSEMBLE_WARM)   # both graphs built outside the timed steps
        st0 = r.stats(1 + ENSEMBLE_WARM)
        k = s.steps - 1 - ENSEMBLE_WARM
        ms_p += r.step_timed(k)
        st = r.stats(k)
        as_p += int(st0[-1, 0]) + int(st[:-1, 0].sum())
        as_p_all += len(s.agents) + int(st0[:, 0].sum()) + int(st[:-1, 0].sum())
        r.agents(sort_by_id=False)
        r.close()
        wall_p += time.perf_counter() - t0
    bat = as_b / (ms_b / 1000.0) if ms_b > 0 else 0.0
    pla = as_p / (ms_p / 1000.0) if ms_p > 0 else 0.0
    return {
        "value": bat, "unit": "agent-steps/s", "plain_value": pla,
        "speedup_vs_plain": bat / pla if pla > 0 else None,
        "runs": n_runs, "steps_per_run": steps, "initial_agents": n0, "cells": cells,
        "timed_steps": timed_steps, "batched_ms": ms_b, "plain_runs": np_runs, "plain_ms": ms_p,
        "launch_tuning": {
            "knobs": "actions CTAs/SM, scatter CTAs/SM, scan cells per thread (0: by grid size), "
                     "warp-per-cell form from this mean occupancy (0: default 24)",
            "bucket": "(log2 agents, log2 mean agents per non-empty cell)",
            "table": {str(list(k)): list(v) for k, v in tuner.table.items()},
            "trials_ms_per_agent_step": {str(list(k)): [[list(c), t] for c, t in v] for k, v in tuner.trials.items()}},
        "final_agents": int(sum(finals)),
        "e2e": {"value": as_job / t_job, "unit": "agent-steps/s", "job_s": t_job,
                "plain_value": as_p_all / wall_p if wall_p > 0 else None, "plain_job_s": wall_p,
                "detail": "admission of every run from host arrays, all steps, download of every run's "
                          "final table; plain: create, upload, all steps, download, one run after another"},
        "generation_s": t_gen,
    }


def measure_served(n_jobs: int, rate: float, device: int, budget: float, seed: int = 7):
    """Served stream: Poisson arrivals, admission under the HBM budget,
    continuous batching, snapshots every 100 steps written by a thread.
    Latency = completion - arrival (wall clock); value = agent-steps of all
    jobs / wall time from the first arrival to the last completion."""
    import tempfile
    from qhg4_gb300.serve import Server, job_stream, summarize
    t_gen = time.perf_counter()
    jobs = job_stream(n_jobs, rate=rate, seed=seed)
    t_gen = time.perf_counter() - t_gen
    need_rows = sum(j.rows for j in jobs)
    need_cells = sum(j.grid.num_cells for j in jobs)
    with tempfile.TemporaryDirectory() as snapdir:
        # the batch is sized for the budget, or for the whole stream when that is smaller
        from qhg4_gb300.serve import BYTES_PER_AGENT, BYTES_PER_CELL
        rows = min(need_rows, int(budget * 0.9 / BYTES_PER_AGENT), 2**31 - 1)
        cells = min(need_cells, int(budget * 0.1 / BYTES_PER_CELL))
        srv = Server(hbm_budget=budget, agent_capacity=rows, cell_capacity=cells, max_runs=256,
                     snapshot_every=100, snapshot_dir=snapdir, chunk=16, device=device)
        t0 = time.perf_counter()
        done = srv.serve(jobs)
        wall = time.perf_counter() - t0
        n_snap = sum(len(j.snapshots) for j in done)
        busy = srv.busy_s
        srv.close()
    first = min(j.arrival for j in jobs)
    res = summarize(done, wall - first)
    res.update({"rate_jobs_per_s": rate, "hbm_budget_gb": budget / 1e9, "batch_rows": rows, "batch_cells": cells,
                "snapshots": n_snap, "gpu_loop_s": busy, "generation_s": t_gen,
                "initial_agents": int(sum(len(j.agents) for j in jobs)),
                "max_wait_s": float(max(j.admitted - j.arrival for j in done))})
    return res


def run_served(args, world, rank, local, dist):
    device = local if world > 1 else args.device
    res = measure_served(args.served_jobs, args.served_rate, device, args.hbm_budget_gb * 1e9, seed=7 + rank)
    if rank == 0:
        line = {"metric": METRIC, "value": res["value"], "unit": "agent-steps/s", "n_gpus": world,
                "steps": None, "warmup": 0, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "int32/f32/f64",
                "data": "synthetic (seeded; shapes and distributions of the configuration)",
                "config": {"workload": "served", "detail": "Poisson arrivals; grid n in {32,64,128,256}, agents "
                           "log-uniform [1e4,1e7], steps U[50,1000]; plain method's actions with per-job "
                           "b0, d0, p", "parallelism": f"replicas x{world}"},
                "served": res}
        print(json.dumps(line), flush=True)
    return 0


def run_ensemble(args, world, rank, local, dist):
    device = local if world > 1 else args.device
    res = measure_ensemble(args.ensemble_runs, args.ensemble_steps, device, args.plain_runs, seed=2024 + rank)
    if rank == 0:
        line = {"metric": METRIC, "value": res["value"], "unit": "agent-steps/s", "n_gpus": world,
                "steps": res["timed_steps"], "warmup": res["steps_per_run"] - res["timed_steps"],
                "ms_per_step": res["batched_ms"] / max(1, res["timed_steps"]), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "int32/f32/f64",
                "data": "synthetic (seeded; shapes and distributions of the configuration)",
                "config": {"workload": "ensemble", "detail": "batched ensemble: runs with grid n in {32,64,128}, "
                           "agents log-uniform [1e4,2e6], per-run b0, d0, p and seed; plain method's actions",
                           "parallelism": f"replicas x{world}"},
                "batched": res}
        print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=195)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS) + ["ensemble", "served"], default="large")
    ap.add_argument("--served-jobs", type=int, default=100)
    ap.add_argument("--served-rate", type=float, default=20.0)
    ap.add_argument("--hbm-budget-gb", type=float, default=150.0)
    ap.add_argument("--ensemble-runs", type=int, default=256)
    ap.add_argument("--ensemble-steps", type=int, default=500)
    ap.add_argument("--plain-runs", type=int, default=256)
    ap.add_argument("--seed", type=int, default=42)
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--profile-steps", type=int, default=3)
    ap.add_argument("--cpu-steps", type=int, default=10)
    ap.add_argument("--e2e-steps", type=int, default=0)
    ap.add_argument("--skip-e2e", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-batched", action="store_true")
    ap.add_argument("--skip-served", action="store_true")
    ap.add_argument("--skip-genetics", action="store_true")
    ap.add_argument("--genetics-steps", type=int, default=20)
    args = ap.parse_args()
    if args.warmup < 0 or args.steps < 0:
        ap.error("steps and warmup must be >= 0")
    world, rank, local, dist = init_dist(args)
    try:
        if args.impl == "reference":
            return run_reference(args, world, rank, dist)
        if args.workload == "ensemble":
            return run_ensemble(args, world, rank, local, dist)
        if args.workload == "served":
            return run_served(args, world, rank, local, dist)
        return run_ours(args, world, rank, local, dist)
    finally:
        if dist is not None:
            dist.destroy_process_group()


if __name__ == "__main__":
    sys.exit(main())
