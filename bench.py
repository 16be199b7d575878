#!/usr/bin/env python
"""Throughput of the EmDee hot path on GB300: atom-steps/s of velocity-Verlet MD.

Workload (the 1M-atom Lennard-Jones box): N = 4*64^3 = 1,048,576 atoms on an fcc
lattice jittered by U(+-0.05 sigma) (seed 86245), reduced density 0.8442
(L = 107.494), lj_cut with rc = 2.5, neighbor skin 0.3, Maxwell-Boltzmann
momenta at T* = 1.5 from EmDee_random_momenta, dt = 0.005.  One step is the
reference's velocity-Verlet loop body (test/common/contained.f90:63-72):
EmDee_boost(dt/2), EmDee_displace(dt), EmDee_boost(dt/2), with the potential
energy and virial of every step (Options%Compute at every step: the workload's
outputs are per-step forces, energy and virial), neighbor lists rebuilt
whenever the skin check fires.  FP32 pair math, FP64 positions, momenta,
energy and virial sums.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

`--impl reference` times the reference algorithm's CPU implementation (the
OpenMP C restatement in oracle/, all host threads) on the same workload.
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = dict(name="lj_fcc_1048576", N=4 * 64 ** 3, rho=0.8442, rc=2.5, skin=0.3, kT=1.5, dt=0.005,
                seed=86245, jitter=0.05, nprop=1)
METRIC = "atom-steps/s"
ORACLE_SO = os.path.join(ROOT, "oracle", "_build", "liboracle_emdee.so")


from emdee_gb300.workloads import KB, fcc, setup_water_box   # noqa: E402

def setup(lib, W, threads=1, precision=None):
    R, L = fcc(W["N"], W["rho"], W["jitter"], W["seed"])
    md = lib.system(threads, 1, W["rc"], W["skin"], W["N"])
    if precision is not None:
        lib.EmDee_set_precision(md, precision)
    lib.EmDee_set_pair_model(md, 1, 1, lib.EmDee_pair_lj_cut(1.0, 1.0), 0.0)
    lib.upload(md, "box", np.array([L]))
    lib.upload(md, "coordinates", R)
    lib.EmDee_random_momenta(C.byref(md), W["kT"], True, W["seed"])
    return md


def workload_config(W, world=1):
    """The config dict both arms print (same workload, same keys)."""
    cfg = {"workload": W["name"], "N": W["N"], "rho": W["rho"], "L": (W["N"] / W["rho"]) ** (1 / 3),
           "rc": W["rc"], "skin": W["skin"], "kT": W["kT"], "dt": W["dt"], "energies_every": W["nprop"],
           "parallelism": "replicas" if world > 1 else "single GPU",
           "l2": "no flush; per-step working set (R, P, F, packed positions, lists) ~0.4 GB > 129 MB L2"}
    return cfg


def vv(lib, md, W, nsteps, step0=0, per_step=None):
    dt, half, nprop = W["dt"], 0.5 * W["dt"], W["nprop"]
    boost, displace, ref, opts = lib.EmDee_boost, lib.EmDee_displace, C.byref(md), md.Options
    for k in range(nsteps):
        opts.Compute = ((step0 + k + 1) % nprop == 0)
        if per_step is not None:
            per_step[0](md)
        boost(ref, 1.0, 0.0, half)
        displace(ref, 1.0, 0.0, dt)
        boost(ref, 1.0, 0.0, half)
        if per_step is not None:
            per_step[1](md)


# ---------------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------------

class Clocks:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.path = tempfile.mktemp(suffix=".csv")
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def fp32_peak_tflops(torch):
    """Dense FP32 (CUDA-core) throughput measured here: cuBLAS SGEMM 8192^3 with
    TF32 disabled, best of 5."""
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    n = 8192
    a = torch.randn(n, n, device="cuda", dtype=torch.float32)
    b = torch.randn(n, n, device="cuda", dtype=torch.float32)
    for _ in range(2):
        a @ b
    best = 0.0
    for _ in range(5):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        a @ b
        e.record()
        e.synchronize()
        best = max(best, 2.0 * n ** 3 / (s.elapsed_time(e) * 1e-3) / 1e12)
    torch.backends.cuda.matmul.allow_tf32 = prev
    del a, b
    torch.cuda.empty_cache()
    return best


def read_traffic(name="pair_lj1m_traffic.txt", key="dram_bytes_per_launch"):
    """A per-launch figure (DRAM bytes by default) from a committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", name)
    try:
        for line in open(p):
            if line.startswith(key):
                return float(line.split()[1])
    except OSError:
        pass
    return None


# ---------------------------------------------------------------------------------
# CPU arm (oracle restatement, all host threads)
# ---------------------------------------------------------------------------------

def cpu_rate(W, budget_s, max_steps, warmup=1):
    from emdee_gb300.emdee import EmDee
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    lib = EmDee(ORACLE_SO)
    threads = os.cpu_count() or 1
    md = setup(lib, W, threads=threads)
    vv(lib, md, W, warmup)
    t0 = time.perf_counter()
    n = 0
    while n < max_steps and (time.perf_counter() - t0) < budget_s:
        vv(lib, md, W, 1, step0=warmup + n)
        n += 1
    t = time.perf_counter() - t0
    return W["N"] * n / t, threads, n, t


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    W = dict(WORKLOAD)
    rate, threads, n, t = cpu_rate(W, budget_s=150.0, max_steps=args.steps, warmup=args.warmup)
    line = {"impl": "reference", "metric": METRIC, "value": rate, "unit": "atom-steps/s", "n_gpus": args.gpus,
            "steps": n, "warmup": args.warmup, "ms_per_step": 1e3 * t / max(n, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded fcc lattice)",
            "config": workload_config(W, world=int(os.environ.get("WORLD_SIZE", "1"))),
            "cpu_baseline": {"value": rate, "unit": "atom-steps/s", "cores": threads, "kind": "port",
                             "sample": "%d velocity-Verlet steps of the full %d-atom box (%.1f s, capped at 150 s)"
                                       % (n, W["N"], t)},
            "e2e": {"value": rate, "unit": "atom-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# ---------------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------------

def link_rates(torch, nbytes, reps=10):
    """Host link rates for reference: one cudaMemcpyAsync of nbytes each way between
    pinned host memory and the device (torch copy_, best of reps, CUDA events)."""
    h = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    d = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    out = {"bytes": nbytes}
    for name, dst, src in (("h2d_gbs", d, h), ("d2h_gbs", h, d)):
        best = 0.0
        for _ in range(reps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            dst.copy_(src, non_blocking=True)
            b.record()
            b.synchronize()
            best = max(best, nbytes / (a.elapsed_time(b) * 1e-3) / 1e9)
        out[name] = best
    del h, d
    return out


def max_over_ranks(x, world, device):
    """The largest value of x over the ranks of the job (x itself for one rank): the
    slowest rank's time defines the whole job's time."""
    if world <= 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank, ms, world, device):
    """Whole-job throughput: the units all ranks processed over the slowest rank's time.
    Returns (rate per second, slowest time in ms)."""
    ms_max = max_over_ranks(ms, world, device)
    return world * units_per_rank / (ms_max * 1e-3), ms_max


def run_gpu(args):
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from emdee_gb300.build import build
    build()
    import emdee_gb300
    lib = emdee_gb300.load()
    W = dict(WORKLOAD)
    N = W["N"]
    md = setup(lib, W, precision=emdee_gb300.MIXED)
    vv(lib, md, W, args.warmup)
    stream = torch.cuda.ExternalStream(lib.EmDee_cuda_stream(md))

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    # ---- timed region (device-resident state) ----
    clocks = Clocks(local)
    launches0 = lib.EmDee_launch_count(md)
    barrier()
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    builds0 = md.Builds
    torch.cuda.nvtx.range_push("timed")   # profilers can filter the timed launches: --nvtx-include timed/
    e0.record(stream)
    vv(lib, md, W, args.steps, step0=args.warmup)
    e1.record(stream)
    e1.synchronize()
    torch.cuda.nvtx.range_pop()
    barrier()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1)
    launches = lib.EmDee_launch_count(md) - launches0
    builds = md.Builds - builds0
    value, ms = job_rate(N * args.steps, ms, world, "cuda")

    # ---- per-kernel device times (same workload, CUDA events on the library stream) ----
    lib.EmDee_profile(md, 1)
    nprof = min(args.steps, 200)
    vv(lib, md, W, nprof, step0=args.warmup + args.steps)
    kms = (C.c_double * 6)()
    kn = (C.c_long * 6)()
    lib.EmDee_kernel_times(md, kms, kn, 6)
    lib.EmDee_profile(md, 0)
    names = ["skin", "build", "pack", "pair", "boost", "move"]
    per_kernel = {nm: {"launches": int(kn[i]), "ms_total": kms[i],
                       "us_per_launch": (1e3 * kms[i] / kn[i]) if kn[i] else None} for i, nm in enumerate(names)}
    listed, within = C.c_long(), C.c_long()
    lib.EmDee_pair_statistics(md, C.byref(listed), C.byref(within))
    flops = 8.0 * listed.value + 22.0 * within.value
    pair_s = kms[3] / kn[3] * 1e-3
    peaks, peak_kind = measured_peaks()
    fp32_peak = fp32_peak_tflops(torch)
    achieved = flops / pair_s / 1e12
    traffic = read_traffic()
    # theoretical FP32 rate: 152 SMs x 128 FMA lanes x 2 FLOP at the SM clock's maximum
    fp32_theory = 152 * 128 * 2 * (clk.get("sm_max_mhz") or 2070.0) * 1e6 / 1e12
    roofline = {"bound": "fp32", "kernel": "k_pair_mixed (pair forces)", "achieved": achieved,
                "peak": fp32_peak, "unit": "TFLOP/s", "frac": achieved / fp32_peak, "traffic": traffic,
                "peak_source": "cuBLAS SGEMM 8192^3, TF32 off, measured in this run",
                "peak_theoretical": fp32_theory, "frac_theoretical": achieved / fp32_theory,
                "flops_per_launch": flops, "half_list_pairs": listed.value, "pairs_within_rc": within.value,
                "us_per_launch": pair_s * 1e6}
    # the pair kernel's binding unit: the SM's shared-memory pipe, one wavefront per clock
    # per SM (wavefronts per launch from the committed ncu capture, ~55 % of them
    # bank-conflict replays of the position gathers)
    waves = read_traffic(key="shared_wavefronts_per_launch")
    smem_peak = 152 * (clk.get("sm_max_mhz") or 2070.0) * 1e6
    roofline_smem = None if waves is None else {
        "bound": "shared-memory pipe", "kernel": "k_pair_mixed (pair forces)",
        "achieved": waves / pair_s, "peak": smem_peak, "unit": "wavefronts/s", "frac": waves / pair_s / smem_peak,
        "wavefronts_per_launch": waves, "source": "profiles/pair_lj1m_traffic.txt (ncu) / CUDA-event launch time"}
    boost_bytes = 72.0 * N   # P read+write, F read (steps with energies only)
    # fused step (two deferred kicks + move + skin displacement + FP32 packing), unit masses:
    # P r/w 48, F 24, R r/w 48, R0 24, build-time position and charge 16, slot 4, packed position 16
    move_bytes = 172.0 * N
    hbm = peaks.get("hbm_gbs", 6800.0)
    boost_gbs = boost_bytes / (kms[4] / kn[4] * 1e-3) / 1e9 if kn[4] else None
    move_gbs = move_bytes / (kms[5] / kn[5] * 1e-3) / 1e9 if kn[5] else None
    roofline_hbm = {"bound": "hbm", "kernel": "k_step_fused (EmDee_displace: deferred boosts, move, skin, pack)",
                    "achieved": move_gbs, "peak": hbm,
                    "unit": "GB/s", "frac": (move_gbs / hbm) if move_gbs else None,
                    "traffic": read_traffic("step_fused_lj1m_traffic.txt"), "bytes_per_launch": move_bytes,
                    "peak_source": peak_kind, "boost_achieved_gbs": boost_gbs}

    # whole step against both ceilings: max(FLOPs / FP32 peak, bytes / HBM peak) per step
    # (pair FLOPs as above; 152 B per atom-step of integrator and force I/O)
    step_flops, step_bytes = flops, 152.0 * N
    step_s = ms / args.steps * 1e-3
    step_floor = max(step_flops / (fp32_peak * 1e12), step_bytes / (hbm * 1e9))
    roofline_step = {"bound": "fp32" if step_flops / (fp32_peak * 1e12) >= step_bytes / (hbm * 1e9) else "hbm",
                     "floor_us": step_floor * 1e6, "measured_us": step_s * 1e6, "frac": step_floor / step_s,
                     "flops_per_step": step_flops, "bytes_per_step": step_bytes}

    # ---- end to end through the C ABI with host buffers ----
    pin = lambda: torch.empty((N, 3), dtype=torch.float64, pin_memory=True).numpy()
    Ph, Rh = pin(), pin()
    lib.EmDee_download(md, b"momenta", Ph.ctypes.data_as(C.c_void_p))

    def pre(m):
        lib.EmDee_upload(C.byref(m), b"momenta", Ph.ctypes.data_as(C.c_void_p))

    def post(m):
        lib.EmDee_download(m, b"coordinates", Rh.ctypes.data_as(C.c_void_p))
        lib.EmDee_download(m, b"momenta", Ph.ctypes.data_as(C.c_void_p))

    ne2e = min(args.steps, 500)
    barrier()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    vv(lib, md, W, ne2e, step0=0, per_step=(pre, post))
    f1.record(stream)
    f1.synchronize()
    barrier()
    e2e_rate, e2e_ms = job_rate(N * ne2e, f0.elapsed_time(f1), world, "cuda")
    e2e = {"value": e2e_rate, "unit": "atom-steps/s", "h2d_bytes_per_step": 24 * N,
           "d2h_bytes_per_step": 48 * N + 40, "steps": ne2e, "ms_per_step": e2e_ms / ne2e,
           "per_step": "EmDee_upload(momenta) from pinned host memory, boost/displace/boost, "
                       "EmDee_download(coordinates) and EmDee_download(momenta) into pinned host memory",
           "link": link_rates(torch, 50 * 2 ** 20)}

    # ---- the other workloads: replica batch and rigid water (throughput only) ----
    extra = {}
    if rank == 0 and world == 1 and not args.no_extra:   # the other workloads: single-GPU runs only
        extra["lj_replicas_256"] = measure_replicas(lib, emdee_gb300, torch, args.replica_steps)
        extra["water_rigid_4096"] = measure_water(lib, emdee_gb300, torch, args.water_steps)
        if not args.no_hmc:
            extra["hmc_binary_lj_8000x64"] = measure_hmc(lib, torch, args.hmc_iterations, args.hmc_configs,
                                                        args.hmc_epochs)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:   # the CPU sample: rank 0 at N = 1 only
        rate, threads, n, t = cpu_rate(W, budget_s=20.0, max_steps=100)
        cpu = {"value": rate, "unit": "atom-steps/s", "cores": threads, "kind": "port",
               "sample": "%d velocity-Verlet steps of the full %d-atom box after 1 warm-up step (%.1f s)"
                         % (n, N, t)}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "atom-steps/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32 pair math, f64 state",
                "data": "synthetic (seeded fcc lattice, Maxwell-Boltzmann momenta)",
                "config": workload_config(W, world=world), "neighbor_builds_in_timed_region": builds,
                "tile_edge_cells": lib.EmDee_tile_edge(md),
                "block_threads": {"build": lib.EmDee_tile_threads(md, 0), "pair": lib.EmDee_tile_threads(md, 1)},
                "clocks": clk, "gpu_launches": int(launches), "roofline": roofline, "roofline_smem": roofline_smem, "roofline_hbm": roofline_hbm,
                "roofline_step": roofline_step,
                "kernels": per_kernel, "e2e": e2e, "cpu_baseline": cpu, "workloads": extra}
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


# 256 Lennard-Jones replicas, per replica from the seed: N ~ U[256, 8192],
# density ~ U[0.70, 0.90], T* ~ U[0.8, 2.0]; rc 2.5, skin 0.3, dt 0.005
REPLICAS = dict(n=256, seed=86245, rc=2.5, skin=0.3, dt=0.005, nprop=100)


def measure_replicas(lib, pkg, torch, steps, count=None):
    rng = np.random.default_rng(REPLICAS["seed"])
    mds, sizes = [], []
    for k in range(REPLICAS["n"] if count is None else count):
        N = int(rng.integers(256, 8193))
        rho, T = float(rng.uniform(0.70, 0.90)), float(rng.uniform(0.8, 2.0))
        R, L = fcc(N, rho, 0.05, REPLICAS["seed"] + k)
        md = lib.system(1, 1, REPLICAS["rc"], REPLICAS["skin"], N)
        lib.EmDee_set_precision(md, pkg.MIXED)
        lib.EmDee_set_pair_model(md, 1, 1, lib.EmDee_pair_lj_cut(1.0, 1.0), 0.0)
        lib.upload(md, "box", np.array([L]))
        lib.upload(md, "coordinates", R)
        lib.EmDee_random_momenta(C.byref(md), T, True, REPLICAS["seed"] + k)
        mds.append(md)
        sizes.append(N)
    arr = (C.POINTER(type(mds[0])) * len(mds))(*[C.pointer(m) for m in mds])
    b = lib.lib.EmDee_replicas_create(len(mds), C.cast(arr, C.c_void_p))
    lib.lib.EmDee_replicas_run(b, 10, REPLICAS["dt"], REPLICAS["nprop"])   # block-size tuning + warm-up
    builds0 = sum(m.Builds for m in mds)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    lib.lib.EmDee_replicas_run(b, steps, REPLICAS["dt"], REPLICAS["nprop"])
    torch.cuda.synchronize()
    t = time.perf_counter() - t0
    total = sum(sizes)
    out = {"metric": METRIC, "value": total * steps / t, "unit": "atom-steps/s", "replicas": len(mds),
           "atoms": total, "N_min": min(sizes), "N_max": max(sizes), "steps": steps, "ms": 1e3 * t,
           "block_size": lib.lib.EmDee_replicas_block_size(b),
           "pair_threads_per_atom": lib.lib.EmDee_replicas_pair_threads(b),
           "tuning": "block size (256, 512, 1024) x pair threads per atom (1, 2), timed on copies of the batch",
           "neighbor_builds": sum(m.Builds for m in mds) - builds0,
           "timing": "host clock around one EmDee_replicas_run (one graph launch: a persistent kernel over all "
                     "replicas, then the results read back), device synchronized on both sides",
           "data": "synthetic (seeded fcc lattices, Maxwell-Boltzmann momenta)"}
    lib.lib.EmDee_replicas_destroy(b)
    for m in mds:
        lib.lib.EmDee_destroy(C.byref(m))
    return out


def measure_water(lib, pkg, torch, steps):
    """4096 rigid SPC/E molecules (12,288 atoms), coul_damped_smoothed(0.2, 1.0),
    rc 10 A, skin 1 A, 300 K, dt 1 fs, exact rigid-body rotation, mixed precision."""
    md = setup_water_box(lib, 4096, 86245, precision=pkg.MIXED)
    lib.EmDee_random_momenta(C.byref(md), KB * 300.0, True, 86245)
    W = dict(dt=1.0, nprop=100)
    vv(lib, md, W, 5)
    stream = torch.cuda.ExternalStream(lib.EmDee_cuda_stream(md))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push("timed")
    e0.record(stream)
    vv(lib, md, W, steps, step0=5)
    e1.record(stream)
    e1.synchronize()
    torch.cuda.nvtx.range_pop()
    ms = e0.elapsed_time(e1)
    out = {"metric": METRIC, "value": 12288 * steps / (ms * 1e-3), "unit": "atom-steps/s", "atoms": 12288,
           "steps": steps, "ms_per_step": ms / steps,
           "timing": "CUDA events on the library stream around the velocity-Verlet loop",
           "errors_vs_fp64": water_errors(lib, pkg, md)}
    lib.lib.EmDee_destroy(C.byref(md))
    return out


def water_errors(lib, pkg, md):
    """Errors of the mixed-precision results at the run's final configuration against
    FP64 arithmetic on the same coordinates: a second system in the library's FP64
    mode, whose forces, energies and virial match the FP64 oracle to 1e-12
    (tests/test_gpu_water_box.py, tests/test_gpu_models.py)."""
    N = 12288
    R = lib.download(md, "coordinates", (N, 3))
    md.Options.Compute = True
    lib.EmDee_compute_forces(C.byref(md))
    F32 = lib.download(md, "forces", (N, 3))
    ref = setup_water_box(lib, 4096, 86245, precision=pkg.FP64)
    lib.upload(ref, "coordinates", R)
    ref.Options.Compute = True
    lib.EmDee_compute_forces(C.byref(ref))
    F64 = lib.download(ref, "forces", (N, 3))
    out = {"force_rel_rms": float(np.sqrt(((F32 - F64) ** 2).sum() / (F64 ** 2).sum())),
           "potential_rel": abs(md.Energy.Potential / ref.Energy.Potential - 1),
           "coulomb_rel": abs(md.Energy.Coulomb / ref.Energy.Coulomb - 1),
           "virial_rel": abs(md.Virial.Total / ref.Virial.Total - 1),
           "reference": "library FP64 mode at the final configuration of the run"}
    lib.lib.EmDee_destroy(C.byref(ref))
    return out


def measure_hmc(lib, torch, iterations, configs, epochs):
    """Surrogate-proposal HMC vs plain HMC on the same GPU: 64 chains of the 80:20 binary
    Lennard-Jones mixture (N = 8000, rho 1.2, T* 0.8, rc 2.5), 20-step trajectories of
    dt 0.004, Metropolis on the exact FP64 Hamiltonian.  The surrogate is trained first on
    configurations, energies and forces from plain MD of the same chains; acceptance and
    ESS/s are also reported for shorter trajectories of both kinds."""
    from emdee_gb300.surrogate import (Chains, Surrogate, ess, force_rmse, generate_data, plain_hmc,
                                       surrogate_hmc, train)
    N, Cn, steps, dt, kT = 8000, 64, 20, 0.004, 0.8
    ch = Chains(lib, Cn, N, 1000)
    t0 = time.perf_counter()
    Rs, Es, Fs = generate_data(ch, configs, 25, dt, kT, 7, burn=1000)
    torch.cuda.synchronize()
    t_data = time.perf_counter() - t0
    B = 8
    m = Surrogate(lib, B, N, ch.L, ch.types)
    m.init_params(3, float(Es.mean()) / N)
    ntr = int(0.9 * configs)
    t0 = time.perf_counter()
    hist = train(m, Rs[:ntr], Es[:ntr], Fs[:ntr], epochs, 3e-3, B, 5)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    rmse = force_rmse(m, Rs[ntr:], Fs[ntr:], B)
    rms = float(Fs[ntr:].double().pow(2).mean().sqrt())
    hm = Surrogate(lib, Cn, N, ch.L, ch.types)
    hm.set_params(m.get_params())
    burn = iterations // 5

    def run(kind, n_it, n_steps, seed):
        if kind == "plain":
            U, acc, secs = plain_hmc(ch, n_it, n_steps, dt, kT, seed)
            far = 0
        else:
            U, acc, secs, far = surrogate_hmc(ch, hm, n_it, n_steps, dt, kT, seed)
        e = ess(U[:, n_it // 5:])
        return {"ess": e, "seconds": secs, "ess_per_s": e / secs, "acceptance": acc, "trajectory_steps": n_steps,
                "iterations": n_it, "paths_beyond_list_skin": far}

    plain = run("plain", iterations, steps, 11)
    sur = run("surrogate", iterations, steps, 12)
    sweep = {}
    for L in (2, 5, 10):
        sweep[str(L)] = {"plain": run("plain", iterations // 2, L, 21 + L),
                         "surrogate": run("surrogate", iterations // 2, L, 31 + L)}
    best = max([sur] + [v["surrogate"] for v in sweep.values()], key=lambda r: r["ess_per_s"])
    best_plain = max([plain] + [v["plain"] for v in sweep.values()], key=lambda r: r["ess_per_s"])
    out = {"metric": "HMC ESS/s (energy-autocorrelation corrected, summed over chains)",
           "chains": Cn, "N": N, "iterations": iterations, "trajectory_steps": steps, "dt": dt,
           "plain": plain, "surrogate": sur,
           "surrogate_over_plain": (sur["ess_per_s"] / plain["ess_per_s"]) if plain["ess_per_s"] > 0 else None,
           "target_surrogate_over_plain": 3.0,
           # each method at its own best trajectory length
           "best_surrogate_over_best_plain": (best["ess_per_s"] / best_plain["ess_per_s"])
           if best_plain["ess_per_s"] > 0 else None,
           "best_trajectory_steps": {"plain": best_plain["trajectory_steps"], "surrogate": best["trajectory_steps"]},
           "by_trajectory_steps": sweep,
           "training": {"configurations": configs, "held_out": configs - ntr, "epochs": epochs, "seconds": t_train,
                        "data_seconds": t_data, "final_losses_energy_force": hist[-1],
                        "force_rmse_held_out": rmse, "force_rms_held_out": rms,
                        "force_rmse_relative": rmse / rms},
           "ess_method": "Sokal automatic window (c = 5) on the exact potential energy, first 20 % dropped"}
    m.close()
    hm.close()
    ch.close()
    return out


def run_workload(args):
    """One secondary workload alone, one JSON line (no headline fields): the replica
    batch (--replicas boxes, --replica-steps steps), the rigid water box (--water-steps
    steps) or repeated surrogate force evaluations of --chains chains of the 8000-atom
    binary mixture."""
    import torch
    from emdee_gb300.build import build
    build()
    import emdee_gb300
    lib = emdee_gb300.load()
    if args.workload == "replicas":
        out = measure_replicas(lib, emdee_gb300, torch, args.replica_steps, args.replicas)
    elif args.workload == "water":
        out = measure_water(lib, emdee_gb300, torch, args.water_steps)
    else:
        from emdee_gb300.surrogate import Chains, Surrogate
        ch = Chains(lib, args.chains, 8000, 1000)
        ch.run(20, 0.004, 20)
        m = Surrogate(lib, args.chains, 8000, ch.L, ch.types)
        m.init_params(3, -6.0)
        R = ch.gather("R")
        m.forces(R)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            E, F = m.forces(R, rebuild=False)
        torch.cuda.synchronize()
        t = time.perf_counter() - t0
        out = {"workload": "surrogate forces", "chains": args.chains, "N": 8000, "evaluations": args.steps,
               "ms_per_evaluation": 1e3 * t / args.steps,
               "network": "tcgen05" if os.environ.get("EMDEE_SG_MMA") != "sync" else "mma.sync"}
        m.close()
        ch.close()
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-extra", action="store_true", help="skip the replica-batch and water measurements")
    ap.add_argument("--replica-steps", type=int, default=1000)
    ap.add_argument("--no-hmc", action="store_true", help="skip the surrogate-HMC measurement")
    ap.add_argument("--hmc-iterations", type=int, default=100)
    ap.add_argument("--hmc-epochs", type=int, default=10)
    ap.add_argument("--hmc-configs", type=int, default=20000)
    ap.add_argument("--water-steps", type=int, default=500)
    ap.add_argument("--atoms", type=int, default=None,
                    help="smaller box of the same density (profiling runs); default 1,048,576")
    ap.add_argument("--workload", default=None, choices=["replicas", "surrogate-forces", "water"],
                    help="run one secondary workload alone and print its measurement (profiling runs)")
    ap.add_argument("--replicas", type=int, default=256, help="replica count of --workload replicas")
    ap.add_argument("--chains", type=int, default=8, help="chains of --workload surrogate-forces")
    args = ap.parse_args()
    if args.workload:
        run_workload(args)
        return
    if args.warmup < 3:
        args.warmup = 3
    if args.atoms:
        WORKLOAD["N"] = args.atoms
        WORKLOAD["name"] = "lj_fcc_%d" % args.atoms
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
