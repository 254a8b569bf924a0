"""Benchmark: Monte Carlo transient of an RLC ladder, batched mixed precision.

Workload (one "step" = one full pass): 2048 instances of a 200-section RLC ladder
(R 50 Ohm, L 10 nH, C 1 pF, each x (1 + 0.1 N(0,1)), seeded), 0-1 V pulse with
100 ps rise and 5 ns width, trapezoidal rule, fixed 1 ps step, 10000 steps; every
unknown (602) is written at every step.  Metric: circuit-timesteps/sec.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload mc_transient|op|ac|uneven|adjoint]

--impl reference times the reference's CPU algorithm (the C restatement in oracle/,
rebuilding and refactoring the matrix every step as krets does) on the host cores.
Prints ONE JSON line on rank 0.  The default workload is the headline above; the others
are the remaining measured configurations of the solve path:
  op       plain operating point of a 1000-resistor ladder with shunts (n = 1001), solves/s
  ac       4096-point AC sweep (Decade 455, 1 Hz - 1 GHz) of a 500-section RC ladder, points/s
  uneven   4096 distinct random netlists (10-5000 nodes), operating point + 2000 BE steps
           at 1 ns each, circuit-timesteps/s
  adjoint  1024 x 1000-section RC ladder, TR 1 ns x 2000 steps, loss sum V(n20)^2 and its
           gradient w.r.t. every R and C (checkpoint every 100 steps), gradients/s
"""
from __future__ import annotations

import argparse
import ctypes
import faulthandler
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

N_INST = 2048
SECTIONS = 200
H = 1e-12
N_STEPS = 10000
SEED = 3
METRIC = "circuit-timesteps/sec batched vs plain GPU form at <=1e-9 rel err vs FP64"
UNIT = "circuit-timesteps/s"
WORKLOAD = "mc_transient_rlc_ladder_2048x200sec_tr_1ps_10000steps"
TRAFFIC_PER_CIRCUIT_STEP = (2.037667e9 + 36.881e6) / (2048 * 200)  # bytes, ncu capture


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu),
                 "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak_hbm():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


# ------------------------------------------------------------------ replicas (N > 1)
def select_device(local):
    """One GPU per rank: restrict the process to its GPU before the first CUDA call (the
    library uses the current device); an inherited device list is indexed by local rank."""
    vis = os.environ.get("CUDA_VISIBLE_DEVICES")
    devs = [d for d in vis.split(",") if d.strip()] if vis else []
    os.environ["CUDA_VISIBLE_DEVICES"] = devs[local % len(devs)] if devs else str(local)
    return os.environ["CUDA_VISIBLE_DEVICES"]


def shard_seed(rank):
    """Seed of a rank's instances: each rank runs its own shard of a larger Monte Carlo
    job (weak scaling), so no two ranks repeat the same values."""
    return SEED + 7919 * rank


def max_over_ranks(seconds, world):
    """The job's time is the slowest rank's (gloo all-reduce; no data-path collective)."""
    if world <= 1:
        return seconds
    import torch
    import torch.distributed as dist
    t = torch.tensor([seconds], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank, steps, world, seconds):
    """Whole-job throughput: the units every rank processed over the slowest rank's time."""
    return units_per_rank * steps * world / seconds


def workload(rank=0):
    from krets_gb300.generators import monte_carlo_values, rlc_ladder
    from krets_gb300.table import element_table
    c = rlc_ladder(SECTIONS)
    t = element_table(c)
    vals = monte_carlo_values(c, N_INST, sigma=0.1, seed=shard_seed(rank))
    return c, t, vals


def errs_vs_oracle(x, ref, cur_mask):
    """(norm-wise, element-wise) error against the FP64 oracle (oracle/compare.py)."""
    from oracle.compare import both
    return both(x, ref, cur_mask)


# ------------------------------------------------------------------ CPU timing (oracle)
def cpu_rate(t, vals, n, idxs, steps, faithful, threads):
    """Time the oracle's TR transient on `idxs` instances over `steps` steps with a
    thread pool (ctypes releases the GIL).  Returns circuit-timesteps/s."""
    from oracle import oracle as O
    O.lib()

    def one(i):
        ti = t.copy()
        ti["value"] = vals[i]
        O.tran(ti, n, H, steps, method="tr", lag=False, faithful=faithful)

    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=threads) as ex:
        list(ex.map(one, idxs))
    dt = time.perf_counter() - t0
    return len(idxs) * steps / dt, dt


def run_reference(args, rank, world):
    if rank != 0:
        return None
    c, t, vals = workload()
    threads = os.cpu_count() or 1
    steps_per_sample = 1000
    idxs = list(range(threads))
    for _ in range(args.warmup):
        cpu_rate(t, vals, c.size, idxs[:1], 50, True, 1)
    rates, times = [], []
    for _ in range(args.steps):
        r, dt = cpu_rate(t, vals, c.size, idxs, steps_per_sample, True, threads)
        rates.append(r)
        times.append(dt)
    value = len(idxs) * steps_per_sample * args.steps / sum(times)
    sample = (f"{len(idxs)} instances x {steps_per_sample} TR steps per step (of {N_INST} x {N_STEPS}), "
              "matrix rebuilt and refactored every step as the reference does")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded splitmix64 Monte Carlo values)",
        "config": {"workload": WORKLOAD, "instances": N_INST, "sections": SECTIONS, "h": H, "n_steps": N_STEPS,
                   "method": "trapezoidal", "seed": shard_seed(0), "parallelism": "host threads"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the Rust reference cannot be built here (no cargo, no crate registry); the C "
                "restatement of its algorithm in oracle/ stands in for it",
    }
    return line


# ------------------------------------------------------------------ GPU arm
def run_ours(args, rank, world):
    from krets_gb300 import _lib
    from krets_gb300.table import is_current_mask

    stage("headline: set-up")
    c, t, vals = workload(rank)
    n = c.size
    g = _lib.GpuCircuit(t, n)
    d_vals = _lib.DeviceArray(vals.shape).upload(vals)
    out_shape = (N_INST, N_STEPS + 1, n)
    d_out = _lib.DeviceArray(out_shape)
    out_bytes = d_out.nbytes

    def step(precision=_lib.PREC_DF):
        g.batch_tran(d_vals, H, N_STEPS, "tr", lag=False, precision=precision, out=d_out, n_inst=N_INST)

    for _ in range(max(3, args.warmup)):
        step()
        g.flush_l2()
    call_ms, kern_ms = [], []
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    l0 = _lib.launch_count()
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        for _ in range(args.steps):
            _lib.lib().krets_device_synchronize()
            step()
            _lib.lib().krets_device_synchronize()
            k, cm = g.timing()
            call_ms.append(cm)
            kern_ms.append(k)
            g.flush_l2()
    if world > 1:
        dist.barrier()
    launches = _lib.launch_count() - l0
    engine = g.last_launch()
    total_s = max_over_ranks(sum(call_ms) / 1e3, world)
    ctsteps = N_INST * N_STEPS
    value = job_rate(ctsteps, args.steps, world, total_s)

    # accuracy: sampled instances against the FP64 oracle over the full 10000 steps
    from oracle import oracle as O
    mask = is_current_mask(c)
    sample_idx = sorted(set(np.linspace(0, N_INST - 1, 32).astype(int).tolist()))
    O.lib()

    def oracle_ref(i):
        ti = t.copy()
        ti["value"] = vals[i]
        return i, O.tran(ti, n, H, N_STEPS, method="tr", lag=False)

    with ThreadPoolExecutor(max_workers=os.cpu_count() or 1) as ex:
        refs = dict(ex.map(oracle_ref, sample_idx))

    def sampled_err():
        worst = [0.0, 0.0]
        for i in sample_idx:
            host = np.empty((N_STEPS + 1, n))
            off = i * (N_STEPS + 1) * n * 8
            _lib.check(_lib.lib().krets_memcpy_d2h(host.ctypes.data_as(_lib.ctypes.c_void_p),
                                                   _lib.ctypes.c_void_p(d_out.ptr + off), host.nbytes))
            e = errs_vs_oracle(host, refs[i], mask)
            worst = [max(worst[0], e[0]), max(worst[1], e[1])]
        return worst

    errs = sampled_err()
    # the other two precision modes of the same engine, one pass each (not the headline)
    stage("headline: precision variants")
    variants = {}
    for name, prec in (("mixed_fp32_lu_df_refinement", _lib.PREC_MIXED), ("fp64", _lib.PREC_FP64)):
        step(prec)
        k, cm = g.timing()
        hist, fallbacks = g.refine_stats()
        e = sampled_err()
        variants[name] = {"value": ctsteps / (cm / 1e3), "unit": UNIT, "kernel_ms": k,
                          "max_rel_err_vs_fp64": e[0], "max_elementwise_err_vs_fp64": e[1]}
        if prec == _lib.PREC_MIXED:
            variants[name]["refinement_histogram"] = [int(v) for v in hist]
            variants[name]["fp64_fallbacks"] = int(fallbacks)

    # probe-only variant: the same double-float run writing one unknown each step, V(n20),
    # which the wavefront reaches within the 10 ns window (0.1 ns per section)
    probe_node = c.index_map["V(n20)"]
    d_probe_out = _lib.DeviceArray((N_INST, N_STEPS + 1, 1))
    probe_ms = []
    for r in range(3):
        g.flush_l2()
        g.batch_tran_probe(d_vals, H, N_STEPS, [probe_node], "tr", lag=False, out=d_probe_out, n_inst=N_INST)
        if r > 0:
            probe_ms.append(g.timing())
    probe_err = [0.0, 0.0]
    for i in sample_idx:
        probe_host = np.empty((N_STEPS + 1, 1))
        _lib.check(_lib.lib().krets_memcpy_d2h(probe_host.ctypes.data_as(_lib.ctypes.c_void_p),
                                               _lib.ctypes.c_void_p(d_probe_out.ptr + i * (N_STEPS + 1) * 8),
                                               probe_host.nbytes))
        e = errs_vs_oracle(probe_host, refs[i][:, [probe_node]], np.zeros(1, bool))
        probe_err = [max(probe_err[0], e[0]), max(probe_err[1], e[1])]
    del d_probe_out
    variants["probe_only_output_node"] = {
        "value": ctsteps / (statistics.mean(cm for _, cm in probe_ms) / 1e3), "unit": UNIT,
        "kernel_ms": statistics.mean(k for k, _ in probe_ms), "output": "V(n20) only, 8 B per circuit-step",
        "max_rel_err_vs_fp64": probe_err[0], "max_elementwise_err_vs_fp64": probe_err[1],
        "v_n20_max": float(np.abs(refs[0][:, probe_node]).max())}

    # plain GPU form: one instance, FP64, level-scheduled single-CTA kernels per step
    plain_steps = 2000
    g1 = _lib.GpuCircuit(t, n)
    g1.tran(H, 100, "tr", lag=False)
    t0 = time.perf_counter()
    g1.tran(H, plain_steps, "tr", lag=False)
    _, plain_ms = g1.timing()
    plain_rate = plain_steps / (plain_ms / 1e3)

    # roofline of the dominant kernel (the batched transient)
    alg_bytes = out_bytes - N_INST * n * 8 + vals.nbytes + N_INST * n * 8  # rows 1..N written, inputs read
    # DRAM bytes per circuit-step of k_tran_dfd from an ncu capture of 304 instances x
    # 1000 steps of the same ladder (dram__bytes_read.sum + dram__bytes_write.sum of that
    # launch divided by its circuit-steps), scaled to this launch
    traffic = TRAFFIC_PER_CIRCUIT_STEP * N_INST * N_STEPS
    k_s = statistics.mean(kern_ms) / 1e3
    peak, peak_kind = measured_peak_hbm()
    achieved = alg_bytes / k_s / 1e9

    stage("headline: CPU baseline")
    # CPU baseline: optimised oracle (factor once) on the host cores, bounded sample
    threads = os.cpu_count() or 1
    r1, dt1 = cpu_rate(t, vals, n, [0], 500, False, 1)
    # the reference's cost model (rebuild and refactor every step) on one core, short sample
    rf1, _ = cpu_rate(t, vals, n, [0], 200, True, 1)
    per_inst_s = N_STEPS / r1
    n_sample = max(threads, min(8 * threads, int(15.0 * threads / max(per_inst_s, 1e-3))))
    cpu_val, cpu_dt = cpu_rate(t, vals, n, list(range(n_sample)), N_STEPS, False, threads)

    stage("headline: end to end")
    # end to end: host values in, host waveforms out, through the C ABI, with the caller's
    # ordinary (pageable) host buffers: where the GPU shares the host's page tables
    # (NVLink-C2C) the kernel writes the waveforms into them in place while it runs, which
    # measured faster in steady state than registering the buffer and copying spans out.
    # The sample is every instance when the waveforms fit in 60 % of the available host
    # memory, else whole waves of the engine (instances resident at once).
    del d_out
    e2e_inst = N_INST
    wave = max(1, engine["instances_per_cta"] * engine["grid"])
    try:
        with open("/proc/meminfo") as f:
            avail_kb = int([ln for ln in f if ln.startswith("MemAvailable")][0].split()[1])
        fit = int(0.60 * avail_kb * 1024 // ((N_STEPS + 1) * n * 8))
        if fit < N_INST:
            e2e_inst = (fit // wave) * wave if fit >= wave else max(64, fit)
    except Exception:
        e2e_inst = 256
    host_out = _lib.host_buffer((e2e_inst, N_STEPS + 1, n))
    host_vals = np.ascontiguousarray(vals[:e2e_inst])
    e2e_ms = []
    for r in range(2 + max(1, min(args.steps, 3))):
        _lib.lib().krets_device_synchronize()
        g.batch_tran(host_vals, H, N_STEPS, "tr", lag=False, precision=_lib.PREC_DF, out=host_out)
        _lib.lib().krets_device_synchronize()
        if r > 1:
            e2e_ms.append(g.timing()[1])
    e2e_val = e2e_inst * N_STEPS * len(e2e_ms) / (sum(e2e_ms) / 1e3)
    e2e_d2h_gbs = e2e_inst * (N_STEPS + 1) * n * 8 * len(e2e_ms) / (sum(e2e_ms) / 1e3) / 1e9
    del host_out
    # the same sample with device-resident buffers: the host I/O's share of the e2e time
    dev_same = _lib.DeviceArray((e2e_inst, N_STEPS + 1, n))
    dvals = _lib.DeviceArray(host_vals.shape).upload(host_vals)
    same_ms = []
    for r in range(3):
        g.batch_tran(dvals, H, N_STEPS, "tr", lag=False, precision=_lib.PREC_DF, out=dev_same, n_inst=e2e_inst)
        if r > 0:
            same_ms.append(g.timing()[1])
    same_val = e2e_inst * N_STEPS * len(same_ms) / (sum(same_ms) / 1e3)
    del dev_same, dvals

    if rank != 0:
        return None
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": max(3, args.warmup), "ms_per_step": statistics.mean(call_ms), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64-factor, double-float (2xfp32) solves",
        "data": "synthetic (seeded splitmix64 Monte Carlo values)",
        "config": {"workload": WORKLOAD, "instances": N_INST, "sections": SECTIONS, "unknowns": n, "h": H,
                   "n_steps": N_STEPS, "method": "trapezoidal", "seed": shard_seed(rank),
                   "precision": "LU factored in FP64, applied as double-float pairs on FP32 pipes",
                   "l2": "flushed between timed steps (512 MB write); outputs 98.6 GB >> L2",
                   "parallelism": "replicas only (instances sharded per GPU)"},
        "max_rel_err_vs_fp64": errs[0],
        "max_elementwise_err_vs_fp64": errs[1],
        "accuracy_sample": f"instances {sample_idx} of {N_INST}, all {N_STEPS + 1} rows x {n} unknowns",
        "engine": engine,
        "precision_variants": variants,
        "plain_form": {"value": plain_rate, "unit": UNIT, "what": "1 instance, FP64, per-step kernels (CUDA graph); linear: factored once and reused, "
                               "as the batched form"},
        "batched_over_plain": value / plain_rate,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                     "traffic_note": "ncu DRAM bytes of a 2048 x 200-step capture scaled per circuit-step",
                     "kernel": f"k_tran_dfd<{engine['threads_per_instance']}, factors in "
                               f"{engine['factors']}>", "algorithmic_bytes_per_launch": alg_bytes},
        "cpu_baseline": {"value": cpu_val, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{n_sample} instances x {N_STEPS} TR steps, factor once, oracle/ C restatement",
                         "one_core_factor_once": r1, "one_core_refactor_every_step": rf1},
        "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": int(host_vals.nbytes),
                "d2h_bytes_per_step": int(e2e_inst * (N_STEPS + 1) * n * 8), "instances": e2e_inst,
                "instances_per_wave": wave, "device_resident_same_instances": same_val,
                "host_buffers": "pageable (ordinary arrays); the kernel writes the waveforms into the host "
                                "buffer in place over NVLink-C2C", "call_ms": e2e_ms,
                "waveform_out_gbs": e2e_d2h_gbs},
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
    }
    return line


# ------------------------------------------------------------------ other workloads
def _timed(args, step, flush, timing):
    """W >= 3 untimed steps, then K steps each bracketed by device synchronisation, L2
    flushed in between; returns per-step (kernel ms, call ms) from the library's events."""
    from krets_gb300 import _lib
    for _ in range(max(3, args.warmup)):
        step()
        flush()
    ks, cs = [], []
    for _ in range(args.steps):
        _lib.lib().krets_device_synchronize()
        step()
        _lib.lib().krets_device_synchronize()
        k, c = timing()
        ks.append(k)
        cs.append(c)
        flush()
    return ks, cs


def _line(args, world, metric, value, unit, workload, extra):
    line = {"metric": metric, "value": value, "unit": unit, "n_gpus": world, "steps": args.steps,
            "warmup": max(3, args.warmup), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "data": "synthetic (seeded splitmix64)", "config": {"workload": workload}}
    line.update(extra)
    return line


def _cpu_pool(fn, items, threads):
    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=threads) as ex:
        list(ex.map(fn, items))
    return time.perf_counter() - t0


def workload_op(args, world, reference):
    from krets_gb300 import _lib
    from krets_gb300.generators import config1_circuit
    from krets_gb300.table import element_table, is_current_mask
    from oracle import oracle as O
    c = config1_circuit()
    t = element_table(c)
    wl = "plain_op_resistor_ladder_1000_with_shunts_n1001"
    threads = os.cpu_count() or 1
    if reference:
        # one OP of one circuit, as krets runs it: a single-threaded solve (a second core
        # cannot shorten it); the all-core figure of independent solves is reported beside
        O.lib()
        reps = 200
        dt1 = _cpu_pool(lambda _: O.op(t, c.size), range(reps), 1)
        v = reps / dt1
        dtn = _cpu_pool(lambda _: O.op(t, c.size), range(reps * threads), threads)
        return _line(args, world, "OP solves/sec", v, "solves/s", wl,
                     {"impl": "reference", "dtype": "f64", "cpu_baseline": {"value": v, "unit": "solves/s",
                      "cores": 1, "kind": "port", "sample": f"{reps} OP solves, one at a time",
                      "independent_solves_all_cores": reps * threads / dtn, "all_cores": threads},
                      "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}})
    g = _lib.GpuCircuit(t, c.size)
    l0 = _lib.launch_count()
    with ClockSampler() as clk:
        ks, cs = _timed(args, g.op, g.flush_l2, g.timing)
    launches = _lib.launch_count() - l0
    x, _ = g.op()
    ref = O.op(t, c.size)
    err = errs_vs_oracle(x, ref, is_current_mask(c))
    reps = 200
    dt = _cpu_pool(lambda _: O.op(t, c.size), range(reps), 1)
    # throughput of independent parameter sets of the same circuit (batched OP, one CTA each)
    bvals = np.tile(t["value"], (1024, 1))
    g.batch_op(bvals)
    g.batch_op(bvals)
    batched_op = 1024 / (g.timing()[0] / 1e3)
    alg = (2000 * 8 + c.size * 8)
    k_s = statistics.mean(ks) / 1e3
    peak, pk = measured_peak_hbm()
    return _line(args, world, "OP solves/sec", 1e3 / statistics.mean(ks), "solves/s", wl, {
        "ms_per_step": statistics.mean(cs), "dtype": "f64", "max_rel_err_vs_fp64": err[0],
        "max_elementwise_err_vs_fp64": err[1],
        "batched_op_1024_parameter_sets": {"value": batched_op, "unit": "solves/s"},
        "roofline": {"bound": "hbm", "achieved": alg / k_s / 1e9, "peak": peak, "unit": "GB/s",
                     "frac": alg / k_s / 1e9 / peak, "traffic": None, "peak_kind": pk, "kernel": "k_op",
                     "algorithmic_bytes_per_launch": alg, "note": "latency bound (one 1001-unknown solve)"},
        "cpu_baseline": {"value": reps / dt, "unit": "solves/s", "cores": 1, "kind": "port",
                         "sample": f"{reps} OP solves, oracle/ C restatement"},
        "e2e": {"value": 1e3 / statistics.mean(cs), "unit": "solves/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": c.size * 8},
        "gpu_launches": int(launches), "clocks": clk.summary()})


def workload_ac(args, world, reference):
    from krets_gb300 import _lib
    from krets_gb300.analyses import AcAnalysis, Decade, generate_frequencies
    from krets_gb300.generators import rc_ladder_ac
    from krets_gb300.table import element_table, is_current_mask
    from oracle import oracle as O
    c = rc_ladder_ac()
    t = element_table(c)
    f = np.array(generate_frequencies(AcAnalysis(Decade(455), 1.0, 1e9)))
    wl = f"ac_sweep_rc_ladder_500sec_{len(f)}pts_decade455_1Hz_1GHz"
    threads = os.cpu_count() or 1
    if reference:
        O.lib()
        chunks = [f[i::threads * 4] for i in range(threads * 4)]
        dt = _cpu_pool(lambda fr: O.ac(t, c.size, fr), chunks, threads)
        v = len(f) / dt
        return _line(args, world, "AC points/sec", v, "points/s", wl,
                     {"impl": "reference", "dtype": "c128", "cpu_baseline": {"value": v, "unit": "points/s",
                      "cores": threads, "kind": "port", "sample": f"all {len(f)} points"},
                      "e2e": {"value": v, "unit": "points/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}})
    g = _lib.GpuCircuit(t, c.size)
    d_out = _lib.DeviceArray((1, len(f), c.size, 2))
    l0 = _lib.launch_count()
    with ClockSampler() as clk:
        ks, cs = _timed(args, lambda: g.batch_ac(None, f, precision=_lib.PREC_MIXED, out=d_out), g.flush_l2,
                        g.timing)
    launches = _lib.launch_count() - l0
    z = g.batch_ac(None, f, precision=_lib.PREC_MIXED)[0]
    e2e_ms = g.timing()[1]
    mask = is_current_mask(c)
    sample = np.arange(len(f))   # every point (the oracle takes ~1 s for all of them)
    refz = O.ac(t, c.size, f[sample])
    err = [0.0, 0.0]
    for j, i in enumerate(sample):   # per frequency point: each is its own system
        e = errs_vs_oracle(z[i], refz[j], mask)
        err = [max(err[0], e[0]), max(err[1], e[1])]
    dt = _cpu_pool(lambda fr: O.ac(t, c.size, fr), [f[:256]], 1)
    alg = len(f) * c.size * 16 + 1000 * 8
    k_s = statistics.mean(ks) / 1e3
    peak, pk = measured_peak_hbm()
    return _line(args, world, "AC points/sec", len(f) / k_s, "points/s", wl, {
        "ms_per_step": statistics.mean(cs), "dtype": "c64 factor, c128 refinement", "max_rel_err_vs_fp64": err[0],
        "max_elementwise_err_vs_fp64": err[1], "accuracy_sample": f"all {len(f)} points",
        "roofline": {"bound": "hbm", "achieved": alg / k_s / 1e9, "peak": peak, "unit": "GB/s",
                     "frac": alg / k_s / 1e9 / peak, "traffic": None, "peak_kind": pk, "kernel": "k_ac_batch<1>",
                     "algorithmic_bytes_per_launch": alg},
        "cpu_baseline": {"value": 256 / dt, "unit": "points/s", "cores": 1, "kind": "port",
                         "sample": "256 points, oracle/ C restatement"},
        "e2e": {"value": len(f) / (e2e_ms / 1e3), "unit": "points/s", "h2d_bytes_per_step": int(f.nbytes),
                "d2h_bytes_per_step": int(z.nbytes)},
        "gpu_launches": int(launches), "clocks": clk.summary()})


UNEVEN_CIRCUITS, UNEVEN_STEPS, UNEVEN_H = 4096, 2000, 1e-9


def fp64_spread(t, n, ref, cur):
    """Element-wise disagreement of two FP64 solvers over a BE trajectory: SciPy's SuperLU
    re-solving each step's right-hand side A x_ref[s] (the oracle's own solution) against
    x_ref[s].  On ill-conditioned netlists it bounds what per-value agreement any FP64
    solver can show."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as sla
    from oracle import oracle as O
    from oracle.compare import elementwise_err
    A, _ = O.assemble(t, n, mode="tran", h=UNEVEN_H, method="be", sol=ref[0])
    As = sp.csc_matrix(A)
    xs = sla.splu(As).solve(np.ascontiguousarray((As @ ref[1:].T)))
    return elementwise_err(xs.T, ref[1:], cur)


def workload_uneven(args, world, reference):
    from krets_gb300 import _lib
    from krets_gb300.generators import uneven_table
    from oracle import oracle as O
    wl = f"uneven_random_netlists_{UNEVEN_CIRCUITS}x10-5000nodes_op_be_1ns_{UNEVEN_STEPS}steps"
    threads = os.cpu_count() or 1
    metric = "circuit-timesteps/sec"
    if reference:
        O.lib()
        # bounded sample: every 64th netlist (sizes across the whole range), 200 steps
        idx = list(range(0, UNEVEN_CIRCUITS, 64))
        tabs = {i: uneven_table(i) for i in idx}
        steps = 200
        dt = _cpu_pool(lambda i: O.tran(tabs[i][0], tabs[i][1], UNEVEN_H, steps, method="be", lag=True), idx,
                       threads)
        v = len(idx) * steps / dt
        return _line(args, world, metric, v, "circuit-timesteps/s", wl,
                     {"impl": "reference", "dtype": "f64", "cpu_baseline": {"value": v, "unit": "circuit-timesteps/s",
                      "cores": threads, "kind": "port",
                      "sample": f"{len(idx)} netlists (every 64th) x {steps} BE steps, factor once"},
                      "e2e": {"value": v, "unit": "circuit-timesteps/s", "h2d_bytes_per_step": 0,
                              "d2h_bytes_per_step": 0}})
    tabs = [uneven_table(i) for i in range(UNEVEN_CIRCUITS)]
    t0 = time.perf_counter()
    m = _lib.MultiCircuit([t for t, _ in tabs], [n for _, n in tabs], method="be", h=UNEVEN_H)
    create_s = time.perf_counter() - t0
    out = _lib.DeviceArray(m.total(UNEVEN_STEPS))
    l0 = _lib.launch_count()
    g_flush = _lib.GpuCircuit(tabs[0][0], tabs[0][1])
    with ClockSampler() as clk:
        ks, cs = _timed(args, lambda: m.tran(UNEVEN_STEPS, out=out), g_flush.flush_l2, m.timing)
    launches = _lib.launch_count() - l0
    info = m.info()
    value = UNEVEN_CIRCUITS * UNEVEN_STEPS / (statistics.mean(ks) / 1e3)
    offs = m.offsets(UNEVEN_STEPS)
    # accuracy: small netlists of every size class and the largest ones (n >= 4000, dense
    # trailing blocks, the global-memory class), every unknown at every step
    ns = np.array([n for _, n in tabs])
    acc_idx = [0, 1, 2, 3, 7] + [int(i) for i in np.nonzero(ns >= 4000)[0][:2]] + [int(ns.argmax())]

    def acc_one(i):
        t, n = tabs[i]
        ref = O.tran(t, n, UNEVEN_H, UNEVEN_STEPS, method="be", lag=True)
        x = np.empty((UNEVEN_STEPS + 1) * n)
        _lib.check(_lib.lib().krets_memcpy_d2h(x.ctypes.data_as(_lib.ctypes.c_void_p),
                                               _lib.ctypes.c_void_p(out.ptr + 8 * int(offs[i])), x.nbytes))
        cur = np.zeros(n, bool)
        cur[t["b"][t["b"] >= 0]] = True
        e = errs_vs_oracle(x.reshape(UNEVEN_STEPS + 1, n), ref, cur)
        return e[0], e[1], fp64_spread(t, n, ref, cur)

    with ThreadPoolExecutor(max_workers=threads) as ex:
        errs = list(ex.map(acc_one, acc_idx))
    # CPU baseline: the same bounded sample as the reference arm, factor once
    idx = list(range(0, UNEVEN_CIRCUITS, 64))
    cdt = _cpu_pool(lambda i: O.tran(tabs[i][0], tabs[i][1], UNEVEN_H, 200, method="be", lag=True), idx, threads)
    # end to end with a host output buffer: every netlist when the waveforms fit in 45 % of
    # the available host memory, else the first netlists up to 8 GB of waveforms
    del out
    try:
        with open("/proc/meminfo") as f:
            avail = int([ln for ln in f if ln.startswith("MemAvailable")][0].split()[1]) * 1024
    except Exception:
        avail = 0
    if m.total(UNEVEN_STEPS) * 8 <= 0.45 * avail:
        k, m2 = len(tabs), m
    else:
        k = 0
        tot = 0
        while k < len(tabs) and tot + (UNEVEN_STEPS + 1) * tabs[k][1] * 8 < 8e9:
            tot += (UNEVEN_STEPS + 1) * tabs[k][1] * 8
            k += 1
        m2 = _lib.MultiCircuit([t for t, _ in tabs[:k]], [n for _, n in tabs[:k]], method="be", h=UNEVEN_H)
    host = np.empty(m2.total(UNEVEN_STEPS))
    host.fill(0.0)
    for _ in range(3):
        m2.tran(UNEVEN_STEPS, out=host)
    e2e_call_s = m2.timing()[1] / 1e3
    e2e = k * UNEVEN_STEPS / e2e_call_s
    alg = (int(info[1]) * UNEVEN_STEPS + int(info[1])) * 8
    k_s = statistics.mean(ks) / 1e3
    peak, pk = measured_peak_hbm()
    return _line(args, world, metric, value, "circuit-timesteps/s", wl, {
        "ms_per_step": statistics.mean(cs), "dtype": "f64-factor, double-float (2xfp32) solves",
        "max_rel_err_vs_fp64": max(e[0] for e in errs), "max_elementwise_err_vs_fp64": max(e[1] for e in errs),
        "fp64_solvers_elementwise_spread": max(e[2] for e in errs),
        "per_netlist_errors": [{"netlist": i, "normwise": e[0], "elementwise": e[1], "fp64_spread": e[2]}
                               for i, e in zip(acc_idx, errs)],
        "accuracy_sample": f"netlists {acc_idx} (n = {[int(ns[i]) for i in acc_idx]}), all steps",
        "circuits": UNEVEN_CIRCUITS, "sum_unknowns": int(info[1]),
        "sum_lu_entries": int(info[2]), "circuits_per_class": info[4:10].tolist(),
        "class_end_ms": (info[10:16] / 1e3).tolist(), "symbolic_s": create_s,
        "roofline": {"bound": "hbm", "achieved": alg / k_s / 1e9, "peak": peak, "unit": "GB/s",
                     "frac": alg / k_s / 1e9 / peak, "traffic": None, "peak_kind": pk,
                     "kernel": "k_multi_tran (all classes)", "algorithmic_bytes_per_launch": alg},
        "cpu_baseline": {"value": len(idx) * 200 / cdt, "unit": "circuit-timesteps/s", "cores": threads,
                         "kind": "port", "sample": f"{len(idx)} netlists (every 64th) x 200 BE steps, factor once"},
        "e2e": {"value": e2e, "unit": "circuit-timesteps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": int(host.nbytes), "circuits": k,
                "with_symbolic_pass": k * UNEVEN_STEPS / (e2e_call_s + create_s * k / UNEVEN_CIRCUITS),
                "note": "with_symbolic_pass adds the host symbolic pass and upload (krets_multi_create) "
                        "of these netlists to the call time"},
        "gpu_launches": int(launches), "clocks": clk.summary()})


ADJ_INST, ADJ_SECTIONS, ADJ_STEPS, ADJ_H, ADJ_K = 1024, 1000, 2000, 1e-9, 100
# DRAM bytes per instance-step of the adjoint (forward k_tran_dfd + reverse k_adjoint_dfd)
# from an ncu capture of 152 instances x 300 steps of the same ladder (0.56 + 704.66 MB
# read, 734.83 MB written): the segment states and lambda histories the two
# halves of the reverse kernel's CTAs exchange through L2/DRAM
ADJ_TRAFFIC_PER_INST_STEP = (0.56e6 + 704.66e6 + 734.83e6) / (152 * 300)


def workload_adjoint(args, world, reference):
    from krets_gb300 import _lib
    from krets_gb300.generators import rc_ladder_step, rc_ladder_step_values
    from krets_gb300.table import element_table
    from oracle import oracle as O
    c = rc_ladder_step(ADJ_SECTIONS)
    t = element_table(c)
    out = c.index_map["V(n20)"]
    wl = f"adjoint_rc_ladder_{ADJ_INST}x{ADJ_SECTIONS}sec_tr_1ns_{ADJ_STEPS}steps_K{ADJ_K}_loss_sum_Vn20_sq"
    threads = os.cpu_count() or 1
    metric = "gradients/sec (loss + d loss / d every R and C)"
    # seeded values per instance (R log-uniform 100 Ohm-10 kOhm, C log-uniform 1-100 pF)
    vals = rc_ladder_step_values(c, ADJ_INST, seed=5)

    def table_of(i):
        ti = t.copy()
        ti["value"] = vals[i]
        return ti

    if reference:
        O.lib()
        n_s = 2 * threads
        dt = _cpu_pool(lambda i: O.adjoint_tran(table_of(i), c.size, ADJ_H, ADJ_STEPS, out), range(n_s), threads)
        v = n_s / dt
        return _line(args, world, metric, v, "gradients/s", wl,
                     {"impl": "reference", "dtype": "f64", "cpu_baseline": {"value": v, "unit": "gradients/s",
                      "cores": threads, "kind": "port", "sample": f"{n_s} FP64 adjoint gradients (oracle/)"},
                      "e2e": {"value": v, "unit": "gradients/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}})
    g = _lib.GpuCircuit(t, c.size)
    l0 = _lib.launch_count()
    res = {}
    with ClockSampler() as clk:
        ks, cs = _timed(args, lambda: res.__setitem__("r", g.adjoint_tran(vals, ADJ_H, ADJ_STEPS, out,
                                                                           checkpoint_every=ADJ_K)),
                        g.flush_l2, g.timing)
    launches = _lib.launch_count() - l0
    loss, grad = res["r"]
    # the two forward passes a gradient is compared with: the loss-only forward that the
    # gradient itself runs (checkpoints, no waveforms), and the transient writing every
    # waveform (16 GB)
    lks, _ = _timed(args, lambda: g.adjoint_tran(vals, ADJ_H, ADJ_STEPS, out, checkpoint_every=ADJ_K,
                                                 gradient=False), g.flush_l2, g.timing)
    fwd = _lib.DeviceArray((ADJ_INST, ADJ_STEPS + 1, c.size))
    fks, _ = _timed(args, lambda: g.batch_tran(vals, ADJ_H, ADJ_STEPS, "tr", lag=False, precision=_lib.PREC_DF,
                                                 out=fwd), g.flush_l2, g.timing)
    del fwd
    # accuracy: loss and gradient of sampled instances against the FP64 CPU adjoint
    samp = [0, ADJ_INST // 2, ADJ_INST - 1]
    with ThreadPoolExecutor(max_workers=threads) as ex:
        refs = list(ex.map(lambda i: O.adjoint_tran(table_of(i), c.size, ADJ_H, ADJ_STEPS, out), samp))
    gerr = max(float(np.max(np.abs(grad[i] - gr)) / np.max(np.abs(gr))) for i, (_, gr) in zip(samp, refs))
    lerr = max(abs(loss[i] - L) / L for i, (L, _) in zip(samp, refs))
    gref = refs[0][1]
    t0v = table_of(0)

    # central differences of the FP64 oracle loss on instance 0's 8 largest R/C gradients
    def fd_at(rel):
        rc = np.isin(t["kind"], (1, 2, 3))
        top = np.argsort(-np.where(rc, np.abs(gref), -1.0))[:8]

        def one(e):
            d = rel * t0v["value"][e]
            tp, tm = t0v.copy(), t0v.copy()
            tp["value"][e] += d
            tm["value"][e] -= d
            return (np.sum(O.tran(tp, c.size, ADJ_H, ADJ_STEPS, method="tr", lag=False)[1:, out] ** 2)
                    - np.sum(O.tran(tm, c.size, ADJ_H, ADJ_STEPS, method="tr", lag=False)[1:, out] ** 2)) / (2 * d)

        with ThreadPoolExecutor(max_workers=threads) as ex:
            fd = np.array(list(ex.map(one, top)))
        return top, fd

    top, fd = fd_at(1e-6)
    fd_err = float(np.max(np.abs(grad[0][top] - fd) / np.abs(fd)))
    fd_floor = float(np.max(np.abs(gref[top] - fd) / np.abs(fd)))  # FP64 adjoint vs the same differences
    # at h = 1e-6 the FP64 loss differences are rounding limited (~1e-6 relative); at
    # h = 1e-4 they are accurate to ~1e-9, so the gradient's own error shows
    top4, fd4 = fd_at(1e-4)
    fd4_err = float(np.max(np.abs(grad[0][top4] - fd4) / np.abs(fd4)))
    n_s = 2 * threads
    cdt = _cpu_pool(lambda i: O.adjoint_tran(table_of(i), c.size, ADJ_H, ADJ_STEPS, out), range(n_s), threads)
    k_s = statistics.mean(ks) / 1e3
    J = (ADJ_STEPS + ADJ_K - 1) // ADJ_K
    alg = ADJ_INST * (2 * c.elements.__len__() * 8 + 2 * J * c.size * 8)
    peak, pk = measured_peak_hbm()
    return _line(args, world, metric, ADJ_INST / k_s, "gradients/s", wl, {
        "ms_per_step": statistics.mean(cs), "dtype": "f64-factor, double-float (2xfp32) solves",
        "config_values": "seeded per instance (R log-U 100 Ohm-10 kOhm, C log-U 1-100 pF)",
        "loss_only_forward_ms": statistics.mean(lks), "waveform_forward_ms": statistics.mean(fks),
        "gradient_over_loss_only_forward": statistics.mean(ks) / statistics.mean(lks),
        "gradient_over_waveform_forward": statistics.mean(ks) / statistics.mean(fks),
        "loss_rel_err_vs_fp64_adjoint": lerr, "grad_rel_err_vs_fp64_adjoint": gerr,
        "accuracy_sample": f"instances {samp} against the FP64 CPU adjoint",
        "grad_rel_err_vs_central_fd_1e-6": fd_err, "fp64_adjoint_rel_err_vs_central_fd_1e-6": fd_floor,
        "grad_rel_err_vs_central_fd_1e-4": fd4_err,
        "roofline": {"bound": "hbm", "achieved": alg / k_s / 1e9, "peak": peak, "unit": "GB/s",
                     "frac": alg / k_s / 1e9 / peak, "traffic": ADJ_TRAFFIC_PER_INST_STEP * ADJ_INST * ADJ_STEPS,
                     "traffic_note": "ncu DRAM bytes of a 152 x 300-step capture scaled per instance-step; "
                                     "beyond the algorithmic bytes: segment states and lambda histories "
                                     "exchanged between the halves of the reverse kernel's CTAs",
                     "peak_kind": pk, "kernel": "k_tran_dfd (forward) + k_adjoint_dfd (reverse)", "algorithmic_bytes_per_launch": alg},
        "cpu_baseline": {"value": n_s / cdt, "unit": "gradients/s", "cores": threads, "kind": "port",
                         "sample": f"{n_s} FP64 adjoint gradients (oracle/)"},
        "e2e": {"value": ADJ_INST / (statistics.mean(cs) / 1e3), "unit": "gradients/s",
                "h2d_bytes_per_step": int(vals.nbytes), "d2h_bytes_per_step": int(grad.nbytes + loss.nbytes)},
        "gpu_launches": int(launches), "clocks": clk.summary()})


WORKLOADS = {"op": workload_op, "ac": workload_ac, "uneven": workload_uneven, "adjoint": workload_adjoint}
CONFIG_NAMES = {"op": "config 1: plain OP", "ac": "config 2: batched AC sweep", "uneven": "config 4: uneven batch",
                "adjoint": "config 5: adjoint sensitivity"}


def compact(line):
    """The fields of another configuration's line that the headline line carries."""
    keep = ("metric", "value", "unit", "impl", "ms_per_step", "max_rel_err_vs_fp64", "max_elementwise_err_vs_fp64",
            "accuracy_sample", "gradient_over_loss_only_forward", "gradient_over_waveform_forward",
            "loss_only_forward_ms", "waveform_forward_ms", "grad_rel_err_vs_fp64_adjoint",
            "grad_rel_err_vs_central_fd_1e-6", "grad_rel_err_vs_central_fd_1e-4", "symbolic_s", "class_end_ms",
            "batched_op_1024_parameter_sets", "gpu_launches", "clocks")
    c = {k: line[k] for k in keep if k in line}
    c["workload"] = line["config"]["workload"]
    if "roofline" in line:
        r = line["roofline"]
        c["roofline"] = {k: r.get(k) for k in ("kernel", "achieved", "peak", "frac", "traffic")}
    for k in ("e2e", "cpu_baseline"):
        if k in line:
            c[k] = line[k]
    return c


def stage(msg):
    """Progress on stderr (the JSON line is the only stdout output)."""
    print(f"[bench {time.strftime('%H:%M:%S')}] {msg}", file=sys.stderr, flush=True)


def other_configs(args, world, reference):
    """Configurations 1, 2, 4 and 5 at --steps 2 each (same timing rules), compacted."""
    a = argparse.Namespace(**vars(args))
    a.steps = 2
    out = {}
    for name, fn in WORKLOADS.items():
        stage(f"other configuration: {name}")
        t0 = time.perf_counter()
        try:
            c = compact(fn(a, world, reference))
        except Exception as e:  # a failing configuration is reported, not hidden
            c = {"error": f"{type(e).__name__}: {e}"}
        c["what"] = CONFIG_NAMES[name]
        c["wall_s"] = time.perf_counter() - t0
        out[name] = c
    return out


def main():
    faulthandler.enable()  # a native crash prints the Python stacks on stderr
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="mc_transient", choices=["mc_transient"] + sorted(WORKLOADS))
    ap.add_argument("--headline-only", action="store_true",
                    help="skip the other configurations' compact lines (other_configs)")
    args = ap.parse_args()
    rank, world, local = dist_env()
    if world > 1:
        # replicas: one process per GPU, instances sharded by replica, no data-path collective;
        # the process group is only for the barrier and the max-over-ranks time
        select_device(local)
        import torch.distributed as dist
        dist.init_process_group("gloo")
    if args.workload != "mc_transient":
        line = WORKLOADS[args.workload](args, world, args.impl == "reference")
        if rank == 0:
            print(json.dumps(line), flush=True)
        return
    if args.impl == "reference":
        line = run_reference(args, rank, world)
    else:
        line = run_ours(args, rank, world)
    if rank == 0 and line is not None:
        # the other configurations of the solve path, on one GPU (single-GPU runs only)
        if world == 1 and not args.headline_only:
            line["other_configs"] = other_configs(args, world, args.impl == "reference")
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
