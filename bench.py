#!/usr/bin/env python3
"""Benchmark of the population evaluator: GPop/s on one GB300.

Metric (the reference's own, src/interpreter/accelerator.cc:922): GPop/s =
sum over programs of size[i] x records / evaluation time, i.e. opcode x record
evaluations per second.

Workload: the polynomial-regression configuration -- 100k records
(x0 ~ U[-5,5], y = degree-4 polynomial with N(0,1) coefficients + N(0,0.01)
noise), 30000 genomes of 8-bit codons decoded by the arithmetic+^2 grammar
into programs of at most 128 opcodes, EF fabs((X)-(Y)), sum, protected
functions, PDP strategy with the reference's lane rule (1024 work-items per
program).  Synthetic data, seeded.

A step is one evaluation of the whole population (what one acc_interpret
call computes): translate + evaluate kernels, fitness + best index.
  value : inputs resident in HBM, device time of K steps (CUDA events on the
          launching stream), L2 flushed between steps outside the events;
  e2e   : the same through ppi_gpu_evaluate with pinned host buffers: H2D of
          phenotype/ephemeral/size and D2H of fitness + best index inside the
          timed region (host wall clock, synchronous call).
Multi-GPU (torchrun): every rank evaluates its own population (weak scaling,
no collective on the data path); value = all ranks' GPop / max rank time.

--impl reference times the reference's CPU implementation of the path (the
oracle port of src/interpreter/sequential.cc + the OpenCL PP kernel's
per-program loop, OpenMP over programs on all host cores) on a bounded sample
of the same workload per step.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "ppi-auto_gb300"))
sys.path.insert(0, ROOT)

METRIC = "GPop/s (opcode x record evals/s) on 1 GB300: batched vs plain, equal fitness"
UNIT = "GPop/s"


def dist_env():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4)
                          if r[5 + k].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    return json.load(open(p)) if os.path.exists(p) else {}


def profile_traffic(workload):
    """Per-launch DRAM bytes of the evaluator kernel from a committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "eval_kernel_%s.md" % workload)
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith("traffic_bytes_per_launch:"):
            return float(line.split(":")[1])
    return None


def cpu_sample(wl, ph, eph, sz, budget_s, threads=0, chunk=200):
    """Oracle port (OpenMP over programs) on the first programs of the
    population, all records, until budget_s of work: (GPop/s, programs, cores)."""
    from oracle import pyoracle
    pyoracle.build()
    o = pyoracle.Oracle(wl.rows, wl.grammar.symbol_table_arrays(), wl.error_fn, wl.cost,
                        wl.reduce_max, wl.protected, False, threads)
    done, ops, t = 0, 0, 0.0
    while done < len(sz) and (t < budget_s or done == 0):
        k = min(chunk, len(sz) - done)
        t0 = time.perf_counter()
        o.evaluate(ph[done:done + k], eph[done:done + k], sz[done:done + k], "PDP",
                   min(wl.nlin, 1024), 1e-6)
        t += time.perf_counter() - t0
        ops += int(sz[done:done + k].sum()) * wl.nlin
        done += k
    cores = threads if threads > 0 else (os.cpu_count() or 1)
    return ops / t / 1e9, done, cores, t


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    from ppi_gpu import workloads
    from oracle import pyoracle
    pyoracle.build()
    wl = workloads.polynomial()
    ph, eph, sz = pyoracle.decode(wl.grammar, wl.genomes, wl.bits_per_gene,
                                  wl.bits_per_constant, wl.lo, wl.hi, wl.max_size)
    # each step: a bounded sample (a fixed slice of the population, all records)
    per_step = 60
    vals = []
    for k in range(args.warmup + args.steps):
        lo = (k * per_step) % (len(sz) - per_step)
        v, n, cores, t = cpu_sample(wl, ph[lo:lo + per_step], eph[lo:lo + per_step],
                                    sz[lo:lo + per_step], 0.0, 0, per_step)
        if k >= args.warmup:
            vals.append((v, t))
    value = float(np.mean([v for v, _ in vals]))
    ms = float(np.mean([t for _, t in vals]) * 1e3)
    sample = "%d programs of the %d-program population x all %d records per step" % (
        per_step, wl.population, wl.nlin)
    line = {"impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": UNIT,
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(ms, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": dict(wl.describe(), impl="oracle port of the reference CPU interpreter"),
            "cpu_baseline": {"value": round(value, 4), "unit": UNIT, "cores": cores,
                             "kind": "port", "sample": sample},
            "e2e": {"value": round(value, 4), "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def run_ours(args):
    import torch
    import ppi_gpu
    from ppi_gpu import workloads
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    wl = workloads.polynomial(seed=1234 + rank, nlin=args.records, population=args.population)
    ev = ppi_gpu.Evaluator(wl.grammar.symbol_table_arrays(), wl.max_size, wl.population,
                           wl.strategy, 0, wl.error_fn, wl.cost, wl.reduce_max, wl.protected,
                           args.math, device=local)
    ev.set_dataset(wl.rows)
    ev.set_grammar(wl.grammar)
    t0 = time.perf_counter()
    ph, eph, sz = ev.decode(wl.genomes, wl.bits_per_gene, wl.bits_per_constant, wl.lo, wl.hi)
    decode_ms = ev.last_kernel_ms()
    n = len(sz)
    ops_per_step = int(sz.astype(np.int64).sum()) * wl.nlin

    dev = torch.device("cuda", local)
    d_ph = torch.from_numpy(ph).to(dev)
    d_eph = torch.from_numpy(eph).to(dev)
    d_sz = torch.from_numpy(sz).to(dev)
    d_fit = torch.empty(n, dtype=torch.float32, device=dev)
    d_best = torch.empty(1, dtype=torch.int32, device=dev)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)   # 256 MiB > L2
    stream = torch.cuda.current_stream(dev)
    sh = stream.cuda_stream

    def step():
        ev.evaluate_device(d_ph.data_ptr(), d_eph.data_ptr(), d_sz.data_ptr(), n, 1e-6,
                           d_fit.data_ptr(), d_best.data_ptr(), sh)

    for _ in range(args.warmup):
        flush.zero_()
        step()
    torch.cuda.synchronize(dev)
    # fitness of the device-resident path equals the host-API path
    fit_host, best_host = ev.evaluate(ph, eph, sz, 1e-6)
    assert np.array_equal(d_fit.cpu().numpy().view(np.int32), fit_host.view(np.int32))
    assert int(d_best.cpu()[0]) == best_host

    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    clocks = ClockSampler(local)
    clocks.start()
    ev_s = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ev_e = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    eval_ms = []
    launches = 0
    for k in range(args.steps):
        flush.zero_()
        ev_s[k].record(stream)
        step()
        ev_e[k].record(stream)
        eval_ms.append(ev.last_stage_ms()[1])
        launches += ev.last_launch_count()
    torch.cuda.synchronize(dev)
    if world > 1:
        torch.distributed.barrier()
    step_ms = [ev_s[k].elapsed_time(ev_e[k]) for k in range(args.steps)]
    total_s = sum(step_ms) / 1e3
    clk = clocks.stop()

    # end to end through the C ABI with pinned host buffers
    h_ph = torch.from_numpy(ph).pin_memory().numpy()
    h_eph = torch.from_numpy(eph).pin_memory().numpy()
    h_sz = torch.from_numpy(sz).pin_memory().numpy()
    for _ in range(args.warmup):
        ev.evaluate(h_ph, h_eph, h_sz, 1e-6)
    if world > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        fit_e2e, best_e2e = ev.evaluate(h_ph, h_eph, h_sz, 1e-6)
    e2e_s = time.perf_counter() - t0
    assert np.array_equal(fit_e2e.view(np.int32), fit_host.view(np.int32))

    tot = torch.tensor([total_s, e2e_s, float(ops_per_step)], dtype=torch.float64, device=dev)
    if world > 1:
        mx = tot.clone()
        torch.distributed.all_reduce(mx[:2], op=torch.distributed.ReduceOp.MAX)
        sm = tot.clone()
        torch.distributed.all_reduce(sm[2:], op=torch.distributed.ReduceOp.SUM)
        total_s, e2e_s, all_ops = float(mx[0]), float(mx[1]), float(sm[2])
    else:
        all_ops = float(ops_per_step)
    if rank != 0:
        return 0

    value = all_ops * args.steps / total_s / 1e9
    e2e = all_ops * args.steps / e2e_s / 1e9
    peaks = measured_peaks()
    sm_count = torch.cuda.get_device_properties(dev).multi_processor_count
    max_mhz = float(peaks.get("sm_max_mhz", 2070.0))
    peak = sm_count * 128 * max_mhz * 1e6 / 1e9          # FP32 lane-ops/s, in G
    eval_mean = float(np.mean(eval_ms))
    achieved = ops_per_step / (eval_mean / 1e3) / 1e9
    traffic = profile_traffic(wl.name)
    cpu_v, cpu_n, cpu_cores, cpu_t = cpu_sample(wl, ph, eph, sz, args.cpu_seconds)
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(total_s * 1e3 / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": dict(wl.describe(), lanes=min(wl.nlin, 1024), math=args.math,
                       sum_size=int(sz.sum()), ops_per_step=ops_per_step,
                       l2="256 MiB buffer written between steps, outside the timed events",
                       decode_ms=round(decode_ms, 3)),
        "e2e": {"value": round(e2e, 3), "unit": UNIT,
                "h2d_bytes_per_step": int(ph.nbytes + eph.nbytes + sz.nbytes),
                "d2h_bytes_per_step": int(n * 4 + 4)},
        "gpu_launches": launches,
        "roofline": {"bound": "fp32_issue", "achieved": round(achieved, 2),
                     "peak": round(peak, 1), "unit": "Gop/s", "frac": round(achieved / peak, 4),
                     "peak_source": "SMs x 128 FP32 lanes x sm_max_mhz (MEASURED_PEAKS.json)",
                     "kernel": "eval_kernel", "kernel_ms": round(eval_mean, 4),
                     "frac_at_median_clock": round(achieved / (sm_count * 128 * clk["sm_mhz"] / 1e3), 4)
                     if clk.get("sm_mhz") else None,
                     "traffic": traffic},
        "cpu_baseline": {"value": round(cpu_v, 4), "unit": UNIT, "cores": cpu_cores,
                         "kind": "port",
                         "sample": "first %d programs x all %d records (%.1f s), oracle port, "
                                   "OpenMP over programs" % (cpu_n, wl.nlin, cpu_t)},
        "clocks": clk,
    }
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--math", default="fast", choices=["fast", "parity", "native"])
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    # smaller cases of the same workload, for profiling captures only
    ap.add_argument("--records", type=int, default=100_000)
    ap.add_argument("--population", type=int, default=30_000)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
