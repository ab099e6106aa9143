#!/usr/bin/env python3
"""Benchmark of the population evaluator: GPop/s on one GB300, batched vs plain.

Metric (the reference's own, src/interpreter/accelerator.cc:922): GPop/s =
sum over programs of size[i] x records / evaluation time, i.e. opcode x record
evaluations per second.

Default workload (--workload uneven): the uneven batch -- 64 independent
populations of 256-30000 programs (log-uniform), program lengths 4-256
opcodes (geometric, mean 40, random valid prefix trees over + - * / sin cos
exp log sqrt ^2), datasets of 100-1M records x 1-32 N(0,1) features with
targets from a random depth-5 expression + N(0,0.05) noise; EF
fabs((X)-(Y)), sum, protected functions, PDP with the reference's lane rule.
Synthetic data, seeded (no public dataset is involved).
A step is one evaluation of every population:
  value : the batched evaluator (ppi_batch_evaluate_device, one persistent
          launch over all populations, CUDA graph, autotuned shape), inputs
          resident in HBM, device time of K steps (CUDA events on the launching
          stream), L2 flushed between steps outside the events;
  plain : the same populations as 64 plain evaluations back to back
          (ppi_gpu_evaluate_device per population), same timing; the line
          asserts bit-identical fitness and best indices;
  e2e   : the batched evaluator through ppi_batch_evaluate with pinned host
          buffers: the upload of phenotype/ephemeral/size (each row's used
          prefix, packed by the library) and D2H of fitness + best indices
          inside the timed region (host wall clock, synchronous call).
--workload polynomial: the polynomial-regression configuration (100k records,
30000 genomes decoded on the GPU into programs <= 128 opcodes), one plain
evaluation per step.
Multi-GPU (torchrun): every rank evaluates its own batch (weak scaling, no
collective on the data path); value = all ranks' GPop / max rank time.

--impl reference times the reference's CPU implementation of the path (the
oracle port of src/interpreter/sequential.cc + the OpenCL kernels' per-program
loops, OpenMP over programs on all host cores) on a bounded sample of the same
workload per step.
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


def aggregate(times, counts, device, world):
    """Weak-scaling aggregation over ranks, the benchmark's only collective:
    the slowest rank's times and the sum of all ranks' work."""
    if world == 1:
        return [float(t) for t in times], [float(c) for c in counts]
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x) for x in times], dtype=torch.float64, device=device)
    c = torch.tensor([float(x) for x in counts], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(c, op=dist.ReduceOp.SUM)
    return t.tolist(), c.tolist()


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    return json.load(open(p)) if os.path.exists(p) else {}


def profile_value(name, key):
    """A figure from a committed ncu summary (profiles/<name>.md, `key: value`)."""
    p = os.path.join(ROOT, "profiles", name + ".md")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith(key + ":"):
            return float(line.split(":")[1])
    return None


def upload_bytes(sz, max_size):
    """Bytes the library's host entry points send for these programs from
    pinned rows (upload.cu): the rows as they are up to 64 MB, else sizes,
    offsets and each row's used prefix of tokens and ephemerals."""
    n = len(sz)
    if n * max_size * 8 <= 64 << 20:
        return n * max_size * 8 + n * 4
    tokens = int(np.where((sz >= 1) & (sz <= max_size), sz, 0).astype(np.int64).sum())
    align8 = lambda x: (x + 7) & ~7
    return align8(n * 4) + n * 8 + align8(tokens * 4) + tokens * 4


def profile_traffic(workload):
    """DRAM bytes (read + written) of one step's kernels from a committed ncu
    summary: the launch list of that workload, else its kernel profile."""
    v = profile_value("launches_" + workload, "traffic_bytes_per_step")
    return v if v is not None else profile_value("eval_kernel_" + workload, "traffic_bytes_per_launch")


def cpu_sample(wl, ph, eph, sz, budget_s, threads=0, chunk=0, alpha=1e-6):
    """Oracle port (OpenMP over programs) on the first programs of the
    population, all records, until budget_s of work:
    (GPop/s, programs, cores, seconds, the programs' fitness)."""
    from oracle import pyoracle
    pyoracle.build()
    o = pyoracle.Oracle(wl.rows, wl.grammar.symbol_table_arrays(), wl.error_fn, wl.cost,
                        wl.reduce_max, wl.protected, False, threads)
    cores = threads if threads > 0 else (os.cpu_count() or 1)
    chunk = chunk or 2 * cores
    done, ops, t, fits = 0, 0, 0.0, []
    while done < len(sz) and (t < budget_s or done == 0):
        k = min(chunk, len(sz) - done)
        t0 = time.perf_counter()
        fits.append(o.evaluate(ph[done:done + k], eph[done:done + k], sz[done:done + k],
                               wl.strategy, 1 if wl.strategy == "PP" else min(wl.nlin, 1024), alpha))
        t += time.perf_counter() - t0
        ops += int(sz[done:done + k].sum()) * wl.nlin
        done += k
    return ops / t / 1e9, done, cores, t, np.concatenate(fits)


def pop_oracle(p, sym, threads=0):
    """The oracle over one population's dataset and settings."""
    from oracle import pyoracle
    return pyoracle.Oracle(p["rows"], sym, p["error_fn"], None, bool(p.get("reduce_max", False)),
                           p["protected"], False, threads)


def batch_cpu_sample(pops, sym, fraction, threads=0, slice_index=0, sm_count=152):
    """Oracle port on a slice of every population's programs (a `fraction` of
    each, and at least one per core: the port runs programs in parallel; slice
    `slice_index` of the population, wrapping), all records, in each
    population's strategy and lane count:
    (GPop/s, programs, cores, seconds, [(population, slice, fitness)])."""
    from oracle import pyoracle
    from ppi_gpu import workloads
    pyoracle.build()
    cores = threads if threads > 0 else (os.cpu_count() or 1)
    ops, t, done, fits = 0, 0.0, 0, []
    for i, p in enumerate(pops):
        k = min(p["n"], max(cores, int(round(p["n"] * fraction))))
        lo = (slice_index * k) % max(1, p["n"] - k + 1)
        sl = slice(lo, lo + k)
        o = pop_oracle(p, sym, threads)
        strategy = p.get("strategy", "PDP")
        lanes = workloads.default_lanes(strategy, p["rows"].shape[0], sm_count)
        t0 = time.perf_counter()
        f = o.evaluate(p["phenotype"][sl], p["ephemeral"][sl], p["size"][sl], strategy, lanes, 0.0)
        t += time.perf_counter() - t0
        fits.append((i, sl, f))
        ops += int(p["size"][sl].astype(np.int64).sum()) * p["rows"].shape[0]
        done += k
    return ops / t / 1e9, done, cores, t, fits


# Input range of each opcode's throughput probe (others: [-3, 3]); binary
# opcodes take the constant 1.375 as right operand.
PROBE_DOMAIN = {"LOG": (1.0, 100.0), "LOG2": (1.0, 100.0), "LOG10": (1.0, 100.0),
                "SQRT": (1.0, 100.0), "EXP": (-5.0, 5.0), "EXP2": (-5.0, 5.0),
                "EXP10": (-3.0, 3.0), "GAMMA": (0.5, 5.0), "POW": (0.5, 3.0)}
_OP_RATES = {}


def op_rates(names, iters=8192):
    """Gop/s of each opcode's arithmetic alone on this GPU (the evaluator's
    fast-math routines in a register loop, libppi_opcost.so), less the loop's
    own cost; cached for the process."""
    import ctypes as C
    from ppi_gpu import build as B
    from ppi_gpu import grammar as G
    if not os.path.exists(B.OPCOST_LIB):
        B.build_opcost()
    L = C.CDLL(B.OPCOST_LIB)
    L.ppi_opcost_measure.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_float, C.c_float,
                                     C.c_float, C.POINTER(C.c_float), C.POINTER(C.c_double)]

    def measure(op, lo, hi):
        ms, n = C.c_float(), C.c_double()
        rc = L.ppi_opcost_measure(op, 1, iters, 3, lo, hi, 1.375, C.byref(ms), C.byref(n))
        if rc != 0:
            raise RuntimeError("op throughput probe failed (CUDA error %d)" % rc)
        return ms.value, n.value

    if "_loop" not in _OP_RATES:
        _OP_RATES["_loop"] = measure(-1, -3.0, 3.0)[0]
    for name in names:
        if name not in _OP_RATES:
            lo, hi = PROBE_DOMAIN.get(name, (-3.0, 3.0))
            ms, n = measure(G.OP[name], lo, hi)
            _OP_RATES[name] = n / max(ms - _OP_RATES["_loop"], 1e-4) / 1e6
    return {k: _OP_RATES[k] for k in names}


def opmix_roofline(achieved, prog_sets):
    """Op-mix-aware ceiling of a workload: its opcode x record count divided
    by the time its operators' arithmetic alone takes at the probed rates
    (terminals -- attributes, constants, literals -- cost nothing, and the
    interpreter, the tile staging and the error reduction cost nothing).
    prog_sets: (phenotype, size, records, symbol table) per population."""
    from ppi_gpu import grammar as G
    hist, total = {}, 0
    for ph, sz, nlin, (sv, so, _) in prog_sets:
        lut = dict(zip(np.asarray(sv).tolist(), np.asarray(so).tolist()))
        toks = ph[np.arange(ph.shape[1])[None, :] < sz[:, None]]
        vals, counts = np.unique(toks, return_counts=True)
        for v, c in zip(vals.tolist(), counts.tolist()):
            op = int(lut.get(v, 0))
            hist[op] = hist.get(op, 0) + c * int(nlin)
        total += int(sz.astype(np.int64).sum()) * int(nlin)
    ops = {G.OPS[o]: n for o, n in hist.items() if o >= G.OP["AND"]}
    rates = op_rates(sorted(ops))
    t = sum(n / (rates[k] * 1e9) for k, n in ops.items())
    ceiling = total / t / 1e9 if t > 0 else None
    return {"ceiling": round(ceiling, 1) if ceiling else None,
            "frac": round(achieved / ceiling, 4) if ceiling else None, "unit": "Gop/s",
            "terminal_share": round(1.0 - sum(ops.values()) / total, 4),
            "op_share": {k: round(n / total, 4) for k, n in sorted(ops.items())},
            "op_rates_gops": {k: round(v, 1) for k, v in sorted(rates.items())},
            "how": "operators' fast-math arithmetic alone, 8 independent values per thread, "
                   "whole GPU (libppi_opcost.so); terminals free"}


def parity_block(gpu, ref, gpu64=None, fp64=None, what="", ref64=None):
    """Fitness of the timed GPU path against the oracle on the same programs
    (the reference's sequential arithmetic in the same strategy's order: only
    the transcendental functions' rounding differs in fast math), and against
    an FP64 re-evaluation of a subsample (the error of float evaluation
    itself).  Relative differences are over programs finite on both sides;
    sentinel agreement is the share of programs both call non-finite or both
    finite."""
    gpu = np.asarray(gpu, np.float32)
    ref = np.asarray(ref, np.float32)
    fin = (gpu < 1e30) & (ref < 1e30)
    rel = np.abs(gpu[fin].astype(np.float64) - ref[fin]) / np.maximum(np.abs(ref[fin]), 1e-30)
    out = {"programs": int(len(gpu)), "against": "oracle port of the reference (sequential.cc "
           "arithmetic, same strategy order)" + what,
           "sentinel_agreement": round(float(((gpu >= 1e30) == (ref >= 1e30)).mean()), 5),
           "bitexact_frac": round(float((gpu.view(np.int32) == ref.view(np.int32)).mean()), 5),
           "max_rel_diff": float(rel.max()) if rel.size else 0.0,
           "median_rel_diff": float(np.median(rel)) if rel.size else 0.0,
           "frac_within_1e-5": round(float((rel <= 1e-5).mean()), 5) if rel.size else 1.0}
    if fp64 is not None:
        f = np.asarray(fp64, np.float64)

        def against_fp64(vals):
            g = np.asarray(vals, np.float64)
            ok = (g < 1e30) & np.isfinite(f)
            r64 = np.abs(g[ok] - f[ok]) / np.maximum(np.abs(f[ok]), 1e-300)
            return {"sentinel_agreement": round(float(((g >= 1e30) == ~np.isfinite(f)).mean()), 5),
                    "max_rel_err": float(r64.max()) if r64.size else 0.0,
                    "median_rel_err": float(np.median(r64)) if r64.size else 0.0,
                    "frac_within_1e-5": round(float((r64 <= 1e-5).mean()), 5) if r64.size else 1.0}
        # the same programs' reference float fitness against FP64: how far
        # float evaluation itself is from FP64 on them
        out["fp64"] = dict(against_fp64(gpu64), programs=int(len(f)),
                           reference_float=against_fp64(ref[:len(f)] if ref64 is None else ref64))
    return out


def batch_config(pops, work, extra):
    nprog = sum(p["n"] for p in pops)
    mixed = len({(p["strategy"], p["error_fn"], bool(p.get("reduce_max", False))) for p in pops}) > 1

    def count(key, v):
        return sum(1 for p in pops if p.get(key) == v)
    settings = ({"strategy": {s: count("strategy", s) for s in ("PP", "DP", "PDP")},
                 "error_fn": {e: count("error_fn", e) for e in ("abs", "squared")},
                 "reduce_max": sum(1 for p in pops if p.get("reduce_max"))}
                if mixed else {"strategy": "PDP", "error_fn": "abs", "reduce_max": False})
    return dict({"workload": "uneven-batch-%dpops%s" % (len(pops), "-mixed" if mixed else ""),
                 "populations": len(pops), "programs": int(nprog),
                 "records": [int(min(p["rows"].shape[0] for p in pops)),
                             int(max(p["rows"].shape[0] for p in pops))],
                 "features": [int(min(p["rows"].shape[1] - 1 for p in pops)),
                              int(max(p["rows"].shape[1] - 1 for p in pops))],
                 "max_size": 256, "mean_size": round(float(np.mean(np.concatenate(
                     [p["size"] for p in pops]))), 2),
                 "protected": True, "ops_per_step": int(work)}, **settings, **extra)


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    from oracle import pyoracle
    pyoracle.build()
    if args.workload in ("polynomial", "iris", "stream"):
        return run_reference_single(args)
    if args.workload == "adjoint":
        print(json.dumps({"impl": "reference", "unavailable":
                          "the reference has no constant adjoint (PPI evaluates fitness only)"}))
        return 0
    from ppi_gpu import workloads
    g, pops = workloads.uneven_batch(seed=11, n_pops=args.populations,
                                     pop_range=(256, args.max_programs),
                                     mixed=getattr(args, "mixed", False))
    sym = g.symbol_table_arrays()
    work = float(sum(int(p["size"].sum()) * p["rows"].shape[0] for p in pops))
    # each step: a bounded sample (a slice of every population's programs,
    # another slice each step, all records), the same fraction as the
    # cpu_baseline of the default line (smaller samples leave the 16 threads
    # waiting on each population's largest program)
    frac = args.cpu_fraction
    vals = []
    for k in range(args.warmup + args.steps):
        v, n, cores, t, _ = batch_cpu_sample(pops, sym, frac, slice_index=k)
        if k >= args.warmup:
            vals.append((v, t))
    value = float(np.mean([v for v, _ in vals]))
    ms = float(np.mean([t for _, t in vals]) * 1e3)
    sample = ("%.1f%% (at least one per core) of every population's programs (%d programs, another "
              "slice each step) x all records per step" % (100 * frac, n))
    line = {"impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": UNIT,
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(ms, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": batch_config(pops, work, {"impl": "oracle port of the reference CPU interpreter"}),
            "cpu_baseline": {"value": round(value, 4), "unit": UNIT, "cores": cores,
                             "kind": "port", "sample": sample},
            "e2e": {"value": round(value, 4), "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def run_reference_single(args):
    """The reference arm of the single-population workloads: the oracle port of
    the reference's CPU interpreter on the same workload as `run_polynomial`,
    each step a slice of the population (all records)."""
    from ppi_gpu import workloads
    from oracle import pyoracle
    if args.workload == "polynomial":
        wl, per_step = workloads.polynomial(nlin=args.records, population=args.population), 60
    elif args.workload == "iris":
        wl = workloads.iris_shaped(population=args.population)
        per_step = wl.population   # the whole population: a few ms of CPU work
    else:
        wl, per_step = workloads.streaming(nlin=args.records, population=args.population), 48
    ph, eph, sz = pyoracle.decode(wl.grammar, wl.genomes, wl.bits_per_gene,
                                  wl.bits_per_constant, wl.lo, wl.hi, wl.max_size)
    per_step = min(per_step, len(sz))
    vals = []
    for k in range(args.warmup + args.steps):
        lo = (k * per_step) % max(1, len(sz) - per_step + 1)
        v, n, cores, t, _ = cpu_sample(wl, ph[lo:lo + per_step], eph[lo:lo + per_step],
                                    sz[lo:lo + per_step], 0.0, 0, per_step)
        if k >= args.warmup:
            vals.append((v, t))
    value = float(np.mean([v for v, _ in vals]))
    ms = float(np.mean([t for _, t in vals]) * 1e3)
    sample = "%d programs of the %d-program population x all %d records per step" % (
        per_step, wl.population, wl.nlin)
    line = {"impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": UNIT,
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(ms, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": dict(wl.describe(), impl="oracle port of the reference CPU interpreter"),
            "cpu_baseline": {"value": round(value, 4), "unit": UNIT, "cores": cores,
                             "kind": "port", "sample": sample},
            "e2e": {"value": round(value, 4), "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def run_batch(args):
    """The uneven batch: batched evaluator vs 64 plain evaluations."""
    import torch
    import ppi_gpu
    from ppi_gpu import workloads
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1 and not torch.distributed.is_initialized():
        import torch.distributed as dist
        dist.init_process_group("nccl")
    g, pops = workloads.uneven_batch(seed=11 + rank, n_pops=args.populations,
                                     pop_range=(256, args.max_programs),
                                     mixed=getattr(args, "mixed", False))
    sym = g.symbol_table_arrays()
    ph = np.concatenate([p["phenotype"] for p in pops])
    eph = np.concatenate([p["ephemeral"] for p in pops])
    sz = np.concatenate([p["size"] for p in pops])
    work = float(sum(int(p["size"].sum()) * p["rows"].shape[0] for p in pops))
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev)
    sh = stream.cuda_stream
    d_ph, d_eph, d_sz = [torch.from_numpy(a).to(dev) for a in (ph, eph, sz)]
    n = len(sz)
    d_fit = torch.empty(n, dtype=torch.float32, device=dev)
    d_best = torch.empty(len(pops), dtype=torch.int32, device=dev)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)   # 256 MiB > L2
    be = ppi_gpu.BatchEvaluator(sym, 256, pops, args.math, device=local)
    flags = ppi_gpu.BATCH_GRAPH | ppi_gpu.BATCH_AUTOTUNE

    def step():
        be.evaluate_device(d_ph.data_ptr(), d_eph.data_ptr(), d_sz.data_ptr(), d_fit.data_ptr(),
                           d_best.data_ptr(), sh, flags)

    t0 = time.perf_counter()
    for _ in range(args.warmup):          # the first step autotunes the shape
        flush.zero_()
        step()
    torch.cuda.synchronize(dev)
    warm_s = time.perf_counter() - t0

    def timed(fn):
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(args.steps)]
        launches = 0
        for k in range(args.steps):
            flush.zero_()
            evs[k][0].record(stream)
            launches += fn()
            evs[k][1].record(stream)
        torch.cuda.synchronize(dev)
        return [a.elapsed_time(b) for a, b in evs], launches

    def batch_step():
        step()
        return be.last_launch_count()

    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    clocks = ClockSampler(local)
    clocks.start()
    step_ms, launches = timed(batch_step)
    clk = clocks.stop()
    if world > 1:
        torch.distributed.barrier()
    fit_b = d_fit.cpu().numpy().copy()
    best_b = d_best.cpu().numpy().copy()

    # plain: one evaluator per population, launched back to back
    plain_evs, offs, begin = [], [], 0
    for p in pops:
        e = ppi_gpu.Evaluator(sym, 256, p["n"], p["strategy"], 0, p["error_fn"], None,
                              bool(p.get("reduce_max", False)), True, args.math, device=local)
        e.set_dataset(p["rows"])
        plain_evs.append(e)
        offs.append(begin)
        begin += p["n"]
    p_fit = torch.empty_like(d_fit)
    p_best = torch.empty_like(d_best)

    def plain_step():
        cnt = 0
        for k, (e, o, p) in enumerate(zip(plain_evs, offs, pops)):
            e.evaluate_device(d_ph[o:].data_ptr(), d_eph[o:].data_ptr(), d_sz[o:].data_ptr(),
                              p["n"], 0.0, p_fit[o:].data_ptr(), p_best[k:].data_ptr(), sh)
            cnt += e.last_launch_count()
        return cnt

    for _ in range(args.warmup):
        plain_step()
    plain_ms, plain_launches = timed(plain_step)
    equal = (np.array_equal(p_fit.cpu().numpy().view(np.int32), fit_b.view(np.int32)) and
             np.array_equal(p_best.cpu().numpy(), best_b))
    assert equal, "batched and plain fitness differ"
    for e in plain_evs:
        e.close()

    # end to end through the C ABI with pinned host buffers
    h_ph = torch.from_numpy(ph).pin_memory().numpy()
    h_eph = torch.from_numpy(eph).pin_memory().numpy()
    h_sz = torch.from_numpy(sz).pin_memory().numpy()
    for _ in range(args.warmup):
        be.evaluate(h_ph, h_eph, h_sz, flags)
    if world > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        fit_e, best_e = be.evaluate(h_ph, h_eph, h_sz, flags)
    e2e_s = time.perf_counter() - t0
    assert np.array_equal(fit_e.view(np.int32), fit_b.view(np.int32))

    total_s = sum(step_ms) / 1e3
    plain_s = sum(plain_ms) / 1e3
    (total_s, e2e_s, plain_s), (all_ops,) = aggregate([total_s, e2e_s, plain_s], [work], dev, world)
    if rank != 0:
        return 0
    value = all_ops * args.steps / total_s / 1e9
    plain_v = all_ops * args.steps / plain_s / 1e9
    e2e = all_ops * args.steps / e2e_s / 1e9
    peaks = measured_peaks()
    sm_count = torch.cuda.get_device_properties(dev).multi_processor_count
    max_mhz = float(peaks.get("sm_max_mhz", 2070.0))
    peak = sm_count * 128 * max_mhz * 1e6 / 1e9          # FP32 lane-ops/s, in G
    block, grid, rows, tune = be.shape()
    kernel_ms = float(np.mean(step_ms))
    cpu_v, cpu_n, cpu_cores, cpu_t, cpu_fits = batch_cpu_sample(pops, sym, args.cpu_fraction,
                                                                sm_count=sm_count)
    parity = batch_parity(pops, sym, fit_b, cpu_fits, offs)
    # issue activity and DRAM traffic of the evaluator kernels over one step
    # of this same configuration (its launch-list capture); the PDP batch
    # falls back to its mid-size profile for the issue activity
    mixed = getattr(args, "mixed", False)
    profile = "uneven-mixed" if mixed else "uneven-batch"
    issue = profile_value("launches_" + profile, "issue_active_frac")
    if issue is None and not mixed:
        issue = profile_value("eval_batch_kernel_uneven-batch-mid", "issue_active_frac")
    traffic = profile_traffic(profile)
    # bytes a step must move at least: every dataset once, the programs in,
    # the fitness and best indices out
    algorithmic = int(sum(p["rows"].nbytes for p in pops) + ph.nbytes + eph.nbytes + sz.nbytes +
                      n * 4 + len(pops) * 4)
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(total_s * 1e3 / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": batch_config(pops, work, {
            "math": args.math, "block": block, "grid": grid, "tile_rows": list(rows),
            "autotune_ms": [round(t, 2) for t in tune], "warmup_s": round(warm_s, 2),
            "l2": "256 MiB buffer written between steps, outside the timed events; "
                  "the batch's datasets (%.0f MB) exceed L2" % (
                      sum(p["rows"].nbytes for p in pops) / 1e6)}),
        "plain": {"value": round(plain_v, 3), "unit": UNIT,
                  "ms_per_step": round(plain_s * 1e3 / args.steps, 4),
                  "launches_per_step": plain_launches // args.steps,
                  "speedup_batched_vs_plain": round(value / plain_v, 3),
                  "equal_fitness": bool(equal)},
        "e2e": {"value": round(e2e, 3), "unit": UNIT,
                "h2d_bytes_per_step": int(upload_bytes(sz, ph.shape[1])),
                "d2h_bytes_per_step": int(n * 4 + len(pops) * 4 + 4)},
        "gpu_launches": launches,
        "roofline": {"bound": "fp32_issue", "achieved": round(all_ops / world / (kernel_ms / 1e3) / 1e9, 2),
                     "peak": round(peak, 1), "unit": "Gop/s",
                     "frac": round(all_ops / world / (kernel_ms / 1e3) / 1e9 / peak, 4),
                     "peak_source": "SMs x 128 FP32 lanes x sm_max_mhz (MEASURED_PEAKS.json)",
                     "kernel": "translate + work order + eval_batch_kernel main and wide pass "
                               "(one graph launch per step)",
                     "kernel_ms": round(kernel_ms, 4),
                     "frac_at_median_clock": round(all_ops / world / (kernel_ms / 1e3) / 1e9 /
                                                   (sm_count * 128 * clk["sm_mhz"] / 1e3), 4)
                     if clk.get("sm_mhz") else None,
                     "issue_active_frac": issue,
                     "traffic": traffic,
                     "traffic_unit": "bytes per step (DRAM read + write, ncu)",
                     "algorithmic_bytes": algorithmic,
                     "traffic_over_algorithmic": round(traffic / algorithmic, 2) if traffic else None,
                     "opmix": opmix_roofline(all_ops / world / (kernel_ms / 1e3) / 1e9,
                                             [(p["phenotype"], p["size"], p["rows"].shape[0], sym)
                                              for p in pops])},
        "cpu_baseline": {"value": round(cpu_v, 4), "unit": UNIT, "cores": cpu_cores,
                         "kind": "port",
                         "sample": "first %.1f%% (at least one per core) of every population's "
                                   "programs (%d) x all records (%.1f s), oracle port, OpenMP "
                                   "over programs" % (
                                       100 * args.cpu_fraction, cpu_n, cpu_t)},
        "parity": parity,
        "clocks": clk,
    }
    return line


def batch_parity(pops, sym, fit_gpu, cpu_fits, offs, fp64_per_pop=2):
    """Parity block of the batch: the GPU fitness of the CPU sample's programs
    against the oracle's, and of its first programs per population against
    an FP64 re-evaluation."""
    from oracle import pyoracle
    gpu, ref, g64, f64, r64 = [], [], [], [], []
    for i, sl, f in cpu_fits:
        p = pops[i]
        gsl = fit_gpu[offs[i] + sl.start: offs[i] + sl.stop]
        gpu.append(gsl)
        ref.append(f)
        k = min(fp64_per_pop, sl.stop - sl.start)
        o = pop_oracle(p, sym)
        sub = slice(sl.start, sl.start + k)
        f64.append(o.evaluate64(p["phenotype"][sub], p["ephemeral"][sub], p["size"][sub]))
        g64.append(gsl[:k])
        r64.append(f[:k])
    return parity_block(np.concatenate(gpu), np.concatenate(ref), np.concatenate(g64),
                        np.concatenate(f64), ", each population in its own strategy and lanes",
                        np.concatenate(r64))


def run_adjoint(args):
    """Constant adjoint (config 4): gradient time vs one forward evaluation,
    accuracy against the FP64 adjoint on a sample, 5 refinement steps."""
    import torch
    import ppi_gpu
    from ppi_gpu import workloads
    from oracle import pyoracle
    g, rows, ph, ep, sz = workloads.adjoint(seed=21)
    n = len(sz)
    sym = g.symbol_table_arrays()
    ev = ppi_gpu.Evaluator(sym, ph.shape[1], n, "PDP", 0, "squared", None, False, True, args.math)
    ev.set_dataset(rows)
    work = float(sz.astype(np.int64).sum()) * rows.shape[0]
    for _ in range(args.warmup):
        ev.evaluate(ph, ep, sz)
        ev.constant_gradient(ph, ep, sz)
    fwd, adj = [], []
    for _ in range(args.steps):
        fit, _ = ev.evaluate(ph, ep, sz)
        fwd.append(ev.last_kernel_ms())
        grad = ev.constant_gradient(ph, ep, sz)
        adj.append(ev.last_kernel_ms())
    fwd_ms, adj_ms = float(np.median(fwd)), float(np.median(adj))
    # accuracy on a sample against the FP64 adjoint
    pyoracle.build()
    o = pyoracle.Oracle(rows, sym, "squared", None, False, True, False)
    k = min(n, 200)
    f64, g64 = o.adjoint64(ph[:k], ep[:k].astype(np.float64), sz[:k])
    _, gff = o.adjoint64(ph[:k], ep[:k].astype(np.float64), sz[:k], float_forward=True)
    # programs whose fitness and gradients are well inside float range
    ok = ((fit[:k] < 1e30) & np.all(np.isfinite(g64), 1) & np.all(np.isfinite(gff), 1) &
          np.all(np.abs(gff) < 1e30, 1) & np.all(np.abs(g64) < 1e30, 1))

    def rel_err(ref, got, rows_ok):
        a, b = ref[rows_ok], got[rows_ok].astype(np.float64)
        scale = np.maximum(np.abs(a).max(1, keepdims=True), 1e-12)
        m = a != 0
        return (np.abs(a - b) / np.maximum(np.abs(a), 1e-6 * scale))[m]
    # well conditioned: the float function's and the double function's
    # gradients agree to 1e-5 (oracle, float vs double forward values)
    cond = np.array([ok[i] and (lambda r: r.size == 0 or r.max() <= 1e-5)(
        rel_err(g64[i:i + 1], gff[i:i + 1], np.array([True]))) for i in range(k)])
    within = float((rel_err(g64, grad[:k], ok) <= 1e-4).mean())
    within_cond = float((rel_err(g64, grad[:k], cond) <= 1e-4).mean())
    # 5 gradient steps on the constants (Adam), re-judged by the plain evaluator
    const = g.symbols["T_CONST"]
    mask = np.zeros(ph.shape, bool)
    for i in range(n):
        mask[i, :sz[i]] = ph[i, :sz[i]] == const
    finite = fit < 3.0e38
    c = torch.from_numpy(ep.copy()).requires_grad_(False)
    opt_m = np.zeros_like(ep, dtype=np.float64)
    opt_v = np.zeros_like(ep, dtype=np.float64)
    cur = ep.astype(np.float64).copy()
    for t in range(1, 6):
        gr = np.nan_to_num(ev.constant_gradient(ph, cur.astype(np.float32), sz)).astype(np.float64)
        gr[~mask] = 0.0
        gr[~finite] = 0.0
        opt_m = 0.9 * opt_m + 0.1 * gr
        opt_v = 0.999 * opt_v + 0.001 * gr * gr
        cur -= 0.05 * (opt_m / (1 - 0.9 ** t)) / (np.sqrt(opt_v / (1 - 0.999 ** t)) + 1e-8)
    fit_end, _ = ev.evaluate(ph, cur.astype(np.float32), sz)
    keep = finite & (fit_end < 3.0e38)
    del c
    line = {"metric": "constant gradient GPop/s (opcode x record, forward + reverse sweep) on 1 GB300",
            "value": round(work / adj_ms / 1e6, 3), "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(adj_ms, 3), "higher_is_better": True,
            "dtype": "f32 (f64 partial sums)", "data": "synthetic (seeded)",
            "config": {"workload": "adjoint-100k-x8-pop10000", "records": int(rows.shape[0]),
                       "features": 8, "population": n, "mean_size": round(float(sz.mean()), 2),
                       "error_fn": "squared", "math": args.math},
            "forward_ms": round(fwd_ms, 3), "forward_gpops": round(work / fwd_ms / 1e6, 3),
            "gradient_over_forward": round(adj_ms / fwd_ms, 3),
            "within_1e-4_of_fp64_adjoint": round(within, 5),
            "within_1e-4_of_fp64_adjoint_well_conditioned": round(within_cond, 5),
            "sample_programs": int(ok.sum()), "well_conditioned_programs": int(cond.sum()),
            "refinement": {"steps": 5, "optimizer": "Adam lr 0.05",
                           "median_fitness_before": float(np.median(fit[keep])),
                           "median_fitness_after": float(np.median(fit_end[keep])),
                           "improved_fraction": round(float((fit_end[keep] < fit[keep]).mean()), 4)},
            "parity": parity_block(fit[:k], o.evaluate(ph[:k], ep[:k], sz[:k], "PDP", ev.lanes, 0.0),
                                   fit[:k], f64, ", forward fitness of the gradient's programs")}
    return line


def run_polynomial(args):
    import torch
    import ppi_gpu
    from ppi_gpu import workloads
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    if args.workload == "polynomial":
        wl = workloads.polynomial(seed=1234 + rank, nlin=args.records, population=args.population)
    elif args.workload == "iris":
        wl = workloads.iris_shaped(seed=99 + rank, population=args.population)
    else:
        wl = workloads.streaming(seed=7 + rank, nlin=args.records, population=args.population)
    ev = ppi_gpu.Evaluator(wl.grammar.symbol_table_arrays(), wl.max_size, wl.population,
                           wl.strategy, 0, wl.error_fn, wl.cost, wl.reduce_max, wl.protected,
                           args.math, device=local)
    ev.set_dataset(wl.rows)
    ev.set_grammar(wl.grammar)
    ev_geo = ev.geometry()
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

    (total_s, e2e_s), (all_ops,) = aggregate([total_s, e2e_s], [float(ops_per_step)], dev, world)
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
    # bytes a step must move at least: the dataset once, the programs in, the
    # fitness out
    algorithmic = int(wl.rows.nbytes + ph.nbytes + eph.nbytes + sz.nbytes + n * 4)
    cpu_v, cpu_n, cpu_cores, cpu_t, cpu_fit = cpu_sample(wl, ph, eph, sz, args.cpu_seconds)
    from oracle import pyoracle
    k64 = min(cpu_n, args.fp64_programs)
    f64 = pyoracle.Oracle(wl.rows, wl.grammar.symbol_table_arrays(), wl.error_fn, wl.cost,
                          wl.reduce_max, wl.protected, False).evaluate64(ph[:k64], eph[:k64],
                                                                         sz[:k64], 1e-6)
    parity = parity_block(fit_host[:cpu_n], cpu_fit, fit_host[:k64], f64,
                          ", %s over %d lanes" % (wl.strategy, ev.lanes))
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(total_s * 1e3 / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": dict(wl.describe(), lanes=ev.lanes, math=args.math,
                       sum_size=int(sz.sum()), ops_per_step=ops_per_step,
                       l2="256 MiB buffer written between steps, outside the timed events",
                       decode_ms=round(decode_ms, 3)),
        "e2e": {"value": round(e2e, 3), "unit": UNIT,
                "h2d_bytes_per_step": int(upload_bytes(sz, ph.shape[1])),
                "d2h_bytes_per_step": int(n * 4 + 4)},
        "gpu_launches": launches,
        "roofline": {"bound": "fp32_issue", "achieved": round(achieved, 2),
                     "peak": round(peak, 1), "unit": "Gop/s", "frac": round(achieved / peak, 4),
                     "peak_source": "SMs x 128 FP32 lanes x sm_max_mhz (MEASURED_PEAKS.json)",
                     "kernel": "eval_kernel", "kernel_ms": round(eval_mean, 4),
                     "frac_at_median_clock": round(achieved / (sm_count * 128 * clk["sm_mhz"] / 1e3), 4)
                     if clk.get("sm_mhz") else None,
                     "issue_active_frac": profile_value("launches_" + wl.name, "issue_active_frac"),
                     "traffic": traffic,
                     "traffic_unit": "bytes per step (DRAM read + write, ncu)",
                     "algorithmic_bytes": algorithmic,
                     "traffic_over_algorithmic": round(traffic / algorithmic, 2) if traffic else None,
                     "record_chunks": ev_geo[2],
                     "opmix": opmix_roofline(achieved, [(ph, sz, wl.nlin,
                                                         wl.grammar.symbol_table_arrays())])},
        "cpu_baseline": {"value": round(cpu_v, 4), "unit": UNIT, "cores": cpu_cores,
                         "kind": "port",
                         "sample": "first %d programs x all %d records (%.1f s), oracle port, "
                                   "OpenMP over programs" % (cpu_n, wl.nlin, cpu_t)},
        "parity": parity,
        "clocks": clk,
    }
    return line


# The benchmark's other configurations, reported beside the headline in the
# default line: (key, workload, population, records, steps at most, CPU seconds).
SUB_CONFIGS = [("iris", "iris", 1000, 150, 5, 3.0),
               ("polynomial", "polynomial", 30_000, 100_000, 5, 5.0),
               ("stream", "stream", 30_000, 4_000_000, 2, 5.0),
               ("adjoint", "adjoint", 10_000, 100_000, 5, 0.0),
               # the uneven batch with each population's strategy (PP / DP /
               # PDP), error function and reduction drawn at random: batched
               # vs plain at identical fitness over mixed settings
               ("uneven_mixed", "uneven-mixed", 0, 0, 3, 0.005)]


def sub_line(line):
    """A configuration's line without the keys the headline already states."""
    drop = ("metric", "n_gpus", "higher_is_better", "scaling", "vs_baseline", "data", "warmup")
    return {k: v for k, v in line.items() if k not in drop}


def run_sub_configs(args):
    out = {}
    for key, workload, population, records, steps, cpu_s in SUB_CONFIGS:
        a = argparse.Namespace(**vars(args))
        a.workload, a.steps = workload, min(args.steps, steps)
        t0 = time.perf_counter()
        if workload == "uneven-mixed":
            a.mixed, a.cpu_fraction = True, cpu_s
            line = run_batch(a)
        else:
            a.population, a.records, a.cpu_seconds = population, records, cpu_s
            line = run_adjoint(a) if workload == "adjoint" else run_polynomial(a)
        sub = sub_line(line)
        sub["wall_s"] = round(time.perf_counter() - t0, 1)
        out[key] = sub
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--math", default="fast", choices=["fast", "parity", "native"])
    ap.add_argument("--workload", default="uneven",
                    choices=["uneven", "uneven-mixed", "polynomial", "iris", "stream", "adjoint"])
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--cpu-fraction", type=float, default=0.015,
                    help="uneven batch: share of every population timed on the CPU")
    # smaller cases of the same workloads, for profiling captures only
    ap.add_argument("--populations", type=int, default=64)
    ap.add_argument("--max-programs", type=int, default=30_000)
    ap.add_argument("--records", type=int, default=100_000)
    ap.add_argument("--population", type=int, default=30_000)
    ap.add_argument("--fp64-programs", type=int, default=16,
                    help="programs re-evaluated in FP64 for the parity block")
    ap.add_argument("--no-configs", action="store_true",
                    help="default workload: skip the other configurations' sub-blocks")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup
    if args.workload == "stream" and args.records == 100_000:
        args.records = 4_000_000
    if args.workload == "iris" and args.population == 30_000:
        args.population = 1000
    args.mixed = args.workload == "uneven-mixed"
    if args.impl == "reference":
        return run_reference(args)
    if args.workload in ("polynomial", "iris", "stream"):
        line = run_polynomial(args)
    elif args.workload == "adjoint":
        line = run_adjoint(args)
    else:
        line = run_batch(args)
        # the other configurations, on one GPU only (under torchrun every rank
        # would hold all GPUs for them)
        if isinstance(line, dict) and dist_env()[1] == 1 and not args.no_configs:
            line["configs"] = run_sub_configs(args)
    if isinstance(line, dict):
        print(json.dumps(line))
    return 0


if __name__ == "__main__":
    sys.exit(main())
