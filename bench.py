"""Throughput of the GB300 amplitude path on the one-circuit, many-boundaries workload, with the
other configurations measured in the same run.

Workload of the headline: a seeded Clifford+T circuit with n=50 qubits, 2000 gates from
{H,S,CX,CZ,T} (exactly 32 T, seed 0: the radical-constrained branch subspace of the cached engine
has 2^29 > 2^22 branches), 4096 uniform output bitstrings y, x = 0, strategy auto (the
reference's Simulator::new default: 16 branch engines of d = 20..22).  One step evaluates all
4096 amplitudes.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

value      branches/s with boundaries resident in HBM (pq_amplitudes_device), CUDA events on
           the launching stream, L2 flushed (512 MiB write) between steps outside the events
e2e        same metric through the public host-buffer call pq_amplitudes (H2D of the
           boundaries and D2H of amplitudes + error bounds inside the timed region)
roofline   enumeration kernel: its FP32 FMA-pipe work (4 ops per enumerated branch) per launch
           over its event-timed duration, against the fma.f32 rate measured on the device and
           the nominal rate (SMs x 128 lanes x 2070 MHz); reference_form beside it: the
           reference engine's integer work for the same branches (5 W_o + 6 W_g int64 ops each)
           against the measured lop3 / popc rates
cfg1_small, cfg3_batched, cfg5_serve
           at N=1 the same line carries the single small amplitude (p50/p99 per call beside the
           CPU restatement's), the uneven 256-circuit batch (one graph launch vs the plain
           per-circuit and per-boundary paths, CPU restatement per branch-dimension bucket) and
           the served Poisson stream (throughput, p50/p99 at the offered load, below saturation
           and saturated); each leg with its own clock summary (nvidia-smi every 10 ms)
readme_statevector
           at N=1 also the reference README's own benchmark table (statevectors of its two seeded
           layered circuits, construction + statevector) beside the published CPU timings
workloads  --workload many_boundaries (default) | batched | serve | small | rotations | sample | estimate
           | readme
cpu_baseline  the CPU oracle (a restatement of the reference engine) on all host threads
--impl reference  times the same CPU restatement on the same workload (bounded sample)
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "polyq-v1.0_gb300"))

WORKLOAD = {"n_qubits": 50, "gates": 2000, "t_count": 32, "circuit_seed": 0, "boundaries": 4096,
            "output_seed": 1, "strategy": "auto"}
# FP32 FMA-pipe operations per enumerated branch in the enumeration kernel's walk
FMA_OPS_PER_BRANCH = 4
# FP32 FMA-pipe ops the bucket walk issues per branch: per group of 8 walked points of a unit of
# 8 chunks (64 branches), 16 paired FMA for the group sums and 8 to merge and add them into their
# buckets, 2 FP32 ops each
BUCKET_OPS_PER_BRANCH = 0.75
# DRAM bytes of one full-size enumeration launch (ncu, dram__bytes_read.sum + dram__bytes_write.sum)
TRAFFIC_BYTES_PER_LAUNCH = 8934656

METRIC = "branches/s and amplitudes/s at <=1e-6 rel err vs FP64; served p50/p99 latency"


def workload():
    from polyq_gb300.rng import random_outputs, workload_many_boundaries
    c = workload_many_boundaries(WORKLOAD["circuit_seed"])
    ys = random_outputs(WORKLOAD["n_qubits"], WORKLOAD["boundaries"], WORKLOAD["output_seed"])
    return c, ys


def config(extra=None):
    cfg = {"workload": "one circuit, many boundaries: n=50, 2000 gates, 32 T (seed 0), 4096 uniform y, x=0, "
                       "strategy auto",
           **WORKLOAD, "l2": "flushed between steps (512 MiB write)", "parallelism": "replicas"}
    if extra:
        cfg.update(extra)
    return cfg


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 10 ms while running (a timed region of
    20 headline steps lasts about 70 ms)."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = str(gpu_index)
        self.lines = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", self.gpu, "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "10"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.perf_counter(), line.strip()))

    def wait_first(self, timeout=3.0):
        """Block until the sampler has produced its first line (so the timed region is covered)."""
        t0 = time.perf_counter()
        while self.proc and not self.lines and time.perf_counter() - t0 < timeout:
            time.sleep(0.01)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self, t0=None, t1=None):
        """Median SM clock and active throttle reasons of the samples taken in [t0, t1] (all
        samples when no window is given or none fell inside it)."""
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        lines = [ln for t, ln in self.lines if t0 is None or (t0 <= t <= t1 + 0.015)]
        if not lines:
            lines = [ln for _, ln in self.lines]
        for ln in lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_init(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if args.impl == "gb300" else "gloo")
        return dist, int(os.environ.get("RANK", "0")), ws, int(os.environ.get("LOCAL_RANK", "0"))
    return None, 0, 1, 0


def max_over_ranks(dist, x):
    """Max of x over all ranks of the process group (x itself without one): the replica
    timing rule, a step lasts as long as the slowest rank."""
    if not dist:
        return x
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_rate(world_size, units_per_rank, ms):
    """Whole-job throughput of N independent replicas: all ranks' units over the slowest
    rank's time (ms)."""
    return world_size * units_per_rank / (ms * 1e-3)


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_rate(circ, ys, sample, threads):
    """CPU restatement of the reference engine on `sample` boundaries: (branches enumerated,
    seconds).  Branches of (boundary, branch engine) pairs whose sum vanishes are not counted:
    neither implementation enumerates them."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    sim = oracle.OracleSim(circ, "auto")
    sub = ys[:sample]
    sim.amplitudes([0], sub[:1], nthreads=threads)  # warm caches
    t0 = time.perf_counter()
    sim.amplitudes([0] * len(sub), sub, nthreads=threads)
    dt = time.perf_counter() - t0
    return sim.last_branches(), dt


def enumerated(L, N, sim, n):
    """Work of the last size-n launch: branches enumerated, reference-form int64 ops
    (5 W_o + 6 W_g per branch: src/normal_form.rs:479-493, src/engine.rs:700-718) and their
    popcount / logic split, plus the branches of each boundary."""
    import ctypes as ct

    import numpy as np
    out = (ct.c_double * 4)()
    per = np.zeros(n, dtype=np.float64)
    N.check(L.pq_sim_enumerated(sim.handle, n, out, per.ctypes.data_as(ct.POINTER(ct.c_double))))
    return out[0], out[1], out[2], out[3], per


def run_reference(args):
    dist, rank, ws, _ = dist_init(args)
    if rank != 0:
        return 0
    circ, ys = workload()
    threads = cpu_threads()
    sample = max(4, int(args.ref_sample))
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    sim = oracle.OracleSim(circ, "auto")
    for w in range(args.warmup):
        sim.amplitudes([0] * 2, ys[:2], nthreads=threads)
    times, branches = [], 0.0
    for k in range(args.steps):
        sub = ys[(k * sample) % len(ys):][:sample]
        t0 = time.perf_counter()
        sim.amplitudes([0] * len(sub), sub, nthreads=threads)
        times.append(time.perf_counter() - t0)
        branches += sim.last_branches()  # enumerated: vanishing (boundary, engine) pairs excluded
    ms = 1e3 * sum(times) / len(times)
    value = branches / sum(times)
    line = {"metric": METRIC, "impl": "reference", "value": value, "unit": "branches/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u64+f64", "data": "synthetic",
            "amplitudes_per_s": sample / (ms * 1e-3),
            "config": config({"sample_per_step": sample}),
            "cpu_baseline": {"value": value, "unit": "branches/s", "cores": threads, "kind": "port",
                             "sample": "%d of the 4096 boundaries per step, same circuit, strategy auto" % sample},
            "e2e": {"value": value, "unit": "branches/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_gb300(args):
    import ctypes as ct

    import numpy as np
    import torch

    dist, rank, ws, local = dist_init(args)
    torch.cuda.set_device(local)
    import polyq_gb300 as pq
    from polyq_gb300 import _native as N
    from polyq_gb300.sim import pack_bits
    L = N.lib()
    N.check(L.pq_init(local))
    circ, ys = workload()
    n = len(ys)
    if args.tuning:
        vals = [int(v) for v in args.tuning.split(",")] + [0]
        pq.set_tuning(inner_dims=vals[0], chunks_per_lane=vals[1], block_warps=vals[2], blocks_per_sm=vals[3],
                      unit_chunks=vals[4])
        args.no_autotune = True
    if args.chunk_tables:
        pq.set_tuning(chunk_tables=1)
    sim = pq.Simulator(circ, "auto")
    stats = sim.stats_full()
    tune_s = time.perf_counter()
    if args.no_autotune:
        tuning = sim.tuning()
    else:
        # launch shape chosen by the library's autotuner on this workload (outside the timed region)
        tuning, _ = sim.autotune([0] * n, ys, reps=2)
    tune_s = time.perf_counter() - tune_s
    xs_h = pack_bits([0] * n, circ.num_qubits)
    ys_h = pack_bits(ys, circ.num_qubits)
    dx = torch.from_numpy(xs_h.view(np.int64)).cuda()
    dy = torch.from_numpy(ys_h.view(np.int64)).cuda()
    dout = torch.zeros(2 * n, dtype=torch.float64, device="cuda")
    derr = torch.zeros(n, dtype=torch.float64, device="cuda")
    stream = torch.cuda.Stream()
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")

    def step_device():
        N.check(L.pq_amplitudes_device(sim.handle, n, ct.c_void_p(dx.data_ptr()), ct.c_void_p(dy.data_ptr()),
                                       ct.c_void_p(dout.data_ptr()), ct.c_void_p(derr.data_ptr()),
                                       ct.c_void_p(stream.cuda_stream)))

    kms = (ct.c_float * 3)()
    clk = ClockSampler(local).__enter__()
    clk.wait_first()
    with torch.cuda.stream(stream):
        for _ in range(max(3, args.warmup)):
            step_device()
        torch.cuda.synchronize()
        # work of one step: branches enumerated (vanishing pairs excluded) and reference-form ops
        branches_step, ops_step, popc_step, logic_step, per_boundary = enumerated(L, N, sim, n)
        peaks = (ct.c_double * 4)()
        fma2 = ct.c_double(0.0)
        tp0 = time.perf_counter()
        N.check(L.pq_measure_peaks(peaks))
        N.check(L.pq_measure_fma2_rate(ct.byref(fma2)))
        peak_clocks = clk.summary(tp0, time.perf_counter())
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        step_ms, enum_ms = [], []
        t_wall0 = time.perf_counter()
        for _ in range(args.steps):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step_device()
            e1.record(stream)
            e1.synchronize()
            step_ms.append(e0.elapsed_time(e1))
            N.check(L.pq_sim_kernel_ms(sim.handle, n, kms))
            enum_ms.append(kms[1])
        torch.cuda.synchronize()
        t_wall1 = time.perf_counter()
        t_wall = t_wall1 - t_wall0
        clocks = clk.summary(t_wall0, t_wall1)
        ms = sum(step_ms) / len(step_ms)
        ms = max_over_ranks(dist, ms)
        value = replica_rate(ws, branches_step, ms)
        # FP32 results of the last step against the device FP64 mode
        got = dout.cpu().numpy().view(np.complex128).copy()
        errb = derr.cpu().numpy().copy()
    ref = sim.amplitudes_fp64([0] * n, ys)
    rel = np.abs(got - ref) / np.abs(ref)
    # e2e through the public host-buffer call
    for _ in range(2):
        sim.amplitudes([0] * n, ys)
    e2e_s = []
    out_h = np.zeros(2 * n)
    err_h = np.zeros(n)
    import ctypes
    P = lambda a, t: a.ctypes.data_as(ctypes.POINTER(t))  # noqa: E731
    t_e2e0 = time.perf_counter()
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        N.check(L.pq_amplitudes(sim.handle, n, P(xs_h, ct.c_uint64), P(ys_h, ct.c_uint64), P(out_h, ct.c_double),
                                P(err_h, ct.c_double)))
        e2e_s.append(time.perf_counter() - t0)
    e2e_clocks = clk.summary(t_e2e0, time.perf_counter())
    e2e_ms = 1e3 * sum(e2e_s) / len(e2e_s)
    e2e_ms = max_over_ranks(dist, e2e_ms)
    e2e_value = replica_rate(ws, branches_step, e2e_ms)
    # roofline of the enumeration kernel against the FP32 FMA pipe.  The per-branch form of the
    # walk adds every branch's hi and lo complex weight pair: four FP32 FMA-pipe ops per branch,
    # the figure the line keeps as its unit so that rates stay comparable.  The bucket walk adds a
    # walked point's entry once for the eight chunks of its unit and issues 0.75 of them per
    # branch (48 per group of 8 points x 8 chunks: 32 for the group sums, 16 to merge them and
    # add them into their buckets); both fractions are reported.  Peak: the measured fma.f32 rate.
    enum_avg = sum(enum_ms) / len(enum_ms)
    lop3, popcr, fmar = peaks[0], peaks[1], peaks[2]
    # nominal FP32 FMA rate: 128 FP32 lanes per SM at the maximum SM clock (2070 MHz)
    fma_nominal = peaks[3] * 128 * 2.07e9
    fma_step = FMA_OPS_PER_BRANCH * branches_step
    achieved = fma_step / (enum_avg * 1e-3)
    # the reference engine's form of the same work: 5 W_o + 6 W_g int64 ops per branch, 2 popc.b32
    # per 64-bit popcount and 2 lop3.b32 per 64-bit logic op, at the measured pipe rates
    t_peak = max(2.0 * popc_step / popcr, 2.0 * logic_step / lop3)
    ops_branch = ops_step / branches_step
    ref_peak = ops_step / t_peak
    ref_achieved = ops_step / (enum_avg * 1e-3)
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:  # the CPU baseline is taken at N=1 only
        threads = cpu_threads()
        sample = max(4, int(args.cpu_sample))
        cbr, dt = cpu_rate(circ, ys, sample, threads)
        cpu = {"value": cbr / dt, "unit": "branches/s", "cores": threads, "kind": "port",
               "sample": "%d of the 4096 boundaries, same circuit and strategy (auto), CPU restatement of the "
                         "reference engine" % sample}
    line = {
        "metric": METRIC, "value": value, "unit": "branches/s", "n_gpus": ws, "steps": args.steps,
        "warmup": max(3, args.warmup), "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u64+f32", "data": "synthetic",
        "amplitudes_per_s": ws * n / (ms * 1e-3),
        "config": config({"branch_engines": stats["num_branches"], "pairs": stats["pairs"],
                          "branches_per_step": branches_step, "branches_counted": "enumerated (boundary, branch "
                          "engine) pairs only; pairs whose sum vanishes are zeros, not enumerated",
                          "wall_s_timed_region": t_wall, "tuning": tuning,
                          "method": "chunk-sum tables: one FP64 lookup per 2^10-branch chunk, branches counted as "
                                    "the reference enumerates them" if args.chunk_tables else
                                    "per-branch Gray enumeration",
                          "tuning_source": "fixed" if args.no_autotune else "pq_sim_autotune (%.1f s)" % tune_s}),
        "precision": {"max_rel_err_vs_fp64": float(np.max(rel)), "median_rel_err_vs_fp64": float(np.median(rel)),
                      "max_errbound_rel": float(np.max(errb / np.abs(ref)))},
        "e2e": {"value": e2e_value, "unit": "branches/s", "ms_per_step": e2e_ms, "clocks": e2e_clocks,
                "h2d_bytes_per_step": int(xs_h.nbytes + ys_h.nbytes),
                "d2h_bytes_per_step": int(out_h.nbytes + err_h.nbytes + 4)},
        "gpu_launches": 4 * args.steps,
        "roofline": {"bound": "fp32", "achieved": achieved / 1e12, "peak": fmar / 1e12, "unit": "Tops/s",
                     "frac": achieved / fmar, "traffic": TRAFFIC_BYTES_PER_LAUNCH,
                     "kernel": "enum_kernel", "kernel_ms": enum_avg,
                     "ops": "%d FP32 FMA-pipe ops per enumerated branch: the per-branch form (every branch's hi "
                            "and lo complex weight pair added)" % FMA_OPS_PER_BRANCH,
                     "executed_ops_per_branch": BUCKET_OPS_PER_BRANCH,
                     "frac_executed": achieved * BUCKET_OPS_PER_BRANCH / FMA_OPS_PER_BRANCH / fmar,
                     "executed_note": "the bucket walk adds each walked point's table entry once for the 8 chunks "
                                      "of its unit (one bucket per point, a Walsh-Hadamard transform per unit), "
                                      "0.75 FP32 FMA-pipe ops per branch: the FMA pipe is not its bound (ncu: "
                                      "profiles/enum_kernel_many_boundaries.md)",
                     "peak_source": "measured fma.f32 rate on this device (pq_measure_peaks), not a vendor figure",
                     "peak_sm_mhz": peak_clocks.get("sm_mhz"),
                     "peak_nominal": fma_nominal / 1e12, "frac_of_nominal": achieved / fma_nominal,
                     "peak_fma_f32x2": fma2.value / 1e12,
                     "frac_of_fma_f32x2": achieved / fma2.value if fma2.value > 0 else None,
                     "peak_fma_f32x2_source": "measured rate of the paired fma.rn.f32x2 form the walk issues "
                                              "(pq_measure_fma2_rate), FP32 ops",
                     "peak_nominal_source": "%d SMs x 128 FP32 lanes x 2070 MHz" % int(peaks[3]),
                     "traffic_source": "dram__bytes_read.sum + dram__bytes_write.sum of one full-size launch, "
                                       "ncu capture in profiles/enum_kernel_many_boundaries.md",
                     "reference_form": {
                         "ops_per_branch": ops_branch, "achieved": ref_achieved / 1e12, "peak": ref_peak / 1e12,
                         "unit": "Tops/s", "frac": ref_achieved / ref_peak,
                         "note": "the reference engine's int64 XOR/AND/POPC work per branch (5 W_o + 6 W_g) per "
                                 "second, against the rate its binding pipe allows at the measured lop3.b32 %.3e/s "
                                 "and popc.b32 %.3e/s; above 1 because the enumeration here does not execute "
                                 "that form" % (lop3, popcr)}},
        "clocks": clocks,
    }
    if args.chunk_tables:
        line["roofline"]["note"] = ("chunk-sum tables: chunks are table lookups, not enumerated; the FP32-pipe "
                                    "figures describe the enumeration and do not apply to this line")
    if cpu:
        line["cpu_baseline"] = cpu
    if rank == 0 and ws == 1 and not args.headline_only:
        # the other configurations, measured in the same run: the small single amplitude, the
        # uneven batch against its plain paths, the served Poisson stream
        line["cfg1_small"] = leg_small(args, clk)
        line["cfg3_batched"] = leg_batched(args, clk, cpu=not args.no_cpu)
        line["cfg5_serve"] = leg_serve(args, clk)
        line["readme_statevector"] = leg_readme(args, clk)
    clk.__exit__(None, None, None)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def _pct(xs, q):
    xs = sorted(xs)
    if not xs:
        return None
    return xs[min(len(xs) - 1, int(q * (len(xs) - 1) + 0.5))]


def _gpu_setup():
    import polyq_gb300 as pq
    from polyq_gb300 import _native as N
    N.check(N.lib().pq_init(0))
    return pq, N


def _bucket(d):
    return "d<=12" if d <= 12 else ("d13-18" if d <= 18 else "d>=19")


def cpu_batched_buckets(circs, dims, outs, enum_per_circuit, threads, budget_s=4.0):
    """CPU restatement on the uneven batch, per branch-dimension bucket: each bucket's
    circuits are evaluated in order (all 64 boundaries for d <= 18, 2 boundaries above) until
    `budget_s` of CPU time is spent; the bucket's remaining circuits are charged their
    enumerated branches (the same (boundary, engine) pairs the device enumerates) at the
    bucket's measured branch rate.  Returns {bucket: {...}}."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    by = {}
    for i, d in enumerate(dims):
        by.setdefault(_bucket(d), []).append(i)
    res = {}
    for key, idx in sorted(by.items()):
        spent, measured, br_meas = 0.0, {}, 0.0
        for i in idx:
            if spent >= budget_s:
                break
            c, d = circs[i][0], dims[i]
            k = 64 if d <= 18 else 2
            r = oracle.OracleSim(c, "auto")
            t0 = time.perf_counter()
            r.amplitudes([0] * k, outs[i][:k], nthreads=threads)
            dt = time.perf_counter() - t0
            spent += dt
            measured[i] = dt * 64.0 / k
            br_meas += r.last_branches() * 64.0 / k
        rate = br_meas / sum(measured.values()) if measured and sum(measured.values()) > 0 else None
        total = sum(measured.values())
        for i in idx:
            if i not in measured and rate:
                total += enum_per_circuit[i] / rate
        res[key] = {"circuits": len(idx), "measured_circuits": len(measured),
                    "cpu_amps_per_s": 64.0 * len(idx) / total if total > 0 else None,
                    "cpu_branches_per_s": rate, "cpu_seconds_for_bucket": total}
    return res


def leg_batched(args, clk=None, cpu=True):
    """Uneven batch: 256 circuits (n ~ U[16,64], 40n gates, T ~ U[8,36]), 64 uniform y each,
    one persistent graph launch per step vs the plain per-circuit and per-boundary paths."""
    import ctypes as ct

    import numpy as np
    import torch

    pq, N = _gpu_setup()
    L = N.lib()
    from polyq_gb300.rng import random_outputs, workload_batch
    if args.tuning:  # a fixed launch shape (profiling): no autotuning
        vals = [int(v) for v in args.tuning.split(",")] + [0]
        pq.set_tuning(inner_dims=vals[0], chunks_per_lane=vals[1], block_warps=vals[2], blocks_per_sm=vals[3],
                      unit_chunks=vals[4])
        args.no_autotune = True
    t0 = time.perf_counter()
    circs = workload_batch(256, seed=3)
    sims = [pq.Simulator(c) for c, _ in circs]
    build_s = time.perf_counter() - t0
    outs = [random_outputs(c.num_qubits, 64, 1000 + i) for i, (c, _) in enumerate(circs)]
    b = pq.Batch(sims, [64] * len(sims))
    xs, ys = b.pack([[0] * 64] * len(sims), outs)
    n = 64 * len(sims)
    t_tune = time.perf_counter()
    if args.no_autotune:
        tuning = None
    else:
        # chunk size, warps per block and chunks per table load chosen by the library's autotuner
        tuning, _ = b.autotune(xs, ys, reps=2)
    t_tune = time.perf_counter() - t_tune
    dx = torch.from_numpy(xs.view(np.int64)).cuda()
    dy = torch.from_numpy(ys.view(np.int64)).cuda()
    dout = torch.zeros(2 * n, dtype=torch.float64, device="cuda")
    stream = torch.cuda.Stream()
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    steps = max(1, args.batch_steps)
    with torch.cuda.stream(stream):
        for _ in range(max(3, args.warmup)):
            b.run_device(ct.c_void_p(dx.data_ptr()), ct.c_void_p(dy.data_ptr()), ct.c_void_p(dout.data_ptr()),
                         None, ct.c_void_p(stream.cuda_stream))
        torch.cuda.synchronize()
        ms, enum_ms = [], []
        kms = (ct.c_float * 3)()
        tw0 = time.perf_counter()
        for _ in range(steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            b.run_device(ct.c_void_p(dx.data_ptr()), ct.c_void_p(dy.data_ptr()), ct.c_void_p(dout.data_ptr()),
                         None, ct.c_void_p(stream.cuda_stream))
            e1.record(stream)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
            N.check(L.pq_batch_kernel_ms(b._h, kms))
            enum_ms.append(kms[1])
        tw1 = time.perf_counter()
    batched_ms = sum(ms) / len(ms)
    enum_avg = sum(enum_ms) / len(enum_ms)
    benum = (ct.c_double * 4)()
    N.check(L.pq_batch_enumerated(b._h, benum))
    got = dout.cpu().numpy().view(np.complex128)
    if args.batch_only:  # profiling: the batched launch alone
        return {"value": n / (batched_ms * 1e-3), "unit": "amplitudes/s", "ms_per_step": batched_ms,
                "enum_kernel_ms": enum_avg, "branches_per_s": benum[0] / (batched_ms * 1e-3), "tuning": tuning}
    # plain path 1: one launch per circuit (its 64 boundaries), host buffers, sequential
    for s, o in zip(sims, outs):
        for _ in range(2):  # plans built (first call) and graphs captured (second) outside the timing
            s.amplitudes([0] * 64, o)
    per_circ, plain_amps = [], []
    tp0 = time.perf_counter()
    for s, o in zip(sims, outs):
        t1 = time.perf_counter()
        plain_amps.append(s.amplitudes([0] * 64, o))
        per_circ.append(time.perf_counter() - t1)
    plain_circ_s = time.perf_counter() - tp0
    plain_all = np.concatenate(plain_amps)
    same = bool(np.array_equal(plain_all, got))
    scale = np.maximum(np.abs(plain_all), 1e-300)
    max_rel_diff = float(np.max(np.abs(plain_all - got) / scale))
    enum_circ = [enumerated(L, N, s, 64)[0] for s in sims]
    # plain path 2: one launch per (circuit, boundary)
    for s, o in zip(sims, outs):
        s.amplitudes_plain([0, 0], o[:2])
    tb0 = time.perf_counter()
    for s, o in zip(sims, outs):
        s.amplitudes_plain([0] * 64, o)
    plain_bnd_s = time.perf_counter() - tb0
    buckets = {}
    for s, t in zip(sims, per_circ):
        bk = buckets.setdefault(_bucket(s.stats_full()["branch_dim"]), [0, 0.0])
        bk[0] += 64
        bk[1] += t
    peaks = (ct.c_double * 4)()
    N.check(L.pq_measure_peaks(peaks))
    achieved = FMA_OPS_PER_BRANCH * benum[0] / (enum_avg * 1e-3)
    leg = {"value": n / (batched_ms * 1e-3), "unit": "amplitudes/s",
           "branches_per_s": benum[0] / (batched_ms * 1e-3), "ms_per_step": batched_ms, "steps": steps,
           "plain_per_circuit_amps_per_s": n / plain_circ_s, "plain_per_boundary_amps_per_s": n / plain_bnd_s,
           "speedup_vs_plain_per_circuit": plain_circ_s / (batched_ms * 1e-3),
           "speedup_vs_plain_per_boundary": plain_bnd_s / (batched_ms * 1e-3),
           "batched_equals_per_circuit_bitwise": same, "batched_vs_per_circuit_max_rel_diff": max_rel_diff,
           "enum_kernel_ms": enum_avg,
           "fma_pipe_frac_of_measured": achieved / peaks[2],
           "fma_pipe_frac_note": "per-branch form (4 FP32 FMA-pipe ops per branch) over the measured fma.f32 rate; "
                                 "the bucket walk executes 0.75 per branch (fraction %.3f)"
                                 % (achieved * BUCKET_OPS_PER_BRANCH / FMA_OPS_PER_BRANCH / peaks[2]),
           "per_d_bucket_amps_per_s_plain_per_circuit": {k: v[0] / v[1] for k, v in sorted(buckets.items())},
           "config": {"workload": "256 circuits, n~U[16,64], 40n gates, T~U[8,36] (seed 3), 64 uniform y each, "
                                  "x=0, strategy auto", "branches_enumerated_per_step": benum[0],
                      "branches_all_engines_per_step": b.branches, "host_build_s": build_s,
                      "l2": "flushed between steps (512 MiB write)", "tuning": tuning,
                      "tuning_source": "fixed" if tuning is None else "pq_batch_autotune (%.1f s)" % t_tune}}
    if clk is not None:
        leg["clocks"] = clk.summary(tw0, tw1)
        leg["clocks_plain_per_circuit"] = clk.summary(tp0, tp0 + plain_circ_s)
    if cpu:
        cb = cpu_batched_buckets(circs, [s.stats_full()["branch_dim"] for s in sims], outs, enum_circ, cpu_threads())
        tot = sum(v["cpu_seconds_for_bucket"] for v in cb.values())
        leg["cpu_baseline"] = {"value": n / tot, "unit": "amplitudes/s", "cores": cpu_threads(), "kind": "port",
                               "per_d_bucket": cb,
                               "sample": "per bucket, circuits in order until 4 s of CPU time (all 64 boundaries "
                                         "for d <= 18, 2 above); the rest charged their enumerated branches at "
                                         "the bucket's measured rate"}
    return leg


def run_batched(args):
    leg = leg_batched(args, cpu=not args.no_cpu)
    line = {"metric": METRIC, "workload": "batched", "n_gpus": 1, "higher_is_better": True, "data": "synthetic",
            "warmup": args.warmup, **leg}
    print(json.dumps(line), flush=True)
    return 0


def _rate(res):
    """Completed results over the span from the first submission to the last completion."""
    if not res:
        return None
    span = max(r["done_s"] for r in res) - min(r["submit_s"] for r in res)
    return len(res) / span if span > 0 else None


def leg_serve(args, clk=None):
    """Poisson stream of amplitude / probability / single-qubit-marginal requests against 64
    resident circuits (n~U[16,64], 40n gates, T~U[8,40]); throughput and p50/p99 latency at the
    offered load and below saturation, beside plain per-request launches."""
    import random

    pq, N = _gpu_setup()
    from polyq_gb300.rng import random_outputs, workload_batch
    from polyq_gb300.serve import MARGINAL, Server
    circs = [c for c, _ in workload_batch(64, seed=5, t_max=40)]
    sims = [pq.Simulator(c) for c in circs]
    srv = Server(sims, max_slots=args.slots, mem_budget_bytes=8 << 30, max_branch_dim=args.max_d)
    rng = random.Random(7)
    marg_qubits = 4  # marginal requests measure one of the first 4 qubits (engines built in warm-up)
    warm = [{"sim": k, "kind": MARGINAL, "x": 0, "qubit": q, "outcome": 0, "tag": -1}
            for k in range(len(sims)) for q in range(min(marg_qubits, circs[k].num_qubits))]
    srv.submit(warm)
    srv.collect(len(warm), 600)

    def make(i):
        k = rng.randrange(len(sims))
        kind = rng.randrange(3)
        n = circs[k].num_qubits
        return {"sim": k, "kind": kind, "x": 0, "y": random_outputs(n, 1, rng.randrange(1 << 30))[0],
                "qubit": rng.randrange(min(marg_qubits, n)), "outcome": rng.randrange(2), "tag": i}

    def load(rate, duration):
        nreq = int(rate * duration)
        arrivals = []
        t = 0.0
        for _ in range(nreq):
            t += rng.expovariate(rate)
            arrivals.append(t)
        reqs = [make(i) for i in range(nreq)]
        start = time.monotonic()
        w0 = time.perf_counter()
        i = 0
        while i < nreq:
            now = time.monotonic() - start
            j = i
            while j < nreq and arrivals[j] <= now:
                j += 1
            if j > i:
                srv.submit(reqs[i:j])
                i = j
            else:
                time.sleep(max(0.0, min(0.0005, arrivals[i] - now)))
        res = srv.collect(nreq, 600)
        w1 = time.perf_counter()
        ok = [r for r in res if r["status"] == 0]
        lat = [r["done_s"] - r["submit_s"] for r in ok]
        fg = [r for r in ok if r["pieces"] == 0]
        lat_fg = [r["done_s"] - r["submit_s"] for r in fg]
        lat_bg = [r["done_s"] - r["submit_s"] for r in ok if r["pieces"] > 0]
        span = (max(r["done_s"] for r in ok) - min(r["submit_s"] for r in ok)) if ok else 0.0
        okt = set(r["tag"] for r in ok if r["pieces"] == 0)  # the plain comparison takes one-wave requests
        out = {"offered_per_s": rate, "requests": nreq, "completed": len(ok),
               "refused": sum(1 for r in res if r["status"] == 3),
               "other_errors": sum(1 for r in res if r["status"] not in (0, 3)),
               "throughput_per_s": len(ok) / span if span > 0 else None,
               "evaluated_at_level": {name: sum(1 for r in ok if r["level"] == lv)
                                      for lv, name in enumerate(("fp32_walk", "chunk_tables", "fp64_walk"))},
               "p50_ms": 1e3 * _pct(lat, 0.5) if lat else None,
               "p99_ms": 1e3 * _pct(lat, 0.99) if lat else None,
               "one_wave": {"completed": len(lat_fg), "throughput_per_s": _rate(fg), "p50_ms": 1e3 * _pct(lat_fg, 0.5) if lat_fg else None,
                            "p99_ms": 1e3 * _pct(lat_fg, 0.99) if lat_fg else None},
               "background_pieces": {"completed": len(lat_bg),
                                     "pieces": sum(r["pieces"] for r in ok if r["pieces"] > 0),
                                     "p50_ms": 1e3 * _pct(lat_bg, 0.5) if lat_bg else None,
                                     "p99_ms": 1e3 * _pct(lat_bg, 0.99) if lat_bg else None}}
        if clk is not None:
            out["clocks"] = clk.summary(w0, w1)
        return out, [q for q in reqs if q["tag"] in okt]

    full, served = load(args.rate, args.duration)
    # below saturation: half the rate the one-wave requests were served at
    cap = full["one_wave"]["throughput_per_s"] or full["throughput_per_s"] or args.rate
    sub, _ = load(0.5 * min(cap, args.rate), args.duration)
    # capacity: four times the offered rate for a quarter of the time (the served rate there is
    # what the server sustains when arrivals outrun it)
    sat, _ = load(4.0 * args.rate, 0.25 * args.duration)
    # plain per-request launches (one synchronous call per request, no batching) on a sample of
    # the requests the server evaluated in one wave
    reqs = served[:300]
    for r in reqs:  # plans built outside the timing
        s = sims[r["sim"]]
        if r["kind"] == MARGINAL:
            s.marginal(0, [(r["qubit"], r["outcome"])])
        else:
            s.amplitudes([0], [r["y"]])
    lat = []
    t0 = time.perf_counter()
    for r in reqs:
        t1 = time.perf_counter()
        s = sims[r["sim"]]
        try:
            if r["kind"] == MARGINAL:
                s.marginal(0, [(r["qubit"], r["outcome"])])
            else:
                s.amplitudes([0], [r["y"]])
        except N.PqError:
            continue
        lat.append(time.perf_counter() - t1)
    plain = {"requests": len(reqs), "completed": len(lat), "throughput_per_s": len(lat) / (time.perf_counter() - t0),
             "p50_ms": 1e3 * _pct(lat, 0.5) if lat else None, "p99_ms": 1e3 * _pct(lat, 0.99) if lat else None}
    srv.close()
    return {"value": full["throughput_per_s"], "unit": "requests/s", "at_offered_load": full,
            "sub_saturation": sub, "saturated": sat, "plain_per_request": plain,
            "config": {"workload": "64 resident circuits n~U[16,64], 40n gates, T~U[8,40] (seed 5); Poisson "
                                   "arrivals; amplitude/probability/marginal 1:1:1; marginals on one of the first "
                                   "4 qubits", "max_slots": args.slots, "max_branch_dim": args.max_d,
                       "duration_s": args.duration}}


def run_serve(args):
    leg = leg_serve(args)
    line = {"metric": METRIC, "workload": "serve", "n_gpus": 1, "data": "synthetic", **leg}
    print(json.dumps(line), flush=True)
    return 0


def leg_small(args, clk=None, cpu_runs=200):
    """One amplitude <0|C|0> and its probability: n=20, 200 gates, 16 T (seed 2, the first seed
    whose <0|C|0> is non-zero), per call through the public host-buffer API, beside the CPU
    restatement's median over `cpu_runs` calls."""
    pq, N = _gpu_setup()
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    from polyq_gb300.rng import workload_small
    c = workload_small(2)
    t0 = time.perf_counter()
    sim = pq.Simulator(c)
    build = time.perf_counter() - t0
    for _ in range(20):
        sim.amplitudes([0], [0])
        sim.probability(0, 0)
    lat, plat = [], []
    w0 = time.perf_counter()
    for _ in range(200):
        t1 = time.perf_counter()
        a = sim.amplitudes([0], [0])[0]
        lat.append(time.perf_counter() - t1)
        t1 = time.perf_counter()
        p = sim.probability(0, 0)
        plat.append(time.perf_counter() - t1)
    w1 = time.perf_counter()
    ref = oracle.OracleSim(c)
    # the reference evaluates a subspace of d < 16 on the calling thread (src/engine.rs:688)
    ref.amplitudes([0], [0], nthreads=1)
    cpu = []
    for _ in range(cpu_runs):
        t1 = time.perf_counter()
        want = ref.amplitudes([0], [0], nthreads=1)[0]
        cpu.append(time.perf_counter() - t1)
    dense = oracle.dense_statevector(c, 0)[0]
    # the same calls at the C-ABI level: buffers packed once, one ctypes call each
    import ctypes as ct

    import numpy as np
    L = N.lib()
    xb = np.zeros(1, dtype=np.uint64)
    yb = np.zeros(1, dtype=np.uint64)
    ob = np.zeros(2)
    P = lambda arr, t: arr.ctypes.data_as(ct.POINTER(t))  # noqa: E731
    gcall = lambda: L.pq_amplitudes(sim.handle, 1, P(xb, ct.c_uint64), P(yb, ct.c_uint64), P(ob, ct.c_double),  # noqa: E731
                                    None)
    ccall = lambda: ref.L.pqo_amplitudes(ref.h, 1, P(xb, ct.c_uint64), P(yb, ct.c_uint64), P(ob, ct.c_double), 1)  # noqa: E731
    for f in (gcall, ccall):
        for _ in range(20):
            f()
    glat, clat = [], []
    for _ in range(max(200, cpu_runs)):
        t1 = time.perf_counter()
        gcall()
        glat.append(time.perf_counter() - t1)
        t1 = time.perf_counter()
        ccall()
        clat.append(time.perf_counter() - t1)
    kms = (ct.c_float * 3)()
    N.check(L.pq_sim_kernel_ms(sim.handle, 1, kms))
    # resident mode: the same calls served by a kernel kept on one SM between requests
    gcall()
    a_regular = complex(ob[0], ob[1])
    sim.set_resident(1.0)
    for _ in range(20):
        gcall()
    rlat, rpy = [], []
    for _ in range(max(200, cpu_runs)):
        t1 = time.perf_counter()
        gcall()
        rlat.append(time.perf_counter() - t1)
        t1 = time.perf_counter()
        ar = sim.amplitudes([0], [0])[0]
        rpy.append(time.perf_counter() - t1)
    a_resident = complex(ob[0], ob[1])
    sim.set_resident(0)
    leg_res = {"c_abi_p50_ms": 1e3 * _pct(rlat, 0.5), "c_abi_p99_ms": 1e3 * _pct(rlat, 0.99),
               "python_p50_ms": 1e3 * _pct(rpy, 0.5), "python_p99_ms": 1e3 * _pct(rpy, 0.99),
               "runs": len(rlat), "identical_to_regular": bool(a_resident == a_regular and ar == a),
               "c_abi_p50_over_cpu_p50": _pct(rlat, 0.5) / _pct(clat, 0.5),
               "note": "pq_sim_set_resident(sim, 1.0): one block stays on one SM and serves one-boundary "
                       "pq_amplitudes calls through mapped host memory"}
    leg_cabi = {"gpu_p50_ms": 1e3 * _pct(glat, 0.5), "gpu_p99_ms": 1e3 * _pct(glat, 0.99),
                "device_ms_last_call": kms[0] + kms[1] + kms[2],
                "cpu_p50_ms": 1e3 * _pct(clat, 0.5), "cpu_p99_ms": 1e3 * _pct(clat, 0.99), "runs": len(glat),
                "note": "pq_amplitudes vs the CPU restatement's pqo_amplitudes (one thread), buffers packed once, "
                        "one ctypes call per amplitude"}
    leg = {"value": 1.0 / _pct(lat, 0.5), "unit": "amplitudes/s (serial calls)", "c_abi_level": leg_cabi,
           "resident": leg_res,
           "amplitude": [a.real, a.imag], "probability": p, "p50_ms": 1e3 * _pct(lat, 0.5),
           "p99_ms": 1e3 * _pct(lat, 0.99), "probability_p50_ms": 1e3 * _pct(plat, 0.5),
           "abs_err_vs_fp64_oracle": abs(a - want), "abs_err_vs_dense": abs(a - dense),
           "prob_abs_err_vs_dense": abs(p - abs(dense) ** 2), "build_s": build, "stats": sim.stats_full(),
           "cpu_baseline": {"p50_ms": 1e3 * _pct(cpu, 0.5), "p99_ms": 1e3 * _pct(cpu, 0.99), "runs": cpu_runs,
                            "cores": 1, "kind": "port", "unit": "ms per amplitude call",
                            "sample": "the same amplitude, %d calls, one thread" % cpu_runs},
           "gpu_p50_over_cpu_p50": _pct(lat, 0.5) / _pct(cpu, 0.5),
           "config": {"workload": "n=20, 200 gates, 16 T (seed 2), <0|C|0>, FP64 complex output"}}
    if clk is not None:
        leg["clocks"] = clk.summary(w0, w1)
    return leg


# The reference README's benchmark table (README.md:203-208; harness src/bin/benchmark.rs:10-28):
# whole statevectors of random_layered(n, rounds) circuits from Rng::new(1000 + n), input 0,
# timed from Simulator::with_options to the last amplitude, on an unspecified CPU ("sandbox").
README_ROWS = [  # n, rounds, published dense / cached / auto ms
    (10, 3, {"dense": 0.07, "cached": 62.0, "auto": 18.4}),
    (12, 2, {"dense": 0.27, "cached": 8.6, "auto": 7.5}),
]


def leg_readme(args, clk=None, runs=10):
    """The reference's own published timings, same circuits and the same timed span (simulator
    construction + statevector), on the GPU beside the CPU restatement on all host threads and
    the published numbers; every GPU statevector checked against the dense oracle (the harness
    asserts max |diff| < 1e-7)."""
    pq, N = _gpu_setup()
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import numpy as np

    import oracle
    from polyq_gb300.rng import Rng, random_layered
    rows = []
    w0 = time.perf_counter()
    for n, rounds, pub in README_ROWS:
        c = random_layered(n, rounds, Rng(1000 + n))
        t1 = time.perf_counter()
        dense = oracle.dense_statevector(c, 0)
        dense_ms = 1e3 * (time.perf_counter() - t1)
        row = {"n": n, "rounds": rounds, "t_count": c.t_count(), "published_ms": pub, "dense_port_ms": dense_ms}
        for strat in ("cached", "auto"):
            wall, built, sv_only, err = [], [], [], 0.0
            sim = None
            for r in range(runs):
                t1 = time.perf_counter()
                sim = pq.Simulator(c, strat)
                t2 = time.perf_counter()
                sv = sim.statevector(0)
                wall.append(time.perf_counter() - t1)
                built.append(t2 - t1)
                err = max(err, float(np.max(np.abs(sv - dense))))
            for r in range(runs):
                t1 = time.perf_counter()
                sim.statevector(0)
                sv_only.append(time.perf_counter() - t1)
            cpu = []
            for r in range(3):
                t1 = time.perf_counter()
                ref = oracle.OracleSim(c, strat)
                ref.amplitudes([0] * (1 << n), list(range(1 << n)))
                cpu.append(time.perf_counter() - t1)
            st = sim.stats_full()
            row[strat] = {"gpu_first_ms": 1e3 * wall[0], "gpu_ms": 1e3 * statistics.median(wall),
                          "construction_ms": 1e3 * statistics.median(built),
                          "gpu_statevector_only_ms": 1e3 * statistics.median(sv_only),
                          "cpu_port_ms": 1e3 * statistics.median(cpu), "cpu_threads": os.cpu_count(),
                          "published_over_gpu": pub[strat] / (1e3 * statistics.median(wall)),
                          "max_abs_err_vs_dense": err, "branch_dim": st["branch_dim"], "pairs": st["pairs"]}
        rows.append(row)
    w1 = time.perf_counter()
    leg = {"rows": rows, "runs": runs,
           "note": "gpu_ms: median over fresh simulators of construction + statevector (the harness's span); "
                   "published_ms: the reference on an unspecified CPU; cpu_port_ms: the CPU restatement here"}
    if clk is not None:
        leg["clocks"] = clk.summary(w0, w1)
    return leg


def run_small(args):
    leg = leg_small(args)
    line = {"metric": METRIC, "workload": "small", "n_gpus": 1, "data": "synthetic", **leg}
    print(json.dumps(line), flush=True)
    return 0


def run_sample(args):
    """Simulator::sample_many on the small circuit (n=20, 200 gates, 16 T, seed 2): shots/s on the
    device (all shots advance together, one launch per qubit) beside the CPU restatement on a
    bounded number of shots; the two give identical samples for the same seed."""
    pq, N = _gpu_setup()
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    from polyq_gb300.rng import workload_small
    c = workload_small(2)
    sim = pq.Simulator(c)
    shots = 4096
    sim.sample_many(0, shots, 1)  # prefix engines built and plans captured outside the timing
    times = []
    for k in range(max(1, args.steps)):
        t0 = time.perf_counter()
        got = sim.sample_many(0, shots, 100 + k)
        times.append(time.perf_counter() - t0)
    gpu_rate = shots / (sum(times) / len(times))
    cpu_shots = 512
    osim = oracle.OracleSim(c)
    osim.sample_many(0, 2, 1)
    t0 = time.perf_counter()
    want = osim.sample_many(0, cpu_shots, 100)
    cpu_s = time.perf_counter() - t0
    line = {"metric": METRIC, "workload": "sample", "value": gpu_rate, "unit": "shots/s", "n_gpus": 1,
            "higher_is_better": True, "data": "synthetic", "shots_per_step": shots,
            "ms_per_step": 1e3 * sum(times) / len(times),
            "same_samples_as_cpu_restatement": sim.sample_many(0, cpu_shots, 100) == want,
            "cpu_baseline": {"value": cpu_shots / cpu_s, "unit": "shots/s", "cores": cpu_threads(), "kind": "port",
                             "sample": "%d shots; prefix engines built per call, shots in parallel" % cpu_shots},
            "config": {"workload": "sample_many: n=20, 200 gates, 16 T (seed 2), x=0, %d shots" % shots}}
    print(json.dumps(line), flush=True)
    return 0


def run_estimate(args):
    """Simulator::amplitude_estimate on the rotation workload as written (n=40, 1500 gates, 24 rz,
    4 layers of 8 CCZ; one cached engine of d = 239, beyond exact enumeration): sampled points
    per second on the device beside the CPU restatement, same seeds, same draws."""
    pq, N = _gpu_setup()
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    from polyq_gb300.rng import workload_rotations
    c = workload_rotations(n=40, ngates=1500, n_rz=24, ccz_layers=4, ccz_per_layer=8, seed=4)
    sim = pq.Simulator(c, "cached")
    samples = 1 << 22
    sim.amplitude_estimate(0, 12345, 1 << 12, 1)
    times, est = [], None
    for k in range(max(1, min(args.steps, 10))):
        t0 = time.perf_counter()
        est = sim.amplitude_estimate(0, 12345, samples, 100 + k)
        times.append(time.perf_counter() - t0)
    ref = oracle.OracleSim(c, "cached")
    cpu_samples = 1 << 15
    t0 = time.perf_counter()
    want = ref.amplitude_estimate(0, 12345, cpu_samples, 100)
    cpu_s = time.perf_counter() - t0
    got = sim.amplitude_estimate(0, 12345, cpu_samples, 100)
    line = {"metric": METRIC, "workload": "estimate", "value": samples / (sum(times) / len(times)),
            "unit": "samples/s", "n_gpus": 1, "higher_is_better": True, "data": "synthetic",
            "ms_per_step": 1e3 * sum(times) / len(times), "samples_per_step": samples,
            "estimate": {"re": est[0], "im": est[1], "stderr": est[2]},
            "same_draws_as_cpu_restatement_rel_diff": abs(complex(got[0], got[1]) - complex(want[0], want[1])) /
            max(abs(complex(want[0], want[1])), want[2], 1e-300),
            "branch_dim": sim.stats_full()["branch_dim"],
            "cpu_baseline": {"value": cpu_samples / cpu_s, "unit": "samples/s", "cores": 1, "kind": "port",
                             "sample": "%d samples, one thread (the restatement's sampler is sequential)" % cpu_samples},
            "config": {"workload": "amplitude_estimate, rotations as written: n=40, 1500 gates, 24 rz, 4x8 CCZ "
                                   "(seed 4), strategy cached, <12345|C|0>"}}
    print(json.dumps(line), flush=True)
    return 0


def run_rotations(args):
    """Arbitrary angles: rz(theta) slots plus CCZ layers, the FP32 path vs device FP64 per
    amplitude; a 20-qubit variant also against the dense statevector."""
    import numpy as np

    pq, N = _gpu_setup()
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    from polyq_gb300.rng import random_outputs, workload_rotations
    res = {}
    # scaled variant: n=40, 1500 gates, 24 rz; CCZ per layer reduced until the branch sum fits 2^30
    chosen = None
    for per_layer in (8, 4, 3, 2, 1):
        c = workload_rotations(n=40, ngates=1500, n_rz=24, ccz_layers=4, ccz_per_layer=per_layer, seed=4)
        st = pq.Simulator(c, host_only=True).stats_full()
        res["n40_ccz_per_layer_%d_branches_per_amp" % per_layer] = st["branches_per_amplitude"]
        if st["branches_per_amplitude"] <= (1 << 36) and chosen is None:
            chosen = (per_layer, c)
    per_layer, c = chosen
    sim = pq.Simulator(c)
    nb = args.boundaries if args.boundaries != 4096 else 64  # about 4e10 branches per amplitude at this size
    ys = random_outputs(40, nb, 4)
    sim.amplitudes([0] * 2, ys[:2])
    t0 = time.perf_counter()
    got, err = sim.amplitudes([0] * nb, ys, with_error=True)
    t32 = time.perf_counter() - t0
    ref = sim.amplitudes_fp64([0] * nb, ys)
    rel = np.abs(got - ref) / np.abs(ref)
    res["n40"] = {"ccz_per_layer": per_layer, "stats": sim.stats_full(), "seconds_fp32_path": t32,
                  "max_rel_err_vs_fp64": float(np.max(rel)), "median_rel_err": float(np.median(rel)),
                  "within_1e-6": float(np.mean(rel <= 1e-6)), "max_bound_over_abs": float(np.max(err / np.abs(ref)))}
    # dense-checkable variant
    c20 = workload_rotations(n=20, ngates=600, n_rz=12, ccz_layers=2, ccz_per_layer=2, seed=4)
    s20 = pq.Simulator(c20)
    sv = oracle.dense_statevector(c20, 0)
    idx = [int(i) for i in np.argsort(-np.abs(sv))[:1024]]
    g20 = s20.amplitudes([0] * len(idx), idx)
    rel20 = np.abs(g20 - sv[idx]) / np.abs(sv[idx])
    res["n20_dense"] = {"stats": s20.stats_full(), "max_rel_err_vs_dense": float(np.max(rel20)),
                        "median_rel_err_vs_dense": float(np.median(rel20)),
                        "prob_max_abs_err": float(np.max(np.abs(s20.probabilities([0] * len(idx), idx) -
                                                                np.abs(sv[idx]) ** 2)))}
    line = {"metric": METRIC, "workload": "rotations", "value": nb / t32, "unit": "amplitudes/s", "data": "synthetic",
            "branches_per_s": enumerated(N.lib(), N, sim, nb)[0] / t32,
            "results": res, "config": {"workload": "n=40, 1500 gates, 24 rz(theta) theta~U[0,2pi) + 4 CCZ layers "
                                                   "(per-layer count reduced until <= 2^36 branches per amplitude); "
                                                   "%d uniform y; n=20 variant vs dense" % nb}}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-sample", type=int, default=320)
    ap.add_argument("--ref-sample", type=int, default=24)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="keep the library's default launch shape")
    ap.add_argument("--chunk-tables", action="store_true",
                    help="sum each chunk from its engine's chunk-sum table (no per-branch enumeration)")
    ap.add_argument("--tuning", default="", help="fixed launch shape inner_dims,chunks_per_lane,block_warps,"
                    "blocks_per_sm[,unit_chunks] (implies --no-autotune)")
    ap.add_argument("--boundaries", type=int, default=4096, help="boundary count (profiling of smaller cases)")
    ap.add_argument("--workload", default="many_boundaries",
                    choices=["many_boundaries", "batched", "serve", "small", "rotations", "sample", "estimate",
                             "readme"])
    ap.add_argument("--rate", type=float, default=5000.0, help="serve: offered requests/s")
    ap.add_argument("--duration", type=float, default=2.0, help="serve: seconds of arrivals")
    ap.add_argument("--slots", type=int, default=256, help="serve: requests per wave")
    ap.add_argument("--max-d", type=int, default=36, help="serve: log2 cap on a request's branches (refused above)")
    ap.add_argument("--batch-steps", type=int, default=20, help="batched: timed launches")
    ap.add_argument("--batch-only", action="store_true", help="batched: the batched launch alone (profiling)")
    ap.add_argument("--headline-only", action="store_true",
                    help="default workload only (no small / batched / serving legs)")
    args = ap.parse_args()
    WORKLOAD["boundaries"] = args.boundaries
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "batched":
        return run_batched(args)
    if args.workload == "serve":
        return run_serve(args)
    if args.workload == "small":
        return run_small(args)
    if args.workload == "readme":
        print(json.dumps({"metric": METRIC, "workload": "readme", "n_gpus": 1, "data": "synthetic",
                          **leg_readme(args)}), flush=True)
        return 0
    if args.workload == "sample":
        return run_sample(args)
    if args.workload == "estimate":
        return run_estimate(args)
    if args.workload == "rotations":
        return run_rotations(args)
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
