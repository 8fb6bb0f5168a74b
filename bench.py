#!/usr/bin/env python
"""Throughput of the TT-rounding hot path on GB300.

Default workload (the headline): batched uneven rounding -- 4096 independent
TTs, TT i seeded with mt19937_64(1000 + i): d ~ U[8,32], n_k ~ {2,4,8}, bond
ranks ~ U[4,96] (feasibility-clipped), entries N(0,1)/sqrt(r_k n_k),
eps = 1e-8, plain FP64, one persistent launch per step.  A step is one
round(const tt&) of every TT: the deep copy of the inputs into the work
arena (round/tt_round.hpp:129-134) plus the sweep kernel.

Prints one JSON line (rank 0).  `--impl reference` times the reference's CPU
algorithm (the oracle port: the reference itself needs Eigen, which is absent)
on the host cores instead.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from concurrent.futures import ThreadPoolExecutor

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = ("TT roundings/sec and matvec_round/sec at rel. err<=1e-8: mixed/learned vs plain "
          "FP64, 1 GB300")
EPS = 1e-8
SEED0 = 1000
# DRAM bytes (read + write) of one mixed round_kernel launch on TTs 1000..1607
# of the batch at the mixed default of 3 CTAs per SM (ncu,
# profiles/round_kernel_batch608_ncu.md).
TRAFFIC_608 = 6.161341952e9 + 9.316889088e9


def measured_peaks(path=None):
    """HBM GB/s and dense BF16 TFLOP/s measured on the GB300s
    (MEASURED_PEAKS.json beside this file), else the published fallback."""
    if path is None:
        path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), float(d["bf16_tflops"]), "measured (MEASURED_PEAKS.json)"
    except (OSError, KeyError, ValueError):
        return 6800.0, 1900.0, "fallback (no measured peaks file)"


def roofline_tensor(flops, kernel_ms, fp64_peak, traffic=None, **extra):
    """Roofline object of a rounding kernel against the dense BF16 tensor
    peak (the configured bound of the mixed path), with the FP64-pipe
    fraction beside it: the sweeps run no tensor-core work, so the tensor
    fraction is small and the FP64 fraction is the informative one for the
    plain FP64 kernel.  The mixed kernel does its arithmetic in df64 on the
    FP32 pipes, so its algorithmic rate can exceed the FP64 peak."""
    _, bf16, src = measured_peaks()
    ach = flops / (kernel_ms / 1e3) / 1e12
    out = {"bound": "tensor", "achieved": ach, "peak": bf16, "unit": "TFLOP/s",
           "frac": ach / bf16, "traffic": traffic, "peak_source": src + ", dense BF16 burst",
           "fp64_pipe": {"achieved": ach, "peak": fp64_peak, "unit": "TFLOP/s",
                         "frac": ach / fp64_peak,
                         "peak_source": "measured FP64 FMA loop on this GPU",
                         "note": "algorithmic FP64 flops over the FP64 FMA peak; a mixed-precision "
                                 "kernel runs them as df64 on the FP32 pipes, so frac > 1 is "
                                 "possible there"},
           "kernel_ms": kernel_ms, "flops_per_launch": flops}
    out.update(extra)
    return out


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--count", type=int, default=4096)
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--cpu-sample", type=int, default=256)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--only", choices=["both", "mixed", "fp64"], default="both",
                    help="batch workload: time one precision only (profiling cases)")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the plan's default launch configuration (profiling cases)")
    ap.add_argument("--gauge", choices=["none", "right_canonical"], default="none",
                    help="round workloads: detail::round (none) or round_right_canonical")
    ap.add_argument("--workload", default="batch",
                    choices=["batch", "round_d10", "matvec_d20", "round_d40", "eval_d32",
                             "sketch_d64"],
                    help="batch = the headline (4096 uneven TTs); the others are the single-"
                         "tensor configurations, measured one JSON line each")
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="mixed")
    ap.add_argument("--method", choices=["svd", "svd_streaming"], default="svd")
    ap.add_argument("--schedule", choices=["auto", "per_tt", "whole_gpu"], default="auto")
    ap.add_argument("--d", type=int, default=0,
                    help="number of cores of round_d40 / matvec_d20 (0 = the configuration's; "
                         "smaller values make short cases for profiling)")
    ap.add_argument("--samples", type=int, default=1 << 20, help="eval_d32 multi-indices")
    return ap.parse_args()


def workload_config(count):
    return {
        "workload": (f"batched uneven rounding: {count} TTs, d~U[8,32], n_k~{{2,4,8}}, "
                     "bond ranks~U[4,96] clipped, N(0,1)/sqrt(r n) cores, eps=1e-8, "
                     "round(const tt&) per TT"),
        "count": count, "eps": EPS, "seeds": f"{SEED0}+i",
        "l2": "inputs (~4.5 GB FP64) exceed L2 (129 MB); no flush needed",
    }


def make_batch(T, count, base):
    with ThreadPoolExecutor(max_workers=min(32, os.cpu_count() or 4)) as ex:
        return list(ex.map(lambda i: T.random_uneven(base + i), range(count)))


class Clocks:
    """nvidia-smi samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                out = ""
            self.lines = [ln for ln in out.splitlines() if ln.strip()]

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in getattr(self, "lines", []):
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


THROTTLE_REASONS = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown")


def clocks_ok(summary, floor=0.85):
    """A timed region counts when no thermal or hardware slowdown was active
    and the median SM clock under load is not stuck well below its maximum
    without a reason (a leftover clock lock).  sw_power_cap is allowed."""
    reasons = set(summary.get("reasons") or [])
    if reasons & set(THROTTLE_REASONS):
        return False
    sm, smax = summary.get("sm_mhz"), summary.get("sm_max_mhz")
    if sm and smax and sm < floor * smax and "sw_power_cap" not in reasons:
        return False
    return True


def any_rank(flag, world, device="cuda"):
    """True on every rank when `flag` is true on any rank (so that all ranks
    take the same branch before the next collective)."""
    if world <= 1:
        return bool(flag)
    import torch
    t = torch.tensor([1.0 if flag else 0.0], device=device, dtype=torch.float64)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return bool(t.item() > 0.0)


def dist_setup(gpus):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def shard_base(rank, count):
    """First seed of a rank's batch: each rank owns `count` distinct TTs
    (weak scaling, no data-path collective)."""
    return SEED0 + rank * count


def max_over_ranks(x, world, device="cuda"):
    """Slowest rank's time (the job's time) when world > 1."""
    if world <= 1:
        return float(x)
    import torch
    t = torch.tensor([float(x)], device=device, dtype=torch.float64)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def run_ours(args):
    import numpy as np
    import torch

    import tensor_train_gb300 as T
    from tensor_train_gb300.flops import round_flops

    rank, world, local = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream

    count = args.count
    base = shard_base(rank, count)  # weak scaling: each rank owns its own batch
    tts = make_batch(T, count, base)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    def measure(precision):
        """Warm-up, then exactly K timed steps of one plan; returns a dict."""
        opts = T.RoundOptions(eps=EPS, precision=precision)
        plan = T.Plan("round", tts, opts=opts)
        plan.upload(sptr)
        torch.cuda.synchronize()
        # Launch configuration by the plan's autotuner, then one CUDA graph
        # per step (deep copy from the pristine inputs + the sweep launch).
        tuned = "default" if args.no_autotune else plan.autotune(sptr)
        plan.graph(True)
        for _ in range(args.warmup):
            plan.run(sptr)
        torch.cuda.synchronize()
        outs = plan.download(sptr)
        bad = [r.status for r in plan.results if r.status != 0]

        def timed_region():
            launches0 = T.kernel_launches()
            ev0 = torch.cuda.Event(enable_timing=True)
            ev1 = torch.cuda.Event(enable_timing=True)
            barrier()
            torch.cuda.synchronize()
            with Clocks(local) as clk:
                ev0.record(stream)
                for _ in range(args.steps):
                    plan.run(sptr)
                ev1.record(stream)
                torch.cuda.synchronize()
            barrier()
            return (T.kernel_launches() - launches0,
                    max_over_ranks(ev0.elapsed_time(ev1), world), clk.summary())

        launches, ms_total, clocks = timed_region()
        # A region that ran throttled or under a clock lock is measured once more.
        remeasured = any_rank(not clocks_ok(clocks), world)
        if remeasured:
            launches, ms_total, clocks = timed_region()
        clocks["remeasured"] = remeasured
        kms = []
        for _ in range(3):
            plan.run(sptr)
            kms.append(plan.kernel_ms())
        io = plan.io_bytes()
        plan.close()
        ms_step = ms_total / args.steps
        return {"opts": opts, "outs": outs, "bad": len(bad), "launches": launches, "tuned": tuned,
                "ms_step": ms_step, "value": count * world / (ms_step / 1e3),
                "kernel_ms": statistics.mean(kms), "clocks": clocks, "io": io}

    if args.only != "both":
        # One precision, no CPU legs: a short case for profilers.
        r = measure(T.precision[args.only])
        print(json.dumps({"workload": f"batch of {count}", "precision": args.only,
                          "ms_per_step": r["ms_step"], "kernel_ms": r["kernel_ms"],
                          "value": r["value"], "autotune": r["tuned"],
                          "device_status_errors": r["bad"]}), flush=True)
        if world > 1:
            torch.distributed.destroy_process_group()
        return
    plain = measure(T.precision.fp64)
    mixed = measure(T.precision.mixed)
    opts = mixed["opts"]
    outs = mixed["outs"]
    value, ms_step, launches = mixed["value"], mixed["ms_step"], mixed["launches"]

    flops = 0.0
    for t_in, t_out in zip(tts, plain["outs"]):
        modes = [c.shape[1] for c in t_in]
        rin = [t_in[0].shape[0]] + [c.shape[-1] for c in t_in]
        rout = [t_out[0].shape[0]] + [c.shape[-1] for c in t_out]
        flops += round_flops(modes, rin, rout)
    peak = max(T.device_fp64_peak() for _ in range(3))
    kernel_ms = mixed["kernel_ms"]
    achieved = flops / (kernel_ms / 1e3) / 1e12
    plain_achieved = flops / (plain["kernel_ms"] / 1e3) / 1e12

    # End to end through the C-ABI with host buffers: pack + H2D + sweep +
    # D2H + unpack inside ttg_round_batch.  Inputs marshalled beforehand.
    import ctypes as C
    srcs = [T._In(t) for t in tts]
    ins = (T._Tensor * count)(*[s.t for s in srcs])
    copts = T._opts(opts)
    h2d, d2h = mixed["io"]
    e2e_ms = []
    for i in range(0 if args.no_e2e else args.e2e_steps + 1):
        outs_c = (T._Tensor * count)()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        st = T.lib().ttg_round_batch(count, ins, C.byref(copts), outs_c, None)
        t1 = time.perf_counter()
        for j in range(count):
            T.lib().ttg_free(C.byref(outs_c[j]))
        assert st == 0, T.lib().ttg_last_error()
        if i > 0:  # first call is the warm-up (pool growth)
            e2e_ms.append((t1 - t0) * 1e3)
    e2e_step = statistics.mean(e2e_ms) if e2e_ms else float("nan")
    e2e_value = count * world / (max_over_ranks(e2e_step, world) / 1e3)

    line = {
        "metric": METRIC, "value": value, "unit": "roundings/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64 in/out; df64 QR, contractions and polish sweeps + f32 Jacobi sweeps",
        "data": "synthetic: seeded uneven random TTs (mt19937_64 + normal_distribution)",
        "config": workload_config(count),
        "precision": "mixed", "parallelism": f"{world} independent shard(s), one GPU each",
        # traffic: DRAM read + write bytes of one mixed round_kernel launch at
        # the mixed default of 3 CTAs per SM, from the ncu capture of a 608-TT slice of
        # this batch (6.161 GB read + 9.317 GB written), scaled to `count`
        # TTs by the TT count; it is per-CTA scratch of the work matrices
        # evicted from L2, set against the algorithmic bytes (input cores read,
        # output cores written).
        "roofline": roofline_tensor(flops, kernel_ms, peak, traffic=TRAFFIC_608 * count / 608,
                                    kernel="round_kernel (precision=mixed)",
                                    flop_model="algorithmic F_round (tensor_train_gb300/flops.py)",
                                    algorithmic_bytes=sum(mixed["io"]),
                                    traffic_over_algorithmic=TRAFFIC_608 * count / 608 /
                                    max(sum(mixed["io"]), 1)),
        "plain_fp64": {"value": plain["value"], "ms_per_step": plain["ms_step"],
                       "kernel_ms": plain["kernel_ms"], "achieved_tflops": plain_achieved,
                       "frac": plain_achieved / peak, "clocks": plain["clocks"],
                       "device_status_errors": plain["bad"]},
        "speedup_mixed_vs_plain_fp64": plain["ms_step"] / ms_step,
        "e2e": {"value": e2e_value, "unit": "roundings/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": e2e_step},
        "gpu_launches": launches,
        "autotune": {"fp64": plain["tuned"], "mixed": mixed["tuned"]},
        "cuda_graph": True,
        "clocks": mixed["clocks"],
        "device_status_errors": mixed["bad"],
    }

    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(tts, outs, args.cpu_sample, plain["outs"])
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def cpu_baseline(tts, gpu_outs, sample, plain_outs=None):
    """The oracle (FP64 port of the reference's round) on the host cores, on
    a strided sample of the same batch; also checks the GPU outputs of the
    sampled TTs against it (ranks and relative Frobenius error)."""
    from oracle import pyoracle as O
    stride = max(1, len(tts) // sample)
    idx = list(range(0, len(tts), stride))[:sample]
    threads = os.cpu_count() or 1
    sec, ref = O.round_many_timed([tts[i] for i in idx], EPS, 0, threads)
    # Parity of every sampled TT (outside the timed region; the oracle's
    # calls release the GIL, so the checks run on all host threads).
    refs = [r.cores() for r in ref]

    def check(j):
        i, yr = idx[j], refs[j]
        ok = O.ranks(gpu_outs[i]) == O.ranks(yr)
        e = O.rel_err(gpu_outs[i], yr)
        pe = None
        if plain_outs is not None:
            ok &= O.ranks(plain_outs[i]) == O.ranks(yr)
            pe = O.rel_err(plain_outs[i], yr)
        return ok, e, pe

    with ThreadPoolExecutor(max_workers=threads) as ex:
        checks = list(ex.map(check, range(len(idx))))
    ranks_ok = all(c[0] for c in checks)
    errs = [c[1] for c in checks]
    perrs = [c[2] for c in checks if c[2] is not None]
    # Extra line: the same rounding through numpy/LAPACK (one process; the
    # BLAS/LAPACK library threads as it likes) on the first 32 sampled TTs.
    from oracle import numpy_round as NR
    few = [tts[i] for i in idx[:32]]
    t0 = time.perf_counter()
    for t in few:
        NR.round_tt(t, EPS)
    np_sec = time.perf_counter() - t0
    return {"value": len(idx) / sec, "unit": "roundings/s", "cores": threads, "kind": "port",
            "sample": f"{len(idx)} of the {len(tts)} TTs (every {stride}th), oracle FP64 "
                      f"round on {threads} host threads, {sec:.2f} s",
            "parity_checked": len(errs), "max_rel_err_vs_oracle": max(errs),
            "max_rel_err_plain_fp64_vs_oracle": max(perrs) if perrs else None,
            "ranks_equal": bool(ranks_ok),
            "numpy_lapack": {"value": len(few) / np_sec, "unit": "roundings/s",
                             "sample": f"{len(few)} of the sampled TTs, numpy.linalg QR/SVD, "
                                       "one process"}}


def run_reference(args):
    """CPU implementation of the path (oracle port: the reference needs
    Eigen, which is absent) on all host threads, same workload."""
    rank, world, _ = dist_setup(args.gpus)
    if rank != 0:
        return
    # The oracle alone: its own generator (bit-identical to the library's
    # ttg_host_random_uneven) builds the inputs, so this arm loads no code of
    # the product library.
    from oracle import pyoracle as O
    threads = os.cpu_count() or 1
    per_step = max(threads * 4, 64)
    need = per_step * (args.steps + args.warmup)
    stride = max(1, args.count // need)
    with ThreadPoolExecutor(max_workers=min(32, threads)) as ex:
        tts = list(ex.map(lambda i: O.random_uneven(SEED0 + i * stride), range(need)))
    times = []
    for s in range(args.warmup + args.steps):
        chunk = tts[s * per_step:(s + 1) * per_step]
        sec, _ = O.round_many_timed(chunk, EPS, 0, threads)
        if s >= args.warmup:
            times.append(sec)
    step = statistics.mean(times)
    value = per_step / step
    line = {
        "metric": METRIC, "value": value, "unit": "roundings/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: seeded uneven random TTs (mt19937_64 + normal_distribution)",
        "config": workload_config(args.count), "impl": "reference",
        "precision": "fp64", "parallelism": f"CPU: {threads} host threads over independent TTs",
        "cpu_baseline": {"value": value, "unit": "roundings/s", "cores": threads, "kind": "port",
                         "sample": f"{per_step} TTs of the batch per step on {threads} threads"},
        "e2e": {"value": value, "unit": "roundings/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def single_inputs(T, workload, d=0, samples=1 << 20):
    """Seeded inputs of the single-tensor configurations (cores scaled by
    1/sqrt(r_k n_k), or 1/sqrt(r m n) for MPO cores).  d > 0 shortens the
    train of round_d40 / matvec_d20 (profiling cases)."""
    if workload == "round_d10":
        a = T.random([4] * 10, 8, 42, fan_in_scale=True)
        b = T.random([4] * 10, 8, 43, fan_in_scale=True)
        return {"tt": T.add(a, b), "eps": 1e-8,
                "desc": "round(add(a,b)): d=10, n=4, a,b random rank 8 (seeds 42/43), eps=1e-8"}
    if workload == "round_d40":
        d = d or 40
        a = T.random([8] * d, 128, 46, fan_in_scale=True)
        b = T.random([8] * d, 128, 47, fan_in_scale=True)
        # ones() gets the same 1/sqrt(r n) core scaling as the random terms;
        # unscaled, its norm 8^20 would swamp a + b and the sum rounds to rank 1.
        ones = [c / (8.0 ** 0.5) for c in T.ones([8] * d)]
        return {"tt": T.add(T.add(a, b), ones), "eps": 1e-8,
                "desc": f"round(a+b+ones): d={d}, n=8, a,b random rank 128 (seeds 46/47), "
                        "ones scaled 1/sqrt(8) per core, interior rank 257, eps=1e-8"}
    if workload == "matvec_d20":
        d = d or 20
        A = T.random_matrix([4] * d, [4] * d, 8, 44, fan_in_scale=True)
        x = T.random([4] * d, 32, 45, fan_in_scale=True)
        return {"A": A, "x": x, "eps": 1e-10,
                "desc": f"matvec_round(A, x): d={d}, m=n=4, MPO rank 8 (seed 44), TT rank 32 "
                        "(seed 45), eps=1e-10"}
    if workload == "eval_d32":
        import numpy as np
        t = T.random([4] * 32, 64, 48, fan_in_scale=True)
        idx = np.random.default_rng(49).integers(0, 4, size=(samples, 32)).astype(np.int32)
        return {"tt": t, "idx": idx,
                "desc": f"eval_batch: d=32, n=4, rank 64 (seed 48), M={samples} uniform indices "
                        "(numpy seed 49)"}
    raise ValueError(workload)


def run_single(args):
    """One JSON line for a single-tensor configuration (not the headline):
    the requested precision is the line's value; round / matvec_round lines
    also time the other precision (mixed vs plain FP64) on the same input."""
    import numpy as np
    import torch

    import tensor_train_gb300 as T
    from tensor_train_gb300.flops import eval_flops, matvec_flops, round_flops

    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream
    inp = single_inputs(T, args.workload, args.d, args.samples)
    desc = inp["desc"] + (", gauge right_canonical" if args.gauge != "none" else "")
    line = {"workload": args.workload, "metric": METRIC, "config": {"workload": desc},
            "steps": args.steps, "warmup": args.warmup, "precision": args.precision,
            "gauge": args.gauge}

    def timed(plan, tune=False):
        plan.upload(sptr)
        if tune:  # launch configuration by the autotuner, then CUDA-graph replays
            plan.tuned = "default" if args.no_autotune else plan.autotune(sptr)
            plan.graph(True)
        for _ in range(args.warmup):
            plan.run(sptr)
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        for attempt in range(2):
            launches0 = T.kernel_launches()
            with Clocks(0) as clk:
                ev0.record(stream)
                for _ in range(args.steps):
                    plan.run(sptr)
                ev1.record(stream)
                torch.cuda.synchronize()
            plan.launches = T.kernel_launches() - launches0
            clocks = clk.summary()
            clocks["remeasured"] = attempt > 0
            if clocks_ok(clocks):
                break
        return ev0.elapsed_time(ev1) / args.steps, clocks

    def e2e(call, nbytes_in, out_bytes):
        """The public host-buffer call (numpy in, numpy out: pack, H2D,
        kernels, D2H, unpack inside the timed region), wall clock."""
        for _ in range(min(args.warmup, 2)):
            out = call()
        steps = max(1, min(args.steps, 5))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(steps):
            out = call()
        sec = (time.perf_counter() - t0) / steps
        return {"value": 1.0 / sec, "ms_per_step": sec * 1e3, "h2d_bytes_per_step": nbytes_in,
                "d2h_bytes_per_step": out_bytes(out)}

    if args.workload == "eval_d32":
        idx_pinned = torch.from_numpy(inp["idx"]).pin_memory()
        plan = T.Plan("eval", inp["tt"], idx_pinned)
        ms, clocks = timed(plan)
        M = inp["idx"].shape[0]
        out = plan.download(sptr)
        ranks = [inp["tt"][0].shape[0]] + [c.shape[-1] for c in inp["tt"]]
        F = eval_flops(ranks, M)
        nbytes = 4 * inp["idx"].size + 8 * M + 8 * sum(c.size for c in inp["tt"])
        peak = max(T.device_fp64_peak() for _ in range(3))
        ee = e2e(lambda: T.eval_batch(inp["tt"], inp["idx"]),
                 4 * inp["idx"].size + 8 * sum(c.size for c in inp["tt"]), lambda o: o.nbytes)
        ee["value"] *= M
        line.update({"value": M / (ms / 1e3), "unit": "evaluations/s", "ms_per_step": ms,
                     "n_gpus": 1, "higher_is_better": True, "dtype": "f64", "clocks": clocks,
                     "e2e": dict(ee, unit="evaluations/s"), "gpu_launches": plan.launches,
                     "roofline": {"bound": "hbm", "achieved": nbytes / (ms / 1e3) / 1e9,
                                  "peak": measured_peaks()[0], "unit": "GB/s",
                                  "frac": nbytes / (ms / 1e3) / 1e9 / measured_peaks()[0],
                                  "traffic": None, "peak_source": measured_peaks()[2],
                                  "bytes_per_launch": nbytes, "flops_per_launch": F,
                                  # the chain of FP64 products, not HBM, bounds this kernel
                                  "fp64_pipe": {"achieved": F / (ms / 1e3) / 1e12, "peak": peak,
                                                "unit": "TFLOP/s",
                                                "frac": F / (ms / 1e3) / 1e12 / peak}}})
        if not args.no_cpu_baseline:
            from oracle import pyoracle as O
            sel = np.arange(0, M, max(1, M // 4096))
            t0 = time.perf_counter()
            ref = O.eval_batch(inp["tt"], inp["idx"][sel])
            sec = time.perf_counter() - t0
            line["cpu_baseline"] = {"value": len(sel) / sec, "unit": "evaluations/s", "cores": 1,
                                    "kind": "port", "sample": f"{len(sel)} of the {M} indices"}
            line["parity_max_abs_err"] = float(np.max(np.abs(out[sel] - ref)))
        print(json.dumps(line), flush=True)
        return

    matvec = args.workload == "matvec_d20"
    unit = "matvec_rounds/s" if matvec else "roundings/s"
    if matvec:
        A, x = inp["A"], inp["x"]
        ra = [A[0].shape[0]] + [c.shape[-1] for c in A]
        rx = [x[0].shape[0]] + [c.shape[-1] for c in x]
        rin = [a * b for a, b in zip(ra, rx)]
        modes = [c.shape[1] for c in A]
        line["method"] = args.method
    else:
        t = inp["tt"]
        modes = [c.shape[1] for c in t]
        rin = [t[0].shape[0]] + [c.shape[-1] for c in t]
    peak = max(T.device_fp64_peak() for _ in range(3))

    def measure(prec):
        opts = T.RoundOptions(eps=inp["eps"], precision=T.precision[prec],
                              schedule=T.schedule[args.schedule],
                              method=T.round_method[args.method] if matvec else T.round_method.svd,
                              gauge=T.round_gauge.none if matvec else T.round_gauge[args.gauge])
        plan = (T.Plan("matvec_round", inp["A"], inp["x"], opts=opts) if matvec
                else T.Plan("round", [inp["tt"]], opts=opts))
        ms, clocks = timed(plan, tune=True)
        kms = []
        for _ in range(3):
            plan.run(sptr)
            kms.append(plan.kernel_ms())
        y = plan.download(sptr)[0]
        sched = plan.schedule()
        tuned = plan.tuned
        plan.close()
        rout = [y[0].shape[0]] + [c.shape[-1] for c in y]
        F = round_flops(modes, rin, rout)
        if matvec:
            F += matvec_flops(ra, rx, modes, [c.shape[2] for c in A])
        kernel_ms = statistics.mean(kms)
        if matvec:
            call = (lambda: T.matvec_round(inp["A"], inp["x"], opts))
            nin = 8 * sum(c.size for c in inp["A"] + inp["x"])
        else:
            call = (lambda: T.round(inp["tt"], opts))
            nin = 8 * sum(c.size for c in inp["tt"])
        ee = e2e(call, nin, lambda o: 8 * sum(c.size for c in o))
        return {"y": y, "ranks_out": rout, "ms": ms, "kernel_ms": kernel_ms, "clocks": clocks,
                "schedule": sched, "flops": F, "tuned": tuned, "launches": plan.launches,
                "achieved": F / (kernel_ms / 1e3) / 1e12, "e2e": ee}

    main = measure(args.precision)
    other_prec = "fp64" if args.precision == "mixed" else "mixed"
    other = measure(other_prec)
    mixed, plain = (main, other) if args.precision == "mixed" else (other, main)
    line.update({"value": 1e3 / main["ms"], "unit": unit, "ms_per_step": main["ms"],
                 "n_gpus": 1, "higher_is_better": True,
                 "dtype": "f64" if args.precision == "fp64" else "f64 (fp32/df64 sweeps)",
                 "e2e": dict(main["e2e"], unit=unit), "gpu_launches": main["launches"],
                 "schedule": main["schedule"], "autotune": main["tuned"], "cuda_graph": True,
                 "ranks_out": main["ranks_out"],
                 "clocks": main["clocks"],
                 "roofline": roofline_tensor(main["flops"], main["kernel_ms"], peak,
                                             flop_model="algorithmic F_round (+ F_matvec) "
                                                        "(tensor_train_gb300/flops.py)"),
                 other_prec if other_prec == "mixed" else "plain_fp64":
                     {"value": 1e3 / other["ms"], "ms_per_step": other["ms"],
                      "kernel_ms": other["kernel_ms"], "schedule": other["schedule"],
                      "autotune": other["tuned"], "e2e": dict(other["e2e"], unit=unit)},
                 "speedup_mixed_vs_plain_fp64": plain["ms"] / mixed["ms"]})
    if not args.no_cpu_baseline:
        from oracle import pyoracle as O
        t0 = time.perf_counter()
        if matvec:
            ref = O.matvec_round(inp["A"], inp["x"], inp["eps"], method=args.method)
        else:
            ref = O.round(inp["tt"], inp["eps"], gauge=args.gauge)
        sec = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": 1.0 / sec, "unit": unit, "cores": 1, "kind": "port",
                                "sample": "one full call (oracle, 1 thread; a single TT does "
                                          "not split over threads)"}
        line["parity"] = {
            "ranks_equal_mixed": O.ranks(ref) == mixed["ranks_out"],
            "ranks_equal_fp64": O.ranks(ref) == plain["ranks_out"],
            "rel_err_mixed_vs_oracle": O.rel_err(mixed["y"], ref),
            "rel_err_fp64_vs_oracle": O.rel_err(plain["y"], ref)}
    print(json.dumps(line), flush=True)


def run_sketch(args):
    """Learned-sketch rounding: d=64, n=4, interior rank 200 TTs whose bond
    spectra decay at rate rho ~ U[0.5, 0.95] per slot, eps=1e-6.  The rank
    model is trained on the exact rounder's ranks over a stream of the same
    family (smaller interior ranks, ~50k bonds); the test batch's sketch ranks
    come from the previous sweep of the same slots.  Reports the learned
    sketch against the exact rounder (mixed and plain FP64) on the same batch."""
    import numpy as np
    import torch

    import tensor_train_gb300 as T
    from tensor_train_gb300 import sketch as S
    from tensor_train_gb300.mlp import RankModel

    torch.cuda.set_device(0)
    eps, d, n = 1e-6, 64, 4
    slots = args.count if args.count != 4096 else 64
    rng = np.random.default_rng(2024)
    rhos = rng.uniform(0.5, 0.95, slots)
    t0 = time.perf_counter()
    # training stream: 8 batches, ranks 48..128, exact rounds give targets
    X, Y, prev = [], [], None
    train_terms = rng.choice([48, 64, 96, 128], slots)
    for b in range(8):
        tts = S.stream_batch(b, rhos, seed0=40000, d=d, n=n, terms=train_terms)
        _, _, stats = S.exact_round_stats(T, tts, eps)
        if prev is not None:
            X.append(S.batch_features(tts, prev))
            Y.append(np.concatenate([np.log(st[:, 2]) for st in stats]))
        prev = stats
    X, Y = np.concatenate(X), np.concatenate(Y).astype(np.float32)
    gen_s = time.perf_counter() - t0
    model = RankModel(S.N_FEATURES, 128, seed=0)
    t0 = time.perf_counter()
    hist = model.train(X, Y, epochs=60, lr=3e-3, batch=4096)
    train_s = time.perf_counter() - t0
    # test stream at full size: sweep 0 exact (features), sweep 1 measured
    warm = S.stream_batch(100, rhos, seed0=90000, d=d, n=n, terms=200)
    _, _, prev = S.exact_round_stats(T, warm, eps)
    del warm
    test = S.stream_batch(101, rhos, seed0=90000, d=d, n=n, terms=200)
    feats = S.batch_features(test, prev)
    t0 = time.perf_counter()
    ranks = S.sketch_ranks(model, feats, test)
    predict_s = time.perf_counter() - t0

    tuned = {}

    def timed(opts, tune=False):
        plan = T.Plan("round", test, opts=opts)
        sptr = torch.cuda.current_stream().cuda_stream
        plan.upload(sptr)
        if tune:  # launch configuration by the autotuner (per TT, or teams of CTAs)
            tuned[int(opts.precision)] = plan.autotune(sptr)
        for _ in range(args.warmup):
            plan.run(sptr)
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record()
        for _ in range(args.steps):
            plan.run(sptr)
        ev1.record()
        torch.cuda.synchronize()
        outs = plan.download(sptr)
        res = plan.results
        plan.close()
        return ev0.elapsed_time(ev1) / args.steps, outs, res

    with Clocks(0) as clk:
        ms_sk, outs_sk, res_sk = timed(T.RoundOptions(eps=eps, method=T.round_method.sketch,
                                                      sketch_ranks=ranks, sketch_seed=5,
                                                      precision=T.precision.mixed))
        ms_ex, outs_ex, _ = timed(T.RoundOptions(eps=eps, precision=T.precision.mixed))
        ms_64, _, _ = timed(T.RoundOptions(eps=eps, precision=T.precision.fp64))
    accepted = sum(r.sketch_state == 1 for r in res_sk)
    rank_dev = max(max(abs(a - b) for a, b in zip(
        [y[0].shape[0]] + [c.shape[-1] for c in y], [e[0].shape[0]] + [c.shape[-1] for c in e]))
        for y, e in zip(outs_sk, outs_ex))
    line = {"workload": "sketch_d64", "metric": METRIC, "unit": "roundings/s",
            "config": {"workload": f"learned-sketch rounding: {slots} TTs d=64 n=4 interior rank "
                                   "200, rho~U[0.5,0.95] per slot, eps=1e-6"},
            "value": slots / (ms_sk / 1e3), "ms_per_step": ms_sk,
            "exact_mixed": {"value": slots / (ms_ex / 1e3), "ms_per_step": ms_ex},
            "exact_plain_fp64": {"value": slots / (ms_64 / 1e3), "ms_per_step": ms_64},
            "speedup_vs_exact_mixed": ms_ex / ms_sk, "speedup_vs_plain_fp64": ms_64 / ms_sk,
            "sketch_accepted": f"{accepted}/{slots}",
            "sketch_bonds_fraction_of_input": float(ranks.sum() /
                                                     sum(sum(c.shape[-1] for c in t[:-1])
                                                         for t in test)),
            "max_rank_deviation_vs_exact": int(rank_dev),
            "training": {"bonds": int(X.shape[0]), "data_s": gen_s, "train_s": train_s,
                         "loss_first": hist[0], "loss_last": hist[-1], "predict_s": predict_s,
                         "mlp_kernel_launches": model.kernel_launches()},
            "clocks": clk.summary()}
    if not args.no_cpu_baseline:
        from oracle import pyoracle as O
        t0 = time.perf_counter()
        ref = O.round(test[0], eps)
        sec = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": 1.0 / sec, "unit": "roundings/s", "cores": 1,
                                "kind": "port", "sample": "one TT of the batch, oracle exact round"}
        line["parity"] = {"rel_err_sketch_vs_oracle": O.rel_err(outs_sk[0], ref),
                          "ranks_within_1": all(abs(a - b) <= 1 for a, b in
                                                zip(O.ranks(outs_sk[0]), O.ranks(ref)))}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "sketch_d64":
        run_sketch(args)
    elif args.workload != "batch":
        run_single(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
