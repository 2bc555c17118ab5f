"""Benchmark of the Johansen null-eigenspectra hot path on GB300.

Workload (the headline configuration): dim 12, T = 10,000 steps, models 0-4.
One step = one batch of R runs for each of the five models, each model a
separate C-ABI request (seeds 1..R, counter-based Philox increments generated
in-kernel), through the mixed-precision path (split-FP16 tensor-core Grams,
FP32 chunks, float-float merge and FP64 Cholesky + tridiagonal QL).

  value   runs/s with results left in device memory (jne_eigs_seeded_device)
  e2e     runs/s through jne_eigs_seeded: eigenvalues copied to host memory
  fp64_plain  runs/s of the plain FP64 fused kernel on the same workload
  mixed_error max relative max-eig / trace error of mixed vs FP64 on identical seeds

`--impl reference` times the CPU restatement of the reference algorithm (the
reference crate is Rust and cannot be built here) on all host cores.
Multi-GPU (torchrun): replicas over disjoint seed ranges, no collective on the
data path; only the timing barrier and a max over ranks.
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

DIM, STEPS, MODELS = 12, 10_000, (0, 1, 2, 3, 4)
METRIC = "runs/s at dim12 T=10k, FP64 vs mixed-precision at stated error; p50/p99 latency"
UNIT = "runs/s"


# DRAM bytes (read + write) of one k_accum_mixed<12> launch (accumulation + fused
# finalize) per run, from an ncu capture of the full 200,000-run launch
# (profiles/k_accum_mixed_dim12_T10k_dram.md): 18,147,072 B read + 771,372,800 B written.
# Algorithmic: 2,352 B of record written and read back, 96 B of eigenvalues per run.
ACCUM_DRAM_BYTES_PER_RUN = (18_147_072 + 771_372_800) / 200_000
# Warp instructions k_accum_mixed<12> issues per run at T = 10,000 (accumulation plus
# the run's share of its fused finalize batch), from an ncu capture of an 8,192-run
# launch (profiles/k_accum_mixed_dim12_T10k_8192runs_full.md): 1,166,615,378 / 8,192.
ACCUM_WARP_INST_PER_RUN = 142_409


def k_of(model: int) -> int:
    return DIM + 1 if model in (1, 3) else DIM


def canonical_flops(model: int) -> float:
    """W = T k (k + 1 + 2 dim): S11 (symmetric) + S10 multiply-adds, 2 flops each."""
    k = k_of(model)
    return STEPS * k * (k + 1 + 2 * DIM)


class ClockSampler:
    """nvidia-smi samples during the timed region (SM clock, throttle reasons)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device, self.proc, self.lines = device, None, []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            self.proc.wait(timeout=5)

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx = float(p[2])
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": mx, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        return {}


def replica_seed_first(rank: int, runs_per_replica: int) -> int:
    """Replicas (one per GPU) take disjoint, consecutive seed ranges: rank r runs seeds
    1 + r R .. (r + 1) R, so N replicas cover seeds 1 .. N R exactly once."""
    return 1 + rank * runs_per_replica


def reduce_max(dist, x: float, device: str) -> float:
    """Max of x over the ranks of the default process group (x itself without one)."""
    if dist is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_sample(oracle, runs_per_model: int, threads: int, seed_first: int = 1):
    """Oracle (dense restatement) on `threads` host threads; returns runs/s."""
    t0 = time.perf_counter()
    for m in MODELS:
        oracle.c_eigs_seeded(m, DIM, STEPS, seed_first, runs_per_model, n_threads=threads)
    dt = time.perf_counter() - t0
    return len(MODELS) * runs_per_model / dt, dt


def cpu_sample_for(oracle, seconds: float, threads: int, batch: int):
    """Repeats `batch` runs per model over fresh seeds until `seconds` of wall
    time have passed; returns (runs/s, runs per model, seconds)."""
    done, total, seed = 0, 0.0, 1
    while total < seconds:
        _, dt = cpu_sample(oracle, batch, threads, seed)
        done, total, seed = done + batch, total + dt, seed + batch
    return len(MODELS) * done / total, done, total


def run_reference(args, rank: int, world: int) -> None:
    if rank != 0:
        return
    import __graft_entry__ as entry

    oracle = entry.load_oracle()
    threads = os.cpu_count() or 1
    per_model = args.cpu_runs or 128 * threads  # ~3 s per step on 16 Neoverse-V2 cores
    for _ in range(args.warmup):
        cpu_sample(oracle, max(threads, per_model // 4), threads)
    times = []
    for _ in range(args.steps):
        _, dt = cpu_sample(oracle, per_model, threads)
        times.append(dt)
    total = sum(times)
    value = len(MODELS) * per_model * args.steps / total
    sample = f"{per_model} runs x 5 models per step (seeds 1..{per_model}), dim {DIM}, T {STEPS}"
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (counter-based Philox normals)",
        "config": {"workload": f"dim {DIM}, T {STEPS}, models 0-4, CPU restatement of the reference algorithm",
                   "runs_per_model_per_step": per_model},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def run_gpu(args, rank: int, world: int) -> None:
    import torch

    import __graft_entry__ as entry

    jne = entry.load_package()
    local = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    eng = jne.Engine(local, chunk=args.chunk)
    R = args.runs
    seed0 = replica_seed_first(rank, R)
    stream = torch.cuda.Stream()
    sptr = stream.cuda_stream
    # requests alternate between two caller streams, so the finalize of one
    # request (on the engine's second stream) overlaps the next accumulation
    streams = [stream, torch.cuda.Stream()]
    outs = {m: torch.empty((R, k_of(m)), dtype=torch.float64, device="cuda") for m in MODELS}

    def step_device(prec):
        for j, m in enumerate(MODELS):
            st = streams[j % 2]
            eng.eigs_seeded_device(m, DIM, STEPS, seed0, R, outs[m].data_ptr(), precision=prec, stream=st.cuda_stream)

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    def max_over_ranks(x: float) -> float:
        return reduce_max(dist, x, "cuda")

    # ---- mixed precision, device-resident outputs (value) ----
    for _ in range(args.warmup):
        step_device(jne.PREC_MIXED)
    barrier()
    step_ms = []
    eng.profile(True)  # per-kernel CUDA events on the launching stream
    eng.profile_read(reset=True)
    with ClockSampler(local) as clk:
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        streams[1].wait_stream(stream)
        marks = []
        for _ in range(args.steps):
            step_device(jne.PREC_MIXED)
            stream.wait_stream(streams[1])
            e = torch.cuda.Event(enable_timing=True)
            e.record(stream)
            streams[1].wait_stream(stream)
            marks.append(e)
        ev1.record(stream)
        barrier()
    ms = max_over_ranks(ev0.elapsed_time(ev1))
    prev = ev0
    for e in marks:
        step_ms.append(prev.elapsed_time(e))
        prev = e
    eng.sync()  # device status of the asynchronous calls
    prof = eng.profile_read(reset=True)
    eng.profile(False)
    runs_per_step = R * len(MODELS) * world
    value = runs_per_step * args.steps / (ms * 1e-3)
    # latency of one request issued alone (device time, synchronous)
    iso = []
    for m in MODELS:
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        eng.eigs_seeded_device(m, DIM, STEPS, seed0, R, outs[m].data_ptr(), precision=jne.PREC_MIXED, stream=sptr)
        b.record(stream)
        b.synchronize()
        iso.append(a.elapsed_time(b))
    eng.sync()
    p50 = float(np.percentile(iso, 50))
    p99 = float(np.percentile(iso, 99))

    # ---- end to end through the host-memory C call (e2e) ----
    host = {m: np.empty((R, k_of(m))) for m in MODELS}

    def step_host():
        for m in MODELS:
            host[m] = eng.eigs_seeded(m, DIM, STEPS, seed0, R, precision=jne.PREC_MIXED)

    step_host()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step_host()
    barrier()
    e2e_s = max_over_ranks(time.perf_counter() - t0)
    e2e = runs_per_step * args.steps / e2e_s
    d2h = sum(R * k_of(m) * 8 for m in MODELS)

    # ---- plain FP64 fused kernel on the same workload (fewer runs) ----
    Rf = args.fp64_runs
    for m in MODELS:
        eng.eigs_seeded_device(m, DIM, STEPS, seed0, Rf, outs[m].data_ptr(), precision=jne.PREC_FP64, stream=sptr)
    barrier()
    f0 = torch.cuda.Event(enable_timing=True)
    f1 = torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    for m in MODELS:
        eng.eigs_seeded_device(m, DIM, STEPS, seed0, Rf, outs[m].data_ptr(), precision=jne.PREC_FP64, stream=sptr)
    f1.record(stream)
    barrier()
    eng.sync()
    fp64_ms = max_over_ranks(f0.elapsed_time(f1))
    fp64_value = Rf * len(MODELS) * world / (fp64_ms * 1e-3)

    # ---- accuracy of mixed vs FP64 on identical seeds (subset) ----
    err = {}
    ns = min(args.err_runs, R)
    for m in MODELS:
        f = eng.eigs_seeded(m, DIM, STEPS, seed0, ns, precision=jne.PREC_FP64)
        x = eng.eigs_seeded(m, DIM, STEPS, seed0, ns, precision=jne.PREC_MIXED)
        err[str(m)] = {"maxeig": float(np.max(np.abs(x[:, 0] - f[:, 0]) / f[:, 0])),
                       "trace": float(np.max(np.abs(x.sum(1) - f.sum(1)) / f.sum(1)))}

    # ---- dominant kernel: mixed accumulation, from the timed region's events ----
    acc_ms, acc_n = prof["accum_mixed"]
    fin_ms, fin_n = prof["finalize"]
    kern = {"accum_mixed": {"launches": acc_n, "total_ms": acc_ms, "mean_ms": acc_ms / max(acc_n, 1)},
            "finalize": {"launches": fin_n, "total_ms": fin_ms, "mean_ms": fin_ms / max(fin_n, 1)},
            "share_accum": acc_ms / max(acc_ms + fin_ms, 1e-9)}
    mean_acc_ms = acc_ms / max(acc_n, 1)
    peaks = measured_peaks()
    bf16 = peaks.get("bf16_tflops")
    W = sum(canonical_flops(m) for m in MODELS) / len(MODELS)
    achieved = W * R / (mean_acc_ms * 1e-3) / 1e12
    traffic = args.traffic if args.traffic is not None else ACCUM_DRAM_BYTES_PER_RUN * R
    roof = {"bound": "tensor", "achieved": achieved, "peak": bf16, "unit": "TFLOP/s",
            "frac": (achieved / bf16) if bf16 else None, "traffic": traffic,
            "traffic_note": "ncu dram bytes of one full 200k-run launch (accumulation + fused finalize), per "
                            "run x runs per launch; algorithmic: 2,352 B/run of records, 96 B/run of eigenvalues",
            "kernel": "k_accum_mixed<12,false,4,true>", "peak_source": "measured bf16_tflops (burst)" if bf16 else "none",
            "flops_per_run": W}
    normals_rate = DIM * STEPS * R / (mean_acc_ms * 1e-3)
    rates = eng.probe_rates()
    rng_peak = args.rng_peak or rates["normals_per_s"]
    issue = {"normals_per_s": normals_rate, "peak_normals_per_s": rng_peak,
             "frac": normals_rate / rng_peak, "probe_rates": rates,
             "note": "normals/s the accumulation kernel draws vs the rate of the same Philox4x32-10 + "
                     "Box-Muller device code alone (jne_probe_rates, measured in this run)"}
    # the tensor work the kernel executes: per 16 steps, 3 Gram blocks x 3 split products of m16n8k16 FP16
    # (4,096 flops each); against mma.sync FP16 (FP32 accumulation) measured by the probe in this run
    mma_flops = 9 * 4096 * (STEPS // 16) * R / (mean_acc_ms * 1e-3)
    roof["tensor_pipe"] = {"executed_tflops": mma_flops / 1e12, "peak_tflops": rates["mma_f16_flops"] / 1e12,
                           "frac": mma_flops / rates["mma_f16_flops"],
                           "note": "executed split-FP16 mma.sync work (not algorithmic flops) vs the measured "
                                   "mma.sync FP16 rate"}

    # SIMT issue, the kernel's binding limit: one warp instruction per cycle per scheduler
    # (4 per SM) at the SM clock sampled in the timed region
    clocks = clk.summary()
    sm_hz = (clocks.get("sm_mhz") or clocks.get("sm_max_mhz") or 0) * 1e6
    issue_peak = torch.cuda.get_device_properties(local).multi_processor_count * 4 * sm_hz
    inst_rate = ACCUM_WARP_INST_PER_RUN * R / (mean_acc_ms * 1e-3)
    issue["warp_issue"] = {"achieved_inst_per_s": inst_rate, "peak_inst_per_s": issue_peak,
                           "frac": inst_rate / issue_peak if issue_peak else None,
                           "inst_per_run": ACCUM_WARP_INST_PER_RUN,
                           "note": "warp instructions per run (ncu) x runs/s of the timed launches vs 4 issue "
                                   "slots per SM per cycle at the sampled SM clock"}

    ragged = bench_ragged60(jne, torch, local, args.ragged_steps) if args.ragged_steps > 0 and rank == 0 else None
    ragged_tuned = (bench_ragged60(jne, torch, local, args.ragged_steps, tune=args.tune_err)
                    if args.ragged_steps > 0 and args.tune_err > 0 and rank == 0 else None)
    precision = bench_precision(jne, torch, local, args.c3_runs) if args.c3_runs > 0 and rank == 0 else None
    tuned_single = (bench_tuned_single(jne, torch, local, args.tune_err)
                    if args.tune_err > 0 and rank == 0 else None)
    # all five models of the same seeds from one pass over the paths (jne_eigs_seeded_models): the path of a
    # seed does not depend on the model, so one accumulation serves five finalizes; host outputs
    eng.eigs_seeded_models(list(MODELS), DIM, STEPS, seed0, R, precision=jne.PREC_MIXED)  # warm, full size
    torch.cuda.synchronize()
    walls = []
    for _ in range(2):
        t0 = time.perf_counter()
        eng.eigs_seeded_models(list(MODELS), DIM, STEPS, seed0, R, precision=jne.PREC_MIXED)
        walls.append(time.perf_counter() - t0)
    one_pass_s = min(walls)
    one_pass = {"runs_per_s": len(MODELS) * R / one_pass_s, "seconds": one_pass_s,
                "workload": f"models 0-4 x {R} seeds, dim {DIM}, T {STEPS}, mixed, one accumulation per seed "
                            "(jne_eigs_seeded_models), eigenvalues copied to host memory; wall clock, the faster "
                            "of two calls after a full-size warm-up",
                "note": "not the headline: the headline runs one request per model, as the reference does"}
    packer = bench_record_packer(jne, torch, eng, args.pack_records) if args.pack_records > 0 and rank == 0 else None
    serving = None
    if rank == 0 and (args.serve_seconds > 0 or args.serve_low_seconds > 0):
        serving = {}
        if args.serve_low_seconds > 0:
            serving["low"] = bench_serving(jne, local, args.serve_low_seconds, rate=args.serve_low_rate)
        if args.serve_seconds > 0:
            serving["high"] = bench_serving(jne, local, args.serve_seconds, rate=args.serve_rate)

    cpu = None
    if rank == 0 and args.cpu_runs != 0:
        oracle = entry.load_oracle()
        threads = os.cpu_count() or 1
        if args.cpu_runs:
            per = args.cpu_runs
            v, dt = cpu_sample(oracle, per, threads)
        else:
            v, per, dt = cpu_sample_for(oracle, args.cpu_seconds, threads, 16 * threads)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{per} runs x 5 models (seeds 1..{per}), dim {DIM}, T {STEPS}, {dt:.1f} s wall"}
        if precision is not None and args.oracle_runs > 0:
            # the oracle as the checker of the precision line: its dense restatement on the increments the
            # kernels draw for the first runs, against the mixed and FP64 results of the same seeds
            precision["vs_oracle"] = precision_vs_oracle(jne, local, oracle, args.oracle_runs, threads)

    if rank == 0:
        print(json.dumps({
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f16x3-split/f32/f64", "data": "synthetic (in-kernel Philox normals)",
            "config": {"workload": f"dim {DIM}, T {STEPS}, models 0-4, {R} runs per model per step "
                                   f"(one request per model), mixed precision",
                       "runs_per_model_per_step": R, "chunk": args.chunk,
                       "l2": "working set larger than L2: moment records of a 5-model step are "
                             f"{R * 294 * 8 * 5 / 1e9:.2f} GB; no inputs (increments generated in-kernel)",
                       "parallelism": f"replicas x{world} over disjoint seed ranges"},
            "latency_ms": {"request_alone_p50": p50, "request_alone_p99": p99,
                           "request": f"{R} runs of one model, issued alone",
                           "step_p50": float(np.percentile(step_ms, 50)), "step_p99": float(np.percentile(step_ms, 99)),
                           "step": "5 requests, one per model, pipelined"},
            "fp64_plain": {"value": fp64_value, "unit": UNIT, "runs_per_model": Rf,
                           "mixed_speedup": value / fp64_value},
            "mixed_error": {"vs": "plain FP64 kernel, identical seeds", "runs_per_model": ns, "per_model": err},
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": d2h},
            "gpu_launches": acc_n + fin_n,
            "roofline": roof, "issue_bound": issue, "kernel_ms": kern,
            "ragged60": ragged, "ragged60_tuned": ragged_tuned, "tuned_single": tuned_single, "serving": serving, "precision_model4": precision, "models_one_pass": one_pass,
            "record_packer": packer,
            "cpu_baseline": cpu, "clocks": clocks,
        }))
    eng.close()
    if dist is not None:
        dist.destroy_process_group()


def ragged60_requests(seed: int = 0xC4):
    """All 60 (model, dim) pairs; T from {1000, 5000, 10000} and runs log-uniform in [1e4, 1e6], per pair."""
    rng = np.random.default_rng(seed)
    reqs = []
    for model in MODELS:
        for dim in range(1, 13):
            reqs.append(dict(model=model, dim=dim, steps=int(rng.choice([1000, 5000, 10000])),
                             n_runs=int(np.exp(rng.uniform(np.log(1e4), np.log(1e6))))))
    return reqs


def tune_classes(eng, classes, max_rel_err: float) -> dict:
    """Autotuner over the (dim, steps) classes of a workload (512 sample runs per model, 16,384-run timed
    launches); returns {"dim x 2^b": chunk} -- the ragged kernel takes the chunk of each tuned shape."""
    out = {}
    for dim, steps in sorted(set(classes)):
        if steps >= 256:
            best, _ = eng.autotune(dim, steps, max_rel_err=max_rel_err, sample_runs=512, time_runs=16384)
            out[f"{dim}x{1 << (steps.bit_length() - 1)}"] = best["chunk"]
    eng.set_chunk(-1)  # CHUNK_TUNED
    return out


def bench_tuned_single(jne, torch, local: int, max_rel_err: float, shapes=((2, 1000), (6, 1000), (12, 10_000))):
    """Single requests (model 0) with the default launch shape and with the autotuned one (2,000 sample runs
    per model for the error bound, timed candidates), device outputs, CUDA events; plus the tuner's table."""
    out = []
    with jne.Engine(local) as eng:
        st = torch.cuda.Stream()
        for dim, steps in shapes:
            best, table = eng.autotune(dim, steps, max_rel_err=max_rel_err, sample_runs=2000)
            runs = int(min(4_000_000, max(65_536, 4e10 / (steps * (dim + 3)))))
            buf = torch.empty((runs, dim), dtype=torch.float64, device="cuda")
            rates = {}
            for mode in (0, -1):  # default rule, then CHUNK_TUNED
                eng.set_chunk(mode)
                eng.eigs_seeded_device(0, dim, steps, 1, runs, buf.data_ptr(), precision=jne.PREC_MIXED,
                                       stream=st.cuda_stream)
                eng.sync()
                a = torch.cuda.Event(enable_timing=True)
                b = torch.cuda.Event(enable_timing=True)
                a.record(st)
                for _ in range(3):
                    eng.eigs_seeded_device(0, dim, steps, 1, runs, buf.data_ptr(), precision=jne.PREC_MIXED,
                                           stream=st.cuda_stream)
                b.record(st)
                b.synchronize()
                eng.sync()
                rates["default" if mode == 0 else "tuned"] = 3 * runs / (a.elapsed_time(b) * 1e-3)
            eng.set_chunk(0)
            out.append({"dim": dim, "steps": steps, "runs": runs, "default_runs_per_s": rates["default"],
                        "tuned_runs_per_s": rates["tuned"], "gain": rates["tuned"] / rates["default"],
                        "chosen": best, "table": table})
    return {"max_rel_err": max_rel_err, "shapes": out,
            "note": "default: chunk rule, 4 blocks per SM, two runs per warp for dims <= 4; tuned: the fastest "
                    "measured shape whose chunk meets the bound on 2,000 runs per model"}


def bench_ragged60(jne, torch, local: int, steps: int, tune: float = 0.0) -> dict:
    """One persistent launch over the ragged 60-pair batch, captured as a CUDA graph and replayed.
    With tune > 0 the chunk lengths come from the autotuner at that error bound."""
    reqs = ragged60_requests()
    total = sum(r["n_runs"] for r in reqs)
    outs = [torch.empty((r["n_runs"], jne.eigen_count(r["model"], r["dim"])), dtype=torch.float64, device="cuda")
            for r in reqs]
    with jne.Engine(local) as eng:
        chunks = tune_classes(eng, [(r["dim"], r["steps"]) for r in reqs], tune) if tune > 0 else None
        plan = eng.plan(reqs, [o.data_ptr() for o in outs])
        stream = torch.cuda.Stream()
        plan.launch(stream.cuda_stream)  # warm-up replay
        eng.sync()
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(steps):
            plan.launch(stream.cuda_stream)
        b.record(stream)
        torch.cuda.synchronize()
        eng.sync()
        ms = a.elapsed_time(b) / steps
        plan.destroy()
    finite = all(bool(torch.isfinite(o).all()) for o in outs)
    return {"runs_per_s": total / (ms * 1e-3), "ms_per_replay": ms, "requests": len(reqs), "total_runs": total,
            "replays": steps, "all_finite": finite, "graph": True,
            "chunks": f"autotuned at max error {tune:g}: {chunks}" if chunks else "default rule",
            "workload": "60 (model, dim) pairs, T in {1000,5000,10000} and runs log-uniform [1e4,1e6] per pair "
                        "(seed 0xC4), mixed precision, one persistent ragged launch + ragged finalize per replay"}


def bench_precision(jne, torch, local: int, runs: int, subset: int = 10_000) -> dict:
    """Model 4, dim 12, T 1e4: `runs` runs in mixed precision (device outputs), and the max-eig / trace error
    of the first `subset` of them against the plain FP64 kernel on the same seeds."""
    k = jne.eigen_count(4, DIM)
    out = torch.empty((runs, k), dtype=torch.float64, device="cuda")
    with jne.Engine(local) as eng:
        stream = torch.cuda.Stream()
        eng.eigs_seeded_device(4, DIM, STEPS, 1, min(runs, 100_000), out.data_ptr(), precision=jne.PREC_MIXED,
                               stream=stream.cuda_stream)  # warm-up
        eng.sync()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        eng.eigs_seeded_device(4, DIM, STEPS, 1, runs, out.data_ptr(), precision=jne.PREC_MIXED,
                               stream=stream.cuda_stream)
        b.record(stream)
        torch.cuda.synchronize()
        eng.sync()
        ms = a.elapsed_time(b)
        ns = min(subset, runs)
        f = eng.eigs_seeded(4, DIM, STEPS, 1, ns, precision=jne.PREC_FP64)
    x = out[:ns].cpu().numpy()
    rel_max = np.abs(x[:, 0] - f[:, 0]) / f[:, 0]
    rel_tr = np.abs(x.sum(1) - f.sum(1)) / f.sum(1)
    return {"runs": runs, "runs_per_s": runs / (ms * 1e-3), "error_subset": ns,
            "maxeig_rel_err": {"max": float(rel_max.max()), "p99": float(np.percentile(rel_max, 99)),
                               "mean": float(rel_max.mean())},
            "trace_rel_err": {"max": float(rel_tr.max()), "p99": float(np.percentile(rel_tr, 99)),
                              "mean": float(rel_tr.mean())},
            "workload": f"model 4, dim {DIM}, T {STEPS}, {runs} runs mixed (seeds 1..{runs}); error of the first "
                        f"{ns} vs the plain FP64 kernel on the same seeds"}


def precision_vs_oracle(jne, local: int, oracle, runs: int, threads: int) -> dict:
    """Model 4, dim 12, T 1e4, seeds 1..runs: max-eig / trace error of the mixed kernel and the normwise error
    of the FP64 kernel against the CPU oracle walking the same increments (exported by the kernels' RNG)."""
    with jne.Engine(local) as eng:
        dB, _ = eng.export_increments(DIM, STEPS, 1, runs)
        mix = eng.eigs_seeded(4, DIM, STEPS, 1, runs, precision=jne.PREC_MIXED)
        f64 = eng.eigs_seeded(4, DIM, STEPS, 1, runs, precision=jne.PREC_FP64)
    ref = oracle.c_eigs_from_increments(4, dB, n_threads=threads)
    rel_max = np.abs(mix[:, 0] - ref[:, 0]) / ref[:, 0]
    rel_tr = np.abs(mix.sum(1) - ref.sum(1)) / ref.sum(1)
    nw = np.max(np.abs(f64 - ref), axis=1) / np.max(np.abs(ref), axis=1)
    return {"runs": runs, "mixed_maxeig_rel_err_max": float(rel_max.max()),
            "mixed_trace_rel_err_max": float(rel_tr.max()), "fp64_normwise_err_max": float(nw.max()),
            "oracle": "C restatement of the dense reference algorithm on the kernels' own increments"}


def bench_record_packer(jne, torch, eng, n: int, k: int = 13, reps: int = 10) -> dict:
    """The .dat sink's device record packer on one sink round's worth of results (n records of k values,
    seeds 1..n), timed with CUDA events on its launching stream, against the measured HBM copy bandwidth;
    beside it the host encoder (jne_dat_append) writing the same records to a file."""
    import tempfile

    nbytes = jne.record_bytes(1, n, k)
    eigs = torch.randn((n, k), dtype=torch.float64, device="cuda")
    buf = torch.empty(nbytes + 16, dtype=torch.uint8, device="cuda")
    st = torch.cuda.Stream()
    torch.cuda.synchronize()

    def launch():
        eng.pack_records_device(1, n, k, eigs.data_ptr(), buf.data_ptr(), nbytes + 16, stream=st.cuda_stream)

    for _ in range(3):
        launch()
    st.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(reps):
        launch()
    e1.record(st)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / reps
    moved = 8 * n * k + nbytes  # values read + records written
    hbm = measured_peaks().get("hbm_gbs")
    gbs = moved / (ms * 1e-3) / 1e9
    host = eigs.cpu().numpy()
    seeds = np.arange(1, n + 1, dtype=np.uint32)
    with tempfile.TemporaryDirectory() as d:
        w = jne.DatWriter(os.path.join(d, "enc.dat"), 1, k - 1, 100)  # model 1: k = dim + 1
        t0 = time.perf_counter()
        w.append(seeds, host)
        host_s = time.perf_counter() - t0
        w.abandon()
    return {"records": n, "values_per_record": k, "bytes": nbytes, "ms_per_launch": ms,
            "records_per_s": n / (ms * 1e-3),
            "roofline": {"bound": "hbm", "achieved": gbs, "peak": hbm, "unit": "GB/s",
                         "frac": gbs / hbm if hbm else None, "algorithmic_bytes": moved,
                         "peak_source": "measured hbm_gbs" if hbm else "none"},
            "host_encode_records_per_s": n / host_s,
            "workload": f"{n} records of {k} f64 (seeds 1..{n}, 1-3 byte ULEB128 seeds) packed on the GPU "
                        f"(k_pack_records, mean of {reps} launches, inputs and output {moved / 1e6:.0f} MB > L2); "
                        "host line: jne_dat_append of the same records into a file (wall clock)"}


def bench_serving(jne, local: int, seconds: float, rate: float = 200.0, seed: int = 0xC5) -> dict:
    """Poisson arrivals (mean `rate` req/s) for `seconds`; model U{0..4}, dim U{1..12}, T log-U[500, 2e4],
    runs log-U[1e3, 1e6], per-request seed; 40 GB budget.  Latency = finish - submit, split into queueing
    (start - submit: waiting for admission and the first iteration) and service (finish - start).  Offered
    load = runs submitted / arrival window; served = runs / makespan (first submit to last finish).  When the
    offered load exceeds what the GPU serves, the backlog grows for the whole window and the latency measures
    how long it takes to drain, not a steady state: the line says so (`saturated`)."""
    rng = np.random.default_rng(seed)
    arrivals, t = [], 0.0
    while True:
        t += rng.exponential(1.0 / rate)
        if t > seconds:
            break
        arrivals.append((t, dict(model=int(rng.integers(0, 5)), dim=int(rng.integers(1, 13)),
                                 steps=int(np.exp(rng.uniform(np.log(500), np.log(2e4)))),
                                 n_runs=int(np.exp(rng.uniform(np.log(1e3), np.log(1e6)))),
                                 base_seed=int(rng.integers(1, 2**62)))))
    total_runs = sum(r["n_runs"] for _, r in arrivals)
    with jne.Engine(local, mem_budget_bytes=40 << 30) as eng:
        with jne.Server(eng) as srv:
            t0 = time.perf_counter()
            ids = []
            for at, r in arrivals:
                delay = at - (time.perf_counter() - t0)
                if delay > 0:
                    time.sleep(delay)
                ids.append(srv.submit(**r))
            done, t_wait = {}, time.perf_counter()
            while len(done) < len(ids):
                if time.perf_counter() - t_wait > 300:
                    raise RuntimeError(f"serving: only {len(done)} of {len(ids)} requests finished")
                for c in srv.wait(timeout_ms=5_000):
                    done[c.id] = c
            for i in ids:
                srv.fetch(i)
    lat = np.array([done[i].finish_s - done[i].submit_s for i in ids])
    queue = np.array([done[i].start_s - done[i].submit_s for i in ids])
    service = np.array([done[i].finish_s - done[i].start_s for i in ids])
    span = max(c.finish_s for c in done.values()) - min(c.submit_s for c in done.values())
    window = max(at for at, _ in arrivals) if arrivals else seconds
    ok = sum(1 for c in done.values() if c.status == jne.JNE_OK)
    offered, served = total_runs / max(window, 1e-9), total_runs / span
    # below saturation the server keeps up: the last request finishes soon after the last arrival; above
    # it a backlog builds and drains after the window
    saturated = bool(span > 1.2 * window + 0.5)

    def pct(x):
        return {"p50": float(np.percentile(x, 50)), "p99": float(np.percentile(x, 99))}

    return {"requests": len(ids), "ok": ok, "offered_req_per_s": rate, "arrival_seconds": seconds,
            "total_runs": total_runs, "offered_runs_per_s": offered, "served_runs_per_s": served,
            "runs_per_s": served, "p50_latency_s": float(np.percentile(lat, 50)),
            "p99_latency_s": float(np.percentile(lat, 99)), "queue_s": pct(queue), "service_s": pct(service),
            "makespan_s": span, "saturated": saturated,
            "note": ("offered load above the served rate: the backlog grows through the arrival window and the "
                     "latencies measure its drain" if saturated else
                     "offered load below the served rate: steady-state latencies"),
            "workload": f"Poisson {rate:g} req/s for {seconds:g} s; model U{{0..4}}, dim U{{1..12}}, "
                        "T log-U[500,2e4], runs log-U[1e3,1e6], per-request seed; continuous batching, "
                        "40 GB budget, mixed precision"}


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--runs", type=int, default=200_000, help="runs per model per step")
    ap.add_argument("--fp64-runs", type=int, default=20_000)
    ap.add_argument("--err-runs", type=int, default=2_000)
    ap.add_argument("--cpu-runs", type=int, default=None, help="CPU sample runs per model (0 = skip)")
    ap.add_argument("--cpu-seconds", type=float, default=15.0, help="CPU baseline sample length without --cpu-runs")
    ap.add_argument("--chunk", type=int, default=0, help="steps per FP32 chunk (0: adaptive, 512 at T=10k)")
    ap.add_argument("--traffic", type=float, default=None,
                    help="ncu dram bytes per accumulation launch (default: the committed capture, scaled by runs)")
    ap.add_argument("--ragged-steps", type=int, default=2, help="timed replays of the ragged 60-pair plan (0: skip)")
    ap.add_argument("--serve-seconds", type=float, default=3.0,
                    help="arrival window of the serving run at --serve-rate (0: skip)")
    ap.add_argument("--serve-rate", type=float, default=200.0, help="Poisson arrivals per second (saturating)")
    ap.add_argument("--serve-low-seconds", type=float, default=20.0,
                    help="arrival window of the serving run at --serve-low-rate (0: skip)")
    ap.add_argument("--serve-low-rate", type=float, default=50.0, help="Poisson arrivals per second (below saturation)")
    ap.add_argument("--tune-err", type=float, default=1e-6,
                    help="error bound of the chunk autotuner for the tuned ragged line (0: skip)")
    ap.add_argument("--oracle-runs", type=int, default=200,
                    help="runs of the model-4 precision line also checked against the CPU oracle (0: skip)")
    ap.add_argument("--c3-runs", type=int, default=10_000_000,
                    help="model-4 precision run: mixed runs (error on the first 10,000 vs FP64; 0: skip)")
    ap.add_argument("--pack-records", type=int, default=1 << 20,
                    help="records of the device record packer line (0: skip)")
    ap.add_argument("--rng-peak", type=float, default=None,
                    help="Philox+Box-Muller normals/s (default: measured live by jne_probe_rates)")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_gpu(args, rank, world)


if __name__ == "__main__":
    main()
