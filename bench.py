"""Benchmark: dense CP-ALS sweeps/s at 512^3 rank 64 on one GB300.

Workload (synthetic, seeded): float32 512x512x512 tensor from a rank-64 CP
model with N(0,1) unit-norm factor columns plus 20 dB Gaussian noise
(tensorly_gb300.workloads.dense_cp_large); rank 64; 50 ALS sweeps per step
(tol=0, fixed count), init='random' with seed 0.  One step = one full
``parafac`` call.  The tensor (512 MiB f32) is larger than L2 (129 MB), so no
L2 flush is needed between steps.

Arms:
  default            tensorly_gb300 on the GPU (precision bf16 = tensor-core
                     MTTKRP + 1 closing f32 sweep, --refine N for N, or
                     --precision native)
  --impl reference   the NumPy restatement of TensorLy's CPU path (oracle/)
                     on the host cores, a bounded sample of sweeps per step

One JSON line on rank 0.  Under torchrun each rank runs an independent
replica (the path does not shard); value = all ranks' sweeps / max time.
"""

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "CP-ALS sweeps/s at 512^3 R64"
UNIT = "sweeps/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--precision", default=os.environ.get("TLGB_BENCH_PRECISION", "bf16"),
                   choices=["bf16", "native"])
    p.add_argument("--size", type=int, default=512)
    p.add_argument("--rank", type=int, default=64)
    p.add_argument("--sweeps", type=int, default=50)
    p.add_argument("--refine", type=int, default=1)
    p.add_argument("--cpu-sweeps", type=int, default=40)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--workload", default="dense",
                   choices=["dense", "batched", "learned", "tucker", "nncp", "reconstruct",
                            "randomised"],
                   help="dense: 512^3 rank-64 CP-ALS (the headline); batched: 4096 uneven "
                        "3-way tensors, 100 sweeps each; learned: time to fit 10000 32^3 "
                        "rank-8 tensors from the learned warm start vs init='svd'; tucker: "
                        "128^4 Tucker-HOOI rank 16^4 (20 iterations) and CP rank 32; nncp: "
                        "non-negative CP (multiplicative updates and HALS) at 512^3 rank 64")
    p.add_argument("--train-samples", type=int, default=200_000,
                   help="learned: tensors the network is trained on (before the timed steps)")
    p.add_argument("--count", type=int, default=4096, help="batched: number of tensors")
    p.add_argument("--no-tune", action="store_true",
                   help="dense: keep the library's tensor-core MTTKRP tile defaults")
    p.add_argument("--no-extras", action="store_true",
                   help="dense: headline line only (no plain-f32, batched and 128^4 sub-objects)")
    p.add_argument("--profile", action="store_true",
                   help="run only the warm-up and timed steps (for ncu launch lists)")
    return p.parse_args()


def job_time_ms(ms, ws, device="cpu"):
    """The job's timed region: the max over the ranks' own timings (ms); one
    rank returns its own."""
    if ws <= 1:
        return ms
    import torch
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


# ----------------------------------------------------------------------------- clocks
class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons while running."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
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
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for name, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(self.rows)}


def measured_peaks():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ----------------------------------------------------------------------------- CPU arm
def cpu_sample(x, init, rank, sweeps):
    """Times `sweeps` ALS sweeps of the NumPy restatement of TensorLy's parafac
    on the host cores; returns (sweeps/s, seconds)."""
    import oracle
    w = np.ones(rank, dtype=x.dtype)
    t0 = time.perf_counter()
    oracle.parafac_sweeps(x, w, init, sweeps)
    dt = time.perf_counter() - t0
    return sweeps / dt, dt


def run_reference(args):
    """The reference arm: TensorLy's CPU path for this workload, timed on the
    host cores.  TensorLy is pure Python and its source tree is not present
    where the bench runs, so the arm runs the NumPy restatement of its
    parafac (oracle/), which makes the same NumPy/LAPACK calls.  The steps
    continue ONE run, as parafac does: ||X|| is computed once before the
    timed steps (tensorly/decomposition/_cp.py:350) and each step carries the
    factors on by `sweeps_per_step` sweeps."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from tensorly_gb300 import workloads
    import oracle
    x, _ = workloads.dense_cp_large(size=args.size, rank=args.rank)
    rs = np.random.RandomState(0)
    factors = [rs.random_sample((args.size, args.rank)).astype(np.float32) for _ in range(3)]
    weights = np.ones(args.rank, dtype=x.dtype)
    cores = os.cpu_count()
    per_step = 2
    norm_x = oracle.tensorly_oracle.norm(x)
    for _ in range(args.warmup):
        weights, factors, _ = oracle.parafac_sweeps(x, weights, factors, per_step, norm_tensor=norm_x)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        weights, factors, _ = oracle.parafac_sweeps(x, weights, factors, per_step, norm_tensor=norm_x)
        times.append(time.perf_counter() - t0)
    value = per_step * args.steps / sum(times)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * sum(times) / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": f"dense CP-ALS {args.size}^3 f32 rank {args.rank}",
                       "step": f"{per_step} ALS sweeps of one continuing run (bounded sample of "
                               f"the {args.sweeps}-sweep run); ||X|| once, as parafac does",
                       "l2": "input larger than L2"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{per_step * args.steps} sweeps of the NumPy restatement "
                                       "of tensorly parafac (explicit KR + GEMM + LAPACK gesv), "
                                       "BLAS on all host cores"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------- GPU arm
def launches_per_step(ndim, sweeps, refine, precision, rank=64):
    """Kernel launches of one parafac call (library structure; matches the
    ncu launch list of a call):
    set-up: the norm (2: partial sums + final) and one Gram per mode (2
    each); in bf16 the tensor split also sums the norm (1 + 1) and the factor
    planes add one launch per mode;
    per sweep and mode: the factorisation (1, with its f64 fallback in the
    same launch), MTTKRP (1; 2 in the closing sweeps: x0 and x1 planes),
    solve (1), Gram reduction (1; the last mode's also computes the fit).
    The last closing sweep runs its last mode's MTTKRP on the SIMT kernel
    (1)."""
    mode_cost = 4
    if precision != "bf16":
        return 2 + 2 * ndim + sweeps * mode_cost * ndim
    setup = 2 + 2 * ndim + ndim
    refine = min(refine, sweeps)
    bf16 = sweeps - refine
    if refine == 0:
        return setup + bf16 * mode_cost * ndim
    closing = mode_cost + 1                      # two MTTKRP launches per mode
    n = setup + bf16 * mode_cost * ndim
    n += (refine - 1) * closing * ndim
    n += closing * (ndim - 1) + mode_cost
    return n


# DRAM bytes (read + write) per launch of the dominant kernel at 512^3 rank 64,
# from one-kernel ncu captures (dram__bytes_read.sum + dram__bytes_write.sum;
# the bf16 figure from the tcgen05 MTTKRP with the default tiles, the native
# one from the SIMT f32 MTTKRP, both at their current builds).
NCU_TRAFFIC = {"native": 537303552 + 5170944, "bf16": 268758784 + 3906816}
KERNEL = {"native": "mttkrp_split_kernel<float,64> + reduce (SIMT f32)",
          "bf16": "mttkrp_tc_kernel (tcgen05 bf16, TMA)"}


def congruence(fa, fb):
    """Mean factor congruence of two CP models after matching components
    (Hungarian assignment on the product over modes of |cosine|)."""
    from scipy.optimize import linear_sum_assignment
    r = fa[0].shape[1]
    c = np.ones((r, r))
    for a, b in zip(fa, fb):
        an = a / np.maximum(np.linalg.norm(a, axis=0), 1e-300)
        bn = b / np.maximum(np.linalg.norm(b, axis=0), 1e-300)
        c *= np.abs(an.T @ bn)
    ri, ci = linear_sum_assignment(-c)
    return float(c[ri, ci].mean())


def run_gpu(args):
    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    import tensorly_gb300 as tg
    tg.build() if not os.path.exists(tg._lib.library_path()) else None
    from tensorly_gb300 import workloads
    dev = torch.device("cuda", torch.cuda.current_device())

    x_np, _ = workloads.dense_cp_large(size=args.size, rank=args.rank)
    rs = np.random.RandomState(0)
    init_np = [rs.random_sample((args.size, args.rank)).astype(np.float32) for _ in range(3)]
    x_host = torch.from_numpy(x_np).pin_memory()
    x = x_host.to(dev)
    init = [torch.from_numpy(f).to(dev) for f in init_np]

    kw = dict(n_iter_max=args.sweeps, tol=0, precision=args.precision,
              refine_sweeps=args.refine, return_errors=True)
    tiles = None
    if args.precision == "bf16" and not args.no_tune:
        # tensor-core MTTKRP tile choices for this tensor (outside the timed region)
        from tensorly_gb300 import autotune
        tiles = autotune.tune_dense(x, args.rank, sweeps=args.sweeps, refine_sweeps=args.refine)

    def step(times=None):
        return tg.parafac(x, args.rank, init=tg.CPTensor((None, init)), mttkrp_times=times, **kw)

    def barrier():
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        cp, errs = step()
    barrier()
    st = torch.cuda.current_stream()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(dev.index)
    clocks.start()
    barrier()
    ev0.record(st)
    for _ in range(args.steps):
        cp, errs = step()
    ev1.record(st)
    barrier()
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1)
    if args.profile:
        if rank == 0:
            print(json.dumps({"profile": True, "ms_per_step": ms / args.steps,
                              "final_rel_error": errs[-1]}), flush=True)
        return
    ms = job_time_ms(ms, ws, device=dev)
    total_sweeps = args.sweeps * args.steps * ws
    value = total_sweeps / (ms / 1000.0)
    final_err = errs[-1]

    # ---- accuracy against an f64 run from the same initial factors (the f64
    # GPU path matches the NumPy reference to 1e-10 in the parity tests)
    acc = None
    f64_factors = None
    errs64 = None
    if rank == 0:
        x64 = x.double()
        cp64, errs64 = tg.parafac(x64, args.rank, init=tg.CPTensor((None, [f.double() for f in init])),
                                  n_iter_max=args.sweeps, tol=0, return_errors=True,
                                  check_every=args.sweeps)
        del x64
        f64_factors = [f.cpu().numpy() for f in cp64.factors]
        acc = {"final_rel_error": final_err, "f64_final_rel_error": errs64[-1],
               "rel_diff": abs(final_err - errs64[-1]) / errs64[-1],
               "congruence": congruence([f.double().cpu().numpy() for f in cp.factors],
                                        f64_factors)}

    # ---- the plain FP32 GPU path on the same step (the metric's comparator):
    # SIMT f32 MTTKRP, same normal equations, same 50 sweeps from the same init
    fp32 = None
    if rank == 0 and ws == 1 and args.precision == "bf16" and not args.no_extras:
        kw32 = dict(kw, precision="native")

        def step32():
            return tg.parafac(x, args.rank, init=tg.CPTensor((None, init)), **kw32)

        for _ in range(max(3, args.warmup // 2)):
            step32()
        n32 = max(3, args.steps // 4)
        barrier()
        f0 = torch.cuda.Event(enable_timing=True)
        f1 = torch.cuda.Event(enable_timing=True)
        f0.record(st)
        for _ in range(n32):
            cp32, errs32 = step32()
        f1.record(st)
        barrier()
        ms32 = f0.elapsed_time(f1) / n32
        v32 = args.sweeps / (ms32 / 1000.0)
        fp32 = {"value": v32, "unit": UNIT, "steps": n32, "ms_per_step": ms32,
                "kernel": KERNEL["native"],
                "final_rel_error": errs32[-1],
                "rel_diff_vs_f64": abs(errs32[-1] - errs64[-1]) / errs64[-1],
                "congruence_vs_f64": congruence([f.double().cpu().numpy() for f in cp32.factors],
                                                f64_factors),
                "bf16_over_fp32": value / v32}

    # ---- end to end through the public API with host buffers (pinned input,
    # results copied back each step)
    init_host = [torch.from_numpy(f) for f in init_np]

    def step_host():
        cp_h, e_h = tg.parafac(x_host, args.rank, init=tg.CPTensor((None, init_host)), **kw)
        return cp_h, e_h

    step_host()
    barrier()
    e0 = time.perf_counter()
    for _ in range(args.steps):
        cp_h, _ = step_host()
    barrier()
    e_ms = (time.perf_counter() - e0) * 1000.0
    e2e_value = args.sweeps * args.steps * ws / (e_ms / 1000.0)
    h2d = x_np.nbytes + sum(f.nbytes for f in init_np)
    d2h = sum(f.nbytes for f in init_np) + 4 * args.rank

    # ---- the dominant kernel: CUDA events around each mode's MTTKRP launch on
    # its stream, in steps identical to the timed ones except that the sweeps
    # are launched directly instead of replayed as graphs (events inside a
    # graph cannot be timed); the last sweep of each kind per step
    timings = []
    for _ in range(args.steps):
        t = {}
        step(t)
        timings.append(t)
    kind = "bf16" if args.precision == "bf16" else "native"
    samples = [v for t in timings for v in t.get(kind, []) if v > 0]
    k_ms = float(np.mean(samples)) if samples else None
    by_kind = {k: float(np.mean([v for t in timings for v in t.get(k, []) if v > 0]))
               for k in ("native", "bf16", "f32_split", "closing")
               if any(v > 0 for t in timings for v in t.get(k, []))}
    esz = 2 if args.precision == "bf16" else 4
    nel = args.size ** 3
    alg_bytes = nel * esz + 2 * args.size * args.rank * (esz + 4) + args.size * args.rank * 4
    achieved = alg_bytes / (k_ms / 1000.0) / 1e9 if k_ms else None
    peak, peak_kind = measured_peaks()

    # ---- CPU baseline: bounded sample of the NumPy restatement (rank 0, N=1)
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        v, dt = cpu_sample(x_np, init_np, args.rank, args.cpu_sweeps)
        cpu = {"value": v, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
               "sample": f"{args.cpu_sweeps} ALS sweeps ({dt:.1f} s) of the NumPy restatement of "
                         "tensorly parafac on the same tensor and init"}
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "bf16+f32" if args.precision == "bf16" else "f32",
        "data": "synthetic",
        "config": {"workload": f"dense CP-ALS {args.size}^3 f32 rank {args.rank}, "
                               f"{args.sweeps} sweeps per step",
                   "precision": args.precision,
                   "refine_sweeps": args.refine if args.precision == "bf16" else 0,
                   "parallelism": "replicas" if ws > 1 else "single GPU",
                   "l2": "input 512 MiB > L2, no flush",
                   "mttkrp_tiles_autotuned": tiles},
        "accuracy_vs_f64": acc,
        "fp32": fp32,
        "bf16_over_fp32": fp32["bf16_over_fp32"] if fp32 else None,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak if achieved else None, "peak_source": peak_kind,
                     "kernel": KERNEL[args.precision],
                     "kernel_ms": k_ms, "kernel_samples": len(samples),
                     "algorithmic_bytes": alg_bytes,
                     "traffic": (NCU_TRAFFIC[args.precision]
                                 if (args.size, args.rank) == (512, 64) else None),
                     "mttkrp_ms_by_sweep_kind": by_kind},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "clocks": clk,
        "gpu_launches": launches_per_step(3, args.sweeps, args.refine, args.precision,
                                          args.rank) * args.steps,
    }
    if ws == 1 and not args.no_extras:
        # the metric's batched half (4096 uneven tensors) and the 128^4 four-way
        # config, each measured here with its own clocks, accuracy and CPU sample
        del x, x_host
        torch.cuda.empty_cache()
        line["batched"] = measure_batched(args, steps=3, warmup=3)
        torch.cuda.empty_cache()
        line["tucker_cp_128x4"] = measure_tucker(args, steps=3, warmup=3)
        torch.cuda.empty_cache()
        line["learned_warm_start"] = measure_learned(args, steps=3, warmup=3)
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------- batched
BATCH_METRIC = "batched CP-ALS decompositions/s (4096 uneven 3-way f32 tensors, 100 sweeps)"


def _batched_workload(count):
    from tensorly_gb300 import workloads
    batch = workloads.batched_uneven(count=count, seed=0)
    return [b[0] for b in batch], [b[1] for b in batch], [b[2] for b in batch]


def _batched_cpu_sample(xs, ranks, seeds, sweeps, n_sample):
    """Per-tensor NumPy restatement of tensorly parafac (the reference's own
    loop over tensors) on the first `n_sample` tensors: decompositions/s."""
    import oracle
    t0 = time.perf_counter()
    for x, r, s in list(zip(xs, ranks, seeds))[:n_sample]:
        init = oracle.random_cp(x.shape, r, random_state=s, dtype=x.dtype)[1]
        oracle.parafac_sweeps(x, np.ones(r, dtype=x.dtype), init, sweeps)
    dt = time.perf_counter() - t0
    return n_sample / dt, dt


def run_batched(args):
    ws_n, rank, _ = dist_env()
    if rank != 0:
        return
    sweeps = args.sweeps if args.sweeps != 50 else 100
    if args.impl == "reference":
        xs, ranks, seeds = _batched_workload(args.count)
        n = len(xs)
        v, dt = _batched_cpu_sample(xs, ranks, seeds, sweeps, max(1, min(n, 16)))
        line = {"metric": BATCH_METRIC, "value": v, "unit": "decomps/s", "n_gpus": args.gpus,
                "steps": 1, "warmup": 0, "ms_per_step": 1000.0 * dt, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "impl": "reference",
                "config": {"workload": f"{n} uneven 3-way tensors, dims 8-64, rank 4-16, "
                                       f"{sweeps} sweeps", "step": "16 tensors (bounded sample)"},
                "cpu_baseline": {"value": v, "unit": "decomps/s", "cores": os.cpu_count(),
                                 "kind": "port", "sample": f"16 tensors x {sweeps} sweeps"},
                "e2e": {"value": v, "unit": "decomps/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return
    print(json.dumps(measure_batched(args, args.steps, args.warmup)), flush=True)


FP32_FFMA_PEAK_TFLOPS = 152 * 128 * 2 * 2.07e9 / 1e12   # nominal, 2070 MHz


def measure_batched(args, steps, warmup):
    """C4 on the GPU: the batched persistent kernel over all tensors, tensors
    resident; accuracy against per-tensor f64 oracle runs on a sample; e2e
    from host tensors; plain per-tensor parafac on the same GPU; CPU sample."""
    import torch
    import tensorly_gb300 as tg
    from tensorly_gb300 import _lib
    sweeps = args.sweeps if args.sweeps != 50 else 100
    xs, ranks, seeds = _batched_workload(args.count)
    n = len(xs)
    tg.build() if not os.path.exists(_lib.library_path()) else None
    from tensorly_gb300 import autotune
    from tensorly_gb300.decomposition import BatchedProblem
    dev = torch.device("cuda", torch.cuda.current_device())
    # device-resident inputs: one buffer of tensors, one of initial factors
    prob = BatchedProblem([torch.from_numpy(x).to(dev) for x in xs], ranks, random_state=seeds)
    choice, tiles = autotune.tune_batched(prob, sweeps=4, reps=2)   # outside the timed region
    final = prob.final
    st = torch.cuda.current_stream()

    def step():
        prob.run(sweeps)

    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(dev.index)
    clocks.start()
    ev0.record(st)
    for _ in range(steps):
        step()
    ev1.record(st)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1) / steps
    value = n / (ms / 1000.0)
    # accuracy: final errors against per-tensor f64 oracle runs on a sample
    import oracle
    fin = final.cpu().numpy()
    # A sample tensor whose f64 run has not settled (its error still moving by
    # more than 1e-6 relative over the last 10 sweeps) is reported apart, with
    # the NumPy f32 run's own distance from f64 beside the batched kernel's:
    # there f32 and f64 ALS take different paths whatever computes them.
    rel, unsettled = [], []
    sample = sorted(set(np.linspace(0, n - 1, min(n, 16)).astype(int).tolist()))
    for t in sample:
        init = oracle.random_cp(xs[t].shape, ranks[t], random_state=seeds[t])[1]
        x64 = xs[t].astype(np.float64)
        _, f64, e64s = oracle.parafac_sweeps(x64, np.ones(ranks[t]), init, sweeps)
        e64 = np.linalg.norm(x64 - oracle.cp_to_tensor((None, f64))) / np.linalg.norm(x64)
        d = abs(fin[t] - e64) / e64
        if len(e64s) > 10 and abs(e64s[-10] - e64s[-1]) > 1e-6 * e64s[-1]:
            _, f32, _ = oracle.parafac_sweeps(xs[t].astype(np.float32),
                                              np.ones(ranks[t], np.float32),
                                              [i.astype(np.float32) for i in init], sweeps)
            e32 = np.linalg.norm(x64 - oracle.cp_to_tensor(
                (None, [f.astype(np.float64) for f in f32]))) / np.linalg.norm(x64)
            unsettled.append({"tensor": int(t), "shape": list(xs[t].shape),
                              "rank": int(ranks[t]), "batched_rel_diff": float(d),
                              "numpy_f32_rel_diff": float(abs(e32 - e64) / e64)})
        else:
            rel.append(d)
    # end to end through the public API with host tensors
    e0 = time.perf_counter()
    tg.parafac_batched(xs, ranks, n_iter_max=sweeps, random_state=seeds)
    torch.cuda.synchronize()
    e_s = time.perf_counter() - e0
    cpu = None
    if not args.no_cpu_baseline:
        v, dt = _batched_cpu_sample(xs, ranks, seeds, sweeps, 16)
        cpu = {"value": v, "unit": "decomps/s", "cores": os.cpu_count(), "kind": "port",
               "sample": f"16 tensors x {sweeps} sweeps ({dt:.1f} s) of the NumPy restatement"}
    # plain per-tensor ALS on the same GPU: the single-tensor parafac, one call per tensor
    n_pt = min(n, 64)
    for t in range(2):
        tg.parafac(torch.from_numpy(xs[t]).to(dev), ranks[t], n_iter_max=sweeps, init="random",
                   random_state=seeds[t], tol=0)
    torch.cuda.synchronize()
    p0 = time.perf_counter()
    for t in range(n_pt):
        tg.parafac(torch.from_numpy(xs[t]).to(dev), ranks[t], n_iter_max=sweeps, init="random",
                   random_state=seeds[t], tol=0)
    torch.cuda.synchronize()
    per_tensor = n_pt / (time.perf_counter() - p0)
    flops = sum(3 * 2 * x.size * r * sweeps for x, r in zip(xs, ranks))
    line = {"metric": BATCH_METRIC, "value": value, "unit": "decomps/s", "n_gpus": 1,
            "steps": steps, "warmup": warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": f"{n} uneven 3-way tensors, dims 8-64, rank 4-16, "
                                   f"{sweeps} sweeps", "l2": "0.76 GB of tensors > L2",
                       "autotuned_threads": choice, "autotuned_outer_tiles": tiles},
            "accuracy_vs_f64": {"max_rel_diff_final_error": float(max(rel)) if rel else None,
                                "median": float(np.median(rel)) if rel else None,
                                "within_1e-4": f"{sum(r < 1e-4 for r in rel)}/{len(rel)}",
                                "sample": f"{len(sample)} tensors spread over the batch, "
                                          "per-tensor f64 oracle runs from the same init; "
                                          "the settled ones above, the others below",
                                "unsettled": unsettled},
            "mttkrp_tflops": flops / (ms / 1000.0) / 1e12,
            "fp32_pipe_frac_of_nominal": flops / (ms / 1000.0) / 1e12 / FP32_FFMA_PEAK_TFLOPS,
            "per_tensor_gpu": {"value": per_tensor, "unit": "decomps/s",
                               "sample": f"{n_pt} tensors, one parafac call each (f32)"},
            "cpu_baseline": cpu,
            "e2e": {"value": n / e_s, "unit": "decomps/s",
                    "h2d_bytes_per_step": int(sum(x.nbytes for x in xs)),
                    "d2h_bytes_per_step": 0},
            "clocks": clk, "gpu_launches": steps}
    return line


LEARNED_METRIC = ("time-to-fit decompositions/s, 10000 held-out 32^3 rank-8 f32 tensors, "
                  "ALS to a 1e-6 error change from the learned warm start")


def _learned_cpu_sample(seeds, n_sample, tol, max_sweeps):
    """The reference's per-tensor parafac (NumPy restatement) from init='svd'
    to the same stop test, on the first `n_sample` tensors: decompositions/s."""
    import oracle
    from oracle import warm_start_oracle as wo
    X, _, _ = wo.generate(seeds[:n_sample], wo.omega())
    t0 = time.perf_counter()
    for x in X:
        oracle.parafac(x.reshape(32, 32, 32).astype(np.float32), 8, n_iter_max=max_sweeps,
                       init="svd", tol=tol)
    dt = time.perf_counter() - t0
    return n_sample / dt, dt


def run_learned(args):
    ws_n, rank, _ = dist_env()
    if rank != 0:
        return
    line = measure_learned(args, args.steps, args.warmup)
    print(json.dumps(line), flush=True)


def measure_learned(args, steps, warmup):
    """The C5 line (learned warm start on 10,000 held-out tensors), as a dict;
    also a sub-object of the default run."""
    import torch
    import tensorly_gb300 as tg
    from tensorly_gb300 import _lib, learned
    n = 10000
    tol, max_sweeps = 1e-6, 300
    seeds = np.arange(10 ** 6, 10 ** 6 + n)
    workload = (f"{n} held-out tensors 32^3 f32 (seeds 1e6..), rank-8 CP with column "
                f"congruence U(0, 0.9) + 1 % noise; network trained on {args.train_samples} "
                f"generated tensors; ALS to |e_(s-1) - e_s| < {tol} (abs_rec_error), "
                f"at most {max_sweeps} sweeps")
    if args.impl == "reference":
        v, dt = _learned_cpu_sample(seeds, 8, tol, max_sweeps)
        line = {"metric": LEARNED_METRIC, "value": v, "unit": "decomps/s", "n_gpus": args.gpus,
                "steps": 1, "warmup": 0, "ms_per_step": 1000.0 * dt, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "impl": "reference",
                "config": {"workload": workload, "step": "8 tensors (bounded sample), init='svd'"},
                "cpu_baseline": {"value": v, "unit": "decomps/s", "cores": os.cpu_count(),
                                 "kind": "port", "sample": "8 tensors, parafac(init='svd', tol)"},
                "e2e": {"value": v, "unit": "decomps/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        return line
    tg.build() if not os.path.exists(_lib.library_path()) else None
    dev = torch.device("cuda", torch.cuda.current_device())
    gen = learned.Generator(dev)
    net = learned.WarmStartNet(seed=0, device=dev)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    losses = net.train(n_samples=args.train_samples, batch=512, lr=1e-3, lr_final=1e-4,
                       generator=gen)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    X, _, _ = gen(seeds)
    torch.cuda.synchronize()
    st = torch.cuda.current_stream()

    def step():   # the learned path: sketch, inference, SVD fallback, ALS to tol
        F, _, _ = learned.warm_start(net, X, gen.omega)
        return learned._als(X, F, max_sweeps, tol=tol)

    for _ in range(warmup):
        step()
    fallback_any = bool(learned.warm_start(net, X, gen.omega)[1].any().item())
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(dev.index)
    clocks.start()
    ev0.record(st)
    for _ in range(steps):
        prob = step()
    ev1.record(st)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1) / steps
    # inference alone: sketch + network + lift for the whole batch
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(5):
        feats, xnorm = learned.sketch(X, gen.omega)
        net.predict(X, feats, xnorm)
    e1.record(st)
    torch.cuda.synchronize()
    infer_ms = e0.elapsed_time(e1) / 5
    res = learned.evaluate(net, seeds, max_sweeps=max_sweeps, tol=tol, generator=gen)
    # end to end: host tensors in, factors and errors back
    Xh = X.cpu().numpy().reshape(n, 32, 32, 32)
    torch.cuda.synchronize()
    h0 = time.perf_counter()
    Xd = torch.from_numpy(Xh).to(dev).reshape(n, -1)
    pe = learned._als(Xd, learned.warm_start(net, Xd, gen.omega)[0], max_sweeps, tol=tol)
    fb = pe.fbuf.cpu()
    fe = pe.final.cpu()
    e2e_s = time.perf_counter() - h0
    cpu = None
    if not args.no_cpu_baseline:
        v, dt = _learned_cpu_sample(seeds, 8, tol, max_sweeps)
        cpu = {"value": v, "unit": "decomps/s", "cores": os.cpu_count(), "kind": "port",
               "sample": f"8 tensors, parafac(init='svd', tol) of the NumPy restatement ({dt:.1f} s)"}

    def stats(k):
        v = res["sweeps_" + k]
        return {"sweeps_mean": float(v.mean()), "sweeps_median": float(np.median(v)),
                "sweeps_p90": float(np.percentile(v, 90)), "ms": res["ms_" + k],
                "decomps_per_s": n / (res["ms_" + k] / 1000.0),
                "frac_at_cap": float((v >= max_sweeps).mean()),
                "median_final_err": float(np.median(res["err_" + k]))}

    line = {"metric": LEARNED_METRIC, "value": n / (ms / 1000.0), "unit": "decomps/s",
            "n_gpus": 1, "steps": steps, "warmup": warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": workload, "l2": "1.3 GB of tensors > L2",
                       "network": "1536-1024-512-768 MLP + sketch skip, "
                                  f"{net.n_params} parameters"},
            "training": {"samples": args.train_samples, "seconds": train_s,
                         "samples_per_s": args.train_samples / train_s,
                         "loss_first_20": float(losses[:20].mean()),
                         "loss_last_20": float(losses[-20:].mean())},
            "inference": {"ms": infer_ms, "tensors_per_s": n / (infer_ms / 1000.0)},
            "starts": {"svd": stats("svd"), "learned": stats("learned"), "warm": stats("warm"),
                       "warm_kept_network_frac": float(1 - res["used_svd"].mean())},
            "cpu_baseline": cpu,
            "e2e": {"value": n / e2e_s, "unit": "decomps/s",
                    "h2d_bytes_per_step": int(Xh.nbytes),
                    "d2h_bytes_per_step": int(fb.numel() * 4 + fe.numel() * 8)},
            # per step: sketch, 3 GEMMs + skip, loss/scale, lift, the batched ALS
            # kernel (+ gram3, eig and scale when a tensor falls back to the SVD start)
            "clocks": clk, "gpu_launches": (8 + (3 if fallback_any else 0)) * steps}
    return line


TUCKER_METRIC = "Tucker-HOOI iterations/s at 128^4 f32 rank 16^4 (init='svd' included)"


def _tucker_cpu_sample(x, n_iter):
    """The NumPy restatement of tucker (init='random', the SVD init alone takes
    minutes on the host) for `n_iter` iterations: iterations/s."""
    import oracle
    t0 = time.perf_counter()
    oracle.tucker(x, rank=[16] * 4, n_iter_max=n_iter, init="random", tol=0, random_state=0)
    dt = time.perf_counter() - t0
    return n_iter / dt, dt


def run_tucker(args):
    ws_n, rank, _ = dist_env()
    if rank != 0:
        return
    if args.impl == "reference":
        from tensorly_gb300 import workloads
        x_np = workloads.cp_tucker_4way()
        v, dt = _tucker_cpu_sample(x_np, 1)
        line = {"metric": TUCKER_METRIC, "value": v, "unit": "iterations/s", "n_gpus": args.gpus,
                "steps": 1, "warmup": 0, "ms_per_step": 1000.0 * dt, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "impl": "reference",
                "config": {"workload": TUCKER_WORKLOAD,
                           "step": "1 HOOI iteration from init='random' (bounded sample)"},
                "cpu_baseline": {"value": v, "unit": "iterations/s", "cores": os.cpu_count(),
                                 "kind": "port", "sample": "1 HOOI iteration, NumPy restatement"},
                "e2e": {"value": v, "unit": "iterations/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return
    print(json.dumps(measure_tucker(args, args.steps, args.warmup)), flush=True)


TUCKER_WORKLOAD = ("128^4 f32: rank-32 CP + 16^4 Tucker (orthonormal factors) + 1 % noise; "
                   "tucker(rank=[16]*4, n_iter_max=20, tol=0, init='svd')")


def measure_tucker(args, steps, warmup):
    """C3 on the GPU: tucker (HOOI, 20 iterations, SVD init) and 4-way CP
    rank 32 (30 sweeps, bf16 and plain f32) on the 128^4 tensor."""
    import torch
    import tensorly_gb300 as tg
    from tensorly_gb300 import _lib, workloads
    n_iter = 20
    x_np = workloads.cp_tucker_4way()
    workload = TUCKER_WORKLOAD
    tg.build() if not os.path.exists(_lib.library_path()) else None
    dev = torch.device("cuda", torch.cuda.current_device())
    x = torch.from_numpy(x_np).to(dev)
    st = torch.cuda.current_stream()

    def step(it=n_iter):
        return tg.tucker(x, rank=[16] * 4, n_iter_max=it, tol=0, init="svd")

    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    clocks = ClockSampler(dev.index)
    clocks.start()
    ev[0].record(st)
    for _ in range(steps):
        core, factors = step()
    ev[1].record(st)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = ev[0].elapsed_time(ev[1]) / steps
    ev[2].record(st)
    step(1)
    ev[3].record(st)
    torch.cuda.synchronize()
    ms1 = ev[2].elapsed_time(ev[3])
    rec = tg.tenalg.multi_mode_dot(core, factors)
    rel_err = float(((x - rec).double().norm() / x.double().norm()).item())
    # the first (largest) TTM of a chain alone: 1 GiB in, 128 MiB out
    U = factors[1].t().contiguous()
    tg.tenalg.mode_dot(x, U, 1)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(10):
        tg.tenalg.mode_dot(x, U, 1)
    e1.record(st)
    torch.cuda.synchronize()
    ttm_ms = e0.elapsed_time(e1) / 10
    ttm_bytes = x.numel() * 4 + x.numel() // 8 * 4 + 16 * 128 * 4
    peak, peak_kind = measured_peaks()
    # CP at the same shape: rank 32, 30 sweeps, bf16 and native f32
    init = tg.initialize_cp(x, 32, init="random", random_state=0)
    cp = {}
    for prec in ("bf16", "native"):
        tg.parafac(x, 32, n_iter_max=2, tol=0, init=init, precision=prec)
        torch.cuda.synchronize()
        c0 = torch.cuda.Event(enable_timing=True)
        c1 = torch.cuda.Event(enable_timing=True)
        c0.record(st)
        _, errs = tg.parafac(x, 32, n_iter_max=30, tol=0, init=init, precision=prec,
                             return_errors=True)
        c1.record(st)
        torch.cuda.synchronize()
        cp[prec] = {"sweeps_per_s": 30 / (c0.elapsed_time(c1) / 1000.0),
                    "final_rel_err": float(errs[-1])}
    # end to end: host tensor in, core and factors back
    torch.cuda.synchronize()
    h0 = time.perf_counter()
    core_h, factors_h = tg.tucker(x_np, rank=[16] * 4, n_iter_max=n_iter, tol=0, init="svd")
    e2e_s = time.perf_counter() - h0
    cpu = None
    if not args.no_cpu_baseline:
        v, dt = _tucker_cpu_sample(x_np, 1)
        cpu = {"value": v, "unit": "iterations/s", "cores": os.cpu_count(), "kind": "port",
               "sample": f"1 HOOI iteration from init='random' of the NumPy restatement ({dt:.1f} s)"}
    line = {"metric": TUCKER_METRIC, "value": n_iter / (ms / 1000.0), "unit": "iterations/s",
            "n_gpus": 1, "steps": steps, "warmup": warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": workload, "l2": "1 GiB input > L2"},
            "ms_per_iteration_after_init": (ms - ms1) / (n_iter - 1),
            "ms_init_plus_one_iteration": ms1,
            "rel_err": rel_err,
            "roofline": {"bound": "hbm", "kernel": "ttm_stream_kernel (first TTM of a chain)",
                         "achieved": ttm_bytes / (ttm_ms / 1000.0) / 1e9, "peak": peak,
                         "unit": "GB/s", "frac": ttm_bytes / (ttm_ms / 1000.0) / 1e9 / peak,
                         "peak_source": peak_kind, "traffic": None, "ms": ttm_ms},
            "cp_rank32_30_sweeps": cp,
            "cpu_baseline": cpu,
            "e2e": {"value": n_iter / e2e_s, "unit": "iterations/s",
                    "h2d_bytes_per_step": int(x_np.nbytes),
                    "d2h_bytes_per_step": int(np.prod(np.shape(core_h))) * 4 + 4 * 128 * 16 * 4},
            # per call: norm (2), init 4 x (Gram tiles, finish, eig, sqrt), per iteration
            # 4 x (3 TTMs + the 4 SVD kernels) + the core's 4 TTMs + its norm (2)
            "clocks": clk, "gpu_launches": (18 + 34 * n_iter) * steps}
    return line




def nncp_metric(n, r):
    return f"non-negative CP iterations/s at {n}^3 f32 rank {r} (multiplicative updates)"


def _nncp_cpu_sample(x, init, n_iter):
    """The NumPy restatement of non_negative_parafac (multiplicative updates)
    for `n_iter` iterations from `init`: iterations/s."""
    import oracle
    t0 = time.perf_counter()
    oracle.non_negative_parafac(x, init[0].shape[1], n_iter_max=n_iter, init=(None, init), tol=0)
    dt = time.perf_counter() - t0
    return n_iter / dt, dt


def run_nncp(args):
    import torch
    import tensorly_gb300 as tg
    from tensorly_gb300 import _lib, workloads
    ws_n, rank, _ = dist_env()
    if rank != 0:
        return
    n_iter = 50
    x_np, _ = workloads.dense_cp_large(size=args.size, rank=args.rank)
    x_np = np.abs(x_np)
    rs = np.random.RandomState(0)
    init_np = [rs.random_sample((args.size, args.rank)).astype(np.float32) for _ in range(3)]
    workload = (f"|dense CP {args.size}^3 f32| (non-negative), rank {args.rank}, "
                f"{n_iter} iterations from a fixed random non-negative init, tol=0")
    if args.impl == "reference":
        v, dt = _nncp_cpu_sample(x_np, init_np, 2)
        line = {"metric": nncp_metric(args.size, args.rank), "value": v, "unit": "iterations/s", "n_gpus": args.gpus,
                "steps": 1, "warmup": 0, "ms_per_step": 1000.0 * dt / 2, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "impl": "reference",
                "config": {"workload": workload, "step": "2 iterations (bounded sample)"},
                "cpu_baseline": {"value": v, "unit": "iterations/s", "cores": os.cpu_count(),
                                 "kind": "port", "sample": "2 iterations of the NumPy restatement"},
                "e2e": {"value": v, "unit": "iterations/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return
    tg.build() if not os.path.exists(_lib.library_path()) else None
    dev = torch.device("cuda", torch.cuda.current_device())
    x = torch.from_numpy(x_np).to(dev)
    init = tg.CPTensor((None, [torch.from_numpy(f).to(dev) for f in init_np]))
    st = torch.cuda.current_stream()

    def timed(fn, reps):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(reps):
            out = fn()
        e1.record(st)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps, out

    clocks = ClockSampler(dev.index)
    clocks.start()
    ms, _ = timed(lambda: tg.non_negative_parafac(x, args.rank, n_iter_max=n_iter, init=init,
                                                  tol=0), args.steps)
    clk = clocks.stop()
    ms_h, _ = timed(lambda: tg.non_negative_parafac_hals(x, args.rank, n_iter_max=10, init=init,
                                                         tol=0), 1)
    ms_c, _ = timed(lambda: tg.constrained_parafac(x, args.rank, n_iter_max=10, init=init,
                                                   non_negative=True, tol_outer=0), 1)
    _, (cp, errs) = timed(lambda: tg.non_negative_parafac(x, args.rank, n_iter_max=n_iter,
                                                          init=init, tol=1e-30,
                                                          return_errors=True), 1)
    h0 = time.perf_counter()
    tg.non_negative_parafac(x_np, args.rank, n_iter_max=n_iter,
                            init=(None, [f.copy() for f in init_np]), tol=0)
    e2e_s = time.perf_counter() - h0
    cpu = None
    if not args.no_cpu_baseline:
        v, dt = _nncp_cpu_sample(x_np, init_np, 2)
        cpu = {"value": v, "unit": "iterations/s", "cores": os.cpu_count(), "kind": "port",
               "sample": f"2 iterations of the NumPy restatement ({dt:.1f} s)"}
    line = {"metric": nncp_metric(args.size, args.rank), "value": n_iter / (ms / 1000.0), "unit": "iterations/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": {"workload": workload, "l2": "512 MiB input > L2"},
            "final_rel_error_50": float(errs[-1]),
            "hals_iterations_per_s": 10 / (ms_h / 1000.0),
            "constrained_nonneg_iterations_per_s": 10 / (ms_c / 1000.0),
            "cpu_baseline": cpu,
            "e2e": {"value": n_iter / e2e_s, "unit": "iterations/s",
                    "h2d_bytes_per_step": int(x_np.nbytes + sum(f.nbytes for f in init_np)),
                    "d2h_bytes_per_step": int(sum(f.nbytes for f in init_np))},
            # per iteration and mode: accum, MTTKRP split kernel, update, Gram partial + reduce
            "clocks": clk, "gpu_launches": 3 * 5 * n_iter * args.steps}
    print(json.dumps(line), flush=True)


def recon_metric(n, r):
    return f"CP reconstructions/s at {n}^3 f32 rank {r} (cp_to_tensor)"


def _recon_cpu_sample(w, fs, reps):
    """The NumPy restatement of cp_to_tensor (dot with the explicit Khatri-Rao
    matrix, BLAS threads on the host cores) `reps` times: calls/s."""
    import oracle
    t0 = time.perf_counter()
    for _ in range(reps):
        oracle.cp_to_tensor((w, fs))
    dt = time.perf_counter() - t0
    return reps / dt, dt


def run_reconstruct(args):
    """cp_to_tensor of a 512^3 rank-64 f32 model: one fused kernel a call,
    writing the 512 MiB tensor (tensorly/cp_tensor.py:433-485)."""
    import torch
    import tensorly_gb300 as tg
    from tensorly_gb300 import _lib
    ws_n, rank, _ = dist_env()
    if rank != 0:
        return
    n, r = args.size, args.rank
    rs = np.random.RandomState(0)
    fs_np = [rs.randn(n, r).astype(np.float32) for _ in range(3)]
    w_np = (rs.rand(r) + 0.5).astype(np.float32)
    workload = f"cp_to_tensor of a {n}^3 f32 rank-{r} CP model (weights, Gaussian factors)"
    if args.impl == "reference":
        v, dt = _recon_cpu_sample(w_np, fs_np, 2)
        line = {"metric": recon_metric(n, r), "value": v, "unit": "reconstructions/s",
                "n_gpus": args.gpus, "steps": 1, "warmup": 0, "ms_per_step": 1000.0 * dt / 2,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic", "impl": "reference",
                "config": {"workload": workload, "step": "2 calls (bounded sample)"},
                "cpu_baseline": {"value": v, "unit": "reconstructions/s",
                                 "cores": os.cpu_count(), "kind": "port",
                                 "sample": "2 calls of the NumPy restatement"},
                "e2e": {"value": v, "unit": "reconstructions/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return
    tg.build() if not os.path.exists(_lib.library_path()) else None
    dev = torch.device("cuda", torch.cuda.current_device())
    fs = [torch.from_numpy(f).to(dev) for f in fs_np]
    w = torch.from_numpy(w_np).to(dev)
    st = torch.cuda.current_stream()
    for _ in range(max(args.warmup, 3)):
        full = tg.cp_to_tensor((w, fs))
    torch.cuda.synchronize()
    clocks = ClockSampler(dev.index)
    clocks.start()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]
    torch.cuda.synchronize()
    for e0, e1 in evs:
        e0.record(st)
        full = tg.cp_to_tensor((w, fs))
        e1.record(st)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = statistics.mean(e0.elapsed_time(e1) for e0, e1 in evs)
    del full
    # end to end: factors from pinned host memory, the full tensor back into it
    fs_h = [torch.from_numpy(f).pin_memory() for f in fs_np]
    w_h = torch.from_numpy(w_np).pin_memory()
    out_h = torch.empty((n, n, n), dtype=torch.float32).pin_memory()
    for _ in range(2):
        out_h.copy_(tg.cp_to_tensor((w_h.to(dev, non_blocking=True),
                                     [f.to(dev, non_blocking=True) for f in fs_h])),
                    non_blocking=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        out_h.copy_(tg.cp_to_tensor((w_h.to(dev, non_blocking=True),
                                     [f.to(dev, non_blocking=True) for f in fs_h])),
                    non_blocking=True)
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / args.steps
    cpu = None
    if not args.no_cpu_baseline:
        v, dt = _recon_cpu_sample(w_np, fs_np, 2)
        cpu = {"value": v, "unit": "reconstructions/s", "cores": os.cpu_count(), "kind": "port",
               "sample": f"2 calls of the NumPy restatement ({dt:.1f} s)"}
    peak, peak_kind = measured_peaks()
    out_bytes = n ** 3 * 4
    alg_bytes = out_bytes + 3 * n * r * 4 + r * 4
    achieved = alg_bytes / (ms / 1000.0) / 1e9
    flops = 2.0 * n ** 3 * r
    sm_mhz = clk.get("sm_mhz") or 2070.0
    fp32_peak = 152 * 128 * 2 * sm_mhz * 1e6 / 1e12          # FFMA pipe, TFLOP/s at that clock
    line = {"metric": recon_metric(n, r), "value": 1000.0 / ms, "unit": "reconstructions/s",
            "n_gpus": 1, "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": {"workload": workload, "l2": "512 MiB output > L2"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": None,
                         "peak_kind": peak_kind, "alg_bytes_per_launch": alg_bytes},
            "fp32_tflops": flops / (ms / 1000.0) / 1e12, "fp32_pipe_peak_tflops": fp32_peak,
            "cpu_baseline": cpu,
            "e2e": {"value": 1.0 / e2e_s, "unit": "reconstructions/s",
                    "h2d_bytes_per_step": int(sum(f.nbytes for f in fs_np) + w_np.nbytes),
                    "d2h_bytes_per_step": int(out_bytes)},
            "clocks": clk, "gpu_launches": args.steps}
    print(json.dumps(line), flush=True)


def rand_metric(n, r, ns):
    return f"randomised CP iterations/s at {n}^3 f32 rank {r} ({ns} samples a mode)"


def run_randomised(args):
    """randomised_parafac on the 512^3 rank-64 dense CP tensor: per iteration
    three sampled mode updates and the reconstruction error
    (tensorly/decomposition/_cp.py:633-762)."""
    import torch
    import tensorly_gb300 as tg
    from tensorly_gb300 import _lib, workloads
    ws_n, rank, _ = dist_env()
    if rank != 0:
        return
    n, r, ns, n_iter = args.size, args.rank, 4096, 20
    x_np, _ = workloads.dense_cp_large(size=n, rank=r)
    workload = (f"randomised_parafac of the dense CP {n}^3 f32 tensor, rank {r}, {ns} samples a "
                f"mode, {n_iter} iterations, init='random' (seed 0), tol=0, max_stagnation=20")

    def cpu_sample(iters):
        import oracle
        t0 = time.perf_counter()
        oracle.randomised_parafac(x_np, r, ns, n_iter_max=iters, tol=0, random_state=0)
        dt = time.perf_counter() - t0
        return iters / dt, dt

    if args.impl == "reference":
        v, dt = cpu_sample(2)
        line = {"metric": rand_metric(n, r, ns), "value": v, "unit": "iterations/s",
                "n_gpus": args.gpus, "steps": 1, "warmup": 0, "ms_per_step": 1000.0 * dt / 2,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic", "impl": "reference",
                "config": {"workload": workload, "step": "2 iterations (bounded sample)"},
                "cpu_baseline": {"value": v, "unit": "iterations/s", "cores": os.cpu_count(),
                                 "kind": "port", "sample": "2 iterations of the NumPy restatement"},
                "e2e": {"value": v, "unit": "iterations/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return
    tg.build() if not os.path.exists(_lib.library_path()) else None
    dev = torch.device("cuda", torch.cuda.current_device())
    x = torch.from_numpy(x_np).to(dev)
    st = torch.cuda.current_stream()
    run = lambda: tg.randomised_parafac(x, r, ns, n_iter_max=n_iter, tol=0, random_state=0,
                                        return_errors=True)
    for _ in range(max(args.warmup, 3)):
        run()
    torch.cuda.synchronize()
    clocks = ClockSampler(dev.index)
    clocks.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(args.steps):
        _, errs = run()
    e1.record(st)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1) / args.steps
    h0 = time.perf_counter()
    for _ in range(args.steps):
        tg.randomised_parafac(x_np, r, ns, n_iter_max=n_iter, tol=0, random_state=0)
    e2e_s = (time.perf_counter() - h0) / args.steps
    cpu = None
    if not args.no_cpu_baseline:
        v, dt = cpu_sample(2)
        cpu = {"value": v, "unit": "iterations/s", "cores": os.cpu_count(), "kind": "port",
               "sample": f"2 iterations of the NumPy restatement ({dt:.1f} s)"}
    line = {"metric": rand_metric(n, r, ns), "value": n_iter / (ms / 1000.0),
            "unit": "iterations/s", "n_gpus": 1, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": workload, "l2": "512 MiB input > L2"},
            "final_rel_error": float(errs[-1]), "cpu_baseline": cpu,
            "e2e": {"value": n_iter / e2e_s, "unit": "iterations/s",
                    "h2d_bytes_per_step": int(x_np.nbytes),
                    "d2h_bytes_per_step": int(3 * n * r * 4)},
            # per iteration: 3 x (gather KR, gather unfolding, Gram, products, factorise, solve)
            # + transpose + residual + final reduction
            "clocks": clk, "gpu_launches": args.steps * n_iter * (3 * 6 + 3)}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.workload == "batched":
        run_batched(args)
    elif args.workload == "learned":
        run_learned(args)
    elif args.workload == "tucker":
        run_tucker(args)
    elif args.workload == "nncp":
        run_nncp(args)
    elif args.workload == "reconstruct":
        run_reconstruct(args)
    elif args.workload == "randomised":
        run_randomised(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
