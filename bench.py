"""Benchmark of the bandwidth-bound hot path on one GB300 (or N replicas).

Workload (one "step"): the plain bandwidth configuration of the reference's
hot path -
    mtv  y = A x,  A 16384 x 16384 row-major, float32   (amt::mtv)
    dot  a . b,    two float32 vectors of length 2^28   (amt::dot_prod)
    mtv  the same in float64
    dot  the same in float64
entries uniform[-1, 1) from seed 1.  Every input is far larger than the
129 MB L2, so no L2 flush is needed between iterations.

Reported metric: GB/s of algorithmic traffic (A once plus the vectors,
i.e. (M*N + M + N) * s for mtv and 2 n s for dot, summed over the four
calls) per second, whole job.

  value     device-resident inputs, kernels timed with CUDA events on the
            launching stream;
  e2e       the same step through the public host-buffer C ABI
            (gbblas_?mtv_host / gbblas_?dot_host) from pinned host memory,
            host<->device copies inside the timed region;
  roofline  the dominant kernel's achieved GB/s against the measured HBM
            copy bandwidth in MEASURED_PEAKS.json;
  cpu_baseline  the CPU oracle (a restatement of the reference's OpenMP
            code, oracle/oracle.c) on the host cores, on a bounded sample.

`--impl reference` times the reference's CPU implementation of the same
workload instead (the compiled reference where it exists, otherwise the
oracle port) and prints the same line with "impl": "reference".

Other workloads (`--workload`, one JSON line per result): precision (the
8192^3 GEMM paths and their errors against FP64), f64 (8192^3 double-precision
GEMM on the FP64 pipes and as the tensor-core Ozaki scheme), batching, serving,
stream_ops, sweep (the reference's size sweeps in its metric formats) and mtm
(the plain 1024^3 single-precision mtm against the FMA-pipe peak).

Multi-GPU: the path does not shard; `--gpus N` under torchrun runs N
independent replicas (weak scaling), max time over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "openmp-blas_gb300"))

M = N = 16384
NDOT = 1 << 28
SEED = 1
FP64_NOMINAL_TFLOPS = 1.25  # GB300 FP64 (vector and tensor), NVIDIA datasheet figure

METRIC = "GEMV GB/s"
UNIT = "GB/s"
WORKLOAD = ("bandwidth path: mtv y=A.x (A 16384x16384 row-major) + dot (2^28), float32 and float64, "
            "U[-1,1) seed 1")


def op_bytes():
    """Algorithmic bytes of each call in one step."""
    return {
        "mtv_f32": (M * N + M + N) * 4,
        "dot_f32": 2 * NDOT * 4,
        "mtv_f64": (M * N + M + N) * 8,
        "dot_f64": 2 * NDOT * 8,
    }


def step_bytes() -> int:
    return sum(op_bytes().values())


def config(extra=None):
    c = {"workload": WORKLOAD, "M": M, "N": N, "dot_n": NDOT, "layout": "row-major",
         "dtypes": ["f32", "f64"], "bytes_per_step": step_bytes(),
         "inputs": "std::mt19937_64(1) draws A, x, a, b in order; U[-1,1) = (draw >> 11) 2^-52 - 1 "
                   "(double), (draw >> 40) 2^-23 - 1 (float)",
         "l2": "inputs larger than L2 (no flush needed)"}
    if extra:
        c.update(extra)
    return c


# ------------------------------------------------------------------ distributed

def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def dist_init(backend: str):
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group(backend=backend)
    return ws, rank, local


def reduce_max(value: float, device=None) -> float:
    """Max of `value` over ranks (identity without a process group)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return value
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier():
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.barrier()


def aggregate(per_rank_units: float, world: int, max_seconds: float) -> float:
    """Whole-job throughput of `world` replicas that each processed
    `per_rank_units` in at most `max_seconds`."""
    return per_rank_units * world / max_seconds


# ------------------------------------------------------------------ clocks

class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons in the background."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int, period_ms: int = 20):
        self.gpu = gpu_index
        self.period = period_ms
        self.proc = None
        self.samples = []  # (host time, line)
        self.reader = None
        self.window = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", str(self.period)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True, bufsize=1)
        except (OSError, FileNotFoundError):
            self.proc = None
        if self.proc is not None:
            def pump():
                for line in self.proc.stdout:
                    self.samples.append((time.time(), line))
            self.reader = threading.Thread(target=pump, daemon=True)
            self.reader.start()
        time.sleep(0.3)
        return self

    def mark(self, t0: float, t1: float) -> None:
        """Host-clock bounds of the timed region."""
        self.window = (t0, t1)

    def __exit__(self, *exc):
        time.sleep(2 * self.period / 1e3)
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.reader is not None:
            self.reader.join(timeout=2)

    def summary(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        for t, line in self.samples:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((t, float(parts[1]), float(parts[2]), parts[5:9]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        inside = rows
        if self.window:
            t0, t1 = self.window
            inside = [r for r in rows if t0 <= r[0] <= t1 + self.period / 1e3]
            if not inside:  # region shorter than one period: the sample right after it
                after = [r for r in rows if r[0] >= t0]
                inside = after[:1] or rows[-1:]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in inside for i, v in enumerate(r[3]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(r[1] for r in inside), "sm_max_mhz": max(r[2] for r in rows),
                "reasons": reasons, "samples": len(inside), "period_ms": self.period}


# ------------------------------------------------------------------ CPU side

def cpu_step_oracle(bufs):
    """One step on the host cores through the oracle's restatement of the
    reference's OpenMP code (oracle/oracle.c; its entry points work on the
    caller's buffers, where the compiled reference's test wrappers copy each
    operand into a tensor first).  Returns the two dot values."""
    from oracle import oracle as O
    O.mtv_raw(1, M, N, bufs["A32"], bufs["x32"], bufs["y32"])
    r32 = O.dot(bufs["a32"], bufs["b32"])
    O.mtv_raw(1, M, N, bufs["A64"], bufs["x64"], bufs["y64"])
    r64 = O.dot(bufs["a64"], bufs["b64"])
    return r32, r64


def oracle_errors(host, y32, y64, results):
    """Every output of the GPU step against the oracle's restatement of the
    reference on the same inputs: max |gpu - oracle| / (2 K eps (|A||x|)_i)
    for mtv (the parity tolerance is 1) and the same ratio for the dots,
    plus the dots against the exact sum (long double)."""
    import numpy as np
    from oracle import oracle as O
    O.set_threads(os.cpu_count() or 1)
    out = {}
    for tag, y in (("32", y32), ("64", y64)):
        A, x = host["A" + tag].numpy(), host["x" + tag].numpy()
        dt = A.dtype
        eps = float(np.finfo(dt).eps)
        ref = np.zeros(M, dt)
        O.mtv_raw(1, M, N, A, x, ref)
        absA = np.abs(A)
        absx = np.abs(x)
        scale = np.zeros(M, dt)
        O.mtv_raw(1, M, N, absA, absx, scale)
        del absA
        tol = 2 * N * eps * scale.astype(np.float64) + np.finfo(np.float64).tiny
        err = np.abs(np.asarray(y, np.float64) - ref.astype(np.float64))
        out["mtv_f" + tag] = {"max_err_over_tol": float((err / tol).max()), "max_abs_err": float(err.max()),
                              "oracle_sum": float(ref.astype(np.float64).sum())}
        a, b = host["a" + tag].numpy(), host["b" + tag].numpy()
        rd = float(O.dot(a, b))
        exact, absdot = O.dot_exact(a, b)
        got = results["dot_f" + tag]
        out["dot_f" + tag] = {"oracle": rd, "exact": exact,
                              "err_over_tol": abs(got - rd) / (2 * NDOT * eps * absdot),
                              "rel_err_vs_exact": abs(got - exact) / abs(exact)}
    out["tolerance"] = "|gpu - oracle| <= 2 K eps (|A||x|) elementwise (K = reduction length); ratio <= 1 passes"
    return out


def link_rate(buf, dev) -> float:
    """Host-to-device copy rate (GB/s) of a pinned host tensor, best of 5."""
    import torch
    d = torch.empty_like(buf, device=dev)
    best = 0.0
    for _ in range(5):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        d.copy_(buf, non_blocking=True)
        torch.cuda.synchronize()
        best = max(best, buf.numel() * buf.element_size() / (time.perf_counter() - t0) / 1e9)
    del d
    return best


def cpu_buffers_from(host):
    import numpy as np
    return {k: (v.numpy() if hasattr(v, "numpy") else v) for k, v in host.items()} | {
        "y32": np.zeros(M, np.float32), "y64": np.zeros(M, np.float64)}


INPUT_KEYS = ("A", "x", "a", "b")


def input_counts():
    """Segment lengths of the bandwidth configuration's seeded inputs, drawn
    in this order from one std::mt19937_64(SEED): A (M*N), x (N), a, b (NDOT)."""
    return [M * N, N, NDOT, NDOT]


def make_cpu_inputs():
    """The seeded inputs as numpy arrays, drawn by the oracle's own
    restatement of the generator (reference arm: no GPU library loaded)."""
    from oracle import oracle as O
    f32, f64 = O.seeded_fill(SEED, input_counts())
    out = {}
    for k, a, b in zip(INPUT_KEYS, f32, f64):
        out[k + "32"], out[k + "64"] = a, b
    return out


def step_results(y32, y64, r32, r64):
    """The numbers both arms print for one step's outputs: dot values and
    checksums of y (sum, sum of squares, first and last entry, in float64),
    so results on the shared seeded inputs can be compared across arms."""
    import numpy as np

    def summary(y):
        y = np.asarray(y, np.float64)
        return {"sum": float(y.sum()), "sumsq": float((y * y).sum()), "first": float(y[0]), "last": float(y[-1])}
    return {"mtv_f32": summary(y32), "mtv_f64": summary(y64), "dot_f32": float(r32), "dot_f64": float(r64)}


def time_cpu(bufs, min_seconds=10.0, max_steps=50):
    """Oracle on all host cores: 1 warm-up step, then steps until min_seconds."""
    from oracle import oracle as O
    O.set_threads(os.cpu_count() or 1)
    cpu_step_oracle(bufs)
    times = []
    t_start = time.perf_counter()
    while len(times) < max_steps and (time.perf_counter() - t_start) < min_seconds:
        t0 = time.perf_counter()
        cpu_step_oracle(bufs)
        times.append(time.perf_counter() - t0)
    return times


def cpu_kind():
    """The bandwidth step on the CPU always runs the oracle port."""
    return "port"


# ------------------------------------------------------------------ GPU arm

def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def fma_peak_tflops(clocks=None):
    """Nominal FP32 FMA-pipe peak of this GPU: SMs x 128 lanes x 2 flop x the
    maximum SM clock (from the clock samples, else the device property)."""
    import torch
    props = torch.cuda.get_device_properties(0)
    mhz = (clocks or {}).get("sm_max_mhz") or 2070.0
    return props.multi_processor_count * 128 * 2 * mhz * 1e6 / 1e12


# (path, accuracy, tensor products per algorithmic flop); "auto" is the
# library's FP32-accurate default (GBBLAS_ACCURACY_AUTO: at these sizes the
# split-FP16 GEMM with its guard)
PRECISION_PATHS = (("auto", 3, 3), ("bf16x6", 4, 6), ("fp16x3", 8, 3), ("bf16x3", 1, 3), ("fp8", 2, None),
                   ("fp32", 0, None))


def precision_inputs(n, set_name):
    """The precision configuration's float32 operands on the host: one
    std::mt19937_64(2) draws A then B, as U[-1,1) ("uniform") or as the
    wide-range set s*m*2^e, m in [1, 2), e in [-10, 10] ("wide")."""
    import numpy as np

    import gbblas
    A, B = np.empty((n, n), np.float32), np.empty((n, n), np.float32)
    kind = gbblas.FILL_UNIFORM if set_name == "uniform" else gbblas.FILL_WIDE
    gbblas.seeded_fill(2, [A.reshape(-1), B.reshape(-1)], None, kind=kind)
    return A, B


def precision_report(n=8192, sets=("uniform", "wide"), paths=None, warmup=1, iters=3, sample=1024,
                     full_matrix=True):
    """C = A*B, M = N = K = n from float32 operands (the precision
    configuration), per input set and arithmetic path: split-BF16 with six
    or three tcgen05 products, split-FP16 with three, FP8-E4M3 with per-128
    K-block scales and plain FP32 on the FMA pipes.  TFLOP/s of 2*M*N*K
    algorithmic flops (CUDA events over `iters` calls after `warmup`), the
    pipe's roofline fraction, max / mean relative error against long-double
    dots on `sample` sampled entries (outside the timed region), and with
    `full_matrix` the same over all M*N entries against the product on the
    FP64 pipes.  Returns {set: {path: record}}."""
    import numpy as np
    import torch

    import gbblas
    from oracle import oracle as O
    paths = paths or [p for p, _, _ in PRECISION_PATHS]
    flops = 2.0 * n ** 3
    rng = np.random.default_rng(2)
    rows, cols = rng.integers(0, n, sample), rng.integers(0, n, sample)
    pp = os.path.join(ROOT, "MEASURED_PEAKS.json")
    peaks = json.load(open(pp)) if os.path.exists(pp) else {}
    sp = torch.cuda.current_stream().cuda_stream or None
    report = {}
    for set_name in sets:
        An, Bn = precision_inputs(n, set_name)
        exact, absx = O.gemm_sample_exact(n, An, n, 1, Bn, n, 1, rows, cols)
        A, B = torch.from_numpy(An).cuda(), torch.from_numpy(Bn).cuda()
        C64 = absAB = None
        if full_matrix:
            # C64 = A B on the FP64 pipes (the FMA kernel, independent of the
            # tensor-core paths checked); |A||B| in FP32 for the normwise scale
            A64, B64 = A.double(), B.double()
            C64 = torch.zeros(n, n, device="cuda", dtype=torch.float64)
            gbblas.call("gbblas_dgemm_ex", n, n, n, A64.data_ptr(), n, 1, B64.data_ptr(), n, 1, C64.data_ptr(), n,
                        1, gbblas.ACCURACY_FP64, sp)
            del A64, B64
            Aa, Ba = A.abs(), B.abs()
            absAB = torch.zeros(n, n, device="cuda")
            gbblas.call("gbblas_sgemm", n, n, n, Aa.data_ptr(), n, 1, Ba.data_ptr(), n, 1, absAB.data_ptr(), n, 1,
                        gbblas.ACCURACY_FP32, sp)
            del Aa, Ba
            gbblas.call("gbblas_check_stream", sp)
        report[set_name] = {}
        C = torch.zeros(n, n, device="cuda")
        for path, acc, products in PRECISION_PATHS:
            if path not in paths:
                continue

            def call():
                gbblas.call("gbblas_sgemm", n, n, n, A.data_ptr(), n, 1, B.data_ptr(), n, 1, C.data_ptr(), n, 1,
                            acc, sp)
            for _ in range(warmup):
                call()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            with ClockSampler(0) as clk:
                t0 = time.time()
                e0.record()
                for _ in range(iters):
                    call()
                e1.record()
                torch.cuda.synchronize()
                clk.mark(t0, time.time())
            gbblas.call("gbblas_check_stream", sp)
            ms = e0.elapsed_time(e1) / iters
            C.zero_()  # one clean product for the error checks
            call()
            got = C.cpu().numpy()[rows, cols].astype(np.float64)
            rel = np.abs(got - exact) / np.maximum(np.abs(exact), 1e-300)
            tf = flops / (ms / 1e3) / 1e12
            rec = {"value": round(tf, 2), "unit": "TFLOP/s", "ms": round(ms, 3),
                   "max_rel_err": float(rel.max()), "mean_rel_err": float(rel.mean()),
                   "max_normwise_err": float((np.abs(got - exact) / absx).max()), "clocks": clk.summary()}
            if full_matrix:
                diff = (C.double() - C64).abs_()
                mag = C64.abs().clamp_min(1e-300)
                rec["full_matrix_vs_fp64"] = {"max_rel_err": float((diff / mag).max()),
                                              "mean_rel_err": float((diff / mag).mean()),
                                              "max_normwise_err": float((diff / absAB.double().clamp_min(1e-300)).max())}
                del diff, mag
            if products and peaks.get("bf16_tflops"):
                rec["roofline"] = {"bound": "tensor", "achieved": round(products * tf, 1),
                                   "peak": peaks["bf16_tflops"], "unit": "TFLOP/s",
                                   "frac": round(products * tf / peaks["bf16_tflops"], 4),
                                   "peak_source": f"{products} BF16/FP16 products per algorithmic flop against "
                                                  "MEASURED_PEAKS.json bf16_tflops (measured, burst)"}
            elif path == "fp8" and peaks.get("bf16_tflops"):
                rec["roofline"] = {"bound": "tensor", "achieved": round(tf, 1), "peak": 2 * peaks["bf16_tflops"],
                                   "unit": "TFLOP/s", "frac": round(tf / (2 * peaks["bf16_tflops"]), 4),
                                   "peak_source": "2 x MEASURED_PEAKS.json bf16_tflops (measured BF16 burst times "
                                                  "the nominal FP8/BF16 ratio; no FP8 peak is measured)"}
            elif path == "fp32":
                fp = fma_peak_tflops(rec["clocks"])
                rec["roofline"] = {"bound": "fma", "achieved": round(tf, 2), "peak": round(fp, 1),
                                   "unit": "TFLOP/s", "frac": round(tf / fp, 4),
                                   "peak_source": "SMs x 128 FP32 FMA lanes x 2 flop x max SM clock (nominal)"}
            report[set_name][path] = rec
        del A, B, C, C64, absAB
        torch.cuda.empty_cache()
    return report


def precision_keys(report, n):
    """The default line's two precision keys from a precision report: the
    FP32-accurate paths against plain FP32 per set, and FP8 per set."""
    cfg = (f"C = A*B, M = N = K = {n} from float32; std::mt19937_64(2) draws A then B: U[-1,1) "
           "(uniform) or s*m*2^e, m in [1,2), e in [-10,10] (wide); 2*M*N*K algorithmic flops; errors vs "
           "long-double dots on sampled entries and vs the full product on the FP64 pipes")
    acc = {"config": cfg}
    fp8 = {"config": cfg}
    for set_name, rec in report.items():
        acc[set_name] = {p: r for p, r in rec.items() if p != "fp8"}
        if "fp32" in rec:
            for p in ("auto", "bf16x6", "fp16x3", "bf16x3"):
                if p in rec:
                    acc[set_name][f"{p}_over_fp32"] = round(rec[p]["value"] / rec["fp32"]["value"], 2)
                    acc[set_name][f"{p}_max_rel_err_below_fp32"] = rec[p]["max_rel_err"] <= rec["fp32"]["max_rel_err"]
        if "fp8" in rec:
            fp8[set_name] = rec["fp8"]
    return acc, fp8


def dgemm_headline(dev, sp):
    """Double-precision GEMM beside the bandwidth line (outside the timed
    region): C = A*B at M = N = K = 8192 from float64 U[-1,1) (seed 4), the
    library default (AUTO: exact BF16 digit products on the tensor cores,
    guarded to the FP64 pipes' error bound) against the FP64 pipes; CUDA
    events over 3 calls (1 on the pipes) after 1 warm-up; max relative error
    against long-double dots on 256 sampled entries.  The two-input-set
    report with the unguarded digit paths is `--workload f64`."""
    import numpy as np
    import torch

    import gbblas
    from oracle import oracle as O
    n = 8192
    g = torch.Generator(device=dev).manual_seed(4)
    A = torch.rand(n, n, generator=g, device=dev, dtype=torch.float64) * 2 - 1
    B = torch.rand(n, n, generator=g, device=dev, dtype=torch.float64) * 2 - 1
    C = torch.zeros(n, n, device=dev, dtype=torch.float64)
    rng = np.random.default_rng(4)
    rows, cols = rng.integers(0, n, 256), rng.integers(0, n, 256)
    exact, _ = O.gemm_sample_exact(n, A.cpu().numpy(), n, 1, B.cpu().numpy(), n, 1, rows, cols)
    out = {"config": "M=N=K=8192 float64 U[-1,1) seed 4, 2*M*N*K flops", "unit": "TFLOP/s"}
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for path, acc, reps in (("auto_tensor_digits", 3, 3), ("fp64_pipes", 5, 1)):
        def call():
            gbblas.call("gbblas_dgemm_ex", n, n, n, A.data_ptr(), n, 1, B.data_ptr(), n, 1, C.data_ptr(), n, 1, acc,
                        sp)
        call()
        torch.cuda.synchronize()
        e0.record()
        for _ in range(reps):
            call()
        e1.record()
        torch.cuda.synchronize()
        gbblas.call("gbblas_check_stream", sp)
        ms = e0.elapsed_time(e1) / reps
        C.zero_()
        call()
        got = C.cpu().numpy()[rows, cols]
        rel = np.abs(got - exact) / np.maximum(np.abs(exact), 1e-300)
        out[path] = {"value": round(2.0 * n ** 3 / (ms / 1e3) / 1e12, 3), "ms": round(ms, 3),
                     "max_rel_err": float(rel.max()), "mean_rel_err": float(rel.mean())}
    out["digits_over_pipes"] = round(out["auto_tensor_digits"]["value"] / out["fp64_pipes"]["value"], 1)
    del A, B, C
    torch.cuda.empty_cache()
    return out


def default_extras(args, dev, sp):
    """The rest of the headline metric, measured after the bandwidth step
    (outside its timed region) so that one default run carries all of it:
    the precision configuration (FP32-accurate paths and FP8 on both input
    sets), double-precision GEMM, the plain 1024^3 mtm, the batching
    configuration and the served latencies.  Each entry carries its own
    roofline and clock record; one that fails records its error and the
    others still run."""
    import copy

    import torch
    out = {}

    def guarded(key, fn):
        t0 = time.perf_counter()
        try:
            out.update(fn()) if key is None else out.__setitem__(key, fn())
        except Exception as e:  # keep the rest of the line
            out[key or "precision"] = {"error": f"{type(e).__name__}: {e}"}
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
        return time.perf_counter() - t0

    def precision():
        rep = precision_report(8192, iters=3, sample=1024)
        acc, fp8 = precision_keys(rep, 8192)
        return {"fp32_accurate_gemm": acc, "fp8": fp8}

    secs = {}
    secs["precision"] = guarded(None, precision)
    secs["fp64_gemm"] = guarded("fp64_gemm", lambda: dgemm_headline(dev, sp))
    a = copy.copy(args)
    a.warmup = max(3, args.warmup)
    secs["mtm_1024"] = guarded("mtm_1024", lambda: mtm_report(a))
    b = copy.copy(args)
    b.steps, b.warmup, b.pool_gb, b.batch_accuracy = 5, 2, 48.0, "bf16x3"
    secs["batching"] = guarded("batching", lambda: batching_report(b))
    c = copy.copy(args)
    c.rates, c.min_requests, c.max_requests, c.lone_requests, c.seconds = [5000, 10000, 20000], 4000, 4000, 4000, 0.0
    c.pool_gb, c.f64_accuracy, c.slice_us = 16.0, "auto", 0
    secs["served"] = guarded("served", lambda: serving_report(c))
    out["extras_seconds"] = {k: round(v, 1) for k, v in secs.items()}
    return out


def run_gpu(args):
    import numpy as np
    import torch

    backend = "nccl"
    ws, rank, local = dist_init(backend)
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    import gbblas
    gbblas.lib()
    gbblas.call("gbblas_init")

    # The seeded inputs, drawn on the host into pinned buffers (the same values
    # the reference arm draws; every rank the same), then uploaded once.  The
    # pinned buffers are also the e2e step's host inputs.
    host = {}
    for k, n in zip(INPUT_KEYS, input_counts()):
        host[k + "32"] = torch.empty(n, dtype=torch.float32, pin_memory=True)
        host[k + "64"] = torch.empty(n, dtype=torch.float64, pin_memory=True)
    gbblas.seeded_fill(SEED, [host[k + "32"] for k in INPUT_KEYS], [host[k + "64"] for k in INPUT_KEYS])
    t = {k: v.to(dev) for k, v in host.items()}
    for tag, dt in (("32", torch.float32), ("64", torch.float64)):
        t["y" + tag] = torch.zeros(M, dtype=dt, device=dev)
        t["r" + tag] = torch.zeros(1, dtype=dt, device=dev)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream(dev)
    sp = stream.cuda_stream or None
    L = gbblas.lib()

    ops = [
        ("mtv_f32", lambda: gbblas.call("gbblas_smtv", 1, M, N, t["A32"].data_ptr(), t["x32"].data_ptr(),
                                        t["y32"].data_ptr(), sp)),
        ("dot_f32", lambda: gbblas.call("gbblas_sdot", NDOT, t["a32"].data_ptr(), t["b32"].data_ptr(),
                                        t["r32"].data_ptr(), sp)),
        ("mtv_f64", lambda: gbblas.call("gbblas_dmtv", 1, M, N, t["A64"].data_ptr(), t["x64"].data_ptr(),
                                        t["y64"].data_ptr(), sp)),
        ("dot_f64", lambda: gbblas.call("gbblas_ddot", NDOT, t["a64"].data_ptr(), t["b64"].data_ptr(),
                                        t["r64"].data_ptr(), sp)),
    ]

    def step():
        for _, f in ops:
            f()

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    # ---- timed region: K steps, per-op events on the launching stream
    nops = len(ops)
    ev = [[(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(nops)]
          for _ in range(args.steps)]
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    launches0 = gbblas.kernel_launches()
    with ClockSampler(local) as clk:
        barrier()
        torch.cuda.synchronize()
        t_host0 = time.time()
        start.record(stream)
        for s in range(args.steps):
            for i, (_, f) in enumerate(ops):
                ev[s][i][0].record(stream)
                f()
                ev[s][i][1].record(stream)
        end.record(stream)
        torch.cuda.synchronize()
        clk.mark(t_host0, time.time())
        barrier()
    launches = gbblas.kernel_launches() - launches0
    clocks = clk.summary()
    total_s = start.elapsed_time(end) / 1e3
    total_s = reduce_max(total_s, dev)
    per_op_ms = {name: statistics.mean(ev[s][i][0].elapsed_time(ev[s][i][1]) for s in range(args.steps))
                 for i, (name, _) in enumerate(ops)}

    sb = step_bytes()
    value = aggregate(sb * args.steps, ws, total_s) / 1e9
    ms_per_step = total_s * 1e3 / args.steps

    # ---- roofline of the dominant kernel
    peak, peak_kind = measured_peaks()
    dom = max(per_op_ms, key=per_op_ms.get)
    ob = op_bytes()
    achieved = ob[dom] / (per_op_ms[dom] / 1e3) / 1e9
    kernels = {name: {"ms": round(per_op_ms[name], 4), "GB_s": round(ob[name] / (per_op_ms[name] / 1e3) / 1e9, 1),
                      "frac_of_hbm": round(ob[name] / (per_op_ms[name] / 1e3) / 1e9 / peak, 4)} for name in per_op_ms}
    # FP64 kernels do one DFMA per 8 (mtv) or 16 (dot) bytes; GB300's FP64 rate (1.25 TFLOP/s
    # nominal, not in MEASURED_PEAKS.json) caps mtv_f64 below HBM speed.
    fp64_flops = {"mtv_f64": 2 * M * N, "dot_f64": 2 * NDOT}
    for name, fl in fp64_flops.items():
        tf = fl / (per_op_ms[name] / 1e3) / 1e12
        kernels[name]["fp64_TFLOPs"] = round(tf, 3)
        kernels[name]["frac_of_fp64_nominal"] = round(tf / FP64_NOMINAL_TFLOPS, 4)
    kernels["mtv_f64"]["bound"] = "fp64"
    traffic = None
    tfile = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tfile):
        traffic = json.load(open(tfile)).get(dom)

    # ---- results on the shared seeded inputs (the reference arm prints the same keys)
    y32, y64 = t["y32"].cpu().numpy(), t["y64"].cpu().numpy()
    results = step_results(y32, y64, t["r32"].item(), t["r64"].item())

    if args.small:
        if rank == 0:
            print(json.dumps({"small_case": True, "per_op_ms": per_op_ms, "gpu_launches": int(launches)}))
        return

    # ---- e2e: the same step through the host-buffer C ABI from pinned memory
    hy32 = torch.zeros(M, dtype=torch.float32, pin_memory=True)
    hy64 = torch.zeros(M, dtype=torch.float64, pin_memory=True)
    hr32 = np.zeros(1, np.float32)
    hr64 = np.zeros(1, np.float64)
    p = {k: v.data_ptr() for k, v in host.items()}

    def e2e_step():
        gbblas.call("gbblas_smtv_host", 1, M, N, p["A32"], p["x32"], hy32.data_ptr())
        gbblas.call("gbblas_sdot_host", NDOT, p["a32"], p["b32"], hr32.ctypes.data)
        gbblas.call("gbblas_dmtv_host", 1, M, N, p["A64"], p["x64"], hy64.data_ptr())
        gbblas.call("gbblas_ddot_host", NDOT, p["a64"], p["b64"], hr64.ctypes.data)

    e2e_steps = max(1, min(args.steps, 5))
    e2e_step()  # warm-up (allocates the staging arena)
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    e2e_s = reduce_max(time.perf_counter() - t0, dev)
    barrier()
    h2d = sum(host[k].numel() * host[k].element_size() for k in host)
    d2h = M * 4 + 4 + M * 8 + 8
    e2e_val = aggregate(sb * e2e_steps, ws, e2e_s) / 1e9
    link = link_rate(host["A64"], dev)
    e2e = {"value": round(e2e_val, 2), "unit": UNIT,
           "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "steps": e2e_steps,
           "api": "gbblas_smtv_host/gbblas_sdot_host/gbblas_dmtv_host/gbblas_ddot_host (pinned host buffers)",
           "link_gbs": round(link, 1), "frac_of_link": round(e2e_val / ws / link, 4),
           "link": "host-to-device copy of one pinned 2 GiB buffer (cudaMemcpyAsync), best of 5, this run"}
    # the host path must give the device path's bits on the same inputs
    e2e_results = step_results(hy32.numpy(), hy64.numpy(), hr32[0], hr64[0])
    e2e["same_results_as_device"] = e2e_results == results

    # ---- errors against the oracle on the same inputs (outside every timed region)
    if rank == 0 and not args.no_cpu:
        results["vs_oracle"] = oracle_errors(host, y32, y64, results)

    # ---- CPU baseline (rank 0 only): the oracle on the host cores
    cpu = None
    if rank == 0 and not args.no_cpu:
        bufs = cpu_buffers_from(host)
        times = time_cpu(bufs, min_seconds=args.cpu_seconds)
        cpu = {"value": round(sb / statistics.mean(times) / 1e9, 3), "unit": UNIT,
               "cores": os.cpu_count(), "kind": cpu_kind(),
               "sample": f"{len(times)} full steps (all four calls at full size) after 1 warm-up, "
                         f"mean {statistics.mean(times) * 1e3:.1f} ms/step, OpenMP on all host cores"}

    extras = {}
    if rank == 0 and not args.no_gemm:
        t.clear()  # the step's device buffers; the pinned host inputs stay for nothing else
        host.clear()
        torch.cuda.empty_cache()
        extras = default_extras(args, dev, sp)

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms_per_step, 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
            "config": config(),
            "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU",
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak,
                         "unit": "GB/s", "frac": round(achieved / peak, 4), "traffic": traffic,
                         "peak_source": f"MEASURED_PEAKS.json hbm_gbs ({peak_kind})"},
            "kernels": kernels,
            "e2e": e2e,
            "cpu_baseline": cpu,
            "gpu_launches": int(launches),
            "clocks": clocks,
            "results": results,
        }
        line.update(extras)
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


# ------------------------------------------------------------------ reference arm

def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return  # one host, one CPU baseline: other ranks exit without work
    from oracle import oracle as O
    O.build(with_ref=False)
    kind = cpu_kind()
    bufs = make_cpu_inputs()
    bufs["y32"] = __import__("numpy").zeros(M, "float32")
    bufs["y64"] = __import__("numpy").zeros(M, "float64")
    O.set_threads(os.cpu_count() or 1)
    for _ in range(args.warmup):
        cpu_step_oracle(bufs)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        cpu_step_oracle(bufs)
    dt = time.perf_counter() - t0
    value = step_bytes() * args.steps / dt / 1e9
    r32, r64 = cpu_step_oracle(bufs)  # the outputs of one more step, for the results key
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dt * 1e3 / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic", "config": config(), "parallelism": "host CPU (OpenMP)",
        "cpu_baseline": {"value": round(value, 3), "unit": UNIT, "cores": os.cpu_count(), "kind": kind,
                         "sample": f"{args.steps} full steps after {args.warmup} warm-up, all host cores; "
                                   "oracle/oracle.c restatement of the reference's OpenMP code, pinned "
                                   "against the compiled reference where its sources exist"},
        "e2e": {"value": round(value, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "results": step_results(bufs["y32"], bufs["y64"], r32, r64),
    }
    print(json.dumps(line), flush=True)


def run_precision(args):
    """The precision configuration: C = A*B, M = N = K = 8192 from float32,
    as split-BF16 (three or six tcgen05 products), split-FP16 (three), FP8-E4M3
    with per-128 K-block scales and plain FP32 (FMA pipe), on two input sets
    (U[-1,1) and wide-range s*m*2^e, e in [-10, 10]); TFLOP/s of 2*M*N*K
    algorithmic flops, max / mean relative error against long-double dots on
    sampled entries, and the same over the full matrix against the product
    computed on the FP64 pipes.  One JSON line per (path, set)."""
    import torch
    torch.cuda.set_device(0)
    n = args.gemm_n
    rep = precision_report(n, sets=args.sets.split(","), paths=args.paths.split(","), warmup=args.warmup,
                           iters=args.gemm_iters, sample=4096)
    for set_name, paths in rep.items():
        for path, rec in paths.items():
            line = {"metric": "GEMM TFLOP/s (float32 operands)", "path": path, "input_set": set_name, "M": n,
                    "N": n, "K": n, "flops": "2*M*N*K algorithmic", "error_sample": "4096 entries vs long double"}
            line.update(rec)
            print(json.dumps(line), flush=True)


def run_f64(args):
    """Double-precision GEMM, M = N = K = --gemm-n (8192) from float64
    operands on two input sets (U[-1,1) and wide-range s*m*2^e, e in
    [-10, 10]): the library default (AUTO: the guarded 7-digit scheme at
    this size), the FP64 pipes (FMA kernel) and the unguarded Ozaki scheme on
    the BF16 tensor cores with 7 and 8 digits.  TFLOP/s of 2*M*N*K algorithmic flops,
    max / mean relative and normwise error against long-double dots on
    sampled entries.  One JSON line per (path, set)."""
    import numpy as np
    import torch

    import gbblas
    from oracle import oracle as O
    torch.cuda.set_device(0)
    n = args.gemm_n
    flops = 2.0 * n ** 3
    g = torch.Generator(device="cuda").manual_seed(4)
    rng = np.random.default_rng(4)
    sample = 1024
    rows = rng.integers(0, n, sample)
    cols = rng.integers(0, n, sample)
    pp = os.path.join(ROOT, "MEASURED_PEAKS.json")
    peaks = json.load(open(pp)) if os.path.exists(pp) else {}
    for set_name in ("uniform", "wide"):
        if set_name not in args.sets.split(","):
            continue
        if set_name == "uniform":
            A = torch.rand(n, n, generator=g, device="cuda", dtype=torch.float64) * 2 - 1
            B = torch.rand(n, n, generator=g, device="cuda", dtype=torch.float64) * 2 - 1
        else:
            def wide():
                s = torch.where(torch.rand(n, n, generator=g, device="cuda") < 0.5, -1.0, 1.0).double()
                m = torch.rand(n, n, generator=g, device="cuda", dtype=torch.float64) + 1.0
                e = torch.randint(-10, 11, (n, n), generator=g, device="cuda").double()
                return s * m * torch.exp2(e)
            A, B = wide(), wide()
        An, Bn = A.cpu().numpy(), B.cpu().numpy()
        exact, absx = O.gemm_sample_exact(n, An, n, 1, Bn, n, 1, rows, cols)
        for path, acc, products in (("auto", 3, 29), ("digits7", 6, 28), ("digits8", 7, 36), ("fp64", 5, None)):
            if path not in args.f64_paths.split(","):
                continue
            C = torch.zeros(n, n, device="cuda", dtype=torch.float64)
            sp = torch.cuda.current_stream().cuda_stream or None

            def call():
                gbblas.call("gbblas_dgemm_ex", n, n, n, A.data_ptr(), n, 1, B.data_ptr(), n, 1, C.data_ptr(), n, 1,
                            acc, sp)
            slow = path == "fp64"
            for _ in range(1 if slow else args.warmup):
                call()
            torch.cuda.synchronize()
            iters = 2 if slow else args.gemm_iters
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            with ClockSampler(0) as clk:
                t0 = time.time()
                e0.record()
                for _ in range(iters):
                    call()
                e1.record()
                torch.cuda.synchronize()
                clk.mark(t0, time.time())
            gbblas.call("gbblas_check_stream", sp)
            ms = e0.elapsed_time(e1) / iters
            C.zero_()
            call()
            got = C.cpu().numpy()[rows, cols]
            rel = np.abs(got - exact) / np.maximum(np.abs(exact), 1e-300)
            normwise = np.abs(got - exact) / absx
            tf = flops / (ms / 1e3) / 1e12
            line = {"metric": "GEMM TFLOP/s (float64 operands)", "path": path, "input_set": set_name,
                    "value": round(tf, 3), "unit": "TFLOP/s", "ms_per_gemm": round(ms, 3), "M": n, "N": n, "K": n,
                    "flops": "2*M*N*K algorithmic", "dtype": "f64", "max_rel_err": float(rel.max()),
                    "mean_rel_err": float(rel.mean()), "max_normwise_err": float(normwise.max()),
                    "error_sample": f"{sample} entries vs long double", "clocks": clk.summary()}
            if products and peaks.get("bf16_tflops"):
                line["tensor_frac"] = round(products * tf / peaks["bf16_tflops"], 4)
                line["tensor_peak"] = (f"{products} BF16 digit products per algorithmic flop vs bf16_tflops "
                                       f"{peaks['bf16_tflops']} (measured, burst)")
            print(json.dumps(line), flush=True)
        del A, B


def batching_shapes(seed=3):
    """512 GEMM shapes (M, N, K log-uniform in [32, 2048], multiples of 8) and
    4096 GEMV shapes (rows, cols log-uniform in [256, 16384])."""
    import numpy as np
    rng = np.random.default_rng(seed)

    def lu(lo, hi, n):
        return np.exp(rng.uniform(np.log(lo), np.log(hi), n))
    g = np.maximum(8, np.round(lu(32, 2048, (512, 3)) / 8) * 8).astype(np.int64)
    r = np.round(lu(256, 16384, 4096)).astype(np.int64)
    c = np.round(lu(256, 16384, 4096)).astype(np.int64)
    return g, r, c, rng


def run_batching(args):
    print(json.dumps(batching_report(args)), flush=True)


def batching_report(args):
    """The batching configuration: one graph-captured batch of 512 GEMMs
    (float32 in, split-BF16 on the tensor cores) and 4096 row-major GEMVs,
    U[-1,1) from seed 3.  The GEMV matrices (243.5 GB in total) are windows
    at random 16-byte-aligned offsets of one pool of U[-1,1) data (--pool-gb),
    so the batch fits next to other users on the GPU; every GEMV still
    streams its whole matrix from HBM.  Reports the batch time, its
    roofline (sum of each problem's roofline time: tensor peak for GEMMs,
    HBM for GEMVs), sampled errors, and the CPU oracle on a sample."""
    import numpy as np
    import torch

    import gbblas
    from oracle import oracle as O
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    acc = {"bf16x3": 1, "bf16x6": 4}[args.batch_accuracy]
    products = {1: 3, 4: 6}[acc]
    g, r, c, rng = batching_shapes()
    gen = torch.Generator(device=dev).manual_seed(3)

    def U(*shape):
        return torch.rand(*shape, generator=gen, device=dev).mul_(2).sub_(1)

    gemms, gemm_t = [], []
    for (M, N, K) in g:
        A, B, C = U(M, K), U(K, N), torch.zeros(M, N, device=dev)
        gemms.append(gbblas.gemm_desc(A, B, C))
        gemm_t.append((A, B, C))
    pool_elems = int(args.pool_gb * (1 << 30)) // 4
    pool = torch.empty(pool_elems, device=dev)
    step = 1 << 28
    for s0 in range(0, pool_elems, step):
        pool[s0:s0 + step].uniform_(-1, 1, generator=gen)
    gemvs, gemv_t = [], []
    for rows, cols in zip(r, c):
        n = int(rows * cols)
        off = int(rng.integers(0, (pool_elems - n) // 4)) * 4
        A = pool[off:off + n].view(int(rows), int(cols))
        x, y = U(int(cols)), torch.zeros(int(rows), device=dev)
        gemvs.append(gbblas.gemv_desc(1, 0, int(rows), int(cols), A, x, y))
        gemv_t.append((A, x, y))
    gemm_flops = float((2 * g.prod(1)).sum())
    gemv_bytes = float(((r * c + r + c) * 4).sum())
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}
    t_gemm_roof = gemm_flops * products / (peaks["bf16_tflops"] * 1e12)
    t_gemv_roof = gemv_bytes / (peaks["hbm_gbs"] * 1e9)
    # the GEMMs' HBM floor: A and B read once in FP32, C read and written (C += A B)
    gemm_bytes = float(((g[:, 0] * g[:, 2] + g[:, 2] * g[:, 1]) * 4 + 2 * g[:, 0] * g[:, 1] * 4).sum())
    t_gemm_mem = gemm_bytes / (peaks["hbm_gbs"] * 1e9)

    def time_batch(batch, iters):
        s = torch.cuda.current_stream()
        for _ in range(args.warmup):
            batch.run(s)
        batch.sync()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        for _ in range(iters):
            batch.run(s)
        e1.record(s)
        batch.sync()
        return e0.elapsed_time(e1) / iters

    launches0 = gbblas.kernel_launches()
    t0 = time.perf_counter()
    b_all = gbblas.Batch(gemms, gemvs, accuracy=acc)
    plan_s = time.perf_counter() - t0
    b_gemm = gbblas.Batch(gemms, [], accuracy=acc)
    b_gemv = gbblas.Batch([], gemvs, accuracy=acc)
    with ClockSampler(0) as clk:
        t_wall0 = time.time()
        ms_all = time_batch(b_all, args.steps)
        clk.mark(t_wall0, time.time())
    ms_gemm = time_batch(b_gemm, args.steps)
    ms_gemv = time_batch(b_gemv, args.steps)
    launches = gbblas.kernel_launches() - launches0

    # sampled errors: fresh C (the timed runs accumulated into it)
    pick_g = rng.choice(len(gemms), 8, replace=False)
    pick_v = rng.choice(len(gemvs), 16, replace=False)
    for A, B, C in gemm_t:
        C.zero_()
    b_gemm.run()
    b_gemm.sync()
    gemm_err = 0.0
    for i in pick_g:
        A, B, C = gemm_t[i]
        ref = A.double() @ B.double()
        scale = A.abs().double() @ B.abs().double()
        gemm_err = max(gemm_err, float(((C.double() - ref).abs() / scale).max()))
    gemv_err = 0.0
    for i in pick_v:
        A, x, y = gemv_t[i]
        ref = A.double() @ x.double()
        scale = A.abs().double() @ x.abs().double()
        gemv_err = max(gemv_err, float(((y.double() - ref).abs() / scale).max()))

    # CPU oracle on a sample (serial per problem, all host cores each)
    cpu = None
    if not args.no_cpu:
        O.set_threads(os.cpu_count() or 1)
        sg = rng.choice(len(gemms), 24, replace=False)
        sv = rng.choice(len(gemvs), 48, replace=False)
        hg = [(gemm_t[i][0].cpu().numpy(), gemm_t[i][1].cpu().numpy()) for i in sg]
        hv = [(gemv_t[i][0].cpu().numpy(), gemv_t[i][1].cpu().numpy()) for i in sv]
        t0 = time.perf_counter()
        for A, B in hg:
            M, K = A.shape
            N = B.shape[1]
            Cc = np.zeros((M, N), np.float32)
            O.gemm_raw(M, N, K, A, K, 1, B, N, 1, Cc, N, 1)
        tg = time.perf_counter() - t0
        t0 = time.perf_counter()
        for A, x in hv:
            yy = np.zeros(A.shape[0], np.float32)
            O.mtv_raw(1, A.shape[0], A.shape[1], np.ascontiguousarray(A), x, yy)
        tv = time.perf_counter() - t0
        fl_s = float(sum(2 * g[i].prod() for i in sg))
        by_s = float(sum((r[i] * c[i] + r[i] + c[i]) * 4 for i in sv))
        est = gemm_flops / (fl_s / tg) + gemv_bytes / (by_s / tv)
        cpu = {"value": round(est * 1e3, 1), "unit": "ms per batch (estimated)", "cores": os.cpu_count(),
               "kind": cpu_kind(), "sample": f"{len(sg)} GEMMs + {len(sv)} GEMVs of the batch run serially on the "
                                              f"oracle ({tg:.2f} s + {tv:.2f} s), scaled by flops and bytes"}
    line = {"metric": "batch ms (512 GEMM + 4096 GEMV, one graph)", "value": round(ms_all, 3), "unit": "ms",
            "higher_is_better": False, "accuracy": args.batch_accuracy,
            "ms_gemm_only": round(ms_gemm, 3), "ms_gemv_only": round(ms_gemv, 3),
            "gemm_TFLOPs": round(gemm_flops / (ms_gemm / 1e3) / 1e12, 1),
            "gemv_GBs": round(gemv_bytes / (ms_gemv / 1e3) / 1e9, 1),
            "roofline": {"ms": round((t_gemm_roof + t_gemv_roof) * 1e3, 3),
                         "frac": round((t_gemm_roof + t_gemv_roof) / (ms_all / 1e3), 4),
                         "gemm_ms": round(t_gemm_roof * 1e3, 3), "gemv_ms": round(t_gemv_roof * 1e3, 3),
                         "gemm_hbm_floor_ms": round(t_gemm_mem * 1e3, 3),
                         "gemm_frac_of_tensor_bound": round(t_gemm_roof / (ms_gemm / 1e3), 4),
                         "gemm_frac_of_hbm_floor": round(t_gemm_mem / (ms_gemm / 1e3), 4),
                         "peaks": "MEASURED_PEAKS.json bf16_tflops (x products) and hbm_gbs; the GEMMs' HBM "
                                  "floor reads A and B once in FP32 and C twice (C += A B)"},
            "plan_s": round(plan_s, 2), "gemm_flops": gemm_flops, "gemv_bytes": gemv_bytes,
            "max_normwise_err": {"gemm": gemm_err, "gemv": gemv_err}, "cpu_baseline": cpu,
            "gpu_launches_incl_graphs": int(launches), "clocks": clk.summary(),
            "config": {"workload": "512 GEMM log-uniform [32,2048] + 4096 GEMV log-uniform [256,16384], seed 3",
                       "gemv_pool_GiB": args.pool_gb}}
    for b in (b_all, b_gemm, b_gemv):
        b.close()
    del gemm_t, gemv_t, pool
    torch.cuda.empty_cache()
    return line


def run_serving(args):
    print(json.dumps(serving_report(args)), flush=True)


def serving_report(args):
    """The serving configuration: Poisson arrivals at each rate of --rates of
    60 % mtm, 30 % mtv, 10 % dot; GEMM and GEMV dims log-uniform in
    [64, 4096], dot lengths log-uniform in [1k, 64M]; 80 % float32 at FP32
    accuracy (AUTO: the guarded split-FP16 GEMM, one FMA kernel below 2^26
    multiply-adds), 20 % float64; operands device
    resident (inputs are windows of a U[-1,1) pool, outputs from the server's
    pool), 64 GiB admission budget.  Per rate: achieved throughput, p50/p99
    latency (overall and per class) against the same requests run alone
    (one request set: each rate replays a prefix of it), and where the
    slowest 1 % of requests spent their time (queued, host launch, device)."""
    import numpy as np
    import torch

    import gbblas
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(5)
    gen = torch.Generator(device=dev).manual_seed(5)
    pool32 = torch.empty(int(args.pool_gb * (1 << 30)) // 8, device=dev).uniform_(-1, 1, generator=gen)
    pool64 = torch.empty(int(args.pool_gb * (1 << 30)) // 16, dtype=torch.float64, device=dev).uniform_(
        -1, 1, generator=gen)
    srv = gbblas.Server(streams=args.streams, max_group=args.max_group, budget_bytes=64 << 30,
                        heavy_streams=args.heavy_streams, heavy_us=args.heavy_us,
                        heavy_sm_percent=args.heavy_sm_percent, slice_us=getattr(args, "slice_us", 0))
    # float64 GEMMs: AUTO (the library default: guarded tensor-core digits
    # where the shape suits) or the FP64 pipes
    f64_acc = 5 if args.f64_accuracy == "fp64" else 3

    def lu(lo, hi):
        return int(round(float(np.exp(rng.uniform(np.log(lo), np.log(hi))))))

    def window(pool, n):
        off = int(rng.integers(0, (pool.numel() - n) // 4)) * 4
        return pool.data_ptr() + off * pool.element_size()

    outs = []

    def make_request():
        u = rng.random()
        f64 = rng.random() < 0.2
        pool = pool64 if f64 else pool32
        es = 8 if f64 else 4
        dt = gbblas.F64 if f64 else gbblas.F32
        if u < 0.6:
            M, N, K = lu(64, 4096), lu(64, 4096), lu(64, 4096)
            out = srv.alloc(M * N * es)
            outs.append(out)
            acc = f64_acc if f64 else 3
            return "mtm", gbblas.Request(gbblas.OP_MTM, dt, acc, 1, M, N, K, window(pool, M * K), window(pool, K * N),
                                         out)
        if u < 0.9:
            M, N = lu(64, 4096), lu(64, 4096)
            out = srv.alloc(M * es)
            outs.append(out)
            return "mtv", gbblas.Request(gbblas.OP_MTV, dt, 3, 1, M, N, 0, window(pool, M * N), window(pool, N), out)
        n = lu(1000, 64 << 20)
        out = srv.alloc(es)
        outs.append(out)
        return "dot", gbblas.Request(gbblas.OP_DOT, dt, 3, 1, n, 0, 0, window(pool, n), window(pool, n), out)

    # warm-up: every path once (kernel loading, scratch growth)
    warm = [make_request() for _ in range(64)]
    srv.run_trace([r for _, r in warm], np.zeros(len(warm)))

    # One request set for every measurement: each rate replays a prefix of it
    # with Poisson arrivals, and the lone latencies are those of the same
    # requests run one at a time (one in the system), so every p99 ratio
    # compares the same requests.
    n_max = int(max(args.max_requests, args.lone_requests))
    shared = [make_request() for _ in range(n_max)]
    lone_lat = np.empty(n_max)
    for i, (_, r) in enumerate(shared):
        lone_lat[i] = srv.wait(srv.submit(r))

    def pct(v, q):
        return float(np.percentile(np.asarray(v), q)) * 1e3 if len(v) else None

    def by_class(lat, reqs):
        out = {"all": lat}
        for cls in ("mtm", "mtv", "dot"):
            out[cls] = lat[[i for i, (c, _) in enumerate(reqs) if c == cls]]
        return out

    lone_p = {k: {"p50_ms": pct(v, 50), "p99_ms": pct(v, 99)} for k, v in by_class(lone_lat, shared).items()}
    lone_p["requests"] = n_max
    results = []
    for rate in args.rates:
        n = int(min(n_max, max(args.min_requests, rate * args.seconds)))
        reqs = shared[:n]
        arrivals = np.cumsum(rng.exponential(1.0 / rate, n))
        base = srv.stats()["submitted"]
        t0 = time.perf_counter()
        lat = srv.run_trace([r for _, r in reqs], arrivals)
        wall = time.perf_counter() - t0
        parts = np.array([srv.request_times(base + i) for i in range(n)])
        by = by_class(lat, reqs)
        lone_n = lone_lat[:n]
        res = {"rate": rate, "requests": n, "throughput_rps": round(n / wall, 1),
               "p50_ms": pct(lat, 50), "p99_ms": pct(lat, 99),
               "lone_p99_ms": pct(lone_n, 99),
               "p99_over_lone_p99": round(pct(lat, 99) / pct(lone_n, 99), 3),
               "p99_slowdown": round(float(np.percentile(lat / lone_n, 99)), 3),
               "per_class": {k: {"p50_ms": pct(v, 50), "p99_ms": pct(v, 99)} for k, v in by.items() if k != "all"}}
        # where the tail's time went: the requests at or above the p99 latency
        tail = lat >= np.percentile(lat, 99)
        res["tail_breakdown_ms"] = {
            "queued": round(float(parts[tail, 0].mean()) * 1e3, 4),
            "host_launch": round(float(parts[tail, 1].mean()) * 1e3, 4),
            "device_and_completion": round(float(parts[tail, 2].mean()) * 1e3, 4),
            "round_size": round(float(parts[tail, 3].mean()), 2),
            "classes": {c: int(sum(1 for i in np.nonzero(tail)[0] if reqs[i][0] == c)) for c in ("mtm", "mtv", "dot")}}
        res["p99_parts_ms"] = {"queued": pct(parts[:, 0], 99), "host_launch": pct(parts[:, 1], 99),
                               "device_and_completion": pct(parts[:, 2], 99)}
        results.append(res)
    for p in outs:
        srv.free(p)
    outs.clear()
    sustained = [r for r in results if r["p99_over_lone_p99"] <= 2.0]
    st = srv.stats()
    line = {"metric": "served p99 latency", "unit": "ms", "higher_is_better": False,
            "value": sustained[-1]["p99_ms"] if sustained else results[0]["p99_ms"],
            "sustained_rate_rps": sustained[-1]["rate"] if sustained else None,
            "lone": lone_p, "rates": results,
            "server": {k: st[k] for k in ("submitted", "completed", "rounds", "peak_inflight_bytes",
                                          "mean_round_size")},
            "config": {"workload": "Poisson 60% mtm / 30% mtv / 10% dot, dims log-uniform [64,4096], "
                                   "dot n log-uniform [1k,64M], 80% f32 (FP32-accurate) / 20% f64, seed 5",
                       "f64_gemm": ("FP64 pipes" if f64_acc == 5 else
                                    "AUTO: guarded 7-digit tensor-core scheme from 2^21 multiply-adds, FP64 pipes below"),
                       "budget_GiB": 64, "streams": args.streams or 16, "max_group": args.max_group or 256,
                       "heavy_streams": args.heavy_streams or 2, "heavy_sm_percent": args.heavy_sm_percent or 75,
                       "heavy_us": args.heavy_us or 300, "slice_us": getattr(args, "slice_us", 0) or 200}}
    srv.close()
    del pool32, pool64
    torch.cuda.empty_cache()
    return line


def run_stream_ops(args):
    """The streaming operations beside the hot path, one JSON line each:
    outer product C += a b^T (C 16384 x 16384 row-major f32; bytes 2*M*N*4 +
    (M+N)*4), out-of-place transpose (16384 x 16384 f32, row-major in and
    out; bytes 2*M*N*4) and element-wise add (2^28 f32; bytes 3*n*4), plus
    their f64 forms.  U[-1,1) from seed 4; every operand is larger than L2.
    GB/s of algorithmic bytes against the measured HBM copy bandwidth; the
    CPU oracle (the reference's code restated) on a 4096^2 / 2^24 sample on
    all host cores."""
    import numpy as np
    import torch

    import gbblas
    from oracle import oracle as O
    torch.cuda.set_device(0)
    peak, peak_kind = measured_peaks()
    g = torch.Generator(device="cuda").manual_seed(4)
    n2 = 16384
    nvec = 1 << 28
    for dt, tdt, pf in ((np.float32, torch.float32, "s"), (np.float64, torch.float64, "d")):
        s = np.dtype(dt).itemsize

        def U(*shape):
            return torch.rand(*shape, generator=g, device="cuda", dtype=tdt) * 2 - 1
        cases = []
        A = U(n2, n2)
        a, b = U(n2), U(n2)
        C = torch.empty(n2, n2, device="cuda", dtype=tdt)
        cases.append(("outer", 2 * n2 * n2 * s + 2 * n2 * s,
                      lambda: gbblas.call(f"gbblas_{pf}outer", 1, n2, n2, a.data_ptr(), b.data_ptr(), A.data_ptr(),
                                          None),
                      f"C {n2}x{n2} row-major += a b^T"))
        cases.append(("transpose", 2 * n2 * n2 * s,
                      lambda: gbblas.call(f"gbblas_{pf}transpose", n2, n2, A.data_ptr(), n2, 1, C.data_ptr(), n2, 1,
                                          None),
                      f"C = A^T, {n2}x{n2} row-major"))
        x, y = U(nvec // (s // 4)), U(nvec // (s // 4))
        z = torch.empty_like(x)
        nv = x.numel()
        cases.append(("ew_add", 3 * nv * s,
                      lambda: gbblas.call(f"gbblas_{pf}ew", 0, nv, x.data_ptr(), y.data_ptr(), z.data_ptr(), None),
                      f"c = a + b, n = {nv}"))
        for name, nbytes, fn, what in cases:
            for _ in range(args.warmup):
                fn()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            iters = 20
            with ClockSampler(0) as clk:
                t0 = time.time()
                e0.record()
                for _ in range(iters):
                    fn()
                e1.record()
                torch.cuda.synchronize()
                clk.mark(t0, time.time())
            gbblas.call("gbblas_check_stream", None)
            ms = e0.elapsed_time(e1) / iters
            gbs = nbytes / (ms / 1e3) / 1e9
            line = {"metric": "streaming op GB/s", "op": name, "dtype": "f32" if s == 4 else "f64",
                    "value": round(gbs, 1), "unit": "GB/s", "ms_per_call": round(ms, 4), "workload": what,
                    "bytes": "algorithmic", "roofline": {"bound": "hbm", "achieved": round(gbs, 1),
                                                        "peak": peak, "unit": "GB/s",
                                                        "frac": round(gbs / peak, 4),
                                                        "peak_source": peak_kind},
                    "clocks": clk.summary()}
            if not args.no_cpu:
                rng = np.random.default_rng(4)
                O.set_threads(os.cpu_count() or 1)
                m = 4096
                if name == "outer":
                    hA = rng.uniform(-1, 1, (m, m)).astype(dt)
                    ha, hb = rng.uniform(-1, 1, m).astype(dt), rng.uniform(-1, 1, m).astype(dt)
                    buf = hA.ravel().copy()
                    run = lambda: getattr(O.lib(), f"orc_{pf}outer")(1, m, m, ha.ctypes.data, hb.ctypes.data,
                                                                          buf.ctypes.data)
                    cb = 2 * m * m * s + 2 * m * s
                    sample = f"{m}x{m}"
                elif name == "transpose":
                    hA = rng.uniform(-1, 1, m * m).astype(dt)
                    hC = np.empty_like(hA)
                    run = lambda: O.transpose_raw(m, m, hA, m, 1, hC, m, 1)
                    cb = 2 * m * m * s
                    sample = f"{m}x{m}"
                else:
                    k = 1 << 24
                    hx, hy = rng.uniform(-1, 1, k).astype(dt), rng.uniform(-1, 1, k).astype(dt)
                    hz = np.empty_like(hx)
                    run = lambda: getattr(O.lib(), f"orc_{pf}ew")(0, k, hx.ctypes.data, hy.ctypes.data,
                                                                       hz.ctypes.data)
                    cb = 3 * k * s
                    sample = f"n = {k}"
                run()
                t0 = time.perf_counter()
                reps = 0
                while time.perf_counter() - t0 < 2.0 or reps < 3:
                    run()
                    reps += 1
                dtc = (time.perf_counter() - t0) / reps
                line["cpu_baseline"] = {"value": round(cb / dtc / 1e9, 2), "unit": "GB/s",
                                        "cores": os.cpu_count(), "kind": "port",
                                        "sample": f"oracle restatement, {sample}, {reps} reps"}
            print(json.dumps(line), flush=True)
        del A, C, a, b, x, y, z
        torch.cuda.empty_cache()


def run_mtm(args):
    print(json.dumps(mtm_report(args)), flush=True)


def mtm_report(args):
    """The plain single-precision mtm configuration: C = A*B, M = N = K = 1024,
    row-major float32, A then B U[-1,1) from seed 0, C zeroed; FP32 on the FMA
    pipes (the default accuracy).  TFLOP/s with 2*M*N*K flops (and the
    reference's M*N*(2K-1) count beside it), CUDA events over 20 calls after 3
    warm-ups, against the FMA-pipe peak; max normwise / relative error against
    FP64 and against the reference's own mtm (the oracle's compiled reference
    where it exists here, else its restatement); the same call from host
    buffers (gbblas_sgemm_host) for e2e; the CPU baseline is the reference
    algorithm on all host cores, mean of 10 after 2 warm-ups."""
    import numpy as np
    import torch

    import gbblas
    from oracle import oracle as O
    torch.cuda.set_device(0)
    n = 1024
    A, B = np.empty((n, n), np.float32), np.empty((n, n), np.float32)
    gbblas.seeded_fill(0, [A.reshape(-1), B.reshape(-1)], None)
    tA, tB = torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()
    tC = torch.zeros(n, n, device="cuda")
    sp = torch.cuda.current_stream().cuda_stream or None

    def call():
        gbblas.call("gbblas_sgemm", n, n, n, tA.data_ptr(), n, 1, tB.data_ptr(), n, 1, tC.data_ptr(), n, 1, 0, sp)
    for _ in range(max(3, args.warmup)):
        call()
    torch.cuda.synchronize()
    iters = 20
    launches0 = gbblas.kernel_launches()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as clk:
        t0 = time.time()
        e0.record()
        for _ in range(iters):
            call()
        e1.record()
        torch.cuda.synchronize()
        clk.mark(t0, time.time())
    launches = gbblas.kernel_launches() - launches0
    gbblas.call("gbblas_check_stream", sp)
    ms = e0.elapsed_time(e1) / iters
    tC.zero_()
    call()
    got = tC.cpu().numpy().astype(np.float64)
    exact = A.astype(np.float64) @ B.astype(np.float64)
    absx = np.abs(A).astype(np.float64) @ np.abs(B).astype(np.float64)
    ref_kind = "reference" if O.ref_available() else "port"
    ref = (O.ref_gemm(A, B, np.zeros((n, n), np.float32), 1, 1, 1) if ref_kind == "reference"
           else O.gemm(A, B, np.zeros((n, n), np.float32), 1, 1, 1)).astype(np.float64)
    tf = 2.0 * n ** 3 / (ms / 1e3) / 1e12
    peak = fma_peak_tflops(clk.summary())
    # e2e: host buffers through the drop-in's C call (copies in and out inside the call)
    Ch = np.zeros((n, n), np.float32)
    for _ in range(2):
        gbblas.call("gbblas_sgemm_host", n, n, n, A.ctypes.data, n, 1, B.ctypes.data, n, 1, Ch.ctypes.data, n, 1, 0)
    reps = 10
    t0 = time.perf_counter()
    for _ in range(reps):
        gbblas.call("gbblas_sgemm_host", n, n, n, A.ctypes.data, n, 1, B.ctypes.data, n, 1, Ch.ctypes.data, n, 1, 0)
    e2e_s = (time.perf_counter() - t0) / reps
    line = {"metric": "plain mtm TFLOP/s (float32, FMA pipes)", "value": round(tf, 3), "unit": "TFLOP/s",
            "n_gpus": 1, "steps": iters, "warmup": max(3, args.warmup), "ms_per_step": round(ms, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "mtm C = A*B, M = N = K = 1024, row-major float32, U[-1,1) from "
                                   "std::mt19937_64(0), A then B",
                       "flops": "2*M*N*K", "l2": "operands fit in L2 (12 MB); repeated calls"},
            "reference_gflops_count": round(n * n * (2 * n - 1) / (ms / 1e3) / 1e9, 1),
            "roofline": {"bound": "fma", "achieved": round(tf, 3), "peak": round(peak, 1), "unit": "TFLOP/s",
                         "frac": round(tf / peak, 4),
                         "peak_source": "SMs x 128 FP32 FMA lanes x 2 flop x max SM clock (nominal)"},
            "max_normwise_err_vs_fp64": float(np.max(np.abs(got - exact) / absx)),
            "max_rel_err_vs_fp64": float(np.max(np.abs(got - exact) / np.maximum(np.abs(exact), 1e-300))),
            "max_normwise_diff_vs_reference": float(np.max(np.abs(got - ref) / absx)),
            "reference_kind": ref_kind,
            "e2e": {"value": round(2.0 * n ** 3 / e2e_s / 1e12, 3), "unit": "TFLOP/s",
                    "h2d_bytes_per_step": 3 * n * n * 4, "d2h_bytes_per_step": n * n * 4,
                    "api": "gbblas_sgemm_host (host buffers)"},
            "gpu_launches": launches, "clocks": clk.summary()}
    if not args.no_cpu:
        O.set_threads(os.cpu_count() or 1)
        fn = O.ref_gemm if ref_kind == "reference" else O.gemm
        Z = np.zeros((n, n), np.float32)
        for _ in range(2):
            fn(A, B, Z, 1, 1, 1)
        t0 = time.perf_counter()
        for _ in range(10):
            fn(A, B, Z, 1, 1, 1)
        cpu_s = (time.perf_counter() - t0) / 10
        line["cpu_baseline"] = {"value": round(2.0 * n ** 3 / cpu_s / 1e12, 4), "unit": "TFLOP/s",
                                "cores": os.cpu_count(), "kind": ref_kind,
                                "sample": f"the full 1024^3 mtm, mean of 10 after 2 warm-ups ({cpu_s * 1e3:.1f} ms)"}
    return line


def run_sweep(args):
    """The reference's benchmark drivers (src/mtm.cpp:355-372, src/mtv.cpp:326-345,
    src/dot.cpp:198-205) on the GPU: the same size sweeps, ones-filled
    operands (make_tensor(..., 1.)), first_order float, MaxIter timed calls per
    size averaged, GFLOP/s = ops / ns with the reference's op counts
    (mtm M*N*(2K-1), mtv and dot as in their drivers), written in the
    reference's metric formats (gbblas/metric.py: csv, summary text).

    Series: "gbblas.GB300" (device-resident operands, CUDA events per call),
    "gbblas.GB300.host" (the drop-in's host-buffer call, wall clock - what
    amt::mtm(...)() costs a host caller), "Boost.ublas.tensor" (the
    reference's algorithm on the host cores through the oracle port, which
    restates it; sizes up to --sweep-cpu-max, 0 beyond)."""
    import numpy as np
    import torch

    import gbblas
    from gbblas.metric import Metric, reference_range
    from oracle import oracle as O
    torch.cuda.set_device(0)
    op = args.sweep_op
    if op == "mtm":
        x = reference_range(32.0, 3 * 1024.0, 32.0, "plus")
        iters = 4
    elif op == "mtv":
        x = reference_range(2.0, float(1 << 16), 2.0, "multiplies")
        iters = 10
    else:
        x = reference_range(2.0, float(1 << 20), 1024.0, "plus")
        iters = 100
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    # GPU peak for the summary: FP32 FMA for mtm (152 SMs x 128 lanes x 2 flop x max clock),
    # HBM-bound ops: flops at the measured copy bandwidth (2 flop per 4-byte element)
    mhz = peaks.get("sm_max_mhz", 2070.0)
    peak = 152 * 128 * 2 * mhz / 1e3 if op == "mtm" else peaks.get("hbm_gbs", 6680.8) / 2.0
    m = Metric(len(x), np.float32, peak=peak)
    gpu, host, cpu = m["gbblas.GB300"], m["gbblas.GB300.host"], m["Boost.ublas.tensor"]
    O.set_threads(os.cpu_count() or 1)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for el in x:
        n = int(el)
        if op == "mtm":
            ops = float(n) * n * (2.0 * n - 1.0)
            A = torch.ones(n * n, device="cuda")
            B = torch.ones(n * n, device="cuda")
            C = torch.zeros(n * n, device="cuda")
            dev_call = lambda: gbblas.call("gbblas_sgemm", n, n, n, A.data_ptr(), 1, n, B.data_ptr(), 1, n,
                                           C.data_ptr(), 1, n, 0, None)
            hA, hB, hC = np.ones(n * n, np.float32), np.ones(n * n, np.float32), np.zeros(n * n, np.float32)
            host_call = lambda: gbblas.call("gbblas_sgemm_host", n, n, n, hA.ctypes.data, 1, n, hB.ctypes.data, 1,
                                            n, hC.ctypes.data, 1, n, 0)
            cpu_call = lambda: O.gemm_raw(n, n, n, hA, 1, n, hB, 1, n, hC, 1, n)
            cpu_ok = n <= args.sweep_cpu_max
        elif op == "mtv":
            ops = float(n) * (2.0 * n - 1.0)
            A = torch.ones(n * n, device="cuda")
            v = torch.ones(n, device="cuda")
            y = torch.zeros(n, device="cuda")
            dev_call = lambda: gbblas.call("gbblas_smtv", 0, n, n, A.data_ptr(), v.data_ptr(), y.data_ptr(), None)
            hA, hv, hy = np.ones(n * n, np.float32), np.ones(n, np.float32), np.zeros(n, np.float32)
            host_call = lambda: gbblas.call("gbblas_smtv_host", 0, n, n, hA.ctypes.data, hv.ctypes.data,
                                            hy.ctypes.data)
            cpu_call = lambda: O.mtv_raw(0, n, n, hA, hv, hy)
            cpu_ok = n <= args.sweep_cpu_max * 16
        else:
            ops = 2.0 * n
            a = torch.ones(n, device="cuda")
            r = torch.zeros(1, device="cuda")
            dev_call = lambda: gbblas.call("gbblas_sdot", n, a.data_ptr(), a.data_ptr(), r.data_ptr(), None)
            ha, hr = np.ones(n, np.float32), np.zeros(1, np.float32)
            host_call = lambda: gbblas.call("gbblas_sdot_host", n, ha.ctypes.data, ha.ctypes.data, hr.ctypes.data)
            cpu_call = lambda: O.dot(ha, ha)
            cpu_ok = True
        dev_call()
        torch.cuda.synchronize()
        ns = 0.0
        for _ in range(iters):
            e0.record()
            dev_call()
            e1.record()
            e1.synchronize()
            ns += e0.elapsed_time(e1) * 1e6
        gpu.update(ops / (ns / iters))
        host_call()
        t0 = time.perf_counter()
        for _ in range(iters):
            host_call()
        host.update(ops / ((time.perf_counter() - t0) * 1e9 / iters))
        if cpu_ok and not args.no_cpu:
            cpu_call()
            t0 = time.perf_counter()
            for _ in range(iters):
                cpu_call()
            cpu.update(ops / ((time.perf_counter() - t0) * 1e9 / iters))
        else:
            cpu.update(0.0)
    gbblas.call("gbblas_check_stream", None)
    csv_path = args.sweep_csv or os.path.join(ROOT, "openmp-blas_gb300", "_build", f"sweep_{op}.csv")
    os.makedirs(os.path.dirname(csv_path), exist_ok=True)
    m.csv(csv_path)
    print(m.str("tensor"), file=sys.stderr)
    line = {"metric": f"{op} sweep GFLOP/s", "unit": "GFLOP/s", "sizes": [int(v) for v in x], "max_iter": iters,
            "series": {k: [round(v, 3) for v in d.plot] for k, d in m.data.items()},
            "summary_peak": round(peak, 1), "csv": os.path.relpath(csv_path, ROOT),
            "cpu": {"kind": "port", "cores": os.cpu_count(), "max_size": args.sweep_cpu_max},
            "config": {"workload": f"reference driver sweep for {op}, first_order float, ones-filled"}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="bandwidth",
                    choices=["bandwidth", "precision", "f64", "batching", "serving", "stream_ops", "sweep", "mtm"])
    ap.add_argument("--sweep-op", default="mtm", choices=["mtm", "mtv", "dot"])
    ap.add_argument("--sweep-cpu-max", type=int, default=1024,
                    help="sweep workload: largest size the CPU series runs (0 beyond)")
    ap.add_argument("--sweep-csv", default=None, help="sweep workload: CSV path (reference metric format)")
    ap.add_argument("--rates", type=float, nargs="+", default=[500, 1000, 2000, 5000, 10000, 20000, 50000])
    ap.add_argument("--seconds", type=float, default=1.0)
    ap.add_argument("--min-requests", type=int, default=400)
    ap.add_argument("--max-requests", type=int, default=4000)
    ap.add_argument("--lone-requests", type=int, default=200,
                    help="serving: size of the shared request set is the larger of this and --max-requests")
    ap.add_argument("--streams", type=int, default=0,
                    help="serving: light rounds in flight at once (0: the library default)")
    ap.add_argument("--max-group", type=int, default=0,
                    help="serving: requests per light round (0: the library default)")
    ap.add_argument("--heavy-sm-percent", type=int, default=0,
                    help="serving: share of the SMs a heavy request may take (0: the library default)")
    ap.add_argument("--heavy-streams", type=int, default=0,
                    help="serving: heavy requests in flight at once (0: the library default)")
    ap.add_argument("--slice-us", type=int, default=0,
                    help="serving: estimated work per slice of a heavy GEMM (0: the library default, "
                         "-1: no slices, the SM cap)")
    ap.add_argument("--heavy-us", type=int, default=0,
                    help="serving: estimated GPU time (us) above which a request is heavy (0: default)")
    ap.add_argument("--pool-gb", type=float, default=48.0)
    ap.add_argument("--f64-accuracy", default="auto", choices=["auto", "fp64"],
                    help="serving: arithmetic of the float64 GEMM requests")
    ap.add_argument("--batch-accuracy", default="bf16x3", choices=["bf16x3", "bf16x6"])
    ap.add_argument("--gemm-n", type=int, default=8192)
    ap.add_argument("--gemm-iters", type=int, default=5)
    ap.add_argument("--paths", default="bf16x3,bf16x6,fp16x3,fp8,fp32",
                    help="precision workload: comma-separated GEMM paths to run")
    ap.add_argument("--sets", default="uniform,wide", help="precision workload: input sets to run")
    ap.add_argument("--f64-paths", default="auto,digits7,digits8,fp64",
                    help="f64 workload: comma-separated double-precision GEMM paths to run")
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gbblas", choices=["gbblas", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-gemm", action="store_true",
                    help="default workload: skip the measurements added beside the bandwidth line "
                         "(precision, FP8, double GEMM, 1024^3 mtm, batching, serving)")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--small", action="store_true",
                    help="profiling case: mtv 8192^2 and dot 2^26 (still larger than L2), "
                         "no e2e and no CPU leg; not a benchmark result")
    args = ap.parse_args()
    if args.small:
        global M, N, NDOT
        M = N = 8192
        NDOT = 1 << 26
        args.no_cpu = True
    if args.warmup < 3 and args.impl == "gbblas":
        print("warning: fewer than 3 warm-up steps", file=sys.stderr)
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "precision":
        run_precision(args)
    elif args.workload == "f64":
        run_f64(args)
    elif args.workload == "batching":
        run_batching(args)
    elif args.workload == "serving":
        run_serving(args)
    elif args.workload == "stream_ops":
        run_stream_ops(args)
    elif args.workload == "sweep":
        run_sweep(args)
    elif args.workload == "mtm":
        run_mtm(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
