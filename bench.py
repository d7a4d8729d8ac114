"""Benchmark: signature forward + reverse pass, paths/s.

Workload (the headline configuration): 4096 piecewise-linear paths, width 5,
depth 5 (3906 tensor coefficients), 256 increments each drawn i.i.d.
N(0, 1/256) per channel, FP64.  One step = the fused forward + reverse launch
over the whole batch: S(x_b) for every path and d/dx sum_b <ell_b, S(x_b)> with
ell_b ~ U[-1, 1].  Inputs and outputs (~340 MB) exceed the 129 MB L2, so no
explicit L2 flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line (rank 0).  `value` times the kernel with inputs resident
in HBM; `e2e` times the same through the public API with pinned host buffers
(H2D of increments + seeds, D2H of signatures + gradients inside the timed
region).  `--impl reference` times the reference's CPU implementation of the
same computation on the host cores (the reference's own CPU strategy, compiled
from its headers into oracle/_ref where they were installed; else the oracle's
C restatement) for a bounded sample of the same workload.  `--gpus N` without
torch.distributed's environment relaunches itself with one process per GPU.
"""
from __future__ import annotations

import argparse
import importlib
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

WIDTH, DEPTH, BATCH, LENGTH = 5, 5, 4096, 256
# DRAM bytes of one headline step under the two-launch schedule, from a
# one-pass ncu capture (dram__bytes_read.sum + dram__bytes_write.sum, nine steps)
# of `python bench.py --steps 2 --warmup 3 --no-cpu-baseline --no-plain
# --schedule 134267008` (the tuner's schedule: two launches, 128 threads, the
# forward launch's top level in the output row, the D-barrier reverse step):
# forward launch 44.3 MB read + 83.1 MB written, reverse launch 199.7 MB read +
# 30.9 MB written -- the compulsory inputs and outputs, the seed's top level
# re-read from L2, not DRAM.  (Schedule 16512, without the top level in the
# row: 335.3 MB.)
TWO_LAUNCH_TRAFFIC_BYTES = 358.0e6
METRIC = "signature fwd+bwd paths/sec (d=5,N=5,L=256) fused vs plain; % of roofline"


def step_fma(width: int, depth: int) -> int:
    """FMAs of one Chen step with a letter-only increment: sum_i (D-i+1) W^i."""
    return sum((depth - i + 1) * width ** i for i in range(1, depth + 1))


def tensor_dim(width: int, depth: int) -> int:
    return sum(width ** i for i in range(depth + 1))


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.file = None

    def start(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=self.file, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        self.file.flush()
        with open(self.file.name) as f:
            rows = [r.strip().split(", ") for r in f if r.strip()]
        os.unlink(self.file.name)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for name, val in zip(names, r[5:9]):
                if val.strip() == "Active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_inputs(seed: int, batch: int):
    rng = np.random.default_rng(seed)
    incr = rng.normal(0.0, 1.0 / np.sqrt(LENGTH), (batch * LENGTH, WIDTH))
    ell = rng.uniform(-1.0, 1.0, (batch, tensor_dim(WIDTH, DEPTH)))
    return incr, ell


def headline_config(batch: int, world: int) -> dict:
    """The workload's description, shared by both arms' JSON lines."""
    return {"workload": "signature_fwd_bwd_w5_d5_l256", "width": WIDTH, "depth": DEPTH, "batch_per_gpu": batch,
            "length": LENGTH, "increments": "N(0,1/256) iid", "seed_functional": "U[-1,1]",
            "l2": "inputs+outputs 340 MB > L2 (no flush needed)", "parallelism": f"replicas x{world}"}


def cpu_reference(steps: int, warmup: int, world: int, rank: int):
    """CPU arm: the signature forward pass and the stored-prefix reverse pass
    on all host cores, each step a bounded sample of the workload's paths.
    Runs the reference itself (its CPU strategy compiled from its headers into
    oracle/_ref by build(), driven through its public operations) where that
    library was built, else the oracle's C restatement of the same algorithm."""
    if rank != 0:
        return None
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    if os.path.exists(O.REF_LIB_PATH):
        impl, kind = O.RefBridge(), "reference"
        what = ("the reference's SingleThreadStrategy<double> through rpp::ops: ft_fmexp forward storing "
                "prefixes, then ft_exp, ft_adj_lmul, ft_adj_rmul per increment")
    else:
        impl, kind = O.Oracle(), "port"
        what = "the oracle's C restatement of the reference's forward and stored-prefix reverse pass"
    cores = os.cpu_count() or 1
    sample = max(cores, 2 * cores)
    incr, ell = make_inputs(1234, sample)
    offs = np.arange(sample + 1, dtype=np.int64) * LENGTH
    for _ in range(max(0, warmup)):
        impl.signature(WIDTH, DEPTH, incr, offs, ell=ell, threads=cores)
    times = []
    for _ in range(steps):
        t0 = time.perf_counter()
        impl.signature(WIDTH, DEPTH, incr, offs, ell=ell, threads=cores)
        times.append(time.perf_counter() - t0)
    total = sum(times)
    return {"value": sample * steps / total, "unit": "paths/s", "cores": cores, "kind": kind,
            "sample": f"{sample} of the {BATCH} paths per step (W5 D5 L256 FP64, forward + stored-prefix "
                      f"reverse; {what}; {cores} threads)",
            "ms_per_step": 1e3 * total / steps}


def plain_path(pkg, strat, cfg, basis, incr, ell, batch, grad):
    """The plain per-operation GPU path over the same workload: L launches of
    ft_fmexp storing every prefix, then per increment (last first) ft_exp,
    ft_adj_lmul, ft_adj_rmul and the exp VJP.  Returns the final signatures."""
    import torch

    W, D, L = WIDTH, DEPTH, LENGTH
    dim = basis.size()
    dev = incr.device
    prefixes = torch.empty(L + 1, batch, dim, dtype=torch.float64, device=dev)
    G, Gn, H, E = (torch.empty(batch, dim, dtype=torch.float64, device=dev) for _ in range(4))
    full = lambda t: pkg.make_tensor_batch(t, dim, 0, D)  # noqa: E731
    # X_k: increment k of every path viewed as the degree-one part of a tensor
    xview = lambda k: pkg.make_tensor_batch(incr, L * W, 1, 1, offset=k * W - 1)  # noqa: E731
    pkg.tensor_set_identity(strat, cfg, full(prefixes[0]), basis, batch).raise_if_failed()
    for k in range(L):
        pkg.ft_fmexp(strat, cfg, full(prefixes[k + 1]), full(prefixes[k]), xview(k), basis, batch).raise_if_failed()
    G.copy_(ell)
    for k in range(L - 1, -1, -1):
        pkg.ft_exp(strat, cfg, full(E), xview(k), basis, batch).raise_if_failed()
        pkg.ft_adj_lmul(strat, cfg, full(H), full(prefixes[k]), full(G), basis, batch).raise_if_failed()
        pkg.exp_letter_vjp(strat, cfg, H, incr, grad, basis, batch, x_stride=L * W, dx_stride=L * W,
                           x_offset=k * W, dx_offset=k * W).raise_if_failed()
        pkg.ft_adj_rmul(strat, cfg, full(Gn), full(E), full(G), basis, batch).raise_if_failed()
        G, Gn = Gn, G
    return prefixes[L]


REF_BLOCK_LIB = os.path.join(ROOT, "baseline", "_build", "libref_block.so")


def _ref_block_lib():
    """The reference's own GPU strategy (BlockStrategy<double, 128, 256>,
    built by `make -C baseline` from the reference's headers), or None."""
    import ctypes
    if not os.path.exists(REF_BLOCK_LIB):
        return None
    lib = ctypes.CDLL(REF_BLOCK_LIB)
    vp, i32, i64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64
    lib.ref_block_tensor_set_identity.argtypes = [vp, i32, i32, vp, i64, i64]
    lib.ref_block_ft_fmexp.argtypes = [vp, i32, i32, vp, i64, vp, i64, vp, i64, i32, i32, i64]
    lib.ref_block_ft_exp.argtypes = [vp, i32, i32, vp, i64, vp, i64, i32, i32, i64]
    lib.ref_block_ft_adj_lmul.argtypes = [vp, i32, i32, vp, i64, vp, i64, vp, i64, i64]
    lib.ref_block_ft_adj_rmul.argtypes = [vp, i32, i32, vp, i64, vp, i64, vp, i64, i64]
    return lib


def plain_reference_path(lib, pkg, strat, cfg, basis, xpad, incr, ell, batch, grad, stream):
    """plain_path with the reference's own GPU kernels: the same loop (L
    ft_fmexp launches storing every prefix, then per increment ft_exp,
    ft_adj_lmul, the exp VJP and ft_adj_rmul), each operation run by the
    reference's BlockStrategy except the exp VJP, which the reference does not
    have (this repository's rpp_gb_exp_letter_vjp, about 2 dim FMAs per path
    and step).  `xpad` holds the increments one element later than `incr`, so
    that the degree-one view of increment k starts inside the allocation."""
    import torch

    W, D, L = WIDTH, DEPTH, LENGTH
    dim = basis.size()
    dev = incr.device
    prefixes = torch.empty(L + 1, batch, dim, dtype=torch.float64, device=dev)
    G, Gn, H, E = (torch.empty(batch, dim, dtype=torch.float64, device=dev) for _ in range(4))
    s = stream.cuda_stream
    xp = xpad.data_ptr()

    def ok(rc, what):
        if rc != 0:
            raise RuntimeError(f"reference {what} failed with code {rc}")

    ok(lib.ref_block_tensor_set_identity(s, W, D, prefixes[0].data_ptr(), dim, batch), "tensor_set_identity")
    for k in range(L):
        ok(lib.ref_block_ft_fmexp(s, W, D, prefixes[k + 1].data_ptr(), dim, prefixes[k].data_ptr(), dim,
                                  xp + 8 * k * W, L * W, 1, 1, batch), "ft_fmexp")
    G.copy_(ell)
    for k in range(L - 1, -1, -1):
        ok(lib.ref_block_ft_exp(s, W, D, E.data_ptr(), dim, xp + 8 * k * W, L * W, 1, 1, batch), "ft_exp")
        ok(lib.ref_block_ft_adj_lmul(s, W, D, H.data_ptr(), dim, prefixes[k].data_ptr(), dim, G.data_ptr(), dim,
                                     batch), "ft_adj_lmul")
        pkg.exp_letter_vjp(strat, cfg, H, incr, grad, basis, batch, x_stride=L * W, dx_stride=L * W,
                           x_offset=k * W, dx_offset=k * W).raise_if_failed()
        ok(lib.ref_block_ft_adj_rmul(s, W, D, Gn.data_ptr(), dim, E.data_ptr(), dim, G.data_ptr(), dim, batch),
           "ft_adj_rmul")
        G, Gn = Gn, G
    return prefixes[L]


# ---------------------------------------------------------------------------
# Other configurations (`--workload`), one JSON line each.  Device-resident
# inputs; CUDA-event timing over `steps` launches after warm-up; FP64 peak
# measured in-run; CPU baseline = the oracle on a bounded sample.
# ---------------------------------------------------------------------------

def _time_launches(torch, fn, steps, warmup, stream):
    for _ in range(max(3, warmup)):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    nvtx = getattr(torch.cuda, "nvtx", None)
    try:
        nvtx.range_push("timed_region")  # lets a profiler select the timed launches
    except Exception:
        nvtx = None
    e0.record(stream)
    for _ in range(steps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    if nvtx is not None:
        nvtx.range_pop()
    return e0.elapsed_time(e1) / 1e3 / steps


def _fp64_peak(pkg, device):
    import ctypes

    out = ctypes.c_double(0)
    rc = pkg.library().rpp_gb_fma_peak(1, device, ctypes.byref(out))
    return out.value if rc == 0 else None


def _line(metric, value, unit, ms, dtype, config, flops=None, peak=None, cpu=None, extra=None):
    roof = None
    if flops is not None and peak:
        ach = flops / (ms / 1e3) / 1e12
        roof = {"bound": "fp64_fma", "achieved": ach, "peak": peak, "unit": "TFLOP/s", "frac": ach / peak,
                "traffic": None, "peak_source": "measured in-run (rpp_gb_fma_peak, FP64)",
                "algorithmic_flops_per_launch": flops}
    line = {"metric": metric, "value": value, "unit": unit, "n_gpus": 1, "ms_per_step": ms,
            "higher_is_better": True, "dtype": dtype, "data": "synthetic", "config": config, "roofline": roof,
            "cpu_baseline": cpu}
    if extra:
        line.update(extra)
    print(json.dumps(line), flush=True)


def workload_ft_mul(pkg, torch, args, peak):
    """Plain batched ft_mul, W4 D4 (341 coefficients), FP64, batch 1024, U[-1,1]."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    W, D, B = 4, 4, 1024
    basis = pkg.TensorBasis(W, D)
    dim = basis.size()
    st = pkg.GB300Strategy(torch.float64)
    rng = np.random.default_rng(11)
    lhs_h, rhs_h = rng.uniform(-1, 1, (B, dim)), rng.uniform(-1, 1, (B, dim))
    lhs, rhs = torch.from_numpy(lhs_h).cuda(), torch.from_numpy(rhs_h).cuda()
    out = torch.empty(B, dim, dtype=torch.float64, device="cuda")
    mk = lambda t: pkg.make_tensor_batch(t, dim, 0, D)  # noqa: E731
    stream = torch.cuda.current_stream()
    ms_eager = 1e3 * _time_launches(torch, lambda: pkg.ft_mul(st, None, mk(out), mk(lhs), mk(rhs), basis, B),
                                    args.steps, args.warmup, stream)
    # A launch of 1024 small products is shorter than the host's call overhead,
    # so eager timing measures the gaps between enqueues: capture REPS launches
    # in a CUDA graph (the per-operation entry points allocate nothing) and
    # time its replays.
    REPS = 20
    cap = torch.cuda.Stream()
    cap.wait_stream(stream)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.stream(cap):
        cfg = pkg.DeviceLaunchConfig(cap)
        pkg.ft_mul(st, cfg, mk(out), mk(lhs), mk(rhs), basis, B).raise_if_failed()  # warm-up on the stream
        torch.cuda.synchronize()
        with torch.cuda.graph(graph, stream=cap):
            for _ in range(REPS):
                pkg.ft_mul(st, cfg, mk(out), mk(lhs), mk(rhs), basis, B)
    stream.wait_stream(cap)
    ms = 1e3 * _time_launches(torch, graph.replay, args.steps, args.warmup, stream) / REPS
    fma = sum((k + 1) * W ** k for k in range(D + 1))
    orc = O.Oracle()
    e = np.zeros((B, dim))
    t0 = time.perf_counter()
    orc.ft_mul(W, D, e, lhs_h, rhs_h, ((0, D), (0, D), (0, D)))
    cpu_s = time.perf_counter() - t0
    err = float(np.max(np.abs(out.cpu().numpy() - e) / np.maximum(1, np.abs(e))))
    _line("ft_mul products/sec (W4 D4 FP64, batch 1024)", B / (ms / 1e3), "products/s", ms, "f64",
          {"workload": "ft_mul_w4_d4_b1024", "fma_per_product": fma, "bytes_per_product": 3 * dim * 8},
          flops=2.0 * fma * B, peak=peak,
          cpu={"value": B / cpu_s, "unit": "products/s", "cores": 1, "kind": "port", "sample": f"{B} products"},
          extra={"parity": {"max_rel_err": err}, "timing": f"CUDA graph of {REPS} launches, replayed",
                 "eager_ms_per_launch": ms_eager})


def workload_logsig(pkg, torch, args, peak, W=5, D=5, B=4096, L=256, seed=3):
    """Log-signatures of B paths of L steps (W5 D5, 4096 x 256: 829 Lie
    coefficients, nnz 10 517; the large mixed shapes W2 D12 and W16 D3, 16 384
    x 64): the signature launch(es) under the tuner's forward-only schedule and
    the fused log-to-Lie epilogue (ft_log + tensor_to_lie in one kernel); the
    unfused ft_log and tensor_to_lie launches are timed beside it."""
    basis, lbasis = pkg.TensorBasis(W, D), pkg.LieBasis(W, D)
    dim, ts = basis.size(), lbasis.true_size()
    st = pkg.GB300Strategy(torch.float64)
    g = torch.Generator(device="cuda").manual_seed(seed)
    incr = torch.randn(B * L, W, dtype=torch.float64, device="cuda", generator=g) / np.sqrt(L)
    sig, log = (torch.empty(B, dim, dtype=torch.float64, device="cuda") for _ in range(2))
    lie = torch.empty(B, ts, dtype=torch.float64, device="cuda")
    t2l = pkg.make_t2l_matrix(lbasis)
    full = lambda t: pkg.make_tensor_batch(t, dim, 0, D)  # noqa: E731
    lieb = pkg.make_lie_batch(lie, ts, 1, D)

    err, schedule, _ = pkg.signature_tune(st, None, incr, basis, B, length=L, out=sig)
    err.raise_if_failed()

    def run():
        pkg.signature(st, None, incr, basis, B, length=L, out=sig).raise_if_failed()
        pkg.tensor_log_to_lie(st, None, lieb, full(sig), lbasis, basis, B, t2l).raise_if_failed()

    stream = torch.cuda.current_stream()
    ms = 1e3 * _time_launches(torch, run, args.steps, args.warmup, stream)
    ms_fused = 1e3 * _time_launches(torch, lambda: pkg.tensor_log_to_lie(st, None, lieb, full(sig), lbasis, basis,
                                                                         B, t2l), args.steps, args.warmup, stream)
    log_fma = sum(sum(k * W ** k for k in range(1, m + 1)) for m in range(1, D + 1))
    flops = 2.0 * B * (L * step_fma(W, D) + log_fma + t2l.nnz())
    ms_sig = 1e3 * _time_launches(torch, lambda: pkg.signature(st, None, incr, basis, B, length=L, out=sig),
                                  args.steps, args.warmup, stream)
    ms_log = 1e3 * _time_launches(torch, lambda: pkg.ft_log(st, None, full(log), full(sig), basis, B),
                                  args.steps, args.warmup, stream)
    ms_t2l = 1e3 * _time_launches(torch, lambda: pkg.tensor_to_lie(st, None, lieb, full(log), lbasis, basis, B, t2l),
                                  args.steps, args.warmup, stream)
    _line(f"log-signature paths/sec (W{W} D{D} L{L} FP64): signature + fused ft_log/tensor_to_lie", B / (ms / 1e3),
          "paths/s", ms, "f64", {"workload": f"logsig_w{W}_d{D}_l{L}_b{B}", "schedule": schedule,
                                 "lie_dim": ts - 1, "t2l_nnz": t2l.nnz()},
          flops=flops, peak=peak,
          extra={"signature_only_ms": ms_sig, "log_to_lie_fused_ms": ms_fused,
                 "log_to_lie_fused_roofline_frac": 2.0 * B * (log_fma + t2l.nnz()) / (ms_fused / 1e3) / 1e12 / peak
                 if peak else None,
                 "unfused_ft_log_ms": ms_log, "unfused_tensor_to_lie_ms": ms_t2l,
                 "ft_log_roofline_frac": 2.0 * B * log_fma / (ms_log / 1e3) / 1e12 / peak if peak else None,
                 "tensor_to_lie_roofline_frac": 2.0 * B * t2l.nnz() / (ms_t2l / 1e3) / 1e12 / peak
                 if peak else None})


def workload_lie_exp(pkg, torch, args, peak):
    """One log-ODE step per tensor, W5 D5, batch 4096, FP64: out = M (x) exp(l2t(lambda))
    through the fused kernel, and through lie_to_tensor + ft_fmexp (two launches)
    for comparison.  lambda ~ U[-0.3, 0.3] on the 828 Lie coefficients."""
    W, D, B = 5, 5, 4096
    basis, lbasis = pkg.TensorBasis(W, D), pkg.LieBasis(W, D)
    dim, ts = basis.size(), lbasis.true_size()
    st = pkg.GB300Strategy(torch.float64)
    g = torch.Generator(device="cuda").manual_seed(4)
    lam = (torch.rand(B, ts, dtype=torch.float64, device="cuda", generator=g) - 0.5) * 0.6
    mult = torch.rand(B, dim, dtype=torch.float64, device="cuda", generator=g) - 0.5
    out, x = (torch.empty(B, dim, dtype=torch.float64, device="cuda") for _ in range(2))
    l2t = pkg.make_l2t_matrix(lbasis)
    full = lambda t: pkg.make_tensor_batch(t, dim, 0, D)  # noqa: E731
    lb = pkg.make_lie_batch(lam, ts, 1, D)
    stream = torch.cuda.current_stream()
    ms = 1e3 * _time_launches(torch, lambda: pkg.lie_to_tensor_exp(st, None, full(out), full(mult), lb, basis, lbasis,
                                                                   B, l2t), args.steps, args.warmup, stream)

    def composed():
        pkg.lie_to_tensor(st, None, full(x), lb, basis, lbasis, B, l2t)
        pkg.ft_fmexp(st, None, full(out), full(mult), full(x), basis, B)

    ms_c = 1e3 * _time_launches(torch, composed, args.steps, args.warmup, stream)
    # fmexp: for d = D..1, out = M + out (x) X/d with X truncated to degrees 1..D-d+1
    fm_fma = sum(min(n, D - d + 1) * W ** n for d in range(1, D + 1) for n in range(1, D + 1))
    flops = 2.0 * B * (fm_fma + l2t.nnz())
    _line("Lie-increment exp steps/sec (W5 D5 FP64, batch 4096): fused lie_to_tensor + ft_fmexp",
          B / (ms / 1e3), "steps/s", ms, "f64", {"workload": "lie_exp_w5_d5_b4096"}, flops=flops, peak=peak,
          extra={"composed_ms": ms_c, "fused_over_composed": ms_c / ms})


def _graph_of(torch, fn):
    """A CUDA graph of fn's launches (captured on a side stream)."""
    stream = torch.cuda.Stream()
    fn()
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    stream.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(stream):
        with torch.cuda.graph(graph, stream=stream):
            fn()
    torch.cuda.current_stream().wait_stream(stream)
    torch.cuda.synchronize()
    return graph


def _best_group(pkg, torch, candidates):
    """The fastest (jobs, schedule) of a grouped launch, timed like the tuner
    (CUDA events, a warm-up call first)."""
    best = None
    for jobs, sched in candidates:
        if not pkg.signature_group(None, jobs, schedule=sched):
            continue
        ms = _time_launches(torch, lambda: pkg.signature_group(None, jobs, schedule=sched), 2, 1,
                            torch.cuda.current_stream())
        if best is None or ms < best[2]:
            best = (jobs, sched, ms)
    return best


def workload_ragged(pkg, torch, args, peak):
    """10,000 paths, lengths U{16..2048}, W8 D4, N(0, 1/len), run once in FP64
    and once in FP32: ONE persistent launch for both precisions
    (rpp_gb_signature_group) replayed from a CUDA graph; beside it the two
    tuned separate launches replayed from one graph."""
    W, D, B = 8, 4, 10_000
    rng = np.random.default_rng(2024)
    lengths = rng.integers(16, 2049, B)
    offsets = np.concatenate([[0], np.cumsum(lengths)]).astype(np.int64)
    incr_h = rng.normal(0, 1, (offsets[-1], W)) / np.sqrt(np.repeat(lengths, lengths))[:, None]
    basis = pkg.TensorBasis(W, D)
    dim = basis.size()
    off_d = torch.from_numpy(offsets).cuda()
    x64 = torch.from_numpy(incr_h).cuda()
    x32 = x64.float()
    st64, st32 = pkg.GB300Strategy(torch.float64), pkg.GB300Strategy(torch.float32)
    s64 = torch.empty(B, dim, dtype=torch.float64, device="cuda")
    s32 = torch.empty(B, dim, dtype=torch.float32, device="cuda")
    t64 = pkg.signature_tune(st64, None, x64, basis, B, offsets=off_d, out=s64)
    t32 = pkg.signature_tune(st32, None, x32, basis, B, offsets=off_d, out=s32)
    t64[0].raise_if_failed()
    t32[0].raise_if_failed()
    cur = torch.cuda.current_stream()
    ms64 = 1e3 * _time_launches(torch, lambda: pkg.signature(st64, None, x64, basis, B, offsets=off_d, out=s64),
                                args.steps, args.warmup, cur)
    ms32 = 1e3 * _time_launches(torch, lambda: pkg.signature(st32, None, x32, basis, B, offsets=off_d, out=s32),
                                args.steps, args.warmup, cur)
    sep = _graph_of(torch, lambda: (pkg.signature(st64, None, x64, basis, B, offsets=off_d, out=s64),
                                    pkg.signature(st32, None, x32, basis, B, offsets=off_d, out=s32)))
    ms_sep = 1e3 * _time_launches(torch, sep.replay, args.steps, args.warmup, cur)
    # the grouped launch: team sizes from the tuned separate launches, and a
    # few alternatives; CTA sizes 640 / 512
    cands = []
    # (team size 0 for the FP32 job: one warp per first letter)
    for th64, th32 in {(t64[1] & 1023, 0), (128, 0), (256, 0), (t64[1] & 1023, t32[1] & 1023), (128, 128),
                       (128, 64), (256, 128)}:
        jobs = [pkg.SignatureJob(st64, x64, basis, B, offsets=off_d, out=s64, threads=th64),
                pkg.SignatureJob(st32, x32, basis, B, offsets=off_d, out=s32, threads=th32)]
        for cta in (640, 512):
            cands.append((jobs, cta))
    jobs, sched, _ = _best_group(pkg, torch, cands)
    graph = _graph_of(torch, lambda: pkg.signature_group(None, jobs, schedule=sched).raise_if_failed())
    ms = 1e3 * _time_launches(torch, graph.replay, args.steps, args.warmup, cur)
    # each job alone in the grouped kernel (its code and team layout against
    # its own tuned launch)
    alone = [1e3 * _time_launches(torch, lambda j=j: pkg.signature_group(None, [j], schedule=sched), args.steps,
                                  args.warmup, cur) for j in jobs]
    err32 = float(torch.max(torch.abs(s32.double() - s64) / torch.clamp(s64.abs(), min=1.0)).item())
    steps_total = int(offsets[-1])
    flops64 = 2.0 * steps_total * step_fma(W, D)
    _line("uneven-length signatures paths/sec (W8 D4, 10k paths, L~U[16,2048]), FP64 + FP32 in one launch",
          B / (ms / 1e3), "paths/s", ms, "f64+f32",
          {"workload": "ragged_w8_d4_b10000", "total_increments": steps_total,
           "graph": "one grouped launch (an FP64 job and an FP32 job)", "group_cta_threads": sched,
           "group_team_threads": {"f64": jobs[0].arg.threads, "f32": jobs[1].arg.threads},
           "schedule": {"f64": t64[1], "f32": t32[1]}},
          extra={"gpu_launches": 2, "separate_launches_ms": ms_sep, "group_over_separate": ms_sep / ms,
                 "group_fp64_job_alone_ms": alone[0], "group_fp32_job_alone_ms": alone[1],
                 "fp64_ms": ms64, "fp32_ms": ms32, "fp64_paths_per_s": B / (ms64 / 1e3),
                 "fp32_paths_per_s": B / (ms32 / 1e3), "fp32_max_rel_err_vs_fp64": err32,
                 "fp64_roofline_frac": flops64 / (ms64 / 1e3) / 1e12 / peak if peak else None,
                 "fp32_tflops": 2.0 * steps_total * step_fma(W, D) / (ms32 / 1e3) / 1e12})


def workload_ragged_fp32(pkg, torch, args, peak):
    """The FP32 half of the uneven-length workload on its own: W8 D4 forward,
    lengths U{16..2048} (the first --batch paths of the 10,000; default all),
    tuned unless --schedule pins a schedule."""
    W, D = 8, 4
    B = 10_000 if args.batch == BATCH else args.batch
    rng = np.random.default_rng(2024)
    lengths = rng.integers(16, 2049, 10_000)[:B]
    offsets = np.concatenate([[0], np.cumsum(lengths)]).astype(np.int64)
    incr_h = rng.normal(0, 1, (offsets[-1], W)) / np.sqrt(np.repeat(lengths, lengths))[:, None]
    basis = pkg.TensorBasis(W, D)
    off_d = torch.from_numpy(offsets).cuda()
    x32 = torch.from_numpy(incr_h).cuda().float()
    st32 = pkg.GB300Strategy(torch.float32)
    s32 = torch.empty(B, basis.size(), dtype=torch.float32, device="cuda")
    sched = args.schedule
    if sched is None:
        err, sched, _ = pkg.signature_tune(st32, None, x32, basis, B, offsets=off_d, out=s32)
        err.raise_if_failed()
    ms = 1e3 * _time_launches(torch, lambda: pkg.signature(st32, None, x32, basis, B, offsets=off_d, out=s32,
                                                           schedule=sched).raise_if_failed(),
                              args.steps, args.warmup, torch.cuda.current_stream())
    flops = 2.0 * int(offsets[-1]) * step_fma(W, D)
    _line("uneven-length signatures paths/sec (W8 D4, L~U[16,2048], FP32 forward)", B / (ms / 1e3), "paths/s", ms,
          "f32", {"workload": f"ragged_fp32_w8_d4_b{B}", "schedule": sched, "total_increments": int(offsets[-1])},
          extra={"fp32_tflops": flops / (ms / 1e3) / 1e12})


def workload_mixed(pkg, torch, args, peak):
    """The large mixed-shape configuration: 16,384 paths of 64 increments
    N(0, 1/64) at width 2 / depth 12 and 16,384 at width 16 / depth 3, FP64,
    forward + reverse: ONE persistent launch for both shapes
    (rpp_gb_signature_group) replayed from a CUDA graph, beside the two tuned
    separate calls replayed from one graph."""
    B, L = 16_384, 64
    cur = torch.cuda.current_stream()
    st = pkg.GB300Strategy(torch.float64)
    parts, fma_total = [], 0
    for W, D in ((2, 12), (16, 3)):
        basis = pkg.TensorBasis(W, D)
        dim = basis.size()
        g = torch.Generator(device="cuda").manual_seed(W * 100 + D)
        incr = torch.randn(B * L, W, dtype=torch.float64, device="cuda", generator=g) / np.sqrt(L)
        ell = torch.rand(B, dim, dtype=torch.float64, device="cuda", generator=g) * 2 - 1
        sig = torch.empty(B, dim, dtype=torch.float64, device="cuda")
        grad = torch.empty_like(incr)
        err, threads, _ = pkg.signature_tune(st, None, incr, basis, B, length=L, out=sig, seed=ell, grad=grad)
        err.raise_if_failed()
        parts.append((basis, incr, ell, sig, grad, threads))
        fma_total += 4 * L * step_fma(W, D) * B

    def separate():
        for basis, incr, ell, sig, grad, _ in parts:
            pkg.signature(st, None, incr, basis, B, length=L, out=sig, seed=ell, grad=grad).raise_if_failed()

    sep = _graph_of(torch, separate)
    ms_sep = 1e3 * _time_launches(torch, sep.replay, args.steps, args.warmup, cur)
    cands = []
    # the deep job's team size, with its cotangent arrays in shared memory or
    # (bit 26) in a global workspace, as its tuned separate call may have them
    for t_deep in (256, 384, 512, 256 | (1 << 26), 320 | (1 << 26), 512 | (1 << 26)):
        jobs = [pkg.SignatureJob(st, incr, basis, B, length=L, out=sig, seed=ell, grad=grad,
                                 threads=t_deep if basis.width == 2 else 128)
                for basis, incr, ell, sig, grad, _ in parts]
        for sched in (640, 512, 640 | (1 << 27), 512 | (1 << 27)):
            cands.append((jobs, sched))
    jobs, sched, _ = _best_group(pkg, torch, cands)
    graph = _graph_of(torch, lambda: pkg.signature_group(None, jobs, schedule=sched).raise_if_failed())
    ms = 1e3 * _time_launches(torch, graph.replay, args.steps, args.warmup, cur)
    alone = [1e3 * _time_launches(torch, lambda j=j: pkg.signature_group(None, [j], schedule=sched), args.steps,
                                  args.warmup, cur) for j in jobs]
    sep_alone = [1e3 * _time_launches(torch, lambda p=p: pkg.signature(st, None, p[1], p[0], B, length=L, out=p[3],
                                                                       seed=p[2], grad=p[4]),
                                      args.steps, args.warmup, cur) for p in parts]
    _line("mixed-shape signature fwd+bwd paths/sec (W2 D12 + W16 D3, 2 x 16,384 paths, L64, FP64) in one launch",
          2 * B / (ms / 1e3), "paths/s", ms, "f64",
          {"workload": "mixed_w2d12_w16d3_b16384_l64", "group_schedule": sched,
           "group_team_threads": [j.arg.threads for j in jobs], "separate_schedules": [p[5] for p in parts]},
          flops=2.0 * fma_total, peak=peak,
          extra={"gpu_launches": 2, "separate_launches_ms": ms_sep, "group_over_separate": ms_sep / ms,
                 "group_job_alone_ms": {"w2d12": alone[0], "w16d3": alone[1]},
                 "separate_alone_ms": {"w2d12": sep_alone[0], "w16d3": sep_alone[1]}})


def workload_fp32(pkg, torch, args, peak):
    """The headline shape in FP32: W5 D5, L256, 4096 paths, forward + reverse
    (and forward only), against the FP32 FMA peak measured in the same run
    (rpp_gb_fma_peak, FP32) and the FP64 oracle (1e-5)."""
    import ctypes
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    W, D, B, L = WIDTH, DEPTH, args.batch, LENGTH
    out = ctypes.c_double(0)
    peak32 = out.value if pkg.library().rpp_gb_fma_peak(0, 0, ctypes.byref(out)) == 0 else None
    basis = pkg.TensorBasis(W, D)
    dim = basis.size()
    st = pkg.GB300Strategy(torch.float32)
    g = torch.Generator(device="cuda").manual_seed(5)
    incr64 = torch.randn(B * L, W, dtype=torch.float64, device="cuda", generator=g) / np.sqrt(L)
    ell64 = torch.rand(B, dim, dtype=torch.float64, device="cuda", generator=g) * 2 - 1
    incr, ell = incr64.float(), ell64.float()
    sig = torch.empty(B, dim, dtype=torch.float32, device="cuda")
    grad = torch.empty_like(incr)
    cur = torch.cuda.current_stream()
    lines = []
    for what, kw, fma in (("fwd+bwd", {"seed": ell, "grad": grad}, 4 * step_fma(W, D)),
                          ("forward", {}, step_fma(W, D))):
        if args.schedule is not None:  # a pinned schedule (profiling captures)
            threads = args.schedule
            kw = dict(kw, schedule=threads)
        else:
            err, threads, _ = pkg.signature_tune(st, None, incr, basis, B, length=L, out=sig, **kw)
            err.raise_if_failed()
        ms = 1e3 * _time_launches(
            torch, lambda: pkg.signature(st, None, incr, basis, B, length=L, out=sig, **kw).raise_if_failed(),
            args.steps, args.warmup, cur)
        flops = 2.0 * fma * L * B
        n = 3
        esig, egrad = O.Oracle().signature(W, D, incr64[:n * L].cpu().numpy(), np.arange(n + 1) * L,
                                           ell=ell64[:n].cpu().numpy() if "seed" in kw else None)
        err_sig = float(np.max(np.abs(sig[:n].double().cpu().numpy() - esig) / np.maximum(1, np.abs(esig))))
        extra = {"fp32_tflops": flops / (ms / 1e3) / 1e12, "fp32_peak_tflops": peak32,
                 "fp32_peak_frac": flops / (ms / 1e3) / 1e12 / peak32 if peak32 else None,
                 "max_rel_err_sig_vs_fp64_oracle": err_sig}
        if "seed" in kw:
            gg = grad[:n * L].double().cpu().numpy()
            extra["max_scaled_err_grad_vs_fp64_oracle"] = float(np.max(np.abs(gg - egrad)) /
                                                                max(1.0, float(np.max(np.abs(egrad)))))
        _line(f"signature {what} paths/sec (W{W} D{D} L{L} FP32)", B / (ms / 1e3), "paths/s", ms, "f32",
              {"workload": f"{what.replace('+', '_')}_w{W}_d{D}_l{L}_b{B}_fp32", "schedule": threads},
              extra=extra)


def workload_fwd_bwd(pkg, torch, args, peak, W, D, B, L, name):
    if args.batch != BATCH:  # an explicit --batch (profiling captures) replaces the workload's batch
        B = args.batch
        name = f"{name.rsplit('_b', 1)[0]}_b{B}"
    basis = pkg.TensorBasis(W, D)
    dim = basis.size()
    st = pkg.GB300Strategy(torch.float64)
    g = torch.Generator(device="cuda").manual_seed(W * 100 + D)
    incr = torch.randn(B * L, W, dtype=torch.float64, device="cuda", generator=g) / np.sqrt(L)
    ell = torch.rand(B, dim, dtype=torch.float64, device="cuda", generator=g) * 2 - 1
    sig = torch.empty(B, dim, dtype=torch.float64, device="cuda")
    grad = torch.empty_like(incr)
    if args.schedule is not None:  # a pinned schedule (profiling captures)
        threads = args.schedule
    else:
        err, threads, _ = pkg.signature_tune(st, None, incr, basis, B, length=L, out=sig, seed=ell, grad=grad)
        err.raise_if_failed()
    ms = 1e3 * _time_launches(
        torch, lambda: pkg.signature(st, None, incr, basis, B, length=L, out=sig, seed=ell, grad=grad,
                                     schedule=args.schedule).raise_if_failed(),
        args.steps, args.warmup, torch.cuda.current_stream())
    _line(f"signature fwd+bwd paths/sec (W{W} D{D} L{L} FP64)", B / (ms / 1e3), "paths/s", ms, "f64",
          {"workload": name, "batch": B, "length": L, "schedule": threads, "threads_per_cta": threads & 1023,
           "ctas_per_sm_cap": (threads >> 10) & 15, "two_launches": bool(threads & (1 << 14)),
           "top_level_in_global": bool(threads & (1 << 15)),
           "cotangent_in_global": bool(threads & (1 << 26)), "d_barrier_reverse": bool(threads & (1 << 27)),
           "cluster_ctas_per_path": ((threads >> 28) & 7) + 1},
          flops=2.0 * 4 * L * step_fma(W, D) * B, peak=peak)


def workload_adjoints(pkg, torch, args, peak, W, D, B):
    """Left and right adjoint multiplies by a random depth-truncated tensor."""
    basis = pkg.TensorBasis(W, D)
    dim = basis.size()
    st = pkg.GB300Strategy(torch.float64)
    g = torch.Generator(device="cuda").manual_seed(5)
    op, arg = (torch.rand(B, dim, dtype=torch.float64, device="cuda", generator=g) - 0.5 for _ in range(2))
    out = torch.empty_like(op)
    mk = lambda t: pkg.make_tensor_batch(t, dim, 0, D)  # noqa: E731
    stream = torch.cuda.current_stream()
    ms_l = 1e3 * _time_launches(torch, lambda: pkg.ft_adj_lmul(st, None, mk(out), mk(op), mk(arg), basis, B),
                                args.steps, args.warmup, stream)
    ms_r = 1e3 * _time_launches(torch, lambda: pkg.ft_adj_rmul(st, None, mk(out), mk(op), mk(arg), basis, B),
                                args.steps, args.warmup, stream)
    fma = sum(W ** m * W ** p for m in range(D + 1) for p in range(D + 1 - m))
    _line(f"adjoint multiplies/sec (W{W} D{D} FP64, batch {B})", B / (ms_l / 1e3), "products/s", ms_l, "f64",
          {"workload": f"adj_lmul_w{W}_d{D}_b{B}", "fma_per_product": fma}, flops=2.0 * fma * B, peak=peak,
          extra={"adj_rmul_ms": ms_r, "adj_rmul_products_per_s": B / (ms_r / 1e3)})


def _binom(n, k):
    c = 1
    for i in range(1, k + 1):
        c = c * (n - k + i) // i
    return c


def shuffle_terms(W, D):
    """Algorithmic FMAs per tensor of each shuffle operation over full degree
    ranges: one per (output coefficient, term) of the reference's sums."""
    st = sum((2 * W) ** n for n in range(D + 1))
    half = sum(W ** n * 2 ** (n - 1) for n in range(1, D + 1))
    adj = sum(W ** n * _binom(n + m, m) * W ** m for n in range(D + 1) for m in range(D - n + 1))
    hl = sum(W ** n * W * _binom(n + m, m) * W ** m for n in range(D) for m in range(D - n))
    hr = sum(W ** n * _binom(n - 1 + m, m) * W ** m for n in range(1, D + 1) for m in range(D - n + 1))
    return {"st_mul": st, "left_hs_mul": half, "st_adj_mul": adj, "left_hs_adj_lmul": hl, "left_hs_adj_rmul": hr}


def workload_shuffle(pkg, torch, args, peak):
    """Shuffle-algebra products and adjoints, W5 D5, batch 4096, FP64, U[-1/2,1/2]
    operands (2 x 128 MB in, 128 MB out per launch: above L2), plus
    tensor_pairing (HBM-bound)."""
    W, D, B = 5, 5, 4096
    basis = pkg.TensorBasis(W, D)
    dim = basis.size()
    st = pkg.GB300Strategy(torch.float64)
    g = torch.Generator(device="cuda").manual_seed(17)
    x, y = (torch.rand(B, dim, dtype=torch.float64, device="cuda", generator=g) - 0.5 for _ in range(2))
    out = torch.empty_like(x)
    mk = lambda t: pkg.make_tensor_batch(t, dim, 0, D)  # noqa: E731
    stream = torch.cuda.current_stream()
    terms = shuffle_terms(W, D)
    for name in ("st_mul", "left_hs_mul", "st_adj_mul", "left_hs_adj_lmul", "left_hs_adj_rmul"):
        fn = getattr(pkg, name)
        ms = 1e3 * _time_launches(torch, lambda: fn(st, None, mk(out), mk(x), mk(y), basis, B), args.steps,
                                  args.warmup, stream)
        _line(f"{name} products/sec (W5 D5 FP64, batch 4096)", B / (ms / 1e3), "products/s", ms, "f64",
              {"workload": f"{name}_w5_d5_b4096", "fma_per_product": terms[name]},
              flops=2.0 * terms[name] * B, peak=peak)
    res = torch.empty(B, dtype=torch.float64, device="cuda")
    ms = 1e3 * _time_launches(torch, lambda: pkg.tensor_pairing(st, None, pkg.make_scalar_batch(res), mk(x), mk(y),
                                                                basis, B), args.steps, args.warmup, stream)
    nbytes = 2 * dim * 8 * B + 8 * B
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            hbm = float(json.load(f)["hbm_gbs"])
        src = "MEASURED_PEAKS.json hbm_gbs"
    except (OSError, KeyError, ValueError):
        hbm, src = 6800.0, "fallback"
    ach = nbytes / (ms / 1e3) / 1e9
    print(json.dumps({"metric": "tensor_pairing pairs/sec (W5 D5 FP64, batch 4096)", "value": B / (ms / 1e3),
                      "unit": "pairs/s", "n_gpus": 1, "ms_per_step": ms, "higher_is_better": True, "dtype": "f64",
                      "data": "synthetic", "config": {"workload": "tensor_pairing_w5_d5_b4096",
                                                      "bytes_per_pair": 2 * dim * 8 + 8},
                      "roofline": {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s",
                                   "frac": ach / hbm, "traffic": None, "peak_source": src}}), flush=True)


def run_workloads(args):
    import torch

    torch.cuda.set_device(0)
    pkg = importlib.import_module("rough-path-primitives_gb300")
    peak = _fp64_peak(pkg, 0)
    todo = args.workload.split(",")
    if "all" in todo:
        todo = ["ft_mul", "logsig", "lie_exp", "ragged", "w6d6", "w2d12", "w16d3", "mixed", "logsig_mixed", "fp32",
                "adjoints", "shuffle"]
    for w in todo:
        if w == "ft_mul":
            workload_ft_mul(pkg, torch, args, peak)
        elif w == "logsig":
            workload_logsig(pkg, torch, args, peak)
        elif w == "logsig_mixed":  # the large mixed shapes' log-signatures
            workload_logsig(pkg, torch, args, peak, 2, 12, 16384, 64, seed=12)
            workload_logsig(pkg, torch, args, peak, 16, 3, 16384, 64, seed=16)
        elif w == "ragged":
            workload_ragged(pkg, torch, args, peak)
        elif w == "w6d6":
            workload_fwd_bwd(pkg, torch, args, peak, 6, 6, 512, 128, "fwd_bwd_w6_d6_l128_b512")
        elif w == "w2d12":
            workload_fwd_bwd(pkg, torch, args, peak, 2, 12, 16384, 64, "fwd_bwd_w2_d12_l64_b16384")
        elif w == "w16d3":
            workload_fwd_bwd(pkg, torch, args, peak, 16, 3, 16384, 64, "fwd_bwd_w16_d3_l64_b16384")
        elif w == "mixed":
            workload_mixed(pkg, torch, args, peak)
        elif w == "fp32":
            workload_fp32(pkg, torch, args, peak)
        elif w == "ragged_fp32":
            workload_ragged_fp32(pkg, torch, args, peak)
        elif w == "lie_exp":
            workload_lie_exp(pkg, torch, args, peak)
        elif w == "shuffle":
            workload_shuffle(pkg, torch, args, peak)
        elif w == "adjoints":
            workload_adjoints(pkg, torch, args, peak, 2, 12, 16384)
            workload_adjoints(pkg, torch, args, peak, 16, 3, 16384)
        else:
            raise SystemExit(f"unknown workload {w}")


def run_reference_arm(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return
    base = cpu_reference(args.steps, args.warmup, world, rank)
    line = {
        "impl": "reference", "metric": METRIC, "value": base["value"], "unit": "paths/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": base["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": headline_config(args.batch, world),
        "cpu_baseline": {k: base[k] for k in ("value", "unit", "cores", "kind", "sample")},
        "e2e": {"value": base["value"], "unit": "paths/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain per-operation GPU comparator")
    ap.add_argument("--batch", type=int, default=BATCH,
                    help="paths per GPU (default: the headline 4096; smaller only for profiling captures)")
    ap.add_argument("--schedule", type=int, default=None,
                    help="pin the signature schedule (rpp_gb_signature_tune's encoding) instead of tuning; "
                         "for profiling captures")
    ap.add_argument("--workload", default=None,
                    help="other configurations instead of the headline: ft_mul, logsig, ragged, w6d6, w2d12, "
                         "w16d3, mixed, fp32, ragged_fp32, adjoints, shuffle, lie_exp or all (comma-separated)")
    args = ap.parse_args()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        # one process per GPU: relaunch this command under torch.distributed.run
        import socket

        with socket.socket() as sock:
            sock.bind(("127.0.0.1", 0))
            port = sock.getsockname()[1]
        cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={args.gpus}",
               "--master-addr=127.0.0.1", f"--master-port={port}", os.path.abspath(__file__)] + sys.argv[1:]
        raise SystemExit(subprocess.call(cmd))
    if args.impl == "reference":
        run_reference_arm(args)
        return
    if args.workload:
        run_workloads(args)
        return

    import torch

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    pkg = importlib.import_module("rough-path-primitives_gb300")
    dev = torch.device("cuda", local)
    basis = pkg.TensorBasis(WIDTH, DEPTH)
    dim = basis.size()
    strat = pkg.GB300Strategy(torch.float64, local)

    # measured FP64 FMA peak (roofline denominator)
    peak = (torch.zeros(1, dtype=torch.float64).numpy()).copy()
    import ctypes

    lib = pkg.library()
    rc = lib.rpp_gb_fma_peak(1, local, peak.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    fp64_peak = float(peak[0]) if rc == 0 else None

    batch = args.batch
    incr_h, ell_h = make_inputs(1000 + rank, batch)
    incr = torch.from_numpy(incr_h).to(dev)
    ell = torch.from_numpy(ell_h).to(dev)
    sig = torch.empty(batch, dim, dtype=torch.float64, device=dev)
    grad = torch.empty_like(incr)
    stream = torch.cuda.current_stream(dev)
    cfg = pkg.DeviceLaunchConfig(stream)

    pinned = args.schedule

    def step():
        pkg.signature(strat, cfg, incr, basis, batch, length=LENGTH, out=sig, seed=ell, grad=grad,
                      schedule=pinned).raise_if_failed()

    if pinned is None:
        # autotune the schedule on this workload (part of the warm-up)
        terr, tuned_threads, tuned_ms = pkg.signature_tune(strat, cfg, incr, basis, batch, length=LENGTH, out=sig,
                                                           seed=ell, grad=grad)
        terr.raise_if_failed()
    else:
        tuned_threads = pinned
    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    per_launch = []
    torch.cuda.synchronize()
    # an NVTX range marks the timed launches (a profiler can select them:
    # ncu --nvtx --nvtx-include "timed_region/")
    nvtx = getattr(torch.cuda, "nvtx", None)
    try:
        nvtx.range_push("timed_region")
    except Exception:  # NVTX unavailable: the range is only a profiling aid
        nvtx = None
    e0.record(stream)
    for _ in range(args.steps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        step()
        b.record(stream)
        per_launch.append((a, b))
    e1.record(stream)
    torch.cuda.synchronize()
    if nvtx is not None:
        nvtx.range_pop()
    clk = clocks.stop()
    elapsed = e0.elapsed_time(e1) / 1e3
    launch_ms = [a.elapsed_time(b) for a, b in per_launch]
    if world > 1:
        t = torch.tensor([elapsed], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        elapsed = float(t.item())
    value = world * batch * args.steps / elapsed

    # end to end through the public API with host buffers: rpp_gb_signature_host
    # copies each step's increments and seeds in from pinned host memory and the
    # signatures and gradients back out, in two chunks whose copies overlap the
    # other chunk's kernels (the schedule recorded by the tuner above)
    incr_p = torch.from_numpy(incr_h).pin_memory()
    ell_p = torch.from_numpy(ell_h).pin_memory()
    sig_p = torch.empty(batch, dim, dtype=torch.float64).pin_memory()
    grad_p = torch.empty(incr_h.shape, dtype=torch.float64).pin_memory()

    incr_d, ell_d = torch.empty_like(incr), torch.empty_like(ell)

    def e2e_step():
        if pinned is None:
            pkg.signature_host(strat, cfg, incr_p, basis, batch, length=LENGTH, out=sig_p, seed=ell_p,
                               grad=grad_p).raise_if_failed()
            return
        # a pinned schedule (profiling runs): the same copies in series around
        # the device call, so the e2e launches use that schedule too
        incr_d.copy_(incr_p, non_blocking=True)
        ell_d.copy_(ell_p, non_blocking=True)
        pkg.signature(strat, cfg, incr_d, basis, batch, length=LENGTH, out=sig, seed=ell_d, grad=grad,
                      schedule=pinned).raise_if_failed()
        sig_p.copy_(sig, non_blocking=True)
        grad_p.copy_(grad, non_blocking=True)

    for _ in range(2):
        e2e_step()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    e0.record(stream)
    for _ in range(args.steps):
        e2e_step()
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_elapsed = e0.elapsed_time(e1) / 1e3
    if world > 1:
        t = torch.tensor([e2e_elapsed], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_elapsed = float(t.item())
    e2e_value = world * batch * args.steps / e2e_elapsed

    # the plain per-operation GPU path on the same inputs
    plain = None
    if not args.no_plain:
        plain_grad = torch.empty_like(incr)
        psig = plain_path(pkg, strat, cfg, basis, incr, ell, batch, plain_grad)  # warm-up
        torch.cuda.synchronize()
        p_times = []
        for _ in range(2):
            e0.record(stream)
            psig = plain_path(pkg, strat, cfg, basis, incr, ell, batch, plain_grad)
            e1.record(stream)
            torch.cuda.synchronize()
            p_times.append(e0.elapsed_time(e1) / 1e3)
        p_s = statistics.mean(p_times)
        agree = float(torch.max(torch.abs(plain_grad - grad) / torch.clamp(torch.abs(grad), min=1.0)).item())
        agree_sig = float(torch.max(torch.abs(psig - sig) / torch.clamp(torch.abs(sig), min=1.0)).item())
        plain = {"value": batch / p_s, "unit": "paths/s", "ms_per_step": 1e3 * p_s,
                 "launches_per_step": 1 + LENGTH + 4 * LENGTH,
                 "kernels": "ft_fmexp x L (stored prefixes), then per increment ft_exp, ft_adj_lmul, "
                            "exp VJP, ft_adj_rmul",
                 "max_rel_diff_vs_fused": {"sig": agree_sig, "grad": agree}}
        del plain_grad, psig
        torch.cuda.empty_cache()

    # the reference's own plain per-operation GPU path (its BlockStrategy) on
    # the same inputs
    plain_ref = None
    ref_lib = None if args.no_plain else _ref_block_lib()
    if ref_lib is not None:
        ref_grad = torch.empty_like(incr)
        xpad = torch.zeros(incr.numel() + 1, dtype=torch.float64, device=dev)
        xpad[1:].copy_(incr.reshape(-1))
        rsig = plain_reference_path(ref_lib, pkg, strat, cfg, basis, xpad, incr, ell, batch, ref_grad, stream)
        torch.cuda.synchronize()
        r_times = []
        for _ in range(2):
            e0.record(stream)
            rsig = plain_reference_path(ref_lib, pkg, strat, cfg, basis, xpad, incr, ell, batch, ref_grad, stream)
            e1.record(stream)
            torch.cuda.synchronize()
            r_times.append(e0.elapsed_time(e1) / 1e3)
        r_s = statistics.mean(r_times)
        agree = float(torch.max(torch.abs(ref_grad - grad) / torch.clamp(torch.abs(grad), min=1.0)).item())
        agree_sig = float(torch.max(torch.abs(rsig - sig) / torch.clamp(torch.abs(sig), min=1.0)).item())
        plain_ref = {"value": batch / r_s, "unit": "paths/s", "ms_per_step": 1e3 * r_s,
                     "launches_per_step": 1 + LENGTH + 4 * LENGTH,
                     "kernels": "the reference's BlockStrategy<double, 128, 256> (its gpu/block operations, "
                                "compiled from its headers for sm_103a): ft_fmexp x L (stored prefixes), then per "
                                "increment ft_exp, ft_adj_lmul, ft_adj_rmul; the exp VJP (no reference "
                                "operation) is this repository's kernel",
                     "max_rel_diff_vs_fused": {"sig": agree_sig, "grad": agree}}
        del ref_grad, rsig, xpad
        torch.cuda.empty_cache()

    # parity spot check of this run's output against the oracle (3 paths)
    if rank == 0:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O

        orc = O.Oracle()
        k = 3
        esig, egrad = orc.signature(WIDTH, DEPTH, incr_h[: k * LENGTH], np.arange(k + 1) * LENGTH, ell=ell_h[:k])
        s_err = float(np.max(np.abs(sig[:k].cpu().numpy() - esig) / np.maximum(1, np.abs(esig))))
        g_err = float(np.max(np.abs(grad[: k * LENGTH].cpu().numpy() - egrad) / np.maximum(1, np.abs(egrad))))

    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return

    fma_per_path = 4 * LENGTH * step_fma(WIDTH, DEPTH)
    flops_per_launch = 2.0 * fma_per_path * batch
    mean_launch_s = statistics.mean(launch_ms) / 1e3
    achieved = flops_per_launch / mean_launch_s / 1e12
    cpu = None if args.no_cpu_baseline else cpu_reference(2, 1, world, rank)
    h2d = incr_h.nbytes + ell_h.nbytes
    d2h = batch * dim * 8 + incr_h.nbytes
    line = {
        "metric": METRIC, "value": value, "unit": "paths/s", "n_gpus": world, "steps": args.steps,
        "warmup": max(3, args.warmup), "ms_per_step": 1e3 * elapsed / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": headline_config(batch, world),
        "kernel": ("fused forward+reverse: a forward launch and a reverse launch per step"
                   if tuned_threads & (1 << 14) else "fused forward+reverse, one launch per step"),
        "schedule": {"threads_per_cta": tuned_threads & 1023,
                     "ctas_per_sm_cap": (tuned_threads >> 10) & 15,
                     "two_launches": bool(tuned_threads & (1 << 14)),
                     "forward_top_level_in_global": bool(tuned_threads & (1 << 15)),
                     "reverse_threads_per_cta": ((tuned_threads >> 16) & 1023) or (tuned_threads & 1023),
                     "cotangent_in_global": bool(tuned_threads & (1 << 26)),
                     "chosen_by": "rpp_gb_signature_tune" if pinned is None else "--schedule"},
        "roofline": {"bound": "fp64_fma", "achieved": achieved, "peak": fp64_peak, "unit": "TFLOP/s",
                     "frac": (achieved / fp64_peak) if fp64_peak else None,
                     "traffic": TWO_LAUNCH_TRAFFIC_BYTES if tuned_threads & (1 << 14) else None,
                     "traffic_unit": "DRAM bytes per step (both launches), ncu capture of the tuned two-launch schedule",
                     "peak_source": "measured in-run (rpp_gb_fma_peak, FP64 FMA chains)",
                     "algorithmic_flops_per_launch": flops_per_launch,
                     "fma_per_path": fma_per_path},
        "cpu_baseline": None if cpu is None else {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")},
        "e2e": {"value": e2e_value, "unit": "paths/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        # signature kernels in the timed region (two per step for the two-launch schedule)
        "gpu_launches": args.steps * (2 if tuned_threads & (1 << 14) else 1),
        "plain": plain,
        "fused_over_plain": (value / world) / plain["value"] if plain else None,
        "plain_reference": plain_ref,
        "fused_over_plain_reference": (value / world) / plain_ref["value"] if plain_ref else None,
        "clocks": clk,
        "parity": {"max_rel_err_sig": s_err, "max_rel_err_grad": g_err, "paths_checked": 3},
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
