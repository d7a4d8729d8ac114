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
region).  `--impl reference` times the CPU oracle (the reference algorithm
restated in C) on the host cores for a bounded sample of the same workload.
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


def cpu_reference(steps: int, warmup: int, world: int, rank: int):
    """CPU arm: the oracle's signature forward + stored-prefix reverse pass on
    all host cores, each step a bounded sample of the workload's paths."""
    if rank != 0:
        return None
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    orc = O.Oracle()
    cores = os.cpu_count() or 1
    sample = max(cores, 2 * cores)
    incr, ell = make_inputs(1234, sample)
    offs = np.arange(sample + 1, dtype=np.int64) * LENGTH
    for _ in range(max(0, warmup)):
        orc.signature(WIDTH, DEPTH, incr, offs, ell=ell, threads=cores)
    times = []
    for _ in range(steps):
        t0 = time.perf_counter()
        orc.signature(WIDTH, DEPTH, incr, offs, ell=ell, threads=cores)
        times.append(time.perf_counter() - t0)
    total = sum(times)
    return {"value": sample * steps / total, "unit": "paths/s", "cores": cores, "kind": "port",
            "sample": f"{sample} of the {BATCH} paths per step (W5 D5 L256 FP64 forward + stored-prefix reverse)",
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


def run_reference_arm(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return
    base = cpu_reference(args.steps, args.warmup, world, rank)
    line = {
        "impl": "reference", "metric": METRIC, "value": base["value"], "unit": "paths/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": base["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "signature_fwd_bwd_w5_d5_l256", "width": WIDTH, "depth": DEPTH, "batch": BATCH,
                   "length": LENGTH, "sample_paths_per_step": base["sample"]},
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
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference_arm(args)
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

    def step():
        pkg.signature(strat, cfg, incr, basis, batch, length=LENGTH, out=sig, seed=ell, grad=grad).raise_if_failed()

    # autotune the CTA size on this workload (part of the warm-up)
    terr, tuned_threads, tuned_ms = pkg.signature_tune(strat, cfg, incr, basis, batch, length=LENGTH, out=sig,
                                                       seed=ell, grad=grad)
    terr.raise_if_failed()
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
    e0.record(stream)
    for _ in range(args.steps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        step()
        b.record(stream)
        per_launch.append((a, b))
    e1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    elapsed = e0.elapsed_time(e1) / 1e3
    launch_ms = [a.elapsed_time(b) for a, b in per_launch]
    if world > 1:
        t = torch.tensor([elapsed], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        elapsed = float(t.item())
    value = world * batch * args.steps / elapsed

    # end to end through the public API with host buffers
    incr_p = torch.from_numpy(incr_h).pin_memory()
    ell_p = torch.from_numpy(ell_h).pin_memory()
    sig_p = torch.empty(batch, dim, dtype=torch.float64).pin_memory()
    grad_p = torch.empty(incr_h.shape, dtype=torch.float64).pin_memory()
    incr_d, ell_d = torch.empty_like(incr), torch.empty_like(ell)

    def e2e_step():
        incr_d.copy_(incr_p, non_blocking=True)
        ell_d.copy_(ell_p, non_blocking=True)
        pkg.signature(strat, cfg, incr_d, basis, batch, length=LENGTH, out=sig, seed=ell_d,
                      grad=grad).raise_if_failed()
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
        "config": {"workload": "signature_fwd_bwd_w5_d5_l256", "width": WIDTH, "depth": DEPTH,
                   "batch_per_gpu": batch, "length": LENGTH, "increments": "N(0,1/256) iid",
                   "seed_functional": "U[-1,1]", "l2": "inputs+outputs 340 MB > L2 (no flush needed)",
                   "kernel": "fused forward+reverse, one launch per step", "parallelism": f"replicas x{world}",
                   "schedule": {"threads_per_cta": tuned_threads, "chosen_by": "rpp_gb_signature_tune"}},
        "roofline": {"bound": "fp64_fma", "achieved": achieved, "peak": fp64_peak, "unit": "TFLOP/s",
                     "frac": (achieved / fp64_peak) if fp64_peak else None, "traffic": None,
                     "peak_source": "measured in-run (rpp_gb_fma_peak, FP64 FMA chains)",
                     "algorithmic_flops_per_launch": flops_per_launch,
                     "fma_per_path": fma_per_path},
        "cpu_baseline": None if cpu is None else {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")},
        "e2e": {"value": e2e_value, "unit": "paths/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": args.steps,
        "plain": plain,
        "fused_over_plain": (value / world) / plain["value"] if plain else None,
        "clocks": clk,
        "parity": {"max_rel_err_sig": s_err, "max_rel_err_grad": g_err, "paths_checked": 3},
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
