"""Several (width, depth) shapes and precisions in one persistent launch
(rpp_gb_signature_group): each job's outputs against the oracle and, bit for
bit, against a separate rpp_gb_signature call whose CTA size is the job's team
size (the team size fixes the order in which the letter gradients' partial
sums are added), the two mixed workloads of the benchmark configurations at
test size, several teams per CTA, a CUDA graph replay, and the refusals."""
import importlib

import numpy as np
import pytest

import oracle as O
from _helpers import TOL_F32, TOL_F64, assert_close, scaled_err

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

pkg = importlib.import_module("rough-path-primitives_gb300")


def make_job(rng, W, D, B, dtype, *, L=None, ragged=None, grad=True, sig=True, threads=0):
    if ragged is not None:
        lengths = rng.integers(ragged[0], ragged[1] + 1, B)
        offsets = np.concatenate([[0], np.cumsum(lengths)]).astype(np.int64)
        incr = rng.normal(0, 1, (int(offsets[-1]), W)) / np.sqrt(np.repeat(np.maximum(lengths, 1), lengths))[:, None]
    else:
        offsets = None
        incr = rng.normal(0, 1 / np.sqrt(L), (B * L, W))
    dim = O.tensor_dim(W, D)
    ell = rng.uniform(-1, 1, (B, dim)) if grad else None
    return {"W": W, "D": D, "B": B, "L": L, "dtype": dtype, "incr": incr, "offsets": offsets, "ell": ell,
            "sig": sig, "threads": threads, "basis": pkg.TensorBasis(W, D)}


def device_args(job):
    dt = job["dtype"]
    B, dim = job["B"], job["basis"].size()
    incr = torch.from_numpy(job["incr"]).to("cuda", dt)
    offs = None if job["offsets"] is None else torch.from_numpy(job["offsets"]).cuda()
    sig = torch.full((B, dim), float("nan"), dtype=dt, device="cuda") if job["sig"] else None
    seed = None if job["ell"] is None else torch.from_numpy(job["ell"]).to("cuda", dt)
    grad = None if seed is None else torch.full(incr.shape, float("nan"), dtype=dt, device="cuda")
    return incr, offs, sig, seed, grad


def as_job(job, args):
    incr, offs, sig, seed, grad = args
    return pkg.SignatureJob(pkg.GB300Strategy(job["dtype"]), incr, job["basis"], job["B"], length=job["L"],
                            offsets=offs, out=sig, seed=seed, grad=grad, threads=job["threads"])


def separate(job, args, schedule):
    incr, offs, sig, seed, grad = args
    err = pkg.signature(pkg.GB300Strategy(job["dtype"]), None, incr, job["basis"], job["B"], length=job["L"],
                        offsets=offs, out=sig, seed=seed, grad=grad, schedule=schedule)
    assert err, err.message


def check_oracle(orc, job, args):
    _, _, sig, _, grad = args
    W, D = job["W"], job["D"]
    offs = job["offsets"] if job["offsets"] is not None else np.arange(job["B"] + 1) * job["L"]
    esig, egrad = orc.signature(W, D, job["incr"], offs, ell=job["ell"])
    tol = TOL_F64 if job["dtype"] == torch.float64 else TOL_F32
    torch.cuda.synchronize()
    if sig is not None:
        assert_close(sig.double().cpu().numpy(), esig, tol, f"W{W} D{D} {job['dtype']} signature")
    if grad is not None:
        e = scaled_err(grad.double().cpu().numpy(), egrad)
        assert e <= tol, f"W{W} D{D} {job['dtype']} gradient: scaled error {e:.3e}"


def run_group_and_separate(orc, jobs, schedule=0):
    grouped = [device_args(j) for j in jobs]
    err = pkg.signature_group(None, [as_job(j, a) for j, a in zip(jobs, grouped)], schedule=schedule)
    assert err, err.message
    torch.cuda.synchronize()
    for j, a in zip(jobs, grouped):
        check_oracle(orc, j, a)
        alone = device_args(j)
        # a letter job (threads 0) against its kernel's explicit schedule
        separate(j, alone, (j["threads"] or (32 | (1 << 16))) | (schedule & (1 << 27)))
        torch.cuda.synchronize()
        for got, want in zip(a[2:], alone[2:]):
            if got is not None:
                assert torch.equal(got, want), f"W{j['W']} D{j['D']} {j['dtype']}: group differs from a separate call"


def test_mixed_shapes_forward_and_reverse(orc):
    """The large mixed-shape workload at test size: width 2 depth 12 (one
    team per CTA, top level in global memory) and width 16 depth 3 (several
    teams of 128 threads per CTA) in one launch, forward + reverse, FP64."""
    rng = np.random.default_rng(51)
    jobs = [make_job(rng, 2, 12, 24, torch.float64, L=16, threads=256),
            make_job(rng, 16, 3, 40, torch.float64, L=16, threads=128)]
    run_group_and_separate(orc, jobs)


def test_cotangent_workspace_jobs(orc):
    """FP64 forward + reverse jobs with bit 26 on their threads keep the
    cotangent level and chains in a per-team slice of a global workspace (the
    form the tuner picks for width 2 depth 12 as a separate call): outputs
    equal a separate call with that schedule bit for bit, beside a job in
    shared memory; ragged, with empty paths."""
    rng = np.random.default_rng(58)
    cot = 1 << 26
    jobs = [make_job(rng, 2, 12, 24, torch.float64, L=16, threads=256 | cot),
            make_job(rng, 16, 3, 40, torch.float64, L=16, threads=128),
            make_job(rng, 3, 4, 50, torch.float64, ragged=(0, 30), threads=128 | cot)]
    run_group_and_separate(orc, jobs)
    run_group_and_separate(orc, jobs, schedule=640 | (1 << 27))


def test_fp32_forward_reverse_jobs_take_letter_warps(orc):
    """FP32 forward + reverse jobs of an instantiated shape (depth >= 3) with
    threads = 0 run the warp-per-letter forward + reverse code inside the
    group (a team of W warps meeting on its named barrier for the letter
    gradients): outputs equal a separate call of that kernel bit for bit and
    the FP64 oracle within 1e-5; the family form (W5 D5), the row form (W8
    D4, ragged with empty paths), gradient-only (W3 D6), beside an FP64 job."""
    rng = np.random.default_rng(59)
    jobs = [make_job(rng, 5, 5, 12, torch.float32, L=20),
            make_job(rng, 8, 4, 30, torch.float32, ragged=(0, 30)),
            make_job(rng, 3, 6, 10, torch.float32, L=11, sig=False),
            make_job(rng, 5, 5, 9, torch.float64, L=13, threads=128)]
    run_group_and_separate(orc, jobs)


def test_fp64_and_fp32_ragged_forward(orc):
    """The uneven-length workload at test size: width 8 depth 4, lengths
    U{1..150}, one FP64 and one FP32 batch in one launch."""
    rng = np.random.default_rng(52)
    jobs = [make_job(rng, 8, 4, 120, torch.float64, ragged=(1, 150), grad=False, threads=128),
            make_job(rng, 8, 4, 120, torch.float32, ragged=(1, 150), grad=False, threads=128)]
    run_group_and_separate(orc, jobs)


@pytest.mark.parametrize("bits", [0, 1 << 27])
def test_four_jobs_gradient_only_and_team_sizes(orc, bits):
    """Four jobs of different team sizes (64 to 160 threads, so 2 to 8 teams
    per 512-thread CTA), one of them gradient-only, in both reverse-step
    forms; empty ragged paths included."""
    rng = np.random.default_rng(53)
    jobs = [make_job(rng, 5, 5, 30, torch.float64, L=24, threads=128),
            make_job(rng, 3, 4, 50, torch.float32, ragged=(0, 40), threads=64),
            make_job(rng, 4, 4, 20, torch.float64, L=12, sig=False, threads=160),
            make_job(rng, 7, 3, 9, torch.float64, L=5, threads=96)]
    run_group_and_separate(orc, jobs, schedule=512 | bits)


def test_fp32_forward_jobs_take_letter_warps(orc):
    """FP32 forward-only jobs of an instantiated shape with threads = 0 run with
    one warp per first letter inside the group; their outputs equal the
    shared-memory kernel's bit for bit (the same fused multiply-adds), beside
    an FP64 job in the same launch."""
    rng = np.random.default_rng(57)
    jobs = [make_job(rng, 8, 4, 90, torch.float32, ragged=(0, 70), grad=False),
            make_job(rng, 5, 5, 40, torch.float32, L=19, grad=False),
            make_job(rng, 8, 4, 60, torch.float64, ragged=(1, 50), grad=False, threads=128)]
    grouped = [device_args(j) for j in jobs]
    err = pkg.signature_group(None, [as_job(j, a) for j, a in zip(jobs, grouped)])
    assert err, err.message
    torch.cuda.synchronize()
    for j, a in zip(jobs, grouped):
        check_oracle(orc, j, a)
        alone = device_args(j)
        separate(j, alone, 128)
        torch.cuda.synchronize()
        assert torch.equal(a[2], alone[2]), f"W{j['W']} D{j['D']} {j['dtype']}: group differs from a separate call"


def test_default_team_sizes(orc):
    """threads = 0: each job takes its shape's heuristic CTA size."""
    rng = np.random.default_rng(56)
    jobs = [make_job(rng, 4, 4, 33, torch.float64, L=20), make_job(rng, 6, 3, 17, torch.float32, L=9)]
    grouped = [device_args(j) for j in jobs]
    err = pkg.signature_group(None, [as_job(j, a) for j, a in zip(jobs, grouped)])
    assert err, err.message
    for j, a in zip(jobs, grouped):
        check_oracle(orc, j, a)


def test_group_in_cuda_graph_replays_eager_results():
    rng = np.random.default_rng(54)
    jobs = [make_job(rng, 2, 12, 16, torch.float64, L=8, threads=256),
            make_job(rng, 8, 4, 64, torch.float32, ragged=(1, 60), threads=128)]
    args = [device_args(j) for j in jobs]
    gjobs = [as_job(j, a) for j, a in zip(jobs, args)]
    err = pkg.signature_group(None, gjobs)
    assert err, err.message
    torch.cuda.synchronize()
    outputs = lambda a: [t for t in (a[2], a[4]) if t is not None]  # noqa: E731  (sig, grad; not the seed)
    eager = [[t.clone() for t in outputs(a)] for a in args]
    stream = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()
    stream.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(stream):
        cfg = pkg.DeviceLaunchConfig(stream)
        with torch.cuda.graph(graph, stream=stream):
            pkg.signature_group(cfg, gjobs).raise_if_failed()
    torch.cuda.current_stream().wait_stream(stream)
    torch.cuda.synchronize()
    for a in args:
        for t in outputs(a):
            t.fill_(float("nan"))
    graph.replay()
    torch.cuda.synchronize()
    for a, e in zip(args, eager):
        for t, want in zip(outputs(a), e):
            assert torch.equal(t, want)


def test_group_refusals():
    lib = pkg.library()
    rng = np.random.default_rng(55)
    big = make_job(rng, 6, 6, 2, torch.float64, L=4, threads=512)
    err = pkg.signature_group(None, [as_job(big, device_args(big))])
    assert not err and err.code == pkg.ErrorCode.NotImplemented
    small = make_job(rng, 2, 3, 2, torch.float64, L=4, threads=64)
    a = device_args(small)
    err = pkg.signature_group(None, [as_job(small, a)] * 9)
    assert not err and err.code == pkg.ErrorCode.InvalidArgument
    odd = make_job(rng, 2, 3, 2, torch.float64, L=4, threads=48)
    err = pkg.signature_group(None, [as_job(odd, device_args(odd))])
    assert not err and err.code == pkg.ErrorCode.InvalidArgument
    flagged = make_job(rng, 2, 3, 2, torch.float64, L=4, threads=64 | (1 << 20))  # not a job bit
    err = pkg.signature_group(None, [as_job(flagged, device_args(flagged))])
    assert not err and err.code == pkg.ErrorCode.InvalidArgument
    err = pkg.signature_group(None, [as_job(small, a)], schedule=768)
    assert not err and err.code == pkg.ErrorCode.InvalidArgument
    rc = lib.rpp_gb_signature_group(None, None, 0, 0)
    assert rc == int(pkg.ErrorCode.InvalidArgument)
