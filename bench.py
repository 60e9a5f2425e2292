"""Benchmark: batched complex eigen-decomposition on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ves|reference] [--split]

Several GPUs (one process per GPU under torchrun): by default every rank
solves its own batch (seed 1 + rank; weak scaling); with --split the one batch
is cut into contiguous ranges of whole SoA blocks (ves_partition_blocks), one
per rank (strong scaling).  Either way the ranks share no data: a barrier and
the max over ranks bracket the timed region.

Workload (one step = one solve of the whole batch): 1,048,576 complex128
16x16 matrices, real and imaginary parts i.i.d. N(0,1) from numpy
default_rng(1), in the reference's SoA layout with thread_cnt = 512; all
eigenvalues and right eigenvectors (zgehrd -> zunghr -> zlahqr -> ztrevc).
The input (4.3 GB) is larger than L2, so no flush is needed between steps.

value   eigensolves/s with the batch resident in HBM, CUDA events around K
        launches of ves_eigensolve on the launching stream.
e2e     the same metric through the reference-facing drop-in eigensolver()
        with pinned HOST buffers: host->device copy of A, solve, device->host
        copy of eigenvalues, eigenvectors and the Schur form (which the
        reference API writes back into A) inside the timed region.
roofline  the solver is FP64-pipe bound: achieved = algorithmic FP64 flops
        per launch (24 n^3 + 20 s n^3 per matrix, s = device-counted QR
        sweeps per eigenvalue) / launch time, against the FP64 FMA rate
        measured on this GPU in this run (MEASURED_PEAKS.json carries no FP64
        figure).  The HBM view (32 n^2 + 16 n bytes per matrix) is reported
        beside it.
cpu_baseline  the oracle's C restatement of the reference CPU path (OpenMP,
        all host cores) on a bounded prefix of the same batch.
forms   the other forms, each on its own batch, each verified (residuals on the
        device; FP32+refine and learned: eigenvalues against the plain FP64 solve of
        the same batch, max and median per-matrix error relative to ||A||_F):
        FP32+refine  n=16 (the same batch) and n=32 (262,144 Gaussian, seed 3,
                     beside plain FP64 on the same batch);
        learned shift  n=16 and n=32 on the family A0 + p1 A1 + p2 A2 + p3 A3
                     (262,144 matrices, parameter seed 6): the network is
                     trained first (200,000 plain-solver solutions, seed 5; not
                     timed), then one step = inference + polish + shift-seeded
                     FP64 solve, against plain FP64 on the same batch;
                     and 1,048,576 x 24x24 with the network specified for that
                     workload (3 hidden layers of 256, GELU; inputs: the 3
                     parameters and the 24 complex diagonal entries);
        mixed-size   500,000 matrices of orders 4..64 (Gaussian, non-normal,
                     clustered; seed 2): one CUDA-graph replay of the binned
                     persistent solve against one launch per order.
        Each form entry carries its own roofline from its algorithmic work
        (device-counted where it is data dependent: QR sweeps, Newton
        corrections and residuals of the refinement, polish steps): FP64
        flops against the FP64 FMA rate probed in this run, FP32 flops
        against the FP32 FMA rate probed in this run, BF16 tensor flops
        against MEASURED_PEAKS.json's bf16_tflops, and 32 n^2 + 16 n bytes per
        matrix against its hbm_gbs; `bound` names the unit whose work takes
        longest at its peak.  The JSON line keeps each form compact; the full
        record of each form is printed to stderr.
Every result is verified after timing: all residuals on the device in FP64
(<= 1e-13 of ||A||_F ||v||); eigenvalue parity with the oracle is the job of
the test suite (tests/test_gpu_fullsize.py runs this workload).

--impl reference times the reference's CPU implementation of the path on the
host cores (the compiled reference where it was built, otherwise the C
restatement) on bounded samples of the same workload.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "vectorized-eigensolver_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "eigensolves/s at n=16,32 at resid≤1e-13; learned-shift, FP32+refine vs plain FP64"
WORKLOAD = dict(name="gauss16", N=1_048_576, n=16, seed=1, tc=512)
RES_TOL = 1e-13

# Roofline denominators, filled in by run_gpu_arm: the FP64 and FP32 FMA rates
# measured on this GPU in this run (flop/s), and MEASURED_PEAKS.json's dense
# BF16 tensor rate (flop/s) and copy bandwidth (B/s).
PEAKS = {}


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def r4(x):
    """A number rounded to 4 significant digits (keeps the JSON line short)."""
    return float("%.4g" % x) if isinstance(x, float) else x


def roofline(seconds, fp64=0.0, fp32=0.0, bf16=0.0, hbm=0.0):
    """Roofline of one step from its ALGORITHMIC work: FP64 / FP32 / BF16 flops
    and HBM bytes.  Per unit, frac = (work / step time) / measured peak; the
    bound is the unit whose work takes longest at its peak, and the top-level
    frac is that lower bound on the step time divided by the step time."""
    units = {"fp64": (fp64, "TFLOP/s", 1e12), "fp32": (fp32, "TFLOP/s", 1e12), "bf16": (bf16, "TFLOP/s", 1e12),
             "hbm": (hbm, "GB/s", 1e9)}
    fracs = {}
    for u, (work, _, _) in units.items():
        if work > 0 and PEAKS.get(u):
            fracs[u] = work / seconds / PEAKS[u]
    bound = max(fracs, key=fracs.get)
    work, unit, scale = units[bound]
    return {"bound": bound, "achieved": r4(work / seconds / scale), "peak": r4(PEAKS[bound] / scale), "unit": unit,
            "frac": r4(fracs[bound]), "fracs": {u: r4(f) for u, f in fracs.items()}}


def fp64_flops(n, sweeps_total, matrices):
    """24 n^3 + 20 s n^3 per matrix (Hessenberg 40/3 n^3, Q 16/3 n^3, back
    substitution and back transformation 16/3 n^3, QR sweeps 20 n^2 per sweep of
    the matrix), summed: sweeps_total = QR sweeps over all `matrices`."""
    return 24.0 * n ** 3 * matrices + 20.0 * n * n * sweeps_total


def hbm_bytes(n, matrices):
    """Read A, write V and the eigenvalues: 32 n^2 + 16 n bytes per matrix."""
    return (32.0 * n * n + 16.0 * n) * matrices


# ----------------------------------------------------------------------------
# distributed plumbing (one process per GPU; independent replicas, no data-path collective)
# ----------------------------------------------------------------------------
def rank_batch(rank):
    """The batch rank `rank` solves: the benchmark workload with seed 1 + rank
    (weak scaling: every GPU gets its own 1,048,576 matrices; no data-path
    exchange between ranks)."""
    w = WORKLOAD
    return dict(N=w["N"], n=w["n"], tc=w["tc"], seed=w["seed"] + rank)


class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None

    def init(self, backend):
        if self.world > 1:
            import torch.distributed as dist
            dist.init_process_group(backend=backend)
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x):
        if not self.pg:
            return x
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64, device="cuda" if self.pg.get_backend() == "nccl" else "cpu")
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def done(self):
        if self.pg:
            self.pg.destroy_process_group()


# ----------------------------------------------------------------------------
# clocks during the timed region
# ----------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ----------------------------------------------------------------------------
# CPU side: the oracle (test infrastructure, used here only as the timed baseline)
# ----------------------------------------------------------------------------
def cpu_time(rA, iA, n, tc, threads, lib, min_seconds):
    import oracle
    N = rA.size // (n * n)
    reps, total = 0, 0.0
    oracle.eigensolve(rA, iA, n, tc, lib=lib, threads=threads)  # warm-up
    while reps == 0 or total < min_seconds:
        t0 = time.perf_counter()
        oracle.eigensolve(rA, iA, n, tc, lib=lib, threads=threads)
        total += time.perf_counter() - t0
        reps += 1
    return N * reps / total, reps, total


def cpu_kind():
    import oracle
    return ("reference", "reference") if oracle.reference() is not None else ("port", "restatement")


# ----------------------------------------------------------------------------
def run_reference_arm(args, d):
    if d.rank != 0:
        return
    w = WORKLOAD
    import workloads
    cores = os.cpu_count() or 1
    kind, lib = cpu_kind()
    sample = args.ref_sample
    rA, iA = workloads.gaussian_soa(w["N"], w["n"], w["seed"], w["tc"])  # the batch; its first `sample` matrices
    k = sample * w["n"] ** 2
    rA, iA = rA[:k].copy(), iA[:k].copy()
    for _ in range(max(args.warmup, 0)):
        cpu_time(rA, iA, w["n"], w["tc"], cores, lib, 0.0)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        import oracle
        oracle.eigensolve(rA, iA, w["n"], w["tc"], lib=lib, threads=cores)
        times.append(time.perf_counter() - t0)
    tot = sum(times)
    val = sample * args.steps / tot
    out = {
        "impl": "reference", "metric": METRIC, "value": val, "unit": "eigensolves/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: complex Gaussian, numpy default_rng(1)",
        "config": {"workload": "1,048,576 complex128 16x16 (SoA thread_cnt=512, seed 1); each step solves "
                               "its first %d matrices on the host CPU" % sample, "n": w["n"]},
        "cpu_baseline": {"value": val, "unit": "eigensolves/s", "cores": cores, "kind": kind,
                         "sample": "first %d matrices of the batch per step, zgehrd->zunghr->zlahqr->ztrevc, "
                                   "OpenMP over all %d host threads" % (sample, cores)},
        "e2e": {"value": val, "unit": "eigensolves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def device_residual_check(dAr, dAi, dEr, dEi, dVr, dVi, n, tc, chunk=1 << 17):
    """max and median over all pairs of ||A v - lambda v|| / (||A||_F ||v||), FP64 on the device."""
    import torch

    def mat(re, im):
        return torch.complex(re.view(-1, n, n, tc).permute(0, 3, 2, 1), im.view(-1, n, n, tc).permute(0, 3, 2, 1)
                             ).reshape(-1, n, n)
    A, V = mat(dAr, dAi), mat(dVr, dVi)
    E = torch.complex(dEr.view(-1, n, tc).permute(0, 2, 1), dEi.view(-1, n, tc).permute(0, 2, 1)).reshape(-1, n)
    worst, nonfinite, parts = 0.0, 0, []
    for s in range(0, A.shape[0], chunk):
        a, e, v = A[s:s + chunk], E[s:s + chunk], V[s:s + chunk]
        r = torch.linalg.vector_norm(torch.matmul(a, v) - v * e[:, None, :], dim=1)
        den = torch.linalg.matrix_norm(a)[:, None] * torch.linalg.vector_norm(v, dim=1)
        q = r / den
        nonfinite += int((~torch.isfinite(q)).sum())
        worst = max(worst, float(torch.nan_to_num(q, nan=0.0).max()))
        parts.append(torch.nan_to_num(q, nan=0.0).flatten().float())
    median = float(torch.cat(parts).median())
    return {"max_residual": worst, "median_residual": median, "nonfinite": nonfinite,
            "checked_matrices": int(A.shape[0])}


def measure_form(name, n, N, seed, tc, precision, warmup, steps):
    """Device-resident eigensolves/s of one form on one seeded Gaussian batch,
    verified on the device afterwards (every residual; for FP32+refine also the
    eigenvalues against a plain FP64 solve of the same batch: max and median over
    the matrices of each matrix's largest distance, relative to ||A||_F).
    Returns the compact entry of the JSON line and the detail record (stderr)."""
    import torch
    import ves
    import workloads
    bc = N // tc
    rA, iA = workloads.gaussian_soa(N, n, seed, tc)
    dAr, dAi = torch.from_numpy(rA).cuda(), torch.from_numpy(iA).cuda()
    del rA, iA
    dEr = torch.empty(N * n, dtype=torch.float64, device="cuda")
    dEi = torch.empty_like(dEr)
    dVr, dVi = torch.empty_like(dAr), torch.empty_like(dAi)
    st = torch.zeros(N, dtype=torch.int32, device="cuda")
    sw = torch.zeros(N, dtype=torch.int32, device="cuda")
    wc = torch.zeros(ves.VES_WORK_COUNTS, dtype=torch.int64, device="cuda")
    opt = ves.default_options(precision=precision)
    wsp = ves.Workspace(n, bc, tc, opt)
    stream = torch.cuda.current_stream()
    run = lambda o=opt, **kw: ves.eigensolve(n, bc, tc, dAr, dAi, dEr, dEi, dVr, dVi, options=o,  # noqa: E731
                                             workspace=wsp, stream=stream, **kw)
    for _ in range(warmup):
        run()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        run()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    # the work of the step (results are deterministic: the same as every timed step)
    run(ves.default_options(precision=precision, work_counts=wc), status=st, sweeps=sw)
    torch.cuda.synchronize()
    ver = device_residual_check(dAr, dAi, dEr, dEi, dVr, dVi, n, tc)
    fbm = (st & 8) != 0
    fb = int(fbm.sum())
    other = int(((st & ~8) != 0).sum())
    swd = sw.double()
    res64, corr32, resff, _ = (int(x) for x in wc.tolist())
    if precision:
        # FP32: the reference path on the matrices that stayed in FP32, the Newton
        # corrections (Z^H r 8n^2, bordered back substitution 4n^2, Z dx 8n^2) and
        # the first residuals (8n^2, in float-float on the FP32 pipe); FP64: the
        # accepting residuals (8n^2 + 16n with the norms) and the fallback solves
        f32 = fp64_flops(n, float(swd[~fbm].sum()), N - fb) + corr32 * 20.0 * n * n + resff * 8.0 * n * n
        f64 = fp64_flops(n, float(swd[fbm].sum()), fb) + res64 * (8.0 * n * n + 16.0 * n)
    else:
        f32, f64 = 0.0, fp64_flops(n, float(swd.sum()), N)
    rl = roofline(ms * 1e-3, fp64=f64, fp32=f32, hbm=hbm_bytes(n, N))
    passed = ver["max_residual"] <= RES_TOL and ver["nonfinite"] == 0 and other == 0
    out = {"form": name, "n": n, "N": N, "value": r4(N / (ms * 1e-3)), "ms": r4(ms), "roofline": rl,
           "s": r4(float(swd.mean()) / n), "max_res": r4(ver["max_residual"]), "passed": passed}
    detail = {"form": name, "n": n, "n_matrices": N, "seed": seed, "steps": steps, "warmup": warmup,
              "median_residual": ver["median_residual"], "nonfinite": ver["nonfinite"], "status_other": other,
              "flops_fp64": f64, "flops_fp32": f32}
    if precision:
        out["fb"] = fb
        detail.update(fp64_fallback_matrices=fb, fp64_residuals=res64, fp32_corrections=corr32,
                      ff_residuals=resff, fp64_residuals_per_pair=res64 / max(1, (N - fb) * n))
        # eigenvalues against the plain FP64 solve of the same batch (untimed)
        dE0r, dE0i = torch.empty_like(dEr), torch.empty_like(dEi)
        ves.eigensolve(n, bc, tc, dAr, dAi, dE0r, dE0i, dVr, dVi, stream=stream)
        torch.cuda.synchronize()
        emax, emed = eig_errors(_vec(dEr, dEi, n, tc), _vec(dE0r, dE0i, n, tc), _mat(dAr, dAi, n, tc))
        out["eig_err"] = r4(emax)
        out["passed"] = passed and emax <= 1e-12
        detail.update(eig_err_vs_fp64_max=emax, eig_err_vs_fp64_median=emed)
        del dE0r, dE0i
    del dAr, dAi, dEr, dEi, dVr, dVi, wsp
    torch.cuda.empty_cache()
    return out, detail


def _mat(re, im, n, tc):
    import torch
    return torch.complex(re.view(-1, n, n, tc).permute(0, 3, 2, 1), im.view(-1, n, n, tc).permute(0, 3, 2, 1)
                         ).reshape(-1, n, n)


def _vec(re, im, n, tc):
    import torch
    return torch.complex(re.view(-1, n, tc).permute(0, 2, 1), im.view(-1, n, tc).permute(0, 2, 1)).reshape(-1, n)


def eig_errors(E1, E0, A, chunk=1 << 16):
    """Per matrix, the largest distance from an eigenvalue in E1 to the nearest one
    in E0, relative to ||A||_F; returns its max and median over the matrices (device)."""
    import torch
    per = []
    for s in range(0, E1.shape[0], chunk):
        d = (E1[s:s + chunk, :, None] - E0[s:s + chunk, None, :]).abs().amin(dim=2).amax(dim=1)
        per.append(d / torch.linalg.matrix_norm(A[s:s + chunk]))
    per = torch.cat(per)
    return float(per.max()), float(per.median())


def eig_distance(E1, E0, A, chunk=1 << 17):
    """max over matrices and eigenvalues of the distance from each eigenvalue in
    E1 to the nearest one in E0, relative to ||A||_F (device)."""
    import torch
    worst = 0.0
    for s in range(0, E1.shape[0], chunk):
        d = (E1[s:s + chunk, :, None] - E0[s:s + chunk, None, :]).abs().amin(dim=2)
        nA = torch.linalg.matrix_norm(A[s:s + chunk])
        worst = max(worst, float((d / nA[:, None]).max()))
    return worst


# Learned-shift configuration per order (chosen on GB300 by sweeping depth,
# Fourier features, epochs, polish steps and gate on a held-out draw):
#   net     ves_shiftnet_config fields (robust Chamfer loss, delta 0.01)
#   epochs  over the 200,000 training solutions
#   polish  Aberth steps on all predictions of a matrix (FP32, on the Hessenberg
#           form; more steps changed nothing on any order), then one FP64 Newton
#           step per prediction inside the solve
#   gate    predictions only while |H(I,I-1)| > gate * ||A||_F / sqrt(n); 0 = always
LEARNED = {
    16: dict(net=dict(hidden=256, layers=4, fourier=8, loss=1, delta=0.01), epochs=150, polish=16, gate=0.0),
    32: dict(net=dict(hidden=256, layers=5, fourier=12, loss=1, delta=0.01), epochs=300, polish=16, gate=0.0),
    # 1,048,576 x 24x24: the network as specified for this workload (inputs: the 3
    # parameters and the 24 complex diagonal entries; 3 hidden layers of 256, GELU)
    24: dict(net=dict(hidden=256, layers=3, fourier=0, loss=1, delta=0.01), epochs=150, polish=16, gate=0.0),
}


def measure_learned(n, N, train_count, steps, tc=512):
    """The learned-shift form on the parametric family A(p) = A0 + p1 A1 + p2 A2
    + p3 A3 (order n): the network is trained (tcgen05 BF16 MLP) on
    `train_count` plain-solver solutions (param seed 5), then on a fresh batch
    (param seed 6) one step = network inference + the shift-seeded FP64 solve
    (predictions polished by Aberth steps in FP32 and one Newton step in FP64),
    against the plain FP64 solve
    of the same batch."""
    import torch
    import ves
    import learned_shift
    cfg = LEARNED[n]
    epochs = cfg["epochs"]
    t0 = time.perf_counter()
    net, losses = learned_shift.train(n, count=train_count, epochs=epochs, batch=1024, lr=1e-3, **cfg["net"])
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    p, rA, iA = learned_shift.family(N, n, param_seed=6, thread_cnt=tc)
    bc = N // tc
    rE0 = torch.empty(N * n, dtype=torch.float64, device="cuda")
    iE0, rE, iE = torch.empty_like(rE0), torch.empty_like(rE0), torch.empty_like(rE0)
    rS, iS = torch.empty_like(rE0), torch.empty_like(rE0)
    rV, iV = torch.empty_like(rA), torch.empty_like(iA)
    sw0, sw, st, fb = (torch.zeros(N, dtype=torch.int32, device="cuda") for _ in range(4))
    ws = ves.Workspace(n, bc, tc)
    lopt = ves.default_options(shift_polish=cfg["polish"], shift_gate=cfg["gate"])
    lws = ves.shifts_workspace(n, bc, tc, lopt)
    pws = net.predict_workspace(N)
    stream = torch.cuda.current_stream()

    def plain(**kw):
        ves.eigensolve(n, bc, tc, rA, iA, rE0, iE0, rV, iV, workspace=ws, stream=stream, **kw)

    def learned(**kw):
        net.predict_into(N, tc, p, rA, iA, rS, iS, pws, stream=stream)
        ves.eigensolve_shifts(n, bc, tc, rA, iA, rE, iE, rV, iV, rS, iS, options=lopt, workspace=lws,
                              stream=stream, **kw)

    def timed(fn):
        for _ in range(2):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps

    ms_plain = timed(plain)
    ms_learned = timed(learned)
    plain(sweeps=sw0)
    wc = torch.zeros(ves.VES_WORK_COUNTS, dtype=torch.int64, device="cuda")
    lopt.work_counts = wc.data_ptr()
    learned(status=st, sweeps=sw, fallbacks=fb)
    torch.cuda.synchronize()
    lopt.work_counts = None
    ver = device_residual_check(rA, iA, rE, iE, rV, iV, n, tc)
    A = _mat(rA, iA, n, tc)
    err = eig_distance(_vec(rE, iE, n, tc), _vec(rE0, iE0, n, tc), A)
    pred_err = (_vec(rS, iS, n, tc)[:, :, None] - _vec(rE0, iE0, n, tc)[:, None, :]).abs().amin(dim=2)
    nA = torch.linalg.matrix_norm(A)
    other = int(((st & ~4) != 0).sum())
    # work of one step: the shift-seeded FP64 solve (its own sweeps); on the FP32
    # pipe the polish (Hessenberg reduction 40/3 n^3 in the pre-pass for n <= 32,
    # 8 n^2 + 10 n per Aberth step on det(H - sI): Hyman's recurrence and the
    # sum over the other predictions, device-counted) and the network's FP32
    # output layer (2 * hidden * 2n); on the tensor cores the BF16 hidden layers
    # (2 * (features * hidden + (layers - 1) * hidden^2) per matrix)
    polish_steps = int(wc[ves.VES_WORK_POLISH])
    h, L, F = cfg["net"]["hidden"], cfg["net"]["layers"], cfg["net"]["fourier"]
    kin = 3 + 2 * 3 * F + 2 * n
    # + the Newton step on each prediction: Hyman's recurrence for r in FP64 (4 n^2),
    # for r' in FP32 (4 n^2, with the FP32 work below)
    f64 = fp64_flops(n, float(sw.double().sum()), N) + (N * 4.0 * n ** 3 if cfg["polish"] > 0 else 0.0)
    f32 = (polish_steps * (8.0 * n * n + 10.0 * n) + (N * 40.0 / 3.0 * n ** 3 if n <= 32 else 0.0) + N * 2.0 * h * 2 * n
           + (N * 4.0 * n ** 3 if cfg["polish"] > 0 else 0.0))
    fbf16 = N * 2.0 * (kin * h + (L - 1) * h * h)
    rl = roofline(ms_learned * 1e-3, fp64=f64, fp32=f32, bf16=fbf16, hbm=hbm_bytes(n, N))
    passed = ver["max_residual"] <= RES_TOL and ver["nonfinite"] == 0 and err <= 1e-12 and other == 0
    out = {"form": "learned shift", "n": n, "N": N, "value": r4(N / (ms_learned * 1e-3)), "ms": r4(ms_learned),
           "vs_plain": r4(ms_plain / ms_learned), "roofline": rl, "s": r4(float(sw.double().mean()) / n),
           "s_plain": r4(float(sw0.double().mean()) / n), "max_res": r4(ver["max_residual"]), "passed": passed}
    detail = {"form": "learned shift", "n": n, "n_matrices": N, "family": "A0 + p1 A1 + p2 A2 + p3 A3, p ~ U[-1,1]^3",
              "plain_fp64_value": N / (ms_plain * 1e-3), "fallback_per_eigenvalue": float(fb.double().mean()) / n,
              "prediction_error_median_rel": float((pred_err / nA[:, None]).median()),
              "train": {"matrices": train_count, "epochs": epochs, "seconds": train_s, "loss_first": losses[0],
                        "loss_last": losses[-1], "network": cfg["net"]},
              "shift_polish": cfg["polish"], "shift_gate": cfg["gate"], "polish_steps": polish_steps,
              "flops_fp64": f64, "flops_fp32": f32, "flops_bf16": fbf16,
              "nonfinite": ver["nonfinite"], "max_eig_err_rel": err}
    del net, rA, iA, rV, iV, ws, lws, pws, A
    torch.cuda.empty_cache()
    return out, detail


def measure_varsize(count, steps, seed=2, max_dim=64):
    """Mixed-size batch (orders uniform in [4, 64]; Gaussian, non-normal and
    clustered families): one persistent size-binned launch (ves_eigensolve_varsize,
    replayed as a CUDA graph) against one ves_eigensolve launch per order."""
    import torch
    import ves
    import workloads
    sizes, by_n = workloads.mixed_families(count, seed=seed, nmax=max_dim, device="cuda", as_list=False)
    dims, re, im = workloads.pack_varsize(sizes, by_n, device="cuda")
    er = torch.empty(int(sizes.sum()), dtype=torch.float64, device="cuda")
    ei = torch.empty_like(er)
    vr, vi = torch.empty_like(re), torch.empty_like(im)
    st = torch.zeros(count, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    o = ves.default_options()
    g = ves.VarsizeGraph(count, max_dim, dims, re, im, er, ei, vr, vi, status=st, options=o)

    def timed(fn, reps):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    ms = timed(lambda: g.launch(stream), steps)
    bad = int((st != 0).sum())
    sw = torch.zeros(count, dtype=torch.int32, device="cuda")
    ves.eigensolve_varsize(count, max_dim, dims, re, im, er, ei, vr, vi, sweeps=sw, options=o)
    torch.cuda.synchronize()
    nd = torch.from_numpy(sizes.astype(np.float64)).cuda()
    flops = float((24.0 * nd ** 3 + 20.0 * sw.double() * nd ** 2).sum())
    # residuals per order bucket (packed column-major per matrix)
    off = np.concatenate([[0], np.cumsum(sizes.astype(np.int64) ** 2)])
    eoff = np.concatenate([[0], np.cumsum(sizes.astype(np.int64))])
    worst = 0.0
    per_n = []
    for n, (idx, _) in sorted(by_n.items()):
        ii = torch.from_numpy(idx).cuda()
        o2 = torch.from_numpy(off[idx]).cuda()[:, None] + torch.arange(n * n, device="cuda")[None]
        e2 = torch.from_numpy(eoff[idx]).cuda()[:, None] + torch.arange(n, device="cuda")[None]
        A = torch.complex(re[o2], im[o2]).view(-1, n, n).transpose(1, 2)
        V = torch.complex(vr[o2], vi[o2]).view(-1, n, n).transpose(1, 2)
        E = torch.complex(er[e2], ei[e2])
        r = torch.linalg.vector_norm(A @ V - V * E[:, None, :], dim=1)
        q = r / (torch.linalg.matrix_norm(A)[:, None] * torch.linalg.vector_norm(V, dim=1))
        worst = max(worst, float(torch.nan_to_num(q, nan=1.0).max()))
        # the per-order baseline: this bucket as its own SoA batch (thread_cnt = bucket size)
        k = len(idx)
        rs = A.real.permute(2, 1, 0).contiguous().reshape(-1)
        is_ = A.imag.permute(2, 1, 0).contiguous().reshape(-1)
        per_n.append((n, k, rs, is_))
        del ii
    del A, V
    bufs = []
    need = 0
    for n, k, rs, is_ in per_n:
        eb = torch.empty(k * n, dtype=torch.float64, device="cuda")
        bufs.append((n, k, rs, is_, eb, torch.empty_like(eb), torch.empty_like(rs), torch.empty_like(is_)))
        need = max(need, ves.lib().ves_eigensolve_workspace_size(n, 1, k, ves.ctypes.byref(o)))
    w = ves.DeviceBuffer(need)  # launches are stream-ordered: one workspace serves all orders

    def per_order():
        for n, k, rs, is_, eb, eb2, vb, vb2 in bufs:
            ves.eigensolve(n, 1, k, rs, is_, eb, eb2, vb, vb2, workspace=w, stream=stream)

    ms_per_order = timed(per_order, max(1, steps // 2))
    rl = roofline(ms * 1e-3, fp64=flops, hbm=float((32.0 * nd * nd + 16.0 * nd).sum()))
    out = {"form": "mixed-size batch", "n": "4..%d" % max_dim, "N": count, "value": r4(count / (ms * 1e-3)),
           "ms": r4(ms), "vs_per_order": r4(ms_per_order / ms), "roofline": rl,
           "s": r4(float(sw.double().sum()) / float(nd.sum())), "max_res": r4(worst),
           "passed": worst <= RES_TOL and bad == 0}
    detail = {"form": "mixed-size batch", "n_matrices": count, "orders": "uniform in [4, %d]" % max_dim,
              "families": "Gaussian / non-normal (cond(V)=1e4) / clustered (4 centres, radius 1e-6)",
              "api": "ves_eigensolve_varsize captured in a CUDA graph, replayed", "flops_fp64": flops,
              "per_order_launches_value": count / (ms_per_order * 1e-3), "status_nonzero": bad}
    del g, bufs, per_n, re, im, vr, vi, er, ei, w
    torch.cuda.empty_cache()
    return out, detail


def flops_per_matrix(n, s):
    return 24.0 * n ** 3 + 20.0 * s * n ** 3


def run_gpu_arm(args, d):
    import torch
    import ves
    import workloads

    torch.cuda.set_device(d.local)
    d.init("nccl")
    w = WORKLOAD
    N, n, tc = w["N"], w["n"], w["tc"]
    bc = N // tc
    if args.split:
        # strong scaling: ONE batch (seed 1) split over the ranks by whole SoA
        # blocks (ves_partition_blocks); each rank solves its part on its own GPU
        log("[bench] generating %d x %dx%d seed %d, split over %d ranks" % (N, n, n, w["seed"], d.world))
        rA, iA = workloads.gaussian_soa(N, n, w["seed"], tc)
        b0, nb = ves.partition_blocks(bc, d.world, d.rank)
        e0, e1 = b0 * tc * n * n, (b0 + nb) * tc * n * n
        rA, iA = rA[e0:e1].copy(), iA[e0:e1].copy()
        N_job, N, bc = N, nb * tc, nb
    else:
        seed = rank_batch(d.rank)["seed"]  # each rank solves its own batch (weak scaling)
        log("[bench] generating %d x %dx%d seed %d" % (N, n, n, seed))
        rA, iA = workloads.gaussian_soa(N, n, seed, tc)
        N_job = N * d.world
    dAr = torch.from_numpy(rA).cuda()
    dAi = torch.from_numpy(iA).cuda()
    dEr = torch.empty(N * n, dtype=torch.float64, device="cuda")
    dEi = torch.empty_like(dEr)
    dVr = torch.empty_like(dAr)
    dVi = torch.empty_like(dAi)
    st = torch.zeros(N, dtype=torch.int32, device="cuda")
    sw = torch.zeros(N, dtype=torch.int32, device="cuda")
    opt = ves.default_options()
    wsp = ves.Workspace(n, bc, tc, opt)
    stream = torch.cuda.current_stream()

    def step(with_stats=False):
        ves.eigensolve(n, bc, tc, dAr, dAi, dEr, dEi, dVr, dVi, status=st if with_stats else None,
                       sweeps=sw if with_stats else None, options=opt, workspace=wsp, stream=stream)

    peak_fp64 = ves.fp64_fma_rate(stream)
    peaks_file = {}
    try:
        peaks_file = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    PEAKS.update(fp64=peak_fp64, fp32=ves.fp32_fma_rate(stream),
                 bf16=peaks_file.get("bf16_tflops", 1900.0) * 1e12, hbm=peaks_file.get("hbm_gbs", 6800.0) * 1e9)
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    clocks = ClockSampler(d.local)
    clocks.start()
    d.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    d.barrier()
    ms = e0.elapsed_time(e1)
    ck = clocks.stop()
    ms_max = d.max(ms)
    value = N_job * args.steps / (ms_max * 1e-3)

    # statistics + verification (outside the timed region)
    step(with_stats=True)
    torch.cuda.synchronize()
    s_mean = float(sw.double().mean()) / n
    bad_status = int((st != 0).sum())
    ver = device_residual_check(dAr, dAi, dEr, dEi, dVr, dVi, n, tc)
    ok = ver["max_residual"] <= RES_TOL and ver["nonfinite"] == 0 and bad_status == 0

    launch_s = ms * 1e-3 / args.steps
    achieved = N * flops_per_matrix(n, s_mean) / launch_s
    hbm_b = hbm_bytes(n, N)
    hbm_peak = PEAKS["hbm"] / 1e9
    traffic = read_traffic()

    # e2e through the drop-in with pinned host buffers
    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(args, rA, iA, n, bc, tc, N)

    cpu = None
    if d.rank == 0 and not args.no_cpu:
        kind, lib = cpu_kind()
        sample = 65_536
        k = sample * n * n
        cores = os.cpu_count() or 1
        val, reps, tot = cpu_time(rA[:k].copy(), iA[:k].copy(), n, tc, cores, lib, 10.0)
        cpu = {"value": val, "unit": "eigensolves/s", "cores": cores, "kind": kind,
               "sample": "first %d matrices of the batch, %d repetitions (%.1f s), OpenMP over %d threads"
                         % (sample, reps, tot, cores)}

    # The other forms, each on its own batch.  The JSON line carries a compact
    # entry per form (value, speed-up, roofline, residual, verdict); the full
    # record of each goes to stderr.
    forms, details = [], []
    want = set(args.forms.split(",")) if args.forms else {"mixed16", "n32", "learned", "learned24", "varsize"}

    def add(res):
        forms.append(res[0])
        details.append(res[1])
        log("[bench] form detail: " + json.dumps(res[1]))

    if d.world == 1 and not args.no_forms:
        if "mixed16" in want:
            log("[bench] FP32+refine form, n=16")
            add(measure_form("FP32+refine", n, N, w["seed"], tc, 1, 2, args.steps))
            forms[-1]["vs_plain"] = r4(forms[-1]["value"] / value)
        if "n32" in want:
            log("[bench] plain FP64 and FP32+refine, n=32")
            add(measure_form("plain FP64", 32, 262_144, 3, 512, 0, 1, 2))
            add(measure_form("FP32+refine", 32, 262_144, 3, 512, 1, 1, 2))
            forms[-1]["vs_plain"] = r4(forms[-1]["value"] / forms[-2]["value"])
        if "learned" in want:
            for ln in (16, 32):
                log("[bench] learned-shift form, n=%d" % ln)
                add(measure_learned(ln, 262_144, 200_000, 2))
        if "learned24" in want:
            log("[bench] learned-shift form, 1,048,576 x 24x24")
            add(measure_learned(24, 1 << 20, 200_000, 2))
        if "varsize" in want:
            log("[bench] mixed-size form")
            add(measure_varsize(500_000, 2))

    d.done()
    if d.rank != 0:
        return
    out = {
        "metric": METRIC, "value": value, "unit": "eigensolves/s", "n_gpus": d.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
        "scaling": "strong" if args.split else "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: complex Gaussian N(0,1)+iN(0,1), numpy default_rng(%s)"
                % ("1, split over the ranks by SoA blocks" if args.split else "seed 1 + rank"),
        "config": {"workload": "1,048,576 complex128 16x16 %s, SoA thread_cnt=512, plain FP64 "
                               "(zgehrd->zunghr->zlahqr->ztrevc)" % ("in total" if args.split else "per GPU"),
                   "n": n, "n_matrices": N_job, "thread_cnt": tc,
                   "form": "plain FP64", "l2": "inputs (4.3 GB) larger than L2; no flush",
                   "sweeps_per_eigenvalue": s_mean},
        "roofline": {"bound": "fp64", "achieved": achieved / 1e12, "peak": peak_fp64 / 1e12, "unit": "TFLOP/s",
                     "frac": achieved / peak_fp64, "traffic": traffic,
                     "peak_source": "FP64 FMA rate measured in this run (ves_fp64_fma_rate); "
                                    "MEASURED_PEAKS.json has no FP64 figure",
                     "flops_per_matrix": flops_per_matrix(n, s_mean),
                     "hbm": {"achieved_gbs": hbm_b / launch_s / 1e9, "peak_gbs": hbm_peak,
                             "frac": hbm_b / launch_s / 1e9 / hbm_peak, "bytes_per_matrix": 32 * n * n + 16 * n,
                             "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)"}},
        "peaks": {"fp64_tflops": r4(PEAKS["fp64"] / 1e12), "fp32_tflops": r4(PEAKS["fp32"] / 1e12),
                  "bf16_tflops": r4(PEAKS["bf16"] / 1e12), "hbm_gbs": r4(PEAKS["hbm"] / 1e9),
                  "source": "FP64/FP32: FMA-rate probes run in this process; BF16, HBM: MEASURED_PEAKS.json"},
        "cpu_baseline": cpu,
        "e2e": e2e,
        "clocks": ck,
        "gpu_launches": args.steps,
        "verify": dict(ver, status_nonzero=bad_status, passed=ok),
        "forms": forms,
    }
    for f in forms:
        rl = f["roofline"]
        log("[bench] %-16s n=%-7s %12.6g eigensolves/s  %-16s roofline %s %.3f of measured  max residual %.2e%s"
            % (f["form"], f["n"], f["value"], ("x%.3g" % f.get("vs_plain", f.get("vs_per_order", 0))),
               rl["bound"], rl["frac"], f["max_res"], "" if f["passed"] else "  FAILED"))
    print(json.dumps(out, separators=(",", ":")), flush=True)
    if not ok or not all(f["passed"] for f in forms):
        log("[bench] VERIFICATION FAILED: %s" % json.dumps([out["verify"]] + details))
        sys.exit(1)


def read_traffic():
    """DRAM bytes per launch of the fused kernel from the committed ncu summary, or None."""
    p = os.path.join(ROOT, "profiles", "fused_fp64_gauss16.md")
    try:
        for ln in open(p):
            if ln.startswith("traffic_bytes_per_launch:"):
                return float(ln.split(":")[1])
    except Exception:
        pass
    return None


def run_e2e(args, rA, iA, n, bc, tc, N):
    import torch
    import ves
    pin = lambda a: torch.from_numpy(a).pin_memory()  # noqa: E731
    hAr0, hAi0 = pin(rA), pin(iA)
    hAr, hAi = torch.empty_like(hAr0).pin_memory(), torch.empty_like(hAi0).pin_memory()
    hEr = torch.empty(N * n, dtype=torch.float64).pin_memory()
    hEi = torch.empty_like(hEr).pin_memory()
    hVr = torch.empty_like(hAr0).pin_memory()
    hVi = torch.empty_like(hAi0).pin_memory()
    arr = [x.numpy() for x in (hAr, hAi, hEr, hEi, hVr, hVi)]
    times = []
    for it in range(args.warmup + args.steps):
        hAr.copy_(hAr0)  # the drop-in overwrites A with T: restore the input (not timed)
        hAi.copy_(hAi0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ves.eigensolver(n, bc, tc, *arr)
        t1 = time.perf_counter()
        if it >= args.warmup:
            times.append(t1 - t0)
    tot = sum(times)
    h2d = 2 * N * n * n * 8
    d2h = 2 * N * n * 8 + 4 * N * n * n * 8
    return {"value": N * len(times) / tot, "unit": "eigensolves/s", "h2d_bytes_per_step": h2d,
            "d2h_bytes_per_step": d2h, "ms_per_step": 1e3 * tot / len(times),
            "api": "eigensolver() drop-in (host pointers, pinned), synchronous"}


def run_ncu_case(args):
    """One solve per form on a small batch (inputs still larger than L2), no
    timing: the case the ncu captures under profiles/ are taken on.
    --ncu-form solve:    FP64 then FP32+refine on N Gaussian n x n matrices;
    --ncu-form shiftnet: network inference (4 tcgen05 GEMMs) on N family matrices
                         (untrained weights: the kernels do the same work);
    --ncu-form varsize:  one mixed-size solve of N family matrices (orders 4..64);
    --ncu-form learned:  polish pre-pass + shift-seeded FP64 solve of N family
                         matrices (predictions: eigenvalues + 1% noise)."""
    import torch
    import ves
    n, N, tc = args.ncu_n, args.ncu_case, 512
    if args.ncu_form == "shiftnet":
        import learned_shift
        p, rA, iA = learned_shift.family(N, n, param_seed=6, thread_cnt=tc)
        net = ves.ShiftNet(dim=n, n_params=3, hidden=256, seed=0)
        rS = torch.empty(N * n, dtype=torch.float64, device="cuda")
        iS = torch.empty_like(rS)
        net.predict(N, tc, p, rA, iA, rS, iS)
        torch.cuda.synchronize()
        print("ncu case done: shift network inference on %d matrices, n=%d" % (N, n))
        return
    if args.ncu_form == "learned":
        import learned_shift
        p, rA, iA = learned_shift.family(N, n, param_seed=6, thread_cnt=tc)
        rE0, iE0, _ = learned_shift.solve_plain(n, N, rA, iA, tc)
        g = torch.Generator(device="cuda").manual_seed(1)
        rS = rE0 + 1e-2 * torch.randn(rE0.shape, generator=g, device="cuda", dtype=torch.float64)
        iS = iE0 + 1e-2 * torch.randn(rE0.shape, generator=g, device="cuda", dtype=torch.float64)
        rE, iE = torch.empty_like(rE0), torch.empty_like(iE0)
        rV, iV = torch.empty_like(rA), torch.empty_like(iA)
        ves.eigensolve_shifts(n, N // tc, tc, rA, iA, rE, iE, rV, iV, rS, iS,
                              options=ves.default_options(shift_polish=16, shift_gate=0.0))
        torch.cuda.synchronize()
        print("ncu case done: polish pre-pass + shift-seeded solve of %d family matrices, n=%d" % (N, n))
        return
    if args.ncu_form == "varsize":
        import workloads
        sizes, by_n = workloads.mixed_families(N, seed=2, device="cuda", as_list=False)
        dims, re, im = workloads.pack_varsize(sizes, by_n, device="cuda")
        er = torch.empty(int(sizes.sum()), dtype=torch.float64, device="cuda")
        ei = torch.empty_like(er)
        vr, vi = torch.empty_like(re), torch.empty_like(im)
        ves.eigensolve_varsize(N, 64, dims, re, im, er, ei, vr, vi)
        torch.cuda.synchronize()
        print("ncu case done: mixed-size solve of %d matrices" % N)
        return
    g = torch.Generator(device="cuda").manual_seed(1)
    rA = torch.randn(N * n * n, dtype=torch.float64, device="cuda", generator=g)
    iA = torch.randn(N * n * n, dtype=torch.float64, device="cuda", generator=g)
    rE = torch.empty(N * n, dtype=torch.float64, device="cuda")
    iE = torch.empty_like(rE)
    rV, iV = torch.empty_like(rA), torch.empty_like(iA)
    for prec in (0, 1):
        opt = ves.default_options(precision=prec)
        ws = ves.Workspace(n, N // tc, tc, opt)
        ves.eigensolve(n, N // tc, tc, rA, iA, rE, iE, rV, iV, options=opt, workspace=ws)
        torch.cuda.synchronize()
    print("ncu case done: %d x %dx%d, FP64 then FP32+refine" % (N, n, n))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ves", choices=["ves", "reference"])
    ap.add_argument("--ref-sample", type=int, default=65_536,
                    help="matrices per step of the CPU reference arm (a prefix of the batch)")
    ap.add_argument("--split", action="store_true",
                    help="strong scaling: split the one 1,048,576-matrix batch over the ranks (default: weak, "
                         "every rank solves its own batch)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-forms", action="store_true",
                    help="skip the FP32+refine, n=32, learned-shift and mixed-size lines")
    ap.add_argument("--forms", default="",
                    help="comma list of the form lines to measure: mixed16, n32, learned, learned24, varsize (default all)")
    ap.add_argument("--ncu-case", type=int, default=0, metavar="N",
                    help="no benchmark: one solve per form on N matrices (for ncu captures)")
    ap.add_argument("--ncu-n", type=int, default=16)
    ap.add_argument("--ncu-form", default="solve", choices=["solve", "shiftnet", "varsize", "learned"])
    args = ap.parse_args()
    if args.ncu_case:
        run_ncu_case(args)
        return
    d = Dist()
    if args.impl == "reference":
        run_reference_arm(args, d)
        return
    run_gpu_arm(args, d)


if __name__ == "__main__":
    main()
