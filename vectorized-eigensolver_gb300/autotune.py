"""Launch-shape autotuner for the persistent solver kernels.

The persistent kernels (FP64 fused solve, FP32 Schur stage of the mixed form,
eigenvalues-only, mixed-size batches) run `blocks_per_sm` blocks of 4 warps
per SM; the best value depends on the order n (register and local-memory
pressure against latency hiding), the precision and, for mixed-size batches,
the size distribution and the binning order.  `tune()` times the candidates on
a synthetic batch of the caller's shape with CUDA events and records the
winner in a JSON cache keyed by device name, form and order; `options()`
returns ves_options carrying the cached choice (library defaults when the
shape was never tuned).

Cache file: `path` argument, else $VES_TUNE_CACHE, else
~/.cache/ves_gb300/tune.json.
"""
import json
import os
import threading

import numpy as np

import ves

CANDIDATE_BPS = (1, 2, 3, 4, 6, 8)
_lock = threading.Lock()


def default_cache_path():
    return os.environ.get("VES_TUNE_CACHE") or os.path.join(os.path.expanduser("~"), ".cache", "ves_gb300",
                                                            "tune.json")


def _key(device_name, form, dim):
    return f"{device_name}|{form}|n={dim}"


def form_name(precision=ves.VES_PREC_FP64, want_vectors=1):
    if not want_vectors:
        return "eigvals"
    return "fp32_refine" if precision == ves.VES_PREC_FP32_REFINE else "fp64"


class TuneCache:
    """JSON map  device|form|n=dim -> {"blocks_per_sm": b, "varsize_order": o, "ms": {...}}."""

    def __init__(self, path=None):
        self.path = path or default_cache_path()
        self.entries = {}
        if os.path.exists(self.path):
            with open(self.path) as f:
                self.entries = json.load(f)

    def get(self, device_name, form, dim):
        return self.entries.get(_key(device_name, form, dim))

    def put(self, device_name, form, dim, entry):
        self.entries[_key(device_name, form, dim)] = entry

    def save(self):
        d = os.path.dirname(self.path)
        if d:
            os.makedirs(d, exist_ok=True)
        tmp = self.path + ".tmp"
        with _lock:
            with open(tmp, "w") as f:
                json.dump(self.entries, f, indent=1, sort_keys=True)
            os.replace(tmp, self.path)


def pick_best(timings):
    """The candidate with the smallest time; ties go to the smaller launch."""
    return min(sorted(timings), key=lambda c: timings[c])


def _device_name():
    import torch
    return torch.cuda.get_device_name(torch.cuda.current_device())


def _time(fn, reps):
    import torch
    fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def tune(dim, N=None, precision=ves.VES_PREC_FP64, want_vectors=1, candidates=CANDIDATE_BPS, reps=2,
         thread_cnt=512, seed=7, cache=None, save=True):
    """Time ves_eigensolve on N Gaussian matrices of order `dim` for each
    blocks_per_sm candidate; store and return the cache entry."""
    import torch
    import workloads
    if N is None:
        N = max(thread_cnt, (1 << 22) // (dim * dim) // thread_cnt * thread_cnt)
    N = max(thread_cnt, N // thread_cnt * thread_cnt)
    rA, iA = workloads.gaussian_soa(N, dim, seed=seed, thread_cnt=thread_cnt)
    rA, iA = torch.from_numpy(rA).cuda(), torch.from_numpy(iA).cuda()
    rE = torch.empty(N * dim, dtype=torch.float64, device="cuda")
    iE = torch.empty_like(rE)
    rV = torch.empty_like(rA) if want_vectors else None
    iV = torch.empty_like(iA) if want_vectors else None
    timings = {}
    for b in candidates:
        o = ves.default_options(precision=precision, want_vectors=want_vectors, blocks_per_sm=b)
        ws = ves.Workspace(dim, N // thread_cnt, thread_cnt, options=o)
        timings[b] = _time(lambda: ves.eigensolve(dim, N // thread_cnt, thread_cnt, rA, iA, rE, iE, rV, iV,
                                                  options=o, workspace=ws), reps)
        del ws
    best = pick_best(timings)
    entry = {"blocks_per_sm": int(best), "ms": {str(k): round(v, 4) for k, v in timings.items()}, "N": int(N)}
    cache = cache if cache is not None else TuneCache()
    cache.put(_device_name(), form_name(precision, want_vectors), dim, entry)
    if save:
        cache.save()
    return entry


def tune_varsize(sizes, by_n=None, max_dim=64, candidates=(2, 4, 8), orders=(0, 1), reps=2, seed=2, cache=None,
                 save=True):
    """Time ves_eigensolve_varsize on a mixed-size batch for each
    (blocks_per_sm, varsize_order); `sizes` is either the batch's order array
    (with `by_n` from workloads.mixed_families(as_list=False)) or a count, in
    which case the mixed-family workload of that count is generated."""
    import torch
    import workloads
    if by_n is None:
        sizes, by_n = workloads.mixed_families(int(sizes), seed=seed, nmax=max_dim, device="cuda", as_list=False)
    dims, re, im = workloads.pack_varsize(sizes, by_n, device="cuda")
    count = len(sizes)
    er = torch.empty(int(np.sum(sizes)), dtype=torch.float64, device="cuda")
    ei = torch.empty_like(er)
    vr, vi = torch.empty_like(re), torch.empty_like(im)
    timings = {}
    for order in orders:
        for b in candidates:
            o = ves.default_options(varsize_order=order, blocks_per_sm=b)
            ws = ves.varsize_workspace(count, max_dim, o)
            timings[(b, order)] = _time(lambda: ves.eigensolve_varsize(count, max_dim, dims, re, im, er, ei, vr, vi,
                                                                       options=o, workspace=ws), reps)
            del ws
    b, order = pick_best(timings)
    entry = {"blocks_per_sm": int(b), "varsize_order": int(order), "count": int(count),
             "ms": {f"{k[0]},{k[1]}": round(v, 4) for k, v in timings.items()}}
    cache = cache if cache is not None else TuneCache()
    cache.put(_device_name(), "varsize", max_dim, entry)
    if save:
        cache.save()
    return entry


def options(dim, precision=ves.VES_PREC_FP64, want_vectors=1, cache=None, device_name=None, **overrides):
    """ves_options with the tuned launch shape for this device, form and order
    (library defaults where nothing was tuned)."""
    cache = cache if cache is not None else TuneCache()
    name = device_name or _device_name()
    e = cache.get(name, form_name(precision, want_vectors), dim)
    kw = dict(precision=precision, want_vectors=want_vectors)
    if e:
        kw["blocks_per_sm"] = e["blocks_per_sm"]
    kw.update(overrides)
    return ves.default_options(**kw)


def varsize_options(max_dim=64, cache=None, device_name=None, **overrides):
    cache = cache if cache is not None else TuneCache()
    name = device_name or _device_name()
    e = cache.get(name, "varsize", max_dim)
    kw = {}
    if e:
        kw = dict(blocks_per_sm=e["blocks_per_sm"], varsize_order=e["varsize_order"])
    kw.update(overrides)
    return ves.default_options(**kw)
