"""The autotuner's cache and selection logic (host only), and on the GPU that a
tuned launch shape changes the speed, never the results."""
import os

import numpy as np
import pytest

import autotune
import ves


def test_pick_best_prefers_fastest_then_smallest():
    assert autotune.pick_best({1: 3.0, 2: 1.0, 4: 1.5}) == 2
    assert autotune.pick_best({4: 1.0, 2: 1.0, 8: 2.0}) == 2
    assert autotune.pick_best({(4, 0): 1.0, (2, 1): 1.0}) == (2, 1)


def test_cache_roundtrip_and_options(tmp_path):
    path = str(tmp_path / "sub" / "tune.json")
    c = autotune.TuneCache(path)
    assert c.get("GPU", "fp64", 16) is None
    c.put("GPU", "fp64", 16, {"blocks_per_sm": 3, "ms": {"3": 1.0}})
    c.put("GPU", "varsize", 64, {"blocks_per_sm": 4, "varsize_order": 1})
    c.save()
    c2 = autotune.TuneCache(path)
    assert c2.get("GPU", "fp64", 16)["blocks_per_sm"] == 3
    o = autotune.options(16, cache=c2, device_name="GPU")
    assert o.blocks_per_sm == 3 and o.precision == ves.VES_PREC_FP64
    o = autotune.options(32, cache=c2, device_name="GPU")  # never tuned: library default
    assert o.blocks_per_sm == 0
    o = autotune.options(16, precision=ves.VES_PREC_FP32_REFINE, cache=c2, device_name="GPU")
    assert o.blocks_per_sm == 0 and o.precision == ves.VES_PREC_FP32_REFINE
    o = autotune.varsize_options(cache=c2, device_name="GPU")
    assert (o.blocks_per_sm, o.varsize_order) == (4, 1)
    assert autotune.options(16, cache=c2, device_name="GPU", blocks_per_sm=5).blocks_per_sm == 5


def test_cache_path_from_env(monkeypatch, tmp_path):
    monkeypatch.setenv("VES_TUNE_CACHE", str(tmp_path / "x.json"))
    assert autotune.default_cache_path() == str(tmp_path / "x.json")


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [ves.VES_PREC_FP64, ves.VES_PREC_FP32_REFINE])
def test_tuned_shape_same_results(tmp_path, precision):
    import torch
    import workloads
    c = autotune.TuneCache(str(tmp_path / "t.json"))
    e = autotune.tune(12, N=8192, precision=precision, candidates=(1, 2, 5), reps=1, cache=c)
    assert e["blocks_per_sm"] in (1, 2, 5) and os.path.exists(c.path)
    n, N, tc = 12, 8192, 512
    rA, iA = (torch.from_numpy(x).cuda() for x in workloads.gaussian_soa(N, n, seed=3, thread_cnt=tc))
    outs = []
    for b in (1, 5, 0):
        o = ves.default_options(precision=precision, blocks_per_sm=b)
        rE = torch.empty(N * n, dtype=torch.float64, device="cuda")
        iE, rV, iV = torch.empty_like(rE), torch.empty_like(rA), torch.empty_like(iA)
        ves.eigensolve(n, N // tc, tc, rA, iA, rE, iE, rV, iV, options=o)
        torch.cuda.synchronize()
        outs.append([t.cpu().numpy() for t in (rE, iE, rV, iV)])
    for other in outs[1:]:
        for a, b in zip(outs[0], other):
            assert np.array_equal(a, b)


@pytest.mark.gpu
def test_tune_varsize_same_results(tmp_path):
    """The mixed-size tuner picks among (blocks_per_sm, order); every choice
    gives the same eigenvalues and eigenvectors."""
    import torch
    import workloads
    c = autotune.TuneCache(str(tmp_path / "t.json"))
    sizes, by_n = workloads.mixed_families(1500, seed=4, nmax=24, device="cuda", as_list=False)
    e = autotune.tune_varsize(sizes, by_n, max_dim=24, candidates=(1, 3), orders=(0, 1), reps=1, cache=c)
    assert (e["blocks_per_sm"], e["varsize_order"]) in {(1, 0), (3, 0), (1, 1), (3, 1)}
    dims, re, im = workloads.pack_varsize(sizes, by_n, device="cuda")
    outs = []
    for b, order in ((1, 0), (3, 1), (0, 0)):
        o = ves.default_options(blocks_per_sm=b, varsize_order=order)
        er = torch.empty(int(sizes.sum()), dtype=torch.float64, device="cuda")
        ei, vr, vi = torch.empty_like(er), torch.empty_like(re), torch.empty_like(im)
        ves.eigensolve_varsize(len(sizes), 24, dims, re, im, er, ei, vr, vi, options=o)
        torch.cuda.synchronize()
        outs.append([t.cpu().numpy() for t in (er, ei, vr, vi)])
    for other in outs[1:]:
        for a, b in zip(outs[0], other):
            assert np.array_equal(a, b)
