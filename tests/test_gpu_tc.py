"""The learned-shift network's BF16 GEMM on the tcgen05 tensor cores against a
plain fp32 product of the same BF16 values.  Shapes with K <= 256, K % 16 == 0
and N % 16 == 0 run the persistent kernel (weights resident in shared memory,
whole-K tiles); the others the K-chunked kernel."""
import pytest

import ves

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("M,N,K", [(128, 256, 64), (300, 256, 64), (1024, 256, 256), (77, 48, 256), (512, 64, 96),
                                   (5, 16, 32), (20000, 256, 256), (3000, 128, 192),
                                   (256, 256, 264), (100, 24, 40), (130, 80, 8)])
@pytest.mark.parametrize("act", [0, 1])
def test_gemm_bf16_matches_fp32_reference(M, N, K, act):
    import torch
    g = torch.Generator(device="cuda").manual_seed(M * 7 + N + K)
    A = torch.randn(M, K, generator=g, device="cuda").to(torch.bfloat16)
    Bt = (torch.randn(N, K, generator=g, device="cuda") / K ** 0.5).to(torch.bfloat16)
    bias = torch.randn(N, generator=g, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    C, Cf = ves.gemm_bf16(A, Bt, bias=bias, act=act, out_bf16=True, out_f32=True, err=err)
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    z = A.float() @ Bt.float().T + bias  # Cf: pre-activation
    ref = torch.nn.functional.gelu(z, approximate="tanh") if act else z
    assert (Cf - z).abs().max().item() <= 1e-4 * (z.abs().max().item() + 1.0)
    assert (C.float() - ref).abs().max().item() <= 1e-2 * (ref.abs().max().item() + 1.0)


@pytest.mark.parametrize("M,N,K", [(128, 256, 64), (300, 256, 64), (1024, 256, 256), (77, 48, 256), (5, 16, 32),
                                   (20000, 256, 256), (3000, 128, 192), (1024, 64, 128)])
def test_gemm_tma_equals_cp_async(M, N, K, monkeypatch):
    """The persistent GEMM loads its operands with TMA tensor-map boxes by
    default and with cp.async under VES_GEMM_TMA=0: the same shared-memory
    contents and the same MMAs, so the same results bit for bit (rows past M
    and N zero-filled by the TMA unit in the partial tiles)."""
    import torch
    g = torch.Generator(device="cuda").manual_seed(M + 3 * N + 5 * K)
    A = torch.randn(M, K, generator=g, device="cuda").to(torch.bfloat16)
    Bt = (torch.randn(N, K, generator=g, device="cuda") / K ** 0.5).to(torch.bfloat16)
    bias = torch.randn(N, generator=g, device="cuda")
    outs = []
    for mode in ("1", "0"):
        monkeypatch.setenv("VES_GEMM_TMA", mode)
        err = torch.zeros(1, dtype=torch.int32, device="cuda")
        C, Cf = ves.gemm_bf16(A, Bt, bias=bias, act=1, out_bf16=True, out_f32=True, err=err)
        torch.cuda.synchronize()
        assert int(err.item()) == 0
        outs.append((C, Cf))
    assert torch.equal(outs[0][0], outs[1][0]) and torch.equal(outs[0][1], outs[1][1])
    z = A.float() @ Bt.float().T + bias
    assert (outs[0][1] - z).abs().max().item() <= 1e-4 * (z.abs().max().item() + 1.0)
