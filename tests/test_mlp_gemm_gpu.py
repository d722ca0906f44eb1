"""tcgen05 BF16 GEMM with fused epilogues against a float64 numpy product of
the same bf16-rounded inputs (through the C ABI)."""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bf16_round(x):
    """Round float32 to bfloat16 (round to nearest even), returned as float32."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def _gelu(x):
    from scipy.special import erf
    return 0.5 * x * (1.0 + erf(x / np.sqrt(2.0)))


def _gelu_grad(x):
    from scipy.special import erf
    return 0.5 * (1.0 + erf(x / np.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / np.sqrt(2 * np.pi)


@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (200, 300, 5), (257, 1500, 512),
                                   (64, 17, 130), (1024, 512, 512)])
@pytest.mark.parametrize("epi", [0, 1, 2])
def test_tc_gemm_matches_numpy(M, N, K, epi):
    torch = pytest.importorskip("torch")
    from oqupy_gb300 import _native as nat
    rng = np.random.default_rng(M * 7 + N * 3 + K + epi)
    A = _bf16_round(rng.normal(size=(M, K)).astype(np.float32))
    B = _bf16_round(rng.normal(size=(N, K)).astype(np.float32) / np.sqrt(K))
    bias = rng.normal(size=N).astype(np.float32)
    z = rng.normal(size=(M, N)).astype(np.float32)
    dev = torch.device("cuda:0")
    tA = torch.from_numpy(A).to(dev).to(torch.bfloat16)
    tB = torch.from_numpy(B).to(dev).to(torch.bfloat16)
    tbias = torch.from_numpy(bias).to(dev)
    tz = torch.from_numpy(z).to(dev)
    zout = torch.zeros(M, N, device=dev)
    outf = torch.zeros(M, N, device=dev)
    outb = torch.zeros(M, N, device=dev, dtype=torch.bfloat16)
    err = torch.zeros(1, device=dev, dtype=torch.int32)
    L = nat.lib()
    nat.check(L.otb_mlp_gemm(tA.data_ptr(), tB.data_ptr(), M, N, K,
                             tbias.data_ptr() if epi != 2 else None, epi,
                             tz.data_ptr() if epi == 2 else None,
                             zout.data_ptr() if epi == 1 else None,
                             outf.data_ptr(), outb.data_ptr(), err.data_ptr(), None))
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    C = A.astype(np.float64) @ B.astype(np.float64).T
    if epi == 0:
        ref = C + bias
    elif epi == 1:
        ref = _gelu(C + bias)
        np.testing.assert_allclose(zout.cpu().numpy(), C + bias, rtol=1e-4, atol=1e-4)
    else:
        ref = C * _gelu_grad(z.astype(np.float64))
    got = outf.cpu().numpy()
    np.testing.assert_allclose(got, ref, rtol=1e-4, atol=1e-4)
    np.testing.assert_allclose(outb.float().cpu().numpy(), ref, rtol=1e-2, atol=1e-2)
