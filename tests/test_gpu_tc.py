"""The tcgen05 BF16 product (trekis_tc_gemm_bf16) against numpy: inputs rounded
to BF16 exactly as the kernel stages them, products accumulated in FP64 here;
the kernel accumulates in FP32, so the tolerance is FP32 rounding of K terms
(relative 1e-5 of the sum of |terms|)."""
import ctypes as C

import numpy as np
import pytest


def bf16(x):
    """Round float32 to bfloat16 (nearest even) and back."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


@pytest.mark.gpu
@pytest.mark.parametrize("M,N,K,trans_a,trans_b,acc", [
    (128, 64, 64, False, False, 0), (200, 70, 100, False, False, 0), (5, 3, 17, True, False, 0),
    (300, 130, 256, True, True, 1), (64, 64, 4096, True, False, 0)])
def test_tc_gemm_matches_numpy(gpu_lib, M, N, K, trans_a, trans_b, acc):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(M * 7 + N * 3 + K)
    a = rng.standard_normal((K, M) if trans_a else (M, K)).astype(np.float32)
    b = rng.standard_normal((N, K) if trans_b else (K, N)).astype(np.float32)
    c0 = rng.standard_normal((M, N)).astype(np.float32)
    A = a.T if trans_a else a
    B = b.T if trans_b else b
    ref = bf16(A).astype(np.float64) @ bf16(B).astype(np.float64) + (c0 if acc else 0.0)
    scale = np.abs(bf16(A)).astype(np.float64) @ np.abs(bf16(B)).astype(np.float64) + (np.abs(c0) if acc else 0.0)
    da = torch.from_numpy(a).cuda()
    db = torch.from_numpy(b).cuda()
    dc = torch.from_numpy(c0.copy()).cuda()
    as_m, as_k = (1, M) if trans_a else (K, 1)
    bs_k, bs_n = (1, K) if trans_b else (N, 1)
    rc = gpu_lib.trekis_tc_gemm_bf16(da.data_ptr(), as_m, as_k, db.data_ptr(), bs_k, bs_n, dc.data_ptr(), N,
                                     M, N, K, acc)
    assert rc == 0, gpu_lib.trekis_last_error()
    got = dc.cpu().numpy().astype(np.float64)
    err = np.abs(got - ref)
    assert np.all(err <= 1e-5 * scale + 1e-6), (np.max(err / (scale + 1e-30)), got[:2, :4], ref[:2, :4])
