"""GPU test of the hand-written tensor-core update C -= A B (o3g_gemm_tf32_sub: tcgen05
kind::tf32 MMAs into tensor memory, TMA-staged operands), the trailing update of the BEM
factorisation, against an FP64 product of the same FP32 operands.

Tolerance: TF32 keeps 10 of the 23 fraction bits of every input, so each product a_ik b_kj
is off by at most 2^-9 of |a_ik b_kj|; the FP32 accumulation adds far less.  Every entry
must therefore be within 2^-9 sum_k |a_ik| |b_kj| (plus 1e-6 of the largest |C|) of the
exact result, and the result must not be the FP32 one (the tensor path is really taken)."""
import ctypes

import numpy as np
import pytest

from omega3d_gb300 import _lib as L

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("m,n,k,pad", [(128, 128, 32, 0), (200, 300, 128, 5), (1000, 513, 512, 3),
                                       (129, 257, 104, 0), (3000, 2000, 512, 32), (64, 1000, 8, 1),
                                       (5000, 3000, 256, 2)])
def test_tf32_update_matches_fp64(cuda, m, n, k, pad):
    import torch
    rng = np.random.default_rng(m + n + k)
    lda, ldb, ldc = m + pad, k + 4 * pad, m + 2 * pad
    A = np.zeros((k, lda), np.float32)      # column-major storage: A[col, row]
    B = np.zeros((n, ldb), np.float32)
    C = np.zeros((n, ldc), np.float32)
    A[:, :m] = rng.normal(size=(k, m))
    B[:, :k] = rng.normal(size=(n, k))
    C[:, :m] = rng.normal(size=(n, m))
    Ad, Bd, Cd = (torch.from_numpy(a).cuda() for a in (A, B, C))
    st = L.lib().o3g_gemm_tf32_sub(m, n, k, Ad.data_ptr(), lda, Bd.data_ptr(), ldb, Cd.data_ptr(), ldc, None)
    assert st == 0, L.lib().o3g_last_error().decode()
    torch.cuda.synchronize()
    got = Cd.cpu().numpy()
    Am = A[:, :m].T.astype(np.float64)      # m x k
    Bm = B[:, :k].T.astype(np.float64)      # k x n
    ref = C[:, :m].T.astype(np.float64) - Am @ Bm
    bound = 2.0 ** -9 * (np.abs(Am) @ np.abs(Bm)) + 1e-6 * np.abs(ref).max()
    err = np.abs(got[:, :m].T - ref)
    assert (err <= bound).all(), (err / bound).max()
    # padding rows of C untouched
    assert np.array_equal(got[:, m:], C[:, m:])
    # not the FP32 product: TF32 inputs leave a visible difference
    f32 = C[:, :m].T - (A[:, :m].T @ B[:, :k].T)
    assert np.abs(got[:, :m].T - f32).max() > 1e-5 * np.abs(f32).max()
