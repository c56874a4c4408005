"""The tcgen05 3xTF32 GEMM against an FP64 product (partial tiles included).
The error is measured against sum_k |a_k b_k| (FP32 accumulation in TMEM) and
must be far below what a single TF32 product gives."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _tf32(x):
    """Round-to-nearest to TF32 (10 explicit mantissa bits)."""
    b = x.astype(np.float32).view(np.uint32).astype(np.uint64)
    b = (b + 0x1000) & 0xFFFFE000
    return b.astype(np.uint32).view(np.float32)


@pytest.mark.parametrize("kernel", [0, 1])
@pytest.mark.parametrize("M,N,K", [(128, 128, 32), (200, 256, 96), (512, 384, 1024), (1000, 130, 516),
                                   (300, 700, 64)])
def test_tf32x3_gemm(cuda, M, N, K, kernel):
    """kernel 0: one 128 x 128 tile per CTA; kernel 1: persistent 128 x 256
    tiles with a double TMEM accumulator (more tiles than SMs in the last case)."""
    import torch
    from bosonsupremacy_gb300 import _lib, autotune
    saved = autotune.get_knobs()
    autotune.set_knobs(gemm_kernel=kernel)
    try:
        _gemm_case(M, N, K)
    finally:
        autotune.set_knobs(**saved)


def _gemm_case(M, N, K):
    import torch
    from bosonsupremacy_gb300 import _lib
    rng = np.random.default_rng(M + N + K)
    A = rng.standard_normal((M, K)).astype(np.float32)
    B = rng.standard_normal((N, K)).astype(np.float32)
    ref = A.astype(np.float64) @ B.astype(np.float64).T
    absum = np.abs(A).astype(np.float64) @ np.abs(B).astype(np.float64).T
    At, Bt = torch.as_tensor(A).cuda(), torch.as_tensor(B).cuda()
    C = torch.full((M, N), float("nan"), dtype=torch.float32, device="cuda")
    h = _lib.Handle.get(0)
    _lib.check(_lib.load().bsg_gemm_tf32x3(h.h, At.data_ptr(), Bt.data_ptr(), C.data_ptr(), M, N, K,
                                           _lib.stream_ptr()), "bsg_gemm_tf32x3")
    got = C.cpu().numpy().astype(np.float64)
    assert np.isfinite(got).all()
    rel = np.abs(got - ref) / absum
    assert rel.max() <= 1e-5, rel.max()
    one_tf32 = np.abs(_tf32(A).astype(np.float64) @ _tf32(B).astype(np.float64).T - ref) / absum
    assert np.median(rel) * 10 <= np.median(one_tf32)


def test_persistent_gemm_many_tiles(cuda):
    """More output tiles than SMs, so every persistent CTA cycles both TMEM
    accumulators several times; both kernels agree to FP32 rounding."""
    import torch
    from bosonsupremacy_gb300 import _lib, autotune
    M, N, K = 4096, 1536, 256
    rng = np.random.default_rng(7)
    A = torch.as_tensor(rng.standard_normal((M, K)).astype(np.float32)).cuda()
    B = torch.as_tensor(rng.standard_normal((N, K)).astype(np.float32)).cuda()
    out = []
    saved = autotune.get_knobs()
    try:
        for kernel in (0, 1):
            autotune.set_knobs(gemm_kernel=kernel)
            C = torch.full((M, N), float("nan"), dtype=torch.float32, device="cuda")
            h = _lib.Handle.get(0)
            _lib.check(_lib.load().bsg_gemm_tf32x3(h.h, A.data_ptr(), B.data_ptr(), C.data_ptr(), M, N, K,
                                                   _lib.stream_ptr()), "bsg_gemm_tf32x3")
            out.append(C.cpu().numpy())
    finally:
        autotune.set_knobs(**saved)
    assert np.isfinite(out[1]).all()
    scale = np.abs(A.cpu().numpy()).astype(np.float64) @ np.abs(B.cpu().numpy()).astype(np.float64).T
    assert (np.abs(out[0].astype(np.float64) - out[1]) / scale).max() <= 1e-6


@pytest.mark.parametrize("M,N,K", [(128, 64, 64), (300, 200, 512), (77, 130, 48), (1000, 512, 2048), (40, 96, 4096)])
def test_sliced_gemm_fp64_accuracy(cuda, M, N, K):
    """bsg_gemm_sliced: FP64 operands cut into fixed-point BF16 slices, the
    slice products summed exactly per level in TMEM.  Rows of very different
    scales (2^-40 .. 2^40) and a zero row; the error is measured against
    K max|a_row| max|b_col| (the slices are fixed point per row) and must
    stay below 2^-36 of it, far below a TF32 or BF16 product's rounding."""
    import torch
    from bosonsupremacy_gb300 import ops
    rng = np.random.default_rng(M * 7 + N * 3 + K)
    A = rng.standard_normal((M, K)) * np.exp2(rng.integers(-40, 40, size=(M, 1)))
    B = rng.standard_normal((N, K)) * np.exp2(rng.integers(-40, 40, size=(N, 1)))
    A[M // 2] = 0.0
    ref = A @ B.T
    got = ops.gemm_sliced(torch.as_tensor(A).cuda(), torch.as_tensor(B).cuda()).cpu().numpy()
    assert np.isfinite(got).all()
    assert (got[M // 2] == 0).all()
    scale = K * np.abs(A).max(1)[:, None] * np.abs(B).max(1)[None, :]
    scale[scale == 0] = 1.0
    err = (np.abs(got - ref) / scale).max()
    absum = np.abs(A) @ np.abs(B).T
    absum[absum == 0] = 1.0
    print(f"sliced GEMM {M}x{N}x{K}: max err {err:.3e} of K max|a| max|b|, "
          f"{(np.abs(got - ref) / absum).max():.3e} of sum|a b|")
    assert err <= 2.0 ** -36, err
