"""The tcgen05 split-BF16 contraction against a torch FP64 reference of the same product."""
import ctypes as C

import pytest
import torch

pytestmark = pytest.mark.gpu


# K > 256 streams the weights through the pipeline stages instead of keeping them resident
@pytest.mark.parametrize("M,N,K", [(128, 256, 256), (300, 256, 256), (257, 200, 64), (1000, 1288, 256),
                                   (645, 324, 976), (130, 40, 264)])
def test_gemm_mixed_matches_fp64(cuda_lib, M, N, K):
    g = torch.Generator(device="cuda").manual_seed(M + N + K)
    A = torch.randn(M, K, device="cuda", generator=g, dtype=torch.float32)
    W = torch.randn(K, N, device="cuda", generator=g, dtype=torch.float32) / K**0.5
    Cm = torch.full((M, N), float("nan"), device="cuda")
    ws = torch.empty(max(4 * N * K, 32768 * -(-N // 128) * -(-K // 64) + 4 * N), dtype=torch.uint8, device="cuda")
    status = torch.zeros(8, dtype=torch.int32, device="cuda")
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = cuda_lib.fire_gemm_mixed(s, M, N, K, C.c_void_p(A.data_ptr()), C.c_void_p(W.data_ptr()),
                                  C.c_void_p(Cm.data_ptr()), C.c_void_p(ws.data_ptr()), C.c_size_t(ws.numel()),
                                  C.c_void_p(status.data_ptr()))
    assert rc == 0
    torch.cuda.synchronize()
    assert int(status[0]) == 0
    ref = A.double() @ W.double()
    err = (Cm.double() - ref).abs().max().item()
    rms = ref.pow(2).mean().sqrt().item()
    bf16 = (A.bfloat16().double() @ W.bfloat16().double() - ref).abs().max().item()
    # K <= 256: scaled FP16 grid, ~2^-20 of a row's (column's) largest value per element; K > 256: split BF16,
    # ~2^-17 relative per product (plain BF16 ~2^-9)
    assert err < 2e-5 * rms * K**0.5, (err, rms, bf16)
    assert err < bf16 / 50


def test_gemm_mixed_rejects_unaligned_rows(cuda_lib):
    """Row strides that are not a multiple of 4 floats cannot use the vector epilogue: rejected, not run."""
    M, N, K = 64, 322, 256
    A = torch.randn(M, K, device="cuda")
    W = torch.randn(K, N, device="cuda")
    Cm = torch.full((M, N), float("nan"), device="cuda")
    ws = torch.empty(max(4 * N * K, 32768 * -(-N // 128) * -(-K // 64) + 4 * N), dtype=torch.uint8, device="cuda")
    status = torch.zeros(8, dtype=torch.int32, device="cuda")
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = cuda_lib.fire_gemm_mixed(s, M, N, K, C.c_void_p(A.data_ptr()), C.c_void_p(W.data_ptr()),
                                  C.c_void_p(Cm.data_ptr()), C.c_void_p(ws.data_ptr()), C.c_size_t(ws.numel()),
                                  C.c_void_p(status.data_ptr()))
    assert rc == 2  # FIRE_ERR_UNSUPPORTED


@pytest.mark.parametrize("M,N,K", [(256, 256, 256), (300, 1288, 256), (130, 200, 64)])
def test_gemm_mixed_exact_and_unbiased(cuda_lib, M, N, K):
    """K <= 256: rows of A and columns of W are scaled and split on the grid of their largest magnitude, so the
    hi x hi products sum exactly whatever the tensor core's accumulation rounding.  Integers of at most 8 bits (times
    powers of two) are all 'hi': the product is exact.  Positive operands (where a truncating accumulation shows as a bias) give a mean
    signed relative error far below the per-element error."""
    g = torch.Generator(device="cuda").manual_seed(M * 7 + N + K)
    ws = torch.empty(32768 * -(-N // 128) * -(-K // 64) + 4 * N, dtype=torch.uint8, device="cuda")
    status = torch.zeros(8, dtype=torch.int32, device="cuda")
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)

    def run(A, W):
        Cm = torch.full((M, N), float("nan"), device="cuda")
        rc = cuda_lib.fire_gemm_mixed(s, M, N, K, C.c_void_p(A.data_ptr()), C.c_void_p(W.data_ptr()),
                                      C.c_void_p(Cm.data_ptr()), C.c_void_p(ws.data_ptr()), C.c_size_t(ws.numel()),
                                      C.c_void_p(status.data_ptr()))
        assert rc == 0
        torch.cuda.synchronize()
        assert int(status[0]) == 0
        return Cm.double()

    A = torch.randint(-127, 128, (M, K), device="cuda", generator=g).float()
    W = torch.randint(-127, 128, (K, N), device="cuda", generator=g).float() * 2.0**-9
    assert torch.equal(run(A, W), A.double() @ W.double())
    A = torch.rand(M, K, device="cuda", generator=g) + 0.5
    W = (torch.rand(K, N, device="cuda", generator=g) + 0.5) / K
    ref = A.double() @ W.double()
    rel = (run(A, W) - ref) / ref
    assert rel.abs().max().item() < 2e-5
    assert abs(rel.mean().item()) < 1e-7, rel.mean().item()
