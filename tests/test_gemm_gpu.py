"""The MLP's BF16 GEMM kernels -- mma.sync (m16n8k16) and tcgen05 (tensor
memory accumulator) -- against an FP64 product of the same bf16 operands, for
the operand layouts the forward and backward passes use."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bf16_bits(x):
    u = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    return (((u + 0x7FFF + ((u >> 16) & 1)) >> 16) & 0xFFFF).astype(np.uint16)


def bits_to_f64(b):
    return (b.astype(np.uint32) << 16).view(np.float32).astype(np.float64)


@pytest.fixture(scope="module")
def ctx():
    from weavess_gb300 import Context
    return Context(0)


def run(ctx, impl, A, B, transA=False, transB=False):
    """A (M x K), B (K x N) logical; stored transposed when asked."""
    M, K = A.shape
    N = B.shape[1]
    a = np.ascontiguousarray(A.T if transA else A)
    b = np.ascontiguousarray(B.T if transB else B)
    sam, sak = (1, M) if transA else (K, 1)
    sbk, sbn = (1, K) if transB else (N, 1)
    C = np.zeros((M, N), np.float32)
    ctx._check(ctx.L.wv_debug_gemm(ctx.h, impl, M, N, K, a.reshape(-1), sam, sak, b.reshape(-1), sbk, sbn, C))
    return C


@pytest.mark.parametrize("impl", [0, 1])
@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (1024, 256, 128), (200, 65, 256), (256, 256, 1000), (7, 9, 33)])
@pytest.mark.parametrize("layout", [(False, False), (True, False), (False, True)])
def test_gemm_integers_exact(ctx, impl, M, N, K, layout):
    """Small integers: every product and partial sum is exact in FP32."""
    rng = np.random.default_rng(M * 7 + N + K)
    A = bf16_bits(rng.integers(-8, 9, size=(M, K)))
    B = bf16_bits(rng.integers(-8, 9, size=(K, N)))
    C = run(ctx, impl, A, B, *layout)
    ref = bits_to_f64(A) @ bits_to_f64(B)
    assert np.array_equal(C.astype(np.float64), ref)


@pytest.mark.parametrize("impl", [0, 1])
def test_gemm_real_values(ctx, impl):
    rng = np.random.default_rng(5)
    A = bf16_bits(rng.normal(size=(300, 256)))
    B = bf16_bits(rng.normal(size=(256, 130)))
    C = run(ctx, impl, A, B)
    ref = bits_to_f64(A) @ bits_to_f64(B)
    assert np.max(np.abs(C - ref)) <= 1e-4 * np.max(np.abs(ref))
