"""tcgen05 split-BF16 GEMM (ttg_tc_gemm_f32) against an FP64 torch product."""
import pytest

pytestmark = pytest.mark.gpu


def _ref(a, b):
    return (a.double() @ b.double())


def _rel(c, ref):
    import torch
    return float(torch.linalg.norm(c.double() - ref) / torch.linalg.norm(ref))


@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (256, 128, 128), (300, 70, 37),
                                   (1000, 128, 10), (129, 33, 200), (5, 1, 2048),
                                   (128, 256, 96)])
def test_tc_gemm_matches_fp64(ttg, M, N, K):
    import torch
    import tensor_train_gb300 as T
    g = torch.Generator(device="cuda").manual_seed(M * 7 + N * 3 + K)
    a = torch.randn(M, K, device="cuda", generator=g)
    b = torch.randn(K, N, device="cuda", generator=g)
    ref = _ref(a, b)
    c3 = T.tc_gemm(a, b, splits=3)
    c1 = T.tc_gemm(a, b, splits=1)
    torch.cuda.synchronize()
    e3, e1 = _rel(c3, ref), _rel(c1, ref)
    # split products: ~2^-17 per operand; plain BF16: ~2^-9 per operand
    assert e3 <= 3e-5, e3
    assert e1 <= 1e-2, e1
    assert e3 * 30 < e1


def test_tc_gemm_transposed_strides(ttg):
    import torch
    import tensor_train_gb300 as T
    g = torch.Generator(device="cuda").manual_seed(5)
    at = torch.randn(96, 200, device="cuda", generator=g)   # a = at^T (200 x 96)
    bt = torch.randn(130, 96, device="cuda", generator=g)   # b = bt^T (96 x 130)
    a, b = at.t(), bt.t()
    assert not a.is_contiguous() and not b.is_contiguous()
    c = T.tc_gemm(a, b, splits=3)
    assert _rel(c, _ref(a, b)) <= 3e-5


def test_tc_gemm_edge_sizes(ttg):
    import torch
    import tensor_train_gb300 as T
    a = torch.randn(17, 0, device="cuda")
    b = torch.randn(0, 9, device="cuda")
    c = T.tc_gemm(a, b)
    assert torch.count_nonzero(c) == 0
    e = T.tc_gemm(torch.randn(0, 8, device="cuda"), torch.randn(8, 4, device="cuda"))
    assert e.shape == (0, 4)
    with pytest.raises(T.TTGError):
        T.tc_gemm(torch.randn(4, 4, device="cuda"), torch.randn(4, 4, device="cuda"), splits=2)
