"""float32 split-BF16 tcgen05 GEMM against the oracle.

Error model: x = hi + lo + r with |x - hi| <= 2^-8|x| and |r| <= 2^-16|x|,
so each product is off by at most ~3 * 2^-16 |ab| (the dropped lo*lo term
plus the split residuals); 3K products are summed in FP32 in TMEM.  The
bound asserted below, relative to |A| @ |B|, is
    3 * 2^-16 + 2 * (3K + 2) * 2^-24.
Small integers (|x| < 256) split exactly (lo = 0), so integer-valued
problems must come out exact.
"""
import numpy as np
import pytest

import numc_gb300 as nc
import oracle
from numc_gb300 import synth

from gpu_util import needs_gpu, rel_err_vs_scale

pytestmark = [pytest.mark.gpu, needs_gpu]
torch = pytest.importorskip("torch")


def bound(K):
    return 3 * 2.0 ** -16 + 2 * (3 * K + 2) * 2.0 ** -24


def _split(a, b, out=None, ws=None):
    ta = torch.from_numpy(np.ascontiguousarray(a)).cuda()
    tb = torch.from_numpy(np.ascontiguousarray(b)).cuda()
    if out is None:
        out = torch.full((a.shape[0], b.shape[1]), float("nan"), device="cuda")
    nc.gemm(ta, tb, out, algo=nc.ALGO_SPLIT_BF16, workspace=ws)
    nc.check_status()
    return out.cpu().numpy()


def test_small_integers_exact():
    a, b = synth.operands("smallint", 128, 64, 128, dtype="float32")
    np.testing.assert_array_equal(_split(a, b), oracle.matmul(a, b))


def test_identity_exact():
    n = 256
    a = (np.arange(n * n) % 4093 + 1).astype(np.float32).reshape(n, n)
    np.testing.assert_array_equal(_split(a, np.eye(n, dtype=np.float32)), a)


@pytest.mark.parametrize("shape", [(128, 64, 128), (256, 512, 384), (129, 65, 131),
                                   (1, 1, 1), (7, 300, 5), (300, 1000, 257),
                                   (1000, 40, 130), (64, 4096, 64)],
                         ids=lambda s: "x".join(map(str, s)))
@pytest.mark.parametrize("kind", ["uniform", "normal", "illscaled"])
def test_split_vs_oracle(shape, kind):
    M, K, N = shape
    a, b = synth.operands(kind, M, K, N, dtype="float32", seed=3)
    got = _split(a, b)
    assert np.isfinite(got).all()
    err = rel_err_vs_scale(got, oracle.matmul(a, b), a, b)
    assert err <= bound(K), (err, bound(K))


def test_strided_operands_and_output():
    M, K, N = 200, 333, 150
    a, b = synth.operands("uniform", M, K, N, dtype="float32", seed=4)
    ta = torch.from_numpy(np.ascontiguousarray(a.T)).cuda().t()
    tb = torch.from_numpy(np.ascontiguousarray(b.T)).cuda().t()
    out = torch.full((N, M), float("nan"), device="cuda").t()
    nc.gemm(ta, tb, out, algo=nc.ALGO_SPLIT_BF16)
    nc.check_status()
    got = out.cpu().numpy()
    assert rel_err_vs_scale(got, oracle.matmul(a, b), a, b) <= bound(K)


def test_caller_workspace():
    M, K, N = 300, 200, 100
    a, b = synth.operands("uniform", M, K, N, dtype="float32", seed=5)
    need = nc.workspace_size("float32", nc.ALGO_SPLIT_BF16, 0, M, K, N)
    assert need > 0
    ws = torch.empty(need, dtype=torch.uint8, device="cuda")
    got = _split(a, b, ws=ws)
    assert rel_err_vs_scale(got, oracle.matmul(a, b), a, b) <= bound(K)
    with pytest.raises(nc.NumcError):
        _split(a, b, ws=ws[: need // 2])


def test_through_numc_matmul():
    M, K, N = 512, 512, 512
    a, b = synth.operands("uniform", M, K, N, dtype="float32", seed=42)
    nc.set_algo("float32", nc.ALGO_SPLIT_BF16)
    try:
        with nc.Ctx() as ctx:
            A, B, C = ctx.from_numpy(a), ctx.from_numpy(b), ctx.zeros((M, N), "float32")
            nc.matmul(A, B, C)
            got = C.numpy()
    finally:
        nc.set_algo("float32", nc.ALGO_SIMT)
    assert rel_err_vs_scale(got, oracle.matmul(a, b), a, b) <= bound(K)


def test_special_values():
    a = np.array([[np.inf, 1.0], [3e38, -2.0]], dtype=np.float32)
    b = np.array([[1.0, 0.5], [2.0, 1.0]], dtype=np.float32)
    got = _split(a, b)
    assert got[0, 0] == np.inf and got[0, 1] == np.inf
    np.testing.assert_allclose(got[1], oracle.matmul(a, b)[1], rtol=1e-4)
