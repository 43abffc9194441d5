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


def bound(K, passes=3):
    if passes == 6:
        # exact 3-plane split; dropped x1*y2 + x2*y1 + x2*y2 <= 3 * 2^-24 |xy|
        return 3 * 2.0 ** -24 + 2 * (6 * K + 2) * 2.0 ** -24
    return 3 * 2.0 ** -16 + 2 * (3 * K + 2) * 2.0 ** -24


def _split(a, b, out=None, ws=None, passes=3):
    ta = torch.from_numpy(np.ascontiguousarray(a)).cuda()
    tb = torch.from_numpy(np.ascontiguousarray(b)).cuda()
    if out is None:
        out = torch.full((a.shape[0], b.shape[1]), float("nan"), device="cuda")
    nc.gemm(ta, tb, out, algo=nc.ALGO_SPLIT_BF16, param=passes, workspace=ws)
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
@pytest.mark.parametrize("passes", [3, 6])
def test_split_vs_oracle(shape, kind, passes):
    M, K, N = shape
    a, b = synth.operands(kind, M, K, N, dtype="float32", seed=3)
    got = _split(a, b, passes=passes)
    assert np.isfinite(got).all()
    err = rel_err_vs_scale(got, oracle.matmul(a, b), a, b)
    assert err <= bound(K, passes), (err, bound(K, passes))


def test_six_passes_reach_float32_accuracy():
    # Six passes represent every float32 exactly and the slab partial sums
    # are added with round-to-nearest, so against a float64-accurate
    # reference the error must not exceed the plain FP32 FMA chain's, and
    # must be well below the 3-pass error.
    M, K, N = 256, 4096, 256
    a, b = synth.operands("normal", M, K, N, dtype="float32", seed=8)
    exact = a.astype(np.float64) @ b.astype(np.float64)
    scale = np.abs(a.astype(np.float64)) @ np.abs(b.astype(np.float64))
    e3 = np.max(np.abs(_split(a, b, passes=3) - exact) / scale)
    e6 = np.max(np.abs(_split(a, b, passes=6) - exact) / scale)
    e_fma = np.max(np.abs(oracle.matmul(a, b) - exact) / scale)
    assert e6 < e3 / 4, (e6, e3)
    assert e6 <= e_fma, (e6, e_fma)


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
