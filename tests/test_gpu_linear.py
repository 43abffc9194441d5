"""numc_linear (out = x @ w + bias) and numc_bmm (batched numc_matmul).

Both are defined by composition with numc's own operations, so results are
checked bit for bit: numc_linear equals numc_matmul(x, w) followed by
adding bias to every row with numc's elementwise add (floats rounded once,
integers modulo 2^bits) — whether the kernel folds the bias into its store
(CUDA-core and split kernels) or runs a separate pass (int8 tensor path,
float64 DMMA and Ozaki); numc_bmm equals numc_matmul on every batch.
"""
import numpy as np
import pytest

import numc_gb300 as nc
import oracle
from numc_gb300 import synth

from gpu_util import needs_gpu

pytestmark = [pytest.mark.gpu, needs_gpu]


def _add_rows(c, bias):
    """numc's elementwise add of bias to every row, in the dtype."""
    with np.errstate(over="ignore"):
        return np.add(c, bias[None, :], dtype=c.dtype)


def _linear(x, w, bias, algo=None, param=0):
    dt = x.dtype
    orig = nc.get_algo(dt.name)
    if algo is not None:
        nc.set_algo(dt.name, algo, param)
    try:
        with nc.Ctx() as ctx:
            X, W = ctx.from_numpy(x), ctx.from_numpy(w)
            Bi = ctx.from_numpy(bias) if bias is not None else None
            O = ctx.zeros((x.shape[0], w.shape[1]), dt)
            nc.linear(X, W, Bi, O)
            Ref = ctx.zeros((x.shape[0], w.shape[1]), dt)
            nc.matmul(X, W, Ref)
            return O.numpy(), Ref.numpy()
    finally:
        nc.set_algo(dt.name, *orig)


@pytest.mark.parametrize("dt", nc.DTYPES)
def test_linear_matches_matmul_plus_bias(dt):
    M, K, N = 130, 300, 70
    x, w = synth.operands("uniform", M, K, N, dtype=dt, seed=31)
    bias = synth.array("uniform", (N,), seed=31, stream=5, dtype=dt)
    got, mm = _linear(x, w, bias)
    np.testing.assert_array_equal(mm, oracle.matmul(x, w))
    np.testing.assert_array_equal(got, _add_rows(oracle.matmul(x, w), bias))


@pytest.mark.parametrize("dt,algo,param", [
    ("int8", nc.ALGO_TC_INT8, 0),            # bias in a separate pass
    ("uint8", nc.ALGO_TC_INT8, 0),
    ("float32", nc.ALGO_SPLIT_FP16, 0),       # bias in the split epilogue
    ("float32", nc.ALGO_SPLIT_BF16, 3),
    ("float64", nc.ALGO_DMMA, 0),             # separate pass
    ("float64", nc.ALGO_OZAKI, 8),
])
def test_linear_other_algorithms(dt, algo, param):
    M, K, N = 300, 1100, 260
    x, w = synth.operands("uniform", M, K, N, dtype=dt, seed=32)
    bias = synth.array("uniform", (N,), seed=32, stream=5, dtype=dt)
    got, mm = _linear(x, w, bias, algo, param)
    np.testing.assert_array_equal(got, _add_rows(mm, bias))
    if dt in ("int8", "uint8"):
        np.testing.assert_array_equal(mm, oracle.matmul(x, w))


def test_linear_without_bias_is_matmul():
    x, w = synth.operands("normal", 64, 96, 48, dtype="float32", seed=33)
    got, mm = _linear(x, w, None)
    np.testing.assert_array_equal(got, mm)


def test_linear_validation():
    with nc.Ctx() as ctx:
        x, w = ctx.zeros((4, 5), "float32"), ctx.zeros((5, 6), "float32")
        out = ctx.zeros((4, 6), "float32")
        L = nc.lib()
        assert L.numc_linear(x.ptr, w.ptr, ctx.zeros((5,), "float32").ptr, out.ptr) == nc.ERR_SHAPE
        assert L.numc_linear(x.ptr, w.ptr, ctx.zeros((6,), "int32").ptr, out.ptr) == nc.ERR_TYPE
        assert L.numc_linear(x.ptr, None, ctx.zeros((6,), "float32").ptr, out.ptr) == nc.ERR_NULL


@pytest.mark.parametrize("dt", ["float32", "int8", "int32", "float64"])
def test_bmm_is_matmul_per_batch(dt):
    B, H, M, K, N = 2, 3, 40, 50, 30
    a = synth.array("uniform", (B, H, M, K), seed=34, stream=1, dtype=dt)
    b = synth.array("uniform", (B, H, K, N), seed=34, stream=2, dtype=dt)
    with nc.Ctx() as ctx:
        O = ctx.zeros((B, H, M, N), dt)
        nc.bmm(ctx.from_numpy(a), ctx.from_numpy(b), O)
        got = O.numpy()
    for i in range(B):
        for h in range(H):
            np.testing.assert_array_equal(got[i, h], oracle.matmul(a[i, h], b[i, h]))


def test_bmm_strided_batches():
    # attention-style: b given as the transpose of a (B, H, N, K) array
    B, H, M, K, N = 2, 2, 24, 32, 24
    a = synth.array("normal", (B, H, M, K), seed=35, stream=1, dtype="float32")
    bt = synth.array("normal", (B, H, N, K), seed=35, stream=2, dtype="float32")
    with nc.Ctx() as ctx:
        Bv = ctx.from_numpy(bt).transpose((0, 1, 3, 2))
        O = ctx.zeros((B, H, M, N), "float32")
        nc.bmm(ctx.from_numpy(a), Bv, O)
        got = O.numpy()
    for i in range(B):
        for h in range(H):
            np.testing.assert_array_equal(got[i, h], oracle.matmul(a[i, h], bt[i, h].T.copy()))


def test_bmm_validation():
    with nc.Ctx() as ctx:
        L = nc.lib()
        a = ctx.zeros((2, 3, 4), "float32")
        assert L.numc_bmm(a.ptr, ctx.zeros((3, 4, 5), "float32").ptr,
                          ctx.zeros((2, 3, 5), "float32").ptr) == nc.ERR_SHAPE
        assert L.numc_bmm(a.ptr, ctx.zeros((2, 4, 5), "float64").ptr,
                          ctx.zeros((2, 3, 5), "float32").ptr) == nc.ERR_TYPE
        assert L.numc_bmm(a.ptr, ctx.zeros((2, 4, 5), "float32").ptr,
                          ctx.zeros((2, 3, 6), "float32").ptr) == nc.ERR_SHAPE
