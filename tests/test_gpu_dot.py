"""numc_dot and numc_matmul_naive on the GPU against numc's own outputs.

Every golden numc_dot case (tests/golden/, generated by numc's numc_dot:
0-D x N-D, 1-D inner products including numc's two-chunk OpenMP split,
N-D x 1-D, 1-D x N-D, the GEMM branch, transposed a / b / out views that
send numc down its naive strided branch, batched 2-D x 3-D) must reproduce
numc's output bit for bit — for floats too, since each branch follows
numc's own arithmetic.  numc_matmul_naive's float goldens likewise.
"""
import numpy as np
import pytest

import numc_gb300 as nc
import oracle

from gpu_util import golden, needs_gpu, sha
from test_oracle import GOLDEN, dot_case_arrays

pytestmark = [pytest.mark.gpu, needs_gpu]

_, ARRAYS = golden()


def _nc_view(ctx, x, perm):
    """numc array equal to x, built the way numc's test views are: the
    contiguous x.transpose(inverse(perm)) transposed by perm."""
    if perm is None:
        return ctx.from_numpy(x)
    inv = np.argsort(perm)
    return ctx.from_numpy(np.ascontiguousarray(np.asarray(x).transpose(inv))).transpose(list(perm))


def _check(case, got):
    if case["stored"] == "full":
        np.testing.assert_array_equal(got.reshape(-1), ARRAYS[case["name"]].reshape(-1))
    else:
        idx = ARRAYS[case["name"] + "__idx"]
        np.testing.assert_array_equal(got.reshape(-1)[idx], ARRAYS[case["name"]])
    assert sha(np.ascontiguousarray(got)) == case["sha256"]


def _run_dot(case, resident):
    a, b, out = dot_case_arrays(case)
    with nc.Ctx() as ctx:
        A = _nc_view(ctx, a, case["perm_a"])
        B = _nc_view(ctx, b, case["perm_b"])
        O = _nc_view(ctx, np.zeros(oracle.dot_shape(a.shape, b.shape), a.dtype),
                     case["perm_out"])
        if resident:
            A.to_device(); B.to_device(); O.to_device()
        nc.dot(A, B, O)
        if resident:
            O.to_host()
        return O.numpy()


@pytest.mark.parametrize("case", GOLDEN["dot_cases"], ids=lambda c: c["name"])
def test_dot_matches_numc(case):
    _check(case, _run_dot(case, resident=False))


@pytest.mark.parametrize("case", [c for c in GOLDEN["dot_cases"]
                                  if c["dtype"] in ("float32", "int8")],
                         ids=lambda c: c["name"])
def test_dot_device_resident(case):
    _check(case, _run_dot(case, resident=True))


@pytest.mark.parametrize("case", GOLDEN["naive_cases"], ids=lambda c: c["name"])
def test_matmul_naive_float_matches_numc(case):
    from numc_gb300 import synth
    M, K, N = case["shape"]
    a, b = synth.operands(case["kind"], M, K, N, seed=case["seed"], dtype=case["dtype"])
    with nc.Ctx() as ctx:
        A, B, C = ctx.from_numpy(a), ctx.from_numpy(b), ctx.zeros((M, N), case["dtype"])
        nc.matmul_naive(A, B, C)
        _check(case, C.numpy())


@pytest.mark.parametrize("dt", ["float32", "int16"])
def test_dot_3d_a_rows_flatten(dt):
    # numc's own row stride (a.strides[0]) reads past a 3-D a; here its
    # leading axes collapse into rows (numpy.dot's result), as the oracle.
    from numc_gb300 import synth
    a = synth.array("uniform", (3, 5, 40), seed=3, stream=1, dtype=dt)
    b = synth.array("uniform", (40, 7), seed=3, stream=2, dtype=dt)
    with nc.Ctx() as ctx:
        O = ctx.zeros((3, 5, 7), dt)
        nc.dot(ctx.from_numpy(a), ctx.from_numpy(b), O)
        np.testing.assert_array_equal(O.numpy(), oracle.dot(a, b))
        with pytest.raises(nc.NumcError):
            nc.dot(ctx.from_numpy(a), ctx.from_numpy(np.zeros((2, 40, 7), dt)),
                   ctx.zeros((3, 5, 2, 7), dt))


def test_dot_follows_the_float32_algorithm():
    # The GEMM branch runs numc_matmul's kernels: with SPLIT_FP16 selected
    # for float32 the result meets that algorithm's bound instead.
    from numc_gb300 import synth
    from gpu_util import rel_err_vs_scale
    a, b = synth.operands("normal", 300, 700, 260, dtype="float32", seed=5)
    orig = nc.get_algo("float32")
    nc.set_algo("float32", nc.ALGO_SPLIT_FP16)
    try:
        with nc.Ctx() as ctx:
            O = ctx.zeros((300, 260), "float32")
            nc.dot(ctx.from_numpy(a), ctx.from_numpy(b), O)
            got = O.numpy()
    finally:
        nc.set_algo("float32", *orig)
    K = 700
    assert rel_err_vs_scale(got, oracle.matmul(a, b), a, b) <= 4 * 2.0 ** -22 + 2 * (3 * K + 2) * 2.0 ** -24
