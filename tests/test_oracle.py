"""The oracle (numc_oracle.c) against numc's own outputs.

tests/golden/ holds outputs of the unmodified numc_matmul (x86-64 AVX2
build) on seeded inputs; the restatement must reproduce every one of them
bit for bit.  Where the reference library itself can be built (x86-64 with
the reference checkout), extra seeded cases compare against it directly.
"""
import hashlib
import json
import os

import numpy as np
import pytest

import oracle
from numc_gb300 import synth

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = json.load(open(os.path.join(HERE, "golden", "golden.json")))
ARRAYS = np.load(os.path.join(HERE, "golden", "golden.npz"))


def _check(case, out):
    if case["stored"] == "full":
        exp = ARRAYS[case["name"]]
        np.testing.assert_array_equal(out, exp.reshape(out.shape))
    else:
        idx = ARRAYS[case["name"] + "__idx"]
        np.testing.assert_array_equal(out.reshape(-1)[idx], ARRAYS[case["name"]])
    assert hashlib.sha256(out.tobytes()).hexdigest() == case["sha256"]


@pytest.mark.parametrize("case", GOLDEN["cases"], ids=lambda c: c["name"])
def test_oracle_matches_numc_golden(case):
    M, K, N = case["shape"]
    a, b = synth.operands(case["kind"], M, K, N, seed=case["seed"],
                          dtype=case["dtype"])
    _check(case, oracle.matmul(a, b, oracle.PROFILE_X86_AVX2))


def test_known_answers():
    # tests/matmul/test_matmul_naive.c:1-30: (2x3)@(3x2)
    a = np.array([[1, 2, 3], [4, 5, 6]])
    b = np.array([[7, 8], [9, 10], [11, 12]])
    for dt in ["int16", "int32", "int64", "float32", "float64", "uint16",
               "uint32", "uint64"]:
        out = oracle.matmul(a.astype(dt), b.astype(dt))
        np.testing.assert_array_equal(out, np.array([[58, 64], [139, 154]]))
    a8 = np.array([[1, 2, 3], [4, 5, 6]], dtype=np.int8)
    b8 = np.array([[1, 2], [3, 4], [5, 6]], dtype=np.int8)
    np.testing.assert_array_equal(oracle.matmul(a8, b8), [[22, 28], [49, 64]])


def test_strided_operands():
    a, b = synth.operands("uniform", 40, 30, 20, dtype="int32")
    at = np.ascontiguousarray(a.T).T      # column-major view of A
    np.testing.assert_array_equal(oracle.matmul(at, b), oracle.matmul(a, b))


def test_empty_and_zero_k():
    for dt in oracle.DTYPES:
        a = np.zeros((3, 0), dtype=dt)
        b = np.zeros((0, 4), dtype=dt)
        assert (oracle.matmul(a, b) == 0).all()
        assert oracle.matmul(np.zeros((0, 5), dt), np.zeros((5, 2), dt)).shape == (0, 2)


def test_profiles_differ_only_for_8bit():
    a, b = synth.operands("uniform", 97, 1100, 203, dtype="int8")
    x86 = oracle.matmul(a, b, oracle.PROFILE_X86_AVX2)
    neon = oracle.matmul(a, b, oracle.PROFILE_ARM_NEON)
    wrap = oracle.matmul(a, b, oracle.PROFILE_WRAP)
    exact = (a.astype(np.int64) @ b.astype(np.int64))
    np.testing.assert_array_equal(wrap, exact.astype(np.int8))
    # NEON full tiles clamp the exact sum once
    np.testing.assert_array_equal(neon[:96, :200],
                                  np.clip(exact, -128, 127)[:96, :200])
    assert (x86 != neon).any()


@pytest.mark.skipif(not oracle.reference_available(),
                    reason="numc reference library not buildable on this host")
@pytest.mark.parametrize("dt", oracle.DTYPES)
def test_oracle_matches_compiled_reference(dt):
    for shape, kind in [((61, 517, 45), "uniform"), ((6, 16, 16), "uniform"),
                        ((300, 90, 260), "smallint")]:
        a, b = synth.operands(kind, *shape, seed=11, dtype=dt)
        np.testing.assert_array_equal(oracle.matmul(a, b), oracle.ref_matmul(a, b))


# ---- numc_matmul_naive (floats) and numc_dot -------------------------------

def view_with_perm(x, perm):
    """x as a view of a contiguous array holding x.transpose(inverse(perm)):
    the same values with the strides numc's transposed operand has."""
    if perm is None:
        return np.array(x, order="C")      # keeps 0-D arrays 0-D
    inv = np.argsort(perm)
    return np.ascontiguousarray(x.transpose(inv)).transpose(perm)


def dot_case_arrays(case):
    """(a, b, out) numpy views of a golden numc_dot case (out zero-filled)."""
    from golden.make_golden import dot_operands
    a, b = dot_operands(case["dtype"], case["a_shape"], case["b_shape"], case["seed"])
    a, b = view_with_perm(a, case["perm_a"]), view_with_perm(b, case["perm_b"])
    out = view_with_perm(np.zeros(oracle.dot_shape(a.shape, b.shape), dtype=a.dtype),
                         case["perm_out"])
    return a, b, out


@pytest.mark.parametrize("case", GOLDEN["naive_cases"], ids=lambda c: c["name"])
def test_oracle_naive_float_matches_numc(case):
    M, K, N = case["shape"]
    a, b = synth.operands(case["kind"], M, K, N, seed=case["seed"], dtype=case["dtype"])
    _check(case, oracle.matmul(a, b, oracle.PROFILE_WRAP))


@pytest.mark.parametrize("case", GOLDEN["dot_cases"], ids=lambda c: c["name"])
def test_oracle_dot_matches_numc(case):
    a, b, out = dot_case_arrays(case)
    got = oracle.dot(a, b, out)
    _check(case, np.ascontiguousarray(got).reshape(oracle.dot_shape(a.shape, b.shape)))
