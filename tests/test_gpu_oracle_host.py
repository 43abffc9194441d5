"""The oracle on the host that runs the GPU tests.

Every GPU test checks against the oracle, and the oracle's register-tile
shape depends on the host ISA (NEON 8 x 12 on aarch64, AVX2 6 x 16 on
x86-64), so its golden-vector checks are repeated on the machine that runs
the GPU tests.  They use no GPU; the gpu mark makes them run where the GPU
tests run.
"""
import pytest

import oracle
from numc_gb300 import synth

from test_oracle import GOLDEN, _check

pytestmark = pytest.mark.gpu

FLOAT_CASES = [c for c in GOLDEN["cases"] if c["dtype"] in ("float32", "float64")]


@pytest.mark.parametrize("case", FLOAT_CASES, ids=lambda c: c["name"])
def test_oracle_float_golden_on_this_host(case):
    M, K, N = case["shape"]
    a, b = synth.operands(case["kind"], M, K, N, seed=case["seed"], dtype=case["dtype"])
    _check(case, oracle.matmul(a, b, oracle.PROFILE_X86_AVX2))
