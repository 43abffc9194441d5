"""The oracle's NEON and AVX-512 profiles against numc's own builds.

tests/golden/golden_isa.{json,npz} hold numc_matmul outputs of numc's
aarch64 NEON build (src/matmul/matmul.c compiled on x86-64 against
oracle/neon_shim/arm_neon.h, a per-lane model of the NEON intrinsics) and
of its x86-64 AVX-512 build, plus numc_dot outputs of the NEON build (made
by tests/golden/make_golden.py isa).  The restatement must reproduce every
one bit for bit: NEON int8/uint8 clamp-once tiles, NEON float32/float64
register tiles and unpacked columns, AVX-512 int8/uint8 12x16 tiles, sums
past 2^31.
"""
import hashlib
import json
import os

import numpy as np
import pytest

import oracle
from numc_gb300 import synth

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = json.load(open(os.path.join(HERE, "golden", "golden_isa.json")))
ARR = np.load(os.path.join(HERE, "golden", "golden_isa.npz"))
PROFILE = {"neon": oracle.PROFILE_ARM_NEON, "avx512": oracle.PROFILE_X86_AVX512}


def check(name, got, entry):
    if entry["stored"] == "full":
        assert np.array_equal(got, ARR[name]), name
    else:
        assert np.array_equal(got.reshape(-1)[ARR[name + "__idx"]], ARR[name]), name
    assert hashlib.sha256(np.ascontiguousarray(got).tobytes()).hexdigest() == entry["sha256"]


@pytest.mark.parametrize("entry", GOLD["cases"], ids=[c["name"] for c in GOLD["cases"]])
def test_oracle_profile_matches_numc_build(entry):
    a, b = synth.operands(entry["kind"], *entry["shape"], seed=entry["seed"], dtype=entry["dtype"])
    check(entry["name"], oracle.matmul(a, b, profile=PROFILE[entry["variant"]]), entry)


@pytest.mark.parametrize("entry", GOLD["dot_cases"], ids=[c["name"] for c in GOLD["dot_cases"]])
def test_neon_numc_dot_gemm_branch_is_naive(entry):
    # numc's NEON build has no numc_dot GEMM table: its N-D branch runs the
    # naive kernels (int8 sums truncated, floats unfused)
    dt = entry["dtype"]
    kind = "normal" if np.dtype(dt).kind == "f" else "uniform"
    a = synth.array(kind, entry["a_shape"], seed=entry["seed"], stream=21, dtype=dt)
    b = synth.array(kind, entry["b_shape"], seed=entry["seed"], stream=22, dtype=dt)
    rows = a.reshape(-1, a.shape[-1])
    got = oracle.matmul(rows, b, profile=oracle.PROFILE_WRAP).reshape(a.shape[:-1] + b.shape[1:])
    check(entry["name"], got, entry)
