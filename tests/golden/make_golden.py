"""Generate golden fixtures from numc's own numc_matmul, numc_matmul_naive
and numc_dot.

Runs the unmodified numc library (compiled from the reference sources by
oracle/Makefile.ref, x86-64 AVX2 build) on seeded inputs from
numc_gb300.synth and records its outputs.  Small outputs are stored whole;
large ones as a SHA-256 of the output bytes plus a seeded sample of entries.

    python tests/golden/make_golden.py      (needs the reference checkout)
    python tests/golden/make_golden.py isa  (numc's NEON and AVX-512 builds)

Writes tests/golden/golden.json and tests/golden/golden.npz, or
tests/golden/golden_isa.json and tests/golden/golden_isa.npz.
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402
from numc_gb300 import synth  # noqa: E402

ALL = oracle.DTYPES
FULL_LIMIT = 1 << 16      # outputs up to 64 KiB are stored whole
SAMPLE = 2048             # entries sampled from larger outputs

# Shapes of numc's matmul tests (tests/matmul/test_matmul.c:713-797 edge
# shapes, :237-303 packed 256^2, :656 128^2, :682-711 67^2, and the 64^2
# identity/cross-check tests), all with numc's (i%7)+1 / (i%5)+1 fill.
NUMC_TEST_SHAPES = [
    (1, 128, 64), (64, 128, 1), (1, 64, 32), (32, 64, 1), (100, 128, 64),
    (64, 128, 100), (100, 128, 100), (50, 64, 50), (144, 256, 64),
    (148, 256, 64), (64, 256, 64), (64, 300, 64), (7, 7, 7), (97, 101, 103),
    (37, 41, 43), (67, 67, 67), (64, 64, 64), (128, 128, 128), (256, 256, 256),
]

# Seeded random cases: both sides of every dtype's unpacked/packed threshold
# (numc's gemmsup thresholds, src/matmul/matmul.c:241-256), ragged shapes,
# several K blocks, and the full-size workloads.
RANDOM_CASES = [
    (dt, "uniform", shape) for dt in ALL for shape in
    [(5, 3, 4), (33, 70, 17), (97, 1100, 203), (200, 200, 200),
     (150, 513, 300), (73, 2049, 37)]
] + [
    ("float32", "normal", (129, 257, 131)),
    ("float32", "illscaled", (96, 200, 80)),
    ("float64", "expspread", (96, 200, 80)),
    ("float32", "uniform", (512, 512, 512)),
    # several column panels of the oracle and of numc (NC = 4080), ragged
    ("float32", "uniform", (150, 300, 833)),
    ("float64", "uniform", (120, 260, 700)),
    ("float32", "normal", (100, 520, 4100)),
    ("int8", "uniform", (1024, 1024, 1024)),
    ("uint8", "uniform", (1024, 1024, 1024)),
    ("int32", "uniform", (1024, 1024, 1024)),
    ("int64", "uniform", (1024, 1024, 1024)),
    ("int8", "uniform", (300, 4100, 4200)),
    ("uint8", "uniform", (300, 4100, 4200)),
]


# numc_matmul_naive on floats (the unfused k-order chains; integers wrap and
# are covered by the int8 wrap profile tests).
NAIVE_CASES = [(dt, kind, shape) for dt in ("float32", "float64")
               for kind, shape in (("uniform", (5, 3, 4)), ("normal", (33, 70, 17)),
                                   ("normal", (97, 300, 103)))]

# numc_dot cases (a shape, b shape, a/b/out axis permutations: a permutation
# other than the identity hands numc a transposed, non-contiguous view).
DOT_SHAPES = [
    ("0d_x_2d", (), (7, 5), None, None, None),
    ("2d_x_0d", (6, 9), (), None, None, None),
    ("1d_x_1d_short", (37,), (37,), None, None, None),
    ("1d_x_1d_blocks", (1000,), (1000,), None, None, None),
    ("1d_x_1d_two_chunks", (150000,), (150000,), None, None, None),
    ("2d_x_1d", (70, 130), (130,), None, None, None),
    ("1d_x_2d", (130,), (130, 45), None, None, None),
    ("2d_x_2d_small", (5, 7, ), (7, 3), None, None, None),
    ("2d_x_2d", (97, 300, ), (300, 103), None, None, None),
    ("2d_x_2d_bT", (64, 200), (200, 50), None, (1, 0), None),
    ("2d_x_2d_aT", (64, 200), (200, 50), (1, 0), None, None),
    ("2d_x_2d_outT", (40, 120), (120, 33), None, None, (1, 0)),
    ("2d_x_3d_batched", (20, 30), (4, 30, 17), None, None, None),
    ("2d_x_3d_batched_bT", (20, 30), (3, 30, 17), None, (0, 2, 1), None),
]
DOT_DTYPES = ["int8", "uint8", "int16", "int32", "uint32", "int64", "float32", "float64"]


def record_op(cases, arrays, name, out, extra):
    entry = {"name": name, **extra,
             "sha256": hashlib.sha256(np.ascontiguousarray(out).tobytes()).hexdigest()}
    if out.nbytes <= FULL_LIMIT:
        arrays[name] = out
        entry["stored"] = "full"
    else:
        rng = np.random.default_rng(7)
        idx = np.sort(rng.choice(out.size, SAMPLE, replace=False))
        arrays[name + "__idx"] = idx.astype(np.int64)
        arrays[name] = out.reshape(-1)[idx]
        entry["stored"] = "sample"
    cases.append(entry)


def dot_operands(dt, ashape, bshape, seed):
    kind = "normal" if np.dtype(dt).kind == "f" else "uniform"
    return (synth.array(kind, ashape, seed=seed, stream=21, dtype=dt),
            synth.array(kind, bshape, seed=seed, stream=22, dtype=dt))


def record(cases, arrays, name, dt, kind, shape, seed=42):
    M, K, N = shape
    a, b = synth.operands(kind, M, K, N, seed=seed, dtype=dt)
    out = oracle.ref_matmul(a, b)
    entry = {"name": name, "dtype": dt, "kind": kind, "shape": [M, K, N],
             "seed": seed,
             "sha256": hashlib.sha256(out.tobytes()).hexdigest()}
    if out.nbytes <= FULL_LIMIT:
        arrays[name] = out
        entry["stored"] = "full"
    else:
        rng = np.random.default_rng(7)
        idx = np.sort(rng.choice(out.size, SAMPLE, replace=False))
        arrays[name + "__idx"] = idx.astype(np.int64)
        arrays[name] = out.reshape(-1)[idx]
        entry["stored"] = "sample"
    cases.append(entry)


# numc's other ISA builds (oracle/Makefile.ref targets avx512 and neon):
# tests/golden/golden_isa.{json,npz}.  NEON: every dtype through numc's
# aarch64 matmul (packed and unpacked float tiles, several column panels,
# the int8/uint8 clamp-once rule with its remainder tiles, sums past
# 2^31); AVX-512: int8/uint8 (its float64 path is the crashing one).
ISA_SHAPES = [(5, 3, 4), (5, 3, 7), (6, 9, 14), (33, 70, 17), (47, 40, 45),
              (97, 300, 103), (129, 257, 131), (200, 200, 200), (150, 513, 300),
              (241, 300, 250)]
ISA_CASES = (
    [("neon", dt, "uniform", sh) for dt in ALL for sh in ISA_SHAPES] +
    [("neon", "float32", "normal", sh) for sh in ISA_SHAPES] +
    [("neon", "float64", "normal", sh) for sh in ISA_SHAPES] +
    [("neon", "float32", "normal", (130, 700, 4100)),
     ("neon", "float64", "normal", (257, 300, 2050)),
     ("neon", "float32", "uniform", (512, 512, 512)),
     ("neon", "int8", "uniform", (1024, 1024, 1024)),
     ("neon", "uint8", "uniform", (1024, 1024, 1024)),
     ("neon", "int8", "uniform", (479, 1030, 33)),
     ("neon", "uint8", "uniform", (479, 1030, 33)),
     ("neon", "int8", "extreme", (7, 300000, 17)),
     ("neon", "uint8", "extreme", (7, 40000, 17)),
     ("neon", "int8", "extreme", (80, 2000, 70))] +
    [("avx512", dt, "uniform", sh) for dt in ("int8", "uint8") for sh in
     ISA_SHAPES + [(479, 1030, 33), (1024, 1024, 1024), (300, 4100, 4200)]] +
    [("avx512", "int8", "extreme", (13, 300000, 35)),
     ("avx512", "uint8", "extreme", (13, 40000, 35)),
     ("avx512", "int8", "extreme", (250, 2000, 70)),
     ("avx512", "uint8", "extreme", (250, 2000, 70))]
)


def make_isa_goldens():
    cases, arrays = [], {}
    for variant, dt, kind, (M, K, N) in ISA_CASES:
        name = f"{variant}_{kind}_{dt}_{M}x{K}x{N}"
        a, b = synth.operands(kind, M, K, N, seed=42, dtype=dt)
        record_op(cases, arrays, name, oracle.ref_matmul(a, b, variant=variant),
                  {"variant": variant, "dtype": dt, "kind": kind, "shape": [M, K, N],
                   "seed": 42})
        print(name, flush=True)
    # numc_dot's N-D GEMM branch of the NEON build: numc's dot.c has no GEMM
    # table there (dot.c:275-288) and runs its naive kernels; dot.c holds no
    # NEON code on that branch, so the build's scalar dot.c is numc's.
    dot_cases = []
    for dt in ("int8", "uint8", "int32", "float32", "float64"):
        for tag, ashape, bshape in (("2d_x_2d", (97, 300), (300, 103)),
                                    ("2d_x_2d_small", (5, 7), (7, 3)),
                                    ("2d_x_2d_panels", (40, 600), (600, 4100))):
            name = f"neon_dot_{tag}_{dt}"
            a, b = dot_operands(dt, ashape, bshape, 42)
            record_op(dot_cases, arrays, name, oracle.ref_dot(a, b, variant="neon"),
                      {"variant": "neon", "dtype": dt, "a_shape": list(ashape),
                       "b_shape": list(bshape), "seed": 42})
    with open(os.path.join(HERE, "golden_isa.json"), "w") as f:
        json.dump({"generator": "numc_matmul and numc_dot of numc's aarch64 NEON build "
                                "(matmul.c compiled against oracle/neon_shim) and "
                                "numc_matmul of its x86-64 AVX-512 build",
                   "cases": cases, "dot_cases": dot_cases}, f, indent=1)
    np.savez_compressed(os.path.join(HERE, "golden_isa.npz"), **arrays)


def main():
    if len(sys.argv) > 1 and sys.argv[1] == "isa":
        return make_isa_goldens()
    if not oracle.reference_available():
        sys.exit("numc reference library cannot be built on this host")
    cases, arrays = [], {}
    for dt in ALL:
        for shape in NUMC_TEST_SHAPES:
            name = f"numctest_{dt}_{'x'.join(map(str, shape))}"
            record(cases, arrays, name, dt, "smallint", shape)
    for dt, kind, shape in RANDOM_CASES:
        name = f"{kind}_{dt}_{'x'.join(map(str, shape))}"
        record(cases, arrays, name, dt, kind, shape)
        print(name, flush=True)
    naive_cases = []
    for dt, kind, shape in NAIVE_CASES:
        M, K, N = shape
        name = f"naive_{kind}_{dt}_{M}x{K}x{N}"
        a, b = synth.operands(kind, M, K, N, seed=42, dtype=dt)
        record_op(naive_cases, arrays, name, oracle.ref_matmul(a, b, naive=True),
                  {"dtype": dt, "kind": kind, "shape": [M, K, N], "seed": 42})
    dot_cases = []
    for dt in DOT_DTYPES:
        for tag, ashape, bshape, pa, pb, po in DOT_SHAPES:
            name = f"dot_{tag}_{dt}"
            if tag == "1d_x_1d_two_chunks":
                # 1.2 MB of operands: numc splits the sum into exactly two
                # OpenMP chunks (with 3 or 4 the order of the chunk sums is
                # up to the OpenMP runtime)
                n = (1200000 // 2) // np.dtype(dt).itemsize
                ashape = bshape = (n,)
            a, b = dot_operands(dt, ashape, bshape, 42)
            out = oracle.ref_dot(a, b, perm_a=pa, perm_b=pb, perm_out=po)
            record_op(dot_cases, arrays, name, out,
                      {"dtype": dt, "a_shape": list(ashape), "b_shape": list(bshape),
                       "perm_a": pa, "perm_b": pb, "perm_out": po, "seed": 42})
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump({"generator": "numc_matmul, numc_matmul_naive and numc_dot, "
                                "x86-64 AVX2 build",
                   "cases": cases, "naive_cases": naive_cases, "dot_cases": dot_cases},
                  f, indent=1)
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **arrays)


if __name__ == "__main__":
    main()
