"""Generate golden fixtures from numc's own numc_matmul.

Runs the unmodified numc library (compiled from the reference sources by
oracle/Makefile.ref, x86-64 AVX2 build) on seeded inputs from
numc_gb300.synth and records its outputs.  Small outputs are stored whole;
large ones as a SHA-256 of the output bytes plus a seeded sample of entries.

    python tests/golden/make_golden.py      (needs the reference checkout)

Writes tests/golden/golden.json and tests/golden/golden.npz.
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


def main():
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
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump({"generator": "numc_matmul, x86-64 AVX2 build",
                   "cases": cases}, f, indent=1)
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **arrays)


if __name__ == "__main__":
    main()
