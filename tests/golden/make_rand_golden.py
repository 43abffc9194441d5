"""Generate golden fixtures from numc's own numc_manual_seed / numc_array_rand.

Runs the unmodified numc library (compiled from the reference sources by
oracle/Makefile.ref) for sequences of numc_array_rand calls in one thread,
with numc's OpenMP maximum thread count set per sequence (the large-array
path splits the stream by thread count).  Outputs up to 64 KiB are stored
whole; larger ones as a SHA-256 of the bytes plus a seeded sample.

    python tests/golden/make_rand_golden.py      (needs the reference checkout)

Writes tests/golden/rand_golden.json and tests/golden/rand_golden.npz.
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402

FULL_LIMIT = 1 << 16
SAMPLE = 2048

# (seed or None for numc's default, OpenMP maximum, [(dtype, shape), ...])
SEQUENCES = [
    (42, 8, [("float32", (1000,)), ("int8", (7,)), ("float64", (3, 5)),
             ("uint16", (700001,)), ("float32", (300000,)), ("int64", (131073,)),
             ("uint8", (3,))]),
    (None, 4, [("int32", (10, 10)), ("float32", (2, 3, 4)), ("uint64", (5,)),
               ("int16", (1,))]),
    # 1 MiB exactly is the small path; one element more the large one
    (5, 6, [("float32", (262144,)), ("float32", (262145,)), ("uint8", (1048576,)),
            ("uint8", (1048577,)), ("float64", (131072,)), ("float64", (131073,))]),
    # ragged chunks over many threads, every dtype
    (123, 16, [("float32", (3000001,)), ("int8", (5000003,)), ("float64", (1048579,)),
               ("uint32", (262147,)), ("int16", (2000002,)), ("uint64", (300001,)),
               ("int32", (777777,)), ("uint16", (999999,)), ("int64", (140000,)),
               ("uint8", (2500001,))]),
    # a 128 MiB float32 fill with the thread count of a 72-core Grace host
    (7, 72, [("float32", (8192, 4096)), ("float32", (3,))]),
]


def main():
    if not oracle.reference_available():
        sys.exit("numc reference library cannot be built on this host")
    cases, arrays = [], {}
    for si, (seed, threads, calls) in enumerate(SEQUENCES):
        outs = oracle.ref_rand_sequence(seed, calls, threads)
        entries = []
        for ci, ((dt, shape), out) in enumerate(zip(calls, outs)):
            name = f"rand_{si}_{ci}"
            e = {"name": name, "dtype": dt, "shape": list(shape),
                 "sha256": hashlib.sha256(np.ascontiguousarray(out).tobytes()).hexdigest()}
            if out.nbytes <= FULL_LIMIT:
                arrays[name] = out
                e["stored"] = "full"
            else:
                rng = np.random.default_rng(7)
                idx = np.sort(rng.choice(out.size, SAMPLE, replace=False))
                arrays[name + "__idx"] = idx.astype(np.int64)
                arrays[name] = out.reshape(-1)[idx]
                e["stored"] = "sample"
            entries.append(e)
        cases.append({"seed": seed, "omp_threads": threads, "calls": entries})
        print(si, flush=True)
    with open(os.path.join(HERE, "rand_golden.json"), "w") as f:
        json.dump({"generator": "numc_manual_seed + numc_array_rand, x86-64 AVX2 build",
                   "sequences": cases}, f, indent=1)
    np.savez_compressed(os.path.join(HERE, "rand_golden.npz"), **arrays)


if __name__ == "__main__":
    main()
