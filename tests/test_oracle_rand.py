"""The oracle's restatement of numc_array_rand against numc's own outputs.

tests/golden/rand_golden.* hold sequences of numc_array_rand calls made by
the compiled numc (make_rand_golden.py): one seed (or numc's default) per
sequence, numc's OpenMP maximum set per sequence, every dtype, both sides of
the 1 MiB single-thread threshold, ragged per-thread chunks.  The oracle
must reproduce every output byte for byte, carrying its state from call to
call as numc's thread-local state carries over.
"""
import hashlib
import json
import os

import numpy as np
import pytest

import oracle

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")


def load_rand_golden():
    with open(os.path.join(GOLDEN, "rand_golden.json")) as f:
        meta = json.load(f)
    arrays = np.load(os.path.join(GOLDEN, "rand_golden.npz"))
    return meta["sequences"], arrays


def check_against_golden(entry, arrays, out):
    """Bytes of `out` equal numc's (whole, or SHA-256 plus sample)."""
    out = np.ascontiguousarray(out)
    assert list(out.shape) == entry["shape"]
    assert out.dtype.name == entry["dtype"]
    name = entry["name"]
    if entry["stored"] == "full":
        want = arrays[name]
        assert out.tobytes() == np.ascontiguousarray(want).tobytes(), name
    else:
        idx = arrays[name + "__idx"]
        got = out.reshape(-1)[idx]
        assert got.tobytes() == arrays[name].tobytes(), name
    assert hashlib.sha256(out.tobytes()).hexdigest() == entry["sha256"], name


SEQS, ARRAYS = load_rand_golden()


@pytest.mark.parametrize("si", range(len(SEQS)))
def test_oracle_rand_matches_numc(si):
    seq = SEQS[si]
    seed = seq["seed"] if seq["seed"] is not None else oracle.RAND_DEFAULT_SEED
    st = oracle.rand_seed(seed)
    for entry in seq["calls"]:
        out = oracle.rand(entry["dtype"], tuple(entry["shape"]), st, seq["omp_threads"])
        check_against_golden(entry, ARRAYS, out)


def test_oracle_rand_ranges():
    st = oracle.rand_seed(3)
    f = oracle.rand("float32", (100000,), st, 4)
    d = oracle.rand("float64", (100000,), st, 4)
    assert f.min() >= 0 and f.max() < 1 and d.min() >= 0 and d.max() < 1


def test_oracle_rand_threads_rule():
    # numc: <= 1 MiB single-threaded, else bytes / 512 KiB capped at the maximum
    assert oracle.rand_threads("float32", 262144, 8) == 0
    assert oracle.rand_threads("float32", 262145, 8) == 2
    assert oracle.rand_threads("float32", 8192 * 4096, 72) == 72
    assert oracle.rand_threads("int8", 1048577, 1) == 1
