"""Shared helpers for the GPU tests."""
import hashlib
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))

try:
    import torch
    HAVE_CUDA = torch.cuda.is_available()
except Exception:  # pragma: no cover
    torch = None
    HAVE_CUDA = False


def golden():
    cases = json.load(open(os.path.join(HERE, "golden", "golden.json")))["cases"]
    arrays = np.load(os.path.join(HERE, "golden", "golden.npz"))
    return cases, arrays


def sha(x):
    return hashlib.sha256(np.ascontiguousarray(x).tobytes()).hexdigest()


def abs_product(a, b):
    """|A| @ |B| in float64 (the scale of every rounding error bound)."""
    return np.abs(a.astype(np.float64)) @ np.abs(b.astype(np.float64))


def rel_err_vs_scale(got, ref, a, b):
    scale = abs_product(a, b)
    d = np.abs(got.astype(np.float64) - ref.astype(np.float64))
    return float(np.max(d / np.maximum(scale, np.finfo(np.float64).tiny))) if d.size else 0.0


def unit_roundoff(dtype):
    return 2.0 ** -24 if np.dtype(dtype) == np.float32 else 2.0 ** -53


needs_gpu = pytest.mark.skipif(not HAVE_CUDA, reason="needs a CUDA GPU")
