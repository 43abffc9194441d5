"""Host-side behaviour of the C-ABI library (no GPU needed).

The library must load, export every function include/numc/*.h declares,
keep numc's array semantics, and return numc's error codes for invalid
calls.  With no GPU it must refuse to compute (NUMC_ERR_INTERNAL) rather
than fall back to the CPU.
"""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

import numc_gb300 as nc

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "numc", "*.h")):
        text = open(h).read()
        for m in re.finditer(r"NUMC_API\s+[^;(]*?\b(numc_\w+)\s*\(", text, re.S):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def L():
    return nc.lib()


def test_exports_every_declared_symbol(L):
    names = declared_functions()
    assert len(names) >= 40
    for n in names:
        assert hasattr(L, n), f"{n} declared in include/numc but not exported"
    bound = {s[0] for s in nc.SIGNATURES}
    assert set(names) - {"numc_set_error_v"} <= bound | {"numc_set_error_v"}


def test_array_basics():
    with nc.Ctx() as ctx:
        x = np.arange(24, dtype=np.int32).reshape(4, 6)
        a = ctx.from_numpy(x)
        assert a.shape == (4, 6) and a.strides == (24, 4) and a.dtype == np.int32
        np.testing.assert_array_equal(a.numpy(), x)
        a.transpose((1, 0))
        assert a.shape == (6, 4) and a.strides == (4, 24) and not a.is_contiguous()
        np.testing.assert_array_equal(a.numpy(), x.T)
        c = a.copy()
        assert c.is_contiguous()
        np.testing.assert_array_equal(c.numpy(), x.T)
        s = ctx.from_numpy(x).slice(1, 1, 6, 2)
        np.testing.assert_array_equal(s.numpy(), x[:, 1:6:2])
        f = ctx.fill((3, 2), np.float64, 2.5)
        assert (f.numpy() == 2.5).all()
        z = ctx.zeros((2, 3), np.uint8)
        assert (z.numpy() == 0).all()


def test_checkpoint_restore():
    with nc.Ctx() as ctx:
        keep = ctx.from_numpy(np.ones((4, 4), np.float32))
        cp = ctx.checkpoint()
        for _ in range(20):
            ctx.create((1024, 1024), np.float64)   # 8 MiB each: new blocks
        ctx.restore(cp)
        np.testing.assert_array_equal(keep.numpy(), np.ones((4, 4), np.float32))
        again = ctx.create((4, 4), np.float32)
        assert again.shape == (4, 4)


def test_create_errors(L):
    assert not L.numc_array_create(None, None, 1, 0)
    assert nc.last_error()[0] == nc.ERR_NULL
    with nc.Ctx() as ctx:
        huge = (ctypes.c_size_t * 2)(1 << 62, 1 << 62)
        assert not L.numc_array_create(ctx.ptr, huge, 2, 0)
        assert nc.last_error()[0] == nc.ERR_SHAPE


def _rc(a, b, out):
    return nc.lib().numc_matmul(a.ptr if a else None, b.ptr if b else None,
                                out.ptr if out else None)


def test_matmul_validation_codes():
    # numc's own error cases (tests/matmul/test_matmul_naive.c:164-240)
    with nc.Ctx() as ctx:
        a = ctx.zeros((2, 3), np.float32)
        b = ctx.zeros((3, 2), np.float32)
        c = ctx.zeros((2, 2), np.float32)
        assert _rc(None, b, c) == nc.ERR_NULL
        assert _rc(a, ctx.zeros((3, 2), np.float64), c) == nc.ERR_TYPE
        assert _rc(a, ctx.zeros((4, 2), np.float32), c) == nc.ERR_SHAPE
        assert _rc(a, b, ctx.zeros((3, 2), np.float32)) == nc.ERR_SHAPE
        assert _rc(ctx.zeros((6,), np.float32), b, c) == nc.ERR_SHAPE
        assert nc.last_error()[1]


def _dot_rc(a, b, out):
    return nc.lib().numc_dot(a.ptr if a else None, b.ptr if b else None,
                             out.ptr if out else None)


def test_dot_validation_codes():
    # numc's _check_dot (src/reduction/dispatch.h:199-281), before any GPU work
    with nc.Ctx() as ctx:
        f = np.float32
        a, b = ctx.zeros((2, 3), f), ctx.zeros((3, 4), f)
        assert _dot_rc(None, b, ctx.zeros((2, 4), f)) == nc.ERR_NULL
        assert _dot_rc(a, ctx.zeros((3, 4), np.int32), ctx.zeros((2, 4), f)) == nc.ERR_TYPE
        assert _dot_rc(a, ctx.zeros((4, 4), f), ctx.zeros((2, 4), f)) == nc.ERR_SHAPE   # axis
        assert _dot_rc(a, b, ctx.zeros((2, 4, 1), f)) == nc.ERR_SHAPE                 # ndim
        assert _dot_rc(a, b, ctx.zeros((4, 2), f)) == nc.ERR_SHAPE                    # shape
        s = ctx.from_numpy(np.array(2.0, dtype=f))
        assert s.shape == ()
        assert _dot_rc(s, b, ctx.zeros((3,), f)) == nc.ERR_SHAPE                      # 0-D
        assert _dot_rc(s, b, ctx.zeros((3, 5), f)) == nc.ERR_SHAPE
        v = ctx.zeros((3,), f)
        assert _dot_rc(v, ctx.zeros((4,), f), ctx.zeros((1,), f)) == nc.ERR_SHAPE
        assert "dot: axis mismatch" in nc.last_error()[1]


@pytest.mark.skipif(nc.device_count() > 0, reason="checks the no-GPU behaviour")
def test_no_cpu_fallback():
    with nc.Ctx() as ctx:
        a = ctx.zeros((2, 3), np.float32)
        b = ctx.zeros((3, 2), np.float32)
        c = ctx.zeros((2, 2), np.float32)
        assert _rc(a, b, c) == nc.ERR_INTERNAL
        assert "no CUDA device" in nc.last_error()[1]


def test_rand_validation():
    # numc's _rand_impl (src/random/random.c:279-296; tests/random/test_rand.c:181-201)
    L = nc.lib()
    sh = (ctypes.c_size_t * 1)(4)
    assert not L.numc_array_rand(None, sh, 1, 8)
    assert nc.last_error()[0] == nc.ERR_NULL
    with nc.Ctx() as ctx:
        assert not L.numc_array_rand(ctx.ptr, None, 1, 8)
        assert nc.last_error()[0] == nc.ERR_NULL
        assert not L.numc_array_rand(ctx.ptr, sh, 0, 8)
        assert nc.last_error()[0] == nc.ERR_NULL
        assert not L.numc_cuda_array_rand(ctx.ptr, sh, 0, 8)
        assert nc.last_error()[0] == nc.ERR_NULL
    assert L.numc_cuda_rand_fill(99, None, 0, None) == nc.ERR_TYPE
    assert nc.rand_threads() > 0
    nc.rand_set_threads(7)
    assert nc.rand_threads() == 7
    nc.rand_set_threads(0)
    assert nc.rand_threads() > 0
    assert L.numc_cuda_rand_set_threads(-1) == nc.ERR_VALUE


@pytest.mark.skipif(nc.device_count() > 0, reason="checks the no-GPU behaviour")
def test_rand_no_cpu_fallback():
    with nc.Ctx() as ctx:
        sh = (ctypes.c_size_t * 1)(16)
        assert not nc.lib().numc_array_rand(ctx.ptr, sh, 1, 8)
        assert nc.last_error()[0] == nc.ERR_INTERNAL


def test_algo_settings():
    orig = nc.get_algo("float64")
    try:
        nc.set_algo("float64", nc.ALGO_OZAKI, 6)
        assert nc.get_algo("float64") == (nc.ALGO_OZAKI, 6)
        with pytest.raises(nc.NumcError):
            nc.set_algo("float64", nc.ALGO_OZAKI, 12)
        with pytest.raises(nc.NumcError):
            nc.set_algo("int32", nc.ALGO_SPLIT_BF16, 0)
    finally:
        nc.set_algo("float64", *orig)


def _up(x, a):
    return (x + a - 1) // a * a


@pytest.mark.parametrize("M,K,N", [(1000, 700, 300), (1, 1, 1), (4096, 4096, 4096), (129, 513, 65)])
def test_workspace_sizes(M, K, N):
    """numc_cuda_gemm_workspace_size: the layouts the kernels carve their
    scratch into (each part 256-byte aligned), computed on the host."""
    kp = _up(K, 512)
    assert nc.workspace_size("int8", nc.ALGO_TC_INT8, 0, M, K, N) == \
        _up(M * kp * 2, 256) + _up(N * kp * 2, 256)
    for s in (4, 8):
        kp = _up(K, 64)
        want = (_up(M * 8, 256) + _up(N * 8, 256) + _up(-(-M // 128) * 8, 256) +
                _up(-(-N // 64) * 8, 256) + _up(s * M * kp * 2, 256) + _up(s * N * kp * 2, 256))
        assert nc.workspace_size("float64", nc.ALGO_OZAKI, s, M, K, N) == want
    assert nc.workspace_size("float32", nc.ALGO_SIMT, 0, M, K, N) == 0
    assert nc.workspace_size("float64", nc.ALGO_DMMA, 0, M, K, N) == 0
    # split products: at least the two 16-bit planes of both operands
    assert nc.workspace_size("float32", nc.ALGO_SPLIT_FP16, 0, M, K, N) >= 4 * (M + N) * _up(K, 64)


def test_int8_tile_schedule_param():
    """NUMC_CUDA_ALGO_TC_INT8's param is the profile plus 16 x the tile
    schedule: every schedule shares the workspace layout; schedules past
    NUMC_INT8_TILE_PAIR256 and unknown profiles are refused (workspace size 0)."""
    M, K, N = 300, 1100, 520
    base = nc.workspace_size("int8", nc.ALGO_TC_INT8, nc.INT8_X86_AVX2, M, K, N)
    assert base > 0
    for tile in (nc.INT8_TILE_AUTO, nc.INT8_TILE_SINGLE, nc.INT8_TILE_PAIR128,
                 nc.INT8_TILE_PAIR256):
        for prof in (nc.INT8_X86_AVX2, nc.INT8_ARM_NEON, nc.INT8_WRAP, nc.INT8_X86_AVX512):
            assert nc.workspace_size("uint8", nc.ALGO_TC_INT8, prof + 16 * tile, M, K, N) == base
    assert nc.workspace_size("int8", nc.ALGO_TC_INT8, 16 * 4, M, K, N) == 0
    assert nc.workspace_size("int8", nc.ALGO_TC_INT8, 16 * 2 + 9, M, K, N) == 0


def test_ctx_device_usage_without_device_arrays():
    with nc.Ctx() as ctx:
        ctx.zeros((4, 4), "float32")
        assert ctx.device_usage() == (0, 0, 0)
    n = ctypes.c_size_t()
    assert nc.lib().numc_cuda_ctx_device_usage(None, ctypes.byref(n), None, None) == nc.ERR_NULL
