"""GPU results against numc: golden fixtures and the oracle.

* Every golden case (outputs of numc's own numc_matmul on seeded inputs) is
  recomputed by numc_matmul on the GPU and must reproduce the SHA-256 of
  numc's output bit for bit — integers at full size (1024^3 int8, uint8,
  int32, int64 and 300x4100x4200 int8/uint8 with numc's saturating stores),
  and floats too: the CUDA-core float kernels follow numc's x86 register
  tiles (FMA chains in full tiles, per-256 K-block sums in the packed
  path's remainder tiles, unfused scalar columns on the unpacked path).
* The tensor-core float kernels are checked against the oracle with the
  error bound written in each test, relative to |A| @ |B|.
* The device-pointer C-ABI (numc_cuda_gemm) is exercised with torch CUDA
  tensors, including transposed views and a caller-provided workspace.
"""
import numpy as np
import pytest

import numc_gb300 as nc
import oracle
from numc_gb300 import synth

from gpu_util import (golden, needs_gpu, rel_err_vs_scale, sha, unit_roundoff)

pytestmark = [pytest.mark.gpu, needs_gpu]

CASES, ARRAYS = golden()


@pytest.fixture(scope="module")
def ctx():
    c = nc.Ctx()
    yield c
    c.free()


def _run_numc(ctx, a, b):
    A, B = ctx.from_numpy(a), ctx.from_numpy(b)
    C = ctx.zeros((a.shape[0], b.shape[1]), a.dtype)
    nc.matmul(A, B, C)
    return C.numpy()


@pytest.mark.parametrize("case", CASES, ids=lambda c: c["name"])
def test_golden_default_algorithms(ctx, case):
    M, K, N = case["shape"]
    dt = case["dtype"]
    a, b = synth.operands(case["kind"], M, K, N, seed=case["seed"], dtype=dt)
    cp = ctx.checkpoint()
    got = _run_numc(ctx, a, b)
    ctx.restore(cp)
    if case["stored"] == "full":
        np.testing.assert_array_equal(got, ARRAYS[case["name"]].reshape(got.shape))
    assert sha(got) == case["sha256"], f"{dt} {M}x{K}x{N} differs from numc"


@pytest.mark.parametrize("dt", ["float32", "float64"])
def test_simt_is_numc_fma_chain(ctx, dt):
    # 96 x 300 x 160 sits on numc's packed path with only full 6x16 (6x8)
    # tiles, where numc computes one FMA chain per output: bit-exact.
    a, b = synth.operands("uniform", 96, 300, 160, dtype=dt)
    got = _run_numc(ctx, a, b)
    np.testing.assert_array_equal(got, oracle.matmul(a, b))


@pytest.mark.parametrize("dt", ["float32", "float64"])
@pytest.mark.parametrize("shape", [(511, 600, 509), (512, 512, 512), (300, 257, 700),
                                   (1000, 700, 1100), (1003, 1024, 997), (70, 300, 4200),
                                   (2000, 600, 1700)],
                         ids=lambda s: "x".join(map(str, s)))
def test_remainder_tiles_every_tile_width(ctx, dt, shape):
    """numc's remainder-tile outputs (per-256 K-block sums) on each tile
    width the CUDA-core kernel picks: 32 and 64 sum them inside the tile
    kernel, 128 in the separate fix-up pass."""
    a, b = synth.operands("uniform", *shape, dtype=dt, seed=shape[1])
    np.testing.assert_array_equal(_run_numc(ctx, a, b), oracle.matmul(a, b))


@pytest.mark.parametrize("dt", ["int8", "uint8"])
@pytest.mark.parametrize("profile", [nc.INT8_X86_AVX2, nc.INT8_ARM_NEON, nc.INT8_WRAP])
def test_int8_profiles(ctx, dt, profile):
    a, b = synth.operands("uniform", 150, 1500, 140, dtype=dt)
    orig = nc.get_algo(dt)
    nc.set_algo(dt, nc.ALGO_SIMT, profile)
    try:
        got = _run_numc(ctx, a, b)
    finally:
        nc.set_algo(dt, *orig)
    np.testing.assert_array_equal(got, oracle.matmul(a, b, profile))


# ---- the device-pointer C-ABI -----------------------------------------------

torch = pytest.importorskip("torch")


def _dev(x):
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


@pytest.mark.parametrize("dt", nc.DTYPES)
def test_cabi_gemm_transposed_views(dt):
    M, K, N = 129, 515, 67
    a, b = synth.operands("uniform", M, K, N, dtype=dt, seed=21)
    ta = _dev(a.T).t()                        # column-major A
    tb = _dev(b)
    out = torch.zeros((N, M), dtype=ta.dtype, device="cuda").t()
    nc.gemm(ta, tb, out, algo=nc.ALGO_SIMT, param=nc.INT8_X86_AVX2)
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    np.testing.assert_array_equal(got, oracle.matmul(a, b))


def test_cabi_gemm_dmma():
    M, K, N = 200, 333, 150
    a, b = synth.operands("expspread", M, K, N, dtype="float64")
    out = torch.empty((M, N), dtype=torch.float64, device="cuda")
    nc.gemm(_dev(a), _dev(b), out, algo=nc.ALGO_DMMA)
    torch.cuda.synchronize()
    assert rel_err_vs_scale(out.cpu().numpy(), oracle.matmul(a, b), a, b) <= (K + 2) * 2.0 ** -53


def test_cabi_gemm_rejects_bad_args():
    x = torch.zeros((4, 4), dtype=torch.float32, device="cuda")
    L = nc.lib()
    rc = L.numc_cuda_gemm(8, nc.ALGO_SIMT, 0, x.data_ptr(), None, x.data_ptr(), 4, 4, 4,
                          4, 1, 4, 1, 4, 1, None, 0, None)
    assert rc == nc.ERR_NULL
    rc = L.numc_cuda_gemm(8, nc.ALGO_DMMA, 0, x.data_ptr(), x.data_ptr(), x.data_ptr(),
                          4, 4, 4, 4, 1, 4, 1, 4, 1, None, 0, None)
    assert rc == nc.ERR_TYPE
