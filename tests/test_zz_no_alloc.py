"""The allocation-free float32 GEMM entry point, numc_cuda_sgemm_split_static.

It serves callers that cannot allocate device memory at call time (work
recorded into CUDA graphs or issued from stream callbacks, services that
forbid allocation after start-up, hosts whose device memory belongs to
another allocator).  It runs the same split-BF16 kernels as numc_cuda_gemm
on a 64 MiB scratch array built into the library, so its results must agree
with numc_cuda_gemm's within the split-BF16 error bound, call after call,
and problems whose scratch would not fit must be refused.

This file is collected last on purpose: it runs the library's static
scratch after everything else has used the GPU, and also passes alone.
"""
import ctypes

import numpy as np
import pytest

import numc_gb300 as nc
import oracle
from numc_gb300 import synth

from gpu_util import needs_gpu, rel_err_vs_scale

pytestmark = [pytest.mark.gpu, needs_gpu]
torch = pytest.importorskip("torch")


def bound(K):
    # same bound as tests/test_gpu_split.py
    return 3 * 2.0 ** -16 + 2 * (3 * K + 2) * 2.0 ** -24


def _static(ta, tb, out, status):
    M, K = ta.shape
    N = tb.shape[1]
    return nc.lib().numc_cuda_sgemm_split_static(
        ta.data_ptr(), tb.data_ptr(), out.data_ptr(), M, K, N,
        ta.stride(0), ta.stride(1), tb.stride(0), tb.stride(1),
        out.stride(0), out.stride(1), status.data_ptr(),
        torch.cuda.current_stream().cuda_stream)


def test_static_scratch_matches_gemm_two_calls_in_a_row():
    status = torch.full((1,), 7, dtype=torch.int32, device="cuda")
    # Two different problems back to back: the second call must not see the
    # first call's scratch contents.
    for seed, (M, K, N), kind in [(1, (300, 257, 200), "normal"),
                                  (2, (512, 1024, 384), "uniform")]:
        a, b = synth.operands(kind, M, K, N, dtype="float32", seed=seed)
        ta = torch.from_numpy(a).cuda()
        tb = torch.from_numpy(b).cuda()
        ref = torch.full((M, N), float("nan"), device="cuda")
        nc.gemm(ta, tb, ref, algo=nc.ALGO_SPLIT_BF16)
        out = torch.full((M, N), float("nan"), device="cuda")
        assert _static(ta, tb, out, status) == 0, nc.last_error()
        torch.cuda.synchronize()
        assert int(status.item()) == 0
        got, want = out.cpu().numpy(), ref.cpu().numpy()
        assert np.isfinite(got).all()
        assert rel_err_vs_scale(got, want, a, b) <= bound(K)
        assert rel_err_vs_scale(got, oracle.matmul(a, b), a, b) <= bound(K)


def test_static_scratch_strided_views():
    M, K, N = 130, 200, 96
    a, b = synth.operands("uniform", M, K, N, dtype="float32", seed=3)
    ta = torch.from_numpy(np.ascontiguousarray(a.T)).cuda().t()
    tb = torch.from_numpy(b).cuda()
    out = torch.full((N, M), float("nan"), device="cuda").t()
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    assert _static(ta, tb, out, status) == 0
    torch.cuda.synchronize()
    assert rel_err_vs_scale(out.cpu().numpy(), oracle.matmul(a, b), a, b) <= bound(K)


def test_static_scratch_rejects_oversize_problem():
    # 4 * (2048 + 2048) * 4096 bytes of split planes exceed the 64 MiB array.
    M, K, N = 2048, 4096, 2048
    ta = torch.zeros((M, K), device="cuda")
    tb = torch.zeros((K, N), device="cuda")
    out = torch.full((M, N), 5.0, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    rc = _static(ta, tb, out, status)
    assert rc == nc.ERR_VALUE
    assert "static scratch" in nc.last_error()[1]
    torch.cuda.synchronize()
    assert bool((out == 5.0).all())       # nothing was launched
