"""The allocation-free float32 GEMM entry point, numc_cuda_sgemm_split_static.

It serves callers that cannot call cudaMalloc when they run a product:
services that forbid device allocation after start-up, and plugins whose
host program owns all device memory through its own allocator.  It runs the
same split-BF16 kernels as numc_cuda_gemm on a 64 MiB scratch array built
into the library, so its results must agree with numc_cuda_gemm's within
the split-BF16 error bound, call after call; problems whose scratch would
not fit must be refused; and once the library's device code is loaded, its
calls must leave the device's free memory unchanged.

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
    """status: a device int32 tensor, or None for the library's own word."""
    M, K = ta.shape
    N = tb.shape[1]
    return nc.lib().numc_cuda_sgemm_split_static(
        ta.data_ptr(), tb.data_ptr(), out.data_ptr(), M, K, N,
        ta.stride(0), ta.stride(1), tb.stride(0), tb.stride(1),
        out.stride(0), out.stride(1), None if status is None else status.data_ptr(),
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
    # 4 * (2048 + 2048) * 4096 bytes of split planes are exactly the 64 MiB
    # of the array; the non-finite flag words make the problem one that
    # does not fit.
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


def test_static_scratch_largest_problem_that_fits():
    # M + N = 4095 at K = 4096: 16 KiB of the array stay free for the flags,
    # while M + N = 4096 (the case above, and this one with one more row)
    # is refused.
    M, K, N = 4031, 4096, 64
    a, b = synth.operands("uniform", M, K, N, dtype="float32", seed=4)
    ta, tb = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    status = torch.full((1,), 7, dtype=torch.int32, device="cuda")
    too_big = torch.zeros((M + 1, K), device="cuda")
    assert _static(too_big, tb, torch.empty((M + 1, N), device="cuda"), status) == nc.ERR_VALUE
    out = torch.full((M, N), float("nan"), device="cuda")
    assert _static(ta, tb, out, status) == 0, nc.last_error()
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    assert rel_err_vs_scale(out.cpu().numpy(), oracle.matmul(a, b), a, b) <= bound(K)


def test_static_scratch_own_status_word_and_no_device_allocation():
    M, K, N = 384, 640, 256
    a, b = synth.operands("normal", M, K, N, dtype="float32", seed=6)
    ta, tb = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    ref = torch.empty((M, N), device="cuda")
    nc.gemm(ta, tb, ref, algo=nc.ALGO_SPLIT_BF16)
    outs = [torch.full((M, N), float("nan"), device="cuda") for _ in range(3)]
    # The first call loads whatever device code is not loaded yet; the two
    # after it must not change the device's free memory.
    assert _static(ta, tb, outs[0], None) == 0, nc.last_error()
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for out in outs[1:]:
        assert _static(ta, tb, out, None) == 0, nc.last_error()
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    nc.check_status()   # the library's word: no bounded wait was abandoned
    want = ref.cpu().numpy()
    for out in outs:
        assert np.array_equal(out.cpu().numpy(), want)
