"""Failure handling, exercised without faulting a GPU.

Host side: numc_cuda_debug_fail_malloc makes the library's next device
allocations fail as they would on a device that is out of memory.  The calls
that needed them return NUMC_ERR_MALLOC, and the library stays usable.

Device side: numc_cuda_debug_wait_timeout shortens every bounded mbarrier
wait of the tensor-core kernels to a few milliseconds and stops their TMA
producers from issuing loads.  No barrier ever completes, so no copy or MMA
is in flight; every wait runs out, the kernel waits for its (zero) issued
MMAs, releases its tensor memory and returns.  The status word then reads
nonzero, the call reports NUMC_ERR_INTERNAL, and the next call on the same
context and stream is correct.
"""
import numpy as np
import pytest

import numc_gb300 as nc
import oracle
from numc_gb300 import synth

from gpu_util import needs_gpu, rel_err_vs_scale

pytestmark = [pytest.mark.gpu, needs_gpu]
torch = pytest.importorskip("torch")

LIMIT_NS = 20_000_000   # 20 ms per abandoned wait


class fail_mallocs:
    def __init__(self, n):
        self.n = n

    def __enter__(self):
        nc.lib().numc_cuda_debug_fail_malloc(self.n)

    def __exit__(self, *exc):
        nc.lib().numc_cuda_debug_fail_malloc(0)


class starved_waits:
    def __enter__(self):
        torch.cuda.synchronize()
        nc.lib().numc_cuda_debug_wait_timeout(LIMIT_NS, 1)

    def __exit__(self, *exc):
        nc.lib().numc_cuda_debug_wait_timeout(0, 0)


def test_matmul_reports_err_malloc_and_recovers():
    a, b = synth.operands("uniform", 96, 130, 70, dtype="float32", seed=11)
    with nc.Ctx() as ctx:      # fresh context: its staging buffer is not allocated yet
        A, B, C = ctx.from_numpy(a), ctx.from_numpy(b), ctx.zeros((96, 70), "float32")
        with fail_mallocs(1000):
            with pytest.raises(nc.NumcError) as ei:
                nc.matmul(A, B, C)
            assert ei.value.code == nc.ERR_MALLOC
            with pytest.raises(nc.NumcError) as ei:
                A.to_device()
            assert ei.value.code == nc.ERR_MALLOC
            assert not A.is_resident()
        nc.matmul(A, B, C)
        assert C.numpy().tobytes() == oracle.matmul(a, b).tobytes()
        A.to_device()
        nc.matmul(A, B, C)
        assert C.numpy().tobytes() == oracle.matmul(a, b).tobytes()


def test_plan_create_reports_err_malloc():
    probs = [(torch.rand((40, 50), device="cuda"), torch.rand((50, 30), device="cuda"),
              torch.empty((40, 30), device="cuda"))]
    with fail_mallocs(1000):
        with pytest.raises(nc.NumcError) as ei:
            nc.GemmPlan(probs, nc.ALGO_SPLIT_FP16)
        assert ei.value.code == nc.ERR_MALLOC
    plan = nc.GemmPlan(probs, nc.ALGO_SPLIT_FP16)
    plan.run()
    torch.cuda.synchronize()
    nc.check_status()
    a, b, c = probs[0]
    a, b = a.cpu().numpy(), b.cpu().numpy()
    assert rel_err_vs_scale(c.cpu().numpy(), oracle.matmul(a, b), a, b) <= 2e-6
    plan.free()


def _gemm_case(dtype, algo, param, shape, seed):
    M, K, N = shape
    a, b = synth.operands("uniform", M, K, N, dtype=dtype, seed=seed)
    ta, tb = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    out = torch.zeros((M, N), dtype=ta.dtype, device="cuda")
    return a, b, ta, tb, out


CASES = [
    # (dtype, algo, param, (M, K, N), bound relative to |A||B|; None = bit-exact vs numc)
    ("float32", nc.ALGO_SPLIT_FP16, 0, (2048, 64, 2048), 2e-6),    # CTA pairs, 256 x 256
    ("float32", nc.ALGO_SPLIT_FP16, 0, (1300, 520, 1100), 2e-6),   # single CTAs, 128 x 128
    ("float32", nc.ALGO_SPLIT_FP16, 0, (300, 520, 270), 2e-6),     # single CTAs, 128 x 64
    ("float32", nc.ALGO_SPLIT_BF16, 6, (300, 520, 270), 2e-6),     # three planes
    ("float32", nc.ALGO_SPLIT_BF16, 3, (300, 520, 270), 2.0 ** -14),
    ("float64", nc.ALGO_OZAKI, 7, (200, 300, 150), 1e-13),         # CTA pairs
    ("int8", nc.ALGO_TC_INT8, nc.INT8_X86_AVX2, (200, 1100, 150), None),
    ("uint8", nc.ALGO_TC_INT8, nc.INT8_X86_AVX2, (200, 1100, 150), None),
    ("int8", nc.ALGO_TC_INT8, nc.INT8_X86_AVX2 + 16 * nc.INT8_TILE_PAIR256, (600, 1100, 520), None),
    ("uint8", nc.ALGO_TC_INT8, nc.INT8_ARM_NEON + 16 * nc.INT8_TILE_PAIR128, (600, 1100, 520), None),
]


@pytest.mark.parametrize("dtype,algo,param,shape,tol", CASES,
                         ids=[f"{c[0]}-algo{c[1]}-{c[2]}" for c in CASES])
def test_abandoned_waits_report_and_recover(dtype, algo, param, shape, tol):
    a, b, ta, tb, out = _gemm_case(dtype, algo, param, shape, seed=3)
    s = torch.cuda.current_stream()
    with starved_waits():
        nc.gemm(ta, tb, out, algo=algo, param=param)   # enqueues fine
        with pytest.raises(nc.NumcError) as ei:
            nc.check_status(s)
        assert ei.value.code == nc.ERR_INTERNAL
        assert "bounded wait" in ei.value.msg
    nc.check_status(s)   # the word was cleared by the read above
    nc.gemm(ta, tb, out, algo=algo, param=param)
    nc.check_status(s)
    got = out.cpu().numpy()
    want = oracle.matmul(a, b, oracle.PROFILE_ARM_NEON if algo == nc.ALGO_TC_INT8 and
                         param % 16 == nc.INT8_ARM_NEON else oracle.PROFILE_X86_AVX2)
    if tol is None:
        assert got.tobytes() == want.tobytes()
    else:
        assert rel_err_vs_scale(got, want, a, b) <= tol


def test_numc_matmul_returns_err_internal_after_abandoned_waits():
    a, b = synth.operands("normal", 260, 384, 200, dtype="float32", seed=9)
    orig = nc.get_algo("float32")
    nc.set_algo("float32", nc.ALGO_SPLIT_FP16)
    try:
        with nc.Ctx() as ctx:
            A, B, C = ctx.from_numpy(a), ctx.from_numpy(b), ctx.zeros((260, 200), "float32")
            with starved_waits():
                with pytest.raises(nc.NumcError) as ei:
                    nc.matmul(A, B, C)
                assert ei.value.code == nc.ERR_INTERNAL
            nc.matmul(A, B, C)
            assert rel_err_vs_scale(C.numpy(), oracle.matmul(a, b), a, b) <= 2e-6
    finally:
        nc.set_algo("float32", *orig)


def test_grouped_plan_reports_abandoned_waits():
    gen = torch.Generator(device="cuda").manual_seed(5)
    probs = []
    for (m, k, n) in [(200, 300, 150), (64, 640, 96), (300, 90, 260)]:
        probs.append((torch.rand((m, k), device="cuda", generator=gen) * 2 - 1,
                      torch.rand((k, n), device="cuda", generator=gen) * 2 - 1,
                      torch.zeros((m, n), device="cuda")))
    plan = nc.GemmPlan(probs, nc.ALGO_SPLIT_FP16, 0)
    info = plan.info()
    assert info["tc128"] + info["tc64"] > 0   # the tensor-core kernel runs
    with starved_waits():
        plan.run()
        with pytest.raises(nc.NumcError) as ei:
            nc.check_status()
        assert ei.value.code == nc.ERR_INTERNAL
    plan.run()
    nc.check_status()
    for a, b, c in probs:
        ah, bh = a.cpu().numpy(), b.cpu().numpy()
        assert rel_err_vs_scale(c.cpu().numpy(), oracle.matmul(ah, bh), ah, bh) <= 2e-6
    plan.free()


def test_static_entry_own_status_word_reports_abandoned_waits():
    M, K, N = 200, 320, 136
    a, b = synth.operands("uniform", M, K, N, dtype="float32", seed=12)
    ta, tb = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    out = torch.zeros((M, N), device="cuda")
    s = torch.cuda.current_stream()

    def call():
        return nc.lib().numc_cuda_sgemm_split_static(
            ta.data_ptr(), tb.data_ptr(), out.data_ptr(), M, K, N, K, 1, N, 1, N, 1, None,
            s.cuda_stream)
    with starved_waits():
        assert call() == 0
        with pytest.raises(nc.NumcError) as ei:
            nc.check_status(s)
        assert ei.value.code == nc.ERR_INTERNAL
    assert call() == 0
    nc.check_status(s)
    assert rel_err_vs_scale(out.cpu().numpy(), oracle.matmul(a, b), a, b) <= 2.0 ** -14
