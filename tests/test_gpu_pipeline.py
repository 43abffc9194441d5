"""numc_matmul with host operands large enough for the row-panel pipeline.

Split GEMMs (SPLIT_FP16, SPLIT_BF16) whose operands live in host memory
overlap the host copies with the work: B is copied and split once, A and C
move panel by panel on their own streams.  Every output's arithmetic is the
same as in one device-resident call, so results must equal numc_cuda_gemm
on the same data bit for bit, whatever the panel boundaries.
"""
import numpy as np
import pytest

import numc_gb300 as nc
import oracle
from numc_gb300 import synth

from gpu_util import needs_gpu, rel_err_vs_scale

pytestmark = [pytest.mark.gpu, needs_gpu]
torch = pytest.importorskip("torch")


def _device_result(a, b, algo, param):
    ta, tb = torch.from_numpy(a).cuda(), torch.from_numpy(np.ascontiguousarray(b)).cuda()
    out = torch.empty((a.shape[0], b.shape[1]), device="cuda")
    nc.gemm(ta, tb, out, algo=algo, param=param)
    nc.check_status()
    return out.cpu().numpy()


def _host_result(a, b, algo, param, b_transposed=False):
    orig = nc.get_algo("float32")
    nc.set_algo("float32", algo, param)
    try:
        with nc.Ctx() as ctx:
            A = ctx.from_numpy(a)
            if b_transposed:
                B = ctx.from_numpy(np.ascontiguousarray(b.T)).transpose([1, 0])
            else:
                B = ctx.from_numpy(b)
            C = ctx.zeros((a.shape[0], b.shape[1]), "float32")
            nc.matmul(A, B, C)
            return C.numpy()
    finally:
        nc.set_algo("float32", *orig)


@pytest.mark.parametrize("shape", [(2048, 1024, 2048), (1500, 640, 4500), (4100, 256, 4100)],
                         ids=lambda s: "x".join(map(str, s)))
@pytest.mark.parametrize("algo,param", [(nc.ALGO_SPLIT_FP16, 0), (nc.ALGO_SPLIT_BF16, 3)])
def test_pipeline_equals_device_call(shape, algo, param):
    M, K, N = shape
    a, b = synth.operands("normal", M, K, N, dtype="float32", seed=17)
    got = _host_result(a, b, algo, param)
    np.testing.assert_array_equal(got, _device_result(a, b, algo, param))


def test_pipeline_transposed_b_and_accuracy():
    M, K, N = 2048, 1024, 2100
    a, b = synth.operands("illscaled", M, K, N, dtype="float32", seed=18)
    got = _host_result(a, b, nc.ALGO_SPLIT_FP16, 0, b_transposed=True)
    np.testing.assert_array_equal(got, _device_result(a, b, nc.ALGO_SPLIT_FP16, 0))
    rows = np.arange(0, M, 97)
    ref = oracle.matmul(a[rows], b)
    bound = 4 * 2.0 ** -22 + 2 * (3 * K + 2) * 2.0 ** -24
    assert rel_err_vs_scale(got[rows], ref, a[rows], b) <= bound


def test_non_contiguous_a_takes_the_plain_path():
    M, K, N = 2048, 1024, 2048
    a, b = synth.operands("uniform", M, K, N, dtype="float32", seed=19)
    orig = nc.get_algo("float32")
    nc.set_algo("float32", nc.ALGO_SPLIT_FP16)
    try:
        with nc.Ctx() as ctx:
            A = ctx.from_numpy(np.ascontiguousarray(a.T)).transpose([1, 0])   # column-major A
            B, C = ctx.from_numpy(b), ctx.zeros((M, N), "float32")
            nc.matmul(A, B, C)
            got = C.numpy()
    finally:
        nc.set_algo("float32", *orig)
    np.testing.assert_array_equal(got, _device_result(a, b, nc.ALGO_SPLIT_FP16, 0))


def test_pipeline_strided_b_moves_whole():
    # B with strided rows and columns (every other column of a wider array):
    # it moves as one column panel; results still equal the device call
    M, K, N = 2048, 1024, 2304
    a, b = synth.operands("normal", M, K, N, dtype="float32", seed=20)
    wide = np.zeros((K, 2 * N), dtype=np.float32)
    wide[:, ::2] = b
    orig = nc.get_algo("float32")
    nc.set_algo("float32", nc.ALGO_SPLIT_FP16)
    try:
        with nc.Ctx() as ctx:
            A = ctx.from_numpy(a)
            B = ctx.from_numpy(wide).slice(1, 0, 2 * N, 2)
            assert B.shape == (K, N) and B.strides == (2 * N * 4, 8)
            C = ctx.zeros((M, N), "float32")
            nc.matmul(A, B, C)
            got = C.numpy()
    finally:
        nc.set_algo("float32", *orig)
    np.testing.assert_array_equal(got, _device_result(a, b, nc.ALGO_SPLIT_FP16, 0))


@pytest.mark.parametrize("shape", [(4096, 512, 4096), (4608, 1024, 1100)],
                         ids=lambda s: "x".join(map(str, s)))
def test_pipeline_panel_grid(shape):
    # four row panels of A, four (or two ragged) column panels of B
    M, K, N = shape
    a, b = synth.operands("uniform", M, K, N, dtype="float32", seed=21)
    got = _host_result(a, b, nc.ALGO_SPLIT_FP16, 0)
    np.testing.assert_array_equal(got, _device_result(a, b, nc.ALGO_SPLIT_FP16, 0))
    got3 = _host_result(a, b, nc.ALGO_SPLIT_BF16, 3)
    np.testing.assert_array_equal(got3, _device_result(a, b, nc.ALGO_SPLIT_BF16, 3))


@pytest.mark.parametrize("panels", ["1", "3", "5"])
def test_panel_count_knob(panels, monkeypatch):
    """NUMC_CUDA_PIPE_PANELS changes only where the panels split."""
    M, K, N = 2304, 1024, 2560   # M K N >= 2^32: the pipeline's threshold
    a, b = synth.operands("normal", M, K, N, dtype="float32", seed=19)
    monkeypatch.setenv("NUMC_CUDA_PIPE_PANELS", panels)
    got = _host_result(a, b, nc.ALGO_SPLIT_FP16, 0)
    np.testing.assert_array_equal(got, _device_result(a, b, nc.ALGO_SPLIT_FP16, 0))
