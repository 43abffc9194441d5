"""float32 GEMM from scaled float16 planes (NUMC_CUDA_ALGO_SPLIT_FP16).

Each row of A and column of B is scaled by a power of two 2^s that puts its
largest magnitude in [2^14, 2^15); then x 2^s = h0 + h1 + r with h0, h1
float16 and |r| <= 2^-22 |x 2^s| (plus 2^-25 absolute where h1 falls below
float16's normal range, i.e. for entries 2^-28 below their row maximum).
Three products h0h0 + h0h1 + h1h0 are exact in FP32 and summed in
tensor-memory FP32 chains of `flush` K slabs, the chains added with
round-to-nearest.  The bound asserted relative to |A| @ |B| is
    4 * 2^-22 + 2 * (3K + 2) * 2^-24,
and against a float64 reference the error must not exceed numc's FP32 FMA
chain (the oracle) on well- and ill-scaled inputs: the point of the method.
"""
import numpy as np
import pytest

import numc_gb300 as nc
import oracle
from numc_gb300 import synth

from gpu_util import needs_gpu, rel_err_vs_scale

pytestmark = [pytest.mark.gpu, needs_gpu]
torch = pytest.importorskip("torch")


def bound(K):
    return 4 * 2.0 ** -22 + 2 * (3 * K + 2) * 2.0 ** -24


def _run(a, b, flush=0, out=None, ws=None, algo=None):
    ta = torch.from_numpy(np.ascontiguousarray(a)).cuda()
    tb = torch.from_numpy(np.ascontiguousarray(b)).cuda()
    if out is None:
        out = torch.full((a.shape[0], b.shape[1]), float("nan"), device="cuda")
    nc.gemm(ta, tb, out, algo=nc.ALGO_SPLIT_FP16 if algo is None else algo, param=flush,
            workspace=ws)
    nc.check_status()
    return out.cpu().numpy()


def test_small_integers_exact():
    a, b = synth.operands("smallint", 128, 64, 128, dtype="float32")
    np.testing.assert_array_equal(_run(a, b), oracle.matmul(a, b))


def test_identity_exact():
    # 13-bit integers need both float16 planes.
    n = 256
    a = (np.arange(n * n) % 4093 + 1).astype(np.float32).reshape(n, n)
    np.testing.assert_array_equal(_run(a, np.eye(n, dtype=np.float32)), a)


@pytest.mark.parametrize("shape", [(128, 64, 128), (256, 512, 384), (129, 65, 131),
                                   (1, 1, 1), (7, 300, 5), (300, 1000, 257),
                                   (1000, 40, 130), (64, 4096, 64)],
                         ids=lambda s: "x".join(map(str, s)))
@pytest.mark.parametrize("kind", ["uniform", "normal", "illscaled"])
def test_vs_oracle(shape, kind):
    M, K, N = shape
    a, b = synth.operands(kind, M, K, N, dtype="float32", seed=3)
    got = _run(a, b)
    assert np.isfinite(got).all()
    err = rel_err_vs_scale(got, oracle.matmul(a, b), a, b)
    assert err <= bound(K), (err, bound(K))


@pytest.mark.parametrize("flush", [1, 2, 4, 8])
def test_flush_intervals(flush):
    M, K, N = 300, 1500, 200
    a, b = synth.operands("normal", M, K, N, dtype="float32", seed=6)
    err = rel_err_vs_scale(_run(a, b, flush), oracle.matmul(a, b), a, b)
    assert err <= bound(K), (err, bound(K))


@pytest.mark.parametrize("kind", ["normal", "illscaled"])
def test_not_less_accurate_than_fp32_fma(kind):
    # Against a float64 reference the scaled float16 split must be at least
    # as accurate as numc's FP32 FMA chain, in max and mean error relative
    # to |A| @ |B|.
    M, K, N = 256, 4096, 256
    a, b = synth.operands(kind, M, K, N, dtype="float32", seed=8)
    exact = a.astype(np.float64) @ b.astype(np.float64)
    scale = np.abs(a.astype(np.float64)) @ np.abs(b.astype(np.float64))
    e16 = np.abs(_run(a, b) - exact) / scale
    efma = np.abs(oracle.matmul(a, b) - exact) / scale
    assert e16.max() <= efma.max(), (e16.max(), efma.max())
    assert e16.mean() <= efma.mean(), (e16.mean(), efma.mean())


def test_extreme_row_and_column_scales():
    # Rows of A and columns of B spread over float32's exponent range,
    # including an all-zero row, an all-subnormal row (scale exponents above
    # 126 take two exact steps) and products that only meet in the normal
    # range after both scales.
    M, K, N = 8, 256, 8
    a, b = synth.operands("normal", M, K, N, dtype="float32", seed=9)
    ra = np.array([2.0 ** 100, 2.0 ** -100, 1.0, 0.0, 2.0 ** -140, 2.0 ** 60, 2.0 ** -30, 3.0])
    cb = np.array([2.0 ** -100, 2.0 ** 100, 2.0 ** 10, 1.0, 2.0 ** 120, 2.0 ** -60, 5.0, 2.0 ** 30])
    a = (a.astype(np.float64) * ra[:, None]).astype(np.float32)
    b = (b.astype(np.float64) * cb[None, :]).astype(np.float32)
    got = _run(a, b).astype(np.float64)
    exact = a.astype(np.float64) @ b.astype(np.float64)
    scale = np.abs(a.astype(np.float64)) @ np.abs(b.astype(np.float64))
    fin = np.isfinite(scale) & (np.abs(exact) < 3e38) & (scale > 1e-30)
    assert np.all(got[3] == 0.0)
    rel = np.abs(got - exact)[fin] / scale[fin]
    assert rel.max() <= bound(K), rel.max()
    # the all-subnormal row: tiny outputs keep float32 relative accuracy
    # where they are normal
    row = 4
    ok = np.abs(exact[row]) > 2.0 ** -100
    assert np.all(np.abs(got[row][ok] - exact[row][ok]) <= 1e-5 * scale[row][ok])


def test_strided_operands_and_output():
    M, K, N = 200, 333, 150
    a, b = synth.operands("illscaled", M, K, N, dtype="float32", seed=4)
    ta = torch.from_numpy(np.ascontiguousarray(a.T)).cuda().t()
    tb = torch.from_numpy(np.ascontiguousarray(b.T)).cuda().t()
    out = torch.full((N, M), float("nan"), device="cuda").t()
    nc.gemm(ta, tb, out, algo=nc.ALGO_SPLIT_FP16)
    nc.check_status()
    assert rel_err_vs_scale(out.cpu().numpy(), oracle.matmul(a, b), a, b) <= bound(K)


def test_general_stride_views():
    # Neither dimension contiguous: the scale pass and split take their
    # scalar paths.
    M, K, N = 70, 190, 90
    a, b = synth.operands("uniform", M, K, N, dtype="float32", seed=12)
    big_a = torch.zeros((M, 2 * K), device="cuda")
    big_a[:, ::2] = torch.from_numpy(a).cuda()
    big_b = torch.zeros((2 * K, 3 * N), device="cuda")
    big_b[::2, ::3] = torch.from_numpy(b).cuda()
    out = torch.full((M, N), float("nan"), device="cuda")
    nc.gemm(big_a[:, ::2], big_b[::2, ::3], out, algo=nc.ALGO_SPLIT_FP16)
    nc.check_status()
    assert rel_err_vs_scale(out.cpu().numpy(), oracle.matmul(a, b), a, b) <= bound(K)


def test_caller_workspace_and_bad_param():
    M, K, N = 300, 200, 100
    a, b = synth.operands("uniform", M, K, N, dtype="float32", seed=5)
    need = nc.workspace_size("float32", nc.ALGO_SPLIT_FP16, 0, M, K, N)
    assert need > nc.workspace_size("float32", nc.ALGO_SPLIT_BF16, 3, M, K, N)
    ws = torch.empty(need, dtype=torch.uint8, device="cuda")
    got = _run(a, b, ws=ws)
    assert rel_err_vs_scale(got, oracle.matmul(a, b), a, b) <= bound(K)
    with pytest.raises(nc.NumcError):
        _run(a, b, ws=ws[: need - 256])
    with pytest.raises(nc.NumcError):
        _run(a, b, flush=3)
    with pytest.raises(nc.NumcError):
        x = torch.zeros((4, 4), dtype=torch.float64, device="cuda")
        nc.gemm(x, x, x, algo=nc.ALGO_SPLIT_FP16)


def test_through_numc_matmul():
    M, K, N = 512, 512, 512
    a, b = synth.operands("uniform", M, K, N, dtype="float32", seed=42)
    orig = nc.get_algo("float32")
    nc.set_algo("float32", nc.ALGO_SPLIT_FP16)
    try:
        with nc.Ctx() as ctx:
            A, B, C = ctx.from_numpy(a), ctx.from_numpy(b), ctx.zeros((M, N), "float32")
            nc.matmul(A, B, C)
            got = C.numpy()
    finally:
        nc.set_algo("float32", *orig)
    assert rel_err_vs_scale(got, oracle.matmul(a, b), a, b) <= bound(K)


def test_special_values():
    a = np.array([[np.inf, 1.0], [3e38, -2.0]], dtype=np.float32)
    b = np.array([[1.0, 0.5], [2.0, 1.0]], dtype=np.float32)
    got = _run(a, b)
    assert got[0, 0] == np.inf and got[0, 1] == np.inf
    np.testing.assert_allclose(got[1], oracle.matmul(a, b)[1], rtol=1e-6)
    a2 = np.array([[np.nan, 1.0], [1.0, 1.0]], dtype=np.float32)
    got2 = _run(a2, b)
    assert np.isnan(got2[0]).all()
    np.testing.assert_array_equal(got2[1], oracle.matmul(a2, b)[1])


_TILE_SCRIPT = r"""
import sys
import numpy as np, torch
import numc_gb300 as nc
from numc_gb300 import synth
out = []
for (M, K, N), kind in [((512, 512, 512), "normal"), ((300, 1500, 260), "illscaled"),
                        ((700, 900, 600), "uniform"), ((2000, 300, 1100), "normal")]:
    a, b = synth.operands(kind, M, K, N, dtype="float32", seed=M + N)
    c = torch.full((M, N), float("nan"), device="cuda")
    nc.gemm(torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda(), c, algo=nc.ALGO_SPLIT_FP16)
    nc.check_status()
    out.append(c.cpu().numpy().ravel())
np.save(sys.argv[1], np.concatenate(out))
"""


@pytest.mark.parametrize("ctas", ["1", "2"])
def test_tile_widths_store_identical_bits(tmp_path, ctas):
    """64-, 128- and 256-column tiles (single CTAs and CTA pairs) run the
    same per-output arithmetic: identical bits, including shapes where the
    default picks each width."""
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    res = {}
    for width in ("64", "128", "256"):
        env = dict(os.environ, NUMC_CUDA_SPLIT_TILE=width, NUMC_CUDA_SPLIT_CTAS=ctas)
        path = str(tmp_path / f"c{width}.npy")
        r = subprocess.run([sys.executable, "-c", _TILE_SCRIPT, path], env=env, cwd=root,
                           capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stderr
        res[width] = np.load(path)
    assert np.isfinite(res["128"]).all()
    np.testing.assert_array_equal(res["128"].view(np.uint32), res["256"].view(np.uint32))
    np.testing.assert_array_equal(res["64"].view(np.uint32), res["256"].view(np.uint32))


# (M, K, N), input kind, with special values
_LAYOUT_CASES = [((300, 1027, 260), "normal", False), ((513, 4097, 200), "illscaled", False),
                 ((64, 8197, 96), "uniform", False), ((256, 8192, 128), "normal", False),
                 ((130, 2048, 72), "normal", True), ((40, 1500, 33), "illscaled", True)]


def _layout_operands(shape, kind, special):
    M, K, N = shape
    a, b = synth.operands(kind, M, K, N, dtype="float32", seed=M + K)
    if special:
        a[3, 17] = np.inf
        a[70 % M, K - 1] = np.nan
        a[5, :] = 0.0
        b[K // 2, 9] = -np.inf
        b[:, 11] = 0.0
    return a, b


_LAYOUT_SCRIPT = r"""
import sys
import numpy as np, torch
import numc_gb300 as nc
sys.path.insert(0, "tests")
from test_gpu_split16 import _LAYOUT_CASES, _layout_operands
out = []
for shape, kind, special in _LAYOUT_CASES:
    M, K, N = shape
    a, b = _layout_operands(shape, kind, special)
    # A as a view with a row stride padded to a multiple of 4 floats: rows
    # k-contiguous and 16-byte aligned even where K is not a multiple of 4
    pa = torch.zeros((M, (K + 3) // 4 * 4 + 4), device="cuda")
    pa[:, :K] = torch.from_numpy(a).cuda()
    tb = torch.from_numpy(b).cuda()
    # column-major views: A's rows contiguous (A split like a row-major B),
    # B's columns contiguous along k (B split like a row-major A)
    ta_t = torch.from_numpy(np.ascontiguousarray(a.T)).cuda().t()
    tb_t = torch.from_numpy(np.ascontiguousarray(b.T)).cuda().t()
    for algo in (nc.ALGO_SPLIT_FP16, nc.ALGO_SPLIT_BF16):
        for ta, tbb in ((torch.from_numpy(a).cuda(), tb), (pa[:, :K], tb), (ta_t, tb_t)):
            c = torch.full((M, N), float("nan"), device="cuda")
            nc.gemm(ta, tbb, c, algo=algo)
            nc.check_status()
            out.append(c.cpu().numpy().ravel())
np.save(sys.argv[1], np.concatenate(out))
"""


def test_split_pass_layouts_write_same_planes(tmp_path):
    """The one-launch scale-and-split kernels (NUMC_CUDA_SPLIT_PASS bit 0:
    each k-contiguous row held in registers; bit 1: rows-contiguous operands
    — a row-major B, a column-major A — held in the registers of a cluster
    of 8 CTAs) write the same planes, maxima and non-finite flags as the
    scale pass followed by the split pass: identical output bits, with
    ragged K and N, K up to and above 8192, padded row strides, column-major
    operands, infinities, NaNs and zero rows and columns, and bfloat16
    planes unchanged; the default's float16 results meet the error bound
    against the oracle."""
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    res = {}
    for v in ("0", "1", "2", "3"):
        path = str(tmp_path / f"c{v}.npy")
        r = subprocess.run([sys.executable, "-c", _LAYOUT_SCRIPT, path],
                           env=dict(os.environ, NUMC_CUDA_SPLIT_PASS=v), cwd=root,
                           capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stderr
        res[v] = np.load(path)
    for v in ("1", "2", "3"):
        np.testing.assert_array_equal(res["0"].view(np.uint32), res[v].view(np.uint32))
    off = 0
    for shape, kind, special in _LAYOUT_CASES:
        M, K, N = shape
        a, b = _layout_operands(shape, kind, special)
        want = None if special else oracle.matmul(a, b)
        for algo in ("fp16", "bf16"):
            for _ in range(3):
                got = res["3"][off:off + M * N].reshape(M, N)
                off += M * N
                if algo == "fp16" and want is not None:
                    assert rel_err_vs_scale(got, want, a, b) <= bound(K), (shape, kind)
    assert off == res["3"].size


def test_programmatic_dependent_launch_changes_no_bits(tmp_path):
    """The GEMM launched with programmatic dependent launch after its
    operand pass (the default) and without it (NUMC_CUDA_PDL=0) store the
    same bits."""
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    res = {}
    for pdl in ("0", "1"):
        path = str(tmp_path / f"c{pdl}.npy")
        r = subprocess.run([sys.executable, "-c", _TILE_SCRIPT, path],
                           env=dict(os.environ, NUMC_CUDA_PDL=pdl), cwd=root,
                           capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stderr
        res[pdl] = np.load(path)
    np.testing.assert_array_equal(res["0"].view(np.uint32), res["1"].view(np.uint32))
