"""float64 Ozaki-sliced tcgen05 GEMM against the oracle.

Error model for s slices of 8 bits: each element is truncated to
|a - a~| < 2^(e_i - 8s) (e_i the row's exponent, max |a_ik| < 2^e_i), the
same for B with f_j, and the dropped diagonals (p + q >= s) add at most
K (s + 1) 2^-8s 2^(e_i+f_j).  Every slice product is exact and the
recombination is integer, so
    |C - AB|_ij <= (s + 3) K 2^-8s 2^(e_i + f_j) + 4 u |A||B|_ij ,
u = 2^-53 for the final rounding.  Integer-valued inputs that fit in the
slices come out exact.
"""
import numpy as np
import pytest

import numc_gb300 as nc
import oracle
from numc_gb300 import synth

from gpu_util import needs_gpu, rel_err_vs_scale

pytestmark = [pytest.mark.gpu, needs_gpu]
torch = pytest.importorskip("torch")


def _oz(a, b, slices, ws=None, out=None):
    ta = torch.from_numpy(np.ascontiguousarray(a)).cuda()
    tb = torch.from_numpy(np.ascontiguousarray(b)).cuda()
    if out is None:
        out = torch.full((a.shape[0], b.shape[1]), float("nan"), dtype=torch.float64,
                         device="cuda")
    nc.gemm(ta, tb, out, algo=nc.ALGO_OZAKI, param=slices, workspace=ws)
    nc.check_status()
    return out.cpu().numpy()


def _bound(a, b, s):
    K = a.shape[1]
    ea = np.frexp(np.abs(a).max(axis=1))[1].astype(np.float64)
    eb = np.frexp(np.abs(b).max(axis=0))[1].astype(np.float64)
    scale = np.ldexp(1.0, (ea[:, None] + eb[None, :]).astype(np.int64))
    absprod = np.abs(a) @ np.abs(b)
    return (s + 3) * K * 2.0 ** (-8 * s) * scale + 4 * 2.0 ** -53 * absprod


def test_small_integers_exact():
    a, b = synth.operands("smallint", 200, 300, 130, dtype="float64")
    for s in (1, 4, 7):
        np.testing.assert_array_equal(_oz(a, b, s), oracle.matmul(a, b))


def test_identity_exact():
    n = 192
    a = synth.operands("uniform", n, n, n, dtype="float64")[0]
    got = _oz(a, np.eye(n), 8)
    # 8 slices keep 64 bits of each row relative to its maximum: entries
    # within 2^11 of the row maximum are reproduced exactly.
    big = np.abs(a) >= np.abs(a).max(axis=1, keepdims=True) / 2048
    np.testing.assert_array_equal(got[big], a[big])


@pytest.mark.parametrize("slices", [3, 4, 5, 6, 7, 8])
@pytest.mark.parametrize("shape", [(128, 64, 128), (130, 1000, 257), (1, 77, 3),
                                   (300, 2100, 64)], ids=lambda s: "x".join(map(str, s)))
def test_ozaki_error_bound(shape, slices):
    M, K, N = shape
    a, b = synth.operands("expspread", M, K, N, dtype="float64", seed=13)
    got = _oz(a, b, slices)
    ref_hi, ref_lo = oracle.dot2_f64(a, b, *np.divmod(np.arange(M * N), N))
    ref = (ref_hi + ref_lo).reshape(M, N)
    err = np.abs(got - ref)
    assert (err <= _bound(a, b, slices)).all(), float((err / _bound(a, b, slices)).max())


def test_more_slices_more_accurate():
    M, K, N = 256, 1024, 256
    a, b = synth.operands("expspread", M, K, N, dtype="float64", seed=2)
    rows, cols = np.divmod(np.arange(0, M * N, 7), N)
    hi, lo = oracle.dot2_f64(a, b, rows, cols)
    absprod = (np.abs(a) @ np.abs(b))[rows, cols]
    errs = []
    for s in (4, 5, 6, 7, 8):
        got = _oz(a, b, s)[rows, cols]
        errs.append(float(np.max(np.abs((got - hi) - lo) / absprod)))
    assert all(e2 < e1 for e1, e2 in zip(errs, errs[1:])), errs
    # 8 slices: at least as accurate as native float64 (DMMA)
    out = torch.empty((M, N), dtype=torch.float64, device="cuda")
    nc.gemm(torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda(), out, algo=nc.ALGO_DMMA)
    torch.cuda.synchronize()
    e_dmma = float(np.max(np.abs((out.cpu().numpy()[rows, cols] - hi) - lo) / absprod))
    assert errs[-1] <= e_dmma, (errs, e_dmma)


def test_strided_and_through_numc_matmul():
    M, K, N = 150, 400, 90
    a, b = synth.operands("expspread", M, K, N, dtype="float64", seed=5)
    ta = torch.from_numpy(np.ascontiguousarray(a.T)).cuda().t()
    tb = torch.from_numpy(np.ascontiguousarray(b.T)).cuda().t()
    out = torch.full((N, M), float("nan"), dtype=torch.float64, device="cuda").t()
    nc.gemm(ta, tb, out, algo=nc.ALGO_OZAKI, param=7)
    nc.check_status()
    assert (np.abs(out.cpu().numpy() - oracle.matmul(a, b)) <= _bound(a, b, 7) * 2).all()
    nc.set_algo("float64", nc.ALGO_OZAKI, 7)
    try:
        with nc.Ctx() as ctx:
            A, B, C = ctx.from_numpy(a), ctx.from_numpy(b), ctx.zeros((M, N), "float64")
            nc.matmul(A, B, C)
            got = C.numpy()
    finally:
        nc.set_algo("float64", nc.ALGO_SIMT)
    assert (np.abs(got - oracle.matmul(a, b)) <= _bound(a, b, 7) * 2).all()


def test_non_finite_fallback():
    a, b = synth.operands("uniform", 140, 70, 200, dtype="float64", seed=6)
    a[3, 5] = np.inf
    b[7, 150] = np.nan
    got = _oz(a, b, 6)
    ref = oracle.matmul(a, b)
    np.testing.assert_array_equal(np.isnan(got), np.isnan(ref))
    np.testing.assert_array_equal(np.isinf(got), np.isinf(ref))
    fin = np.isfinite(ref)
    assert rel_err_vs_scale(got[fin], ref[fin], np.ones((1, 1)), np.ones((1, 1))) < 1e-6 or \
        np.allclose(got[fin], ref[fin], rtol=1e-12, atol=1e-12)


def test_zero_rows_and_k():
    a, b = synth.operands("uniform", 64, 96, 64, dtype="float64", seed=7)
    a[5] = 0.0
    b[:, 9] = 0.0
    got = _oz(a, b, 5)
    assert (got[5] == 0).all() and (got[:, 9] == 0).all()
    z = _oz(np.zeros((4, 0)), np.zeros((0, 3)), 5)
    assert (z == 0).all()


def test_tiny_and_subnormal_scales():
    # rows and columns whose maxima are tiny or subnormal: exponents come
    # from the bit patterns, slices must still reproduce the product
    a, b = synth.operands("uniform", 70, 90, 50, dtype="float64", seed=8)
    a[3] *= 2.0 ** -1030          # subnormal row
    a[4] *= 2.0 ** -900           # tiny normal row
    b[:, 7] *= 2.0 ** 600         # huge column
    got = _oz(a, b, 8)
    # Reference on power-of-two rescaled operands (no underflow in the
    # compensated dot products), scaled back with one rounding.
    ra = np.zeros(70, dtype=np.int64); ra[3], ra[4] = 1030, 900
    cb = np.zeros(50, dtype=np.int64); cb[7] = -600
    a_s, b_s = np.ldexp(a, ra[:, None]), np.ldexp(b, cb[None, :])
    hi, lo = oracle.dot2_f64(a_s, b_s, *np.divmod(np.arange(70 * 50), 50))
    ref = np.ldexp((hi + lo).reshape(70, 50), -(ra[:, None] + cb[None, :]))
    bound = np.ldexp(_bound(a_s, b_s, 8), -(ra[:, None] + cb[None, :]))
    # results in the subnormal range are rounded to multiples of 2^-1074
    assert (np.abs(got - ref) <= bound + 2.0 ** -1074).all()
    nz = ref[3] != 0
    assert np.all(np.signbit(got[3][nz]) == np.signbit(ref[3][nz]))


_KERNEL_SCRIPT = r"""
import sys
import numpy as np, torch
import numc_gb300 as nc
from numc_gb300 import synth
out = []
for (M, K, N), s in [((300, 2100, 264), 7), ((520, 700, 130), 8), ((1, 77, 3), 5)]:
    a, b = synth.operands("expspread", M, K, N, dtype="float64", seed=13)
    c = torch.full((M, N), float("nan"), dtype=torch.float64, device="cuda")
    nc.gemm(torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda(), c, algo=nc.ALGO_OZAKI, param=s)
    nc.check_status()
    out.append(c.cpu().numpy().ravel())
np.save(sys.argv[1], np.concatenate(out))
"""


@pytest.mark.parametrize("ctas", ["1", "2"], ids=["single_cta", "cta_pairs"])
def test_both_kernels_within_bound(tmp_path, ctas):
    """The CTA-pair kernel (default) and the single-CTA kernel
    (NUMC_CUDA_OZAKI_CTAS=1) each meet the error bound; the pair kernel
    rounds each diagonal's sum once instead of each chunk's."""
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    path = str(tmp_path / "c.npy")
    r = subprocess.run([sys.executable, "-c", _KERNEL_SCRIPT, path],
                       env=dict(os.environ, NUMC_CUDA_OZAKI_CTAS=ctas), cwd=root,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    got_all = np.load(path)
    off = 0
    for (M, K, N), s in [((300, 2100, 264), 7), ((520, 700, 130), 8), ((1, 77, 3), 5)]:
        a, b = synth.operands("expspread", M, K, N, dtype="float64", seed=13)
        got = got_all[off:off + M * N].reshape(M, N)
        off += M * N
        hi, lo = oracle.dot2_f64(a, b, *np.divmod(np.arange(M * N), N))
        err = np.abs(got - (hi + lo).reshape(M, N))
        assert (err <= _bound(a, b, s)).all(), (ctas, M, float((err / _bound(a, b, s)).max()))


def test_long_k_flushes_partial_sums_within_a_diagonal():
    """K = 70000, s = 8: the last diagonals have more chunks (over 2048) than
    the CTA-pair kernel's FP32 partial sums hold exactly, so they are folded
    into the int64 accumulators mid-diagonal; the bound still holds."""
    M, K, N = 130, 70000, 140
    a, b = synth.operands("expspread", M, K, N, dtype="float64", seed=17)
    got = _oz(a, b, 8)
    hi, lo = oracle.dot2_f64(a, b, *np.divmod(np.arange(M * N), N))
    err = np.abs(got - (hi + lo).reshape(M, N))
    assert (err <= _bound(a, b, 8)).all(), float((err / _bound(a, b, 8)).max())
