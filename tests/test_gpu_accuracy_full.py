"""Accuracy at the benchmark configurations' own sizes.

The fast paths exist to be faster at equal or better error than the plain
kernels, so these tests measure both on the full-size inputs and compare:

  * float32 8192^3, entries N(0,1) and the ill-scaled variant (row i of A
    times 10^u_i, column j of B times 10^v_j, u, v ~ U(-4, 4)): the 3-pass
    split from scaled float16 planes must not exceed the plain FP32-SIMT
    kernel's (numc's FMA chain) max or mean relative error on 512 sampled
    outputs against float64-accurate compensated dot products;
  * float64 4096^3, entries U[-1,1) x 2^e, e ~ U(-20, 20): Ozaki slicing with
    s = 4..8 slices against the DMMA kernel on 256 outputs checked against
    double-double dot products; the error may only shrink as slices are
    added, and s >= 7 must be at or below DMMA's;
  * 2048 uneven float32 problems plus 256 MLP chains, one grouped plan per
    phase: the float16-plane plans must not exceed the plain grouped plans'
    max or mean error relative to |A||B|.

Each test prints its table (pytest -s shows it).
"""
import numpy as np
import pytest

import numc_gb300 as nc
import oracle
from numc_gb300 import synth

from gpu_util import needs_gpu

pytestmark = [pytest.mark.gpu, needs_gpu]
torch = pytest.importorskip("torch")

SEED = 42


def _points(n, rows, cols, seed=7):
    rng = np.random.default_rng(seed)
    return rng.integers(0, rows, n), rng.integers(0, cols, n)


def _rel(got, ref, absprod):
    d = np.abs(got.astype(np.float64) - ref)
    rel = d / np.maximum(np.abs(ref), 2.0 ** -60 * absprod)
    return float(rel.max()), float(rel.mean())


@pytest.fixture(scope="module")
def f32_8192():
    M = N = K = 8192
    a_h = synth.normal(SEED, 3, (M, K), np.float32)
    b_h = synth.normal(SEED, 4, (K, N), np.float32)
    return a_h, b_h


@pytest.mark.parametrize("case", ["well_scaled", "ill_scaled"])
def test_f32_8192_split16_not_less_accurate_than_plain(f32_8192, case):
    a_h, b_h = f32_8192
    M, K = a_h.shape
    N = b_h.shape[1]
    a = torch.from_numpy(a_h).cuda()
    b = torch.from_numpy(b_h).cuda()
    if case == "ill_scaled":
        u, v = synth.ill_scales(SEED, M, N)
        a = (a.double() * torch.from_numpy(u).cuda()[:, None]).float()
        b = (b.double() * torch.from_numpy(v).cuda()[None, :]).float()
        a_h, b_h = a.cpu().numpy(), b.cpu().numpy()
    rows, cols = _points(512, M, N)
    ref = oracle.dot_f32_ref(a_h, b_h, rows, cols)
    absprod = oracle.dot_f32_ref(np.abs(a_h), np.abs(b_h), rows, cols)
    c = torch.empty((M, N), device="cuda")
    res = {}
    for name, algo in (("split16", nc.ALGO_SPLIT_FP16), ("plain", nc.ALGO_SIMT)):
        c.fill_(float("nan"))
        nc.gemm(a, b, c, algo=algo)
        nc.check_status()
        res[name] = _rel(c.cpu().numpy()[rows, cols], ref, absprod)
    print(f"\nf32 8192^3 {case}: max / mean relative error, 512 outputs: "
          f"split16 {res['split16'][0]:.3g} / {res['split16'][1]:.3g}, "
          f"plain {res['plain'][0]:.3g} / {res['plain'][1]:.3g}")
    assert res["split16"][0] <= res["plain"][0]
    assert res["split16"][1] <= res["plain"][1]


def test_f64_4096_ozaki_error_per_slice_count():
    a, b = synth.operands("expspread", 4096, 4096, 4096, dtype="float64")
    ta, tb = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    c = torch.empty((4096, 4096), dtype=torch.float64, device="cuda")
    rows, cols = _points(256, 4096, 4096)
    hi, lo = oracle.dot2_f64(a, b, rows, cols)
    absprod, _ = oracle.dot2_f64(np.abs(a), np.abs(b), rows, cols)
    err = {}
    for name, algo, param in [("dmma", nc.ALGO_DMMA, 0)] + \
            [(f"s{s}", nc.ALGO_OZAKI, s) for s in (4, 5, 6, 7, 8)]:
        c.fill_(float("nan"))
        nc.gemm(ta, tb, c, algo=algo, param=param)
        nc.check_status()
        got = c.cpu().numpy()[rows, cols]
        err[name] = float((np.abs((got - hi) - lo) / absprod).max())
    print("\nf64 4096^3 max error / (|A||B|), 256 outputs vs double-double: " +
          ", ".join(f"{k} {v:.3g}" for k, v in err.items()))
    for s in (4, 5, 6, 7):
        assert err[f"s{s + 1}"] <= err[f"s{s}"]
    assert err["s7"] <= err["dmma"]
    assert err["s8"] <= err["dmma"]


def test_grouped_2048_plus_mlp_chains_not_less_accurate_than_plain():
    dev = torch.device("cuda")
    dims, probs, chains, _ = synth.grouped_case(torch, dev, SEED)
    stats = {}
    for name, algo in (("split16", nc.ALGO_SPLIT_FP16), ("plain", nc.ALGO_SIMT)):
        for _, _, c in probs:
            c.fill_(float("nan"))
        p0 = nc.GemmPlan([(a, b, c) for a, b, c in probs], algo)
        p1 = nc.GemmPlan([(x, w1, h) for x, w1, _, h, _ in chains], algo)
        p2 = nc.GemmPlan([(h, w2, y) for _, _, w2, h, y in chains], algo)
        p0.run()
        p1.run()
        p2.run()
        torch.cuda.synchronize()
        nc.check_status()
        errs = []
        # every 97th problem and every 32nd chain (both of its GEMMs, the
        # second against the first's computed output), 64 outputs each
        pairs = [(probs[i][0], probs[i][1], probs[i][2], i) for i in range(0, len(probs), 97)]
        for j in range(0, len(chains), 32):
            x, w1, w2, h, y = chains[j]
            pairs += [(x, w1, h, 5000 + j), (h, w2, y, 6000 + j)]
        for a, b, c, seed in pairs:
            ah, bh = a.cpu().numpy(), b.cpu().numpy()
            r, cc = _points(64, ah.shape[0], bh.shape[1], seed=seed)
            ref = oracle.dot_f32_ref(ah, bh, r, cc)
            absp = oracle.dot_f32_ref(np.abs(ah), np.abs(bh), r, cc)
            errs.append(np.abs(c.cpu().numpy()[r, cc].astype(np.float64) - ref) / absp)
        errs = np.concatenate(errs)
        stats[name] = (float(errs.max()), float(errs.mean()))
        for pl in (p0, p1, p2):
            pl.free()
    print(f"\ngrouped 2048 + 256 chains, error / (|A||B|) max / mean: "
          f"split16 {stats['split16'][0]:.3g} / {stats['split16'][1]:.3g}, "
          f"plain {stats['plain'][0]:.3g} / {stats['plain'][1]:.3g}")
    assert stats["split16"][0] <= stats["plain"][0]
    assert stats["split16"][1] <= stats["plain"][1]
