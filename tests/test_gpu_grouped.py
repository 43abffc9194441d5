"""Grouped float32 GEMM plans (numc_cuda_gemm_plan_*, numc_matmul_grouped).

Every problem of a plan must match the oracle: the CUDA-core variant is
numc's FMA chain (same bound as the single-problem SIMT kernel), the
split-BF16 variants meet the 3-pass bound of test_gpu_split.py and the
scaled float16 variants (the default) the bound of test_gpu_split16.py.
Plans run directly, replayed as CUDA graphs with changed inputs, and
captured by the caller (an MLP chain, two dependent plans in one graph).
"""
import numpy as np
import pytest

import numc_gb300 as nc
import oracle
from numc_gb300 import synth

from gpu_util import needs_gpu, rel_err_vs_scale

pytestmark = [pytest.mark.gpu, needs_gpu]
torch = pytest.importorskip("torch")


def split_bound(K):
    return 3 * 2.0 ** -16 + 2 * (3 * K + 2) * 2.0 ** -24


def f16_bound(K):
    return 4 * 2.0 ** -22 + 2 * (3 * K + 2) * 2.0 ** -24


BOUND = {nc.ALGO_SPLIT_BF16: split_bound, nc.ALGO_SPLIT_FP16: f16_bound}


def simt_bound(K):
    return (K + 2) * 2.0 ** -24


def random_problems(n, lo=16, hi=1024, seed=0):
    rng = np.random.default_rng(seed)
    dims = np.exp(rng.uniform(np.log(lo), np.log(hi), (n, 3))).round().astype(int)
    probs = []
    for i, (M, N, K) in enumerate(dims):
        a, b = synth.operands("uniform", M, K, N, dtype="float32", seed=1000 + i)
        ta = torch.from_numpy(a).cuda()
        tb = torch.from_numpy(b).cuda()
        out = torch.full((M, N), float("nan"), device="cuda")
        probs.append((ta, tb, out, a, b))
    return probs


def check_all(probs, bound):
    for ta, tb, out, a, b in probs:
        got = out.cpu().numpy()
        assert np.isfinite(got).all()
        assert rel_err_vs_scale(got, oracle.matmul(a, b), a, b) <= bound(a.shape[1])


@pytest.mark.parametrize("param", [0, 128, 64])
@pytest.mark.parametrize("algo", [nc.ALGO_SPLIT_FP16, nc.ALGO_SPLIT_BF16])
def test_split_plan_matches_oracle(param, algo):
    probs = random_problems(40, seed=1)
    plan = nc.GemmPlan([(p[0], p[1], p[2]) for p in probs], algo, param)
    plan.run()
    nc.check_status()
    check_all(probs, lambda K: max(BOUND[algo](K), simt_bound(K)))
    info = plan.info()
    assert sum(info[k] for k in ("tc128", "tc64", "simt")) == 40
    if param == 128:
        assert info["tc128"] == 40
    plan.free()


def test_simt_plan_is_numc_arithmetic():
    probs = random_problems(30, hi=300, seed=2)
    plan = nc.GemmPlan([(p[0], p[1], p[2]) for p in probs], nc.ALGO_SIMT)
    plan.run()
    torch.cuda.synchronize()
    for ta, tb, out, a, b in probs:
        single = torch.empty_like(out)
        nc.gemm(ta, tb, single, algo=nc.ALGO_SIMT)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(out.cpu().numpy(), single.cpu().numpy())
    check_all(probs, simt_bound)


@pytest.mark.parametrize("algo", [nc.ALGO_SPLIT_FP16, nc.ALGO_SPLIT_BF16])
def test_graph_replay_sees_new_inputs(algo):
    probs = random_problems(12, seed=3)
    plan = nc.GemmPlan([(p[0], p[1], p[2]) for p in probs], algo)
    plan.run(graph=True)
    for ta, tb, out, a, b in probs:     # new values, same buffers
        ta.mul_(-2.0)
    plan.run(graph=True)
    nc.check_status()
    for ta, tb, out, a, b in probs:
        got = out.cpu().numpy()
        a2 = a * np.float32(-2.0)
        assert rel_err_vs_scale(got, oracle.matmul(a2, b), a2, b) <= \
            max(BOUND[algo](a.shape[1]), simt_bound(a.shape[1]))


def test_mlp_chains_in_one_captured_graph():
    # 16 chains X[256,784] @ W1[784,128] -> H; H @ W2[128,10] -> Y
    chains = []
    for c in range(16):
        x = synth.uniform(7, 100 + c, (256, 784))
        w1 = (0.05 * synth.normal(7, 200 + c, (784, 128))).astype(np.float32)
        w2 = (0.05 * synth.normal(7, 300 + c, (128, 10))).astype(np.float32)
        t = [torch.from_numpy(v).cuda() for v in (x, w1, w2)]
        h = torch.empty((256, 128), device="cuda")
        y = torch.empty((256, 10), device="cuda")
        chains.append((x, w1, w2, t, h, y))
    p1 = nc.GemmPlan([(t[0], t[1], h) for _, _, _, t, h, _ in chains])
    p2 = nc.GemmPlan([(h, t[2], y) for _, _, _, t, h, y in chains])
    s = torch.cuda.Stream()
    p1.run(stream=s)           # warm (first use loads kernels)
    p2.run(stream=s)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        p1.run(stream=s)
        p2.run(stream=s)
    for _, _, _, _, h, y in chains:
        h.zero_(); y.zero_()
    g.replay()
    torch.cuda.synchronize()
    nc.check_status()
    for x, w1, w2, t, h, y in chains:
        ref_h = oracle.matmul(x, w1)
        assert rel_err_vs_scale(h.cpu().numpy(), ref_h, x, w1) <= f16_bound(784)
        ref_y = oracle.matmul(ref_h, w2)
        err = np.abs(y.cpu().numpy().astype(np.float64) - ref_y)
        assert err.max() <= 1e-4 * (np.abs(ref_h) @ np.abs(w2)).max()


@pytest.mark.parametrize("f32_algo", [nc.ALGO_AUTO, nc.ALGO_SPLIT_BF16])
def test_numc_matmul_grouped_host_arrays(f32_algo):
    rng = np.random.default_rng(4)
    orig = nc.get_algo("float32")
    nc.set_algo("float32", f32_algo)
    bound = f16_bound if f32_algo == nc.ALGO_AUTO else split_bound
    try:
        _grouped_host_arrays(rng, bound)
    finally:
        nc.set_algo("float32", *orig)


def test_grouped_f16_not_less_accurate_than_fp32_fma():
    # Over a plan of mixed shapes, the scaled float16 split must not lose
    # to numc's FP32 FMA chain against a float64 reference (max and mean
    # error relative to |A| @ |B|).
    probs = random_problems(30, lo=64, hi=1024, seed=9)
    plan = nc.GemmPlan([(p[0], p[1], p[2]) for p in probs], nc.ALGO_SPLIT_FP16, 128)
    plan.run()
    nc.check_status()
    e16, efma = [], []
    for ta, tb, out, a, b in probs:
        exact = a.astype(np.float64) @ b.astype(np.float64)
        scale = np.abs(a.astype(np.float64)) @ np.abs(b.astype(np.float64))
        e16.append(np.abs(out.cpu().numpy() - exact) / scale)
        efma.append(np.abs(oracle.matmul(a, b) - exact) / scale)
    e16 = np.concatenate([x.ravel() for x in e16])
    efma = np.concatenate([x.ravel() for x in efma])
    assert e16.max() <= efma.max(), (e16.max(), efma.max())
    assert e16.mean() <= efma.mean(), (e16.mean(), efma.mean())


def _grouped_host_arrays(rng, bound):
    with nc.Ctx() as ctx:
        As, Bs, Cs, refs = [], [], [], []
        for i in range(10):
            M, K, N = rng.integers(1, 300, 3)
            a, b = synth.operands("uniform", M, K, N, dtype="float32", seed=i)
            A, B = ctx.from_numpy(a), ctx.from_numpy(b)
            if i % 3 == 0:
                A.to_device()
            As.append(A); Bs.append(B); Cs.append(ctx.zeros((M, N), "float32"))
            refs.append((a, b))
        nc.matmul_grouped(As, Bs, Cs)
        for C, (a, b) in zip(Cs, refs):
            K = a.shape[1]
            assert rel_err_vs_scale(C.numpy(), oracle.matmul(a, b), a, b) <= \
                max(bound(K), simt_bound(K))
        # integer dtypes loop numc_matmul, bit-exact
        a, b = synth.operands("uniform", 50, 600, 40, dtype="int8")
        A, B, C = ctx.from_numpy(a), ctx.from_numpy(b), ctx.zeros((50, 40), "int8")
        nc.matmul_grouped([A], [B], [C])
        np.testing.assert_array_equal(C.numpy(), oracle.matmul(a, b))


def test_empty_and_degenerate_problems():
    z = torch.zeros((0, 5), device="cuda")
    w = torch.ones((5, 3), device="cuda")
    e = torch.zeros((0, 3), device="cuda")
    a = torch.ones((4, 0), device="cuda")
    b = torch.ones((0, 6), device="cuda")
    o = torch.full((4, 6), 3.0, device="cuda")
    plan = nc.GemmPlan([(z, w, e), (a, b, o)])
    plan.run()
    torch.cuda.synchronize()
    assert bool((o == 0).all())


def test_f16_plan_across_the_fused_pass_limit():
    # float16 plans scale and split problems with K <= 1024 in one fused
    # pass, larger K in two; both kinds in one plan, tensor-core variant
    # forced, one fused problem with an infinity (its tiles fall back to
    # numc's FMA chains)
    shapes = [(300, 1000, 200), (257, 1024, 130), (300, 1025, 200), (129, 1100, 64),
              (64, 2000, 128), (100, 3, 70)]
    probs = []
    for i, (M, K, N) in enumerate(shapes):
        a, b = synth.operands("normal", M, K, N, dtype="float32", seed=2000 + i)
        if i == 1:
            a[5, 17] = np.inf
        probs.append((torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda(),
                      torch.full((M, N), float("nan"), device="cuda"), a, b))
    plan = nc.GemmPlan([(p[0], p[1], p[2]) for p in probs], nc.ALGO_SPLIT_FP16, 128)
    plan.run()
    nc.check_status()
    for i, (ta, tb, out, a, b) in enumerate(probs):
        got = out.cpu().numpy()
        ref = oracle.matmul(a, b)
        fin = np.isfinite(ref)
        np.testing.assert_array_equal(np.isfinite(got), fin)
        np.testing.assert_array_equal(got[~fin], ref[~fin])   # same infinities / NaN pattern
        if i == 1:
            assert not fin[5].all()
        rows = np.where(fin.all(axis=1))[0]
        K = a.shape[1]
        assert rel_err_vs_scale(got[rows], ref[rows], a[rows], b) <= \
            max(f16_bound(K), simt_bound(K))
    plan.free()


@pytest.mark.parametrize("param", [2128, 4128, 2064, 4064])
@pytest.mark.parametrize("algo", [nc.ALGO_SPLIT_FP16, nc.ALGO_SPLIT_BF16])
def test_split_k_plans_match_oracle(param, algo):
    """K cut into 2 or 4 slices per tile: the slices' partial sums added in
    K order by the reduction pass, then rescaled — the same bound."""
    probs = random_problems(24, lo=16, hi=1500, seed=5)
    plan = nc.GemmPlan([(p[0], p[1], p[2]) for p in probs], algo, param)
    plan.run()
    nc.check_status()
    check_all(probs, BOUND[algo])
    first = [p[2].clone() for p in probs]
    plan.run()          # deterministic: the same bits on a second run
    torch.cuda.synchronize()
    for (_, _, out, _, _), f in zip(probs, first):
        assert torch.equal(out, f)
    plan.free()


def test_split_k_strided_output_and_non_finite_inputs():
    M, K, N = 150, 700, 90
    a, b = synth.operands("normal", M, K, N, dtype="float32", seed=8)
    a[3, 5] = np.inf
    b[10, 70] = np.nan
    ta, tb = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    out_t = torch.full((N, M), 7.0, device="cuda")
    out = out_t.t()                                   # column stride != 1
    plan = nc.GemmPlan([(ta, tb, out)], nc.ALGO_SPLIT_FP16, 4128)
    plan.run()
    nc.check_status()
    got = out.cpu().numpy()
    want = oracle.matmul(a, b)
    fin = np.isfinite(want)
    # rows / columns with a non-finite input: numc's FMA chains exactly
    np.testing.assert_array_equal(np.isnan(got), np.isnan(want))
    np.testing.assert_array_equal(got[3, :][~np.isnan(want[3, :])], want[3, :][~np.isnan(want[3, :])])
    np.testing.assert_array_equal(got[:, 70], want[:, 70])
    a0, b0 = np.nan_to_num(a, posinf=0.0), np.nan_to_num(b)
    mask = fin.copy()
    mask[3, :] = False
    mask[:, 70] = False
    err = np.abs(got[mask] - want[mask]) / np.maximum(np.abs(a0) @ np.abs(b0), 1e-30)[mask]
    assert err.max() <= f16_bound(K)
    plan.free()
