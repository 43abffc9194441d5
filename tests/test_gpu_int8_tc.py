"""int8/uint8 on the tcgen05 tensor path: bit-exact with numc.

Every stored byte must equal numc's own (golden SHA-256 at 1024^3 and
300x4100x4200) and the oracle's for each store-rule profile, including
shapes with remainder tiles and K not a multiple of numc's 512 block, on
every tile schedule: single CTAs (128 x 64 tiles, and 128 x 128 once those
give every SM one) and persistent CTA pairs (256 x 128, 256 x 256), each
with every store-rule profile.
"""
import numpy as np
import pytest

import numc_gb300 as nc
import oracle
from numc_gb300 import synth

from gpu_util import golden, needs_gpu, sha

pytestmark = [pytest.mark.gpu, needs_gpu]
torch = pytest.importorskip("torch")
CASES, _ = golden()


def _tc(a, b, profile, tile=nc.INT8_TILE_AUTO):
    ta = torch.from_numpy(np.ascontiguousarray(a)).cuda()
    tb = torch.from_numpy(np.ascontiguousarray(b)).cuda()
    out = torch.full((a.shape[0], b.shape[1]), 77, dtype=ta.dtype, device="cuda")
    nc.gemm(ta, tb, out, algo=nc.ALGO_TC_INT8, param=profile + 16 * tile)
    nc.check_status()
    return out.cpu().numpy()


@pytest.mark.parametrize("dt", ["int8", "uint8"])
@pytest.mark.parametrize("profile", [nc.INT8_X86_AVX2, nc.INT8_ARM_NEON, nc.INT8_WRAP])
@pytest.mark.parametrize("shape", [(150, 1500, 140), (97, 1100, 203), (5, 3, 4),
                                   (300, 513, 64), (128, 64, 65), (200, 4096, 300),
                                   # enough 128-column tiles for the 128 x 128 tile kernel
                                   (2000, 700, 1250), (2304, 1536, 1280)],
                         ids=lambda s: "x".join(map(str, s)))
def test_profiles_vs_oracle(dt, profile, shape):
    a, b = synth.operands("uniform", *shape, dtype=dt, seed=sum(shape))
    np.testing.assert_array_equal(_tc(a, b, profile), oracle.matmul(a, b, profile))


ORACLE_PROFILE = {nc.INT8_X86_AVX2: oracle.PROFILE_X86_AVX2, nc.INT8_ARM_NEON: oracle.PROFILE_ARM_NEON,
                  nc.INT8_WRAP: oracle.PROFILE_WRAP, nc.INT8_X86_AVX512: oracle.PROFILE_X86_AVX512}


@pytest.mark.parametrize("dt", ["int8", "uint8"])
@pytest.mark.parametrize("tile", [nc.INT8_TILE_SINGLE, nc.INT8_TILE_PAIR128, nc.INT8_TILE_PAIR256],
                         ids=["single", "pair128", "pair256"])
@pytest.mark.parametrize("profile", [nc.INT8_X86_AVX2, nc.INT8_ARM_NEON, nc.INT8_WRAP,
                                     nc.INT8_X86_AVX512], ids=["x86", "neon", "wrap", "avx512"])
@pytest.mark.parametrize("shape", [(5, 3, 4), (300, 1100, 517), (97, 513, 203),
                                   # several tiles per pair, an odd CTA below the last row
                                   (1300, 1536, 1100)],
                         ids=lambda s: "x".join(map(str, s)))
def test_tile_schedules_vs_oracle(dt, tile, profile, shape):
    a, b = synth.operands("extreme" if shape[1] > 1000 else "uniform", *shape, dtype=dt,
                          seed=7 + sum(shape))
    np.testing.assert_array_equal(_tc(a, b, profile, tile),
                                  oracle.matmul(a, b, ORACLE_PROFILE[profile]))


@pytest.mark.parametrize("dt", ["int8", "uint8"])
@pytest.mark.parametrize("tile", [nc.INT8_TILE_PAIR128, nc.INT8_TILE_PAIR256])
def test_pair_schedules_golden_sha_1024(dt, tile):
    case = [c for c in CASES if c["dtype"] == dt and c["kind"] == "uniform"
            and tuple(c["shape"]) == (1024, 1024, 1024)][0]
    a, b = synth.operands("uniform", 1024, 1024, 1024, seed=case["seed"], dtype=dt)
    assert sha(_tc(a, b, nc.INT8_X86_AVX2, tile)) == case["sha256"]


def test_pair_schedule_strided_output():
    """A transposed (column-major) output takes the byte-store path."""
    a, b = synth.operands("uniform", 600, 900, 520, dtype="int8", seed=11)
    ta, tb = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    for tile in (nc.INT8_TILE_PAIR128, nc.INT8_TILE_PAIR256):
        out = torch.full((520, 600), 77, dtype=torch.int8, device="cuda").t()
        nc.gemm(ta, tb, out, algo=nc.ALGO_TC_INT8, param=nc.INT8_X86_AVX2 + 16 * tile)
        nc.check_status()
        np.testing.assert_array_equal(out.cpu().numpy(), oracle.matmul(a, b))


def test_tile_schedule_out_of_range_is_refused():
    a = torch.zeros((4, 4), dtype=torch.int8, device="cuda")
    with pytest.raises(nc.NumcError) as ei:
        nc.gemm(a, a, a.clone(), algo=nc.ALGO_TC_INT8, param=16 * 4)
    assert ei.value.code == nc.ERR_VALUE


@pytest.mark.parametrize("case", [c for c in CASES if c["dtype"] in ("int8", "uint8")
                                  and c["kind"] == "uniform"], ids=lambda c: c["name"])
def test_golden_sha(case):
    M, K, N = case["shape"]
    a, b = synth.operands("uniform", M, K, N, seed=case["seed"], dtype=case["dtype"])
    prof = nc.INT8_WRAP if M * K * N <= 192 ** 3 else nc.INT8_X86_AVX2
    assert sha(_tc(a, b, prof)) == case["sha256"]


def test_strided_and_through_numc_matmul():
    a, b = synth.operands("uniform", 130, 700, 90, dtype="int8", seed=3)
    ta = torch.from_numpy(np.ascontiguousarray(a.T)).cuda().t()
    tb = torch.from_numpy(b).cuda()
    out = torch.empty((90, 130), dtype=torch.int8, device="cuda").t()
    nc.gemm(ta, tb, out, algo=nc.ALGO_TC_INT8, param=nc.INT8_X86_AVX2)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out.cpu().numpy(), oracle.matmul(a, b))
    orig = nc.get_algo("int8")
    nc.set_algo("int8", nc.ALGO_TC_INT8, nc.INT8_X86_AVX2)
    try:
        with nc.Ctx() as ctx:
            A, B, C = ctx.from_numpy(a), ctx.from_numpy(b), ctx.zeros((130, 90), "int8")
            nc.matmul(A, B, C)
            np.testing.assert_array_equal(C.numpy(), oracle.matmul(a, b))
    finally:
        nc.set_algo("int8", *orig)


@pytest.mark.parametrize("dt", ["int8", "uint8"])
def test_unaligned_and_general_strides(dt):
    """Operand rows off the 16-byte grid, a column-sliced B (rows contiguous
    but unaligned) and a B with no unit stride at all."""
    a, b = synth.operands("uniform", 130, 700, 90, dtype=dt, seed=5)
    want = oracle.matmul(a, b)
    abig = np.zeros((130, 703), a.dtype)
    abig[:, 1:701] = a
    ta = torch.from_numpy(abig).cuda()[:, 1:701]              # k contiguous, rows unaligned
    bsl = np.zeros((700, 93), b.dtype)
    bsl[:, 3:93] = b
    tb1 = torch.from_numpy(bsl).cuda()[:, 3:93]               # columns contiguous, unaligned
    bst = np.zeros((700, 180), b.dtype)
    bst[:, ::2] = b
    tb2 = torch.from_numpy(bst).cuda()[:, ::2]                # no unit stride
    for tb in (tb1, tb2):
        out = torch.full((130, 90), 77, dtype=ta.dtype, device="cuda")
        nc.gemm(ta, tb, out, algo=nc.ALGO_TC_INT8, param=nc.INT8_X86_AVX2)
        nc.check_status()
        np.testing.assert_array_equal(out.cpu().numpy(), want)


@pytest.mark.parametrize("dt", ["int8", "uint8"])
@pytest.mark.parametrize("profile", [nc.INT8_X86_AVX2, nc.INT8_ARM_NEON, nc.INT8_X86_AVX512],
                         ids=["x86", "neon", "avx512"])
@pytest.mark.parametrize("tile", [nc.INT8_TILE_SINGLE, nc.INT8_TILE_PAIR256],
                         ids=["single", "pair256"])
def test_long_k_sums_past_2_31(dt, profile, tile):
    """K = 140000 with every entry at the dtype's extreme: the exact int32
    sums pass 2^31 (the clamp-once rules narrow the wrapped sum), the x86
    rule folds 274 blocks (uint8 block sums past 2^24); against the oracle."""
    M, K, N = 260, 140000, 264
    a, b = synth.operands("extreme", M, K, N, dtype=dt, seed=21)
    np.testing.assert_array_equal(_tc(a, b, profile, tile),
                                  oracle.matmul(a, b, ORACLE_PROFILE[profile]))
