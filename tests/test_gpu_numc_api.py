"""numc's own matmul tests, run through numc_matmul on the GPU backend.

Ports the behaviour of tests/matmul/test_matmul.c and
tests/matmul/test_matmul_naive.c of numc: the same shapes, fills and
tolerances, called through the same C API (here via ctypes).
"""
import numpy as np
import pytest

import numc_gb300 as nc
import oracle
from numc_gb300 import synth

from gpu_util import needs_gpu

pytestmark = [pytest.mark.gpu, needs_gpu]

ALL = nc.DTYPES
N = 64


@pytest.fixture
def ctx():
    c = nc.Ctx()
    yield c
    c.free()


@pytest.mark.parametrize("dt", ALL)
def test_identity(ctx, dt):
    # test_matmul.c:15-42 and the per-dtype identity tests: A @ I == A
    a = (np.arange(N * N) % 97 + 1).astype(dt).reshape(N, N)
    A, I, C = ctx.from_numpy(a), ctx.from_numpy(np.eye(N, dtype=dt)), ctx.zeros((N, N), dt)
    nc.matmul(A, I, C)
    np.testing.assert_array_equal(C.numpy(), a)


@pytest.mark.parametrize("dt", ALL)
def test_known_result_ones(ctx, dt):
    # test_matmul.c:44-75: ones(2,N) @ ones(N,2) == N
    A = ctx.fill((2, N), dt, 1)
    B = ctx.fill((N, 2), dt, 1)
    C = ctx.zeros((2, 2), dt)
    nc.matmul(A, B, C)
    assert (C.numpy() == N).all()


@pytest.mark.parametrize("dt", ["int16", "int32", "int64", "float32", "float64",
                                "uint16", "uint32", "uint64"])
def test_naive_known_answer(ctx, dt):
    # test_matmul_naive.c:1-8
    A = ctx.from_numpy(np.array([[1, 2, 3], [4, 5, 6]], dtype=dt))
    B = ctx.from_numpy(np.array([[7, 8], [9, 10], [11, 12]], dtype=dt))
    for fn in (nc.matmul, nc.matmul_naive):
        C = ctx.zeros((2, 2), dt)
        fn(A, B, C)
        np.testing.assert_array_equal(C.numpy(), [[58, 64], [139, 154]])


def test_naive_int8_known_answer(ctx):
    # test_matmul_naive.c:20-30
    A = ctx.from_numpy(np.array([[1, 2, 3], [4, 5, 6]], dtype=np.int8))
    B = ctx.from_numpy(np.array([[1, 2], [3, 4], [5, 6]], dtype=np.int8))
    C = ctx.zeros((2, 2), "int8")
    nc.matmul_naive(A, B, C)
    np.testing.assert_array_equal(C.numpy(), [[22, 28], [49, 64]])


EDGE = [(1, 128, 64), (64, 128, 1), (100, 128, 64), (64, 128, 100),
        (100, 128, 100), (50, 64, 50), (144, 256, 64), (148, 256, 64),
        (64, 256, 64), (64, 300, 64), (7, 7, 7), (97, 101, 103), (37, 41, 43),
        (67, 67, 67), (256, 256, 256)]


@pytest.mark.parametrize("shape", EDGE, ids=lambda s: "x".join(map(str, s)))
@pytest.mark.parametrize("dt", ALL)
def test_edge_shapes_vs_naive_and_oracle(ctx, dt, shape):
    # DEFINE_EDGE_TEST (test_matmul.c:713-797): (i%7)+1, (i%5)+1 fills,
    # GEMM vs naive; here also against numc's own arithmetic (the oracle).
    M, K, Nn = shape
    a, b = synth.operands("smallint", M, K, Nn, dtype=dt)
    A, B = ctx.from_numpy(a), ctx.from_numpy(b)
    C, Cn = ctx.zeros((M, Nn), dt), ctx.zeros((M, Nn), dt)
    nc.matmul(A, B, C)
    nc.matmul_naive(A, B, Cn)
    np.testing.assert_array_equal(C.numpy(), oracle.matmul(a, b, oracle.PROFILE_X86_AVX2))
    np.testing.assert_array_equal(Cn.numpy(), oracle.matmul(a, b, oracle.PROFILE_WRAP))


@pytest.mark.parametrize("dt", ["float32", "int32"])
def test_double_transpose_operand(ctx, dt):
    # test_matmul.c:590-654: a double in-place transpose is the identity
    a, b = synth.operands("smallint", N, N, N, dtype=dt)
    A, B = ctx.from_numpy(a), ctx.from_numpy(b)
    C1, C2 = ctx.zeros((N, N), dt), ctx.zeros((N, N), dt)
    nc.matmul(A, B, C1)
    B.transpose((1, 0)).transpose((1, 0))
    A.transpose((1, 0)).transpose((1, 0))
    nc.matmul(A, B, C2)
    np.testing.assert_array_equal(C1.numpy(), C2.numpy())


@pytest.mark.parametrize("dt", ["float32", "float64", "int8", "uint16", "int64"])
def test_true_transposed_views(ctx, dt):
    # Strided operands numc accepts but mishandles (it assumes unit column
    # strides for B and out, src/matmul/matmul.c:358-362): the GPU path
    # honours every stride.
    M, K, Nn = 45, 300, 37
    a, b = synth.operands("uniform", M, K, Nn, dtype=dt)
    At = ctx.from_numpy(np.ascontiguousarray(a.T)).transpose((1, 0))
    Bt = ctx.from_numpy(np.ascontiguousarray(b.T)).transpose((1, 0))
    C = ctx.zeros((Nn, M), dt).transpose((1, 0))
    nc.matmul(At, Bt, C)
    # numc's arithmetic on the same values (floats included: bit-exact)
    ref = oracle.matmul(a, b, oracle.PROFILE_WRAP if dt in ("int8", "uint8") else 0)
    np.testing.assert_array_equal(C.numpy(), ref)


def test_strided_slice_output_keeps_gaps(ctx):
    a, b = synth.operands("uniform", 20, 30, 10, dtype="int32")
    big = ctx.fill((20, 25), "int32", 7)
    view = big.slice(1, 0, 20, 2)           # columns 0,2,...,18
    nc.matmul(ctx.from_numpy(a), ctx.from_numpy(b), view)
    full = big.numpy()
    np.testing.assert_array_equal(full[:, 0:20:2], oracle.matmul(a, b))
    assert (full[:, 1:20:2] == 7).all() and (full[:, 20:] == 7).all()


def test_errors_on_gpu_path(ctx):
    a = ctx.zeros((2, 3), "float32")
    with pytest.raises(nc.NumcError) as e:
        nc.matmul(a, ctx.zeros((4, 2), "float32"), ctx.zeros((2, 2), "float32"))
    assert e.value.code == nc.ERR_SHAPE
    with pytest.raises(nc.NumcError) as e:
        nc.matmul(a, ctx.zeros((3, 2), "int32"), ctx.zeros((2, 2), "float32"))
    assert e.value.code == nc.ERR_TYPE


def test_zero_sized(ctx):
    for dt in ALL:
        C = ctx.fill((3, 4), dt, 5)
        nc.matmul(ctx.zeros((3, 0), dt), ctx.zeros((0, 4), dt), C)
        assert (C.numpy() == 0).all()
        nc.matmul(ctx.zeros((0, 5), dt), ctx.zeros((5, 4), dt), ctx.zeros((0, 4), dt))


def test_device_residency_chain(ctx):
    # X @ W1 -> H (resident), H @ W2 -> Y, all in HBM; host copies only at
    # the ends.
    x, w1 = synth.operands("uniform", 64, 96, 80, dtype="float64")
    _, w2 = synth.operands("uniform", 1, 80, 24, dtype="float64", seed=9)
    X, W1, W2 = (ctx.from_numpy(t).to_device() for t in (x, w1, w2))
    H = ctx.zeros((64, 80), "float64").to_device()
    Y = ctx.zeros((64, 24), "float64").to_device()
    nc.matmul(X, W1, H)
    nc.matmul(H, W2, Y)
    assert Y.is_resident()
    Y.to_host()
    ref = oracle.matmul(oracle.matmul(x, w1), w2)
    np.testing.assert_allclose(Y.numpy(), ref, rtol=1e-12, atol=1e-12)
    # A host write to a resident array updates the device copy too.
    W2.write(np.zeros_like(w2))
    nc.matmul(H, W2, Y)
    Y.to_host()
    assert (Y.numpy() == 0).all()


def test_checkpoint_frees_device_arrays(ctx):
    keep = ctx.from_numpy(np.ones((8, 8), "float32")).to_device()
    cp = ctx.checkpoint()
    for _ in range(4):
        ctx.zeros((512, 512), "float32").to_device()
    ctx.restore(cp)
    out = ctx.zeros((8, 8), "float32")
    nc.matmul(keep, keep, out)
    assert (out.numpy() == 8).all()


def test_device_arena_slabs_bump_rewind_and_reuse(ctx):
    """Device memory comes from 64 MiB slabs by bump allocation: many small
    resident arrays share one slab, restore rewinds it and the next arrays
    reuse the space, an array above the slab size gets a slab of its own,
    and results stay correct throughout."""
    slab = 64 << 20
    assert ctx.device_usage() == (0, 0, 0)
    keep = ctx.from_numpy(np.full((8, 8), 2.0, "float32")).to_device()
    n0, r0, u0 = ctx.device_usage()
    assert (n0, r0) == (1, slab) and u0 == 256
    cp = ctx.checkpoint()
    arrs = [ctx.from_numpy(np.full((16, 16), float(i), "float32")).to_device() for i in range(200)]
    n1, r1, u1 = ctx.device_usage()
    assert (n1, r1) == (1, slab) and u1 == 256 + 200 * 1024   # 16*16*4 bytes each
    out = ctx.zeros((16, 16), "float32")
    nc.matmul(arrs[3], arrs[5], out)
    assert (out.numpy() == 3 * 5 * 16).all()
    big = ctx.zeros((5000, 4000), "float32").to_device()   # 80 MB: a slab of its own
    n2, r2, u2 = ctx.device_usage()
    assert n2 == 2 and r2 == slab + 5000 * 4000 * 4
    ctx.restore(cp)
    n3, r3, u3 = ctx.device_usage()
    assert (n3, r3, u3) == (2, r2, 256)                      # slabs kept, rewound
    again = [ctx.from_numpy(np.full((16, 16), 1.0, "float32")).to_device() for _ in range(10)]
    assert ctx.device_usage() == (2, r2, 256 + 10 * 1024)    # space reused, no new slab
    out = ctx.zeros((8, 8), "float32")
    nc.matmul(keep, keep, out)
    assert (out.numpy() == 32).all()
    out2 = ctx.zeros((16, 16), "float32")
    nc.matmul(again[0], again[9], out2)
    assert (out2.numpy() == 16).all()


def test_device_arena_released_by_ctx_free():
    torch = pytest.importorskip("torch")
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    c = nc.Ctx()
    for _ in range(3):
        c.zeros((4096, 4096), "float32").to_device()
    assert c.device_usage()[0] == 3
    assert torch.cuda.mem_get_info()[0] <= free0 - 3 * (64 << 20)
    c.free()
    assert torch.cuda.mem_get_info()[0] >= free0 - (8 << 20)
