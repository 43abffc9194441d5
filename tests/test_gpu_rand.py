"""numc_array_rand on the GPU against numc's own outputs and the oracle.

numc's generator state is per host thread, so every sequence runs in a
fresh thread: an unseeded sequence starts from numc's default seed there,
exactly as in the golden run.  Every value must match byte for byte: the
committed golden outputs of the compiled numc (tests/golden/rand_golden.*,
numc's single-thread and per-thread-chunk layouts, every dtype, ragged
chunks, the 1 MiB threshold on both sides), and the oracle at sizes and
thread counts the fixtures do not hold.
"""
import threading

import numpy as np
import pytest

import numc_gb300 as nc
import oracle
from gpu_util import needs_gpu
from test_oracle_rand import SEQS, ARRAYS, check_against_golden

pytestmark = [pytest.mark.gpu, needs_gpu]


def in_fresh_thread(fn):
    box = {}

    def body():
        try:
            box["out"] = fn()
        except BaseException as e:   # re-raised in the caller
            box["err"] = e
    t = threading.Thread(target=body)
    t.start()
    t.join()
    if "err" in box:
        raise box["err"]
    return box["out"]


def run_sequence(seed, threads, calls, device):
    def body():
        nc.rand_set_threads(threads)
        if seed is not None:
            nc.manual_seed(seed)
        outs = []
        with nc.Ctx() as ctx:
            for dt, shape in calls:
                if device:
                    arr = ctx.rand_device(shape, dt)
                    assert arr.is_resident()
                    arr.to_host()
                else:
                    arr = ctx.rand(shape, dt)
                outs.append(arr.numpy().copy())
        return outs
    try:
        return in_fresh_thread(body)
    finally:
        nc.rand_set_threads(0)


@pytest.mark.parametrize("device", [False, True], ids=["host", "resident"])
@pytest.mark.parametrize("si", range(len(SEQS)))
def test_rand_matches_numc_golden(si, device):
    seq = SEQS[si]
    calls = [(e["dtype"], tuple(e["shape"])) for e in seq["calls"]]
    outs = run_sequence(seq["seed"], seq["omp_threads"], calls, device)
    for entry, out in zip(seq["calls"], outs):
        check_against_golden(entry, ARRAYS, out)


@pytest.mark.parametrize("threads", [1, 5, 144])
def test_rand_matches_oracle_large(threads):
    # 16 Mi float32 (several warps per numc thread, ragged last chunk), a
    # small fill, 1 Mi + 7 int64, a small fill, each continuing the state
    calls = [("float32", (4001, 4003)), ("uint8", (3,)), ("int64", (1 << 20) + 7),
             ("float64", (5,))]
    calls = [(dt, sh if isinstance(sh, tuple) else (sh,)) for dt, sh in calls]
    outs = run_sequence(99, threads, calls, device=False)
    st = oracle.rand_seed(99)
    for (dt, shape), out in zip(calls, outs):
        want = oracle.rand(dt, shape, st, threads)
        assert out.tobytes() == want.tobytes(), (dt, shape, threads)


def test_rand_fill_unaligned_device_pointer():
    import torch

    def body():
        nc.manual_seed(2024)
        base = torch.empty(600_001, dtype=torch.float32, device="cuda")
        view = base[1:]                      # 4 bytes past a 16-byte boundary
        nc.rand_fill(view)
        small = torch.empty(11, dtype=torch.int16, device="cuda")
        nc.rand_fill(small[1:])
        torch.cuda.synchronize()
        return view.cpu().numpy(), small[1:].cpu().numpy()
    nc.rand_set_threads(3)
    try:
        got, got16 = in_fresh_thread(body)
    finally:
        nc.rand_set_threads(0)
    st = oracle.rand_seed(2024)
    assert got.tobytes() == oracle.rand("float32", got.shape, st, 3).tobytes()
    assert got16.tobytes() == oracle.rand("int16", got16.shape, st, 3).tobytes()


def test_rand_seed_reproducible_and_distinct():
    # numc's own checks (tests/random/test_rand.c:8-47): the same seed gives
    # the same values, different seeds different ones, floats in [0, 1)
    def draw(seed):
        def body():
            nc.manual_seed(seed)
            with nc.Ctx() as ctx:
                return ctx.rand((1000,), "float32").numpy().copy()
        return in_fresh_thread(body)
    a, b, c = draw(42), draw(42), draw(43)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    assert a.min() >= 0.0 and a.max() < 1.0


def test_rand_empty_and_errors():
    def body():
        nc.manual_seed(1)
        with nc.Ctx() as ctx:
            e = ctx.rand((0, 5), "float32")
            assert e.shape == (0, 5)
            # an empty fill leaves the state where it was
            x = ctx.rand((9,), "int32").numpy().copy()
        return x
    x = in_fresh_thread(body)
    st = oracle.rand_seed(1)
    assert x.tobytes() == oracle.rand("int32", (9,), st, 1).tobytes()
