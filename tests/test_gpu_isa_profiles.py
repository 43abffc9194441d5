"""The GPU against numc's NEON and AVX-512 builds (ISA profiles).

numc selects its kernels for the ISA it is compiled on, so its int8/uint8
store rules and its float register tiles differ between its x86-64 AVX2,
x86-64 AVX-512 and aarch64 NEON builds.  The library reproduces each build
(NumcInt8Profile as `param`, or the process-wide numc_cuda_set_isa_profile,
whose default is the host's build).  These tests compare the CUDA kernels
with numc's own outputs of the other two builds (tests/golden/golden_isa.*:
NEON numc_matmul and numc_dot for every dtype, AVX-512 numc_matmul for
int8/uint8), bit for bit, on the CUDA-core kernels and the int8 tensor
path, through the device-pointer C-ABI and through numc_matmul / numc_dot.
"""
import hashlib
import json
import os
import platform
import subprocess
import sys

import numpy as np
import pytest

import numc_gb300 as nc
import oracle
from numc_gb300 import synth

from gpu_util import needs_gpu

pytestmark = [pytest.mark.gpu, needs_gpu]
torch = pytest.importorskip("torch")

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = json.load(open(os.path.join(HERE, "golden", "golden_isa.json")))
ARR = np.load(os.path.join(HERE, "golden", "golden_isa.npz"))
PROFILE = {"neon": nc.INT8_ARM_NEON, "avx512": nc.INT8_X86_AVX512}


def check(name, got, entry):
    if entry["stored"] == "full":
        np.testing.assert_array_equal(got.reshape(-1), ARR[name].reshape(-1), err_msg=name)
    assert hashlib.sha256(np.ascontiguousarray(got).tobytes()).hexdigest() == entry["sha256"], name


def _operands(entry):
    return synth.operands(entry["kind"], *entry["shape"], seed=entry["seed"], dtype=entry["dtype"])


def _algos(entry):
    dt = entry["dtype"]
    algos = [nc.ALGO_SIMT]
    if dt in ("int8", "uint8"):
        algos.append(nc.ALGO_TC_INT8)
    return algos


CASES = [(c, algo) for c in GOLD["cases"] for algo in _algos(c)]


@pytest.mark.parametrize("entry,algo", CASES,
                         ids=[f"{c['name']}-algo{a}" for c, a in CASES])
def test_cabi_gemm_reproduces_numc_build(entry, algo):
    a, b = _operands(entry)
    ta, tb = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    out = torch.zeros((a.shape[0], b.shape[1]), dtype=ta.dtype, device="cuda")
    nc.gemm(ta, tb, out, algo=algo, param=PROFILE[entry["variant"]])
    nc.check_status()
    check(entry["name"], out.cpu().numpy(), entry)


@pytest.fixture
def neon_profile():
    before = nc.get_isa_profile()
    nc.set_isa_profile(nc.INT8_ARM_NEON)
    yield
    nc.set_isa_profile(before)


NEON_API = [c for c in GOLD["cases"] if c["variant"] == "neon" and
            (c["shape"][0] * c["shape"][1] * c["shape"][2] <= 1 << 28)]


@pytest.mark.parametrize("entry", NEON_API, ids=[c["name"] for c in NEON_API])
def test_numc_matmul_under_neon_profile(neon_profile, entry):
    """numc_matmul with the process-wide profile (as on an aarch64 host):
    the default algorithm of each dtype."""
    a, b = _operands(entry)
    with nc.Ctx() as ctx:
        A, B = ctx.from_numpy(a), ctx.from_numpy(b)
        C = ctx.zeros((a.shape[0], b.shape[1]), a.dtype)
        nc.matmul(A, B, C)
        check(entry["name"], C.numpy(), entry)


@pytest.mark.parametrize("entry", GOLD["dot_cases"], ids=[c["name"] for c in GOLD["dot_cases"]])
def test_numc_dot_under_neon_profile(neon_profile, entry):
    dt = entry["dtype"]
    kind = "normal" if np.dtype(dt).kind == "f" else "uniform"
    a = synth.array(kind, entry["a_shape"], seed=entry["seed"], stream=21, dtype=dt)
    b = synth.array(kind, entry["b_shape"], seed=entry["seed"], stream=22, dtype=dt)
    with nc.Ctx() as ctx:
        A, B = ctx.from_numpy(a), ctx.from_numpy(b)
        out = ctx.zeros(oracle.dot_shape(a.shape, b.shape), dt)
        nc.dot(A, B, out)
        check(entry["name"], out.numpy(), entry)


def test_grouped_cuda_core_problems_follow_neon_profile(neon_profile):
    gen = torch.Generator(device="cuda").manual_seed(3)
    probs = []
    for (m, k, n) in [(131, 700, 4100), (47, 40, 45), (129, 257, 131), (8, 520, 12)]:
        probs.append((torch.randn((m, k), device="cuda", generator=gen),
                      torch.randn((k, n), device="cuda", generator=gen),
                      torch.zeros((m, n), device="cuda")))
    plan = nc.GemmPlan(probs, nc.ALGO_SIMT)
    plan.run()
    nc.check_status()
    for a, b, c in probs:
        ah, bh = a.cpu().numpy(), b.cpu().numpy()
        np.testing.assert_array_equal(c.cpu().numpy(),
                                      oracle.matmul(ah, bh, oracle.PROFILE_ARM_NEON))
    plan.free()


def test_default_profile_is_the_hosts_build():
    """Without NUMC_CUDA_ISA_PROFILE the library reproduces numc as built for
    this host: NEON on aarch64, AVX2 on x86-64 (fresh process)."""
    env = {k: v for k, v in os.environ.items() if k != "NUMC_CUDA_ISA_PROFILE"}
    code = ("import numc_gb300 as nc; print(nc.get_isa_profile())")
    out = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True,
                         cwd=os.path.dirname(HERE), timeout=300)
    assert out.returncode == 0, out.stderr
    want = nc.INT8_ARM_NEON if platform.machine() in ("aarch64", "arm64") else nc.INT8_X86_AVX2
    assert int(out.stdout.strip()) == want


def test_profile_setter_rejects_unknown_values():
    with pytest.raises(nc.NumcError) as ei:
        nc.set_isa_profile(7)
    assert ei.value.code == nc.ERR_VALUE
