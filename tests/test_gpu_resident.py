"""Device-resident array lifecycle: chains of calls that stay in HBM.

numc_array_copy and numc_array_contiguous of a device-resident array run on
the GPU (a gather kernel) and leave the result resident, so a chain
to_device -> transpose view -> contiguous / copy -> numc_matmul / numc_dot
with a resident output moves no array data between host and device until
the caller asks for it (numc_cuda_transfer_bytes counts every such byte).
"""
import numpy as np
import pytest

import numc_gb300 as nc
import oracle
from numc_gb300 import synth

from gpu_util import needs_gpu

pytestmark = [pytest.mark.gpu, needs_gpu]


@pytest.mark.parametrize("dt", ["float32", "int8", "int64", "float64"])
def test_contiguous_and_copy_stay_on_device(dt):
    a, b = synth.operands("uniform", 70, 90, 50, dtype=dt, seed=2)
    with nc.Ctx() as ctx:
        At = ctx.from_numpy(np.ascontiguousarray(a.T)).to_device()   # (90, 70) resident
        B = ctx.from_numpy(b).to_device()
        C = ctx.zeros((70, 50), dt).to_device()
        before = nc.transfer_bytes()
        A = At.transpose((1, 0))              # (70, 90) strided view, resident
        Ac = A.copy()                         # gathered on the GPU
        assert Ac.is_resident() and Ac.is_contiguous()
        A.contiguous()                        # re-laid out on the GPU, in place
        assert A.is_resident() and A.is_contiguous()
        nc.matmul(Ac, B, C)
        assert nc.transfer_bytes() == before, "the chain copied array data through the host"
        C.to_host()
        np.testing.assert_array_equal(C.numpy(), oracle.matmul(a, b))
        np.testing.assert_array_equal(A.to_host().numpy(), a)
        np.testing.assert_array_equal(Ac.to_host().numpy(), a)


def test_copy_of_host_current_resident_array_keeps_both():
    a = synth.array("uniform", (3, 4, 5), seed=4, dtype="int16")
    with nc.Ctx() as ctx:
        X = ctx.from_numpy(a).to_device()     # host and device both current
        V = X.transpose((2, 0, 1))
        Y = V.copy()
        assert Y.is_resident()
        np.testing.assert_array_equal(Y.numpy(), a.transpose(2, 0, 1))   # host copy made too
        np.testing.assert_array_equal(Y.to_host().numpy(), a.transpose(2, 0, 1))


def test_dot_on_resident_views_without_transfers():
    a = synth.array("normal", (40, 64), seed=6, stream=1, dtype="float32")
    b = synth.array("normal", (3, 64, 30), seed=6, stream=2, dtype="float32")
    with nc.Ctx() as ctx:
        A = ctx.from_numpy(a).to_device()
        B = ctx.from_numpy(b).to_device()
        O = ctx.zeros((40, 3, 30), "float32").to_device()
        before = nc.transfer_bytes()
        nc.dot(A, B, O)
        assert nc.transfer_bytes() == before
        np.testing.assert_array_equal(O.to_host().numpy(), oracle.dot(a, b))
