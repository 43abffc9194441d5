import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

# The golden fixtures and the oracle's default profile are numc's x86-64
# AVX2 build, while the library defaults to the build of the host it runs
# on (NEON on aarch64).  Tests pin the x86 profile unless they select
# another one (tests/test_gpu_isa_profiles.py covers NEON, AVX-512 and the
# host default in a fresh process).
os.environ.setdefault("NUMC_CUDA_ISA_PROFILE", "x86")


def pytest_configure(config):
    config.addinivalue_line(
        "markers", "gpu: needs a CUDA GPU (sm_103a) and the built extension")
