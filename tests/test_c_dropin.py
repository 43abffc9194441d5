"""The drop-in at the C level: C programs built against include/numc/ and
linked to libnumc_gb300.so with a plain C compiler.

* tests/c/dropin_matmul.c (this repository's): numc_matmul,
  numc_matmul_naive, transposed views, numc's error codes and numc's
  kernel-table call through numc_cuda_gemm_host, every dtype, checked
  against C loops.  Compiled with -Wall -Wextra -Werror on any host; run on
  the GPU.
* numc's own tests/matmul/test_matmul.c and test_matmul_naive.c, where a
  numc checkout is present (the development host): compiled unchanged with
  numc's -std=c2x against these headers and linked to this library — the
  source- and link-level proof that numc's callers relink unchanged.
"""
import os
import shutil
import subprocess

import pytest

import numc_gb300 as nc

from gpu_util import needs_gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
INCLUDE = os.path.join(ROOT, "include")
LIBDIR = os.path.dirname(nc.LIB_PATH)
NUMC_TESTS = "/root/reference/tests/matmul"

pytestmark = pytest.mark.skipif(shutil.which("gcc") is None, reason="needs a C compiler")


def _build(src, out, std="c11", extra=()):
    if not os.path.exists(nc.LIB_PATH):
        pytest.skip("library not built")
    cmd = ["gcc", f"-std={std}", "-O2", *extra, "-I", INCLUDE, src, "-L", LIBDIR,
           "-lnumc_gb300", f"-Wl,-rpath,{LIBDIR}", "-lm", "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def test_dropin_program_compiles_and_links(tmp_path):
    _build(os.path.join(HERE, "c", "dropin_matmul.c"), str(tmp_path / "dropin"),
           extra=("-Wall", "-Wextra", "-Werror"))


@pytest.mark.skipif(not os.path.isdir(NUMC_TESTS), reason="numc checkout not present")
@pytest.mark.parametrize("name", ["test_matmul", "test_matmul_naive"])
def test_numc_own_matmul_tests_link_unchanged(tmp_path, name):
    _build(os.path.join(NUMC_TESTS, name + ".c"), str(tmp_path / name), std="c2x")


@pytest.mark.gpu
@needs_gpu
def test_dropin_program_runs_on_gpu(tmp_path):
    exe = _build(os.path.join(HERE, "c", "dropin_matmul.c"), str(tmp_path / "dropin"))
    env = dict(os.environ)
    r = subprocess.run([exe], capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert ", 0 failures" in r.stdout
