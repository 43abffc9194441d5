"""Build recipe for the oracle (test infrastructure only).

``build_oracle()`` compiles ``oracle/numc_oracle.c`` (the CPU restatement of
numc's matmul arithmetic) into ``oracle/_build/liboracle.so``.
``build_reference(variant)`` compiles the unmodified numc sources from a
local reference checkout into ``oracle/_ref/`` through ``oracle/Makefile.ref``
(the AVX2 build, the AVX-512 build, or the NEON matmul on the intrinsic model
in ``oracle/neon_shim``); it only runs where that checkout exists and the
host is x86-64.
"""
import os
import platform
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
ORACLE_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libnumc_ref.so")
REF_SRC = "/root/reference"
# numc builds the recipe can make: (make target, library)
REF_VARIANTS = {
    "avx2": ("all", REF_SO),
    "avx512": ("avx512", os.path.join(HERE, "_ref", "libnumc_ref_avx512.so")),
    "neon": ("neon", os.path.join(HERE, "_ref", "libnumc_ref_neon.so")),
}


def build_oracle(force=False):
    src = os.path.join(HERE, "numc_oracle.c")
    micro = os.path.join(HERE, "numc_oracle_micro.c")
    dot = os.path.join(HERE, "numc_oracle_dot.c")
    rand = os.path.join(HERE, "numc_oracle_rand.c")
    deps = [src, micro, dot, rand, os.path.join(HERE, "numc_oracle_micro.h")]
    if (not force and os.path.exists(ORACLE_SO)
            and os.path.getmtime(ORACLE_SO) >= max(os.path.getmtime(d) for d in deps)):
        return ORACLE_SO
    os.makedirs(os.path.dirname(ORACLE_SO), exist_ok=True)
    flags = ["-O3", "-std=c11", "-fPIC"]
    if platform.machine() in ("x86_64", "AMD64"):
        flags.append("-mfma")  # vector FMA; aarch64 has it natively
    micro_o = ORACLE_SO + ".micro.o"
    # The micro-kernels rely on contraction of `a * b + acc` into FMA; the
    # rest of the oracle must not be contracted (numc's scalar edges are not).
    subprocess.check_call(["gcc", *flags, "-ffp-contract=fast", "-c", micro,
                           "-o", micro_o])
    tmp = ORACLE_SO + ".tmp"
    subprocess.check_call(["gcc", *flags, "-fopenmp", "-shared",
                           "-ffp-contract=off", src, dot, rand, micro_o, "-o", tmp, "-lm"])
    os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def reference_buildable():
    return (os.path.isdir(os.path.join(REF_SRC, "src"))
            and platform.machine() in ("x86_64", "AMD64")
            and shutil.which("make") is not None)


def build_reference(variant="avx2"):
    """Returns the path of the compiled reference build `variant` (avx2:
    numc's x86-64 AVX2 build; avx512: its AVX-512 build; neon: its aarch64
    NEON matmul through oracle/neon_shim), or None if not buildable."""
    target, path = REF_VARIANTS[variant]
    if os.path.exists(path):
        return path
    if not reference_buildable():
        return None
    subprocess.check_call(
        ["make", "-f", os.path.join("oracle", "Makefile.ref"),
         f"-j{os.cpu_count() or 4}", f"REF={REF_SRC}", target],
        cwd=ROOT, stdout=subprocess.DEVNULL)
    return path if os.path.exists(path) else None


if __name__ == "__main__":
    print(build_oracle(force=True))
    print(build_reference())
