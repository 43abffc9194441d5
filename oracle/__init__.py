"""Oracle for numc's matmul (TEST INFRASTRUCTURE ONLY).

Two checkers live here, both CPU-only:

* ``matmul(a, b, profile)`` and ``dot(a, b)`` — the C restatements in
  ``numc_oracle.c`` and ``numc_oracle_dot.c`` (build on any host; they are
  what GPU parity tests compare against).
* ``ref_matmul(a, b)`` and ``ref_dot(a, b, perms)`` — the unmodified numc
  library compiled from the reference sources (x86-64 hosts with the
  reference checkout only); used to pin the restatements and to generate the
  golden fixtures in tests/golden/.

The product library never imports this package.
"""
import ctypes
import os

import numpy as np

from . import build as _build

# numc's NumcDType numbering (include/numc/dtype.h:21-32)
DTYPES = ["int8", "int16", "int32", "int64", "uint8", "uint16", "uint32",
          "uint64", "float32", "float64"]
DTYPE_CODE = {name: i for i, name in enumerate(DTYPES)}

PROFILE_X86_AVX2 = 0
PROFILE_ARM_NEON = 1
PROFILE_WRAP = 2          # numc_matmul_naive (floats: unfused chains)
PROFILE_X86_PACKED = 3    # numc's x86 packed kernels called directly (numc_dot)
PROFILE_X86_AVX512 = 4    # numc's x86-64 AVX-512 build (int8/uint8 store rule)

_lib = None
_refs = {}


def _load():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        lib = ctypes.CDLL(path)
        i64 = ctypes.c_int64
        vp = ctypes.c_void_p
        lib.oracle_matmul.argtypes = [ctypes.c_int, vp, vp, vp, i64, i64, i64,
                                      i64, i64, i64, i64, i64, i64,
                                      ctypes.c_int, ctypes.c_int]
        lib.oracle_matmul.restype = ctypes.c_int
        lib.oracle_dot2_f64.argtypes = [vp, vp, i64, i64, vp, vp, i64, vp, vp]
        lib.oracle_dot_f32_ref.argtypes = [vp, vp, i64, i64, vp, vp, i64, vp]
        lib.oracle_num_threads.restype = ctypes.c_int
        ci = ctypes.c_int
        lib.oracle_dot.argtypes = [ci, vp, ci, vp, vp, ci, vp, ci, vp, vp, ci, vp, ci, vp, vp]
        lib.oracle_dot.restype = ci
        lib.oracle_rand_seed.argtypes = [ctypes.c_uint64, vp]
        lib.oracle_rand_fill.argtypes = [ci, vp, i64, ci, vp]
        lib.oracle_rand_fill.restype = ci
        lib.oracle_rand_threads.argtypes = [ci, i64, ci]
        lib.oracle_rand_threads.restype = ci
        _lib = lib
    return _lib


def num_threads():
    return _load().oracle_num_threads()


def matmul(a, b, profile=PROFILE_X86_AVX2, nthreads=0):
    """numc's result of a @ b for 2-D numpy arrays of one numc dtype."""
    lib = _load()
    assert a.dtype == b.dtype and a.ndim == 2 and b.ndim == 2
    assert a.shape[1] == b.shape[0]
    M, K = a.shape
    N = b.shape[1]
    es = a.dtype.itemsize
    out = np.empty((M, N), dtype=a.dtype)
    rc = lib.oracle_matmul(
        DTYPE_CODE[a.dtype.name], a.ctypes.data, b.ctypes.data, out.ctypes.data,
        M, K, N, a.strides[0] // es, a.strides[1] // es, b.strides[0] // es,
        b.strides[1] // es, out.strides[0] // es, out.strides[1] // es,
        profile, nthreads)
    if rc != 0:
        raise RuntimeError("oracle_matmul failed")
    return out


def dot2_f64(a, b, rows, cols):
    """Double-double (Dot2) values of (a @ b)[rows, cols] for float64 a, b."""
    lib = _load()
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    rows = np.ascontiguousarray(rows, dtype=np.int64)
    cols = np.ascontiguousarray(cols, dtype=np.int64)
    hi = np.empty(len(rows)); lo = np.empty(len(rows))
    lib.oracle_dot2_f64(a.ctypes.data, b.ctypes.data, a.shape[1], b.shape[1],
                        rows.ctypes.data, cols.ctypes.data, len(rows),
                        hi.ctypes.data, lo.ctypes.data)
    return hi, lo


def dot_f32_ref(a, b, rows, cols):
    """float64-accurate values of (a @ b)[rows, cols] for float32 a, b."""
    lib = _load()
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = np.ascontiguousarray(b, dtype=np.float32)
    rows = np.ascontiguousarray(rows, dtype=np.int64)
    cols = np.ascontiguousarray(cols, dtype=np.int64)
    out = np.empty(len(rows))
    lib.oracle_dot_f32_ref(a.ctypes.data, b.ctypes.data, a.shape[1],
                           b.shape[1], rows.ctypes.data, cols.ctypes.data,
                           len(rows), out.ctypes.data)
    return out


def dot_shape(ashape, bshape):
    """numc_dot's output shape (numpy.dot's rule)."""
    if len(ashape) == 0:
        return tuple(bshape)
    if len(bshape) == 0:
        return tuple(ashape)
    if len(ashape) == 1 and len(bshape) == 1:
        return (1,)
    return tuple(ashape[:-1]) + tuple(bshape[:-2]) + ((bshape[-1],) if len(bshape) > 1 else ())


def _estrides(x):
    return [s // x.itemsize for s in x.strides]


def dot(a, b, out=None):
    """numc's result of numc_dot(a, b, out) for numpy arrays (any strides).

    `out` may be given (a writable view with the output shape) to exercise
    strided outputs; it is returned."""
    lib = _load()
    assert a.dtype == b.dtype
    if out is None:
        out = np.zeros(dot_shape(a.shape, b.shape), dtype=a.dtype)
    i64 = ctypes.c_int64

    def arr(vals):
        return (i64 * max(1, len(vals)))(*vals)
    ac = int(a.ndim == 1 and a.strides[0] == a.itemsize)
    bc = int(b.ndim == 1 and b.strides[0] == b.itemsize)
    rc = lib.oracle_dot(DTYPE_CODE[a.dtype.name],
                        a.ctypes.data, a.ndim, arr(a.shape), arr(_estrides(a)), ac,
                        b.ctypes.data, b.ndim, arr(b.shape), arr(_estrides(b)), bc,
                        out.ctypes.data, out.ndim, arr(out.shape), arr(_estrides(out)))
    if rc != 0:
        raise ValueError(f"oracle_dot: unsupported operands (code {rc})")
    return out


# numc's default seed for a thread that never called numc_manual_seed
# (src/random/kernel.h:123-126)
RAND_DEFAULT_SEED = 0xdeadbeefcafe1234


def rand_seed(seed=RAND_DEFAULT_SEED):
    """numc's four-lane xoshiro256** state after numc_manual_seed(seed), as
    16 uint64 words in numc's layout (word * 4 + lane)."""
    st = np.zeros(16, dtype=np.uint64)
    _load().oracle_rand_seed(int(seed) & (2**64 - 1), st.ctypes.data)
    return st


def rand_threads(dtype, n, max_threads):
    """numc's fill thread count (0: the single-threaded small path)."""
    return _load().oracle_rand_threads(DTYPE_CODE[np.dtype(dtype).name], int(n), int(max_threads))


def rand(dtype, shape, state, max_threads):
    """numc_array_rand(shape, dtype) from `state` (updated in place, as
    numc's thread-local state is) with numc's OpenMP maximum of
    `max_threads` threads.  Returns the array."""
    dt = np.dtype(dtype)
    assert state.dtype == np.uint64 and state.size == 16 and state.flags.c_contiguous
    out = np.empty(shape, dtype=dt)
    rc = _load().oracle_rand_fill(DTYPE_CODE[dt.name], out.ctypes.data, out.size,
                                  int(max_threads), state.ctypes.data)
    if rc != 0:
        raise RuntimeError("oracle_rand_fill failed")
    return out


# -- the compiled reference ------------------------------------------------

def reference_available(variant="avx2"):
    return os.path.exists(_build.REF_VARIANTS[variant][1]) or _build.reference_buildable()


def _load_ref(variant="avx2"):
    if variant not in _refs:
        path = _build.build_reference(variant)
        if path is None:
            raise RuntimeError(f"numc reference library ({variant}) not buildable here")
        lib = ctypes.CDLL(path)
        vp = ctypes.c_void_p
        lib.numc_ctx_create.restype = vp
        lib.numc_ctx_free.argtypes = [vp]
        lib.numc_array_create.restype = vp
        lib.numc_array_create.argtypes = [vp, vp, ctypes.c_size_t, ctypes.c_int]
        lib.numc_array_write.argtypes = [vp, vp]
        lib.numc_array_data.restype = vp
        lib.numc_array_data.argtypes = [vp]
        lib.numc_array_transpose.argtypes = [vp, vp]
        lib.numc_matmul.argtypes = [vp, vp, vp]
        lib.numc_matmul.restype = ctypes.c_int
        lib.numc_matmul_naive.argtypes = [vp, vp, vp]
        lib.numc_matmul_naive.restype = ctypes.c_int
        lib.numc_dot.argtypes = [vp, vp, vp]
        lib.numc_dot.restype = ctypes.c_int
        lib.numc_manual_seed.argtypes = [ctypes.c_uint64]
        lib.numc_array_rand.restype = vp
        lib.numc_array_rand.argtypes = [vp, vp, ctypes.c_size_t, ctypes.c_int]
        _refs[variant] = lib
    return _refs[variant]


def ref_matmul(a, b, naive=False, variant="avx2"):
    """Run numc's own numc_matmul (or numc_matmul_naive) on contiguous a, b,
    in numc's build `variant` (avx2, avx512 or neon)."""
    lib = _load_ref(variant)
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    M, K = a.shape
    N = b.shape[1]
    code = DTYPE_CODE[a.dtype.name]
    ctx = lib.numc_ctx_create()
    try:
        def make(shape, src=None):
            sh = (ctypes.c_size_t * 2)(*shape)
            arr = lib.numc_array_create(ctx, sh, 2, code)
            if not arr:
                raise MemoryError("numc_array_create failed")
            if src is not None:
                lib.numc_array_write(arr, src.ctypes.data)
            return arr
        pa, pb, pc = make((M, K), a), make((K, N), b), make((M, N))
        fn = lib.numc_matmul_naive if naive else lib.numc_matmul
        if naive:  # the naive kernel accumulates into out: start from zero
            z = np.zeros((M, N), dtype=a.dtype)
            lib.numc_array_write(pc, z.ctypes.data)
        rc = fn(pa, pb, pc)
        if rc != 0:
            raise RuntimeError(f"numc_matmul returned {rc}")
        out = np.empty((M, N), dtype=a.dtype)
        ctypes.memmove(out.ctypes.data, lib.numc_array_data(pc), out.nbytes)
        return out
    finally:
        lib.numc_ctx_free(ctx)


def ref_dot(a, b, perm_a=None, perm_b=None, perm_out=None, variant="avx2"):
    """numc's own numc_dot(a, b, out).  Each operand (and out) is created in
    numc as a contiguous array holding x.transpose(inverse(perm)) and then
    viewed with numc_array_transpose(perm), so a perm other than the identity
    gives numc a strided, non-contiguous view equal to x."""
    lib = _load_ref(variant)
    code = DTYPE_CODE[a.dtype.name]
    oshape = dot_shape(a.shape, b.shape)
    ctx = lib.numc_ctx_create()
    try:
        def make(x_shape, perm, src=None):
            nd = len(x_shape)
            perm = list(range(nd)) if perm is None else list(perm)
            inv = np.argsort(perm)
            base_shape = [x_shape[i] for i in inv]   # x = base.transpose(perm)
            sh = (ctypes.c_size_t * max(1, nd))(*base_shape)
            arr = lib.numc_array_create(ctx, sh, nd, code)
            if not arr:
                raise MemoryError("numc_array_create failed")
            if src is not None:
                base = np.ascontiguousarray(np.asarray(src).transpose(inv))
                lib.numc_array_write(arr, base.ctypes.data)
            else:
                z = np.zeros(base_shape, dtype=a.dtype)
                lib.numc_array_write(arr, z.ctypes.data)
            if perm != list(range(nd)):
                ax = (ctypes.c_size_t * nd)(*perm)
                if lib.numc_array_transpose(arr, ax) != 0:
                    raise RuntimeError("numc_array_transpose failed")
            return arr, base_shape, inv
        pa, _, _ = make(a.shape, perm_a, a)
        pb, _, _ = make(b.shape, perm_b, b)
        po, obase, oinv = make(oshape, perm_out)
        rc = lib.numc_dot(pa, pb, po)
        if rc != 0:
            raise RuntimeError(f"numc_dot returned {rc}")
        base = np.empty(obase, dtype=a.dtype)
        ctypes.memmove(base.ctypes.data, lib.numc_array_data(po), base.nbytes)
        perm = list(range(len(oshape))) if perm_out is None else list(perm_out)
        return np.ascontiguousarray(base.transpose(perm)).reshape(oshape)
    finally:
        lib.numc_ctx_free(ctx)


def ref_rand_sequence(seed, calls, omp_threads):
    """numc's own numc_array_rand over `calls` [(dtype, shape), ...] in one
    thread after numc_manual_seed(seed) (no seeding if seed is None), with
    numc's OpenMP maximum set to `omp_threads`.  Returns the arrays."""
    import threading
    lib = _load_ref()
    gomp = ctypes.CDLL("libgomp.so.1")
    result = {}

    def body():
        gomp.omp_set_num_threads(int(omp_threads))
        if seed is not None:
            lib.numc_manual_seed(int(seed) & (2**64 - 1))
        ctx = lib.numc_ctx_create()
        try:
            outs = []
            for dtype, shape in calls:
                dt = np.dtype(dtype)
                sh = (ctypes.c_size_t * len(shape))(*shape)
                arr = lib.numc_array_rand(ctx, sh, len(shape), DTYPE_CODE[dt.name])
                if not arr:
                    raise RuntimeError("numc_array_rand failed")
                out = np.empty(shape, dtype=dt)
                ctypes.memmove(out.ctypes.data, lib.numc_array_data(arr), out.nbytes)
                outs.append(out)
            result["outs"] = outs
        finally:
            lib.numc_ctx_free(ctx)

    # a fresh thread: numc's PRNG state is thread-local, so an unseeded
    # sequence starts from numc's default seed
    th = threading.Thread(target=body)
    th.start()
    th.join()
    return result["outs"]
