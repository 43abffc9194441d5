"""numc_gb300 — numc's matmul hot path on GB300 (sm_103a).

The product is the C-ABI shared library ``libnumc_gb300.so`` (headers in
include/numc/).  This module is a thin ctypes binding of it with the shape of
numc's C API, used by the tests and the benchmark: ``Ctx``/``Array`` mirror
NumcCtx/NumcArray, ``matmul`` is numc_matmul, and ``gemm`` is the
device-pointer entry numc_cuda_gemm for torch CUDA tensors.

There is no CPU fallback: if the library is not built, importing works but
every call raises ``NumcLibraryMissing``.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libnumc_gb300.so")

DTYPES = ["int8", "int16", "int32", "int64", "uint8", "uint16", "uint32",
          "uint64", "float32", "float64"]
CODE = {n: i for i, n in enumerate(DTYPES)}

# NumcErrorCode (include/numc/error.h)
ERR_NONE, ERR_NULL, ERR_MALLOC, ERR_SHAPE = 0, -1, -2, -3
ERR_TYPE, ERR_BOUNDS, ERR_VALUE, ERR_INTERNAL = -4, -5, -6, -99

# NumcCudaAlgo (include/numc/cuda.h)
(ALGO_DEFAULT, ALGO_SIMT, ALGO_SPLIT_BF16, ALGO_DMMA, ALGO_OZAKI, ALGO_AUTO, ALGO_TC_INT8,
 ALGO_SPLIT_FP16) = range(8)
INT8_X86_AVX2, INT8_ARM_NEON, INT8_WRAP, INT8_X86_AVX512 = 0, 1, 2, 3
INT8_TILE_AUTO, INT8_TILE_SINGLE, INT8_TILE_PAIR128, INT8_TILE_PAIR256 = 0, 1, 2, 3


class NumcLibraryMissing(RuntimeError):
    pass


class NumcError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"numc error {code}: {msg}")
        self.code = code
        self.msg = msg


class _Err(ctypes.Structure):
    _fields_ = [("code", ctypes.c_int), ("msg", ctypes.c_char_p)]


class _Checkpoint(ctypes.Structure):
    _fields_ = [("_block", ctypes.c_void_p), ("_index", ctypes.c_size_t)]


class _Slice(ctypes.Structure):
    _fields_ = [("axis", ctypes.c_size_t), ("start", ctypes.c_size_t),
                ("stop", ctypes.c_size_t), ("step", ctypes.c_size_t)]


_lib = None

# (name, restype, argtypes) for every exported function.
_VP, _SZ, _I, _IP = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_ssize_t
SIGNATURES = [
    ("numc_ctx_create", _VP, []),
    ("numc_ctx_free", None, [_VP]),
    ("numc_ctx_checkpoint", _Checkpoint, [_VP]),
    ("numc_ctx_restore", None, [_VP, _Checkpoint]),
    ("numc_array_create", _VP, [_VP, _VP, _SZ, _I]),
    ("numc_array_zeros", _VP, [_VP, _VP, _SZ, _I]),
    ("numc_array_fill", _VP, [_VP, _VP, _SZ, _I, _VP]),
    ("numc_array_copy", _VP, [_VP]),
    ("numc_array_write", None, [_VP, _VP]),
    ("numc_array_transpose", _I, [_VP, _VP]),
    ("numc_array_transpose_copy", _VP, [_VP, _VP]),
    ("numc_array_slice", _VP, [_VP, ctypes.POINTER(_Slice)]),
    ("numc_array_is_contiguous", ctypes.c_bool, [_VP]),
    ("numc_array_contiguous", _I, [_VP]),
    ("numc_array_size", _SZ, [_VP]),
    ("numc_array_capacity", _SZ, [_VP]),
    ("numc_array_elem_size", _SZ, [_VP]),
    ("numc_array_ndim", _SZ, [_VP]),
    ("numc_array_shape", None, [_VP, _VP]),
    ("numc_array_strides", None, [_VP, _VP]),
    ("numc_array_dtype", _I, [_VP]),
    ("numc_array_data", _VP, [_VP]),
    ("numc_matmul", _I, [_VP, _VP, _VP]),
    ("numc_matmul_naive", _I, [_VP, _VP, _VP]),
    ("numc_dot", _I, [_VP, _VP, _VP]),
    ("numc_linear", _I, [_VP, _VP, _VP, _VP]),
    ("numc_bmm", _I, [_VP, _VP, _VP]),
    ("numc_cuda_transfer_bytes", ctypes.c_uint64, []),
    ("numc_cuda_ctx_device_usage", _I, [_VP, ctypes.POINTER(ctypes.c_size_t),
                                        ctypes.POINTER(ctypes.c_size_t),
                                        ctypes.POINTER(ctypes.c_size_t)]),
    ("numc_set_error", _I, [_I, ctypes.c_char_p]),
    ("numc_get_error", _Err, []),
    ("numc_log_error", None, [_VP]),
    ("numc_cuda_device_count", _I, []),
    ("numc_cuda_set_algo", _I, [_I, _I, _I]),
    ("numc_cuda_get_algo", _I, [_I, ctypes.POINTER(_I), ctypes.POINTER(_I)]),
    ("numc_cuda_set_isa_profile", _I, [_I]),
    ("numc_cuda_get_isa_profile", _I, []),
    ("numc_cuda_array_to_device", _I, [_VP]),
    ("numc_cuda_array_to_host", _I, [_VP]),
    ("numc_cuda_array_device_data", _VP, [_VP]),
    ("numc_cuda_array_is_resident", _I, [_VP]),
    ("numc_cuda_ctx_stream", _VP, [_VP]),
    ("numc_cuda_ctx_synchronize", _I, [_VP]),
    ("numc_cuda_gemm_workspace_size", _SZ, [_I, _I, _I, _SZ, _SZ, _SZ]),
    ("numc_cuda_gemm", _I, [_I, _I, _I, _VP, _VP, _VP, _SZ, _SZ, _SZ,
                            _IP, _IP, _IP, _IP, _IP, _IP, _VP, _SZ, _VP]),
    ("numc_cuda_check_status", _I, [_VP]),
    ("numc_cuda_gemm_host", _I, [_I, _VP, _VP, _VP, _SZ, _SZ, _SZ, _IP, _IP, _IP, _IP]),
    ("numc_cuda_debug_fail_malloc", _I, [_I]),
    ("numc_cuda_debug_wait_timeout", _I, [ctypes.c_ulonglong, _I]),
    ("numc_cuda_launch_count", ctypes.c_uint64, []),
    ("numc_cuda_gemm_plan_create", _VP, [_I, _I, _I, _VP, _SZ]),
    ("numc_cuda_gemm_plan_run", _I, [_VP, _VP]),
    ("numc_cuda_gemm_plan_run_graph", _I, [_VP, _VP]),
    ("numc_cuda_gemm_plan_info", _I, [_VP, ctypes.POINTER(_I), ctypes.POINTER(_I),
                                      ctypes.POINTER(_I), ctypes.POINTER(_SZ)]),
    ("numc_cuda_gemm_plan_free", None, [_VP]),
    ("numc_matmul_grouped", _I, [_VP, _VP, _VP, _SZ]),
    ("numc_cuda_sgemm_split_static", _I, [_VP, _VP, _VP, _SZ, _SZ, _SZ, _IP, _IP, _IP, _IP,
                                          _IP, _IP, _VP, _VP]),
    ("numc_manual_seed", None, [ctypes.c_uint64]),
    ("numc_array_rand", _VP, [_VP, _VP, _SZ, _I]),
    ("numc_cuda_array_rand", _VP, [_VP, _VP, _SZ, _I]),
    ("numc_cuda_rand_fill", _I, [_I, _VP, _SZ, _VP]),
    ("numc_cuda_rand_set_threads", _I, [_I]),
    ("numc_cuda_rand_threads", _I, []),
    ("numc_cuda_phase_timing", _I, [_I]),
    ("numc_cuda_phase_times", _I, [ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                                   ctypes.POINTER(ctypes.c_uint64)]),
]


def lib():
    """The loaded C library; raises NumcLibraryMissing if it is not built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise NumcLibraryMissing(
                f"{LIB_PATH} is not built; run `python -m numc_gb300.build`")
        L = ctypes.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def last_error():
    e = lib().numc_get_error()
    return e.code, (e.msg or b"").decode(errors="replace")


def check(rc):
    if rc != 0:
        code, msg = last_error()
        raise NumcError(rc, msg)
    return rc


def device_count():
    return lib().numc_cuda_device_count()


def set_algo(dtype, algo, param=-1):
    """Process-wide algorithm of `dtype`; param -1 = the algorithm's default
    (for int8/uint8 and CUDA-core floats: the process-wide ISA profile)."""
    check(lib().numc_cuda_set_algo(CODE[np.dtype(dtype).name], algo, param))


def get_algo(dtype):
    a, p = ctypes.c_int(), ctypes.c_int()
    check(lib().numc_cuda_get_algo(CODE[np.dtype(dtype).name], ctypes.byref(a), ctypes.byref(p)))
    return a.value, p.value


def set_isa_profile(profile):
    """Which numc build's results to reproduce (INT8_X86_AVX2, INT8_ARM_NEON
    or INT8_X86_AVX512) where numc's arithmetic depends on its ISA."""
    check(lib().numc_cuda_set_isa_profile(profile))


def get_isa_profile():
    return lib().numc_cuda_get_isa_profile()


def launch_count():
    return lib().numc_cuda_launch_count()


def transfer_bytes():
    """Bytes of array data copied between host and device so far."""
    return lib().numc_cuda_transfer_bytes()


class Ctx:
    """NumcCtx: owns every Array created from it."""

    def __init__(self):
        self.ptr = lib().numc_ctx_create()
        if not self.ptr:
            raise NumcError(*last_error())

    def free(self):
        if self.ptr:
            lib().numc_ctx_free(self.ptr)
            self.ptr = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.free()

    def checkpoint(self):
        return lib().numc_ctx_checkpoint(self.ptr)

    def restore(self, cp):
        lib().numc_ctx_restore(self.ptr, cp)

    def stream(self):
        return lib().numc_cuda_ctx_stream(self.ptr)

    def device_usage(self):
        """(slabs, reserved_bytes, used_bytes) of the context's device arena."""
        n, r, u = ctypes.c_size_t(), ctypes.c_size_t(), ctypes.c_size_t()
        check(lib().numc_cuda_ctx_device_usage(self.ptr, ctypes.byref(n), ctypes.byref(r),
                                               ctypes.byref(u)))
        return n.value, r.value, u.value

    def synchronize(self):
        check(lib().numc_cuda_ctx_synchronize(self.ptr))

    def _make(self, fn, shape, dtype, *extra):
        shape = tuple(int(s) for s in shape)
        sh = (ctypes.c_size_t * max(1, len(shape)))(*shape)
        p = fn(self.ptr, sh, len(shape), CODE[np.dtype(dtype).name], *extra)
        if not p:
            raise NumcError(*last_error())
        return Array(p, self)

    def create(self, shape, dtype):
        return self._make(lib().numc_array_create, shape, dtype)

    def zeros(self, shape, dtype):
        return self._make(lib().numc_array_zeros, shape, dtype)

    def fill(self, shape, dtype, value):
        v = np.array(value, dtype=dtype)
        return self._make(lib().numc_array_fill, shape, dtype, v.ctypes.data)

    def rand(self, shape, dtype):
        """numc_array_rand: numc's uniform values, generated on the GPU and
        copied into the host buffer."""
        return self._make(lib().numc_array_rand, shape, dtype)

    def rand_device(self, shape, dtype):
        """numc_cuda_array_rand: the same values, left resident in HBM."""
        return self._make(lib().numc_cuda_array_rand, shape, dtype)

    def from_numpy(self, x):
        x = np.array(x, order="C")      # a C-contiguous copy; 0-D stays 0-D
        arr = self.create(x.shape, x.dtype)
        arr.write(x)
        return arr


class Array:
    """NumcArray handle (owned by its Ctx)."""

    def __init__(self, ptr, ctx):
        self.ptr = ptr
        self.ctx = ctx

    @property
    def ndim(self):
        return lib().numc_array_ndim(self.ptr)

    @property
    def shape(self):
        n = self.ndim
        buf = (ctypes.c_size_t * max(1, n))()
        lib().numc_array_shape(self.ptr, buf)
        return tuple(buf[:n])

    @property
    def strides(self):
        n = self.ndim
        buf = (ctypes.c_size_t * max(1, n))()
        lib().numc_array_strides(self.ptr, buf)
        return tuple(buf[:n])

    @property
    def dtype(self):
        return np.dtype(DTYPES[lib().numc_array_dtype(self.ptr)])

    def write(self, x):
        x = np.ascontiguousarray(x, dtype=self.dtype)
        assert x.size == lib().numc_array_size(self.ptr)
        lib().numc_array_write(self.ptr, x.ctypes.data)

    def numpy(self):
        """Copy of the host data as a numpy array with this view's strides."""
        L = lib()
        data = L.numc_array_data(self.ptr)
        n = L.numc_array_size(self.ptr)
        es = self.dtype.itemsize
        if n == 0:
            return np.zeros(self.shape, dtype=self.dtype)
        shape, strides = self.shape, self.strides
        span = es + sum((s - 1) * st for s, st in zip(shape, strides))
        raw = (ctypes.c_char * span).from_address(data)
        base = np.frombuffer(raw, dtype=np.uint8)
        view = np.lib.stride_tricks.as_strided(base.view(self.dtype) if span % es == 0
                                               else base[: span - span % es].view(self.dtype),
                                               shape=shape, strides=strides)
        return np.array(view)

    def transpose(self, axes):
        ax = (ctypes.c_size_t * len(axes))(*axes)
        if lib().numc_array_transpose(self.ptr, ax) != 0:
            raise NumcError(*last_error())
        return self

    def slice(self, axis, start=0, stop=0, step=1):
        s = _Slice(axis, start, stop, step)
        p = lib().numc_array_slice(self.ptr, ctypes.byref(s))
        if not p:
            raise NumcError(*last_error())
        return Array(p, self.ctx)

    def copy(self):
        p = lib().numc_array_copy(self.ptr)
        if not p:
            raise NumcError(*last_error())
        return Array(p, self.ctx)

    def contiguous(self):
        """numc_array_contiguous: re-lay this array out row-major in place."""
        if lib().numc_array_contiguous(self.ptr) != 0:
            raise NumcError(*last_error())
        return self

    def is_contiguous(self):
        return lib().numc_array_is_contiguous(self.ptr)

    def to_device(self):
        check(lib().numc_cuda_array_to_device(self.ptr))
        return self

    def to_host(self):
        check(lib().numc_cuda_array_to_host(self.ptr))
        return self

    def is_resident(self):
        return bool(lib().numc_cuda_array_is_resident(self.ptr))

    def device_ptr(self):
        return lib().numc_cuda_array_device_data(self.ptr)


def matmul(a, b, out):
    """numc_matmul(a, b, out); raises NumcError on a nonzero return."""
    return check(lib().numc_matmul(a.ptr if a else None, b.ptr if b else None,
                                   out.ptr if out else None))


def matmul_naive(a, b, out):
    return check(lib().numc_matmul_naive(a.ptr, b.ptr, out.ptr))


def linear(x, w, bias, out):
    """numc_linear(x, w, bias, out): out = x @ w + bias (bias may be None)."""
    return check(lib().numc_linear(x.ptr if x else None, w.ptr if w else None,
                                   bias.ptr if bias else None, out.ptr if out else None))


def bmm(a, b, out):
    """numc_bmm(a, b, out): batched numc_matmul over the leading axes."""
    return check(lib().numc_bmm(a.ptr if a else None, b.ptr if b else None,
                                out.ptr if out else None))


def dot(a, b, out):
    """numc_dot(a, b, out); raises NumcError on a nonzero return."""
    return check(lib().numc_dot(a.ptr if a else None, b.ptr if b else None,
                                out.ptr if out else None))


def workspace_size(dtype, algo, param, M, K, N):
    return lib().numc_cuda_gemm_workspace_size(CODE[np.dtype(dtype).name], algo, param, M, K, N)


def gemm(a, b, out, algo=ALGO_DEFAULT, param=-1, workspace=None, stream=None):
    """numc_cuda_gemm on 2-D torch CUDA tensors (any element strides).

    `workspace` is an optional torch uint8 CUDA tensor; `stream` a
    torch.cuda.Stream (default: the current stream)."""
    import torch
    dt = CODE[str(a.dtype).replace("torch.", "")]
    M, K = a.shape
    N = b.shape[1]
    if stream is None:
        stream = torch.cuda.current_stream()
    ws_ptr, ws_bytes = (workspace.data_ptr(), workspace.numel()) if workspace is not None else (None, 0)
    rc = lib().numc_cuda_gemm(dt, algo, param, a.data_ptr(), b.data_ptr(), out.data_ptr(),
                              M, K, N, a.stride(0), a.stride(1), b.stride(0), b.stride(1),
                              out.stride(0), out.stride(1), ws_ptr, ws_bytes,
                              stream.cuda_stream)
    return check(rc)


def manual_seed(seed):
    """numc_manual_seed for the calling thread."""
    lib().numc_manual_seed(int(seed) & (2**64 - 1))


def rand_set_threads(threads):
    """numc's OpenMP maximum that the large-array rand layout follows (0: default)."""
    check(lib().numc_cuda_rand_set_threads(int(threads)))


def rand_threads():
    return lib().numc_cuda_rand_threads()


def rand_fill(t, stream=None):
    """numc_cuda_rand_fill over a contiguous torch CUDA tensor (numc's dtype
    of the same name; float32/float64 or an integer type)."""
    import torch
    assert t.is_contiguous()
    dt = CODE[str(t.dtype).replace("torch.", "")]
    if stream is None:
        stream = torch.cuda.current_stream()
    return check(lib().numc_cuda_rand_fill(dt, t.data_ptr(), t.numel(), stream.cuda_stream))


def check_status(stream=None):
    import torch
    if stream is None:
        stream = torch.cuda.current_stream()
    return check(lib().numc_cuda_check_status(stream.cuda_stream))


def phase_timing(enable):
    check(lib().numc_cuda_phase_timing(1 if enable else 0))


def phase_times():
    """(prep_ms_total, gemm_ms_total, calls) since phase_timing(True)."""
    p, g, n = ctypes.c_double(), ctypes.c_double(), ctypes.c_uint64()
    check(lib().numc_cuda_phase_times(ctypes.byref(p), ctypes.byref(g), ctypes.byref(n)))
    return p.value, g.value, n.value


class GemmDesc(ctypes.Structure):
    """NumcCudaGemmDesc."""
    _fields_ = [("a", ctypes.c_void_p), ("b", ctypes.c_void_p), ("out", ctypes.c_void_p),
                ("M", ctypes.c_size_t), ("K", ctypes.c_size_t), ("N", ctypes.c_size_t),
                ("rsa", ctypes.c_ssize_t), ("csa", ctypes.c_ssize_t),
                ("rsb", ctypes.c_ssize_t), ("csb", ctypes.c_ssize_t),
                ("rso", ctypes.c_ssize_t), ("cso", ctypes.c_ssize_t)]


class GemmPlan:
    """A grouped GEMM plan over torch CUDA tensors (a_i @ b_i -> out_i)."""

    def __init__(self, problems, algo=ALGO_DEFAULT, param=0):
        n = len(problems)
        self._keep = problems            # tensors must outlive the plan
        arr = (GemmDesc * max(1, n))()
        for i, (a, b, out) in enumerate(problems):
            arr[i] = GemmDesc(a.data_ptr(), b.data_ptr(), out.data_ptr(), a.shape[0],
                              a.shape[1], b.shape[1], a.stride(0), a.stride(1),
                              b.stride(0), b.stride(1), out.stride(0), out.stride(1))
        self.ptr = lib().numc_cuda_gemm_plan_create(CODE["float32"], algo, param, arr, n)
        if not self.ptr:
            raise NumcError(*last_error())

    def run(self, stream=None, graph=False):
        import torch
        s = (stream or torch.cuda.current_stream()).cuda_stream
        fn = lib().numc_cuda_gemm_plan_run_graph if graph else lib().numc_cuda_gemm_plan_run
        check(fn(self.ptr, s))

    def info(self):
        a, b, c, w = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_size_t()
        check(lib().numc_cuda_gemm_plan_info(self.ptr, ctypes.byref(a), ctypes.byref(b),
                                             ctypes.byref(c), ctypes.byref(w)))
        return {"tc128": a.value, "tc64": b.value, "simt": c.value, "workspace_bytes": w.value}

    def free(self):
        if self.ptr:
            lib().numc_cuda_gemm_plan_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def matmul_grouped(As, Bs, Outs):
    """numc_matmul_grouped over lists of Array."""
    n = len(As)
    pa = (ctypes.c_void_p * max(1, n))(*[x.ptr for x in As])
    pb = (ctypes.c_void_p * max(1, n))(*[x.ptr for x in Bs])
    po = (ctypes.c_void_p * max(1, n))(*[x.ptr for x in Outs])
    return check(lib().numc_matmul_grouped(pa, pb, po, n))
