"""Seeded synthetic matmul inputs (splitmix64 streams).

Every operand is drawn from its own splitmix64 stream, selected by
``(seed, stream)``, so any array can be regenerated bit-for-bit on any host
from two integers.  splitmix64 is Steele, Lea and Flood's generator
("Fast splittable pseudorandom number generators", OOPSLA 2014), the same
generator numc uses to seed its xoshiro256** state (src/random/kernel.h:46-51).

Value maps (x is a 64-bit draw):
  float32 uniform [lo, hi):  u = (x >> 40) * 2^-24
  float64 uniform [lo, hi):  u = (x >> 11) * 2^-53
  integers uniform [lo, hi]: lo + ((x >> 32) * (hi - lo + 1)) >> 32
  normal:                    Box-Muller on two float64 uniforms

Bit-for-bit on every host: the logarithm, cosine and exponential needed by
Box-Muller and the ill-scaled factors are evaluated here from IEEE
additions, multiplications, divisions and square roots in a fixed order
(series after exact range reduction), never through the platform's libm,
whose last bits differ between x86-64 and aarch64 builds.
"""
import math

import numpy as np

_CHUNK = 1 << 20
_LN2 = 0.6931471805599453        # float64 nearest ln 2
_LN10 = 2.302585092994046        # float64 nearest ln 10
_TWO_PI = 6.283185307179586      # float64 nearest 2 pi
# log(m) = 2 z sum z^2n / (2n + 1), z = (m - 1) / (m + 1), |z| <= 1/3
_LOG_C = [1.0 / (2 * n + 1) for n in range(19)]
# cos x = sum (-1)^n x^2n / (2n)!, 0 <= x <= pi / 2
_COS_C = [(-1.0) ** n / math.factorial(2 * n) for n in range(14)]
# exp r = sum r^n / n!, |r| <= ln 2 / 2
_EXP_C = [1.0 / math.factorial(n) for n in range(20)]


def _horner(coeffs, x):
    s = np.full_like(x, coeffs[-1])
    for c in reversed(coeffs[:-1]):
        s *= x
        s += c
    return s


def _log01(u):
    """ln u for float64 u in (0, 1]."""
    m, e = np.frexp(u)                       # u = m 2^e exactly, m in [0.5, 1)
    z = (m - 1.0) / (m + 1.0)
    return e * _LN2 + 2.0 * z * _horner(_LOG_C, z * z)


def _cos2pi(v):
    """cos(2 pi v) for float64 v in [0, 1)."""
    w = np.where(v >= 0.5, v - 1.0, v)       # exact, in [-0.5, 0.5)
    r = np.abs(w)
    flip = r > 0.25
    r = np.where(flip, 0.5 - r, r)           # exact, in [0, 0.25]
    x = _TWO_PI * r
    c = _horner(_COS_C, x * x)
    return np.where(flip, -c, c)


def _exp(y):
    """e^y for float64 y of moderate size (|y| < 700)."""
    k = np.rint(y / _LN2)
    r = y - k * _LN2
    return np.ldexp(_horner(_EXP_C, r), k.astype(np.int64))

GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)
_STREAM = np.uint64(0xD1B54A32D192ED03)


def _mix(z):
    with np.errstate(over="ignore"):
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
    return z ^ (z >> np.uint64(31))


def draws(seed, stream, n, start=0):
    """n consecutive splitmix64 outputs of stream `stream` under `seed`,
    beginning with output number `start`."""
    with np.errstate(over="ignore"):
        base = _mix(np.uint64(seed) ^ (np.uint64(stream) * _STREAM))
        idx = np.arange(start + 1, start + n + 1, dtype=np.uint64)
        return _mix(base + idx * GOLDEN)


def _parallel_chunks(n, fn):
    """fn(s, e) for consecutive chunks [s, e) of range(n), on a thread pool
    (numpy releases the interpreter lock in its array loops)."""
    spans = [(s, min(n, s + _CHUNK)) for s in range(0, n, _CHUNK)]
    if len(spans) <= 1:
        for s, e in spans:
            fn(s, e)
        return
    from concurrent.futures import ThreadPoolExecutor
    import os
    with ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 1)) as ex:
        list(ex.map(lambda se: fn(*se), spans))


def uniform(seed, stream, shape, lo=-1.0, hi=1.0, dtype=np.float32):
    n = int(np.prod(shape))
    x = draws(seed, stream, n)
    if np.dtype(dtype) == np.float32:
        u = (x >> np.uint64(40)).astype(np.float64) * 2.0 ** -24
    else:
        u = (x >> np.uint64(11)).astype(np.float64) * 2.0 ** -53
    return (lo + (hi - lo) * u).astype(dtype).reshape(shape)


def integers(seed, stream, shape, lo, hi, dtype):
    n = int(np.prod(shape))
    x = draws(seed, stream, n)
    span = np.uint64(hi - lo + 1)
    with np.errstate(over="ignore"):
        v = ((x >> np.uint64(32)) * span) >> np.uint64(32)
    return (v.astype(np.int64) + lo).astype(dtype).reshape(shape)


def normal(seed, stream, shape, dtype=np.float32):
    n = int(np.prod(shape))
    out = np.empty(n, dtype=dtype)

    def chunk(s, e):                          # element i uses draws 2i, 2i + 1
        xs = draws(seed, stream, 2 * (e - s), start=2 * s)
        u1 = ((xs[0::2] >> np.uint64(11)).astype(np.float64) + 1.0) * 2.0 ** -53
        u2 = (xs[1::2] >> np.uint64(11)).astype(np.float64) * 2.0 ** -53
        z = np.sqrt(-2.0 * _log01(u1)) * _cos2pi(u2)
        out[s:e] = z.astype(dtype)
    _parallel_chunks(n, chunk)
    return out.reshape(shape)


def ill_scales(seed, M, N):
    """Row factors 10^u_i of A and column factors 10^v_j of B, u, v ~ U(-4, 4),
    for the ill-scaled workload (applied to the `normal` operands)."""
    u = uniform(seed, 7, (M,), -4.0, 4.0, np.float64)
    v = uniform(seed, 8, (N,), -4.0, 4.0, np.float64)
    return _exp(u * _LN10), _exp(v * _LN10)


# Value ranges of the integer-exactness workload (1024^3).
INT_RANGES = {
    "int8": (-128, 127), "uint8": (0, 255), "int16": (-32768, 32767),
    "uint16": (0, 65535), "int32": (-1000, 1000), "uint32": (0, 2000),
    "int64": (-(1 << 20), 1 << 20), "uint64": (0, 1 << 21),
}


def operands(kind, M, K, N, seed=42, dtype="float32"):
    """(A, B) for one workload kind:

    uniform     entries uniform in [-1, 1) (float) or INT_RANGES (integers)
    normal      entries N(0, 1)
    illscaled   the `normal` operands with row i of A times 10^u_i and column
                j of B times 10^v_j, u, v ~ U(-4, 4) (float64 product, then
                rounded to the dtype)
    expspread   float64 uniform [-1, 1) times 2^e, e integer U(-20, 20)
                per element
    smallint    numc's own test fill: A[i] = (i % 7) + 1, B[i] = (i % 5) + 1
    extreme     integers only: each entry the dtype's maximum with
                probability 7/8, else its minimum (long K drives the int32
                sums of 8-bit products past 2^31: saturation and
                wraparound cases)
    """
    dt = np.dtype(dtype)
    if kind == "smallint":
        a = ((np.arange(M * K) % 7) + 1).astype(dt).reshape(M, K)
        b = ((np.arange(K * N) % 5) + 1).astype(dt).reshape(K, N)
        return a, b
    if kind == "uniform":
        if dt.kind == "f":
            return (uniform(seed, 1, (M, K), dtype=dt),
                    uniform(seed, 2, (K, N), dtype=dt))
        lo, hi = INT_RANGES[dt.name]
        return (integers(seed, 1, (M, K), lo, hi, dt),
                integers(seed, 2, (K, N), lo, hi, dt))
    if kind == "normal":
        return normal(seed, 3, (M, K), dt), normal(seed, 4, (K, N), dt)
    if kind == "extreme":
        info = np.iinfo(dt)
        pick_a = integers(seed, 13, (M, K), 0, 7, np.int64)
        pick_b = integers(seed, 14, (K, N), 0, 7, np.int64)
        return (np.where(pick_a == 0, info.min, info.max).astype(dt),
                np.where(pick_b == 0, info.min, info.max).astype(dt))
    if kind == "illscaled":
        a, b = normal(seed, 3, (M, K), dt), normal(seed, 4, (K, N), dt)
        u, v = ill_scales(seed, M, N)
        return ((a.astype(np.float64) * u[:, None]).astype(dt),
                (b.astype(np.float64) * v[None, :]).astype(dt))
    if kind == "expspread":
        a = uniform(seed, 9, (M, K), dtype=np.float64)
        b = uniform(seed, 10, (K, N), dtype=np.float64)
        ea = integers(seed, 11, (M, K), -20, 20, np.int64)
        eb = integers(seed, 12, (K, N), -20, 20, np.int64)
        return ((np.ldexp(a, ea)).astype(dt), (np.ldexp(b, eb)).astype(dt))
    raise ValueError(f"unknown workload kind {kind!r}")


def array(kind, shape, seed=42, stream=1, dtype="float32"):
    """One seeded array of any shape: `uniform` (as in operands) or `normal`
    (float dtypes), from stream `stream` of `seed`."""
    dt = np.dtype(dtype)
    shape = tuple(int(s) for s in shape)
    if kind == "normal" and dt.kind == "f":
        return normal(seed, stream, shape, dt)
    if dt.kind == "f":
        return uniform(seed, stream, shape, dtype=dt)
    lo, hi = INT_RANGES[dt.name]
    return integers(seed, stream, shape, lo, hi, dt)


def grouped_case(torch, dev, seed=42, problems=2048, chains=256):
    """The batched uneven workload as torch CUDA tensors: `problems`
    float32 matmuls with M, N, K each log-uniform in [16, 1024] (rounded),
    entries U[-1, 1), plus `chains` MLP chains X[256,784] -> W1[784,128] ->
    W2[128,10] with X ~ U[-1, 1) and W ~ N(0, 0.05).  Drawn on the device
    from torch generators seeded with `seed`.  Returns (dims, probs, chains,
    algorithmic flops): probs[i] = (a, b, out), chains[i] = (x, w1, w2, h, y)."""
    rng = np.random.default_rng(seed)
    dims = np.exp(rng.uniform(np.log(16), np.log(1024), (problems, 3))).round().astype(int)
    gen = torch.Generator(device=dev).manual_seed(seed)
    probs = []
    for (Mi, Ni, Ki) in dims:
        a = torch.rand((Mi, Ki), device=dev, generator=gen) * 2 - 1
        b = torch.rand((Ki, Ni), device=dev, generator=gen) * 2 - 1
        probs.append((a, b, torch.empty((Mi, Ni), device=dev)))
    mlp = []
    for _ in range(chains):
        x = torch.rand((256, 784), device=dev, generator=gen) * 2 - 1
        w1 = torch.randn((784, 128), device=dev, generator=gen) * 0.05
        w2 = torch.randn((128, 10), device=dev, generator=gen) * 0.05
        mlp.append((x, w1, w2, torch.empty((256, 128), device=dev),
                    torch.empty((256, 10), device=dev)))
    flops = float(sum(2.0 * m * n * k for m, n, k in dims)) + \
        chains * 2.0 * 256 * (784 * 128 + 128 * 10)
    return dims, probs, mlp, flops
