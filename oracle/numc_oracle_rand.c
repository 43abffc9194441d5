/*
 * numc_oracle_rand.c — CPU restatement of numc's uniform random fill
 * (numc_manual_seed / numc_array_rand: src/random/kernel.h,
 * src/random/random.c).
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA backend's random
 * fill; the product library never links, loads or calls it.
 *
 * State (kernel.h:40-41): four xoshiro256** streams ("lanes") in numc's
 * structure-of-arrays layout st[word * 4 + lane].
 *
 * Seeding (prng_seed, kernel.h:100-121): lane 0 = four successive
 * splitmix64 outputs of the seed; lane l + 1 = lane l advanced 2^128 steps
 * by xoshiro256's published jump polynomial.  A thread that never seeded
 * uses seed 0xdeadbeefcafe1234 (kernel.h:123-126).
 *
 * One xoshiro256** step (kernel.h:177-189): output rotl(s1 * 5, 7) * 9,
 * then t = s1 << 17; s2 ^= s0; s3 ^= s1; s1 ^= s2; s0 ^= s3; s2 ^= t;
 * s3 = rotl(s3, 45).
 *
 * One numc_array_rand call over n elements of `size` bytes
 * (DEFINE_RAND_KERNEL, kernel.h:296-400; the float64 AVX2 variant,
 * random.c:68-180, converts the same raw values the same way):
 *  - n * size <= 1 MiB (NUMC_OMP_BYTE_THRESHOLD): element 4j + l is lane
 *    l's j-th output for j < n / 4; the n % 4 tail elements continue lane 0.
 *    Afterwards every lane has advanced n / 4 steps and lane 0 n % 4 more.
 *  - otherwise T = n * size / 512 KiB threads, at most the OpenMP
 *    maximum (NUMC_OMP_CAP_THREADS, internal.h:102-107), chunk =
 *    ceil(n / T); thread t covers [t * chunk, min(t * chunk + chunk, n)).
 *    With X(m) the output of lane 0's state after m steps, element
 *    start + 4j + l is X(start + l + j) for j < J = len / 4, and element
 *    start + 4J + r is X(start + J + r).  Afterwards every lane has
 *    advanced n steps.
 * Conversion (random.c:28-39, kernel.h:200-212): integers keep the low
 * bits of the raw value; float32 is (raw >> 41 | 0x3F800000) - 1.0f and
 * float64 (raw >> 11 | 0x3FF0000000000000) - 1.0, both exact.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

static uint64_t rotl64(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

static uint64_t splitmix64(uint64_t *x) {
  uint64_t z = (*x += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

/* one step of stream s[0..3]; returns its output */
static uint64_t step(uint64_t s[4]) {
  const uint64_t r = rotl64(s[1] * 5, 7) * 9;
  const uint64_t t = s[1] << 17;
  s[2] ^= s[0];
  s[3] ^= s[1];
  s[1] ^= s[2];
  s[0] ^= s[3];
  s[2] ^= t;
  s[3] = rotl64(s[3], 45);
  return r;
}

/* xoshiro256's published 2^128-step jump polynomial */
static void jump128(uint64_t s[4]) {
  static const uint64_t J[4] = {0x180ec6d33cfd0abaull, 0xd5a61266f0c9392cull,
                                0xa9582618e03fc9aaull, 0x39abdc4529b1661cull};
  uint64_t a[4] = {0, 0, 0, 0};
  for (int i = 0; i < 4; i++)
    for (int b = 0; b < 64; b++) {
      if (J[i] & (1ull << b))
        for (int w = 0; w < 4; w++) a[w] ^= s[w];
      step(s);
    }
  memcpy(s, a, sizeof a);
}

void oracle_rand_seed(uint64_t seed, uint64_t st[16]) {
  uint64_t base[4];
  for (int w = 0; w < 4; w++) base[w] = splitmix64(&seed);
  for (int w = 0; w < 4; w++) st[w * 4 + 0] = base[w];
  for (int l = 1; l < 4; l++) {
    jump128(base);
    for (int w = 0; w < 4; w++) st[w * 4 + l] = base[w];
  }
}

static void lane_get(const uint64_t st[16], int l, uint64_t s[4]) {
  for (int w = 0; w < 4; w++) s[w] = st[w * 4 + l];
}
static void lane_put(uint64_t st[16], int l, const uint64_t s[4]) {
  for (int w = 0; w < 4; w++) st[w * 4 + l] = s[w];
}

static void store(int dtype, void *out, int64_t i, uint64_t raw) {
  switch (dtype) {
  case 0: case 4: ((uint8_t *)out)[i] = (uint8_t)raw; break;      /* int8, uint8 */
  case 1: case 5: ((uint16_t *)out)[i] = (uint16_t)raw; break;    /* int16, uint16 */
  case 2: case 6: ((uint32_t *)out)[i] = (uint32_t)raw; break;    /* int32, uint32 */
  case 3: case 7: ((uint64_t *)out)[i] = raw; break;              /* int64, uint64 */
  case 8: {
    const uint32_t bits = (uint32_t)(raw >> 41) | 0x3F800000u;
    float v;
    memcpy(&v, &bits, sizeof v);
    ((float *)out)[i] = v - 1.0f;
    break;
  }
  default: {
    const uint64_t bits = (raw >> 11) | 0x3FF0000000000000ull;
    double v;
    memcpy(&v, &bits, sizeof v);
    ((double *)out)[i] = v - 1.0;
    break;
  }
  }
}

static const int kSize[10] = {1, 2, 4, 8, 1, 2, 4, 8, 4, 8};

/* numc's thread count for the large path: n * size / 512 KiB capped at
 * max_threads (numc's omp_get_max_threads()), at least 1. */
int oracle_rand_threads(int dtype, int64_t n, int max_threads) {
  const int64_t bytes = n * kSize[dtype];
  if (bytes <= (1 << 20)) return 0; /* small path */
  int64_t t = bytes / (1 << 19);
  if (t > max_threads) t = max_threads;
  return t < 1 ? 1 : (int)t;
}

/* One numc_array_rand fill of n elements; st is advanced as numc advances
 * its thread-local state.  Returns 0, or -1 on a bad dtype. */
int oracle_rand_fill(int dtype, void *out, int64_t n, int max_threads, uint64_t st[16]) {
  if (dtype < 0 || dtype > 9 || n < 0) return -1;
  const int T = oracle_rand_threads(dtype, n, max_threads);
  if (T == 0) {
    const int64_t J = n / 4;
    for (int l = 0; l < 4; l++) {
      uint64_t s[4];
      lane_get(st, l, s);
      for (int64_t j = 0; j < J; j++) store(dtype, out, 4 * j + l, step(s));
      if (l == 0)
        for (int64_t i = 4 * J; i < n; i++) store(dtype, out, i, step(s));
      lane_put(st, l, s);
    }
    return 0;
  }
  /* X(m) for m in [0, n + 3): every value the threads use */
  uint64_t *X = (uint64_t *)malloc((size_t)(n + 3) * sizeof(uint64_t));
  if (!X) return -1;
  uint64_t s[4];
  lane_get(st, 0, s);
  for (int64_t m = 0; m < n + 3; m++) X[m] = step(s);
  const int64_t chunk = (n + T - 1) / T;
  for (int t = 0; t < T; t++) {
    const int64_t start = (int64_t)t * chunk;
    if (start >= n) break;
    const int64_t end = start + chunk < n ? start + chunk : n;
    const int64_t J = (end - start) / 4;
    for (int64_t j = 0; j < J; j++)
      for (int l = 0; l < 4; l++) store(dtype, out, start + 4 * j + l, X[start + l + j]);
    for (int64_t i = start + 4 * J; i < end; i++)
      store(dtype, out, i, X[start + J + (i - start - 4 * J)]);
  }
  free(X);
  for (int l = 0; l < 4; l++) {
    lane_get(st, l, s);
    for (int64_t m = 0; m < n; m++) step(s);
    lane_put(st, l, s);
  }
  return 0;
}
