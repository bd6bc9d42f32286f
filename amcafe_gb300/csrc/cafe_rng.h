// The reference's random streams, restated for host and device code.
//
// AMCAFE draws every random number from std::default_random_engine, which in
// libstdc++ is minstd_rand0 (x <- 16807 x mod 2^31-1, seed s mod m, 0 -> 1),
// through std::uniform_real_distribution<double>(0,1), which calls
// std::generate_canonical<double,53>: with range r = 2^31-2 it takes k = 2
// engine outputs and returns ((x1-1) + (x2-1) r) / r^2 evaluated in double
// (r^2 rounded to double), clamped below 1. Call sites: VoxelsCA.C:340-341,
// 380, 483 (per-step ruq offsets and nucleation draws), SampleOrientation.C:
// 128-135 (orientations). The device needs random access into a stream, so
// jump-ahead by k outputs is 16807^k mod m by square-and-multiply.
#ifndef CAFE_RNG_H
#define CAFE_RNG_H
#include <stdint.h>

#if defined(__CUDACC__)
#define RNG_HD __host__ __device__ __forceinline__
#else
#define RNG_HD static inline
#endif

#define CAFE_MINSTD_A 16807u
#define CAFE_MINSTD_M 2147483647u

RNG_HD uint32_t cafe_minstd_seed(uint64_t s) {
  uint32_t x = (uint32_t)(s % CAFE_MINSTD_M);
  return x == 0 ? 1u : x;
}
RNG_HD uint32_t cafe_minstd_next(uint32_t x) {
  return (uint32_t)(((uint64_t)x * CAFE_MINSTD_A) % CAFE_MINSTD_M);
}
// a^k mod m
RNG_HD uint32_t cafe_minstd_pow(uint64_t k) {
  uint64_t r = 1, b = CAFE_MINSTD_A;
  while (k) {
    if (k & 1) r = (r * b) % CAFE_MINSTD_M;
    b = (b * b) % CAFE_MINSTD_M;
    k >>= 1;
  }
  return (uint32_t)r;
}
// state after advancing k outputs
RNG_HD uint32_t cafe_minstd_skip(uint32_t x, uint64_t k) {
  return (uint32_t)(((uint64_t)x * cafe_minstd_pow(k)) % CAFE_MINSTD_M);
}

// generate_canonical<double,53> from two consecutive outputs x1, x2.
RNG_HD double cafe_canonical(uint32_t x1, uint32_t x2) {
  const double r = 2147483646.0;
  const double r2 = 4611686009837453316.0;  // (2^31-2)^2 rounded to double
  double sum = (double)(x1 - 1u);
  sum = sum + (double)(x2 - 1u) * r;
  double ret = sum / r2;
  if (ret >= 1.0) ret = 0x1.fffffffffffffp-1;
  return ret;
}

// Sequential uniform stream: each call consumes two engine outputs.
struct cafe_uniform_stream {
  uint32_t x;
};
RNG_HD double cafe_uniform_next(cafe_uniform_stream *s) {
  uint32_t x1 = cafe_minstd_next(s->x);
  uint32_t x2 = cafe_minstd_next(x1);
  s->x = x2;
  return cafe_canonical(x1, x2);
}
// The i-th uniform (0-based) of the stream seeded with `seed`.
RNG_HD double cafe_uniform_at(uint32_t seed_state, uint64_t i) {
  uint32_t x1 = cafe_minstd_skip(seed_state, 2 * i + 1);
  uint32_t x2 = cafe_minstd_next(x1);
  return cafe_canonical(x1, x2);
}
#endif
