// Mersenne twister of the McICA generator (mcica_random_numbers.f90:77-306),
// device side.  The reference's int32 arithmetic with logical ishft is uint32
// arithmetic; getRandomReal is u32 / (2^32 - 1) in double precision.
#pragma once
#include <stdint.h>

namespace gbmt {

__device__ __forceinline__ uint32_t temper(uint32_t y) {
  uint32_t x = y ^ (y >> 11);
  x ^= (x << 7) & 0x9d2c5680u;
  x ^= (x << 15) & 0xefc60000u;
  return x ^ (x >> 18);
}
__device__ __forceinline__ uint32_t twist(uint32_t u, uint32_t v) {
  return (((u & 0x80000000u) | (v & 0x7fffffffu)) >> 1) ^ ((v & 1u) ? 0x9908b0dfu : 0u);
}
__device__ __forceinline__ double real(uint32_t u) { return (double)u / 4294967295.0; }

// First n <= 226 outputs of MT(seed) as getRandomReal values.  They need the
// initial state words 0..n and 397..396+n only (nextState's first loop).
// lo must hold n+1 words of scratch.
__device__ inline void first_reals(uint32_t seed, int n, uint32_t* lo, double* out, int stride) {
  uint32_t s = seed;
  lo[0] = s;
  for (int i = 1; i <= n; ++i) {
    s = 1812433253u * (s ^ (s >> 30)) + (uint32_t)i;
    lo[i] = s;
  }
  for (int i = n + 1; i < 397; ++i) s = 1812433253u * (s ^ (s >> 30)) + (uint32_t)i;
  for (int k = 0; k < n; ++k) {
    s = 1812433253u * (s ^ (s >> 30)) + (uint32_t)(397 + k);  // word 397 + k
    out[(long long)k * stride] = real(temper(s ^ twist(lo[k], lo[k + 1])));
  }
}

}  // namespace gbmt
