// Exact kappa sums on the integer pipes, for the factored Q1 assembly.
//
// GB300 issues FP64 arithmetic at 1/64 of the FP32 rate; an FP64 factored row costs 19 additions (the
// kappa sums S(off)), 27 products K(off) * S(off) and the residual's 27 FMAs.  The additions are done here
// on the integer pipes, exactly: the 8 conductivities around a node go to 64-bit fixed point with a
// per-row scale (kappa = m * 2^(e - 1075), m the 53-bit significand and e the biased exponent, becomes
// m << (7 - (emax - e))), exact whenever every nonzero kappa of the row lies within 2^7 of the row's
// largest (else the row takes the FP64 instructions); sums of up to 8 such values stay below 2^63 and are
// exact; each sum is then rounded once to FP64 (nearest, ties to even) by integer operations.  So S(off)
// is the correctly rounded exact sum, where FP64 additions round every partial sum.  (Forming the
// products exactly on the integer pipes as well -- a 117-bit product rounded once -- was measured: about
// 40 integer instructions per entry moved the bound to the integer pipes and gained 5 %.)
#pragma once
#include <cstdint>

namespace mrgfix {

__host__ __device__ __forceinline__ int clz64(uint64_t x) {
#ifdef __CUDA_ARCH__
  return __clzll((long long)x);
#else
  return x ? __builtin_clzll(x) : 64;
#endif
}

// RN(s * 2^(emax - 1082)) as an FP64 bit pattern, for a fixed-point kappa sum s < 2^63 (s = 0 gives +0).
// Requires emax >= 60 (the result is then a normal number); the caller checks it once per row.
__host__ __device__ __forceinline__ uint64_t fix_to_f64_bits(uint64_t s, int emax) {
  if (s == 0) return 0;
  const int L = 64 - clz64(s);                   // bit length, 1..63
  const uint64_t e1 = (uint64_t)(L + emax - 61);  // biased exponent of the result, minus one
  if (L <= 53) return (e1 << 52) + (s << (53 - L));
  const int sh = L - 53;                          // 1..10 bits below the significand
  // round to nearest, ties to even: add half an ulp minus one plus the kept lsb, then truncate; a carry
  // to 2^53 moves into the exponent field
  const uint64_t bias = (1ull << (sh - 1)) - 1u + ((s >> sh) & 1u);
  return (e1 << 52) + ((s + bias) >> sh);
}

}  // namespace mrgfix
