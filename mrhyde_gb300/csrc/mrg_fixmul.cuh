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
// Requires emax >= 60 (the result is then a normal number); the caller checks it once per row.  Branch-free
// apart from s = 0 (an earlier form with a separate exact branch for short sums measured 3 % slower in the
// Q1 row kernel, which rounds 13 sums a row).
__host__ __device__ __forceinline__ uint64_t fix_to_f64_bits(uint64_t s, int emax) {
  if (s == 0) return 0;
  // normalise: the leading one to bit 63 (s < 2^63, so z >= 1); the top 53 bits are the significand and
  // the 11 below it are rounded off (all zero when s has at most 53 significant bits)
  const int z = clz64(s);
  const uint64_t t = s << z;
  const uint64_t m = t >> 11;
  const uint32_t rem = (uint32_t)t & 0x7ffu;
  // nearest, ties to even; m + 1 = 2^53 carries into the exponent field
  const uint64_t up = (rem > 0x400u || (rem == 0x400u && (m & 1u))) ? 1u : 0u;
  // value = t 2^(emax - 1082 - z), t / 2^63 in [1, 2): biased exponent emax + 4 - z, field minus one
  return ((uint64_t)(emax + 3 - z) << 52) + m + up;
}

// RN(k * s) as an FP64 bit pattern (magnitude only) for two positive normal doubles given by their 53-bit
// significands (implicit bit set) mk, ms and the sum of their biased exponents: the exact 106-bit product
// from four 32 x 32-bit partial products, rounded once to nearest, ties to even -- the bits an FP64
// multiply returns.  Requires a normal result: 1 <= ek + es - 1023 (+1) <= 2046, checked by the caller.
__host__ __device__ __forceinline__ uint64_t mul_bits(uint64_t mk, uint64_t ms, int esum) {
  const uint64_t kl = mk & 0xffffffffull, kh = mk >> 32, sl = ms & 0xffffffffull, sh = ms >> 32;
  const uint64_t lo = kl * sl;
  const uint64_t mid = kl * sh + kh * sl;  // < 2^54
  const uint64_t plo = lo + (mid << 32);
  const uint64_t phi = kh * sh + (mid >> 32) + (plo < lo ? 1u : 0u);
  // product = phi 2^64 + plo in [2^104, 2^106); keep its top 53 bits
  const bool top = (phi >> 41) != 0;
  uint64_t m = top ? (phi << 11) | (plo >> 53) : (phi << 12) | (plo >> 52);
  const uint64_t rem = top ? (plo & ((1ull << 53) - 1)) : (plo & ((1ull << 52) - 1));
  const uint64_t half = top ? (1ull << 52) : (1ull << 51);
  m += (rem > half || (rem == half && (m & 1u))) ? 1u : 0u;
  // m in [2^52, 2^53]: adding it to (E - 1) << 52 sets the exponent field E (a carry to 2^53 moves into it)
  const uint64_t E = (uint64_t)(esum - 1023 + (top ? 1 : 0));
  return ((E - 1) << 52) + m;
}

// RN(x) as an FP32 bit pattern (nearest, ties to even) for an FP64 bit pattern b whose biased exponent
// lies in [897, 1150], i.e. whose magnitude is in [2^-126, 2^128): the 8-bit exponent is the FP64 one
// rebiased (1023 -> 127), the 23-bit significand its top 23 bits, and the 29 bits dropped round it, a
// carry into the exponent included (the largest values round to infinity as IEEE 754 prescribes).  About
// ten integer operations, where the FP64 -> FP32 conversion instruction issues at the FP64 rate.  Returns
// false for every other exponent (zero, subnormal, underflowing, overflowing, infinite or NaN input),
// which the caller converts with the conversion instruction.
__host__ __device__ __forceinline__ bool f64_to_f32_bits(uint64_t b, uint32_t& out) {
  const uint32_t hi = (uint32_t)(b >> 32), lo = (uint32_t)b;
  const uint32_t e = (hi >> 20) & 0x7ffu;
  if (e - 897u > 253u) return false;
  uint32_t f = (hi & 0x80000000u) | (((hi & 0x7fffffffu) - (896u << 20)) << 3) | (lo >> 29);
  // dropped bits rem < 2^29: round up iff rem > 2^28, or rem == 2^28 and f is odd
  f += ((lo & 0x1fffffffu) + (f & 1u) + 0x0fffffffu) >> 29;
  out = f;
  return true;
}

#ifdef __CUDACC__
__device__ __forceinline__ float f64_to_f32_rn(double x) {
  uint32_t f;
  if (f64_to_f32_bits((uint64_t)__double_as_longlong(x), f)) return __uint_as_float(f);
  return __double2float_rn(x);
}
#endif

}  // namespace mrgfix
