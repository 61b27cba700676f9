"""Host check of the integer-pipe FP64 helpers of the Q1 assembly (mrhyde_gb300/csrc/mrg_fixmul.cuh), which
must return exactly the bits of the FP64 operations they replace:

* fix_to_f64_bits(s, emax): a 64-bit fixed-point kappa sum rounded once to FP64 (nearest, ties to even),
  against the exact value s * 2^(emax - 1082) held in a long double (64-bit or wider significand) and
  rounded by the conversion to double;
* mul_bits(mk, ms, ek + es): the product of two normal doubles, against the IEEE multiply;
* f64_to_f32_bits(b): an FP64 value rounded to FP32 (nearest, ties to even), against the host's
  conversion, over FP32's whole normal range, ties, carries into the exponent and overflow to infinity,
  and declining (for the conversion instruction) exactly outside that range.

The header's device functions compile as plain C++ here; the checker is built with the host compiler and
runs a few million random and structured cases in about a second.
"""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "mrhyde_gb300", "csrc")

CHECKER = r"""
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <cmath>
#include <random>
#define __host__
#define __device__
#define __forceinline__ inline
#include "mrg_fixmul.cuh"

static uint64_t bits(double d) { uint64_t u; std::memcpy(&u, &d, 8); return u; }
static double dbl(uint64_t u) { double d; std::memcpy(&d, &u, 8); return d; }

int main() {
  std::mt19937_64 g(2024);
  long bad = 0, tot = 0;
  // ---- fix_to_f64_bits: sums of up to 8 significands shifted by up to 7 bits (s < 2^63), any emax
  for (long i = 0; i < 2000000; ++i) {
    const int terms = 1 + (int)(g() % 8);
    uint64_t s = 0;
    for (int t = 0; t < terms; ++t) s += ((g() & 0xfffffffffffffull) | (1ull << 52)) << (g() % 8);
    if (g() % 16 == 0) s >>= (g() % 60);  // short sums too
    const int emax = 60 + (int)(g() % 1983);
    const long double exact = std::ldexp((long double)s, emax - 1082);
    const double want = (double)exact;
    if (!(want > 0.0) || std::isinf(want) || bits(want) < (1ull << 52)) continue;  // normal results only
    ++tot;
    if (mrgfix::fix_to_f64_bits(s, emax) != bits(want)) {
      if (bad < 5) std::printf("fix: s=%llu emax=%d\n", (unsigned long long)s, emax);
      ++bad;
    }
  }
  // ---- mul_bits
  auto mul = [&](uint64_t a, uint64_t b) {
    const int ea = (int)(a >> 52), eb = (int)(b >> 52);
    const int E = ea + eb - 1023;
    if (E < 2 || E > 2044) return;  // the callers' range
    const uint64_t ma = (a & 0xfffffffffffffull) | (1ull << 52), mb = (b & 0xfffffffffffffull) | (1ull << 52);
    ++tot;
    if (mrgfix::mul_bits(ma, mb, ea + eb) != bits(dbl(a) * dbl(b))) {
      if (bad < 5) std::printf("mul: %a * %a\n", dbl(a), dbl(b));
      ++bad;
    }
  };
  for (long i = 0; i < 3000000; ++i)
    mul(((uint64_t)(1 + g() % 2046) << 52) | (g() & 0xfffffffffffffull),
        ((uint64_t)(1 + g() % 2046) << 52) | (g() & 0xfffffffffffffull));
  const uint64_t pats[] = {0, 1, 2, 3, 0xfffffffffffffull, 0x8000000000000ull, 0x8000000000001ull,
                           0x7ffffffffffffull, 0xffffffffull, 0x100000000ull, 0xfffff00000000ull,
                           0x5555555555555ull, 0xaaaaaaaaaaaaaull, 0xfffull};
  for (uint64_t pa : pats)
    for (uint64_t pb : pats)
      for (int ea = 900; ea < 1150; ea += 7)
        for (int eb = 900; eb < 1150; eb += 11) mul(((uint64_t)ea << 52) | pa, ((uint64_t)eb << 52) | pb);
  for (long i = 0; i < 1000000; ++i)  // 2- and 3-bit significands: exact products and ties
    mul((1023ull << 52) | (g() & 0xfffffffffffffull), (1023ull << 52) | ((g() & 0x3ull) << 50));
  // ---- f64_to_f32_bits
  auto cvt = [&](uint64_t b) {
    const int e = (int)((b >> 52) & 0x7ff);
    uint32_t f = 0;
    const bool ok = mrgfix::f64_to_f32_bits(b, f);
    ++tot;
    if (ok != (e >= 897 && e <= 1150)) {
      if (bad < 5) std::printf("cvt range: %a\n", dbl(b));
      ++bad;
      return;
    }
    if (!ok) return;
    const float want = (float)dbl(b);
    uint32_t wb;
    std::memcpy(&wb, &want, 4);
    if (f != wb) {
      if (bad < 5) std::printf("cvt: %a -> %08x want %08x\n", dbl(b), f, wb);
      ++bad;
    }
  };
  for (long i = 0; i < 3000000; ++i)
    cvt(((g() & 1) << 63) | ((uint64_t)(880 + g() % 290) << 52) | (g() & 0xfffffffffffffull));
  // the 29 dropped bits at and around the tie, odd and even kept significands, all-ones carries
  const uint64_t low[] = {0, 1, 0x0fffffff, 0x10000000, 0x10000001, 0x1fffffff, 0x30000000, 0x20000000};
  for (int e = 890; e <= 1160; ++e)
    for (uint64_t lw : low)
      for (uint64_t top : {0ull, 1ull, 2ull, 3ull, 0x7ffffeull, 0x7fffffull, 0x400000ull})
        for (uint64_t sgn : {0ull, 1ull}) cvt((sgn << 63) | ((uint64_t)e << 52) | (top << 29) | lw);
  std::printf("%ld %ld\n", tot, bad);
  return bad != 0;
}
"""


def test_integer_fp64_helpers_match_fp64_operations(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    src = tmp_path / "fixmul_check.cpp"
    exe = tmp_path / "fixmul_check"
    src.write_text(CHECKER)
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", CSRC, str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    tot, bad = map(int, out.stdout.split()[-2:])
    assert out.returncode == 0 and bad == 0, out.stdout
    assert tot > 7_000_000
