// Exact slicing helpers shared by the tensor-core kernels (M update, exp): power-of-two
// scales, signed 7- and 8-bit digits as FP16 (BF16 for the exp's 65..128-wide form),
// tcgen05 descriptors, exact int64 recombination.  See k_tensor.cu for the scheme.
#pragma once
#include <cuda_bf16.h>

#include "w90g.cuh"

namespace w90g {
namespace {

constexpr int kS = 7;            // digits per operand
constexpr int kDiag = kS;        // diagonals d = 2 .. S+1
constexpr int kTileRows = 128;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// shared-memory matrix descriptor: canonical K-major layout, no swizzle
//   start address, LBO = byte stride between core matrices along K,
//   SBO = byte stride between 8-row groups, version 1 (bit 46), layout 0
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFF);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// instruction descriptor, kind::f16: D = F32, A = B = BF16, both K-major, N, M = 128
// (one MMA never mixes BF16 and FP16 operands)
__host__ __device__ constexpr uint32_t idesc_bf16(int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(kTileRows >> 4) << 24);
}

// the same with A = B = F16 (the FP16 digit planes of the M update and of the exp's
// second product form)
__host__ __device__ constexpr uint32_t idesc_f16(int N) {
  return (1u << 4) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(kTileRows >> 4) << 24);
}

// element (row, k) of a K-major tile with K_real columns, in bytes
__device__ __forceinline__ uint32_t kmaj_off(int row, int k, int kreal) {
  return (uint32_t)((row >> 3) * (kreal >> 3) * 128 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

// exact BF16 bits of a small integer (|x| < 2^22): 1.5*2^23 magic, top 16 bits
__device__ __forceinline__ uint16_t int_to_bf16(int x) {
  const float f = __int_as_float(0x4B400000 + x) - 12582912.0f;
  return (uint16_t)(__float_as_uint(f) >> 16);
}

// exact integer value of an integer-valued float with |f| < 2^22
__device__ __forceinline__ int float_to_int_exact(float f) {
  return __float_as_int(f + 12582912.0f) - 0x4B400000;
}

// |v| as an ordered integer (non-negative doubles compare like their bit patterns)
__device__ __forceinline__ unsigned long long abs_bits(double v) {
  return (unsigned long long)__double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFull;
}

// exponent e with |v| < 2^e from the bits of |v| (0 for v == 0); integer ops only
__device__ __forceinline__ int exp_above_bits(unsigned long long ab) {
  return ab ? (int)(ab >> 52) - 1022 : 0;
}

// N = round(v * 2^(49 - e)) as a signed integer (|N| <= 2^49), integer ops only
__device__ __forceinline__ long long scaled_int(double v, int e) {
  const long long bits = __double_as_longlong(v);
  const int be = (int)((bits >> 52) & 0x7FF);
  if (be == 0) return 0;   // zero / subnormal
  const long long mant = (bits & 0x000FFFFFFFFFFFFFLL) | 0x0010000000000000LL;
  // v = mant * 2^(be - 1075);  v * 2^(49-e) = mant * 2^(be - 1026 - e)
  const int sh = 1026 + e - be;    // right shift >= 3 since |v| < 2^e
  long long n;
  if (sh >= 62) n = 0;
  else n = (mant + (1LL << (sh - 1))) >> sh;
  return (bits < 0) ? -n : n;
}

// signed 7-bit digits of N (|N| <= 2^49), extracted from the bottom:
// x_7..x_2 in [-64, 63], x_1 the remaining top part (|x_1| <= 128); N = sum_t x_t 2^(7(7-t))
__device__ __forceinline__ void digits7(long long n, int x[kS]) {
#pragma unroll
  for (int t = kS - 1; t > 0; --t) {
    const int lo = (int)n & 127;
    const int d = lo - ((lo & 64) << 1);     // centred in [-64, 63]
    x[t] = d;
    n = (n - d) >> 7;
  }
  x[0] = (int)n;
}

// 8-digit form (56 bits, used by the exp kernel): N = round(v * 2^(56 - e)), |N| <= 2^56
__device__ __forceinline__ long long scaled_int56(double v, int e) {
  const long long bits = __double_as_longlong(v);
  const int be = (int)((bits >> 52) & 0x7FF);
  if (be == 0) return 0;
  const long long mant = (bits & 0x000FFFFFFFFFFFFFLL) | 0x0010000000000000LL;
  // v * 2^(56-e) = mant * 2^(be - 1019 - e); the right shift is >= -3 since |v| < 2^e
  const int sh = 1019 + e - be;
  long long n;
  if (sh >= 62) n = 0;
  else if (sh > 0) n = (mant + (1LL << (sh - 1))) >> sh;
  else n = mant << (-sh);
  return (bits < 0) ? -n : n;
}

// 8 signed 7-bit digits of N (|N| <= 2^56): x_8..x_2 in [-64, 63], |x_1| <= 128,
// N = sum_t x_t 2^(7(8-t))
__device__ __forceinline__ void digits8(long long n, int x[8]) {
#pragma unroll
  for (int t = 7; t > 0; --t) {
    const int lo = (int)n & 127;
    const int d = lo - ((lo & 64) << 1);
    x[t] = d;
    n = (n - d) >> 7;
  }
  x[0] = (int)n;
}

// 8-bit-digit form (56 bits in 7 digits): N = round(v * 2^(55 - e)), |N| <= 2^55
__device__ __forceinline__ long long scaled_int55(double v, int e) {
  const long long bits = __double_as_longlong(v);
  const int be = (int)((bits >> 52) & 0x7FF);
  if (be == 0) return 0;
  const long long mant = (bits & 0x000FFFFFFFFFFFFFLL) | 0x0010000000000000LL;
  // v * 2^(55-e) = mant * 2^(be - 1020 - e); the right shift is >= -2 since |v| < 2^e
  const int sh = 1020 + e - be;
  long long n;
  if (sh >= 62) n = 0;
  else if (sh > 0) n = (mant + (1LL << (sh - 1))) >> sh;
  else n = mant << (-sh);
  return (bits < 0) ? -n : n;
}

// 7 signed 8-bit digits of N (|N| <= 2^55): x_7..x_2 in [-128, 127], |x_1| <= 128,
// N = sum_t x_t 2^(8(7-t)); every digit is an exact BF16 value
__device__ __forceinline__ void digits7x8(long long n, int x[7]) {
#pragma unroll
  for (int t = 6; t > 0; --t) {
    const int lo = (int)n & 255;
    const int d = lo - ((lo & 128) << 1);
    x[t] = d;
    n = (n - d) >> 8;
  }
  x[0] = (int)n;
}

// x - c for both halves of a packed FP16 pair (c packed likewise)
__device__ __forceinline__ uint32_t f16x2_sub(uint32_t x, uint32_t c) {
  uint32_t r;
  asm("sub.rn.f16x2 %0, %1, %2;" : "=r"(r) : "r"(x), "r"(c));
  return r;
}

// FP16 bits of a small integer (|x| <= 2048: exact)
__device__ __forceinline__ uint16_t int_to_f16(int x) {
  uint16_t r;
  asm("cvt.rn.f16.s32 %0, %1;" : "=h"(r) : "r"(x));
  return r;
}

// The seven 7-bit digit planes of 8 values scaled by 2^(49 - ex) (negated first when neg),
// as packed FP16 pairs: w[t][i / 2] holds digit t of values i (low half) and i + 1 -- the
// digits of digits7, without its serial recoding.  With C = 64 (1 + 2^7 + ... + 2^35), bits
// 7t'..7t'+6 of N + C are digit 6 - t' plus 64 (adding 64 at every lower digit position
// turns the centred digits into the plain 7-bit fields of N + C), and the top digit is
// (N + C) >> 42 (arithmetic), in [-128, 128].  Two values' 14-bit windows side by side in
// one word (one byte permute) give two fields of both per mask; with 0x6400 above it a
// field b is the FP16 number 1024 + b, so one packed subtraction of 1088 (top digit: of
// 1152, after adding 128) leaves the digits.  Exact: FP16 holds the integers to 2048, and
// the difference of two of them is rounded to itself.
__device__ __forceinline__ void pack_digits7(uint32_t (&w)[kS][4], const double (&v)[8], int ex, bool neg) {
#pragma unroll
  for (int i = 0; i < 8; i += 2) {
    const long long ma = scaled_int(neg ? -v[i] : v[i], ex) + 0x20408102040LL;
    const long long mb = scaled_int(neg ? -v[i + 1] : v[i + 1], ex) + 0x20408102040LL;
    const uint32_t la = (uint32_t)ma, lb = (uint32_t)mb;
    const uint32_t ha = (uint32_t)((unsigned long long)ma >> 32), hb = (uint32_t)((unsigned long long)mb >> 32);
    // bits 0-13, 14-27 and 28-41 of a (low half) and b (high half)
    const uint32_t q[3] = {__byte_perm(la, lb, 0x5410), __byte_perm(la >> 14, lb >> 14, 0x5410),
                           __byte_perm(__funnelshift_r(la, ha, 28), __funnelshift_r(lb, hb, 28), 0x5410)};
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      w[6 - 2 * j][i >> 1] = f16x2_sub((q[j] & 0x007F007Fu) | 0x64006400u, 0x64406440u);
      w[5 - 2 * j][i >> 1] = f16x2_sub(((q[j] >> 7) & 0x007F007Fu) | 0x64006400u, 0x64406440u);
    }
    const uint32_t ta = (uint32_t)((int)(ma >> 42) + 128), tb = (uint32_t)((int)(mb >> 42) + 128);
    w[0][i >> 1] = f16x2_sub(ta | (tb << 16) | 0x64006400u, 0x64806480u);
  }
}

// exact integer value of an integer-valued float with |f| < 2^24
__device__ __forceinline__ int float_to_int_exact24(float f) {
  return (fabsf(f) < 4194304.0f) ? float_to_int_exact(f) : __float2int_rn(f);
}

// double of S * 2^sc for a 128-bit S, rounded to nearest even, integer ops only
__device__ __forceinline__ double int128_scaled_to_double(__int128 S, int sc) {
  if (S == 0) return 0.0;
  const unsigned long long sign = (S < 0) ? 0x8000000000000000ull : 0ull;
  unsigned __int128 a = (S < 0) ? (unsigned __int128)(-S) : (unsigned __int128)S;
  const unsigned long long hi = (unsigned long long)(a >> 64), lo = (unsigned long long)a;
  const int lz = hi ? __clzll(hi) : 64 + __clzll(lo);
  a <<= lz;                                          // leading 1 at bit 127
  const unsigned long long top = (unsigned long long)(a >> 64);
  const bool sticky = (unsigned long long)a != 0ull;
  unsigned long long m = top >> 11;                  // 53 bits
  const unsigned long long rem = top & 0x7FFull;
  if (rem > 0x400ull || (rem == 0x400ull && (sticky || (m & 1ull)))) m += 1ull;
  int ex = 127 - lz + sc;
  if (m >> 53) {
    m >>= 1;
    ex += 1;
  }
  const unsigned long long bits = sign | ((unsigned long long)(ex + 1023) << 52) | (m & 0x000FFFFFFFFFFFFFull);
  return __longlong_as_double((long long)bits);
}

// exact double of S * 2^sc (|S| < 2^63) with integer ops only (round to nearest even)
__device__ __forceinline__ double int64_scaled_to_double(long long S, int sc) {
  if (S == 0) return 0.0;
  const unsigned long long sign = (S < 0) ? 0x8000000000000000ull : 0ull;
  unsigned long long a = (S < 0) ? (unsigned long long)(-S) : (unsigned long long)S;
  const int lz = __clzll(a);
  a <<= lz;                                   // leading 1 at bit 63
  // keep 53 bits: round to nearest even on the 11 dropped bits
  unsigned long long m = a >> 11;
  const unsigned long long rem = a & 0x7FFull;
  if (rem > 0x400ull || (rem == 0x400ull && (m & 1ull))) m += 1ull;
  int ex = 63 - lz + sc;                      // value = m * 2^(ex - 52)
  if (m >> 53) {                              // rounding carried into a new bit
    m >>= 1;
    ex += 1;
  }
  const unsigned long long bits = sign | ((unsigned long long)(ex + 1023) << 52) | (m & 0x000FFFFFFFFFFFFFull);
  return __longlong_as_double((long long)bits);
}

// sum_d D_d 2^(8(6-d)) * 2^sc for the 7 diagonal accumulators of the 8-bit-digit scheme
// (|D_d| < 2^24): the top four and the bottom three diagonals are combined exactly in
// int64 (< 2^49 and < 2^41), converted exactly, and added once in FP64 (one rounding).
// (Rounding their exact int128 sum with integer ops gives the same bits but measured
// slower.)
__device__ __forceinline__ double recombine7x8(const uint32_t* dd, int stride, int sc) {
  long long hi = float_to_int_exact24(__uint_as_float(dd[0]));
#pragma unroll
  for (int d = 1; d < 4; ++d) hi = (hi << 8) + float_to_int_exact24(__uint_as_float(dd[d * stride]));
  long long lo = float_to_int_exact24(__uint_as_float(dd[4 * stride]));
#pragma unroll
  for (int d = 5; d < 7; ++d) lo = (lo << 8) + float_to_int_exact24(__uint_as_float(dd[d * stride]));
  return int64_scaled_to_double(hi, sc + 24) + int64_scaled_to_double(lo, sc);
}

// Spin limits of the mbarrier waits.  A wait that runs out of W90G_SPIN_LIMIT tries makes
// the kernel record an error; before it leaves, the kernel waits again (up to
// W90G_DRAIN_LIMIT tries) for the asynchronous work it has issued -- MMAs tracked by a
// commit, bulk copies tracked by a transaction count -- so that no MMA or copy still
// writes shared or tensor memory that the CTA gives back.  A test build sets a tiny
// W90G_SPIN_LIMIT to drive that path.
#ifndef W90G_SPIN_LIMIT
#define W90G_SPIN_LIMIT (1 << 20)
#endif
#ifndef W90G_DRAIN_LIMIT
#define W90G_DRAIN_LIMIT (1 << 22)
#endif

__device__ __forceinline__ bool mbar_try(uint32_t addr, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(addr), "r"(parity)
      : "memory");
  return ok != 0;
}

// the drain after a timed-out wait: the same phase, the long limit
__device__ __forceinline__ bool mbar_drain(uint32_t addr, uint32_t parity) {
  for (int it = 0; it < W90G_DRAIN_LIMIT; ++it)
    if (mbar_try(addr, parity)) return true;
  return false;
}

__device__ __forceinline__ bool mbar_wait(uint32_t addr, uint32_t parity) {
  for (int it = 0; it < W90G_SPIN_LIMIT; ++it)
    if (mbar_try(addr, parity)) return true;
  return false;
}

// Tile geometry.  Complex dimensions are processed in chunks of CW = min(WP, 32) complex
// indices; a chunk's real index l < CW is the real part of complex index chunk*CW + l and
// l >= CW its imaginary part.  KC = NC = 2*CW real entries per chunk, NCH chunks along K
// and along N (W up to 128).  Shared memory holds the S digit slices of one A chunk
// (128 x KC) and one B chunk (NC x KC); TMEM holds the S diagonals of one N chunk.
template <int WP>
struct TileSmem {
  static constexpr int CW = WP < 32 ? WP : 32;
  static constexpr int KC = 2 * CW;
  static constexpr int NC = 2 * CW;
  static constexpr int NCH = WP / CW;
  static constexpr int A_BYTES = kTileRows * KC * 2;
  static constexpr int B_BYTES = NC * KC * 2;
  static constexpr int TMEM_COLS = (kDiag * NC <= 128) ? 128 : ((kDiag * NC <= 256) ? 256 : 512);
  static constexpr size_t BYTES = (size_t)kS * (A_BYTES + B_BYTES) + 1024;
};

}  // namespace

}  // namespace w90g
