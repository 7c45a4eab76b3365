// Goldilocks field arithmetic for sm_103a: p = 2^64 - 2^32 + 1.
//
// Same field and the same canonical results as the reference's CPU field
// (crates/bignum/src/ntt.rs:159-284): every function returns a value in
// [0, p) when its inputs are in [0, p).  The reduction uses
// 2^64 = 2^32 - 1 (mod p) and 2^96 = -1 (mod p), computed with 32-bit
// IMAD / IADD carry chains in inline PTX.
#pragma once
#include <cstdint>

namespace gl {

constexpr uint64_t P = 0xFFFFFFFF00000001ull;
constexpr uint64_t EPS = 0xFFFFFFFFull;  // 2^64 mod p

__device__ __forceinline__ uint32_t lo32(uint64_t x) { return (uint32_t)x; }
__device__ __forceinline__ uint32_t hi32(uint64_t x) { return (uint32_t)(x >> 32); }
__device__ __forceinline__ uint64_t mk64(uint32_t lo, uint32_t hi) {
  return ((uint64_t)hi << 32) | lo;
}

// a + b mod p.
__device__ __forceinline__ uint64_t add(uint64_t a, uint64_t b) {
  uint64_t s = a + b;
  // overflow: the wrapped value lost 2^64 = EPS (mod p)
  s += (s < a) ? EPS : 0;
  return (s >= P) ? s - P : s;
}

// a - b mod p.
__device__ __forceinline__ uint64_t sub(uint64_t a, uint64_t b) {
  uint64_t d = a - b;
  // borrow: the wrapped value gained 2^64 = EPS (mod p)
  return (a < b) ? d - EPS : d;
}

__device__ __forceinline__ uint64_t neg(uint64_t a) { return a ? P - a : 0; }

// Reduce the 128-bit value (x3, x2, x1, x0) (32-bit words, little end first)
// mod p:  x = (x1:x0) + x2*2^64 + x3*2^96 = (x1:x0) + x2*(2^32-1) - x3.
__device__ __forceinline__ uint64_t reduce128(uint64_t lo, uint64_t hi) {
  uint32_t x2 = lo32(hi), x3 = hi32(hi);
  uint64_t t = lo - x3;
  t -= (lo < (uint64_t)x3) ? EPS : 0;  // borrow: +p == -EPS after the wrap
  uint64_t u = ((uint64_t)x2 << 32) - x2;  // x2 * (2^32 - 1) < p
  uint64_t r = t + u;
  r += (r < u) ? EPS : 0;
  return (r >= P) ? r - P : r;
}

// 64x64 -> 128 product from four 32x32 partial products.
__device__ __forceinline__ void mul128(uint64_t a, uint64_t b, uint64_t& lo, uint64_t& hi) {
  uint32_t r0, r1, r2, r3;
  uint32_t a0 = lo32(a), a1 = hi32(a), b0 = lo32(b), b1 = hi32(b);
  asm("{\n\t"
      "mul.lo.u32 %0, %4, %6;\n\t"
      "mul.hi.u32 %1, %4, %6;\n\t"
      "mul.lo.u32 %2, %5, %7;\n\t"
      "mul.hi.u32 %3, %5, %7;\n\t"
      "mad.lo.cc.u32 %1, %4, %7, %1;\n\t"
      "madc.hi.cc.u32 %2, %4, %7, %2;\n\t"
      "addc.u32 %3, %3, 0;\n\t"
      "mad.lo.cc.u32 %1, %5, %6, %1;\n\t"
      "madc.hi.cc.u32 %2, %5, %6, %2;\n\t"
      "addc.u32 %3, %3, 0;\n\t"
      "}"
      : "=&r"(r0), "=&r"(r1), "=&r"(r2), "=&r"(r3)
      : "r"(a0), "r"(a1), "r"(b0), "r"(b1));
  lo = mk64(r0, r1);
  hi = mk64(r2, r3);
}

// a * b mod p.
__device__ __forceinline__ uint64_t mul(uint64_t a, uint64_t b) {
  uint64_t lo, hi;
  mul128(a, b, lo, hi);
  return reduce128(lo, hi);
}

// x * 2^s mod p for 0 <= s < 192 (2 is a 192nd root of unity: 2^96 = -1).
__device__ __forceinline__ uint64_t shl(uint64_t x, int s) {
  bool negate = s >= 96;
  if (negate) s -= 96;
  uint64_t r;
  if (s == 0) {
    r = (x >= P) ? x - P : x;
  } else if (s < 64) {
    r = reduce128(x << s, x >> (64 - s));
  } else {
    // x * 2^s = (x << (s - 64)) * 2^64; with y = x << (s-64) as (yh:yl),
    // y*2^64 = yl*2^64 + yh*2^128, 2^64 = EPS and 2^128 = -2^32 (mod p).
    int t = s - 64;
    uint64_t yl = t ? (x << t) : x;
    uint64_t yh = t ? (x >> (64 - t)) : 0;  // < 2^32
    // yl * 2^64 as 128-bit (yl in the high word) reduces as yl * EPS:
    uint64_t a = reduce128(0, yl);
    // yh * 2^128 = -(yh * 2^32) (mod p); yh*2^32 < 2^64.
    uint64_t b = yh << 32;
    b = (b >= P) ? b - P : b;
    r = sub(a, b);
  }
  return negate ? neg(r) : r;
}

// base^e mod p.
__device__ __forceinline__ uint64_t pow(uint64_t base, uint64_t e) {
  uint64_t acc = 1;
  while (e) {
    if (e & 1) acc = mul(acc, base);
    e >>= 1;
    if (e) base = mul(base, base);
  }
  return acc;
}

}  // namespace gl
