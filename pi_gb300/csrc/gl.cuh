// Goldilocks field arithmetic for sm_103a: p = 2^64 - 2^32 + 1.
//
// Same field as the reference's CPU code (crates/bignum/src/ntt.rs:159-284).
// Inside the transforms values are kept "weak": any 64-bit word congruent to
// the field element (so possibly in [p, 2^64)).  add / sub / mul accept weak
// inputs and return weak outputs; canon() gives the canonical representative
// in [0, p), which is what leaves the engine.  The reduction uses
// 2^64 = 2^32 - 1 (mod p) and 2^96 = -1 (mod p), written as 32-bit carry
// chains in inline PTX (the integer ALU pipe is the binding resource).
#pragma once
#include <cstdint>

namespace gl {

constexpr uint64_t P = 0xFFFFFFFF00000001ull;
constexpr uint64_t EPS = 0xFFFFFFFFull;  // 2^64 mod p

__device__ __forceinline__ uint32_t lo32(uint64_t x) { return (uint32_t)x; }
__device__ __forceinline__ uint32_t hi32(uint64_t x) { return (uint32_t)(x >> 32); }
__device__ __forceinline__ uint64_t mk64(uint32_t lo, uint32_t hi) { return ((uint64_t)hi << 32) | lo; }

// a + b (weak in, weak out).  A carry out of 64 bits is worth 2^64 = EPS;
// adding EPS back can carry once more (only when both inputs are >= p-ish),
// and that second carry is folded the same way.
__device__ __forceinline__ uint64_t add(uint64_t a, uint64_t b) {
  uint32_t z0, z1;
  asm("{\n\t.reg .u32 c, m;\n\t"
      "add.cc.u32 %0, %2, %4;\n\t"
      "addc.cc.u32 %1, %3, %5;\n\t"
      "addc.u32 c, 0, 0;\n\t"
      "neg.s32 m, c;\n\t"
      "add.cc.u32 %0, %0, m;\n\t"
      "addc.cc.u32 %1, %1, 0;\n\t"
      "addc.u32 c, 0, 0;\n\t"
      "neg.s32 m, c;\n\t"
      "add.cc.u32 %0, %0, m;\n\t"
      "addc.u32 %1, %1, 0;\n\t"
      "}"
      : "=&r"(z0), "=&r"(z1)
      : "r"(lo32(a)), "r"(hi32(a)), "r"(lo32(b)), "r"(hi32(b)));
  return mk64(z0, z1);
}

// a - b (weak in, weak out).  A borrow is worth -2^64 = -EPS; subtracting
// EPS can borrow once more, folded the same way.
__device__ __forceinline__ uint64_t sub(uint64_t a, uint64_t b) {
  uint32_t z0, z1;
  asm("{\n\t.reg .u32 m;\n\t"
      "sub.cc.u32 %0, %2, %4;\n\t"
      "subc.cc.u32 %1, %3, %5;\n\t"
      "subc.u32 m, 0, 0;\n\t"
      "sub.cc.u32 %0, %0, m;\n\t"
      "subc.cc.u32 %1, %1, 0;\n\t"
      "subc.u32 m, 0, 0;\n\t"
      "sub.cc.u32 %0, %0, m;\n\t"
      "subc.u32 %1, %1, 0;\n\t"
      "}"
      : "=&r"(z0), "=&r"(z1)
      : "r"(lo32(a)), "r"(hi32(a)), "r"(lo32(b)), "r"(hi32(b)));
  return mk64(z0, z1);
}

// Canonical representative in [0, p).
__device__ __forceinline__ uint64_t canon(uint64_t x) { return x >= P ? x - P : x; }

__device__ __forceinline__ uint64_t neg(uint64_t a) { return sub(0, a); }

// 128-bit value (x3 x2 x1 x0) -> weak 64-bit:  (x1:x0) - x3 + x2 * (2^32 - 1).
__device__ __forceinline__ uint64_t reduce_words(uint32_t r0, uint32_t r1, uint32_t r2, uint32_t r3) {
  uint32_t z0, z1;
  asm("{\n\t.reg .u32 t0, t1, b, u0, u1, c;\n\t"
      "sub.cc.u32 t0, %2, %5;\n\t"      // t = (x1:x0) - x3
      "subc.cc.u32 t1, %3, 0;\n\t"
      "subc.u32 b, 0, 0;\n\t"           // borrow mask: -2^64 = -EPS
      "sub.cc.u32 t0, t0, b;\n\t"       // cannot borrow again
      "subc.u32 t1, t1, 0;\n\t"
      "sub.cc.u32 u0, 0, %4;\n\t"       // u = x2 * (2^32 - 1)
      "subc.u32 u1, %4, 0;\n\t"
      "add.cc.u32 t0, t0, u0;\n\t"      // t + u
      "addc.cc.u32 t1, t1, u1;\n\t"
      "addc.u32 c, 0, 0;\n\t"
      "neg.s32 c, c;\n\t"               // carry: +2^64 = +EPS (cannot carry again)
      "add.cc.u32 %0, t0, c;\n\t"
      "addc.u32 %1, t1, 0;\n\t"
      "}"
      : "=r"(z0), "=r"(z1)
      : "r"(r0), "r"(r1), "r"(r2), "r"(r3));
  return mk64(z0, z1);
}

__device__ __forceinline__ uint64_t reduce128(uint64_t lo, uint64_t hi) {
  return reduce_words(lo32(lo), hi32(lo), lo32(hi), hi32(hi));
}

// 64x64 -> 128 product from four 32x32 partial products.
__device__ __forceinline__ void mul128(uint64_t a, uint64_t b, uint32_t& r0, uint32_t& r1, uint32_t& r2,
                                       uint32_t& r3) {
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
      : "r"(lo32(a)), "r"(hi32(a)), "r"(lo32(b)), "r"(hi32(b)));
}

// a * b mod p (weak in, weak out).
__device__ __forceinline__ uint64_t mul(uint64_t a, uint64_t b) {
  uint32_t r0, r1, r2, r3;
  mul128(a, b, r0, r1, r2, r3);
  return reduce_words(r0, r1, r2, r3);
}

// x * 2^s mod p for a compile-time 0 <= s < 192 (2^96 = -1, 2^192 = 1).
template <int S>
__device__ __forceinline__ uint64_t shl(uint64_t x) {
  static_assert(S >= 0 && S < 192, "shift out of range");
  if constexpr (S >= 96) {
    return neg(shl<S - 96>(x));
  } else if constexpr (S == 0) {
    return x;
  } else if constexpr (S < 64) {
    uint64_t lo = x << S, hi = x >> (64 - S);
    return reduce128(lo, hi);
  } else {
    // x * 2^S = (x << (S-64)) * 2^64; with y = x << (S-64) = (yh:yl),
    // y * 2^64 = yl * 2^64 + yh * 2^128 and 2^128 = -2^32 (mod p).
    constexpr int T = S - 64;
    uint64_t yl = T ? (x << T) : x;
    uint64_t yh = T ? (x >> (64 - T)) : 0;  // < 2^32
    return sub(reduce128(0, yl), yh << 32);
  }
}

// base^e mod p (canonical result).
__device__ __forceinline__ uint64_t pow(uint64_t base, uint64_t e) {
  uint64_t acc = 1;
  while (e) {
    if (e & 1) acc = mul(acc, base);
    e >>= 1;
    if (e) base = mul(base, base);
  }
  return canon(acc);
}

}  // namespace gl
