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

// 128-bit value (x3 x2 x1 x0) -> weak 64-bit:  (x1:x0) + x2 * (2^32 - 1) - x3.
// u = x2 * (2^32 - 1) comes from one wide multiply; the sum's net carry
// k in {-1, 0, 1} is worth k * 2^64 = k * EPS, and adding that cannot carry
// again (|k * EPS| is far from both ends of the 64-bit range).
__device__ __forceinline__ uint64_t reduce_words(uint32_t r0, uint32_t r1, uint32_t r2, uint32_t r3) {
  uint64_t u;
  asm("mul.wide.u32 %0, %1, 0xFFFFFFFF;" : "=l"(u) : "r"(r2));
  uint32_t z0, z1;
  asm("{\n\t.reg .u32 k, nk, hk, u0, u1;\n\t"
      "mov.b64 {u0, u1}, %6;\n\t"
      "add.cc.u32 %0, %2, u0;\n\t"
      "addc.cc.u32 %1, %3, u1;\n\t"
      "addc.u32 k, 0, 0;\n\t"
      "sub.cc.u32 %0, %0, %5;\n\t"
      "subc.cc.u32 %1, %1, 0;\n\t"
      "subc.u32 k, k, 0;\n\t"
      "neg.s32 nk, k;\n\t"           // k * EPS = (k >> 31 : -k) for k in {-1, 0, 1}
      "shr.s32 hk, k, 31;\n\t"
      "add.cc.u32 %0, %0, nk;\n\t"
      "addc.u32 %1, %1, hk;\n\t"
      "}"
      : "=&r"(z0), "=&r"(z1)
      : "r"(r0), "r"(r1), "r"(r2), "r"(r3), "l"(u));
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

// ------------------------------------------------------------ lazy values
// Inside the radix-8 / radix-4 butterflies values are carried "lazy": a
// 64-bit word plus a small signed count k of 2^64 overflows,
//   value = l + h 2^32 + k 2^64   (= l + h 2^32 + k EPS  mod p).
// Adding or subtracting two lazy values is one 96-bit add (three carry-chain
// instructions) with no modular fix-up; fold() turns a lazy value back into a
// weak 64-bit word once, at the end of the butterfly network.
struct Lz {
  uint32_t l, h;
  int32_t k;
};

__device__ __forceinline__ Lz lz(uint64_t x) { return Lz{lo32(x), hi32(x), 0}; }

__device__ __forceinline__ Lz lz_add(Lz x, Lz y) {
  Lz z;
  asm("add.cc.u32 %0, %3, %6;\n\taddc.cc.u32 %1, %4, %7;\n\taddc.u32 %2, %5, %8;"
      : "=r"(z.l), "=r"(z.h), "=r"(z.k)
      : "r"(x.l), "r"(x.h), "r"(x.k), "r"(y.l), "r"(y.h), "r"(y.k));
  return z;
}

__device__ __forceinline__ Lz lz_sub(Lz x, Lz y) {
  Lz z;
  asm("sub.cc.u32 %0, %3, %6;\n\tsubc.cc.u32 %1, %4, %7;\n\tsubc.u32 %2, %5, %8;"
      : "=r"(z.l), "=r"(z.h), "=r"(z.k)
      : "r"(x.l), "r"(x.h), "r"(x.k), "r"(y.l), "r"(y.h), "r"(y.k));
  return z;
}

// (h:l) + w * EPS for a signed |w| < 2^31 -> weak 64-bit.  As a 96-bit
// signed sum, (h:l) - w + w 2^32 has top word c in {-1, 0, 1}; c * EPS is
// added back as in reduce_words.
__device__ __forceinline__ uint64_t fold_words(uint32_t l, uint32_t h, int32_t w) {
  uint32_t z0, z1;
  asm("{\n\t.reg .u32 wh, c, nc, hc;\n\t"
      "shr.s32 wh, %4, 31;\n\t"
      "sub.cc.u32 %0, %2, %4;\n\t"
      "subc.cc.u32 %1, %3, wh;\n\t"
      "subc.u32 c, 0, wh;\n\t"
      "add.cc.u32 %1, %1, %4;\n\t"
      "addc.u32 c, c, wh;\n\t"
      "neg.s32 nc, c;\n\t"
      "shr.s32 hc, c, 31;\n\t"
      "add.cc.u32 %0, %0, nc;\n\t"
      "addc.u32 %1, %1, hc;\n\t"
      "}"
      : "=&r"(z0), "=&r"(z1)
      : "r"(l), "r"(h), "r"(w));
  return mk64(z0, z1);
}

__device__ __forceinline__ uint64_t fold(Lz x) { return fold_words(x.l, x.h, x.k); }

// a * b as a lazy value with k in {-1, 0}: with u = x2 EPS + (EPS - x3)
// (which cannot overflow 64 bits), a b = (x1:x0) + u - EPS and -EPS = -2^64.
__device__ __forceinline__ Lz lz_mul(uint64_t a, uint64_t b) {
  uint32_t r0, r1, r2, r3;
  mul128(a, b, r0, r1, r2, r3);
  uint64_t u;
  asm("mad.wide.u32 %0, %1, 0xFFFFFFFF, %2;" : "=l"(u) : "r"(r2), "l"((uint64_t)(~r3)));
  Lz z;
  asm("add.cc.u32 %0, %3, %5;\n\taddc.cc.u32 %1, %4, %6;\n\taddc.u32 %2, 0xFFFFFFFF, 0;"
      : "=r"(z.l), "=r"(z.h), "=r"(z.k)
      : "r"(r0), "r"(r1), "r"(lo32(u)), "r"(hi32(u)));
  return z;
}

// Shifts that leave their result lazy (no fold), for the radix-8 / radix-4
// butterflies.  Derivations, with x = l + h 2^32 + k 2^64:
//  * x 2^24 = (l << 24) + funnel(l, h, 24) 2^32 + ((h >> 8) + k 2^24) 2^64: the
//    overflow count grows to |k| < 2^28 (|x.k| < 2^6 in), which lz_add,
//    lz_sub and fold accept but another shift does not;
//  * x 2^48 = w1 2^32 + w2 2^64 + w3 2^96 with w1 = l << 16, w2 = funnel(l, h, 16),
//    w3 = (h >> 16) + k 2^16; with 2^64 = 2^32 - 1 and 2^96 = -1 this is
//    w2 EPS + w1 2^32 - w3, a 96-bit value with k in {-1 .. 2} (|x.k| < 2^15 in);
//  * x 2^72 = y 2^64 for y = x 2^8 = y0 + y1 2^32 + y2 2^64 (y0 = l << 8,
//    y1 = funnel(l, h, 8), y2 = (h >> 24) + k 2^8); with 2^128 = -2^32 this is
//    y0 EPS - y1 - y2 2^32, k in {-1 .. 1} (|x.k| < 2^23 in).
__device__ __forceinline__ Lz lz_shl24_wide(Lz x) {
  Lz z;
  z.l = x.l << 24;
  z.h = __funnelshift_l(x.l, x.h, 24);
  z.k = (int32_t)(x.h >> 8) + (int32_t)((uint32_t)x.k << 24);
  return z;
}

__device__ __forceinline__ Lz lz_shl48_n(Lz x) {
  const uint32_t w1 = x.l << 16, w2 = __funnelshift_l(x.l, x.h, 16);
  const int32_t w3 = (int32_t)(x.h >> 16) + (int32_t)((uint32_t)x.k << 16);
  uint64_t u;
  asm("mul.wide.u32 %0, %1, 0xFFFFFFFF;" : "=l"(u) : "r"(w2));
  Lz z;
  asm("{\n\t.reg .u32 sh, u0, u1;\n\t"
      "mov.b64 {u0, u1}, %5;\n\t"
      "shr.s32 sh, %4, 31;\n\t"
      "sub.cc.u32 %0, u0, %4;\n\t"
      "subc.cc.u32 %1, u1, sh;\n\t"
      "subc.u32 %2, 0, sh;\n\t"
      "add.cc.u32 %1, %1, %3;\n\t"
      "addc.u32 %2, %2, 0;\n\t"
      "}"
      : "=&r"(z.l), "=&r"(z.h), "=&r"(z.k)
      : "r"(w1), "r"(w3), "l"(u));
  return z;
}

__device__ __forceinline__ Lz lz_shl72_n(Lz x) {
  const uint32_t y0 = x.l << 8, y1 = __funnelshift_l(x.l, x.h, 8);
  const int32_t y2 = (int32_t)(x.h >> 24) + (int32_t)((uint32_t)x.k << 8);
  uint64_t u;
  asm("mul.wide.u32 %0, %1, 0xFFFFFFFF;" : "=l"(u) : "r"(y0));
  Lz z;
  asm("{\n\t.reg .u32 sh, u0, u1;\n\t"
      "mov.b64 {u0, u1}, %5;\n\t"
      "shr.s32 sh, %4, 31;\n\t"
      "sub.cc.u32 %0, u0, %3;\n\t"
      "subc.cc.u32 %1, u1, %4;\n\t"
      "subc.u32 %2, 0, sh;\n\t"
      "}"
      : "=&r"(z.l), "=&r"(z.h), "=&r"(z.k)
      : "r"(y1), "r"(y2), "l"(u));
  return z;
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
