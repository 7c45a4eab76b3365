// Goldilocks NTT building blocks shared by the multiply kernels.
//
// Transform structure (this engine's design, not the reference's): a
// length-N = 2^L transform is split into HBM passes of radix R_p = 2^r_p.
// Pass p works on blocks of M_p = R_p * S_p consecutive words and, inside a
// block, on R_p rows of stride S_p.  The forward direction is a
// decimation-in-frequency split: per column j it takes the R_p-point DFT
// over the rows, multiplies output row f by w_M^(f*j) and stores it back in
// place, so every output row is an independent length-S_p problem for the
// next pass.  The spectrum ends in a fixed digit-reversed order; the
// pointwise product does not care, and the inverse passes (the exact mirror)
// restore natural order.  This is the reference's four-step decomposition
// (crates/bignum/src/ntt.rs:905-1105) without the transposes: strided tiles
// are read as coalesced 64-byte (or wider) row segments.
//
// Inside a pass the R_p-point DFT runs in shared memory as rounds of radix
// 8 (or 4 / 2) held in registers.  2 is a 192nd root of unity mod p, and the
// root tables are built so that the 8th root of unity is 2^24: the
// butterflies' internal twiddles are constant shifts.
#pragma once
#include <cstdint>
#include <type_traits>
#include "gl.cuh"

namespace pimul {

// Root tables.  rho is a primitive 2^32-th root of unity with
// rho^(2^26) = 8 (the 64th root of unity is 2^3).  Every twiddle of every
// transform length is a power of rho.
struct Roots {
  const uint64_t* lo;   // rho^e, e in [0, 2^16)
  const uint64_t* hi;   // rho^(e * 2^16), e in [0, 2^16)
  const uint64_t* w12;  // w_4096^t = rho^(t * 2^20), t in [0, 4096)
  const uint64_t* lvl;  // per-level tables: w_(2^k)^x at lvl[2^k + x], 1 <= k <= LVL_MAX
  const uint64_t* near; // w_(2^L)^(+-x) for x < 4096, LVL_MAX < L <= 32 (see near_table)
};

constexpr int LVL_MAX = 20;
constexpr int NEAR_LEVELS = 32 - LVL_MAX;  // transform lengths 2^21 .. 2^32

// The 4096 powers w_(2^L)^x (inverse: w_(2^L)^-x), x < 4096, of a length
// 2^L > 2^LVL_MAX.  A first-pass twiddle w^(f (j0 + jj)) with f jj < 4096
// is w^(f j0) (staged per CTA) times one entry of this 32 KB table, which
// stays in L1, instead of two loads from the 512 KB rho tables.
__device__ __forceinline__ const uint64_t* near_table(const Roots& R, int L, bool inverse) {
  return R.near + ((size_t)(L - LVL_MAX - 1) * 2 + (inverse ? 1 : 0)) * 4096;
}

// rho^e for e in [0, 2^32).
__device__ __forceinline__ uint64_t rho_pow(const Roots& R, uint32_t e) {
  uint64_t a = __ldg(R.lo + (e & 0xFFFFu));
  uint32_t h = e >> 16;
  return h ? gl::mul(a, __ldg(R.hi + h)) : a;
}

// w_M^x for M = 2^mlog, x in [0, M); inverse gives w_M^(-x).  Levels up
// to 2^20 read one contiguous table; longer ones combine two table entries.
__device__ __forceinline__ uint64_t root_pow(const Roots& R, int mlog, uint64_t x, bool inverse) {
  uint64_t m = 1ull << mlog;
  x &= m - 1;
  if (inverse) x = (m - x) & (m - 1);
  if (mlog <= LVL_MAX) return __ldg(R.lvl + m + x);
  return rho_pow(R, (uint32_t)(x << (32 - mlog)));
}

// root_pow for an exponent already reduced mod 2^32 (x is taken mod 2^mlog),
// with 32-bit index arithmetic.
__device__ __forceinline__ uint64_t root_pow32(const Roots& R, int mlog, uint32_t x, bool inverse) {
  const uint32_t mask = mlog >= 32 ? 0xFFFFFFFFu : (1u << mlog) - 1;
  x &= mask;
  if (inverse) x = (0u - x) & mask;
  if (mlog <= LVL_MAX) return __ldg(R.lvl + (1u << mlog) + x);
  return rho_pow(R, x << (32 - mlog));
}

// w_(2^mlog)^x for x < 2^mlog <= 4096 from the 4096-entry table (forward or inverse).
__device__ __forceinline__ uint64_t round_tw(const Roots& R, int mlog, uint32_t x, bool inverse) {
  uint32_t t = x << (12 - mlog);
  if (inverse) t = (4096u - t) & 4095u;
  return __ldg(R.w12 + t);
}

// Shared-memory index with one pad word per 16 to spread 8-byte banks.
__host__ __device__ __forceinline__ constexpr uint32_t spad(uint32_t lin) { return lin + (lin >> 4); }

// spad(base | (m << s)) = spad(base) + spad_step(m, s) whenever base has zero
// bits where m << s lands (the bits below 4 either come from base alone or
// the shifted m stays inside one 16-word run): per-element shared-memory
// offsets of a butterfly group are compile-time constants.
__host__ __device__ __forceinline__ constexpr uint32_t spad_step(uint32_t m, int s) {
  return (m << s) + ((m << s) >> 4);
}

// Asynchronous 8-byte global -> shared copy (no register round trip), and
// the wait for all of this thread's outstanding copies.
__device__ __forceinline__ void cp_async8(uint64_t* smem_dst, const uint64_t* gsrc) {
  const uint32_t s = (uint32_t)__cvta_generic_to_shared(smem_dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(s), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Bulk prefetch of [src, src + bytes) into L2 (no completion to wait for);
// src 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void prefetch_l2_bulk(const void* src, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}

// DIF radix-2 butterfly with a constant shift twiddle 2^S (S = 0: none).
template <int S>
__device__ __forceinline__ void bfly_dif(uint64_t& a, uint64_t& b) {
  uint64_t u = a, w = b;
  a = gl::add(u, w);
  b = gl::shl<S>(gl::sub(u, w));
}

// Forward DFT of 2^B values in registers: v[k] <- sum_m v[m] w^(m k), with
// w = 2^(192 / 2^B) (the 8th root of unity is 2^24).  Natural-order output.
// Radix 4 and 8 run on lazy values (see gl.cuh) and fold once per output;
// the internal twiddles are the lazy shifts of gl.cuh.  Inputs are lazy
// with |k| <= 1 (e.g. products from lz_mul).
template <int B>
__device__ __forceinline__ void dft_fwd_lz(const gl::Lz* x, uint64_t* v) {
  using namespace gl;
  if constexpr (B == 1) {
    v[0] = fold(lz_add(x[0], x[1]));
    v[1] = fold(lz_sub(x[0], x[1]));
  } else if constexpr (B == 2) {
    Lz a0 = lz_add(x[0], x[2]), c = lz_sub(x[0], x[2]);
    Lz a1 = lz_add(x[1], x[3]);
    Lz d = lz_shl48_n(lz_sub(x[1], x[3]));
    v[0] = fold(lz_add(a0, a1));
    v[1] = fold(lz_add(c, d));
    v[2] = fold(lz_sub(a0, a1));
    v[3] = fold(lz_sub(c, d));
  } else {
    static_assert(B == 3, "radix 2, 4 or 8");
    // stage 1: x_m +- x_(m+4); the differences d_m carry the twiddle w^m
    Lz a0 = lz_add(x[0], x[4]), d0 = lz_sub(x[0], x[4]);
    Lz a1 = lz_add(x[1], x[5]), d1 = lz_sub(x[1], x[5]);
    Lz a2 = lz_add(x[2], x[6]), d2 = lz_sub(x[2], x[6]);
    Lz a3 = lz_add(x[3], x[7]), d3 = lz_sub(x[3], x[7]);
    // even outputs: radix 4 on the sums
    Lz c0 = lz_add(a0, a2), c2 = lz_sub(a0, a2);
    Lz c1 = lz_add(a1, a3), c3 = lz_shl48_n(lz_sub(a1, a3));
    v[0] = fold(lz_add(c0, c1));
    v[4] = fold(lz_sub(c0, c1));
    v[2] = fold(lz_add(c2, c3));
    v[6] = fold(lz_sub(c2, c3));
    // odd outputs: radix 4 on b_m = w^m d_m.  With g = w^2 d3,
    // b1 + b3 = w (d1 + g) and (b1 - b3) w^2 = w^3 (d1 - g), so every shift
    // acts on a value with a small overflow count and the one by w (24 bits)
    // can stay lazy
    Lz b2 = lz_shl48_n(d2);
    Lz e0 = lz_add(d0, b2), e2 = lz_sub(d0, b2);
    Lz g = lz_shl48_n(d3);
    Lz e1 = lz_shl24_wide(lz_add(d1, g)), e3 = lz_shl72_n(lz_sub(d1, g));
    v[1] = fold(lz_add(e0, e1));
    v[5] = fold(lz_sub(e0, e1));
    v[3] = fold(lz_add(e2, e3));
    v[7] = fold(lz_sub(e2, e3));
  }
}

// dft_fwd_lz<3> for inputs whose upper half x[4..7] is zero: stage 1 is
// then a_m = d_m = x_m.  A lazy sum or difference with zero leaves the lazy
// value unchanged, so the outputs are those of dft_fwd_lz<3> bit for bit.
__device__ __forceinline__ void dft_fwd_lz_half8(const gl::Lz* x, uint64_t* v) {
  using namespace gl;
  Lz c0 = lz_add(x[0], x[2]), c2 = lz_sub(x[0], x[2]);
  Lz c1 = lz_add(x[1], x[3]), c3 = lz_shl48_n(lz_sub(x[1], x[3]));
  v[0] = fold(lz_add(c0, c1));
  v[4] = fold(lz_sub(c0, c1));
  v[2] = fold(lz_add(c2, c3));
  v[6] = fold(lz_sub(c2, c3));
  Lz b2 = lz_shl48_n(x[2]);
  Lz e0 = lz_add(x[0], b2), e2 = lz_sub(x[0], b2);
  Lz g = lz_shl48_n(x[3]);
  Lz e1 = lz_shl24_wide(lz_add(x[1], g)), e3 = lz_shl72_n(lz_sub(x[1], g));
  v[1] = fold(lz_add(e0, e1));
  v[5] = fold(lz_sub(e0, e1));
  v[3] = fold(lz_add(e2, e3));
  v[7] = fold(lz_sub(e2, e3));
}

template <int B>
__device__ __forceinline__ void dft_fwd(uint64_t* v) {
  if constexpr (B == 1) {
    bfly_dif<0>(v[0], v[1]);
  } else {
    gl::Lz x[1 << B];
#pragma unroll
    for (int k = 0; k < (1 << B); k++) x[k] = gl::lz(v[k]);
    dft_fwd_lz<B>(x, v);
  }
}

// Unscaled inverse of dft_fwd on lazy inputs (|k| <= 1, e.g. twiddle
// products from lz_mul): v[m] <- sum_k x[k] w^(-m k)  (= 2^B * original).
// w^-s = -w^(96 - s): the DIT butterfly u +- w^-s b becomes u -+ 2^(96-s) b.
template <int B>
__device__ __forceinline__ void dft_inv_lz(const gl::Lz* x, uint64_t* v) {
  using namespace gl;
  if constexpr (B == 1) {
    v[0] = fold(lz_add(x[0], x[1]));
    v[1] = fold(lz_sub(x[0], x[1]));
  } else if constexpr (B == 2) {
    // inputs in bit-reversed order (x0, x2, x1, x3)
    Lz s = lz_add(x[0], x[2]), d = lz_sub(x[0], x[2]);
    Lz t = lz_add(x[1], x[3]);
    Lz e = lz_shl48_n(lz_sub(x[1], x[3]));
    v[0] = fold(lz_add(s, t));
    v[2] = fold(lz_sub(s, t));
    v[1] = fold(lz_sub(d, e));
    v[3] = fold(lz_add(d, e));
  } else {
    static_assert(B == 3, "radix 2, 4 or 8");
    // inputs in bit-reversed order (x0, x4, x2, x6, x1, x5, x3, x7)
    Lz s01 = lz_add(x[0], x[4]), d01 = lz_sub(x[0], x[4]);
    Lz s23 = lz_add(x[2], x[6]), d23 = lz_sub(x[2], x[6]);
    Lz s45 = lz_add(x[1], x[5]), d45 = lz_sub(x[1], x[5]);
    Lz s67 = lz_add(x[3], x[7]), d67 = lz_sub(x[3], x[7]);
    Lz t23 = lz_shl48_n(d23), t67 = lz_shl48_n(d67);
    Lz v0 = lz_add(s01, s23), v2 = lz_sub(s01, s23);
    Lz v1 = lz_sub(d01, t23), v3 = lz_add(d01, t23);
    Lz v4 = lz_add(s45, s67), v6 = lz_sub(s45, s67);
    Lz v5 = lz_sub(d45, t67), v7 = lz_add(d45, t67);
    Lz t5 = lz_shl72_n(v5), t6 = lz_shl48_n(v6), t7 = lz_shl24_wide(v7);
    v[0] = fold(lz_add(v0, v4));
    v[4] = fold(lz_sub(v0, v4));
    v[1] = fold(lz_sub(v1, t5));
    v[5] = fold(lz_add(v1, t5));
    v[2] = fold(lz_sub(v2, t6));
    v[6] = fold(lz_add(v2, t6));
    v[3] = fold(lz_sub(v3, t7));
    v[7] = fold(lz_add(v3, t7));
  }
}

template <int B>
__device__ __forceinline__ void dft_inv(uint64_t* v) {
  gl::Lz x[1 << B];
#pragma unroll
  for (int k = 0; k < (1 << B); k++) x[k] = gl::lz(v[k]);
  dft_inv_lz<B>(x, v);
}

// ---------------------------------------------------------------- rounds
// Round split of an r-bit in-tile DFT: radix-8 rounds first, then radix 4
// or 2 (two radix-4 rounds instead of 8 + 2).
__host__ __device__ constexpr int rp_count(int r) {
  int n = 0;
  while (r > 0) {
    int b = r >= 3 ? 3 : r;
    if (r == 4) b = 2;
    r -= b;
    n++;
  }
  return n;
}

__host__ __device__ constexpr int rp_bits(int r, int q) {
  int i = 0;
  while (r > 0) {
    int b = r >= 3 ? 3 : r;
    if (r == 4) b = 2;
    if (i == q) return b;
    r -= b;
    i++;
  }
  return 0;
}

// Sub-problem size (log2) at the start of round q.
__host__ __device__ constexpr int rp_mlog(int r, int q) {
  int m = r;
  for (int i = 0; i < q; i++) m -= rp_bits(r, i);
  return m;
}

// Item order of a round: with one pad word per 16, a half-warp of some
// rounds puts two or four lanes on one 8-byte bank (rows 64 words apart
// land 4 banks apart).  Up to two swaps of item-number bits, a bijection on
// the round's items, spread them; the swaps per round come from a model of
// the padded layout, packed as a1 | b1 << 4 | a2 << 8 | b2 << 12 (a == b:
// no swap).
template <int R, int T, int BC, int MLOG>
__host__ __device__ constexpr int round_swaps() {
  return (T == 3 && BC == 0 && R == 9 && MLOG == 3)   ? (3 | 4 << 4)
         : (T == 0 && R == 9 && MLOG == 6)             ? (3 | 4 << 4)
         : (T == 3 && (R == 8 || R == 7) && MLOG == 2) ? (3 | 5 << 4)
         : (T == 3 && R == 6 && MLOG == 3)             ? (3 | 4 << 4)
         : (T == 0 && R == 6 && MLOG == 6)             ? (3 | 4 << 4)
         : (T == 0 && R == 7 && MLOG == 4)             ? (0 | 4 << 4 | 1 << 8 | 5 << 12)
         : (T == 0 && R == 8 && MLOG == 5)             ? (0 | 1 << 4 | 1 << 8 | 4 << 12)
                                                       : 0;
}

template <int A, int B>
__device__ __forceinline__ uint32_t swap_bits(uint32_t w) {
  if constexpr (A == B) {
    return w;
  } else {
    const uint32_t d = ((w >> A) ^ (w >> B)) & 1u;
    return w ^ (d << A) ^ (d << B);
  }
}

template <int S>
__device__ __forceinline__ uint32_t round_item(uint32_t w) {
  return swap_bits<(S >> 8) & 15, (S >> 12) & 15>(swap_bits<S & 15, (S >> 4) & 15>(w));
}

// Tile of 2^BC blocks x 2^R rows x 2^T columns in shared memory; element
// (row, col) of the flattened (BC+R)-bit row index at spad(row << T | col).
// One forward round of radix 2^B over sub-problems of 2^MLOG rows.
// One forward round of radix 2^B over sub-problems of 2^MLOG rows.  The
// twiddles of the previous round (radix 2^PB over 2^PMLOG rows, PB = 0: none)
// are applied here, to the inputs, as lazy products that feed the DFT
// directly: element row r had position jp' = r mod 2^MLOG and output index
// k' = (r >> MLOG) mod 2^PB there, twiddle w_(2^PMLOG)^(k' jp').
// tw512 holds the 2^TWLOG roots w^t of one fixed length (512 in the pass
// kernels, 4096 in the one-CTA merge of whole transforms).  HALF: the first
// radix-8 round of a tile whose rows 2^(R-1) .. 2^R - 1 are zero (they are
// not read; every row is written).
template <int R, int T, int BC, int B, int MLOG, int NT, int PB, int PMLOG, int TWLOG = 9, bool HALF = false>
__device__ __forceinline__ void round_fwd_t(uint64_t* sm, const uint64_t* tw512, int tid) {
  constexpr int SLOG = MLOG - B;
  constexpr int ITEMS = 1 << (BC + R + T - B);
  static_assert(ITEMS % NT == 0, "tile must split evenly over the threads");
  static_assert(!HALF || (B == 3 && PB == 0 && MLOG == R && BC == 0), "HALF: the first radix-8 round of one block");
#pragma unroll 2
  for (int it = 0; it < ITEMS / NT; it++) {
    const uint32_t w = round_item<round_swaps<R, T, BC, MLOG>()>(it * NT + tid);
    const uint32_t j = w & ((1u << T) - 1);
    const uint32_t rest = w >> T;
    const uint32_t jp = rest & ((1u << SLOG) - 1);
    const uint32_t row0 = ((rest >> SLOG) << MLOG) + jp;
    const uint32_t sb = spad((row0 << T) | j);  // bits [SLOG+T, MLOG+T) are zero
    uint64_t v[1 << B];
    gl::Lz x[1 << B];
    if constexpr (HALF) {
#pragma unroll
      for (int m = 0; m < 4; m++) x[m] = gl::lz(sm[sb + spad_step(m, SLOG + T)]);
      dft_fwd_lz_half8(x, v);
#pragma unroll
      for (int k = 0; k < 8; k++) sm[sb + spad_step(k, SLOG + T)] = v[k];
      continue;
    }
#pragma unroll
    for (int m = 0; m < (1 << B); m++) v[m] = sm[sb + spad_step(m, SLOG + T)];
    if constexpr (PB > 0) {
      static_assert(PMLOG - PB == MLOG, "rounds must nest");
      const uint32_t kp = (rest >> SLOG) & ((1u << PB) - 1);
      const uint32_t base = (kp * jp) << (TWLOG - PMLOG), step = (kp << SLOG) << (TWLOG - PMLOG);
#pragma unroll
      for (int m = 0; m < (1 << B); m++) x[m] = gl::lz_mul(v[m], tw512[base + m * step]);
    } else {
#pragma unroll
      for (int m = 0; m < (1 << B); m++) x[m] = gl::lz(v[m]);
    }
    dft_fwd_lz<B>(x, v);
#pragma unroll
    for (int k = 0; k < (1 << B); k++) sm[sb + spad_step(k, SLOG + T)] = v[k];
  }
}

// Pass twiddle applied by the first inverse round: none.
struct NoPassTw {};

// One inverse round; the first one executed (SLOG = 0, no round twiddles)
// multiplies its inputs by the pass twiddles of the tile when a functor is
// given (ptw(row0, k, col) for tile row row0 + k, row0 a multiple of 2^B),
// feeding the lazy products straight into the DFT.
template <int R, int T, int BC, int B, int MLOG, int NT, class F, int TWLOG = 9>
__device__ __forceinline__ void round_inv_t(uint64_t* sm, const uint64_t* tw512, int tid, const F& ptw) {
  constexpr int SLOG = MLOG - B;
  constexpr int ITEMS = 1 << (BC + R + T - B);
  constexpr bool PTW = !std::is_same<F, NoPassTw>::value;
  static_assert(ITEMS % NT == 0, "tile must split evenly over the threads");
#pragma unroll 2
  for (int it = 0; it < ITEMS / NT; it++) {
    const uint32_t w = round_item<round_swaps<R, T, BC, MLOG>()>(it * NT + tid);
    const uint32_t j = w & ((1u << T) - 1);
    const uint32_t rest = w >> T;
    const uint32_t jp = rest & ((1u << SLOG) - 1);
    const uint32_t row0 = ((rest >> SLOG) << MLOG) + jp;
    const uint32_t sb = spad((row0 << T) | j);  // bits [SLOG+T, MLOG+T) are zero
    uint64_t v[1 << B];
    gl::Lz x[1 << B];
#pragma unroll
    for (int k = 0; k < (1 << B); k++) v[k] = sm[sb + spad_step(k, SLOG + T)];
    if constexpr (SLOG == 0 && PTW) {
      // rows row0 + k, row0 a multiple of 2^B
#pragma unroll
      for (int k = 0; k < (1 << B); k++) x[k] = gl::lz_mul(v[k], ptw(row0, k, j));
    } else {
      x[0] = gl::lz(v[0]);
      const uint32_t jps = jp << (TWLOG - MLOG);
#pragma unroll
      for (int k = 1; k < (1 << B); k++) {
        if constexpr (SLOG > 0) {
          x[k] = gl::lz_mul(v[k], tw512[((1u << TWLOG) - k * jps) & ((1u << TWLOG) - 1)]);
        } else {
          x[k] = gl::lz(v[k]);
        }
      }
    }
    dft_inv_lz<B>(x, v);
#pragma unroll
    for (int m = 0; m < (1 << B); m++) sm[sb + spad_step(m, SLOG + T)] = v[m];
  }
}

// HALF: rows 2^(R-1) .. 2^R - 1 of the tile are zero on entry (an operand
// that fills at most half of its transform); only the first round uses it.
template <int R, int T, int BC, int NT, bool HALF = false, int Q = 0>
__device__ __forceinline__ void tile_fwd_t(uint64_t* sm, const uint64_t* tw512, int tid) {
  if constexpr (Q < rp_count(R)) {
    round_fwd_t<R, T, BC, rp_bits(R, Q), rp_mlog(R, Q), NT, (Q > 0 ? rp_bits(R, Q - 1) : 0),
                (Q > 0 ? rp_mlog(R, Q - 1) : 0), 9, HALF && Q == 0>(sm, tw512, tid);
    __syncthreads();
    tile_fwd_t<R, T, BC, NT, false, Q + 1>(sm, tw512, tid);
  }
}

template <int R, int T, int BC, int NT, int Q = rp_count(R) - 1, class F = NoPassTw>
__device__ __forceinline__ void tile_inv_t(uint64_t* sm, const uint64_t* tw512, int tid, const F& ptw = F()) {
  if constexpr (Q >= 0) {
    round_inv_t<R, T, BC, rp_bits(R, Q), rp_mlog(R, Q), NT>(sm, tw512, tid, ptw);
    __syncthreads();
    tile_inv_t<R, T, BC, NT, Q - 1>(sm, tw512, tid);
  }
}

// Rounds of a contiguous pass with one warp per 512-word chunk of the tile
// (2^(9-R) blocks of 2^R words): a chunk's data never leaves its warp, so the
// rounds synchronise with __syncwarp instead of the whole CTA.  smc is the
// chunk's base in shared memory (its words at smc + spad(i), i < 512).
template <int R, int Q = 0>
__device__ __forceinline__ void chunk_fwd_t(uint64_t* smc, const uint64_t* tw512, int lane) {
  if constexpr (Q < rp_count(R)) {
    round_fwd_t<R, 0, 9 - R, rp_bits(R, Q), rp_mlog(R, Q), 32, (Q > 0 ? rp_bits(R, Q - 1) : 0),
                (Q > 0 ? rp_mlog(R, Q - 1) : 0)>(smc, tw512, lane);
    __syncwarp();
    chunk_fwd_t<R, Q + 1>(smc, tw512, lane);
  }
}

// ptw: factors multiplied into the first inverse round's inputs as lazy
// products (ptw(row0, k, 0) for chunk word row0 + k), e.g. a pointwise product.
template <int R, int Q = rp_count(R) - 1, class F = NoPassTw>
__device__ __forceinline__ void chunk_inv_t(uint64_t* smc, const uint64_t* tw512, int lane, const F& ptw = F()) {
  if constexpr (Q >= 0) {
    round_inv_t<R, 0, 9 - R, rp_bits(R, Q), rp_mlog(R, Q), 32>(smc, tw512, lane, ptw);
    __syncwarp();
    chunk_inv_t<R, Q - 1>(smc, tw512, lane);
  }
}

// Frequency index held at tile row `row` after the rounds of an R-bit DFT
// (mixed-radix digit reversal of the row index).
// (A bit permutation: row_freq_t(a | b) = row_freq_t(a) | row_freq_t(b) for
// disjoint bit sets, which lets callers split a row into a per-thread part
// and a compile-time part.)
template <int R>
__host__ __device__ __forceinline__ constexpr uint32_t row_freq_t(uint32_t row) {
  uint32_t f = 0;
  int rem = R, sh = 0;
#pragma unroll
  for (int q = 0; q < rp_count(R); q++) {
    int b = rp_bits(R, q);
    rem -= b;
    f |= ((row >> rem) & ((1u << b) - 1)) << sh;
    sh += b;
  }
  return f;
}

// ------------------------------------------------- runtime-geometry rounds
// Used by the one-CTA multiply, whose transform length varies per call.
struct TileGeom {
  int r, t, bc;
};

template <int B>
__device__ __forceinline__ void round_fwd(uint64_t* sm, TileGeom g, int mlog, const Roots& R, int tid,
                                          int nthreads) {
  const int slog = mlog - B;
  const int items_log = g.bc + g.r + g.t - B;
  const uint32_t tmask = (1u << g.t) - 1, smask = (1u << slog) - 1;
  for (uint32_t w = tid; w < (1u << items_log); w += nthreads) {
    uint32_t j = w & tmask;
    uint32_t rest = w >> g.t;
    uint32_t jp = rest & smask;
    uint32_t row0 = ((rest >> slog) << mlog) + jp;
    uint64_t v[1 << B];
#pragma unroll
    for (int m = 0; m < (1 << B); m++) v[m] = sm[spad(((row0 + (m << slog)) << g.t) | j)];
    dft_fwd<B>(v);
    if (slog > 0) {
#pragma unroll
      for (int k = 1; k < (1 << B); k++) v[k] = gl::mul(v[k], round_tw(R, mlog, k * jp, false));
    }
#pragma unroll
    for (int k = 0; k < (1 << B); k++) sm[spad(((row0 + (k << slog)) << g.t) | j)] = v[k];
  }
}

template <int B>
__device__ __forceinline__ void round_inv(uint64_t* sm, TileGeom g, int mlog, const Roots& R, int tid,
                                          int nthreads) {
  const int slog = mlog - B;
  const int items_log = g.bc + g.r + g.t - B;
  const uint32_t tmask = (1u << g.t) - 1, smask = (1u << slog) - 1;
  for (uint32_t w = tid; w < (1u << items_log); w += nthreads) {
    uint32_t j = w & tmask;
    uint32_t rest = w >> g.t;
    uint32_t jp = rest & smask;
    uint32_t row0 = ((rest >> slog) << mlog) + jp;
    uint64_t v[1 << B];
    gl::Lz x[1 << B];
#pragma unroll
    for (int k = 0; k < (1 << B); k++) v[k] = sm[spad(((row0 + (k << slog)) << g.t) | j)];
    x[0] = gl::lz(v[0]);
#pragma unroll
    for (int k = 1; k < (1 << B); k++)
      x[k] = slog > 0 ? gl::lz_mul(v[k], round_tw(R, mlog, k * jp, true)) : gl::lz(v[k]);
    dft_inv_lz<B>(x, v);
#pragma unroll
    for (int m = 0; m < (1 << B); m++) sm[spad(((row0 + (m << slog)) << g.t) | j)] = v[m];
  }
}

__device__ __forceinline__ void tile_dft_fwd(uint64_t* sm, TileGeom g, const Roots& R, int tid, int nthreads) {
  int mlog = g.r, rem = g.r;
  while (rem > 0) {
    int b = rem >= 3 ? 3 : rem;
    if (rem == 4) b = 2;
    if (b == 3) round_fwd<3>(sm, g, mlog, R, tid, nthreads);
    else if (b == 2) round_fwd<2>(sm, g, mlog, R, tid, nthreads);
    else round_fwd<1>(sm, g, mlog, R, tid, nthreads);
    mlog -= b;
    rem -= b;
    __syncthreads();
  }
}

__device__ __forceinline__ void tile_dft_inv(uint64_t* sm, TileGeom g, const Roots& R, int tid, int nthreads) {
  int bits[8], n = 0, rem = g.r;
  while (rem > 0) {
    int b = rem >= 3 ? 3 : rem;
    if (rem == 4) b = 2;
    bits[n++] = b;
    rem -= b;
  }
  int mlog = 0;
  for (int q = n - 1; q >= 0; q--) {
    int b = bits[q];
    mlog += b;
    if (b == 3) round_inv<3>(sm, g, mlog, R, tid, nthreads);
    else if (b == 2) round_inv<2>(sm, g, mlog, R, tid, nthreads);
    else round_inv<1>(sm, g, mlog, R, tid, nthreads);
    __syncthreads();
  }
}

}  // namespace pimul
