// Goldilocks NTT building blocks shared by the multiply kernels.
//
// Transform structure (design of this engine, not of the reference): a
// length-N = 2^L transform is split into HBM passes of radix R_p = 2^r_p.
// Pass p works on blocks of M_p = R_p * S_p consecutive words and, inside a
// block, on R_p rows of stride S_p.  The forward direction is a
// decimation-in-frequency split: per column j it takes the R_p-point DFT
// over the rows, multiplies output row f by w_M^(f*j) and stores it back in
// place, so that every output row is an independent length-S_p problem for
// the next pass.  The spectrum ends in a fixed digit-reversed order; the
// pointwise product does not care, and the inverse passes (the exact mirror)
// restore natural order.  This is the same decomposition as the reference's
// four-step transform (crates/bignum/src/ntt.rs:905-1105) without the
// transposes: strided tiles are read with coalesced 128-byte row segments.
//
// Inside a pass the R_p-point DFT runs in shared memory as rounds of
// radix 2, 4 or 8 held in registers; the radix-8 butterflies use the
// 8th roots of unity 2^24 and 2^48 (2 is a 192nd root of unity mod p), so
// their internal twiddles are shifts rather than general multiplies.
#pragma once
#include <cstdint>
#include "gl.cuh"

namespace pimul {

// Root tables: rho is a primitive 2^32-th root of unity chosen so that
// rho^(2^26) = 8, i.e. the 64th root of unity is 2^3.  Every twiddle of every
// transform length is a power of rho.
struct Roots {
  const uint64_t* lo;   // rho^e, e in [0, 2^16)
  const uint64_t* hi;   // rho^(e * 2^16), e in [0, 2^16)
  const uint64_t* w12;  // w_4096^t = rho^(t * 2^20), t in [0, 4096)
};

// rho^e for e in [0, 2^32).
__device__ __forceinline__ uint64_t rho_pow(const Roots& R, uint32_t e) {
  uint64_t a = __ldg(R.lo + (e & 0xFFFFu));
  uint32_t h = e >> 16;
  return h ? gl::mul(a, __ldg(R.hi + h)) : a;
}

// w_(2^mlog)^x for x < 2^mlog <= 4096 (forward), or its inverse.
__device__ __forceinline__ uint64_t round_tw(const Roots& R, int mlog, uint32_t x, bool inverse) {
  uint32_t t = x << (12 - mlog);
  if (inverse) t = (4096u - t) & 4095u;
  return __ldg(R.w12 + t);
}

// Shared-memory index with one pad word per 16 to spread 8-byte banks.
__device__ __forceinline__ uint32_t spad(uint32_t lin) { return lin + (lin >> 4); }

template <int B>
__device__ __forceinline__ void reg_bitrev(uint64_t* v) {
  if constexpr (B == 2) {
    uint64_t t = v[1]; v[1] = v[2]; v[2] = t;
  } else if constexpr (B == 3) {
    uint64_t t = v[1]; v[1] = v[4]; v[4] = t;
    t = v[3]; v[3] = v[6]; v[6] = t;
  }
}

// Forward DFT of 2^B values in registers: v[k] <- sum_m v[m] w^(m k), with
// w = 2^(192 / 2^B).  Output in natural order.
template <int B>
__device__ __forceinline__ void dft_fwd(uint64_t* v) {
#pragma unroll
  for (int h = (1 << B) / 2; h >= 1; h >>= 1) {
#pragma unroll
    for (int g = 0; g < (1 << B); g += 2 * h) {
#pragma unroll
      for (int m = 0; m < h; m++) {
        uint64_t u = v[g + m], w = v[g + m + h];
        v[g + m] = gl::add(u, w);
        uint64_t d = gl::sub(u, w);
        v[g + m + h] = (m == 0) ? d : gl::shl(d, (96 / h) * m);
      }
    }
  }
  reg_bitrev<B>(v);
}

// Unscaled inverse of dft_fwd: v[m] <- sum_k v[k] w^(-m k)  (= 2^B * x[m]).
template <int B>
__device__ __forceinline__ void dft_inv(uint64_t* v) {
  reg_bitrev<B>(v);
#pragma unroll
  for (int h = 1; h < (1 << B); h <<= 1) {
#pragma unroll
    for (int g = 0; g < (1 << B); g += 2 * h) {
#pragma unroll
      for (int m = 0; m < h; m++) {
        uint64_t u = v[g + m];
        uint64_t w = (m == 0) ? v[g + m + h] : gl::shl(v[g + m + h], 192 - (96 / h) * m);
        v[g + m] = gl::add(u, w);
        v[g + m + h] = gl::sub(u, w);
      }
    }
  }
}

// Tile geometry in shared memory: (2^bc blocks) x (2^r rows) x (2^t columns),
// element (blk,row,col) at spad(((blk << r) + row) << t | col).  A round
// treats the 2^(bc+r) tile rows as consecutive sub-problems of 2^mlog rows.
struct TileGeom {
  int r, t, bc;
};

// One forward round of radix 2^B on sub-problems of size 2^mlog.
template <int B>
__device__ __forceinline__ void round_fwd(uint64_t* sm, TileGeom g, int mlog, const Roots& R,
                                          int tid, int nthreads) {
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

// Mirror of round_fwd (unscaled).
template <int B>
__device__ __forceinline__ void round_inv(uint64_t* sm, TileGeom g, int mlog, const Roots& R,
                                          int tid, int nthreads) {
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
    for (int k = 0; k < (1 << B); k++) v[k] = sm[spad(((row0 + (k << slog)) << g.t) | j)];
    if (slog > 0) {
#pragma unroll
      for (int k = 1; k < (1 << B); k++) v[k] = gl::mul(v[k], round_tw(R, mlog, k * jp, true));
    }
    dft_inv<B>(v);
#pragma unroll
    for (int m = 0; m < (1 << B); m++) sm[spad(((row0 + (m << slog)) << g.t) | j)] = v[m];
  }
}

// Round split of an r-bit pass: radix-8 rounds first, then one radix-4 or
// radix-2 round (or two radix-4 rounds instead of 8 + 2).
struct RoundPlan {
  int n;
  int bits[6];
};

__host__ __device__ inline RoundPlan round_plan(int r) {
  RoundPlan p{0, {0, 0, 0, 0, 0, 0}};
  int rem = r;
  while (rem > 0) {
    int b = rem >= 3 ? 3 : rem;
    if (rem == 4) b = 2;
    p.bits[p.n++] = b;
    rem -= b;
  }
  return p;
}

// All rounds of an r-bit in-tile DFT (forward).
__device__ __forceinline__ void tile_dft_fwd(uint64_t* sm, TileGeom g, const RoundPlan& rp,
                                             const Roots& R, int tid, int nthreads) {
  int mlog = g.r;
  for (int q = 0; q < rp.n; q++) {
    int b = rp.bits[q];
    if (b == 3) round_fwd<3>(sm, g, mlog, R, tid, nthreads);
    else if (b == 2) round_fwd<2>(sm, g, mlog, R, tid, nthreads);
    else round_fwd<1>(sm, g, mlog, R, tid, nthreads);
    mlog -= b;
    __syncthreads();
  }
}

__device__ __forceinline__ void tile_dft_inv(uint64_t* sm, TileGeom g, const RoundPlan& rp,
                                             const Roots& R, int tid, int nthreads) {
  int mlog = 0;
  for (int q = rp.n - 1; q >= 0; q--) {
    int b = rp.bits[q];
    mlog += b;
    if (b == 3) round_inv<3>(sm, g, mlog, R, tid, nthreads);
    else if (b == 2) round_inv<2>(sm, g, mlog, R, tid, nthreads);
    else round_inv<1>(sm, g, mlog, R, tid, nthreads);
    __syncthreads();
  }
}

// Frequency index held at tile row `row` after the rounds of `rp`
// (mixed-radix digit reversal of the row index).
__device__ __forceinline__ uint32_t row_freq(uint32_t row, int r, const RoundPlan& rp) {
  uint32_t f = 0;
  int rem = r, sh = 0;
  for (int q = 0; q < rp.n; q++) {
    int b = rp.bits[q];
    rem -= b;
    f |= ((row >> rem) & ((1u << b) - 1)) << sh;
    sh += b;
  }
  return f;
}

}  // namespace pimul
