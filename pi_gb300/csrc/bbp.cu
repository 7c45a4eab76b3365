// Batched BBP hex-digit extraction on sm_103a.
//
// Same result, bit for bit, as the reference's extractor
// (crates/pi-core/src/bbp.rs:52-140): for a position n it returns the top
// 32 bits of 4*S1 - 2*S4 - S5 - S6 (wrapping u64 fixed point), where
// S_j = sum_{k<=n} floor(((16^(n-k) mod d) << 64) / d) + tail_j, d = 8k+j,
// and tail_j is the f64 sum of 20 terms 1/(16^o (8(n+o)+j)) converted with
// a truncating cast.
//
// GPU design: the (position, series, k) space is cut into equal work items
// of 2^16 terms, run by a persistent grid (one full wave of CTAs); each
// warp adds its partial sum to its (position, series) slot with a 64-bit
// atomic.  The wrapping u64 sum is associative and commutative, so any
// split of k gives the same bits.  Each term floor((16^e mod d) 2^64 / d) is an exact 2-adic
// quotient (bbp_term): 2^(4e + 64 - t) mod m by Montgomery squarings and
// doublings on the odd part m of d = 2^t m (32-bit arithmetic below 2^32,
// 64-bit above), then one product with m^-1 mod 2^64; no term divides or
// converts a 64-bit integer to floating point (on this GPU those
// conversions run on the FP64 pipe).  The f64 tail uses explicitly rounded
// IEEE operations (no FMA contraction), so it matches the reference's f64
// arithmetic exactly.
// A stop flag in mapped host memory is read every 16 work items per warp
// (like bbp.rs:88-92); no thread ever waits on it.
#include <cuda_runtime.h>
#include <chrono>
#include <cstdint>
#include <cstring>
#include <string>
#include <thread>
#include <vector>
#include <algorithm>

#include "../../include/pimul.h"

namespace pimul_bbp {

static thread_local std::string t_err;
static int fail(int code, const std::string& m) {
  t_err = m;
  return code;
}

// -m^-1 mod 2^64 for odd m: Newton steps x <- x (2 - m x), each doubling the
// correct low bits (5 from the start value), three in 32-bit arithmetic and
// one in 64-bit.
__device__ __forceinline__ uint64_t neg_inv64(uint64_t m) {
  const uint32_t m0 = (uint32_t)m;
  uint32_t x = (3 * m0) ^ 2;
  x *= 2 - m0 * x;
  x *= 2 - m0 * x;
  x *= 2 - m0 * x;
  uint64_t y = x;
  y *= 2 - m * y;
  return 0 - y;
}

// Montgomery product a*b*2^-64 mod m, a, b < m < 2^34, m odd.
__device__ __forceinline__ uint64_t mont_mul(uint64_t a, uint64_t b, uint64_t m, uint64_t minv) {
  uint64_t tlo = a * b, thi = __umul64hi(a, b);
  uint64_t u = tlo * minv;
  uint64_t uhi = __umul64hi(u, m);
  uint64_t carry = (tlo != 0);  // tlo + ulo == 0 mod 2^64
  uint64_t r = thi + uhi + carry;
  return r >= m ? r - m : r;
}

// r mod m in [0, m) for a signed r with |r| < 2^62 and 1 <= m < 2^34, from
// a float reciprocal rm ~ 1/m (relative error below 2^-22): every estimate
// floor(r rm) leaves |r| at most 2^-21 of its size plus m, so three passes
// and a short final correction (bounded) reach [0, m).
__device__ __forceinline__ uint64_t mod_est(int64_t r, uint64_t m, float rm, int64_t* qacc = nullptr) {
  int64_t q = 0;
#pragma unroll
  for (int it = 0; it < 3; it++) {
    if (r >= 0 && (uint64_t)r < m) break;
    const int64_t c = __float2ll_rd(__fmul_rn((float)r, rm));
    r -= c * (int64_t)m;
    q += c;
  }
  for (int it = 0; it < 8 && r < 0; it++) r += (int64_t)m, q--;
  for (int it = 0; it < 8 && (uint64_t)r >= m; it++) r -= (int64_t)m, q++;
  if (qacc) *qacc += q;
  return (uint64_t)r;
}

// 2^64 mod m for odd 3 <= m < 2^34: q0 ~ 2^64 / m from the float
// reciprocal, then 2^64 - q0 m = (0 - q0 m) mod 2^64 is within 2^43 of the
// remainder and mod_est finishes.
__device__ __forceinline__ uint64_t pow2_64_mod(uint64_t m, float rm) {
  const uint64_t q0 = __float2ull_rz(__fmul_rn(rm, 18446744073709551616.0f));
  return mod_est((int64_t)(0 - q0 * m), m, rm);
}

// Montgomery product a*b*2^-32 mod m for a, b < m < 2^32, m odd: t + u m
// can pass 2^64 when m is near 2^32, so its carry is kept.
// In 32-bit words: t = a b = (th:tl), u = tl minv, and t + u m has low word
// 0 with a carry into the high word exactly when tl != 0; the high word sum
// th + hi(u m) + (tl != 0) is r = c 2^32 + h < 2m, and r >= m iff
// c - borrow(h - m) >= 0, in which case the result is h - m mod 2^32.
__device__ __forceinline__ uint32_t mont_mul32(uint32_t a, uint32_t b, uint32_t m, uint32_t minv) {
  uint32_t r;
  asm("{\n\t.reg .u32 tl, th, u, uh, z, c, d;\n\t.reg .pred p;\n\t"
      "mul.lo.u32 tl, %1, %2;\n\t"
      "mul.hi.u32 th, %1, %2;\n\t"
      "mul.lo.u32 u, tl, %4;\n\t"
      "mul.hi.u32 uh, u, %3;\n\t"
      "add.cc.u32 z, tl, 0xFFFFFFFF;\n\t"
      "addc.cc.u32 th, th, uh;\n\t"
      "addc.u32 c, 0, 0;\n\t"
      "sub.cc.u32 d, th, %3;\n\t"
      "subc.u32 c, c, 0;\n\t"
      "setp.ge.s32 p, c, 0;\n\t"
      "selp.u32 %0, d, th, p;\n\t"
      "}"
      : "=r"(r)
      : "r"(a), "r"(b), "r"(m), "r"(minv));
  return r;
}

// The same product for m < 2^31: t + u m < 2^62 + 2^63 cannot carry out of
// 64 bits and r = th + hi(u m) + (tl != 0) < 2m < 2^32, so the reduction is
// min(r, r - m) (r - m wraps above r exactly when r < m).
__device__ __forceinline__ uint32_t mont_mul31(uint32_t a, uint32_t b, uint32_t m, uint32_t minv) {
  uint32_t r;
  asm("{\n\t.reg .u32 tl, th, u, uh, z, s, d;\n\t"
      "mul.lo.u32 tl, %1, %2;\n\t"
      "mul.hi.u32 th, %1, %2;\n\t"
      "mul.lo.u32 u, tl, %4;\n\t"
      "mul.hi.u32 uh, u, %3;\n\t"
      "add.cc.u32 z, tl, 0xFFFFFFFF;\n\t"
      "addc.u32 s, th, uh;\n\t"
      "sub.u32 d, s, %3;\n\t"
      "min.u32 %0, s, d;\n\t"
      "}"
      : "=r"(r)
      : "r"(a), "r"(b), "r"(m), "r"(minv));
  return r;
}

// 2x mod m for x < m < 2^31: 2x < 2^32, min(2x, 2x - m).
__device__ __forceinline__ uint32_t dbl_mod31(uint32_t x, uint32_t m) {
  const uint32_t y = x + x;
  return min(y, y - m);
}

// 2x mod m for x < m < 2^32 (the same carry and borrow test).
__device__ __forceinline__ uint32_t dbl_mod32(uint32_t x, uint32_t m) {
  uint32_t r;
  asm("{\n\t.reg .u32 lo, c, d;\n\t.reg .pred p;\n\t"
      "add.cc.u32 lo, %1, %1;\n\t"
      "addc.u32 c, 0, 0;\n\t"
      "sub.cc.u32 d, lo, %2;\n\t"
      "subc.u32 c, c, 0;\n\t"
      "setp.ge.s32 p, c, 0;\n\t"
      "selp.u32 %0, d, lo, p;\n\t"
      "}"
      : "=r"(r)
      : "r"(x), "r"(m));
  return r;
}

// 16^e mod m for odd 3 <= m < 2^32 in 32-bit Montgomery arithmetic (the
// moduli of positions below about 5.4e8): a square is one wide multiply and
// two narrow ones, and the factor 16 is a Montgomery product with 16 R.
__device__ __forceinline__ uint64_t pow16_mod_odd32(uint64_t e, uint32_t m, float rm) {
  const uint32_t minv = (uint32_t)neg_inv64(m);
  const uint64_t q0 = __float2ull_rz(__fmul_rn(rm, 4294967296.0f));
  const uint32_t r1 = (uint32_t)mod_est((int64_t)((1ull << 32) - q0 * m), m, rm);  // R mod m
  const uint32_t b16 = (uint32_t)mod_est((int64_t)((uint64_t)r1 << 4), m, rm);     // 16 R mod m
  uint32_t x = r1;
  if (e) {
    const int top = 63 - __clzll((long long)e);
    x = b16;
    for (int b = top - 1; b >= 0; b--) {
      x = mont_mul32(x, x, m, minv);
      if ((e >> b) & 1) x = mont_mul32(x, b16, m, minv);
    }
  }
  return mont_mul32(x, 1, m, minv);  // out of Montgomery form
}

// 16^e mod d for 1 <= d < 2^34 (d == 1 -> 0, like bbp.rs:123-125).
__device__ __forceinline__ uint64_t pow16_mod(uint64_t e, uint64_t d) {
  if (d == 1) return 0;
  int t = __ffsll((long long)d) - 1;  // d = 2^t * m, m odd
  uint64_t m = d >> t;
  uint64_t rm_ = 0;   // 16^e mod m
  uint64_t minv = 0;  // -m^-1 mod 2^64 (m > 1)
  if (m > 1 && m < (1ull << 32)) {
    minv = neg_inv64(m);
    rm_ = pow16_mod_odd32(e, (uint32_t)m, __frcp_rn((float)m));
  } else if (m > 1) {
    const float rm = __frcp_rn((float)m);
    minv = neg_inv64(m);
    const uint64_t r1 = pow2_64_mod(m, rm);           // Montgomery one
    const uint64_t base = mod_est((int64_t)(r1 << 4), m, rm);  // 16 in Montgomery form
    uint64_t x = r1;
    if (e) {
      int top = 63 - __clzll((long long)e);
      x = base;
      for (int b = top - 1; b >= 0; b--) {
        x = mont_mul(x, x, m, minv);
        // times 16: Montgomery form is linear, so a shift and a reduction
        if ((e >> b) & 1) x = mod_est((int64_t)(x << 4), m, rm);
      }
    }
    rm_ = mont_mul(x, 1, m, minv);  // out of Montgomery form
  }
  // 16^e mod 2^t: 0 if 4e >= t, else 16^e (e = 0 gives 1)
  uint64_t r2 = (4 * e >= (uint64_t)t) ? 0 : (1ull << (4 * e));
  if (t == 0) return rm_;
  // CRT: x = rm (mod m), x = r2 (mod 2^t), x < d: x = rm + m s with
  // s = (r2 - rm) m^-1 (mod 2^t), m^-1 from the Montgomery constant
  const uint64_t mask = (1ull << t) - 1;
  const uint64_t inv = m > 1 ? (0 - minv) : 1;
  const uint64_t s2 = ((r2 - rm_) * inv) & mask;
  return rm_ + m * s2;
}

// 2^E mod m for odd 3 <= m < 2^32 and E >= 1 in 32-bit Montgomery
// arithmetic (R = 2^32): x runs through the Montgomery forms of 2^(prefix
// of E), one square per bit and one doubling per set bit.  R mod m comes
// from a 32-bit remainder; nothing converts 64-bit integers to floats.
// SMALL: m < 2^31, where the Montgomery product and the doubling need no
// carry out of 32 bits (mont_mul31, dbl_mod31).
template <bool SMALL>
__device__ __forceinline__ uint32_t mm32(uint32_t a, uint32_t b, uint32_t m, uint32_t minv) {
  if constexpr (SMALL) return mont_mul31(a, b, m, minv);
  else return mont_mul32(a, b, m, minv);
}
template <bool SMALL>
__device__ __forceinline__ uint32_t dbl32(uint32_t x, uint32_t m) {
  if constexpr (SMALL) return dbl_mod31(x, m);
  else return dbl_mod32(x, m);
}

template <bool SMALL>
__device__ __forceinline__ uint32_t pow2_mod_odd32(uint64_t E, uint32_t m, uint32_t minv) {
  uint32_t x = (0u - m) % m;  // R mod m: the Montgomery form of 1
  // bits 32 and up (E < 2^40) first, then the low word's 32 bits unrolled
  // with the current bit in the sign position; while x is the Montgomery
  // one (leading zeros of a small E) squaring leaves it unchanged
  const uint32_t eh = (uint32_t)(E >> 32);
  if (eh) {
    const int top = 31 - __clz((int)eh);
    x = dbl32<SMALL>(x, m);
    for (int b = top - 1; b >= 0; b--) {
      x = mm32<SMALL>(x, x, m, minv);
      if ((eh >> b) & 1) x = dbl32<SMALL>(x, m);
    }
  }
  uint32_t el = (uint32_t)E;
#pragma unroll
  for (int b = 0; b < 32; b++) {
    x = mm32<SMALL>(x, x, m, minv);
    if ((int32_t)el < 0) x = dbl32<SMALL>(x, m);
    el <<= 1;
  }
  return mm32<SMALL>(x, 1, m, minv);
}

// The same for odd 2^32 <= m < 2^34 in 64-bit Montgomery arithmetic.
__device__ __forceinline__ uint64_t pow2_mod_odd64(uint64_t E, uint64_t m, uint64_t minv) {
  uint64_t x = pow2_64_mod(m, __frcp_rn((float)m));  // R mod m (R = 2^64)
  const int top = 63 - __clzll((long long)E);
  for (int b = top; b >= 0; b--) {
    if (b != top) x = mont_mul(x, x, m, minv);
    if ((E >> b) & 1) {
      x <<= 1;  // < 2^35
      if (x >= m) x -= m;
    }
  }
  return mont_mul(x, 1, m, minv);
}

// One term of bbp.rs:117-140, floor((16^e mod d) 2^64 / d) for
// 1 <= d < 2^34, without a division.  With d = 2^t m (m odd) and
// p = 16^e mod d < d, p 2^(64-t) = q m + r' with q < 2^64 and
// r' = p 2^(64-t) mod m = 2^(4e + 64 - t) mod m, so q is the exact 2-adic
// quotient (p 2^(64-t) - r') m^-1 mod 2^64, and p 2^(64-t) mod 2^64 needs
// only p mod 2^t = 16^e mod 2^t.  d = 1 gives 0 (bbp.rs:123-125).
__device__ __forceinline__ uint64_t bbp_term(uint64_t e, uint64_t d) {
  if (d == 1) return 0;
  const int t = __ffsll((long long)d) - 1;
  const uint64_t m = d >> t;
  const uint64_t lo = (t == 0 || 4 * e >= (uint64_t)t) ? 0 : (1ull << (4 * e + 64 - (uint64_t)t));
  if (m == 1) return lo;
  const uint64_t E = 4 * e + 64 - (uint64_t)t;
  const uint64_t minv = neg_inv64(m);  // -m^-1 mod 2^64
  const uint64_t r = m < (1ull << 31)   ? (uint64_t)pow2_mod_odd32<true>(E, (uint32_t)m, (uint32_t)minv)
                     : m < (1ull << 32) ? (uint64_t)pow2_mod_odd32<false>(E, (uint32_t)m, (uint32_t)minv)
                                        : pow2_mod_odd64(E, m, minv);
  return (lo - r) * (0 - minv);
}

// floor(p * 2^64 / d) for p < d < 2^34 (the quotient fits in 64 bits): long
// division in steps of 30, 30 and 4 bits (r << 30 < 2^64), each quotient
// digit from the float reciprocal and mod_est's correction.
__device__ __forceinline__ uint64_t frac64(uint64_t p, uint64_t d) {
  const float rd = __frcp_rn((float)d);
  uint64_t r = p, q = 0;
  const int steps[3] = {30, 30, 4};
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const uint64_t x = r << steps[k];
    int64_t qd = (int64_t)__float2ull_rz(__fmul_rn((float)x, rd));
    r = mod_est((int64_t)(x - (uint64_t)qd * d), d, rd, &qd);
    q = (q << steps[k]) | (uint64_t)qd;
  }
  return q;
}

constexpr int BBP_THREADS = 256;
constexpr uint64_t CHUNK_TERMS = 1ull << 16;  // terms per work item (256 per thread)
constexpr uint32_t POLL_CHUNKS = 16;          // stop flag read every 16 items per warp

// Persistent grid over equal work items: item c is chunk c - first[p] of
// pair p = (position p / 4, series j_(p mod 4)), i.e. terms
// k in [CHUNK_TERMS (c - first[p]), min(+CHUNK_TERMS, n + 1)), with
// first[] the prefix sums of the pairs' chunk counts (first[npairs] =
// total).  Positions uniform in [0, 8e8) make the pairs' term counts differ
// by orders of magnitude; equal items keep every SM busy to the end.  Each
// warp adds its wrapping partial sum to sums[p] with one 64-bit atomic
// (wrapping addition is associative, so the bits do not depend on order).
__global__ void __launch_bounds__(BBP_THREADS)
k_bbp_series(const uint64_t* __restrict__ pos, uint32_t npairs, const uint64_t* __restrict__ first,
             unsigned long long* __restrict__ sums, const volatile int* stop, int* status) {
  const uint32_t js[4] = {1, 4, 5, 6};
  const uint64_t total = first[npairs];
  const unsigned lane = threadIdx.x & 31;
  uint32_t iter = 0;
  for (uint64_t c = blockIdx.x; c < total; c += gridDim.x, iter++) {
    if (stop && iter % POLL_CHUNKS == 0) {
      int s = 0;
      if (lane == 0) s = *stop;
      if (__shfl_sync(0xFFFFFFFFu, s, 0)) {
        if (lane == 0) *status = 1;
        return;
      }
    }
    // the pair of item c: the last p with first[p] <= c
    uint32_t lo = 0, hi = npairs;
    while (hi - lo > 1) {
      const uint32_t mid = (lo + hi) >> 1;
      if (first[mid] <= c) lo = mid;
      else hi = mid;
    }
    const uint64_t n = pos[lo >> 2], j = js[lo & 3];
    const uint64_t k0 = (c - first[lo]) * CHUNK_TERMS;
    const uint64_t k1 = min(k0 + CHUNK_TERMS, n + 1);
    uint64_t acc = 0;
    for (uint64_t k = k0 + threadIdx.x; k < k1; k += BBP_THREADS) acc += bbp_term(n - k, 8 * k + j);
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xFFFFFFFFu, acc, o);
    if (lane == 0 && acc) atomicAdd(sums + lo, (unsigned long long)acc);
  }
}

// f64 tail of series j at n, operation for operation as bbp.rs:100-115.
__device__ uint64_t tail_fixed(uint64_t n, uint64_t j) {
  double tail = 0.0;
  double factor = 1.0;
  for (int off = 1; off <= 20; off++) {
    factor = __dmul_rn(factor, 16.0);  // 16^off, exact
    uint64_t k = n + (uint64_t)off;
    double denom = (double)(8 * k + j);
    double term = __ddiv_rn(1.0, __dmul_rn(factor, denom));
    if (term == 0.0) break;
    tail = __dadd_rn(tail, term);
  }
  return __double2ull_rz(__dmul_rn(tail, 18446744073709551616.0));
}

__global__ void k_bbp_combine(const uint64_t* __restrict__ pos, uint32_t npos, const uint64_t* __restrict__ sums,
                              uint32_t* __restrict__ digits) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npos) return;
  const uint64_t n = pos[i];
  uint64_t s1 = sums[4 * i + 0] + tail_fixed(n, 1);
  uint64_t s4 = sums[4 * i + 1] + tail_fixed(n, 4);
  uint64_t s5 = sums[4 * i + 2] + tail_fixed(n, 5);
  uint64_t s6 = sums[4 * i + 3] + tail_fixed(n, 6);
  uint64_t c = 4 * s1 - 2 * s4 - s5 - s6;  // bbp.rs:70-73, wrapping
  digits[i] = (uint32_t)(c >> 32);
}

// The reference's building blocks for given (e, d, p), 16^e mod d and
// floor(p 2^64 / d), each on its own (the series kernel fuses them in
// bbp_term); for checking.
__global__ void k_bbp_modops(const uint64_t* e, const uint64_t* d, const uint64_t* p, uint32_t n, uint64_t* pw,
                             uint64_t* fr) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  pw[i] = pow16_mod(e[i], d[i]);
  fr[i] = frac64(p[i], d[i]);
}

__global__ void k_bbp_terms(const uint64_t* e, const uint64_t* d, uint32_t n, uint64_t* out) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = bbp_term(e[i], d[i]);
}

}  // namespace pimul_bbp

using namespace pimul_bbp;

#define BCU(call)                                                                        \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess) { rc = fail(PIMUL_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); goto done; } \
  } while (0)

extern "C" const char* pimul_bbp_last_error(void) { return t_err.c_str(); }

// 16^e[i] mod d[i] and floor(p[i] 2^64 / d[i]) on the device (d < 2^34,
// p < d): the modular building blocks of the extractor, for checking.
extern "C" int pimul_bbp_modops(const uint64_t* e, const uint64_t* d, const uint64_t* p, size_t n, uint64_t* pow16,
                                uint64_t* frac) {
  if (n == 0) return PIMUL_OK;
  if (!e || !d || !p || !pow16 || !frac) return fail(PIMUL_EINVAL, "null pointer");
  for (size_t i = 0; i < n; i++)
    if (d[i] == 0 || d[i] >= (1ull << 34) || p[i] >= d[i]) return fail(PIMUL_EINVAL, "need 1 <= d < 2^34, p < d");
  int rc = PIMUL_OK;
  uint64_t* buf = nullptr;
  BCU(cudaMalloc((void**)&buf, 5 * n * 8));
  BCU(cudaMemcpy(buf, e, n * 8, cudaMemcpyHostToDevice));
  BCU(cudaMemcpy(buf + n, d, n * 8, cudaMemcpyHostToDevice));
  BCU(cudaMemcpy(buf + 2 * n, p, n * 8, cudaMemcpyHostToDevice));
  k_bbp_modops<<<(unsigned)((n + 255) / 256), 256>>>(buf, buf + n, buf + 2 * n, (uint32_t)n, buf + 3 * n, buf + 4 * n);
  BCU(cudaGetLastError());
  BCU(cudaMemcpy(pow16, buf + 3 * n, n * 8, cudaMemcpyDeviceToHost));
  BCU(cudaMemcpy(frac, buf + 4 * n, n * 8, cudaMemcpyDeviceToHost));
done:
  if (buf) cudaFree(buf);
  return rc;
}

// floor((16^e[i] mod d[i]) 2^64 / d[i]) on the device, the term the
// series kernel sums (d < 2^34, e < 2^40), for checking.
extern "C" int pimul_bbp_terms(const uint64_t* e, const uint64_t* d, size_t n, uint64_t* out) {
  if (n == 0) return PIMUL_OK;
  if (!e || !d || !out) return fail(PIMUL_EINVAL, "null pointer");
  if (n > (1u << 30)) return fail(PIMUL_EINVAL, "too many terms for one call");
  for (size_t i = 0; i < n; i++)
    if (d[i] == 0 || d[i] >= (1ull << 34) || e[i] >= (1ull << 40)) return fail(PIMUL_EINVAL, "need 1 <= d < 2^34, e < 2^40");
  int rc = PIMUL_OK;
  uint64_t* buf = nullptr;
  BCU(cudaMalloc((void**)&buf, 3 * n * 8));
  BCU(cudaMemcpy(buf, e, n * 8, cudaMemcpyHostToDevice));
  BCU(cudaMemcpy(buf + n, d, n * 8, cudaMemcpyHostToDevice));
  k_bbp_terms<<<(unsigned)((n + 255) / 256), 256>>>(buf, buf + n, (uint32_t)n, buf + 2 * n);
  BCU(cudaGetLastError());
  BCU(cudaMemcpy(out, buf + 2 * n, n * 8, cudaMemcpyDeviceToHost));
done:
  if (buf) cudaFree(buf);
  return rc;
}

// Batched hex digits: digits[i] = 8 hex digits of pi at positions[i].
extern "C" int pimul_bbp_hex_digits(const uint64_t* positions, size_t count, uint32_t* digits,
                                    const volatile int* stop) {
  if (count == 0) return PIMUL_OK;
  if (!positions || !digits) return fail(PIMUL_EINVAL, "null pointer");
  if (count > (1u << 28)) return fail(PIMUL_EINVAL, "too many positions for one call (max 2^28)");
  for (size_t i = 0; i < count; i++)
    if (positions[i] > (1ull << 31)) return fail(PIMUL_EINVAL, "position above 2^31 (modulus would exceed 2^34)");
  int rc = PIMUL_OK;
  cudaStream_t st = nullptr;
  uint64_t* d_pos = nullptr;
  uint64_t* d_sums = nullptr;
  uint64_t* d_first = nullptr;
  std::vector<uint64_t> first;
  uint32_t* d_dig = nullptr;
  int* h_flag = nullptr;
  int* d_flag = nullptr;
  int* h_status = nullptr;
  int* d_status = nullptr;
  BCU(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  BCU(cudaMallocAsync((void**)&d_pos, count * 8, st));
  BCU(cudaMallocAsync((void**)&d_sums, count * 4 * 8, st));
  BCU(cudaMallocAsync((void**)&d_dig, count * 4, st));
  BCU(cudaHostAlloc((void**)&h_flag, sizeof(int), cudaHostAllocMapped));
  BCU(cudaHostAlloc((void**)&h_status, sizeof(int), cudaHostAllocMapped));
  *h_flag = 0;
  *h_status = 0;
  BCU(cudaHostGetDevicePointer((void**)&d_flag, h_flag, 0));
  BCU(cudaHostGetDevicePointer((void**)&d_status, h_status, 0));
  {
    // work items: chunks of CHUNK_TERMS terms per (position, series) pair
    first.resize(4 * count + 1);
    first[0] = 0;
    for (size_t p = 0; p < 4 * count; p++)
      first[p + 1] = first[p] + (positions[p / 4] + 1 + CHUNK_TERMS - 1) / CHUNK_TERMS;
    int dev = 0, sms = 0, per_sm = 0;
    BCU(cudaGetDevice(&dev));
    BCU(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    BCU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bbp_series, BBP_THREADS, 0));
    const uint64_t grid = std::max<uint64_t>(1, std::min<uint64_t>(first.back(), (uint64_t)sms * std::max(per_sm, 1)));
    BCU(cudaMallocAsync((void**)&d_first, first.size() * 8, st));
    BCU(cudaMemcpyAsync(d_pos, positions, count * 8, cudaMemcpyHostToDevice, st));
    BCU(cudaMemcpyAsync(d_first, first.data(), first.size() * 8, cudaMemcpyHostToDevice, st));
    BCU(cudaMemsetAsync(d_sums, 0, count * 4 * 8, st));
    k_bbp_series<<<(unsigned)grid, BBP_THREADS, 0, st>>>(d_pos, (uint32_t)(4 * count), d_first,
                                                         (unsigned long long*)d_sums,
                                                         stop ? (const volatile int*)d_flag : nullptr, d_status);
  }
  k_bbp_combine<<<(unsigned)((count + 255) / 256), 256, 0, st>>>(d_pos, (uint32_t)count, d_sums, d_dig);
  BCU(cudaGetLastError());
  // Wait, forwarding the caller's stop flag to the kernels (bounded sleep
  // steps; the kernels only read the flag).
  while (true) {
    cudaError_t q = cudaStreamQuery(st);
    if (q == cudaSuccess) break;
    if (q != cudaErrorNotReady) BCU(q);
    if (stop && *stop) *(volatile int*)h_flag = 1;
    std::this_thread::sleep_for(std::chrono::microseconds(200));
  }
  if (*(volatile int*)h_status) {
    rc = fail(PIMUL_ECANCELED, "stopped by the caller's flag");
    goto done;
  }
  BCU(cudaMemcpyAsync(digits, d_dig, count * 4, cudaMemcpyDeviceToHost, st));
  BCU(cudaStreamSynchronize(st));
done:
  if (st) cudaStreamSynchronize(st);
  if (d_pos) cudaFreeAsync(d_pos, st);
  if (d_sums) cudaFreeAsync(d_sums, st);
  if (d_first) cudaFreeAsync(d_first, st);
  if (d_dig) cudaFreeAsync(d_dig, st);
  if (st) {
    cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
  }
  if (h_flag) cudaFreeHost(h_flag);
  if (h_status) cudaFreeHost(h_status);
  return rc;
}
