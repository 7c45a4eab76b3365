// Decimal conversion with its nodes in HBM.
//
// The level-synchronous divide and conquer of the batched pi pipeline: every
// node x of level k (x < P_(k+1) = P_k^2, P_k = 10^(19 * 2^k)) splits into
// x div P_k and x mod P_k, all nodes of a level at once, from the top level
// down to leaves below 10^1216, which a kernel prints.  An integer has one
// decimal string, so the output equals the reference's recursive conversion
// (crates/bignum/src/integer.rs:892-983, 10^19 chunks at integer.rs:887-888).
//
// Per level, with V = a reciprocal of P no larger than floor(2^sh / P):
//   q = (x_hi V) >> (sh - 64 t)    a strided product batch
//                         (mul_batch_strided) + a shift kernel, where
//                         x_hi = x >> 64 t drops the t = |P| - 2 low limbs
//                         (they move x / P by less than 2^-64): a product
//                         of 2|P| + 5 limbs instead of 3|P|, half the
//                         transform length; q <= x div P
//   r = x - q P           a strided product batch and a strided subtraction
//                         (addsub_strided, PIMUL_SUB_MOD: only the low
//                         |P| + 1 limbs, which hold r < 2P)
//   while r >= P: r -= P, q += 1    compare kernels; the host reads a count
// With V the exact floor at the top level and chained below it (see
// pi_host.cpp make_dec_plan), the estimate before the floor is below x / P
// by less than 2^-62, so the correction runs only when x / P falls that
// close above an integer; it is bounded at three rounds.
//
// Slots: the outputs of level k are 2n nodes of w = |P_k| + 1 limbs, q at
// slot 2i and r at slot 2i + 1 (the digit order), zero-padded.  The leaves
// (w = 65 limbs, 64 chunks of 19 digits) are printed one node per thread
// into shared memory and stored as 16-byte vectors.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../include/pimul.h"
#include "dec.h"
#include "hostcopy.h"
#include "wrapmul.h"

namespace pidec {
namespace {

constexpr uint64_t CHUNK = 10000000000000000000ull;  // 10^19, bit 63 set
constexpr int LEAF_CH = 1 << LEAF_K;                 // chunks per leaf
constexpr int LEAF_W = LEAF_CH + 1;                  // leaf slot: |10^1216| = 64 limbs, plus one
constexpr int LEAF_DIGITS = 19 * LEAF_CH;            // 1216 (a multiple of 16)
constexpr int LEAF_THREADS = 32;  // 38 KB of staged digits per CTA
static_assert(LEAF_DIGITS % 16 == 0, "leaf rows are stored as 16-byte vectors");

// floor((2^128 - 1) / 10^19) - 2^64 (Moller and Granlund, "Improved division
// by invariant integers", 2011: the reciprocal of a normalized divisor).
constexpr uint64_t CHUNK_INV = (uint64_t)((~(unsigned __int128)0) / CHUNK - ((unsigned __int128)1 << 64));

// (u1:u0) div 10^19 for u1 < 10^19 (Algorithm 4 of the same paper).
__device__ __forceinline__ uint64_t div_chunk(uint64_t u1, uint64_t u0, uint64_t& r) {
  uint64_t q0 = CHUNK_INV * u1;
  uint64_t q1 = __umul64hi(CHUNK_INV, u1);
  q0 += u0;
  q1 += u1 + 1 + (q0 < u0 ? 1 : 0);
  uint64_t rr = u0 - q1 * CHUNK;
  if (rr > q0) {
    q1--;
    rr += CHUNK;
  }
  if (rr >= CHUNK) {
    q1++;
    rr -= CHUNK;
  }
  r = rr;
  return q1;
}

// dst slot j = bits [sh + 64 j, sh + 64 j + 64) of src slot, bits outside
// [0, 64 src_len) reading as zero (sh < 0 shifts left).
__global__ void k_shr_slots(const uint64_t* __restrict__ src, uint64_t src_stride, uint64_t src_len, int64_t sh,
                            uint64_t* __restrict__ dst, uint64_t dst_stride, uint64_t dst_len, uint64_t n) {
  const int64_t ws = sh >> 6;  // floor
  const unsigned bs = (unsigned)(sh & 63);
  for (uint64_t node = blockIdx.y; node < n; node += gridDim.y) {
    const uint64_t* s = src + node * src_stride;
    uint64_t* d = dst + node * dst_stride;
    for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < dst_len;
         j += (uint64_t)gridDim.x * blockDim.x) {
      const int64_t i = ws + (int64_t)j;
      const uint64_t lo = i >= 0 && (uint64_t)i < src_len ? s[i] : 0;
      const uint64_t hi = i + 1 >= 0 && (uint64_t)(i + 1) < src_len ? s[i + 1] : 0;
      d[j] = bs ? (lo >> bs) | (hi << (64 - bs)) : lo;
    }
  }
}

// lo[i] = low word of x[i] a, hi[i + 1] = high word (lo[n] = hi[0] = 0):
// x a = lo + hi with one addition.
__global__ void k_mul_small_split(const uint64_t* __restrict__ x, uint64_t n, uint64_t a, uint64_t* __restrict__ lo,
                                  uint64_t* __restrict__ hi) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= n; i += (uint64_t)gridDim.x * blockDim.x) {
    lo[i] = i < n ? x[i] * a : 0;
    hi[i] = i > 0 ? __umul64hi(x[i - 1], a) : 0;
  }
}

// top[node] = 1 + the highest limb where r and P (zero-extended) differ;
// top must be zero on entry.
__global__ void k_cmp_top(const uint64_t* __restrict__ r, uint64_t r_stride, uint64_t w,
                          const uint64_t* __restrict__ P, uint64_t lp, uint64_t n, unsigned long long* top) {
  for (uint64_t node = blockIdx.y; node < n; node += gridDim.y) {
    const uint64_t* a = r + node * r_stride;
    uint64_t best = 0;
    for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < w; j += (uint64_t)gridDim.x * blockDim.x)
      if (a[j] != (j < lp ? P[j] : 0)) best = j + 1;
    for (int o = 16; o > 0; o >>= 1) {
      const uint64_t other = __shfl_down_sync(0xFFFFFFFFu, best, o);
      best = other > best ? other : best;
    }
    if ((threadIdx.x & 31) == 0 && best) atomicMax(&top[node], (unsigned long long)best);
  }
}

// flag[node] = (r >= P); count += flags.
__global__ void k_cmp_flag(const uint64_t* __restrict__ r, uint64_t r_stride, const uint64_t* __restrict__ P,
                           uint64_t lp, uint64_t n, const unsigned long long* __restrict__ top,
                           uint8_t* __restrict__ flag, unsigned int* count) {
  const uint64_t node = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (node >= n) return;
  const uint64_t t = top[node];
  bool ge = true;  // equal
  if (t) {
    const uint64_t j = t - 1;
    ge = r[node * r_stride + j] > (j < lp ? P[j] : 0);
  }
  flag[node] = ge ? 1 : 0;
  if (ge) atomicAdd(count, 1u);
}

// Test hook: q -= 1 for every nonzero q (one thread per node), so that every
// remainder needs the correction.
__global__ void k_lower_q(uint64_t* q, uint64_t stride, uint64_t w, uint64_t n) {
  const uint64_t node = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (node >= n) return;
  uint64_t* a = q + node * stride;
  uint64_t j = 0;
  while (j < w && a[j] == 0) j++;
  if (j == w) return;
  a[j] -= 1;
  for (uint64_t i = 0; i < j; i++) a[i] = ~0ull;
}

// Nineteen digits of v < 10^19 at p[0..19).
__device__ __forceinline__ void put19(char* p, uint64_t v) {
  const uint64_t hi = v / 1000000000000ull;  // < 10^7
  const uint64_t lo = v - hi * 1000000000000ull;
  uint32_t a = (uint32_t)hi, b = (uint32_t)(lo / 1000000u), c = (uint32_t)(lo % 1000000u);
#pragma unroll
  for (int i = 6; i >= 0; i--) {
    p[i] = (char)('0' + a % 10u);
    a /= 10u;
  }
#pragma unroll
  for (int i = 12; i >= 7; i--) {
    p[i] = (char)('0' + b % 10u);
    b /= 10u;
  }
#pragma unroll
  for (int i = 18; i >= 13; i--) {
    p[i] = (char)('0' + c % 10u);
    c /= 10u;
  }
}

// Leaves (slots of LEAF_W limbs, values below 10^1216) to LEAF_DIGITS
// characters each: 64 divisions by 10^19 per node in registers, the digits
// staged in shared memory and stored as 16-byte vectors.
__global__ void __launch_bounds__(LEAF_THREADS) k_dec_leaves(const uint64_t* __restrict__ nodes, uint64_t n,
                                                             char* __restrict__ out) {
  __shared__ __align__(16) char buf[LEAF_THREADS * LEAF_DIGITS];
  const uint64_t first = (uint64_t)blockIdx.x * LEAF_THREADS;
  const uint64_t node = first + threadIdx.x;
  if (node < n) {
    uint64_t x[LEAF_W];
    const uint64_t* s = nodes + node * LEAF_W;
#pragma unroll
    for (int j = 0; j < LEAF_W; j++) x[j] = s[j];
    char* my = buf + threadIdx.x * LEAF_DIGITS;
#pragma unroll 1
    for (int c = 0; c < LEAF_CH; c++) {
      uint64_t r = 0;
#pragma unroll
      for (int j = LEAF_W - 1; j >= 0; j--) x[j] = div_chunk(r, x[j], r);
      put19(my + LEAF_DIGITS - 19 * (c + 1), r);
    }
  }
  __syncthreads();
  const uint64_t cnt = n - first < (uint64_t)LEAF_THREADS ? n - first : (uint64_t)LEAF_THREADS;
  const uint64_t vecs = cnt * LEAF_DIGITS / 16;
  uint4* dst = reinterpret_cast<uint4*>(out + first * LEAF_DIGITS);
  const uint4* src = reinterpret_cast<const uint4*>(buf);
  for (uint64_t i = threadIdx.x; i < vecs; i += LEAF_THREADS) dst[i] = src[i];
}

// *bad = 1 if any of s[0..len) is not '0'.
__global__ void k_zero_prefix(const char* __restrict__ s, uint64_t len, int* bad) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += (uint64_t)gridDim.x * blockDim.x)
    if (s[i] != '0') *bad = 1;
}

double now_ms() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

dim3 slot_grid(uint64_t len, uint64_t n) {
  const uint64_t bx = std::min<uint64_t>((len + 255) / 256, 1u << 20);
  const uint64_t by = std::min<uint64_t>(n, 65535);
  return dim3((unsigned)std::max<uint64_t>(bx, 1), (unsigned)std::max<uint64_t>(by, 1));
}

// Device allocations of one conversion, freed on the stream at the end.
struct Arena {
  cudaStream_t st = nullptr;
  std::vector<void*> live;
  ~Arena() {
    for (void* p : live) cudaFreeAsync(p, st);
    if (st) {
      cudaStreamSynchronize(st);
      cudaStreamDestroy(st);
    }
  }
  template <class T>
  int get(T** p, size_t count) {
    *p = nullptr;
    if (cudaMallocAsync((void**)p, std::max<size_t>(count, 1) * sizeof(T), st) != cudaSuccess) {
      cudaGetLastError();
      return PIMUL_ENOMEM;
    }
    live.push_back(*p);
    return PIMUL_OK;
  }
  void put(void* p) {
    auto it = std::find(live.begin(), live.end(), p);
    if (it == live.end()) return;
    live.erase(it);
    cudaFreeAsync(p, st);
  }
};

}  // namespace

int to_decimal_device(const uint64_t* x, size_t nx, bool x_on_device, int K, const Level* lv, bool lv_on_device,
                      char* out, size_t want, double* ms) {
  if (!x || !nx || !lv || !out || K <= LEAF_K || K > 40) return PIMUL_EINVAL;
  if (lv[LEAF_K].lp + 1 != (size_t)LEAF_W) return PIMUL_EINVAL;
  const size_t total = (size_t)19 << K;
  if (want > total) return PIMUL_EINVAL;
  const bool lower_q = getenv("PIMUL_DEC_TEST_LOWER_Q") != nullptr;
  double t0 = now_ms();
  Arena A;
  if (cudaStreamCreateWithFlags(&A.st, cudaStreamNonBlocking) != cudaSuccess) return PIMUL_ECUDA;
  const cudaStream_t st = A.st;
  int rc = PIMUL_OK;
  auto cu = [&](cudaError_t e) {
    if (e != cudaSuccess && !rc) rc = e == cudaErrorMemoryAllocation ? PIMUL_ENOMEM : PIMUL_ECUDA;
    return rc == PIMUL_OK;
  };
  // divisors and reciprocals: in place on the device, or uploaded into one buffer
  std::vector<size_t> poff(K), voff(K);
  std::vector<const uint64_t*> dPk(K, nullptr), dVk(K, nullptr);
  size_t pv = 0;
  for (int k = LEAF_K; k < K; k++) {
    if (!lv[k].P || !lv[k].V || !lv[k].lp || !lv[k].lv) return PIMUL_EINVAL;
    poff[k] = pv, pv += lv[k].lp;
    voff[k] = pv, pv += lv[k].lv;
  }
  uint64_t* dpv = nullptr;
  uint64_t* cur = nullptr;
  uint64_t* one = nullptr;
  if ((!lv_on_device && (rc = A.get(&dpv, pv))) || (rc = A.get(&cur, nx)) || (rc = A.get(&one, 1))) return rc;
  for (int k = LEAF_K; k < K && !rc; k++) {
    if (lv_on_device) {
      dPk[k] = lv[k].P;
      dVk[k] = lv[k].V;
      continue;
    }
    rc = pimul::host_to_device(dpv + poff[k], lv[k].P, lv[k].lp * 8, st);
    if (!rc) rc = pimul::host_to_device(dpv + voff[k], lv[k].V, lv[k].lv * 8, st);
    dPk[k] = dpv + poff[k];
    dVk[k] = dpv + voff[k];
  }
  if (!rc && x_on_device) cu(cudaMemcpyAsync(cur, x, nx * 8, cudaMemcpyDeviceToDevice, st));
  if (!rc && !x_on_device) rc = pimul::host_to_device(cur, x, nx * 8, st);
  const uint64_t one_h = 1;
  cu(cudaMemcpyAsync(one, &one_h, 8, cudaMemcpyHostToDevice, st));
  cu(cudaStreamSynchronize(st));  // one_h is on this stack frame
  if (rc) return rc;
  double t1 = now_ms();
  size_t n = 1, w_in = nx;
  std::vector<pimul_addsub_job> aj;
  std::vector<uint8_t> hflag;
  const bool timing = getenv("PIMUL_PI_TIMING") != nullptr;
  for (int k = K - 1; k >= LEAF_K && !rc; k--) {
    const double tl0 = timing ? now_ms() : 0;
    double tl_launch = 0;
    const Level& L = lv[k];
    const uint64_t* dP = dPk[k];
    const uint64_t* dV = dVk[k];
    // t low limbs of x left out of the quotient estimate (x_hi keeps one)
    const size_t t = std::min(L.lp >= 3 ? L.lp - 2 : 0, w_in - 1);
    const size_t w = L.lp + 1, hi_w = w_in - t, prod_w = hi_w + L.lv, qp_w = w + L.lp;
    if (L.sh < 64 * t) return PIMUL_EINVAL;
    uint64_t *nxt = nullptr, *prod = nullptr, *qp = nullptr;
    if ((rc = A.get(&nxt, 2 * n * w)) || (rc = A.get(&prod, n * prod_w))) break;
    // q = (x_hi V) >> (sh - 64 t) into the even slots
    if ((rc = pimul::mul_batch_strided(cur + t, w_in, hi_w, dV, L.lv, prod, prod_w, n, st))) break;
    k_shr_slots<<<slot_grid(w, n), 256, 0, st>>>(prod, prod_w, prod_w, (int64_t)(L.sh - 64 * t), nxt, 2 * w, w,
                                                 n);
    if (lower_q) k_lower_q<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(nxt, 2 * w, w, n);
    if (!cu(cudaGetLastError())) break;
    A.put(prod);
    // r = (x - q P) mod 2^(64 w) into the odd slots
    if ((rc = A.get(&qp, n * qp_w))) break;
    if ((rc = pimul::mul_batch_strided(nxt, 2 * w, w, dP, L.lp, qp, qp_w, n, st))) break;
    if ((rc = pimul::addsub_strided(cur, w_in, std::min(w_in, w), qp, qp_w, w, nxt + w, 2 * w, w, PIMUL_SUB_MOD, n,
                                    st)))
      break;
    A.put(qp);
    if (timing) tl_launch = now_ms() - tl0;
    // while r >= P: r -= P, q += 1
    unsigned long long* top = nullptr;
    uint8_t* flag = nullptr;
    unsigned int* count = nullptr;
    if ((rc = A.get(&top, n)) || (rc = A.get(&flag, n)) || (rc = A.get(&count, 1))) break;
    for (int round = 0; !rc; round++) {
      cu(cudaMemsetAsync(top, 0, n * 8, st));
      cu(cudaMemsetAsync(count, 0, 4, st));
      k_cmp_top<<<slot_grid(w, n), 256, 0, st>>>(nxt + w, 2 * w, w, dP, L.lp, n, top);
      k_cmp_flag<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(nxt + w, 2 * w, dP, L.lp, n, top, flag, count);
      unsigned int h_count = 0;
      cu(cudaGetLastError());
      cu(cudaMemcpyAsync(&h_count, count, 4, cudaMemcpyDeviceToHost, st));
      cu(cudaStreamSynchronize(st));
      if (rc || h_count == 0) break;
      if (round == 3) {
        rc = PIMUL_EINVAL;  // the reciprocal is not within a unit: not a valid plan
        break;
      }
      hflag.resize(n);
      cu(cudaMemcpyAsync(hflag.data(), flag, n, cudaMemcpyDeviceToHost, st));
      cu(cudaStreamSynchronize(st));
      if (rc) break;
      aj.clear();
      for (size_t i = 0; i < n; i++) {
        if (!hflag[i]) continue;
        uint64_t* q = nxt + 2 * i * w;
        uint64_t* r = q + w;
        aj.push_back(pimul_addsub_job{r, w, dP, L.lp, r, w, 1});
        aj.push_back(pimul_addsub_job{q, w, one, 1, q, w, 0});
      }
      rc = pimul_addsub_batch(aj.data(), aj.size(), st);
    }
    A.put(top);
    A.put(flag);
    A.put(count);
    A.put(cur);
    if (timing)
      fprintf(stderr, "[pimul]   conversion level %d: %zu nodes of %zu limbs, %.1f ms (products and subtraction queued in %.1f)\n",
              k, n, w_in, now_ms() - tl0, tl_launch);
    cur = nxt;
    n *= 2;
    w_in = w;
  }
  if (rc) return rc;
  double t2 = now_ms();
  // leaves -> characters; the leading total - want must be zeros
  char* chars = nullptr;
  int* bad = nullptr;
  if ((rc = A.get(&chars, total)) || (rc = A.get(&bad, 1))) return rc;
  cu(cudaMemsetAsync(bad, 0, sizeof(int), st));
  k_dec_leaves<<<(unsigned)((n + LEAF_THREADS - 1) / LEAF_THREADS), LEAF_THREADS, 0, st>>>(cur, n, chars);
  const size_t skip = total - want;
  if (skip)
    k_zero_prefix<<<(unsigned)std::min<size_t>((skip + 255) / 256, 152 * 16), 256, 0, st>>>(chars, skip, bad);
  cu(cudaGetLastError());
  int h_bad = 0;
  cu(cudaMemcpyAsync(&h_bad, bad, sizeof(int), cudaMemcpyDeviceToHost, st));
  cu(cudaStreamSynchronize(st));
  if (rc) return rc;
  if (h_bad) return PIMUL_EINVAL;
  if ((rc = pimul::device_to_host(out, chars + skip, want, st))) return rc;
  if (ms) {
    ms[0] = t1 - t0;
    ms[1] = t2 - t1;
    ms[2] = now_ms() - t2;
  }
  return PIMUL_OK;
}


// ---------------------------------------------------------- final assembly
// pi 10^(D-1) = W Q / (A Q - |T|) with W = 426880 sqrt(10005) 10^(D-1)
// (chudnovsky.rs:146-204 followed by util.rs:25-83's scaling), from the
// binary splitting's root Q and |T| where they lie in HBM:
//   den = top limbs of A Q - |T|, normalized to nl = ceil((prec + 192) / 64)
//         limbs with the top bit set (den ~ dn 2^ed);
//   R   ~ 2^(128 nl) / dn by Newton's iteration with precision doubling,
//         each step from h = 64m to c = 64m' bits (m' = min(2m - 1, nl)):
//           E = 2^(h+c) - D_c Y_h    (D_c = the top m' limbs of dn; E >= 0)
//           Y_c = Y_h 2^(c-h) + floor(Y_h E / 2^(2h)) - 4
//         Y stays at or below rho 2^h (rho = 2^(64 nl) / dn): E needs only
//         the low m' + 1 limbs of -D_c Y_h, and the -4 covers the
//         truncation of D_c (at most 4 units of Y_c);
//   ip  = floor(W Q_top R 2^e), Q_top = the top nl limbs of Q.
namespace {

// floor(2^(64 s) / d) for a small host divisor d (restoring division).
std::vector<uint64_t> host_recip_pow2(const std::vector<uint64_t>& d, size_t s) {
  const size_t nd = d.size();
  std::vector<uint64_t> q(s + 1, 0), r(nd + 1, 0);
  for (size_t bit = 64 * s + 1; bit-- > 0;) {
    // r = 2 r + (bit == 64 s)
    uint64_t carry = bit == 64 * s ? 1 : 0;
    for (size_t i = 0; i <= nd; i++) {
      const uint64_t nc = r[i] >> 63;
      r[i] = (r[i] << 1) | carry;
      carry = nc;
    }
    // r >= d ?
    int c = r[nd] ? 1 : 0;
    for (size_t i = nd; c == 0 && i-- > 0;) c = r[i] > d[i] ? 1 : (r[i] < d[i] ? -1 : 0);
    if (c >= 0) {
      uint64_t borrow = 0;
      for (size_t i = 0; i <= nd; i++) {
        const uint64_t di = i < nd ? d[i] : 0;
        const uint64_t t = r[i] - di;
        const uint64_t b1 = r[i] < di, b2 = t < borrow;
        r[i] = t - borrow;
        borrow = b1 | b2;
      }
      q[bit >> 6] |= 1ull << (bit & 63);
    }
  }
  while (!q.empty() && q.back() == 0) q.pop_back();
  return q;
}

}  // namespace

// Y ~ 2^(128 nl) / dn for dn = dnorm[0..nl) (device, top bit set, nl >= 3):
// Newton's iteration with precision doubling from Y_(64 m0) found on the
// host from the top limbs of dn; each step h -> c = 2h - 64 bits computes
// E = 2^(h+c) - D_c Y_h from the low limbs of one product and
// Y_c = Y_h 2^(c-h) + floor(Y_h E / 2^(2h)) - 4, so Y stays an underestimate
// and lands within 4 units.  *Yout (nl + 1 limbs) comes from Ar.
static int recip_newton(Arena& Ar, const uint64_t* dnorm, size_t nl, uint64_t** Yout) {
  const cudaStream_t st = Ar.st;
  int rc = PIMUL_OK;
  auto cu = [&](cudaError_t e) {
    if (e != cudaSuccess && !rc) rc = e == cudaErrorMemoryAllocation ? PIMUL_ENOMEM : PIMUL_ECUDA;
    return rc == PIMUL_OK;
  };
  *Yout = nullptr;
  if (nl < 3) return PIMUL_EINVAL;
  uint64_t* consts = nullptr;
  if ((rc = Ar.get(&consts, 1))) return rc;
  const size_t m0 = std::min<size_t>(8, nl - 2), k0 = m0 + 2;
  std::vector<uint64_t> dtop(k0);
  cu(cudaMemcpyAsync(dtop.data(), dnorm + (nl - k0), k0 * 8, cudaMemcpyDeviceToHost, st));
  cu(cudaStreamSynchronize(st));
  if (rc) return rc;
  // ceil of the truncated divisor keeps Y below rho 2^h
  for (size_t i = 0; i < k0 && ++dtop[i] == 0; i++) {
  }
  if (dtop.back() == 0) dtop.push_back(1);
  std::vector<uint64_t> y0 = host_recip_pow2(dtop, k0 + m0);
  y0.resize(m0 + 1, 0);
  uint64_t* Y = nullptr;
  if ((rc = Ar.get(&Y, m0 + 1))) return rc;
  cu(cudaMemcpyAsync(Y, y0.data(), (m0 + 1) * 8, cudaMemcpyHostToDevice, st));
  const uint64_t four = 4;
  cu(cudaMemcpyAsync(consts, &four, 8, cudaMemcpyHostToDevice, st));
  cu(cudaStreamSynchronize(st));  // y0 and four are host locals
  size_t m = m0;
  while (!rc && m < nl) {
    const size_t mp = std::min(2 * m - 1, nl);
    const uint64_t* Dc = dnorm + (nl - mp);
    uint64_t *Pr = nullptr, *E = nullptr, *YE = nullptr, *Yn = nullptr;
    if ((rc = Ar.get(&Pr, mp + m + 1)) || (rc = Ar.get(&E, mp + 1))) break;
    if ((rc = pimul::mul_wrapped(Dc, mp, Y, m + 1, Pr, st))) break;
    pimul_addsub_job je{nullptr, 0, Pr, mp + 1, E, mp + 1, PIMUL_SUB_MOD};  // E = 2^(h+c) - Pr
    if ((rc = pimul_addsub_batch(&je, 1, st))) break;
    Ar.put(Pr);
    if ((rc = Ar.get(&YE, m + mp + 2)) || (rc = Ar.get(&Yn, mp + 1))) break;
    if ((rc = pimul::mul_wrapped(Y, m + 1, E, mp + 1, YE, st))) break;
    if (mp > m) cu(cudaMemsetAsync(Yn, 0, (mp - m) * 8, st));
    cu(cudaMemcpyAsync(Yn + (mp - m), Y, (m + 1) * 8, cudaMemcpyDeviceToDevice, st));
    if (rc) break;
    pimul_addsub_job ja{Yn, mp + 1, YE + 2 * m, mp - m + 2, Yn, mp + 1, 0};
    if ((rc = pimul_addsub_batch(&ja, 1, st))) break;
    pimul_addsub_job js{Yn, mp + 1, consts, 1, Yn, mp + 1, 1};
    if ((rc = pimul_addsub_batch(&js, 1, st))) break;
    Ar.put(E);
    Ar.put(YE);
    Ar.put(Y);
    Y = Yn;
    m = mp;
  }
  Ar.put(consts);
  if (rc) return rc;
  *Yout = Y;
  return PIMUL_OK;
}

static int quotient_tail(Arena& Ar, const uint64_t* den, size_t wn, int64_t den_exp, const uint64_t* n_top, size_t lq,
                         int64_t n_exp, const uint64_t* wm, size_t wl, int64_t we, bool w_dev, uint64_t prec,
                         uint64_t** d_ip, size_t* ipn, double* ms, double t0);

int final_assembly_device(const uint64_t* dQ, size_t qn, uint64_t q_off, const uint64_t* dT, size_t tn,
                          uint64_t t_off, uint64_t A, const uint64_t* wm, size_t wl, int64_t we, bool w_dev,
                          uint64_t prec, uint64_t** d_ip, size_t* ipn, double* ms) {
  if (!dQ || !qn || (tn && !dT) || !wm || !wl || !d_ip || !ipn || !A) return PIMUL_EINVAL;
  *d_ip = nullptr;
  *ipn = 0;
  const double t0 = now_ms();
  Arena Ar;
  if (cudaStreamCreateWithFlags(&Ar.st, cudaStreamNonBlocking) != cudaSuccess) return PIMUL_ECUDA;
  const cudaStream_t st = Ar.st;
  int rc = PIMUL_OK;
  auto cu = [&](cudaError_t e) {
    if (e != cudaSuccess && !rc) rc = e == cudaErrorMemoryAllocation ? PIMUL_ENOMEM : PIMUL_ECUDA;
    return rc == PIMUL_OK;
  };
  const size_t nl = (prec + 192 + 63) / 64;
  // den window: limbs [s0, qt + 1) of A Q - |T| (qt = Q's length with its
  // offset; carries from below s0 are dropped: a relative error below
  // 2^-(64 nl)); the stored parts of Q and |T| must reach down to s0
  const size_t qt = qn + q_off, tt = tn + t_off;
  const size_t dn = qt + 1, s0 = dn > nl + 2 ? dn - (nl + 2) : 0, wn = dn - s0;
  if (tt > dn || s0 < q_off || (tt > s0 && s0 < t_off) || qn < std::min(qt, nl)) return PIMUL_EINVAL;
  uint64_t *lo = nullptr, *hi = nullptr, *den = nullptr;
  if ((rc = Ar.get(&lo, wn)) || (rc = Ar.get(&hi, wn)) || (rc = Ar.get(&den, wn))) return rc;
  k_mul_small_split<<<(unsigned)std::min<uint64_t>((wn + 255) / 256, 1u << 20), 256, 0, st>>>(
      dQ + (s0 - q_off), qt - s0, A, lo, hi);
  if (!cu(cudaGetLastError())) return rc;
  pimul_addsub_job j1{lo, wn, hi, wn, den, wn, 0};
  if ((rc = pimul_addsub_batch(&j1, 1, st))) return rc;
  if (tt > s0) {
    pimul_addsub_job j2{den, wn, dT + (s0 - t_off), tt - s0, den, wn, 1};
    if ((rc = pimul_addsub_batch(&j2, 1, st))) return rc;
  }
  Ar.put(lo);
  Ar.put(hi);
  // W Q / den with Q's top lq = min(qt, nl) limbs
  const size_t lq = std::min(qt, nl);
  return quotient_tail(Ar, den, wn, 64 * (int64_t)s0, dQ + (qn - lq), lq, 64 * (int64_t)(qt - lq), wm, wl, we, w_dev,
                       prec, d_ip, ipn, ms, t0);
}

// floor(W N / D): D = den[0..wn) 2^den_exp on the device, N = n_top[0..lq)
// 2^n_exp (lq <= nl, its top limbs), W = wm 2^we on the host (in device
// memory when w_dev).  D's top
// 64 nl bits are normalised, R ~ 2^(128 nl) / D comes from Newton's
// iteration (precision doubling from 576 bits found on the host), and the
// quotient is floor(W (N_top R >> 64 lq) 2^e).
static int quotient_tail(Arena& Ar, const uint64_t* den, size_t wn, int64_t den_exp, const uint64_t* n_top, size_t lq,
                         int64_t n_exp, const uint64_t* wm, size_t wl, int64_t we, bool w_dev, uint64_t prec,
                         uint64_t** d_ip, size_t* ipn, double* ms, double t0) {
  const cudaStream_t st = Ar.st;
  int rc = PIMUL_OK;
  auto cu = [&](cudaError_t e) {
    if (e != cudaSuccess && !rc) rc = e == cudaErrorMemoryAllocation ? PIMUL_ENOMEM : PIMUL_ECUDA;
    return rc == PIMUL_OK;
  };
  const size_t nl = (prec + 192 + 63) / 64;
  if (!den || !wn || !n_top || !lq || lq > nl || !wm || !wl || !d_ip || !ipn) return PIMUL_EINVAL;
  uint64_t* dnorm = nullptr;
  if ((rc = Ar.get(&dnorm, nl))) return rc;
  // bit length of the window, then dn = its top 64 nl bits
  uint64_t top[3] = {0, 0, 0};
  const size_t nt = std::min<size_t>(3, wn);
  cu(cudaMemcpyAsync(top, den + (wn - nt), nt * 8, cudaMemcpyDeviceToHost, st));
  cu(cudaStreamSynchronize(st));
  if (rc) return rc;
  int64_t B = 0;
  for (size_t i = nt; i-- > 0 && !B;)
    if (top[i]) B = 64 * (int64_t)(wn - nt + i) + 64 - __builtin_clzll(top[i]);
  if (B <= 64 * (int64_t)(wn - nt)) return PIMUL_EINVAL;  // the divisor vanishes in its top limbs
  const int64_t shn = B - 64 * (int64_t)nl;
  k_shr_slots<<<slot_grid(nl, 1), 256, 0, st>>>(den, 0, wn, shn, dnorm, 0, nl, 1);
  if (!cu(cudaGetLastError())) return rc;
  const int64_t ed = den_exp + shn;  // D ~ dn 2^ed
  uint64_t* Y = nullptr;
  if ((rc = recip_newton(Ar, dnorm, nl, &Y))) return rc;
  const double t1 = now_ms();
  // ip = floor(W N_top R 2^e2)
  uint64_t *X1 = nullptr, *X2 = nullptr, *dW = nullptr;
  if ((rc = Ar.get(&X1, lq + nl + 1))) return rc;
  if ((rc = pimul::mul_wrapped(n_top, lq, Y, nl + 1, X1, st))) return rc;
  Ar.put(Y);
  const uint64_t* Wd = wm;
  if (!w_dev) {
    if ((rc = Ar.get(&dW, wl)) || (rc = pimul::host_to_device(dW, wm, wl * 8, st))) return rc;
    Wd = dW;
  }
  if ((rc = Ar.get(&X2, wl + nl + 1))) return rc;
  if ((rc = pimul::mul_wrapped(Wd, wl, X1 + lq, nl + 1, X2, st))) return rc;
  // W N / D ~ X2 2^(64 lq) * 2^(we + n_exp - 128 nl - ed)
  const int64_t e2 = we + 64 * (int64_t)lq + n_exp - 128 * (int64_t)nl - ed;
  const int64_t ip_bits = 64 * (int64_t)(wl + nl + 1) + e2;
  if (e2 > 0 || ip_bits <= 0) return PIMUL_EINVAL;
  const size_t n_ip = (size_t)((ip_bits + 63) / 64);
  uint64_t* ip = nullptr;
  if (cudaMalloc((void**)&ip, n_ip * 8) != cudaSuccess) {
    cudaGetLastError();
    return PIMUL_ENOMEM;
  }
  k_shr_slots<<<slot_grid(n_ip, 1), 256, 0, st>>>(X2, 0, wl + nl + 1, -e2, ip, 0, n_ip, 1);
  cu(cudaGetLastError());
  cu(cudaStreamSynchronize(st));
  if (rc) {
    cudaFree(ip);
    return rc;
  }
  size_t len = n_ip;
  // trimmed length (the top limbs of the estimate may be zero)
  std::vector<uint64_t> tail(std::min<size_t>(n_ip, 4));
  while (len) {
    const size_t k = std::min(len, tail.size());
    if (cudaMemcpy(tail.data(), ip + (len - k), k * 8, cudaMemcpyDeviceToHost) != cudaSuccess) {
      cudaFree(ip);
      return PIMUL_ECUDA;
    }
    size_t z = 0;
    while (z < k && tail[k - 1 - z] == 0) z++;
    len -= z;
    if (z < k) break;
  }
  *d_ip = ip;
  *ipn = len;
  if (ms) {
    ms[0] = t1 - t0;
    ms[1] = now_ms() - t1;
  }
  return PIMUL_OK;
}

int quotient_device(const uint64_t* den, size_t wn, int64_t den_exp, const uint64_t* n_top, size_t lq, int64_t n_exp,
                    const uint64_t* wm, size_t wl, int64_t we, bool w_dev, uint64_t prec, uint64_t** d_ip,
                    size_t* ipn, double* ms) {
  if (!d_ip || !ipn) return PIMUL_EINVAL;
  *d_ip = nullptr;
  *ipn = 0;
  Arena Ar;
  if (cudaStreamCreateWithFlags(&Ar.st, cudaStreamNonBlocking) != cudaSuccess) return PIMUL_ECUDA;
  return quotient_tail(Ar, den, wn, den_exp, n_top, lq, n_exp, wm, wl, we, w_dev, prec, d_ip, ipn, ms, now_ms());
}

void free_levels_device(DevLevels* L) {
  if (!L) return;
  for (uint64_t* p : L->bufs) cudaFree(p);
  L->bufs.clear();
  L->lv.clear();
  L->K = 0;
}

// P_0 = 10^19, P_k = P_(k-1)^2 (exact; the length and bit count of each read
// back from its top two limbs), s_k = 2 bits(P_k) + 64.  At the top level
// T = K - 1, with nl = |P_T| + 1 limbs and dn = P_T 2^(64 nl - bits(P_T)),
// Newton's Y ~ 2^(128 nl) / dn (an underestimate within 4 units) gives
// V_T = Y >> (64 |P_T| - bits(P_T)) <= floor(2^(s_T) / P_T); below it
// V_(k-1) = (P_(k-1) V_k) >> (s_k - s_(k-1)), also an underestimate
// (P_k = P_(k-1)^2) within a few units.  A quotient estimate
// floor(x V_k / 2^(s_k)) for x < P_k^2 then falls short of x div P_k by
// less than one plus a few times 2^-64, which the conversion's correction
// rounds take.
int build_levels_device(int K, DevLevels* out, double* ms) {
  if (!out || K <= LEAF_K || K > 40) return PIMUL_EINVAL;
  free_levels_device(out);
  const double t0 = now_ms();
  Arena A;
  int prio_lo = 0, prio_hi = 0;
  cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi);
  if (cudaStreamCreateWithPriority(&A.st, cudaStreamNonBlocking, prio_hi) != cudaSuccess) return PIMUL_ECUDA;
  const cudaStream_t st = A.st;
  int rc = PIMUL_OK;
  auto cu = [&](cudaError_t e) {
    if (e != cudaSuccess && !rc) rc = e == cudaErrorMemoryAllocation ? PIMUL_ENOMEM : PIMUL_ECUDA;
    return rc == PIMUL_OK;
  };
  auto keep = [&](uint64_t** p, size_t limbs) {
    *p = nullptr;
    if (rc) return;
    if (cudaMalloc((void**)p, std::max<size_t>(limbs, 1) * 8) != cudaSuccess) {
      cudaGetLastError();
      rc = PIMUL_ENOMEM;
      return;
    }
    out->bufs.push_back(*p);
  };
  auto trimmed = [&](const uint64_t* x, size_t n) -> size_t {
    size_t len = 0;
    if (rc) return 0;
    const uint64_t* arr[1] = {x};
    size_t lens[1] = {n};
    rc = pimul_top_limbs(arr, lens, 1, &len, st);
    return len;
  };
  std::vector<uint64_t*> P(K, nullptr), V(K, nullptr);
  std::vector<size_t> lp(K, 0), lv(K, 0);
  std::vector<uint64_t> bits(K, 0), sh(K, 0);
  keep(&P[0], 1);
  const uint64_t chunk = CHUNK;
  if (!rc) cu(cudaMemcpyAsync(P[0], &chunk, 8, cudaMemcpyHostToDevice, st));
  lp[0] = 1;
  bits[0] = 64;
  for (int k = 1; k < K && !rc; k++) {
    keep(&P[k], 2 * lp[k - 1]);
    if (rc) break;
    rc = pimul_mul_device(P[k - 1], lp[k - 1], P[k - 1], lp[k - 1], P[k], st);  // a square
    uint64_t top2[2] = {0, 0};
    if (!rc) cu(cudaMemcpyAsync(top2, P[k] + 2 * lp[k - 1] - 2, 16, cudaMemcpyDeviceToHost, st));
    cu(cudaStreamSynchronize(st));
    if (rc) break;
    lp[k] = top2[1] ? 2 * lp[k - 1] : 2 * lp[k - 1] - 1;
    const uint64_t tw = top2[1] ? top2[1] : top2[0];
    bits[k] = 64 * (lp[k] - 1) + 64 - __builtin_clzll(tw);
  }
  for (int k = 0; k < K; k++) sh[k] = 2 * bits[k] + 64;
  if (rc) return rc;
  // the top level's reciprocal
  const int T = K - 1;
  const size_t nl = lp[T] + 1;
  uint64_t* dnorm = nullptr;
  if ((rc = A.get(&dnorm, nl))) return rc;
  k_shr_slots<<<slot_grid(nl, 1), 256, 0, st>>>(P[T], 0, lp[T], -(int64_t)(64 * nl - bits[T]), dnorm, 0, nl, 1);
  if (!cu(cudaGetLastError())) return rc;
  uint64_t* Y = nullptr;
  if ((rc = recip_newton(A, dnorm, nl, &Y))) return rc;
  keep(&V[T], nl + 1);
  if (rc) return rc;
  k_shr_slots<<<slot_grid(nl + 1, 1), 256, 0, st>>>(Y, 0, nl + 1, (int64_t)(64 * lp[T] - bits[T]), V[T], 0, nl + 1, 1);
  if (!cu(cudaGetLastError())) return rc;
  lv[T] = trimmed(V[T], nl + 1);
  A.put(Y);
  A.put(dnorm);
  for (int k = T - 1; k >= LEAF_K && !rc; k--) {
    const size_t pw = lp[k] + lv[k + 1];
    const uint64_t d = sh[k + 1] - sh[k];
    const size_t vw = pw - d / 64;
    uint64_t* prod = nullptr;
    if ((rc = A.get(&prod, pw))) break;
    if ((rc = pimul_mul_device(P[k], lp[k], V[k + 1], lv[k + 1], prod, st))) break;
    keep(&V[k], vw);
    if (rc) break;
    k_shr_slots<<<slot_grid(vw, 1), 256, 0, st>>>(prod, 0, pw, (int64_t)d, V[k], 0, vw, 1);
    if (!cu(cudaGetLastError())) break;
    lv[k] = trimmed(V[k], vw);
    A.put(prod);
  }
  cu(cudaStreamSynchronize(st));
  if (rc) return rc;
  out->K = K;
  out->lv.assign(K, Level{nullptr, 0, nullptr, 0, 0});
  for (int k = LEAF_K; k < K; k++) out->lv[k] = Level{P[k], lp[k], V[k], lv[k], sh[k]};
  if (ms) ms[0] = now_ms() - t0;
  return PIMUL_OK;
}

}  // namespace pidec
