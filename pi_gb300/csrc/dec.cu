// Decimal conversion with its nodes in HBM.
//
// The level-synchronous divide and conquer of the batched pi pipeline: every
// node x of level k (x < P_(k+1) = P_k^2, P_k = 10^(19 * 2^k)) splits into
// x div P_k and x mod P_k, all nodes of a level at once, from the top level
// down to leaves below 10^608, which a kernel prints.  An integer has one
// decimal string, so the output equals the reference's recursive conversion
// (crates/bignum/src/integer.rs:892-983, 10^19 chunks at integer.rs:887-888).
//
// Per level, with V = a reciprocal of P no larger than floor(2^sh / P):
//   q = (x_hi V) >> (sh - 64 t)    pimul_mul_batch + a shift kernel, where
//                         x_hi = x >> 64 t drops the t = |P| - 2 low limbs
//                         (they move x / P by less than 2^-64): a product
//                         of 2|P| + 5 limbs instead of 3|P|, half the
//                         transform length; q <= x div P
//   r = x - q P           pimul_mul_batch + pimul_addsub_batch (PIMUL_SUB_MOD:
//                         only the low |P| + 1 limbs, which hold r < 2P)
//   while r >= P: r -= P, q += 1    compare kernels; the host reads a count
// With V the exact floor at the top level and chained below it (see
// pi_host.cpp make_dec_plan), the estimate before the floor is below x / P
// by less than 2^-62, so the correction runs only when x / P falls that
// close above an integer; it is bounded at three rounds.
//
// Slots: the outputs of level k are 2n nodes of w = |P_k| + 1 limbs, q at
// slot 2i and r at slot 2i + 1 (the digit order), zero-padded.  The leaves
// (w = 33 limbs, 32 chunks of 19 digits) are printed one node per thread
// into shared memory and stored as 16-byte vectors.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../include/pimul.h"
#include "dec.h"
#include "hostcopy.h"

namespace pidec {
namespace {

constexpr uint64_t CHUNK = 10000000000000000000ull;  // 10^19, bit 63 set
constexpr int LEAF_CH = 1 << LEAF_K;                 // chunks per leaf
constexpr int LEAF_W = LEAF_CH + 1;                  // leaf slot: |10^608| = 32 limbs, plus one
constexpr int LEAF_DIGITS = 19 * LEAF_CH;            // 608 (a multiple of 16)
constexpr int LEAF_THREADS = 64;
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

// dst slot j = bits [sh + 64 j, sh + 64 j + 64) of src slot (zero past src_len).
__global__ void k_shr_slots(const uint64_t* __restrict__ src, uint64_t src_stride, uint64_t src_len, uint64_t sh,
                            uint64_t* __restrict__ dst, uint64_t dst_stride, uint64_t dst_len, uint64_t n) {
  const uint64_t ws = sh >> 6;
  const unsigned bs = (unsigned)(sh & 63);
  for (uint64_t node = blockIdx.y; node < n; node += gridDim.y) {
    const uint64_t* s = src + node * src_stride;
    uint64_t* d = dst + node * dst_stride;
    for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < dst_len;
         j += (uint64_t)gridDim.x * blockDim.x) {
      const uint64_t i = ws + j;
      const uint64_t lo = i < src_len ? s[i] : 0;
      const uint64_t hi = i + 1 < src_len ? s[i + 1] : 0;
      d[j] = bs ? (lo >> bs) | (hi << (64 - bs)) : lo;
    }
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

// Leaves (slots of LEAF_W limbs, values below 10^608) to LEAF_DIGITS
// characters each: 32 divisions by 10^19 per node in registers, the digits
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

int to_decimal_device(const uint64_t* x, size_t nx, int K, const Level* lv, char* out, size_t want, double* ms) {
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
  // divisors and reciprocals, one buffer
  std::vector<size_t> poff(K), voff(K);
  size_t pv = 0;
  for (int k = LEAF_K; k < K; k++) {
    if (!lv[k].P || !lv[k].V || !lv[k].lp || !lv[k].lv) return PIMUL_EINVAL;
    poff[k] = pv, pv += lv[k].lp;
    voff[k] = pv, pv += lv[k].lv;
  }
  uint64_t* dpv = nullptr;
  uint64_t* cur = nullptr;
  uint64_t* one = nullptr;
  if ((rc = A.get(&dpv, pv)) || (rc = A.get(&cur, nx)) || (rc = A.get(&one, 1))) return rc;
  for (int k = LEAF_K; k < K && !rc; k++) {
    rc = pimul::host_to_device(dpv + poff[k], lv[k].P, lv[k].lp * 8, st);
    if (!rc) rc = pimul::host_to_device(dpv + voff[k], lv[k].V, lv[k].lv * 8, st);
  }
  if (!rc) rc = pimul::host_to_device(cur, x, nx * 8, st);
  const uint64_t one_h = 1;
  cu(cudaMemcpyAsync(one, &one_h, 8, cudaMemcpyHostToDevice, st));
  cu(cudaStreamSynchronize(st));  // one_h is on this stack frame
  if (rc) return rc;
  double t1 = now_ms();
  size_t n = 1, w_in = nx;
  std::vector<pimul_job> jobs;
  std::vector<pimul_addsub_job> aj;
  std::vector<uint8_t> hflag;
  for (int k = K - 1; k >= LEAF_K && !rc; k--) {
    const Level& L = lv[k];
    const uint64_t* dP = dpv + poff[k];
    const uint64_t* dV = dpv + voff[k];
    // t low limbs of x left out of the quotient estimate (x_hi keeps one)
    const size_t t = std::min(L.lp >= 3 ? L.lp - 2 : 0, w_in - 1);
    const size_t w = L.lp + 1, hi_w = w_in - t, prod_w = hi_w + L.lv, qp_w = w + L.lp;
    if (L.sh < 64 * t) return PIMUL_EINVAL;
    uint64_t *nxt = nullptr, *prod = nullptr, *qp = nullptr;
    if ((rc = A.get(&nxt, 2 * n * w)) || (rc = A.get(&prod, n * prod_w))) break;
    // q = (x_hi V) >> (sh - 64 t) into the even slots
    jobs.resize(n);
    for (size_t i = 0; i < n; i++) jobs[i] = pimul_job{cur + i * w_in + t, hi_w, dV, L.lv, prod + i * prod_w};
    if ((rc = pimul_mul_batch(jobs.data(), n, st))) break;
    k_shr_slots<<<slot_grid(w, n), 256, 0, st>>>(prod, prod_w, prod_w, L.sh - 64 * t, nxt, 2 * w, w, n);
    if (lower_q) k_lower_q<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(nxt, 2 * w, w, n);
    if (!cu(cudaGetLastError())) break;
    A.put(prod);
    // r = (x - q P) mod 2^(64 w) into the odd slots
    if ((rc = A.get(&qp, n * qp_w))) break;
    for (size_t i = 0; i < n; i++) jobs[i] = pimul_job{nxt + 2 * i * w, w, dP, L.lp, qp + i * qp_w};
    if ((rc = pimul_mul_batch(jobs.data(), n, st))) break;
    aj.resize(n);
    for (size_t i = 0; i < n; i++)
      aj[i] = pimul_addsub_job{cur + i * w_in, std::min(w_in, w), qp + i * qp_w, w, nxt + (2 * i + 1) * w, w,
                               PIMUL_SUB_MOD};
    if ((rc = pimul_addsub_batch(aj.data(), n, st))) break;
    A.put(qp);
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

}  // namespace pidec
