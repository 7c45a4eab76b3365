// Batched BBP hex-digit extraction on sm_103a.
//
// Same result, bit for bit, as the reference's extractor
// (crates/pi-core/src/bbp.rs:52-140): for a position n it returns the top
// 32 bits of 4*S1 - 2*S4 - S5 - S6 (wrapping u64 fixed point), where
// S_j = sum_{k<=n} floor(((16^(n-k) mod d) << 64) / d) + tail_j, d = 8k+j,
// and tail_j is the f64 sum of 20 terms 1/(16^o (8(n+o)+j)) converted with
// a truncating cast.
//
// GPU design: the (position, series, k) space is flattened; every CTA owns
// one (position, series) pair and its threads stride over k.  The wrapping
// u64 sum is associative and commutative, so any split of k gives the same
// bits.  16^e mod d uses 64-bit Montgomery multiplication for the odd part
// of d (d = 8k+4 and 8k+6 are even: the power-of-two factor is restored by
// CRT).  The f64 tail uses explicitly rounded IEEE operations (no FMA
// contraction), so it matches the reference's f64 arithmetic exactly.
// A stop flag in mapped host memory is polled every 10^4 terms (like
// bbp.rs:88-92); no thread ever waits on it.
#include <cuda_runtime.h>
#include <chrono>
#include <cstdint>
#include <cstring>
#include <string>
#include <thread>

#include "../../include/pimul.h"

namespace pimul_bbp {

static thread_local std::string t_err;
static int fail(int code, const std::string& m) {
  t_err = m;
  return code;
}

// -m^-1 mod 2^64 for odd m (Newton: each step doubles the correct bits).
__device__ __forceinline__ uint64_t neg_inv64(uint64_t m) {
  uint64_t x = (3 * m) ^ 2;  // 5 correct bits
#pragma unroll
  for (int i = 0; i < 4; i++) x *= 2 - m * x;
  return 0 - x;
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

// 16^e mod d for 1 <= d < 2^34 (d == 1 -> 0, like bbp.rs:123-125).
__device__ __forceinline__ uint64_t pow16_mod(uint64_t e, uint64_t d) {
  if (d == 1) return 0;
  int t = __ffsll((long long)d) - 1;  // d = 2^t * m, m odd
  uint64_t m = d >> t;
  uint64_t rm = 0;  // 16^e mod m
  if (m > 1) {
    uint64_t minv = neg_inv64(m);
    uint64_t r1 = (0 - m) % m;  // 2^64 mod m: Montgomery one
    uint64_t base = (r1 << 4) % m;  // 16 * 2^64 mod m (r1 < m < 2^34)
    uint64_t x = r1;
    if (e) {
      int top = 63 - __clzll((long long)e);
      x = base;
      for (int b = top - 1; b >= 0; b--) {
        x = mont_mul(x, x, m, minv);
        if ((e >> b) & 1) x = mont_mul(x, base, m, minv);
      }
    }
    rm = mont_mul(x, 1, m, minv);  // out of Montgomery form
  }
  // 16^e mod 2^t: 0 if 4e >= t, else 16^e (t <= 2 here; e = 0 gives 1)
  uint64_t r2 = (4 * e >= (uint64_t)t) ? 0 : (1ull << (4 * e));
  if (t == 0) return rm;
  // CRT: x = rm (mod m), x = r2 (mod 2^t), x < d
  uint64_t mask = (1ull << t) - 1;
  // m * s = r2 - rm (mod 2^t); m odd so m^-1 mod 2^t exists (t <= 2: m^-1 = m)
  uint64_t s = ((r2 - rm) * m) & mask;
  return rm + m * s;
}

// floor(p * 2^64 / d) for p < d < 2^34 (the quotient fits in 64 bits):
// long division in three 32-bit-safe steps.
__device__ __forceinline__ uint64_t frac64(uint64_t p, uint64_t d) {
  uint64_t q = 0, r = p;
  // 64 = 30 + 30 + 4 bits; r < d < 2^34 so r << 30 < 2^64
  uint64_t x = r << 30;
  uint64_t q1 = x / d;
  r = x - q1 * d;
  x = r << 30;
  uint64_t q2 = x / d;
  r = x - q2 * d;
  x = r << 4;
  uint64_t q3 = x / d;
  q = (q1 << 34) | (q2 << 4) | q3;
  return q;
}

constexpr int BBP_THREADS = 256;
constexpr uint64_t POLL_EVERY = 10000;

// One CTA per (position, series): partial wrapping sums of the modular part.
__global__ void __launch_bounds__(BBP_THREADS)
k_bbp_series(const uint64_t* __restrict__ pos, uint32_t npos, uint64_t* __restrict__ sums,
             const volatile int* stop, int* status) {
  const uint32_t pair = blockIdx.x;
  const uint32_t pi = pair >> 2;
  const uint32_t js[4] = {1, 4, 5, 6};
  const uint64_t j = js[pair & 3];
  const uint64_t n = pos[pi];
  uint64_t acc = 0;
  uint64_t done = 0;
  for (uint64_t k = threadIdx.x; k <= n; k += BBP_THREADS) {
    if (stop && (done++ % POLL_EVERY) == 0 && *stop) {
      *status = 1;
      break;
    }
    uint64_t d = 8 * k + j;
    uint64_t p = pow16_mod(n - k, d);
    acc += frac64(p, d);
  }
  // block reduction of the wrapping sums
  __shared__ uint64_t red[BBP_THREADS / 32];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xFFFFFFFFu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint64_t s = 0;
    for (int w = 0; w < BBP_THREADS / 32; w++) s += red[w];
    sums[pair] = s;
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

}  // namespace pimul_bbp

using namespace pimul_bbp;

#define BCU(call)                                                                        \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess) { rc = fail(PIMUL_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); goto done; } \
  } while (0)

extern "C" const char* pimul_bbp_last_error(void) { return t_err.c_str(); }

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
  BCU(cudaMemcpyAsync(d_pos, positions, count * 8, cudaMemcpyHostToDevice, st));
  k_bbp_series<<<(unsigned)(4 * count), BBP_THREADS, 0, st>>>(d_pos, (uint32_t)count, d_sums,
                                                              stop ? (const volatile int*)d_flag : nullptr,
                                                              d_status);
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
  if (d_dig) cudaFreeAsync(d_dig, st);
  if (st) {
    cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
  }
  if (h_flag) cudaFreeHost(h_flag);
  if (h_status) cudaFreeHost(h_status);
  return rc;
}
