// Gauss-Legendre AGM on the device (crates/pi-core/src/algorithm/
// gauss_legendre.rs:61-151): a, b, t live in HBM as limb-aligned fixed
// point numbers (nf fraction limbs below one integer limb), so truncating a
// value to m fraction limbs is a pointer offset and a product's rescaling
// drops whole limbs.
//
//   a = 1, b = sqrt(1/2), t = 1/4, p = 1; repeat ceil(log2 prec) + 2 times:
//     a' = (a + b) / 2,  b' = sqrt(a b),  t -= p (a - a')^2,  p *= 2
//   pi = (a + b)^2 / (4 t)
//
// sqrt(x) = x y with y = 1/sqrt(x) from Newton's iteration
// y' = y - y (x y^2 - 1) / 2, kept from one AGM step to the next: the new x
// differs from the old by about 2 (a - b), so y starts that accurate, and
// each step runs at twice the accuracy it starts from (|x y^2 - 1| measured
// on the device), the last ones at full precision.  The caller turns
// (a + b)^2 and t into floor(pi 10^(D-1)) with the device quotient (dec.cu)
// and converts it on the device; with 64 guard bits beyond the reference's
// working precision the digits are the reference's.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../include/pimul.h"
#include "agm.h"
#include "dec.h"
#include "hostcopy.h"
#include "wrapmul.h"

namespace piagm {
namespace {

// dst[j] = bits [sh + 64 j, sh + 64 j + 64) of src (zero outside; sh < 0 shifts left).
__global__ void k_shift(const uint64_t* __restrict__ src, uint64_t src_len, int64_t sh, uint64_t* __restrict__ dst,
                        uint64_t dst_len) {
  const int64_t ws = sh >> 6;
  const unsigned bs = (unsigned)(sh & 63);
  for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < dst_len;
       j += (uint64_t)gridDim.x * blockDim.x) {
    const int64_t i = ws + (int64_t)j;
    const uint64_t lo = i >= 0 && (uint64_t)i < src_len ? src[i] : 0;
    const uint64_t hi = i + 1 >= 0 && (uint64_t)(i + 1) < src_len ? src[i + 1] : 0;
    dst[j] = bs ? (lo >> bs) | (hi << (64 - bs)) : lo;
  }
}

// lo[i] = low word of x[i] c, hi[i] = high word of x[i - 1] c, for
// i in [0, n] (lo[n] = hi[0] = 0): x c = lo + hi.
__global__ void k_mul_word_split(const uint64_t* __restrict__ x, uint64_t n, uint64_t c, uint64_t* __restrict__ lo,
                                 uint64_t* __restrict__ hi) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= n; i += (uint64_t)gridDim.x * blockDim.x) {
    lo[i] = i < n ? x[i] * c : 0;
    hi[i] = i > 0 ? __umul64hi(x[i - 1], c) : 0;
  }
}

double now_ms() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// The run's device state: values of W = nf + 1 limbs and scratch.
struct Agm {
  cudaStream_t st = nullptr;
  size_t nf = 0, W = 0;
  int rc = PIMUL_OK;
  std::vector<uint64_t*> bufs;
  ~Agm() {
    for (uint64_t* p : bufs) cudaFreeAsync(p, st);
    if (st) {
      cudaStreamSynchronize(st);
      cudaStreamDestroy(st);
    }
  }
  uint64_t* alloc(size_t limbs) {
    uint64_t* p = nullptr;
    if (rc) return nullptr;
    if (cudaMallocAsync((void**)&p, std::max<size_t>(limbs, 1) * 8, st) != cudaSuccess) {
      cudaGetLastError();
      rc = PIMUL_ENOMEM;
      return nullptr;
    }
    bufs.push_back(p);
    if (cudaMemsetAsync(p, 0, std::max<size_t>(limbs, 1) * 8, st) != cudaSuccess) rc = PIMUL_ECUDA;
    return p;
  }
  void cu(cudaError_t e) {
    if (e != cudaSuccess && !rc) rc = e == cudaErrorMemoryAllocation ? PIMUL_ENOMEM : PIMUL_ECUDA;
  }
  void shift(const uint64_t* src, size_t src_len, int64_t sh, uint64_t* dst, size_t dst_len) {
    if (rc) return;
    const unsigned blocks = (unsigned)std::min<size_t>((dst_len + 255) / 256, 1u << 16);
    k_shift<<<std::max(1u, blocks), 256, 0, st>>>(src, src_len, sh, dst, dst_len);
    cu(cudaGetLastError());
  }
  // z[0..n+1) = x[0..n) c for a one-word c (lo, hi: n + 1 limbs of
  // scratch; z may not alias x), asynchronous
  void mul_word(const uint64_t* x, size_t n, uint64_t c, uint64_t* z, uint64_t* lo, uint64_t* hi) {
    if (rc) return;
    const unsigned blocks = (unsigned)std::min<size_t>((n + 256) / 256, 1u << 16);
    k_mul_word_split<<<std::max(1u, blocks), 256, 0, st>>>(x, n, c, lo, hi);
    cu(cudaGetLastError());
    if (rc) return;
    pimul_addsub_job j{lo, n + 1, hi, n + 1, z, n + 1, 0};  // x c < 2^(64 (n + 1)): no carry out
    rc = pimul::svc_addsub(&j, 1, st);
  }
  // z = x + y or x - y (x >= y; sub = PIMUL_SUB_MOD: modulo, asynchronous)
  // over W limbs (in place allowed)
  void addsub(const uint64_t* x, const uint64_t* y, uint64_t* z, int sub) {
    if (rc) return;
    pimul_addsub_job j{x, W, y, W, z, W, sub};
    rc = pimul_addsub_batch(&j, 1, st);
  }
  // z = x y at m fraction limbs: the top m + 1 limbs of each factor, the
  // product's top m + 1 limbs above its m lowest, lower limbs of z zeroed
  size_t n_mul = 0, n_full = 0;
  void mul(const uint64_t* x, const uint64_t* y, uint64_t* z, size_t m, uint64_t* tmp) {
    if (rc) return;
    n_mul++;
    if (m == nf) n_full++;
    const size_t off = nf - m;
    rc = pimul::mul_wrapped(x + off, m + 1, y + off, m + 1, tmp, st);
    if (rc) return;
    if (off) cu(cudaMemsetAsync(z, 0, off * 8, st));
    cu(cudaMemcpyAsync(z + off, tmp + m, (m + 1) * 8, cudaMemcpyDeviceToDevice, st));
  }
  // z = |x - y| over W limbs; near convergence a and b cross by an ulp of
  // rounding, so the order is not known in advance
  void absdiff(const uint64_t* x, const uint64_t* y, uint64_t* z) {
    if (rc) return;
    pimul_addsub_job j{x, W, y, W, z, W, PIMUL_SUB_MOD};
    rc = pimul_addsub_batch(&j, 1, st);
    if (!rc && (limb(z, W - 1) >> 63)) {  // wrapped: y > x
      pimul_addsub_job k{y, W, x, W, z, W, PIMUL_SUB_MOD};
      rc = pimul_addsub_batch(&k, 1, st);
    }
  }
  uint64_t limb(const uint64_t* x, size_t i) {
    uint64_t v = 0;
    if (rc) return 0;
    cu(cudaMemcpyAsync(&v, x + i, 8, cudaMemcpyDeviceToHost, st));
    cu(cudaStreamSynchronize(st));
    return v;
  }
  size_t trimmed(const uint64_t* x, size_t n) {
    size_t len = 0;
    if (rc) return 0;
    const uint64_t* arr[1] = {x};
    size_t lens[1] = {n};
    rc = pimul_top_limbs(arr, lens, 1, &len, st);
    return len;
  }
};

// Refines y ~ 1/sqrt(x), given to about acc limbs, by y' = y (3 - x y^2) / 2,
// which has no sign to decide, so the reduced-precision steps queue on the
// stream without a host round trip.  Their precisions are planned down
// from nf (each a little over half the next), so the first full-precision
// step starts from more than half the limbs and leaves y correct to nf - 1;
// full-precision steps measure |x y^2 - 1| first (at most 8 of them).
void inv_sqrt(Agm& G, const uint64_t* x, uint64_t* y, size_t acc, const uint64_t* one, const uint64_t* three,
              uint64_t* u, uint64_t* v, uint64_t* d, uint64_t* tmp) {
  const size_t nf = G.nf;
  std::vector<size_t> plan{nf};
  // x -> (x + 1) / 2 + 3 decreases strictly above 7: the loop ends
  while (plan.back() > std::max<size_t>(2 * acc + 6, 8)) plan.push_back((plan.back() + 1) / 2 + 3);
  std::reverse(plan.begin(), plan.end());
  auto update = [&](size_t m) {
    G.addsub(three, v, d, PIMUL_SUB_MOD);  // 3 - x y^2 > 0
    G.mul(y, d, u, m, tmp);
    G.shift(u, G.W, 1, y, G.W);  // y (3 - x y^2) / 2
  };
  // from a start that is right to a few bits only (acc = 0), six cheap
  // steps at two limbs bring it to the plan's first precision
  for (int k = 0; acc == 0 && k < 6 && !G.rc; k++) {
    G.mul(y, y, u, std::min<size_t>(2, nf), tmp);
    G.mul(x, u, v, std::min<size_t>(2, nf), tmp);
    update(std::min<size_t>(2, nf));
  }
  for (size_t k = 0; k + 1 < plan.size() && !G.rc; k++) {
    G.mul(y, y, u, plan[k], tmp);
    G.mul(x, u, v, plan[k], tmp);
    update(plan[k]);
  }
  for (int full = 0; full < 8 && !G.rc; full++) {
    G.mul(y, y, u, nf, tmp);
    G.mul(x, u, v, nf, tmp);
    G.absdiff(v, one, d);
    const size_t L = G.trimmed(d, G.W);
    const size_t got = nf > L ? nf - L : 0;  // limbs of accuracy before this step
    if (got + 1 >= nf) return;                // converged already
    update(nf);
    if (2 * got >= nf + 1) return;  // the step squared an error below 2^(-32 (nf + 1))
  }
  if (!G.rc) G.rc = PIMUL_EINVAL;  // no convergence: not expected for x in (0, 4)
}

}  // namespace

int agm_device(uint64_t prec, AgmOut* out, double* ms) {
  if (!out || prec < 64) return PIMUL_EINVAL;
  *out = AgmOut{};
  const double t0 = now_ms();
  Agm G;
  if (cudaStreamCreateWithFlags(&G.st, cudaStreamNonBlocking) != cudaSuccess) return PIMUL_ECUDA;
  G.nf = (prec + 64 + 63) / 64 + 1;
  G.W = G.nf + 1;
  const size_t nf = G.nf, W = G.W;
  uint64_t* a = G.alloc(W);
  uint64_t* b = G.alloc(W);
  uint64_t* t = G.alloc(W);
  uint64_t* y = G.alloc(W);
  uint64_t* x = G.alloc(W);
  uint64_t* an = G.alloc(W);
  uint64_t* u = G.alloc(W);
  uint64_t* v = G.alloc(W);
  uint64_t* d = G.alloc(W);
  uint64_t* one = G.alloc(W);
  uint64_t* three = G.alloc(W);
  uint64_t* tmp = G.alloc(2 * W + 2);
  if (G.rc) return G.rc;
  // constants: 1, 1/2, 1/4, and y ~ 1/sqrt(1/2) = sqrt(2) from an f64
  const uint64_t h_one = 1, h_three = 3, h_half = 1ull << 63, h_quarter = 1ull << 62;
  const double frac = std::sqrt(2.0) - 1.0;
  const uint64_t h_y[2] = {(uint64_t)std::ldexp(frac, 64), 1};
  G.cu(cudaMemcpyAsync(one + nf, &h_one, 8, cudaMemcpyHostToDevice, G.st));
  G.cu(cudaMemcpyAsync(three + nf, &h_three, 8, cudaMemcpyHostToDevice, G.st));
  G.cu(cudaMemcpyAsync(a + nf, &h_one, 8, cudaMemcpyHostToDevice, G.st));
  G.cu(cudaMemcpyAsync(x + nf - 1, &h_half, 8, cudaMemcpyHostToDevice, G.st));
  G.cu(cudaMemcpyAsync(t + nf - 1, &h_quarter, 8, cudaMemcpyHostToDevice, G.st));
  G.cu(cudaMemcpyAsync(y + nf - 1, h_y, 16, cudaMemcpyHostToDevice, G.st));
  G.cu(cudaStreamSynchronize(G.st));  // host constants are locals
  // b = sqrt(1/2) = x y
  inv_sqrt(G, x, y, 0, one, three, u, v, d, tmp);
  G.mul(x, y, b, nf, tmp);
  const uint32_t iters = (uint32_t)std::ceil(std::log2((double)prec)) + 2;
  const bool timing = getenv("PIMUL_PI_TIMING") != nullptr;
  for (uint32_t it = 0; it < iters && !G.rc; it++) {
    const double ti = now_ms();
    const size_t m0 = G.n_mul, f0 = G.n_full;
    // a' = (a + b) / 2
    G.addsub(a, b, u, 0);
    G.shift(u, W, 1, an, W);
    // y's accuracy for the new x = a b: about 2 |a - b| relative
    G.absdiff(a, b, d);
    const size_t ld = G.trimmed(d, W);
    const size_t acc = ld + 1 < nf ? nf - ld - 1 : 0;
    G.mul(a, b, x, nf, tmp);
    inv_sqrt(G, x, y, acc, one, three, u, v, d, tmp);
    // t -= 2^it (a - a')^2: |a - a'| has lsq limbs, its square only
    // matters in its limbs above the fraction's nf
    G.absdiff(a, an, d);
    const size_t lsq = G.trimmed(d, W);
    if (lsq && 2 * lsq > nf) {
      if (!G.rc) G.rc = pimul::mul_wrapped(d, lsq, d, lsq, tmp, G.st);
      G.shift(tmp, 2 * lsq, 64 * (int64_t)nf - it, u, W);  // (a - a')^2 2^it at nf fraction limbs
      G.addsub(t, u, t, 1);
    }
    // b = x y, a = a'
    G.mul(x, y, b, nf, tmp);
    G.cu(cudaMemcpyAsync(a, an, W * 8, cudaMemcpyDeviceToDevice, G.st));
    if (timing) {
      G.cu(cudaStreamSynchronize(G.st));
      fprintf(stderr, "[pimul] agm step %u: %zu products (%zu at full length), acc %zu of %zu limbs, %.1f ms\n", it,
              G.n_mul - m0, G.n_full - f0, acc, nf, now_ms() - ti);
    }
  }
  // (a + b)^2 at 2 nf fraction limbs, t at nf
  G.addsub(a, b, u, 0);
  if (!G.rc) G.rc = pimul::mul_wrapped(u, W, u, W, tmp, G.st);
  uint64_t* num = nullptr;
  uint64_t* den = nullptr;
  if (!G.rc && (cudaMalloc((void**)&num, 2 * W * 8) != cudaSuccess || cudaMalloc((void**)&den, W * 8) != cudaSuccess)) {
    cudaGetLastError();
    G.rc = PIMUL_ENOMEM;
  }
  if (num) G.cu(cudaMemcpyAsync(num, tmp, 2 * W * 8, cudaMemcpyDeviceToDevice, G.st));
  if (den) G.cu(cudaMemcpyAsync(den, t, W * 8, cudaMemcpyDeviceToDevice, G.st));
  G.cu(cudaStreamSynchronize(G.st));
  if (G.rc) {
    if (num) cudaFree(num);
    if (den) cudaFree(den);
    return G.rc;
  }
  *out = AgmOut{num, 2 * W, -128 * (int64_t)nf, den, W, -64 * (int64_t)nf};
  if (ms) ms[0] = now_ms() - t0;
  return PIMUL_OK;
}

namespace {

// 5^e into a cudaMalloc'd buffer: r = 5, then for each bit of e below the
// top one r = r^2 (and r = 5 r when the bit is set), each product exact and
// trimmed to its length (read back: a few dozen steps).
int pow5(Agm& G, uint64_t e, DevNum* out) {
  const size_t cap = (size_t)((double)e * 2.321928094887362 / 64.0) + 4;  // limbs of 5^e, plus room
  uint64_t* A = G.alloc(cap);
  uint64_t* B = G.alloc(cap);
  uint64_t* lo = G.alloc(cap);
  uint64_t* hi = G.alloc(cap);
  if (G.rc) return G.rc;
  const uint64_t start = e ? 5 : 1;
  G.cu(cudaMemcpyAsync(A, &start, 8, cudaMemcpyHostToDevice, G.st));
  G.cu(cudaStreamSynchronize(G.st));  // start is a local
  size_t L = 1;
  const int nb = e ? 64 - __builtin_clzll(e) : 0;
  for (int i = nb - 2; i >= 0 && !G.rc; i--) {
    if (2 * L + 1 > cap) return G.rc = PIMUL_EINVAL;  // not reached: cap bounds 5^e with room
    G.rc = pimul::mul_wrapped(A, L, A, L, B, G.st);  // a square (same operand)
    size_t L2 = 2 * L;
    if ((e >> i) & 1) {
      G.mul_word(B, L2, 5, A, lo, hi);
      L2++;
    } else {
      std::swap(A, B);
    }
    L = G.trimmed(A, L2);
  }
  if (G.rc) return G.rc;
  uint64_t* m = nullptr;
  if (cudaMalloc((void**)&m, L * 8) != cudaSuccess) {
    cudaGetLastError();
    return G.rc = PIMUL_ENOMEM;
  }
  G.cu(cudaMemcpyAsync(m, A, L * 8, cudaMemcpyDeviceToDevice, G.st));
  G.cu(cudaStreamSynchronize(G.st));
  if (G.rc) {
    cudaFree(m);
    return G.rc;
  }
  *out = DevNum{m, L, 0};
  return PIMUL_OK;
}

}  // namespace

int pow5_device(uint64_t e, DevNum* out) {
  if (!out) return PIMUL_EINVAL;
  *out = DevNum{};
  Agm G;
  if (cudaStreamCreateWithFlags(&G.st, cudaStreamNonBlocking) != cudaSuccess) return PIMUL_ECUDA;
  return pow5(G, e, out);
}

// sqrt(10005) = 2^7 sqrt(x) with x = 10005 / 2^14 in (1/2, 1); y ~ 1/sqrt(x)
// in fixed point (nf fraction limbs below one integer limb) by
// y' = y (3 - x y^2) / 2 at the planned precisions (x y^2 is a one-word
// multiplication and a shift, not a product), three steps at three limbs
// from an f64 start first.  From y = (1 + e)/sqrt(x) a step gives
// (1 - 3e^2/2 - e^3/2)/sqrt(x), and the truncations cost a few units of the
// step's last limb, so a step at m limbs from an input right to m' limbs,
// 2 m' >= m + 2, leaves y right to 64 m - 4 bits.  Then
// W = 426880 sqrt(10005) 5^(D-1) 2^(D-1) = (426880 * 10005 y) 5^(D-1) 2^(D-8).
int chudnovsky_w_device(uint64_t digits, uint64_t prec, DevNum* out, double* ms) {
  if (!out || !digits || prec < 64) return PIMUL_EINVAL;
  *out = DevNum{};
  const double t0 = now_ms();
  Agm G;
  int prio_lo = 0, prio_hi = 0;
  cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi);
  if (cudaStreamCreateWithPriority(&G.st, cudaStreamNonBlocking, prio_hi) != cudaSuccess) return PIMUL_ECUDA;
  G.nf = (prec + 128 + 63) / 64 + 1;
  G.W = G.nf + 1;
  const size_t nf = G.nf, W = G.W;
  constexpr uint64_t N = 10005, SH = 14, C2 = 426880ull * 10005ull;
  uint64_t* y = G.alloc(W);
  uint64_t* u = G.alloc(W);
  uint64_t* v = G.alloc(W);
  uint64_t* d = G.alloc(W);
  uint64_t* three = G.alloc(W);
  uint64_t* s = G.alloc(W + 2);
  uint64_t* lo = G.alloc(W + 2);
  uint64_t* hi = G.alloc(W + 2);
  uint64_t* tmp = G.alloc(2 * W + 2);
  if (G.rc) return G.rc;
  const uint64_t h_three = 3;
  const double frac = std::ldexp(1.0, (int)(SH / 2)) / std::sqrt((double)N) - 1.0;  // 1/sqrt(x) - 1
  const uint64_t h_y[2] = {(uint64_t)std::ldexp(frac, 64), 1};
  G.cu(cudaMemcpyAsync(three + nf, &h_three, 8, cudaMemcpyHostToDevice, G.st));
  G.cu(cudaMemcpyAsync(y + nf - 1, h_y, 16, cudaMemcpyHostToDevice, G.st));
  G.cu(cudaStreamSynchronize(G.st));  // host constants are locals
  auto step = [&](size_t m) {
    const size_t off = nf - m;
    G.mul(y, y, u, m, tmp);                      // y^2
    G.mul_word(u + off, m + 1, N, s, lo, hi);    // y^2 N (m + 2 limbs)
    G.shift(s, m + 2, (int64_t)SH, v + off, m + 1);  // x y^2
    G.addsub(three, v, d, PIMUL_SUB_MOD);        // 3 - x y^2 > 0
    G.mul(y, d, u, m, tmp);
    G.shift(u, W, 1, y, W);
  };
  std::vector<size_t> plan{nf};
  // m -> (m + 1) / 2 + 1 decreases strictly above 3
  while (plan.back() > 3) plan.push_back((plan.back() + 1) / 2 + 1);
  std::reverse(plan.begin(), plan.end());
  for (int k = 0; k < 3; k++) step(std::min<size_t>(3, nf));
  for (size_t m : plan)
    if (m > 3) step(m);
  // 426880 * 10005 y (W + 1 limbs, nf fraction limbs), then times 5^(D-1)
  G.mul_word(y, W, C2, s, lo, hi);
  DevNum p5;
  if (!G.rc) G.rc = pow5(G, digits - 1, &p5);
  if (G.rc) {
    if (p5.mant) cudaFree(p5.mant);
    return G.rc;
  }
  const size_t full = W + 1 + p5.limbs, keep = std::min(full, nf + 2);
  uint64_t* prod = G.alloc(full);
  if (!G.rc) G.rc = pimul::mul_wrapped(s, W + 1, p5.mant, p5.limbs, prod, G.st);
  uint64_t* m = nullptr;
  if (!G.rc && cudaMalloc((void**)&m, keep * 8) != cudaSuccess) {
    cudaGetLastError();
    G.rc = PIMUL_ENOMEM;
  }
  if (m) G.cu(cudaMemcpyAsync(m, prod + (full - keep), keep * 8, cudaMemcpyDeviceToDevice, G.st));
  G.cu(cudaStreamSynchronize(G.st));
  cudaFree(p5.mant);
  if (G.rc) {
    if (m) cudaFree(m);
    return G.rc;
  }
  *out = DevNum{m, keep, (int64_t)digits - 8 - 64 * (int64_t)nf + 64 * (int64_t)(full - keep)};
  if (ms) ms[0] = now_ms() - t0;
  return PIMUL_OK;
}

}  // namespace piagm
