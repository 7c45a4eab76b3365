// pimul engine: Goldilocks NTT big-integer multiply on one GB300 (sm_103a).
//
// Host orchestration + kernels for the plain drop-in multiply
// (include/pimul.h: pimul_mul, pimul_mul_device).  The algorithm follows the
// reference's mul_mag_ntt (crates/bignum/src/ntt.rs:806-865): pack limbs into
// 16-bit coefficients, forward-transform both operands, multiply pointwise,
// inverse-transform, carry-normalise back to limbs.  Results are exact, so
// every product equals the reference's bit for bit.
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <atomic>
#include <mutex>
#include <string>
#include <vector>

#include "gl.cuh"
#include "ntt_kernels.cuh"
#include "../../include/pimul.h"

namespace pimul {

// ------------------------------------------------------------------ errors
static thread_local std::string t_err;

static int fail(int code, const std::string& msg) {
  t_err = msg;
  return code;
}

#define CU(call)                                                                   \
  do {                                                                             \
    cudaError_t e_ = (call);                                                       \
    if (e_ != cudaSuccess)                                                         \
      return fail(e_ == cudaErrorMemoryAllocation ? PIMUL_ENOMEM : PIMUL_ECUDA,    \
                  std::string(#call) + ": " + cudaGetErrorString(e_));             \
  } while (0)

// ------------------------------------------------------------------ launch stats
// Launch counters per kernel class, and optional CUDA-event timing of every
// launch on the stream it runs on (pimul_stats_enable).
enum KClass { K_PACK, K_PASS_FWD, K_PASS_INV, K_POINTWISE, K_CARRY, K_SMALL, K_NCLASS };
static const char* k_names[K_NCLASS] = {"pack", "pass_fwd", "pass_inv", "pointwise", "carry", "small"};
static std::atomic<uint64_t> g_launch[K_NCLASS];
static std::atomic<int> g_timing{0};
struct Pending {
  int cls;
  cudaEvent_t a, b;
};
static std::mutex g_tmu;
static std::vector<Pending> g_pending;
static std::vector<cudaEvent_t> g_evpool;
static double g_ms[K_NCLASS];
static uint64_t g_timed[K_NCLASS];

static cudaEvent_t ev_get() {
  cudaEvent_t e = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_tmu);
    if (!g_evpool.empty()) {
      e = g_evpool.back();
      g_evpool.pop_back();
    }
  }
  if (!e) cudaEventCreate(&e);
  return e;
}

struct KTimer {
  int cls;
  cudaStream_t st;
  cudaEvent_t a = nullptr;
  KTimer(int c, cudaStream_t s, bool on = true) : cls(c), st(s) {
    if (!on) return;
    g_launch[c].fetch_add(1, std::memory_order_relaxed);
    if (g_timing.load(std::memory_order_relaxed)) {
      a = ev_get();
      cudaEventRecord(a, st);
    }
  }
  ~KTimer() {
    if (a) {
      cudaEvent_t b = ev_get();
      cudaEventRecord(b, st);
      std::lock_guard<std::mutex> lk(g_tmu);
      g_pending.push_back(Pending{cls, a, b});
    }
  }
};

static void stats_drain() {
  std::vector<Pending> p;
  {
    std::lock_guard<std::mutex> lk(g_tmu);
    p.swap(g_pending);
  }
  for (auto& x : p) {
    cudaEventSynchronize(x.b);
    float ms = 0;
    cudaEventElapsedTime(&ms, x.a, x.b);
    std::lock_guard<std::mutex> lk(g_tmu);
    g_ms[x.cls] += ms;
    g_timed[x.cls] += 1;
    g_evpool.push_back(x.a);
    g_evpool.push_back(x.b);
  }
}

// ------------------------------------------------------------------ host field
namespace hf {
constexpr uint64_t P = gl::P;
static uint64_t mul(uint64_t a, uint64_t b) {
  unsigned __int128 x = (unsigned __int128)a * b;
  uint64_t lo = (uint64_t)x, hi = (uint64_t)(x >> 64);
  uint64_t x2 = hi & 0xFFFFFFFFull, x3 = hi >> 32;
  uint64_t t = lo - x3;
  if (lo < x3) t -= gl::EPS;
  uint64_t u = (x2 << 32) - x2;
  uint64_t r = t + u;
  if (r < u) r += gl::EPS;
  return r >= P ? r - P : r;
}
static uint64_t pow(uint64_t b, uint64_t e) {
  uint64_t a = 1;
  while (e) {
    if (e & 1) a = mul(a, b);
    e >>= 1;
    b = mul(b, b);
  }
  return a;
}
}  // namespace hf

// rho: primitive 2^32-th root of unity with rho^(2^26) = 8.  Powers of the
// generator 7 (crates/bignum/src/ntt.rs:172) give the 2^32-th roots; the
// odd power t is picked so that the 64th root of unity is exactly 2^3.
static uint64_t find_rho() {
  uint64_t w0 = hf::pow(7, (hf::P - 1) >> 32);
  for (uint64_t t = 1; t < 64; t += 2) {
    uint64_t r = hf::pow(w0, t);
    if (hf::pow(r, 1ull << 26) == 8) return r;
  }
  return 0;
}

// ------------------------------------------------------------------ kernels
// Geometry of the HBM passes.  All pass tiles hold 2^13 words (64 KiB plus
// padding) and are processed by 256 threads:
//   first pass (p = 0):   2^R rows x 2^(13-R) columns of the single block
//   middle passes:        2^(9-R) blocks x 2^R rows x 16 columns
//   last pass (S = 1):    2^(13-R) contiguous blocks of 2^R words
// Column tiles read 128-byte (or wider) row segments.
constexpr int PASS_THREADS = 256;
constexpr int TILE_LOG = 13;

static inline size_t pass_smem_bytes(int tile_log) { return ((size_t)1 << tile_log) * 17 / 16 * 8 + 512 * 8; }

// Load the 512 forward roots w_512^t into shared memory (round twiddles).
__device__ __forceinline__ void load_tw512(uint64_t* tw, const Roots& R) {
  for (int t = threadIdx.x; t < 512; t += blockDim.x) tw[t] = __ldg(R.lvl + 512 + t);
}

// Elements per thread in a 2^13-word tile, processed in groups of 8 so that
// every thread keeps 16 independent global loads in flight.
constexpr int PER_THREAD = (1 << 13) / 256;

// Forward pass 0 with the limb -> 16-bit coefficient split fused in
// (crates/bignum/src/ntt.rs:640-665): element (i, j) of the tile is
// coefficient n = i * 2^S + j0 + j, i.e. 16-bit slice n % 4 of limb n / 4;
// limbs past nl are zero (the reference's zero tail).
template <int R>
__global__ void __launch_bounds__(PASS_THREADS) k_fwd_first(const uint64_t* __restrict__ limbs, uint64_t nl,
                                                             uint64_t* __restrict__ data, int L, Roots RT) {
  constexpr int T = TILE_LOG - R;
  extern __shared__ uint64_t sm[];
  uint64_t* tw = sm + spad(1u << TILE_LOG);
  const int tid = threadIdx.x;
  const int S = L - R;
  const uint64_t j0 = (uint64_t)blockIdx.x << T;
  load_tw512(tw, RT);
  // each thread expands whole limbs: 2^R rows x 2^(T-2) limbs
  for (uint32_t q = tid; q < (1u << (R + T - 2)); q += PASS_THREADS) {
    uint32_t i = q >> (T - 2), c4 = q & ((1u << (T - 2)) - 1);
    uint64_t li = (((uint64_t)i << S) + j0) / 4 + c4;
    uint64_t x = li < nl ? __ldg(limbs + li) : 0;
    uint32_t base = (i << T) + 4 * c4;
    sm[spad(base + 0)] = x & 0xFFFF;
    sm[spad(base + 1)] = (x >> 16) & 0xFFFF;
    sm[spad(base + 2)] = (x >> 32) & 0xFFFF;
    sm[spad(base + 3)] = x >> 48;
  }
  __syncthreads();
  tile_fwd_t<R, T, 0, PASS_THREADS>(sm, tw, tid);
#pragma unroll 1
  for (int g = 0; g < PER_THREAD; g += 8) {
    uint64_t t8[8];
#pragma unroll
    for (int q = 0; q < 8; q++) {
      uint32_t lin = (g + q) * PASS_THREADS + tid;
      uint32_t i = lin >> T, j = lin & ((1u << T) - 1);
      t8[q] = root_pow(RT, L, (uint64_t)row_freq_t<R>(i) * (j0 + j), false);
    }
#pragma unroll
    for (int q = 0; q < 8; q++) {
      uint32_t lin = (g + q) * PASS_THREADS + tid;
      uint32_t i = lin >> T, j = lin & ((1u << T) - 1);
      data[((uint64_t)i << S) + j0 + j] = gl::mul(sm[spad(lin)], t8[q]);
    }
  }
}

// Middle column pass: 2^(9-R) blocks x 2^R rows x 16 columns; forward pass
// twiddles w_M^(f*j) after the rounds, inverse ones before.
template <int R, bool FWD>
__global__ void __launch_bounds__(PASS_THREADS) k_col_mid(uint64_t* __restrict__ data, int S, Roots RT) {
  constexpr int T = 4, BC = 9 - R;
  extern __shared__ uint64_t sm[];
  uint64_t* tw = sm + spad(1u << TILE_LOG);
  const int tid = threadIdx.x;
  const int mlog = R + S;
  const uint64_t ct = blockIdx.x & ((1u << (S - T)) - 1);
  const uint64_t b0 = ((uint64_t)blockIdx.x >> (S - T)) << BC;
  const uint64_t j0 = ct << T;
  load_tw512(tw, RT);
  auto gaddr = [&](uint32_t lin) {
    uint32_t j = lin & 15, i = (lin >> 4) & ((1u << R) - 1), blk = lin >> (4 + R);
    return ((b0 + blk) << mlog) + ((uint64_t)i << S) + j0 + j;
  };
#pragma unroll 1
  for (int g = 0; g < PER_THREAD; g += 8) {
    uint64_t v8[8], t8[8];
#pragma unroll
    for (int q = 0; q < 8; q++) v8[q] = data[gaddr((g + q) * PASS_THREADS + tid)];
    if (!FWD) {
#pragma unroll
      for (int q = 0; q < 8; q++) {
        uint32_t lin = (g + q) * PASS_THREADS + tid;
        uint32_t i = (lin >> 4) & ((1u << R) - 1);
        t8[q] = root_pow(RT, mlog, (uint64_t)row_freq_t<R>(i) * (j0 + (lin & 15)), true);
      }
#pragma unroll
      for (int q = 0; q < 8; q++) v8[q] = gl::mul(v8[q], t8[q]);
    }
#pragma unroll
    for (int q = 0; q < 8; q++) sm[spad((g + q) * PASS_THREADS + tid)] = v8[q];
  }
  __syncthreads();
  if (FWD) tile_fwd_t<R, T, BC, PASS_THREADS>(sm, tw, tid);
  else tile_inv_t<R, T, BC, PASS_THREADS>(sm, tw, tid);
#pragma unroll 1
  for (int g = 0; g < PER_THREAD; g += 8) {
    uint64_t t8[8];
    if (FWD) {
#pragma unroll
      for (int q = 0; q < 8; q++) {
        uint32_t lin = (g + q) * PASS_THREADS + tid;
        uint32_t i = (lin >> 4) & ((1u << R) - 1);
        t8[q] = root_pow(RT, mlog, (uint64_t)row_freq_t<R>(i) * (j0 + (lin & 15)), false);
      }
    }
#pragma unroll
    for (int q = 0; q < 8; q++) {
      uint32_t lin = (g + q) * PASS_THREADS + tid;
      uint64_t v = sm[spad(lin)];
      data[gaddr(lin)] = FWD ? gl::mul(v, t8[q]) : v;
    }
  }
}

// Last forward pass (stride 1): 2^(13-R) contiguous blocks of 2^R words.
template <int R>
__global__ void __launch_bounds__(PASS_THREADS) k_fwd_last(uint64_t* __restrict__ data, Roots RT) {
  constexpr int BC = TILE_LOG - R;
  extern __shared__ uint64_t sm[];
  uint64_t* tw = sm + spad(1u << TILE_LOG);
  const int tid = threadIdx.x;
  uint64_t* base = data + ((uint64_t)blockIdx.x << TILE_LOG);
  load_tw512(tw, RT);
  for (uint32_t lin = tid; lin < (1u << TILE_LOG); lin += PASS_THREADS) sm[spad(lin)] = base[lin];
  __syncthreads();
  tile_fwd_t<R, 0, BC, PASS_THREADS>(sm, tw, tid);
  for (uint32_t lin = tid; lin < (1u << TILE_LOG); lin += PASS_THREADS) base[lin] = sm[spad(lin)];
}

// Fused middle of the multiply on one contiguous tile: last forward pass of
// b, pointwise product with the spectrum of a (times N^-1, the inverse's
// 1/N, crates/bignum/src/ntt.rs:383-390 and 845-853), first inverse pass;
// the result overwrites b's array.  SQUARE: a's own spectrum is squared.
template <int R, bool SQUARE>
__global__ void __launch_bounds__(PASS_THREADS) k_mid(uint64_t* __restrict__ b, const uint64_t* __restrict__ a,
                                                       uint64_t ninv, Roots RT) {
  constexpr int BC = TILE_LOG - R;
  extern __shared__ uint64_t sm[];
  uint64_t* tw = sm + spad(1u << TILE_LOG);
  const int tid = threadIdx.x;
  const uint64_t off = (uint64_t)blockIdx.x << TILE_LOG;
  load_tw512(tw, RT);
  for (uint32_t lin = tid; lin < (1u << TILE_LOG); lin += PASS_THREADS) sm[spad(lin)] = b[off + lin];
  __syncthreads();
  tile_fwd_t<R, 0, BC, PASS_THREADS>(sm, tw, tid);
  for (uint32_t lin = tid; lin < (1u << TILE_LOG); lin += PASS_THREADS) {
    uint64_t x = sm[spad(lin)];
    uint64_t y = SQUARE ? x : a[off + lin];
    sm[spad(lin)] = gl::mul(gl::mul(x, y), ninv);
  }
  __syncthreads();
  tile_inv_t<R, 0, BC, PASS_THREADS>(sm, tw, tid);
  for (uint32_t lin = tid; lin < (1u << TILE_LOG); lin += PASS_THREADS) b[off + lin] = sm[spad(lin)];
}

// ---- carry normalisation (crates/bignum/src/ntt.rs:676-791) --------------
// Coefficients are grouped in windows of 16 (= 4 limbs).  Window w has value
// V_w = sum_t c[16w+t] 2^(16t) = lo_w + hi_w 2^256.  The product is
// sum_w (lo_w + hi_(w-1)) 2^(256w); s_w = lo_w + hi_(w-1) may carry one bit
// (g_w) into window w+1, which a run of all-ones windows (p_w) propagates.
// Carries are resolved with a carry-lookahead scan over (g, p) bit vectors:
// with A = g|p and B = g, the carry into each window is bit w of
// (A + B + cin) ^ A ^ B.

struct Win {
  uint64_t l[4];
  uint64_t hi;
};

// Window value from 16 canonical coefficients (u128 accumulator, as the
// reference's unpack loop, ntt.rs:694-707).
__device__ __forceinline__ Win fold16(const uint64_t* c16, int stride) {
  Win r;
  unsigned __int128 acc = 0;
#pragma unroll
  for (int k = 0; k < 4; k++) {
#pragma unroll
    for (int q = 0; q < 4; q++) acc += (unsigned __int128)c16[(4 * k + q) * stride] << (16 * q);
    r.l[k] = (uint64_t)acc;
    acc >>= 64;
  }
  r.hi = (uint64_t)acc;
  return r;
}

// Inverse pass 0 (natural order out) fused with the window fold: each tile
// row holds 2^T consecutive coefficients = 2^(T-4) windows; every window
// writes its low 4 limbs to the output and its high part to H.
template <int R>
__global__ void __launch_bounds__(PASS_THREADS) k_inv_first_carry(const uint64_t* __restrict__ data, int L,
                                                                   uint64_t* __restrict__ out, uint64_t nlimbs,
                                                                   uint64_t* __restrict__ H, uint64_t nwin,
                                                                   Roots RT) {
  constexpr int T = TILE_LOG - R;
  extern __shared__ uint64_t sm[];
  uint64_t* tw = sm + spad(1u << TILE_LOG);
  const int tid = threadIdx.x;
  const int S = L - R;
  const uint64_t j0 = (uint64_t)blockIdx.x << T;
  load_tw512(tw, RT);
#pragma unroll 1
  for (int g = 0; g < PER_THREAD; g += 8) {
    uint64_t v8[8], t8[8];
#pragma unroll
    for (int q = 0; q < 8; q++) {
      uint32_t lin = (g + q) * PASS_THREADS + tid;
      uint32_t i = lin >> T, j = lin & ((1u << T) - 1);
      v8[q] = data[((uint64_t)i << S) + j0 + j];
    }
#pragma unroll
    for (int q = 0; q < 8; q++) {
      uint32_t lin = (g + q) * PASS_THREADS + tid;
      uint32_t i = lin >> T, j = lin & ((1u << T) - 1);
      t8[q] = root_pow(RT, L, (uint64_t)row_freq_t<R>(i) * (j0 + j), true);
    }
#pragma unroll
    for (int q = 0; q < 8; q++) sm[spad((g + q) * PASS_THREADS + tid)] = gl::mul(v8[q], t8[q]);
  }
  __syncthreads();
  tile_inv_t<R, T, 0, PASS_THREADS>(sm, tw, tid);
  for (uint32_t q = tid; q < (1u << (TILE_LOG - 4)); q += PASS_THREADS) {
    uint32_t i = q >> (T - 4), k = q & ((1u << (T - 4)) - 1);
    uint64_t w = ((((uint64_t)i << S) + j0) >> 4) + k;
    if (w >= nwin) continue;
    uint64_t c[16];
    uint32_t b = (i << T) + 16 * k;
#pragma unroll
    for (int t = 0; t < 16; t++) c[t] = gl::canon(sm[spad(b + t)]);
    Win v = fold16(c, 1);
#pragma unroll
    for (int t = 0; t < 4; t++)
      if (4 * w + t < nlimbs) out[4 * w + t] = v.l[t];
    H[w] = v.hi;
  }
}

constexpr int CARRY_THREADS = 256;  // windows per CTA

// Carry pass 1: s_w = lo_w + hi_(w-1) written back as the output limbs; per
// window (g, p), per warp the (A, B) masks, per CTA the chunk's carry out
// for carry in 0 and 1.
__global__ void __launch_bounds__(CARRY_THREADS)
k_carry_local(uint64_t* __restrict__ out, uint64_t nlimbs, const uint64_t* __restrict__ H, uint64_t nwin,
              uint32_t* __restrict__ masks, uint8_t* __restrict__ chunk_gp) {
  __shared__ uint32_t sA[CARRY_THREADS / 32], sB[CARRY_THREADS / 32];
  const uint64_t w = (uint64_t)blockIdx.x * CARRY_THREADS + threadIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  bool g = false, p = false;
  if (w < nwin) {
    uint64_t base = 4 * w;
    uint64_t l0 = base + 0 < nlimbs ? out[base + 0] : 0;
    uint64_t l1 = base + 1 < nlimbs ? out[base + 1] : 0;
    uint64_t l2 = base + 2 < nlimbs ? out[base + 2] : 0;
    uint64_t l3 = base + 3 < nlimbs ? out[base + 3] : 0;
    uint64_t hprev = w > 0 ? H[w - 1] : 0;
    uint64_t s0 = l0 + hprev;
    uint64_t c = s0 < hprev;
    uint64_t s1 = l1 + c;  c = c && s1 == 0;
    uint64_t s2 = l2 + c;  c = c && s2 == 0;
    uint64_t s3 = l3 + c;  c = c && s3 == 0;
    g = c != 0;
    p = (s0 & s1 & s2 & s3) == ~0ull;
    if (base + 0 < nlimbs) out[base + 0] = s0;
    if (base + 1 < nlimbs) out[base + 1] = s1;
    if (base + 2 < nlimbs) out[base + 2] = s2;
    if (base + 3 < nlimbs) out[base + 3] = s3;
  }
  uint32_t A = __ballot_sync(0xFFFFFFFFu, g || p);
  uint32_t Bm = __ballot_sync(0xFFFFFFFFu, g);
  if (lane == 0) {
    uint64_t wi = (uint64_t)blockIdx.x * (CARRY_THREADS / 32) + warp;
    masks[2 * wi] = A;
    masks[2 * wi + 1] = Bm;
    sA[warp] = A;
    sB[warp] = Bm;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t cg = 0, cp = 1;  // chunk carry out for carry in 0 / 1
    for (int k = 0; k < CARRY_THREADS / 32; k++) {
      uint64_t sg = (uint64_t)sA[k] + sB[k] + cg;
      uint64_t sp = (uint64_t)sA[k] + sB[k] + cp;
      cg = (uint32_t)(sg >> 32);
      cp = (uint32_t)(sp >> 32);
    }
    chunk_gp[blockIdx.x] = (uint8_t)(cg | (cp << 1));
  }
}

// Carry pass 2: carry into every chunk.  One CTA; each thread walks a
// contiguous segment of chunks, the segment results are chained by thread 0.
constexpr int SCAN_THREADS = 1024;
__global__ void __launch_bounds__(SCAN_THREADS)
k_carry_scan(const uint8_t* __restrict__ chunk_gp, uint64_t nchunk, uint8_t* __restrict__ chunk_cin) {
  __shared__ uint8_t seg_g[SCAN_THREADS], seg_p[SCAN_THREADS], seg_cin[SCAN_THREADS];
  const uint64_t per = (nchunk + SCAN_THREADS - 1) / SCAN_THREADS;
  const uint64_t lo = threadIdx.x * per, hi = lo + per < nchunk ? lo + per : nchunk;
  uint8_t cg = 0, cp = 1;  // segment carry out for carry in 0 / 1
  for (uint64_t k = lo; k < hi; k++) {
    uint8_t gp = chunk_gp[k];
    uint8_t o0 = gp & 1, o1 = (gp >> 1) & 1;
    cg = cg ? o1 : o0;
    cp = cp ? o1 : o0;
  }
  seg_g[threadIdx.x] = cg;
  seg_p[threadIdx.x] = cp;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint8_t cin = 0;
    for (int k = 0; k < SCAN_THREADS; k++) {
      seg_cin[k] = cin;
      cin = cin ? seg_p[k] : seg_g[k];
    }
  }
  __syncthreads();
  uint8_t cin = seg_cin[threadIdx.x];
  for (uint64_t k = lo; k < hi; k++) {
    chunk_cin[k] = cin;
    uint8_t gp = chunk_gp[k];
    cin = cin ? ((gp >> 1) & 1) : (gp & 1);
  }
}

// Carry pass 3: add the incoming carry to every window that receives one.
__global__ void __launch_bounds__(CARRY_THREADS)
k_carry_apply(uint64_t nwin, uint64_t* __restrict__ out, uint64_t nlimbs, const uint32_t* __restrict__ masks,
              const uint8_t* __restrict__ chunk_cin) {
  const uint64_t w = (uint64_t)blockIdx.x * CARRY_THREADS + threadIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t cin = chunk_cin[blockIdx.x];
  const uint64_t wbase = (uint64_t)blockIdx.x * (CARRY_THREADS / 32);
  for (int k = 0; k < warp; k++) {
    uint64_t s = (uint64_t)masks[2 * (wbase + k)] + masks[2 * (wbase + k) + 1] + cin;
    cin = (uint32_t)(s >> 32);
  }
  uint32_t A = masks[2 * (wbase + warp)], Bm = masks[2 * (wbase + warp) + 1];
  uint32_t carries = (A + Bm + cin) ^ A ^ Bm;
  if (w < nwin && ((carries >> lane) & 1)) {
    uint64_t base = 4 * w;
    for (int k = 0; k < 4 && base + k < nlimbs; k++) {
      if (++out[base + k] != 0) break;
    }
  }
}

// ---- whole multiply in one CTA (N <= 2^SMALL_LOG_MAX) --------------------
constexpr int SMALL_THREADS = 256;
constexpr int SMALL_LOG_MAX = 12;

// Dynamic shared memory of the one-CTA multiply for N = 2^L (two padded arrays).
static inline size_t small_smem_bytes(int L) { return 2 * (((size_t)1 << L) * 17 / 16) * 8; }

struct SmallJob {
  const uint64_t* a;
  const uint64_t* b;
  uint64_t* out;
  uint32_t la, lb;
};

__device__ void small_multiply(const SmallJob& job, const Roots& R, uint64_t* smA, uint64_t* smB) {
  const int tid = threadIdx.x;
  const uint32_t la = job.la, lb = job.lb;
  const uint32_t n_out = 4 * la + 4 * lb - 1;
  int L = 0;
  while ((1u << L) < n_out) L++;
  const uint32_t N = 1u << L;
  const bool square = job.a == job.b && la == lb;
  for (uint32_t i = tid; i < N; i += SMALL_THREADS) {
    uint32_t l = i >> 2, sh = 16 * (i & 3);
    smA[spad(i)] = l < la ? (job.a[l] >> sh) & 0xFFFF : 0;
    if (!square) smB[spad(i)] = l < lb ? (job.b[l] >> sh) & 0xFFFF : 0;
  }
  __syncthreads();
  TileGeom g{L, 0, 0};
  tile_dft_fwd(smA, g, R, tid, SMALL_THREADS);
  if (!square) tile_dft_fwd(smB, g, R, tid, SMALL_THREADS);
  // times N^-1 = 2^(-L) = 2^(192 - L)
  const uint64_t ninv = gl::pow(2, 192 - L);
  for (uint32_t i = tid; i < N; i += SMALL_THREADS) {
    uint64_t x = smA[spad(i)];
    uint64_t y = square ? x : smB[spad(i)];
    smA[spad(i)] = gl::mul(gl::mul(x, y), ninv);
  }
  __syncthreads();
  tile_dft_inv(smA, g, R, tid, SMALL_THREADS);
  // carry: windows of 16 coefficients, one per thread (N/16 <= 256)
  const uint32_t nwin = (n_out + 15) / 16, nl = la + lb;
  uint64_t* sH = smB;  // reuse: B no longer needed
  __shared__ uint32_t sA[SMALL_THREADS / 32], sBm[SMALL_THREADS / 32];
  Win v{{0, 0, 0, 0}, 0};
  const uint32_t w = tid;
  if (w < nwin) {
    uint64_t c[16];
#pragma unroll
    for (int t = 0; t < 16; t++) {
      uint32_t idx = 16 * w + t;
      c[t] = idx < N ? gl::canon(smA[spad(idx)]) : 0;
    }
    v = fold16(c, 1);
  }
  __syncthreads();
  if (w < nwin) sH[w] = v.hi;  // nwin <= N/16 words fit in the B region
  __syncthreads();
  uint64_t hprev = (w > 0 && w - 1 < nwin) ? sH[w - 1] : 0;
  uint64_t s0 = v.l[0] + hprev;
  uint64_t c = s0 < hprev;
  uint64_t s1 = v.l[1] + c;  c = c && s1 == 0;
  uint64_t s2 = v.l[2] + c;  c = c && s2 == 0;
  uint64_t s3 = v.l[3] + c;  c = c && s3 == 0;
  bool gg = w < nwin && c;
  bool pp = w < nwin && (s0 & s1 & s2 & s3) == ~0ull;
  uint32_t A = __ballot_sync(0xFFFFFFFFu, gg || pp), Bm = __ballot_sync(0xFFFFFFFFu, gg);
  if ((tid & 31) == 0) { sA[tid >> 5] = A; sBm[tid >> 5] = Bm; }
  __syncthreads();
  uint32_t cin = 0;
  for (int k = 0; k < (tid >> 5); k++) {
    uint64_t s = (uint64_t)sA[k] + sBm[k] + cin;
    cin = (uint32_t)(s >> 32);
  }
  uint32_t carries = (A + Bm + cin) ^ A ^ Bm;
  if ((carries >> (tid & 31)) & 1) {
    if (++s0 == 0) if (++s1 == 0) if (++s2 == 0) ++s3;
  }
  if (w < nwin) {
    uint32_t base = 4 * w;
    if (base + 0 < nl) job.out[base + 0] = s0;
    if (base + 1 < nl) job.out[base + 1] = s1;
    if (base + 2 < nl) job.out[base + 2] = s2;
    if (base + 3 < nl) job.out[base + 3] = s3;
  }
}

__global__ void __launch_bounds__(SMALL_THREADS) k_small_mul(SmallJob job, Roots R) {
  extern __shared__ uint64_t sm[];
  const uint32_t n_out = 4 * job.la + 4 * job.lb - 1;
  int L = 0;
  while ((1u << L) < n_out) L++;
  uint32_t N = 1u << L;
  small_multiply(job, R, sm, sm + spad(N));
}

// ------------------------------------------------------------------ host side
static int log2_ceil(uint64_t x) {
  int L = 0;
  while ((1ull << L) < x) L++;
  return L;
}

// Host copies of the root tables: lo, hi, w12, level tables (in this order).
constexpr size_t ROOT_WORDS = 2 * 65536 + 4096 + (2u << LVL_MAX);

static void build_roots(uint64_t* t) {
  uint64_t rho = find_rho();
  uint64_t* lo = t;
  uint64_t* hi = lo + 65536;
  uint64_t* w12 = hi + 65536;
  uint64_t* lvl = w12 + 4096;
  uint64_t x = 1;
  for (int i = 0; i < 65536; i++) { lo[i] = x; x = hf::mul(x, rho); }
  uint64_t step = x;  // rho^(2^16)
  x = 1;
  for (int i = 0; i < 65536; i++) { hi[i] = x; x = hf::mul(x, step); }
  uint64_t w4096 = hf::pow(rho, 1ull << 20);
  x = 1;
  for (int i = 0; i < 4096; i++) { w12[i] = x; x = hf::mul(x, w4096); }
  // level k (1 <= k <= LVL_MAX): w_(2^k)^x at lvl[2^k + x]; level k is every
  // other entry of level k+1, starting from the longest
  const uint32_t top = 1u << LVL_MAX;
  uint64_t wm = hf::pow(rho, 1ull << (32 - LVL_MAX));
  x = 1;
  for (uint32_t i = 0; i < top; i++) { lvl[top + i] = x; x = hf::mul(x, wm); }
  for (int k = LVL_MAX - 1; k >= 1; k--)
    for (uint32_t i = 0; i < (1u << k); i++) lvl[(1u << k) + i] = lvl[(2u << k) + 2 * i];
  lvl[0] = lvl[1] = 1;
}

static Roots roots_at(const uint64_t* d) {
  return Roots{d, d + 65536, d + 2 * 65536, d + 2 * 65536 + 4096};
}

struct DeviceState {
  int device = -1;
  bool ready = false;
  uint64_t* d_roots = nullptr;
  Roots roots{};
  cudaMemPool_t pool = nullptr;
};

static std::mutex g_mu;
static DeviceState g_dev;
static thread_local cudaStream_t t_stream = nullptr;
static thread_local int t_stream_dev = -1;

// Opt every pass kernel into its dynamic shared memory.
template <int R>
static cudaError_t set_smem_attrs_r() {
  int bytes = (int)pass_smem_bytes(TILE_LOG);
  cudaError_t e = cudaSuccess;
  if (R >= 7) {
    e = cudaFuncSetAttribute(k_fwd_first<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_inv_first_carry<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  }
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_col_mid<R, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_col_mid<R, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_fwd_last<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_mid<R, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_mid<R, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  return e;
}

static cudaError_t set_smem_attrs() {
  cudaError_t e = set_smem_attrs_r<6>();
  if (e == cudaSuccess) e = set_smem_attrs_r<7>();
  if (e == cudaSuccess) e = set_smem_attrs_r<8>();
  if (e == cudaSuccess) e = set_smem_attrs_r<9>();
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_small_mul, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)small_smem_bytes(SMALL_LOG_MAX));
  return e;
}

static int ensure_init(int device) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (g_dev.ready) {
    if (device >= 0 && device != g_dev.device)
      return fail(PIMUL_EINVAL, "pimul already initialised on another device");
    return PIMUL_OK;
  }
  if (device < 0) device = 0;
  CU(cudaSetDevice(device));
  std::vector<uint64_t> tables(ROOT_WORDS);
  build_roots(tables.data());
  CU(cudaMalloc(&g_dev.d_roots, ROOT_WORDS * 8));
  CU(cudaMemcpy(g_dev.d_roots, tables.data(), ROOT_WORDS * 8, cudaMemcpyHostToDevice));
  g_dev.roots = roots_at(g_dev.d_roots);
  CU(cudaDeviceGetDefaultMemPool(&g_dev.pool, device));
  uint64_t thr = UINT64_MAX;  // keep freed blocks cached in the pool
  CU(cudaMemPoolSetAttribute(g_dev.pool, cudaMemPoolAttrReleaseThreshold, &thr));
  CU(set_smem_attrs());
  g_dev.device = device;
  g_dev.ready = true;
  return PIMUL_OK;
}

static int get_stream(cudaStream_t* s) {
  int rc = ensure_init(-1);
  if (rc) return rc;
  if (!t_stream || t_stream_dev != g_dev.device) {
    CU(cudaSetDevice(g_dev.device));
    CU(cudaStreamCreateWithFlags(&t_stream, cudaStreamNonBlocking));
    t_stream_dev = g_dev.device;
  }
  CU(cudaSetDevice(g_dev.device));
  *s = t_stream;
  return PIMUL_OK;
}

// Split L bits into HBM passes of at most 9 bits (each radix 2^6 .. 2^9).
struct Plan {
  int L;
  int np;
  int r[5];
};

static Plan make_plan(int L) {
  Plan p{L, 0, {0, 0, 0, 0, 0}};
  int np = (L + 8) / 9;
  if (np < 2) np = 2;
  int base = L / np, extra = L % np;
  for (int i = 0; i < np; i++) p.r[i] = base + (i < extra ? 1 : 0);
  p.np = np;
  return p;
}

// Scratch of one large product.
struct Scratch {
  uint64_t* A;     // N words
  uint64_t* B;     // N words (unused for a square)
  uint64_t* H;     // high parts of the carry windows, nwin words
  uint8_t* aux;    // carry-scan flags
};

struct Sizes {
  uint64_t n_out, N, nwin, nchunk, nwarp, aux_bytes;
  int L;
};

static Sizes sizes_for(uint64_t la, uint64_t lb) {
  Sizes z;
  z.n_out = 4 * la + 4 * lb - 1;
  z.L = log2_ceil(z.n_out);
  z.N = 1ull << z.L;
  z.nwin = (z.n_out + 15) / 16;
  z.nchunk = (z.nwin + CARRY_THREADS - 1) / CARRY_THREADS;
  z.nwarp = z.nchunk * (CARRY_THREADS / 32);
  z.aux_bytes = z.nwarp * 8 + z.nchunk * 2 + 64;
  return z;
}


// Launch helpers (template dispatch on the pass radix).
#define PIMUL_DISPATCH_R(r, CALL)          \
  switch (r) {                             \
    case 6: { constexpr int RR = 6; CALL; } break; \
    case 7: { constexpr int RR = 7; CALL; } break; \
    case 8: { constexpr int RR = 8; CALL; } break; \
    default: { constexpr int RR = 9; CALL; } break; \
  }

struct Launcher {
  cudaStream_t st;
  bool stats;  // count and (optionally) time launches
  const Roots& R;
};

static void run_transform_fwd(const Launcher& X, const uint64_t* limbs, uint64_t nl, uint64_t* data,
                              const Plan& pl, bool last) {
  const int L = pl.L;
  const unsigned grid = (unsigned)(1ull << (L - TILE_LOG));
  const size_t smem = pass_smem_bytes(TILE_LOG);
  {
    KTimer kt(K_PACK, X.st, X.stats);
    PIMUL_DISPATCH_R(pl.r[0], (k_fwd_first<(RR < 7 ? 7 : RR)><<<grid, PASS_THREADS, smem, X.st>>>(limbs, nl, data, L, X.R)));
  }
  int consumed = pl.r[0];
  for (int p = 1; p < pl.np - 1; p++) {
    consumed += pl.r[p];
    int S = L - consumed;
    KTimer kt(K_PASS_FWD, X.st, X.stats);
    PIMUL_DISPATCH_R(pl.r[p], (k_col_mid<RR, true><<<grid, PASS_THREADS, smem, X.st>>>(data, S, X.R)));
  }
  if (last) {
    KTimer kt(K_PASS_FWD, X.st, X.stats);
    PIMUL_DISPATCH_R(pl.r[pl.np - 1], (k_fwd_last<RR><<<grid, PASS_THREADS, smem, X.st>>>(data, X.R)));
  }
}

// out[0 .. la+lb) = a * b for N >= 2^13 using the given scratch.
static void run_multiply(const Launcher& X, const uint64_t* d_a, uint64_t la, const uint64_t* d_b, uint64_t lb,
                         uint64_t* d_out, const Scratch& sc, const Sizes& z) {
  const bool square = d_a == d_b && la == lb;
  const Plan pl = make_plan(z.L);
  const unsigned grid = (unsigned)(1ull << (z.L - TILE_LOG));
  const size_t smem = pass_smem_bytes(TILE_LOG);
  const uint64_t ninv = hf::pow(hf::pow(2, 191), z.L);  // 2^-L (2^192 = 1)
  const int rl = pl.r[pl.np - 1];
  uint64_t* C;
  if (square) {
    run_transform_fwd(X, d_a, la, sc.A, pl, false);
    KTimer kt(K_POINTWISE, X.st, X.stats);
    PIMUL_DISPATCH_R(rl, (k_mid<RR, true><<<grid, PASS_THREADS, smem, X.st>>>(sc.A, sc.A, ninv, X.R)));
    C = sc.A;
  } else {
    run_transform_fwd(X, d_a, la, sc.A, pl, true);
    run_transform_fwd(X, d_b, lb, sc.B, pl, false);
    KTimer kt(K_POINTWISE, X.st, X.stats);
    PIMUL_DISPATCH_R(rl, (k_mid<RR, false><<<grid, PASS_THREADS, smem, X.st>>>(sc.B, sc.A, ninv, X.R)));
    C = sc.B;
  }
  int consumed = z.L - rl;
  for (int p = pl.np - 2; p >= 1; p--) {
    int S = z.L - consumed;
    consumed -= pl.r[p];
    KTimer kt(K_PASS_INV, X.st, X.stats);
    PIMUL_DISPATCH_R(pl.r[p], (k_col_mid<RR, false><<<grid, PASS_THREADS, smem, X.st>>>(C, S, X.R)));
  }
  const uint64_t nlimbs = la + lb;
  {
    KTimer kt(K_PASS_INV, X.st, X.stats);
    PIMUL_DISPATCH_R(pl.r[0], (k_inv_first_carry<(RR < 7 ? 7 : RR)><<<grid, PASS_THREADS, smem, X.st>>>(
                                  C, z.L, d_out, nlimbs, sc.H, z.nwin, X.R)));
  }
  uint32_t* masks = reinterpret_cast<uint32_t*>(sc.aux);
  uint8_t* chunk_gp = sc.aux + z.nwarp * 8;
  uint8_t* chunk_cin = chunk_gp + z.nchunk;
  {
    KTimer kt(K_CARRY, X.st, X.stats);
    k_carry_local<<<(unsigned)z.nchunk, CARRY_THREADS, 0, X.st>>>(d_out, nlimbs, sc.H, z.nwin, masks, chunk_gp);
    k_carry_scan<<<1, SCAN_THREADS, 0, X.st>>>(chunk_gp, z.nchunk, chunk_cin);
    k_carry_apply<<<(unsigned)z.nchunk, CARRY_THREADS, 0, X.st>>>(z.nwin, d_out, nlimbs, masks, chunk_cin);
  }
  if (X.stats) g_launch[K_CARRY].fetch_add(2, std::memory_order_relaxed);
}

// Device multiply: d_out[0 .. la+lb) = a * b, scratch from the memory pool.
static int mul_device(const uint64_t* d_a, uint64_t la, const uint64_t* d_b, uint64_t lb, uint64_t* d_out,
                      cudaStream_t st) {
  if (la == 0 || lb == 0) return PIMUL_OK;
  const Sizes z = sizes_for(la, lb);
  if (z.L > 32) return fail(PIMUL_EINVAL, "transform length above 2^32");
  const Roots& R = g_dev.roots;
  const bool square = d_a == d_b && la == lb;
  if (z.L <= SMALL_LOG_MAX) {
    SmallJob job{d_a, d_b, d_out, (uint32_t)la, (uint32_t)lb};
    {
      KTimer kt(K_SMALL, st, true);
      k_small_mul<<<1, SMALL_THREADS, small_smem_bytes(z.L), st>>>(job, R);
    }
    CU(cudaGetLastError());
    return PIMUL_OK;
  }
  Scratch sc{nullptr, nullptr, nullptr, nullptr};
  cudaError_t e = cudaMallocAsync((void**)&sc.A, z.N * 8, g_dev.pool, st);
  if (e == cudaSuccess && !square) e = cudaMallocAsync((void**)&sc.B, z.N * 8, g_dev.pool, st);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&sc.H, z.nwin * 8, g_dev.pool, st);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&sc.aux, z.aux_bytes, g_dev.pool, st);
  if (e != cudaSuccess) {
    if (sc.A) cudaFreeAsync(sc.A, st);
    if (sc.B) cudaFreeAsync(sc.B, st);
    if (sc.H) cudaFreeAsync(sc.H, st);
    cudaGetLastError();
    return fail(PIMUL_ENOMEM, std::string("scratch allocation: ") + cudaGetErrorString(e));
  }
  Launcher X{st, true, R};
  run_multiply(X, d_a, la, d_b, lb, d_out, sc, z);
  cudaError_t le = cudaGetLastError();
  cudaFreeAsync(sc.A, st);
  if (sc.B) cudaFreeAsync(sc.B, st);
  cudaFreeAsync(sc.H, st);
  cudaFreeAsync(sc.aux, st);
  if (le != cudaSuccess) return fail(PIMUL_ECUDA, std::string("kernel launch: ") + cudaGetErrorString(le));
  return PIMUL_OK;
}

}  // namespace pimul

// ====================================================================== C ABI
using namespace pimul;

extern "C" {

const char* pimul_version(void) { return "pimul 0.2 (sm_103a)"; }

const char* pimul_last_error(void) { return t_err.c_str(); }

int pimul_init(int device) { return ensure_init(device); }

int pimul_shutdown(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_dev.ready) return PIMUL_OK;
  cudaSetDevice(g_dev.device);
  cudaDeviceSynchronize();
  cudaFree(g_dev.d_roots);
  if (g_dev.pool) cudaMemPoolTrimTo(g_dev.pool, 0);
  g_dev = DeviceState{};
  return PIMUL_OK;
}

int pimul_plan(size_t la, size_t lb, uint64_t* n_transform, int* passes) {
  if (!n_transform || !passes) return fail(PIMUL_EINVAL, "null output pointer");
  if (la == 0 || lb == 0) { *n_transform = 0; *passes = 0; return PIMUL_OK; }
  int L = log2_ceil(4 * (uint64_t)la + 4 * (uint64_t)lb - 1);
  if (L > 32) return fail(PIMUL_EINVAL, "transform length above 2^32");
  *n_transform = 1ull << L;
  *passes = L <= SMALL_LOG_MAX ? 0 : make_plan(L).np;
  return PIMUL_OK;
}

int pimul_stats_enable(int on) {
  g_timing.store(on ? 1 : 0);
  return PIMUL_OK;
}

int pimul_stats_reset(void) {
  stats_drain();
  std::lock_guard<std::mutex> lk(g_tmu);
  for (int i = 0; i < K_NCLASS; i++) {
    g_launch[i].store(0);
    g_ms[i] = 0;
    g_timed[i] = 0;
  }
  return PIMUL_OK;
}

int pimul_stats_get(int kclass, const char** name, uint64_t* launches, uint64_t* timed, double* ms) {
  if (kclass < 0 || kclass >= K_NCLASS) return fail(PIMUL_EINVAL, "kernel class out of range");
  stats_drain();
  std::lock_guard<std::mutex> lk(g_tmu);
  if (name) *name = k_names[kclass];
  if (launches) *launches = g_launch[kclass].load();
  if (timed) *timed = g_timed[kclass];
  if (ms) *ms = g_ms[kclass];
  return PIMUL_OK;
}

int pimul_sync(void) {
  cudaStream_t st;
  int rc = get_stream(&st);
  if (rc) return rc;
  CU(cudaStreamSynchronize(st));
  return PIMUL_OK;
}

int pimul_mul_device(const uint64_t* d_a, size_t la, const uint64_t* d_b, size_t lb, uint64_t* d_out,
                     void* stream) {
  if (la && lb && (!d_a || !d_b || !d_out)) return fail(PIMUL_EINVAL, "null device pointer");
  cudaStream_t st;
  int rc = get_stream(&st);
  if (rc) return rc;
  if (stream) st = (cudaStream_t)stream;
  return mul_device(d_a, la, d_b, lb, d_out, st);
}

int pimul_mul(const uint64_t* a, size_t la, const uint64_t* b, size_t lb, uint64_t* out, size_t out_cap,
              size_t* out_len) {
  if (!out_len) return fail(PIMUL_EINVAL, "null out_len");
  *out_len = 0;
  if (la == 0 || lb == 0) return PIMUL_OK;  // empty means zero (ntt.rs:807-809)
  if (!a || !b || !out) return fail(PIMUL_EINVAL, "null pointer");
  if (out_cap < la + lb) return fail(PIMUL_EINVAL, "out_cap < la + lb");
  if (log2_ceil(4 * (uint64_t)la + 4 * (uint64_t)lb - 1) > 32)
    return fail(PIMUL_EINVAL, "transform length above 2^32");
  cudaStream_t st;
  int rc = get_stream(&st);
  if (rc) return rc;
  const bool square = a == b && la == lb;
  uint64_t *da = nullptr, *db = nullptr, *dout = nullptr;
  cudaError_t e = cudaMallocAsync((void**)&da, la * 8, g_dev.pool, st);
  if (e == cudaSuccess && !square) e = cudaMallocAsync((void**)&db, lb * 8, g_dev.pool, st);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&dout, (la + lb) * 8, g_dev.pool, st);
  if (e != cudaSuccess) {
    if (da) cudaFreeAsync(da, st);
    if (db) cudaFreeAsync(db, st);
    cudaGetLastError();
    return fail(PIMUL_ENOMEM, std::string("operand allocation: ") + cudaGetErrorString(e));
  }
  cudaMemcpyAsync(da, a, la * 8, cudaMemcpyHostToDevice, st);
  if (!square) cudaMemcpyAsync(db, b, lb * 8, cudaMemcpyHostToDevice, st);
  rc = mul_device(da, la, square ? da : db, lb, dout, st);
  if (rc == PIMUL_OK) cudaMemcpyAsync(out, dout, (la + lb) * 8, cudaMemcpyDeviceToHost, st);
  cudaFreeAsync(da, st);
  if (db) cudaFreeAsync(db, st);
  cudaFreeAsync(dout, st);
  cudaError_t se = cudaStreamSynchronize(st);
  if (rc) return rc;
  if (se != cudaSuccess) return fail(PIMUL_ECUDA, std::string("multiply: ") + cudaGetErrorString(se));
  size_t n = la + lb;
  while (n && out[n - 1] == 0) n--;  // trimmed, as the reference's unpack (ntt.rs:713-716)
  *out_len = n;
  return PIMUL_OK;
}

}  // extern "C"

// ====================================================================
// Multiply entry point that allocates nothing (pimul_mul_device_noalloc)
// ====================================================================
// Some callers cannot allocate device memory at the moment they multiply:
// a host that has handed the whole GPU to another allocator (a framework's
// caching allocator, a fixed arena reserved at start-up), a latency-bound
// loop where cudaMalloc's implicit device synchronisation is not allowed,
// or an embedding runtime whose rule is "allocate at init, never in the
// steady state".  For them this variant takes its scratch from a
// file-scope device array instead of the stream-ordered pool.
//
// Limits and sharing rules:
//  * scratch holds two transform arrays of at most 2^20 words plus the carry
//    windows and scan flags: la + lb <= 262144 limbs (transform length
//    N <= 2^20); larger products are rejected with PIMUL_EINVAL.  The
//    scratch (16.5 MiB) and this path's own root tables (17 MiB) stay
//    resident on every GPU that loads this library, until the process exits.
//  * every call uses the same array, and the array keeps the previous call's
//    contents; the kernels overwrite every scratch word before reading it,
//    so nothing needs clearing.  Calls whose work overlaps on the GPU
//    (different streams, or different host threads without ordering) race
//    on the array and corrupt each other's results: serialise them.
//  * the first call on each device does a one-time set-up with that device
//    current: it resolves the arrays' device addresses with
//    cudaGetSymbolAddress and copies the root tables in with a synchronous
//    cudaMemcpyToSymbol.  Make that first call before any stream capture.
namespace pimul {
constexpr int NOALLOC_LOG_MAX = 20;
constexpr uint64_t NOALLOC_N_MAX = 1ull << NOALLOC_LOG_MAX;
constexpr uint64_t NOALLOC_WIN_MAX = NOALLOC_N_MAX / 16;
constexpr uint64_t NOALLOC_CHUNK_MAX = (NOALLOC_WIN_MAX + CARRY_THREADS - 1) / CARRY_THREADS;
constexpr uint64_t NOALLOC_AUX_WORDS = (NOALLOC_CHUNK_MAX * (CARRY_THREADS / 32) * 8 + 2 * NOALLOC_CHUNK_MAX + 64) / 8 + 1;

static __device__ __align__(256) uint64_t g_noalloc_scratch[2 * NOALLOC_N_MAX + NOALLOC_WIN_MAX + NOALLOC_AUX_WORDS];
static __device__ __align__(256) uint64_t g_noalloc_roots[ROOT_WORDS];

struct NoAllocDev {
  bool ready = false;
  uint64_t* scratch = nullptr;  // device address of g_noalloc_scratch on this device
  Roots roots{};
};
static std::mutex g_na_mu;
static NoAllocDev g_na[64];
static uint64_t g_na_host_roots[ROOT_WORDS];  // staging, no heap use

static int noalloc_setup(NoAllocDev** out) {
  int dev = 0;
  CU(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(PIMUL_EINVAL, "device index out of range");
  std::lock_guard<std::mutex> lk(g_na_mu);
  NoAllocDev& d = g_na[dev];
  if (!d.ready) {
    build_roots(g_na_host_roots);
    uint64_t* scratch = nullptr;
    uint64_t* roots = nullptr;
    cudaError_t e = cudaGetSymbolAddress((void**)&scratch, g_noalloc_scratch);
    if (e != cudaSuccess) return fail(PIMUL_ECUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
    e = cudaGetSymbolAddress((void**)&roots, g_noalloc_roots);
    if (e != cudaSuccess) return fail(PIMUL_ECUDA, std::string("cudaGetSymbolAddress(roots): ") + cudaGetErrorString(e));
    CU(cudaMemcpyToSymbol(g_noalloc_roots, g_na_host_roots, sizeof(g_na_host_roots)));
    CU(set_smem_attrs());
    d.scratch = scratch;
    d.roots = roots_at(roots);
    d.ready = true;
  }
  *out = &d;
  return PIMUL_OK;
}

static int mul_device_noalloc(const uint64_t* d_a, uint64_t la, const uint64_t* d_b, uint64_t lb, uint64_t* d_out,
                              cudaStream_t st) {
  NoAllocDev* nd = nullptr;
  int rc = noalloc_setup(&nd);
  if (rc) return rc;
  const Sizes z = sizes_for(la, lb);
  const Roots& R = nd->roots;
  if (z.L <= SMALL_LOG_MAX) {  // whole product in one CTA's shared memory: no scratch
    SmallJob job{d_a, d_b, d_out, (uint32_t)la, (uint32_t)lb};
    k_small_mul<<<1, SMALL_THREADS, small_smem_bytes(z.L), st>>>(job, R);
    CU(cudaGetLastError());
    return PIMUL_OK;
  }
  Scratch sc;
  sc.A = nd->scratch;
  sc.B = nd->scratch + NOALLOC_N_MAX;
  sc.H = nd->scratch + 2 * NOALLOC_N_MAX;
  sc.aux = reinterpret_cast<uint8_t*>(nd->scratch + 2 * NOALLOC_N_MAX + NOALLOC_WIN_MAX);
  Launcher X{st, false, R};  // no statistics hook: its event timing would create CUDA events
  run_multiply(X, d_a, la, d_b, lb, d_out, sc, z);
  CU(cudaGetLastError());
  return PIMUL_OK;
}
}  // namespace pimul

extern "C" int pimul_mul_device_noalloc(const uint64_t* d_a, size_t la, const uint64_t* d_b, size_t lb,
                                        uint64_t* d_out, void* stream) {
  if (la == 0 || lb == 0) return PIMUL_OK;
  if (!d_a || !d_b || !d_out) return fail(PIMUL_EINVAL, "null device pointer");
  if (la + lb > NOALLOC_N_MAX / 4)
    return fail(PIMUL_EINVAL, "product too large for the no-alloc scratch: la + lb must be <= 262144 limbs "
                              "(transform length <= 2^20)");
  return mul_device_noalloc(d_a, la, d_b, lb, d_out, (cudaStream_t)stream);
}
