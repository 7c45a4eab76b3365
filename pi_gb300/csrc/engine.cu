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
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <functional>
#include <thread>
#include <unordered_map>
#include <atomic>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "gl.cuh"
#include "ntt_kernels.cuh"
#include "../../include/pimul.h"
#include "hostcopy.h"
#include "splitmerge.h"

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
// Geometry of the HBM passes.  Pass tiles hold 2^12 words (32 KiB plus
// padding, so that five CTAs share an SM) and are processed by 256 threads:
//   first pass (p = 0):   2^R rows x 2^(12-R) columns of the single block
//   middle passes:        2^(9-R) blocks x 2^R rows x 8 columns
//   last pass (S = 1):    2^(12-R) contiguous blocks of 2^R words
// Column tiles read 64-byte (or wider) row segments; first-pass rows hold at
// least 8 consecutive coefficients, one carry window.
constexpr int PASS_THREADS = 256;
constexpr int TILE_LOG = 12;
// Resident CTAs per SM the pass kernels are register-limited for.
#ifndef PIMUL_PASS_MIN_CTAS
#define PIMUL_PASS_MIN_CTAS 5
#endif
constexpr int PASS_MIN_CTAS = PIMUL_PASS_MIN_CTAS;

static inline size_t pass_smem_bytes(int tile_log) { return ((size_t)1 << tile_log) * 17 / 16 * 8 + 512 * 8; }

// Load the 512 forward roots w_512^t into shared memory (round twiddles).
__device__ __forceinline__ void load_tw512(uint64_t* tw, const Roots& R) {
  for (int t = threadIdx.x; t < 512; t += blockDim.x) tw[t] = __ldg(R.lvl + 512 + t);
}

// Elements per thread in a pass tile, processed in groups of 8 so that
// every thread keeps 8 independent global loads in flight.
constexpr int PER_THREAD = (1 << TILE_LOG) / PASS_THREADS;

// One product of a batch (or the only product of a plain call): operands,
// output and its scratch.  Kernels take `const Job* jobs, Job one`: with a
// device array, blockIdx.y selects the product; with jobs == nullptr the
// by-value `one` is used (no descriptor upload for single products).
struct Job {
  const uint64_t* a;
  const uint64_t* b;
  uint64_t* out;
  uint64_t* A;  // N words: a's spectrum (and the product for a square)
  uint64_t* B;  // N words: b's spectrum and the product (unused for a square)
  uint64_t* H;  // high parts of the carry windows
  uint8_t* aux; // carry-scan flags
  uint64_t la, lb;
  const uint64_t* X;  // spectrum added to the pointwise product (a sum of two products), or null
  uint64_t nout;      // output limbs (0: la + lb); with JF_COEFF, output coefficients
  uint32_t flags;     // JF_* roles inside a batch (0: a plain product)
  // A wrapped product runs a cyclic transform of length N shorter than its
  // wrap + N coefficients: coefficient N + i (i < wrap) lands on i.  low
  // holds the exact coefficients 0 .. wrap - 1 (from a short product of the
  // operands' low limbs), so that coefficient i is low[i] and N + i the
  // cyclic value minus low[i].
  const uint64_t* low;
  uint64_t wrap;
};

// Roles of a product inside a batch.  A spectrum shared by several products
// with the same operand b is computed once, by its owner (JF_B_FULL); the
// others point B at it (JF_B_SHARED) and skip b's passes.  With a full
// spectrum in B, k_mid only multiplies and writes the product to A.  An
// addend (JF_ADDEND) produces no output: its pointwise product A * B stays
// in A, where the job it is added to reads it as X.
constexpr uint32_t JF_B_SHARED = 1;
constexpr uint32_t JF_B_FULL = 2;
constexpr uint32_t JF_ADDEND = 4;
// The product's canonical coefficients 0 .. nout - 1 go to out (no carry):
// the low part of a wrapped product.
constexpr uint32_t JF_COEFF = 8;

__device__ __forceinline__ Job job_of(const Job* jobs, const Job& one) {
  if (jobs) return jobs[blockIdx.y];
  return one;
}
__device__ __forceinline__ bool is_square(const Job& J) { return J.a == J.b && J.la == J.lb; }
// b's own passes are skipped for a square and for a borrowed spectrum.
__device__ __forceinline__ bool skips_b(const Job& J) { return is_square(J) || (J.flags & JF_B_SHARED); }
__device__ __forceinline__ bool b_spectrum(const Job& J) { return (J.flags & (JF_B_SHARED | JF_B_FULL)) != 0; }
__host__ __device__ __forceinline__ uint64_t job_nout(const Job& J) { return J.nout ? J.nout : J.la + J.lb; }
// Array a pass works on: 0 = A, 1 = B, 2 = the product array.
__device__ __forceinline__ uint64_t* job_array(const Job& J, int which) {
  if (which == 0) return J.A;
  if (which == 1) return J.B;
  return is_square(J) || b_spectrum(J) ? J.A : J.B;
}

// Forward pass 0 with the limb -> 16-bit coefficient split fused in
// (crates/bignum/src/ntt.rs:640-665): element (i, j) of the tile is
// coefficient n = i * 2^S + j0 + j, i.e. 16-bit slice n % 4 of limb n / 4;
// limbs past nl are zero (the reference's zero tail).  which = 0: operand a,
// 1: operand b (squares skip b).
// twf: the pass's twiddle table (tw_first), or null to compute the twiddles.
template <int R>
__global__ void __launch_bounds__(PASS_THREADS, PASS_MIN_CTAS) k_fwd_first(const Job* jobs, Job one, int which, int L, Roots RT,
                                                                           const uint64_t* __restrict__ twf) {
  constexpr int T = TILE_LOG - R;
  const Job J = job_of(jobs, one);
  if (which == 1 && skips_b(J)) return;
  const uint64_t* __restrict__ limbs = which ? J.b : J.a;
  const uint64_t nl = which ? J.lb : J.la;
  uint64_t* __restrict__ data = which ? J.B : J.A;
  extern __shared__ uint64_t sm[];
  uint64_t* tw = sm + spad(1u << TILE_LOG);
  const int tid = threadIdx.x;
  const int S = L - R;
  const uint64_t j0 = (uint64_t)blockIdx.x << T;
  load_tw512(tw, RT);
  // an operand of at most 2^(L-3) limbs leaves rows 2^(R-1) and up zero
  // (coefficients N/2 and up): they are neither written nor read
  const bool half = 4 * nl <= (1ull << (L - 1));
  // each thread expands whole limbs: 2^R rows (2^(R-1) if half) x 2^(T-2) limbs
  const uint32_t nq = half ? 1u << (R + T - 3) : 1u << (R + T - 2);
  for (uint32_t q = tid; q < nq; q += PASS_THREADS) {
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
  if (half)
    tile_fwd_t<R, T, 0, PASS_THREADS, true>(sm, tw, tid);
  else
    tile_fwd_t<R, T, 0, PASS_THREADS>(sm, tw, tid);
  // element e of this thread: lin = e * 256 + tid, row (e << TL) + (tid >> T),
  // column tid & (2^T - 1); address and twiddle exponent split into a
  // per-thread part and a compile-time part
  constexpr int TL = 8 - T;
  const uint32_t tlo = tid >> T, jj = tid & ((1u << T) - 1);
  const uint64_t gbase = ((uint64_t)tlo << S) + j0 + jj;
  if (twf) {
    // twiddles laid out like the data: one coalesced load each
#pragma unroll 2
    for (int g = 0; g < PER_THREAD; g += 8) {
      uint64_t t8[8];
#pragma unroll
      for (int q = 0; q < 8; q++) t8[q] = __ldg(twf + gbase + ((uint64_t)((g + q) << TL) << S));
#pragma unroll
      for (int q = 0; q < 8; q++)
        data[gbase + ((uint64_t)((g + q) << TL) << S)] = gl::mul(sm[spad((g + q) * PASS_THREADS + tid)], t8[q]);
    }
    return;
  }
  if (L > LVL_MAX) {
    // w^(f (j0 + jj)) = w^(f j0) w^(f jj): the first factor for the tile's
    // 2^R frequencies replaces the round twiddles in tw (the rounds are
    // done), the second (f jj < 4096) comes from the L1-resident near table
    for (uint32_t f = tid; f < (1u << R); f += PASS_THREADS) tw[f] = root_pow32(RT, L, f * (uint32_t)j0, false);
    __syncthreads();
    const uint64_t* __restrict__ nt = near_table(RT, L, false);
    const uint32_t f0 = row_freq_t<R>(tlo);
#pragma unroll 2
    for (int g = 0; g < PER_THREAD; g += 8) {
      uint64_t t8[8];
#pragma unroll
      for (int q = 0; q < 8; q++) {
        const uint32_t f = f0 + row_freq_t<R>((g + q) << TL);
        t8[q] = gl::mul(tw[f], __ldg(nt + f * jj));
      }
#pragma unroll
      for (int q = 0; q < 8; q++)
        data[gbase + ((uint64_t)((g + q) << TL) << S)] = gl::mul(sm[spad((g + q) * PASS_THREADS + tid)], t8[q]);
    }
    return;
  }
  const uint32_t Jc = (uint32_t)(j0 + jj);
  const uint32_t eJ = row_freq_t<R>(tlo) * Jc;
#pragma unroll 2
  for (int g = 0; g < PER_THREAD; g += 8) {
    uint64_t t8[8];
#pragma unroll
    for (int q = 0; q < 8; q++) t8[q] = root_pow32(RT, L, eJ + row_freq_t<R>((g + q) << TL) * Jc, false);
#pragma unroll
    for (int q = 0; q < 8; q++)
      data[gbase + ((uint64_t)((g + q) << TL) << S)] = gl::mul(sm[spad((g + q) * PASS_THREADS + tid)], t8[q]);
  }
}

// Middle column pass: 2^(9-R) blocks x 2^R rows x 2^T columns; forward pass
// twiddles w_M^(f*j) after the rounds, inverse ones before.
// twm: the pass's twiddle table (tw_mid), or null to compute the twiddles.
template <int R, bool FWD>
__global__ void __launch_bounds__(PASS_THREADS, PASS_MIN_CTAS) k_col_mid(const Job* jobs, Job one, int which, int S, Roots RT,
                                                                         const uint64_t* __restrict__ twm) {
  constexpr int T = TILE_LOG - 9, BC = 9 - R;
  constexpr int TL = 8 - T;  // row bits covered by tid >> T
  static_assert(R >= TL, "thread index must stay inside one block's rows");
  constexpr uint32_t TM = (1u << T) - 1, RM = (1u << R) - 1;
  const Job J = job_of(jobs, one);
  if (FWD && which == 1 && skips_b(J)) return;
  if (!FWD && (J.flags & JF_ADDEND)) return;
  uint64_t* __restrict__ data = job_array(J, which);
  extern __shared__ uint64_t sm[];
  uint64_t* tw = sm + spad(1u << TILE_LOG);
  const int tid = threadIdx.x;
  const int mlog = R + S;
  const uint64_t ct = blockIdx.x & ((1u << (S - T)) - 1);
  const uint64_t b0 = ((uint64_t)blockIdx.x >> (S - T)) << BC;
  const uint64_t j0 = ct << T;
  // element q of this thread (lin = q * 256 + tid): block q >> (R - TL), row
  // ((q << TL) & RM) + (tid >> T), column tid & TM
  const uint32_t tlo = tid >> T, jj = tid & TM;
  const uint64_t gbase = (b0 << mlog) + ((uint64_t)tlo << S) + j0 + jj;
  auto gaddr = [&](int q) {
    return gbase + ((uint64_t)(q >> (R - TL)) << mlog) + ((uint64_t)((q << TL) & RM) << S);
  };
#pragma unroll
  for (int q = 0; q < PER_THREAD; q++) cp_async8(sm + spad(q * PASS_THREADS + tid), data + gaddr(q));
  load_tw512(tw, RT);
  cp_async_wait_all();
  __syncthreads();
  const uint32_t Jc = (uint32_t)(j0 + jj);
  if (FWD) {
    tile_fwd_t<R, T, BC, PASS_THREADS>(sm, tw, tid);
    // outgoing pass twiddles w_M^(f*j)
    const uint32_t eJ = row_freq_t<R>(tlo) * Jc;
    // table: twm[r 2^S + j] for row r of the block and column j
    const uint64_t tbase = ((uint64_t)tlo << S) + j0 + jj;
#pragma unroll 1
    for (int g = 0; g < PER_THREAD; g += 8) {
      uint64_t t8[8];
      if (twm) {
#pragma unroll
        for (int q = 0; q < 8; q++) t8[q] = __ldg(twm + tbase + ((uint64_t)(((g + q) << TL) & RM) << S));
      } else {
#pragma unroll
        for (int q = 0; q < 8; q++)
          t8[q] = root_pow32(RT, mlog, eJ + row_freq_t<R>(((g + q) << TL) & RM) * Jc, false);
      }
#pragma unroll
      for (int q = 0; q < 8; q++) data[gaddr(g + q)] = gl::mul(sm[spad((g + q) * PASS_THREADS + tid)], t8[q]);
    }
  } else {
    // incoming pass twiddles w_M^-(f*j), applied by the first inverse round
    // (tile row row0 + k is row (row0 + k) & RM of its block)
    auto ptw = [&](uint32_t row0, int k, uint32_t j) {
      if (twm) return __ldg(twm + ((uint64_t)((row0 & RM) + (uint32_t)k) << S) + j0 + j);
      const uint32_t f = row_freq_t<R>(row0 & RM) + row_freq_t<R>((uint32_t)k);
      return root_pow32(RT, mlog, f * (uint32_t)(j0 + j), true);
    };
    tile_inv_t<R, T, BC, PASS_THREADS, rp_count(R) - 1>(sm, tw, tid, ptw);
#pragma unroll
    for (int q = 0; q < PER_THREAD; q++) data[gaddr(q)] = sm[spad(q * PASS_THREADS + tid)];
  }
}

// Last forward pass (stride 1): 2^(13-R) contiguous blocks of 2^R words, of
// operand a (which = 0) or, for a full spectrum of b (JF_B_FULL), of b.
// Squares skip it: their last pass is fused into k_mid.
template <int R>
__global__ void __launch_bounds__(PASS_THREADS, PASS_MIN_CTAS) k_fwd_last(const Job* jobs, Job one, int which,
                                                                          Roots RT) {
  static_assert(R <= 9 && PASS_THREADS == 256 && TILE_LOG == 12, "eight warps, one 512-word chunk each");
  const Job J = job_of(jobs, one);
  if (is_square(J)) return;
  if (which == 1 && !(J.flags & JF_B_FULL)) return;
  extern __shared__ uint64_t sm[];
  uint64_t* tw = sm + spad(1u << TILE_LOG);
  // warp w owns the tile's 512-word chunk w (whole blocks): after the round
  // twiddles are staged, only __syncwarp separates its rounds
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint64_t* chunk = (which ? J.B : J.A) + ((uint64_t)blockIdx.x << TILE_LOG) + ((uint32_t)warp << 9);
  uint64_t* smc = sm + spad((uint32_t)warp << 9);
#pragma unroll
  for (int q = 0; q < 16; q++) cp_async8(smc + spad(q * 32 + lane), chunk + q * 32 + lane);
  load_tw512(tw, RT);
  cp_async_wait_all();
  __syncthreads();
  chunk_fwd_t<R>(smc, tw, lane);
#pragma unroll
  for (int q = 0; q < 16; q++) chunk[q * 32 + lane] = smc[spad(q * 32 + lane)];
}

// Fused middle of the multiply on one contiguous tile: last forward pass of
// b, pointwise product with the spectrum of a (plus X for a sum of two
// products; times N^-1, the inverse's 1/N, crates/bignum/src/ntt.rs:383-390
// and 845-853), first inverse pass; the result overwrites b's array.  A
// square transforms and squares a's array in place; with b's full spectrum
// in B (shared or owned) the last pass is skipped and the result goes to A.
// EXT = false: plain products only (no shared spectrum, no addend), the
// form every single product and every batch without those roles uses.
// ninv = 0: no scaling here (the inverse first pass's twiddle table carries N^-1).
template <int R, bool EXT>
__global__ void __launch_bounds__(PASS_THREADS, PASS_MIN_CTAS) k_mid(const Job* jobs, Job one, uint64_t ninv, Roots RT) {
  static_assert(R <= 9 && PASS_THREADS == 256 && TILE_LOG == 12, "eight warps, one 512-word chunk each");
  const Job J = job_of(jobs, one);
  if (EXT && (J.flags & JF_ADDEND)) return;
  const bool sq = is_square(J), spec = EXT && b_spectrum(J);
  const uint64_t* cin = sq ? J.A : J.B;
  uint64_t* cout = sq || spec ? J.A : J.B;
  const uint64_t* a = J.A;
  const uint64_t* __restrict__ X = J.X;
  extern __shared__ uint64_t sm[];
  uint64_t* tw = sm + spad(1u << TILE_LOG);
  const int tid = threadIdx.x;
  const uint64_t off = (uint64_t)blockIdx.x << TILE_LOG;
  // warp w owns the tile's 512-word chunk w (whole blocks) from load to store
  const int warp = tid >> 5, lane = tid & 31;
  const uint64_t coff = off + ((uint32_t)warp << 9);
  uint64_t* smc = sm + spad((uint32_t)warp << 9);
#pragma unroll
  for (int q = 0; q < 16; q++) cp_async8(smc + spad(q * 32 + lane), cin + coff + q * 32 + lane);
  // a's (and the addend's) tile is read after b's rounds: start it towards
  // L2 now (tiles are 32 KB at 32 KB offsets of 256-byte aligned arrays)
  if (tid == 0) {
    if (!sq) prefetch_l2_bulk(a + off, (8u << TILE_LOG));
    if (EXT && X) prefetch_l2_bulk(X + off, (8u << TILE_LOG));
  }
  load_tw512(tw, RT);
  cp_async_wait_all();
  __syncthreads();
  if (!spec) chunk_fwd_t<R>(smc, tw, lane);
  if (EXT && X) {
    // sum of two products: a b + X, then the inverse rounds
#pragma unroll 4
    for (int q = 0; q < 16; q++) {
      const uint32_t lin = q * 32 + lane;
      uint64_t x = smc[spad(lin)];
      uint64_t p = gl::add(gl::mul(x, sq ? x : a[coff + lin]), X[coff + lin]);
      smc[spad(lin)] = ninv ? gl::mul(p, ninv) : p;
    }
    __syncwarp();
    chunk_inv_t<R>(smc, tw, lane);
  } else {
    // the pointwise product (times N^-1 when the inverse first pass's table
    // does not carry it) enters the first inverse round as lazy products
    auto pw = [&](uint32_t row0, int k, uint32_t) {
      const uint32_t lin = row0 + (uint32_t)k;
      const uint64_t y = sq ? smc[spad(lin)] : a[coff + lin];
      return ninv ? gl::mul(y, ninv) : y;
    };
    chunk_inv_t<R>(smc, tw, lane, pw);
  }
#pragma unroll
  for (int q = 0; q < 16; q++) cout[coff + q * 32 + lane] = smc[spad(q * 32 + lane)];
}

// Addends: A <- A * B (spectra, element by element), read later as X.
__global__ void __launch_bounds__(256) k_pointwise_addend(const Job* jobs, Job one, uint64_t n) {
  const Job J = job_of(jobs, one);
  if (!(J.flags & JF_ADDEND)) return;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    J.A[i] = gl::mul(J.A[i], J.B[i]);
}

// ---- carry normalisation (crates/bignum/src/ntt.rs:676-791) --------------
// Coefficients are grouped in windows of 8 (= 2 limbs).  Window w has value
// V_w = sum_t c[8w+t] 2^(16t) = lo_w + hi_w 2^128 (hi_w < 2^49).  The
// product is sum_w (lo_w + hi_(w-1)) 2^(128w); s_w = lo_w + hi_(w-1) may
// carry one bit (g_w) into window w+1, which a run of all-ones windows (p_w)
// propagates.  Carries are resolved with a carry-lookahead scan over (g, p)
// bit vectors: with A = g|p and B = g, the carry into each window is bit w of
// (A + B + cin) ^ A ^ B.
constexpr int WIN_COEFFS = 8;
constexpr int WIN_LIMBS = 2;

struct Win2 {
  uint64_t l[2];
  uint64_t hi;
};

// Window value from 8 canonical coefficients (u128 accumulator, as the
// reference's unpack loop, ntt.rs:694-707).
__device__ __forceinline__ Win2 fold8(const uint64_t* c8) {
  Win2 r;
  unsigned __int128 acc = 0;
#pragma unroll
  for (int k = 0; k < 2; k++) {
#pragma unroll
    for (int q = 0; q < 4; q++) acc += (unsigned __int128)c8[4 * k + q] << (16 * q);
    r.l[k] = (uint64_t)acc;
    acc >>= 64;
  }
  r.hi = (uint64_t)acc;
  return r;
}

// 16-coefficient windows of the one-CTA multiply (its own carry chain).
struct Win {
  uint64_t l[4];
  uint64_t hi;
};

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

constexpr int CARRY_THREADS = 256;  // windows per CTA

// Windows of an output of nout limbs (4 nout - 1 coefficients).
__host__ __device__ __forceinline__ uint64_t n_windows_out(uint64_t nout) {
  return (4 * nout - 1 + WIN_COEFFS - 1) / WIN_COEFFS;
}
__host__ __device__ __forceinline__ uint64_t n_windows(uint64_t la, uint64_t lb) { return n_windows_out(la + lb); }
__host__ __device__ __forceinline__ uint64_t n_chunks(uint64_t nwin) {
  return (nwin + CARRY_THREADS - 1) / CARRY_THREADS;
}
// Carry-scan flag layout inside Job::aux: per warp (A, B) masks, then per
// chunk the (g, p) byte and the carry-in byte.
__host__ __device__ __forceinline__ uint64_t aux_bytes_for(uint64_t nwin) {
  uint64_t nc = n_chunks(nwin);
  return nc * (CARRY_THREADS / 32) * 8 + 2 * nc + 64;
}

// Inverse pass 0 (natural order out) fused with the window fold: each tile
// row holds 2^T consecutive coefficients = 2^(T-3) windows; every window
// writes its low 2 limbs to the output and its high part to H.
// twi: the pass's twiddle table (tw_first, inverse, with N^-1), or null to
// compute the twiddles (the caller then scales by N^-1 in k_mid).
template <int R>
__global__ void __launch_bounds__(PASS_THREADS, PASS_MIN_CTAS) k_inv_first_carry(const Job* jobs, Job one, int L, Roots RT,
                                                                                 const uint64_t* __restrict__ twi) {
  constexpr int T = TILE_LOG - R;
  const Job J = job_of(jobs, one);
  if (J.flags & JF_ADDEND) return;
  const uint64_t* __restrict__ data = job_array(J, 2);
  uint64_t* __restrict__ out = J.out;
  uint64_t* __restrict__ H = J.H;
  const uint64_t nlimbs = job_nout(J), nwin = n_windows_out(nlimbs);
  extern __shared__ uint64_t sm[];
  uint64_t* tw = sm + spad(1u << TILE_LOG);
  const int tid = threadIdx.x;
  const int S = L - R;
  const uint64_t j0 = (uint64_t)blockIdx.x << T;
  constexpr int TL = 8 - T;
  const uint64_t gbase = ((uint64_t)(tid >> T) << S) + j0 + (tid & ((1u << T) - 1));
#pragma unroll
  for (int q = 0; q < PER_THREAD; q++)
    cp_async8(sm + spad(q * PASS_THREADS + tid), data + gbase + ((uint64_t)(q << TL) << S));
  if (twi) {
    load_tw512(tw, RT);
    cp_async_wait_all();
    __syncthreads();
    // inverse pass twiddles (times N^-1) from the table, laid out like the data
    auto ptw = [&](uint32_t row0, int k, uint32_t j) {
      return __ldg(twi + ((uint64_t)(row0 + (uint32_t)k) << S) + j0 + j);
    };
    tile_inv_t<R, T, 0, PASS_THREADS, rp_count(R) - 1>(sm, tw, tid, ptw);
  } else if (L > LVL_MAX) {
    // inverse pass twiddles w^-(f (j0 + j)) = w^-(f j0) w^-(f j): the first
    // factor for the tile's 2^R frequencies is staged in tw, which the
    // first inverse round does not need for round twiddles (its sub-problems
    // are the radix itself); the round twiddles are loaded after it
    constexpr int QL = rp_count(R) - 1;
    static_assert(rp_mlog(R, QL) == rp_bits(R, QL), "the first inverse round has no round twiddles");
    for (uint32_t f = tid; f < (1u << R); f += PASS_THREADS) tw[f] = root_pow32(RT, L, f * (uint32_t)j0, true);
    cp_async_wait_all();
    __syncthreads();
    const uint64_t* __restrict__ nt = near_table(RT, L, true);
    auto ptw = [&](uint32_t row0, int k, uint32_t j) {
      const uint32_t f = row_freq_t<R>(row0) + row_freq_t<R>((uint32_t)k);
      return gl::mul(tw[f], __ldg(nt + f * j));
    };
    round_inv_t<R, T, 0, rp_bits(R, QL), rp_mlog(R, QL), PASS_THREADS>(sm, tw, tid, ptw);
    __syncthreads();
    load_tw512(tw, RT);
    __syncthreads();
    tile_inv_t<R, T, 0, PASS_THREADS, QL - 1>(sm, tw, tid);
  } else {
    load_tw512(tw, RT);
    cp_async_wait_all();
    __syncthreads();
    // inverse pass twiddles w_N^-(f*j), applied by the first inverse round
    auto ptw = [&](uint32_t row0, int k, uint32_t j) {
      const uint32_t f = row_freq_t<R>(row0) + row_freq_t<R>((uint32_t)k);
      return root_pow32(RT, L, f * (uint32_t)(j0 + j), true);
    };
    tile_inv_t<R, T, 0, PASS_THREADS, rp_count(R) - 1>(sm, tw, tid, ptw);
  }
  const bool coeff = (J.flags & JF_COEFF) != 0;
  const uint64_t wtop = (1ull << L) >> 3;  // a wrapped product's windows past the transform: w + wtop
  for (uint32_t q = tid; q < (1u << (TILE_LOG - 3)); q += PASS_THREADS) {
    uint32_t i = q >> (T - 3), k = q & ((1u << (T - 3)) - 1);
    uint64_t w = ((((uint64_t)i << S) + j0) >> 3) + k;
    uint64_t c[8];
    uint32_t b = (i << T) + 8 * k;
#pragma unroll
    for (int t = 0; t < 8; t++) c[t] = gl::canon(sm[spad(b + t)]);
    if (coeff) {
#pragma unroll
      for (int t = 0; t < 8; t++)
        if (8 * w + t < nlimbs) out[8 * w + t] = c[t];
      continue;
    }
    if (w >= nwin) continue;
    if (J.wrap) {
      // coefficient 8w + t: low[8w + t] below wrap; N + 8w + t: the rest of the cyclic value
      uint64_t d[8];
#pragma unroll
      for (int t = 0; t < 8; t++) {
        const uint64_t pos = 8 * w + t;
        const uint64_t lo = pos < J.wrap ? J.low[pos] : c[t];
        d[t] = c[t] - lo;
        c[t] = lo;
      }
      const uint64_t w2 = w + wtop;
      if (w2 < nwin) {
        const Win2 v2 = fold8(d);
#pragma unroll
        for (int t = 0; t < 2; t++)
          if (2 * w2 + t < nlimbs) out[2 * w2 + t] = v2.l[t];
        H[w2] = v2.hi;
      }
    }
    Win2 v = fold8(c);
#pragma unroll
    for (int t = 0; t < 2; t++)
      if (2 * w + t < nlimbs) out[2 * w + t] = v.l[t];
    H[w] = v.hi;
  }
}

// Carry pass 1 (grid.x = chunk, grid.y = product): s_w = lo_w + hi_(w-1)
// written back as the output limbs; per window (g, p), per warp the (A, B)
// masks, per CTA the chunk's carry out for carry in 0 and 1.
__global__ void __launch_bounds__(CARRY_THREADS) k_carry_local(const Job* jobs, Job one) {
  const Job J = job_of(jobs, one);
  if (J.flags & (JF_ADDEND | JF_COEFF)) return;
  const uint64_t nlimbs = job_nout(J), nwin = n_windows_out(nlimbs), nchunk = n_chunks(nwin);
  if (blockIdx.x >= nchunk) return;  // uniform per CTA
  uint64_t* __restrict__ out = J.out;
  const uint64_t* __restrict__ H = J.H;
  uint32_t* masks = reinterpret_cast<uint32_t*>(J.aux);
  uint8_t* chunk_gp = J.aux + nchunk * (CARRY_THREADS / 32) * 8;
  __shared__ uint32_t sA[CARRY_THREADS / 32], sB[CARRY_THREADS / 32];
  const uint64_t w = (uint64_t)blockIdx.x * CARRY_THREADS + threadIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  bool g = false, p = false;
  if (w < nwin) {
    uint64_t base = WIN_LIMBS * w;
    uint64_t l0 = base + 0 < nlimbs ? out[base + 0] : 0;
    uint64_t l1 = base + 1 < nlimbs ? out[base + 1] : 0;
    uint64_t hprev = w > 0 ? H[w - 1] : 0;
    uint64_t s0 = l0 + hprev;
    uint64_t c = s0 < hprev;
    uint64_t s1 = l1 + c;  c = c && s1 == 0;
    g = c != 0;
    p = (s0 & s1) == ~0ull;
    if (base + 0 < nlimbs) out[base + 0] = s0;
    if (base + 1 < nlimbs) out[base + 1] = s1;
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

// Carry pass 2 (one CTA per product): carry into every chunk.  Each thread
// walks a contiguous segment of chunks, the segment results are chained by
// thread 0.
constexpr int SCAN_THREADS = 1024;
// Carry function of a run of chunks as two bits: bit 0 = carry out for carry
// in 0, bit 1 = carry out for carry in 1 (the chunk's (g, p) byte has the
// same layout).  Identity: 0b10.  Running `first`, then `then`:
__device__ __forceinline__ uint32_t cf_then(uint32_t first, uint32_t then) {
  const uint32_t o0 = (then >> (first & 1)) & 1;
  const uint32_t o1 = (then >> ((first >> 1) & 1)) & 1;
  return o0 | (o1 << 1);
}

// Carry pass 2 (one CTA per product): the carry into every chunk, as an
// exclusive scan of the chunks' carry functions.  Each thread composes a
// contiguous run (16-byte loads), the CTA scans the runs with warp shuffles,
// and each thread writes its run's carries in.
__global__ void __launch_bounds__(SCAN_THREADS) k_carry_scan(const Job* jobs, Job one) {
  const Job J = job_of(jobs, one);
  if (J.flags & (JF_ADDEND | JF_COEFF)) return;
  const uint64_t nchunk = n_chunks(n_windows_out(job_nout(J)));
  const uint8_t* chunk_gp = J.aux + nchunk * (CARRY_THREADS / 32) * 8;  // 64-byte aligned
  uint8_t* chunk_cin = const_cast<uint8_t*>(chunk_gp) + nchunk;
  __shared__ uint32_t warp_f[SCAN_THREADS / 32];
  const uint64_t per = ((nchunk + SCAN_THREADS - 1) / SCAN_THREADS + 15) & ~15ull;  // a multiple of 16
  const uint64_t lo = threadIdx.x * per, hi = lo + per < nchunk ? lo + per : nchunk;
  uint32_t f = 2;  // identity
  uint64_t k = lo;
  for (; k + 16 <= hi; k += 16) {
    const uint4 v = *reinterpret_cast<const uint4*>(chunk_gp + k);
    const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int q = 0; q < 16; q++) f = cf_then(f, (w[q >> 2] >> (8 * (q & 3))) & 3);
  }
  for (; k < hi; k++) f = cf_then(f, chunk_gp[k] & 3);
  // exclusive scan of the threads' functions
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t inc = f;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t prev = __shfl_up_sync(0xFFFFFFFFu, inc, o);
    if (lane >= o) inc = cf_then(prev, inc);
  }
  if (lane == 31) warp_f[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    uint32_t winc = lane < SCAN_THREADS / 32 ? warp_f[lane] : 2;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t prev = __shfl_up_sync(0xFFFFFFFFu, winc, o);
      if (lane >= o) winc = cf_then(prev, winc);
    }
    const uint32_t wexc = __shfl_up_sync(0xFFFFFFFFu, winc, 1);
    __syncwarp();
    if (lane < SCAN_THREADS / 32) warp_f[lane] = lane ? wexc : 2;
  }
  __syncthreads();
  const uint32_t in_warp = __shfl_up_sync(0xFFFFFFFFu, inc, 1);
  const uint32_t before = cf_then(warp_f[warp], lane ? in_warp : 2);
  uint32_t cin = before & 1;  // carry into this run (the product's carry in is 0)
  for (k = lo; k < hi; k++) {
    chunk_cin[k] = (uint8_t)cin;
    cin = (chunk_gp[k] >> cin) & 1;
  }
}

// Carry pass 3: add the incoming carry to every window that receives one.
__global__ void __launch_bounds__(CARRY_THREADS) k_carry_apply(const Job* jobs, Job one) {
  const Job J = job_of(jobs, one);
  if (J.flags & (JF_ADDEND | JF_COEFF)) return;
  const uint64_t nlimbs = job_nout(J), nwin = n_windows_out(nlimbs), nchunk = n_chunks(nwin);
  if (blockIdx.x >= nchunk) return;
  uint64_t* __restrict__ out = J.out;
  const uint32_t* masks = reinterpret_cast<const uint32_t*>(J.aux);
  const uint8_t* chunk_cin = J.aux + nchunk * (CARRY_THREADS / 32) * 8 + nchunk;
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
    uint64_t base = WIN_LIMBS * w;
    for (int k = 0; k < WIN_LIMBS && base + k < nlimbs; k++) {
      if (++out[base + k] != 0) break;
    }
  }
}

// ---- whole multiply in one CTA (N <= 2^SMALL_LOG_MAX) --------------------
constexpr int SMALL_THREADS = 256;
constexpr int SMALL_LOG_MAX = 12;

// Dynamic shared memory of the one-CTA multiply for N = 2^L (two padded arrays).
__host__ __device__ __forceinline__ size_t small_smem_bytes(int L) { return 2 * (((size_t)1 << L) * 17 / 16) * 8; }

struct SmallJob {
  const uint64_t* a;
  const uint64_t* b;
  uint64_t* out;
  uint32_t la, lb;
};

// Threads per product: an eighth of the transform length (one radix-8
// butterfly per thread and round), at least a warp; SMALL_THREADS / G
// products of one length run side by side in a CTA.
__host__ __device__ __forceinline__ int small_group_threads(int L) {
  const int g = (1 << L) / 8;
  return g < 32 ? 32 : (g > SMALL_THREADS ? SMALL_THREADS : g);
}
// Dynamic shared memory of a CTA running products of length 2^L.
__host__ __device__ __forceinline__ size_t small_cta_smem(int L) {
  return (size_t)(SMALL_THREADS / small_group_threads(L)) * small_smem_bytes(L);
}

// count (<= SMALL_THREADS / G(L)) consecutive jobs of length 2^L from first.
struct SmallChunk {
  uint32_t first, count;
  int L;
};

// Forward (or unscaled inverse) transforms of NA arrays of 2^L words by a
// group of NT threads: the pass kernels' rounds (radix 8, then 4) with
// compile-time geometry, each round's twiddles applied as lazy products by
// the next one, from the 4096-entry table of 4096th roots; one CTA barrier
// per round.  Bit i of act: array i is transformed (idle groups and skipped
// arrays pass the barriers only).
template <int L, int NT, int NA, int Q = 0>
__device__ __forceinline__ void group_fwd_c(uint64_t* a0, uint64_t* a1, uint64_t* a2, const uint64_t* tw, int tid,
                                            unsigned act) {
  if constexpr (Q < rp_count(L)) {
    constexpr int B = rp_bits(L, Q), MLOG = rp_mlog(L, Q);
    constexpr int PB = Q > 0 ? rp_bits(L, Q - 1) : 0, PMLOG = Q > 0 ? rp_mlog(L, Q - 1) : 0;
    if (act & 1) round_fwd_t<L, 0, 0, B, MLOG, NT, PB, PMLOG, 12>(a0, tw, tid);
    if constexpr (NA > 1) if (act & 2) round_fwd_t<L, 0, 0, B, MLOG, NT, PB, PMLOG, 12>(a1, tw, tid);
    if constexpr (NA > 2) if (act & 4) round_fwd_t<L, 0, 0, B, MLOG, NT, PB, PMLOG, 12>(a2, tw, tid);
    __syncthreads();
    group_fwd_c<L, NT, NA, Q + 1>(a0, a1, a2, tw, tid, act);
  }
}

template <int L, int NT, int Q = rp_count(L) - 1>
__device__ __forceinline__ void group_inv_c(uint64_t* a0, const uint64_t* tw, int tid, bool act) {
  if constexpr (Q >= 0) {
    if (act) round_inv_t<L, 0, 0, rp_bits(L, Q), rp_mlog(L, Q), NT, NoPassTw, 12>(a0, tw, tid, NoPassTw());
    __syncthreads();
    group_inv_c<L, NT, Q - 1>(a0, tw, tid, act);
  }
}

// One product by the G threads of a group (gtid = thread in the group, gw0
// = the CTA-wide index of the group's first warp).  Inactive groups run
// every barrier and ballot with no work, so a CTA's groups stay in step.
__device__ void small_multiply(const SmallJob& job, bool active, int L, const Roots& R, uint64_t* smA, uint64_t* smB,
                               int gtid, int G, int gw0) {
  const int tid = threadIdx.x;
  const uint32_t la = active ? job.la : 0, lb = active ? job.lb : 0;
  const uint32_t N = 1u << L;
  const uint32_t n_out = active ? 4 * la + 4 * lb - 1 : 0;
  const bool square = active && job.a == job.b && la == lb;
  // one limb per thread and step -> its four 16-bit coefficients
  for (uint32_t l = gtid; active && l < N / 4; l += G) {
    const uint64_t xa = l < la ? job.a[l] : 0;
#pragma unroll
    for (int q = 0; q < 4; q++) smA[spad(4 * l + q)] = (xa >> (16 * q)) & 0xFFFF;
    if (!square) {
      const uint64_t xb = l < lb ? job.b[l] : 0;
#pragma unroll
      for (int q = 0; q < 4; q++) smB[spad(4 * l + q)] = (xb >> (16 * q)) & 0xFFFF;
    }
  }
  __syncthreads();
  TileGeom g{L, 0, 0};
  const int rt = active ? gtid : (1 << 30);  // an inactive group's rounds do no work
  tile_dft_fwd(smA, g, R, rt, G);
  tile_dft_fwd(smB, g, R, square ? (1 << 30) : rt, G);
  // times N^-1 = 2^(-L): with 2^96 = -1 and 2^64 = 2^32 - 1 (mod p),
  // 2^(-L) = -2^(96-L) = p - (2^(64-L) - 2^(32-L)) for 1 <= L <= 32
  const uint64_t ninv = gl::P - ((1ull << (64 - L)) - (1ull << (32 - L)));
  for (uint32_t i = gtid; active && i < N; i += G) {
    uint64_t x = smA[spad(i)];
    uint64_t y = square ? x : smB[spad(i)];
    smA[spad(i)] = gl::mul(gl::mul(x, y), ninv);
  }
  __syncthreads();
  tile_dft_inv(smA, g, R, rt, G);
  // carry: windows of 16 coefficients, one per thread (N/16 <= G)
  const uint32_t nwin = (n_out + 15) / 16, nl = la + lb;
  uint64_t* sH = smB;  // reuse: B no longer needed
  __shared__ uint32_t sA[SMALL_THREADS / 32], sBm[SMALL_THREADS / 32];
  Win v{{0, 0, 0, 0}, 0};
  const uint32_t w = gtid;
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
  for (int k = gw0; k < (tid >> 5); k++) {
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

// Chunks of same-length products; with device lists the CTAs stride over
// the chunks (a persistent kernel over a size-sorted batch).  jobs ==
// nullptr: the single product `one`.
__global__ void __launch_bounds__(SMALL_THREADS, 4) k_small_mul(const SmallJob* jobs, const SmallChunk* chunks,
                                                               SmallJob one, uint32_t nchunks, Roots R) {
  extern __shared__ uint64_t sm[];
  for (uint32_t k = blockIdx.x; k < nchunks; k += gridDim.x) {
    SmallChunk ch;
    if (chunks) {
      ch = chunks[k];
    } else {
      const uint32_t n_out = 4 * one.la + 4 * one.lb - 1;
      int L = 0;
      while ((1u << L) < n_out) L++;
      ch = SmallChunk{0, 1, L};
    }
    const int G = small_group_threads(ch.L);
    const uint32_t grp = threadIdx.x / G;
    const bool active = grp < ch.count;
    const SmallJob job = active ? (jobs ? jobs[ch.first + grp] : one) : SmallJob{};
    const uint32_t sp = spad(1u << ch.L);
    uint64_t* base = sm + (size_t)grp * 2 * sp;
    small_multiply(job, active, ch.L, R, base, base + sp, (int)(threadIdx.x % G), G, (int)(grp * G / 32));
    __syncthreads();
  }
}

// ---- merged binary-splitting levels (one node pair per thread group) ------
// The lowest levels of a Chudnovsky splitting segment hold hundreds of
// thousands of node pairs whose products all fit one CTA's shared memory.
// A group of G = N/8 threads merges one pair (L, R) into
//   P = P_L P_R,  Q = Q_L Q_R,  T = T_L Q_R + P_L T_R
// (magnitudes; crates/pi-core/src/algorithm/chudnovsky.rs:377-413).  The
// spectra of Q_R and P_L serve two products each and T's two products are
// added in the transform domain: six forward and three inverse transforms
// per pair instead of eight and four, no temporaries in HBM and no separate
// addition.  Three padded arrays per group; every CTA holds 512 threads and
// 3 * 2^12 padded words whatever the level's length (2^L / 8 threads and
// 3 * 2^L words per group).
constexpr int MERGE_THREADS = 512;

struct MergeLevel {
  const uint64_t* in;
  const uint32_t* in_len;
  uint64_t* out;
  uint32_t* out_len;
  uint32_t sp, sq, st, op, oq, ot;
  uint32_t n_in;
  int L;
  int* bad;
};

__host__ __device__ __forceinline__ int merge_group_threads(int L) {
  const int g = (1 << L) / 8;
  return g < 32 ? 32 : g;
}
__host__ __device__ __forceinline__ size_t merge_cta_smem(int L) {
  return (size_t)(MERGE_THREADS / merge_group_threads(L)) * 3 * spad(1u << L) * 8;
}

// Limbs x[0..n) -> 16-bit coefficients of an array of 2^Lp words (zero tail).
__device__ __forceinline__ void group_pack(uint64_t* sm, const uint64_t* x, uint32_t n, int Lp, int tid, int G) {
  for (uint32_t l = tid; l < (1u << Lp) / 4; l += G) {
    const uint64_t v = l < n ? x[l] : 0;
#pragma unroll
    for (int q = 0; q < 4; q++) sm[spad(4 * l + q)] = (v >> (16 * q)) & 0xFFFF;
  }
}

// Carry normalisation of a group's inverse-transformed array (exact
// convolution values, below 2^45) into nl limbs at out, one 16-coefficient
// window per thread (nl <= 2^Lp / 4 + 1, so the windows fit G = 2^Lp / 8
// threads); sH (a free array) holds the windows' high parts.  Returns the
// trimmed length to every thread of the group.  Same window arithmetic as
// the one-CTA multiply above.
__device__ uint32_t group_carry_store(const uint64_t* smX, int Lp, uint32_t nl, uint64_t* out, uint64_t* sH,
                                      bool active, int gtid, int G, int gw0, uint32_t* sA, uint32_t* sBm,
                                      uint32_t* sTop) {
  const int tid = threadIdx.x;
  const uint32_t N = 1u << Lp;
  const uint32_t n_out = active && nl ? 4 * nl - 1 : 0;
  const uint32_t nwin = (n_out + 15) / 16;
  const uint32_t w = gtid;
  Win v{{0, 0, 0, 0}, 0};
  if (w < nwin) {
    uint64_t c[16];
#pragma unroll
    for (int t = 0; t < 16; t++) {
      const uint32_t idx = 16 * w + t;
      c[t] = idx < N ? gl::canon(smX[spad(idx)]) : 0;
    }
    v = fold16(c, 1);
  }
  __syncthreads();
  if (w < nwin) sH[w] = v.hi;
  __syncthreads();
  const uint64_t hprev = (w > 0 && w - 1 < nwin) ? sH[w - 1] : 0;
  uint64_t s0 = v.l[0] + hprev;
  uint64_t c = s0 < hprev;
  uint64_t s1 = v.l[1] + c;  c = c && s1 == 0;
  uint64_t s2 = v.l[2] + c;  c = c && s2 == 0;
  uint64_t s3 = v.l[3] + c;  c = c && s3 == 0;
  const bool gg = w < nwin && c;
  const bool pp = w < nwin && (s0 & s1 & s2 & s3) == ~0ull;
  const uint32_t A = __ballot_sync(0xFFFFFFFFu, gg || pp), Bm = __ballot_sync(0xFFFFFFFFu, gg);
  if ((tid & 31) == 0) {
    sA[tid >> 5] = A;
    sBm[tid >> 5] = Bm;
  }
  __syncthreads();
  uint32_t cin = 0;
  for (int k = gw0; k < (tid >> 5); k++) {
    const uint64_t s = (uint64_t)sA[k] + sBm[k] + cin;
    cin = (uint32_t)(s >> 32);
  }
  const uint32_t carries = (A + Bm + cin) ^ A ^ Bm;
  if ((carries >> (tid & 31)) & 1) {
    if (++s0 == 0) if (++s1 == 0) if (++s2 == 0) ++s3;
  }
  uint32_t top = 0;
  if (w < nwin) {
    const uint32_t base = 4 * w;
    const uint64_t s[4] = {s0, s1, s2, s3};
#pragma unroll
    for (int q = 0; q < 4; q++)
      if (base + q < nl) {
        out[base + q] = s[q];
        if (s[q]) top = base + q + 1;
      }
  }
  top = __reduce_max_sync(0xFFFFFFFFu, top);
  if ((tid & 31) == 0) sTop[tid >> 5] = top;
  __syncthreads();
  uint32_t t = 0;
  for (int k = gw0; k < gw0 + G / 32; k++) t = max(t, sTop[k]);
  __syncthreads();  // sTop is reused by the next call
  return t;
}

// One node pair (pair = true) or the copy of an odd last node (copy = true)
// by one group of G = 2^L / 8 threads; an idle group passes the same
// barriers.  Every pair of the level runs transforms of 2^L points (a pair
// that needs fewer gets a longer transform, which changes nothing).
template <int L>
__device__ void merge_item(const MergeLevel& M, const uint64_t* tw, uint32_t item, bool pair, bool copy,
                           uint64_t* X1, uint64_t* X2, uint64_t* X3, int gtid, int gw0, uint32_t* sA, uint32_t* sBm,
                           uint32_t* sTop) {
  constexpr int G = (1 << L) / 8;
  constexpr uint32_t N = 1u << L;
  const size_t in_stride = (size_t)M.sp + M.sq + M.st, out_stride = (size_t)M.op + M.oq + M.ot;
  uint64_t* zp = M.out + (size_t)item * out_stride;
  uint64_t* zq = zp + M.op;
  uint64_t* zt = zq + M.oq;
  if (copy) {
    const uint32_t i = M.n_in - 1;
    const uint64_t* p = M.in + (size_t)i * in_stride;
    const uint32_t pn = M.in_len[3 * i], qn = M.in_len[3 * i + 1], tn = M.in_len[3 * i + 2];
    for (uint32_t k = gtid; k < pn; k += G) zp[k] = p[k];
    for (uint32_t k = gtid; k < qn; k += G) zq[k] = p[M.sp + k];
    for (uint32_t k = gtid; k < tn; k += G) zt[k] = p[M.sp + M.sq + k];
    if (gtid == 0) {
      M.out_len[3 * item] = pn;
      M.out_len[3 * item + 1] = qn;
      M.out_len[3 * item + 2] = tn;
    }
  }
  uint32_t pl = 0, ql = 0, tl = 0, pr = 0, qr = 0, tr = 0;
  const uint64_t *PL = nullptr, *QL = nullptr, *TL = nullptr, *PR = nullptr, *QR = nullptr, *TR = nullptr;
  if (pair) {
    const uint32_t l = 2 * item, r = l + 1;
    pl = M.in_len[3 * l], ql = M.in_len[3 * l + 1], tl = M.in_len[3 * l + 2];
    pr = M.in_len[3 * r], qr = M.in_len[3 * r + 1], tr = M.in_len[3 * r + 2];
    PL = M.in + (size_t)l * in_stride, QL = PL + M.sp, TL = QL + M.sq;
    PR = M.in + (size_t)r * in_stride, QR = PR + M.sp, TR = QR + M.sq;
  }
  const uint32_t n_p = pl + pr, n_q = ql + qr, n_t = max(tl + qr, pl + tr) + 1;
  // output coefficients of the longest product: 4 len - 1 <= 2^L
  const uint32_t need = max(max(n_p, n_q), max(tl + qr, pl + tr));
  const bool fits = 4ull * need <= N + 1ull && n_p <= M.op && n_q <= M.oq && n_t <= M.ot;
  if (pair && !fits && gtid == 0) atomicExch(M.bad, 1);
  const bool act = pair && fits;
  // N^-1 = 2^-L = p - (2^(64-L) - 2^(32-L))  (2^96 = -1, 2^64 = 2^32 - 1)
  constexpr uint64_t ninv = gl::P - ((1ull << (64 - L)) - (1ull << (32 - L)));

  // Q_R, T_L, Q_L: X2 <- T_L Q_R, X3 <- Q_L Q_R N^-1
  if (act) {
    group_pack(X1, QR, qr, L, gtid, G);
    group_pack(X2, TL, tl, L, gtid, G);
    group_pack(X3, QL, ql, L, gtid, G);
  }
  __syncthreads();
  group_fwd_c<L, G, 3>(X1, X2, X3, tw, gtid, act ? 7u : 0u);
  for (uint32_t i = gtid; act && i < N; i += G) {
    const uint64_t y = X1[spad(i)];
    X2[spad(i)] = gl::mul(X2[spad(i)], y);
    X3[spad(i)] = gl::mul(gl::mul(X3[spad(i)], y), ninv);
  }
  __syncthreads();
  group_inv_c<L, G>(X3, tw, gtid, act);
  const uint32_t q_len = group_carry_store(X3, L, n_q, zq, X1, act, gtid, G, gw0, sA, sBm, sTop);
  // P_L, T_R: X2 <- (T_L Q_R + P_L T_R) N^-1, X1 keeps P_L's spectrum
  if (act) {
    group_pack(X1, PL, pl, L, gtid, G);
    group_pack(X3, TR, tr, L, gtid, G);
  }
  __syncthreads();
  group_fwd_c<L, G, 2>(X1, X3, nullptr, tw, gtid, act ? 3u : 0u);
  for (uint32_t i = gtid; act && i < N; i += G)
    X2[spad(i)] = gl::mul(gl::add(X2[spad(i)], gl::mul(X1[spad(i)], X3[spad(i)])), ninv);
  __syncthreads();
  group_inv_c<L, G>(X2, tw, gtid, act);
  const uint32_t t_len = group_carry_store(X2, L, n_t, zt, X3, act, gtid, G, gw0, sA, sBm, sTop);
  // P_R: X2 <- P_L P_R N^-1
  if (act) group_pack(X2, PR, pr, L, gtid, G);
  __syncthreads();
  group_fwd_c<L, G, 1>(X2, nullptr, nullptr, tw, gtid, act ? 1u : 0u);
  for (uint32_t i = gtid; act && i < N; i += G) X2[spad(i)] = gl::mul(gl::mul(X2[spad(i)], X1[spad(i)]), ninv);
  __syncthreads();
  group_inv_c<L, G>(X2, tw, gtid, act);
  const uint32_t p_len = group_carry_store(X2, L, n_p, zp, X3, act, gtid, G, gw0, sA, sBm, sTop);
  if (act && gtid == 0) {
    M.out_len[3 * item] = p_len;
    M.out_len[3 * item + 1] = q_len;
    M.out_len[3 * item + 2] = t_len;
  }
}

// Persistent over the level's items (pairs, then the odd last node): each
// CTA runs MERGE_THREADS / G groups side by side.  8 <= L <= 12.
template <int L>
__global__ void __launch_bounds__(MERGE_THREADS, 2) k_split_merge(MergeLevel M, Roots R) {
  extern __shared__ uint64_t sm[];
  __shared__ uint32_t sA[MERGE_THREADS / 32], sBm[MERGE_THREADS / 32], sTop[MERGE_THREADS / 32];
  constexpr int G = (1 << L) / 8;
  constexpr uint32_t gpc = MERGE_THREADS / G, words = spad(1u << L);
  const uint32_t grp = threadIdx.x / G;
  const int gtid = (int)(threadIdx.x % G);
  const uint32_t np = M.n_in / 2, items = np + (M.n_in & 1);
  const uint32_t nchunks = (items + gpc - 1) / gpc;
  uint64_t* X1 = sm + (size_t)grp * 3 * words;
  for (uint32_t k = blockIdx.x; k < nchunks; k += gridDim.x) {
    const uint32_t item = k * gpc + grp;
    merge_item<L>(M, R.w12, item, item < np, item == np && (M.n_in & 1), X1, X1 + words, X1 + 2 * words, gtid,
                  (int)(grp * G / 32), sA, sBm, sTop);
    __syncthreads();
  }
}

// ------------------------------------------------------------------ host side
static int log2_ceil(uint64_t x) { return x <= 1 ? 0 : 64 - __builtin_clzll(x - 1); }

// Host copies of the root tables: lo, hi, w12, level tables (in this order).
constexpr size_t ROOT_WORDS = 2 * 65536 + 4096 + (2u << LVL_MAX) + (size_t)NEAR_LEVELS * 2 * 4096;

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
  // near tables: w_(2^L)^(+-x) = rho^(+-x 2^(32-L)) for x < 4096
  uint64_t* nt = lvl + (2u << LVL_MAX);
  for (int L = LVL_MAX + 1; L <= 32; L++)
    for (int dir = 0; dir < 2; dir++)
      for (uint32_t xx = 0; xx < 4096; xx++) {
        const uint32_t e0 = (uint32_t)((uint64_t)xx << (32 - L));
        const uint32_t e = dir ? 0u - e0 : e0;
        nt[((size_t)(L - LVL_MAX - 1) * 2 + dir) * 4096 + xx] = hf::mul(lo[e & 0xFFFFu], hi[e >> 16]);
      }
}

static Roots roots_at(const uint64_t* d) {
  return Roots{d, d + 65536, d + 2 * 65536, d + 2 * 65536 + 4096, d + 2 * 65536 + 4096 + (2u << LVL_MAX)};
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
    e = cudaFuncSetAttribute(k_small_mul, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)small_cta_smem(SMALL_LOG_MAX));
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_split_merge<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)merge_cta_smem(8));
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_split_merge<9>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)merge_cta_smem(9));
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_split_merge<10>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)merge_cta_smem(10));
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_split_merge<11>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)merge_cta_smem(11));
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_split_merge<12>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)merge_cta_smem(12));
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

// ------------------------------------------------------------- host copies
// cudaMemcpy from or to PAGEABLE host memory (the limb arrays of a host
// driver) runs through the driver's bounce buffer at a few GB/s.  From 1 MiB
// up such copies are staged instead: host threads copy 32 MiB chunks into
// one of two pinned buffers while the copy engine drains (or fills) the
// other.  Pinned or registered host memory is copied directly.
constexpr size_t STAGE_MIN = (size_t)1 << 20;
constexpr size_t STAGE_CHUNK = (size_t)32 << 20;

// memcpy on all host cores: a fixed set of workers, one copy at a time.
class CopyPool {
 public:
  void copy(void* dst, const void* src, size_t bytes) {
    std::call_once(once_, [this] { start(); });
    if (bytes < ((size_t)4 << 20) || workers_ == 0) {
      memcpy(dst, src, bytes);
      return;
    }
    std::lock_guard<std::mutex> run(run_mu_);
    {
      std::lock_guard<std::mutex> lk(mu_);
      dst_ = static_cast<char*>(dst);
      src_ = static_cast<const char*>(src);
      bytes_ = bytes;
      pending_ = workers_;
      gen_++;
    }
    cv_.notify_all();
    part(0);
    std::unique_lock<std::mutex> lk(mu_);
    done_.wait(lk, [this] { return pending_ == 0; });
  }

 private:
  void start() {
    unsigned hw = std::thread::hardware_concurrency();
    workers_ = (int)std::min(hw ? hw : 1u, 16u) - 1;
    for (int i = 0; i < workers_; i++) std::thread([this, i] { run(i + 1); }).detach();
  }
  void part(int id) {
    const size_t n = (size_t)workers_ + 1;
    const size_t per = ((bytes_ + n - 1) / n + 63) & ~(size_t)63;
    const size_t lo = std::min(bytes_, per * id), hi = std::min(bytes_, lo + per);
    if (hi > lo) memcpy(dst_ + lo, src_ + lo, hi - lo);
  }
  void run(int id) {
    uint64_t seen = 0;
    for (;;) {
      {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [&] { return gen_ != seen; });
        seen = gen_;
      }
      part(id);
      std::lock_guard<std::mutex> lk(mu_);
      if (--pending_ == 0) done_.notify_one();
    }
  }
  std::once_flag once_;
  std::mutex run_mu_, mu_;
  std::condition_variable cv_, done_;
  int workers_ = 0, pending_ = 0;
  uint64_t gen_ = 0;
  char* dst_ = nullptr;
  const char* src_ = nullptr;
  size_t bytes_ = 0;
};
static CopyPool& copy_pool() {
  static CopyPool* p = new CopyPool;  // workers are detached: never destroyed
  return *p;
}

struct StageBuf {
  void* h[2] = {nullptr, nullptr};
  cudaEvent_t ev[2] = {nullptr, nullptr};  // last copy-engine use of h[j]
  int device = -1;
};
static std::mutex g_stage_mu;
static std::vector<StageBuf*> g_stage_free, g_stage_all;

static StageBuf* stage_acquire() {
  int dev = 0;
  cudaGetDevice(&dev);
  {
    // a free buffer whose last copies are done, else (up to four buffers
    // per device) a new one, else any free one: the caller would wait for
    // a busy buffer's copies, i.e. for the work queued before them
    std::lock_guard<std::mutex> lk(g_stage_mu);
    int any = -1, mine = 0;
    for (StageBuf* x : g_stage_all) mine += x->device == dev;
    for (size_t i = 0; i < g_stage_free.size(); i++) {
      StageBuf* x = g_stage_free[i];
      if (x->device != dev) continue;
      if (any < 0) any = (int)i;
      if (cudaEventQuery(x->ev[0]) == cudaSuccess && cudaEventQuery(x->ev[1]) == cudaSuccess) {
        g_stage_free.erase(g_stage_free.begin() + i);
        return x;
      }
    }
    cudaGetLastError();  // cudaEventQuery's cudaErrorNotReady
    if (any >= 0 && mine >= 4) {
      StageBuf* x = g_stage_free[any];
      g_stage_free.erase(g_stage_free.begin() + any);
      return x;
    }
  }
  StageBuf* b = new StageBuf;
  b->device = dev;
  for (int j = 0; j < 2; j++) {
    if (cudaHostAlloc(&b->h[j], STAGE_CHUNK, cudaHostAllocPortable) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->ev[j], cudaEventDisableTiming) != cudaSuccess) {
      cudaGetLastError();
      for (int k = 0; k < 2; k++) {
        if (b->h[k]) cudaFreeHost(b->h[k]);
        if (b->ev[k]) cudaEventDestroy(b->ev[k]);
      }
      delete b;
      return nullptr;
    }
  }
  std::lock_guard<std::mutex> lk(g_stage_mu);
  g_stage_all.push_back(b);
  return b;
}
static void stage_release(StageBuf* b) {
  std::lock_guard<std::mutex> lk(g_stage_mu);
  g_stage_free.push_back(b);
}

// Uploads below STAGE_MIN from pageable memory go through a ring of small
// pinned slots: a plain cudaMemcpyAsync from pageable memory synchronises
// its stream first, so every batch call (its descriptor image) would wait
// for the work already queued instead of preparing the next launch.
constexpr int RING_SLOTS = 16;
struct SmallRing {
  std::mutex mu;
  void* h[RING_SLOTS] = {};
  cudaEvent_t ev[RING_SLOTS] = {};  // the last copy from each slot
  int next = 0;
  int device = -1;
  bool ok = false;
};
static SmallRing& small_ring() {
  static SmallRing* r = new SmallRing;  // pinned slots live until exit
  return *r;
}

static bool is_pageable(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return true;
  }
  return a.type == cudaMemoryTypeUnregistered;
}

// A small pageable upload through the ring; false when the ring cannot be
// set up (the caller then copies directly).
static bool ring_upload(void* dst, const void* src, size_t bytes, cudaStream_t st, cudaError_t* err) {
  SmallRing& r = small_ring();
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(r.mu);
  if (r.device != dev) {
    if (r.device >= 0) return false;  // set up on another device
    for (int k = 0; k < RING_SLOTS; k++)
      if (cudaHostAlloc(&r.h[k], STAGE_MIN, cudaHostAllocPortable) != cudaSuccess ||
          cudaEventCreateWithFlags(&r.ev[k], cudaEventDisableTiming) != cudaSuccess) {
        cudaGetLastError();
        r.device = dev;
        r.ok = false;
        return false;
      }
    r.device = dev;
    r.ok = true;
  }
  if (!r.ok) return false;
  const int k = r.next;
  r.next = (k + 1) % RING_SLOTS;
  cudaError_t e = cudaEventSynchronize(r.ev[k]);  // the copy RING_SLOTS uploads ago is done
  if (e == cudaSuccess) {
    memcpy(r.h[k], src, bytes);
    e = cudaMemcpyAsync(dst, r.h[k], bytes, cudaMemcpyHostToDevice, st);
  }
  if (e == cudaSuccess) e = cudaEventRecord(r.ev[k], st);
  *err = e;
  return true;
}

int host_to_device(void* dst, const void* src, size_t bytes, cudaStream_t st) {
  if (!bytes) return PIMUL_OK;
  const bool pageable = is_pageable(src);
  if (pageable && bytes < STAGE_MIN) {
    cudaError_t e = cudaSuccess;
    if (ring_upload(dst, src, bytes, st, &e)) {
      if (e != cudaSuccess) return fail(PIMUL_ECUDA, std::string("small upload: ") + cudaGetErrorString(e));
      return PIMUL_OK;
    }
  }
  StageBuf* b = bytes >= STAGE_MIN && pageable ? stage_acquire() : nullptr;
  if (!b) {
    CU(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st));
    return PIMUL_OK;
  }
  cudaError_t e = cudaSuccess;
  int j = 0;
  for (size_t off = 0; off < bytes && e == cudaSuccess; off += STAGE_CHUNK, j ^= 1) {
    const size_t n = std::min(STAGE_CHUNK, bytes - off);
    e = cudaEventSynchronize(b->ev[j]);  // the copy engine is done with h[j]
    if (e != cudaSuccess) break;
    copy_pool().copy(b->h[j], static_cast<const char*>(src) + off, n);
    e = cudaMemcpyAsync(static_cast<char*>(dst) + off, b->h[j], n, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaEventRecord(b->ev[j], st);
  }
  stage_release(b);
  if (e != cudaSuccess) return fail(PIMUL_ECUDA, std::string("staged upload: ") + cudaGetErrorString(e));
  return PIMUL_OK;
}

int device_to_host(void* dst, const void* src, size_t bytes, cudaStream_t st) {
  if (!bytes) return PIMUL_OK;
  StageBuf* b = bytes >= STAGE_MIN && is_pageable(dst) ? stage_acquire() : nullptr;
  if (!b) {
    CU(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    return PIMUL_OK;
  }
  const size_t nch = (bytes + STAGE_CHUNK - 1) / STAGE_CHUNK;
  auto issue = [&](size_t i) {
    const size_t off = i * STAGE_CHUNK, n = std::min(STAGE_CHUNK, bytes - off);
    const int j = (int)(i & 1);
    cudaError_t e = cudaEventSynchronize(b->ev[j]);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(b->h[j], static_cast<const char*>(src) + off, n, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaEventRecord(b->ev[j], st);
    return e;
  };
  cudaError_t e = issue(0);
  for (size_t i = 0; i < nch && e == cudaSuccess; i++) {
    // chunk i + 1 lands in the other buffer while chunk i is copied out
    if (i + 1 < nch) e = issue(i + 1);
    if (e == cudaSuccess) e = cudaEventSynchronize(b->ev[i & 1]);
    if (e != cudaSuccess) break;
    const size_t off = i * STAGE_CHUNK, n = std::min(STAGE_CHUNK, bytes - off);
    copy_pool().copy(static_cast<char*>(dst) + off, b->h[i & 1], n);
  }
  stage_release(b);
  if (e != cudaSuccess) return fail(PIMUL_ECUDA, std::string("staged download: ") + cudaGetErrorString(e));
  return PIMUL_OK;
}

int set_error(int code, const char* msg) { return fail(code, msg); }

void release_host_staging() {
  std::lock_guard<std::mutex> lk(g_stage_mu);
  for (StageBuf* b : g_stage_all) {
    for (int j = 0; j < 2; j++) {
      cudaEventSynchronize(b->ev[j]);
      cudaEventDestroy(b->ev[j]);
      cudaFreeHost(b->h[j]);
    }
    delete b;
  }
  g_stage_all.clear();
  g_stage_free.clear();
  SmallRing& r = small_ring();
  std::lock_guard<std::mutex> rl(r.mu);
  for (int k = 0; k < RING_SLOTS; k++) {
    if (r.ev[k]) {
      cudaEventSynchronize(r.ev[k]);
      cudaEventDestroy(r.ev[k]);
    }
    if (r.h[k]) cudaFreeHost(r.h[k]);
    r.ev[k] = nullptr;
    r.h[k] = nullptr;
  }
  r.device = -1;
  r.ok = false;
  r.next = 0;
}

// L bits split into np HBM passes of radix 2^r[0] .. 2^r[np - 1].
struct Plan {
  int L;
  int np;
  int r[5];
};

// Pass-count override per L chosen by the autotuner (0 = default).
static std::atomic<int> g_tuned_np[33];
// Persistent grid of the one-CTA kernel in a batch: CTAs per SM (autotuned).
static std::atomic<int> g_small_ctas_per_sm{4};

static int default_np(int L) {
  int np = (L + 8) / 9;
  return np < 2 ? 2 : np;
}

// A plan is valid when every pass radix is 2^6 .. 2^9 and the first one at
// least 2^7 (the compiled kernels).
static bool plan_valid(const Plan& p) {
  if (p.np < 2 || p.np > 5 || p.r[0] < 7) return false;
  for (int i = 0; i < p.np; i++)
    if (p.r[i] < 6 || p.r[i] > 9) return false;
  return true;
}

static int plan_rounds(const Plan& p) {
  int n = 0;
  for (int i = 0; i < p.np; i++) n += rp_count(p.r[i]);
  return n;
}

// np passes for 2^L points: among the valid splits, the one with the fewest
// radix-8/4 rounds (a pass of 2^6 or 2^9 is all radix-8 rounds, one of 2^7
// or 2^8 needs radix-4 rounds: 2^21 as 9 + 6 + 6 is 7 rounds, 7 + 7 + 7 is
// 9), the even split when it ties.  Each round costs every element its
// round twiddles and a shared-memory round trip.
static Plan split_plan(int L, int np) {
  Plan even{L, np, {0, 0, 0, 0, 0}};
  for (int i = 0; i < np; i++) even.r[i] = L / np + (i < L % np ? 1 : 0);
  Plan best = even;
  int best_rounds = plan_valid(even) ? plan_rounds(even) : 1 << 30;
  Plan cur{L, np, {0, 0, 0, 0, 0}};
  // radices from 9 down, first pass 7..9, the others 6..9
  std::function<void(int, int)> walk = [&](int i, int left) {
    if (i == np - 1) {
      cur.r[i] = left;
      if (plan_valid(cur) && plan_rounds(cur) < best_rounds) {
        best = cur;
        best_rounds = plan_rounds(cur);
      }
      return;
    }
    for (int r = 9; r >= (i == 0 ? 7 : 6); r--) {
      cur.r[i] = r;
      walk(i + 1, left - r);
    }
  };
  if (np >= 2 && np <= 5) walk(0, L);
  return best;
}

// Splits are tabulated once for 2^0 .. 2^32 points (the entry points reject
// longer transforms) and 2 .. 5 passes; any other request gets an invalid
// plan (np 0, which plan_valid rejects).
static Plan make_plan_np(int L, int np) {
  if (L < 0 || L > 32 || np < 2 || np > 5) return Plan{L, 0, {0, 0, 0, 0, 0}};
  static Plan table[33][6];
  static std::once_flag once;
  std::call_once(once, [] {
    for (int l = 0; l <= 32; l++)
      for (int n = 2; n <= 5; n++) table[l][n] = split_plan(l, n);
  });
  return table[L][np];
}

static Plan make_plan(int L) {
  int np = (L >= 0 && L <= 32) ? g_tuned_np[L].load(std::memory_order_relaxed) : 0;
  if (np) {
    Plan p = make_plan_np(L, np);
    if (plan_valid(p)) return p;
  }
  return make_plan_np(L, default_np(L));
}

struct Sizes {
  uint64_t n_out, N, nwin, nchunk, aux_bytes;
  int L;
};

static Sizes sizes_for(uint64_t la, uint64_t lb) {
  Sizes z;
  z.n_out = 4 * la + 4 * lb - 1;
  z.L = log2_ceil(z.n_out);
  z.N = 1ull << z.L;
  z.nwin = n_windows(la, lb);
  z.nchunk = n_chunks(z.nwin);
  z.aux_bytes = aux_bytes_for(z.nwin);
  return z;
}

// Scratch bytes of one large product (A, B unless square, H, aux), each
// piece rounded to 256 bytes.
static uint64_t round256(uint64_t x) { return (x + 255) & ~255ull; }
__host__ __device__ __forceinline__ uint64_t round_up_u64(uint64_t x, uint64_t m) { return (x + m - 1) / m * m; }
static uint64_t scratch_bytes(uint64_t la, uint64_t lb, bool square) {
  Sizes z = sizes_for(la, lb);
  return round256(z.N * 8) * (square ? 1 : 2) + round256(z.nwin * 8) + round256(z.aux_bytes);
}
static void carve_scratch(Job& J, uint8_t* base, bool square) {
  Sizes z = sizes_for(J.la, J.lb);
  J.A = reinterpret_cast<uint64_t*>(base);
  base += round256(z.N * 8);
  if (!square) {
    J.B = reinterpret_cast<uint64_t*>(base);
    base += round256(z.N * 8);
  } else {
    J.B = nullptr;
  }
  J.H = reinterpret_cast<uint64_t*>(base);
  base += round256(z.nwin * 8);
  J.aux = base;
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
  cudaEvent_t b_ready = nullptr;  // operand b's upload (plain host-buffer call): waited on before its first pass
  bool tables = true;             // read pass twiddles from the cached tables (false: compute them)
};

// ---------------------------------------------------------------- twiddle tables
// Pass twiddles can be read from tables laid out like the data they
// multiply, one coalesced load per element, instead of being computed from
// the root tables (a product of two table entries per element in the first
// passes, a scattered lookup in a 2^(R+S)-entry level table in the middle
// ones).  With f_R the digit-reversed row frequency (row_freq_t<R>):
//   first pass of length N = 2^L, radix 2^R, S = L - R:
//     forward  tw[i 2^S + J] = w_N^(f_R(i) J)
//     inverse  tw[i 2^S + J] = w_N^-(f_R(i) J) N^-1   (the inverse's 1/N for free)
//   middle pass of radix 2^R and stride 2^S, M = 2^(R+S):
//     tw[r 2^S + j] = w_M^(+-f_R(r) j)
// Tables are built once per shape, on first use, and kept until
// pimul_shutdown (the reference keeps its twiddles in a cache too,
// crates/bignum/src/ntt.rs:571-611), up to a byte cap; first passes longer
// than 2^TW_LOG_MAX compute their twiddles.
constexpr int TW_LOG_MAX = 28;

template <int R>
__global__ void k_tw_first(uint64_t* tw, int L, int inv, uint64_t scale, Roots RT) {
  const int S = L - R;
  const uint64_t n = 1ull << L, smask = (1ull << S) - 1;
  for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < n; e += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t i = (uint32_t)(e >> S), J = (uint32_t)(e & smask);
    uint64_t t = root_pow32(RT, L, row_freq_t<R>(i) * J, inv != 0);
    if (inv) t = gl::mul(t, scale);
    tw[e] = gl::canon(t);
  }
}

template <int R>
__global__ void k_tw_mid(uint64_t* tw, int S, int inv, Roots RT) {
  const int M = R + S;
  const uint64_t n = 1ull << M, smask = (1ull << S) - 1;
  for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < n; e += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t r = (uint32_t)(e >> S), j = (uint32_t)(e & smask);
    tw[e] = gl::canon(root_pow32(RT, M, row_freq_t<R>(r) * j, inv != 0));
  }
}

struct TwCache {
  std::mutex mu;
  std::unordered_map<uint64_t, uint64_t*> tables;
  uint64_t bytes = 0;
  uint64_t cap = 8ull << 30;
  cudaStream_t st = nullptr;
};
static TwCache& tw_cache() {
  static TwCache* c = new TwCache;  // never destroyed: usable during static destruction
  return *c;
}

// The table of one pass (kind 0: first pass, R + S = L; kind 1: middle pass),
// built on first use.  Null (compute the twiddles) when the shape is above
// TW_LOG_MAX or the cap, while `caller` is capturing a graph (a table is
// never built inside a capture), or when allocating it fails.
static const uint64_t* tw_table(int kind, int R, int S, bool inv, cudaStream_t caller) {
  if (kind == 0 && R + S > TW_LOG_MAX) return nullptr;
  const uint64_t key = ((uint64_t)kind << 24) | ((uint64_t)R << 16) | ((uint64_t)S << 8) | (inv ? 1u : 0u);
  TwCache& c = tw_cache();
  std::lock_guard<std::mutex> lk(c.mu);
  auto it = c.tables.find(key);
  if (it != c.tables.end()) return it->second;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (caller && (cudaStreamIsCapturing(caller, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone)) return nullptr;
  const uint64_t words = 1ull << (R + S);
  if (c.bytes + 8 * words > c.cap) return nullptr;
  if (!c.st && cudaStreamCreateWithFlags(&c.st, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    c.st = nullptr;
    return nullptr;
  }
  uint64_t* d = nullptr;
  if (cudaMalloc(&d, 8 * words) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  const unsigned blocks = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(words / 256, 152 * 16));
  const Roots& RT = g_dev.roots;
  if (kind == 0) {
    const uint64_t ninv = hf::pow(hf::pow(2, 191), (uint64_t)(R + S));  // 2^-L (2^192 = 1)
    PIMUL_DISPATCH_R(R, (k_tw_first<RR><<<blocks, 256, 0, c.st>>>(d, R + S, inv ? 1 : 0, ninv, RT)));
  } else {
    PIMUL_DISPATCH_R(R, (k_tw_mid<RR><<<blocks, 256, 0, c.st>>>(d, S, inv ? 1 : 0, RT)));
  }
  if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(c.st) != cudaSuccess) {
    cudaFree(d);
    return nullptr;
  }
  c.tables[key] = d;
  c.bytes += 8 * words;
  return d;
}

// Pointers of every pass table of a length-2^L plan (null entries: compute).
struct PassTables {
  const uint64_t* first_fwd = nullptr;
  const uint64_t* first_inv = nullptr;  // carries N^-1: k_mid then skips its scaling
  const uint64_t* mid_fwd[5] = {};
  const uint64_t* mid_inv[5] = {};
};
static PassTables pass_tables(const Plan& pl, cudaStream_t caller) {
  PassTables t;
  const int L = pl.L;
  t.first_fwd = tw_table(0, pl.r[0], L - pl.r[0], false, caller);
  t.first_inv = tw_table(0, pl.r[0], L - pl.r[0], true, caller);
  int consumed = pl.r[0];
  for (int p = 1; p < pl.np - 1; p++) {
    consumed += pl.r[p];
    t.mid_fwd[p] = tw_table(1, pl.r[p], L - consumed, false, caller);
    t.mid_inv[p] = tw_table(1, pl.r[p], L - consumed, true, caller);
  }
  return t;
}

static void tw_release_all() {
  TwCache& c = tw_cache();
  std::lock_guard<std::mutex> lk(c.mu);
  for (auto& kv : c.tables) cudaFree(kv.second);
  c.tables.clear();
  c.bytes = 0;
  if (c.st) cudaStreamDestroy(c.st);
  c.st = nullptr;
}

// All launches of the large-product pipeline for `nj` products sharing the
// transform length 2^L: the products come from the device array `jobs`
// (blockIdx.y) or, for nj == 1 and jobs == nullptr, from `one`.
// max_chunk: largest carry-chunk count among the products.
static void run_large(const Launcher& X, const Job* jobs, const Job& one, uint32_t nj, int L, uint64_t max_chunk,
                      bool any_b_full = false, bool any_addend = false) {
  const Plan pl = make_plan(L);
  const dim3 grid((unsigned)(1ull << (L - TILE_LOG)), nj);
  const size_t smem = pass_smem_bytes(TILE_LOG);
  const PassTables tw = X.tables ? pass_tables(pl, X.st) : PassTables{};
  // 2^-L (2^192 = 1); 0 when the inverse first pass's table applies it
  const uint64_t ninv = tw.first_inv ? 0 : hf::pow(hf::pow(2, 191), L);
  const int rl = pl.r[pl.np - 1];
  for (int which = 0; which < 2; which++) {
    if (which == 1 && X.b_ready) cudaStreamWaitEvent(X.st, X.b_ready, 0);
    {
      KTimer kt(K_PACK, X.st, X.stats);
      PIMUL_DISPATCH_R(pl.r[0], (k_fwd_first<(RR < 7 ? 7 : RR)><<<grid, PASS_THREADS, smem, X.st>>>(jobs, one, which, L, X.R,
                                                                                                   tw.first_fwd)));
    }
    int consumed = pl.r[0];
    for (int p = 1; p < pl.np - 1; p++) {
      consumed += pl.r[p];
      KTimer kt(K_PASS_FWD, X.st, X.stats);
      PIMUL_DISPATCH_R(pl.r[p], (k_col_mid<RR, true><<<grid, PASS_THREADS, smem, X.st>>>(jobs, one, which, L - consumed, X.R,
                                                                                        tw.mid_fwd[p])));
    }
    if (which == 0 || any_b_full) {
      KTimer kt(K_PASS_FWD, X.st, X.stats);
      PIMUL_DISPATCH_R(rl, (k_fwd_last<RR><<<grid, PASS_THREADS, smem, X.st>>>(jobs, one, which, X.R)));
    }
  }
  if (any_addend) {
    KTimer kt(K_POINTWISE, X.st, X.stats);
    const uint64_t n = 1ull << L;
    k_pointwise_addend<<<dim3((unsigned)std::min<uint64_t>(n / 1024, 4096), nj), 256, 0, X.st>>>(jobs, one, n);
  }
  {
    KTimer kt(K_POINTWISE, X.st, X.stats);
    if (any_b_full || any_addend) {
      PIMUL_DISPATCH_R(rl, (k_mid<RR, true><<<grid, PASS_THREADS, smem, X.st>>>(jobs, one, ninv, X.R)));
    } else {
      PIMUL_DISPATCH_R(rl, (k_mid<RR, false><<<grid, PASS_THREADS, smem, X.st>>>(jobs, one, ninv, X.R)));
    }
  }
  int consumed = L - rl;
  for (int p = pl.np - 2; p >= 1; p--) {
    int S = L - consumed;
    consumed -= pl.r[p];
    KTimer kt(K_PASS_INV, X.st, X.stats);
    PIMUL_DISPATCH_R(pl.r[p], (k_col_mid<RR, false><<<grid, PASS_THREADS, smem, X.st>>>(jobs, one, 2, S, X.R, tw.mid_inv[p])));
  }
  {
    KTimer kt(K_PASS_INV, X.st, X.stats);
    PIMUL_DISPATCH_R(pl.r[0], (k_inv_first_carry<(RR < 7 ? 7 : RR)><<<grid, PASS_THREADS, smem, X.st>>>(jobs, one, L, X.R,
                                                                                                         tw.first_inv)));
  }
  {
    KTimer kt(K_CARRY, X.st, X.stats);
    const dim3 cgrid((unsigned)max_chunk, nj);
    k_carry_local<<<cgrid, CARRY_THREADS, 0, X.st>>>(jobs, one);
    k_carry_scan<<<dim3(1, nj), SCAN_THREADS, 0, X.st>>>(jobs, one);
    k_carry_apply<<<cgrid, CARRY_THREADS, 0, X.st>>>(jobs, one);
  }
  if (X.stats) g_launch[K_CARRY].fetch_add(2, std::memory_order_relaxed);
}

// Device multiply: d_out[0 .. la+lb) = a * b, scratch from the memory pool.
static int mul_device(const uint64_t* d_a, uint64_t la, const uint64_t* d_b, uint64_t lb, uint64_t* d_out,
                      cudaStream_t st, cudaEvent_t b_ready = nullptr) {
  if (la == 0 || lb == 0) return PIMUL_OK;
  const Sizes z = sizes_for(la, lb);
  if (z.L > 32) return fail(PIMUL_EINVAL, "transform length above 2^32");
  const Roots& R = g_dev.roots;
  const bool square = d_a == d_b && la == lb;
  if (z.L <= SMALL_LOG_MAX) {
    if (b_ready) cudaStreamWaitEvent(st, b_ready, 0);
    SmallJob job{d_a, d_b, d_out, (uint32_t)la, (uint32_t)lb};
    {
      KTimer kt(K_SMALL, st, true);
      k_small_mul<<<1, SMALL_THREADS, small_cta_smem(z.L), st>>>(nullptr, nullptr, job, 1, R);
    }
    CU(cudaGetLastError());
    return PIMUL_OK;
  }
  uint8_t* base = nullptr;
  cudaError_t e = cudaMallocAsync((void**)&base, scratch_bytes(la, lb, square), g_dev.pool, st);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(PIMUL_ENOMEM, std::string("scratch allocation: ") + cudaGetErrorString(e));
  }
  Job J{d_a, d_b, d_out, nullptr, nullptr, nullptr, nullptr, la, lb};
  carve_scratch(J, base, square);
  Launcher X{st, true, R, b_ready};
  run_large(X, nullptr, J, 1, z.L, z.nchunk);
  cudaError_t le = cudaGetLastError();
  cudaFreeAsync(base, st);
  if (le != cudaSuccess) return fail(PIMUL_ECUDA, std::string("kernel launch: ") + cudaGetErrorString(le));
  return PIMUL_OK;
}

// ------------------------------------------------------------------ batches
// A batch of independent products (and sums of two products) on device
// buffers.  Products are grouped by transform length: lengths up to 2^12
// run as one CTA per product in a persistent kernel over a size-sorted list;
// longer ones run the pass pipeline once per length with one grid row
// (blockIdx.y) per descriptor.  Within a group of one length, products whose
// operand b is the same array share b's spectrum (computed once), and a sum
// a1 b1 + a2 b2 runs as two descriptors whose spectra are added before one
// inverse transform and one carry pass.

// One unit of a batch: a b, or a b + a2 b2 (la2 > 0; large lengths only).
struct Unit {
  const uint64_t* a;
  uint64_t la;
  const uint64_t* b;
  uint64_t lb;
  const uint64_t* a2;
  uint64_t la2;
  const uint64_t* b2;
  uint64_t lb2;
  uint64_t* out;
  uint64_t nout;
  int forceL = 0;                 // transform length (log2) when not the one nout implies
  bool coeff = false;             // JF_COEFF: nout canonical coefficients to out, no carry
  const uint64_t* low = nullptr;  // a wrapped product's low coefficients (Job::low)
  uint64_t wrap = 0;              // and their count (Job::wrap)
};

struct BatchLayout {
  std::vector<uint32_t> small;  // unit indices, size-sorted descending
  struct Desc {
    uint32_t unit;
    bool second;             // the a2 b2 half of a sum (an addend)
    uint32_t flags;          // JF_*
    int64_t owner = -1;      // descriptor whose B this one borrows
    int64_t addend = -1;     // descriptor whose A holds this one's X
    uint64_t off_a = 0, off_b = 0, off_h = 0, off_aux = 0;
  };
  std::vector<Desc> desc;  // large descriptors in launch order
  struct Bucket {
    int L;
    size_t d0, nd;
    uint64_t max_chunk;
    bool any_b_full, any_addend;
  };
  std::vector<Bucket> large;
  uint64_t arena_bytes = 0;
  int small_L = 0;  // largest L among the small jobs
  std::vector<SmallChunk> chunks;  // the small jobs in same-length chunks
  size_t small_smem = 0;           // dynamic shared memory of their CTAs
};

// Scratch bound of one group of same-length descriptors in a batch.  Only
// the descriptors of one group share spectra, so a group should hold every
// product of a splitting level's pairs: at the top of a 10^9-digit tree one
// pair's products take 32 GiB at 2^29 points.  PIMUL_BATCH_ARENA_GIB sets it.
static const uint64_t BATCH_ARENA_CAP = [] {
  const char* e = getenv("PIMUL_BATCH_ARENA_GIB");
  const long long g = e ? atoll(e) : 96;
  return (uint64_t)(g > 0 ? g : 96) << 30;
}();

static int unit_log_n(const Unit& u) {
  if (u.la == 0 || u.lb == 0) return -1;
  if (u.forceL) return u.forceL;
  return log2_ceil(4 * u.nout - 1);
}

// share: let products with the same operand b borrow one spectrum (a batch
// plan lays out a shape without pointers and never shares).
static int layout_batch(const Unit* units, size_t n, BatchLayout& B, bool share) {
  std::vector<int> Ls(n);
  for (size_t i = 0; i < n; i++) {
    Ls[i] = unit_log_n(units[i]);
    if (Ls[i] > 32) return fail(PIMUL_EINVAL, "transform length above 2^32 in batch");
  }
  std::vector<std::vector<uint32_t>> byL(33);
  for (size_t i = 0; i < n; i++) {
    if (Ls[i] < 0) continue;
    if (Ls[i] <= SMALL_LOG_MAX && units[i].la2) return fail(PIMUL_EINVAL, "a sum of products below 2^13 in the pass pipeline");
    if (Ls[i] <= SMALL_LOG_MAX) {
      B.small.push_back((uint32_t)i);
      if (Ls[i] > B.small_L) B.small_L = Ls[i];
    } else {
      byL[Ls[i]].push_back((uint32_t)i);
    }
  }
  // longest transforms first (a bucket pass by length, O(n))
  {
    std::vector<std::vector<uint32_t>> sb(SMALL_LOG_MAX + 1);
    for (uint32_t i : B.small) sb[Ls[i]].push_back(i);
    B.small.clear();
    for (int L = SMALL_LOG_MAX; L >= 0; L--) {
      const uint32_t per = SMALL_THREADS / small_group_threads(L);
      for (size_t k = 0; k < sb[L].size(); k += per)
        B.chunks.push_back(SmallChunk{(uint32_t)(B.small.size() + k), (uint32_t)std::min<size_t>(per, sb[L].size() - k), L});
      if (!sb[L].empty()) B.small_smem = std::max(B.small_smem, small_cta_smem(L));
      B.small.insert(B.small.end(), sb[L].begin(), sb[L].end());
    }
  }
  // Groups of one length: at most 65535 descriptors (grid.y) whose scratch
  // fits BATCH_ARENA_CAP; groups run one after another on the stream, so
  // they all reuse the same arena.
  uint64_t arena = 0;
  for (int L = 32; L > SMALL_LOG_MAX; L--) {
    if (byL[L].empty()) continue;
    const uint64_t N = 1ull << L;
    size_t s = 0;
    while (s < byL[L].size()) {
      BatchLayout::Bucket bk{L, B.desc.size(), 0, 0, false, false};
      // the group's units: descriptor count and a scratch bound (no sharing)
      uint64_t bound = 0;
      size_t e = s;
      for (; e < byL[L].size(); e++) {
        const Unit& u = units[byL[L][e]];
        const size_t nd = u.la2 ? 2 : 1;
        const uint64_t need = round256(N * 8) * 2 * nd + round256(n_windows_out(u.nout) * 8) +
                              round256(aux_bytes_for(n_windows_out(u.nout)));
        if (e > s && (bk.nd + nd > 65535 || bound + need > BATCH_ARENA_CAP)) break;
        bk.nd += nd;
        bound += need;
      }
      // descriptors; the first of several with the same b owns its spectrum
      std::unordered_map<const uint64_t*, std::vector<size_t>> by_b;
      for (size_t k = s; k < e; k++) {
        const uint32_t ui = byL[L][k];
        const Unit& u = units[ui];
        BatchLayout::Desc d1;
        d1.unit = ui;
        d1.second = false;
        d1.flags = 0;
        B.desc.push_back(d1);
        const size_t i1 = B.desc.size() - 1;
        const bool sq1 = u.a == u.b && u.la == u.lb;
        if (share && !sq1) by_b[u.b].push_back(i1);
        if (u.la2) {
          BatchLayout::Desc d2;
          d2.unit = ui;
          d2.second = true;
          d2.flags = JF_ADDEND;
          B.desc.push_back(d2);
          const size_t i2 = B.desc.size() - 1;
          B.desc[i1].addend = (int64_t)i2;
          if (share) by_b[u.b2].push_back(i2);
          bk.any_addend = true;
        }
      }
      for (auto& kv : by_b) {
        std::vector<size_t>& v = kv.second;
        // same array and same length
        std::unordered_map<uint64_t, size_t> owner_of;
        for (size_t di : v) {
          const BatchLayout::Desc& d = B.desc[di];
          const uint64_t lb = d.second ? units[d.unit].lb2 : units[d.unit].lb;
          auto it = owner_of.find(lb);
          if (it == owner_of.end()) {
            owner_of.emplace(lb, di);
          } else {
            B.desc[di].flags |= JF_B_SHARED;
            B.desc[di].owner = (int64_t)it->second;
            B.desc[it->second].flags |= JF_B_FULL;
          }
        }
      }
      // an addend needs b's full spectrum; scratch offsets
      uint64_t off = 0;
      for (size_t di = bk.d0; di < bk.d0 + bk.nd; di++) {
        BatchLayout::Desc& d = B.desc[di];
        const Unit& u = units[d.unit];
        if ((d.flags & JF_ADDEND) && !(d.flags & JF_B_SHARED)) d.flags |= JF_B_FULL;
        if (d.flags & JF_B_FULL) bk.any_b_full = true;
        const bool sq = !d.second && u.a == u.b && u.la == u.lb;
        d.off_a = off;
        off += round256(N * 8);
        if (!sq && !(d.flags & JF_B_SHARED)) {
          d.off_b = off;
          off += round256(N * 8);
        }
        if (!d.second) {
          const uint64_t nwin = n_windows_out(u.nout);
          d.off_h = off;
          off += round256(nwin * 8);
          d.off_aux = off;
          off += round256(aux_bytes_for(nwin));
          bk.max_chunk = std::max<uint64_t>(bk.max_chunk, n_chunks(nwin));
        }
      }
      arena = std::max(arena, off);
      B.large.push_back(bk);
      s = e;
    }
  }
  B.arena_bytes = arena;
  return PIMUL_OK;
}

// Host images of the device descriptors, in launch order: small jobs first,
// then each large bucket.
// Bytes of the small jobs' descriptors and chunks at the head of the image.
static size_t small_desc_bytes(const BatchLayout& B) {
  return round256(B.small.size() * sizeof(SmallJob)) + round256(B.chunks.size() * sizeof(SmallChunk));
}

static void fill_descriptors(const Unit* units, const BatchLayout& B, uint8_t* arena, SmallJob* sd, Job* ld) {
  size_t k = 0;
  for (uint32_t i : B.small)
    sd[k++] = SmallJob{units[i].a, units[i].b, units[i].out, (uint32_t)units[i].la, (uint32_t)units[i].lb};
  SmallChunk* sc = reinterpret_cast<SmallChunk*>(reinterpret_cast<uint8_t*>(sd) + round256(B.small.size() * sizeof(SmallJob)));
  for (size_t c = 0; c < B.chunks.size(); c++) sc[c] = B.chunks[c];
  for (size_t di = 0; di < B.desc.size(); di++) {
    const BatchLayout::Desc& d = B.desc[di];
    const Unit& u = units[d.unit];
    Job J{};
    if (d.second) {
      J.a = u.a2, J.la = u.la2, J.b = u.b2, J.lb = u.lb2;
      J.out = nullptr;
      J.nout = u.la2 + u.lb2;
    } else {
      J.a = u.a, J.la = u.la, J.b = u.b, J.lb = u.lb;
      J.out = u.out;
      J.nout = u.nout;
      J.low = u.low;
      J.wrap = u.wrap;
    }
    J.flags = d.flags | (!d.second && u.coeff ? JF_COEFF : 0);
    const bool sq = !d.second && u.a == u.b && u.la == u.lb;
    J.A = reinterpret_cast<uint64_t*>(arena + d.off_a);
    if (d.flags & JF_B_SHARED)
      J.B = reinterpret_cast<uint64_t*>(arena + B.desc[d.owner].off_b);
    else
      J.B = sq ? nullptr : reinterpret_cast<uint64_t*>(arena + d.off_b);
    J.H = d.second ? nullptr : reinterpret_cast<uint64_t*>(arena + d.off_h);
    J.aux = d.second ? nullptr : arena + d.off_aux;
    J.X = d.addend >= 0 ? reinterpret_cast<const uint64_t*>(arena + B.desc[d.addend].off_a) : nullptr;
    ld[di] = J;
  }
}

static void launch_batch(const Launcher& X, const BatchLayout& B, const SmallJob* d_small, const Job* d_large) {
  if (!B.small.empty()) {
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, g_dev.device);
    uint64_t grid = (uint64_t)sms * (uint64_t)g_small_ctas_per_sm.load();
    if (grid > B.chunks.size()) grid = B.chunks.size();
    const SmallChunk* d_chunks = reinterpret_cast<const SmallChunk*>(reinterpret_cast<const uint8_t*>(d_small) +
                                                                     round256(B.small.size() * sizeof(SmallJob)));
    KTimer kt(K_SMALL, X.st, X.stats);
    k_small_mul<<<(unsigned)grid, SMALL_THREADS, B.small_smem, X.st>>>(d_small, d_chunks, SmallJob{},
                                                                      (uint32_t)B.chunks.size(), X.R);
  }
  for (const auto& bk : B.large)
    run_large(X, d_large + bk.d0, Job{}, (uint32_t)bk.nd, bk.L, bk.max_chunk, bk.any_b_full, bk.any_addend);
}

// The calling thread's buffer for a batch's host descriptor image, kept and
// grown: a fresh image per call (tens of MB at the lowest levels of a
// conversion) cost its page faults every time.  host_to_device has staged
// the image before it returns, so the next call may overwrite it.
static uint8_t* host_image(size_t bytes) {
  thread_local std::unique_ptr<uint8_t[]> buf;
  thread_local size_t cap = 0;
  if (bytes > cap) {
    cap = std::max(bytes, cap + cap / 2);
    buf.reset(new uint8_t[cap]);
  }
  return buf.get();
}

static int run_units(const Unit* units, size_t n, cudaStream_t st, bool share) {
  BatchLayout B;
  int rc = layout_batch(units, n, B, share);
  if (rc) return rc;
  const size_t ns = B.small.size(), nl = B.desc.size();
  if (ns + nl == 0) return PIMUL_OK;
  const size_t desc_bytes = small_desc_bytes(B) + nl * sizeof(Job);
  uint8_t* dev = nullptr;
  cudaError_t e = cudaMallocAsync((void**)&dev, round256(B.arena_bytes) + desc_bytes, g_dev.pool, st);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(PIMUL_ENOMEM, std::string("batch scratch allocation: ") + cudaGetErrorString(e));
  }
  uint8_t* arena = dev;
  uint8_t* desc = dev + round256(B.arena_bytes);
  uint8_t* host = host_image(desc_bytes);  // every used byte is written below
  SmallJob* hs = reinterpret_cast<SmallJob*>(host);
  Job* hl = reinterpret_cast<Job*>(host + small_desc_bytes(B));
  fill_descriptors(units, B, arena, hs, hl);
  // descriptors of a large batch go up through the staged copy
  if (host_to_device(desc, host, desc_bytes, st)) e = cudaErrorUnknown;
  if (e == cudaSuccess) {
    Launcher X{st, true, g_dev.roots};
    launch_batch(X, B, reinterpret_cast<SmallJob*>(desc), reinterpret_cast<Job*>(desc + small_desc_bytes(B)));
    e = cudaGetLastError();
  }
  // the host image must outlive the copy (pageable source: staged before return)
  cudaFreeAsync(dev, st);
  if (e != cudaSuccess) return fail(PIMUL_ECUDA, std::string("batch launch: ") + cudaGetErrorString(e));
  return PIMUL_OK;
}

static Unit unit_of(const pimul_job& j) {
  return Unit{j.a, j.la, j.b, j.lb, nullptr, 0, nullptr, 0, j.out, j.la + j.lb};
}

static int mul_batch(const pimul_job* jobs, size_t n, cudaStream_t st) {
  std::vector<Unit> u(n);
  for (size_t i = 0; i < n; i++) u[i] = unit_of(jobs[i]);
  return run_units(u.data(), n, st, true);
}

// A batch plan: the layout, arena and descriptors of a fixed batch shape,
// with every launch captured once into a CUDA graph.  Running it writes the
// new operand pointers into a pinned staging image, and one graph launch
// copies the descriptors in and runs all kernels.
struct BatchPlan {
  std::vector<uint64_t> la, lb;
  BatchLayout B;
  uint8_t* dev = nullptr;      // arena + descriptors
  uint8_t* staging = nullptr;  // pinned host image of the descriptors
  size_t desc_bytes = 0, ns = 0, nl = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t done = nullptr;
  bool launched = false;
};

static int plan_create(const size_t* la, const size_t* lb, size_t n, BatchPlan** out) {
  int rc = ensure_init(-1);
  if (rc) return rc;
  CU(cudaSetDevice(g_dev.device));
  auto* P = new BatchPlan();
  P->la.assign(la, la + n);
  P->lb.assign(lb, lb + n);
  // shape-only jobs (distinct dummy pointers: no job is a square)
  std::vector<Unit> shape(n);
  for (size_t i = 0; i < n; i++)
    shape[i] = unit_of(pimul_job{nullptr, la[i], (const uint64_t*)(uintptr_t)(8 + 16 * i), lb[i], nullptr});
  rc = layout_batch(shape.data(), n, P->B, false);
  if (rc) { delete P; return rc; }
  P->ns = P->B.small.size();
  P->nl = P->B.desc.size();
  P->desc_bytes = small_desc_bytes(P->B) + P->nl * sizeof(Job);
  cudaError_t e = cudaMalloc((void**)&P->dev, round256(P->B.arena_bytes) + P->desc_bytes + 256);
  if (e == cudaSuccess) e = cudaMallocHost((void**)&P->staging, P->desc_bytes + 256);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&P->done, cudaEventDisableTiming);
  cudaStream_t cs = nullptr;
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
  if (e == cudaSuccess) {
    // twiddle tables are never built inside a capture: build them first
    for (size_t i = 0; i < n; i++) {
      const int L = log2_ceil(4 * (uint64_t)la[i] + 4 * (uint64_t)lb[i] - 1);
      if (la[i] && lb[i] && L > SMALL_LOG_MAX) pass_tables(make_plan(L), nullptr);
    }
    uint8_t* desc = P->dev + round256(P->B.arena_bytes);
    e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      cudaMemcpyAsync(desc, P->staging, P->desc_bytes, cudaMemcpyHostToDevice, cs);
      Launcher X{cs, false, g_dev.roots};
      launch_batch(X, P->B, reinterpret_cast<SmallJob*>(desc), reinterpret_cast<Job*>(desc + small_desc_bytes(P->B)));
      e = cudaStreamEndCapture(cs, &P->graph);
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&P->exec, P->graph, 0);
  }
  if (cs) cudaStreamDestroy(cs);
  if (e != cudaSuccess) {
    cudaGetLastError();
    if (P->exec) cudaGraphExecDestroy(P->exec);
    if (P->graph) cudaGraphDestroy(P->graph);
    if (P->dev) cudaFree(P->dev);
    if (P->staging) cudaFreeHost(P->staging);
    if (P->done) cudaEventDestroy(P->done);
    delete P;
    return fail(e == cudaErrorMemoryAllocation ? PIMUL_ENOMEM : PIMUL_ECUDA,
                std::string("batch plan: ") + cudaGetErrorString(e));
  }
  *out = P;
  return PIMUL_OK;
}

static int plan_run(BatchPlan* P, const pimul_job* jobs, size_t n, cudaStream_t st) {
  if (n != P->la.size()) return fail(PIMUL_EINVAL, "batch size differs from the plan");
  for (size_t i = 0; i < n; i++)
    if (jobs[i].la != P->la[i] || jobs[i].lb != P->lb[i]) return fail(PIMUL_EINVAL, "job sizes differ from the plan");
  // the previous run's descriptor copy must have read the staging image
  if (P->launched) CU(cudaEventSynchronize(P->done));
  SmallJob* hs = reinterpret_cast<SmallJob*>(P->staging);
  Job* hl = reinterpret_cast<Job*>(P->staging + small_desc_bytes(P->B));
  std::vector<Unit> u(n);
  for (size_t i = 0; i < n; i++) u[i] = unit_of(jobs[i]);
  fill_descriptors(u.data(), P->B, P->dev, hs, hl);
  CU(cudaGraphLaunch(P->exec, st));
  CU(cudaEventRecord(P->done, st));
  P->launched = true;
  return PIMUL_OK;
}

static void plan_destroy(BatchPlan* P) {
  if (!P) return;
  if (P->launched) cudaEventSynchronize(P->done);
  if (P->exec) cudaGraphExecDestroy(P->exec);
  if (P->graph) cudaGraphDestroy(P->graph);
  if (P->dev) cudaFree(P->dev);
  if (P->staging) cudaFreeHost(P->staging);
  if (P->done) cudaEventDestroy(P->done);
  delete P;
}

// ------------------------------------------------------------------ autotuner
// Times the candidate pass splits for each length in [Lmin, Lmax] on a
// batch of `reps` synthetic products (device-resident), keeps the fastest,
// and tunes the one-CTA kernel's persistent grid on a batch of small
// products.  The choice only changes the schedule; products are identical.
static int autotune(int Lmin, int Lmax, int reps, char* report, size_t cap) {
  int rc = ensure_init(-1);
  if (rc) return rc;
  cudaStream_t st;
  rc = get_stream(&st);
  if (rc) return rc;
  std::string rep = "{";
  cudaEvent_t e0, e1;
  CU(cudaEventCreate(&e0));
  CU(cudaEventCreate(&e1));
  auto time_batch = [&](std::vector<pimul_job>& js, float* ms_out) -> int {
    for (int w = 0; w < 2; w++) {
      int r2 = mul_batch(js.data(), js.size(), st);
      if (r2) return r2;
    }
    cudaEventRecord(e0, st);
    for (int w = 0; w < 3; w++) {
      int r2 = mul_batch(js.data(), js.size(), st);
      if (r2) return r2;
    }
    cudaEventRecord(e1, st);
    CU(cudaEventSynchronize(e1));
    CU(cudaEventElapsedTime(ms_out, e0, e1));
    return PIMUL_OK;
  };
  // operands: one buffer of random-ish limbs, reused by every synthetic job
  // large lengths read 2 * max_limbs input words and write reps * 2 * max_limbs;
  // the small-kernel batch reads 1024 words and writes 4096 * 1024
  const uint64_t max_limbs = Lmax >= 3 ? (1ull << (Lmax - 3)) : 1;
  const uint64_t in_words = std::max<uint64_t>(2 * max_limbs, 1024);
  const uint64_t out_words = std::max<uint64_t>((uint64_t)reps * 2 * max_limbs, 4096ull * 1024);
  uint64_t* d_in = nullptr;
  uint64_t* d_out = nullptr;
  CU(cudaMallocAsync((void**)&d_in, in_words * 8, g_dev.pool, st));
  CU(cudaMallocAsync((void**)&d_out, out_words * 8, g_dev.pool, st));
  CU(cudaMemsetAsync(d_in, 0xA5, in_words * 8, st));
  bool first = true;
  for (int L = std::max(Lmin, SMALL_LOG_MAX + 1); L <= Lmax && L <= 32; L++) {
    uint64_t limbs = (1ull << (L - 3)) - 1;  // la = lb: 4(la+lb) - 1 < 2^L
    std::vector<pimul_job> js(reps);
    for (int k = 0; k < reps; k++)
      js[k] = pimul_job{d_in, limbs, d_in + limbs, limbs, d_out + (uint64_t)k * 2 * limbs};
    int best_np = 0;
    float best = 1e30f;
    for (int np = 2; np <= 5; np++) {
      if (!plan_valid(make_plan_np(L, np))) continue;
      g_tuned_np[L].store(np);
      float ms = 0;
      rc = time_batch(js, &ms);
      if (rc) break;
      if (ms < best) { best = ms; best_np = np; }
    }
    if (rc) break;
    g_tuned_np[L].store(best_np);
    char buf[96];
    snprintf(buf, sizeof buf, "%s\"np_%d\": %d", first ? "" : ", ", L, best_np);
    rep += buf;
    first = false;
  }
  if (!rc && Lmin <= SMALL_LOG_MAX) {
    // small kernel: CTAs per SM for a batch of 4096 products of 16..512 limbs
    std::vector<pimul_job> js(4096);
    for (int k = 0; k < 4096; k++) {
      uint64_t l = 16 + (k * 37) % 497;
      js[k] = pimul_job{d_in, l, d_in + l, l, d_out + (uint64_t)k * 1024};
    }
    int best_c = 4;
    float best = 1e30f;
    for (int c : {1, 2, 3, 4, 6, 8}) {
      g_small_ctas_per_sm.store(c);
      float ms = 0;
      rc = time_batch(js, &ms);
      if (rc) break;
      if (ms < best) { best = ms; best_c = c; }
    }
    g_small_ctas_per_sm.store(best_c);
    char buf[96];
    snprintf(buf, sizeof buf, "%s\"small_ctas_per_sm\": %d", first ? "" : ", ", best_c);
    rep += buf;
  }
  rep += "}";
  cudaFreeAsync(d_in, st);
  cudaFreeAsync(d_out, st);
  cudaStreamSynchronize(st);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (report && cap) {
    strncpy(report, rep.c_str(), cap - 1);
    report[cap - 1] = 0;
  }
  return rc;
}

// ------------------------------------------------------------------ service
// Served form: device-resident integers (handles) and an asynchronous
// multiply service.  submit() queues a request and returns its result handle
// at once; the handle can feed later requests before it is computed
// (dependencies are CUDA events, never a host round trip).  A service thread
// admits queued requests while their memory fits the HBM budget, launches
// each admitted group as one batch on one of several streams (continuous
// batching: new requests join as earlier ones complete and release memory,
// and groups on different streams overlap on the device), and records every
// request's latency from submit to completion.
struct SvcHandle {
  uint64_t* d = nullptr;
  uint64_t limbs = 0;        // stored length (a product stores la + lb limbs)
  cudaEvent_t ready = nullptr;  // recorded after the producing batch (or upload)
  bool pending = false;      // produced by a request not yet launched
  int64_t producer = -1;     // ticket of the producing request
  bool freed = false;
  uint64_t bytes = 0;
  int readers = 0;           // queued or running requests that read this handle
  bool borrowed = false;     // the caller's device memory (pimul_adopt): never freed here
  bool release = false;      // pimul_release: free once its producer and readers are done
};

struct SvcRequest {
  uint64_t ticket;
  int op;  // 0 multiply, 1 square, 2 add, 3 subtract (PIMUL_OP_*)
  int L = 0;  // transform length (log2) of a product, from the input lengths at submit
  uint64_t a, b, out;  // handle ids
  double t_submit;
  double t_done = 0;
  uint64_t scratch = 0;
  int state = 0;  // 0 queued, 1 launched, 2 done, 3 cancelled
};

struct SvcBatch {
  cudaEvent_t done;
  std::vector<uint64_t> tickets;
  uint64_t scratch = 0;
  int stream = 0;
};

struct Service {
  std::mutex mu;
  std::condition_variable cv;       // wakes the service thread
  std::condition_variable done_cv;  // wakes waiters
  std::thread th;
  bool running = false, stop = false;
  uint64_t budget = 120ull << 30;
  uint64_t in_use = 0;  // handle bytes + scratch of launched requests
  uint64_t next_handle = 1, next_ticket = 1;
  std::unordered_map<uint64_t, SvcHandle> handles;
  std::unordered_map<uint64_t, SvcRequest> requests;
  std::deque<uint64_t> queue;
  std::vector<SvcBatch> inflight;
  std::vector<cudaStream_t> streams;
  std::vector<int> stream_busy;
  std::vector<double> latencies;  // seconds, completed requests
  uint64_t completed = 0, batches = 0;
  int max_batch = 4096;
  int big_log_n = 24;  // requests with transforms of 2^big_log_n and longer run alone on stream 0
  bool dirty = true;   // something admission depends on changed since the last admission pass
  // Handles' memory (uploads and results) comes from a pool of its own:
  // after a long run of plain products allocating and freeing scratch on
  // another stream, allocations from the shared pool on the service's
  // stream took about 0.1-0.2 ms each, and a thread submitting a tree of
  // 2000 requests spent half a second in them.
  cudaMemPool_t pool = nullptr;
};
// Heap-allocated and never destroyed: its thread is joined by an atexit
// handler (registered after the CUDA runtime's, so it runs first).
static Service& svc_obj() {
  static Service* s = new Service();
  return *s;
}
#define g_svc (svc_obj())

static void svc_atexit() {
  std::unique_lock<std::mutex> lk(g_svc.mu);
  if (!g_svc.running) return;
  g_svc.stop = true;
  g_svc.cv.notify_all();
  lk.unlock();
  if (g_svc.th.joinable()) g_svc.th.join();
  lk.lock();
  g_svc.running = false;
}

static double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

static void svc_loop();

static int svc_start() {
  int rc = ensure_init(-1);
  if (rc) return rc;
  std::lock_guard<std::mutex> lk(g_svc.mu);
  if (g_svc.running) return PIMUL_OK;
  CU(cudaSetDevice(g_dev.device));
  if (g_svc.streams.empty()) {
    // stream 0: highest priority, reserved for large requests (one per
    // group) so they run at near-solo speed; streams 1-4 carry batched
    // groups of smaller requests
    int lo = 0, hi = 0;
    CU(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    for (int i = 0; i < 5; i++) {
      cudaStream_t s;
      CU(cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, i == 0 ? hi : lo));
      g_svc.streams.push_back(s);
      g_svc.stream_busy.push_back(0);
    }
  }
  if (!g_svc.pool) {
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = g_dev.device;
    CU(cudaMemPoolCreate(&g_svc.pool, &props));
    uint64_t thr = UINT64_MAX;  // keep freed handle memory for later requests
    CU(cudaMemPoolSetAttribute(g_svc.pool, cudaMemPoolAttrReleaseThreshold, &thr));
  }
  g_svc.stop = false;
  g_svc.running = true;
  g_svc.th = std::thread(svc_loop);
  static bool registered = (std::atexit(svc_atexit), true);
  (void)registered;
  return PIMUL_OK;
}

// Free a handle whose producer has been launched and whose readers are done
// (the free is ordered after the producer's batch on stream 0).
static void svc_free_now(uint64_t id) {
  auto it = g_svc.handles.find(id);
  if (it == g_svc.handles.end()) return;
  SvcHandle& h = it->second;
  if (h.ready) {
    cudaStreamWaitEvent(g_svc.streams[0], h.ready, 0);
    cudaEventDestroy(h.ready);
  }
  if (!h.borrowed && h.d) cudaFreeAsync(h.d, g_svc.streams[0]);
  g_svc.in_use -= h.bytes;
  g_svc.handles.erase(it);
}

// Released handles that have become free.
static void svc_free_released() {
  std::vector<uint64_t> done;
  for (auto& kv : g_svc.handles)
    if (kv.second.release && !kv.second.pending && kv.second.readers <= 0) done.push_back(kv.first);
  for (uint64_t id : done) svc_free_now(id);
}


int svc_addsub(const pimul_addsub_job* jobs, size_t n, cudaStream_t st);  // unchecked, asynchronous (below)

// Group kind of a request: 0 a product below the big length, 1 a big
// product (alone on stream 0), 2 an addition or subtraction.
static int svc_kind(const SvcRequest& r) {
  if (r.op >= 2) return 2;
  return r.L >= g_svc.big_log_n ? 1 : 0;
}

static bool svc_ready(const SvcRequest& r) {
  return !g_svc.handles[r.a].pending && !g_svc.handles[r.b].pending;
}

// One group: the kind of the first ready request in the queue whose stream
// is free (stream 0 for a big product, a free batch stream otherwise), then
// every ready request of that kind among the first SVC_SCAN queued (in
// order), within the budget.  A request whose input is not launched yet
// waits without holding back the ready ones behind it (continuous batching
// of whatever is ready).  Returns whether a group was launched.
constexpr size_t SVC_SCAN = 1 << 14;

static bool svc_admit(std::unique_lock<std::mutex>& lk) {
  if (g_svc.queue.empty()) return false;
  // the free streams first: with none, nothing can be admitted and the
  // queue is not scanned (the submitting threads share this mutex)
  int batch_si = -1;
  for (size_t i = 1; i < g_svc.streams.size(); i++)
    if (!g_svc.stream_busy[i]) { batch_si = (int)i; break; }
  const bool big_free = !g_svc.stream_busy[0];
  if (batch_si < 0 && !big_free) return false;
  int kind = -1;
  size_t scanned = 0;
  for (auto it = g_svc.queue.begin(); it != g_svc.queue.end() && scanned < SVC_SCAN; ++it, ++scanned) {
    const SvcRequest& r = g_svc.requests[*it];
    if (!svc_ready(r)) continue;
    const int k = svc_kind(r);
    if (k == 1 ? big_free : batch_si >= 0) {
      kind = k;
      break;
    }
  }
  if (kind < 0) return false;
  const int si = kind == 1 ? 0 : batch_si;
  std::vector<uint64_t> take;
  uint64_t add = 0;
  scanned = 0;
  for (auto it = g_svc.queue.begin();
       it != g_svc.queue.end() && scanned < SVC_SCAN && (int)take.size() < g_svc.max_batch; scanned++) {
    SvcRequest& r = g_svc.requests[*it];
    if (!svc_ready(r) || svc_kind(r) != kind) {
      ++it;
      continue;
    }
    if (g_svc.in_use + add + r.scratch > g_svc.budget && !(take.empty() && g_svc.inflight.empty())) break;
    take.push_back(*it);
    add += r.scratch;
    it = g_svc.queue.erase(it);
    if (kind == 1) break;  // a big request forms its own group
  }
  if (take.empty()) return false;
  cudaStream_t st = g_svc.streams[si];
  const bool linear = g_svc.requests[take.front()].op >= 2;
  std::vector<pimul_job> jobs;
  std::vector<pimul_addsub_job> asj;
  jobs.reserve(take.size());
  for (uint64_t t : take) {
    SvcRequest& r = g_svc.requests[t];
    SvcHandle& A = g_svc.handles[r.a];
    SvcHandle& B = g_svc.handles[r.b];
    SvcHandle& O = g_svc.handles[r.out];
    if (A.ready) cudaStreamWaitEvent(st, A.ready, 0);
    if (r.op != 1 && B.ready) cudaStreamWaitEvent(st, B.ready, 0);
    if (O.ready) cudaStreamWaitEvent(st, O.ready, 0);  // result buffer allocated
    if (linear) {
      // out = a + b (max + 1 limbs) or a - b (a's limbs; a >= b): no carry
      // or borrow can leave the output, so nothing is checked
      asj.push_back(pimul_addsub_job{A.d, A.limbs, B.d, B.limbs, O.d, O.limbs, r.op == 3 ? PIMUL_SUB_MOD : 0});
    } else {
      const uint64_t* pa = A.d;
      const uint64_t* pb = r.op == 1 ? A.d : B.d;
      uint64_t lb = r.op == 1 ? A.limbs : B.limbs;
      jobs.push_back(pimul_job{pa, A.limbs, pb, lb, O.d});
    }
    r.state = 1;
  }
  SvcBatch bt;
  bt.stream = si;
  bt.scratch = add;
  bt.tickets = take;
  g_svc.in_use += add;
  lk.unlock();
  int rc = linear ? svc_addsub(asj.data(), asj.size(), st) : mul_batch(jobs.data(), jobs.size(), st);
  cudaEventCreateWithFlags(&bt.done, cudaEventDisableTiming);
  cudaEventRecord(bt.done, st);
  lk.lock();
  for (uint64_t t : take) {
    SvcRequest& r = g_svc.requests[t];
    SvcHandle& O = g_svc.handles[r.out];
    cudaEvent_t e;
    cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    cudaEventRecord(e, st);
    if (O.ready) cudaEventDestroy(O.ready);
    O.ready = e;
    O.pending = false;
    if (rc) r.state = 3;
  }
  g_svc.stream_busy[si] = 1;
  g_svc.inflight.push_back(std::move(bt));
  g_svc.batches++;
  return true;
}

static bool svc_reap(std::unique_lock<std::mutex>& lk) {
  bool any = false;
  for (size_t i = 0; i < g_svc.inflight.size();) {
    SvcBatch& bt = g_svc.inflight[i];
    if (cudaEventQuery(bt.done) == cudaSuccess) {
      double t = now_s();
      for (uint64_t tk : bt.tickets) {
        SvcRequest& r = g_svc.requests[tk];
        if (r.state != 3) r.state = 2;
        r.t_done = t;
        auto ia = g_svc.handles.find(r.a);
        if (ia != g_svc.handles.end()) ia->second.readers--;
        if (r.b != r.a) {
          auto ib = g_svc.handles.find(r.b);
          if (ib != g_svc.handles.end()) ib->second.readers--;
        }
        g_svc.latencies.push_back(t - r.t_submit);
        g_svc.completed++;
      }
      g_svc.in_use -= bt.scratch;
      g_svc.stream_busy[bt.stream] = 0;
      svc_free_released();
      cudaEventDestroy(bt.done);
      g_svc.inflight.erase(g_svc.inflight.begin() + i);
      g_svc.done_cv.notify_all();
      any = true;
    } else {
      i++;
    }
  }
  return any;
}

static void svc_loop() {
  cudaSetDevice(g_dev.device);
  std::unique_lock<std::mutex> lk(g_svc.mu);
  while (!g_svc.stop) {
    if (svc_reap(lk)) g_svc.dirty = true;  // streams and budget freed
    // admission only after a change (a submission, a completion, a release,
    // a new budget or policy), and again after every group it launched
    if (g_svc.dirty) g_svc.dirty = svc_admit(lk);
    if (g_svc.inflight.empty() && g_svc.queue.empty()) {
      g_svc.cv.wait_for(lk, std::chrono::milliseconds(50));
    } else {
      // bounded poll: completions are checked every 20 us while work is in flight
      g_svc.cv.wait_for(lk, std::chrono::microseconds(20));
    }
  }
}

static uint64_t svc_new_handle(uint64_t limbs, uint64_t* d, bool pending, uint64_t bytes) {
  uint64_t id = g_svc.next_handle++;
  SvcHandle h;
  h.d = d;
  h.limbs = limbs;
  h.pending = pending;
  h.bytes = bytes;
  g_svc.handles[id] = h;
  return id;
}

void noalloc_forget();  // defined with the no-alloc entry point below
}  // namespace pimul

// ====================================================================== C ABI
using namespace pimul;

extern "C" {

const char* pimul_version(void) { return "pimul 0.2 (sm_103a)"; }

const char* pimul_last_error(void) { return t_err.c_str(); }

int pimul_init(int device) { return ensure_init(device); }

int pimul_shutdown(void) {
  pimul::noalloc_forget();
  {
    std::unique_lock<std::mutex> sl(g_svc.mu);
    if (g_svc.running) {
      g_svc.stop = true;
      g_svc.cv.notify_all();
      sl.unlock();
      if (g_svc.th.joinable()) g_svc.th.join();
      sl.lock();
      g_svc.running = false;
    }
  }
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_dev.ready) return PIMUL_OK;
  cudaSetDevice(g_dev.device);
  cudaDeviceSynchronize();
  release_host_staging();
  tw_release_all();
  cudaFree(g_dev.d_roots);
  if (g_dev.pool) cudaMemPoolTrimTo(g_dev.pool, 0);
  if (g_svc.pool) cudaMemPoolTrimTo(g_svc.pool, 0);  // handles still held keep their memory
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

int pimul_mul_batch(const pimul_job* jobs, size_t n, void* stream) {
  if (n && !jobs) return fail(PIMUL_EINVAL, "null job list");
  for (size_t i = 0; i < n; i++)
    if (jobs[i].la && jobs[i].lb && (!jobs[i].a || !jobs[i].b || !jobs[i].out))
      return fail(PIMUL_EINVAL, "null device pointer in batch");
  cudaStream_t st;
  int rc = get_stream(&st);
  if (rc) return rc;
  if (stream) st = (cudaStream_t)stream;
  return mul_batch(jobs, n, st);
}

int pimul_batch_plan_create(const size_t* la, const size_t* lb, size_t n, pimul_batch_plan** plan) {
  if (!plan || (n && (!la || !lb))) return fail(PIMUL_EINVAL, "null argument");
  BatchPlan* P = nullptr;
  int rc = plan_create(la, lb, n, &P);
  if (rc) return rc;
  *plan = reinterpret_cast<pimul_batch_plan*>(P);
  return PIMUL_OK;
}

int pimul_batch_plan_run(pimul_batch_plan* plan, const pimul_job* jobs, size_t n, void* stream) {
  if (!plan || (n && !jobs)) return fail(PIMUL_EINVAL, "null argument");
  for (size_t i = 0; i < n; i++)
    if (jobs[i].la && jobs[i].lb && (!jobs[i].a || !jobs[i].b || !jobs[i].out))
      return fail(PIMUL_EINVAL, "null device pointer in batch");
  cudaStream_t st;
  int rc = get_stream(&st);
  if (rc) return rc;
  if (stream) st = (cudaStream_t)stream;
  return plan_run(reinterpret_cast<BatchPlan*>(plan), jobs, n, st);
}

int pimul_batch_plan_destroy(pimul_batch_plan* plan) {
  plan_destroy(reinterpret_cast<BatchPlan*>(plan));
  return PIMUL_OK;
}

int pimul_autotune(int log_n_min, int log_n_max, int reps, char* report, size_t report_cap) {
  if (log_n_min < 1 || log_n_max > 28 || log_n_min > log_n_max || reps < 1)
    return fail(PIMUL_EINVAL, "autotune range must lie in [1, 28] and reps >= 1");
  return autotune(log_n_min, log_n_max, reps, report, report_cap);
}

int pimul_tuning_set(int log_n, int passes, int small_ctas_per_sm) {
  if (log_n >= 0 && log_n <= 32) {
    if (passes && !plan_valid(make_plan_np(log_n, passes))) return fail(PIMUL_EINVAL, "no kernels for that split");
    g_tuned_np[log_n].store(passes);
  }
  if (small_ctas_per_sm > 0) g_small_ctas_per_sm.store(small_ctas_per_sm);
  return PIMUL_OK;
}

int pimul_twiddle_cache(uint64_t max_bytes, uint64_t* held) {
  TwCache& c = tw_cache();
  std::lock_guard<std::mutex> lk(c.mu);
  c.cap = max_bytes;
  if (held) *held = c.bytes;
  return PIMUL_OK;
}

int pimul_set_budget(uint64_t bytes) {
  std::lock_guard<std::mutex> lk(g_svc.mu);
  g_svc.budget = bytes;
  g_svc.dirty = true;
  return PIMUL_OK;
}

int pimul_upload(const uint64_t* host, size_t n, uint64_t* handle) {
  if (!handle || (n && !host)) return fail(PIMUL_EINVAL, "null argument");
  int rc = svc_start();
  if (rc) return rc;
  uint64_t bytes = round256(std::max<uint64_t>(n, 1) * 8);
  {
    std::lock_guard<std::mutex> lk(g_svc.mu);
    if (g_svc.in_use + bytes > g_svc.budget) return fail(PIMUL_ENOMEM, "upload exceeds the HBM budget");
    g_svc.in_use += bytes;
  }
  cudaStream_t st;
  rc = get_stream(&st);
  if (rc) return rc;
  uint64_t* d = nullptr;
  cudaError_t e = cudaMallocAsync((void**)&d, bytes, g_svc.pool, st);
  if (e == cudaSuccess && n && host_to_device(d, host, n * 8, st)) e = cudaErrorUnknown;
  cudaEvent_t ev = nullptr;
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventRecord(ev, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // the host buffer may be reused on return
  std::lock_guard<std::mutex> lk(g_svc.mu);
  if (e != cudaSuccess) {
    g_svc.in_use -= bytes;
    cudaGetLastError();
    return fail(PIMUL_ENOMEM, std::string("upload: ") + cudaGetErrorString(e));
  }
  uint64_t id = svc_new_handle(n, d, false, bytes);
  g_svc.handles[id].ready = ev;
  *handle = id;
  return PIMUL_OK;
}

int pimul_submit(int op, uint64_t a, uint64_t b, uint64_t* out_handle, uint64_t* ticket) {
  if (!out_handle || !ticket || op < PIMUL_OP_MUL || op > PIMUL_OP_SUB) return fail(PIMUL_EINVAL, "bad argument");
  int rc = svc_start();
  if (rc) return rc;
  std::lock_guard<std::mutex> lk(g_svc.mu);
  auto ia = g_svc.handles.find(a);
  auto ib = g_svc.handles.find(op == PIMUL_OP_SQR ? a : b);
  if (ia == g_svc.handles.end() || ib == g_svc.handles.end() || ia->second.freed || ib->second.freed)
    return fail(PIMUL_ENOTFOUND, "unknown or freed handle");
  uint64_t la = ia->second.limbs, lb = ib->second.limbs;
  const bool linear = op == PIMUL_OP_ADD || op == PIMUL_OP_SUB;
  // a sum keeps every carry in max + 1 limbs; a difference (a >= b) fits in max
  uint64_t outl = op == PIMUL_OP_ADD ? std::max(la, lb) + 1 : op == PIMUL_OP_SUB ? std::max(la, lb) : la + lb;
  uint64_t obytes = round256(std::max<uint64_t>(outl, 1) * 8);
  uint64_t scratch =
      (!linear && la && lb && sizes_for(la, lb).L > SMALL_LOG_MAX) ? scratch_bytes(la, lb, false) : 0;
  if (!linear && la && lb && sizes_for(la, lb).L > 32) return fail(PIMUL_EINVAL, "transform length above 2^32");
  if (obytes + scratch > g_svc.budget) return fail(PIMUL_ENOMEM, "request larger than the HBM budget");
  uint64_t* d = nullptr;
  cudaError_t e = cudaMallocFromPoolAsync((void**)&d, obytes, g_svc.pool, g_svc.streams[0]);
  if (e == cudaSuccess) e = cudaMemsetAsync(d, 0, obytes, g_svc.streams[0]);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(PIMUL_ENOMEM, std::string("result allocation: ") + cudaGetErrorString(e));
  }
  // the result buffer must exist before any batch stream writes it
  cudaEvent_t alloc_ev;
  cudaEventCreateWithFlags(&alloc_ev, cudaEventDisableTiming);
  cudaEventRecord(alloc_ev, g_svc.streams[0]);
  g_svc.in_use += obytes;
  uint64_t oid = svc_new_handle(outl, d, true, obytes);
  g_svc.handles[oid].ready = alloc_ev;
  uint64_t t = g_svc.next_ticket++;
  SvcRequest r;
  r.ticket = t;
  r.op = op;
  r.L = (!linear && la && lb) ? log2_ceil(4 * la + 4 * lb - 1) : 0;
  r.a = a;
  r.b = op == PIMUL_OP_SQR ? a : b;
  r.out = oid;
  r.t_submit = now_s();
  r.scratch = scratch;
  g_svc.handles[oid].producer = (int64_t)t;
  ia->second.readers++;
  if (r.b != r.a) g_svc.handles[r.b].readers++;
  g_svc.requests[t] = r;
  g_svc.queue.push_back(t);
  g_svc.dirty = true;
  *out_handle = oid;
  *ticket = t;
  g_svc.cv.notify_one();
  return PIMUL_OK;
}

int pimul_wait(uint64_t ticket, int64_t timeout_us) {
  std::unique_lock<std::mutex> lk(g_svc.mu);
  auto it = g_svc.requests.find(ticket);
  if (it == g_svc.requests.end()) return fail(PIMUL_ENOTFOUND, "unknown ticket");
  SvcRequest* rp = &it->second;  // element pointers survive rehashing
  auto pred = [&] { return rp->state >= 2; };
  if (timeout_us < 0) {
    g_svc.done_cv.wait(lk, pred);
  } else if (!g_svc.done_cv.wait_for(lk, std::chrono::microseconds(timeout_us), pred)) {
    return fail(PIMUL_ETIMEDOUT, "request not finished within the timeout");
  }
  return rp->state == 3 ? fail(PIMUL_ECUDA, "request failed") : PIMUL_OK;
}

int pimul_handle_size(uint64_t handle, size_t* limbs) {
  std::lock_guard<std::mutex> lk(g_svc.mu);
  auto it = g_svc.handles.find(handle);
  if (it == g_svc.handles.end() || it->second.freed || !limbs) return fail(PIMUL_ENOTFOUND, "unknown handle");
  *limbs = it->second.limbs;
  return PIMUL_OK;
}

int pimul_download(uint64_t handle, uint64_t* host, size_t cap, size_t* len) {
  if (!len) return fail(PIMUL_EINVAL, "null len");
  uint64_t* d;
  uint64_t n;
  cudaEvent_t ready;
  int64_t producer;
  {
    std::lock_guard<std::mutex> lk(g_svc.mu);
    auto it = g_svc.handles.find(handle);
    if (it == g_svc.handles.end() || it->second.freed) return fail(PIMUL_ENOTFOUND, "unknown handle");
    d = it->second.d;
    n = it->second.limbs;
    producer = it->second.producer;
  }
  if (producer >= 0) {
    int rc = pimul_wait((uint64_t)producer, -1);
    if (rc) return rc;
  }
  {
    std::lock_guard<std::mutex> lk(g_svc.mu);
    ready = g_svc.handles[handle].ready;
  }
  if (cap < n) return fail(PIMUL_EINVAL, "capacity below the stored length");
  cudaStream_t st;
  int rc = get_stream(&st);
  if (rc) return rc;
  if (ready) CU(cudaStreamWaitEvent(st, ready, 0));
  rc = device_to_host(host, d, n * 8, st);
  if (rc) return rc;
  size_t m = n;
  while (m && host[m - 1] == 0) m--;
  *len = m;
  return PIMUL_OK;
}

int pimul_free(uint64_t handle) {
  std::unique_lock<std::mutex> lk(g_svc.mu);
  auto it = g_svc.handles.find(handle);
  if (it == g_svc.handles.end() || it->second.freed) return fail(PIMUL_ENOTFOUND, "unknown or already freed handle");
  int64_t producer = it->second.producer;
  lk.unlock();
  if (producer >= 0) pimul_wait((uint64_t)producer, -1);
  lk.lock();
  // requests that read the handle must finish first
  g_svc.done_cv.wait(lk, [&] {
    auto f = g_svc.handles.find(handle);
    return f == g_svc.handles.end() || f->second.readers <= 0;
  });
  auto f = g_svc.handles.find(handle);
  if (f == g_svc.handles.end()) return fail(PIMUL_ENOTFOUND, "handle freed concurrently");
  svc_free_now(handle);
  g_svc.dirty = true;
  return PIMUL_OK;
}

int pimul_release(uint64_t handle) {
  std::lock_guard<std::mutex> lk(g_svc.mu);
  auto it = g_svc.handles.find(handle);
  if (it == g_svc.handles.end() || it->second.freed || it->second.release)
    return fail(PIMUL_ENOTFOUND, "unknown, freed or released handle");
  it->second.release = true;
  if (!it->second.pending && it->second.readers <= 0) {
    svc_free_now(handle);
    g_svc.dirty = true;
  }
  return PIMUL_OK;
}

int pimul_adopt(const uint64_t* d, size_t n, uint64_t* handle) {
  if (!handle || (n && !d)) return fail(PIMUL_EINVAL, "null argument");
  int rc = svc_start();
  if (rc) return rc;
  std::lock_guard<std::mutex> lk(g_svc.mu);
  uint64_t id = svc_new_handle(n, const_cast<uint64_t*>(d), false, 0);
  g_svc.handles[id].borrowed = true;
  *handle = id;
  return PIMUL_OK;
}

int pimul_handle_device(uint64_t handle, const uint64_t** d, size_t* limbs) {
  if (!d || !limbs) return fail(PIMUL_EINVAL, "null argument");
  int64_t producer;
  {
    std::lock_guard<std::mutex> lk(g_svc.mu);
    auto it = g_svc.handles.find(handle);
    if (it == g_svc.handles.end() || it->second.freed) return fail(PIMUL_ENOTFOUND, "unknown handle");
    producer = it->second.producer;
  }
  if (producer >= 0) {
    int rc = pimul_wait((uint64_t)producer, -1);
    if (rc) return rc;
  }
  std::lock_guard<std::mutex> lk(g_svc.mu);
  auto it = g_svc.handles.find(handle);
  if (it == g_svc.handles.end()) return fail(PIMUL_ENOTFOUND, "handle freed concurrently");
  *d = it->second.d;
  *limbs = it->second.limbs;
  return PIMUL_OK;
}

int pimul_service_stats(double* p50_ms, double* p99_ms, uint64_t* completed, uint64_t* batches, uint64_t* in_use) {
  std::lock_guard<std::mutex> lk(g_svc.mu);
  std::vector<double> v = g_svc.latencies;
  std::sort(v.begin(), v.end());
  auto pct = [&](double q) { return v.empty() ? 0.0 : 1e3 * v[std::min(v.size() - 1, (size_t)(q * (v.size() - 1) + 0.5))]; };
  if (p50_ms) *p50_ms = pct(0.50);
  if (p99_ms) *p99_ms = pct(0.99);
  if (completed) *completed = g_svc.completed;
  if (batches) *batches = g_svc.batches;
  if (in_use) *in_use = g_svc.in_use;
  return PIMUL_OK;
}

int pimul_service_config(int big_log_n, int max_batch) {
  std::lock_guard<std::mutex> lk(g_svc.mu);
  if (big_log_n > 0) g_svc.big_log_n = big_log_n;
  if (max_batch > 0) g_svc.max_batch = max_batch;
  g_svc.dirty = true;
  return PIMUL_OK;
}

int pimul_service_reset_stats(void) {
  std::lock_guard<std::mutex> lk(g_svc.mu);
  g_svc.latencies.clear();
  g_svc.completed = 0;
  g_svc.batches = 0;
  return PIMUL_OK;
}

// ------------------------------------------------- batched add / subtract
// out = x + y or x - y (x >= y) for many limb arrays at once, the additions
// and subtractions of a binary-splitting level done where its products
// live.  Same carry-lookahead structure as the product's carry pass: windows
// of 4 limbs add with carry-in 0 and report (generate, propagate); a scan
// over chunk summaries gives every window its carry; windows that receive
// one ripple it (+1 / -1) through their limbs.  A carry or borrow out of the
// top limb is reported (it means x < y for a subtraction).
constexpr int AS_THREADS = 256;
constexpr int AS_W = 4;

struct AsJob {
  const uint64_t* x;
  const uint64_t* y;
  uint64_t* out;
  uint64_t nx, ny, nout;
  uint8_t* aux;  // per-warp masks, per-chunk (g, p) and carry-in bytes
  uint32_t sub;
  uint32_t check;  // report a carry or borrow out of the top limb
};

__host__ __device__ __forceinline__ uint64_t as_nwin(uint64_t nout) { return (nout + AS_W - 1) / AS_W; }
__host__ __device__ __forceinline__ uint64_t as_nchunk(uint64_t nout) {
  return (as_nwin(nout) + AS_THREADS - 1) / AS_THREADS;
}
__host__ __device__ __forceinline__ uint64_t as_aux_bytes(uint64_t nout) {
  uint64_t nc = as_nchunk(nout);
  return round_up_u64(nc * (AS_THREADS / 32) * 8 + 2 * nc + 16, 16);
}

__global__ void __launch_bounds__(AS_THREADS) k_as_local(const AsJob* jobs) {
  const AsJob J = jobs[blockIdx.y];
  const uint64_t nwin = as_nwin(J.nout), nchunk = as_nchunk(J.nout);
  if (blockIdx.x >= nchunk) return;
  uint32_t* masks = reinterpret_cast<uint32_t*>(J.aux);
  uint8_t* chunk_gp = J.aux + nchunk * (AS_THREADS / 32) * 8;
  __shared__ uint32_t sA[AS_THREADS / 32], sB[AS_THREADS / 32];
  const uint64_t w = (uint64_t)blockIdx.x * AS_THREADS + threadIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  bool g = false, p = false;
  if (w < nwin) {
    uint64_t c = 0;
    bool all = true;
#pragma unroll
    for (int t = 0; t < AS_W; t++) {
      const uint64_t i = AS_W * w + t;
      if (i >= J.nout) break;
      const uint64_t xi = i < J.nx ? J.x[i] : 0, yi = i < J.ny ? J.y[i] : 0;
      uint64_t z;
      if (J.sub) {
        const uint64_t d = xi - yi;
        const uint64_t b1 = xi < yi, b2 = d < c;
        z = d - c;
        c = b1 | b2;
        all = all && z == 0;
      } else {
        const uint64_t s0 = xi + yi;
        const uint64_t c1 = s0 < xi;
        z = s0 + c;
        c = c1 | (z < s0);
        all = all && z == ~0ull;
      }
      J.out[i] = z;
    }
    g = c != 0;
    p = all;
  }
  const uint32_t A = __ballot_sync(0xFFFFFFFFu, g || p);
  const uint32_t Bm = __ballot_sync(0xFFFFFFFFu, g);
  if (lane == 0) {
    const uint64_t wi = (uint64_t)blockIdx.x * (AS_THREADS / 32) + warp;
    masks[2 * wi] = A;
    masks[2 * wi + 1] = Bm;
    sA[warp] = A;
    sB[warp] = Bm;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t cg = 0, cp = 1;  // chunk carry out for carry in 0 / 1
    for (int k = 0; k < AS_THREADS / 32; k++) {
      uint64_t sg = (uint64_t)sA[k] + sB[k] + cg;
      uint64_t sp = (uint64_t)sA[k] + sB[k] + cp;
      cg = (uint32_t)(sg >> 32);
      cp = (uint32_t)(sp >> 32);
    }
    chunk_gp[blockIdx.x] = (uint8_t)(cg | (cp << 1));
  }
}

// One CTA per job: carry into every chunk (segments of chunks per thread,
// chained by thread 0).
__global__ void __launch_bounds__(1024) k_as_scan(const AsJob* jobs) {
  const AsJob J = jobs[blockIdx.x];
  const uint64_t nchunk = as_nchunk(J.nout);
  const uint8_t* chunk_gp = J.aux + nchunk * (AS_THREADS / 32) * 8;
  uint8_t* chunk_cin = J.aux + nchunk * (AS_THREADS / 32) * 8 + nchunk;
  __shared__ uint8_t seg_g[1024], seg_p[1024], seg_cin[1024];
  const uint64_t per = (nchunk + 1023) / 1024;
  const uint64_t lo = threadIdx.x * per, hi = lo + per < nchunk ? lo + per : nchunk;
  uint8_t cg = 0, cp = 1;
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
    // only the first ceil(nchunk / per) segments hold chunks
    const int used = (int)((nchunk + per - 1) / per);
    uint8_t cin = 0;
    for (int k = 0; k < used; k++) {
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

// Windows that receive a carry ripple it; the top window's carry out
// (generated, or propagated from its carry in) sets *overflow.
__global__ void __launch_bounds__(AS_THREADS) k_as_apply(const AsJob* jobs, int* overflow) {
  const AsJob J = jobs[blockIdx.y];
  const uint64_t nwin = as_nwin(J.nout), nchunk = as_nchunk(J.nout);
  if (blockIdx.x >= nchunk) return;
  const uint32_t* masks = reinterpret_cast<const uint32_t*>(J.aux);
  const uint8_t* chunk_cin = J.aux + nchunk * (AS_THREADS / 32) * 8 + nchunk;
  const uint64_t w = (uint64_t)blockIdx.x * AS_THREADS + threadIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t cin = nchunk == 1 ? 0 : chunk_cin[blockIdx.x];  // one chunk: no scan ran
  const uint64_t wbase = (uint64_t)blockIdx.x * (AS_THREADS / 32);
  for (int k = 0; k < warp; k++) {
    uint64_t s = (uint64_t)masks[2 * (wbase + k)] + masks[2 * (wbase + k) + 1] + cin;
    cin = (uint32_t)(s >> 32);
  }
  const uint32_t A = masks[2 * (wbase + warp)], Bm = masks[2 * (wbase + warp) + 1];
  const uint32_t carries = (A + Bm + cin) ^ A ^ Bm;
  if (J.check && w + 1 == nwin) {
    const uint32_t g = (Bm >> lane) & 1, pg = (A >> lane) & 1, c = (carries >> lane) & 1;
    if (g || (pg && c)) atomicExch(overflow, 1);
  }
  if (w < nwin && ((carries >> lane) & 1)) {
    for (int t = 0; t < AS_W; t++) {
      const uint64_t i = AS_W * w + t;
      if (i >= J.nout) break;
      if (J.sub) {
        if (J.out[i]-- != 0) break;
      } else {
        if (++J.out[i] != 0) break;
      }
    }
  }
}

// Highest nonzero limb + 1 of each array (0 for zero): *len must be zero
// on entry; CTAs scan 2^12-limb chunks and keep the maximum.
__global__ void __launch_bounds__(256) k_top_limb(const uint64_t* const* arrs, const uint64_t* n, uint64_t* len) {
  const uint32_t j = blockIdx.y;
  const uint64_t lo = (uint64_t)blockIdx.x << 12;
  if (lo >= n[j]) return;
  const uint64_t hi = lo + 4096 < n[j] ? lo + 4096 : n[j];
  const uint64_t* a = arrs[j];
  uint64_t best = 0;
  for (uint64_t i = lo + threadIdx.x; i < hi; i += 256)
    if (a[i]) best = i + 1;
  for (int o = 16; o > 0; o >>= 1) {
    uint64_t other = __shfl_down_sync(0xFFFFFFFFu, best, o);
    best = other > best ? other : best;
  }
  if ((threadIdx.x & 31) == 0 && best) atomicMax((unsigned long long*)&len[j], (unsigned long long)best);
}

// Batched add/subtract on `st` (asynchronous); *d_overflow (device int,
// zeroed by the caller) is set when a carry or borrow leaves a top limb.
static int addsub_launch(const pimul_addsub_job* jobs, size_t n, cudaStream_t st, int* d_overflow, bool unchecked) {
  if (n == 0) return PIMUL_OK;
  uint64_t aux_total = 0, max_chunk = 0;
  for (size_t i = 0; i < n; i++) {
    aux_total += as_aux_bytes(jobs[i].nout);
    max_chunk = std::max<uint64_t>(max_chunk, as_nchunk(jobs[i].nout));
  }
  const uint64_t desc = round_up_u64(n * sizeof(AsJob), 256);
  uint8_t* dev = nullptr;
  cudaError_t e = cudaMallocAsync((void**)&dev, desc + aux_total, g_dev.pool, st);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(PIMUL_ENOMEM, std::string("add/subtract scratch: ") + cudaGetErrorString(e));
  }
  AsJob* h = reinterpret_cast<AsJob*>(host_image(n * sizeof(AsJob)));
  uint64_t off = desc;
  for (size_t i = 0; i < n; i++) {
    h[i] = AsJob{jobs[i].x, jobs[i].y, jobs[i].out, jobs[i].nx, jobs[i].ny, jobs[i].nout, dev + off,
                 (uint32_t)(jobs[i].sub != 0), (uint32_t)(!unchecked && jobs[i].sub != PIMUL_SUB_MOD)};
    off += as_aux_bytes(jobs[i].nout);
  }
  if (host_to_device(dev, h, n * sizeof(AsJob), st)) e = cudaErrorUnknown;
  if (e == cudaSuccess) {
    const AsJob* dj = reinterpret_cast<const AsJob*>(dev);
    for (size_t j0 = 0; j0 < n; j0 += 65535) {
      const unsigned nj = (unsigned)std::min<size_t>(65535, n - j0);
      k_as_local<<<dim3((unsigned)max_chunk, nj), AS_THREADS, 0, st>>>(dj + j0);
      if (max_chunk > 1) k_as_scan<<<nj, 1024, 0, st>>>(dj + j0);
      k_as_apply<<<dim3((unsigned)max_chunk, nj), AS_THREADS, 0, st>>>(dj + j0, d_overflow);
    }
    e = cudaGetLastError();
  }
  // the host image is pageable: the copy has been staged before return
  cudaFreeAsync(dev, st);
  if (e != cudaSuccess) return fail(PIMUL_ECUDA, std::string("add/subtract launch: ") + cudaGetErrorString(e));
  return PIMUL_OK;
}

int pimul_addsub_batch(const pimul_addsub_job* jobs, size_t n, void* stream) {
  if (n && !jobs) return fail(PIMUL_EINVAL, "null job list");
  for (size_t i = 0; i < n; i++) {
    const pimul_addsub_job& j = jobs[i];
    if (j.nout && !j.out) return fail(PIMUL_EINVAL, "null output");
    if ((j.nx && !j.x) || (j.ny && !j.y)) return fail(PIMUL_EINVAL, "null operand");
    if (j.nout < std::max(j.nx, j.ny)) return fail(PIMUL_EINVAL, "output shorter than an operand");
  }
  cudaStream_t st;
  int rc = get_stream(&st);
  if (rc) return rc;
  if (stream) st = (cudaStream_t)stream;
  int* d_flag = nullptr;
  CU(cudaMallocAsync((void**)&d_flag, sizeof(int), g_dev.pool, st));
  CU(cudaMemsetAsync(d_flag, 0, sizeof(int), st));
  bool all_mod = true;
  for (size_t i = 0; i < n && all_mod; i++) all_mod = jobs[i].sub == PIMUL_SUB_MOD;
  rc = addsub_launch(jobs, n, st, d_flag, false);
  if (all_mod) {  // nothing to check: stay asynchronous
    cudaFreeAsync(d_flag, st);
    return rc;
  }
  int h_flag = 0;
  if (!rc) {
    cudaError_t e = cudaMemcpyAsync(&h_flag, d_flag, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) rc = fail(PIMUL_ECUDA, std::string("add/subtract: ") + cudaGetErrorString(e));
  }
  cudaFreeAsync(d_flag, st);
  if (!rc && h_flag) rc = fail(PIMUL_EINVAL, "carry or borrow out of the top limb (x < y in a subtraction?)");
  return rc;
}

// Wrapped products (PIMUL_BATCH_WRAP): a unit of 2^20 points or more whose
// coefficients fill at most 5/8 of its transform, with every operand within
// half of it, runs as a cyclic product of half the length; the coefficients
// that wrap around (wrap of them, at most a quarter of the half length) are
// separated again with the exact low coefficients of the product, from a
// short product of the operands' low limbs computed first (coefficients
// out, no carry).  plan_wraps marks the eligible units (forceL, wrap) and
// returns their short products, whose output buffers (and the units' low
// pointers) the caller assigns from one allocation of `words` words.
struct WrapPlan {
  std::vector<Unit> low;      // the short products, in the order of the wrapped units
  std::vector<size_t> which;  // the wrapped units
  uint64_t words = 0;
};

static WrapPlan plan_wraps(std::vector<Unit>& units) {
  WrapPlan W;
  for (size_t i = 0; i < units.size(); i++) {
    Unit& u = units[i];
    if (u.coeff || u.forceL || !u.la || !u.lb) continue;
    const int L = log2_ceil(4 * u.nout - 1);
    if (L < 20 || L > 32) continue;
    const uint64_t Nw = 1ull << (L - 1);
    const uint64_t n1 = 4 * (u.la + u.lb), n2 = u.la2 ? 4 * (u.la2 + u.lb2) : 0;
    const uint64_t ncoef = std::max(n1, n2) - 1;
    if (ncoef <= Nw || ncoef - Nw > Nw / 4) continue;
    if (4 * u.la > Nw || 4 * u.lb > Nw || 4 * u.la2 > Nw || 4 * u.lb2 > Nw) continue;
    const uint64_t m = ncoef - Nw, ml = (m + 3) / 4;  // wrapped coefficients; limbs holding them
    Unit lo{};
    lo.a = u.a, lo.la = std::min(u.la, ml), lo.b = u.b, lo.lb = std::min(u.lb, ml);
    if (u.la2) lo.a2 = u.a2, lo.la2 = std::min(u.la2, ml), lo.b2 = u.b2, lo.lb2 = std::min(u.lb2, ml);
    const uint64_t nl = std::max(4 * (lo.la + lo.lb), lo.la2 ? 4 * (lo.la2 + lo.lb2) : 0) - 1;
    lo.forceL = std::max(SMALL_LOG_MAX + 1, log2_ceil(nl));
    lo.coeff = true;
    lo.nout = m;
    W.low.push_back(lo);
    W.which.push_back(i);
    u.forceL = L - 1;
    u.wrap = m;
    W.words += round_up_u64(m, 32);
  }
  return W;
}

static int sum_batch_impl(const pimul_sum_job* jobs, size_t n, cudaStream_t st, bool allow_wrap);

int pimul_sum_batch(const pimul_sum_job* jobs, size_t n, void* stream) {
  cudaStream_t st;
  int rc = get_stream(&st);
  if (rc) return rc;
  if (stream) st = (cudaStream_t)stream;
  return sum_batch_impl(jobs, n, st, false);
}

int pimul_sum_batch_ex(const pimul_sum_job* jobs, size_t n, void* stream, unsigned flags) {
  if (flags & ~PIMUL_BATCH_WRAP) return fail(PIMUL_EINVAL, "unknown batch flags");
  cudaStream_t st;
  int rc = get_stream(&st);
  if (rc) return rc;
  if (stream) st = (cudaStream_t)stream;
  return sum_batch_impl(jobs, n, st, (flags & PIMUL_BATCH_WRAP) != 0);
}

static int sum_batch_impl(const pimul_sum_job* jobs, size_t n, cudaStream_t st, bool allow_wrap) {
  int rc = PIMUL_OK;
  if (n && !jobs) return fail(PIMUL_EINVAL, "null job list");
  // fused sums go to the pass pipeline; a sum of short products (or with a
  // square) is two products into scratch and one batched addition
  std::vector<Unit> units;
  units.reserve(n);
  std::vector<size_t> fb;  // jobs computed as two products + an addition
  std::vector<std::pair<uint64_t*, uint64_t>> zero;  // output limbs above the result
  uint64_t tmp_words = 0;
  for (size_t i = 0; i < n; i++) {
    const pimul_sum_job& j = jobs[i];
    const bool p1 = j.la1 && j.lb1, p2 = j.la2 && j.lb2;
    if ((p1 && (!j.a1 || !j.b1)) || (p2 && (!j.a2 || !j.b2))) return fail(PIMUL_EINVAL, "null operand");
    const uint64_t n1 = p1 ? j.la1 + j.lb1 : 0, n2 = p2 ? j.la2 + j.lb2 : 0;
    const uint64_t need = std::max(n1, n2) + (p1 && p2 ? 1 : 0);
    if (j.nout < need) return fail(PIMUL_EINVAL, "nout below max(la1 + lb1, la2 + lb2) + 1");
    if (j.nout && !j.out) return fail(PIMUL_EINVAL, "null output");
    if (j.nout > need) zero.emplace_back(j.out + need, j.nout - need);
    if (!p1 && !p2) continue;
    if (p1 != p2) {
      units.push_back(p1 ? Unit{j.a1, j.la1, j.b1, j.lb1, nullptr, 0, nullptr, 0, j.out, n1}
                         : Unit{j.a2, j.la2, j.b2, j.lb2, nullptr, 0, nullptr, 0, j.out, n2});
      continue;
    }
    const bool sq = (j.a1 == j.b1 && j.la1 == j.lb1) || (j.a2 == j.b2 && j.la2 == j.lb2);
    const int L = log2_ceil(4 * need - 1);
    if (L > 32) return fail(PIMUL_EINVAL, "transform length above 2^32 in batch");
    // fused only when both products already need that transform length (a
    // shorter second product would run at twice its own length)
    const bool same = log2_ceil(4 * n1 - 1) == L && log2_ceil(4 * n2 - 1) == L;
    if (sq || L <= SMALL_LOG_MAX || !same) {
      fb.push_back(i);
      tmp_words += n1 + n2;
      continue;
    }
    units.push_back(Unit{j.a1, j.la1, j.b1, j.lb1, j.a2, j.la2, j.b2, j.lb2, j.out, need});
  }
  uint8_t* tmp = nullptr;
  std::vector<pimul_addsub_job> aj;
  if (!fb.empty()) {
    CU(cudaMallocAsync((void**)&tmp, tmp_words * 8 + 256, g_dev.pool, st));
    uint64_t* t = reinterpret_cast<uint64_t*>(tmp + 256);  // first 256 bytes: the overflow flag
    for (size_t i : fb) {
      const pimul_sum_job& j = jobs[i];
      const uint64_t n1 = j.la1 + j.lb1, n2 = j.la2 + j.lb2;
      units.push_back(Unit{j.a1, j.la1, j.b1, j.lb1, nullptr, 0, nullptr, 0, t, n1});
      units.push_back(Unit{j.a2, j.la2, j.b2, j.lb2, nullptr, 0, nullptr, 0, t + n1, n2});
      aj.push_back(pimul_addsub_job{t, n1, t + n1, n2, j.out, std::max(n1, n2) + 1, 0});
      t += n1 + n2;
    }
  }
  for (const auto& z : zero) {
    cudaError_t e = cudaMemsetAsync(z.first, 0, z.second * 8, st);
    if (e != cudaSuccess && !rc) rc = fail(PIMUL_ECUDA, std::string("sum batch: ") + cudaGetErrorString(e));
  }
  // wrapped units: their low coefficients first, into one buffer
  uint64_t* lowbuf = nullptr;
  if (!rc && allow_wrap) {
    WrapPlan W = plan_wraps(units);
    if (!W.low.empty()) {
      cudaError_t e = cudaMallocAsync((void**)&lowbuf, W.words * 8, g_dev.pool, st);
      if (e != cudaSuccess) {
        cudaGetLastError();
        rc = fail(PIMUL_ENOMEM, std::string("wrapped products: ") + cudaGetErrorString(e));
      } else {
        uint64_t off = 0;
        for (size_t k = 0; k < W.low.size(); k++) {
          W.low[k].out = lowbuf + off;
          units[W.which[k]].low = lowbuf + off;
          off += round_up_u64(W.low[k].nout, 32);
        }
        rc = run_units(W.low.data(), W.low.size(), st, true);
      }
    }
  }
  if (!rc) rc = run_units(units.data(), units.size(), st, true);
  if (lowbuf) cudaFreeAsync(lowbuf, st);
  if (!rc && !aj.empty()) {
    cudaError_t e = cudaMemsetAsync(tmp, 0, sizeof(int), st);
    if (e == cudaSuccess) rc = addsub_launch(aj.data(), aj.size(), st, reinterpret_cast<int*>(tmp), false);
    else rc = fail(PIMUL_ECUDA, std::string("sum batch: ") + cudaGetErrorString(e));
  }
  if (tmp) cudaFreeAsync(tmp, st);
  return rc;
}

int pimul_top_limbs(const uint64_t* const* arrays, const size_t* lens, size_t n, size_t* out_lens, void* stream) {
  if (n == 0) return PIMUL_OK;
  if (!arrays || !lens || !out_lens) return fail(PIMUL_EINVAL, "null argument");
  cudaStream_t st;
  int rc = get_stream(&st);
  if (rc) return rc;
  if (stream) st = (cudaStream_t)stream;
  uint64_t max_chunk = 0;
  for (size_t i = 0; i < n; i++) max_chunk = std::max<uint64_t>(max_chunk, (lens[i] + 4095) / 4096);
  if (max_chunk == 0) {
    for (size_t i = 0; i < n; i++) out_lens[i] = 0;
    return PIMUL_OK;
  }
  const uint64_t bytes = round_up_u64(n * 8, 256);
  uint8_t* dev = nullptr;
  CU(cudaMallocAsync((void**)&dev, 3 * bytes, g_dev.pool, st));
  std::vector<uint64_t> hn(lens, lens + n);
  if (!rc) rc = host_to_device(dev, arrays, n * 8, st);
  if (!rc) rc = host_to_device(dev + bytes, hn.data(), n * 8, st);
  if (rc) {
    cudaFreeAsync(dev, st);
    return rc;
  }
  CU(cudaMemsetAsync(dev + 2 * bytes, 0, n * 8, st));
  for (size_t j0 = 0; j0 < n; j0 += 65535) {
    const unsigned nj = (unsigned)std::min<size_t>(65535, n - j0);
    k_top_limb<<<dim3((unsigned)max_chunk, nj), 256, 0, st>>>(
        reinterpret_cast<const uint64_t* const*>(dev) + j0, reinterpret_cast<const uint64_t*>(dev + bytes) + j0,
        reinterpret_cast<uint64_t*>(dev + 2 * bytes) + j0);
  }
  CU(cudaGetLastError());
  std::vector<uint64_t> res(n);
  rc = device_to_host(res.data(), dev + 2 * bytes, n * 8, st);
  cudaFreeAsync(dev, st);
  if (rc) return rc;
  for (size_t i = 0; i < n; i++) out_lens[i] = (size_t)res[i];
  return PIMUL_OK;
}

// pimul_mul's contract through the served form: upload, submit, wait,
// download, free.  A drop-in multiply backend for host drivers that want
// every product to pass through the service.
int pimul_mul_served(const uint64_t* a, size_t la, const uint64_t* b, size_t lb, uint64_t* out, size_t out_cap,
                     size_t* out_len) {
  if (!out_len) return fail(PIMUL_EINVAL, "null out_len");
  *out_len = 0;
  if (la == 0 || lb == 0) return PIMUL_OK;
  if (!a || !b || !out) return fail(PIMUL_EINVAL, "null pointer");
  if (out_cap < la + lb) return fail(PIMUL_EINVAL, "out_cap < la + lb");
  const bool sq = a == b && la == lb;
  uint64_t ha = 0, hb = 0, hc = 0, ticket = 0;
  bool has_a = false, has_b = false, has_c = false;
  int rc = pimul_upload(a, la, &ha);
  has_a = rc == PIMUL_OK;
  if (!rc && !sq) {
    rc = pimul_upload(b, lb, &hb);
    has_b = rc == PIMUL_OK;
  }
  if (!rc) {
    rc = pimul_submit(sq ? PIMUL_OP_SQR : PIMUL_OP_MUL, ha, sq ? ha : hb, &hc, &ticket);
    has_c = rc == PIMUL_OK;
  }
  if (!rc) rc = pimul_wait(ticket, -1);
  if (!rc) rc = pimul_download(hc, out, out_cap, out_len);
  if (has_c) pimul_free(hc);
  if (has_b) pimul_free(hb);
  if (has_a) pimul_free(ha);
  return rc;
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
  // a is uploaded first; b follows on a helper stream while a's forward
  // transform runs, and b's first pass waits for it
  rc = host_to_device(da, a, la * 8, st);
  thread_local cudaStream_t t_copy = nullptr;
  thread_local cudaEvent_t t_ev[2] = {nullptr, nullptr};
  thread_local int t_copy_dev = -1;
  cudaEvent_t b_ready = nullptr;
  if (!square) {
    if (!t_copy || t_copy_dev != g_dev.device) {
      CU(cudaStreamCreateWithFlags(&t_copy, cudaStreamNonBlocking));
      CU(cudaEventCreateWithFlags(&t_ev[0], cudaEventDisableTiming));
      CU(cudaEventCreateWithFlags(&t_ev[1], cudaEventDisableTiming));
      t_copy_dev = g_dev.device;
    }
    CU(cudaEventRecord(t_ev[0], st));  // after db's allocation and a's upload
    CU(cudaStreamWaitEvent(t_copy, t_ev[0], 0));
    if (!rc) rc = host_to_device(db, b, lb * 8, t_copy);
    CU(cudaEventRecord(t_ev[1], t_copy));
    b_ready = t_ev[1];
  }
  if (!rc) rc = mul_device(da, la, square ? da : db, lb, dout, st, b_ready);
  if (rc && b_ready) cudaStreamWaitEvent(st, b_ready, 0);  // db is freed below
  if (rc == PIMUL_OK) rc = device_to_host(out, dout, (la + lb) * 8, st);
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
//    scratch (17 MiB) and this path's own root tables (18 MiB) stay
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
//    pimul_shutdown forgets the set-up, so a call after a cudaDeviceReset
//    (made after pimul_shutdown) resolves the addresses and copies the
//    tables again.
namespace pimul {
// The service's additions and subtractions: no carry or borrow can leave
// their outputs (sums get max + 1 limbs, differences are of a >= b), so the
// batch is launched unchecked and stays asynchronous.
int svc_addsub(const pimul_addsub_job* jobs, size_t n, cudaStream_t st) {
  return ::addsub_launch(jobs, n, st, nullptr, true);
}

// ---- strided batches: n operations of one shape at fixed strides --------
// (a level of the decimal conversion holds up to 5 * 10^5 nodes of one
// shape).  The descriptors are written by a kernel instead of the host, so
// queueing such a batch costs a few launches whatever n is.

// Descriptors and chunks of n products (a + i sa) * b -> out + i so, all of
// one transform length 2^L <= 2^SMALL_LOG_MAX, per products per chunk.
__global__ void k_fill_small(SmallJob* jobs, SmallChunk* chunks, SmallJob base, uint64_t sa, uint64_t so, uint32_t n,
                             uint32_t per, int L) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  jobs[i] = SmallJob{base.a + (uint64_t)i * sa, base.b, base.out + (uint64_t)i * so, base.la, base.lb};
  if (i < ((uint64_t)n + per - 1) / per) chunks[i] = SmallChunk{i * per, per < n - i * per ? per : n - i * per, L};
}

int mul_batch_strided(const uint64_t* a, uint64_t sa, size_t la, const uint64_t* b, size_t lb, uint64_t* out,
                      uint64_t so, size_t n, cudaStream_t st) {
  if (!n) return PIMUL_OK;
  const int L = la && lb ? log2_ceil(4 * (uint64_t)(la + lb) - 1) : -1;
  if (L < 0 || L > SMALL_LOG_MAX || n > 0xFFFFFFFFull) {
    // the pass pipeline, or an empty product: the general batch
    std::vector<pimul_job> jobs(n);
    for (size_t i = 0; i < n; i++) jobs[i] = pimul_job{a + i * sa, la, b, lb, out + i * so};
    return pimul_mul_batch(jobs.data(), n, st);
  }
  cudaStream_t own;
  int rc = get_stream(&own);  // initialises the engine on first use
  if (rc) return rc;
  const uint32_t per = SMALL_THREADS / small_group_threads(L);
  const size_t nch = (n + per - 1) / per;
  const size_t jb = round256(n * sizeof(SmallJob));
  uint8_t* dev = nullptr;
  cudaError_t e = cudaMallocAsync((void**)&dev, jb + nch * sizeof(SmallChunk), g_dev.pool, st);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(PIMUL_ENOMEM, std::string("strided batch descriptors: ") + cudaGetErrorString(e));
  }
  SmallJob* dj = reinterpret_cast<SmallJob*>(dev);
  SmallChunk* dc = reinterpret_cast<SmallChunk*>(dev + jb);
  k_fill_small<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(dj, dc, SmallJob{a, b, out, (uint32_t)la, (uint32_t)lb},
                                                           sa, so, (uint32_t)n, per, L);
  int sms = 152;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, g_dev.device);
  const uint64_t grid = std::min<uint64_t>((uint64_t)sms * (uint64_t)g_small_ctas_per_sm.load(), nch);
  k_small_mul<<<(unsigned)grid, SMALL_THREADS, small_cta_smem(L), st>>>(dj, dc, SmallJob{}, (uint32_t)nch, g_dev.roots);
  e = cudaGetLastError();
  cudaFreeAsync(dev, st);
  if (e != cudaSuccess) return fail(PIMUL_ECUDA, std::string("strided batch launch: ") + cudaGetErrorString(e));
  return PIMUL_OK;
}

__global__ void k_fill_as(AsJob* jobs, AsJob base, uint64_t sx, uint64_t sy, uint64_t so, uint64_t saux, uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  AsJob j = base;
  j.x += (uint64_t)i * sx;
  j.y += (uint64_t)i * sy;
  j.out += (uint64_t)i * so;
  j.aux += (uint64_t)i * saux;
  jobs[i] = j;
}

int addsub_strided(const uint64_t* x, uint64_t sx, size_t nx, const uint64_t* y, uint64_t sy, size_t ny, uint64_t* out,
                   uint64_t so, size_t nout, int sub, size_t n, cudaStream_t st) {
  if (!n || !nout) return PIMUL_OK;
  if (nout < std::max(nx, ny)) return fail(PIMUL_EINVAL, "output shorter than an operand");
  if (n > 0xFFFFFFFFull) {
    std::vector<pimul_addsub_job> jobs(n);
    for (size_t i = 0; i < n; i++) jobs[i] = pimul_addsub_job{x + i * sx, nx, y + i * sy, ny, out + i * so, nout, sub};
    return svc_addsub(jobs.data(), n, st);
  }
  const uint64_t saux = as_aux_bytes(nout), nchunk = as_nchunk(nout);
  const uint64_t desc = round_up_u64(n * sizeof(AsJob), 256);
  uint8_t* dev = nullptr;
  cudaError_t e = cudaMallocAsync((void**)&dev, desc + n * saux, g_dev.pool, st);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(PIMUL_ENOMEM, std::string("strided add/subtract scratch: ") + cudaGetErrorString(e));
  }
  AsJob* dj = reinterpret_cast<AsJob*>(dev);
  k_fill_as<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(
      dj, AsJob{x, y, out, nx, ny, nout, dev + desc, (uint32_t)(sub != 0), 0u}, sx, sy, so, saux, (uint32_t)n);
  for (size_t j0 = 0; j0 < n; j0 += 65535) {
    const unsigned nj = (unsigned)std::min<size_t>(65535, n - j0);
    k_as_local<<<dim3((unsigned)nchunk, nj), AS_THREADS, 0, st>>>(dj + j0);
    if (nchunk > 1) k_as_scan<<<nj, 1024, 0, st>>>(dj + j0);
    k_as_apply<<<dim3((unsigned)nchunk, nj), AS_THREADS, 0, st>>>(dj + j0, nullptr);
  }
  e = cudaGetLastError();
  cudaFreeAsync(dev, st);
  if (e != cudaSuccess) return fail(PIMUL_ECUDA, std::string("strided add/subtract launch: ") + cudaGetErrorString(e));
  return PIMUL_OK;
}
}  // namespace pimul

namespace pimul {
constexpr int NOALLOC_LOG_MAX = 20;
constexpr uint64_t NOALLOC_N_MAX = 1ull << NOALLOC_LOG_MAX;
constexpr uint64_t NOALLOC_WIN_MAX = NOALLOC_N_MAX / WIN_COEFFS;
constexpr uint64_t NOALLOC_CHUNK_MAX = (NOALLOC_WIN_MAX + CARRY_THREADS - 1) / CARRY_THREADS;
constexpr uint64_t NOALLOC_AUX_WORDS = (NOALLOC_CHUNK_MAX * (CARRY_THREADS / 32) * 8 + 2 * NOALLOC_CHUNK_MAX + 64) / 8 + 1;
static_assert(NOALLOC_AUX_WORDS * 8 >= NOALLOC_CHUNK_MAX * (CARRY_THREADS / 32) * 8 + 2 * NOALLOC_CHUNK_MAX + 64,
              "no-alloc carry flags must fit");

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

// Forget every device's set-up (pimul_shutdown): the next no-alloc call on a
// device resolves the symbol addresses and copies the root tables again, as
// it must after a cudaDeviceReset.
void noalloc_forget() {
  std::lock_guard<std::mutex> lk(g_na_mu);
  for (NoAllocDev& d : g_na) d = NoAllocDev{};
}

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
    k_small_mul<<<1, SMALL_THREADS, small_cta_smem(z.L), st>>>(nullptr, nullptr, job, 1, R);
    CU(cudaGetLastError());
    return PIMUL_OK;
  }
  const bool square = d_a == d_b && la == lb;
  Job J{d_a, d_b, d_out, nullptr, nullptr, nullptr, nullptr, la, lb};
  J.A = nd->scratch;
  J.B = square ? nullptr : nd->scratch + NOALLOC_N_MAX;
  J.H = nd->scratch + 2 * NOALLOC_N_MAX;
  J.aux = reinterpret_cast<uint8_t*>(nd->scratch + 2 * NOALLOC_N_MAX + NOALLOC_WIN_MAX);
  Launcher X{st, false, R};  // no statistics hook: its event timing would create CUDA events
  X.tables = false;          // nor the twiddle tables, which are allocated on first use
  run_large(X, nullptr, J, 1, z.L, z.nchunk);
  CU(cudaGetLastError());
  return PIMUL_OK;
}
}  // namespace pimul

extern "C" int pimul_mul_device_noalloc(const uint64_t* d_a, size_t la, const uint64_t* d_b, size_t lb,
                                        uint64_t* d_out, void* stream) {
  if (la == 0 || lb == 0) return PIMUL_OK;
  if (!d_a || !d_b || !d_out) return fail(PIMUL_EINVAL, "null device pointer");
  // each operand is checked before the sum is formed, so that no size_t
  // wrap-around can let an oversized pair through
  if (la > NOALLOC_N_MAX / 4 || lb > NOALLOC_N_MAX / 4 - la)
    return fail(PIMUL_EINVAL, "product too large for the no-alloc scratch: la + lb must be <= 262144 limbs "
                              "(transform length <= 2^20)");
  return mul_device_noalloc(d_a, la, d_b, lb, d_out, (cudaStream_t)stream);
}

// ---------------------------------------- merged splitting levels (internal)
namespace pimerge {

int prepare() { return pimul::ensure_init(-1); }

int merge_level(const Level& lv, int* d_bad, cudaStream_t stream) {
  using namespace pimul;
  if (lv.L < MIN_LOG || lv.L > MAX_LOG || !d_bad || lv.op < lv.sp || lv.oq < lv.sq || lv.ot < lv.st)
    return PIMUL_EINVAL;
  if (lv.n_in < 2) return PIMUL_OK;
  int rc = ensure_init(-1);
  if (rc) return rc;
  const MergeLevel M{lv.in, lv.in_len, lv.out, lv.out_len, lv.sp, lv.sq, lv.st, lv.op, lv.oq, lv.ot,
                     lv.n_in, lv.L, d_bad};
  const uint32_t gpc = MERGE_THREADS / merge_group_threads(lv.L);
  const uint32_t items = lv.n_in / 2 + (lv.n_in & 1);
  const uint32_t nchunks = (items + gpc - 1) / gpc;
  int sms = 152;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, g_dev.device);
  const uint32_t grid = std::min<uint32_t>(nchunks, (uint32_t)sms * 2);
  const size_t smem = merge_cta_smem(lv.L);
  switch (lv.L) {
    case 8: k_split_merge<8><<<grid, MERGE_THREADS, smem, stream>>>(M, g_dev.roots); break;
    case 9: k_split_merge<9><<<grid, MERGE_THREADS, smem, stream>>>(M, g_dev.roots); break;
    case 10: k_split_merge<10><<<grid, MERGE_THREADS, smem, stream>>>(M, g_dev.roots); break;
    case 11: k_split_merge<11><<<grid, MERGE_THREADS, smem, stream>>>(M, g_dev.roots); break;
    default: k_split_merge<12><<<grid, MERGE_THREADS, smem, stream>>>(M, g_dev.roots); break;
  }
  g_launch[K_SMALL].fetch_add(1, std::memory_order_relaxed);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(PIMUL_ECUDA, std::string("merged splitting level: ") + cudaGetErrorString(e));
  return PIMUL_OK;
}

}  // namespace pimerge
