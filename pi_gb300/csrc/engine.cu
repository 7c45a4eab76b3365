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
  KTimer(int c, cudaStream_t s) : cls(c), st(s) {
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
struct PassArgs {
  uint64_t* data;
  int L;   // log2 N
  int r;   // log2 rows (radix of this pass)
  int s;   // log2 row stride (columns of a block)
  int t;   // log2 columns per tile
  int bc;  // log2 blocks per tile
  RoundPlan rp;
};

constexpr int PASS_THREADS = 512;
constexpr int TILE_LOG_MAX = 13;  // 8192 words (64 KiB) per tile

// Dynamic shared memory of a pass tile of 2^tile_log words (padded).
static inline size_t pass_smem_bytes(int tile_log) { return ((size_t)1 << tile_log) * 17 / 16 * 8; }

__device__ __forceinline__ uint64_t tile_gaddr(const PassArgs& a, uint32_t lin, uint64_t b0, uint64_t j0) {
  uint32_t j = lin & ((1u << a.t) - 1);
  uint32_t i = (lin >> a.t) & ((1u << a.r) - 1);
  uint32_t blk = lin >> (a.t + a.r);
  return ((b0 + blk) << (a.r + a.s)) + ((uint64_t)i << a.s) + j0 + j;
}

// One forward pass: load tile, R-point DFT per column, outgoing twiddle
// w_M^(f*j) with M = 2^(r+s), store in place.
__global__ void __launch_bounds__(PASS_THREADS) k_pass_fwd(PassArgs a, Roots R) {
  extern __shared__ uint64_t sm[];
  const int tid = threadIdx.x;
  const uint32_t E = 1u << (a.r + a.t + a.bc);
  const uint64_t ct = blockIdx.x & ((1u << (a.s - a.t)) - 1);
  const uint64_t bt = (uint64_t)blockIdx.x >> (a.s - a.t);
  const uint64_t j0 = ct << a.t, b0 = bt << a.bc;
  for (uint32_t lin = tid; lin < E; lin += PASS_THREADS) sm[spad(lin)] = a.data[tile_gaddr(a, lin, b0, j0)];
  __syncthreads();
  TileGeom g{a.r, a.t, a.bc};
  tile_dft_fwd(sm, g, a.rp, R, tid, PASS_THREADS);
  const int mlog = a.r + a.s;
  for (uint32_t lin = tid; lin < E; lin += PASS_THREADS) {
    uint64_t v = sm[spad(lin)];
    if (a.s > 0) {
      uint32_t i = (lin >> a.t) & ((1u << a.r) - 1);
      uint64_t jg = j0 + (lin & ((1u << a.t) - 1));
      uint64_t f = row_freq(i, a.r, a.rp);
      uint32_t e = (uint32_t)((f * jg) << (32 - mlog));
      if (e) v = gl::mul(v, rho_pow(R, e));
    }
    a.data[tile_gaddr(a, lin, b0, j0)] = v;
  }
}

// Mirror of k_pass_fwd: incoming twiddle w_M^(-f*j), inverse rounds.
__global__ void __launch_bounds__(PASS_THREADS) k_pass_inv(PassArgs a, Roots R) {
  extern __shared__ uint64_t sm[];
  const int tid = threadIdx.x;
  const uint32_t E = 1u << (a.r + a.t + a.bc);
  const uint64_t ct = blockIdx.x & ((1u << (a.s - a.t)) - 1);
  const uint64_t bt = (uint64_t)blockIdx.x >> (a.s - a.t);
  const uint64_t j0 = ct << a.t, b0 = bt << a.bc;
  const int mlog = a.r + a.s;
  for (uint32_t lin = tid; lin < E; lin += PASS_THREADS) {
    uint64_t v = a.data[tile_gaddr(a, lin, b0, j0)];
    if (a.s > 0) {
      uint32_t i = (lin >> a.t) & ((1u << a.r) - 1);
      uint64_t jg = j0 + (lin & ((1u << a.t) - 1));
      uint64_t f = row_freq(i, a.r, a.rp);
      uint32_t e = (uint32_t)((f * jg) << (32 - mlog));
      if (e) v = gl::mul(v, rho_pow(R, (uint32_t)(0u - e)));
    }
    sm[spad(lin)] = v;
  }
  __syncthreads();
  TileGeom g{a.r, a.t, a.bc};
  tile_dft_inv(sm, g, a.rp, R, tid, PASS_THREADS);
  for (uint32_t lin = tid; lin < E; lin += PASS_THREADS) a.data[tile_gaddr(a, lin, b0, j0)] = sm[spad(lin)];
}

// Limbs -> 16-bit coefficients, zero tail (crates/bignum/src/ntt.rs:640-665).
__global__ void k_pack(const uint64_t* __restrict__ limbs, uint64_t nl, uint64_t* __restrict__ c, uint64_t n) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (; i < n / 4; i += stride) {
    uint64_t l = i < nl ? limbs[i] : 0;
    ulonglong2 lo = make_ulonglong2(l & 0xFFFF, (l >> 16) & 0xFFFF);
    ulonglong2 hi = make_ulonglong2((l >> 32) & 0xFFFF, l >> 48);
    reinterpret_cast<ulonglong2*>(c)[2 * i] = lo;
    reinterpret_cast<ulonglong2*>(c)[2 * i + 1] = hi;
  }
}

// Pointwise a <- a * b * n^-1 (the inverse's 1/N folded in).
__global__ void k_pointwise(uint64_t* __restrict__ a, const uint64_t* __restrict__ b, uint64_t n, uint64_t ninv) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (; i < n; i += stride) a[i] = gl::mul(gl::mul(a[i], b[i]), ninv);
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

__device__ __forceinline__ Win window_value(const uint64_t* c) {
  Win r;
  unsigned __int128 acc = 0;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const ulonglong2* p = reinterpret_cast<const ulonglong2*>(c + 4 * k);
    ulonglong2 x = p[0], y = p[1];
    acc += (unsigned __int128)x.x;
    acc += (unsigned __int128)x.y << 16;
    acc += (unsigned __int128)y.x << 32;
    acc += (unsigned __int128)y.y << 48;
    r.l[k] = (uint64_t)acc;
    acc >>= 64;
  }
  r.hi = (uint64_t)acc;
  return r;
}

constexpr int CARRY_THREADS = 256;  // windows per CTA

// Pass 1: per window s_w (stored as output limbs), flags; per warp the
// (A, B) masks; per CTA the chunk's (generate, propagate) pair.
__global__ void __launch_bounds__(CARRY_THREADS)
k_carry_local(const uint64_t* __restrict__ coef, uint64_t nwin, uint64_t* __restrict__ out, uint64_t nlimbs,
              uint32_t* __restrict__ masks, uint8_t* __restrict__ chunk_gp) {
  __shared__ uint32_t sA[CARRY_THREADS / 32], sB[CARRY_THREADS / 32];
  const uint64_t w = (uint64_t)blockIdx.x * CARRY_THREADS + threadIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  Win v{{0, 0, 0, 0}, 0};
  if (w < nwin) v = window_value(coef + 16 * w);
  uint64_t hprev = __shfl_up_sync(0xFFFFFFFFu, v.hi, 1);
  if (lane == 0) hprev = (w > 0 && w - 1 < nwin) ? window_value(coef + 16 * (w - 1)).hi : 0;
  // s = lo + hprev
  uint64_t s0 = v.l[0] + hprev;
  uint64_t c = s0 < hprev;
  uint64_t s1 = v.l[1] + c;  c = c && s1 == 0;
  uint64_t s2 = v.l[2] + c;  c = c && s2 == 0;
  uint64_t s3 = v.l[3] + c;  c = c && s3 == 0;
  bool g = c != 0 && w < nwin;
  bool p = w < nwin && (s0 & s1 & s2 & s3) == ~0ull;
  if (w < nwin) {
    uint64_t base = 4 * w;
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
    // chunk generate: carry out with cin = 0; propagate: carry out with cin = 1
    uint32_t cg = 0, cp = 1;
    for (int k = 0; k < CARRY_THREADS / 32; k++) {
      uint64_t sg = (uint64_t)sA[k] + sB[k] + cg;
      uint64_t sp = (uint64_t)sA[k] + sB[k] + cp;
      cg = (uint32_t)(sg >> 32);
      cp = (uint32_t)(sp >> 32);
    }
    chunk_gp[blockIdx.x] = (uint8_t)(cg | (cp << 1));
  }
}

// Pass 2: carry into every chunk.  One CTA; each thread walks a contiguous
// segment of chunks, the segment results are chained by thread 0.
constexpr int SCAN_THREADS = 1024;
__global__ void __launch_bounds__(SCAN_THREADS)
k_carry_scan(const uint8_t* __restrict__ chunk_gp, uint64_t nchunk, uint8_t* __restrict__ chunk_cin) {
  __shared__ uint8_t seg_g[SCAN_THREADS], seg_p[SCAN_THREADS], seg_cin[SCAN_THREADS];
  const uint64_t per = (nchunk + SCAN_THREADS - 1) / SCAN_THREADS;
  const uint64_t lo = threadIdx.x * per, hi = lo + per < nchunk ? lo + per : nchunk;
  uint8_t cg = 0, cp = 1;  // carry out for cin = 0 / cin = 1
  for (uint64_t k = lo; k < hi; k++) {
    uint8_t gp = chunk_gp[k];
    uint8_t g0 = gp & 1, g1 = (gp >> 1) & 1;
    cg = cg ? g1 : g0;
    cp = cp ? g1 : g0;
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

// Pass 3: add the incoming carry to every window that receives one.
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
  RoundPlan rp = round_plan(L);
  tile_dft_fwd(smA, g, rp, R, tid, SMALL_THREADS);
  if (!square) tile_dft_fwd(smB, g, rp, R, tid, SMALL_THREADS);
  // n^-1 = (p+1)/2 raised to L, i.e. 2^(-L) = 2^(192-L)
  for (uint32_t i = tid; i < N; i += SMALL_THREADS) {
    uint64_t x = smA[spad(i)];
    uint64_t y = square ? x : smB[spad(i)];
    smA[spad(i)] = gl::shl(gl::mul(x, y), 192 - L);
  }
  __syncthreads();
  tile_dft_inv(smA, g, rp, R, tid, SMALL_THREADS);
  // carry: windows of 16 coefficients, one per thread (N/16 <= 256)
  const uint32_t nwin = (n_out + 15) / 16, nl = la + lb;
  uint64_t* sH = smB;  // reuse: B no longer needed
  __shared__ uint32_t sA[SMALL_THREADS / 32], sBm[SMALL_THREADS / 32];
  Win v{{0, 0, 0, 0}, 0};
  const uint32_t w = tid;
  if (w < nwin) {
    unsigned __int128 acc = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
#pragma unroll
      for (int q = 0; q < 4; q++) {
        uint32_t idx = 16 * w + 4 * k + q;
        uint64_t cv = idx < N ? smA[spad(idx)] : 0;
        acc += (unsigned __int128)cv << (16 * q);
      }
      v.l[k] = (uint64_t)acc;
      acc >>= 64;
    }
    v.hi = (uint64_t)acc;
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
struct DeviceState {
  int device = -1;
  bool ready = false;
  uint64_t* d_lo = nullptr;
  uint64_t* d_hi = nullptr;
  uint64_t* d_w12 = nullptr;
  Roots roots{};
  cudaMemPool_t pool = nullptr;
};

static std::mutex g_mu;
static DeviceState g_dev;
static thread_local cudaStream_t t_stream = nullptr;
static thread_local int t_stream_dev = -1;

static int ensure_init(int device) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (g_dev.ready) {
    if (device >= 0 && device != g_dev.device)
      return fail(PIMUL_EINVAL, "pimul already initialised on another device");
    return PIMUL_OK;
  }
  if (device < 0) device = 0;
  CU(cudaSetDevice(device));
  uint64_t rho = find_rho();
  if (!rho) return fail(PIMUL_ECUDA, "root-of-unity search failed");
  std::vector<uint64_t> lo(1 << 16), hi(1 << 16), w12(4096);
  // powers by repeated multiplication; tables are exact field values
  uint64_t x = 1;
  for (int i = 0; i < (1 << 16); i++) { lo[i] = x; x = hf::mul(x, rho); }
  uint64_t step = x;  // rho^(2^16)
  x = 1;
  for (int i = 0; i < (1 << 16); i++) { hi[i] = x; x = hf::mul(x, step); }
  uint64_t w4096 = hf::pow(rho, 1ull << 20);
  x = 1;
  for (int i = 0; i < 4096; i++) { w12[i] = x; x = hf::mul(x, w4096); }
  CU(cudaMalloc(&g_dev.d_lo, lo.size() * 8));
  CU(cudaMalloc(&g_dev.d_hi, hi.size() * 8));
  CU(cudaMalloc(&g_dev.d_w12, w12.size() * 8));
  CU(cudaMemcpy(g_dev.d_lo, lo.data(), lo.size() * 8, cudaMemcpyHostToDevice));
  CU(cudaMemcpy(g_dev.d_hi, hi.data(), hi.size() * 8, cudaMemcpyHostToDevice));
  CU(cudaMemcpy(g_dev.d_w12, w12.data(), w12.size() * 8, cudaMemcpyHostToDevice));
  g_dev.roots = Roots{g_dev.d_lo, g_dev.d_hi, g_dev.d_w12};
  CU(cudaDeviceGetDefaultMemPool(&g_dev.pool, device));
  uint64_t thr = UINT64_MAX;  // keep freed blocks cached in the pool
  CU(cudaMemPoolSetAttribute(g_dev.pool, cudaMemPoolAttrReleaseThreshold, &thr));
  int smem_max = 0;
  CU(cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, device));
  size_t pass_smem = pass_smem_bytes(TILE_LOG_MAX);
  size_t small_smem = small_smem_bytes(SMALL_LOG_MAX);
  CU(cudaFuncSetAttribute(k_pass_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pass_smem));
  CU(cudaFuncSetAttribute(k_pass_inv, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pass_smem));
  CU(cudaFuncSetAttribute(k_small_mul, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)small_smem));
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

static int log2_ceil(uint64_t x) {
  int L = 0;
  while ((1ull << L) < x) L++;
  return L;
}

// Split L bits into HBM passes of at most 9 bits.
struct Plan {
  int L;
  int np;
  int r[5];
};

static Plan make_plan(int L) {
  Plan p{L, 0, {0, 0, 0, 0, 0}};
  int np = (L + 8) / 9;
  if (np < 1) np = 1;
  int base = L / np, extra = L % np;
  for (int i = 0; i < np; i++) p.r[i] = base + (i < extra ? 1 : 0);
  p.np = np;
  return p;
}

static PassArgs pass_args(uint64_t* data, const Plan& pl, int p) {
  PassArgs a;
  a.data = data;
  a.L = pl.L;
  a.r = pl.r[p];
  int consumed = 0;
  for (int q = 0; q <= p; q++) consumed += pl.r[q];
  a.s = pl.L - consumed;
  a.t = a.s < 4 ? a.s : 4;
  int bc = TILE_LOG_MAX - a.r - a.t;
  int nblocks_log = pl.L - (a.r + a.s);
  if (bc > nblocks_log) bc = nblocks_log;
  if (bc < 0) bc = 0;
  a.bc = bc;
  a.rp = round_plan(a.r);
  return a;
}

static void launch_pass(const PassArgs& a, bool inverse, const Roots& R, cudaStream_t st) {
  uint64_t tiles = 1ull << (a.L - (a.r + a.t + a.bc));
  size_t smem = pass_smem_bytes(a.r + a.t + a.bc);
  KTimer kt(inverse ? K_PASS_INV : K_PASS_FWD, st);
  if (inverse) k_pass_inv<<<(unsigned)tiles, PASS_THREADS, smem, st>>>(a, R);
  else k_pass_fwd<<<(unsigned)tiles, PASS_THREADS, smem, st>>>(a, R);
}

static void transform(uint64_t* data, const Plan& pl, bool inverse, const Roots& R, cudaStream_t st) {
  if (!inverse) {
    for (int p = 0; p < pl.np; p++) launch_pass(pass_args(data, pl, p), false, R, st);
  } else {
    for (int p = pl.np - 1; p >= 0; p--) launch_pass(pass_args(data, pl, p), true, R, st);
  }
}

static unsigned grid_for(uint64_t n, int threads) {
  uint64_t b = (n + threads - 1) / threads;
  uint64_t cap = 152ull * 16;
  return (unsigned)(b < cap ? (b ? b : 1) : cap);
}

// Device multiply: d_out[0 .. la+lb) = a * b.
static int mul_device(const uint64_t* d_a, uint64_t la, const uint64_t* d_b, uint64_t lb, uint64_t* d_out,
                      cudaStream_t st) {
  if (la == 0 || lb == 0) return PIMUL_OK;
  const uint64_t n_out = 4 * la + 4 * lb - 1;
  const int L = log2_ceil(n_out);
  if (L > 32) return fail(PIMUL_EINVAL, "transform length above 2^32");
  const Roots& R = g_dev.roots;
  const bool square = d_a == d_b && la == lb;
  if (L <= SMALL_LOG_MAX) {
    SmallJob job{d_a, d_b, d_out, (uint32_t)la, (uint32_t)lb};
    size_t smem = small_smem_bytes(L);
    {
      KTimer kt(K_SMALL, st);
      k_small_mul<<<1, SMALL_THREADS, smem, st>>>(job, R);
    }
    CU(cudaGetLastError());
    return PIMUL_OK;
  }
  const uint64_t N = 1ull << L;
  const Plan pl = make_plan(L);
  const uint64_t nwin = (n_out + 15) / 16;
  const uint64_t nchunk = (nwin + CARRY_THREADS - 1) / CARRY_THREADS;
  const uint64_t nwarp = nchunk * (CARRY_THREADS / 32);
  uint64_t *A = nullptr, *B = nullptr;
  uint8_t* aux = nullptr;
  size_t aux_bytes = nwarp * 8 + nchunk * 2 + 64;
  CU(cudaMallocAsync((void**)&A, N * 8, g_dev.pool, st));
  if (!square) {
    cudaError_t e = cudaMallocAsync((void**)&B, N * 8, g_dev.pool, st);
    if (e != cudaSuccess) {
      cudaFreeAsync(A, st);
      return fail(PIMUL_ENOMEM, std::string("scratch allocation: ") + cudaGetErrorString(e));
    }
  }
  {
    cudaError_t e = cudaMallocAsync((void**)&aux, aux_bytes, g_dev.pool, st);
    if (e != cudaSuccess) {
      cudaFreeAsync(A, st);
      if (B) cudaFreeAsync(B, st);
      return fail(PIMUL_ENOMEM, std::string("scratch allocation: ") + cudaGetErrorString(e));
    }
  }
  {
    KTimer kt(K_PACK, st);
    k_pack<<<grid_for(N / 4, 256), 256, 0, st>>>(d_a, la, A, N);
  }
  transform(A, pl, false, R, st);
  if (!square) {
    {
      KTimer kt(K_PACK, st);
      k_pack<<<grid_for(N / 4, 256), 256, 0, st>>>(d_b, lb, B, N);
    }
    transform(B, pl, false, R, st);
  }
  uint64_t ninv = hf::pow(hf::pow(2, 191), L);  // 2^-L = (2^191)^L since 2^192 = 1
  {
    KTimer kt(K_POINTWISE, st);
    k_pointwise<<<grid_for(N, 256), 256, 0, st>>>(A, square ? A : B, N, ninv);
  }
  transform(A, pl, true, R, st);
  uint32_t* masks = reinterpret_cast<uint32_t*>(aux);
  uint8_t* chunk_gp = aux + nwarp * 8;
  uint8_t* chunk_cin = chunk_gp + nchunk;
  const uint64_t nlimbs = la + lb;
  {
    KTimer kt(K_CARRY, st);
    k_carry_local<<<(unsigned)nchunk, CARRY_THREADS, 0, st>>>(A, nwin, d_out, nlimbs, masks, chunk_gp);
    k_carry_scan<<<1, SCAN_THREADS, 0, st>>>(chunk_gp, nchunk, chunk_cin);
    k_carry_apply<<<(unsigned)nchunk, CARRY_THREADS, 0, st>>>(nwin, d_out, nlimbs, masks, chunk_cin);
  }
  g_launch[K_CARRY].fetch_add(2, std::memory_order_relaxed);
  cudaError_t le = cudaGetLastError();
  cudaFreeAsync(A, st);
  if (B) cudaFreeAsync(B, st);
  cudaFreeAsync(aux, st);
  if (le != cudaSuccess) return fail(PIMUL_ECUDA, std::string("kernel launch: ") + cudaGetErrorString(le));
  return PIMUL_OK;
}

}  // namespace pimul

// ====================================================================== C ABI
using namespace pimul;

extern "C" {

const char* pimul_version(void) { return "pimul 0.1 (sm_103a)"; }

const char* pimul_last_error(void) { return t_err.c_str(); }

int pimul_init(int device) { return ensure_init(device); }

int pimul_shutdown(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_dev.ready) return PIMUL_OK;
  cudaSetDevice(g_dev.device);
  cudaDeviceSynchronize();
  cudaFree(g_dev.d_lo);
  cudaFree(g_dev.d_hi);
  cudaFree(g_dev.d_w12);
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
  CU(cudaMallocAsync((void**)&da, la * 8, g_dev.pool, st));
  if (!square) {
    cudaError_t e = cudaMallocAsync((void**)&db, lb * 8, g_dev.pool, st);
    if (e != cudaSuccess) { cudaFreeAsync(da, st); return fail(PIMUL_ENOMEM, "input allocation failed"); }
  }
  {
    cudaError_t e = cudaMallocAsync((void**)&dout, (la + lb) * 8, g_dev.pool, st);
    if (e != cudaSuccess) {
      cudaFreeAsync(da, st);
      if (db) cudaFreeAsync(db, st);
      return fail(PIMUL_ENOMEM, "output allocation failed");
    }
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
//    scan's flags: la + lb <= 262144 limbs (transform length N <= 2^20);
//    larger products are rejected with PIMUL_EINVAL.  The array (16 MiB
//    plus 1 MiB of root tables) stays resident on every GPU that loads this
//    library, until the process exits.
//  * every call uses the same array, and the array keeps the previous call's
//    contents; the kernels overwrite every scratch word before reading it,
//    so nothing needs clearing.  Calls whose work overlaps on the GPU
//    (different streams, or different host threads without ordering) race
//    on the array and corrupt each other's results: serialise them.
//  * the first call on each device does a one-time set-up with that device
//    current: it resolves the arrays' device addresses with
//    cudaGetSymbolAddress and copies the root tables in with a synchronous
//    cudaMemcpyToSymbol.  Make that first call before any stream capture.
constexpr int NOALLOC_LOG_MAX = 20;
constexpr uint64_t NOALLOC_N_MAX = 1ull << NOALLOC_LOG_MAX;
constexpr uint64_t NOALLOC_WIN_MAX = NOALLOC_N_MAX / 16;
constexpr uint64_t NOALLOC_CHUNK_MAX = (NOALLOC_WIN_MAX + CARRY_THREADS - 1) / CARRY_THREADS;
constexpr uint64_t NOALLOC_AUX_WORDS = (NOALLOC_CHUNK_MAX * (CARRY_THREADS / 32) * 8 + 2 * NOALLOC_CHUNK_MAX + 64) / 8 + 1;
constexpr size_t NOALLOC_ROOT_WORDS = 2 * 65536 + 4096;

static __device__ __align__(256) uint64_t g_noalloc_scratch[2 * NOALLOC_N_MAX + NOALLOC_AUX_WORDS];
static __device__ __align__(256) uint64_t g_noalloc_roots[NOALLOC_ROOT_WORDS];

struct NoAllocDev {
  bool ready = false;
  uint64_t* scratch = nullptr;  // device address of g_noalloc_scratch on this device
  Roots roots{};
};
static std::mutex g_na_mu;
static NoAllocDev g_na[64];
static uint64_t g_na_host_roots[NOALLOC_ROOT_WORDS];  // staging, no heap use

static int noalloc_setup(NoAllocDev** out) {
  int dev = 0;
  CU(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(PIMUL_EINVAL, "device index out of range");
  std::lock_guard<std::mutex> lk(g_na_mu);
  NoAllocDev& d = g_na[dev];
  if (!d.ready) {
    uint64_t rho = find_rho();
    if (!rho) return fail(PIMUL_ECUDA, "root-of-unity search failed");
    uint64_t* lo = g_na_host_roots;
    uint64_t* hi = lo + 65536;
    uint64_t* w12 = hi + 65536;
    uint64_t x = 1;
    for (int i = 0; i < 65536; i++) { lo[i] = x; x = hf::mul(x, rho); }
    uint64_t step = x;
    x = 1;
    for (int i = 0; i < 65536; i++) { hi[i] = x; x = hf::mul(x, step); }
    uint64_t w4096 = hf::pow(rho, 1ull << 20);
    x = 1;
    for (int i = 0; i < 4096; i++) { w12[i] = x; x = hf::mul(x, w4096); }
    uint64_t* scratch = nullptr;
    uint64_t* roots = nullptr;
    cudaError_t e = cudaGetSymbolAddress((void**)&scratch, g_noalloc_scratch);
    if (e != cudaSuccess) return fail(PIMUL_ECUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
    e = cudaGetSymbolAddress((void**)&roots, g_noalloc_roots);
    if (e != cudaSuccess) return fail(PIMUL_ECUDA, std::string("cudaGetSymbolAddress(roots): ") + cudaGetErrorString(e));
    CU(cudaMemcpyToSymbol(g_noalloc_roots, g_na_host_roots, sizeof(g_na_host_roots)));
    CU(cudaFuncSetAttribute(k_pass_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pass_smem_bytes(TILE_LOG_MAX)));
    CU(cudaFuncSetAttribute(k_pass_inv, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pass_smem_bytes(TILE_LOG_MAX)));
    CU(cudaFuncSetAttribute(k_small_mul, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)small_smem_bytes(SMALL_LOG_MAX)));
    d.scratch = scratch;
    d.roots = Roots{roots, roots + 65536, roots + 2 * 65536};
    d.ready = true;
  }
  *out = &d;
  return PIMUL_OK;
}

// A pass launch without the statistics hook (whose event timing would
// create CUDA events).
static void noalloc_pass(const PassArgs& a, bool inverse, const Roots& R, cudaStream_t st) {
  uint64_t tiles = 1ull << (a.L - (a.r + a.t + a.bc));
  size_t smem = pass_smem_bytes(a.r + a.t + a.bc);
  if (inverse) k_pass_inv<<<(unsigned)tiles, PASS_THREADS, smem, st>>>(a, R);
  else k_pass_fwd<<<(unsigned)tiles, PASS_THREADS, smem, st>>>(a, R);
}

static int mul_device_noalloc(const uint64_t* d_a, uint64_t la, const uint64_t* d_b, uint64_t lb, uint64_t* d_out,
                              cudaStream_t st) {
  NoAllocDev* nd = nullptr;
  int rc = noalloc_setup(&nd);
  if (rc) return rc;
  const uint64_t n_out = 4 * la + 4 * lb - 1;
  const int L = log2_ceil(n_out);
  const Roots& R = nd->roots;
  const bool square = d_a == d_b && la == lb;
  if (L <= SMALL_LOG_MAX) {  // whole product in one CTA's shared memory: no scratch
    SmallJob job{d_a, d_b, d_out, (uint32_t)la, (uint32_t)lb};
    k_small_mul<<<1, SMALL_THREADS, small_smem_bytes(L), st>>>(job, R);
    CU(cudaGetLastError());
    return PIMUL_OK;
  }
  const uint64_t N = 1ull << L;
  const Plan pl = make_plan(L);
  const uint64_t nwin = (n_out + 15) / 16;
  const uint64_t nchunk = (nwin + CARRY_THREADS - 1) / CARRY_THREADS;
  const uint64_t nwarp = nchunk * (CARRY_THREADS / 32);
  uint64_t* A = nd->scratch;
  uint64_t* B = nd->scratch + NOALLOC_N_MAX;
  uint8_t* aux = reinterpret_cast<uint8_t*>(nd->scratch + 2 * NOALLOC_N_MAX);
  k_pack<<<grid_for(N / 4, 256), 256, 0, st>>>(d_a, la, A, N);
  for (int p = 0; p < pl.np; p++) noalloc_pass(pass_args(A, pl, p), false, R, st);
  if (!square) {
    k_pack<<<grid_for(N / 4, 256), 256, 0, st>>>(d_b, lb, B, N);
    for (int p = 0; p < pl.np; p++) noalloc_pass(pass_args(B, pl, p), false, R, st);
  }
  uint64_t ninv = hf::pow(hf::pow(2, 191), L);
  k_pointwise<<<grid_for(N, 256), 256, 0, st>>>(A, square ? A : B, N, ninv);
  for (int p = pl.np - 1; p >= 0; p--) noalloc_pass(pass_args(A, pl, p), true, R, st);
  uint32_t* masks = reinterpret_cast<uint32_t*>(aux);
  uint8_t* chunk_gp = aux + nwarp * 8;
  uint8_t* chunk_cin = chunk_gp + nchunk;
  const uint64_t nlimbs = la + lb;
  k_carry_local<<<(unsigned)nchunk, CARRY_THREADS, 0, st>>>(A, nwin, d_out, nlimbs, masks, chunk_gp);
  k_carry_scan<<<1, SCAN_THREADS, 0, st>>>(chunk_gp, nchunk, chunk_cin);
  k_carry_apply<<<(unsigned)nchunk, CARRY_THREADS, 0, st>>>(nwin, d_out, nlimbs, masks, chunk_cin);
  CU(cudaGetLastError());
  return PIMUL_OK;
}

extern "C" int pimul_mul_device_noalloc(const uint64_t* d_a, size_t la, const uint64_t* d_b, size_t lb,
                                        uint64_t* d_out, void* stream) {
  if (la == 0 || lb == 0) return PIMUL_OK;
  if (!d_a || !d_b || !d_out) return fail(PIMUL_EINVAL, "null device pointer");
  if (la + lb > NOALLOC_N_MAX / 4)
    return fail(PIMUL_EINVAL, "product too large for the no-alloc scratch: la + lb must be <= 262144 limbs "
                              "(transform length <= 2^20)");
  return mul_device_noalloc(d_a, la, d_b, lb, d_out, (cudaStream_t)stream);
}
