// Binary-splitting leaves on the device.
//
// P, Q, T of short runs of consecutive Chudnovsky terms
// (crates/pi-core/src/algorithm/chudnovsky.rs:377-413), one warp per run:
//   p_k = -(6k-5)(2k-1)(6k-1),  q_k = (C^3/24) k^3,  t_k = p_k (A + B k)
// then the run's terms merged pairwise level by level,
//   P = P_L P_R,  Q = Q_L Q_R,  T = T_L Q_R + P_L T_R,
// with every level in the warp's shared memory.  Magnitudes are stored and
// the signs are the static ones of the splitting (P of m terms has sign
// (-1)^m, every T < 0), so |T| = |T_L| Q_R + (-1)^(m_L) |P_L| |T_R|; a
// merge whose |T| would come out negative is reported (the caller then
// takes the host path).  A product is computed by a group of lanes, each
// owning a run of output columns: 192-bit signed column sums (T's two
// products go into the same sums), the carries propagated along the lane's
// run and then from lane to lane.  An integer result is unique, so the
// values are those of the host's leaf path.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <vector>

#include "../../include/pimul.h"
#include "leaves.h"

namespace pileaf {
namespace {

constexpr uint64_t CH_A = 13591409, CH_B = 545140134;  // chudnovsky.rs:57-58
constexpr uint64_t C3_OVER_24 = 10939058860032000ull;  // chudnovsky.rs:61
constexpr int LW_WARPS = 4;                            // leaves (warps) per CTA

// Fixed slots of a level whose nodes hold at most m terms (k < 2^31):
// |p_k| < 2^100, q_k < 2^147, |t_k| < 2^161, so |P| < 2^(100 m) fits 2m
// limbs, Q 3m, and |T| < m 2^(146.3 (m - 1) + 161) fits 3m + 2 limbs; the
// T slot holds 3m + 3, the untrimmed length of the merge that makes it.
__device__ __forceinline__ uint32_t slot_words(uint32_t m) { return 8 * m + 3; }
__device__ __forceinline__ uint32_t q_at(uint32_t m) { return 2 * m; }
__device__ __forceinline__ uint32_t t_at(uint32_t m) { return 5 * m; }
constexpr uint32_t LEVEL_WORDS = 11 * MAX_TERMS;  // the largest level: MAX_TERMS single terms

struct Lens {
  uint16_t p, q, t;
};

// z[0..nz) = x1 y1 + (sub ? -1 : +1) x2 y2 (x2 == nullptr: x1 y1 only), with
// nz = x1y1's untrimmed length, plus one limb for a sum of two, by the G
// lanes of a group (gl = lane in the group, gmask = the group's lanes).
// Returns the trimmed length to every lane of the group; *bad = 1 (and
// nothing written) if nz > cap, and *bad = 1 if the result is negative.
__device__ uint32_t grp_mul(const uint64_t* x1, uint32_t nx1, const uint64_t* y1, uint32_t ny1, const uint64_t* x2,
                            uint32_t nx2, const uint64_t* y2, uint32_t ny2, bool sub, uint64_t* z, uint32_t cap,
                            uint32_t gl, uint32_t G, unsigned gmask, uint32_t src0, int* bad) {
  const uint32_t n1 = (nx1 && ny1) ? nx1 + ny1 : 0;
  const uint32_t n2 = (x2 && nx2 && ny2) ? nx2 + ny2 : 0;
  const uint32_t nz = n2 ? max(n1, n2) + 1 : n1;
  if (nz > cap) {
    if (gl == 0) *bad = 1;
    return 0;
  }
  const uint32_t c = (nz + G - 1) / G;
  const uint32_t k0 = min(nz, gl * c), k1 = min(nz, k0 + c);
  __int128 carry = 0;  // signed carry into column k, in units of 2^(64 k)
  for (uint32_t k = k0; k < k1; k++) {
    uint64_t lo = 0;
    __int128 hi = 0;  // the column sum is lo + hi 2^64
    if (n1) {
      const uint32_t i0 = k + 1 > ny1 ? k + 1 - ny1 : 0, i1 = min(k, nx1 - 1);
      for (uint32_t i = i0; i <= i1; i++) {
        const unsigned __int128 pr = (unsigned __int128)x1[i] * y1[k - i];
        const uint64_t plo = (uint64_t)pr;
        lo += plo;
        hi += (__int128)(pr >> 64) + (lo < plo ? 1 : 0);
      }
    }
    if (n2) {
      const uint32_t i0 = k + 1 > ny2 ? k + 1 - ny2 : 0, i1 = min(k, nx2 - 1);
      for (uint32_t i = i0; i <= i1; i++) {
        const unsigned __int128 pr = (unsigned __int128)x2[i] * y2[k - i];
        const uint64_t plo = (uint64_t)pr;
        if (sub) {
          hi -= (__int128)(pr >> 64) + (lo < plo ? 1 : 0);
          lo -= plo;
        } else {
          lo += plo;
          hi += (__int128)(pr >> 64) + (lo < plo ? 1 : 0);
        }
      }
    }
    const uint64_t clo = (uint64_t)carry;
    const uint64_t nlo = lo + clo;
    carry = hi + (carry >> 64) + (nlo < clo ? 1 : 0);
    z[k] = nlo;
  }
  // carries from lane to lane: lane s adds the final carry out of lane s - 1
  for (uint32_t s = 1; s < G; s++) {
    const uint64_t vlo = __shfl_sync(gmask, (uint64_t)carry, src0 + s - 1);
    const uint64_t vhi = __shfl_sync(gmask, (uint64_t)((unsigned __int128)carry >> 64), src0 + s - 1);
    if (gl == s) {
      __int128 v = (__int128)(((unsigned __int128)vhi << 64) | vlo);
      for (uint32_t k = k0; k < k1 && v != 0; k++) {
        const uint64_t wlo = (uint64_t)v;
        const uint64_t nlo = z[k] + wlo;
        v = (v >> 64) + (nlo < wlo ? 1 : 0);
        z[k] = nlo;
      }
      carry += v;
    }
  }
  // the carry out of the top column must vanish (a negative |T| shows here)
  if (gl == G - 1 && carry != 0) *bad = 1;
  __syncwarp(gmask);
  uint32_t top = 0;
  for (uint32_t k = k0; k < k1; k++)
    if (z[k]) top = k + 1;
  for (uint32_t o = 1; o < G; o <<= 1) top = max(top, __shfl_xor_sync(gmask, top, o));
  return top;
}

// p_k, q_k, t_k (magnitudes) into the term slot at z (P at 0, Q at 2, T at 5).
__device__ Lens term_values(uint64_t k, uint64_t* z) {
  const unsigned __int128 f = (unsigned __int128)(6 * k - 5) * (2 * k - 1);
  const unsigned __int128 p = f * (6 * k - 1);  // < 2^100
  const unsigned __int128 k2 = (unsigned __int128)k * k;
  const unsigned __int128 k3 = k2 * k;  // < 2^93
  // q = C^3/24 k^3 and t = p (A + B k): 128 x 64 -> 192 bits
  auto mul192 = [](unsigned __int128 a, uint64_t b, uint64_t* out) {
    const unsigned __int128 lo = (unsigned __int128)(uint64_t)a * b;
    const unsigned __int128 hi = (unsigned __int128)(uint64_t)(a >> 64) * b + (lo >> 64);
    out[0] = (uint64_t)lo;
    out[1] = (uint64_t)hi;
    out[2] = (uint64_t)(hi >> 64);
  };
  Lens L;
  z[0] = (uint64_t)p;
  z[1] = (uint64_t)(p >> 64);
  L.p = z[1] ? 2 : 1;
  mul192(k3, C3_OVER_24, z + 2);
  L.q = z[4] ? 3 : (z[3] ? 2 : 1);
  mul192(p, CH_A + CH_B * k, z + 5);
  L.t = z[7] ? 3 : (z[6] ? 2 : 1);
  return L;
}

// One warp per leaf; *bad = 1 when a value breaks the static signs or
// outgrows its slot (nothing past a slot is written).
__global__ void __launch_bounds__(32 * LW_WARPS) k_leaves(uint64_t a0, uint64_t b, uint32_t m, uint32_t nleaf,
                                                         uint64_t* out, uint32_t sp, uint32_t sq, uint32_t st,
                                                         uint32_t* lens, uint8_t* signs, int* bad) {
  __shared__ uint64_t s_buf[LW_WARPS][2][LEVEL_WORDS];
  __shared__ Lens s_len[LW_WARPS][2][MAX_TERMS];
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t leaf = blockIdx.x * LW_WARPS + warp;
  if (leaf >= nleaf) return;
  const uint64_t ka = a0 + (uint64_t)leaf * m;
  const uint64_t kb = ka + m < b ? ka + m : b;
  uint32_t n = (uint32_t)(kb - ka);
  uint64_t* cur = s_buf[warp][0];
  uint64_t* nxt = s_buf[warp][1];
  Lens* lc = s_len[warp][0];
  Lens* ln = s_len[warp][1];
  for (uint32_t i = lane; i < n; i += 32) lc[i] = term_values(ka + i, cur + i * slot_words(1));
  __syncwarp();
  uint32_t tm = 1;  // terms per full node of the current level
  while (n > 1) {
    const uint32_t np = n / 2, m2 = 2 * tm;
    uint32_t G = 1;
    while (G * 2 * np <= 32) G *= 2;  // lanes per pair
    const uint32_t gi = lane / G, gl = lane % G, src0 = gi * G;
    const unsigned gmask = G == 32 ? 0xFFFFFFFFu : ((1u << G) - 1) << src0;
    const uint32_t si = slot_words(tm), so = slot_words(m2);
    for (uint32_t pr = gi; pr < np; pr += 32 / G) {
      const uint64_t* L = cur + (2 * pr) * si;
      const uint64_t* R = L + si;
      const Lens a = lc[2 * pr], c = lc[2 * pr + 1];
      uint64_t* z = nxt + pr * so;
      Lens zl;
      zl.p = (uint16_t)grp_mul(L, a.p, R, c.p, nullptr, 0, nullptr, 0, false, z, q_at(m2), gl, G, gmask, src0, bad);
      zl.q = (uint16_t)grp_mul(L + q_at(tm), a.q, R + q_at(tm), c.q, nullptr, 0, nullptr, 0, false, z + q_at(m2),
                               t_at(m2) - q_at(m2), gl, G, gmask, src0, bad);
      // |T| = |T_L| Q_R + (-1)^(m_L) |P_L| |T_R|: a left node holds tm terms
      zl.t = (uint16_t)grp_mul(L + t_at(tm), a.t, R + q_at(tm), c.q, L, a.p, R + t_at(tm), c.t, (tm & 1) != 0,
                               z + t_at(m2), slot_words(m2) - t_at(m2), gl, G, gmask, src0, bad);
      if (zl.t > 3 * m2 + 2 && gl == 0) *bad = 1;
      if (gl == 0) ln[pr] = zl;
    }
    if (n & 1) {  // the odd last node moves up unchanged
      const uint64_t* o = cur + (n - 1) * si;
      uint64_t* z = nxt + np * so;
      const Lens a = lc[n - 1];
      for (uint32_t j = lane; j < a.p; j += 32) z[j] = o[j];
      for (uint32_t j = lane; j < a.q; j += 32) z[q_at(m2) + j] = o[q_at(tm) + j];
      for (uint32_t j = lane; j < a.t; j += 32) z[t_at(m2) + j] = o[t_at(tm) + j];
      if (lane == 0) ln[np] = a;
    }
    __syncwarp();
    n = np + (n & 1);
    tm = m2;
    uint64_t* t = cur;
    cur = nxt;
    nxt = t;
    Lens* tl = lc;
    lc = ln;
    ln = tl;
  }
  const Lens r = lc[0];
  if (r.p > sp || r.q > sq || r.t > st) {
    if (lane == 0) *bad = 1;
    return;
  }
  uint64_t* slot = out + (uint64_t)leaf * (sp + sq + st);
  for (uint32_t j = lane; j < r.p; j += 32) slot[j] = cur[j];
  for (uint32_t j = lane; j < r.q; j += 32) slot[sp + j] = cur[q_at(tm) + j];
  for (uint32_t j = lane; j < r.t; j += 32) slot[sp + sq + j] = cur[t_at(tm) + j];
  if (lane == 0) {
    lens[3 * leaf + 0] = r.p;
    lens[3 * leaf + 1] = r.q;
    lens[3 * leaf + 2] = r.t;
    signs[leaf] = (uint8_t)(((kb - ka) & 1 ? 1 : 0) | 2);  // static signs: P ~ (-1)^terms, T < 0
  }
}

}  // namespace

int leaves_device(uint64_t a0, uint64_t b, uint32_t m, uint32_t nleaf, uint32_t sp, uint32_t sq, uint32_t st,
                  uint64_t* d_out, uint32_t* lens, uint8_t* signs, cudaStream_t stream) {
  // the slot bounds of k_leaves hold for terms k < 2^31
  if (!m || m > MAX_TERMS || !d_out || !lens || !signs || a0 < 1 || b > (1ull << 31)) return PIMUL_EINVAL;
  if (!nleaf) return PIMUL_OK;
  if ((uint64_t)nleaf * m < b - a0 || (uint64_t)(nleaf - 1) * m >= b - a0) return PIMUL_EINVAL;
  uint8_t* dev = nullptr;
  const size_t lb = ((size_t)nleaf * 3 * 4 + 255) & ~(size_t)255, sb = ((size_t)nleaf + 255) & ~(size_t)255;
  if (cudaMallocAsync((void**)&dev, lb + sb + 256, stream) != cudaSuccess) {
    cudaGetLastError();
    return PIMUL_ENOMEM;
  }
  uint32_t* d_lens = reinterpret_cast<uint32_t*>(dev);
  uint8_t* d_signs = dev + lb;
  int* d_bad = reinterpret_cast<int*>(dev + lb + sb);
  int rc = PIMUL_OK;
  int h_bad = 0;
  if (cudaMemsetAsync(d_bad, 0, sizeof(int), stream) != cudaSuccess) rc = PIMUL_ECUDA;
  if (!rc) {
    k_leaves<<<(nleaf + LW_WARPS - 1) / LW_WARPS, 32 * LW_WARPS, 0, stream>>>(a0, b, m, nleaf, d_out, sp, sq, st,
                                                                            d_lens, d_signs, d_bad);
    if (cudaGetLastError() != cudaSuccess) rc = PIMUL_ECUDA;
  }
  if (!rc && (cudaMemcpyAsync(lens, d_lens, (size_t)nleaf * 3 * 4, cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
              cudaMemcpyAsync(signs, d_signs, nleaf, cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
              cudaMemcpyAsync(&h_bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
              cudaStreamSynchronize(stream) != cudaSuccess))
    rc = PIMUL_ECUDA;
  cudaFreeAsync(dev, stream);
  if (!rc && h_bad) rc = PIMUL_EINVAL;
  return rc;
}

}  // namespace pileaf
