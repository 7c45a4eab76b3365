// Binary-splitting leaves on the device.
//
// P, Q, T of short runs of consecutive Chudnovsky terms
// (crates/pi-core/src/algorithm/chudnovsky.rs:377-413), one thread per run:
//   p_k = -(6k-5)(2k-1)(6k-1),  q_k = (C^3/24) k^3,  t_k = p_k (A + B k)
// then the run's terms merged pairwise level by level,
//   P = P_L P_R,  Q = Q_L Q_R,  T = T_L Q_R + P_L T_R,
// with schoolbook products on the thread's local buffers (the same
// arithmetic as the host's flat leaf path in pi_host.cpp, and an integer
// result is unique, so the values are the host's).  A level of m terms
// holds about 12 limbs per term, so a 64-term run needs two 960-limb level
// buffers and two product temporaries: about 24 KB of local memory per
// thread, which stays in L1/L2.
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
constexpr uint32_t BUF = 14 * MAX_TERMS + 64;          // limbs of one level
constexpr uint32_t TMP = 8 * MAX_TERMS + 16;           // limbs of one product temporary

struct Node {
  uint16_t po, qo, to;  // offsets of |P|, Q, |T| in the level buffer
  uint16_t pn, qn, tn;  // trimmed lengths
  bool ps, ts;          // P < 0, T < 0
};

__device__ __forceinline__ uint32_t trim(const uint64_t* x, uint32_t n) {
  while (n && x[n - 1] == 0) n--;
  return n;
}

// z[0..nx+ny) = x y (schoolbook); returns the trimmed length.
__device__ uint32_t mulw(const uint64_t* x, uint32_t nx, const uint64_t* y, uint32_t ny, uint64_t* z) {
  if (!nx || !ny) return 0;
  for (uint32_t i = 0; i < nx + ny; i++) z[i] = 0;
  for (uint32_t i = 0; i < nx; i++) {
    const uint64_t xi = x[i];
    uint64_t carry = 0;
    for (uint32_t j = 0; j < ny; j++) {
      const uint64_t lo = xi * y[j];
      uint64_t hi = __umul64hi(xi, y[j]);
      uint64_t s = z[i + j] + lo;
      hi += s < lo;
      s += carry;
      hi += s < carry;  // the 128-bit sum z + x y + carry fits: no overflow of hi
      z[i + j] = s;
      carry = hi;
    }
    z[i + ny] = carry;
  }
  return trim(z, nx + ny);
}

__device__ int cmpw(const uint64_t* x, uint32_t nx, const uint64_t* y, uint32_t ny) {
  if (nx != ny) return nx < ny ? -1 : 1;
  for (uint32_t i = nx; i-- > 0;)
    if (x[i] != y[i]) return x[i] < y[i] ? -1 : 1;
  return 0;
}

// z = (sx ? -|x| : |x|) + (sy ? -|y| : |y|); returns |z|'s length, sign in sz.
__device__ uint32_t add_signed(const uint64_t* x, uint32_t nx, bool sx, const uint64_t* y, uint32_t ny, bool sy,
                               uint64_t* z, bool& sz) {
  if (sx == sy) {
    if (nx < ny) {
      const uint64_t* t = x;
      x = y;
      y = t;
      uint32_t tn = nx;
      nx = ny;
      ny = tn;
    }
    uint64_t c = 0;
    for (uint32_t i = 0; i < nx; i++) {
      const uint64_t yi = i < ny ? y[i] : 0;
      const uint64_t s = x[i] + yi;
      const uint64_t c1 = s < yi;
      z[i] = s + c;
      c = c1 | (z[i] < s);
    }
    z[nx] = c;
    sz = sx;
    return trim(z, nx + 1);
  }
  const int c = cmpw(x, nx, y, ny);
  if (c == 0) {
    sz = false;
    return 0;
  }
  if (c < 0) {
    const uint64_t* t = x;
    x = y;
    y = t;
    uint32_t tn = nx;
    nx = ny;
    ny = tn;
    sx = sy;
  }
  uint64_t borrow = 0;
  for (uint32_t i = 0; i < nx; i++) {
    const uint64_t yi = i < ny ? y[i] : 0;
    const uint64_t d = x[i] - yi - borrow;
    borrow = (x[i] < yi || (x[i] == yi && borrow)) ? 1 : 0;
    z[i] = d;
  }
  sz = sx;
  return trim(z, nx);
}

// *bad = 1 and no further writes when a leaf's buffers or slot are too small.
__global__ void __launch_bounds__(64) k_leaves(uint64_t a0, uint64_t b, uint32_t m, uint32_t nleaf, uint64_t* out,
                                               uint32_t sp, uint32_t sq, uint32_t st, uint32_t* lens,
                                               uint8_t* signs, int* bad) {
  const uint32_t leaf = blockIdx.x * blockDim.x + threadIdx.x;
  if (leaf >= nleaf) return;
  const uint64_t ka = a0 + (uint64_t)leaf * m;
  const uint64_t kb = ka + m < b ? ka + m : b;
  uint32_t n = (uint32_t)(kb - ka);
  uint64_t buf0[BUF], buf1[BUF], tq[TMP], pt[TMP];
  Node nodes[MAX_TERMS], next[MAX_TERMS / 2 + 1];
  uint64_t* cur = buf0;
  uint64_t* nxt = buf1;
  uint32_t off = 0;
  for (uint32_t i = 0; i < n; i++) {
    const uint64_t k = ka + i;
    // p = -(6k-5)(2k-1)(6k-1), q = (C^3/24) k^3, t = p (A + B k)
    const uint64_t f1 = 6 * k - 5, f2 = 2 * k - 1, f3 = 6 * k - 1;
    uint64_t pm[2] = {f1 * f2, __umul64hi(f1, f2)};
    uint64_t p3[3], k2[2] = {k * k, __umul64hi(k, k)}, kk[1] = {k}, k3[3], c3[1] = {C3_OVER_24}, q4[4];
    uint64_t ff[1] = {f3};
    const uint32_t pn = mulw(pm, trim(pm, 2), ff, 1, p3);
    const uint32_t k3n = mulw(k2, trim(k2, 2), kk, 1, k3);
    const uint32_t qn = mulw(k3, k3n, c3, 1, q4);
    uint64_t ab[2];
    ab[0] = CH_B * k;
    ab[1] = __umul64hi(CH_B, k);
    ab[0] += CH_A;
    ab[1] += ab[0] < CH_A;
    uint64_t t5[5];
    const uint32_t tn = mulw(p3, pn, ab, trim(ab, 2), t5);
    Node& nd = nodes[i];
    nd.po = (uint16_t)off, nd.pn = (uint16_t)pn;
    for (uint32_t j = 0; j < pn; j++) cur[off + j] = p3[j];
    off += pn;
    nd.qo = (uint16_t)off, nd.qn = (uint16_t)qn;
    for (uint32_t j = 0; j < qn; j++) cur[off + j] = q4[j];
    off += qn;
    nd.to = (uint16_t)off, nd.tn = (uint16_t)tn;
    for (uint32_t j = 0; j < tn; j++) cur[off + j] = t5[j];
    off += tn;
    nd.ps = true;
    nd.ts = true;
  }
  while (n > 1) {
    const uint32_t np = n / 2;
    uint32_t o = 0;
    for (uint32_t i = 0; i < np; i++) {
      const Node L = nodes[2 * i];
      const Node R = nodes[2 * i + 1];
      Node z;
      if (o + L.pn + R.pn + L.qn + R.qn + (L.tn + R.qn > L.pn + R.tn ? L.tn + R.qn : L.pn + R.tn) + 1 > BUF ||
          L.tn + R.qn > TMP || L.pn + R.tn > TMP) {
        *bad = 1;
        return;
      }
      z.po = (uint16_t)o;
      z.pn = (uint16_t)mulw(cur + L.po, L.pn, cur + R.po, R.pn, nxt + o);
      z.ps = L.ps != R.ps;
      o += z.pn;
      z.qo = (uint16_t)o;
      z.qn = (uint16_t)mulw(cur + L.qo, L.qn, cur + R.qo, R.qn, nxt + o);
      o += z.qn;
      const uint32_t a1 = mulw(cur + L.to, L.tn, cur + R.qo, R.qn, tq);
      const uint32_t a2 = mulw(cur + L.po, L.pn, cur + R.to, R.tn, pt);
      bool zs = false;
      z.to = (uint16_t)o;
      z.tn = (uint16_t)add_signed(tq, a1, L.ts, pt, a2, L.ps != R.ts, nxt + o, zs);
      z.ts = zs;
      o += z.tn;
      next[i] = z;
    }
    if (n & 1) {
      const Node L = nodes[n - 1];
      if (o + L.pn + L.qn + L.tn > BUF) {
        *bad = 1;
        return;
      }
      Node z = L;
      z.po = (uint16_t)o;
      for (uint32_t j = 0; j < L.pn; j++) nxt[o + j] = cur[L.po + j];
      o += L.pn;
      z.qo = (uint16_t)o;
      for (uint32_t j = 0; j < L.qn; j++) nxt[o + j] = cur[L.qo + j];
      o += L.qn;
      z.to = (uint16_t)o;
      for (uint32_t j = 0; j < L.tn; j++) nxt[o + j] = cur[L.to + j];
      o += L.tn;
      next[np] = z;
    }
    n = np + (n & 1);
    for (uint32_t i = 0; i < n; i++) nodes[i] = next[i];
    uint64_t* t = cur;
    cur = nxt;
    nxt = t;
  }
  const Node r = nodes[0];
  if (r.pn > sp || r.qn > sq || r.tn > st) {
    *bad = 1;
    return;
  }
  uint64_t* slot = out + (uint64_t)leaf * (sp + sq + st);
  for (uint32_t j = 0; j < r.pn; j++) slot[j] = cur[r.po + j];
  for (uint32_t j = 0; j < r.qn; j++) slot[sp + j] = cur[r.qo + j];
  for (uint32_t j = 0; j < r.tn; j++) slot[sp + sq + j] = cur[r.to + j];
  lens[3 * leaf + 0] = r.pn;
  lens[3 * leaf + 1] = r.qn;
  lens[3 * leaf + 2] = r.tn;
  signs[leaf] = (uint8_t)((r.ps ? 1 : 0) | (r.ts ? 2 : 0));
}

}  // namespace

int leaves_device(uint64_t a0, uint64_t b, uint32_t m, uint32_t nleaf, uint32_t sp, uint32_t sq, uint32_t st,
                  uint64_t* d_out, uint32_t* lens, uint8_t* signs, cudaStream_t stream) {
  if (!m || m > MAX_TERMS || !d_out || !lens || !signs || a0 < 1) return PIMUL_EINVAL;
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
    k_leaves<<<(nleaf + 63) / 64, 64, 0, stream>>>(a0, b, m, nleaf, d_out, sp, sq, st, d_lens, d_signs, d_bad);
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
