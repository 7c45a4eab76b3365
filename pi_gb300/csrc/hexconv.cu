// Decimal -> hexadecimal conversion of pi's digits with every big step in HBM.
//
// verify-hex's conversion (crates/pi-cli/src/verify_hex.rs:553-629): for the
// text "3.d_1...d_E" (surrounding whitespace trimmed), N = 3 d_1 ... d_E read
// as a D = E + 1 digit integer and h = floor(E log2(10) / 4) (f64, as the
// reference computes it),
//     m = floor(N 16^h / 10^E),
// and the output is "3." followed by m's hex digits after its leading 3, in
// lower case (integer.rs:169-177 prints the top limb unpadded, so m's hex
// string has no leading zeros).  The reference parses N digit by digit
// (integer.rs:127-148, quadratic in D) and divides with its Newton division
// (integer.rs:1004-1083); here:
//   parse   one thread per 19-digit chunk (k_chunks, which also checks the
//           digits), one thread per leaf of 2^LK chunks by Horner's rule
//           (k_parse_leaves), then level by level x = hi P_k + lo with
//           P_k = 10^(19 2^k): all products of a level in one strided
//           batch (P_k is every job's b; the descriptors are written by a
//           kernel) and one strided addition; high nodes made only of the
//           zero chunks above the top digit are not multiplied;
//   divide  10^E = 10^(E mod 19 + 19 (q mod 2^LK)) (host, at most 64 limbs)
//           times P_j for each bit j >= LK of q = E div 19, then the device
//           Newton quotient of Chudnovsky's final assembly
//           (pidec::quotient_device, relative error far below 2^-64 at
//           4h + 64 bits, so its floor is m - 1, m or m + 1), and the exact
//           floor from the remainder N 2^(4h) - m' 10^E taken modulo
//           2^(64 (|10^E| + 1)): after one decrement it lies in [0, 3 10^E),
//           and each of at most three rounds subtracts 10^E and reads one
//           sign bit;
//   print   one thread per hex digit.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/pimul.h"
#include "dec.h"
#include "hostcopy.h"

namespace pihex {
namespace {

constexpr uint64_t CHUNK = 10000000000000000000ull;  // 10^19 (integer.rs:887-888)
constexpr int LK_MAX = 6;                            // leaves of 64 chunks (1216 digits)
constexpr uint32_t LEAF_W_MAX = 64;                  // limbs of 10^1216

double now_ms() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

unsigned grid_for(uint64_t n, unsigned threads) {
  return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((n + threads - 1) / threads, 152ull * 64));
}

// c[i] = the 19 digits ending 19 i digits from the right of the D-digit
// string 3 d_1 ... d_E (digit j is text[0] for j = 0, text[j + 1] after the
// point); chunks above the top digit are 0.  *bad = 1 if a digit character
// is not in '0'..'9'.  text holds D + 1 bytes.
__global__ void k_chunks(const char* __restrict__ text, uint64_t D, uint64_t nch, uint64_t* __restrict__ c,
                         int* __restrict__ bad) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nch; i += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t v = 0;
    if (19 * i < D) {
      const uint64_t hi = D - 19 * i, lo = hi > 19 ? hi - 19 : 0;
      for (uint64_t j = lo; j < hi; j++) {
        const unsigned d = (unsigned)(unsigned char)text[j ? j + 1 : 0] - (unsigned)'0';
        if (d > 9) *bad = 1;
        v = v * 10 + (d > 9 ? 0 : d);
      }
    }
    c[i] = v;
  }
}

// Leaf i = the integer of the 2^lk chunks c[i 2^lk ..) (Horner's rule from
// the top chunk) into out + i w, zero above its top limb.  Every value of
// 2^lk chunks is below 10^(19 2^lk) < 2^(64 w), so w limbs hold it.
__global__ void k_parse_leaves(const uint64_t* __restrict__ c, int lk, uint64_t nleaf, uint32_t w,
                               uint64_t* __restrict__ out) {
  uint64_t acc[LEAF_W_MAX];
  const uint32_t m = 1u << lk;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nleaf;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t* ci = c + i * m;
    uint32_t used = 0;
    for (uint32_t j = m; j-- > 0;) {
      uint64_t carry = ci[j];
      for (uint32_t t = 0; t < used; t++) {
        const uint64_t lo = acc[t] * CHUNK;
        const uint64_t hi = __umul64hi(acc[t], CHUNK);
        const uint64_t s = lo + carry;
        carry = hi + (s < lo);
        acc[t] = s;
      }
      if (carry && used < w) acc[used++] = carry;
    }
    uint64_t* o = out + i * w;
    for (uint32_t t = 0; t < w; t++) o[t] = t < used ? acc[t] : 0;
  }
}

// dst[0..w) = the low w limbs of src[0..n) 2^s.
__global__ void k_shl_low(const uint64_t* __restrict__ src, uint64_t n, uint64_t s, uint64_t* __restrict__ dst,
                          uint64_t w) {
  const int64_t ws = (int64_t)(s >> 6);
  const unsigned bs = (unsigned)(s & 63);
  for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < w; j += (uint64_t)gridDim.x * blockDim.x) {
    const int64_t i = (int64_t)j - ws;
    const uint64_t a = i >= 0 && (uint64_t)i < n ? src[i] : 0;
    const uint64_t b = i >= 1 && (uint64_t)(i - 1) < n ? src[i - 1] : 0;
    dst[j] = bs ? (a << bs) | (b >> (64 - bs)) : a;
  }
}

// out[i] = hex digit h - 1 - i of m (digit t = bits 4t .. 4t + 3), i < h.
__global__ void k_hex_digits(const uint64_t* __restrict__ m, uint64_t h, char* __restrict__ out) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < h; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t t = h - 1 - i;
    const unsigned v = (unsigned)(m[t >> 4] >> (4 * (t & 15))) & 15u;
    out[i] = (char)(v < 10 ? '0' + v : 'a' + (v - 10));
  }
}

// 10^e as host limbs (e small: a few hundred 19-digit steps at most).
std::vector<uint64_t> pow10_host(uint64_t e) {
  std::vector<uint64_t> x{1};
  while (e) {
    const uint64_t k = std::min<uint64_t>(e, 19);
    uint64_t f = 1;
    for (uint64_t i = 0; i < k; i++) f *= 10;
    unsigned __int128 carry = 0;
    for (uint64_t& v : x) {
      carry += (unsigned __int128)v * f;
      v = (uint64_t)carry;
      carry >>= 64;
    }
    if (carry) x.push_back((uint64_t)carry);
    e -= k;
  }
  return x;
}

bool is_space(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\v' || c == '\f'; }

// Device allocations on one stream, freed (stream-ordered) at scope exit.
struct Scope {
  cudaStream_t st = nullptr;
  std::vector<void*> live;
  ~Scope() {
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
      return pimul::set_error(PIMUL_ENOMEM, "decimal to hex: device allocation failed");
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
}  // namespace pihex

extern "C" int pimul_decimal_to_hex(const char* text, size_t len, char* out, size_t cap, size_t* out_len,
                                    double* phase_ms) {
  using namespace pihex;
  using pimul::set_error;
  if (!out_len || (len && !text)) return set_error(PIMUL_EINVAL, "decimal to hex: null argument");
  size_t b = 0, e = len;
  while (b < e && is_space(text[b])) b++;
  while (e > b && is_space(text[e - 1])) e--;
  const char* s = text + b;
  const size_t n = e - b;
  if (n < 2 || s[0] != '3' || s[1] != '.') return set_error(PIMUL_EINVAL, "the decimal text doesn't start with \"3.\"");
  const uint64_t E = n - 2;
  if (E > 0xFFFFFFFFull) return set_error(PIMUL_EINVAL, "fractional decimal digit count exceeds u32::MAX");
  const double log_16_10 = std::log2(10.0) / 4.0;  // verify_hex.rs:584-585
  const uint64_t h = (uint32_t)((double)E * log_16_10);
  *out_len = h + 2;
  if (!out || cap < h + 2) return set_error(PIMUL_EINVAL, "decimal to hex: output shorter than the hex text");
  if (phase_ms)
    for (int i = 0; i < 4; i++) phase_ms[i] = 0;
  out[0] = '3';
  out[1] = '.';
  if (E == 0) return PIMUL_OK;  // m = 3

  const double t0 = now_ms();
  Scope A;
  if (cudaStreamCreateWithFlags(&A.st, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    return set_error(PIMUL_ECUDA, "decimal to hex: stream creation failed");
  }
  const cudaStream_t st = A.st;
  int rc = PIMUL_OK;
  auto cu = [&](cudaError_t err, const char* what) {
    if (err != cudaSuccess && !rc)
      rc = set_error(err == cudaErrorMemoryAllocation ? PIMUL_ENOMEM : PIMUL_ECUDA,
                     (std::string("decimal to hex: ") + what + ": " + cudaGetErrorString(err)).c_str());
    return rc == PIMUL_OK;
  };
  auto top_limb = [&](const uint64_t* p, uint64_t* v) {
    cu(cudaMemcpyAsync(v, p, 8, cudaMemcpyDeviceToHost, st), "read back");
    cu(cudaStreamSynchronize(st), "synchronize");
    return rc;
  };

  // ------------------------------------------------------------ parse
  const uint64_t D = E + 1, nch = (D + 18) / 19;
  int K = 0;
  while ((1ull << K) < nch) K++;
  const int LK = std::min(K, LK_MAX);
  const uint64_t nall = 1ull << K, nleaf = nall >> LK;
  char* dtext = nullptr;
  uint64_t *dc = nullptr, *cur = nullptr;
  int* dbad = nullptr;
  if ((rc = A.get(&dtext, n)) || (rc = A.get(&dc, nall)) || (rc = A.get(&dbad, 1))) return rc;
  if ((rc = pimul::host_to_device(dtext, s, n, st))) return rc;
  cu(cudaMemsetAsync(dbad, 0, sizeof(int), st), "memset");
  k_chunks<<<grid_for(nall, 256), 256, 0, st>>>(dtext, D, nall, dc, dbad);
  if (!cu(cudaGetLastError(), "chunk kernel")) return rc;
  A.put(dtext);
  const std::vector<uint64_t> p_leaf = pow10_host(19ull << LK);
  const uint32_t w0 = (uint32_t)p_leaf.size();
  if (w0 > LEAF_W_MAX) return set_error(PIMUL_EINVAL, "decimal to hex: leaf too wide");
  if ((rc = A.get(&cur, nleaf * w0))) return rc;
  k_parse_leaves<<<grid_for(nleaf, 128), 128, 0, st>>>(dc, LK, nleaf, w0, cur);
  if (!cu(cudaGetLastError(), "leaf kernel")) return rc;
  A.put(dc);
  int hbad = 0;
  cu(cudaMemcpyAsync(&hbad, dbad, sizeof(int), cudaMemcpyDeviceToHost, st), "read back");
  cu(cudaStreamSynchronize(st), "synchronize");
  if (rc) return rc;
  if (hbad) return set_error(PIMUL_EINVAL, "the decimal text has non-digit characters after \"3.\"");

  // P_k = 10^(19 2^k) for LK <= k < K: P_LK from the host, then squarings
  std::vector<uint64_t*> dP(K + 1, nullptr);
  std::vector<size_t> lP(K + 1, 0);
  if ((rc = A.get(&dP[LK], w0))) return rc;
  if ((rc = pimul::host_to_device(dP[LK], p_leaf.data(), w0 * 8, st))) return rc;
  lP[LK] = w0;
  for (int k = LK; k + 1 < K; k++) {
    if ((rc = A.get(&dP[k + 1], 2 * lP[k]))) return rc;
    if ((rc = pimul_mul_device(dP[k], lP[k], dP[k], lP[k], dP[k + 1], st))) return rc;
    uint64_t top = 0;
    if ((rc = top_limb(dP[k + 1] + 2 * lP[k] - 1, &top))) return rc;
    lP[k + 1] = top ? 2 * lP[k] : 2 * lP[k] - 1;
  }

  // levels: node i of level k + 1 = node 2i + 1 of level k times P_k plus
  // node 2i.  A level-k node holds 2^k chunks, so the high node of pair i
  // is zero when (2i + 1) 2^k >= nch: only the first nh pairs multiply; the
  // others copy their low node up.  Every node and product has the same
  // (zero-padded) width, so both run as strided batches; the sums stay
  // below P_(k+1) and fit wn limbs.
  size_t w = w0;
  uint64_t nn = nleaf;
  for (int k = LK; k < K; k++) {
    const size_t wn = k + 1 < K ? lP[k + 1] : 2 * lP[k];
    const uint64_t half = nn / 2, span = 1ull << k;
    const uint64_t nh = nch <= span ? 0 : std::min<uint64_t>(half, (nch - span + 2 * span - 1) >> (k + 1));
    uint64_t *nxt = nullptr, *prod = nullptr;
    if ((rc = A.get(&nxt, half * wn)) || (rc = A.get(&prod, std::max<uint64_t>(nh, 1) * 2 * w))) return rc;
    if ((rc = pimul::mul_batch_strided(cur + w, 2 * w, w, dP[k], w, prod, 2 * w, nh, st))) return rc;
    if ((rc = pimul::addsub_strided(prod, 2 * w, std::min(2 * w, wn), cur, 2 * w, w, nxt, wn, wn, 0, nh, st)))
      return rc;
    if ((rc = pimul::addsub_strided(cur + 2 * nh * w, 2 * w, w, nullptr, 0, 0, nxt + nh * wn, wn, wn, 0, half - nh,
                                    st)))
      return rc;
    A.put(prod);
    A.put(cur);
    cur = nxt;
    w = wn;
    nn = half;
  }
  size_t nN = 0;
  {
    const uint64_t* one_arr = cur;
    if ((rc = pimul_top_limbs(&one_arr, &w, 1, &nN, st))) return rc;
  }
  if (nN == 0) return set_error(PIMUL_EINVAL, "decimal to hex: the parsed value is zero");
  const double t1 = now_ms();

  // ------------------------------------------------------------ 10^E
  const uint64_t q = E / 19, r = E % 19;
  const std::vector<uint64_t> q_small = pow10_host(r + 19 * (q & ((1ull << LK) - 1)));
  size_t nQ = q_small.size();
  uint64_t* dQ = nullptr;
  if ((rc = A.get(&dQ, nQ))) return rc;
  if ((rc = pimul::host_to_device(dQ, q_small.data(), nQ * 8, st))) return rc;
  for (int j = LK; j < K; j++) {
    if (!((q >> j) & 1)) continue;
    uint64_t* t = nullptr;
    if ((rc = A.get(&t, nQ + lP[j]))) return rc;
    if ((rc = pimul_mul_device(dQ, nQ, dP[j], lP[j], t, st))) return rc;
    uint64_t top = 0;
    if ((rc = top_limb(t + nQ + lP[j] - 1, &top))) return rc;
    A.put(dQ);
    dQ = t;
    nQ = top ? nQ + lP[j] : nQ + lP[j] - 1;
  }
  for (int k = LK; k < K; k++) A.put(dP[k]);
  cu(cudaStreamSynchronize(st), "synchronize");
  if (rc) return rc;
  const double t2 = now_ms();

  // ------------------------------------------------------------ quotient
  const uint64_t prec = 4 * h + 64;
  const uint64_t one_h = 1;
  uint64_t* ip = nullptr;
  size_t nip = 0;
  if ((rc = pidec::quotient_device(dQ, nQ, 0, cur, nN, 0, &one_h, 1, (int64_t)(4 * h), false, prec, &ip, &nip, nullptr)))
    return rc;
  const size_t nm = (4 * h + 2 + 63) / 64 + 1;  // m < 2^(4h + 2), and a limb for an estimate above it
  uint64_t *dm = nullptr, *d_one = nullptr;
  if (nip > nm) {
    cudaFree(ip);
    return set_error(PIMUL_EINVAL, "decimal to hex: quotient estimate out of range");
  }
  if ((rc = A.get(&dm, nm)) || (rc = A.get(&d_one, 1))) {
    cudaFree(ip);
    return rc;
  }
  cu(cudaMemsetAsync(dm, 0, nm * 8, st), "memset");
  if (nip) cu(cudaMemcpyAsync(dm, ip, nip * 8, cudaMemcpyDeviceToDevice, st), "copy");
  cu(cudaMemcpyAsync(d_one, &one_h, 8, cudaMemcpyHostToDevice, st), "copy");
  cu(cudaStreamSynchronize(st), "synchronize");  // one_h is on this stack frame; ip is copied
  cudaFree(ip);
  if (rc) return rc;
  // m' = estimate - 1 <= m
  pimul_addsub_job dec1{dm, nm, d_one, 1, dm, nm, 1};
  if ((rc = pimul_addsub_batch(&dec1, 1, st))) return rc;
  // r = N 2^(4h) - m' 10^E modulo 2^(64 wr), in [0, 3 10^E)
  const size_t wr = nQ + 1;
  uint64_t *lowN = nullptr, *prod = nullptr, *rr = nullptr, *r2 = nullptr;
  if ((rc = A.get(&lowN, wr)) || (rc = A.get(&prod, nm + nQ)) || (rc = A.get(&rr, wr)) || (rc = A.get(&r2, wr)))
    return rc;
  k_shl_low<<<grid_for(wr, 256), 256, 0, st>>>(cur, nN, 4 * h, lowN, wr);
  if (!cu(cudaGetLastError(), "shift kernel")) return rc;
  if ((rc = pimul_mul_device(dm, nm, dQ, nQ, prod, st))) return rc;
  pimul_addsub_job jr{lowN, wr, prod, std::min(wr, nm + nQ), rr, wr, PIMUL_SUB_MOD};
  if ((rc = pimul_addsub_batch(&jr, 1, st))) return rc;
  uint64_t top = 0;
  if ((rc = top_limb(rr + wr - 1, &top))) return rc;
  if (top >> 63) return set_error(PIMUL_EINVAL, "decimal to hex: quotient estimate more than one above the floor");
  for (int round = 0;; round++) {
    pimul_addsub_job js{rr, wr, dQ, nQ, r2, wr, PIMUL_SUB_MOD};
    if ((rc = pimul_addsub_batch(&js, 1, st))) return rc;
    if ((rc = top_limb(r2 + wr - 1, &top))) return rc;
    if (top >> 63) break;  // r < 10^E: m' = m
    if (round == 3) return set_error(PIMUL_EINVAL, "decimal to hex: quotient estimate more than two below the floor");
    std::swap(rr, r2);
    pimul_addsub_job inc{dm, nm, d_one, 1, dm, nm, 0};
    if ((rc = pimul_addsub_batch(&inc, 1, st))) return rc;
  }
  // m >> 4h must be 3 (verify_hex.rs:599-604: a leading '3')
  {
    const size_t l0 = (size_t)((4 * h) >> 6);
    uint64_t hi[3] = {0, 0, 0};
    const size_t cnt = std::min<size_t>(3, nm - l0);
    cu(cudaMemcpyAsync(hi, dm + l0, cnt * 8, cudaMemcpyDeviceToHost, st), "read back");
    cu(cudaStreamSynchronize(st), "synchronize");
    if (rc) return rc;
    const unsigned bs = (unsigned)((4 * h) & 63);
    const uint64_t v = bs ? (hi[0] >> bs) | (hi[1] << (64 - bs)) : hi[0];
    const uint64_t above = bs ? (hi[1] >> bs) | (hi[2] << (64 - bs)) : hi[1];
    if (v != 3 || above != 0 || (bs ? hi[2] >> bs : hi[2]) != 0)
      return set_error(PIMUL_EINVAL, "internal: hex conversion didn't produce a leading '3'");
  }
  const double t3 = now_ms();

  // ------------------------------------------------------------ print
  if (h) {
    char* dh = nullptr;
    if ((rc = A.get(&dh, h))) return rc;
    k_hex_digits<<<grid_for(h, 256), 256, 0, st>>>(dm, h, dh);
    if (!cu(cudaGetLastError(), "hex kernel")) return rc;
    if ((rc = pimul::device_to_host(out + 2, dh, h, st))) return rc;
  }
  if (phase_ms) {
    phase_ms[0] = t1 - t0;
    phase_ms[1] = t2 - t1;
    phase_ms[2] = t3 - t2;
    phase_ms[3] = now_ms() - t3;
  }
  return PIMUL_OK;
}
