// Internal interface between the host pi pipeline (pi_host.cpp) and the
// device-resident decimal conversion (dec.cu).  Not part of the C ABI.
#pragma once
#include <cstddef>
#include <cstdint>
#include <utility>
#include <vector>

namespace pidec {

// One level of the divide and conquer: divisor P = 10^(19 * 2^k) and a
// reciprocal V <= floor(2^sh / P), both host limb arrays (little-endian).
struct Level {
  const uint64_t* P;
  size_t lp;
  const uint64_t* V;
  size_t lv;
  uint64_t sh;
};

// Base-10^19 chunks per leaf (levels k >= LEAF_K run on the device).
constexpr int LEAF_K = 6;

// Writes the last `want` of the 19 * 2^K decimal digits of x (zero-padded on
// the left) to out, with x split level by level on the device (levels K-1
// down to LEAF_K, level k at lv[k]: host arrays, or device memory when
// lv_on_device) and the leaves printed by a kernel.  x (host memory, or
// device memory ready for use when x_on_device) must be below
// 10^(19 * 2^K); PIMUL_EINVAL if x has more than `want` digits.
// ms (optional, 3 entries): upload, levels, leaves + download.
int to_decimal_device(const uint64_t* x, size_t nx, bool x_on_device, int K, const Level* lv, bool lv_on_device,
                      char* out, size_t want, double* ms);

// Levels LEAF_K..K-1 of the conversion with P_k and V_k in device memory
// (lv[k] holds device pointers; bufs owns them).  Move-only.
struct DevLevels;
void free_levels_device(DevLevels* L);
struct DevLevels {
  int K = 0;
  std::vector<Level> lv;
  std::vector<uint64_t*> bufs;
  DevLevels() = default;
  DevLevels(const DevLevels&) = delete;
  DevLevels& operator=(const DevLevels&) = delete;
  DevLevels(DevLevels&& o) noexcept : K(o.K), lv(std::move(o.lv)), bufs(std::move(o.bufs)) { o.K = 0; }
  DevLevels& operator=(DevLevels&& o) noexcept {
    if (this != &o) {
      free_levels_device(this);
      K = o.K;
      lv = std::move(o.lv);
      bufs = std::move(o.bufs);
      o.K = 0;
    }
    return *this;
  }
  ~DevLevels() { free_levels_device(this); }
};

// Builds the levels of a 19 * 2^K-digit conversion on the device (K > LEAF_K):
// P_k = 10^(19 * 2^k) by repeated squaring and V_k <= floor(2^(s_k) / P_k),
// s_k = 2 bits(P_k) + 64, within a few units of the floor (a Newton
// reciprocal at the top level, V_(k-1) = (P_(k-1) V_k) >> (s_k - s_(k-1))
// below it).  Its stream has the device's highest priority.  ms (optional):
// time.
int build_levels_device(int K, DevLevels* out, double* ms);

// Chudnovsky's final assembly with Q and |T| in HBM (chudnovsky.rs:146-204
// up to the decimal scaling of util.rs:25-83): *d_ip (allocated here, freed
// by the caller with cudaFree) receives floor(W Q / (A Q - |T|)) in *ipn
// limbs, with W = wm 2^we (the constant 426880 sqrt(10005) times the
// decimal scale: host limbs, or device memory when w_dev) and
// Q = dQ[0..qn) 2^(64 q_off), |T| = dT[0..tn)
// 2^(64 t_off).  The quotient comes from the top prec + 192 bits of each
// operand and a Newton reciprocal run on the device, so its relative error
// is below 2^-(prec + 100).  ms (optional, 2 entries): reciprocal, products.
int final_assembly_device(const uint64_t* dQ, size_t qn, uint64_t q_off, const uint64_t* dT, size_t tn,
                          uint64_t t_off, uint64_t A, const uint64_t* wm, size_t wl, int64_t we, bool w_dev,
                          uint64_t prec, uint64_t** d_ip, size_t* ipn, double* ms);

// floor(W N / D) with D = den[0..wn) 2^den_exp and N = n_top[0..lq) 2^n_exp
// in device memory (ready for use; lq <= (prec + 192 + 63) / 64 top limbs
// of N, D's top limb nonzero within its top three), W = wm 2^we on the
// host (in device memory when w_dev): the final assembly's Newton
// reciprocal and products for any quotient.  *d_ip is freed by the caller
// with cudaFree.
int quotient_device(const uint64_t* den, size_t wn, int64_t den_exp, const uint64_t* n_top, size_t lq, int64_t n_exp,
                    const uint64_t* wm, size_t wl, int64_t we, bool w_dev, uint64_t prec, uint64_t** d_ip,
                    size_t* ipn, double* ms);

// Top limbs of Q (and of A Q + |T|) that final_assembly_device reads.
inline uint64_t final_assembly_top_limbs(uint64_t prec) { return (prec + 192 + 63) / 64 + 3; }

}  // namespace pidec
