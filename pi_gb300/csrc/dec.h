// Internal interface between the host pi pipeline (pi_host.cpp) and the
// device-resident decimal conversion (dec.cu).  Not part of the C ABI.
#pragma once
#include <cstddef>
#include <cstdint>

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
// down to LEAF_K, level k at lv[k]) and the leaves printed by a kernel.
// x (host memory, or device memory ready for use when x_on_device) must be
// below 10^(19 * 2^K); PIMUL_EINVAL if x has more than `want` digits.
// ms (optional, 3 entries): upload, levels, leaves + download.
int to_decimal_device(const uint64_t* x, size_t nx, bool x_on_device, int K, const Level* lv, char* out, size_t want,
                      double* ms);

// Chudnovsky's final assembly with Q and |T| in HBM (chudnovsky.rs:146-204
// up to the decimal scaling of util.rs:25-83): *d_ip (allocated here, freed
// by the caller with cudaFree) receives floor(W Q / (A Q - |T|)) in *ipn
// limbs, with W = wm 2^we (the constant 426880 sqrt(10005) times the
// decimal scale, host limbs) and Q = dQ[0..qn) 2^(64 q_off), |T| = dT[0..tn)
// 2^(64 t_off).  The quotient comes from the top prec + 192 bits of each
// operand and a Newton reciprocal run on the device, so its relative error
// is below 2^-(prec + 100).  ms (optional, 2 entries): reciprocal, products.
int final_assembly_device(const uint64_t* dQ, size_t qn, uint64_t q_off, const uint64_t* dT, size_t tn,
                          uint64_t t_off, uint64_t A, const uint64_t* wm, size_t wl, int64_t we, uint64_t prec,
                          uint64_t** d_ip, size_t* ipn, double* ms);

// floor(W N / D) with D = den[0..wn) 2^den_exp and N = n_top[0..lq) 2^n_exp
// in device memory (ready for use; lq <= (prec + 192 + 63) / 64 top limbs
// of N, D's top limb nonzero within its top three), W = wm 2^we on the
// host: the final assembly's Newton reciprocal and products for any
// quotient.  *d_ip is freed by the caller with cudaFree.
int quotient_device(const uint64_t* den, size_t wn, int64_t den_exp, const uint64_t* n_top, size_t lq, int64_t n_exp,
                    const uint64_t* wm, size_t wl, int64_t we, uint64_t prec, uint64_t** d_ip, size_t* ipn,
                    double* ms);

// Top limbs of Q (and of A Q + |T|) that final_assembly_device reads.
inline uint64_t final_assembly_top_limbs(uint64_t prec) { return (prec + 192 + 63) / 64 + 3; }

}  // namespace pidec
