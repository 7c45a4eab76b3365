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
constexpr int LEAF_K = 5;

// Writes the last `want` of the 19 * 2^K decimal digits of x (zero-padded on
// the left) to out, with x split level by level on the device (levels K-1
// down to LEAF_K, level k at lv[k]) and the leaves printed by a kernel.
// x < 10^(19 * 2^K) is required; PIMUL_EINVAL if x has more than `want`
// digits.  ms (optional, 3 entries): upload, levels, leaves + download.
int to_decimal_device(const uint64_t* x, size_t nx, int K, const Level* lv, char* out, size_t want, double* ms);

}  // namespace pidec
