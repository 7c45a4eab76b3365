// Internal interface between the host pi pipeline (pi_host.cpp) and the
// device Gauss-Legendre iteration (agm.cu).  Not part of the C ABI.
#pragma once
#include <cstddef>
#include <cstdint>

namespace piagm {

// The AGM's result: pi = num 2^num_exp / (4 den 2^den_exp), both in device
// memory (cudaMalloc; the caller frees them).
struct AgmOut {
  uint64_t* num = nullptr;
  size_t num_limbs = 0;
  int64_t num_exp = 0;
  uint64_t* den = nullptr;
  size_t den_limbs = 0;
  int64_t den_exp = 0;
};

// The Gauss-Legendre AGM at `prec` bits (plus 64 guard bits) on the device:
// (a + b)^2 and t after ceil(log2 prec) + 2 steps.  ms (optional): time.
int agm_device(uint64_t prec, AgmOut* out, double* ms);

}  // namespace piagm
