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

// A number in device memory: mant[0..limbs) 2^exp (cudaMalloc; the caller
// frees mant with cudaFree).
struct DevNum {
  uint64_t* mant = nullptr;
  size_t limbs = 0;
  int64_t exp = 0;
};

// 5^e exactly (exp = 0), by left-to-right binary powering on the device.
int pow5_device(uint64_t e, DevNum* out);

// Chudnovsky's constant times the decimal scale, W = 426880 sqrt(10005)
// 10^(D-1) (chudnovsky.rs:118-126 and util.rs:25-83), on the device with a
// relative error below 2^-(prec + 128): sqrt(10005) from Newton's iteration
// for an inverse square root, 10^(D-1) = 5^(D-1) 2^(D-1) with 5^(D-1)
// exact.  The stream has the device's highest priority.  ms (optional):
// time.
int chudnovsky_w_device(uint64_t digits, uint64_t prec, DevNum* out, double* ms);

}  // namespace piagm
