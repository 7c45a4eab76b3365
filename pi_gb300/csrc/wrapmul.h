// Internal helper of the device pi drivers (dec.cu, agm.cu).  Not part of
// the C ABI.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

#include "../../include/pimul.h"

namespace pimul {

// pimul_mul_device's product (la + lb limbs at out) through the batch with
// PIMUL_BATCH_WRAP: a long product that would half fill its transform runs
// as a cyclic product of half the length, with the same result.
inline int mul_wrapped(const uint64_t* a, size_t la, const uint64_t* b, size_t lb, uint64_t* out, cudaStream_t st) {
  if (!la || !lb) return pimul_mul_device(a, la, b, lb, out, st);
  const pimul_sum_job j{a, la, b, lb, nullptr, 0, nullptr, 0, out, la + lb};
  return pimul_sum_batch_ex(&j, 1, st, PIMUL_BATCH_WRAP);
}

}  // namespace pimul
