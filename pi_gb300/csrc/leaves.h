// Internal interface between the host pi pipeline (pi_host.cpp) and the
// device leaf kernel (leaves.cu).  Not part of the C ABI.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace pileaf {

// Terms per leaf the kernel accepts.
constexpr uint32_t MAX_TERMS = 64;

// P, Q, T of nleaf consecutive leaves of m terms each, the first starting at
// term a0 and the last ending at b, into d_out: leaf i owns the slot
// d_out + i (sp + sq + st) with |P| at offset 0, Q at sp and |T| at sp + sq.
// lens[3 i + 0..2] receive the trimmed lengths of |P|, Q, |T| and signs[i]
// the signs (bit 0: P < 0, bit 1: T < 0).  Synchronous on `stream`.
// PIMUL_EINVAL if a value outgrows its slot (nothing past a slot is
// written), a merge inside a leaf breaks the splitting's static signs,
// m > MAX_TERMS or b > 2^31.
int leaves_device(uint64_t a0, uint64_t b, uint32_t m, uint32_t nleaf, uint32_t sp, uint32_t sq, uint32_t st,
                  uint64_t* d_out, uint32_t* lens, uint8_t* signs, cudaStream_t stream);

}  // namespace pileaf
