// Internal: copies between the device and host memory that may be pageable,
// the error message of the C ABI, the unchecked batched addition and the
// strided batches (defined in engine.cu, used by the engine's host entry
// points, dec.cu, agm.cu and hexconv.cu).  Not part of the C ABI.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

#include "../../include/pimul.h"

namespace pimul {

// dst (device) <- src (host), ordered on st.  On return src may be reused;
// the last chunk may still be in flight on st.
int host_to_device(void* dst, const void* src, size_t bytes, cudaStream_t st);

// dst (host) <- src (device), ordered after the work already on st.
// Synchronous: dst holds the data on return.
int device_to_host(void* dst, const void* src, size_t bytes, cudaStream_t st);

// Frees the pinned staging buffers (device idle).
void release_host_staging();

// Sets the calling thread's pimul_last_error() message; returns code.
int set_error(int code, const char* msg);

// Batched additions and subtractions launched without the carry-out check
// (for callers whose outputs have room for every carry, and differences
// x - y with x >= y): asynchronous on st.
int svc_addsub(const pimul_addsub_job* jobs, size_t n, cudaStream_t st);

// n products out + i so = (a + i sa) * b (la, lb, la + lb limbs; b shared),
// the same results as pimul_mul_batch on the n jobs.  Products of transform
// length up to 2^12 get their descriptors from a kernel (no host loop over
// the jobs, no descriptor upload); longer ones go through pimul_mul_batch.
// Asynchronous on st.
int mul_batch_strided(const uint64_t* a, uint64_t sa, size_t la, const uint64_t* b, size_t lb, uint64_t* out,
                      uint64_t so, size_t n, cudaStream_t st);

// n unchecked additions or subtractions (sub as in pimul_addsub_job) of one
// shape: out + i so = (x + i sx) +- (y + i sy) over nout limbs, descriptors
// written by a kernel.  Asynchronous on st.
int addsub_strided(const uint64_t* x, uint64_t sx, size_t nx, const uint64_t* y, uint64_t sy, size_t ny, uint64_t* out,
                   uint64_t so, size_t nout, int sub, size_t n, cudaStream_t st);

}  // namespace pimul
