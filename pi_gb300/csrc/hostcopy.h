// Internal: copies between the device and host memory that may be pageable,
// the error message of the C ABI and the unchecked batched addition (defined
// in engine.cu, used by the engine's host entry points, dec.cu, agm.cu and
// hexconv.cu).  Not part of the C ABI.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>

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

}  // namespace pimul
