// Internal interface between the host pi pipeline (pi_host.cpp) and the
// merged binary-splitting level kernel (engine.cu).  Not part of the C ABI.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace pimerge {

// Longest transform (log2) a merged level takes: every product of a node
// pair stays inside one CTA's shared memory.
constexpr int MAX_LOG = 12;
// Shortest transform (log2) of a merged level: shorter pairs run at 2^8.
constexpr int MIN_LOG = 8;

// One level of the splitting tree in fixed slots.  Node i of the level is
// |P| at in + i (sp + sq + st), Q at + sp, |T| at + sp + sq, with its
// trimmed lengths at in_len[3 i .. 3 i + 2]; pair (2 i, 2 i + 1) becomes
// node i of the next level in slots of op, oq, ot words (an odd last node is
// copied up).  Every left node must hold an even number of terms, so that
// T = |T_L| Q_R + |P_L| |T_R| is a sum of magnitudes.  L: the longest
// transform (log2) any pair of the level needs, which sizes the thread groups.
struct Level {
  const uint64_t* in;
  const uint32_t* in_len;
  uint64_t* out;
  uint32_t* out_len;
  uint32_t sp, sq, st, op, oq, ot;
  uint32_t n_in;
  int L;
};

// Initialises the engine on the current device (root tables, kernel
// attributes) so that merge_level itself makes no set-up call: call it
// before capturing merge_level in a graph.
int prepare();

// Enqueues one merged level on `stream`: no allocation and no
// synchronisation, so a run of levels can be captured in a CUDA graph.
// *d_bad (device memory) is set to 1 if a pair needs a longer transform than
// lv.L or outgrows its slot (that pair is then not written).  PIMUL_EINVAL
// for L outside [MIN_LOG, MAX_LOG] or a slot smaller than the level below it.
int merge_level(const Level& lv, int* d_bad, cudaStream_t stream);

}  // namespace pimerge
