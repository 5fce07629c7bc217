// Morton sort of one or two point sets (hd_msort.cu), used by the spatial
// preparation of the LBVH and grid variants.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "hd_internal.h"

namespace hdg {

// One set to sort: its caller-order points, its frame and its buffers.
struct MsortSet {
  const float* P;          // caller's points, row-major n x dims
  uint64_t n;
  const Frame* fr;         // frame the codes are formed in (device)
  uint32_t shift;          // bin of a code = code >> shift
  uint32_t nbins;          // 2^(30 - shift)
  uint32_t* bins;          // nbins counters: counts, then starts, then ends
  uint32_t* tile_sums;     // scan scratch, nbins / 2048 + 1 entries
  float4* pts;             // out: sorted (x, y, z, caller index)
  uint32_t* codes;         // out: sorted codes
  float4* tpts;            // scratch of n records for bins above 4096 records
  uint32_t* tcodes;
  uint32_t* mid_list;      // bins of 33..4096 records (list_cap entries)
  uint32_t* big_list;      // bins of more than 4096 records (list_cap entries)
  uint32_t* counters;      // [0] mid count, [1] big count (4 words, zeroed per sort)
  uint32_t* status;        // solve status word: kErrInternal on an overflow
  uint32_t list_cap;
  uint32_t L;              // leaf size (power of two <= 32)
  float4* leaf_boxes;      // out: lo, hi per leaf
};
struct MsortSets {
  MsortSet s[2];
};

// Bin shift for a set of n points (about n/8 bins, 2^10 .. 2^21).
uint32_t msort_shift(uint64_t n);

// Sorts `count` sets (1 or 2, in shared launches) on stream st; the frames
// must already be on the device.  ss.s[k].bins etc. must be allocated.
hd_status msort_run(Ctx& c, MsortSets& ss, int count, int dims, cudaStream_t st);

}  // namespace hdg
