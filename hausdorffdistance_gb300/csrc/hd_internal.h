// Host-side internals shared by the translation units of libhdgpu.so.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/hd_gpu.h"

namespace hdg {

// Device scalars of one directed solve, zeroed with one memset per solve.
struct DevScalars {
  unsigned long long max_key;     // packed (d2 bits, ~ia) running maximum
  unsigned long long min_key;     // packed (d2 bits, ib) certifying argmin
  unsigned long long next;        // work-queue head (visit index)
  unsigned long long pairs;       // pair distances evaluated
  unsigned long long nodes;       // index nodes / cells visited
  unsigned long long next2;       // second queue head
  uint32_t heavy_count;           // deferred points
  uint32_t status;                // error bits (kErr*)
  uint32_t sample_count;
  uint32_t pad;
  // Finalised result written by the finalize kernel.
  double d2_64;                   // FP64 squared distance of (ia, ib)
  float d2;                       // FP32 squared distance (max-min)
  uint32_t ia, ib;
  uint32_t pad2;
  uint32_t mbr_ord[2][2][4];      // [set][lo/hi][dim], order-preserving uints
};

// A growable device buffer cached in the context across solves.
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
};

enum BufSlot {
  kBufA = 0,      // caller's A copied to the device (host-pointer solves)
  kBufB,
  kBufPackB,      // packed / permuted B (float2, float4 or padded rows)
  kBufPackA,
  kBufHeavy,      // deferred early-break entries
  kBufScalars,    // DevScalars[2] (one per direction)
  kBufKeys,       // sort keys
  kBufKeysAlt,
  kBufVals,       // sort values
  kBufValsAlt,
  kBufNodes,      // LBVH nodes / grid cell table
  kBufLeafBox,
  kBufAux,        // parents / flags / cell offsets
  kBufAux2,
  kBufCubTemp,
  kBufSample,
  kBufBf16A,      // split-BF16 operands
  kBufBf16B,
  kBufNormsA,
  kBufNormsB,
  kBufRowMin,
  kBufCand,
  kBufBatch,
  kBufBatch2,
  kNumBufs
};

struct Ctx {
  int device = 0;
  int num_sms = 0;
  hd_options opt{};
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  DevBuf bufs[kNumBufs];
  void* host_pinned = nullptr;   // pinned result staging
  size_t host_pinned_bytes = 0;
  std::string last_error;
  uint64_t launches = 0;
  cudaEvent_t ev[12] = {};
  bool timing = false;
  int ev_used = 0;
  cudaGraphExec_t batch_graph = nullptr;
};

// Result of one directed solve, on the host.
struct DirResult {
  float d2 = 0.0f;
  uint32_t ia = 0, ib = 0;
  double d2_64 = 0.0;
  uint64_t pairs = 0, nodes = 0;
  int variant = 0;
  double err_bound = 0.0;
  uint64_t rechecked = 0;
};

// Inputs of one directed solve, resident on the device (row-major floats).
struct DirInput {
  const float* A;
  uint64_t nA;
  const float* B;
  uint64_t nB;
  int dims;
  int dir;      // 0: A->B, 1: B->A (selects the DevScalars slot)
  bool count;
};

// Records the first failure on the context and returns its status.
hd_status fail(Ctx& c, hd_status s, const std::string& msg);
hd_status cuda_fail(Ctx& c, cudaError_t e, const char* what);

// Returns the buffer, growing it (contents not kept) when smaller than bytes.
hd_status ensure(Ctx& c, BufSlot slot, size_t bytes, void** out);

// Counts a kernel launch and checks for launch errors.
hd_status after_launch(Ctx& c, const char* what);

DevScalars* scalars(Ctx& c, int dir);

// Directed solvers; each leaves its result in DevScalars[dir] (finalized).
hd_status run_eb(Ctx& c, const DirInput& in);
hd_status run_brute(Ctx& c, const DirInput& in);
hd_status run_lbvh(Ctx& c, const DirInput& in);
hd_status run_grid(Ctx& c, const DirInput& in);
hd_status run_bf16(Ctx& c, const DirInput& in, DirResult* extra);
hd_status select_variant(Ctx& c, const DirInput& in, int* variant);

// Common tail: exact argmin of A[ia] over B, FP64 recomputation, written to
// DevScalars[dir].  Used by every variant.
hd_status certify(Ctx& c, const DirInput& in);

// Event-based phase timing (HD_TIMING).
void mark(Ctx& c, int phase_event);

uint64_t pick_multiplier(uint64_t n, uint64_t seed);

}  // namespace hdg

struct hd_ctx : public hdg::Ctx {};
