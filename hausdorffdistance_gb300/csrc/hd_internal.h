// Host-side internals shared by the translation units of libhdgpu.so.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/hd_gpu.h"

namespace hdg {

// Bits of a sorted key that hold the Morton code (bit 30 marks the set in
// the fused sort of small sets).
constexpr uint32_t kCodeMask = (1u << 30) - 1u;
// Code bits below a sorted set's low_bits are left out of its sort (three
// radix passes of 8 bits): the sorted order is exact only above them, so
// every consumer compares codes through the set's mask.  Per-set sorts of
// large sets keep 24 code bits (cells of 2^-8 of the frame per axis in 3-D,
// 2^-12 in 2-D); the fused sort of small sets keeps 23 code bits and the set
// bit 30.  Grid levels never go finer than the sorted bits.
constexpr int kSortLowBitsSplit = 6;
constexpr int kSortLowBitsFused = 7;
__host__ __device__ constexpr uint32_t sorted_mask(int low_bits) {
  return kCodeMask & ~((1u << low_bits) - 1u);
}
// From this many points (|A| + |B|) the two sets are sorted as independent
// chains, each in its own frame (and, for host inputs, A's sort overlaps
// B's copy); below it one fused chain in a common frame has fewer launches
// and aligned Morton orders.
constexpr uint64_t kSplitMinPoints = 4000000;

// Device scalars of one directed solve, zeroed with one memset per solve.
struct DevScalars {
  unsigned long long max_key;     // packed (d2 bits, ~ia) running maximum
  unsigned long long min_key;     // packed (d2 bits, ib) certifying argmin
  unsigned long long next;        // work-queue head (visit index)
  unsigned long long pairs;       // pair distances evaluated
  unsigned long long nodes;       // index nodes / cells visited
  unsigned long long leaves;      // leaf / cell visits (HD_COUNT_PAIRS)
  uint32_t heavy_count;           // deferred points
  uint32_t status;                // error bits (kErr*)
  uint32_t sample_count;
  uint32_t heavy_mark;            // EB: deferred entries already finished
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
  kBufScalars,    // DevScalars[2] (one per direction) + spatial frame
  kBufKeys,       // sort keys (scratch)
  kBufKeysAlt,
  kBufVals,       // sort values (scratch)
  kBufValsAlt,
  kBufSorted0,    // Morton-sorted points of set 0 / set 1 (float4 x,y,z,index)
  kBufSorted1,
  kBufCodes0,     // leaf boxes of both sorted sets
  kBufCodes1,
  kBufNodes0,     // LBVH nodes or grid cell table of set 0 / set 1
  kBufNodes1,
  kBufBoxes,      // LBVH build scratch: per-node boxes
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
  kBufGroupOffs,  // offsets of a grouped host-input batch (device copy)
  kBufF64A,       // FP64 input path: caller's double A / B on the device
  kBufF64B,
  kBufF64Aux,     // FP64 scalars and candidate lists
  kBufF64Rows,    // FP64 nearest distance and column of every walked row
  kNumBufs
};

// Cubic Morton frame of a sorted point set (device resident, two of them
// after the two DevScalars in the scalars buffer; frame k belongs to
// c.sorted[k], or frame 0 to both sets when they share a common frame).  A
// query set's points are coded in the target set's frame (frame_code)
// wherever they meet the target's sorted codes.
struct Frame {
  float lo[3], hi[3];
  float scale, extent;  // quantisation scale (cells per unit), max extent
  int bits, dims;       // Morton bits per axis, dimensionality
};

#ifdef __CUDACC__
__device__ __forceinline__ uint32_t morton_spread2(uint32_t x) {  // 16 bits -> even bits
  x &= 0xFFFFu;
  x = (x | (x << 8)) & 0x00FF00FFu;
  x = (x | (x << 4)) & 0x0F0F0F0Fu;
  x = (x | (x << 2)) & 0x33333333u;
  x = (x | (x << 1)) & 0x55555555u;
  return x;
}
__device__ __forceinline__ uint32_t morton_spread3(uint32_t x) {  // 10 bits -> every 3rd bit
  x &= 0x3FFu;
  x = (x | (x << 16)) & 0x030000FFu;
  x = (x | (x << 8)) & 0x0300F00Fu;
  x = (x | (x << 4)) & 0x030C30C3u;
  x = (x | (x << 2)) & 0x09249249u;
  return x;
}
// Cell index of coordinate v along one axis, clamped to the frame.
__device__ __forceinline__ uint32_t frame_quant(float v, float lo, float scale, uint32_t maxq) {
  float q = (v - lo) * scale;
  q = fminf(fmaxf(q, 0.0f), (float) maxq);
  return (uint32_t) q;
}
// Morton code of a point in frame f (points outside the frame clamp to its
// border cells), D = f.dims.  D is a template parameter on purpose: one
// body that chose between the 2-D and 3-D interleave at run time produced
// wrong y bits inside one kernel on sm_103a (nvcc 13.0) while the same
// arithmetic written without the run-time branch was right, so every caller
// is instantiated per dimensionality.
template <int D>
__device__ __forceinline__ uint32_t frame_code(const Frame& f, float x, float y, float z) {
  const uint32_t maxq = (1u << f.bits) - 1u;
  const uint32_t qx = frame_quant(x, f.lo[0], f.scale, maxq);
  const uint32_t qy = frame_quant(y, f.lo[1], f.scale, maxq);
  if constexpr (D == 2) {
    (void) z;
    return morton_spread2(qx) | (morton_spread2(qy) << 1);
  } else {
    const uint32_t qz = frame_quant(z, f.lo[2], f.scale, maxq);
    return morton_spread3(qx) | (morton_spread3(qy) << 1) | (morton_spread3(qz) << 2);
  }
}
#endif

// A point set in Morton order: float4 (x, y, z|0, caller index as bits).
struct SortedSet {
  float4* pts = nullptr;
  uint32_t* codes = nullptr;   // sorted Morton codes (30 bits) in this set's frame
  const Frame* frame = nullptr;  // that frame (device)
  float4* leaf_boxes = nullptr;  // per leaf of leaf_size points: lo, hi
  uint32_t leaf_size = 16;
  uint64_t n = 0;
  int dims = 0;
  const float* src = nullptr;  // device pointer it was sorted from
  int low_bits = kSortLowBitsSplit;                // code bits left out of the sort
  uint32_t mask = sorted_mask(kSortLowBitsSplit);  // the sorted code bits
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
  void* sel_pinned = nullptr;    // pinned staging of the selector's samples
  size_t sel_pinned_bytes = 0;
  void* batch_pinned = nullptr;  // pinned staging of grouped batch results
  size_t batch_pinned_bytes = 0;
  std::string last_error;
  uint64_t launches = 0;
  // Timing events (HD_TIMING): [12*dir + phase] per direction, 24/25 = the
  // whole call.  Read after the call's final synchronisation.
  cudaEvent_t ev[26] = {};
  bool timing = false;
  int ev_base = 0;
  // Batched solve: instantiated graphs and the launch shapes they were
  // captured for (reused while the shape, buffers and stream are unchanged);
  // several, because a host-input batch runs as a few groups of problems.
  static constexpr int kBatchGraphs = 16;
  cudaGraphExec_t batch_graphs[kBatchGraphs] = {};
  uint64_t batch_keys[kBatchGraphs][17] = {};
  uint64_t batch_stamp[kBatchGraphs] = {};
  uint64_t batch_clock = 0;
  // Host-input batches: group copies run on their own stream, one event per
  // group.
  static constexpr int kBatchGroups = 16;
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t copy_ev[kBatchGroups] = {};
  // Side stream and fork/join events (created on first use): the batch
  // graph's second branch and the LBVH packet positions beside the build.
  cudaStream_t batch_side = nullptr;
  // Single solves: the kernel sequence of an LBVH or EB solve is captured the
  // second time the same shape runs back to back and replayed while it stays
  // the same (pointers, sizes, flags, chosen variants, stream, buffers).
  cudaGraphExec_t solve_graph = nullptr;
  uint64_t solve_key[11] = {};
  bool solve_key_seen = false;      // solve_key ran once uncaptured
  bool solve_graph_valid = false;   // solve_graph replays solve_key
  uint64_t solve_graph_launches = 0;
  uint64_t buf_gen = 0;             // bumped by every (re)allocation
  cudaEvent_t batch_fork = nullptr, batch_join = nullptr;
  // Per-solve cache: the Morton-sorted sets (slot 0 = call's A, 1 = call's B)
  // are shared by both directions of an undirected solve.
  SortedSet sorted[2];
  bool sorted_valid = false;
  // Sampler statistic of the last AUTO decision per direction (p80 of the
  // sampled early-break iteration counts; 0 when no sample was drawn).
  double last_p80[2] = {0.0, 0.0};
  double last_mean[2] = {0.0, 0.0};
  // Grid statistics of the last AUTO decision per direction (query fraction
  // outside the target's box, target occupancy skew; 0 when not drawn).
  double last_outside[2] = {0.0, 0.0};
  // The selector's sampled scans already raised this direction's running
  // maximum (the EB variant then skips its own seed pass).
  bool seeded[2] = {false, false};
  double last_skew[2] = {0.0, 0.0};
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
// Creates the context's side stream and fork/join events on first use.
hd_status ensure_side(Ctx& c);

DevScalars* scalars(Ctx& c, int dir);

// Directed solvers; each leaves its result in DevScalars[dir] (finalized).
hd_status run_eb(Ctx& c, const DirInput& in);
hd_status run_brute(Ctx& c, const DirInput& in);
hd_status run_eb_nd(Ctx& c, const DirInput& in);  // EB for n_dims other than 2, 3
hd_status run_lbvh(Ctx& c, const DirInput& in);
// Both directions of an undirected solve with shared launches.
hd_status run_lbvh_pair(Ctx& c, const DirInput& ab, const DirInput& ba);
hd_status run_grid(Ctx& c, const DirInput& in);
hd_status run_bf16(Ctx& c, const DirInput& in, DirResult* extra);
// Test hook: the BF16 kernel's approximate row minima (no certification).
hd_status bf16_rowmin_debug(Ctx& c, const DirInput& in, float* rowmin_host);
hd_status select_variant(Ctx& c, const DirInput& in, int* variant);
// AUTO for the ndir directions of one call at once (ins[d].dir == d; the
// directions query and target the same two sets): one sample of each set, one
// read-back.  v[d] receives each direction's variant.
hd_status select_variants(Ctx& c, const DirInput* ins, int ndir, int* v);
// The selector's choice when the sizes alone decide it (no sampling of the
// data); false when it needs the sample pass.
bool select_variant_by_size(const Ctx& c, uint64_t nA, uint64_t nB, int dims, int* variant);

// FP64 input path (hd_f64.cu) and its hooks into the LBVH solve.
// A row of a list: the caller's row index and its FP32 nearest squared
// distance over the rounded sets (float bits).
struct RowEntry {
  uint32_t row;
  uint32_t min32;
};
// A built tree of one direction's target set: packed nodes, the root's
// index (device), the Morton-sorted points (float4 x, y, z, caller index)
// in leaves of `leaf` points.
struct LbvhTree {
  const float4* nodes;
  const uint32_t* root;
  const float4* pts;
  uint64_t n;
  uint32_t leaf;
};
// run_lbvh_f64 solves the cut sets in FP32 with a listing query pass (a row
// stops only once its minimum is at or below soft_stop(running maximum,
// soft_r[k]); rows that stay open are listed in cand[k] with their FP32
// minima, count in *cand_count[k], at most cand_cap stored), records each
// direction's tree and calls f64_seed after certification.
struct F64Plan {
  LbvhTree tree[2];
  RowEntry* cand[2];
  uint32_t* cand_count[2];
  uint32_t cand_cap;
  float soft_r[2];  // bound on |d(x, y) - d(cut x, cut y)|, rounded up
  void* state;      // the FP64 solve's own data (hd_f64.cu)
};
hd_status run_lbvh_f64(Ctx& c, const DirInput* ins, int count, F64Plan* plan);
hd_status f64_seed(Ctx& c, F64Plan& plan, int count);

// Common tail: exact argmin of A[ia] over B, FP64 recomputation, written to
// DevScalars[dir].  Used by every variant.
hd_status certify(Ctx& c, const DirInput& in);

// Resets both directions' DevScalars (allocating the scalars buffer).
hd_status init_scalars(Ctx& c);

// Context-free forms used by hd_solve_eb_noalloc.
cudaError_t certify_on_stream(cudaStream_t st, int num_sms, const float* A, const float* B,
                              uint64_t nB, int dims, DevScalars* sc);
cudaError_t init_scalars_on_stream(cudaStream_t st, DevScalars* sc, int n);

// Event-based phase timing (HD_TIMING).
void mark(Ctx& c, int phase_event);

uint64_t pick_multiplier(uint64_t n, uint64_t seed);

// Spatial preparation (hd_spatial.cu).
Frame* frame(Ctx& c, int set);
size_t scalars_bytes();
// Morton-sorts the call's two point sets (both, once per hd_solve) and
// returns the ones matching a directed input: *q = in.A, *t = in.B.
hd_status spatial_prepare(Ctx& c, const DirInput& in, const SortedSet** q,
                          const SortedSet** t);
// Host inputs: copies A, sorts it while B is copied on the side stream,
// then sorts B (sets c.sorted, c.sorted_valid); *dA, *dB = device copies.
hd_status spatial_upload_sort(Ctx& c, const float* hA, uint64_t nA, const float* hB, uint64_t nB,
                              int dims, const float** dA, const float** dB);
// k random positions in [0, n) (with replacement), k from opt.sample_rate.
hd_status make_sample(Ctx& c, uint64_t n, uint64_t seed, uint32_t* k, uint32_t** list);

}  // namespace hdg

struct hd_ctx : public hdg::Ctx {};
