// Batched Hausdorff distances: many independent 2-D / 3-D problems of uneven
// sizes in one CUDA-graph launch of a persistent kernel.  No counterpart in
// the reference, which solves one pair per hd_exec run; the per-problem
// baseline (hd_solve_batch_plain) runs the plain early-break solve once per
// problem with its own launches.
//
// Work decomposition.  A problem-direction (problem p, A->B or B->A) is cut
// into items of 32 query rows; one warp processes one item, one lane per
// row.  Items are ordered largest problem first (longest-processing-time
// order over |A|*|B|); warps take items in a grid-stride sweep over that
// order, so there is no queue atomic per item.  Three passes, captured in one
// graph:
//   1. window bound: every row takes the minimum over a few points of the
//      other set around its relative position, an upper bound on its
//      nearest-neighbour distance; the largest bound per problem-direction
//      (with its row) is kept;
//   2. seed: one warp per problem-direction computes the exact nearest
//      neighbour of that row and starts the running maximum with it;
//   3. sweep: every row scans with early break against that maximum.
//
// Per row: a circular scan of the other set, starting at the row's relative
// position (row * |Y| / |X|), so that sets stored in a spatially coherent
// order (polylines, scans) meet their nearest points within a few steps; the
// row stops as soon as its running minimum is at or below its problem's
// running maximum, or completes and raises that maximum with one 64-bit
// atomicMax (distance bits, ~row).  Squared distances use the reference
// formula, so results are bit-identical to the single-problem solve.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <numeric>
#include <vector>

#include "hd_common.cuh"
#include "hd_internal.h"
#include "hd_tuning.h"

namespace hdg {
namespace {

constexpr int kBatchThreads = 256;
constexpr int kCheckEvery = 8;     // pairs between early-break checks
constexpr int kRefreshEvery = 64;  // pairs between reloads of the running maximum

struct PD {
  float d2;
  uint32_t ia, ib;
  uint32_t valid;
};

template <int D>
__device__ __forceinline__ float pt_d2(const float* __restrict__ X, uint64_t i,
                                       const float* __restrict__ Y, uint64_t j) {
  if constexpr (D == 2) {
    const float2 a = *reinterpret_cast<const float2*>(X + 2 * i);
    const float2 b = *reinterpret_cast<const float2*>(Y + 2 * j);
    return d2_2(a.x, a.y, b.x, b.y);
  } else {
    return d2_3(X[3 * i], X[3 * i + 1], X[3 * i + 2], Y[3 * j], Y[3 * j + 1], Y[3 * j + 2]);
  }
}

// Decodes a global item index into (sorted problem rank, direction, item);
// item numbers start at 1.
__device__ __forceinline__ void decode_item(uint64_t w, int ndir,
                                            const uint64_t* __restrict__ rest_prefix,
                                            uint32_t nprob, const hd_problem* __restrict__ probs,
                                            const uint32_t* __restrict__ order, uint32_t* r_out,
                                            int* d_out, uint64_t* item_out) {
  uint32_t lo = 0, hi = nprob;  // rest_prefix[lo] <= w < rest_prefix[hi]
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (rest_prefix[mid] <= w)
      lo = mid;
    else
      hi = mid;
  }
  const uint64_t local = w - rest_prefix[lo];
  const hd_problem pr = probs[order[lo]];
  const uint64_t it0 = (pr.n_a + 31) / 32;  // items of direction 0
  *r_out = lo;
  if (local < it0 || ndir == 1) {
    *d_out = 0;
    *item_out = local + 1;
  } else {
    *d_out = 1;
    *item_out = local - it0 + 1;
  }
}

constexpr int kWindow = 4;  // window half-width of the bound pass

// Pass 1 (mode 0) and pass 3 (mode 1) over items of 32 rows.
//   mode 0: each row takes the minimum over a window of 2*kWindow+1 points
//           of the other set around its relative position, an upper bound on
//           its nearest-neighbour distance; the warp's largest bound (with its
//           row) goes to ubound[problem-direction] by one atomicMax.
//   mode 1: each row scans the other set circularly from the start of that
//           window with early break against the running maximum.
template <int D>
__global__ void __launch_bounds__(kBatchThreads)
    k_batch(const float* __restrict__ A, const float* __restrict__ B,
            const hd_problem* __restrict__ probs, const uint32_t* __restrict__ order,
            const uint64_t* __restrict__ rest_prefix, uint32_t nprob, int ndir, uint64_t total,
            int mode, unsigned long long* __restrict__ keys,
            unsigned long long* __restrict__ ubound) {
  const int lane = threadIdx.x & 31;
  const uint64_t warps = (uint64_t) gridDim.x * (kBatchThreads / 32);
  for (uint64_t w = (uint64_t) blockIdx.x * (kBatchThreads / 32) + (threadIdx.x >> 5); w < total;
       w += warps) {
    uint32_t r;
    int d;
    uint64_t item;
    decode_item(w, ndir, rest_prefix, nprob, probs, order, &r, &d, &item);
    const uint32_t p = order[r];
    const hd_problem pr = probs[p];
    const float* X = d == 0 ? A + pr.offset_a * D : B + pr.offset_b * D;
    const float* Y = d == 0 ? B + pr.offset_b * D : A + pr.offset_a * D;
    const uint64_t nx = d == 0 ? pr.n_a : pr.n_b, ny = d == 0 ? pr.n_b : pr.n_a;
    const uint64_t row = (item - 1) * 32 + lane;  // warp-uniform item
    const bool valid = row < nx;
    const uint64_t w0 = ny > 2 * kWindow + 1 ? (uint64_t) (2 * kWindow + 1) : ny;
    uint64_t j = valid ? ((row * ny) / nx + ny - (w0 >> 1)) % ny : 0;
    if (mode == 0) {
      float u = -1.0f;
      if (valid) {
        u = INFINITY;
        for (uint64_t k = 0; k < w0; ++k) {
          u = fminf(u, pt_d2<D>(X, row, Y, j));
          j = (j + 1 == ny) ? 0 : j + 1;
        }
      }
      unsigned long long kk = valid ? pack_max(u, (uint32_t) row) : 0ull;
#pragma unroll
      for (int o = 16; o; o >>= 1) {
        const unsigned long long v = __shfl_xor_sync(0xFFFFFFFFu, kk, o);
        kk = v > kk ? v : kk;
      }
      if (lane == 0 && kk) atomicMax(ubound + 2 * (uint64_t) p + d, kk);
      continue;
    }
    if (!valid) continue;
    unsigned long long* key = keys + 2 * (uint64_t) p + d;
    float thr = threshold_of(ld_relaxed_u64(key));
    float cmin = INFINITY;
    bool broke = false;
    for (uint64_t step = 0; step < ny;) {
      const uint64_t chunk = min((uint64_t) kCheckEvery, ny - step);
      for (uint64_t u = 0; u < chunk; ++u) {
        cmin = fminf(cmin, pt_d2<D>(X, row, Y, j));
        j = (j + 1 == ny) ? 0 : j + 1;
      }
      step += chunk;
      if (cmin <= thr) {
        broke = true;
        break;
      }
      if ((step % kRefreshEvery) == 0) thr = threshold_of(ld_relaxed_u64(key));
    }
    if (!broke) atomicMax(key, pack_max(cmin, (uint32_t) row));
  }
}

// Pass 2: one warp per problem-direction computes the exact nearest-neighbour
// distance of the row with the largest window bound (lanes split the other
// set) and starts the running maximum with it.  That row is the most likely
// maximiser, so the threshold is at or near its final value from the start.
template <int D>
__global__ void k_batch_seed(const float* __restrict__ A, const float* __restrict__ B,
                             const hd_problem* __restrict__ probs, uint32_t nprob, int ndir,
                             const unsigned long long* __restrict__ ubound,
                             unsigned long long* __restrict__ keys) {
  const int lane = threadIdx.x & 31;
  const uint64_t w = (uint64_t) blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  if (w >= (uint64_t) nprob * ndir) return;
  const uint32_t p = (uint32_t) (w / ndir);
  const int d = (int) (w % ndir);
  const unsigned long long ub = ubound[2 * (uint64_t) p + d];
  if (ub == 0) return;
  const hd_problem pr = probs[p];
  const float* X = d == 0 ? A + pr.offset_a * D : B + pr.offset_b * D;
  const float* Y = d == 0 ? B + pr.offset_b * D : A + pr.offset_a * D;
  const uint64_t ny = d == 0 ? pr.n_b : pr.n_a;
  const uint32_t row = unpack_max_index(ub);
  float m = INFINITY;
  for (uint64_t j = lane; j < ny; j += 32) m = fminf(m, pt_d2<D>(X, row, Y, j));
#pragma unroll
  for (int o = 16; o; o >>= 1) m = fminf(m, __shfl_xor_sync(0xFFFFFFFFu, m, o));
  if (lane == 0) atomicMax(keys + 2 * (uint64_t) p + d, pack_max(m, row));
}

// Certification per problem-direction: one warp scans the other set for the
// argmin of the certifying row (lowest index among ties).
template <int D>
__global__ void k_batch_certify(const float* __restrict__ A, const float* __restrict__ B,
                                const hd_problem* __restrict__ probs, uint32_t nprob, int ndir,
                                const unsigned long long* __restrict__ keys, PD* __restrict__ pd) {
  const int lane = threadIdx.x & 31;
  const uint64_t w = (uint64_t) blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  if (w >= (uint64_t) nprob * ndir) return;
  const uint32_t p = (uint32_t) (w / ndir);
  const int d = (int) (w % ndir);
  const hd_problem pr = probs[p];
  const unsigned long long key = keys[2 * (uint64_t) p + d];
  if (key == 0) {
    if (lane == 0) pd[2 * (uint64_t) p + d] = PD{0.0f, 0, 0, 0};
    return;
  }
  const float* X = d == 0 ? A + pr.offset_a * D : B + pr.offset_b * D;
  const float* Y = d == 0 ? B + pr.offset_b * D : A + pr.offset_a * D;
  const uint64_t ny = d == 0 ? pr.n_b : pr.n_a;
  const uint32_t ia = unpack_max_index(key);
  unsigned long long best = ~0ull;
  for (uint64_t j = lane; j < ny; j += 32) {
    const unsigned long long k = pack_min(pt_d2<D>(X, ia, Y, j), (uint32_t) j);
    best = k < best ? k : best;
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    const unsigned long long v = __shfl_xor_sync(0xFFFFFFFFu, best, o);
    best = v < best ? v : best;
  }
  if (lane == 0) {
    const float d2 = __uint_as_float((uint32_t) (key >> 32));
    const uint32_t ok = (uint32_t) (best >> 32) == (uint32_t) (key >> 32);
    pd[2 * (uint64_t) p + d] = PD{d2, ia, (uint32_t) (best & 0xFFFFFFFFull), ok ? 1u : 2u};
  }
}

__global__ void k_batch_finalize(const PD* __restrict__ pd, uint32_t nprob, int ndir,
                                 hd_batch_result* __restrict__ out, uint32_t* __restrict__ bad) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nprob) return;
  const PD a = pd[2 * (uint64_t) p];
  int win = 0;
  PD w = a;
  if (ndir == 2) {
    const PD b = pd[2 * (uint64_t) p + 1];
    if (b.d2 > a.d2) {
      w = b;
      win = 1;
    }
    if (b.valid != 1) atomicAdd(bad, 1u);
  }
  if (a.valid != 1) atomicAdd(bad, 1u);
  out[p] = hd_batch_result{__fsqrt_rn(w.d2), w.ia, w.ib, win};
}

struct BatchPlan {
  std::vector<uint32_t> order;
  std::vector<uint64_t> rest_prefix;
  uint64_t total = 0;
};

hd_status make_plan(const hd_problem* probs, uint64_t n, int ndir, BatchPlan* plan) {
  plan->order.resize(n);
  std::iota(plan->order.begin(), plan->order.end(), 0u);
  std::stable_sort(plan->order.begin(), plan->order.end(), [&](uint32_t x, uint32_t y) {
    return (double) probs[x].n_a * (double) probs[x].n_b >
           (double) probs[y].n_a * (double) probs[y].n_b;
  });
  plan->rest_prefix.resize(n + 1);
  uint64_t acc = 0;
  for (uint64_t r = 0; r < n; ++r) {
    plan->rest_prefix[r] = acc;
    const hd_problem& p = probs[plan->order[r]];
    acc += (p.n_a + 31) / 32;
    if (ndir == 2) acc += (p.n_b + 31) / 32;
  }
  plan->rest_prefix[n] = acc;
  plan->total = acc;
  return HD_OK;
}

hd_status check_problems(Ctx& c, const hd_problem* probs, uint64_t n, uint64_t ta, uint64_t tb) {
  for (uint64_t i = 0; i < n; ++i) {
    const hd_problem& p = probs[i];
    if (p.n_a == 0 || p.n_b == 0)
      return fail(c, HD_ERR_INVALID_ARG, "problem " + std::to_string(i) + " has an empty set");
    if (p.offset_a + p.n_a > ta || p.offset_b + p.n_b > tb)
      return fail(c, HD_ERR_INVALID_ARG, "problem " + std::to_string(i) + " is out of range");
    if (p.n_a >= 0xFFFFFFFFull || p.n_b >= 0xFFFFFFFFull)
      return fail(c, HD_ERR_INVALID_ARG, "problem sets are limited to 2^32-2 points");
  }
  return HD_OK;
}

}  // namespace

hd_status batch_solve(Ctx& c, const float* A, uint64_t total_a, const float* B, uint64_t total_b,
                      int dims, const hd_problem* probs, uint64_t n, uint32_t flags,
                      hd_batch_result* out) {
  if (!A || !B || !probs || !out || n == 0) return fail(c, HD_ERR_INVALID_ARG, "bad arguments");
  if (dims != 2 && dims != 3) return fail(c, HD_ERR_UNSUPPORTED, "batches need n_dims 2 or 3");
  if (n >= 0xFFFFFFFFull) return fail(c, HD_ERR_INVALID_ARG, "too many problems");
  if (flags & ~(HD_UNDIRECTED | HD_DEVICE_PTRS)) return fail(c, HD_ERR_INVALID_ARG, "bad flags");
  hd_status s;
  if ((s = check_problems(c, probs, n, total_a, total_b)) != HD_OK) return s;
  const int ndir = (flags & HD_UNDIRECTED) ? 2 : 1;
  BatchPlan plan;
  make_plan(probs, n, ndir, &plan);

  // Device layout in one buffer: problems | order | rest prefix | keys | PD |
  // results | bad counter.
  const size_t b_probs = n * sizeof(hd_problem);
  const size_t b_order = ((n * 4 + 255) / 256) * 256;
  const size_t b_prefix = ((n + 1) * 8 + 255) / 256 * 256;
  const size_t b_keys = n * 2 * 8;  // also the size of the window-bound words
  const size_t b_pd = n * 2 * sizeof(PD);
  const size_t b_out = ((n * sizeof(hd_batch_result) + 255) / 256) * 256;
  const size_t total_bytes = b_probs + b_order + b_prefix + 2 * b_keys + b_pd + b_out + 256;
  void* buf;
  if ((s = ensure(c, kBufBatch, total_bytes, &buf)) != HD_OK) return s;
  char* base = (char*) buf;
  hd_problem* d_probs = (hd_problem*) base;
  uint32_t* d_order = (uint32_t*) (base + b_probs);
  uint64_t* d_prefix = (uint64_t*) (base + b_probs + b_order);
  unsigned long long* d_keys = (unsigned long long*) (base + b_probs + b_order + b_prefix);
  unsigned long long* d_ub = (unsigned long long*) ((char*) d_keys + b_keys);
  PD* d_pd = (PD*) ((char*) d_ub + b_keys);
  hd_batch_result* d_out = (hd_batch_result*) ((char*) d_pd + b_pd);
  uint32_t* d_bad = (uint32_t*) ((char*) d_out + b_out);

  const float* dA = A;
  const float* dB = B;
  cudaError_t e;
  if (!(flags & HD_DEVICE_PTRS)) {
    void *pa, *pb;
    if ((s = ensure(c, kBufA, total_a * dims * 4, &pa)) != HD_OK) return s;
    if ((s = ensure(c, kBufB, total_b * dims * 4, &pb)) != HD_OK) return s;
    if ((e = cudaMemcpyAsync(pa, A, total_a * dims * 4, cudaMemcpyHostToDevice, c.stream)) != cudaSuccess)
      return cuda_fail(c, e, "copy A");
    if ((e = cudaMemcpyAsync(pb, B, total_b * dims * 4, cudaMemcpyHostToDevice, c.stream)) != cudaSuccess)
      return cuda_fail(c, e, "copy B");
    dA = (const float*) pa;
    dB = (const float*) pb;
  }
  if ((e = cudaMemcpyAsync(d_probs, probs, b_probs, cudaMemcpyHostToDevice, c.stream)) != cudaSuccess ||
      (e = cudaMemcpyAsync(d_order, plan.order.data(), n * 4, cudaMemcpyHostToDevice, c.stream)) != cudaSuccess ||
      (e = cudaMemcpyAsync(d_prefix, plan.rest_prefix.data(), (n + 1) * 8, cudaMemcpyHostToDevice,
                           c.stream)) != cudaSuccess)
    return cuda_fail(c, e, "copy batch plan");

  // One graph: reset, persistent solve, certification, finalisation.
  int occ = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, dims == 2 ? k_batch<2> : k_batch<3>,
                                                kBatchThreads, 0);
  occ = std::max(occ, 1);
  const uint64_t warps_needed = plan.total;
  const int grid = (int) std::max<uint64_t>(
      1, std::min<uint64_t>((uint64_t) c.num_sms * occ, (warps_needed + 7) / 8));
  cudaGraph_t graph = nullptr;
  e = cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return cuda_fail(c, e, "begin capture");
  cudaMemsetAsync(d_keys, 0, b_keys, c.stream);
  cudaMemsetAsync(d_ub, 0, b_keys, c.stream);
  cudaMemsetAsync(d_bad, 0, 4, c.stream);
  const uint64_t pdw = n * ndir;  // problem-directions, one warp each
  for (int pass = 0; pass < 3; ++pass) {
    if (pass == 1) {
      const unsigned sb = (unsigned) ((pdw * 32 + 255) / 256);
      if (dims == 2)
        k_batch_seed<2><<<sb, 256, 0, c.stream>>>(dA, dB, d_probs, (uint32_t) n, ndir, d_ub, d_keys);
      else
        k_batch_seed<3><<<sb, 256, 0, c.stream>>>(dA, dB, d_probs, (uint32_t) n, ndir, d_ub, d_keys);
      continue;
    }
    const int mode = pass == 0 ? 0 : 1;
    if (dims == 2)
      k_batch<2><<<grid, kBatchThreads, 0, c.stream>>>(dA, dB, d_probs, d_order, d_prefix,
                                                       (uint32_t) n, ndir, plan.total, mode,
                                                       d_keys, d_ub);
    else
      k_batch<3><<<grid, kBatchThreads, 0, c.stream>>>(dA, dB, d_probs, d_order, d_prefix,
                                                       (uint32_t) n, ndir, plan.total, mode,
                                                       d_keys, d_ub);
  }
  const uint64_t cw = n * ndir;
  const unsigned cblocks = (unsigned) ((cw * 32 + 255) / 256);
  if (dims == 2)
    k_batch_certify<2><<<cblocks, 256, 0, c.stream>>>(dA, dB, d_probs, (uint32_t) n, ndir, d_keys, d_pd);
  else
    k_batch_certify<3><<<cblocks, 256, 0, c.stream>>>(dA, dB, d_probs, (uint32_t) n, ndir, d_keys, d_pd);
  k_batch_finalize<<<(unsigned) ((n + 255) / 256), 256, 0, c.stream>>>(d_pd, (uint32_t) n, ndir,
                                                                        d_out, d_bad);
  e = cudaStreamEndCapture(c.stream, &graph);
  if (e != cudaSuccess) return cuda_fail(c, e, "end capture");
  cudaGraphExec_t exec = nullptr;
  e = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return cuda_fail(c, e, "instantiate graph");
  e = cudaGraphLaunch(exec, c.stream);
  c.launches += 5;
  if (e != cudaSuccess) {
    cudaGraphExecDestroy(exec);
    return cuda_fail(c, e, "graph launch");
  }
  uint32_t bad = 0;
  if ((e = cudaMemcpyAsync(out, d_out, n * sizeof(hd_batch_result), cudaMemcpyDeviceToHost,
                           c.stream)) != cudaSuccess ||
      (e = cudaMemcpyAsync(&bad, d_bad, 4, cudaMemcpyDeviceToHost, c.stream)) != cudaSuccess ||
      (e = cudaStreamSynchronize(c.stream)) != cudaSuccess) {
    cudaGraphExecDestroy(exec);
    return cuda_fail(c, e, "batch solve");
  }
  cudaGraphExecDestroy(exec);
  if (bad) return fail(c, HD_ERR_CUDA, "batch certification mismatch");
  return HD_OK;
}

hd_status batch_solve_plain(Ctx& c, const float* A, uint64_t total_a, const float* B,
                            uint64_t total_b, int dims, const hd_problem* probs, uint64_t n,
                            uint32_t flags, hd_batch_result* out) {
  if (!A || !B || !probs || !out || n == 0) return fail(c, HD_ERR_INVALID_ARG, "bad arguments");
  if (dims != 2 && dims != 3) return fail(c, HD_ERR_UNSUPPORTED, "batches need n_dims 2 or 3");
  if (flags & ~(HD_UNDIRECTED | HD_DEVICE_PTRS)) return fail(c, HD_ERR_INVALID_ARG, "bad flags");
  hd_status s;
  if ((s = check_problems(c, probs, n, total_a, total_b)) != HD_OK) return s;
  const uint32_t solve_flags = (flags & HD_UNDIRECTED) | HD_DEVICE_PTRS;
  const float* dA = A;
  const float* dB = B;
  cudaError_t e;
  if (!(flags & HD_DEVICE_PTRS)) {
    // Inputs go to separate slots from the per-problem solves' own buffers.
    void *pa, *pb;
    if ((s = ensure(c, kBufBatch, total_a * dims * 4, &pa)) != HD_OK) return s;
    if ((s = ensure(c, kBufBatch2, total_b * dims * 4, &pb)) != HD_OK) return s;
    if ((e = cudaMemcpyAsync(pa, A, total_a * dims * 4, cudaMemcpyHostToDevice, c.stream)) != cudaSuccess ||
        (e = cudaMemcpyAsync(pb, B, total_b * dims * 4, cudaMemcpyHostToDevice, c.stream)) != cudaSuccess)
      return cuda_fail(c, e, "copy inputs");
    dA = (const float*) pa;
    dB = (const float*) pb;
  }
  for (uint64_t i = 0; i < n; ++i) {
    hd_result r;
    s = hd_solve(&static_cast<hd_ctx&>(c), dA + probs[i].offset_a * dims, probs[i].n_a,
                 dB + probs[i].offset_b * dims, probs[i].n_b, dims, solve_flags, HD_VARIANT_EB, &r);
    if (s != HD_OK) return s;
    out[i] = hd_batch_result{r.hd_f32, (uint32_t) r.ia, (uint32_t) r.ib, r.direction};
  }
  return HD_OK;
}

}  // namespace hdg

using namespace hdg;

extern "C" {

hd_status hd_solve_batch(hd_ctx* c, const float* A, uint64_t total_a, const float* B,
                         uint64_t total_b, int n_dims, const hd_problem* probs,
                         uint64_t n_problems, uint32_t flags, hd_batch_result* out) {
  if (!c) return HD_ERR_INVALID_ARG;
  c->last_error.clear();
  cudaSetDevice(c->device);
  return batch_solve(*c, A, total_a, B, total_b, n_dims, probs, n_problems, flags, out);
}

hd_status hd_solve_batch_plain(hd_ctx* c, const float* A, uint64_t total_a, const float* B,
                               uint64_t total_b, int n_dims, const hd_problem* probs,
                               uint64_t n_problems, uint32_t flags, hd_batch_result* out) {
  if (!c) return HD_ERR_INVALID_ARG;
  c->last_error.clear();
  cudaSetDevice(c->device);
  return batch_solve_plain(*c, A, total_a, B, total_b, n_dims, probs, n_problems, flags, out);
}

}  // extern "C"
