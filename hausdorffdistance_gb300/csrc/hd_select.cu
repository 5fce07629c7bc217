// AUTO variant selector driven by sampler statistics.
//
// Replaces the reference's hybrid decision (src/hd_impl/hausdorff_distance_hybrid.h:
// 128-199: EB over ceil(|A| * sample_rate) sampled points with per-point
// iteration counters, percentiles of the sorted counters, and
// "p80 < eb_only_threshold" from a generated XGBoost tree,
// src/models/tree_ebonlythreshold_3d.h) with a project-written rule:
//
//   1. Eight points of A get their exact nearest-neighbour distance (one
//      grid-wide scan of B) and seed the running maximum.  Then k further
//      points of A (k = sample_rate * |A|, clamped to [64, 256]) run the
//      early-break scan against B, one CTA each, B visited in a pseudo-random
//      order, counting the B points each visited before it stopped (capped at
//      16,384).  Seeds and completed samples also seed the running maximum
//      that the chosen variant starts from.
//   2. The EB cost of the full set is ~ |A| * p80 pairs; the index-based cost
//      is ~ |A| + |B| point operations.  EB is chosen when
//          ratio = |A| * p80 / (|A| + |B|)  <  eb_only_threshold,
//      otherwise the LBVH (the grid when the table says so).  The threshold
//      comes from the autotuner's table (hausdorffdistance_gb300/autotune.py
//      fits it over a sweep of workloads) unless hd_options overrides it.
//   3. Size bands from the same table: problems with |A| * |B| up to
//      eb_small_pairs take EB and problems from index_min_pairs up take the
//      index, both without sampling (the sweep shows the choice there does
//      not depend on the data); inputs with n_dims other than 2 or 3 take the
//      split-BF16 tiles when n_dims is a multiple of 16 and the pair count is
//      large, else the FP32 scan.
#include <algorithm>
#include <cfloat>
#include <vector>

#include "hd_common.cuh"
#include "hd_internal.h"
#include "hd_tuning.h"

namespace hdg {
namespace {

constexpr uint32_t kSampleCap = 16384;

__global__ void __launch_bounds__(256)
    k_sample_eb(const float* __restrict__ A, Perm pA, const float* __restrict__ B, Perm pB,
                uint64_t nB, int dims, uint32_t cap, DevScalars* sc, uint32_t* __restrict__ iters) {
  __shared__ float red[8];
  __shared__ float s_thr;
  const uint32_t e = blockIdx.x;
  const uint32_t ia = (uint32_t) pA(e);
  float a[3] = {A[(uint64_t) ia * dims], A[(uint64_t) ia * dims + 1],
                dims == 3 ? A[(uint64_t) ia * dims + 2] : 0.0f};
  float cmin = INFINITY;
  const uint64_t limit = min((uint64_t) cap, nB);
  uint64_t done = 0;
  bool broke = false;
  const uint64_t step = 256 * 8;
  while (done < limit) {
    float m = INFINITY;
    const uint64_t end = min(limit, done + step);
    for (uint64_t j = done + threadIdx.x; j < end; j += 256) {
      const uint64_t b = pB(j);
      const float d = dims == 2 ? d2_2(a[0], a[1], B[2 * b], B[2 * b + 1])
                                : d2_3(a[0], a[1], a[2], B[3 * b], B[3 * b + 1], B[3 * b + 2]);
      m = fminf(m, d);
    }
    done = end;
#pragma unroll
    for (int o = 16; o; o >>= 1) m = fminf(m, __shfl_xor_sync(0xFFFFFFFFu, m, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    if (threadIdx.x == 0) s_thr = threshold_of(ld_relaxed_u64(&sc->max_key));
    __syncthreads();
    for (int k = 0; k < 8; ++k) cmin = fminf(cmin, red[k]);
    const float thr = s_thr;
    __syncthreads();
    if (cmin <= thr) {
      broke = true;
      break;
    }
  }
  if (threadIdx.x == 0) {
    iters[e] = (uint32_t) done;
    // A sample that scanned all of B without stopping has its exact minimum.
    if (!broke && done == nB) atomicMax(&sc->max_key, pack_max(cmin, ia));
  }
}

// Seeds for the sampler: kSeeds points of A get their exact nearest-neighbour
// distance from a grid-wide scan (blockIdx.y = seed, every CTA a slice of B,
// one atomicMin per CTA on the squared distance's bits), so the sampled
// early-break counts below are measured against a real running maximum.
constexpr int kSeeds = 8;

__global__ void __launch_bounds__(256)
    k_seed_scan(const float* __restrict__ A, Perm pA, uint32_t offset, const float* __restrict__ B,
                uint64_t nB, int dims, uint32_t* __restrict__ seed_min) {
  __shared__ uint32_t red[8];
  const uint32_t ia = (uint32_t) pA(offset + blockIdx.y);
  const float a0 = A[(uint64_t) ia * dims], a1 = A[(uint64_t) ia * dims + 1];
  const float a2 = dims == 3 ? A[(uint64_t) ia * dims + 2] : 0.0f;
  float m = INFINITY;
  for (uint64_t j = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; j < nB;
       j += (uint64_t) gridDim.x * blockDim.x) {
    m = fminf(m, dims == 2 ? d2_2(a0, a1, B[2 * j], B[2 * j + 1])
                           : d2_3(a0, a1, a2, B[3 * j], B[3 * j + 1], B[3 * j + 2]));
  }
  uint32_t u = __float_as_uint(m);
#pragma unroll
  for (int o = 16; o; o >>= 1) u = min(u, __shfl_xor_sync(0xFFFFFFFFu, u, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = u;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t b = red[0];
    for (int k = 1; k < 8; ++k) b = min(b, red[k]);
    atomicMin(&seed_min[blockIdx.y], b);
  }
}

__global__ void k_seed_finish(Perm pA, uint32_t offset, const uint32_t* __restrict__ seed_min,
                              DevScalars* sc) {
  const uint32_t e = threadIdx.x;
  if (e < kSeeds)
    atomicMax(&sc->max_key, pack_max(__uint_as_float(seed_min[e]), (uint32_t) pA(offset + e)));
}

}  // namespace

bool select_variant_by_size(const Ctx& c, uint64_t nA, uint64_t nB, int dims, int* v) {
  const Tuning& tu = tuning();
  const double pairs = (double) nA * (double) nB;
  if (dims != 2 && dims != 3) {
    *v = (dims % 16 == 0 && pairs >= tu.bf16_min_pairs) ? HD_VARIANT_BF16 : HD_VARIANT_EB;
    return true;
  }
  const bool sample = c.opt.always_sample != 0;
  if (!sample && pairs <= tu.eb_small_pairs) {
    *v = HD_VARIANT_EB;
    return true;
  }
  if (!sample && pairs >= tu.index_min_pairs) {
    *v = tu.prefer_grid ? HD_VARIANT_GRID : HD_VARIANT_LBVH;
    return true;
  }
  return false;
}

hd_status select_variant(Ctx& c, const DirInput& in, int* v) {
  const Tuning& tu = tuning();
  if (select_variant_by_size(c, in.nA, in.nB, in.dims, v)) return HD_OK;
  const double rate = c.opt.sample_rate > 0 ? c.opt.sample_rate : 0.01;
  uint32_t k = (uint32_t) std::min<double>(std::max<double>(rate * (double) in.nA, 64.0), 256.0);
  k = (uint32_t) std::min<uint64_t>(k, in.nA);
  void* buf;
  hd_status s = ensure(c, kBufCand, (size_t) (k + kSeeds) * 4, &buf);
  if (s != HD_OK) return s;
  DevScalars* sc = scalars(c, in.dir);
  const uint64_t seed = c.opt.seed;
  Perm pA{in.nA, pick_multiplier(in.nA, seed + 11), (seed * 1299709u) % in.nA};
  Perm pB{in.nB, pick_multiplier(in.nB, seed + 13), (seed * 15485863u) % in.nB};
  if (in.nA > k) {
    uint32_t* seed_min = (uint32_t*) buf + k;
    cudaError_t e0 = cudaMemsetAsync(seed_min, 0xFF, kSeeds * 4, c.stream);
    if (e0 != cudaSuccess) return cuda_fail(c, e0, "memset");
    const unsigned gx = (unsigned) std::max<uint64_t>(
        1, std::min<uint64_t>((in.nB + 255) / 256, (uint64_t) c.num_sms * 2));
    k_seed_scan<<<dim3(gx, kSeeds), 256, 0, c.stream>>>(in.A, pA, k, in.B, in.nB, in.dims,
                                                        seed_min);
    if ((s = after_launch(c, "seed_scan")) != HD_OK) return s;
    k_seed_finish<<<1, 32, 0, c.stream>>>(pA, k, seed_min, sc);
    if ((s = after_launch(c, "seed_finish")) != HD_OK) return s;
  }
  k_sample_eb<<<k, 256, 0, c.stream>>>(in.A, pA, in.B, pB, in.nB, in.dims, kSampleCap, sc,
                                       (uint32_t*) buf);
  if ((s = after_launch(c, "sample_eb")) != HD_OK) return s;
  std::vector<uint32_t> it(k);
  cudaError_t e = cudaMemcpyAsync(it.data(), buf, (size_t) k * 4, cudaMemcpyDeviceToHost, c.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "sample statistics");
  std::sort(it.begin(), it.end());
  const double p80 = it[(size_t) (0.8 * (k - 1))];
  const double ratio = (double) in.nA * p80 / (double) (in.nA + in.nB);
  const double thr = c.opt.eb_only_threshold ? (double) c.opt.eb_only_threshold : tu.eb_ratio;
  c.last_p80[in.dir] = p80;
  if (ratio < thr) {
    *v = HD_VARIANT_EB;
  } else {
    *v = tu.prefer_grid ? HD_VARIANT_GRID : HD_VARIANT_LBVH;
  }
  return HD_OK;
}

}  // namespace hdg
