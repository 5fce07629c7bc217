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
//      early-break scan against B, one warp each, B visited in a
//      pseudo-random order, counting the B points each visited before it
//      stopped (in rounds of 64, capped at 16,384).  Seeds and completed samples also seed the running maximum
//      that the chosen variant starts from.
//   2. The EB cost of the full set is ~ |A| * mean pairs, mean being the
//      average of the sampled counts; the index-based cost is ~ |A| + |B|
//      point operations.  EB is chosen when
//          ratio = |A| * mean / (|A| + |B|)  <  eb_ratio
//      (points that break after a few pairs: heavily duplicated data, or a
//      running maximum far above the typical nearest-neighbour distance).
//      The reference thresholds the 80th percentile instead; the mean keeps
//      the slow tail (say 5% of points that scan all of B), which is most of
//      the EB's work and which an 80th percentile does not see.  The p80 is
//      still reported.  The sample runs up to eb_sample_max_pairs.
//   3. Otherwise an index: the uniform grid or the LBVH, from two statistics
//      of small strided samples of both sets (1,024 points each; the same
//      two samples serve both directions of an undirected solve, read back
//      with the early-break counts in one copy), computed on the host:
//        outside  the fraction of query samples outside the target sample's
//                 box (padded by 1%): queries far from every target point
//                 make the grid's ring search grow without bound;
//        skew     the target's cell-occupancy skew at the grid's resolution
//                 (the reference's rule: |B| / n_points_cell cells over B's
//                 box): the number of target-sample pairs that share a cell
//                 divided by the number a uniform set would give (birthday
//                 statistic, ~1 for uniform data; clustered or planar data,
//                 whose cells are mostly empty and partly crowded, give many
//                 times more).  It plays the role of the reference's grid
//                 histogram Gini feature (src/models/features.h).
//      The grid is chosen when outside <= grid_max_outside and skew <=
//      grid_max_skew, else the LBVH.  An undirected solve takes the grid only
//      when both directions qualify (otherwise both directions share the
//      fused LBVH launches).
//   4. Size bands from the same table: problems with |A| * |B| up to
//      eb_small_pairs take EB and problems from index_min_pairs up take the
//      LBVH, both without sampling (at the largest sizes the grid's worst
//      cases cost tens of times the LBVH while its best cases save ~20%);
//      inputs with n_dims other than 2 or 3 take the split-BF16 tiles when
//      n_dims is a multiple of 16 and the pair count is large, else the FP32
//      scan.
//   All thresholds come from the autotuner's table
//   (hausdorffdistance_gb300/autotune.py fits them over a sweep of
//   workloads); hd_options.eb_only_threshold overrides eb_ratio.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <vector>

#include "hd_common.cuh"
#include "hd_internal.h"
#include "hd_tuning.h"

namespace hdg {
namespace {

constexpr uint32_t kSampleCap = 16384;

// Sampled early-break scans: one warp per sampled point of A, B visited in
// a pseudo-random order, 64 B points per round (two per lane), a warp vote
// after every round; the count of B points visited before the point stopped
// (or the cap) is its statistic.
__global__ void __launch_bounds__(256)
    k_sample_eb(const float* __restrict__ A, Perm pA, uint32_t k, const float* __restrict__ B,
                Perm pB, uint64_t nB, int dims, uint32_t cap, DevScalars* sc,
                uint32_t* __restrict__ iters) {
  const uint32_t e = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (e >= k) return;
  const uint32_t ia = (uint32_t) pA(e);
  const float a0 = A[(uint64_t) ia * dims], a1 = A[(uint64_t) ia * dims + 1];
  const float a2 = dims == 3 ? A[(uint64_t) ia * dims + 2] : 0.0f;
  float cmin = INFINITY;
  const uint64_t limit = min((uint64_t) cap, nB);
  uint64_t done = 0;
  bool broke = false;
  unsigned long long key = 0;
  while (done < limit) {
    const uint64_t end = min(limit, done + 64);
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const uint64_t j = done + lane + 32 * u;
      if (j < end) {
        const uint64_t b = pB(j);
        const float d = dims == 2 ? d2_2(a0, a1, B[2 * b], B[2 * b + 1])
                                  : d2_3(a0, a1, a2, B[3 * b], B[3 * b + 1], B[3 * b + 2]);
        cmin = fminf(cmin, d);
      }
    }
    done = end;
    float m = cmin;
#pragma unroll
    for (int o = 16; o; o >>= 1) m = fminf(m, __shfl_xor_sync(0xFFFFFFFFu, m, o));
    cmin = m;
    if (lane == 0) key = ld_relaxed_u64(&sc->max_key);
    if (cmin <= threshold_of(__shfl_sync(0xFFFFFFFFu, key, 0))) {
      broke = true;
      break;
    }
  }
  if (lane == 0) {
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

// Strided sample of m points of P (point i*n/m), rows of dims floats.
__global__ void k_gather_sample(const float* __restrict__ P, uint64_t n, int dims, uint32_t m,
                                float* __restrict__ out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  const uint64_t src = (uint64_t) i * n / m;
  for (int d = 0; d < dims; ++d) out[(uint64_t) i * dims + d] = P[src * dims + d];
}

constexpr uint32_t kStatSamples = 1024;

// Grid statistics of a query sample q (mq points) against a target sample t
// (mt points) of a target set of nT points (see the rule above).
void grid_stats(const float* q, uint32_t mq, const float* t, uint32_t mt, int dims, uint64_t nT,
                uint32_t npc, double* outside, double* skew) {
  double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
  for (int d = 0; d < dims; ++d) {
    lo[d] = INFINITY;
    hi[d] = -INFINITY;
    for (uint32_t i = 0; i < mt; ++i) {
      lo[d] = std::min(lo[d], (double) t[(size_t) i * dims + d]);
      hi[d] = std::max(hi[d], (double) t[(size_t) i * dims + d]);
    }
    const double pad = 0.01 * (hi[d] - lo[d]);
    lo[d] -= pad;
    hi[d] += pad;
  }
  uint32_t out = 0;
  for (uint32_t i = 0; i < mq; ++i)
    for (int d = 0; d < dims; ++d) {
      const double v = q[(size_t) i * dims + d];
      if (v < lo[d] || v > hi[d]) {
        ++out;
        break;
      }
    }
  *outside = mq ? (double) out / mq : 0.0;
  // The reference's cell size: |B| / n_points_cell cells over the box (zero
  // extents count as 1e-5, as uniform_grid.h does).
  double vol = 1.0;
  for (int d = 0; d < dims; ++d) vol *= hi[d] > lo[d] ? hi[d] - lo[d] : 1e-5;
  const double cells = std::max(1.0, (double) nT / std::max<uint32_t>(npc, 1));
  const double side = std::pow(vol / cells, 1.0 / dims);
  std::vector<uint64_t> keys(mt);
  for (uint32_t i = 0; i < mt; ++i) {
    uint64_t k = 0;
    for (int d = 0; d < dims; ++d) {
      const double c = std::floor((t[(size_t) i * dims + d] - lo[d]) / side);
      k = k * 2097152u + (uint64_t) std::min(std::max(c, 0.0), 2097151.0);
    }
    keys[i] = k;
  }
  std::sort(keys.begin(), keys.end());
  double same = 0.0;
  for (uint32_t i = 0, j; i < mt; i = j) {
    for (j = i + 1; j < mt && keys[j] == keys[i]; ++j) {
    }
    const double c = j - i;
    same += c * (c - 1.0) / 2.0;
  }
  const double expect = (double) mt * (mt - 1.0) / 2.0 / cells;
  *skew = same / std::max(expect, 1e-9);
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
    *v = HD_VARIANT_LBVH;
    return true;
  }
  return false;
}

hd_status select_variants(Ctx& c, const DirInput* ins, int ndir, int* v) {
  const Tuning& tu = tuning();
  bool need = false, decided[2] = {false, false};
  for (int d = 0; d < ndir; ++d) {
    decided[d] = select_variant_by_size(c, ins[d].nA, ins[d].nB, ins[d].dims, &v[d]);
    need |= !decided[d];
  }
  if (!need) return HD_OK;
  // One sample of each set serves both directions (query in one, target in
  // the other); the early-break samples run per direction.  Everything comes
  // back in one copy, with one synchronisation.
  const int dims = ins[0].dims;
  const float* P[2] = {ins[0].A, ins[0].B};
  const uint64_t nP[2] = {ins[0].nA, ins[0].nB};
  const uint32_t m[2] = {(uint32_t) std::min<uint64_t>(nP[0], kStatSamples),
                         (uint32_t) std::min<uint64_t>(nP[1], kStatSamples)};
  uint32_t k[2] = {0, 0};
  const double rate = c.opt.sample_rate > 0 ? c.opt.sample_rate : 0.01;
  for (int d = 0; d < ndir; ++d) {
    if (decided[d]) continue;
    const double pairs = (double) ins[d].nA * (double) ins[d].nB;
    if (c.opt.always_sample == 0 && pairs > tu.eb_sample_max_pairs) continue;
    uint32_t kk = (uint32_t) std::min<double>(std::max<double>(rate * (double) ins[d].nA, 64.0),
                                              256.0);
    k[d] = (uint32_t) std::min<uint64_t>(kk, ins[d].nA);
  }
  // Layout (32-bit words): iteration counts of direction 0 and 1, seed
  // minima of both, sample of set 0 (the call's A), sample of set 1.
  const size_t o_it[2] = {0, k[0]};
  const size_t o_seed = (size_t) k[0] + k[1];
  const size_t o_smp[2] = {o_seed + 2 * kSeeds, o_seed + 2 * kSeeds + (size_t) m[0] * dims};
  const size_t words = o_smp[1] + (size_t) m[1] * dims;
  void* buf;
  hd_status s = ensure(c, kBufCand, words * 4, &buf);
  if (s != HD_OK) return s;
  if (c.sel_pinned_bytes < words * 4) {
    if (c.sel_pinned) cudaFreeHost(c.sel_pinned);
    c.sel_pinned = nullptr;
    c.sel_pinned_bytes = 0;
    if (cudaMallocHost(&c.sel_pinned, words * 4) != cudaSuccess) {
      (void) cudaGetLastError();
      return fail(c, HD_ERR_OOM, "pinned staging for the selector");
    }
    c.sel_pinned_bytes = words * 4;
  }
  uint32_t* w = (uint32_t*) buf;
  for (int t = 0; t < 2; ++t) {
    k_gather_sample<<<(m[t] + 255) / 256, 256, 0, c.stream>>>(P[t], nP[t], dims, m[t],
                                                              (float*) (w + o_smp[t]));
    if ((s = after_launch(c, "gather_sample")) != HD_OK) return s;
  }
  const uint64_t seed = c.opt.seed;
  for (int d = 0; d < ndir; ++d) {
    if (k[d] == 0) continue;
    const DirInput& in = ins[d];
    DevScalars* sc = scalars(c, in.dir);
    Perm pA{in.nA, pick_multiplier(in.nA, seed + 11), (seed * 1299709u) % in.nA};
    Perm pB{in.nB, pick_multiplier(in.nB, seed + 13), (seed * 15485863u) % in.nB};
    if (in.nA > k[d]) {
      uint32_t* seed_min = w + o_seed + (size_t) d * kSeeds;
      cudaError_t e0 = cudaMemsetAsync(seed_min, 0xFF, kSeeds * 4, c.stream);
      if (e0 != cudaSuccess) return cuda_fail(c, e0, "memset");
      const unsigned gx = (unsigned) std::max<uint64_t>(
          1, std::min<uint64_t>((in.nB + 255) / 256, (uint64_t) c.num_sms * 2));
      k_seed_scan<<<dim3(gx, kSeeds), 256, 0, c.stream>>>(in.A, pA, k[d], in.B, in.nB, in.dims,
                                                          seed_min);
      if ((s = after_launch(c, "seed_scan")) != HD_OK) return s;
      k_seed_finish<<<1, 32, 0, c.stream>>>(pA, k[d], seed_min, sc);
      if ((s = after_launch(c, "seed_finish")) != HD_OK) return s;
    }
    k_sample_eb<<<(k[d] * 32 + 255) / 256, 256, 0, c.stream>>>(
        in.A, pA, k[d], in.B, pB, in.nB, in.dims, kSampleCap, sc, w + o_it[d]);
    if ((s = after_launch(c, "sample_eb")) != HD_OK) return s;
    c.seeded[in.dir] = in.nA > k[d];
  }
  uint32_t* h = (uint32_t*) c.sel_pinned;
  cudaError_t e = cudaMemcpyAsync(h, buf, words * 4, cudaMemcpyDeviceToHost, c.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "sample statistics");
  for (int d = 0; d < ndir; ++d) {
    if (decided[d]) continue;
    const DirInput& in = ins[d];
    // Direction d queries set q against set t (set 0 is the call's A).
    const int q = in.A == P[0] && in.nA == nP[0] ? 0 : 1, t = 1 - q;
    double outside = 0.0, skew = 0.0;
    grid_stats(reinterpret_cast<const float*>(h + o_smp[q]), m[q],
               reinterpret_cast<const float*>(h + o_smp[t]), m[t], dims, nP[t],
               c.opt.n_points_cell, &outside, &skew);
    c.last_outside[in.dir] = outside;
    c.last_skew[in.dir] = skew;
    double p80 = 0.0, mean = 0.0;
    if (k[d] > 0) {
      std::vector<uint32_t> it(h + o_it[d], h + o_it[d] + k[d]);
      std::sort(it.begin(), it.end());
      p80 = it[(size_t) (0.8 * (k[d] - 1))];
      for (uint32_t x : it) mean += x;
      mean /= k[d];
    }
    c.last_p80[in.dir] = p80;
    c.last_mean[in.dir] = mean;
    const double ratio = (double) in.nA * mean / (double) (in.nA + in.nB);
    const double thr = c.opt.eb_only_threshold ? (double) c.opt.eb_only_threshold : tu.eb_ratio;
    if (k[d] > 0 && ratio < thr)
      v[d] = HD_VARIANT_EB;
    else if (outside <= tu.grid_max_outside && skew <= tu.grid_max_skew)
      v[d] = HD_VARIANT_GRID;
    else
      v[d] = HD_VARIANT_LBVH;
  }
  return HD_OK;
}

hd_status select_variant(Ctx& c, const DirInput& in, int* v) {
  return select_variants(c, &in, 1, v);
}

}  // namespace hdg
