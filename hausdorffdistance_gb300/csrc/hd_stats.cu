// Point-set statistics for hd_exec's JSON log (hd_compute_stats in
// include/hd_gpu.h): bounding box, density, and the occupancy of the
// reference's statistics grid — the per-file "Grid", "MBR" and "Density"
// entries of src/run_hausdorff_distance.cu:150-185, whose grid is
// src/index/uniform_grid.h (CalculateGridResolution :222-244, Insert
// :343-484, ComputeHistogram :673-693) and whose Gini index is
// src/running_stats.h:33-62.
//
// The counting runs on the device: the box (one atomic per CTA and dimension
// on order-preserving integers), one counter per grid cell (atomic
// increments into a dense array), the largest count and the number of
// non-empty cells, then a histogram of the per-cell counts.  The host turns
// that histogram into the Gini index, the median and the percentile table
// (the counts' sorted order is the histogram's order, so nothing is sorted);
// the grid's shape and the percentile table follow the reference's own
// arithmetic and its HdrHistogram output (hd_stats_host.h).
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <vector>

#include "hd_common.cuh"
#include "hd_internal.h"
#include "hd_stats_host.h"

namespace hdg {
namespace {

constexpr uint64_t kStatsMaxCells = 1ull << 28;  // dense counters: at most 1 GiB
constexpr uint32_t kStatsMaxHist = 1u << 24;     // per-cell counts histogrammed exactly

template <int D>
__global__ void k_stats_mbr(const float* __restrict__ P, uint64_t n, uint32_t* __restrict__ ord) {
  float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
  for (uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < n;
       i += (uint64_t) gridDim.x * blockDim.x)
#pragma unroll
    for (int k = 0; k < D; ++k) {
      const float v = P[i * D + k];
      lo[k] = fminf(lo[k], v);
      hi[k] = fmaxf(hi[k], v);
    }
#pragma unroll
  for (int k = 0; k < D; ++k) {
    float a = lo[k], b = hi[k];
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      a = fminf(a, __shfl_xor_sync(0xFFFFFFFFu, a, o));
      b = fmaxf(b, __shfl_xor_sync(0xFFFFFFFFu, b, o));
    }
    if ((threadIdx.x & 31) == 0) {
      atomicMin(&ord[k], f2ord(a));
      atomicMax(&ord[4 + k], f2ord(b));
    }
  }
}

// A point's cell per axis as the reference computes it
// (UniformGrid::CalculateCellPos, src/index/uniform_grid.h:138-159):
// (p - lo) / extent * size in float, clamped to [0, size - 1], truncated.
struct StatsGrid {
  float lo[3], extent[3];
  uint32_t size[3];
};

template <int D>
__global__ void k_stats_count(const float* __restrict__ P, uint64_t n, StatsGrid g,
                              uint32_t* __restrict__ counts) {
  for (uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < n;
       i += (uint64_t) gridDim.x * blockDim.x) {
    uint64_t cell = 0;
#pragma unroll
    for (int k = D - 1; k >= 0; --k) {
      const float norm = __fdiv_rn(__fsub_rn(P[i * D + k], g.lo[k]), g.extent[k]);
      float c = __fmul_rn(norm, (float) g.size[k]);
      c = fminf(fmaxf(c, 0.0f), __fsub_rn((float) g.size[k], 1.0f));
      cell = cell * g.size[k] + (uint32_t) c;
    }
    atomicAdd(&counts[cell], 1u);
  }
}

// Largest count and number of non-empty cells.
__global__ void k_stats_reduce(const uint32_t* __restrict__ counts, uint64_t cells,
                               uint32_t* __restrict__ out) {
  uint32_t mx = 0, ne = 0;
  for (uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < cells;
       i += (uint64_t) gridDim.x * blockDim.x) {
    const uint32_t c = counts[i];
    mx = max(mx, c);
    ne += c ? 1u : 0u;
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    mx = max(mx, __shfl_xor_sync(0xFFFFFFFFu, mx, o));
    ne += __shfl_xor_sync(0xFFFFFFFFu, ne, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(&out[0], mx);
    atomicAdd(&out[1], ne);
  }
}

__global__ void k_stats_hist(const uint32_t* __restrict__ counts, uint64_t cells, uint32_t nbins,
                             uint32_t* __restrict__ hist) {
  for (uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < cells;
       i += (uint64_t) gridDim.x * blockDim.x) {
    const uint32_t c = counts[i];
    if (c) atomicAdd(&hist[min(c, nbins - 1)], 1u);
  }
}

}  // namespace
}  // namespace hdg

using namespace hdg;

extern "C" hd_status hd_compute_stats(hd_ctx* c, const float* P, uint64_t n, int n_dims,
                                    uint32_t n_points_cell, uint32_t flags, hd_point_stats* out) {
  if (!c) return HD_ERR_INVALID_ARG;
  c->last_error.clear();
  if (!P || !out || n == 0) return fail(*c, HD_ERR_INVALID_ARG, "null pointer or empty set");
  if (n_dims != 2 && n_dims != 3)
    return fail(*c, HD_ERR_UNSUPPORTED, "point statistics need n_dims 2 or 3");
  if (n_points_cell == 0) return fail(*c, HD_ERR_INVALID_ARG, "n_points_cell must be positive");
  if (flags & ~HD_DEVICE_PTRS) return fail(*c, HD_ERR_INVALID_ARG, "unknown flag bits");
  cudaSetDevice(c->device);
  memset(out, 0, sizeof(*out));
  out->n_dims = n_dims;
  out->n_points_cell = n_points_cell;
  out->n_points = n;
  hd_status s;
  cudaError_t e;
  const float* dP = P;
  if (!(flags & HD_DEVICE_PTRS)) {
    void* p;
    if ((s = ensure(*c, kBufA, (size_t) n * n_dims * 4, &p)) != HD_OK) return s;
    if ((e = cudaMemcpyAsync(p, P, (size_t) n * n_dims * 4, cudaMemcpyHostToDevice, c->stream)) !=
        cudaSuccess)
      return cuda_fail(*c, e, "copy points");
    dP = (const float*) p;
  }
  void* sv;
  if ((s = ensure(*c, kBufSample, 64, &sv)) != HD_OK) return s;
  uint32_t* small = (uint32_t*) sv;
  uint32_t init[16];
  for (int k = 0; k < 4; ++k) {
    init[k] = 0xFFFFFFFFu;
    init[4 + k] = 0u;
  }
  for (int k = 8; k < 16; ++k) init[k] = 0u;
  if ((e = cudaMemcpyAsync(small, init, sizeof(init), cudaMemcpyHostToDevice, c->stream)) !=
      cudaSuccess)
    return cuda_fail(*c, e, "stats init");
  const unsigned g = (unsigned) std::max<uint64_t>(
      1, std::min<uint64_t>((n + 255) / 256, (uint64_t) c->num_sms * 8));
  cudaEvent_t t0 = c->ev[24], t1 = c->ev[25];
  cudaEventRecord(t0, c->stream);
  if (n_dims == 2)
    k_stats_mbr<2><<<g, 256, 0, c->stream>>>(dP, n, small);
  else
    k_stats_mbr<3><<<g, 256, 0, c->stream>>>(dP, n, small);
  if ((s = after_launch(*c, "stats_mbr")) != HD_OK) return s;
  uint32_t ord[8];
  if ((e = cudaMemcpyAsync(ord, small, sizeof(ord), cudaMemcpyDeviceToHost, c->stream)) !=
          cudaSuccess ||
      (e = cudaStreamSynchronize(c->stream)) != cudaSuccess)
    return cuda_fail(*c, e, "stats box");
  // The reference's grid shape on its non-empty box, in its arithmetic
  // (hd_stats_host.h).
  float lo32[3], hi32[3];
  for (int k = 0; k < n_dims; ++k) {
    lo32[k] = ord2f(ord[k]);
    hi32[k] = ord2f(ord[4 + k]);
  }
  stats::GridShape shape;
  if (!stats::grid_shape(lo32, hi32, n_dims, n, n_points_cell, kStatsMaxCells, &shape))
    return fail(*c, HD_ERR_UNSUPPORTED, "statistics grid too large");
  StatsGrid grid{};
  for (int k = 0; k < n_dims; ++k) {
    out->lower[k] = shape.lower[k];
    out->upper[k] = shape.upper[k];
    out->grid_size[k] = shape.size[k];
    grid.size[k] = shape.size[k];
    grid.lo[k] = shape.lower[k];
    grid.extent[k] = shape.extent[k];
  }
  const uint64_t cells = shape.total_cells;
  out->density = shape.density;
  out->total_cells = cells;
  out->cell_diagonal = shape.cell_diagonal;
  void* cv;
  if ((s = ensure(*c, kBufKeys, cells * 4, &cv)) != HD_OK) return s;
  uint32_t* counts = (uint32_t*) cv;
  if ((e = cudaMemsetAsync(counts, 0, cells * 4, c->stream)) != cudaSuccess)
    return cuda_fail(*c, e, "stats counts");
  if (n_dims == 2)
    k_stats_count<2><<<g, 256, 0, c->stream>>>(dP, n, grid, counts);
  else
    k_stats_count<3><<<g, 256, 0, c->stream>>>(dP, n, grid, counts);
  if ((s = after_launch(*c, "stats_count")) != HD_OK) return s;
  const unsigned gc = (unsigned) std::max<uint64_t>(
      1, std::min<uint64_t>((cells + 255) / 256, (uint64_t) c->num_sms * 8));
  k_stats_reduce<<<gc, 256, 0, c->stream>>>(counts, cells, small + 8);
  if ((s = after_launch(*c, "stats_reduce")) != HD_OK) return s;
  cudaEventRecord(t1, c->stream);
  uint32_t red[2];
  if ((e = cudaMemcpyAsync(red, small + 8, sizeof(red), cudaMemcpyDeviceToHost, c->stream)) !=
          cudaSuccess ||
      (e = cudaStreamSynchronize(c->stream)) != cudaSuccess)
    return cuda_fail(*c, e, "stats reduce");
  float ms = 0.0f;
  if (cudaEventElapsedTime(&ms, t0, t1) == cudaSuccess) out->build_ms = ms;
  out->max_points = red[0];
  out->nonempty_cells = red[1];
  const uint32_t nbins = (uint32_t) std::min<uint64_t>((uint64_t) red[0] + 1, kStatsMaxHist);
  void* hv;
  if ((s = ensure(*c, kBufVals, (size_t) nbins * 4, &hv)) != HD_OK) return s;
  if ((e = cudaMemsetAsync(hv, 0, (size_t) nbins * 4, c->stream)) != cudaSuccess)
    return cuda_fail(*c, e, "stats histogram");
  k_stats_hist<<<gc, 256, 0, c->stream>>>(counts, cells, nbins, (uint32_t*) hv);
  if ((s = after_launch(*c, "stats_hist")) != HD_OK) return s;
  std::vector<uint32_t> hist(nbins);
  if ((e = cudaMemcpyAsync(hist.data(), hv, (size_t) nbins * 4, cudaMemcpyDeviceToHost,
                           c->stream)) != cudaSuccess ||
      (e = cudaStreamSynchronize(c->stream)) != cudaSuccess)
    return cuda_fail(*c, e, "stats histogram");
  // Gini index over the non-empty cells' counts in ascending order
  // (sum_i (2i - m + 1) v_i / (m * total), running_stats.h:33-62); values of
  // equal count occupy consecutive ranks, so each histogram bin adds its
  // value times the sum of its ranks' weights.
  const double m = (double) out->nonempty_cells;
  double total = 0.0, weighted = 0.0, rank = 0.0;
  uint32_t median = 0;
  const uint64_t median_rank = out->nonempty_cells / 2;
  for (uint32_t v = 1; v < nbins; ++v) {
    const double cnt = hist[v];
    if (cnt == 0) continue;
    const double w = cnt * (2.0 * rank + cnt - 1.0) - cnt * (m - 1.0);
    weighted += w * v;
    total += cnt * v;
    if ((uint64_t) rank <= median_rank && median_rank < (uint64_t) (rank + cnt)) median = v;
    rank += cnt;
  }
  out->gini_index = (m > 0 && total > 0) ? weighted / (m * total) : 0.0;
  out->median_points = median;
  // The percentile table as the reference's HdrHistogram prints it.
  const auto rows = stats::hdr_percentiles(hist.data(), nbins, out->nonempty_cells, 3);
  out->n_hist = (uint32_t) std::min<size_t>(rows.size(), HD_STATS_HIST_ROWS);
  for (uint32_t r = 0; r < out->n_hist; ++r) {
    out->hist_value[r] = rows[r].value;
    out->hist_percentile[r] = rows[r].percentile;
    out->hist_count[r] = rows[r].count;
  }
  return HD_OK;
}
