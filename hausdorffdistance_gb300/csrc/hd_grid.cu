// Grid variant: a uniform grid over B read straight off the Morton sort, and
// a ring-expanding cell search per A point with early break.
//
// Replaces the reference's uniform grid (src/index/uniform_grid.h:222-244
// resolution, :343-484 insert, :542-589 tight cell boxes) and its use as the
// RT search's primitive set (hausdorff_distance_hybrid.h:203-227).
//
// Build: in B's cubic Morton frame, grid level g groups 2^g x 2^g
// (x 2^g) finest Morton cells into one grid cell, so a grid cell is a
// contiguous run of the Morton-sorted points — no counting, scan or scatter.
// The level follows the reference's resolution rule (cell side s =
// (volume * k / n)^(1/d), uniform_grid.h:222-244) rounded to a power of two,
// capped at 2^24 cells.  A dense table gives each cell its [start, end) run;
// 0xFFFFFFFF marks an empty cell.  Cell boxes are the regular cells widened
// by a few ulps of the frame (the reference pads with nextafter,
// uniform_grid.h:106-128) so every point lies inside its cell's box.
//
// Query (one thread per A point, points in Morton order so neighbouring
// threads search neighbouring cells): rings r = 0, 1, 2, ... of cells around
// the point's cell.  A cell is scanned only if its box is nearer than the
// running minimum; the point stops early once some B point is within the
// running maximum, and stops exactly once a whole ring's nearest box is no
// nearer than the running minimum (box distances only grow with r).  Points
// that need more rings than a fixed budget are finished by a CTA-per-point
// scan over B.
#include <cfloat>

#include "hd_common.cuh"
#include "hd_internal.h"

namespace hdg {
namespace {

struct GridParams {
  float lo[3];
  float side;      // cell side (frame units)
  float eps;       // box widening
  uint32_t g;      // level: Morton bits per axis dropped
  uint32_t cpa;    // cells per axis
  uint32_t shift;  // d * g
  uint32_t ncells;
  uint32_t mask;   // the target set's sorted code bits
  uint32_t pad[2];
};

constexpr uint32_t kMaxCells = 1u << 24;

__device__ __forceinline__ uint32_t compact2(uint32_t x) {
  x &= 0x55555555u;
  x = (x | (x >> 1)) & 0x33333333u;
  x = (x | (x >> 2)) & 0x0F0F0F0Fu;
  x = (x | (x >> 4)) & 0x00FF00FFu;
  x = (x | (x >> 8)) & 0x0000FFFFu;
  return x;
}
__device__ __forceinline__ uint32_t compact3(uint32_t x) {
  x &= 0x09249249u;
  x = (x | (x >> 2)) & 0x030C30C3u;
  x = (x | (x >> 4)) & 0x0300F00Fu;
  x = (x | (x >> 8)) & 0x030000FFu;
  x = (x | (x >> 16)) & 0x000003FFu;
  return x;
}

__global__ void k_grid_params(const Frame* __restrict__ fr, const uint32_t* __restrict__ ordB,
                              uint64_t nB, int dims, uint32_t k, int low_bits, GridParams* gp) {
  if (threadIdx.x != 0) return;
  const int bits = fr->bits;
  // Reference resolution rule on B's own box (zero extents -> 1e-5,
  // mbr.h:288-296).
  double vol = 1.0;
  for (int d = 0; d < dims; ++d) {
    double e = (double) ord2f(ordB[4 + d]) - (double) ord2f(ordB[d]);
    vol *= e > 0.0 ? e : 1e-5;
  }
  double s = pow(vol * (double) k / (double) nB, 1.0 / dims);
  const double fine = fr->scale > 0.0f ? 1.0 / (double) fr->scale : 1.0;
  int g = (int) floor(log2(fmax(s / fine, 1.0)) + 0.5);
  const int cap_bits = dims == 2 ? 12 : 8;  // cells per axis <= 2^(24/d)
  g = max(g, bits - cap_bits);
  // A cell must be a run of the sort: its code drops every unsorted bit.
  g = max(g, (low_bits + dims - 1) / dims);
  g = min(max(g, 0), bits);
  gp->g = (uint32_t) g;
  gp->shift = (uint32_t) (dims * g);
  gp->cpa = 1u << (bits - g);
  gp->ncells = dims == 2 ? gp->cpa * gp->cpa : gp->cpa * gp->cpa * gp->cpa;
  gp->mask = sorted_mask(low_bits);
  gp->side = (float) ((double) (1u << g) * fine);
  for (int d = 0; d < 3; ++d) gp->lo[d] = fr->lo[d];
  float mag = 0.0f;
  for (int d = 0; d < 3; ++d) mag = fmaxf(mag, fmaxf(fabsf(fr->lo[d]), fabsf(fr->hi[d])));
  gp->eps = 4e-6f * (fr->extent + mag) + 1e-30f;
}

__global__ void k_grid_clear(const GridParams* __restrict__ gp, uint2* __restrict__ table) {
  const uint32_t n = gp->ncells;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    table[i] = make_uint2(0xFFFFFFFFu, 0u);
}

__device__ __forceinline__ uint32_t cell_linear(uint32_t cellcode, int dims, uint32_t cpa) {
  if (dims == 2) return compact2(cellcode) + cpa * compact2(cellcode >> 1);
  return compact3(cellcode) + cpa * (compact3(cellcode >> 1) + cpa * compact3(cellcode >> 2));
}

__global__ void k_grid_runs(const uint32_t* __restrict__ codes, uint64_t n, int dims,
                            const GridParams* __restrict__ gp, uint2* __restrict__ table) {
  const uint32_t shift = gp->shift, cpa = gp->cpa, mask = gp->mask;
  for (uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < n;
       i += (uint64_t) gridDim.x * blockDim.x) {
    const uint32_t c = (codes[i] & mask) >> shift;
    const bool first = i == 0 || ((codes[i - 1] & mask) >> shift) != c;
    const bool last = i + 1 == n || ((codes[i + 1] & mask) >> shift) != c;
    if (first || last) {
      const uint32_t lin = cell_linear(c, dims, cpa);
      if (first) table[lin].x = (uint32_t) i;
      if (last) table[lin].y = (uint32_t) (i + 1);
    }
  }
}

// Squared distance from p to a cell box, rounded like the pair formula
// (monotone, so never above the FP32 distance to a point inside the box).
template <int D>
__device__ __forceinline__ float cell_d2(const float* p, const int* c, const GridParams& gp) {
  float s = 0.0f;
#pragma unroll
  for (int k = 0; k < D; ++k) {
    const float lo = __fadd_rn(__fmaf_rn((float) c[k], gp.side, gp.lo[k]), -gp.eps);
    const float hi = __fadd_rn(__fmaf_rn((float) (c[k] + 1), gp.side, gp.lo[k]), gp.eps);
    const float d = fmaxf(fmaxf(__fsub_rn(lo, p[k]), __fsub_rn(p[k], hi)), 0.0f);
    const float q = __fmul_rn(d, d);
    s = k == 0 ? q : __fadd_rn(s, q);
  }
  return s;
}

struct Deferred {
  uint32_t qpos;  // position in the sorted query set
  float cmin;
};

template <int D, bool COUNT>
__global__ void __launch_bounds__(128)
    k_grid_query(const float4* __restrict__ Q, const Frame* __restrict__ tframe, uint64_t nQ,
                 const float4* __restrict__ B, const uint2* __restrict__ table,
                 const GridParams* __restrict__ gpp, int ring_cap, uint32_t pstride, int phase,
                 DevScalars* sc, Deferred* __restrict__ deferred, uint32_t* defer_count) {
  const GridParams gp = *gpp;
  const uint64_t t = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x;
  // Phase 0 takes every pstride-th warp-sized group of queries (a coherent
  // sample spread over the set), phase 1 the others.
  const uint64_t grp = t >> 5, lane = t & 31;
  uint64_t g2 = phase == 0 ? grp * pstride : grp + grp / (pstride - 1) + 1;
  const uint64_t i = g2 * 32 + lane;
  if (i >= nQ) return;
  const float4 q4 = Q[i];
  const float p[3] = {q4.x, q4.y, q4.z};
  // Home cell: the point's cell in the target set's frame at the grid level
  // (points outside that frame start from its border cells).
  const Frame tf = *tframe;
  const uint32_t maxq = (1u << tf.bits) - 1u;
  int home[3];
  home[0] = (int) (frame_quant(p[0], tf.lo[0], tf.scale, maxq) >> gp.g);
  home[1] = (int) (frame_quant(p[1], tf.lo[1], tf.scale, maxq) >> gp.g);
  home[2] = D == 3 ? (int) (frame_quant(p[2], tf.lo[2], tf.scale, maxq) >> gp.g) : 0;
  const int cpa = (int) gp.cpa;
  float cmin = INFINITY;
  float thr = threshold_of(ld_relaxed_u64(&sc->max_key));
  unsigned long long pairs = 0, cells = 0;
  bool done = false, exact = false;
  int r = 0;
  for (; r <= ring_cap && !done; ++r) {
    float ring_min = INFINITY;
    bool any_cell = false;
    const int zlo = D == 3 ? -r : 0, zhi = D == 3 ? r : 0;
    for (int dz = zlo; dz <= zhi && !done; ++dz) {
      const int cz = home[2] + dz;
      if (D == 3 && (cz < 0 || cz >= cpa)) continue;
      for (int dy = -r; dy <= r && !done; ++dy) {
        const int cy = home[1] + dy;
        if (cy < 0 || cy >= cpa) continue;
        const bool face = (dz == -r || dz == r || dy == -r || dy == r) && (D == 3 || dy == -r || dy == r);
        // On a face row every dx is in the ring; otherwise only dx = +-r.
        const int step = (face || r == 0) ? 1 : 2 * r;
        for (int dx = -r; dx <= r; dx += step) {
          const int cx = home[0] + dx;
          if (cx < 0 || cx >= cpa) continue;
          any_cell = true;
          const int c[3] = {cx, cy, cz};
          const float bd = cell_d2<D>(p, c, gp);
          ring_min = fminf(ring_min, bd);
          if (!(bd < cmin)) continue;
          const uint32_t lin = D == 2 ? (uint32_t) (cx + cpa * cy)
                                      : (uint32_t) (cx + cpa * (cy + cpa * cz));
          const uint2 run = table[lin];
          if (COUNT) ++cells;
          if (run.x == 0xFFFFFFFFu) continue;
          // The early break is tested after every point: a cell can hold a
          // very long run (many copies of one point, dense cluster cores).
          uint32_t j = run.x;
          while (j < run.y) {
            const float4 b = B[j++];
            const float d = D == 2 ? d2_2(p[0], p[1], b.x, b.y)
                                   : d2_3(p[0], p[1], p[2], b.x, b.y, b.z);
            cmin = fminf(cmin, d);
            if (cmin <= thr) break;
          }
          if (COUNT) pairs += j - run.x;
          if (cmin <= thr) {
            done = true;  // early break: cannot raise the maximum
            break;
          }
        }
      }
    }
    if (done) break;
    if (!any_cell || !(ring_min < cmin)) {
      // No cell left, or no cell of this or any later ring can hold a
      // strictly nearer point: cmin is the exact nearest distance.
      exact = true;
      done = true;
      break;
    }
    thr = threshold_of(ld_relaxed_u64(&sc->max_key));
    if (cmin <= thr) {
      done = true;
      break;
    }
  }
  if (exact) {
    atomicMax(&sc->max_key, pack_max(cmin, __float_as_uint(q4.w)));
  } else if (!done) {
    const uint32_t slot = atomicAdd(defer_count, 1u);
    deferred[slot] = Deferred{(uint32_t) i, cmin};
  }
  if (COUNT) {
    atomicAdd(&sc->pairs, pairs);
    atomicAdd(&sc->leaves, cells);
  }
}

// Deferred points: one CTA each, all threads over the sorted B, early break.
// The scan starts at the query's own position in B's Morton order (binary
// search of its code in B's frame) and grows outward in alternating forward and backward
// chunks, so the spatially nearest B points, which decide the early break,
// come first; a point that does not break still visits every B point.
template <int D>
__global__ void __launch_bounds__(256)
    k_grid_deferred(const float4* __restrict__ Q, const Frame* __restrict__ tframe,
                    const float4* __restrict__ B, const uint32_t* __restrict__ bcodes, uint64_t nB,
                    uint32_t mask, const Deferred* __restrict__ list, const uint32_t* count,
                    DevScalars* sc) {
  __shared__ float red[8];
  __shared__ float s_thr;
  constexpr uint64_t kChunk = 256 * 64;
  const uint32_t n = *count;
  for (uint32_t e = blockIdx.x; e < n; e += gridDim.x) {
    const Deferred dfr = list[e];
    const float4 q = Q[dfr.qpos];
    const uint32_t code = frame_code<D>(*tframe, q.x, q.y, q.z) & mask;
    // First B position whose code is >= the query's (every thread finds the
    // same one).
    uint64_t lo = 0, hi = nB;
    while (lo < hi) {
      const uint64_t mid = (lo + hi) >> 1;
      if ((bcodes[mid] & mask) < code) lo = mid + 1;
      else hi = mid;
    }
    const uint64_t p0 = lo;
    float cmin = dfr.cmin;
    bool broke = false;
    // Chunk k: forward block k/2 = [p0 + (k/2) kChunk, +kChunk) for even k,
    // backward block k/2 = [p0 - (k/2 + 1) kChunk, p0 - (k/2) kChunk) for
    // odd k, clipped to [0, nB); together they cover [0, nB) once.
    for (uint64_t k = 0;; ++k) {
      const uint64_t f = k >> 1;
      uint64_t b0, b1;
      if ((k & 1) == 0) {
        b0 = p0 + f * kChunk;
        b1 = min(nB, b0 + kChunk);
      } else {
        const uint64_t back = f * kChunk;
        b1 = p0 > back ? p0 - back : 0;
        b0 = b1 > kChunk ? b1 - kChunk : 0;
      }
      const bool fwd_left = p0 + f * kChunk < nB;
      const bool bwd_left = p0 > f * kChunk;
      if (!fwd_left && !bwd_left) break;
      float m = INFINITY;
      for (uint64_t j = b0 + threadIdx.x; j < b1; j += 256) {
        const float4 b = B[j];
        m = fminf(m, D == 2 ? d2_2(q.x, q.y, b.x, b.y) : d2_3(q.x, q.y, q.z, b.x, b.y, b.z));
      }
#pragma unroll
      for (int o = 16; o; o >>= 1) m = fminf(m, __shfl_xor_sync(0xFFFFFFFFu, m, o));
      if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
      if (threadIdx.x == 0) s_thr = threshold_of(ld_relaxed_u64(&sc->max_key));
      __syncthreads();
      for (int w = 0; w < 8; ++w) cmin = fminf(cmin, red[w]);
      const float thr = s_thr;
      __syncthreads();
      if (cmin <= thr) {
        broke = true;
        break;
      }
    }
    if (!broke && threadIdx.x == 0) atomicMax(&sc->max_key, pack_max(cmin, __float_as_uint(q.w)));
  }
}

}  // namespace

hd_status run_grid(Ctx& c, const DirInput& in) {
  if (in.dims != 2 && in.dims != 3) return fail(c, HD_ERR_UNSUPPORTED, "grid needs n_dims 2 or 3");
  hd_status s;
  const SortedSet *q, *t;
  if ((s = spatial_prepare(c, in, &q, &t)) != HD_OK) return s;
  mark(c, 1);
  DevScalars* sc = scalars(c, in.dir);
  void *gpv, *table, *defl;
  if ((s = ensure(c, kBufAux2, sizeof(GridParams) + 16, &gpv)) != HD_OK) return s;
  if ((s = ensure(c, in.dir == 0 ? kBufNodes0 : kBufNodes1, (size_t) kMaxCells * sizeof(uint2),
                  &table)) != HD_OK)
    return s;
  if ((s = ensure(c, kBufHeavy, q->n * sizeof(Deferred) + 16, &defl)) != HD_OK) return s;
  GridParams* gp = (GridParams*) gpv;
  uint32_t* defer_count = (uint32_t*) ((char*) gpv + sizeof(GridParams));
  // The set this grid indexes is the call's A for direction 1, B otherwise.
  const uint32_t* ordT = &scalars(c, 0)->mbr_ord[t == &c.sorted[0] ? 0 : 1][0][0];
  const uint32_t k = c.opt.n_points_cell ? c.opt.n_points_cell : 8;
  k_grid_params<<<1, 32, 0, c.stream>>>(t->frame, ordT, t->n, in.dims, k, t->low_bits, gp);
  if ((s = after_launch(c, "grid_params")) != HD_OK) return s;
  cudaError_t e = cudaMemsetAsync(defer_count, 0, 4, c.stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "memset");
  k_grid_clear<<<c.num_sms * 8, 256, 0, c.stream>>>(gp, (uint2*) table);
  if ((s = after_launch(c, "grid_clear")) != HD_OK) return s;
  {
    int grid = (int) std::min<uint64_t>((t->n + 255) / 256, (uint64_t) c.num_sms * 16);
    k_grid_runs<<<std::max(grid, 1), 256, 0, c.stream>>>(t->codes, t->n, in.dims, gp,
                                                        (uint2*) table);
    if ((s = after_launch(c, "grid_runs")) != HD_OK) return s;
  }
  mark(c, 2);
  const int ring_cap = in.dims == 2 ? 24 : 6;
  const uint64_t groups = (q->n + 31) / 32;
  const uint32_t pstride = groups >= 4096 ? 64 : (groups >= 256 ? 16 : 2);
  for (int phase = 0; phase < 2; ++phase) {
    const uint64_t ng = phase == 0 ? (groups + pstride - 1) / pstride
                                   : groups - (groups + pstride - 1) / pstride;
    if (ng == 0) {
      mark(c, 3);
      continue;
    }
    const unsigned blocks = (unsigned) ((ng * 32 + 127) / 128);
    if (in.dims == 2) {
      if (in.count)
        k_grid_query<2, true><<<blocks, 128, 0, c.stream>>>(
            q->pts, t->frame, q->n, t->pts, (const uint2*) table, gp, ring_cap, pstride, phase, sc,
            (Deferred*) defl, defer_count);
      else
        k_grid_query<2, false><<<blocks, 128, 0, c.stream>>>(
            q->pts, t->frame, q->n, t->pts, (const uint2*) table, gp, ring_cap, pstride, phase, sc,
            (Deferred*) defl, defer_count);
    } else {
      if (in.count)
        k_grid_query<3, true><<<blocks, 128, 0, c.stream>>>(
            q->pts, t->frame, q->n, t->pts, (const uint2*) table, gp, ring_cap, pstride, phase, sc,
            (Deferred*) defl, defer_count);
      else
        k_grid_query<3, false><<<blocks, 128, 0, c.stream>>>(
            q->pts, t->frame, q->n, t->pts, (const uint2*) table, gp, ring_cap, pstride, phase, sc,
            (Deferred*) defl, defer_count);
    }
    if ((s = after_launch(c, "grid_query")) != HD_OK) return s;
    if (phase == 0) mark(c, 3);
  }
  mark(c, 4);
  if (in.dims == 2)
    k_grid_deferred<2><<<c.num_sms * 2, 256, 0, c.stream>>>(q->pts, t->frame, t->pts, t->codes, t->n,
                                                           t->mask, (const Deferred*) defl,
                                                           defer_count, sc);
  else
    k_grid_deferred<3><<<c.num_sms * 2, 256, 0, c.stream>>>(q->pts, t->frame, t->pts, t->codes, t->n,
                                                           t->mask, (const Deferred*) defl,
                                                           defer_count, sc);
  if ((s = after_launch(c, "grid_deferred")) != HD_OK) return s;
  return certify(c, in);
}

}  // namespace hdg
