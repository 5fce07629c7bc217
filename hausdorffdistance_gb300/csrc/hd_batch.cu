// Batched Hausdorff distances: many independent 2-D / 3-D problems of uneven
// sizes in one CUDA-graph launch.  No counterpart in the reference, which
// solves one pair per hd_exec run; the per-problem baseline
// (hd_solve_batch_plain) runs the plain early-break solve once per problem
// with its own launches.
//
// Work decomposition.  A problem-direction (problem p, A->B or B->A) is cut
// into items of 32 query rows; one warp processes one item, one lane per
// row.  Items are ordered largest problem first (longest-processing-time
// order over |A|*|B|, computed on the device by a radix sort inside the
// graph).  Warps take chunks of consecutive items in grid-stride order and
// walk from item to item, so the item -> problem lookup is one binary search
// per chunk.  The graph runs:
//   plan:   sort keys, radix sort, item counts, exclusive scan;
//   window: every row takes the minimum over a few points of the other set
//           around its relative position (row * |Y| / |X|), an upper bound on
//           its nearest-neighbour distance, stored per row; per
//           problem-direction the row with the largest bound in each residue
//           class (row mod 8) is kept;
//   seed:   the exact nearest-neighbour distances of those 8 rows, computed
//           over stripes of the other set by all items of the
//           problem-direction; between them the 8 rows nearly always contain
//           the maximiser, so the sweep starts at or near the final
//           threshold;
//   fold:   the seed minima start each running maximum;
//   sweep:  a row whose window bound is at or below the running maximum is
//           settled by that one read; the others scan the other set
//           circularly on from their window with early break; a row still
//           open after kShortScan pairs is queued;
//   long:   one warp per queued row finishes its scan (lanes split the other
//           set, early break by warp vote);
//   certify, finalize.
//
// A row that completes its scan raises its problem's running maximum with
// one 64-bit atomicMax (distance bits, ~row).  Squared distances use the
// reference formula, so results are bit-identical to the single-problem
// solve.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include "hd_common.cuh"
#include "hd_internal.h"
#include "hd_tuning.h"

namespace hdg {
namespace {

constexpr int kBatchThreads = 256;
constexpr int kCheckEvery = 8;   // pairs between early-break checks of a row
constexpr int kShortScan = 64;   // pairs a row scans alone before it is queued
constexpr int kSlots = 8;        // seed rows per problem-direction (row mod 8)
constexpr int kLongIlp = 8;      // independent loads per lane per long-pass round
constexpr int kSmallMax = 65536; // largest one-warp threshold accepted
constexpr int kBestFirst = 32;    // one-warp path: exact best-first scans before the sweep
constexpr uint32_t kPipeRows = 65536;  // directions above this many rows use the multi-pass pipeline
constexpr int kSeedGroup = 8;    // items per seed stripe
constexpr uint64_t kLongCap = 1ull << 21;  // queued long rows at most
constexpr uint32_t kNoSeed = 0xFFFFFFFFu;  // empty seed minimum (above every float)

enum Pass : int { kPassWindow = 0, kPassSeed = 1, kPassSweep = 2 };

struct PD {
  float d2;
  uint32_t ia, ib;
  uint32_t valid;
};

// A row whose short scan did not settle it: problem, direction, row, the
// circular position its scan reached and its running minimum.
struct LongRow {
  uint32_t p, d, row, j;
  float cmin;
  uint32_t pad[3];
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

__device__ __host__ __forceinline__ uint64_t items_of(uint64_t n) { return (n + 31) / 32; }

// Items of a direction whose query set has nx rows in the multi-pass
// pipeline: directions of at most pipe_rows rows go to the CTA or one-warp
// path.
__device__ __host__ __forceinline__ uint64_t large_items(uint64_t nx, uint32_t pipe_rows) {
  return nx > (uint64_t) pipe_rows ? items_of(nx) : 0;
}

// Walks the items of the multi-pass pipeline in plan order: (sorted problem
// rank r, direction d, item number within the direction), skipping the
// directions of the one-warp path.  init() is one binary search over the
// item prefix; next() steps to the following item.  Problems with an item
// come first in plan order, so next() never has to skip a problem.
struct Cursor {
  const hd_problem* probs;
  const uint32_t* order;
  uint32_t nprob;
  int ndir;
  uint32_t pipe_rows;  // directions above this many rows are the pipeline's items
  uint32_t r, p;
  int d;
  uint64_t item, nitems, it0, it1;
  hd_problem pr;

  __device__ void load(uint32_t rank) {
    r = rank;
    p = order[rank];
    pr = probs[p];
    it0 = large_items(pr.n_a, pipe_rows);
    it1 = ndir == 2 ? large_items(pr.n_b, pipe_rows) : 0;
  }
  __device__ void init(uint64_t w, const uint64_t* __restrict__ prefix) {
    uint32_t lo = 0, hi = nprob;  // prefix[lo] <= w < prefix[hi]
    while (hi - lo > 1) {
      const uint32_t mid = (lo + hi) >> 1;
      if (prefix[mid] <= w)
        lo = mid;
      else
        hi = mid;
    }
    load(lo);
    const uint64_t local = w - prefix[lo];
    if (local < it0) {
      d = 0;
      item = local;
      nitems = it0;
    } else {
      d = 1;
      item = local - it0;
      nitems = it1;
    }
  }
  __device__ void next() {
    if (++item < nitems) return;
    item = 0;
    if (d == 0 && it1 > 0) {
      d = 1;
      nitems = it1;
    } else if (r + 1 < nprob) {
      load(r + 1);
      d = it0 > 0 ? 0 : 1;
      nitems = it0 > 0 ? it0 : it1;
    }
  }
  __device__ uint64_t pd() const { return 2 * (uint64_t) p + d; }
  __device__ uint64_t nx() const { return d == 0 ? pr.n_a : pr.n_b; }
  __device__ uint64_t ny() const { return d == 0 ? pr.n_b : pr.n_a; }
};

struct BatchArgs {
  const float* A;
  const float* B;
  const hd_problem* probs;
  const uint32_t* order;
  const uint64_t* prefix;  // item prefix over sorted ranks, nprob + 1 entries
  uint32_t nprob;
  int ndir;
  uint64_t total;                  // items
  unsigned long long* keys;        // running maximum per problem-direction
  unsigned long long* ubound;      // window bound per problem-direction and class
  uint32_t* smin;                  // seed minima (float bits) per problem-direction and class
  float* wb_a;                     // window bound per row of A (direction A->B)
  float* wb_b;                     // window bound per row of B (direction B->A)
  LongRow* longq;
  unsigned long long* long_count;
  uint64_t long_cap;
  uint32_t small_rows;             // one-warp path: directions up to this many rows
  uint32_t pipe_rows;              // CTA path up to this many rows; multi-pass pipeline above
  uint32_t n_big;                  // problems (first in plan order) with a direction above small_rows
  uint32_t chunk;                  // consecutive items per warp step
  uint32_t window;                 // half-width of the bound window
  PD* pd;                          // certified result per problem-direction
};

// First position of a row's circular scan: the start of the window of w0
// points centred on the row's relative position row * |Y| / |X| (computed in
// float: the position is only a starting point, any value in [0, ny) is
// correct).
__device__ __forceinline__ uint32_t scan_start(uint32_t row, float ratio, uint32_t ny,
                                               uint32_t half) {
  uint32_t c = (uint32_t) ((float) row * ratio);
  c = c < ny ? c : ny - 1;
  return c >= half ? c - half : c + (ny - half);
}

template <int D>
__device__ __forceinline__ void load_pt(const float* __restrict__ P, uint64_t i, float* v) {
  if constexpr (D == 2) {
    const float2 q = *reinterpret_cast<const float2*>(P + 2 * i);
    v[0] = q.x;
    v[1] = q.y;
  } else {
#pragma unroll
    for (int t = 0; t < D; ++t) v[t] = P[D * i + t];
  }
}

template <int D>
__device__ __forceinline__ float d2_of(const float* a, const float* b) {
  if constexpr (D == 2)
    return d2_2(a[0], a[1], b[0], b[1]);
  else
    return d2_3(a[0], a[1], a[2], b[0], b[1], b[2]);
}

// Minimum over `count` consecutive points of Y from position j (circular),
// starting from cmin; loads are issued in groups of 8 so that they overlap.
// j advances past the points scanned.
template <int D>
__device__ __forceinline__ float scan_run(const float* __restrict__ X, uint32_t row,
                                          const float* __restrict__ Y, uint32_t& j, uint32_t ny,
                                          uint32_t count, float cmin) {
  float x[D];
  load_pt<D>(X, row, x);
  if (j + (uint64_t) count <= ny) {
    // No wrap: consecutive points at fixed offsets from one base pointer.
    const float* yp = Y + (uint64_t) j * D;
    uint32_t k = 0;
    for (; k + 8 <= count; k += 8, yp += 8 * D) {
      float y[8][D];
#pragma unroll
      for (int u = 0; u < 8; ++u) load_pt<D>(yp, u, y[u]);
#pragma unroll
      for (int u = 0; u < 8; ++u) cmin = fminf(cmin, d2_of<D>(x, y[u]));
    }
    for (; k < count; ++k, yp += D) {
      float y[D];
      load_pt<D>(yp, 0, y);
      cmin = fminf(cmin, d2_of<D>(x, y));
    }
    j += count;
    if (j == ny) j = 0;
    return cmin;
  }
  uint32_t k = 0;
  for (; k + 8 <= count; k += 8) {
    float y[8][D];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      load_pt<D>(Y, j, y[u]);
      j = (j + 1 == ny) ? 0 : j + 1;
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) cmin = fminf(cmin, d2_of<D>(x, y[u]));
  }
  for (; k < count; ++k) {
    float y[D];
    load_pt<D>(Y, j, y);
    cmin = fminf(cmin, d2_of<D>(x, y));
    j = (j + 1 == ny) ? 0 : j + 1;
  }
  return cmin;
}

__device__ __forceinline__ float warp_min(float v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v = fminf(v, __shfl_xor_sync(0xFFFFFFFFu, v, o));
  return v;
}

// Window pass, one item: each row's minimum over 2*window+1 points of the
// other set centred on its relative position, stored per row; the largest
// bound (with its row) of each residue class goes to
// ubound[problem-direction][class].
template <int D>
__device__ __forceinline__ void window_item(const BatchArgs& a, const Cursor& cu, int lane,
                                            const float* X, const float* Y, uint32_t nx,
                                            uint32_t ny) {
  const uint32_t row = (uint32_t) cu.item * 32 + lane;
  const bool valid = row < nx;
  const uint32_t w0 = ny > 2 * a.window + 1 ? 2 * a.window + 1 : ny;
  float u = -1.0f;
  if (valid) {
    uint32_t j = scan_start(row, (float) ny / (float) nx, ny, w0 >> 1);
    u = scan_run<D>(X, row, Y, j, ny, w0, INFINITY);
  }
  if (valid) (cu.d == 0 ? a.wb_a + cu.pr.offset_a : a.wb_b + cu.pr.offset_b)[row] = u;
  // Row r's class is r % kSlots = lane % kSlots (items start at multiples of
  // 32): reduce over the lanes of a class, one atomicMax per class.
  unsigned long long kk = valid ? pack_max(u, row) : 0ull;
#pragma unroll
  for (int o = 16; o >= kSlots; o >>= 1) {
    const unsigned long long v = __shfl_xor_sync(0xFFFFFFFFu, kk, o);
    kk = v > kk ? v : kk;
  }
  if (lane < kSlots && kk) atomicMax(a.ubound + cu.pd() * kSlots + lane, kk);
}

// Seed pass: the items of a problem-direction form groups of kSeedGroup;
// the first item of group g of NG covers stripe [g*|Y|/NG, (g+1)*|Y|/NG) of
// the other set and lowers the seed rows' minima over that stripe.  The
// stripes partition the other set, so after the pass smin holds each seed
// row's exact nearest-neighbour distance.
template <int D>
__device__ __forceinline__ void seed_item(const BatchArgs& a, const Cursor& cu, int lane,
                                          const float* X, const float* Y, uint32_t nx,
                                          uint32_t ny) {
  if (cu.item % kSeedGroup) return;
  const uint64_t NG = (items_of(nx) + kSeedGroup - 1) / kSeedGroup;
  const uint64_t g = cu.item / kSeedGroup;
  const uint32_t lo = (uint32_t) (g * ny / NG), hi = (uint32_t) ((g + 1) * ny / NG);
  if (lo >= hi) return;
  const unsigned long long* ub = a.ubound + cu.pd() * kSlots;
  float x[kSlots][D];
  bool has[kSlots];
  float m[kSlots];
#pragma unroll
  for (int k = 0; k < kSlots; ++k) {
    const unsigned long long u = ub[k];
    has[k] = u != 0;
    const uint64_t r = has[k] ? unpack_max_index(u) : 0;  // an empty class repeats row 0
#pragma unroll
    for (int t = 0; t < D; ++t) x[k][t] = X[r * D + t];
    m[k] = INFINITY;
  }
#pragma unroll 4
  for (uint32_t j = lo + lane; j < hi; j += 32) {
    float y[D];
#pragma unroll
    for (int t = 0; t < D; ++t) y[t] = Y[(uint64_t) j * D + t];  // sets reach 2^32 - 2 points
#pragma unroll
    for (int k = 0; k < kSlots; ++k) {
      if constexpr (D == 2)
        m[k] = fminf(m[k], d2_2(x[k][0], x[k][1], y[0], y[1]));
      else
        m[k] = fminf(m[k], d2_3(x[k][0], x[k][1], x[k][2], y[0], y[1], y[2]));
    }
  }
  uint32_t* sm = a.smin + cu.pd() * kSlots;
#pragma unroll
  for (int k = 0; k < kSlots; ++k) {
    const float v = warp_min(m[k]);
    if (lane == k && has[k]) {
      const uint32_t bits = __float_as_uint(v);
      if (bits < *(volatile uint32_t*) (sm + k)) atomicMin(sm + k, bits);
    }
  }
}

// Fold: one thread per problem-direction starts the running maximum with the
// seed rows' exact minima.
__global__ void k_batch_fold(const unsigned long long* __restrict__ ubound,
                             const uint32_t* __restrict__ smin, uint64_t npd,
                             unsigned long long* __restrict__ keys) {
  const uint64_t t = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= npd) return;
  unsigned long long best = 0;
  for (int k = 0; k < kSlots; ++k) {
    const uint32_t bits = smin[t * kSlots + k];
    if (bits == kNoSeed) continue;
    const unsigned long long kk =
        pack_max(__uint_as_float(bits), unpack_max_index(ubound[t * kSlots + k]));
    best = kk > best ? kk : best;
  }
  if (best) keys[t] = best;  // one-warp directions have no seeds and keep their own key
}

// Sweep pass, one item: a row whose window bound is at or below the running
// maximum is settled without a pair; the others continue their circular scan
// after the window, up to kShortScan pairs in all; rows still open are queued
// for the long pass (or, with the queue full, finish alone).
template <int D>
__device__ __forceinline__ void sweep_item(const BatchArgs& a, const Cursor& cu, int lane,
                                           const float* X, const float* Y, uint32_t nx,
                                           uint32_t ny) {
  unsigned long long* key = a.keys + cu.pd();
  float thr = threshold_of(ld_relaxed_u64(key));
  const uint32_t row = (uint32_t) cu.item * 32 + lane;
  const bool valid = row < nx;
  float cmin = valid ? (cu.d == 0 ? a.wb_a + cu.pr.offset_a : a.wb_b + cu.pr.offset_b)[row]
                     : 0.0f;
  bool broke = !valid || cmin <= thr;
  if (__all_sync(0xFFFFFFFFu, broke)) return;
  const uint32_t w0 = ny > 2 * a.window + 1 ? 2 * a.window + 1 : ny;
  uint32_t j = 0;
  if (!broke) {
    j = scan_start(row, (float) ny / (float) nx, ny, w0 >> 1) + w0;
    if (j >= ny) j -= ny;
  }
  uint32_t step = w0;
  const uint32_t limit = ny < (uint32_t) kShortScan ? ny : (uint32_t) kShortScan;
  while (!broke && step < limit) {
    const uint32_t chunk = min((uint32_t) kCheckEvery, limit - step);
    cmin = scan_run<D>(X, row, Y, j, ny, chunk, cmin);
    step += chunk;
    broke = cmin <= thr;
  }
  if (!broke && step < ny) broke = cmin <= threshold_of(ld_relaxed_u64(key));
  const bool pending = !broke && step < ny;
  if (!broke && !pending) atomicMax(key, pack_max(cmin, row));
  const unsigned ballot = __ballot_sync(0xFFFFFFFFu, pending);
  if (!ballot) return;
  unsigned long long base = 0;
  if (lane == 0) base = atomicAdd(a.long_count, (unsigned long long) __popc(ballot));
  base = __shfl_sync(0xFFFFFFFFu, base, 0);
  if (!pending) return;
  const unsigned long long slot = base + __popc(ballot & ((1u << lane) - 1u));
  if (slot < a.long_cap) {
    a.longq[slot] = LongRow{cu.p, (uint32_t) cu.d, row, j, cmin, {0, 0, 0}};
    return;
  }
  // Queue full: this lane finishes the row itself.
  thr = threshold_of(ld_relaxed_u64(key));
  while (step < ny) {
    const uint32_t chunk = min((uint32_t) kCheckEvery, ny - step);
    for (uint32_t u = 0; u < chunk; ++u) {
      cmin = fminf(cmin, pt_d2<D>(X, row, Y, j));
      j = (j + 1 == ny) ? 0 : j + 1;
    }
    step += chunk;
    if (cmin <= thr) return;
    if ((step % 64) == 0) thr = threshold_of(ld_relaxed_u64(key));
  }
  atomicMax(key, pack_max(cmin, row));
}

template <int D, int PASS>
__global__ void __launch_bounds__(kBatchThreads, PASS == kPassSeed ? 3 : 4)
    k_batch_pass(BatchArgs a) {
  const int lane = threadIdx.x & 31;
  Cursor cu;
  cu.probs = a.probs;
  cu.order = a.order;
  cu.nprob = a.nprob;
  cu.ndir = a.ndir;
  cu.pipe_rows = a.pipe_rows;
  const uint64_t nw = (uint64_t) gridDim.x * (kBatchThreads / 32);
  for (uint64_t chunk = (uint64_t) blockIdx.x * (kBatchThreads / 32) + (threadIdx.x >> 5);
       chunk * a.chunk < a.total; chunk += nw) {
    const uint64_t base = chunk * a.chunk;
    const uint64_t end = min(base + a.chunk, a.total);
    cu.init(base, a.prefix);
    for (uint64_t w = base; w < end; ++w) {
      if (w > base) cu.next();
      const float* X = cu.d == 0 ? a.A + cu.pr.offset_a * D : a.B + cu.pr.offset_b * D;
      const float* Y = cu.d == 0 ? a.B + cu.pr.offset_b * D : a.A + cu.pr.offset_a * D;
      const uint32_t nx = (uint32_t) cu.nx(), ny = (uint32_t) cu.ny();
      if constexpr (PASS == kPassWindow)
        window_item<D>(a, cu, lane, X, Y, nx, ny);
      else if constexpr (PASS == kPassSeed)
        seed_item<D>(a, cu, lane, X, Y, nx, ny);
      else
        sweep_item<D>(a, cu, lane, X, Y, nx, ny);
    }
  }
}

// Long pass: one warp per queued row finishes its circular scan from the
// position the short scan reached, lanes splitting the remaining points,
// with a warp-wide early-break vote every 4 rounds.
template <int D>
__global__ void __launch_bounds__(kBatchThreads) k_batch_long(BatchArgs a) {
  const int lane = threadIdx.x & 31;
  const uint64_t nw = (uint64_t) gridDim.x * (kBatchThreads / 32);
  const uint64_t cnt = min((uint64_t) *(volatile unsigned long long*) a.long_count, a.long_cap);
  for (uint64_t e = (uint64_t) blockIdx.x * (kBatchThreads / 32) + (threadIdx.x >> 5); e < cnt;
       e += nw) {
    const LongRow L = a.longq[e];
    const hd_problem pr = a.probs[L.p];
    const float* X = L.d == 0 ? a.A + pr.offset_a * D : a.B + pr.offset_b * D;
    const float* Y = L.d == 0 ? a.B + pr.offset_b * D : a.A + pr.offset_a * D;
    const uint64_t ny = L.d == 0 ? pr.n_b : pr.n_a;
    unsigned long long* key = a.keys + 2 * (uint64_t) L.p + L.d;
    float thr = threshold_of(ld_relaxed_u64(key));
    float cmin = lane == 0 ? L.cmin : INFINITY;
    const uint64_t rem = ny - kShortScan;
    float x[D];
#pragma unroll
    for (int t = 0; t < D; ++t) x[t] = X[(uint64_t) L.row * D + t];
    // Rounds of kLongIlp independent loads per lane (32 * kLongIlp pairs per
    // warp), then one warp-wide early-break vote.
    bool broke = false;
    int round = 0;
    for (uint64_t t0 = 0; t0 < rem; t0 += 32 * kLongIlp) {
      float y[kLongIlp][D];
#pragma unroll
      for (int u = 0; u < kLongIlp; ++u) {
        const uint64_t t = t0 + (uint64_t) u * 32 + lane;
        uint64_t jj = L.j + t;  // L.j < ny and t < ny: one subtraction wraps
        if (jj >= ny) jj -= ny;
        if (t < rem) {
#pragma unroll
          for (int k = 0; k < D; ++k) y[u][k] = Y[jj * D + k];
        } else {
#pragma unroll
          for (int k = 0; k < D; ++k) y[u][k] = INFINITY;
        }
      }
#pragma unroll
      for (int u = 0; u < kLongIlp; ++u) {
        const uint64_t t = t0 + (uint64_t) u * 32 + lane;
        float d2;
        if constexpr (D == 2)
          d2 = d2_2(x[0], x[1], y[u][0], y[u][1]);
        else
          d2 = d2_3(x[0], x[1], x[2], y[u][0], y[u][1], y[u][2]);
        if (t < rem) cmin = fminf(cmin, d2);
      }
      if (warp_min(cmin) <= thr) {
        broke = true;
        break;
      }
      if ((++round & 7) == 0) thr = threshold_of(ld_relaxed_u64(key));
    }
    if (broke) continue;
    const float m = warp_min(cmin);
    if (lane == 0 && m > threshold_of(ld_relaxed_u64(key))) atomicMax(key, pack_max(m, L.row));
  }
}

// One-warp path: a warp solves a whole problem-direction of at most
// small_rows query rows with the same steps as the multi-pass pipeline —
// window bounds (stored per row and read back by the lane that wrote them),
// the 8 residue-class seeds, the sweep with early break, open rows scanned by
// the whole warp — with no pass boundary in between.  Warps take
// problem-directions in plan order.
template <int D>
__device__ __forceinline__ void small_direction(const BatchArgs& a, uint32_t p, int d,
                                                const hd_problem& pr, float* wb, int lane) {
  const float* X = d == 0 ? a.A + pr.offset_a * D : a.B + pr.offset_b * D;
  const float* Y = d == 0 ? a.B + pr.offset_b * D : a.A + pr.offset_a * D;
  const uint32_t nx = (uint32_t) (d == 0 ? pr.n_a : pr.n_b);
  const uint32_t ny = (uint32_t) (d == 0 ? pr.n_b : pr.n_a);
  const float ratio = (float) ny / (float) nx;
  const uint32_t w0 = ny > 2 * a.window + 1 ? 2 * a.window + 1 : ny;
  const uint32_t half = w0 >> 1;

  // Window bounds, one per row (an upper bound on the row's nearest-neighbour
  // distance); each row is read back only by the lane that wrote it.
  for (uint32_t row = lane; row < nx; row += 32) {
    uint32_t j = scan_start(row, ratio, ny, half);
    wb[row] = scan_run<D>(X, row, Y, j, ny, w0, INFINITY);
  }
  __syncwarp();

  // Best first: the row with the largest bound gets an exact scan (lanes
  // split the other set, early break once the row cannot raise the maximum),
  // then the next, until no bound exceeds the maximum — every other row is
  // then settled by its bound alone.  A scanned row's bound is set to -1.
  // After kBestFirst rows the sweep below settles the rest.
  unsigned long long best = 0;
  float thr = -1.0f;
  bool all_settled = false;
  for (int it = 0; it < kBestFirst; ++it) {
    unsigned long long cand = 0;
    for (uint32_t row = lane; row < nx; row += 32) {
      const float u = wb[row];
      if (u > thr) {
        const unsigned long long kk = pack_max(u, row);
        cand = kk > cand ? kk : cand;
      }
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      const unsigned long long v = __shfl_xor_sync(0xFFFFFFFFu, cand, o);
      cand = v > cand ? v : cand;
    }
    if (cand == 0) {
      all_settled = true;
      break;
    }
    const uint32_t r = unpack_max_index(cand);
    float xr[D];
#pragma unroll
    for (int t = 0; t < D; ++t) xr[t] = X[(uint64_t) r * D + t];
    float cm = __uint_as_float((uint32_t) (cand >> 32));  // its bound: a real distance
    bool broke = false;
    for (uint64_t t0 = 0; t0 < ny; t0 += 32 * kLongIlp) {
      float y[kLongIlp][D];
#pragma unroll
      for (int u = 0; u < kLongIlp; ++u) {
        const uint64_t jj = t0 + (uint64_t) u * 32 + lane;
#pragma unroll
        for (int k = 0; k < D; ++k) y[u][k] = jj < ny ? Y[jj * D + k] : INFINITY;
      }
#pragma unroll
      for (int u = 0; u < kLongIlp; ++u) {
        const uint64_t jj = t0 + (uint64_t) u * 32 + lane;
        float d2;
        if constexpr (D == 2)
          d2 = d2_2(xr[0], xr[1], y[u][0], y[u][1]);
        else
          d2 = d2_3(xr[0], xr[1], xr[2], y[u][0], y[u][1], y[u][2]);
        if (jj < ny) cm = fminf(cm, d2);
      }
      if (warp_min(cm) <= thr) {
        broke = true;
        break;
      }
    }
    if (!broke) {
      const unsigned long long kr = pack_max(warp_min(cm), r);
      if (kr > best) {
        best = kr;
        thr = threshold_of(best);
      }
    }
    if (lane == (int) (r & 31)) wb[r] = -1.0f;
    __syncwarp();
  }

  // Sweep.
  const uint32_t limit = ny < (uint32_t) kShortScan ? ny : (uint32_t) kShortScan;
  for (uint32_t row0 = 0; !all_settled && row0 < nx; row0 += 32) {
    const uint32_t row = row0 + lane;
    const bool valid = row < nx;
    float cmin = valid ? wb[row] : 0.0f;
    bool broke = !valid || cmin <= thr;
    if (__all_sync(0xFFFFFFFFu, broke)) continue;
    uint32_t j = 0;
    if (!broke) {
      j = scan_start(row, ratio, ny, half) + w0;
      if (j >= ny) j -= ny;
    }
    uint32_t step = w0;
    while (!broke && step < limit) {
      const uint32_t chunk = min((uint32_t) kCheckEvery, limit - step);
      cmin = scan_run<D>(X, row, Y, j, ny, chunk, cmin);
      step += chunk;
      broke = cmin <= thr;
    }
    const bool pending = !broke && step < ny;
    // Rows that completed their scan raise the maximum.
    unsigned long long kk = (!broke && !pending) ? pack_max(cmin, row) : 0ull;
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      const unsigned long long v = __shfl_xor_sync(0xFFFFFFFFu, kk, o);
      kk = v > kk ? v : kk;
    }
    if (kk > best) {
      best = kk;
      thr = threshold_of(best);
    }
    // Open rows: the whole warp finishes each in turn.
    unsigned open = __ballot_sync(0xFFFFFFFFu, pending);
    while (open) {
      const int src = __ffs(open) - 1;
      open &= open - 1;
      const uint32_t r = __shfl_sync(0xFFFFFFFFu, row, src);
      const uint32_t js = __shfl_sync(0xFFFFFFFFu, j, src);
      float c = __shfl_sync(0xFFFFFFFFu, cmin, src);
      if (c <= thr) continue;
      float xr[D];
#pragma unroll
      for (int t = 0; t < D; ++t) xr[t] = X[(uint64_t) r * D + t];
      const uint64_t rem = ny - kShortScan;
      float cm = INFINITY;
      bool done = false;
      for (uint64_t t0 = 0; t0 < rem; t0 += 32 * kLongIlp) {
        float y[kLongIlp][D];
#pragma unroll
        for (int u = 0; u < kLongIlp; ++u) {
          const uint64_t t = t0 + (uint64_t) u * 32 + lane;
          uint64_t jj = js + t;  // js < ny and t < ny: one subtraction wraps
          if (jj >= ny) jj -= ny;
#pragma unroll
          for (int k = 0; k < D; ++k) y[u][k] = t < rem ? Y[(uint64_t) jj * D + k] : INFINITY;
        }
#pragma unroll
        for (int u = 0; u < kLongIlp; ++u) {
          const uint64_t t = t0 + (uint64_t) u * 32 + lane;
          float d2;
          if constexpr (D == 2)
            d2 = d2_2(xr[0], xr[1], y[u][0], y[u][1]);
          else
            d2 = d2_3(xr[0], xr[1], xr[2], y[u][0], y[u][1], y[u][2]);
          if (t < rem) cm = fminf(cm, d2);
        }
        if (fminf(c, warp_min(cm)) <= thr) {
          done = true;
          break;
        }
      }
      if (done) continue;
      c = fminf(c, warp_min(cm));
      const unsigned long long kr = pack_max(c, r);
      if (kr > best) {
        best = kr;
        thr = threshold_of(best);
      }
    }
  }
  // Certification here, where the rows are at hand: the argmin of the
  // certifying row (lowest index among ties), as k_batch_certify does for
  // the pipeline's directions.
  const uint32_t rc = unpack_max_index(best);
  float xc[D];
  load_pt<D>(X, rc, xc);
  unsigned long long am = ~0ull;
#pragma unroll 4
  for (uint32_t j = lane; j < ny; j += 32) {
    float y[D];
    load_pt<D>(Y, j, y);
    const unsigned long long k = pack_min(d2_of<D>(xc, y), j);
    am = k < am ? k : am;
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    const unsigned long long v = __shfl_xor_sync(0xFFFFFFFFu, am, o);
    am = v < am ? v : am;
  }
  if (lane == 0) {
    a.keys[2 * (uint64_t) p + d] = best;
    const bool ok = (uint32_t) (am >> 32) == (uint32_t) (best >> 32);
    a.pd[2 * (uint64_t) p + d] = PD{__uint_as_float((uint32_t) (best >> 32)), rc,
                                    (uint32_t) (am & 0xFFFFFFFFull), ok ? 1u : 2u};
  }
}

// Block-wide reductions over the kBatchThreads threads (result in every
// thread).  `red` is shared scratch of one word per warp.
__device__ __forceinline__ unsigned long long block_max_u64(unsigned long long v,
                                                            unsigned long long* red) {
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    const unsigned long long w = __shfl_xor_sync(0xFFFFFFFFu, v, o);
    v = w > v ? w : v;
  }
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  v = red[0];
#pragma unroll
  for (int k = 1; k < kBatchThreads / 32; ++k) v = red[k] > v ? red[k] : v;
  __syncthreads();
  return v;
}

__device__ __forceinline__ float block_min_f(float v, float* red) {
  v = warp_min(v);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  v = red[0];
#pragma unroll
  for (int k = 1; k < kBatchThreads / 32; ++k) v = fminf(v, red[k]);
  __syncthreads();
  return v;
}

// CTA path: the whole block solves one problem-direction of small_rows+1 ..
// pipe_rows query rows with the one-warp path's algorithm — window bounds
// (per row), best-first exact scans (all threads over the other set, an
// early-break vote every 2048 pairs), and after kBestFirst rows a sweep of
// the rows still above the maximum, one warp per row.
template <int D>
__device__ __forceinline__ void cta_direction(const BatchArgs& a, uint32_t p, int d,
                                              const hd_problem& pr, float* wb) {
  __shared__ unsigned long long s_red[kBatchThreads / 32];
  __shared__ float s_redf[kBatchThreads / 32];
  __shared__ unsigned long long s_best;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const float* X = d == 0 ? a.A + pr.offset_a * D : a.B + pr.offset_b * D;
  const float* Y = d == 0 ? a.B + pr.offset_b * D : a.A + pr.offset_a * D;
  const uint32_t nx = (uint32_t) (d == 0 ? pr.n_a : pr.n_b);
  const uint32_t ny = (uint32_t) (d == 0 ? pr.n_b : pr.n_a);
  const float ratio = (float) ny / (float) nx;
  const uint32_t w0 = ny > 2 * a.window + 1 ? 2 * a.window + 1 : ny;
  const uint32_t half = w0 >> 1;
  for (uint32_t row = tid; row < nx; row += kBatchThreads) {
    uint32_t j = scan_start(row, ratio, ny, half);
    wb[row] = scan_run<D>(X, row, Y, j, ny, w0, INFINITY);
  }
  __syncthreads();

  unsigned long long best = 0;
  float thr = -1.0f;
  bool settled = false;
  for (int it = 0; it < kBestFirst; ++it) {
    unsigned long long cand = 0;
    for (uint32_t row = tid; row < nx; row += kBatchThreads) {
      const float u = wb[row];
      if (u > thr) {
        const unsigned long long kk = pack_max(u, row);
        cand = kk > cand ? kk : cand;
      }
    }
    cand = block_max_u64(cand, s_red);
    if (cand == 0) {
      settled = true;
      break;
    }
    const uint32_t r = unpack_max_index(cand);
    float xr[D];
    load_pt<D>(X, r, xr);
    float cm = __uint_as_float((uint32_t) (cand >> 32));  // its bound: a real distance
    bool broke = false;
    for (uint64_t t0 = 0; t0 < ny; t0 += (uint64_t) kBatchThreads * kLongIlp) {
      float y[kLongIlp][D];
#pragma unroll
      for (int u = 0; u < kLongIlp; ++u) {
        const uint64_t jj = t0 + (uint64_t) u * kBatchThreads + tid;
#pragma unroll
        for (int k = 0; k < D; ++k) y[u][k] = jj < ny ? Y[jj * D + k] : INFINITY;
      }
#pragma unroll
      for (int u = 0; u < kLongIlp; ++u) {
        const uint64_t jj = t0 + (uint64_t) u * kBatchThreads + tid;
        const float d2 = d2_of<D>(xr, y[u]);
        if (jj < ny) cm = fminf(cm, d2);
      }
      if (__syncthreads_or(cm <= thr)) {
        broke = true;
        break;
      }
    }
    if (!broke) {
      const unsigned long long kr = pack_max(block_min_f(cm, s_redf), r);
      if (kr > best) {
        best = kr;
        thr = threshold_of(best);
      }
    }
    if (tid == 0) wb[r] = -1.0f;
    __syncthreads();
  }
  if (!settled) {
    // Rows still above the maximum: one warp per row, lanes over the other
    // set; the block's maximum is shared through s_best.
    if (tid == 0) s_best = best;
    __syncthreads();
    for (uint32_t row = warp; row < nx; row += kBatchThreads / 32) {
      const float u = wb[row];
      const float t = threshold_of(*(volatile unsigned long long*) &s_best);
      if (!(u > t)) continue;
      float xr[D];
      load_pt<D>(X, row, xr);
      float cm = u;
      bool broke = false;
      for (uint64_t t0 = 0; t0 < ny; t0 += 32 * kLongIlp) {
        float y[kLongIlp][D];
#pragma unroll
        for (int v = 0; v < kLongIlp; ++v) {
          const uint64_t jj = t0 + (uint64_t) v * 32 + lane;
#pragma unroll
          for (int k = 0; k < D; ++k) y[v][k] = jj < ny ? Y[jj * D + k] : INFINITY;
        }
#pragma unroll
        for (int v = 0; v < kLongIlp; ++v) {
          const uint64_t jj = t0 + (uint64_t) v * 32 + lane;
          const float d2 = d2_of<D>(xr, y[v]);
          if (jj < ny) cm = fminf(cm, d2);
        }
        if (warp_min(cm) <= threshold_of(*(volatile unsigned long long*) &s_best)) {
          broke = true;
          break;
        }
      }
      if (broke) continue;
      const float m = warp_min(cm);  // all lanes: full-warp shuffles
      if (lane == 0) atomicMax(&s_best, pack_max(m, row));
      __syncwarp();
    }
    __syncthreads();
    best = s_best;
    __syncthreads();
  }
  // Certification (block-wide argmin of the certifying row).
  const uint32_t rc = unpack_max_index(best);
  float xc[D];
  load_pt<D>(X, rc, xc);
  unsigned long long am = ~0ull;
#pragma unroll 4
  for (uint32_t j = tid; j < ny; j += kBatchThreads) {
    float y[D];
    load_pt<D>(Y, j, y);
    const unsigned long long k = pack_min(d2_of<D>(xc, y), j);
    am = k < am ? k : am;
  }
  am = ~block_max_u64(~am, s_red);  // min via the complement
  if (tid == 0) {
    a.keys[2 * (uint64_t) p + d] = best;
    const bool ok = (uint32_t) (am >> 32) == (uint32_t) (best >> 32);
    a.pd[2 * (uint64_t) p + d] = PD{__uint_as_float((uint32_t) (best >> 32)), rc,
                                    (uint32_t) (am & 0xFFFFFFFFull), ok ? 1u : 2u};
  }
}

template <int D>
__global__ void __launch_bounds__(kBatchThreads) k_batch_small(BatchArgs a) {
  const int lane = threadIdx.x & 31;
  // First the CTA-path directions, one per block: they sit among the first
  // n_big ranks of the plan, largest first.
  for (uint64_t q = blockIdx.x; q < (uint64_t) a.n_big * a.ndir; q += gridDim.x) {
    const uint32_t r = (uint32_t) (q / a.ndir);
    const int d = (int) (q % a.ndir);
    const uint32_t p = a.order[r];
    const hd_problem pr = a.probs[p];
    const uint64_t nx = d == 0 ? pr.n_a : pr.n_b;
    if (nx <= (uint64_t) a.small_rows || nx > (uint64_t) a.pipe_rows) continue;
    cta_direction<D>(a, p, d, pr, d == 0 ? a.wb_a + pr.offset_a : a.wb_b + pr.offset_b);
  }
  // Then the one-warp directions, one per warp.
  const uint64_t nw = (uint64_t) gridDim.x * (kBatchThreads / 32);
  const uint64_t npd = (uint64_t) a.nprob * a.ndir;
  for (uint64_t q = (uint64_t) blockIdx.x * (kBatchThreads / 32) + (threadIdx.x >> 5); q < npd;
       q += nw) {
    const uint32_t r = (uint32_t) (q / a.ndir);
    const int d = (int) (q % a.ndir);
    const uint32_t p = a.order[r];
    const hd_problem pr = a.probs[p];
    if ((d == 0 ? pr.n_a : pr.n_b) > (uint64_t) a.small_rows) continue;
    small_direction<D>(a, p, d, pr, d == 0 ? a.wb_a + pr.offset_a : a.wb_b + pr.offset_b, lane);
  }
}

// Plan: sort keys and the item count of each sorted rank.  Three groups, each
// largest |A|*|B| first (stable by problem index): problems with a direction
// in the multi-pass pipeline, then problems with a CTA-path direction, then
// the rest (key = maxpairs - pairs + group * (maxpairs + 1)).
// Entry nprob of the counts is 0, so that an exclusive scan over nprob + 1
// entries gives the item prefix with the total at the end.
__global__ void k_plan_keys(const hd_problem* __restrict__ probs, uint32_t n, int ndir,
                            uint32_t small_rows, uint32_t pipe_rows, uint64_t maxpairs,
                            unsigned long long* __restrict__ keys,
                            uint32_t* __restrict__ vals) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const hd_problem pr = probs[i];
  const uint64_t big = ndir == 2 ? max(pr.n_a, pr.n_b) : pr.n_a;
  const uint64_t group = big > pipe_rows ? 0 : (big > small_rows ? 1 : 2);
  const uint64_t pairs = min((uint64_t) (pr.n_a * pr.n_b), maxpairs);  // maxpairs < 2^62
  keys[i] = maxpairs - pairs + group * (maxpairs + 1);
  vals[i] = i;
}

__global__ void k_plan_counts(const hd_problem* __restrict__ probs,
                              const uint32_t* __restrict__ order, uint32_t n, int ndir,
                              uint32_t pipe_rows, uint64_t* __restrict__ cnt) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r > n) return;
  if (r == n) {
    cnt[n] = 0;
    return;
  }
  const hd_problem pr = probs[order[r]];
  cnt[r] = large_items(pr.n_a, pipe_rows) + (ndir == 2 ? large_items(pr.n_b, pipe_rows) : 0);
}

// Certification per problem-direction: one warp scans the other set for the
// argmin of the certifying row (lowest index among ties).
template <int D>
__global__ void k_batch_certify(const float* __restrict__ A, const float* __restrict__ B,
                                const hd_problem* __restrict__ probs, uint32_t nprob, int ndir,
                                const unsigned long long* __restrict__ keys, PD* __restrict__ pd,
                                uint32_t pipe_rows) {
  const int lane = threadIdx.x & 31;
  const uint64_t w = (uint64_t) blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  if (w >= (uint64_t) nprob * ndir) return;
  const uint32_t p = (uint32_t) (w / ndir);
  const int d = (int) (w % ndir);
  const hd_problem pr = probs[p];
  // The one-warp and CTA paths certify their own directions.
  if ((d == 0 ? pr.n_a : pr.n_b) <= pipe_rows) return;
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
#pragma unroll 4
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

// The problems of a batch, given either as an hd_problem array or as two
// offset arrays (problem i owns rows oa[i]..oa[i+1] of A and ob[i]..ob[i+1]
// of B; a decreasing pair gives a huge count, rejected as out of range).
struct ProblemSource {
  const hd_problem* probs = nullptr;
  const uint64_t* oa = nullptr;
  const uint64_t* ob = nullptr;
  // Device copies of oa / ob when already uploaded (grouped batches).
  const uint64_t* doa = nullptr;
  const uint64_t* dob = nullptr;
  hd_problem get(uint64_t i) const {
    if (probs) return probs[i];
    return hd_problem{oa[i], oa[i + 1] - oa[i], ob[i], ob[i + 1] - ob[i]};
  }
};

// Problems from offsets, on the device (one thread per problem).
__global__ void k_probs_from_offsets(const uint64_t* __restrict__ oa,
                                     const uint64_t* __restrict__ ob, uint64_t n,
                                     hd_problem* __restrict__ probs) {
  const uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x;
  if (i >= n) return;
  probs[i] = hd_problem{oa[i], oa[i + 1] - oa[i], ob[i], ob[i + 1] - ob[i]};
}

hd_status check_problems(Ctx& c, const ProblemSource& src, uint64_t n, uint64_t ta, uint64_t tb) {
  for (uint64_t i = 0; i < n; ++i) {
    const hd_problem p = src.get(i);
    if (p.n_a == 0 || p.n_b == 0)
      return fail(c, HD_ERR_INVALID_ARG, "problem " + std::to_string(i) + " has an empty set");
    if (p.offset_a > ta || p.n_a > ta - p.offset_a || p.offset_b > tb || p.n_b > tb - p.offset_b)
      return fail(c, HD_ERR_INVALID_ARG, "problem " + std::to_string(i) + " is out of range");
    if (p.n_a >= 0xFFFFFFFFull || p.n_b >= 0xFFFFFFFFull)
      return fail(c, HD_ERR_INVALID_ARG, "problem sets are limited to 2^32-2 points");
  }
  return HD_OK;
}


// Bump allocator over one device buffer, 256-byte aligned pieces.
struct Layout {
  size_t off = 0;
  size_t take(size_t bytes) {
    const size_t o = off;
    off += (bytes + 255) / 256 * 256;
    return o;
  }
};

// Everything one batched-solve graph is captured from.
struct BatchGraph {
  BatchArgs args;
  int dims, ndir, end_bit;
  uint64_t n, maxpairs;
  char* base;             // the batch buffer; reset region starts here
  size_t zero_bytes;      // keys and window bounds per class (reset to 0)
  unsigned long long* ctr;    // long-row count, certification mismatch count
  size_t o_smin, smin_bytes;  // seed minima (reset to 0xFF bytes)
  size_t o_pkeys, o_pkeys2, o_pvals, o_cnt, o_tmp, cub_tmp;
  PD* pd;
  hd_batch_result* out;
  uint32_t* bad;
  const void* fns[5];     // window, seed, sweep, long, one-warp path
  int grids[5];
};

// Resets the graph's per-call words with a kernel (no memset node that could
// queue behind copies): keys and window bounds to 0, seed minima to all ones,
// the two counters to 0.
__global__ void k_batch_reset(uint4* __restrict__ zero, size_t zero16, uint4* __restrict__ ones,
                              size_t ones16, unsigned long long* __restrict__ ctr) {
  const size_t stride = (size_t) gridDim.x * blockDim.x;
  const size_t t = blockIdx.x * (size_t) blockDim.x + threadIdx.x;
  for (size_t i = t; i < zero16; i += stride) zero[i] = make_uint4(0u, 0u, 0u, 0u);
  for (size_t i = t; i < ones16; i += stride) ones[i] = make_uint4(~0u, ~0u, ~0u, ~0u);
  if (t < 2) ctr[t] = 0ull;
}

hd_status capture_batch_graph(Ctx& c, const BatchGraph& g, cudaGraphExec_t* out) {
  auto at = [&](size_t o) { return (void*) (g.base + o); };
  const BatchArgs& a = g.args;
  const uint32_t n = (uint32_t) g.n;
  const unsigned pblocks = (unsigned) ((g.n + 1 + 255) / 256);
  cudaGraph_t graph = nullptr;
  cudaError_t e = cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return cuda_fail(c, e, "begin capture");
  {
    // Both regions are whole multiples of 256 bytes (Layout pieces).
    const size_t z16 = g.zero_bytes / 16, o16 = g.smin_bytes / 16;
    const size_t work = std::max<size_t>(std::max(z16, o16), 2);
    const unsigned rb = (unsigned) std::min<size_t>((work + 255) / 256, (size_t) c.num_sms * 8);
    k_batch_reset<<<rb, 256, 0, c.stream>>>((uint4*) g.base, z16, (uint4*) at(g.o_smin), o16,
                                            g.ctr);
  }
  k_plan_keys<<<pblocks, 256, 0, c.stream>>>(a.probs, n, g.ndir, a.small_rows, a.pipe_rows,
                                            g.maxpairs,
                                            (unsigned long long*) at(g.o_pkeys),
                                            (uint32_t*) at(g.o_pvals));
  size_t tb = g.cub_tmp;
  cub::DeviceRadixSort::SortPairs(at(g.o_tmp), tb, (const unsigned long long*) at(g.o_pkeys),
                                  (unsigned long long*) at(g.o_pkeys2),
                                  (const uint32_t*) at(g.o_pvals), const_cast<uint32_t*>(a.order),
                                  (int64_t) n, 0, g.end_bit, c.stream);
  k_plan_counts<<<pblocks, 256, 0, c.stream>>>(a.probs, a.order, n, g.ndir, a.pipe_rows,
                                              (uint64_t*) at(g.o_cnt));
  tb = g.cub_tmp;
  cub::DeviceScan::ExclusiveSum(at(g.o_tmp), tb, (const uint64_t*) at(g.o_cnt),
                                const_cast<uint64_t*>(a.prefix), (int64_t) (g.n + 1), c.stream);
  BatchArgs kernel_args = a;
  void* kargs[] = {&kernel_args};
  // Fork: the one-warp path runs on a side branch of the graph, beside the
  // multi-pass pipeline; both join before certification.
  cudaEventRecord(c.batch_fork, c.stream);
  cudaStreamWaitEvent(c.batch_side, c.batch_fork, 0);
  cudaLaunchKernel(g.fns[4], dim3(g.grids[4]), dim3(kBatchThreads), kargs, 0, c.batch_side);
  cudaEventRecord(c.batch_join, c.batch_side);
  const uint64_t npd = g.n * g.ndir;
  for (int k = 0; k < 4; ++k) {
    if (k == 2)  // between seed and sweep
      k_batch_fold<<<(unsigned) ((npd + 255) / 256), 256, 0, c.stream>>>(a.ubound, a.smin, npd,
                                                                         a.keys);
    cudaLaunchKernel(g.fns[k], dim3(g.grids[k]), dim3(kBatchThreads), kargs, 0, c.stream);
  }
  cudaStreamWaitEvent(c.stream, c.batch_join, 0);
  const unsigned cblocks = (unsigned) ((g.n * g.ndir * 32 + 255) / 256);
  if (g.dims == 2)
    k_batch_certify<2><<<cblocks, 256, 0, c.stream>>>(a.A, a.B, a.probs, n, g.ndir, a.keys, g.pd,
                                                      a.pipe_rows);
  else
    k_batch_certify<3><<<cblocks, 256, 0, c.stream>>>(a.A, a.B, a.probs, n, g.ndir, a.keys, g.pd,
                                                      a.pipe_rows);
  k_batch_finalize<<<(unsigned) ((g.n + 255) / 256), 256, 0, c.stream>>>(g.pd, n, g.ndir, g.out,
                                                                          g.bad);
  e = cudaStreamEndCapture(c.stream, &graph);
  if (e != cudaSuccess) return cuda_fail(c, e, "end capture");
  cudaGraphExec_t exec = nullptr;
  e = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return cuda_fail(c, e, "instantiate graph");
  *out = exec;
  return HD_OK;
}

// The cached graph for a launch shape: a hit, or a capture into the least
// recently used slot.
hd_status batch_graph_for(Ctx& c, const BatchGraph& g, const uint64_t* key,
                          cudaGraphExec_t* out) {
  int slot = -1, lru = 0;
  for (int i = 0; i < Ctx::kBatchGraphs; ++i) {
    if (c.batch_graphs[i] && std::memcmp(key, c.batch_keys[i], sizeof(c.batch_keys[i])) == 0) {
      slot = i;
      break;
    }
    if (c.batch_stamp[i] < c.batch_stamp[lru]) lru = i;
  }
  if (slot < 0) {
    slot = lru;
    cudaGraphExec_t exec = nullptr;
    hd_status s = capture_batch_graph(c, g, &exec);
    if (s != HD_OK) return s;
    if (c.batch_graphs[slot]) cudaGraphExecDestroy(c.batch_graphs[slot]);
    c.batch_graphs[slot] = exec;
    std::memcpy(c.batch_keys[slot], key, sizeof(c.batch_keys[slot]));
  }
  c.batch_stamp[slot] = ++c.batch_clock;
  *out = c.batch_graphs[slot];
  return HD_OK;
}

}  // namespace

// stage_bad != null: the results and the mismatch word are only queued (to
// out and *stage_bad, both pinned host memory) and the call returns without
// waiting; the caller synchronises and checks *stage_bad.
hd_status batch_solve(Ctx& c, const float* A, uint64_t total_a, const float* B, uint64_t total_b,
                      int dims, const ProblemSource& src, uint64_t n, uint32_t flags,
                      hd_batch_result* out, uint32_t* stage_bad = nullptr) {
  if (!A || !B || !(src.probs || (src.oa && src.ob)) || !out || n == 0)
    return fail(c, HD_ERR_INVALID_ARG, "bad arguments");
  if (dims != 2 && dims != 3) return fail(c, HD_ERR_UNSUPPORTED, "batches need n_dims 2 or 3");
  if (n >= 0xFFFFFFFFull) return fail(c, HD_ERR_INVALID_ARG, "too many problems");
  if (flags & ~(HD_UNDIRECTED | HD_DEVICE_PTRS)) return fail(c, HD_ERR_INVALID_ARG, "bad flags");
  hd_status s;
  // A group of a grouped batch was validated with the whole batch.
  if (!src.doa && (s = check_problems(c, src, n, total_a, total_b)) != HD_OK) return s;
  const int ndir = (flags & HD_UNDIRECTED) ? 2 : 1;
  const uint32_t small_rows = std::min<uint32_t>(c.opt.batch_small_rows, kSmallMax);
  const uint32_t pipe_rows = std::max<uint32_t>(small_rows, kPipeRows);
  const uint32_t chunk = std::max<uint32_t>(1, c.opt.batch_chunk);
  uint64_t total = 0, rows = 0, maxpairs = 0, n_big = 0;
  for (uint64_t i = 0; i < n; ++i) {
    const hd_problem p = src.get(i);
    total += large_items(p.n_a, pipe_rows) + (ndir == 2 ? large_items(p.n_b, pipe_rows) : 0);
    rows += p.n_a + (ndir == 2 ? p.n_b : 0);
    maxpairs = std::max<uint64_t>(maxpairs, p.n_a * p.n_b);
    n_big += (p.n_a > small_rows || (ndir == 2 && p.n_b > small_rows)) ? 1 : 0;
  }
  BatchGraph g{};
  g.dims = dims;
  g.ndir = ndir;
  g.n = n;
  // Plan keys stay below 3 * maxpairs + 3 (largest-first order among
  // problems above 2^62 pairs is not needed).
  maxpairs = std::min<uint64_t>(maxpairs, (1ull << 62) - 1);
  g.maxpairs = maxpairs;
  g.end_bit = 1;
  while (g.end_bit < 64 && ((3 * maxpairs + 2) >> g.end_bit)) ++g.end_bit;
  const uint64_t long_cap = std::min<uint64_t>(rows, kLongCap);

  // CUB temporary storage for the plan's sort and scan.
  size_t sort_tmp = 0, scan_tmp = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, sort_tmp, (const unsigned long long*) nullptr,
                                  (unsigned long long*) nullptr, (const uint32_t*) nullptr,
                                  (uint32_t*) nullptr, (int64_t) n, 0, g.end_bit, c.stream);
  cub::DeviceScan::ExclusiveSum(nullptr, scan_tmp, (const uint64_t*) nullptr, (uint64_t*) nullptr,
                                (int64_t) (n + 1), c.stream);
  g.cub_tmp = std::max(sort_tmp, scan_tmp);

  // Device layout in one buffer; the words reset inside the graph come
  // first: keys and window bounds (zero), seed minima (0xFF bytes).
  Layout L;
  const size_t o_keys = L.take(n * 2 * 8);
  const size_t o_ub = L.take(n * 2 * kSlots * 8);
  g.zero_bytes = L.off;
  g.o_smin = L.take(n * 2 * kSlots * 4);
  g.smin_bytes = L.off - g.o_smin;
  const size_t o_ctr = L.take(2 * 8);  // long-row count, mismatch count
  const size_t o_wb_a = L.take(total_a * 4);
  const size_t o_wb_b = L.take(ndir == 2 ? total_b * 4 : 0);
  const size_t o_probs = L.take(n * sizeof(hd_problem));
  const size_t o_offs = L.take(src.probs || src.doa ? 0 : 2 * (n + 1) * 8);
  g.o_pkeys = L.take(n * 8);
  g.o_pkeys2 = L.take(n * 8);
  g.o_pvals = L.take(n * 4);
  const size_t o_order = L.take(n * 4);
  g.o_cnt = L.take((n + 1) * 8);
  const size_t o_prefix = L.take((n + 1) * 8);
  const size_t o_pd = L.take(n * 2 * sizeof(PD));
  const size_t o_out = L.take(n * sizeof(hd_batch_result));
  g.o_tmp = L.take(g.cub_tmp);
  const size_t o_long = L.take(long_cap * sizeof(LongRow));
  void* buf;
  if ((s = ensure(c, kBufBatch, L.off, &buf)) != HD_OK) return s;
  g.base = (char*) buf;
  auto at = [&](size_t o) { return (void*) (g.base + o); };
  unsigned long long* d_ctr = (unsigned long long*) at(o_ctr);
  g.pd = (PD*) at(o_pd);
  g.out = (hd_batch_result*) at(o_out);
  g.ctr = d_ctr;
  g.bad = (uint32_t*) (d_ctr + 1);

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
  if (src.probs) {
    if ((e = cudaMemcpyAsync(at(o_probs), src.probs, n * sizeof(hd_problem),
                             cudaMemcpyHostToDevice, c.stream)) != cudaSuccess)
      return cuda_fail(c, e, "copy problems");
  } else {
    const uint64_t* d_oa = src.doa;
    const uint64_t* d_ob = src.dob;
    if (!d_oa) {
      uint64_t* oa_up = (uint64_t*) at(o_offs);
      uint64_t* ob_up = oa_up + (n + 1);
      if ((e = cudaMemcpyAsync(oa_up, src.oa, (n + 1) * 8, cudaMemcpyHostToDevice, c.stream)) !=
              cudaSuccess ||
          (e = cudaMemcpyAsync(ob_up, src.ob, (n + 1) * 8, cudaMemcpyHostToDevice, c.stream)) !=
              cudaSuccess)
        return cuda_fail(c, e, "copy offsets");
      d_oa = oa_up;
      d_ob = ob_up;
    }
    k_probs_from_offsets<<<(unsigned) ((n + 255) / 256), 256, 0, c.stream>>>(
        d_oa, d_ob, n, (hd_problem*) at(o_probs));
    if ((s = after_launch(c, "problems from offsets")) != HD_OK) return s;
  }

  BatchArgs& args = g.args;
  args.A = dA;
  args.B = dB;
  args.probs = (const hd_problem*) at(o_probs);
  args.order = (const uint32_t*) at(o_order);
  args.prefix = (const uint64_t*) at(o_prefix);
  args.nprob = (uint32_t) n;
  args.ndir = ndir;
  args.total = total;
  args.keys = (unsigned long long*) at(o_keys);
  args.ubound = (unsigned long long*) at(o_ub);
  args.smin = (uint32_t*) at(g.o_smin);
  args.wb_a = (float*) at(o_wb_a);
  args.wb_b = (float*) at(o_wb_b);
  args.longq = (LongRow*) at(o_long);
  args.long_count = d_ctr;
  args.long_cap = long_cap;
  args.small_rows = small_rows;
  args.pipe_rows = pipe_rows;
  args.n_big = (uint32_t) n_big;
  args.chunk = chunk;
  args.window = c.opt.batch_window;
  args.pd = g.pd;

  // Persistent grids: resident blocks of each kernel, at most one warp per
  // chunk of items (or per queued row).
  if (dims == 2) {
    g.fns[0] = (const void*) k_batch_pass<2, kPassWindow>;
    g.fns[1] = (const void*) k_batch_pass<2, kPassSeed>;
    g.fns[2] = (const void*) k_batch_pass<2, kPassSweep>;
    g.fns[3] = (const void*) k_batch_long<2>;
    g.fns[4] = (const void*) k_batch_small<2>;
  } else {
    g.fns[0] = (const void*) k_batch_pass<3, kPassWindow>;
    g.fns[1] = (const void*) k_batch_pass<3, kPassSeed>;
    g.fns[2] = (const void*) k_batch_pass<3, kPassSweep>;
    g.fns[3] = (const void*) k_batch_long<3>;
    g.fns[4] = (const void*) k_batch_small<3>;
  }
  const uint64_t chunks = (total + chunk - 1) / chunk;
  for (int k = 0; k < 5; ++k) {
    int occ = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, g.fns[k], kBatchThreads, 0);
    const uint64_t warps = k < 3 ? chunks : (k == 3 ? long_cap : n * ndir);
    g.grids[k] = (int) std::max<uint64_t>(
        1, std::min<uint64_t>((uint64_t) c.num_sms * std::max(occ, 1), (warps + 7) / 8));
  }

  // One graph: reset, plan, window, seed, sweep, long rows, certification,
  // finalisation.  Captured once per launch shape; the per-call input (the
  // problems) is read from device memory.
  const uint64_t key[17] = {(uint64_t) dims, n,        (uint64_t) ndir, (uint64_t) dA,
                            (uint64_t) dB,   total_a,  total_b,         (uint64_t) g.base,
                            (uint64_t) L.off, total,   maxpairs,        long_cap,
                            (uint64_t) c.stream, small_rows, chunk, c.opt.batch_window, n_big};
  static_assert(sizeof(key) == sizeof(c.batch_keys[0]), "batch key size");
  if ((s = ensure_side(c)) != HD_OK) return s;
  cudaGraphExec_t exec = nullptr;
  if ((s = batch_graph_for(c, g, key, &exec)) != HD_OK) return s;
  e = cudaGraphLaunch(exec, c.stream);
  c.launches += 11;  // own kernels: reset, plan keys, plan counts, one-warp path, window, seed,
                     // fold, sweep, long, certify, finalize
  if (e != cudaSuccess) return cuda_fail(c, e, "graph launch");
  if (stage_bad) {
    if ((e = cudaMemcpyAsync(out, g.out, n * sizeof(hd_batch_result), cudaMemcpyDeviceToHost,
                             c.stream)) != cudaSuccess ||
        (e = cudaMemcpyAsync(stage_bad, g.bad, 4, cudaMemcpyDeviceToHost, c.stream)) != cudaSuccess)
      return cuda_fail(c, e, "batch solve");
    return HD_OK;
  }
  uint32_t bad = 0;
  if ((e = cudaMemcpyAsync(out, g.out, n * sizeof(hd_batch_result), cudaMemcpyDeviceToHost,
                           c.stream)) != cudaSuccess ||
      (e = cudaMemcpyAsync(&bad, g.bad, 4, cudaMemcpyDeviceToHost, c.stream)) != cudaSuccess ||
      (e = cudaStreamSynchronize(c.stream)) != cudaSuccess)
    return cuda_fail(c, e, "batch solve");
  if (bad) return fail(c, HD_ERR_CUDA, "batch certification mismatch");
  return HD_OK;
}

// Host points given by offsets: the problems run as a few groups of
// consecutive problems (about kGroupBytes of points each).  Every group's
// point ranges are copied on the copy stream up front, and group j is solved
// as soon as its own copies have landed, so the host link keeps streaming
// later groups while the GPU solves earlier ones.  Offsets are validated on
// the whole batch first (non-empty problems inside the sets, which makes
// them increasing), so every copied range lies inside A and B.
constexpr uint64_t kGroupBytes = 96ull << 20;

hd_status batch_solve_grouped(Ctx& c, const float* A, uint64_t total_a, const float* B,
                              uint64_t total_b, int dims, const uint64_t* oa, const uint64_t* ob,
                              uint64_t n, uint32_t flags, hd_batch_result* out) {
  ProblemSource all;
  all.oa = oa;
  all.ob = ob;
  const uint64_t bytes = (total_a + total_b) * (uint64_t) (dims > 0 ? dims : 0) * 4;
  const int K = (int) std::min<uint64_t>(Ctx::kBatchGroups, bytes / kGroupBytes);
  if ((flags & HD_DEVICE_PTRS) || K < 2 || n < 64 * (uint64_t) K || !A || !B || !out ||
      (dims != 2 && dims != 3))
    return batch_solve(c, A, total_a, B, total_b, dims, all, n, flags, out);
  if (flags & ~(HD_UNDIRECTED | HD_DEVICE_PTRS)) return fail(c, HD_ERR_INVALID_ARG, "bad flags");
  hd_status s;
  if ((s = check_problems(c, all, n, total_a, total_b)) != HD_OK) return s;
  // Group boundaries: equal shares of the points of both sets.
  uint64_t cut[Ctx::kBatchGroups + 1];
  int ng = 0;
  cut[0] = 0;
  const uint64_t span = (oa[n] - oa[0]) + (ob[n] - ob[0]);
  for (uint64_t i = 1; i < n && ng + 1 < K; ++i) {
    const uint64_t done = (oa[i] - oa[0]) + (ob[i] - ob[0]);
    if (done * (uint64_t) K >= span * (uint64_t) (ng + 1)) cut[++ng] = i;
  }
  cut[++ng] = n;
  void *pa, *pb, *po;
  if ((s = ensure(c, kBufA, total_a * dims * 4, &pa)) != HD_OK) return s;
  if ((s = ensure(c, kBufB, total_b * dims * 4, &pb)) != HD_OK) return s;
  if ((s = ensure(c, kBufGroupOffs, 2 * (n + 1) * 8, &po)) != HD_OK) return s;
  if ((s = ensure_side(c)) != HD_OK) return s;
  cudaError_t e;
  if (!c.copy_stream) {
    if ((e = cudaStreamCreateWithFlags(&c.copy_stream, cudaStreamNonBlocking)) != cudaSuccess)
      return cuda_fail(c, e, "copy stream");
    for (auto& ev : c.copy_ev)
      if ((e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming)) != cudaSuccess)
        return cuda_fail(c, e, "copy events");
  }
  // The copies start after everything already queued on the call's stream.
  if ((e = cudaEventRecord(c.batch_fork, c.stream)) != cudaSuccess ||
      (e = cudaStreamWaitEvent(c.copy_stream, c.batch_fork, 0)) != cudaSuccess)
    return cuda_fail(c, e, "fork");
  // The offsets go first, so no group's solve waits behind the point copies
  // for them (copies to the device share one queue).
  uint64_t* d_oa = (uint64_t*) po;
  uint64_t* d_ob = d_oa + (n + 1);
  if ((e = cudaMemcpyAsync(d_oa, oa, (n + 1) * 8, cudaMemcpyHostToDevice, c.copy_stream)) !=
          cudaSuccess ||
      (e = cudaMemcpyAsync(d_ob, ob, (n + 1) * 8, cudaMemcpyHostToDevice, c.copy_stream)) !=
          cudaSuccess) {
    cudaStreamSynchronize(c.copy_stream);
    return cuda_fail(c, e, "copy offsets");
  }
  const size_t row = (size_t) dims * sizeof(float);
  for (int j = 0; j < ng; ++j) {
    const uint64_t a0 = oa[cut[j]], a1 = oa[cut[j + 1]], b0 = ob[cut[j]], b1 = ob[cut[j + 1]];
    e = cudaMemcpyAsync((char*) pa + a0 * row, (const char*) A + a0 * row, (a1 - a0) * row,
                        cudaMemcpyHostToDevice, c.copy_stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync((char*) pb + b0 * row, (const char*) B + b0 * row, (b1 - b0) * row,
                          cudaMemcpyHostToDevice, c.copy_stream);
    if (e == cudaSuccess) e = cudaEventRecord(c.copy_ev[j], c.copy_stream);
    if (e != cudaSuccess) {
      cudaStreamSynchronize(c.copy_stream);
      return cuda_fail(c, e, "copy points");
    }
  }
  // Results of all groups are staged in pinned memory and the host waits
  // once, at the end (the groups share the batch buffer, in stream order).
  const size_t stage = n * sizeof(hd_batch_result) + 16 * sizeof(uint32_t);
  if (c.batch_pinned_bytes < stage) {
    if (c.batch_pinned) cudaFreeHost(c.batch_pinned);
    c.batch_pinned = nullptr;
    c.batch_pinned_bytes = 0;
    if ((e = cudaMallocHost(&c.batch_pinned, stage)) != cudaSuccess) {
      c.batch_pinned = nullptr;
      cudaStreamSynchronize(c.copy_stream);
      return fail(c, HD_ERR_OOM, "pinned staging of batch results");
    }
    c.batch_pinned_bytes = stage;
  }
  hd_batch_result* staged = (hd_batch_result*) c.batch_pinned;
  uint32_t* bad = (uint32_t*) (staged + n);
  s = HD_OK;
  for (int j = 0; j < ng && s == HD_OK; ++j) {
    if ((e = cudaStreamWaitEvent(c.stream, c.copy_ev[j], 0)) != cudaSuccess) {
      s = cuda_fail(c, e, "wait for copies");
      break;
    }
    ProblemSource grp;
    grp.oa = oa + cut[j];
    grp.ob = ob + cut[j];
    grp.doa = d_oa + cut[j];
    grp.dob = d_ob + cut[j];
    s = batch_solve(c, (const float*) pa, total_a, (const float*) pb, total_b, dims, grp,
                    cut[j + 1] - cut[j], (flags & HD_UNDIRECTED) | HD_DEVICE_PTRS,
                    staged + cut[j], bad + j);
  }
  // No copy may still read the caller's buffers when the call returns, and
  // no staged result may still be in flight.
  e = cudaStreamSynchronize(c.stream);
  const cudaError_t e2 = cudaStreamSynchronize(c.copy_stream);
  if (s != HD_OK) return s;
  if (e != cudaSuccess) return cuda_fail(c, e, "batch solve");
  if (e2 != cudaSuccess) return cuda_fail(c, e2, "copy points");
  for (int j = 0; j < ng; ++j)
    if (bad[j]) return fail(c, HD_ERR_CUDA, "batch certification mismatch");
  std::memcpy(out, staged, n * sizeof(hd_batch_result));
  return HD_OK;
}

hd_status batch_solve_plain(Ctx& c, const float* A, uint64_t total_a, const float* B,
                            uint64_t total_b, int dims, const hd_problem* probs, uint64_t n,
                            uint32_t flags, hd_batch_result* out) {
  if (!A || !B || !probs || !out || n == 0) return fail(c, HD_ERR_INVALID_ARG, "bad arguments");
  if (dims != 2 && dims != 3) return fail(c, HD_ERR_UNSUPPORTED, "batches need n_dims 2 or 3");
  if (flags & ~(HD_UNDIRECTED | HD_DEVICE_PTRS)) return fail(c, HD_ERR_INVALID_ARG, "bad flags");
  hd_status s;
  if ((s = check_problems(c, ProblemSource{probs}, n, total_a, total_b)) != HD_OK) return s;
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
  return batch_solve(*c, A, total_a, B, total_b, n_dims, ProblemSource{probs}, n_problems, flags,
                     out);
}

hd_status hd_solve_batch_offsets(hd_ctx* c, const float* A, uint64_t total_a, const float* B,
                                 uint64_t total_b, int n_dims, const uint64_t* offsets_a,
                                 const uint64_t* offsets_b, uint64_t n_problems, uint32_t flags,
                                 hd_batch_result* out) {
  if (!c) return HD_ERR_INVALID_ARG;
  c->last_error.clear();
  cudaSetDevice(c->device);
  if (!offsets_a || !offsets_b || n_problems == 0)
    return fail(*c, HD_ERR_INVALID_ARG, "bad arguments");
  return batch_solve_grouped(*c, A, total_a, B, total_b, n_dims, offsets_a, offsets_b, n_problems,
                             flags, out);
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
