// FP64 input path: the exact FP64 Hausdorff distance of double-precision
// point sets.  The reference declares double point types and a disabled
// -is_double dispatch (src/run_hausdorff_distance.cu:56-62) that would
// instantiate its algorithms with double coordinates and double squared
// distances (the template of src/geoms/distance.h:17-24).
//
// GB300 runs FP64 at a small fraction of its FP32 rate, so the search stays
// in FP32 and FP64 arithmetic is spent only where FP32 values cannot decide.
// Directed h(X, Y), n_dims 2 or 3 (the LBVH route):
//  1. X and Y are rounded to float; dX = max |x_k - fl(x_k)| over X's
//     coordinates (likewise dY).  A point moves by at most sqrt(D)·dX when
//     rounded, so the exact distances of a rounded pair and of the original
//     pair differ by at most r = sqrt(D)·(dX + dY).
//  2. The FP32 LBVH solve of the rounded sets certifies a row i* and its
//     FP32 nearest squared distance.
//  3. Seed: the exact FP64 nearest neighbour of x_{i*} (the walk below)
//     gives L = min_j d64(x_{i*}, y_j)^2 <= h64^2.
//  4. A float threshold T is derived from L so that every rounded pair with
//     FP32 squared distance <= T has FP64 squared distance < L.  A second
//     query pass over the same trees, with the running maximum frozen at T,
//     stops each row that has such a pair and lists the others with their
//     FP32 minima; every row whose FP64 nearest distance is >= L is listed.
//  5. Each listed row's FP64 nearest neighbour is found by a walk of the
//     same tree (FP64 box bounds and FP64 pair distances); a walk stops once
//     an upper bound of its distance is strictly below the running FP64
//     maximum (seeded with L).  The answer is the largest completed
//     distance, the lowest row among equal ones, and that row's lowest
//     column.
// When the list overflows (rows that nearly all tie: a lattice and its
// translate) step 5 walks every row.  Other n_dims, coordinates beyond
// +-1e18 and the eb / brute variants use an FP64 scan instead.
//
// Rounding bounds, with u = 2^-24, v = 2^-53 and D + 2 rounded operations
// per squared distance over non-negative terms: the FP32 formula gives
// d32^2 >= e^2 (1 - u)^(D+2) - (D+2) 2^-126 for the exact distance e of the
// rounded pair (the absolute term covers underflow, even with flush to
// zero); the FP64 formula gives d64^2 <= d^2 (1 + v)^(D+2) + (D+2) 2^-1074
// for the exact distance d of the original pair; and |d - e| <= r.  The code
// applies them with a further relative margin of 2^-40, which covers the
// rounding of its own double arithmetic.
#include <cfloat>
#include <cmath>
#include <cstring>

#include "hd_common.cuh"
#include "hd_internal.h"

namespace hdg {
namespace {

constexpr uint32_t kLeafBit = 0x80000000u;
constexpr uint32_t kListCap = 1u << 20;  // listed rows per direction
constexpr double kRangeLimit = 1e18;     // |coordinate| the LBVH route accepts
constexpr uint32_t kF64NonFinite = 1u, kF64Range = 2u;
constexpr int kWalkStack = 64;           // one entry per tree level at most
constexpr double kMargin = 0x1p-40;
constexpr int kWalkThreads = 128;
constexpr int kScanThreads = 128;

struct RoundStats {
  unsigned long long dmax;  // max |x - fl(x)| over the set's coordinates (double bits)
  uint32_t flags;           // kF64NonFinite | kF64Range
  uint32_t pad;
};

struct F64Dir {
  unsigned long long max64;  // running FP64 maximum (double bits; values >= +0)
  unsigned long long pick;   // (row << 32) | column of the answer (atomicMin)
  double seed_d2;            // the seed row's FP64 nearest squared distance
  uint32_t seed_row, seed_col;
  uint32_t cand_count;       // rows listed by the frozen pass (may exceed the cap)
  float thr;                 // frozen threshold (-1: none)
};

// Device layout of kBufF64Aux; the two candidate lists follow it.
struct F64Aux {
  RoundStats round[2];  // per set: 0 = A, 1 = B
  F64Dir dir[2];
  DevScalars frozen[2];
  RowEntry seed[2];
  double seed_min[2];
  uint32_t seed_col[2];
};
constexpr size_t kAuxBytes = (sizeof(F64Aux) + 255) / 256 * 256;

__device__ __forceinline__ unsigned long long dbits(double v) {
  return (unsigned long long) __double_as_longlong(v);
}
__device__ __forceinline__ double bits_d(unsigned long long b) {
  return __longlong_as_double((long long) b);
}

// The reference formula in FP64: per-dimension difference, squared, summed
// left to right, no FMA.
template <int D>
__device__ __forceinline__ double d2_64(const double* x, const double* y) {
  double d = __dsub_rn(x[0], y[0]);
  double s = __dmul_rn(d, d);
#pragma unroll
  for (int k = 1; k < D; ++k) {
    d = __dsub_rn(x[k], y[k]);
    s = __dadd_rn(s, __dmul_rn(d, d));
  }
  return s;
}

// An upper bound of the FP64 nearest squared distance of a row whose FP32
// nearest squared distance over the rounded sets is m32 (+inf: none known).
template <int D>
__device__ __forceinline__ double upper_from32(float m32, double rxy) {
  if (!(m32 < INFINITY)) return INFINITY;
  const double e2 = ((double) m32 + (D + 2) * 0x1p-126) / (1.0 - (D + 2) * 0x1p-24);
  const double d = sqrt(e2) * (1.0 + kMargin) + rxy;
  return d * d * (1.0 + kMargin) + 0x1p-1000;
}

// A lower bound of the FP64 squared distance from x to every original point
// whose rounded point lies in the box (float bounds), ry = how far a
// target point moves when rounded.
template <int D>
__device__ __forceinline__ double box_lb64(const double* x, const float4& xy, float lz, float hz,
                                           double ry) {
  const double g0 = fmax(fmax((double) xy.x - x[0], x[0] - (double) xy.z), 0.0);
  const double g1 = fmax(fmax((double) xy.y - x[1], x[1] - (double) xy.w), 0.0);
  double s = g0 * g0 + g1 * g1;
  if (D == 3) {
    const double g2 = fmax(fmax((double) lz - x[2], x[2] - (double) hz), 0.0);
    s += g2 * g2;
  }
  const double d = sqrt(s) * (1.0 - kMargin) - ry;
  if (d <= 0.0) return 0.0;
  return d * d * (1.0 - kMargin) - 0x1p-1000;
}

// Rounds a set to float (Xf may be null: check only) and records the
// largest rounding displacement of a coordinate and the range flags.
__global__ void k_f64_round(const double* __restrict__ X, uint64_t total, float* __restrict__ Xf,
                            RoundStats* st) {
  double dm = 0.0;
  uint32_t fl = 0;
  for (uint64_t t = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; t < total;
       t += (uint64_t) gridDim.x * blockDim.x) {
    const double x = X[t];
    const float f = __double2float_rn(x);
    if (!isfinite(x))
      fl |= kF64NonFinite;
    else if (fabs(x) > kRangeLimit)
      fl |= kF64Range;
    if (Xf) Xf[t] = f;
    // Exact: f is x rounded to float, so x and f are within a factor of two
    // (or f = 0 and the difference is x).
    const double d = fabs(x - (double) f);
    if (d > dm) dm = d;
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    dm = fmax(dm, __shfl_xor_sync(0xFFFFFFFFu, dm, o));
    fl |= __shfl_xor_sync(0xFFFFFFFFu, fl, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (dm > 0.0) atomicMax(&st->dmax, dbits(dm));
    if (fl) atomicOr(&st->flags, fl);
  }
}

__global__ void k_f64_init(F64Aux* aux) {
  const int k = threadIdx.x;
  if (k < 2) {
    F64Dir z;
    z.max64 = 0ull;
    z.pick = ~0ull;
    z.seed_d2 = -1.0;
    z.seed_row = z.seed_col = 0u;
    z.cand_count = 0u;
    z.thr = -1.0f;
    aux->dir[k] = z;
    aux->round[k].dmax = 0ull;
    aux->round[k].flags = 0u;
  }
}

// The seed rows: each direction's FP32-certified row and its FP32 minimum.
__global__ void k_f64_seed_entries(const DevScalars* sc, F64Aux* aux, int count) {
  const int k = threadIdx.x;
  if (k < count) aux->seed[k] = RowEntry{sc[k].ia, __float_as_uint(sc[k].d2)};
}

// Rows walked by one launch (blockIdx.y = direction).
struct WalkArgs {
  const double* X;        // query set, caller's rows
  const double* Y;        // target set, caller's rows
  LbvhTree t;             // the target's tree over its rounded points
  const RowEntry* list;   // rows to walk, or null: every row of X
  uint64_t n_rows;
  double ry;              // bound on a target point's displacement by rounding
  double rxy;             // the same for a pair
  F64Dir* f;
  double* row_min;        // per walked row: FP64 nearest squared distance, -1 if stopped
  uint32_t* row_col;      // and its lowest nearest column
  uint32_t* status;
};
struct WalkSets {
  WalkArgs d[2];
};

// Exact FP64 nearest neighbour of each walked row: thread per row,
// depth-first with the nearer child first and the farther one stacked with
// its bound (one entry per level: the tree is at most 64 levels deep).
// A subtree is skipped when its bound exceeds the best distance so far
// (never when equal, so that the lowest column among ties is found); the
// walk stops once its best (an upper bound of the row's distance) is
// strictly below the running maximum.
template <int D>
__global__ void __launch_bounds__(kWalkThreads) k_f64_walk(WalkSets ws) {
  const WalkArgs& w = ws.d[blockIdx.y];
  const uint64_t k = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x;
  if (k >= w.n_rows) return;
  uint32_t row;
  double best = INFINITY;
  if (w.list) {
    const RowEntry e = w.list[k];
    row = e.row;
    best = upper_from32<D>(__uint_as_float(e.min32), w.rxy);
  } else {
    row = (uint32_t) k;
  }
  double x[D];
#pragma unroll
  for (int i = 0; i < D; ++i) x[i] = w.X[(uint64_t) row * D + i];
  uint32_t col = 0xFFFFFFFFu;
  uint32_t stk[kWalkStack];
  double slb[kWalkStack];
  int sp = 0;
  uint32_t node = *w.t.root;
  bool have = true;
  bool stopped = best < bits_d(ld_relaxed_u64(&w.f->max64));
  while (!stopped) {
    if (!have) {
      if (sp == 0) break;
      --sp;
      if (slb[sp] > best) continue;
      node = stk[sp];
    }
    have = true;
    if (node & kLeafBit) {
      const uint64_t p0 = (uint64_t) (node & ~kLeafBit) * w.t.leaf;
      const uint32_t cnt = (uint32_t) min((uint64_t) w.t.leaf, w.t.n - p0);
      for (uint32_t t = 0; t < cnt; ++t) {
        const uint32_t j = __float_as_uint(w.t.pts[p0 + t].w);
        double y[D];
#pragma unroll
        for (int i = 0; i < D; ++i) y[i] = w.Y[(uint64_t) j * D + i];
        const double d = d2_64<D>(x, y);
        if (d < best || (d == best && j < col)) {
          best = d;
          col = j;
        }
      }
      have = false;
      if (best < bits_d(ld_relaxed_u64(&w.f->max64))) stopped = true;
      continue;
    }
    const float4* nd = w.t.nodes + 4 * (uint64_t) node;
    const float4 n0 = nd[0], n1 = nd[1], n3 = nd[3];
    const float4 n2 = D == 3 ? nd[2] : make_float4(0.f, 0.f, 0.f, 0.f);
    const double lbL = box_lb64<D>(x, n0, n2.x, n2.y, w.ry);
    const double lbR = box_lb64<D>(x, n1, n2.z, n2.w, w.ry);
    const uint32_t left = __float_as_uint(n3.x), right = __float_as_uint(n3.y);
    const bool wL = lbL <= best, wR = lbR <= best;
    if (wL && wR) {
      if (sp == kWalkStack) {
        atomicOr(w.status, kErrInternal);
        stopped = true;
        break;
      }
      const bool nearL = lbL <= lbR;
      stk[sp] = nearL ? right : left;
      slb[sp] = nearL ? lbR : lbL;
      ++sp;
      node = nearL ? left : right;
    } else if (wL) {
      node = left;
    } else if (wR) {
      node = right;
    } else {
      have = false;
    }
  }
  if (stopped) {
    w.row_min[k] = -1.0;
    w.row_col[k] = 0u;
    return;
  }
  if (col == 0xFFFFFFFFu) {
    // The starting bound guarantees a point at or below it.
    atomicOr(w.status, kErrInternal);
    w.row_min[k] = -1.0;
    w.row_col[k] = 0u;
    return;
  }
  w.row_min[k] = best;
  w.row_col[k] = col;
  atomicMax(&w.f->max64, dbits(best));
}

// Frozen thresholds from the seeds (thread per direction).
__global__ void k_f64_prepare(F64Aux* aux, int count, int D, double rxy0, double rxy1) {
  const int k = threadIdx.x;
  if (k >= count) return;
  const double rxy = k == 0 ? rxy0 : rxy1;
  F64Dir& f = aux->dir[k];
  const double L = aux->seed_min[k];
  DevScalars z;
  memset(&z, 0, sizeof(z));
  z.min_key = ~0ull;
  if (L < 0.0) z.status = kErrInternal;  // a seed walk cannot stop
  f.seed_d2 = L;
  f.seed_row = aux->seed[k].row;
  f.seed_col = aux->seed_col[k];
  float T = -1.0f;
  if (L >= 0x1p-1000) {
    const double S = sqrt(L) * (1.0 - kMargin) - rxy;
    if (S > 0.0) {
      const double td =
          S * S * (1.0 - (D + 2) * 0x1p-24) * (1.0 - kMargin) - (D + 2) * 0x1p-126;
      if (td > 0.0) T = td >= (double) FLT_MAX ? FLT_MAX : __double2float_rd(td);
    }
  }
  f.thr = T;
  z.max_key = T >= 0.0f ? pack_max(T, 0u) : 0ull;
  aux->frozen[k] = z;
}

// FP64 scan: thread per row of X, every warp visiting Y from its own start
// (broadcast loads); EB stops a row once its minimum is strictly below the
// running maximum.  D = 0: n_dims at run time.
template <int D, bool EB>
__global__ void __launch_bounds__(kScanThreads)
    k_f64_scan(const double* __restrict__ X, uint64_t row_begin, uint64_t row_end,
               const double* __restrict__ Y, uint64_t nY, int dims, F64Dir* f,
               double* __restrict__ row_min, uint32_t* __restrict__ row_col) {
  const uint64_t i = row_begin + blockIdx.x * (uint64_t) blockDim.x + threadIdx.x;
  if (i >= row_end) return;
  const int nd = D ? D : dims;
  double x[D ? D : 1];
  if (D) {
#pragma unroll
    for (int k = 0; k < (D ? D : 1); ++k) x[k] = X[i * nd + k];
  }
  const double* xr = X + i * nd;
  const uint64_t j0 = ((i >> 5) * 2654435761ull) % nY;
  double best = INFINITY;
  uint32_t col = 0xFFFFFFFFu;
  bool stopped = false;
  uint64_t j = j0;
  for (uint64_t t = 0; t < nY; ++t) {
    double d;
    if (D) {
      double y[D ? D : 1];
#pragma unroll
      for (int k = 0; k < (D ? D : 1); ++k) y[k] = __ldg(Y + j * nd + k);
      d = d2_64<D ? D : 1>(x, y);
    } else {
      const double* yr = Y + j * nd;
      double e = __dsub_rn(xr[0], __ldg(yr));
      d = __dmul_rn(e, e);
      for (int k = 1; k < nd; ++k) {
        e = __dsub_rn(xr[k], __ldg(yr + k));
        d = __dadd_rn(d, __dmul_rn(e, e));
      }
    }
    if (d < best || (d == best && (uint32_t) j < col)) {
      best = d;
      col = (uint32_t) j;
    }
    if (++j == nY) j = 0;
    if (EB && (t & 63) == 63 && best < bits_d(ld_relaxed_u64(&f->max64))) {
      stopped = true;
      break;
    }
  }
  if (stopped) {
    row_min[i] = -1.0;
    row_col[i] = 0u;
    return;
  }
  row_min[i] = best;
  row_col[i] = col;
  atomicMax(&f->max64, dbits(best));
}

// The answer: the lowest row whose completed distance equals the maximum
// (and its column); the seed row takes part when it has one.
__global__ void k_f64_pick(const double* __restrict__ row_min, const uint32_t* __restrict__ row_col,
                           const RowEntry* __restrict__ list, uint64_t n, F64Dir* f) {
  const unsigned long long m = f->max64;
  unsigned long long best = ~0ull;
  for (uint64_t k = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; k < n;
       k += (uint64_t) gridDim.x * blockDim.x) {
    const double v = row_min[k];
    if (v >= 0.0 && dbits(v) == m) {
      const uint32_t row = list ? list[k].row : (uint32_t) k;
      const unsigned long long key = ((unsigned long long) row << 32) | row_col[k];
      best = key < best ? key : best;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0 && f->seed_d2 >= 0.0 && dbits(f->seed_d2) == m) {
    const unsigned long long key = ((unsigned long long) f->seed_row << 32) | f->seed_col;
    best = key < best ? key : best;
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    const unsigned long long v = __shfl_xor_sync(0xFFFFFFFFu, best, o);
    best = v < best ? v : best;
  }
  if ((threadIdx.x & 31) == 0 && best != ~0ull) atomicMin(&f->pick, best);
}

// Per-call host state shared with f64_seed.
struct F64Call {
  const double* X[2];
  const double* Y[2];
  double ry[2], rxy[2];
  int dims;
  F64Aux* aux;
  double* seed_min;
  uint32_t* seed_col;
};

hd_status launch_walks(Ctx& c, const WalkSets& ws, int count, uint64_t max_rows, int dims) {
  if (max_rows == 0) return HD_OK;
  const dim3 grid((unsigned) ((max_rows + kWalkThreads - 1) / kWalkThreads), count);
  if (dims == 2)
    k_f64_walk<2><<<grid, kWalkThreads, 0, c.stream>>>(ws);
  else
    k_f64_walk<3><<<grid, kWalkThreads, 0, c.stream>>>(ws);
  return after_launch(c, "f64_walk");
}

template <int D>
hd_status launch_scan(Ctx& c, bool eb, const double* X, uint64_t nX, const double* Y, uint64_t nY,
                      int dims, F64Dir* f, double* row_min, uint32_t* row_col) {
  auto kern = eb ? k_f64_scan<D, true> : k_f64_scan<D, false>;
  // EB: a first wave of one CTA per SM seeds the running maximum before the
  // remaining rows start.
  const uint64_t first = eb ? std::min<uint64_t>(nX, (uint64_t) c.num_sms * kScanThreads) : nX;
  uint64_t b = 0;
  for (uint64_t e : {first, nX}) {
    if (e <= b) continue;
    const unsigned blocks = (unsigned) ((e - b + kScanThreads - 1) / kScanThreads);
    kern<<<blocks, kScanThreads, 0, c.stream>>>(X, b, e, Y, nY, dims, f, row_min, row_col);
    hd_status s = after_launch(c, "f64_scan");
    if (s != HD_OK) return s;
    b = e;
  }
  return HD_OK;
}

hd_status pick(Ctx& c, const double* row_min, const uint32_t* row_col, const RowEntry* list,
               uint64_t n, F64Dir* f) {
  const int grid = (int) std::max<uint64_t>(
      1, std::min<uint64_t>((n + 255) / 256, (uint64_t) c.num_sms * 4));
  k_f64_pick<<<grid, 256, 0, c.stream>>>(row_min, row_col, list, n, f);
  return after_launch(c, "f64_pick");
}

hd_status status_of(Ctx& c, uint32_t st) {
  if (st & kErrWaitTimeout) return fail(c, HD_ERR_DEVICE_TIMEOUT, "a bounded device wait ran out");
  if (st & kErrQueueOverflow) return fail(c, HD_ERR_CUDA, "device queue overflow");
  if (st & kErrInternal) return fail(c, HD_ERR_CUDA, "internal consistency check failed");
  return HD_OK;
}

}  // namespace

// Seed walks and frozen thresholds (called by the LBVH solve once the FP32
// directions are certified).
hd_status f64_seed(Ctx& c, F64Plan& plan, int count) {
  F64Call& call = *reinterpret_cast<F64Call*>(plan.state);
  k_f64_seed_entries<<<1, 32, 0, c.stream>>>(scalars(c, 0), call.aux, count);
  hd_status s = after_launch(c, "f64_seed_entries");
  if (s != HD_OK) return s;
  WalkSets ws;
  for (int k = 0; k < count; ++k) {
    WalkArgs& w = ws.d[k];
    w.X = call.X[k];
    w.Y = call.Y[k];
    w.t = plan.tree[k];
    w.list = &call.aux->seed[k];
    w.n_rows = 1;
    w.ry = call.ry[k];
    w.rxy = call.rxy[k];
    w.f = &call.aux->dir[k];
    w.row_min = call.seed_min + k;
    w.row_col = call.seed_col + k;
    // k_f64_prepare rewrites the frozen scalars after this walk: its errors
    // go to the direction's own scalars.
    w.status = &scalars(c, k)->status;
  }
  if (count == 1) ws.d[1] = ws.d[0];
  if ((s = launch_walks(c, ws, count, 1, call.dims)) != HD_OK) return s;
  k_f64_prepare<<<1, 32, 0, c.stream>>>(call.aux, count, call.dims, call.rxy[0],
                                        count > 1 ? call.rxy[1] : 0.0);
  return after_launch(c, "f64_prepare");
}

}  // namespace hdg

using namespace hdg;

extern "C" {

hd_status hd_solve_f64(hd_ctx* c, const double* A, uint64_t n_a, const double* B,
                       uint64_t n_b, int n_dims, uint32_t flags, int variant, hd_result* out) {
  if (!c) return HD_ERR_INVALID_ARG;
  c->last_error.clear();
  if (!out || !A || !B) return fail(*c, HD_ERR_INVALID_ARG, "null pointer argument");
  if (n_a == 0 || n_b == 0) return fail(*c, HD_ERR_INVALID_ARG, "empty point set");
  if (n_a >= 0xFFFFFFFFull || n_b >= 0xFFFFFFFFull)
    return fail(*c, HD_ERR_INVALID_ARG, "point sets are limited to 2^32-2 points");
  if (n_dims < 1 || n_dims > 256)
    return fail(*c, HD_ERR_INVALID_ARG, "n_dims must be in [1, 256]");
  if (flags & ~(HD_UNDIRECTED | HD_DEVICE_PTRS | HD_COUNT_PAIRS | HD_TIMING))
    return fail(*c, HD_ERR_INVALID_ARG, "unknown flag bits");
  if (variant < 0) variant = c->opt.variant;
  if (variant > HD_VARIANT_BRUTE) return fail(*c, HD_ERR_INVALID_ARG, "unknown variant");
  if (variant == HD_VARIANT_GRID || variant == HD_VARIANT_BF16)
    return fail(*c, HD_ERR_UNSUPPORTED,
                "the FP64 input path takes the auto, lbvh, eb and brute variants");
  const bool spatial_dims = n_dims == 2 || n_dims == 3;
  if (variant == HD_VARIANT_LBVH && !spatial_dims)
    return fail(*c, HD_ERR_UNSUPPORTED, "the LBVH variant needs n_dims 2 or 3");
  cudaSetDevice(c->device);
  memset(out, 0, sizeof(*out));
  out->hd_ba = -1.0;
  c->timing = (flags & HD_TIMING) != 0;
  c->sorted_valid = false;
  c->ev_base = 0;
  if (c->timing) cudaEventRecord(c->ev[24], c->stream);
  const bool undirected = (flags & HD_UNDIRECTED) != 0;
  const int ndir = undirected ? 2 : 1;
  const uint64_t nn[2] = {n_a, n_b};
  hd_status s;

  // Inputs on the device.
  const double* d64[2] = {A, B};
  if (!(flags & HD_DEVICE_PTRS)) {
    for (int k = 0; k < 2; ++k) {
      void* p;
      const size_t bytes = (size_t) nn[k] * n_dims * sizeof(double);
      if ((s = ensure(*c, k == 0 ? kBufF64A : kBufF64B, bytes, &p)) != HD_OK) return s;
      cudaError_t e = cudaMemcpyAsync(p, k == 0 ? A : B, bytes, cudaMemcpyHostToDevice, c->stream);
      if (e != cudaSuccess) return cuda_fail(*c, e, "copy inputs to device");
      d64[k] = (const double*) p;
    }
  }
  void* auxp;
  const size_t list_bytes = (size_t) kListCap * sizeof(RowEntry);
  if ((s = ensure(*c, kBufF64Aux, kAuxBytes + 2 * list_bytes, &auxp)) != HD_OK) return s;
  F64Aux* aux = (F64Aux*) auxp;
  RowEntry* lists = (RowEntry*) ((char*) auxp + kAuxBytes);
  if ((s = init_scalars(*c)) != HD_OK) return s;
  k_f64_init<<<1, 32, 0, c->stream>>>(aux);
  if ((s = after_launch(*c, "f64_init")) != HD_OK) return s;

  // Round both sets to float (into the FP32 path's input buffers) and
  // measure the rounding; the scan route only checks the values.
  bool lbvh = spatial_dims && (variant == HD_VARIANT_AUTO || variant == HD_VARIANT_LBVH);
  const float* f32[2] = {nullptr, nullptr};
  for (int k = 0; k < 2; ++k) {
    void* p = nullptr;
    if (lbvh && (s = ensure(*c, k == 0 ? kBufA : kBufB, (size_t) nn[k] * n_dims * 4, &p)) != HD_OK)
      return s;
    f32[k] = (const float*) p;
    const uint64_t total = nn[k] * (uint64_t) n_dims;
    const int grid =
        (int) std::max<uint64_t>(1, std::min<uint64_t>((total + 255) / 256, (uint64_t) c->num_sms * 8));
    k_f64_round<<<grid, 256, 0, c->stream>>>(d64[k], total, (float*) p, &aux->round[k]);
    if ((s = after_launch(*c, "f64_round")) != HD_OK) return s;
  }
  static_assert(sizeof(F64Aux) + 1024 <= 4096, "pinned staging");
  F64Aux* h = reinterpret_cast<F64Aux*>((char*) c->host_pinned + 1024);
  auto read_aux = [&]() -> hd_status {
    cudaError_t e = cudaMemcpyAsync(h, aux, sizeof(F64Aux), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    return e == cudaSuccess ? HD_OK : cuda_fail(*c, e, "f64 read-back");
  };
  if ((s = read_aux()) != HD_OK) return s;
  const uint32_t rflags = h->round[0].flags | h->round[1].flags;
  if (rflags & kF64NonFinite) return fail(*c, HD_ERR_INVALID_ARG, "NaN or infinite coordinate");
  if (lbvh && (rflags & kF64Range)) {
    if (variant == HD_VARIANT_LBVH)
      return fail(*c, HD_ERR_UNSUPPORTED,
                  "coordinates beyond +-1e18 need the eb or brute variant on the FP64 path");
    lbvh = false;
  }
  double rset[2];
  for (int k = 0; k < 2; ++k) {
    double dm;
    std::memcpy(&dm, &h->round[k].dmax, sizeof(dm));
    rset[k] = std::sqrt((double) n_dims) * dm * (1.0 + kMargin);
  }

  int used = lbvh ? HD_VARIANT_LBVH : (variant == HD_VARIANT_BRUTE ? HD_VARIANT_BRUTE : HD_VARIANT_EB);
  uint64_t walked[2] = {0, 0};
  if (lbvh) {
    F64Call call;
    call.dims = n_dims;
    call.aux = aux;
    call.seed_min = aux->seed_min;
    call.seed_col = aux->seed_col;
    DirInput ins[2];
    for (int k = 0; k < ndir; ++k) {
      call.X[k] = d64[k];
      call.Y[k] = d64[1 - k];
      call.ry[k] = rset[1 - k];
      call.rxy[k] = (rset[0] + rset[1]) * (1.0 + kMargin);
      ins[k] = DirInput{f32[k], nn[k], f32[1 - k], nn[1 - k], n_dims, k,
                        (flags & HD_COUNT_PAIRS) != 0};
    }
    F64Plan plan;
    std::memset(&plan, 0, sizeof(plan));
    plan.cand_cap = kListCap;
    plan.state = &call;
    for (int k = 0; k < ndir; ++k) {
      plan.frozen[k] = &aux->frozen[k];
      plan.cand[k] = lists + (size_t) k * kListCap;
      plan.cand_count[k] = &aux->dir[k].cand_count;
    }
    if ((s = run_lbvh_f64(*c, ins, ndir, &plan)) != HD_OK) return s;
    if ((s = read_aux()) != HD_OK) return s;
    DevScalars hs[2];
    cudaError_t e = cudaMemcpy(hs, scalars(*c, 0), sizeof(hs), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(*c, e, "f64 read-back");
    for (int k = 0; k < ndir; ++k) {
      if ((s = status_of(*c, hs[k].status | h->frozen[k].status)) != HD_OK) return s;
      out->visited_pairs += hs[k].pairs;
      out->visited_nodes += hs[k].nodes;
      out->visited_leaves += hs[k].leaves;
    }
    // Walk the listed rows, or every row when a list overflowed.
    uint64_t off[2] = {0, 0}, total = 0;
    for (int k = 0; k < ndir; ++k) {
      walked[k] = h->dir[k].cand_count <= kListCap ? h->dir[k].cand_count : nn[k];
      off[k] = total;
      total += walked[k];
    }
    void* rows;
    if ((s = ensure(*c, kBufF64Rows, total * (sizeof(double) + sizeof(uint32_t)) + 16, &rows)) !=
        HD_OK)
      return s;
    double* row_min = (double*) rows;
    uint32_t* row_col = (uint32_t*) (row_min + total);
    WalkSets ws;
    for (int k = 0; k < ndir; ++k) {
      WalkArgs& w = ws.d[k];
      w.X = call.X[k];
      w.Y = call.Y[k];
      w.t = plan.tree[k];
      w.list = h->dir[k].cand_count <= kListCap ? plan.cand[k] : nullptr;
      w.n_rows = walked[k];
      w.ry = call.ry[k];
      w.rxy = call.rxy[k];
      w.f = &aux->dir[k];
      w.row_min = row_min + off[k];
      w.row_col = row_col + off[k];
      w.status = &aux->frozen[k].status;
    }
    if (ndir == 1) ws.d[1] = ws.d[0];
    if ((s = launch_walks(*c, ws, ndir, std::max(walked[0], walked[1]), n_dims)) != HD_OK)
      return s;
    for (int k = 0; k < ndir; ++k)
      if ((s = pick(*c, ws.d[k].row_min, ws.d[k].row_col, ws.d[k].list, walked[k],
                    &aux->dir[k])) != HD_OK)
        return s;
  } else {
    void* rows;
    const uint64_t total = n_a + (undirected ? n_b : 0);
    if ((s = ensure(*c, kBufF64Rows, total * (sizeof(double) + sizeof(uint32_t)) + 16, &rows)) !=
        HD_OK)
      return s;
    double* row_min = (double*) rows;
    uint32_t* row_col = (uint32_t*) (row_min + total);
    uint64_t off = 0;
    const bool eb = used == HD_VARIANT_EB;
    for (int k = 0; k < ndir; ++k) {
      const double* X = d64[k];
      const double* Y = d64[1 - k];
      F64Dir* f = &aux->dir[k];
      if (n_dims == 2)
        s = launch_scan<2>(*c, eb, X, nn[k], Y, nn[1 - k], n_dims, f, row_min + off, row_col + off);
      else if (n_dims == 3)
        s = launch_scan<3>(*c, eb, X, nn[k], Y, nn[1 - k], n_dims, f, row_min + off, row_col + off);
      else
        s = launch_scan<0>(*c, eb, X, nn[k], Y, nn[1 - k], n_dims, f, row_min + off, row_col + off);
      if (s != HD_OK) return s;
      if ((s = pick(*c, row_min + off, row_col + off, nullptr, nn[k], f)) != HD_OK) return s;
      walked[k] = nn[k];
      off += nn[k];
    }
  }
  if (c->timing) cudaEventRecord(c->ev[25], c->stream);
  if ((s = read_aux()) != HD_OK) return s;
  if (lbvh)
    for (int k = 0; k < ndir; ++k)
      if ((s = status_of(*c, h->frozen[k].status)) != HD_OK) return s;
  double v[2] = {-1.0, -1.0};
  for (int k = 0; k < ndir; ++k) {
    std::memcpy(&v[k], &h->dir[k].max64, sizeof(double));
    if (h->dir[k].pick == ~0ull) return fail(*c, HD_ERR_CUDA, "internal consistency check failed");
  }
  out->hd_ab = std::sqrt(v[0]);
  int win = 0;
  if (undirected) {
    out->hd_ba = std::sqrt(v[1]);
    if (v[1] > v[0]) win = 1;
  }
  out->hd = std::sqrt(v[win]);
  out->hd_f32 = (float) out->hd;
  out->direction = win;
  out->ia = h->dir[win].pick >> 32;
  out->ib = h->dir[win].pick & 0xFFFFFFFFull;
  out->variant_used = used;
  out->variant_used_ba = undirected ? used : -1;
  out->rechecked = walked[0] + walked[1];
  if (c->timing) {
    float t = 0;
    if (cudaEventElapsedTime(&t, c->ev[24], c->ev[25]) == cudaSuccess) out->ms = t;
  }
  return HD_OK;
}

}  // extern "C"
