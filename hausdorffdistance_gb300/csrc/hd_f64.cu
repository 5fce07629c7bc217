// FP64 input path: the exact FP64 Hausdorff distance of double-precision
// point sets.  The reference declares double point types and a disabled
// -is_double dispatch (src/run_hausdorff_distance.cu:56-62) that would
// instantiate its algorithms with double coordinates and double squared
// distances (the template of src/geoms/distance.h:17-24).
//
// GB300 runs FP64 arithmetic at a small fraction of its FP32 rate, so the
// search stays in FP32 and integer arithmetic, and FP64 is spent only on the
// pair distances FP32 values cannot decide.  Directed h(X, Y), n_dims 2 or 3
// (the LBVH route):
//  1. X and Y are cut to float by dropping mantissa bits (integer
//     operations); a coordinate then moves by less than one float ulp of its
//     magnitude, so with dX = that ulp at the largest exponent of X, a point
//     moves by at most rX = sqrt(D)·dX, and the exact distances of a cut pair
//     and of the original pair differ by at most r = rX + rY.
//  2. The FP32 LBVH solve of the cut sets certifies a row i* and its FP32
//     nearest squared distance M (the FP32 max-min of the cut sets).
//  3. Seed: the exact FP64 nearest neighbour of x_{i*} (the walk below)
//     gives L = min_j d64(x_{i*}, y_j)^2 <= h64^2.
//  4. A float threshold T is derived from L so that every cut pair with FP32
//     squared distance <= T has FP64 squared distance < L: rows with an FP32
//     minimum <= T are settled.  The query pass of step 2 cannot know T, but
//     T >= G(M) >= G(running maximum) for a G that needs M alone (every cut
//     pair of x_{i*} is at FP32 squared distance >= M, which bounds L from
//     below; hd_lbvh.cu's soft_stop computes G rounding toward zero:
//     sqrt(G + a) = sqrt(thr - a)(1 - 1e-5) - 2.01 r, a the absolute term).
//     So that pass stops a row only at or below G(running maximum) and lists
//     every row that stays open with its FP32 minimum; each row with an FP32
//     minimum > T is listed.
//  5. Each listed row with an FP32 minimum > T FP64 nearest neighbour is found by a walk of the
//     same tree, one warp per row: boxes and points are tested in FP32
//     against a float threshold P derived from the row's best FP64 distance
//     (anything above P is provably farther in FP64), and only points within
//     P get an FP64 distance.  A walk stops once its best (an upper bound of
//     its distance) is strictly below the running FP64 maximum (seeded with
//     L).  The answer is the largest completed distance, the lowest row
//     among equal ones, and that row's lowest column.
// When the list overflows (rows that nearly all tie: a lattice and its
// translate) step 5 walks every row.  Other n_dims, coordinates beyond
// +-1e18 and the eb / brute variants use an FP64 scan instead.
//
// Rounding bounds, with u = 2^-24, v = 2^-53 and D + 2 rounded operations
// per squared distance over non-negative terms: an FP32 squared distance
// lies within e^2 (1 -+ u)^(D+2) -+ (D+2) 2^-126 of the exact squared
// distance e^2 of the cut pair (the absolute term covers underflow, even
// with flush to zero), and the same holds for the FP32 squared distance to a
// box; the FP64 formula lies within d^2 (1 -+ v)^(D+2) -+ (D+2) 2^-1074 of
// the exact d^2 of the original pair; and |d - e| <= r.  The code applies
// these with a further relative margin of 2^-40, which covers the rounding
// of its own double arithmetic.
#include <cfloat>
#include <cmath>
#include <cstring>

#include "hd_common.cuh"
#include "hd_internal.h"

namespace hdg {
namespace {

constexpr uint32_t kLeafBit = 0x80000000u;
constexpr uint32_t kListCap = 1u << 20;  // listed rows per direction
// |coordinate| the LBVH route accepts (1e18: FP32 squared distances of cut
// points stay finite for n_dims <= 3).
constexpr unsigned long long kRangeBits = 0x43ABC16D674EC800ull;
constexpr uint32_t kF64NonFinite = 1u, kF64Range = 2u, kF64Tiny = 4u;
constexpr double kMargin = 0x1p-40;
constexpr int kScanThreads = 128;
constexpr int kWalkWarps = 4;
constexpr int kWalkStack = 2048;  // stack entries per warp (shared memory)

struct RoundStats {
  uint32_t emax;   // largest biased double exponent of a coordinate cut to a normal float
  uint32_t flags;  // kF64NonFinite | kF64Range | kF64Tiny (a nonzero |x| < 2^-126)
};

struct F64Dir {
  unsigned long long max64;  // running FP64 maximum (double bits; values >= +0)
  unsigned long long pick;   // (row << 32) | column of the answer (atomicMin)
  double seed_d2;            // the seed row's FP64 nearest squared distance
  uint32_t seed_row, seed_col;
  uint32_t cand_count;       // rows listed by the query pass (may exceed the cap)
  float thr;                 // T: listed rows at or below it are settled (-1: none)
  uint32_t status;           // kErr* of the FP64 kernels
  uint32_t walked;           // rows whose nearest neighbour was searched in FP64
};

// Device layout of kBufF64Aux; the two candidate lists follow it.
struct F64Aux {
  RoundStats round[2];  // per set: 0 = A, 1 = B
  F64Dir dir[2];
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

// x cut to float by integer operations: the sign, the exponent rebiased,
// the top 23 mantissa bits (truncation, |x - cut| < one float ulp of |x|).
// Magnitudes below 2^-126 become a signed zero (displacement < 2^-126);
// magnitudes of 2^128 and above (never on the LBVH route) become infinity.
__device__ __forceinline__ float cut_to_float(double x) {
  const unsigned long long u = dbits(x);
  const uint32_t hi = (uint32_t) (u >> 32);
  const uint32_t ex = (hi >> 20) & 0x7FFu;
  uint32_t f = hi & 0x80000000u;
  if (ex >= 1023u + 128u)
    f |= 0x7F800000u;
  else if (ex >= 1023u - 126u)
    f |= ((ex - 1023u + 127u) << 23) | (uint32_t) ((u >> 29) & 0x7FFFFFu);
  return __uint_as_float(f);
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

// FP32 squared distance of cut points (any correctly rounded order).
template <int D>
__device__ __forceinline__ float d2_32(const float* q, const float4& b) {
  const float dx = __fsub_rn(q[0], b.x), dy = __fsub_rn(q[1], b.y);
  float s = __fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy));
  if (D == 3) {
    const float dz = __fsub_rn(q[2], b.z);
    s = __fadd_rn(s, __fmul_rn(dz, dz));
  }
  return s;
}

// FP32 squared distance from a cut point to a box (0 inside).
template <int D>
__device__ __forceinline__ float box_d2_32(const float* q, const float4& xy, float lz, float hz) {
  const float gx = fmaxf(fmaxf(__fsub_rn(xy.x, q[0]), __fsub_rn(q[0], xy.z)), 0.0f);
  const float gy = fmaxf(fmaxf(__fsub_rn(xy.y, q[1]), __fsub_rn(q[1], xy.w)), 0.0f);
  float s = __fadd_rn(__fmul_rn(gx, gx), __fmul_rn(gy, gy));
  if (D == 3) {
    const float gz = fmaxf(fmaxf(__fsub_rn(lz, q[2]), __fsub_rn(q[2], hz)), 0.0f);
    s = __fadd_rn(s, __fmul_rn(gz, gz));
  }
  return s;
}

// An upper bound of the FP64 nearest squared distance of a row whose FP32
// nearest squared distance over the cut sets is m32 (+inf: none known).
template <int D>
__device__ __forceinline__ double upper_from32(float m32, double rxy) {
  if (!(m32 < INFINITY)) return INFINITY;
  const double e2 = ((double) m32 + (D + 2) * 0x1p-126) / (1.0 - (D + 2) * 0x1p-24);
  const double d = sqrt(e2) * (1.0 + kMargin) + rxy;
  return d * d * (1.0 + kMargin) + 0x1p-1000;
}

// The float threshold P of a row whose best FP64 squared distance so far is
// best: a cut point (or box) whose FP32 squared distance from the cut row
// exceeds P is at FP64 squared distance > best from the row (every original
// point behind it).  +inf while best is unknown.
template <int D>
__device__ __forceinline__ float prune32(double best, double rxy) {
  if (!(best < INFINITY)) return INFINITY;
  const double d = sqrt((best + 0x1p-1000) / (1.0 - kMargin)) * (1.0 + kMargin) + rxy;
  const double p =
      (d * d * (1.0 + (D + 2) * 0x1p-24 * 1.01) + (D + 2) * 0x1p-126) * (1.0 + kMargin);
  return p >= (double) FLT_MAX ? INFINITY : __double2float_ru(p);
}

// Cuts a set to float (Xf may be null: check only); records the largest
// exponent, non-finite and out-of-range values, and tiny magnitudes.
// Integer operations only.
__global__ void k_f64_round(const double* __restrict__ X, uint64_t total, float* __restrict__ Xf,
                            RoundStats* st) {
  uint32_t emax = 0, fl = 0;
  for (uint64_t t = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; t < total;
       t += (uint64_t) gridDim.x * blockDim.x) {
    const double x = X[t];
    const unsigned long long a = dbits(x) & 0x7FFFFFFFFFFFFFFFull;
    const uint32_t ex = (uint32_t) (a >> 52);
    if (ex == 0x7FFu)
      fl |= kF64NonFinite;
    else if (a > kRangeBits)
      fl |= kF64Range;
    if (ex >= 1023u - 126u)
      emax = max(emax, ex);
    else if (a != 0ull)
      fl |= kF64Tiny;
    if (Xf) Xf[t] = cut_to_float(x);
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    emax = max(emax, __shfl_xor_sync(0xFFFFFFFFu, emax, o));
    fl |= __shfl_xor_sync(0xFFFFFFFFu, fl, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (emax) atomicMax(&st->emax, emax);
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
    z.status = 0u;
    z.walked = 0u;
    aux->dir[k] = z;
    aux->round[k].emax = 0u;
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
  LbvhTree t;             // the target's tree over its cut points
  const RowEntry* list;   // rows to walk, or null: every row of X
  uint64_t n_rows;
  double rxy;             // bound on |d(x, y) - d(cut x, cut y)|
  F64Dir* f;
  double* row_min;        // per walked row: FP64 nearest squared distance, -1 if stopped
  uint32_t* row_col;      // and its lowest nearest column
  uint32_t* status;
};
struct WalkSets {
  WalkArgs d[2];
};

// The lexicographically smaller of (d, j) over the warp.
__device__ __forceinline__ void warp_min_pair(double& d, uint32_t& j) {
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    const double od = __shfl_xor_sync(0xFFFFFFFFu, d, o);
    const uint32_t oj = __shfl_xor_sync(0xFFFFFFFFu, j, o);
    if (od < d || (od == d && oj < j)) {
      d = od;
      j = oj;
    }
  }
}

// Exact FP64 nearest neighbour of each walked row, one warp per row.  Up to
// 32 stacked subtrees are expanded per step (one per lane; the stack lives in
// shared memory); a subtree or point is skipped when its FP32 squared
// distance from the cut row exceeds the row's threshold P (never when its
// FP64 distance could equal the best, so that the lowest column among ties
// is found); points within P get their FP64 distance.  A row without a
// starting bound first descends to the nearest leaf along one path.  The
// walk stops once the best (an upper bound of the row's distance) is
// strictly below the running maximum.  A walk that would overflow the stack
// sets kErrInternal (the solve fails) rather than drop a subtree.
template <int D>
__global__ void __launch_bounds__(kWalkWarps * 32) k_f64_walk(WalkSets ws) {
  __shared__ uint32_t stk[kWalkWarps][kWalkStack];
  const WalkArgs& w = ws.d[blockIdx.y];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint64_t k = blockIdx.x * (uint64_t) kWalkWarps + warp;
  if (k >= w.n_rows) return;
  uint32_t* st = stk[warp];
  uint32_t row;
  double best = INFINITY;
  if (w.list) {
    const RowEntry e = w.list[k];
    row = e.row;
    // Listed rows at or below T are settled below the seed (the seed walk
    // itself runs before T exists: thr is -1 then).
    const float T = w.f->thr;
    if (T >= 0.0f && __uint_as_float(e.min32) <= T) {
      if (lane == 0) {
        w.row_min[k] = -1.0;
        w.row_col[k] = 0u;
      }
      return;
    }
    best = upper_from32<D>(__uint_as_float(e.min32), w.rxy);
    if (lane == 0) atomicAdd(&w.f->walked, 1u);
  } else {
    row = (uint32_t) k;
  }
  double x[D];
  float q[D];
#pragma unroll
  for (int i = 0; i < D; ++i) {
    x[i] = w.X[(uint64_t) row * D + i];
    q[i] = cut_to_float(x[i]);
  }
  uint32_t col = 0xFFFFFFFFu;
  float P = prune32<D>(best, w.rxy);
  auto read_max = [&]() {
    unsigned long long m = 0;
    if (lane == 0) m = ld_relaxed_u64(&w.f->max64);
    return bits_d(__shfl_sync(0xFFFFFFFFu, m, 0));
  };
  // Scans leaf `leaf` on this lane: FP64 distances of its points within P.
  auto scan_leaf = [&](uint32_t leaf, double& lb, uint32_t& lc) {
    const uint64_t p0 = (uint64_t) leaf * w.t.leaf;
    const uint32_t cnt = (uint32_t) min((uint64_t) w.t.leaf, w.t.n - p0);
    for (uint32_t t = 0; t < cnt; ++t) {
      const float4 b = w.t.pts[p0 + t];
      if (d2_32<D>(q, b) > P) continue;
      const uint32_t j = __float_as_uint(b.w);
      double y[D];
#pragma unroll
      for (int i = 0; i < D; ++i) y[i] = w.Y[(uint64_t) j * D + i];
      const double d = d2_64<D>(x, y);
      if (d < lb || (d == lb && j < lc)) {
        lb = d;
        lc = j;
      }
    }
  };
  uint32_t root = *w.t.root;
  if (!(best < INFINITY)) {
    // No bound yet: lane 0 follows the nearer child down to a leaf, whose
    // scan gives one.
    uint32_t node = root;
    if (lane == 0) {
      while (!(node & kLeafBit)) {
        const float4* nd = w.t.nodes + 4 * (uint64_t) node;
        const float4 n0 = nd[0], n1 = nd[1], n3 = nd[3];
        const float4 n2 = D == 3 ? nd[2] : make_float4(0.f, 0.f, 0.f, 0.f);
        const float dL = box_d2_32<D>(q, n0, n2.x, n2.y);
        const float dR = box_d2_32<D>(q, n1, n2.z, n2.w);
        node = __float_as_uint(dL <= dR ? n3.x : n3.y);
      }
    }
    node = __shfl_sync(0xFFFFFFFFu, node, 0);
    double lb = INFINITY;
    uint32_t lc = 0xFFFFFFFFu;
    if (lane == 0) scan_leaf(node & ~kLeafBit, lb, lc);
    lb = __shfl_sync(0xFFFFFFFFu, lb, 0);
    lc = __shfl_sync(0xFFFFFFFFu, lc, 0);
    best = lb;
    col = lc;
    // P stays +inf until a point is found (a leaf scan with P = +inf
    // evaluates every point, so one was).
    P = prune32<D>(best, w.rxy);
  }
  bool stopped = best < read_max();
  if (lane == 0) st[0] = root;
  int sp = 1;
  __syncwarp();
  int round = 0;
  while (sp > 0 && !stopped) {
    const int take = min(sp, 32);
    const bool has = lane < take;
    const uint32_t node = has ? st[sp - take + lane] : 0u;
    sp -= take;
    __syncwarp();
    uint32_t push0 = 0, push1 = 0;
    int npush = 0;
    double lb = best;
    uint32_t lc = col;
    if (has) {
      if (node & kLeafBit) {
        scan_leaf(node & ~kLeafBit, lb, lc);
      } else {
        const float4* nd = w.t.nodes + 4 * (uint64_t) node;
        const float4 n0 = nd[0], n1 = nd[1], n3 = nd[3];
        const float4 n2 = D == 3 ? nd[2] : make_float4(0.f, 0.f, 0.f, 0.f);
        const float dL = box_d2_32<D>(q, n0, n2.x, n2.y);
        const float dR = box_d2_32<D>(q, n1, n2.z, n2.w);
        const uint32_t left = __float_as_uint(n3.x), right = __float_as_uint(n3.y);
        const bool wL = dL <= P, wR = dR <= P;
        // Nearer child pushed last, so that it is popped first.
        if (wL && wR) {
          push0 = dL <= dR ? right : left;
          push1 = dL <= dR ? left : right;
          npush = 2;
        } else if (wL || wR) {
          push0 = wL ? left : right;
          npush = 1;
        }
      }
    }
    warp_min_pair(lb, lc);
    if (lb < best || (lb == best && lc < col)) {
      best = lb;
      col = lc;
      P = prune32<D>(best, w.rxy);
    }
    // Compact the pushes: lanes in order, two slots per lane at most.
    int off = npush;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xFFFFFFFFu, off, o);
      if (lane >= o) off += v;
    }
    const int total = __shfl_sync(0xFFFFFFFFu, off, 31);
    off -= npush;
    if (sp + total > kWalkStack) {
      if (lane == 0) atomicOr(w.status, kErrInternal);
      stopped = true;
      break;
    }
    if (npush > 0) st[sp + off] = push0;
    if (npush > 1) st[sp + off + 1] = push1;
    sp += total;
    __syncwarp();
    if ((++round & 7) == 0 && best < read_max()) stopped = true;
  }
  if (!stopped && best < read_max()) stopped = true;
  if (lane != 0) return;
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

// T from the seeds (thread per direction).
__global__ void k_f64_prepare(F64Aux* aux, int count, int D, double rxy0, double rxy1) {
  const int k = threadIdx.x;
  if (k >= count) return;
  const double rxy = k == 0 ? rxy0 : rxy1;
  F64Dir& f = aux->dir[k];
  const double L = aux->seed_min[k];
  if (L < 0.0) f.status |= kErrInternal;  // a seed walk cannot stop
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
  double rxy[2];
  int dims;
  F64Aux* aux;
  double* seed_min;
  uint32_t* seed_col;
};

hd_status launch_walks(Ctx& c, const WalkSets& ws, int count, uint64_t max_rows, int dims) {
  if (max_rows == 0) return HD_OK;
  const dim3 grid((unsigned) ((max_rows + kWalkWarps - 1) / kWalkWarps), count);
  if (dims == 2)
    k_f64_walk<2><<<grid, kWalkWarps * 32, 0, c.stream>>>(ws);
  else
    k_f64_walk<3><<<grid, kWalkWarps * 32, 0, c.stream>>>(ws);
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

// Seed walks and T (called by the LBVH solve once the FP32
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
    w.rxy = call.rxy[k];
    w.f = &call.aux->dir[k];
    w.row_min = call.seed_min + k;
    w.row_col = call.seed_col + k;
    w.status = &call.aux->dir[k].status;
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
  // How far a point moves when cut to float: less than one float ulp per
  // coordinate at the set's largest exponent (2^-126 for tiny magnitudes).
  double rset[2];
  for (int k = 0; k < 2; ++k) {
    double dm = 0.0;
    if (h->round[k].emax) dm = std::ldexp(1.0, (int) h->round[k].emax - 1023 - 23);
    if (h->round[k].flags & kF64Tiny) dm = std::max(dm, 0x1p-126);
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
      call.rxy[k] = (rset[0] + rset[1]) * (1.0 + kMargin);
      ins[k] = DirInput{f32[k], nn[k], f32[1 - k], nn[1 - k], n_dims, k,
                        (flags & HD_COUNT_PAIRS) != 0};
    }
    F64Plan plan;
    std::memset(&plan, 0, sizeof(plan));
    plan.cand_cap = kListCap;
    plan.state = &call;
    for (int k = 0; k < ndir; ++k) {
      plan.cand[k] = lists + (size_t) k * kListCap;
      plan.cand_count[k] = &aux->dir[k].cand_count;
      // The bound as a float, rounded up.
      float rf = (float) call.rxy[k];
      if ((double) rf < call.rxy[k]) rf = std::nextafter(rf, INFINITY);
      plan.soft_r[k] = rf;
    }
    if ((s = run_lbvh_f64(*c, ins, ndir, &plan)) != HD_OK) return s;
    if ((s = read_aux()) != HD_OK) return s;
    DevScalars hs[2];
    cudaError_t e = cudaMemcpy(hs, scalars(*c, 0), sizeof(hs), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(*c, e, "f64 read-back");
    for (int k = 0; k < ndir; ++k) {
      if ((s = status_of(*c, hs[k].status | h->dir[k].status)) != HD_OK) return s;
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
      w.rxy = call.rxy[k];
      w.f = &aux->dir[k];
      w.row_min = row_min + off[k];
      w.row_col = row_col + off[k];
      w.status = &aux->dir[k].status;
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
      if ((s = status_of(*c, h->dir[k].status)) != HD_OK) return s;
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
  if (lbvh)
    // Rows searched in FP64: the seed, the listed rows above T, or every row
    // when a list overflowed.
    for (int k = 0; k < ndir; ++k)
      walked[k] = h->dir[k].walked + (h->dir[k].cand_count > kListCap ? nn[k] : 0);
  out->rechecked = walked[0] + walked[1];
  if (c->timing) {
    float t = 0;
    if (cudaEventElapsedTime(&t, c->ev[24], c->ev[25]) == cudaSuccess) out->ms = t;
  }
  return HD_OK;
}

}  // extern "C"
