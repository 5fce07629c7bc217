// LBVH variant: a linear BVH over Morton-sorted B — the binary radix tree of
// Karras ("Maximizing Parallelism in the Construction of BVHs, Octrees, and
// k-d Trees", HPG 2012), built together with its boxes in one agglomerative
// bottom-up pass (Apetrei, CGVC 2014) — and a warp-packet nearest-neighbour
// traversal with early break.
//
// It replaces the reference's OptiX/RT-core search
// (src/hd_impl/hausdorff_distance_ray_tracing.h:63-236 with the programs of
// src/rt/shaders/shaders_nn_uniform_grid_3d.cu:16-180 and the accel
// build/refit of src/rt/rt_engine.h:290-314): GB300 has no RT cores.  The
// reference grows a search radius over rounds and refits its BVH each round
// (hybrid.h:349-371); a nearest-neighbour traversal needs no radius, so the
// tree is built once and every A point is finished in one pass.
//
// Semantics per A point (as the reference's intersection program,
// shaders_nn_uniform_grid_3d.cu:69-105): stop as soon as some B point is at
// or below the running maximum (it cannot raise it), stop a subtree when its
// box is no nearer than the current minimum, and stop outright when a whole
// non-empty box lies within the running maximum (maxDist^2 <= cmax2, the
// shader's :83-86 shortcut, taken here with a relative safety margin so that
// FP32 rounding can never wrongly stop a point).  A point that is never
// stopped ends with its exact nearest-neighbour distance and raises the
// maximum with one 64-bit atomicMax.
//
// Layout in HBM:
//   sorted points  float4 (x, y, z, caller index)       16 B / point
//   leaves         implicit: leaf i = points [i*L, i*L+L), L <= 32
//   nodes          4 x float4 per internal node: (lo.x, lo.y, hi.x, hi.y) of
//                  the left child, the same of the right child, (lo.z, hi.z)
//                  of both, and the two child references (bit 31 set =
//                  leaf)                                               64 B
// A traversal step loads one node (all lanes the same address: one
// broadcast; 2-D trees skip the z quarter) and tests both children for
// every lane of the packet.  x and y of a box sit in aligned register pairs,
// so the box distances use the packed pair instructions.
#include <cfloat>

#include "hd_common.cuh"
#include "hd_internal.h"

namespace hdg {
namespace {

constexpr uint32_t kLeafBit = 0x80000000u;
constexpr int kQueryWarps = 4;
constexpr int kStack = 64;
// Queries per lane of a warp packet (QPL): two for large query sets, where
// every broadcast load then serves 64 queries; one for small sets, whose
// packets would otherwise be too few to fill the GPU.
constexpr uint64_t kQplTwoMinQueries = 4000000;
// A packet that has visited `budget` nodes and leaves (an option, tuned)
// queues its open queries for the deferred pass instead of finishing them
// alone: a query whose nearest neighbour is far (an outlier) must prove that
// a large empty ball is empty, and one warp walking that proof serially would
// hold the whole launch.
constexpr uint32_t kDeferCap = 1u << 16;  // queued queries per direction at most

// A queued query: its position in the sorted query set and its running
// minimum (float bits) when it was queued.
struct Deferred {
  uint32_t item;
  uint32_t gmin;
};

// Common-prefix length of the keys of leaves i and i+1 (i + 1 < nL).  A
// leaf's key is its first point's sorted Morton code with the leaf index
// appended, which makes every key distinct.
__device__ __forceinline__ int leaf_delta(const uint32_t* __restrict__ codes, uint32_t L,
                                          uint32_t i, uint32_t mask) {
  const uint64_t ki = ((uint64_t) (codes[(uint64_t) i * L] & mask) << 32) | (uint64_t) i;
  const uint64_t kj = ((uint64_t) (codes[(uint64_t) (i + 1) * L] & mask) << 32) | (uint64_t) (i + 1);
  return __clzll(ki ^ kj);
}

// Arrival count at a parent with release and acquire semantics (GPU scope):
// it publishes this thread's writes to whichever thread arrives second, and
// the second arriver sees the first one's (the RMW chain on the flag carries
// the synchronisation), without full fences.
__device__ __forceinline__ uint32_t arrive_acq_rel(uint32_t* p) {
  uint32_t old;
  asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], 1;" : "=r"(old) : "l"(p) : "memory");
  return old;
}

// Agglomerative build of the binary radix tree over the leaves' keys, with
// boxes, in one bottom-up pass (after Apetrei, "Fast and Simple Agglomerative
// LBVH Construction", CGVC 2014): it yields the tree of Karras' construction
// (HPG 2012) without its per-node searches.  A thread starts at a leaf with
// the range [l, r] = [i, i].  The node's parent is internal node r (the node
// is its left child) when the key pair (r, r+1) shares a longer prefix than
// (l-1, l), else internal node l-1 (right child); the ends of the array
// decide alone.  Each arriver writes its half of the parent's packed node
// (its box and reference) and its outer range bound, then arrives; the first
// to arrive stops, the second reads its sibling's half, forms the union box
// and climbs with the merged range.  The thread that completes [0, nL-1]
// records the root.
__device__ __forceinline__ void agglomerate_body(const uint32_t* __restrict__ codes, uint32_t L,
                                                 uint32_t nL,
                                                 const float4* __restrict__ leaf_boxes,
                                                 uint32_t* flags, uint32_t* bound, uint32_t* root,
                                                 float4* nodes, uint32_t mask) {
  const uint32_t leaf = blockIdx.x * blockDim.x + threadIdx.x;
  if (nL == 1) {
    // Single leaf: a root whose right child is an empty box (never visited).
    if (leaf == 0) {
      const float4 lo = leaf_boxes[0], hi = leaf_boxes[1];
      nodes[0] = make_float4(lo.x, lo.y, hi.x, hi.y);
      nodes[1] = make_float4(FLT_MAX, FLT_MAX, -FLT_MAX, -FLT_MAX);
      nodes[2] = make_float4(lo.z, hi.z, FLT_MAX, -FLT_MAX);
      nodes[3] = make_float4(__uint_as_float(kLeafBit), __uint_as_float(kLeafBit), 0.f, 0.f);
      *root = 0;
    }
    return;
  }
  if (leaf >= nL) return;
  float4 lo = leaf_boxes[2 * (uint64_t) leaf], hi = leaf_boxes[2 * (uint64_t) leaf + 1];
  uint32_t l = leaf, r = leaf, me = leaf | kLeafBit;
  for (;;) {
    const bool left_child = l == 0 || (r != nL - 1 && leaf_delta(codes, L, r, mask) >
                                                           leaf_delta(codes, L, l - 1, mask));
    const uint32_t p = left_child ? r : l - 1;
    const int side = left_child ? 0 : 1;
    float4* o = nodes + 4 * (uint64_t) p;
    o[side] = make_float4(lo.x, lo.y, hi.x, hi.y);
    reinterpret_cast<float2*>(o + 2)[side] = make_float2(lo.z, hi.z);
    reinterpret_cast<uint32_t*>(o + 3)[side] = me;
    bound[2 * (uint64_t) p + side] = left_child ? l : r;
    if (arrive_acq_rel(&flags[p]) == 0) return;
    const float4 sxy = __ldcg(o + (1 - side));
    const float2 sz = __ldcg(reinterpret_cast<const float2*>(o + 2) + (1 - side));
    const uint32_t other = __ldcg(&bound[2 * (uint64_t) p + (1 - side)]);
    lo = make_float4(fminf(lo.x, sxy.x), fminf(lo.y, sxy.y), fminf(lo.z, sz.x), 0.f);
    hi = make_float4(fmaxf(hi.x, sxy.z), fmaxf(hi.y, sxy.w), fmaxf(hi.z, sz.y), 0.f);
    if (left_child)
      r = other;
    else
      l = other;
    me = p;
    if (l == 0 && r == nL - 1) {
      *root = p;
      return;
    }
  }
}

// Squared distance from q to the box [lo, hi] (0 inside), with xy = (lo.x,
// lo.y, hi.x, hi.y), rounded exactly like the pair formula (same non-fused
// operations in the same order).
// Rounding is monotone, so for every point b in the box this value is <= the
// FP32 squared distance of (p, b): pruning a box whose value is >= the current
// minimum can never skip a strictly smaller pair distance.
template <int D>
__device__ __forceinline__ float box_min_d2(const float4& q, const float4& xy, float lz, float hz) {
  const float2 p = make_float2(q.x, q.y);
  const float2 below = sub2_rn(make_float2(xy.x, xy.y), p);
  const float2 above = sub2_rn(p, make_float2(xy.z, xy.w));
  const float dx = fmaxf(fmaxf(below.x, above.x), 0.0f);
  const float dy = fmaxf(fmaxf(below.y, above.y), 0.0f);
  const float2 sq = __fmul2_rn(make_float2(dx, dy), make_float2(dx, dy));
  float s = __fadd_rn(sq.x, sq.y);
  if constexpr (D == 3) {
    const float dz = fmaxf(fmaxf(__fsub_rn(lz, q.z), __fsub_rn(q.z, hz)), 0.0f);
    s = __fadd_rn(s, __fmul_rn(dz, dz));
  }
  return s;
}

// Largest squared distance from p to the box (an estimate; callers compare
// it with a safety margin).
template <int D>
__device__ __forceinline__ float box_max_d2(const float4& q, const float4& xy, float lz, float hz) {
  float dx = fmaxf(fabsf(q.x - xy.x), fabsf(xy.z - q.x));
  float dy = fmaxf(fabsf(q.y - xy.y), fabsf(xy.w - q.y));
  float s = dx * dx + dy * dy;
  if constexpr (D == 3) {
    float dz = fmaxf(fabsf(q.z - lz), fabsf(hz - q.z));
    s += dz * dz;
  }
  return s;
}

// Safety factor for the "whole box within the maximum" shortcut: the FP32
// box bound and the FP32 pair formula each carry a few ulps of rounding.
constexpr float kMaxDistMargin = 1.0f + 1.0f / 65536.0f;

// The FP64 input path's listing pass stops a row only below soft_stop(thr):
// a lower bound, from the running maximum thr alone, of the threshold under
// which an FP32 distance proves an FP64 distance below the final answer's
// seed (the bound is derived in hd_f64.cu; every step here rounds toward
// zero, r = how far a cut pair's distance can move).  -1: no row stops.
__device__ __forceinline__ float soft_stop(float thr, float r) {
  if (!(thr >= 0.0f)) return -1.0f;
  const float abs32 = 5.0f * 0x1p-126f;  // (n_dims + 2) 2^-126, n_dims <= 3
  const float base = __fsub_rd(thr, abs32);
  if (!(base > 0.0f)) return -1.0f;
  const float sg = __fsub_rd(__fmul_rd(__fsqrt_rd(base), 0.99999f), __fmul_ru(2.01f, r));
  if (!(sg > 0.0f)) return -1.0f;
  const float g = __fsub_rd(__fmul_rd(__fmul_rd(sg, sg), 0.999999f), abs32);
  return g > 0.0f ? g : -1.0f;
}

// Division of a 32-bit value by a run-time constant d, with the multiplier
// m and shifts s1, s2 prepared on the host (Granlund and Montgomery,
// "Division by Invariant Integers using Multiplication", PLDI 1994):
// q = (t + ((n - t) >> s1)) >> s2 with t = umulhi(m, n).
struct FastDiv {
  uint32_t m, s1, s2;
};
static FastDiv make_fastdiv(uint32_t d) {
  uint32_t l = 0;
  while (l < 32 && (1ull << l) < d) ++l;
  const uint64_t m = ((1ull << 32) * ((1ull << l) - d)) / d + 1;
  return FastDiv{(uint32_t) m, l < 1 ? l : 1u, l > 0 ? l - 1 : 0u};
}
// Starts a load of the 128-byte line at p into L1 (a hint: nothing waits
// for it).  Every caller passes an address inside its array.
__device__ __forceinline__ void prefetch_l1(const void* p) {
  asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
}

__device__ __forceinline__ uint32_t fastdiv(uint32_t n, FastDiv f) {
  const uint32_t t = __umulhi(f.m, n);
  return (t + ((n - t) >> f.s1)) >> f.s2;
}

// Warp-packet traversal of 32 * QPL consecutive Morton-sorted queries.
// LT: leaf size known at compile time (16, the tuned size), or 0 for a
// runtime leaf size L.
template <int D, bool COUNT, int LT, int QPL>
__device__ __forceinline__ void lbvh_query_body(const float4* __restrict__ Q, uint64_t nItems, uint32_t pstride,
                 uint64_t rows, FastDiv rows_div, const uint32_t* __restrict__ ppos,
                 const float4* __restrict__ nodes, const float4* __restrict__ B, uint64_t nB,
                 uint32_t L, DevScalars* sc, Deferred* __restrict__ defer, uint32_t budget,
                 uint32_t root, RowEntry* __restrict__ cand, uint32_t* cand_count,
                 uint32_t cand_cap, float soft_r) {
  __shared__ uint32_t stk[kQueryWarps][kStack];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const unsigned below = (1u << lane) - 1u;
  // Packets (kP = 32 * QPL consecutive Morton-sorted queries, QPL per lane:
  // items lane, 32 + lane, ...) are visited in a transposed order: warp w
  // takes packet (w mod rows) * pstride + w / rows.  The first `rows` warps
  // — the first wave — are every pstride-th packet, spread over the whole
  // Morton range, so the running maximum rises to nearly its final value
  // while the bulk of the packets is still queued (the reference samples
  // with EB for the same purpose, hybrid.h:128-168).  Two queries per lane
  // let every broadcast load of a leaf point or a node serve 64 queries and
  // halve the chains of dependent loads per query.
  // 32-bit arithmetic: packet counts stay below 2^27 (point sets < 2^32).
  constexpr uint64_t kP = 32 * QPL;
  const uint32_t w = blockIdx.x * kQueryWarps + warp;
  const uint32_t r32 = (uint32_t) rows;
  const uint32_t wq = fastdiv(w, rows_div);
  const uint64_t packet = (uint64_t) (w - wq * r32) * pstride + wq;
  if (packet * kP >= nItems) return;
  uint64_t item[QPL];
  bool act[QPL];
  float4 q[QPL];
  float cmin[QPL];
#pragma unroll
  for (int h = 0; h < QPL; ++h) {
    item[h] = packet * kP + 32 * h + lane;
    act[h] = item[h] < nItems;
    q[h] = act[h] ? Q[item[h]] : make_float4(0.f, 0.f, 0.f, 0.f);
    cmin[h] = INFINITY;
  }
  float dstk[kStack];
  unsigned long long key = 0;
  if (lane == 0) key = ld_relaxed_u64(&sc->max_key);
  float thr = threshold_of(__shfl_sync(0xFFFFFFFFu, key, 0));
  // A query stops once its minimum is at or below `stop`: the running
  // maximum, or in the listing pass its soft bound.
  float stop = cand ? soft_stop(thr, soft_r) : thr;
  unsigned long long pairs = 0, visits = 0, leafv = 0;
  uint32_t work = 0;  // nodes and leaves this packet has visited
  bool may_defer = defer != nullptr;
  auto open = [&]() {
    bool o = false;
#pragma unroll
    for (int h = 0; h < QPL; ++h) o = o || act[h];
    return o;
  };
  auto count_pairs = [&](uint64_t k) {
#pragma unroll
    for (int h = 0; h < QPL; ++h) pairs += k * (uint64_t) __popc(__ballot_sync(0xFFFFFFFFu, act[h]));
  };
  // Some open query of this lane is above the stop level.
  auto needs = [&](const float* m) {
    bool o = false;
#pragma unroll
    for (int h = 0; h < QPL; ++h) o = o || (act[h] && m[h] > stop);
    return o;
  };
  // Slots of this lane's open queries in a list counted by *counter: one
  // atomic per warp; the open queries of copy h follow those of copy h - 1.
  auto list_slots = [&](uint32_t* counter, uint32_t* slot) {
    unsigned o[QPL];
    uint32_t total = 0;
#pragma unroll
    for (int h = 0; h < QPL; ++h) {
      o[h] = __ballot_sync(0xFFFFFFFFu, act[h]);
      total += __popc(o[h]);
    }
    uint32_t base = 0;
    if (lane == 0 && total) base = atomicAdd(counter, total);
    base = __shfl_sync(0xFFFFFFFFu, base, 0);
#pragma unroll
    for (int h = 0; h < QPL; ++h) {
      slot[h] = base + __popc(o[h] & below);
      base += __popc(o[h]);
    }
  };

  // Scans one leaf with every lane of the packet (points read as broadcast
  // loads, four at a time, each tested against both of a lane's queries);
  // stops as soon as no query still needs a point, and stops the queries
  // that found a point within the running maximum.
  auto scan_leaf = [&](uint32_t leaf) {
    const uint64_t s = (uint64_t) leaf * (LT ? (uint32_t) LT : L);
    const float4* lp = B + s;
    // A full 16-point leaf is two 128-byte lines: start the second now.
    if (LT == 16 && s + 16 <= nB) prefetch_l1(lp + 8);
    float m[QPL];
#pragma unroll
    for (int h = 0; h < QPL; ++h) m[h] = cmin[h];
    int k = 0;
    bool settled = false;  // every open query is within the running maximum
    if (LT && s + LT <= nB) {
      // Full leaf of a compile-time size: fixed offsets, no clamping.
#pragma unroll
      for (int k0 = 0; k0 < (LT ? LT : 4); k0 += 4) {
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const float4 b = __ldg(lp + k0 + u);
#pragma unroll
          for (int h = 0; h < QPL; ++h) m[h] = fminf(m[h], d2_pt_packed<D>(q[h], b));
        }
        k = k0 + 4;
        if (!__any_sync(0xFFFFFFFFu, needs(m))) {
          settled = true;
          break;
        }
      }
    } else {
      const int cnt = (int) min((uint64_t) L, nB - s);
      for (; k < cnt; k += 4) {
        // Every lane reads the same point: one broadcast load per point.
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const float4 b = __ldg(lp + min(k + u, cnt - 1));
#pragma unroll
          for (int h = 0; h < QPL; ++h) m[h] = fminf(m[h], d2_pt_packed<D>(q[h], b));
        }
        if (!__any_sync(0xFFFFFFFFu, needs(m))) {
          k += 4;
          settled = true;
          break;
        }
      }
      k = min(k, cnt);
    }
#pragma unroll
    for (int h = 0; h < QPL; ++h)
      if (act[h]) cmin[h] = m[h];
    ++work;
    if (COUNT) {
      ++leafv;
      count_pairs((uint64_t) k);
    }
    // The running maximum is re-read only when some query is still open.
    if (!settled) {
      if (lane == 0) key = ld_relaxed_u64(&sc->max_key);
      thr = threshold_of(__shfl_sync(0xFFFFFFFFu, key, 0));
      stop = cand ? soft_stop(thr, soft_r) : thr;
    }
#pragma unroll
    for (int h = 0; h < QPL; ++h)
      if (act[h] && cmin[h] <= stop) act[h] = false;
  };

  {
    // Warm start: a query's Morton code in B's frame locates it in B's
    // sorted codes, so the B leaves at the packet's position (precomputed
    // per packet) are spatially close.  Scanning that leaf and its
    // neighbours lets most queries stop before any traversal, and gives the
    // others a small running minimum that prunes the traversal.
    const uint32_t lshift = __ffs(L) - 1;  // L is a power of two
    const uint32_t nL = (uint32_t) ((nB + L - 1) >> lshift);
    // Both ends of the packet are looked up: a packet can straddle a jump of
    // the Morton curve, and then its two ends sit in different regions.
    const uint32_t leaf0 = min(ppos[2 * packet] >> lshift, nL - 1);
    const uint32_t leaf1 = min(ppos[2 * packet + 1] >> lshift, nL - 1);
    scan_leaf(leaf0);
    if (leaf1 != leaf0 && __any_sync(0xFFFFFFFFu, open())) scan_leaf(leaf1);
    if (leaf0 + 1 < nL && leaf0 + 1 != leaf1 && __any_sync(0xFFFFFFFFu, open()))
      scan_leaf(leaf0 + 1);
    if (leaf0 > 0 && __any_sync(0xFFFFFFFFu, open())) scan_leaf(leaf0 - 1);
  }

  int sp = 0;
  uint32_t next = root;
  bool have = true;
  for (;;) {
    if (!__any_sync(0xFFFFFFFFu, open())) break;
    if (may_defer && work >= budget) {
      // Over budget: queue the open queries (as many as the queue holds;
      // queries beyond it finish here, with no budget).
      may_defer = false;
      uint32_t slot[QPL];
      list_slots(&sc->heavy_count, slot);
#pragma unroll
      for (int h = 0; h < QPL; ++h)
        if (act[h] && slot[h] < kDeferCap) {
          defer[slot[h]] = Deferred{(uint32_t) item[h], __float_as_uint(cmin[h])};
          act[h] = false;
        }
      continue;
    }
    if (have && !(next & kLeafBit)) {
      // Internal node: test both children for both queries of every lane.
      const float4* nd = nodes + 4 * (uint64_t) next;
      const float4 n0 = nd[0], n1 = nd[1], n3 = nd[3];
      const float4 n2 = D == 3 ? nd[2] : make_float4(0.f, 0.f, 0.f, 0.f);
      ++work;
      if (COUNT) ++visits;
      // Per lane: the nearest box distance among its queries that want a
      // child (+inf when none does).
      float dLm = INFINITY, dRm = INFINITY;
#pragma unroll
      for (int h = 0; h < QPL; ++h) {
        if (act[h] && stop >= 0.0f) {
          const float mL = box_max_d2<D>(q[h], n0, n2.x, n2.y);
          const float mR = box_max_d2<D>(q[h], n1, n2.z, n2.w);
          if (fminf(mL, mR) * kMaxDistMargin <= stop) act[h] = false;
        }
        const float dL = box_min_d2<D>(q[h], n0, n2.x, n2.y);
        const float dR = box_min_d2<D>(q[h], n1, n2.z, n2.w);
        if (act[h] && dL < cmin[h]) dLm = fminf(dLm, dL);
        if (act[h] && dR < cmin[h]) dRm = fminf(dRm, dR);
      }
      const bool wL = dLm < INFINITY, wR = dRm < INFINITY;
      const uint32_t bL = __ballot_sync(0xFFFFFFFFu, wL);
      const uint32_t bR = __ballot_sync(0xFFFFFFFFu, wR);
      const uint32_t left = __float_as_uint(n3.x), right = __float_as_uint(n3.y);
      if (bL && bR) {
        const int preferL = __popc(__ballot_sync(0xFFFFFFFFu, wL && (!wR || dLm <= dRm)));
        const int preferR = __popc(__ballot_sync(0xFFFFFFFFu, wR && (!wL || dRm < dLm)));
        const bool nearL = preferL >= preferR;
        if (sp < kStack) {
          if (lane == 0) stk[warp][sp] = nearL ? right : left;
          dstk[sp] = nearL ? dRm : dLm;
          ++sp;
        } else if (lane == 0) {
          // Cannot happen: the tree is at most 64 levels deep (distinct
          // 64-bit keys) and one entry is pushed per level.
          atomicOr(&sc->status, kErrInternal);
        }
        __syncwarp();
        next = nearL ? left : right;
      } else if (bL) {
        next = left;
      } else if (bR) {
        next = right;
      } else {
        have = false;
      }
      continue;
    }
    if (have) {
      scan_leaf(next & ~kLeafBit);
      have = false;
      continue;
    }
    // Pop the next subtree any query still needs.  The stacked distance is
    // the nearest of the lane's wanting queries, so a query with a larger
    // minimum may revisit a subtree it does not need (never the converse).
    if (sp == 0) break;
    --sp;
    next = stk[warp][sp];
    bool want = false;
#pragma unroll
    for (int h = 0; h < QPL; ++h) want = want || (act[h] && dstk[sp] < cmin[h]);
    have = __any_sync(0xFFFFFFFFu, want);
  }
  if (cand) {
    // Listing pass (FP64 refinement): the rows still open are listed with
    // their FP32 minima (and raise the maximum like any other).
    uint32_t slot[QPL];
    list_slots(cand_count, slot);
#pragma unroll
    for (int h = 0; h < QPL; ++h)
      if (act[h] && slot[h] < cand_cap)
        cand[slot[h]] = RowEntry{__float_as_uint(q[h].w), __float_as_uint(cmin[h])};
  }
#pragma unroll
  for (int h = 0; h < QPL; ++h)
    if (act[h]) atomicMax(&sc->max_key, pack_max(cmin[h], __float_as_uint(q[h].w)));
  if (COUNT && lane == 0) {
    atomicAdd(&sc->pairs, pairs);
    atomicAdd(&sc->nodes, visits);
    atomicAdd(&sc->leaves, leafv);
  }
}

// Positions of every packet's first and last query in B's sorted codes
// (lower bounds), one thread per packet end.
// The query's code in the target set's frame: its own sorted code when both
// sets share one frame (qcodes != null), else computed from the point.
template <int D>
__device__ __forceinline__ void packet_pos_body(uint32_t kp, const float4* __restrict__ Q,
                                                const uint32_t* __restrict__ qcodes, uint64_t nQ,
                                                const Frame* __restrict__ tframe,
                                                const uint32_t* __restrict__ bcodes, uint64_t nB,
                                                uint32_t mask, uint32_t* __restrict__ pos) {
  const uint64_t t = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x;
  const uint64_t p = t >> 1;
  if (p * kp >= nQ) return;
  const uint64_t q = (t & 1) ? min(p * kp + kp - 1, nQ - 1) : p * kp;
  uint32_t target;
  if (qcodes) {
    target = qcodes[q] & mask;
  } else {
    const float4 qp = Q[q];
    target = frame_code<D>(*tframe, qp.x, qp.y, qp.z) & mask;
  }
  uint64_t lo = 0, hi = nB;
  while (lo < hi) {
    const uint64_t mid = (lo + hi) >> 1;
    if ((bcodes[mid] & mask) < target)
      lo = mid + 1;
    else
      hi = mid;
  }
  pos[t] = (uint32_t) lo;
}

// The same kernels over one or two point sets at once (blockIdx.y picks the
// set): an undirected solve builds both trees and answers both directions'
// queries in shared launches, so the two halves fill each other's tails.
struct BuildSet {
  const float4* pts;
  const uint32_t* codes;
  uint64_t n;
  uint32_t L, nL, nI;
  const float4* leaf_boxes;
  uint32_t* flags;   // arrivals per internal node (zeroed before the build)
  uint32_t* bound;   // two range bounds per internal node
  uint32_t* root;    // the root's internal node index
  float4* nodes;
  uint32_t mask;     // the set's sorted code bits
};
struct BuildSets {
  BuildSet s[2];
};

// Chains of dependent atomics: full occupancy (8 blocks of 256 threads per
// SM) matters more than a few spilled values.
__global__ void __launch_bounds__(256, 8) k_agglomerate(BuildSets b) {
  const BuildSet& S = b.s[blockIdx.y];
  agglomerate_body(S.codes, S.L, S.nL, S.leaf_boxes, S.flags, S.bound, S.root, S.nodes, S.mask);
}

struct QuerySet {
  const uint32_t* root;  // root of the target tree (internal node index)
  Deferred* defer;   // queue of over-budget queries (kDeferCap entries)
  uint32_t budget;   // visits per packet before its open queries are queued
  const float4* Q;
  uint64_t nQ;
  uint32_t pstride;
  uint64_t rows;
  FastDiv rows_div;  // division by rows
  const uint32_t* ppos;
  const float4* nodes;
  const float4* B;
  uint64_t nB;
  uint32_t L;
  DevScalars* sc;
  const Frame* tframe;      // frame of the target set's codes
  const uint32_t* qcodes;   // the query set's sorted codes when in that frame, else null
  const uint32_t* bcodes;
  uint32_t mask;            // the target set's sorted code bits
  uint32_t kp;              // queries per packet: 32 x queries per lane
  // Listing pass of the FP64 input path only (else null): rows that stay
  // open are also listed here, and rows stop only below soft_stop(thr,
  // soft_r).
  RowEntry* cand;
  uint32_t* cand_count;
  uint32_t cand_cap;
  float soft_r;
};
struct QuerySets {
  QuerySet d[2];
};

template <int D, bool COUNT, int LT, int QPL>
__global__ void __launch_bounds__(kQueryWarps * 32) k_lbvh_query(QuerySets qs) {
  const QuerySet& S = qs.d[blockIdx.y];
  lbvh_query_body<D, COUNT, LT, QPL>(S.Q, S.nQ, S.pstride, S.rows, S.rows_div, S.ppos, S.nodes, S.B,
                                S.nB, S.L, S.sc, S.defer, S.budget, *S.root, S.cand,
                                S.cand_count, S.cand_cap, S.soft_r);
}

// Deferred pass: one warp per queued query walks the tree with 32 stack
// entries popped per step (one per lane) instead of one, so the proof that a
// large ball is empty takes 1/32 of the serial steps.  Subtrees whose box is
// not nearer than the query's running minimum are pruned; the walk stops once
// that minimum is at or below the running maximum.  The stack lives in
// shared memory; a walk that would overflow it sets kErrInternal (the solve
// then fails) rather than drop a subtree.
constexpr int kDeferWarps = 4;
constexpr int kDeferStack = 3072;

template <int D, bool COUNT>
__global__ void __launch_bounds__(kDeferWarps * 32) k_lbvh_defer(QuerySets qs) {
  __shared__ uint32_t stk[kDeferWarps][kDeferStack];
  const QuerySet& S = qs.d[blockIdx.y];
  const uint32_t cnt = min(*(volatile uint32_t*) &S.sc->heavy_count, kDeferCap);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint32_t* st = stk[warp];
  const uint32_t nw = gridDim.x * kDeferWarps;
  unsigned long long pairs = 0, visits = 0, leafv = 0;
  // The running maximum is read by lane 0 and broadcast: the walk below must
  // see one value per warp.
  // The stop level of the pass (the running maximum, or in the listing pass
  // its soft bound), read by lane 0 and broadcast: the walk below must see
  // one value per warp.
  auto read_thr = [&]() {
    unsigned long long key = 0;
    if (lane == 0) key = ld_relaxed_u64(&S.sc->max_key);
    const float t = threshold_of(__shfl_sync(0xFFFFFFFFu, key, 0));
    return S.cand ? soft_stop(t, S.soft_r) : t;
  };
  for (uint32_t e = blockIdx.x * kDeferWarps + warp; e < cnt; e += nw) {
    const Deferred de = S.defer[e];
    const float4 q = S.Q[de.item];
    float m = __uint_as_float(de.gmin);
    float thr = read_thr();
    if (lane == 0) st[0] = *S.root;
    int sp = 1;
    __syncwarp();
    int round = 0;
    while (sp > 0 && m > thr) {
      const int k = min(sp, 32);
      const bool has = lane < k;
      const uint32_t node = has ? st[sp - k + lane] : 0;
      sp -= k;
      __syncwarp();
      uint32_t push0 = 0, push1 = 0;
      int npush = 0;
      float lm = m;
      if (has) {
        if (node & kLeafBit) {
          const uint64_t p0 = (uint64_t) (node & ~kLeafBit) * S.L;
          const uint32_t c = (uint32_t) min((uint64_t) S.L, S.nB - p0);
          for (uint32_t t = 0; t < c; ++t) {
            const float4 b = S.B[p0 + t];
            lm = fminf(lm, d2_pt_packed<D>(q, b));
          }
          if (COUNT) {
            pairs += c;
            ++leafv;
          }
        } else {
          const float4* nd = S.nodes + 4 * (uint64_t) node;
          const float4 n0 = nd[0], n1 = nd[1], n3 = nd[3];
          const float4 n2 = D == 3 ? nd[2] : make_float4(0.f, 0.f, 0.f, 0.f);
          const float dL = box_min_d2<D>(q, n0, n2.x, n2.y);
          const float dR = box_min_d2<D>(q, n1, n2.z, n2.w);
          const uint32_t left = __float_as_uint(n3.x), right = __float_as_uint(n3.y);
          // Nearer child pushed last, so that it is popped first.
          const bool wL = dL < m, wR = dR < m;
          if (wL && wR) {
            push0 = dL <= dR ? right : left;
            push1 = dL <= dR ? left : right;
            npush = 2;
          } else if (wL || wR) {
            push0 = wL ? left : right;
            npush = 1;
          }
          if (COUNT) ++visits;
        }
      }
      m = fminf(m, lm);
#pragma unroll
      for (int o = 16; o; o >>= 1) m = fminf(m, __shfl_xor_sync(0xFFFFFFFFu, m, o));
      // Compact the pushes: lanes in order, two slots per lane at most.
      int off = npush;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xFFFFFFFFu, off, o);
        if (lane >= o) off += v;
      }
      const int total = __shfl_sync(0xFFFFFFFFu, off, 31);
      off -= npush;  // exclusive prefix
      if (sp + total > kDeferStack) {
        if (lane == 0) atomicOr(&S.sc->status, kErrInternal);
        break;
      }
      if (npush > 0) st[sp + off] = push0;
      if (npush > 1) st[sp + off + 1] = push1;
      sp += total;
      __syncwarp();
      if ((++round & 15) == 0) thr = read_thr();
    }
    thr = read_thr();
    if (lane == 0 && m > thr) {
      if (S.cand) {
        const uint32_t slot = atomicAdd(S.cand_count, 1u);
        if (slot < S.cand_cap) S.cand[slot] = RowEntry{__float_as_uint(q.w), __float_as_uint(m)};
      }
      atomicMax(&S.sc->max_key, pack_max(m, __float_as_uint(q.w)));
    }
    __syncwarp();
  }
  if (COUNT) {
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      pairs += __shfl_xor_sync(0xFFFFFFFFu, pairs, o);
      visits += __shfl_xor_sync(0xFFFFFFFFu, visits, o);
      leafv += __shfl_xor_sync(0xFFFFFFFFu, leafv, o);
    }
    if (lane == 0 && (pairs || leafv || visits)) {
      atomicAdd(&S.sc->pairs, pairs);
      atomicAdd(&S.sc->nodes, visits);
      atomicAdd(&S.sc->leaves, leafv);
    }
  }
}

template <int D>
__global__ void k_packet_pos(QuerySets qs) {
  const QuerySet& S = qs.d[blockIdx.y];
  packet_pos_body<D>(S.kp, S.Q, S.qcodes, S.nQ, S.tframe, S.bcodes, S.nB, S.mask,
                     const_cast<uint32_t*>(S.ppos));
}

}  // namespace

// Builds the LBVHs of `count` sorted sets (tree k into node slot k).
static hd_status build_lbvhs(Ctx& c, const SortedSet* const* sets, int count, BuildSets* out) {
  // Leaves hold a power of two of points (at most 32): the query kernel
  // turns positions into leaf indices with a shift.
  const uint32_t L = sets[0]->leaf_size;  // fixed by the gather's leaf boxes
  hd_status s;
  uint64_t internal_total = 0;
  uint64_t nL[2], nI[2];
  for (int k = 0; k < count; ++k) {
    nL[k] = (sets[k]->n + L - 1) / L;
    nI[k] = std::max<uint64_t>(nL[k] - 1, 1);
    internal_total += nI[k];
    if (sets[k]->leaf_size != L) return fail(c, HD_ERR_CUDA, "leaf sizes differ");
  }
  // Flags of all sets first (one memset clears them), then the bounds, then
  // one root word per set.
  void* aux2;
  if ((s = ensure(c, kBufAux2, (internal_total * 3 + 2) * 4, &aux2)) != HD_OK) return s;
  uint32_t* flags_base = (uint32_t*) aux2;
  uint32_t* bound_base = flags_base + internal_total;
  uint32_t* roots = bound_base + 2 * internal_total;
  uint64_t off_int = 0, maxL = 0;
  for (int k = 0; k < count; ++k) {
    void* nodes;
    if ((s = ensure(c, k == 0 ? kBufNodes0 : kBufNodes1, nI[k] * 4 * sizeof(float4), &nodes)) !=
        HD_OK)
      return s;
    BuildSet& b = out->s[k];
    b.pts = sets[k]->pts;
    b.codes = sets[k]->codes;
    b.n = sets[k]->n;
    b.L = L;
    b.nL = (uint32_t) nL[k];
    b.nI = (uint32_t) nI[k];
    b.leaf_boxes = sets[k]->leaf_boxes;
    b.flags = flags_base + off_int;
    b.bound = bound_base + 2 * off_int;
    b.root = roots + k;
    b.nodes = (float4*) nodes;
    b.mask = sets[k]->mask;
    off_int += nI[k];
    maxL = std::max(maxL, nL[k]);
  }
  if (count == 1) out->s[1] = out->s[0];
  cudaError_t e = cudaMemsetAsync(flags_base, 0, internal_total * 4, c.stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "memset flags");
  const dim3 gl((unsigned) ((maxL + 255) / 256), count);
  k_agglomerate<<<gl, 256, 0, c.stream>>>(*out);
  return after_launch(c, "agglomerate");
}

// Directed LBVH solves of `count` directions (1, or 2 for an undirected solve)
// with shared launches.  With a plan (the FP64 input path), the query pass
// is the listing pass (rows stop only below the soft bound and the open ones
// are listed), and the certified FP32 solve is followed by f64_seed.
static hd_status run_lbvh_dirs(Ctx& c, const DirInput* ins, int count, F64Plan* plan) {
  const int dims = ins[0].dims;
  if (dims != 2 && dims != 3) return fail(c, HD_ERR_UNSUPPORTED, "LBVH needs n_dims 2 or 3");
  hd_status s;
  const SortedSet *q[2], *t[2];
  for (int k = 0; k < count; ++k)
    if ((s = spatial_prepare(c, ins[k], &q[k], &t[k])) != HD_OK) return s;
  mark(c, 1);
  QuerySets qs;
  // Two queries per lane when the launch answers at least
  // kQplTwoMinQueries queries.
  uint64_t total_queries = 0;
  for (int k = 0; k < count; ++k) total_queries += q[k]->n;
  const bool qpl2 = total_queries >= kQplTwoMinQueries;
  const uint32_t kp = qpl2 ? 64u : 32u;
  uint64_t packets[2], maxppos = 0;
  for (int k = 0; k < count; ++k) {
    packets[k] = (q[k]->n + kp - 1) / kp;
    maxppos += 2 * packets[k];
  }
  void* ppos;
  if ((s = ensure(c, kBufSample, maxppos * 4, &ppos)) != HD_OK) return s;
  // Deferred-query queues, one per direction.
  void* defer;
  if ((s = ensure(c, kBufHeavy, (uint64_t) count * kDeferCap * sizeof(Deferred), &defer)) != HD_OK)
    return s;
  if ((s = ensure_side(c)) != HD_OK) return s;
  uint64_t off = 0, max_pos_threads = 0;
  for (int k = 0; k < count; ++k) {
    QuerySet& d = qs.d[k];
    d.Q = q[k]->pts;
    d.nQ = q[k]->n;
    d.ppos = (const uint32_t*) ppos + off;
    d.B = t[k]->pts;
    d.nB = t[k]->n;
    d.tframe = t[k]->frame;
    d.qcodes = q[k]->frame == t[k]->frame ? q[k]->codes : nullptr;
    d.bcodes = t[k]->codes;
    d.mask = t[k]->mask;
    d.kp = kp;
    d.cand = plan ? plan->cand[k] : nullptr;
    d.cand_count = plan ? plan->cand_count[k] : nullptr;
    d.cand_cap = plan ? plan->cand_cap : 0u;
    d.soft_r = plan ? plan->soft_r[k] : 0.0f;
    off += 2 * packets[k];
    max_pos_threads = std::max<uint64_t>(max_pos_threads, 2 * packets[k]);
  }
  if (count == 1) qs.d[1] = qs.d[0];
  // Packet positions need only the sorted sets: they run on the side
  // stream while the (latency-bound) tree build runs on the main one.
  cudaEventRecord(c.batch_fork, c.stream);
  cudaStreamWaitEvent(c.batch_side, c.batch_fork, 0);
  const dim3 pgrid((unsigned) ((max_pos_threads + 255) / 256), count);
  if (dims == 2)
    k_packet_pos<2><<<pgrid, 256, 0, c.batch_side>>>(qs);
  else
    k_packet_pos<3><<<pgrid, 256, 0, c.batch_side>>>(qs);
  if ((s = after_launch(c, "packet_pos")) != HD_OK) return s;
  cudaEventRecord(c.batch_join, c.batch_side);
  BuildSets bs;
  if ((s = build_lbvhs(c, t, count, &bs)) != HD_OK) return s;
  mark(c, 2);
  cudaStreamWaitEvent(c.stream, c.batch_join, 0);
  uint64_t max_warps = 0;
  for (int k = 0; k < count; ++k) {
    QuerySet& d = qs.d[k];
    const uint32_t pstride = packets[k] >= 4096 ? 64 : (packets[k] >= 256 ? 16 : 1);
    d.pstride = pstride;
    d.rows = (packets[k] + pstride - 1) / pstride;
    d.rows_div = make_fastdiv((uint32_t) d.rows);
    d.nodes = bs.s[k].nodes;
    d.root = bs.s[k].root;
    d.L = bs.s[k].L;
    d.sc = scalars(c, ins[k].dir);
    d.defer = (Deferred*) defer + (uint64_t) k * kDeferCap;
    d.budget = c.opt.lbvh_budget;
    max_warps = std::max<uint64_t>(max_warps, d.rows * pstride);
  }
  if (count == 1) qs.d[1] = qs.d[0];
  mark(c, 3);
  const dim3 grid((unsigned) ((max_warps + kQueryWarps - 1) / kQueryWarps), count);
  const bool l16 = bs.s[0].L == 16;
  auto launch_queries = [&](bool cnt) -> hd_status {
    // Kernel per (n_dims, counting, leaf size 16 or any, queries per lane).
    static const void* const table[2][2][2][2] = {
        {{{(const void*) k_lbvh_query<2, false, 0, 1>, (const void*) k_lbvh_query<2, false, 0, 2>},
          {(const void*) k_lbvh_query<2, false, 16, 1>, (const void*) k_lbvh_query<2, false, 16, 2>}},
         {{(const void*) k_lbvh_query<2, true, 0, 1>, (const void*) k_lbvh_query<2, true, 0, 2>},
          {(const void*) k_lbvh_query<2, true, 16, 1>, (const void*) k_lbvh_query<2, true, 16, 2>}}},
        {{{(const void*) k_lbvh_query<3, false, 0, 1>, (const void*) k_lbvh_query<3, false, 0, 2>},
          {(const void*) k_lbvh_query<3, false, 16, 1>, (const void*) k_lbvh_query<3, false, 16, 2>}},
         {{(const void*) k_lbvh_query<3, true, 0, 1>, (const void*) k_lbvh_query<3, true, 0, 2>},
          {(const void*) k_lbvh_query<3, true, 16, 1>, (const void*) k_lbvh_query<3, true, 16, 2>}}}};
    const void* fn = table[dims == 3][cnt][l16][qpl2];
    void* qargs[] = {&qs};
    cudaLaunchKernel(fn, grid, dim3(kQueryWarps * 32), qargs, 0, c.stream);
    hd_status r;
    if ((r = after_launch(c, "lbvh_query")) != HD_OK) return r;
    // Queries queued by over-budget packets (usually none: the launch then
    // returns at once).
    const dim3 dgrid((unsigned) (c.num_sms * 4), count);
    if (dims == 2) {
      if (cnt)
        k_lbvh_defer<2, true><<<dgrid, kDeferWarps * 32, 0, c.stream>>>(qs);
      else
        k_lbvh_defer<2, false><<<dgrid, kDeferWarps * 32, 0, c.stream>>>(qs);
    } else {
      if (cnt)
        k_lbvh_defer<3, true><<<dgrid, kDeferWarps * 32, 0, c.stream>>>(qs);
      else
        k_lbvh_defer<3, false><<<dgrid, kDeferWarps * 32, 0, c.stream>>>(qs);
    }
    return after_launch(c, "lbvh_defer");
  };
  if ((s = launch_queries(ins[0].count)) != HD_OK) return s;
  mark(c, 4);
  for (int k = 0; k < count; ++k)
    if ((s = certify(c, ins[k])) != HD_OK) return s;
  if (plan) {
    for (int k = 0; k < count; ++k)
      plan->tree[k] = LbvhTree{bs.s[k].nodes, bs.s[k].root, t[k]->pts, t[k]->n, bs.s[k].L};
    if ((s = f64_seed(c, *plan, count)) != HD_OK) return s;
  }
  return HD_OK;
}

hd_status run_lbvh(Ctx& c, const DirInput& in) { return run_lbvh_dirs(c, &in, 1, nullptr); }

hd_status run_lbvh_pair(Ctx& c, const DirInput& ab, const DirInput& ba) {
  const DirInput ins[2] = {ab, ba};
  return run_lbvh_dirs(c, ins, 2, nullptr);
}

hd_status run_lbvh_f64(Ctx& c, const DirInput* ins, int count, F64Plan* plan) {
  return run_lbvh_dirs(c, ins, count, plan);
}

}  // namespace hdg
