// Persistent early-break (EB) scan for 2-D and 3-D inputs.
//
// Replaces the reference's GPU early-break kernel
// (src/hd_impl/hausdorff_distance_early_break.h:117-219: one block per A
// point, threads striding over B, a cub::BlockReduce every 32 iterations and
// a CAS-loop float atomicMax) and the hybrid's block / cooperative-grid EB
// kernels (src/hd_impl/hausdorff_distance_hybrid.h:519-694).
//
// Design (GB300-first):
//  * B is copied once into a visit-ordered, padded array of float2 (2-D) or
//    float4 (3-D) points: coalesced 16-byte loads, 16-byte aligned tiles.
//  * k_eb_main is persistent: every CTA streams B tiles of 256 points into a
//    shared-memory double buffer with the TMA bulk-copy engine
//    (cp.async.bulk + mbarrier), and each thread carries 4 A points ("slots")
//    against every point of the tile (shared-memory broadcast reads).  A slot
//    that stops — its running minimum at or below the running maximum (early
//    break), a full cycle over B (completed: atomicMax), or more than the
//    per-point cap of tiles (deferred) — is refilled at the next tile boundary
//    from a global visit queue with one warp-aggregated atomicAdd; once the
//    queue is drained and at most 1/8 of a CTA's threads still hold a point,
//    those points are deferred too and the CTA retires.  Because
//    B's visit order is a pseudo-random permutation, a slot may start at any
//    tile and wrap around: no slot waits for a CTA-wide restart.
//  * Deferred points — the ones whose nearest neighbour is farther than the
//    running maximum — and the seeds that start the maximum (the first 152
//    visited points, before the main pass, so that it never starts from a
//    zero threshold; the reference's hybrid seeds it with an MBR lower bound
//    and a sample, hybrid.h:111-142) are finished by the tile-wise list
//    scan k_eb_list: groups of up to 256 points against chunks of B's tiles
//    staged in shared memory; a group raises the running maximum as soon as
//    its last chunk is done, so later groups break early.
//  * The running maximum is one 64-bit word (squared-distance bits, ~index):
//    a single atomicMax on the bit pattern — no CAS loop — which also keeps
//    the certifying A index.
#include <cfloat>
#include <cmath>
#include <cstring>

#include "hd_common.cuh"
#include "hd_internal.h"
#include "hd_tuning.h"

namespace hdg {
namespace {

constexpr int kEbThreads = 256;
constexpr int kEbTile = 256;          // B points per tile (== kEbThreads)
constexpr int kEbSlots = 4;           // A points carried per thread
constexpr uint32_t kCapPairs = 8192;  // per-point pairs before deferral (no-alloc entry point)
constexpr uint32_t kWaitLimit = 1u << 26;
constexpr uint32_t kListChunks = 64;  // B chunks per group in the list scan, at least
constexpr int kHeavySlots = 4;        // deferred points a CTA carries at once
constexpr uint32_t kHeavyStepTiles = 32;  // tiles between a CTA's reductions
// Checkpoints of the main pass: after the first 1/16 of the visit order
// (when each part is at least one full wave of the grid), the deferred
// points listed so far are finished before the pass goes on.  Measured on
// the 10M mixtures: one checkpoint at 1/16 beats 1/8, {1/16, 1/4} and
// {1/16, 1/2} (clusters3d 38.6 against 42.7, 44.6, 45.1 ms).
constexpr uint64_t kEbCheckDiv[] = {16};
constexpr int kEbMaxParts = (int) (sizeof(kEbCheckDiv) / sizeof(kEbCheckDiv[0])) + 1;

template <int D>
struct EbPt;
template <>
struct EbPt<2> {
  using T = float2;
};
template <>
struct EbPt<3> {
  using T = float4;
};

struct HeavyEntry {
  uint32_t ia;         // caller's index of the A point
  uint32_t next_tile;  // first tile still to visit
  uint32_t remaining;  // tiles still to visit
  float cmin;          // running minimum so far
};

template <int D>
__device__ __forceinline__ void load_a(const float* __restrict__ A, uint64_t i,
                                       float& x, float& y, float& z) {
  if constexpr (D == 2) {
    float2 v = *reinterpret_cast<const float2*>(A + 2 * i);
    x = v.x;
    y = v.y;
    z = 0.0f;
  } else {
    x = A[3 * i];
    y = A[3 * i + 1];
    z = A[3 * i + 2];
  }
}

template <int D>
__global__ void k_eb_pack(const float* __restrict__ B, uint64_t nB, Perm perm,
                          typename EbPt<D>::T* __restrict__ out, uint64_t nPad) {
  for (uint64_t j = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; j < nPad;
       j += (uint64_t) gridDim.x * blockDim.x) {
    if constexpr (D == 2) {
      float2 v = make_float2(INFINITY, INFINITY);
      if (j < nB) v = *reinterpret_cast<const float2*>(B + 2 * perm(j));
      out[j] = v;
    } else {
      float4 v = make_float4(INFINITY, INFINITY, INFINITY, 0.0f);
      if (j < nB) {
        uint64_t s = perm(j);
        v = make_float4(B[3 * s], B[3 * s + 1], B[3 * s + 2], 0.0f);
      }
      out[j] = v;
    }
  }
}

template <int D>
__device__ __forceinline__ float tile_d2(float ax, float ay, float az,
                                         float bx, float by, float bz) {
  if constexpr (D == 2) {
    return d2_2(ax, ay, bx, by);
  } else {
    return d2_3(ax, ay, az, bx, by, bz);
  }
}

// S: A points carried per thread (4 for large sets; 2 or 1 when the set is
// too small to give every SM a full complement of 4-slot CTAs).
template <int D, int S = kEbSlots>
__global__ void __launch_bounds__(kEbThreads)
    k_eb_main(const float* __restrict__ A, Perm permA, uint64_t a_begin,
              uint64_t a_end, const typename EbPt<D>::T* __restrict__ Bp,
              uint32_t nTiles, uint32_t capTiles, DevScalars* sc,
              HeavyEntry* heavy, uint32_t heavy_cap) {
  using PT = typename EbPt<D>::T;
  constexpr uint32_t kTileBytes = kEbTile * sizeof(PT);
  __shared__ __align__(128) PT tile[2][kEbTile];
  __shared__ __align__(8) uint64_t full[2];

  const int tid = threadIdx.x;
  const int lane = tid & 31;
  float ax[S], ay[S], az[S], cm[S];
  uint32_t ia[S], vis[S];
  bool act[S];
  unsigned long long pairs = 0;
  bool exhausted = false;
#pragma unroll
  for (int r = 0; r < S; ++r) {
    act[r] = false;
    ax[r] = ay[r] = az[r] = 0.0f;
    cm[r] = FLT_MAX;
    ia[r] = 0;
    vis[r] = 0;
  }

  // Warp-aggregated refill of every free slot from the visit queue.
  auto refill = [&]() {
    if (exhausted) return;
    uint32_t masks[S];
    uint32_t total = 0;
#pragma unroll
    for (int r = 0; r < S; ++r) {
      masks[r] = __ballot_sync(0xFFFFFFFFu, !act[r]);
      total += __popc(masks[r]);
    }
    if (total == 0) return;
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(&sc->next, (unsigned long long) total);
    base = __shfl_sync(0xFFFFFFFFu, base, 0);
    const uint32_t lt = (1u << lane) - 1u;
    uint32_t before = 0;
#pragma unroll
    for (int r = 0; r < S; ++r) {
      if (!act[r]) {
        uint64_t v = a_begin + base + before + __popc(masks[r] & lt);
        if (v < a_end) {
          uint64_t i = permA(v);
          ia[r] = (uint32_t) i;
          load_a<D>(A, i, ax[r], ay[r], az[r]);
          cm[r] = FLT_MAX;
          vis[r] = 0;
          act[r] = true;
        }
      }
      before += __popc(masks[r]);
    }
    if (a_begin + base + total >= a_end) exhausted = true;
  };

  if (tid == 0) {
    mbar_init(&full[0], 1);
    mbar_init(&full[1], 1);
    fence_barrier_init();
  }
  __syncthreads();
  refill();

  uint32_t tcur = (uint32_t) (((uint64_t) blockIdx.x * nTiles) / gridDim.x);
  if (tid == 0) {
    mbar_expect_tx(&full[0], kTileBytes);
    tma_load_1d(&tile[0][0], Bp + (uint64_t) tcur * kEbTile, kTileBytes, &full[0]);
  }

  // Running maximum as of the last tile boundary (mid-tile early stop).
  float thr_prev;
  {
    unsigned long long k0 = 0;
    if (lane == 0) k0 = ld_relaxed_u64(&sc->max_key);
    thr_prev = threshold_of(__shfl_sync(0xFFFFFFFFu, k0, 0));
  }
  uint32_t i = 0;
  bool failed = false;
  for (;; ++i) {
    const int buf = i & 1;
    const uint32_t tnext = (tcur + 1 == nTiles) ? 0 : tcur + 1;
    if (tid == 0) {
      // Buffer buf^1 was released by every thread at the end of iteration i-1.
      mbar_expect_tx(&full[buf ^ 1], kTileBytes);
      tma_load_1d(&tile[buf ^ 1][0], Bp + (uint64_t) tnext * kEbTile, kTileBytes,
                  &full[buf ^ 1]);
    }
    bool ok = mbar_wait(&full[buf], (i >> 1) & 1, &sc->status, kWaitLimit);
    if (__syncthreads_or(!ok)) {
      failed = true;
      break;
    }

    // The tile in chunks of 32 points: a warp whose open slots are all at or
    // below the maximum read at the last boundary stops early (they would
    // break at the boundary anyway), which matters for data where points
    // break after a few pairs.
#pragma unroll 1
    for (int c0 = 0; c0 < kEbTile; c0 += 32) {
      if constexpr (D == 2) {
        const float4* t4 = reinterpret_cast<const float4*>(&tile[buf][0]) + c0 / 2;
#pragma unroll 4
        for (int p = 0; p < 16; ++p) {
          float4 b = t4[p];
#pragma unroll
          for (int r = 0; r < S; ++r) {
            cm[r] = fminf(cm[r], d2_2(ax[r], ay[r], b.x, b.y));
            cm[r] = fminf(cm[r], d2_2(ax[r], ay[r], b.z, b.w));
          }
        }
      } else {
#pragma unroll 4
        for (int p = 0; p < 32; ++p) {
          float4 b = tile[buf][c0 + p];
#pragma unroll
          for (int r = 0; r < S; ++r)
            cm[r] = fminf(cm[r], d2_3(ax[r], ay[r], az[r], b.x, b.y, b.z));
        }
      }
      bool open = false;
#pragma unroll
      for (int r = 0; r < S; ++r) open |= act[r] && cm[r] > thr_prev;
      if (!__any_sync(0xFFFFFFFFu, open)) break;
    }

    // Slot bookkeeping at the tile boundary.
    unsigned long long key = 0;
    if (lane == 0) key = ld_relaxed_u64(&sc->max_key);
    key = __shfl_sync(0xFFFFFFFFu, key, 0);
    const float thr = threshold_of(key);
    thr_prev = thr;
#pragma unroll
    for (int r = 0; r < S; ++r) {
      if (!act[r]) continue;
      pairs += kEbTile;
      vis[r] += 1;
      if (cm[r] <= thr) {
        act[r] = false;  // early break: cannot raise the maximum
      } else if (vis[r] == nTiles) {
        atomicMax(&sc->max_key, pack_max(cm[r], ia[r]));
        act[r] = false;  // full cycle: exact minimum
      } else if (vis[r] >= capTiles) {
        uint32_t s = atomicAdd(&sc->heavy_count, 1u);
        if (s < heavy_cap) {
          heavy[s] = HeavyEntry{ia[r], tnext, nTiles - vis[r], cm[r]};
        } else {
          atomicOr(&sc->status, kErrQueueOverflow);
        }
        act[r] = false;
      }
    }
    refill();
    bool any = false;
#pragma unroll
    for (int r = 0; r < S; ++r) any |= act[r];
    tcur = tnext;
    const int busy = __syncthreads_count(any);  // threads with an active slot
    if (busy == 0) break;
    if (busy * 8 <= kEbThreads && __syncthreads_and(exhausted)) {
      // Nothing left to refill from and at most 1/8 of the threads busy:
      // every thread would keep computing for a few stragglers, so hand
      // them to the per-point kernel (all 256 threads on one point) instead.
#pragma unroll
      for (int r = 0; r < S; ++r) {
        if (!act[r]) continue;
        uint32_t s = atomicAdd(&sc->heavy_count, 1u);
        if (s < heavy_cap) {
          heavy[s] = HeavyEntry{ia[r], tcur, nTiles - vis[r], cm[r]};
        } else {
          atomicOr(&sc->status, kErrQueueOverflow);
        }
        act[r] = false;
      }
      break;
    }
  }
  // One prefetch is still in flight (issued at the top of the last
  // iteration); wait for it so the CTA never exits with a copy pending.
  if (tid == 0 && !failed) mbar_wait(&full[(i & 1) ^ 1], ((i + 1) >> 1) & 1, &sc->status, kWaitLimit);
  if (pairs) atomicAdd(&sc->pairs, pairs);
}

// Points finished outside the persistent pass — the seeds that start the
// running maximum, and the points deferred past the pair cap (the far ones
// that decide the distance) — are scanned tile-wise: a work item is a group
// of up to 256 listed points (one per thread) against one chunk of B's
// tiles, streamed through a shared-memory double buffer with the TMA bulk
// copy as in k_eb_main, so every B point loaded serves 256 pairs.  A point's
// minimum over its chunks is combined with an atomicMin on the float's bits
// (non-negative floats order as their bit patterns).  Items are taken group
// by group, and the CTA that completes a group's last chunk raises the
// running maximum with that group's points at once: the maximum climbs while
// later groups are still scanning, so their points stop early, as the
// reference's early break does (early_break.h:76).  An item stops once every
// point of its group is at or below the running maximum: such a point cannot
// raise it, and the partial minimum it records is at or below it too.
template <int D>
__global__ void __launch_bounds__(kEbThreads)
    k_eb_list(const float* __restrict__ A, const typename EbPt<D>::T* __restrict__ Bp,
              uint32_t nTiles, HeavyEntry* list, uint32_t* group_done, uint32_t n_host,
              const uint32_t* n_dev, uint32_t cap, DevScalars* sc) {
  using PT = typename EbPt<D>::T;
  constexpr uint32_t kTileBytes = kEbTile * sizeof(PT);
  __shared__ __align__(128) PT tile[2][kEbTile];
  __shared__ __align__(8) uint64_t full[2];
  __shared__ bool s_last;
  const int tid = threadIdx.x;
  const uint32_t n = n_dev ? min(*n_dev, cap) : n_host;
  if (n == 0) return;
  const uint32_t groups = (n + kEbThreads - 1) / kEbThreads;
  // At least kListChunks chunks per group, so that the CTAs running at one
  // time share a few groups (B chunks reused through L2, groups completing
  // one after another); more when there are few groups.
  const uint32_t chunks =
      max(1u, min(nTiles, max(kListChunks, (2 * gridDim.x + groups - 1) / groups)));
  const uint32_t items = groups * chunks;
  if (tid == 0) {
    mbar_init(&full[0], 1);
    mbar_init(&full[1], 1);
    fence_barrier_init();
  }
  __syncthreads();
  uint32_t it = 0;  // tiles this CTA has consumed (buffer it & 1, parity (it >> 1) & 1)
  unsigned long long pairs = 0;
  for (uint32_t w = blockIdx.x; w < items; w += gridDim.x) {
    const uint32_t group = w / chunks, chunk = w - group * chunks;
    const uint32_t t0 = (uint32_t) (((uint64_t) chunk * nTiles) / chunks);
    const uint32_t t1 = (uint32_t) (((uint64_t) (chunk + 1) * nTiles) / chunks);
    const uint32_t e = group * kEbThreads + tid;
    float ax = 0.f, ay = 0.f, az = 0.f, m = FLT_MAX;
    uint32_t ia = 0;
    if (e < n) {
      const HeavyEntry h = list[e];
      load_a<D>(A, h.ia, ax, ay, az);
      m = h.cmin;
      ia = h.ia;
    }
    unsigned long long key = 0;
    if ((tid & 31) == 0) key = ld_relaxed_u64(&sc->max_key);
    key = __shfl_sync(0xFFFFFFFFu, key, 0);
    bool act = e < n && m > threshold_of(key);
    if (__syncthreads_or(act)) {
      if (tid == 0) {
        mbar_expect_tx(&full[it & 1], kTileBytes);
        tma_load_1d(&tile[it & 1][0], Bp + (uint64_t) t0 * kEbTile, kTileBytes, &full[it & 1]);
      }
      for (uint32_t t = t0;;) {
        const int buf = it & 1;
        const bool more = t + 1 < t1;
        if (tid == 0 && more) {
          // Buffer buf^1 was released by every thread at the end of the
          // last tile (the barrier below).
          mbar_expect_tx(&full[buf ^ 1], kTileBytes);
          tma_load_1d(&tile[buf ^ 1][0], Bp + (uint64_t) (t + 1) * kEbTile, kTileBytes,
                      &full[buf ^ 1]);
        }
        const bool ok = mbar_wait(&full[buf], (it >> 1) & 1, &sc->status, kWaitLimit);
        if (__syncthreads_or(!ok)) {
          // A copy did not arrive in time: the status bit fails the solve.
          if (pairs) atomicAdd(&sc->pairs, pairs);
          return;
        }
        if (act) {
          if constexpr (D == 2) {
            const float4* t4 = reinterpret_cast<const float4*>(&tile[buf][0]);
#pragma unroll 8
            for (int p = 0; p < kEbTile / 2; ++p) {
              const float4 b = t4[p];
              m = fminf(m, d2_2(ax, ay, b.x, b.y));
              m = fminf(m, d2_2(ax, ay, b.z, b.w));
            }
          } else {
#pragma unroll 8
            for (int p = 0; p < kEbTile; ++p) {
              const float4 b = tile[buf][p];
              m = fminf(m, d2_3(ax, ay, az, b.x, b.y, b.z));
            }
          }
          pairs += kEbTile;
        }
        ++it;
        ++t;
        if ((tid & 31) == 0) key = ld_relaxed_u64(&sc->max_key);
        key = __shfl_sync(0xFFFFFFFFu, key, 0);
        if (act && m <= threshold_of(key)) act = false;
        const bool any = __syncthreads_or(act);
        if (!more) break;
        if (!any) {
          // Early break of the whole group: drain the prefetch in flight.
          if (tid == 0) mbar_wait(&full[it & 1], (it >> 1) & 1, &sc->status, kWaitLimit);
          ++it;
          __syncthreads();
          break;
        }
      }
    }
    if (e < n) atomicMin(reinterpret_cast<unsigned int*>(&list[e].cmin), __float_as_uint(m));
    // The CTA completing the group's last chunk raises the maximum with the
    // group's points whose minimum over all of B stayed above it.
    __threadfence();
    __syncthreads();
    if (tid == 0) s_last = atomicAdd(&group_done[group], 1u) == chunks - 1;
    __syncthreads();
    if (s_last && e < n) {
      __threadfence();
      const float gm = __uint_as_float(__ldcg(reinterpret_cast<const unsigned int*>(&list[e].cmin)));
      if (gm > threshold_of(ld_relaxed_u64(&sc->max_key)))
        atomicMax(&sc->max_key, pack_max(gm, ia));
    }
  }
  if (pairs) atomicAdd(&sc->pairs, pairs);
}

// Deferred points: the CTA's threads all stride over B (every thread loads
// one point of each tile), carrying kHeavySlots listed points at once, so
// that every B point loaded serves kHeavySlots pairs.  Every kHeavyStepTiles
// tiles the CTA reduces each slot's minimum and re-reads the running
// maximum: a slot whose minimum is at or below it is freed (early break), a
// slot that has covered B's whole tile ring raises the maximum and is freed,
// and free slots take the CTA's next list entries (entries blockIdx.x,
// blockIdx.x + gridDim.x, ...).  Points thus finish one after another and
// the maximum climbs while the rest of the list is still open, as in the
// reference's early break (early_break.h:63-85).  A point keeps the running
// minimum of its main-pass tiles and scans the whole ring from the CTA's
// current position (the few tiles it already saw cost next to nothing); all
// CTAs start at tile 0 and move at about the same pace, so they read B's
// tiles through L2.
template <int D>
__global__ void __launch_bounds__(kEbThreads)
    k_eb_heavy(const float* __restrict__ A, const typename EbPt<D>::T* __restrict__ Bp,
               uint32_t nTiles, DevScalars* sc, const HeavyEntry* __restrict__ list,
               const uint32_t* n_dev, uint32_t cap, const uint32_t* first_dev) {
  constexpr int P = kHeavySlots;
  __shared__ float red[kEbThreads / 32][P];
  __shared__ float s_thr;
  const int tid = threadIdx.x;
  const uint32_t n = min(*n_dev, cap);
  float ax[P], ay[P], az[P], cmin[P];
  uint32_t ia[P], done[P];
  bool act[P];
  // Entries [first, n): an earlier deferred pass finished those below first.
  uint32_t next = (first_dev ? *first_dev : 0u) + blockIdx.x;  // next list entry of this CTA
  auto take = [&](int s) {
    act[s] = next < n;
    if (act[s]) {
      const HeavyEntry h = list[next];
      ia[s] = h.ia;
      load_a<D>(A, h.ia, ax[s], ay[s], az[s]);
      cmin[s] = h.cmin;
      done[s] = 0;
      next += gridDim.x;
    } else {
      ax[s] = ay[s] = az[s] = 0.0f;
      cmin[s] = FLT_MAX;
    }
  };
#pragma unroll
  for (int s = 0; s < P; ++s) take(s);
  unsigned long long pairs = 0;
  uint32_t t = 0;  // this CTA's position in B's tile ring
  for (;;) {
    bool any = false;
#pragma unroll
    for (int s = 0; s < P; ++s) any |= act[s];
    if (!any) break;
    const uint32_t step = min((uint32_t) kHeavyStepTiles, nTiles);
    float m[P];
#pragma unroll
    for (int s = 0; s < P; ++s) m[s] = FLT_MAX;
    // The step's tiles t .. t+step-1 around the ring: at most two contiguous
    // runs, each walked with one pointer (groups of 8 loads issued before any
    // is used).
    for (uint32_t k = 0; k < step;) {
      const uint32_t run = min(step - k, nTiles - t);
      const typename EbPt<D>::T* p = Bp + (uint64_t) t * kEbTile + tid;
      uint32_t u = 0;
      for (; u + 8 <= run; u += 8, p += 8 * kEbTile) {
        typename EbPt<D>::T b[8];
#pragma unroll
        for (int v = 0; v < 8; ++v) b[v] = p[v * kEbTile];
#pragma unroll
        for (int v = 0; v < 8; ++v)
#pragma unroll
          for (int s = 0; s < P; ++s) {
            if (!act[s]) continue;
            if constexpr (D == 2)
              m[s] = fminf(m[s], d2_2(ax[s], ay[s], b[v].x, b[v].y));
            else
              m[s] = fminf(m[s], d2_3(ax[s], ay[s], az[s], b[v].x, b[v].y, b[v].z));
          }
      }
      for (; u < run; ++u, p += kEbTile) {
        const auto b = *p;
#pragma unroll
        for (int s = 0; s < P; ++s) {
          if (!act[s]) continue;
          if constexpr (D == 2)
            m[s] = fminf(m[s], d2_2(ax[s], ay[s], b.x, b.y));
          else
            m[s] = fminf(m[s], d2_3(ax[s], ay[s], az[s], b.x, b.y, b.z));
        }
      }
      k += run;
      t += run;
      if (t == nTiles) t = 0;
    }
#pragma unroll
    for (int s = 0; s < P; ++s) {
      if (!act[s]) continue;
      pairs += step;
      float w = m[s];
#pragma unroll
      for (int o = 16; o; o >>= 1) w = fminf(w, __shfl_xor_sync(0xFFFFFFFFu, w, o));
      if ((tid & 31) == 0) red[tid >> 5][s] = w;
    }
    // One thread reads the shared maximum so that every thread of the CTA
    // takes the same decisions.
    if (tid == 0) s_thr = threshold_of(ld_relaxed_u64(&sc->max_key));
    __syncthreads();
    const float thr = s_thr;
#pragma unroll
    for (int s = 0; s < P; ++s) {
      if (!act[s]) continue;
      float bm = red[0][s];
#pragma unroll
      for (int k = 1; k < kEbThreads / 32; ++k) bm = fminf(bm, red[k][s]);
      cmin[s] = fminf(cmin[s], bm);
      done[s] += step;
      if (cmin[s] <= thr) {
        take(s);  // early break: this point cannot raise the maximum
      } else if (done[s] >= nTiles) {
        if (tid == 0) atomicMax(&sc->max_key, pack_max(cmin[s], ia[s]));
        take(s);  // whole ring scanned: exact minimum
      }
    }
    __syncthreads();
  }
  if (tid == 0 && pairs) atomicAdd(&sc->pairs, pairs * kEbTile);
}

// Between the early checkpoint and the bulk of the main pass: the deferred
// entries listed so far are finished, and the bulk's visit counter starts
// again at zero.
__global__ void k_eb_mark_heavy(DevScalars* sc) {
  sc->heavy_mark = sc->heavy_count;
  sc->next = 0;
}

// The seed list: the first n visit positions of A, nothing scanned yet.
__global__ void k_eb_seed_list(Perm permA, uint32_t n, uint32_t nTiles, HeavyEntry* list) {
  const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < n) list[e] = HeavyEntry{(uint32_t) permA(e), 0u, nTiles, FLT_MAX};
}

// Seeds, or the deferred points, through the tile-wise list scan
// (stream-level, shared by the context path and the allocation-free entry
// point).  n_dev: device count of listed points (deferred points), or null
// with n_host (seeds).  group_done: one zeroed counter per group of 256 list
// entries (cap / 256 + 1 words).
template <int D>
cudaError_t eb_list_pass(cudaStream_t st, int num_sms, const float* A,
                         const typename EbPt<D>::T* Bp, uint32_t nTiles, HeavyEntry* list,
                         uint32_t* group_done, uint32_t n_host, const uint32_t* n_dev,
                         uint32_t cap, DevScalars* sc) {
  cudaError_t e = cudaMemsetAsync(group_done, 0, ((size_t) cap / kEbThreads + 1) * 4, st);
  if (e != cudaSuccess) return e;
  k_eb_list<D><<<num_sms * 4, kEbThreads, 0, st>>>(A, Bp, nTiles, list, group_done, n_host, n_dev,
                                                   cap, sc);
  return cudaGetLastError();
}

template <int D>
hd_status run_eb_dim(Ctx& c, const DirInput& in) {
  using PT = typename EbPt<D>::T;
  const uint64_t nTiles64 = (in.nB + kEbTile - 1) / kEbTile;
  if (nTiles64 >= 0xFFFFFFFFull) return fail(c, HD_ERR_INVALID_ARG, "B too large");
  const uint32_t nTiles = (uint32_t) nTiles64;
  const uint64_t nPad = nTiles64 * kEbTile;
  void *pb = nullptr, *ph = nullptr;
  hd_status s;
  if ((s = ensure(c, kBufPackB, nPad * sizeof(PT), &pb)) != HD_OK) return s;
  // The point list, then one completion counter per group of 256 entries.
  if ((s = ensure(c, kBufHeavy, in.nA * sizeof(HeavyEntry) + (in.nA / kEbThreads + 1) * 4, &ph)) !=
      HD_OK)
    return s;
  uint32_t* group_done = (uint32_t*) ((HeavyEntry*) ph + in.nA);
  DevScalars* sc = scalars(c, in.dir);
  const uint64_t seed = c.opt.seed;
  Perm pB{in.nB, pick_multiplier(in.nB, seed + 1), (seed * 7919u) % in.nB};
  Perm pA{in.nA, pick_multiplier(in.nA, seed + 2), (seed * 104729u) % in.nA};

  {
    int grid = (int) std::min<uint64_t>((nPad + 255) / 256, (uint64_t) c.num_sms * 16);
    k_eb_pack<D><<<grid, 256, 0, c.stream>>>(in.B, in.nB, pB, (PT*) pb, nPad);
    if ((s = after_launch(c, "eb_pack")) != HD_OK) return s;
  }
  mark(c, 1);
  mark(c, 2);
  // Seeds: the first visited A points, scanned in full (the running maximum
  // is still zero) by the tile-wise list pass.  Their list entries sit at the
  // end of the deferred-point list, which the main pass fills from the start.
  // An AUTO solve whose selector already scanned seeds and a sample of A
  // against B starts from the maximum they set instead.
  const uint32_t n_seed =
      c.seeded[in.dir] ? 0u : (uint32_t) std::min<uint64_t>(in.nA, (uint64_t) c.num_sms);
  HeavyEntry* seeds = (HeavyEntry*) ph + (in.nA - n_seed);
  if (n_seed > 0) {
    k_eb_seed_list<<<(n_seed + 255) / 256, 256, 0, c.stream>>>(pA, n_seed, nTiles, seeds);
    if ((s = after_launch(c, "eb_seed_list")) != HD_OK) return s;
    cudaError_t e = eb_list_pass<D>(c.stream, c.num_sms, in.A, (const PT*) pb, nTiles, seeds,
                                    group_done, n_seed, nullptr, n_seed, sc);
    c.launches += 1;
    if (e != cudaSuccess) return cuda_fail(c, e, "eb_seed");
  }
  mark(c, 3);
  if (in.nA > n_seed) {
    // Slots per thread: the most (4, 2, 1) that still fill every resident CTA
    // of a full grid, so that a small set spreads over all SMs instead of
    // leaving most of them idle (every slot of a thread is computed).
    const void* fns[3] = {(const void*) k_eb_main<D, 4>, (const void*) k_eb_main<D, 2>,
                          (const void*) k_eb_main<D, 1>};
    const int slots[3] = {4, 2, 1};
    const uint64_t rest = in.nA - n_seed;
    int pick = 2, occ = 1;
    for (int k = 0; k < 3; ++k) {
      int o = 0;
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, fns[k], kEbThreads, 0);
      o = std::max(1, o);
      if (rest >= (uint64_t) c.num_sms * o * kEbThreads * slots[k] || k == 2) {
        pick = k;
        occ = o;
        break;
      }
    }
    const uint64_t per_cta = (uint64_t) kEbThreads * slots[pick];
    const uint64_t want = (rest + per_cta - 1) / per_cta;
    int grid = (int) std::max<uint64_t>(1, std::min<uint64_t>(want, (uint64_t) c.num_sms * occ));
    // Pairs a point scans before it is paused (deferred): an option, else
    // clamp(|B| / div, min, max) from the tuning table.  Pausing is not only
    // a tail guard: a paused point resumes under a higher running maximum.
    uint64_t cap = c.opt.eb_cap_pairs;
    if (cap == 0)
      cap = std::min<uint64_t>(std::max<uint64_t>(in.nB / tuning().eb_cap_div, tuning().eb_cap_min),
                               tuning().eb_cap_max);
    uint32_t capTiles = (uint32_t) std::max<uint64_t>(1, cap / kEbTile);
    const float* a_ptr = in.A;
    const PT* b_ptr = (const PT*) pb;
    HeavyEntry* h_ptr = (HeavyEntry*) ph;
    uint32_t heavy_cap = (uint32_t) (in.nA - n_seed);
    // Checkpoints: the main pass runs in parts; after each part the points
    // it deferred are finished before the next part starts.  Deferred points
    // include the outliers, whose distances are the ones that lift the
    // running maximum to its final level; finished early, they let the rest
    // break sooner (clusters3d 10M 49.5 -> 38.6 ms with one checkpoint at
    // 1/16).  A checkpoint is kept only when every part fills a full wave.
    const uint64_t wave = (uint64_t) grid * per_cta;
    uint64_t ends[kEbMaxParts];
    int parts = 0;
    uint64_t last = n_seed;
    for (uint64_t div : kEbCheckDiv) {
      const uint64_t e = n_seed + rest / div;
      if (e >= last + wave && in.nA >= e + wave) {
        ends[parts++] = e;
        last = e;
      }
    }
    ends[parts++] = in.nA;
    uint64_t a_begin = n_seed;
    for (int part = 0; part < parts; ++part) {
      uint64_t a_end = ends[part];
      if (part > 0) {
        // A fresh visit counter, and the deferred pass starts after the
        // entries the earlier passes finished.
        k_eb_mark_heavy<<<1, 1, 0, c.stream>>>(sc);
        if ((s = after_launch(c, "eb_mark")) != HD_OK) return s;
      }
      void* args[] = {&a_ptr, &pA, &a_begin, &a_end, &b_ptr, (void*) &nTiles, &capTiles, &sc,
                      &h_ptr, &heavy_cap};
      cudaLaunchKernel(fns[pick], dim3(grid), dim3(kEbThreads), args, 0, c.stream);
      if ((s = after_launch(c, "eb_main")) != HD_OK) return s;
      if (part == parts - 1) mark(c, 4);
      k_eb_heavy<D><<<c.num_sms * 4, kEbThreads, 0, c.stream>>>(
          in.A, (const PT*) pb, nTiles, sc, (const HeavyEntry*) ph, &sc->heavy_count, heavy_cap,
          part > 0 ? &sc->heavy_mark : nullptr);
      if ((s = after_launch(c, "eb_deferred")) != HD_OK) return s;
      a_begin = a_end;
    }
  } else {
    mark(c, 4);
  }
  return certify(c, in);
}

}  // namespace

hd_status run_eb(Ctx& c, const DirInput& in) {
  if (in.dims == 2) return run_eb_dim<2>(c, in);
  if (in.dims == 3) return run_eb_dim<3>(c, in);
  return run_eb_nd(c, in);
}

}  // namespace hdg

// ---------------------------------------------------------------------------
// Early-break solve without any allocation.
//
// Some callers cannot allocate device memory while they call us: code that
// runs under a fixed memory budget handed out up front (a serving process
// that reserves all of its HBM at start-up, an embedded caching allocator
// that must not be bypassed), or host code in a phase where cudaMalloc /
// cudaFree would synchronise the device and stall work the caller keeps in
// flight.  hd_solve_eb_noalloc serves them: it runs the same persistent
// early-break kernels as hd_solve's EB variant, but every byte of scratch it
// needs (the visit-ordered copy of B, the deferred-point list and the two
// result words) lives in the file-scope device array below, sized once for
// point sets of up to kNoAllocMaxPoints points.  The array is part of the
// loaded library, so each GPU that loads it holds kNoAllocBytes (about
// 32 MiB) until the process exits.
namespace hdg {
namespace {

constexpr uint64_t kNoAllocMaxPoints = 1ull << 20;
constexpr size_t kNoAllocScalarBytes = 1024;  // two DevScalars, padded
constexpr size_t kNoAllocHeavyBytes = kNoAllocMaxPoints * sizeof(HeavyEntry);
constexpr size_t kNoAllocPackBytes = kNoAllocMaxPoints * sizeof(float4);
constexpr size_t kNoAllocGroupBytes = (kNoAllocMaxPoints / kEbThreads + 1) * 4;  // list groups
constexpr size_t kNoAllocBytes =
    kNoAllocScalarBytes + kNoAllocHeavyBytes + kNoAllocPackBytes + kNoAllocGroupBytes;
static_assert(2 * sizeof(DevScalars) <= kNoAllocScalarBytes, "scalar area too small");

// In host code this name is only a host-side stand-in for the symbol: its
// device address comes from cudaGetSymbolAddress (see noalloc_scratch).
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

// Device address of the scratch array in the current context.  It is looked
// up on every call rather than cached: the address belongs to the context
// the library's module is loaded in, so it changes after a device reset or
// under another context on the same device.  The lookup is a host-side table
// read and allocates nothing.
cudaError_t noalloc_scratch(unsigned char** out) {
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess) return e;
  *out = (unsigned char*) p;
  return cudaSuccess;
}

template <int D>
cudaError_t noalloc_direction(cudaStream_t st, int num_sms, const float* A, uint64_t nA,
                              const float* B, uint64_t nB, unsigned char* base,
                              DevScalars* sc) {
  using PT = typename EbPt<D>::T;
  const uint32_t nTiles = (uint32_t) ((nB + kEbTile - 1) / kEbTile);
  const uint64_t nPad = (uint64_t) nTiles * kEbTile;
  HeavyEntry* heavy = (HeavyEntry*) (base + kNoAllocScalarBytes);
  PT* pb = (PT*) (base + kNoAllocScalarBytes + kNoAllocHeavyBytes);
  uint32_t* group_done =
      (uint32_t*) (base + kNoAllocScalarBytes + kNoAllocHeavyBytes + kNoAllocPackBytes);
  Perm pB{nB, pick_multiplier(nB, 1), 0};
  Perm pA{nA, pick_multiplier(nA, 2), 0};
  int grid = (int) std::min<uint64_t>((nPad + 255) / 256, (uint64_t) num_sms * 16);
  k_eb_pack<D><<<grid, 256, 0, st>>>(B, nB, pB, pb, nPad);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const uint32_t n_seed = (uint32_t) std::min<uint64_t>(nA, (uint64_t) num_sms);
  HeavyEntry* seeds = heavy + (nA - n_seed);
  k_eb_seed_list<<<(n_seed + 255) / 256, 256, 0, st>>>(pA, n_seed, nTiles, seeds);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if ((e = eb_list_pass<D>(st, num_sms, A, pb, nTiles, seeds, group_done, n_seed, nullptr, n_seed,
                           sc)) != cudaSuccess)
    return e;
  if (nA > n_seed) {
    // Slots per thread chosen as hd_solve's EB variant chooses them: the most
    // (4, 2, 1) that still fill every resident CTA of a full grid.
    const void* fns[3] = {(const void*) k_eb_main<D, 4>, (const void*) k_eb_main<D, 2>,
                          (const void*) k_eb_main<D, 1>};
    const int slots[3] = {4, 2, 1};
    const uint64_t rest = nA - n_seed;
    int pick = 2, occ = 1;
    for (int k = 0; k < 3; ++k) {
      int o = 0;
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, fns[k], kEbThreads, 0);
      o = std::max(1, o);
      if (rest >= (uint64_t) num_sms * o * kEbThreads * slots[k] || k == 2) {
        pick = k;
        occ = o;
        break;
      }
    }
    const uint64_t per_cta = (uint64_t) kEbThreads * slots[pick];
    const uint64_t want = (rest + per_cta - 1) / per_cta;
    const int g = (int) std::max<uint64_t>(1, std::min<uint64_t>(want, (uint64_t) num_sms * occ));
    uint32_t capTiles = std::max<uint32_t>(1, kCapPairs / kEbTile);
    const float* a_ptr = A;
    const PT* b_ptr = pb;
    uint32_t heavy_cap = (uint32_t) (nA - n_seed);
    uint64_t a_begin = n_seed, a_end = nA;
    void* args[] = {&a_ptr, &pA, &a_begin, &a_end, &b_ptr, (void*) &nTiles, &capTiles, &sc,
                    &heavy, &heavy_cap};
    if ((e = cudaLaunchKernel(fns[pick], dim3(g), dim3(kEbThreads), args, 0, st)) != cudaSuccess)
      return e;
    k_eb_heavy<D><<<num_sms * 4, kEbThreads, 0, st>>>(A, pb, nTiles, sc, heavy, &sc->heavy_count,
                                                      heavy_cap, nullptr);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  return certify_on_stream(st, num_sms, A, B, nB, D, sc);
}

}  // namespace
}  // namespace hdg

extern "C" HD_API hd_status hd_solve_eb_noalloc(const float* A, uint64_t n_a, const float* B,
                                                uint64_t n_b, int n_dims, uint32_t flags,
                                                void* stream, hd_result* out) {
  using namespace hdg;
  if (!A || !B || !out) return HD_ERR_INVALID_ARG;
  if (n_a == 0 || n_b == 0) return HD_ERR_INVALID_ARG;
  if (n_dims != 2 && n_dims != 3) return HD_ERR_INVALID_ARG;
  if (flags & ~(HD_UNDIRECTED | HD_DEVICE_PTRS)) return HD_ERR_INVALID_ARG;
  // Inputs beyond the fixed scratch capacity are rejected, never truncated.
  if (n_a > kNoAllocMaxPoints || n_b > kNoAllocMaxPoints) return HD_ERR_INVALID_ARG;
  cudaStream_t st = (cudaStream_t) stream;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return HD_ERR_NO_DEVICE;
  int num_sms = 0;
  e = cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess || num_sms <= 0) return HD_ERR_NO_DEVICE;
  unsigned char* base = nullptr;
  if ((e = noalloc_scratch(&base)) != cudaSuccess) return HD_ERR_CUDA;
  DevScalars* sc = (DevScalars*) base;
  const bool undirected = (flags & HD_UNDIRECTED) != 0;
  const int ndir = undirected ? 2 : 1;
  // The scratch keeps the previous call's contents: reset the result words.
  e = init_scalars_on_stream(st, sc, 2);
  for (int d = 0; d < ndir && e == cudaSuccess; ++d) {
    const float* x = d == 0 ? A : B;
    const float* y = d == 0 ? B : A;
    const uint64_t nx = d == 0 ? n_a : n_b, ny = d == 0 ? n_b : n_a;
    e = n_dims == 2 ? noalloc_direction<2>(st, num_sms, x, nx, y, ny, base, sc + d)
                    : noalloc_direction<3>(st, num_sms, x, nx, y, ny, base, sc + d);
  }
  if (e != cudaSuccess) {
    // Kernels queued before the failing launch still write the shared
    // array: let them finish so that a retry (on any stream) does not race
    // with them.
    (void) cudaStreamSynchronize(st);
    (void) cudaGetLastError();
    return e == cudaErrorNoKernelImageForDevice ? HD_ERR_NO_DEVICE : HD_ERR_CUDA;
  }
  DevScalars h[2];
  e = cudaMemcpyAsync(h, sc, sizeof(h), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return HD_ERR_CUDA;
  for (int d = 0; d < ndir; ++d) {
    if (h[d].status & kErrWaitTimeout) return HD_ERR_DEVICE_TIMEOUT;
    if (h[d].status) return HD_ERR_CUDA;
  }
  memset(out, 0, sizeof(*out));
  out->hd_ab = std::sqrt(h[0].d2_64);
  out->hd_ba = undirected ? std::sqrt(h[1].d2_64) : -1.0;
  const int win = (undirected && h[1].d2 > h[0].d2) ? 1 : 0;
  out->hd_f32 = std::sqrt(h[win].d2);
  out->hd = std::sqrt(h[win].d2_64);
  out->direction = win;
  out->ia = h[win].ia;
  out->ib = h[win].ib;
  out->visited_pairs = h[0].pairs + (undirected ? h[1].pairs : 0);
  out->variant_used = HD_VARIANT_EB;
  out->variant_used_ba = undirected ? HD_VARIANT_EB : -1;
  return HD_OK;
}
