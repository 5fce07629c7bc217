// Morton sort of one or two point sets: the spatial order every LBVH and
// grid solve starts from.  It replaces a generic key/index radix sort
// followed by a random gather of the points (the shape of the reference's
// grid build, src/index/uniform_grid.h:343-484: sort, binary-search counting,
// atomic scatter) with a sort designed around the data it moves:
//
//  1. count    one pass over the caller's points: Morton code in the set's
//              frame, one atomic increment of the code's bin (its top
//              `30 - shift` bits; about n/8 bins, at most 2^21, so the
//              counters stay in L2).
//  2. scan     exclusive prefix sums of the bin counts (three small launches).
//  3. scatter  a second pass over the caller's points: the record (x, y, z,
//              caller index) and its code go straight to a slot of their bin
//              (atomic cursor).  No index array and no later gather: the
//              coordinates are read once, in the caller's order, coalesced.
//  4. local    every bin is put in full code order in place: bins of up to
//              32 records (nearly all) by a warp bitonic sort in registers,
//              bins of up to kCap records by one CTA in shared memory, larger
//              bins by one CTA that partitions them on the next 8 code bits
//              (ping-ponging with a scratch copy) until the parts fit.
//  5. leaves   the bounding box of every leaf of L consecutive sorted points.
//
// Records of equal code keep no particular order (nothing depends on it:
// results are exact whatever the order; certification picks the lowest
// caller index by itself).
#include <cfloat>

#include "hd_common.cuh"
#include "hd_internal.h"
#include "hd_msort.h"

namespace hdg {
namespace {

constexpr int kScanTile = 2048;      // bins per CTA in the scan
constexpr int kLocalBins = 4;        // bins per warp in the local pass
constexpr uint32_t kCap = 4096;      // records a CTA sorts in shared memory
constexpr int kSortThreads = 512;
constexpr int kBigStack = 1280;      // pending parts of one large bin

__device__ __forceinline__ const MsortSet& set_of(const MsortSets& s) { return s.s[blockIdx.y]; }

// Sum of v over the CTA (every thread gets it).
__device__ __forceinline__ uint32_t block_sum_u32(uint32_t v) {
  __shared__ uint32_t part[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
  __syncthreads();
  if (lane == 0) part[warp] = v;
  __syncthreads();
  uint32_t t = 0;
  for (int w = 0; w < (int) (blockDim.x >> 5); ++w) t += part[w];
  return t;
}

// Exclusive prefix sum of v over the CTA in thread order.
__device__ __forceinline__ uint32_t block_exclusive_scan_u32(uint32_t v) {
  __shared__ uint32_t part[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
    if (lane >= o) x += y;
  }
  __syncthreads();
  if (lane == 31) part[warp] = x;
  __syncthreads();
  uint32_t before = 0;
  for (int w = 0; w < warp; ++w) before += part[w];
  return before + x - v;
}

template <int D>
__device__ __forceinline__ void load_point(const float* __restrict__ P, uint64_t i, float& x,
                                           float& y, float& z) {
  x = P[i * D];
  y = P[i * D + 1];
  z = D == 3 ? P[i * D + 2] : 0.0f;
}

template <int D>
__global__ void __launch_bounds__(256) k_ms_count(MsortSets ss) {
  const MsortSet& S = set_of(ss);
  const Frame f = *S.fr;
  for (uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < S.n;
       i += (uint64_t) gridDim.x * blockDim.x) {
    float x, y, z;
    load_point<D>(S.P, i, x, y, z);
    atomicAdd(&S.bins[frame_code<D>(f, x, y, z) >> S.shift], 1u);
  }
}

// Scan, step 1: the sum of every tile of kScanTile bins.
__global__ void __launch_bounds__(256) k_ms_scan_tiles(MsortSets ss) {
  const MsortSet& S = set_of(ss);
  const uint32_t t0 = blockIdx.x * kScanTile;
  if (t0 >= S.nbins) return;
  uint32_t v = 0;
  for (uint32_t i = t0 + threadIdx.x; i < min(S.nbins, t0 + kScanTile); i += blockDim.x)
    v += S.bins[i];
  v = block_sum_u32(v);
  if (threadIdx.x == 0) S.tile_sums[blockIdx.x] = v;
}

// Scan, step 2: exclusive sums of the tile sums (one CTA per set; at most
// 2^21 / kScanTile = 1024 tiles).
__global__ void __launch_bounds__(1024) k_ms_scan_top(MsortSets ss) {
  const MsortSet& S = set_of(ss);
  const uint32_t tiles = (S.nbins + kScanTile - 1) / kScanTile;
  const uint32_t i = threadIdx.x;
  const uint32_t v = i < tiles ? S.tile_sums[i] : 0u;
  const uint32_t ex = block_exclusive_scan_u32(v);
  if (i < tiles) S.tile_sums[i] = ex;
}

// Scan, step 3: exclusive bin starts, written over the counts.
__global__ void __launch_bounds__(256) k_ms_scan_apply(MsortSets ss) {
  const MsortSet& S = set_of(ss);
  const uint32_t t0 = blockIdx.x * kScanTile;
  if (t0 >= S.nbins) return;
  constexpr int kPer = kScanTile / 256;
  uint32_t v[kPer];
  uint32_t sum = 0;
#pragma unroll
  for (int k = 0; k < kPer; ++k) {
    const uint32_t b = t0 + threadIdx.x * kPer + k;
    v[k] = b < S.nbins ? S.bins[b] : 0u;
    sum += v[k];
  }
  uint32_t run = block_exclusive_scan_u32(sum) + S.tile_sums[blockIdx.x];
#pragma unroll
  for (int k = 0; k < kPer; ++k) {
    const uint32_t b = t0 + threadIdx.x * kPer + k;
    if (b < S.nbins) S.bins[b] = run;
    run += v[k];
  }
}

// After the scatter bins[b] is the end of bin b, i.e. the start of bin b+1.
__device__ __forceinline__ uint32_t bin_begin(const MsortSet& S, uint32_t b) {
  return b == 0 ? 0u : S.bins[b - 1];
}

template <int D>
__global__ void __launch_bounds__(256) k_ms_scatter(MsortSets ss) {
  const MsortSet& S = set_of(ss);
  const Frame f = *S.fr;
  for (uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < S.n;
       i += (uint64_t) gridDim.x * blockDim.x) {
    float x, y, z;
    load_point<D>(S.P, i, x, y, z);
    const uint32_t code = frame_code<D>(f, x, y, z);
    const uint32_t slot = atomicAdd(&S.bins[code >> S.shift], 1u);
    S.pts[slot] = make_float4(x, y, z, __uint_as_float((uint32_t) i));
    S.codes[slot] = code;
  }
}

// Sorts the records [rs, re) (at most 32) of one warp by code, in place:
// bitonic network over (code, lane) in registers, records moved by shuffles.
__device__ __forceinline__ void warp_sort_range(const MsortSet& S, uint32_t rs, uint32_t re,
                                                int lane) {
  const uint32_t m = re - rs;
  float4 p = make_float4(0.f, 0.f, 0.f, 0.f);
  uint32_t k = 0xFFFFFFFFu;
  if ((uint32_t) lane < m) {
    p = S.pts[rs + lane];
    k = S.codes[rs + lane];
  }
  uint32_t v = (uint32_t) lane;
  const uint32_t k_in = k;
#pragma unroll
  for (int size = 2; size <= 32; size <<= 1) {
#pragma unroll
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      const uint32_t ok = __shfl_xor_sync(0xFFFFFFFFu, k, stride);
      const uint32_t ov = __shfl_xor_sync(0xFFFFFFFFu, v, stride);
      const bool up = (lane & size) == 0 || size == 32;
      const bool lower = (lane & stride) == 0;
      const bool other_less = ok < k || (ok == k && ov < v);
      if (lower == up ? other_less : !other_less) {
        k = ok;
        v = ov;
      }
    }
  }
  // Nothing to write when the range was already in order.
  if (!__any_sync(0xFFFFFFFFu, (uint32_t) lane < m && k != k_in)) return;
  float4 q;
  q.x = __shfl_sync(0xFFFFFFFFu, p.x, v);
  q.y = __shfl_sync(0xFFFFFFFFu, p.y, v);
  q.z = __shfl_sync(0xFFFFFFFFu, p.z, v);
  q.w = __shfl_sync(0xFFFFFFFFu, p.w, v);
  if ((uint32_t) lane < m) {
    S.pts[rs + lane] = q;
    S.codes[rs + lane] = k;
  }
}

// Local pass: warp w takes bins [w*kLocalBins, (w+1)*kLocalBins).  A range of
// at most 32 records is sorted as one (its bins are already in order, so the
// whole range in code order is the answer); otherwise bin by bin, handing
// bins of more than 32 records to the CTA passes through two lists.
__global__ void __launch_bounds__(256) k_ms_local(MsortSets ss) {
  const MsortSet& S = set_of(ss);
  const int lane = threadIdx.x & 31;
  const uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t b0 = w * kLocalBins;
  if (b0 >= S.nbins) return;
  const uint32_t b1 = min(S.nbins, b0 + kLocalBins);
  const uint32_t rs = bin_begin(S, b0), re = S.bins[b1 - 1];
  if (re - rs <= 1) return;
  if (re - rs <= 32) {
    warp_sort_range(S, rs, re, lane);
    return;
  }
  for (uint32_t b = b0; b < b1; ++b) {
    const uint32_t s = bin_begin(S, b), e = S.bins[b];
    const uint32_t m = e - s;
    if (m <= 1) continue;
    if (m <= 32) {
      warp_sort_range(S, s, e, lane);
    } else if (lane == 0) {
      // Larger bins: one CTA each (kCap at most in shared memory, beyond
      // that the partitioning pass).
      if (m <= kCap) {
        const uint32_t slot = atomicAdd(&S.counters[0], 1u);
        if (slot < S.list_cap) S.mid_list[slot] = b;
        else atomicOr(S.status, kErrInternal);
      } else {
        const uint32_t slot = atomicAdd(&S.counters[1], 1u);
        if (slot < S.list_cap) S.big_list[slot] = b;
        else atomicOr(S.status, kErrInternal);
      }
    }
  }
}

// Shared-memory sort of up to kCap records src[s, e) (codes sc, points sp)
// into the final arrays at [s, e): bitonic network over (code, position).
struct SortSmem {
  uint32_t key[kCap];
  uint16_t idx[kCap];
  float4 pt[kCap];
};

__device__ void cta_sort_range(const MsortSet& S, const uint32_t* __restrict__ sc,
                               const float4* __restrict__ sp, uint32_t s, uint32_t e,
                               SortSmem& sm) {
  const uint32_t m = e - s;
  uint32_t P = 1;
  while (P < m) P <<= 1;
  for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) {
    if (i < m) {
      sm.key[i] = sc[s + i];
      sm.pt[i] = sp[s + i];
    } else {
      sm.key[i] = 0xFFFFFFFFu;
    }
    sm.idx[i] = (uint16_t) i;
  }
  __syncthreads();
  for (uint32_t size = 2; size <= P; size <<= 1) {
    for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
      for (uint32_t t = threadIdx.x; t < P / 2; t += blockDim.x) {
        // Pair (i, i + stride) with i's stride bit clear.
        const uint32_t i = 2 * t - (t & (stride - 1));
        const uint32_t j = i + stride;
        const bool up = (i & size) == 0;
        const uint32_t ki = sm.key[i], kj = sm.key[j];
        const uint16_t vi = sm.idx[i], vj = sm.idx[j];
        const bool j_less = kj < ki || (kj == ki && vj < vi);
        if (up == j_less) {
          sm.key[i] = kj;
          sm.key[j] = ki;
          sm.idx[i] = vj;
          sm.idx[j] = vi;
        }
      }
      __syncthreads();
    }
  }
  for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) {
    S.pts[s + i] = sm.pt[sm.idx[i]];
    S.codes[s + i] = sm.key[i];
  }
  __syncthreads();
}

// Bins of 33..kCap records, one CTA each (grid-stride over the list).
__global__ void __launch_bounds__(kSortThreads) k_ms_mid(MsortSets ss) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SortSmem& sm = *reinterpret_cast<SortSmem*>(smem_raw);
  const MsortSet& S = set_of(ss);
  const uint32_t cnt = min(*(volatile uint32_t*) &S.counters[0], S.list_cap);
  for (uint32_t k = blockIdx.x; k < cnt; k += gridDim.x) {
    const uint32_t b = S.mid_list[k];
    cta_sort_range(S, S.codes, S.pts, bin_begin(S, b), S.bins[b], sm);
  }
}

// Bins of more than kCap records, one CTA each: partition on the next 8 code
// bits (count, scan, scatter into the other buffer), then sort the parts
// that fit in shared memory and partition the others again.  After all 30
// bits a part holds one code and needs no order.  The pending parts live in
// a shared-memory stack; a part that would overflow it sets the set's error
// counter (the solve then fails) rather than being dropped.
struct BigSmem {
  SortSmem sort;
  uint32_t hist[256];
  uint32_t stk_s[kBigStack], stk_e[kBigStack];
  uint8_t stk_b[kBigStack], stk_t[kBigStack];
  int sp;
  uint32_t nonempty;
};

__global__ void __launch_bounds__(kSortThreads) k_ms_big(MsortSets ss) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  BigSmem& sm = *reinterpret_cast<BigSmem*>(smem_raw);
  const MsortSet& S = set_of(ss);
  const uint32_t cnt = min(*(volatile uint32_t*) &S.counters[1], S.list_cap);
  for (uint32_t k = blockIdx.x; k < cnt; k += gridDim.x) {
    const uint32_t b = S.big_list[k];
    if (threadIdx.x == 0) {
      sm.stk_s[0] = bin_begin(S, b);
      sm.stk_e[0] = S.bins[b];
      sm.stk_b[0] = (uint8_t) S.shift;  // code bits below this are unordered
      sm.stk_t[0] = 0;                  // 0: records are in the final arrays
      sm.sp = 1;
    }
    __syncthreads();
    while (sm.sp > 0) {
      const int top = sm.sp - 1;
      const uint32_t s = sm.stk_s[top], e = sm.stk_e[top];
      const uint32_t lo = sm.stk_b[top];
      const bool in_tmp = sm.stk_t[top] != 0;
      __syncthreads();
      if (threadIdx.x == 0) sm.sp = top;
      const uint32_t* sc = in_tmp ? S.tcodes : S.codes;
      const float4* sp = in_tmp ? S.tpts : S.pts;
      const uint32_t m = e - s;
      if (m <= kCap) {
        cta_sort_range(S, sc, sp, s, e, sm.sort);
        continue;
      }
      if (lo == 0) {
        // One code throughout: copy back if the records sit in the scratch.
        if (in_tmp)
          for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) {
            S.pts[s + i] = sp[s + i];
            S.codes[s + i] = sc[s + i];
          }
        __syncthreads();
        continue;
      }
      const uint32_t d = min(lo, 8u), nb = lo - d;
      const uint32_t mask = (1u << d) - 1u;
      for (uint32_t i = threadIdx.x; i < 256; i += blockDim.x) sm.hist[i] = 0;
      __syncthreads();
      for (uint32_t i = threadIdx.x; i < m; i += blockDim.x)
        atomicAdd(&sm.hist[(sc[s + i] >> nb) & mask], 1u);
      __syncthreads();
      if (threadIdx.x == 0) {
        uint32_t run = s, parts = 0;
        for (uint32_t q = 0; q <= mask; ++q) {
          const uint32_t c = sm.hist[q];
          sm.hist[q] = run;
          run += c;
          parts += c ? 1u : 0u;
        }
        sm.nonempty = parts;
      }
      __syncthreads();
      if (sm.nonempty == 1) {
        // Every record has the same digit: nothing moves, go one digit down.
        if (threadIdx.x == 0) {
          sm.stk_s[top] = s;
          sm.stk_e[top] = e;
          sm.stk_b[top] = (uint8_t) nb;
          sm.stk_t[top] = in_tmp ? 1 : 0;
          sm.sp = top + 1;
        }
        __syncthreads();
        continue;
      }
      uint32_t* dc = in_tmp ? S.codes : S.tcodes;
      float4* dp = in_tmp ? S.pts : S.tpts;
      // Part starts, kept for the stack before the scatter advances them.
      if (threadIdx.x == 0) {
        int p = top;
        for (uint32_t q = 0; q <= mask; ++q) {
          const uint32_t qs = sm.hist[q];
          const uint32_t qe = q < mask ? sm.hist[q + 1] : e;
          if (qe > qs) {
            if (p < kBigStack) {
              sm.stk_s[p] = qs;
              sm.stk_e[p] = qe;
              sm.stk_b[p] = (uint8_t) nb;
              sm.stk_t[p] = in_tmp ? 0 : 1;
            }
            ++p;
          }
        }
        if (p > kBigStack) {
          atomicOr(S.status, kErrInternal);
          p = kBigStack;
        }
        sm.sp = p;
      }
      __syncthreads();
      for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) {
        const uint32_t c = sc[s + i];
        const uint32_t slot = atomicAdd(&sm.hist[(c >> nb) & mask], 1u);
        dc[slot] = c;
        dp[slot] = sp[s + i];
      }
      __syncthreads();
    }
    __syncthreads();
  }
}

// Leaf boxes: lanes of a warp cover whole leaves of L (a power of two <= 32)
// consecutive sorted points; min/max by shuffles.
__global__ void __launch_bounds__(256) k_ms_leaves(MsortSets ss) {
  const MsortSet& S = set_of(ss);
  const uint64_t stride = (uint64_t) gridDim.x * blockDim.x;
  for (uint64_t j0 = blockIdx.x * (uint64_t) blockDim.x + (threadIdx.x & ~31u); j0 < S.n;
       j0 += stride) {
    const uint64_t j = j0 + (threadIdx.x & 31u);
    const bool valid = j < S.n;
    float lx = FLT_MAX, ly = FLT_MAX, lz = FLT_MAX, hx = -FLT_MAX, hy = -FLT_MAX, hz = -FLT_MAX;
    if (valid) {
      const float4 p = S.pts[j];
      lx = hx = p.x;
      ly = hy = p.y;
      lz = hz = p.z;
    }
    for (uint32_t o = 1; o < S.L; o <<= 1) {
      lx = fminf(lx, __shfl_xor_sync(0xFFFFFFFFu, lx, o));
      ly = fminf(ly, __shfl_xor_sync(0xFFFFFFFFu, ly, o));
      lz = fminf(lz, __shfl_xor_sync(0xFFFFFFFFu, lz, o));
      hx = fmaxf(hx, __shfl_xor_sync(0xFFFFFFFFu, hx, o));
      hy = fmaxf(hy, __shfl_xor_sync(0xFFFFFFFFu, hy, o));
      hz = fmaxf(hz, __shfl_xor_sync(0xFFFFFFFFu, hz, o));
    }
    if (valid && (j & (S.L - 1)) == 0) {
      const uint64_t leaf = j / S.L;
      S.leaf_boxes[2 * leaf] = make_float4(lx, ly, lz, 0.f);
      S.leaf_boxes[2 * leaf + 1] = make_float4(hx, hy, hz, 0.f);
    }
  }
}

}  // namespace

uint32_t msort_shift(uint64_t n) {
  // About n/8 bins, between 2^10 and 2^21.
  uint32_t bits = 10;
  while (bits < 21 && (1ull << bits) < (n + 7) / 8) ++bits;
  return 30u - bits;
}

hd_status msort_run(Ctx& c, MsortSets& ss, int count, int dims, cudaStream_t st) {
  hd_status s;
  cudaFuncSetAttribute(k_ms_mid, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int) sizeof(SortSmem));
  cudaFuncSetAttribute(k_ms_big, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int) sizeof(BigSmem));
  uint64_t maxn = 0;
  uint32_t maxbins = 0;
  for (int k = 0; k < count; ++k) {
    maxn = std::max<uint64_t>(maxn, ss.s[k].n);
    maxbins = std::max(maxbins, ss.s[k].nbins);
    cudaError_t e = cudaMemsetAsync(ss.s[k].bins, 0, (size_t) ss.s[k].nbins * 4, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(ss.s[k].counters, 0, 4 * sizeof(uint32_t), st);
    if (e != cudaSuccess) return cuda_fail(c, e, "memset sort counters");
  }
  // A set with fewer bins than the other leaves its extra CTAs idle.
  if (count == 1) ss.s[1] = ss.s[0];
  const unsigned ny = (unsigned) count;
  const unsigned gpts = (unsigned) std::max<uint64_t>(
      1, std::min<uint64_t>((maxn + 255) / 256, (uint64_t) c.num_sms * 8));
  if (dims == 2)
    k_ms_count<2><<<dim3(gpts, ny), 256, 0, st>>>(ss);
  else
    k_ms_count<3><<<dim3(gpts, ny), 256, 0, st>>>(ss);
  if ((s = after_launch(c, "msort_count")) != HD_OK) return s;
  const unsigned tiles = (maxbins + kScanTile - 1) / kScanTile;
  k_ms_scan_tiles<<<dim3(tiles, ny), 256, 0, st>>>(ss);
  if ((s = after_launch(c, "msort_scan_tiles")) != HD_OK) return s;
  k_ms_scan_top<<<dim3(1, ny), 1024, 0, st>>>(ss);
  if ((s = after_launch(c, "msort_scan_top")) != HD_OK) return s;
  k_ms_scan_apply<<<dim3(tiles, ny), 256, 0, st>>>(ss);
  if ((s = after_launch(c, "msort_scan_apply")) != HD_OK) return s;
  if (dims == 2)
    k_ms_scatter<2><<<dim3(gpts, ny), 256, 0, st>>>(ss);
  else
    k_ms_scatter<3><<<dim3(gpts, ny), 256, 0, st>>>(ss);
  if ((s = after_launch(c, "msort_scatter")) != HD_OK) return s;
  const uint64_t warps = (maxbins + kLocalBins - 1) / kLocalBins;
  k_ms_local<<<dim3((unsigned) ((warps * 32 + 255) / 256), ny), 256, 0, st>>>(ss);
  if ((s = after_launch(c, "msort_local")) != HD_OK) return s;
  k_ms_mid<<<dim3((unsigned) c.num_sms * 2, ny), kSortThreads, sizeof(SortSmem), st>>>(ss);
  if ((s = after_launch(c, "msort_mid")) != HD_OK) return s;
  k_ms_big<<<dim3((unsigned) c.num_sms, ny), kSortThreads, sizeof(BigSmem), st>>>(ss);
  if ((s = after_launch(c, "msort_big")) != HD_OK) return s;
  k_ms_leaves<<<dim3(gpts, ny), 256, 0, st>>>(ss);
  return after_launch(c, "msort_leaves");
}

}  // namespace hdg
