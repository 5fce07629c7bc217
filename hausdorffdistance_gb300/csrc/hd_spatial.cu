// Spatial preparation shared by the LBVH and grid variants: bounding boxes,
// Morton codes in a cubic frame, a radix sort, and a gather into Morton
// order as float4 (x, y, z, caller index).  Large sets run as two
// independent chains, each set in its own frame (main stream and side
// stream), so for host inputs A is sorted while B is still being copied;
// small sets run one fused chain in a common frame.
//
// Replaces the reference's MBR reduction (src/geoms/mbr.h:307-321: thrust
// for_each with CAS float atomics per point) and the first half of the grid
// build (src/index/uniform_grid.h:343-484: occupancy bitset, copy_if, sort,
// binary-search counting, atomic scatter): here the sort itself produces the
// cell order, because a cubic Morton frame makes every grid level a prefix of
// the code.
#include <cub/device/device_radix_sort.cuh>

#include <cfloat>

#include "hd_common.cuh"
#include "hd_internal.h"

namespace hdg {
namespace {

// Bounding boxes of one or two sets in one launch (blockIdx.y = set): per-thread
// min/max, a warp reduction, one shared atomic per warp and one global
// atomic per CTA and dimension on the order-preserving integer image of the
// float.  When the array is 16-byte aligned, 4 points (3-D) or 2 points (2-D)
// are read per three or one 16-byte loads.
__device__ __forceinline__ void mbr_acc(float* lo, float* hi, int k, float v) {
  lo[k] = fminf(lo[k], v);
  hi[k] = fmaxf(hi[k], v);
}

__global__ void k_mbr2(const float* __restrict__ P0, uint64_t n0, const float* __restrict__ P1,
                       uint64_t n1, int dims, uint32_t* __restrict__ ord0,
                       uint32_t* __restrict__ ord1) {
  const float* P = blockIdx.y ? P1 : P0;
  const uint64_t n = blockIdx.y ? n1 : n0;
  uint32_t* ord = blockIdx.y ? ord1 : ord0;
  float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX};
  float hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
  const uint64_t tid = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x;
  const uint64_t stride = (uint64_t) gridDim.x * blockDim.x;
  uint64_t done = 0;
  if ((reinterpret_cast<uintptr_t>(P) & 15) == 0) {
    const float4* P4 = reinterpret_cast<const float4*>(P);
    if (dims == 3) {
      const uint64_t groups = n / 4;
      for (uint64_t g = tid; g < groups; g += stride) {
        const float4 f0 = P4[3 * g], f1 = P4[3 * g + 1], f2 = P4[3 * g + 2];
        mbr_acc(lo, hi, 0, f0.x); mbr_acc(lo, hi, 1, f0.y); mbr_acc(lo, hi, 2, f0.z);
        mbr_acc(lo, hi, 0, f0.w); mbr_acc(lo, hi, 1, f1.x); mbr_acc(lo, hi, 2, f1.y);
        mbr_acc(lo, hi, 0, f1.z); mbr_acc(lo, hi, 1, f1.w); mbr_acc(lo, hi, 2, f2.x);
        mbr_acc(lo, hi, 0, f2.y); mbr_acc(lo, hi, 1, f2.z); mbr_acc(lo, hi, 2, f2.w);
      }
      done = groups * 4;
    } else if (dims == 2) {
      const uint64_t groups = n / 2;
      for (uint64_t g = tid; g < groups; g += stride) {
        const float4 f = P4[g];
        mbr_acc(lo, hi, 0, f.x); mbr_acc(lo, hi, 1, f.y);
        mbr_acc(lo, hi, 0, f.z); mbr_acc(lo, hi, 1, f.w);
      }
      done = groups * 2;
    }
  }
  for (uint64_t i = done + tid; i < n; i += stride)
    for (int k = 0; k < dims; ++k) mbr_acc(lo, hi, k, P[i * dims + k]);
  __shared__ uint32_t s_lo[3], s_hi[3];
  if (threadIdx.x < 3) {
    s_lo[threadIdx.x] = 0xFFFFFFFFu;
    s_hi[threadIdx.x] = 0u;
  }
  __syncthreads();
  for (int k = 0; k < dims; ++k) {
    float a = lo[k], b = hi[k];
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      a = fminf(a, __shfl_xor_sync(0xFFFFFFFFu, a, o));
      b = fmaxf(b, __shfl_xor_sync(0xFFFFFFFFu, b, o));
    }
    if ((threadIdx.x & 31) == 0) {
      atomicMin(&s_lo[k], f2ord(a));
      atomicMax(&s_hi[k], f2ord(b));
    }
  }
  __syncthreads();
  if (threadIdx.x < (unsigned) dims) {
    atomicMin(&ord[threadIdx.x], s_lo[threadIdx.x]);
    atomicMax(&ord[4 + threadIdx.x], s_hi[threadIdx.x]);
  }
}

__global__ void k_frame(const uint32_t* __restrict__ ordA, const uint32_t* __restrict__ ordB,
                        int dims, int use_a, int use_b, Frame* fr) {
  if (threadIdx.x != 0) return;
  float ext = 0.0f;
  for (int k = 0; k < 3; ++k) {
    float lo = FLT_MAX, hi = -FLT_MAX;
    if (k < dims) {
      if (use_a) {
        lo = fminf(lo, ord2f(ordA[k]));
        hi = fmaxf(hi, ord2f(ordA[4 + k]));
      }
      if (use_b) {
        lo = fminf(lo, ord2f(ordB[k]));
        hi = fmaxf(hi, ord2f(ordB[4 + k]));
      }
    } else {
      lo = hi = 0.0f;
    }
    fr->lo[k] = lo;
    fr->hi[k] = hi;
    ext = fmaxf(ext, hi - lo);
  }
  // 30-bit codes in both cases.
  const int bits = dims == 2 ? 15 : 10;
  fr->bits = bits;
  fr->dims = dims;
  fr->extent = ext;
  // Cubic frame: one scale for every axis so that Morton levels are cubes.
  fr->scale = ext > 0.0f ? (float) ((1u << bits) - 1) / ext : 0.0f;
}

// Morton codes of one set in its frame: key = code, value = row.
template <int D>
__global__ void k_morton1(const float* __restrict__ P, uint64_t n, const Frame* __restrict__ fr,
                          uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
  const Frame f = *fr;
  for (uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < n;
       i += (uint64_t) gridDim.x * blockDim.x) {
    const float x = P[i * D], y = P[i * D + 1];
    const float z = D == 3 ? P[i * D + 2] : 0.0f;
    keys[i] = frame_code<D>(f, x, y, z);
    vals[i] = (uint32_t) i;
  }
}

// Gathers one sorted set into float4 (x, y, z, caller index) and, in the
// same pass, the bounding box of every leaf of L consecutive sorted points
// (L a power of two <= 32; lanes of a warp cover whole leaves, reduced with
// shuffles).
__global__ void k_gather1(const float* __restrict__ P, uint64_t n, int dims,
                          const uint32_t* __restrict__ order, float4* __restrict__ out, uint32_t L,
                          float4* __restrict__ lb) {
  const uint64_t stride = (uint64_t) gridDim.x * blockDim.x;
  for (uint64_t j0 = blockIdx.x * (uint64_t) blockDim.x + (threadIdx.x & ~31u); j0 < n; j0 += stride) {
    const uint64_t j = j0 + (threadIdx.x & 31u);
    const bool valid = j < n;
    float4 p = make_float4(0.f, 0.f, 0.f, 0.f);
    float lx = FLT_MAX, ly = FLT_MAX, lz = FLT_MAX, hx = -FLT_MAX, hy = -FLT_MAX, hz = -FLT_MAX;
    if (valid) {
      const uint64_t r = order[j];
      p.x = P[r * dims];
      p.y = P[r * dims + 1];
      p.z = dims == 3 ? P[r * dims + 2] : 0.0f;
      p.w = __uint_as_float((uint32_t) r);
      out[j] = p;
      lx = hx = p.x;
      ly = hy = p.y;
      lz = hz = p.z;
    }
    for (uint32_t o = 1; o < L; o <<= 1) {
      lx = fminf(lx, __shfl_xor_sync(0xFFFFFFFFu, lx, o));
      ly = fminf(ly, __shfl_xor_sync(0xFFFFFFFFu, ly, o));
      lz = fminf(lz, __shfl_xor_sync(0xFFFFFFFFu, lz, o));
      hx = fmaxf(hx, __shfl_xor_sync(0xFFFFFFFFu, hx, o));
      hy = fmaxf(hy, __shfl_xor_sync(0xFFFFFFFFu, hy, o));
      hz = fmaxf(hz, __shfl_xor_sync(0xFFFFFFFFu, hz, o));
    }
    if (valid && (j & (L - 1)) == 0) {
      const uint64_t leaf = j / L;
      lb[2 * leaf] = make_float4(lx, ly, lz, 0.f);
      lb[2 * leaf + 1] = make_float4(hx, hy, hz, 0.f);
    }
  }
}

// Morton codes of both sets in one launch (blockIdx.y = set); the key carries
// the set in bit 30 so one radix sort orders A's points and then B's.
__global__ void k_morton2(const float* __restrict__ A, uint64_t nA, const float* __restrict__ B,
                          uint64_t nB, int dims, const Frame* __restrict__ fr,
                          uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
  const float* P = blockIdx.y ? B : A;
  const uint64_t n = blockIdx.y ? nB : nA;
  const uint64_t base = blockIdx.y ? nA : 0;
  const uint32_t setbit = blockIdx.y ? (1u << 30) : 0u;
  const float lo0 = fr->lo[0], lo1 = fr->lo[1], lo2 = fr->lo[2], s = fr->scale;
  const uint32_t maxq = (1u << fr->bits) - 1u;
  for (uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < n;
       i += (uint64_t) gridDim.x * blockDim.x) {
    uint32_t code;
    if (dims == 2) {
      code = morton_spread2(frame_quant(P[2 * i], lo0, s, maxq)) |
             (morton_spread2(frame_quant(P[2 * i + 1], lo1, s, maxq)) << 1);
    } else {
      code = morton_spread3(frame_quant(P[3 * i], lo0, s, maxq)) |
             (morton_spread3(frame_quant(P[3 * i + 1], lo1, s, maxq)) << 1) |
             (morton_spread3(frame_quant(P[3 * i + 2], lo2, s, maxq)) << 2);
    }
    keys[base + i] = code | setbit;
    vals[base + i] = (uint32_t) (base + i);
  }
}

// Gathers the sorted sets (blockIdx.y = set) into float4 (x, y, z, index
// within its own set) and, in the same pass, the bounding box of every leaf
// of L consecutive sorted points (L a power of two <= 32; lanes of a warp
// cover whole leaves, reduced with shuffles).
__global__ void k_gather2(const float* __restrict__ A, uint64_t nA, const float* __restrict__ B,
                          uint64_t nB, int dims, const uint32_t* __restrict__ order,
                          float4* __restrict__ out, uint32_t L, float4* __restrict__ leaf_boxes,
                          uint64_t leaf_off_b) {
  const bool setb = blockIdx.y != 0;
  const float* P = setb ? B : A;
  const uint64_t n = setb ? nB : nA;
  const uint64_t base = setb ? nA : 0;
  float4* lb = leaf_boxes + (setb ? 2 * leaf_off_b : 0);
  const uint64_t stride = (uint64_t) gridDim.x * blockDim.x;
  for (uint64_t j0 = blockIdx.x * (uint64_t) blockDim.x + (threadIdx.x & ~31u); j0 < n; j0 += stride) {
    const uint64_t j = j0 + (threadIdx.x & 31u);
    const bool valid = j < n;
    float4 p = make_float4(0.f, 0.f, 0.f, 0.f);
    float lx = FLT_MAX, ly = FLT_MAX, lz = FLT_MAX, hx = -FLT_MAX, hy = -FLT_MAX, hz = -FLT_MAX;
    if (valid) {
      const uint64_t v = order[base + j];
      const uint64_t r = setb ? v - nA : v;
      p.x = P[r * dims];
      p.y = P[r * dims + 1];
      p.z = dims == 3 ? P[r * dims + 2] : 0.0f;
      p.w = __uint_as_float((uint32_t) r);
      out[base + j] = p;
      lx = hx = p.x;
      ly = hy = p.y;
      lz = hz = p.z;
    }
    for (uint32_t o = 1; o < L; o <<= 1) {
      lx = fminf(lx, __shfl_xor_sync(0xFFFFFFFFu, lx, o));
      ly = fminf(ly, __shfl_xor_sync(0xFFFFFFFFu, ly, o));
      lz = fminf(lz, __shfl_xor_sync(0xFFFFFFFFu, lz, o));
      hx = fmaxf(hx, __shfl_xor_sync(0xFFFFFFFFu, hx, o));
      hy = fmaxf(hy, __shfl_xor_sync(0xFFFFFFFFu, hy, o));
      hz = fmaxf(hz, __shfl_xor_sync(0xFFFFFFFFu, hz, o));
    }
    if (valid && (j & (L - 1)) == 0) {
      const uint64_t leaf = j / L;
      lb[2 * leaf] = make_float4(lx, ly, lz, 0.f);
      lb[2 * leaf + 1] = make_float4(hx, hy, hz, 0.f);
    }
  }
}

// Stratified sample of k positions in [0, n): position i lies in stratum
// [i*n/k, (i+1)*n/k) at an offset drawn from a counter-based hash
// (splitmix64).  It stands in for the reference's per-sample curand draws
// with replacement (src/sampler.h:26, :50-65).  Over a Morton-sorted set the
// positions come out sorted, so 32 consecutive samples form a spatially
// coherent packet while the sample still covers the whole set.
__global__ void k_sample(uint64_t n, uint32_t k, uint64_t seed, uint32_t* __restrict__ out) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= k) return;
  uint64_t z = seed + 0x9E3779B97F4A7C15ull * (i + 1);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  const uint64_t lo = (uint64_t) i * n / k, hi = (uint64_t) (i + 1) * n / k;
  const uint64_t w = hi > lo ? hi - lo : 1;
  out[i] = (uint32_t) min(lo + z % w, n - 1);
}

int grid_for(Ctx& c, uint64_t n, int per = 256) {
  uint64_t g = (n + per - 1) / per;
  g = std::min<uint64_t>(g, (uint64_t) c.num_sms * 16);
  return (int) std::max<uint64_t>(g, 1);
}

}  // namespace

Frame* frame(Ctx& c, int set) {
  return reinterpret_cast<Frame*>(reinterpret_cast<DevScalars*>(c.bufs[kBufScalars].p) + 2) + set;
}

namespace {

// Scratch of both sets' sorts, allocated before either chain launches (an
// allocation may synchronise the device).  Set 1 uses the upper halves.
struct SortScratch {
  uint32_t *keys, *keys2, *vals, *vals2;
  unsigned char* tmp;
  size_t tmp_bytes, tmp_stride;
  float4* pts;
  float4* lboxes;
  uint64_t nA, leaves_a;
  uint32_t L;
};

hd_status sort_scratch(Ctx& c, uint64_t nA, uint64_t nB, bool fused, SortScratch* x) {
  const uint64_t n = nA + nB;
  uint32_t L = c.opt.leaf_size ? std::min<uint32_t>(c.opt.leaf_size, 32) : 16;
  while (L & (L - 1)) L &= L - 1;
  const uint64_t leaves_a = (nA + L - 1) / L, leaves_b = (nB + L - 1) / L;
  hd_status s;
  void *keys, *keys2, *vals, *vals2, *tmp, *pts, *lboxes;
  if ((s = ensure(c, kBufKeys, n * 4, &keys)) != HD_OK) return s;
  if ((s = ensure(c, kBufKeysAlt, n * 4, &keys2)) != HD_OK) return s;
  if ((s = ensure(c, kBufVals, n * 4, &vals)) != HD_OK) return s;
  if ((s = ensure(c, kBufValsAlt, n * 4, &vals2)) != HD_OK) return s;
  if ((s = ensure(c, kBufSorted0, n * sizeof(float4), &pts)) != HD_OK) return s;
  if ((s = ensure(c, kBufCodes0, (leaves_a + leaves_b) * 2 * sizeof(float4), &lboxes)) != HD_OK)
    return s;
  // Fused: one sort of both sets (set in bit 30); else one sort per set,
  // each with its own temporary region.
  size_t tmp_bytes = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, (const uint32_t*) keys, (uint32_t*) keys2,
                                  (const uint32_t*) vals, (uint32_t*) vals2,
                                  (int64_t) (fused ? n : std::max(nA, nB)),
                                  fused ? kSortLowBitsFused : kSortLowBitsSplit, fused ? 31 : 30,
                                  c.stream);
  const size_t stride = (tmp_bytes + 255) & ~(size_t) 255;
  if ((s = ensure(c, kBufCubTemp, (fused ? 1 : 2) * stride, &tmp)) != HD_OK) return s;
  *x = SortScratch{(uint32_t*) keys, (uint32_t*) keys2, (uint32_t*) vals, (uint32_t*) vals2,
                   (unsigned char*) tmp, tmp_bytes, stride, (float4*) pts, (float4*) lboxes,
                   nA, leaves_a, L};
  return HD_OK;
}

// Sorts set k (0 = the call's A, 1 = its B) on stream st: bounding box, its
// frame, Morton codes, radix sort, gather with leaf boxes.
hd_status sort_set(Ctx& c, int k, const float* P, uint64_t n, int dims, const SortScratch& x,
                   cudaStream_t st, SortedSet* out) {
  hd_status s;
  const uint64_t base = k ? x.nA : 0;
  uint32_t* ord = &scalars(c, 0)->mbr_ord[k][0][0];
  Frame* fr = frame(c, k);
  {
    const int gx = grid_for(c, (n + 3) / 4, 256);
    k_mbr2<<<dim3(gx, 1), 256, 0, st>>>(P, n, P, n, dims, ord, ord);
    if ((s = after_launch(c, "mbr")) != HD_OK) return s;
  }
  k_frame<<<1, 32, 0, st>>>(ord, ord, dims, 1, 0, fr);
  if ((s = after_launch(c, "frame")) != HD_OK) return s;
  if (dims == 2)
    k_morton1<2><<<grid_for(c, n), 256, 0, st>>>(P, n, fr, x.keys + base, x.vals + base);
  else
    k_morton1<3><<<grid_for(c, n), 256, 0, st>>>(P, n, fr, x.keys + base, x.vals + base);
  if ((s = after_launch(c, "morton")) != HD_OK) return s;
  size_t tb = x.tmp_bytes;
  cudaError_t e = cub::DeviceRadixSort::SortPairs(
      x.tmp + (size_t) k * x.tmp_stride, tb, (const uint32_t*) x.keys + base, x.keys2 + base,
      (const uint32_t*) x.vals + base, x.vals2 + base, (int64_t) n, kSortLowBitsSplit, 30, st);
  if (e != cudaSuccess) return cuda_fail(c, e, "radix sort");
  float4* lb = x.lboxes + (k ? 2 * x.leaves_a : 0);
  k_gather1<<<grid_for(c, n), 256, 0, st>>>(P, n, dims, x.vals2 + base, x.pts + base, x.L, lb);
  if ((s = after_launch(c, "gather")) != HD_OK) return s;
  SortedSet& o = *out;
  o.pts = x.pts + base;
  o.codes = x.keys2 + base;
  o.frame = fr;
  o.leaf_boxes = lb;
  o.leaf_size = x.L;
  o.n = n;
  o.dims = dims;
  o.src = P;
  o.low_bits = kSortLowBitsSplit;
  o.mask = sorted_mask(kSortLowBitsSplit);
  return HD_OK;
}

}  // namespace

// Small sets: one fused chain (both boxes, one common frame, both sets'
// codes, one sort with the set in bit 30, both gathers), so a query set's
// Morton order matches the target's exactly and the launches are few.
static hd_status spatial_sort_fused(Ctx& c, const float* A, uint64_t nA, const float* B,
                                    uint64_t nB, int dims, SortedSet* sa, SortedSet* sb) {
  hd_status s;
  SortScratch x;
  if ((s = sort_scratch(c, nA, nB, true, &x)) != HD_OK) return s;
  DevScalars* sc = scalars(c, 0);
  {
    const int gx = grid_for(c, (std::max(nA, nB) + 3) / 4, 256);
    k_mbr2<<<dim3(gx, 2), 256, 0, c.stream>>>(A, nA, B, nB, dims, &sc->mbr_ord[0][0][0],
                                              &sc->mbr_ord[1][0][0]);
    if ((s = after_launch(c, "mbr")) != HD_OK) return s;
  }
  Frame* fr = frame(c, 0);
  k_frame<<<1, 32, 0, c.stream>>>(&sc->mbr_ord[0][0][0], &sc->mbr_ord[1][0][0], dims, 1, 1, fr);
  if ((s = after_launch(c, "frame")) != HD_OK) return s;
  {
    const int gx = grid_for(c, std::max(nA, nB));
    k_morton2<<<dim3(gx, 2), 256, 0, c.stream>>>(A, nA, B, nB, dims, fr, x.keys, x.vals);
    if ((s = after_launch(c, "morton")) != HD_OK) return s;
  }
  size_t tb = x.tmp_bytes;
  cudaError_t e = cub::DeviceRadixSort::SortPairs(x.tmp, tb, (const uint32_t*) x.keys, x.keys2,
                                                  (const uint32_t*) x.vals, x.vals2,
                                                  (int64_t) (nA + nB), kSortLowBitsFused, 31,
                                                  c.stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "radix sort");
  k_gather2<<<dim3(grid_for(c, std::max(nA, nB)), 2), 256, 0, c.stream>>>(
      A, nA, B, nB, dims, x.vals2, x.pts, x.L, x.lboxes, x.leaves_a);
  if ((s = after_launch(c, "gather")) != HD_OK) return s;
  const uint32_t mask = sorted_mask(kSortLowBitsFused);
  *sa = SortedSet{x.pts, x.keys2, fr, x.lboxes, x.L, nA, dims, A, kSortLowBitsFused, mask};
  *sb = SortedSet{x.pts + nA, x.keys2 + nA, fr, x.lboxes + 2 * x.leaves_a, x.L, nB, dims, B,
                  kSortLowBitsFused, mask};
  return HD_OK;
}

// Large sets: A's chain (own frame) on the main stream, B's on the side
// stream, joined before anything reads the sorted sets.
static hd_status spatial_sort(Ctx& c, const float* A, uint64_t nA, const float* B,
                              uint64_t nB, int dims, SortedSet* sa, SortedSet* sb) {
  if (nA + nB < kSplitMinPoints) return spatial_sort_fused(c, A, nA, B, nB, dims, sa, sb);
  hd_status s;
  SortScratch x;
  if ((s = sort_scratch(c, nA, nB, false, &x)) != HD_OK) return s;
  if ((s = ensure_side(c)) != HD_OK) return s;
  cudaError_t e;
  if ((e = cudaEventRecord(c.batch_fork, c.stream)) != cudaSuccess ||
      (e = cudaStreamWaitEvent(c.batch_side, c.batch_fork, 0)) != cudaSuccess)
    return cuda_fail(c, e, "fork");
  if ((s = sort_set(c, 0, A, nA, dims, x, c.stream, sa)) != HD_OK) return s;
  if ((s = sort_set(c, 1, B, nB, dims, x, c.batch_side, sb)) != HD_OK) return s;
  if ((e = cudaEventRecord(c.batch_join, c.batch_side)) != cudaSuccess ||
      (e = cudaStreamWaitEvent(c.stream, c.batch_join, 0)) != cudaSuccess)
    return cuda_fail(c, e, "join");
  return HD_OK;
}

hd_status spatial_upload_sort(Ctx& c, const float* hA, uint64_t nA, const float* hB, uint64_t nB,
                              int dims, const float** dA, const float** dB) {
  hd_status s;
  void *pa, *pb;
  if ((s = ensure(c, kBufA, (size_t) nA * dims * sizeof(float), &pa)) != HD_OK) return s;
  if ((s = ensure(c, kBufB, (size_t) nB * dims * sizeof(float), &pb)) != HD_OK) return s;
  SortScratch x;
  if ((s = sort_scratch(c, nA, nB, false, &x)) != HD_OK) return s;
  if ((s = ensure_side(c)) != HD_OK) return s;
  cudaError_t e;
  // A's copy first, alone on the link; B's copy starts when it is done and
  // runs beside A's sort.
  if ((e = cudaMemcpyAsync(pa, hA, (size_t) nA * dims * sizeof(float), cudaMemcpyHostToDevice,
                           c.stream)) != cudaSuccess)
    return cuda_fail(c, e, "copy inputs to device");
  if ((e = cudaEventRecord(c.batch_fork, c.stream)) != cudaSuccess ||
      (e = cudaStreamWaitEvent(c.batch_side, c.batch_fork, 0)) != cudaSuccess)
    return cuda_fail(c, e, "fork");
  if ((s = sort_set(c, 0, (const float*) pa, nA, dims, x, c.stream, &c.sorted[0])) != HD_OK)
    return s;
  if ((e = cudaMemcpyAsync(pb, hB, (size_t) nB * dims * sizeof(float), cudaMemcpyHostToDevice,
                           c.batch_side)) != cudaSuccess)
    return cuda_fail(c, e, "copy inputs to device");
  if ((s = sort_set(c, 1, (const float*) pb, nB, dims, x, c.batch_side, &c.sorted[1])) != HD_OK)
    return s;
  if ((e = cudaEventRecord(c.batch_join, c.batch_side)) != cudaSuccess ||
      (e = cudaStreamWaitEvent(c.stream, c.batch_join, 0)) != cudaSuccess)
    return cuda_fail(c, e, "join");
  c.sorted_valid = true;
  *dA = (const float*) pa;
  *dB = (const float*) pb;
  return HD_OK;
}

size_t scalars_bytes() { return 2 * sizeof(DevScalars) + 2 * sizeof(Frame); }

hd_status spatial_prepare(Ctx& c, const DirInput& in, const SortedSet** q,
                          const SortedSet** t) {
  if (!c.sorted_valid) {
    // Direction 0 of the call: A is the call's A.
    hd_status s = spatial_sort(c, in.A, in.nA, in.B, in.nB, in.dims, &c.sorted[0], &c.sorted[1]);
    if (s != HD_OK) return s;
    c.sorted_valid = true;
  }
  const SortedSet* x = (c.sorted[0].src == in.A && c.sorted[0].n == in.nA) ? &c.sorted[0]
                                                                            : &c.sorted[1];
  const SortedSet* y = (x == &c.sorted[0]) ? &c.sorted[1] : &c.sorted[0];
  if (x->src != in.A || y->src != in.B)
    return fail(c, HD_ERR_CUDA, "spatial cache does not match the directed input");
  *q = x;
  *t = y;
  return HD_OK;
}

hd_status make_sample(Ctx& c, uint64_t n, uint64_t seed, uint32_t* k_out, uint32_t** list) {
  double rate = c.opt.sample_rate > 0 ? c.opt.sample_rate : 0.01;
  uint64_t k = (uint64_t) std::ceil((double) n * rate);
  k = std::max<uint64_t>(k, std::min<uint64_t>(n, 1024));
  k = std::min<uint64_t>(k, 4096);
  void* p;
  hd_status s = ensure(c, kBufSample, k * 4, &p);
  if (s != HD_OK) return s;
  k_sample<<<(unsigned) ((k + 255) / 256), 256, 0, c.stream>>>(n, (uint32_t) k, seed,
                                                               (uint32_t*) p);
  if ((s = after_launch(c, "sample")) != HD_OK) return s;
  *k_out = (uint32_t) k;
  *list = (uint32_t*) p;
  return HD_OK;
}

}  // namespace hdg
