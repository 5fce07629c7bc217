// Spatial preparation shared by the LBVH and grid variants: one fused pass
// for both bounding boxes, Morton codes in a common cubic frame, a radix sort
// per set, and a gather into Morton order as float4 (x, y, z, caller index).
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

// Bounding boxes of both sets in one launch (blockIdx.y = set): per-thread
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
  // 30-bit codes in both cases, leaving bit 30 for the set when both sets
  // are sorted together.
  const int bits = dims == 2 ? 15 : 10;
  fr->bits = bits;
  fr->dims = dims;
  fr->extent = ext;
  // Cubic frame: one scale for every axis so that Morton levels are cubes.
  fr->scale = ext > 0.0f ? (float) ((1u << bits) - 1) / ext : 0.0f;
}

__device__ __forceinline__ uint32_t spread2(uint32_t x) {  // 16 bits -> even bits
  x &= 0xFFFFu;
  x = (x | (x << 8)) & 0x00FF00FFu;
  x = (x | (x << 4)) & 0x0F0F0F0Fu;
  x = (x | (x << 2)) & 0x33333333u;
  x = (x | (x << 1)) & 0x55555555u;
  return x;
}
__device__ __forceinline__ uint32_t spread3(uint32_t x) {  // 10 bits -> every 3rd bit
  x &= 0x3FFu;
  x = (x | (x << 16)) & 0x030000FFu;
  x = (x | (x << 8)) & 0x0300F00Fu;
  x = (x | (x << 4)) & 0x030C30C3u;
  x = (x | (x << 2)) & 0x09249249u;
  return x;
}

__device__ __forceinline__ uint32_t quant(float v, float lo, float scale, uint32_t maxq) {
  float q = (v - lo) * scale;
  q = fminf(fmaxf(q, 0.0f), (float) maxq);
  return (uint32_t) q;
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
      code = spread2(quant(P[2 * i], lo0, s, maxq)) |
             (spread2(quant(P[2 * i + 1], lo1, s, maxq)) << 1);
    } else {
      code = spread3(quant(P[3 * i], lo0, s, maxq)) |
             (spread3(quant(P[3 * i + 1], lo1, s, maxq)) << 1) |
             (spread3(quant(P[3 * i + 2], lo2, s, maxq)) << 2);
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

Frame* frame(Ctx& c) {
  return reinterpret_cast<Frame*>(reinterpret_cast<DevScalars*>(c.bufs[kBufScalars].p) + 2);
}

static hd_status spatial_sort(Ctx& c, const float* A, uint64_t nA, const float* B,
                              uint64_t nB, int dims, SortedSet* sa, SortedSet* sb) {
  const bool need_a = true, need_b = true;
  hd_status s;
  DevScalars* sc = scalars(c, 0);
  // One bounding box per set (both boxes feed the common frame).
  {
    const int gx = grid_for(c, (std::max(nA, nB) + 3) / 4, 256);
    k_mbr2<<<dim3(gx, 2), 256, 0, c.stream>>>(A, nA, B, nB, dims, &sc->mbr_ord[0][0][0],
                                              &sc->mbr_ord[1][0][0]);
    if ((s = after_launch(c, "mbr")) != HD_OK) return s;
  }
  k_frame<<<1, 32, 0, c.stream>>>(&sc->mbr_ord[0][0][0], &sc->mbr_ord[1][0][0], dims, 1, 1,
                                  frame(c));
  if ((s = after_launch(c, "frame")) != HD_OK) return s;

  // One sort of both sets: key = 30-bit code | set << 30, value = global row.
  const uint64_t n = nA + nB;
  uint32_t L = c.opt.leaf_size ? std::min<uint32_t>(c.opt.leaf_size, 32) : 16;
  while (L & (L - 1)) L &= L - 1;
  const uint64_t leaves_a = (nA + L - 1) / L, leaves_b = (nB + L - 1) / L;
  void *keys, *keys2, *vals, *vals2, *tmp, *pts, *lboxes;
  if ((s = ensure(c, kBufKeys, n * 4, &keys)) != HD_OK) return s;
  if ((s = ensure(c, kBufKeysAlt, n * 4, &keys2)) != HD_OK) return s;
  if ((s = ensure(c, kBufVals, n * 4, &vals)) != HD_OK) return s;
  if ((s = ensure(c, kBufValsAlt, n * 4, &vals2)) != HD_OK) return s;
  if ((s = ensure(c, kBufSorted0, n * sizeof(float4), &pts)) != HD_OK) return s;
  if ((s = ensure(c, kBufCodes0, (leaves_a + leaves_b) * 2 * sizeof(float4), &lboxes)) != HD_OK)
    return s;
  size_t tmp_bytes = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, (const uint32_t*) keys, (uint32_t*) keys2,
                                  (const uint32_t*) vals, (uint32_t*) vals2, (int64_t) n, 0, 31,
                                  c.stream);
  if ((s = ensure(c, kBufCubTemp, tmp_bytes, &tmp)) != HD_OK) return s;
  {
    const int gx = grid_for(c, std::max(nA, nB));
    k_morton2<<<dim3(gx, 2), 256, 0, c.stream>>>(A, nA, B, nB, dims, frame(c), (uint32_t*) keys,
                                                (uint32_t*) vals);
    if ((s = after_launch(c, "morton")) != HD_OK) return s;
  }
  size_t tb = tmp_bytes;
  cudaError_t e = cub::DeviceRadixSort::SortPairs(tmp, tb, (const uint32_t*) keys,
                                                  (uint32_t*) keys2, (const uint32_t*) vals,
                                                  (uint32_t*) vals2, (int64_t) n, 0, 31, c.stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "radix sort");
  k_gather2<<<dim3(grid_for(c, std::max(nA, nB)), 2), 256, 0, c.stream>>>(
      A, nA, B, nB, dims, (const uint32_t*) vals2, (float4*) pts, L, (float4*) lboxes, leaves_a);
  if ((s = after_launch(c, "gather")) != HD_OK) return s;
  *sa = SortedSet{(float4*) pts, (uint32_t*) keys2, (float4*) lboxes, L, nA, dims, A};
  *sb = SortedSet{(float4*) pts + nA, (uint32_t*) keys2 + nA, (float4*) lboxes + 2 * leaves_a, L,
                  nB, dims, B};
  (void) need_a;
  (void) need_b;
  return HD_OK;
}

size_t scalars_bytes() { return 2 * sizeof(DevScalars) + sizeof(Frame); }

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
