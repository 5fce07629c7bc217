// Spatial preparation shared by the LBVH and grid variants: bounding boxes,
// cubic Morton frames, and the Morton sort of both sets into float4 (x, y, z,
// caller index) with leaf boxes (hd_msort.cu).  Both sets are sorted in
// shared launches; below kSplitMinPoints points they share one frame, above
// it each set has its own.  For host inputs A is copied and sorted while B is
// still being copied (two streams).
//
// Replaces the reference's MBR reduction (src/geoms/mbr.h:307-321: thrust
// for_each with CAS float atomics per point) and the first half of the grid
// build (src/index/uniform_grid.h:343-484: occupancy bitset, copy_if, sort,
// binary-search counting, atomic scatter): here the sort itself produces the
// cell order, because a cubic Morton frame makes every grid level a prefix of
// the code.
#include "hd_common.cuh"
#include "hd_internal.h"
#include "hd_msort.h"

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

// Buffers of both sets' sorts (set 1 after set 0 in every array), allocated
// before anything launches (an allocation may synchronise the device).
hd_status sort_buffers(Ctx& c, const float* A, uint64_t nA, const float* B, uint64_t nB,
                       MsortSets* ss) {
  const uint64_t n = nA + nB;
  uint32_t L = c.opt.leaf_size ? std::min<uint32_t>(c.opt.leaf_size, 32) : 16;
  while (L & (L - 1)) L &= L - 1;
  const uint64_t ns[2] = {nA, nB};
  uint32_t shift[2], nbins[2], caps[2];
  uint64_t leaves[2];
  for (int k = 0; k < 2; ++k) {
    shift[k] = msort_shift(ns[k]);
    nbins[k] = 1u << (30 - shift[k]);
    caps[k] = (uint32_t) (ns[k] / 33 + 2);
    leaves[k] = (ns[k] + L - 1) / L;
  }
  hd_status s;
  void *pts, *codes, *tpts, *tcodes, *bins, *aux, *lboxes;
  if ((s = ensure(c, kBufSorted0, n * sizeof(float4), &pts)) != HD_OK) return s;
  if ((s = ensure(c, kBufKeys, n * 4, &codes)) != HD_OK) return s;
  if ((s = ensure(c, kBufSorted1, n * sizeof(float4), &tpts)) != HD_OK) return s;
  if ((s = ensure(c, kBufKeysAlt, n * 4, &tcodes)) != HD_OK) return s;
  if ((s = ensure(c, kBufVals, ((uint64_t) nbins[0] + nbins[1]) * 4, &bins)) != HD_OK) return s;
  const uint64_t tiles = 1024 + 1;
  const uint64_t aux_words = 2 * tiles + 2 * ((uint64_t) caps[0] + caps[1]) + 8;
  if ((s = ensure(c, kBufValsAlt, aux_words * 4, &aux)) != HD_OK) return s;
  if ((s = ensure(c, kBufCodes0, (leaves[0] + leaves[1]) * 2 * sizeof(float4), &lboxes)) != HD_OK)
    return s;
  uint32_t* w = (uint32_t*) aux;
  uint32_t* counters = w;  // 4 words per set
  w += 8;
  uint64_t off = 0, boff = 0, loff = 0;
  const float* P[2] = {A, B};
  for (int k = 0; k < 2; ++k) {
    MsortSet& m = ss->s[k];
    m.P = P[k];
    m.n = ns[k];
    m.fr = frame(c, k);
    m.shift = shift[k];
    m.nbins = nbins[k];
    m.bins = (uint32_t*) bins + boff;
    m.tile_sums = w;
    w += tiles;
    m.pts = (float4*) pts + off;
    m.codes = (uint32_t*) codes + off;
    m.tpts = (float4*) tpts + off;
    m.tcodes = (uint32_t*) tcodes + off;
    m.mid_list = w;
    w += caps[k];
    m.big_list = w;
    w += caps[k];
    m.counters = counters + 4 * k;
    m.status = &scalars(c, 0)->status;
    m.list_cap = caps[k];
    m.L = L;
    m.leaf_boxes = (float4*) lboxes + 2 * loff;
    off += ns[k];
    boff += nbins[k];
    loff += leaves[k];
  }
  return HD_OK;
}

SortedSet sorted_of(const MsortSet& m, int dims) {
  SortedSet o;
  o.pts = m.pts;
  o.codes = m.codes;
  o.frame = m.fr;
  o.leaf_boxes = m.leaf_boxes;
  o.leaf_size = m.L;
  o.n = m.n;
  o.dims = dims;
  o.src = m.P;
  return o;
}

// Bounding box and frame of set k on stream st (its own frame).
hd_status frame_one(Ctx& c, int k, const float* P, uint64_t n, int dims, cudaStream_t st) {
  hd_status s;
  uint32_t* ord = &scalars(c, 0)->mbr_ord[k][0][0];
  const int gx = grid_for(c, (n + 3) / 4, 256);
  k_mbr2<<<dim3(gx, 1), 256, 0, st>>>(P, n, P, n, dims, ord, ord);
  if ((s = after_launch(c, "mbr")) != HD_OK) return s;
  k_frame<<<1, 32, 0, st>>>(ord, ord, dims, 1, 0, frame(c, k));
  return after_launch(c, "frame");
}

}  // namespace

// Sorts both sets in shared launches.  Below kSplitMinPoints points the two
// sets share one cubic frame (a query set's Morton order then matches the
// target's exactly); from there on each set has its own frame.
static hd_status spatial_sort(Ctx& c, const float* A, uint64_t nA, const float* B, uint64_t nB,
                              int dims, SortedSet* sa, SortedSet* sb) {
  hd_status s;
  MsortSets ss;
  if ((s = sort_buffers(c, A, nA, B, nB, &ss)) != HD_OK) return s;
  DevScalars* sc = scalars(c, 0);
  {
    const int gx = grid_for(c, (std::max(nA, nB) + 3) / 4, 256);
    k_mbr2<<<dim3(gx, 2), 256, 0, c.stream>>>(A, nA, B, nB, dims, &sc->mbr_ord[0][0][0],
                                              &sc->mbr_ord[1][0][0]);
    if ((s = after_launch(c, "mbr")) != HD_OK) return s;
  }
  if (nA + nB < kSplitMinPoints) {
    k_frame<<<1, 32, 0, c.stream>>>(&sc->mbr_ord[0][0][0], &sc->mbr_ord[1][0][0], dims, 1, 1,
                                    frame(c, 0));
    if ((s = after_launch(c, "frame")) != HD_OK) return s;
    ss.s[1].fr = frame(c, 0);
  } else {
    for (int k = 0; k < 2; ++k) {
      k_frame<<<1, 32, 0, c.stream>>>(&sc->mbr_ord[k][0][0], &sc->mbr_ord[k][0][0], dims, 1, 0,
                                      frame(c, k));
      if ((s = after_launch(c, "frame")) != HD_OK) return s;
    }
  }
  if ((s = msort_run(c, ss, 2, dims, c.stream)) != HD_OK) return s;
  *sa = sorted_of(ss.s[0], dims);
  *sb = sorted_of(ss.s[1], dims);
  return HD_OK;
}

hd_status spatial_upload_sort(Ctx& c, const float* hA, uint64_t nA, const float* hB, uint64_t nB,
                              int dims, const float** dA, const float** dB) {
  hd_status s;
  void *pa, *pb;
  if ((s = ensure(c, kBufA, (size_t) nA * dims * sizeof(float), &pa)) != HD_OK) return s;
  if ((s = ensure(c, kBufB, (size_t) nB * dims * sizeof(float), &pb)) != HD_OK) return s;
  MsortSets ss;
  if ((s = sort_buffers(c, (const float*) pa, nA, (const float*) pb, nB, &ss)) != HD_OK) return s;
  if ((s = ensure_side(c)) != HD_OK) return s;
  cudaError_t e;
  // A's copy first, alone on the link; B's copy starts when it is done and
  // runs beside A's sort (each set in its own frame).
  if ((e = cudaMemcpyAsync(pa, hA, (size_t) nA * dims * sizeof(float), cudaMemcpyHostToDevice,
                           c.stream)) != cudaSuccess)
    return cuda_fail(c, e, "copy inputs to device");
  if ((e = cudaEventRecord(c.batch_fork, c.stream)) != cudaSuccess ||
      (e = cudaStreamWaitEvent(c.batch_side, c.batch_fork, 0)) != cudaSuccess)
    return cuda_fail(c, e, "fork");
  MsortSets one;
  one.s[0] = ss.s[0];
  if ((s = frame_one(c, 0, (const float*) pa, nA, dims, c.stream)) != HD_OK) return s;
  if ((s = msort_run(c, one, 1, dims, c.stream)) != HD_OK) return s;
  if ((e = cudaMemcpyAsync(pb, hB, (size_t) nB * dims * sizeof(float), cudaMemcpyHostToDevice,
                           c.batch_side)) != cudaSuccess)
    return cuda_fail(c, e, "copy inputs to device");
  one.s[0] = ss.s[1];
  if ((s = frame_one(c, 1, (const float*) pb, nB, dims, c.batch_side)) != HD_OK) return s;
  if ((s = msort_run(c, one, 1, dims, c.batch_side)) != HD_OK) return s;
  if ((e = cudaEventRecord(c.batch_join, c.batch_side)) != cudaSuccess ||
      (e = cudaStreamWaitEvent(c.stream, c.batch_join, 0)) != cudaSuccess)
    return cuda_fail(c, e, "join");
  c.sorted[0] = sorted_of(ss.s[0], dims);
  c.sorted[1] = sorted_of(ss.s[1], dims);
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
