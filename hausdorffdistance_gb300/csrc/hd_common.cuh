// Shared device helpers for the sm_103a Hausdorff kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <cfloat>

namespace hdg {

constexpr uint32_t kInvalid = 0xFFFFFFFFu;

// Squared distance formed exactly as the reference forms it
// (src/geoms/distance.h:17-24, built with --fmad=false): per-dimension
// difference, squared, summed left to right.  The _rn intrinsics are never
// contracted into FMAs, whatever the -fmad setting of the translation unit.
__device__ __forceinline__ float d2_2(float ax, float ay, float bx, float by) {
  float dx = __fsub_rn(ax, bx);
  float dy = __fsub_rn(ay, by);
  return __fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy));
}

__device__ __forceinline__ float d2_3(float ax, float ay, float az, float bx,
                                      float by, float bz) {
  float dx = __fsub_rn(ax, bx);
  float dy = __fsub_rn(ay, by);
  float dz = __fsub_rn(az, bz);
  return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)),
                   __fmul_rn(dz, dz));
}

// Two FP32 differences a - b in one packed instruction: fma(b, -1, a) has an
// exact product, so its single rounding gives exactly __fsub_rn(a, b) per
// component (signed zeros included); __ffma2_rn / __fmul2_rn round each
// component like __fmaf_rn / __fmul_rn.
__device__ __forceinline__ float2 sub2_rn(float2 a, float2 b) {
  return __ffma2_rn(b, make_float2(-1.0f, -1.0f), a);
}

// The same squared distance of two float4 points, bit for bit, with x and y
// through the packed pair forms: fewer issue slots where both points already
// sit in registers as float4 (the LBVH leaf scans); with scattered scalar
// operands the packing moves cost more than they save.
template <int D>
__device__ __forceinline__ float d2_pt_packed(const float4& a, const float4& b) {
  const float2 d = sub2_rn(make_float2(a.x, a.y), make_float2(b.x, b.y));
  const float2 p = __fmul2_rn(d, d);
  if constexpr (D == 2) {
    return __fadd_rn(p.x, p.y);
  } else {
    const float dz = __fsub_rn(a.z, b.z);
    return __fadd_rn(__fadd_rn(p.x, p.y), __fmul_rn(dz, dz));
  }
}

template <int D>
__device__ __forceinline__ float d2_pt(const float4& a, const float4& b) {
  if constexpr (D == 2) {
    return d2_2(a.x, a.y, b.x, b.y);
  } else {
    return d2_3(a.x, a.y, a.z, b.x, b.y, b.z);
  }
}

// Generic n-dimensional FP32 squared distance, same summation order.
__device__ __forceinline__ float d2_n(const float* a, const float* b, int d) {
  float s = 0.0f;
  for (int k = 0; k < d; ++k) {
    float t = __fsub_rn(a[k], b[k]);
    float q = __fmul_rn(t, t);
    s = (k == 0) ? q : __fadd_rn(s, q);
  }
  return s;
}

// The running maximum is kept as one 64-bit word: the squared distance's bit
// pattern (non-negative floats order like their bit patterns) in the high
// half and the complement of the A index in the low half, so a single
// atomicMax keeps the largest distance and, among equal distances, the
// lowest index.  0 means "no point completed yet".
__device__ __forceinline__ unsigned long long pack_max(float d2, uint32_t ia) {
  return ((unsigned long long) __float_as_uint(d2) << 32) |
         (unsigned long long) (kInvalid - ia);
}
__host__ __device__ __forceinline__ uint32_t unpack_max_index(unsigned long long k) {
  return kInvalid - (uint32_t) (k & 0xFFFFFFFFull);
}

// Threshold that lets a point stop early: its running minimum at or below
// the current maximum.  -1 while no point has completed.
__device__ __forceinline__ float threshold_of(unsigned long long key) {
  return key ? __uint_as_float((uint32_t) (key >> 32)) : -1.0f;
}

__device__ __forceinline__ unsigned long long ld_relaxed_u64(
    const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p));
  return v;
}

// Minimum with index, packed for atomicMin: distance bits high, index low.
__device__ __forceinline__ unsigned long long pack_min(float d2, uint32_t ib) {
  return ((unsigned long long) __float_as_uint(d2) << 32) | ib;
}

// Order-preserving float <-> uint for atomic min/max of signed floats.
__device__ __forceinline__ uint32_t f2ord(float f) {
  uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__host__ __device__ __forceinline__ float ord2f(uint32_t u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
#else
  uint32_t v = (u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u;
  float f;
  __builtin_memcpy(&f, &v, 4);
  return f;
#endif
}

// Visit-order permutation j -> (j * mul + add) mod n, a bijection because
// gcd(mul, n) == 1.  It stands in for the reference's thrust::shuffle of the
// inputs (early_break.h:132-136): with mul near n/phi consecutive visits are
// spread over the whole index range, which is what early break needs.
struct Perm {
  uint64_t n, mul, add;
  __host__ __device__ __forceinline__ uint64_t operator()(uint64_t j) const {
    return (j * mul + add) % n;
  }
};

// Error bits written to the context's device status word.
enum : uint32_t {
  kErrWaitTimeout = 1u,   // an mbarrier / flag wait hit its iteration cap
  kErrQueueOverflow = 2u, // a device queue ran past its capacity
  kErrInternal = 4u
};

// Bounded mbarrier wait: returns false (and records kErrWaitTimeout) after
// `limit` polls instead of spinning forever.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity,
                                          uint32_t* status, uint32_t limit) {
  uint32_t addr = (uint32_t) __cvta_generic_to_shared(bar);
  for (uint32_t it = 0; it < limit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n"
        " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(addr), "r"(parity)
        : "memory");
    if (done) return true;
  }
  atomicOr(status, kErrWaitTimeout);
  return false;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  uint32_t addr = (uint32_t) __cvta_generic_to_shared(bar);
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(addr), "r"(count)
               : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  uint32_t addr = (uint32_t) __cvta_generic_to_shared(bar);
  asm volatile(
      "mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(addr),
      "r"(bytes)
      : "memory");
}

__device__ __forceinline__ void fence_barrier_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// 1-D bulk copy global -> shared through the TMA engine, completing on an
// mbarrier.  dst, src 16-byte aligned; bytes a multiple of 16.
__device__ __forceinline__ void tma_load_1d(void* dst_smem, const void* src,
                                            uint32_t bytes, uint64_t* bar) {
  uint32_t d = (uint32_t) __cvta_generic_to_shared(dst_smem);
  uint32_t b = (uint32_t) __cvta_generic_to_shared(bar);
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes "
      "[%0], [%1], %2, [%3];" ::"r"(d),
      "l"(src), "r"(bytes), "r"(b)
      : "memory");
}

}  // namespace hdg
