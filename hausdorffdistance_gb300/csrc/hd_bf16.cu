// Split-BF16 tensor-core variant for high-dimensional inputs (n_dims a
// multiple of 16, up to 256).  No counterpart in the reference, which only
// handles n_dims 2 and 3 (src/main.cpp:134-135).
//
// ||a - b||^2 = ||a||^2 + ||b||^2 - 2 a.b.  Each coordinate is split into
// bf16 hi = bf16(x) and lo = bf16(x - hi); a.b is taken as
// hi.hi + hi.lo + lo.hi (three products, FP32 accumulation in tensor memory)
// by tcgen05.mma kind::f16 on sm_103a.  Per A row the epilogue keeps the
// approximate minimum over B of ||b||^2 - 2 a.b.  A rigorous per-row error
// bound E_i (split residuals, the dropped lo.lo product, FP32 accumulation
// and the FP32 rounding of the reference formula) then certifies the
// result: every row whose interval [m_i - E_i, m_i + E_i] can reach the
// largest lower bound max_j (m_j - E_j) is re-scanned exactly with the FP32
// reference formula, and the maximum over those rows is the exact FP32
// Hausdorff distance — bit-identical to the FP32 scans.  The certifying
// pair's distance is then recomputed in FP64 (certify()).
//
// Kernel shape (one CTA per 256 A rows = two 128-row regions, 6 warps, 1 CTA
// per SM):
//   warp 0      producer: TMA bulk copies (cp.async.bulk) of the A block once
//               and of B tiles (256 rows, hi+lo) into a 2-stage ring
//   warp 1      allocates 512 TMEM columns; one lane issues the MMAs:
//               per B tile and A region, 3 products x (Kp/16) MMAs of
//               M=128, N=256, K=16 into the region's 256-column FP32
//               accumulator (region r at columns r*256); the two regions
//               alternate, so one is computed while the other is read out
//   warps 2-5   epilogue: tcgen05.ld of the accumulator (one TMEM lane per
//               pair of A rows, one per region), min over the tile of
//               ||b||^2 - 2 acc
// N = 256 keeps the MMA's shared-memory operand reads (A 4 KB + B 8 KB per
// 128 x 256 x 16 step) below the SM's shared-memory bandwidth, which an
// N = 128 step (8 KB per half as many cycles) saturates; both A regions
// read every B tile, so each B tile is streamed from L2 once per 256 A rows.
// Operands are pre-packed in global memory in the no-swizzle K-major
// core-matrix layout (8 rows x 16 bytes per core matrix), so every tile is
// one contiguous bulk copy.  No TMA multicast.
#include <cuda_bf16.h>

#include <cfloat>
#include <cmath>

#include "hd_common.cuh"
#include "hd_internal.h"

namespace hdg {
namespace {

constexpr int kBM = 128;   // rows of one A region (UMMA M)
constexpr int kAM = 256;   // A rows per CTA: two 128-row regions sharing every B tile
constexpr int kBN = 256;   // B rows per tile (UMMA N)
constexpr int kStages = 2; // B tiles in flight (ring of shared-memory stages)
constexpr int kThreads = 192;
constexpr uint32_t kTmemCols = 512;
constexpr uint32_t kWaitLimit = 1u << 24;
// Dynamic shared memory per CTA: the A block (64 KB) and two B stages (64 KB
// each) at Kp = 64; smaller Kp use a prefix.
constexpr uint32_t kSmemBytes = 192 * 1024;

// Byte offset of element (row, k) inside one packed operand region of R rows:
// core matrix (chunk c = k/8, group g = row/8) at (c * R/8 + g) * 128 bytes,
// row row%8 at 16-byte stride, element k%8 at 2-byte stride.
__host__ __device__ __forceinline__ uint32_t pack_off(uint32_t row, uint32_t k, uint32_t R) {
  return ((k >> 3) * (R >> 3) + (row >> 3)) * 128u + (row & 7u) * 16u + (k & 7u) * 2u;
}

// One thread per (row, 8-element chunk): splits, writes hi and lo chunks.
// Tile t of rows [t*R, t*R+R) occupies 2 * R * Kp * 2 bytes: hi then lo.
__global__ void k_bf16_pack(const float* __restrict__ X, uint64_t n, int D, int Kp, int R,
                            uint64_t nPad, unsigned char* __restrict__ out,
                            float* __restrict__ norms, uint32_t* __restrict__ maxnorm_ord,
                            int pad_norm_inf) {
  const uint64_t chunks = (uint64_t) Kp / 8;
  const uint64_t total = nPad * chunks;
  for (uint64_t t = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; t < total;
       t += (uint64_t) gridDim.x * blockDim.x) {
    const uint64_t row = t / chunks;
    const uint32_t c = (uint32_t) (t % chunks);
    __align__(16) __nv_bfloat16 hi[8], lo[8];
    float part = 0.0f;
    for (int e = 0; e < 8; ++e) {
      const int k = (int) c * 8 + e;
      const float v = (row < n && k < D) ? X[row * D + k] : 0.0f;
      const __nv_bfloat16 h = __float2bfloat16_rn(v);
      const float r = v - __bfloat162float(h);
      hi[e] = h;
      lo[e] = __float2bfloat16_rn(r);
      part = fmaf(v, v, part);
    }
    const uint64_t tile = row / R;
    const uint32_t rr = (uint32_t) (row % R);
    unsigned char* base = out + tile * (uint64_t) (2 * R * Kp * 2);
    const uint32_t off = pack_off(rr, c * 8, (uint32_t) R);
    *reinterpret_cast<uint4*>(base + off) = *reinterpret_cast<const uint4*>(hi);
    *reinterpret_cast<uint4*>(base + (uint64_t) R * Kp * 2 + off) =
        *reinterpret_cast<const uint4*>(lo);
    // Row norm: reduce the chunk partials of one row (chunks of a row are
    // consecutive threads).
    atomicAdd(&norms[row], part);
  }
  (void) maxnorm_ord;
  (void) pad_norm_inf;
}

__global__ void k_bf16_norm_finish(float* __restrict__ norms, uint64_t n, uint64_t nPad,
                                   uint32_t* __restrict__ maxnorm_ord, int pad_inf) {
  uint32_t local = 0;
  for (uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < nPad;
       i += (uint64_t) gridDim.x * blockDim.x) {
    if (i < n) {
      local = max(local, f2ord(sqrtf(norms[i])));
    } else if (pad_inf) {
      norms[i] = INFINITY;  // padded B rows never win a minimum
    }
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) local = max(local, __shfl_xor_sync(0xFFFFFFFFu, local, o));
  if ((threadIdx.x & 31) == 0) atomicMax(maxnorm_ord, local);
}

// ---- tcgen05 / mbarrier helpers (inline PTX) --------------------------------

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t) __cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Shared-memory matrix descriptor, no swizzle, K-major.
__device__ __forceinline__ uint64_t make_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t) ((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t) ((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t) ((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t) 1 << 46;  // descriptor version for tcgen05
  // base offset 0, relative LBO mode, layout type 0 = no swizzle
  return d;
}

// Instruction descriptor: kind::f16, A = B = BF16, D = F32, both K-major,
// M = 128, N = 256.
__host__ __device__ constexpr uint32_t make_idesc() {
  return (1u << 4)                        // D format F32
         | (1u << 7)                      // A format BF16
         | (1u << 10)                     // B format BF16
         | ((uint32_t) (kBN >> 3) << 17)  // N >> 3
         | ((uint32_t) (kBM >> 4) << 24);  // M >> 4
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n"
      " setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(da), "l"(db), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}

// Named barrier over n threads that also returns whether any of them passed
// v = true (the same answer in every participating thread).
__device__ __forceinline__ bool bar_any(uint32_t id, uint32_t n, bool v) {
  uint32_t r;
  asm volatile(
      "{\n .reg .pred p, q;\n"
      " setp.ne.u32 q, %1, 0;\n"
      " bar.red.or.pred p, %2, %3, q;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(r)
      : "r"((uint32_t) v), "r"(id), "r"(n)
      : "memory");
  return r != 0;
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// Two 32-column loads, one wait.
__device__ __forceinline__ void tmem_ld32x2(uint32_t taddr, float* v) {
  uint32_t r[64];
#define HD_TMEM_LD32(OFF, BASE)                                                                 \
  asm volatile(                                                                                 \
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "                                                 \
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"                                 \
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"                \
      : "=r"(r[BASE + 0]), "=r"(r[BASE + 1]), "=r"(r[BASE + 2]), "=r"(r[BASE + 3]),             \
        "=r"(r[BASE + 4]), "=r"(r[BASE + 5]), "=r"(r[BASE + 6]), "=r"(r[BASE + 7]),             \
        "=r"(r[BASE + 8]), "=r"(r[BASE + 9]), "=r"(r[BASE + 10]), "=r"(r[BASE + 11]),           \
        "=r"(r[BASE + 12]), "=r"(r[BASE + 13]), "=r"(r[BASE + 14]), "=r"(r[BASE + 15]),         \
        "=r"(r[BASE + 16]), "=r"(r[BASE + 17]), "=r"(r[BASE + 18]), "=r"(r[BASE + 19]),         \
        "=r"(r[BASE + 20]), "=r"(r[BASE + 21]), "=r"(r[BASE + 22]), "=r"(r[BASE + 23]),         \
        "=r"(r[BASE + 24]), "=r"(r[BASE + 25]), "=r"(r[BASE + 26]), "=r"(r[BASE + 27]),         \
        "=r"(r[BASE + 28]), "=r"(r[BASE + 29]), "=r"(r[BASE + 30]), "=r"(r[BASE + 31])          \
      : "r"(taddr + (OFF)))
  HD_TMEM_LD32(0u, 0);
  HD_TMEM_LD32(32u, 32);
#undef HD_TMEM_LD32
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 64; ++i) v[i] = __uint_as_float(r[i]);
}

// Error bound on |approx - FP32 reference| squared distance for a row of norm
// a against rows of norm at most b, K = padded dimension.  Terms: the split
// residuals and the dropped lo.lo product (4 * 2^-18 |a||b|), FP32
// accumulation of 3K products with truncation allowed ((3K + 16) 2^-23
// |a||b|), the epilogue's FP32 additions (2^-21 (|a| + |b|)^2) and the
// reference formula's own rounding ((K + 2) 2^-24 (|a| + |b|)^2); doubled.
__device__ __forceinline__ double row_bound(double a, double b, int K) {
  const double c = 4.0 * ldexp(1.0, -18) + (3.0 * K + 16.0) * ldexp(1.0, -23);
  const double s = (a + b) * (a + b);
  const double e = 2.0 * c * a * b + ldexp(1.0, -21) * s + (K + 2.0) * ldexp(1.0, -24) * s;
  return 2.0 * e + 1e-30;
}

struct Bf16Scalars {
  uint32_t bmax_ord;   // max ||b|| (order-preserving bits)
  uint32_t lo_ord;     // max_i (m_i - E_i) (order-preserving bits)
  uint32_t cand;       // candidate count
  uint32_t status;
};

template <int Kp>
__global__ void __launch_bounds__(kThreads, 1)
    k_bf16_rowmin(const unsigned char* __restrict__ Apack, const unsigned char* __restrict__ Bpack,
                  const float* __restrict__ anorm, const float* __restrict__ bnorm, uint64_t nA,
                  uint32_t nTilesB, float* __restrict__ rowmin, Bf16Scalars* bs) {
  constexpr uint32_t kAReg = kBM * Kp * 2;   // bytes of one A region's hi (or lo) operand
  constexpr uint32_t kBReg = kBN * Kp * 2;   // bytes of one B tile's hi (or lo) operand
  constexpr uint32_t kABlock = 4 * kAReg;    // A block: (hi, lo) of region 0, then of region 1
  constexpr uint32_t kBTile = 2 * kBReg;     // B tile: hi, lo
  static_assert(kABlock + kStages * kBTile <= kSmemBytes, "operands exceed shared memory");
  static_assert(2 * kBN <= kTmemCols, "accumulators exceed the TMEM allocation");
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ __align__(8) uint64_t a_full, b_full[kStages], b_empty[kStages], acc_full[2],
      acc_empty[2];
  __shared__ uint32_t tmem_base;
  __shared__ __align__(16) float s_bn[2][kBN];

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  unsigned char* sA = smem;
  unsigned char* sB = smem + kABlock;

  if (threadIdx.x == 0) {
    mbar_init(&a_full, 1);
    for (int i = 0; i < kStages; ++i) {
      mbar_init(&b_full[i], 1);
      mbar_init(&b_empty[i], 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(&acc_full[i], 1);
      mbar_init(&acc_empty[i], 128);
    }
    fence_barrier_init();
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_base)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base;
  uint32_t* status = &bs->status;
  bool ok = true;

  if (warp == 0) {
    if (lane == 0) {
      mbar_expect_tx(&a_full, kABlock);
      tma_load_1d(sA, Apack + (uint64_t) blockIdx.x * kABlock, kABlock, &a_full);
      for (uint32_t t = 0; t < nTilesB && ok; ++t) {
        const uint32_t st = t % kStages;
        if (t >= kStages) ok = mbar_wait(&b_empty[st], ((t / kStages) - 1) & 1, status, kWaitLimit);
        if (!ok) break;
        mbar_expect_tx(&b_full[st], kBTile);
        tma_load_1d(sB + st * kBTile, Bpack + (uint64_t) t * kBTile, kBTile, &b_full[st]);
      }
      // Every issued copy must land before the CTA may exit: wait for the
      // MMAs of the last tile of every stage.
      const uint32_t first = nTilesB > (uint32_t) kStages ? nTilesB - kStages : 0;
      for (uint32_t t = first; t < nTilesB && ok; ++t)
        ok = mbar_wait(&b_empty[t % kStages], (t / kStages) & 1, status, kWaitLimit);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      constexpr uint32_t idesc = make_idesc();
      // K-major, no swizzle: LBO = next 8-element chunk along K (one column
      // of core matrices further: 16 of them in a 128-row A region, 32 in a
      // 256-row B tile), SBO = next 8-row group (one core matrix further).
      constexpr uint32_t kLboA = (kBM / 8) * 128u, kLboB = (kBN / 8) * 128u, kSbo = 128u;
      ok = mbar_wait(&a_full, 0, status, kWaitLimit);
      const uint32_t a0 = smem_u32(sA);
      for (uint32_t t = 0; t < nTilesB && ok; ++t) {
        const uint32_t st = t % kStages;
        ok = mbar_wait(&b_full[st], (t / kStages) & 1, status, kWaitLimit);
        if (!ok) break;
        const uint32_t b_hi = smem_u32(sB + st * kBTile), b_lo = b_hi + kBReg;
        // Region r's accumulator is free once the epilogue has read it for
        // tile t - 1; region 0's MMAs of tile t run while the epilogue still
        // reads region 1 of tile t - 1.
#pragma unroll
        for (int r = 0; r < 2 && ok; ++r) {
          if (t >= 1) ok = mbar_wait(&acc_empty[r], (t - 1) & 1, status, kWaitLimit);
          if (!ok) break;
          tc_fence_after();
          const uint32_t a_hi = a0 + (uint32_t) r * 2u * kAReg, a_lo = a_hi + kAReg;
          const uint32_t d = tmem + (uint32_t) r * kBN;
          uint32_t acc = 0;
#pragma unroll
          for (int prod = 0; prod < 3; ++prod) {
            const uint32_t ar = prod == 2 ? a_lo : a_hi;
            const uint32_t br = prod == 1 ? b_lo : b_hi;
#pragma unroll
            for (int s = 0; s < Kp / 16; ++s) {
              const uint64_t da = make_desc(ar + (uint32_t) s * 2u * kLboA, kLboA, kSbo);
              const uint64_t db = make_desc(br + (uint32_t) s * 2u * kLboB, kLboB, kSbo);
              mma_bf16(d, da, db, idesc, acc);
              acc = 1;
            }
          }
          mma_commit(&acc_full[r]);
        }
        if (ok) mma_commit(&b_empty[st]);
      }
    }
  } else {
    // Epilogue: warp w reads TMEM lanes [32 (w % 4), +32), one row of each A
    // region per thread.  ||b||^2 of a tile is fetched one tile ahead into
    // registers (its load latency hides behind the current tile) and staged
    // in shared memory; eight independent partial minima per row keep the
    // FP32 pipes busy.  A failed wait in any epilogue thread ends the loop in
    // all of them (bar_any).
    const int quad = warp & 3;
    const int etid = (warp - 2) * 32 + lane;  // 0..127
    const uint32_t lrow = (uint32_t) (quad * 32 + lane);
    const uint32_t tlane = (uint32_t) (quad * 32) << 16;
    float m8[2][8];
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
      for (int q = 0; q < 8; ++q) m8[r][q] = INFINITY;
    const float2* bn2 = reinterpret_cast<const float2*>(bnorm);
    float2 bn_next = nTilesB ? __ldg(bn2 + etid) : make_float2(0.0f, 0.0f);
    for (uint32_t t = 0; t < nTilesB && ok; ++t) {
      const int buf = t & 1;
      reinterpret_cast<float2*>(s_bn[buf])[etid] = bn_next;
      if (t + 1 < nTilesB) bn_next = __ldg(bn2 + (uint64_t) (t + 1) * (kBN / 2) + etid);
      const float4* bn4 = reinterpret_cast<const float4*>(s_bn[buf]);
#pragma unroll
      for (int r = 0; r < 2; ++r) {
        const bool got = mbar_wait(&acc_full[r], t & 1, status, kWaitLimit);
        // Also a barrier over the epilogue threads: this tile's norms are
        // written, and the reads of the buffer's previous contents (tile
        // t - 2) are done.
        if (bar_any(1, 128, !got)) {
          ok = false;
          break;
        }
        tc_fence_after();
#pragma unroll 1
        for (int cc = 0; cc < kBN / 64; ++cc) {
          float v[64];
          tmem_ld32x2(tmem + tlane + (uint32_t) r * kBN + cc * 64, v);
#pragma unroll
          for (int j4 = 0; j4 < 16; ++j4) {
            const float4 bn = bn4[cc * 16 + j4];
            const int q = (j4 & 1) * 4;
            m8[r][q + 0] = fminf(m8[r][q + 0], fmaf(-2.0f, v[4 * j4 + 0], bn.x));
            m8[r][q + 1] = fminf(m8[r][q + 1], fmaf(-2.0f, v[4 * j4 + 1], bn.y));
            m8[r][q + 2] = fminf(m8[r][q + 2], fmaf(-2.0f, v[4 * j4 + 2], bn.z));
            m8[r][q + 3] = fminf(m8[r][q + 3], fmaf(-2.0f, v[4 * j4 + 3], bn.w));
          }
        }
        tc_fence_before();
        mbar_arrive(&acc_empty[r]);
      }
    }
    if (ok) {
      const double bmax = (double) ord2f(bs->bmax_ord);
#pragma unroll
      for (int r = 0; r < 2; ++r) {
        float m = m8[r][0];
#pragma unroll
        for (int q = 1; q < 8; ++q) m = fminf(m, m8[r][q]);
        const uint64_t row = (uint64_t) blockIdx.x * kAM + (uint64_t) r * kBM + lrow;
        if (row < nA) {
          const float an = anorm[row];
          const float mi = an + m;
          rowmin[row] = mi;
          const double E = row_bound(sqrt((double) an), bmax, Kp);
          atomicMax(&bs->lo_ord, f2ord((float) ((double) mi - E)));
        }
      }
    }
  }
  // Every MMA of this CTA has completed once the epilogue consumed the last
  // accumulator (or the loops gave up); only then is TMEM released.
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 1) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(kTmemCols)
                 : "memory");
  }
}

__global__ void k_bf16_candidates(const float* __restrict__ rowmin, const float* __restrict__ anorm,
                                  uint64_t nA, int Kp, Bf16Scalars* bs, uint32_t* __restrict__ list) {
  const double L = (double) ord2f(bs->lo_ord);
  const double bmax = (double) ord2f(bs->bmax_ord);
  for (uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < nA;
       i += (uint64_t) gridDim.x * blockDim.x) {
    const double E = row_bound(sqrt((double) anorm[i]), bmax, Kp);
    if ((double) rowmin[i] + E >= L) {
      const uint32_t s = atomicAdd(&bs->cand, 1u);
      list[s] = (uint32_t) i;
    }
  }
}

// Exact FP32 re-scan of the candidate rows with the reference formula: every
// CTA takes a slice of B for one candidate (blockIdx.y strides over the
// candidates), and the slice minima meet in one atomicMin per CTA on the
// squared distance's bits (non-negative floats order like their bits).
__global__ void __launch_bounds__(256)
    k_bf16_recheck(const float* __restrict__ A, const float* __restrict__ B, uint64_t nB, int D,
                   const uint32_t* __restrict__ list, const Bf16Scalars* bs,
                   uint32_t* __restrict__ cand_min) {
  __shared__ __align__(16) float sa[256];
  __shared__ uint32_t red[8];
  const uint32_t n = bs->cand;
  const bool vec = (D % 4) == 0 && ((reinterpret_cast<uintptr_t>(B) & 15) == 0);
  for (uint32_t e = blockIdx.y; e < n; e += gridDim.y) {
    const uint32_t ia = list[e];
    __syncthreads();
    for (int k = threadIdx.x; k < D; k += blockDim.x) sa[k] = A[(uint64_t) ia * D + k];
    __syncthreads();
    float m = INFINITY;
    for (uint64_t j = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; j < nB;
         j += (uint64_t) gridDim.x * blockDim.x) {
      const float* br = B + j * D;
      float s = 0.0f;
      if (vec) {
        const float4* b4 = reinterpret_cast<const float4*>(br);
        for (int k4 = 0; k4 < D / 4; ++k4) {
          const float4 b = __ldg(b4 + k4);
          const float d0 = __fsub_rn(sa[4 * k4], b.x), d1 = __fsub_rn(sa[4 * k4 + 1], b.y);
          const float d2 = __fsub_rn(sa[4 * k4 + 2], b.z), d3 = __fsub_rn(sa[4 * k4 + 3], b.w);
          s = k4 == 0 ? __fmul_rn(d0, d0) : __fadd_rn(s, __fmul_rn(d0, d0));
          s = __fadd_rn(s, __fmul_rn(d1, d1));
          s = __fadd_rn(s, __fmul_rn(d2, d2));
          s = __fadd_rn(s, __fmul_rn(d3, d3));
        }
      } else {
        s = d2_n(sa, br, D);
      }
      m = fminf(m, s);
    }
    uint32_t u = __float_as_uint(m);
#pragma unroll
    for (int o = 16; o; o >>= 1) u = min(u, __shfl_xor_sync(0xFFFFFFFFu, u, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = u;
    __syncthreads();
    if (threadIdx.x == 0) {
      uint32_t b = red[0];
      for (int k = 1; k < 8; ++k) b = min(b, red[k]);
      atomicMin(&cand_min[e], b);
    }
  }
}

__global__ void k_bf16_recheck_final(const uint32_t* __restrict__ list, const Bf16Scalars* bs,
                                     const uint32_t* __restrict__ cand_min, DevScalars* sc) {
  const uint32_t n = bs->cand;
  for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x)
    atomicMax(&sc->max_key, pack_max(__uint_as_float(cand_min[e]), list[e]));
}

template <int Kp>
hd_status run_bf16_k(Ctx& c, const DirInput& in, DirResult* extra, float* rowmin_host) {
  hd_status s;
  const uint64_t nCta = (in.nA + kAM - 1) / kAM, nTB = (in.nB + kBN - 1) / kBN;
  if (nCta >= (1u << 31) || nTB >= 0xFFFFFFFFull) return fail(c, HD_ERR_INVALID_ARG, "too large");
  const uint64_t padA = nCta * kAM, padB = nTB * kBN;
  void *pa, *pb, *na, *nb, *rm, *cand, *bsv;
  if ((s = ensure(c, kBufBf16A, padA * Kp * 4, &pa)) != HD_OK) return s;
  if ((s = ensure(c, kBufBf16B, padB * Kp * 4, &pb)) != HD_OK) return s;
  if ((s = ensure(c, kBufNormsA, padA * 4, &na)) != HD_OK) return s;
  if ((s = ensure(c, kBufNormsB, padB * 4, &nb)) != HD_OK) return s;
  if ((s = ensure(c, kBufRowMin, padA * 4, &rm)) != HD_OK) return s;
  if ((s = ensure(c, kBufCand, in.nA * 8 + 128, &cand)) != HD_OK) return s;
  if ((s = ensure(c, kBufAux2, sizeof(Bf16Scalars), &bsv)) != HD_OK) return s;
  Bf16Scalars* bs = (Bf16Scalars*) bsv;
  cudaError_t e;
  if ((e = cudaMemsetAsync(na, 0, padA * 4, c.stream)) != cudaSuccess) return cuda_fail(c, e, "memset");
  if ((e = cudaMemsetAsync(nb, 0, padB * 4, c.stream)) != cudaSuccess) return cuda_fail(c, e, "memset");
  if ((e = cudaMemsetAsync(bs, 0, sizeof(Bf16Scalars), c.stream)) != cudaSuccess)
    return cuda_fail(c, e, "memset");
  const int g = c.num_sms * 16;
  k_bf16_pack<<<g, 256, 0, c.stream>>>(in.A, in.nA, in.dims, Kp, kBM, padA, (unsigned char*) pa,
                                       (float*) na, nullptr, 0);
  if ((s = after_launch(c, "bf16_pack_a")) != HD_OK) return s;
  k_bf16_pack<<<g, 256, 0, c.stream>>>(in.B, in.nB, in.dims, Kp, kBN, padB, (unsigned char*) pb,
                                       (float*) nb, nullptr, 0);
  if ((s = after_launch(c, "bf16_pack_b")) != HD_OK) return s;
  // A's norm maximum is not needed; B's gives the bound.
  k_bf16_norm_finish<<<c.num_sms * 4, 256, 0, c.stream>>>((float*) nb, in.nB, padB, &bs->bmax_ord, 1);
  if ((s = after_launch(c, "bf16_norms")) != HD_OK) return s;
  mark(c, 1);
  mark(c, 2);
  mark(c, 3);
  auto kern = k_bf16_rowmin<Kp>;
  cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) kSmemBytes);
  kern<<<(unsigned) nCta, kThreads, kSmemBytes, c.stream>>>(
      (const unsigned char*) pa, (const unsigned char*) pb, (const float*) na, (const float*) nb,
      in.nA, (uint32_t) nTB, (float*) rm, bs);
  if ((s = after_launch(c, "bf16_rowmin")) != HD_OK) return s;
  mark(c, 4);
  if (rowmin_host) {
    e = cudaMemcpyAsync(rowmin_host, rm, in.nA * 4, cudaMemcpyDeviceToHost, c.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "rowmin copy");
    Bf16Scalars h;
    e = cudaMemcpy(&h, bs, sizeof(h), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(c, e, "bf16 scalars");
    if (h.status) return fail(c, HD_ERR_DEVICE_TIMEOUT, "a bounded device wait ran out");
    return HD_OK;
  }
  k_bf16_candidates<<<c.num_sms * 4, 256, 0, c.stream>>>((const float*) rm, (const float*) na, in.nA,
                                                         Kp, bs, (uint32_t*) cand);
  if ((s = after_launch(c, "bf16_candidates")) != HD_OK) return s;
  DevScalars* sc = scalars(c, in.dir);
  // Candidate minima live after the candidate list (one uint per row of A).
  uint32_t* cand_min = (uint32_t*) cand + in.nA + 16;
  if ((e = cudaMemsetAsync(cand_min, 0xFF, in.nA * 4, c.stream)) != cudaSuccess)
    return cuda_fail(c, e, "memset");
  k_bf16_recheck<<<dim3(c.num_sms * 2, 16), 256, 0, c.stream>>>(in.A, in.B, in.nB, in.dims,
                                                               (const uint32_t*) cand, bs, cand_min);
  if ((s = after_launch(c, "bf16_recheck")) != HD_OK) return s;
  k_bf16_recheck_final<<<c.num_sms, 256, 0, c.stream>>>((const uint32_t*) cand, bs, cand_min, sc);
  if ((s = after_launch(c, "bf16_recheck_final")) != HD_OK) return s;
  // Bound and recheck statistics for the result (small copy, after the work).
  Bf16Scalars h;
  e = cudaMemcpyAsync(&h, bs, sizeof(h), cudaMemcpyDeviceToHost, c.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "bf16 scalars");
  if (h.status) {
    // Propagate a wait timeout to the solve's status word.
    e = cudaMemsetAsync(&sc->status, 0xFF, 1, c.stream);
    (void) e;
    return fail(c, HD_ERR_DEVICE_TIMEOUT, "a bounded device wait ran out in the BF16 kernel");
  }
  if (extra) {
    extra->rechecked = h.cand;
    // Report the bound of the largest-norm pair (||a|| ~ ||b|| ~ max ||b||).
    const double b = (double) ord2f(h.bmax_ord);
    const double cK = 4.0 * std::ldexp(1.0, -18) + (3.0 * Kp + 16.0) * std::ldexp(1.0, -23);
    const double sq = 4.0 * b * b;
    extra->err_bound = 2.0 * (2.0 * cK * b * b + std::ldexp(1.0, -21) * sq +
                              (Kp + 2.0) * std::ldexp(1.0, -24) * sq);
  }
  return certify(c, in);
}

hd_status run_bf16_impl(Ctx& c, const DirInput& in, DirResult* extra, float* rowmin_host) {
  if (in.dims % 16 != 0 || in.dims > 256)
    return fail(c, HD_ERR_UNSUPPORTED, "the BF16 variant needs n_dims % 16 == 0 and <= 256");
  switch (in.dims) {
  case 16: return run_bf16_k<16>(c, in, extra, rowmin_host);
  case 32: return run_bf16_k<32>(c, in, extra, rowmin_host);
  case 48: return run_bf16_k<48>(c, in, extra, rowmin_host);
  case 64: return run_bf16_k<64>(c, in, extra, rowmin_host);
  default: return fail(c, HD_ERR_UNSUPPORTED, "BF16 tiles are built for n_dims 16, 32, 48, 64");
  }
}

}  // namespace

hd_status run_bf16(Ctx& c, const DirInput& in, DirResult* extra) {
  return run_bf16_impl(c, in, extra, nullptr);
}

hd_status bf16_rowmin_debug(Ctx& c, const DirInput& in, float* rowmin_host) {
  return run_bf16_impl(c, in, nullptr, rowmin_host);
}

}  // namespace hdg
