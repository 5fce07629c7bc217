// FP32 scans for any n_dims (the reference supports only 2 and 3,
// src/main.cpp:134-135; this path serves the high-dimensional workload and the
// plain all-pairs baseline of every workload).
//
// Layout: B is copied once into a visit-ordered array of rows padded with
// zeros to Dp floats (Dp = the next size in {4, 8, 16, 32, 64, 128, 256}).
// Zero padding leaves the FP32 squared distance unchanged: the padded terms
// are (0 - 0)^2 = +0 added after the real ones, and s + 0 == s.  Rows past
// |B| carry +inf in their first coordinate so they never win a minimum.
//
// k_nd_scan: one A row per thread (in registers), 128 rows per CTA; the CTA
// streams tiles of 32 B rows through a shared-memory double buffer with the
// TMA bulk-copy engine (cp.async.bulk + mbarrier) and every thread reads
// each B row as a shared-memory broadcast.  EB mode stops a row once its
// running minimum is at or below the running maximum and leaves the CTA's
// loop when every row has stopped; BRUTE mode scans all of B.  Squared
// distances use the reference formula (difference, square, left-to-right sum,
// no FMA), so results are exact FP32 max-min values.
#include <cfloat>

#include "hd_common.cuh"
#include "hd_internal.h"

namespace hdg {
namespace {

constexpr int kNdThreads = 128;
constexpr int kNdTileRows = 32;
constexpr uint32_t kNdWait = 1u << 26;

template <int Dp>
__global__ void k_nd_pack(const float* __restrict__ B, uint64_t nB, int D, Perm perm,
                          float* __restrict__ out, uint64_t nPad) {
  const uint64_t total = nPad * Dp;
  for (uint64_t t = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; t < total;
       t += (uint64_t) gridDim.x * blockDim.x) {
    const uint64_t j = t / Dp;
    const int k = (int) (t % Dp);
    float v;
    if (j < nB) {
      v = k < D ? B[perm(j) * D + k] : 0.0f;
    } else {
      v = k == 0 ? INFINITY : 0.0f;
    }
    out[t] = v;
  }
}

template <int Dp, bool EB>
__global__ void __launch_bounds__(kNdThreads)
    k_nd_scan(const float* __restrict__ A, uint64_t row_begin, uint64_t row_end, int D,
              Perm permA, const float* __restrict__ Bp, uint32_t nTiles, DevScalars* sc) {
  constexpr uint32_t kTileFloats = kNdTileRows * Dp;
  constexpr uint32_t kTileBytes = kTileFloats * 4;
  extern __shared__ __align__(128) float smem[];
  float* tile0 = smem;
  float* tile1 = smem + kTileFloats;
  __shared__ __align__(8) uint64_t full[2];
  __shared__ float s_thr;

  const int tid = threadIdx.x;
  const uint64_t row = row_begin + (uint64_t) blockIdx.x * kNdThreads + tid;
  bool active = row < row_end;
  uint32_t ia = 0;
  float a[Dp];
  if (active) ia = (uint32_t) permA(row);
  const float* arow = A + (uint64_t) ia * D;
#pragma unroll
  for (int k = 0; k < Dp; ++k) a[k] = (active && k < D) ? arow[k] : 0.0f;
  float cmin = INFINITY;
  if (tid == 0) {
    mbar_init(&full[0], 1);
    mbar_init(&full[1], 1);
    fence_barrier_init();
  }
  __syncthreads();
  // Every CTA starts at its own tile so that early-break CTAs sample
  // different parts of B first.
  uint32_t t = (uint32_t) (((uint64_t) blockIdx.x * 2654435761ull) % nTiles);
  if (tid == 0) {
    mbar_expect_tx(&full[0], kTileBytes);
    tma_load_1d(tile0, Bp + (uint64_t) t * kTileFloats, kTileBytes, &full[0]);
  }
  uint32_t i = 0;
  bool failed = false;
  for (; i < nTiles; ++i) {
    const int buf = i & 1;
    const uint32_t tn = (t + 1 == nTiles) ? 0 : t + 1;
    if (tid == 0 && i + 1 < nTiles) {
      mbar_expect_tx(&full[buf ^ 1], kTileBytes);
      tma_load_1d(buf ? tile0 : tile1, Bp + (uint64_t) tn * kTileFloats, kTileBytes,
                  &full[buf ^ 1]);
    }
    const bool ok = mbar_wait(&full[buf], (i >> 1) & 1, &sc->status, kNdWait);
    if (__syncthreads_or(!ok)) {
      failed = true;
      break;
    }
    const float4* tb = reinterpret_cast<const float4*>(buf ? tile1 : tile0);
    float m = cmin;
#pragma unroll 2
    for (int r = 0; r < kNdTileRows; ++r) {
      float s = 0.0f;
#pragma unroll
      for (int k4 = 0; k4 < Dp / 4; ++k4) {
        const float4 b = tb[r * (Dp / 4) + k4];
        const float d0 = __fsub_rn(a[4 * k4], b.x);
        const float d1 = __fsub_rn(a[4 * k4 + 1], b.y);
        const float d2 = __fsub_rn(a[4 * k4 + 2], b.z);
        const float d3 = __fsub_rn(a[4 * k4 + 3], b.w);
        s = k4 == 0 ? __fmul_rn(d0, d0) : __fadd_rn(s, __fmul_rn(d0, d0));
        s = __fadd_rn(s, __fmul_rn(d1, d1));
        s = __fadd_rn(s, __fmul_rn(d2, d2));
        s = __fadd_rn(s, __fmul_rn(d3, d3));
      }
      m = fminf(m, s);
    }
    if (active) cmin = m;
    t = tn;
    if (EB) {
      if (tid == 0) s_thr = threshold_of(ld_relaxed_u64(&sc->max_key));
      __syncthreads();
      if (active && cmin <= s_thr) active = false;
      if (!__syncthreads_or(active)) {
        ++i;
        break;
      }
    } else {
      __syncthreads();
    }
  }
  // The prefetch issued in the last iteration may still be in flight.
  if (tid == 0 && !failed && i < nTiles)
    mbar_wait(&full[i & 1], (i >> 1) & 1, &sc->status, kNdWait);
  if (active) atomicMax(&sc->max_key, pack_max(cmin, ia));
}

template <int Dp>
hd_status run_nd_dim(Ctx& c, const DirInput& in, bool eb) {
  const uint64_t nTiles64 = (in.nB + kNdTileRows - 1) / kNdTileRows;
  if (nTiles64 >= 0xFFFFFFFFull) return fail(c, HD_ERR_INVALID_ARG, "B too large");
  const uint32_t nTiles = (uint32_t) nTiles64;
  const uint64_t nPad = nTiles64 * kNdTileRows;
  void* pb;
  hd_status s;
  if ((s = ensure(c, kBufPackB, nPad * Dp * sizeof(float), &pb)) != HD_OK) return s;
  DevScalars* sc = scalars(c, in.dir);
  const uint64_t seed = c.opt.seed;
  Perm pB{in.nB, pick_multiplier(in.nB, seed + 1), (seed * 7919u) % in.nB};
  Perm pA{in.nA, eb ? pick_multiplier(in.nA, seed + 2) : 1, 0};
  {
    const uint64_t total = nPad * Dp;
    int grid = (int) std::min<uint64_t>((total + 255) / 256, (uint64_t) c.num_sms * 32);
    k_nd_pack<Dp><<<std::max(grid, 1), 256, 0, c.stream>>>(in.B, in.nB, in.dims, pB, (float*) pb,
                                                          nPad);
    if ((s = after_launch(c, "nd_pack")) != HD_OK) return s;
  }
  mark(c, 1);
  mark(c, 2);
  const size_t smem = 2 * kNdTileRows * Dp * sizeof(float);
  auto kern = eb ? k_nd_scan<Dp, true> : k_nd_scan<Dp, false>;
  cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
  // EB: a first wave of one CTA per SM completes and seeds the running
  // maximum before the remaining rows start.
  const uint64_t seed_rows = eb ? std::min<uint64_t>(in.nA, (uint64_t) c.num_sms * kNdThreads) : 0;
  if (seed_rows) {
    const unsigned blocks = (unsigned) ((seed_rows + kNdThreads - 1) / kNdThreads);
    kern<<<blocks, kNdThreads, smem, c.stream>>>(in.A, 0, seed_rows, in.dims, pA, (const float*) pb,
                                                 nTiles, sc);
    if ((s = after_launch(c, "nd_scan_seed")) != HD_OK) return s;
  }
  mark(c, 3);
  if (in.nA > seed_rows) {
    const unsigned blocks = (unsigned) ((in.nA - seed_rows + kNdThreads - 1) / kNdThreads);
    kern<<<blocks, kNdThreads, smem, c.stream>>>(in.A, seed_rows, in.nA, in.dims, pA,
                                                 (const float*) pb, nTiles, sc);
    if ((s = after_launch(c, "nd_scan")) != HD_OK) return s;
  }
  mark(c, 4);
  return certify(c, in);
}

hd_status run_nd(Ctx& c, const DirInput& in, bool eb) {
  const int d = in.dims;
  if (d <= 4) return run_nd_dim<4>(c, in, eb);
  if (d <= 8) return run_nd_dim<8>(c, in, eb);
  if (d <= 16) return run_nd_dim<16>(c, in, eb);
  if (d <= 32) return run_nd_dim<32>(c, in, eb);
  if (d <= 64) return run_nd_dim<64>(c, in, eb);
  if (d <= 128) return run_nd_dim<128>(c, in, eb);
  return fail(c, HD_ERR_UNSUPPORTED, "the FP32 scans support n_dims up to 128");
}

}  // namespace

hd_status run_brute(Ctx& c, const DirInput& in) { return run_nd(c, in, false); }

hd_status run_eb_nd(Ctx& c, const DirInput& in) { return run_nd(c, in, true); }

}  // namespace hdg
