// CPU early-break Hausdorff distance: hd_exec's -execution cpu, and the
// independent answer of its -check (the reference re-runs its CPU
// early-break for -check, src/run_hausdorff_distance.cu:366-389).
//
// The algorithm is the reference's CPU path
// (HausdorffDistanceEarlyBreak::CalculateDistance,
// src/hd_impl/hausdorff_distance_early_break.h:44-115): both sets shuffled
// with one std::mt19937(seed) (A first, then B), A split into one contiguous
// slice per thread, each A point scanning B in order until its running minimum
// drops strictly below the shared running maximum, which rises by a
// compare-and-swap.  Squared distances are formed as the reference forms them
// (per-dimension difference, squared, summed left to right in the coordinate
// type: float, or double for -is_double); the driver is built with
// -ffp-contract=off so that no multiply-add is fused.  Rows of any n_dims are
// accepted.  This is an explicit execution mode of the driver, never a
// fallback of the GPU path.
#pragma once

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <numeric>
#include <random>
#include <thread>
#include <vector>

namespace hd {

struct CpuEarlyBreakResult {
  double distance = 0.0;      // directed h(A, B) (a float value for float rows)
  uint64_t compared_pairs = 0;
  double shuffle_ms = 0.0;
  double compute_ms = 0.0;    // the reference's ReportedTime
};

template <typename T>
inline T SquaredDistance(const T* a, const T* b, int dims) {
  T s = 0;
  for (int k = 0; k < dims; ++k) {
    const T d = a[k] - b[k];
    const T sq = d * d;
    s = k == 0 ? sq : s + sq;
  }
  return s;
}

// Directed h(A, B) of n_a x dims and n_b x dims row-major points (copied,
// never modified).
template <typename T>
inline CpuEarlyBreakResult CpuEarlyBreak(const T* A, uint64_t n_a, const T* B, uint64_t n_b,
                                         int dims, uint32_t seed, unsigned n_threads) {
  CpuEarlyBreakResult r;
  const auto t0 = std::chrono::steady_clock::now();
  // Shuffling row indices with the engine's swap sequence moves the rows as
  // shuffling the rows themselves would.
  std::mt19937 engine(seed);
  std::vector<uint64_t> ra(n_a), rb(n_b);
  std::iota(ra.begin(), ra.end(), uint64_t{0});
  std::iota(rb.begin(), rb.end(), uint64_t{0});
  std::shuffle(ra.begin(), ra.end(), engine);
  std::shuffle(rb.begin(), rb.end(), engine);
  std::vector<T> a(n_a * dims), b(n_b * dims);
  for (uint64_t i = 0; i < n_a; ++i) std::memcpy(&a[i * dims], A + ra[i] * dims, sizeof(T) * dims);
  for (uint64_t j = 0; j < n_b; ++j) std::memcpy(&b[j * dims], B + rb[j] * dims, sizeof(T) * dims);
  const auto t1 = std::chrono::steady_clock::now();

  const unsigned nt = std::max(1u, n_threads);
  const uint64_t per = (n_a + nt - 1) / nt;
  std::atomic<T> cmax2{T(0)};
  std::atomic<uint64_t> compared{0};
  auto work = [&](unsigned t) {
    const uint64_t begin = std::min<uint64_t>(n_a, (uint64_t) t * per);
    const uint64_t end = std::min<uint64_t>(n_a, begin + per);
    uint64_t local = 0;
    for (uint64_t i = begin; i < end; ++i) {
      T cmin2 = std::numeric_limits<T>::max();
      const T* p = &a[i * dims];
      for (uint64_t j = 0; j < n_b; ++j) {
        const T d = SquaredDistance(p, &b[j * dims], dims);
        ++local;
        if (d < cmin2) cmin2 = d;
        if (cmin2 < cmax2.load(std::memory_order_relaxed)) break;
      }
      if (cmin2 != std::numeric_limits<T>::max()) {
        T prev = cmax2.load();
        while (prev < cmin2 && !cmax2.compare_exchange_weak(prev, cmin2)) {
        }
      }
    }
    compared += local;
  };
  if (nt == 1) {
    work(0);
  } else {
    std::vector<std::thread> pool;
    for (unsigned t = 0; t < nt; ++t) pool.emplace_back(work, t);
    for (auto& th : pool) th.join();
  }
  const auto t2 = std::chrono::steady_clock::now();
  r.distance = (double) std::sqrt(cmax2.load());
  r.compared_pairs = compared.load();
  r.shuffle_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
  r.compute_ms = std::chrono::duration<double, std::milli>(t2 - t1).count();
  return r;
}

}  // namespace hd
