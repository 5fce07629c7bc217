// C++ mirror of the reference's algorithm seam
// hd::HausdorffDistance<COORD_T,N_DIMS> (src/hausdorff_distance.h:15-43) over
// libhdgpu.so's C ABI (include/hd_gpu.h).  Same class names for the variants
// the engine provides, same CalculateDistance(points_a, points_b) call and
// the same required stats keys ("Algorithm", "Execution", "ReportedTime").
// COORD_T float solves through hd_solve; COORD_T double through hd_solve_f64
// (the reference's double instantiation, which its driver leaves disabled,
// src/run_hausdorff_distance.cu:56-62).  Differences: the inputs are never
// permuted, errors throw hd::Error with the library's status instead of
// aborting, and every class runs on the GPU.
#pragma once
#include <cstdint>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "hd_gpu.h"
#include "json.h"

namespace hd {

template <int N, typename T = float>
struct Point {
  T c[N];
};

class Error : public std::runtime_error {
 public:
  Error(hd_status s, const std::string& msg)
      : std::runtime_error(std::string(hd_status_string(s)) + ": " + msg), status(s) {}
  hd_status status;
};

template <typename COORD_T, int N_DIMS>
class HausdorffDistance {
 public:
  static_assert(std::is_same<COORD_T, float>::value || std::is_same<COORD_T, double>::value,
                "coordinates are float or double");
  using point_t = Point<N_DIMS, COORD_T>;

  HausdorffDistance(int variant, const hd_options* opt, const char* algorithm)
      : algorithm_(algorithm) {
    hd_options o;
    if (opt)
      o = *opt;
    else
      hd_default_options(&o);
    o.variant = variant;
    hd_status s = hd_create(&ctx_, &o);
    if (s != HD_OK) throw Error(s, "cannot create a context (no sm_103a device?)");
  }
  virtual ~HausdorffDistance() {
    if (ctx_) hd_destroy(ctx_);
  }
  HausdorffDistance(const HausdorffDistance&) = delete;
  HausdorffDistance& operator=(const HausdorffDistance&) = delete;

  // Directed h(A,B) (undirected = false) or H(A,B), host vectors.
  COORD_T CalculateDistance(std::vector<point_t>& points_a, std::vector<point_t>& points_b,
                            bool undirected = false) {
    return Solve(reinterpret_cast<const COORD_T*>(points_a.data()), points_a.size(),
                 reinterpret_cast<const COORD_T*>(points_b.data()), points_b.size(),
                 undirected ? HD_UNDIRECTED : 0u);
  }

  // Same on row-major arrays (host or, with on_device, device memory).
  COORD_T CalculateDistance(const COORD_T* a, uint64_t n_a, const COORD_T* b, uint64_t n_b,
                            bool undirected, bool on_device) {
    return Solve(a, n_a, b, n_b, (undirected ? HD_UNDIRECTED : 0u) | (on_device ? HD_DEVICE_PTRS : 0u));
  }

  const Json& get_stats() const {
    if (!stats_.contains("Algorithm") || !stats_.contains("Execution") ||
        !stats_.contains("ReportedTime"))
      throw std::logic_error("stats are filled by CalculateDistance");
    return stats_;
  }
  const hd_result& last_result() const { return result_; }
  hd_ctx* context() { return ctx_; }

 protected:
  COORD_T Solve(const COORD_T* a, uint64_t na, const COORD_T* b, uint64_t nb, uint32_t flags) {
    flags |= HD_TIMING | HD_COUNT_PAIRS;
    hd_status s;
    if constexpr (std::is_same<COORD_T, double>::value)
      s = hd_solve_f64(ctx_, a, na, b, nb, N_DIMS, flags, -1, &result_);
    else
      s = hd_solve(ctx_, a, na, b, nb, N_DIMS, flags, -1, &result_);
    if (s != HD_OK) throw Error(s, hd_last_error(ctx_));
    static const char* names[] = {"auto", "eb", "grid", "lbvh", "bf16", "brute"};
    stats_ = Json::Object();
    stats_["Algorithm"] = algorithm_;
    stats_["Execution"] = "GPU";
    stats_["ReportedTime"] = result_.ms;
    stats_["VariantUsed"] = names[result_.variant_used < 0 || result_.variant_used > 5
                                      ? 0
                                      : result_.variant_used];
    stats_["ComparedPairs"] = (unsigned long long) result_.visited_pairs;
    stats_["VisitedNodes"] = (unsigned long long) result_.visited_nodes;
    stats_["HD64"] = result_.hd;
    Json pair = Json::Array();
    pair.push_back((unsigned long long) result_.ia);
    pair.push_back((unsigned long long) result_.ib);
    stats_["CertifyingPair"] = pair;
    stats_["Direction"] = result_.direction;
    Json phases = Json::Object();
    const char* pn[] = {"Prep", "Build", "Sample", "Main", "Tail", "Certify"};
    for (int i = 0; i < 6; ++i) phases[pn[i]] = result_.phase_ms[i];
    stats_["PhaseTimes"] = phases;
    if constexpr (std::is_same<COORD_T, double>::value)
      return result_.hd;
    else
      return result_.hd_f32;
  }

  hd_ctx* ctx_ = nullptr;
  std::string algorithm_;
  Json stats_;
  hd_result result_{};
};

#define HD_DEFINE_VARIANT(NAME, VARIANT, LABEL)                                    \
  template <typename COORD_T, int N_DIMS>                                         \
  class NAME : public HausdorffDistance<COORD_T, N_DIMS> {                         \
   public:                                                                         \
    explicit NAME(const hd_options* opt = nullptr)                                 \
        : HausdorffDistance<COORD_T, N_DIMS>(VARIANT, opt, LABEL) {}               \
  };

// early_break.h; hybrid.h (sampler-driven selector); ray_tracing.h (the
// RT-core search rebuilt as an LBVH); uniform_grid.h based search; the
// split-BF16 tensor-core tiles and the plain all-pairs scan (no reference
// class).
HD_DEFINE_VARIANT(HausdorffDistanceEarlyBreak, HD_VARIANT_EB, "Early Break")
HD_DEFINE_VARIANT(HausdorffDistanceHybrid, HD_VARIANT_AUTO, "Hybrid")
HD_DEFINE_VARIANT(HausdorffDistanceRayTracing, HD_VARIANT_LBVH, "LBVH")
HD_DEFINE_VARIANT(HausdorffDistanceGrid, HD_VARIANT_GRID, "Uniform Grid")
HD_DEFINE_VARIANT(HausdorffDistanceBF16, HD_VARIANT_BF16, "Split BF16")
HD_DEFINE_VARIANT(HausdorffDistanceBrute, HD_VARIANT_BRUTE, "Brute Force")
#undef HD_DEFINE_VARIANT

}  // namespace hd
