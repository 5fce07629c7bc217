// ORACLE — test infrastructure, not product code.
//
// CPU restatement of the reference's Hausdorff-distance path, used only by
// tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py, and
// only to check results (or as the timed CPU baseline), never as the thing
// being measured.  Parity is pinned: tests/test_oracle.py checks this restatement
// against outputs of the reference's own CPU early-break code compiled from
// its sources (oracle/build_ref.sh -> oracle/_ref/ref_eb), committed as
// tests/golden/*.json by tests/golden/make_golden.py.
//
// Exported (extern "C", loaded with ctypes):
//   hd_oracle_eb      early-break directed HD exactly as the reference's CPU
//                     path computes it (seeded shuffle, static thread split,
//                     strict `cmin2 < cmax2` break, CAS max), including the
//                     compared-pair count.
//   hd_oracle_exact   exact directed max-min with the certifying pair
//                     (argmax a, argmin b; lowest index on ties), squared
//                     distances formed either in FP32 exactly as the
//                     reference forms them or in FP64.  A k-d tree on B with
//                     conservative pruning keeps large inputs tractable.
//
// Build: g++ -O2 -std=c++17 -ffp-contract=off -pthread -shared -fPIC.
// -ffp-contract=off matters: the reference builds with fmad off
// (CMakeLists.txt:122) and aarch64 compilers would otherwise fuse a*a+b*b.
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

namespace {

// Squared distance formed the way src/geoms/distance.h:17-24 forms it:
// per-dimension difference, squared, summed left to right, no FMA.
inline float dist2_f32(const float* a, const float* b, int dims) {
  float s = 0.0f;
  for (int k = 0; k < dims; ++k) {
    float d = a[k] - b[k];
    float sq = d * d;
    s = (k == 0) ? sq : s + sq;
  }
  return s;
}

inline double dist2_f64(const float* a, const float* b, int dims) {
  double s = 0.0;
  for (int k = 0; k < dims; ++k) {
    double d = (double) a[k] - (double) b[k];
    s += d * d;
  }
  return s;
}

template <int N>
struct Pt {
  float c[N];
};

// Restatement of HausdorffDistanceEarlyBreak::CalculateDistance (CPU)
// src/hd_impl/hausdorff_distance_early_break.h:44-115.
template <int N>
void eb_impl(const float* A, uint64_t nA, const float* B, uint64_t nB, int seed,
             int n_threads, uint64_t limit_a, float* out_hd,
             uint64_t* out_pairs, double* out_compute_ms,
             double* out_shuffle_ms) {
  using P = Pt<N>;
  std::vector<P> pa(nA), pb(nB);
  if (nA) std::memcpy(pa.data(), A, sizeof(P) * nA);
  if (nB) std::memcpy(pb.data(), B, sizeof(P) * nB);

  auto t0 = std::chrono::high_resolution_clock::now();
  // early_break.h:50-52 — one engine, A shuffled first, then B.
  std::mt19937 g(seed);
  std::shuffle(pa.begin(), pa.end(), g);
  std::shuffle(pb.begin(), pb.end(), g);
  auto t1 = std::chrono::high_resolution_clock::now();

  // A bounded sample (limit_a > 0) keeps only the first limit_a points of
  // the shuffled A: an unbiased subset, used for time-boxed CPU baselines.
  uint64_t na_used = (limit_a > 0 && limit_a < nA) ? limit_a : nA;
  uint64_t thread_count = (uint64_t) std::max(1, n_threads);
  uint64_t avg_points = (na_used + thread_count - 1) / thread_count;
  std::atomic<float> cmax2{0.0f};
  std::atomic<uint64_t> compared{0};

  auto compute = [&](uint64_t tid) {
    uint64_t begin = tid * avg_points;
    uint64_t end = std::min(begin + avg_points, na_used);
    uint64_t local = 0;
    for (uint64_t i = begin; i < end; ++i) {
      float cmin2 = std::numeric_limits<float>::max();
      for (uint64_t j = 0; j < nB; ++j) {
        float d = dist2_f32(pa[i].c, pb[j].c, N);
        ++local;
        if (d < cmin2) cmin2 = d;
        if (cmin2 < cmax2.load()) break;  // early_break.h:76
      }
      if (cmin2 != std::numeric_limits<float>::max()) {
        float prev = cmax2.load();
        while (prev < cmin2 && !cmax2.compare_exchange_weak(prev, cmin2)) {
        }
      }
    }
    compared += local;
  };

  if (thread_count == 1) {
    compute(0);
  } else {
    std::vector<std::thread> ts;
    for (uint64_t t = 0; t < thread_count; ++t) ts.emplace_back(compute, t);
    for (auto& t : ts) t.join();
  }
  auto t2 = std::chrono::high_resolution_clock::now();
  // early_break.h:114 returns sqrt of the float max: a correctly rounded
  // float square root.
  *out_hd = std::sqrt(cmax2.load());
  *out_pairs = compared.load();
  *out_shuffle_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
  *out_compute_ms = std::chrono::duration<double, std::milli>(t2 - t1).count();
}

// ---------------------------------------------------------------------------
// Exact max-min with certifying pair.  k-d tree on B (median split on the
// widest dimension, leaves of up to 16 points).  Pruning compares the
// FP64 distance to the splitting plane with the current best inflated by a
// relative margin of 1e-4, which exceeds the rounding error of the FP32
// squared-distance formula for up to 64 dimensions, so a pruned subtree can
// never hold a point at or below the current best — ties included.
struct KdNode {
  int32_t left, right;  // children, or -1 for a leaf
  int32_t dim;
  float split;
  uint64_t begin, end;  // range in perm for leaves
};

struct KdTree {
  int dims = 0;
  const float* pts = nullptr;
  std::vector<uint64_t> perm;
  std::vector<KdNode> nodes;

  int32_t build(uint64_t b, uint64_t e) {
    KdNode n{-1, -1, 0, 0.0f, b, e};
    int32_t id = (int32_t) nodes.size();
    nodes.push_back(n);
    if (e - b <= 16) return id;
    int best_dim = 0;
    float best_ext = -1.0f;
    for (int k = 0; k < dims; ++k) {
      float lo = std::numeric_limits<float>::infinity(), hi = -lo;
      for (uint64_t i = b; i < e; ++i) {
        float v = pts[perm[i] * dims + k];
        lo = std::min(lo, v);
        hi = std::max(hi, v);
      }
      if (hi - lo > best_ext) {
        best_ext = hi - lo;
        best_dim = k;
      }
    }
    if (best_ext <= 0.0f) return id;  // all points identical: keep a leaf
    uint64_t mid = b + (e - b) / 2;
    std::nth_element(perm.begin() + b, perm.begin() + mid, perm.begin() + e,
                     [&](uint64_t x, uint64_t y) {
                       return pts[x * dims + best_dim] < pts[y * dims + best_dim];
                     });
    float split = pts[perm[mid] * dims + best_dim];
    int32_t l = build(b, mid);
    int32_t r = build(mid, e);
    nodes[id].left = l;
    nodes[id].right = r;
    nodes[id].dim = best_dim;
    nodes[id].split = split;
    return id;
  }

  void init(const float* p, uint64_t n, int d) {
    pts = p;
    dims = d;
    perm.resize(n);
    std::iota(perm.begin(), perm.end(), 0);
    nodes.clear();
    nodes.reserve(2 * (n / 8 + 1));
    if (n) build(0, n);
  }

  // Nearest neighbour of q under metric M (0 = FP32 formula, 1 = FP64).
  template <int M>
  void query(int32_t id, const float* q, double& best, uint64_t& best_idx) const {
    const KdNode& n = nodes[id];
    if (n.left < 0) {
      for (uint64_t i = n.begin; i < n.end; ++i) {
        uint64_t j = perm[i];
        double d = M == 0 ? (double) dist2_f32(q, pts + j * dims, dims)
                          : dist2_f64(q, pts + j * dims, dims);
        if (d < best || (d == best && j < best_idx)) {
          best = d;
          best_idx = j;
        }
      }
      return;
    }
    double diff = (double) q[n.dim] - (double) n.split;
    int32_t near = diff < 0 ? n.left : n.right;
    int32_t far = diff < 0 ? n.right : n.left;
    query<M>(near, q, best, best_idx);
    // Points in the left subtree have coordinate <= split, the right >=.
    if (diff * diff <= best * (1.0 + 1e-4)) query<M>(far, q, best, best_idx);
  }
};

template <int M>
void exact_impl(const float* A, uint64_t nA, const float* B, uint64_t nB,
                int dims, int n_threads, double* hd2, uint64_t* ia,
                uint64_t* ib) {
  KdTree tree;
  tree.init(B, nB, dims);
  int T = std::max(1, n_threads);
  std::vector<double> tbest(T, -1.0);
  std::vector<uint64_t> ta(T, 0), tb(T, 0);
  std::atomic<uint64_t> next{0};
  const uint64_t chunk = 1024;
  auto work = [&](int t) {
    for (;;) {
      uint64_t b0 = next.fetch_add(chunk);
      if (b0 >= nA) break;
      uint64_t e0 = std::min(nA, b0 + chunk);
      for (uint64_t i = b0; i < e0; ++i) {
        double best = std::numeric_limits<double>::infinity();
        uint64_t bi = 0;
        tree.query<M>(0, A + i * dims, best, bi);
        if (best > tbest[t] || (best == tbest[t] && i < ta[t])) {
          tbest[t] = best;
          ta[t] = i;
          tb[t] = bi;
        }
      }
    }
  };
  std::vector<std::thread> ts;
  for (int t = 0; t < T; ++t) ts.emplace_back(work, t);
  for (auto& t : ts) t.join();
  double best = -1.0;
  uint64_t ba = 0, bb = 0;
  for (int t = 0; t < T; ++t) {
    if (tbest[t] > best || (tbest[t] == best && ta[t] < ba)) {
      best = tbest[t];
      ba = ta[t];
      bb = tb[t];
    }
  }
  *hd2 = best;
  *ia = ba;
  *ib = bb;
}

}  // namespace

extern "C" {

// Returns 0 on success, -1 for unsupported dims or empty inputs.
int hd_oracle_eb(const float* A, uint64_t nA, const float* B, uint64_t nB,
                 int dims, int seed, int n_threads, uint64_t limit_a,
                 float* out_hd, uint64_t* out_pairs, double* out_compute_ms,
                 double* out_shuffle_ms) {
  if (nA == 0 || nB == 0) return -1;
  if (dims == 2) {
    eb_impl<2>(A, nA, B, nB, seed, n_threads, limit_a, out_hd, out_pairs,
               out_compute_ms, out_shuffle_ms);
    return 0;
  }
  if (dims == 3) {
    eb_impl<3>(A, nA, B, nB, seed, n_threads, limit_a, out_hd, out_pairs,
               out_compute_ms, out_shuffle_ms);
    return 0;
  }
  return -1;
}

// precision: 32 = squared distances as the reference's FP32 formula,
//            64 = squared distances in FP64 from the float coordinates.
int hd_oracle_exact(const float* A, uint64_t nA, const float* B, uint64_t nB,
                    int dims, int precision, int n_threads, double* hd2,
                    uint64_t* ia, uint64_t* ib) {
  if (nA == 0 || nB == 0 || dims < 1) return -1;
  if (precision == 32)
    exact_impl<0>(A, nA, B, nB, dims, n_threads, hd2, ia, ib);
  else if (precision == 64)
    exact_impl<1>(A, nA, B, nB, dims, n_threads, hd2, ia, ib);
  else
    return -1;
  return 0;
}

// FP32 squared distance of one pair exactly as the reference forms it.
float hd_oracle_dist2_f32(const float* a, const float* b, int dims) {
  return dist2_f32(a, b, dims);
}

}  // extern "C"
