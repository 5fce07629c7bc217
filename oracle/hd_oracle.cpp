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
//                     conservative pruning and the early-break rule keeps
//                     large inputs tractable.
//   hd_oracle_exact_batch  the same for many independent problems.
//   hd_oracle_exact_f64    exact directed max-min of FP64 coordinates in FP64.
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

// The same formula in FP64, from float or double coordinates.
template <typename T>
inline double dist2_f64(const T* a, const T* b, int dims) {
  double s = 0.0;
  for (int k = 0; k < dims; ++k) {
    double d = (double) a[k] - (double) b[k];
    double sq = d * d;
    s = (k == 0) ? sq : s + sq;
  }
  return s;
}

// Metric M over coordinates T: 0 = the FP32 formula (float coordinates
// only), 1 = FP64.
template <int M, typename T>
inline double dist2_m(const T* a, const T* b, int dims) {
  if constexpr (M == 0)
    return (double) dist2_f32(a, b, dims);
  else
    return dist2_f64(a, b, dims);
}

template <int N>
struct Pt {
  float c[N];
};

// Restatement of HausdorffDistanceEarlyBreak::CalculateDistance (CPU)
// src/hd_impl/hausdorff_distance_early_break.h:44-115.
//
// begin_a / limit_a select a window [begin_a, limit_a) of the shuffled A
// (limit_a 0 = to the end) and cmax2_init the running maximum it starts
// from: the whole run is begin_a = 0, cmax2_init = 0.  Windows exist for
// bounded CPU baselines: the per-point cost of the scan can only fall as the
// running maximum rises, so a window timed from the final maximum bounds the
// cost of the same points in the full run from below.
template <int N>
void eb_impl(const float* A, uint64_t nA, const float* B, uint64_t nB, int seed,
             int n_threads, uint64_t begin_a, uint64_t limit_a, float cmax2_init,
             float* out_hd, uint64_t* out_pairs, double* out_compute_ms,
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
  const uint64_t first = std::min(begin_a, na_used);
  uint64_t thread_count = (uint64_t) std::max(1, n_threads);
  uint64_t avg_points = (na_used - first + thread_count - 1) / thread_count;
  std::atomic<float> cmax2{cmax2_init};
  std::atomic<uint64_t> compared{0};

  auto compute = [&](uint64_t tid) {
    uint64_t begin = first + tid * avg_points;
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

// The same algorithm for any number of dimensions (rows of `dims` floats,
// moved as rows by the same seeded shuffle).  The reference supports n_dims 2
// and 3 only; this form is the restatement applied to other n_dims and is not
// reference code.
void eb_impl_dims(const float* A, uint64_t nA, const float* B, uint64_t nB, int dims, int seed,
                  int n_threads, uint64_t begin_a, uint64_t limit_a, float cmax2_init,
                  float* out_hd, uint64_t* out_pairs, double* out_compute_ms,
                  double* out_shuffle_ms) {
  auto t0 = std::chrono::high_resolution_clock::now();
  // Shuffle row indices with the reference's engine sequence (A, then B),
  // then gather rows.
  std::mt19937 g(seed);
  std::vector<uint64_t> ia(nA), ib(nB);
  std::iota(ia.begin(), ia.end(), 0);
  std::iota(ib.begin(), ib.end(), 0);
  std::shuffle(ia.begin(), ia.end(), g);
  std::shuffle(ib.begin(), ib.end(), g);
  std::vector<float> pa(nA * dims), pb(nB * dims);
  for (uint64_t i = 0; i < nA; ++i) std::memcpy(&pa[i * dims], A + ia[i] * dims, 4 * dims);
  for (uint64_t j = 0; j < nB; ++j) std::memcpy(&pb[j * dims], B + ib[j] * dims, 4 * dims);
  auto t1 = std::chrono::high_resolution_clock::now();
  uint64_t na_used = (limit_a > 0 && limit_a < nA) ? limit_a : nA;
  const uint64_t first = std::min(begin_a, na_used);
  uint64_t thread_count = (uint64_t) std::max(1, n_threads);
  uint64_t avg_points = (na_used - first + thread_count - 1) / thread_count;
  std::atomic<float> cmax2{cmax2_init};
  std::atomic<uint64_t> compared{0};
  auto compute = [&](uint64_t tid) {
    uint64_t begin = first + tid * avg_points;
    uint64_t end = std::min(begin + avg_points, na_used);
    uint64_t local = 0;
    for (uint64_t i = begin; i < end; ++i) {
      float cmin2 = std::numeric_limits<float>::max();
      for (uint64_t j = 0; j < nB; ++j) {
        float d = dist2_f32(&pa[i * dims], &pb[j * dims], dims);
        ++local;
        if (d < cmin2) cmin2 = d;
        if (cmin2 < cmax2.load()) break;
      }
      if (cmin2 != std::numeric_limits<float>::max()) {
        float prev = cmax2.load();
        while (prev < cmin2 && !cmax2.compare_exchange_weak(prev, cmin2)) {
        }
      }
    }
    compared += local;
  };
  std::vector<std::thread> ts;
  for (uint64_t t = 0; t < thread_count; ++t) ts.emplace_back(compute, t);
  for (auto& t : ts) t.join();
  auto t2 = std::chrono::high_resolution_clock::now();
  *out_hd = std::sqrt(cmax2.load());
  *out_pairs = compared.load();
  *out_shuffle_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
  *out_compute_ms = std::chrono::duration<double, std::milli>(t2 - t1).count();
}

// ---------------------------------------------------------------------------
// Exact max-min with certifying pair.  k-d tree on B (median split on the
// widest dimension, leaves of up to 16 points), built in parallel below the
// top levels.  Pruning compares the FP64 distance to the splitting plane with
// the current best inflated by a relative margin of 1e-4, which exceeds the
// rounding error of the FP32 squared-distance formula for up to 64
// dimensions, so a pruned subtree can never hold a point at or below the
// current best — ties included.
//
// Early break (the reference's rule, early_break.h:76, applied to the tree
// search): a query stops as soon as it has found a point strictly nearer than
// the largest nearest-neighbour distance already established by any thread.
// Such a query cannot reach the maximum, and every query whose nearest
// neighbour is at or above the final maximum runs to completion, so the
// maximum and its lowest-index certifying pair are exact.
template <typename T>
struct KdNode {
  int32_t left, right;  // children, or -1 for a leaf
  int32_t dim;
  T split;
  uint64_t begin, end;  // range in perm for leaves
};

template <typename T>
struct KdTree {
  int dims = 0;
  const T* pts = nullptr;
  std::vector<uint64_t> perm;
  std::vector<T> tp;  // coordinates in tree order (perm applied)
  std::vector<KdNode<T>> nodes;
  std::atomic<int32_t> used{0};

  int32_t alloc_node(uint64_t b, uint64_t e) {
    int32_t id = used.fetch_add(1);
    nodes[id] = KdNode<T>{-1, -1, 0, T(0), b, e};
    return id;
  }

  // Builds the subtree over perm[b, e); subtrees at depth < par_depth are
  // built on their own threads.
  int32_t build(uint64_t b, uint64_t e, int depth, int par_depth) {
    int32_t id = alloc_node(b, e);
    if (e - b <= 16) return id;
    int best_dim = 0;
    T best_ext = T(-1);
    for (int k = 0; k < dims; ++k) {
      T lo = std::numeric_limits<T>::infinity(), hi = -lo;
      for (uint64_t i = b; i < e; ++i) {
        T v = pts[perm[i] * dims + k];
        lo = std::min(lo, v);
        hi = std::max(hi, v);
      }
      if (hi - lo > best_ext) {
        best_ext = hi - lo;
        best_dim = k;
      }
    }
    if (best_ext <= T(0)) return id;  // all points identical: keep a leaf
    uint64_t mid = b + (e - b) / 2;
    std::nth_element(perm.begin() + b, perm.begin() + mid, perm.begin() + e,
                     [&](uint64_t x, uint64_t y) {
                       return pts[x * dims + best_dim] < pts[y * dims + best_dim];
                     });
    T split = pts[perm[mid] * dims + best_dim];
    int32_t l, r;
    if (depth < par_depth && e - b > 65536) {
      int32_t lr = -1;
      std::thread t([&] { lr = build(b, mid, depth + 1, par_depth); });
      r = build(mid, e, depth + 1, par_depth);
      t.join();
      l = lr;
    } else {
      l = build(b, mid, depth + 1, par_depth);
      r = build(mid, e, depth + 1, par_depth);
    }
    nodes[id].left = l;
    nodes[id].right = r;
    nodes[id].dim = best_dim;
    nodes[id].split = split;
    return id;
  }

  void init(const T* p, uint64_t n, int d, int n_threads) {
    pts = p;
    dims = d;
    perm.resize(n);
    std::iota(perm.begin(), perm.end(), 0);
    // Every split leaves at least 8 points on each side, so there are at
    // most n/8 + 1 leaves.
    nodes.assign(2 * (n / 8 + 2), KdNode<T>{});
    used = 0;
    int par_depth = 0;
    while ((1 << par_depth) < std::max(1, n_threads)) ++par_depth;
    if (n) build(0, n, 0, par_depth);
    // Leaves scan contiguous coordinates instead of following perm into the
    // caller's array.
    tp.resize(n * (uint64_t) d);
    const uint64_t nt = (uint64_t) std::max(1, n_threads);
    std::vector<std::thread> ts;
    for (uint64_t t = 0; t < nt; ++t)
      ts.emplace_back([&, t] {
        for (uint64_t i = t * n / nt; i < (t + 1) * n / nt; ++i)
          std::memcpy(&tp[i * d], pts + perm[i] * d, sizeof(T) * d);
      });
    for (auto& t : ts) t.join();
  }

  // Nearest neighbour of q under metric M (0 = FP32 formula, 1 = FP64),
  // abandoned (returns true) once best < stop.
  template <int M>
  bool query(int32_t id, const T* q, double& best, uint64_t& best_idx, double stop) const {
    const KdNode<T>& n = nodes[id];
    if (n.left < 0) {
      const T* p = &tp[n.begin * dims];
      for (uint64_t i = n.begin; i < n.end; ++i, p += dims) {
        double d = dist2_m<M>(q, p, dims);
        if (d <= best) {
          const uint64_t j = perm[i];
          if (d < best || j < best_idx) {
            best = d;
            best_idx = j;
          }
        }
      }
      return best < stop;
    }
    double diff = (double) q[n.dim] - (double) n.split;
    int32_t near = diff < 0 ? n.left : n.right;
    int32_t far = diff < 0 ? n.right : n.left;
    if (query<M>(near, q, best, best_idx, stop)) return true;
    // Points in the left subtree have coordinate <= split, the right >=.
    if (diff * diff <= best * (1.0 + 1e-4)) return query<M>(far, q, best, best_idx, stop);
    return false;
  }
};

void atomic_max(std::atomic<double>& a, double v) {
  double prev = a.load();
  while (prev < v && !a.compare_exchange_weak(prev, v)) {
  }
}

template <int M, typename T>
void exact_tree(const KdTree<T>& tree, const T* A, uint64_t nA, int dims, int n_threads,
                double* hd2, uint64_t* ia, uint64_t* ib) {
  const int nt = std::max(1, n_threads);
  std::vector<double> tbest(nt, -1.0);
  std::vector<uint64_t> ta(nt, 0), tb(nt, 0);
  std::atomic<uint64_t> next{0};
  std::atomic<double> gbest{-1.0};
  // Queries are visited in a pseudo-random order (j -> j*mul mod nA) so that
  // the shared maximum rises early, as the reference's shuffle makes it.
  uint64_t mul = 1;
  if (nA > 2) {
    mul = (uint64_t) ((double) nA * 0.6180339887498949) | 1u;
    while (std::gcd(mul, nA) != 1) mul += 2;
  }
  const uint64_t chunk = 256;
  auto work = [&](int t) {
    for (;;) {
      uint64_t b0 = next.fetch_add(chunk);
      if (b0 >= nA) break;
      uint64_t e0 = std::min(nA, b0 + chunk);
      double stop = gbest.load(std::memory_order_relaxed);
      for (uint64_t v = b0; v < e0; ++v) {
        const uint64_t i = (uint64_t) (((unsigned __int128) v * mul) % nA);
        double best = std::numeric_limits<double>::infinity();
        uint64_t bi = 0;
        if (tree.template query<M>(0, A + i * dims, best, bi, stop)) continue;
        if (best > tbest[t] || (best == tbest[t] && i < ta[t])) {
          tbest[t] = best;
          ta[t] = i;
          tb[t] = bi;
          atomic_max(gbest, best);
          stop = std::max(stop, best);
        }
      }
    }
  };
  std::vector<std::thread> ts;
  for (int t = 0; t < nt; ++t) ts.emplace_back(work, t);
  for (auto& t : ts) t.join();
  double best = -1.0;
  uint64_t ba = 0, bb = 0;
  for (int t = 0; t < nt; ++t) {
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

template <int M, typename T>
void exact_impl(const T* A, uint64_t nA, const T* B, uint64_t nB,
                int dims, int n_threads, double* hd2, uint64_t* ia,
                uint64_t* ib) {
  KdTree<T> tree;
  tree.init(B, nB, dims, n_threads);
  exact_tree<M>(tree, A, nA, dims, n_threads, hd2, ia, ib);
}

// One small problem, single-threaded: brute force with early break against
// the running maximum (the same exactness argument as exact_tree).
template <int M, typename T>
void exact_small(const T* A, uint64_t nA, const T* B, uint64_t nB, int dims,
                 double* hd2, uint64_t* ia, uint64_t* ib) {
  double gbest = -1.0;
  uint64_t ba = 0, bb = 0;
  for (uint64_t i = 0; i < nA; ++i) {
    double best = std::numeric_limits<double>::infinity();
    uint64_t bi = 0;
    bool broke = false;
    for (uint64_t j = 0; j < nB; ++j) {
      double d = dist2_m<M>(A + i * dims, B + j * dims, dims);
      if (d < best) {
        best = d;
        bi = j;
        if (best < gbest) {
          broke = true;
          break;
        }
      }
    }
    if (!broke && best > gbest) {
      gbest = best;
      ba = i;
      bb = bi;
    }
  }
  *hd2 = gbest;
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
    eb_impl<2>(A, nA, B, nB, seed, n_threads, 0, limit_a, 0.0f, out_hd, out_pairs,
               out_compute_ms, out_shuffle_ms);
    return 0;
  }
  if (dims == 3) {
    eb_impl<3>(A, nA, B, nB, seed, n_threads, 0, limit_a, 0.0f, out_hd, out_pairs,
               out_compute_ms, out_shuffle_ms);
    return 0;
  }
  return -1;
}

// The same scan over the window [begin_a, end_a) of the shuffled A, starting
// from the running maximum cmax2_init (bounded CPU baselines).
int hd_oracle_eb_window(const float* A, uint64_t nA, const float* B, uint64_t nB,
                        int dims, int seed, int n_threads, uint64_t begin_a, uint64_t end_a,
                        float cmax2_init, float* out_hd, uint64_t* out_pairs,
                        double* out_compute_ms, double* out_shuffle_ms) {
  if (nA == 0 || nB == 0) return -1;
  if (dims == 2) {
    eb_impl<2>(A, nA, B, nB, seed, n_threads, begin_a, end_a, cmax2_init, out_hd, out_pairs,
               out_compute_ms, out_shuffle_ms);
    return 0;
  }
  if (dims == 3) {
    eb_impl<3>(A, nA, B, nB, seed, n_threads, begin_a, end_a, cmax2_init, out_hd, out_pairs,
               out_compute_ms, out_shuffle_ms);
    return 0;
  }
  if (dims >= 1) {
    eb_impl_dims(A, nA, B, nB, dims, seed, n_threads, begin_a, end_a, cmax2_init, out_hd,
                 out_pairs, out_compute_ms, out_shuffle_ms);
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

// Many independent problems (problem p: A rows offsets_a[p]..offsets_a[p+1]-1,
// B rows offsets_b[p]..): the exact max-min of each, directed or undirected
// (the larger direction; A->B on ties), problems spread over n_threads
// threads.  Outputs per problem: squared distance, certifying pair relative
// to the problem's start, direction.
int hd_oracle_exact_batch(const float* A, const float* B, const uint64_t* offsets_a,
                          const uint64_t* offsets_b, uint64_t n_problems, int dims,
                          int precision, int undirected, int n_threads, double* hd2,
                          uint64_t* ia, uint64_t* ib, int32_t* direction) {
  if (dims < 1 || (precision != 32 && precision != 64)) return -1;
  for (uint64_t p = 0; p < n_problems; ++p)
    if (offsets_a[p + 1] <= offsets_a[p] || offsets_b[p + 1] <= offsets_b[p]) return -1;
  std::atomic<uint64_t> next{0};
  auto one_dir = [&](const float* X, uint64_t nx, const float* Y, uint64_t ny, double* h,
                     uint64_t* x, uint64_t* y) {
    if (nx * ny <= (uint64_t) 1 << 22) {
      if (precision == 32)
        exact_small<0>(X, nx, Y, ny, dims, h, x, y);
      else
        exact_small<1>(X, nx, Y, ny, dims, h, x, y);
    } else {
      if (precision == 32)
        exact_impl<0>(X, nx, Y, ny, dims, 1, h, x, y);
      else
        exact_impl<1>(X, nx, Y, ny, dims, 1, h, x, y);
    }
  };
  auto work = [&]() {
    for (;;) {
      uint64_t p = next.fetch_add(1);
      if (p >= n_problems) break;
      const float* X = A + offsets_a[p] * dims;
      const float* Y = B + offsets_b[p] * dims;
      const uint64_t nx = offsets_a[p + 1] - offsets_a[p], ny = offsets_b[p + 1] - offsets_b[p];
      double h0;
      uint64_t x0, y0;
      one_dir(X, nx, Y, ny, &h0, &x0, &y0);
      int32_t dir = 0;
      if (undirected) {
        double h1;
        uint64_t x1, y1;
        one_dir(Y, ny, X, nx, &h1, &x1, &y1);
        // The larger squared distance decides (compared in the metric's own
        // precision); ties keep A->B.
        const bool win = precision == 32 ? (float) h1 > (float) h0 : h1 > h0;
        if (win) {
          h0 = h1;
          x0 = x1;
          y0 = y1;
          dir = 1;
        }
      }
      hd2[p] = h0;
      ia[p] = x0;
      ib[p] = y0;
      direction[p] = dir;
    }
  };
  int T = std::max(1, n_threads);
  std::vector<std::thread> ts;
  for (int t = 0; t < T; ++t) ts.emplace_back(work);
  for (auto& t : ts) t.join();
  return 0;
}

// Exact directed max-min of FP64 coordinates with FP64 squared distances
// formed by the same formula in double (the reference's distance template
// instantiated for double points, src/geoms/distance.h:17-24, as its disabled
// -is_double dispatch would, src/run_hausdorff_distance.cu:56-62), with the
// certifying pair (lowest indices on ties).
int hd_oracle_exact_f64(const double* A, uint64_t nA, const double* B, uint64_t nB, int dims,
                        int n_threads, double* hd2, uint64_t* ia, uint64_t* ib) {
  if (nA == 0 || nB == 0 || dims < 1) return -1;
  if (nA * nB <= (uint64_t) 1 << 22)
    exact_small<1>(A, nA, B, nB, dims, hd2, ia, ib);
  else
    exact_impl<1>(A, nA, B, nB, dims, n_threads, hd2, ia, ib);
  return 0;
}

// FP32 squared distance of one pair exactly as the reference forms it.
float hd_oracle_dist2_f32(const float* a, const float* b, int dims) {
  return dist2_f32(a, b, dims);
}

}  // extern "C"
