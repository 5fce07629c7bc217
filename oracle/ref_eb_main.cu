// Driver around the reference's own CPU early-break implementation,
// hd::HausdorffDistanceEarlyBreak<float,N>::CalculateDistance(vector&, vector&)
// (src/hd_impl/hausdorff_distance_early_break.h:44-115).  It is compiled by
// oracle/build_ref.sh straight from the reference sources (never copied) into
// oracle/_ref/ref_eb, and is used only to pin the oracle (golden vectors) and
// as the reference CPU arm of the benchmark where it can be built.
//
// usage: ref_eb <A.bin> <B.bin> <n_dims> <seed> <n_threads> [repeat] [limit_a]
// Input files use the reference's serialize layout (loader.h:150-185): a
// size_t count followed by count packed points (floats, or doubles for
// ref_eb64).  Prints one JSON line.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <vector>

#include "utils/launcher.h"
#include "hd_impl/hausdorff_distance_early_break.h"

// Coordinate type of the instantiation: float (ref_eb) or, built with
// -DREF_COORD=double, the reference's double instantiation (ref_eb64), whose
// input files hold doubles.
#ifndef REF_COORD
#define REF_COORD float
#endif
using coord_t = REF_COORD;

template <typename P>
static std::vector<P> read_bin(const char* path) {
  std::ifstream ifs(path, std::ios::binary);
  if (!ifs) {
    fprintf(stderr, "cannot open %s\n", path);
    exit(2);
  }
  size_t n = 0;
  ifs.read(reinterpret_cast<char*>(&n), sizeof(n));
  std::vector<P> v(n);
  if (n) ifs.read(reinterpret_cast<char*>(v.data()), sizeof(P) * n);
  return v;
}

template <int N>
static int run(int argc, char** argv) {
  using point_t = typename cuda_vec<coord_t, N>::type;
  auto a0 = read_bin<point_t>(argv[1]);
  auto b0 = read_bin<point_t>(argv[2]);
  int seed = atoi(argv[4]);
  int threads = atoi(argv[5]);
  int repeat = argc > 6 ? atoi(argv[6]) : 1;
  long long limit_a = argc > 7 ? atoll(argv[7]) : -1;
  typename hd::HausdorffDistanceEarlyBreak<coord_t, N>::Config cfg;
  cfg.seed = seed;
  cfg.n_threads = threads;
  hd::HausdorffDistanceEarlyBreak<coord_t, N> eb(cfg);
  printf("{\"n_a\": %zu, \"n_b\": %zu, \"runs\": [", a0.size(), b0.size());
  for (int r = 0; r < repeat; ++r) {
    // The reference shuffles its inputs in place; every repeat starts from
    // the file order so that repeats are identical.
    auto a = a0;
    auto b = b0;
    const coord_t hd_val = eb.CalculateDistance(a, b);
    (void) limit_a;
    const auto& st = eb.get_stats();
    unsigned long long bits = 0;
    memcpy(&bits, &hd_val, sizeof(coord_t));
    printf(sizeof(coord_t) == 4 ? "%s{\"hd\": %.9g, \"hd_bits\": %llu, \"compared_pairs\": %llu, "
                                  "\"compute_ms\": %.6f, \"shuffle_ms\": %.6f, \"threads\": %d}"
                                : "%s{\"hd\": %.17g, \"hd_bits\": %llu, \"compared_pairs\": %llu, "
                                  "\"compute_ms\": %.6f, \"shuffle_ms\": %.6f, \"threads\": %d}",
           r ? ", " : "", (double) hd_val, bits,
           (unsigned long long) st.at("ComparedPairs").template get<uint64_t>(),
           st.at("ComputeTime").template get<double>(),
           st.at("ShuffleTime").template get<double>(), threads);
  }
  printf("]}\n");
  return 0;
}

int main(int argc, char** argv) {
  if (argc < 6) {
    fprintf(stderr,
            "usage: %s A.bin B.bin n_dims seed n_threads [repeat]\n", argv[0]);
    return 2;
  }
  int dims = atoi(argv[3]);
  if (dims == 2) return run<2>(argc, argv);
  if (dims == 3) return run<3>(argc, argv);
  fprintf(stderr, "n_dims must be 2 or 3\n");
  return 2;
}
