// Driver around the host-side part of the reference's per-file statistics
// (src/run_hausdorff_distance.cu:150-185): the point set's box made non-empty
// (Mbr::ToNonemptyMBR, src/geoms/mbr.h:288-296), the statistics grid's
// resolution (UniformGrid::CalculateGridResolution,
// src/index/uniform_grid.h:222-244) and the density (count / Mbr::get_volume).
// Compiled by oracle/build_ref.sh straight from the reference sources (never
// copied) into oracle/_ref/ref_stats.  Test infrastructure: it generates the
// golden vectors of hd_compute_stats's grid shape (tests/golden/make_golden.py).
//
// usage: ref_stats <in.bin> <n_dims> <n_points_cell>
// Prints "lower... upper... size... density" on one line (floats as %.9g).
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <vector>

#include "index/uniform_grid.h"

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
static int run(char** argv) {
  using point_t = typename cuda_vec<float, N>::type;
  auto pts = read_bin<point_t>(argv[1]);
  hd::Mbr<float, N> mbr;
  mbr.Expand(pts);
  const auto ne = mbr.ToNonemptyMBR();
  const auto size = hd::UniformGrid<float, N>::CalculateGridResolution(ne, pts.size(),
                                                                       atoi(argv[3]));
  const float density = pts.size() / ne.get_volume();
  for (int k = 0; k < N; ++k) printf("%.9g ", ne.lower(k));
  for (int k = 0; k < N; ++k) printf("%.9g ", ne.upper(k));
  for (int k = 0; k < N; ++k) printf("%u ", reinterpret_cast<const unsigned*>(&size.x)[k]);
  printf("%.9g\n", density);
  return 0;
}

int main(int argc, char** argv) {
  if (argc < 4) {
    fprintf(stderr, "usage: ref_stats <in.bin> <n_dims> <n_points_cell>\n");
    return 2;
  }
  const int dims = atoi(argv[2]);
  if (dims == 2) return run<2>(argv);
  if (dims == 3) return run<3>(argv);
  fprintf(stderr, "n_dims must be 2 or 3\n");
  return 2;
}
