// Driver around the reference's own point preprocessing,
// hd::NormalizePoints and hd::TranslatePoints
// (src/loaders/translate_points.h:42-79), compiled by oracle/build_ref.sh
// straight from the reference sources (never copied) into oracle/_ref/ref_prep.
// Test infrastructure: it generates golden vectors for hd_exec's -normalize
// and -translate (tests/golden/make_golden.py).
//
// usage: ref_prep <in.bin> <out.bin> <n_dims> <normalize 0|1> <translate ratio>
// Reads points in the reference's serialize layout (loader.h:150-185),
// applies NormalizePoints when asked, then TranslatePoints on axis 0 when the
// ratio is not 0 (the order of run_hausdorff_distance.cu:124-133), and writes
// the result in the same layout.
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <vector>

#include "loaders/translate_points.h"

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
  if (atoi(argv[4])) hd::NormalizePoints(pts);
  const double ratio = strtod(argv[5], nullptr);
  if (ratio != 0) hd::TranslatePoints(pts, 0, ratio);
  std::ofstream ofs(argv[2], std::ios::binary);
  const size_t n = pts.size();
  ofs.write(reinterpret_cast<const char*>(&n), sizeof(n));
  if (n) ofs.write(reinterpret_cast<const char*>(pts.data()), sizeof(point_t) * n);
  return ofs ? 0 : 3;
}

int main(int argc, char** argv) {
  if (argc < 6) {
    fprintf(stderr, "usage: ref_prep <in.bin> <out.bin> <n_dims> <normalize> <translate>\n");
    return 2;
  }
  const int dims = atoi(argv[3]);
  if (dims == 2) return run<2>(argv);
  if (dims == 3) return run<3>(argv);
  fprintf(stderr, "n_dims must be 2 or 3\n");
  return 2;
}
