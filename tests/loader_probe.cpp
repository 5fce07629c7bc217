// Prints the points a loader returns, for tests/test_loaders.py.
// usage: loader_probe <path> <type> <dims> <limit> [normalize] [translate]
#include <cstdio>
#include <cstdlib>
#include <string>

#include "loaders.h"

int main(int argc, char** argv) {
  if (argc < 5) return 2;
  try {
    hd::PointSet ps = hd::LoadPoints(argv[1], argv[2], std::atoi(argv[3]), std::atoll(argv[4]), "");
    if (argc > 5 && std::atoi(argv[5])) hd::NormalizePoints(ps);
    if (argc > 6) hd::TranslatePoints(ps, 0, std::atof(argv[6]));
    std::printf("%zu\n", ps.size());
    for (size_t i = 0; i < ps.size(); ++i) {
      for (int k = 0; k < ps.dims; ++k) std::printf("%s%.9g", k ? " " : "", ps.xyz[i * ps.dims + k]);
      std::printf("\n");
    }
  } catch (const std::exception& e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 1;
  }
  return 0;
}
