// Runs the statistics helpers of hausdorffdistance_gb300/csrc/hd_stats_host.h
// for tests/test_stats_host.py.
//   hdr_probe rows    stdin: n_nonempty nbins, then "value count" pairs;
//                     stdout: one "value percentile count" line per row, with
//                     the formats of hdr_percentiles_print's CLASSIC output
//                     (%.3f, %f), which the reference parses back.
//   hdr_probe grid    stdin: dims n n_points_cell, then dims lows, dims highs;
//                     stdout: the grid shape.
#include <cstdio>
#include <cstring>
#include <vector>

#include "hd_stats_host.h"

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  if (!std::strcmp(argv[1], "rows")) {
    unsigned long long n_nonempty = 0, nbins = 0, v, c;
    if (std::scanf("%llu %llu", &n_nonempty, &nbins) != 2) return 2;
    std::vector<uint32_t> hist(nbins, 0);
    while (std::scanf("%llu %llu", &v, &c) == 2)
      if (v < nbins) hist[v] += (uint32_t) c;
    for (const auto& r : hdg::stats::hdr_percentiles(hist.data(), nbins, n_nonempty, 3))
      std::printf("%.3f %f %llu\n", r.value, r.percentile, (unsigned long long) r.count);
    return 0;
  }
  int dims = 0;
  unsigned long long n = 0;
  unsigned npc = 0;
  float lo[3], hi[3];
  if (std::scanf("%d %llu %u", &dims, &n, &npc) != 3 || dims < 2 || dims > 3) return 2;
  for (int k = 0; k < dims; ++k)
    if (std::scanf("%f", &lo[k]) != 1) return 2;
  for (int k = 0; k < dims; ++k)
    if (std::scanf("%f", &hi[k]) != 1) return 2;
  hdg::stats::GridShape g;
  if (!hdg::stats::grid_shape(lo, hi, dims, n, npc, 1ull << 28, &g)) {
    std::printf("too large\n");
    return 0;
  }
  for (int k = 0; k < dims; ++k)
    std::printf("%u %.9g %.9g\n", g.size[k], (double) g.upper[k], (double) g.extent[k]);
  std::printf("%llu %.17g %.17g\n", (unsigned long long) g.total_cells, g.density, g.cell_diagonal);
  return 0;
}
