// Host-side arithmetic of hd_compute_stats, kept free of CUDA so that the CPU
// tests compile it alone: the statistics grid's shape as the reference
// computes it, and the percentile table its log prints.
#pragma once
#include <cmath>
#include <cstdint>
#include <limits>
#include <vector>

namespace hdg {
namespace stats {

// The reference's statistics grid over a point set's box
// (src/run_hausdorff_distance.cu:150-185 with Mbr::ToNonemptyMBR,
// src/geoms/mbr.h:288-296, and UniformGrid::CalculateGridResolution and
// GetCellDigonalLength, src/index/uniform_grid.h:222-244,695-705), in the
// same arithmetic: float box and extents (a zero extent becomes lower + 1e-5
// rounded to float, or one float step where that rounds back), the cell side
// s = sqrt (2-D) or cbrt (3-D) of volume * n_points_cell / n in double, the
// volume a double product of the float extents and n the count as a 32-bit
// unsigned integer, ceil(extent / s) cells per axis, the density as the float
// count over the float volume, and the cell diagonal in float.
struct GridShape {
  float lower[3], upper[3], extent[3];
  uint32_t size[3];
  uint64_t total_cells;
  double density;
  double cell_diagonal;
};

// False when an axis would need 2^32 cells or more, or the grid more than
// max_cells cells.
inline bool grid_shape(const float* lo, const float* hi, int dims, uint64_t n,
                       uint32_t n_points_cell, uint64_t max_cells, GridShape* g) {
  double volume = 1.0;
  float volume32 = 1.0f;
  for (int k = 0; k < dims; ++k) {
    const float l = lo[k];
    float u = hi[k];
    if (u - l == 0.0f) u = (float) ((double) l + 1e-5);
    // Where that still rounds back to the lower corner (|lower| of about 128
    // or more) the reference stops on the zero volume; here the axis spans
    // one float step instead.
    if (u - l == 0.0f) u = std::nextafter(l, std::numeric_limits<float>::infinity());
    g->lower[k] = l;
    g->upper[k] = u;
    g->extent[k] = u - l;
    volume *= (double) g->extent[k];
    volume32 *= g->extent[k];
  }
  const double q = volume * (double) n_points_cell / (double) (uint32_t) n;
  const double s = dims == 2 ? std::sqrt(q) : std::cbrt(q);
  uint64_t total = 1;
  float sum2 = 0.0f;
  for (int k = 0; k < dims; ++k) {
    double c = std::ceil((double) g->extent[k] / s);
    if (!(c >= 1.0)) c = 1.0;
    if (c > 4294967295.0) return false;
    g->size[k] = (uint32_t) c;
    total *= g->size[k];
    if (total > max_cells) return false;
    // Float multiply and add, each rounded once (through double, where the
    // product of two floats is exact), so no compiler fuses them.
    const float unit = g->extent[k] / (float) g->size[k];
    const float sq = (float) ((double) unit * (double) unit);
    sum2 = (float) ((double) sum2 + (double) sq);
  }
  g->total_cells = total;
  g->density = (double) ((float) n / volume32);
  g->cell_diagonal = (double) std::sqrt(sum2);
  return true;
}

// HdrHistogram_c (the reference's HdrHistogram dependency, absent here) with
// the reference's settings: hdr_init(1, n_nonempty, 3) and
// hdr_percentiles_print(h, ..., ticks_per_half_distance = 3, 1.0, CLASSIC)
// (src/index/uniform_grid.h:675-693, src/running_stats.h:106-140).
// Three significant figures: values below 2048 are kept exactly; above, a
// value v in [1024 * 2^b, 2048 * 2^b) falls in a bucket of 2^b equal values
// and is reported as its bucket's highest value.
inline uint64_t hdr_highest_equivalent(uint64_t v) {
  if (v < 2048) return v;
  int top = 63;
  while (!((v >> top) & 1)) --top;
  const int b = top - 10;
  return ((v >> b) << b) + ((uint64_t) 1 << b) - 1;
}

struct PercentileRow {
  double value;       // the bucket's highest equivalent value
  double percentile;  // the iteration's target percentile / 100
  uint64_t count;     // cumulative count at the value
};

// Percentile rows from hist[v] = number of non-empty cells holding v points
// (v in [1, nbins)).  Values at or above the histogram's trackable limit (the
// smallest power-of-two multiple of 2048 beyond n_nonempty) are not recorded,
// as hdr_record_value refuses them.  The iteration: a target percentile
// starting at 0; the next value whose cumulative share reaches the target is
// reported at that target (so one value may be reported at several targets),
// and the target then moves up by 100 / (ticks * 2^(floor(log2(100 /
// (100 - target))) + 1)), i.e. `ticks` steps per halving of the distance to
// 100 %; once every recorded cell is counted, one last row at 100 %.
// n_nonempty below 2 is invalid for hdr_init (the reference then prints
// through an uninitialised histogram pointer); it is treated as 2, which gives
// the rows the reference's logs show for such inputs.
inline std::vector<PercentileRow> hdr_percentiles(const uint32_t* hist, uint64_t nbins,
                                                  uint64_t n_nonempty, int ticks) {
  uint64_t untrackable = 2048;
  const uint64_t highest = n_nonempty < 2 ? 2 : n_nonempty;
  while (untrackable <= highest) untrackable <<= 1;
  // Recorded counts per reported value, in increasing value order.
  std::vector<uint64_t> vals, cnts;
  uint64_t total = 0;
  for (uint64_t v = 1; v < nbins && v < untrackable; ++v) {
    if (!hist[v]) continue;
    const uint64_t e = hdr_highest_equivalent(v);
    if (vals.empty() || vals.back() != e) {
      vals.push_back(e);
      cnts.push_back(0);
    }
    cnts.back() += hist[v];
    total += hist[v];
  }
  std::vector<PercentileRow> rows;
  double target = 0.0;
  bool seen_last = false;
  size_t idx = 0;
  bool started = false;
  uint64_t cum = 0, value = 0, count = 0;
  auto advance = [&]() {
    if (!(cum < total) || (started && idx + 1 >= vals.size()) || vals.empty()) return false;
    idx = started ? idx + 1 : 0;
    started = true;
    value = vals[idx];
    count = cnts[idx];
    cum += count;
    return true;
  };
  for (;;) {
    if (!(cum < total)) {
      if (seen_last) break;
      seen_last = true;
      rows.push_back({(double) value, 1.0, cum});
      continue;
    }
    if (!started && !advance()) break;
    bool found = false;
    do {
      const double current = (100.0 * (double) cum) / (double) total;
      if (count != 0 && target <= current) {
        rows.push_back({(double) value, target / 100.0, cum});
        const int64_t temp = (int64_t) (std::log(100 / (100.0 - target)) / std::log(2)) + 1;
        const int64_t half = (int64_t) std::pow(2, (double) temp);
        target += 100.0 / (double) (ticks * half);
        found = true;
        break;
      }
    } while (advance());
    if (!found) break;
  }
  return rows;
}

}  // namespace stats
}  // namespace hdg
