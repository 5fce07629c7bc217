// Selector and launch constants chosen by the autotuner
// (hausdorffdistance_gb300/autotune.py writes hd_tuning_table.h).
#pragma once

namespace hdg {

struct Tuning {
  double eb_small_pairs;  // |A|*|B| at or below which AUTO takes EB unsampled
  double index_min_pairs; // |A|*|B| from which AUTO takes the index unsampled
  double eb_ratio;        // EB when |A| * p80 / (|A| + |B|) is below this
  double bf16_min_pairs;  // n_dims % 16 == 0: BF16 tiles from this |A|*|B| up
  double eb_sample_max_pairs;  // the EB sample runs up to this |A|*|B|
  double grid_max_outside;     // grid only when at most this query fraction is outside
  double grid_max_skew;        // grid only when the target's occupancy skew is at most this
  unsigned leaf_size;     // LBVH points per leaf
  unsigned batch_small_rows;  // batches: directions up to this many rows take one warp
  unsigned batch_chunk;       // batches: consecutive items per warp step
  unsigned batch_window;      // batches: half-width of the bound window
  unsigned lbvh_budget;       // LBVH: per-packet visits before queries are deferred
  unsigned eb_cap_div, eb_cap_min, eb_cap_max;  // EB deferral cap: clamp(|B| / div, min, max)
};

const Tuning& tuning();

}  // namespace hdg
