// The autotuned constants (hd_tuning_table.h, written by
// hausdorffdistance_gb300/autotune.py from its sweep) as the one Tuning
// struct the selector, the batched solver and the launch code read.  Stands in
// for the reference's parameter models (src/models/*, chosen through
// src/hd_impl/hausdorff_distance_hybrid.h:708-778).
#include "hd_tuning.h"
#include "hd_tuning_table.h"

namespace hdg {

const Tuning& tuning() {
  static const Tuning t{HD_TUNED_EB_SMALL_PAIRS, HD_TUNED_INDEX_MIN_PAIRS, HD_TUNED_EB_RATIO,
                        HD_TUNED_BF16_MIN_PAIRS, HD_TUNED_EB_SAMPLE_MAX_PAIRS,
                        HD_TUNED_GRID_MAX_OUTSIDE, HD_TUNED_GRID_MAX_SKEW, HD_TUNED_LEAF_SIZE,
                        HD_TUNED_BATCH_SMALL_ROWS,
                        HD_TUNED_BATCH_CHUNK, HD_TUNED_BATCH_WINDOW, HD_TUNED_LBVH_BUDGET,
                        HD_TUNED_EB_CAP_DIV, HD_TUNED_EB_CAP_MIN, HD_TUNED_EB_CAP_MAX};
  return t;
}

}  // namespace hdg
