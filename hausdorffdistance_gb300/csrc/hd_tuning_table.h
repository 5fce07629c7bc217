// Generated by hausdorffdistance_gb300/autotune.py — do not edit by hand.
#pragma once
#define HD_TUNED_EB_SMALL_PAIRS 1e+06
#define HD_TUNED_INDEX_MIN_PAIRS 4e+06
#define HD_TUNED_EB_RATIO 0
#define HD_TUNED_BF16_MIN_PAIRS 67108864.0
#define HD_TUNED_PREFER_GRID 0
#define HD_TUNED_LEAF_SIZE 16
#define HD_TUNED_BATCH_SMALL_ROWS 8192
#define HD_TUNED_BATCH_CHUNK 16
#define HD_TUNED_BATCH_WINDOW 4
#define HD_TUNED_LBVH_BUDGET 256
