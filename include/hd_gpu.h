/*
 * hd_gpu.h — C ABI of libhdgpu.so, the GB300 (sm_103a) Hausdorff-distance
 * engine.
 *
 * It replaces the reference's algorithm seam
 *   hd::HausdorffDistance<COORD_T,N_DIMS>::CalculateDistance(...)
 *   (src/hausdorff_distance.h:21-32)
 * and the variant factory + repeat loop that drive it
 *   (src/run_hausdorff_distance.cu:220-357).
 * Plain pointers and sizes only; no C++ types cross the boundary, no
 * exceptions escape.  Every call returns an hd_status.
 *
 * Semantics (identical to the reference's -execution=cpu result):
 *   directed   h(A,B) = max_{a in A} min_{b in B} ||a - b||
 *   undirected H(A,B) = max(h(A,B), h(B,A))
 * Squared distances are formed in FP32 as the reference forms them
 * (src/geoms/distance.h:17-24: per-dimension difference, squared, summed left
 * to right, no FMA), min/max are exact, and hd_f32 is the correctly rounded
 * float square root: bit-identical to the reference CPU early-break.  The
 * certifying pair (ia, ib) achieves it; hd is its distance recomputed in FP64.
 *
 * Threading: one hd_ctx per host thread.  A context owns one CUDA stream
 * (or borrows the caller's, see hd_set_stream) and a cached device arena.
 * Inputs are const: unlike the reference (which shuffles its inputs in place,
 * early_break.h:50-52), nothing the caller passes is modified.
 */
#ifndef HD_GPU_H
#define HD_GPU_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define HD_API __attribute__((visibility("default")))
#else
#define HD_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef enum hd_status {
  HD_OK = 0,
  HD_ERR_INVALID_ARG = 1,    /* null pointer, zero size, bad n_dims/flags     */
  HD_ERR_OOM = 2,            /* device or pinned allocation failed            */
  HD_ERR_DEVICE_TIMEOUT = 3, /* a bounded device wait ran out (status word)   */
  HD_ERR_CUDA = 4,           /* any other CUDA runtime error                  */
  HD_ERR_UNSUPPORTED = 5,    /* variant not available for these inputs       */
  HD_ERR_NO_DEVICE = 6       /* no CUDA device or the library was built for   */
                             /* another architecture                          */
} hd_status;

/* Variants.  The reference's -variant names map as: eb -> HD_VARIANT_EB,
 * hybrid -> HD_VARIANT_AUTO, rt -> HD_VARIANT_LBVH (GB300 has no RT cores;
 * the OptiX search of src/hd_impl/hausdorff_distance_ray_tracing.h:63-236 is
 * rebuilt as a plain-CUDA LBVH). */
typedef enum hd_variant {
  HD_VARIANT_AUTO = 0,  /* sampler-driven selector (hybrid.h:86-409 analogue) */
  HD_VARIANT_EB = 1,    /* persistent early-break scan (early_break.h:117-219)*/
  HD_VARIANT_GRID = 2,  /* Morton-sorted uniform grid + ring search           */
  HD_VARIANT_LBVH = 3,  /* LBVH nearest-neighbour with early break            */
  HD_VARIANT_BF16 = 4,  /* split-BF16 tcgen05 tiles + exact FP32 recheck      */
  HD_VARIANT_BRUTE = 5  /* plain FP32 all-pairs (no early break)              */
} hd_variant;

/* hd_solve flags */
#define HD_DIRECTED 0u
#define HD_UNDIRECTED 1u   /* max(h(A,B), h(B,A))                              */
#define HD_DEVICE_PTRS 2u  /* A and B are device pointers (no H2D copy)        */
#define HD_COUNT_PAIRS 4u  /* instrumented run: fill visited_pairs/nodes       */
#define HD_TIMING 8u       /* record per-phase CUDA-event times in hd_result   */

typedef struct hd_options {
  int device;              /* CUDA device ordinal                             */
  int variant;             /* hd_variant used when a call does not override   */
  uint64_t seed;           /* visit-order permutation / sampler seed          */
  double sample_rate;      /* selector sample fraction of |A| (hybrid.h:134)  */
  uint32_t n_points_cell;  /* grid: target points per cell (uniform_grid.h:222)*/
  uint32_t leaf_size;      /* LBVH: points per leaf (<= 32)                    */
  uint32_t eb_only_threshold; /* selector: p80 sample iterations below which  */
                              /* plain EB is chosen (hybrid.h:171); 0 = table */
  uint32_t always_sample;  /* selector: draw the sample statistic even where  */
                           /* the size bands decide alone (autotuning)        */
  uint32_t batch_small_rows; /* batches: directions of at most this many query */
                             /* rows take the one-warp path (1..65536); 0 = table */
  uint32_t batch_chunk;    /* batches: consecutive items per warp step (1..64); */
                           /* 0 = table                                        */
  uint32_t batch_window;   /* batches: half-width of the bound window (1..8);  */
                           /* 0 = table                                        */
  uint32_t lbvh_budget;    /* LBVH: nodes + leaves a packet visits before its  */
                           /* open queries go to the deferred pass; 0 = table */
  uint32_t eb_cap_pairs;   /* EB: pairs a point scans in the persistent kernel */
                           /* before it is deferred (>= 256); 0 = from |B| by */
                           /* the tuning table                                 */
  uint32_t reserved[2];
} hd_options;

typedef struct hd_result {
  double hd;               /* FP64 distance of the certifying pair            */
  float hd_f32;            /* FP32 result, bit-identical to reference CPU EB   */
  int32_t direction;       /* 0: pair is (A[ia], B[ib]); 1: (B[ib'], A[ia'])  */
                           /* i.e. for direction 1, ia indexes B, ib indexes A */
  uint64_t ia, ib;         /* certifying pair indices (caller's order)         */
  double hd_ab, hd_ba;     /* FP64 directed distances (hd_ba < 0 if directed)  */
  uint64_t visited_pairs;  /* pair distances evaluated (HD_COUNT_PAIRS)        */
  uint64_t visited_nodes;  /* internal index nodes visited (HD_COUNT_PAIRS)   */
  double ms;               /* device time of the whole solve (HD_TIMING)       */
  double phase_ms[8];      /* HD_TIMING: prep, build, sample, query, tail,     */
                           /* certify, copy-in, other                          */
  int32_t variant_used;    /* hd_variant actually run (direction A->B)         */
  int32_t variant_used_ba; /* and for B->A when undirected                     */
  double err_bound;        /* BF16: bound on |approx - exact| squared distance */
  uint64_t rechecked;      /* BF16: rows rechecked exactly in FP32; LBVH:      */
                           /* queries over the traversal budget (finished by  */
                           /* the deferred pass); EB: points deferred past    */
                           /* the per-point pair cap                           */
  uint64_t visited_leaves; /* index leaves / cells scanned (HD_COUNT_PAIRS)    */
  double sample_p80[2];    /* AUTO: 80th percentile of the sampled early-break */
                           /* iteration counts per direction (0 = no sample)   */
  double grid_outside[2];  /* AUTO: fraction of sampled query points outside   */
                           /* the target's box, per direction (0 = not drawn)  */
  double grid_skew[2];     /* AUTO: target cell-occupancy skew at the grid's   */
                           /* resolution, ~1 for uniform data (0 = not drawn)  */
  double sample_mean[2];   /* AUTO: mean of the sampled early-break iteration  */
                           /* counts (capped), per direction (0 = no sample)   */
} hd_result;

/* One problem of a batch: A[offset_a .. offset_a+n_a), B[offset_b ..).
 * Offsets are in points, into the arrays given to hd_solve_batch. */
typedef struct hd_problem {
  uint64_t offset_a, n_a;
  uint64_t offset_b, n_b;
} hd_problem;

typedef struct hd_batch_result {
  float hd_f32;            /* per-problem result (same semantics as hd_result) */
  uint32_t ia, ib;         /* certifying pair, relative to the problem's start */
  int32_t direction;
} hd_batch_result;

/* Statistics of one point set (hd_compute_stats): the per-file "Grid", "MBR"
 * and "Density" entries the reference writes to its JSON log
 * (src/run_hausdorff_distance.cu:150-185). */
#define HD_STATS_HIST_ROWS 96
typedef struct hd_point_stats {
  int32_t n_dims;              /* 2 or 3                                        */
  uint32_t n_points_cell;      /* target points per cell of the statistics grid */
  uint64_t n_points;
  double lower[3], upper[3];   /* bounding box (a zero extent widened to 1e-5)  */
  double density;              /* n_points / box volume                         */
  uint32_t grid_size[3];       /* cells per axis: ceil(extent / s),             */
                               /* s = (volume * n_points_cell / n)^(1/d)        */
  uint32_t max_points;         /* most points in one cell                      */
  uint64_t total_cells;
  uint64_t nonempty_cells;
  uint32_t median_points;      /* median count over the non-empty cells        */
  uint32_t n_hist;             /* rows of the percentile table below           */
  double gini_index;           /* Gini index of the non-empty cells' counts    */
  double cell_diagonal;        /* length of a cell's diagonal                  */
  double build_ms;             /* device time of the box and cell counts       */
  double hist_value[HD_STATS_HIST_ROWS];      /* points per cell at ...         */
  double hist_percentile[HD_STATS_HIST_ROWS]; /* ... this fraction of the cells */
  uint64_t hist_count[HD_STATS_HIST_ROWS];    /* cells at or below the value    */
} hd_point_stats;

typedef struct hd_ctx hd_ctx;

/* Fills *opt with defaults (device 0, AUTO, seed 0, sample_rate 0.01,
 * n_points_cell 8, leaf_size 16). */
HD_API void hd_default_options(hd_options* opt);

/* Creates a context on opt->device (opt may be NULL for defaults).
 * Replaces the variant construction in run_hausdorff_distance.cu:220-334. */
HD_API hd_status hd_create(hd_ctx** ctx, const hd_options* opt);

/* Destroys the context and releases its arena and stream. */
HD_API hd_status hd_destroy(hd_ctx* ctx);

/* Makes the context launch on a caller-owned stream (a cudaStream_t passed
 * as void*); NULL restores the context's own stream. */
HD_API hd_status hd_set_stream(hd_ctx* ctx, void* cuda_stream);

/* Computes the Hausdorff distance of A (n_a x n_dims floats, row-major) and
 * B (n_b x n_dims).  n_dims 2 or 3 for every variant; n_dims in [1, 128] for
 * EB and BRUTE; BF16 takes n_dims 16, 32, 48 or 64.  variant < 0 uses the
 * context default.  Synchronous: returns after the result is on the host.
 * Replaces HausdorffDistance::CalculateDistance (hausdorff_distance.h:21-32),
 * both the CPU and the GPU overload. */
HD_API hd_status hd_solve(hd_ctx* ctx, const float* A, uint64_t n_a, const float* B,
                   uint64_t n_b, int n_dims, uint32_t flags, int variant,
                   hd_result* out);

/* FP64 input path: the Hausdorff distance of double-precision point sets,
 * exact in FP64 (squared distances formed in double by the same formula:
 * per-dimension difference, squared, summed left to right, no FMA).
 * Replaces the reference's double instantiations behind its disabled
 * -is_double dispatch (run_hausdorff_distance.cu:56-62, the
 * RunHausdorffDistanceImpl<double, 2|3> cases).
 *
 * A is n_a x n_dims doubles, B n_b x n_dims (row-major; host pointers, or
 * device pointers with HD_DEVICE_PTRS).  variant: HD_VARIANT_AUTO or
 * HD_VARIANT_LBVH (n_dims 2 or 3: FP32 tree search on the sets rounded to
 * float, FP64 only for the rows the FP32 values cannot settle), or
 * HD_VARIANT_EB / HD_VARIANT_BRUTE (an FP64 scan, n_dims in [1, 256]);
 * the grid and BF16 variants return HD_ERR_UNSUPPORTED.  AUTO takes the
 * scan for other n_dims and for coordinates beyond +-1e18.  NaN or infinite
 * coordinates return HD_ERR_INVALID_ARG.
 *
 * Results in *out: hd, hd_ab, hd_ba are the FP64 distances; ia, ib,
 * direction the certifying pair (lowest row, then lowest column among
 * ties; direction 1 only when B->A is strictly larger); hd_f32 = hd
 * rounded to float; variant_used the path taken; rechecked the rows whose
 * nearest neighbour was searched in FP64; flags HD_COUNT_PAIRS (the FP32
 * search's counts) and HD_TIMING (ms only) as for hd_solve. */
HD_API hd_status hd_solve_f64(hd_ctx* ctx, const double* A, uint64_t n_a, const double* B,
                              uint64_t n_b, int n_dims, uint32_t flags, int variant,
                              hd_result* out);

/* Solves many independent problems (2-D or 3-D) in one graph-captured
 * persistent launch.  A/B hold all problems' points back to back; probs[i]
 * gives each problem's ranges; out[i] receives its result.  flags as for
 * hd_solve (HD_UNDIRECTED, HD_DEVICE_PTRS).  No counterpart in the
 * reference, which solves one pair per hd_exec run. */
HD_API hd_status hd_solve_batch(hd_ctx* ctx, const float* A, uint64_t total_a,
                         const float* B, uint64_t total_b, int n_dims,
                         const hd_problem* probs, uint64_t n_problems,
                         uint32_t flags, hd_batch_result* out);

/* The same batched solve with the problems given as offsets: problem i owns
 * rows offsets_a[i] .. offsets_a[i+1]-1 of A and offsets_b[i] ..
 * offsets_b[i+1]-1 of B (n_problems + 1 entries each, host memory).  Saves
 * building an hd_problem array; the problems are expanded on the device.
 * Decreasing offsets or empty problems are rejected (HD_ERR_INVALID_ARG).
 * No counterpart in the reference. */
HD_API hd_status hd_solve_batch_offsets(hd_ctx* ctx, const float* A, uint64_t total_a,
                                 const float* B, uint64_t total_b, int n_dims,
                                 const uint64_t* offsets_a, const uint64_t* offsets_b,
                                 uint64_t n_problems, uint32_t flags, hd_batch_result* out);

/* Same batch computed with one plain early-break launch per problem and
 * direction (the per-pair baseline the batched form is compared against). */
HD_API hd_status hd_solve_batch_plain(hd_ctx* ctx, const float* A, uint64_t total_a,
                               const float* B, uint64_t total_b, int n_dims,
                               const hd_problem* probs, uint64_t n_problems,
                               uint32_t flags, hd_batch_result* out);

/* Early-break Hausdorff distance that allocates nothing.
 *
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory while they call in: a process that hands all of its HBM to its own
 * pool at start-up, or host code in a phase where a cudaMalloc/cudaFree
 * (which synchronise the device) would stall work it keeps in flight.  It
 * runs the EB variant's kernels with all scratch in one fixed device array
 * inside libhdgpu.so (about 32 MiB, held by every GPU that loads the library
 * until the process exits) and calls no cudaMalloc, cudaFree or other
 * allocating routine.
 *
 * A and B are DEVICE pointers (n x n_dims floats, n_dims 2 or 3) on the
 * current device; flags may hold HD_UNDIRECTED (HD_DEVICE_PTRS is implied).
 * Work is queued on `stream` (a cudaStream_t, NULL = default stream) and the
 * call returns after the result is in *out (same fields and FP32 bit-exact
 * result as hd_solve with HD_VARIANT_EB; no timing).  n_a and n_b are limited
 * to 1,048,576 points each: larger inputs return HD_ERR_INVALID_ARG before any
 * device work.  Every call looks up the array's device address in the current
 * context (cudaGetSymbolAddress, which allocates nothing), so the address
 * stays right after a device reset or under another context.  The call waits
 * for its stream to finish its own work before it returns (it reads the result
 * back and synchronises the stream); if a launch fails part-way, it also waits
 * for the kernels it already queued before returning the error.  Because it
 * synchronises, it cannot be recorded into a CUDA graph: do not call it while
 * its stream (or any stream, under a global-mode capture) is capturing.  Every call
 * shares the one array, which keeps the last call's contents (each call resets
 * what must start at zero): calls that overlap on the GPU — from two host
 * threads, or on two streams — race on it and must be serialised by the
 * caller. */
HD_API hd_status hd_solve_eb_noalloc(const float* A, uint64_t n_a, const float* B,
                                     uint64_t n_b, int n_dims, uint32_t flags,
                                     void* stream, hd_result* out);

/* Test hook for the split-BF16 tensor-core kernel: writes, for every row of
 * A (host pointers, n_dims % 16 == 0, <= 64), the kernel's approximate
 * min over B of ||a - b||^2 before certification into rowmin_out[n_a].
 * No counterpart in the reference. */
HD_API hd_status hd_debug_bf16_rowmin(hd_ctx* ctx, const float* A, uint64_t n_a,
                                      const float* B, uint64_t n_b, int n_dims,
                                      float* rowmin_out);

/* Bounding box, density and the occupancy of the reference's statistics
 * grid (n_points_cell points per cell on average) of one 2-D or 3-D point set,
 * host or device pointer (HD_DEVICE_PTRS), computed on the device.  Replaces
 * the per-file statistics pass of src/run_hausdorff_distance.cu:150-185
 * (UniformGrid::Insert and ComputeHistogram, src/index/uniform_grid.h:343-484,
 * 673-693, and gini_index_thrust, src/running_stats.h:33-62).  Grids of more
 * than 2^28 cells return HD_ERR_UNSUPPORTED. */
HD_API hd_status hd_compute_stats(hd_ctx* ctx, const float* points, uint64_t n, int n_dims,
                                uint32_t n_points_cell, uint32_t flags, hd_point_stats* out);

/* Message for the last failing call on this context (never NULL). */
HD_API const char* hd_last_error(hd_ctx* ctx);

/* Name of a status code. */
HD_API const char* hd_status_string(hd_status s);

/* Number of kernels of this library launched by the context so far. */
HD_API uint64_t hd_kernel_launches(hd_ctx* ctx);

/* Library version string. */
HD_API const char* hd_version(void);

#ifdef __cplusplus
}
#endif
#endif /* HD_GPU_H */
