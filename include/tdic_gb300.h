/*
 * tdic_gb300.h -- C ABI of the GB300 (sm_103a) 2D subset-DIC hot path.
 *
 * Drop-in boundary for lbd-hfut/Traditional-DIC.  The reference has no C ABI; its seams are
 *   - the per-POI virtual call SubsetSolver::solve_with_interpolators
 *     (include/dic/subset/solver/subset_solver.hpp:39-65), called inside the propagation heap
 *     loop of ReliabilityPropagation::propagate (src/subset/seed/reliability_propagation.cpp:283-389);
 *   - the pybind entry _traditional_dic.subset.compute(reference, deformed, config, roi)
 *     (bindings/python/bind_subset.cpp:253-356) that wraps SubsetDIC::compute
 *     (src/subset/subset_dic.cpp:39-105).
 * Every entry point below names the reference interface it replaces.  Plain C types only:
 * pointers, sizes, POD structs.  Nothing throws across this boundary; every call returns a
 * tdic_status and tdic_last_error() holds the message of the last failure on the context.
 *
 * Threading: a context is internally locked (one call at a time per context); use one
 * context per host thread for concurrency.  Streams are passed as void* (cudaStream_t);
 * NULL means the context's own stream.
 */
#ifndef TDIC_GB300_H
#define TDIC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum tdic_status {
    TDIC_OK = 0,
    TDIC_INVALID_ARG = 1,   /* reference: std::invalid_argument / pybind TypeError, ValueError */
    TDIC_OOM = 2,           /* device allocation or admission refused */
    TDIC_CUDA_ERROR = 3,    /* a CUDA runtime error (message in tdic_last_error) */
    TDIC_TIMEOUT = 4,       /* a bounded device-side wait ran out */
    TDIC_UNSUPPORTED = 5    /* a route or size this path does not cover (a batch of other routes, ...) */
} tdic_status;

typedef enum tdic_dtype { TDIC_U8 = 0, TDIC_U16 = 1, TDIC_F32 = 2, TDIC_F64 = 3 } tdic_dtype;

typedef enum tdic_memory { TDIC_HOST = 0, TDIC_DEVICE = 1 } tdic_memory;

typedef enum tdic_precision { TDIC_FP32_MIXED = 0, TDIC_FP64 = 1 } tdic_precision;

/* Shared-memory staging of a solver group (first-order ZNSSD route; the other routes always
 * stage in full).  FULL: the coefficient window under the warped subset and four per-sample
 * arrays; LEAN: only the per-sample arrays the iterations write, the reference values and
 * gradients re-read from the staged reference window; LEAN_NO_WINDOW: LEAN, and the spline
 * stencils read from the (L2-resident) coefficient image.  AUTO takes the mode that keeps the
 * most solver groups resident (the fullest staging among equals); a mode whose shared memory
 * does not fit returns TDIC_UNSUPPORTED. */
typedef enum tdic_staging {
    TDIC_STAGING_AUTO = 0, TDIC_STAGING_FULL = 1, TDIC_STAGING_LEAN = 2, TDIC_STAGING_LEAN_NO_WINDOW = 3
} tdic_staging;

/* Per-POI status ordinals = dic::SolverStatus (include/dic/core/types.hpp:35-40). */
enum { TDIC_SUCCESS = 0, TDIC_NOT_CONVERGED = 1, TDIC_INVALID_INPUT = 2, TDIC_NUMERICAL_FAILURE = 3 };

/* The knobs of dic::SubsetConfig reachable from the pybind config dict
 * (include/dic/subset/subset_config.hpp:33-50, include/dic/initialization/seed_config.hpp:32-68,
 * include/dic/interpolation/bspline.hpp:42-67), C++ defaults from tdic_config_default().
 * propagation_mode and precision are GPU-only knobs (the reference has neither).  The visit
 * order of the propagation: 1 = the reference's own serial heap order (its results, reproduced
 * on the device in rounds), 2 = dataflow (a grid point is solved as soon as its parent one step
 * toward the seed is accepted; the fastest), 0 = frontier waves. */
typedef struct tdic_config {
    int32_t subset_radius;             /* subset.radius                               15 */
    int32_t max_iterations;            /* optimization.max_iterations                 30 */
    double convergence_threshold;      /* optimization.convergence_threshold        1e-3 */
    int32_t optimizer;                 /* optimization.method: 0 icgn, 1 fgn           0 */
    int32_t shape_order;               /* shape_function.order                          1 */
    int32_t criterion;                 /* correlation.criterion: 1 znssd, 0 ssd         1 */
    int32_t degree;                    /* interpolation.degree (1, 3; else 5)           5 */
    int32_t border;                    /* B-spline border (>= 3)                        3 */
    int32_t propagation_spacing;       /* reliability_propagation.spacing (gap count)   5 */
    double propagation_max_znssd;      /* reliability_propagation.max_znssd           0.5 */
    int32_t is_subset_radius;          /* initialization.integer_search.subset_radius  10 */
    int32_t is_search_radius;          /* initialization.integer_search.search_radius  30 */
    int32_t sift_enabled;              /* initialization.integer_search.sift_enabled    0 */
    int32_t pyramid_enabled;           /* ....pyramid_enabled                           1 */
    int32_t pyramid_scale;             /* ....pyramid_scale                             4 */
    int32_t pyramid_refinement_radius; /* ....pyramid_refinement_radius                 4 */
    int32_t sp_enabled;                /* initialization.subpixel_refinement.enabled    1 */
    int32_t sp_subset_radius;          /* ....subset_radius                            15 */
    int32_t sp_max_iterations;         /* ....max_iterations                           30 */
    int32_t precision;                 /* tdic_precision (GPU only)         FP32_MIXED */
    double sp_convergence_threshold;   /* ....convergence_threshold                  1e-3 */
    int32_t seed_count;                /* seed_selection.seed_count                   256 */
    int32_t kmeans_iterations;         /* seed_selection.kmeans_iterations             20 */
    double seed_max_znssd;             /* seed_selection.max_znssd                    0.2 */
    double min_displacement_norm;      /* seed_selection.min_displacement_norm          0 */
    double min_texture_std;            /* seed_selection.min_texture_std                0 */
    int32_t kmeans_sample_limit;       /* seed_selection.kmeans_sample_limit        20000 */
    int32_t propagation_mode;          /* 1 heap (reference), 2 dataflow, 0 waves       2 */
    /* Masked subsets (SubsetConfig, subset_config.hpp:40-42; set from the YAML subset section,
     * yaml_parser.cpp:103-111, not from the pybind dict): samples outside the ROI are left out of
     * each subset, and SubsetDIC::compute pads the images (subset_dic.cpp:53-56). */
    int32_t truncate_roi_subsets;      /* subset.truncate_roi_subsets                    0 */
    int32_t min_valid_samples;         /* subset.min_valid_samples                       12 */
    double min_valid_sample_ratio;     /* subset.min_valid_sample_ratio                 0.5 */
    /* GPU only: shared-memory staging of the first-order ZNSSD solves (tdic_staging); the choice
     * changes speed and shared-memory needs, never a result. */
    int32_t staging;                   /* tdic_staging                                AUTO */
    int32_t pad_;
} tdic_config;

/* One POI for a batched solve: centre (rounded to the nearest pixel as icgn.cpp:472-473),
 * initial guess u, v, du_dx, du_dy, dv_dx, dv_dy and initial.confidence. */
typedef struct tdic_poi_in {
    double x, y;
    double p0[6];
    double confidence;
} tdic_poi_in;

/* dic::Displacement2D (include/dic/core/result.hpp:32-51) plus additive fields: zncc =
 * clamp(1 - correlation / 2, -1, 1), iterations (loop bodies entered), converged (strict
 * |dp| < threshold; the reference's `valid` is also true when the loop ran out with a finite
 * correlation, icgn.cpp:620-625).  correlation is the ZNSSD, or the SSD when criterion = 0.
 * q: the second-order terms d2u_dx2, d2u_dxdy, d2u_dy2, d2v_dx2, d2v_dxdy, d2v_dy2 (zero for
 * the first-order shape function). */
typedef struct tdic_poi_out {
    double p[6];
    double correlation;
    double zncc;
    int32_t iterations;
    int8_t status;
    int8_t valid;
    int8_t converged;
    int8_t pad_;
    double q[6];
} tdic_poi_out;

/* The propagation seed (PropagationSeed, reliability_propagation.hpp:35-39). */
typedef struct tdic_seed {
    double x, y;
    double p[6];
    double correlation;
    int32_t found;
    int32_t pad_;
} tdic_seed;

/* Structure-of-arrays grid result, one entry per grid point i = gy * grid_w + gx
 * (reliability_propagation.cpp:159-176); keys of results_to_dict (bind_subset.cpp:102-153)
 * plus zncc / iterations / converged / status and the second-order terms of
 * dic::Displacement2D (result.hpp:42-47; zero for the first-order shape function).  Any
 * pointer may be NULL (not written). */
typedef struct tdic_grid_out {
    double* x; double* y; double* u; double* v;
    double* du_dx; double* du_dy; double* dv_dx; double* dv_dy;
    double* correlation; double* zncc;
    uint8_t* valid; int8_t* status; int32_t* iterations; uint8_t* converged;
    double* d2u_dx2; double* d2u_dxdy; double* d2u_dy2; double* d2v_dx2; double* d2v_dxdy; double* d2v_dy2;
} tdic_grid_out;

typedef struct tdic_ctx tdic_ctx;
typedef struct tdic_pair tdic_pair;

/* Defaults of dic::SubsetConfig{} (subset_config.hpp:33-50). */
void tdic_config_default(tdic_config* cfg);

/* Output grid size: ceil(W / stride) x ceil(H / stride), stride = spacing + 1
 * (reliability_propagation.cpp:154-160). */
void tdic_grid_dims(int32_t width, int32_t height, int32_t spacing, int32_t* grid_w, int32_t* grid_h);

/* Context: one device, one stream, a caching device-memory pool and per-radius sample tables.
 * (No reference counterpart: the reference builds its state per call.) */
tdic_status tdic_ctx_create(int32_t device, tdic_ctx** out);
void tdic_ctx_destroy(tdic_ctx* ctx);
/* The message of the context's last failure; with ctx == NULL, that of this thread's last failed
 * tdic_ctx_create ("null context" if none). */
const char* tdic_last_error(const tdic_ctx* ctx);
/* Bytes the pool holds on the device (allocated, live + cached). */
size_t tdic_ctx_device_bytes(const tdic_ctx* ctx);
/* The last heap-order propagation (propagation_mode 1) on this context: device rounds after
 * the dataflow pass, the solves they ran and the host time of the heap simulations
 * (host_sim_ms may be NULL).  No counterpart in the reference. */
tdic_status tdic_ctx_heap_stats(const tdic_ctx* ctx, int32_t* rounds, int64_t* solves, double* host_sim_ms);

/* Image pair on the device: the reference image (float32, as dic::Image stores it,
 * image.hpp:58-81) and the deformed image's B-spline coefficients of `degree` with `border`
 * (BSplineImagePreprocessor::compute, bspline.cpp:270-300 / form_coefficients :369-392;
 * exact_prefilter = 0 gives the clamp-padded, non-deconvolved coefficients of compute_lazy
 * used by seed refinement, seed_selector.cpp:166-173).  `reference`/`deformed` are host or
 * device pointers of `dtype` per `memory`, row-major H x W with row stride `pitch` elements
 * (0 = width).  Runs kernels K1 (prefilter) and the image conversion; async on `stream`. */
tdic_status tdic_pair_create(tdic_ctx* ctx, const void* reference, const void* deformed,
                             int32_t width, int32_t height, int32_t pitch, tdic_dtype dtype,
                             tdic_memory memory, int32_t degree, int32_t border,
                             int32_t exact_prefilter, int32_t precision, void* stream,
                             tdic_pair** out);
/* Recompute an existing pair from new images of the same shape (no allocation). */
tdic_status tdic_pair_update(tdic_pair* pair, const void* reference, const void* deformed,
                             int32_t pitch, tdic_dtype dtype, tdic_memory memory, void* stream);
/* Waits for the work enqueued on the pair through this library (on any stream), then frees it.
 * Work captured in a CUDA graph is not tracked: synchronise its stream after replaying first. */
void tdic_pair_destroy(tdic_pair* pair);
/* Copy the coefficient image ((H+2B) x (W+2B), float32 or float64 per the pair's precision)
 * into a host buffer of `bytes` bytes; for tests. */
tdic_status tdic_pair_coefficients(tdic_pair* pair, void* host_out, size_t bytes);
/* Copy the pair's float32 reference and deformed images (H x W each, what dic::Image holds:
 * integer pixels exactly, float64 pixels rounded to float32) into host buffers of W*H floats;
 * either pointer may be NULL; for tests. */
tdic_status tdic_pair_images(tdic_pair* pair, float* reference_out, float* deformed_out);

/* Reference-image gradients, kernel K2 (build_reference_gradient_cache,
 * reliability_propagation.cpp:84-112): central differences on raw pixels, one-sided at the
 * border.  gx/gy are host float64 arrays of H*W. */
tdic_status tdic_reference_gradient(tdic_pair* pair, double* gx, double* gy);

/* Batched per-POI solve: replaces SubsetSolver::solve_with_interpolators (subset_solver.hpp:
 * 39-65 -> icgn.cpp:384-405, forward_gauss_newton.cpp:117-142) for n POIs at once, on the
 * route of cfg: optimizer (0 ICGN, 1 FGN) x shape_order (1, 2) x criterion (1 ZNSSD, 0 SSD),
 * i.e. icgn.cpp:446-627, 832-988, 1168-1362, 1576-1739 and forward_gauss_newton.cpp:188-399,
 * 622-794, 1069-1297, 1540-1739.  in/out are host or device pointers per `memory`. */
tdic_status tdic_solve_pois(tdic_ctx* ctx, tdic_pair* pair, const tdic_config* cfg,
                            const tdic_poi_in* in, int32_t n, tdic_poi_out* out,
                            tdic_memory memory, void* stream);

/* Masked per-POI solve: replaces SubsetSolver::solve_with_mask (icgn.cpp:407-432,
 * forward_gauss_newton.cpp:144-170; the routes at icgn.cpp:629-818, 990-1154, 1364-1562,
 * 1741-1912 and forward_gauss_newton.cpp:401-604, 796-968, 1299-1522, 1741-1941).  roi: host
 * H x W mask of the pair's image (NULL = every pixel valid).  The centre must be a ROI pixel (no
 * margin check); samples outside the image or the ROI are left out, and at least
 * max(6 or 12, cfg->min_valid_samples, ceil(cfg->min_valid_sample_ratio * full circle)) must
 * remain (else status InvalidInput).  in/out as tdic_solve_pois. */
tdic_status tdic_solve_pois_masked(tdic_ctx* ctx, tdic_pair* pair, const tdic_config* cfg,
                                   const uint8_t* roi, const tdic_poi_in* in, int32_t n,
                                   tdic_poi_out* out, tdic_memory memory, void* stream);

/* recommended_subset_padding (src/subset/padding.cpp:28-36) when cfg->truncate_roi_subsets, else 0. */
int32_t tdic_subset_padding(const tdic_config* cfg);
/* Output grid of tdic_subset_compute: tdic_grid_dims, or with truncate_roi_subsets the grid of the
 * padded image restricted to points inside the image (subset_dic.cpp:92-104). */
void tdic_subset_grid_dims(int32_t width, int32_t height, const tdic_config* cfg, int32_t* grid_w,
                           int32_t* grid_h);

/* Propagation over the POI grid from one seed: replaces the heap loop of
 * ReliabilityPropagation::propagate (reliability_propagation.cpp:130-394).  With
 * cfg->truncate_roi_subsets every solve is masked by roi (NULL = all pixels); the images are
 * used as given (SubsetDIC::compute pads them first: tdic_subset_compute does).  The grid
 * geometry, seed alignment (:201-264), neighbour admission (:303-323), guess extrapolation
 * (:326-329) and acceptance rule (:359-368) are the reference's; the visit order is
 * cfg->propagation_mode:
 *   1  the reference's heap order (:270-389), with its results: rounds of a host simulation of
 *      the heap over a device result table and device solves of the points whose parent or
 *      guess changed, until the simulation meets no stale result (two or three rounds);
 *   2  dataflow (each point solved from its parent one step toward the seed as soon as that
 *      parent is accepted, the other axis's parent if it failed; unreached points swept by
 *      waves): one launch, the fastest; results differ from the heap order's at the
 *      convergence threshold's level, as the guesses come from other neighbours;
 *   0  frontier waves (every admissible neighbour of wave w's accepted set is solved in wave
 *      w+1 from the parent with the lowest ZNSSD, ties to the lowest parent index).
 * roi: host uint8 H x W mask (NULL = all valid).  out: host or device arrays per `memory`
 * of grid_w*grid_h entries.  *points_computed = accepted points including the seed (0 means
 * the seed could not be placed: SubsetDIC::compute then returns the empty result). */
tdic_status tdic_propagate(tdic_ctx* ctx, tdic_pair* pair, const tdic_config* cfg,
                           const tdic_seed* seed, const uint8_t* roi, tdic_grid_out* out,
                           tdic_memory memory, int32_t* points_computed, void* stream);

/* tdic_propagate without device allocation (no counterpart in the reference, whose CPU
 * propagation has nothing to allocate on a device).  For callers that cannot allocate device
 * memory at propagation time: a real-time loop that must not stall on cudaMalloc's device
 * synchronisation, or a process whose device memory belongs to another allocator.  The same
 * kernel runs with its scratch in one static device array of about 15.8 MiB per device,
 * which caps the call at 131072 grid points and 32768 subset samples (radius <= 100), and a
 * call with masked subsets (cfg->truncate_roi_subsets, solved as tdic_propagate solves them)
 * at 2^22 image pixels; larger calls fail with TDIC_INVALID_ARG.  out_device: device arrays
 * of grid_w*grid_h entries (NULL entries skipped); roi: host mask as for tdic_propagate.  The pair and the context are made
 * beforehand with the calls above, which do allocate.  The first call on a device looks up the
 * array's device address (set-up, once per device; under the driver's lazy module loading this
 * is also when the array's memory is committed on the device); make that first call before any
 * stream capture.  Every call on a device shares the array and finds the previous call's contents,
 * which it re-initialises; calls that overlapped on the GPU would race, so this entry point
 * holds a process-wide lock and waits for its stream before returning, also when it fails. */
tdic_status tdic_propagate_noalloc(tdic_ctx* ctx, tdic_pair* pair, const tdic_config* cfg,
                                   const tdic_seed* seed, const uint8_t* roi,
                                   const tdic_grid_out* out_device, int32_t* points_computed,
                                   void* stream);

/* Batched propagation: several image pairs in one persistent launch over a shared work queue
 * (no counterpart in the reference, which propagates one pair per SubsetDIC::compute call).
 * Job j propagates pairs[j] from seeds[j] with cfgs[j] exactly as tdic_propagate does in the
 * dataflow order (same results); subset radius, spacing, iterations, thresholds and ROI
 * (rois[j]: host H x W mask or NULL; rois may be NULL) may differ between jobs, the spline
 * degree, precision and optimizer may not; propagation_mode must be 2.  With
 * truncate_roi_subsets (in every job or in none) the solves are masked by each job's ROI, as
 * tdic_propagate's.  At most 512 jobs and 2^22 grid points per job.  The batch owns device outputs (tdic_batch_outputs) and scratch;
 * its pairs must outlive it.
 *   tdic_batch_tune    times each launch configuration (warps per POI, groups per block) on
 *                      this batch and keeps the fastest; optional (untuned, FP32 batches use
 *                      three 4-warp groups per block, one block per SM: the single-pair shape).
 *   tdic_batch_launch  enqueues one propagation of every job on `stream` and returns without
 *                      waiting: device memsets and kernel launches only, so it can be captured
 *                      in a CUDA graph and replayed (synchronise the replay stream before
 *                      destroying the batch or its pairs: replays are not tracked).
 *   tdic_batch_finish  waits for `stream` and reports points_computed[j] (0: the seed of job j
 *                      could not be placed, its grid holds the defaults). */
typedef struct tdic_batch tdic_batch;
tdic_status tdic_batch_create(tdic_ctx* ctx, int32_t n, tdic_pair* const* pairs,
                              const tdic_config* cfgs, const tdic_seed* seeds,
                              const uint8_t* const* rois, void* stream, tdic_batch** out);
tdic_status tdic_batch_tune(tdic_batch* batch, void* stream);
tdic_status tdic_batch_launch(tdic_batch* batch, void* stream);
tdic_status tdic_batch_finish(tdic_batch* batch, void* stream, int32_t* points_computed);
/* Device arrays (grid_w*grid_h entries each) of job j's results; valid until the batch is
 * destroyed, rewritten by every launch. */
tdic_status tdic_batch_outputs(tdic_batch* batch, int32_t job, tdic_grid_out* device_arrays);
/* Copy job j's grid into host arrays (NULL entries skipped); waits for `stream`. */
tdic_status tdic_batch_results(tdic_batch* batch, int32_t job, const tdic_grid_out* host_arrays, void* stream);
/* Launch the batch on `sms` SMs' worth of thread blocks (0 = the whole device; default).  The
 * propagation holds its SMs for its whole duration, so leaving some free lets kernels on other
 * streams (the preparation of the next requests in a serving loop) run alongside it. */
tdic_status tdic_batch_set_sms(tdic_batch* batch, int32_t sms);
/* The launch configuration in use: warps per POI, solver groups per thread block and the
 * shared-memory staging (tdic_staging; staging may be NULL). */
tdic_status tdic_batch_config(tdic_batch* batch, int32_t* warps_per_poi, int32_t* groups_per_block,
                              int32_t* staging);
void tdic_batch_destroy(tdic_batch* batch);

/* Seed selection: SeedSelector::select_best_seed (seed_selector.cpp:146-205) with k-means
 * candidates (:207-317), integer search (integer_search.cpp:333-432, kernel K5) and subpixel
 * ICGN refinement on the non-prefiltered spline (subset_initializer.cpp:152-204).  `lazy` is
 * a pair created with exact_prefilter = 0 over the same images; reference_host is the host
 * float32 reference (texture statistics).  seed->found = 0 when no candidate passes. */
tdic_status tdic_select_seed(tdic_ctx* ctx, tdic_pair* lazy, const float* reference_host,
                             const uint8_t* roi, const tdic_config* cfg, tdic_seed* seed,
                             void* stream);

/* Integer search: IntegerSearchInitializer::estimate (integer_search.cpp:333-432, kernel K5) at
 * n integer points (x[i], y[i]) of the pair's reference, searching its deformed image (the
 * pair's float32 images; either prefilter): the pyramid (multigrid) stage, the full-sample
 * refinement around its optimum, the local +-search window and the local-preference rule.
 * Out, per point: the integer displacement (u, v), its ZNCC (FP64, rounded as the reference's)
 * and ok = 0 where the reference returns no estimate.  With cfg->truncate_roi_subsets the
 * masked search over roi (host H x W mask; every pixel when NULL), as seed selection uses it.
 * At most 65535 points per call (TDIC_INVALID_ARG beyond). */
tdic_status tdic_integer_search(tdic_ctx* ctx, tdic_pair* pair, const tdic_config* cfg,
                                const int32_t* x, const int32_t* y, int32_t n, const uint8_t* roi,
                                double* u, double* v, double* zncc, uint8_t* ok, void* stream);

/* SubsetDIC::compute up to the propagation (subset_dic.cpp:39-64): creates the pair from host
 * images (as tdic_pair_create with the exact prefilter) and selects its seed (as
 * tdic_select_seed, on a seed spline built from the uploaded images; texture statistics on the
 * raw host images).  The caller propagates (tdic_propagate, or one job of a tdic_batch) and
 * destroys *pair_out.  seed_out->found = 0 means SubsetDIC::compute's empty result.
 * With cfg->truncate_roi_subsets the pair is the padded one tdic_subset_compute works on: both
 * images mirror-padded by pad = tdic_subset_padding(cfg) on every side (float32, (width + 2 pad)
 * x (height + 2 pad)), the seed in padded coordinates.  Propagate it with the padded ROI (0 in
 * the padding, roi or all ones inside) and keep the grid points with 0 <= x - pad < width and
 * 0 <= y - pad < height, shifted back by pad: tdic_subset_compute's result. */
tdic_status tdic_subset_prepare(tdic_ctx* ctx, const void* reference, const void* deformed,
                                int32_t width, int32_t height, tdic_dtype dtype,
                                const uint8_t* roi, const tdic_config* cfg, void* stream,
                                tdic_pair** pair_out, tdic_seed* seed_out);

/* Least-squares strain of 2D point displacements: dic::compute_least_squares_strain_2d
 * (src/postprocess/least_squares_strain.cpp:11-78), as bound by
 * _traditional_dic.postprocess.compute_least_squares_strain_2d.  points, displacement: host
 * arrays of n (x, y) / (u, v) pairs; neighbours within `radius` (the point included) give a plane
 * fit of u and v; green_lagrange != 0 gives E = (H + H^T + H^T H) / 2, else the small strain.
 * Points or displacements that are not finite are left out (valid = 0, sample_count = 0).
 * TDIC_INVALID_ARG unless radius > 0 and min_samples >= 3 (the reference's check). */
typedef struct tdic_ls_strain {
    double du_dx, du_dy, dv_dx, dv_dy;
    double exx, eyy, exy;
    int32_t sample_count;
    uint8_t valid;
    uint8_t pad_[3];
} tdic_ls_strain;
tdic_status tdic_ls_strain_2d(tdic_ctx* ctx, const double* points, const double* displacement,
                              int32_t n, double radius, int32_t min_samples, int32_t green_lagrange,
                              tdic_ls_strain* out, void* stream);

/* The displacement CSV of the subset workflow, save_subset_csv
 * (python/traditional_dic/workflows/subset_2d.py:34-54), byte for byte: the header
 * "x,y,u,v,du_dx,du_dy,dv_dx,dv_dy,correlation,valid", then one row per grid point with each
 * float64 as Python's str() writes it (shortest round-trip digits; positional for decimal
 * exponents -4 .. 15, else scientific) and valid as 0 or 1, CRLF line ends as csv.writer ends
 * them.  grid: the arrays x .. correlation and valid of n points, host or device per `memory`
 * (device arrays are read straight from the device); formatted on every host thread.  ctx may
 * be NULL for host arrays (no device is touched; tdic_last_error(NULL) then holds a failure's
 * message). */
tdic_status tdic_write_subset_csv(tdic_ctx* ctx, const char* path, const tdic_grid_out* grid, tdic_memory memory,
                                  int32_t n);

/* Whole pybind path: _traditional_dic.subset.compute (bind_subset.cpp:253-315) ->
 * SubsetDIC::compute (subset_dic.cpp:39-105).  Host images of `dtype`, host roi (NULL = full
 * image), host outputs of grid_w*grid_h entries (tdic_subset_grid_dims).  *n_points =
 * grid_w*grid_h, or 0 for the reference's empty result (no seed found, or nothing computed).
 * With cfg->truncate_roi_subsets (masked subsets; x and y outputs required) the images are padded
 * as SubsetDIC::compute pads them, the grid points are gx * step - pad, and seed_out is in image
 * coordinates. */
tdic_status tdic_subset_compute(tdic_ctx* ctx, const void* reference, const void* deformed,
                                int32_t width, int32_t height, tdic_dtype dtype,
                                const uint8_t* roi, const tdic_config* cfg, tdic_grid_out* out,
                                int32_t* n_points, tdic_seed* seed_out, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* TDIC_GB300_H */
