/*
 * tdic_oracle.h -- FP64 CPU restatement of the Traditional-DIC 2D subset-DIC hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity checker for the GB300 CUDA path and
 * the timed CPU baseline ("port") of bench.py.  Nothing in the product links, loads or calls
 * it; only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg do.
 *
 * Every function restates a function of the reference (lbd-hfut/Traditional-DIC); the
 * reference file:line is given beside each declaration and again in tdic_oracle.cpp.  The
 * reference itself cannot be compiled here: every hot-path file includes <Eigen/Dense> and
 * <unsupported/Eigen/FFT>, and Eigen 3.4 (cmake/Dependencies.cmake:3-14, fetched from the
 * network) is absent.  Parity of this restatement is pinned by (a) a numpy transcription of
 * the reference's FFT deconvolution (bspline.cpp:191-244), (b) a numpy transcription of the
 * reference's local polynomial block evaluation (bspline.cpp:96-175, 320-340), (c) analytic
 * known-answer tests (linear-image reproduction, pure translation / affine recovery),
 * (d) numpy.linalg for the 6x6 solves and (e) golden vectors (tests/golden/subset_icgn_256.npz)
 * from an independent numpy transcription of the prefilter and of solve_first_order_znssd
 * (tests/golden/make_golden.py), which this library reproduces to 1e-10 (coefficients) and
 * 1e-8 px (per-POI parameters, identical iteration counts and statuses).  No reference-produced
 * golden vectors exist for this path (tests/data/f0/subset_ring/baseline.npz is missing from
 * the reference checkout) and the reference cannot be run here, so parity at the level of
 * Eigen's LDLT / kissfft rounding (~1e-15 relative) is unpinned.
 */
#ifndef TDIC_ORACLE_H
#define TDIC_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Reachable knobs of dic::SubsetConfig (subset_config.hpp:33-50, seed_config.hpp:32-68,
 * bspline.hpp:42-67) with the C++ defaults; the field order matches tdic_config in
 * include/tdic_gb300.h so one ctypes structure serves both libraries. */
typedef struct orc_config {
    int32_t subset_radius;             /* 15 */
    int32_t max_iterations;            /* 30 */
    double convergence_threshold;      /* 1e-3 */
    int32_t optimizer;                 /* 0 = ICGN, 1 = forward Gauss-Newton */
    int32_t shape_order;               /* 1 (2 = second order) */
    int32_t criterion;                 /* 1 = ZNSSD, 0 = SSD */
    int32_t degree;                    /* 5 (1, 3, 5) */
    int32_t border;                    /* 3 (raised to >= 3) */
    int32_t propagation_spacing;       /* 5 (gap count; stride = spacing + 1) */
    double propagation_max_znssd;      /* 0.5 */
    int32_t is_subset_radius;          /* 10 */
    int32_t is_search_radius;          /* 30 */
    int32_t sift_enabled;              /* 0 */
    int32_t pyramid_enabled;           /* 1 */
    int32_t pyramid_scale;             /* 4 */
    int32_t pyramid_refinement_radius; /* 4 */
    int32_t sp_enabled;                /* 1 */
    int32_t sp_subset_radius;          /* 15 */
    int32_t sp_max_iterations;         /* 30 */
    int32_t precision;                 /* product-only knob (0 FP32-mixed, 1 FP64); unused here */
    double sp_convergence_threshold;   /* 1e-3 */
    int32_t seed_count;                /* 256 */
    int32_t kmeans_iterations;         /* 20 */
    double seed_max_znssd;             /* 0.2 */
    double min_displacement_norm;      /* 0 */
    double min_texture_std;            /* 0 */
    int32_t kmeans_sample_limit;       /* 20000 */
    int32_t propagation_mode;          /* 1 = reliability-guided heap order (reference, default), 0 = frontier waves,
                                          2 = dataflow (axis parents toward the seed) + frontier-wave cleanup */
    int32_t truncate_roi_subsets;      /* subset.truncate_roi_subsets (YAML only)        0 */
    int32_t min_valid_samples;         /* subset.min_valid_samples                       12 */
    double min_valid_sample_ratio;     /* subset.min_valid_sample_ratio                 0.5 */
    int32_t staging;                   /* product-only knob (shared-memory staging); unused here */
    int32_t pad_;
} orc_config;

/* Per-POI solver result; mirrors dic::Displacement2D (result.hpp:32-51) plus the additive
 * fields iterations / converged.  status uses dic::SolverStatus ordinals (types.hpp:35-40):
 * 0 Success, 1 NotConverged, 2 InvalidInput, 3 NumericalFailure. */
typedef struct orc_poi_result {
    double p[6];          /* u, v, du_dx, du_dy, dv_dx, dv_dy */
    double correlation;   /* ZNSSD (SSD) at the pre-update parameters of the last iteration */
    int32_t iterations;   /* loop bodies entered */
    int8_t status;
    int8_t valid;
    int8_t converged;     /* strict: |dp| < threshold was reached */
    int8_t pad_;
    double q[6];          /* second order: d2u_dx2, d2u_dxdy, d2u_dy2, d2v_dx2, d2v_dxdy, d2v_dy2 (else 0) */
} orc_poi_result;

/* Structure-of-arrays grid output (bind_subset.cpp:102-153 plus additive keys). */
typedef struct orc_grid_out {
    double* x; double* y; double* u; double* v;
    double* du_dx; double* du_dy; double* dv_dx; double* dv_dy;
    double* correlation;
    uint8_t* valid; int8_t* status; int32_t* iterations; uint8_t* converged;
    /* second-order terms (Displacement2D d2u_dx2 ... d2v_dy2); NULL = not written */
    double* d2u_dx2; double* d2u_dxdy; double* d2u_dy2; double* d2v_dx2; double* d2v_dxdy; double* d2v_dy2;
} orc_grid_out;

/* Seed placed by the seed selector (seed_selector.cpp:146-205). */
typedef struct orc_seed {
    double x, y;
    double p[6];
    double correlation;
    int32_t found;
    int32_t pad_;
} orc_seed;

void orc_config_default(orc_config* cfg);

/* bspline.cpp:342-367 */
double orc_bspline_basis(double x, int derivative_order, int degree);
/* bspline.cpp:320-340; qk is (degree+1)^2 row-major */
int orc_bspline_qk(int degree, double* qk);
/* bspline.cpp:369-392 (+177-244): exact = 1 -> half-sample symmetric pad by border and periodic
 * deconvolution of rows then columns; exact = 0 -> clamp pad, no deconvolution.
 * coeffs is (h + 2*border) x (w + 2*border) row-major.  Returns 0 on success. */
int orc_prefilter(const float* image, int w, int h, int degree, int border, int exact, double* coeffs);
/* bspline.cpp:458-474 and 476-500 through the local polynomial block of bspline.cpp:153-175 */
double orc_interp_value(const double* coeffs, int w, int h, int degree, int border, double x, double y);
void orc_interp_gradient(const double* coeffs, int w, int h, int degree, int border,
                         double x, double y, double* gx, double* gy);
/* reliability_propagation.cpp:84-112 */
void orc_reference_gradient(const float* image, int w, int h, double* gx, double* gy);

/* ICGNSolver (optimizer 0) / ForwardGaussNewtonSolver (optimizer 1) ::solve_with_interpolators
 * for each POI, routed on shape_order (1, 2) and criterion (1 ZNSSD, 0 SSD): icgn.cpp:446-627,
 * 832-988, 1168-1362, 1576-1739; forward_gauss_newton.cpp:188-399, 622-794, 1069-1297,
 * 1540-1739.  ref_gx/ref_gy may be NULL (central differences on the fly, icgn.cpp:42-53).
 * confidence0 may be NULL (initial.confidence = 0).  Returns 0, or -1 for a bad degree. */
int orc_solve_pois(const float* ref, int w, int h, const double* ref_gx, const double* ref_gy,
                   const double* coeffs, int degree, int border, const orc_config* cfg,
                   int n, const double* xy, const double* p0, const double* confidence0,
                   orc_poi_result* out);
/* solve_with_mask (icgn.cpp:407-432, forward_gauss_newton.cpp:144-170): the masked routes
 * (icgn.cpp:629-818, 990-1154, 1364-1562, 1741-1912; forward_gauss_newton.cpp:401-604, 796-968,
 * 1299-1522, 1741-1941) over the ROI mask `roi` (h x w, NULL = every pixel valid). */
int orc_solve_pois_masked(const float* ref, int w, int h, const uint8_t* roi, const double* ref_gx,
                          const double* ref_gy, const double* coeffs, int degree, int border,
                          const orc_config* cfg, int n, const double* xy, const double* p0,
                          const double* confidence0, orc_poi_result* out);

void orc_grid_dims(int w, int h, int spacing, int* grid_w, int* grid_h);

/* reliability_propagation.cpp:130-394 with one seed; roi may be NULL (all valid).
 * coeffs are the prefiltered deformed coefficients, ref_gx/ref_gy the gradient cache.
 * Returns points_computed (0 means the seed could not be placed). */
int orc_propagate(const float* ref, int w, int h, const uint8_t* roi,
                  const double* ref_gx, const double* ref_gy, const double* coeffs,
                  const orc_config* cfg, const orc_seed* seed, int max_solves, orc_grid_out* out,
                  int* solves_done);
/* orc_propagate with the points of each frontier wave (propagation_mode 0) or dataflow diagonal
 * (mode 2) solved on `threads` host threads; the heap order (mode 1) stays serial.  The output
 * does not depend on `threads`. */
int orc_propagate_threads(const float* ref, int w, int h, const uint8_t* roi,
                          const double* ref_gx, const double* ref_gy, const double* coeffs,
                          const orc_config* cfg, const orc_seed* seed, int max_solves,
                          orc_grid_out* out, int* solves_done, int threads);

/* integer_search.cpp:333-432 */
int orc_integer_search(const float* ref, const float* def, int w, int h, const orc_config* cfg,
                       double px, double py, double* u, double* v, double* zncc);
/* estimate_with_mask_interpolators (integer_search.cpp:447-545) over the ROI `roi` (h x w). */
int orc_integer_search_masked(const float* ref, const float* def, int w, int h, const uint8_t* roi,
                              const orc_config* cfg, double px, double py, double* u, double* v,
                              double* zncc);
/* seed_selector.cpp:146-317 with sift disabled; candidates (x,y) pairs are written to
 * cand_xy (capacity cand_cap) when non-NULL. */
int orc_select_seed(const float* ref, const float* def, int w, int h, const uint8_t* roi,
                    const orc_config* cfg, orc_seed* seed, double* cand_xy, int cand_cap,
                    int* n_candidates);
/* subset_dic.cpp:39-105 + bind_subset.cpp:253-315: returns the number of output points
 * (grid_w*grid_h) or 0 for the empty result.  With truncate_roi_subsets the images are
 * mirror-padded and the ROI zero-padded by recommended_subset_padding (src/subset/padding.cpp:28-36),
 * the grid is laid over the padded image and only its points inside the original image are
 * written, shifted back (subset_dic.cpp:53-104): size `out` for orc_truncated_grid_dims. */
int orc_subset_compute(const float* ref, const float* def, int w, int h, const uint8_t* roi,
                       const orc_config* cfg, orc_grid_out* out, orc_seed* seed_out);
/* recommended_subset_padding (padding.cpp:28-36) and the grid of the padded image. */
int orc_subset_padding(const orc_config* cfg);
void orc_truncated_grid_dims(int w, int h, const orc_config* cfg, int* grid_w, int* grid_h);

#ifdef __cplusplus
}
#endif
#endif
