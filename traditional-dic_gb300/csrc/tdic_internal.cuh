// Internal declarations shared by the translation units of libtdic_gb300.so.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/tdic_gb300.h"

namespace tdic {

// ---------------------------------------------------------------------------------------
// Errors: every CUDA call is checked; the first failure is recorded on the context and
// turned into a tdic_status.  Nothing throws across the C ABI.
// ---------------------------------------------------------------------------------------
struct Error {
    tdic_status code;
    std::string msg;
};

#define TDIC_CUDA_TRY(expr)                                                                  \
    do {                                                                                     \
        cudaError_t e_ = (expr);                                                             \
        if (e_ != cudaSuccess) {                                                             \
            (void)cudaGetLastError(); /* a non-sticky error must not surface in a later call */ \
            throw ::tdic::Error{TDIC_CUDA_ERROR, std::string(#expr) + ": " + cudaGetErrorString(e_)}; \
        }                                                                                    \
    } while (0)

#define TDIC_REQUIRE(cond, code, text)                                                       \
    do {                                                                                     \
        if (!(cond)) throw ::tdic::Error{(code), (text)};                                    \
    } while (0)

// ---------------------------------------------------------------------------------------
// Caching device-memory pool: blocks are kept after release and reused by size class, so a
// steady stream of pairs / propagations does no cudaMalloc after warm-up.
// ---------------------------------------------------------------------------------------
class DevicePool {
public:
    void* acquire(size_t bytes);
    void release(void* p);
    void trim();
    size_t held_bytes() const { return held_; }
    ~DevicePool() { trim(); }

private:
    static size_t size_class(size_t bytes);
    std::multimap<size_t, void*> free_;
    std::map<void*, size_t> live_;
    size_t held_ = 0;
};

struct Buffer {
    DevicePool* pool = nullptr;
    void* ptr = nullptr;
    size_t bytes = 0;
    Buffer() = default;
    Buffer(DevicePool* p, size_t b) : pool(p), ptr(b ? p->acquire(b) : nullptr), bytes(b) {}
    Buffer(const Buffer&) = delete;
    Buffer& operator=(const Buffer&) = delete;
    Buffer(Buffer&& o) noexcept { *this = std::move(o); }
    Buffer& operator=(Buffer&& o) noexcept {
        reset();
        pool = o.pool; ptr = o.ptr; bytes = o.bytes;
        o.ptr = nullptr; o.bytes = 0;
        return *this;
    }
    ~Buffer() { reset(); }
    void reset() {
        if (ptr && pool) pool->release(ptr);
        ptr = nullptr;
        bytes = 0;
    }
    template <typename T> T* as() const { return static_cast<T*>(ptr); }
};

// Circular-subset sample offsets (dx, dy) in the reference's row-major order
// (icgn.cpp:484-510: dy outer, dx inner, dx^2 + dy^2 <= r^2), one table per radius.
struct SampleTable {
    Buffer offsets;  // short2[n]
    int n = 0;
};

}  // namespace tdic

struct tdic_ctx {
    int device = 0;
    int num_sms = 0;
    int max_smem_optin = 0;  // dynamic shared memory a CTA may opt in to
    int* dev_err = nullptr;  // device error flag of bounded in-kernel waits (0 = none)
    cudaStream_t stream = nullptr;
    std::recursive_mutex mu;
    std::string last_error;
    tdic::DevicePool pool;
    std::map<int, tdic::SampleTable> tables;
    // Pairs hold device memory of this context's pool: the context outlives its pairs.
    // tdic_ctx_destroy with live pairs only marks the context; the last tdic_pair_destroy frees it.
    int live_pairs = 0;
    bool destroy_requested = false;
    // the last heap-order propagation: device rounds after the dataflow pass, and solves in them
    int heap_rounds = 0;
    long long heap_solves = 0;
    double heap_sim_ms = 0.0;  // host time in the heap simulations
    // the set-up precompute order of the last grid and seed (grid points by distance from it)
    tdic::Buffer pre_order;
    int pre_key[3] = {-1, -1, -1};
    int pre_count = 0;
};

struct tdic_pair {
    tdic_ctx* ctx = nullptr;
    int w = 0, h = 0, border = 3, degree = 3, precision = 0, exact = 1;
    int cw = 0, ch = 0;        // coefficient image size (w + 2B) x (h + 2B)
    int rpitch = 0;            // floats per row of ref / def_f (128-byte multiple: TMA row stride)
    int cpitch = 0;            // elements per row of coef (128-byte multiple)
    tdic::Buffer ref;          // float32 H x W reference, row pitch rpitch (dic::Image stores float)
    tdic::Buffer coef;         // T coefficients of the deformed image, ch rows of cpitch
    tdic::Buffer def_f;        // float32 H x W deformed, row pitch rpitch (seed search, lazy pairs)
    tdic::Buffer staging;      // raw input staging for host uploads (reference, then deformed)
    cudaEvent_t last_use = nullptr;  // recorded after the last work enqueued on the pair
    ~tdic_pair() {
        if (last_use) cudaEventDestroy(last_use);
    }
};

namespace tdic {

// B-spline local polynomial matrix qk (bspline.cpp:320-340) for degree 1, 3, 5.
void build_qk(int degree, double* qk);

const SampleTable& sample_table(tdic_ctx* ctx, int radius);

// True while `s` is being captured into a CUDA graph: captured work runs only when the graph
// is replayed, so it is not tracked by the last-use events.
inline bool capturing(cudaStream_t s) {
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    TDIC_CUDA_TRY(cudaStreamIsCapturing(s, &st));
    return st != cudaStreamCaptureStatusNone;
}

// Mark the pair as used by the work enqueued so far on `s` (its destruction waits for it).
inline void mark_use(tdic_pair* p, cudaStream_t s) {
    if (p && p->last_use && !capturing(s)) TDIC_CUDA_TRY(cudaEventRecord(p->last_use, s));
}

// Kernel launchers (prefilter.cu) --------------------------------------------------------
void launch_convert(const void* src, int w, int h, int pitch, tdic_dtype dtype, float* dst, int dst_pitch,
                    cudaStream_t s);
void launch_prefilter(tdic_pair* pair, const float* image, cudaStream_t s);
void launch_pair_setup(tdic_pair* pair, const void* ref, const void* def, int pitch, tdic_dtype dtype,
                       cudaStream_t s);
void launch_reference_gradient(const float* img, int w, int h, int pitch, double* gx, double* gy, cudaStream_t s);

// Hot path (hotpath.cu) -------------------------------------------------------------------
struct SolveLaunch {
    const tdic_poi_in* in;
    tdic_poi_out* out;
    int n;
    int* fetch;  // work counter (zeroed by the launcher)
    // masked subsets (solve_with_mask): device ROI of the pair's image (w x h bytes), or NULL
    const uint8_t* roi = nullptr;
};
void launch_solve(tdic_ctx* ctx, tdic_pair* pair, const tdic_config& cfg, const SolveLaunch& L, cudaStream_t s);
// Throws TDIC_TIMEOUT when a bounded in-kernel wait gave up; clears the flag.  Synchronises s.
void check_device_error(tdic_ctx* ctx, cudaStream_t s);

struct PropagateLaunch {
    int gw, gh, step;
    const uint8_t* roi_grid;   // gw*gh admission by ROI at grid points (1 = valid)
    // seed
    int seed_idx;              // grid index of the aligned seed
    int seed_solve;            // 1 when the aligned point differs from the raw seed
    double seed_p[6];
    double seed_corr;
    // outputs (device SoA; NULL entries skipped)
    tdic_grid_out out;
    // scratch
    int* claim; unsigned long long* key; void* params; int* order; int* counters; int* fetch;
    unsigned int* barrier;  // [count, generation]
    int* flags;             // [error, no_seed, accepted]
    // dataflow order (propagation_mode 2)
    int mode;
    int sgx, sgy;
    int* dstate; int* dcnt; unsigned long long* dq; float* kcorr;
    // subset sample offsets; NULL = the context's table for the radius
    const short2* offsets; int n_offsets;
    // masked subsets (truncate_roi_subsets): device ROI of the pair's image (w x h bytes), or NULL
    const uint8_t* roi_px = nullptr;
    // a round of the heap order (mode 3): the tree of this round, the result table
    const int* tchild_off = nullptr; const int* tchild = nullptr; const int* tcont = nullptr;
    // set-up cache of the grid (first-order ZNSSD ICGN; see Env::sc_*) and the order in which
    // idle solver groups fill it, with its ticket counter (zeroed by the caller); NULL = none
    void* sc_hinv = nullptr; void* sc_fmn = nullptr; int* sc_state = nullptr;
    const int* pre_order = nullptr; int pre_count = 0; int* pre_ticket = nullptr;
    void* rcorr = nullptr; void* rq = nullptr; unsigned char* rmeta = nullptr; int* riters = nullptr;
};
void launch_propagate(tdic_ctx* ctx, tdic_pair* pair, const tdic_config& cfg, const PropagateLaunch& L,
                      cudaStream_t s);

// The set-up cache of a propagation grid (first-order ZNSSD ICGN without masked subsets): per
// grid point the reference side of the solve, filled by idle solver groups ahead of the solves
// and by every solve that computes it.  setup_cache_prepare sizes it in the pair's precision,
// zeroes its states and ticket on `s` and sets the fields of L (the precompute order, grid
// points by Manhattan distance from the seed, is kept by the context for the next call).
struct SetupCache {
    Buffer hinv, fmn, state, ticket;
};
inline bool setup_cache_applies(const tdic_config& c) {
    return c.optimizer == 0 && c.shape_order == 1 && c.criterion == 1 && !c.truncate_roi_subsets;
}
void setup_cache_prepare(tdic_ctx* ctx, tdic_pair* pair, int gw, int gh, int sgx, int sgy, SetupCache& c,
                         PropagateLaunch& L, cudaStream_t s);
size_t propagate_param_bytes(int precision);
void launch_init_grid(const tdic_grid_out& out, int gw, int gh, int step, cudaStream_t s);
// Outputs of a heap-order propagation from its result table (parameters and correlations in the
// pair's precision) and the host's acceptance flags (heap_order.cu).
void launch_emit_tree(const tdic_grid_out& out, int gw, int gh, int step, int precision, const void* params,
                      const void* rcorr, const void* rq, const unsigned char* rmeta, const int* riters,
                      const unsigned char* accepted, cudaStream_t s);
// ReliabilityPropagation::propagate in the reference's own heap order on the device
// (heap_order.cu); the arguments of propagate_impl.
void heap_propagate(tdic_ctx* ctx, tdic_pair* pair, const tdic_config& cfg, const tdic_seed& seed,
                    const uint8_t* roi, const tdic_grid_out& out_dev, int32_t* points_computed, cudaStream_t s);

// Seed search (seed.cu) -------------------------------------------------------------------
struct SearchResult { int u, v; double zncc; int ok; };
// Nearest-centre assignment of k-means (run_kmeans, seed_selector.cpp:69-104) on the device:
// assign[i] = the lowest-index centre at the smallest squared distance from point i.
class KmeansAssigner {
public:
    KmeansAssigner(tdic_ctx* ctx, const int* px, const int* py, int m, int k, cudaStream_t s);
    void assign(const double* cx, const double* cy, int* assign_host);
    // `iters` whole iterations (assignment, sums, new centres) on the device, one sync at the end;
    // the same centres as assign() plus the host sums in point order (the sums are exact).
    void run(double* cx, double* cy, int iters);
private:
    tdic_ctx* ctx_;
    cudaStream_t s_;
    int m_, k_;
    float cbound_ = 0.0f;  // above every |coordinate| of the points
    float kabs_ = 0.0f;    // the FP32 filter's absolute error term
    int filter_ = 0;       // the FP32 distance filter applies (coordinates below 2^22)
    Buffer pts_, ctr_, ctr32_, out_, acc_;
};
// roi (host mask of the pair's image, or NULL): the masked search of truncate_roi_subsets.
void integer_search_batch(tdic_ctx* ctx, tdic_pair* lazy, const tdic_config& cfg, const int* cx, const int* cy,
                          int n, SearchResult* out, cudaStream_t s, const uint8_t* roi = nullptr);

// The subset workflow's displacement CSV (results.cpp) from host or device arrays.
void write_subset_csv(const char* path, const tdic_grid_out& grid, tdic_memory memory, int32_t n);

// Least-squares strain (strain.cu).
void ls_strain_2d(tdic_ctx* ctx, const double* points, const double* disp, int n, double radius, int min_samples,
                  int green, tdic_ls_strain* out, cudaStream_t s);

// Batched propagation (several image pairs in one persistent launch).  Grid points of a batch
// are tagged with their job in queue items: 22 bits of point, the job above.
constexpr int kMaxBatchJobs = 512;
struct BatchSeed {
    int ok;            // the seed is placed (reliability_propagation.cpp:201-216)
    int idx, gx, gy;   // aligned grid point
    int solve;         // 1 when the aligned point differs from the raw seed
    double p[6];
    double corr;
};
// A batch plan of one precision (batch.cu is compiled once per precision).
struct BatchPlanBase {
    virtual ~BatchPlanBase() = default;
    virtual int config_count() const = 0;
    // warps per POI, groups per block, tdic_staging of launch configuration `config`
    virtual void config_info(int config, int* warps_per_poi, int* groups_per_block, int* staging) const = 0;
    virtual void launch(int config, cudaStream_t s) = 0;
    virtual void finish(int32_t* computed, int* err, cudaStream_t s) = 0;
    virtual tdic_grid_out outputs(int job) const = 0;
    virtual void grid(int job, int32_t* gw, int32_t* gh) const = 0;
    virtual void set_sms(int sms) = 0;
};
// plan builders of the four batch units (precision x plain / masked-subset route)
#define TDIC_BATCH_BUILDER(name)                                                                              \
    std::unique_ptr<BatchPlanBase> name(tdic_ctx* ctx, int n, tdic_pair* const* pairs, const tdic_config* cfgs, \
                                        const BatchSeed* seeds, const std::vector<std::vector<uint8_t>>& rois,  \
                                        cudaStream_t s);
TDIC_BATCH_BUILDER(batch_build_f32)
TDIC_BATCH_BUILDER(batch_build_f64)
TDIC_BATCH_BUILDER(batch_build_f32_masked)
TDIC_BATCH_BUILDER(batch_build_f64_masked)
#undef TDIC_BATCH_BUILDER
inline std::unique_ptr<BatchPlanBase> batch_build(tdic_ctx* ctx, int n, tdic_pair* const* pairs,
                                                  const tdic_config* cfgs, const BatchSeed* seeds,
                                                  const std::vector<std::vector<uint8_t>>& rois, cudaStream_t s) {
    const bool fp64 = pairs[0]->precision == TDIC_FP64;
    if (cfgs[0].truncate_roi_subsets)
        return fp64 ? batch_build_f64_masked(ctx, n, pairs, cfgs, seeds, rois, s)
                    : batch_build_f32_masked(ctx, n, pairs, cfgs, seeds, rois, s);
    return fp64 ? batch_build_f64(ctx, n, pairs, cfgs, seeds, rois, s)
                : batch_build_f32(ctx, n, pairs, cfgs, seeds, rois, s);
}
inline int batch_config_count(BatchPlanBase* p) { return p->config_count(); }
inline void batch_config_info(BatchPlanBase* p, int config, int* warps_per_poi, int* groups_per_block, int* staging) {
    p->config_info(config, warps_per_poi, groups_per_block, staging);
}
inline void batch_launch(BatchPlanBase* p, int config, cudaStream_t s) { p->launch(config, s); }
inline void batch_finish(BatchPlanBase* p, int32_t* computed, int* err, cudaStream_t s) { p->finish(computed, err, s); }
inline tdic_grid_out batch_outputs(BatchPlanBase* p, int job) { return p->outputs(job); }
inline void batch_grid(BatchPlanBase* p, int job, int32_t* gw, int32_t* gh) { p->grid(job, gw, gh); }
inline void batch_set_sms(BatchPlanBase* p, int sms) { p->set_sms(sms); }

}  // namespace tdic
