// The batched propagation (several image pairs in one persistent launch, first-order ZNSSD):
// its plan, launch configurations and launches.  Compiled once per precision
// (-DTDIC_BATCH_FP64=0: FP32-mixed, 1: FP64) and solver route (-DTDIC_BATCH_VAR=0: plain, 4:
// masked subsets) so the four sets of batch kernels build side by side with the single-pair
// kernels of hotpath.cu.
#include "hotpath.cuh"

#ifndef TDIC_BATCH_FP64
#error "compile with -DTDIC_BATCH_FP64=0 or 1"
#endif
#ifndef TDIC_BATCH_VAR
#error "compile with -DTDIC_BATCH_VAR=0 or 4"
#endif

namespace tdic {

namespace {

#if TDIC_BATCH_FP64
using BatchT = double;
#else
using BatchT = float;
#endif
constexpr int kBatchVar = TDIC_BATCH_VAR;

// tdic_staging of a kernel staging mode
int staging_code(int stage) {
    return (stage & kStageLean) ? ((stage & kStageNoCoefWindow) ? TDIC_STAGING_LEAN_NO_WINDOW : TDIC_STAGING_LEAN)
                                : TDIC_STAGING_FULL;
}

template <typename T, int VAR>
int BatchPlan<T, VAR>::config_count() const {
    return static_cast<int>(configs.size());
}

template <typename T, int VAR>
void BatchPlan<T, VAR>::config_info(int config, int* warps_per_poi, int* groups_per_block, int* staging) const {
    *warps_per_poi = configs[config].G;
    *groups_per_block = configs[config].gpb;
    *staging = staging_code(configs[config].stage);
}

template <typename T, int VAR>
void BatchPlan<T, VAR>::launch(int config, cudaStream_t s) {
    batch_plan_launch(*this, config, s);
}

template <typename T, int VAR>
void BatchPlan<T, VAR>::finish(int32_t* computed, int* err, cudaStream_t s) {
    std::vector<int> flags(4 * static_cast<size_t>(n));
    int e = 0;
    TDIC_CUDA_TRY(cudaMemcpyAsync(flags.data(), d_flags.ptr, sizeof(int) * flags.size(), cudaMemcpyDeviceToHost, s));
    TDIC_CUDA_TRY(cudaMemcpyAsync(&e, d_misc.template as<int>() + 12, sizeof(int), cudaMemcpyDeviceToHost, s));
    TDIC_CUDA_TRY(cudaStreamSynchronize(s));
    *err = e;
    for (int j = 0; j < n; ++j) computed[j] = (seed_ok[j] && !flags[4 * j + 1]) ? flags[4 * j + 2] : 0;
}

template <typename T, int VAR>
tdic_grid_out BatchPlan<T, VAR>::outputs(int job) const {
    return outs[job];
}

template <typename T, int VAR>
void BatchPlan<T, VAR>::grid(int job, int32_t* gw_out, int32_t* gh_out) const {
    *gw_out = gw[job];
    *gh_out = gh[job];
}

template <typename T, int VAR>
void BatchPlan<T, VAR>::set_sms(int sms_) {
    sms = sms_ <= 0 ? num_sms : std::min(sms_, num_sms);
}

}  // namespace

// This unit's copy of the B-spline constant tables (each unit that includes hotpath.cuh has its own),
// and its plan builder.
#define TDIC_BATCH_NAME2(a, b) a##b
#define TDIC_BATCH_NAME(a, b) TDIC_BATCH_NAME2(a, b)
#if TDIC_BATCH_FP64
#define TDIC_BATCH_SUFFIX_P f64
#else
#define TDIC_BATCH_SUFFIX_P f32
#endif
#if TDIC_BATCH_VAR
#define TDIC_BATCH_SUFFIX TDIC_BATCH_NAME(TDIC_BATCH_SUFFIX_P, _masked)
#else
#define TDIC_BATCH_SUFFIX TDIC_BATCH_SUFFIX_P
#endif

void TDIC_BATCH_NAME(upload_qk_batch_, TDIC_BATCH_SUFFIX)() { upload_qk_local(); }

std::unique_ptr<BatchPlanBase> TDIC_BATCH_NAME(batch_build_, TDIC_BATCH_SUFFIX)(
    tdic_ctx* ctx, int n, tdic_pair* const* pairs, const tdic_config* cfgs, const BatchSeed* seeds,
    const std::vector<std::vector<uint8_t>>& rois, cudaStream_t s) {
    return batch_plan_build<BatchT, kBatchVar>(ctx, n, pairs, cfgs, seeds, rois, s);
}

}  // namespace tdic
