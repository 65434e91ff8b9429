// The batched propagation (several image pairs in one persistent launch, first-order ZNSSD):
// its plan, launch configurations and launches.  Compiled once per precision
// (-DTDIC_BATCH_FP64=0: FP32-mixed, 1: FP64) so the two sets of batch kernels build side by side
// with the single-pair kernels of hotpath.cu.
#include "hotpath.cuh"

#ifndef TDIC_BATCH_FP64
#error "compile with -DTDIC_BATCH_FP64=0 or 1"
#endif

namespace tdic {

namespace {

#if TDIC_BATCH_FP64
using BatchT = double;
#else
using BatchT = float;
#endif

// tdic_staging of a kernel staging mode
int staging_code(int stage) {
    return (stage & kStageLean) ? ((stage & kStageNoCoefWindow) ? TDIC_STAGING_LEAN_NO_WINDOW : TDIC_STAGING_LEAN)
                                : TDIC_STAGING_FULL;
}

template <typename T>
int BatchPlan<T>::config_count() const {
    return static_cast<int>(configs.size());
}

template <typename T>
void BatchPlan<T>::config_info(int config, int* warps_per_poi, int* groups_per_block, int* staging) const {
    *warps_per_poi = configs[config].G;
    *groups_per_block = configs[config].gpb;
    *staging = staging_code(configs[config].stage);
}

template <typename T>
void BatchPlan<T>::launch(int config, cudaStream_t s) {
    batch_plan_launch(*this, config, s);
}

template <typename T>
void BatchPlan<T>::finish(int32_t* computed, int* err, cudaStream_t s) {
    std::vector<int> flags(4 * static_cast<size_t>(n));
    int e = 0;
    TDIC_CUDA_TRY(cudaMemcpyAsync(flags.data(), d_flags.ptr, sizeof(int) * flags.size(), cudaMemcpyDeviceToHost, s));
    TDIC_CUDA_TRY(cudaMemcpyAsync(&e, d_misc.template as<int>() + 12, sizeof(int), cudaMemcpyDeviceToHost, s));
    TDIC_CUDA_TRY(cudaStreamSynchronize(s));
    *err = e;
    for (int j = 0; j < n; ++j) computed[j] = (seed_ok[j] && !flags[4 * j + 1]) ? flags[4 * j + 2] : 0;
}

template <typename T>
tdic_grid_out BatchPlan<T>::outputs(int job) const {
    return outs[job];
}

template <typename T>
void BatchPlan<T>::grid(int job, int32_t* gw_out, int32_t* gh_out) const {
    *gw_out = gw[job];
    *gh_out = gh[job];
}

template <typename T>
void BatchPlan<T>::set_sms(int sms_) {
    sms = sms_ <= 0 ? num_sms : std::min(sms_, num_sms);
}

}  // namespace

// This unit's copy of the B-spline constant tables (each unit that includes hotpath.cuh has its own).
#if TDIC_BATCH_FP64
void upload_qk_batch_f64() { upload_qk_local(); }
#else
void upload_qk_batch_f32() { upload_qk_local(); }
#endif

#if TDIC_BATCH_FP64
std::unique_ptr<BatchPlanBase> batch_build_f64(tdic_ctx* ctx, int n, tdic_pair* const* pairs, const tdic_config* cfgs,
                                               const BatchSeed* seeds, const std::vector<std::vector<uint8_t>>& rois,
                                               cudaStream_t s) {
    return batch_plan_build<BatchT>(ctx, n, pairs, cfgs, seeds, rois, s);
}
#else
std::unique_ptr<BatchPlanBase> batch_build_f32(tdic_ctx* ctx, int n, tdic_pair* const* pairs, const tdic_config* cfgs,
                                               const BatchSeed* seeds, const std::vector<std::vector<uint8_t>>& rois,
                                               cudaStream_t s) {
    return batch_plan_build<BatchT>(ctx, n, pairs, cfgs, seeds, rois, s);
}
#endif

}  // namespace tdic
