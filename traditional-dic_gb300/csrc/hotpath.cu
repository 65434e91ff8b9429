// External entry points of the hot path.  This unit holds the first-order ZNSSD kernels (route
// 0) and the batched propagation; variants.cu is compiled once per other solver route (1: SSD,
// 2: second order, 3: second-order SSD, 4: first-order ZNSSD on the generic solver, which masked
// subsets use), so the routes build in parallel.  Routes 1-3 handle masked subsets themselves.
#include "hotpath.cuh"

namespace tdic {

// Defined in variants.cu, one set per route.
void upload_qk_route1();
void upload_qk_route2();
void upload_qk_route3();
void upload_qk_route4();
void launch_solve_route1(tdic_ctx*, tdic_pair*, const tdic_config&, const SolveLaunch&, cudaStream_t);
void launch_solve_route2(tdic_ctx*, tdic_pair*, const tdic_config&, const SolveLaunch&, cudaStream_t);
void launch_solve_route3(tdic_ctx*, tdic_pair*, const tdic_config&, const SolveLaunch&, cudaStream_t);
void launch_solve_route4(tdic_ctx*, tdic_pair*, const tdic_config&, const SolveLaunch&, cudaStream_t);
void launch_propagate_route1(tdic_ctx*, tdic_pair*, const tdic_config&, const PropagateLaunch&, cudaStream_t);
void launch_propagate_route2(tdic_ctx*, tdic_pair*, const tdic_config&, const PropagateLaunch&, cudaStream_t);
void launch_propagate_route3(tdic_ctx*, tdic_pair*, const tdic_config&, const PropagateLaunch&, cudaStream_t);
void launch_propagate_route4(tdic_ctx*, tdic_pair*, const tdic_config&, const PropagateLaunch&, cudaStream_t);

void upload_qk_constants() {
    upload_qk_local();
    upload_qk_route1();
    upload_qk_route2();
    upload_qk_route3();
    upload_qk_route4();
}

void launch_init_grid(const tdic_grid_out& out, int gw, int gh, int step, cudaStream_t s) {
    const int n = gw * gh;
    init_grid_kernel<<<(n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096, 256, 0, s>>>(out, gw, gh, step);
    TDIC_CUDA_TRY(cudaGetLastError());
}

size_t propagate_param_bytes(int precision) {
    (void)precision;
    return 6 * sizeof(double);
}

// Route of a solve: bit 0 SSD, bit 1 second order; masked first-order ZNSSD runs on route 4.
int solver_route(const tdic_config& cfg, bool masked) {
    const int r = (cfg.criterion == 0 ? 1 : 0) | (cfg.shape_order == 2 ? 2 : 0);
    return (r == 0 && masked) ? 4 : r;
}

void launch_solve(tdic_ctx* ctx, tdic_pair* pair, const tdic_config& cfg, const SolveLaunch& L, cudaStream_t s) {
    if (L.n <= 0) return;
    switch (solver_route(cfg, L.roi != nullptr)) {
        case 1: launch_solve_route1(ctx, pair, cfg, L, s); break;
        case 2: launch_solve_route2(ctx, pair, cfg, L, s); break;
        case 3: launch_solve_route3(ctx, pair, cfg, L, s); break;
        case 4: launch_solve_route4(ctx, pair, cfg, L, s); break;
        default: solve_route<0>(ctx, pair, cfg, L, s); break;
    }
}

void launch_propagate(tdic_ctx* ctx, tdic_pair* pair, const tdic_config& cfg, const PropagateLaunch& L,
                      cudaStream_t s) {
    switch (solver_route(cfg, L.roi_px != nullptr)) {
        case 1: launch_propagate_route1(ctx, pair, cfg, L, s); break;
        case 2: launch_propagate_route2(ctx, pair, cfg, L, s); break;
        case 3: launch_propagate_route3(ctx, pair, cfg, L, s); break;
        case 4: launch_propagate_route4(ctx, pair, cfg, L, s); break;
        default: propagate_route<0>(ctx, pair, cfg, L, s); break;
    }
}

std::unique_ptr<BatchPlanBase> batch_build(tdic_ctx* ctx, int n, tdic_pair* const* pairs, const tdic_config* cfgs,
                                           const BatchSeed* seeds, const std::vector<std::vector<uint8_t>>& rois,
                                           cudaStream_t s) {
    if (pairs[0]->precision == TDIC_FP64) return batch_plan_build<double>(ctx, n, pairs, cfgs, seeds, rois, s);
    return batch_plan_build<float>(ctx, n, pairs, cfgs, seeds, rois, s);
}

int batch_config_count(BatchPlanBase* p) {
    if (auto* b = dynamic_cast<BatchPlan<double>*>(p)) return static_cast<int>(b->configs.size());
    return static_cast<int>(static_cast<BatchPlan<float>*>(p)->configs.size());
}

void batch_launch(BatchPlanBase* p, int config, cudaStream_t s) {
    if (auto* b = dynamic_cast<BatchPlan<double>*>(p)) batch_plan_launch(*b, config, s);
    else batch_plan_launch(*static_cast<BatchPlan<float>*>(p), config, s);
}

template <typename T>
void batch_read(BatchPlan<T>& b, int32_t* computed, int* err, cudaStream_t s) {
    std::vector<int> flags(4 * static_cast<size_t>(b.n));
    int e = 0;
    TDIC_CUDA_TRY(cudaMemcpyAsync(flags.data(), b.d_flags.ptr, sizeof(int) * flags.size(), cudaMemcpyDeviceToHost, s));
    TDIC_CUDA_TRY(cudaMemcpyAsync(&e, b.d_misc.template as<int>() + 12, sizeof(int), cudaMemcpyDeviceToHost, s));
    TDIC_CUDA_TRY(cudaStreamSynchronize(s));
    *err = e;
    for (int j = 0; j < b.n; ++j)
        computed[j] = (b.seed_ok[j] && !flags[4 * j + 1]) ? flags[4 * j + 2] : 0;
}

void batch_finish(BatchPlanBase* p, int32_t* computed, int* err, cudaStream_t s) {
    if (auto* b = dynamic_cast<BatchPlan<double>*>(p)) batch_read(*b, computed, err, s);
    else batch_read(*static_cast<BatchPlan<float>*>(p), computed, err, s);
}

tdic_grid_out batch_outputs(BatchPlanBase* p, int job) {
    if (auto* b = dynamic_cast<BatchPlan<double>*>(p)) return b->outs[job];
    return static_cast<BatchPlan<float>*>(p)->outs[job];
}

void batch_set_sms(BatchPlanBase* p, int sms) {
    if (auto* b = dynamic_cast<BatchPlan<double>*>(p)) { b->sms = sms <= 0 ? b->num_sms : std::min(sms, b->num_sms); return; }
    auto* f = static_cast<BatchPlan<float>*>(p);
    f->sms = sms <= 0 ? f->num_sms : std::min(sms, f->num_sms);
}

void batch_grid(BatchPlanBase* p, int job, int32_t* gw, int32_t* gh) {
    if (auto* b = dynamic_cast<BatchPlan<double>*>(p)) { *gw = b->gw[job]; *gh = b->gh[job]; return; }
    auto* f = static_cast<BatchPlan<float>*>(p);
    *gw = f->gw[job];
    *gh = f->gh[job];
}

void batch_config_info(BatchPlanBase* p, int config, int* warps_per_poi, int* groups_per_block) {
    if (auto* b = dynamic_cast<BatchPlan<double>*>(p)) {
        *warps_per_poi = b->configs[config].G; *groups_per_block = b->configs[config].gpb;
    } else {
        auto* f = static_cast<BatchPlan<float>*>(p);
        *warps_per_poi = f->configs[config].G; *groups_per_block = f->configs[config].gpb;
    }
}

}  // namespace tdic
