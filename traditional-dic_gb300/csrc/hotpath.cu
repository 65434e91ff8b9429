// External entry points of the hot path.  This unit holds the first-order ZNSSD kernels (route
// 0) of single pairs; batch.cu the batched propagation; variants.cu is compiled once per other
// solver route (1: SSD, 2: second order, 3: second-order SSD, 4: first-order ZNSSD on the generic
// solver, which masked subsets use), so the routes build in parallel.  Routes 1-3 handle masked subsets themselves.
#include "hotpath.cuh"

namespace tdic {

// Defined in variants.cu, one set per route.
void upload_qk_route1();
void upload_qk_route2();
void upload_qk_route3();
void upload_qk_route4();
void upload_qk_batch_f32();
void upload_qk_batch_f64();
void upload_qk_batch_f32_masked();
void upload_qk_batch_f64_masked();
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
    upload_qk_batch_f32();
    upload_qk_batch_f64();
    upload_qk_batch_f32_masked();
    upload_qk_batch_f64_masked();
}

void launch_init_grid(const tdic_grid_out& out, int gw, int gh, int step, cudaStream_t s) {
    const int n = gw * gh;
    init_grid_kernel<<<(n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096, 256, 0, s>>>(out, gw, gh, step);
    TDIC_CUDA_TRY(cudaGetLastError());
}

void launch_emit_tree(const tdic_grid_out& out, int gw, int gh, int step, int precision, const void* params,
                      const void* rcorr, const void* rq, const unsigned char* rmeta, const int* riters,
                      const unsigned char* accepted, cudaStream_t s) {
    const int n = gw * gh;
    const int blocks = (n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096;
    if (precision == TDIC_FP64)
        emit_tree_kernel<double><<<blocks, 256, 0, s>>>(out, gw, gh, step, static_cast<const double*>(params),
                                                         static_cast<const double*>(rcorr),
                                                         static_cast<const double*>(rq), rmeta, riters, accepted);
    else
        emit_tree_kernel<float><<<blocks, 256, 0, s>>>(out, gw, gh, step, static_cast<const float*>(params),
                                                        static_cast<const float*>(rcorr),
                                                        static_cast<const float*>(rq), rmeta, riters, accepted);
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

}  // namespace tdic
