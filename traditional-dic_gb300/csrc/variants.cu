// Kernels of one solver route other than first-order ZNSSD, selected at compile time by
// TDIC_ROUTE: 1 = SSD objective (icgn.cpp:832-988, forward_gauss_newton.cpp:622-794),
// 2 = second-order shape function (icgn.cpp:1168-1362, forward_gauss_newton.cpp:1069-1297),
// 3 = second-order SSD (icgn.cpp:1576-1739, forward_gauss_newton.cpp:1540-1739),
// 4 = first-order ZNSSD on the generic solver, for masked subsets (icgn.cpp:629-818,
// forward_gauss_newton.cpp:401-604).  Routes 1-3 also serve their masked counterparts.  The
// build compiles this file once per route; hotpath.cu dispatches to the entry points below.
#include "hotpath.cuh"

#ifndef TDIC_ROUTE
#error "compile with -DTDIC_ROUTE=1, 2, 3 or 4"
#endif

#define TDIC_CAT2(a, b) a##b
#define TDIC_CAT(a, b) TDIC_CAT2(a, b)

namespace tdic {

void TDIC_CAT(upload_qk_route, TDIC_ROUTE)() { upload_qk_local(); }

void TDIC_CAT(launch_solve_route, TDIC_ROUTE)(tdic_ctx* ctx, tdic_pair* pair, const tdic_config& cfg,
                                               const SolveLaunch& L, cudaStream_t s) {
    solve_route<TDIC_ROUTE>(ctx, pair, cfg, L, s);
}

void TDIC_CAT(launch_propagate_route, TDIC_ROUTE)(tdic_ctx* ctx, tdic_pair* pair, const tdic_config& cfg,
                                                   const PropagateLaunch& L, cudaStream_t s) {
    propagate_route<TDIC_ROUTE>(ctx, pair, cfg, L, s);
}

}  // namespace tdic
