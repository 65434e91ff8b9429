// K3 / K4: first-order ZNSSD ICGN and FGN per POI, batched and inside the frontier-wave
// propagation kernel.
//
// One cooperative group of G warps owns one POI at a time.  The reference subset (circular,
// icgn.cpp:484-510) is staged in shared memory as {normalised reference value f^, gx, gy} per
// sample; each iteration warps the samples, gathers the (d+1)^2 B-spline coefficient window of
// every warped point from the L2-resident coefficient image, evaluates the spline with
// separable weights w_m(t) = sum_r qk[r][m] t^r (qk of bspline.cpp:320-340, so the value equals
// the reference's local polynomial block evaluation, bspline.cpp:96-113/153-175), and reduces
// the ZNSSD residual and J^T r across the group with warp shuffles.  Precision of the FP32-mixed
// build: interpolation, residual and the 6x6 algebra in float with Kahan-compensated
// normalisation sums whose totals are combined in double.  On GB300 an FP64 instruction holds
// an SMSP's FP64 unit ~64 cycles and a double divide ~670 cycles, so FP64 is kept off the
// per-iteration path; the Hessian is an FP32-accumulated sum, so factorising it in FP64 would
// add cost but no accuracy.  The FP64 build is the same code with every T = double.
#pragma once

#include "tdic_internal.cuh"

#include <algorithm>
#include <atomic>
#include <type_traits>

#include <cuda.h>
#include <cudaTypedefs.h>

#include <cmath>

namespace tdic {

namespace {

constexpr double kEps = 1e-12;   // icgn.cpp:13
constexpr unsigned long long kSpinLimit = 1ull << 26;  // bounded waits (~2 s with backoff)

__constant__ double c_qk_d[3][36];
__constant__ float c_qk_f[3][36];

template <typename T> __device__ __forceinline__ T qk_at(int deg_slot, int i);
template <> __device__ __forceinline__ float qk_at<float>(int s, int i) { return c_qk_f[s][i]; }
template <> __device__ __forceinline__ double qk_at<double>(int s, int i) { return c_qk_d[s][i]; }

template <int DEG> struct Slot { static constexpr int value = DEG == 1 ? 0 : (DEG == 3 ? 1 : 2); };

// ---------------------------------------------------------------------------------------
// Small helpers
// ---------------------------------------------------------------------------------------
template <typename T> struct Kahan {
    T s = T(0), c = T(0);
    __device__ __forceinline__ void add(T x) {
        const T y = x - c;
        const T t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ __forceinline__ T value() const { return s - c; }
};

// Group barrier.  The non-aligned form: a group reaches its barriers from lane-divergent code
// (`if (tid < K)` blocks, strided loops over fewer entries than threads), where the aligned
// bar.sync (every lane of a warp at the same instruction) is undefined and was seen to deadlock.
__device__ __forceinline__ void named_bar(int id, int nthreads) {
    asm volatile("barrier.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

// Reduce-scatter of K values over a warp by recursive halving: at each of log2(KP) levels a
// lane keeps one half of its values and trades the other half with its partner, so the K
// sums take KP - 1 shuffles (KP = K rounded up to a power of two) instead of 5K; the levels
// left over for KP < 32 finish the sum of one value.  Lane l ends with the warp total of value
// (l >> (5 - log2 KP)) & (KP - 1).
template <int K> struct Pow2Ceil {
    static constexpr int value = K <= 1 ? 1 : K <= 2 ? 2 : K <= 4 ? 4 : K <= 8 ? 8 : K <= 16 ? 16 : 32;
    static constexpr int log2 = K <= 1 ? 0 : K <= 2 ? 1 : K <= 4 ? 2 : K <= 8 ? 3 : K <= 16 ? 4 : 5;
};

template <int K, typename T>
__device__ __forceinline__ T warp_scatter_sum(const T (&v)[K], int lane) {
    static_assert(K >= 1 && K <= 32, "at most one value per lane");
    constexpr int KP = Pow2Ceil<K>::value, LG = Pow2Ceil<K>::log2;
    T w[KP];
#pragma unroll
    for (int j = 0; j < KP; ++j) w[j] = j < K ? v[j] : T(0);
#pragma unroll
    for (int lev = 0; lev < LG; ++lev) {
        const int o = 16 >> lev;
        const int half = KP >> (lev + 1);
        const bool upper = (lane & o) != 0;
#pragma unroll
        for (int j = 0; j < half; ++j) {
            const T send = upper ? w[j] : w[j + half];
            const T keep = upper ? w[j + half] : w[j];
            w[j] = keep + __shfl_xor_sync(0xffffffffu, send, o);
        }
    }
    T r = w[0];
#pragma unroll
    for (int lev = LG; lev < 5; ++lev) r += __shfl_xor_sync(0xffffffffu, r, 16 >> lev);
    return r;
}

// All-reduce K values over the group: every thread ends with the same sums (summed in the same
// order), so redundant scalar math stays bit-identical across the group's warps.  A warp
// reduce-scatter, then, for K <= 8, every thread adds the G warp partials of each value itself
// (one barrier); for larger K thread k < K adds those of value k and everyone reads the K
// totals after a second barrier (summing K*G partials in every thread would spill).  Both
// forms add the partials in warp order.  `red` holds two buffers of 32*G values used
// alternately (parity `rp`): a buffer is rewritten only after every thread has passed the
// barrier of the reduction in between, which it reaches after its last read of the buffer.
template <int G, int K, typename T>
__device__ __forceinline__ void group_sum(T (&v)[K], T* red_base, int& rp, int tid, int bar_id) {
    static_assert(G == 1 || K * (G + 1) <= 32 * G, "reduction scratch: G*K partials + K totals per buffer");
    constexpr int LG = Pow2Ceil<K>::log2;
    const int lane = tid & 31;
    const T r = warp_scatter_sum<K, T>(v, lane);
    const int idx = (lane >> (5 - LG)) & ((1 << LG) - 1);
    if constexpr (G == 1) {
#pragma unroll
        for (int k = 0; k < K; ++k) v[k] = __shfl_sync(0xffffffffu, r, k << (5 - LG));
    } else {
        T* red = red_base + rp * 32 * G;
        rp ^= 1;
        const int warp = tid >> 5;
        if ((lane & ((1 << (5 - LG)) - 1)) == 0 && idx < K) red[warp * K + idx] = r;
        named_bar(bar_id, 32 * G);
        if constexpr (K <= 8) {
#pragma unroll
            for (int k = 0; k < K; ++k) {
                T acc = red[k];
#pragma unroll
                for (int w = 1; w < G; ++w) acc += red[w * K + k];
                v[k] = acc;
            }
        } else {
            T* tot = red + G * K;
            if (tid < K) {
                T acc = red[tid];
#pragma unroll
                for (int w = 1; w < G; ++w) acc += red[w * K + tid];
                tot[tid] = acc;
            }
            named_bar(bar_id, 32 * G);
#pragma unroll
            for (int k = 0; k < K; ++k) v[k] = tot[k];
        }
    }
}

template <int G>
__device__ __forceinline__ void group_sync(int bar_id) {
    if constexpr (G == 1) __syncwarp();
    else named_bar(bar_id, 32 * G);
}

template <int G>
__device__ __forceinline__ bool group_any(bool p, int* flag, int tid, int bar_id) {
    const bool w = __any_sync(0xffffffffu, p);
    if constexpr (G == 1) {
        return w;
    } else {
        named_bar(bar_id, 32 * G);
        if (tid == 0) *flag = 0;
        named_bar(bar_id, 32 * G);
        if (w && (tid & 31) == 0) *flag = 1;
        named_bar(bar_id, 32 * G);
        return *flag != 0;
    }
}

// ---------------------------------------------------------------------------------------
// TMA (cp.async.bulk.tensor) and mbarrier helpers.  Every wait is bounded: on timeout the
// caller records an error and leaves the kernel.
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ int ld_acquire_s32(const int* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_s32(int* p, int v) {
    asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ int floor_to(int v, int a) {  // largest multiple of a not above v (a > 0)
    const int r = v % a;
    return v - (r < 0 ? r + a : r);
}
constexpr long long kTmaSpinLimit = 1ll << 22;  // try_wait suspends in hardware between polls

template <typename T> __device__ __forceinline__ bool finite6(const T* p) {
    bool ok = true;
#pragma unroll
    for (int i = 0; i < 6; ++i) ok = ok && isfinite(p[i]);
    return ok;
}

// ---------------------------------------------------------------------------------------
// 6x6 LDLT with symmetric diagonal pivoting and sign tracking: success / positivity
// semantics of Eigen::LDLT as used at icgn.cpp:538-542 and forward_gauss_newton.cpp:354-358;
// solve applies the pseudo-inverse of D (zero where |D_ii| is not above the smallest normal).
// ---------------------------------------------------------------------------------------
// Smallest normal of M (the pseudo-inverse threshold of the LDLT solve).
template <typename M> __device__ __forceinline__ M tiny_normal();
template <> __device__ __forceinline__ float tiny_normal<float>() { return 1.17549435e-38f; }
template <> __device__ __forceinline__ double tiny_normal<double>() { return 2.2250738585072014e-308; }

template <typename M>
struct Ldlt6 {
    M m[6][6];
    M dinv[6];  // reciprocal of each pivot (0 where |D_ii| is below DBL_MIN)
    int t[6];
    int sign;  // 0 zero, 1 positive semidefinite, 2 negative semidefinite, 3 indefinite
    bool ok;

    __device__ void factor(const M (&a)[6][6]) {
#pragma unroll
        for (int i = 0; i < 6; ++i)
#pragma unroll
            for (int j = 0; j < 6; ++j) m[i][j] = a[i][j];
        sign = 0;
        ok = true;
        bool found_zero = false;
        for (int k = 0; k < 6; ++k) {
            int big = k;
            M bigv = fabs(m[k][k]);
            for (int i = k + 1; i < 6; ++i)
                if (fabs(m[i][i]) > bigv) { bigv = fabs(m[i][i]); big = i; }
            t[k] = big;
            if (big != k) {
                for (int j = 0; j < k; ++j) { const M x = m[k][j]; m[k][j] = m[big][j]; m[big][j] = x; }
                for (int i = big + 1; i < 6; ++i) { const M x = m[i][k]; m[i][k] = m[i][big]; m[i][big] = x; }
                { const M x = m[k][k]; m[k][k] = m[big][big]; m[big][big] = x; }
                for (int i = k + 1; i < big; ++i) { const M x = m[i][k]; m[i][k] = m[big][i]; m[big][i] = x; }
            }
            if (k > 0) {
                M temp[6];
                for (int j = 0; j < k; ++j) temp[j] = m[j][j] * m[k][j];
                M s = M(0);
                for (int j = 0; j < k; ++j) s += m[k][j] * temp[j];
                m[k][k] -= s;
                for (int i = k + 1; i < 6; ++i) {
                    M si = M(0);
                    for (int j = 0; j < k; ++j) si += m[i][j] * temp[j];
                    m[i][k] -= si;
                }
            }
            const M akk = m[k][k];
            const bool pivot_valid = fabs(akk) > M(0);
            if (k == 0 && !pivot_valid) {
                sign = 0;
                for (int j = 0; j < 6; ++j) { t[j] = j; dinv[j] = M(0); for (int i = 0; i < 6; ++i) m[i][j] = M(0); }
                ok = true;
                return;
            }
            if (pivot_valid) {
                const M r = M(1) / akk;
                for (int i = k + 1; i < 6; ++i) m[i][k] *= r;
            } else {
                for (int i = k + 1; i < 6; ++i) ok = ok && (m[i][k] == M(0));
            }
            if (found_zero && pivot_valid) ok = false;
            else if (!pivot_valid) found_zero = true;
            if (sign == 1) { if (akk < M(0)) sign = 3; }
            else if (sign == 2) { if (akk > M(0)) sign = 3; }
            else if (sign == 0) { if (akk > M(0)) sign = 1; else if (akk < M(0)) sign = 2; }
        }
        for (int i = 0; i < 6; ++i) dinv[i] = fabs(m[i][i]) > tiny_normal<M>() ? M(1) / m[i][i] : M(0);
    }
    __device__ bool good() const { return ok && (sign == 1 || sign == 0); }
    __device__ void solve(const M (&b)[6], M (&x)[6]) const {
        for (int i = 0; i < 6; ++i) x[i] = b[i];
        for (int k = 0; k < 6; ++k) { const M v = x[k]; x[k] = x[t[k]]; x[t[k]] = v; }
        for (int i = 0; i < 6; ++i) { M s = x[i]; for (int j = 0; j < i; ++j) s -= m[i][j] * x[j]; x[i] = s; }
        for (int i = 0; i < 6; ++i) x[i] *= dinv[i];
        for (int i = 5; i >= 0; --i) { M s = x[i]; for (int j = i + 1; j < 6; ++j) s -= m[j][i] * x[j]; x[i] = s; }
        for (int k = 5; k >= 0; --k) { const M v = x[k]; x[k] = x[t[k]]; x[t[k]] = v; }
    }
};

// icgn.cpp:83-120
template <typename M>
__device__ __forceinline__ void ic_update(const M (&p)[6], const M (&dp)[6], M (&o)[6]) {
    const M du = p[0], dv = p[1], dudx = p[2], dudy = p[3], dvdx = p[4], dvdy = p[5];
    const M dp0 = dp[0], dp1 = dp[1], dp2 = dp[2], dp3 = dp[3], dp4 = dp[4], dp5 = dp[5];
    const M den = dp2 + dp5 + dp2 * dp5 - dp3 * dp4 + M(1);
    if (fabs(den) <= M(kEps)) {
        for (int i = 0; i < 6; ++i) o[i] = M(NAN);
        return;
    }
    // one reciprocal instead of twelve divisions (same closed form, rounding differs by ~1 ulp)
    const M r = M(1) / den;
    const M a = dp0 + dp0 * dp5 - dp1 * dp3, b = dp1 - dp0 * dp4 + dp1 * dp2;
    o[0] = du - ((dudx + M(1)) * a) * r - (dudy * b) * r;
    o[1] = dv - ((dvdy + M(1)) * b) * r - (dvdx * a) * r;
    o[2] = ((dp5 + M(1)) * (dudx + M(1))) * r - (dp4 * dudy) * r - M(1);
    o[3] = (dudy * (dp2 + M(1))) * r - (dp3 * (dudx + M(1))) * r;
    o[4] = (dvdx * (dp5 + M(1))) * r - (dp4 * (dvdy + M(1))) * r;
    o[5] = ((dp2 + M(1)) * (dvdy + M(1))) * r - (dp3 * dvdx) * r - M(1);
}

// forward_gauss_newton.cpp:64-76
template <typename M>
__device__ __forceinline__ void compose_warp(const M (&p)[6], const M (&dp)[6], M (&pn)[6]) {
    pn[0] = dp[0] + p[0] + p[2] * dp[0] + p[3] * dp[1];
    pn[1] = dp[1] + p[1] + p[4] * dp[0] + p[5] * dp[1];
    pn[2] = dp[2] + p[2] * (M(1) + dp[2]) + p[3] * dp[4];
    pn[3] = dp[3] + p[2] * dp[3] + p[3] * (M(1) + dp[5]);
    pn[4] = dp[4] + p[4] * (M(1) + dp[2]) + p[5] * dp[4];
    pn[5] = dp[5] + p[4] * dp[3] + p[5] * (M(1) + dp[5]);
}

// ---------------------------------------------------------------------------------------
// B-spline evaluation from the coefficient image
// ---------------------------------------------------------------------------------------
template <int DEG, typename T>
__device__ __forceinline__ void weights(T t, T (&w)[DEG + 1]) {
    constexpr int NB = DEG + 1;
#pragma unroll
    for (int m = 0; m < NB; ++m) {
        T acc = qk_at<T>(Slot<DEG>::value, DEG * NB + m);
#pragma unroll
        for (int r = DEG - 1; r >= 0; --r) acc = acc * t + qk_at<T>(Slot<DEG>::value, r * NB + m);
        w[m] = acc;
    }
}

template <int DEG, typename T>
__device__ __forceinline__ void dweights(T t, T (&w)[DEG + 1]) {
    constexpr int NB = DEG + 1;
#pragma unroll
    for (int m = 0; m < NB; ++m) {
        T acc = T(DEG) * qk_at<T>(Slot<DEG>::value, DEG * NB + m);
#pragma unroll
        for (int r = DEG - 1; r >= 1; --r) acc = acc * t + T(r) * qk_at<T>(Slot<DEG>::value, r * NB + m);
        w[m] = acc;
    }
}

// Shared-memory staging modes of a solve (bits; see group_smem_bytes) and the per-sample arrays
// each keeps.
enum { kStageFull = 0, kStageLean = 1, kStageNoCoefWindow = 2 };
__host__ __device__ __forceinline__ int sample_arrays(int opt, int stage) {
    return (stage & kStageLean) ? (opt == 1 ? 3 : 1) : 4;
}

template <typename T>
struct Env {
    const float* ref;      // H x W float32 reference
    const T* coef;         // (H + 2B) x (W + 2B) coefficients
    int w, h, cw, border;
    int radius, n, nmax;   // samples of this radius; nmax = smem capacity per group
    const short2* off;     // sample offsets
    int max_iter;
    double thr;
    double inv_n;          // 1 / n
    int rpitch, cpitch;    // row pitches (elements) of ref and coef
    int rbx, rby;          // TMA box of the reference window (floats)
    int cbx, cby;          // TMA box of the coefficient window (T)
    int* err;              // device error flag (TMA wait timeout)
    // masked subsets (solve_with_mask): ROI of the image (w x h bytes, row pitch w) or NULL;
    // min_keep = max(NP, min_valid_samples, ceil(min_valid_sample_ratio * n))
    const uint8_t* roi;
    int min_keep;
    // shared-memory staging of the single-pair kernels (a batched launch takes its own from
    // the launch's Shape): kStage* bits and the per-sample arrays it keeps
    int stage = kStageFull;
    int narr = 4;
    // Set-up cache of a propagation grid (first-order ZNSSD ICGN), or NULL: per grid point the
    // reference side of the solve -- inverse Hessian (36 values of the solve's scalar type),
    // mean and inverse norm of the subset (2 values of T) and a state (0 not computed, 1 ready,
    // 2 the set-up fails: NumericalFailure).  Idle solver groups fill it ahead of the solves.
    void* sc_hinv = nullptr;
    T* sc_fmn = nullptr;
    int* sc_state = nullptr;
};

// Per-POI result in the solve's own precision (float on the FP32-mixed path); outputs are
// widened to double when they are written.
template <typename M>
struct Result {
    M p[6];
    M q[6];  // second-order terms d2u_dx2, d2u_dxdy, d2u_dy2, d2v_dx2, d2v_dxdy, d2v_dy2 (else 0)
    M corr;
    int iters;
    int status;
    bool valid;
    bool conv;
};

template <typename M>
__device__ __forceinline__ void result_init(Result<M>& r, const M (&p0)[6], M conf) {
    r.p[0] = p0[0];
    r.p[1] = p0[1];
    r.p[2] = r.p[3] = r.p[4] = r.p[5] = M(0);
#pragma unroll
    for (int k = 0; k < 6; ++k) r.q[k] = M(0);
    r.corr = conf;
    r.iters = 0;
    r.status = TDIC_INVALID_INPUT;
    r.valid = false;
    r.conv = false;
}

// Per-iteration scalar type: the FP32-mixed build keeps the 6x6 algebra, the parameter vector,
// its update and the normalisation algebra in float; the FP64 build is double throughout.
template <typename T> struct MixedOf { using type = T; };


// Unpivoted LDL^T of a 6x6 symmetric matrix, fully unrolled in registers.  Succeeds only when
// every pivot is positive and finite; for such (numerically positive definite) matrices the
// pivoted factorisation of icgn.cpp:538 reports success and isPositive() as well, so the
// outcome is the same.  Anything else falls back to the pivoted Ldlt6.
template <typename M>
struct FastLdlt6 {
    M L[6][6];
    M D[6];
    M dinv[6];
    __device__ __forceinline__ bool factor(const M (&H)[6][6]) {
        bool ok = true;
#pragma unroll
        for (int j = 0; j < 6; ++j) {
            M LD[6];  // L[j][k] * D[k]
#pragma unroll
            for (int k = 0; k < j; ++k) LD[k] = L[j][k] * D[k];
            M d = H[j][j];
#pragma unroll
            for (int k = 0; k < j; ++k) d -= L[j][k] * LD[k];
            ok = ok && (d > M(0)) && isfinite(d);
            D[j] = d;
            dinv[j] = M(1) / d;
#pragma unroll
            for (int i = j + 1; i < 6; ++i) {
                M v = H[i][j];
#pragma unroll
                for (int k = 0; k < j; ++k) v -= L[i][k] * LD[k];
                L[i][j] = v * dinv[j];
            }
        }
        return ok;
    }
    // x = H^-1 b
    __device__ __forceinline__ void solve(const M (&b)[6], M (&x)[6]) const {
        M y[6];
#pragma unroll
        for (int i = 0; i < 6; ++i) {
            M v = b[i];
#pragma unroll
            for (int k = 0; k < i; ++k) v -= L[i][k] * y[k];
            y[i] = v;
        }
#pragma unroll
        for (int i = 5; i >= 0; --i) {
            M v = y[i] * dinv[i];
#pragma unroll
            for (int k = i + 1; k < 6; ++k) v -= L[k][i] * x[k];
            x[i] = v;
        }
    }
};

// Factorise H and store H^-1 (row-major, 36 values) in shared memory; returns false when the
// reference's LDLT would fail or report a matrix that is not positive semidefinite.
template <int G, typename M>
__device__ bool factor_inverse(const M (&H)[6][6], M* s_hinv, int tid, int bar_id) {
    FastLdlt6<M> f;
    bool good = f.factor(H);
    if (good) {
        if (tid < 6) {
            M e6[6] = {M(0), M(0), M(0), M(0), M(0), M(0)}, col[6];
            e6[tid] = M(1);
            f.solve(e6, col);
#pragma unroll
            for (int i = 0; i < 6; ++i) s_hinv[i * 6 + tid] = col[i];
        }
    } else {
        Ldlt6<M> g;
        g.factor(H);
        good = g.good();
        if (good && tid < 6) {
            M e6[6] = {M(0), M(0), M(0), M(0), M(0), M(0)}, col[6];
            e6[tid] = M(1);
            g.solve(e6, col);
            for (int i = 0; i < 6; ++i) s_hinv[i * 6 + tid] = col[i];
        }
    }
    return good;
}

template <int G, typename M>
__device__ bool factor_solve(const M (&H)[6][6], const M (&b)[6], M (&x)[6]) {
    FastLdlt6<M> f;
    if (f.factor(H)) { f.solve(b, x); return true; }
    Ldlt6<M> g;
    g.factor(H);
    if (!g.good()) return false;
    g.solve(b, x);
    return true;
}

// ---------------------------------------------------------------------------------------
// Helpers of the other solver routes: SSD objective, second-order shape function
// (12 parameters u, v, ux, uy, vx, vy, uxx, uxy, uyy, vxx, vxy, vyy).
// ---------------------------------------------------------------------------------------

// group_sum over more values than one reduction buffer holds, in chunks.
template <int G, int K, typename T>
__device__ __forceinline__ void group_sum_n(T (&v)[K], T* red, int& rp, int tid, int bar_id) {
    constexpr int C = G == 1 ? 32 : (32 * G) / (G + 1);
    if constexpr (K <= C) {
        group_sum<G, K, T>(v, red, rp, tid, bar_id);
    } else {
        T a[C], b[K - C];
#pragma unroll
        for (int k = 0; k < C; ++k) a[k] = v[k];
#pragma unroll
        for (int k = 0; k < K - C; ++k) b[k] = v[C + k];
        group_sum<G, C, T>(a, red, rp, tid, bar_id);
        group_sum_n<G, K - C, T>(b, red, rp, tid, bar_id);
#pragma unroll
        for (int k = 0; k < C; ++k) v[k] = a[k];
#pragma unroll
        for (int k = 0; k < K - C; ++k) v[C + k] = b[k];
    }
}

// Steepest-descent row of the 12-parameter warp: SD_k = c_k * m_j(k), c in {a, b} (gradient
// components) and m = [1, lx, ly, lx^2/2, lx ly, ly^2/2] (icgn.cpp:142-165):
// c(k) = bit k of 0xE32 (0: a, 1: b), j(k) = nibble k of 0x543543212100.
__device__ __forceinline__ int sd_c(int k) { return (0xE32 >> k) & 1; }
__device__ __forceinline__ int sd_j(int k) { return static_cast<int>((0x543543212100ull >> (4 * k)) & 0xF); }
// Exponents of lx, ly in m_j, and whether m_j carries the factor 1/2.
__device__ __forceinline__ int m_ex(int j) { return (0x012010 >> (4 * j)) & 0xF; }   // {0,1,0,2,1,0}
__device__ __forceinline__ int m_ey(int j) { return (0x210100 >> (4 * j)) & 0xF; }   // {0,0,1,0,1,2}
__device__ __forceinline__ bool m_half(int j) { return j == 3 || j == 5; }

// The 15 monomials lx^a ly^b of degree <= 4 in the order (0,0) (1,0) (0,1) (2,0) (1,1) (0,2)
// (3,0) ... (0,4): index d(d+1)/2 + b for degree d = a + b.  Small integers: exact in float.
template <typename T>
__device__ __forceinline__ void monomials15(T lx, T ly, T (&m)[15]) {
    const T x2 = lx * lx, y2 = ly * ly, xy = lx * ly;
    m[0] = T(1); m[1] = lx; m[2] = ly;
    m[3] = x2; m[4] = xy; m[5] = y2;
    m[6] = x2 * lx; m[7] = x2 * ly; m[8] = lx * y2; m[9] = y2 * ly;
    m[10] = x2 * x2; m[11] = x2 * xy; m[12] = x2 * y2; m[13] = xy * y2; m[14] = y2 * y2;
}

// Entry (k, l) of the 12x12 Gauss-Newton Hessian from the 45 sums S[u * 15 + mono] with
// u = 0 (aa), 1 (ab), 2 (bb): H_kl = sum c_k c_l m_j(k) m_j(l), the halves applied exactly.
template <typename M>
__device__ __forceinline__ M hess12_entry(const M* S, int k, int l) {
    const int jk = sd_j(k), jl = sd_j(l);
    const int a = m_ex(jk) + m_ex(jl), b = m_ey(jk) + m_ey(jl), d = a + b;
    const int u = sd_c(k) + sd_c(l);
    M v = S[u * 15 + d * (d + 1) / 2 + b];
    if (m_half(jk)) v *= M(0.5);
    if (m_half(jl)) v *= M(0.5);
    return v;
}

// LDL^T with symmetric diagonal pivoting for N x N (Eigen::LDLT semantics, see Ldlt6), from a
// row-major matrix in memory; the fallback of the unpivoted group factorisation below.
template <int N, typename M>
struct LdltN {
    M m[N][N];
    M dinv[N];
    int t[N];
    int sign;
    bool ok;
    __device__ void factor(const M* a) {
        for (int i = 0; i < N; ++i)
            for (int j = 0; j < N; ++j) m[i][j] = a[i * N + j];
        sign = 0;
        ok = true;
        bool found_zero = false;
        for (int k = 0; k < N; ++k) {
            int big = k;
            M bigv = fabs(m[k][k]);
            for (int i = k + 1; i < N; ++i)
                if (fabs(m[i][i]) > bigv) { bigv = fabs(m[i][i]); big = i; }
            t[k] = big;
            if (big != k) {
                for (int j = 0; j < k; ++j) { const M x = m[k][j]; m[k][j] = m[big][j]; m[big][j] = x; }
                for (int i = big + 1; i < N; ++i) { const M x = m[i][k]; m[i][k] = m[i][big]; m[i][big] = x; }
                { const M x = m[k][k]; m[k][k] = m[big][big]; m[big][big] = x; }
                for (int i = k + 1; i < big; ++i) { const M x = m[i][k]; m[i][k] = m[big][i]; m[big][i] = x; }
            }
            if (k > 0) {
                M temp[N];
                for (int j = 0; j < k; ++j) temp[j] = m[j][j] * m[k][j];
                M s = M(0);
                for (int j = 0; j < k; ++j) s += m[k][j] * temp[j];
                m[k][k] -= s;
                for (int i = k + 1; i < N; ++i) {
                    M si = M(0);
                    for (int j = 0; j < k; ++j) si += m[i][j] * temp[j];
                    m[i][k] -= si;
                }
            }
            const M akk = m[k][k];
            const bool pivot_valid = fabs(akk) > M(0);
            if (k == 0 && !pivot_valid) {
                sign = 0;
                for (int j = 0; j < N; ++j) { t[j] = j; dinv[j] = M(0); for (int i = 0; i < N; ++i) m[i][j] = M(0); }
                ok = true;
                return;
            }
            if (pivot_valid) {
                const M r = M(1) / akk;
                for (int i = k + 1; i < N; ++i) m[i][k] *= r;
            } else {
                for (int i = k + 1; i < N; ++i) ok = ok && (m[i][k] == M(0));
            }
            if (found_zero && pivot_valid) ok = false;
            else if (!pivot_valid) found_zero = true;
            if (sign == 1) { if (akk < M(0)) sign = 3; }
            else if (sign == 2) { if (akk > M(0)) sign = 3; }
            else if (sign == 0) { if (akk > M(0)) sign = 1; else if (akk < M(0)) sign = 2; }
        }
        for (int i = 0; i < N; ++i) dinv[i] = fabs(m[i][i]) > tiny_normal<M>() ? M(1) / m[i][i] : M(0);
    }
    __device__ bool good() const { return ok && (sign == 1 || sign == 0); }
    __device__ void solve(const M* b, M* x) const {
        for (int i = 0; i < N; ++i) x[i] = b[i];
        for (int k = 0; k < N; ++k) { const M v = x[k]; x[k] = x[t[k]]; x[t[k]] = v; }
        for (int i = 0; i < N; ++i) { M s = x[i]; for (int j = 0; j < i; ++j) s -= m[i][j] * x[j]; x[i] = s; }
        for (int i = 0; i < N; ++i) x[i] *= dinv[i];
        for (int i = N - 1; i >= 0; --i) { M s = x[i]; for (int j = i + 1; j < N; ++j) s -= m[j][i] * x[j]; x[i] = s; }
        for (int k = N - 1; k >= 0; --k) { const M v = x[k]; x[k] = x[t[k]]; x[t[k]] = v; }
    }
};

// Unpivoted right-looking LDL^T of the symmetric 12x12 matrix A (row-major, shared memory, lower
// triangle used) by the whole group, one barrier per column.  Afterwards A[k][k] = D_k,
// A[i][k] = L_ik D_k for i > k (the column is left unscaled, so a step's reads and writes never
// overlap) and dinv[k] = 1 / D_k.  Returns false, on every thread alike, at the first pivot that
// is not positive and finite: for a positive definite matrix every unpivoted pivot is positive,
// and anything else is left to the pivoted LdltN (Eigen's semantics for semidefinite input).
template <int G, typename M>
__device__ bool ldlt12_group(M* A, M* dinv, int tid, int bar_id) {
    constexpr int NT = 32 * G;
    group_sync<G>(bar_id);  // A complete
    for (int k = 0; k < 12; ++k) {
        const M d = A[k * 12 + k];
        if (!(d > M(0)) || !isfinite(d)) return false;
        const M rd = M(1) / d;
        const int m = 11 - k;
        for (int t = tid; t < m * m; t += NT) {
            const int i = k + 1 + t / m, j = k + 1 + t % m;
            if (j <= i) A[i * 12 + j] -= A[i * 12 + k] * (A[j * 12 + k] * rd);
        }
        if (tid == 0) dinv[k] = rd;
        group_sync<G>(bar_id);
    }
    return true;
}

// x = A^-1 b from the factor of ldlt12_group.
template <typename M>
__device__ __forceinline__ void ldlt12_solve(const M* A, const M* dinv, const M (&b)[12], M (&x)[12]) {
    M z[12];
#pragma unroll
    for (int i = 0; i < 12; ++i) {
        M v = b[i];
#pragma unroll
        for (int k = 0; k < i; ++k) v -= (A[i * 12 + k] * dinv[k]) * z[k];
        z[i] = v;
    }
#pragma unroll
    for (int i = 11; i >= 0; --i) {
        M v = z[i] * dinv[i];
#pragma unroll
        for (int k = i + 1; k < 12; ++k) v -= (A[k * 12 + i] * dinv[i]) * x[k];
        x[i] = v;
    }
}

// Rows 0 and 1 of the second-order warp matrix G'(p) (icgn.cpp:196-261).
template <typename M>
__device__ __forceinline__ void warp_rows01(const M (&p)[12], M (&B)[2][6]) {
    B[0][0] = p[0]; B[0][1] = M(1) + p[2]; B[0][2] = p[3]; B[0][3] = M(0.5) * p[6]; B[0][4] = p[7]; B[0][5] = M(0.5) * p[8];
    B[1][0] = p[1]; B[1][1] = p[4]; B[1][2] = M(1) + p[5]; B[1][3] = M(0.5) * p[9]; B[1][4] = p[10]; B[1][5] = M(0.5) * p[11];
}

// The full 6x6 G'(p) with its rows in the order (2, 0, 1, 3, 4, 5): row 2 of G' is (1, 0, ..., 0),
// so for a small increment this order is close to the identity.
template <typename M>
__device__ __forceinline__ void warp_matrix_perm(const M (&p)[12], M (&G)[6][6]) {
    const M u = p[0], v = p[1], ux = p[2], uy = p[3], vx = p[4], vy = p[5];
    const M uxx = p[6], uxy = p[7], uyy = p[8], vxx = p[9], vxy = p[10], vyy = p[11];
    G[0][0] = M(1); G[0][1] = M(0); G[0][2] = M(0); G[0][3] = M(0); G[0][4] = M(0); G[0][5] = M(0);
    G[1][0] = u; G[1][1] = M(1) + ux; G[1][2] = uy; G[1][3] = M(0.5) * uxx; G[1][4] = uxy; G[1][5] = M(0.5) * uyy;
    G[2][0] = v; G[2][1] = vx; G[2][2] = M(1) + vy; G[2][3] = M(0.5) * vxx; G[2][4] = vxy; G[2][5] = M(0.5) * vyy;
    G[3][0] = u * u; G[3][1] = M(2) * u * (M(1) + ux); G[3][2] = M(2) * u * uy;
    G[3][3] = M(1) + M(2) * ux + ux * ux + u * uxx; G[3][4] = M(2) * (uy + ux * uy + u * uxy); G[3][5] = uy * uy + u * uyy;
    G[4][0] = u * v; G[4][1] = v + u * vx + v * ux; G[4][2] = u + u * vy + v * uy;
    G[4][3] = vx + ux * vx + M(0.5) * (u * vxx + v * uxx);
    G[4][4] = M(1) + vy + ux + ux * vy + uy * vx + u * vxy + v * uxy;
    G[4][5] = uy + uy * vy + M(0.5) * (u * vyy + v * uyy);
    G[5][0] = v * v; G[5][1] = M(2) * v * vx; G[5][2] = M(2) * v * (M(1) + vy);
    G[5][3] = vx * vx + v * vxx; G[5][4] = M(2) * (vx + vx * vy + v * vxy); G[5][5] = M(1) + M(2) * vy + vy * vy + v * vyy;
}

template <typename M> __device__ __forceinline__ M mach_eps();
template <> __device__ __forceinline__ float mach_eps<float>() { return 1.1920929e-7f; }
template <> __device__ __forceinline__ double mach_eps<double>() { return 2.220446049250313e-16; }

// Parameters from rows 0, 1 of G'(p_new) (extract_from_warp_matrix, icgn.cpp:265-287).
template <typename M>
__device__ __forceinline__ void params_from_rows(const M (&N)[2][6], M (&pn)[12]) {
    pn[0] = N[0][0]; pn[2] = N[0][1] - M(1); pn[3] = N[0][2]; pn[6] = M(2) * N[0][3]; pn[7] = N[0][4]; pn[8] = M(2) * N[0][5];
    pn[1] = N[1][0]; pn[4] = N[1][1]; pn[5] = N[1][2] - M(1); pn[9] = M(2) * N[1][3]; pn[10] = N[1][4]; pn[11] = M(2) * N[1][5];
}

// Full-pivoting 6x6 inverse with Eigen::FullPivLU's pivot order and rank test (icgn.cpp:325-329);
// false when the rank is below 6.  Local memory: only the rare fallback of ic_update2 runs it.
template <typename M>
__device__ bool fullpiv_inverse6(const M (&a)[6][6], M (&inv)[6][6]) {
    M lu[6][6];
    for (int i = 0; i < 6; ++i) for (int j = 0; j < 6; ++j) lu[i][j] = a[i][j];
    int rt[6], ct[6];
    int nonzero = 6;
    M maxpivot = M(0);
    for (int k = 0; k < 6; ++k) {
        int br = k, bc = k;
        M big = M(-1);
        for (int c = k; c < 6; ++c)
            for (int r = k; r < 6; ++r)
                if (fabs(lu[r][c]) > big) { big = fabs(lu[r][c]); br = r; bc = c; }
        if (big == M(0)) {
            nonzero = k;
            for (int i = k; i < 6; ++i) { rt[i] = i; ct[i] = i; }
            break;
        }
        if (big > maxpivot) maxpivot = big;
        rt[k] = br; ct[k] = bc;
        if (br != k) for (int j = 0; j < 6; ++j) { const M x = lu[k][j]; lu[k][j] = lu[br][j]; lu[br][j] = x; }
        if (bc != k) for (int i = 0; i < 6; ++i) { const M x = lu[i][k]; lu[i][k] = lu[i][bc]; lu[i][bc] = x; }
        for (int r = k + 1; r < 6; ++r) lu[r][k] /= lu[k][k];
        for (int c = k + 1; c < 6; ++c)
            for (int r = k + 1; r < 6; ++r) lu[r][c] -= lu[r][k] * lu[k][c];
    }
    int rank = 0;
    const M thr = maxpivot * (M(6) * mach_eps<M>());
    for (int i = 0; i < nonzero; ++i) rank += fabs(lu[i][i]) > thr ? 1 : 0;
    if (rank != 6) return false;
    int q[6] = {0, 1, 2, 3, 4, 5};
    for (int k = 0; k < 6; ++k) { const int x = q[k]; q[k] = q[ct[k]]; q[ct[k]] = x; }
    for (int col = 0; col < 6; ++col) {
        M c[6] = {M(0), M(0), M(0), M(0), M(0), M(0)};
        c[col] = M(1);
        for (int k = 0; k < 6; ++k) { const M x = c[k]; c[k] = c[rt[k]]; c[rt[k]] = x; }
        for (int i = 0; i < 6; ++i) for (int j = 0; j < i; ++j) c[i] -= lu[i][j] * c[j];
        for (int i = 5; i >= 0; --i) {
            for (int j = i + 1; j < 6; ++j) c[i] -= lu[i][j] * c[j];
            c[i] /= lu[i][i];
        }
        for (int i = 0; i < 6; ++i) inv[q[i]][col] = c[i];
    }
    return true;
}

// Second-order inverse-compositional update (icgn.cpp:308-357):
// G'(p_new) = G'(p) G'(dp)^-1 P^-1, read back from rows 0 and 1.  With G'' = G'(dp) rows in the
// order (2, 0, 1, 3, 4, 5), G'(dp)^-1 = G''^-1 times the same row permutation as columns, and that
// permutation cancels P^-1: rows 0, 1 of G'(p_new) = rows 0, 1 of G'(p) times G''^-1.  G'' is near
// the identity, so it is factorised without pivoting (compile-time indices, registers) and the two
// rows solved against the factor.  A pivot at or below the rank threshold of Eigen::FullPivLU
// (6 eps |largest pivot|) or not finite sends the update through the full-pivoting inverse, and a
// rank-deficient G'(dp) to the reference's additive fallback p - dp.
template <typename M>
__device__ void ic_update2(const M (&p)[12], const M (&dp)[12], M (&pn)[12]) {
    M B[2][6];
    warp_rows01(p, B);
    M A[6][6];
    warp_matrix_perm(dp, A);
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        const M r = M(1) / A[k][k];
#pragma unroll
        for (int i = k + 1; i < 6; ++i) {
            A[i][k] *= r;
#pragma unroll
            for (int j = k + 1; j < 6; ++j) A[i][j] -= A[i][k] * A[k][j];
        }
    }
    M big = M(0);
    bool fin = true;
#pragma unroll
    for (int k = 0; k < 6; ++k) { big = fmax(big, fabs(A[k][k])); fin = fin && isfinite(A[k][k]); }
    bool ok = fin;
    const M thr = big * (M(6) * mach_eps<M>());
#pragma unroll
    for (int k = 0; k < 6; ++k) ok = ok && fabs(A[k][k]) > thr;
    M N[2][6];
    if (ok) {
        // Z U = B, then Y L = Z (L unit lower, U upper)
#pragma unroll
        for (int r = 0; r < 2; ++r) {
            M Z[6];
#pragma unroll
            for (int j = 0; j < 6; ++j) {
                M v = B[r][j];
#pragma unroll
                for (int k = 0; k < j; ++k) v -= Z[k] * A[k][j];
                Z[j] = v / A[j][j];
            }
#pragma unroll
            for (int j = 5; j >= 0; --j) {
                M v = Z[j];
#pragma unroll
                for (int k = j + 1; k < 6; ++k) v -= N[r][k] * A[k][j];
                N[r][j] = v;
            }
        }
    } else {
        M Gfull[6][6], Gi[6][6], P[6][6];
        warp_matrix_perm(dp, P);
        // back to the reference's row order (0, 1, 2, 3, 4, 5) for the full-pivoting inverse
        for (int j = 0; j < 6; ++j) { Gfull[0][j] = P[1][j]; Gfull[1][j] = P[2][j]; Gfull[2][j] = P[0][j]; }
        for (int i = 3; i < 6; ++i) for (int j = 0; j < 6; ++j) Gfull[i][j] = P[i][j];
        if (!fullpiv_inverse6(Gfull, Gi)) {
            for (int k = 0; k < 12; ++k) pn[k] = p[k] - dp[k];
            return;
        }
        M X[2][6];
        for (int r = 0; r < 2; ++r)
            for (int c = 0; c < 6; ++c) { M s = M(0); for (int k = 0; k < 6; ++k) s += B[r][k] * Gi[k][c]; X[r][c] = s; }
        for (int r = 0; r < 2; ++r) {  // P^-1: columns (0, 1, 2) <- (2, 0, 1)
            N[r][0] = X[r][2]; N[r][1] = X[r][0]; N[r][2] = X[r][1];
            for (int c = 3; c < 6; ++c) N[r][c] = X[r][c];
        }
    }
    params_from_rows(N, pn);
}

// Forward composition of the second-order warp (forward_gauss_newton.cpp:1025-1053).
template <typename M>
__device__ __forceinline__ void compose_warp2(const M (&p)[12], const M (&dp)[12], M (&pn)[12]) {
    pn[0] = dp[0] + p[0] + p[2] * dp[0] + p[3] * dp[1];
    pn[1] = dp[1] + p[1] + p[4] * dp[0] + p[5] * dp[1];
    pn[2] = dp[2] + p[2] * (M(1) + dp[2]) + p[3] * dp[4] + p[6] * dp[0] + p[7] * dp[1];
    pn[3] = dp[3] + p[2] * dp[3] + p[3] * (M(1) + dp[5]) + p[7] * dp[0] + p[8] * dp[1];
    pn[4] = dp[4] + p[4] * (M(1) + dp[2]) + p[5] * dp[4] + p[9] * dp[0] + p[10] * dp[1];
    pn[5] = dp[5] + p[4] * dp[3] + p[5] * (M(1) + dp[5]) + p[10] * dp[0] + p[11] * dp[1];
    pn[6] = dp[6] + p[2] * dp[6] + p[3] * dp[9] + p[6] * (M(1) + M(2) * dp[2]) + M(2) * p[7] * dp[4];
    pn[7] = dp[7] + p[2] * dp[7] + p[3] * dp[10] + p[6] * dp[3] + p[7] * (M(1) + dp[2] + dp[5]) + p[8] * dp[4];
    pn[8] = dp[8] + p[2] * dp[8] + p[3] * dp[11] + p[7] * dp[3] + p[8] * (M(1) + M(2) * dp[5]);
    pn[9] = dp[9] + p[4] * dp[6] + p[5] * dp[9] + p[9] * (M(1) + M(2) * dp[2]) + M(2) * p[10] * dp[4];
    pn[10] = dp[10] + p[4] * dp[7] + p[5] * dp[10] + p[9] * dp[3] + p[10] * (M(1) + dp[2] + dp[5]) + p[11] * dp[4];
    pn[11] = dp[11] + p[4] * dp[8] + p[5] * dp[11] + p[10] * dp[3] + p[11] * (M(1) + M(2) * dp[5]);
}

template <int N, typename M> __device__ __forceinline__ bool finite_n(const M (&p)[N]) {
    bool f = true;
#pragma unroll
    for (int k = 0; k < N; ++k) f = f && isfinite(p[k]);
    return f;
}

__host__ __device__ __forceinline__ size_t round128(size_t b) { return (b + 127) & ~size_t(127); }

// Per-group shared memory, each part 128-byte aligned (TMA destinations):
// [coefficient window cbx*cby T][reference window rbx*rby float][mbarrier + matrix region of
// `mat` doubles (the 6x6 inverse: 36; second order: the 12x12 factor and inverse) + ints]
// [2 x 32*G T reduction scratch][narr*nmax T per-sample arrays].
//
// Staging modes (a layout choice only: the results are the same bit for bit):
//   full (0)        the coefficient window and four per-sample arrays: f^, the two gradients
//                   (ICGN: reference gradients; FGN: deformed spline gradients) and g;
//   lean (1)        the per-sample arrays the iterations write (ICGN: g; FGN: g and the two
//                   deformed gradients); f^ and the reference gradients are recomputed from the
//                   staged reference window when they are read;
//   lean, no coefficient window (3)   as lean, and every spline stencil is read from the
//                   L2-resident coefficient image instead of a staged window.
// Lean staging is the first-order ZNSSD solver's (route 0); it lets large subsets fit (FP64 at
// radius 41) and more solver groups share an SM.
constexpr int kMat6 = 36;
constexpr int kMat12 = 2 * 144 + 12 + 52;  // factor, inverse (or copy), 1 / D, the 45 Hessian sums
template <typename T>
__host__ __device__ __forceinline__ size_t group_smem_bytes(int nmax, int G, int rbx, int rby, int cbx, int cby,
                                                            int mat = kMat6, int stage = kStageFull, int narr = 4) {
    size_t b = (stage & kStageNoCoefWindow) ? 0 : round128(static_cast<size_t>(cbx) * cby * sizeof(T));
    b += round128(static_cast<size_t>(rbx) * rby * sizeof(float));
    b += round128(16 + static_cast<size_t>(mat) * sizeof(double) + 32);
    b += round128((static_cast<size_t>(64) * G + static_cast<size_t>(narr) * nmax) * sizeof(T));
    return b;
}
// CTA prefix: the sample-offset table shared by all groups.
__host__ __device__ __forceinline__ size_t cta_prefix_bytes(int nmax) { return round128(sizeof(short2) * nmax); }

template <typename T>
struct GroupSmem {
    T* cwin;       // nullptr without a coefficient window
    float* rwin;
    uint64_t* bar;
    double* hinv;
    int* ints;
    T* red;
    T* sm;
    int stage;
    __device__ GroupSmem(unsigned char* base, int gi, int nmax, int G, int rbx, int rby, int cbx, int cby,
                         int mat = kMat6, int stage_ = kStageFull, int narr = 4) {
        stage = stage_;
        unsigned char* g = base + gi * group_smem_bytes<T>(nmax, G, rbx, rby, cbx, cby, mat, stage_, narr);
        if (stage_ & kStageNoCoefWindow) {
            cwin = nullptr;
        } else {
            cwin = reinterpret_cast<T*>(g);
            g += round128(static_cast<size_t>(cbx) * cby * sizeof(T));
        }
        rwin = reinterpret_cast<float*>(g);
        g += round128(static_cast<size_t>(rbx) * rby * sizeof(float));
        bar = reinterpret_cast<uint64_t*>(g);
        hinv = reinterpret_cast<double*>(g + 16);
        ints = reinterpret_cast<int*>(g + 16 + static_cast<size_t>(mat) * sizeof(double));
        g += round128(16 + static_cast<size_t>(mat) * sizeof(double) + 32);
        red = reinterpret_cast<T*>(g);
        sm = red + 64 * G;
    }
};

constexpr int kDriftMargin = 3;  // px of parameter drift covered by the staged coefficient window

// Warp this thread's samples, interpolate from the staged coefficient window (global memory for
// a stencil outside it), store g (and for FGN the spline gradient), accumulate the shifted
// normalisation sums.  Returns false if a warped point left the image.
// NP = 12: the second-order warp (icgn.cpp:167-182); SUMS = false (SSD): no normalisation sums;
// s_chk (masked subsets): samples whose entry is NaN lie outside the ROI and are skipped.
template <int DEG, typename T, bool GRAD, int NP = 6, bool SUMS = true>
__device__ __forceinline__ bool warp_interp(const Env<T>& e, int cx, int cy, const T (&p)[NP], T fm, T* s_g, T* s_gx,
                                            T* s_gy, const short2* off, const T* cwin, int wc0, int wr0, int tid,
                                            int nt, Kahan<T>& sg, Kahan<T>& sg2, const T* s_chk = nullptr) {
    const int ww = cwin ? e.cbx : 0, wh = cwin ? e.cby : 0;  // no window: every stencil from global memory
    constexpr int NB = DEG + 1, OFF = DEG / 2;
    // window position of the stencil corner of a sample at integer offset (ix, iy) from the centre
    const int lc0 = cx + e.border - OFF - wc0, lr0 = cy + e.border - OFF - wr0;
    const bool has_win = cwin != nullptr;
    const unsigned uw = has_win ? static_cast<unsigned>(ww - NB) : 0u, uh = has_win ? static_cast<unsigned>(wh - NB) : 0u;
    bool ok = true;
    const T xlo = T(-cx), ylo = T(-cy), xhi = T(e.w - 1 - cx), yhi = T(e.h - 1 - cy);
#pragma unroll 2
    for (int i = tid; i < e.n; i += nt) {
        if (s_chk != nullptr && isnan(s_chk[i])) continue;
        const short2 o = off[i];
        const T lx = T(o.x), ly = T(o.y);
        T tx = ((lx + p[0]) + p[2] * lx) + p[3] * ly;
        T ty = ((ly + p[1]) + p[4] * lx) + p[5] * ly;
        if constexpr (NP == 12) {
            const T x2 = lx * lx * T(0.5), xy = lx * ly, y2 = ly * ly * T(0.5);
            tx = ((tx + p[6] * x2) + p[7] * xy) + p[8] * y2;
            ty = ((ty + p[9] * x2) + p[10] * xy) + p[11] * y2;
        }
        if (!(tx >= xlo && ty >= ylo && tx <= xhi && ty <= yhi)) { ok = false; continue; }
        const T fx = floor(tx), fy = floor(ty);
        const int ix = static_cast<int>(fx), iy = static_cast<int>(fy);
        const T dx = tx - fx, dy = ty - fy;
        T wx[NB], wy[NB];
        weights<DEG, T>(dx, wx);
        weights<DEG, T>(dy, wy);
        const int lc = ix + lc0, lr = iy + lr0;  // stencil corner in the window
        T c[NB][NB];
        // a window, 0 <= lc <= ww - NB and 0 <= lr <= wh - NB (unsigned compares)
        if (has_win && static_cast<unsigned>(lc) <= uw && static_cast<unsigned>(lr) <= uh) {
            const T* b = cwin + lr * ww + lc;
#pragma unroll
            for (int m = 0; m < NB; ++m)
#pragma unroll
                for (int q = 0; q < NB; ++q) c[m][q] = b[m * ww + q];
        } else {
            const int col = lc + wc0, row = lr + wr0;  // stencil corner in the coefficient image
            const T* b = e.coef + static_cast<size_t>(row) * e.cpitch + col;
#pragma unroll
            for (int m = 0; m < NB; ++m)
#pragma unroll
                for (int q = 0; q < NB; ++q) c[m][q] = __ldg(b + m * e.cpitch + q);
        }
        T g = T(0);
#pragma unroll
        for (int m = 0; m < NB; ++m) {
            T rs = T(0);
#pragma unroll
            for (int q = 0; q < NB; ++q) rs += wx[q] * c[m][q];
            g += wy[m] * rs;
        }
        s_g[i] = g;
        if constexpr (GRAD) {
            T dwx[NB], dwy[NB];
            dweights<DEG, T>(dx, dwx);
            dweights<DEG, T>(dy, dwy);
            T gx = T(0), gy = T(0);
#pragma unroll
            for (int m = 0; m < NB; ++m) {
                T rx = T(0), r0 = T(0);
#pragma unroll
                for (int q = 0; q < NB; ++q) { rx += dwx[q] * c[m][q]; r0 += wx[q] * c[m][q]; }
                gx += wy[m] * rx;
                gy += dwy[m] * r0;
            }
            s_gx[i] = gx;
            s_gy[i] = gy;
        }
        if constexpr (SUMS) {
            const T gs = g - fm;
            sg.add(gs);
            sg2.add(gs * gs);
        }
    }
    return ok;
}

template <typename M>
__device__ __forceinline__ void hessian_from_sums(const M (&S)[18], M scale, M (&Hm)[6][6]) {
    // S(u, v) with u in {aa, ab, bb}, v in {1, lx, ly, lx^2, lx ly, ly^2}; SD = [a, b, a lx, a ly, b lx, b ly]
    auto s = [&](int u, int v) { return S[u * 6 + v]; };
    Hm[0][0] = s(0, 0); Hm[0][1] = s(1, 0); Hm[0][2] = s(0, 1); Hm[0][3] = s(0, 2); Hm[0][4] = s(1, 1); Hm[0][5] = s(1, 2);
    Hm[1][1] = s(2, 0); Hm[1][2] = s(1, 1); Hm[1][3] = s(1, 2); Hm[1][4] = s(2, 1); Hm[1][5] = s(2, 2);
    Hm[2][2] = s(0, 3); Hm[2][3] = s(0, 4); Hm[2][4] = s(1, 3); Hm[2][5] = s(1, 4);
    Hm[3][3] = s(0, 5); Hm[3][4] = s(1, 4); Hm[3][5] = s(1, 5);
    Hm[4][4] = s(2, 3); Hm[4][5] = s(2, 4);
    Hm[5][5] = s(2, 5);
#pragma unroll
    for (int i = 0; i < 6; ++i)
#pragma unroll
        for (int j = i; j < 6; ++j) { Hm[i][j] *= scale; Hm[j][i] = Hm[i][j]; }
}

// TMA staging of one POI: thread 0 issues two 2-D tensor loads on the group's mbarrier, the
// reference window (subset + one-pixel halo, x rounded down to 16 bytes) and the coefficient
// window under the subset warped by the initial guess (+ drift margin, spline stencil).  The
// wait is bounded: on timeout the error word is set and false returned (the copy may still
// land in shared memory, so the kernel must leave).
template <int DEG, typename T, int G, typename M>
__device__ __forceinline__ bool stage_windows(const Env<T>& e, const CUtensorMap* tm_ref, const CUtensorMap* tm_coef,
                                              int cx, int cy, const M (&p0)[6], const GroupSmem<T>& gs,
                                              uint32_t& phase, int tid, int bar_id, int& rx0, int& ry0, int& wc0,
                                              int& wr0, bool with_coef = true, const int* acquire_state = nullptr,
                                              bool early = false) {
    constexpr int OFF = DEG / 2;
    const int r = e.radius;
    rx0 = floor_to(cx - r - 1, 4);  // 16-byte aligned x (float)
    ry0 = cy - r - 1;
    constexpr int kAlign = 16 / static_cast<int>(sizeof(T));
    {
        // the box only needs the warped corners to a pixel (the drift margin is 3 px): float
        // arithmetic keeps this off the GB300's narrow FP64 pipe
        const float q0 = static_cast<float>(p0[0]), q1 = static_cast<float>(p0[1]), q2 = static_cast<float>(p0[2]),
                    q3 = static_cast<float>(p0[3]), q4 = static_cast<float>(p0[4]), q5 = static_cast<float>(p0[5]);  // no-ops on the FP32 path
        const float rf = static_cast<float>(r);
        const float ax = fabsf(q2) * rf + fabsf(q3) * rf, ay = fabsf(q4) * rf + fabsf(q5) * rf;
        const float txmin = -rf + q0 - ax, tymin = -rf + q1 - ay;
        const float txmax = rf + q0 + ax, tymax = rf + q1 + ay;
        // a non-finite or absurd guess stages an arbitrary in-range box; samples outside it
        // read global memory (and warps leaving the image end the solve anyway)
        const bool sane = txmin > -1e6f && txmax < 1e6f && tymin > -1e6f && tymax < 1e6f;
        const int c0 = sane ? cx + static_cast<int>(floorf(txmin)) - kDriftMargin + e.border - OFF : 0;
        const int r0 = sane ? cy + static_cast<int>(floorf(tymin)) - kDriftMargin + e.border - OFF : 0;
        wc0 = floor_to(min(max(c0, -e.cbx), e.cw), kAlign);
        wr0 = min(max(r0, -e.cby), e.h + 2 * e.border);
    }
    // early: the caller's every read of the windows precedes a group barrier it has passed, so
    // thread 0 issues the copies at once; the barrier below then publishes what thread 0 read
    // with acquire order (acquire_state -> ints[4]) while the copies are in flight
    if (!early) group_sync<G>(bar_id);  // previous readers of the windows are done
    const bool coef = with_coef && gs.cwin != nullptr;
    if (tid == 0) {
        fence_proxy_async();
        mbar_expect_tx(gs.bar, static_cast<uint32_t>(e.rbx * e.rby * sizeof(float) +
                                                     (coef ? e.cbx * e.cby * sizeof(T) : 0)));
        tma_load_2d(gs.rwin, tm_ref, rx0, ry0, gs.bar);
        if (coef) tma_load_2d(gs.cwin, tm_coef, wc0, wr0, gs.bar);
        if (acquire_state != nullptr) gs.ints[4] = ld_acquire_s32(acquire_state);
    }
    if (early) group_sync<G>(bar_id);
    long long spins = 0;
    while (!mbar_try_wait(gs.bar, phase)) {
        if (++spins > kTmaSpinLimit) {
            atomicExch(e.err, 3);
            return false;
        }
    }
    phase ^= 1u;
    return true;
}

// Products that must round on their own (no contraction into a following add), so that a value
// recomputed in a register equals the one the full staging mode stores and reloads.
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }

// Reference sample at (x, y) from the staged reference window: the raw value and the gradient of
// the reference gradient cache (reliability_propagation.cpp:84-112: central differences, one-sided
// at the image border; multiplying by 0.5 or 1 is exact).
template <typename T>
__device__ __forceinline__ void ref_gradient(const float* rwin, int rww, int rx0, int ry0, int W, int H, int x, int y,
                                             T& a, T& b) {
    const int xm = max(0, x - 1), xp = min(W - 1, x + 1), ym = max(0, y - 1), yp = min(H - 1, y + 1);
    a = (T(rwin[(y - ry0) * rww + (xp - rx0)]) - T(rwin[(y - ry0) * rww + (xm - rx0)])) *
        (xp - xm == 2 ? T(0.5) : T(1));
    b = (T(rwin[(yp - ry0) * rww + (x - rx0)]) - T(rwin[(ym - ry0) * rww + (x - rx0)])) *
        (yp - ym == 2 ? T(0.5) : T(1));
}

// The reference side of a solve (icgn.cpp:470-545; forward_gauss_newton.cpp:230-262): the
// subset's mean and norm from compensated shifted sums and, for ICGN, the Hessian from 18 sums
// and its inverse in the group's s_hinv.  With `store`, the raw reference values and (ICGN) the
// reference gradients go to s_fn, s_a, s_b and f^ is formed in s_fn.  Returns TDIC_SUCCESS or
// TDIC_NUMERICAL_FAILURE.  A solve and the set-up precompute run this same code, so a cached
// set-up holds the values the solve would compute.
template <int OPT, int G, typename T, typename M>
__device__ __forceinline__ int ref_setup(const Env<T>& e, const short2* off, int cx, int cy, const GroupSmem<T>& gs,
                                         int rx0, int ry0, bool store, T* s_fn, T* s_a, T* s_b, int& rp, int tid,
                                         int bar_id, T& fm, T& inv_norm) {
    constexpr int NT = 32 * G;
    M* s_hinv = reinterpret_cast<M*>(gs.hinv);
    T* red = gs.red;
    const int W = e.w, H = e.h, rww = e.rbx;
    const float fshift = gs.rwin[(cy - ry0) * rww + (cx - rx0)];  // centre pixel: sums of f - fshift
    Kahan<T> k1, k2;
    T hs[18];
#pragma unroll
    for (int k = 0; k < 18; ++k) hs[k] = T(0);
    for (int i = tid; i < e.n; i += NT) {
        const short2 o = off[i];
        const int x = cx + o.x, y = cy + o.y;
        const float f = gs.rwin[(y - ry0) * rww + (x - rx0)];
        if (store) s_fn[i] = T(f);
        const T fd = T(f) - T(fshift);
        k1.add(fd);
        k2.add(fd * fd);
        if constexpr (OPT == 0) {
            T a, b;
            ref_gradient<T>(gs.rwin, rww, rx0, ry0, W, H, x, y, a, b);
            if (store) {
                s_a[i] = a;
                s_b[i] = b;
            }
            const T lx = T(o.x), ly = T(o.y);
            const T q[3] = {a * a, a * b, b * b};
            const T m6[6] = {T(1), lx, ly, lx * lx, lx * ly, ly * ly};
#pragma unroll
            for (int u = 0; u < 3; ++u)
#pragma unroll
                for (int v = 0; v < 6; ++v) hs[u * 6 + v] += q[u] * m6[v];
        }
    }
    T v20[20];
    v20[0] = k1.value();
    v20[1] = k2.value();
#pragma unroll
    for (int k = 0; k < 18; ++k) v20[2 + k] = hs[k];
    if constexpr (OPT == 0) {
        group_sum<G, 20>(v20, red, rp, tid, bar_id);
    } else {
        T v2s[2] = {v20[0], v20[1]};
        group_sum<G, 2>(v2s, red, rp, tid, bar_id);
        v20[0] = v2s[0];
        v20[1] = v2s[1];
    }
    // normalisation: mean = shift + S1/N, sum (f - mean)^2 = S2 - S1 * (S1/N), the latter as one
    // fused multiply-add (a single rounding of the exact difference); the compensated sums
    // S1, S2 carry the accuracy.
    const M inv_n = M(e.inv_n);
    const M s1 = static_cast<M>(v20[0]), s2 = static_cast<M>(v20[1]);
    const M mshift = s1 * inv_n;
    const M ss = fma(-s1, mshift, s2);
    if (!(ss > M(kEps * kEps))) return TDIC_NUMERICAL_FAILURE;  // |f - mean| <= 1e-12
    fm = T(M(fshift) + mshift);
    inv_norm = T(1) / sqrt(T(ss));
    if (store)
        for (int i = tid; i < e.n; i += NT) s_fn[i] = mul_rn(s_fn[i] - fm, inv_norm);
    if constexpr (OPT == 0) {
        M S[18];
#pragma unroll
        for (int k = 0; k < 18; ++k) S[k] = static_cast<M>(v20[2 + k]);
        M Hm[6][6];
        hessian_from_sums<M>(S, M(2) * inv_norm * inv_norm, Hm);
        if (!factor_inverse<G, M>(Hm, s_hinv, tid, bar_id)) return TDIC_NUMERICAL_FAILURE;
    }
    return TDIC_SUCCESS;
}

// Fill the set-up cache entry of grid point `idx` at (cx, cy) (ICGN, first-order ZNSSD): stage the
// reference window, run ref_setup, store the inverse Hessian, mean and norm, then publish the
// state with release semantics.  Points the solve never sets up (outside the margin, too few
// samples) are left alone.  Returns false only when the TMA wait timed out.
template <int DEG, typename T, int G>
__device__ bool precompute_setup(const Env<T>& e, const CUtensorMap* tm_ref, const short2* off, int cx, int cy,
                                 const GroupSmem<T>& gs, uint32_t& phase, int tid, int bar_id, int idx) {
    using M = typename MixedOf<T>::type;
    constexpr int NT = 32 * G;
    const int r = e.radius;
    if (e.w <= 0 || r < 1 || e.max_iter < 0 || e.n < 6) return true;
    if (cx - r < 0 || cy - r < 0 || cx + r >= e.w || cy + r >= e.h) return true;
    const M p0[6] = {M(0), M(0), M(0), M(0), M(0), M(0)};
    int rx0, ry0, wc0, wr0;
    if (!stage_windows<DEG, T, G, M>(e, tm_ref, nullptr, cx, cy, p0, gs, phase, tid, bar_id, rx0, ry0, wc0, wr0,
                                     false))
        return false;
    int rp = 0;
    T fm, inv_norm;
    const int st = ref_setup<0, G, T, M>(e, off, cx, cy, gs, rx0, ry0, false, nullptr, nullptr, nullptr, rp, tid,
                                         bar_id, fm, inv_norm);
    group_sync<G>(bar_id);  // the inverse is complete in shared memory
    if (st == TDIC_SUCCESS) {
        const M* s_hinv = reinterpret_cast<const M*>(gs.hinv);
        M* hin = reinterpret_cast<M*>(e.sc_hinv) + 36 * static_cast<size_t>(idx);
        for (int k = tid; k < 36; k += NT) hin[k] = s_hinv[k];
        if (tid == 0) {
            e.sc_fmn[2 * static_cast<size_t>(idx)] = fm;
            e.sc_fmn[2 * static_cast<size_t>(idx) + 1] = inv_norm;
        }
    }
    group_sync<G>(bar_id);  // every thread's stores precede thread 0's release
    if (tid == 0) {
        __threadfence();
        st_release_s32(e.sc_state + idx, st == TDIC_SUCCESS ? 1 : 2);
    }
    return true;
}

// The per-POI solve.  OPT 0 = ICGN (icgn.cpp:446-627), 1 = FGN (forward_gauss_newton.cpp:188-399).
// `off` is the sample-offset table in shared memory; `phase` the parity of the group's
// mbarrier (flips once per staged POI).  Returns false only when a TMA wait timed out (the
// kernel must then leave: the copy may still land in shared memory).
template <int OPT, int DEG, typename T, int G>
__device__ bool solve_poi(const Env<T>& e, const CUtensorMap* tm_ref, const CUtensorMap* tm_coef, const short2* off,
                          int cx, int cy, const typename MixedOf<T>::type (&p0)[6],
                          typename MixedOf<T>::type conf, const GroupSmem<T>& gs, uint32_t& phase, int tid,
                          int bar_id, Result<typename MixedOf<T>::type>& R, int sc_idx = -1) {
    using M = typename MixedOf<T>::type;
    constexpr int NT = 32 * G;
    M* s_hinv = reinterpret_cast<M*>(gs.hinv);
    T* red = gs.red;
    result_init(R, p0, conf);
    int rp = 0;  // reduction-buffer parity
    const int r = e.radius;
    if (e.w <= 0 || r < 1 || e.max_iter < 0) return true;
    if (cx - r < 0 || cy - r < 0 || cx + r >= e.w || cy + r >= e.h) return true;
    if (e.n < 6) return true;
    // per-sample arrays (full staging: f^, gradients, g; lean: what the iterations write)
    const bool lean = (gs.stage & kStageLean) != 0;
    T* s_fn = lean ? nullptr : gs.sm;
    T* s_a = lean ? (OPT == 1 ? gs.sm : nullptr) : gs.sm + e.nmax;            // ICGN: reference gx; FGN: deformed gx
    T* s_b = lean ? (OPT == 1 ? gs.sm + e.nmax : nullptr) : gs.sm + 2 * e.nmax;  // ICGN: reference gy; FGN: deformed gy
    T* s_g = lean ? (OPT == 1 ? gs.sm + 2 * e.nmax : gs.sm) : gs.sm + 3 * e.nmax;
    const int W = e.w, H = e.h;

    // a cached set-up of this grid point (ICGN): thread 0 reads its state while the staging
    // copies fly, and the staging's barrier publishes it to the group (one decision for the
    // whole group).  The staging starts at once: every read of the windows by this group
    // precedes a group barrier (the reductions of the set-up and of every iteration).
    const bool cache = OPT == 0 && e.sc_state != nullptr && sc_idx >= 0;
    int rx0, ry0, wc0, wr0;
    if (!stage_windows<DEG, T, G, M>(e, tm_ref, tm_coef, cx, cy, p0, gs, phase, tid, bar_id, rx0, ry0, wc0, wr0, true,
                                     cache ? e.sc_state + sc_idx : nullptr, true))
        return false;
    const int cstate = cache ? gs.ints[4] : 0;
    const int rww = e.rbx;
    T fm, inv_norm;
    if (cstate == 2) { R.status = TDIC_NUMERICAL_FAILURE; return true; }
    if (cstate == 1) {
        // the values ref_setup gives, computed by another group: mean, norm, inverse Hessian
        fm = __ldcg(e.sc_fmn + 2 * static_cast<size_t>(sc_idx));
        inv_norm = __ldcg(e.sc_fmn + 2 * static_cast<size_t>(sc_idx) + 1);
        const M* hin = reinterpret_cast<const M*>(e.sc_hinv) + 36 * static_cast<size_t>(sc_idx);
        for (int k = tid; k < 36; k += NT) s_hinv[k] = __ldcg(hin + k);
        if (!lean)
            for (int i = tid; i < e.n; i += NT) {
                const short2 o = off[i];
                const int x = cx + o.x, y = cy + o.y;
                s_fn[i] = mul_rn(T(gs.rwin[(y - ry0) * rww + (x - rx0)]) - fm, inv_norm);
                T a, b;
                ref_gradient<T>(gs.rwin, rww, rx0, ry0, W, H, x, y, a, b);
                s_a[i] = a;
                s_b[i] = b;
            }
    } else {
        const int st = ref_setup<OPT, G, T, M>(e, off, cx, cy, gs, rx0, ry0, !lean, s_fn, s_a, s_b, rp, tid, bar_id,
                                               fm, inv_norm);
        if (st != TDIC_SUCCESS) { R.status = st; return true; }
    }
    const M inv_n = M(e.inv_n), thr = M(e.thr);
    group_sync<G>(bar_id);  // f^ (and the inverse) visible to the whole group
    if (cache && cstate == 0 && tid < 32) {
        // publish this set-up for later solves of the point (warp 0; the others go on)
        M* hin = reinterpret_cast<M*>(e.sc_hinv) + 36 * static_cast<size_t>(sc_idx);
        for (int k = tid; k < 36; k += 32) hin[k] = s_hinv[k];
        if (tid == 0) {
            e.sc_fmn[2 * static_cast<size_t>(sc_idx)] = fm;
            e.sc_fmn[2 * static_cast<size_t>(sc_idx) + 1] = inv_norm;
        }
        __syncwarp();
        if (tid == 0) {
            __threadfence();
            st_release_s32(e.sc_state + sc_idx, 1);
        }
    }

    M p[6];
    for (int k = 0; k < 6; ++k) p[k] = p0[k];
    M corr = M(INFINITY);
    bool converged = false;
    const M gscale = M(2) * inv_norm;
    for (int it = 0; it < e.max_iter; ++it) {
        R.iters = it + 1;
        T pt[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) pt[k] = static_cast<T>(p[k]);
        Kahan<T> sg, sg2;
        const bool ok = warp_interp<DEG, T, OPT == 1>(e, cx, cy, pt, fm, s_g, s_a, s_b, off, gs.cwin, wc0, wr0, tid,
                                                      NT, sg, sg2);
        // one reduction carries the two normalisation sums and the out-of-image count
        T v3[3] = {sg.value(), sg2.value(), ok ? T(0) : T(1)};
        group_sum<G, 3>(v3, red, rp, tid, bar_id);
        if (v3[2] != T(0)) { R.status = TDIC_INVALID_INPUT; return true; }
        // mean of (g - fm) and sum (g - mean)^2, as in the set-up
        const M gmr = static_cast<M>(v3[0]) * inv_n;
        const M var = fma(-static_cast<M>(v3[0]), gmr, static_cast<M>(v3[1]));
        if (!(var > M(kEps * kEps))) { R.status = TDIC_NUMERICAL_FAILURE; return true; }  // |g - mean| <= 1e-12
        const T gsh = T(gmr);
        const T inv_gn = T(1) / sqrt(T(var));
        M dp[6];
        if constexpr (OPT == 0) {
            T q[7];
#pragma unroll
            for (int k = 0; k < 7; ++k) q[k] = T(0);
            if (!lean) {
                for (int i = tid; i < e.n; i += NT) {
                    const short2 o = off[i];
                    const T lx = T(o.x), ly = T(o.y);
                    const T diff = s_fn[i] - ((s_g[i] - fm) - gsh) * inv_gn;
                    const T da = diff * s_a[i], db = diff * s_b[i];
                    q[0] += da; q[1] += db; q[2] += da * lx; q[3] += da * ly; q[4] += db * lx; q[5] += db * ly;
                    q[6] += diff * diff;
                }
            } else {
                // f^ and the reference gradients from the staged window, as the set-up made them
                for (int i = tid; i < e.n; i += NT) {
                    const short2 o = off[i];
                    const int x = cx + o.x, y = cy + o.y;
                    const T lx = T(o.x), ly = T(o.y);
                    const T fn = mul_rn(T(gs.rwin[(y - ry0) * rww + (x - rx0)]) - fm, inv_norm);
                    T a, b;
                    ref_gradient<T>(gs.rwin, rww, rx0, ry0, W, H, x, y, a, b);
                    const T diff = fn - ((s_g[i] - fm) - gsh) * inv_gn;
                    const T da = diff * a, db = diff * b;
                    q[0] += da; q[1] += db; q[2] += da * lx; q[3] += da * ly; q[4] += db * lx; q[5] += db * ly;
                    q[6] += diff * diff;
                }
            }
            group_sum<G, 7>(q, red, rp, tid, bar_id);
            corr = static_cast<M>(q[6]);
            M grad[6];
#pragma unroll
            for (int k = 0; k < 6; ++k) grad[k] = static_cast<M>(q[k]) * gscale;
#pragma unroll
            for (int i = 0; i < 6; ++i) {
                M sacc = M(0);
#pragma unroll
                for (int j = 0; j < 6; ++j) sacc += s_hinv[i * 6 + j] * grad[j];
                dp[i] = -sacc;
            }
        } else {
            // FGN: SD from the deformed spline gradient through dW/dz (forward_gauss_newton.cpp:44-60)
            const T p2 = pt[2], p3 = pt[3], p4 = pt[4], p5 = pt[5];
            T q[25];
#pragma unroll
            for (int k = 0; k < 25; ++k) q[k] = T(0);
            for (int i = tid; i < e.n; i += NT) {
                const short2 o = off[i];
                const T lx = T(o.x), ly = T(o.y);
                const T gx = s_a[i], gy = s_b[i];
                const T ae = gx * (T(1) + p2) + gy * p4;
                const T be = gx * p3 + gy * (T(1) + p5);
                const T fn = lean ? mul_rn(T(gs.rwin[(cy + o.y - ry0) * rww + (cx + o.x - rx0)]) - fm, inv_norm)
                                  : s_fn[i];
                const T diff = fn - ((s_g[i] - fm) - gsh) * inv_gn;
                const T qq[3] = {ae * ae, ae * be, be * be};
                const T m6[6] = {T(1), lx, ly, lx * lx, lx * ly, ly * ly};
#pragma unroll
                for (int u = 0; u < 3; ++u)
#pragma unroll
                    for (int v = 0; v < 6; ++v) q[u * 6 + v] += qq[u] * m6[v];
                const T da = diff * ae, db = diff * be;
                q[18] += da; q[19] += db; q[20] += da * lx; q[21] += da * ly; q[22] += db * lx; q[23] += db * ly;
                q[24] += diff * diff;
            }
            group_sum<G, 25>(q, red, rp, tid, bar_id);
            corr = static_cast<M>(q[24]);
            M S[18];
#pragma unroll
            for (int k = 0; k < 18; ++k) S[k] = static_cast<M>(q[k]);
            M Hm[6][6];
            hessian_from_sums<M>(S, M(2) * inv_norm * inv_norm, Hm);
            M grad[6];
#pragma unroll
            for (int k = 0; k < 6; ++k) grad[k] = static_cast<M>(q[18 + k]) * gscale;
            if (!factor_solve<G, M>(Hm, grad, dp)) { R.status = TDIC_NUMERICAL_FAILURE; return true; }
        }
        if (!finite6(dp)) { R.status = TDIC_NUMERICAL_FAILURE; return true; }
        M dn2 = M(0);
#pragma unroll
        for (int k = 0; k < 6; ++k) dn2 += dp[k] * dp[k];
        M dn = sqrt(dn2);
        M pn[6];
        if constexpr (OPT == 0) {
            ic_update<M>(p, dp, pn);
        } else {
            if (dn > M(0.5)) {  // forward_gauss_newton.cpp:367-371
                const M sc = M(0.5) / dn;
#pragma unroll
                for (int k = 0; k < 6; ++k) dp[k] *= sc;
                dn = M(0.5);
            }
            compose_warp<M>(p, dp, pn);
        }
#pragma unroll
        for (int k = 0; k < 6; ++k) p[k] = pn[k];
        if (!finite6(p)) { R.status = TDIC_NUMERICAL_FAILURE; return true; }
        if (dn < thr) { converged = true; break; }
    }
    for (int k = 0; k < 6; ++k) R.p[k] = p[k];
    R.corr = corr;
    R.conv = converged;
    if (!converged && isfinite(corr)) converged = true;
    R.status = converged ? TDIC_SUCCESS : TDIC_NOT_CONVERGED;
    R.valid = converged;
    return true;
}

// The other solver routes, VAR bit 0: SSD objective, bit 1: second-order shape function.
//   ICGN icgn.cpp:832-988 (first-order SSD), 1168-1362 (second-order ZNSSD), 1576-1739 (SSD)
//   FGN  forward_gauss_newton.cpp:622-794, 1069-1297, 1540-1739
// Same staging, sample loop, group reductions and precision split as solve_poi.  SSD works on
// raw values: residual f - g, Hessian and gradient without the 2/|f| factors, no normalisation
// sums.  Second order adds the six curvature terms to the warp and the steepest descent; the
// 12x12 Hessian comes from 45 sums (3 gradient products x 15 monomials of degree <= 4) and is
// factorised by the group in shared memory, ICGN once (its inverse kept), FGN every iteration
// after the 1e-4 max-diagonal damping term (forward_gauss_newton.cpp:1242-1245); the update is
// ic_update2 / compose_warp2.  FGN caps the step at 0.5 (ZNSSD) or 0.35 (SSD); first-order SSD
// tests convergence on the norm before the cap (forward_gauss_newton.cpp:764, 774).
template <int OPT, int DEG, typename T, int G, int VAR>
__device__ bool solve_poi_var(const Env<T>& e, const CUtensorMap* tm_ref, const CUtensorMap* tm_coef,
                              const short2* off, int cx, int cy, const typename MixedOf<T>::type (&p0)[6],
                              typename MixedOf<T>::type conf, const GroupSmem<T>& gs, uint32_t& phase, int tid,
                              int bar_id, Result<typename MixedOf<T>::type>& R) {
    using M = typename MixedOf<T>::type;
    constexpr bool SSD = (VAR & 1) != 0;
    constexpr int NP = (VAR & 2) ? 12 : 6;
    constexpr int NM = NP == 12 ? 15 : 6;  // monomials of the Hessian sums
    constexpr int NH = 3 * NM;             // sums: (aa, ab, bb) x monomials
    constexpr int NT = 32 * G;
    // matrix region: 6x6 inverse | A (144) B (144) 1/D (12) S (45) for 12x12
    M* mat = reinterpret_cast<M*>(gs.hinv);
    M* mA = mat;
    M* mB = mat + 144;
    M* mD = mat + 288;
    M* mS = mat + 300;
    T* red = gs.red;
    result_init(R, p0, conf);
    int rp = 0;
    const int r = e.radius;
    // masked subsets (solve_with_mask, icgn.cpp:629-704 and siblings): the centre must be a ROI
    // pixel (no margin check); samples outside the image or the ROI are left out (marked NaN in
    // s_fn) and at least e.min_keep must remain
    const bool masked = e.roi != nullptr;
    if (e.w <= 0 || r < 1 || e.max_iter < 0) return true;
    if (masked) {
        if (cx < 0 || cy < 0 || cx >= e.w || cy >= e.h || e.roi[static_cast<size_t>(cy) * e.w + cx] == 0) return true;
    } else {
        if (cx - r < 0 || cy - r < 0 || cx + r >= e.w || cy + r >= e.h) return true;
        if (e.n < NP) return true;
    }
    T* s_fn = gs.sm;              // ZNSSD: normalised reference f^; SSD: raw f
    T* s_a = gs.sm + e.nmax;      // ICGN: reference gx; FGN: deformed gx
    T* s_b = gs.sm + 2 * e.nmax;  // ICGN: reference gy; FGN: deformed gy
    T* s_g = gs.sm + 3 * e.nmax;
    const int W = e.w, H = e.h;

    int rx0, ry0, wc0, wr0;
    if (!stage_windows<DEG, T, G, M>(e, tm_ref, tm_coef, cx, cy, p0, gs, phase, tid, bar_id, rx0, ry0, wc0, wr0))
        return false;

    // --- set-up pass: reference values, (ZNSSD) shifted sums, (ICGN) gradients and Hessian sums
    const int rww = e.rbx;
    const float fshift = gs.rwin[(cy - ry0) * rww + (cx - rx0)];
    Kahan<T> k1, k2;
    T hs[NH];
#pragma unroll
    for (int k = 0; k < NH; ++k) hs[k] = T(0);
    T kept = T(0);
    for (int i = tid; i < e.n; i += NT) {
        const short2 o = off[i];
        const int x = cx + o.x, y = cy + o.y;
        if (masked && (x < 0 || y < 0 || x >= W || y >= H || e.roi[static_cast<size_t>(y) * W + x] == 0)) {
            s_fn[i] = T(NAN);
            continue;
        }
        kept += T(1);
        const float f = gs.rwin[(y - ry0) * rww + (x - rx0)];
        s_fn[i] = T(f);
        if constexpr (!SSD) {
            const T fd = T(f) - T(fshift);
            k1.add(fd);
            k2.add(fd * fd);
        }
        if constexpr (OPT == 0) {
            // reference gradient cache, reliability_propagation.cpp:84-112
            const int xm = max(0, x - 1), xp = min(W - 1, x + 1), ym = max(0, y - 1), yp = min(H - 1, y + 1);
            const T a = (T(gs.rwin[(y - ry0) * rww + (xp - rx0)]) - T(gs.rwin[(y - ry0) * rww + (xm - rx0)])) *
                        (xp - xm == 2 ? T(0.5) : T(1));
            const T b = (T(gs.rwin[(yp - ry0) * rww + (x - rx0)]) - T(gs.rwin[(ym - ry0) * rww + (x - rx0)])) *
                        (yp - ym == 2 ? T(0.5) : T(1));
            s_a[i] = a;
            s_b[i] = b;
            const T lx = T(o.x), ly = T(o.y);
            const T q[3] = {a * a, a * b, b * b};
            T m[NM];
            if constexpr (NP == 12) {
                monomials15<T>(lx, ly, m);
            } else {
                m[0] = T(1); m[1] = lx; m[2] = ly; m[3] = lx * lx; m[4] = lx * ly; m[5] = ly * ly;
            }
#pragma unroll
            for (int u = 0; u < 3; ++u)
#pragma unroll
                for (int v = 0; v < NM; ++v) hs[u * NM + v] += q[u] * m[v];
        }
    }
    // one reduction: (ZNSSD) the two shifted sums, (ICGN) the Hessian sums, the kept count
    constexpr int KS = SSD ? 0 : 2, KH = OPT == 0 ? NH : 0, K0 = KS + KH + 1;
    T v0[K0];
    if constexpr (KS > 0) {
        v0[0] = k1.value();
        v0[1] = k2.value();
    }
    if constexpr (KH > 0) {
#pragma unroll
        for (int k = 0; k < NH; ++k) v0[KS + k] = hs[k];
    }
    v0[K0 - 1] = kept;
    group_sum_n<G, K0, T>(v0, red, rp, tid, bar_id);
    const int nkept = static_cast<int>(v0[K0 - 1]);
    if (masked && nkept < e.min_keep) return true;  // too few ROI samples: InvalidInput
    // the reference divides by the kept count: 1 / n rounded as the host's double reciprocal
    const M inv_n = masked ? M(1.0 / static_cast<double>(nkept)) : M(e.inv_n), thr = M(e.thr);
    T fm = T(0), inv_norm = T(1);
    if constexpr (!SSD) {
        const M s1 = static_cast<M>(v0[0]), s2 = static_cast<M>(v0[1]);
        const M mshift = s1 * inv_n;
        const M ss = fma(-s1, mshift, s2);
        if (!(ss > M(kEps * kEps))) { R.status = TDIC_NUMERICAL_FAILURE; return true; }  // |f - mean| <= 1e-12
        fm = T(M(fshift) + mshift);
        inv_norm = T(1) / sqrt(T(ss));
        for (int i = tid; i < e.n; i += NT) s_fn[i] = (s_fn[i] - fm) * inv_norm;
    }
    const M hscale = SSD ? M(1) : M(2) * M(inv_norm) * M(inv_norm);
    const M gscale = SSD ? M(1) : M(2) * M(inv_norm);
    const M* hinv = mat;  // ICGN: the inverse Hessian, NP x NP row-major
    if constexpr (OPT == 0) {
        if constexpr (NP == 6) {
            M S[18];
#pragma unroll
            for (int k = 0; k < 18; ++k) S[k] = static_cast<M>(v0[KS + k]);
            M Hm[6][6];
            hessian_from_sums<M>(S, hscale, Hm);
            if (!factor_inverse<G, M>(Hm, mat, tid, bar_id)) { R.status = TDIC_NUMERICAL_FAILURE; return true; }
        } else {
            for (int t = tid; t < NH; t += NT) {  // NT may be 32 < 45
                M sv = M(0);
#pragma unroll
                for (int k = 0; k < NH; ++k) sv = k == t ? static_cast<M>(v0[KS + k]) : sv;
                mS[t] = sv;
            }
            group_sync<G>(bar_id);
            for (int t = tid; t < 144; t += NT) {
                const M h = hess12_entry<M>(mS, t / 12, t % 12) * hscale;
                mA[t] = h;
                mB[t] = h;
            }
            if (ldlt12_group<G, M>(mA, mD, tid, bar_id)) {
                if (tid < 12) {  // column tid of the inverse
                    M ecol[12], col[12];
#pragma unroll
                    for (int k = 0; k < 12; ++k) ecol[k] = k == tid ? M(1) : M(0);
                    ldlt12_solve<M>(mA, mD, ecol, col);
#pragma unroll
                    for (int k = 0; k < 12; ++k) mB[k * 12 + tid] = col[k];
                }
                hinv = mB;
            } else {
                // not numerically positive definite: the pivoted factorisation decides (rare)
                LdltN<12, M> g;
                g.factor(mB);
                if (!g.good()) { R.status = TDIC_NUMERICAL_FAILURE; return true; }
                group_sync<G>(bar_id);  // every thread has read B
                if (tid < 12) {
                    M ecol[12], col[12];
                    for (int k = 0; k < 12; ++k) ecol[k] = k == tid ? M(1) : M(0);
                    g.solve(ecol, col);
                    for (int k = 0; k < 12; ++k) mA[k * 12 + tid] = col[k];
                }
                hinv = mA;
            }
        }
    }
    group_sync<G>(bar_id);  // f^ (and the inverse) visible to the whole group

    M p[NP];
#pragma unroll
    for (int k = 0; k < NP; ++k) p[k] = k < 6 ? p0[k] : M(0);
    M corr = M(INFINITY);
    bool converged = false;
    for (int it = 0; it < e.max_iter; ++it) {
        R.iters = it + 1;
        T pt[NP];
#pragma unroll
        for (int k = 0; k < NP; ++k) pt[k] = static_cast<T>(p[k]);
        Kahan<T> sg, sg2;
        const bool ok = warp_interp<DEG, T, OPT == 1, NP, !SSD>(e, cx, cy, pt, fm, s_g, s_a, s_b, off, gs.cwin, wc0,
                                                                wr0, tid, NT, sg, sg2, masked ? s_fn : nullptr);
        T gsh = T(0), inv_gn = T(1);
        if constexpr (!SSD) {
            T v3[3] = {sg.value(), sg2.value(), ok ? T(0) : T(1)};
            group_sum<G, 3>(v3, red, rp, tid, bar_id);
            if (v3[2] != T(0)) { R.status = TDIC_INVALID_INPUT; return true; }
            const M gmr = static_cast<M>(v3[0]) * inv_n;
            const M var = fma(-static_cast<M>(v3[0]), gmr, static_cast<M>(v3[1]));
            if (!(var > M(kEps * kEps))) { R.status = TDIC_NUMERICAL_FAILURE; return true; }  // |g - mean| <= 1e-12
            gsh = T(gmr);
            inv_gn = T(1) / sqrt(T(var));
        } else {
            T v1[1] = {ok ? T(0) : T(1)};
            group_sum<G, 1>(v1, red, rp, tid, bar_id);
            if (v1[0] != T(0)) { R.status = TDIC_INVALID_INPUT; return true; }
        }
        M dp[NP];
        if constexpr (OPT == 0) {
            T q[NP + 1];
#pragma unroll
            for (int k = 0; k <= NP; ++k) q[k] = T(0);
            for (int i = tid; i < e.n; i += NT) {
                if (masked && isnan(s_fn[i])) continue;
                const short2 o = off[i];
                const T lx = T(o.x), ly = T(o.y);
                const T diff = SSD ? s_fn[i] - s_g[i] : s_fn[i] - ((s_g[i] - fm) - gsh) * inv_gn;
                const T da = diff * s_a[i], db = diff * s_b[i];
                q[0] += da; q[1] += db; q[2] += da * lx; q[3] += da * ly; q[4] += db * lx; q[5] += db * ly;
                if constexpr (NP == 12) {
                    const T x2 = lx * lx * T(0.5), xy = lx * ly, y2 = ly * ly * T(0.5);
                    q[6] += da * x2; q[7] += da * xy; q[8] += da * y2; q[9] += db * x2; q[10] += db * xy; q[11] += db * y2;
                }
                q[NP] += diff * diff;
            }
            group_sum_n<G, NP + 1, T>(q, red, rp, tid, bar_id);
            corr = static_cast<M>(q[NP]);
            M grad[NP];
#pragma unroll
            for (int k = 0; k < NP; ++k) grad[k] = static_cast<M>(q[k]) * gscale;
#pragma unroll
            for (int i = 0; i < NP; ++i) {
                M sacc = M(0);
#pragma unroll
                for (int j = 0; j < NP; ++j) sacc += hinv[i * NP + j] * grad[j];
                dp[i] = -sacc;
            }
        } else {
            // SD from the deformed spline gradient through dW/dz (forward_gauss_newton.cpp:44-60, 986-1019)
            constexpr int KQ = NH + NP + 1;
            T q[KQ];
#pragma unroll
            for (int k = 0; k < KQ; ++k) q[k] = T(0);
            for (int i = tid; i < e.n; i += NT) {
                if (masked && isnan(s_fn[i])) continue;
                const short2 o = off[i];
                const T lx = T(o.x), ly = T(o.y);
                const T gx = s_a[i], gy = s_b[i];
                T ae, be;
                if constexpr (NP == 6) {
                    ae = gx * (T(1) + pt[2]) + gy * pt[4];
                    be = gx * pt[3] + gy * (T(1) + pt[5]);
                } else {
                    const T a00 = T(1) + pt[2] + pt[6] * lx + pt[7] * ly;
                    const T a01 = pt[3] + pt[7] * lx + pt[8] * ly;
                    const T a10 = pt[4] + pt[9] * lx + pt[10] * ly;
                    const T a11 = T(1) + pt[5] + pt[10] * lx + pt[11] * ly;
                    ae = gx * a00 + gy * a10;
                    be = gx * a01 + gy * a11;
                }
                const T diff = SSD ? s_fn[i] - s_g[i] : s_fn[i] - ((s_g[i] - fm) - gsh) * inv_gn;
                const T qq[3] = {ae * ae, ae * be, be * be};
                T m[NM];
                if constexpr (NP == 12) {
                    monomials15<T>(lx, ly, m);
                } else {
                    m[0] = T(1); m[1] = lx; m[2] = ly; m[3] = lx * lx; m[4] = lx * ly; m[5] = ly * ly;
                }
#pragma unroll
                for (int u = 0; u < 3; ++u)
#pragma unroll
                    for (int v = 0; v < NM; ++v) q[u * NM + v] += qq[u] * m[v];
                const T da = diff * ae, db = diff * be;
                q[NH + 0] += da; q[NH + 1] += db; q[NH + 2] += da * lx; q[NH + 3] += da * ly;
                q[NH + 4] += db * lx; q[NH + 5] += db * ly;
                if constexpr (NP == 12) {
                    const T x2 = lx * lx * T(0.5), xy = lx * ly, y2 = ly * ly * T(0.5);
                    q[NH + 6] += da * x2; q[NH + 7] += da * xy; q[NH + 8] += da * y2;
                    q[NH + 9] += db * x2; q[NH + 10] += db * xy; q[NH + 11] += db * y2;
                }
                q[NH + NP] += diff * diff;
            }
            group_sum_n<G, KQ, T>(q, red, rp, tid, bar_id);
            corr = static_cast<M>(q[NH + NP]);
            M grad[NP];
#pragma unroll
            for (int k = 0; k < NP; ++k) grad[k] = static_cast<M>(q[NH + k]) * gscale;
            if constexpr (NP == 6) {
                M S[18];
#pragma unroll
                for (int k = 0; k < 18; ++k) S[k] = static_cast<M>(q[k]);
                M Hm[6][6];
                hessian_from_sums<M>(S, hscale, Hm);
                if (!factor_solve<G, M>(Hm, grad, dp)) { R.status = TDIC_NUMERICAL_FAILURE; return true; }
            } else {
                for (int t = tid; t < NH; t += NT) {  // NT may be 32 < 45
                    M sv = M(0);
#pragma unroll
                    for (int k = 0; k < NH; ++k) sv = k == t ? static_cast<M>(q[k]) : sv;
                    mS[t] = sv;
                }
                group_sync<G>(bar_id);
                M dmax = M(0);
#pragma unroll
                for (int k = 0; k < 12; ++k) {
                    const M dk = hess12_entry<M>(mS, k, k) * hscale;
                    dmax = k == 0 ? dk : fmax(dmax, dk);
                }
                // forward_gauss_newton.cpp:1242-1245, 1682-1685, 1886-1889 (not the masked ZNSSD route)
                const M lambda = (!masked || SSD) ? M(1e-4) * dmax : M(0);
                for (int t = tid; t < 144; t += NT) {
                    const int i = t / 12, j = t % 12;
                    M h = hess12_entry<M>(mS, i, j) * hscale;
                    if (i == j) h += lambda;
                    mA[t] = h;
                    mB[t] = h;
                }
                if (ldlt12_group<G, M>(mA, mD, tid, bar_id)) {
                    ldlt12_solve<M>(mA, mD, grad, dp);
                } else {
                    LdltN<12, M> g;
                    g.factor(mB);
                    if (!g.good()) { R.status = TDIC_NUMERICAL_FAILURE; return true; }
                    g.solve(grad, dp);
                }
            }
        }
        if (!finite_n<NP>(dp)) { R.status = TDIC_NUMERICAL_FAILURE; return true; }
        M dn2 = M(0);
#pragma unroll
        for (int k = 0; k < NP; ++k) dn2 += dp[k] * dp[k];
        M dn = sqrt(dn2);
        M pn[NP];
        if constexpr (OPT == 0) {
            if constexpr (NP == 6) ic_update<M>(p, dp, pn);
            else ic_update2<M>(p, dp, pn);
        } else {
            // step cap and whether convergence sees the capped norm, per route (unmasked
            // forward_gauss_newton.cpp:367-371, 763-767, 1260-1264, 1700-1705; masked 572-576,
            // 936-940, 1485-1489, 1902-1906)
            const M cap = SSD ? M(0.35) : ((masked && NP == 12) ? M(0.3) : M(0.5));
            const bool test_capped = masked ? !(NP == 12 && !SSD) : !(NP == 6 && SSD);
            if (dn > cap) {
                const M sc = cap / dn;
#pragma unroll
                for (int k = 0; k < NP; ++k) dp[k] *= sc;
                if (test_capped) dn = cap;
            }
            if constexpr (NP == 6) compose_warp<M>(p, dp, pn);
            else compose_warp2<M>(p, dp, pn);
        }
#pragma unroll
        for (int k = 0; k < NP; ++k) p[k] = pn[k];
        if (!finite_n<NP>(p)) { R.status = TDIC_NUMERICAL_FAILURE; return true; }
        if (dn < thr) { converged = true; break; }
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) R.p[k] = p[k];
    if constexpr (NP == 12) {
#pragma unroll
        for (int k = 0; k < 6; ++k) R.q[k] = p[6 + k];
    }
    R.corr = corr;
    R.conv = converged;
    if (!converged && isfinite(corr)) converged = true;
    R.status = converged ? TDIC_SUCCESS : TDIC_NOT_CONVERGED;
    R.valid = converged;
    return true;
}

// The solve of route VAR (0: first-order ZNSSD, solve_poi; else solve_poi_var).
template <int OPT, int DEG, typename T, int G, int VAR>
__device__ __forceinline__ bool solve_any(const Env<T>& e, const CUtensorMap* tm_ref, const CUtensorMap* tm_coef,
                                          const short2* off, int cx, int cy,
                                          const typename MixedOf<T>::type (&p0)[6], typename MixedOf<T>::type conf,
                                          const GroupSmem<T>& gs, uint32_t& phase, int tid, int bar_id,
                                          Result<typename MixedOf<T>::type>& R, int sc_idx = -1) {
    if constexpr (VAR == 0)
        return solve_poi<OPT, DEG, T, G>(e, tm_ref, tm_coef, off, cx, cy, p0, conf, gs, phase, tid, bar_id, R, sc_idx);
    else return solve_poi_var<OPT, DEG, T, G, VAR>(e, tm_ref, tm_coef, off, cx, cy, p0, conf, gs, phase, tid, bar_id, R);
}

template <typename M>
__device__ __forceinline__ void write_out(tdic_poi_out* o, const Result<M>& R) {
    for (int k = 0; k < 6; ++k) o->p[k] = static_cast<double>(R.p[k]);
    const double corr = static_cast<double>(R.corr);
    o->correlation = corr;
    const double z = 1.0 - 0.5 * corr;
    o->zncc = isfinite(corr) ? fmax(-1.0, fmin(1.0, z)) : -1.0;
    o->iterations = R.iters;
    o->status = static_cast<int8_t>(R.status);
    o->valid = R.valid ? 1 : 0;
    o->converged = R.conv ? 1 : 0;
    o->pad_ = 0;
    for (int k = 0; k < 6; ++k) o->q[k] = static_cast<double>(R.q[k]);
}

// Broadcast one int from group thread 0 to the group.
template <int G>
__device__ __forceinline__ int group_bcast(int v, int* slot, int tid, int bar_id) {
    if constexpr (G == 1) {
        return __shfl_sync(0xffffffffu, v, 0);
    } else {
        named_bar(bar_id, 32 * G);
        if (tid == 0) *slot = v;
        named_bar(bar_id, 32 * G);
        return *slot;
    }
}

// Broadcast three ints from group thread 0 (slots[0..2]) with one pair of barriers.
template <int G>
__device__ __forceinline__ void group_bcast3(int& a, int& b, int& c, int* slots, int tid, int bar_id) {
    if constexpr (G == 1) {
        a = __shfl_sync(0xffffffffu, a, 0);
        b = __shfl_sync(0xffffffffu, b, 0);
        c = __shfl_sync(0xffffffffu, c, 0);
    } else {
        named_bar(bar_id, 32 * G);
        if (tid == 0) { slots[0] = a; slots[1] = b; slots[2] = c; }
        named_bar(bar_id, 32 * G);
        a = slots[0];
        b = slots[1];
        c = slots[2];
    }
}

// Shared-memory shape of a launch: the sample-offset tables it stages (one per subset radius)
// and the per-group capacities (samples, reference and coefficient windows).  `total` is the
// number of grid points of all its jobs (the work-queue capacity).
struct Shape {
    const short2* tab;
    int ntab;
    int nmax, rbx, rby, cbx, cby;
    int total;
    int mat = kMat6;  // doubles of each group's matrix region
    int stage = kStageFull;  // staging mode of the groups' shared memory
    int narr = 4;            // per-sample arrays of each group (sample_arrays)
};

template <typename T>
__host__ __device__ inline Shape shape_of(const Env<T>& e, int total, int mat = kMat6) {
    return Shape{e.off, e.n, e.nmax, e.rbx, e.rby, e.cbx, e.cby, total, mat, e.stage, e.narr};
}

template <typename T, int G>
__device__ __forceinline__ GroupSmem<T> group_smem(unsigned char* smem_raw, const Shape& sh, int gi) {
    return GroupSmem<T>(smem_raw + cta_prefix_bytes(sh.ntab), gi, sh.nmax, G, sh.rbx, sh.rby, sh.cbx, sh.cby, sh.mat,
                        sh.stage, sh.narr);
}

// Kernel preamble: copy the sample-offset tables into shared memory (CTA-wide) and initialise
// each group's mbarrier.  Returns the shared tables.
template <typename T, int G>
__device__ short2* kernel_preamble(const Shape& sh, int* err, const CUtensorMap* tm_ref, const CUtensorMap* tm_coef,
                                   unsigned char* smem_raw, int gi, int tid, bool group_member = true) {
    // TMA destinations need 128-byte alignment; the layout assumes an aligned dynamic base.
    if ((smem_u32(smem_raw) & 127u) != 0u) {
        if (threadIdx.x == 0) atomicExch(err, 4);
        return nullptr;
    }
    short2* s_off = reinterpret_cast<short2*>(smem_raw);
    for (int i = threadIdx.x; i < sh.ntab; i += blockDim.x) s_off[i] = sh.tab[i];
    if (tid == 0 && group_member) {
        GroupSmem<T> gs = group_smem<T, G>(smem_raw, sh, gi);
        mbar_init(gs.bar, 1);
        fence_proxy_async();
    }
    if (threadIdx.x == 0 && tm_ref != nullptr) {
        asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(tm_ref)) : "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(tm_coef)) : "memory");
    }
    __syncthreads();
    return s_off;
}

// ---------------------------------------------------------------------------------------
// Batched solve: persistent groups pull POIs from a work counter.
// ---------------------------------------------------------------------------------------
template <int OPT, int DEG, typename T, int G, int VAR = 0>
__global__ void solve_batch_kernel(const __grid_constant__ Env<T> e, const __grid_constant__ CUtensorMap tm_ref,
                                   const __grid_constant__ CUtensorMap tm_coef, const tdic_poi_in* __restrict__ in,
                                   tdic_poi_out* __restrict__ out, int n, int* fetch) {
    using M = typename MixedOf<T>::type;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int gi = threadIdx.x / (32 * G), tid = threadIdx.x % (32 * G);
    const Shape sh = shape_of(e, 0, (VAR & 2) ? kMat12 : kMat6);
    short2* s_off = kernel_preamble<T, G>(sh, e.err, &tm_ref, &tm_coef, smem_raw, gi, tid);
    if (s_off == nullptr) return;
    GroupSmem<T> gs = group_smem<T, G>(smem_raw, sh, gi);
    int* ints = gs.ints;
    const int bar_id = 1 + gi;
    uint32_t phase = 0;
    while (true) {
        int job = 0;
        if (tid == 0) job = atomicAdd(fetch, 1);
        job = group_bcast<G>(job, ints + 1, tid, bar_id);
        if (job >= n) break;
        const tdic_poi_in pin = in[job];
        M p0[6];
        for (int k = 0; k < 6; ++k) p0[k] = static_cast<M>(pin.p0[k]);
        // icgn.cpp:472-473: std::round (halves away from zero), as CUDA's round()
        const int rx = static_cast<int>(round(pin.x)), ry = static_cast<int>(round(pin.y));
        Result<M> R;
        if (!solve_any<OPT, DEG, T, G, VAR>(e, &tm_ref, &tm_coef, s_off, rx, ry, p0, static_cast<M>(pin.confidence),
                                            gs, phase, tid, bar_id, R))
            return;  // a TMA wait timed out: e.err is set
        if (tid == 0) write_out(out + job, R);
    }
}

// ---------------------------------------------------------------------------------------
// Frontier-wave propagation (persistent, cooperative launch, own bounded grid barrier).
// ---------------------------------------------------------------------------------------
struct PropEnv {
    int gw, gh, step;
    const uint8_t* roi_grid;
    int seed_idx, seed_solve;
    double seed_p[6];
    double seed_corr;
    double max_znssd;
    tdic_grid_out out;
    int* claim;
    unsigned long long* key;
    void* params;   // six parameters per grid point, in the solve's precision
    int* order;
    int* counters;  // [0] wave-list tail, [1] queue head
    unsigned long long* qword;  // queue tail (high 32) : items in flight + 2^31 (low 32)
    int* fetch;     // per wave
    unsigned int* barrier;
    int* flags;     // [1] no seed, [2] accepted count of this job
    int* err;       // error word of the launch (a bounded wait ran out)
    int jtag;       // job index << kJobShift in queue items and wave lists (0 for one job)
    // dataflow order (mode 2)
    int mode;
    int sgx, sgy;                 // seed grid coordinates
    int* dstate;                  // 0 pending, 2 accepted, 3 rejected, 4 orphan
    int* dcnt;                    // parents resolved so far
    unsigned long long* dq;       // queue items: parent (high 32, -1 = orphan) : point (low 32)
    float* kcorr;                 // ZNSSD of accepted points (wave keys of the clean-up)
    // set-up precompute (single pair, ICGN, the Env's set-up cache): grid points in the order
    // idle solver groups set them up (nearest the seed first), their count and the ticket counter
    const int* pre_order;
    int pre_count;
    int* pre_ticket;
    // explicit tree (mode 3, a round of the heap order): every queued point is solved from its
    // tree parent and its tree children are queued after it; the raw result of every solve
    // (accepted or not) goes to the result table, the host decides acceptance
    const int* tchild_off;        // children of point n: tchild[tchild_off[n] .. tchild_off[n+1])
    const int* tchild;
    const int* tcont;             // the child the solving group continues with (-1: none)
    void* rcorr;                  // correlation of each solve, in the solve's precision
    void* rq;                     // second-order terms of each solve (6 per point), or NULL
    unsigned char* rmeta;         // status | valid << 2 | converged << 3
    int* riters;                  // iterations of each solve
};

enum { kDfPending = 0, kDfAccepted = 2, kDfRejected = 3, kDfOrphan = 4 };
enum { kModeWaves = 0, kModeDataflow = 2, kModeTree = 3 };

// A launch over several jobs (image pairs) tags the grid points of its queue items and wave
// lists with the job: point index in the low kJobShift bits, job above.
constexpr int kJobShift = 22;
constexpr int kPointMask = (1 << kJobShift) - 1;
static_assert(kMaxBatchJobs <= (1 << (31 - kJobShift)), "job index must fit above the point bits");

__device__ __forceinline__ int ld_cg(const int* p) { return __ldcg(p); }

// Grid-wide barrier over the co-resident blocks (bar: count, generation, snapshot).  With
// `snap`, the last block to arrive copies *snap into bar[2] while every other block waits, so
// all blocks read the same value after the barrier (the wave-list tail: appends of the next
// wave may start as soon as the barrier opens).
__device__ bool grid_barrier(unsigned int* bar, int* err, const int* snap = nullptr) {
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned int* vgen = bar + 1;
        const unsigned int gen = *vgen;
        __threadfence();
        const unsigned int arrived = atomicAdd(bar, 1u);
        if (arrived == gridDim.x - 1) {
            if (snap) bar[2] = static_cast<unsigned int>(*reinterpret_cast<const volatile int*>(snap));
            atomicExch(bar, 0u);
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            unsigned long long spins = 0;
            while (*vgen == gen) {
                if (++spins > kSpinLimit) { atomicExch(err, 1); break; }
                __nanosleep(32);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return *reinterpret_cast<volatile int*>(err) == 0;
}

template <typename M>
__device__ __forceinline__ void store_params(M* params, int idx, const Result<M>& R) {
    for (int k = 0; k < 6; ++k) params[static_cast<size_t>(idx) * 6 + k] = R.p[k];
}

// SO: the second-order terms are written too (the grid defaults already hold zeros for them).
template <typename M, bool SO = false>
__device__ void store_outputs(const PropEnv& pe, int idx, const Result<M>& R) {
    const tdic_grid_out& o = pe.out;
    if (o.u) o.u[idx] = static_cast<double>(R.p[0]);
    if (o.v) o.v[idx] = static_cast<double>(R.p[1]);
    if (o.du_dx) o.du_dx[idx] = static_cast<double>(R.p[2]);
    if (o.du_dy) o.du_dy[idx] = static_cast<double>(R.p[3]);
    if (o.dv_dx) o.dv_dx[idx] = static_cast<double>(R.p[4]);
    if (o.dv_dy) o.dv_dy[idx] = static_cast<double>(R.p[5]);
    const double corr = static_cast<double>(R.corr);
    if (o.correlation) o.correlation[idx] = corr;
    if (o.zncc) o.zncc[idx] = fmax(-1.0, fmin(1.0, 1.0 - 0.5 * corr));
    if (o.valid) o.valid[idx] = 1;
    if (o.status) o.status[idx] = TDIC_SUCCESS;
    if (o.iterations) o.iterations[idx] = R.iters;
    if (o.converged) o.converged[idx] = R.conv ? 1 : 0;
    if constexpr (SO) {
        if (o.d2u_dx2) o.d2u_dx2[idx] = static_cast<double>(R.q[0]);
        if (o.d2u_dxdy) o.d2u_dxdy[idx] = static_cast<double>(R.q[1]);
        if (o.d2u_dy2) o.d2u_dy2[idx] = static_cast<double>(R.q[2]);
        if (o.d2v_dx2) o.d2v_dx2[idx] = static_cast<double>(R.q[3]);
        if (o.d2v_dxdy) o.d2v_dxdy[idx] = static_cast<double>(R.q[4]);
        if (o.d2v_dy2) o.d2v_dy2[idx] = static_cast<double>(R.q[5]);
    }
}

template <typename M, bool SO = false>
__device__ void store_grid(const PropEnv& pe, M* params, int idx, const Result<M>& R) {
    store_params(params, idx, R);
    store_outputs<M, SO>(pe, idx, R);
}

// Claim the admissible 4-neighbours of accepted point n for wave `next` and offer n as their
// parent (key = float ZNSSD bits : parent index, atomicMin).  reliability_propagation.cpp:290-323.
__device__ void expand(const PropEnv& pe, int w, int h, int radius, int n, float corr, int next) {
    const int step = pe.step;
    const int nx = (n % pe.gw) * step, ny = (n / pe.gw) * step;
    const unsigned long long k = (static_cast<unsigned long long>(__float_as_uint(corr)) << 32) |
                                 static_cast<unsigned int>(n);
    const int dxs[4] = {0, step, 0, -step}, dys[4] = {-step, 0, step, 0};  // up, right, down, left
    for (int d = 0; d < 4; ++d) {
        const int mx = nx + dxs[d], my = ny + dys[d];
        if (mx < 0 || my < 0 || mx >= w || my >= h) continue;
        const int m = (my / step) * pe.gw + mx / step;
        int c = ld_cg(pe.claim + m);
        if (c == 0) {
            const bool admissible = pe.roi_grid[m] != 0 && mx - radius >= 0 && my - radius >= 0 && mx + radius < w &&
                                    my + radius < h;
            if (!admissible) { atomicCAS(pe.claim + m, 0, -1); continue; }
            const int old = atomicCAS(pe.claim + m, 0, next + 1);
            if (old == 0) {
                const int pos = atomicAdd(pe.counters, 1);
                pe.order[pos] = m | pe.jtag;
                c = next + 1;
            } else {
                c = old;
            }
        }
        if (c == next + 1) atomicMin(pe.key + m, k);
    }
}

// Dataflow order: primary parent = one step toward the seed along the dominant axis (x on
// ties), secondary parent = one step along the other axis (absent on the seed's row/column).
__device__ __forceinline__ void df_parents(const PropEnv& pe, int n, int& p1, int& p2) {
    const int gx = n % pe.gw, gy = n / pe.gw;
    const int dx = gx - pe.sgx, dy = gy - pe.sgy;
    const int sx = dx > 0 ? 1 : -1, sy = dy > 0 ? 1 : -1;
    p2 = -1;
    if (abs(dx) >= abs(dy)) {
        p1 = gy * pe.gw + gx - sx;
        if (dy != 0) p2 = (gy - sy) * pe.gw + gx;
    } else {
        p1 = (gy - sy) * pe.gw + gx;
        if (dx != 0) p2 = gy * pe.gw + gx - sx;
    }
}

// Release / acquire fences at GPU scope (cheaper than the sequentially consistent
// __threadfence); they order the message-passing patterns below.
__device__ __forceinline__ void fence_acq_rel() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }
__device__ __forceinline__ void st_release_u64(unsigned long long* p, unsigned long long v) {
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
constexpr unsigned int kInFlightBias = 0x80000000u;  // in-flight count = low word - bias

// Queue item: parent point (high 32, -1 = orphan) : tagged point (low 32).
__device__ __forceinline__ unsigned long long df_item(int parent, int c) {
    return (static_cast<unsigned long long>(static_cast<unsigned int>(parent)) << 32) | static_cast<unsigned int>(c);
}

// Add (k to the queue tail, dflight to the in-flight count) in one 64-bit atomic and publish k
// items.  The in-flight count sits in the low word with an offset of 2^31, so it never borrows.
__device__ __forceinline__ void df_publish(const PropEnv& pe, const unsigned long long* items, int k, int dflight) {
    const unsigned long long add = (static_cast<unsigned long long>(k) << 32) +
                                   static_cast<unsigned long long>(static_cast<long long>(dflight));
    if (k == 0) {
        if (dflight != 0) atomicAdd(pe.qword, add);  // result unused: a reduction, no round trip
        return;
    }
    const int pos = static_cast<int>(atomicAdd(pe.qword, add) >> 32);
    for (int i = 0; i < k; ++i) st_release_u64(pe.dq + pos + i, items[i]);  // release: n's state first
}

// n has been resolved: its state (and, if accepted, its parameters) are written.  Its children
// are the 4-neighbours one step farther from the seed.  A child is queued from its primary
// parent as soon as that one is accepted; otherwise the last of its parents to resolve
// decides: secondary parent if accepted, else orphan.  Exactly one thread decides each child
// (the accepted primary, or the unique last parent when the primary failed), so no further
// claim is needed.
//
// Children that n decides alone are published first, with one atomic, so they wait on no
// other memory round trip; the parent counters follow.  `cont` (from df_pick_cont, or -1) is
// a child whose primary parent is n (accepted) that the caller solves itself instead of
// queueing it, which takes the queue off the critical path of a chain of primary parents.
// `self_in_flight` is 1 when n itself was counted in flight (a queued or continued item); the
// continued child inherits that count, otherwise the last atomic gives it up.
__device__ int df_children(const PropEnv& pe, int n, int (&kid)[4], int (&kp1)[4], int (&kp2)[4]) {
    const int gx = n % pe.gw, gy = n / pe.gw;
    const int dn = abs(gx - pe.sgx) + abs(gy - pe.sgy);
    const int cxs[4] = {gx, gx + 1, gx, gx - 1}, cys[4] = {gy - 1, gy, gy + 1, gy};
    int nk = 0;
    for (int d = 0; d < 4; ++d) {
        const int cx = cxs[d], cy = cys[d];
        if (cx < 0 || cy < 0 || cx >= pe.gw || cy >= pe.gh) continue;
        if (abs(cx - pe.sgx) + abs(cy - pe.sgy) != dn + 1) continue;
        kid[nk] = cy * pe.gw + cx;
        df_parents(pe, kid[nk], kp1[nk], kp2[nk]);
        ++nk;
    }
    return nk;
}

// Length of the longest primary-parent chain below grid point c (the depth of its subtree).
// With the primary parent one step toward the seed along the dominant axis (x on ties), a
// point off the diagonal band owns only the rest of its row (|dx| > |dy|) or column
// (|dx| < |dy| - 1); a diagonal point, and the point just before it on the y side that is the
// diagonal point's primary parent, reach the far corner of their quadrant.
__device__ __forceinline__ int df_depth(const PropEnv& pe, int c) {
    const int dx = c % pe.gw - pe.sgx, dy = c / pe.gw - pe.sgy;
    const int ax = abs(dx), ay = abs(dy);
    const int ex = dx > 0 ? pe.gw - 1 - pe.sgx : (dx < 0 ? pe.sgx : max(pe.sgx, pe.gw - 1 - pe.sgx));
    const int ey = dy > 0 ? pe.gh - 1 - pe.sgy : (dy < 0 ? pe.sgy : max(pe.sgy, pe.gh - 1 - pe.sgy));
    if (ax > ay) return ex - ax;
    if (ax < ay - 1) return ey - ay;
    return (ex - ax) + (ey - ay);
}

// The child an accepted n continues with: of the children whose primary parent is n, the one
// with the deepest subtree (the first in up, right, down, left order on ties), so that the
// longest chains run without a queue hand-off; -1 if none.  Only scheduling depends on it.
__device__ int df_pick_cont(const PropEnv& pe, int n, bool accepted) {
    if (!accepted) return -1;
    int kid[4], kp1[4], kp2[4];
    const int nk = df_children(pe, n, kid, kp1, kp2);
    int best = -1, best_depth = -1;
    for (int i = 0; i < nk; ++i) {
        if (kp1[i] != n) continue;
        const int dep = df_depth(pe, kid[i]);
        if (dep > best_depth) { best = kid[i]; best_depth = dep; }
    }
    return best;
}

__device__ void df_resolve(const PropEnv& pe, int n, bool accepted, int self_in_flight, int cont) {
    int kid[4], kp1[4], kp2[4];
    const int nk = df_children(pe, n, kid, kp1, kp2);
    // children decided by n alone: accepted primary (queued, or continued), failed single parent
    unsigned long long push[4];
    int k = 0;
    for (int i = 0; i < nk; ++i) {
        if (kp1[i] == n && accepted) {
            if (kid[i] != cont) push[k++] = df_item(n, kid[i] | pe.jtag);
        } else if (kp2[i] < 0) {
            push[k++] = df_item(-1, kid[i] | pe.jtag);  // its only parent failed: orphan
        }
    }
    const int handed = cont >= 0 ? self_in_flight : 0;  // n's in-flight count passes to the continued child
    df_publish(pe, push, k, k + (cont >= 0 ? 1 : 0) - handed);
    // children with two parents: count the parents, the second one decides
    bool counted = false;
    for (int i = 0; i < nk; ++i) counted |= kp2[i] >= 0;
    if (counted) fence_acq_rel();  // publish n's state before any child counter update
    int k2 = 0;
    for (int i = 0; i < nk; ++i) {
        if (kp2[i] < 0) continue;
        if (kp1[i] == n && accepted) {
            atomicAdd(pe.dcnt + kid[i], 1);  // keep the count for the other parent (no round trip)
        } else if (atomicAdd(pe.dcnt + kid[i], 1) == 1) {  // the second of two parents to resolve
            fence_acq_rel();
            if (ld_cg(pe.dstate + kp1[i]) != kDfAccepted)
                push[k2++] = df_item(ld_cg(pe.dstate + kp2[i]) == kDfAccepted ? kp2[i] : -1, kid[i] | pe.jtag);
        }
    }
    df_publish(pe, push, k2, k2 - (self_in_flight - handed));
}

// Tree mode: n has been solved; queue its tree children except `cont` (which the solving group
// continues with and which inherits n's in-flight count).
__device__ void tree_resolve(const PropEnv& pe, int n, int cont) {
    unsigned long long push[4];
    int k = 0;
    for (int i = pe.tchild_off[n]; i < pe.tchild_off[n + 1] && k < 4; ++i) {
        const int c = pe.tchild[i];
        if (c != cont) push[k++] = df_item(n, c | pe.jtag);
    }
    df_publish(pe, push, k, k - (cont >= 0 ? 0 : 1));
}

// Propagation groups: 4 warps per POI and one resolver warp per CTA, one CTA per SM.  FP32:
// three groups per CTA (456 groups on 152 SMs).  Per-POI latency on the dataflow critical path
// bounds the propagation, and a solve shares its SM's issue slots with the other groups there:
// measured on 2048^2, r = 15 (dataflow, FP32), four groups per SM (two CTAs of two, or one of
// four) took 9.1-9.2 ms, three 8.4 ms (the register budget of one 416-thread CTA also removes
// the spills), two 10.0 ms (too few groups for the widest wavefronts); 8 warps per POI were
// 14-17% slower.  FP64: two groups per CTA, whose 288 threads leave room for the FP64 registers.
constexpr int kPropG = 4;
template <typename T> struct PropShape {
    static constexpr int groups = sizeof(T) == 4 ? 3 : 2;         // solver groups per CTA
    static constexpr int threads = 32 * kPropG * groups + 32;    // with the resolver warp
    static constexpr int min_blocks = 1;                         // resident CTAs per SM
};

// The batched launch's kernel shapes: narrow, up to 288 threads (two 4-warp groups or one 8-warp
// group and the resolver warp) and two CTAs per SM; wide (FP32), three 4-warp groups and the
// resolver warp in one 416-thread CTA per SM, as the single-pair launch.  The tuner times both.
template <int WIDE> struct BatchBounds {
    static constexpr int threads = WIDE ? 416 : 288;
    static constexpr int min_blocks = WIDE ? 1 : 2;
};

// Dataflow hand-over between a solver group and the resolver warp of its block (shared memory).
template <typename P>
struct DfSlot {
    int post;    // 1: a solved point waits for the resolver
    int want;    // 1: the group waits for a queued item
    int ready;   // 1: item in (c, par); 2: propagation finished; 3: error
    int n, state, cont, iters, conv;
    int status, valid;  // the raw solve outcome (tree mode)
    int c, par;
    P p[6];
    P q[6];  // second-order terms
    P corr;
};

__device__ __forceinline__ int vld(const int* p) { return *reinterpret_cast<const volatile int*>(p); }
__device__ __forceinline__ void vst(int* p, int v) { *reinterpret_cast<volatile int*>(p) = v; }

// Where a propagation launch finds its jobs.  OneJob: one image pair, everything in kernel
// parameters.  JobTable: several pairs, per-job environments and tensor maps in device memory,
// grid points tagged with the job in queue items and wave lists.
template <typename T>
struct OneJob {
    const Env<T>& e;
    const PropEnv& pe;
    const CUtensorMap* tr;
    const CUtensorMap* tc;
    __device__ int count() const { return 1; }
    __device__ int job_of(int) const { return 0; }
    __device__ int point_of(int c) const { return c; }
    __device__ const Env<T>& env(int) const { return e; }
    __device__ const PropEnv& prop(int) const { return pe; }
    __device__ const CUtensorMap* tm_ref(int) const { return tr; }
    __device__ const CUtensorMap* tm_coef(int) const { return tc; }
    __device__ int table(int) const { return 0; }
};

template <typename T>
struct BatchJob {
    Env<T> e;
    PropEnv pe;
    int table;  // first entry of the job's sample-offset table in the staged tables
};

template <typename T>
struct JobTable {
    const BatchJob<T>* jobs;
    int n;
    const CUtensorMap* maps;  // reference and coefficient map of each job
    __device__ int count() const { return n; }
    __device__ int job_of(int c) const { return c >> kJobShift; }
    __device__ int point_of(int c) const { return c & kPointMask; }
    __device__ Env<T> env(int j) const { return jobs[j].e; }
    __device__ const PropEnv& prop(int j) const { return jobs[j].pe; }
    __device__ const CUtensorMap* tm_ref(int j) const { return maps + 2 * j; }
    __device__ const CUtensorMap* tm_coef(int j) const { return maps + 2 * j + 1; }
    __device__ int table(int j) const { return jobs[j].table; }
};

// One lane of the resolver warp serves one solver group: it settles the points the group posts
// (parameters, state, children, outputs) and fetches queue items when the group asks for one.
// The group never waits on these global-memory round trips unless its queue runs dry.
template <typename P, typename Src, bool SO = false>
__device__ void df_resolver_lane(const Src& src, DfSlot<P>* slot, int* s_done, int total) {
    const PropEnv& g = src.prop(0);  // queue, counters and error word are shared by all jobs
    int ticket = -1;
    unsigned long long idle = 0;
    while (true) {
        bool progress = false;
        if (vld(&slot->post) == 1) {
            __threadfence_block();
            const int tagged = slot->n, st = slot->state, cont = slot->cont;
            const PropEnv& pe = src.prop(src.job_of(tagged));
            const int n = src.point_of(tagged);
            P* params = reinterpret_cast<P*>(pe.params);
            Result<P> R;
            for (int k = 0; k < 6; ++k) R.p[k] = slot->p[k];
            if constexpr (SO)
                for (int k = 0; k < 6; ++k) R.q[k] = slot->q[k];
            R.corr = slot->corr;
            R.iters = slot->iters;
            R.conv = slot->conv != 0;
            if (pe.mode == kModeTree) {
                // every solve's raw result; the host's heap simulation decides acceptance
                store_params(params, n, R);
                reinterpret_cast<P*>(pe.rcorr)[n] = R.corr;
                if constexpr (SO)
                    for (int k = 0; k < 6; ++k) reinterpret_cast<P*>(pe.rq)[static_cast<size_t>(n) * 6 + k] = R.q[k];
                pe.rmeta[n] = static_cast<unsigned char>((slot->status & 3) | (slot->valid ? 4 : 0) | (R.conv ? 8 : 0));
                pe.riters[n] = R.iters;
                tree_resolve(pe, n, cont);
            } else {
                const bool acc = st == kDfAccepted;
                if (acc) {
                    store_params(params, n, R);
                    pe.kcorr[n] = static_cast<float>(R.corr);
                }
                pe.dstate[n] = st;
                df_resolve(pe, n, acc, 1, cont);
                if (acc) {
                    store_outputs<P, SO>(pe, n, R);
                    atomicAdd(pe.flags + 2, 1);
                }
            }
            __threadfence_block();
            vst(&slot->post, 0);
            progress = true;
        }
        if (vld(&slot->want) == 1) {
            int deliver = 0;
            if (vld(s_done)) {
                deliver = 2;
            } else if (*reinterpret_cast<volatile int*>(g.err) != 0) {
                deliver = 3;
            } else {
                // At most `total` - 1 points are ever queued (each once, never a seed), so a
                // ticket beyond the array can only end by completion; it reads nothing.
                if (ticket < 0) ticket = atomicAdd(g.counters + 1, 1);
                const unsigned long long it = ticket < total ? ld_acquire_u64(g.dq + ticket) : ~0ull;
                if (it != ~0ull) {  // acquire: the parent's parameters were released before it
                    slot->c = static_cast<int>(it & 0xffffffffull);
                    slot->par = static_cast<int>(it >> 32);
                    ticket = -1;
                    deliver = 1;
                } else if (static_cast<unsigned int>(__ldcg(g.qword) & 0xffffffffull) == kInFlightBias) {
                    vst(s_done, 1);  // nothing queued or running anywhere
                    deliver = 2;
                }
            }
            if (deliver != 0) {
                vst(&slot->want, 0);
                __threadfence_block();
                vst(&slot->ready, deliver);
                if (deliver != 1) return;
                progress = true;
            }
        }
        if (progress) {
            idle = 0;
        } else {
            if (++idle > kSpinLimit) {
                atomicExch(g.err, 1);
                vst(&slot->ready, 3);
                return;
            }
            __nanosleep(idle < 64 ? 20 : 100);
        }
    }
}

// Guess extrapolation from an accepted neighbour (reliability_propagation.cpp:326-329).
template <typename P>
__device__ __forceinline__ void extrapolate(const P (&pp)[6], P ddx, P ddy, P (&p0)[6]) {
    p0[0] = pp[0] + pp[2] * ddx + pp[3] * ddy;
    p0[1] = pp[1] + pp[4] * ddx + pp[5] * ddy;
    p0[2] = pp[2]; p0[3] = pp[3]; p0[4] = pp[4]; p0[5] = pp[5];
}

// The acceptance rule of reliability_propagation.cpp:359-368.
template <typename P>
__device__ __forceinline__ bool acceptable(const Result<P>& R, const P (&p0)[6], P cutoff, P max_znssd) {
    return R.valid && R.status == TDIC_SUCCESS && R.corr < max_znssd && fabs(p0[0] - R.p[0]) < cutoff &&
           fabs(p0[1] - R.p[1]) < cutoff && finite6(R.p) && isfinite(R.corr);
}

// The propagation.  Blocks hold `gpb` solver groups of G warps and one resolver warp.
// Launched cooperatively (co-resident blocks, own grid barrier).
template <int OPT, int DEG, typename T, int G, typename Src, int VAR = 0>
__device__ __forceinline__ void propagate_body(const Src& src, const Shape& sh) {
    using P = typename MixedOf<T>::type;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int gpb = static_cast<int>(blockDim.x - 32) / (32 * G);
    const int gi = threadIdx.x / (32 * G), tid = threadIdx.x % (32 * G);
    const bool solver = gi < gpb;
    const PropEnv& g = src.prop(0);  // shared queue, wave lists, barrier and error word
    const bool one = src.count() == 1;
    short2* s_tab = kernel_preamble<T, G>(sh, g.err, one ? src.tm_ref(0) : nullptr, one ? src.tm_coef(0) : nullptr,
                                          smem_raw, gi, tid, solver);
    if (s_tab == nullptr) {  // every block takes this path together: nothing waits on a barrier yet
        if (threadIdx.x == 0) atomicExch(g.err, 1);
        return;
    }
    GroupSmem<T> gs = group_smem<T, G>(smem_raw, sh, solver ? gi : 0);
    int* ints = gs.ints;
    const int bar_id = 1 + gi;
    uint32_t phase = 0;
    unsigned char* ctl = smem_raw + cta_prefix_bytes(sh.ntab) +
                         gpb * group_smem_bytes<T>(sh.nmax, G, sh.rbx, sh.rby, sh.cbx, sh.cby, sh.mat, sh.stage, sh.narr);
    DfSlot<P>* slots = reinterpret_cast<DfSlot<P>*>(ctl);
    int* s_done = reinterpret_cast<int*>(ctl + round128(gpb * sizeof(DfSlot<P>)));
    if (threadIdx.x < gpb) {
        DfSlot<P>* sl = slots + threadIdx.x;
        sl->post = 0; sl->want = 0; sl->ready = 0;
    }
    if (threadIdx.x == 0) *s_done = 0;

    // Prologue: place each job's seed (reliability_propagation.cpp:201-278), one group per job.
    for (int j = blockIdx.x; j < src.count(); j += gridDim.x) {
        if (gi != 0) continue;
        const PropEnv& pe = src.prop(j);
        auto&& e = src.env(j);
        if (pe.seed_idx < 0) continue;  // no seed placed for this job
        P* params = reinterpret_cast<P*>(pe.params);
        Result<P> R;
        bool ok = true;
        if (pe.seed_solve) {
            const int sx = (pe.seed_idx % pe.gw) * pe.step, sy = (pe.seed_idx / pe.gw) * pe.step;
            P sp[6];
            for (int k = 0; k < 6; ++k) sp[k] = static_cast<P>(pe.seed_p[k]);
            if (!solve_any<OPT, DEG, T, G, VAR>(e, src.tm_ref(j), src.tm_coef(j), s_tab + src.table(j), sx, sy, sp,
                                                static_cast<P>(pe.seed_corr), gs, phase, tid, bar_id, R)) {
                if (tid == 0) { pe.flags[1] = 1; atomicExch(g.err, 1); }
                ok = false;
            }
            ok = ok && R.valid && R.status == TDIC_SUCCESS && finite6(R.p) && isfinite(R.corr);
        } else {
            for (int k = 0; k < 6; ++k) R.p[k] = static_cast<P>(pe.seed_p[k]);
            for (int k = 0; k < 6; ++k) R.q[k] = P(0);
            R.corr = static_cast<P>(pe.seed_corr);
            R.iters = 0;
            R.status = TDIC_SUCCESS;
            R.valid = true;
            R.conv = false;
        }
        if (tid == 0) {
            if (!ok) {
                pe.flags[1] = 1;
            } else {
                store_grid<P, (VAR & 2) != 0>(pe, params, pe.seed_idx, R);
                pe.claim[pe.seed_idx] = 1;
                pe.flags[2] = 1;
                if (pe.mode == 2) {
                    pe.kcorr[pe.seed_idx] = static_cast<float>(fmax(P(0), R.corr));
                    pe.dstate[pe.seed_idx] = kDfAccepted;
                    df_resolve(pe, pe.seed_idx, true, 0, -1);
                } else {
                    __threadfence();
                    expand(pe, e.w, e.h, e.radius, pe.seed_idx, static_cast<float>(fmax(P(0), R.corr)), 1);
                }
            }
        }
    }
    if (!grid_barrier(g.barrier, g.err, g.counters)) return;
    if (one && *reinterpret_cast<volatile int*>(g.flags + 1)) return;

    if (g.mode == kModeDataflow || g.mode == kModeTree) {
        // ---- dataflow phase: no grid-wide synchronisation ------------------------------------
        if (solver) {
            DfSlot<P>* slot = slots + gi;
            // A group continues with a child whose primary parent it just accepted (every
            // thread derives the same child); otherwise it asks its resolver lane for an item.
            int cont_c = -1, cont_p = -1;
            P cp[6];
            bool asked = false;          // thread 0: a request to the resolver lane is open
            bool precompute = one && OPT == 0 && VAR == 0 && src.env(0).sc_state != nullptr && g.pre_order != nullptr;
            while (true) {
                // state: 0 item, 1 done, 2 error, 3 precompute the set-up of point item_c
                int item_c = cont_c, item_p = cont_p, state = 0;
                if (cont_c < 0) {
                    if (tid == 0) {
                        if (!asked) {
                            vst(&slot->ready, 0);
                            __threadfence_block();
                            vst(&slot->want, 1);
                            asked = true;
                        }
                        unsigned long long spins = 0;
                        while (true) {
                            const int r = vld(&slot->ready);
                            if (r != 0) {
                                __threadfence_block();
                                state = r == 1 ? 0 : (r == 2 ? 1 : 2);
                                item_c = slot->c;
                                item_p = slot->par;
                                asked = false;
                                break;
                            }
                            if (precompute) {
                                // nothing to solve yet: set up a point ahead of the wavefront
                                const int k = atomicAdd(g.pre_ticket, 1);
                                if (k < g.pre_count) {
                                    state = 3;
                                    item_c = g.pre_order[k];
                                    break;
                                }
                                precompute = false;
                            }
                            if (++spins > kSpinLimit) { atomicExch(g.err, 1); state = 2; break; }
                            __nanosleep(spins < 64 ? 20 : 200);
                        }
                    }
                    group_bcast3<G>(state, item_c, item_p, ints + 1, tid, bar_id);
                    if (state == 3) {
                        const PropEnv& pe = src.prop(0);
                        const int nx = (item_c % pe.gw) * pe.step, ny = (item_c / pe.gw) * pe.step;
                        if (pe.roi_grid[item_c] != 0 && !precompute_setup<DEG, T, G>(src.env(0), src.tm_ref(0), s_tab + src.table(0), nx, ny, gs,
                                                         phase, tid, bar_id, item_c)) {
                            if (tid == 0) atomicExch(g.err, 1);
                            return;  // TMA wait timed out
                        }
                        continue;
                    }
                    if (state != 0) break;
                }
                const int j = src.job_of(item_c), n = src.point_of(item_c);
                const PropEnv& pe = src.prop(j);
                auto&& e = src.env(j);
                const P cutoff = static_cast<P>(pe.step), max_znssd = static_cast<P>(pe.max_znssd);
                const int nx = (n % pe.gw) * pe.step, ny = (n / pe.gw) * pe.step;
                bool accepted = false;
                int new_state = kDfOrphan;
                Result<P> R;
                R.iters = 0;
                R.conv = false;
                R.status = TDIC_INVALID_INPUT;
                R.valid = false;
                R.corr = P(0);
                for (int k = 0; k < 6; ++k) R.p[k] = R.q[k] = P(0);
                if (item_p >= 0) {
                    const bool admissible = pe.roi_grid[n] != 0 && nx - e.radius >= 0 && ny - e.radius >= 0 &&
                                            nx + e.radius < e.w && ny + e.radius < e.h;
                    new_state = kDfRejected;
                    if (admissible) {
                        P pp[6];
                        if (cont_c >= 0) {
                            for (int k = 0; k < 6; ++k) pp[k] = cp[k];
                        } else {
                            const P* params = reinterpret_cast<const P*>(pe.params);
                            for (int k = 0; k < 6; ++k) pp[k] = __ldcg(params + static_cast<size_t>(item_p) * 6 + k);
                        }
                        P p0[6];
                        extrapolate(pp, static_cast<P>(nx - (item_p % pe.gw) * pe.step),
                                    static_cast<P>(ny - (item_p / pe.gw) * pe.step), p0);
                        if (!solve_any<OPT, DEG, T, G, VAR>(e, src.tm_ref(j), src.tm_coef(j), s_tab + src.table(j), nx,
                                                            ny, p0, P(0), gs, phase, tid, bar_id, R, n)) {
                            if (tid == 0) atomicExch(g.err, 1);
                            return;  // TMA wait timed out
                        }
                        accepted = acceptable(R, p0, cutoff, max_znssd);
                        if (accepted) new_state = kDfAccepted;
                    }
                }
                const int next = pe.mode == kModeTree ? pe.tcont[n] : df_pick_cont(pe, n, accepted);
                if (tid == 0) {
                    // hand n to the resolver lane (its slot holds one point; normally long free)
                    unsigned long long spins = 0;
                    while (vld(&slot->post) != 0) {
                        if (++spins > kSpinLimit) { atomicExch(g.err, 1); break; }
                        __nanosleep(20);
                    }
                    slot->n = item_c; slot->state = new_state; slot->cont = next;
                    slot->iters = R.iters; slot->conv = R.conv ? 1 : 0;
                    slot->status = R.status; slot->valid = R.valid ? 1 : 0;
                    for (int k = 0; k < 6; ++k) slot->p[k] = R.p[k];
                    if constexpr ((VAR & 2) != 0)
                        for (int k = 0; k < 6; ++k) slot->q[k] = R.q[k];
                    slot->corr = R.corr;
                    __threadfence_block();
                    vst(&slot->post, 1);
                }
                if (next >= 0)
                    for (int k = 0; k < 6; ++k) cp[k] = R.p[k];
                cont_c = next >= 0 ? (next | pe.jtag) : -1;
                cont_p = n;
            }
        } else {
            const int lane = threadIdx.x & 31;
            if (lane < gpb) df_resolver_lane<P, Src, (VAR & 2) != 0>(src, slots + lane, s_done, sh.total);
            __syncwarp();
        }
        if (g.mode == kModeTree) return;  // a tree round ends with its queue: no clean-up waves
        if (!grid_barrier(g.barrier, g.err)) return;
        // ---- clean-up: orphans are reached by frontier waves from every accepted point ------
        for (int j = 0; j < src.count(); ++j) {
            const PropEnv& pe = src.prop(j);
            const int ng = pe.gw * pe.gh;
            for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ng; i += gridDim.x * blockDim.x) {
                const int st = ld_cg(pe.dstate + i);
                if (st == kDfAccepted || st == kDfRejected) pe.claim[i] = 1;
            }
        }
        if (!grid_barrier(g.barrier, g.err)) return;
        for (int j = 0; j < src.count(); ++j) {
            const PropEnv& pe = src.prop(j);
            const Env<T>& e = src.env(j);
            const int ng = pe.gw * pe.gh;
            for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ng; i += gridDim.x * blockDim.x)
                if (ld_cg(pe.dstate + i) == kDfAccepted) expand(pe, e.w, e.h, e.radius, i, __ldcg(pe.kcorr + i), 1);
        }
        if (!grid_barrier(g.barrier, g.err, g.counters)) return;
    }

    // ---- frontier waves -----------------------------------------------------------------
    int start = 0;
    int end = static_cast<int>(__ldcg(g.barrier + 2));  // the wave-list tail at the last barrier
    for (int wave = 1; start < end; ++wave) {
        const int count = end - start;
        while (solver) {
            int i = 0;
            if (tid == 0) i = atomicAdd(g.fetch + wave, 1);
            i = group_bcast<G>(i, ints + 1, tid, bar_id);
            if (i >= count) break;
            const int tagged = ld_cg(g.order + start + i);
            const int j = src.job_of(tagged), n = src.point_of(tagged);
            const PropEnv& pe = src.prop(j);
            auto&& e = src.env(j);
            const P cutoff = static_cast<P>(pe.step), max_znssd = static_cast<P>(pe.max_znssd);
            P* params = reinterpret_cast<P*>(pe.params);
            const unsigned long long kk = __ldcg(pe.key + n);
            const int parent = static_cast<int>(kk & 0xffffffffull);
            P pp[6];
            for (int k = 0; k < 6; ++k) pp[k] = __ldcg(params + static_cast<size_t>(parent) * 6 + k);
            const int nx = (n % pe.gw) * pe.step, ny = (n / pe.gw) * pe.step;
            P p0[6];
            extrapolate(pp, static_cast<P>(nx - (parent % pe.gw) * pe.step),
                        static_cast<P>(ny - (parent / pe.gw) * pe.step), p0);
            Result<P> R;
            if (!solve_any<OPT, DEG, T, G, VAR>(e, src.tm_ref(j), src.tm_coef(j), s_tab + src.table(j), nx, ny, p0,
                                                P(0), gs, phase, tid, bar_id, R, n)) {
                if (tid == 0) atomicExch(g.err, 1);
                return;  // TMA wait timed out
            }
            if (acceptable(R, p0, cutoff, max_znssd) && tid == 0) {
                store_grid<P, (VAR & 2) != 0>(pe, params, n, R);
                atomicAdd(pe.flags + 2, 1);
                __threadfence();
                expand(pe, e.w, e.h, e.radius, n, static_cast<float>(R.corr), wave + 1);
            }
        }
        if (!grid_barrier(g.barrier, g.err, g.counters)) return;
        start = end;
        end = static_cast<int>(__ldcg(g.barrier + 2));
    }
}

template <int OPT, int DEG, typename T, int G, int VAR = 0>
__global__ void __launch_bounds__(PropShape<T>::threads, PropShape<T>::min_blocks)
    propagate_kernel(const __grid_constant__ Env<T> e, const __grid_constant__ CUtensorMap tm_ref,
                     const __grid_constant__ CUtensorMap tm_coef, const __grid_constant__ PropEnv pe) {
    propagate_body<OPT, DEG, T, G, OneJob<T>, VAR>(OneJob<T>{e, pe, &tm_ref, &tm_coef},
                                                   shape_of(e, pe.gw * pe.gh, (VAR & 2) ? kMat12 : kMat6));
}

template <int OPT, int DEG, typename T, int G, int WIDE, int VAR>
__global__ void __launch_bounds__(BatchBounds<WIDE>::threads, sizeof(T) == 4 ? BatchBounds<WIDE>::min_blocks : 1)
    propagate_batch_kernel(const BatchJob<T>* __restrict__ jobs, int njobs, const CUtensorMap* __restrict__ maps,
                           const __grid_constant__ Shape sh) {
    propagate_body<OPT, DEG, T, G, JobTable<T>, VAR>(JobTable<T>{jobs, njobs, maps}, sh);
}

__global__ void init_grid_kernel(tdic_grid_out o, int gw, int gh, int step) {
    const int n = gw * gh;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (o.x) o.x[i] = static_cast<double>((i % gw) * step);
        if (o.y) o.y[i] = static_cast<double>((i / gw) * step);
        if (o.u) o.u[i] = 0.0;
        if (o.v) o.v[i] = 0.0;
        if (o.du_dx) o.du_dx[i] = 0.0;
        if (o.du_dy) o.du_dy[i] = 0.0;
        if (o.dv_dx) o.dv_dx[i] = 0.0;
        if (o.dv_dy) o.dv_dy[i] = 0.0;
        if (o.correlation) o.correlation[i] = 0.0;
        if (o.zncc) o.zncc[i] = 1.0;
        if (o.valid) o.valid[i] = 0;
        if (o.status) o.status[i] = TDIC_INVALID_INPUT;
        if (o.iterations) o.iterations[i] = 0;
        if (o.converged) o.converged[i] = 0;
        if (o.d2u_dx2) o.d2u_dx2[i] = 0.0;
        if (o.d2u_dxdy) o.d2u_dxdy[i] = 0.0;
        if (o.d2u_dy2) o.d2u_dy2[i] = 0.0;
        if (o.d2v_dx2) o.d2v_dx2[i] = 0.0;
        if (o.d2v_dxdy) o.d2v_dxdy[i] = 0.0;
        if (o.d2v_dy2) o.d2v_dy2[i] = 0.0;
    }
}

// The grid outputs of a heap-order propagation: the raw result of each point the host's heap
// simulation accepted (reliability_propagation.cpp:359-368: stored with status Success and
// valid), the defaults of init_grid_kernel elsewhere.
template <typename P>
__global__ void emit_tree_kernel(tdic_grid_out o, int gw, int gh, int step, const P* params, const P* rcorr,
                                 const P* rq, const unsigned char* rmeta, const int* riters,
                                 const unsigned char* accepted) {
    const int n = gw * gh;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const bool a = accepted[i] != 0;
        const size_t b6 = static_cast<size_t>(i) * 6;
        auto pv = [&](int k) { return a ? static_cast<double>(params[b6 + k]) : 0.0; };
        auto qv = [&](int k) { return (a && rq) ? static_cast<double>(rq[b6 + k]) : 0.0; };
        const double corr = a ? static_cast<double>(rcorr[i]) : 0.0;
        if (o.x) o.x[i] = static_cast<double>((i % gw) * step);
        if (o.y) o.y[i] = static_cast<double>((i / gw) * step);
        if (o.u) o.u[i] = pv(0);
        if (o.v) o.v[i] = pv(1);
        if (o.du_dx) o.du_dx[i] = pv(2);
        if (o.du_dy) o.du_dy[i] = pv(3);
        if (o.dv_dx) o.dv_dx[i] = pv(4);
        if (o.dv_dy) o.dv_dy[i] = pv(5);
        if (o.correlation) o.correlation[i] = corr;
        if (o.zncc) o.zncc[i] = a ? fmax(-1.0, fmin(1.0, 1.0 - 0.5 * corr)) : 1.0;
        if (o.valid) o.valid[i] = a ? 1 : 0;
        if (o.status) o.status[i] = a ? TDIC_SUCCESS : TDIC_INVALID_INPUT;
        if (o.iterations) o.iterations[i] = a ? riters[i] : 0;
        if (o.converged) o.converged[i] = (a && (rmeta[i] & 8)) ? 1 : 0;
        if (o.d2u_dx2) o.d2u_dx2[i] = qv(0);
        if (o.d2u_dxdy) o.d2u_dxdy[i] = qv(1);
        if (o.d2u_dy2) o.d2u_dy2[i] = qv(2);
        if (o.d2v_dx2) o.d2v_dx2[i] = qv(3);
        if (o.d2v_dxdy) o.d2v_dxdy[i] = qv(4);
        if (o.d2v_dy2) o.d2v_dy2[i] = qv(5);
    }
}

// ---------------------------------------------------------------------------------------
// Dispatch
// ---------------------------------------------------------------------------------------
template <typename T>
Env<T> make_env(tdic_ctx* ctx, tdic_pair* pair, const tdic_config& cfg, int radius, int max_iter, double thr,
                const short2* off = nullptr, int n_off = 0, const uint8_t* roi = nullptr) {
    if (!off) {
        const SampleTable& tab = sample_table(ctx, radius);
        off = tab.offsets.as<short2>();
        n_off = tab.n;
    }
    Env<T> e;
    e.ref = pair->ref.as<float>();
    e.coef = pair->coef.as<T>();
    e.w = pair->w; e.h = pair->h; e.cw = pair->cw; e.border = pair->border;
    e.radius = radius; e.n = n_off; e.nmax = n_off;
    e.off = off;
    e.max_iter = max_iter;
    e.thr = thr;
    e.inv_n = n_off > 0 ? 1.0 / n_off : 0.0;
    e.rpitch = pair->rpitch;
    e.cpitch = pair->cpitch;
    // Reference window: the subset with a one-pixel halo, x rounded down to 4 floats (16 B).
    e.rby = 2 * radius + 3;
    e.rbx = (2 * radius + 3 + 3 + 3) / 4 * 4;
    // Coefficient window: the subset warped by the initial guess (a few px of growth for the
    // gradient terms), a drift margin on both sides and the spline stencil, x rounded down to
    // 16 bytes.  Stencils that fall outside it read global memory.
    const int nb = pair->degree + 1;
    const int align = 16 / static_cast<int>(sizeof(T));
    const int cside = 2 * radius + 1 + 4 + 2 * kDriftMargin + nb;
    e.cby = cside;
    e.cbx = (cside + align - 1 + align - 1) / align * align;
    TDIC_REQUIRE(e.rbx <= 256 && e.rby <= 256 && e.cbx <= 256 && e.cby <= 256, TDIC_UNSUPPORTED,
                 "subset radius too large for a TMA box");
    e.err = ctx->dev_err;
    // masked subsets keep at least max(NP, min_valid_samples, ceil(ratio * full circle)) samples
    // (icgn.cpp:702-706, 1434-1438 and siblings)
    e.roi = roi;
    const int np = cfg.shape_order == 2 ? 12 : 6;
    e.min_keep = roi ? std::max(np, std::max(cfg.min_valid_samples,
                                             static_cast<int>(std::ceil(cfg.min_valid_sample_ratio * n_off))))
                     : 0;
    return e;
}

struct TensorMaps {
    CUtensorMap ref;
    CUtensorMap coef;
};

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    // looked up once; contexts on other host threads may race the first lookup and store the
    // same pointer
    static std::atomic<PFN_cuTensorMapEncodeTiled_v12000> fn{nullptr};
    PFN_cuTensorMapEncodeTiled_v12000 f = fn.load(std::memory_order_acquire);
    if (!f) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        TDIC_CUDA_TRY(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q));
        TDIC_REQUIRE(q == cudaDriverEntryPointSuccess && p, TDIC_CUDA_ERROR, "cuTensorMapEncodeTiled unavailable");
        f = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
        fn.store(f, std::memory_order_release);
    }
    return f;
}

void encode_2d(CUtensorMap* m, CUtensorMapDataType dt, size_t es, const void* base, int w, int h, int pitch, int bx,
               int by) {
    const cuuint64_t dims[2] = {static_cast<cuuint64_t>(w), static_cast<cuuint64_t>(h)};
    const cuuint64_t strides[1] = {static_cast<cuuint64_t>(pitch) * es};
    const cuuint32_t box[2] = {static_cast<cuuint32_t>(bx), static_cast<cuuint32_t>(by)};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = encode_fn()(m, dt, 2, const_cast<void*>(base), dims, strides, box, estr,
                                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                   CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    TDIC_REQUIRE(r == CUDA_SUCCESS, TDIC_CUDA_ERROR, "cuTensorMapEncodeTiled failed (" + std::to_string(int(r)) + ")");
}

template <typename T>
TensorMaps make_tensor_maps(const tdic_pair* pair, const Env<T>& e) {
    TensorMaps t;
    encode_2d(&t.ref, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, pair->ref.ptr, pair->w, pair->h, pair->rpitch, e.rbx, e.rby);
    encode_2d(&t.coef, sizeof(T) == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, sizeof(T),
              pair->coef.ptr, pair->cw, pair->ch, pair->cpitch, e.cbx, e.cby);
    return t;
}

// Shared-memory staging of a launch: each mode the request allows (tdic_staging; routes other
// than first-order ZNSSD stage in full) with its groups per block (at most gpb_max, shrunk until
// the block fits) and resident blocks per SM.  The mode with the most resident solver groups
// wins, the fullest staging among equals.  The kernel's dynamic shared-memory attribute is left
// at the chosen size (raised only, when `raise_only`: a batch keeps one bound for all its
// configurations).
struct StageChoice {
    int stage = -1, narr = 4, gpb = 0, per_sm = 0;
    size_t smem = 0;
};

template <typename T, typename K>
StageChoice choose_staging(tdic_ctx* ctx, K kern, int requested, bool lean_ok, int opt, int nmax, int G, int rbx,
                           int rby, int cbx, int cby, int mat, size_t prefix, size_t ctl, int gpb_max,
                           int extra_threads, bool raise_only = false) {
    int cands[3], nc = 0;
    if (!lean_ok || requested == TDIC_STAGING_FULL) {
        cands[nc++] = kStageFull;
    } else if (requested == TDIC_STAGING_LEAN) {
        cands[nc++] = kStageLean;
    } else if (requested == TDIC_STAGING_LEAN_NO_WINDOW) {
        cands[nc++] = kStageLean | kStageNoCoefWindow;
    } else {
        cands[nc++] = kStageFull;
        cands[nc++] = kStageLean;
        cands[nc++] = kStageLean | kStageNoCoefWindow;
    }
    StageChoice best;
    cudaFuncAttributes fa{};
    TDIC_CUDA_TRY(cudaFuncGetAttributes(&fa, kern));
    int attr = fa.maxDynamicSharedSizeBytes;
    for (int c = 0; c < nc; ++c) {
        const int stage = cands[c], narr = sample_arrays(opt, stage);
        const size_t per_group = group_smem_bytes<T>(nmax, G, rbx, rby, cbx, cby, mat, stage, narr);
        int gpb = gpb_max;
        while (gpb > 1 && prefix + gpb * per_group + ctl > static_cast<size_t>(ctx->max_smem_optin)) --gpb;
        const size_t smem = prefix + gpb * per_group + ctl;
        if (smem > static_cast<size_t>(ctx->max_smem_optin)) continue;
        if (static_cast<int>(smem) > attr) {
            TDIC_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
            attr = static_cast<int>(smem);
        }
        int per_sm = 0;
        TDIC_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32 * G * gpb + extra_threads, smem));
        if (per_sm <= 0) continue;
        if (best.stage < 0 || per_sm * gpb > best.per_sm * best.gpb) best = StageChoice{stage, narr, gpb, per_sm, smem};
    }
    TDIC_REQUIRE(best.stage >= 0, TDIC_UNSUPPORTED, "subset radius too large for shared memory");
    if (!raise_only)
        TDIC_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(best.smem)));
    return best;
}

constexpr int kGroupsPerBlockBatch = 4;  // 4 warps of 1-warp groups

template <int OPT, int DEG, typename T, int VAR = 0>
void solve_typed(tdic_ctx* ctx, tdic_pair* pair, const tdic_config& cfg, const SolveLaunch& L, cudaStream_t s) {
    constexpr int G = 1;
    Env<T> e = make_env<T>(ctx, pair, cfg, cfg.subset_radius, cfg.max_iterations, cfg.convergence_threshold,
                           nullptr, 0, L.roi);
    const TensorMaps tm = make_tensor_maps<T>(pair, e);
    auto kern = solve_batch_kernel<OPT, DEG, T, G, VAR>;
    const StageChoice sc = choose_staging<T>(ctx, kern, cfg.staging, VAR == 0, OPT, e.nmax, G, e.rbx, e.rby, e.cbx,
                                             e.cby, (VAR & 2) ? kMat12 : kMat6, cta_prefix_bytes(e.nmax), 0,
                                             kGroupsPerBlockBatch, 0);
    e.stage = sc.stage;
    e.narr = sc.narr;
    const int gpb = sc.gpb;
    int blocks = sc.per_sm * ctx->num_sms;
    const int need = (L.n + gpb - 1) / gpb;
    if (blocks > need) blocks = need < 1 ? 1 : need;
    TDIC_CUDA_TRY(cudaMemsetAsync(L.fetch, 0, sizeof(int), s));
    kern<<<blocks, 32 * G * gpb, sc.smem, s>>>(e, tm.ref, tm.coef, L.in, L.out, L.n, L.fetch);
    TDIC_CUDA_TRY(cudaGetLastError());
}

template <int OPT, typename T, int VAR = 0>
void solve_deg(tdic_ctx* ctx, tdic_pair* pair, const tdic_config& cfg, const SolveLaunch& L, cudaStream_t s) {
    switch (pair->degree) {
        case 1: solve_typed<OPT, 1, T, VAR>(ctx, pair, cfg, L, s); break;
        case 3: solve_typed<OPT, 3, T, VAR>(ctx, pair, cfg, L, s); break;
        default: solve_typed<OPT, 5, T, VAR>(ctx, pair, cfg, L, s); break;
    }
}

template <int OPT, int DEG, typename T, int VAR = 0>
void propagate_typed(tdic_ctx* ctx, tdic_pair* pair, const tdic_config& cfg, const PropagateLaunch& L, cudaStream_t s) {
    constexpr int G = kPropG;
    Env<T> e = make_env<T>(ctx, pair, cfg, cfg.subset_radius, cfg.max_iterations, cfg.convergence_threshold,
                           L.offsets, L.n_offsets, L.roi_px);
    TensorMaps tm = make_tensor_maps<T>(pair, e);
    using P = typename MixedOf<T>::type;
    const size_t ctl = round128(PropShape<T>::groups * sizeof(DfSlot<P>)) + 128;  // resolver hand-over
    auto kern = propagate_kernel<OPT, DEG, T, G, VAR>;
    const StageChoice sc = choose_staging<T>(ctx, kern, cfg.staging, VAR == 0, OPT, e.nmax, G, e.rbx, e.rby, e.cbx,
                                             e.cby, (VAR & 2) ? kMat12 : kMat6, cta_prefix_bytes(e.nmax), ctl,
                                             PropShape<T>::groups, 32);
    e.stage = sc.stage;
    e.narr = sc.narr;
    if (VAR == 0 && OPT == 0 && L.sc_state != nullptr) {
        e.sc_hinv = L.sc_hinv;
        e.sc_fmn = static_cast<T*>(L.sc_fmn);
        e.sc_state = L.sc_state;
    }
    const size_t smem = sc.smem;
    const int threads = 32 * G * sc.gpb + 32;  // solver groups + the resolver warp
    const int blocks = sc.per_sm * ctx->num_sms;
    PropEnv pe;
    pe.gw = L.gw; pe.gh = L.gh; pe.step = L.step;
    pe.roi_grid = L.roi_grid;
    pe.seed_idx = L.seed_idx; pe.seed_solve = L.seed_solve;
    for (int k = 0; k < 6; ++k) pe.seed_p[k] = L.seed_p[k];
    pe.seed_corr = L.seed_corr;
    pe.max_znssd = cfg.propagation_max_znssd;
    pe.out = L.out;
    pe.claim = L.claim; pe.key = L.key; pe.order = L.order; pe.counters = L.counters; pe.fetch = L.fetch;
    pe.params = L.key + static_cast<size_t>(L.gw) * L.gh;  // the parameters follow the keys
    pe.barrier = L.barrier; pe.flags = L.flags; pe.err = L.flags; pe.jtag = 0;
    pe.mode = L.mode; pe.sgx = L.sgx; pe.sgy = L.sgy;
    pe.dstate = L.dstate; pe.dcnt = L.dcnt; pe.dq = L.dq; pe.kcorr = L.kcorr;
    pe.qword = reinterpret_cast<unsigned long long*>(L.counters + 4);
    pe.tchild_off = L.tchild_off; pe.tchild = L.tchild; pe.tcont = L.tcont;
    pe.pre_order = e.sc_state != nullptr ? L.pre_order : nullptr;
    pe.pre_count = L.pre_count;
    pe.pre_ticket = L.pre_ticket;
    pe.rcorr = L.rcorr; pe.rq = L.rq; pe.rmeta = L.rmeta; pe.riters = L.riters;
    if (L.params) pe.params = L.params;  // a heap-order round keeps its parameters across rounds
    const int n = L.gw * L.gh;
    if (L.mode != kModeTree) {  // a tree round writes only its result table
        init_grid_kernel<<<(n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096, 256, 0, s>>>(L.out, L.gw, L.gh, L.step);
        TDIC_CUDA_TRY(cudaGetLastError());
    }
    void* args[] = {&e, &tm.ref, &tm.coef, &pe};
    TDIC_CUDA_TRY(cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(kern), dim3(blocks), dim3(threads), args,
                                              smem, s));
}

// ---------------------------------------------------------------------------------------
// Batched propagation: several image pairs in one persistent launch.
// ---------------------------------------------------------------------------------------
// VAR: the solver route of every job (0 first-order ZNSSD; 4 the same with masked subsets).
template <typename T, int VAR>
struct BatchPlan final : BatchPlanBase {
    using P = typename MixedOf<T>::type;
    int n = 0, opt = 0, deg = 3;
    size_t total = 0;
    std::vector<size_t> off;            // first grid point of each job
    std::vector<int> gw, gh, step, seed_ok;
    std::vector<BatchJob<T>> jobs;      // host copy of the job table
    std::vector<tdic_grid_out> outs;    // device outputs of each job
    Shape sh{};
    Buffer d_jobs, d_maps, d_tab, d_roi, d_claim, d_key, d_params, d_dstate, d_dcnt, d_kcorr, d_dq, d_order, d_fetch,
        d_misc, d_flags, d_out;
    std::vector<Buffer> d_roi_px;       // masked subsets: each job's pixel ROI (W x H bytes)
    // launch configurations: (warps per POI, groups per CTA) -> grid size and shared memory
    struct Config { int G, gpb, blocks, threads; size_t smem; int per_sm; int stage, narr, wide; };
    std::vector<Config> configs;
    int chosen = 0;
    int sms = 0;      // SMs' worth of blocks a launch uses (fewer than the device leaves room for other work)
    int num_sms = 0;
    // BatchPlanBase (defined in batch.cu, the only unit that builds plans)
    int config_count() const override;
    void config_info(int config, int* warps_per_poi, int* groups_per_block, int* staging) const override;
    void launch(int config, cudaStream_t s) override;
    void finish(int32_t* computed, int* err, cudaStream_t s) override;
    tdic_grid_out outputs(int job) const override;
    void grid(int job, int32_t* gw_out, int32_t* gh_out) const override;
    void set_sms(int sms_) override;
};

// The launch configurations of (G warps per POI, gpb groups per block): each staging mode the
// request allows that fits, kept when it makes more groups resident than the fuller modes before
// it (a leaner mode that fits no more groups only re-reads what the fuller one stages).
template <int OPT, int DEG, typename T, int G, int WIDE, int VAR>
void batch_kernel_setup(BatchPlan<T, VAR>& b, tdic_ctx* ctx, int gpb, int requested) {
    const size_t prefix = cta_prefix_bytes(b.sh.ntab);
    const size_t ctl = round128(gpb * sizeof(DfSlot<typename MixedOf<T>::type>)) + 128;
    const int threads = 32 * G * gpb + 32;
    static_assert(G * 32 + 32 <= BatchBounds<WIDE>::threads, "a group and the resolver fit the kernel's bound");
    if (threads > BatchBounds<WIDE>::threads) return;
    auto kern = propagate_batch_kernel<OPT, DEG, T, G, WIDE, VAR>;
    const int stages[3] = {kStageFull, kStageLean, kStageLean | kStageNoCoefWindow};
    // the masked route stages in full only
    const int want = VAR != 0 ? 0 : requested == TDIC_STAGING_FULL ? 0 : requested == TDIC_STAGING_LEAN ? 1
                   : requested == TDIC_STAGING_LEAN_NO_WINDOW ? 2 : -1;
    int best_groups = 0;
    for (int k = 0; k < 3; ++k) {
        if (want >= 0 && k != want) continue;
        const int stage = stages[k], narr = sample_arrays(OPT, stage);
        const size_t per_group = group_smem_bytes<T>(b.sh.nmax, G, b.sh.rbx, b.sh.rby, b.sh.cbx, b.sh.cby, kMat6, stage,
                                                     narr);
        const size_t smem = prefix + gpb * per_group + ctl;
        if (smem > static_cast<size_t>(ctx->max_smem_optin)) continue;
        // the attribute is an upper bound shared by every configuration of this kernel: only raise it
        cudaFuncAttributes fa{};
        TDIC_CUDA_TRY(cudaFuncGetAttributes(&fa, kern));
        if (static_cast<int>(smem) > fa.maxDynamicSharedSizeBytes)
            TDIC_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
        int per_sm = 0;
        TDIC_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem));
        if (per_sm <= 0 || per_sm * gpb <= best_groups) continue;
        best_groups = per_sm * gpb;
        b.configs.push_back({G, gpb, per_sm * ctx->num_sms, threads, smem, per_sm, stage, narr, WIDE});
    }
}

template <int OPT, int DEG, typename T, int G, int WIDE, int VAR>
void batch_kernel_launch(BatchPlan<T, VAR>& b, const typename BatchPlan<T, VAR>::Config& c, cudaStream_t s) {
    cudaLaunchConfig_t lc = {};
    lc.gridDim = dim3(std::min(c.blocks, c.per_sm * std::max(1, b.sms)));
    lc.blockDim = dim3(c.threads);
    lc.dynamicSmemBytes = c.smem;
    lc.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;  // co-resident blocks: the kernel has a grid barrier
    attr[0].val.cooperative = 1;
    lc.attrs = attr;
    lc.numAttrs = 1;
    Shape sh = b.sh;
    sh.stage = c.stage;
    sh.narr = c.narr;
    TDIC_CUDA_TRY(cudaLaunchKernelEx(&lc, propagate_batch_kernel<OPT, DEG, T, G, WIDE, VAR>, b.d_jobs.template as<BatchJob<T>>(),
                                     b.n, b.d_maps.template as<CUtensorMap>(), sh));
}

template <int OPT, int DEG, typename T, int VAR>
void batch_configs(BatchPlan<T, VAR>& b, tdic_ctx* ctx, int requested) {
    b.configs.clear();
    // the first configuration is the untuned default: in FP32 the single-pair launch's shape
    if constexpr (sizeof(T) == 4) batch_kernel_setup<OPT, DEG, T, 4, 1, VAR>(b, ctx, 3, requested);
    batch_kernel_setup<OPT, DEG, T, 4, 0, VAR>(b, ctx, 2, requested);
    batch_kernel_setup<OPT, DEG, T, 4, 0, VAR>(b, ctx, 1, requested);
    batch_kernel_setup<OPT, DEG, T, 8, 0, VAR>(b, ctx, 1, requested);
    TDIC_REQUIRE(!b.configs.empty(), TDIC_UNSUPPORTED, "batch: subset radius too large for shared memory");
}

template <int OPT, int DEG, typename T, int VAR>
void batch_dispatch(BatchPlan<T, VAR>& b, const typename BatchPlan<T, VAR>::Config& c, cudaStream_t s) {
    if (c.G == 8) batch_kernel_launch<OPT, DEG, T, 8, 0, VAR>(b, c, s);
    else if (c.wide) batch_kernel_launch<OPT, DEG, T, 4, 1, VAR>(b, c, s);
    else batch_kernel_launch<OPT, DEG, T, 4, 0, VAR>(b, c, s);
}

template <typename T, typename F>
void with_opt_deg(int opt, int deg, F&& f) {
    if (opt == 1) {
        if (deg == 1) f(std::integral_constant<int, 1>{}, std::integral_constant<int, 1>{});
        else if (deg == 3) f(std::integral_constant<int, 1>{}, std::integral_constant<int, 3>{});
        else f(std::integral_constant<int, 1>{}, std::integral_constant<int, 5>{});
    } else {
        if (deg == 1) f(std::integral_constant<int, 0>{}, std::integral_constant<int, 1>{});
        else if (deg == 3) f(std::integral_constant<int, 0>{}, std::integral_constant<int, 3>{});
        else f(std::integral_constant<int, 0>{}, std::integral_constant<int, 5>{});
    }
}

template <typename T, int VAR>
std::unique_ptr<BatchPlanBase> batch_plan_build(tdic_ctx* ctx, int n, tdic_pair* const* pairs, const tdic_config* cfgs,
                                                const BatchSeed* seeds, const std::vector<std::vector<uint8_t>>& rois,
                                                cudaStream_t s) {
    using P = typename MixedOf<T>::type;
    auto b = std::make_unique<BatchPlan<T, VAR>>();
    b->n = n;
    b->opt = cfgs[0].optimizer;
    b->deg = pairs[0]->degree;
    // sample-offset tables, one per radius, concatenated
    std::vector<int> radii;
    for (int j = 0; j < n; ++j) radii.push_back(cfgs[j].subset_radius);
    std::sort(radii.begin(), radii.end());
    radii.erase(std::unique(radii.begin(), radii.end()), radii.end());
    std::vector<short2> tab;
    std::vector<int> tab_off(radii.size()), tab_n(radii.size());
    for (size_t k = 0; k < radii.size(); ++k) {
        const int r = radii[k];
        tab_off[k] = static_cast<int>(tab.size());
        for (int dy = -r; dy <= r; ++dy)
            for (int dx = -r; dx <= r; ++dx)
                if (dx * dx + dy * dy <= r * r) tab.push_back(make_short2(static_cast<short>(dx), static_cast<short>(dy)));
        tab_n[k] = static_cast<int>(tab.size()) - tab_off[k];
    }
    b->d_tab = Buffer(&ctx->pool, sizeof(short2) * tab.size());
    TDIC_CUDA_TRY(cudaMemcpyAsync(b->d_tab.ptr, tab.data(), sizeof(short2) * tab.size(), cudaMemcpyHostToDevice, s));
    // grid geometry and point offsets
    b->off.resize(n + 1);
    b->gw.resize(n); b->gh.resize(n); b->step.resize(n); b->seed_ok.resize(n);
    size_t total = 0;
    for (int j = 0; j < n; ++j) {
        int32_t gw, gh;
        tdic_grid_dims(pairs[j]->w, pairs[j]->h, cfgs[j].propagation_spacing, &gw, &gh);
        TDIC_REQUIRE(static_cast<long long>(gw) * gh <= kPointMask + 1LL, TDIC_INVALID_ARG,
                     "batch: a job has more than 2^22 grid points");
        b->gw[j] = gw; b->gh[j] = gh; b->step[j] = std::max(0, cfgs[j].propagation_spacing) + 1;
        b->off[j] = total;
        total += static_cast<size_t>(gw) * gh;
    }
    b->off[n] = total;
    b->total = total;
    TDIC_REQUIRE(total < (1ull << 31), TDIC_INVALID_ARG, "batch: more than 2^31 grid points in total");
    // device buffers: per-point scratch of all jobs, shared queue state, outputs
    b->d_roi = Buffer(&ctx->pool, total);
    b->d_claim = Buffer(&ctx->pool, sizeof(int) * total);
    b->d_key = Buffer(&ctx->pool, sizeof(unsigned long long) * total);
    b->d_params = Buffer(&ctx->pool, sizeof(P) * 6 * total);
    b->d_dstate = Buffer(&ctx->pool, sizeof(int) * total);
    b->d_dcnt = Buffer(&ctx->pool, sizeof(int) * total);
    b->d_kcorr = Buffer(&ctx->pool, sizeof(float) * total);
    b->d_dq = Buffer(&ctx->pool, sizeof(unsigned long long) * total);
    b->d_order = Buffer(&ctx->pool, sizeof(int) * total);
    b->d_fetch = Buffer(&ctx->pool, sizeof(int) * (total + 2));
    b->d_misc = Buffer(&ctx->pool, 64);
    b->d_flags = Buffer(&ctx->pool, sizeof(int) * 4 * n);
    b->d_out = Buffer(&ctx->pool, (10 * sizeof(double) + sizeof(int32_t) + 3) * total);
    double* dbl = b->d_out.template as<double>();
    int32_t* it = reinterpret_cast<int32_t*>(dbl + 10 * total);
    uint8_t* bytes = reinterpret_cast<uint8_t*>(it + total);
    // ROI at the grid points, per job (host masks of W x H, or all valid)
    std::vector<uint8_t> roi_grid(total, 1);
    for (int j = 0; j < n; ++j)
        if (!rois[j].empty())
            for (int i = 0; i < b->gw[j] * b->gh[j]; ++i)
                roi_grid[b->off[j] + i] =
                    rois[j][static_cast<size_t>((i / b->gw[j]) * b->step[j]) * pairs[j]->w + (i % b->gw[j]) * b->step[j]];
    TDIC_CUDA_TRY(cudaMemcpyAsync(b->d_roi.ptr, roi_grid.data(), total, cudaMemcpyHostToDevice, s));
    // environments, capacities and tensor maps
    Shape sh{b->d_tab.template as<short2>(), static_cast<int>(tab.size()), 0, 0, 0, 0, 0, static_cast<int>(total)};
    std::vector<Env<T>> envs(n);
    if constexpr (VAR != 0) b->d_roi_px.resize(n);
    for (int j = 0; j < n; ++j) {
        const int k = static_cast<int>(std::lower_bound(radii.begin(), radii.end(), cfgs[j].subset_radius) - radii.begin());
        const uint8_t* roi_px = nullptr;
        if constexpr (VAR != 0) {
            // masked subsets: the pixel ROI on the device (every pixel valid when none is given)
            const size_t np = static_cast<size_t>(pairs[j]->w) * pairs[j]->h;
            b->d_roi_px[j] = Buffer(&ctx->pool, np);
            if (!rois[j].empty())
                TDIC_CUDA_TRY(cudaMemcpyAsync(b->d_roi_px[j].ptr, rois[j].data(), np, cudaMemcpyHostToDevice, s));
            else
                TDIC_CUDA_TRY(cudaMemsetAsync(b->d_roi_px[j].ptr, 1, np, s));
            roi_px = b->d_roi_px[j].template as<uint8_t>();
        }
        envs[j] = make_env<T>(ctx, pairs[j], cfgs[j], cfgs[j].subset_radius, cfgs[j].max_iterations,
                              cfgs[j].convergence_threshold, b->d_tab.template as<short2>() + tab_off[k], tab_n[k],
                              roi_px);
        sh.nmax = std::max(sh.nmax, envs[j].n);
        sh.rbx = std::max(sh.rbx, envs[j].rbx); sh.rby = std::max(sh.rby, envs[j].rby);
        sh.cbx = std::max(sh.cbx, envs[j].cbx); sh.cby = std::max(sh.cby, envs[j].cby);
    }
    b->sh = sh;
    std::vector<CUtensorMap> maps(2 * static_cast<size_t>(n));
    b->jobs.resize(n);
    b->outs.resize(n);
    unsigned char* misc = b->d_misc.template as<unsigned char>();
    int* m = reinterpret_cast<int*>(misc);
    for (int j = 0; j < n; ++j) {
        const int k = static_cast<int>(std::lower_bound(radii.begin(), radii.end(), cfgs[j].subset_radius) - radii.begin());
        Env<T> e = envs[j];
        e.nmax = sh.nmax;  // the per-group arrays are laid out for the largest subset
        const TensorMaps tm = make_tensor_maps<T>(pairs[j], e);
        maps[2 * j] = tm.ref;
        maps[2 * j + 1] = tm.coef;
        const size_t o = b->off[j];
        tdic_grid_out go{};
        go.x = dbl + 0 * total + o; go.y = dbl + 1 * total + o; go.u = dbl + 2 * total + o; go.v = dbl + 3 * total + o;
        go.du_dx = dbl + 4 * total + o; go.du_dy = dbl + 5 * total + o; go.dv_dx = dbl + 6 * total + o;
        go.dv_dy = dbl + 7 * total + o; go.correlation = dbl + 8 * total + o; go.zncc = dbl + 9 * total + o;
        go.iterations = it + o;
        go.valid = bytes + o;
        go.status = reinterpret_cast<int8_t*>(bytes + total + o);
        go.converged = bytes + 2 * total + o;
        b->outs[j] = go;
        PropEnv pe{};
        pe.gw = b->gw[j]; pe.gh = b->gh[j]; pe.step = b->step[j];
        pe.roi_grid = b->d_roi.template as<uint8_t>() + o;
        pe.seed_idx = seeds[j].ok ? seeds[j].idx : -1;
        pe.seed_solve = seeds[j].solve;
        for (int q = 0; q < 6; ++q) pe.seed_p[q] = seeds[j].p[q];
        pe.seed_corr = seeds[j].corr;
        pe.max_znssd = cfgs[j].propagation_max_znssd;
        pe.out = go;
        pe.claim = b->d_claim.template as<int>() + o;
        pe.key = b->d_key.template as<unsigned long long>() + o;
        pe.params = b->d_params.template as<P>() + 6 * o;
        pe.order = b->d_order.template as<int>();
        pe.counters = m;                                            // [0] wave-list tail, [1] queue head
        pe.qword = reinterpret_cast<unsigned long long*>(m + 4);    // queue tail : in flight + 2^31
        pe.barrier = reinterpret_cast<unsigned int*>(m + 8);
        pe.err = m + 12;
        pe.fetch = b->d_fetch.template as<int>();
        pe.flags = b->d_flags.template as<int>() + 4 * j;
        pe.jtag = j << kJobShift;
        pe.mode = 2;
        pe.sgx = seeds[j].gx; pe.sgy = seeds[j].gy;
        pe.dstate = b->d_dstate.template as<int>() + o;
        pe.dcnt = b->d_dcnt.template as<int>() + o;
        pe.dq = b->d_dq.template as<unsigned long long>();
        pe.kcorr = b->d_kcorr.template as<float>() + o;
        b->jobs[j].e = e;
        b->jobs[j].pe = pe;
        b->jobs[j].table = tab_off[k];
        b->seed_ok[j] = seeds[j].ok;
    }
    b->d_jobs = Buffer(&ctx->pool, sizeof(BatchJob<T>) * n);
    b->d_maps = Buffer(&ctx->pool, sizeof(CUtensorMap) * maps.size());
    TDIC_CUDA_TRY(cudaMemcpyAsync(b->d_jobs.ptr, b->jobs.data(), sizeof(BatchJob<T>) * n, cudaMemcpyHostToDevice, s));
    TDIC_CUDA_TRY(cudaMemcpyAsync(b->d_maps.ptr, maps.data(), sizeof(CUtensorMap) * maps.size(), cudaMemcpyHostToDevice, s));
    TDIC_CUDA_TRY(cudaStreamSynchronize(s));  // host staging vectors go out of scope
    with_opt_deg<T>(b->opt, b->deg, [&](auto O, auto D) {
        batch_configs<decltype(O)::value, decltype(D)::value, T, VAR>(*b, ctx, cfgs[0].staging);
    });
    b->num_sms = ctx->num_sms;
    b->sms = ctx->num_sms;
    return b;
}

// Everything one propagation of the batch needs, enqueued on `s` without a host wait.
template <typename T, int VAR>
void batch_plan_launch(BatchPlan<T, VAR>& b, int config, cudaStream_t s) {
    const size_t total = b.total;
    TDIC_CUDA_TRY(cudaMemsetAsync(b.d_claim.ptr, 0, sizeof(int) * total, s));
    TDIC_CUDA_TRY(cudaMemsetAsync(b.d_key.ptr, 0xff, sizeof(unsigned long long) * total, s));
    TDIC_CUDA_TRY(cudaMemsetAsync(b.d_dstate.ptr, 0, sizeof(int) * total, s));
    TDIC_CUDA_TRY(cudaMemsetAsync(b.d_dcnt.ptr, 0, sizeof(int) * total, s));
    TDIC_CUDA_TRY(cudaMemsetAsync(b.d_dq.ptr, 0xff, sizeof(unsigned long long) * total, s));
    TDIC_CUDA_TRY(cudaMemsetAsync(b.d_fetch.ptr, 0, sizeof(int) * (total + 2), s));
    TDIC_CUDA_TRY(cudaMemsetAsync(b.d_flags.ptr, 0, sizeof(int) * 4 * b.n, s));
    TDIC_CUDA_TRY(cudaMemsetAsync(b.d_misc.ptr, 0, 64, s));
    TDIC_CUDA_TRY(cudaMemsetAsync(b.d_misc.template as<unsigned char>() + 19, 0x80, 1, s));  // in-flight bias 2^31
    for (int j = 0; j < b.n; ++j) {
        const int np = b.gw[j] * b.gh[j];
        init_grid_kernel<<<std::min((np + 255) / 256, 4096), 256, 0, s>>>(b.outs[j], b.gw[j], b.gh[j], b.step[j]);
    }
    TDIC_CUDA_TRY(cudaGetLastError());
    const auto& c = b.configs[config];
    with_opt_deg<T>(b.opt, b.deg, [&](auto O, auto D) { batch_dispatch<decltype(O)::value, decltype(D)::value, T, VAR>(b, c, s); });
}

template <int OPT, typename T, int VAR = 0>
void propagate_deg(tdic_ctx* ctx, tdic_pair* pair, const tdic_config& cfg, const PropagateLaunch& L, cudaStream_t s) {
    switch (pair->degree) {
        case 1: propagate_typed<OPT, 1, T, VAR>(ctx, pair, cfg, L, s); break;
        case 3: propagate_typed<OPT, 3, T, VAR>(ctx, pair, cfg, L, s); break;
        default: propagate_typed<OPT, 5, T, VAR>(ctx, pair, cfg, L, s); break;
    }
}

// Solver-route launchers of this translation unit (every unit that includes this header has
// its own kernels and its own copy of the B-spline constant tables).
template <int VAR>
void solve_route(tdic_ctx* ctx, tdic_pair* pair, const tdic_config& cfg, const SolveLaunch& L, cudaStream_t s) {
    const bool fp64 = pair->precision == TDIC_FP64;
    if (cfg.optimizer == 1) {
        if (fp64) solve_deg<1, double, VAR>(ctx, pair, cfg, L, s); else solve_deg<1, float, VAR>(ctx, pair, cfg, L, s);
    } else {
        if (fp64) solve_deg<0, double, VAR>(ctx, pair, cfg, L, s); else solve_deg<0, float, VAR>(ctx, pair, cfg, L, s);
    }
}

template <int VAR>
void propagate_route(tdic_ctx* ctx, tdic_pair* pair, const tdic_config& cfg, const PropagateLaunch& L,
                     cudaStream_t s) {
    const bool fp64 = pair->precision == TDIC_FP64;
    if (cfg.optimizer == 1) {
        if (fp64) propagate_deg<1, double, VAR>(ctx, pair, cfg, L, s);
        else propagate_deg<1, float, VAR>(ctx, pair, cfg, L, s);
    } else {
        if (fp64) propagate_deg<0, double, VAR>(ctx, pair, cfg, L, s);
        else propagate_deg<0, float, VAR>(ctx, pair, cfg, L, s);
    }
}

// Upload the qk matrices of degrees 1, 3, 5 (bspline.cpp:320-340) into this unit's tables.
void upload_qk_local() {
    double qd[3][36] = {};
    float qf[3][36] = {};
    const int degs[3] = {1, 3, 5};
    for (int k = 0; k < 3; ++k) {
        build_qk(degs[k], qd[k]);
        for (int i = 0; i < 36; ++i) qf[k][i] = static_cast<float>(qd[k][i]);
    }
    TDIC_CUDA_TRY(cudaMemcpyToSymbol(c_qk_d, qd, sizeof(qd)));
    TDIC_CUDA_TRY(cudaMemcpyToSymbol(c_qk_f, qf, sizeof(qf)));
}

}  // namespace

}  // namespace tdic
