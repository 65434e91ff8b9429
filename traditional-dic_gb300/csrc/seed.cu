// K5: integer-displacement ZNCC search for seed candidates
// (IntegerSearchInitializer::estimate_with_interpolators, integer_search.cpp:333-432).
//
// Per candidate: a coarse search over every displacement that keeps the subset inside the
// image, on a pyramid_scale-strided grid with the pyramid_scale-strided circular samples
// (search_ncorr_multigrid :208-265); a full-sample refinement around the coarse optimum; a
// full-sample local search over +-search_radius; the local-preference rule (:267-280).  The
// winner of each search is the reference's: the circular-subset ZNCC of circular_subset_zncc
// (:129-166) in FP64 decides, ties keep the first position in the reference's v-major scan
// order; FP32 scores only select the positions that are rescored in FP64.
#include "tdic_internal.cuh"

#include <algorithm>
#include <cfloat>
#include <cmath>

namespace tdic {

namespace {

constexpr double kEps = 1e-12;

struct CandGeom {
    int cx, cy;
    int min_u, max_u, min_v, max_v;  // coarse range
    int inside;                      // the candidate's subset lies inside the image (masked: enough ROI samples)
    // the candidate's sample tables: coarse (pyramid-strided) and full, as (first entry, count)
    // in the concatenated offset arrays; one shared table each unless the subsets are masked
    int c_start, c_n, f_start, f_n;
};

struct Best {
    double z;
    int idx;
};

__device__ __forceinline__ bool better(double z, int idx, double bz, int bidx) {
    // strict '>' in scan order: a larger score wins, equal scores keep the earlier position
    if (z > bz) return true;
    if (z == bz && idx < bidx) return true;
    return false;
}

// The search scores every position in FP32 and rescores in FP64, exactly as
// circular_subset_zncc (integer_search.cpp:129-166: sums in sample order, each operation
// rounded once, no fused multiply-add), only the positions whose FP32 score is within
// kScoreMargin of the FP32 maximum, or whose deformed subset is nearly flat.  The FP32 score
// of a textured subset is within n * 2^-23 (~4e-5 for 317 samples) of the FP64 one, well
// inside kScoreMargin / 2, so the FP64 maximum is always among the rescored positions and the
// winner (with the reference's scan-order tie rule) is the reference's.
constexpr float kScoreMargin = 1e-3f;

// Reference samples of one candidate (shared memory): FP64 values and their mean and norm in
// the reference's order, plus FP32 copies for the scoring pass.
struct RefSet {
    double* r64;
    float* r32;
    double* stats;  // mean, norm
    float* fstats;  // mean, norm, sum of centred FP32 values
};

__device__ void load_ref(const float* __restrict__ ref, int pitch, const short2* off, int n, int cx, int cy,
                         const RefSet& rs) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const float v = __ldg(ref + static_cast<size_t>(cy + off[i].y) * pitch + cx + off[i].x);
        rs.r64[i] = static_cast<double>(v);
        rs.r32[i] = v;
    }
    __syncthreads();
    if (threadIdx.x == 0) {  // sample_mean, sample_norm (integer_search.cpp:111-127)
        double m = 0.0;
        for (int i = 0; i < n; ++i) m = __dadd_rn(m, rs.r64[i]);
        m = n > 0 ? __ddiv_rn(m, static_cast<double>(n)) : 0.0;
        double q = 0.0;
        for (int i = 0; i < n; ++i) {
            const double d = __dsub_rn(rs.r64[i], m);
            q = __dadd_rn(q, __dmul_rn(d, d));
        }
        rs.stats[0] = m;
        rs.stats[1] = q;
        const float mf = static_cast<float>(m);
        float sr = 0.0f;
        for (int i = 0; i < n; ++i) sr += rs.r32[i] - mf;
        rs.fstats[0] = mf;
        rs.fstats[1] = static_cast<float>(q);
        rs.fstats[2] = sr;
    }
    __syncthreads();
}

// circular_subset_zncc in FP64, rounded as on the reference's host.  The caller guarantees
// that the subset lies inside the image.
__device__ double zncc64(const float* __restrict__ def, int pitch, const short2* off, const double* r64, int n,
                         double rm, double rn, int cx, int cy, int u, int v) {
    if (n == 0 || rn <= kEps) return -INFINITY;
    double dm = 0.0;
    for (int i = 0; i < n; ++i)
        dm = __dadd_rn(dm, static_cast<double>(__ldg(def + static_cast<size_t>(cy + v + off[i].y) * pitch + cx + u + off[i].x)));
    dm = __ddiv_rn(dm, static_cast<double>(n));
    double num = 0.0, dn = 0.0;
    for (int i = 0; i < n; ++i) {
        const double rd = __dsub_rn(r64[i], rm);
        const double dd = __dsub_rn(
            static_cast<double>(__ldg(def + static_cast<size_t>(cy + v + off[i].y) * pitch + cx + u + off[i].x)), dm);
        num = __dadd_rn(num, __dmul_rn(rd, dd));
        dn = __dadd_rn(dn, __dmul_rn(dd, dd));
    }
    if (dn <= kEps) return -INFINITY;
    return __ddiv_rn(num, __dsqrt_rn(__dmul_rn(rn, dn)));
}

// FP32 score of the same position.  The mean is refined by the sum of the centred values
// (first-order correction of its rounding); `rescore` marks a nearly flat deformed subset
// (norm below 1e-3 of the mean square), where the FP32 score is not trusted.
__device__ float zncc32(const float* __restrict__ def, int pitch, const short2* off, const float* r32, int n, float rm,
                        float rn, float sr, int cx, int cy, int u, int v, bool& rescore) {
    rescore = false;
    if (n == 0) return -INFINITY;
    const float* base = def + static_cast<size_t>(cy + v) * pitch + cx + u;
    float dm = 0.0f;
    for (int i = 0; i < n; ++i) dm += __ldg(base + off[i].y * pitch + off[i].x);
    const float inv_n = 1.0f / static_cast<float>(n);
    dm *= inv_n;
    float num = 0.0f, dn = 0.0f, s1 = 0.0f, q2 = 0.0f;
    for (int i = 0; i < n; ++i) {
        const float d = __ldg(base + off[i].y * pitch + off[i].x);
        const float dd = d - dm;
        num = fmaf(r32[i] - rm, dd, num);
        dn = fmaf(dd, dd, dn);
        s1 += dd;
        q2 = fmaf(d, d, q2);
    }
    const float c = s1 * inv_n;
    num = fmaf(-c, sr, num);
    dn = fmaf(-c, s1, dn);
    if (!(dn > 1e-3f * q2 * inv_n)) { rescore = true; return -INFINITY; }
    return num * rsqrtf(rn * dn);
}

__device__ float block_max(float z, float* sf) {
    for (int o = 16; o > 0; o >>= 1) z = fmaxf(z, __shfl_xor_sync(0xffffffffu, z, o));
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sf[warp] = z;
    __syncthreads();
    const int nw = blockDim.x >> 5;
    float m = -INFINITY;
    for (int i = 0; i < nw; ++i) m = fmaxf(m, sf[i]);
    return m;
}

__device__ void block_argmax(double& z, int& idx, double* sz, int* si) {
    for (int o = 16; o > 0; o >>= 1) {
        const double oz = __shfl_down_sync(0xffffffffu, z, o);
        const int oi = __shfl_down_sync(0xffffffffu, idx, o);
        if (better(oz, oi, z, idx)) { z = oz; idx = oi; }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) { sz[warp] = z; si[warp] = idx; }
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
        z = lane < nw ? sz[lane] : -INFINITY;
        idx = lane < nw ? si[lane] : 0x7fffffff;
        for (int o = 16; o > 0; o >>= 1) {
            const double oz = __shfl_down_sync(0xffffffffu, z, o);
            const int oi = __shfl_down_sync(0xffffffffu, idx, o);
            if (better(oz, oi, z, idx)) { z = oz; idx = oi; }
        }
    }
    __syncthreads();
}

// Shared memory of the search kernels: FP64 samples, FP32 samples, statistics, reduction
// scratch, offsets.
struct SearchSmem {
    RefSet rs;
    double* sz;
    int* si;
    float* sf;
    short2* off;
    __device__ SearchSmem(unsigned char* smem, int n) {
        rs.r64 = reinterpret_cast<double*>(smem);
        rs.stats = rs.r64 + n;
        sz = rs.stats + 2;
        rs.r32 = reinterpret_cast<float*>(sz + 32);
        rs.fstats = rs.r32 + n;
        sf = rs.fstats + 4;
        si = reinterpret_cast<int*>(sf + 32);
        off = reinterpret_cast<short2*>(si + 32);
    }
};

size_t search_smem_bytes(size_t n) {
    return sizeof(double) * (n + 2 + 32) + sizeof(float) * (n + 4 + 32) + sizeof(int) * 32 + sizeof(short2) * n + 16;
}

// Coarse search (search_ncorr_multigrid's first stage, :208-247): grid.y = candidate, grid.x
// tiles the positions, kCoarsePerThread consecutive blocks' worth per block.  One pass: every
// thread keeps the FP32 scores of its positions in registers, the block takes their maximum
// and rescores in FP64 the positions within kScoreMargin of it (or nearly flat), and writes the
// tile's best (FP64 score, first in scan order).  The tile's maximum is at most the candidate's,
// so every position near the candidate's FP32 maximum is rescored in its tile; a position
// rescored only because its tile's maximum is lower scores, in FP64, more than kScoreMargin / 2
// below the winner and cannot win.  The best over the tiles is the two-pass search's winner.
constexpr int kCoarsePerThread = 16;
constexpr int kCoarseThreads = 256;

//
// Every deformed sample of the coarse stage lies on the lattice x, y = 0 mod cstep: position
// u = r - cx + cstep * ui and offset dx = -r + cstep * a give x = cx + u + dx = cstep * (ui + a).
// The kernel reads them from `dec` (dec[j * dpitch + i] = def[cstep * j][cstep * i]) at the
// lattice offsets doff = ((dx + r) / cstep, (dy + r) / cstep), in the order of coff: the same
// values in the same order, with a warp's positions on consecutive floats.
__global__ void __launch_bounds__(kCoarseThreads)
coarse_kernel(const float* __restrict__ ref, int pitch, const float* __restrict__ dec, int dpitch,
              const CandGeom* __restrict__ geo, const short2* __restrict__ coff, const short2* __restrict__ doff,
              int cn, int cstep, Best* __restrict__ partial, int tiles) {
    extern __shared__ __align__(16) unsigned char smem[];
    const CandGeom g = geo[blockIdx.y];
    cn = g.c_n;
    coff += g.c_start;
    doff += g.c_start;
    SearchSmem sm(smem, cn);
    short2* const soff = sm.off + cn;  // lattice offsets, after the reference offsets
    if (!g.inside) {  // uniform per block: no reference read outside the image
        if (threadIdx.x == 0) partial[blockIdx.y * tiles + blockIdx.x] = Best{-INFINITY, 0x7fffffff};
        return;
    }
    for (int i = threadIdx.x; i < cn; i += blockDim.x) {
        sm.off[i] = coff[i];
        soff[i] = doff[i];
    }
    __syncthreads();
    load_ref(ref, pitch, sm.off, cn, g.cx, g.cy, sm.rs);
    const int nu = g.max_u >= g.min_u ? (g.max_u - g.min_u) / cstep + 1 : 0;
    const int nv = g.max_v >= g.min_v ? (g.max_v - g.min_v) / cstep + 1 : 0;
    const int npos = nu * nv;
    const float rm = sm.rs.fstats[0], rn = sm.rs.fstats[1], sr = sm.rs.fstats[2];
    const int t0 = blockIdx.x * (kCoarsePerThread * kCoarseThreads) + threadIdx.x;
    float z32[kCoarsePerThread];
    unsigned flat_bits = 0;
    float best = -INFINITY;
#pragma unroll
    for (int k = 0; k < kCoarsePerThread; ++k) {
        const int t = t0 + k * kCoarseThreads;
        z32[k] = -INFINITY;
        if (t < npos) {
            const int vi = t / nu, ui = t - vi * nu;
            bool flat;
            z32[k] = zncc32(dec, dpitch, soff, sm.rs.r32, cn, rm, rn, sr, 0, 0, ui, vi, flat);
            flat_bits |= flat ? 1u << k : 0u;
            best = fmaxf(best, z32[k]);
        }
    }
    const float thr = block_max(best, sm.sf) - kScoreMargin;
    double bz = -INFINITY;
    int bi = 0x7fffffff;
#pragma unroll
    for (int k = 0; k < kCoarsePerThread; ++k) {
        const int t = t0 + k * kCoarseThreads;
        if (t >= npos || !((flat_bits >> k & 1u) || z32[k] >= thr)) continue;
        const int vi = t / nu, ui = t - vi * nu;
        const double z = zncc64(dec, dpitch, soff, sm.rs.r64, cn, sm.rs.stats[0], sm.rs.stats[1], 0, 0, ui, vi);
        if (better(z, t, bz, bi)) { bz = z; bi = t; }
    }
    block_argmax(bz, bi, sm.sz, sm.si);
    if (threadIdx.x == 0) partial[blockIdx.y * tiles + blockIdx.x] = Best{bz, bi};
}

// The coarse lattice of the deformed image: dec[j * dw + i] = def[cstep * j][cstep * i].
__global__ void decimate_kernel(const float* __restrict__ def, int pitch, int cstep, float* __restrict__ dec, int dw,
                                int dh) {
    const long long total = static_cast<long long>(dw) * dh;
    for (long long q = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; q < total;
         q += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int j = static_cast<int>(q / dw), i = static_cast<int>(q - static_cast<long long>(j) * dw);
        dec[q] = __ldg(def + static_cast<size_t>(j) * cstep * pitch + static_cast<size_t>(i) * cstep);
    }
}

// Exact block-wide argmaxes of circular_subset_zncc over two windows at once (either may be
// empty): A at (ua + t % nua, va + t / nua), B at (ub + t % nub, vb + t / nub), t in scan order,
// positions whose subset lies inside the image.  FP32 maxima of both in one sweep, then FP64
// rescoring near each maximum in one sweep: the two windows' serial FP64 sums run on different
// threads side by side.  Each window's result is its own argmax (the first of the best in its
// scan order), as if it were searched alone.
struct Window {
    int u0, v0, nu, nv;
    __device__ int size() const { return nu * nv; }
};

__device__ void window_argmax2(const float* __restrict__ def, int w, int h, int pitch, int r, const CandGeom& g,
                               const SearchSmem& sm, int n, const Window& A, const Window& B, double& bza, int& bia,
                               double& bzb, int& bib) {
    const float rm = sm.rs.fstats[0], rn = sm.rs.fstats[1], sr = sm.rs.fstats[2];
    const int na = A.size(), total = na + B.size();
    auto at = [&](int t, int& u, int& v) {  // the position of combined index t
        if (t < na) { u = A.u0 + t % A.nu; v = A.v0 + t / A.nu; return; }
        const int q = t - na;
        u = B.u0 + q % B.nu;
        v = B.v0 + q / B.nu;
    };
    float besta = -INFINITY, bestb = -INFINITY;
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
        int u, v;
        at(t, u, v);
        const int x = g.cx + u, y = g.cy + v;
        if (!(x - r >= 0 && y - r >= 0 && x + r < w && y + r < h)) continue;
        bool flat;
        const float z = zncc32(def, pitch, sm.off, sm.rs.r32, n, rm, rn, sr, g.cx, g.cy, u, v, flat);
        if (t < na) besta = fmaxf(besta, z); else bestb = fmaxf(bestb, z);
    }
    const float thra = block_max(besta, sm.sf) - kScoreMargin;
    const float thrb = block_max(bestb, sm.sf) - kScoreMargin;
    bza = -INFINITY; bia = 0x7fffffff;
    bzb = -INFINITY; bib = 0x7fffffff;
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
        int u, v;
        at(t, u, v);
        const int x = g.cx + u, y = g.cy + v;
        if (!(x - r >= 0 && y - r >= 0 && x + r < w && y + r < h)) continue;
        bool flat;
        const float z32 = zncc32(def, pitch, sm.off, sm.rs.r32, n, rm, rn, sr, g.cx, g.cy, u, v, flat);
        if (!(flat || z32 >= (t < na ? thra : thrb))) continue;
        const double z = zncc64(def, pitch, sm.off, sm.rs.r64, n, sm.rs.stats[0], sm.rs.stats[1], g.cx, g.cy, u, v);
        if (t < na) {
            if (better(z, t, bza, bia)) { bza = z; bia = t; }
        } else if (better(z, t - na, bzb, bib)) {
            bzb = z;
            bib = t - na;
        }
    }
    block_argmax(bza, bia, sm.sz, sm.si);
    block_argmax(bzb, bib, sm.sz, sm.si);
}

// Full-sample refinement around the coarse optimum and the local +-search window, then the
// local-preference rule.  One block per candidate.
constexpr int kFineThreads = 1024;

__global__ void __launch_bounds__(kFineThreads) fine_kernel(const float* __restrict__ ref, const float* __restrict__ def, int w, int h, int pitch, int r,
                            const CandGeom* __restrict__ geo, const short2* __restrict__ foff, int fn,
                            const Best* __restrict__ partial, int tiles, int cstep, int rr, int search, int coarse_ok_all,
                            const int* __restrict__ coarse_ok, SearchResult* __restrict__ out) {
    extern __shared__ __align__(16) unsigned char smem[];
    const CandGeom g = geo[blockIdx.x];
    fn = g.f_n;
    foff += g.f_start;
    SearchSmem sm(smem, fn);
    __shared__ double s_cz;
    __shared__ int s_cu, s_cv;
    if (!g.inside) {
        if (threadIdx.x == 0) out[blockIdx.x] = SearchResult{0, 0, -INFINITY, 0};
        return;
    }
    for (int i = threadIdx.x; i < fn; i += blockDim.x) sm.off[i] = foff[i];
    __syncthreads();
    load_ref(ref, pitch, sm.off, fn, g.cx, g.cy, sm.rs);
    const bool full_ok = !(fn == 0 || sm.rs.stats[1] <= kEps);
    // coarse winner
    if (threadIdx.x == 0) {
        double z = -INFINITY;
        int idx = 0x7fffffff;
        const bool have = coarse_ok_all && coarse_ok[blockIdx.x] && g.min_u <= g.max_u && g.min_v <= g.max_v;
        if (have)
            for (int b = 0; b < tiles; ++b) {
                const Best c = partial[blockIdx.x * tiles + b];
                if (better(c.z, c.idx, z, idx)) { z = c.z; idx = c.idx; }
            }
        const int nu = g.max_u >= g.min_u ? (g.max_u - g.min_u) / cstep + 1 : 1;
        s_cz = have ? z : -INFINITY;
        if (have && idx != 0x7fffffff) {
            s_cu = g.min_u + (idx % nu) * cstep;
            s_cv = g.min_v + (idx / nu) * cstep;
        } else {
            s_cu = 0;
            s_cv = 0;
        }
    }
    __syncthreads();
    // window A: the full-sample refinement around the coarse optimum; window B: the local
    // +-search window (independent of A), searched together
    const bool have_global = coarse_ok_all && coarse_ok[blockIdx.x] && g.min_u <= g.max_u && g.min_v <= g.max_v;
    const bool en_a = have_global && isfinite(s_cz) && full_ok;
    const bool en_b = search > 0 && full_ok;
    Window A{0, 0, 0, 0}, B{0, 0, 0, 0};
    if (en_a) {
        A.u0 = max(g.min_u, s_cu - rr);
        A.v0 = max(g.min_v, s_cv - rr);
        A.nu = min(g.max_u, s_cu + rr) - A.u0 + 1;
        A.nv = min(g.max_v, s_cv + rr) - A.v0 + 1;
    }
    if (en_b) B = Window{-search, -search, 2 * search + 1, 2 * search + 1};
    double bza, bzb;
    int bia, bib;
    window_argmax2(def, w, h, pitch, r, g, sm, fn, A, B, bza, bia, bzb, bib);
    if (threadIdx.x == 0) {
        double best_z = s_cz;
        int best_u = s_cu, best_v = s_cv;
        if (en_a) {
            best_z = bza;
            if (bia != 0x7fffffff) { best_u = A.u0 + bia % A.nu; best_v = A.v0 + bia / A.nu; } else { best_u = 0; best_v = 0; }
        }
        if (en_b) {
            const int lu = bib != 0x7fffffff ? B.u0 + bib % B.nu : 0;
            const int lv = bib != 0x7fffffff ? B.v0 + bib / B.nu : 0;
            // prefer_local_when_ambiguous
            if (!isfinite(bzb)) {
            } else if (!isfinite(best_z)) { best_z = bzb; best_u = lu; best_v = lv; }
            else if (bzb + 0.02 >= best_z) { best_z = bzb; best_u = lu; best_v = lv; }
        }
        out[blockIdx.x] = SearchResult{best_u, best_v, best_z, (isfinite(best_z) && full_ok) ? 1 : 0};
    }
}

// One thread per point.  Each squared distance is rounded as the reference's
// dx * dx + dy * dy on a host without fused multiply-add (product, product, sum), so the
// nearest centre and its ties resolve as there.
__global__ void kmeans_assign_kernel(const int2* __restrict__ pts, int m, const double2* __restrict__ ctr, int k,
                                     int* __restrict__ assign) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= m) return;
    const double x = static_cast<double>(pts[j].x), y = static_cast<double>(pts[j].y);
    int best = 0;
    double bd = INFINITY;
    for (int i = 0; i < k; ++i) {
        const double2 c = __ldg(ctr + i);  // same address across the warp: one broadcast load
        const double dx = __dsub_rn(x, c.x), dy = __dsub_rn(y, c.y);
        const double d2 = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
        if (d2 < bd) { bd = d2; best = i; }
    }
    assign[j] = best;
}

// One k-means iteration's assignment and centre sums.  The points are integer pixels and the
// sums stay far below 2^53, so the FP64 sums of run_kmeans (seed_selector.cpp:84-104) are exact
// whatever the order: they are accumulated here as integers (per block in shared memory, 32-bit,
// then atomically into the 64-bit `acc` = [sum x, sum y, count] per centre).  kKmeansLanes lanes
// share a point: each scans every kKmeansLanes-th centre, and the lanes' (distance, index) minima
// combine to the first centre at the smallest distance, which is the sequential scan's choice.
constexpr int kKmeansLanes = 8;

//
// FP32 filter (filter != 0, every coordinate below cb <= 2^22, points exact in float): with the
// centres rounded to float (|c - c32| <= u |c| <= u cb, u = 2^-24) and the distance
// d32 = dx32^2 + dy32^2 rounded in float, |d32 - d2| <= 2u cb (|dx32| + |dy32|) + 4u d32 +
// 4u^2 cb^2 (to first order in u), where d2 is the FP64 distance.  err32 = 1e-6 (cb (|dx32| +
// |dy32|) + d32) + kabs, kabs = 16u^2 cb^2 + 1e-6, bounds it at least four times over.  A centre
// can hold the FP64 minimum (or tie with it) only if d32 - err32 <= U = min over the centres of
// (d32 + err32), so only those are scored in FP64, and the FP64 scan over them gives the full
// scan's choice.
__device__ __forceinline__ float kmeans_d32(float x, float y, float2 c, float cb, float kabs, float& err) {
    const float dx = __fsub_rn(x, c.x), dy = __fsub_rn(y, c.y);
    const float d = __fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy));
    err = 1e-6f * (cb * (fabsf(dx) + fabsf(dy)) + d) + kabs;
    return d;
}

__global__ void kmeans_step_kernel(const int2* __restrict__ pts, int m, const double2* __restrict__ ctr,
                                   const float2* __restrict__ ctr32, int k, float cb, float kabs, int filter,
                                   unsigned long long* __restrict__ acc) {
    extern __shared__ unsigned int s_acc[];  // 3 * k
    for (int i = threadIdx.x; i < 3 * k; i += blockDim.x) s_acc[i] = 0u;
    __syncthreads();
    const int gt = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = gt / kKmeansLanes, sub = gt % kKmeansLanes;
    int best = -1;
    double bd = INFINITY;
    int2 pt = make_int2(0, 0);
    if (j < m) pt = pts[j];
    const float xf = static_cast<float>(pt.x), yf = static_cast<float>(pt.y);
    float ub = INFINITY;  // upper bound of the FP64 minimum
    if (filter && j < m)
        for (int i = sub; i < k; i += kKmeansLanes) {
            float err;
            const float d = kmeans_d32(xf, yf, __ldg(ctr32 + i), cb, kabs, err);
            ub = fminf(ub, d + err);
        }
#pragma unroll
    for (int o = kKmeansLanes / 2; o > 0; o >>= 1) ub = fminf(ub, __shfl_xor_sync(0xffffffffu, ub, o));
    if (j < m) {
        const double x = static_cast<double>(pt.x), y = static_cast<double>(pt.y);
        for (int i = sub; i < k; i += kKmeansLanes) {
            if (filter) {
                float err;
                const float d = kmeans_d32(xf, yf, __ldg(ctr32 + i), cb, kabs, err);
                if (d - err > ub) continue;
            }
            const double2 c = __ldg(ctr + i);
            const double dx = __dsub_rn(x, c.x), dy = __dsub_rn(y, c.y);
            const double d2 = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
            if (d2 < bd) { bd = d2; best = i; }
        }
    }
#pragma unroll
    for (int o = kKmeansLanes / 2; o > 0; o >>= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, bd, o);
        const int oi = __shfl_xor_sync(0xffffffffu, best, o);
        if (ob < bd || (ob == bd && static_cast<unsigned>(oi) < static_cast<unsigned>(best))) {
            bd = ob;
            best = oi;
        }
    }
    if (j < m && sub == 0 && best >= 0) {
        atomicAdd(s_acc + 3 * best, static_cast<unsigned int>(pt.x));
        atomicAdd(s_acc + 3 * best + 1, static_cast<unsigned int>(pt.y));
        atomicAdd(s_acc + 3 * best + 2, 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 3 * k; i += blockDim.x)
        if (s_acc[i]) atomicAdd(acc + i, static_cast<unsigned long long>(s_acc[i]));
}

// New centres (sum / count, as on the reference's host) for every centre with members; the sums
// are cleared for the next iteration.
__global__ void kmeans_update_kernel(double2* __restrict__ ctr, float2* __restrict__ ctr32, int k,
                                     unsigned long long* __restrict__ acc) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k) return;
    const unsigned long long n = acc[3 * i + 2];
    if (n > 0) {
        const double c = static_cast<double>(n);
        const double2 v = make_double2(__ddiv_rn(static_cast<double>(acc[3 * i]), c),
                                       __ddiv_rn(static_cast<double>(acc[3 * i + 1]), c));
        ctr[i] = v;
        ctr32[i] = make_float2(__double2float_rn(v.x), __double2float_rn(v.y));
    }
    acc[3 * i] = acc[3 * i + 1] = acc[3 * i + 2] = 0ull;
}

std::vector<short2> circle_offsets(int r, int step) {
    std::vector<short2> o;
    step = step < 1 ? 1 : step;
    for (int dy = -r; dy <= r; dy += step)
        for (int dx = -r; dx <= r; dx += step)
            if (dx * dx + dy * dy <= r * r) o.push_back(make_short2(static_cast<short>(dx), static_cast<short>(dy)));
    return o;
}

}  // namespace

KmeansAssigner::KmeansAssigner(tdic_ctx* ctx, const int* px, const int* py, int m, int k, cudaStream_t s)
    : ctx_(ctx), s_(s), m_(m), k_(k), pts_(&ctx->pool, sizeof(int2) * std::max(m, 1)),
      ctr_(&ctx->pool, sizeof(double2) * std::max(k, 1)), ctr32_(&ctx->pool, sizeof(float2) * std::max(k, 1)),
      out_(&ctx->pool, sizeof(int) * std::max(m, 1)), acc_(&ctx->pool, sizeof(unsigned long long) * 3 * std::max(k, 1)) {
    std::vector<int2> p(m);
    long long big = 0;  // the largest |coordinate|: the centres (means of the points) lie within it
    for (int i = 0; i < m; ++i) {
        p[i] = make_int2(px[i], py[i]);
        big = std::max(big, std::max(std::llabs(px[i]), std::llabs(py[i])));
    }
    cbound_ = static_cast<float>(big + 1);
    const double ucb = std::ldexp(static_cast<double>(big + 1), -24);
    kabs_ = static_cast<float>(16.0 * ucb * ucb + 1e-6);
    filter_ = big + 1 <= (1LL << 22) ? 1 : 0;
    TDIC_CUDA_TRY(cudaMemcpyAsync(pts_.ptr, p.data(), sizeof(int2) * m, cudaMemcpyHostToDevice, s_));
    TDIC_CUDA_TRY(cudaStreamSynchronize(s_));  // p is a local
}

void KmeansAssigner::run(double* cx, double* cy, int iters) {
    std::vector<double2> c(k_);
    std::vector<float2> c32(k_);
    for (int i = 0; i < k_; ++i) {
        c[i] = make_double2(cx[i], cy[i]);
        c32[i] = make_float2(static_cast<float>(cx[i]), static_cast<float>(cy[i]));  // round to nearest
    }
    TDIC_CUDA_TRY(cudaMemcpyAsync(ctr_.ptr, c.data(), sizeof(double2) * k_, cudaMemcpyHostToDevice, s_));
    TDIC_CUDA_TRY(cudaMemcpyAsync(ctr32_.ptr, c32.data(), sizeof(float2) * k_, cudaMemcpyHostToDevice, s_));
    TDIC_CUDA_TRY(cudaMemsetAsync(acc_.ptr, 0, sizeof(unsigned long long) * 3 * k_, s_));
    const size_t smem = sizeof(unsigned int) * 3 * k_;
    const long long threads = static_cast<long long>(m_) * kKmeansLanes;
    const int blocks = static_cast<int>((threads + 255) / 256);
    for (int it = 0; it < iters; ++it) {
        kmeans_step_kernel<<<blocks, 256, smem, s_>>>(pts_.as<int2>(), m_, ctr_.as<double2>(), ctr32_.as<float2>(),
                                                      k_, cbound_, kabs_, filter_, acc_.as<unsigned long long>());
        TDIC_CUDA_TRY(cudaGetLastError());
        kmeans_update_kernel<<<(k_ + 127) / 128, 128, 0, s_>>>(ctr_.as<double2>(), ctr32_.as<float2>(), k_,
                                                               acc_.as<unsigned long long>());
        TDIC_CUDA_TRY(cudaGetLastError());
    }
    TDIC_CUDA_TRY(cudaMemcpyAsync(c.data(), ctr_.ptr, sizeof(double2) * k_, cudaMemcpyDeviceToHost, s_));
    TDIC_CUDA_TRY(cudaStreamSynchronize(s_));  // c is a local
    for (int i = 0; i < k_; ++i) { cx[i] = c[i].x; cy[i] = c[i].y; }
}

void KmeansAssigner::assign(const double* cx, const double* cy, int* assign_host) {
    std::vector<double2> c(k_);
    for (int i = 0; i < k_; ++i) c[i] = make_double2(cx[i], cy[i]);
    TDIC_CUDA_TRY(cudaMemcpyAsync(ctr_.ptr, c.data(), sizeof(double2) * k_, cudaMemcpyHostToDevice, s_));
    kmeans_assign_kernel<<<(m_ + 255) / 256, 256, 0, s_>>>(pts_.as<int2>(), m_, ctr_.as<double2>(), k_, out_.as<int>());
    TDIC_CUDA_TRY(cudaGetLastError());
    TDIC_CUDA_TRY(cudaMemcpyAsync(assign_host, out_.ptr, sizeof(int) * m_, cudaMemcpyDeviceToHost, s_));
    TDIC_CUDA_TRY(cudaStreamSynchronize(s_));
}

// roi (host, w x h, or NULL): estimate_with_mask_interpolators (integer_search.cpp:447-545) - the
// centre must be a ROI pixel, each candidate's samples are its ROI samples (in the reference's
// order), at least min_required_samples of them (max(12, ceil(0.5 * full circle))) for the full
// set, and for the coarse set before the multigrid stage runs.
void integer_search_batch(tdic_ctx* ctx, tdic_pair* lazy, const tdic_config& cfg, const int* cx, const int* cy, int n,
                          SearchResult* out_host, cudaStream_t s, const uint8_t* roi) {
    if (n <= 0) return;
    TDIC_REQUIRE(n <= 65535, TDIC_INVALID_ARG, "integer search: at most 65535 points per call (one grid row each)");
    const int w = lazy->w, h = lazy->h;
    const int r = cfg.is_subset_radius < 1 ? 1 : cfg.is_subset_radius;
    const int search = cfg.is_search_radius < 0 ? 0 : cfg.is_search_radius;
    const int cstep = cfg.pyramid_enabled ? (cfg.pyramid_scale < 1 ? 1 : cfg.pyramid_scale) : 1;
    int rr = cfg.pyramid_refinement_radius < 1 ? 1 : cfg.pyramid_refinement_radius;
    rr = std::max(rr, static_cast<int>(std::ceil(1.5 * static_cast<double>(r))));
    rr = std::max(rr, cstep);
    const auto foff_full = circle_offsets(r, 1);
    const auto coff_full = circle_offsets(r, cstep);
    std::vector<CandGeom> geo(n);
    std::vector<int> ok(n, 0), cok(n, 0);
    std::vector<short2> foff, coff;
    auto need = [&](int step) {  // min_required_samples (integer_search.cpp:47-50)
        return std::max(12, static_cast<int>(std::ceil(0.5 * static_cast<double>(circle_offsets(r, step).size()))));
    };
    if (!roi) {
        foff = foff_full;
        coff = coff_full;
    }
    for (int i = 0; i < n; ++i) {
        CandGeom& g = geo[i];
        g.cx = cx[i];
        g.cy = cy[i];
        g.min_u = r - cx[i];
        g.max_u = w - 1 - r - cx[i];
        g.min_v = r - cy[i];
        g.max_v = h - 1 - r - cy[i];
        if (!roi) {
            ok[i] = (cx[i] - r >= 0 && cy[i] - r >= 0 && cx[i] + r < w && cy[i] + r < h) ? 1 : 0;
            cok[i] = ok[i];
            g.c_start = 0; g.c_n = static_cast<int>(coff.size());
            g.f_start = 0; g.f_n = static_cast<int>(foff.size());
        } else {
            auto keep = [&](const short2& o) {
                const int x = cx[i] + o.x, y = cy[i] + o.y;
                return x >= 0 && y >= 0 && x < w && y < h && roi[static_cast<size_t>(y) * w + x] != 0;
            };
            const bool centre = cx[i] >= 0 && cy[i] >= 0 && cx[i] < w && cy[i] < h &&
                                roi[static_cast<size_t>(cy[i]) * w + cx[i]] != 0;
            g.f_start = static_cast<int>(foff.size());
            for (const short2& o : foff_full) if (centre && keep(o)) foff.push_back(o);
            g.f_n = static_cast<int>(foff.size()) - g.f_start;
            g.c_start = static_cast<int>(coff.size());
            for (const short2& o : coff_full) if (centre && keep(o)) coff.push_back(o);
            g.c_n = static_cast<int>(coff.size()) - g.c_start;
            ok[i] = centre && g.f_n >= need(1) ? 1 : 0;
            cok[i] = ok[i] && g.c_n >= need(cstep) ? 1 : 0;
            if (!cok[i]) g.c_n = 0;  // no multigrid stage: every coarse score is -inf
        }
        g.inside = ok[i];
    }
    if (foff.empty()) foff.push_back(make_short2(0, 0));  // keep the device tables non-empty
    if (coff.empty()) coff.push_back(make_short2(0, 0));
    int cmax = 1, fmax = 1;
    for (const CandGeom& g : geo) { cmax = std::max(cmax, g.c_n); fmax = std::max(fmax, g.f_n); }
    // A flat coarse subset (coarse_ref_norm <= eps) scores -inf everywhere in the coarse search,
    // the reference's outcome of skipping the multigrid stage (integer_search.cpp:381-397).
    Buffer d_geo(&ctx->pool, sizeof(CandGeom) * n), d_coff(&ctx->pool, sizeof(short2) * coff.size()),
        d_foff(&ctx->pool, sizeof(short2) * foff.size()), d_cok(&ctx->pool, sizeof(int) * n),
        d_out(&ctx->pool, sizeof(SearchResult) * n);
    // coarse tiles: enough for the candidate with the most positions
    long long npos_max = 1;
    for (const CandGeom& g : geo) {
        const long long nu = g.max_u >= g.min_u ? (g.max_u - g.min_u) / cstep + 1 : 0;
        const long long nv = g.max_v >= g.min_v ? (g.max_v - g.min_v) / cstep + 1 : 0;
        npos_max = std::max(npos_max, nu * nv);
    }
    constexpr long long kPerTile = static_cast<long long>(kCoarsePerThread) * kCoarseThreads;
    TDIC_REQUIRE(npos_max < (1LL << 31) - kPerTile, TDIC_INVALID_ARG, "integer search: too many positions");
    const int tiles = static_cast<int>((npos_max + kPerTile - 1) / kPerTile);
    Buffer d_part(&ctx->pool, sizeof(Best) * static_cast<size_t>(tiles) * n);
    TDIC_CUDA_TRY(cudaMemcpyAsync(d_geo.ptr, geo.data(), sizeof(CandGeom) * n, cudaMemcpyHostToDevice, s));
    TDIC_CUDA_TRY(cudaMemcpyAsync(d_coff.ptr, coff.data(), sizeof(short2) * coff.size(), cudaMemcpyHostToDevice, s));
    TDIC_CUDA_TRY(cudaMemcpyAsync(d_foff.ptr, foff.data(), sizeof(short2) * foff.size(), cudaMemcpyHostToDevice, s));
    TDIC_CUDA_TRY(cudaMemcpyAsync(d_cok.ptr, cok.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
    // lattice offsets of the coarse samples (dx = -r + cstep * a, so dx + r is a multiple of cstep)
    std::vector<short2> doff(coff.size());
    for (size_t i = 0; i < coff.size(); ++i)
        doff[i] = make_short2(static_cast<short>((coff[i].x + r) / cstep), static_cast<short>((coff[i].y + r) / cstep));
    Buffer d_doff(&ctx->pool, sizeof(short2) * doff.size());
    TDIC_CUDA_TRY(cudaMemcpyAsync(d_doff.ptr, doff.data(), sizeof(short2) * doff.size(), cudaMemcpyHostToDevice, s));
    const size_t csm = search_smem_bytes(static_cast<size_t>(cmax)) + sizeof(short2) * static_cast<size_t>(cmax);
    const size_t fsm = search_smem_bytes(static_cast<size_t>(fmax));
    TDIC_CUDA_TRY(cudaFuncSetAttribute(coarse_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(csm)));
    TDIC_CUDA_TRY(cudaFuncSetAttribute(fine_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(fsm)));
    const float* dref = lazy->ref.as<float>();
    const float* ddef = lazy->def_f.as<float>();
    // the coarse lattice of the deformed image (the image itself when cstep is 1)
    const int dw = (w - 1) / cstep + 1, dh = (h - 1) / cstep + 1;
    Buffer d_dec(&ctx->pool, cstep > 1 ? sizeof(float) * static_cast<size_t>(dw) * dh : 0);
    const float* dec = ddef;
    int dpitch = lazy->rpitch;
    if (cstep > 1) {
        const long long total = static_cast<long long>(dw) * dh;
        const int blocks = static_cast<int>(std::min<long long>((total + 255) / 256, 4096));
        decimate_kernel<<<blocks, 256, 0, s>>>(ddef, lazy->rpitch, cstep, d_dec.as<float>(), dw, dh);
        TDIC_CUDA_TRY(cudaGetLastError());
        dec = d_dec.as<float>();
        dpitch = dw;
    }
    coarse_kernel<<<dim3(tiles, n), kCoarseThreads, csm, s>>>(dref, lazy->rpitch, dec, dpitch, d_geo.as<CandGeom>(),
                                                              d_coff.as<short2>(), d_doff.as<short2>(),
                                                              static_cast<int>(coff.size()), cstep,
                                                              d_part.as<Best>(), tiles);
    TDIC_CUDA_TRY(cudaGetLastError());
    // one block per candidate: 1024 threads (the search windows' positions over every warp the
    // block can hold; the argmax and its scan-order tie rule do not depend on the block size)
    fine_kernel<<<n, kFineThreads, fsm, s>>>(dref, ddef, w, h, lazy->rpitch, r, d_geo.as<CandGeom>(), d_foff.as<short2>(),
                                    static_cast<int>(foff.size()), d_part.as<Best>(), tiles, cstep, rr, search, 1,
                                    d_cok.as<int>(), d_out.as<SearchResult>());
    TDIC_CUDA_TRY(cudaGetLastError());
    TDIC_CUDA_TRY(cudaMemcpyAsync(out_host, d_out.ptr, sizeof(SearchResult) * n, cudaMemcpyDeviceToHost, s));
    TDIC_CUDA_TRY(cudaStreamSynchronize(s));
    for (int i = 0; i < n; ++i)
        if (!ok[i]) out_host[i] = SearchResult{0, 0, -INFINITY, 0};
}

}  // namespace tdic
