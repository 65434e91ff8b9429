// ReliabilityPropagation::propagate in the reference's own visit order on the device.
//
// The reference pops one grid point at a time from a min-heap on ZNSSD and solves every
// admissible, not yet calculated 4-neighbour of it from its parameters
// (src/subset/seed/reliability_propagation.cpp:270-389).  So every solved point has one parent
// -- the first of its accepted neighbours to be popped -- and its result depends only on that
// parent's result.  The order is serial, but it is a function of the results: given every
// point's result, the pops, the parents and the acceptances follow by simulating the heap.
//
// Rounds.  A result table holds, per grid point, the raw solve result of the last time the point
// was solved, the parent it was solved from and the version of that parent's result it used.
//   0. The dataflow propagation fills the table with results from other parents.
//   1. The host simulates the reference's heap loop over the table (the pops, the
//      neighbour admission, the guesses, the acceptance rule and the seed handling of
//      reliability_propagation.cpp:241-389).  Each solve it meets takes the table's result; the
//      point is `dirty` when that result was not computed from this parent's present result.
//   2. No dirty point: the simulation used the right result for every solve, so it is the
//      reference's propagation; its accepted points are the output.
//   3. Otherwise the device solves, in one persistent launch (propagate_kernel in tree mode),
//      every dirty point from its simulated parent and, after it, every point below it in the
//      simulated tree (their guesses change with it), and the host simulates again.
// Every round makes the prefix of the simulated pop sequence that uses exact results longer (the
// first dirty point's parent was exact, so its new result is), so the rounds end; in practice
// after two or three (the parent choices move only where two ZNSSD keys are close).
#include "tdic_internal.cuh"
#include "tie_heap.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <limits>

namespace tdic {

namespace {

int nearest_index(int c, int step, int limit) {  // reliability_propagation.cpp:77-82
    const int idx = static_cast<int>(std::llround(static_cast<double>(c) / static_cast<double>(step)));
    return std::clamp(idx, 0, limit - 1);
}

bool roi_at(const uint8_t* roi, int w, int h, int x, int y) {
    if (x < 0 || y < 0 || x >= w || y >= h) return false;
    return roi == nullptr || roi[static_cast<size_t>(y) * w + x] != 0;
}

constexpr int kMaxRounds = 10000;
constexpr int kUnknownParent = -3;  // results of the dataflow pass: parent not recorded

// The host's copy of the result table and the heap simulation over it, in the solve's precision P
// (the device's acceptance test and guess extrapolation are restated in P).
template <typename P>
struct HeapTable {
    int gw = 0, gh = 0, step = 1, w = 0, h = 0, radius = 0, seed = 0;
    P max_znssd = P(0);
    const uint8_t* roi_grid = nullptr;  // host, gw * gh
    std::vector<P> p;                   // 6 per point
    std::vector<P> corr;
    std::vector<uint8_t> meta;          // status | valid << 2 | converged << 3
    std::vector<uint8_t> have;          // a result is in the table
    std::vector<int> par, ver, src;     // parent solved from, version of the result, parent's version used
    // the last simulation
    std::vector<int> newpar;            // parent of every solve (-1 seed, -2 not solved)
    std::vector<uint8_t> accepted;
    std::vector<int> dirty;
    // What the simulation reads of a solved point, packed (refresh() after a table change): its
    // key, displacement, where its result came from, and the parent-independent part of the
    // acceptance rule (valid, Success, correlation < max_znssd, finite).
    struct Rec {
        double corr;
        P u, v;
        int par, src;
        uint8_t have, ok;
    };
    std::vector<Rec> rec;

    void init(int n) {
        p.assign(6 * static_cast<size_t>(n), P(0));
        corr.assign(n, P(0));
        meta.assign(n, 0);
        have.assign(n, 0);
        par.assign(n, -2);
        ver.assign(n, 0);
        src.assign(n, -1);
        newpar.assign(n, -2);
        accepted.assign(n, 0);
        rec.assign(n, Rec{0.0, P(0), P(0), -2, -1, 0, 0});
    }

    void refresh(int i) {
        const P* r = &p[static_cast<size_t>(i) * 6];
        const bool finite = std::isfinite(r[0]) && std::isfinite(r[1]) && std::isfinite(r[2]) && std::isfinite(r[3]) &&
                            std::isfinite(r[4]) && std::isfinite(r[5]) && std::isfinite(corr[i]);
        Rec& q = rec[i];
        q.corr = static_cast<double>(corr[i]);
        q.u = r[0];
        q.v = r[1];
        q.par = par[i];
        q.src = src[i];
        q.have = have[i];
        q.ok = (meta[i] & 4) && (meta[i] & 3) == TDIC_SUCCESS && corr[i] < max_znssd && finite;
    }

    // The guess of reliability_propagation.cpp:326-329 as the device computes it, from parameters
    // pp of the parent, ddx / ddy px away.
    static void guess(const P* pp, P ddx, P ddy, P (&g)[2]) {
        g[0] = std::fma(pp[3], ddy, std::fma(pp[2], ddx, pp[0]));
        g[1] = std::fma(pp[5], ddy, std::fma(pp[4], ddx, pp[1]));
    }

    // Every pop is recorded (pop_step, calc_step), so the next simulation can start at the first
    // pop that meets a result the round in between changed: the pops before it are the same.
    std::vector<int> calc_step;         // pop at which a point was marked calculated (-1: never)
    std::vector<int> pop_step;          // pop at which a point was popped (-1: never)
    bool sim_valid = false;             // calc_step / pop_step describe the table's last simulation

    TieHeap<P> pq;  // the reference's queue (tie_heap.h), reused by every exact simulation

    // Bucket queue over non-negative keys (ZNSSD and SSD values): the bit pattern of a
    // non-negative double orders like the value; the span of the patterns the simulation can
    // push (the table's keys) is cut into 2^18 buckets of equal width (a 1 MB head array to reset per
    // simulation), a bucket holds its points in a list and a three-level bitmap finds the lowest
    // non-empty bucket.  A pop takes the
    // bucket's smallest key; two equal keys in the queue at once would leave the order to
    // the binary heap's tie rule, so the queue reports a tie and the caller repeats the
    // simulation with the binary heap itself (TieHeap).
    struct BucketQueue {
        static constexpr int kBits = 18;
        std::vector<int> head, next;
        std::vector<uint64_t> key, l0, l1;
        uint64_t l2[4] = {0, 0, 0, 0};
        size_t count = 0;
        bool tie = false;
        uint64_t lo = 0, hi = 0;
        int shift = 0;
        static uint64_t bits_of(double k) {
            uint64_t b;
            std::memcpy(&b, &k, sizeof(b));
            return k == 0.0 ? 0 : b;  // -0.0 is 0
        }
        // keys to come lie in [klo, khi] (both >= 0)
        void init(int n, double klo, double khi) {
            lo = bits_of(klo);
            hi = bits_of(khi);
            shift = 0;
            while (((hi - lo) >> shift) >= (uint64_t(1) << kBits)) ++shift;
            head.assign(size_t(1) << kBits, -1);
            next.assign(n, -1);
            key.assign(n, 0);
            l0.assign((size_t(1) << kBits) / 64, 0);
            l1.assign(l0.size() / 64, 0);
            l2[0] = l2[1] = l2[2] = l2[3] = 0;
            count = 0;
            tie = false;
        }
        bool push(double k, int n) {
            if (!(k >= 0.0)) return false;  // negative or NaN: not orderable here
            const uint64_t b = bits_of(k);
            if (b < lo || b > hi) return false;
            key[n] = b;
            const size_t bk = static_cast<size_t>((b - lo) >> shift);
            next[n] = head[bk];
            head[bk] = n;
            l0[bk >> 6] |= 1ull << (bk & 63);
            l1[bk >> 12] |= 1ull << ((bk >> 6) & 63);
            l2[bk >> 18] |= 1ull << ((bk >> 12) & 63);
            ++count;
            return true;
        }
        int pop() {
            int w2 = 0;
            while (l2[w2] == 0) ++w2;
            const size_t i1 = static_cast<size_t>(w2) * 64 + __builtin_ctzll(l2[w2]);
            const size_t i0 = i1 * 64 + __builtin_ctzll(l1[i1]);
            const size_t bk = i0 * 64 + __builtin_ctzll(l0[i0]);
            int best = head[bk], best_prev = -1, prev = best;
            for (int it = next[best]; it >= 0; prev = it, it = next[it])
                if (key[it] < key[best]) { best = it; best_prev = prev; }
            for (int it = head[bk]; it >= 0; it = next[it])
                if (it != best && key[it] == key[best]) tie = true;
            if (best_prev < 0) head[bk] = next[best]; else next[best_prev] = next[best];
            if (head[bk] < 0) {
                l0[i0] &= ~(1ull << (bk & 63));
                if (l0[i0] == 0) {
                    l1[i1] &= ~(1ull << (i0 & 63));
                    if (l1[i1] == 0) l2[w2] &= ~(1ull << (i1 & 63));
                }
            }
            --count;
            return best;
        }
        bool empty() const { return count == 0; }
    };
    BucketQueue bq;

    // The heap loop of reliability_propagation.cpp:270-389 over the table, from the start of the
    // pop sequence or, given the points the last round changed, from the first pop that meets
    // one of them.
    void simulate(const std::vector<int>* changed = nullptr) {
        const int total = gw * gh;
        int k0 = 0;
        if (changed && sim_valid) {
            k0 = std::numeric_limits<int>::max();
            for (const int x : *changed)
                if (calc_step[x] >= 0) k0 = std::min(k0, calc_step[x]);  // the pop of its parent
            k0 = std::min(k0, total);
        }
        if (!tied && simulate_from(total, k0, false)) return;
        // a tie: the reference's own queue decides, from the start; a table whose keys tied once
        // (a float table's often do) goes to it directly from then on
        tied = true;
        simulate_from(total, 0, true);
    }
    bool tied = false;  // a simulation of this table met two equal keys in the queue

    // Returns false when the bucket queue met a tie (nothing usable was produced).
    bool simulate_from(int total, int k0, bool exact_queue) {
        std::vector<uint8_t> calculated(total, 0);
        if (k0 > 0) {
            // the state after the first k0 pops of the last simulation: every point met before
            // pop k0 kept its result (the round solved only points met later), so it is clean
            for (int i = 0; i < total; ++i) {
                if (calc_step[i] >= 0 && calc_step[i] < k0) {
                    calculated[i] = 1;
                } else {
                    calc_step[i] = -1;
                    newpar[i] = i == seed ? -1 : -2;
                    accepted[i] = i == seed;
                }
                if (pop_step[i] >= k0) pop_step[i] = -1;
            }
            calculated[seed] = 1;
            dirty.clear();
        } else {
            std::fill(newpar.begin(), newpar.end(), -2);
            std::fill(accepted.begin(), accepted.end(), 0);
            calc_step.assign(total, -1);
            pop_step.assign(total, -1);
            dirty.clear();
            calculated[seed] = 1;
            accepted[seed] = 1;
            newpar[seed] = -1;
        }
        pq.n = 0;
        const double seed_key = std::max(0.0, static_cast<double>(corr[seed]));
        if (!exact_queue) {
            double klo = seed_key, khi = seed_key;
            for (int i = 0; i < total; ++i)
                if (rec[i].have && rec[i].corr >= 0.0) {
                    klo = std::min(klo, rec[i].corr);
                    khi = std::max(khi, rec[i].corr);
                }
            bq.init(total, klo, khi);
        }
        auto push = [&](double k, int n) -> bool {
            if (exact_queue) { pq.push(static_cast<P>(k), n); return true; }  // a P key: exact
            return bq.push(k, n);
        };
        int pops = 0;
        if (k0 == 0) {
            if (!push(seed_key, seed)) return false;
        } else {
            // in the queue after k0 pops: points accepted before pop k0 and not popped by then
            pops = k0;
            for (int i = 0; i < total; ++i)
                if (accepted[i] && pop_step[i] < 0 && (i == seed || calc_step[i] >= 0))
                    if (!push(i == seed ? seed_key : rec[i].corr, i)) return false;
        }
        const int dxs[4] = {0, step, 0, -step}, dys[4] = {-step, 0, step, 0};  // up, right, down, left
        const int gdx[4] = {0, 1, 0, -1}, gdy[4] = {-1, 0, 1, 0};
        const P cutoff = static_cast<P>(step);
        for (;;) {
            int n;
            if (exact_queue) {
                if (pq.empty()) break;
                n = pq.top();
                pq.pop();
            } else {
                if (bq.empty()) break;
                n = bq.pop();
                if (bq.tie) return false;
            }
            const int k = pops++;
            pop_step[n] = k;
            const int gy = n / gw, gx = n - gy * gw;
            const int vn = ver[n];
            const P* pp = &p[static_cast<size_t>(n) * 6];
            for (int d = 0; d < 4; ++d) {
                const int gnx = gx + gdx[d], gny = gy + gdy[d];  // the neighbour (px + dxs[d], py + dys[d])
                const int nx = gnx * step, ny = gny * step;
                if (nx < 0 || ny < 0 || nx >= w || ny >= h) continue;
                if (gnx >= gw || gny >= gh) continue;
                const int m = gny * gw + gnx;
                if (calculated[m]) continue;
                calculated[m] = 1;
                calc_step[m] = k;
                if (!roi_grid[m]) continue;
                if (nx - radius < 0 || ny - radius < 0 || nx + radius >= w || ny + radius >= h) continue;
                newpar[m] = n;
                const Rec& r = rec[m];
                if (!(r.have && r.par == n && r.src == vn)) dirty.push_back(m);
                if (!r.have || !r.ok) continue;  // never solved, or refused whatever the guess
                P g[2];
                guess(pp, static_cast<P>(dxs[d]), static_cast<P>(dys[d]), g);
                if (std::fabs(g[0] - r.u) < cutoff && std::fabs(g[1] - r.v) < cutoff) {  // :359-368
                    accepted[m] = 1;
                    if (!push(r.corr, m)) return false;
                }
            }
        }
        sim_valid = true;
        return true;
    }
};

// The tree of one round: the points to solve (every dirty point and every point below one in the
// simulated tree), their children, the child each solving group continues with (the one with the
// deepest subtree) and the roots (points whose parent keeps its result).
struct RoundTree {
    std::vector<int> child_off, child, cont, roots, order;  // order: the solved points, parents first
};

void build_round(const std::vector<int>& newpar, const std::vector<int>& dirty, int seed, int total, RoundTree& t) {
    t.child_off.assign(total + 1, 0);
    for (int i = 0; i < total; ++i)
        if (newpar[i] >= 0) ++t.child_off[newpar[i] + 1];
    for (int i = 0; i < total; ++i) t.child_off[i + 1] += t.child_off[i];
    t.child.assign(t.child_off[total], 0);
    {
        std::vector<int> fill(t.child_off.begin(), t.child_off.end() - 1);
        for (int i = 0; i < total; ++i)  // ascending point index within each parent
            if (newpar[i] >= 0) t.child[fill[newpar[i]]++] = i;
    }
    std::vector<uint8_t> is_dirty(total, 0), in_round(total, 0);
    for (int d : dirty) is_dirty[d] = 1;
    // breadth-first from the seed: a point is solved this round when it or an ancestor is dirty
    t.order.clear();
    t.roots.clear();
    std::vector<int> bfs;
    bfs.reserve(total);
    bfs.push_back(seed);
    for (size_t k = 0; k < bfs.size(); ++k) {
        const int x = bfs[k];
        for (int i = t.child_off[x]; i < t.child_off[x + 1]; ++i) {
            const int c = t.child[i];
            in_round[c] = is_dirty[c] || in_round[x];
            if (in_round[c]) {
                t.order.push_back(c);
                if (!in_round[x]) t.roots.push_back(c);
            }
            bfs.push_back(c);
        }
    }
    // continuation: the child with the deepest subtree (children of a point solved this round are
    // all solved this round)
    std::vector<int> height(total, 0);
    t.cont.assign(total, -1);
    for (auto it = t.order.rbegin(); it != t.order.rend(); ++it) {
        const int x = *it;
        int best = -1, bh = -1;
        for (int i = t.child_off[x]; i < t.child_off[x + 1]; ++i)
            if (height[t.child[i]] > bh) { bh = height[t.child[i]]; best = t.child[i]; }
        t.cont[x] = best;
        height[x] = 1 + (bh < 0 ? 0 : bh);
    }
}

template <typename P>
void heap_rounds(tdic_ctx* ctx, tdic_pair* pair, const tdic_config& cfg, const tdic_seed& seed, const uint8_t* roi,
                 const tdic_grid_out& out, int32_t* points_computed, cudaStream_t s) {
    const int w = pair->w, h = pair->h;
    const int step = std::max(0, cfg.propagation_spacing) + 1;
    int32_t gw, gh;
    tdic_grid_dims(w, h, cfg.propagation_spacing, &gw, &gh);
    const int n = gw * gh;
    const bool so = cfg.shape_order == 2;
    *points_computed = 0;
    // seed alignment (reliability_propagation.cpp:201-216)
    const int sxr = static_cast<int>(std::round(seed.x)), syr = static_cast<int>(std::round(seed.y));
    bool seed_ok = seed.found != 0 && roi_at(roi, w, h, sxr, syr);
    int gxs = 0, gys = 0;
    if (seed_ok) {
        gxs = nearest_index(sxr, step, gw);
        gys = nearest_index(syr, step, gh);
        seed_ok = roi_at(roi, w, h, gxs * step, gys * step);
    }
    if (!seed_ok) {
        launch_init_grid(out, gw, gh, step, s);
        check_device_error(ctx, s);
        return;
    }
    const int sidx = gys * gw + gxs;
    std::vector<uint8_t> roi_grid(n, 1);
    if (roi)
        for (int i = 0; i < n; ++i) roi_grid[i] = roi[static_cast<size_t>((i / gw) * step) * w + (i % gw) * step] ? 1 : 0;

    // device state: the dataflow pass's scratch, then the rounds' tree and result table
    Buffer d_roi(&ctx->pool, n), claim(&ctx->pool, sizeof(int) * n);
    Buffer keyparams(&ctx->pool, (sizeof(unsigned long long) + 6 * sizeof(double)) * n);
    Buffer order(&ctx->pool, sizeof(int) * n), fetch(&ctx->pool, sizeof(int) * (n + 2)), misc(&ctx->pool, 64);
    Buffer dstate(&ctx->pool, sizeof(int) * n), dcnt(&ctx->pool, sizeof(int) * n);
    Buffer dq(&ctx->pool, sizeof(unsigned long long) * n), kcorr(&ctx->pool, sizeof(float) * n);
    Buffer t_off(&ctx->pool, sizeof(int) * (n + 1)), t_child(&ctx->pool, sizeof(int) * n), t_cont(&ctx->pool, sizeof(int) * n);
    Buffer r_corr(&ctx->pool, sizeof(P) * n), r_q(&ctx->pool, so ? sizeof(P) * 6 * n : 0);
    Buffer r_meta(&ctx->pool, n), r_iters(&ctx->pool, sizeof(int) * n), d_acc(&ctx->pool, n);
    Buffer o_corr(&ctx->pool, sizeof(double) * n), o_iters(&ctx->pool, sizeof(int32_t) * n);
    Buffer o_valid(&ctx->pool, n), o_conv(&ctx->pool, n), o_q(&ctx->pool, so ? sizeof(double) * 6 * n : 0);
    Buffer d_roi_px(&ctx->pool, cfg.truncate_roi_subsets ? static_cast<size_t>(w) * h : 0);
    if (cfg.truncate_roi_subsets) {
        if (roi) TDIC_CUDA_TRY(cudaMemcpyAsync(d_roi_px.ptr, roi, static_cast<size_t>(w) * h, cudaMemcpyHostToDevice, s));
        else TDIC_CUDA_TRY(cudaMemsetAsync(d_roi_px.ptr, 1, static_cast<size_t>(w) * h, s));
    }
    TDIC_CUDA_TRY(cudaMemcpyAsync(d_roi.ptr, roi_grid.data(), n, cudaMemcpyHostToDevice, s));
    P* d_params = reinterpret_cast<P*>(keyparams.as<unsigned long long>() + n);
    int* m = misc.as<int>();

    auto reset_queue = [&](unsigned long long tail) {  // head 0; tail : in flight (bias 2^31)
        TDIC_CUDA_TRY(cudaMemsetAsync(misc.ptr, 0, 64, s));
        const unsigned long long q0 = (tail << 32) | (0x80000000ull + tail);
        TDIC_CUDA_TRY(cudaMemcpyAsync(m + 4, &q0, sizeof(q0), cudaMemcpyHostToDevice, s));
        TDIC_CUDA_TRY(cudaMemsetAsync(dq.ptr, 0xff, sizeof(unsigned long long) * n, s));
    };
    PropagateLaunch L{};
    L.gw = gw; L.gh = gh; L.step = step;
    L.roi_grid = d_roi.as<uint8_t>();
    L.roi_px = cfg.truncate_roi_subsets ? d_roi_px.as<uint8_t>() : nullptr;
    L.claim = claim.as<int>();
    L.key = keyparams.as<unsigned long long>();
    L.order = order.as<int>();
    L.counters = m;
    L.barrier = reinterpret_cast<unsigned int*>(m + 8);
    L.flags = m + 12;
    L.fetch = fetch.as<int>();
    L.sgx = gxs; L.sgy = gys;
    L.dstate = dstate.as<int>(); L.dcnt = dcnt.as<int>();
    L.dq = dq.as<unsigned long long>(); L.kcorr = kcorr.as<float>();
    SetupCache cache;  // shared by every round: a point's set-up does not change
    if (setup_cache_applies(cfg)) setup_cache_prepare(ctx, pair, gw, gh, gxs, gys, cache, L, s);

    // ---- round 0: the dataflow propagation (its parents are not the heap's) ---------------------
    tdic_grid_out o0{};
    o0.correlation = o_corr.as<double>();
    o0.valid = o_valid.as<uint8_t>();
    o0.iterations = o_iters.as<int32_t>();
    o0.converged = o_conv.as<uint8_t>();
    if (so) {  // the seed's second-order terms (the parameter table keeps the first-order six)
        double* q = o_q.as<double>();
        o0.d2u_dx2 = q; o0.d2u_dxdy = q + n; o0.d2u_dy2 = q + 2 * static_cast<size_t>(n);
        o0.d2v_dx2 = q + 3 * static_cast<size_t>(n); o0.d2v_dxdy = q + 4 * static_cast<size_t>(n);
        o0.d2v_dy2 = q + 5 * static_cast<size_t>(n);
    }
    TDIC_CUDA_TRY(cudaMemsetAsync(dstate.ptr, 0, sizeof(int) * n, s));
    TDIC_CUDA_TRY(cudaMemsetAsync(dcnt.ptr, 0, sizeof(int) * n, s));
    TDIC_CUDA_TRY(cudaMemsetAsync(claim.ptr, 0, sizeof(int) * n, s));
    TDIC_CUDA_TRY(cudaMemsetAsync(keyparams.ptr, 0xff, sizeof(unsigned long long) * n, s));
    TDIC_CUDA_TRY(cudaMemsetAsync(fetch.ptr, 0, sizeof(int) * (n + 2), s));
    reset_queue(0);
    L.mode = 2;
    L.seed_idx = sidx;
    L.seed_solve = (gxs * step != sxr || gys * step != syr) ? 1 : 0;
    for (int k = 0; k < 6; ++k) L.seed_p[k] = seed.p[k];
    L.seed_corr = seed.correlation;
    L.out = o0;
    launch_propagate(ctx, pair, cfg, L, s);
    int flags[3] = {0, 0, 0};
    HeapTable<P> t;
    t.gw = gw; t.gh = gh; t.step = step; t.w = w; t.h = h; t.radius = cfg.subset_radius; t.seed = sidx;
    t.max_znssd = static_cast<P>(cfg.propagation_max_znssd);
    t.roi_grid = roi_grid.data();
    t.init(n);
    std::vector<double> c0(n);
    std::vector<uint8_t> v0(n), conv0(n);
    std::vector<int32_t> it0(n);
    TDIC_CUDA_TRY(cudaMemcpyAsync(flags, L.flags, sizeof(flags), cudaMemcpyDeviceToHost, s));
    TDIC_CUDA_TRY(cudaMemcpyAsync(t.p.data(), d_params, sizeof(P) * 6 * n, cudaMemcpyDeviceToHost, s));
    TDIC_CUDA_TRY(cudaMemcpyAsync(c0.data(), o0.correlation, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    TDIC_CUDA_TRY(cudaMemcpyAsync(v0.data(), o0.valid, n, cudaMemcpyDeviceToHost, s));
    TDIC_CUDA_TRY(cudaMemcpyAsync(it0.data(), o0.iterations, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, s));
    TDIC_CUDA_TRY(cudaMemcpyAsync(conv0.data(), o0.converged, n, cudaMemcpyDeviceToHost, s));
    check_device_error(ctx, s);
    TDIC_REQUIRE(flags[0] == 0, TDIC_TIMEOUT, "propagation: a bounded in-kernel wait timed out");
    if (flags[1]) {  // the aligned seed failed: the reference returns no point (the defaults)
        launch_init_grid(out, gw, gh, step, s);
        check_device_error(ctx, s);
        return;
    }
    for (int i = 0; i < n; ++i) {
        if (!v0[i]) continue;
        t.corr[i] = static_cast<P>(c0[i]);  // exact: the outputs hold the P values widened
        t.meta[i] = static_cast<uint8_t>(TDIC_SUCCESS | 4 | (conv0[i] ? 8 : 0));
        t.have[i] = 1;
        t.par[i] = kUnknownParent;
    }
    t.par[sidx] = -1;
    t.ver[sidx] = 1;
    for (int i = 0; i < n; ++i) t.refresh(i);
    // the seed's entry of the device result table (the rounds never solve it again; its
    // first-order parameters are in the parameter table already)
    {
        const P sc = t.corr[sidx];
        const unsigned char sm = t.meta[sidx];
        const int si = it0[sidx];
        P sq[6] = {};
        if (so)
            for (int k = 0; k < 6; ++k) {
                double v = 0.0;
                TDIC_CUDA_TRY(cudaMemcpy(&v, o_q.as<double>() + static_cast<size_t>(k) * n + sidx, sizeof(double),
                                         cudaMemcpyDeviceToHost));
                sq[k] = static_cast<P>(v);
            }
        TDIC_CUDA_TRY(cudaMemcpyAsync(r_corr.as<P>() + sidx, &sc, sizeof(P), cudaMemcpyHostToDevice, s));
        TDIC_CUDA_TRY(cudaMemcpyAsync(r_meta.as<unsigned char>() + sidx, &sm, 1, cudaMemcpyHostToDevice, s));
        TDIC_CUDA_TRY(cudaMemcpyAsync(r_iters.as<int>() + sidx, &si, sizeof(int), cudaMemcpyHostToDevice, s));
        if (so)
            TDIC_CUDA_TRY(cudaMemcpyAsync(r_q.as<P>() + 6 * static_cast<size_t>(sidx), sq, sizeof(sq),
                                          cudaMemcpyHostToDevice, s));
        TDIC_CUDA_TRY(cudaStreamSynchronize(s));  // the host values above go out of scope
    }

    // ---- rounds ------------------------------------------------------------------------------
    RoundTree rt;
    std::vector<P> rc(n);
    std::vector<unsigned char> rm(n);
    int rounds = 0;
    ctx->heap_rounds = 0;
    ctx->heap_solves = 0;
    ctx->heap_sim_ms = 0.0;
    std::vector<int> changed;  // points the last round solved again
    for (;;) {
        const auto t_sim = std::chrono::steady_clock::now();
        t.simulate(rounds > 0 ? &changed : nullptr);
        ctx->heap_sim_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_sim).count();
        if (t.dirty.empty()) break;
        TDIC_REQUIRE(++rounds <= kMaxRounds, TDIC_TIMEOUT, "heap-order propagation did not settle");
        build_round(t.newpar, t.dirty, sidx, n, rt);
        std::vector<unsigned long long> items(rt.roots.size());
        for (size_t k = 0; k < rt.roots.size(); ++k)
            items[k] = (static_cast<unsigned long long>(static_cast<unsigned int>(t.newpar[rt.roots[k]])) << 32) |
                       static_cast<unsigned int>(rt.roots[k]);
        reset_queue(items.size());
        TDIC_CUDA_TRY(cudaMemcpyAsync(dq.ptr, items.data(), sizeof(unsigned long long) * items.size(),
                                      cudaMemcpyHostToDevice, s));
        TDIC_CUDA_TRY(cudaMemcpyAsync(t_off.ptr, rt.child_off.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, s));
        if (!rt.child.empty())
            TDIC_CUDA_TRY(cudaMemcpyAsync(t_child.ptr, rt.child.data(), sizeof(int) * rt.child.size(),
                                          cudaMemcpyHostToDevice, s));
        TDIC_CUDA_TRY(cudaMemcpyAsync(t_cont.ptr, rt.cont.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
        L.mode = 3;
        L.seed_idx = -1;  // placed in round 0
        L.seed_solve = 0;
        L.tchild_off = t_off.as<int>(); L.tchild = t_child.as<int>(); L.tcont = t_cont.as<int>();
        L.rcorr = r_corr.ptr; L.rq = so ? r_q.ptr : nullptr;
        L.rmeta = r_meta.as<unsigned char>(); L.riters = r_iters.as<int>();
        launch_propagate(ctx, pair, cfg, L, s);
        TDIC_CUDA_TRY(cudaMemcpyAsync(flags, L.flags, sizeof(flags), cudaMemcpyDeviceToHost, s));
        TDIC_CUDA_TRY(cudaMemcpyAsync(t.p.data(), d_params, sizeof(P) * 6 * n, cudaMemcpyDeviceToHost, s));
        TDIC_CUDA_TRY(cudaMemcpyAsync(rc.data(), r_corr.ptr, sizeof(P) * n, cudaMemcpyDeviceToHost, s));
        TDIC_CUDA_TRY(cudaMemcpyAsync(rm.data(), r_meta.ptr, n, cudaMemcpyDeviceToHost, s));
        check_device_error(ctx, s);
        TDIC_REQUIRE(flags[0] == 0, TDIC_TIMEOUT, "propagation: a bounded in-kernel wait timed out");
        ctx->heap_rounds = rounds;
        ctx->heap_solves += static_cast<long long>(rt.order.size());
        changed = rt.order;
        for (const int x : rt.order) {  // parents first: a child records its parent's new version
            t.corr[x] = rc[x];
            t.meta[x] = rm[x];
            t.have[x] = 1;
            t.par[x] = t.newpar[x];
            t.ver[x] += 1;
            t.src[x] = t.ver[t.newpar[x]];
            t.refresh(x);
        }
    }
    // ---- outputs: the accepted points of the last simulation -------------------------------
    int computed = 0;
    for (int i = 0; i < n; ++i) computed += t.accepted[i];
    TDIC_CUDA_TRY(cudaMemcpyAsync(d_acc.ptr, t.accepted.data(), n, cudaMemcpyHostToDevice, s));
    launch_emit_tree(out, gw, gh, step, pair->precision, d_params, r_corr.ptr, so ? r_q.ptr : nullptr,
                     r_meta.as<unsigned char>(), r_iters.as<int>(), d_acc.as<unsigned char>(), s);
    check_device_error(ctx, s);
    *points_computed = computed;
}

}  // namespace

void heap_propagate(tdic_ctx* ctx, tdic_pair* pair, const tdic_config& cfg, const tdic_seed& seed, const uint8_t* roi,
                    const tdic_grid_out& out_dev, int32_t* points_computed, cudaStream_t s) {
    if (pair->precision == TDIC_FP64) heap_rounds<double>(ctx, pair, cfg, seed, roi, out_dev, points_computed, s);
    else heap_rounds<float>(ctx, pair, cfg, seed, roi, out_dev, points_computed, s);
}

}  // namespace tdic
