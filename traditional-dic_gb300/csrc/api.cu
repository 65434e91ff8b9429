// C ABI of libtdic_gb300 (declared in include/tdic_gb300.h).  Host-side orchestration only:
// argument checks, device memory from the context pool, the seed-alignment and grid geometry
// of ReliabilityPropagation::propagate, k-means seed candidates of SeedSelector, and the
// stream-ordered launches of the kernels in prefilter.cu, hotpath.cu and seed.cu.
#include "tdic_internal.cuh"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <mutex>
#include <numeric>

namespace tdic {

void upload_qk_constants();

// ---------------------------------------------------------------------------------------
// DevicePool
// ---------------------------------------------------------------------------------------
size_t DevicePool::size_class(size_t bytes) {
    if (bytes <= 4096) return 4096;
    size_t c = 4096;
    while (c < bytes && c < (size_t(1) << 26)) c <<= 1;         // powers of two up to 64 MiB
    if (c >= bytes) return c;
    const size_t chunk = size_t(1) << 24;                       // then 16 MiB granules
    return (bytes + chunk - 1) / chunk * chunk;
}

void* DevicePool::acquire(size_t bytes) {
    const size_t c = size_class(bytes);
    auto it = free_.find(c);
    void* p = nullptr;
    if (it != free_.end()) {
        p = it->second;
        free_.erase(it);
    } else {
        cudaError_t e = cudaMalloc(&p, c);
        if (e != cudaSuccess) {
            trim();
            e = cudaMalloc(&p, c);
            if (e != cudaSuccess) {
                (void)cudaGetLastError();
                throw Error{TDIC_OOM, "device allocation of " + std::to_string(c) + " bytes failed"};
            }
        }
        held_ += c;
    }
    live_[p] = c;
    return p;
}

void DevicePool::release(void* p) {
    auto it = live_.find(p);
    if (it == live_.end()) return;
    free_.emplace(it->second, p);
    live_.erase(it);
}

void DevicePool::trim() {
    for (auto& kv : free_) {
        cudaFree(kv.second);
        held_ -= kv.first;
    }
    free_.clear();
}

// ---------------------------------------------------------------------------------------
// B-spline qk matrix (bspline.cpp:320-367), host side
// ---------------------------------------------------------------------------------------
namespace {
int fact(int n) { int v = 1; for (int i = 2; i <= n; ++i) v *= i; return v; }
int comb(int n, int k) { return (k < 0 || k > n) ? 0 : fact(n) / (fact(k) * fact(n - k)); }
double basis(double x, int r, int d) {
    if (r < 0 || r > d) return 0.0;
    const int dfac = fact(d) / fact(d - r);
    double sum = 0.0;
    for (int k = 0; k <= d + 1; ++k) {
        const double sign = k % 2 == 0 ? 1.0 : -1.0;
        const double shift = static_cast<double>(d + 1) / 2.0 - static_cast<double>(k);
        const double xx = x + shift;
        sum += sign * comb(d + 1, k) * dfac * (xx > 0.0 ? std::pow(xx, d - r) : 0.0);
    }
    return sum / static_cast<double>(fact(d));
}
}  // namespace

void build_qk(int d, double* qk) {
    const int n = d + 1, off = d / 2;
    for (int r = 0; r < n; ++r)
        for (int c = 0; c < n; ++c) {
            const double sign = r % 2 == 0 ? 1.0 : -1.0;
            qk[r * n + c] = sign * basis(static_cast<double>(-off + c), r, d) / static_cast<double>(fact(r));
        }
}

void check_device_error(tdic_ctx* ctx, cudaStream_t s) {
    int v = 0;
    TDIC_CUDA_TRY(cudaMemcpyAsync(&v, ctx->dev_err, sizeof(int), cudaMemcpyDeviceToHost, s));
    TDIC_CUDA_TRY(cudaStreamSynchronize(s));
    if (v != 0) {
        TDIC_CUDA_TRY(cudaMemsetAsync(ctx->dev_err, 0, sizeof(int), s));
        throw Error{TDIC_TIMEOUT, "a bounded in-kernel wait (TMA copy) timed out"};
    }
}

void setup_cache_prepare(tdic_ctx* ctx, tdic_pair* pair, int gw, int gh, int sgx, int sgy, SetupCache& c,
                         PropagateLaunch& L, cudaStream_t s) {
    const size_t n = static_cast<size_t>(gw) * gh;
    const size_t m = pair->precision == TDIC_FP64 ? sizeof(double) : sizeof(float);
    c.hinv = Buffer(&ctx->pool, 36 * m * n);
    c.fmn = Buffer(&ctx->pool, 2 * m * n);
    c.state = Buffer(&ctx->pool, sizeof(int) * n);
    c.ticket = Buffer(&ctx->pool, sizeof(int));
    TDIC_CUDA_TRY(cudaMemsetAsync(c.state.ptr, 0, sizeof(int) * n, s));
    TDIC_CUDA_TRY(cudaMemsetAsync(c.ticket.ptr, 0, sizeof(int), s));
    const int key[3] = {gw, gh, sgy * gw + sgx};
    if (!(key[0] == ctx->pre_key[0] && key[1] == ctx->pre_key[1] && key[2] == ctx->pre_key[2])) {
        // counting sort of the grid points by Manhattan distance from the seed (index order within)
        const int dmax = gw + gh;
        std::vector<int> count(dmax + 2, 0), order(n);
        for (size_t i = 0; i < n; ++i)
            ++count[std::abs(static_cast<int>(i % gw) - sgx) + std::abs(static_cast<int>(i / gw) - sgy) + 1];
        for (int d = 0; d <= dmax; ++d) count[d + 1] += count[d];
        for (size_t i = 0; i < n; ++i)
            order[count[std::abs(static_cast<int>(i % gw) - sgx) + std::abs(static_cast<int>(i / gw) - sgy)]++] =
                static_cast<int>(i);
        // the copy must land before `order` goes out of scope
        ctx->pre_key[0] = -1;
        ctx->pre_order = Buffer(&ctx->pool, sizeof(int) * n);
        TDIC_CUDA_TRY(cudaMemcpyAsync(ctx->pre_order.ptr, order.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
        TDIC_CUDA_TRY(cudaStreamSynchronize(s));
        ctx->pre_key[0] = key[0]; ctx->pre_key[1] = key[1]; ctx->pre_key[2] = key[2];
        ctx->pre_count = static_cast<int>(n);
    }
    L.sc_hinv = c.hinv.ptr;
    L.sc_fmn = c.fmn.ptr;
    L.sc_state = c.state.as<int>();
    L.pre_order = ctx->pre_order.as<int>();
    L.pre_count = ctx->pre_count;
    L.pre_ticket = c.ticket.as<int>();
}

const SampleTable& sample_table(tdic_ctx* ctx, int radius) {
    auto it = ctx->tables.find(radius);
    if (it != ctx->tables.end()) return it->second;
    std::vector<short2> off;
    for (int dy = -radius; dy <= radius; ++dy)
        for (int dx = -radius; dx <= radius; ++dx)
            if (dx * dx + dy * dy <= radius * radius) off.push_back(make_short2(static_cast<short>(dx), static_cast<short>(dy)));
    SampleTable t;
    t.n = static_cast<int>(off.size());
    t.offsets = Buffer(&ctx->pool, sizeof(short2) * std::max<size_t>(off.size(), 1));
    TDIC_CUDA_TRY(cudaMemcpy(t.offsets.ptr, off.data(), sizeof(short2) * off.size(), cudaMemcpyHostToDevice));
    auto res = ctx->tables.emplace(radius, std::move(t));
    return res.first->second;
}

}  // namespace tdic

using namespace tdic;

namespace {

template <typename F>
tdic_status guarded(tdic_ctx* ctx, F&& f) {
    if (!ctx) return TDIC_INVALID_ARG;
    std::lock_guard<std::recursive_mutex> lock(ctx->mu);
    try {
        f();
        return TDIC_OK;
    } catch (const Error& e) {
        ctx->last_error = e.msg;
        return e.code;
    } catch (const std::exception& e) {
        ctx->last_error = e.what();
        return TDIC_INVALID_ARG;
    }
}

cudaStream_t pick(tdic_ctx* ctx, void* s) { return s ? static_cast<cudaStream_t>(s) : ctx->stream; }

size_t dtype_size(tdic_dtype t) {
    switch (t) {
        case TDIC_U8: return 1;
        case TDIC_U16: return 2;
        case TDIC_F32: return 4;
        case TDIC_F64: return 8;
    }
    return 0;
}

bool first_order_znssd(const tdic_config& c) { return c.shape_order == 1 && c.criterion == 1; }

int normalized_degree(int d) { return (d == 1 || d == 3) ? d : 5; }

void check_config(const tdic_config& c) {
    TDIC_REQUIRE(c.optimizer == 0 || c.optimizer == 1, TDIC_INVALID_ARG, "optimizer must be 0 (icgn) or 1 (fgn)");
    TDIC_REQUIRE(c.shape_order == 1 || c.shape_order == 2, TDIC_INVALID_ARG, "shape_order must be 1 or 2");
    TDIC_REQUIRE(c.criterion == 0 || c.criterion == 1, TDIC_INVALID_ARG, "criterion must be 1 (znssd) or 0 (ssd)");
    TDIC_REQUIRE(c.subset_radius >= 1 && c.subset_radius <= 100, TDIC_INVALID_ARG, "subset radius must be in [1, 100]");
    TDIC_REQUIRE(c.max_iterations >= 0, TDIC_INVALID_ARG, "max_iterations must be >= 0");
    TDIC_REQUIRE(c.propagation_spacing < (1 << 30), TDIC_INVALID_ARG, "propagation spacing must be below 2^30");
}

void check_memory(tdic_memory mem) {
    TDIC_REQUIRE(mem == TDIC_HOST || mem == TDIC_DEVICE, TDIC_INVALID_ARG, "memory must be TDIC_HOST or TDIC_DEVICE");
}

// The pair's device images from the caller's (host: staged through one upload buffer holding
// both; device: read in place): exact cubic / quintic pairs in one fused launch (float32
// reference, float32 deformed copy, coefficients), others by conversion plus a padded copy.
void pair_compute(tdic_pair* p, const void* ref, const void* def, int pitch, tdic_dtype dtype, tdic_memory mem,
                  cudaStream_t s) {
    const size_t es = dtype_size(dtype);
    TDIC_REQUIRE(es != 0, TDIC_INVALID_ARG, "unknown dtype");
    check_memory(mem);
    const int pt = pitch > 0 ? pitch : p->w;
    TDIC_REQUIRE(pt >= p->w, TDIC_INVALID_ARG, "pitch smaller than width");
    const void* dref = ref;
    const void* ddef = def;
    if (mem == TDIC_HOST) {
        const size_t bytes = es * static_cast<size_t>(pt) * p->h;
        const size_t slot = (bytes + 255) / 256 * 256;
        if (p->staging.bytes < 2 * slot) p->staging = Buffer(&p->ctx->pool, 2 * slot);
        auto* base = static_cast<unsigned char*>(p->staging.ptr);
        TDIC_CUDA_TRY(cudaMemcpyAsync(base, ref, bytes, cudaMemcpyHostToDevice, s));
        TDIC_CUDA_TRY(cudaMemcpyAsync(base + slot, def, bytes, cudaMemcpyHostToDevice, s));
        dref = base;
        ddef = base + slot;
    }
    if (p->exact && p->degree != 1) {
        launch_pair_setup(p, dref, ddef, pt, dtype, s);
        return;
    }
    launch_convert(dref, p->w, p->h, pt, dtype, p->ref.as<float>(), p->rpitch, s);
    launch_convert(ddef, p->w, p->h, pt, dtype, p->def_f.as<float>(), p->rpitch, s);
    launch_prefilter(p, p->def_f.as<float>(), s);
}

int nearest_grid_index(int c, int step, int limit) {  // reliability_propagation.cpp:77-82
    const int idx = static_cast<int>(std::llround(static_cast<double>(c) / static_cast<double>(step)));
    return std::clamp(idx, 0, limit - 1);
}

bool roi_ok(const uint8_t* roi, int w, int h, int x, int y) {
    if (x < 0 || y < 0 || x >= w || y >= h) return false;
    return roi == nullptr || roi[static_cast<size_t>(y) * w + x] != 0;
}

// Device SoA output, either the caller's device arrays or pool buffers copied back.
struct GridBuffers {
    Buffer d[20];
    tdic_grid_out dev{};
};

void alloc_grid(tdic_ctx* ctx, GridBuffers& g, int n, const tdic_grid_out* host_wanted) {
    double** dptrs[16] = {&g.dev.x, &g.dev.y, &g.dev.u, &g.dev.v, &g.dev.du_dx, &g.dev.du_dy, &g.dev.dv_dx, &g.dev.dv_dy,
                          &g.dev.correlation, &g.dev.zncc, &g.dev.d2u_dx2, &g.dev.d2u_dxdy, &g.dev.d2u_dy2,
                          &g.dev.d2v_dx2, &g.dev.d2v_dxdy, &g.dev.d2v_dy2};
    double* const* hptrs[16] = {&host_wanted->x, &host_wanted->y, &host_wanted->u, &host_wanted->v, &host_wanted->du_dx,
                                &host_wanted->du_dy, &host_wanted->dv_dx, &host_wanted->dv_dy, &host_wanted->correlation,
                                &host_wanted->zncc, &host_wanted->d2u_dx2, &host_wanted->d2u_dxdy, &host_wanted->d2u_dy2,
                                &host_wanted->d2v_dx2, &host_wanted->d2v_dxdy, &host_wanted->d2v_dy2};
    for (int i = 0; i < 16; ++i) {
        const int slot = i < 10 ? i : i + 4;
        if (*hptrs[i]) {
            g.d[slot] = Buffer(&ctx->pool, sizeof(double) * n);
            *dptrs[i] = g.d[slot].as<double>();
        }
    }
    if (host_wanted->valid) { g.d[10] = Buffer(&ctx->pool, n); g.dev.valid = g.d[10].as<uint8_t>(); }
    if (host_wanted->status) { g.d[11] = Buffer(&ctx->pool, n); g.dev.status = g.d[11].as<int8_t>(); }
    if (host_wanted->iterations) { g.d[12] = Buffer(&ctx->pool, sizeof(int32_t) * n); g.dev.iterations = g.d[12].as<int32_t>(); }
    if (host_wanted->converged) { g.d[13] = Buffer(&ctx->pool, n); g.dev.converged = g.d[13].as<uint8_t>(); }
}

void copy_grid_back(const GridBuffers& g, const tdic_grid_out* h, int n, cudaStream_t s) {
    auto cp = [&](void* dst, const void* src, size_t bytes) {
        if (dst && src) TDIC_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s));
    };
    cp(h->x, g.dev.x, 8 * n); cp(h->y, g.dev.y, 8 * n); cp(h->u, g.dev.u, 8 * n); cp(h->v, g.dev.v, 8 * n);
    cp(h->du_dx, g.dev.du_dx, 8 * n); cp(h->du_dy, g.dev.du_dy, 8 * n); cp(h->dv_dx, g.dev.dv_dx, 8 * n);
    cp(h->dv_dy, g.dev.dv_dy, 8 * n); cp(h->correlation, g.dev.correlation, 8 * n); cp(h->zncc, g.dev.zncc, 8 * n);
    cp(h->valid, g.dev.valid, n); cp(h->status, g.dev.status, n); cp(h->iterations, g.dev.iterations, 4 * n);
    cp(h->converged, g.dev.converged, n);
    cp(h->d2u_dx2, g.dev.d2u_dx2, 8 * n); cp(h->d2u_dxdy, g.dev.d2u_dxdy, 8 * n); cp(h->d2u_dy2, g.dev.d2u_dy2, 8 * n);
    cp(h->d2v_dx2, g.dev.d2v_dx2, 8 * n); cp(h->d2v_dxdy, g.dev.d2v_dxdy, 8 * n); cp(h->d2v_dy2, g.dev.d2v_dy2, 8 * n);
}

void propagate_impl(tdic_ctx* ctx, tdic_pair* pair, const tdic_config& cfg, const tdic_seed& seed, const uint8_t* roi,
                    const tdic_grid_out* out, tdic_memory mem, int32_t* points_computed, cudaStream_t s) {
    check_config(cfg);
    check_memory(mem);
    TDIC_REQUIRE(pair->exact == 1, TDIC_INVALID_ARG, "propagation needs a pair with the exact prefilter");
    TDIC_REQUIRE(cfg.propagation_mode >= 0 && cfg.propagation_mode <= 2, TDIC_INVALID_ARG,
                 "propagation_mode must be 0 (frontier waves), 1 (heap order) or 2 (dataflow)");
    const int w = pair->w, h = pair->h;
    const int step = std::max(0, cfg.propagation_spacing) + 1;
    int32_t gw, gh;
    tdic_grid_dims(w, h, cfg.propagation_spacing, &gw, &gh);
    const int n = gw * gh;
    *points_computed = 0;
    // Seed alignment on the host (reliability_propagation.cpp:201-216).
    const int sxr = static_cast<int>(std::round(seed.x)), syr = static_cast<int>(std::round(seed.y));
    bool seed_ok = seed.found != 0 && roi_ok(roi, w, h, sxr, syr);
    int gxs = 0, gys = 0;
    if (seed_ok) {
        gxs = nearest_grid_index(sxr, step, gw);
        gys = nearest_grid_index(syr, step, gh);
        seed_ok = roi_ok(roi, w, h, gxs * step, gys * step);
    }
    // ROI at the grid points
    std::vector<uint8_t> roi_grid(n, 1);
    if (roi)
        for (int i = 0; i < n; ++i) roi_grid[i] = roi[static_cast<size_t>((i / gw) * step) * w + (i % gw) * step] ? 1 : 0;
    GridBuffers gb;
    if (mem == TDIC_DEVICE) gb.dev = *out; else alloc_grid(ctx, gb, n, out);
    if (cfg.propagation_mode == 1) {  // the reference's own visit order, in rounds (heap_order.cu)
        heap_propagate(ctx, pair, cfg, seed, roi, gb.dev, points_computed, s);
        if (mem == TDIC_HOST) copy_grid_back(gb, out, n, s);
        TDIC_CUDA_TRY(cudaStreamSynchronize(s));
        return;
    }
    Buffer d_roi(&ctx->pool, n);
    Buffer claim(&ctx->pool, sizeof(int) * n);
    Buffer keyparams(&ctx->pool, (sizeof(unsigned long long) + propagate_param_bytes(pair->precision)) * n);
    Buffer order(&ctx->pool, sizeof(int) * n);
    Buffer fetch(&ctx->pool, sizeof(int) * (n + 2));
    Buffer misc(&ctx->pool, 64);
    const bool dataflow = cfg.propagation_mode == 2;
    Buffer dstate(&ctx->pool, dataflow ? sizeof(int) * n : 0), dcnt(&ctx->pool, dataflow ? sizeof(int) * n : 0),
        dq(&ctx->pool, dataflow ? sizeof(unsigned long long) * n : 0), kcorr(&ctx->pool, dataflow ? sizeof(float) * n : 0);
    if (dataflow) {
        TDIC_CUDA_TRY(cudaMemsetAsync(dstate.ptr, 0, sizeof(int) * n, s));
        TDIC_CUDA_TRY(cudaMemsetAsync(dcnt.ptr, 0, sizeof(int) * n, s));
        TDIC_CUDA_TRY(cudaMemsetAsync(dq.ptr, 0xff, sizeof(unsigned long long) * n, s));
    }
    TDIC_CUDA_TRY(cudaMemcpyAsync(d_roi.ptr, roi_grid.data(), n, cudaMemcpyHostToDevice, s));
    TDIC_CUDA_TRY(cudaMemsetAsync(claim.ptr, 0, sizeof(int) * n, s));
    TDIC_CUDA_TRY(cudaMemsetAsync(keyparams.ptr, 0xff, sizeof(unsigned long long) * n, s));
    TDIC_CUDA_TRY(cudaMemsetAsync(fetch.ptr, 0, sizeof(int) * (n + 2), s));
    TDIC_CUDA_TRY(cudaMemsetAsync(misc.ptr, 0, 64, s));
    {   // queue word: tail 0, in-flight bias 2^31 (low word)
        const unsigned long long q0 = 0x80000000ull;
        TDIC_CUDA_TRY(cudaMemcpyAsync(misc.as<int>() + 4, &q0, sizeof(q0), cudaMemcpyHostToDevice, s));
    }
    // truncate_roi_subsets: the solves take the masked routes over the pixel ROI
    // (reliability_propagation.cpp:233-238, 341-347)
    Buffer d_roi_px(&ctx->pool, cfg.truncate_roi_subsets ? static_cast<size_t>(w) * h : 0);
    if (cfg.truncate_roi_subsets) {
        if (roi) TDIC_CUDA_TRY(cudaMemcpyAsync(d_roi_px.ptr, roi, static_cast<size_t>(w) * h, cudaMemcpyHostToDevice, s));
        else TDIC_CUDA_TRY(cudaMemsetAsync(d_roi_px.ptr, 1, static_cast<size_t>(w) * h, s));
    }
    PropagateLaunch L{};
    L.gw = gw; L.gh = gh; L.step = step;
    L.roi_grid = d_roi.as<uint8_t>();
    L.roi_px = cfg.truncate_roi_subsets ? d_roi_px.as<uint8_t>() : nullptr;
    L.seed_idx = gys * gw + gxs;
    L.seed_solve = (gxs * step != sxr || gys * step != syr) ? 1 : 0;
    for (int k = 0; k < 6; ++k) L.seed_p[k] = seed.p[k];
    L.seed_corr = seed.correlation;
    L.out = gb.dev;
    L.claim = claim.as<int>();
    L.key = keyparams.as<unsigned long long>();
    L.params = nullptr;
    L.order = order.as<int>();
    int* m = misc.as<int>();
    L.counters = m;                  // [0] wave-list tail, [1] queue head, [4..5] 64-bit queue word
    L.barrier = reinterpret_cast<unsigned int*>(m + 8);
    L.flags = m + 12;                // [0] error [1] no seed [2] accepted
    L.fetch = fetch.as<int>();
    L.mode = cfg.propagation_mode;
    L.sgx = gxs;
    L.sgy = gys;
    L.dstate = dstate.as<int>(); L.dcnt = dcnt.as<int>();
    L.dq = dq.as<unsigned long long>(); L.kcorr = kcorr.as<float>();
    if (!seed_ok) {
        // Output every grid point with defaults; points_computed = 0.
        L.seed_idx = 0;
        L.seed_solve = 0;
    }
    SetupCache cache;
    if (seed_ok && setup_cache_applies(cfg)) setup_cache_prepare(ctx, pair, gw, gh, gxs, gys, cache, L, s);
    if (seed_ok) launch_propagate(ctx, pair, cfg, L, s);
    else launch_init_grid(L.out, gw, gh, step, s);  // every grid point with its defaults
    int flags[3] = {0, 0, 0};
    if (seed_ok) TDIC_CUDA_TRY(cudaMemcpyAsync(flags, L.flags, sizeof(flags), cudaMemcpyDeviceToHost, s));
    if (mem == TDIC_HOST) copy_grid_back(gb, out, n, s);
    check_device_error(ctx, s);
    TDIC_REQUIRE(flags[0] == 0, TDIC_TIMEOUT, "propagation: a bounded in-kernel wait timed out");
    *points_computed = (seed_ok && !flags[1]) ? flags[2] : 0;
}

// ---------------------------------------------------------------------------------------
// Seed candidates (seed_selector.cpp:33-108, 207-317, 388-452), truncate_roi_subsets false.
// ---------------------------------------------------------------------------------------
struct Pt { int x, y; };

template <typename Acc>
double texture_std(const Acc& ref, int w, int h, int r, int x, int y) {
    if (x - r < 0 || y - r < 0 || x + r >= w || y + r >= h) return 0.0;
    double sum = 0.0, sq = 0.0;
    int cnt = 0;
    for (int yy = y - r; yy <= y + r; ++yy)
        for (int xx = x - r; xx <= x + r; ++xx) {
            const double v = ref(static_cast<size_t>(yy) * w + xx);
            sum += v; sq += v * v; ++cnt;
        }
    const double mn = sum / cnt;
    return std::sqrt(std::max(0.0, sq / cnt - mn * mn));
}

// The candidate points of SeedSelector (ROI and the subset margin), in row-major order,
// addressed by rank without materialising them (a 2048^2 image has four million).
class ValidPoints {
public:
    ValidPoints(int w, int h, const uint8_t* roi, int rad, bool margin)
        : w_(w), h_(h), roi_(roi), x0_(margin ? rad : 0), x1_(margin ? w - 1 - rad : w - 1),
          y0_(margin ? rad : 0), y1_(margin ? h - 1 - rad : h - 1), rows_(std::max(0, h)) {
        total_ = 0;
        for (int y = 0; y < h_; ++y) {
            long long c = 0;
            if (y >= y0_ && y <= y1_ && x1_ >= x0_) {
                if (!roi_) {
                    c = x1_ - x0_ + 1;
                } else {
                    const uint8_t* r = roi_ + static_cast<size_t>(y) * w_;
                    for (int x = x0_; x <= x1_; ++x) c += r[x] != 0;
                }
            }
            rows_[y] = c;
            total_ += c;
        }
    }
    long long size() const { return total_; }
    // The points of the given ranks (ascending, repeats allowed).
    std::vector<Pt> select(const std::vector<long long>& ranks) const {
        std::vector<Pt> out;
        out.reserve(ranks.size());
        long long base = 0;
        int y = 0;
        std::vector<int> xs;  // valid x of row y (with a ROI)
        int xs_row = -1;
        for (const long long rk : ranks) {
            while (y < h_ && base + rows_[y] <= rk) base += rows_[y++];
            if (y >= h_) break;
            const long long k = rk - base;
            if (!roi_) {
                out.push_back({x0_ + static_cast<int>(k), y});
            } else {
                if (xs_row != y) {
                    xs.clear();
                    const uint8_t* r = roi_ + static_cast<size_t>(y) * w_;
                    for (int x = x0_; x <= x1_; ++x)
                        if (r[x]) xs.push_back(x);
                    xs_row = y;
                }
                out.push_back({xs[static_cast<size_t>(k)], y});
            }
        }
        return out;
    }
private:
    int w_, h_;
    const uint8_t* roi_;
    int x0_, x1_, y0_, y1_;
    std::vector<long long> rows_;
    long long total_;
};

// SeedSelector's candidate points (seed_selector.cpp:207-317): a deterministic sample of the
// ROI points, k-means centres, and the texture check with its nearest-50 fallback.  The
// nearest-centre assignment of each k-means iteration runs on the device; the centre sums
// are accumulated here in point order, as in run_kmeans.
template <typename Acc>
std::vector<std::pair<int, int>> seed_candidates(tdic_ctx* ctx, const Acc& ref, int w, int h, const uint8_t* roi,
                                                 const tdic_config& c, cudaStream_t s) {
    std::vector<std::pair<int, int>> out;
    const int rad = std::max(std::max(1, c.is_subset_radius), std::max(1, c.sp_subset_radius));
    // is_candidate_margin_valid (seed_selector.cpp:388-422): truncating widens the margin by the
    // search radius and asks for enough ROI pixels in the circle of radius `rad`; the first pool
    // of points is then every ROI point inside that margin (:219-229)
    const bool trunc = c.truncate_roi_subsets != 0;
    const int margin = rad + (trunc ? std::max(0, c.is_search_radius) : 0);
    auto margin_ok = [&](int x, int y) {
        if (x - margin < 0 || y - margin < 0 || x + margin >= w || y + margin >= h) return false;
        if (!trunc) return true;
        int valid = 0, full = 0;
        for (int yy = y - rad; yy <= y + rad; ++yy)
            for (int xx = x - rad; xx <= x + rad; ++xx) {
                if ((xx - x) * (xx - x) + (yy - y) * (yy - y) > rad * rad) continue;
                ++full;
                valid += roi_ok(roi, w, h, xx, yy) ? 1 : 0;
            }
        const int need = std::max(c.min_valid_samples,
                                  static_cast<int>(std::ceil(c.min_valid_sample_ratio * static_cast<double>(full))));
        return valid >= std::max(6, need);
    };
    ValidPoints vp(w, h, roi, margin, true);
    if (vp.size() == 0) vp = ValidPoints(w, h, roi, margin, false);
    const long long npts = vp.size();
    if (npts == 0) return out;
    const int requested = std::max(1, c.seed_count);
    const int limit = std::max(1, c.kmeans_sample_limit);
    std::vector<long long> ranks;
    if (npts <= limit) {
        ranks.resize(static_cast<size_t>(npts));
        std::iota(ranks.begin(), ranks.end(), 0LL);
    } else {
        const double st = static_cast<double>(npts - 1) / static_cast<double>(limit - 1);
        for (int i = 0; i < limit; ++i)
            ranks.push_back(std::min<long long>(std::llround(static_cast<double>(i) * st), npts - 1));
    }
    const std::vector<Pt> sp = vp.select(ranks);
    const int tr = std::max(1, c.is_subset_radius);
    if (requested == 1) {
        double best = -1.0;
        Pt bp{};
        bool found = false;
        for (const auto& p : sp) {
            if (!margin_ok(p.x, p.y)) continue;
            const double t = texture_std(ref, w, h, tr, p.x, p.y);
            if (!found || t > best) { best = t; bp = p; found = true; }
        }
        if (found) out.emplace_back(bp.x, bp.y);
        return out;
    }
    const int count = std::min(requested, static_cast<int>(sp.size()));
    std::vector<double> cx(count), cy(count);
    const double st = count == 1 ? 0.0 : static_cast<double>(sp.size() - 1U) / static_cast<double>(count - 1);
    for (int i = 0; i < count; ++i) {
        const auto idx = static_cast<size_t>(std::llround(static_cast<double>(i) * st));
        const auto& p = sp[std::min(idx, sp.size() - 1U)];
        cx[i] = p.x;
        cy[i] = p.y;
    }
    const int iters = std::max(0, c.kmeans_iterations);
    if (iters > 0) {
        const int m = static_cast<int>(sp.size());
        std::vector<int> px(m), py(m);
        for (int j = 0; j < m; ++j) { px[j] = sp[j].x; py[j] = sp[j].y; }
        KmeansAssigner ka(ctx, px.data(), py.data(), m, count, s);
        if (count <= 2048) {  // per-block sums in shared memory (12 bytes per centre)
            ka.run(cx.data(), cy.data(), iters);
        } else {
            std::vector<int> asg(m);
            std::vector<double> sx(count), sy(count);
            std::vector<int> cnt(count);
            for (int it = 0; it < iters; ++it) {
                ka.assign(cx.data(), cy.data(), asg.data());
                std::fill(sx.begin(), sx.end(), 0.0);
                std::fill(sy.begin(), sy.end(), 0.0);
                std::fill(cnt.begin(), cnt.end(), 0);
                for (int j = 0; j < m; ++j) {
                    sx[asg[j]] += px[j];
                    sy[asg[j]] += py[j];
                    ++cnt[asg[j]];
                }
                for (int i = 0; i < count; ++i)
                    if (cnt[i] > 0) { cx[i] = sx[i] / cnt[i]; cy[i] = sy[i] / cnt[i]; }
            }
        }
    }
    for (int i = 0; i < count; ++i) {
        const int rx = static_cast<int>(std::llround(cx[i])), ry = static_cast<int>(std::llround(cy[i]));
        if (roi_ok(roi, w, h, rx, ry) && margin_ok(rx, ry) && texture_std(ref, w, h, tr, rx, ry) >= c.min_texture_std) {
            out.emplace_back(rx, ry);
            continue;
        }
        std::vector<size_t> ord(sp.size());
        std::iota(ord.begin(), ord.end(), 0U);
        const double ccx = cx[i], ccy = cy[i];
        std::sort(ord.begin(), ord.end(), [&](size_t l, size_t r) {
            const double lx = sp[l].x - ccx, ly = sp[l].y - ccy, qx = sp[r].x - ccx, qy = sp[r].y - ccy;
            return lx * lx + ly * ly < qx * qx + qy * qy;
        });
        const size_t lim = std::min<size_t>(50U, ord.size());
        double best = -1.0;
        Pt bp = sp[ord.front()];
        for (size_t k = 0; k < lim; ++k) {
            const auto& p = sp[ord[k]];
            const double t = texture_std(ref, w, h, tr, p.x, p.y);
            if (t > best) { best = t; bp = p; }
        }
        out.emplace_back(bp.x, bp.y);
    }
    return out;
}

double znssd_from_zncc(double z) {  // integer_search.cpp:25-31
    if (!std::isfinite(z)) return std::numeric_limits<double>::infinity();
    return std::max(0.0, 2.0 * (1.0 - std::max(-1.0, std::min(1.0, z))));
}

// Host view of the raw reference as dic::Image float values.
struct HostImage {
    const void* p;
    tdic_dtype t;
    float operator()(size_t i) const {
        switch (t) {
            case TDIC_U8: return static_cast<const uint8_t*>(p)[i];
            case TDIC_U16: return static_cast<const uint16_t*>(p)[i];
            case TDIC_F32: return static_cast<const float*>(p)[i];
            case TDIC_F64: return static_cast<float>(static_cast<const double*>(p)[i]);
        }
        return 0.0f;
    }
};

void select_seed_impl(tdic_ctx* ctx, tdic_pair* lazy, const HostImage& ref_host, const uint8_t* roi, const tdic_config& c,
                      tdic_seed* seed, cudaStream_t s) {
    std::memset(seed, 0, sizeof(*seed));
    const int w = lazy->w, h = lazy->h;
    const auto cands = seed_candidates(ctx, ref_host, w, h, roi, c, s);
    if (c.sift_enabled) return;  // without OpenCV the SIFT prior finds no match: no seed
    const int n = static_cast<int>(cands.size());
    if (n == 0) return;
    std::vector<int> cx(n), cy(n);
    for (int i = 0; i < n; ++i) { cx[i] = cands[i].first; cy[i] = cands[i].second; }
    // truncate_roi_subsets: masked integer search and masked refinement (subset_initializer.cpp:
    // 140-149, 206-245) over the ROI (every pixel when none is given)
    std::vector<uint8_t> ones;
    const uint8_t* mroi = nullptr;
    if (c.truncate_roi_subsets) {
        if (!roi) ones.assign(static_cast<size_t>(w) * h, 1);
        mroi = roi ? roi : ones.data();
    }
    std::vector<SearchResult> sr(n);
    integer_search_batch(ctx, lazy, c, cx.data(), cy.data(), n, sr.data(), s, mroi);
    // subpixel refinement: ICGN on the non-prefiltered spline (subset_initializer.cpp:152-204)
    std::vector<tdic_poi_in> in;
    std::vector<int> who;
    for (int i = 0; i < n; ++i) {
        if (!sr[i].ok) continue;
        tdic_poi_in q{};
        q.x = cx[i]; q.y = cy[i];
        q.p0[0] = sr[i].u; q.p0[1] = sr[i].v;
        q.confidence = znssd_from_zncc(sr[i].zncc);
        in.push_back(q);
        who.push_back(i);
    }
    std::vector<tdic_poi_out> ref_out(in.size());
    const bool refine = c.sp_enabled != 0;
    if (refine && !in.empty()) {
        tdic_config sc = c;
        sc.subset_radius = std::max(1, c.sp_subset_radius);
        sc.max_iterations = std::max(0, c.sp_max_iterations);
        sc.convergence_threshold = c.sp_convergence_threshold;
        sc.optimizer = 0;
        sc.shape_order = 1;
        Buffer d_in(&ctx->pool, sizeof(tdic_poi_in) * in.size()), d_out(&ctx->pool, sizeof(tdic_poi_out) * in.size()),
            d_fetch(&ctx->pool, sizeof(int));
        TDIC_CUDA_TRY(cudaMemcpyAsync(d_in.ptr, in.data(), sizeof(tdic_poi_in) * in.size(), cudaMemcpyHostToDevice, s));
        SolveLaunch L{d_in.as<tdic_poi_in>(), d_out.as<tdic_poi_out>(), static_cast<int>(in.size()), d_fetch.as<int>()};
        Buffer d_mroi(&ctx->pool, mroi ? static_cast<size_t>(w) * h : 0);
        if (mroi) {
            TDIC_CUDA_TRY(cudaMemcpyAsync(d_mroi.ptr, mroi, static_cast<size_t>(w) * h, cudaMemcpyHostToDevice, s));
            L.roi = d_mroi.as<uint8_t>();
        }
        launch_solve(ctx, lazy, sc, L, s);
        TDIC_CUDA_TRY(cudaMemcpyAsync(ref_out.data(), d_out.ptr, sizeof(tdic_poi_out) * in.size(), cudaMemcpyDeviceToHost, s));
        check_device_error(ctx, s);
    }
    bool found = false;
    double bq = 0.0, bnorm = 0.0;
    for (size_t k = 0; k < in.size(); ++k) {
        double p[6] = {in[k].p0[0], in[k].p0[1], 0, 0, 0, 0};
        double conf = in[k].confidence, quality = conf;
        if (refine && ref_out[k].valid && ref_out[k].status == TDIC_SUCCESS) {
            for (int j = 0; j < 6; ++j) p[j] = ref_out[k].p[j];
            conf = ref_out[k].correlation;
            quality = conf;
        }
        if (!std::isfinite(p[0]) || !std::isfinite(p[1]) || !std::isfinite(conf)) continue;
        const double nrm = std::hypot(p[0], p[1]);
        if (!(quality <= c.seed_max_znssd) || !(nrm >= c.min_displacement_norm)) continue;
        bool better = !found;
        if (found) {  // seed_is_better, seed_selector.cpp:110-133
            if (quality < bq - 1e-9) better = true;
            else if (quality > bq + 1e-9) better = false;
            else better = nrm > bnorm;
        }
        if (better) {
            found = true;
            bq = quality;
            bnorm = nrm;
            seed->x = cx[who[k]];
            seed->y = cy[who[k]];
            for (int j = 0; j < 6; ++j) seed->p[j] = p[j];
            seed->correlation = conf;
            seed->found = 1;
        }
    }
}

}  // namespace

extern "C" {

void tdic_config_default(tdic_config* c) {
    std::memset(c, 0, sizeof(*c));
    c->subset_radius = 15; c->max_iterations = 30; c->convergence_threshold = 1e-3;
    c->optimizer = 0; c->shape_order = 1; c->criterion = 1; c->degree = 5; c->border = 3;
    c->propagation_spacing = 5; c->propagation_max_znssd = 0.5;
    c->is_subset_radius = 10; c->is_search_radius = 30; c->sift_enabled = 0; c->pyramid_enabled = 1;
    c->pyramid_scale = 4; c->pyramid_refinement_radius = 4;
    c->sp_enabled = 1; c->sp_subset_radius = 15; c->sp_max_iterations = 30; c->precision = TDIC_FP32_MIXED;
    c->sp_convergence_threshold = 1e-3;
    c->seed_count = 256; c->kmeans_iterations = 20; c->seed_max_znssd = 0.2;
    c->min_displacement_norm = 0.0; c->min_texture_std = 0.0; c->kmeans_sample_limit = 20000;
    c->propagation_mode = 2;
    c->truncate_roi_subsets = 0; c->min_valid_samples = 12; c->min_valid_sample_ratio = 0.5;
    c->staging = TDIC_STAGING_AUTO; c->pad_ = 0;
}

void tdic_grid_dims(int32_t w, int32_t h, int32_t spacing, int32_t* gw, int32_t* gh) {
    const int64_t step = static_cast<int64_t>(std::max(0, spacing)) + 1;  // 64-bit: no overflow near INT32_MAX
    *gw = static_cast<int32_t>((std::max<int64_t>(0, w) + step - 1) / step);
    *gh = static_cast<int32_t>((std::max<int64_t>(0, h) + step - 1) / step);
}

namespace {
// the message of this thread's last failed tdic_ctx_create or context-free call (there is no
// context to hold it)
thread_local std::string g_create_error;
}  // namespace

tdic_status tdic_ctx_create(int32_t device, tdic_ctx** out) {
    if (!out) return TDIC_INVALID_ARG;
    *out = nullptr;
    auto* ctx = new tdic_ctx();
    ctx->device = device;
    tdic_status st = guarded(ctx, [&] {
        TDIC_CUDA_TRY(cudaSetDevice(device));
        TDIC_CUDA_TRY(cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device));
        TDIC_CUDA_TRY(cudaDeviceGetAttribute(&ctx->max_smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device));
        TDIC_CUDA_TRY(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
        TDIC_CUDA_TRY(cudaMalloc(&ctx->dev_err, sizeof(int)));
        TDIC_CUDA_TRY(cudaMemset(ctx->dev_err, 0, sizeof(int)));
        upload_qk_constants();
    });
    if (st != TDIC_OK) {
        g_create_error = ctx->last_error;
        delete ctx;
        return st;
    }
    *out = ctx;
    return TDIC_OK;
}

namespace {
void ctx_free(tdic_ctx* ctx) {
    cudaSetDevice(ctx->device);
    cudaDeviceSynchronize();
    ctx->tables.clear();
    ctx->pool.trim();
    if (ctx->dev_err) cudaFree(ctx->dev_err);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
}
}  // namespace

void tdic_ctx_destroy(tdic_ctx* ctx) {
    if (!ctx) return;
    {
        std::lock_guard<std::recursive_mutex> lock(ctx->mu);
        if (ctx->live_pairs > 0) {  // freed by the last tdic_pair_destroy
            ctx->destroy_requested = true;
            return;
        }
        ctx_free(ctx);
    }
    delete ctx;
}

const char* tdic_last_error(const tdic_ctx* ctx) {
    if (ctx) return ctx->last_error.c_str();
    return g_create_error.empty() ? "null context" : g_create_error.c_str();
}

size_t tdic_ctx_device_bytes(const tdic_ctx* ctx) { return ctx ? ctx->pool.held_bytes() : 0; }

tdic_status tdic_ctx_heap_stats(const tdic_ctx* ctx, int32_t* rounds, int64_t* solves, double* host_sim_ms) {
    if (!ctx || !rounds || !solves) return TDIC_INVALID_ARG;
    *rounds = ctx->heap_rounds;
    *solves = ctx->heap_solves;
    if (host_sim_ms) *host_sim_ms = ctx->heap_sim_ms;
    return TDIC_OK;
}

tdic_status tdic_pair_create(tdic_ctx* ctx, const void* reference, const void* deformed, int32_t width, int32_t height,
                             int32_t pitch, tdic_dtype dtype, tdic_memory memory, int32_t degree, int32_t border,
                             int32_t exact_prefilter, int32_t precision, void* stream, tdic_pair** out) {
    if (!out) return TDIC_INVALID_ARG;
    *out = nullptr;
    return guarded(ctx, [&] {
        TDIC_REQUIRE(reference && deformed, TDIC_INVALID_ARG, "Cannot precompute B-spline data for an empty image.");
        TDIC_REQUIRE(width > 0 && height > 0, TDIC_INVALID_ARG, "Cannot precompute B-spline data for an empty image.");
        // POI grids are counted and indexed in int32 (a grid point per pixel at spacing 0)
        TDIC_REQUIRE((static_cast<int64_t>(width) + 64) * (static_cast<int64_t>(height) + 64) <= INT32_MAX, TDIC_INVALID_ARG,
                     "image of " + std::to_string(width) + " x " + std::to_string(height) +
                         " pixels exceeds the 2^31-point limit of the POI grid");
        TDIC_REQUIRE(degree == 1 || degree == 3 || degree == 5, TDIC_INVALID_ARG,
                     "Only B-spline degree 1, 3, and 5 are supported; got " + std::to_string(degree) + ".");
        TDIC_REQUIRE(precision == TDIC_FP32_MIXED || precision == TDIC_FP64, TDIC_INVALID_ARG, "unknown precision");
        TDIC_CUDA_TRY(cudaSetDevice(ctx->device));
        auto* p = new tdic_pair();
        p->ctx = ctx;
        p->w = width; p->h = height;
        p->border = std::max(3, border);
        p->degree = degree;
        p->precision = precision;
        p->exact = exact_prefilter ? 1 : 0;
        p->cw = width + 2 * p->border;
        p->ch = height + 2 * p->border;
        p->rpitch = (width + 31) / 32 * 32;
        const int per128 = precision == TDIC_FP64 ? 16 : 32;
        p->cpitch = (p->cw + per128 - 1) / per128 * per128;
        try {
            const size_t es = precision == TDIC_FP64 ? 8 : 4;
            p->ref = Buffer(&ctx->pool, sizeof(float) * static_cast<size_t>(p->rpitch) * height);
            p->def_f = Buffer(&ctx->pool, sizeof(float) * static_cast<size_t>(p->rpitch) * height);
            p->coef = Buffer(&ctx->pool, es * static_cast<size_t>(p->cpitch) * p->ch);
            TDIC_CUDA_TRY(cudaEventCreateWithFlags(&p->last_use, cudaEventDisableTiming));
            pair_compute(p, reference, deformed, pitch, dtype, memory, pick(ctx, stream));
            mark_use(p, pick(ctx, stream));
        } catch (...) {
            delete p;
            throw;
        }
        ctx->live_pairs += 1;
        *out = p;
    });
}

tdic_status tdic_pair_update(tdic_pair* pair, const void* reference, const void* deformed, int32_t pitch,
                             tdic_dtype dtype, tdic_memory memory, void* stream) {
    if (!pair) return TDIC_INVALID_ARG;
    return guarded(pair->ctx, [&] {
        TDIC_REQUIRE(reference && deformed, TDIC_INVALID_ARG, "null image");
        pair_compute(pair, reference, deformed, pitch, dtype, memory, pick(pair->ctx, stream));
        mark_use(pair, pick(pair->ctx, stream));
    });
}

void tdic_pair_destroy(tdic_pair* pair) {
    if (!pair) return;
    tdic_ctx* ctx = pair->ctx;
    bool free_ctx = false;
    {
        std::lock_guard<std::recursive_mutex> lock(ctx->mu);
        cudaSetDevice(ctx->device);
        // work enqueued on any stream may still read the pair's buffers: wait for the last of it
        if (pair->last_use) cudaEventSynchronize(pair->last_use);
        (void)cudaGetLastError();  // nothing to report from a destructor
        delete pair;
        ctx->live_pairs -= 1;
        if (ctx->destroy_requested && ctx->live_pairs == 0) {
            ctx_free(ctx);
            free_ctx = true;
        }
    }
    if (free_ctx) delete ctx;
}

tdic_status tdic_pair_coefficients(tdic_pair* pair, void* host_out, size_t bytes) {
    if (!pair) return TDIC_INVALID_ARG;
    return guarded(pair->ctx, [&] {
        const size_t es = pair->precision == TDIC_FP64 ? 8 : 4;
        const size_t dense = es * static_cast<size_t>(pair->cw) * pair->ch;
        TDIC_REQUIRE(host_out && bytes >= dense, TDIC_INVALID_ARG, "output buffer too small");
        TDIC_CUDA_TRY(cudaDeviceSynchronize());
        TDIC_CUDA_TRY(cudaMemcpy2D(host_out, es * pair->cw, pair->coef.ptr, es * pair->cpitch, es * pair->cw, pair->ch,
                                   cudaMemcpyDeviceToHost));
    });
}

tdic_status tdic_pair_images(tdic_pair* pair, float* reference_out, float* deformed_out) {
    if (!pair) return TDIC_INVALID_ARG;
    return guarded(pair->ctx, [&] {
        TDIC_CUDA_TRY(cudaDeviceSynchronize());
        const size_t row = sizeof(float) * pair->w, dpitch = sizeof(float) * pair->rpitch;
        if (reference_out)
            TDIC_CUDA_TRY(cudaMemcpy2D(reference_out, row, pair->ref.ptr, dpitch, row, pair->h, cudaMemcpyDeviceToHost));
        if (deformed_out)
            TDIC_CUDA_TRY(cudaMemcpy2D(deformed_out, row, pair->def_f.ptr, dpitch, row, pair->h, cudaMemcpyDeviceToHost));
    });
}

tdic_status tdic_reference_gradient(tdic_pair* pair, double* gx, double* gy) {
    if (!pair) return TDIC_INVALID_ARG;
    return guarded(pair->ctx, [&] {
        TDIC_REQUIRE(gx && gy, TDIC_INVALID_ARG, "null output");
        tdic_ctx* ctx = pair->ctx;
        const size_t n = static_cast<size_t>(pair->w) * pair->h;
        Buffer dx(&ctx->pool, 8 * n), dy(&ctx->pool, 8 * n);
        launch_reference_gradient(pair->ref.as<float>(), pair->w, pair->h, pair->rpitch, dx.as<double>(), dy.as<double>(),
                                  ctx->stream);
        TDIC_CUDA_TRY(cudaMemcpyAsync(gx, dx.ptr, 8 * n, cudaMemcpyDeviceToHost, ctx->stream));
        TDIC_CUDA_TRY(cudaMemcpyAsync(gy, dy.ptr, 8 * n, cudaMemcpyDeviceToHost, ctx->stream));
        mark_use(pair, ctx->stream);
        TDIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    });
}

tdic_status tdic_solve_pois(tdic_ctx* ctx, tdic_pair* pair, const tdic_config* cfg, const tdic_poi_in* in, int32_t n,
                            tdic_poi_out* out, tdic_memory memory, void* stream) {
    return guarded(ctx, [&] {
        TDIC_REQUIRE(pair && cfg, TDIC_INVALID_ARG, "null pair or config");
        TDIC_REQUIRE(n >= 0, TDIC_INVALID_ARG, "negative POI count");
        check_config(*cfg);
        check_memory(memory);
        if (n == 0) return;
        TDIC_REQUIRE(in && out, TDIC_INVALID_ARG, "null POI arrays");
        TDIC_CUDA_TRY(cudaSetDevice(ctx->device));
        cudaStream_t s = pick(ctx, stream);
        Buffer fetch(&ctx->pool, sizeof(int));
        if (memory == TDIC_DEVICE) {
            launch_solve(ctx, pair, *cfg, SolveLaunch{in, out, n, fetch.as<int>()}, s);
            mark_use(pair, s);
            check_device_error(ctx, s);  // synchronises: keeps `fetch` alive until the kernel is done
            return;
        }
        Buffer d_in(&ctx->pool, sizeof(tdic_poi_in) * n), d_out(&ctx->pool, sizeof(tdic_poi_out) * n);
        TDIC_CUDA_TRY(cudaMemcpyAsync(d_in.ptr, in, sizeof(tdic_poi_in) * n, cudaMemcpyHostToDevice, s));
        launch_solve(ctx, pair, *cfg, SolveLaunch{d_in.as<tdic_poi_in>(), d_out.as<tdic_poi_out>(), n, fetch.as<int>()}, s);
        mark_use(pair, s);
        TDIC_CUDA_TRY(cudaMemcpyAsync(out, d_out.ptr, sizeof(tdic_poi_out) * n, cudaMemcpyDeviceToHost, s));
        check_device_error(ctx, s);
    });
}

tdic_status tdic_solve_pois_masked(tdic_ctx* ctx, tdic_pair* pair, const tdic_config* cfg, const uint8_t* roi,
                                   const tdic_poi_in* in, int32_t n, tdic_poi_out* out, tdic_memory memory,
                                   void* stream) {
    return guarded(ctx, [&] {
        TDIC_REQUIRE(pair && cfg, TDIC_INVALID_ARG, "null pair or config");
        TDIC_REQUIRE(n >= 0, TDIC_INVALID_ARG, "negative POI count");
        check_config(*cfg);
        check_memory(memory);
        if (n == 0) return;
        TDIC_REQUIRE(in && out, TDIC_INVALID_ARG, "null POI arrays");
        TDIC_CUDA_TRY(cudaSetDevice(ctx->device));
        cudaStream_t s = pick(ctx, stream);
        const size_t px = static_cast<size_t>(pair->w) * pair->h;
        Buffer fetch(&ctx->pool, sizeof(int)), d_roi(&ctx->pool, px);
        if (roi) TDIC_CUDA_TRY(cudaMemcpyAsync(d_roi.ptr, roi, px, cudaMemcpyHostToDevice, s));
        else TDIC_CUDA_TRY(cudaMemsetAsync(d_roi.ptr, 1, px, s));
        SolveLaunch L{in, out, n, fetch.as<int>()};
        L.roi = d_roi.as<uint8_t>();
        if (memory == TDIC_DEVICE) {
            launch_solve(ctx, pair, *cfg, L, s);
            mark_use(pair, s);
            check_device_error(ctx, s);
            return;
        }
        Buffer d_in(&ctx->pool, sizeof(tdic_poi_in) * n), d_out(&ctx->pool, sizeof(tdic_poi_out) * n);
        TDIC_CUDA_TRY(cudaMemcpyAsync(d_in.ptr, in, sizeof(tdic_poi_in) * n, cudaMemcpyHostToDevice, s));
        L.in = d_in.as<tdic_poi_in>();
        L.out = d_out.as<tdic_poi_out>();
        launch_solve(ctx, pair, *cfg, L, s);
        mark_use(pair, s);
        TDIC_CUDA_TRY(cudaMemcpyAsync(out, d_out.ptr, sizeof(tdic_poi_out) * n, cudaMemcpyDeviceToHost, s));
        check_device_error(ctx, s);
    });
}

int32_t tdic_subset_padding(const tdic_config* c) {  // recommended_subset_padding, padding.cpp:28-36
    if (!c || !c->truncate_roi_subsets) return 0;
    const int ir = std::max(1, c->is_subset_radius), sr = std::max(1, c->sp_subset_radius);
    return std::max(0, c->is_search_radius) + std::max(c->subset_radius, std::max(ir, sr)) + std::max(0, c->border);
}

void tdic_subset_grid_dims(int32_t w, int32_t h, const tdic_config* c, int32_t* gw, int32_t* gh) {
    const int pad = tdic_subset_padding(c);
    const int step = std::max(0, c ? c->propagation_spacing : 5) + 1;
    auto count = [&](int n) {  // padded grid points gx * step - pad inside [0, n)
        if (n <= 0) return 0;
        const int lo = (pad + step - 1) / step, hi = (n - 1 + pad) / step;
        return std::max(0, hi - lo + 1);
    };
    *gw = count(w);
    *gh = count(h);
}

tdic_status tdic_propagate(tdic_ctx* ctx, tdic_pair* pair, const tdic_config* cfg, const tdic_seed* seed,
                           const uint8_t* roi, tdic_grid_out* out, tdic_memory memory, int32_t* points_computed,
                           void* stream) {
    return guarded(ctx, [&] {
        TDIC_REQUIRE(pair && cfg && seed && out && points_computed, TDIC_INVALID_ARG, "null argument");
        TDIC_CUDA_TRY(cudaSetDevice(ctx->device));
        propagate_impl(ctx, pair, *cfg, *seed, roi, out, memory, points_computed, pick(ctx, stream));
        mark_use(pair, pick(ctx, stream));
    });
}

tdic_status tdic_select_seed(tdic_ctx* ctx, tdic_pair* lazy, const float* reference_host, const uint8_t* roi,
                             const tdic_config* cfg, tdic_seed* seed, void* stream) {
    return guarded(ctx, [&] {
        TDIC_REQUIRE(lazy && reference_host && cfg && seed, TDIC_INVALID_ARG, "null argument");
        TDIC_CUDA_TRY(cudaSetDevice(ctx->device));
        select_seed_impl(ctx, lazy, HostImage{reference_host, TDIC_F32}, roi, *cfg, seed, pick(ctx, stream));
        mark_use(lazy, pick(ctx, stream));
    });
}

tdic_status tdic_integer_search(tdic_ctx* ctx, tdic_pair* pair, const tdic_config* cfg, const int32_t* x,
                                const int32_t* y, int32_t n, const uint8_t* roi, double* u, double* v, double* zncc,
                                uint8_t* ok, void* stream) {
    return guarded(ctx, [&] {
        TDIC_REQUIRE(pair && cfg && n >= 0, TDIC_INVALID_ARG, "null argument");
        if (n == 0) return;
        TDIC_REQUIRE(x && y && u && v && zncc && ok, TDIC_INVALID_ARG, "null argument");
        check_config(*cfg);
        TDIC_CUDA_TRY(cudaSetDevice(ctx->device));
        // masked subsets search over the ROI (every pixel when none is given), as seed selection
        std::vector<uint8_t> ones;
        const uint8_t* mroi = nullptr;
        if (cfg->truncate_roi_subsets) {
            if (!roi) ones.assign(static_cast<size_t>(pair->w) * pair->h, 1);
            mroi = roi ? roi : ones.data();
        }
        std::vector<SearchResult> sr(n);
        integer_search_batch(ctx, pair, *cfg, x, y, n, sr.data(), pick(ctx, stream), mroi);
        mark_use(pair, pick(ctx, stream));
        for (int i = 0; i < n; ++i) {
            u[i] = sr[i].u;
            v[i] = sr[i].v;
            zncc[i] = sr[i].zncc;
            ok[i] = sr[i].ok ? 1 : 0;
        }
    });
}

// SubsetDIC::compute up to the propagation (subset_dic.cpp:39-64): the pair from the host
// images, the seed on the clamp-padded non-deconvolved spline of the same images
// (seed_selector.cpp:166-173; the seed pair reuses the uploaded images), host texture statistics
// on the raw images.
static void prepare_impl(tdic_ctx* ctx, const void* reference, const void* deformed, int32_t width, int32_t height,
                  tdic_dtype dtype, const uint8_t* roi, const tdic_config& cfg, cudaStream_t s, tdic_pair** pair_out,
                  tdic_seed* seed_out) {
    const int degree = normalized_degree(cfg.degree);
    tdic_pair* pair = nullptr;
    tdic_status st = tdic_pair_create(ctx, reference, deformed, width, height, 0, dtype, TDIC_HOST, degree, cfg.border, 1,
                                      cfg.precision, s, &pair);
    if (st != TDIC_OK) throw Error{st, ctx->last_error};
    try {
        tdic_pair* lazy = nullptr;
        st = tdic_pair_create(ctx, pair->ref.ptr, pair->def_f.ptr, width, height, pair->rpitch, TDIC_F32, TDIC_DEVICE,
                              degree, cfg.border, 0, cfg.precision, s, &lazy);
        if (st != TDIC_OK) throw Error{st, ctx->last_error};
        tdic_seed seed{};
        try {
            select_seed_impl(ctx, lazy, HostImage{reference, dtype}, roi, cfg, &seed, s);
            mark_use(lazy, s);
        } catch (...) {
            tdic_pair_destroy(lazy);
            throw;
        }
        tdic_pair_destroy(lazy);
        *seed_out = seed;
    } catch (...) {
        tdic_pair_destroy(pair);
        throw;
    }
    *pair_out = pair;
}

// The inputs of SubsetDIC::compute with truncate_roi_subsets (subset_dic.cpp:53-65): both
// images mirror-padded and the ROI zero-padded by recommended_subset_padding (padding.cpp:11-24,
// 28-36, 55-85) on every side, the images as float32.
struct PaddedInputs {
    int pad = 0, pw = 0, ph = 0;
    std::vector<float> reference, deformed;
    std::vector<uint8_t> roi;  // ph x pw: 0 in the padding, the caller's ROI (or 1) inside
};

static PaddedInputs pad_inputs(const void* reference, const void* deformed, int w, int h, tdic_dtype dtype,
                               const uint8_t* roi, const tdic_config& cfg) {
    PaddedInputs P;
    P.pad = tdic_subset_padding(&cfg);
    P.pw = w + 2 * P.pad;
    P.ph = h + 2 * P.pad;
    const int pad = P.pad, pw = P.pw, ph = P.ph;
    const HostImage ri{reference, dtype}, di{deformed, dtype};
    auto mirror = [](int i, int n) {
        if (n <= 1) return 0;
        while (i < 0 || i >= n) i = i < 0 ? -i - 1 : 2 * n - i - 1;
        return i;
    };
    P.reference.resize(static_cast<size_t>(pw) * ph);
    P.deformed.resize(P.reference.size());
    P.roi.assign(P.reference.size(), 0);
    std::vector<int> mx(pw);
    for (int x = 0; x < pw; ++x) mx[x] = mirror(x - pad, w);
    for (int y = 0; y < ph; ++y) {
        const size_t row = static_cast<size_t>(mirror(y - pad, h)) * w;
        for (int x = 0; x < pw; ++x) {
            P.reference[static_cast<size_t>(y) * pw + x] = ri(row + mx[x]);
            P.deformed[static_cast<size_t>(y) * pw + x] = di(row + mx[x]);
        }
    }
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x)
            P.roi[static_cast<size_t>(y + pad) * pw + x + pad] = roi ? (roi[static_cast<size_t>(y) * w + x] != 0) : 1;
    return P;
}

// SubsetDIC::compute with truncate_roi_subsets (subset_dic.cpp:53-104): seed and propagation
// over the padded pair, then the grid points inside the original image, shifted back (a padded
// grid point gx * step is the image point gx * step - pad).
static void truncated_compute(tdic_ctx* ctx, const void* reference, const void* deformed, int w, int h,
                              tdic_dtype dtype, const uint8_t* roi, const tdic_config& cfg, tdic_grid_out* out,
                              int32_t* n_points, tdic_seed* seed_out, cudaStream_t s) {
    const PaddedInputs P = pad_inputs(reference, deformed, w, h, dtype, roi, cfg);
    const int pad = P.pad, pw = P.pw, ph = P.ph;
    tdic_pair* pair = nullptr;
    tdic_seed seed{};
    prepare_impl(ctx, P.reference.data(), P.deformed.data(), pw, ph, TDIC_F32, P.roi.data(), cfg, s, &pair, &seed);
    int32_t gw, gh;
    tdic_grid_dims(pw, ph, cfg.propagation_spacing, &gw, &gh);
    const size_t n = static_cast<size_t>(gw) * gh;
    // padded-grid host outputs for the arrays the caller asked for (x, y always: the crop needs them)
    std::vector<double> dbl[16];
    std::vector<uint8_t> u8[2];
    std::vector<int8_t> st;
    std::vector<int32_t> it;
    tdic_grid_out t{};
    double** tdp[16] = {&t.x, &t.y, &t.u, &t.v, &t.du_dx, &t.du_dy, &t.dv_dx, &t.dv_dy, &t.correlation, &t.zncc,
                        &t.d2u_dx2, &t.d2u_dxdy, &t.d2u_dy2, &t.d2v_dx2, &t.d2v_dxdy, &t.d2v_dy2};
    double* const odp[16] = {out->x, out->y, out->u, out->v, out->du_dx, out->du_dy, out->dv_dx, out->dv_dy,
                             out->correlation, out->zncc, out->d2u_dx2, out->d2u_dxdy, out->d2u_dy2, out->d2v_dx2,
                             out->d2v_dxdy, out->d2v_dy2};
    for (int k = 0; k < 16; ++k)
        if (odp[k] || k < 2) { dbl[k].assign(n, 0.0); *tdp[k] = dbl[k].data(); }
    if (out->valid) { u8[0].assign(n, 0); t.valid = u8[0].data(); }
    if (out->converged) { u8[1].assign(n, 0); t.converged = u8[1].data(); }
    if (out->status) { st.assign(n, 0); t.status = st.data(); }
    if (out->iterations) { it.assign(n, 0); t.iterations = it.data(); }
    int32_t computed = 0;
    try {
        if (seed.found) {
            propagate_impl(ctx, pair, cfg, seed, P.roi.data(), &t, TDIC_HOST, &computed, s);
            mark_use(pair, s);
        }
    } catch (...) {
        tdic_pair_destroy(pair);
        throw;
    }
    tdic_pair_destroy(pair);
    if (seed_out) {
        *seed_out = seed;
        if (seed.found) { seed_out->x -= pad; seed_out->y -= pad; }
    }
    if (computed == 0) return;
    int32_t k = 0;
    for (size_t i = 0; i < n; ++i) {
        const double x = t.x[i] - pad, y = t.y[i] - pad;
        if (x < 0.0 || y < 0.0 || x >= w || y >= h) continue;
        for (int f = 0; f < 16; ++f)
            if (odp[f]) odp[f][k] = (*tdp[f])[i];
        out->x[k] = x;
        out->y[k] = y;
        if (out->valid) out->valid[k] = t.valid[i];
        if (out->converged) out->converged[k] = t.converged[i];
        if (out->status) out->status[k] = t.status[i];
        if (out->iterations) out->iterations[k] = t.iterations[i];
        ++k;
    }
    *n_points = k;
}

tdic_status tdic_write_subset_csv(tdic_ctx* ctx, const char* path, const tdic_grid_out* grid, tdic_memory memory,
                                  int32_t n) {
    auto body = [&] {
        TDIC_REQUIRE(grid != nullptr, TDIC_INVALID_ARG, "null argument");
        check_memory(memory);
        if (memory == TDIC_DEVICE) {
            TDIC_REQUIRE(ctx != nullptr, TDIC_INVALID_ARG, "device arrays need a context");
            TDIC_CUDA_TRY(cudaSetDevice(ctx->device));
        }
        write_subset_csv(path, *grid, memory, n);
    };
    if (ctx) return guarded(ctx, body);
    // host arrays without a context: the message goes where tdic_last_error(NULL) reads it
    g_create_error.clear();
    try {
        body();
        return TDIC_OK;
    } catch (const Error& e) {
        g_create_error = e.msg;
        return e.code;
    } catch (const std::exception& e) {
        g_create_error = e.what();
        return TDIC_INVALID_ARG;
    }
}

tdic_status tdic_ls_strain_2d(tdic_ctx* ctx, const double* points, const double* displacement, int32_t n,
                              double radius, int32_t min_samples, int32_t green_lagrange, tdic_ls_strain* out,
                              void* stream) {
    return guarded(ctx, [&] {
        TDIC_REQUIRE(n >= 0, TDIC_INVALID_ARG, "points and displacement must both be Nx2 matrices");
        TDIC_REQUIRE(radius > 0.0 && min_samples >= 3, TDIC_INVALID_ARG,
                     "radius must be positive and min_samples at least 3");
        if (n == 0) return;
        TDIC_REQUIRE(points && displacement && out, TDIC_INVALID_ARG, "null argument");
        TDIC_CUDA_TRY(cudaSetDevice(ctx->device));
        ls_strain_2d(ctx, points, displacement, n, radius, min_samples, green_lagrange ? 1 : 0, out, pick(ctx, stream));
    });
}

tdic_status tdic_subset_prepare(tdic_ctx* ctx, const void* reference, const void* deformed, int32_t width,
                                int32_t height, tdic_dtype dtype, const uint8_t* roi, const tdic_config* cfg,
                                void* stream, tdic_pair** pair_out, tdic_seed* seed_out) {
    return guarded(ctx, [&] {
        TDIC_REQUIRE(cfg && pair_out && seed_out && reference && deformed, TDIC_INVALID_ARG, "null argument");
        TDIC_REQUIRE(width > 0 && height > 0, TDIC_INVALID_ARG, "empty image");
        *pair_out = nullptr;
        std::memset(seed_out, 0, sizeof(*seed_out));
        check_config(*cfg);
        TDIC_CUDA_TRY(cudaSetDevice(ctx->device));
        if (cfg->truncate_roi_subsets) {
            // the padded pair and its seed (padded coordinates), as tdic_subset_compute makes them;
            // the host copies of the padded images are staged before their copies return
            const PaddedInputs P = pad_inputs(reference, deformed, width, height, dtype, roi, *cfg);
            prepare_impl(ctx, P.reference.data(), P.deformed.data(), P.pw, P.ph, TDIC_F32, P.roi.data(), *cfg,
                         pick(ctx, stream), pair_out, seed_out);
            return;
        }
        prepare_impl(ctx, reference, deformed, width, height, dtype, roi, *cfg, pick(ctx, stream), pair_out, seed_out);
    });
}

tdic_status tdic_subset_compute(tdic_ctx* ctx, const void* reference, const void* deformed, int32_t width,
                                int32_t height, tdic_dtype dtype, const uint8_t* roi, const tdic_config* cfg,
                                tdic_grid_out* out, int32_t* n_points, tdic_seed* seed_out, void* stream) {
    return guarded(ctx, [&] {
        TDIC_REQUIRE(cfg && out && n_points, TDIC_INVALID_ARG, "null argument");
        *n_points = 0;
        if (!reference || !deformed || width <= 0 || height <= 0) return;  // SubsetDIC::compute: empty result
        check_config(*cfg);
        TDIC_CUDA_TRY(cudaSetDevice(ctx->device));
        cudaStream_t s = pick(ctx, stream);
        if (cfg->truncate_roi_subsets) {
            TDIC_REQUIRE(out->x && out->y, TDIC_INVALID_ARG, "masked subsets: x and y outputs are required");
            truncated_compute(ctx, reference, deformed, width, height, dtype, roi, *cfg, out, n_points, seed_out, s);
            return;
        }
        tdic_pair* pair = nullptr;
        tdic_seed seed{};
        prepare_impl(ctx, reference, deformed, width, height, dtype, roi, *cfg, s, &pair, &seed);
        if (seed_out) *seed_out = seed;
        int32_t computed = 0;
        try {
            if (seed.found) {
                propagate_impl(ctx, pair, *cfg, seed, roi, out, TDIC_HOST, &computed, s);
                mark_use(pair, s);
            }
        } catch (...) {
            tdic_pair_destroy(pair);
            throw;
        }
        tdic_pair_destroy(pair);
        if (computed == 0) return;
        int32_t gw, gh;
        tdic_grid_dims(width, height, cfg->propagation_spacing, &gw, &gh);
        *n_points = gw * gh;
    });
}

}  // extern "C"

// ---------------------------------------------------------------------------------------
// Propagation without allocation.  Some callers cannot allocate device memory at the time
// they propagate: a real-time loop that must not stall on cudaMalloc's device
// synchronisation, or a host process whose device memory is handed out by another allocator
// that it may not bypass.  tdic_propagate_noalloc runs the same propagation kernel with its
// scratch (work queue, claims, keys, parameters, sample offsets, ROI at the grid points) in
// one file-scope device array instead of the context pool.
// ---------------------------------------------------------------------------------------
namespace {

constexpr int kNoAllocMaxPoints = 131072;   // grid points per call (e.g. a 362 x 362 grid)
constexpr int kNoAllocMaxOffsets = 32768;   // subset samples (a circle of radius 100 has 31417)
constexpr int kNoAllocMaxPixels = 1 << 22;  // image pixels of a masked call (e.g. 2048 x 2048)

struct NoAllocLayout {
    size_t roi, claim, key, order, fetch, misc, dstate, dcnt, dq, kcorr, offsets, roi_px, total;
};

constexpr size_t align256(size_t v) { return (v + 255) / 256 * 256; }

constexpr NoAllocLayout noalloc_layout(size_t n, size_t n_off, size_t px) {
    NoAllocLayout l{};
    size_t o = 0;
    l.roi = o;     o = align256(o + n);
    l.claim = o;   o = align256(o + 4 * n);
    l.key = o;     o = align256(o + (8 + 6 * 8) * n);   // keys then six float64 parameters
    l.order = o;   o = align256(o + 4 * n);
    l.fetch = o;   o = align256(o + 4 * (n + 2));
    l.misc = o;    o = align256(o + 64);
    l.dstate = o;  o = align256(o + 4 * n);
    l.dcnt = o;    o = align256(o + 4 * n);
    l.dq = o;      o = align256(o + 8 * n);
    l.kcorr = o;   o = align256(o + 4 * n);
    l.offsets = o; o = align256(o + 4 * n_off);
    l.roi_px = o;  o = align256(o + px);                 // masked subsets: the pixel ROI
    l.total = o;
    return l;
}

constexpr size_t kNoAllocBytes =
    noalloc_layout(kNoAllocMaxPoints, kNoAllocMaxOffsets, kNoAllocMaxPixels).total;  // about 15.8 MiB

// One instance per device, created when the module is loaded on that device.
static __device__ __align__(256) unsigned char noalloc_scratch[kNoAllocBytes];

constexpr int kNoAllocMaxDevices = 64;
std::mutex noalloc_mu;                                    // held for a whole call
unsigned char* noalloc_ptr[kNoAllocMaxDevices] = {};      // address of the array, per device

// Set-up, once per device, with that device current: the array's device address.
unsigned char* noalloc_scratch_ptr(int device) {
    TDIC_REQUIRE(device >= 0 && device < kNoAllocMaxDevices, TDIC_UNSUPPORTED, "device ordinal out of range");
    if (!noalloc_ptr[device]) {
        unsigned char* ptr = nullptr;
        TDIC_CUDA_TRY(cudaGetSymbolAddress((void**)&ptr, noalloc_scratch));
        noalloc_ptr[device] = ptr;
    }
    return noalloc_ptr[device];
}

// Host-side staging of what the kernel reads from the host (the ROI at the grid points and the
// subset's sample offsets): one static host buffer per field, filled under noalloc_mu and sent
// with one copy each.  A pageable host-to-device copy returns once its source has been staged,
// and every call waits for its stream before it releases the lock, so the next call may refill
// the buffers.
unsigned char noalloc_host_roi[kNoAllocMaxPoints];
short2 noalloc_host_offsets[kNoAllocMaxOffsets];

void propagate_noalloc_impl(tdic_ctx* ctx, tdic_pair* pair, const tdic_config& cfg, const tdic_seed& seed,
                            const uint8_t* roi, const tdic_grid_out* out, int32_t* points_computed, cudaStream_t s) {
    check_config(cfg);
    TDIC_REQUIRE(pair->exact == 1, TDIC_INVALID_ARG, "propagation needs a pair with the exact prefilter");
    TDIC_REQUIRE(cfg.propagation_mode == 0 || cfg.propagation_mode == 2, TDIC_UNSUPPORTED,
                 "no-allocation propagation: propagation_mode 0 (frontier waves) or 2 (dataflow) only (the heap order's "
                 "rounds keep a result table and a tree per call)");
    const int w = pair->w, h = pair->h;
    const int step = std::max(0, cfg.propagation_spacing) + 1;
    int32_t gw, gh;
    tdic_grid_dims(w, h, cfg.propagation_spacing, &gw, &gh);
    const int n = gw * gh;
    const int r = cfg.subset_radius;
    int n_off = 0;
    for (int dy = -r; dy <= r; ++dy)
        for (int dx = -r; dx <= r; ++dx) n_off += dx * dx + dy * dy <= r * r;
    TDIC_REQUIRE(n <= kNoAllocMaxPoints, TDIC_INVALID_ARG,
                 "tdic_propagate_noalloc: the grid has " + std::to_string(n) + " points; its static scratch holds at most " +
                     std::to_string(kNoAllocMaxPoints) + " (use tdic_propagate)");
    TDIC_REQUIRE(n_off <= kNoAllocMaxOffsets, TDIC_INVALID_ARG,
                 "tdic_propagate_noalloc: the subset has more samples than its static scratch holds");
    const bool masked = cfg.truncate_roi_subsets != 0;
    TDIC_REQUIRE(!masked || static_cast<size_t>(w) * h <= static_cast<size_t>(kNoAllocMaxPixels), TDIC_INVALID_ARG,
                 "tdic_propagate_noalloc: masked subsets need the image's pixel ROI; its static scratch holds at most " +
                     std::to_string(kNoAllocMaxPixels) + " pixels (use tdic_propagate)");
    *points_computed = 0;
    const int sxr = static_cast<int>(std::round(seed.x)), syr = static_cast<int>(std::round(seed.y));
    bool seed_ok = seed.found != 0 && roi_ok(roi, w, h, sxr, syr);
    int gxs = 0, gys = 0;
    if (seed_ok) {
        gxs = nearest_grid_index(sxr, step, gw);
        gys = nearest_grid_index(syr, step, gh);
        seed_ok = roi_ok(roi, w, h, gxs * step, gys * step);
    }
    unsigned char* base = noalloc_scratch_ptr(ctx->device);
    constexpr NoAllocLayout lay = noalloc_layout(kNoAllocMaxPoints, kNoAllocMaxOffsets, kNoAllocMaxPixels);
    // The array keeps the previous call's contents: everything the kernel reads before it
    // writes is set here.
    for (int i = 0; i < n; ++i)
        noalloc_host_roi[i] = roi ? (roi[static_cast<size_t>((i / gw) * step) * w + (i % gw) * step] ? 1 : 0) : 1;
    // the row-major order of the context's table, so the sums run in the same order
    int k_off = 0;
    for (int dy = -r; dy <= r; ++dy)
        for (int dx = -r; dx <= r; ++dx)
            if (dx * dx + dy * dy <= r * r)
                noalloc_host_offsets[k_off++] = make_short2(static_cast<short>(dx), static_cast<short>(dy));
    TDIC_CUDA_TRY(cudaMemcpyAsync(base + lay.roi, noalloc_host_roi, n, cudaMemcpyHostToDevice, s));
    TDIC_CUDA_TRY(cudaMemcpyAsync(base + lay.offsets, noalloc_host_offsets, sizeof(short2) * n_off,
                                  cudaMemcpyHostToDevice, s));
    TDIC_CUDA_TRY(cudaMemsetAsync(base + lay.claim, 0, sizeof(int) * n, s));
    TDIC_CUDA_TRY(cudaMemsetAsync(base + lay.key, 0xff, sizeof(unsigned long long) * n, s));
    TDIC_CUDA_TRY(cudaMemsetAsync(base + lay.fetch, 0, sizeof(int) * (n + 2), s));
    TDIC_CUDA_TRY(cudaMemsetAsync(base + lay.misc, 0, 64, s));
    TDIC_CUDA_TRY(cudaMemsetAsync(base + lay.misc + 19, 0x80, 1, s));  // queue word: tail 0, in-flight bias 2^31
    TDIC_CUDA_TRY(cudaMemsetAsync(base + lay.dstate, 0, sizeof(int) * n, s));
    TDIC_CUDA_TRY(cudaMemsetAsync(base + lay.dcnt, 0, sizeof(int) * n, s));
    TDIC_CUDA_TRY(cudaMemsetAsync(base + lay.dq, 0xff, sizeof(unsigned long long) * n, s));
    // truncate_roi_subsets: the masked routes read the pixel ROI, as tdic_propagate's (a pageable
    // source is staged before the copy returns; the call waits for its stream in any case)
    const size_t px = static_cast<size_t>(w) * h;
    if (masked) {
        if (roi) TDIC_CUDA_TRY(cudaMemcpyAsync(base + lay.roi_px, roi, px, cudaMemcpyHostToDevice, s));
        else TDIC_CUDA_TRY(cudaMemsetAsync(base + lay.roi_px, 1, px, s));
    }
    PropagateLaunch L{};
    L.gw = gw; L.gh = gh; L.step = step;
    L.roi_grid = base + lay.roi;
    L.roi_px = masked ? base + lay.roi_px : nullptr;
    L.seed_idx = seed_ok ? gys * gw + gxs : 0;
    L.seed_solve = seed_ok && (gxs * step != sxr || gys * step != syr) ? 1 : 0;
    for (int k = 0; k < 6; ++k) L.seed_p[k] = seed.p[k];
    L.seed_corr = seed.correlation;
    L.out = *out;
    L.claim = reinterpret_cast<int*>(base + lay.claim);
    L.key = reinterpret_cast<unsigned long long*>(base + lay.key);
    L.params = nullptr;
    L.order = reinterpret_cast<int*>(base + lay.order);
    int* m = reinterpret_cast<int*>(base + lay.misc);
    L.counters = m;
    L.barrier = reinterpret_cast<unsigned int*>(m + 8);
    L.flags = m + 12;
    L.fetch = reinterpret_cast<int*>(base + lay.fetch);
    L.mode = cfg.propagation_mode;
    L.sgx = gxs; L.sgy = gys;
    L.dstate = reinterpret_cast<int*>(base + lay.dstate);
    L.dcnt = reinterpret_cast<int*>(base + lay.dcnt);
    L.dq = reinterpret_cast<unsigned long long*>(base + lay.dq);
    L.kcorr = reinterpret_cast<float*>(base + lay.kcorr);
    L.offsets = reinterpret_cast<const short2*>(base + lay.offsets);
    L.n_offsets = n_off;
    if (seed_ok) launch_propagate(ctx, pair, cfg, L, s);
    else launch_init_grid(L.out, gw, gh, step, s);
    int flags[3] = {0, 0, 0};
    if (seed_ok) TDIC_CUDA_TRY(cudaMemcpyAsync(flags, L.flags, sizeof(flags), cudaMemcpyDeviceToHost, s));
    check_device_error(ctx, s);
    TDIC_REQUIRE(flags[0] == 0, TDIC_TIMEOUT, "propagation: a bounded in-kernel wait timed out");
    *points_computed = (seed_ok && !flags[1]) ? flags[2] : 0;
}

}  // namespace

extern "C" {

tdic_status tdic_propagate_noalloc(tdic_ctx* ctx, tdic_pair* pair, const tdic_config* cfg, const tdic_seed* seed,
                                   const uint8_t* roi, const tdic_grid_out* out_device, int32_t* points_computed,
                                   void* stream) {
    return guarded(ctx, [&] {
        TDIC_REQUIRE(pair && cfg && seed && out_device && points_computed, TDIC_INVALID_ARG, "null argument");
        TDIC_CUDA_TRY(cudaSetDevice(ctx->device));
        std::lock_guard<std::mutex> lock(noalloc_mu);
        cudaStream_t s = pick(ctx, stream);
        try {
            propagate_noalloc_impl(ctx, pair, *cfg, *seed, roi, out_device, points_computed, s);
        } catch (...) {
            // copies or memsets into the shared array may still be queued: let them land before
            // the next call may touch the array
            (void)cudaStreamSynchronize(s);
            throw;
        }
        mark_use(pair, s);
    });
}

}  // extern "C"

// ---------------------------------------------------------------------------------------
// Batched propagation: several image pairs (each with its own radius, spacing, threshold, ROI
// and seed) in one persistent launch over a shared work queue.
// ---------------------------------------------------------------------------------------
struct tdic_batch {
    tdic_ctx* ctx = nullptr;
    int n = 0;
    std::vector<tdic_pair*> pairs;
    std::unique_ptr<tdic::BatchPlanBase> plan;
    int config = 0;
    cudaEvent_t last_use = nullptr;  // recorded after the last launch
    ~tdic_batch() {
        if (last_use) cudaEventDestroy(last_use);
    }
};

namespace {

// Every launch of the batch reads its pairs and writes its own buffers.
void batch_mark(tdic_batch* b, cudaStream_t s) {
    if (capturing(s)) return;
    for (tdic_pair* p : b->pairs) mark_use(p, s);
    TDIC_CUDA_TRY(cudaEventRecord(b->last_use, s));
}

void batch_create_impl(tdic_ctx* ctx, int n, tdic_pair* const* pairs, const tdic_config* cfgs, const tdic_seed* seeds,
                       const uint8_t* const* rois, cudaStream_t s, tdic_batch** out) {
    TDIC_REQUIRE(n >= 1 && n <= kMaxBatchJobs, TDIC_INVALID_ARG, "batch: 1 to 512 image pairs");
    const tdic_pair* p0 = pairs[0];
    TDIC_REQUIRE(p0 != nullptr, TDIC_INVALID_ARG, "batch: null pair");
    std::vector<BatchSeed> bs(n);
    std::vector<std::vector<uint8_t>> roi_copy(n);
    for (int j = 0; j < n; ++j) {
        const tdic_pair* p = pairs[j];
        const tdic_config& c = cfgs[j];
        TDIC_REQUIRE(p != nullptr, TDIC_INVALID_ARG, "batch: null pair");
        check_config(c);
        TDIC_REQUIRE(p->ctx == ctx, TDIC_INVALID_ARG, "batch: every pair must belong to the context");
        TDIC_REQUIRE(p->exact == 1, TDIC_INVALID_ARG, "batch: propagation needs pairs with the exact prefilter");
        TDIC_REQUIRE(p->degree == p0->degree && p->precision == p0->precision, TDIC_INVALID_ARG,
                     "batch: every pair must have the same spline degree and precision");
        TDIC_REQUIRE(c.optimizer == cfgs[0].optimizer, TDIC_INVALID_ARG, "batch: every job must use the same optimizer");
        TDIC_REQUIRE(first_order_znssd(c), TDIC_UNSUPPORTED,
                     "batch: only the first-order ZNSSD route (propagate others one pair at a time)");
        TDIC_REQUIRE((c.truncate_roi_subsets != 0) == (cfgs[0].truncate_roi_subsets != 0), TDIC_INVALID_ARG,
                     "batch: every job must use masked subsets, or none");
        TDIC_REQUIRE(c.propagation_mode == 2, TDIC_UNSUPPORTED, "batch: only the dataflow order (propagation_mode 2)");
        // seed alignment (reliability_propagation.cpp:201-216), as tdic_propagate
        const uint8_t* roi = rois ? rois[j] : nullptr;
        const int w = p->w, h = p->h, step = std::max(0, c.propagation_spacing) + 1;
        int32_t gw, gh;
        tdic_grid_dims(w, h, c.propagation_spacing, &gw, &gh);
        const tdic_seed& sd = seeds[j];
        const int sxr = static_cast<int>(std::round(sd.x)), syr = static_cast<int>(std::round(sd.y));
        BatchSeed& b = bs[j];
        b.ok = sd.found != 0 && roi_ok(roi, w, h, sxr, syr);
        if (b.ok) {
            b.gx = nearest_grid_index(sxr, step, gw);
            b.gy = nearest_grid_index(syr, step, gh);
            b.ok = roi_ok(roi, w, h, b.gx * step, b.gy * step);
        }
        if (b.ok) {
            b.idx = b.gy * gw + b.gx;
            b.solve = (b.gx * step != sxr || b.gy * step != syr) ? 1 : 0;
        } else {
            b.idx = -1; b.gx = 0; b.gy = 0; b.solve = 0;
        }
        for (int k = 0; k < 6; ++k) b.p[k] = sd.p[k];
        b.corr = sd.correlation;
        if (roi) roi_copy[j].assign(roi, roi + static_cast<size_t>(w) * h);
    }
    auto b = std::make_unique<tdic_batch>();
    b->ctx = ctx;
    b->n = n;
    b->pairs.assign(pairs, pairs + n);
    TDIC_CUDA_TRY(cudaEventCreateWithFlags(&b->last_use, cudaEventDisableTiming));
    b->plan = batch_build(ctx, n, pairs, cfgs, bs.data(), roi_copy, s);
    ++ctx->live_pairs;  // the batch holds buffers of the context's pool
    *out = b.release();
}

}  // namespace

extern "C" {

tdic_status tdic_batch_create(tdic_ctx* ctx, int32_t n, tdic_pair* const* pairs, const tdic_config* cfgs,
                              const tdic_seed* seeds, const uint8_t* const* rois, void* stream, tdic_batch** out) {
    return guarded(ctx, [&] {
        TDIC_REQUIRE(pairs && cfgs && seeds && out, TDIC_INVALID_ARG, "null argument");
        *out = nullptr;
        TDIC_CUDA_TRY(cudaSetDevice(ctx->device));
        batch_create_impl(ctx, n, pairs, cfgs, seeds, rois, pick(ctx, stream), out);
    });
}

tdic_status tdic_batch_tune(tdic_batch* b, void* stream) {
    if (!b) return TDIC_INVALID_ARG;
    return guarded(b->ctx, [&] {
        TDIC_CUDA_TRY(cudaSetDevice(b->ctx->device));
        cudaStream_t s = pick(b->ctx, stream);
        const int nc = batch_config_count(b->plan.get());
        cudaEvent_t e0, e1;
        TDIC_CUDA_TRY(cudaEventCreate(&e0));
        TDIC_CUDA_TRY(cudaEventCreate(&e1));
        float best = 0.0f;
        int best_c = 0;
        try {
            for (int c = 0; c < nc; ++c) {
                batch_launch(b->plan.get(), c, s);  // warm-up of this configuration
                TDIC_CUDA_TRY(cudaEventRecord(e0, s));
                batch_launch(b->plan.get(), c, s);
                TDIC_CUDA_TRY(cudaEventRecord(e1, s));
                batch_mark(b, s);
                TDIC_CUDA_TRY(cudaEventSynchronize(e1));
                float ms = 0.0f;
                TDIC_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
                if (c == 0 || ms < best) { best = ms; best_c = c; }
            }
        } catch (...) {
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            throw;
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        check_device_error(b->ctx, s);
        b->config = best_c;
    });
}

tdic_status tdic_batch_launch(tdic_batch* b, void* stream) {
    if (!b) return TDIC_INVALID_ARG;
    return guarded(b->ctx, [&] {
        cudaStream_t s = pick(b->ctx, stream);
        batch_launch(b->plan.get(), b->config, s);
        batch_mark(b, s);
    });
}

tdic_status tdic_batch_finish(tdic_batch* b, void* stream, int32_t* points_computed) {
    if (!b) return TDIC_INVALID_ARG;
    return guarded(b->ctx, [&] {
        TDIC_REQUIRE(points_computed, TDIC_INVALID_ARG, "null argument");
        cudaStream_t s = pick(b->ctx, stream);
        int err = 0;
        batch_finish(b->plan.get(), points_computed, &err, s);
        check_device_error(b->ctx, s);
        TDIC_REQUIRE(err == 0, TDIC_TIMEOUT, "batch propagation: a bounded in-kernel wait timed out");
    });
}

tdic_status tdic_batch_outputs(tdic_batch* b, int32_t job, tdic_grid_out* device_arrays) {
    if (!b) return TDIC_INVALID_ARG;
    return guarded(b->ctx, [&] {
        TDIC_REQUIRE(device_arrays && job >= 0 && job < b->n, TDIC_INVALID_ARG, "batch: job out of range");
        *device_arrays = batch_outputs(b->plan.get(), job);
    });
}

tdic_status tdic_batch_results(tdic_batch* b, int32_t job, const tdic_grid_out* host_arrays, void* stream) {
    if (!b) return TDIC_INVALID_ARG;
    return guarded(b->ctx, [&] {
        TDIC_REQUIRE(host_arrays && job >= 0 && job < b->n, TDIC_INVALID_ARG, "batch: job out of range");
        cudaStream_t s = pick(b->ctx, stream);
        GridBuffers g;
        g.dev = batch_outputs(b->plan.get(), job);
        int32_t gw = 0, gh = 0;
        batch_grid(b->plan.get(), job, &gw, &gh);
        copy_grid_back(g, host_arrays, gw * gh, s);
        TDIC_CUDA_TRY(cudaStreamSynchronize(s));
    });
}

tdic_status tdic_batch_set_sms(tdic_batch* b, int32_t sms) {
    if (!b) return TDIC_INVALID_ARG;
    return guarded(b->ctx, [&] { batch_set_sms(b->plan.get(), sms); });
}

tdic_status tdic_batch_config(tdic_batch* b, int32_t* warps_per_poi, int32_t* groups_per_block, int32_t* staging) {
    if (!b) return TDIC_INVALID_ARG;
    return guarded(b->ctx, [&] {
        TDIC_REQUIRE(warps_per_poi && groups_per_block, TDIC_INVALID_ARG, "null argument");
        int g = 0, k = 0, st = 0;
        batch_config_info(b->plan.get(), b->config, &g, &k, &st);
        *warps_per_poi = g;
        *groups_per_block = k;
        if (staging) *staging = st;
    });
}

void tdic_batch_destroy(tdic_batch* b) {
    if (!b) return;
    tdic_ctx* ctx = b->ctx;
    bool free_ctx = false;
    {
        std::lock_guard<std::recursive_mutex> lock(ctx->mu);
        cudaSetDevice(ctx->device);
        if (b->last_use) cudaEventSynchronize(b->last_use);  // the last launch may still run
        (void)cudaGetLastError();  // nothing to report from a destructor
        delete b;
        ctx->live_pairs -= 1;
        if (ctx->destroy_requested && ctx->live_pairs == 0) {
            ctx_free(ctx);
            free_ctx = true;
        }
    }
    if (free_ctx) delete ctx;
}

}  // extern "C"
