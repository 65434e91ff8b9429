// K1: B-spline coefficient prefilter, K2: reference-image gradients, image conversion.
//
// K1 computes BSplineImagePreprocessor::form_coefficients (bspline.cpp:369-392): the image is
// padded by `border` pixels with half-sample symmetry (symmetric_index, bspline.cpp:78-89) and
// every row, then every column, of the (H+2B) x (W+2B) padded image is deconvolved by the
// sampled B-spline kernel with PERIODIC boundary over the padded length (the reference does it
// with an FFT, bspline.cpp:191-244).  Here the exact periodic inverse is a cascade of first-order
// recursive filters (the poles z of the sampled kernel, gain prod (1 - z)^2 per dimension), run
// block-parallel in the manner of Nehab, Maximo, Lima and Hoppe ("GPU-efficient recursive
// filtering and summed-area tables", SIGGRAPH Asia 2011): the line is cut into short segments,
// each filtered from a zero state, and the state each segment should have started from is a
// carry from the preceding segments, added back as carry * z^(i+1).
//
// prefilter_fused_kernel: one CTA per output tile of TH rows x TW columns of coefficients, with a
// margin of M samples on every side (indices taken modulo the padded size, which is what
// periodicity means; a margin of M leaves a truncation error of order |z|^M, below the rounding
// error of the type).  Column sweep: thread c owns padded column c of the tile, reads its
// TH + 2M raw samples straight from the source image (coalesced across the warp), runs the
// causal recursion downwards and the anti-causal one upwards, and leaves the TH central rows in
// shared memory.  Row pass: a warp owns one row of 32 x 8 samples, each lane 8 consecutive
// samples in registers; lanes filter their segment from a zero state and take the carry of the
// K = M / 8 lanes before (causal) or after (anti-causal) them by shuffles.  The same launch writes
// the float32 copies of the reference and deformed images that the rest of the pair needs, for
// the pixels of its tile, so the whole pair set-up reads each raw image once:
//   bytes = 2 W H sizeof(In) + 2 W H 4 + (W+2B)(H+2B) sizeof(T).
#include "tdic_internal.cuh"

#include <type_traits>

namespace tdic {

namespace {

__host__ __device__ inline int sym_index(int v, int size) {
    const int period = 2 * size;
    int w = v % period;
    if (w < 0) w += period;
    return w < size ? w : period - 1 - w;
}
__host__ __device__ inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }
__host__ __device__ inline int wrap(int v, int n) { int r = v % n; return r < 0 ? r + n : r; }

template <typename In> __device__ inline float load_px(const In* p) { return static_cast<float>(__ldg(p)); }

// An integer pixel as float: OR-ing it into the mantissa of 2^23 and subtracting 2^23 is exact
// below 2^23 and takes two full-rate instructions instead of a conversion.
__device__ __forceinline__ float px_float(uint32_t v) { return __int_as_float(0x4B000000 | v) - 8388608.0f; }
template <typename In> __device__ __forceinline__ float px_float(In v) {
    if constexpr (sizeof(In) <= 2) return px_float(static_cast<uint32_t>(v));
    else return static_cast<float>(v);
}

// Poles of the sampled cubic / quintic B-spline kernels (same closed forms as the oracle).
struct Poles {
    double z[2];
    int n;
    double gain;
};
Poles poles_for(int degree) {
    Poles p{};
    if (degree == 3) {
        p.n = 1;
        p.z[0] = std::sqrt(3.0) - 2.0;
    } else if (degree == 5) {
        p.n = 2;
        const double s = std::sqrt(105.0), w1 = -13.0 + s, w2 = -13.0 - s;
        p.z[0] = 0.5 * (w1 + std::sqrt(w1 * w1 - 4.0));
        p.z[1] = 0.5 * (w2 + std::sqrt(w2 * w2 - 4.0));
    }
    p.gain = 1.0;  // per 1-D pass; the 2-D tile applies it once per dimension
    for (int k = 0; k < p.n; ++k) p.gain *= (1.0 - p.z[k]) * (1.0 - p.z[k]);
    return p;
}

// Tile geometry per coefficient type and degree: margin M (a multiple of the 8 samples a lane
// owns, with |z_max|^M below the unit roundoff of T) and TH output rows per tile.
template <typename T, int DEG> struct PfGeom;
template <> struct PfGeom<float, 3> { static constexpr int M = 16, TH = 32; };
template <> struct PfGeom<float, 5> { static constexpr int M = 32, TH = 32; };
template <> struct PfGeom<double, 3> { static constexpr int M = 32, TH = 16; };
template <> struct PfGeom<double, 5> { static constexpr int M = 56, TH = 16; };
constexpr int kSR = 8;          // samples per lane in the row pass
constexpr int kRS = 32 * kSR;   // tile columns with margins (= threads per CTA, one per column)

// Integer pixels (u8, u16) of tiles away from the image edges are staged into shared memory by
// 16-byte asynchronous copies of whole tile rows, so every byte a CTA needs is in flight at once;
// float inputs and edge tiles (reflection, periodic wrap) are read per element.
template <typename In> struct PfStage {
    static constexpr bool on = sizeof(In) <= 2;
    static constexpr int es = static_cast<int>(sizeof(In));
    static constexpr int NCH = on ? (kRS * es + 30) / 16 : 0;  // 16-byte chunks per staged row
};

template <typename T, int DEG> struct PfTile {
    static constexpr int M = PfGeom<T, DEG>::M, TH = PfGeom<T, DEG>::TH;
    static constexpr int TW = kRS - 2 * M;           // output columns per tile
    static constexpr int NR = TH + 2 * M;            // rows the column sweep reads
    static constexpr int K = (M + kSR - 1) / kSR;    // lanes a row carry spans
    static constexpr int E = 16 / static_cast<int>(sizeof(T));  // elements per 16-byte chunk
    static constexpr int CL = kSR / E;               // chunks per lane
    // bytes: coefficient rows, row offsets and staging shifts, staged deformed and reference rows
    template <typename In>
    static constexpr size_t smem() {
        return static_cast<size_t>(TH + M) * kRS * sizeof(T) + (2 * NR + TH) * sizeof(int) +
               static_cast<size_t>(NR + TH) * PfStage<In>::NCH * 16;
    }
};

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Shared-memory position of tile column c: 16-byte chunks XOR-swizzled so that the row pass's
// vector loads (lane l reads chunks CL*l .. CL*l + CL-1) hit distinct banks.
template <typename T, int DEG>
__device__ __forceinline__ int pf_phys(int c) {
    using P = PfTile<T, DEG>;
    const int k = c / P::E;
    return (k ^ ((k >> 3) & (P::CL - 1))) * P::E + (c % P::E);
}

// One pole over the 32 x kSR samples of a warp row held as a[] (lane l: samples 8l .. 8l+7).
template <typename T, int K>
__device__ __forceinline__ void row_pole(T (&a)[kSR], T z, int lane) {
    T zp[kSR + 1];
    zp[0] = T(1);
#pragma unroll
    for (int i = 1; i <= kSR; ++i) zp[i] = zp[i - 1] * z;
#pragma unroll
    for (int i = 1; i < kSR; ++i) a[i] = a[i] + z * a[i - 1];  // causal, zero state
    T carry = T(0), m = T(1);
#pragma unroll
    for (int k = 1; k <= K; ++k) {  // true state at the end of the previous segment
        const T e = __shfl_up_sync(0xffffffffu, a[kSR - 1], k);
        if (lane >= k) carry += m * e;
        m *= zp[kSR];
    }
#pragma unroll
    for (int i = 0; i < kSR; ++i) a[i] += zp[i + 1] * carry;
#pragma unroll
    for (int i = kSR - 2; i >= 0; --i) a[i] = a[i] + z * a[i + 1];  // anti-causal, zero state
    carry = T(0);
    m = T(1);
#pragma unroll
    for (int k = 1; k <= K; ++k) {  // true state at the start of the next segment
        const T f = __shfl_down_sync(0xffffffffu, a[0], k);
        if (lane + k < 32) carry += m * f;
        m *= zp[kSR];
    }
#pragma unroll
    for (int i = 0; i < kSR; ++i) a[i] += zp[kSR - i] * carry;
}

template <typename T> struct Vec16;
template <> struct Vec16<float> { using type = float4; };
template <> struct Vec16<double> { using type = double2; };

template <typename In, typename T, int DEG>
__global__ void __launch_bounds__(kRS) prefilter_fused_kernel(
    const In* __restrict__ def, const In* __restrict__ ref, int pitch, int w, int h, int border, int cw, int ch,
    int opitch, T z0, T z1, T g2, T* __restrict__ coef, float* __restrict__ def_f, float* __restrict__ ref_f,
    int fpitch) {
    using P = PfTile<T, DEG>;
    constexpr int M = P::M, TH = P::TH, TW = P::TW, NR = P::NR;
    using V = typename Vec16<T>::type;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    using ST = PfStage<In>;
    constexpr int NCH = ST::NCH, es = ST::es;
    T* buf = reinterpret_cast<T*>(smem_raw);  // (TH + M) rows x kRS: rows M .. NR-1 of the tile
    int* srow = reinterpret_cast<int*>(buf + (TH + M) * kRS);  // row offsets (elements)
    int* dsh = srow + NR;                                      // byte offset of each staged row's first
    int* rsh = dsh + NR;                                       // pixel: deformed; reference (central rows)
    unsigned char* sdef = reinterpret_cast<unsigned char*>(rsh + TH);  // NR staged rows of NCH chunks
    unsigned char* sref = sdef + NR * NCH * 16;                         // TH staged rows
    const int x0 = blockIdx.x * TW, y0 = blockIdx.y * TH;
    const int c = threadIdx.x;
    // tile column c is image column xs + c when the tile is clear of the image edges
    const int xs = x0 - M - border;
    const bool staged = ST::on && xs * es >= 16 && (w - xs - kRS) * es >= 32;
    for (int r = c; r < NR; r += kRS) {
        srow[r] = sym_index(wrap(y0 - M + r, ch) - border, h) * pitch;
        if (staged) {
            dsh[r] = r * NCH * 16 + static_cast<int>(reinterpret_cast<uintptr_t>(def + srow[r] + xs) & 15);
            if (r >= M && r < M + TH)
                rsh[r - M] = (r - M) * NCH * 16 + static_cast<int>(reinterpret_cast<uintptr_t>(ref + srow[r] + xs) & 15);
        }
    }
    const int pxc = x0 - M + c;  // padded column (unwrapped)
    const int sx = sym_index(wrap(pxc, cw) - border, w);
    const int pc = pf_phys<T, DEG>(c);
    const int ix = pxc - border;
    const bool own = c >= M && c < M + TW && pxc < cw && ix >= 0 && ix < w;  // an image column of this tile
    __syncthreads();
    if (ST::on && staged) {
        // the 16-byte chunks covering bytes [xs*es - shift, xs*es + kRS*es + 30) of each row: inside
        // the row by the edge margins required above
        constexpr int NCHD = NCH > 0 ? NCH : 1;  // (integer pixels only)
        for (int q = c; q < NR * NCH; q += kRS) {
            const int r = q / NCHD, k = q - r * NCHD;
            cp_async16(sdef + q * 16,
                       reinterpret_cast<const unsigned char*>(def + srow[r] + xs) - (dsh[r] - r * NCH * 16) + 16 * k);
        }
        for (int q = c; q < TH * NCH; q += kRS) {
            const int r = q / NCHD, k = q - r * NCHD;
            cp_async16(sref + q * 16,
                       reinterpret_cast<const unsigned char*>(ref + srow[M + r] + xs) - (rsh[r] - r * NCH * 16) + 16 * k);
        }
        cp_async_wait_all();
        __syncthreads();
    }

    // Column sweep, causal (downwards) from a zero state at the top margin, 16 rows per batch:
    // every load of a batch (deformed rows, and the reference pixels this thread converts) is
    // issued before the first use, so a warp waits for memory once per batch, not once per row.
    // Three forms of straight-line code, one branch per CTA: staged rows with one common
    // alignment shift (the row pitch a multiple of 16 bytes); staged rows with per-row shifts;
    // per-element loads, which also write the float32 copies of the owned pixels (staged tiles
    // write theirs at the end, with 16-byte stores).
    // The gain g2 is applied once, when the row pass stores the coefficients.
    const int iy0 = y0 - M - border;  // image row of tile row r: iy0 + r (central rows are not wrapped)
    const bool uni = (static_cast<long long>(pitch) * es) % 16 == 0;
    const int sd0 = staged ? static_cast<int>(reinterpret_cast<uintptr_t>(def + xs) & 15) : 0;  // the common shift
    const unsigned char* dcol = sdef + sd0 + c * es;  // this thread's column in the staged rows
    float* dfo = def_f + ix;
    float* rfo = ref_f + ix;
    T yc0 = T(0), yc1 = T(0);
    // form: 1 staged, common shift; 2 staged, per-row shifts; 3 per element
    auto sweep = [&](auto form_tag) {
        constexpr int F = decltype(form_tag)::value;
#pragma unroll
        for (int r0 = 0; r0 < NR; r0 += 16) {
            float v[16], rv[16];
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                const int r = r0 + i;
                if constexpr (F <= 1) v[i] = px_float(*reinterpret_cast<const In*>(dcol + r * NCH * 16));
                else if constexpr (F == 2) v[i] = px_float(*reinterpret_cast<const In*>(sdef + dsh[r] + c * es));
                else v[i] = px_float(__ldg(def + srow[r] + sx));
                rv[i] = 0.0f;
                if constexpr (F == 3) {
                    if (r >= M && r < M + TH && own && static_cast<unsigned>(iy0 + r) < static_cast<unsigned>(h))
                        rv[i] = px_float(__ldg(ref + srow[r] + sx));
                }
            }
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                const int r = r0 + i;
                yc0 = static_cast<T>(v[i]) + z0 * yc0;
                T o = yc0;
                if (DEG == 5) {
                    yc1 = yc0 + z1 * yc1;
                    o = yc1;
                }
                if (r >= M) buf[(r - M) * kRS + pc] = o;
                if (F == 3 && r >= M && r < M + TH && own && static_cast<unsigned>(iy0 + r) < static_cast<unsigned>(h)) {
                    const int at = (iy0 + r) * fpitch;
                    dfo[at] = v[i];
                    rfo[at] = rv[i];
                }
            }
        }
    };
    if (ST::on && staged && uni) sweep(std::integral_constant<int, 1>{});
    else if (ST::on && staged) sweep(std::integral_constant<int, 2>{});
    else sweep(std::integral_constant<int, 3>{});
    // Anti-causal (upwards) from a zero state at the bottom margin; the TH central rows stay.
    T ya0 = T(0), ya1 = T(0);
#pragma unroll
    for (int r = NR - 1; r >= M; --r) {
        T o = buf[(r - M) * kRS + pc];
        ya0 = o + z0 * ya0;
        o = ya0;
        if (DEG == 5) {
            ya1 = ya0 + z1 * ya1;
            o = ya1;
        }
        if (r < M + TH) buf[(r - M) * kRS + pc] = o;
    }
    __syncthreads();

    // Row pass: warp per tile row, lane l holds samples 8l .. 8l+7 of the kRS columns.
    const int warp = c >> 5, lane = c & 31;
    const bool out_lane = lane * kSR >= M && lane * kSR + kSR <= M + TW;
    for (int rr = warp; rr < TH; rr += kRS / 32) {
        const int oy = y0 + rr;
        if (oy >= ch) break;
        T a[kSR];
#pragma unroll
        for (int j = 0; j < P::CL; ++j) {
            const int k = P::CL * lane + j;
            const int pk = k ^ ((k >> 3) & (P::CL - 1));
            const V q = *reinterpret_cast<const V*>(buf + rr * kRS + pk * P::E);
            const T* qs = reinterpret_cast<const T*>(&q);
#pragma unroll
            for (int e = 0; e < P::E; ++e) a[j * P::E + e] = qs[e];
        }
        row_pole<T, P::K>(a, z0, lane);
        if (DEG == 5) row_pole<T, P::K>(a, z1, lane);
#pragma unroll
        for (int i = 0; i < kSR; ++i) a[i] *= g2;
        const int cx = x0 - M + lane * kSR;  // padded column of a[0]
        if (out_lane) {
            T* dst = coef + static_cast<size_t>(oy) * opitch + cx;
            if (cx + kSR <= cw) {
#pragma unroll
                for (int j = 0; j < P::CL; ++j) {
                    V q;
                    T* qs = reinterpret_cast<T*>(&q);
#pragma unroll
                    for (int e = 0; e < P::E; ++e) qs[e] = a[j * P::E + e];
                    *reinterpret_cast<V*>(dst + j * P::E) = q;
                }
            } else {
#pragma unroll
                for (int i = 0; i < kSR; ++i)
                    if (cx + i < cw) dst[i] = a[i];
            }
        }
    }
    // Float32 copies of the owned pixels of a staged tile from its staged rows: 4 columns per
    // lane and 16-byte stores over the aligned column groups that cover the owned columns (a
    // group shared with the next tile is written by both, with the same values).
    if constexpr (ST::on) {
        if (staged) {
            const int g0 = (x0 - border) & ~3, ng = (((x0 - border + TW) + 3 & ~3) - g0) >> 2;
            for (int q = warp; q < 2 * TH; q += kRS / 32) {
                const int rr = q >> 1;
                const int iy = y0 - border + rr;
                if (static_cast<unsigned>(iy) >= static_cast<unsigned>(h)) continue;
                const unsigned char* srow_b = (q & 1) ? sref + rsh[rr] : sdef + dsh[M + rr];
                float* drow = ((q & 1) ? ref_f : def_f) + static_cast<size_t>(iy) * fpitch;
                for (int gq = lane; gq < ng; gq += 32) {
                    const int col = g0 + 4 * gq;
                    const unsigned char* sp = srow_b + (col - xs) * es;
                    float4 f;
                    f.x = px_float(*reinterpret_cast<const In*>(sp));
                    f.y = px_float(*reinterpret_cast<const In*>(sp + es));
                    f.z = px_float(*reinterpret_cast<const In*>(sp + 2 * es));
                    f.w = px_float(*reinterpret_cast<const In*>(sp + 3 * es));
                    *reinterpret_cast<float4*>(drow + col) = f;
                }
            }
        }
    }
}

// Degree 1 (the deconvolution kernel is the identity) and the non-exact "lazy" coefficients
// (clamp padding, no deconvolution: form_coefficients with use_exact_prefilter = false).
template <typename In, typename T>
__global__ void pad_copy_kernel(const In* __restrict__ img, int w, int h, int pitch, int border, int cw, int ch,
                                int opitch, int symmetric, T* __restrict__ out) {
    const size_t n = static_cast<size_t>(cw) * ch;
    for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<size_t>(gridDim.x) * blockDim.x) {
        const int py = static_cast<int>(i / cw), px = static_cast<int>(i - static_cast<size_t>(py) * cw);
        const int sy = symmetric ? sym_index(py - border, h) : clampi(py - border, 0, h - 1);
        const int sx = symmetric ? sym_index(px - border, w) : clampi(px - border, 0, w - 1);
        out[static_cast<size_t>(py) * opitch + px] = static_cast<T>(load_px(img + static_cast<size_t>(sy) * pitch + sx));
    }
}

template <typename In>
__global__ void convert_kernel(const In* __restrict__ src, int w, int h, int pitch, float* __restrict__ dst,
                               int dpitch) {
    const size_t n = static_cast<size_t>(w) * h;
    for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<size_t>(gridDim.x) * blockDim.x) {
        const int y = static_cast<int>(i / w), x = static_cast<int>(i - static_cast<size_t>(y) * w);
        dst[static_cast<size_t>(y) * dpitch + x] = static_cast<float>(src[static_cast<size_t>(y) * pitch + x]);
    }
}

// K2 (reliability_propagation.cpp:84-112): central differences on raw pixels, one-sided (/1)
// at the border.
__global__ void gradient_kernel(const float* __restrict__ img, int w, int h, int pitch, double* __restrict__ gx,
                                double* __restrict__ gy) {
    const size_t n = static_cast<size_t>(w) * h;
    for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<size_t>(gridDim.x) * blockDim.x) {
        const int y = static_cast<int>(i / w), x = static_cast<int>(i - static_cast<size_t>(y) * w);
        const int xm = max(0, x - 1), xp = min(w - 1, x + 1), ym = max(0, y - 1), yp = min(h - 1, y + 1);
        gx[i] = (static_cast<double>(img[static_cast<size_t>(y) * pitch + xp]) - static_cast<double>(img[static_cast<size_t>(y) * pitch + xm])) /
                static_cast<double>(max(1, xp - xm));
        gy[i] = (static_cast<double>(img[static_cast<size_t>(yp) * pitch + x]) - static_cast<double>(img[static_cast<size_t>(ym) * pitch + x])) /
                static_cast<double>(max(1, yp - ym));
    }
}

int grid_for(size_t n, int threads) {
    const size_t b = (n + threads - 1) / threads;
    return static_cast<int>(b < 1 ? 1 : (b > 65535 * 8 ? 65535 * 8 : b));
}

template <typename In, typename T, int DEG>
void launch_fused(const tdic_pair* p, const In* ref, const In* def, int pitch, const Poles& pl, T* coef,
                  cudaStream_t s) {
    using P = PfTile<T, DEG>;
    TDIC_REQUIRE(static_cast<long long>(pitch) * p->h < (1LL << 31) &&
                     static_cast<long long>(p->rpitch) * p->h < (1LL << 31),
                 TDIC_UNSUPPORTED, "image larger than 2^31 elements");
    const dim3 grid((p->cw + P::TW - 1) / P::TW, (p->ch + P::TH - 1) / P::TH);
    constexpr size_t smem = P::template smem<In>();
    TDIC_CUDA_TRY(cudaFuncSetAttribute(prefilter_fused_kernel<In, T, DEG>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(smem)));
    prefilter_fused_kernel<In, T, DEG><<<grid, kRS, smem, s>>>(
        def, ref, pitch, p->w, p->h, p->border, p->cw, p->ch, p->cpitch, T(pl.z[0]), T(pl.n > 1 ? pl.z[1] : 0.0),
        T(pl.gain * pl.gain), coef, p->def_f.as<float>(), p->ref.as<float>(), p->rpitch);  // one gain per 1-D pass
    TDIC_CUDA_TRY(cudaGetLastError());
}

template <typename In, typename T>
void pair_setup_typed(const tdic_pair* p, const In* ref, const In* def, int pitch, T* coef, cudaStream_t s) {
    const Poles pl = poles_for(p->degree);
    if (p->degree == 3) launch_fused<In, T, 3>(p, ref, def, pitch, pl, coef, s);
    else launch_fused<In, T, 5>(p, ref, def, pitch, pl, coef, s);
}

template <typename In>
void pair_setup_in(const tdic_pair* p, const void* ref, const void* def, int pitch, cudaStream_t s) {
    const In* r = static_cast<const In*>(ref);
    const In* d = static_cast<const In*>(def);
    if (p->precision == TDIC_FP64) pair_setup_typed<In, double>(p, r, d, pitch, p->coef.as<double>(), s);
    else pair_setup_typed<In, float>(p, r, d, pitch, p->coef.as<float>(), s);
}

}  // namespace

void launch_convert(const void* src, int w, int h, int pitch, tdic_dtype dtype, float* dst, int dst_pitch,
                    cudaStream_t s) {
    const int g = grid_for(static_cast<size_t>(w) * h, 256);
    switch (dtype) {
        case TDIC_U8: convert_kernel<uint8_t><<<g, 256, 0, s>>>(static_cast<const uint8_t*>(src), w, h, pitch, dst, dst_pitch); break;
        case TDIC_U16: convert_kernel<uint16_t><<<g, 256, 0, s>>>(static_cast<const uint16_t*>(src), w, h, pitch, dst, dst_pitch); break;
        case TDIC_F32: convert_kernel<float><<<g, 256, 0, s>>>(static_cast<const float*>(src), w, h, pitch, dst, dst_pitch); break;
        case TDIC_F64: convert_kernel<double><<<g, 256, 0, s>>>(static_cast<const double*>(src), w, h, pitch, dst, dst_pitch); break;
    }
    TDIC_CUDA_TRY(cudaGetLastError());
}

// Coefficients of the non-exact ("lazy") and degree-1 pairs: a padded copy of the float32 deformed
// image (dic::Image holds float, and a float64 numpy input is rounded to float by the reference
// binding, bind_subset.cpp:50-64).
void launch_prefilter(tdic_pair* pair, const float* image, cudaStream_t s) {
    TDIC_REQUIRE(!pair->exact || pair->degree == 1, TDIC_INVALID_ARG, "exact cubic/quintic pairs use launch_pair_setup");
    const size_t n = static_cast<size_t>(pair->cw) * pair->ch;
    if (pair->precision == TDIC_FP64)
        pad_copy_kernel<float, double><<<grid_for(n, 256), 256, 0, s>>>(image, pair->w, pair->h, pair->rpitch,
                                                                         pair->border, pair->cw, pair->ch, pair->cpitch,
                                                                         pair->exact, pair->coef.as<double>());
    else
        pad_copy_kernel<float, float><<<grid_for(n, 256), 256, 0, s>>>(image, pair->w, pair->h, pair->rpitch,
                                                                       pair->border, pair->cw, pair->ch, pair->cpitch,
                                                                       pair->exact, pair->coef.as<float>());
    TDIC_CUDA_TRY(cudaGetLastError());
}

// Exact cubic / quintic pair set-up from the raw images in one launch (prefilter_fused_kernel):
// ref, def device images of `dtype` with `pitch` elements per row; writes pair->ref, pair->def_f
// (float32, rounded as the reference binding rounds a float64 input) and pair->coef.
void launch_pair_setup(tdic_pair* pair, const void* ref, const void* def, int pitch, tdic_dtype dtype,
                       cudaStream_t s) {
    TDIC_REQUIRE(pair->exact && (pair->degree == 3 || pair->degree == 5), TDIC_INVALID_ARG,
                 "pair set-up kernel needs an exact cubic or quintic pair");
    switch (dtype) {
        case TDIC_U8: pair_setup_in<uint8_t>(pair, ref, def, pitch, s); break;
        case TDIC_U16: pair_setup_in<uint16_t>(pair, ref, def, pitch, s); break;
        case TDIC_F32: pair_setup_in<float>(pair, ref, def, pitch, s); break;
        case TDIC_F64: pair_setup_in<double>(pair, ref, def, pitch, s); break;
    }
}

void launch_reference_gradient(const float* img, int w, int h, int pitch, double* gx, double* gy, cudaStream_t s) {
    gradient_kernel<<<grid_for(static_cast<size_t>(w) * h, 256), 256, 0, s>>>(img, w, h, pitch, gx, gy);
    TDIC_CUDA_TRY(cudaGetLastError());
}

}  // namespace tdic
