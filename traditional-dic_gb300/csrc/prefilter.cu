// K1: B-spline coefficient prefilter, K2: reference-image gradients, image conversion.
//
// K1 computes BSplineImagePreprocessor::form_coefficients (bspline.cpp:369-392): the image is
// padded by `border` pixels with half-sample symmetry (symmetric_index, bspline.cpp:78-89) and
// every row, then every column, of the (H+2B) x (W+2B) padded image is deconvolved by the
// sampled B-spline kernel with PERIODIC boundary over the padded length (the reference does it
// with an FFT, bspline.cpp:191-244).  Here the exact periodic inverse is applied as a cascade of
// first-order recursive filters (poles of the sampled kernel; gain prod (1 - z)^2) on shared-
// memory tiles: each CTA loads an output tile plus a margin of M samples on every side (indices
// taken modulo the padded size, which is what periodicity means), runs the row recursions then
// the column recursions in shared memory and writes the central tile.  A margin of M samples
// leaves a truncation error of order |z_max|^M, chosen below the rounding error of the type.
// Traffic: the raw image is read once from HBM (tiles overlap only in L2) and the coefficients
// are written once: W*H*b_in + (W+2B)(H+2B)*sizeof(T) bytes.
#include "tdic_internal.cuh"

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

// Margin so that |z_max|^M * M stays below the unit roundoff of T.
template <typename T, int DEG> struct Margin;
template <> struct Margin<float, 3> { static constexpr int M = 16; };
template <> struct Margin<float, 5> { static constexpr int M = 28; };
template <> struct Margin<double, 3> { static constexpr int M = 32; };
template <> struct Margin<double, 5> { static constexpr int M = 52; };

template <typename T> struct TileW { static constexpr int value = 64; };

// One recursive pole pass over n samples at stride `st` in shared memory (causal then
// anti-causal, zero state beyond the window).
template <typename T>
__device__ inline void pole_pass(T* x, int n, int st, T z) {
    T acc = T(0);
    for (int i = 0; i < n; ++i) {
        acc = x[i * st] + z * acc;
        x[i * st] = acc;
    }
    acc = T(0);
    for (int i = n - 1; i >= 0; --i) {
        acc = x[i * st] + z * acc;
        x[i * st] = acc;
    }
}

template <typename In, typename T, int DEG>
__global__ void __launch_bounds__(128) prefilter_tile_kernel(const In* __restrict__ img, int w, int h, int pitch,
                                                             int border, int cw, int ch, int opitch, T z0, T z1,
                                                             T gain, T* __restrict__ out) {
    constexpr int M = Margin<T, DEG>::M;
    constexpr int TW = TileW<T>::value;
    constexpr int L = TW + 2 * M;  // tile side with margins
    constexpr int P = L + 1;       // padded row stride (odd: conflict-free row walks for 4-byte T)
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* s = reinterpret_cast<T*>(smem_raw);
    const int tx0 = blockIdx.x * TW, ty0 = blockIdx.y * TW;
    // Load the tile with margins: padded coordinate -> periodic wrap -> symmetric source index.
    for (int i = threadIdx.x; i < L * L; i += blockDim.x) {
        const int r = i / L, c = i - r * L;
        const int py = wrap(ty0 - M + r, ch), px = wrap(tx0 - M + c, cw);
        const int sy = sym_index(py - border, h), sx = sym_index(px - border, w);
        s[r * P + c] = gain * static_cast<T>(load_px(img + static_cast<size_t>(sy) * pitch + sx));
    }
    __syncthreads();
    // Row recursions: one thread per tile row.
    for (int r = threadIdx.x; r < L; r += blockDim.x) {
        pole_pass<T>(s + r * P, L, 1, z0);
        if (DEG == 5) pole_pass<T>(s + r * P, L, 1, z1);
    }
    __syncthreads();
    // Column recursions: only the central TW columns are needed.
    for (int c = threadIdx.x; c < TW; c += blockDim.x) {
        pole_pass<T>(s + M + c, L, P, z0);
        if (DEG == 5) pole_pass<T>(s + M + c, L, P, z1);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < TW * TW; i += blockDim.x) {
        const int r = i / TW, c = i - r * TW;
        const int oy = ty0 + r, ox = tx0 + c;
        if (oy < ch && ox < cw) out[static_cast<size_t>(oy) * opitch + ox] = s[(M + r) * P + M + c];
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

template <typename In, typename T>
void prefilter_typed(const In* img, int w, int h, int pitch, int border, int cw, int ch, int opitch, int degree,
                     int exact, T* out, cudaStream_t s) {
    if (!exact || degree == 1) {
        pad_copy_kernel<In, T><<<grid_for(static_cast<size_t>(cw) * ch, 256), 256, 0, s>>>(img, w, h, pitch, border, cw,
                                                                                         ch, opitch, exact, out);
        return;
    }
    const Poles p = poles_for(degree);
    constexpr int TW = TileW<T>::value;
    dim3 grid((cw + TW - 1) / TW, (ch + TW - 1) / TW);
    if (degree == 3) {
        constexpr int M = Margin<T, 3>::M, L = TW + 2 * M;
        const size_t smem = static_cast<size_t>(L) * (L + 1) * sizeof(T);
        TDIC_CUDA_TRY(cudaFuncSetAttribute(prefilter_tile_kernel<In, T, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           static_cast<int>(smem)));
        prefilter_tile_kernel<In, T, 3><<<grid, 128, smem, s>>>(img, w, h, pitch, border, cw, ch, opitch, T(p.z[0]), T(0),
                                                                T(p.gain * p.gain), out);  // one gain per 1-D pass
    } else {
        constexpr int M = Margin<T, 5>::M, L = TW + 2 * M;
        const size_t smem = static_cast<size_t>(L) * (L + 1) * sizeof(T);
        TDIC_CUDA_TRY(cudaFuncSetAttribute(prefilter_tile_kernel<In, T, 5>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           static_cast<int>(smem)));
        prefilter_tile_kernel<In, T, 5><<<grid, 128, smem, s>>>(img, w, h, pitch, border, cw, ch, opitch, T(p.z[0]), T(p.z[1]),
                                                                T(p.gain * p.gain), out);  // one gain per 1-D pass
    }
    TDIC_CUDA_TRY(cudaGetLastError());
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

// The deformed image is read through its float32 copy (dic::Image holds float, and a float64
// numpy input is rounded to float by the reference binding, bind_subset.cpp:50-64).
void launch_prefilter(tdic_pair* pair, const float* image, cudaStream_t s) {
    if (pair->precision == TDIC_FP64)
        prefilter_typed<float, double>(image, pair->w, pair->h, pair->rpitch, pair->border, pair->cw, pair->ch,
                                       pair->cpitch, pair->degree, pair->exact, pair->coef.as<double>(), s);
    else
        prefilter_typed<float, float>(image, pair->w, pair->h, pair->rpitch, pair->border, pair->cw, pair->ch,
                                      pair->cpitch, pair->degree, pair->exact, pair->coef.as<float>(), s);
}

void launch_reference_gradient(const float* img, int w, int h, int pitch, double* gx, double* gy, cudaStream_t s) {
    gradient_kernel<<<grid_for(static_cast<size_t>(w) * h, 256), 256, 0, s>>>(img, w, h, pitch, gx, gy);
    TDIC_CUDA_TRY(cudaGetLastError());
}

}  // namespace tdic
