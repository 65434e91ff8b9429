// Least-squares strain of 2D point displacements on the device
// (dic::compute_least_squares_strain_2d, src/postprocess/least_squares_strain.cpp:11-78).
//
// Per point: the neighbours within `radius` (the point itself included), found through square
// buckets of side `radius` as in the reference; a plane fit u = a0 + a1 dx + a2 dy (and v) in
// FP64 through the normal equations, solved by LDL^T with diagonal pivoting.  The normal
// matrix's diagonal holds the squared column norms of the design matrix and its Schur
// complements the norms of the projected columns, so the pivot sequence is that of the
// column-pivoted Householder QR the reference uses; a rank-deficient fit gets the same basic
// solution (zero for the dependent columns).  Green-Lagrange or small strain from the gradient.
#include "tdic_internal.cuh"

#include <algorithm>
#include <cmath>
#include <unordered_map>

namespace tdic {

namespace {

struct StrainOut {
    double du_dx, du_dy, dv_dx, dv_dy, exx, eyy, exy;
    int sample_count;
    int valid;
};

// Solve the 3x3 symmetric positive semi-definite system N x = b for two right-hand sides with
// pivoted LDL^T; columns whose pivot falls below `tol` times the largest diagonal are dependent
// and get zero.  Returns false when nothing is solvable.
__device__ bool solve3_pivoted(double (&n)[3][3], double (&b)[2][3], double (&x)[2][3]) {
    int perm[3] = {0, 1, 2};
    double dmax = fmax(n[0][0], fmax(n[1][1], n[2][2]));
    if (!(dmax > 0.0) || !isfinite(dmax)) return false;
    const double tol = 1e-13 * dmax;
    int rank = 0;
    double l[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    double d[3] = {0, 0, 0};
    for (int k = 0; k < 3; ++k) {
        // pivot: the largest remaining diagonal of the Schur complement
        int piv = k;
        for (int i = k + 1; i < 3; ++i)
            if (n[i][i] > n[piv][piv]) piv = i;
        if (piv != k) {
            for (int c = 0; c < 3; ++c) { const double t = n[k][c]; n[k][c] = n[piv][c]; n[piv][c] = t; }
            for (int r = 0; r < 3; ++r) { const double t = n[r][k]; n[r][k] = n[r][piv]; n[r][piv] = t; }
            for (int c = 0; c < k; ++c) { const double t = l[k][c]; l[k][c] = l[piv][c]; l[piv][c] = t; }
            const int t = perm[k]; perm[k] = perm[piv]; perm[piv] = t;
        }
        if (!(n[k][k] > tol)) break;
        d[k] = n[k][k];
        l[k][k] = 1.0;
        for (int i = k + 1; i < 3; ++i) l[i][k] = n[i][k] / d[k];
        for (int i = k + 1; i < 3; ++i)
            for (int j = k + 1; j < 3; ++j) n[i][j] -= l[i][k] * d[k] * l[j][k];
        ++rank;
    }
    if (rank == 0) return false;
    for (int r = 0; r < 2; ++r) {
        double y[3];
        for (int i = 0; i < rank; ++i) {  // forward substitution on the leading block
            double s = b[r][perm[i]];
            for (int j = 0; j < i; ++j) s -= l[i][j] * y[j];
            y[i] = s;
        }
        for (int i = 0; i < rank; ++i) y[i] /= d[i];
        double z[3] = {0, 0, 0};
        for (int i = rank - 1; i >= 0; --i) {
            double s = y[i];
            for (int j = i + 1; j < rank; ++j) s -= l[j][i] * z[j];
            z[i] = s;
        }
        for (int i = 0; i < 3; ++i) x[r][perm[i]] = i < rank ? z[i] : 0.0;
    }
    return true;
}

__global__ void ls_strain_kernel(const double* __restrict__ pts, const double* __restrict__ disp, int n,
                                 const int* __restrict__ bucket_of, const int* __restrict__ bstart,
                                 const int* __restrict__ bitems, int bx0, int by0, int nbx, int nby, double radius,
                                 int min_samples, int green, StrainOut* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    StrainOut o{0, 0, 0, 0, 0, 0, 0, 0, 0};
    const int b = bucket_of[i];
    if (b < 0) {  // not finite: left out, as the reference
        out[i] = o;
        return;
    }
    const double x0 = pts[2 * i], y0 = pts[2 * i + 1];
    const double r2 = radius * radius;
    const int bxi = b % nbx, byi = b / nbx;
    double nm[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    double rhs[2][3] = {{0, 0, 0}, {0, 0, 0}};
    int count = 0;
    for (int dy = -1; dy <= 1; ++dy) {
        for (int dx = -1; dx <= 1; ++dx) {
            const int qx = bxi + dx, qy = byi + dy;
            if (qx < 0 || qy < 0 || qx >= nbx || qy >= nby) continue;
            const int q = qy * nbx + qx;
            for (int k = bstart[q]; k < bstart[q + 1]; ++k) {
                const int j = bitems[k];
                const double ex = pts[2 * j] - x0, ey = pts[2 * j + 1] - y0;
                if (ex * ex + ey * ey > r2) continue;
                const double a[3] = {1.0, ex, ey};
                for (int r = 0; r < 3; ++r)
                    for (int c = 0; c < 3; ++c) nm[r][c] += a[r] * a[c];
                for (int r = 0; r < 3; ++r) {
                    rhs[0][r] += a[r] * disp[2 * j];
                    rhs[1][r] += a[r] * disp[2 * j + 1];
                }
                ++count;
            }
        }
    }
    o.sample_count = count;
    (void)bx0;
    (void)by0;
    double sol[2][3];
    if (count >= min_samples && solve3_pivoted(nm, rhs, sol)) {
        bool fin = true;
        for (int r = 0; r < 2; ++r)
            for (int c = 0; c < 3; ++c) fin = fin && isfinite(sol[r][c]);
        if (fin) {
            o.du_dx = sol[0][1]; o.du_dy = sol[0][2]; o.dv_dx = sol[1][1]; o.dv_dy = sol[1][2];
            if (green) {  // E = (H + H^T + H^T H) / 2
                const double h00 = o.du_dx, h01 = o.du_dy, h10 = o.dv_dx, h11 = o.dv_dy;
                o.exx = 0.5 * (2.0 * h00 + h00 * h00 + h10 * h10);
                o.eyy = 0.5 * (2.0 * h11 + h01 * h01 + h11 * h11);
                o.exy = 0.5 * (h01 + h10 + h00 * h01 + h10 * h11);
            } else {
                o.exx = o.du_dx;
                o.eyy = o.dv_dy;
                o.exy = 0.5 * (o.du_dy + o.dv_dx);
            }
            o.valid = 1;
        }
    }
    out[i] = o;
}

}  // namespace

void ls_strain_2d(tdic_ctx* ctx, const double* points, const double* disp, int n, double radius, int min_samples,
                  int green, tdic_ls_strain* out, cudaStream_t s) {
    if (n <= 0) return;
    // buckets of side `radius` over the finite points (reference: floor(coordinate / radius))
    std::vector<int> bucket_of(n, -1);
    long long bx0 = 0, by0 = 0, bx1 = -1, by1 = -1;
    bool any = false;
    std::vector<std::pair<long long, long long>> key(n);
    for (int i = 0; i < n; ++i) {
        const double x = points[2 * i], y = points[2 * i + 1], u = disp[2 * i], v = disp[2 * i + 1];
        if (!(std::isfinite(x) && std::isfinite(y) && std::isfinite(u) && std::isfinite(v))) continue;
        const long long kx = static_cast<long long>(std::floor(x / radius)), ky = static_cast<long long>(std::floor(y / radius));
        key[i] = {kx, ky};
        if (!any) { bx0 = bx1 = kx; by0 = by1 = ky; any = true; }
        bx0 = std::min(bx0, kx); bx1 = std::max(bx1, kx); by0 = std::min(by0, ky); by1 = std::max(by1, ky);
        bucket_of[i] = 0;
    }
    const long long nbx = any ? bx1 - bx0 + 1 : 1, nby = any ? by1 - by0 + 1 : 1;
    TDIC_REQUIRE(nbx * nby <= (1LL << 28), TDIC_INVALID_ARG,
                 "least-squares strain: the radius is too small for the extent of the points");
    std::vector<int> start(static_cast<size_t>(nbx * nby) + 1, 0);
    for (int i = 0; i < n; ++i)
        if (bucket_of[i] >= 0) {
            bucket_of[i] = static_cast<int>((key[i].second - by0) * nbx + (key[i].first - bx0));
            ++start[bucket_of[i] + 1];
        }
    for (size_t q = 1; q < start.size(); ++q) start[q] += start[q - 1];
    std::vector<int> items(std::max(1, start.back())), fill(start.begin(), start.end() - 1);
    for (int i = 0; i < n; ++i)  // each bucket lists its points in index order, as the reference
        if (bucket_of[i] >= 0) items[fill[bucket_of[i]]++] = i;
    Buffer d_pts(&ctx->pool, 16 * static_cast<size_t>(n)), d_disp(&ctx->pool, 16 * static_cast<size_t>(n)),
        d_bof(&ctx->pool, 4 * static_cast<size_t>(n)), d_start(&ctx->pool, 4 * start.size()),
        d_items(&ctx->pool, 4 * items.size()), d_out(&ctx->pool, sizeof(StrainOut) * static_cast<size_t>(n));
    TDIC_CUDA_TRY(cudaMemcpyAsync(d_pts.ptr, points, 16 * static_cast<size_t>(n), cudaMemcpyHostToDevice, s));
    TDIC_CUDA_TRY(cudaMemcpyAsync(d_disp.ptr, disp, 16 * static_cast<size_t>(n), cudaMemcpyHostToDevice, s));
    TDIC_CUDA_TRY(cudaMemcpyAsync(d_bof.ptr, bucket_of.data(), 4 * static_cast<size_t>(n), cudaMemcpyHostToDevice, s));
    TDIC_CUDA_TRY(cudaMemcpyAsync(d_start.ptr, start.data(), 4 * start.size(), cudaMemcpyHostToDevice, s));
    TDIC_CUDA_TRY(cudaMemcpyAsync(d_items.ptr, items.data(), 4 * items.size(), cudaMemcpyHostToDevice, s));
    ls_strain_kernel<<<(n + 127) / 128, 128, 0, s>>>(d_pts.as<double>(), d_disp.as<double>(), n, d_bof.as<int>(),
                                                     d_start.as<int>(), d_items.as<int>(), static_cast<int>(bx0),
                                                     static_cast<int>(by0), static_cast<int>(nbx), static_cast<int>(nby),
                                                     radius, min_samples, green, d_out.as<StrainOut>());
    TDIC_CUDA_TRY(cudaGetLastError());
    std::vector<StrainOut> host(n);
    TDIC_CUDA_TRY(cudaMemcpyAsync(host.data(), d_out.ptr, sizeof(StrainOut) * static_cast<size_t>(n),
                                  cudaMemcpyDeviceToHost, s));
    TDIC_CUDA_TRY(cudaStreamSynchronize(s));
    for (int i = 0; i < n; ++i) {
        const StrainOut& o = host[i];
        out[i] = tdic_ls_strain{o.du_dx, o.du_dy, o.dv_dx, o.dv_dy, o.exx, o.eyy, o.exy, o.sample_count,
                                static_cast<uint8_t>(o.valid), {0, 0, 0}};
    }
}

}  // namespace tdic
