/*
 * tdic_oracle.cpp -- FP64 CPU restatement of the Traditional-DIC 2D subset-DIC hot path.
 *
 * TEST INFRASTRUCTURE ONLY (parity checker and CPU baseline); see tdic_oracle.h for what
 * pins it.  Plain C++17, no Eigen.  Each function cites the reference file:line it follows.
 * Two deliberate, documented differences in mechanism (not in result):
 *   - the periodic deconvolution of bspline.cpp:191-244 (Eigen::FFT / kissfft) is computed
 *     with the exact periodic recursive filter (poles of the sampled B-spline kernel, causal
 *     and anti-causal passes with closed-form periodic initial values); both are the exact
 *     inverse of the same circulant system, so they agree to rounding (~1e-13);
 *   - the 6x6 LDLT of Eigen (icgn.cpp:538, forward_gauss_newton.cpp:355) is restated as
 *     symmetric diagonal pivoting LDLT with the same success / positivity semantics.
 * The "frontier" propagation mode is not a reference behaviour: it is the deterministic wave
 * rule that the GPU path uses, restated here so the GPU can be checked mode-for-mode.
 */
#include "tdic_oracle.h"

#include <algorithm>
#include <array>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <condition_variable>
#include <cstdint>
#include <cstring>
#include <functional>
#include <limits>
#include <mutex>
#include <numeric>
#include <queue>
#include <thread>
#include <vector>

namespace {

constexpr double kEps = 1e-12;  // icgn.cpp:13, forward_gauss_newton.cpp:11, integer_search.cpp:10
constexpr double kInf = std::numeric_limits<double>::infinity();
constexpr double kNaN = std::numeric_limits<double>::quiet_NaN();

enum Status : int8_t { kSuccess = 0, kNotConverged = 1, kInvalidInput = 2, kNumericalFailure = 3 };

int factorial(int n) { int v = 1; for (int i = 2; i <= n; ++i) v *= i; return v; }
int combination(int n, int k) {
    if (k < 0 || k > n) return 0;
    return factorial(n) / (factorial(k) * factorial(n - k));
}
double plus_power(double x, int p) { return x > 0.0 ? std::pow(x, p) : 0.0; }  // bspline.cpp:68-71
int clamp_index(int v, int lo, int hi) { return std::max(lo, std::min(v, hi)); }  // bspline.cpp:73-76
int symmetric_index(int v, int size) {  // bspline.cpp:78-89
    if (size <= 0) return 0;
    const int period = 2 * size;
    int w = v % period;
    if (w < 0) w += period;
    return w < size ? w : period - 1 - w;
}

double basis(double x, int r, int d) {  // bspline.cpp:342-367
    if (r < 0 || r > d) return 0.0;
    const int dfac = factorial(d) / factorial(d - r);
    double sum = 0.0;
    for (int k = 0; k <= d + 1; ++k) {
        const double sign = k % 2 == 0 ? 1.0 : -1.0;
        const double coef = sign * static_cast<double>(combination(d + 1, k));
        const double shift = static_cast<double>(d + 1) / 2.0 - static_cast<double>(k);
        sum += coef * static_cast<double>(dfac) * plus_power(x + shift, d - r);
    }
    return sum / static_cast<double>(factorial(d));
}

bool valid_degree(int d) { return d == 1 || d == 3 || d == 5; }

void build_qk(int d, double* qk) {  // bspline.cpp:320-340
    const int n = d + 1, off = d / 2;
    for (int r = 0; r < n; ++r)
        for (int c = 0; c < n; ++c) {
            const double x = static_cast<double>(-off + c);
            const double sign = r % 2 == 0 ? 1.0 : -1.0;
            qk[r * n + c] = sign * basis(x, r, d) / static_cast<double>(factorial(r));
        }
}

// ---------------------------------------------------------------------------------------
// Exact periodic deconvolution by the sampled B-spline kernel (restates the result of
// bspline.cpp:177-244).  Poles: cubic z = sqrt(3) - 2; quintic z = roots of
// z^4 + 26 z^3 + 66 z^2 + 26 z + 1 with |z| < 1 (w = z + 1/z solves w^2 + 26 w + 64 = 0).
// Gain prod (1 - z)^2 makes the DC response 1.
// ---------------------------------------------------------------------------------------
int spline_poles(int d, double* z) {
    if (d == 3) { z[0] = std::sqrt(3.0) - 2.0; return 1; }
    if (d == 5) {
        const double s = std::sqrt(105.0);
        const double w1 = -13.0 + s, w2 = -13.0 - s;
        z[0] = 0.5 * (w1 + std::sqrt(w1 * w1 - 4.0));
        z[1] = 0.5 * (w2 + std::sqrt(w2 * w2 - 4.0));
        return 2;
    }
    return 0;
}

void deconvolve_periodic(double* s, int L, std::ptrdiff_t stride, int d, std::vector<double>& tmp) {
    double z[2];
    const int np = spline_poles(d, z);
    if (np == 0) return;
    tmp.resize(static_cast<std::size_t>(L));
    double gain = 1.0;
    for (int k = 0; k < np; ++k) gain *= (1.0 - z[k]) * (1.0 - z[k]);
    for (int i = 0; i < L; ++i) tmp[i] = s[i * stride] * gain;
    for (int k = 0; k < np; ++k) {
        const double zk = z[k];
        const double zl = std::pow(zk, L);
        // causal: y[0] = sum_{j<L} z^j x[-j mod L] / (1 - z^L)
        double acc = 0.0, zj = 1.0;
        for (int j = 0; j < L; ++j) {
            acc += zj * tmp[(L - j) % L];
            zj *= zk;
            if (std::fabs(zj) < 1e-300) break;
        }
        tmp[0] = acc / (1.0 - zl);
        for (int i = 1; i < L; ++i) tmp[i] += zk * tmp[i - 1];
        // anti-causal: c[L-1] = sum_{j<L} z^j y[(L-1+j) mod L] / (1 - z^L)
        acc = 0.0; zj = 1.0;
        for (int j = 0; j < L; ++j) {
            acc += zj * tmp[(L - 1 + j) % L];
            zj *= zk;
            if (std::fabs(zj) < 1e-300) break;
        }
        tmp[L - 1] = acc / (1.0 - zl);
        for (int i = L - 2; i >= 0; --i) tmp[i] += zk * tmp[i + 1];
    }
    for (int i = 0; i < L; ++i) s[i * stride] = tmp[i];
}

// ---------------------------------------------------------------------------------------
// Interpolation through the local polynomial block qk * C * qk^T (bspline.cpp:153-175,
// 418-424) evaluated as in evaluate_polynomial{,_dx,_dy} (bspline.cpp:96-151).
// ---------------------------------------------------------------------------------------
struct Spline {
    const double* c = nullptr;
    int w = 0, h = 0, d = 3, border = 3, cw = 0, ch = 0;
    double qk[36];
    void init(const double* coeffs, int w_, int h_, int d_, int b_) {
        c = coeffs; w = w_; h = h_; d = d_; border = std::max(3, b_);
        cw = w + 2 * border; ch = h + 2 * border;
        build_qk(d, qk);
    }
    void block(int ix, int iy, double* out) const {  // bspline.cpp:153-175
        const int n = d + 1, off = d / 2;
        const int top = iy + border - off, left = ix + border - off;
        double cb[36], t[36];
        for (int r = 0; r < n; ++r) {
            const int sy = clamp_index(top + r, 0, ch - 1);
            for (int q = 0; q < n; ++q) cb[r * n + q] = c[static_cast<std::size_t>(sy) * cw + clamp_index(left + q, 0, cw - 1)];
        }
        for (int i = 0; i < n; ++i)  // t = qk * cb
            for (int j = 0; j < n; ++j) {
                double s = 0.0;
                for (int k = 0; k < n; ++k) s += qk[i * n + k] * cb[k * n + j];
                t[i * n + j] = s;
            }
        for (int i = 0; i < n; ++i)  // out = t * qk^T
            for (int j = 0; j < n; ++j) {
                double s = 0.0;
                for (int k = 0; k < n; ++k) s += t[i * n + k] * qk[j * n + k];
                out[i * n + j] = s;
            }
    }
    void locate(double x, double y, int& ix, int& iy, double& dx, double& dy) const {  // bspline.cpp:465-468
        ix = clamp_index(static_cast<int>(std::floor(x)), 0, w - 1);
        iy = clamp_index(static_cast<int>(std::floor(y)), 0, h - 1);
        dx = x - static_cast<double>(ix);
        dy = y - static_cast<double>(iy);
    }
    double value(double x, double y) const {  // bspline.cpp:458-474, 96-113
        int ix, iy; double dx, dy;
        locate(x, y, ix, iy, dx, dy);
        double b[36];
        block(ix, iy, b);
        const int n = d + 1;
        double v = 0.0, yp = 1.0;
        for (int r = 0; r < n; ++r) {
            double xp = 1.0;
            for (int q = 0; q < n; ++q) { v += b[r * n + q] * yp * xp; xp *= dx; }
            yp *= dy;
        }
        return v;
    }
    void gradient(double x, double y, double& gx, double& gy) const {  // bspline.cpp:476-500, 115-151
        int ix, iy; double dx, dy;
        locate(x, y, ix, iy, dx, dy);
        double b[36];
        block(ix, iy, b);
        const int n = d + 1;
        double vx = 0.0, yp = 1.0;
        for (int r = 0; r < n; ++r) {
            double xp = 1.0;
            for (int q = 1; q < n; ++q) { vx += static_cast<double>(q) * b[r * n + q] * yp * xp; xp *= dx; }
            yp *= dy;
        }
        double vy = 0.0;
        yp = 1.0;
        for (int r = 1; r < n; ++r) {
            double xp = 1.0;
            for (int q = 0; q < n; ++q) { vy += static_cast<double>(r) * b[r * n + q] * yp * xp; xp *= dx; }
            yp *= dy;
        }
        gx = vx; gy = vy;
    }
};

void form_coefficients(const float* img, int w, int h, int d, int border, bool exact, double* out) {
    // bspline.cpp:369-392
    border = std::max(3, border);
    const int cw = w + 2 * border, ch = h + 2 * border;
    for (int y = 0; y < ch; ++y) {
        const int sy = exact ? symmetric_index(y - border, h) : clamp_index(y - border, 0, h - 1);
        for (int x = 0; x < cw; ++x) {
            const int sx = exact ? symmetric_index(x - border, w) : clamp_index(x - border, 0, w - 1);
            out[static_cast<std::size_t>(y) * cw + x] = static_cast<double>(img[static_cast<std::size_t>(sy) * w + sx]);
        }
    }
    if (exact) {
        std::vector<double> tmp;
        for (int y = 0; y < ch; ++y) deconvolve_periodic(out + static_cast<std::size_t>(y) * cw, cw, 1, d, tmp);
        for (int x = 0; x < cw; ++x) deconvolve_periodic(out + x, ch, cw, d, tmp);
    }
}

// ---------------------------------------------------------------------------------------
// N x N LDLT (N = 6 first order, 12 second order) with symmetric diagonal pivoting and sign
// tracking: restates the factorisation semantics relied on by icgn.cpp:538-542, 1262-1266 /
// forward_gauss_newton.cpp:354-358, 1249-1253 (info() == Success, isPositive()) and the
// pseudo-inverse solve of D.
// ---------------------------------------------------------------------------------------
template <int N>
struct LdltN {
    double m[N][N];
    int t[N];
    enum { kZero, kPosSemi, kNegSemi, kIndef } sign = kZero;
    bool ok = true;

    void factor(const double a[N][N]) {
        for (int i = 0; i < N; ++i) for (int j = 0; j < N; ++j) m[i][j] = a[i][j];
        sign = kZero;
        ok = true;
        bool found_zero = false;
        double temp[N];
        for (int k = 0; k < N; ++k) {
            int big = k;
            double bigv = std::fabs(m[k][k]);
            for (int i = k + 1; i < N; ++i) if (std::fabs(m[i][i]) > bigv) { bigv = std::fabs(m[i][i]); big = i; }
            t[k] = big;
            if (big != k) {
                for (int j = 0; j < k; ++j) std::swap(m[k][j], m[big][j]);
                for (int i = big + 1; i < N; ++i) std::swap(m[i][k], m[i][big]);
                std::swap(m[k][k], m[big][big]);
                for (int i = k + 1; i < big; ++i) { const double tmp = m[i][k]; m[i][k] = m[big][i]; m[big][i] = tmp; }
            }
            if (k > 0) {
                for (int j = 0; j < k; ++j) temp[j] = m[j][j] * m[k][j];
                double s = 0.0;
                for (int j = 0; j < k; ++j) s += m[k][j] * temp[j];
                m[k][k] -= s;
                for (int i = k + 1; i < N; ++i) {
                    double si = 0.0;
                    for (int j = 0; j < k; ++j) si += m[i][j] * temp[j];
                    m[i][k] -= si;
                }
            }
            const double akk = m[k][k];
            const bool pivot_valid = std::fabs(akk) > 0.0;
            if (k == 0 && !pivot_valid) {
                sign = kZero;
                for (int j = 0; j < N; ++j) { t[j] = j; for (int i = 0; i < N; ++i) m[i][j] = 0.0; }
                ok = true;
                return;
            }
            if (pivot_valid) {
                for (int i = k + 1; i < N; ++i) m[i][k] /= akk;
            } else {
                for (int i = k + 1; i < N; ++i) ok = ok && (m[i][k] == 0.0);
            }
            if (found_zero && pivot_valid) ok = false;
            else if (!pivot_valid) found_zero = true;
            if (sign == kPosSemi) { if (akk < 0.0) sign = kIndef; }
            else if (sign == kNegSemi) { if (akk > 0.0) sign = kIndef; }
            else if (sign == kZero) { if (akk > 0.0) sign = kPosSemi; else if (akk < 0.0) sign = kNegSemi; }
        }
    }
    bool success() const { return ok; }
    bool positive() const { return sign == kPosSemi || sign == kZero; }
    void solve(const double b[N], double x[N]) const {
        for (int i = 0; i < N; ++i) x[i] = b[i];
        for (int k = 0; k < N; ++k) std::swap(x[k], x[t[k]]);
        for (int i = 0; i < N; ++i) { double s = x[i]; for (int j = 0; j < i; ++j) s -= m[i][j] * x[j]; x[i] = s; }
        for (int i = 0; i < N; ++i) { const double dd = m[i][i]; x[i] = std::fabs(dd) > DBL_MIN ? x[i] / dd : 0.0; }
        for (int i = N - 1; i >= 0; --i) { double s = x[i]; for (int j = i + 1; j < N; ++j) s -= m[j][i] * x[j]; x[i] = s; }
        for (int k = N - 1; k >= 0; --k) std::swap(x[k], x[t[k]]);
    }
};
using Ldlt6 = LdltN<6>;

// ---------------------------------------------------------------------------------------
// 6x6 LU with full pivoting: the Eigen::FullPivLU semantics used by the second-order
// inverse-compositional update (icgn.cpp:325-329): pivot = first largest |entry| of the
// remaining corner in column-major order, rank counted against 6 * DBL_EPSILON * |largest
// pivot|, inverse = the solve of the identity (row permutation, unit-lower and upper
// substitution, column permutation).
// ---------------------------------------------------------------------------------------
bool fullpiv_inverse6(const double a[6][6], double inv[6][6]) {
    double lu[6][6];
    for (int i = 0; i < 6; ++i) for (int j = 0; j < 6; ++j) lu[i][j] = a[i][j];
    int rt[6], ct[6];
    int nonzero = 6;
    double maxpivot = 0.0;
    for (int k = 0; k < 6; ++k) {
        int br = k, bc = k;
        double big = -1.0;
        for (int c = k; c < 6; ++c)
            for (int r = k; r < 6; ++r)
                if (std::fabs(lu[r][c]) > big) { big = std::fabs(lu[r][c]); br = r; bc = c; }
        if (big == 0.0) {
            nonzero = k;
            for (int i = k; i < 6; ++i) { rt[i] = i; ct[i] = i; }
            break;
        }
        if (big > maxpivot) maxpivot = big;
        rt[k] = br; ct[k] = bc;
        if (br != k) for (int j = 0; j < 6; ++j) std::swap(lu[k][j], lu[br][j]);
        if (bc != k) for (int i = 0; i < 6; ++i) std::swap(lu[i][k], lu[i][bc]);
        for (int r = k + 1; r < 6; ++r) lu[r][k] /= lu[k][k];
        for (int c = k + 1; c < 6; ++c)
            for (int r = k + 1; r < 6; ++r) lu[r][c] -= lu[r][k] * lu[k][c];
    }
    int rank = 0;
    const double thr = maxpivot * (6.0 * DBL_EPSILON);
    for (int i = 0; i < nonzero; ++i) rank += std::fabs(lu[i][i]) > thr ? 1 : 0;
    if (rank != 6) return false;
    int q[6] = {0, 1, 2, 3, 4, 5};
    for (int k = 0; k < 6; ++k) std::swap(q[k], q[ct[k]]);
    for (int col = 0; col < 6; ++col) {
        double c[6] = {0, 0, 0, 0, 0, 0};
        c[col] = 1.0;
        for (int k = 0; k < 6; ++k) std::swap(c[k], c[rt[k]]);
        for (int i = 0; i < 6; ++i) for (int j = 0; j < i; ++j) c[i] -= lu[i][j] * c[j];
        for (int i = 5; i >= 0; --i) {
            for (int j = i + 1; j < 6; ++j) c[i] -= lu[i][j] * c[j];
            c[i] /= lu[i][i];
        }
        for (int i = 0; i < 6; ++i) inv[q[i]][col] = c[i];
    }
    return true;
}

bool finite6(const double* p) { for (int i = 0; i < 6; ++i) if (!std::isfinite(p[i])) return false; return true; }

// icgn.cpp:83-120
void ic_update(const double* p, const double* dp, double* out) {
    const double du = p[0], dv = p[1], dudx = p[2], dudy = p[3], dvdx = p[4], dvdy = p[5];
    const double dp0 = dp[0], dp1 = dp[1], dp2 = dp[2], dp3 = dp[3], dp4 = dp[4], dp5 = dp[5];
    const double den = dp2 + dp5 + dp2 * dp5 - dp3 * dp4 + 1.0;
    if (std::fabs(den) <= kEps) { for (int i = 0; i < 6; ++i) out[i] = kNaN; return; }
    out[0] = du - ((dudx + 1.0) * (dp0 + dp0 * dp5 - dp1 * dp3)) / den - (dudy * (dp1 - dp0 * dp4 + dp1 * dp2)) / den;
    out[1] = dv - ((dvdy + 1.0) * (dp1 - dp0 * dp4 + dp1 * dp2)) / den - (dvdx * (dp0 + dp0 * dp5 - dp1 * dp3)) / den;
    out[2] = ((dp5 + 1.0) * (dudx + 1.0)) / den - (dp4 * dudy) / den - 1.0;
    out[3] = (dudy * (dp2 + 1.0)) / den - (dp3 * (dudx + 1.0)) / den;
    out[4] = (dvdx * (dp5 + 1.0)) / den - (dp4 * (dvdy + 1.0)) / den;
    out[5] = ((dp2 + 1.0) * (dvdy + 1.0)) / den - (dp3 * dvdx) / den - 1.0;
}

// forward_gauss_newton.cpp:64-76
void compose_warp(const double* p, const double* dp, double* pn) {
    pn[0] = dp[0] + p[0] + p[2] * dp[0] + p[3] * dp[1];
    pn[1] = dp[1] + p[1] + p[4] * dp[0] + p[5] * dp[1];
    pn[2] = dp[2] + p[2] * (1.0 + dp[2]) + p[3] * dp[4];
    pn[3] = dp[3] + p[2] * dp[3] + p[3] * (1.0 + dp[5]);
    pn[4] = dp[4] + p[4] * (1.0 + dp[2]) + p[5] * dp[4];
    pn[5] = dp[5] + p[4] * dp[3] + p[5] * (1.0 + dp[5]);
}

// Second-order shape function: parameters [u, v, ux, uy, vx, vy, uxx, uxy, uyy, vxx, vxy, vyy].

// The 6x6 warp matrix G'(p) (icgn.cpp:196-261): maps [1, x, y, x^2, xy, y^2] to
// [x', y', 1, x'^2, x'y', y'^2] up to second order.
void warp_matrix2(const double* p, double G[6][6]) {
    const double u = p[0], v = p[1], ux = p[2], uy = p[3], vx = p[4], vy = p[5];
    const double uxx = p[6], uxy = p[7], uyy = p[8], vxx = p[9], vxy = p[10], vyy = p[11];
    for (int i = 0; i < 6; ++i) for (int j = 0; j < 6; ++j) G[i][j] = 0.0;
    G[0][0] = u; G[0][1] = 1.0 + ux; G[0][2] = uy; G[0][3] = 0.5 * uxx; G[0][4] = uxy; G[0][5] = 0.5 * uyy;
    G[1][0] = v; G[1][1] = vx; G[1][2] = 1.0 + vy; G[1][3] = 0.5 * vxx; G[1][4] = vxy; G[1][5] = 0.5 * vyy;
    G[2][0] = 1.0;
    G[3][0] = u * u; G[3][1] = 2.0 * u * (1.0 + ux); G[3][2] = 2.0 * u * uy;
    G[3][3] = 1.0 + 2.0 * ux + ux * ux + u * uxx; G[3][4] = 2.0 * (uy + ux * uy + u * uxy); G[3][5] = uy * uy + u * uyy;
    G[4][0] = u * v; G[4][1] = v + u * vx + v * ux; G[4][2] = u + u * vy + v * uy;
    G[4][3] = vx + ux * vx + 0.5 * (u * vxx + v * uxx);
    G[4][4] = 1.0 + vy + ux + ux * vy + uy * vx + u * vxy + v * uxy;
    G[4][5] = uy + uy * vy + 0.5 * (u * vyy + v * uyy);
    G[5][0] = v * v; G[5][1] = 2.0 * v * vx; G[5][2] = 2.0 * v * (1.0 + vy);
    G[5][3] = vx * vx + v * vxx; G[5][4] = 2.0 * (vx + vx * vy + v * vxy); G[5][5] = 1.0 + 2.0 * vy + vy * vy + v * vyy;
}

// icgn.cpp:308-357: G'(p_new) = G'(p) * G'(dp)^-1 * P^-1, parameters read back from rows 0 and 1
// (extract_from_warp_matrix, icgn.cpp:265-287); additive p - dp when G'(dp) is not invertible.
void ic_update2(const double* p, const double* dp, double* out) {
    double Gp[6][6], Gd[6][6], Gi[6][6];
    warp_matrix2(p, Gp);
    warp_matrix2(dp, Gd);
    if (!fullpiv_inverse6(Gd, Gi)) { for (int i = 0; i < 12; ++i) out[i] = p[i] - dp[i]; return; }
    double X[2][6];
    for (int r = 0; r < 2; ++r)
        for (int c = 0; c < 6; ++c) { double s = 0.0; for (int k = 0; k < 6; ++k) s += Gp[r][k] * Gi[k][c]; X[r][c] = s; }
    // P^-1 moves columns (0, 1, 2) to (1, 2, 0): new column 0 = old 2, 1 = old 0, 2 = old 1.
    double N[2][6];
    for (int r = 0; r < 2; ++r) { N[r][0] = X[r][2]; N[r][1] = X[r][0]; N[r][2] = X[r][1]; for (int c = 3; c < 6; ++c) N[r][c] = X[r][c]; }
    out[0] = N[0][0]; out[2] = N[0][1] - 1.0; out[3] = N[0][2]; out[6] = 2.0 * N[0][3]; out[7] = N[0][4]; out[8] = 2.0 * N[0][5];
    out[1] = N[1][0]; out[4] = N[1][1]; out[5] = N[1][2] - 1.0; out[9] = 2.0 * N[1][3]; out[10] = N[1][4]; out[11] = 2.0 * N[1][5];
}

// forward_gauss_newton.cpp:1025-1053: W(p) o W(dp) to second order in (lx, ly), first in dp.
void compose_warp2(const double* p, const double* dp, double* pn) {
    pn[0] = dp[0] + p[0] + p[2] * dp[0] + p[3] * dp[1];
    pn[1] = dp[1] + p[1] + p[4] * dp[0] + p[5] * dp[1];
    pn[2] = dp[2] + p[2] * (1.0 + dp[2]) + p[3] * dp[4] + p[6] * dp[0] + p[7] * dp[1];
    pn[3] = dp[3] + p[2] * dp[3] + p[3] * (1.0 + dp[5]) + p[7] * dp[0] + p[8] * dp[1];
    pn[4] = dp[4] + p[4] * (1.0 + dp[2]) + p[5] * dp[4] + p[9] * dp[0] + p[10] * dp[1];
    pn[5] = dp[5] + p[4] * dp[3] + p[5] * (1.0 + dp[5]) + p[10] * dp[0] + p[11] * dp[1];
    pn[6] = dp[6] + p[2] * dp[6] + p[3] * dp[9] + p[6] * (1.0 + 2.0 * dp[2]) + 2.0 * p[7] * dp[4];
    pn[7] = dp[7] + p[2] * dp[7] + p[3] * dp[10] + p[6] * dp[3] + p[7] * (1.0 + dp[2] + dp[5]) + p[8] * dp[4];
    pn[8] = dp[8] + p[2] * dp[8] + p[3] * dp[11] + p[7] * dp[3] + p[8] * (1.0 + 2.0 * dp[5]);
    pn[9] = dp[9] + p[4] * dp[6] + p[5] * dp[9] + p[9] * (1.0 + 2.0 * dp[2]) + 2.0 * p[10] * dp[4];
    pn[10] = dp[10] + p[4] * dp[7] + p[5] * dp[10] + p[9] * dp[3] + p[10] * (1.0 + dp[2] + dp[5]) + p[11] * dp[4];
    pn[11] = dp[11] + p[4] * dp[8] + p[5] * dp[11] + p[10] * dp[3] + p[11] * (1.0 + 2.0 * dp[5]);
}

struct GradSource {  // reference_gradient_at, icgn.cpp:55-71 / central difference icgn.cpp:42-53
    const float* img; int w, h;
    const double* gx; const double* gy;
    void at(int x, int y, double& ox, double& oy) const {
        if (gx && gy) { ox = gx[static_cast<std::size_t>(y) * w + x]; oy = gy[static_cast<std::size_t>(y) * w + x]; return; }
        const int xm = std::max(0, x - 1), xp = std::min(w - 1, x + 1);
        const int ym = std::max(0, y - 1), yp = std::min(h - 1, y + 1);
        ox = (static_cast<double>(img[static_cast<std::size_t>(y) * w + xp]) - static_cast<double>(img[static_cast<std::size_t>(y) * w + xm])) / static_cast<double>(std::max(1, xp - xm));
        oy = (static_cast<double>(img[static_cast<std::size_t>(yp) * w + x]) - static_cast<double>(img[static_cast<std::size_t>(ym) * w + x])) / static_cast<double>(std::max(1, yp - ym));
    }
};

struct SolverCfg {
    int radius; int max_iter; double thr; int optimizer;
    int order = 1;      // shape function: 1 first order (6 parameters), 2 second order (12)
    bool ssd = false;   // objective: SSD instead of ZNSSD
    // masked subsets (solve_with_mask, truncate_roi_subsets): samples outside the image or the
    // ROI are left out; NULL = the full circular subset of solve_with_interpolators
    const uint8_t* roi = nullptr;
    int min_valid = 12;
    double ratio = 0.5;
};

// Subset samples of the masked routes (icgn.cpp:629-704 and its siblings): the centre must be a
// ROI pixel (no margin check); a circle sample counts towards the full count, and is kept only
// inside the image and the ROI; at least max(NP, min_valid_samples, ceil(ratio * full)) kept.
inline bool masked_centre_ok(const SolverCfg& c, int w, int h, int cx, int cy) {
    return cx >= 0 && cy >= 0 && cx < w && cy < h && c.roi[static_cast<std::size_t>(cy) * w + cx] != 0;
}
inline bool masked_keep(const SolverCfg& c, int w, int h, int x, int y) {
    return x >= 0 && y >= 0 && x < w && y < h && c.roi[static_cast<std::size_t>(y) * w + x] != 0;
}
inline int masked_min_samples(const SolverCfg& c, int np, int full) {
    return std::max(np, std::max(c.min_valid, static_cast<int>(std::ceil(c.ratio * static_cast<double>(full)))));
}

void init_result(orc_poi_result& r, const double* p0, double conf) {
    // icgn.cpp:454-462: u, v from the initial guess, gradients default to zero.
    for (int i = 0; i < 6; ++i) { r.p[i] = 0.0; r.q[i] = 0.0; }
    r.p[0] = p0[0]; r.p[1] = p0[1];
    r.correlation = conf;
    r.iterations = 0; r.status = kInvalidInput; r.valid = 0; r.converged = 0; r.pad_ = 0;
}

// Shape-function terms of one sample: m = [1, lx, ly, lx^2/2, lx ly, ly^2/2]; the steepest
// descent row for gradient (a, b) is [a m0, b m0, a m1, a m2, b m1, b m2, a m3, a m4, a m5,
// b m3, b m4, b m5] (icgn.cpp:142-165 second order; the first six for first order).
template <int NP>
void sd_row(double a, double b, double lx, double ly, double* sd) {
    sd[0] = a; sd[1] = b; sd[2] = a * lx; sd[3] = a * ly; sd[4] = b * lx; sd[5] = b * ly;
    if constexpr (NP == 12) {
        const double x2 = lx * lx * 0.5, y2 = ly * ly * 0.5, xy = lx * ly;
        sd[6] = a * x2; sd[7] = a * xy; sd[8] = a * y2; sd[9] = b * x2; sd[10] = b * xy; sd[11] = b * y2;
    }
}

// Warped sample position (icgn.cpp:555-558 first order; warp_second_order icgn.cpp:167-182).
template <int NP>
void warp_pt(int cx, int cy, double lx, double ly, const double* p, double& wx, double& wy) {
    if constexpr (NP == 6) {
        wx = static_cast<double>(cx) + lx + p[0] + p[2] * lx + p[3] * ly;
        wy = static_cast<double>(cy) + ly + p[1] + p[4] * lx + p[5] * ly;
    } else {
        const double x2 = lx * lx * 0.5, y2 = ly * ly * 0.5, xy = lx * ly;
        wx = static_cast<double>(cx) + lx + p[0] + p[2] * lx + p[3] * ly + p[6] * x2 + p[7] * xy + p[8] * y2;
        wy = static_cast<double>(cy) + ly + p[1] + p[4] * lx + p[5] * ly + p[9] * x2 + p[10] * xy + p[11] * y2;
    }
}

void store_params(orc_poi_result& res, const double* p, int np) {
    for (int k = 0; k < 6; ++k) res.p[k] = p[k];
    for (int k = 0; k < 6; ++k) res.q[k] = np == 12 ? p[6 + k] : 0.0;
}

struct Sample { double lx, ly, ref, refn, sd[12]; };

// ICGN, first order (NP = 6) or second order (NP = 12), ZNSSD or SSD:
//   icgn.cpp:446-627   first-order ZNSSD      icgn.cpp:832-988    first-order SSD
//   icgn.cpp:1168-1362 second-order ZNSSD     icgn.cpp:1576-1739  second-order SSD
// SSD drops the normalisation (raw residual f - g, Hessian and gradient without the 2/|f|
// factors); second order needs 12 samples and updates through the warp matrix (ic_update2).
template <int NP>
orc_poi_result solve_icgn(const float* ref, int w, int h, const GradSource& gs, const Spline& sp,
                          const SolverCfg& cfg, double px, double py, const double* p0, double conf) {
    orc_poi_result res;
    init_result(res, p0, conf);
    if (w <= 0 || h <= 0 || cfg.radius < 1 || cfg.max_iter < 0) return res;
    const int cx = static_cast<int>(std::round(px)), cy = static_cast<int>(std::round(py));
    const int r = cfg.radius;
    const bool masked = cfg.roi != nullptr;
    if (masked ? !masked_centre_ok(cfg, w, h, cx, cy) : (cx - r < 0 || cy - r < 0 || cx + r >= w || cy + r >= h))
        return res;
    std::vector<Sample> s;
    s.reserve(static_cast<std::size_t>((2 * r + 1) * (2 * r + 1)));
    double mean = 0.0;
    int full = 0;
    for (int dy = -r; dy <= r; ++dy)
        for (int dx = -r; dx <= r; ++dx) {
            if (dx * dx + dy * dy > r * r) continue;
            ++full;
            if (masked && !masked_keep(cfg, w, h, cx + dx, cy + dy)) continue;
            Sample q;
            q.lx = dx; q.ly = dy;
            q.ref = static_cast<double>(ref[static_cast<std::size_t>(cy + dy) * w + cx + dx]);
            double gx, gy;
            gs.at(cx + dx, cy + dy, gx, gy);
            sd_row<NP>(gx, gy, q.lx, q.ly, q.sd);
            mean += q.ref;
            s.push_back(q);
        }
    if (static_cast<int>(s.size()) < (masked ? masked_min_samples(cfg, NP, full) : NP)) return res;
    const double N = static_cast<double>(s.size());
    double norm = 1.0;
    if (!cfg.ssd) {
        mean /= N;
        norm = 0.0;
        for (const auto& q : s) { const double df = q.ref - mean; norm += df * df; }
        norm = std::sqrt(norm);
        if (norm <= kEps) { res.status = kNumericalFailure; return res; }
        for (auto& q : s) q.refn = (q.ref - mean) / norm;
    }
    double H[NP][NP] = {};
    for (const auto& q : s) for (int i = 0; i < NP; ++i) for (int j = 0; j < NP; ++j) H[i][j] += q.sd[i] * q.sd[j];
    if (!cfg.ssd) {
        const double hs = 2.0 / (norm * norm);
        for (int i = 0; i < NP; ++i) for (int j = 0; j < NP; ++j) H[i][j] *= hs;
    }
    LdltN<NP> f;
    f.factor(H);
    if (!f.success() || !f.positive()) { res.status = kNumericalFailure; return res; }
    double p[NP];
    for (int i = 0; i < NP; ++i) p[i] = i < 6 ? p0[i] : 0.0;
    double corr = kInf;
    bool converged = false;
    std::vector<double> g(s.size());
    for (int it = 0; it < cfg.max_iter; ++it) {
        res.iterations = it + 1;
        double gm = 0.0;
        for (std::size_t i = 0; i < s.size(); ++i) {
            double wx, wy;
            warp_pt<NP>(cx, cy, s[i].lx, s[i].ly, p, wx, wy);
            if (!(wx >= 0.0 && wy >= 0.0 && wx <= static_cast<double>(w - 1) && wy <= static_cast<double>(h - 1))) {
                res.status = kInvalidInput;
                return res;
            }
            g[i] = sp.value(wx, wy);
            gm += g[i];
        }
        double grad[NP] = {};
        corr = 0.0;
        if (!cfg.ssd) {
            gm /= N;
            double gn = 0.0;
            for (double v : g) { const double df = v - gm; gn += df * df; }
            gn = std::sqrt(gn);
            if (gn <= kEps) { res.status = kNumericalFailure; return res; }
            for (std::size_t i = 0; i < s.size(); ++i) {
                const double nd = s[i].refn - (g[i] - gm) / gn;
                for (int k = 0; k < NP; ++k) grad[k] += nd * s[i].sd[k];
                corr += nd * nd;
            }
            for (int k = 0; k < NP; ++k) grad[k] *= 2.0 / norm;
        } else {
            for (std::size_t i = 0; i < s.size(); ++i) {
                const double rd = s[i].ref - g[i];
                for (int k = 0; k < NP; ++k) grad[k] += rd * s[i].sd[k];
                corr += rd * rd;
            }
        }
        double dp[NP];
        f.solve(grad, dp);
        for (int k = 0; k < NP; ++k) dp[k] = -dp[k];
        bool fin = true;
        for (int k = 0; k < NP; ++k) fin = fin && std::isfinite(dp[k]);
        if (!fin) { res.status = kNumericalFailure; return res; }
        double dn = 0.0;
        for (int k = 0; k < NP; ++k) dn += dp[k] * dp[k];
        dn = std::sqrt(dn);
        double pn[NP];
        if constexpr (NP == 6) ic_update(p, dp, pn);
        else ic_update2(p, dp, pn);
        for (int k = 0; k < NP; ++k) p[k] = pn[k];
        fin = true;
        for (int k = 0; k < NP; ++k) fin = fin && std::isfinite(p[k]);
        if (!fin) { res.status = kNumericalFailure; return res; }
        if (dn < cfg.thr) { converged = true; break; }
    }
    store_params(res, p, NP);
    res.correlation = corr;
    res.converged = converged ? 1 : 0;
    if (!converged && std::isfinite(corr)) converged = true;
    res.status = converged ? kSuccess : kNotConverged;
    res.valid = converged ? 1 : 0;
    return res;
}

// Forward Gauss-Newton, first or second order, ZNSSD or SSD:
//   forward_gauss_newton.cpp:188-399   first-order ZNSSD (step cap 0.5)
//   forward_gauss_newton.cpp:622-794   first-order SSD (cap 0.35; converges on the uncapped norm)
//   forward_gauss_newton.cpp:1069-1297 second-order ZNSSD (LM term 1e-4 max diag, cap 0.5)
//   forward_gauss_newton.cpp:1540-1739 second-order SSD (LM term, cap 0.35)
// SD from the deformed spline gradient through dW/dz at the sample (:44-60, :986-1019).
template <int NP>
orc_poi_result solve_fgn(const float* ref, int w, int h, const Spline& sp, const SolverCfg& cfg,
                         double px, double py, const double* p0, double conf) {
    orc_poi_result res;
    init_result(res, p0, conf);
    if (w <= 0 || h <= 0 || cfg.radius < 1 || cfg.max_iter < 0) return res;
    const int cx = static_cast<int>(std::round(px)), cy = static_cast<int>(std::round(py));
    const int r = cfg.radius;
    const bool masked = cfg.roi != nullptr;
    if (masked ? !masked_centre_ok(cfg, w, h, cx, cy) : (cx - r < 0 || cy - r < 0 || cx + r >= w || cy + r >= h))
        return res;
    std::vector<Sample> s;
    double mean = 0.0;
    int full = 0;
    for (int dy = -r; dy <= r; ++dy)
        for (int dx = -r; dx <= r; ++dx) {
            if (dx * dx + dy * dy > r * r) continue;
            ++full;
            if (masked && !masked_keep(cfg, w, h, cx + dx, cy + dy)) continue;
            Sample q;
            q.lx = dx; q.ly = dy;
            q.ref = static_cast<double>(ref[static_cast<std::size_t>(cy + dy) * w + cx + dx]);
            mean += q.ref;
            s.push_back(q);
        }
    if (static_cast<int>(s.size()) < (masked ? masked_min_samples(cfg, NP, full) : NP)) return res;
    const double N = static_cast<double>(s.size());
    double norm = 1.0;
    if (!cfg.ssd) {
        mean /= N;
        norm = 0.0;
        for (const auto& q : s) { const double df = q.ref - mean; norm += df * df; }
        norm = std::sqrt(norm);
        if (norm <= kEps) { res.status = kNumericalFailure; return res; }
        for (auto& q : s) q.refn = (q.ref - mean) / norm;
    }
    // Step cap, whether convergence is tested on the capped norm, and the damping term per route
    // (forward_gauss_newton.cpp: unmasked 367-379, 763-774, 1242-1271, 1682-1713; masked 572-584,
    // 936-948, 1485-1496, 1886-1915): the masked second-order ZNSSD route has no damping term,
    // caps at 0.3 and tests the norm before the cap; the masked first-order SSD route tests the capped one.
    const double cap = cfg.ssd ? 0.35 : (masked && NP == 12 ? 0.3 : 0.5);
    const bool test_capped = masked ? !(NP == 12 && !cfg.ssd) : !(NP == 6 && cfg.ssd);
    const bool damping = NP == 12 && (!masked || cfg.ssd);
    double p[NP];
    for (int i = 0; i < NP; ++i) p[i] = i < 6 ? p0[i] : 0.0;
    double corr = kInf;
    bool converged = false;
    std::vector<double> g(s.size());
    for (int it = 0; it < cfg.max_iter; ++it) {
        res.iterations = it + 1;
        double gm = 0.0;
        for (std::size_t i = 0; i < s.size(); ++i) {
            double wx, wy;
            warp_pt<NP>(cx, cy, s[i].lx, s[i].ly, p, wx, wy);
            if (!(wx >= 0.0 && wy >= 0.0 && wx <= static_cast<double>(w - 1) && wy <= static_cast<double>(h - 1))) {
                res.status = kInvalidInput;
                return res;
            }
            g[i] = sp.value(wx, wy);
            gm += g[i];
        }
        double gn = 1.0;
        if (!cfg.ssd) {
            gm /= N;
            gn = 0.0;
            for (double v : g) { const double df = v - gm; gn += df * df; }
            gn = std::sqrt(gn);
            if (gn <= kEps) { res.status = kNumericalFailure; return res; }
        }
        double H[NP][NP] = {};
        double grad[NP] = {};
        corr = 0.0;
        for (std::size_t i = 0; i < s.size(); ++i) {
            const double lx = s[i].lx, ly = s[i].ly;
            double wx, wy;
            warp_pt<NP>(cx, cy, lx, ly, p, wx, wy);
            double gx, gy;
            sp.gradient(wx, wy, gx, gy);
            double gxe, gye;
            if constexpr (NP == 6) {
                gxe = gx * (1.0 + p[2]) + gy * p[4];
                gye = gx * p[3] + gy * (1.0 + p[5]);
            } else {
                const double a00 = 1.0 + p[2] + p[6] * lx + p[7] * ly;
                const double a01 = p[3] + p[7] * lx + p[8] * ly;
                const double a10 = p[4] + p[9] * lx + p[10] * ly;
                const double a11 = 1.0 + p[5] + p[10] * lx + p[11] * ly;
                gxe = gx * a00 + gy * a10;
                gye = gx * a01 + gy * a11;
            }
            double sd[NP];
            sd_row<NP>(gxe, gye, lx, ly, sd);
            const double nd = cfg.ssd ? s[i].ref - g[i] : s[i].refn - (g[i] - gm) / gn;
            for (int a = 0; a < NP; ++a) { for (int b = 0; b < NP; ++b) H[a][b] += sd[a] * sd[b]; grad[a] += nd * sd[a]; }
            corr += nd * nd;
        }
        if (!cfg.ssd) {
            const double hs = 2.0 / (norm * norm);
            for (int a = 0; a < NP; ++a) for (int b = 0; b < NP; ++b) H[a][b] *= hs;
            for (int a = 0; a < NP; ++a) grad[a] *= 2.0 / norm;
        }
        if (damping) {  // forward_gauss_newton.cpp:1242-1245, 1682-1685, 1886-1889
            double dmax = H[0][0];
            for (int a = 1; a < NP; ++a) dmax = std::max(dmax, H[a][a]);
            const double lambda = 1e-4 * dmax;
            for (int a = 0; a < NP; ++a) H[a][a] += lambda;
        }
        LdltN<NP> f;
        f.factor(H);
        if (!f.success() || !f.positive()) { res.status = kNumericalFailure; return res; }
        double dp[NP];
        f.solve(grad, dp);
        bool fin = true;
        for (int k = 0; k < NP; ++k) fin = fin && std::isfinite(dp[k]);
        if (!fin) { res.status = kNumericalFailure; return res; }
        double dn = 0.0;
        for (int k = 0; k < NP; ++k) dn += dp[k] * dp[k];
        dn = std::sqrt(dn);
        const double dn_raw = dn;
        if (dn > cap) {  // forward_gauss_newton.cpp:367-371, 763-767, 1260-1264, 1700-1705
            for (int k = 0; k < NP; ++k) dp[k] *= cap / dn;
            dn = cap;
        }
        const double dn_test = test_capped ? dn : dn_raw;
        double pn[NP];
        if constexpr (NP == 6) compose_warp(p, dp, pn);
        else compose_warp2(p, dp, pn);
        for (int k = 0; k < NP; ++k) p[k] = pn[k];
        fin = true;
        for (int k = 0; k < NP; ++k) fin = fin && std::isfinite(p[k]);
        if (!fin) { res.status = kNumericalFailure; return res; }
        if (dn_test < cfg.thr) { converged = true; break; }
    }
    store_params(res, p, NP);
    res.correlation = corr;
    res.converged = converged ? 1 : 0;
    if (!converged && std::isfinite(corr)) converged = true;
    res.status = converged ? kSuccess : kNotConverged;
    res.valid = converged ? 1 : 0;
    return res;
}

// ICGNSolver / ForwardGaussNewtonSolver::solve_with_interpolators dispatch (icgn.cpp:384-405,
// forward_gauss_newton.cpp:117-142).
orc_poi_result solve_one(const float* ref, int w, int h, const GradSource& gs, const Spline& sp,
                         const SolverCfg& cfg, double px, double py, const double* p0, double conf) {
    if (cfg.optimizer == 1)
        return cfg.order == 2 ? solve_fgn<12>(ref, w, h, sp, cfg, px, py, p0, conf)
                              : solve_fgn<6>(ref, w, h, sp, cfg, px, py, p0, conf);
    return cfg.order == 2 ? solve_icgn<12>(ref, w, h, gs, sp, cfg, px, py, p0, conf)
                          : solve_icgn<6>(ref, w, h, gs, sp, cfg, px, py, p0, conf);
}

SolverCfg solver_cfg(const orc_config& c) {
    SolverCfg s{c.subset_radius, c.max_iterations, c.convergence_threshold, c.optimizer};
    s.order = c.shape_order == 2 ? 2 : 1;
    s.ssd = c.criterion == 0;
    return s;
}

bool all_finite7(const orc_poi_result& r) {  // reliability_propagation.cpp:67-75
    return finite6(r.p) && std::isfinite(r.correlation);
}

struct QueueItem {  // reliability_propagation.cpp:44-53
    double corrcoef;
    int gx, gy;
    double p[6];
    bool operator<(const QueueItem& o) const { return corrcoef > o.corrcoef; }
};

void clear_grid(orc_grid_out* out, int gw, int gh, int step) {
    const int n = gw * gh;
    for (int i = 0; i < n; ++i) {
        out->x[i] = static_cast<double>((i % gw) * step);
        out->y[i] = static_cast<double>((i / gw) * step);
        out->u[i] = out->v[i] = out->du_dx[i] = out->du_dy[i] = out->dv_dx[i] = out->dv_dy[i] = 0.0;
        out->correlation[i] = 0.0;
        out->valid[i] = 0;
        out->status[i] = kInvalidInput;
        out->iterations[i] = 0;
        out->converged[i] = 0;
        double* d2[6] = {out->d2u_dx2, out->d2u_dxdy, out->d2u_dy2, out->d2v_dx2, out->d2v_dxdy, out->d2v_dy2};
        for (double* a : d2) if (a) a[i] = 0.0;
    }
}

void store(orc_grid_out* out, int idx, const orc_poi_result& r) {
    out->u[idx] = r.p[0]; out->v[idx] = r.p[1];
    out->du_dx[idx] = r.p[2]; out->du_dy[idx] = r.p[3]; out->dv_dx[idx] = r.p[4]; out->dv_dy[idx] = r.p[5];
    out->correlation[idx] = r.correlation;
    out->valid[idx] = r.valid;
    out->status[idx] = r.status;
    out->iterations[idx] = r.iterations;
    out->converged[idx] = r.converged;
    double* d2[6] = {out->d2u_dx2, out->d2u_dxdy, out->d2u_dy2, out->d2v_dx2, out->d2v_dxdy, out->d2v_dy2};
    for (int k = 0; k < 6; ++k) if (d2[k]) d2[k][idx] = r.q[k];
}

bool roi_valid(const uint8_t* roi, int w, int h, int x, int y) {
    if (x < 0 || y < 0 || x >= w || y >= h) return false;
    return roi == nullptr || roi[static_cast<std::size_t>(y) * w + x] != 0;
}

int nearest_grid_index(int c, int step, int limit) {  // reliability_propagation.cpp:77-82
    const int idx = static_cast<int>(std::llround(static_cast<double>(c) / static_cast<double>(step)));
    return std::clamp(idx, 0, limit - 1);
}

float corr_key(double c) { return static_cast<float>(c); }

// A fixed team of host threads that runs one indexed loop at a time: the solves of one frontier
// wave or one dataflow diagonal, which read only the previous wave's results.  The calling thread
// works too; run() returns when every index is done.
class Team {
public:
    explicit Team(int n) : n_(std::max(1, n)) {
        for (int t = 1; t < n_; ++t) th_.emplace_back([this] { worker(); });
    }
    ~Team() {
        {
            std::lock_guard<std::mutex> l(mu_);
            stop_ = true;
            ++gen_;
        }
        cv_.notify_all();
        for (auto& t : th_) t.join();
    }
    void run(int count, const std::function<void(int)>& f) {
        if (n_ == 1 || count < 2) {
            for (int i = 0; i < count; ++i) f(i);
            return;
        }
        {
            std::lock_guard<std::mutex> l(mu_);
            f_ = &f;
            count_ = count;
            next_.store(0);
            active_ = n_ - 1;
            ++gen_;
        }
        cv_.notify_all();
        drain();
        std::unique_lock<std::mutex> l(mu_);
        done_.wait(l, [this] { return active_ == 0; });
        f_ = nullptr;
    }

private:
    void drain() {
        for (int i = next_.fetch_add(1); i < count_; i = next_.fetch_add(1)) (*f_)(i);
    }
    void worker() {
        std::uint64_t seen = 0;
        for (;;) {
            {
                std::unique_lock<std::mutex> l(mu_);
                cv_.wait(l, [&] { return gen_ != seen; });
                seen = gen_;
                if (stop_) return;
            }
            drain();
            std::lock_guard<std::mutex> l(mu_);
            if (--active_ == 0) done_.notify_one();
        }
    }
    int n_;
    std::vector<std::thread> th_;
    std::mutex mu_;
    std::condition_variable cv_, done_;
    const std::function<void(int)>* f_ = nullptr;
    int count_ = 0, active_ = 0;
    std::atomic<int> next_{0};
    std::uint64_t gen_ = 0;
    bool stop_ = false;
};

// reliability_propagation.cpp:130-394 (mode 1, heap order), the frontier-wave rule (mode 0) and
// the dataflow order with frontier-wave cleanup (mode 2).  Modes 0 and 2 solve the points of a
// wave (a diagonal) on `threads` host threads; the result does not depend on the thread count.
int propagate(const float* ref, int w, int h, const uint8_t* roi, const GradSource& gs, const Spline& sp,
              const orc_config& c, const orc_seed& seed, int max_solves, orc_grid_out* out, int* solves_done,
              int threads = 1) {
    int solves = 0;
    if (solves_done) *solves_done = 0;
    const int spacing = std::max(0, c.propagation_spacing);
    if (w <= 0 || h <= 0 || c.subset_radius < 1) return 0;
    const int step = spacing + 1;
    const int gw = (w + step - 1) / step, gh = (h + step - 1) / step;
    clear_grid(out, gw, gh, step);
    const int radius = c.subset_radius;
    SolverCfg scfg = solver_cfg(c);
    std::vector<uint8_t> ones;
    if (c.truncate_roi_subsets) {  // solve_with_mask (reliability_propagation.cpp:233-238, 341-347)
        if (roi == nullptr) ones.assign(static_cast<std::size_t>(w) * h, 1);
        scfg.roi = roi ? roi : ones.data();
        scfg.min_valid = c.min_valid_samples;
        scfg.ratio = c.min_valid_sample_ratio;
    }
    std::vector<uint8_t> calc(static_cast<std::size_t>(gw) * gh, 0);
    const double cutoff_corr = c.propagation_max_znssd, cutoff_disp = static_cast<double>(step);
    int computed = 0;

    const int sxr = static_cast<int>(std::round(seed.x)), syr = static_cast<int>(std::round(seed.y));
    if (sxr < 0 || syr < 0 || sxr >= w || syr >= h) return 0;
    if (!roi_valid(roi, w, h, sxr, syr)) return 0;
    const int gxs = nearest_grid_index(sxr, step, gw), gys = nearest_grid_index(syr, step, gh);
    const int sx = gxs * step, sy = gys * step;
    if (sx < 0 || sy < 0 || sx >= w || sy >= h) return 0;
    if (!roi_valid(roi, w, h, sx, sy)) return 0;
    const int sidx = gys * gw + gxs;
    orc_poi_result aligned;
    for (int k = 0; k < 6; ++k) { aligned.p[k] = seed.p[k]; aligned.q[k] = 0.0; }
    aligned.correlation = seed.correlation;
    aligned.iterations = 0; aligned.status = kSuccess; aligned.valid = 1; aligned.converged = 0;
    if (sx != sxr || sy != syr) {
        aligned = solve_one(ref, w, h, gs, sp, scfg, sx, sy, seed.p, seed.correlation);
        ++solves;
        if (!aligned.valid || aligned.status != kSuccess || !all_finite7(aligned)) { if (solves_done) *solves_done = solves; return 0; }
    }
    calc[sidx] = 1;
    store(out, sidx, aligned);
    out->valid[sidx] = 1;
    out->status[sidx] = kSuccess;
    ++computed;

    auto try_neighbor = [&](int popx, int popy, int n, int& nx, int& ny, int& nidx) -> bool {
        const int offs[4][2] = {{0, -step}, {step, 0}, {0, step}, {-step, 0}};  // up, right, down, left
        nx = popx + offs[n][0]; ny = popy + offs[n][1];
        if (nx < 0 || ny < 0 || nx >= w || ny >= h) return false;
        const int gnx = nx / step, gny = ny / step;
        if (gnx < 0 || gny < 0 || gnx >= gw || gny >= gh) return false;
        nidx = gny * gw + gnx;
        if (calc[nidx]) return false;
        if (!roi_valid(roi, w, h, nx, ny)) { calc[nidx] = 1; return false; }
        if (nx - radius < 0 || ny - radius < 0 || nx + radius >= w || ny + radius >= h) { calc[nidx] = 1; return false; }
        return true;
    };
    auto accept = [&](const orc_poi_result& r, double iu, double iv) {  // :359-368
        return r.valid && r.status == kSuccess && r.correlation < cutoff_corr &&
               std::fabs(iu - r.p[0]) < cutoff_disp && std::fabs(iv - r.p[1]) < cutoff_disp && all_finite7(r);
    };

    if (c.propagation_mode == 1) {
        std::priority_queue<QueueItem> q;
        QueueItem si;
        si.corrcoef = std::max(0.0, aligned.correlation);
        si.gx = gxs; si.gy = gys;
        for (int k = 0; k < 6; ++k) si.p[k] = aligned.p[k];
        q.push(si);
        while (!q.empty()) {
            const QueueItem it = q.top();
            q.pop();
            const int popx = it.gx * step, popy = it.gy * step;
            for (int n = 0; n < 4; ++n) {
                if (max_solves >= 0 && solves >= max_solves) { if (solves_done) *solves_done = solves; return computed; }
                int nx, ny, nidx;
                if (!try_neighbor(popx, popy, n, nx, ny, nidx)) continue;
                const double ddx = nx - popx, ddy = ny - popy;
                double p0[6];
                p0[0] = it.p[0] + it.p[2] * ddx + it.p[3] * ddy;
                p0[1] = it.p[1] + it.p[4] * ddx + it.p[5] * ddy;
                p0[2] = it.p[2]; p0[3] = it.p[3]; p0[4] = it.p[4]; p0[5] = it.p[5];
                const orc_poi_result r = solve_one(ref, w, h, gs, sp, scfg, nx, ny, p0, 0.0);
                ++solves;
                calc[nidx] = 1;
                if (accept(r, p0[0], p0[1])) {
                    store(out, nidx, r);
                    ++computed;
                    QueueItem nxt;
                    nxt.corrcoef = r.correlation;
                    nxt.gx = nx / step; nxt.gy = ny / step;
                    for (int k = 0; k < 6; ++k) nxt.p[k] = r.p[k];
                    q.push(nxt);
                }
            }
        }
    } else {
        std::vector<int> best_parent(static_cast<std::size_t>(gw) * gh, -1);
        std::vector<float> best_key(static_cast<std::size_t>(gw) * gh, 0.0f);
        std::vector<double> pp(static_cast<std::size_t>(gw) * gh * 6, 0.0);
        std::vector<double> pcorr(static_cast<std::size_t>(gw) * gh, 0.0);
        for (int k = 0; k < 6; ++k) pp[static_cast<std::size_t>(sidx) * 6 + k] = aligned.p[k];
        pcorr[sidx] = std::max(0.0, aligned.correlation);
        auto solve_from = [&](int nidx, int pidx, orc_poi_result& r, double* p0) {
            const double* pp0 = &pp[static_cast<std::size_t>(pidx) * 6];
            const int nx = (nidx % gw) * step, ny = (nidx / gw) * step;
            const double ddx = nx - (pidx % gw) * step, ddy = ny - (pidx / gw) * step;
            p0[0] = pp0[0] + pp0[2] * ddx + pp0[3] * ddy;
            p0[1] = pp0[1] + pp0[4] * ddx + pp0[5] * ddy;
            p0[2] = pp0[2]; p0[3] = pp0[3]; p0[4] = pp0[4]; p0[5] = pp0[5];
            r = solve_one(ref, w, h, gs, sp, scfg, nx, ny, p0, 0.0);
        };
        // Solves todo[i] from parent par[i] for every i on the team (each reads only accepted
        // points of earlier waves), then returns the results in todo order.
        Team team(threads);
        std::vector<orc_poi_result> res;
        std::vector<std::array<double, 6>> res_p0;
        auto solve_all = [&](const std::vector<int>& todo, const std::vector<int>& par) {
            res.assign(todo.size(), orc_poi_result{});
            res_p0.assign(todo.size(), std::array<double, 6>{});
            team.run(static_cast<int>(todo.size()),
                     [&](int i) { solve_from(todo[i], par[i], res[i], res_p0[i].data()); });
            solves += static_cast<int>(todo.size());
        };
        auto keep = [&](int nidx, const orc_poi_result& r) {
            store(out, nidx, r);
            ++computed;
            for (int k = 0; k < 6; ++k) pp[static_cast<std::size_t>(nidx) * 6 + k] = r.p[k];
            pcorr[nidx] = r.correlation;
        };
        // Frontier waves: every unclaimed, admissible 4-neighbour of the wave-w accepted set
        // is solved in wave w+1 from the parent with the lowest (float) ZNSSD, ties to the
        // lowest parent grid index.
        auto run_waves = [&](std::vector<int> frontier) {
            while (!frontier.empty()) {
                std::vector<int> next;
                for (const int pidx : frontier) {
                    const int popx = (pidx % gw) * step, popy = (pidx / gw) * step;
                    const float key = corr_key(pcorr[pidx]);
                    for (int n = 0; n < 4; ++n) {
                        int nx, ny, nidx;
                        const int offs[4][2] = {{0, -step}, {step, 0}, {0, step}, {-step, 0}};
                        nx = popx + offs[n][0]; ny = popy + offs[n][1];
                        if (nx < 0 || ny < 0 || nx >= w || ny >= h) continue;
                        nidx = (ny / step) * gw + nx / step;
                        if (best_parent[nidx] >= 0) {  // already a candidate of this wave
                            if (key < best_key[nidx] || (key == best_key[nidx] && pidx < best_parent[nidx])) {
                                best_key[nidx] = key; best_parent[nidx] = pidx;
                            }
                            continue;
                        }
                        if (!try_neighbor(popx, popy, n, nx, ny, nidx)) continue;
                        best_parent[nidx] = pidx; best_key[nidx] = key;
                        next.push_back(nidx);
                    }
                }
                std::vector<int> acc, todo, par;
                for (int nidx : next) {
                    calc[nidx] = 1;
                    if (max_solves >= 0 && solves + static_cast<int>(todo.size()) >= max_solves) continue;
                    todo.push_back(nidx);
                    par.push_back(best_parent[nidx]);
                }
                solve_all(todo, par);
                for (std::size_t i = 0; i < todo.size(); ++i) {
                    if (accept(res[i], res_p0[i][0], res_p0[i][1])) {
                        keep(todo[i], res[i]);
                        acc.push_back(todo[i]);
                    }
                }
                for (int nidx : next) best_parent[nidx] = -2;  // resolved; never a candidate again
                frontier.swap(acc);
            }
        };
        if (c.propagation_mode == 2) {
            // Dataflow order: every grid point's primary parent is one step toward the seed
            // along its dominant axis (x on ties), its secondary parent one step along the
            // other axis.  A point is solved from its primary parent if that one was accepted,
            // else from its secondary parent if accepted; otherwise it is an orphan.  Orphans
            // are then reached by frontier waves from every accepted point.
            enum : int8_t { kPend = 0, kAcc = 2, kRej = 3, kOrphan = 4 };
            std::vector<int8_t> st(static_cast<std::size_t>(gw) * gh, kPend);
            st[sidx] = kAcc;
            const int sgx = gxs, sgy = gys;
            const int maxd = std::max(sgx, gw - 1 - sgx) + std::max(sgy, gh - 1 - sgy);
            auto sgn = [](int v) { return v > 0 ? 1 : -1; };
            std::vector<int> todo, par;
            for (int d = 1; d <= maxd; ++d) {
                // the parents of diagonal d lie on diagonal d - 1: its points are independent
                todo.clear();
                par.clear();
                for (int gy = 0; gy < gh; ++gy) {
                    const int rem = d - std::abs(gy - sgy);
                    if (rem < 0) continue;
                    const int xs[2] = {sgx - rem, sgx + rem};
                    for (int t = 0; t < (rem == 0 ? 1 : 2); ++t) {
                        const int gx = xs[t];
                        if (gx < 0 || gx >= gw) continue;
                        const int nidx = gy * gw + gx;
                        const int dx = gx - sgx, dy = gy - sgy;
                        int p1, p2 = -1;
                        if (std::abs(dx) >= std::abs(dy)) {
                            p1 = gy * gw + (gx - sgn(dx));
                            if (dy != 0) p2 = (gy - sgn(dy)) * gw + gx;
                        } else {
                            p1 = (gy - sgn(dy)) * gw + gx;
                            if (dx != 0) p2 = gy * gw + (gx - sgn(dx));
                        }
                        int parent = -1;
                        if (st[p1] == kAcc) parent = p1;
                        else if (p2 >= 0 && st[p2] == kAcc) parent = p2;
                        if (parent < 0) { st[nidx] = kOrphan; continue; }
                        const int nx = gx * step, ny = gy * step;
                        const bool admissible = roi_valid(roi, w, h, nx, ny) && nx - radius >= 0 && ny - radius >= 0 &&
                                                nx + radius < w && ny + radius < h;
                        calc[nidx] = 1;
                        if (!admissible || (max_solves >= 0 && solves + static_cast<int>(todo.size()) >= max_solves)) {
                            st[nidx] = kRej;
                            continue;
                        }
                        todo.push_back(nidx);
                        par.push_back(parent);
                    }
                }
                solve_all(todo, par);
                for (std::size_t i = 0; i < todo.size(); ++i) {
                    if (accept(res[i], res_p0[i][0], res_p0[i][1])) { keep(todo[i], res[i]); st[todo[i]] = kAcc; }
                    else st[todo[i]] = kRej;
                }
            }
            std::vector<int> all_acc;
            for (int i = 0; i < gw * gh; ++i) if (st[i] == kAcc) all_acc.push_back(i);
            run_waves(all_acc);
        } else {
            run_waves(std::vector<int>{sidx});
        }
    }
    if (solves_done) *solves_done = solves;
    return computed;
}

// ---------------------------------------------------------------------------------------
// Integer search (integer_search.cpp:129-280, 333-432).
// ---------------------------------------------------------------------------------------
struct ISample { int dx, dy; double v; };
struct Cand { int u = 0, v = 0; double zncc = -kInf; };

std::vector<ISample> circ_samples(const float* ref, int w, int cx, int cy, int r, int step) {  // :60-80
    step = std::max(1, step);
    std::vector<ISample> s;
    for (int dy = -r; dy <= r; dy += step)
        for (int dx = -r; dx <= r; dx += step) {
            if (dx * dx + dy * dy > r * r) continue;
            s.push_back({dx, dy, static_cast<double>(ref[static_cast<std::size_t>(cy + dy) * w + cx + dx])});
        }
    return s;
}
// collect_masked_reference_samples (integer_search.cpp:82-108): samples inside the image and the ROI.
std::vector<ISample> circ_samples_masked(const float* ref, int w, int h, const uint8_t* roi, int cx, int cy, int r,
                                         int step) {
    step = std::max(1, step);
    std::vector<ISample> s;
    for (int dy = -r; dy <= r; dy += step)
        for (int dx = -r; dx <= r; dx += step) {
            if (dx * dx + dy * dy > r * r) continue;
            const int x = cx + dx, y = cy + dy;
            if (x < 0 || y < 0 || x >= w || y >= h || !roi[static_cast<std::size_t>(y) * w + x]) continue;
            s.push_back({dx, dy, static_cast<double>(ref[static_cast<std::size_t>(y) * w + x])});
        }
    return s;
}
int full_circle_count(int r, int step) {  // integer_search.cpp:33-45
    step = std::max(1, step);
    int n = 0;
    for (int dy = -r; dy <= r; dy += step)
        for (int dx = -r; dx <= r; dx += step) n += dx * dx + dy * dy <= r * r ? 1 : 0;
    return n;
}
int min_required_samples(int r, int step) {  // integer_search.cpp:47-50
    return std::max(12, static_cast<int>(std::ceil(0.5 * full_circle_count(r, step))));
}
double s_mean(const std::vector<ISample>& s) { double m = 0; for (auto& q : s) m += q.v; return s.empty() ? 0.0 : m / static_cast<double>(s.size()); }
double s_norm(const std::vector<ISample>& s, double m) { double n = 0; for (auto& q : s) { const double d = q.v - m; n += d * d; } return n; }

double circ_zncc(const float* def, int w, int h, const std::vector<ISample>& s, double rm, double rn, int cx, int cy, int u, int v) {  // :129-166
    if (s.empty() || rn <= kEps) return -kInf;
    double dm = 0.0;
    for (auto& q : s) {
        const int x = cx + u + q.dx, y = cy + v + q.dy;
        if (x < 0 || y < 0 || x >= w || y >= h) return -kInf;
        dm += static_cast<double>(def[static_cast<std::size_t>(y) * w + x]);
    }
    dm /= static_cast<double>(s.size());
    double num = 0.0, dn = 0.0;
    for (auto& q : s) {
        const double rd = q.v - rm;
        const double dd = static_cast<double>(def[static_cast<std::size_t>(cy + v + q.dy) * w + cx + u + q.dx]) - dm;
        num += rd * dd;
        dn += dd * dd;
    }
    if (dn <= kEps) return -kInf;
    return num / std::sqrt(rn * dn);
}

Cand search_disp(const float* def, int w, int h, const std::vector<ISample>& s, double rm, double rn,
                 int cx, int cy, int r, int minu, int maxu, int minv, int maxv, int step) {  // :168-206
    Cand best;
    step = std::max(1, step);
    for (int v = minv; v <= maxv; v += step)
        for (int u = minu; u <= maxu; u += step) {
            const int x = cx + u, y = cy + v;
            if (!(x - r >= 0 && y - r >= 0 && x + r < w && y + r < h)) continue;
            const double z = circ_zncc(def, w, h, s, rm, rn, cx, cy, u, v);
            if (z > best.zncc) { best.u = u; best.v = v; best.zncc = z; }
        }
    return best;
}

// roi != NULL: estimate_with_mask_interpolators (integer_search.cpp:447-545): the centre must be a
// ROI pixel, the samples are the ROI ones and at least min_required_samples of them.
bool integer_search(const float* ref, const float* def, int w, int h, const orc_config& c,
                    double px, double py, double& ou, double& ov, double& oz, const uint8_t* roi = nullptr) {
    const int cx = static_cast<int>(std::round(px)), cy = static_cast<int>(std::round(py));
    const int r = std::max(1, c.is_subset_radius);
    if (roi) {
        if (!(cx >= 0 && cy >= 0 && cx < w && cy < h) || !roi[static_cast<std::size_t>(cy) * w + cx]) return false;
    } else if (!(cx - r >= 0 && cy - r >= 0 && cx + r < w && cy + r < h)) {
        return false;
    }
    const auto s = roi ? circ_samples_masked(ref, w, h, roi, cx, cy, r, 1) : circ_samples(ref, w, cx, cy, r, 1);
    if (roi && static_cast<int>(s.size()) < min_required_samples(r, 1)) return false;
    const double rm = s_mean(s), rn = s_norm(s, rm);
    if (s.empty() || rn <= kEps) return false;
    const int search = std::max(0, c.is_search_radius);
    const int cstep = c.pyramid_enabled ? std::max(1, std::max(1, c.pyramid_scale)) : 1;
    const auto cs = roi ? circ_samples_masked(ref, w, h, roi, cx, cy, r, cstep) : circ_samples(ref, w, cx, cy, r, cstep);
    const double crm = s_mean(cs), crn = s_norm(cs, crm);
    Cand best;
    const bool coarse_ok = roi ? static_cast<int>(cs.size()) >= min_required_samples(r, cstep) : !cs.empty();
    if (coarse_ok && crn > kEps) {  // search_ncorr_multigrid :208-265
        const int minu = r - cx, maxu = w - 1 - r - cx, minv = r - cy, maxv = h - 1 - r - cy;
        if (!(minu > maxu || minv > maxv)) {
            const Cand coarse = search_disp(def, w, h, cs, crm, crn, cx, cy, r, minu, maxu, minv, maxv, cstep);
            if (!std::isfinite(coarse.zncc)) {
                best = coarse;
            } else {
                const int rr = std::max(std::max(std::max(1, c.pyramid_refinement_radius),
                                                 static_cast<int>(std::ceil(1.5 * static_cast<double>(r)))), cstep);
                best = search_disp(def, w, h, s, rm, rn, cx, cy, r,
                                   std::max(minu, coarse.u - rr), std::min(maxu, coarse.u + rr),
                                   std::max(minv, coarse.v - rr), std::min(maxv, coarse.v + rr), 1);
            }
        }
    }
    if (search > 0) {
        const Cand local = search_disp(def, w, h, s, rm, rn, cx, cy, r, -search, search, -search, search, 1);
        // prefer_local_when_ambiguous :267-280
        if (!std::isfinite(local.zncc)) { /* keep global */ }
        else if (!std::isfinite(best.zncc)) best = local;
        else if (local.zncc + 0.02 >= best.zncc) best = local;
    }
    if (!std::isfinite(best.zncc)) return false;
    ou = best.u; ov = best.v; oz = best.zncc;
    return true;
}

double znssd_from_zncc(double z) {  // integer_search.cpp:25-31
    if (!std::isfinite(z)) return kInf;
    return std::max(0.0, 2.0 * (1.0 - std::max(-1.0, std::min(1.0, z))));
}

// ---------------------------------------------------------------------------------------
// Seed selection (seed_selector.cpp:146-317, 388-539) with sift disabled and
// truncate_roi_subsets false (pybind never sets it).
// ---------------------------------------------------------------------------------------
struct SeedEval { double x = 0, y = 0; double p[6] = {}; double corr = 0, quality = 0, norm = 0; bool valid = false; bool passed = false; };

double texture_std(const float* ref, int w, int h, int r, int x, int y) {  // :424-452
    if (x - r < 0 || y - r < 0 || x + r >= w || y + r >= h) return 0.0;
    double sum = 0.0, sq = 0.0;
    int cnt = 0;
    for (int yy = y - r; yy <= y + r; ++yy)
        for (int xx = x - r; xx <= x + r; ++xx) {
            const double v = static_cast<double>(ref[static_cast<std::size_t>(yy) * w + xx]);
            sum += v; sq += v * v; ++cnt;
        }
    if (cnt == 0) return 0.0;
    const double m = sum / cnt;
    return std::sqrt(std::max(0.0, sq / cnt - m * m));
}

struct Pt { int x, y; };

std::vector<Pt> det_sample(const std::vector<Pt>& pts, int limit) {  // :33-47
    if (limit <= 0 || static_cast<int>(pts.size()) <= limit) return pts;
    std::vector<Pt> out;
    const double st = static_cast<double>(pts.size() - 1U) / static_cast<double>(limit - 1);
    for (int i = 0; i < limit; ++i) {
        const auto idx = static_cast<std::size_t>(std::llround(static_cast<double>(i) * st));
        out.push_back(pts[std::min(idx, pts.size() - 1U)]);
    }
    return out;
}

std::vector<std::pair<double, double>> gen_candidates(const float* ref, int w, int h, const uint8_t* roi, const orc_config& c) {  // :207-317
    std::vector<std::pair<double, double>> cands;
    const int rad = std::max(std::max(1, c.is_subset_radius), std::max(1, c.sp_subset_radius));
    const bool trunc = c.truncate_roi_subsets != 0;
    // is_candidate_margin_valid (:388-422): the search radius widens the margin when truncating,
    // and the circle of radius `rad` must then hold enough ROI pixels
    const int margin = rad + (trunc ? std::max(0, c.is_search_radius) : 0);
    auto margin_ok = [&](int x, int y) {
        if (x - margin < 0 || y - margin < 0 || x + margin >= w || y + margin >= h) return false;
        if (!trunc) return true;
        int valid = 0, full = 0;
        for (int yy = y - rad; yy <= y + rad; ++yy)
            for (int xx = x - rad; xx <= x + rad; ++xx) {
                const int dx = xx - x, dy = yy - y;
                if (dx * dx + dy * dy > rad * rad) continue;
                ++full;
                valid += roi_valid(roi, w, h, xx, yy) ? 1 : 0;
            }
        const int need = std::max(c.min_valid_samples,
                                  static_cast<int>(std::ceil(c.min_valid_sample_ratio * static_cast<double>(full))));
        return valid >= std::max(6, need);
    };
    std::vector<Pt> pts;
    if (trunc) {  // :219-229: ROI points inside the search margin (no sample count)
        for (int y = margin; y < h - margin; ++y) for (int x = margin; x < w - margin; ++x) if (roi_valid(roi, w, h, x, y)) pts.push_back({x, y});
    } else {
        for (int y = 0; y < h; ++y) for (int x = 0; x < w; ++x) if (roi_valid(roi, w, h, x, y) && margin_ok(x, y)) pts.push_back({x, y});
    }
    if (pts.empty()) for (int y = 0; y < h; ++y) for (int x = 0; x < w; ++x) if (roi_valid(roi, w, h, x, y)) pts.push_back({x, y});
    if (pts.empty()) return cands;
    const int requested = std::max(1, c.seed_count);
    const auto sp = det_sample(pts, std::max(1, c.kmeans_sample_limit));
    const int tr = std::max(1, c.is_subset_radius);
    if (requested == 1) {
        double best = -1.0; Pt bp{}; bool found = false;
        for (const auto& p : sp) {
            if (!margin_ok(p.x, p.y)) continue;
            const double t = texture_std(ref, w, h, tr, p.x, p.y);
            if (!found || t > best) { best = t; bp = p; found = true; }
        }
        if (found) cands.emplace_back(bp.x, bp.y);
        return cands;
    }
    // initialize_centers :49-67
    const int count = std::min(requested, static_cast<int>(sp.size()));
    std::vector<double> cxs, cys;
    const double st = count == 1 ? 0.0 : static_cast<double>(sp.size() - 1U) / static_cast<double>(count - 1);
    for (int i = 0; i < count; ++i) {
        const auto idx = static_cast<std::size_t>(std::llround(static_cast<double>(i) * st));
        const auto& p = sp[std::min(idx, sp.size() - 1U)];
        cxs.push_back(p.x); cys.push_back(p.y);
    }
    // run_kmeans :69-108
    const int iters = std::max(0, c.kmeans_iterations);
    std::vector<double> sx(count), sy(count);
    std::vector<int> cnt(count);
    for (int it = 0; it < iters; ++it) {
        std::fill(sx.begin(), sx.end(), 0.0); std::fill(sy.begin(), sy.end(), 0.0); std::fill(cnt.begin(), cnt.end(), 0);
        for (const auto& p : sp) {
            std::size_t best = 0; double bd = kInf;
            for (int i = 0; i < count; ++i) {
                const double dx = p.x - cxs[i], dy = p.y - cys[i];
                const double d2 = dx * dx + dy * dy;
                if (d2 < bd) { bd = d2; best = static_cast<std::size_t>(i); }
            }
            sx[best] += p.x; sy[best] += p.y; ++cnt[best];
        }
        for (int i = 0; i < count; ++i) if (cnt[i] > 0) { cxs[i] = sx[i] / cnt[i]; cys[i] = sy[i] / cnt[i]; }
    }
    for (int i = 0; i < count; ++i) {
        const int rx = static_cast<int>(std::llround(cxs[i])), ry = static_cast<int>(std::llround(cys[i]));
        if (roi_valid(roi, w, h, rx, ry) && margin_ok(rx, ry) && texture_std(ref, w, h, tr, rx, ry) >= c.min_texture_std) {
            cands.emplace_back(rx, ry);
            continue;
        }
        std::vector<std::size_t> order(sp.size());
        std::iota(order.begin(), order.end(), 0U);
        const double ccx = cxs[i], ccy = cys[i];
        std::sort(order.begin(), order.end(), [&](std::size_t l, std::size_t r) {
            const double lx = sp[l].x - ccx, ly = sp[l].y - ccy, qx = sp[r].x - ccx, qy = sp[r].y - ccy;
            return lx * lx + ly * ly < qx * qx + qy * qy;
        });
        const std::size_t lim = std::min<std::size_t>(50U, order.size());
        double best = -1.0; Pt bp = sp[order.front()];
        for (std::size_t k = 0; k < lim; ++k) {
            const auto& p = sp[order[k]];
            const double t = texture_std(ref, w, h, tr, p.x, p.y);
            if (t > best) { best = t; bp = p; }
        }
        cands.emplace_back(bp.x, bp.y);
    }
    return cands;
}

bool select_seed(const float* ref, const float* def, int w, int h, const uint8_t* roi, const orc_config& c,
                 orc_seed& seed, std::vector<std::pair<double, double>>* cands_out) {
    seed = orc_seed{};
    seed.found = 0;
    const auto cands = gen_candidates(ref, w, h, roi, c);
    if (cands_out) *cands_out = cands;
    if (c.sift_enabled) return false;  // sift_initializer.cpp:53-55 without OpenCV: no match, no seed
    // Lazy, non-prefiltered deformed spline (seed_selector.cpp:166-173).
    const int border = std::max(3, c.border);
    std::vector<double> lazy;
    Spline sp;
    const bool refine = c.sp_enabled != 0;
    if (refine) {
        lazy.resize(static_cast<std::size_t>(w + 2 * border) * (h + 2 * border));
        form_coefficients(def, w, h, c.degree, border, false, lazy.data());
        sp.init(lazy.data(), w, h, c.degree, border);
    }
    GradSource gs{ref, w, h, nullptr, nullptr};  // reference interpolator is empty -> central differences
    // subset_initializer.cpp:165-177: the subpixel solver is first-order ICGN with the configured objective
    SolverCfg scfg{std::max(1, c.sp_subset_radius), std::max(0, c.sp_max_iterations), c.sp_convergence_threshold, 0};
    scfg.ssd = c.criterion == 0;
    // truncate_roi_subsets: masked integer search and masked refinement (subset_initializer.cpp:140-149, 206-245)
    std::vector<uint8_t> ones;
    const uint8_t* mask = nullptr;
    if (c.truncate_roi_subsets) {
        if (roi == nullptr) ones.assign(static_cast<std::size_t>(w) * h, 1);
        mask = roi ? roi : ones.data();
        scfg.roi = mask;
        scfg.min_valid = c.min_valid_samples;
        scfg.ratio = c.min_valid_sample_ratio;
    }
    SeedEval best;
    bool found = false;
    for (const auto& cd : cands) {
        SeedEval ev;
        ev.x = cd.first; ev.y = cd.second;
        double iu, iv, iz;
        if (!integer_search(ref, def, w, h, c, cd.first, cd.second, iu, iv, iz, mask)) continue;
        double p[6] = {iu, iv, 0, 0, 0, 0};
        double conf = znssd_from_zncc(iz), quality = conf;
        if (refine) {  // subset_initializer.cpp:152-204
            const orc_poi_result r = solve_icgn<6>(ref, w, h, gs, sp, scfg, cd.first, cd.second, p, conf);
            if (r.valid && r.status == kSuccess) {
                for (int k = 0; k < 6; ++k) p[k] = r.p[k];
                conf = r.correlation;
                quality = r.correlation;
            }
        }
        if (!std::isfinite(p[0]) || !std::isfinite(p[1]) || !std::isfinite(conf)) continue;  // :507-512
        for (int k = 0; k < 6; ++k) ev.p[k] = p[k];
        ev.corr = conf;
        ev.quality = quality;
        ev.norm = std::hypot(p[0], p[1]);
        ev.passed = quality <= c.seed_max_znssd;
        ev.valid = true;
        if (ev.valid && ev.passed && ev.norm >= c.min_displacement_norm) {
            bool better = !found;
            if (found) {  // seed_is_better :110-133 (ZNSSD metric)
                if (ev.quality < best.quality - 1e-9) better = true;
                else if (ev.quality > best.quality + 1e-9) better = false;
                else better = ev.norm > best.norm;
            }
            if (better) { best = ev; found = true; }
        }
    }
    if (!found) return false;
    seed.x = best.x; seed.y = best.y;
    for (int k = 0; k < 6; ++k) seed.p[k] = best.p[k];
    seed.correlation = best.corr;
    seed.found = 1;
    return true;
}

int mirror_index(int i, int n) {  // padding.cpp:11-24
    if (n <= 1) return 0;
    while (i < 0 || i >= n) i = i < 0 ? -i - 1 : 2 * n - i - 1;
    return i;
}

}  // namespace

extern "C" {

void orc_config_default(orc_config* c) {
    std::memset(c, 0, sizeof(*c));
    c->subset_radius = 15; c->max_iterations = 30; c->convergence_threshold = 1e-3;
    c->optimizer = 0; c->shape_order = 1; c->criterion = 1; c->degree = 5; c->border = 3;
    c->propagation_spacing = 5; c->propagation_max_znssd = 0.5;
    c->is_subset_radius = 10; c->is_search_radius = 30; c->sift_enabled = 0; c->pyramid_enabled = 1;
    c->pyramid_scale = 4; c->pyramid_refinement_radius = 4;
    c->sp_enabled = 1; c->sp_subset_radius = 15; c->sp_max_iterations = 30; c->precision = 0;
    c->sp_convergence_threshold = 1e-3;
    c->seed_count = 256; c->kmeans_iterations = 20; c->seed_max_znssd = 0.2;
    c->min_displacement_norm = 0.0; c->min_texture_std = 0.0; c->kmeans_sample_limit = 20000;
    c->propagation_mode = 1;
    c->truncate_roi_subsets = 0; c->min_valid_samples = 12; c->min_valid_sample_ratio = 0.5;
    c->staging = 0; c->pad_ = 0;
}

double orc_bspline_basis(double x, int r, int d) { return valid_degree(d) ? basis(x, r, d) : kNaN; }

int orc_bspline_qk(int d, double* qk) {
    if (!valid_degree(d)) return -1;
    build_qk(d, qk);
    return 0;
}

int orc_prefilter(const float* image, int w, int h, int d, int border, int exact, double* coeffs) {
    if (!valid_degree(d) || w <= 0 || h <= 0 || !image || !coeffs) return -1;
    form_coefficients(image, w, h, d, border, exact != 0, coeffs);
    return 0;
}

double orc_interp_value(const double* coeffs, int w, int h, int d, int border, double x, double y) {
    Spline sp;
    sp.init(coeffs, w, h, d, border);
    return sp.value(x, y);
}

void orc_interp_gradient(const double* coeffs, int w, int h, int d, int border, double x, double y, double* gx, double* gy) {
    Spline sp;
    sp.init(coeffs, w, h, d, border);
    sp.gradient(x, y, *gx, *gy);
}

void orc_reference_gradient(const float* img, int w, int h, double* gx, double* gy) {
    GradSource gs{img, w, h, nullptr, nullptr};
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) gs.at(x, y, gx[static_cast<std::size_t>(y) * w + x], gy[static_cast<std::size_t>(y) * w + x]);
}

int orc_solve_pois(const float* ref, int w, int h, const double* ref_gx, const double* ref_gy,
                   const double* coeffs, int d, int border, const orc_config* cfg,
                   int n, const double* xy, const double* p0, const double* conf0, orc_poi_result* out) {
    if (!valid_degree(d)) return -1;
    Spline sp;
    sp.init(coeffs, w, h, d, border);
    GradSource gs{ref, w, h, ref_gx, ref_gy};
    const SolverCfg scfg = solver_cfg(*cfg);
    for (int i = 0; i < n; ++i)
        out[i] = solve_one(ref, w, h, gs, sp, scfg, xy[2 * i], xy[2 * i + 1], p0 + 6 * i, conf0 ? conf0[i] : 0.0);
    return 0;
}

int orc_solve_pois_masked(const float* ref, int w, int h, const uint8_t* roi, const double* ref_gx,
                          const double* ref_gy, const double* coeffs, int d, int border, const orc_config* cfg,
                          int n, const double* xy, const double* p0, const double* conf0, orc_poi_result* out) {
    if (!valid_degree(d)) return -1;
    Spline sp;
    sp.init(coeffs, w, h, d, border);
    GradSource gs{ref, w, h, ref_gx, ref_gy};
    std::vector<uint8_t> ones;
    if (!roi) ones.assign(static_cast<std::size_t>(w) * h, 1);
    SolverCfg scfg = solver_cfg(*cfg);
    scfg.roi = roi ? roi : ones.data();
    scfg.min_valid = cfg->min_valid_samples;
    scfg.ratio = cfg->min_valid_sample_ratio;
    for (int i = 0; i < n; ++i)
        out[i] = solve_one(ref, w, h, gs, sp, scfg, xy[2 * i], xy[2 * i + 1], p0 + 6 * i, conf0 ? conf0[i] : 0.0);
    return 0;
}

void orc_grid_dims(int w, int h, int spacing, int* gw, int* gh) {
    const int step = std::max(0, spacing) + 1;
    *gw = (w + step - 1) / step;
    *gh = (h + step - 1) / step;
}

int orc_propagate(const float* ref, int w, int h, const uint8_t* roi, const double* ref_gx, const double* ref_gy,
                  const double* coeffs, const orc_config* cfg, const orc_seed* seed, int max_solves,
                  orc_grid_out* out, int* solves_done) {
    return orc_propagate_threads(ref, w, h, roi, ref_gx, ref_gy, coeffs, cfg, seed, max_solves, out, solves_done, 1);
}

int orc_propagate_threads(const float* ref, int w, int h, const uint8_t* roi, const double* ref_gx,
                          const double* ref_gy, const double* coeffs, const orc_config* cfg, const orc_seed* seed,
                          int max_solves, orc_grid_out* out, int* solves_done, int threads) {
    Spline sp;
    sp.init(coeffs, w, h, cfg->degree, cfg->border);
    GradSource gs{ref, w, h, ref_gx, ref_gy};
    return propagate(ref, w, h, roi, gs, sp, *cfg, *seed, max_solves, out, solves_done, threads);
}

int orc_integer_search(const float* ref, const float* def, int w, int h, const orc_config* cfg,
                       double px, double py, double* u, double* v, double* zncc) {
    return integer_search(ref, def, w, h, *cfg, px, py, *u, *v, *zncc) ? 1 : 0;
}

int orc_integer_search_masked(const float* ref, const float* def, int w, int h, const uint8_t* roi,
                              const orc_config* cfg, double px, double py, double* u, double* v, double* zncc) {
    return integer_search(ref, def, w, h, *cfg, px, py, *u, *v, *zncc, roi) ? 1 : 0;
}

int orc_select_seed(const float* ref, const float* def, int w, int h, const uint8_t* roi, const orc_config* cfg,
                    orc_seed* seed, double* cand_xy, int cand_cap, int* n_candidates) {
    std::vector<std::pair<double, double>> cands;
    const bool ok = select_seed(ref, def, w, h, roi, *cfg, *seed, &cands);
    if (n_candidates) *n_candidates = static_cast<int>(cands.size());
    if (cand_xy)
        for (int i = 0; i < static_cast<int>(cands.size()) && i < cand_cap; ++i) { cand_xy[2 * i] = cands[i].first; cand_xy[2 * i + 1] = cands[i].second; }
    return ok ? 1 : 0;
}

int orc_subset_padding(const orc_config* c) {  // padding.cpp:28-36
    const int ir = std::max(1, c->is_subset_radius), sr = std::max(1, c->sp_subset_radius);
    return std::max(0, c->is_search_radius) + std::max(c->subset_radius, std::max(ir, sr)) + std::max(0, c->border);
}

void orc_truncated_grid_dims(int w, int h, const orc_config* c, int* gw, int* gh) {
    const int pad = c->truncate_roi_subsets ? orc_subset_padding(c) : 0;
    const int step = std::max(0, c->propagation_spacing) + 1;
    auto count = [&](int n) {  // grid points gx * step - pad inside [0, n)
        if (n <= 0) return 0;
        const int lo = (pad + step - 1) / step, hi = (n - 1 + pad) / step;
        return std::max(0, hi - lo + 1);
    };
    *gw = count(w);
    *gh = count(h);
}

int orc_subset_compute(const float* ref, const float* def, int w, int h, const uint8_t* roi,
                       const orc_config* cfg, orc_grid_out* out, orc_seed* seed_out) {
    if (w <= 0 || h <= 0 || !ref || !def) return 0;
    if (cfg->truncate_roi_subsets) {
        // subset_dic.cpp:53-104: mirror-padded images, zero-padded ROI, the padded result cropped
        const int pad = orc_subset_padding(cfg);
        const int pw = w + 2 * pad, ph = h + 2 * pad;
        std::vector<float> pr(static_cast<std::size_t>(pw) * ph), pd(pr.size());
        std::vector<uint8_t> pm(pr.size(), 0);
        for (int y = 0; y < ph; ++y)
            for (int x = 0; x < pw; ++x) {
                const std::size_t s = static_cast<std::size_t>(mirror_index(y - pad, h)) * w + mirror_index(x - pad, w);
                pr[static_cast<std::size_t>(y) * pw + x] = ref[s];
                pd[static_cast<std::size_t>(y) * pw + x] = def[s];
            }
        for (int y = 0; y < h; ++y)
            for (int x = 0; x < w; ++x)
                pm[static_cast<std::size_t>(y + pad) * pw + x + pad] = roi ? (roi[static_cast<std::size_t>(y) * w + x] != 0) : 1;
        orc_config c = *cfg;
        c.truncate_roi_subsets = 1;
        int gw, gh;
        orc_grid_dims(pw, ph, c.propagation_spacing, &gw, &gh);
        const std::size_t n = static_cast<std::size_t>(gw) * gh;
        std::vector<double> d[16];
        for (auto& a : d) a.assign(n, 0.0);
        std::vector<uint8_t> valid(n), conv(n);
        std::vector<int8_t> status(n);
        std::vector<int32_t> iters(n);
        orc_grid_out t{d[0].data(), d[1].data(), d[2].data(), d[3].data(), d[4].data(), d[5].data(), d[6].data(),
                       d[7].data(), d[8].data(), valid.data(), status.data(), iters.data(), conv.data(),
                       d[9].data(), d[10].data(), d[11].data(), d[12].data(), d[13].data(), d[14].data()};
        orc_seed seed;
        const bool found = select_seed(pr.data(), pd.data(), pw, ph, pm.data(), c, seed, nullptr);
        if (found) { seed.x -= pad; seed.y -= pad; }
        if (seed_out) *seed_out = seed;
        if (!found) return 0;
        seed.x += pad; seed.y += pad;
        const int border = std::max(3, c.border);
        std::vector<double> coeffs(static_cast<std::size_t>(pw + 2 * border) * (ph + 2 * border));
        form_coefficients(pd.data(), pw, ph, c.degree, border, true, coeffs.data());
        std::vector<double> gx(pr.size()), gy(pr.size());
        orc_reference_gradient(pr.data(), pw, ph, gx.data(), gy.data());
        Spline sp;
        sp.init(coeffs.data(), pw, ph, c.degree, border);
        GradSource gs{pr.data(), pw, ph, gx.data(), gy.data()};
        if (propagate(pr.data(), pw, ph, pm.data(), gs, sp, c, seed, -1, &t, nullptr) == 0) return 0;
        int k = 0;
        for (std::size_t i = 0; i < n; ++i) {
            const double x = t.x[i] - pad, y = t.y[i] - pad;
            if (x < 0.0 || y < 0.0 || x >= w || y >= h) continue;
            out->x[k] = x; out->y[k] = y;
            out->u[k] = t.u[i]; out->v[k] = t.v[i];
            out->du_dx[k] = t.du_dx[i]; out->du_dy[k] = t.du_dy[i]; out->dv_dx[k] = t.dv_dx[i]; out->dv_dy[k] = t.dv_dy[i];
            out->correlation[k] = t.correlation[i];
            out->valid[k] = t.valid[i]; out->status[k] = t.status[i]; out->iterations[k] = t.iterations[i];
            out->converged[k] = t.converged[i];
            double* src2[6] = {t.d2u_dx2, t.d2u_dxdy, t.d2u_dy2, t.d2v_dx2, t.d2v_dxdy, t.d2v_dy2};
            double* dst2[6] = {out->d2u_dx2, out->d2u_dxdy, out->d2u_dy2, out->d2v_dx2, out->d2v_dxdy, out->d2v_dy2};
            for (int j = 0; j < 6; ++j) if (dst2[j]) dst2[j][k] = src2[j][i];
            ++k;
        }
        return k;
    }
    orc_seed seed;
    if (!select_seed(ref, def, w, h, roi, *cfg, seed, nullptr)) { if (seed_out) *seed_out = seed; return 0; }
    if (seed_out) *seed_out = seed;
    const int border = std::max(3, cfg->border);
    std::vector<double> coeffs(static_cast<std::size_t>(w + 2 * border) * (h + 2 * border));
    form_coefficients(def, w, h, cfg->degree, border, true, coeffs.data());
    std::vector<double> gx(static_cast<std::size_t>(w) * h), gy(static_cast<std::size_t>(w) * h);
    orc_reference_gradient(ref, w, h, gx.data(), gy.data());
    Spline sp;
    sp.init(coeffs.data(), w, h, cfg->degree, border);
    GradSource gs{ref, w, h, gx.data(), gy.data()};
    const int computed = propagate(ref, w, h, roi, gs, sp, *cfg, seed, -1, out, nullptr);
    if (computed == 0) return 0;
    int gw, gh;
    orc_grid_dims(w, h, cfg->propagation_spacing, &gw, &gh);
    return gw * gh;
}

}  // extern "C"
