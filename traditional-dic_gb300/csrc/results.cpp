// Result files of the subset workflow written natively: the displacement CSV of
// python/traditional_dic/workflows/subset_2d.py:34-54 (save_subset_csv), byte for byte.
//
// The reference writes each row with Python's csv module, numbers through str(): a float64 as the
// shortest decimal string that reads back to the same double (Python's repr), in positional
// notation for decimal exponents -4 .. 15 (with ".0" when there is no fractional digit) and in
// scientific notation otherwise ("1e-05", "1.5e+16", at least two exponent digits); `valid` as
// the integer 0 or 1.  The shortest digits come from std::to_chars, which gives the shortest
// round-trip representation; the layout rules are Python's.  Rows are formatted on every host
// thread in chunks and written in order.
#include "tdic_internal.cuh"

#include <algorithm>
#include <atomic>
#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

namespace tdic {

// str() of a Python float (float_repr_style "short"), appended to `out`.
void append_py_float(std::string& out, double v) {
    if (std::isnan(v)) { out += "nan"; return; }
    if (std::isinf(v)) { out += v < 0 ? "-inf" : "inf"; return; }
    if (v == 0.0) { out += std::signbit(v) ? "-0.0" : "0.0"; return; }
    char buf[64];
    const auto r = std::to_chars(buf, buf + sizeof(buf), v, std::chars_format::scientific);
    // buf: [-]d[.ddd]e(+|-)XX
    const char* p = buf;
    const char* end = r.ptr;
    if (*p == '-') { out += '-'; ++p; }
    std::string digits;
    while (p < end && *p != 'e') {
        if (*p != '.') digits += *p;
        ++p;
    }
    const int exp = std::atoi(std::string(p + 1, end).c_str());  // value = d.ddd x 10^exp
    const int nd = static_cast<int>(digits.size());
    if (exp >= -4 && exp < 16) {
        if (exp >= 0) {
            if (nd <= exp + 1) {
                out += digits;
                out.append(static_cast<size_t>(exp + 1 - nd), '0');
                out += ".0";
            } else {
                out.append(digits, 0, static_cast<size_t>(exp + 1));
                out += '.';
                out.append(digits, static_cast<size_t>(exp + 1), std::string::npos);
            }
        } else {
            out += "0.";
            out.append(static_cast<size_t>(-exp - 1), '0');
            out += digits;
        }
    } else {
        out += digits[0];
        if (nd > 1) {
            out += '.';
            out.append(digits, 1, std::string::npos);
        }
        out += 'e';
        out += exp < 0 ? '-' : '+';
        const int a = exp < 0 ? -exp : exp;
        if (a < 10) out += '0';
        out += std::to_string(a);
    }
}

}  // namespace tdic

namespace {

// Host copies of the columns a CSV needs (from host or device arrays).
struct Columns {
    std::vector<std::vector<double>> d;  // x y u v du_dx du_dy dv_dx dv_dy correlation
    std::vector<uint8_t> valid;
};

void gather(const tdic_grid_out& g, tdic_memory mem, int32_t n, Columns& c) {
    const double* src[9] = {g.x, g.y, g.u, g.v, g.du_dx, g.du_dy, g.dv_dx, g.dv_dy, g.correlation};
    for (const double* s : src) TDIC_REQUIRE(s != nullptr, TDIC_INVALID_ARG, "subset CSV: every column is needed");
    TDIC_REQUIRE(g.valid != nullptr, TDIC_INVALID_ARG, "subset CSV: every column is needed");
    c.d.assign(9, std::vector<double>(static_cast<size_t>(n)));
    c.valid.resize(static_cast<size_t>(n));
    for (int k = 0; k < 9; ++k) {
        if (mem == TDIC_DEVICE)
            TDIC_CUDA_TRY(cudaMemcpy(c.d[k].data(), src[k], sizeof(double) * n, cudaMemcpyDeviceToHost));
        else
            std::memcpy(c.d[k].data(), src[k], sizeof(double) * n);
    }
    if (mem == TDIC_DEVICE) TDIC_CUDA_TRY(cudaMemcpy(c.valid.data(), g.valid, n, cudaMemcpyDeviceToHost));
    else std::memcpy(c.valid.data(), g.valid, n);
}

void write_csv(const char* path, const Columns& c, int32_t n) {
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const int chunks = static_cast<int>(std::min<long long>(hw * 4, std::max<long long>(1, n / 4096)));
    std::vector<std::string> parts(chunks);
    auto work = [&](int t) {
        const long long lo = static_cast<long long>(n) * t / chunks, hi = static_cast<long long>(n) * (t + 1) / chunks;
        std::string& s = parts[t];
        s.reserve(static_cast<size_t>(hi - lo) * 160);
        for (long long i = lo; i < hi; ++i) {
            for (int k = 0; k < 9; ++k) {
                tdic::append_py_float(s, c.d[k][i]);
                s += ',';
            }
            s += c.valid[i] ? '1' : '0';
            s += "\r\n";  // csv.writer's default line terminator
        }
    };
    {
        std::vector<std::thread> th;
        const int nt = static_cast<int>(std::min<unsigned>(hw, static_cast<unsigned>(chunks)));
        std::atomic<int> next{0};
        for (int t = 0; t < nt; ++t)
            th.emplace_back([&] {
                for (int k = next++; k < chunks; k = next++) work(k);
            });
        for (auto& x : th) x.join();
    }
    FILE* f = std::fopen(path, "wb");
    TDIC_REQUIRE(f != nullptr, TDIC_INVALID_ARG, std::string("subset CSV: cannot open ") + path);
    const char* header = "x,y,u,v,du_dx,du_dy,dv_dx,dv_dy,correlation,valid\r\n";
    bool ok = std::fwrite(header, 1, std::strlen(header), f) == std::strlen(header);
    for (const auto& s : parts) ok = ok && std::fwrite(s.data(), 1, s.size(), f) == s.size();
    ok = (std::fclose(f) == 0) && ok;
    TDIC_REQUIRE(ok, TDIC_INVALID_ARG, std::string("subset CSV: write failed for ") + path);
}

}  // namespace

namespace tdic {

void write_subset_csv(const char* path, const tdic_grid_out& grid, tdic_memory memory, int32_t n) {
    TDIC_REQUIRE(path != nullptr && n >= 0, TDIC_INVALID_ARG, "subset CSV: null path or negative size");
    Columns c;
    gather(grid, memory, n, c);
    write_csv(path, c, n);
}

}  // namespace tdic
