// Host-side construction of the kernel function's tables: the values the reference tabulates
// (sph/include/sph/sph_kernel_tables.hpp:30-157) and the cubic pieces of the mixed passes.  Plain
// C++ (no CUDA), so that a CPU test can check the pieces against the closed form and against the
// reference's linear interpolant.
#pragma once

#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

namespace sphgb::tables {

// sinc(pi/2 v) and its derivative (sph/include/sph/kernels.hpp:35-61)
inline double sincStd(double v)
{
    if (v == 0.0) return 1.0;
    const double pv = M_PI_2 * v;
    return std::sin(pv) / pv;
}
inline double sincStdDeriv(double v)
{
    if (v == 0.0) return 0.0;
    const double pv = M_PI_2 * v;
    const double s = std::sin(pv) / pv;
    return s * M_PI_2 * ((std::cos(pv) / std::sin(pv)) - 1.0 / pv);
}

// sinc and its first two derivatives in v (x = pi v / 2), by series below x = 1e-2
inline void sincDerivs(double v, double& s, double& s1, double& s2)
{
    const double a = M_PI_2, x = a * v;
    if (x < 1e-2) {
        const double x2 = x * x;
        s = 1.0 - x2 / 6.0 + x2 * x2 / 120.0 - x2 * x2 * x2 / 5040.0;
        s1 = a * x * (-1.0 / 3.0 + x2 / 30.0 - x2 * x2 / 840.0);
        s2 = a * a * (-1.0 / 3.0 + x2 / 10.0 - x2 * x2 / 168.0);
        return;
    }
    const double sn = std::sin(x), cs = std::cos(x);
    s = sn / x;
    s1 = a * (x * cs - sn) / (x * x);
    s2 = a * a * (-x * x * sn - 2.0 * x * cs + 2.0 * sn) / (x * x * x);
}

// per interval of [0, 2] the cubic Hermite piece through f and f' at both ends, as coefficients
// {c0 c1 c2 c3} of c0 + t (c1 + t (c2 + t c3)), t in [0, 1) (FP32 for the mixed passes, FP64 for the
// smooth form of the FP64 passes)
template<class R>
inline void hermiteTable(const std::vector<double>& f, const std::vector<double>& d, double dv, std::vector<R>& out)
{
    const int m = int(f.size()) - 1;
    out.resize(4 * size_t(m));
    for (int k = 0; k < m; ++k) {
        const double f0 = f[k], f1 = f[k + 1], d0 = dv * d[k], d1 = dv * d[k + 1];
        out[4 * k] = R(f0);
        out[4 * k + 1] = R(d0);
        out[4 * k + 2] = R(3.0 * (f1 - f0) - 2.0 * d0 - d1);
        out[4 * k + 3] = R(2.0 * (f0 - f1) + d0 + d1);
    }
}

// 3D normalisation of sinc^n on [0, 2] by composite Simpson with 2000 intervals, odd and even
// samples summed in ascending order (sph/include/sph/sph_kernel_tables.hpp:30-77)
inline double kernelNormalisation(double n)
{
    auto f = [n](double x) { return 4.0 * M_PI * x * x * std::pow(sincStd(x), n); };
    const int intervals = 2000;
    const double a = 0.0, b = 2.0, hs = (b - a) / double(intervals);
    std::vector<double> odd(intervals / 2), even(intervals / 2 - 1);
    for (size_t i = 0; i < odd.size(); ++i) odd[i] = f(a + double(2 * (i + 1) - 1) * hs);
    for (size_t i = 0; i < even.size(); ++i) even[i] = f(a + double(2 * (i + 1)) * hs);
    std::sort(odd.begin(), odd.end());
    std::sort(even.begin(), even.end());
    double s = hs / 3.0 *
               (f(a) + f(b) + 4.0 * std::accumulate(odd.begin(), odd.end(), 0.0) +
                2.0 * std::accumulate(even.begin(), even.end(), 0.0));
    return 1.0 / s;
}

// W = sinc^n and dW/dv as cubic pieces on `intervals` equal intervals of [0, 2] (node values and
// first derivatives from the closed form; W'' at the nodes for the pieces of dW/dv)
template<class R>
inline void hermitePieces(double n, int intervals, std::vector<R>& w32, std::vector<R>& dw32)
{
    const double dv = 2.0 / intervals;
    std::vector<double> w(intervals + 1), w1(intervals + 1), w2(intervals + 1);
    for (int k = 0; k <= intervals; ++k) {
        double sv, s1, s2;
        sincDerivs(k * dv, sv, s1, s2);
        sv = std::max(sv, 0.0);
        w[k] = std::pow(sv, n);
        w1[k] = n * std::pow(sv, n - 1) * s1;
        w2[k] = sv > 0.0 ? n * (n - 1) * std::pow(sv, n - 2) * s1 * s1 + n * std::pow(sv, n - 1) * s2 : 0.0;
    }
    hermiteTable(w, w1, dv, w32);
    hermiteTable(w1, w2, dv, dw32);
}

}  // namespace sphgb::tables
