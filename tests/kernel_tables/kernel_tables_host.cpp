// CPU check of the mixed passes' kernel function (sphexa_gb300/csrc/kernel_tables.hpp): the cubic
// pieces evaluated in FP32 exactly as the device lookup does (x = v * intervals / 2, k = int(x),
// Horner with fmaf) against the closed form of sinc^n and its derivative, and against the FP64
// linear interpolant on the reference's 20000-point table that the FP64 passes use.
#include <cmath>
#include <vector>

#include "kernel_tables.hpp"

using namespace sphgb::tables;

namespace {

float hermEval32(const std::vector<float>& c, int intervals, float v)
{
    const float x = v * (0.5f * float(intervals));
    const int k = int(x);
    if (k >= intervals) return 0.f;
    const float t = x - float(k);
    const float* q = c.data() + 4 * k;
    return std::fmaf(std::fmaf(std::fmaf(q[3], t, q[2]), t, q[1]), t, q[0]);
}

double linear(const std::vector<double>& tab, double v)
{
    const int n = int(tab.size());
    const double dx = 2.0 / (n - 1);
    const double x = v / dx;
    const int k = int(x);
    if (k >= n - 1) return 0.0;
    return tab[k] + (tab[k + 1] - tab[k]) * (x - k);
}

}  // namespace

// out: [0] max |W_cubic32 - W| / max W, [1] max |W_cubic32 - W_linear64| / max W,
//      [2] max |dW_cubic32 - dW| / max |dW|, [3] max |dW_cubic32 - dW_linear64| / max |dW|
extern "C" int kt_errors(double n, int intervals, int samples, double* out)
{
    std::vector<float> hw, hd;
    hermitePieces(n, intervals, hw, hd);
    const int tableSize = 20000;
    std::vector<double> wl(tableSize), dl(tableSize);
    for (int i = 0; i < tableSize; ++i) {
        const double v = i * (2.0 / (tableSize - 1));
        wl[i] = std::pow(sincStd(v), n);
        dl[i] = n * std::pow(sincStd(v), n - 1) * sincStdDeriv(v);
    }
    double e[4] = {0, 0, 0, 0}, wMax = 0, dMax = 0;
    for (int s = 0; s < samples; ++s) {
        const float v32 = float(2.0 * (s + 0.5) / samples);
        const double v = double(v32);
        double sv, s1, s2;
        sincDerivs(v, sv, s1, s2);
        sv = std::max(sv, 0.0);
        const double w = std::pow(sv, n), dw = n * std::pow(sv, n - 1) * s1;
        const double wc = hermEval32(hw, intervals, v32), dc = hermEval32(hd, intervals, v32);
        wMax = std::max(wMax, std::fabs(w));
        dMax = std::max(dMax, std::fabs(dw));
        e[0] = std::max(e[0], std::fabs(wc - w));
        e[1] = std::max(e[1], std::fabs(wc - linear(wl, v)));
        e[2] = std::max(e[2], std::fabs(dc - dw));
        e[3] = std::max(e[3], std::fabs(dc - linear(dl, v)));
    }
    out[0] = e[0] / wMax;
    out[1] = e[1] / wMax;
    out[2] = e[2] / dMax;
    out[3] = e[3] / dMax;
    return 0;
}
