//  filter_driver.cpp -- the design filters of PANSLBM2's template API (HeavisideFilter,
//  DensityFilter) called with three weight functors, built on the drop-in headers and the GB300
//  library: the default hat weight, a hat on a design region with the identity elsewhere (the
//  production drivers' form, recognised and built on the device), and a Gaussian weight (any
//  other functor: evaluated per (node, tap) on the host, pl_filter_weighted on the device).
//
//  usage: filter_driver <input.bin> <output.bin>
//  input:  int32 nd, lx, ly, lz; float64 R, beta; then N float64 each: s, dfdrho
//  output: for each functor (default hat, region hat, Gaussian): filtered variable, filtered
//          sensitivity, density-filtered s (3 x 3 x N float64)
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "../../dropin/src/particle/d2q9.h"
#include "../../dropin/src/particle/d3q15.h"
#include "../../dropin/src/utility/heavisidefilter.h"
#include "../../dropin/src/utility/densityfilter.h"

using namespace PANSLBM2;

template<class P>
static void run(P &p, double R, double beta, const std::vector<double> &s, const std::vector<double> &d, FILE *out,
                int ly) {
    auto put = [&](const std::vector<double> &v) { std::fwrite(v.data(), sizeof(double), v.size(), out); };
    //  1. the default hat weight
    put(HeavisideFilter::GetFilteredVariable(p, R, beta, s));
    put(HeavisideFilter::GetFilteredSensitivity(p, R, beta, s, d));
    put(DensityFilter::GetFilteredValue(p, R, s));
    //  2. the hat weight between cells of the design region j < ly / 2, the identity elsewhere
    //     (the production drivers' masked form)
    const int half = ly / 2;
    auto region = [=](int i1, int j1, int k1, int i2, int j2, int k2) {
        const bool in1 = j1 < half, in2 = j2 < half;
        if (in1 && in2) return (R - std::sqrt(std::pow(i1 - i2, 2.0) + std::pow(j1 - j2, 2.0) + std::pow(k1 - k2, 2.0))) / R;
        return (i1 == i2 && j1 == j2 && k1 == k2) ? 1.0 : 0.0;
    };
    put(HeavisideFilter::GetFilteredVariable(p, R, beta, s, region));
    put(HeavisideFilter::GetFilteredSensitivity(p, R, beta, s, d, region));
    put(DensityFilter::GetFilteredValue(p, R, s, region));
    //  3. a Gaussian weight exp(-distance^2 / R), not of that form
    auto gauss = [=](int i1, int j1, int k1, int i2, int j2, int k2) {
        return std::exp(-(std::pow(i1 - i2, 2.0) + std::pow(j1 - j2, 2.0) + std::pow(k1 - k2, 2.0)) / R);
    };
    put(HeavisideFilter::GetFilteredVariable(p, R, beta, s, gauss));
    put(HeavisideFilter::GetFilteredSensitivity(p, R, beta, s, d, gauss));
    put(DensityFilter::GetFilteredValue(p, R, s, gauss));
}

int main(int argc, char **argv) {
    if (argc != 3) { std::fprintf(stderr, "usage: %s <input.bin> <output.bin>\n", argv[0]); return 2; }
    FILE *fp = std::fopen(argv[1], "rb");
    if (!fp) { std::perror(argv[1]); return 2; }
    int hdr[4];
    double ph[2];
    if (std::fread(hdr, sizeof(int), 4, fp) != 4 || std::fread(ph, sizeof(double), 2, fp) != 2) return 2;
    const size_t n = (size_t)hdr[1] * hdr[2] * hdr[3];
    std::vector<double> s(n), d(n);
    if (std::fread(s.data(), sizeof(double), n, fp) != n || std::fread(d.data(), sizeof(double), n, fp) != n) return 2;
    std::fclose(fp);
    FILE *out = std::fopen(argv[2], "wb");
    if (!out) { std::perror(argv[2]); return 2; }
    if (hdr[0] == 2) {
        D2Q9<double> p(hdr[1], hdr[2]);
        run(p, ph[0], ph[1], s, d, out, hdr[2]);
    } else {
        D3Q15<double> p(hdr[1], hdr[2], hdr[3]);
        run(p, ph[0], ph[1], s, d, out, hdr[2]);
    }
    std::fclose(out);
    return 0;
}
