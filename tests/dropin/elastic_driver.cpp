//  elastic_driver.cpp -- the compliance-sensitivity loop of the reference's test/elsens.cpp,
//  written against PANSLBM2's template API (D2Q9, EL, AEL) and built on the drop-in headers
//  (dropin/src) and the GB300 library. It runs the loops of the golden case elsens_q9
//  (tests/golden/cases.py: elsens_run) with the reference's calls in the same order, reading its
//  inputs from and writing its outputs to raw binary files, so the test can compare them with
//  the reference's outputs.
//
//  usage: elastic_driver <input.bin> <output.bin>
//  input:  int32 nx, ny, steps_fwd, steps_adj; float64 tau, stress0; then N float64 each: rho gamma
//  output: f (9*N, direction-major), rx ry ux uy sxx sxy syx syy, fa (9*N),
//          irho imx imy isxx isxy isyx isyy, dfds
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "../../dropin/src/particle/d2q9.h"
#include "../../dropin/src/equation/elastic.h"
#include "../../dropin/src/equation/adjointelastic.h"
#include "../../dropin/src/utility/normalize.h"

using namespace PANSLBM2;

static void put(FILE *fp, const double *p, size_t n) { std::fwrite(p, sizeof(double), n, fp); }

static std::vector<double> populations(D2Q9<double> &p) {
    p.CopyToHost();
    std::vector<double> out((size_t)9 * p.nxyz);
    for (int idx = 0; idx < p.nxyz; ++idx) {
        out[idx] = p.f0[idx];
        for (int c = 1; c < 9; ++c) out[(size_t)c * p.nxyz + idx] = p.f[D2Q9<double>::IndexF(idx, c)];
    }
    return out;
}

int main(int argc, char **argv) {
    if (argc != 3) { std::fprintf(stderr, "usage: %s <input.bin> <output.bin>\n", argv[0]); return 2; }
    FILE *fp = std::fopen(argv[1], "rb");
    if (!fp) { std::perror(argv[1]); return 2; }
    int hdr[4];
    double ph[2];
    if (std::fread(hdr, sizeof(int), 4, fp) != 4 || std::fread(ph, sizeof(double), 2, fp) != 2) return 2;
    const int lx = hdr[0], ly = hdr[1], tf = hdr[2], ta = hdr[3];
    const double tau = ph[0], stress0 = ph[1];
    const size_t n = (size_t)lx * ly;
    std::vector<double> rho(n), gamma(n);
    if (std::fread(rho.data(), sizeof(double), n, fp) != n || std::fread(gamma.data(), sizeof(double), n, fp) != n) return 2;
    std::fclose(fp);

    D2Q9<double> pf(lx, ly);
    std::vector<double> ux(n, 0.0), uy(n, 0.0), rx(n, 0.0), ry(n, 0.0), sxx(n, 0.0), sxy(n, 0.0), syx(n, 0.0), syy(n, 0.0);
    std::vector<double> irho(n, 0.0), imx(n, 0.0), imy(n, 0.0), isxx(n, 0.0), isxy(n, 0.0), isyx(n, 0.0), isyy(n, 0.0);
    std::vector<double> dfds(n, 0.0);
    auto wall = [=](int _i, int _j) { return _i == 0 ? 1 : 0; };
    auto tx = [=](int _i, int _j) { return 0.0; };
    auto ty = [=](int _i, int _j) { return (_i == lx - 1 && std::fabs(_j - 0.5 * ly) < 0.2 * ly) ? stress0 : 0.0; };
    auto free = [=](int _i, int _j) { return _i != 0; };

    EL::InitialCondition(pf, rho.data(), ux.data(), uy.data(), sxx.data(), sxy.data(), syx.data(), syy.data());
    for (int t = 1; t <= tf; ++t) {
        EL::MacroExtendedCollide(pf, rho.data(), ux.data(), uy.data(), sxx.data(), sxy.data(), syx.data(), syy.data(), tau,
                                 gamma.data(), true);
        pf.Stream();
        pf.BoundaryCondition(wall);
        EL::BoundaryConditionSetStress(pf, tx, ty, free);
        pf.SmoothCorner();
        for (size_t idx = 0; idx < n; ++idx) { rx[idx] += ux[idx]; ry[idx] += uy[idx]; }
    }
    FILE *out = std::fopen(argv[2], "wb");
    if (!out) { std::perror(argv[2]); return 2; }
    put(out, populations(pf).data(), 9 * n);
    for (const std::vector<double> *v : {&rx, &ry, &ux, &uy, &sxx, &sxy, &syx, &syy}) put(out, v->data(), n);

    AEL::InitialCondition(pf, irho.data(), imx.data(), imy.data(), isxx.data(), isxy.data(), isyx.data(), isyy.data(),
                          gamma.data());
    for (int t = 1; t <= ta; ++t) {
        AEL::MacroCollide(pf, irho.data(), imx.data(), imy.data(), isxx.data(), isxy.data(), isyx.data(), isyy.data(), tau,
                          gamma.data(), true);
        pf.iStream();
        pf.iBoundaryCondition(wall);
        AEL::iBoundaryConditionSetStress(pf, tx, ty, rho.data(), free);
        pf.SmoothCorner();
    }
    put(out, populations(pf).data(), 9 * n);
    for (const std::vector<double> *v : {&irho, &imx, &imy, &isxx, &isxy, &isyx, &isyy}) put(out, v->data(), n);
    AEL::SensitivityCompliance(pf, dfds.data(), sxx.data(), sxy.data(), syx.data(), syy.data(), irho.data(), isxx.data(),
                               isxy.data(), isyx.data(), isyy.data());
    Normalize(dfds.data(), (int)n);
    put(out, dfds.data(), n);
    std::fclose(out);
    return 0;
}
