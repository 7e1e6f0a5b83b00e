//  nsin_channel_driver.cpp -- an incompressible Brinkman channel written against PANSLBM2's
//  template API (D2Q9, NSin, ANSin), built on the drop-in headers (dropin/src) and the GB300
//  library. It runs the loops of the golden case nsinch_q9 (tests/golden/cases.py: nsin_run) with
//  the reference's calls in the same order, reading its inputs from and writing its outputs to
//  raw binary files, so the test can compare them with the reference's outputs.
//
//  usage: nsin_channel_driver <input.bin> <output.bin>
//  input:  int32 nx, ny, steps_fwd, steps_adj; float64 nu, eps;
//          then N float64 each: alpha dads uin rho0 ux0 uy0 ip0 iux0 iuy0
//  output: f (9*N, direction-major), rho ux uy, fa (9*N), ip iux iuy imx imy, sens
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "../../dropin/src/particle/d2q9.h"
#include "../../dropin/src/equation/nsincompressible.h"
#include "../../dropin/src/equation/adjointnsincompressible.h"

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
    const int nx = hdr[0], ny = hdr[1], tf = hdr[2], ta = hdr[3];
    const double nu = ph[0], eps = ph[1];
    const size_t n = (size_t)nx * ny;
    std::vector<std::vector<double>> A(9, std::vector<double>(n));
    for (auto &v : A)
        if (std::fread(v.data(), sizeof(double), n, fp) != n) return 2;
    std::fclose(fp);
    const std::vector<double> &alpha = A[0], &dads = A[1], &uin = A[2];

    D2Q9<double> p(nx, ny);
    std::vector<double> rho(n), ux(n), uy(n);
    auto wall = [](int, int) { return 1; };
    auto all = [](int, int) { return true; };
    NSin::InitialCondition(p, A[3].data(), A[4].data(), A[5].data());
    for (int t = 1; t <= tf; ++t) {
        NSin::MacroBrinkmanCollide(p, rho.data(), ux.data(), uy.data(), nu, alpha.data(), true);
        if (t == tf) break;
        p.Stream();
        p.BoundaryConditionAlongYEdge(0, -1, wall);
        p.BoundaryConditionAlongYEdge(ny - 1, 1, wall);
        NSin::BoundaryConditionSetUAlongXEdge(p, 0, -1, [&](int i, int j) { return uin[i + nx * j]; },
                                              [](int, int) { return 0.0; }, all);
        NSin::BoundaryConditionSetRhoAlongXEdge(p, nx - 1, 1, [](int, int) { return 1.0; }, [](int, int) { return 0.0; }, all);
    }
    FILE *out = std::fopen(argv[2], "wb");
    if (!out) { std::perror(argv[2]); return 2; }
    put(out, populations(p).data(), 9 * n);
    put(out, rho.data(), n);
    put(out, ux.data(), n);
    put(out, uy.data(), n);

    std::vector<double> ip(n), iux(n), iuy(n), imx(n), imy(n), s(n, 0.0);
    ANSin::InitialCondition(p, ux.data(), uy.data(), A[6].data(), A[7].data(), A[8].data());
    for (int t = 1; t <= ta; ++t) {
        ANSin::MacroBrinkmanCollide(p, rho.data(), ux.data(), uy.data(), ip.data(), iux.data(), iuy.data(), imx.data(),
                                    imy.data(), nu, alpha.data(), true);
        if (t == ta) break;
        p.iStream();
        p.iBoundaryConditionAlongYEdge(0, -1, wall);
        p.iBoundaryConditionAlongYEdge(ny - 1, 1, wall);
        ANSin::iBoundaryConditionSetUAlongXEdge(p, 0, -1, all, eps);
        ANSin::iBoundaryConditionSetRhoAlongXEdge(p, nx - 1, 1, all);
    }
    put(out, populations(p).data(), 9 * n);
    for (const std::vector<double> *v : {&ip, &iux, &iuy, &imx, &imy}) put(out, v->data(), n);
    ANSin::SensitivityBrinkman(p, s.data(), ux.data(), uy.data(), imx.data(), imy.data(), dads.data());
    put(out, s.data(), n);
    std::fclose(out);
    return 0;
}
