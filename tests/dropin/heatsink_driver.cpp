//  heatsink_driver.cpp -- a heat-sink driver written against PANSLBM2's template API, built
//  on the drop-in headers (dropin/src) and the GB300 library. It runs the heat-sink time loops
//  of the golden cases hsfwd_* / hsadj_* (tests/golden/cases.py: the calls of
//  production/heatsink.cpp:142-212 in the same order), reading its inputs from and writing its
//  outputs to raw binary files, so the test can compare them with the reference's outputs.
//
//  usage: heatsink_driver <fwd|adj> <input.bin> <output.bin>
//  input:  int32 nd, lx, ly, lz, steps_fwd, steps_adj; float64 nu, gx, gy, gz, tem0, qn, L;
//          then N float64 each: alpha kappa dads dkds rho0 ux0 uy0 uz0 tem0 ip0 iux0 iuy0 iuz0
//          it0 iqx0 iqy0 iqz0
//  output: fwd: f (q*N, direction-major), g, rho ux uy uz tem qx qy qz
//          adj: f, g, ip iux iuy iuz imx imy imz item iqx iqy iqz, sens0..sens3
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "../../dropin/src/particle/d2q9.h"
#include "../../dropin/src/particle/d3q15.h"
#include "../../dropin/src/equation/advection.h"
#include "../../dropin/src/equation/adjointadvection.h"
#include "../../dropin/src/utility/residual.h"

using namespace PANSLBM2;

struct Input {
    int nd, lx, ly, lz, tf, ta;
    double nu, gx, gy, gz, tem0, qn, L;
    std::vector<std::vector<double>> a;   // 17 fields
};

static Input read_input(const char *path) {
    Input in;
    FILE *fp = std::fopen(path, "rb");
    if (!fp) { std::perror(path); std::exit(2); }
    int hdr[6];
    double ph[7];
    if (std::fread(hdr, sizeof(int), 6, fp) != 6 || std::fread(ph, sizeof(double), 7, fp) != 7) std::exit(2);
    in.nd = hdr[0]; in.lx = hdr[1]; in.ly = hdr[2]; in.lz = hdr[3]; in.tf = hdr[4]; in.ta = hdr[5];
    in.nu = ph[0]; in.gx = ph[1]; in.gy = ph[2]; in.gz = ph[3]; in.tem0 = ph[4]; in.qn = ph[5]; in.L = ph[6];
    const size_t n = (size_t)in.lx * in.ly * in.lz;
    in.a.assign(17, std::vector<double>(n));
    for (auto &v : in.a)
        if (std::fread(v.data(), sizeof(double), n, fp) != n) std::exit(2);
    std::fclose(fp);
    return in;
}

static void put(FILE *fp, const double *p, size_t n) { std::fwrite(p, sizeof(double), n, fp); }

//  populations of one particle, direction-major p[c*N + idx], from the host mirrors f0 / f
template<class P>
static std::vector<double> populations(P &p) {
    p.CopyToHost();
    std::vector<double> out((size_t)P::nc * p.nxyz);
    for (int idx = 0; idx < p.nxyz; ++idx) {
        out[idx] = p.f0[idx];
        for (int c = 1; c < P::nc; ++c) out[(size_t)c * p.nxyz + idx] = p.f[P::IndexF(idx, c)];
    }
    return out;
}

int run2d(const Input &in, bool adj, FILE *out) {
    const int lx = in.lx, ly = in.ly;
    const double tem0 = in.tem0, qn = in.qn, L = in.L;
    D2Q9<double> pf(lx, ly), pg(lx, ly);
    const int n = pf.nxyz;
    std::vector<double> rho(n), ux(n), uy(n), uxp(n), uyp(n), tem(n), qx(n), qy(n), qxp(n), qyp(n), gi((size_t)n * 9);
    const auto &A = in.a;
    NS::InitialCondition(pf, A[4].data(), A[5].data(), A[6].data());
    AD::InitialCondition(pg, A[8].data(), A[5].data(), A[6].data());
    double *pux = ux.data(), *puy = uy.data(), *puxp = uxp.data(), *puyp = uyp.data();
    double *pqx = qx.data(), *pqy = qy.data(), *pqxp = qxp.data(), *pqyp = qyp.data();
    for (int t = 1; t <= in.tf; ++t) {
        AD::MacroBrinkmanCollideNaturalConvection(pf, rho.data(), pux, puy, A[0].data(), in.nu, pg, tem.data(), pqx, pqy,
                                                  A[1].data(), in.gx, in.gy, tem0, true, gi.data());
        if (t == in.tf) break;
        pf.Stream();
        pg.Stream();
        pf.BoundaryCondition([=](int _i, int _j) { return _i == 0 ? 2 : 1; });
        AD::BoundaryConditionSetT(pg, [=](int _i, int _j) { return tem0; }, pux, puy,
                                  [=](int _i, int _j) { return _i == lx - 1 || _j == ly - 1; });
        AD::BoundaryConditionSetQ(pg, [=](int _i, int _j) { return (_j == 0 && _i < L) ? qn : 0.0; }, pux, puy,
                                  A[1].data(), [=](int _i, int _j) { return _j == 0; });
        pg.BoundaryCondition([=](int _i, int _j) { return _i == 0 ? 2 : 0; });
        pf.SmoothCorner();
        pg.SmoothCorner();
        std::swap(pux, puxp); std::swap(puy, puyp); std::swap(pqx, pqxp); std::swap(pqy, pqyp);
    }
    if (!adj) {
        put(out, populations(pf).data(), (size_t)9 * n);
        put(out, populations(pg).data(), (size_t)9 * n);
        std::vector<double> zero(n, 0.0);
        for (const double *p : std::vector<const double *>{rho.data(), pux, puy, zero.data(), tem.data(), pqx, pqy, zero.data()})
            put(out, p, n);
        return 0;
    }
    std::vector<double> ip(n), iux(n), iuy(n), imx(n), imy(n), item(n), iqx(n), iqy(n), igi((size_t)n * 9);
    ANS::InitialCondition(pf, pux, puy, A[9].data(), A[10].data(), A[11].data());
    AAD::InitialCondition(pg, pux, puy, A[13].data(), A[14].data(), A[15].data());
    for (int t = 1; t <= in.ta; ++t) {
        AAD::MacroBrinkmanCollideNaturalConvection(pf, rho.data(), pux, puy, ip.data(), iux.data(), iuy.data(), imx.data(),
                                                   imy.data(), A[0].data(), in.nu, pg, tem.data(), item.data(), iqx.data(),
                                                   iqy.data(), A[1].data(), in.gx, in.gy, true, igi.data());
        if (t == in.ta) break;
        pf.iStream();
        pg.iStream();
        AAD::iBoundaryConditionSetT(pg, pux, puy, [=](int _i, int _j) { return _i == lx - 1 || _j == ly - 1; });
        AAD::iBoundaryConditionSetQ(pg, pux, puy, [=](int _i, int _j) { return _j == 0; });
        AAD::iBoundaryConditionSetQ(pg, pux, puy, [=](int _i, int _j) { return _j == 0 && _i < L; }, 1.0);
        pg.iBoundaryCondition([=](int _i, int _j) { return _i == 0 ? 2 : 0; });
        pf.iBoundaryCondition([=](int _i, int _j) { return _i == 0 ? 2 : 1; });
        pf.SmoothCorner();
        pg.SmoothCorner();
    }
    put(out, populations(pf).data(), (size_t)9 * n);
    put(out, populations(pg).data(), (size_t)9 * n);
    std::vector<double> zero(n, 0.0);
    for (const double *p : std::vector<const double *>{ip.data(), iux.data(), iuy.data(), zero.data(), imx.data(), imy.data(),
                                                       zero.data(), item.data(), iqx.data(), iqy.data(), zero.data()})
        put(out, p, n);
    std::vector<double> s(n);
    std::fill(s.begin(), s.end(), 0.0);
    AAD::SensitivityTemperatureAtHeatSource(pg, s.data(), pux, puy, imx.data(), imy.data(), A[2].data(), tem.data(),
                                            item.data(), iqx.data(), iqy.data(), gi.data(), igi.data(), A[1].data(),
                                            A[3].data(), [=](int _i, int _j) { return (_j == 0 && _i < L) ? qn : 0.0; },
                                            [=](int _i, int _j) { return _j == 0 && _i < L; });
    put(out, s.data(), n);
    std::fill(s.begin(), s.end(), 0.0);
    AAD::SensitivityBrinkmanDiffusivity(pg, s.data(), pux, puy, imx.data(), imy.data(), A[2].data(), tem.data(), item.data(),
                                        iqx.data(), iqy.data(), gi.data(), igi.data(), A[1].data(), A[3].data());
    put(out, s.data(), n);
    std::fill(s.begin(), s.end(), 0.0);
    AAD::SensitivityHeatExchange(pg, s.data(), pux, puy, imx.data(), imy.data(), A[2].data(), tem.data(), item.data(),
                                 A[3].data());
    put(out, s.data(), n);
    std::fill(s.begin(), s.end(), 0.0);
    ANS::SensitivityBrinkman(pf, s.data(), pux, puy, imx.data(), imy.data(), A[2].data());
    put(out, s.data(), n);
    return 0;
}

int run3d(const Input &in, bool adj, FILE *out) {
    const int lx = in.lx, ly = in.ly, lz = in.lz;
    const double tem0 = in.tem0, qn = in.qn, L = in.L;
    D3Q15<double> pf(lx, ly, lz), pg(lx, ly, lz);
    const int n = pf.nxyz;
    std::vector<double> rho(n), ux(n), uy(n), uz(n), uxp(n), uyp(n), uzp(n), tem(n), qx(n), qy(n), qz(n), qxp(n), qyp(n),
        qzp(n), gi((size_t)n * 15);
    const auto &A = in.a;
    NS::InitialCondition(pf, A[4].data(), A[5].data(), A[6].data(), A[7].data());
    AD::InitialCondition(pg, A[8].data(), A[5].data(), A[6].data(), A[7].data());
    double *pux = ux.data(), *puy = uy.data(), *puz = uz.data(), *puxp = uxp.data(), *puyp = uyp.data(), *puzp = uzp.data();
    double *pqx = qx.data(), *pqy = qy.data(), *pqz = qz.data(), *pqxp = qxp.data(), *pqyp = qyp.data(), *pqzp = qzp.data();
    double last_res[2] = {0.0, 0.0};
    const auto t0 = std::chrono::steady_clock::now();
    for (int t = 1; t <= in.tf; ++t) {
        AD::MacroBrinkmanCollideNaturalConvection(pf, rho.data(), pux, puy, puz, A[0].data(), in.nu, pg, tem.data(), pqx, pqy,
                                                  pqz, A[1].data(), in.gx, in.gy, in.gz, tem0, true, gi.data());
        if (t == in.tf) break;
        if (t % 100 == 0) {
            // the residual check of production/heatsink3D.cpp's loop, without its early exit (the
            // step count stays fixed)
            last_res[0] = Residual(pux, puy, puz, puxp, puyp, puzp, n);
            last_res[1] = Residual(pqx, pqy, pqz, pqxp, pqyp, pqzp, n);
        }
        pf.Stream();
        pg.Stream();
        pf.BoundaryCondition([=](int _i, int _j, int _k) { return (_i == 0 || _k == 0) ? 2 : 1; });
        AD::BoundaryConditionSetT(pg, [=](int _i, int _j, int _k) { return tem0; }, pux, puy, puz,
                                  [=](int _i, int _j, int _k) { return _i == lx - 1 || _j == ly - 1 || _k == lz - 1; });
        AD::BoundaryConditionSetQ(pg, [=](int _i, int _j, int _k) { return (_j == 0 && _i < L && _k < L) ? qn : 0.0; },
                                  pux, puy, puz, A[1].data(), [=](int _i, int _j, int _k) { return _j == 0; });
        pg.BoundaryCondition([=](int _i, int _j, int _k) { return (_i == 0 || _k == 0) ? 2 : 0; });
        pf.SmoothCorner();
        pg.SmoothCorner();
        std::swap(pux, puxp); std::swap(puy, puyp); std::swap(puz, puzp);
        std::swap(pqx, pqxp); std::swap(pqy, pqyp); std::swap(pqz, pqzp);
    }
    if (!adj) {
        // the time loop's wall time (its outputs written back by the next call, CopyToHost below)
        const auto pop = populations(pf);
        std::fprintf(stderr, "loop_seconds %.6f steps %d residuals %.3e %.3e\n",
                     std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(), in.tf,
                     last_res[0], last_res[1]);
        put(out, pop.data(), (size_t)15 * n);
        put(out, populations(pg).data(), (size_t)15 * n);
        for (const double *p : std::vector<const double *>{rho.data(), pux, puy, puz, tem.data(), pqx, pqy, pqz})
            put(out, p, n);
        return 0;
    }
    std::vector<double> ip(n), iux(n), iuy(n), iuz(n), imx(n), imy(n), imz(n), item(n), iqx(n), iqy(n), iqz(n),
        igi((size_t)n * 15);
    ANS::InitialCondition(pf, pux, puy, puz, A[9].data(), A[10].data(), A[11].data(), A[12].data());
    AAD::InitialCondition(pg, pux, puy, puz, A[13].data(), A[14].data(), A[15].data(), A[16].data());
    for (int t = 1; t <= in.ta; ++t) {
        AAD::MacroBrinkmanCollideNaturalConvection(pf, rho.data(), pux, puy, puz, ip.data(), iux.data(), iuy.data(), iuz.data(),
                                                   imx.data(), imy.data(), imz.data(), A[0].data(), in.nu, pg, tem.data(),
                                                   item.data(), iqx.data(), iqy.data(), iqz.data(), A[1].data(), in.gx, in.gy,
                                                   in.gz, true, igi.data());
        if (t == in.ta) break;
        pf.iStream();
        pg.iStream();
        AAD::iBoundaryConditionSetT(pg, pux, puy, puz, [=](int _i, int _j, int _k) { return _i == lx - 1 || _j == ly - 1 || _k == lz - 1; });
        AAD::iBoundaryConditionSetQ(pg, pux, puy, puz, [=](int _i, int _j, int _k) { return _j == 0; });
        AAD::iBoundaryConditionSetQ(pg, pux, puy, puz, [=](int _i, int _j, int _k) { return _j == 0 && _i < L && _k < L; }, 1.0);
        pg.iBoundaryCondition([=](int _i, int _j, int _k) { return (_i == 0 || _k == 0) ? 2 : 0; });
        pf.iBoundaryCondition([=](int _i, int _j, int _k) { return (_i == 0 || _k == 0) ? 2 : 1; });
        pf.SmoothCorner();
        pg.SmoothCorner();
    }
    put(out, populations(pf).data(), (size_t)15 * n);
    put(out, populations(pg).data(), (size_t)15 * n);
    for (const double *p : std::vector<const double *>{ip.data(), iux.data(), iuy.data(), iuz.data(), imx.data(), imy.data(),
                                                       imz.data(), item.data(), iqx.data(), iqy.data(), iqz.data()})
        put(out, p, n);
    std::vector<double> s(n, 0.0);
    AAD::SensitivityTemperatureAtHeatSource(pg, s.data(), pux, puy, puz, imx.data(), imy.data(), imz.data(), A[2].data(),
                                            tem.data(), item.data(), iqx.data(), iqy.data(), iqz.data(), gi.data(), igi.data(),
                                            A[1].data(), A[3].data(),
                                            [=](int _i, int _j, int _k) { return (_j == 0 && _i < L && _k < L) ? qn : 0.0; },
                                            [=](int _i, int _j, int _k) { return _j == 0 && _i < L && _k < L; });
    put(out, s.data(), n);
    std::fill(s.begin(), s.end(), 0.0);
    AAD::SensitivityBrinkmanDiffusivity(pg, s.data(), pux, puy, puz, imx.data(), imy.data(), imz.data(), A[2].data(),
                                        tem.data(), item.data(), iqx.data(), iqy.data(), iqz.data(), gi.data(), igi.data(),
                                        A[1].data(), A[3].data());
    put(out, s.data(), n);
    std::fill(s.begin(), s.end(), 0.0);
    AAD::SensitivityHeatExchange(pg, s.data(), pux, puy, puz, imx.data(), imy.data(), imz.data(), A[2].data(), tem.data(),
                                 item.data(), A[3].data());
    put(out, s.data(), n);
    std::fill(s.begin(), s.end(), 0.0);
    ANS::SensitivityBrinkman(pf, s.data(), pux, puy, puz, imx.data(), imy.data(), imz.data(), A[2].data());
    put(out, s.data(), n);
    return 0;
}

int main(int argc, char **argv) {
    if (argc != 4) { std::fprintf(stderr, "usage: %s <fwd|adj> <input.bin> <output.bin>\n", argv[0]); return 2; }
    const bool adj = std::string(argv[1]) == "adj";
    Input in = read_input(argv[2]);
    FILE *out = std::fopen(argv[3], "wb");
    if (!out) { std::perror(argv[3]); return 2; }
    const int rc = in.nd == 2 ? run2d(in, adj, out) : run3d(in, adj, out);
    std::fclose(out);
    return rc;
}
