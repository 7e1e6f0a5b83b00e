// ref_mma.cpp -- binds the reference's own MMA<double> (utility/mma.h of the PANSLBM2 sources,
// included where they lie) to a C entry point, to produce golden vectors of the MMA update.
// Test infrastructure only.
#include <vector>

#include "src/utility/mma.h"

extern "C" void ref_mma_run(int n, int m, double a0, const double *a, const double *c, const double *d,
                            const double *xmin, const double *xmax, double move, int iters, double *x,
                            const double *f, const double *dfdx, const double *g, const double *dgdx, double *xhist) {
    PANSLBM2::MMA<double> opt(n, m, a0, std::vector<double>(a, a + m), std::vector<double>(c, c + m),
                              std::vector<double>(d, d + m), std::vector<double>(xmin, xmin + n),
                              std::vector<double>(xmax, xmax + n));
    opt.move = move;
    std::vector<double> xk(x, x + n);
    for (int it = 0; it < iters; ++it) {
        std::vector<double> df(dfdx + (size_t)it * n, dfdx + (size_t)(it + 1) * n);
        std::vector<double> gv(g + (size_t)it * m, g + (size_t)(it + 1) * m);
        std::vector<std::vector<double>> dg(m);
        for (int i = 0; i < m; ++i)
            dg[i].assign(dgdx + ((size_t)it * m + i) * n, dgdx + ((size_t)it * m + i + 1) * n);
        opt.UpdateVariables(xk, f[it], df, gv, dg);
        for (int j = 0; j < n; ++j) xhist[(size_t)it * n + j] = xk[j];
    }
    for (int j = 0; j < n; ++j) x[j] = xk[j];
}
