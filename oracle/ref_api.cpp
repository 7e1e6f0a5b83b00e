// ref_api.cpp -- exports the oracle API names from the reference-backed library, dispatching on
// the lattice (q = 9 -> D2Q9 translation unit, q = 15 -> D3Q15 translation unit). TEST ONLY.
#include "oracle.h"
#include <cmath>
#ifdef _OPENMP
#include <omp.h>
#endif

#define DECL(dim)                                                                                         \
    extern "C" void ref##dim##_stream(const ol_lat *, double *, int);                                    \
    extern "C" void ref##dim##_apply_bc(const ol_lat *, double *, double *, const ol_bc *);             \
    extern "C" void ref##dim##_smooth_corner(const ol_lat *, double *);                                  \
    extern "C" void ref##dim##_smooth_at(const ol_lat *, double *, int, int, int, int, int, int);       \
    extern "C" void ref##dim##_smooth_line(const ol_lat *, double *, int, int, int, int, int);          \
    extern "C" void ref##dim##_collide(const ol_lat *, int, double *, double *, const ol_fields *, const ol_phys *, int); \
    extern "C" void ref##dim##_init(const ol_lat *, int, double *, const ol_fields *);                   \
    extern "C" void ref##dim##_sensitivity(const ol_lat *, int, double *, const ol_fields *, const double *, const double *, const double *, const double *, const double *, const int *); \
    extern "C" void ref##dim##_heaviside_var(const ol_lat *, double, double, const double *, const int *, double *); \
    extern "C" void ref##dim##_heaviside_sens(const ol_lat *, double, double, const double *, const double *, const int *, double *); \
    extern "C" void ref##dim##_density_filter(const ol_lat *, double, const double *, const int *, double *); \
    extern "C" void ref##dim##_filter_table(const ol_lat *, int, double, double, const double *, const double *, const double *, double *);
DECL(2)
DECL(3)
extern "C" double ref_residual(int, int, const double *const *, const double *const *);
extern "C" void ref_normalize(double *, int);

#define DISPATCH(fn, ...) do { if (L->q == 9) ref2_##fn(__VA_ARGS__); else ref3_##fn(__VA_ARGS__); } while (0)

extern "C" {
int ol_nnodes(const ol_lat *L) { return L->nx * L->ny * (L->q == 9 ? 1 : L->nz); }
void ol_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}
void ol_stream(const ol_lat *L, double *f, int inverse) { DISPATCH(stream, L, f, inverse); }
void ol_apply_bc(const ol_lat *L, double *f, double *g, const ol_bc *bc) { DISPATCH(apply_bc, L, f, g, bc); }
void ol_smooth_corner(const ol_lat *L, double *f) { DISPATCH(smooth_corner, L, f); }
void ol_smooth_at(const ol_lat *L, double *f, int i, int j, int k, int dx, int dy, int dz) { DISPATCH(smooth_at, L, f, i, j, k, dx, dy, dz); }
void ol_smooth_line(const ol_lat *L, double *f, int p, int a, int b, int da, int db) { DISPATCH(smooth_line, L, f, p, a, b, da, db); }
void ol_collide(const ol_lat *L, int kind, double *f, double *g, const ol_fields *F, const ol_phys *P, int save) { DISPATCH(collide, L, kind, f, g, F, P, save); }
void ol_init(const ol_lat *L, int which, double *f, const ol_fields *F) { DISPATCH(init, L, which, f, F); }
void ol_sensitivity(const ol_lat *L, int which, double *dfds, const ol_fields *F, const double *dads, const double *dkds,
                    const double *g, const double *ig, const double *qn, const int *mask) {
    DISPATCH(sensitivity, L, which, dfds, F, dads, dkds, g, ig, qn, mask);
}
void ol_heaviside_var(const ol_lat *L, double R, double beta, const double *s, const int *mask, double *out) { DISPATCH(heaviside_var, L, R, beta, s, mask, out); }
void ol_heaviside_sens(const ol_lat *L, double R, double beta, const double *s, const double *d, const int *mask, double *out) { DISPATCH(heaviside_sens, L, R, beta, s, d, mask, out); }
void ol_density_filter(const ol_lat *L, double R, const double *v, const int *mask, double *out) { DISPATCH(density_filter, L, R, v, mask, out); }
int ol_filter_ntaps(const ol_lat *L, double R) {
    const int nR = (int)R, three = L->q != 9;
    int m = 0;
    for (int a = -nR; a <= nR; ++a)
        for (int b = -nR; b <= nR; ++b)
            for (int c = (three ? -nR : 0); c <= (three ? nR : 0); ++c)
                if (std::sqrt(std::pow((double)a, 2.0) + std::pow((double)b, 2.0) + std::pow((double)c, 2.0)) <= R) ++m;
    return m;
}
void ol_filter_table(const ol_lat *L, int op, double R, double beta, const double *a, const double *b, const double *w,
                     double *out) {
    DISPATCH(filter_table, L, op, R, beta, a, b, w, out);
}
double ol_residual(int n, int ncomp, const double *const *a, const double *const *b) { return ref_residual(n, ncomp, a, b); }
void ol_normalize(double *v, int n) { ref_normalize(v, n); }
}
