/*
 * oracle.c -- CPU restatement of the PANSLBM2 hot path (TEST INFRASTRUCTURE ONLY).
 *
 * Used by tests/ as the checker of the CUDA library, and by bench.py as the timed CPU
 * baseline ("port"). Never linked into the product. Every routine cites the reference
 * function (path:line inside the PANSLBM2 project) whose arithmetic it restates. The
 * evaluation order of each expression follows the reference so that, compiled with
 * -ffp-contract=off, results agree bit-for-bit with the reference's scalar path
 * (checked by tests/test_oracle_vs_reference.py where the reference sources exist).
 *
 * Layout: f[c*N + idx] (rest population included), idx = i + nx*(j + ny*k).
 */
#include "oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ---- lattice tables (src/particle/d2q9.h:160-163, src/particle/d3q15.h:251-254) ---- */
static const int CX9[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
static const int CY9[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};
static const int CZ9[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
static const double W9[9] = {4.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0,
                             1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0};
static const int CX15[15] = {0, 1, 0, 0, -1, 0, 0, 1, -1, 1, 1, -1, 1, -1, -1};
static const int CY15[15] = {0, 0, 1, 0, 0, -1, 0, 1, 1, -1, 1, -1, -1, 1, -1};
static const int CZ15[15] = {0, 0, 0, 1, 0, 0, -1, 1, 1, 1, -1, -1, -1, -1, 1};
static const double W15[15] = {2.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0,
                               1.0 / 9.0, 1.0 / 72.0, 1.0 / 72.0, 1.0 / 72.0, 1.0 / 72.0,
                               1.0 / 72.0, 1.0 / 72.0, 1.0 / 72.0, 1.0 / 72.0};

typedef struct {
    int q, nd, nx, ny, nz, n;
    const int *c[3];
    const double *w;
} lat_t;

static lat_t mk(const ol_lat *L) {
    lat_t t;
    t.q = L->q;
    t.nx = L->nx;
    t.ny = L->ny;
    t.nz = (L->q == 9) ? 1 : L->nz;
    t.n = t.nx * t.ny * t.nz;
    if (L->q == 9) {
        t.nd = 2; t.c[0] = CX9; t.c[1] = CY9; t.c[2] = CZ9; t.w = W9;
    } else {
        t.nd = 3; t.c[0] = CX15; t.c[1] = CY15; t.c[2] = CZ15; t.w = W15;
    }
    return t;
}

int ol_nnodes(const ol_lat *L) { lat_t t = mk(L); return t.n; }

void ol_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* single-step periodic wrap of D2Q9::Index / D3Q15::Index (d2q9.h:80-84, d3q15.h:136-141) */
static inline int wrap(int i, int n) { return i == -1 ? n - 1 : (i == n ? 0 : i); }
static inline int IDX(const lat_t *t, int i, int j, int k) {
    return wrap(i, t->nx) + t->nx * (wrap(j, t->ny) + t->ny * wrap(k, t->nz));
}
#define F(arr, c, idx) (arr)[(size_t)(c) * (size_t)t->n + (size_t)(idx)]

static int opp_of(const lat_t *t, int c) {
    for (int e = 0; e < t->q; ++e)
        if (t->c[0][e] == -t->c[0][c] && t->c[1][e] == -t->c[1][c] && t->c[2][e] == -t->c[2][c]) return e;
    return -1;
}
static int refl_of(const lat_t *t, int c, int a) {
    int v[3] = {t->c[0][c], t->c[1][c], t->c[2][c]};
    v[a] = -v[a];
    for (int e = 0; e < t->q; ++e)
        if (t->c[0][e] == v[0] && t->c[1][e] == v[1] && t->c[2][e] == v[2]) return e;
    return -1;
}

/* ---- streaming: D2Q9::Stream (d2q9.h:165-295, serial branch 282-291), iStream (297-427),
 *      D3Q15::Stream (d3q15.h:256-617, serial branch 601-614), iStream (619-980) ---- */
void ol_stream(const ol_lat *L, double *f, int inverse) {
    lat_t T = mk(L); const lat_t *t = &T;
    static double *tmp = NULL;
    static size_t cap = 0;
    const size_t need = (size_t)t->n * (size_t)t->q;
    if (need > cap) { free(tmp); tmp = (double *)malloc(sizeof(double) * need); cap = need; }
    int s = inverse ? 1 : -1;
#pragma omp parallel for collapse(2)
    for (int k = 0; k < t->nz; ++k)
        for (int j = 0; j < t->ny; ++j)
            for (int i = 0; i < t->nx; ++i) {
                int idx = IDX(t, i, j, k);
                F(tmp, 0, idx) = F(f, 0, idx);
                for (int c = 1; c < t->q; ++c) {
                    int src = IDX(t, i + s * t->c[0][c], j + s * t->c[1][c], k + s * t->c[2][c]);
                    F(tmp, c, idx) = F(f, c, src);
                }
            }
    memcpy(f, tmp, sizeof(double) * need);
}

/* ---- face iteration helper: node (i,j,k) on the face axis=a at local position p ---- */
typedef void (*node_fn)(const lat_t *t, int idx, int i, int j, int k, void *ctx);
static void for_face(const lat_t *t, int a, int p, node_fn fn, void *ctx) {
    int n[3] = {t->nx, t->ny, t->nz};
    if (p < 0 || p >= n[a]) return;
    int b = (a + 1) % 3, c = (a + 2) % 3;
    if (t->nd == 2 && a == 2) return;
    for (int u = 0; u < n[b]; ++u)
        for (int v = 0; v < n[c]; ++v) {
            int x[3]; x[a] = p; x[b] = u; x[c] = v;
            fn(t, IDX(t, x[0], x[1], x[2]), x[0], x[1], x[2], ctx);
        }
}

/* ---- bounce-back / mirror walls ------------------------------------------------------
 * D2Q9::BoundaryConditionAlongX/YEdge (d2q9.h:429-501), iBoundaryConditionAlong* (503-575),
 * D3Q15::BoundaryConditionAlongX/Y/ZFace (d3q15.h:982-1110), iBoundaryCondition* (1112-1239).
 * Forward: incoming populations (c_a == -dir) copied from the opposite (BARRIER = 1) or from
 * the reflection across the face (MIRROR = 2). Adjoint: outgoing populations (c_a == dir).
 * Quirk kept: D3Q15 forward MIRROR on the +x side writes node (nx-1, j, k) whatever the
 * requested plane (d3q15.h:1013). */
typedef struct { const ol_bc *bc; double *f, *g; } bcctx;

static void wall_node(const lat_t *t, int idx, int i, int j, int k, void *vctx) {
    bcctx *x = (bcctx *)vctx;
    const ol_bc *bc = x->bc;
    int type = bc->type[idx];
    int a = bc->axis, d = bc->dir, adj = (bc->kind == OL_BC_IWALL);
    if (type != 1 && type != 2) return;
    int node = idx;
    if (!adj && t->nd == 3 && a == 0 && d == 1 && type == 2) node = IDX(t, t->nx - 1, j, k);
    double *f = x->f;
    for (int c = 1; c < t->q; ++c) {
        int ca = t->c[a][c];
        if (adj ? (ca != d) : (ca != -d)) continue;
        int src = (type == 1) ? opp_of(t, c) : refl_of(t, c, a);
        F(f, c, node) = F(f, src, node);
    }
    (void)i;
}

/* ---- NS Zou-He velocity / pressure BCs -----------------------------------------------
 * NS::BoundaryConditionSetUAlong{X,Y}Edge (navierstokes.h:91-146), ...AlongX/Y/ZFace
 * (148-257); SetRhoAlong* (259-426). rho0 from the tangential and outgoing sums, normal
 * momentum rho0*u_n/(6 | 12), tangential momenta (0.5 | 0.25)*(f_t+ - f_t- - rho0*u_t);
 * incoming f_c = f_opp(c) with the momentum terms applied in x, y, z order. */
static void zouhe_node(const lat_t *t, int idx, int i, int j, int k, void *vctx) {
    bcctx *x = (bcctx *)vctx;
    const ol_bc *bc = x->bc;
    if (!bc->type[idx]) return;
    double *f = x->f;
    int a = bc->axis, d = bc->dir, nd = t->nd;
    double u[3] = {0, 0, 0}, rho0;
    double sT = 0.0, sO = 0.0;
    int first = 1;
    for (int c = 0; c < t->q; ++c) {
        if (t->c[a][c] == 0) { if (first) { sT = F(f, c, idx); first = 0; } else sT += F(f, c, idx); }
    }
    first = 1;
    for (int c = 0; c < t->q; ++c) {
        if (t->c[a][c] == d) { if (first) { sO = F(f, c, idx); first = 0; } else sO += F(f, c, idx); }
    }
    double S = sT + 2.0 * sO;
    if (bc->kind == OL_BC_NS_U) {
        /* uscale: time-varying inflow (CPU extension; 1 = the reference routine) */
        u[0] = bc->uscale * bc->v0[idx]; u[1] = bc->uscale * bc->v1[idx]; if (nd == 3) u[2] = bc->uscale * bc->v2[idx];
        rho0 = S / (d < 0 ? 1.0 - u[a] : 1.0 + u[a]);
    } else {
        /* SetRho: v0 = rho, v1 = first tangential (cyclic), v2 = second tangential */
        rho0 = bc->v0[idx];
        if (nd == 2) {
            u[1 - a] = bc->v1[idx];
        } else {
            u[(a + 1) % 3] = bc->v1[idx];
            u[(a + 2) % 3] = bc->v2[idx];
        }
        u[a] = (d < 0) ? 1.0 - S / rho0 : -1.0 + S / rho0;
    }
    double m[3];
    double kn = (nd == 2) ? 6.0 : 12.0, kt = (nd == 2) ? 0.5 : 0.25, kc = (nd == 2) ? 4.0 : 8.0;
    for (int b = 0; b < nd; ++b) {
        if (b == a) m[b] = rho0 * u[b] / kn;
        else {
            int cp = -1, cm = -1;
            for (int c = 1; c < t->q; ++c) {
                int ok = 1;
                for (int e = 0; e < nd; ++e) if (e != b && t->c[e][c] != 0) ok = 0;
                if (!ok) continue;
                if (t->c[b][c] == 1) cp = c;
                if (t->c[b][c] == -1) cm = c;
            }
            m[b] = kt * (F(f, cp, idx) - F(f, cm, idx) - rho0 * u[b]);
        }
    }
    for (int c = 1; c < t->q; ++c) {
        if (t->c[a][c] != -d) continue;
        int o = opp_of(t, c);
        int diag = 0;
        for (int b = 0; b < nd; ++b) if (b != a && t->c[b][c] != 0) diag = 1;
        double v = F(f, o, idx);
        if (!diag) {
            v = (t->c[a][c] > 0) ? v + kc * m[a] : v - kc * m[a];
        } else {
            for (int b = 0; b < nd; ++b) {
                int cb = t->c[b][c];
                if (b == a) v = (cb > 0) ? v + m[b] : v - m[b];
                else v = (cb > 0) ? v - m[b] : v + m[b];
            }
        }
        F(f, c, idx) = v;
    }
    (void)i; (void)j; (void)k;
}

/* ---- AD Dirichlet / Neumann BCs ------------------------------------------------------
 * AD::BoundaryConditionSetTAlong* (advection.h:97-238): tem0 = 6(T - sum known)/(1 + 3 u.n_in),
 * incoming g_c = tem0 (1 + 3 c.u) / (1/w_c).
 * AD::BoundaryConditionSetQAlong* (advection.h:240-381 constant kappa, 383-524 per node):
 * tem0 = 6((1 + 1/(6 kappa)) qn + sum outgoing)/(1 - 3 u.n_in), same incoming update. */
static double one_plus_3cu(const lat_t *t, int c, const double *u) {
    double acc = 1.0;
    for (int b = 0; b < t->nd; ++b) {
        int cb = t->c[b][c];
        if (cb > 0) acc += 3.0 * u[b];
        else if (cb < 0) acc -= 3.0 * u[b];
    }
    return acc;
}
static double inv_w(const lat_t *t, int c) {
    int s = 0;
    for (int b = 0; b < t->nd; ++b) s += abs(t->c[b][c]);
    if (s == 1) return 9.0;
    return (t->nd == 2) ? 36.0 : 72.0;
}
static void adbc_node(const lat_t *t, int idx, int i, int j, int k, void *vctx) {
    bcctx *x = (bcctx *)vctx;
    const ol_bc *bc = x->bc;
    if (!bc->type[idx]) return;
    double *g = x->f;
    int a = bc->axis, d = bc->dir, nin = -d;
    double u[3] = {bc->ux[idx], bc->uy[idx], t->nd == 3 ? bc->uz[idx] : 0.0};
    double tem0;
    if (bc->kind == OL_BC_AD_T) {
        double s = bc->v0[idx];
        for (int c = 0; c < t->q; ++c) if (t->c[a][c] != -d) s -= F(g, c, idx);
        tem0 = 6.0 * s / (nin > 0 ? 1.0 + 3.0 * u[a] : 1.0 - 3.0 * u[a]);
    } else {
        double kap = (bc->kind == OL_BC_AD_Q) ? bc->diffusivity[idx] : bc->kappa;
        double s = (1.0 + 1.0 / (6.0 * kap)) * bc->v0[idx];
        for (int c = 1; c < t->q; ++c) if (t->c[a][c] == d) s += F(g, c, idx);
        tem0 = 6.0 * s / (nin > 0 ? 1.0 - 3.0 * u[a] : 1.0 + 3.0 * u[a]);
    }
    for (int c = 1; c < t->q; ++c) {
        if (t->c[a][c] != -d) continue;
        F(g, c, idx) = tem0 * one_plus_3cu(t, c, u) / inv_w(t, c);
    }
    (void)i; (void)j; (void)k;
}

/* ---- ANS adjoint BCs ------------------------------------------------------------------
 * ANS::iBoundaryConditionSetUAlong{X,Y}Edge (adjointnavierstokes.h:95-143; the y-edge form
 * uses ux in both terms, kept), ...AlongX/Y/ZFace (145-254); iBoundaryConditionSetRho*
 * (256-392): rho0 from the inward populations, outgoing f_c = f_opp(c) -/+ rho0. */
static double tsum(const lat_t *t, const double *f, int idx, int a, int d, int b) {
    /* sum over diagonal populations with c_a == -d of sign(c_b) f_c, increasing c */
    double s = 0.0;
    for (int c = 1; c < t->q; ++c) {
        if (t->c[a][c] != -d) continue;
        int diag = 0;
        for (int e = 0; e < t->nd; ++e) if (e != a && t->c[e][c] != 0) diag = 1;
        if (!diag) continue;
        if (t->c[b][c] > 0) s += F(f, c, idx);
        else if (t->c[b][c] < 0) s -= F(f, c, idx);
    }
    return s;
}
static double nsum(const lat_t *t, const double *f, int idx, int a, int d, double kc) {
    /* kc * f_normal + sum of diagonal inward populations (increasing c) */
    double s = 0.0; int first = 1;
    for (int c = 1; c < t->q; ++c) {
        if (t->c[a][c] != -d) continue;
        int diag = 0;
        for (int e = 0; e < t->nd; ++e) if (e != a && t->c[e][c] != 0) diag = 1;
        if (!diag) { s = kc * F(f, c, idx); first = 0; break; }
    }
    (void)first;
    for (int c = 1; c < t->q; ++c) {
        if (t->c[a][c] != -d) continue;
        int diag = 0;
        for (int e = 0; e < t->nd; ++e) if (e != a && t->c[e][c] != 0) diag = 1;
        if (diag) s += F(f, c, idx);
    }
    return s;
}
static void ans_node(const lat_t *t, int idx, int i, int j, int k, void *vctx) {
    bcctx *x = (bcctx *)vctx;
    const ol_bc *bc = x->bc;
    if (!bc->type[idx]) return;
    double *f = x->f;
    int a = bc->axis, d = bc->dir, nd = t->nd;
    double rho0;
    if (bc->kind == OL_BC_ANS_RHO) {
        rho0 = nsum(t, f, idx, a, d, nd == 2 ? 4.0 : 8.0) / (nd == 2 ? 3.0 : 6.0);
        for (int c = 1; c < t->q; ++c) if (t->c[a][c] == d) F(f, c, idx) = F(f, opp_of(t, c), idx) - rho0;
        return;
    }
    double u[3] = {bc->uscale * bc->v0[idx], bc->uscale * bc->v1[idx], nd == 3 ? bc->uscale * bc->v2[idx] : 0.0};
    if (nd == 2) {
        double un = u[0], ut = (a == 0) ? u[1] : u[0];  /* y edges use ux twice (reference) */
        int b = 1 - a;
        double ns = nsum(t, f, idx, a, d, 4.0);
        double ts = tsum(t, f, idx, a, d, b);
        double num = (d < 0) ? -2.0 * bc->eps + un * ns : -2.0 * bc->eps - un * ns;
        num += 3.0 * ut * ts;
        rho0 = num / (3.0 * (d < 0 ? 1.0 - un : 1.0 + un));
    } else {
        double num = -4.0 * bc->eps;
        for (int b = 0; b < 3; ++b) {
            if (b == a) {
                double ns = nsum(t, f, idx, a, d, 8.0);
                num = (d < 0) ? num + u[a] * ns : num - u[a] * ns;
            } else {
                num += 3.0 * u[b] * tsum(t, f, idx, a, d, b);
            }
        }
        rho0 = num / (6.0 * (d < 0 ? 1.0 - u[a] : 1.0 + u[a]));
    }
    for (int c = 1; c < t->q; ++c) if (t->c[a][c] == d) F(f, c, idx) = F(f, opp_of(t, c), idx) + rho0;
    (void)i; (void)j; (void)k;
}

/* ---- incompressible NS boundary conditions (D2Q9) -------------------------------------
 * NSin::BoundaryConditionSetUAlong{X,Y}Edge (nsincompressible.h:46-90) and SetRhoAlong*
 * (92-140). With the edge normal a, tangent b and side d: the unknown normal population is its
 * opposite - d (2 u_n / 3); an unknown diagonal is its opposite - d (u_n / 6) - c_b (f_b+ - f_b- - u_t) / 2.
 * SetRho first recovers u_n = -d (rho - S), S = f_0 + f_b+ + f_b- + 2 (sum of the known normal
 * and diagonal populations of side d, increasing c).
 * ANSin::iBoundaryConditionSetUAlong{X,Y}Edge (adjointnsincompressible.h:49-92): every unknown
 * adjoint population is its opposite - 2 eps / 3. */
static int straight2(const lat_t *t, int a, int s) {
    for (int c = 1; c < t->q; ++c) if (t->c[a][c] == s && t->c[1 - a][c] == 0) return c;
    return 0;
}
static void nsin_node(const lat_t *t, int idx, int i, int j, int k, void *vctx) {
    bcctx *x = (bcctx *)vctx;
    const ol_bc *bc = x->bc;
    if (!bc->type[idx]) return;
    double *f = x->f;
    int a = bc->axis, d = bc->dir, b = 1 - a;
    if (bc->kind == OL_BC_ANSIN_U) {
        for (int c = 1; c < t->q; ++c)
            if (t->c[a][c] == d) F(f, c, idx) = F(f, opp_of(t, c), idx) - 2.0 * bc->eps / 3.0;
        return;
    }
    int tp = straight2(t, b, 1), tm = straight2(t, b, -1);
    double un, ut;
    if (bc->kind == OL_BC_NSIN_U) {
        un = (a == 0) ? bc->v0[idx] : bc->v1[idx];
        ut = (a == 0) ? bc->v1[idx] : bc->v0[idx];
    } else {
        double rho = bc->v0[idx], so = 0.0;
        int first = 1;
        ut = bc->v1[idx];
        for (int c = 1; c < t->q; ++c) {
            if (t->c[a][c] != d) continue;
            if (first) { so = F(f, c, idx); first = 0; } else so += F(f, c, idx);
        }
        double S = F(f, 0, idx) + F(f, tp, idx) + F(f, tm, idx) + 2.0 * so;
        un = (d < 0) ? rho - S : -rho + S;
    }
    double X = F(f, tp, idx) - F(f, tm, idx) - ut;
    for (int c = 1; c < t->q; ++c) {
        if (t->c[a][c] != -d) continue;
        double v = F(f, opp_of(t, c), idx);
        if (t->c[b][c] == 0) {
            F(f, c, idx) = (d < 0) ? v + 2.0 * un / 3.0 : v - 2.0 * un / 3.0;
        } else {
            v = (d < 0) ? v + un / 6.0 : v - un / 6.0;
            F(f, c, idx) = (t->c[b][c] > 0) ? v - 0.5 * X : v + 0.5 * X;
        }
    }
    (void)i; (void)j; (void)k;
}

/* ---- AAD adjoint BCs ------------------------------------------------------------------
 * AAD::iBoundaryConditionSetTAlong* (adjointadvection.h:152-300), iSetQAlong* (302-484,
 * with the missing 3.0 factors on the +y / +-z D3Q15 faces kept), iSetRhoAlong* (486-751). */
static const int *TANG3(int a) {
    static const int o0[2] = {1, 2}, o1[2] = {2, 0}, o2[2] = {0, 1};
    return a == 0 ? o0 : (a == 1 ? o1 : o2);
}
static void aad_node(const lat_t *t, int idx, int i, int j, int k, void *vctx) {
    bcctx *x = (bcctx *)vctx;
    const ol_bc *bc = x->bc;
    int type = bc->type[idx];
    if (!type) return;
    int a = bc->axis, d = bc->dir, nd = t->nd, nin = -d;
    double u[3] = {bc->ux[idx], bc->uy[idx], nd == 3 ? bc->uz[idx] : 0.0};
    double rho0;
    if (bc->kind == OL_BC_AAD_T) {
        double *g = x->f;
        if (nd == 2) {
            /* 4 (1 + 3 c.u) g_normal + sum over inward diagonals (1 + 3 c.u) g_c, normal first */
            int cn = -1;
            for (int c = 1; c < t->q; ++c) if (t->c[a][c] == -d && t->c[1 - a][c] == 0) cn = c;
            double num = 4.0 * one_plus_3cu(t, cn, u) * F(g, cn, idx);
            for (int c = 1; c < t->q; ++c) {
                if (t->c[a][c] != -d || t->c[1 - a][c] == 0) continue;
                num += one_plus_3cu(t, c, u) * F(g, c, idx);
            }
            double den = nin > 0 ? 1.0 + 3.0 * u[a] : 1.0 - 3.0 * u[a];
            rho0 = -num / (6.0 * den);
        } else {
            double den = nin > 0 ? 1.0 + 3.0 * u[a] : 1.0 - 3.0 * u[a];
            const int *tb = TANG3(a);
            rho0 = -nsum(t, g, idx, a, d, 8.0) / 12.0
                   - u[tb[0]] * tsum(t, g, idx, a, d, tb[0]) / (4.0 * den)
                   - u[tb[1]] * tsum(t, g, idx, a, d, tb[1]) / (4.0 * den);
        }
        for (int c = 1; c < t->q; ++c) if (t->c[a][c] == d) F(g, c, idx) = rho0;
        return;
    }
    if (bc->kind == OL_BC_AAD_Q) {
        double *g = x->f;
        double pre = nin > 0 ? 1.0 + 3.0 * u[a] : 1.0 - 3.0 * u[a];
        double post = nin > 0 ? 1.0 - 3.0 * u[a] : 1.0 + 3.0 * u[a];
        if (nd == 2) {
            int b = 1 - a;
            double num = pre * nsum(t, g, idx, a, d, 4.0) + 3.0 * u[b] * tsum(t, g, idx, a, d, b) - 12.0 * bc->eps;
            rho0 = num / (6.0 * post);
        } else {
            const int *tb = TANG3(a);
            double k3 = (a == 0 || (a == 1 && d < 0)) ? 3.0 : 1.0;   /* reference factor pattern */
            double num = pre * nsum(t, g, idx, a, d, 8.0);
            if (k3 == 3.0) {
                num += 3.0 * u[tb[0]] * tsum(t, g, idx, a, d, tb[0]);
                num += 3.0 * u[tb[1]] * tsum(t, g, idx, a, d, tb[1]);
            } else {
                num += u[tb[0]] * tsum(t, g, idx, a, d, tb[0]);
                num += u[tb[1]] * tsum(t, g, idx, a, d, tb[1]);
            }
            num -= 24.0 * bc->eps;
            rho0 = num / (12.0 * post);
        }
        for (int c = 1; c < t->q; ++c) if (t->c[a][c] == d) F(g, c, idx) = rho0;
        return;
    }
    /* OL_BC_AAD_RHO: writes the NS adjoint set f using the AD adjoint set g (type 1 SetT, 2 SetQ) */
    {
        double *f = x->f, *g = x->g;
        double rho = bc->rho[idx], tem = bc->tem[idx];
        double pre = nin > 0 ? 1.0 + 3.0 * u[a] : 1.0 - 3.0 * u[a];
        double post = nin > 0 ? 1.0 - 3.0 * u[a] : 1.0 + 3.0 * u[a];
        double r0, flux0 = 0.0;
        if (nd == 2) {
            int b = 1 - a;
            r0 = -nsum(t, f, idx, a, d, 4.0) / 3.0;
            if (type == 1) flux0 = tem * u[b] * tsum(t, g, idx, a, d, b) / (2.0 * pre * rho);
            else if (type == 2) flux0 = -tem * (nsum(t, g, idx, a, d, 4.0) / 3.0 + u[b] * tsum(t, g, idx, a, d, b) / 2.0) / (post * rho);
        } else {
            const int *tb = TANG3(a);
            r0 = -nsum(t, f, idx, a, d, 8.0) / 6.0;
            double tt = u[tb[0]] * tsum(t, g, idx, a, d, tb[0]) / 4.0 + u[tb[1]] * tsum(t, g, idx, a, d, tb[1]) / 4.0;
            if (type == 1) flux0 = tem * tt / (rho * pre);
            else if (type == 2) flux0 = -tem * (nsum(t, g, idx, a, d, 8.0) / 6.0 + u[tb[0]] * tsum(t, g, idx, a, d, tb[0]) / 4.0
                                               + u[tb[1]] * tsum(t, g, idx, a, d, tb[1]) / 4.0) / (rho * post);
        }
        double obj0 = bc->eps * 2.0 * tem / (post * rho);
        for (int c = 1; c < t->q; ++c)
            if (t->c[a][c] == d) F(f, c, idx) = F(f, opp_of(t, c), idx) + r0 + flux0 + obj0;
    }
    (void)i; (void)j; (void)k;
}

/* ---- elastic stress BCs (D2Q9) ---------------------------------------------------------
 * EL::BoundaryConditionSetStressAlong{X,Y}Edge (elastic.h:60-104): the three unknown
 * populations from the known ones on the same node and the traction (tx, ty).
 * AEL::iBoundaryConditionSetStressAlong{X,Y}Edge (adjointelastic.h:48-92): the three outgoing
 * adjoint populations, with the traction divided by the node's density. The D2Q9 indices are
 * spelled out as the reference does. */
static void el_stress_node(const lat_t *t, int idx, int i, int j, int k, void *vctx) {
    bcctx *x = (bcctx *)vctx;
    const ol_bc *bc = x->bc;
    if (!bc->type[idx]) return;
    double *f = x->f;
    const double tx = bc->v0[idx], ty = bc->v1[idx];
#define E(c) F(f, c, idx)
    if (bc->kind == OL_BC_EL_STRESS) {
        if (bc->axis == 0 && bc->dir == -1) {
            E(1) = E(3) - 4.0 * (E(3) + E(6) + E(7)) / 3.0 + 2.0 * tx / 3.0;
            E(5) = E(6) - (E(3) + E(6) + E(7)) / 3.0 + (tx + 3.0 * ty) / 6.0;
            E(8) = E(7) - (E(3) + E(6) + E(7)) / 3.0 + (tx - 3.0 * ty) / 6.0;
        } else if (bc->axis == 0) {
            E(3) = E(1) - 4.0 * (E(1) + E(5) + E(8)) / 3.0 - 2.0 * tx / 3.0;
            E(6) = E(5) - (E(1) + E(5) + E(8)) / 3.0 - (tx - 3.0 * ty) / 6.0;
            E(7) = E(8) - (E(1) + E(5) + E(8)) / 3.0 - (tx + 3.0 * ty) / 6.0;
        } else if (bc->dir == -1) {
            E(2) = E(4) - 4.0 * (E(4) + E(7) + E(8)) / 3.0 + 2.0 * ty / 3.0;
            E(5) = E(8) - (E(4) + E(7) + E(8)) / 3.0 + (ty + 3.0 * tx) / 6.0;
            E(6) = E(7) - (E(4) + E(7) + E(8)) / 3.0 + (ty - 3.0 * tx) / 6.0;
        } else {
            E(4) = E(2) - 4.0 * (E(2) + E(5) + E(6)) / 3.0 - 2.0 * ty / 3.0;
            E(7) = E(6) - (E(2) + E(5) + E(6)) / 3.0 - (ty + 3.0 * tx) / 6.0;
            E(8) = E(5) - (E(2) + E(5) + E(6)) / 3.0 - (ty - 3.0 * tx) / 6.0;
        }
    } else {
        const double rho = bc->rho[idx];
        if (bc->axis == 0 && bc->dir == -1) {
            E(3) = E(1) - (4.0 * E(1) + E(5) + E(8)) / 3.0 + 2.0 * tx / rho;
            E(6) = E(5) - (4.0 * E(1) + E(5) + E(8)) / 3.0 + 2.0 * (tx - ty) / rho;
            E(7) = E(8) - (4.0 * E(1) + E(5) + E(8)) / 3.0 + 2.0 * (tx + ty) / rho;
        } else if (bc->axis == 0) {
            E(1) = E(3) - (4.0 * E(3) + E(6) + E(7)) / 3.0 - 2.0 * tx / rho;
            E(5) = E(6) - (4.0 * E(3) + E(6) + E(7)) / 3.0 - 2.0 * (tx + ty) / rho;
            E(8) = E(7) - (4.0 * E(3) + E(6) + E(7)) / 3.0 - 2.0 * (tx - ty) / rho;
        } else if (bc->dir == -1) {
            E(4) = E(2) - (4.0 * E(2) + E(5) + E(6)) / 3.0 + 2.0 * ty / rho;
            E(7) = E(6) - (4.0 * E(2) + E(5) + E(6)) / 3.0 + 2.0 * (ty + tx) / rho;
            E(8) = E(5) - (4.0 * E(2) + E(5) + E(6)) / 3.0 + 2.0 * (ty - tx) / rho;
        } else {
            E(2) = E(4) - (4.0 * E(4) + E(7) + E(8)) / 3.0 - 2.0 * ty / rho;
            E(5) = E(8) - (4.0 * E(4) + E(7) + E(8)) / 3.0 - 2.0 * (ty + tx) / rho;
            E(6) = E(7) - (4.0 * E(4) + E(7) + E(8)) / 3.0 - 2.0 * (ty - tx) / rho;
        }
    }
#undef E
    (void)t; (void)i; (void)j; (void)k;
}

void ol_apply_bc(const ol_lat *L, double *f, double *g, const ol_bc *bc) {
    lat_t T = mk(L); const lat_t *t = &T;
    bcctx x; x.bc = bc; x.f = f; x.g = g;
    node_fn fn = NULL;
    switch (bc->kind) {
    case OL_BC_WALL: case OL_BC_IWALL: fn = wall_node; break;
    case OL_BC_NS_U: case OL_BC_NS_RHO: fn = zouhe_node; break;
    case OL_BC_AD_T: case OL_BC_AD_Q: case OL_BC_AD_QC: fn = adbc_node; break;
    case OL_BC_ANS_U: case OL_BC_ANS_RHO: fn = ans_node; break;
    case OL_BC_AAD_T: case OL_BC_AAD_Q: case OL_BC_AAD_RHO: fn = aad_node; break;
    case OL_BC_NSIN_U: case OL_BC_NSIN_RHO: case OL_BC_ANSIN_U: if (t->nd != 2) return; fn = nsin_node; break;
    case OL_BC_EL_STRESS: case OL_BC_AEL_STRESS: if (t->nd != 2) return; fn = el_stress_node; break;
    default: return;
    }
    for_face(t, bc->axis, bc->pos, fn, &x);
}

/* ---- corner / edge smoothing ----------------------------------------------------------
 * D2Q9::SmoothCornerAt (d2q9.h:577-587), SmoothCorner (127-132); D3Q15::SmoothCornerAlong*
 * (d3q15.h:1241-1287), SmoothCornerAt (1289-1303), SmoothCorner (199-220). */
void ol_smooth_at(const ol_lat *L, double *f, int i, int j, int k, int dx, int dy, int dz) {
    lat_t T = mk(L); const lat_t *t = &T;
    if (i < 0 || i >= t->nx || j < 0 || j >= t->ny) return;
    if (t->nd == 2) {
        int idx = IDX(t, i, j, 0), ix = IDX(t, i - dx, j, 0), iy = IDX(t, i, j - dy, 0);
        for (int c = 0; c < t->q; ++c) F(f, c, idx) = 0.5 * (F(f, c, ix) + F(f, c, iy));
    } else {
        if (k < 0 || k >= t->nz) return;
        int idx = IDX(t, i, j, k), ix = IDX(t, i - dx, j, k), iy = IDX(t, i, j - dy, k), iz = IDX(t, i, j, k - dz);
        for (int c = 0; c < t->q; ++c) F(f, c, idx) = (F(f, c, ix) + F(f, c, iy) + F(f, c, iz)) / 3.0;
    }
}

void ol_smooth_line(const ol_lat *L, double *f, int plane, int pa, int pb, int da, int db) {
    lat_t T = mk(L); const lat_t *t = &T;
    if (t->nd != 3) return;
    if (plane == 0) {           /* AlongYZ(j, k, dy, dz): line along x */
        int j = pa, k = pb;
        if (j < 0 || j >= t->ny || k < 0 || k >= t->nz) return;
        for (int i = 0; i < t->nx; ++i) {
            int idx = IDX(t, i, j, k), iy = IDX(t, i, j - da, k), iz = IDX(t, i, j, k - db);
            for (int c = 0; c < t->q; ++c) F(f, c, idx) = 0.5 * (F(f, c, iy) + F(f, c, iz));
        }
    } else if (plane == 1) {    /* AlongZX(k, i, dz, dx): line along y */
        int k = pa, i = pb;
        if (k < 0 || k >= t->nz || i < 0 || i >= t->nx) return;
        for (int j = 0; j < t->ny; ++j) {
            int idx = IDX(t, i, j, k), iz = IDX(t, i, j, k - da), ix = IDX(t, i - db, j, k);
            for (int c = 0; c < t->q; ++c) F(f, c, idx) = 0.5 * (F(f, c, iz) + F(f, c, ix));
        }
    } else {                    /* AlongXY(i, j, dx, dy): line along z */
        int i = pa, j = pb;
        if (i < 0 || i >= t->nx || j < 0 || j >= t->ny) return;
        for (int k = 0; k < t->nz; ++k) {
            int idx = IDX(t, i, j, k), ix = IDX(t, i - da, j, k), iy = IDX(t, i, j - db, k);
            for (int c = 0; c < t->q; ++c) F(f, c, idx) = 0.5 * (F(f, c, ix) + F(f, c, iy));
        }
    }
}

void ol_smooth_corner(const ol_lat *L, double *f) {
    lat_t T = mk(L); const lat_t *t = &T;
    int lx = t->nx, ly = t->ny, lz = t->nz;
    if (t->nd == 2) {
        ol_smooth_at(L, f, 0, 0, 0, -1, -1, 0);
        ol_smooth_at(L, f, 0, ly - 1, 0, -1, 1, 0);
        ol_smooth_at(L, f, lx - 1, 0, 0, 1, -1, 0);
        ol_smooth_at(L, f, lx - 1, ly - 1, 0, 1, 1, 0);
        return;
    }
    ol_smooth_line(L, f, 0, 0, 0, -1, -1);
    ol_smooth_line(L, f, 0, ly - 1, 0, 1, -1);
    ol_smooth_line(L, f, 0, ly - 1, lz - 1, 1, 1);
    ol_smooth_line(L, f, 0, 0, lz - 1, -1, 1);
    ol_smooth_line(L, f, 1, 0, 0, -1, -1);
    ol_smooth_line(L, f, 1, lz - 1, 0, 1, -1);
    ol_smooth_line(L, f, 1, lz - 1, lx - 1, 1, 1);
    ol_smooth_line(L, f, 1, 0, lx - 1, -1, 1);
    ol_smooth_line(L, f, 2, 0, 0, -1, -1);
    ol_smooth_line(L, f, 2, lx - 1, 0, 1, -1);
    ol_smooth_line(L, f, 2, lx - 1, ly - 1, 1, 1);
    ol_smooth_line(L, f, 2, 0, ly - 1, -1, 1);
    ol_smooth_at(L, f, 0, 0, 0, -1, -1, -1);
    ol_smooth_at(L, f, lx - 1, 0, 0, 1, -1, -1);
    ol_smooth_at(L, f, lx - 1, ly - 1, 0, 1, 1, -1);
    ol_smooth_at(L, f, 0, ly - 1, 0, -1, 1, -1);
    ol_smooth_at(L, f, 0, 0, lz - 1, -1, -1, 1);
    ol_smooth_at(L, f, lx - 1, 0, lz - 1, 1, -1, 1);
    ol_smooth_at(L, f, lx - 1, ly - 1, lz - 1, 1, 1, 1);
    ol_smooth_at(L, f, 0, ly - 1, lz - 1, -1, 1, 1);
}

/* ---- per-node physics (all arrays are the node's q values) --------------------------- */
/* NS::Macro (navierstokes.h:15-50) */
static void ns_macro(const lat_t *t, const double *f, double *rho, double *u) {
    double r = f[0], m[3] = {0.0, 0.0, 0.0};
    for (int c = 1; c < t->q; ++c) {
        double v = f[c];
        r += v;
        for (int b = 0; b < t->nd; ++b) m[b] += t->c[b][c] * v;
    }
    double inv = 1.0 / r;
    *rho = r;
    for (int b = 0; b < t->nd; ++b) u[b] = m[b] * inv;
    if (t->nd == 2) u[2] = 0.0;
}
/* NS::Equilibrium (navierstokes.h:52-70) */
static void ns_eq(const lat_t *t, double *feq, double rho, const double *u) {
    double uu = (t->nd == 2) ? 1.0 - 1.5 * (u[0] * u[0] + u[1] * u[1])
                             : 1.0 - 1.5 * (u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
    for (int c = 0; c < t->q; ++c) {
        double ciu = (t->nd == 2) ? t->c[0][c] * u[0] + t->c[1][c] * u[1]
                                  : t->c[0][c] * u[0] + t->c[1][c] * u[1] + t->c[2][c] * u[2];
        feq[c] = t->w[c] * rho * (3.0 * ciu + 4.5 * ciu * ciu + uu);
    }
}
static inline double cdot(const lat_t *t, int c, const double *u) {
    return (t->nd == 2) ? t->c[0][c] * u[0] + t->c[1][c] * u[1]
                        : t->c[0][c] * u[0] + t->c[1][c] * u[1] + t->c[2][c] * u[2];
}
static inline double vdot(const lat_t *t, const double *a, const double *b) {
    return (t->nd == 2) ? a[0] * b[0] + a[1] * b[1] : a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}
/* NS::ExternalForceBrinkman (navierstokes.h:72-88) */
static void ns_brinkman(const lat_t *t, double *f, double rho, const double *u, double alpha) {
    double coef = 3.0 * alpha * rho / (rho + alpha);
    for (int c = 1; c < t->q; ++c) f[c] -= coef * t->w[c] * cdot(t, c, u);
}
/* AD::Macro (advection.h:16-51) */
static void ad_macro(const lat_t *t, const double *g, const double *u, double omg, double *tem, double *q) {
    double T_ = g[0], s[3] = {0.0, 0.0, 0.0};
    for (int c = 1; c < t->q; ++c) {
        double v = g[c];
        T_ += v;
        for (int b = 0; b < t->nd; ++b) s[b] += t->c[b][c] * v;
    }
    double coef = 1.0 - 0.5 * omg;
    *tem = T_;
    for (int b = 0; b < t->nd; ++b) q[b] = coef * (s[b] - T_ * u[b]);
    if (t->nd == 2) q[2] = 0.0;
}
/* AD::Equilibrium (advection.h:53-69) */
static void ad_eq(const lat_t *t, double *geq, double tem, const double *u) {
    for (int c = 0; c < t->q; ++c) geq[c] = t->w[c] * tem * (1.0 + 3.0 * cdot(t, c, u));
}
/* AD::ExternalForceNaturalConvection (advection.h:71-85) */
static void ad_nc_force(const lat_t *t, double *f, double tem, const double *gv, double tem0) {
    for (int c = 1; c < t->q; ++c) f[c] += 3.0 * t->w[c] * cdot(t, c, gv) * (tem - tem0);
}
/* AD::ExternalForceHeatExchange (advection.h:87-95) */
static void ad_heatex(const lat_t *t, double *g, double tem, double beta) {
    double coef = beta * (1.0 - tem) / (1.0 + beta);
    g[0] += t->w[0] * coef;
    for (int c = 1; c < t->q; ++c) g[c] += t->w[c] * coef;
}
/* Volumetric heat source (CPU extension, no reference routine; parity unpinned): g_c += w_c Q,
 * the same form as the heat-exchange term above with a fixed source Q */
static void ad_source(const lat_t *t, double *g, double qsrc) {
    for (int c = 0; c < t->q; ++c) g[c] += t->w[c] * qsrc;
}
/* ANS::Macro (adjointnavierstokes.h:15-57) */
static void ans_macro(const lat_t *t, const double *f, const double *u, double *ip, double *iu, double *im) {
    double uu = vdot(t, u, u);
    double w0 = t->w[0];
    *ip = f[0] * w0 * (1.0 - 1.5 * uu);
    for (int b = 0; b < t->nd; ++b) { iu[b] = -f[0] * w0 * u[b]; im[b] = 0.0; }
    for (int c = 1; c < t->q; ++c) {
        double ciu = cdot(t, c, u);
        double fei = f[c] * t->w[c];
        *ip += fei * (1.0 + 3.0 * ciu + 4.5 * ciu * ciu - 1.5 * uu);
        for (int b = 0; b < t->nd; ++b) iu[b] += fei * (t->c[b][c] + 3.0 * ciu * t->c[b][c] - u[b]);
        for (int b = 0; b < t->nd; ++b) im[b] += fei * t->c[b][c];
    }
    if (t->nd == 2) { iu[2] = 0.0; im[2] = 0.0; }
}
/* ANS::Equilibrium (adjointnavierstokes.h:59-73) */
static void ans_eq(const lat_t *t, double *feq, const double *u, double ip, const double *iu) {
    for (int c = 0; c < t->q; ++c) {
        double s = (t->nd == 2)
            ? iu[0] * (t->c[0][c] - u[0]) + iu[1] * (t->c[1][c] - u[1])
            : iu[0] * (t->c[0][c] - u[0]) + iu[1] * (t->c[1][c] - u[1]) + iu[2] * (t->c[2][c] - u[2]);
        feq[c] = ip + 3.0 * s;
    }
}
/* ANS::ExternalForceBrinkman (adjointnavierstokes.h:75-93) */
static void ans_brinkman(const lat_t *t, double *f, double rho, const double *u, const double *im, double alpha) {
    double coef = 3.0 * alpha / (rho + alpha);
    f[0] -= -coef * vdot(t, u, im);
    for (int c = 1; c < t->q; ++c) {
        double s = (t->nd == 2)
            ? (t->c[0][c] - u[0]) * im[0] + (t->c[1][c] - u[1]) * im[1]
            : (t->c[0][c] - u[0]) * im[0] + (t->c[1][c] - u[1]) * im[1] + (t->c[2][c] - u[2]) * im[2];
        f[c] -= coef * s;
    }
}
/* AAD::Macro (adjointadvection.h:22-50) */
static void aad_macro(const lat_t *t, const double *g, double *item, double *iq) {
    double it = t->w[0] * g[0];
    double s[3] = {0.0, 0.0, 0.0};
    for (int c = 1; c < t->q; ++c) {
        double gei = t->w[c] * g[c];
        it += gei;
        for (int b = 0; b < t->nd; ++b) s[b] += gei * t->c[b][c];
    }
    *item = it;
    for (int b = 0; b < 3; ++b) iq[b] = s[b];
}
/* AAD::Equilibrium (adjointadvection.h:52-68) */
static void aad_eq(const lat_t *t, double *geq, double item, const double *iq, const double *u) {
    double coef = item + 3.0 * vdot(t, u, iq);
    for (int c = 0; c < t->q; ++c) geq[c] = coef;
}
/* AAD::ExternalForceBrinkman (adjointadvection.h:70-102) */
static void aad_brinkman(const lat_t *t, double *f, double rho, const double *u, const double *im,
                         double tem, const double *iq, double omg, double alpha) {
    double coef = 3.0 / (rho + alpha);
    double X[3];
    for (int b = 0; b < t->nd; ++b) X[b] = tem * iq[b] * omg - alpha * im[b];
    double s0 = (t->nd == 2) ? -u[0] * X[0] + -u[1] * X[1] : -u[0] * X[0] + -u[1] * X[1] + -u[2] * X[2];
    f[0] += coef * s0;
    for (int c = 1; c < t->q; ++c) {
        double s = (t->nd == 2)
            ? (t->c[0][c] - u[0]) * X[0] + (t->c[1][c] - u[1]) * X[1]
            : (t->c[0][c] - u[0]) * X[0] + (t->c[1][c] - u[1]) * X[1] + (t->c[2][c] - u[2]) * X[2];
        f[c] += coef * s;
    }
}
/* AAD::ExternalForceHeatExchange (adjointadvection.h:104-112) */
static void aad_heatex(const lat_t *t, double *g, double item, double beta) {
    double coef = beta * (1.0 + item) / (1.0 + beta);
    g[0] -= coef;
    for (int c = 1; c < t->q; ++c) g[c] -= coef;
}
/* adjoint source of a volumetric objective J = sum_x w(x) T(x) (CPU extension, parity unpinned):
 * dJ/dg_c = w for every c, added in the convention of AAD::ExternalForceHeatExchange above,
 * whose "1" term is the derivative of its heat-exchange objective */
static void aad_objective_source(const lat_t *t, double *g, double w) {
    for (int c = 0; c < t->q; ++c) g[c] += w;
}
/* AAD::ExternalForceNaturalConvection (adjointadvection.h:114-132) */
static void aad_nc(const lat_t *t, double *g, const double *im, const double *gv) {
    double coef = 3.0 * vdot(t, im, gv);
    g[0] += coef;
    for (int c = 1; c < t->q; ++c) g[c] += coef;
}
/* AAD::ExternalForceMassFlow (adjointadvection.h:134-150) */
static void aad_massflow(const lat_t *t, double *f, double rho, const double *u, const double *dv) {
    f[0] += vdot(t, u, dv) / rho;
    for (int c = 1; c < t->q; ++c) {
        double s = (t->nd == 2)
            ? (t->c[0][c] - u[0]) * dv[0] + (t->c[1][c] - u[1]) * dv[1]
            : (t->c[0][c] - u[0]) * dv[0] + (t->c[1][c] - u[1]) * dv[1] + (t->c[2][c] - u[2]) * dv[2];
        f[c] -= s / rho;
    }
}
static inline void bgk(const lat_t *t, double *f, const double *feq, double om) {
    double iom = 1.0 - om;
    for (int c = 0; c < t->q; ++c) f[c] = iom * f[c] + om * feq[c];
}

/* ---- incompressible variants (D2Q9 only in the reference) ------------------------------ */
/* NSin::Macro (nsincompressible.h:13-25): rho and the momentum sums, no division by rho */
static void nsin_macro(const lat_t *t, const double *f, double *rho, double *u) {
    double r = f[0], m[2] = {0.0, 0.0};
    for (int c = 1; c < t->q; ++c) {
        double v = f[c];
        r += v;
        for (int b = 0; b < 2; ++b) m[b] += t->c[b][c] * v;
    }
    *rho = r;
    u[0] = m[0]; u[1] = m[1]; u[2] = 0.0;
}
/* NSin::Equilibrium (nsincompressible.h:27-35): w (3 c.u + 4.5 (c.u)^2 + rho - 1.5 u.u) */
static void nsin_eq(const lat_t *t, double *feq, double rho, const double *u) {
    double rhouu = rho - 1.5 * (u[0] * u[0] + u[1] * u[1]);
    for (int c = 0; c < t->q; ++c) {
        double ciu = t->c[0][c] * u[0] + t->c[1][c] * u[1];
        feq[c] = t->w[c] * (3.0 * ciu + 4.5 * ciu * ciu + rhouu);
    }
}
/* NSin::ExternalForceBrinkman (nsincompressible.h:37-44) has NS's form: ns_brinkman. */
/* ANSin::Macro (adjointnsincompressible.h:13-30): ip = sum w f, iu_b = sum w f (c_b + 3 (c.u) c_b - u_b),
 * im_b = sum w f c_b */
static void ansin_macro(const lat_t *t, const double *f, const double *u, double *ip, double *iu, double *im) {
    double w0 = t->w[0];
    *ip = f[0] * w0;
    for (int b = 0; b < 2; ++b) { iu[b] = -f[0] * w0 * u[b]; im[b] = 0.0; }
    for (int c = 1; c < t->q; ++c) {
        double ciu = t->c[0][c] * u[0] + t->c[1][c] * u[1];
        double fei = f[c] * t->w[c];
        *ip += fei;
        for (int b = 0; b < 2; ++b) iu[b] += fei * (t->c[b][c] + 3.0 * ciu * t->c[b][c] - u[b]);
        for (int b = 0; b < 2; ++b) im[b] += fei * t->c[b][c];
    }
    iu[2] = 0.0; im[2] = 0.0;
}
/* ANSin::Equilibrium (adjointnsincompressible.h:32-38): ip + 3 iu.c */
static void ansin_eq(const lat_t *t, double *feq, double ip, const double *iu) {
    for (int c = 0; c < t->q; ++c) feq[c] = ip + 3.0 * (iu[0] * t->c[0][c] + iu[1] * t->c[1][c]);
}
/* ANSin::ExternalForceBrinkman (adjointnsincompressible.h:40-47): f_c -= 3 alpha/(1 + alpha) c.im */
static void ansin_brinkman(const lat_t *t, double *f, const double *im, double alpha) {
    double coef = 3.0 * alpha / (1.0 + alpha);
    for (int c = 1; c < t->q; ++c) f[c] -= coef * (t->c[0][c] * im[0] + t->c[1][c] * im[1]);
}

/* ---- elastic LBM (D2Q9 only in the reference) ------------------------------------------- */
/* EL::Macro (elastic.h:17-47): u = (sum_{c>=1} c f) / rho, s_ab = -sum_{c>=1} c_a c_b f; the
 * topology-optimisation overload scales s by gamma. s = {sxx, sxy, syx, syy}. */
static void el_macro(const lat_t *t, const double *f, double rho, double *u, double *s) {
    double ux = 0.0, uy = 0.0, sxx = 0.0, sxy = 0.0, syx = 0.0, syy = 0.0;
    for (int c = 1; c < t->q; ++c) {
        const double v = f[c];
        const int cx = t->c[0][c], cy = t->c[1][c];
        ux += cx * v;
        uy += cy * v;
        sxx -= cx * cx * v;
        sxy -= cx * cy * v;
        syx -= cy * cx * v;
        syy -= cy * cy * v;
    }
    const double invrho = 1.0 / rho;
    u[0] = ux * invrho; u[1] = uy * invrho;
    s[0] = sxx; s[1] = sxy; s[2] = syx; s[3] = syy;
}
/* EL::Equilibrium (elastic.h:49-58): w (3 rho c.u - 4.5 c.s.c + 1.5 tr s) */
static void el_eq(const lat_t *t, double *feq, double rho, const double *u, const double *s) {
    for (int c = 0; c < t->q; ++c) {
        const int cx = t->c[0][c], cy = t->c[1][c];
        const double ciu = cx * u[0] + cy * u[1];
        const double cisci = cx * s[0] * cx + cx * s[1] * cy + cy * s[2] * cx + cy * s[3] * cy;
        const double trss = s[0] + s[3];
        feq[c] = t->w[c] * (3.0 * rho * ciu - 4.5 * cisci + 1.5 * trss);
    }
}
/* AEL::Macro (adjointelastic.h:16-35): irho = sum w f, im = sum w c f, is_ab = sum w c_a c_b f.
 * m = {irho, imx, imy, isxx, isxy, isyx, isyy} */
static void ael_macro(const lat_t *t, const double *f, double *m) {
    double irho = t->w[0] * f[0], imx = 0.0, imy = 0.0, isxx = 0.0, isxy = 0.0, isyx = 0.0, isyy = 0.0;
    for (int c = 1; c < t->q; ++c) {
        const double v = f[c], e = t->w[c];
        const int cx = t->c[0][c], cy = t->c[1][c];
        irho += e * v;
        imx += e * cx * v;
        imy += e * cy * v;
        isxx += e * cx * cx * v;
        isxy += e * cx * cy * v;
        isyx += e * cy * cx * v;
        isyy += e * cy * cy * v;
    }
    m[0] = irho; m[1] = imx; m[2] = imy; m[3] = isxx; m[4] = isxy; m[5] = isyx; m[6] = isyy;
}
/* AEL::Equilibrium (adjointelastic.h:37-46): 3 im.c + 4.5 gamma c.is.c - 1.5 gamma irho |c|^2 */
static void ael_eq(const lat_t *t, double *feq, const double *m, double gamma) {
    for (int c = 0; c < t->q; ++c) {
        const int cx = t->c[0][c], cy = t->c[1][c];
        const double imc = m[1] * cx + m[2] * cy;
        const double cisc = cx * m[3] * cx + cx * m[4] * cy + cy * m[5] * cx + cy * m[6] * cy;
        const double irhocc = m[0] * (cx * cx + cy * cy);
        feq[c] = 3.0 * imc + 4.5 * gamma * cisc - 1.5 * gamma * irhocc;
    }
}

/* ---- collide kernels ------------------------------------------------------------------
 * NS::MacroCollide / MacroBrinkmanCollide (navierstokes.h:430-546)
 * AD::MacroCollide{Force,Natural}Convection (advection.h:528-712),
 *     MacroBrinkmanCollide{HeatExchange,ForceConvection,NaturalConvection} (714-1044)
 * ANS::MacroBrinkmanCollide (adjointnavierstokes.h:396-470)
 * AAD::MacroBrinkmanCollide{HeatExchange,ForceConvection,NaturalConvection,
 *     NaturalConvectionMassFlow} (adjointadvection.h:892-1355)
 * NSin::MacroCollide / MacroBrinkmanCollide (nsincompressible.h:144-200),
 * ANSin::MacroBrinkmanCollide (adjointnsincompressible.h:143-178)
 * EL::MacroCollide / MacroExtendedCollide (elastic.h:109-166), AEL::MacroCollide
 * (adjointelastic.h:96-125) */
void ol_collide(const ol_lat *L, int kind, double *fa, double *ga, const ol_fields *Fd, const ol_phys *P, int save) {
    lat_t T = mk(L); const lat_t *t = &T;
    const int n = t->n, q = t->q, nd = t->nd;
    const double omf = 1.0 / (3.0 * P->nu + 0.5);
    const double gv[3] = {P->gx, P->gy, P->gz};
#pragma omp parallel for schedule(static)
    for (int idx = 0; idx < n; ++idx) {
        double f[15], g[15], feq[15], geq[15];
        for (int c = 0; c < q; ++c) f[c] = fa[(size_t)c * n + idx];
        if (ga) for (int c = 0; c < q; ++c) g[c] = ga[(size_t)c * n + idx];
        double omg = 0.0;
        if (kind == OL_AD_NATURAL || kind == OL_AD_FORCE || kind == OL_AAD_NATURAL || kind == OL_AAD_FORCE ||
            kind == OL_AAD_MASSFLOW)
            omg = 1.0 / (3.0 * Fd->diffusivity[idx] + 0.5);
        else if (ga)
            omg = 1.0 / (3.0 * P->diff + 0.5);
        if (kind == OL_EL_COLLIDE || kind == OL_EL_EXTENDED) {
            /* EL::MacroCollide / MacroExtendedCollide (elastic.h:109-166), omega = 1 / tau */
            const double rho = Fd->rho[idx], om = 1.0 / P->tau;
            double u[2], sg[4];
            el_macro(t, f, rho, u, sg);
            if (kind == OL_EL_EXTENDED) {
                const double gm = Fd->gamma[idx];
                for (int m = 0; m < 4; ++m) sg[m] *= gm;
            }
            if (save) {
                Fd->ux[idx] = u[0]; Fd->uy[idx] = u[1];
                Fd->sxx[idx] = sg[0]; Fd->sxy[idx] = sg[1]; Fd->syx[idx] = sg[2]; Fd->syy[idx] = sg[3];
            }
            el_eq(t, feq, rho, u, sg);
            bgk(t, f, feq, om);
        } else if (kind == OL_AEL_COLLIDE) {
            /* AEL::MacroCollide (adjointelastic.h:96-125) */
            const double om = 1.0 / P->tau;
            double m[7];
            ael_macro(t, f, m);
            if (save) {
                Fd->ip[idx] = m[0]; Fd->imx[idx] = m[1]; Fd->imy[idx] = m[2];
                Fd->isxx[idx] = m[3]; Fd->isxy[idx] = m[4]; Fd->isyx[idx] = m[5]; Fd->isyy[idx] = m[6];
            }
            ael_eq(t, feq, m, Fd->gamma[idx]);
            bgk(t, f, feq, om);
        } else if (kind == OL_NSIN_COLLIDE || kind == OL_NSIN_BRINKMAN) {
            double rho, u[3];
            nsin_macro(t, f, &rho, u);
            if (kind == OL_NSIN_BRINKMAN) {
                ns_brinkman(t, f, rho, u, Fd->alpha[idx]);
                nsin_macro(t, f, &rho, u);
            }
            if (save) { Fd->rho[idx] = rho; Fd->ux[idx] = u[0]; Fd->uy[idx] = u[1]; }
            nsin_eq(t, feq, rho, u);
            bgk(t, f, feq, omf);
        } else if (kind == OL_ANSIN_BRINKMAN) {
            double u[3] = {Fd->ux[idx], Fd->uy[idx], 0.0};
            double ip, iu[3], im[3];
            ansin_macro(t, f, u, &ip, iu, im);
            ansin_brinkman(t, f, im, Fd->alpha[idx]);
            ansin_macro(t, f, u, &ip, iu, im);
            if (save) {
                Fd->ip[idx] = ip; Fd->iux[idx] = iu[0]; Fd->iuy[idx] = iu[1];
                Fd->imx[idx] = im[0]; Fd->imy[idx] = im[1];
            }
            ansin_eq(t, feq, ip, iu);
            bgk(t, f, feq, omf);
        } else if (kind <= OL_AD_FORCE_NOBRINK) {
            double rho, u[3], tem = 0.0, qv[3] = {0, 0, 0};
            ns_macro(t, f, &rho, u);
            if (ga) ad_macro(t, g, u, omg, &tem, qv);
            if (kind == OL_NS_BRINKMAN || kind == OL_AD_FORCE || kind == OL_AD_HEATEX) {
                ns_brinkman(t, f, rho, u, Fd->alpha[idx]);
                ns_macro(t, f, &rho, u);
                if (kind == OL_AD_HEATEX) ad_heatex(t, g, tem, Fd->beta[idx]);
                if (kind == OL_AD_FORCE && Fd->hsrc) ad_source(t, g, Fd->hsrc[idx]);
                if (ga) ad_macro(t, g, u, omg, &tem, qv);
            } else if (kind == OL_AD_NATURAL) {
                ad_nc_force(t, f, tem, gv, P->tem0);
                ns_brinkman(t, f, rho, u, Fd->alpha[idx]);
                ns_macro(t, f, &rho, u);
                ad_macro(t, g, u, omg, &tem, qv);
            } else if (kind == OL_AD_NATURAL_NOBRINK) {
                ad_nc_force(t, f, tem, gv, P->tem0);
                ns_macro(t, f, &rho, u);
                ad_macro(t, g, u, omg, &tem, qv);
            }
            if (save) {
                Fd->rho[idx] = rho; Fd->ux[idx] = u[0]; Fd->uy[idx] = u[1]; if (nd == 3) Fd->uz[idx] = u[2];
                if (ga) {
                    Fd->tem[idx] = tem; Fd->qx[idx] = qv[0]; Fd->qy[idx] = qv[1]; if (nd == 3) Fd->qz[idx] = qv[2];
                    if (Fd->gsnap && (kind == OL_AD_NATURAL || kind == OL_AD_FORCE))
                        for (int c = 0; c < q; ++c) Fd->gsnap[(size_t)q * idx + c] = g[c];
                }
            }
            ns_eq(t, feq, rho, u);
            bgk(t, f, feq, omf);
            if (ga) { ad_eq(t, geq, tem, u); bgk(t, g, geq, omg); }
        } else {
            double rho = Fd->rho[idx];
            double u[3] = {Fd->ux[idx], Fd->uy[idx], nd == 3 ? Fd->uz[idx] : 0.0};
            double ip, iu[3], im[3], item = 0.0, iq[3] = {0, 0, 0};
            ans_macro(t, f, u, &ip, iu, im);
            if (kind == OL_ANS_BRINKMAN) {
                ans_brinkman(t, f, rho, u, im, Fd->alpha[idx]);
                ans_macro(t, f, u, &ip, iu, im);
            } else {
                double tem = Fd->tem[idx];
                aad_macro(t, g, &item, iq);
                if (kind == OL_AAD_MASSFLOW) {
                    double dv[3] = {Fd->dirx[idx], Fd->diry[idx], nd == 3 ? Fd->dirz[idx] : 0.0};
                    aad_massflow(t, f, rho, u, dv);
                }
                aad_brinkman(t, f, rho, u, im, tem, iq, omg, Fd->alpha[idx]);
                ans_macro(t, f, u, &ip, iu, im);
                if (kind == OL_AAD_NATURAL || kind == OL_AAD_MASSFLOW) {
                    aad_nc(t, g, im, gv);
                    aad_macro(t, g, &item, iq);
                } else if (kind == OL_AAD_HEATEX) {
                    aad_heatex(t, g, item, Fd->beta[idx]);
                    aad_macro(t, g, &item, iq);
                } else if (kind == OL_AAD_FORCE && Fd->objw) {
                    aad_objective_source(t, g, Fd->objw[idx]);
                    aad_macro(t, g, &item, iq);
                }
            }
            if (save) {
                Fd->ip[idx] = ip; Fd->iux[idx] = iu[0]; Fd->iuy[idx] = iu[1];
                Fd->imx[idx] = im[0]; Fd->imy[idx] = im[1];
                /* the D3Q15 ForceConvection adjoint never stores iuz (adjointadvection.h:1074-1084) */
                if (nd == 3) { if (kind != OL_AAD_FORCE) Fd->iuz[idx] = iu[2]; Fd->imz[idx] = im[2]; }
                if (ga) {
                    Fd->item[idx] = item; Fd->iqx[idx] = iq[0]; Fd->iqy[idx] = iq[1]; if (nd == 3) Fd->iqz[idx] = iq[2];
                    if (Fd->gsnap && kind != OL_AAD_HEATEX)
                        for (int c = 0; c < q; ++c) Fd->gsnap[(size_t)q * idx + c] = g[c];
                }
            }
            ans_eq(t, feq, u, ip, iu);
            bgk(t, f, feq, omf);
            if (ga) { aad_eq(t, geq, item, iq, u); bgk(t, g, geq, omg); }
        }
        for (int c = 0; c < q; ++c) fa[(size_t)c * n + idx] = f[c];
        if (ga) for (int c = 0; c < q; ++c) ga[(size_t)c * n + idx] = g[c];
    }
}

/* ---- initial conditions: NS::InitialCondition (navierstokes.h:548-572), AD:: (advection.h:
 *      1046-1070), ANS:: (adjointnavierstokes.h:472-498), AAD:: (adjointadvection.h:1357-1381),
 *      NSin:: (nsincompressible.h:202-212), ANSin:: (adjointnsincompressible.h:180-192),
 *      EL:: (elastic.h:168-179), AEL:: (adjointelastic.h:127-138) */
void ol_init(const ol_lat *L, int which, double *fa, const ol_fields *Fd) {
    lat_t T = mk(L); const lat_t *t = &T;
    const int n = t->n, q = t->q, nd = t->nd;
#pragma omp parallel for schedule(static)
    for (int idx = 0; idx < n; ++idx) {
        double eq[15];
        if (which == 6) {
            const double u[2] = {Fd->ux[idx], Fd->uy[idx]};
            const double sg[4] = {Fd->sxx[idx], Fd->sxy[idx], Fd->syx[idx], Fd->syy[idx]};
            el_eq(t, eq, Fd->rho[idx], u, sg);
            for (int c = 0; c < q; ++c) fa[(size_t)c * n + idx] = eq[c];
            continue;
        }
        if (which == 7) {
            const double m[7] = {Fd->ip[idx], Fd->imx[idx], Fd->imy[idx], Fd->isxx[idx], Fd->isxy[idx],
                                 Fd->isyx[idx], Fd->isyy[idx]};
            ael_eq(t, eq, m, Fd->gamma[idx]);
            for (int c = 0; c < q; ++c) fa[(size_t)c * n + idx] = eq[c];
            continue;
        }
        double u[3] = {Fd->ux[idx], Fd->uy[idx], nd == 3 ? Fd->uz[idx] : 0.0};
        if (which == 0) ns_eq(t, eq, Fd->rho[idx], u);
        else if (which == 1) ad_eq(t, eq, Fd->tem[idx], u);
        else if (which == 2) {
            double iu[3] = {Fd->iux[idx], Fd->iuy[idx], nd == 3 ? Fd->iuz[idx] : 0.0};
            ans_eq(t, eq, u, Fd->ip[idx], iu);
        } else if (which == 4) {
            nsin_eq(t, eq, Fd->rho[idx], u);
        } else if (which == 5) {
            double iu[3] = {Fd->iux[idx], Fd->iuy[idx], 0.0};
            ansin_eq(t, eq, Fd->ip[idx], iu);
        } else {
            double iq[3] = {Fd->iqx[idx], Fd->iqy[idx], nd == 3 ? Fd->iqz[idx] : 0.0};
            aad_eq(t, eq, Fd->item[idx], iq, u);
        }
        for (int c = 0; c < q; ++c) fa[(size_t)c * n + idx] = eq[c];
    }
}

/* ---- sensitivities --------------------------------------------------------------------
 * AAD::SensitivityTemperatureAtHeatSource (adjointadvection.h:1495-1543) with boundary terms
 * (753-888). The D3Q15 scalar overload passes (_ux,_uy,_uz,_ig) into parameters declared
 * (_ux,_uy,_ig,_uz) (adjointadvection.h:805 vs 1537); the production drivers use the AVX
 * overload (adjointadvection_avx.h:81-186, 1459-1513) whose order is correct, and that
 * order is restated here. The +y / +-z D3Q15 terms carry no factor 3.0 on the tangential
 * velocities (adjointadvection.h:851-852, 874-875, 880-881), kept. */
void ol_sensitivity(const ol_lat *L, int which, double *dfds, const ol_fields *Fd, const double *dads,
                    const double *dkds, const double *g, const double *ig, const double *qn, const int *mask) {
    lat_t T = mk(L); const lat_t *t = &T;
    const int n = t->n, q = t->q, nd = t->nd;
    if (which == 4) {
        /* AEL::SensitivityCompliance (adjointelastic.h:149-155) */
        for (int idx = 0; idx < n; ++idx)
            dfds[idx] += (4.5 * (Fd->sxx[idx] * Fd->isxx[idx] + Fd->sxy[idx] * Fd->isxy[idx] +
                                 Fd->syx[idx] * Fd->isyx[idx] + Fd->syy[idx] * Fd->isyy[idx]) -
                          1.5 * Fd->ip[idx] * (Fd->sxx[idx] + Fd->syy[idx]));
        return;
    }
    for (int idx = 0; idx < n; ++idx) {
        double u[3] = {Fd->ux[idx], Fd->uy[idx], nd == 3 ? Fd->uz[idx] : 0.0};
        double im[3] = {Fd->imx[idx], Fd->imy[idx], nd == 3 ? Fd->imz[idx] : 0.0};
        if (which == 3) { dfds[idx] += 3.0 * dads[idx] * vdot(t, u, im); continue; }
        if (which == 2) {
            dfds[idx] += 3.0 * dads[idx] * vdot(t, u, im) - dkds[idx] * (1.0 - Fd->tem[idx]) * (1.0 + Fd->item[idx]);
            continue;
        }
        dfds[idx] += 3.0 * dads[idx] * vdot(t, u, im);
        double sumg = 0.0;
        for (int c = 0; c < q; ++c) sumg += g[(size_t)q * idx + c] * ig[(size_t)q * idx + c];
        double iq[3] = {Fd->iqx[idx], Fd->iqy[idx], nd == 3 ? Fd->iqz[idx] : 0.0};
        dfds[idx] += -3.0 / pow(3.0 * Fd->diffusivity[idx] + 0.5, 2.0) * dkds[idx] *
                     (sumg - Fd->tem[idx] * (Fd->item[idx] + 3.0 * vdot(t, u, iq)));
    }
    if (which != 0) return;
    /* boundary terms on each side of each axis, in the reference order xmin, xmax, ymin, ... */
    int lens[3] = {t->nx, t->ny, t->nz};
    for (int a = 0; a < nd; ++a) {
        for (int s = 0; s < 2; ++s) {
            int d = s == 0 ? -1 : 1, p = s == 0 ? 0 : lens[a] - 1;
            int b = (a + 1) % 3, cc = (a + 2) % 3;
            int nb = (nd == 2 && b == 2) ? 1 : lens[b], nc2 = (nd == 2 && cc == 2) ? 1 : lens[cc];
            for (int uu = 0; uu < nb; ++uu)
                for (int vv = 0; vv < nc2; ++vv) {
                    int x[3]; x[a] = p; x[b] = uu; x[cc] = vv;
                    if (nd == 2) x[2] = 0;
                    int idx = IDX(t, x[0], x[1], x[2]);
                    if (!mask[idx]) continue;
                    double u[3] = {Fd->ux[idx], Fd->uy[idx], nd == 3 ? Fd->uz[idx] : 0.0};
                    const double *igp = ig + (size_t)q * idx;
                    int nin = -d;
                    double pre = nin > 0 ? 1.0 + 3.0 * u[a] : 1.0 - 3.0 * u[a];
                    double post = nin > 0 ? 1.0 - 3.0 * u[a] : 1.0 + 3.0 * u[a];
                    /* inward set of the snapshot: normal (x kc) + diagonals, increasing c */
                    double ns = 0.0, kc = nd == 2 ? 4.0 : 8.0;
                    for (int c = 1; c < q; ++c) {
                        if (t->c[a][c] != -d) continue;
                        int diag = 0; for (int e = 0; e < nd; ++e) if (e != a && t->c[e][c] != 0) diag = 1;
                        if (!diag) ns = (nd == 2 ? -6.0 : -12.0) + kc * igp[c];
                    }
                    for (int c = 1; c < q; ++c) {
                        if (t->c[a][c] != -d) continue;
                        int diag = 0; for (int e = 0; e < nd; ++e) if (e != a && t->c[e][c] != 0) diag = 1;
                        if (diag) ns += igp[c];
                    }
                    double num;
                    if (nd == 2) {
                        int bb = 1 - a;
                        double ts = 0.0;
                        for (int c = 1; c < q; ++c) {
                            if (t->c[a][c] != -d || t->c[bb][c] == 0) continue;
                            ts = (t->c[bb][c] > 0) ? ts + igp[c] : ts - igp[c];
                        }
                        num = pre * ns + 3.0 * u[bb] * ts;
                        dfds[idx] += qn[idx] * dkds[idx] * num / (36.0 * post * pow(Fd->diffusivity[idx], 2.0));
                    } else {
                        const int *tb = TANG3(a);
                        double k3 = (a == 0 || (a == 1 && d < 0)) ? 3.0 : 1.0;
                        double ts0 = 0.0, ts1 = 0.0;
                        for (int c = 1; c < q; ++c) {
                            if (t->c[a][c] != -d) continue;
                            int diag = 0; for (int e = 0; e < nd; ++e) if (e != a && t->c[e][c] != 0) diag = 1;
                            if (!diag) continue;
                            ts0 = (t->c[tb[0]][c] > 0) ? ts0 + igp[c] : ts0 - igp[c];
                            ts1 = (t->c[tb[1]][c] > 0) ? ts1 + igp[c] : ts1 - igp[c];
                        }
                        if (k3 == 3.0) num = pre * ns + 3.0 * u[tb[0]] * ts0 + 3.0 * u[tb[1]] * ts1;
                        else num = pre * ns + u[tb[0]] * ts0 + u[tb[1]] * ts1;
                        dfds[idx] += qn[idx] * dkds[idx] * num / (72.0 * post * pow(Fd->diffusivity[idx], 2.0));
                    }
                }
        }
    }
}

/* ---- filters ----------------------------------------------------------------------------
 * HeavisideFilter::GetFilteredVariable (heavisidefilter.h:404-579, projection at :560),
 * GetFilteredSensitivity (586-899: chain rule, then a second pass normalised by the target
 * cell's weight sum), DensityFilter::GetFilteredValue (densityfilter.h:10-515). No periodic
 * wrap: taps outside the lattice are skipped. */
static double fweight(const lat_t *t, double R, const int *mask, int i1, int j1, int k1, int i2, int j2, int k2) {
    if (!mask || (mask[IDX(t, i1, j1, k1)] && mask[i2 + t->nx * (j2 + t->ny * k2)]))
        return (R - sqrt(pow(i1 - i2, 2.0) + pow(j1 - j2, 2.0) + pow(k1 - k2, 2.0))) / R;
    return (i1 == i2 && j1 == j2 && k1 == k2) ? 1.0 : 0.0;
}
typedef struct { double ws, w; } wsum_t;
static wsum_t filt_at(const lat_t *t, double R, const double *v, const int *mask, int i1, int j1, int k1) {
    int nR = (int)R;
    wsum_t r = {0.0, 0.0};
    for (int i2 = i1 - nR; i2 <= i1 + nR; ++i2)
        for (int j2 = j1 - nR; j2 <= j1 + nR; ++j2)
            for (int k2 = k1 - nR; k2 <= k1 + nR; ++k2) {
                double dist = sqrt(pow(i1 - i2, 2.0) + pow(j1 - j2, 2.0) + pow(k1 - k2, 2.0));
                if (dist > R) continue;
                if (i2 < 0 || i2 >= t->nx || j2 < 0 || j2 >= t->ny || k2 < 0 || k2 >= t->nz) continue;
                double w = fweight(t, R, mask, i1, j1, k1, i2, j2, k2);
                r.ws += w * v[i2 + t->nx * (j2 + t->ny * k2)];
                r.w += w;
            }
    return r;
}
void ol_heaviside_var(const ol_lat *L, double R, double beta, const double *s, const int *mask, double *out) {
    lat_t T = mk(L); const lat_t *t = &T;
#pragma omp parallel for collapse(2)
    for (int k = 0; k < t->nz; ++k)
        for (int j = 0; j < t->ny; ++j)
            for (int i = 0; i < t->nx; ++i) {
                wsum_t r = filt_at(t, R, s, mask, i, j, k);
                out[IDX(t, i, j, k)] = 0.5 * (tanh(0.5 * beta) + tanh(beta * (r.ws / r.w - 0.5))) / tanh(0.5 * beta);
            }
}
void ol_heaviside_sens(const ol_lat *L, double R, double beta, const double *s, const double *dfdrho,
                       const int *mask, double *out) {
    lat_t T = mk(L); const lat_t *t = &T;
    double *tmp = (double *)malloc(sizeof(double) * (size_t)t->n);
#pragma omp parallel for collapse(2)
    for (int k = 0; k < t->nz; ++k)
        for (int j = 0; j < t->ny; ++j)
            for (int i = 0; i < t->nx; ++i) {
                wsum_t r = filt_at(t, R, s, mask, i, j, k);
                int idx = IDX(t, i, j, k);
                double d = 0.5 * beta * (1.0 - pow(tanh(beta * (r.ws / r.w - 0.5)), 2.0)) / tanh(0.5 * beta);
                tmp[idx] = dfdrho[idx] * d;
            }
#pragma omp parallel for collapse(2)
    for (int k = 0; k < t->nz; ++k)
        for (int j = 0; j < t->ny; ++j)
            for (int i = 0; i < t->nx; ++i) {
                wsum_t r = filt_at(t, R, tmp, mask, i, j, k);
                out[IDX(t, i, j, k)] = r.ws / r.w;
            }
    free(tmp);
}
void ol_density_filter(const ol_lat *L, double R, const double *v, const int *mask, double *out) {
    lat_t T = mk(L); const lat_t *t = &T;
#pragma omp parallel for collapse(2)
    for (int k = 0; k < t->nz; ++k)
        for (int j = 0; j < t->ny; ++j)
            for (int i = 0; i < t->nx; ++i) {
                wsum_t r = filt_at(t, R, v, mask, i, j, k);
                out[IDX(t, i, j, k)] = r.ws / r.w;
            }
}

/* Filters with a general weight functor (heavisidefilter.h:452-475, 770-800; densityfilter.h):
 * the functor's values come as a table w[node][tap], the taps being the offsets with distance
 * <= R in the (i2, j2, k2) loop order (2D: k2 = k1 only); out-of-lattice taps are skipped. */
static int ntaps(const lat_t *t, double R) {
    int nR = (int)R, m = 0;
    for (int a = -nR; a <= nR; ++a)
        for (int b = -nR; b <= nR; ++b)
            for (int c = (t->nd == 3 ? -nR : 0); c <= (t->nd == 3 ? nR : 0); ++c)
                if (sqrt(pow((double)a, 2.0) + pow((double)b, 2.0) + pow((double)c, 2.0)) <= R) ++m;
    return m;
}
static wsum_t filt_tab(const lat_t *t, double R, const double *v, const double *w, int ntap, int i1, int j1, int k1) {
    int nR = (int)R, tap = 0;
    size_t row = (size_t)IDX(t, i1, j1, k1) * (size_t)ntap;
    wsum_t r = {0.0, 0.0};
    for (int i2 = i1 - nR; i2 <= i1 + nR; ++i2)
        for (int j2 = j1 - nR; j2 <= j1 + nR; ++j2)
            for (int k2 = (t->nd == 3 ? k1 - nR : k1); k2 <= (t->nd == 3 ? k1 + nR : k1); ++k2) {
                double dist = sqrt(pow(i1 - i2, 2.0) + pow(j1 - j2, 2.0) + pow(k1 - k2, 2.0));
                if (dist > R) continue;
                int tp = tap++;
                if (i2 < 0 || i2 >= t->nx || j2 < 0 || j2 >= t->ny || k2 < 0 || k2 >= t->nz) continue;
                double wt = w[row + tp];
                r.ws += wt * v[i2 + t->nx * (j2 + t->ny * k2)];
                r.w += wt;
            }
    return r;
}
int ol_filter_ntaps(const ol_lat *L, double R) { lat_t T = mk(L); return ntaps(&T, R); }
void ol_filter_table(const ol_lat *L, int op, double R, double beta, const double *a, const double *b,
                     const double *w, double *out) {
    lat_t T = mk(L); const lat_t *t = &T;
    int nt = ntaps(t, R);
    double *tmp = NULL;
    if (op == 1) tmp = (double *)malloc(sizeof(double) * (size_t)t->n);
#pragma omp parallel for collapse(2)
    for (int k = 0; k < t->nz; ++k)
        for (int j = 0; j < t->ny; ++j)
            for (int i = 0; i < t->nx; ++i) {
                wsum_t r = filt_tab(t, R, a, w, nt, i, j, k);
                int idx = IDX(t, i, j, k);
                if (op == 0) out[idx] = 0.5 * (tanh(0.5 * beta) + tanh(beta * (r.ws / r.w - 0.5))) / tanh(0.5 * beta);
                else if (op == 1) tmp[idx] = b[idx] * (0.5 * beta * (1.0 - pow(tanh(beta * (r.ws / r.w - 0.5)), 2.0)) / tanh(0.5 * beta));
                else out[idx] = r.ws / r.w;
            }
    if (op == 1) {
#pragma omp parallel for collapse(2)
        for (int k = 0; k < t->nz; ++k)
            for (int j = 0; j < t->ny; ++j)
                for (int i = 0; i < t->nx; ++i) {
                    wsum_t r = filt_tab(t, R, tmp, w, nt, i, j, k);
                    out[IDX(t, i, j, k)] = r.ws / r.w;
                }
        free(tmp);
    }
}

/* ---- Residual (residual.h:8-51) / Normalize (normalize.h:8-23) ------------------------- */
double ol_residual(int n, int ncomp, const double *const *a, const double *const *b) {
    double s0 = 0.0, s1 = 0.0;
    for (int idx = 0; idx < n; ++idx) {
        double d0 = 0.0, d1 = 0.0;
        for (int m = 0; m < ncomp; ++m) {
            double e = pow(a[m][idx] - b[m][idx], 2.0), v = pow(a[m][idx], 2.0);
            if (m == 0) { d0 = e; d1 = v; } else { d0 += e; d1 += v; }
        }
        s0 += d0;
        s1 += d1;
    }
    return sqrt(s0 / s1);
}
void ol_normalize(double *v, int n) {
    double vmax = 0.0;
    for (int idx = 0; idx < n; ++idx) if (vmax < fabs(v[idx])) vmax = fabs(v[idx]);
    for (int idx = 0; idx < n; ++idx) v[idx] /= vmax;
}
