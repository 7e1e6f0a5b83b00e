/*
 * oracle.h -- CPU restatement of PANSLBM2's lattice-Boltzmann topology-optimisation
 * hot path (TEST INFRASTRUCTURE ONLY).
 *
 * This header is implemented twice:
 *   - oracle.c        : a plain-C restatement of the reference algorithm (FP64, OpenMP);
 *   - ref_harness.cpp : a thin wrapper that calls the reference's own header templates
 *                       (built only where the reference sources are present).
 * Tests compare the two call-for-call, then use the restatement as the checker for the
 * CUDA library. Nothing in the product path links or calls this code.
 *
 * Conventions (this oracle's own, not the reference's):
 *   - populations are structure-of-arrays, rest population included:
 *       f[c*N + idx], c = 0..q-1, idx = i + nx*j + nx*ny*k;
 *   - the g / ig snapshot arrays use the reference's scalar layout snap[q*idx + c];
 *   - per-node functor values are passed as full-lattice arrays (value at node idx);
 *   - 2D lattices have nz == 1 and ignore z arguments.
 */
#ifndef PANSLBM_ORACLE_H
#define PANSLBM_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct { int q, nx, ny, nz; } ol_lat;

/* Field bundle passed to collide / init / sensitivity routines. Unused members may be NULL. */
typedef struct {
    double *rho, *ux, *uy, *uz;                 /* NS macros                                   */
    double *tem, *qx, *qy, *qz;                 /* AD macros                                   */
    double *ip, *iux, *iuy, *iuz;               /* ANS adjoint pressure / velocity             */
    double *imx, *imy, *imz;                    /* ANS adjoint momentum                        */
    double *item, *iqx, *iqy, *iqz;             /* AAD adjoint temperature / flux              */
    const double *alpha;                        /* Brinkman resistance alpha[N]                */
    const double *diffusivity;                  /* per-node diffusivity kappa[N]               */
    const double *beta;                         /* heat-exchange coefficient beta[N]           */
    const double *dirx, *diry, *dirz;           /* mass-flow objective direction weights       */
    double *gsnap;                              /* g (fwd) / ig (adj) snapshot, snap[q*idx+c]  */
    /* elastic kinds (D2Q9): EL reads rho as its density input and saves ux, uy and the stress
     * sxx..syy; AEL saves irho in ip, imx / imy in imx / imy and the adjoint stress isxx..isyy */
    double *sxx, *sxy, *syx, *syy;
    double *isxx, *isxy, *isyx, *isyy;
    const double *gamma;                        /* stress scale gamma[N] (EL extended, AEL)    */
    /* CPU extension for the forced-convection heat-sink configurations (no reference routine;
     * parity vs the reference unpinned, this restatement is the oracle): with OL_AD_FORCE,
     * hsrc[idx] is a volumetric heat source added as w_c * hsrc to g before the final AD macro;
     * with OL_AAD_FORCE, objw[idx] = dJ/dT of a volumetric objective J = sum objw * T, added to
     * every adjoint g population before a final AAD macro. NULL = off (the reference routine). */
    const double *hsrc;
    const double *objw;
} ol_fields;

typedef struct {
    double nu;              /* kinematic viscosity                      */
    double diff;            /* constant diffusivity (siblings that take a scalar kappa) */
    double gx, gy, gz;      /* buoyancy vector                          */
    double tem0;            /* reference temperature                    */
    double tau;             /* relaxation time of the elastic kinds     */
} ol_phys;

/* Collide kinds */
enum {
    OL_NS_COLLIDE = 0,            /* NS::MacroCollide                                    */
    OL_NS_BRINKMAN = 1,           /* NS::MacroBrinkmanCollide                            */
    OL_AD_NATURAL = 2,            /* AD::MacroBrinkmanCollideNaturalConvection           */
    OL_AD_FORCE = 3,              /* AD::MacroBrinkmanCollideForceConvection             */
    OL_AD_HEATEX = 4,             /* AD::MacroBrinkmanCollideHeatExchange                */
    OL_AD_NATURAL_NOBRINK = 5,    /* AD::MacroCollideNaturalConvection                   */
    OL_AD_FORCE_NOBRINK = 6,      /* AD::MacroCollideForceConvection                     */
    OL_NSIN_COLLIDE = 7,          /* NSin::MacroCollide (D2Q9)                           */
    OL_NSIN_BRINKMAN = 8,         /* NSin::MacroBrinkmanCollide (D2Q9)                   */
    OL_ANS_BRINKMAN = 10,         /* ANS::MacroBrinkmanCollide                           */
    OL_AAD_NATURAL = 11,          /* AAD::MacroBrinkmanCollideNaturalConvection          */
    OL_AAD_FORCE = 12,            /* AAD::MacroBrinkmanCollideForceConvection            */
    OL_AAD_HEATEX = 13,           /* AAD::MacroBrinkmanCollideHeatExchange               */
    OL_AAD_MASSFLOW = 14,         /* AAD::MacroBrinkmanCollideNaturalConvectionMassFlow  */
    OL_ANSIN_BRINKMAN = 15,       /* ANSin::MacroBrinkmanCollide (D2Q9)                  */
    OL_EL_COLLIDE = 16,           /* EL::MacroCollide (D2Q9)                             */
    OL_EL_EXTENDED = 17,          /* EL::MacroExtendedCollide (D2Q9)                     */
    OL_AEL_COLLIDE = 18           /* AEL::MacroCollide (D2Q9)                            */
};

/* Boundary-condition kinds applied along one edge (2D) / face (3D) */
enum {
    OL_BC_WALL = 0,       /* BoundaryConditionAlong*  (type[] : 1 BARRIER, 2 MIRROR)         */
    OL_BC_IWALL = 1,      /* iBoundaryConditionAlong*                                        */
    OL_BC_NS_U = 2,       /* NS::BoundaryConditionSetUAlong*     (v0,v1,v2 = ux,uy,uz)        */
    OL_BC_NS_RHO = 3,     /* NS::BoundaryConditionSetRhoAlong*   (v0 = rho, v1 = us, v2 = ut) */
    OL_BC_AD_T = 4,       /* AD::BoundaryConditionSetTAlong*     (v0 = T)                    */
    OL_BC_AD_Q = 5,       /* AD::BoundaryConditionSetQAlong*     (v0 = qn, per-node kappa)   */
    OL_BC_AD_QC = 6,      /* AD::BoundaryConditionSetQAlong*     (v0 = qn, constant kappa)   */
    OL_BC_ANS_U = 7,      /* ANS::iBoundaryConditionSetUAlong*   (v0,v1,v2 = ux,uy,uz; eps)  */
    OL_BC_ANS_RHO = 8,    /* ANS::iBoundaryConditionSetRhoAlong*                             */
    OL_BC_AAD_T = 9,      /* AAD::iBoundaryConditionSetTAlong*                               */
    OL_BC_AAD_Q = 10,     /* AAD::iBoundaryConditionSetQAlong*   (eps)                       */
    OL_BC_AAD_RHO = 11,   /* AAD::iBoundaryConditionSetRhoAlong* (type[]: 1 SetT, 2 SetQ; eps; acts on f and g) */
    OL_BC_NSIN_U = 12,    /* NSin::BoundaryConditionSetUAlong{X,Y}Edge   (v0,v1 = ux,uy)     */
    OL_BC_NSIN_RHO = 13,  /* NSin::BoundaryConditionSetRhoAlong{X,Y}Edge (v0 = rho, v1 = us) */
    OL_BC_ANSIN_U = 14,   /* ANSin::iBoundaryConditionSetUAlong{X,Y}Edge (eps); ANSin's iSetRho
                           * is ANS's (OL_BC_ANS_RHO)                                      */
    OL_BC_EL_STRESS = 15, /* EL::BoundaryConditionSetStressAlong{X,Y}Edge   (v0,v1 = tx,ty)  */
    OL_BC_AEL_STRESS = 16 /* AEL::iBoundaryConditionSetStressAlong{X,Y}Edge (v0,v1 = tx,ty; rho) */
};

typedef struct {
    int kind;               /* OL_BC_*                                               */
    int axis;               /* 0 = x, 1 = y, 2 = z                                    */
    int pos;                /* global index of the edge / face along axis             */
    int dir;                /* -1 (min side) or +1 (max side)                         */
    const int *type;        /* per-node selector: wall type / mask / SetT-SetQ choice */
    const double *v0, *v1, *v2;   /* per-node values                              */
    const double *ux, *uy, *uz;   /* macro velocity arrays read by AD/AAD BCs     */
    const double *rho, *tem;      /* forward macros read by AAD iSetRho           */
    const double *diffusivity;    /* per-node kappa (OL_BC_AD_Q)                  */
    double kappa;                 /* constant kappa (OL_BC_AD_QC)                 */
    double eps;                   /* objective weight of adjoint BCs              */
    double uscale;                /* factor on the prescribed velocity of NS SetU / ANS iSetU
                                   * (time-varying inflow u(t) = uscale * u; CPU extension,
                                   * 1 = the reference routine)                    */
} ol_bc;

/* lattice geometry ------------------------------------------------------- */
int  ol_nnodes(const ol_lat *L);

/* D2Q9::Stream / iStream, D3Q15::Stream / iStream (inverse = 1). In place. */
void ol_stream(const ol_lat *L, double *f, int inverse);

/* Apply one edge / face boundary condition. f: population set the BC writes
 * (g for AD/AAD kinds); for OL_BC_AAD_RHO, f = NS adjoint set and g = AD adjoint set. */
void ol_apply_bc(const ol_lat *L, double *f, double *g, const ol_bc *bc);

/* SmoothCorner (full sequence), SmoothCornerAt (2D: dz ignored), 3D line smoothing. */
void ol_smooth_corner(const ol_lat *L, double *f);
void ol_smooth_at(const ol_lat *L, double *f, int i, int j, int k, int dx, int dy, int dz);
void ol_smooth_line(const ol_lat *L, double *f, int plane, int a, int b, int da, int db);  /* plane 0=YZ,1=ZX,2=XY */

/* Collide (macro + forces + BGK). f: NS set, g: AD set (NULL for NS-only kinds). */
void ol_collide(const ol_lat *L, int kind, double *f, double *g, const ol_fields *F,
                const ol_phys *P, int save);

/* Initial conditions: 0 NS, 1 AD, 2 ANS, 3 AAD, 4 NSin (rho, u), 5 ANSin (ip, iu),
 * 6 EL (rho, u, sxx..syy), 7 AEL (irho = ip, imx, imy, isxx..isyy, gamma) */
void ol_init(const ol_lat *L, int which, double *f, const ol_fields *F);

/* Sensitivities.
 *   which 0: AAD::SensitivityTemperatureAtHeatSource (qn[] values, mask[] selector)
 *   which 1: AAD::SensitivityBrinkmanDiffusivity
 *   which 2: AAD::SensitivityHeatExchange (dkds = dbds)
 *   which 3: ANS::SensitivityBrinkman
 *   which 4: AEL::SensitivityCompliance (stress sxx..syy, irho = ip, isxx..isyy; D2Q9)
 * g, ig: snapshots in snap[q*idx+c] layout. */
void ol_sensitivity(const ol_lat *L, int which, double *dfds, const ol_fields *F,
                    const double *dads, const double *dkds, const double *g, const double *ig,
                    const double *qn, const int *mask);

/* Filters. Weight: hat (R - dist)/R between two design cells (mask[] != 0, or mask == NULL),
 * identity (1 on the diagonal, 0 off it) otherwise -- the production drivers' filter weight. */
void ol_heaviside_var(const ol_lat *L, double R, double beta, const double *s, const int *mask, double *out);
void ol_heaviside_sens(const ol_lat *L, double R, double beta, const double *s, const double *dfdrho,
                       const int *mask, double *out);
void ol_density_filter(const ol_lat *L, double R, const double *v, const int *mask, double *out);
/* the same filters with a general weight functor given as a table w[node][tap] (taps: offsets
 * with distance <= R in the (i2, j2, k2) loop order; 2D: k2 = k1). op 0: Heaviside variable of
 * a (beta); 1: Heaviside sensitivity (a = s, b = dfdrho); 2: filtered average of a. */
int ol_filter_ntaps(const ol_lat *L, double R);
void ol_filter_table(const ol_lat *L, int op, double R, double beta, const double *a, const double *b,
                     const double *w, double *out);

/* Residual (residual.h) over ncomp components, Normalize (normalize.h). */
double ol_residual(int n, int ncomp, const double *const *a, const double *const *b);
void   ol_normalize(double *v, int n);

/* Threads used by the OpenMP loops (0 = runtime default). */
void ol_set_threads(int n);

#ifdef __cplusplus
}
#endif
#endif
