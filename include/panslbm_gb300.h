/*
 * panslbm_gb300.h -- C ABI of the GB300 lattice-Boltzmann topology-optimisation library.
 *
 * The reference (PANSLBM2) is a header-only C++ template library with no FFI; its
 * "interface" is the set of template functions the production drivers call. Each entry point
 * below replaces one group of those calls. The C++ template layer in dropin/src (the
 * reference's header paths, namespaces and signatures) is built on these symbols; other host
 * languages bind them directly. All pointers named `host*` are host memory; device memory is
 * owned by the library and never crosses this boundary (pl_residual_device_noalloc excepted).
 *
 * Every call returns PL_OK (0) or a negative error code; pl_last_error() describes the last
 * failure of the calling thread. Calls are asynchronous on the lattice's CUDA stream except
 * where a host buffer is written (get / download calls synchronise).
 */
#ifndef PANSLBM_GB300_H
#define PANSLBM_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define PL_OK 0
#define PL_ERR_ARG (-1)          /* invalid argument (size, kind, pointer)               */
#define PL_ERR_CUDA (-2)         /* CUDA runtime error                                   */
#define PL_ERR_UNSUPPORTED (-3)  /* kind / storage combination not built                 */
#define PL_ERR_STATE (-4)        /* call order violated (e.g. snapshot before a collide) */
#define PL_ERR_ALLOC (-5)        /* device allocation failed                             */
#define PL_ERR_NONFINITE (-6)    /* non-finite value detected by a reduction             */

/* pl_solve status */
#define PL_CONVERGED 1
#define PL_MAX_STEPS 2
#define PL_DIVERGED 3

/* population storage (compute is FP64 for PL_FP64, FP32 otherwise; 16-bit storage holds
 * populations shifted by w_c * shift of their set) */
#define PL_FP64 0
#define PL_FP32 1
#define PL_FP16 2
#define PL_BF16 3

/* collide kinds: one per reference collide routine */
#define PL_NS_COLLIDE 0           /* NS::MacroCollide                         navierstokes.h:430-483   */
#define PL_NS_BRINKMAN 1          /* NS::MacroBrinkmanCollide                 navierstokes.h:485-546   */
#define PL_AD_NATURAL 2           /* AD::MacroBrinkmanCollideNaturalConvection advection.h:928-1044    */
#define PL_AD_FORCE 3             /* AD::MacroBrinkmanCollideForceConvection  advection.h:812-926      */
#define PL_AD_HEATEX 4            /* AD::MacroBrinkmanCollideHeatExchange     advection.h:714-810      */
#define PL_AD_NATURAL_NOBRINK 5   /* AD::MacroCollideNaturalConvection        advection.h:616-712      */
#define PL_AD_FORCE_NOBRINK 6     /* AD::MacroCollideForceConvection          advection.h:528-614      */
#define PL_NSIN_COLLIDE 7         /* NSin::MacroCollide (D2Q9)                nsincompressible.h:144-169 */
#define PL_NSIN_BRINKMAN 8        /* NSin::MacroBrinkmanCollide (D2Q9)        nsincompressible.h:171-200 */
#define PL_ANS_BRINKMAN 10        /* ANS::MacroBrinkmanCollide                adjointnavierstokes.h:396-470 */
#define PL_AAD_NATURAL 11         /* AAD::MacroBrinkmanCollideNaturalConvection adjointadvection.h:1111-1230 */
#define PL_AAD_FORCE 12           /* AAD::MacroBrinkmanCollideForceConvection adjointadvection.h:995-1109 */
#define PL_AAD_HEATEX 13          /* AAD::MacroBrinkmanCollideHeatExchange    adjointadvection.h:892-993 */
#define PL_AAD_MASSFLOW 14        /* AAD::MacroBrinkmanCollideNaturalConvectionMassFlow adjointadvection.h:1232-1355 */
#define PL_ANSIN_BRINKMAN 15      /* ANSin::MacroBrinkmanCollide (D2Q9)       adjointnsincompressible.h:143-178 */
#define PL_EL_COLLIDE 16          /* EL::MacroCollide (D2Q9; rate 1/tau)      elastic.h:109-136        */
#define PL_EL_EXTENDED 17         /* EL::MacroExtendedCollide (D2Q9)          elastic.h:138-166        */
#define PL_AEL_COLLIDE 18         /* AEL::MacroCollide (D2Q9; adjoint)        adjointelastic.h:96-125  */

/* boundary-program op kinds */
#define PL_BC_WALL 0      /* (D2Q9|D3Q15)::BoundaryConditionAlong*   type: 1 BARRIER, 2 MIRROR  */
#define PL_BC_IWALL 1     /* (D2Q9|D3Q15)::iBoundaryConditionAlong*                             */
#define PL_BC_NS_U 2      /* NS::BoundaryConditionSetUAlong*        v0,v1,v2 = ux,uy,uz          */
#define PL_BC_NS_RHO 3    /* NS::BoundaryConditionSetRhoAlong*      v0 = rho, v1/v2 tangential   */
#define PL_BC_AD_T 4      /* AD::BoundaryConditionSetTAlong*        v0 = T                       */
#define PL_BC_AD_Q 5      /* AD::BoundaryConditionSetQAlong*        v0 = qn, per-node kappa      */
#define PL_BC_AD_QC 6     /* AD::BoundaryConditionSetQAlong*        v0 = qn, constant `kappa`    */
#define PL_BC_ANS_U 7     /* ANS::iBoundaryConditionSetUAlong*      v0..v2 = u, `eps`            */
#define PL_BC_ANS_RHO 8   /* ANS::iBoundaryConditionSetRhoAlong*                                 */
#define PL_BC_AAD_T 9     /* AAD::iBoundaryConditionSetTAlong*                                   */
#define PL_BC_AAD_Q 10    /* AAD::iBoundaryConditionSetQAlong*      `eps`                        */
#define PL_BC_AAD_RHO 11  /* AAD::iBoundaryConditionSetRhoAlong*    type: 1 SetT, 2 SetQ; `eps`  */
#define PL_BC_NSIN_U 12   /* NSin::BoundaryConditionSetUAlong{X,Y}Edge   v0,v1 = ux,uy (D2Q9)    */
#define PL_BC_NSIN_RHO 13 /* NSin::BoundaryConditionSetRhoAlong{X,Y}Edge v0 = rho, v1 = us      */
#define PL_BC_ANSIN_U 14  /* ANSin::iBoundaryConditionSetUAlong{X,Y}Edge `eps`; ANSin's iSetRho
                           * is ANS's (PL_BC_ANS_RHO)                                            */
#define PL_BC_EL_STRESS 15  /* EL::BoundaryConditionSetStressAlong{X,Y}Edge   v0,v1 = tx,ty (D2Q9) */
#define PL_BC_AEL_STRESS 16 /* AEL::iBoundaryConditionSetStressAlong{X,Y}Edge v0,v1 = tx,ty,
                             * v2 = the rho argument (D2Q9)                                       */
#define PL_SMOOTH_CORNER 20  /* SmoothCorner()                                                   */
#define PL_SMOOTH_AT 21      /* SmoothCornerAt(i,j[,k],di,dj[,dk])                               */
#define PL_SMOOTH_LINE 22    /* SmoothCornerAlong{YZ,ZX,XY}: axis = 0,1,2; (i,j) = line, (di,dj)  */

/* node fields exchanged with the host (double arrays of nx*ny*nz, idx = i + nx*(j + ny*k)) */
#define PL_ALPHA 0   /* Brinkman resistance                         */
#define PL_KAPPA 1   /* per-node diffusivity                        */
#define PL_BETA 2    /* heat-exchange coefficient                   */
#define PL_DIRX 3    /* mass-flow objective weights                 */
#define PL_DIRY 4
#define PL_DIRZ 5
#define PL_DENSITY 6 /* EL density rho (the input array of the EL collides) */
#define PL_GAMMA 7   /* EL / AEL stress scale gamma                 */
#define PL_RHO 8     /* forward macros stored by the last saving collide */
#define PL_UX 9
#define PL_UY 10
#define PL_UZ 11
#define PL_TEM 12
#define PL_QX 13
#define PL_QY 14
#define PL_QZ 15
#define PL_IP 16     /* adjoint macros stored by the last saving adjoint collide */
#define PL_IUX 17
#define PL_IUY 18
#define PL_IUZ 19
#define PL_IMX 20
#define PL_IMY 21
#define PL_IMZ 22
#define PL_ITEM 23
#define PL_IQX 24
#define PL_IQY 25
#define PL_IQZ 26
/* the elastic kinds store their macros in the planes above: EL ux, uy in PL_UX, PL_UY and the
 * stress in the T / q planes; AEL irho in PL_IP, imx, imy in PL_IMX, PL_IMY and the adjoint
 * stress in the adjoint T / q planes */
#define PL_SXX PL_TEM
#define PL_SXY PL_QX
#define PL_SYX PL_QY
#define PL_SYY PL_QZ
#define PL_IRHO PL_IP
#define PL_ISXX PL_ITEM
#define PL_ISXY PL_IQX
#define PL_ISYX PL_IQY
#define PL_ISYY PL_IQZ
#define PL_FWD_RHO 32   /* forward solution read by adjoint collides and adjoint BCs */
#define PL_FWD_UX 33
#define PL_FWD_UY 34
#define PL_FWD_UZ 35
#define PL_FWD_TEM 36
#define PL_DFDS 37      /* device sensitivity accumulator of pl_sensitivity_device          */
#define PL_DADS 38      /* its inputs dalpha/ds, dkappa/ds and the heat-source flux qn       */
#define PL_DKDS 39
#define PL_QN 40
#define PL_ACC 41       /* a free accumulator for pl_accumulate                              */
/* forced-convection heat-sink extension (no counterpart in the reference, whose heat sinks take
 * their heat through a boundary flux): while set, PL_AD_FORCE collides add the volumetric heat
 * source Q(x) as w_c * Q to g before their final AD macro, and PL_AAD_FORCE collides add the
 * objective weight w(x) = dJ/dT(x) of a volumetric objective J = sum w T to every adjoint g
 * population before a final AAD macro. pl_set_field(h, field, NULL) switches the term off. */
#define PL_HEAT_SOURCE 42
#define PL_OBJ_WEIGHT 43

typedef struct pl_lattice_s *pl_lattice;

typedef struct {
    double nu;            /* viscosity (BGK rate 1/(3 nu + 1/2))                */
    double diff;          /* constant diffusivity of the siblings that take one  */
    double gx, gy, gz;    /* buoyancy vector                                    */
    double tem0;          /* reference temperature                              */
    double tau;           /* relaxation time of the EL / AEL kinds (rate 1/tau)  */
} pl_phys;

/* One boundary routine call, recorded in call order into a boundary program. Per-node
 * selectors/values are full-lattice host arrays (the reference's functor of global (i,j,k)
 * evaluated at every node); NULL selects 1 (walls: BARRIER) and NULL values use c0..c2. */
typedef struct {
    int kind;                 /* PL_BC_* or PL_SMOOTH_*                                  */
    int lat;                  /* walls / smoothing: 0 NS set (pf), 1 AD set (pg)          */
    int axis, pos, dir;       /* edge/face: axis 0/1/2, global position, side -1/+1      */
    const int *type;
    const double *v0, *v1, *v2;
    double c0, c1, c2;
    double eps, kappa;
    int i, j, k, di, dj, dk;  /* smoothing arguments                                     */
} pl_bc_desc;

/* lattice pair (NS set + AD set) ---------------------------------------------------------
 * replaces D2Q9<T>(lx, ly) / D3Q15<T>(lx, ly, lz) construction (d2q9.h:28-58,
 * d3q15.h:28-86) for one particle pair pf/pg sharing a geometry. */
int pl_create(int q, int nx, int ny, int nz, int storage, pl_lattice *out);
int pl_destroy(pl_lattice h);
const char *pl_last_error(void);
int pl_synchronize(pl_lattice h);
/* launch on a caller-owned CUDA stream (a cudaStream_t passed as void*; NULL = legacy default
 * stream) instead of the lattice's own non-blocking stream */
int pl_set_stream(pl_lattice h, void *stream);
/* launch options (no counterpart in the reference, which has no launch policy):
 *  PL_OPT_GRAPHS         1: pl_steps, and pl_solve between its residual checks, replay a
 *                        captured two-step CUDA graph; 0 (default):
 *                        eager launches, which keep the boundary streams' priority
 *  PL_OPT_SIDE_PRIORITY  1 (default): the boundary chains run on high-priority streams; 0:
 *                        lowest priority */
#define PL_OPT_GRAPHS 1
#define PL_OPT_SIDE_PRIORITY 2
/*  PL_OPT_STOCHASTIC_ROUNDING  16-bit storage only. 0 (default): the collide stores round to
 *                        nearest; 1: they round stochastically (unbiased), so increments below half
 *                        a 16-bit ulp -- a small source added every step -- still accumulate in
 *                        expectation. Replayed graphs reuse their captured seeds. */
#define PL_OPT_STOCHASTIC_ROUNDING 3
/*  PL_OPT_SNAPSHOT_IN_STEP  1: every saving collide / step of a kind with a snapshot writes its
 *                        snapshot slot in the same pass, so the pl_snapshot call that follows
 *                        runs no kernel (for sweeps that take a snapshot at every step);
 *                        0 (default): pl_snapshot re-evaluates the last collide's input state. */
#define PL_OPT_SNAPSHOT_IN_STEP 4
int pl_set_option(pl_lattice h, int option, int value);
/* time-varying inflow (no counterpart in the reference, whose inflows are constant): the
 * prescribed velocity of every NS SetU / ANS iSetU op is multiplied by `scale` in the steps that
 * follow (default 1; a transient driver sets u(t)/u_max before each step) */
int pl_set_inflow_scale(pl_lattice h, double scale);
/* shift of 16-bit population storage, per set (default: f 1.0, g 0.0) */
int pl_set_shift(pl_lattice h, double shift_f, double shift_g);

/* populations: host buffer of q*N doubles, direction-major (p[c*N + idx]); set 0 = pf, 1 = pg */
int pl_set_populations(pl_lattice h, int set, const double *host);
int pl_get_populations(pl_lattice h, int set, double *host);

/* node fields */
int pl_set_field(pl_lattice h, int field, const double *host);
int pl_get_field(pl_lattice h, int field, double *host);
/* a macroscopic field (PL_RHO..PL_QZ, PL_IP..PL_IQZ) of the last (age 0) or the previous (age 1)
 * saving collide of its family; the device keeps both (the residual compares them), so a caller
 * that mirrors host arrays can leave outputs on the device until it needs them (no counterpart in
 * the reference, whose routines write host arrays directly) */
int pl_get_saved_field(pl_lattice h, int field, int age, double *host);
/* copy the forward macros of the last saving collide into PL_FWD_* */
int pl_freeze_forward(pl_lattice h);

/* boundary programs: the edge/face routines and smoothing of one time step, in call order
 * (replaces the per-step BoundaryCondition* / SetT / SetQ / iSet* / SmoothCorner* calls) */
int pl_program_create(pl_lattice h, const pl_bc_desc *descs, int n, int *prog);
int pl_program_destroy(pl_lattice h, int prog);

/* initial conditions: which 0 NS::InitialCondition(rho,u), 1 AD::(T,u), 2 ANS::(u; ip,iu),
 * 3 AAD::(u; iT,iq), 4 NSin::(rho,u), 5 ANSin::(ip,iu) (D2Q9; ux, uy may be NULL).
 * a0..a3 = the scalar/vector inputs, ux..uz = the velocity argument. For the adjoint seeds (2, 3)
 * ux = uy = uz = NULL takes the frozen forward velocity already on the device (pl_freeze_forward)
 * and a0 = NULL a zero adjoint state, so an adjoint solve starts without host traffic. */
int pl_init(pl_lattice h, int which, const double *a0, const double *a1, const double *a2, const double *a3,
            const double *ux, const double *uy, const double *uz);

/* elastic initial conditions (D2Q9): which 0 EL::InitialCondition (elastic.h:168-179), in = rho,
 * ux, uy, sxx, sxy, syx, syy; 1 AEL::InitialCondition (adjointelastic.h:127-138), in = irho,
 * imx, imy, isxx, isxy, isyx, isyy with gamma taken from PL_GAMMA. Seven host arrays of N. */
int pl_init_elastic(pl_lattice h, int which, const double *const *in);

/* one collide in place (the reference's Macro*Collide* call) */
int pl_collide(pl_lattice h, int kind, const pl_phys *ph, int save);
/* one fused step: Stream/iStream + program `prog` (-1: none) + collide of kind */
int pl_step(pl_lattice h, int kind, const pl_phys *ph, int prog, int save);
/* n fused steps without saving (device-resident inner loop) */
int pl_steps(pl_lattice h, int kind, const pl_phys *ph, int prog, int n);
/* Stream + program without a collide. mode 0: Stream, 1: iStream (adjoint inputs),
 * 2: program only (forward inputs), 3: program only (adjoint inputs); both_sets 0: pf only */
int pl_stream(pl_lattice h, int mode, int prog, int both_sets);

/* The reference driver loop (production/heatsink.cpp:142-174 forward, 183-212 adjoint):
 * collide, then up to max_steps-1 fused steps, checking every `check_every` steps the
 * residual (residual.h) of velocity and flux (forward) or adjoint velocity and flux
 * (adjoint) against `tol`. Returns PL_OK and sets *status / *steps / res[0..1]. */
int pl_solve(pl_lattice h, int kind, const pl_phys *ph, int prog, int max_steps, int check_every, double tol,
             int *status, int *steps, double *res);

/* snapshot of the g populations the last collide stored (gi / igi of the reference):
 * slot 0 forward, 1 adjoint; host may be NULL (kept on the device for pl_sensitivity).
 * host layout: snap[q*idx + c] (the reference's scalar layout). */
int pl_snapshot(pl_lattice h, int slot, double *host);
/* load a snapshot slot from a host array in the same layout (a gi / igi the caller kept, e.g.
 * one per time step of a transient sweep) for the next pl_sensitivity */
int pl_set_snapshot(pl_lattice h, int slot, const double *host);

/* Residual(...) of residual.h over the current (a) and previous (b) saved macros:
 * family 0 = (ux,uy[,uz]), 1 = (qx,qy[,qz]), 2 = (iux,iuy[,iuz]), 3 = (iqx,iqy[,iqz]). */
int pl_residual(pl_lattice h, int family, double *out);
/* Residual of arbitrary host arrays (ncomp of a, ncomp of b, n each) */
int pl_residual_host(pl_lattice h, int n, int ncomp, const double *const *a, const double *const *b, double *out);
/* Residual of caller-owned DEVICE arrays (a[m], b[m]: n doubles each, m < ncomp <= 3) on
 * `stream` (a cudaStream_t as void*, NULL = legacy default stream); *out = sqrt(sum (a-b)^2 /
 * sum a^2), the same value pl_residual_host gives. No counterpart in the reference (its
 * Residual runs on host arrays). Allocates nothing: its scratch is a fixed 16 KB device array
 * in the library, shared by all calls on a device. The first call on each device looks that
 * array up (make it before any stream capture on the device); calls from several host threads
 * that can overlap on the GPU race on it and must be serialised. The arrays must live on the
 * current device (or be managed memory), else PL_ERR_ARG. Returns after the result has been
 * copied to *out; PL_ERR_NONFINITE (with *out set) when an input value is not finite. */
int pl_residual_device_noalloc(long long n, int ncomp, const double *const *a, const double *const *b, void *stream,
                               double *out);

/* sensitivities (dfds host array of N, accumulated into like the reference):
 * which 0 AAD::SensitivityTemperatureAtHeatSource (adjointadvection.h:1495-1543, qn/mask per node)
 *       1 AAD::SensitivityBrinkmanDiffusivity     (adjointadvection.h:1459-1493)
 *       2 AAD::SensitivityHeatExchange            (adjointadvection.h:1443-1457, dkds = dbds)
 *       3 ANS::SensitivityBrinkman                (adjointnavierstokes.h:540-554)
 * reads PL_FWD_* (forward), the adjoint macros, PL_KAPPA and the two snapshots. */
int pl_sensitivity(pl_lattice h, int which, double *dfds, const double *dads, const double *dkds, const double *qn,
                   const int *mask);

/* Checkpointed sweeps (no counterpart in the reference, whose transient drivers keep every time
 * step's fields in host memory, production/heatsink_transient.cpp:45-52): device-resident stores,
 * numbered slots allocated on first use and kept until pl_store_release / pl_destroy.
 *   PL_STORE_POPS  both population sets of the current buffer (a checkpoint);
 *   PL_STORE_FWD   rho, ux, uy, uz, T saved by the last saving forward collide; pl_load puts them
 *                  in PL_FWD_* (the adjoint collides' and adjoint routines' forward inputs);
 *   PL_STORE_SNAP  the forward g snapshot (pl_snapshot slot 0); pl_load puts it back in slot 0.
 * Slots are numbered 0 .. 65535 per kind. */
#define PL_STORE_POPS 0
#define PL_STORE_FWD 1
#define PL_STORE_SNAP 2
int pl_store(pl_lattice h, int what, int slot);
int pl_load(pl_lattice h, int what, int slot);
int pl_store_release(pl_lattice h);
/* exchange the forward snapshot (slot 0) with PL_STORE_SNAP slot `slot`, without a copy: a sweep
 * that takes each step's snapshot once and reads it back once moves it in and out this way */
int pl_store_swap_snapshot(pl_lattice h, int slot);
/* pl_sensitivity on the device: accumulates into the device field PL_DFDS (reset it with
 * pl_set_field, read it with pl_get_field), so a transient sweep adds one term per time step
 * (production/heatsink_transient.cpp:191-194) without host traffic. dads, dkds, qn and mask are
 * uploaded when non-NULL and reused by later calls when NULL. */
int pl_sensitivity_device(pl_lattice h, int which, const double *dads, const double *dkds, const double *qn,
                          const int *mask);
/* dst += a * src over the lattice: dst a device accumulator (PL_DFDS..PL_ACC), src any field
 * pl_get_field reads (e.g. PL_TEM of the last saving collide, for a time-integrated objective) */
int pl_accumulate(pl_lattice h, int dst, int src, double a);

/* AEL::SensitivityCompliance (adjointelastic.h:149-155), D2Q9: dfds (host, N) is accumulated
 * into; in = nine host arrays sxx, sxy, syx, syy, irho, isxx, isxy, isyx, isyy, or NULL for the
 * stress of the last saving EL collide and the adjoint of the last saving AEL collide. */
int pl_sensitivity_compliance(pl_lattice h, double *dfds, const double *const *in);

/* filters (heavisidefilter.h:404-899, densityfilter.h:10-515). mask: NULL = hat weight
 * everywhere; else hat weight between two design cells (mask != 0), identity otherwise. */
int pl_heaviside_var(pl_lattice h, double R, double beta, const double *s, const int *mask, double *out);
int pl_heaviside_sens(pl_lattice h, double R, double beta, const double *s, const double *dfdrho, const int *mask,
                      double *out);
int pl_density_filter(pl_lattice h, double R, const double *v, const int *mask, double *out);
/* the filters with a general weight functor (the `_weight(i1, j1, k1, i2, j2, k2)` argument of
 * HeavisideFilter::GetFilteredVariable / GetFilteredSensitivity, heavisidefilter.h:404-899, and
 * DensityFilter::GetFilteredValue, densityfilter.h:10-515). pl_filter_taps lists the taps of
 * radius R (offsets with distance <= R) in the reference's (i2, j2, k2) loop order: *ntap, and
 * di/dj/dk when non-NULL (room for (2 floor(R) + 1)^d entries). weights[node * ntap + t] is the
 * functor's value for node and node + tap t (taps outside the lattice are skipped, as there).
 * op 0: Heaviside projection of the filtered s (a = s, beta); 1: Heaviside sensitivity (a = s,
 * b = dfdrho); 2: filtered average of a (DensityFilter). */
int pl_filter_taps(pl_lattice h, double R, int *ntap, int *di, int *dj, int *dk);
int pl_filter_weighted(pl_lattice h, int op, double R, double beta, const double *a, const double *b,
                       const double *weights, double *out);
/* Normalize (normalize.h:8-23), in place on a host array of n */
int pl_normalize(pl_lattice h, double *v, int n);

/* MMA design-variable update on the device (Svanberg's method of moving asymptotes), FP64:
 * replaces MMA<T>(n, m, a0, a, c, d, xmin, xmax) (utility/mma.h:62-86) and
 * MMA<T>::UpdateVariables (utility/mma.h:196-548) for 1 <= m <= 4 constraints. Host arrays:
 * a, c, d of m; xmin, xmax, xk, dfdx of n; g of m; dgdx of m rows of n. xk is updated in place.
 * pl_mma_set_param: which 0 move, 1 asyinit, 2 asydecr, 3 asyincr, 4 albefa, 5 raa0, 6 epsvalue
 * (the public members of MMA<T>, mma.h:97-105; defaults 0.5, 0.5, 0.7, 1.2, 0.1, 1e-5, 1e-6). */
typedef struct pl_mma_s *pl_mma;
int pl_mma_create(int n, int m, double a0, const double *a, const double *c, const double *d, const double *xmin,
                  const double *xmax, pl_mma *out);
int pl_mma_set_param(pl_mma h, int which, double value);
int pl_mma_update(pl_mma h, double *xk, double f, const double *dfdx, const double *g, const double *dgdx);
int pl_mma_destroy(pl_mma h);
/* the optimizer's history, for ImportSetting / ExportSetting (mma.h:142-194): outer counter k,
 * previous objective, x of the two previous updates, asymptotes L and U (host arrays of n) */
int pl_mma_get_state(pl_mma h, int *k, double *previous, double *xkm2, double *xkm1, double *L, double *U);
int pl_mma_set_state(pl_mma h, int k, double previous, const double *xkm2, const double *xkm1, const double *L,
                     const double *U);

/* host-side fault injection (no counterpart in the reference, which has no error paths): after
 * `after` further successful device allocations by the library, the next one fails and returns
 * PL_ERR_ALLOC as an out-of-memory device would; -1 switches it off. For tests of callers'
 * error handling; nothing on the device faults. */
int pl_debug_fail_alloc(long long after);

/* Learned warm start (no counterpart in the reference): a 3D convolutional U-Net over an
 * nx x ny x nz volume in the lattice's node order, trained and evaluated on the GPU's tensor
 * cores (tcgen05 implicit-GEMM convolutions, BF16 weights and activations, FP32 accumulation,
 * Adam on FP32 master weights). `levels` resolution levels with base_channels * 2^l channels
 * (each volume extent divisible by 2^(levels-1)); 16 input channels (channel 0 = the design,
 * channels 1.. = static features) and 16 output channels (the first `targets` are trained).
 * Parameters are flattened per layer as weights [cout][taps][cin] then biases [cout], layers
 * in the order encoder (level 0..L-1: conv1, conv2), decoder (level L-2..0: conv1, conv2),
 * head (1x1x1). */
typedef struct pl_unet_s *pl_unet;
int pl_unet_create(int nx, int ny, int nz, int levels, int base_channels, int in_channels, int out_channels,
                   int max_batch, pl_unet *out);
int pl_unet_destroy(pl_unet u);
long long pl_unet_param_count(pl_unet u);
int pl_unet_init_params(pl_unet u, unsigned long long seed);
int pl_unet_get_params(pl_unet u, float *host);
int pl_unet_set_params(pl_unet u, const float *host);
/* one forward pass on host inputs x [batch][voxel][16] (FP32, rounded to BF16) -> y [batch][voxel][16] */
int pl_unet_forward(pl_unet u, int batch, const float *x_host, float *y_host);
/* the backward pass of the last forward for dL/dy = dy [batch][voxel][16]; the parameter
 * gradients are read with pl_unet_gradients (same layout as the parameters) */
int pl_unet_backward(pl_unet u, int batch, const float *dy_host);
int pl_unet_gradients(pl_unet u, float *host);
/* training set on the device: `nsamples` (design, targets) pairs; static features [voxel][nfeat]
 * (nfeat <= 15) shared by all samples; pl_unet_add_sample stores one design (nvox doubles) and
 * its targets [targets][nvox] */
int pl_unet_dataset_reserve(pl_unet u, int nsamples, int targets);
int pl_unet_set_static(pl_unet u, const float *feat, int nfeat);
int pl_unet_add_sample(pl_unet u, int slot, const double *design, const double *targets);
/* the same from a lattice's device fields, without host traffic: targets = the frozen forward
 * solution (rho - 1, ux, uy, uz, T) and the last saved adjoint macros (ip, iux, iuy, iuz, iT,
 * iqx, iqy, iqz) of lattice h (same node count) */
int pl_unet_add_sample_lattice(pl_unet u, int slot, const double *design, pl_lattice h);
/* train on samples 0..nsamples-1 (targets normalised per channel over them) for `epochs`
 * shuffled passes of mini-batches, Adam with a cosine-decaying learning rate (lr down to lr/20);
 * loss_per_epoch (may be NULL) receives the mean squared error of the normalised targets per
 * epoch */
int pl_unet_train(pl_unet u, int nsamples, int epochs, int batch, double lr, unsigned long long seed,
                  double *loss_per_epoch);
/* the target normalisation (mean, std per target channel), e.g. to restore a trained model */
int pl_unet_set_norm(pl_unet u, const float *mean, const float *stdv);
int pl_unet_get_norm(pl_unet u, float *mean, float *stdv);
/* prediction for one design: out [targets][nvox] (de-normalised, FP64) */
int pl_unet_predict(pl_unet u, const double *design, double *out);

/* FP64 fused multiply-add throughput of the current device in TFLOP/s (2 flops per FMA), from a
 * short kernel of independent FMA chains: the roofline denominator of the FP64 collide kinds (no
 * counterpart in the reference) */
int pl_probe_fp64_fma(double *tflops);

/* last step kernel time (ms) measured with CUDA events on the lattice stream, and number
 * of kernels launched since creation */
int pl_stats(pl_lattice h, double *last_step_ms, long long *launches);

#ifdef __cplusplus
}
#endif
#endif
