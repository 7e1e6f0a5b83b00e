// ref_harness.cpp -- binds the oracle API (oracle.h) to the PANSLBM2 reference's own header
// templates, so the C restatement in oracle.c can be checked call-for-call against the
// reference itself (TEST INFRASTRUCTURE ONLY).
//
// Compiled twice (REF_DIM=2 with src/particle/d2q9.h, REF_DIM=3 with src/particle/d3q15.h:
// the two headers define the same BARRIER/MIRROR constants and cannot share a translation
// unit) from the reference sources where they lie; see oracle/build.py. Populations are
// copied between the oracle's SoA layout and the reference particle object's AoS layout.
#include <cmath>
#include <cstring>
#include <vector>
#if REF_DIM == 2
#include "src/particle/d2q9.h"
#define PCLASS D2Q9
#define NAME(x) ref2_##x
#else
#include "src/particle/d3q15.h"
#define PCLASS D3Q15
#define NAME(x) ref3_##x
#endif
#include "src/equation/navierstokes.h"
#include "src/equation/advection.h"
#include "src/equation/adjointnavierstokes.h"
#include "src/equation/adjointadvection.h"
#if REF_DIM == 2
#include "src/equation/nsincompressible.h"
#include "src/equation/adjointnsincompressible.h"
#include "src/equation/elastic.h"
#include "src/equation/adjointelastic.h"
#endif
#include "src/utility/heavisidefilter.h"
#include "src/utility/densityfilter.h"
#include "src/utility/residual.h"
#include "src/utility/normalize.h"
#include "oracle.h"

using namespace PANSLBM2;
typedef PCLASS<double> Lat;

static Lat *make(const ol_lat *L) {
#if REF_DIM == 2
    return new Lat(L->nx, L->ny);
#else
    return new Lat(L->nx, L->ny, L->nz);
#endif
}
static void load(Lat &p, const double *f) {
    const int n = p.nxyz;
    for (int idx = 0; idx < n; ++idx) {
        p.f0[idx] = f[idx];
        for (int c = 1; c < Lat::nc; ++c) p.f[Lat::IndexF(idx, c)] = f[(size_t)c * n + idx];
    }
}
static void store(const Lat &p, double *f) {
    const int n = p.nxyz;
    for (int idx = 0; idx < n; ++idx) {
        f[idx] = p.f0[idx];
        for (int c = 1; c < Lat::nc; ++c) f[(size_t)c * n + idx] = p.f[Lat::IndexF(idx, c)];
    }
}

#if REF_DIM == 2
#define NID(i, j, k) ((i) + L->nx * (j))
#define FI(expr) [&](int i, int j) { return (int)(expr); }
#define FD(expr) [&](int i, int j) { return (double)(expr); }
#else
#define NID(i, j, k) ((i) + L->nx * ((j) + L->ny * (k)))
#define FI(expr) [&](int i, int j, int k) { return (int)(expr); }
#define FD(expr) [&](int i, int j, int k) { return (double)(expr); }
#endif

extern "C" void NAME(stream)(const ol_lat *L, double *f, int inverse) {
    Lat *p = make(L);
    load(*p, f);
    if (inverse) p->iStream(); else p->Stream();
    store(*p, f);
    delete p;
}

extern "C" void NAME(apply_bc)(const ol_lat *L, double *f, double *g, const ol_bc *bc) {
    Lat *p = make(L), *q = make(L);
    load(*p, f);
    if (g) load(*q, g);
    const int *ty = bc->type;
    const double *v0 = bc->v0, *v1 = bc->v1, *v2 = bc->v2;
    int a = bc->axis, pos = bc->pos, d = bc->dir;
    (void)v2;
#if REF_DIM == 2
    auto T = FI(ty[NID(i, j, 0)]);
    auto V0 = FD(v0[NID(i, j, 0)]);
    auto V1 = FD(v1[NID(i, j, 0)]);
    switch (bc->kind) {
    case OL_BC_WALL: if (a == 0) p->BoundaryConditionAlongXEdge(pos, d, T); else p->BoundaryConditionAlongYEdge(pos, d, T); break;
    case OL_BC_IWALL: if (a == 0) p->iBoundaryConditionAlongXEdge(pos, d, T); else p->iBoundaryConditionAlongYEdge(pos, d, T); break;
    case OL_BC_NS_U: if (a == 0) NS::BoundaryConditionSetUAlongXEdge(*p, pos, d, V0, V1, T); else NS::BoundaryConditionSetUAlongYEdge(*p, pos, d, V0, V1, T); break;
    case OL_BC_NS_RHO: if (a == 0) NS::BoundaryConditionSetRhoAlongXEdge(*p, pos, d, V0, V1, T); else NS::BoundaryConditionSetRhoAlongYEdge(*p, pos, d, V0, V1, T); break;
    case OL_BC_AD_T: if (a == 0) AD::BoundaryConditionSetTAlongXEdge(*p, pos, d, V0, bc->ux, bc->uy, T); else AD::BoundaryConditionSetTAlongYEdge(*p, pos, d, V0, bc->ux, bc->uy, T); break;
    case OL_BC_AD_Q: if (a == 0) AD::BoundaryConditionSetQAlongXEdge(*p, pos, d, V0, bc->ux, bc->uy, bc->diffusivity, T); else AD::BoundaryConditionSetQAlongYEdge(*p, pos, d, V0, bc->ux, bc->uy, bc->diffusivity, T); break;
    case OL_BC_AD_QC: if (a == 0) AD::BoundaryConditionSetQAlongXEdge(*p, pos, d, V0, bc->ux, bc->uy, bc->kappa, T); else AD::BoundaryConditionSetQAlongYEdge(*p, pos, d, V0, bc->ux, bc->uy, bc->kappa, T); break;
    case OL_BC_ANS_U: if (a == 0) ANS::iBoundaryConditionSetUAlongXEdge(*p, pos, d, V0, V1, T, bc->eps); else ANS::iBoundaryConditionSetUAlongYEdge(*p, pos, d, V0, V1, T, bc->eps); break;
    case OL_BC_ANS_RHO: if (a == 0) ANS::iBoundaryConditionSetRhoAlongXEdge(*p, pos, d, T); else ANS::iBoundaryConditionSetRhoAlongYEdge(*p, pos, d, T); break;
    case OL_BC_AAD_T: if (a == 0) AAD::iBoundaryConditionSetTAlongXEdge(*p, pos, d, bc->ux, bc->uy, T); else AAD::iBoundaryConditionSetTAlongYEdge(*p, pos, d, bc->ux, bc->uy, T); break;
    case OL_BC_AAD_Q: if (a == 0) AAD::iBoundaryConditionSetQAlongXEdge(*p, pos, d, bc->ux, bc->uy, T, bc->eps); else AAD::iBoundaryConditionSetQAlongYEdge(*p, pos, d, bc->ux, bc->uy, T, bc->eps); break;
    case OL_BC_AAD_RHO: if (a == 0) AAD::iBoundaryConditionSetRhoAlongXEdge(*p, *q, pos, d, bc->rho, bc->ux, bc->uy, bc->tem, T, bc->eps); else AAD::iBoundaryConditionSetRhoAlongYEdge(*p, *q, pos, d, bc->rho, bc->ux, bc->uy, bc->tem, T, bc->eps); break;
    case OL_BC_NSIN_U: if (a == 0) NSin::BoundaryConditionSetUAlongXEdge(*p, pos, d, V0, V1, T); else NSin::BoundaryConditionSetUAlongYEdge(*p, pos, d, V0, V1, T); break;
    case OL_BC_NSIN_RHO: if (a == 0) NSin::BoundaryConditionSetRhoAlongXEdge(*p, pos, d, V0, V1, T); else NSin::BoundaryConditionSetRhoAlongYEdge(*p, pos, d, V0, V1, T); break;
    case OL_BC_ANSIN_U: if (a == 0) ANSin::iBoundaryConditionSetUAlongXEdge(*p, pos, d, T, bc->eps); else ANSin::iBoundaryConditionSetUAlongYEdge(*p, pos, d, T, bc->eps); break;
    case OL_BC_EL_STRESS: if (a == 0) EL::BoundaryConditionSetStressAlongXEdge(*p, pos, d, V0, V1, T); else EL::BoundaryConditionSetStressAlongYEdge(*p, pos, d, V0, V1, T); break;
    case OL_BC_AEL_STRESS: if (a == 0) AEL::iBoundaryConditionSetStressAlongXEdge(*p, pos, d, V0, V1, bc->rho, T); else AEL::iBoundaryConditionSetStressAlongYEdge(*p, pos, d, V0, V1, bc->rho, T); break;
    }
#else
    auto T = FI(ty[NID(i, j, k)]);
    auto V0 = FD(v0[NID(i, j, k)]);
    auto V1 = FD(v1[NID(i, j, k)]);
    auto V2 = FD(v2[NID(i, j, k)]);
#define FACE3(stmtx, stmty, stmtz) do { if (a == 0) { stmtx; } else if (a == 1) { stmty; } else { stmtz; } } while (0)
    switch (bc->kind) {
    case OL_BC_WALL: FACE3(p->BoundaryConditionAlongXFace(pos, d, T), p->BoundaryConditionAlongYFace(pos, d, T), p->BoundaryConditionAlongZFace(pos, d, T)); break;
    case OL_BC_IWALL: FACE3(p->iBoundaryConditionAlongXFace(pos, d, T), p->iBoundaryConditionAlongYFace(pos, d, T), p->iBoundaryConditionAlongZFace(pos, d, T)); break;
    case OL_BC_NS_U: FACE3(NS::BoundaryConditionSetUAlongXFace(*p, pos, d, V0, V1, V2, T), NS::BoundaryConditionSetUAlongYFace(*p, pos, d, V0, V1, V2, T), NS::BoundaryConditionSetUAlongZFace(*p, pos, d, V0, V1, V2, T)); break;
    case OL_BC_NS_RHO: FACE3(NS::BoundaryConditionSetRhoAlongXFace(*p, pos, d, V0, V1, V2, T), NS::BoundaryConditionSetRhoAlongYFace(*p, pos, d, V0, V1, V2, T), NS::BoundaryConditionSetRhoAlongZFace(*p, pos, d, V0, V1, V2, T)); break;
    case OL_BC_AD_T: FACE3(AD::BoundaryConditionSetTAlongXFace(*p, pos, d, V0, bc->ux, bc->uy, bc->uz, T), AD::BoundaryConditionSetTAlongYFace(*p, pos, d, V0, bc->ux, bc->uy, bc->uz, T), AD::BoundaryConditionSetTAlongZFace(*p, pos, d, V0, bc->ux, bc->uy, bc->uz, T)); break;
    case OL_BC_AD_Q: FACE3(AD::BoundaryConditionSetQAlongXFace(*p, pos, d, V0, bc->ux, bc->uy, bc->uz, bc->diffusivity, T), AD::BoundaryConditionSetQAlongYFace(*p, pos, d, V0, bc->ux, bc->uy, bc->uz, bc->diffusivity, T), AD::BoundaryConditionSetQAlongZFace(*p, pos, d, V0, bc->ux, bc->uy, bc->uz, bc->diffusivity, T)); break;
    case OL_BC_AD_QC: FACE3(AD::BoundaryConditionSetQAlongXFace(*p, pos, d, V0, bc->ux, bc->uy, bc->uz, bc->kappa, T), AD::BoundaryConditionSetQAlongYFace(*p, pos, d, V0, bc->ux, bc->uy, bc->uz, bc->kappa, T), AD::BoundaryConditionSetQAlongZFace(*p, pos, d, V0, bc->ux, bc->uy, bc->uz, bc->kappa, T)); break;
    case OL_BC_ANS_U: FACE3(ANS::iBoundaryConditionSetUAlongXFace(*p, pos, d, V0, V1, V2, T, bc->eps), ANS::iBoundaryConditionSetUAlongYFace(*p, pos, d, V0, V1, V2, T, bc->eps), ANS::iBoundaryConditionSetUAlongZFace(*p, pos, d, V0, V1, V2, T, bc->eps)); break;
    case OL_BC_ANS_RHO: FACE3(ANS::iBoundaryConditionSetRhoAlongXFace(*p, pos, d, T), ANS::iBoundaryConditionSetRhoAlongYFace(*p, pos, d, T), ANS::iBoundaryConditionSetRhoAlongZFace(*p, pos, d, T)); break;
    case OL_BC_AAD_T: FACE3(AAD::iBoundaryConditionSetTAlongXFace(*p, pos, d, bc->ux, bc->uy, bc->uz, T), AAD::iBoundaryConditionSetTAlongYFace(*p, pos, d, bc->ux, bc->uy, bc->uz, T), AAD::iBoundaryConditionSetTAlongZFace(*p, pos, d, bc->ux, bc->uy, bc->uz, T)); break;
    case OL_BC_AAD_Q: FACE3(AAD::iBoundaryConditionSetQAlongXFace(*p, pos, d, bc->ux, bc->uy, bc->uz, T, bc->eps), AAD::iBoundaryConditionSetQAlongYFace(*p, pos, d, bc->ux, bc->uy, bc->uz, T, bc->eps), AAD::iBoundaryConditionSetQAlongZFace(*p, pos, d, bc->ux, bc->uy, bc->uz, T, bc->eps)); break;
    case OL_BC_AAD_RHO: break;   /* the D3Q15 overloads do not compile when instantiated (adjointadvection.h:583) */
    }
#endif
    store(*p, f);
    if (g) store(*q, g);
    delete p;
    delete q;
}

extern "C" void NAME(smooth_corner)(const ol_lat *L, double *f) {
    Lat *p = make(L); load(*p, f); p->SmoothCorner(); store(*p, f); delete p;
}
extern "C" void NAME(smooth_at)(const ol_lat *L, double *f, int i, int j, int k, int dx, int dy, int dz) {
    Lat *p = make(L); load(*p, f);
#if REF_DIM == 2
    (void)k; (void)dz;
    p->SmoothCornerAt(i, j, dx, dy);
#else
    p->SmoothCornerAt(i, j, k, dx, dy, dz);
#endif
    store(*p, f); delete p;
}
extern "C" void NAME(smooth_line)(const ol_lat *L, double *f, int plane, int a, int b, int da, int db) {
    Lat *p = make(L); load(*p, f);
#if REF_DIM == 3
    if (plane == 0) p->SmoothCornerAlongYZ(a, b, da, db);
    else if (plane == 1) p->SmoothCornerAlongZX(a, b, da, db);
    else p->SmoothCornerAlongXY(a, b, da, db);
#else
    (void)plane; (void)a; (void)b; (void)da; (void)db;
#endif
    store(*p, f); delete p;
}

extern "C" void NAME(collide)(const ol_lat *L, int kind, double *f, double *g, const ol_fields *F, const ol_phys *P, int save) {
    Lat *p = make(L), *q = make(L);
    load(*p, f);
    if (g) load(*q, g);
    double nu = P->nu, diff = P->diff, gx = P->gx, gy = P->gy, tem0 = P->tem0;
#if REF_DIM == 2
    switch (kind) {
    case OL_NS_COLLIDE: NS::MacroCollide(*p, F->rho, F->ux, F->uy, nu, save); break;
    case OL_NS_BRINKMAN: NS::MacroBrinkmanCollide(*p, F->rho, F->ux, F->uy, nu, F->alpha, save); break;
    case OL_AD_NATURAL: AD::MacroBrinkmanCollideNaturalConvection(*p, F->rho, F->ux, F->uy, F->alpha, nu, *q, F->tem, F->qx, F->qy, F->diffusivity, gx, gy, tem0, save, F->gsnap); break;
    case OL_AD_FORCE: AD::MacroBrinkmanCollideForceConvection(*p, F->rho, F->ux, F->uy, F->alpha, nu, *q, F->tem, F->qx, F->qy, F->diffusivity, save, F->gsnap); break;
    case OL_AD_HEATEX: AD::MacroBrinkmanCollideHeatExchange(*p, F->rho, F->ux, F->uy, F->alpha, nu, *q, F->tem, F->qx, F->qy, F->beta, diff, save); break;
    case OL_AD_NATURAL_NOBRINK: AD::MacroCollideNaturalConvection(*p, F->rho, F->ux, F->uy, nu, *q, F->tem, F->qx, F->qy, diff, gx, gy, tem0, save); break;
    case OL_AD_FORCE_NOBRINK: AD::MacroCollideForceConvection(*p, F->rho, F->ux, F->uy, nu, *q, F->tem, F->qx, F->qy, diff, save); break;
    case OL_ANS_BRINKMAN: ANS::MacroBrinkmanCollide(*p, F->rho, F->ux, F->uy, F->ip, F->iux, F->iuy, F->imx, F->imy, nu, F->alpha, save); break;
    case OL_AAD_NATURAL: AAD::MacroBrinkmanCollideNaturalConvection(*p, F->rho, F->ux, F->uy, F->ip, F->iux, F->iuy, F->imx, F->imy, F->alpha, nu, *q, F->tem, F->item, F->iqx, F->iqy, F->diffusivity, gx, gy, save, F->gsnap); break;
    case OL_AAD_FORCE: AAD::MacroBrinkmanCollideForceConvection(*p, F->rho, F->ux, F->uy, F->ip, F->iux, F->iuy, F->imx, F->imy, F->alpha, nu, *q, F->tem, F->item, F->iqx, F->iqy, F->diffusivity, save, F->gsnap); break;
    case OL_AAD_HEATEX: AAD::MacroBrinkmanCollideHeatExchange(*p, F->rho, F->ux, F->uy, F->ip, F->iux, F->iuy, F->imx, F->imy, F->alpha, nu, *q, F->tem, F->item, F->iqx, F->iqy, F->beta, diff, save); break;
    case OL_AAD_MASSFLOW: AAD::MacroBrinkmanCollideNaturalConvectionMassFlow(*p, F->rho, F->ux, F->uy, F->ip, F->iux, F->iuy, F->imx, F->imy, F->alpha, nu, *q, F->tem, F->item, F->iqx, F->iqy, F->diffusivity, gx, gy, F->dirx, F->diry, save, F->gsnap); break;
    case OL_NSIN_COLLIDE: NSin::MacroCollide(*p, F->rho, F->ux, F->uy, nu, save); break;
    case OL_NSIN_BRINKMAN: NSin::MacroBrinkmanCollide(*p, F->rho, F->ux, F->uy, nu, F->alpha, save); break;
    case OL_ANSIN_BRINKMAN: ANSin::MacroBrinkmanCollide(*p, F->rho, F->ux, F->uy, F->ip, F->iux, F->iuy, F->imx, F->imy, nu, F->alpha, save); break;
    case OL_EL_COLLIDE: EL::MacroCollide(*p, F->rho, F->ux, F->uy, F->sxx, F->sxy, F->syx, F->syy, P->tau, save); break;
    case OL_EL_EXTENDED: EL::MacroExtendedCollide(*p, F->rho, F->ux, F->uy, F->sxx, F->sxy, F->syx, F->syy, P->tau, F->gamma, save); break;
    case OL_AEL_COLLIDE: AEL::MacroCollide(*p, F->ip, F->imx, F->imy, F->isxx, F->isxy, F->isyx, F->isyy, P->tau, F->gamma, save); break;
    }
#else
    double gz = P->gz;
    switch (kind) {
    case OL_NS_COLLIDE: NS::MacroCollide(*p, F->rho, F->ux, F->uy, F->uz, nu, save); break;
    case OL_NS_BRINKMAN: NS::MacroBrinkmanCollide(*p, F->rho, F->ux, F->uy, F->uz, nu, F->alpha, save); break;
    case OL_AD_NATURAL: AD::MacroBrinkmanCollideNaturalConvection(*p, F->rho, F->ux, F->uy, F->uz, F->alpha, nu, *q, F->tem, F->qx, F->qy, F->qz, F->diffusivity, gx, gy, gz, tem0, save, F->gsnap); break;
    case OL_AD_FORCE: AD::MacroBrinkmanCollideForceConvection(*p, F->rho, F->ux, F->uy, F->uz, F->alpha, nu, *q, F->tem, F->qx, F->qy, F->qz, F->diffusivity, save, F->gsnap); break;
    case OL_AD_HEATEX: AD::MacroBrinkmanCollideHeatExchange(*p, F->rho, F->ux, F->uy, F->uz, F->alpha, nu, *q, F->tem, F->qx, F->qy, F->qz, F->beta, diff, save); break;
    case OL_AD_NATURAL_NOBRINK: AD::MacroCollideNaturalConvection(*p, F->rho, F->ux, F->uy, F->uz, nu, *q, F->tem, F->qx, F->qy, F->qz, diff, gx, gy, gz, tem0, save); break;
    case OL_AD_FORCE_NOBRINK: AD::MacroCollideForceConvection(*p, F->rho, F->ux, F->uy, F->uz, nu, *q, F->tem, F->qx, F->qy, F->qz, diff, save); break;
    case OL_ANS_BRINKMAN: ANS::MacroBrinkmanCollide(*p, F->rho, F->ux, F->uy, F->uz, F->ip, F->iux, F->iuy, F->iuz, F->imx, F->imy, F->imz, nu, F->alpha, save); break;
    case OL_AAD_NATURAL: AAD::MacroBrinkmanCollideNaturalConvection(*p, F->rho, F->ux, F->uy, F->uz, F->ip, F->iux, F->iuy, F->iuz, F->imx, F->imy, F->imz, F->alpha, nu, *q, F->tem, F->item, F->iqx, F->iqy, F->iqz, F->diffusivity, gx, gy, gz, save, F->gsnap); break;
    case OL_AAD_FORCE: AAD::MacroBrinkmanCollideForceConvection(*p, F->rho, F->ux, F->uy, F->uz, F->ip, F->iux, F->iuy, F->iuz, F->imx, F->imy, F->imz, F->alpha, nu, *q, F->tem, F->item, F->iqx, F->iqy, F->iqz, F->diffusivity, save, F->gsnap); break;
    case OL_AAD_HEATEX: AAD::MacroBrinkmanCollideHeatExchange(*p, F->rho, F->ux, F->uy, F->uz, F->ip, F->iux, F->iuy, F->iuz, F->imx, F->imy, F->imz, F->alpha, nu, *q, F->tem, F->item, F->iqx, F->iqy, F->iqz, F->beta, diff, save); break;
    case OL_AAD_MASSFLOW: AAD::MacroBrinkmanCollideNaturalConvectionMassFlow(*p, F->rho, F->ux, F->uy, F->uz, F->ip, F->iux, F->iuy, F->iuz, F->imx, F->imy, F->imz, F->alpha, nu, *q, F->tem, F->item, F->iqx, F->iqy, F->iqz, F->diffusivity, gx, gy, gz, F->dirx, F->diry, F->dirz, save, F->gsnap); break;
    }
#endif
    store(*p, f);
    if (g) store(*q, g);
    delete p;
    delete q;
}

extern "C" void NAME(init)(const ol_lat *L, int which, double *f, const ol_fields *F) {
    Lat *p = make(L);
#if REF_DIM == 2
    if (which == 0) NS::InitialCondition(*p, F->rho, F->ux, F->uy);
    else if (which == 1) AD::InitialCondition(*p, F->tem, F->ux, F->uy);
    else if (which == 2) ANS::InitialCondition(*p, F->ux, F->uy, F->ip, F->iux, F->iuy);
    else if (which == 4) NSin::InitialCondition(*p, F->rho, F->ux, F->uy);
    else if (which == 5) ANSin::InitialCondition(*p, F->ux, F->uy, F->ip, F->iux, F->iuy);
    else if (which == 6) EL::InitialCondition(*p, F->rho, F->ux, F->uy, F->sxx, F->sxy, F->syx, F->syy);
    else if (which == 7) AEL::InitialCondition(*p, F->ip, F->imx, F->imy, F->isxx, F->isxy, F->isyx, F->isyy, F->gamma);
    else AAD::InitialCondition(*p, F->ux, F->uy, F->item, F->iqx, F->iqy);
#else
    if (which == 0) NS::InitialCondition(*p, F->rho, F->ux, F->uy, F->uz);
    else if (which == 1) AD::InitialCondition(*p, F->tem, F->ux, F->uy, F->uz);
    else if (which == 2) ANS::InitialCondition(*p, F->ux, F->uy, F->uz, F->ip, F->iux, F->iuy, F->iuz);
    else AAD::InitialCondition(*p, F->ux, F->uy, F->uz, F->item, F->iqx, F->iqy, F->iqz);
#endif
    store(*p, f);
    delete p;
}

extern "C" void NAME(sensitivity)(const ol_lat *L, int which, double *dfds, const ol_fields *F, const double *dads,
                                  const double *dkds, const double *g, const double *ig, const double *qn, const int *mask) {
    Lat *p = make(L);
    auto QN = FD(qn[NID(i, j, k)]);
    auto M = FI(mask[NID(i, j, k)]);
#if REF_DIM == 2
    if (which == 0) AAD::SensitivityTemperatureAtHeatSource(*p, dfds, F->ux, F->uy, F->imx, F->imy, dads, F->tem, F->item, F->iqx, F->iqy, g, ig, F->diffusivity, dkds, QN, M);
    else if (which == 1) AAD::SensitivityBrinkmanDiffusivity(*p, dfds, F->ux, F->uy, F->imx, F->imy, dads, F->tem, F->item, F->iqx, F->iqy, g, ig, F->diffusivity, dkds);
    else if (which == 2) AAD::SensitivityHeatExchange(*p, dfds, F->ux, F->uy, F->imx, F->imy, dads, F->tem, F->item, dkds);
    else if (which == 4) AEL::SensitivityCompliance(*p, dfds, F->sxx, F->sxy, F->syx, F->syy, F->ip, F->isxx, F->isxy, F->isyx, F->isyy);
    else ANS::SensitivityBrinkman(*p, dfds, F->ux, F->uy, F->imx, F->imy, dads);
#else
    if (which == 0) {
        /* bulk terms, then the six face terms with (_ig, _uz) bound to the parameters of those
         * names (the scalar wrapper at adjointadvection.h:1537 swaps them) */
        AAD::SensitivityBrinkmanDiffusivity(*p, dfds, F->ux, F->uy, F->uz, F->imx, F->imy, F->imz, dads, F->tem, F->item, F->iqx, F->iqy, F->iqz, g, ig, F->diffusivity, dkds);
        AAD::SensitivityTemperatureAtHeatSourceAlongXFace(*p, 0, -1, F->ux, F->uy, ig, F->uz, dfds, F->diffusivity, dkds, QN, M);
        AAD::SensitivityTemperatureAtHeatSourceAlongXFace(*p, p->lx - 1, 1, F->ux, F->uy, ig, F->uz, dfds, F->diffusivity, dkds, QN, M);
        AAD::SensitivityTemperatureAtHeatSourceAlongYFace(*p, 0, -1, F->ux, F->uy, ig, F->uz, dfds, F->diffusivity, dkds, QN, M);
        AAD::SensitivityTemperatureAtHeatSourceAlongYFace(*p, p->ly - 1, 1, F->ux, F->uy, ig, F->uz, dfds, F->diffusivity, dkds, QN, M);
        AAD::SensitivityTemperatureAtHeatSourceAlongZFace(*p, 0, -1, F->ux, F->uy, ig, F->uz, dfds, F->diffusivity, dkds, QN, M);
        AAD::SensitivityTemperatureAtHeatSourceAlongZFace(*p, p->lz - 1, 1, F->ux, F->uy, ig, F->uz, dfds, F->diffusivity, dkds, QN, M);
    }
    else if (which == 1) AAD::SensitivityBrinkmanDiffusivity(*p, dfds, F->ux, F->uy, F->uz, F->imx, F->imy, F->imz, dads, F->tem, F->item, F->iqx, F->iqy, F->iqz, g, ig, F->diffusivity, dkds);
    else if (which == 2) AAD::SensitivityHeatExchange(*p, dfds, F->ux, F->uy, F->uz, F->imx, F->imy, F->imz, dads, F->tem, F->item, dkds);
    else ANS::SensitivityBrinkman(*p, dfds, F->ux, F->uy, F->uz, F->imx, F->imy, F->imz, dads);
#endif
    delete p;
}

/* filter weight: hat between two design cells, identity otherwise (production drivers) */
#define WEIGHT_LAMBDA                                                                              \
    [&](int i1, int j1, int k1, int i2, int j2, int k2) {                                        \
        auto inb = [&](int i, int j, int k) { return 0 <= i && i < L->nx && 0 <= j && j < L->ny && 0 <= k && k < nzz; }; \
        bool des = !mask || (inb(i1, j1, k1) && inb(i2, j2, k2) && mask[i1 + L->nx * (j1 + L->ny * k1)] && mask[i2 + L->nx * (j2 + L->ny * k2)]); \
        if (des) return (R - sqrt(pow(i1 - i2, 2.0) + pow(j1 - j2, 2.0) + pow(k1 - k2, 2.0))) / R; \
        return (i1 == i2 && j1 == j2 && k1 == k2) ? 1.0 : 0.0;                                   \
    }

extern "C" void NAME(heaviside_var)(const ol_lat *L, double R, double beta, const double *s, const int *mask, double *out) {
    Lat *p = make(L);
    int nzz = p->nz;
    std::vector<double> sv(s, s + p->nxyz);
    std::vector<double> r = HeavisideFilter::GetFilteredVariable(*p, R, beta, sv, WEIGHT_LAMBDA);
    std::memcpy(out, r.data(), sizeof(double) * p->nxyz);
    delete p;
}
extern "C" void NAME(heaviside_sens)(const ol_lat *L, double R, double beta, const double *s, const double *dfdrho, const int *mask, double *out) {
    Lat *p = make(L);
    int nzz = p->nz;
    std::vector<double> sv(s, s + p->nxyz), dv(dfdrho, dfdrho + p->nxyz);
    std::vector<double> r = HeavisideFilter::GetFilteredSensitivity(*p, R, beta, sv, dv, WEIGHT_LAMBDA);
    std::memcpy(out, r.data(), sizeof(double) * p->nxyz);
    delete p;
}
extern "C" void NAME(density_filter)(const ol_lat *L, double R, const double *v, const int *mask, double *out) {
    Lat *p = make(L);
    int nzz = p->nz;
    std::vector<double> vv(v, v + p->nxyz);
    std::vector<double> r = DensityFilter::GetFilteredValue(*p, R, vv, WEIGHT_LAMBDA);
    std::memcpy(out, r.data(), sizeof(double) * p->nxyz);
    delete p;
}

/* the filters with a general weight functor: the reference's own routines called with a functor
 * that reads the table w[node][tap] (taps: offsets within R in the (i2, j2, k2) loop order; 2D:
 * k2 = k1 only, the other offsets are never inside the lattice) */
extern "C" void NAME(filter_table)(const ol_lat *L, int op, double R, double beta, const double *a, const double *b,
                                   const double *w, double *out) {
    Lat *p = make(L);
    const int nR = (int)R, span = 2 * nR + 1;
    std::vector<int> tapix((size_t)span * span * span, -1);
    int nt = 0;
    for (int da = -nR; da <= nR; ++da)
        for (int db = -nR; db <= nR; ++db)
            for (int dc = (REF_DIM == 3 ? -nR : 0); dc <= (REF_DIM == 3 ? nR : 0); ++dc)
                if (sqrt(pow((double)da, 2.0) + pow((double)db, 2.0) + pow((double)dc, 2.0)) <= R)
                    tapix[((size_t)(da + nR) * span + (db + nR)) * span + (dc + nR)] = nt++;
    const int nx = L->nx, ny = L->ny;
    auto weight = [&](int i1, int j1, int k1, int i2, int j2, int k2) {
        const int t = tapix[((size_t)(i2 - i1 + nR) * span + (j2 - j1 + nR)) * span + (k2 - k1 + nR)];
        if (t < 0) return 0.0;
        return w[((size_t)i1 + (size_t)nx * ((size_t)j1 + (size_t)ny * k1)) * nt + t];
    };
    std::vector<double> av(a, a + p->nxyz), r;
    if (op == 0) r = HeavisideFilter::GetFilteredVariable(*p, R, beta, av, weight);
    else if (op == 1) r = HeavisideFilter::GetFilteredSensitivity(*p, R, beta, av, std::vector<double>(b, b + p->nxyz), weight);
    else r = DensityFilter::GetFilteredValue(*p, R, av, weight);
    std::memcpy(out, r.data(), sizeof(double) * p->nxyz);
    delete p;
}

#if REF_DIM == 2
extern "C" double ref_residual(int n, int ncomp, const double *const *a, const double *const *b) {
    if (ncomp == 1) return Residual(a[0], b[0], n);
    if (ncomp == 2) return Residual(a[0], a[1], b[0], b[1], n);
    return Residual(a[0], a[1], a[2], b[0], b[1], b[2], n);
}
extern "C" void ref_normalize(double *v, int n) { Normalize(v, n); }
#endif
