// physics.cuh -- per-node lattice-Boltzmann arithmetic of the NS / AD forward and adjoint
// collides (device code). Each routine restates the reference routine cited beside it with
// the same evaluation order, so FP64 builds compiled without FMA contraction reproduce the
// reference's scalar results; FP32 builds are the throughput path.
#pragma once
#include "common.h"
#include "lattice.cuh"

namespace pl {

// c . u over the non-zero components of c, left to right (x, y, z)
template <class L, class T> __device__ __forceinline__ T cdot(int c, T u0, T u1, T u2) {
    T s = T(0);
    bool first = true;
    const int a0 = L::cx(c), a1 = L::cy(c), a2 = L::cz(c);
    if (a0 != 0) { s = a0 > 0 ? u0 : -u0; first = false; }
    if (a1 != 0) { if (first) { s = a1 > 0 ? u1 : -u1; first = false; } else s = a1 > 0 ? s + u1 : s - u1; }
    if (L::ND == 3 && a2 != 0) { if (first) { s = a2 > 0 ? u2 : -u2; } else s = a2 > 0 ? s + u2 : s - u2; }
    return s;
}
template <class L, class T> __device__ __forceinline__ T vdot(const T *a, const T *b) {
    return L::ND == 2 ? a[0] * b[0] + a[1] * b[1] : a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}
template <class L, class T> __device__ __forceinline__ T wt(int c) { return L::template w<T>(c); }

// NS::Macro (navierstokes.h:15-50)
template <class L, class T> __device__ __forceinline__ void ns_macro(const T *f, T &rho, T *u) {
    T r = f[0], m0 = T(0), m1 = T(0), m2 = T(0);
#pragma unroll
    for (int c = 1; c < L::Q; ++c) {
        const T v = f[c];
        r += v;
        if (L::cx(c) == 1) m0 += v; else if (L::cx(c) == -1) m0 -= v;
        if (L::cy(c) == 1) m1 += v; else if (L::cy(c) == -1) m1 -= v;
        if (L::cz(c) == 1) m2 += v; else if (L::cz(c) == -1) m2 -= v;
    }
    const T inv = T(1) / r;
    rho = r;
    u[0] = m0 * inv;
    u[1] = m1 * inv;
    u[2] = L::ND == 3 ? m2 * inv : T(0);
}
// NS::Equilibrium (navierstokes.h:52-70), fused into the BGK relaxation
template <class L, class T> __device__ __forceinline__ T ns_feq(int c, T rho, const T *u, T uu) {
    const T ciu = cdot<L, T>(c, u[0], u[1], u[2]);
    return wt<L, T>(c) * rho * (T(3) * ciu + T(4.5) * ciu * ciu + uu);
}
template <class L, class T> __device__ __forceinline__ T ns_uu(const T *u) {
    return L::ND == 2 ? T(1) - T(1.5) * (u[0] * u[0] + u[1] * u[1])
                      : T(1) - T(1.5) * (u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
}
// NS::ExternalForceBrinkman (navierstokes.h:72-88)
template <class L, class T> __device__ __forceinline__ void ns_brinkman(T *f, T rho, const T *u, T alpha) {
    const T coef = T(3) * alpha * rho / (rho + alpha);
#pragma unroll
    for (int c = 1; c < L::Q; ++c) f[c] -= coef * wt<L, T>(c) * cdot<L, T>(c, u[0], u[1], u[2]);
}
// AD::Macro (advection.h:16-51)
template <class L, class T> __device__ __forceinline__ void ad_macro(const T *g, const T *u, T omg, T &tem, T *q) {
    T t = g[0], s0 = T(0), s1 = T(0), s2 = T(0);
#pragma unroll
    for (int c = 1; c < L::Q; ++c) {
        const T v = g[c];
        t += v;
        if (L::cx(c) == 1) s0 += v; else if (L::cx(c) == -1) s0 -= v;
        if (L::cy(c) == 1) s1 += v; else if (L::cy(c) == -1) s1 -= v;
        if (L::cz(c) == 1) s2 += v; else if (L::cz(c) == -1) s2 -= v;
    }
    const T coef = T(1) - T(0.5) * omg;
    tem = t;
    q[0] = coef * (s0 - t * u[0]);
    q[1] = coef * (s1 - t * u[1]);
    q[2] = L::ND == 3 ? coef * (s2 - t * u[2]) : T(0);
}
// AD::Equilibrium (advection.h:53-69)
template <class L, class T> __device__ __forceinline__ T ad_geq(int c, T tem, const T *u) {
    return wt<L, T>(c) * tem * (T(1) + T(3) * cdot<L, T>(c, u[0], u[1], u[2]));
}
// AD::ExternalForceNaturalConvection (advection.h:71-85)
template <class L, class T> __device__ __forceinline__ void ad_nc_force(T *f, T tem, T gx, T gy, T gz, T tem0) {
#pragma unroll
    for (int c = 1; c < L::Q; ++c) f[c] += T(3) * wt<L, T>(c) * cdot<L, T>(c, gx, gy, gz) * (tem - tem0);
}
// AD::ExternalForceHeatExchange (advection.h:87-95)
template <class L, class T> __device__ __forceinline__ void ad_heatex(T *g, T tem, T beta) {
    const T coef = beta * (T(1) - tem) / (T(1) + beta);
#pragma unroll
    for (int c = 0; c < L::Q; ++c) g[c] += wt<L, T>(c) * coef;
}
// ANS::Macro (adjointnavierstokes.h:15-57)
template <class L, class T> __device__ __forceinline__ void ans_macro(const T *f, const T *u, T &ip, T *iu, T *im) {
    const T uu = vdot<L, T>(u, u);
    const T w0 = wt<L, T>(0);
    ip = f[0] * w0 * (T(1) - T(1.5) * uu);
#pragma unroll
    for (int b = 0; b < 3; ++b) { iu[b] = -f[0] * w0 * u[b]; im[b] = T(0); }
#pragma unroll
    for (int c = 1; c < L::Q; ++c) {
        const T ciu = cdot<L, T>(c, u[0], u[1], u[2]);
        const T fei = f[c] * wt<L, T>(c);
        ip += fei * (T(1) + T(3) * ciu + T(4.5) * ciu * ciu - T(1.5) * uu);
#pragma unroll
        for (int b = 0; b < L::ND; ++b) {
            const T cb = T(comp<L>(c, b));
            iu[b] += fei * (cb + T(3) * ciu * cb - u[b]);
        }
#pragma unroll
        for (int b = 0; b < L::ND; ++b) {
            const int cb = comp<L>(c, b);
            if (cb == 1) im[b] += fei; else if (cb == -1) im[b] -= fei;
        }
    }
    if (L::ND == 2) { iu[2] = T(0); im[2] = T(0); }
}
// ANS::Equilibrium (adjointnavierstokes.h:59-73)
template <class L, class T> __device__ __forceinline__ T ans_feq(int c, const T *u, T ip, const T *iu) {
    const T s = L::ND == 2
        ? iu[0] * (T(L::cx(c)) - u[0]) + iu[1] * (T(L::cy(c)) - u[1])
        : iu[0] * (T(L::cx(c)) - u[0]) + iu[1] * (T(L::cy(c)) - u[1]) + iu[2] * (T(L::cz(c)) - u[2]);
    return ip + T(3) * s;
}
// ANS::ExternalForceBrinkman (adjointnavierstokes.h:75-93)
template <class L, class T> __device__ __forceinline__ void ans_brinkman(T *f, T rho, const T *u, const T *im, T alpha) {
    const T coef = T(3) * alpha / (rho + alpha);
    f[0] -= -coef * vdot<L, T>(u, im);
#pragma unroll
    for (int c = 1; c < L::Q; ++c) {
        const T s = L::ND == 2
            ? (T(L::cx(c)) - u[0]) * im[0] + (T(L::cy(c)) - u[1]) * im[1]
            : (T(L::cx(c)) - u[0]) * im[0] + (T(L::cy(c)) - u[1]) * im[1] + (T(L::cz(c)) - u[2]) * im[2];
        f[c] -= coef * s;
    }
}
// AAD::Macro (adjointadvection.h:22-50)
template <class L, class T> __device__ __forceinline__ void aad_macro(const T *g, T &item, T *iq) {
    T it = wt<L, T>(0) * g[0], s0 = T(0), s1 = T(0), s2 = T(0);
#pragma unroll
    for (int c = 1; c < L::Q; ++c) {
        const T gei = wt<L, T>(c) * g[c];
        it += gei;
        if (L::cx(c) == 1) s0 += gei; else if (L::cx(c) == -1) s0 -= gei;
        if (L::cy(c) == 1) s1 += gei; else if (L::cy(c) == -1) s1 -= gei;
        if (L::cz(c) == 1) s2 += gei; else if (L::cz(c) == -1) s2 -= gei;
    }
    item = it;
    iq[0] = s0; iq[1] = s1; iq[2] = s2;
}
// AAD::ExternalForceBrinkman (adjointadvection.h:70-102)
template <class L, class T> __device__ __forceinline__ void aad_brinkman(T *f, T rho, const T *u, const T *im, T tem,
                                                                        const T *iq, T omg, T alpha) {
    const T coef = T(3) / (rho + alpha);
    T X[3];
#pragma unroll
    for (int b = 0; b < 3; ++b) X[b] = tem * iq[b] * omg - alpha * im[b];
    const T s0 = L::ND == 2 ? -u[0] * X[0] + -u[1] * X[1] : -u[0] * X[0] + -u[1] * X[1] + -u[2] * X[2];
    f[0] += coef * s0;
#pragma unroll
    for (int c = 1; c < L::Q; ++c) {
        const T s = L::ND == 2
            ? (T(L::cx(c)) - u[0]) * X[0] + (T(L::cy(c)) - u[1]) * X[1]
            : (T(L::cx(c)) - u[0]) * X[0] + (T(L::cy(c)) - u[1]) * X[1] + (T(L::cz(c)) - u[2]) * X[2];
        f[c] += coef * s;
    }
}
// AAD::ExternalForceHeatExchange (adjointadvection.h:104-112)
template <class L, class T> __device__ __forceinline__ void aad_heatex(T *g, T item, T beta) {
    const T coef = beta * (T(1) + item) / (T(1) + beta);
#pragma unroll
    for (int c = 0; c < L::Q; ++c) g[c] -= coef;
}
// Volumetric heat source of the forced-convection heat sink (no reference routine): g_c += w_c Q,
// the form of the heat-exchange term with a fixed source
template <class L, class T> __device__ __forceinline__ void ad_source(T *g, T qsrc) {
#pragma unroll
    for (int c = 0; c < L::Q; ++c) g[c] += wt<L, T>(c) * qsrc;
}
// Its adjoint objective source: J = sum_x w(x) T(x) gives dJ/dg_c = w for every c, added in the
// convention of the heat-exchange adjoint above (whose "1" is its objective's derivative)
template <class L, class T> __device__ __forceinline__ void aad_objsrc(T *g, T w) {
#pragma unroll
    for (int c = 0; c < L::Q; ++c) g[c] += w;
}
// AAD::ExternalForceNaturalConvection (adjointadvection.h:114-132)
template <class L, class T> __device__ __forceinline__ void aad_nc(T *g, const T *im, const T *gv) {
    const T coef = T(3) * vdot<L, T>(im, gv);
#pragma unroll
    for (int c = 0; c < L::Q; ++c) g[c] += coef;
}
// AAD::ExternalForceMassFlow (adjointadvection.h:134-150)
template <class L, class T> __device__ __forceinline__ void aad_massflow(T *f, T rho, const T *u, const T *dv) {
    f[0] += vdot<L, T>(u, dv) / rho;
#pragma unroll
    for (int c = 1; c < L::Q; ++c) {
        const T s = L::ND == 2
            ? (T(L::cx(c)) - u[0]) * dv[0] + (T(L::cy(c)) - u[1]) * dv[1]
            : (T(L::cx(c)) - u[0]) * dv[0] + (T(L::cy(c)) - u[1]) * dv[1] + (T(L::cz(c)) - u[2]) * dv[2];
        f[c] -= s / rho;
    }
}

// ---- incompressible variants (D2Q9) -------------------------------------------------------
// NSin::Macro (nsincompressible.h:13-25): rho and the momentum sums, without the division by rho
template <class L, class T> __device__ __forceinline__ void nsin_macro(const T *f, T &rho, T *u) {
    T r = f[0], m0 = T(0), m1 = T(0);
#pragma unroll
    for (int c = 1; c < L::Q; ++c) {
        const T v = f[c];
        r += v;
        if (L::cx(c) == 1) m0 += v; else if (L::cx(c) == -1) m0 -= v;
        if (L::cy(c) == 1) m1 += v; else if (L::cy(c) == -1) m1 -= v;
    }
    rho = r;
    u[0] = m0; u[1] = m1; u[2] = T(0);
}
// NSin::Equilibrium (nsincompressible.h:27-35); rhouu = rho - 1.5 u.u
template <class L, class T> __device__ __forceinline__ T nsin_feq(int c, const T *u, T rhouu) {
    const T ciu = cdot<L, T>(c, u[0], u[1], T(0));
    return wt<L, T>(c) * (T(3) * ciu + T(4.5) * ciu * ciu + rhouu);
}
// ANSin::Macro (adjointnsincompressible.h:13-30)
template <class L, class T> __device__ __forceinline__ void ansin_macro(const T *f, const T *u, T &ip, T *iu, T *im) {
    const T w0 = wt<L, T>(0);
    ip = f[0] * w0;
    iu[0] = -f[0] * w0 * u[0]; iu[1] = -f[0] * w0 * u[1];
    im[0] = T(0); im[1] = T(0);
#pragma unroll
    for (int c = 1; c < L::Q; ++c) {
        const T ciu = cdot<L, T>(c, u[0], u[1], T(0));
        const T fei = f[c] * wt<L, T>(c);
        ip += fei;
#pragma unroll
        for (int b = 0; b < 2; ++b) {
            const T cb = T(comp<L>(c, b));
            iu[b] += fei * (cb + T(3) * ciu * cb - u[b]);
        }
#pragma unroll
        for (int b = 0; b < 2; ++b) {
            const int cb = comp<L>(c, b);
            if (cb == 1) im[b] += fei; else if (cb == -1) im[b] -= fei;
        }
    }
    iu[2] = T(0); im[2] = T(0);
}
// ANSin::Equilibrium (adjointnsincompressible.h:32-38)
template <class L, class T> __device__ __forceinline__ T ansin_feq(int c, T ip, const T *iu) {
    return ip + T(3) * cdot<L, T>(c, iu[0], iu[1], T(0));
}
// ANSin::ExternalForceBrinkman (adjointnsincompressible.h:40-47)
template <class L, class T> __device__ __forceinline__ void ansin_brinkman(T *f, const T *im, T alpha) {
    const T coef = T(3) * alpha / (T(1) + alpha);
#pragma unroll
    for (int c = 1; c < L::Q; ++c) f[c] -= coef * cdot<L, T>(c, im[0], im[1], T(0));
}

template <class T> __device__ __forceinline__ T ldT(const void *p, int idx) { return static_cast<const T *>(p)[idx]; }

// ---- elastic LBM (EL / AEL), D2Q9 only in the reference ----------------------------------
// EL::Macro (elastic.h:17-47): u = (sum_{c>=1} c f) / rho, s_ab = -sum_{c>=1} c_a c_b f.
// s = {sxx, sxy, syx, syy}.
template <class L, class T> __device__ __forceinline__ void el_macro(const T *f, T rho, T *u, T *s) {
    T ux = T(0), uy = T(0), sxx = T(0), sxy = T(0), syx = T(0), syy = T(0);
#pragma unroll
    for (int c = 1; c < L::Q; ++c) {
        const T v = f[c], cx = T(comp<L>(c, 0)), cy = T(comp<L>(c, 1));
        ux += cx * v;
        uy += cy * v;
        sxx -= cx * cx * v;
        sxy -= cx * cy * v;
        syx -= cy * cx * v;
        syy -= cy * cy * v;
    }
    const T invrho = T(1) / rho;
    u[0] = ux * invrho; u[1] = uy * invrho; u[2] = T(0);
    s[0] = sxx; s[1] = sxy; s[2] = syx; s[3] = syy;
}
// EL::Equilibrium (elastic.h:49-58): w (3 rho c.u - 4.5 c.s.c + 1.5 tr s)
template <class L, class T> __device__ __forceinline__ T el_feq(int c, T rho, const T *u, const T *s) {
    const T cx = T(comp<L>(c, 0)), cy = T(comp<L>(c, 1));
    const T ciu = cx * u[0] + cy * u[1];
    const T cisci = cx * s[0] * cx + cx * s[1] * cy + cy * s[2] * cx + cy * s[3] * cy;
    const T trss = s[0] + s[3];
    return wt<L, T>(c) * (T(3) * rho * ciu - T(4.5) * cisci + T(1.5) * trss);
}
// AEL::Macro (adjointelastic.h:16-35): m = {irho, imx, imy, isxx, isxy, isyx, isyy} with
// irho = sum w f, im = sum w c f, is_ab = sum w c_a c_b f
template <class L, class T> __device__ __forceinline__ void ael_macro(const T *f, T *m) {
    T irho = wt<L, T>(0) * f[0], imx = T(0), imy = T(0), isxx = T(0), isxy = T(0), isyx = T(0), isyy = T(0);
#pragma unroll
    for (int c = 1; c < L::Q; ++c) {
        const T v = f[c], e = wt<L, T>(c), cx = T(comp<L>(c, 0)), cy = T(comp<L>(c, 1));
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
// AEL::Equilibrium (adjointelastic.h:37-46): 3 im.c + 4.5 gamma c.is.c - 1.5 gamma irho |c|^2
template <class L, class T> __device__ __forceinline__ T ael_feq(int c, const T *m, T gamma) {
    const int icx = comp<L>(c, 0), icy = comp<L>(c, 1);
    const T cx = T(icx), cy = T(icy);
    const T imc = m[1] * cx + m[2] * cy;
    const T cisc = cx * m[3] * cx + cx * m[4] * cy + cy * m[5] * cx + cy * m[6] * cy;
    const T irhocc = m[0] * T(icx * icx + icy * icy);
    return T(3) * imc + T(4.5) * gamma * cisc - T(1.5) * gamma * irhocc;
}

// EL::MacroCollide / MacroExtendedCollide (elastic.h:109-166) and AEL::MacroCollide
// (adjointelastic.h:96-125) for one node; the BGK rate is 1 / tau
template <class L, class T, int K>
__device__ __forceinline__ void collide_elastic(T *f, int idx, const KArgs &a, bool save, T *uout) {
    constexpr int Q = L::Q;
    const T om = T(1) / T(a.ph.tau), iom = T(1) - om;
    if (K == K_EL_COLLIDE || K == K_EL_EXTENDED) {
        const T rho = ldT<T>(a.elrho, idx);
        T u[3], s[4];
        el_macro<L, T>(f, rho, u, s);
        if (K == K_EL_EXTENDED) {
            const T gm = ldT<T>(a.gamma, idx);
#pragma unroll
            for (int m = 0; m < 4; ++m) s[m] *= gm;
        }
        if (save) {
            if (a.out[1]) a.out[1][idx] = double(u[0]);
            if (a.out[2]) a.out[2][idx] = double(u[1]);
#pragma unroll
            for (int m = 0; m < 4; ++m) if (a.out[4 + m]) a.out[4 + m][idx] = double(s[m]);
        }
        if (uout) { uout[0] = u[0]; uout[1] = u[1]; uout[2] = T(0); }
#pragma unroll
        for (int c = 0; c < Q; ++c) f[c] = iom * f[c] + om * el_feq<L, T>(c, rho, u, s);
    } else {
        T m[7];
        ael_macro<L, T>(f, m);
        if (save) {
            if (a.out[0]) a.out[0][idx] = double(m[0]);
            if (a.out[4]) a.out[4][idx] = double(m[1]);
            if (a.out[5]) a.out[5][idx] = double(m[2]);
#pragma unroll
            for (int k = 0; k < 4; ++k) if (a.out[7 + k]) a.out[7 + k][idx] = double(m[3 + k]);
        }
        const T gm = ldT<T>(a.gamma, idx);
#pragma unroll
        for (int c = 0; c < Q; ++c) f[c] = iom * f[c] + om * ael_feq<L, T>(c, m, gm);
    }
}

// NSin::MacroCollide / MacroBrinkmanCollide (nsincompressible.h:144-200) and
// ANSin::MacroBrinkmanCollide (adjointnsincompressible.h:143-178) for one node
template <class L, class T, int K>
__device__ __forceinline__ void collide_incompressible(T *f, int idx, const KArgs &a, bool save, T *uout) {
    constexpr int Q = L::Q;
    const T omf = T(1) / (T(3) * T(a.ph.nu) + T(0.5));
    const T iomf = T(1) - omf;
    if (K == K_NSIN_COLLIDE || K == K_NSIN_BRINKMAN) {
        T rho, u[3];
        nsin_macro<L, T>(f, rho, u);
        if (K == K_NSIN_BRINKMAN) {
            ns_brinkman<L, T>(f, rho, u, ldT<T>(a.alpha, idx));
            nsin_macro<L, T>(f, rho, u);
        }
        if (save) {
            if (a.out[0]) a.out[0][idx] = double(rho);
            if (a.out[1]) a.out[1][idx] = double(u[0]);
            if (a.out[2]) a.out[2][idx] = double(u[1]);
        }
        if (uout) { uout[0] = u[0]; uout[1] = u[1]; uout[2] = T(0); }
        const T rhouu = rho - T(1.5) * (u[0] * u[0] + u[1] * u[1]);
#pragma unroll
        for (int c = 0; c < Q; ++c) f[c] = iomf * f[c] + omf * nsin_feq<L, T>(c, u, rhouu);
    } else {
        const T u[3] = {ldT<T>(a.fwd[1], idx), ldT<T>(a.fwd[2], idx), T(0)};
        T ip, iu[3], im[3];
        ansin_macro<L, T>(f, u, ip, iu, im);
        ansin_brinkman<L, T>(f, im, ldT<T>(a.alpha, idx));
        ansin_macro<L, T>(f, u, ip, iu, im);
        if (save) {
            if (a.out[0]) a.out[0][idx] = double(ip);
            if (a.out[1]) a.out[1][idx] = double(iu[0]);
            if (a.out[2]) a.out[2][idx] = double(iu[1]);
            if (a.out[4]) a.out[4][idx] = double(im[0]);
            if (a.out[5]) a.out[5][idx] = double(im[1]);
        }
#pragma unroll
        for (int c = 0; c < Q; ++c) f[c] = iomf * f[c] + omf * ansin_feq<L, T>(c, ip, iu);
    }
}

// Macro + forces + BGK for one node, one reference collide routine per kind:
// NS::MacroCollide / MacroBrinkmanCollide (navierstokes.h:430-546); AD::MacroCollide{Force,
// Natural}Convection, MacroBrinkmanCollide{HeatExchange,ForceConvection,NaturalConvection}
// (advection.h:528-1044); ANS::MacroBrinkmanCollide (adjointnavierstokes.h:396-470);
// AAD::MacroBrinkmanCollide{HeatExchange,ForceConvection,NaturalConvection,
// NaturalConvectionMassFlow} (adjointadvection.h:892-1355).
// f, g: pre-collision populations in, post-collision out. When `snap` is non-null the
// snapshot (the g populations at the point the reference saves them) is written to it.
template <class L, class T, int K>
__device__ __forceinline__ void collide_node(T *f, T *g, int idx, const KArgs &a, bool save, double *snap,
                                             long long np, T *uout) {
    if constexpr (kind_incompressible(K)) {
        collide_incompressible<L, T, K>(f, idx, a, save, uout);
        return;
    }
    if constexpr (kind_elastic(K)) {
        collide_elastic<L, T, K>(f, idx, a, save, uout);
        return;
    }
    constexpr int Q = L::Q;
    const T omf = T(1) / (T(3) * T(a.ph.nu) + T(0.5));
    T omg = T(0);
    if (K == K_AD_NATURAL || K == K_AD_FORCE || K == K_AAD_NATURAL || K == K_AAD_FORCE || K == K_AAD_MASSFLOW)
        omg = T(1) / (T(3) * ldT<T>(a.kappa, idx) + T(0.5));
    else if (kind_has_g(K))
        omg = T(1) / (T(3) * T(a.ph.diff) + T(0.5));
    const T gv[3] = {T(a.ph.gx), T(a.ph.gy), T(a.ph.gz)};
    if (!kind_is_adjoint(K)) {
        T rho, u[3], tem = T(0), q[3] = {T(0), T(0), T(0)};
        ns_macro<L, T>(f, rho, u);
        if (kind_has_g(K)) ad_macro<L, T>(g, u, omg, tem, q);
        if (K == K_NS_BRINKMAN || K == K_AD_FORCE || K == K_AD_HEATEX) {
            ns_brinkman<L, T>(f, rho, u, ldT<T>(a.alpha, idx));
            ns_macro<L, T>(f, rho, u);
            if (K == K_AD_HEATEX) ad_heatex<L, T>(g, tem, ldT<T>(a.beta, idx));
            if (K == K_AD_FORCE && a.hsrc) ad_source<L, T>(g, ldT<T>(a.hsrc, idx));
            if (kind_has_g(K)) ad_macro<L, T>(g, u, omg, tem, q);
        } else if (K == K_AD_NATURAL) {
            ad_nc_force<L, T>(f, tem, gv[0], gv[1], gv[2], T(a.ph.tem0));
            ns_brinkman<L, T>(f, rho, u, ldT<T>(a.alpha, idx));
            ns_macro<L, T>(f, rho, u);
            ad_macro<L, T>(g, u, omg, tem, q);
        } else if (K == K_AD_NATURAL_NOBRINK) {
            ad_nc_force<L, T>(f, tem, gv[0], gv[1], gv[2], T(a.ph.tem0));
            ns_macro<L, T>(f, rho, u);
            ad_macro<L, T>(g, u, omg, tem, q);
        }
        if (save) {
            if (a.out[0]) a.out[0][idx] = double(rho);
            if (a.out[1]) a.out[1][idx] = double(u[0]);
            if (a.out[2]) a.out[2][idx] = double(u[1]);
            if (L::ND == 3 && a.out[3]) a.out[3][idx] = double(u[2]);
            if (kind_has_g(K)) {
                if (a.out[4]) a.out[4][idx] = double(tem);
                if (a.out[5]) a.out[5][idx] = double(q[0]);
                if (a.out[6]) a.out[6][idx] = double(q[1]);
                if (L::ND == 3 && a.out[7]) a.out[7][idx] = double(q[2]);
            }
        }
        if (uout) { uout[0] = u[0]; uout[1] = u[1]; uout[2] = u[2]; }
        if (snap && kind_has_snapshot(K)) {
#pragma unroll
            for (int c = 0; c < Q; ++c) snap[c * np + idx] = double(g[c]);
        }
        const T uu = ns_uu<L, T>(u);
        const T iomf = T(1) - omf;
#pragma unroll
        for (int c = 0; c < Q; ++c) f[c] = iomf * f[c] + omf * ns_feq<L, T>(c, rho, u, uu);
        if (kind_has_g(K)) {
            const T iomg = T(1) - omg;
#pragma unroll
            for (int c = 0; c < Q; ++c) g[c] = iomg * g[c] + omg * ad_geq<L, T>(c, tem, u);
        }
    } else {
        const T rho = ldT<T>(a.fwd[0], idx);
        const T u[3] = {ldT<T>(a.fwd[1], idx), ldT<T>(a.fwd[2], idx), L::ND == 3 ? ldT<T>(a.fwd[3], idx) : T(0)};
        T ip, iu[3], im[3], item = T(0), iq[3] = {T(0), T(0), T(0)};
        ans_macro<L, T>(f, u, ip, iu, im);
        if (K == K_ANS_BRINKMAN) {
            ans_brinkman<L, T>(f, rho, u, im, ldT<T>(a.alpha, idx));
            ans_macro<L, T>(f, u, ip, iu, im);
        } else {
            const T tem = ldT<T>(a.fwd[4], idx);
            aad_macro<L, T>(g, item, iq);
            if (K == K_AAD_MASSFLOW) {
                const T dv[3] = {ldT<T>(a.dirx, idx), ldT<T>(a.diry, idx), L::ND == 3 ? ldT<T>(a.dirz, idx) : T(0)};
                aad_massflow<L, T>(f, rho, u, dv);
            }
            aad_brinkman<L, T>(f, rho, u, im, tem, iq, omg, ldT<T>(a.alpha, idx));
            ans_macro<L, T>(f, u, ip, iu, im);
            if (K == K_AAD_NATURAL || K == K_AAD_MASSFLOW) {
                aad_nc<L, T>(g, im, gv);
                aad_macro<L, T>(g, item, iq);
            } else if (K == K_AAD_HEATEX) {
                aad_heatex<L, T>(g, item, ldT<T>(a.beta, idx));
                aad_macro<L, T>(g, item, iq);
            } else if (K == K_AAD_FORCE && a.objw) {
                aad_objsrc<L, T>(g, ldT<T>(a.objw, idx));
                aad_macro<L, T>(g, item, iq);
            }
        }
        if (save) {
            if (a.out[0]) a.out[0][idx] = double(ip);
            if (a.out[1]) a.out[1][idx] = double(iu[0]);
            if (a.out[2]) a.out[2][idx] = double(iu[1]);
            // the D3Q15 ForceConvection adjoint never stores iuz (adjointadvection.h:1074-1084)
            if (L::ND == 3 && K != K_AAD_FORCE && a.out[3]) a.out[3][idx] = double(iu[2]);
            if (a.out[4]) a.out[4][idx] = double(im[0]);
            if (a.out[5]) a.out[5][idx] = double(im[1]);
            if (L::ND == 3 && a.out[6]) a.out[6][idx] = double(im[2]);
            if (kind_has_g(K)) {
                if (a.out[7]) a.out[7][idx] = double(item);
                if (a.out[8]) a.out[8][idx] = double(iq[0]);
                if (a.out[9]) a.out[9][idx] = double(iq[1]);
                if (L::ND == 3 && a.out[10]) a.out[10][idx] = double(iq[2]);
            }
        }
        if (snap && kind_has_snapshot(K)) {
#pragma unroll
            for (int c = 0; c < Q; ++c) snap[c * np + idx] = double(g[c]);
        }
        const T iomf = T(1) - omf;
#pragma unroll
        for (int c = 0; c < Q; ++c) f[c] = iomf * f[c] + omf * ans_feq<L, T>(c, u, ip, iu);
        if (kind_has_g(K)) {
            const T geq = item + T(3) * vdot<L, T>(u, iq);
            const T iomg = T(1) - omg;
#pragma unroll
            for (int c = 0; c < Q; ++c) g[c] = iomg * g[c] + omg * geq;
        }
    }
}

}  // namespace pl
