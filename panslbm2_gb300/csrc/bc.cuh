// bc.cuh -- boundary-program ops applied to one node's populations (device code).
//
// Each op is one reference boundary routine restricted to one node of its edge/face:
//   walls        D2Q9/D3Q15::(i)BoundaryConditionAlong* (d2q9.h:429-575, d3q15.h:982-1239)
//   NS Zou-He    NS::BoundaryConditionSetU/SetRhoAlong* (navierstokes.h:90-426)
//   AD           AD::BoundaryConditionSetT/SetQAlong* (advection.h:97-524)
//   ANS adjoint  ANS::iBoundaryConditionSetU/SetRhoAlong* (adjointnavierstokes.h:95-392)
//   AAD adjoint  AAD::iBoundaryConditionSetT/SetQ/SetRhoAlong* (adjointadvection.h:152-751)
//   incompressible (D2Q9) NSin::BoundaryConditionSetU/SetRhoAlong* (nsincompressible.h:46-140),
//                ANSin::iBoundaryConditionSetUAlong* (adjointnsincompressible.h:49-92)
// The face of an op is (axis a, side d); "inward" populations have c_a == -d.
#pragma once
#include "physics.cuh"

namespace pl {

template <class L> __device__ __forceinline__ int cmp(int c, int a) { return comp<L>(c, a); }

template <class L> __device__ __forceinline__ bool diag_of(int c, int a) {
    bool r = false;
#pragma unroll
    for (int e = 0; e < L::ND; ++e) if (e != a && cmp<L>(c, e) != 0) r = true;
    return r;
}
template <class L> __device__ __forceinline__ int opp_d(int c) { return opp<L>(c); }
template <class L> __device__ __forceinline__ int refl_d(int c, int a) {
    return a == 0 ? refl<L>(c, 0) : (a == 1 ? refl<L>(c, 1) : refl<L>(c, 2));
}

template <class L, class T> __device__ __forceinline__ T one_plus_3cu(int c, const T *u) {
    T acc = T(1);
#pragma unroll
    for (int b = 0; b < L::ND; ++b) {
        const int cb = cmp<L>(c, b);
        if (cb > 0) acc += T(3) * u[b]; else if (cb < 0) acc -= T(3) * u[b];
    }
    return acc;
}
template <class L, class T> __device__ __forceinline__ T inv_w(int c) {
    int s = 0;
#pragma unroll
    for (int b = 0; b < L::ND; ++b) s += abs(cmp<L>(c, b));
    return s == 1 ? T(9) : (L::ND == 2 ? T(36) : T(72));
}
// sum over inward diagonals of sign(c_b) p_c, increasing c
template <class L, class T> __device__ __forceinline__ T tsum(const T *p, int a, int d, int b) {
    T s = T(0);
#pragma unroll
    for (int c = 1; c < L::Q; ++c) {
        if (cmp<L>(c, a) != -d || !diag_of<L>(c, a)) continue;
        const int cb = cmp<L>(c, b);
        if (cb > 0) s += p[c]; else if (cb < 0) s -= p[c];
    }
    return s;
}
// kc * p_normal + sum of inward diagonals
template <class L, class T> __device__ __forceinline__ T nsum(const T *p, int a, int d, T kc) {
    T s = T(0);
#pragma unroll
    for (int c = 1; c < L::Q; ++c)
        if (cmp<L>(c, a) == -d && !diag_of<L>(c, a)) s = kc * p[c];
#pragma unroll
    for (int c = 1; c < L::Q; ++c)
        if (cmp<L>(c, a) == -d && diag_of<L>(c, a)) s += p[c];
    return s;
}
__device__ __forceinline__ void tang3(int a, int &t0, int &t1) {
    t0 = a == 0 ? 1 : (a == 1 ? 2 : 0);
    t1 = a == 0 ? 2 : (a == 1 ? 0 : 1);
}

// NS::BoundaryConditionSetU / SetRho on face (A, D) (navierstokes.h:90-426). setu: val = the
// velocity (inflow scale applied); else val[0] = rho and val[1], val[2] the tangential velocity.
// A and D are compile-time constants: the interior kernel calls this for its face nodes and
// apply_op dispatches to it over the six faces, so both paths run the same arithmetic.
template <class L, class T, int A, int D>
__device__ __forceinline__ void ns_face_ud(bool setu, const T *val, T *p) {
    constexpr int Q = L::Q, ND = L::ND;
    T u[3] = {T(0), T(0), T(0)};
    T sT = T(0), sO = T(0);
    bool first = true;
#pragma unroll
    for (int c = 0; c < Q; ++c)
        if (cmp<L>(c, A) == 0) { if (first) { sT = p[c]; first = false; } else sT += p[c]; }
    first = true;
#pragma unroll
    for (int c = 0; c < Q; ++c)
        if (cmp<L>(c, A) == D) { if (first) { sO = p[c]; first = false; } else sO += p[c]; }
    const T S = sT + T(2) * sO;
    T rho0;
    if (setu) {
        u[0] = val[0]; u[1] = val[1]; if (ND == 3) u[2] = val[2];
        rho0 = S / (D < 0 ? T(1) - u[A] : T(1) + u[A]);
    } else {
        rho0 = val[0];
        if (ND == 2) u[1 - A] = val[1];
        else { u[(A + 1) % 3] = val[1]; u[(A + 2) % 3] = val[2]; }
        u[A] = D < 0 ? T(1) - S / rho0 : T(-1) + S / rho0;
    }
    const T kn = ND == 2 ? T(6) : T(12), kt = ND == 2 ? T(0.5) : T(0.25), kc = ND == 2 ? T(4) : T(8);
    T m[3];
#pragma unroll
    for (int b = 0; b < ND; ++b) {
        if (b == A) m[b] = rho0 * u[b] / kn;
        else {
            T fp = T(0), fm = T(0);
#pragma unroll
            for (int c = 1; c < Q; ++c) {
                if (diag_of<L>(c, b)) continue;
                if (cmp<L>(c, b) == 1) fp = p[c];
                if (cmp<L>(c, b) == -1) fm = p[c];
            }
            m[b] = kt * (fp - fm - rho0 * u[b]);
        }
    }
    T src[Q];
#pragma unroll
    for (int c = 0; c < Q; ++c) src[c] = p[c];
#pragma unroll
    for (int c = 1; c < Q; ++c) {
        if (cmp<L>(c, A) != -D) continue;
        T v = src[opp_d<L>(c)];
        if (!diag_of<L>(c, A)) {
            v = cmp<L>(c, A) > 0 ? v + kc * m[A] : v - kc * m[A];
        } else {
#pragma unroll
            for (int b = 0; b < ND; ++b) {
                const int cb = cmp<L>(c, b);
                if (b == A) v = cb > 0 ? v + m[b] : v - m[b];
                else v = cb > 0 ? v - m[b] : v + m[b];
            }
        }
        p[c] = v;
    }
}

// ANS::iBoundaryConditionSetU / SetRho on face (A, D) (adjointnavierstokes.h:95-392); u the
// velocity (inflow scale applied), eps the objective weight of the edge
template <class L, class T, int A, int D>
__device__ __forceinline__ void ans_face_ud(bool setu, T eps, const T *u, T *p) {
    constexpr int Q = L::Q, ND = L::ND;
    T rho0;
    if (!setu) {
        rho0 = nsum<L, T>(p, A, D, ND == 2 ? T(4) : T(8)) / (ND == 2 ? T(3) : T(6));
        T src[Q];
#pragma unroll
        for (int c = 0; c < Q; ++c) src[c] = p[c];
#pragma unroll
        for (int c = 1; c < Q; ++c) if (cmp<L>(c, A) == D) p[c] = src[opp_d<L>(c)] - rho0;
        return;
    }
    if (ND == 2) {
        const T un = u[0], ut = A == 0 ? u[1] : u[0];   // y edges use ux twice (reference)
        constexpr int B = 1 - A;
        const T ns = nsum<L, T>(p, A, D, T(4));
        const T ts = tsum<L, T>(p, A, D, B);
        T num = D < 0 ? T(-2) * eps + un * ns : T(-2) * eps - un * ns;
        num += T(3) * ut * ts;
        rho0 = num / (T(3) * (D < 0 ? T(1) - un : T(1) + un));
    } else {
        T num = T(-4) * eps;
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            if (b == A) {
                const T ns = nsum<L, T>(p, A, D, T(8));
                num = D < 0 ? num + u[A] * ns : num - u[A] * ns;
            } else {
                num += T(3) * u[b] * tsum<L, T>(p, A, D, b);
            }
        }
        rho0 = num / (T(6) * (D < 0 ? T(1) - u[A] : T(1) + u[A]));
    }
    T src[Q];
#pragma unroll
    for (int c = 0; c < Q; ++c) src[c] = p[c];
#pragma unroll
    for (int c = 1; c < Q; ++c) if (cmp<L>(c, A) == D) p[c] = src[opp_d<L>(c)] + rho0;
}

// runtime face -> the face-templated NS / ANS routine
template <class L, class T>
__device__ __forceinline__ void ns_ud(int A, int d, bool setu, const T *val, T *p) {
    switch (A * 2 + (d > 0 ? 1 : 0)) {
    case 0: ns_face_ud<L, T, 0, -1>(setu, val, p); break;
    case 1: ns_face_ud<L, T, 0, 1>(setu, val, p); break;
    case 2: ns_face_ud<L, T, 1, -1>(setu, val, p); break;
    case 3: ns_face_ud<L, T, 1, 1>(setu, val, p); break;
    case 4: if (L::ND == 3) ns_face_ud<L, T, 2, -1>(setu, val, p); break;
    case 5: if (L::ND == 3) ns_face_ud<L, T, 2, 1>(setu, val, p); break;
    default: break;
    }
}
template <class L, class T>
__device__ __forceinline__ void ans_ud(int A, int d, bool setu, T eps, const T *u, T *p) {
    switch (A * 2 + (d > 0 ? 1 : 0)) {
    case 0: ans_face_ud<L, T, 0, -1>(setu, eps, u, p); break;
    case 1: ans_face_ud<L, T, 0, 1>(setu, eps, u, p); break;
    case 2: ans_face_ud<L, T, 1, -1>(setu, eps, u, p); break;
    case 3: ans_face_ud<L, T, 1, 1>(setu, eps, u, p); break;
    case 4: if (L::ND == 3) ans_face_ud<L, T, 2, -1>(setu, eps, u, p); break;
    case 5: if (L::ND == 3) ans_face_ud<L, T, 2, 1>(setu, eps, u, p); break;
    default: break;
    }
}

// wall copy on one population set; every array index is a compile-time constant after
// unrolling (the runtime axis only selects among constants), so the set stays in registers
template <class L, class T>
__device__ __forceinline__ void wall_set(T *p, int A, int d, bool adj, int type) {
    constexpr int Q = L::Q;
    T src[Q];
#pragma unroll
    for (int c = 0; c < Q; ++c) src[c] = p[c];
#pragma unroll
    for (int c = 1; c < Q; ++c) {
        const int ca = A == 0 ? L::cx(c) : (A == 1 ? L::cy(c) : L::cz(c));
        if (adj ? (ca != d) : (ca != -d)) continue;
        const T r = A == 0 ? src[refl<L>(c, 0)] : (A == 1 ? src[refl<L>(c, 1)] : src[refl<L>(c, 2)]);
        p[c] = type == 1 ? src[opp<L>(c)] : r;
    }
}

template <class L, class T, bool SIMPLE = false>
__device__ __forceinline__ void apply_op(const Op &op, T *f, T *g, int node, const KArgs &a,
                                         const T *upre = nullptr, T kpre = T(0)) {
    const int A = op.axis, d = op.dir, nin = -d;
    constexpr int Q = L::Q, ND = L::ND;
    if (SIMPLE && !op_is_simple(op.kind)) return;
    switch (op.kind) {
    case BC_WALL:
    case BC_IWALL: {
        const bool adj = op.kind == BC_IWALL;
        if (op.lat) wall_set<L, T>(g, A, d, adj, op.sub);
        else wall_set<L, T>(f, A, d, adj, op.sub);
        break;
    }
    case BC_NS_U:
    case BC_NS_RHO: if constexpr (!SIMPLE) {
        T val[3];
        if (op.kind == BC_NS_U) {
            // uscale: time-varying inflow u(t) = uscale * u (1 = the reference routine)
            val[0] = T(a.uscale * op.v0); val[1] = T(a.uscale * op.v1); val[2] = ND == 3 ? T(a.uscale * op.v2) : T(0);
        } else {
            val[0] = T(op.v0); val[1] = T(op.v1); val[2] = ND == 3 ? T(op.v2) : T(0);
        }
        ns_ud<L, T>(A, d, op.kind == BC_NS_U, val, f);
    } break;
    case BC_AD_T:
    case BC_AD_Q:
    case BC_AD_QC: {
        T *p = g;
        T u[3];
        if (upre) { u[0] = upre[0]; u[1] = upre[1]; u[2] = upre[2]; }
        else { u[0] = T(a.bcu[0][node]); u[1] = T(a.bcu[1][node]); u[2] = ND == 3 ? T(a.bcu[2][node]) : T(0); }
        T tem0;
        if (op.kind == BC_AD_T) {
            T s = T(op.v0);
#pragma unroll
            for (int c = 0; c < Q; ++c) if (cmp<L>(c, A) != -d) s -= p[c];
            tem0 = T(6) * s / (nin > 0 ? T(1) + T(3) * u[A] : T(1) - T(3) * u[A]);
        } else {
            const T kap = op.kind == BC_AD_Q ? (upre ? kpre : T(a.bckappa[node])) : T(op.v1);
            T s = (T(1) + T(1) / (T(6) * kap)) * T(op.v0);
#pragma unroll
            for (int c = 1; c < Q; ++c) if (cmp<L>(c, A) == d) s += p[c];
            tem0 = T(6) * s / (nin > 0 ? T(1) - T(3) * u[A] : T(1) + T(3) * u[A]);
        }
#pragma unroll
        for (int c = 1; c < Q; ++c)
            if (cmp<L>(c, A) == -d) p[c] = tem0 * one_plus_3cu<L, T>(c, u) / inv_w<L, T>(c);
        break;
    }
    case BC_ANS_U:
    case BC_ANS_RHO: if constexpr (!SIMPLE) {
        const T u[3] = {T(a.uscale * op.v0), T(a.uscale * op.v1), ND == 3 ? T(a.uscale * op.v2) : T(0)};
        ans_ud<L, T>(A, d, op.kind == BC_ANS_U, T(op.eps), u, f);
    } break;
    case BC_AAD_T:
    case BC_AAD_Q: {
        T *p = g;
        T u[3];
        if (upre) { u[0] = upre[0]; u[1] = upre[1]; u[2] = upre[2]; }
        else { u[0] = T(a.bcu[0][node]); u[1] = T(a.bcu[1][node]); u[2] = ND == 3 ? T(a.bcu[2][node]) : T(0); }
        const T pre = nin > 0 ? T(1) + T(3) * u[A] : T(1) - T(3) * u[A];
        const T post = nin > 0 ? T(1) - T(3) * u[A] : T(1) + T(3) * u[A];
        T rho0;
        if (op.kind == BC_AAD_T) {
            if (ND == 2) {
                T num = T(0);
#pragma unroll
                for (int c = 1; c < Q; ++c)
                    if (cmp<L>(c, A) == -d && !diag_of<L>(c, A)) num = T(4) * one_plus_3cu<L, T>(c, u) * p[c];
#pragma unroll
                for (int c = 1; c < Q; ++c)
                    if (cmp<L>(c, A) == -d && diag_of<L>(c, A)) num += one_plus_3cu<L, T>(c, u) * p[c];
                rho0 = -num / (T(6) * pre);
            } else {
                int t0, t1;
                tang3(A, t0, t1);
                rho0 = -nsum<L, T>(p, A, d, T(8)) / T(12) - u[t0] * tsum<L, T>(p, A, d, t0) / (T(4) * pre)
                       - u[t1] * tsum<L, T>(p, A, d, t1) / (T(4) * pre);
            }
        } else {
            if (ND == 2) {
                const int b = 1 - A;
                const T num = pre * nsum<L, T>(p, A, d, T(4)) + T(3) * u[b] * tsum<L, T>(p, A, d, b) - T(12) * T(op.eps);
                rho0 = num / (T(6) * post);
            } else {
                int t0, t1;
                tang3(A, t0, t1);
                const bool k3 = (A == 0 || (A == 1 && d < 0));   // reference factor pattern
                T num = pre * nsum<L, T>(p, A, d, T(8));
                if (k3) {
                    num += T(3) * u[t0] * tsum<L, T>(p, A, d, t0);
                    num += T(3) * u[t1] * tsum<L, T>(p, A, d, t1);
                } else {
                    num += u[t0] * tsum<L, T>(p, A, d, t0);
                    num += u[t1] * tsum<L, T>(p, A, d, t1);
                }
                num -= T(24) * T(op.eps);
                rho0 = num / (T(12) * post);
            }
        }
#pragma unroll
        for (int c = 1; c < Q; ++c) if (cmp<L>(c, A) == d) p[c] = rho0;
        break;
    }
    case BC_AAD_RHO: if constexpr (!SIMPLE) {
        const T u[3] = {T(a.bcu[0][node]), T(a.bcu[1][node]), ND == 3 ? T(a.bcu[2][node]) : T(0)};
        const T rho = T(a.bcrho[node]), tem = T(a.bctem[node]);
        const T pre = nin > 0 ? T(1) + T(3) * u[A] : T(1) - T(3) * u[A];
        const T post = nin > 0 ? T(1) - T(3) * u[A] : T(1) + T(3) * u[A];
        T r0, flux0 = T(0);
        const int type = op.sub;
        if (ND == 2) {
            const int b = 1 - A;
            r0 = -nsum<L, T>(f, A, d, T(4)) / T(3);
            if (type == 1) flux0 = tem * u[b] * tsum<L, T>(g, A, d, b) / (T(2) * pre * rho);
            else if (type == 2)
                flux0 = -tem * (nsum<L, T>(g, A, d, T(4)) / T(3) + u[b] * tsum<L, T>(g, A, d, b) / T(2)) / (post * rho);
        } else {
            int t0, t1;
            tang3(A, t0, t1);
            r0 = -nsum<L, T>(f, A, d, T(8)) / T(6);
            const T tt = u[t0] * tsum<L, T>(g, A, d, t0) / T(4) + u[t1] * tsum<L, T>(g, A, d, t1) / T(4);
            if (type == 1) flux0 = tem * tt / (rho * pre);
            else if (type == 2)
                flux0 = -tem * (nsum<L, T>(g, A, d, T(8)) / T(6) + u[t0] * tsum<L, T>(g, A, d, t0) / T(4)
                                + u[t1] * tsum<L, T>(g, A, d, t1) / T(4)) / (rho * post);
        }
        const T obj0 = T(op.eps) * T(2) * tem / (post * rho);
        T src[Q];
#pragma unroll
        for (int c = 0; c < Q; ++c) src[c] = f[c];
#pragma unroll
        for (int c = 1; c < Q; ++c) if (cmp<L>(c, A) == d) f[c] = src[opp_d<L>(c)] + r0 + flux0 + obj0;
        break;
    } break;
    case BC_NSIN_U:
    case BC_NSIN_RHO:
    case BC_ANSIN_U: if constexpr (!SIMPLE && ND == 2) {
        // NSin::BoundaryConditionSetU/SetRhoAlong{X,Y}Edge (nsincompressible.h:46-140),
        // ANSin::iBoundaryConditionSetUAlong{X,Y}Edge (adjointnsincompressible.h:49-92)
        T *p = f;
        T src[Q];
#pragma unroll
        for (int c = 0; c < Q; ++c) src[c] = p[c];
        if (op.kind == BC_ANSIN_U) {
            const T de = T(2) * T(op.eps) / T(3);
#pragma unroll
            for (int c = 1; c < Q; ++c) if (cmp<L>(c, A) == d) p[c] = src[opp_d<L>(c)] - de;
            break;
        }
        const int b = 1 - A;
        T ftp = T(0), ftm = T(0);
#pragma unroll
        for (int c = 1; c < Q; ++c) {
            if (cmp<L>(c, A) != 0) continue;
            if (cmp<L>(c, b) == 1) ftp = src[c];
            if (cmp<L>(c, b) == -1) ftm = src[c];
        }
        T un, ut;
        if (op.kind == BC_NSIN_U) {
            un = A == 0 ? T(op.v0) : T(op.v1);
            ut = A == 0 ? T(op.v1) : T(op.v0);
        } else {
            const T rho = T(op.v0);
            ut = T(op.v1);
            T so = T(0);
            bool first = true;
#pragma unroll
            for (int c = 1; c < Q; ++c)
                if (cmp<L>(c, A) == d) { if (first) { so = src[c]; first = false; } else so += src[c]; }
            const T S = src[0] + ftp + ftm + T(2) * so;
            un = d < 0 ? rho - S : -rho + S;
        }
        const T X = ftp - ftm - ut;
#pragma unroll
        for (int c = 1; c < Q; ++c) {
            if (cmp<L>(c, A) != -d) continue;
            T v = src[opp_d<L>(c)];
            if (cmp<L>(c, b) == 0) {
                p[c] = d < 0 ? v + T(2) * un / T(3) : v - T(2) * un / T(3);
            } else {
                v = d < 0 ? v + un / T(6) : v - un / T(6);
                p[c] = cmp<L>(c, b) > 0 ? v - T(0.5) * X : v + T(0.5) * X;
            }
        }
        break;
    } break;
    case BC_EL_STRESS:
    case BC_AEL_STRESS: if constexpr (!SIMPLE && ND == 2 && Q == 9) {
        // EL::BoundaryConditionSetStressAlong{X,Y}Edge (elastic.h:60-104): the three incoming
        // populations from the node's known ones and the traction (tx, ty);
        // AEL::iBoundaryConditionSetStressAlong{X,Y}Edge (adjointelastic.h:48-92): the three
        // outgoing adjoint populations, traction over the node's density (v2). D2Q9 indices.
        T *p = f;
        const T tx = T(op.v0), ty = T(op.v1);
        if (op.kind == BC_EL_STRESS) {
            if (A == 0 && d < 0) {
                const T s = p[3] + p[6] + p[7];
                p[1] = p[3] - T(4) * s / T(3) + T(2) * tx / T(3);
                p[5] = p[6] - s / T(3) + (tx + T(3) * ty) / T(6);
                p[8] = p[7] - s / T(3) + (tx - T(3) * ty) / T(6);
            } else if (A == 0) {
                const T s = p[1] + p[5] + p[8];
                p[3] = p[1] - T(4) * s / T(3) - T(2) * tx / T(3);
                p[6] = p[5] - s / T(3) - (tx - T(3) * ty) / T(6);
                p[7] = p[8] - s / T(3) - (tx + T(3) * ty) / T(6);
            } else if (d < 0) {
                const T s = p[4] + p[7] + p[8];
                p[2] = p[4] - T(4) * s / T(3) + T(2) * ty / T(3);
                p[5] = p[8] - s / T(3) + (ty + T(3) * tx) / T(6);
                p[6] = p[7] - s / T(3) + (ty - T(3) * tx) / T(6);
            } else {
                const T s = p[2] + p[5] + p[6];
                p[4] = p[2] - T(4) * s / T(3) - T(2) * ty / T(3);
                p[7] = p[6] - s / T(3) - (ty + T(3) * tx) / T(6);
                p[8] = p[5] - s / T(3) - (ty - T(3) * tx) / T(6);
            }
        } else {
            const T rho = T(op.v2);
            if (A == 0 && d < 0) {
                const T s = (T(4) * p[1] + p[5] + p[8]) / T(3);
                p[3] = p[1] - s + T(2) * tx / rho;
                p[6] = p[5] - s + T(2) * (tx - ty) / rho;
                p[7] = p[8] - s + T(2) * (tx + ty) / rho;
            } else if (A == 0) {
                const T s = (T(4) * p[3] + p[6] + p[7]) / T(3);
                p[1] = p[3] - s - T(2) * tx / rho;
                p[5] = p[6] - s - T(2) * (tx + ty) / rho;
                p[8] = p[7] - s - T(2) * (tx - ty) / rho;
            } else if (d < 0) {
                const T s = (T(4) * p[2] + p[5] + p[6]) / T(3);
                p[4] = p[2] - s + T(2) * ty / rho;
                p[7] = p[6] - s + T(2) * (ty + tx) / rho;
                p[8] = p[5] - s + T(2) * (ty - tx) / rho;
            } else {
                const T s = (T(4) * p[4] + p[7] + p[8]) / T(3);
                p[2] = p[4] - s - T(2) * ty / rho;
                p[5] = p[8] - s - T(2) * (ty + tx) / rho;
                p[6] = p[7] - s - T(2) * (ty - tx) / rho;
            }
        }
        break;
    } break;
    default:
        break;
    }
}

// out-of-line copy for the recursive replay path (keeps code size bounded)
template <class L, class T>
__device__ __noinline__ void apply_op_ni(const Op &op, T *f, T *g, int node, const KArgs &a) {
    apply_op<L, T>(op, f, g, node, a);
}

// ---- simple ops specialised on the face (axis A, side D) ---------------------------------------
// Same arithmetic as apply_op; with A and D known at compile time every direction test folds,
// leaving straight-line code. Used by the interior kernel for boundary nodes.
// vals: the op's values (InlineRec::val); uscale the inflow scale of NS SetU / ANS iSetU.
template <class L, class T, int A, int D>
__device__ __forceinline__ void simple_face_op(int sk, int lat, int type, const double *vals, double uscale, T *f,
                                               T *g, const T *u, T kp) {
    constexpr int Q = L::Q, ND = L::ND, NIN = -D;
    const T v0 = T(vals[0]), v1 = T(vals[1]);
    switch (sk) {
    case 0:   // BC_WALL
    case 1: { // BC_IWALL
        T *p = lat ? g : f;
        T src[Q];
#pragma unroll
        for (int c = 0; c < Q; ++c) src[c] = p[c];
        if (sk == 0) {
#pragma unroll
            for (int c = 1; c < Q; ++c)
                if (comp<L>(c, A) == -D) p[c] = type == 1 ? src[opp<L>(c)] : src[refl<L>(c, A)];
        } else {
#pragma unroll
            for (int c = 1; c < Q; ++c)
                if (comp<L>(c, A) == D) p[c] = type == 1 ? src[opp<L>(c)] : src[refl<L>(c, A)];
        }
        break;
    }
    case 2:   // BC_AD_T
    case 3:   // BC_AD_Q
    case 4: { // BC_AD_QC
        T tem0;
        if (sk == 2) {
            T s = v0;
#pragma unroll
            for (int c = 0; c < Q; ++c) if (comp<L>(c, A) != -D) s -= g[c];
            tem0 = T(6) * s / (NIN > 0 ? T(1) + T(3) * u[A] : T(1) - T(3) * u[A]);
        } else {
            const T kap = sk == 3 ? kp : v1;
            T s = (T(1) + T(1) / (T(6) * kap)) * v0;
#pragma unroll
            for (int c = 1; c < Q; ++c) if (comp<L>(c, A) == D) s += g[c];
            tem0 = T(6) * s / (NIN > 0 ? T(1) - T(3) * u[A] : T(1) + T(3) * u[A]);
        }
#pragma unroll
        for (int c = 1; c < Q; ++c)
            if (comp<L>(c, A) == -D) g[c] = tem0 * one_plus_3cu<L, T>(c, u) / inv_w<L, T>(c);
        break;
    }
    case 5:   // BC_AAD_T
    case 6: { // BC_AAD_Q
        const T pre = NIN > 0 ? T(1) + T(3) * u[A] : T(1) - T(3) * u[A];
        const T post = NIN > 0 ? T(1) - T(3) * u[A] : T(1) + T(3) * u[A];
        T rho0;
        if (sk == 5) {
            if (ND == 2) {
                T num = T(0);
#pragma unroll
                for (int c = 1; c < Q; ++c)
                    if (comp<L>(c, A) == -D && !diag_of<L>(c, A)) num = T(4) * one_plus_3cu<L, T>(c, u) * g[c];
#pragma unroll
                for (int c = 1; c < Q; ++c)
                    if (comp<L>(c, A) == -D && diag_of<L>(c, A)) num += one_plus_3cu<L, T>(c, u) * g[c];
                rho0 = -num / (T(6) * pre);
            } else {
                constexpr int T0 = A == 0 ? 1 : (A == 1 ? 2 : 0), T1 = A == 0 ? 2 : (A == 1 ? 0 : 1);
                rho0 = -nsum<L, T>(g, A, D, T(8)) / T(12) - u[T0] * tsum<L, T>(g, A, D, T0) / (T(4) * pre)
                       - u[T1] * tsum<L, T>(g, A, D, T1) / (T(4) * pre);
            }
        } else {
            if (ND == 2) {
                constexpr int B = 1 - A;
                const T num = pre * nsum<L, T>(g, A, D, T(4)) + T(3) * u[B] * tsum<L, T>(g, A, D, B) - T(12) * v0;
                rho0 = num / (T(6) * post);
            } else {
                constexpr int T0 = A == 0 ? 1 : (A == 1 ? 2 : 0), T1 = A == 0 ? 2 : (A == 1 ? 0 : 1);
                constexpr bool K3 = (A == 0 || (A == 1 && D < 0));
                T num = pre * nsum<L, T>(g, A, D, T(8));
                if (K3) {
                    num += T(3) * u[T0] * tsum<L, T>(g, A, D, T0);
                    num += T(3) * u[T1] * tsum<L, T>(g, A, D, T1);
                } else {
                    num += u[T0] * tsum<L, T>(g, A, D, T0);
                    num += u[T1] * tsum<L, T>(g, A, D, T1);
                }
                num -= T(24) * v0;
                rho0 = num / (T(12) * post);
            }
        }
#pragma unroll
        for (int c = 1; c < Q; ++c) if (comp<L>(c, A) == D) g[c] = rho0;
        break;
    }
    case 7:   // BC_NS_U
    case 8: { // BC_NS_RHO
        T val[3];
        if (sk == 7) { val[0] = T(uscale * vals[0]); val[1] = T(uscale * vals[1]); val[2] = ND == 3 ? T(uscale * vals[2]) : T(0); }
        else { val[0] = T(vals[0]); val[1] = T(vals[1]); val[2] = ND == 3 ? T(vals[2]) : T(0); }
        ns_face_ud<L, T, A, D>(sk == 7, val, f);
        break;
    }
    case 9:    // BC_ANS_U
    case 10: { // BC_ANS_RHO
        const T uu[3] = {T(uscale * vals[0]), T(uscale * vals[1]), ND == 3 ? T(uscale * vals[2]) : T(0)};
        ans_face_ud<L, T, A, D>(sk == 9, T(vals[3]), uu, f);
        break;
    }
    default:
        break;
    }
}

template <class L, class T>
__device__ __forceinline__ void simple_op(int axis, int dir, int sk, int lat, int type, const double *vals,
                                          double uscale, T *f, T *g, const T *u, T kp) {
    const int face = axis * 2 + (dir > 0 ? 1 : 0);
    switch (face) {
    case 0: simple_face_op<L, T, 0, -1>(sk, lat, type, vals, uscale, f, g, u, kp); break;
    case 1: simple_face_op<L, T, 0, 1>(sk, lat, type, vals, uscale, f, g, u, kp); break;
    case 2: simple_face_op<L, T, 1, -1>(sk, lat, type, vals, uscale, f, g, u, kp); break;
    case 3: simple_face_op<L, T, 1, 1>(sk, lat, type, vals, uscale, f, g, u, kp); break;
    case 4: if (L::ND == 3) simple_face_op<L, T, 2, -1>(sk, lat, type, vals, uscale, f, g, u, kp); break;
    case 5: if (L::ND == 3) simple_face_op<L, T, 2, 1>(sk, lat, type, vals, uscale, f, g, u, kp); break;
    default: break;
    }
}

}  // namespace pl
