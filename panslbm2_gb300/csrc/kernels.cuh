// kernels.cuh -- population kernels of the fused lattice-Boltzmann step.
//
// One time step of the reference loop is  collide -> Stream -> boundary routines -> smoothing
// (e.g. production/heatsink.cpp:142-174). Here the step is regrouped as
//     pull-stream + boundary program + collide      (one pass over HBM per step)
// split into an interior kernel (every node without boundary ops: pull, collide, store) and a
// boundary kernel (nodes with ops: pull, replay the recorded ops in call order -- recursing
// into neighbours for the averaging of SmoothCorner* -- then the same collide).
// Populations are structure-of-arrays: plane c of set s at  buf + (s*Q + c)*np.
#pragma once
#include "bc.cuh"

namespace pl {

constexpr int kBlock = 256;

template <class L> __device__ __forceinline__ void coords(const Geo &g, int idx, int &i, int &j, int &k) {
    i = idx % g.nx;
    const int r = idx / g.nx;
    if (L::ND == 2) { j = r; k = 0; }
    else { j = r % g.ny; k = r / g.ny; }
}
template <class L> __device__ __forceinline__ bool is_interior(const Geo &g, int i, int j, int k) {
    return i > 0 && i < g.nx - 1 && j > 0 && j < g.ny - 1 && (L::ND == 2 || (k > 0 && k < g.nz - 1));
}
template <class L> __device__ __forceinline__ bool skip_boundary(const Geo &g, int idx, int i, int j, int k) {
    if (g.flags) return g.flags[idx] != 0;
    const uint32_t m = g.face_mask;
    return ((m & 1u) && i == 0) || ((m & 2u) && i == g.nx - 1) || ((m & 4u) && j == 0) ||
           ((m & 8u) && j == g.ny - 1) || (L::ND == 3 && (((m & 16u) && k == 0) || ((m & 32u) && k == g.nz - 1)));
}
__device__ __forceinline__ int wrap1(int i, int n) { return i < 0 ? n - 1 : (i >= n ? 0 : i); }

// Load one node's populations from `src`, pulled along direction sgn*c (sgn = -1: Stream,
// +1: iStream) when `pull`, else in place. Periodic single-step wrap (d2q9.h:80-84).
template <class L, class S, bool HAS_G>
__device__ __forceinline__ void load_node(const S *__restrict__ src, const Geo &g, int idx, int i, int j, int k,
                                          bool pull, int sgn, bool interior, typename Store<S>::T *f,
                                          typename Store<S>::T *gg, typename Store<S>::T sf,
                                          typename Store<S>::T sg) {
    using T = typename Store<S>::T;
    constexpr int Q = L::Q;
    const long long np = g.np;
#pragma unroll
    for (int c = 0; c < Q; ++c) {
        int s = idx;
        if (pull && c > 0) {
            const int dx = sgn * L::cx(c), dy = sgn * L::cy(c), dz = sgn * L::cz(c);
            if (interior) s = idx + dx + g.nx * (dy + g.ny * dz);
            else s = wrap1(i + dx, g.nx) + g.nx * (wrap1(j + dy, g.ny) + g.ny * (L::ND == 3 ? wrap1(k + dz, g.nz) : 0));
        }
        f[c] = Store<S>::dec(Store<S>::ld(src + (long long)c * np + s), L::template w<T>(c) * sf);
        if (HAS_G) gg[c] = Store<S>::dec(Store<S>::ld(src + (long long)(Q + c) * np + s), L::template w<T>(c) * sg);
    }
}
template <class L, class S, bool HAS_G>
__device__ __forceinline__ void store_node(S *__restrict__ dst, const Geo &g, int idx, const typename Store<S>::T *f,
                                           const typename Store<S>::T *gg, typename Store<S>::T sf,
                                           typename Store<S>::T sg) {
    using T = typename Store<S>::T;
    constexpr int Q = L::Q;
#pragma unroll
    for (int c = 0; c < Q; ++c) {
        Store<S>::st(dst + (long long)c * g.np + idx, Store<S>::enc(f[c], L::template w<T>(c) * sf));
        if (HAS_G) Store<S>::st(dst + (long long)(Q + c) * g.np + idx, Store<S>::enc(gg[c], L::template w<T>(c) * sg));
    }
}

// the collide's store with stochastic rounding for 16-bit storage when a.sr is set
template <class L, class S, bool HAS_G>
__device__ __forceinline__ void store_collided(const KArgs &a, int idx, const typename Store<S>::T *f,
                                               const typename Store<S>::T *gg, typename Store<S>::T sf,
                                               typename Store<S>::T sg) {
    using T = typename Store<S>::T;
    constexpr bool SIXTEEN = sizeof(S) == 2;
    if (!SIXTEEN || !a.sr) {
        store_node<L, S, HAS_G>(static_cast<S *>(a.dst), a.geo, idx, f, gg, sf, sg);
        return;
    }
    constexpr int Q = L::Q;
    S *dst = static_cast<S *>(a.dst);
    uint32_t st = sr_hash(uint32_t(idx), a.sr_seed);
#pragma unroll
    for (int c = 0; c < Q; ++c) {
        const uint32_t r = sr_next(st);
        dst[(long long)c * a.geo.np + idx] = StoreSR<S>::enc(f[c], L::template w<T>(c) * sf, r);
        if (HAS_G) dst[(long long)(Q + c) * a.geo.np + idx] = StoreSR<S>::enc(gg[c], L::template w<T>(c) * sg, r >> 16);
    }
}

// ---- interior kernel --------------------------------------------------------------------
// PULL: stream + boundary program (fused step); otherwise collide in place. With a staged
// boundary program (a.icode), nodes on a face or flagged carry a code: -2 = handled by the
// side path (smoothing targets, ops this kind does not apply inline), >= 0 = simple ops applied
// here, after the pull, in call order (kinds with kind_inline_bc only). Without one, the
// face mask / flags select the nodes the recursive boundary kernel handles.
template <class L> __device__ __forceinline__ bool on_face(const Geo &g, int i, int j, int k) {
    return i == 0 || i == g.nx - 1 || j == 0 || j == g.ny - 1 || (L::ND == 3 && (k == 0 || k == g.nz - 1));
}
// After the pull: the node's inline boundary ops, the collide, the boundary velocity the next
// step's ops read, and the store. Only the op application diverges; every lane of a warp
// shares the collide.
// the node's inline boundary ops (InlineRec `code`), in call order
template <class L, class T>
__device__ __forceinline__ void inline_ops(const KArgs &a, int idx, int code, T *f, T *g) {
    const InlineRec &rec = a.irec[code];
    T up[3] = {T(0), T(0), T(0)}, kp = T(0);
    if (a.bcu[0]) { up[0] = T(a.bcu[0][idx]); up[1] = T(a.bcu[1][idx]); if (L::ND == 3) up[2] = T(a.bcu[2][idx]); }
    if (a.bckappa) kp = T(a.bckappa[idx]);
    const uint64_t code16 = rec.code;
    const uint32_t nops = rec.nops;
    for (int m = 0; m < (int)nops; ++m) {
        const uint32_t b = uint32_t(code16 >> (16 * m)) & 0xffffu;
        simple_op<L, T>(int((b >> 4) & 3u), (b & 64u) ? 1 : -1, int(b & 15u), (b & 128u) ? 1 : 0,
                        (b & 256u) ? 2 : 1, rec.val[m], a.uscale, f, g, up, kp);
    }
}

template <class L, class S, int K>
__device__ __forceinline__ void node_tail(const KArgs &a, int idx, int code, typename Store<S>::T *f,
                                          typename Store<S>::T *g, typename Store<S>::T sf,
                                          typename Store<S>::T sg) {
    using T = typename Store<S>::T;
    constexpr bool HG = kind_has_g(K);
    constexpr bool INL = kind_inline_bc(K);
    if constexpr (INL) {
        if (code >= 0) inline_ops<L, T>(a, idx, code, f, g);
    }
    T u[3];
    collide_node<L, T, K>(f, g, idx, a, a.save != 0, a.snap_coll, a.geo.np, (INL && !kind_is_adjoint(K)) ? u : nullptr);
    if constexpr (INL && !kind_is_adjoint(K)) {
        if (code >= 0 && a.bcu_out[0]) {
            a.bcu_out[0][idx] = double(u[0]);
            a.bcu_out[1][idx] = double(u[1]);
            if (L::ND == 3) a.bcu_out[2][idx] = double(u[2]);
        }
    }
    store_collided<L, S, HG>(a, idx, f, g, sf, sg);
}

// Launched on a (ceil(nx/32), ceil(ny/8), nz) grid of 32 x 8 blocks: lane = x within a 32-node
// tile (128-byte aligned accesses), warp = row; coordinates come from the block and thread
// indices. (Moving the x-face nodes into warps of their own was measured slower: it splits the
// 32-byte sectors at x = 0 and x = nx - 1 between two warps' stores.)
template <class L, class S, int K, bool PULL>
__global__ void __launch_bounds__(kBlock, 4) k_interior(KArgs a) {
    using T = typename Store<S>::T;
    constexpr bool HG = kind_has_g(K);
    constexpr bool INL = kind_inline_bc(K);
    const int nx = a.geo.nx;
    const int i = blockIdx.x * 32 + threadIdx.x, j = blockIdx.y * 8 + threadIdx.y;
    if (i >= nx || j >= a.geo.ny) return;
    const int k = blockIdx.z;
    const int idx = i + nx * (j + a.geo.ny * k);
    int code = -1;
    if (PULL) {
        if (a.icode) {
            const bool cand = a.geo.flags ? a.geo.flags[idx] != 0 : on_face<L>(a.geo, i, j, k);
            if (cand) code = a.icode[idx];
            if (code == -2 || (!INL && code >= 0)) return;
        } else if (skip_boundary<L>(a.geo, idx, i, j, k)) {
            return;
        }
    }
    T f[L::Q], g[L::Q];
    const T sf = T(a.ph.shift_f), sg = T(a.ph.shift_g);
    load_node<L, S, HG>(static_cast<const S *>(a.src), a.geo, idx, i, j, k, PULL, kind_is_adjoint(K) ? 1 : -1,
                        is_interior<L>(a.geo, i, j, k), f, g, sf, sg);
    node_tail<L, S, K>(a, idx, PULL ? code : -1, f, g, sf, sg);
}

// Stream + boundary program without collide over a staged program (both population sets):
// the same split as the fused step -- this kernel pulls every node the side kernels do not
// own and applies its inline ops; the direct and staged-smoothing nodes are stored by
// k_bnd_direct_stream / k_bnd_post_stream. Same grid as k_interior.
template <class L, class S>
__global__ void __launch_bounds__(kBlock, 4) k_interior_stream(KArgs a, int sgn) {
    using T = typename Store<S>::T;
    const int nx = a.geo.nx;
    const int i = blockIdx.x * 32 + threadIdx.x, j = blockIdx.y * 8 + threadIdx.y;
    if (i >= nx || j >= a.geo.ny) return;
    const int k = blockIdx.z;
    const int idx = i + nx * (j + a.geo.ny * k);
    int code = -1;
    const bool cand = a.geo.flags ? a.geo.flags[idx] != 0 : on_face<L>(a.geo, i, j, k);
    if (cand) code = a.icode[idx];
    if (code == -2) return;
    T f[L::Q], g[L::Q];
    const T sf = T(a.ph.shift_f), sg = T(a.ph.shift_g);
    load_node<L, S, true>(static_cast<const S *>(a.src), a.geo, idx, i, j, k, true, sgn, is_interior<L>(a.geo, i, j, k),
                          f, g, sf, sg);
    if (code >= 0) inline_ops<L, T>(a, idx, code, f, g);
    store_node<L, S, true>(static_cast<S *>(a.dst), a.geo, idx, f, g, sf, sg);
}

// ---- boundary program replay ----------------------------------------------------------------
// State of `node` after every op recorded before `seq_limit` (the reference applies edge
// routines in call order; SmoothCorner* reads neighbours as they stand at that point).
// the pull of eval_node for a node without boundary ops (slot_of < 0), inlined so f and g
// stay in registers
template <class L, class S, bool HG>
__device__ __forceinline__ void pull_node(const KArgs &a, int node, int sgn, typename Store<S>::T *f,
                                          typename Store<S>::T *g) {
    using T = typename Store<S>::T;
    int i, j, k;
    coords<L>(a.geo, node, i, j, k);
    load_node<L, S, HG>(static_cast<const S *>(a.src), a.geo, node, i, j, k, a.pull != 0, sgn,
                        is_interior<L>(a.geo, i, j, k), f, g, T(a.ph.shift_f), T(a.ph.shift_g));
}

template <class L, class S, int D>
__device__ __noinline__ void eval_node(const KArgs &a, int node, int seq_limit, typename Store<S>::T *f, typename Store<S>::T *g,
                          bool has_g, int sgn) {
    using T = typename Store<S>::T;
    constexpr int Q = L::Q;
    int i, j, k;
    coords<L>(a.geo, node, i, j, k);
    const T sf = T(a.ph.shift_f), sg = T(a.ph.shift_g);
    if (has_g) load_node<L, S, true>(static_cast<const S *>(a.src), a.geo, node, i, j, k, a.pull != 0, sgn,
                                     is_interior<L>(a.geo, i, j, k), f, g, sf, sg);
    else load_node<L, S, false>(static_cast<const S *>(a.src), a.geo, node, i, j, k, a.pull != 0, sgn,
                                is_interior<L>(a.geo, i, j, k), f, g, sf, sg);
    const int slot = a.slot_of[node];
    if (slot < 0) return;
    const int o1 = a.bstart[slot + 1];
    for (int o = a.bstart[slot]; o < o1; ++o) {
        const Op op = a.ops[o];
        if (op.seq >= seq_limit) break;
        if (op.kind == BC_SMOOTH) {
            if constexpr (D == 0) {
                atomicOr(a.err, ERR_RECURSION);   // chain deeper than any reference smoothing sequence
            } else {
                T acc[Q];
                const int nn = op.sub;
                for (int m = 0; m < nn; ++m) {
                    T fn[Q], gn[Q];
                    eval_node<L, S, D - 1>(a, op.nbr[m], op.seq, fn, gn, has_g, sgn);
                    const T *p = op.lat ? gn : fn;
#pragma unroll
                    for (int c = 0; c < Q; ++c) acc[c] = m == 0 ? p[c] : acc[c] + p[c];
                }
                T *p = op.lat ? g : f;
#pragma unroll
                for (int c = 0; c < Q; ++c) p[c] = nn == 2 ? T(0.5) * acc[c] : acc[c] / T(3);
            }
        } else {
            apply_op_ni<L, T>(op, f, g, node, a);
        }
    }
}

template <class L, class S, int K>
__global__ void __launch_bounds__(128) k_boundary(KArgs a) {
    using T = typename Store<S>::T;
    constexpr bool HG = kind_has_g(K);
    const int s = blockIdx.x * 128 + threadIdx.x;
    if (s >= a.nb) return;
    const int idx = a.bnode[s];
    T f[L::Q], g[L::Q];
    eval_node<L, S, 4>(a, idx, 0x7fffffff, f, g, HG, kind_is_adjoint(K) ? 1 : -1);
    T u[3];
    collide_node<L, T, K>(f, g, idx, a, a.save != 0, a.snap_coll, a.geo.np, !kind_is_adjoint(K) ? u : nullptr);
    if (!kind_is_adjoint(K) && a.bcu_out[0]) {
        a.bcu_out[0][idx] = double(u[0]);
        a.bcu_out[1][idx] = double(u[1]);
        if (L::ND == 3) a.bcu_out[2][idx] = double(u[2]);
    }
    const T sf = T(a.ph.shift_f), sg = T(a.ph.shift_g);
    store_collided<L, S, HG>(a, idx, f, g, sf, sg);
}

// ---- staged boundary path -------------------------------------------------------------------
// pre-collision state of staged node s: pull + its non-smoothing ops -> scratch
template <class L, class S>
__device__ __forceinline__ void bnd_pre_node(const KArgs &a, int s) {
    using T = typename Store<S>::T;
    constexpr int Q = L::Q;
    const int node = a.snode[s];
    int i, j, k;
    coords<L>(a.geo, node, i, j, k);
    T f[Q], g[Q];
    const T sf = T(a.ph.shift_f), sg = T(a.ph.shift_g);
    load_node<L, S, true>(static_cast<const S *>(a.src), a.geo, node, i, j, k, a.pull != 0, a.sgn,
                          is_interior<L>(a.geo, i, j, k), f, g, sf, sg);
    for (int o = a.sstart[s]; o < a.sstart[s + 1]; ++o) apply_op<L, T>(a.sops[o], f, g, node, a);
    T *tb = static_cast<T *>(a.tbuf);
#pragma unroll
    for (int c = 0; c < Q; ++c) {
        tb[(long long)c * a.ns + s] = f[c];
        tb[(long long)(Q + c) * a.ns + s] = g[c];
    }
}
// value of population plane `plane` under smoothing expression e: the reference's averages,
// (a + b) * 0.5 and (a + b + c) / 3 with operands in call order
template <class T, int D>
__device__ __noinline__ T smooth_eval(const SmoothNode *ex, int e, const T *tb, long long plane, int nslot, int *err) {
    if constexpr (D == 0) {
        atomicOr(err, ERR_SMOOTH_DEPTH);
        return T(0);
    } else {
        const SmoothNode x = ex[e];
        T v[3];
#pragma unroll
        for (int m = 0; m < 3; ++m) {
            if (m >= x.nnbr) { v[m] = T(0); continue; }
            const int ch = x.child[m];
            v[m] = ch < 0 ? tb[plane * nslot + (-ch - 1)] : smooth_eval<T, D - 1>(ex, ch, tb, plane, nslot, err);
        }
        const T s2 = v[0] + v[1];
        return x.nnbr == 3 ? (s2 + v[2]) / T(3) : T(0.5) * s2;
    }
}

// ---- snapshot: the collide's pre-relaxation g (what the reference stores in gi / igi) ----
template <class L, class S, int K>
__global__ void __launch_bounds__(128) k_snapshot(KArgs a) {
    using T = typename Store<S>::T;
    const int idx = blockIdx.x * 128 + threadIdx.x;
    if (idx >= a.geo.n) return;
    const int sgn = kind_is_adjoint(K) ? 1 : -1;
    if (a.slot_of[idx] < 0) {
        // no boundary op writes this node and no smoothing reads it: eval_node would only pull it,
        // so pull it here, into registers (eval_node's arrays live in local memory)
        T f[L::Q], g[L::Q];
        pull_node<L, S, true>(a, idx, sgn, f, g);
        collide_node<L, T, K>(f, g, idx, a, false, a.snap, a.geo.np, nullptr);
        return;
    }
    T f[L::Q], g[L::Q];
    eval_node<L, S, 4>(a, idx, 0x7fffffff, f, g, true, sgn);
    collide_node<L, T, K>(f, g, idx, a, false, a.snap, a.geo.np, nullptr);
}

// ---- stream + boundary program without collide (pre-collision state to dst) ----------------
template <class L, class S>
__global__ void __launch_bounds__(128) k_stream_program(KArgs a, int has_g, int sgn) {
    using T = typename Store<S>::T;
    const int idx = blockIdx.x * 128 + threadIdx.x;
    if (idx >= a.geo.n) return;
    const T sf = T(a.ph.shift_f), sg = T(a.ph.shift_g);
    if (a.slot_of[idx] < 0) {
        // pull only (as in k_snapshot): registers instead of eval_node's local-memory arrays
        T f[L::Q], g[L::Q];
        if (has_g) {
            pull_node<L, S, true>(a, idx, sgn, f, g);
            store_node<L, S, true>(static_cast<S *>(a.dst), a.geo, idx, f, g, sf, sg);
        } else {
            pull_node<L, S, false>(a, idx, sgn, f, g);
            store_node<L, S, false>(static_cast<S *>(a.dst), a.geo, idx, f, g, sf, sg);
        }
        return;
    }
    T f[L::Q], g[L::Q];
    eval_node<L, S, 4>(a, idx, 0x7fffffff, f, g, has_g != 0, sgn);
    if (has_g) store_node<L, S, true>(static_cast<S *>(a.dst), a.geo, idx, f, g, sf, sg);
    else store_node<L, S, false>(static_cast<S *>(a.dst), a.geo, idx, f, g, sf, sg);
}

// ---- equilibrium initial conditions (navierstokes.h:548-572, advection.h:1046-1070,
//      adjointnavierstokes.h:472-498, adjointadvection.h:1357-1381) ---------------------------
// which: 0 NS (rho,u), 1 AD (T,u), 2 ANS (ip,iu; u), 3 AAD (iT,iq; u), 4 NSin (rho,u),
// 5 ANSin (ip,iu) (nsincompressible.h:202-212, adjointnsincompressible.h:180-192), 6 EL (in0 rho,
// u, in1..in3 + uz = sxx, sxy, syx, syy; elastic.h:168-179), 7 AEL (in0 irho, u = imx, imy,
// in1..in3 + uz = isxx, isxy, isyx, isyy, gamma field; adjointelastic.h:127-138). in[]: double
// fields.
template <class L, class S>
__global__ void k_init(KArgs a, int which, const double *in0, const double *in1, const double *in2,
                       const double *in3, const double *ux, const double *uy, const double *uz) {
    using T = typename Store<S>::T;
    const int idx = blockIdx.x * kBlock + threadIdx.x;
    if (idx >= a.geo.n) return;
    constexpr int Q = L::Q;
    const T u[3] = {T(ux[idx]), T(uy[idx]), (L::ND == 3 && which < 6) ? T(uz[idx]) : T(0)};
    S *dst = static_cast<S *>(a.dst);
    const int set = (which == 1 || which == 3) ? 1 : 0;
    const T sh = set ? T(a.ph.shift_g) : T(a.ph.shift_f);
    T eq[Q];
    if (which == 0) {
        const T uu = ns_uu<L, T>(u);
#pragma unroll
        for (int c = 0; c < Q; ++c) eq[c] = ns_feq<L, T>(c, T(in0[idx]), u, uu);
    } else if (which == 1) {
#pragma unroll
        for (int c = 0; c < Q; ++c) eq[c] = ad_geq<L, T>(c, T(in0[idx]), u);
    } else if (which == 2) {
        const T iu[3] = {T(in1[idx]), T(in2[idx]), L::ND == 3 ? T(in3[idx]) : T(0)};
#pragma unroll
        for (int c = 0; c < Q; ++c) eq[c] = ans_feq<L, T>(c, u, T(in0[idx]), iu);
    } else if (which == 4) {
        const T rhouu = T(in0[idx]) - T(1.5) * (u[0] * u[0] + u[1] * u[1]);
#pragma unroll
        for (int c = 0; c < Q; ++c) eq[c] = nsin_feq<L, T>(c, u, rhouu);
    } else if (which == 5) {
        const T iu[3] = {T(in1[idx]), T(in2[idx]), T(0)};
#pragma unroll
        for (int c = 0; c < Q; ++c) eq[c] = ansin_feq<L, T>(c, T(in0[idx]), iu);
    } else if (which == 6) {
        const T sg[4] = {T(in1[idx]), T(in2[idx]), T(in3[idx]), T(uz[idx])};
#pragma unroll
        for (int c = 0; c < Q; ++c) eq[c] = el_feq<L, T>(c, T(in0[idx]), u, sg);
    } else if (which == 7) {
        const T m[7] = {T(in0[idx]), u[0], u[1], T(in1[idx]), T(in2[idx]), T(in3[idx]), T(uz[idx])};
        const T gm = ldT<T>(a.gamma, idx);
#pragma unroll
        for (int c = 0; c < Q; ++c) eq[c] = ael_feq<L, T>(c, m, gm);
    } else {
        const T iq[3] = {T(in1[idx]), T(in2[idx]), L::ND == 3 ? T(in3[idx]) : T(0)};
        const T v = T(in0[idx]) + T(3) * vdot<L, T>(u, iq);
#pragma unroll
        for (int c = 0; c < Q; ++c) eq[c] = v;
    }
#pragma unroll
    for (int c = 0; c < Q; ++c)
        Store<S>::st(dst + (long long)(set * Q + c) * a.geo.np + idx, Store<S>::enc(eq[c], L::template w<T>(c) * sh));
}

// population transfer between the storage format and double SoA (host exchange)
template <class L, class S>
__global__ void k_decode(const S *src, double *out, long long np, int n, int set, double shift) {
    using T = typename Store<S>::T;
    const long long t = (long long)blockIdx.x * kBlock + threadIdx.x;
    if (t >= (long long)L::Q * n) return;
    const int c = int(t / n), idx = int(t % n);
    out[t] = double(Store<S>::dec(src[(long long)(set * L::Q + c) * np + idx], L::template w<T>(c) * T(shift)));
}
template <class L, class S>
__global__ void k_encode(const double *in, S *dst, long long np, int n, int set, double shift) {
    using T = typename Store<S>::T;
    const long long t = (long long)blockIdx.x * kBlock + threadIdx.x;
    if (t >= (long long)L::Q * n) return;
    const int c = int(t / n), idx = int(t % n);
    dst[(long long)(set * L::Q + c) * np + idx] = Store<S>::enc(T(in[t]), L::template w<T>(c) * T(shift));
}

}  // namespace pl
