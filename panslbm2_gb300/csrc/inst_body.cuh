// inst_body.cuh -- explicit kernel instantiations and launch switch for one
// (lattice, storage) pair. Included by inst_<lattice>_<storage>{,_adj,_misc,_aux,_side}.cu with PL_LAT,
// PL_STORE and PL_NAME defined; PL_ALL_KINDS selects every collide kind (else the primary ones
// only) and PL_INCOMPRESSIBLE adds the D2Q9-only NSin / ANSin kinds, PL_ELASTIC the D2Q9-only
// EL / AEL kinds. PL_PART splits one pair over five translation units compiled in parallel
// (each kernel is the same code in any split): 1, 4, 5 the collide / step launches of the kind
// groups A, B, C, 2 the auxiliary launches (standalone stream, init, host transfer), 3 the
// side-stream boundary kernels.
#include "kernels.cuh"
#include "launch.h"

namespace pl {

#define PL_CAT2(a, b) a##b
#define PL_CAT(a, b) PL_CAT2(a, b)

using TC = Store<PL_STORE>::T;

// step launches by kind group: A the forward inline-boundary kinds (and the launch switch),
// B the adjoint inline-boundary kinds, C every other kind
#ifndef PL_PART
#define PL_STEP_A 1
#define PL_STEP_B 1
#define PL_STEP_C 1
#define PL_PART_AUX 1
#define PL_PART_SIDE 1
#else
#define PL_STEP_A (PL_PART == 1)
#define PL_STEP_B (PL_PART == 4)
#define PL_STEP_C (PL_PART == 5)
#define PL_PART_AUX (PL_PART == 2)
#define PL_PART_SIDE (PL_PART == 3)
#endif
#define PL_PART_STEP (PL_STEP_A || PL_STEP_B || PL_STEP_C)

#if PL_PART_SIDE

// collide of a runtime kind (uniform over the grid), for the boundary kernels
static __device__ __forceinline__ void collide_any(int kind, TC *f, TC *g, int idx, const KArgs &a, bool save, TC *u) {
    switch (kind) {
    case K_AD_NATURAL: collide_node<PL_LAT, TC, K_AD_NATURAL>(f, g, idx, a, save, a.snap_coll, a.geo.np, u); break;
    case K_AD_FORCE: collide_node<PL_LAT, TC, K_AD_FORCE>(f, g, idx, a, save, a.snap_coll, a.geo.np, u); break;
    case K_AAD_NATURAL: collide_node<PL_LAT, TC, K_AAD_NATURAL>(f, g, idx, a, save, a.snap_coll, a.geo.np, nullptr); break;
    case K_AAD_FORCE: collide_node<PL_LAT, TC, K_AAD_FORCE>(f, g, idx, a, save, a.snap_coll, a.geo.np, nullptr); break;
    case K_NS_COLLIDE: collide_node<PL_LAT, TC, K_NS_COLLIDE>(f, g, idx, a, save, a.snap_coll, a.geo.np, u); break;
#ifdef PL_ALL_KINDS
    case K_NS_BRINKMAN: collide_node<PL_LAT, TC, K_NS_BRINKMAN>(f, g, idx, a, save, a.snap_coll, a.geo.np, u); break;
    case K_AD_HEATEX: collide_node<PL_LAT, TC, K_AD_HEATEX>(f, g, idx, a, save, a.snap_coll, a.geo.np, u); break;
    case K_AD_NATURAL_NOBRINK: collide_node<PL_LAT, TC, K_AD_NATURAL_NOBRINK>(f, g, idx, a, save, a.snap_coll, a.geo.np, u); break;
    case K_AD_FORCE_NOBRINK: collide_node<PL_LAT, TC, K_AD_FORCE_NOBRINK>(f, g, idx, a, save, a.snap_coll, a.geo.np, u); break;
    case K_ANS_BRINKMAN: collide_node<PL_LAT, TC, K_ANS_BRINKMAN>(f, g, idx, a, save, a.snap_coll, a.geo.np, nullptr); break;
    case K_AAD_HEATEX: collide_node<PL_LAT, TC, K_AAD_HEATEX>(f, g, idx, a, save, a.snap_coll, a.geo.np, nullptr); break;
    case K_AAD_MASSFLOW: collide_node<PL_LAT, TC, K_AAD_MASSFLOW>(f, g, idx, a, save, a.snap_coll, a.geo.np, nullptr); break;
#endif
#if defined(PL_ALL_KINDS) && defined(PL_INCOMPRESSIBLE)
    case K_NSIN_COLLIDE: collide_node<PL_LAT, TC, K_NSIN_COLLIDE>(f, g, idx, a, save, a.snap_coll, a.geo.np, u); break;
    case K_NSIN_BRINKMAN: collide_node<PL_LAT, TC, K_NSIN_BRINKMAN>(f, g, idx, a, save, a.snap_coll, a.geo.np, u); break;
    case K_ANSIN_BRINKMAN: collide_node<PL_LAT, TC, K_ANSIN_BRINKMAN>(f, g, idx, a, save, a.snap_coll, a.geo.np, nullptr); break;
#endif
#if defined(PL_ALL_KINDS) && defined(PL_ELASTIC)
    case K_EL_COLLIDE: collide_node<PL_LAT, TC, K_EL_COLLIDE>(f, g, idx, a, save, a.snap_coll, a.geo.np, u); break;
    case K_EL_EXTENDED: collide_node<PL_LAT, TC, K_EL_EXTENDED>(f, g, idx, a, save, a.snap_coll, a.geo.np, u); break;
    case K_AEL_COLLIDE: collide_node<PL_LAT, TC, K_AEL_COLLIDE>(f, g, idx, a, save, a.snap_coll, a.geo.np, nullptr); break;
#endif
    default: break;
    }
}

static __device__ __forceinline__ void finish_boundary(int kind, TC *f, TC *g, int node, const KArgs &a) {
    constexpr int Q = PL_LAT::Q;
    TC u[3] = {TC(0), TC(0), TC(0)};
    collide_any(kind, f, g, node, a, a.save != 0, u);
    if (!kind_is_adjoint(kind) && a.bcu_out[0]) {
        a.bcu_out[0][node] = double(u[0]);
        a.bcu_out[1][node] = double(u[1]);
        if (PL_LAT::ND == 3) a.bcu_out[2][node] = double(u[2]);
    }
    const TC sf = TC(a.ph.shift_f), sg = TC(a.ph.shift_g);
    store_collided<PL_LAT, PL_STORE, true>(a, node, f, g, sf, sg);
    (void)Q;
}

// direct: boundary nodes no smoothing op writes: pull + ops in call order + collide + store
static __global__ void __launch_bounds__(128) k_bnd_direct(KArgs a, int kind) {
    constexpr int Q = PL_LAT::Q;
    const int s = blockIdx.x * 128 + threadIdx.x;
    if (s >= a.ndir) return;
    const int node = a.dnode[s];
    int i, j, k;
    coords<PL_LAT>(a.geo, node, i, j, k);
    TC f[Q], g[Q];
    const TC sf = TC(a.ph.shift_f), sg = TC(a.ph.shift_g);
    load_node<PL_LAT, PL_STORE, true>(static_cast<const PL_STORE *>(a.src), a.geo, node, i, j, k, a.pull != 0, a.sgn,
                                      is_interior<PL_LAT>(a.geo, i, j, k), f, g, sf, sg);
    for (int o = a.dstart[s]; o < a.dstart[s + 1]; ++o) apply_op<PL_LAT, TC>(a.dops[o], f, g, node, a);
    finish_boundary(kind, f, g, node, a);
}
// staged path for the nodes smoothing touches: pre-collision states into scratch (pre), then
// per target the composed smoothing expressions, the collide and the store (post)
static __global__ void __launch_bounds__(128) k_bnd_pre(KArgs a) {
    const int s = blockIdx.x * 128 + threadIdx.x;
    if (s < a.ns) bnd_pre_node<PL_LAT, PL_STORE>(a, s);
}
// one warp per target: lane l < 2Q evaluates the smoothing expression of set l / Q, population
// l % Q; lane 0 then collides and stores the target
constexpr int kPostWarps = 4;
static __global__ void __launch_bounds__(32 * kPostWarps) k_bnd_post(KArgs a, int kind) {
    constexpr int Q = PL_LAT::Q;
    __shared__ TC val[kPostWarps][2 * Q];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int t = blockIdx.x * kPostWarps + w;
    if (t >= a.nt) return;
    const int idx = a.snode[a.tslot[t]];
    const TC *tb = static_cast<const TC *>(a.tbuf);
    if (lane < 2 * Q) {
        const int lat = lane / Q;
        const int root = a.troot[2 * t + lat];
        const long long plane = lane;   // = lat * Q + c
        val[w][lane] = root < 0 ? tb[plane * a.ns + (-root - 1)]
                                : smooth_eval<TC, kSmoothDepth>(a.sexpr, root, tb, plane, a.ns, a.err);
    }
    __syncwarp();
    if (lane == 0) {
        TC f[Q], g[Q];
#pragma unroll
        for (int c = 0; c < Q; ++c) { f[c] = val[w][c]; g[c] = val[w][Q + c]; }
        finish_boundary(kind, f, g, idx, a);
    }
}

// stream-only counterparts of the staged boundary kernels: the same pull, ops and smoothing
// expressions, then the store of the pre-collision state
static __global__ void __launch_bounds__(128) k_bnd_direct_stream(KArgs a) {
    constexpr int Q = PL_LAT::Q;
    const int s = blockIdx.x * 128 + threadIdx.x;
    if (s >= a.ndir) return;
    const int node = a.dnode[s];
    int i, j, k;
    coords<PL_LAT>(a.geo, node, i, j, k);
    TC f[Q], g[Q];
    const TC sf = TC(a.ph.shift_f), sg = TC(a.ph.shift_g);
    load_node<PL_LAT, PL_STORE, true>(static_cast<const PL_STORE *>(a.src), a.geo, node, i, j, k, true, a.sgn,
                                      is_interior<PL_LAT>(a.geo, i, j, k), f, g, sf, sg);
    for (int o = a.dstart[s]; o < a.dstart[s + 1]; ++o) apply_op<PL_LAT, TC>(a.dops[o], f, g, node, a);
    store_node<PL_LAT, PL_STORE, true>(static_cast<PL_STORE *>(a.dst), a.geo, node, f, g, sf, sg);
}
static __global__ void __launch_bounds__(32 * kPostWarps) k_bnd_post_stream(KArgs a) {
    constexpr int Q = PL_LAT::Q;
    __shared__ TC val[kPostWarps][2 * Q];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int t = blockIdx.x * kPostWarps + w;
    if (t >= a.nt) return;
    const int idx = a.snode[a.tslot[t]];
    const TC *tb = static_cast<const TC *>(a.tbuf);
    if (lane < 2 * Q) {
        const int lat = lane / Q;
        const int root = a.troot[2 * t + lat];
        const long long plane = lane;
        val[w][lane] = root < 0 ? tb[plane * a.ns + (-root - 1)]
                                : smooth_eval<TC, kSmoothDepth>(a.sexpr, root, tb, plane, a.ns, a.err);
    }
    __syncwarp();
    if (lane == 0) {
        TC f[Q], g[Q];
#pragma unroll
        for (int c = 0; c < Q; ++c) { f[c] = val[w][c]; g[c] = val[w][Q + c]; }
        store_node<PL_LAT, PL_STORE, true>(static_cast<PL_STORE *>(a.dst), a.geo, idx, f, g, TC(a.ph.shift_f),
                                           TC(a.ph.shift_g));
    }
}

// the side-stream chains: the direct nodes on `side`, the staged nodes (pre -> post) on `side2`
void PL_CAT(side_step_, PL_NAME)(const KArgs &a, int kind, cudaStream_t side, cudaStream_t side2) {
    if (a.ndir > 0) k_bnd_direct<<<(a.ndir + 127) / 128, 128, 0, side>>>(a, kind);
    if (a.ns > 0) {
        k_bnd_pre<<<(a.ns + 127) / 128, 128, 0, side2>>>(a);
        if (a.nt > 0) k_bnd_post<<<(a.nt + kPostWarps - 1) / kPostWarps, 32 * kPostWarps, 0, side2>>>(a, kind);
    }
}
void PL_CAT(side_stream_, PL_NAME)(const KArgs &a, cudaStream_t side, cudaStream_t side2) {
    if (a.ndir > 0) k_bnd_direct_stream<<<(a.ndir + 127) / 128, 128, 0, side>>>(a);
    if (a.ns > 0) {
        k_bnd_pre<<<(a.ns + 127) / 128, 128, 0, side2>>>(a);
        if (a.nt > 0) k_bnd_post_stream<<<(a.nt + kPostWarps - 1) / kPostWarps, 32 * kPostWarps, 0, side2>>>(a);
    }
}
#endif  // PL_PART_SIDE

static dim3 interior_grid(const Geo &g) {
    return dim3((g.nx + 31) / 32, (g.ny + 7) / 8, PL_LAT::ND == 2 ? 1 : g.nz);
}

#if PL_PART_STEP

// the pull part of a fused step
template <int K>
static void launch_pull(const KArgs &a, cudaStream_t st) {
    k_interior<PL_LAT, PL_STORE, K, true><<<interior_grid(a.geo), dim3(32, 8), 0, st>>>(a);
}

template <int K>
static void run_kind(int op, bool save, const KArgs &a, cudaStream_t st) {
    switch (op) {
    case OP_COLLIDE:
        k_interior<PL_LAT, PL_STORE, K, false><<<interior_grid(a.geo), dim3(32, 8), 0, st>>>(a);
        break;
    case OP_STEP:
        if (a.nb > 0 && a.staged) {
            // two boundary chains on side streams, concurrent with the interior kernel
            cudaStream_t side = static_cast<cudaStream_t>(a.side), side2 = static_cast<cudaStream_t>(a.side2);
            cudaEventRecord(static_cast<cudaEvent_t>(a.ev_fork), st);
            cudaStreamWaitEvent(side, static_cast<cudaEvent_t>(a.ev_fork), 0);
            cudaStreamWaitEvent(side2, static_cast<cudaEvent_t>(a.ev_fork), 0);
            PL_CAT(side_step_, PL_NAME)(a, K, side, side2);
            launch_pull<K>(a, st);
            cudaEventRecord(static_cast<cudaEvent_t>(a.ev_join), side);
            cudaEventRecord(static_cast<cudaEvent_t>(a.ev_join2), side2);
            cudaStreamWaitEvent(st, static_cast<cudaEvent_t>(a.ev_join), 0);
            cudaStreamWaitEvent(st, static_cast<cudaEvent_t>(a.ev_join2), 0);
        } else {
            launch_pull<K>(a, st);
            if (a.nb > 0) k_boundary<PL_LAT, PL_STORE, K><<<(a.nb + 127) / 128, 128, 0, st>>>(a);
        }
        break;
    case OP_BOUNDARY:
        if (a.nb > 0) k_boundary<PL_LAT, PL_STORE, K><<<(a.nb + 127) / 128, 128, 0, st>>>(a);
        break;
    case OP_SNAPSHOT:
        k_snapshot<PL_LAT, PL_STORE, K><<<(a.geo.n + 127) / 128, 128, 0, st>>>(a);
        break;
    }
}

#if PL_STEP_A
static int launch_group_a(int kind, int op, bool save, const KArgs &a, cudaStream_t st) {
    switch (kind) {
    case K_AD_NATURAL: run_kind<K_AD_NATURAL>(op, save, a, st); return 0;
    case K_AD_FORCE: run_kind<K_AD_FORCE>(op, save, a, st); return 0;
    default: return -1;
    }
}
#endif

#if PL_STEP_B
int PL_CAT(launch_adj_, PL_NAME)(int kind, int op, bool save, const KArgs &a, cudaStream_t st) {
    switch (kind) {
    case K_AAD_NATURAL: run_kind<K_AAD_NATURAL>(op, save, a, st); return 0;
    case K_AAD_FORCE: run_kind<K_AAD_FORCE>(op, save, a, st); return 0;
    default: return -1;
    }
}
#endif

#if PL_STEP_C
int PL_CAT(launch_misc_, PL_NAME)(int kind, int op, bool save, const KArgs &a, cudaStream_t st) {
    switch (kind) {
    case K_NS_COLLIDE: run_kind<K_NS_COLLIDE>(op, save, a, st); return 0;
#ifdef PL_ALL_KINDS
    case K_NS_BRINKMAN: run_kind<K_NS_BRINKMAN>(op, save, a, st); return 0;
    case K_AD_HEATEX: run_kind<K_AD_HEATEX>(op, save, a, st); return 0;
    case K_AD_NATURAL_NOBRINK: run_kind<K_AD_NATURAL_NOBRINK>(op, save, a, st); return 0;
    case K_AD_FORCE_NOBRINK: run_kind<K_AD_FORCE_NOBRINK>(op, save, a, st); return 0;
    case K_ANS_BRINKMAN: run_kind<K_ANS_BRINKMAN>(op, save, a, st); return 0;
    case K_AAD_HEATEX: run_kind<K_AAD_HEATEX>(op, save, a, st); return 0;
    case K_AAD_MASSFLOW: run_kind<K_AAD_MASSFLOW>(op, save, a, st); return 0;
#endif
#if defined(PL_ALL_KINDS) && defined(PL_INCOMPRESSIBLE)
    case K_NSIN_COLLIDE: run_kind<K_NSIN_COLLIDE>(op, save, a, st); return 0;
    case K_NSIN_BRINKMAN: run_kind<K_NSIN_BRINKMAN>(op, save, a, st); return 0;
    case K_ANSIN_BRINKMAN: run_kind<K_ANSIN_BRINKMAN>(op, save, a, st); return 0;
#endif
#if defined(PL_ALL_KINDS) && defined(PL_ELASTIC)
    case K_EL_COLLIDE: run_kind<K_EL_COLLIDE>(op, save, a, st); return 0;
    case K_EL_EXTENDED: run_kind<K_EL_EXTENDED>(op, save, a, st); return 0;
    case K_AEL_COLLIDE: run_kind<K_AEL_COLLIDE>(op, save, a, st); return 0;
#endif
    default: return -1;
    }
}
#endif

#if PL_STEP_A
// every kind built for this (lattice, storage): the three groups in turn; -1 = not built
int PL_CAT(launch_, PL_NAME)(int kind, int op, bool save, const KArgs &a, cudaStream_t st) {
    if (launch_group_a(kind, op, save, a, st) == 0) return 0;
    if (PL_CAT(launch_adj_, PL_NAME)(kind, op, save, a, st) == 0) return 0;
    return PL_CAT(launch_misc_, PL_NAME)(kind, op, save, a, st);
}
#endif

#endif  // PL_PART_STEP

#if PL_PART_AUX
void PL_CAT(aux_, PL_NAME)(int op, const KArgs &a, int which, const double *const *in, int has_g, int sgn,
                           double *host_or_dev, int set, double shift, cudaStream_t st) {
    const int n = a.geo.n;
    switch (op) {
    case AUX_STREAM_PROGRAM:
        if (a.staged && a.icode && has_g && a.pull && a.nb > 0) {
            // the fused step's split without its collide: side chains concurrent with the pull
            cudaStream_t side = static_cast<cudaStream_t>(a.side), side2 = static_cast<cudaStream_t>(a.side2);
            cudaEventRecord(static_cast<cudaEvent_t>(a.ev_fork), st);
            cudaStreamWaitEvent(side, static_cast<cudaEvent_t>(a.ev_fork), 0);
            cudaStreamWaitEvent(side2, static_cast<cudaEvent_t>(a.ev_fork), 0);
            PL_CAT(side_stream_, PL_NAME)(a, side, side2);
            k_interior_stream<PL_LAT, PL_STORE><<<interior_grid(a.geo), dim3(32, 8), 0, st>>>(a, sgn);
            cudaEventRecord(static_cast<cudaEvent_t>(a.ev_join), side);
            cudaEventRecord(static_cast<cudaEvent_t>(a.ev_join2), side2);
            cudaStreamWaitEvent(st, static_cast<cudaEvent_t>(a.ev_join), 0);
            cudaStreamWaitEvent(st, static_cast<cudaEvent_t>(a.ev_join2), 0);
        } else {
            k_stream_program<PL_LAT, PL_STORE><<<(n + 127) / 128, 128, 0, st>>>(a, has_g, sgn);
        }
        break;
    case AUX_INIT:
        k_init<PL_LAT, PL_STORE><<<(n + kBlock - 1) / kBlock, kBlock, 0, st>>>(a, which, in[0], in[1], in[2], in[3],
                                                                              in[4], in[5], in[6]);
        break;
    case AUX_DECODE: {
        const long long tot = (long long)PL_LAT::Q * n;
        k_decode<PL_LAT, PL_STORE><<<(unsigned)((tot + kBlock - 1) / kBlock), kBlock, 0, st>>>(
            static_cast<const PL_STORE *>(a.src), host_or_dev, a.geo.np, n, set, shift);
        break;
    }
    case AUX_ENCODE: {
        const long long tot = (long long)PL_LAT::Q * n;
        k_encode<PL_LAT, PL_STORE><<<(unsigned)((tot + kBlock - 1) / kBlock), kBlock, 0, st>>>(
            host_or_dev, static_cast<PL_STORE *>(a.dst), a.geo.np, n, set, shift);
        break;
    }
    }
}
#endif  // PL_PART_AUX

}  // namespace pl
