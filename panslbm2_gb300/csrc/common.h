// common.h -- host/device shared descriptors of the CUDA library.
#pragma once
#include <stdint.h>

namespace pl {

// Collide kinds (one per reference collide routine; see include/panslbm_gb300.h).
enum Kind {
    K_NS_COLLIDE = 0, K_NS_BRINKMAN = 1, K_AD_NATURAL = 2, K_AD_FORCE = 3, K_AD_HEATEX = 4,
    K_AD_NATURAL_NOBRINK = 5, K_AD_FORCE_NOBRINK = 6, K_NSIN_COLLIDE = 7, K_NSIN_BRINKMAN = 8,
    K_ANS_BRINKMAN = 10, K_AAD_NATURAL = 11, K_AAD_FORCE = 12, K_AAD_HEATEX = 13, K_AAD_MASSFLOW = 14,
    K_ANSIN_BRINKMAN = 15, K_EL_COLLIDE = 16, K_EL_EXTENDED = 17, K_AEL_COLLIDE = 18
};
__host__ __device__ constexpr bool kind_is_adjoint(int k) { return (k >= 10 && k <= 15) || k == K_AEL_COLLIDE; }
// the elastic variants (EL / AEL), defined by the reference for D2Q9 only
__host__ __device__ constexpr bool kind_elastic(int k) {
    return k == K_EL_COLLIDE || k == K_EL_EXTENDED || k == K_AEL_COLLIDE;
}
// the incompressible variants (NSin / ANSin), defined by the reference for D2Q9 only
__host__ __device__ constexpr bool kind_incompressible(int k) {
    return k == K_NSIN_COLLIDE || k == K_NSIN_BRINKMAN || k == K_ANSIN_BRINKMAN;
}
__host__ __device__ constexpr bool kind_has_g(int k) {
    return !(k == K_NS_COLLIDE || k == K_NS_BRINKMAN || k == K_ANS_BRINKMAN || kind_incompressible(k) ||
             kind_elastic(k));
}
__host__ __device__ constexpr bool kind_node_kappa(int k) {
    return k == K_AD_NATURAL || k == K_AD_FORCE || k == K_AAD_NATURAL || k == K_AAD_FORCE || k == K_AAD_MASSFLOW;
}
// kinds whose interior kernel applies the simple boundary ops inline
__host__ __device__ constexpr bool kind_inline_bc(int k) {
    return k == K_AD_NATURAL || k == K_AD_FORCE || k == K_AAD_NATURAL || k == K_AAD_FORCE;
}
__host__ __device__ constexpr bool kind_has_snapshot(int k) {
    return k == K_AD_NATURAL || k == K_AD_FORCE || k == K_AAD_NATURAL || k == K_AAD_FORCE || k == K_AAD_MASSFLOW;
}

// Boundary-program op kinds (same numbering as the oracle) plus smoothing.
enum BcKind {
    BC_WALL = 0, BC_IWALL = 1, BC_NS_U = 2, BC_NS_RHO = 3, BC_AD_T = 4, BC_AD_Q = 5, BC_AD_QC = 6,
    BC_ANS_U = 7, BC_ANS_RHO = 8, BC_AAD_T = 9, BC_AAD_Q = 10, BC_AAD_RHO = 11,
    BC_NSIN_U = 12, BC_NSIN_RHO = 13, BC_ANSIN_U = 14,   // D2Q9 only
    BC_EL_STRESS = 15, BC_AEL_STRESS = 16,               // D2Q9 only
    BC_SMOOTH = 20
};

// ops the interior kernel applies inline (walls, NS SetU / SetRho, AD SetT / SetQ, ANS iSetU /
// iSetRho, AAD iSetT / iSetQ)
__host__ __device__ constexpr bool op_is_simple(int k) {
    return k == BC_WALL || k == BC_IWALL || k == BC_AD_T || k == BC_AD_Q || k == BC_AD_QC || k == BC_AAD_T ||
           k == BC_AAD_Q || k == BC_NS_U || k == BC_NS_RHO || k == BC_ANS_U || k == BC_ANS_RHO;
}

// Compact record of the simple ops of one boundary node, read by the interior kernel in one
// round trip: op m is bits 16m..16m+15 of `code` (bits 0-3 simple kind index, 4-5 axis, 6 side
// (+1 when set), 7 set (g when set), 8 wall type (MIRROR when set)); val[m] its values:
// [0] T / qn / eps (AAD iSetQ) / u_x / rho, [1] constant kappa / u_y, [2] u_z, [3] eps (ANS).
struct InlineRec {
    uint64_t code;
    uint32_t nops, pad;
    double val[4][4];
};
constexpr int kInlineMaxOps = 4;
__host__ __device__ constexpr int simple_index(int k) {
    return k == BC_WALL ? 0 : k == BC_IWALL ? 1 : k == BC_AD_T ? 2 : k == BC_AD_Q ? 3 : k == BC_AD_QC ? 4
         : k == BC_AAD_T ? 5 : k == BC_AAD_Q ? 6 : k == BC_NS_U ? 7 : k == BC_NS_RHO ? 8 : k == BC_ANS_U ? 9 : 10;
}

// One boundary-program op as applied at one node. `lat` selects the population set the op
// writes (0 = NS set f, 1 = AD set g). For BC_SMOOTH, nnbr neighbours are averaged.
struct Op {
    int32_t kind;
    int8_t axis, dir, lat, sub;   // sub: wall type (1 BARRIER, 2 MIRROR) / iSetRho type / nnbr
    int32_t seq;                  // position in the recorded call order
    int32_t node;                 // node the op writes (differs from the owner for the
                                  // D3Q15 +x MIRROR quirk)
    int32_t nbr[3];
    double v0, v1, v2, eps;
};

// One smoothing average of the staged boundary path: the mean of nnbr operands, each either
// another average (child >= 0: its index) or the pre-smoothing value of a boundary-scratch slot
// (child < 0: slot -child-1). The smoothing calls of a step compose, in call order, into one
// such expression per (target, population set).
struct SmoothNode {
    int32_t child[3];
    int32_t nnbr;
};
constexpr int kSmoothDepth = 8;   // deepest composition the device evaluates

struct Geo {
    int nx, ny, nz, n;    // lattice extents, node count
    long long np;         // plane stride of one population (n rounded up)
    uint32_t face_mask;   // bit a*2+s: face (axis a, side s) carries boundary ops
    const uint8_t *flags; // optional per-node "has boundary ops" flags (interior lines)
};

struct Phys { double nu, diff, gx, gy, gz, tem0, shift_f, shift_g, tau; };

// Arguments of every population kernel. Field pointers are device pointers; `T*` members are
// stored as void* and cast to the kernel's compute type.
struct KArgs {
    Geo geo;
    const void *src;            // populations read (f planes then g planes)
    void *dst;                  // populations written
    const void *alpha, *kappa, *beta, *dirx, *diry, *dirz;   // design fields, compute type
    const void *fwd[5];         // adjoint kinds: forward rho, ux, uy, uz, tem (compute type)
    const void *elrho, *gamma;  // elastic kinds: density and stress scale (compute type)
    // forced-convection heat-sink extension (compute type, null = off): AD_FORCE adds the
    // volumetric heat source hsrc as w_c * hsrc to g; AAD_FORCE adds the volumetric objective
    // weight objw (dJ/dT) to every adjoint g population
    const void *hsrc, *objw;
    double uscale;              // factor on the prescribed velocity of NS SetU / ANS iSetU ops
    int sr;                     // 16-bit storage: stochastic rounding of the collide's stores
    uint32_t sr_seed;           // per-launch seed of the stochastic rounding
    double *out[11];            // macro outputs (forward: rho,ux,uy,uz,tem,qx,qy,qz;
                                //  adjoint: ip,iux,iuy,iuz,imx,imy,imz,item,iqx,iqy,iqz;
                                //  EL: ux,uy in 1,2 and sxx,sxy,syx,syy in 4..7;
                                //  AEL: irho 0, imx,imy 4,5, isxx,isxy,isyx,isyy 7..10)
    double *snap;               // pre-collision g snapshot, [q][np] planes (k_snapshot)
    double *snap_coll;          // the same, written by a saving collide or step itself
                                // (PL_OPT_SNAPSHOT_IN_STEP), else null
    // boundary program
    const int *bnode;           // boundary nodes (sorted)
    const int *bstart;          // CSR op offsets per boundary node
    const Op *ops;
    const int *slot_of;         // node -> boundary slot or -1
    int nb;
    const double *bcu[3];       // velocity read by AD / AAD boundary ops
    const double *bcrho, *bctem;  // forward rho / T read by AAD iSetRho
    const double *bckappa;      // per-node kappa read by AD SetQ
    double *bcu_out[3];         // where this step stores the new velocity of boundary nodes
    // staged boundary path. Boundary nodes no smoothing op writes take the direct kernel
    // (dnode, CSR dstart/dops); the nodes smoothing reads or writes (snode, CSR sstart/sops)
    // go through the scratch buffer: pre (ops) -> smoothing levels -> post (the nt targets).
    int staged;
    const int *icode;           // per node, read for face / flagged nodes: -1 no ops, -2 side
                                // path, >= 0 index of its InlineRec (ops applied inline)
    const InlineRec *irec;
    int ndir, ns, nt;
    const int *dnode, *dstart;
    const Op *dops;
    const int *snode, *sstart, *tslot;
    const Op *sops;
    const SmoothNode *sexpr;    // smoothing averages
    const int *troot;           // per target t and set: troot[2t+lat] >= 0 average, < 0 slot -v-1
    void *tbuf;                 // scratch: 2*Q planes of ns compute-type values
    void *side, *side2;         // host: cudaStream_t of the two boundary chains
    void *ev_fork, *ev_join, *ev_join2;   // host: cudaEvent_t
    int sgn;                    // -1 Stream, +1 iStream
    Phys ph;
    int pull;                   // 1: stream (pull) before the boundary program
    int save;                   // 1: write macro outputs
    int *err;                   // device error word (bit flags)
};

enum ErrBits { ERR_RECURSION = 1, ERR_BAD_OP = 2, ERR_SMOOTH_DEPTH = 4 };

}  // namespace pl
