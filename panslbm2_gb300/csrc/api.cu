// api.cu -- C ABI of the library (include/panslbm_gb300.h): lattice-pair handles, boundary
// program compilation, fused step / solve loop, snapshots, sensitivities, filters.
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <map>
#include <string>
#include <unordered_map>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "../../include/panslbm_gb300.h"
#include "common.h"
#include "fields.h"
#include "launch.h"

using pl::KArgs;
using pl::Op;

namespace {

thread_local std::string g_err;

// NVTX range around a C-ABI call (visible in Nsight timelines; no cost without a profiler)
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
};
#define PL_RANGE(name) NvtxRange nvtx_range_(name)

int fail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

#define CK(x)                                                                                     \
    do {                                                                                          \
        cudaError_t e_ = (x);                                                                     \
        if (e_ != cudaSuccess) return fail(PL_ERR_CUDA, "%s: %s", #x, cudaGetErrorString(e_));    \
    } while (0)

struct Program {
    bool valid = false;
    int nb = 0, nops = 0, nslot = 0;
    int *bnode = nullptr, *bstart = nullptr, *slot_of = nullptr;
    Op *ops = nullptr;
    uint8_t *flags = nullptr;
    uint32_t face_mask = 0;
    // staged boundary path
    bool staged = false;
    int ndir = 0, ndir_all = 0, ns = 0, nt = 0;
    int *icode = nullptr;
    pl::InlineRec *irec = nullptr;
    int *dnode = nullptr, *dstart = nullptr, *snode = nullptr, *sstart = nullptr, *tslot = nullptr;
    int *dnode_all = nullptr, *dstart_all = nullptr;
    Op *dops = nullptr, *sops = nullptr, *dops_all = nullptr;
    pl::SmoothNode *sexpr = nullptr;  // composed smoothing averages
    int *troot = nullptr;             // per target and set: average or scratch slot
    void *tbuf = nullptr;
};

struct Taps {
    int ntap = 0;
    int *di = nullptr, *dj = nullptr, *dk = nullptr;
    double *hat = nullptr;
};

typedef int (*LaunchFn)(int, int, bool, const KArgs &, cudaStream_t);
typedef void (*AuxFn)(int, const KArgs &, int, const double *const *, int, int, double *, int, double, cudaStream_t);

}  // namespace

struct pl_lattice_s {
    int q = 0, nd = 0, nx = 0, ny = 0, nz = 1, n = 0;
    long long np = 0;
    int storage = PL_FP32;
    bool fp32 = true;
    size_t ssize = 4, csize = 4;
    cudaStream_t st = nullptr;
    bool own_stream = false;
    void *pop[2] = {nullptr, nullptr};
    int cur = 0;
    double shift_f = 1.0, shift_g = 0.0;
    double *fld[48] = {nullptr};     // double fields by PL_* id (design inputs, forward solution)
    void *cfld[15] = {nullptr};      // compute-type copies: alpha,kappa,beta,dirx,diry,dirz,frho,fux,fuy,fuz,ftem,
                                     // EL density, gamma, heat source, objective weight
    double *fwd[2][8] = {{nullptr}};
    double *adj[2][11] = {{nullptr}};
    int fwd_next = 0, adj_next = 0;  // slot the next collide writes
    int fwd_saved = -1, adj_saved = -1, fwd_prev_saved = -1, adj_prev_saved = -1;
    int fwd_latest = -1;             // slot written by the last forward collide (boundary u)
    std::vector<Program> progs;
    double *snap[2] = {nullptr, nullptr};
    bool snap_ok[2] = {false, false};   // the snapshot buffer holds a taken / loaded snapshot
    bool snap_in_step = false;          // PL_OPT_SNAPSHOT_IN_STEP
    bool snap_fresh[2] = {false, false};   // the last collide of the family wrote the snapshot
    // last collide, for snapshots
    int last_kind = -1, last_src = -1, last_prog = -1, last_pull = 0, last_bcu_slot = -1;
    pl_phys last_ph{};
    // scratch
    double *partial = nullptr;
    int *nonfinite = nullptr;
    double *dout = nullptr;
    int *err = nullptr;
    double *scratch[8] = {nullptr};
    int *iscratch = nullptr;
    std::map<std::pair<int, long long>, Taps> taps;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaStream_t side = nullptr, side2 = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_join2 = nullptr;
    double last_ms = 0.0;
    long long launches = 0;
    LaunchFn launch = nullptr;
    AuxFn aux = nullptr;
    // CUDA graphs of two fused steps (one ping-pong period), keyed by the step inputs
    struct GraphKey {
        int kind, prog, cur, fwd_next, adj_next, fwd_latest;
        pl_phys ph;
        const void *hsrc, *objw;   // source fields in use (their pointers are baked into the graph)
        double uscale;
        bool operator<(const GraphKey &o) const { return memcmp(this, &o, sizeof *this) < 0; }
    };
    struct GraphEntry { cudaGraphExec_t exec; long long launches; };
    int side_prio = 0, prio_lo = 0, prio_hi = 0;
    std::map<GraphKey, GraphEntry> graphs;
    bool use_graphs = true;
    // device stores of a checkpointed sweep, per kind (populations, forward macros, snapshot)
    std::vector<void *> store[3];
    std::vector<char> snap_filled;   // PL_STORE_SNAP slots that hold a snapshot
    int *sens_mask = nullptr;        // source mask of pl_sensitivity_device
    double *wtab = nullptr;          // per-(node, tap) filter weights of pl_filter_weighted
    size_t wtab_len = 0;
    double uscale = 1.0;             // pl_set_inflow_scale
    bool sr = false;                 // PL_OPT_STOCHASTIC_ROUNDING
    uint32_t sr_count = 0;           // launches so far (seeds the stochastic rounding)
};

namespace {

LaunchFn pick_launch(int q, int s) {
    if (q == 9) return s == PL_FP64 ? pl::launch_d2q9_f64 : s == PL_FP32 ? pl::launch_d2q9_f32 : s == PL_FP16 ? pl::launch_d2q9_f16 : pl::launch_d2q9_bf16;
    return s == PL_FP64 ? pl::launch_d3q15_f64 : s == PL_FP32 ? pl::launch_d3q15_f32 : s == PL_FP16 ? pl::launch_d3q15_f16 : pl::launch_d3q15_bf16;
}
AuxFn pick_aux(int q, int s) {
    if (q == 9) return s == PL_FP64 ? pl::aux_d2q9_f64 : s == PL_FP32 ? pl::aux_d2q9_f32 : s == PL_FP16 ? pl::aux_d2q9_f16 : pl::aux_d2q9_bf16;
    return s == PL_FP64 ? pl::aux_d3q15_f64 : s == PL_FP32 ? pl::aux_d3q15_f32 : s == PL_FP16 ? pl::aux_d3q15_f16 : pl::aux_d3q15_bf16;
}

// host-side fault injection for tests (pl_debug_fail_alloc): after this many more successful
// device allocations the next one fails as if the device were out of memory; -1 = off
std::atomic<long long> g_fail_alloc_after{-1};

int dalloc(void **p, size_t bytes) {
    long long left = g_fail_alloc_after.load();
    while (left >= 0 && !g_fail_alloc_after.compare_exchange_weak(left, left - 1)) {}
    if (left == 0) {
        *p = nullptr;
        return fail(PL_ERR_ALLOC, "cudaMalloc(%zu): injected allocation failure", bytes);
    }
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) { *p = nullptr; cudaGetLastError(); return fail(PL_ERR_ALLOC, "cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e)); }
    return PL_OK;
}
int dzero(pl_lattice h, void *p, size_t bytes) {
    CK(cudaMemsetAsync(p, 0, bytes, h->st));
    return PL_OK;
}
int ensure_d(pl_lattice h, double **p, size_t count) {
    if (*p) return PL_OK;
    int r = dalloc((void **)p, sizeof(double) * count);
    if (r) return r;
    return dzero(h, *p, sizeof(double) * count);
}
int check_launch(pl_lattice h, int nk) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(PL_ERR_CUDA, "kernel launch: %s", cudaGetErrorString(e));
    h->launches += nk;
    return PL_OK;
}
bool valid_kind(int k) { return (k >= 0 && k <= 8) || (k >= 10 && k <= 18); }
// NSin / ANSin exist for D2Q9 only (nsincompressible.h, adjointnsincompressible.h)
int check_kind(pl_lattice h, int kind) {
    if (!valid_kind(kind)) return fail(PL_ERR_ARG, "unknown collide kind %d", kind);
    if ((pl::kind_incompressible(kind) || pl::kind_elastic(kind)) && h->nd != 2)
        return fail(PL_ERR_UNSUPPORTED, "kind %d is D2Q9 only", kind);
    return PL_OK;
}
int field_index_c(int f) {
    if (f >= PL_ALPHA && f <= PL_DIRZ) return f;
    if (f >= PL_FWD_RHO && f <= PL_FWD_TEM) return 6 + (f - PL_FWD_RHO);
    if (f == PL_DENSITY || f == PL_GAMMA) return 11 + (f - PL_DENSITY);
    if (f == PL_HEAT_SOURCE || f == PL_OBJ_WEIGHT) return 13 + (f - PL_HEAT_SOURCE);
    return -1;
}
// make sure a compute-type copy of field f exists and is current
int sync_cfield(pl_lattice h, int f) {
    int ci = field_index_c(f);
    if (ci < 0) return PL_OK;
    int r = ensure_d(h, &h->fld[f], h->n);
    if (r) return r;
    if (!h->cfld[ci]) { r = dalloc(&h->cfld[ci], h->csize * h->n); if (r) return r; }
    pl::launch_to_compute(h->fld[f], h->cfld[ci], h->n, h->fp32, h->st);
    return check_launch(h, 1);
}
int ensure_cfield(pl_lattice h, int f) {
    int ci = field_index_c(f);
    if (ci < 0) return fail(PL_ERR_ARG, "field %d has no compute copy", f);
    if (h->cfld[ci]) return PL_OK;
    return sync_cfield(h, f);
}

// ---- boundary program compilation ----------------------------------------------------------
int node_id(pl_lattice h, int i, int j, int k) {
    auto w = [](int v, int n) { return v == -1 ? n - 1 : (v == n ? 0 : v); };
    return w(i, h->nx) + h->nx * (w(j, h->ny) + h->ny * (h->nd == 3 ? w(k, h->nz) : 0));
}

int compile_program(pl_lattice h, const pl_bc_desc *descs, int ndesc, Program &P) {
    std::vector<Op> ops;
    int seq = 0;
    const int n[3] = {h->nx, h->ny, h->nz};
    auto smooth_op = [&](int lat, int node, int a, int b, int c, int nn) {
        Op o;
        memset(&o, 0, sizeof o);
        o.kind = pl::BC_SMOOTH; o.lat = (int8_t)lat; o.sub = (int8_t)nn; o.seq = seq; o.node = node;
        o.nbr[0] = a; o.nbr[1] = b; o.nbr[2] = c;
        ops.push_back(o);
    };
    auto smooth_at = [&](int lat, int i, int j, int k, int dx, int dy, int dz) {
        if (i < 0 || i >= h->nx || j < 0 || j >= h->ny) return;
        if (h->nd == 2) {
            smooth_op(lat, node_id(h, i, j, 0), node_id(h, i - dx, j, 0), node_id(h, i, j - dy, 0), -1, 2);
        } else {
            if (k < 0 || k >= h->nz) return;
            smooth_op(lat, node_id(h, i, j, k), node_id(h, i - dx, j, k), node_id(h, i, j - dy, k), node_id(h, i, j, k - dz), 3);
        }
    };
    auto smooth_line = [&](int lat, int plane, int pa, int pb, int da, int db) {
        if (h->nd != 3) return;
        if (plane == 0) {
            if (pa < 0 || pa >= h->ny || pb < 0 || pb >= h->nz) return;
            for (int i = 0; i < h->nx; ++i)
                smooth_op(lat, node_id(h, i, pa, pb), node_id(h, i, pa - da, pb), node_id(h, i, pa, pb - db), -1, 2);
        } else if (plane == 1) {
            if (pa < 0 || pa >= h->nz || pb < 0 || pb >= h->nx) return;
            for (int j = 0; j < h->ny; ++j)
                smooth_op(lat, node_id(h, pb, j, pa), node_id(h, pb, j, pa - da), node_id(h, pb - db, j, pa), -1, 2);
        } else {
            if (pa < 0 || pa >= h->nx || pb < 0 || pb >= h->ny) return;
            for (int k = 0; k < h->nz; ++k)
                smooth_op(lat, node_id(h, pa, pb, k), node_id(h, pa - da, pb, k), node_id(h, pa, pb - db, k), -1, 2);
        }
    };
    for (int di = 0; di < ndesc; ++di) {
        const pl_bc_desc &d = descs[di];
        if (d.kind == PL_SMOOTH_CORNER) {
            const int lx = h->nx, ly = h->ny, lz = h->nz, lat = d.lat;
            if (h->nd == 2) {
                smooth_at(lat, 0, 0, 0, -1, -1, 0); ++seq;
                smooth_at(lat, 0, ly - 1, 0, -1, 1, 0); ++seq;
                smooth_at(lat, lx - 1, 0, 0, 1, -1, 0); ++seq;
                smooth_at(lat, lx - 1, ly - 1, 0, 1, 1, 0); ++seq;
            } else {
                // d3q15.h:199-220
                smooth_line(lat, 0, 0, 0, -1, -1); ++seq;
                smooth_line(lat, 0, ly - 1, 0, 1, -1); ++seq;
                smooth_line(lat, 0, ly - 1, lz - 1, 1, 1); ++seq;
                smooth_line(lat, 0, 0, lz - 1, -1, 1); ++seq;
                smooth_line(lat, 1, 0, 0, -1, -1); ++seq;
                smooth_line(lat, 1, lz - 1, 0, 1, -1); ++seq;
                smooth_line(lat, 1, lz - 1, lx - 1, 1, 1); ++seq;
                smooth_line(lat, 1, 0, lx - 1, -1, 1); ++seq;
                smooth_line(lat, 2, 0, 0, -1, -1); ++seq;
                smooth_line(lat, 2, lx - 1, 0, 1, -1); ++seq;
                smooth_line(lat, 2, lx - 1, ly - 1, 1, 1); ++seq;
                smooth_line(lat, 2, 0, ly - 1, -1, 1); ++seq;
                smooth_at(lat, 0, 0, 0, -1, -1, -1); ++seq;
                smooth_at(lat, lx - 1, 0, 0, 1, -1, -1); ++seq;
                smooth_at(lat, lx - 1, ly - 1, 0, 1, 1, -1); ++seq;
                smooth_at(lat, 0, ly - 1, 0, -1, 1, -1); ++seq;
                smooth_at(lat, 0, 0, lz - 1, -1, -1, 1); ++seq;
                smooth_at(lat, lx - 1, 0, lz - 1, 1, -1, 1); ++seq;
                smooth_at(lat, lx - 1, ly - 1, lz - 1, 1, 1, 1); ++seq;
                smooth_at(lat, 0, ly - 1, lz - 1, -1, 1, 1); ++seq;
            }
            continue;
        }
        if (d.kind == PL_SMOOTH_AT) { smooth_at(d.lat, d.i, d.j, d.k, d.di, d.dj, d.dk); ++seq; continue; }
        if (d.kind == PL_SMOOTH_LINE) { smooth_line(d.lat, d.axis, d.i, d.j, d.di, d.dj); ++seq; continue; }
        if (d.kind < PL_BC_WALL || d.kind > PL_BC_AEL_STRESS)
            return fail(PL_ERR_ARG, "program desc %d: unknown kind %d", di, d.kind);
        if (d.kind >= PL_BC_NSIN_U && h->nd != 2)
            return fail(PL_ERR_UNSUPPORTED, "program desc %d: kind %d is D2Q9 only", di, d.kind);
        if (d.axis < 0 || d.axis >= h->nd || (d.dir != -1 && d.dir != 1))
            return fail(PL_ERR_ARG, "program desc %d: axis %d / dir %d invalid", di, d.axis, d.dir);
        const int a = d.axis, p = d.pos;
        if (p >= 0 && p < n[a]) {
            const int b = (a + 1) % 3, c = (a + 2) % 3;
            const int nb_ = (h->nd == 2 && b == 2) ? 1 : n[b], nc_ = (h->nd == 2 && c == 2) ? 1 : n[c];
            int lat = 0;
            if (d.kind == PL_BC_WALL || d.kind == PL_BC_IWALL) lat = d.lat;
            else if (d.kind == PL_BC_AD_T || d.kind == PL_BC_AD_Q || d.kind == PL_BC_AD_QC || d.kind == PL_BC_AAD_T ||
                     d.kind == PL_BC_AAD_Q) lat = 1;
            for (int u = 0; u < nb_; ++u)
                for (int v = 0; v < nc_; ++v) {
                    int x[3]; x[a] = p; x[b] = u; x[c] = v;
                    if (h->nd == 2) x[2] = 0;
                    const int idx = x[0] + h->nx * (x[1] + h->ny * x[2]);
                    const int t = d.type ? d.type[idx] : 1;
                    if (d.kind == PL_BC_WALL || d.kind == PL_BC_IWALL) { if (t != 1 && t != 2) continue; }
                    else if (t == 0) continue;
                    Op o;
                    memset(&o, 0, sizeof o);
                    o.kind = d.kind; o.axis = (int8_t)a; o.dir = (int8_t)d.dir; o.lat = (int8_t)lat; o.sub = (int8_t)t;
                    o.seq = seq; o.node = idx;
                    // D3Q15 forward MIRROR on the +x side writes node (nx-1, j, k) (d3q15.h:1013)
                    if (d.kind == PL_BC_WALL && h->nd == 3 && a == 0 && d.dir == 1 && t == 2)
                        o.node = (h->nx - 1) + h->nx * (x[1] + h->ny * x[2]);
                    o.v0 = d.v0 ? d.v0[idx] : d.c0;
                    o.v1 = d.v1 ? d.v1[idx] : d.c1;
                    o.v2 = d.v2 ? d.v2[idx] : d.c2;
                    if (d.kind == PL_BC_AD_QC) o.v1 = d.kappa;
                    o.eps = d.eps;
                    o.nbr[0] = o.nbr[1] = o.nbr[2] = -1;
                    ops.push_back(o);
                }
        }
        ++seq;
    }
    // group by node, keep call order inside a node
    std::stable_sort(ops.begin(), ops.end(), [](const Op &x, const Op &y) { return x.node < y.node; });
    std::vector<int> slot_of(h->n, -1), bstart, opnodes;
    for (size_t o = 0; o < ops.size(); ++o) {
        if (o == 0 || ops[o].node != ops[o - 1].node) {
            slot_of[ops[o].node] = (int)opnodes.size();
            opnodes.push_back(ops[o].node);
            bstart.push_back((int)o);
        }
    }
    bstart.push_back((int)ops.size());
    // every node whose state a smoothing op reads belongs to the boundary set as well
    std::vector<int> req = opnodes;
    for (const Op &o : ops)
        if (o.kind == pl::BC_SMOOTH)
            for (int m = 0; m < o.sub; ++m) req.push_back(o.nbr[m]);
    std::sort(req.begin(), req.end());
    req.erase(std::unique(req.begin(), req.end()), req.end());
    // skip mode: geometric when every such node lies on a domain face
    auto on_face_bits = [&](int idx) {
        const int i = idx % h->nx, r = idx / h->nx, j = r % h->ny, k = r / h->ny;
        uint32_t m = 0;
        if (i == 0) m |= 1; if (i == h->nx - 1) m |= 2; if (j == 0) m |= 4; if (j == h->ny - 1) m |= 8;
        if (h->nd == 3) { if (k == 0) m |= 16; if (k == h->nz - 1) m |= 32; }
        return m;
    };
    bool geometric = true;
    uint32_t mask = 0;
    for (int nd_ : req) {
        const uint32_t m = on_face_bits(nd_);
        if (!m) { geometric = false; break; }
        mask |= m;
    }
    std::vector<int> bnodes;
    std::vector<uint8_t> flags;
    if (geometric) {
        for (int idx = 0; idx < h->n; ++idx) if (on_face_bits(idx) & mask) bnodes.push_back(idx);
    } else {
        bnodes = req;
        flags.assign(h->n, 0);
        for (int nd_ : req) flags[nd_] = 1;
    }
    P.nb = (int)bnodes.size();
    P.nops = (int)ops.size();
    P.nslot = (int)opnodes.size();
    P.face_mask = geometric ? mask : 0;

    // staged path: valid when, at every node, the non-smoothing ops all come before the
    // smoothing ops, and every node a smoothing op reads has no non-smoothing op after it
    std::vector<int> bslot(h->n, -1);
    for (int b = 0; b < P.nb; ++b) bslot[bnodes[b]] = b;
    std::vector<int> last_plain(h->n, -1), first_smooth(h->n, 0x7fffffff);
    for (const Op &o : ops) {
        if (o.kind == pl::BC_SMOOTH) first_smooth[o.node] = std::min(first_smooth[o.node], o.seq);
        else last_plain[o.node] = std::max(last_plain[o.node], o.seq);
    }
    bool staged = true;
    for (const Op &o : ops) {
        if (o.kind != pl::BC_SMOOTH) continue;
        if (last_plain[o.node] > first_smooth[o.node]) staged = false;
        for (int m = 0; m < o.sub; ++m) if (last_plain[o.nbr[m]] > o.seq) staged = false;
    }
    {
        // ... and when the composed smoothing averages nest no deeper than the device evaluates
        std::vector<const Op *> sm;
        for (const Op &o : ops) if (o.kind == pl::BC_SMOOTH) sm.push_back(&o);
        std::stable_sort(sm.begin(), sm.end(), [](const Op *x, const Op *y) { return x->seq < y->seq; });
        std::map<long long, int> depth;   // (set, node) -> nesting of its current value
        for (const Op *o : sm) {
            int d = 0;
            for (int m = 0; m < o->sub; ++m) {
                auto it = depth.find((long long)o->lat * h->n + o->nbr[m]);
                if (it != depth.end()) d = std::max(d, it->second);
            }
            depth[(long long)o->lat * h->n + o->node] = d + 1;
            if (d + 1 > pl::kSmoothDepth) staged = false;
        }
    }
    // direct set D (boundary nodes no smoothing op writes), staged set S (nodes smoothing reads
    // or writes), targets T (nodes smoothing writes)
    std::vector<int> dnode, dstart, snode, sstart, tslot, dnode_all, dstart_all, icode;
    std::vector<pl::InlineRec> irec;
    std::vector<Op> dops, sops, dops_all;
    std::vector<pl::SmoothNode> sexpr;
    std::vector<int> troot;
    if (staged) {
        std::vector<char> is_t(h->n, 0), is_s(h->n, 0);
        for (const Op &o : ops)
            if (o.kind == pl::BC_SMOOTH) {
                is_t[o.node] = is_s[o.node] = 1;
                for (int m = 0; m < o.sub; ++m) is_s[o.nbr[m]] = 1;
            }
        auto plain_ops = [&](int node, std::vector<Op> &out) {
            const int sl = slot_of[node];
            if (sl >= 0)
                for (int o = bstart[sl]; o < bstart[sl + 1]; ++o)
                    if (ops[o].kind != pl::BC_SMOOTH) out.push_back(ops[o]);
        };
        // interior codes: smoothing targets and nodes with ops the interior kernel does not
        // apply go to the side path; other op nodes are applied inline (inline kinds) or by
        // the direct kernel (other kinds)
        icode.assign(h->n, -1);
        // nodes with the same ops and values share one record (walls, fluxes): fewer distinct
        // records for the face lanes of a warp to read
        std::unordered_map<std::string, int> rec_index;
        for (size_t sl = 0; sl < opnodes.size(); ++sl) {
            const int node = opnodes[sl];
            if (is_t[node]) { icode[node] = -2; continue; }
            bool simple = bstart[sl + 1] - bstart[sl] <= pl::kInlineMaxOps;
            for (int o = bstart[sl]; o < bstart[sl + 1]; ++o)
                if (!pl::op_is_simple(ops[o].kind)) simple = false;

            if (simple) {
                pl::InlineRec rec;
                memset(&rec, 0, sizeof rec);
                for (int o = bstart[sl]; o < bstart[sl + 1]; ++o) {
                    const Op &op = ops[o];
                    const int m = o - bstart[sl];
                    const uint64_t b = (uint64_t)pl::simple_index(op.kind) | ((uint64_t)op.axis << 4) |
                                       (op.dir > 0 ? 64u : 0u) | (op.lat ? 128u : 0u) | (op.sub == 2 ? 256u : 0u);
                    rec.code |= b << (16 * m);
                    rec.val[m][0] = (op.kind == pl::BC_AAD_Q) ? op.eps : op.v0;
                    rec.val[m][1] = op.v1;
                    rec.val[m][2] = op.v2;
                    rec.val[m][3] = op.eps;
                }
                rec.nops = (uint32_t)(bstart[sl + 1] - bstart[sl]);
                const std::string key(reinterpret_cast<const char *>(&rec), sizeof rec);
                auto it = rec_index.find(key);
                if (it == rec_index.end()) {
                    it = rec_index.emplace(key, (int)irec.size()).first;
                    irec.push_back(rec);
                }
                icode[node] = it->second;
            } else {
                icode[node] = -2;
            }
            if (!simple) { dnode.push_back(node); dstart.push_back((int)dops.size()); plain_ops(node, dops); }
            dnode_all.push_back(node); dstart_all.push_back((int)dops_all.size()); plain_ops(node, dops_all);
        }
        dstart.push_back((int)dops.size());
        dstart_all.push_back((int)dops_all.size());
        if (!geometric)
            for (int node = 0; node < h->n; ++node) if (is_s[node]) flags[node] = 1;
        std::vector<int> sslot(h->n, -1);
        for (int node = 0; node < h->n; ++node)
            if (is_s[node]) { sslot[node] = (int)snode.size(); snode.push_back(node); sstart.push_back((int)sops.size()); plain_ops(node, sops); }
        sstart.push_back((int)sops.size());
        for (int node = 0; node < h->n; ++node) if (is_t[node]) tslot.push_back(sslot[node]);
        // smoothing ops in call order, composed into one expression per (target, set): a
        // node's current value is its pre-smoothing scratch slot until an average writes it
        std::vector<const Op *> sm;
        for (const Op &o : ops) if (o.kind == pl::BC_SMOOTH) sm.push_back(&o);
        std::stable_sort(sm.begin(), sm.end(), [](const Op *x, const Op *y) { return x->seq < y->seq; });
        const size_t NS = snode.size();
        std::vector<int> cur(2 * NS);
        for (size_t sl = 0; sl < NS; ++sl) cur[sl] = cur[NS + sl] = -(int)sl - 1;
        for (const Op *o : sm) {
            const size_t L0 = o->lat ? NS : 0;
            pl::SmoothNode x;
            memset(&x, 0, sizeof x);
            x.nnbr = o->sub;
            for (int m = 0; m < o->sub; ++m) x.child[m] = cur[L0 + sslot[o->nbr[m]]];
            sexpr.push_back(x);
            cur[L0 + sslot[o->node]] = (int)sexpr.size() - 1;
        }
        for (int sl : tslot) { troot.push_back(cur[sl]); troot.push_back(cur[NS + sl]); }
        P.ndir = (int)dnode.size(); P.ndir_all = (int)dnode_all.size(); P.ns = (int)snode.size(); P.nt = (int)tslot.size();
    }
    P.staged = staged;

    int r;
    if ((r = dalloc((void **)&P.slot_of, sizeof(int) * h->n))) return r;
    CK(cudaMemcpyAsync(P.slot_of, slot_of.data(), sizeof(int) * h->n, cudaMemcpyHostToDevice, h->st));
    if (P.nb) {
        if ((r = dalloc((void **)&P.bnode, sizeof(int) * P.nb))) return r;
        CK(cudaMemcpyAsync(P.bnode, bnodes.data(), sizeof(int) * P.nb, cudaMemcpyHostToDevice, h->st));
    }
    if ((r = dalloc((void **)&P.bstart, sizeof(int) * bstart.size()))) return r;
    CK(cudaMemcpyAsync(P.bstart, bstart.data(), sizeof(int) * bstart.size(), cudaMemcpyHostToDevice, h->st));
    if (P.nops) {
        if ((r = dalloc((void **)&P.ops, sizeof(Op) * P.nops))) return r;
        CK(cudaMemcpyAsync(P.ops, ops.data(), sizeof(Op) * P.nops, cudaMemcpyHostToDevice, h->st));
    }
    if (staged && P.nb) {
        auto up_i = [&](int **dst, const std::vector<int> &v) -> int {
            if (v.empty()) return PL_OK;
            int rr = dalloc((void **)dst, sizeof(int) * v.size());
            if (rr) return rr;
            CK(cudaMemcpyAsync(*dst, v.data(), sizeof(int) * v.size(), cudaMemcpyHostToDevice, h->st));
            return PL_OK;
        };
        auto up_o = [&](Op **dst, const std::vector<Op> &v) -> int {
            if (v.empty()) return PL_OK;
            int rr = dalloc((void **)dst, sizeof(Op) * v.size());
            if (rr) return rr;
            CK(cudaMemcpyAsync(*dst, v.data(), sizeof(Op) * v.size(), cudaMemcpyHostToDevice, h->st));
            return PL_OK;
        };
        if ((r = up_i(&P.dnode, dnode)) || (r = up_i(&P.dstart, dstart)) || (r = up_i(&P.snode, snode)) ||
            (r = up_i(&P.sstart, sstart)) || (r = up_i(&P.tslot, tslot)) || (r = up_o(&P.dops, dops)) ||
            (r = up_o(&P.sops, sops)) || (r = up_i(&P.dnode_all, dnode_all)) ||
            (r = up_i(&P.dstart_all, dstart_all)) || (r = up_o(&P.dops_all, dops_all)) || (r = up_i(&P.icode, icode)))
            return r;
        if (!irec.empty()) {
            if ((r = dalloc((void **)&P.irec, sizeof(pl::InlineRec) * irec.size()))) return r;
            CK(cudaMemcpyAsync(P.irec, irec.data(), sizeof(pl::InlineRec) * irec.size(), cudaMemcpyHostToDevice, h->st));
        }
        if (!sexpr.empty()) {
            if ((r = dalloc((void **)&P.sexpr, sizeof(pl::SmoothNode) * sexpr.size()))) return r;
            CK(cudaMemcpyAsync(P.sexpr, sexpr.data(), sizeof(pl::SmoothNode) * sexpr.size(), cudaMemcpyHostToDevice, h->st));
        }
        if (P.ns && (r = dalloc(&P.tbuf, h->csize * 2 * h->q * (size_t)P.ns))) return r;
        if ((r = up_i(&P.troot, troot))) return r;
    }
    if (!geometric) {
        if ((r = dalloc((void **)&P.flags, h->n))) return r;
        CK(cudaMemcpyAsync(P.flags, flags.data(), h->n, cudaMemcpyHostToDevice, h->st));
    }
    CK(cudaStreamSynchronize(h->st));   // host vectors die here
    P.valid = true;
    return PL_OK;
}

void free_program(Program &P) {
    cudaFree(P.bnode); cudaFree(P.bstart); cudaFree(P.slot_of); cudaFree(P.ops); cudaFree(P.flags);
    cudaFree(P.dnode); cudaFree(P.dstart); cudaFree(P.snode); cudaFree(P.sstart); cudaFree(P.tslot);
    cudaFree(P.dops); cudaFree(P.sops); cudaFree(P.sexpr); cudaFree(P.tbuf); cudaFree(P.troot);
    cudaFree(P.icode); cudaFree(P.irec); cudaFree(P.dnode_all); cudaFree(P.dstart_all); cudaFree(P.dops_all);
    P = Program();
}

// ---- kernel argument assembly ------------------------------------------------------------
int build_args(pl_lattice h, int kind, const pl_phys *ph, int prog, int src, int dst, bool save, bool pull,
               int bcu_slot, KArgs &a, bool kind_inputs = true) {
    memset(&a, 0, sizeof a);
    a.geo.nx = h->nx; a.geo.ny = h->ny; a.geo.nz = h->nz; a.geo.n = h->n; a.geo.np = h->np;
    a.src = h->pop[src];
    a.dst = dst >= 0 ? h->pop[dst] : nullptr;
    a.ph.nu = ph ? ph->nu : 0.0; a.ph.diff = ph ? ph->diff : 0.0;
    a.ph.gx = ph ? ph->gx : 0.0; a.ph.gy = ph ? ph->gy : 0.0; a.ph.gz = ph ? ph->gz : 0.0;
    a.ph.tem0 = ph ? ph->tem0 : 0.0;
    a.ph.tau = ph ? ph->tau : 0.0;
    a.ph.shift_f = h->shift_f; a.ph.shift_g = h->shift_g;
    a.pull = pull ? 1 : 0;
    a.save = save ? 1 : 0;
    a.err = h->err;
    a.uscale = h->uscale;
    a.sr = (h->sr && h->ssize == 2) ? 1 : 0;
    a.sr_seed = 0x9E3779B9u * (++h->sr_count);
    const bool adjk = pl::kind_is_adjoint(kind);
    const bool elk = pl::kind_elastic(kind);
    a.sgn = adjk ? 1 : -1;
    // inputs required by the kind
    int r;
    if (!kind_inputs) goto program;
    if (elk) {
        if (kind != PL_AEL_COLLIDE) {
            if (!h->fld[PL_DENSITY]) return fail(PL_ERR_STATE, "kind %d needs PL_DENSITY", kind);
            if ((r = ensure_cfield(h, PL_DENSITY))) return r;
            a.elrho = h->cfld[11];
        }
        if (kind != PL_EL_COLLIDE) {
            if (!h->fld[PL_GAMMA]) return fail(PL_ERR_STATE, "kind %d needs PL_GAMMA", kind);
            if ((r = ensure_cfield(h, PL_GAMMA))) return r;
            a.gamma = h->cfld[12];
        }
    }
    if (kind == PL_NS_BRINKMAN || kind == PL_NSIN_BRINKMAN || kind == PL_AD_NATURAL || kind == PL_AD_FORCE ||
        kind == PL_AD_HEATEX || (adjk && !elk)) {
        if (!h->fld[PL_ALPHA]) return fail(PL_ERR_STATE, "kind %d needs PL_ALPHA", kind);
        if ((r = ensure_cfield(h, PL_ALPHA))) return r;
        a.alpha = h->cfld[0];
    }
    if (pl::kind_node_kappa(kind)) {
        if (!h->fld[PL_KAPPA]) return fail(PL_ERR_STATE, "kind %d needs PL_KAPPA", kind);
        if ((r = ensure_cfield(h, PL_KAPPA))) return r;
        a.kappa = h->cfld[1];
    }
    if (kind == PL_AD_HEATEX || kind == PL_AAD_HEATEX) {
        if (!h->fld[PL_BETA]) return fail(PL_ERR_STATE, "kind %d needs PL_BETA", kind);
        if ((r = ensure_cfield(h, PL_BETA))) return r;
        a.beta = h->cfld[2];
    }
    if (kind == PL_AD_FORCE && h->fld[PL_HEAT_SOURCE]) {
        if ((r = ensure_cfield(h, PL_HEAT_SOURCE))) return r;
        a.hsrc = h->cfld[13];
    }
    if (kind == PL_AAD_FORCE && h->fld[PL_OBJ_WEIGHT]) {
        if ((r = ensure_cfield(h, PL_OBJ_WEIGHT))) return r;
        a.objw = h->cfld[14];
    }
    if (kind == PL_AAD_MASSFLOW) {
        for (int f = PL_DIRX; f <= (h->nd == 3 ? PL_DIRZ : PL_DIRY); ++f) {
            if (!h->fld[f]) return fail(PL_ERR_STATE, "PL_AAD_MASSFLOW needs the direction fields");
            if ((r = ensure_cfield(h, f))) return r;
        }
        a.dirx = h->cfld[3]; a.diry = h->cfld[4]; a.dirz = h->cfld[5];
    }
    if (adjk && !elk) {
        for (int f = PL_FWD_RHO; f <= PL_FWD_TEM; ++f) {
            if (f == PL_FWD_UZ && h->nd == 2) continue;
            if (f == PL_FWD_TEM && (kind == PL_ANS_BRINKMAN || kind == PL_ANSIN_BRINKMAN)) continue;
            if (f == PL_FWD_RHO && kind == PL_ANSIN_BRINKMAN) continue;   // ANSin reads u only
            if (!h->fld[f]) return fail(PL_ERR_STATE, "adjoint kind %d needs the forward solution (pl_freeze_forward)", kind);
            if ((r = ensure_cfield(h, f))) return r;
            a.fwd[f - PL_FWD_RHO] = h->cfld[6 + f - PL_FWD_RHO];
        }
    }
    // macro outputs
    if (!adjk) {
        for (int m = 0; m < 8; ++m) { if ((r = ensure_d(h, &h->fwd[h->fwd_next][m], h->n))) return r; }
        if (save) for (int m = 0; m < 8; ++m) a.out[m] = h->fwd[h->fwd_next][m];
        a.bcu_out[0] = h->fwd[h->fwd_next][1]; a.bcu_out[1] = h->fwd[h->fwd_next][2]; a.bcu_out[2] = h->fwd[h->fwd_next][3];
    } else {
        for (int m = 0; m < 11; ++m) { if ((r = ensure_d(h, &h->adj[h->adj_next][m], h->n))) return r; }
        if (save) for (int m = 0; m < 11; ++m) a.out[m] = h->adj[h->adj_next][m];
    }
program:
    // boundary program
    if (prog >= 0) {
        if (prog >= (int)h->progs.size() || !h->progs[prog].valid) return fail(PL_ERR_ARG, "program %d invalid", prog);
        const Program &P = h->progs[prog];
        a.bnode = P.bnode; a.bstart = P.bstart; a.ops = P.ops; a.slot_of = P.slot_of; a.nb = P.nb;
        a.geo.face_mask = P.face_mask; a.geo.flags = P.flags;
        a.staged = P.staged ? 1 : 0;
        a.ns = P.ns; a.nt = P.nt;
        a.icode = P.staged ? P.icode : nullptr;
        a.irec = P.irec;
        if (pl::kind_inline_bc(kind) && kind_inputs) { a.ndir = P.ndir; a.dnode = P.dnode; a.dstart = P.dstart; a.dops = P.dops; }
        else { a.ndir = P.ndir_all; a.dnode = P.dnode_all; a.dstart = P.dstart_all; a.dops = P.dops_all; }
        a.snode = P.snode; a.sstart = P.sstart; a.sops = P.sops; a.tslot = P.tslot;
        a.sexpr = P.sexpr; a.troot = P.troot; a.tbuf = P.tbuf;
        a.side = h->side; a.side2 = h->side2; a.ev_fork = h->ev_fork; a.ev_join = h->ev_join; a.ev_join2 = h->ev_join2;
        // velocity read by AD/AAD ops
        if (!adjk) {
            const int s = bcu_slot >= 0 ? bcu_slot : 0;
            for (int m = 0; m < 3; ++m) { if ((r = ensure_d(h, &h->fwd[s][1 + m], h->n))) return r; }
            a.bcu[0] = h->fwd[s][1]; a.bcu[1] = h->fwd[s][2]; a.bcu[2] = h->fwd[s][3];
        } else {
            for (int f = PL_FWD_RHO; f <= PL_FWD_TEM; ++f) { if ((r = ensure_d(h, &h->fld[f], h->n))) return r; }
            a.bcu[0] = h->fld[PL_FWD_UX]; a.bcu[1] = h->fld[PL_FWD_UY]; a.bcu[2] = h->fld[PL_FWD_UZ];
            a.bcrho = h->fld[PL_FWD_RHO]; a.bctem = h->fld[PL_FWD_TEM];
        }
        if ((r = ensure_d(h, &h->fld[PL_KAPPA], h->n))) return r;
        a.bckappa = h->fld[PL_KAPPA];
    } else {
        a.slot_of = nullptr;
        a.nb = 0;
    }
    if (!a.slot_of) {
        // eval_node reads slot_of; give it an all -1 map
        if (!h->iscratch) {
            if ((r = dalloc((void **)&h->iscratch, sizeof(int) * h->n))) return r;
            CK(cudaMemsetAsync(h->iscratch, 0xff, sizeof(int) * h->n, h->st));
        }
        a.slot_of = h->iscratch;
    }
    return PL_OK;
}

void after_collide(pl_lattice h, int kind, bool save, int src, int prog, bool pull, int bcu_slot, const pl_phys *ph) {
    h->last_kind = kind; h->last_src = src; h->last_prog = prog; h->last_pull = pull ? 1 : 0;
    h->last_bcu_slot = bcu_slot;
    if (ph) h->last_ph = *ph;
    if (!pl::kind_is_adjoint(kind)) {
        h->fwd_latest = h->fwd_next;
        if (save) { h->fwd_prev_saved = h->fwd_saved; h->fwd_saved = h->fwd_next; }
        h->fwd_next ^= 1;
    } else {
        if (save) { h->adj_prev_saved = h->adj_saved; h->adj_saved = h->adj_next; }
        h->adj_next ^= 1;
    }
}

// a saving collide of a snapshot kind writes its snapshot itself when PL_OPT_SNAPSHOT_IN_STEP is set
int snapshot_target(pl_lattice h, int kind, bool save, double **out) {
    const int slot = pl::kind_is_adjoint(kind) ? 1 : 0;
    *out = nullptr;
    if (!(h->snap_in_step && save && pl::kind_has_snapshot(kind))) { h->snap_fresh[slot] = false; return PL_OK; }
    int r = ensure_d(h, &h->snap[slot], (size_t)h->q * h->np);
    if (r) return r;
    *out = h->snap[slot];
    return PL_OK;
}
void snapshot_taken(pl_lattice h, int kind, const double *snap) {
    const int slot = pl::kind_is_adjoint(kind) ? 1 : 0;
    h->snap_fresh[slot] = snap != nullptr;
    if (snap) h->snap_ok[slot] = true;
}

int do_collide(pl_lattice h, int kind, const pl_phys *ph, bool save) {
    if (int e = check_kind(h, kind)) return e;
    const bool adjk = pl::kind_is_adjoint(kind);
    if (!adjk) save = true;   // boundary ops of the next step read this velocity
    double *snap = nullptr;
    int r = snapshot_target(h, kind, save, &snap);
    if (r) return r;
    KArgs a;
    r = build_args(h, kind, ph, -1, h->cur, h->cur ^ 1, save, false, -1, a);
    if (r) return r;
    a.snap_coll = snap;
    if (h->launch(kind, pl::OP_COLLIDE, save, a, h->st)) return fail(PL_ERR_UNSUPPORTED, "kind %d not built for this storage", kind);
    if ((r = check_launch(h, 1))) return r;
    snapshot_taken(h, kind, snap);
    after_collide(h, kind, save, h->cur, -1, false, -1, ph);
    h->cur ^= 1;
    return PL_OK;
}

int do_step(pl_lattice h, int kind, const pl_phys *ph, int prog, bool save) {
    if (int e = check_kind(h, kind)) return e;
    const int bcu_slot = h->fwd_latest;
    double *snap = nullptr;
    int r = snapshot_target(h, kind, save, &snap);
    if (r) return r;
    KArgs a;
    r = build_args(h, kind, ph, prog, h->cur, h->cur ^ 1, save, true, bcu_slot, a);
    if (r) return r;
    a.snap_coll = snap;
    if (h->launch(kind, pl::OP_STEP, save, a, h->st)) return fail(PL_ERR_UNSUPPORTED, "kind %d not built for this storage", kind);
    if ((r = check_launch(h, a.nb > 0 ? (a.staged ? 1 + (a.ndir > 0) + (a.ns > 0 ? 2 : 0) : 2) : 1))) return r;
    snapshot_taken(h, kind, snap);
    after_collide(h, kind, save, h->cur, prog, true, bcu_slot, ph);
    h->cur ^= 1;
    return PL_OK;
}

int residual_family(pl_lattice h, int fam, double *out3, bool sync) {
    const bool adjk = fam >= 2;
    const int s = adjk ? h->adj_saved : h->fwd_saved, p = adjk ? h->adj_prev_saved : h->fwd_prev_saved;
    if (s < 0 || p < 0 || s == p) return fail(PL_ERR_STATE, "residual needs two saved collides");
    pl::ResidArgs ra;
    memset(&ra, 0, sizeof ra);
    ra.ncomp = h->nd;
    ra.n = h->n;
    for (int m = 0; m < h->nd; ++m) {
        int fi;
        if (fam == 0) fi = 1 + m; else if (fam == 1) fi = 5 + m; else if (fam == 2) fi = 1 + m; else fi = 8 + m;
        ra.a[m] = adjk ? h->adj[s][fi] : h->fwd[s][fi];
        ra.b[m] = adjk ? h->adj[p][fi] : h->fwd[p][fi];
    }
    const int nblk = pl::resid_blocks(h->n);
    pl::launch_residual(ra, h->partial, nblk, h->nonfinite, h->dout + 3 * (fam & 1), h->st);
    int r = check_launch(h, 2);
    if (r) return r;
    if (sync) {
        CK(cudaMemcpyAsync(out3, h->dout + 3 * (fam & 1), sizeof(double) * 3, cudaMemcpyDeviceToHost, h->st));
        CK(cudaStreamSynchronize(h->st));
    }
    return PL_OK;
}

int upload(pl_lattice h, double *dst, const double *host, size_t count) {
    CK(cudaMemcpyAsync(dst, host, sizeof(double) * count, cudaMemcpyHostToDevice, h->st));
    return PL_OK;
}
int download(pl_lattice h, double *host, const double *src, size_t count) {
    CK(cudaMemcpyAsync(host, src, sizeof(double) * count, cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    return PL_OK;
}

Taps *get_taps(pl_lattice h, double R) {
    long long key;
    memcpy(&key, &R, sizeof key);
    auto it = h->taps.find({h->nd, key});
    if (it != h->taps.end()) return &it->second;
    const int nR = (int)R;
    std::vector<int> di, dj, dk;
    std::vector<double> hat;
    for (int a = -nR; a <= nR; ++a)
        for (int b = -nR; b <= nR; ++b)
            for (int c = -nR; c <= nR; ++c) {
                const double dist = std::sqrt(std::pow((double)a, 2.0) + std::pow((double)b, 2.0) + std::pow((double)c, 2.0));
                if (dist > R) continue;
                if (h->nd == 2 && c != 0) continue;
                di.push_back(a); dj.push_back(b); dk.push_back(c);
                hat.push_back((R - dist) / R);
            }
    Taps t;
    t.ntap = (int)di.size();
    auto release = [&t]() {
        cudaFree(t.di); cudaFree(t.dj); cudaFree(t.dk); cudaFree(t.hat);
        return (Taps *)nullptr;
    };
    if (dalloc((void **)&t.di, sizeof(int) * t.ntap) || dalloc((void **)&t.dj, sizeof(int) * t.ntap) ||
        dalloc((void **)&t.dk, sizeof(int) * t.ntap) || dalloc((void **)&t.hat, sizeof(double) * t.ntap))
        return release();
    const cudaError_t e[4] = {
        cudaMemcpy(t.di, di.data(), sizeof(int) * t.ntap, cudaMemcpyHostToDevice),
        cudaMemcpy(t.dj, dj.data(), sizeof(int) * t.ntap, cudaMemcpyHostToDevice),
        cudaMemcpy(t.dk, dk.data(), sizeof(int) * t.ntap, cudaMemcpyHostToDevice),
        cudaMemcpy(t.hat, hat.data(), sizeof(double) * t.ntap, cudaMemcpyHostToDevice)};
    for (cudaError_t x : e)
        if (x != cudaSuccess) {
            fail(PL_ERR_CUDA, "filter taps upload: %s", cudaGetErrorString(x));
            return release();
        }
    return &(h->taps[{h->nd, key}] = t);
}

int scratch(pl_lattice h, int i, double **p) {
    int r = ensure_d(h, &h->scratch[i], h->n > 0 ? (size_t)h->n * (h->q) : 1);
    *p = h->scratch[i];
    return r;
}

}  // namespace

// ==================================================================================== C ABI
int pl::record_error(int code, const char *msg) { return fail(code, "%s", msg); }

int pl::lattice_sample_fields(pl_lattice h, const double **p, long long *n) {
    if (!h || !p || !n) return fail(PL_ERR_ARG, "bad arguments");
    static const int fwd[5] = {PL_FWD_RHO, PL_FWD_UX, PL_FWD_UY, PL_FWD_UZ, PL_FWD_TEM};
    for (int m = 0; m < 5; ++m) p[m] = h->fld[fwd[m]];
    static const int adj[8] = {0, 1, 2, 3, 7, 8, 9, 10};   // ip, iu, iT, iq in the adjoint macro planes
    for (int m = 0; m < 8; ++m) p[5 + m] = h->adj_saved >= 0 ? h->adj[h->adj_saved][adj[m]] : nullptr;
    if (!p[0] || !p[4]) return fail(PL_ERR_STATE, "no frozen forward solution (pl_freeze_forward)");
    if (h->adj_saved < 0) return fail(PL_ERR_STATE, "no saved adjoint collide");
    *n = h->n;
    return PL_OK;
}

cudaStream_t pl::lattice_stream(pl_lattice h) { return h ? h->st : nullptr; }

extern "C" {

const char *pl_last_error(void) { return g_err.c_str(); }

int pl_debug_fail_alloc(long long after) {
    g_fail_alloc_after.store(after < 0 ? -1 : after);
    return PL_OK;
}

int pl_create(int q, int nx, int ny, int nz, int storage, pl_lattice *out) {
    if (!out) return fail(PL_ERR_ARG, "out is NULL");
    *out = nullptr;
    if (q != 9 && q != 15) return fail(PL_ERR_ARG, "q must be 9 (D2Q9) or 15 (D3Q15), got %d", q);
    if (nx < 2 || ny < 2 || (q == 15 && nz < 2)) return fail(PL_ERR_ARG, "lattice %dx%dx%d too small", nx, ny, nz);
    if (storage < PL_FP64 || storage > PL_BF16) return fail(PL_ERR_ARG, "unknown storage %d", storage);
    const long long n = (long long)nx * ny * (q == 15 ? nz : 1);
    if (n > (1ll << 31) / 16) return fail(PL_ERR_ARG, "lattice of %lld nodes exceeds the 32-bit plane index", n);
    // the boundary kernel replays smoothing chains with nested calls (about 1.3 KB of stack per
    // thread); raise this context's per-thread stack limit when it is below that
    size_t stack = 0;
    if (cudaDeviceGetLimit(&stack, cudaLimitStackSize) == cudaSuccess && stack < 2048)
        cudaDeviceSetLimit(cudaLimitStackSize, 2048);
    cudaGetLastError();
    pl_lattice h = new pl_lattice_s();
    h->q = q; h->nd = q == 9 ? 2 : 3; h->nx = nx; h->ny = ny; h->nz = q == 9 ? 1 : nz; h->n = (int)n;
    h->np = (n + 63) / 64 * 64;
    h->storage = storage;
    h->fp32 = storage != PL_FP64;
    h->ssize = storage == PL_FP64 ? 8 : storage == PL_FP32 ? 4 : 2;
    h->csize = h->fp32 ? 4 : 8;
    h->launch = pick_launch(q, storage);
    h->aux = pick_aux(q, storage);
    int r = PL_OK;
    if (cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking) != cudaSuccess) {
        delete h;
        return fail(PL_ERR_CUDA, "cudaStreamCreate failed (no CUDA device?)");
    }
    h->own_stream = true;
    const size_t popbytes = h->ssize * (size_t)h->np * 2 * q;
    for (int b = 0; b < 2 && !r; ++b) r = dalloc(&h->pop[b], popbytes);
    if (!r) r = dalloc((void **)&h->partial, sizeof(double) * 2 * 1024);
    if (!r) r = dalloc((void **)&h->nonfinite, sizeof(int));
    if (!r) r = dalloc((void **)&h->err, sizeof(int));
    if (!r) r = dalloc((void **)&h->dout, sizeof(double) * 8);
    if (r) { pl_destroy(h); return r; }
    cudaMemsetAsync(h->pop[0], 0, popbytes, h->st);
    cudaMemsetAsync(h->pop[1], 0, popbytes, h->st);
    cudaMemsetAsync(h->nonfinite, 0, sizeof(int), h->st);
    cudaMemsetAsync(h->err, 0, sizeof(int), h->st);
    cudaEventCreate(&h->ev0);
    cudaEventCreate(&h->ev1);
    // boundary chains run on high-priority streams so their blocks are scheduled as soon as the
    // interior kernel frees resources, instead of after its last block has been dispatched
    int prio_lo = 0, prio_hi = 0;
    cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi);
    h->prio_lo = prio_lo;
    h->prio_hi = prio_hi;
    h->side_prio = prio_hi;
    cudaStreamCreateWithPriority(&h->side, cudaStreamNonBlocking, h->side_prio);
    cudaStreamCreateWithPriority(&h->side2, cudaStreamNonBlocking, h->side_prio);
    h->use_graphs = false;   // eager launches keep the side-stream priority (faster here)
    cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&h->ev_join2, cudaEventDisableTiming);
    if (cudaStreamSynchronize(h->st) != cudaSuccess) { pl_destroy(h); return fail(PL_ERR_CUDA, "init failed"); }
    *out = h;
    return PL_OK;
}

int pl_destroy(pl_lattice h) {
    if (!h) return PL_OK;
    if (h->st) cudaStreamSynchronize(h->st);
    for (auto &kv : h->graphs) cudaGraphExecDestroy(kv.second.exec);
    h->graphs.clear();
    for (auto &P : h->progs) free_program(P);
    for (auto &kv : h->taps) { cudaFree(kv.second.di); cudaFree(kv.second.dj); cudaFree(kv.second.dk); cudaFree(kv.second.hat); }
    cudaFree(h->pop[0]); cudaFree(h->pop[1]);
    for (auto *p : h->fld) cudaFree(p);
    for (auto *p : h->cfld) cudaFree(p);
    for (int s = 0; s < 2; ++s) { for (auto *p : h->fwd[s]) cudaFree(p); for (auto *p : h->adj[s]) cudaFree(p); cudaFree(h->snap[s]); }
    for (auto *p : h->scratch) cudaFree(p);
    cudaFree(h->iscratch); cudaFree(h->partial); cudaFree(h->nonfinite); cudaFree(h->err); cudaFree(h->dout);
    for (auto &v : h->store) for (void *p : v) cudaFree(p);
    cudaFree(h->sens_mask);
    cudaFree(h->wtab);
    if (h->ev0) cudaEventDestroy(h->ev0);
    if (h->ev1) cudaEventDestroy(h->ev1);
    if (h->side) { cudaStreamSynchronize(h->side); cudaStreamDestroy(h->side); }
    if (h->side2) { cudaStreamSynchronize(h->side2); cudaStreamDestroy(h->side2); }
    if (h->ev_fork) cudaEventDestroy(h->ev_fork);
    if (h->ev_join) cudaEventDestroy(h->ev_join);
    if (h->ev_join2) cudaEventDestroy(h->ev_join2);
    if (h->own_stream && h->st) cudaStreamDestroy(h->st);
    delete h;
    return PL_OK;
}

int pl_synchronize(pl_lattice h) {
    if (!h) return fail(PL_ERR_ARG, "null handle");
    CK(cudaStreamSynchronize(h->st));
    int err = 0;
    CK(cudaMemcpy(&err, h->err, sizeof(int), cudaMemcpyDeviceToHost));
    if (err) return fail(PL_ERR_STATE, "device reported error bits 0x%x (boundary program too deep)", err);
    return PL_OK;
}

int pl_set_stream(pl_lattice h, void *stream) {
    if (!h) return fail(PL_ERR_ARG, "null handle");
    CK(cudaStreamSynchronize(h->st));
    if (h->own_stream) cudaStreamDestroy(h->st);
    h->st = static_cast<cudaStream_t>(stream);
    h->own_stream = false;
    return PL_OK;
}

int pl_set_option(pl_lattice h, int option, int value) {
    if (!h) return fail(PL_ERR_ARG, "null handle");
    if (value != 0 && value != 1) return fail(PL_ERR_ARG, "option value must be 0 or 1");
    if (option == PL_OPT_GRAPHS) {
        h->use_graphs = value == 1;
        return PL_OK;
    }
    if (option == PL_OPT_SNAPSHOT_IN_STEP) {
        h->snap_in_step = value == 1;
        return PL_OK;
    }
    if (option == PL_OPT_STOCHASTIC_ROUNDING) {
        h->sr = value == 1;
        for (auto &kv : h->graphs) cudaGraphExecDestroy(kv.second.exec);
        h->graphs.clear();
        return PL_OK;
    }
    if (option == PL_OPT_SIDE_PRIORITY) {
        const int prio = value ? h->prio_hi : h->prio_lo;
        if (prio == h->side_prio) return PL_OK;
        CK(cudaStreamSynchronize(h->st));
        CK(cudaStreamSynchronize(h->side));
        CK(cudaStreamSynchronize(h->side2));
        cudaStreamDestroy(h->side);
        cudaStreamDestroy(h->side2);
        h->side = h->side2 = nullptr;
        CK(cudaStreamCreateWithPriority(&h->side, cudaStreamNonBlocking, prio));
        CK(cudaStreamCreateWithPriority(&h->side2, cudaStreamNonBlocking, prio));
        h->side_prio = prio;
        for (auto &kv : h->graphs) cudaGraphExecDestroy(kv.second.exec);
        h->graphs.clear();
        return PL_OK;
    }
    return fail(PL_ERR_ARG, "unknown option");
}

int pl_set_inflow_scale(pl_lattice h, double s) {
    if (!h || !std::isfinite(s)) return fail(PL_ERR_ARG, "bad arguments");
    h->uscale = s;
    return PL_OK;
}

int pl_set_shift(pl_lattice h, double sf, double sg) {
    if (!h) return fail(PL_ERR_ARG, "null handle");
    h->shift_f = sf;
    h->shift_g = sg;
    return PL_OK;
}

int pl_set_populations(pl_lattice h, int set, const double *host) {
    if (!h || !host || (set != 0 && set != 1)) return fail(PL_ERR_ARG, "bad arguments");
    double *buf;
    int r = scratch(h, 0, &buf);
    if (r) return r;
    if ((r = upload(h, buf, host, (size_t)h->q * h->n))) return r;
    KArgs a;
    memset(&a, 0, sizeof a);
    a.geo.n = h->n; a.geo.np = h->np; a.dst = h->pop[h->cur];
    h->aux(pl::AUX_ENCODE, a, 0, nullptr, 0, 0, buf, set, set ? h->shift_g : h->shift_f, h->st);
    return check_launch(h, 1);
}

int pl_get_populations(pl_lattice h, int set, double *host) {
    if (!h || !host || (set != 0 && set != 1)) return fail(PL_ERR_ARG, "bad arguments");
    double *buf;
    int r = scratch(h, 0, &buf);
    if (r) return r;
    KArgs a;
    memset(&a, 0, sizeof a);
    a.geo.n = h->n; a.geo.np = h->np; a.src = h->pop[h->cur];
    h->aux(pl::AUX_DECODE, a, 0, nullptr, 0, 0, buf, set, set ? h->shift_g : h->shift_f, h->st);
    if ((r = check_launch(h, 1))) return r;
    return download(h, host, buf, (size_t)h->q * h->n);
}

int pl_set_field(pl_lattice h, int f, const double *host) {
    PL_RANGE("pl_set_field");
    if (h && !host && (f == PL_HEAT_SOURCE || f == PL_OBJ_WEIGHT)) {
        // switch the source term off: queued launches keep their pointers, so free in order
        CK(cudaStreamSynchronize(h->st));
        const int ci = field_index_c(f);
        cudaFree(h->fld[f]); h->fld[f] = nullptr;
        cudaFree(h->cfld[ci]); h->cfld[ci] = nullptr;
        return PL_OK;
    }
    if (!h || !host) return fail(PL_ERR_ARG, "bad arguments");
    int r;
    if ((f >= PL_ALPHA && f <= PL_GAMMA) || (f >= PL_FWD_RHO && f <= PL_OBJ_WEIGHT)) {
        if (f == PL_KAPPA) {
            // a diffusivity <= 0 gives a relaxation rate 1/(3 kappa + 1/2) >= 2: the AD collide
            // is then unstable, so refuse it before it reaches the device
            for (int i = 0; i < h->n; ++i)
                if (!(host[i] > 0.0) || !std::isfinite(host[i]))
                    return fail(PL_ERR_ARG, "PL_KAPPA[%d] = %g: the diffusivity must be finite and > 0", i, host[i]);
        }
        if ((r = ensure_d(h, &h->fld[f], h->n))) return r;
        if ((r = upload(h, h->fld[f], host, h->n))) return r;
        return sync_cfield(h, f);
    }
    if (f >= PL_RHO && f <= PL_QZ) {
        int s = h->fwd_saved >= 0 ? h->fwd_saved : 0;
        if ((r = ensure_d(h, &h->fwd[s][f - PL_RHO], h->n))) return r;
        if (h->fwd_saved < 0) { h->fwd_saved = s; h->fwd_latest = s; h->fwd_next = s ^ 1; }
        return upload(h, h->fwd[s][f - PL_RHO], host, h->n);
    }
    if (f >= PL_IP && f <= PL_IQZ) {
        int s = h->adj_saved >= 0 ? h->adj_saved : 0;
        if ((r = ensure_d(h, &h->adj[s][f - PL_IP], h->n))) return r;
        if (h->adj_saved < 0) { h->adj_saved = s; h->adj_next = s ^ 1; }
        return upload(h, h->adj[s][f - PL_IP], host, h->n);
    }
    return fail(PL_ERR_ARG, "unknown field %d", f);
}

int pl_get_field(pl_lattice h, int f, double *host) {
    PL_RANGE("pl_get_field");
    if (!h || !host) return fail(PL_ERR_ARG, "bad arguments");
    const double *src = nullptr;
    if ((f >= PL_ALPHA && f <= PL_GAMMA) || (f >= PL_FWD_RHO && f <= PL_OBJ_WEIGHT)) src = h->fld[f];
    else if (f >= PL_RHO && f <= PL_QZ) src = h->fwd_saved >= 0 ? h->fwd[h->fwd_saved][f - PL_RHO] : nullptr;
    else if (f >= PL_IP && f <= PL_IQZ) src = h->adj_saved >= 0 ? h->adj[h->adj_saved][f - PL_IP] : nullptr;
    else return fail(PL_ERR_ARG, "unknown field %d", f);
    if (!src) return fail(PL_ERR_STATE, "field %d has no value yet", f);
    return download(h, host, src, h->n);
}

int pl_get_saved_field(pl_lattice h, int f, int age, double *host) {
    PL_RANGE("pl_get_saved_field");
    if (!h || !host || (age != 0 && age != 1)) return fail(PL_ERR_ARG, "bad arguments");
    const double *src = nullptr;
    if (f >= PL_RHO && f <= PL_QZ) {
        const int s = age == 0 ? h->fwd_saved : h->fwd_prev_saved;
        src = s >= 0 ? h->fwd[s][f - PL_RHO] : nullptr;
    } else if (f >= PL_IP && f <= PL_IQZ) {
        const int s = age == 0 ? h->adj_saved : h->adj_prev_saved;
        src = s >= 0 ? h->adj[s][f - PL_IP] : nullptr;
    } else {
        return fail(PL_ERR_ARG, "field %d is not a saved macroscopic field", f);
    }
    if (!src) return fail(PL_ERR_STATE, "no save of age %d holds field %d", age, f);
    return download(h, host, src, h->n);
}

int pl_freeze_forward(pl_lattice h) {
    if (!h) return fail(PL_ERR_ARG, "null handle");
    if (h->fwd_saved < 0) return fail(PL_ERR_STATE, "no saved forward collide");
    static const int map[5] = {0, 1, 2, 3, 4};
    int r;
    for (int m = 0; m < 5; ++m) {
        const int f = PL_FWD_RHO + m;
        if ((r = ensure_d(h, &h->fld[f], h->n))) return r;
        const double *src = h->fwd[h->fwd_saved][map[m]];
        if (!src) continue;
        CK(cudaMemcpyAsync(h->fld[f], src, sizeof(double) * h->n, cudaMemcpyDeviceToDevice, h->st));
        if ((r = sync_cfield(h, f))) return r;
    }
    return PL_OK;
}

int pl_program_create(pl_lattice h, const pl_bc_desc *descs, int n, int *prog) {
    PL_RANGE("pl_program_create");
    if (!h || (!descs && n) || !prog) return fail(PL_ERR_ARG, "bad arguments");
    Program P;
    int r = compile_program(h, descs, n, P);
    if (r) { free_program(P); return r; }
    h->progs.push_back(P);
    *prog = (int)h->progs.size() - 1;
    return PL_OK;
}

int pl_program_destroy(pl_lattice h, int prog) {
    if (!h || prog < 0 || prog >= (int)h->progs.size()) return fail(PL_ERR_ARG, "bad program");
    cudaStreamSynchronize(h->st);
    for (auto it = h->graphs.begin(); it != h->graphs.end();) {
        if (it->first.prog == prog) { cudaGraphExecDestroy(it->second.exec); it = h->graphs.erase(it); }
        else ++it;
    }
    free_program(h->progs[prog]);
    return PL_OK;
}

int pl_init(pl_lattice h, int which, const double *a0, const double *a1, const double *a2, const double *a3,
            const double *ux, const double *uy, const double *uz) {
    PL_RANGE("pl_init");
    const bool adj_seed = which == 2 || which == 3;
    if (!h || which < 0 || which > 5 || (!a0 && !adj_seed)) return fail(PL_ERR_ARG, "bad arguments");
    if (which >= 4 && h->nd != 2) return fail(PL_ERR_UNSUPPORTED, "init %d is D2Q9 only", which);
    // the adjoint seeds may take the frozen forward velocity on the device (ux == NULL) and a zero
    // adjoint state (a0..a3 == NULL), so that an adjoint solve starts without host traffic
    const bool dev_u = adj_seed && !ux && !uy && !uz;
    if (dev_u && (!h->fld[PL_FWD_UX] || !h->fld[PL_FWD_UY] || (h->nd == 3 && !h->fld[PL_FWD_UZ])))
        return fail(PL_ERR_STATE, "init %d without a velocity needs the frozen forward solution", which);
    if (which != 5 && !dev_u && (!ux || !uy || (h->nd == 3 && !uz))) return fail(PL_ERR_ARG, "init %d needs the velocity", which);
    if (which == 5 && (!a1 || !a2)) return fail(PL_ERR_ARG, "adjoint init needs a1..a3");
    if (adj_seed && a0 && (!a1 || !a2 || (h->nd == 3 && !a3))) return fail(PL_ERR_ARG, "adjoint init needs a1..a3");
    double *buf;
    int r = scratch(h, 1, &buf);   // q*N doubles >= 7*N
    if (r) return r;
    const double *hs[7] = {a0, a1, a2, a3, ux, uy, uz};
    const double *in[7];
    for (int m = 0; m < 7; ++m) {
        double *d = buf + (size_t)m * h->n;
        in[m] = d;
        if (dev_u && m >= 4 && m - 4 < h->nd) {
            in[m] = h->fld[PL_FWD_UX + (m - 4)];   // device-resident forward velocity
            continue;
        }
        if (hs[m] && (m < 4 || m - 4 < h->nd)) { if ((r = upload(h, d, hs[m], h->n))) return r; }
        else { CK(cudaMemsetAsync(d, 0, sizeof(double) * h->n, h->st)); }
    }
    KArgs a;
    memset(&a, 0, sizeof a);
    a.geo.n = h->n; a.geo.np = h->np; a.dst = h->pop[h->cur];
    a.ph.shift_f = h->shift_f; a.ph.shift_g = h->shift_g;
    h->aux(pl::AUX_INIT, a, which, in, 0, 0, nullptr, 0, 0.0, h->st);
    if ((r = check_launch(h, 1))) return r;
    return pl_synchronize(h);
}

int pl_init_elastic(pl_lattice h, int which, const double *const *in) {
    if (!h || !in || (which != 0 && which != 1)) return fail(PL_ERR_ARG, "bad arguments");
    if (h->nd != 2) return fail(PL_ERR_UNSUPPORTED, "the elastic initial conditions are D2Q9 only");
    for (int m = 0; m < 7; ++m)
        if (!in[m]) return fail(PL_ERR_ARG, "elastic init needs seven arrays (array %d is NULL)", m);
    int r;
    KArgs a;
    memset(&a, 0, sizeof a);
    if (which == 1) {
        if (!h->fld[PL_GAMMA]) return fail(PL_ERR_STATE, "AEL init needs PL_GAMMA");
        if ((r = ensure_cfield(h, PL_GAMMA))) return r;
        a.gamma = h->cfld[12];
    }
    double *buf;
    if ((r = scratch(h, 1, &buf))) return r;   // q*N doubles >= 7*N
    // kernel slots (in0, in1, in2, in3, ux, uy, uz) <- (rho | irho, s.., u | im, s..)
    static const int slot_of_input[7] = {0, 4, 5, 1, 2, 3, 6};
    const double *dev[7];
    for (int m = 0; m < 7; ++m) {
        double *d = buf + (size_t)slot_of_input[m] * h->n;
        if ((r = upload(h, d, in[m], h->n))) return r;
        dev[slot_of_input[m]] = d;
    }
    a.geo.n = h->n; a.geo.np = h->np; a.dst = h->pop[h->cur];
    a.ph.shift_f = h->shift_f; a.ph.shift_g = h->shift_g;
    h->aux(pl::AUX_INIT, a, 6 + which, dev, 0, 0, nullptr, 0, 0.0, h->st);
    if ((r = check_launch(h, 1))) return r;
    return pl_synchronize(h);
}

int pl_collide(pl_lattice h, int kind, const pl_phys *ph, int save) {
    PL_RANGE("pl_collide");
    if (!h || !ph) return fail(PL_ERR_ARG, "bad arguments");
    return do_collide(h, kind, ph, save != 0);
}

int pl_step(pl_lattice h, int kind, const pl_phys *ph, int prog, int save) {
    PL_RANGE("pl_step");
    if (!h || !ph) return fail(PL_ERR_ARG, "bad arguments");
    return do_step(h, kind, ph, prog, save != 0);
}

static int run_steps(pl_lattice h, int kind, const pl_phys *ph, int prog, int n) {
    int r;
    // n fused steps without saves. Two steps return every buffer and slot to its parity, so
    // they are captured once into a CUDA graph and replayed (no per-kernel host launch cost).
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(h->st, &cs);
    const bool graphs = h->use_graphs && h->st != nullptr && cs == cudaStreamCaptureStatusNone && n >= 4;
    int done = 0;
    if (graphs) {
        pl_lattice_s::GraphKey key;
        memset(&key, 0, sizeof key);
        key.kind = kind; key.prog = prog; key.ph = *ph;
        key.hsrc = kind == PL_AD_FORCE ? h->fld[PL_HEAT_SOURCE] : nullptr;
        key.objw = kind == PL_AAD_FORCE ? h->fld[PL_OBJ_WEIGHT] : nullptr;
        key.uscale = h->uscale;
        for (int warm = 0; warm < 2; ++warm) {   // settle allocations and parity before capture
            key.cur = h->cur; key.fwd_next = h->fwd_next; key.adj_next = h->adj_next; key.fwd_latest = h->fwd_latest;
            if (h->graphs.count(key)) break;
            if ((r = do_step(h, kind, ph, prog, false))) return r;
            ++done;
        }
        key.cur = h->cur; key.fwd_next = h->fwd_next; key.adj_next = h->adj_next; key.fwd_latest = h->fwd_latest;
        auto it = h->graphs.find(key);
        if (it == h->graphs.end()) {
            const long long l0 = h->launches;
            cudaGraph_t g = nullptr;
            CK(cudaStreamBeginCapture(h->st, cudaStreamCaptureModeRelaxed));
            int rr = do_step(h, kind, ph, prog, false);
            if (!rr) rr = do_step(h, kind, ph, prog, false);
            cudaError_t e = cudaStreamEndCapture(h->st, &g);
            if (rr) { if (g) cudaGraphDestroy(g); return rr; }
            if (e != cudaSuccess) return fail(PL_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
            // stream priority is not part of a captured launch: give the boundary-chain kernel
            // nodes (every kernel smaller than the full-lattice grid) the side streams' priority
            size_t nn = 0;
            cudaGraphGetNodes(g, nullptr, &nn);
            std::vector<cudaGraphNode_t> nodes(nn);
            if (nn) cudaGraphGetNodes(g, nodes.data(), &nn);
            for (auto nd_ : nodes) {
                cudaGraphNodeType ty;
                if (cudaGraphNodeGetType(nd_, &ty) != cudaSuccess || ty != cudaGraphNodeTypeKernel) continue;
                cudaKernelNodeParams kp;
                if (cudaGraphKernelNodeGetParams(nd_, &kp) != cudaSuccess) continue;
                const long long threads = (long long)kp.gridDim.x * kp.blockDim.x;
                if (threads >= h->n) continue;
                cudaKernelNodeAttrValue v;
                memset(&v, 0, sizeof v);
                v.priority = h->side_prio;
                cudaGraphKernelNodeSetAttribute(nd_, cudaKernelNodeAttributePriority, &v);
            }
            cudaGetLastError();
            cudaGraphExec_t ex = nullptr;
            e = cudaGraphInstantiate(&ex, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) return fail(PL_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
            const long long per = h->launches - l0;
            h->launches = l0;   // captured, not launched: the replays below count them
            it = h->graphs.emplace(key, pl_lattice_s::GraphEntry{ex, per}).first;
            // the capture advanced the host state by one period; this first replay runs it
            CK(cudaGraphLaunch(ex, h->st));
            h->launches += per;
            done += 2;
        }
        while (n - done >= 2) {
            CK(cudaGraphLaunch(it->second.exec, h->st));
            h->launches += it->second.launches;
            done += 2;
        }
    }
    for (; done < n; ++done) {
        if ((r = do_step(h, kind, ph, prog, false))) return r;
    }
    return PL_OK;
}

int pl_steps(pl_lattice h, int kind, const pl_phys *ph, int prog, int n) {
    PL_RANGE("pl_steps");
    if (!h || !ph || n < 0) return fail(PL_ERR_ARG, "bad arguments");
    if (int e = check_kind(h, kind)) return e;
    CK(cudaEventRecord(h->ev0, h->st));
    int r = run_steps(h, kind, ph, prog, n);
    if (r) return r;
    CK(cudaEventRecord(h->ev1, h->st));
    return PL_OK;
}

int pl_stream(pl_lattice h, int mode, int prog, int both_sets) {
    PL_RANGE("pl_stream");
    if (!h || mode < 0 || mode > 3) return fail(PL_ERR_ARG, "bad arguments");
    const bool inverse = mode == 1, nopull = mode >= 2, adjin = mode == 1 || mode == 3;
    KArgs a;
    int r = build_args(h, adjin ? PL_ANS_BRINKMAN : PL_NS_COLLIDE, nullptr, prog, h->cur, h->cur ^ 1, false, !nopull,
                       h->fwd_latest, a, false);
    if (r) return r;
    // a staged program streams through the fused step's split (inline ops in the pull kernel,
    // side chains for the other boundary nodes): the direct set is then the non-inline nodes
    const bool split = prog >= 0 && a.staged && a.icode && !nopull && both_sets && a.nb > 0;
    if (split) {
        const Program &P = h->progs[prog];
        a.ndir = P.ndir; a.dnode = P.dnode; a.dstart = P.dstart; a.dops = P.dops;
    }
    h->aux(pl::AUX_STREAM_PROGRAM, a, 0, nullptr, both_sets, inverse ? 1 : -1, nullptr, 0, 0.0, h->st);
    if ((r = check_launch(h, split ? 1 + (a.ndir > 0) + (a.ns > 0 ? 2 : 0) : 1))) return r;
    h->cur ^= 1;
    h->last_kind = -1;
    return PL_OK;
}

int pl_solve(pl_lattice h, int kind, const pl_phys *ph, int prog, int max_steps, int check_every, double tol,
             int *status, int *steps, double *res) {
    PL_RANGE("pl_solve");
    if (!h || !ph || max_steps < 1 || check_every < 1 || !status || !steps) return fail(PL_ERR_ARG, "bad arguments");
    const bool adjk = pl::kind_is_adjoint(kind);
    const int fa = adjk ? 2 : 0, fb = adjk ? 3 : 1;
    const bool has_g = pl::kind_has_g(kind);
    *status = PL_MAX_STEPS;
    *steps = max_steps;
    double r0[3] = {0, 0, 0}, r1[3] = {0, 0, 0};
    CK(cudaMemsetAsync(h->nonfinite, 0, sizeof(int), h->st));
    CK(cudaEventRecord(h->ev0, h->st));
    int r;
    auto is_save = [&](int t) {
        return (t % check_every == 0) || (t % check_every == check_every - 1) || check_every == 1;
    };
    for (int t = 1; t <= max_steps; ++t) {
        const bool save = is_save(t);
        if (t == 1) r = do_collide(h, kind, ph, true);
        else if (!save && h->use_graphs) {
            // the steps up to the next saving one replay the captured two-step graph
            int t1 = t;
            while (t1 < max_steps && !is_save(t1 + 1)) ++t1;
            r = run_steps(h, kind, ph, prog, t1 - t + 1);
            t = t1;
        } else r = do_step(h, kind, ph, prog, save);
        if (r) return r;
        if (t % check_every == 0 && t > 1) {
            if ((r = residual_family(h, fa, r0, false))) return r;
            if (has_g && (r = residual_family(h, fb, r1, false))) return r;
            double outv[6];
            int bad = 0;
            CK(cudaMemcpyAsync(outv, h->dout, sizeof(double) * 6, cudaMemcpyDeviceToHost, h->st));
            CK(cudaMemcpyAsync(&bad, h->nonfinite, sizeof(int), cudaMemcpyDeviceToHost, h->st));
            CK(cudaStreamSynchronize(h->st));
            r0[2] = outv[2];
            r1[2] = has_g ? outv[5] : 0.0;
            if (bad || !std::isfinite(r0[2]) || (has_g && !std::isfinite(r1[2]))) {
                *status = PL_DIVERGED;
                *steps = t;
                break;
            }
            if (r0[2] < tol && (!has_g || r1[2] < tol)) {
                *status = PL_CONVERGED;
                *steps = t;
                break;
            }
        }
    }
    CK(cudaEventRecord(h->ev1, h->st));
    CK(cudaEventSynchronize(h->ev1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, h->ev0, h->ev1);
    h->last_ms = ms;
    if (res) { res[0] = r0[2]; res[1] = r1[2]; }
    return pl_synchronize(h);
}

int pl_snapshot(pl_lattice h, int slot, double *host) {
    PL_RANGE("pl_snapshot");
    if (!h || (slot != 0 && slot != 1)) return fail(PL_ERR_ARG, "bad arguments");
    if (h->last_kind < 0) return fail(PL_ERR_STATE, "no collide to take a snapshot of");
    if (pl::kind_is_adjoint(h->last_kind) != (slot == 1)) return fail(PL_ERR_STATE, "last collide does not match slot %d", slot);
    if (!pl::kind_has_snapshot(h->last_kind)) return fail(PL_ERR_STATE, "kind %d stores no snapshot", h->last_kind);
    int r = ensure_d(h, &h->snap[slot], (size_t)h->q * h->np);
    if (r) return r;
    if (h->snap_fresh[slot]) goto taken;   // the last collide wrote it (PL_OPT_SNAPSHOT_IN_STEP)
    {
    // the last collide read population buffer last_src; re-evaluate its input state
    const int saved_next = pl::kind_is_adjoint(h->last_kind) ? h->adj_next : h->fwd_next;
    KArgs a;
    r = build_args(h, h->last_kind, &h->last_ph, h->last_prog, h->last_src, -1, false, h->last_pull != 0,
                   h->last_bcu_slot, a);
    (void)saved_next;
    if (r) return r;
    if (h->last_prog < 0) a.pull = 0;
    a.snap = h->snap[slot];
    if (h->launch(h->last_kind, pl::OP_SNAPSHOT, false, a, h->st)) return fail(PL_ERR_UNSUPPORTED, "snapshot kind");
    if ((r = check_launch(h, 1))) return r;
    }
taken:
    h->snap_ok[slot] = true;
    if (host) {
        double *buf;
        if ((r = scratch(h, 2, &buf))) return r;
        pl::launch_snap_to_node_major(h->snap[slot], h->np, h->n, h->q, buf, h->st);
        if ((r = check_launch(h, 1))) return r;
        return download(h, host, buf, (size_t)h->q * h->n);
    }
    return PL_OK;
}

int pl_set_snapshot(pl_lattice h, int slot, const double *host) {
    if (!h || !host || (slot != 0 && slot != 1)) return fail(PL_ERR_ARG, "bad arguments");
    int r = ensure_d(h, &h->snap[slot], (size_t)h->q * h->np);
    if (r) return r;
    double *buf;
    if ((r = scratch(h, 2, &buf))) return r;
    if ((r = upload(h, buf, host, (size_t)h->q * h->n))) return r;
    pl::launch_node_major_to_snap(buf, h->np, h->n, h->q, h->snap[slot], h->st);
    h->snap_ok[slot] = true;
    h->snap_fresh[slot] = false;
    return check_launch(h, 1);
}

int pl_residual(pl_lattice h, int family, double *out) {
    PL_RANGE("pl_residual");
    if (!h || !out || family < 0 || family > 3) return fail(PL_ERR_ARG, "bad arguments");
    double o[3];
    int r = residual_family(h, family, o, true);
    if (r) return r;
    *out = o[2];
    return PL_OK;
}

int pl_residual_host(pl_lattice h, int n, int ncomp, const double *const *a, const double *const *b, double *out) {
    PL_RANGE("pl_residual_host");
    if (!h || !a || !b || !out || ncomp < 1 || ncomp > 3 || n < 1 || n > h->n * h->q / 6) return fail(PL_ERR_ARG, "bad arguments");
    double *buf;
    int r = scratch(h, 3, &buf);
    if (r) return r;
    pl::ResidArgs ra;
    memset(&ra, 0, sizeof ra);
    ra.ncomp = ncomp;
    ra.n = n;
    for (int m = 0; m < ncomp; ++m) {
        double *da = buf + (size_t)(2 * m) * n, *db = buf + (size_t)(2 * m + 1) * n;
        if ((r = upload(h, da, a[m], n)) || (r = upload(h, db, b[m], n))) return r;
        ra.a[m] = da;
        ra.b[m] = db;
    }
    CK(cudaMemsetAsync(h->nonfinite, 0, sizeof(int), h->st));
    pl::launch_residual(ra, h->partial, pl::resid_blocks(n), h->nonfinite, h->dout, h->st);
    if ((r = check_launch(h, 2))) return r;
    double o[3];
    if ((r = download(h, o, h->dout, 3))) return r;
    *out = o[2];
    return PL_OK;
}

int pl_sensitivity(pl_lattice h, int which, double *dfds, const double *dads, const double *dkds, const double *qn,
                   const int *mask) {
    PL_RANGE("pl_sensitivity");
    if (!h || !dfds || !dads || which < 0 || which > 3) return fail(PL_ERR_ARG, "bad arguments");
    if ((which <= 2 && !dkds) || (which == 0 && (!qn || !mask))) return fail(PL_ERR_ARG, "missing dkds / qn / mask");
    if (h->adj_saved < 0) return fail(PL_ERR_STATE, "no saved adjoint collide");
    if (which <= 1 && (!h->snap_ok[0] || !h->snap_ok[1])) return fail(PL_ERR_STATE, "take both snapshots (pl_snapshot) first");
    for (int f = PL_FWD_RHO; f <= PL_FWD_TEM; ++f)
        if (!h->fld[f]) return fail(PL_ERR_STATE, "forward solution not set (pl_freeze_forward)");
    double *buf;
    int r = scratch(h, 4, &buf);   // q*N >= 5*N
    if (r) return r;
    double *d_dfds = buf, *d_dads = buf + h->n, *d_dkds = buf + 2 * (size_t)h->n, *d_qn = buf + 3 * (size_t)h->n;
    int *d_mask = reinterpret_cast<int *>(buf + 4 * (size_t)h->n);
    if ((r = upload(h, d_dfds, dfds, h->n)) || (r = upload(h, d_dads, dads, h->n))) return r;
    if (dkds && (r = upload(h, d_dkds, dkds, h->n))) return r;
    if (qn && (r = upload(h, d_qn, qn, h->n))) return r;
    if (mask) CK(cudaMemcpyAsync(d_mask, mask, sizeof(int) * h->n, cudaMemcpyHostToDevice, h->st));
    if ((r = ensure_d(h, &h->fld[PL_KAPPA], h->n))) return r;
    pl::SensArgs s;
    memset(&s, 0, sizeof s);
    s.which = which; s.n = h->n; s.nx = h->nx; s.ny = h->ny; s.nz = h->nz; s.np = h->np;
    s.dfds = d_dfds; s.dads = d_dads; s.dkds = d_dkds; s.qn = d_qn; s.mask = d_mask;
    s.ux = h->fld[PL_FWD_UX]; s.uy = h->fld[PL_FWD_UY]; s.uz = h->fld[PL_FWD_UZ]; s.tem = h->fld[PL_FWD_TEM];
    const int sa = h->adj_saved;
    s.imx = h->adj[sa][4]; s.imy = h->adj[sa][5]; s.imz = h->adj[sa][6];
    s.item = h->adj[sa][7]; s.iqx = h->adj[sa][8]; s.iqy = h->adj[sa][9]; s.iqz = h->adj[sa][10];
    s.kappa = h->fld[PL_KAPPA];
    s.g = h->snap[0]; s.ig = h->snap[1];
    pl::launch_sensitivity(h->q, s, h->st);
    if ((r = check_launch(h, 1))) return r;
    return download(h, dfds, d_dfds, h->n);
}

int pl_sensitivity_compliance(pl_lattice h, double *dfds, const double *const *in) {
    if (!h || !dfds) return fail(PL_ERR_ARG, "bad arguments");
    if (h->nd != 2) return fail(PL_ERR_UNSUPPORTED, "the compliance sensitivity is D2Q9 only");
    double *buf;
    int r = scratch(h, 4, &buf);   // q*N = 9*N: dfds + up to 8 inputs; the ninth in scratch 5
    if (r) return r;
    double *sc5;
    if ((r = scratch(h, 5, &sc5))) return r;
    const double *dev[9];
    if (in) {
        for (int m = 0; m < 9; ++m) {
            if (!in[m]) return fail(PL_ERR_ARG, "compliance sensitivity input %d is NULL", m);
            double *d = m < 8 ? buf + (size_t)(m + 1) * h->n : sc5;
            if ((r = upload(h, d, in[m], h->n))) return r;
            dev[m] = d;
        }
    } else {
        // the stress of the last saving EL collide and the adjoint of the last saving AEL collide
        if (h->fwd_saved < 0 || h->adj_saved < 0) return fail(PL_ERR_STATE, "no saved EL / AEL collide");
        const int fs = h->fwd_saved, as = h->adj_saved;
        static const int adj_plane[5] = {0, 7, 8, 9, 10};
        for (int m = 0; m < 4; ++m) dev[m] = h->fwd[fs][4 + m];
        for (int m = 0; m < 5; ++m) dev[4 + m] = h->adj[as][adj_plane[m]];
        for (int m = 0; m < 9; ++m)
            if (!dev[m]) return fail(PL_ERR_STATE, "saved EL / AEL macros missing");
    }
    if ((r = upload(h, buf, dfds, h->n))) return r;
    pl::launch_compliance(h->n, buf, dev, h->st);
    if ((r = check_launch(h, 1))) return r;
    return download(h, dfds, buf, h->n);
}

// ---- checkpointed sweeps --------------------------------------------------------------------
constexpr int kMaxStoreSlots = 1 << 16;   // per kind; a slot is a whole-lattice buffer
static size_t store_bytes(pl_lattice h, int what) {
    if (what == PL_STORE_POPS) return (size_t)2 * h->q * h->np * h->ssize;
    if (what == PL_STORE_FWD) return sizeof(double) * 5 * (size_t)h->n;
    return sizeof(double) * (size_t)h->q * h->np;
}

int pl_store(pl_lattice h, int what, int slot) {
    PL_RANGE("pl_store");
    if (!h || what < PL_STORE_POPS || what > PL_STORE_SNAP || slot < 0 || slot >= kMaxStoreSlots)
        return fail(PL_ERR_ARG, "bad arguments (slot %d of at most %d)", slot, kMaxStoreSlots);
    std::vector<void *> &v = h->store[what];
    if ((int)v.size() <= slot) v.resize(slot + 1, nullptr);
    int r;
    const size_t bytes = store_bytes(h, what);
    if (!v[slot] && (r = dalloc(&v[slot], bytes))) return r;
    char *dst = static_cast<char *>(v[slot]);
    if (what == PL_STORE_POPS) {
        CK(cudaMemcpyAsync(dst, h->pop[h->cur], bytes, cudaMemcpyDeviceToDevice, h->st));
    } else if (what == PL_STORE_FWD) {
        if (h->fwd_saved < 0) return fail(PL_ERR_STATE, "no saved forward collide");
        for (int m = 0; m < 5; ++m) {
            const double *src = h->fwd[h->fwd_saved][m];
            double *d = reinterpret_cast<double *>(dst) + (size_t)m * h->n;
            if (src) { CK(cudaMemcpyAsync(d, src, sizeof(double) * h->n, cudaMemcpyDeviceToDevice, h->st)); }
            else { CK(cudaMemsetAsync(d, 0, sizeof(double) * h->n, h->st)); }
        }
    } else {
        if (!h->snap_ok[0]) return fail(PL_ERR_STATE, "no forward snapshot (pl_snapshot slot 0)");
        CK(cudaMemcpyAsync(dst, h->snap[0], bytes, cudaMemcpyDeviceToDevice, h->st));
        if ((int)h->snap_filled.size() <= slot) h->snap_filled.resize(slot + 1, 0);
        h->snap_filled[slot] = 1;
    }
    return PL_OK;
}

int pl_load(pl_lattice h, int what, int slot) {
    PL_RANGE("pl_load");
    if (!h || what < PL_STORE_POPS || what > PL_STORE_SNAP || slot < 0) return fail(PL_ERR_ARG, "bad arguments");
    const std::vector<void *> &v = h->store[what];
    if ((int)v.size() <= slot || !v[slot] ||
        (what == PL_STORE_SNAP && ((int)h->snap_filled.size() <= slot || !h->snap_filled[slot])))
        return fail(PL_ERR_STATE, "store %d slot %d is empty", what, slot);
    const char *src = static_cast<const char *>(v[slot]);
    int r;
    if (what == PL_STORE_POPS) {
        CK(cudaMemcpyAsync(h->pop[h->cur], src, store_bytes(h, what), cudaMemcpyDeviceToDevice, h->st));
        h->last_kind = -1;
        h->snap_fresh[0] = h->snap_fresh[1] = false;
    } else if (what == PL_STORE_FWD) {
        for (int m = 0; m < 5; ++m) {
            const int f = PL_FWD_RHO + m;
            if ((r = ensure_d(h, &h->fld[f], h->n))) return r;
            CK(cudaMemcpyAsync(h->fld[f], reinterpret_cast<const double *>(src) + (size_t)m * h->n, sizeof(double) * h->n,
                               cudaMemcpyDeviceToDevice, h->st));
            if ((r = sync_cfield(h, f))) return r;
        }
    } else {
        if ((r = ensure_d(h, &h->snap[0], (size_t)h->q * h->np))) return r;
        CK(cudaMemcpyAsync(h->snap[0], src, store_bytes(h, what), cudaMemcpyDeviceToDevice, h->st));
        h->snap_ok[0] = true;
        h->snap_fresh[0] = false;
    }
    return PL_OK;
}

int pl_store_swap_snapshot(pl_lattice h, int slot) {
    if (!h || slot < 0 || slot >= kMaxStoreSlots) return fail(PL_ERR_ARG, "bad arguments (slot %d)", slot);
    std::vector<void *> &v = h->store[PL_STORE_SNAP];
    if ((int)v.size() <= slot) v.resize(slot + 1, nullptr);
    int r;
    const size_t bytes = store_bytes(h, PL_STORE_SNAP);
    if (!v[slot] && (r = dalloc(&v[slot], bytes))) return r;
    if (!h->snap[0] && (r = ensure_d(h, &h->snap[0], (size_t)h->q * h->np))) return r;
    // launches already queued keep the pointers they were given; stream order does the rest.
    // An empty slot may take the current snapshot, but the snapshot buffer then holds nothing a
    // sensitivity may read until the next pl_snapshot / pl_load / swap of a filled slot.
    if ((int)h->snap_filled.size() <= slot) h->snap_filled.resize(slot + 1, 0);
    void *t = v[slot];
    v[slot] = h->snap[0];
    h->snap[0] = static_cast<double *>(t);
    const bool was_ok = h->snap_ok[0];
    h->snap_fresh[0] = false;
    h->snap_ok[0] = h->snap_filled[slot] != 0;
    h->snap_filled[slot] = was_ok ? 1 : 0;
    return PL_OK;
}

int pl_store_release(pl_lattice h) {
    if (!h) return fail(PL_ERR_ARG, "null handle");
    CK(cudaStreamSynchronize(h->st));
    for (auto &v : h->store) { for (void *p : v) cudaFree(p); v.clear(); }
    h->snap_filled.clear();
    return PL_OK;
}

int pl_sensitivity_device(pl_lattice h, int which, const double *dads, const double *dkds, const double *qn,
                          const int *mask) {
    PL_RANGE("pl_sensitivity_device");
    if (!h || which < 0 || which > 3) return fail(PL_ERR_ARG, "bad arguments");
    if (h->adj_saved < 0) return fail(PL_ERR_STATE, "no saved adjoint collide");
    if (which <= 1 && (!h->snap_ok[0] || !h->snap_ok[1])) return fail(PL_ERR_STATE, "take both snapshots (pl_snapshot) first");
    for (int f = PL_FWD_RHO; f <= PL_FWD_TEM; ++f)
        if (!h->fld[f]) return fail(PL_ERR_STATE, "forward solution not set (pl_freeze_forward / pl_load)");
    int r;
    const double *hin[3] = {dads, dkds, qn};
    for (int m = 0; m < 3; ++m) {
        const int f = PL_DADS + m;
        if (hin[m]) {
            if ((r = ensure_d(h, &h->fld[f], h->n)) || (r = upload(h, h->fld[f], hin[m], h->n))) return r;
        }
    }
    if (mask) {
        if (!h->sens_mask && (r = dalloc((void **)&h->sens_mask, sizeof(int) * h->n))) return r;
        CK(cudaMemcpyAsync(h->sens_mask, mask, sizeof(int) * h->n, cudaMemcpyHostToDevice, h->st));
    }
    if (!h->fld[PL_DADS] || (which <= 2 && !h->fld[PL_DKDS]) || (which == 0 && (!h->fld[PL_QN] || !h->sens_mask)))
        return fail(PL_ERR_STATE, "sensitivity inputs not given yet");
    if ((r = ensure_d(h, &h->fld[PL_DFDS], h->n))) return r;
    if ((r = ensure_d(h, &h->fld[PL_KAPPA], h->n))) return r;
    pl::SensArgs sa;
    memset(&sa, 0, sizeof sa);
    sa.which = which; sa.n = h->n; sa.nx = h->nx; sa.ny = h->ny; sa.nz = h->nz; sa.np = h->np;
    sa.dfds = h->fld[PL_DFDS]; sa.dads = h->fld[PL_DADS]; sa.dkds = h->fld[PL_DKDS]; sa.qn = h->fld[PL_QN];
    sa.mask = h->sens_mask;
    sa.ux = h->fld[PL_FWD_UX]; sa.uy = h->fld[PL_FWD_UY]; sa.uz = h->fld[PL_FWD_UZ]; sa.tem = h->fld[PL_FWD_TEM];
    const int as = h->adj_saved;
    sa.imx = h->adj[as][4]; sa.imy = h->adj[as][5]; sa.imz = h->adj[as][6];
    sa.item = h->adj[as][7]; sa.iqx = h->adj[as][8]; sa.iqy = h->adj[as][9]; sa.iqz = h->adj[as][10];
    sa.kappa = h->fld[PL_KAPPA];
    sa.g = h->snap[0]; sa.ig = h->snap[1];
    pl::launch_sensitivity(h->q, sa, h->st);
    return check_launch(h, 1);
}

int pl_accumulate(pl_lattice h, int dst, int src, double a) {
    if (!h || dst < PL_DFDS || dst > PL_ACC) return fail(PL_ERR_ARG, "bad arguments");
    const double *s = nullptr;
    if ((src >= PL_ALPHA && src <= PL_GAMMA) || (src >= PL_FWD_RHO && src <= PL_ACC)) s = h->fld[src];
    else if (src >= PL_RHO && src <= PL_QZ) s = h->fwd_saved >= 0 ? h->fwd[h->fwd_saved][src - PL_RHO] : nullptr;
    else if (src >= PL_IP && src <= PL_IQZ) s = h->adj_saved >= 0 ? h->adj[h->adj_saved][src - PL_IP] : nullptr;
    else return fail(PL_ERR_ARG, "unknown field %d", src);
    if (!s) return fail(PL_ERR_STATE, "field %d has no value yet", src);
    int r;
    if ((r = ensure_d(h, &h->fld[dst], h->n))) return r;
    pl::launch_axpy(h->n, h->fld[dst], s, a, h->st);
    return check_launch(h, 1);
}

static int filter_common(pl_lattice h, int op, double R, double beta, const double *s, const double *d,
                         const int *mask, double *out, const double *wtab = nullptr) {
    if (!h || !s || !out || !(R > 0.0) || (op == 1 && !d)) return fail(PL_ERR_ARG, "bad arguments");
    Taps *t = get_taps(h, R);
    if (!t) return fail(PL_ERR_ALLOC, "filter taps");
    double *buf;
    int r = scratch(h, 5, &buf);
    if (r) return r;
    double *ds = buf, *dd = buf + h->n, *tmp = buf + 2 * (size_t)h->n, *dout = buf + 3 * (size_t)h->n;
    int *dm = reinterpret_cast<int *>(buf + 4 * (size_t)h->n);
    if ((r = upload(h, ds, s, h->n))) return r;
    if (d && (r = upload(h, dd, d, h->n))) return r;
    if (mask) CK(cudaMemcpyAsync(dm, mask, sizeof(int) * h->n, cudaMemcpyHostToDevice, h->st));
    if (wtab) {
        const size_t len = (size_t)h->n * t->ntap;
        if (h->wtab_len < len) {
            cudaFree(h->wtab);
            h->wtab = nullptr;
            h->wtab_len = 0;
            if ((r = dalloc((void **)&h->wtab, sizeof(double) * len))) return r;
            h->wtab_len = len;
        }
        if ((r = upload(h, h->wtab, wtab, len))) return r;
    }
    pl::FiltArgs f;
    f.n = h->n; f.nx = h->nx; f.ny = h->ny; f.nz = h->nz; f.ntap = t->ntap;
    f.di = t->di; f.dj = t->dj; f.dk = t->dk; f.hat = t->hat; f.mask = mask ? dm : nullptr; f.beta = beta;
    f.wtab = wtab ? h->wtab : nullptr;
    pl::launch_filter(op, f, ds, dd, tmp, dout, h->st);
    if ((r = check_launch(h, op == 1 ? 2 : 1))) return r;
    return download(h, out, dout, h->n);
}

int pl_heaviside_var(pl_lattice h, double R, double beta, const double *s, const int *mask, double *out) {
    PL_RANGE("pl_heaviside_var");
    return filter_common(h, 0, R, beta, s, nullptr, mask, out);
}
int pl_heaviside_sens(pl_lattice h, double R, double beta, const double *s, const double *dfdrho, const int *mask,
                      double *out) {
    PL_RANGE("pl_heaviside_sens");
    return filter_common(h, 1, R, beta, s, dfdrho, mask, out);
}
int pl_density_filter(pl_lattice h, double R, const double *v, const int *mask, double *out) {
    PL_RANGE("pl_density_filter");
    return filter_common(h, 2, R, 0.0, v, nullptr, mask, out);
}

int pl_filter_taps(pl_lattice h, double R, int *ntap, int *di, int *dj, int *dk) {
    if (!h || !ntap || !(R > 0.0)) return fail(PL_ERR_ARG, "bad arguments");
    const int nR = (int)R;
    int m = 0;
    for (int a = -nR; a <= nR; ++a)
        for (int b = -nR; b <= nR; ++b)
            for (int c = -nR; c <= nR; ++c) {
                const double dist = std::sqrt(std::pow((double)a, 2.0) + std::pow((double)b, 2.0) + std::pow((double)c, 2.0));
                if (dist > R || (h->nd == 2 && c != 0)) continue;
                if (di) di[m] = a;
                if (dj) dj[m] = b;
                if (dk) dk[m] = c;
                ++m;
            }
    *ntap = m;
    return PL_OK;
}

int pl_filter_weighted(pl_lattice h, int op, double R, double beta, const double *a, const double *b,
                       const double *weights, double *out) {
    PL_RANGE("pl_filter_weighted");
    if (!h || op < 0 || op > 2 || !weights) return fail(PL_ERR_ARG, "bad arguments");
    return filter_common(h, op, R, beta, a, op == 1 ? b : nullptr, nullptr, out, weights);
}

int pl_normalize(pl_lattice h, double *v, int n) {
    PL_RANGE("pl_normalize");
    if (!h || !v || n < 1 || n > h->n * h->q) return fail(PL_ERR_ARG, "bad arguments");
    double *buf;
    int r = scratch(h, 6, &buf);
    if (r) return r;
    if ((r = upload(h, buf, v, n))) return r;
    const int nblk = pl::resid_blocks(n);
    pl::launch_normalize(buf, n, h->partial, nblk, h->st);
    if ((r = check_launch(h, 2))) return r;
    return download(h, v, buf, n);
}

int pl_stats(pl_lattice h, double *last_ms, long long *launches) {
    if (!h) return fail(PL_ERR_ARG, "null handle");
    if (last_ms) {
        float ms = 0.f;
        if (cudaEventQuery(h->ev1) == cudaSuccess && cudaEventElapsedTime(&ms, h->ev0, h->ev1) == cudaSuccess) h->last_ms = ms;
        *last_ms = h->last_ms;
    }
    if (launches) *launches = h->launches;
    return PL_OK;
}

}  // extern "C"
