//  runtime.h -- the device runtime under the drop-in headers of this tree.
//
//  The drop-in headers keep PANSLBM2's template API (D2Q9 / D3Q15 particles, the NS / AD / ANS /
//  AAD routines, the filters, Residual and Normalize). Underneath, particles run on handles of
//  the GB300 library (include/panslbm_gb300.h), one handle per NS + AD particle pair:
//
//  * a particle owns a handle from its construction and keeps its populations in set 0 (NS
//    role) or set 1 (AD role) of it; the first routine that couples an NS and an AD particle (a
//    coupled collide) moves the AD particle's populations into the NS particle's handle, and
//    both share that handle from then on;
//  * Stream / iStream and the boundary routines are recorded, not run. The next collide checks
//    that the record is one driver time step (each set streamed once, every boundary routine
//    after the stream of the set it touches) and runs it as one fused step: stream + recorded
//    boundary program + collide. A program is compiled once and reused while the recorded
//    calls and their functor values repeat. Any other order runs call by call;
//  * routines with host outputs (saved macros) copy them to the caller's arrays before they
//    return, as the reference writes them. Host inputs (alpha, kappa, the forward solution) are
//    uploaded again only when their contents changed since the last upload;
//  * the g snapshot a collide saves (gi / igi) stays on the device until it is needed: by a
//    sensitivity routine, which uses it in place, or by a collide that saves the next snapshot
//    into a different host array, which first copies it to its own host array.
//
//  Boundary functors are evaluated on the host, on the nodes the routine touches. Their values
//  are cached per functor type and captured state (the bytes of the functor object), which
//  holds for the reference drivers' functors: pure functions of the global coordinates and of
//  the values they capture. PANSLBM2_GPU_NO_FUNCTOR_CACHE=1 evaluates them at every call.
//
//  Errors abort with the library's message (the reference's routines return void and assert).
//  The storage precision of a particle follows T (FP64 for double, FP32 for float) unless
//  PANSLBM2_GPU_STORAGE is fp64, fp32, fp16 or bf16.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <type_traits>
#include <typeinfo>
#include <utility>
#include <vector>

#include "panslbm_gb300.h"
#include "../utility/vtkio.h"

namespace PANSLBM2 {
namespace {
const int BARRIER = 1;
const int MIRROR = 2;
}  // namespace

namespace gpu {

[[noreturn]] inline void die(const char *what, const char *detail = nullptr) {
    std::fprintf(stderr, "panslbm_gb300: %s%s%s\n", what, detail ? ": " : "", detail ? detail : "");
    std::abort();
}

inline void ck(int rc, const char *what) {
    if (rc != PL_OK) die(what, pl_last_error());
}

inline bool env_flag(const char *name) {
    const char *v = std::getenv(name);
    return v && v[0] == '1';
}

template <class T>
int storage_of() {
    const char *v = std::getenv("PANSLBM2_GPU_STORAGE");
    if (v) {
        if (!std::strcmp(v, "fp64")) return PL_FP64;
        if (!std::strcmp(v, "fp32")) return PL_FP32;
        if (!std::strcmp(v, "fp16")) return PL_FP16;
        if (!std::strcmp(v, "bf16")) return PL_BF16;
        die("PANSLBM2_GPU_STORAGE must be fp64, fp32, fp16 or bf16", v);
    }
    return std::is_same<T, double>::value ? PL_FP64 : PL_FP32;
}

//  host values as the double arrays the library exchanges (no copy for T = double)
template <class T>
struct AsDouble {
    std::vector<double> buf;
    const double *p = nullptr;
    AsDouble(const T *src, size_t n) {
        if (!src) return;
        if (std::is_same<T, double>::value) { p = reinterpret_cast<const double *>(src); return; }
        buf.assign(src, src + n);
        p = buf.data();
    }
};

template <class T>
void to_host(T *dst, const std::vector<double> &src) {
    for (size_t i = 0; i < src.size(); ++i) dst[i] = T(src[i]);
}

inline uint64_t fnv(const void *data, size_t bytes, uint64_t h = 1469598103934665603ull) {
    const unsigned char *p = static_cast<const unsigned char *>(data);
    for (size_t i = 0; i < bytes; ++i) { h ^= p[i]; h *= 1099511628211ull; }
    return h;
}

//  a functor of (i, j) on a 2D lattice, of (i, j, k) on a 3D one
template <int ND, class F>
auto at(const F &f, int i, int j, int k) {
    if constexpr (ND == 2) return f(i, j);
    else return f(i, j, k);
}

// ------------------------------------------------------------------------- functor values
//  One lattice-sized array per functor (type + captured state), filled plane by plane as
//  routines ask for them, so the face calls of one routine share one array.
struct FieldEntry {
    std::vector<int> ints;
    std::vector<double> reals;
    std::vector<std::pair<int, int>> planes;   // (axis, pos) already evaluated
    bool has(int axis, int pos) const {
        for (auto &p : planes)
            if (p.first == axis && p.second == pos) return true;
        return false;
    }
};

inline std::map<std::string, std::shared_ptr<FieldEntry>> &functor_cache() {
    static std::map<std::string, std::shared_ptr<FieldEntry>> c;
    return c;
}

template <class F>
bool cacheable() {
    return std::is_trivially_copyable<F>::value && !env_flag("PANSLBM2_GPU_NO_FUNCTOR_CACHE");
}

template <class F>
std::string functor_key(const F &f, const char *tag, int nx, int ny, int nz) {
    std::string key = std::string(typeid(F).name()) + "|" + tag + "|" + std::to_string(nx) + "x" + std::to_string(ny) +
                      "x" + std::to_string(nz) + "|";
    key.append(reinterpret_cast<const char *>(&f), sizeof(F));
    return key;
}

inline std::vector<int> &values_of(FieldEntry &e, int *) { return e.ints; }
inline std::vector<double> &values_of(FieldEntry &e, double *) { return e.reals; }

//  A functor evaluated on one plane: its lattice-sized array and a key for its values there.
template <class V>
struct Evaluated {
    std::shared_ptr<FieldEntry> entry;
    const V *data = nullptr;
    uint64_t key = 0;
};

//  call(i, j, k) evaluates the functor at one node of the plane (axis, pos)
template <class V, class F, class Fn>
Evaluated<V> evaluate(const F &f, const char *tag, int axis, int pos, int nx, int ny, int nz, Fn call) {
    std::shared_ptr<FieldEntry> e;
    const bool cache = cacheable<F>();
    if (cache) {
        auto &slot = functor_cache()[functor_key(f, tag, nx, ny, nz)];
        if (!slot) slot = std::make_shared<FieldEntry>();
        e = slot;
    } else {
        e = std::make_shared<FieldEntry>();
    }
    std::vector<V> &v = values_of(*e, static_cast<V *>(nullptr));
    if (v.empty()) v.assign((size_t)nx * ny * nz, V());
    Evaluated<V> out;
    out.entry = e;
    out.data = v.data();
    const int lo[3] = {axis == 0 ? pos : 0, axis == 1 ? pos : 0, axis == 2 ? pos : 0};
    const int hi[3] = {axis == 0 ? pos + 1 : nx, axis == 1 ? pos + 1 : ny, axis == 2 ? pos + 1 : nz};
    if (!e->has(axis, pos)) {
        for (int k = lo[2]; k < hi[2]; ++k)
            for (int j = lo[1]; j < hi[1]; ++j)
                for (int i = lo[0]; i < hi[0]; ++i) v[i + (size_t)nx * (j + (size_t)ny * k)] = V(call(i, j, k));
        e->planes.push_back({axis, pos});
    }
    if (cache) {
        const void *id = e.get();
        out.key = fnv(&id, sizeof id, fnv(tag, std::strlen(tag)));
    } else {
        uint64_t k = fnv(tag, std::strlen(tag));
        for (int kk = lo[2]; kk < hi[2]; ++kk)
            for (int j = lo[1]; j < hi[1]; ++j)
                for (int i = lo[0]; i < hi[0]; ++i) k = fnv(&v[i + (size_t)nx * (j + (size_t)ny * kk)], sizeof(V), k);
        out.key = k;
    }
    return out;
}

// ------------------------------------------------------------------------- boundary records
enum Inputs { IN_NONE = 0, IN_FORWARD = 1, IN_ADJOINT = 2 };

//  One recorded boundary routine call. Its per-node arrays are lattice-sized; the library reads
//  them on the edge / face / line of the call only.
struct BcRec {
    pl_bc_desc d;
    std::vector<std::shared_ptr<FieldEntry>> keep;   // keeps the arrays d points into alive
    uint64_t key = 0;                                // identity of the call and its values
    int sets = 0;                                    // bit s: touches population set s
    int inputs = IN_NONE;                            // macroscopic inputs the call reads
    const void *vel = nullptr;                       // the x velocity array the call names
};

inline BcRec make_rec(int kind, int lat, int axis, int pos, int dir, const Evaluated<int> *type,
                      const Evaluated<double> *v0 = nullptr, const Evaluated<double> *v1 = nullptr,
                      const Evaluated<double> *v2 = nullptr) {
    BcRec r;
    std::memset(&r.d, 0, sizeof r.d);
    r.d.kind = kind; r.d.lat = lat; r.d.axis = axis; r.d.pos = pos; r.d.dir = dir;
    uint64_t k = fnv(&r.d, sizeof r.d);
    if (type) { r.keep.push_back(type->entry); r.d.type = type->data; k = fnv(&type->key, 8, k); }
    const Evaluated<double> *vs[3] = {v0, v1, v2};
    const double **dst[3] = {&r.d.v0, &r.d.v1, &r.d.v2};
    for (int m = 0; m < 3; ++m) {
        if (!vs[m]) continue;
        r.keep.push_back(vs[m]->entry);
        *dst[m] = vs[m]->data;
        k = fnv(&vs[m]->key, 8, k);
    }
    r.key = k;
    return r;
}

//  a smoothing call (no functor)
inline BcRec make_smooth(int kind, int lat, int axis, int i, int j, int k, int di, int dj, int dk) {
    BcRec r;
    std::memset(&r.d, 0, sizeof r.d);
    r.d.kind = kind; r.d.lat = lat; r.d.axis = axis;
    r.d.i = i; r.d.j = j; r.d.k = k; r.d.di = di; r.d.dj = dj; r.d.dk = dk;
    r.key = fnv(&r.d, sizeof r.d);
    r.sets = 1 << lat;
    return r;
}

inline void finish_rec(BcRec &r, int sets, int inputs, double eps = 0.0, double kappa = 0.0,
                       const void *vel = nullptr) {
    r.sets = sets;
    r.inputs = inputs;
    r.vel = vel;
    r.d.eps = eps;
    r.d.kappa = kappa;
    r.key = fnv(&eps, 8, fnv(&kappa, 8, r.key));
}

// ------------------------------------------------------------------------- pairs
struct Shadow {
    const void *ptr = nullptr;
    std::vector<double> copy;
    long long epoch = -1;   // the phase it was last compared in
};

struct Pair;
//  host arrays the saving collides wrote -> their pair (for Residual)
inline std::map<const void *, Pair *> &saved_arrays() {
    static std::map<const void *, Pair *> m;
    return m;
}

//  Host output arrays whose values are still on the device: a saving collide leaves its outputs in
//  the library's two save slots per family and records here which save each host array stands
//  for. A family defers only inside a residual-driven loop: from the first Residual that the
//  library answers from that family's device slots until the next phase boundary. There, outputs
//  are written back when the driver reaches the boundary (an initial condition, a sensitivity, a
//  filter, an export, a population copy: sync_outputs) or just before their save slot is
//  overwritten (two saves later, when the array is not saved into again), and the residual reads
//  the device slots. Outside such a loop (a driver that reads the outputs on the host every step,
//  as test/elsens.cpp sums the displacement) every saving collide writes its outputs back.
//  PANSLBM2_GPU_EAGER_OUTPUTS=1 writes back after every saving collide, always.
struct Pending {
    const void *key;  // the host array
    Pair *pair;
    bool adjoint;
    int m;            // index in the family's outputs (rho ux uy uz tem qx qy qz / ip .. iqz)
    long long gen;    // the family's save generation
    bool is_float;
};
inline std::map<const void *, Pending> &pending_outputs() {
    static std::map<const void *, Pending> m;
    return m;
}
//  phases seen so far: host inputs are compared with their last upload once per phase
inline long long &input_epoch() {
    static long long e = 0;
    return e;
}
inline void sync_outputs();
inline std::vector<Pair *> &live_pairs() {
    static std::vector<Pair *> v;
    return v;
}

struct Pair {
    pl_lattice h = nullptr;
    int q = 0, nx = 0, ny = 0, nz = 1, n = 0, nd = 2;
    void *member[2] = {nullptr, nullptr};

    // recorded work since the last collide
    struct Ev { int what; int set; int inverse; int rec; };   // what 0: stream, 1: boundary call
    std::vector<Ev> queue;
    std::vector<BcRec> recs;
    std::map<std::vector<uint64_t>, int> programs;

    std::map<int, Shadow> shadows;   // host inputs last uploaded, per library field id

    // host arrays of the last two saving collides (forward: rho ux uy uz tem qx qy qz;
    // adjoint: ip iux iuy iuz imx imy imz item iqx iqy iqz)
    const void *fwd_save[8] = {}, *fwd_prev[8] = {};
    const void *adj_save[11] = {}, *adj_prev[11] = {};
    bool fwd_saved = false, adj_saved = false;
    long long fwd_gen = 0, adj_gen = 0;   // saves per family
    bool defer[2] = {false, false};       // forward / adjoint: inside a residual-driven loop

    // snapshots: the host array the device slot stands for, and whether the device copy still
    // has to be taken from the last collide
    const void *snap_owner[2] = {nullptr, nullptr};
    bool snap_pending[2] = {false, false};
    bool snap_float[2] = {false, false};

    Pair() { live_pairs().push_back(this); }
    Pair(const Pair &) = delete;
    ~Pair() {
        auto &lp = live_pairs();
        for (size_t i = 0; i < lp.size(); ++i)
            if (lp[i] == this) { lp.erase(lp.begin() + i); break; }
        auto &sa = saved_arrays();
        for (auto it = sa.begin(); it != sa.end();) {
            if (it->second == this) it = sa.erase(it);
            else ++it;
        }
        write_back([](const Pending &) { return true; });
        if (h) pl_destroy(h);
    }

    //  copy the pending host outputs of this pair that `pick` selects from the device
    template <class Pick>
    void write_back(Pick pick) {
        auto &po = pending_outputs();
        std::vector<double> tmp;
        for (auto it = po.begin(); it != po.end();) {
            const Pending &e = it->second;
            if (e.pair != this || !pick(e)) { ++it; continue; }
            const long long age = (e.adjoint ? adj_gen : fwd_gen) - e.gen;
            if (h && age <= 1) {
                tmp.resize(n);
                ck(pl_get_saved_field(h, (e.adjoint ? PL_IP : PL_RHO) + e.m, int(age), tmp.data()),
                   "pl_get_saved_field");
                if (e.is_float) to_host(static_cast<float *>(const_cast<void *>(it->first)), tmp);
                else std::memcpy(const_cast<void *>(it->first), tmp.data(), sizeof(double) * n);
            }
            it = po.erase(it);
        }
    }

    //  upload a host input when it is new or changed (PANSLBM2_GPU_TRUST_INPUTS=1: when new)
    template <class T>
    void input(int field, const T *p) {
        if (!p) return;
        Shadow &s = shadows[field];
        static const bool trust = env_flag("PANSLBM2_GPU_TRUST_INPUTS");
        if (trust && s.ptr == p && s.copy.size() == (size_t)n) return;
        // within one phase (between two phase-boundary calls) a known input is not compared again
        if (s.ptr == p && s.copy.size() == (size_t)n && s.epoch == input_epoch()) return;
        s.epoch = input_epoch();
        if (s.ptr == p && s.copy.size() == (size_t)n) {
            bool equal;
            if (std::is_same<T, double>::value) equal = std::memcmp(s.copy.data(), p, sizeof(double) * n) == 0;
            else {
                equal = true;
                for (int i = 0; i < n && equal; ++i) equal = s.copy[i] == double(p[i]);
            }
            if (equal) return;
        }
        s.ptr = p;
        s.copy.assign(p, p + n);
        ck(pl_set_field(h, field, s.copy.data()), "pl_set_field");
    }

    //  an adjoint macro (index m of ip iux iuy iuz imx imy imz item iqx iqy iqz) the device must
    //  hold: the last adjoint save if the caller names its array, else the caller's values
    template <class T>
    void adjoint_input(int m, const T *p) {
        if (!p || (adj_saved && adj_save[m] == p)) return;
        AsDouble<T> v(p, n);
        ck(pl_set_field(h, PL_IP + m, v.p), "pl_set_field");
    }

    //  a forward-solution field the caller does not pass (the library reads all five)
    void forward_default(int field) {
        if (shadows.count(field)) return;
        std::vector<double> zero(n, 0.0);
        shadows[field].ptr = nullptr;
        ck(pl_set_field(h, field, zero.data()), "pl_set_field");
    }

    int program_for(const std::vector<int> &idx) {
        if (idx.empty()) return -1;
        std::vector<uint64_t> key;
        for (int i : idx) key.push_back(recs[i].key);
        auto it = programs.find(key);
        if (it != programs.end()) return it->second;
        if (programs.size() >= 64) {   // the recorded values keep changing: start over
            for (auto &kv : programs) pl_program_destroy(h, kv.second);
            programs.clear();
        }
        std::vector<pl_bc_desc> d;
        for (int i : idx) d.push_back(recs[i].d);
        int prog = -1;
        ck(pl_program_create(h, d.data(), (int)d.size(), &prog), "pl_program_create");
        programs[key] = prog;
        return prog;
    }

    //  the library's forward boundary routines read the velocity of the last collide
    void check_velocity(const BcRec &r) const {
        if (r.inputs != IN_FORWARD || !r.vel) return;
        if (fwd_saved && r.vel == fwd_save[1]) return;
        die("a boundary routine names a velocity array other than the one the last saving collide wrote; "
            "the device uses the velocity of the last collide");
    }

    //  take a pending snapshot into its device slot (before the populations move on)
    void settle_snapshot(int slot, const void *next_owner, bool next_saves) {
        if (!snap_pending[slot]) return;
        snap_pending[slot] = false;
        if (next_saves && next_owner == snap_owner[slot]) return;   // superseded
        if (next_saves && snap_owner[slot]) {
            // the slot is about to stand for another host array: give this one its values
            std::vector<double> tmp((size_t)n * q);
            ck(pl_snapshot(h, slot, tmp.data()), "pl_snapshot");
            if (snap_float[slot]) to_host(static_cast<float *>(const_cast<void *>(snap_owner[slot])), tmp);
            else std::memcpy(const_cast<void *>(snap_owner[slot]), tmp.data(), sizeof(double) * tmp.size());
        } else {
            ck(pl_snapshot(h, slot, nullptr), "pl_snapshot");
        }
    }

    void settle_all() {
        settle_snapshot(0, nullptr, false);
        settle_snapshot(1, nullptr, false);
    }

    //  make the device snapshot slot hold the host array p
    template <class T>
    void use_snapshot(int slot, const T *p) {
        if (!p) die("a sensitivity routine needs the g and ig snapshots");
        if (snap_owner[slot] == p) {
            if (snap_pending[slot]) { ck(pl_snapshot(h, slot, nullptr), "pl_snapshot"); snap_pending[slot] = false; }
            return;
        }
        AsDouble<T> v(p, (size_t)n * q);
        ck(pl_set_snapshot(h, slot, v.p), "pl_set_snapshot");
    }

    void stream_sets(const bool sets[2], int inverse) {
        if (sets[0] && sets[1]) { ck(pl_stream(h, inverse, -1, 1), "pl_stream"); return; }
        const int keep = sets[0] ? 1 : 0;   // the set that is not streamed keeps its values
        std::vector<double> tmp((size_t)n * q);
        ck(pl_get_populations(h, keep, tmp.data()), "pl_get_populations");
        ck(pl_stream(h, inverse, -1, 1), "pl_stream");
        ck(pl_set_populations(h, keep, tmp.data()), "pl_set_populations");
    }

    //  run the recorded work call by call
    void flush() {
        if (queue.empty()) return;
        settle_all();
        size_t i = 0;
        while (i < queue.size()) {
            if (queue[i].what == 0) {
                bool sets[2] = {false, false};
                const int inv = queue[i].inverse;
                size_t j = i;
                while (j < queue.size() && queue[j].what == 0 && queue[j].inverse == inv && !sets[queue[j].set]) {
                    sets[queue[j].set] = true;
                    ++j;
                }
                stream_sets(sets, inv);
                i = j;
            } else {
                std::vector<int> run;
                int inputs = IN_NONE;
                size_t j = i;
                while (j < queue.size() && queue[j].what == 1) {
                    const BcRec &r = recs[queue[j].rec];
                    if (r.inputs != IN_NONE && inputs != IN_NONE && r.inputs != inputs) break;
                    if (r.inputs != IN_NONE) inputs = r.inputs;
                    check_velocity(r);
                    run.push_back(queue[j].rec);
                    ++j;
                }
                ck(pl_stream(h, inputs == IN_ADJOINT ? 3 : 2, program_for(run), 1), "pl_stream (boundary routines)");
                i = j;
            }
        }
        queue.clear();
        recs.clear();
    }

    //  the recorded work is one driver time step for a collide
    bool fusable(bool adjoint, bool has_g, std::vector<int> &idx) const {
        int streamed[2] = {0, 0};
        for (const Ev &e : queue) {
            if (e.what == 0) {
                if (e.inverse != (adjoint ? 1 : 0) || streamed[e.set]) return false;
                streamed[e.set] = 1;
            } else {
                const BcRec &r = recs[e.rec];
                if (r.inputs != IN_NONE && r.inputs != (adjoint ? IN_ADJOINT : IN_FORWARD)) return false;
                for (int s = 0; s < 2; ++s)
                    if ((r.sets >> s & 1) && !streamed[s]) return false;
                idx.push_back(e.rec);
            }
        }
        return streamed[0] && (has_g ? streamed[1] != 0 : streamed[1] == 0);
    }

    //  one collide of the reference; outs: the host arrays the routine saves into
    template <class T>
    void collide(int kind, const pl_phys &ph, bool save, T *const *outs, int nouts, T *snap) {
        const bool adjoint = (kind >= PL_ANS_BRINKMAN && kind <= PL_ANSIN_BRINKMAN) || kind == PL_AEL_COLLIDE;
        const bool has_g = !(kind == PL_NS_COLLIDE || kind == PL_NS_BRINKMAN || kind == PL_ANS_BRINKMAN ||
                             kind == PL_NSIN_COLLIDE || kind == PL_NSIN_BRINKMAN || kind == PL_ANSIN_BRINKMAN ||
                             kind == PL_EL_COLLIDE || kind == PL_EL_EXTENDED || kind == PL_AEL_COLLIDE);
        const int slot = adjoint ? 1 : 0;
        const bool saves_snap = save && snap != nullptr;
        if (save) {
            // the save about to be written reuses the slot of the save before last: host arrays
            // that still stand for that save, and are not saved into again now, take it first
            const long long gen = adjoint ? adj_gen : fwd_gen;
            write_back([&](const Pending &e) {
                if (e.adjoint != adjoint || gen - e.gen < 1) return false;
                for (int m = 0; m < nouts; ++m) if (outs[m] && (const void *)outs[m] == e.key) return false;
                return true;
            });
        }
        std::vector<int> idx;
        if (!queue.empty() && fusable(adjoint, has_g, idx)) {
            settle_snapshot(0, adjoint ? nullptr : snap, !adjoint && saves_snap);
            settle_snapshot(1, adjoint ? snap : nullptr, adjoint && saves_snap);
            for (int i : idx) check_velocity(recs[i]);
            ck(pl_step(h, kind, &ph, program_for(idx), save ? 1 : 0), "pl_step");
            queue.clear();
            recs.clear();
        } else {
            flush();
            settle_snapshot(0, adjoint ? nullptr : snap, !adjoint && saves_snap);
            settle_snapshot(1, adjoint ? snap : nullptr, adjoint && saves_snap);
            ck(pl_collide(h, kind, &ph, save ? 1 : 0), "pl_collide");
        }
        if (save) {
            const void **cur = adjoint ? adj_save : fwd_save, **prev = adjoint ? adj_prev : fwd_prev;
            const long long gen = ++(adjoint ? adj_gen : fwd_gen);
            for (int m = 0; m < nouts; ++m) {
                prev[m] = cur[m];
                cur[m] = outs[m];
                if (!outs[m]) continue;
                // the values stay on the device until the host needs them (sync_outputs)
                pending_outputs()[outs[m]] = Pending{outs[m], this, adjoint, m, gen, !std::is_same<T, double>::value};
                saved_arrays()[outs[m]] = this;
            }
            (adjoint ? adj_saved : fwd_saved) = true;
            static const bool eager = env_flag("PANSLBM2_GPU_EAGER_OUTPUTS");
            if (eager || !defer[slot]) write_back([&](const Pending &e) { return e.adjoint == adjoint; });
        }
        if (saves_snap) {
            snap_owner[slot] = snap;
            snap_pending[slot] = true;
            snap_float[slot] = !std::is_same<T, double>::value;
        }
    }

    void record_stream(int set, int inverse) { queue.push_back({0, set, inverse, -1}); }

    void record(BcRec &&r) {
        recs.push_back(std::move(r));
        queue.push_back({1, -1, 0, (int)recs.size() - 1});
    }

    //  the library residual family whose current / previous saves are (a, b), or -1
    int residual_family(const void *const *a, const void *const *b, int ncomp) const {
        for (int fam = 0; fam < 4; ++fam) {
            const bool adj = fam >= 2;
            if (adj ? !adj_saved : !fwd_saved) continue;
            const int first = fam == 0 ? 1 : fam == 1 ? 5 : fam == 2 ? 1 : 8;
            const void *const *cur = adj ? adj_save : fwd_save;
            const void *const *prev = adj ? adj_prev : fwd_prev;
            bool ok = ncomp == nd;
            for (int m = 0; m < ncomp && ok; ++m) ok = cur[first + m] == a[m] && prev[first + m] == b[m];
            if (ok) return fam;
        }
        return -1;
    }
};

//  phase boundary: every host output array takes its value from the device, and host inputs are
//  compared with their uploads again at their next use
inline void sync_outputs() {
    for (Pair *p : live_pairs()) {
        p->write_back([](const Pending &) { return true; });
        p->defer[0] = p->defer[1] = false;
    }
    ++input_epoch();
}
//  the VTK exporters read host arrays through the driver's functors: sync before they do
inline const bool vtk_hook_set = (vtkio::host_sync_hook() = &sync_outputs, true);

//  Base of the drop-in particles: the handle binding and the particle's role (0 NS set, 1 AD
//  set, -1 not known yet).
template <class T>
struct Particle {
    std::shared_ptr<Pair> pair;
    int set = 0;
    int role = -1;

    void bind(int q, int nx, int ny, int nz) {
        pair = std::make_shared<Pair>();
        pair->q = q; pair->nx = nx; pair->ny = ny; pair->nz = nz; pair->n = nx * ny * nz;
        pair->nd = q == 9 ? 2 : 3;
        ck(pl_create(q, nx, ny, q == 9 ? 1 : nz, storage_of<T>(), &pair->h), "pl_create");
        pair->member[0] = this;
    }

    //  fix the role on first use; a particle still alone moves its populations to that set
    void claim(int r) {
        if (role == r) return;
        if (role == -1 && pair->member[0] == this && pair->member[1] == nullptr) {
            if (r == 1) {
                pair->flush();
                std::vector<double> tmp((size_t)pair->n * pair->q);
                ck(pl_get_populations(pair->h, 0, tmp.data()), "pl_get_populations");
                ck(pl_set_populations(pair->h, 1, tmp.data()), "pl_set_populations");
            }
            role = r;
            set = r;
            return;
        }
        die(r ? "an NS particle is used as the AD set of a routine" : "an AD particle is used as the NS set of a routine");
    }
};

//  Share one handle between the NS particle f and the AD particle g.
template <class T, template <class> class P, template <class> class Q>
Pair &couple(P<T> &f, Q<T> &g) {
    Particle<T> &pf = f.gpu_particle(), &pg = g.gpu_particle();
    if (pf.pair == pg.pair && pf.role == 0 && pg.role == 1) return *pf.pair;
    pf.claim(0);
    pg.claim(1);
    if (pf.pair == pg.pair) return *pf.pair;
    if (pf.pair->member[1]) die("the NS particle is already coupled to another AD particle");
    if (pg.pair->member[0] != &pg) die("the AD particle is already coupled to another NS particle");
    if (pf.pair->q != pg.pair->q || pf.pair->n != pg.pair->n) die("coupled particles differ in lattice");
    Pair &src = *pg.pair;
    src.flush();
    src.settle_all();
    std::vector<double> tmp((size_t)src.n * src.q);
    ck(pl_get_populations(src.h, 1, tmp.data()), "pl_get_populations");
    Pair &dst = *pf.pair;
    dst.flush();
    ck(pl_set_populations(dst.h, 1, tmp.data()), "pl_set_populations");
    pg.pair = pf.pair;   // releases the AD particle's own handle
    pg.set = 1;
    dst.member[1] = &pg;
    return dst;
}

//  the handle of a particle used in role r
template <class T, template <class> class P>
Pair &own(P<T> &p, int r) {
    Particle<T> &pp = p.gpu_particle();
    pp.claim(r);
    return *pp.pair;
}

inline Pair &any_pair() {
    if (live_pairs().empty()) die("this routine needs a lattice on the device: construct a particle first");
    return *live_pairs().front();
}

//  One edge / face / line routine: evaluate its type functor and up to three value functors on
//  the plane (axis, pos) and record it on the particle's handle.
struct NoF {};

template <int ND, class F>
Evaluated<double> eval_values(const F &f, Pair &pr, int axis, int pos) {
    return evaluate<double>(f, "v", axis, pos, pr.nx, pr.ny, pr.nz,
                            [&](int i, int j, int k) { return double(at<ND>(f, i, j, k)); });
}

template <class T, template <class> class P, class Ff, class F0 = NoF, class F1 = NoF, class F2 = NoF>
void record_bc(P<T> &p, int role, int kind, int axis, int pos, int dir, const Ff &type, int inputs,
               const void *vel = nullptr, double eps = 0.0, double kappa = 0.0, const F0 &f0 = F0(),
               const F1 &f1 = F1(), const F2 &f2 = F2()) {
    Pair &pr = own(p, role);
    constexpr int ND = P<T>::nd;
    Evaluated<int> et = evaluate<int>(type, "t", axis, pos, pr.nx, pr.ny, pr.nz,
                                      [&](int i, int j, int k) { return int(at<ND>(type, i, j, k)); });
    Evaluated<double> e0, e1, e2;
    if constexpr (!std::is_same<F0, NoF>::value) e0 = eval_values<ND>(f0, pr, axis, pos);
    if constexpr (!std::is_same<F1, NoF>::value) e1 = eval_values<ND>(f1, pr, axis, pos);
    if constexpr (!std::is_same<F2, NoF>::value) e2 = eval_values<ND>(f2, pr, axis, pos);
    BcRec r = make_rec(kind, role, axis, pos, dir, &et, e0.data ? &e0 : nullptr, e1.data ? &e1 : nullptr,
                       e2.data ? &e2 : nullptr);
    finish_rec(r, 1 << role, inputs, eps, kappa, vel);
    pr.record(std::move(r));
}

//  the whole-boundary routines visit xmin, xmax, ymin, ymax[, zmin, zmax]
template <class P, class Fn>
void each_face(const P &p, Fn fn) {
    fn(0, 0, -1);
    fn(0, p.lx - 1, 1);
    fn(1, 0, -1);
    fn(1, p.ly - 1, 1);
    if (P::nd == 3) {
        fn(2, 0, -1);
        fn(2, p.lz - 1, 1);
    }
}

//  The sensitivity routines: which 0 TemperatureAtHeatSource, 1 BrinkmanDiffusivity,
//  2 HeatExchange (dkds = dbds), 3 ANS::SensitivityBrinkman. dfds is accumulated into.
template <class T>
void sensitivity(Pair &pr, int which, T *dfds, const T *dads, const T *dkds, const T *ux, const T *uy, const T *uz,
                 const T *tem, const T *imx, const T *imy, const T *imz, const T *item, const T *iqx, const T *iqy,
                 const T *iqz, const T *kappa, const T *g, const T *ig, const double *qn, const int *mask) {
    pr.flush();
    pr.settle_all();
    sync_outputs();
    pr.input(PL_FWD_UX, ux);
    pr.input(PL_FWD_UY, uy);
    pr.input(PL_FWD_UZ, uz);
    pr.input(PL_FWD_TEM, tem);
    for (int f = PL_FWD_RHO; f <= PL_FWD_TEM; ++f) pr.forward_default(f);
    const T *adj[7] = {imx, imy, imz, item, iqx, iqy, iqz};
    for (int m = 0; m < 7; ++m) pr.adjoint_input(4 + m, adj[m]);
    pr.input(PL_KAPPA, kappa);
    if (which <= 1) {
        pr.use_snapshot(0, g);
        pr.use_snapshot(1, ig);
    }
    AsDouble<T> a(dads, pr.n), k(dkds, pr.n);
    std::vector<double> d(dfds, dfds + pr.n);
    ck(pl_sensitivity(pr.h, which, d.data(), a.p, k.p, qn, mask), "pl_sensitivity");
    to_host(dfds, d);
}

//  qn and mask of a heat-source sensitivity: the functors on the faces of the lattice
template <int ND, class Fv, class Ff>
void face_values(const Pair &pr, const Fv &qnbc, const Ff &bctype, std::vector<double> &qn, std::vector<int> &mask) {
    qn.assign(pr.n, 0.0);
    mask.assign(pr.n, 0);
    const int len[3] = {pr.nx, pr.ny, pr.nz};
    for (int k = 0; k < pr.nz; ++k)
        for (int j = 0; j < pr.ny; ++j)
            for (int i = 0; i < pr.nx; ++i) {
                const int c[3] = {i, j, k};
                bool face = false;
                for (int a = 0; a < ND; ++a) face = face || c[a] == 0 || c[a] == len[a] - 1;
                if (!face) continue;
                const size_t idx = i + (size_t)pr.nx * (j + (size_t)pr.ny * k);
                qn[idx] = double(at<ND>(qnbc, i, j, k));
                mask[idx] = int(at<ND>(bctype, i, j, k));
            }
}

//  The library filters with the hat weight (R - |d|) / R, either everywhere or only between two
//  masked nodes (identity elsewhere): the form of the drivers' weights. Infer that mask from a
//  weight functor of global coordinates (i1, j1, k1, i2, j2, k2) and verify the functor against
//  it on every tap inside the lattice. Returns an empty vector for "hat everywhere"; aborts if
//  the functor has another form. Cached per functor type, captured state and radius.
struct FilterPlan {
    std::vector<int> mask;        // hat weight between mask cells (empty: everywhere)
    bool general = false;         // the functor is not of that form: use `table`
    std::vector<double> table;    // [node][tap] functor values (pl_filter_taps order)
};
//  The drivers' weight functors are the hat weight (R - distance) / R, everywhere or between two
//  cells of a design region with the identity elsewhere: that region is inferred and checked
//  on every tap, and the device builds the weights itself. Any other functor is evaluated on
//  every (node, tap) pair into a table for pl_filter_weighted.
template <class F>
std::shared_ptr<const FilterPlan> filter_plan(const Pair &pr, double R, const F &w) {
    static std::map<std::string, std::shared_ptr<const FilterPlan>> cache;
    std::string key;
    if (cacheable<F>()) {
        key = functor_key(w, "filter", pr.nx, pr.ny, pr.nz);
        key.append(reinterpret_cast<const char *>(&R), sizeof R);
        auto it = cache.find(key);
        if (it != cache.end()) return it->second;
    }
    const int nR = (int)R;
    struct Tap { int a, b, c; double hat; };
    std::vector<Tap> taps;
    for (int a = -nR; a <= nR; ++a)
        for (int b = -nR; b <= nR; ++b)
            for (int c = (pr.nd == 3 ? -nR : 0); c <= (pr.nd == 3 ? nR : 0); ++c) {
                const double d = std::sqrt(std::pow((double)a, 2.0) + std::pow((double)b, 2.0) + std::pow((double)c, 2.0));
                if (d <= R) taps.push_back({a, b, c, (R - d) / R});
            }
    auto inside = [&](int i, int j, int k) { return 0 <= i && i < pr.nx && 0 <= j && j < pr.ny && 0 <= k && k < pr.nz; };
    auto idx = [&](int i, int j, int k) { return i + (size_t)pr.nx * (j + (size_t)pr.ny * k); };
    auto plan = std::make_shared<FilterPlan>();
    std::vector<int> m(pr.n, 0);
    for (int k = 0; k < pr.nz; ++k)
        for (int j = 0; j < pr.ny; ++j)
            for (int i = 0; i < pr.nx; ++i)
                for (const Tap &t : taps) {
                    if (t.a == 0 && t.b == 0 && t.c == 0) continue;
                    if (!inside(i + t.a, j + t.b, k + t.c)) continue;
                    if (double(w(i, j, k, i + t.a, j + t.b, k + t.c)) != 0.0) { m[idx(i, j, k)] = 1; break; }
                }
    bool all = true, hat = true;
    for (int k = 0; k < pr.nz && hat; ++k)
        for (int j = 0; j < pr.ny && hat; ++j)
            for (int i = 0; i < pr.nx && hat; ++i) {
                const int mi = m[idx(i, j, k)];
                all = all && mi;
                for (const Tap &t : taps) {
                    const int i2 = i + t.a, j2 = j + t.b, k2 = k + t.c;
                    if (!inside(i2, j2, k2)) continue;
                    const bool center = t.a == 0 && t.b == 0 && t.c == 0;
                    const double expect = (mi && m[idx(i2, j2, k2)]) ? t.hat : (center ? 1.0 : 0.0);
                    if (double(w(i, j, k, i2, j2, k2)) != expect) { hat = false; break; }
                }
            }
    if (hat) {
        if (!all) plan->mask.swap(m);
    } else {
        const size_t nt = taps.size();
        plan->general = true;
        plan->table.assign((size_t)pr.n * nt, 0.0);
        for (int k = 0; k < pr.nz; ++k)
            for (int j = 0; j < pr.ny; ++j)
                for (int i = 0; i < pr.nx; ++i)
                    for (size_t t = 0; t < nt; ++t) {
                        const int i2 = i + taps[t].a, j2 = j + taps[t].b, k2 = k + taps[t].c;
                        if (inside(i2, j2, k2)) plan->table[idx(i, j, k) * nt + t] = double(w(i, j, k, i2, j2, k2));
                    }
    }
    if (!key.empty()) cache[key] = plan;
    return plan;
}

template <class T>
pl_phys phys(T nu, T diff, T gx, T gy, T gz, T tem0) {
    pl_phys ph{};
    ph.nu = double(nu); ph.diff = double(diff); ph.gx = double(gx); ph.gy = double(gy); ph.gz = double(gz);
    ph.tem0 = double(tem0);
    return ph;
}

//  the elastic kinds relax at 1 / tau
template <class T>
pl_phys phys_tau(T tau) {
    pl_phys ph{};
    ph.tau = double(tau);
    return ph;
}

//  A caller's node array read as a functor of (i, j[, k]) (local = global coordinates on one
//  device). It holds a shared_ptr, so it is not trivially copyable and record_bc evaluates it
//  afresh on every call: the caller may rewrite the array between calls.
template <class T>
struct NodeValues {
    const T *p;
    int nx, ny;
    std::shared_ptr<int> fresh = std::make_shared<int>(0);
    NodeValues(const T *p_, int nx_, int ny_) : p(p_), nx(nx_), ny(ny_) {}
    double operator()(int i, int j) const { return double(p[i + (size_t)nx * j]); }
    double operator()(int i, int j, int k) const { return double(p[i + (size_t)nx * (j + (size_t)ny * k)]); }
};

}  // namespace gpu
}  // namespace PANSLBM2
