// inst_body.cuh -- explicit kernel instantiations and launch switch for one
// (lattice, storage) pair. Included by inst_<lattice>_<storage>.cu with PL_LAT, PL_STORE and
// PL_NAME defined; PL_ALL_KINDS selects every collide kind (else the primary ones only).
#include "kernels.cuh"
#include "launch.h"

namespace pl {

#define PL_CAT2(a, b) a##b
#define PL_CAT(a, b) PL_CAT2(a, b)

template <int K>
static void run_kind(int op, bool save, const KArgs &a, cudaStream_t st) {
    const int gi = (a.geo.n + kBlock - 1) / kBlock;
    switch (op) {
    case OP_COLLIDE:
        if (save) k_interior<PL_LAT, PL_STORE, K, true, false><<<gi, kBlock, 0, st>>>(a);
        else k_interior<PL_LAT, PL_STORE, K, false, false><<<gi, kBlock, 0, st>>>(a);
        break;
    case OP_STEP:
        if (save) k_interior<PL_LAT, PL_STORE, K, true, true><<<gi, kBlock, 0, st>>>(a);
        else k_interior<PL_LAT, PL_STORE, K, false, true><<<gi, kBlock, 0, st>>>(a);
        if (a.nb > 0) k_boundary<PL_LAT, PL_STORE, K><<<(a.nb + 127) / 128, 128, 0, st>>>(a);
        break;
    case OP_BOUNDARY:
        if (a.nb > 0) k_boundary<PL_LAT, PL_STORE, K><<<(a.nb + 127) / 128, 128, 0, st>>>(a);
        break;
    case OP_SNAPSHOT:
        k_snapshot<PL_LAT, PL_STORE, K><<<(a.geo.n + 127) / 128, 128, 0, st>>>(a);
        break;
    }
}

int PL_CAT(launch_, PL_NAME)(int kind, int op, bool save, const KArgs &a, cudaStream_t st) {
    switch (kind) {
    case K_AD_NATURAL: run_kind<K_AD_NATURAL>(op, save, a, st); return 0;
    case K_AD_FORCE: run_kind<K_AD_FORCE>(op, save, a, st); return 0;
    case K_AAD_NATURAL: run_kind<K_AAD_NATURAL>(op, save, a, st); return 0;
    case K_AAD_FORCE: run_kind<K_AAD_FORCE>(op, save, a, st); return 0;
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
    default: return -1;
    }
}

void PL_CAT(aux_, PL_NAME)(int op, const KArgs &a, int which, const double *const *in, int has_g, int sgn,
                           double *host_or_dev, int set, double shift, cudaStream_t st) {
    const int n = a.geo.n;
    switch (op) {
    case AUX_STREAM_PROGRAM:
        k_stream_program<PL_LAT, PL_STORE><<<(n + 127) / 128, 128, 0, st>>>(a, has_g, sgn);
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

}  // namespace pl
