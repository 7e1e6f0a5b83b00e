// unet.cu -- the learned warm start: a 3D convolutional U-Net that predicts the converged
// macroscopic fields (rho, u, T and their adjoints) of the steady heat-sink problem from the
// filtered design, trained on (design, converged field) pairs the solver produces. Forward,
// backward and optimizer run on the device: convolutions as tcgen05 implicit GEMMs fed by TMA
// (unet_kernels.cuh), BF16 activations and weights, FP32 accumulation, FP32 master weights
// with Adam. The reference has no learned component; this is the library's own.
//
// Network (levels L, base channels c, C_l = c 2^l): encoder level l = two 3x3x3 convolutions
// (C_{l-1} -> C_l -> C_l, ReLU) then 2x2x2 average pooling; decoder level l = nearest
// upsampling of level l+1, concatenation with the encoder output of level l, two 3x3x3
// convolutions (C_l + C_{l+1} -> C_l -> C_l, ReLU); a 1x1x1 head to the output channels. Loss:
// mean squared error of the normalised targets.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <random>
#include <string>
#include <vector>

#include "../../include/panslbm_gb300.h"
#include "launch.h"
#include "unet_kernels.cuh"

using pl::unet::bf16;

namespace {

int uerr(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    return pl::record_error(code, buf);
}

#define UCK(x)                                                                                    \
    do {                                                                                          \
        cudaError_t e_ = (x);                                                                     \
        if (e_ != cudaSuccess) return uerr(PL_ERR_CUDA, "%s: %s", #x, cudaGetErrorString(e_));    \
    } while (0)

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

CUtensorMapSwizzle swz(int bytes) {
    return bytes == 128 ? CU_TENSOR_MAP_SWIZZLE_128B : bytes == 64 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_32B;
}

// 5D map over a channels-last activation [B][Z][Y][X][C] (BF16), box {ck, tx, ty, 1, 1}
int map_act(CUtensorMap *m, const bf16 *p, int C, int X, int Y, int Z, int B, int ck, int tx, int ty) {
    auto fn = encode_fn();
    if (!fn) return uerr(PL_ERR_CUDA, "cuTensorMapEncodeTiled is unavailable");
    cuuint64_t dims[5] = {cuuint64_t(C), cuuint64_t(X), cuuint64_t(Y), cuuint64_t(Z), cuuint64_t(B)};
    cuuint64_t strides[4] = {cuuint64_t(C) * 2, cuuint64_t(C) * 2 * X, cuuint64_t(C) * 2 * X * Y,
                             cuuint64_t(C) * 2 * X * Y * Z};
    cuuint32_t box[5] = {cuuint32_t(ck), cuuint32_t(tx), cuuint32_t(ty), 1, 1};
    cuuint32_t es[5] = {1, 1, 1, 1, 1};
    CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<bf16 *>(p), dims, strides, box, es,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, swz(ck * 2), CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return uerr(PL_ERR_CUDA, "activation tensor map (C %d, box %d x %d x %d): CUresult %d", C, ck, tx, ty, int(r));
    return PL_OK;
}
// 2D map over weights [rows][K] (BF16), box {ck, rows}
int map_w(CUtensorMap *m, const bf16 *p, int K, int rows, int ck) {
    auto fn = encode_fn();
    if (!fn) return uerr(PL_ERR_CUDA, "cuTensorMapEncodeTiled is unavailable");
    cuuint64_t dims[2] = {cuuint64_t(K), cuuint64_t(rows)};
    cuuint64_t strides[1] = {cuuint64_t(K) * 2};
    cuuint32_t box[2] = {cuuint32_t(ck), cuuint32_t(rows)};
    cuuint32_t es[2] = {1, 1};
    CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<bf16 *>(p), dims, strides, box, es,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, swz(ck * 2), CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return uerr(PL_ERR_CUDA, "weight tensor map (K %d, rows %d): CUresult %d", K, rows, int(r));
    return PL_OK;
}

// input-channel chunk per MMA stage: the widest of 64, 32, 16 that divides c
int chunk(int c) { return c % 64 == 0 ? 64 : c % 32 == 0 ? 32 : 16; }

struct Level {
    int X, Y, Z;
    long long V;     // voxels of one sample
    int tx, ty, ntx, nty;
};

struct Buf {
    bf16 *p = nullptr;
    int C = 0, level = 0;
};

struct Conv {
    int cin = 0, cout = 0, taps = 27, level = 0;
    float *w = nullptr, *b = nullptr, *gw = nullptr, *gb = nullptr, *mw = nullptr, *vw = nullptr, *mb = nullptr,
          *vb = nullptr;
    bf16 *wb = nullptr, *wt = nullptr;
    Buf in, out;            // input tensor; output tensor (channel slice [out_off, +cout) of out)
    int out_off = 0, relu = 1;
    Buf dz, din;            // gradient at the output (pre-activation) and at the input
    const Buf *din_mask = nullptr;
    bool need_dgrad = true;
    CUtensorMap mapX, mapW, mapD, mapWt;
    long long nw() const { return (long long)cout * taps * cin; }
};

}  // namespace

struct pl_unet_s {
    int L = 4, base = 16, cin = 16, cout = 16, bmax = 1;
    std::vector<Level> lev;
    std::vector<Conv> convs;         // order: enc l c1, enc l c2 (l = 0..L-1), dec l c1, c2 (l = L-2..0), head
    std::vector<void *> allocs;
    Buf in0;
    float *pred = nullptr;           // [B][V0][cout] FP32
    bf16 *dpred = nullptr;
    std::vector<Buf> e1, cat, pool, d1, d2, ge1, ge2, gd1, gd2, gcat, gpool;
    Buf bot, gbot;
    double *dacc = nullptr;
    int *err = nullptr;
    cudaStream_t st = nullptr;
    long long step = 0;              // Adam steps taken
    // dataset
    int nds = 0, cused = 0, nstat = 0;
    float *ds_design = nullptr, *ds_target = nullptr, *stat = nullptr;
    float *mean = nullptr, *inv_std = nullptr, *stdv = nullptr;
    std::vector<float> h_mean, h_std;
    bf16 *tgt = nullptr;             // normalised batch targets [B][V0][cout]
    float *design_tmp = nullptr;
    double *pred64 = nullptr;
    int smem_conv_max = 0, smem_wgrad_max = 0;
};

namespace {

int ualloc(pl_unet u, void **p, size_t bytes) {
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) { *p = nullptr; cudaGetLastError(); return uerr(PL_ERR_ALLOC, "cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e)); }
    u->allocs.push_back(*p);
    return cudaMemsetAsync(*p, 0, bytes, u->st) == cudaSuccess ? PL_OK : uerr(PL_ERR_CUDA, "memset");
}
int mkbuf(pl_unet u, Buf &b, int C, int level) {
    b.C = C;
    b.level = level;
    return ualloc(u, (void **)&b.p, sizeof(bf16) * (size_t)u->bmax * u->lev[level].V * C);
}

int round1k(int b) { return (b + 1023) & ~1023; }
// unused shared memory after the barriers: operand descriptors address only the stage buffers,
// and this margin keeps every address an MMA could form from a descriptor inside the CTA's
// allocation
constexpr int kSmemGuard = 16 * 1024;
// stage buffers are 1024-byte aligned (the 128-byte swizzle atom), see k_conv
// Four stages: the CTAs are latency-bound chains of small TMA boxes, and at 16-32 channels four
// stages keep 5-6 CTAs resident per SM, which measured faster (12.0 vs 13.7 ms per training
// iteration on 160x160x80) than eight stages at three CTAs.
int conv_stages(int ck, int n) {
    const int stage = round1k(128 * ck * 2) + round1k(n * ck * 2);
    return std::max(2, std::min(4, (184 * 1024) / stage));
}
int conv_smem(int ck, int n) {
    const int S = conv_stages(ck, n);
    return S * (round1k(128 * ck * 2) + round1k(n * ck * 2)) + 1024 + (2 * S + 1) * 8 + 16 + kSmemGuard;
}
// Two stages: a stage holds a 32 KB A tile, so two stages let two CTAs share an SM; measured
// faster (9.5 vs 12.0 ms per training iteration) than five stages at one CTA per SM.
int wgrad_stages(int cout) {
    (void)cout;
    return 2;
}
int wgrad_smem(int cout) {
    const int S = wgrad_stages(cout);
    return S * (128 * 128 * 2 + 128 * cout * 2) + 1024 + (2 * S + 1) * 8 + 16 + kSmemGuard;
}

// one implicit-GEMM convolution: in (map mA, chunk ck, K channels cin) x weights (map mB) ->
// output channels n into out / out32
int launch_conv(pl_unet u, const CUtensorMap &mA, const CUtensorMap &mB, int level, int cin, int ck, int n, int taps,
                int batch, const float *bias, int relu, const bf16 *mask, int mask_ld, bf16 *out, int out_ld,
                int out_off, float *out32) {
    const Level &lv = u->lev[level];
    pl::unet::ConvArgs a;
    memset(&a, 0, sizeof a);
    a.X = lv.X; a.Y = lv.Y; a.Z = lv.Z;
    a.cin = cin; a.cout = n; a.taps = taps; a.ck = ck;
    a.tx = lv.tx; a.ty = lv.ty; a.ntx = lv.ntx;
    a.stages = conv_stages(ck, n);
    a.bias = bias; a.relu = relu; a.mask = mask; a.mask_ld = mask_ld;
    a.out = out; a.out_ld = out_ld; a.out_off = out_off; a.out32 = out32;
    a.err = u->err;
    dim3 grid(lv.ntx * lv.nty, lv.Z, batch);
    pl::unet::k_conv<<<grid, 128, conv_smem(ck, n), u->st>>>(mA, mB, a);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? PL_OK : uerr(PL_ERR_CUDA, "k_conv launch: %s", cudaGetErrorString(e));
}

int launch_wgrad(pl_unet u, Conv &c, int batch) {
    const Level &lv = u->lev[c.level];
    pl::unet::WgradArgs a;
    memset(&a, 0, sizeof a);
    a.X = lv.X; a.Y = lv.Y; a.Z = lv.Z; a.B = batch;
    a.cin = c.cin; a.cout = c.cout; a.taps = c.taps;
    a.cw = chunk(c.cin);
    a.nw = std::min(64, c.cout);
    a.tx = lv.tx; a.ty = lv.ty; a.ntx = lv.ntx; a.nty = lv.nty;
    a.ktiles = batch * lv.Z * lv.nty * lv.ntx;
    a.stages = wgrad_stages(c.cout);
    a.dw = c.gw;
    a.err = u->err;
    const int blocks = c.taps * (c.cin / a.cw);
    const int mtiles = (blocks + (128 / a.cw) - 1) / (128 / a.cw);
    int ksplit = std::max(1, std::min(a.ktiles, (2 * 152 + mtiles - 1) / mtiles));
    a.kper = (a.ktiles + ksplit - 1) / ksplit;
    ksplit = (a.ktiles + a.kper - 1) / a.kper;
    pl::unet::k_wgrad<<<dim3(mtiles, ksplit), 128, wgrad_smem(c.cout), u->st>>>(c.mapX, c.mapD, a);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return uerr(PL_ERR_CUDA, "k_wgrad launch: %s", cudaGetErrorString(e));
    const long long nvox = (long long)batch * lv.V;
    pl::unet::k_bias_grad<<<std::min<long long>(1024, (nvox + 255) / 256 + 1), 256, 0, u->st>>>(c.dz.p, c.cout, nvox, c.gb);
    e = cudaGetLastError();
    return e == cudaSuccess ? PL_OK : uerr(PL_ERR_CUDA, "k_bias_grad launch: %s", cudaGetErrorString(e));
}

unsigned blocks_for(long long n, int bs = 256) { return unsigned((n + bs - 1) / bs); }

int forward(pl_unet u, int batch) {
    const int L = u->L;
    int r;
    for (int l = 0; l < L; ++l) {
        const Level &lv = u->lev[l];
        if (l > 0) {
            const Buf &src = (l - 1 < L - 1) ? u->cat[l - 1] : u->bot;
            const Level &up = u->lev[l - 1];
            const long long tot = (long long)batch * lv.V * (u->pool[l - 1].C / 8);
            pl::unet::k_pool<<<blocks_for(tot), 256, 0, u->st>>>(src.p, src.C, 0, u->pool[l - 1].p, u->pool[l - 1].C,
                                                                 up.X, up.Y, up.Z, batch);
        }
        for (int k = 0; k < 2; ++k) {
            Conv &c = u->convs[2 * l + k];
            if ((r = launch_conv(u, c.mapX, c.mapW, l, c.cin, chunk(c.cin), c.cout, c.taps, batch, c.b, c.relu, nullptr,
                                 0, c.out.p, c.out.C, c.out_off, nullptr)))
                return r;
        }
    }
    int ci = 2 * L;
    for (int l = L - 2; l >= 0; --l) {
        const Level &lv = u->lev[l];
        const Buf &low = (l == L - 2) ? u->bot : u->d2[l + 1];
        const long long tot = (long long)batch * lv.V * (low.C / 8);
        pl::unet::k_upsample<<<blocks_for(tot), 256, 0, u->st>>>(low.p, low.C, u->cat[l].p, u->cat[l].C, u->e1[l].C,
                                                                 lv.X, lv.Y, lv.Z, batch);
        for (int k = 0; k < 2; ++k, ++ci) {
            Conv &c = u->convs[ci];
            if ((r = launch_conv(u, c.mapX, c.mapW, l, c.cin, chunk(c.cin), c.cout, c.taps, batch, c.b, c.relu, nullptr,
                                 0, c.out.p, c.out.C, c.out_off, nullptr)))
                return r;
        }
    }
    Conv &h = u->convs.back();
    return launch_conv(u, h.mapX, h.mapW, 0, h.cin, chunk(h.cin), h.cout, 1, batch, h.b, 0, nullptr, 0, nullptr, 0, 0,
                       u->pred);
}

// backward of conv c: weight and bias gradients, then (if needed) the input gradient
int conv_back(pl_unet u, Conv &c, int batch) {
    int r;
    if ((r = launch_wgrad(u, c, batch))) return r;
    if (!c.need_dgrad) return PL_OK;
    const bf16 *mask = c.din_mask ? c.din_mask->p : nullptr;
    const int mld = c.din_mask ? c.din_mask->C : 0;
    return launch_conv(u, c.mapD, c.mapWt, c.level, c.cout, chunk(c.cout), c.cin, c.taps, batch, nullptr, 0, mask, mld,
                       c.din.p, c.din.C, 0, nullptr);
}

int backward(pl_unet u, int batch) {
    const int L = u->L;
    int r;
    for (auto &c : u->convs) {
        UCK(cudaMemsetAsync(c.gw, 0, sizeof(float) * c.nw(), u->st));
        UCK(cudaMemsetAsync(c.gb, 0, sizeof(float) * c.cout, u->st));
    }
    if ((r = conv_back(u, u->convs.back(), batch))) return r;          // head -> gd2[0]
    // decoder, level 0 upwards (reverse of the forward order)
    int ci = (int)u->convs.size() - 2;
    for (int l = 0; l <= L - 2; ++l, ci -= 2) {
        Conv &c2 = u->convs[ci], &c1 = u->convs[ci - 1];
        if ((r = conv_back(u, c2, batch))) return r;                   // gd2 -> gd1
        if ((r = conv_back(u, c1, batch))) return r;                   // gd1 -> gcat (masked by cat)
        const Level &lv = u->lev[l];
        Buf &dlow = (l + 1 == L - 1) ? u->gbot : u->gd2[l + 1];
        const long long tot = (long long)batch * u->lev[l + 1].V * (dlow.C / 8);
        pl::unet::k_upsample_back<<<blocks_for(tot), 256, 0, u->st>>>(u->gcat[l].p, u->gcat[l].C, u->e1[l].C, dlow.p,
                                                                     dlow.C, lv.X, lv.Y, lv.Z, batch);
    }
    // bottom and encoder, deepest first
    for (int l = L - 1; l >= 0; --l) {
        Conv &c1 = u->convs[2 * l], &c2 = u->convs[2 * l + 1];
        if (l < L - 1) {
            const Level &lv = u->lev[l];
            const long long tot = (long long)batch * lv.V * (u->ge2[l].C / 8);
            pl::unet::k_pool_back<<<blocks_for(tot), 256, 0, u->st>>>(u->gcat[l].p, u->gcat[l].C, u->gpool[l].p,
                                                                     u->cat[l].p, u->cat[l].C, u->ge2[l].p, u->ge2[l].C,
                                                                     lv.X, lv.Y, lv.Z, batch);
        }
        if ((r = conv_back(u, c2, batch))) return r;
        if ((r = conv_back(u, c1, batch))) return r;
    }
    return PL_OK;
}

int adam(pl_unet u, double lr, float gscale) {
    ++u->step;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float bc1 = float(1.0 - std::pow(0.9, double(u->step))), bc2 = float(1.0 - std::pow(0.999, double(u->step)));
    for (auto &c : u->convs) {
        pl::unet::k_adam<<<blocks_for(c.nw()), 256, 0, u->st>>>(c.w, c.gw, c.mw, c.vw, c.nw(), float(lr), b1, b2, eps, bc1,
                                                                bc2, gscale, c.wb, c.wt, c.cout, c.taps, c.cin);
        pl::unet::k_adam<<<blocks_for(c.cout), 256, 0, u->st>>>(c.b, c.gb, c.mb, c.vb, c.cout, float(lr), b1, b2, eps, bc1,
                                                               bc2, gscale, nullptr, nullptr, 0, 1, 1);
    }
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? PL_OK : uerr(PL_ERR_CUDA, "adam: %s", cudaGetErrorString(e));
}

int refresh_bf16(pl_unet u) {
    for (auto &c : u->convs)
        pl::unet::k_weights_bf16<<<blocks_for(c.nw()), 256, 0, u->st>>>(c.w, c.nw(), c.wb, c.wt, c.cout, c.taps, c.cin);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? PL_OK : uerr(PL_ERR_CUDA, "weights: %s", cudaGetErrorString(e));
}

int check_err(pl_unet u) {
    int h = 0;
    UCK(cudaMemcpyAsync(&h, u->err, sizeof h, cudaMemcpyDeviceToHost, u->st));
    UCK(cudaStreamSynchronize(u->st));
    if (h) {
        cudaMemsetAsync(u->err, 0, sizeof(int), u->st);
        return uerr(PL_ERR_CUDA, "tensor-core pipeline wait timed out (flags %d)", h);
    }
    return PL_OK;
}

int build(pl_unet u) {
    int r;
    const int L = u->L;
    auto C = [&](int l) { return u->base << l; };
    if ((r = mkbuf(u, u->in0, u->cin, 0))) return r;
    u->e1.resize(L); u->cat.resize(L); u->pool.resize(L); u->d1.resize(L); u->d2.resize(L);
    u->ge1.resize(L); u->ge2.resize(L); u->gd1.resize(L); u->gd2.resize(L); u->gcat.resize(L); u->gpool.resize(L);
    for (int l = 0; l < L; ++l) {
        if ((r = mkbuf(u, u->e1[l], C(l), l)) || (r = mkbuf(u, u->ge1[l], C(l), l))) return r;
        if (l < L - 1) {
            if ((r = mkbuf(u, u->cat[l], C(l) + C(l + 1), l)) || (r = mkbuf(u, u->gcat[l], C(l) + C(l + 1), l)) ||
                (r = mkbuf(u, u->pool[l], C(l), l + 1)) || (r = mkbuf(u, u->gpool[l], C(l), l + 1)) ||
                (r = mkbuf(u, u->d1[l], C(l), l)) || (r = mkbuf(u, u->d2[l], C(l), l)) ||
                (r = mkbuf(u, u->gd1[l], C(l), l)) || (r = mkbuf(u, u->gd2[l], C(l), l)) ||
                (r = mkbuf(u, u->ge2[l], C(l), l)))
                return r;
        }
    }
    if ((r = mkbuf(u, u->bot, C(L - 1), L - 1)) || (r = mkbuf(u, u->gbot, C(L - 1), L - 1))) return r;
    u->ge2[L - 1] = u->gbot;
    const long long V0 = u->lev[0].V;
    if ((r = ualloc(u, (void **)&u->pred, sizeof(float) * u->bmax * V0 * u->cout))) return r;
    if ((r = ualloc(u, (void **)&u->dpred, sizeof(bf16) * u->bmax * V0 * u->cout))) return r;
    if ((r = ualloc(u, (void **)&u->tgt, sizeof(bf16) * u->bmax * V0 * u->cout))) return r;
    if ((r = ualloc(u, (void **)&u->dacc, sizeof(double) * 2))) return r;
    if ((r = ualloc(u, (void **)&u->err, sizeof(int)))) return r;
    // layers
    u->convs.clear();
    for (int l = 0; l < L; ++l) {
        Conv c1, c2;
        c1.level = c2.level = l;
        c1.cin = l == 0 ? u->cin : C(l - 1); c1.cout = C(l);
        c1.in = l == 0 ? u->in0 : u->pool[l - 1];
        c1.out = u->e1[l];
        c1.dz = u->ge1[l];
        c1.need_dgrad = l > 0;
        if (l > 0) c1.din = u->gpool[l - 1];
        c2.cin = C(l); c2.cout = C(l);
        c2.in = u->e1[l];
        c2.out = l < L - 1 ? u->cat[l] : u->bot;
        c2.dz = u->ge2[l];
        c2.din = u->ge1[l];
        u->convs.push_back(c1);
        u->convs.push_back(c2);
    }
    for (int l = L - 2; l >= 0; --l) {
        Conv c1, c2;
        c1.level = c2.level = l;
        c1.cin = C(l) + C(l + 1); c1.cout = C(l);
        c1.in = u->cat[l]; c1.out = u->d1[l]; c1.dz = u->gd1[l]; c1.din = u->gcat[l];
        c2.cin = C(l); c2.cout = C(l);
        c2.in = u->d1[l]; c2.out = u->d2[l]; c2.dz = u->gd2[l]; c2.din = u->gd1[l];
        u->convs.push_back(c1);
        u->convs.push_back(c2);
    }
    {
        Conv h;
        h.level = 0; h.cin = C(0); h.cout = u->cout; h.taps = 1; h.relu = 0;
        h.in = L > 1 ? u->d2[0] : u->bot;
        h.dz.p = u->dpred; h.dz.C = u->cout; h.dz.level = 0;
        h.din = L > 1 ? u->gd2[0] : u->gbot;
        u->convs.push_back(h);
    }
    // masks of the input gradients: the ReLU derivative of the tensor each conv reads
    for (auto &c : u->convs) {
        if (!c.need_dgrad) continue;
        if (c.in.p == nullptr) continue;
        bool is_pool = false;
        for (int l = 0; l + 1 < L; ++l) is_pool |= (c.in.p == u->pool[l].p);
        if (is_pool) continue;   // pooling is linear: no mask
        c.din_mask = &c.in;
    }
    // parameters and maps
    for (auto &c : u->convs) {
        const long long nw = c.nw();
        if ((r = ualloc(u, (void **)&c.w, sizeof(float) * nw)) || (r = ualloc(u, (void **)&c.gw, sizeof(float) * nw)) ||
            (r = ualloc(u, (void **)&c.mw, sizeof(float) * nw)) || (r = ualloc(u, (void **)&c.vw, sizeof(float) * nw)) ||
            (r = ualloc(u, (void **)&c.b, sizeof(float) * c.cout)) || (r = ualloc(u, (void **)&c.gb, sizeof(float) * c.cout)) ||
            (r = ualloc(u, (void **)&c.mb, sizeof(float) * c.cout)) || (r = ualloc(u, (void **)&c.vb, sizeof(float) * c.cout)) ||
            (r = ualloc(u, (void **)&c.wb, sizeof(bf16) * nw)) || (r = ualloc(u, (void **)&c.wt, sizeof(bf16) * nw)))
            return r;
        const Level &lv = u->lev[c.level];
        if ((r = map_act(&c.mapX, c.in.p, c.in.C, lv.X, lv.Y, lv.Z, u->bmax, chunk(c.cin), lv.tx, lv.ty))) return r;
        if ((r = map_w(&c.mapW, c.wb, c.taps * c.cin, c.cout, chunk(c.cin)))) return r;
        if ((r = map_act(&c.mapD, c.dz.p, c.cout, lv.X, lv.Y, lv.Z, u->bmax, chunk(c.cout), lv.tx, lv.ty))) return r;
        if ((r = map_w(&c.mapWt, c.wt, c.taps * c.cout, c.cin, chunk(c.cout)))) return r;
        if (c.in.C != c.cin) return uerr(PL_ERR_ARG, "internal: conv input has %d channels, expected %d", c.in.C, c.cin);
        u->smem_conv_max = std::max(u->smem_conv_max, std::max(conv_smem(chunk(c.cin), c.cout), conv_smem(chunk(c.cout), c.cin)));
        u->smem_wgrad_max = std::max(u->smem_wgrad_max, wgrad_smem(c.cout));
    }
    UCK(cudaFuncSetAttribute(pl::unet::k_conv, cudaFuncAttributeMaxDynamicSharedMemorySize, u->smem_conv_max));
    UCK(cudaFuncSetAttribute(pl::unet::k_wgrad, cudaFuncAttributeMaxDynamicSharedMemorySize, u->smem_wgrad_max));
    return PL_OK;
}

int init_params(pl_unet u, unsigned long long seed) {
    std::mt19937_64 rng(seed);
    std::normal_distribution<float> nd(0.f, 1.f);
    for (size_t k = 0; k < u->convs.size(); ++k) {
        Conv &c = u->convs[k];
        const bool head = k + 1 == u->convs.size();
        const float sd = head ? std::sqrt(1.0f / float(c.taps * c.cin)) : std::sqrt(2.0f / float(c.taps * c.cin));
        std::vector<float> w(c.nw()), b(c.cout, 0.f);
        for (auto &x : w) x = sd * nd(rng);
        UCK(cudaMemcpyAsync(c.w, w.data(), sizeof(float) * w.size(), cudaMemcpyHostToDevice, u->st));
        UCK(cudaMemcpyAsync(c.b, b.data(), sizeof(float) * b.size(), cudaMemcpyHostToDevice, u->st));
        UCK(cudaMemsetAsync(c.mw, 0, sizeof(float) * c.nw(), u->st));
        UCK(cudaMemsetAsync(c.vw, 0, sizeof(float) * c.nw(), u->st));
        UCK(cudaMemsetAsync(c.mb, 0, sizeof(float) * c.cout, u->st));
        UCK(cudaMemsetAsync(c.vb, 0, sizeof(float) * c.cout, u->st));
        UCK(cudaStreamSynchronize(u->st));
    }
    u->step = 0;
    return refresh_bf16(u);
}

}  // namespace

// -------------------------------------------------------------------------------------- C ABI
extern "C" {

int pl_unet_create(int nx, int ny, int nz, int levels, int base_channels, int in_channels, int out_channels,
                   int max_batch, pl_unet *out) {
    if (!out) return uerr(PL_ERR_ARG, "out is NULL");
    *out = nullptr;
    if (levels < 1 || levels > 5 || base_channels < 16 || base_channels % 16 || (base_channels << (levels - 1)) > 256 ||
        in_channels != 16 || out_channels != 16 || max_batch < 1)
        return uerr(PL_ERR_ARG, "unsupported U-Net shape (levels 1..5, base a multiple of 16 with base*2^(levels-1) <= "
                                "256, 16 input and 16 output channels)");
    const int f = 1 << (levels - 1);
    if (nx < 4 * f || ny < 1 * f || nz < f || nx % f || ny % f || nz % f)
        return uerr(PL_ERR_ARG, "volume %d x %d x %d must be divisible by 2^(levels-1) = %d (x >= %d)", nx, ny, nz, f, 4 * f);
    if (!encode_fn()) return uerr(PL_ERR_CUDA, "cuTensorMapEncodeTiled is unavailable");
    pl_unet u = new pl_unet_s();
    u->L = levels; u->base = base_channels; u->cin = in_channels; u->cout = out_channels; u->bmax = max_batch;
    if (cudaStreamCreateWithFlags(&u->st, cudaStreamNonBlocking) != cudaSuccess) {
        delete u;
        return uerr(PL_ERR_CUDA, "cudaStreamCreate failed (no CUDA device?)");
    }
    for (int l = 0; l < levels; ++l) {
        Level lv;
        lv.X = nx >> l; lv.Y = ny >> l; lv.Z = nz >> l;
        lv.V = (long long)lv.X * lv.Y * lv.Z;
        lv.tx = 32;
        while (lv.tx > 4 && lv.X % lv.tx) lv.tx /= 2;
        if (lv.tx > lv.X) lv.tx = 4;
        lv.ty = 128 / lv.tx;
        lv.ntx = (lv.X + lv.tx - 1) / lv.tx;
        lv.nty = (lv.Y + lv.ty - 1) / lv.ty;
        u->lev.push_back(lv);
    }
    int r = build(u);
    if (!r) r = init_params(u, 1234);
    if (r) { pl_unet_destroy(u); return r; }
    *out = u;
    return PL_OK;
}

int pl_unet_destroy(pl_unet u) {
    if (!u) return PL_OK;
    if (u->st) cudaStreamSynchronize(u->st);
    for (void *p : u->allocs) cudaFree(p);
    if (u->st) cudaStreamDestroy(u->st);
    delete u;
    return PL_OK;
}

long long pl_unet_param_count(pl_unet u) {
    if (!u) return -1;
    long long n = 0;
    for (auto &c : u->convs) n += c.nw() + c.cout;
    return n;
}

int pl_unet_init_params(pl_unet u, unsigned long long seed) {
    if (!u) return uerr(PL_ERR_ARG, "null handle");
    return init_params(u, seed);
}

int pl_unet_get_params(pl_unet u, float *host) {
    if (!u || !host) return uerr(PL_ERR_ARG, "bad arguments");
    size_t o = 0;
    for (auto &c : u->convs) {
        UCK(cudaMemcpyAsync(host + o, c.w, sizeof(float) * c.nw(), cudaMemcpyDeviceToHost, u->st));
        o += c.nw();
        UCK(cudaMemcpyAsync(host + o, c.b, sizeof(float) * c.cout, cudaMemcpyDeviceToHost, u->st));
        o += c.cout;
    }
    UCK(cudaStreamSynchronize(u->st));
    return PL_OK;
}

int pl_unet_set_params(pl_unet u, const float *host) {
    if (!u || !host) return uerr(PL_ERR_ARG, "bad arguments");
    size_t o = 0;
    for (auto &c : u->convs) {
        UCK(cudaMemcpyAsync(c.w, host + o, sizeof(float) * c.nw(), cudaMemcpyHostToDevice, u->st));
        o += c.nw();
        UCK(cudaMemcpyAsync(c.b, host + o, sizeof(float) * c.cout, cudaMemcpyHostToDevice, u->st));
        o += c.cout;
    }
    int r = refresh_bf16(u);
    if (r) return r;
    UCK(cudaStreamSynchronize(u->st));
    return PL_OK;
}

int pl_unet_gradients(pl_unet u, float *host) {
    if (!u || !host) return uerr(PL_ERR_ARG, "bad arguments");
    size_t o = 0;
    for (auto &c : u->convs) {
        UCK(cudaMemcpyAsync(host + o, c.gw, sizeof(float) * c.nw(), cudaMemcpyDeviceToHost, u->st));
        o += c.nw();
        UCK(cudaMemcpyAsync(host + o, c.gb, sizeof(float) * c.cout, cudaMemcpyDeviceToHost, u->st));
        o += c.cout;
    }
    UCK(cudaStreamSynchronize(u->st));
    return PL_OK;
}

int pl_unet_forward(pl_unet u, int batch, const float *x_host, float *y_host) {
    if (!u || !x_host || batch < 1 || batch > u->bmax) return uerr(PL_ERR_ARG, "bad arguments");
    const long long V0 = u->lev[0].V;
    const long long nx = (long long)batch * V0 * u->cin;
    std::vector<bf16> xb(nx);
    for (long long i = 0; i < nx; ++i) xb[i] = __float2bfloat16_rn(x_host[i]);
    UCK(cudaMemcpyAsync(u->in0.p, xb.data(), sizeof(bf16) * nx, cudaMemcpyHostToDevice, u->st));
    int r = forward(u, batch);
    if (r) return r;
    if ((r = check_err(u))) return r;
    if (y_host) {
        UCK(cudaMemcpyAsync(y_host, u->pred, sizeof(float) * batch * V0 * u->cout, cudaMemcpyDeviceToHost, u->st));
        UCK(cudaStreamSynchronize(u->st));
    }
    return PL_OK;
}

int pl_unet_backward(pl_unet u, int batch, const float *dy_host) {
    if (!u || !dy_host || batch < 1 || batch > u->bmax) return uerr(PL_ERR_ARG, "bad arguments");
    const long long n = (long long)batch * u->lev[0].V * u->cout;
    std::vector<bf16> d(n);
    for (long long i = 0; i < n; ++i) d[i] = __float2bfloat16_rn(dy_host[i]);
    UCK(cudaMemcpyAsync(u->dpred, d.data(), sizeof(bf16) * n, cudaMemcpyHostToDevice, u->st));
    int r = backward(u, batch);
    if (r) return r;
    return check_err(u);
}

int pl_unet_dataset_reserve(pl_unet u, int nsamples, int targets) {
    if (!u || nsamples < 1 || targets < 1 || targets > u->cout) return uerr(PL_ERR_ARG, "bad arguments");
    const long long V0 = u->lev[0].V;
    int r;
    if (u->ds_design) return uerr(PL_ERR_STATE, "dataset already reserved");
    if ((r = ualloc(u, (void **)&u->ds_design, sizeof(float) * nsamples * V0)) ||
        (r = ualloc(u, (void **)&u->ds_target, sizeof(float) * nsamples * V0 * targets)) ||
        (r = ualloc(u, (void **)&u->mean, sizeof(float) * 16)) || (r = ualloc(u, (void **)&u->inv_std, sizeof(float) * 16)) ||
        (r = ualloc(u, (void **)&u->stdv, sizeof(float) * 16)) ||
        (r = ualloc(u, (void **)&u->design_tmp, sizeof(float) * V0)) ||
        (r = ualloc(u, (void **)&u->pred64, sizeof(double) * V0 * targets)))
        return r;
    u->nds = nsamples;
    u->cused = targets;
    u->h_mean.assign(16, 0.f);
    u->h_std.assign(16, 1.f);
    return PL_OK;
}

int pl_unet_set_static(pl_unet u, const float *feat, int nfeat) {
    if (!u || !feat || nfeat < 0 || nfeat > u->cin - 1) return uerr(PL_ERR_ARG, "bad arguments (at most %d static features)", u->cin - 1);
    const long long V0 = u->lev[0].V;
    int r;
    if (!u->stat && (r = ualloc(u, (void **)&u->stat, sizeof(float) * V0 * (u->cin - 1)))) return r;
    UCK(cudaMemcpyAsync(u->stat, feat, sizeof(float) * V0 * nfeat, cudaMemcpyHostToDevice, u->st));
    UCK(cudaStreamSynchronize(u->st));
    u->nstat = nfeat;
    return PL_OK;
}

int pl_unet_add_sample(pl_unet u, int slot, const double *design, const double *targets) {
    if (!u || !design || !targets || slot < 0 || slot >= u->nds) return uerr(PL_ERR_ARG, "bad arguments");
    const long long V0 = u->lev[0].V;
    std::vector<float> d(V0), t(V0 * u->cused);
    for (long long v = 0; v < V0; ++v) d[v] = float(design[v]);
    for (int c = 0; c < u->cused; ++c)
        for (long long v = 0; v < V0; ++v) t[v * u->cused + c] = float(targets[c * V0 + v]);
    UCK(cudaMemcpyAsync(u->ds_design + slot * V0, d.data(), sizeof(float) * V0, cudaMemcpyHostToDevice, u->st));
    UCK(cudaMemcpyAsync(u->ds_target + slot * V0 * u->cused, t.data(), sizeof(float) * V0 * u->cused,
                        cudaMemcpyHostToDevice, u->st));
    UCK(cudaStreamSynchronize(u->st));
    return PL_OK;
}

int pl_unet_add_sample_lattice(pl_unet u, int slot, const double *design, pl_lattice h) {
    if (!u || !design || !h || slot < 0 || slot >= u->nds) return uerr(PL_ERR_ARG, "bad arguments");
    const long long V0 = u->lev[0].V;
    pl::unet::SampleSrc src;
    memset(&src, 0, sizeof src);
    long long n = 0;
    int r = pl::lattice_sample_fields(h, src.f, &n);
    if (r) return r;
    if (n != V0) return uerr(PL_ERR_ARG, "lattice has %lld nodes, the network %lld voxels", n, V0);
    if (u->cused > 13) return uerr(PL_ERR_ARG, "a lattice sample has 13 target fields");
    // order the lattice's work before the copy: its stream finishes the solve first
    UCK(cudaStreamSynchronize(pl::lattice_stream(h)));
    std::vector<float> d(V0);
    for (long long v = 0; v < V0; ++v) d[v] = float(design[v]);
    UCK(cudaMemcpyAsync(u->ds_design + slot * V0, d.data(), sizeof(float) * V0, cudaMemcpyHostToDevice, u->st));
    pl::unet::k_capture<<<blocks_for(V0 * u->cused), 256, 0, u->st>>>(src, u->cused, V0,
                                                                      u->ds_target + slot * V0 * u->cused);
    UCK(cudaGetLastError());
    UCK(cudaStreamSynchronize(u->st));
    return PL_OK;
}

int pl_unet_set_norm(pl_unet u, const float *mean, const float *stdv) {
    if (!u || !mean || !stdv || !u->mean) return uerr(PL_ERR_ARG, "bad arguments (reserve the dataset first)");
    for (int c = 0; c < u->cused; ++c) {
        u->h_mean[c] = mean[c];
        u->h_std[c] = stdv[c] > 0 ? stdv[c] : 1.f;
    }
    std::vector<float> inv(16, 1.f);
    for (int c = 0; c < 16; ++c) inv[c] = 1.f / u->h_std[c];
    UCK(cudaMemcpyAsync(u->mean, u->h_mean.data(), sizeof(float) * 16, cudaMemcpyHostToDevice, u->st));
    UCK(cudaMemcpyAsync(u->stdv, u->h_std.data(), sizeof(float) * 16, cudaMemcpyHostToDevice, u->st));
    UCK(cudaMemcpyAsync(u->inv_std, inv.data(), sizeof(float) * 16, cudaMemcpyHostToDevice, u->st));
    UCK(cudaStreamSynchronize(u->st));
    return PL_OK;
}

int pl_unet_get_norm(pl_unet u, float *mean, float *stdv) {
    if (!u || !mean || !stdv || !u->mean) return uerr(PL_ERR_ARG, "bad arguments");
    for (int c = 0; c < u->cused; ++c) { mean[c] = u->h_mean[c]; stdv[c] = u->h_std[c]; }
    return PL_OK;
}

int pl_unet_train(pl_unet u, int nsamples, int epochs, int batch, double lr, unsigned long long seed,
                  double *loss_per_epoch) {
    if (!u || nsamples < 1 || nsamples > u->nds || epochs < 1 || batch < 1 || batch > u->bmax || !(lr > 0))
        return uerr(PL_ERR_ARG, "bad arguments");
    const long long V0 = u->lev[0].V;
    int r;
    // target normalisation from the samples used
    {
        UCK(cudaMemsetAsync(u->dacc, 0, sizeof(double) * 2, u->st));
        double *d = nullptr;
        UCK(cudaMalloc((void **)&d, sizeof(double) * 32));
        UCK(cudaMemsetAsync(d, 0, sizeof(double) * 32, u->st));
        pl::unet::k_channel_stats<<<1024, 256, 0, u->st>>>(u->ds_target, (long long)nsamples * V0, u->cused, d, d + 16);
        std::vector<double> h(32);
        UCK(cudaMemcpyAsync(h.data(), d, sizeof(double) * 32, cudaMemcpyDeviceToHost, u->st));
        UCK(cudaStreamSynchronize(u->st));
        cudaFree(d);
        std::vector<float> mean(16, 0.f), sd(16, 1.f);
        const double n = double(nsamples) * V0;
        for (int c = 0; c < u->cused; ++c) {
            mean[c] = float(h[c] / n);
            const double var = std::max(0.0, h[16 + c] / n - (h[c] / n) * (h[c] / n));
            sd[c] = var > 1e-30 ? float(std::sqrt(var)) : 1.f;
        }
        if ((r = pl_unet_set_norm(u, mean.data(), sd.data()))) return r;
    }
    std::mt19937_64 rng(seed);
    std::vector<int> perm(nsamples);
    for (int i = 0; i < nsamples; ++i) perm[i] = i;
    const double scale = 1.0 / (double(V0) * u->cused);
    for (int ep = 0; ep < epochs; ++ep) {
        std::shuffle(perm.begin(), perm.end(), rng);
        // cosine decay of the learning rate from lr to lr / 20 over the epochs
        const double ep_lr = lr * (0.05 + 0.95 * 0.5 * (1.0 + std::cos(3.14159265358979323846 * ep / std::max(1, epochs - 1))));
        UCK(cudaMemsetAsync(u->dacc, 0, sizeof(double), u->st));
        int nb = 0;
        for (int s0 = 0; s0 + batch <= nsamples; s0 += batch, ++nb) {
            for (int b = 0; b < batch; ++b) {
                const int k = perm[s0 + b];
                pl::unet::k_make_input<<<blocks_for(V0 * u->cin), 256, 0, u->st>>>(
                    u->ds_design + k * V0, u->stat, u->nstat, V0, u->cin, u->in0.p + b * V0 * u->cin);
                pl::unet::k_make_target<<<blocks_for(V0 * u->cout), 256, 0, u->st>>>(
                    u->ds_target + k * V0 * u->cused, u->cused, u->mean, u->inv_std, V0, u->cout, u->tgt + b * V0 * u->cout);
            }
            if ((r = forward(u, batch))) return r;
            pl::unet::k_mse<<<blocks_for((long long)batch * V0 * u->cout), 256, 0, u->st>>>(
                u->pred, u->tgt, u->dpred, u->cout, u->cused, (long long)batch * V0, scale / batch, u->dacc);
            if ((r = backward(u, batch))) return r;
            if ((r = adam(u, ep_lr, 1.0f))) return r;
        }
        double acc = 0;
        UCK(cudaMemcpyAsync(&acc, u->dacc, sizeof(double), cudaMemcpyDeviceToHost, u->st));
        if ((r = check_err(u))) return r;
        if (loss_per_epoch) loss_per_epoch[ep] = acc / (double(nb) * batch * V0 * u->cused);
    }
    return PL_OK;
}

int pl_unet_predict(pl_unet u, const double *design, double *out) {
    if (!u || !design || !out || !u->mean) return uerr(PL_ERR_ARG, "bad arguments (reserve and train first)");
    const long long V0 = u->lev[0].V;
    std::vector<float> d(V0);
    for (long long v = 0; v < V0; ++v) d[v] = float(design[v]);
    UCK(cudaMemcpyAsync(u->design_tmp, d.data(), sizeof(float) * V0, cudaMemcpyHostToDevice, u->st));
    pl::unet::k_make_input<<<blocks_for(V0 * u->cin), 256, 0, u->st>>>(u->design_tmp, u->stat, u->nstat, V0, u->cin,
                                                                        u->in0.p);
    int r = forward(u, 1);
    if (r) return r;
    pl::unet::k_denorm<<<blocks_for(V0 * u->cused), 256, 0, u->st>>>(u->pred, u->cout, u->cused, u->mean, u->stdv, V0,
                                                                     u->pred64);
    if ((r = check_err(u))) return r;
    UCK(cudaMemcpyAsync(out, u->pred64, sizeof(double) * V0 * u->cused, cudaMemcpyDeviceToHost, u->st));
    UCK(cudaStreamSynchronize(u->st));
    return PL_OK;
}

}  // extern "C"
