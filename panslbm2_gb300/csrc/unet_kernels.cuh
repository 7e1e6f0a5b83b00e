// unet_kernels.cuh -- device kernels of the learned warm start: a 3D convolutional U-Net over
// channels-last BF16 activations [B][Z][Y][X][C], trained and evaluated on the GB300's 5th-
// generation tensor cores.
//
//  k_conv   implicit-GEMM 3x3x3 (or 1x1x1) convolution, used for the forward pass and for the
//           input gradient (dgrad: the same GEMM with the flipped, transposed weights). One CTA
//           computes 128 output voxels (a tx x ty patch of one z slice) x all N output channels:
//           D[128 x N] (FP32, TMEM) = sum over taps and input-channel chunks of
//           A[128 voxels x ck] (TMA box of the input, shifted by the tap, zero-filled outside the
//           volume) x B[N x ck] (TMA box of the weights), both K-major in shared memory.
//           Warp 0 issues the TMA loads, warp 1 the tcgen05.mma, all four warps read the
//           accumulator back (tcgen05.ld) for the epilogue (bias, ReLU, ReLU-derivative mask,
//           BF16 store into a channel slice of the output).
//  k_wgrad  weight gradient dW[co][tap][ci] = sum_v dZ[v][co] X[v + tap][ci]: D[128 rows of
//           (tap, ci) x N = Cout] accumulated over 128-voxel K steps, A assembled from
//           128 / cw TMA boxes of X (one per (tap, channel block)), B one box of dZ: both tiles
//           arrive voxel-major, i.e. MN-major operands. Split over voxel ranges; the FP32 partial
//           sums are added into dW with atomics.
//  elementwise: average pooling and its adjoint, nearest upsampling into the concatenation and
//           its adjoint, bias gradient, loss, Adam, batch assembly.
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

#include "tc.cuh"

namespace pl {
namespace unet {

using bf16 = __nv_bfloat16;

enum UErr { UERR_TIMEOUT_PRODUCER = 1, UERR_TIMEOUT_MMA = 2, UERR_TIMEOUT_EPILOGUE = 4 };

struct ConvArgs {
    int X, Y, Z;            // volume of this level
    int cin, cout;          // K channels per tap, N
    int taps;               // 27 (3x3x3, tap = (dz+1)*9 + (dy+1)*3 + dx+1) or 1
    int ck;                 // input channels per stage (16, 32 or 64; = swizzle span / 2)
    int tx, ty, ntx;        // 128-voxel patch (tx * ty = 128), patches per x row
    int stages;
    const float *bias;      // [cout] or null
    int relu;               // apply ReLU in the epilogue
    const bf16 *mask;       // multiply by (mask > 0): the ReLU derivative of the layer below
    int mask_ld;
    bf16 *out;              // BF16 output [voxel][out_ld], channels [out_off, out_off + cout)
    int out_ld, out_off;
    float *out32;           // FP32 output [voxel][cout] instead of out (network head)
    int *err;
};

__device__ __forceinline__ void record(int *err, int bit) {
    if (err) atomicOr(err, bit);
}

__device__ __forceinline__ uint8_t *align1k(uint8_t *p) {
    return reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(p) + 1023) & ~uintptr_t(1023));
}

__device__ __forceinline__ void tap_offset(int taps, int tap, int &dx, int &dy, int &dz) {
    if (taps == 1) { dx = dy = dz = 0; return; }
    dx = tap % 3 - 1;
    dy = (tap / 3) % 3 - 1;
    dz = tap / 9 - 1;
}

__global__ void __launch_bounds__(128) k_conv(const __grid_constant__ CUtensorMap tmA,
                                              const __grid_constant__ CUtensorMap tmB, ConvArgs a) {
    extern __shared__ uint8_t smraw[];
    uint8_t *sm = align1k(smraw);
    const int S = a.stages;
    const uint32_t abytes = 128u * a.ck * 2u, bbytes = uint32_t(a.cout) * a.ck * 2u;
    // every stage buffer starts on a 1024-byte boundary (the 128-byte swizzle atom)
    const uint32_t astride = (abytes + 1023u) & ~1023u, bstride = (bbytes + 1023u) & ~1023u;
    uint8_t *sA = sm;
    uint8_t *sB = sm + S * astride;
    uint64_t *full = reinterpret_cast<uint64_t *>(sB + S * bstride);
    uint64_t *empty = full + S;
    uint64_t *done = empty + S;
    uint32_t *tslot = reinterpret_cast<uint32_t *>(done + 1);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int x0 = (blockIdx.x % a.ntx) * a.tx, y0 = (blockIdx.x / a.ntx) * a.ty;
    const int z = blockIdx.y, b = blockIdx.z;
    const uint32_t ncols = tc::tmem_cols(a.cout);
    if (threadIdx.x == 0) {
        tc::tma_prefetch_desc(&tmA);
        tc::tma_prefetch_desc(&tmB);
        for (int s = 0; s < S; ++s) { tc::mbar_init(full + s, 1); tc::mbar_init(empty + s, 1); }
        tc::mbar_init(done, 1);
        tc::mbar_fence_init();
    }
    if (warp == 1) tc::tmem_alloc(tslot, ncols);
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = *tslot;
    const int nchunk = a.cin / a.ck, nk = a.taps * nchunk;
    const uint32_t span = uint32_t(a.ck) * 2u, lay = tc::layout_code(int(span));

    if (warp == 0 && lane == 0) {
        // producer: one stage = the tap-shifted input box and the matching weight box
        int issued = 0;
        for (int it = 0; it < nk; ++it) {
            const int s = it % S;
            if (it >= S && !tc::mbar_wait(empty + s, ((it / S) - 1) & 1)) { record(a.err, UERR_TIMEOUT_PRODUCER); break; }
            const int tap = it / nchunk, ch = it % nchunk;
            int dx, dy, dz;
            tap_offset(a.taps, tap, dx, dy, dz);
            tc::mbar_expect_tx(full + s, abytes + bbytes);
            tc::tma_load_5d(sA + s * astride, &tmA, full + s, ch * a.ck, x0 + dx, y0 + dy, z + dz, b);
            tc::tma_load_2d(sB + s * bstride, &tmB, full + s, tap * a.cin + ch * a.ck, 0);
            ++issued;
        }
        // the copies in flight land before this CTA can leave
        for (int it = (issued > S ? issued - S : 0); it < issued; ++it) {
            if (!tc::mbar_wait(full + it % S, (it / S) & 1)) { record(a.err, UERR_TIMEOUT_PRODUCER); break; }
        }
    } else if (warp == 1 && lane == 0) {
        // MMA issuer
        const uint32_t idesc = tc::idesc_bf16(128, a.cout, 0, 0);
        for (int it = 0; it < nk; ++it) {
            const int s = it % S;
            if (!tc::mbar_wait(full + s, (it / S) & 1)) { record(a.err, UERR_TIMEOUT_MMA); break; }
            tc::fence_after();
            const uint32_t aa = tc::saddr(sA + s * astride), ba = tc::saddr(sB + s * bstride);
            for (int k = 0; k < a.ck / 16; ++k) {
                const uint64_t ad = tc::sdesc(aa + 32u * k, 16u, 8u * span, lay);
                const uint64_t bd = tc::sdesc(ba + 32u * k, 16u, 8u * span, lay);
                tc::mma_bf16(tmem, ad, bd, idesc, (it | k) != 0 ? 1u : 0u);
            }
            tc::mma_commit(empty + s);
        }
        tc::mma_commit(done);   // fires when every MMA above has completed
    }
    __syncwarp();
    // epilogue: thread t of warp w owns accumulator row 32 w + t (one voxel of the patch)
    if (!tc::mbar_wait(done, 0)) record(a.err, UERR_TIMEOUT_EPILOGUE);
    tc::fence_after();
    const int m = warp * 32 + lane;
    const int vx = x0 + m % a.tx, vy = y0 + m / a.tx;
    const bool valid = vx < a.X && vy < a.Y;
    const long long vox = (((long long)(b) * a.Z + z) * a.Y + vy) * a.X + vx;
    for (int c0 = 0; c0 < a.cout; c0 += 16) {
        float v[16];
        tc::tmem_ld16(tmem + (uint32_t(warp * 32) << 16) + uint32_t(c0), v);
        if (!valid) continue;
        if (a.bias) {
#pragma unroll
            for (int i = 0; i < 16; ++i) v[i] += a.bias[c0 + i];
        }
        if (a.relu) {
#pragma unroll
            for (int i = 0; i < 16; ++i) v[i] = fmaxf(v[i], 0.f);
        }
        if (a.mask) {
            const uint4 *mp = reinterpret_cast<const uint4 *>(a.mask + vox * a.mask_ld + c0);
            uint4 mv[2] = {mp[0], mp[1]};
            const bf16 *mb = reinterpret_cast<const bf16 *>(mv);
#pragma unroll
            for (int i = 0; i < 16; ++i) v[i] = __bfloat162float(mb[i]) > 0.f ? v[i] : 0.f;
        }
        if (a.out32) {
            float4 *op = reinterpret_cast<float4 *>(a.out32 + vox * a.cout + c0);
#pragma unroll
            for (int i = 0; i < 4; ++i) op[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
        } else {
            uint4 ov[2];
            bf16 *ob = reinterpret_cast<bf16 *>(ov);
#pragma unroll
            for (int i = 0; i < 16; ++i) ob[i] = __float2bfloat16_rn(v[i]);
            uint4 *op = reinterpret_cast<uint4 *>(a.out + vox * a.out_ld + a.out_off + c0);
            op[0] = ov[0];
            op[1] = ov[1];
        }
    }
    tc::fence_before();
    __syncthreads();
    if (warp == 1) tc::tmem_dealloc(tmem, ncols);
}

struct WgradArgs {
    int X, Y, Z, B;         // volume and batch
    int cin, cout, taps;
    int cw;                 // channel width of one A block (16, 32, 64): 128 / cw blocks per M tile
    int nw;                 // channel width of one B block (min(64, cout))
    int tx, ty, ntx, nty;   // 128-voxel patch and patch counts
    int ktiles;             // voxel patches in the whole batch
    int kper;               // patches per CTA (split of the voxel reduction)
    int stages;
    float *dw;              // [cout][taps * cin], accumulated into
    int *err;
};

__global__ void __launch_bounds__(128) k_wgrad(const __grid_constant__ CUtensorMap tmX,
                                               const __grid_constant__ CUtensorMap tmD, WgradArgs a) {
    extern __shared__ uint8_t smraw[];
    uint8_t *sm = align1k(smraw);
    const int S = a.stages;
    const int nblk_a = 128 / a.cw, nblk_b = a.cout / a.nw;
    const uint32_t ablk = 128u * a.cw * 2u, bblk = 128u * a.nw * 2u;
    const uint32_t abytes = nblk_a * ablk, bbytes = nblk_b * bblk;
    uint8_t *sA = sm;
    uint8_t *sB = sm + S * abytes;
    uint64_t *full = reinterpret_cast<uint64_t *>(sB + S * bbytes);
    uint64_t *empty = full + S;
    uint64_t *done = empty + S;
    uint32_t *tslot = reinterpret_cast<uint32_t *>(done + 1);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int chunks = a.cin / a.cw, total_blk = a.taps * chunks;
    const int mt = blockIdx.x;                         // M tile: blocks mt*nblk_a .. +nblk_a-1
    const int k0 = blockIdx.y * a.kper;
    const int k1 = min(a.ktiles, k0 + a.kper);
    const int nk = max(0, k1 - k0);
    int nvalid = 0;                                     // A blocks of this M tile inside the taps
    for (int j = 0; j < nblk_a; ++j) nvalid += (mt * nblk_a + j < total_blk) ? 1 : 0;
    const uint32_t ncols = tc::tmem_cols(a.cout);
    if (threadIdx.x == 0) {
        tc::tma_prefetch_desc(&tmX);
        tc::tma_prefetch_desc(&tmD);
        for (int s = 0; s < S; ++s) { tc::mbar_init(full + s, 1); tc::mbar_init(empty + s, 1); }
        tc::mbar_init(done, 1);
        tc::mbar_fence_init();
    }
    if (warp == 1) tc::tmem_alloc(tslot, ncols);
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = *tslot;
    if (warp == 0 && lane == 0) {
        int issued = 0;
        for (int it = 0; it < nk; ++it) {
            const int s = it % S;
            if (it >= S && !tc::mbar_wait(empty + s, ((it / S) - 1) & 1)) { record(a.err, UERR_TIMEOUT_PRODUCER); break; }
            // voxel patch kt -> (batch, z, patch row, patch column)
            int kt = k0 + it;
            const int px = kt % a.ntx; kt /= a.ntx;
            const int py = kt % a.nty; kt /= a.nty;
            const int z = kt % a.Z, bb = kt / a.Z;
            const int x0 = px * a.tx, y0 = py * a.ty;
            tc::mbar_expect_tx(full + s, nvalid * ablk + bbytes);
            for (int j = 0; j < nblk_a; ++j) {
                const int g = mt * nblk_a + j;
                if (g >= total_blk) break;
                const int tap = g / chunks, ch = g % chunks;
                int dx, dy, dz;
                tap_offset(a.taps, tap, dx, dy, dz);
                tc::tma_load_5d(sA + s * abytes + j * ablk, &tmX, full + s, ch * a.cw, x0 + dx, y0 + dy, z + dz, bb);
            }
            for (int j = 0; j < nblk_b; ++j)
                tc::tma_load_5d(sB + s * bbytes + j * bblk, &tmD, full + s, j * a.nw, x0, y0, z, bb);
            ++issued;
        }
        for (int it = (issued > S ? issued - S : 0); it < issued; ++it) {
            if (!tc::mbar_wait(full + it % S, (it / S) & 1)) { record(a.err, UERR_TIMEOUT_PRODUCER); break; }
        }
    } else if (warp == 1 && lane == 0) {
        const uint32_t idesc = tc::idesc_bf16(128, a.cout, 1, 1);
        const uint32_t la = tc::layout_code(a.cw * 2), lb = tc::layout_code(a.nw * 2);
        const uint32_t sbo_a = 8u * a.cw * 2u, sbo_b = 8u * a.nw * 2u;
        for (int it = 0; it < nk; ++it) {
            const int s = it % S;
            if (!tc::mbar_wait(full + s, (it / S) & 1)) { record(a.err, UERR_TIMEOUT_MMA); break; }
            tc::fence_after();
            const uint32_t aa = tc::saddr(sA + s * abytes), ba = tc::saddr(sB + s * bbytes);
#pragma unroll
            for (int k = 0; k < 8; ++k) {   // 128 voxels = 8 MMA K steps of 16 (two 8-row groups)
                const uint64_t ad = tc::sdesc(aa + 2u * k * sbo_a, ablk, sbo_a, la);
                const uint64_t bd = tc::sdesc(ba + 2u * k * sbo_b, bblk, sbo_b, lb);
                tc::mma_bf16(tmem, ad, bd, idesc, (it | k) != 0 ? 1u : 0u);
            }
            tc::mma_commit(empty + s);
        }
        tc::mma_commit(done);
    }
    __syncwarp();
    if (!tc::mbar_wait(done, 0)) record(a.err, UERR_TIMEOUT_EPILOGUE);
    tc::fence_after();
    // row m of D: A block g = mt * nblk_a + m / cw, channel (g % chunks) * cw + m % cw of tap g / chunks
    const int m = warp * 32 + lane;
    const int g = mt * nblk_a + m / a.cw;
    const bool valid = nk > 0 && g < total_blk;
    const int tap = g / chunks, ci = (g % chunks) * a.cw + m % a.cw;
    const long long ld = (long long)a.taps * a.cin;
    for (int c0 = 0; c0 < a.cout; c0 += 16) {
        float v[16];
        tc::tmem_ld16(tmem + (uint32_t(warp * 32) << 16) + uint32_t(c0), v);
        if (!valid) continue;
#pragma unroll
        for (int i = 0; i < 16; ++i) atomicAdd(a.dw + (c0 + i) * ld + (long long)tap * a.cin + ci, v[i]);
    }
    tc::fence_before();
    __syncthreads();
    if (warp == 1) tc::tmem_dealloc(tmem, ncols);
}

// ---- elementwise kernels ---------------------------------------------------------------------
// average pooling 2x2x2 of src [B][Z][Y][X][ld] channels [off, off + C) -> dst [B][Z/2][Y/2][X/2][C];
// one thread per (coarse voxel, 8-channel group)
__global__ void k_pool(const bf16 *src, int ld, int off, bf16 *dst, int C, int X, int Y, int Z, int B) {
    const int Xc = X / 2, Yc = Y / 2, Zc = Z / 2, G = C / 8;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long tot = (long long)B * Zc * Yc * Xc * G;
    if (t >= tot) return;
    const int gq = int(t % G);
    long long v = t / G;
    const int x = int(v % Xc); v /= Xc;
    const int y = int(v % Yc); v /= Yc;
    const int z = int(v % Zc);
    const int b = int(v / Zc);
    float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int d = 0; d < 8; ++d) {
        const long long fv = (((long long)(b) * Z + 2 * z + (d >> 2)) * Y + 2 * y + ((d >> 1) & 1)) * X + 2 * x + (d & 1);
        const uint4 u = *reinterpret_cast<const uint4 *>(src + fv * ld + off + gq * 8);
        const bf16 *e = reinterpret_cast<const bf16 *>(&u);
#pragma unroll
        for (int i = 0; i < 8; ++i) acc[i] += __bfloat162float(e[i]);
    }
    uint4 o;
    bf16 *oe = reinterpret_cast<bf16 *>(&o);
#pragma unroll
    for (int i = 0; i < 8; ++i) oe[i] = __float2bfloat16_rn(0.125f * acc[i]);
    *reinterpret_cast<uint4 *>(dst + (t / G) * C + gq * 8) = o;
}

// gradient into the skip tensor: dz[v][c] = skip_grad[v][c] (channels [0, C) of the
// concatenation gradient, already masked) + (act[v][c] > 0) * dpool[parent(v)][c] / 8
__global__ void k_pool_back(const bf16 *dcat, int ldcat, const bf16 *dpool, const bf16 *act, int ldact, bf16 *dz,
                            int C, int X, int Y, int Z, int B) {
    const int G = C / 8;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long tot = (long long)B * Z * Y * X * G;
    if (t >= tot) return;
    const int gq = int(t % G);
    long long v = t / G;
    const int x = int(v % X); long long r = v / X;
    const int y = int(r % Y); r /= Y;
    const int z = int(r % Z);
    const int b = int(r / Z);
    const long long pv = (((long long)(b) * (Z / 2) + z / 2) * (Y / 2) + y / 2) * (X / 2) + x / 2;
    const uint4 uc = *reinterpret_cast<const uint4 *>(dcat + v * ldcat + gq * 8);
    const uint4 up = *reinterpret_cast<const uint4 *>(dpool + pv * C + gq * 8);
    const uint4 ua = *reinterpret_cast<const uint4 *>(act + v * ldact + gq * 8);
    const bf16 *ec = reinterpret_cast<const bf16 *>(&uc), *ep = reinterpret_cast<const bf16 *>(&up),
               *ea = reinterpret_cast<const bf16 *>(&ua);
    uint4 o;
    bf16 *oe = reinterpret_cast<bf16 *>(&o);
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const float p = __bfloat162float(ea[i]) > 0.f ? 0.125f * __bfloat162float(ep[i]) : 0.f;
        oe[i] = __float2bfloat16_rn(__bfloat162float(ec[i]) + p);
    }
    *reinterpret_cast<uint4 *>(dz + v * C + gq * 8) = o;
}

// nearest upsampling: cat[v][off + c] = low[parent(v)][c], c < C
__global__ void k_upsample(const bf16 *low, int C, bf16 *cat, int ldcat, int off, int X, int Y, int Z, int B) {
    const int G = C / 8;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long tot = (long long)B * Z * Y * X * G;
    if (t >= tot) return;
    const int gq = int(t % G);
    long long v = t / G;
    const int x = int(v % X); long long r = v / X;
    const int y = int(r % Y); r /= Y;
    const int z = int(r % Z);
    const int b = int(r / Z);
    const long long pv = (((long long)(b) * (Z / 2) + z / 2) * (Y / 2) + y / 2) * (X / 2) + x / 2;
    *reinterpret_cast<uint4 *>(cat + v * ldcat + off + gq * 8) = *reinterpret_cast<const uint4 *>(low + pv * C + gq * 8);
}

// adjoint of the upsampling: dlow[p][c] = sum of the 8 children's dcat[child][off + c]
__global__ void k_upsample_back(const bf16 *dcat, int ldcat, int off, bf16 *dlow, int C, int X, int Y, int Z, int B) {
    const int Xc = X / 2, Yc = Y / 2, Zc = Z / 2, G = C / 8;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long tot = (long long)B * Zc * Yc * Xc * G;
    if (t >= tot) return;
    const int gq = int(t % G);
    long long v = t / G;
    const int x = int(v % Xc); v /= Xc;
    const int y = int(v % Yc); v /= Yc;
    const int z = int(v % Zc);
    const int b = int(v / Zc);
    float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int d = 0; d < 8; ++d) {
        const long long fv = (((long long)(b) * Z + 2 * z + (d >> 2)) * Y + 2 * y + ((d >> 1) & 1)) * X + 2 * x + (d & 1);
        const uint4 u = *reinterpret_cast<const uint4 *>(dcat + fv * ldcat + off + gq * 8);
        const bf16 *e = reinterpret_cast<const bf16 *>(&u);
#pragma unroll
        for (int i = 0; i < 8; ++i) acc[i] += __bfloat162float(e[i]);
    }
    uint4 o;
    bf16 *oe = reinterpret_cast<bf16 *>(&o);
#pragma unroll
    for (int i = 0; i < 8; ++i) oe[i] = __float2bfloat16_rn(acc[i]);
    *reinterpret_cast<uint4 *>(dlow + (t / G) * C + gq * 8) = o;
}

// bias gradient: db[c] += sum over voxels of dz[v][c]; blocks of 256 threads stride over voxels
__global__ void k_bias_grad(const bf16 *dz, int C, long long nvox, float *db) {
    __shared__ float part[256];
    const int c = threadIdx.x % C, lanes = 256 / C;
    float s = 0.f;
    for (long long v = (long long)blockIdx.x * lanes + threadIdx.x / C; v < nvox; v += (long long)gridDim.x * lanes)
        s += __bfloat162float(dz[v * C + c]);
    part[threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.x < C) {
        float t = 0.f;
        for (int k = 0; k < lanes; ++k) t += part[k * C + threadIdx.x];
        atomicAdd(db + threadIdx.x, t);
    }
}

// loss: mean squared error over the first `cused` of C channels; writes dpred (BF16) and adds
// the block's sum of squares to *acc (FP64)
__global__ void k_mse(const float *pred, const bf16 *tgt, bf16 *dpred, int C, int cused, long long nvox, double scale,
                      double *acc) {
    __shared__ double part[256];
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double sq = 0.0;
    if (t < nvox * C) {
        const int c = int(t % C);
        float d = 0.f;
        if (c < cused) {
            d = pred[t] - __bfloat162float(tgt[t]);
            sq = double(d) * d;
        }
        dpred[t] = __float2bfloat16_rn(float(2.0 * scale) * d);
    }
    part[threadIdx.x] = sq;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) part[threadIdx.x] += part[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(acc, part[0]);
}

// Adam on FP32 master weights; refreshes the BF16 forward copy [cout][taps][cin] and the
// flipped, transposed dgrad copy [cin][taps][cout] (tap -> taps - 1 - tap)
__global__ void k_adam(float *w, const float *g, float *m, float *v, long long n, float lr, float b1, float b2,
                       float eps, float bc1, float bc2, float gscale, bf16 *wb, bf16 *wt, int cout, int taps, int cin) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i] * gscale;
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
    w[i] = wi;
    if (wb) {
        const bf16 h = __float2bfloat16_rn(wi);
        wb[i] = h;
        if (wt) {
            const int ci = int(i % cin);
            const long long r = i / cin;
            const int tap = int(r % taps), co = int(r / taps);
            wt[((long long)ci * taps + (taps - 1 - tap)) * cout + co] = h;
        }
    }
}

// BF16 copies of the master weights (after a host upload)
__global__ void k_weights_bf16(const float *w, long long n, bf16 *wb, bf16 *wt, int cout, int taps, int cin) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const bf16 h = __float2bfloat16_rn(w[i]);
    wb[i] = h;
    if (wt) {
        const int ci = int(i % cin);
        const long long r = i / cin;
        const int tap = int(r % taps), co = int(r / taps);
        wt[((long long)ci * taps + (taps - 1 - tap)) * cout + co] = h;
    }
}

// network input: channel 0 = the sample's design field, channels 1.. = the static features
__global__ void k_make_input(const float *design, const float *stat, int nstat, long long nvox, int C, bf16 *out) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nvox * C) return;
    const int c = int(t % C);
    const long long v = t / C;
    float x = 0.f;
    if (c == 0) x = design[v];
    else if (c - 1 < nstat) x = stat[v * nstat + (c - 1)];
    out[t] = __float2bfloat16_rn(x);
}

// normalised targets: out[v][c] = (raw[v][c] - mean[c]) / std[c] for c < cused, 0 above
__global__ void k_make_target(const float *raw, int cused, const float *mean, const float *inv_std, long long nvox,
                              int C, bf16 *out) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nvox * C) return;
    const int c = int(t % C);
    const long long v = t / C;
    const float x = c < cused ? (raw[v * cused + c] - mean[c]) * inv_std[c] : 0.f;
    out[t] = __float2bfloat16_rn(x);
}

// per-channel sums and sums of squares of raw [n][cused] (FP64 accumulation)
__global__ void k_channel_stats(const float *raw, long long n, int cused, double *sum, double *sq) {
    __shared__ double ps[32], pq[32];
    if (threadIdx.x < 32) { ps[threadIdx.x] = 0.0; pq[threadIdx.x] = 0.0; }
    __syncthreads();
    double ls[16] = {0}, lq[16] = {0};
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x)
        for (int c = 0; c < cused && c < 16; ++c) {
            const double x = raw[v * cused + c];
            ls[c] += x;
            lq[c] += x * x;
        }
    for (int c = 0; c < cused && c < 16; ++c) {
        atomicAdd(&ps[c], ls[c]);
        atomicAdd(&pq[c], lq[c]);
    }
    __syncthreads();
    if (threadIdx.x < cused) {
        atomicAdd(sum + threadIdx.x, ps[threadIdx.x]);
        atomicAdd(sq + threadIdx.x, pq[threadIdx.x]);
    }
}

// a training sample's targets from a lattice's FP64 device fields: out[v][c] = f_c[v] (rho - 1 for
// c = 0), zero for a missing field
struct SampleSrc { const double *f[16]; };
__global__ void k_capture(SampleSrc src, int cused, long long nvox, float *out) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nvox * cused) return;
    const int c = int(t % cused);
    const long long v = t / cused;
    const double *f = src.f[c];
    out[t] = f ? float(f[v] - (c == 0 ? 1.0 : 0.0)) : 0.f;
}

// de-normalised prediction: out[c][v] = pred[v][c] * std[c] + mean[c] (c < cused), FP64
__global__ void k_denorm(const float *pred, int C, int cused, const float *mean, const float *stdv, long long nvox,
                         double *out) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nvox * cused) return;
    const int c = int(t / nvox);
    const long long v = t % nvox;
    out[t] = double(pred[v * C + c]) * stdv[c] + mean[c];
}

}  // namespace unet
}  // namespace pl
