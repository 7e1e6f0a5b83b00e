// fields.cu -- node-field kernels: residual and max-abs reductions (FP64, deterministic two-pass),
// sensitivities, density / Heaviside filters.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include "fields.h"
#include "lattice.cuh"

namespace pl {

constexpr int kRB = 256;   // reduction block

// ---- Residual (residual.h:8-51): sum (a-b)^2 and sum a^2 over ncomp components ----------
// pass 1: one FP64 partial pair per block (fixed tree, so results are reproducible); pass 2:
// one block folds the partials in block order. Non-finite inputs are counted.
__global__ void k_resid_partial(ResidArgs r, double *partial, int *nonfinite) {
    __shared__ double s0[kRB], s1[kRB];
    double a0 = 0.0, a1 = 0.0;
    int bad = 0;
    for (long long idx = (long long)blockIdx.x * kRB + threadIdx.x; idx < r.n; idx += (long long)gridDim.x * kRB) {
        double d0 = 0.0, d1 = 0.0;
        for (int m = 0; m < r.ncomp; ++m) {
            const double x = r.a[m][idx], y = r.b[m][idx];
            const double e = (x - y) * (x - y), v = x * x;
            if (m == 0) { d0 = e; d1 = v; } else { d0 += e; d1 += v; }
            if (!isfinite(x)) bad = 1;
        }
        a0 += d0;
        a1 += d1;
    }
    s0[threadIdx.x] = a0;
    s1[threadIdx.x] = a1;
    __syncthreads();
    for (int w = kRB / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) { s0[threadIdx.x] += s0[threadIdx.x + w]; s1[threadIdx.x] += s1[threadIdx.x + w]; }
        __syncthreads();
    }
    if (threadIdx.x == 0) { partial[2 * blockIdx.x] = s0[0]; partial[2 * blockIdx.x + 1] = s1[0]; }
    if (bad) atomicOr(nonfinite, 1);
}
__global__ void k_resid_final(const double *partial, int nblk, double *out) {
    __shared__ double s0[kRB], s1[kRB];
    double a0 = 0.0, a1 = 0.0;
    for (int b = threadIdx.x; b < nblk; b += kRB) { a0 += partial[2 * b]; a1 += partial[2 * b + 1]; }
    s0[threadIdx.x] = a0;
    s1[threadIdx.x] = a1;
    __syncthreads();
    for (int w = kRB / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) { s0[threadIdx.x] += s0[threadIdx.x + w]; s1[threadIdx.x] += s1[threadIdx.x + w]; }
        __syncthreads();
    }
    if (threadIdx.x == 0) { out[0] = s0[0]; out[1] = s1[0]; out[2] = sqrt(s0[0] / s1[0]); }
}
int resid_blocks(long long n) {
    long long b = (n + kRB - 1) / kRB;
    return (int)(b < 1024 ? (b < 1 ? 1 : b) : 1024);
}
void launch_residual(const ResidArgs &r, double *partial, int nblk, int *nonfinite, double *out, cudaStream_t st) {
    k_resid_partial<<<nblk, kRB, 0, st>>>(r, partial, nonfinite);
    k_resid_final<<<1, kRB, 0, st>>>(partial, nblk, out);
}

// ---- Normalize (normalize.h:8-23) -------------------------------------------------------
__global__ void k_maxabs_partial(const double *v, long long n, double *partial) {
    __shared__ double s[kRB];
    double m = 0.0;
    for (long long i = (long long)blockIdx.x * kRB + threadIdx.x; i < n; i += (long long)gridDim.x * kRB)
        m = fmax(m, fabs(v[i]));
    s[threadIdx.x] = m;
    __syncthreads();
    for (int w = kRB / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) s[threadIdx.x] = fmax(s[threadIdx.x], s[threadIdx.x + w]);
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = s[0];
}
__global__ void k_scale_div(double *v, long long n, const double *partial, int nblk) {
    __shared__ double vmax;
    if (threadIdx.x == 0) {
        double m = 0.0;
        for (int b = 0; b < nblk; ++b) m = fmax(m, partial[b]);
        vmax = m;
    }
    __syncthreads();
    for (long long i = (long long)blockIdx.x * kRB + threadIdx.x; i < n; i += (long long)gridDim.x * kRB) v[i] /= vmax;
}
void launch_normalize(double *v, long long n, double *partial, int nblk, cudaStream_t st) {
    k_maxabs_partial<<<nblk, kRB, 0, st>>>(v, n, partial);
    k_scale_div<<<nblk, kRB, 0, st>>>(v, n, partial, nblk);
}

// ---- sensitivities ------------------------------------------------------------------------
// Bulk Brinkman + diffusivity terms (adjointadvection.h:1459-1511) then the flux-boundary terms
// of the faces in the reference order xmin, xmax, ymin, ymax, zmin, zmax (753-888; D3Q15 uses
// the argument order of the overload the drivers call, adjointadvection_avx.h:1459-1513).
template <class L>
__device__ void sens_node(const SensArgs &s, int idx) {
    constexpr int Q = L::Q, ND = L::ND;
    const double u[3] = {s.ux[idx], s.uy[idx], ND == 3 ? s.uz[idx] : 0.0};
    const double im[3] = {s.imx[idx], s.imy[idx], ND == 3 ? s.imz[idx] : 0.0};
    const double uim = ND == 2 ? u[0] * im[0] + u[1] * im[1] : u[0] * im[0] + u[1] * im[1] + u[2] * im[2];
    double d = s.dfds[idx];
    if (s.which == 3) { s.dfds[idx] = d + 3.0 * s.dads[idx] * uim; return; }
    if (s.which == 2) {
        s.dfds[idx] = d + (3.0 * s.dads[idx] * uim - s.dkds[idx] * (1.0 - s.tem[idx]) * (1.0 + s.item[idx]));
        return;
    }
    d += 3.0 * s.dads[idx] * uim;
    double sumg = 0.0;
    for (int c = 0; c < Q; ++c) sumg += s.g[(long long)c * s.np + idx] * s.ig[(long long)c * s.np + idx];
    const double iq[3] = {s.iqx[idx], s.iqy[idx], ND == 3 ? s.iqz[idx] : 0.0};
    const double uiq = ND == 2 ? u[0] * iq[0] + u[1] * iq[1] : u[0] * iq[0] + u[1] * iq[1] + u[2] * iq[2];
    const double k3 = 3.0 * s.kappa[idx] + 0.5;
    d += -3.0 / (k3 * k3) * s.dkds[idx] * (sumg - s.tem[idx] * (s.item[idx] + 3.0 * uiq));
    if (s.which == 0 && s.mask[idx]) {
        const int i = idx % s.nx, r = idx / s.nx;
        const int j = ND == 2 ? r : r % s.ny, k = ND == 2 ? 0 : r / s.ny;
        const int pos[3] = {i, j, k}, len[3] = {s.nx, s.ny, s.nz};
        for (int a = 0; a < ND; ++a) {
            for (int sd = 0; sd < 2; ++sd) {
                const int dd = sd == 0 ? -1 : 1;
                if (pos[a] != (sd == 0 ? 0 : len[a] - 1)) continue;
                const int nin = -dd;
                const double pre = nin > 0 ? 1.0 + 3.0 * u[a] : 1.0 - 3.0 * u[a];
                const double post = nin > 0 ? 1.0 - 3.0 * u[a] : 1.0 + 3.0 * u[a];
                double ns = 0.0;
                const double kc = ND == 2 ? 4.0 : 8.0;
                for (int c = 1; c < Q; ++c) {
                    if (comp<L>(c, a) != -dd) continue;
                    bool diag = false;
                    for (int e = 0; e < ND; ++e) if (e != a && comp<L>(c, e) != 0) diag = true;
                    if (!diag) ns = (ND == 2 ? -6.0 : -12.0) + kc * s.ig[(long long)c * s.np + idx];
                }
                for (int c = 1; c < Q; ++c) {
                    if (comp<L>(c, a) != -dd) continue;
                    bool diag = false;
                    for (int e = 0; e < ND; ++e) if (e != a && comp<L>(c, e) != 0) diag = true;
                    if (diag) ns += s.ig[(long long)c * s.np + idx];
                }
                const double kap = s.kappa[idx];
                if (ND == 2) {
                    const int b = 1 - a;
                    double ts = 0.0;
                    for (int c = 1; c < Q; ++c) {
                        if (comp<L>(c, a) != -dd || comp<L>(c, b) == 0) continue;
                        ts = comp<L>(c, b) > 0 ? ts + s.ig[(long long)c * s.np + idx] : ts - s.ig[(long long)c * s.np + idx];
                    }
                    const double num = pre * ns + 3.0 * u[b] * ts;
                    d += s.qn[idx] * s.dkds[idx] * num / (36.0 * post * (kap * kap));
                } else {
                    const int t0 = a == 0 ? 1 : (a == 1 ? 2 : 0), t1 = a == 0 ? 2 : (a == 1 ? 0 : 1);
                    const bool k3f = (a == 0 || (a == 1 && dd < 0));
                    double ts0 = 0.0, ts1 = 0.0;
                    for (int c = 1; c < Q; ++c) {
                        if (comp<L>(c, a) != -dd) continue;
                        bool diag = false;
                        for (int e = 0; e < ND; ++e) if (e != a && comp<L>(c, e) != 0) diag = true;
                        if (!diag) continue;
                        const double v = s.ig[(long long)c * s.np + idx];
                        ts0 = comp<L>(c, t0) > 0 ? ts0 + v : ts0 - v;
                        ts1 = comp<L>(c, t1) > 0 ? ts1 + v : ts1 - v;
                    }
                    const double num = k3f ? pre * ns + 3.0 * u[t0] * ts0 + 3.0 * u[t1] * ts1
                                           : pre * ns + u[t0] * ts0 + u[t1] * ts1;
                    d += s.qn[idx] * s.dkds[idx] * num / (72.0 * post * (kap * kap));
                }
            }
        }
    }
    s.dfds[idx] = d;
}
template <class L> __global__ void k_sens(SensArgs s) {
    const int idx = blockIdx.x * kRB + threadIdx.x;
    if (idx < s.n) sens_node<L>(s, idx);
}
void launch_sensitivity(int q, const SensArgs &s, cudaStream_t st) {
    const int g = (s.n + kRB - 1) / kRB;
    if (q == 9) k_sens<D2Q9><<<g, kRB, 0, st>>>(s);
    else k_sens<D3Q15><<<g, kRB, 0, st>>>(s);
}

// AEL::SensitivityCompliance (adjointelastic.h:149-155), in the reference's expression order with
// every product and sum rounded on its own (no contraction), so it matches the CPU bit for bit
struct CompArgs { const double *in[9]; };
__global__ void k_compliance(int n, double *dfds, CompArgs c) {
    const int i = blockIdx.x * kRB + threadIdx.x;
    if (i >= n) return;
    const double sxx = c.in[0][i], sxy = c.in[1][i], syx = c.in[2][i], syy = c.in[3][i];
    double ss = __dmul_rn(sxx, c.in[5][i]);
    ss = __dadd_rn(ss, __dmul_rn(sxy, c.in[6][i]));
    ss = __dadd_rn(ss, __dmul_rn(syx, c.in[7][i]));
    ss = __dadd_rn(ss, __dmul_rn(syy, c.in[8][i]));
    const double tr = __dmul_rn(__dmul_rn(1.5, c.in[4][i]), __dadd_rn(sxx, syy));
    dfds[i] = __dadd_rn(dfds[i], __dsub_rn(__dmul_rn(4.5, ss), tr));
}
void launch_compliance(int n, double *dfds, const double *const *in, cudaStream_t st) {
    CompArgs c;
    for (int m = 0; m < 9; ++m) c.in[m] = in[m];
    k_compliance<<<(n + kRB - 1) / kRB, kRB, 0, st>>>(n, dfds, c);
}

__global__ void k_axpy(int n, double *dst, const double *src, double a) {
    const int i = blockIdx.x * kRB + threadIdx.x;
    if (i < n) dst[i] = __dadd_rn(dst[i], __dmul_rn(a, src[i]));
}
void launch_axpy(int n, double *dst, const double *src, double a, cudaStream_t st) {
    k_axpy<<<(n + kRB - 1) / kRB, kRB, 0, st>>>(n, dst, src, a);
}

// ---- filters ------------------------------------------------------------------------------
// Taps of the (2 nR + 1)^d box with distance <= R, in the reference's (i2, j2, k2) loop order,
// with their hat weights (R - dist)/R computed on the host in FP64; or, for a general weight
// functor, one weight per (node, tap) from the caller's table.
__device__ __forceinline__ void filt_node(const FiltArgs &f, const double *v, int idx, double &ws, double &w) {
    const int i = idx % f.nx, r = idx / f.nx, j = r % f.ny, k = r / f.ny;
    const bool m1 = f.mask ? f.mask[idx] != 0 : true;
    ws = 0.0;
    w = 0.0;
    for (int t = 0; t < f.ntap; ++t) {
        const int i2 = i + f.di[t], j2 = j + f.dj[t], k2 = k + f.dk[t];
        if (i2 < 0 || i2 >= f.nx || j2 < 0 || j2 >= f.ny || k2 < 0 || k2 >= f.nz) continue;
        const int id2 = i2 + f.nx * (j2 + f.ny * k2);
        double wt;
        if (f.wtab) wt = f.wtab[(long long)idx * f.ntap + t];
        else if (!f.mask || (m1 && f.mask[id2])) wt = f.hat[t];
        else wt = (f.di[t] == 0 && f.dj[t] == 0 && f.dk[t] == 0) ? 1.0 : 0.0;
        ws += wt * v[id2];
        w += wt;
    }
}
__global__ void k_heaviside_var(FiltArgs f, const double *s, double *out) {
    const int idx = blockIdx.x * kRB + threadIdx.x;
    if (idx >= f.n) return;
    double ws, w;
    filt_node(f, s, idx, ws, w);
    out[idx] = 0.5 * (tanh(0.5 * f.beta) + tanh(f.beta * (ws / w - 0.5))) / tanh(0.5 * f.beta);
}
__global__ void k_heaviside_chain(FiltArgs f, const double *s, const double *dfdrho, double *tmp) {
    const int idx = blockIdx.x * kRB + threadIdx.x;
    if (idx >= f.n) return;
    double ws, w;
    filt_node(f, s, idx, ws, w);
    const double th = tanh(f.beta * (ws / w - 0.5));
    tmp[idx] = dfdrho[idx] * (0.5 * f.beta * (1.0 - th * th) / tanh(0.5 * f.beta));
}
__global__ void k_filter_avg(FiltArgs f, const double *v, double *out) {
    const int idx = blockIdx.x * kRB + threadIdx.x;
    if (idx >= f.n) return;
    double ws, w;
    filt_node(f, v, idx, ws, w);
    out[idx] = ws / w;
}
void launch_filter(int op, const FiltArgs &f, const double *a, const double *b, double *tmp, double *out,
                   cudaStream_t st) {
    const int g = (f.n + kRB - 1) / kRB;
    if (op == 0) k_heaviside_var<<<g, kRB, 0, st>>>(f, a, out);
    else if (op == 1) {
        k_heaviside_chain<<<g, kRB, 0, st>>>(f, a, b, tmp);
        k_filter_avg<<<g, kRB, 0, st>>>(f, tmp, out);
    } else k_filter_avg<<<g, kRB, 0, st>>>(f, a, out);
}

// ---- misc -----------------------------------------------------------------------------------
__global__ void k_d2c_f32(const double *in, float *out, int n) {
    const int i = blockIdx.x * kRB + threadIdx.x;
    if (i < n) out[i] = float(in[i]);
}
void launch_to_compute(const double *in, void *out, int n, bool fp32, cudaStream_t st) {
    if (fp32) k_d2c_f32<<<(n + kRB - 1) / kRB, kRB, 0, st>>>(in, static_cast<float *>(out), n);
    else cudaMemcpyAsync(out, in, sizeof(double) * n, cudaMemcpyDeviceToDevice, st);
}
__global__ void k_transpose_snap(const double *snap, long long np, int n, int q, double *out) {
    const long long t = (long long)blockIdx.x * kRB + threadIdx.x;
    if (t >= (long long)n * q) return;
    const int idx = int(t / q), c = int(t % q);
    out[t] = snap[(long long)c * np + idx];
}
void launch_snap_to_node_major(const double *snap, long long np, int n, int q, double *out, cudaStream_t st) {
    const long long tot = (long long)n * q;
    k_transpose_snap<<<(unsigned)((tot + kRB - 1) / kRB), kRB, 0, st>>>(snap, np, n, q, out);
}
__global__ void k_untranspose_snap(const double *in, long long np, int n, int q, double *snap) {
    const long long t = (long long)blockIdx.x * kRB + threadIdx.x;
    if (t >= (long long)n * q) return;
    const int idx = int(t / q), c = int(t % q);
    snap[(long long)c * np + idx] = in[t];
}
void launch_node_major_to_snap(const double *in, long long np, int n, int q, double *snap, cudaStream_t st) {
    const long long tot = (long long)n * q;
    k_untranspose_snap<<<(unsigned)((tot + kRB - 1) / kRB), kRB, 0, st>>>(in, np, n, q, snap);
}

}  // namespace pl
