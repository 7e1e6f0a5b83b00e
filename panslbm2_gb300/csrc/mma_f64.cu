// mma_f64.cu -- the design-variable update of Svanberg's method of moving asymptotes on the
// device: MMA<T>::UpdateVariables of the reference (utility/mma.h:196-548), FP64.
//
// The n design variables and everything of length n live on the device; the per-variable work
// (asymptotes, move limits, p/q coefficients, the primal-dual Newton direction, step bounds and
// the KKT residual) runs in kernels, and its sums over n are deterministic two-stage reductions
// (fixed block tree, blocks folded in order). The m (<= kMmaMaxM) dual quantities, the (m+1) x
// (m+1) Newton system (solvels, mma.h:13-55) and the line-search control stay on the host, in
// the reference's order. Compiled without FMA contraction like the other FP64 units; sums over
// n are ordered differently from the reference's serial loops.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "../../include/panslbm_gb300.h"
#include "launch.h"

namespace {

constexpr int kMmaMaxM = 4;
constexpr int kMaxSums = kMmaMaxM * (kMmaMaxM + 2);
constexpr int kRT = 256;     // threads per block
constexpr int kMaxBlocks = 1024;

struct MmaArgs {
    int n, m, k;
    double asyinit, asydecr, asyincr, albefa, move, raa0;
    double eps, tau;
    double lambda[kMmaMaxM], dlambda[kMmaMaxM];
    const double *xk, *dfdx, *dgdx;   // dgdx: m rows of n
    double *xmin, *xmax, *xkm1, *xkm2, *L, *U, *alpha, *beta, *p0, *q0, *p, *q;
    double *x, *gsi, *ita, *G, *Dx, *deltilx, *dx, *dgsi, *dita, *xt, *gsit, *itat;
    double *partial;                  // kMaxBlocks x nsum
};

// block-wide fixed-order sums of `nsum` values per thread into partial[block * nsum + s]
template <int NS>
__device__ __forceinline__ void block_sums(double (&v)[NS], int nsum, double *partial, bool use_max) {
    __shared__ double sm[kRT / 32][kMaxSums];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int s = 0; s < nsum; ++s) {
        double x = v[s];
        for (int o = 16; o > 0; o >>= 1) {
            const double y = __shfl_down_sync(0xffffffffu, x, o);
            x = use_max ? fmax(x, y) : x + y;
        }
        if (lane == 0) sm[w][s] = x;
    }
    __syncthreads();
    if (threadIdx.x < nsum) {
        double x = sm[0][threadIdx.x];
        for (int k = 1; k < kRT / 32; ++k) x = use_max ? fmax(x, sm[k][threadIdx.x]) : x + sm[k][threadIdx.x];
        partial[(size_t)blockIdx.x * nsum + threadIdx.x] = x;
    }
}

// asymptotes, move limits, p0/q0, p/q, the inner loop's starting point; sums b_i (mma.h:198-280)
__global__ void __launch_bounds__(kRT) k_mma_prep(MmaArgs a) {
    double v[kMmaMaxM];
    for (int i = 0; i < kMmaMaxM; ++i) v[i] = 0.0;
    for (int j = blockIdx.x * kRT + threadIdx.x; j < a.n; j += gridDim.x * kRT) {
        const double xk = a.xk[j], range = a.xmax[j] - a.xmin[j];
        double L, U;
        if (a.k < 2) {
            L = xk - a.asyinit * range;
            U = xk + a.asyinit * range;
        } else {
            const double xm1 = a.xkm1[j], xm2 = a.xkm2[j];
            const double tmp = (xk - xm1) * (xm1 - xm2);
            if (tmp < 0.0) {
                L = xk - a.asydecr * (xm1 - a.L[j]);
                U = xk + a.asydecr * (a.U[j] - xm1);
            } else if (tmp > 0.0) {
                L = xk - a.asyincr * (xm1 - a.L[j]);
                U = xk + a.asyincr * (a.U[j] - xm1);
            } else {
                L = xk - (xm1 - a.L[j]);
                U = xk + (a.U[j] - xm1);
            }
        }
        L = fmin(fmax(xk - 10.0 * range, L), xk - 0.01 * range);
        U = fmin(fmax(xk + 0.01 * range, U), xk + 10.0 * range);
        a.L[j] = L;
        a.U[j] = U;
        const double al = fmax(fmax(a.xmin[j], L + a.albefa * (xk - L)), xk - a.move * range);
        const double be = fmin(fmin(a.xmax[j], U - a.albefa * (U - xk)), xk + a.move * range);
        a.alpha[j] = al;
        a.beta[j] = be;
        const double ux2 = pow(U - xk, 2.0), xl2 = pow(xk - L, 2.0);
        {
            const double dp = fmax(a.dfdx[j], 0.0), dm = fmax(-a.dfdx[j], 0.0);
            a.p0[j] = ux2 * (1.001 * dp + 0.001 * dm + a.raa0 / range);
            a.q0[j] = xl2 * (0.001 * dp + 1.001 * dm + a.raa0 / range);
        }
        for (int i = 0; i < a.m; ++i) {
            const double gr = a.dgdx[(size_t)i * a.n + j];
            const double dp = fmax(gr, 0.0), dm = fmax(-gr, 0.0);
            const double pij = ux2 * (1.001 * dp + 0.001 * dm + a.raa0 / range);
            const double qij = xl2 * (0.001 * dp + 1.001 * dm + a.raa0 / range);
            a.p[(size_t)i * a.n + j] = pij;
            a.q[(size_t)i * a.n + j] = qij;
            v[i] += pij / (U - xk) + qij / (xk - L);
        }
        const double x = 0.5 * (al + be);
        a.x[j] = x;
        a.gsi[j] = fmax(1.0, 1.0 / (x - al));
        a.ita[j] = fmax(1.0, 1.0 / (be - x));
    }
    block_sums<kMmaMaxM>(v, a.m, a.partial, false);
}

// per-variable coefficients of one inner iteration; sums deltillambda_i, A_ij, B_i (mma.h:329-392)
__global__ void __launch_bounds__(kRT) k_mma_coef(MmaArgs a) {
    const int m = a.m;
    double v[kMaxSums];
    for (int s = 0; s < kMaxSums; ++s) v[s] = 0.0;
    for (int j = blockIdx.x * kRT + threadIdx.x; j < a.n; j += gridDim.x * kRT) {
        const double x = a.x[j], L = a.L[j], U = a.U[j];
        double pl = a.p0[j], ql = a.q0[j];
        for (int i = 0; i < m; ++i) {
            pl += a.lambda[i] * a.p[(size_t)i * a.n + j];
            ql += a.lambda[i] * a.q[(size_t)i * a.n + j];
        }
        double Gj[kMmaMaxM];
        for (int i = 0; i < m; ++i)
            Gj[i] = a.p[(size_t)i * a.n + j] / pow(U - x, 2.0) - a.q[(size_t)i * a.n + j] / pow(x - L, 2.0);
        const double xa = x - a.alpha[j], bx = a.beta[j] - x;
        const double Dx = 2.0 * pl / pow(U - x, 3.0) + 2.0 * ql / pow(x - L, 3.0) + a.gsi[j] / xa + a.ita[j] / bx;
        const double dtx = pl / pow(U - x, 2.0) - ql / pow(x - L, 2.0) - a.eps / xa + a.eps / bx;
        for (int i = 0; i < m; ++i) a.G[(size_t)i * a.n + j] = Gj[i];
        a.Dx[j] = Dx;
        a.deltilx[j] = dtx;
        for (int i = 0; i < m; ++i) v[i] += a.p[(size_t)i * a.n + j] / (U - x) + a.q[(size_t)i * a.n + j] / (x - L);
        for (int ii = 0; ii < m; ++ii)
            for (int jj = 0; jj < m; ++jj) v[m + ii * m + jj] += Gj[ii] * Gj[jj] / Dx;
        for (int ii = 0; ii < m; ++ii) v[m + m * m + ii] -= Gj[ii] * dtx / Dx;
    }
    block_sums<kMaxSums>(v, m * (m + 2), a.partial, false);
}

// the Newton direction of the variables and its step bound (mma.h:394-407, 444-470)
__global__ void __launch_bounds__(kRT) k_mma_dir(MmaArgs a) {
    double v[1] = {0.0};
    for (int j = blockIdx.x * kRT + threadIdx.x; j < a.n; j += gridDim.x * kRT) {
        const double Dx = a.Dx[j];
        double dx = -a.deltilx[j] / Dx;
        for (int i = 0; i < a.m; ++i) dx -= a.G[(size_t)i * a.n + j] * a.dlambda[i] / Dx;
        const double x = a.x[j], xa = x - a.alpha[j], bx = a.beta[j] - x, gsi = a.gsi[j], ita = a.ita[j];
        const double dgsi = -gsi * dx / xa - gsi + a.eps / xa;
        const double dita = ita * dx / bx - ita + a.eps / bx;
        a.dx[j] = dx;
        a.dgsi[j] = dgsi;
        a.dita[j] = dita;
        const double t = fmax(fmax(fmax(-1.01 * dx / xa, 1.01 * dx / bx), -1.01 * dgsi / gsi), -1.01 * dita / ita);
        if (v[0] < t) v[0] = t;
    }
    block_sums<1>(v, 1, a.partial, true);
}

// KKT residual terms of the variables at x + tau dx (written to xt, gsit, itat); sums the
// (5.9a/e/f) norm and g_i (mma.h:551-597). `lambda` is the trial lambda.
__global__ void __launch_bounds__(kRT) k_mma_kkt(MmaArgs a) {
    double v[1 + kMmaMaxM];
    for (int s = 0; s <= kMmaMaxM; ++s) v[s] = 0.0;
    for (int j = blockIdx.x * kRT + threadIdx.x; j < a.n; j += gridDim.x * kRT) {
        const double x = a.x[j] + a.tau * a.dx[j];
        const double gsi = a.gsi[j] + a.tau * a.dgsi[j];
        const double ita = a.ita[j] + a.tau * a.dita[j];
        a.xt[j] = x;
        a.gsit[j] = gsi;
        a.itat[j] = ita;
        const double L = a.L[j], U = a.U[j];
        double pl = a.p0[j], ql = a.q0[j];
        for (int i = 0; i < a.m; ++i) {
            pl += a.lambda[i] * a.p[(size_t)i * a.n + j];
            ql += a.lambda[i] * a.q[(size_t)i * a.n + j];
            v[1 + i] += a.p[(size_t)i * a.n + j] / (U - x) + a.q[(size_t)i * a.n + j] / (x - L);
        }
        v[0] += pow(pl / pow(U - x, 2.0) - ql / pow(x - L, 2.0) - gsi + ita, 2.0);
        v[0] += pow(gsi * (x - a.alpha[j]) - a.eps, 2.0);
        v[0] += pow(ita * (a.beta[j] - x) - a.eps, 2.0);
    }
    block_sums<1 + kMmaMaxM>(v, 1 + a.m, a.partial, false);
}

__global__ void k_mma_fold(const double *partial, int nblk, int nsum, int use_max, double *out) {
    const int s = threadIdx.x;
    if (s >= nsum) return;
    double x = partial[s];
    for (int b = 1; b < nblk; ++b) x = use_max ? fmax(x, partial[(size_t)b * nsum + s]) : x + partial[(size_t)b * nsum + s];
    out[s] = x;
}

// Gaussian elimination with partial pivoting (solvels, mma.h:13-55), row-major (m+1)^2
std::vector<double> solvels(std::vector<double> A, std::vector<double> b) {
    const int N = (int)b.size();
    auto at = [&](int i, int j) -> double & { return A[(size_t)i * N + j]; };
    for (int i = 0; i < N - 1; i++) {
        double pivot = fabs(at(i, i));
        int pivoti = i;
        for (int j = i + 1; j < N; j++)
            if (pivot < fabs(at(j, i))) { pivot = fabs(at(j, i)); pivoti = j; }
        if (pivoti != i) {
            std::swap(b[i], b[pivoti]);
            for (int j = i; j < N; j++) std::swap(at(i, j), at(pivoti, j));
        }
        for (int j = i + 1; j < N; j++) {
            for (int k = i + 1; k < N; k++) at(j, k) -= at(i, k) * at(j, i) / at(i, i);
            b[j] -= b[i] * at(j, i) / at(i, i);
        }
    }
    std::vector<double> x(N);
    for (int i = N - 1; i >= 0; i--) {
        x[i] = b[i];
        for (int j = N - 1; j > i; j--) x[i] -= x[j] * at(i, j);
        x[i] /= at(i, i);
    }
    return x;
}

}  // namespace

struct pl_mma_s {
    int n = 0, m = 0, k = 0;
    double a0 = 0.0, previous = 0.0;
    std::vector<double> a, c, d;
    double params[7] = {0.5, 0.5, 0.7, 1.2, 0.1, 1.0e-5, 1.0e-6};   // move asyinit asydecr asyincr albefa raa0 epsvalue
    cudaStream_t st = nullptr;
    double *buf = nullptr;          // all device arrays
    double *fold = nullptr;         // folded sums (device)
    MmaArgs args;
    int nblk = 1;
};

static int mma_err(const char *msg) { return pl::record_error(PL_ERR_ARG, msg); }
static int mma_cuda(cudaError_t e) { return e == cudaSuccess ? PL_OK : pl::record_error(PL_ERR_CUDA, cudaGetErrorString(e)); }

extern "C" {

int pl_mma_create(int n, int m, double a0, const double *a, const double *c, const double *d, const double *xmin,
                  const double *xmax, pl_mma *out) {
    if (!out || n < 1 || m < 1 || m > kMmaMaxM || !a || !c || !d || !xmin || !xmax)
        return mma_err("pl_mma_create: n >= 1, 1 <= m <= 4 and all arrays are required");
    *out = nullptr;
    pl_mma h = new pl_mma_s;
    h->n = n; h->m = m; h->a0 = a0;
    h->a.assign(a, a + m); h->c.assign(c, c + m); h->d.assign(d, d + m);
    h->nblk = std::min(kMaxBlocks, std::max(1, (n + kRT - 1) / kRT));
    // arrays of n: xmin xmax xkm1 xkm2 L U alpha beta p0 q0 x gsi ita Dx deltilx dx dgsi dita xt gsit itat
    //              xk dfdx (21 + 2); arrays of m*n: p q G dgdx (4)
    const size_t nn = (size_t)n, n1 = 23, nm = 4;
    const size_t total = n1 * nn + nm * (size_t)m * nn + (size_t)kMaxBlocks * kMaxSums;
    cudaError_t e = cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&h->buf, sizeof(double) * total);
    if (e == cudaSuccess) e = cudaMalloc(&h->fold, sizeof(double) * kMaxSums);
    if (e != cudaSuccess) { pl_mma_destroy(h); return pl::record_error(PL_ERR_ALLOC, cudaGetErrorString(e)); }
    double *p = h->buf;
    MmaArgs &A = h->args;
    memset(&A, 0, sizeof A);
    A.n = n; A.m = m;
    double **slots[] = {&A.xmin, &A.xmax, &A.xkm1, &A.xkm2, &A.L, &A.U, &A.alpha, &A.beta, &A.p0, &A.q0, &A.x, &A.gsi,
                        &A.ita, &A.Dx, &A.deltilx, &A.dx, &A.dgsi, &A.dita, &A.xt, &A.gsit, &A.itat};
    for (double **s : slots) { *s = p; p += nn; }
    double *xk = p; p += nn;
    double *dfdx = p; p += nn;
    A.xk = xk; A.dfdx = dfdx;
    A.p = p; p += (size_t)m * nn;
    A.q = p; p += (size_t)m * nn;
    A.G = p; p += (size_t)m * nn;
    A.dgdx = p; p += (size_t)m * nn;
    A.partial = p;
    e = cudaMemcpyAsync(A.xmin, xmin, sizeof(double) * nn, cudaMemcpyHostToDevice, h->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(A.xmax, xmax, sizeof(double) * nn, cudaMemcpyHostToDevice, h->st);
    if (e == cudaSuccess) e = cudaMemsetAsync(A.xkm1, 0, sizeof(double) * nn, h->st);
    if (e == cudaSuccess) e = cudaMemsetAsync(A.xkm2, 0, sizeof(double) * nn, h->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
    if (e != cudaSuccess) { pl_mma_destroy(h); return mma_cuda(e); }
    *out = h;
    return PL_OK;
}

int pl_mma_destroy(pl_mma h) {
    if (!h) return PL_OK;
    if (h->st) cudaStreamSynchronize(h->st);
    cudaFree(h->buf);
    cudaFree(h->fold);
    if (h->st) cudaStreamDestroy(h->st);
    delete h;
    return PL_OK;
}

int pl_mma_set_param(pl_mma h, int which, double value) {
    if (!h || which < 0 || which > 6) return mma_err("pl_mma_set_param: unknown parameter");
    h->params[which] = value;
    return PL_OK;
}

int pl_mma_get_state(pl_mma h, int *k, double *previous, double *xkm2, double *xkm1, double *L, double *U) {
    if (!h || !k || !previous || !xkm2 || !xkm1 || !L || !U) return mma_err("pl_mma_get_state: null argument");
    *k = h->k;
    *previous = h->previous;
    const size_t bytes = sizeof(double) * h->n;
    cudaError_t e;
    if ((e = cudaMemcpyAsync(xkm2, h->args.xkm2, bytes, cudaMemcpyDeviceToHost, h->st)) ||
        (e = cudaMemcpyAsync(xkm1, h->args.xkm1, bytes, cudaMemcpyDeviceToHost, h->st)) ||
        (e = cudaMemcpyAsync(L, h->args.L, bytes, cudaMemcpyDeviceToHost, h->st)) ||
        (e = cudaMemcpyAsync(U, h->args.U, bytes, cudaMemcpyDeviceToHost, h->st)) || (e = cudaStreamSynchronize(h->st)))
        return mma_cuda(e);
    return PL_OK;
}

int pl_mma_set_state(pl_mma h, int k, double previous, const double *xkm2, const double *xkm1, const double *L,
                     const double *U) {
    if (!h || k < 0 || !xkm2 || !xkm1 || !L || !U) return mma_err("pl_mma_set_state: bad argument");
    h->k = k;
    h->previous = previous;
    const size_t bytes = sizeof(double) * h->n;
    cudaError_t e;
    if ((e = cudaMemcpyAsync(h->args.xkm2, xkm2, bytes, cudaMemcpyHostToDevice, h->st)) ||
        (e = cudaMemcpyAsync(h->args.xkm1, xkm1, bytes, cudaMemcpyHostToDevice, h->st)) ||
        (e = cudaMemcpyAsync(h->args.L, L, bytes, cudaMemcpyHostToDevice, h->st)) ||
        (e = cudaMemcpyAsync(h->args.U, U, bytes, cudaMemcpyHostToDevice, h->st)) || (e = cudaStreamSynchronize(h->st)))
        return mma_cuda(e);
    return PL_OK;
}

int pl_mma_update(pl_mma h, double *xk, double f, const double *dfdx, const double *g, const double *dgdx) {
    if (!h || !xk || !dfdx || !g || !dgdx) return mma_err("pl_mma_update: null argument");
    const int n = h->n, m = h->m;
    MmaArgs &A = h->args;
    cudaStream_t st = h->st;
    cudaError_t e;
    int r;
    // host helper: fold the block partials of the last kernel into `nsum` values
    auto fold = [&](int nsum, bool use_max, double *outv) -> int {
        k_mma_fold<<<1, 64, 0, st>>>(A.partial, h->nblk, nsum, use_max ? 1 : 0, h->fold);
        cudaError_t ee = cudaMemcpyAsync(outv, h->fold, sizeof(double) * nsum, cudaMemcpyDeviceToHost, st);
        if (ee == cudaSuccess) ee = cudaStreamSynchronize(st);
        return mma_cuda(ee);
    };
    if ((e = cudaMemcpyAsync(const_cast<double *>(A.xk), xk, sizeof(double) * n, cudaMemcpyHostToDevice, st)) ||
        (e = cudaMemcpyAsync(const_cast<double *>(A.dfdx), dfdx, sizeof(double) * n, cudaMemcpyHostToDevice, st)) ||
        (e = cudaMemcpyAsync(const_cast<double *>(A.dgdx), dgdx, sizeof(double) * n * m, cudaMemcpyHostToDevice, st)))
        return mma_cuda(e);
    A.k = h->k;
    A.move = h->params[0]; A.asyinit = h->params[1]; A.asydecr = h->params[2]; A.asyincr = h->params[3];
    A.albefa = h->params[4]; A.raa0 = h->params[5];
    const int nb = h->nblk;
    k_mma_prep<<<nb, kRT, 0, st>>>(A);
    double bsum[kMmaMaxM];
    if ((r = fold(m, false, bsum))) return r;
    std::vector<double> b(m);
    for (int i = 0; i < m; i++) b[i] = bsum[i] - g[i];

    // inner loop (mma.h:283-540); host state of the m dual variables
    double eps = 1.0, z = 1.0, zeta = 1.0;
    std::vector<double> y(m, 1.0), lambda(m, 1.0), s(m, 1.0), mu(m);
    for (int i = 0; i < m; i++) mu[i] = std::max(1.0, 0.5 * h->c[i]);
    const std::vector<double> &av = h->a, &cv = h->c, &dv = h->d;
    // KKT norm at the trial point (tau, trial duals); writes the trial variables on the device
    auto kkt = [&](double tau, const std::vector<double> &yt, double zt, const std::vector<double> &lt,
                   const std::vector<double> &mt, double zetat, const std::vector<double> &stv, double *norm) -> int {
        A.tau = tau;
        A.eps = eps;
        for (int i = 0; i < m; i++) A.lambda[i] = lt[i];
        k_mma_kkt<<<nb, kRT, 0, st>>>(A);
        double sums[1 + kMmaMaxM];
        int rr = fold(1 + m, false, sums);
        if (rr) return rr;
        double nrm = sums[0];
        for (int i = 0; i < m; i++) {
            nrm += pow(cv[i] + dv[i] * yt[i] - lt[i] - mt[i], 2.0);
            nrm += pow(sums[1 + i] - av[i] * zt - yt[i] + stv[i] - b[i], 2.0);
            nrm += pow(mt[i] * yt[i] - eps, 2.0);
            nrm += pow(lt[i] * stv[i] - eps, 2.0);
        }
        double la = 0.0;
        for (int i = 0; i < m; i++) la += lt[i] * av[i];
        nrm += pow(h->a0 - zetat - la, 2.0);
        nrm += pow(zetat * zt - eps, 2.0);
        *norm = sqrt(nrm);
        return PL_OK;
    };
    for (int l = 0; eps > 1.0e-7 && l < 10000; l++) {
        A.eps = eps;
        for (int i = 0; i < m; i++) A.lambda[i] = lambda[i];
        k_mma_coef<<<nb, kRT, 0, st>>>(A);
        double sums[kMaxSums];
        if ((r = fold(m * (m + 2), false, sums))) return r;
        std::vector<double> Dy(m), Dlambda(m), deltily(m), deltillambda(m), Dlambday(m), deltillambday(m);
        for (int i = 0; i < m; i++) {
            Dy[i] = dv[i] + mu[i] / y[i];
            Dlambda[i] = s[i] / lambda[i];
            deltily[i] = cv[i] + dv[i] * y[i] - lambda[i] - eps / y[i];
        }
        double la = 0.0;
        for (int i = 0; i < m; i++) la += lambda[i] * av[i];
        const double deltilz = h->a0 - eps / z - la;
        for (int i = 0; i < m; i++) {
            deltillambda[i] = sums[i] - av[i] * z - y[i] - b[i] + eps / lambda[i];
            Dlambday[i] = Dlambda[i] + 1.0 / Dy[i];
            deltillambday[i] = deltillambda[i] + deltily[i] / Dy[i];
        }
        // Newton direction of the duals: the (m+1) system of the n > m branch
        std::vector<double> Am((size_t)(m + 1) * (m + 1), 0.0), B(m + 1);
        for (int ii = 0; ii < m; ii++) {
            for (int jj = 0; jj < m; jj++) Am[(size_t)ii * (m + 1) + jj] = sums[m + ii * m + jj];
            Am[(size_t)ii * (m + 1) + ii] += Dlambday[ii];
            Am[(size_t)ii * (m + 1) + m] = av[ii];
            Am[(size_t)m * (m + 1) + ii] = av[ii];
        }
        Am[(size_t)m * (m + 1) + m] = -zeta / z;
        for (int ii = 0; ii < m; ii++) B[ii] = sums[m + m * m + ii] + deltillambday[ii];
        B[m] = deltilz;
        const std::vector<double> dlz = solvels(Am, B);
        std::vector<double> dlambda(m), dy(m), dmu(m), ds(m);
        for (int i = 0; i < m; i++) { dlambda[i] = dlz[i]; A.dlambda[i] = dlz[i]; }
        const double dz = dlz[m];
        k_mma_dir<<<nb, kRT, 0, st>>>(A);
        double txmax;
        if ((r = fold(1, true, &txmax))) return r;
        for (int i = 0; i < m; i++) {
            dy[i] = dlambda[i] / Dy[i] - deltily[i] / Dy[i];
            dmu[i] = -mu[i] * dy[i] / y[i] - mu[i] + eps / y[i];
            ds[i] = -s[i] * dlambda[i] / lambda[i] - s[i] + eps / lambda[i];
        }
        const double dzeta = -zeta * dz / z - zeta + eps / z;
        double tymax = 0.0;
        for (int i = 0; i < m; i++) {
            const double t = std::max({-1.01 * dy[i] / y[i], -1.01 * dlambda[i] / lambda[i], -1.01 * dmu[i] / mu[i],
                                       -1.01 * ds[i] / s[i]});
            if (tymax < t) tymax = t;
        }
        double tau = 1.0 / std::max({1.0, txmax, tymax, -1.01 * dz / z, -1.01 * dzeta / zeta});
        double deltawl;
        if ((r = kkt(0.0, y, z, lambda, mu, zeta, s, &deltawl))) return r;
        std::vector<double> yt(m), lt(m), mt(m), stv(m);
        double zt = z, zetat = zeta, deltawlp1 = 0.0;
        for (int ll = 0; ll < 50; ll++) {
            for (int i = 0; i < m; i++) {
                yt[i] = y[i] + tau * dy[i];
                lt[i] = lambda[i] + tau * dlambda[i];
                mt[i] = mu[i] + tau * dmu[i];
                stv[i] = s[i] + tau * ds[i];
            }
            zt = z + tau * dz;
            zetat = zeta + tau * dzeta;
            if ((r = kkt(tau, yt, zt, lt, mt, zetat, stv, &deltawlp1))) return r;
            if (deltawlp1 < deltawl) break;
            tau *= 0.5;
        }
        // accept the last trial point: swap the trial arrays in
        std::swap(A.x, A.xt);
        std::swap(A.gsi, A.gsit);
        std::swap(A.ita, A.itat);
        y = yt; z = zt; lambda = lt; mu = mt; zeta = zetat; s = stv;
        eps *= deltawlp1 < 0.9 * eps ? 0.1 : 1.0;
    }
    // outer counters and history (mma.h:541-547)
    h->previous = f;
    h->k++;
    if ((e = cudaMemcpyAsync(A.xkm2, A.xkm1, sizeof(double) * n, cudaMemcpyDeviceToDevice, st)) ||
        (e = cudaMemcpyAsync(A.xkm1, A.xk, sizeof(double) * n, cudaMemcpyDeviceToDevice, st)) ||
        (e = cudaMemcpyAsync(xk, A.x, sizeof(double) * n, cudaMemcpyDeviceToHost, st)) ||
        (e = cudaStreamSynchronize(st)))
        return mma_cuda(e);
    return PL_OK;
}

}  // extern "C"
