// fields.h -- node-field kernels (reductions, sensitivities, filters): argument blocks and
// launchers.
#pragma once
#include <cuda_runtime.h>

namespace pl {

struct ResidArgs {
    const double *a[3], *b[3];
    int ncomp;
    long long n;
};
int resid_blocks(long long n);
// out[0] = sum (a-b)^2, out[1] = sum a^2, out[2] = sqrt(out[0]/out[1])
void launch_residual(const ResidArgs &r, double *partial, int nblk, int *nonfinite, double *out, cudaStream_t st);
void launch_normalize(double *v, long long n, double *partial, int nblk, cudaStream_t st);

struct SensArgs {
    int which, n, nx, ny, nz;
    long long np;
    double *dfds;
    const double *dads, *dkds, *qn;
    const int *mask;
    const double *ux, *uy, *uz, *tem;              // forward solution
    const double *imx, *imy, *imz, *item, *iqx, *iqy, *iqz;   // adjoint macros
    const double *kappa;
    const double *g, *ig;                           // snapshots, [q][np]
};
void launch_sensitivity(int q, const SensArgs &s, cudaStream_t st);
// AEL::SensitivityCompliance: dfds[i] += 4.5 s:is - 1.5 irho tr s; in = sxx, sxy, syx, syy, irho,
// isxx, isxy, isyx, isyy (device arrays of n)
void launch_compliance(int n, double *dfds, const double *const *in, cudaStream_t st);
// dst[i] += a * src[i]
void launch_axpy(int n, double *dst, const double *src, double a, cudaStream_t st);

struct FiltArgs {
    int n, nx, ny, nz, ntap;
    const int *di, *dj, *dk;
    const double *hat;
    const int *mask;
    double beta;
    const double *wtab;   // [n][ntap] weights of a general weight functor; replaces hat and mask
};
// op 0: Heaviside projection of the filtered value; 1: Heaviside sensitivity (two passes,
// tmp = N doubles); 2: plain filtered average (DensityFilter)
void launch_filter(int op, const FiltArgs &f, const double *a, const double *b, double *tmp, double *out,
                   cudaStream_t st);
void launch_to_compute(const double *in, void *out, int n, bool fp32, cudaStream_t st);
void launch_snap_to_node_major(const double *snap, long long np, int n, int q, double *out, cudaStream_t st);
void launch_node_major_to_snap(const double *in, long long np, int n, int q, double *snap, cudaStream_t st);

}  // namespace pl
