// noalloc.cu -- pl_residual_device_noalloc: the Residual reduction (residual.h:8-51 of the
// reference) over caller-owned device arrays, with its scratch in a fixed device array of this
// file, so that the call allocates no device or pinned memory.
//
// Which callers need it: pl_residual_host stages its inputs in the handle's grow-only scratch
// pool and reduces into the handle's partial buffer, so it can cudaMalloc on first use or when
// a larger n arrives. A caller that has reserved nearly all of the device memory for lattice
// populations and fields (a large 3D lattice) has no room for that, and a caller that queues
// steps on several streams cannot accept the device-wide synchronisation a cudaMalloc / cudaFree
// brings. Such a caller keeps its macroscopic fields on the device and checks convergence here.
//
// Contract:
//  * scratch: g_scratch holds kMaxPartials FP64 partial pairs (one per reduction block; the
//    reduction never uses more blocks than that) and the three results; g_nonfinite is the
//    non-finite flag of the first pass. Every partial and result is written before it is read;
//    the flag is cleared by each call before its kernels run and read back with the results:
//    a non-finite input value makes the call return PL_ERR_NONFINITE (the status the solve
//    loop reports as divergence), with *out still set. Nothing has to be zeroed by the caller.
//  * pointers: a[m] and b[m] must be device memory of the current device, or managed memory;
//    host memory and device memory of another GPU are rejected with PL_ERR_ARG before any
//    kernel runs.
//  * setup: the first call on a device, with that device current, looks the two symbols up
//    (cudaGetSymbolAddress) and keeps their addresses; later calls on that device reuse them.
//    Make the first call on each device before beginning any stream capture on it.
//  * concurrency: all calls on one device share the one scratch array. Each call waits for its
//    own stream before it returns, so calls from one host thread never overlap; calls from
//    several host threads whose kernels can be on the GPU at the same time race on the scratch
//    and must be serialised by the caller.
//  * the reduction is the same two-pass FP64 tree as pl_residual_host (same block count for the
//    same n), so both entry points give the same value on the same data.
#include <cuda_runtime.h>
#include <stdio.h>

#include <mutex>

#include "../../include/panslbm_gb300.h"
#include "fields.h"
#include "launch.h"

namespace {

constexpr int kMaxPartials = 1024;                    // resid_blocks() never returns more
constexpr int kResultOffset = 2 * kMaxPartials;        // out[0..2] follow the partial pairs
constexpr int kScratchDoubles = kResultOffset + 4;     // 2052 doubles = 16,416 bytes

static __device__ __align__(256) double g_scratch[kScratchDoubles];
static __device__ __align__(256) int g_nonfinite;

constexpr int kMaxDevices = 64;
std::mutex g_mu;
double *g_scratch_addr[kMaxDevices];
int *g_flag_addr[kMaxDevices];

int err(int code, const char *msg) { return pl::record_error(code, msg); }

int cuda_err(const char *what, cudaError_t e) {
    char buf[256];
    snprintf(buf, sizeof buf, "%s: %s", what, cudaGetErrorString(e));
    return pl::record_error(PL_ERR_CUDA, buf);
}

// memory the current device `dev` can read without peer access: its own device memory, or
// managed memory
bool device_readable(const void *p, int dev) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (at.type == cudaMemoryTypeManaged) return true;
    return at.type == cudaMemoryTypeDevice && at.device == dev;
}

}  // namespace

extern "C" int pl_residual_device_noalloc(long long n, int ncomp, const double *const *a, const double *const *b,
                                          void *stream, double *out) {
    if (!a || !b || !out) return err(PL_ERR_ARG, "a, b and out must not be NULL");
    if (ncomp < 1 || ncomp > 3) return err(PL_ERR_ARG, "ncomp must be 1, 2 or 3");
    if (n < 1) return err(PL_ERR_ARG, "n must be at least 1");
    const int nblk = pl::resid_blocks(n);
    if (nblk > kMaxPartials) return err(PL_ERR_ARG, "reduction needs more partials than the static scratch holds");
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_err("cudaGetDevice", e);
    if (dev < 0 || dev >= kMaxDevices) return err(PL_ERR_ARG, "device ordinal beyond the supported range");
    for (int m = 0; m < ncomp; ++m)
        if (!device_readable(a[m], dev) || !device_readable(b[m], dev))
            return err(PL_ERR_ARG, "a[m] and b[m] must be device pointers of the current device (or managed)");
    double *scratch;
    int *flag;
    {
        std::lock_guard<std::mutex> lock(g_mu);
        if (!g_scratch_addr[dev]) {
            void *ps = nullptr, *pf = nullptr;
            if ((e = cudaGetSymbolAddress(&ps, g_scratch)) != cudaSuccess) return cuda_err("cudaGetSymbolAddress(scratch)", e);
            if ((e = cudaGetSymbolAddress(&pf, g_nonfinite)) != cudaSuccess) return cuda_err("cudaGetSymbolAddress(flag)", e);
            g_scratch_addr[dev] = static_cast<double *>(ps);
            g_flag_addr[dev] = static_cast<int *>(pf);
        }
        scratch = g_scratch_addr[dev];
        flag = g_flag_addr[dev];
    }

    cudaStream_t st = static_cast<cudaStream_t>(stream);
    pl::ResidArgs ra;
    ra.ncomp = ncomp;
    ra.n = n;
    for (int m = 0; m < 3; ++m) {
        ra.a[m] = m < ncomp ? a[m] : nullptr;
        ra.b[m] = m < ncomp ? b[m] : nullptr;
    }
    if ((e = cudaMemsetAsync(flag, 0, sizeof(int), st)) != cudaSuccess) return cuda_err("cudaMemsetAsync", e);
    pl::launch_residual(ra, scratch, nblk, flag, scratch + kResultOffset, st);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_err("residual launch", e);
    double o[3];
    int nonfinite = 0;
    if ((e = cudaMemcpyAsync(o, scratch + kResultOffset, sizeof o, cudaMemcpyDeviceToHost, st)) != cudaSuccess)
        return cuda_err("cudaMemcpyAsync", e);
    if ((e = cudaMemcpyAsync(&nonfinite, flag, sizeof nonfinite, cudaMemcpyDeviceToHost, st)) != cudaSuccess)
        return cuda_err("cudaMemcpyAsync", e);
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return cuda_err("cudaStreamSynchronize", e);
    *out = o[2];
    if (nonfinite) return err(PL_ERR_NONFINITE, "non-finite value in the residual inputs");
    return PL_OK;
}
