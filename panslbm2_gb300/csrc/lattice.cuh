// lattice.cuh -- D2Q9 / D3Q15 velocity sets and population storage formats.
//
// Velocity order and weights follow the reference particle classes exactly
// (src/particle/d2q9.h:160-163, src/particle/d3q15.h:251-254): boundary conditions are
// written against these indices, so the order is part of the interface.
#pragma once
#include <cuda_fp16.h>
#include <cuda_bf16.h>
#include <stdint.h>

namespace pl {

struct D2Q9 {
    static constexpr int Q = 9, ND = 2;
    __host__ __device__ static constexpr int cx(int c) {
        return c == 1 ? 1 : c == 3 ? -1 : c == 5 ? 1 : c == 6 ? -1 : c == 7 ? -1 : c == 8 ? 1 : 0;
    }
    __host__ __device__ static constexpr int cy(int c) {
        return c == 2 ? 1 : c == 4 ? -1 : c == 5 ? 1 : c == 6 ? 1 : c == 7 ? -1 : c == 8 ? -1 : 0;
    }
    __host__ __device__ static constexpr int cz(int) { return 0; }
    // weight numerators over 36
    __host__ __device__ static constexpr int w36(int c) { return c == 0 ? 16 : (c <= 4 ? 4 : 1); }
    template <class T> __host__ __device__ static constexpr T w(int c) {
        return c == 0 ? T(4.0 / 9.0) : (c <= 4 ? T(1.0 / 9.0) : T(1.0 / 36.0));
    }
};

struct D3Q15 {
    static constexpr int Q = 15, ND = 3;
    __host__ __device__ static constexpr int cx(int c) {
        return c == 1 ? 1 : c == 4 ? -1 : c == 7 ? 1 : c == 8 ? -1 : c == 9 ? 1 : c == 10 ? 1 : c == 11 ? -1
             : c == 12 ? 1 : c == 13 ? -1 : c == 14 ? -1 : 0;
    }
    __host__ __device__ static constexpr int cy(int c) {
        return c == 2 ? 1 : c == 5 ? -1 : c == 7 ? 1 : c == 8 ? 1 : c == 9 ? -1 : c == 10 ? 1 : c == 11 ? -1
             : c == 12 ? -1 : c == 13 ? 1 : c == 14 ? -1 : 0;
    }
    __host__ __device__ static constexpr int cz(int c) {
        return c == 3 ? 1 : c == 6 ? -1 : c == 7 ? 1 : c == 8 ? 1 : c == 9 ? 1 : c == 10 ? -1 : c == 11 ? -1
             : c == 12 ? -1 : c == 13 ? -1 : c == 14 ? 1 : 0;
    }
    template <class T> __host__ __device__ static constexpr T w(int c) {
        return c == 0 ? T(2.0 / 9.0) : (c <= 6 ? T(1.0 / 9.0) : T(1.0 / 72.0));
    }
};

template <class L> __host__ __device__ constexpr int comp(int c, int a) {
    return a == 0 ? L::cx(c) : (a == 1 ? L::cy(c) : L::cz(c));
}
template <class L> __host__ __device__ constexpr int opp(int c) {
    int r = 0;
    for (int e = 0; e < L::Q; ++e)
        if (L::cx(e) == -L::cx(c) && L::cy(e) == -L::cy(c) && L::cz(e) == -L::cz(c)) r = e;
    return r;
}
template <class L> __host__ __device__ constexpr int refl(int c, int a) {
    int v0 = L::cx(c), v1 = L::cy(c), v2 = L::cz(c);
    if (a == 0) v0 = -v0; else if (a == 1) v1 = -v1; else v2 = -v2;
    int r = 0;
    for (int e = 0; e < L::Q; ++e)
        if (L::cx(e) == v0 && L::cy(e) == v1 && L::cz(e) == v2) r = e;
    return r;
}
template <class L> __host__ __device__ constexpr bool is_diag(int c, int a) {
    // non-zero component along an axis other than a
    return (a != 0 && L::cx(c) != 0) || (a != 1 && L::cy(c) != 0) || (a != 2 && L::cz(c) != 0);
}

// ---- population storage ------------------------------------------------------------------
// Storage type S holds either the population itself (float, double) or the population minus
// a per-direction shift w_c*s0 (half, bfloat16: "shifted" storage keeps the O(1) equilibrium
// part out of the 16-bit mantissa). Compute type is float for 32/16-bit storage, double for
// double storage.
template <class S> struct Store;
template <> struct Store<float> {
    using T = float;
    __device__ __forceinline__ static float ld(const float *p) { return __ldg(p); }
    __device__ __forceinline__ static void st(float *p, float v) { *p = v; }
    __device__ __forceinline__ static float dec(float v, float) { return v; }
    __device__ __forceinline__ static float enc(float v, float) { return v; }
};
template <> struct Store<double> {
    using T = double;
    __device__ __forceinline__ static double ld(const double *p) { return __ldg(p); }
    __device__ __forceinline__ static void st(double *p, double v) { *p = v; }
    __device__ __forceinline__ static double dec(double v, double) { return v; }
    __device__ __forceinline__ static double enc(double v, double) { return v; }
};
template <> struct Store<__half> {
    using T = float;
    __device__ __forceinline__ static __half ld(const __half *p) { return __ldg(p); }
    __device__ __forceinline__ static void st(__half *p, __half v) { *p = v; }
    __device__ __forceinline__ static float dec(__half v, float shift) { return __half2float(v) + shift; }
    __device__ __forceinline__ static __half enc(float v, float shift) { return __float2half_rn(v - shift); }
};
template <> struct Store<__nv_bfloat16> {
    using T = float;
    __device__ __forceinline__ static __nv_bfloat16 ld(const __nv_bfloat16 *p) { return __ldg(p); }
    __device__ __forceinline__ static void st(__nv_bfloat16 *p, __nv_bfloat16 v) { *p = v; }
    __device__ __forceinline__ static float dec(__nv_bfloat16 v, float shift) { return __bfloat162float(v) + shift; }
    __device__ __forceinline__ static __nv_bfloat16 enc(float v, float shift) { return __float2bfloat16_rn(v - shift); }
};

// ---- stochastic rounding of 16-bit stores ----------------------------------------------------
// Round-to-nearest discards every increment below half a 16-bit ulp, so a small source added each
// step (a heat source of 1e-3 on temperatures of order 1) never accumulates. Rounding up with
// probability (x - lo) / (hi - lo) keeps the expected stored value equal to x. r: 16 random bits.
// Other storage types round to nearest.
template <class S> struct StoreSR {
    __device__ __forceinline__ static S enc(typename Store<S>::T v, typename Store<S>::T shift, uint32_t) {
        return Store<S>::enc(v, shift);
    }
};
template <> struct StoreSR<__nv_bfloat16> {
    __device__ __forceinline__ static __nv_bfloat16 enc(float v, float shift, uint32_t r) {
        const float x = v - shift;
        uint32_t b = __float_as_uint(x);
        if ((b & 0x7f800000u) != 0x7f800000u) b += (r & 0xffffu);   // finite: add below the kept bits
        return __ushort_as_bfloat16((unsigned short)(b >> 16));
    }
};
template <> struct StoreSR<__half> {
    __device__ __forceinline__ static __half enc(float v, float shift, uint32_t r) {
        const float x = v - shift;
        const __half lo = __float2half_rz(x);
        const unsigned short lb = __half_as_ushort(lo);
        if ((lb & 0x7c00u) == 0x7c00u) return lo;                      // inf / nan
        const __half hi = __ushort_as_half((unsigned short)(lb + 1));  // next magnitude away from 0
        const float flo = __half2float(lo), fhi = __half2float(hi);
        const float p = (x - flo) / (fhi - flo);
        return float(r & 0xffffu) * (1.0f / 65536.0f) < p ? hi : lo;
    }
};
// per-node random stream: a hashed seed, then xorshift32 per value
__device__ __forceinline__ uint32_t sr_hash(uint32_t a, uint32_t b) {
    uint32_t h = a * 0x9E3779B1u ^ (b + 0x7F4A7C15u) * 0x85EBCA77u;
    h ^= h >> 15; h *= 0x2C1B3C6Du; h ^= h >> 12; h *= 0x297A2D39u; h ^= h >> 15;
    return h | 1u;
}
__device__ __forceinline__ uint32_t sr_next(uint32_t &s) {
    s ^= s << 13; s ^= s >> 17; s ^= s << 5;
    return s;
}

}  // namespace pl
