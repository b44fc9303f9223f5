// pgb_device.cuh -- device-side building blocks shared by the kernels.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include "pgb_internal.h"

namespace pgb {

// ---------------------------------------------------------------------------
// FP64 plain form.  Translation units that include these are compiled with
// -fmad=false so that every product and sum rounds once, in the order the
// reference writes it.
// ---------------------------------------------------------------------------

// Container::putInBC (include/container.h:50-54), all directions periodic.
__device__ __forceinline__ double min_image(double x, double L, double Linv) {
    return x - L * floor(x * Linv + 0.5);
}

__device__ __forceinline__ double3 sep64(const PathView& v, int s, int p1, int p2) {
    // Path::getSeparation(bead1, bead2) = r1 - r2 in BC (path.h:179-184)
    const double* x = v.pos + (size_t)s * 3 * v.Ne;
    double3 d;
    d.x = min_image(x[p1] - x[p2], v.side[0], v.sideInv[0]);
    d.y = min_image(x[v.Ne + p1] - x[v.Ne + p2], v.side[1], v.sideInv[1]);
    d.z = min_image(x[2 * v.Ne + p1] - x[2 * v.Ne + p2], v.side[2], v.sideInv[2]);
    return d;
}

__device__ __forceinline__ double dot3(double3 a, double3 b) {
    double r = 0.0;
    r += a.x * b.x; r += a.y * b.y; r += a.z * b.z;
    return r;
}

// TabulatedPotential::direct (include/potential.h:249-260); extremal values 0.
__device__ __forceinline__ double table_direct(const double* T, double r, double dr, int len) {
    double q = r / dr;
    if (!(q < (double)len)) return 0.0;     // also catches NaN
    int k = (int)q;
    if (k <= 0) return 0.0;
    return __ldg(T + k);
}

__device__ __forceinline__ double V64(const PathView& v, double3 d) {
    return table_direct(v.tV, sqrt(dot3(d, d)), v.dr, v.tableLength);
}
__device__ __forceinline__ double3 gradV64(const PathView& v, double3 d) {
    double rn = sqrt(dot3(d, d));
    double g = table_direct(v.tdV, rn, v.dr, v.tableLength) / rn;
    return make_double3(g * d.x, g * d.y, g * d.z);
}
__device__ __forceinline__ double grad2V64(const PathView& v, double3 d) {
    return table_direct(v.td2V, sqrt(dot3(d, d)), v.dr, v.tableLength);
}

// Worm::getState (include/worm.h:110-118): 0 HEADTAIL, 1 SPECIAL, 2 NONE
__device__ __forceinline__ int bead_state(const PathView& v, int s, int p) {
    if ((s == v.worm[0] && p == v.worm[1]) || (s == v.worm[2] && p == v.worm[3])) return 0;
    if ((s == v.worm[4] && p == v.worm[5]) || (s == v.worm[6] && p == v.worm[7])) return 1;
    return 2;
}
// Worm::factor(state1, bead2) (src/worm.cpp:108-118)
__device__ __forceinline__ double pair_factor(int st1, int st2) {
    if (st1 == 2 && st2 == 2) return 1.0;
    if (st1 == 0 && st2 == 0) return 0.0;
    return 0.5;
}

// ---------------------------------------------------------------------------
// Reductions (shuffle based; no warp-synchronous shared-memory code).
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T warp_sum(T x) {
    #pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    return x;
}

// Block-wide sum; every thread gets the result.  `red` needs blockDim/32
// entries.  Deterministic for a fixed block size.
template <typename T>
__device__ __forceinline__ T block_sum(T x, T* red) {
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    x = warp_sum(x);
    __syncthreads();
    if (lane == 0) red[w] = x;
    __syncthreads();
    T t = T(0);
    for (int i = 0; i < nw; ++i) t += red[i];
    return t;
}

// Round to nearest (ties to even) for |x| < 2^22 with two FP32 adds: adding
// and removing 1.5 * 2^23 drops the fraction bits.  Unlike rintf this stays
// on the FMA/ALU pipes; __fadd_rn/__fsub_rn are never contracted or
// reassociated.
__device__ __forceinline__ float rint_add(float x) {
    return __fsub_rn(__fadd_rn(x, 12582912.0f), 12582912.0f);
}

// ---------------------------------------------------------------------------
// FP32 Aziz pair evaluation (mixed precision).  Analytic form of
// AzizPotential::valueV / valuedVdr (potential.cpp:1821-1870) with the
// damping F(x) = exp(-max(D/x - 1, 0)^2) written branch-free.  Valid for
// x >= 0.01 (the hard-core branch below that is never reached by physical
// configurations; the self pair is excluded by the callers).
// ---------------------------------------------------------------------------
struct AzizF {
    float rm, rminv, A, eps, alpha, beta, D, C6, C8, C10, eps_rm;
};

inline AzizF make_aziz_f(const AzizParams& a) {
    AzizF f;
    f.rm = (float)a.rm; f.rminv = (float)(1.0 / a.rm); f.A = (float)a.A;
    f.eps = (float)a.epsilon; f.alpha = (float)a.alpha; f.beta = (float)a.beta;
    f.D = (float)a.D; f.C6 = (float)a.C6; f.C8 = (float)a.C8; f.C10 = (float)a.C10;
    f.eps_rm = (float)(a.epsilon / a.rm);
    return f;
}

__device__ __forceinline__ float aziz_v32(float r2, const AzizF& a) {
    float rinv = rsqrtf(r2);
    float x = r2 * rinv * a.rminv;
    float ix = rinv * a.rm;
    float ix2 = ix * ix;
    float ix6 = ix2 * ix2 * ix2;
    float poly = ix6 * fmaf(ix2, fmaf(ix2, a.C10, a.C8), a.C6);
    float urep = a.A * __expf(x * fmaf(a.beta, x, -a.alpha));
    float t = fmaxf(fmaf(a.D, ix, -1.0f), 0.0f);
    float F = __expf(-t * t);
    return a.eps * fmaf(-poly, F, urep);
}

// returns (dV/dr)/r so that gradV = g * sep
__device__ __forceinline__ float aziz_g32(float r2, const AzizF& a) {
    float rinv = rsqrtf(r2);
    float x = r2 * rinv * a.rminv;
    float ix = rinv * a.rm;
    float ix2 = ix * ix;
    float ix6 = ix2 * ix2 * ix2;
    float e = __expf(x * fmaf(a.beta, x, -a.alpha));
    float T1 = a.A * fmaf(2.0f * a.beta, x, -a.alpha) * e;
    float t = fmaxf(fmaf(a.D, ix, -1.0f), 0.0f);
    float F = __expf(-t * t);
    float p1 = ix * ix6 * fmaf(ix2, fmaf(ix2, 10.0f * a.C10, 8.0f * a.C8), 6.0f * a.C6);
    float p0 = ix6 * fmaf(ix2, fmaf(ix2, a.C10, a.C8), a.C6);
    float dF = 2.0f * a.D * ix2 * t * F;
    float dvdr = a.eps_rm * (T1 + p1 * F - p0 * dF);
    return dvdr * rinv;
}

// V and (dV/dr)/r together (shared exponentials)
__device__ __forceinline__ void aziz_vg32(float r2, const AzizF& a, float& V, float& g) {
    float rinv = rsqrtf(r2);
    float x = r2 * rinv * a.rminv;
    float ix = rinv * a.rm;
    float ix2 = ix * ix;
    float ix6 = ix2 * ix2 * ix2;
    float e = __expf(x * fmaf(a.beta, x, -a.alpha));
    float t = fmaxf(fmaf(a.D, ix, -1.0f), 0.0f);
    float F = __expf(-t * t);
    float p0 = ix6 * fmaf(ix2, fmaf(ix2, a.C10, a.C8), a.C6);
    V = a.eps * fmaf(-p0, F, a.A * e);
    float T1 = a.A * fmaf(2.0f * a.beta, x, -a.alpha) * e;
    float p1 = ix * ix6 * fmaf(ix2, fmaf(ix2, 10.0f * a.C10, 8.0f * a.C8), 6.0f * a.C6);
    float dF = 2.0f * a.D * ix2 * t * F;
    g = a.eps_rm * (T1 + p1 * F - p0 * dF) * rinv;
}

__device__ __forceinline__ float min_image32(float x, float L, float Linv) {
    return fmaf(-L, rint_add(x * Linv), x);
}

// Kahan-compensated FP32 accumulator, folded into FP64 at the end.
struct KahanF {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float x) {
        float y = x - c;
        float t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};

// Sums over the warp without the FP64 pipe.  Each butterfly step adds the
// leading parts with an error-free TwoSum (Knuth) and carries the error with
// the trailing parts, so the pair (hi, lo) keeps about 48 bits.  TwoSum's
// error term is exact whichever operand comes first, so every lane ends with
// the same bits.
__device__ __forceinline__ float2 ff_butterfly(float hi, float lo) {
    #pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float h2 = __shfl_xor_sync(0xffffffffu, hi, o);
        const float l2 = __shfl_xor_sync(0xffffffffu, lo, o);
        const float sum = hi + h2;
        const float bp = sum - hi;
        const float err = (hi - (sum - bp)) + (h2 - bp);
        hi = sum;
        lo = (lo + l2) + err;
    }
    return make_float2(hi, lo);
}

// the lanes' Kahan accumulators (value s - c) summed as a (hi, lo) pair
__device__ __forceinline__ float2 warp_ff(const KahanF& k) { return ff_butterfly(k.s, -k.c); }

// the same rounded to FP64 once
__device__ __forceinline__ double warp_sum_ff(const KahanF& k) {
    const float2 v = warp_ff(k);
    return (double)v.x + (double)v.y;
}

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), counter-based RNG.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint4 philox4x32(uint4 c, uint2 k) {
    #pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
        uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
        c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
        k.x += 0x9E3779B9u; k.y += 0xBB67AE85u;
    }
    return c;
}

// sum_j exp(2 pi i n . u_j) over the n beads su[0..n) (u = r / L per
// dimension, turns), for one wave vector n = q L / 2 pi.  The phase is
// reduced in turns per dimension with an exact FMA remainder,
//     frac_d = fma(n_d, u_d, -rint(n_d u_d)),
// then once more after the sum, so __sincosf always sees |angle| <= pi.
// 32-bead partial sums are added with Kahan compensation.
__device__ __forceinline__ float2 rho_partial(const float4* __restrict__ su, int n, float nx,
                                              float ny, float nz) {
    KahanF re, im;
    int j = 0;
    while (j < n) {
        float cr = 0.f, ci = 0.f;
        const int jend = min(n, j + 32);
        #pragma unroll 4
        for (; j < jend; ++j) {
            const float4 u = su[j];
            const float fx = fmaf(nx, u.x, -rint_add(nx * u.x));
            const float fy = fmaf(ny, u.y, -rint_add(ny * u.y));
            const float fz = fmaf(nz, u.z, -rint_add(nz * u.z));
            float f = fx + fy + fz;
            f -= rint_add(f);
            float sn, cs;
            __sincosf(6.28318530717958647692f * f, &sn, &cs);
            cr += cs;
            ci += sn;
        }
        re.add(cr);
        im.add(ci);
    }
    return make_float2(re.s - re.c, im.s - im.c);
}

// Fixed-point form of the phase for lattice wave vectors q = 2 pi n / L
// (integer n_d).  With positions as 32-bit fractions of the box,
// U_d = round(r_d / L_d 2^32) mod 2^32, the phase in turns is
// n . U / 2^32, and the 32-bit integer multiply-adds wrap exactly modulo one
// turn: no rounding, no range reduction.  The top 23 bits (rounded) become an
// angle in [-pi, pi) through an exponent trick on the add pipe.
__device__ __forceinline__ int fixed_turns(double u) {
    // u = r / L; |u| <= 1 for positions inside the box
    return (int)(unsigned int)(long long)rint(u * 4294967296.0);
}

__device__ __forceinline__ float2 rho_partial_lattice(const int4* __restrict__ su, int n, int nx,
                                                      int ny, int nz) {
    KahanF re, im;
    int j = 0;
    while (j < n) {
        float cr = 0.f, ci = 0.f;
        const int jend = min(n, j + 32);
        #pragma unroll 4
        for (; j < jend; ++j) {
            const int4 u = su[j];
            // unsigned arithmetic: the products wrap modulo 2^32 by definition
            const unsigned int p = (unsigned int)nx * (unsigned int)u.x + (unsigned int)ny * (unsigned int)u.y +
                                   (unsigned int)nz * (unsigned int)u.z + 0x80000100u;
            const float t = __uint_as_float(0x4B000000u | (p >> 9)) - 8388608.0f;   // [0, 2^23)
            float sn, cs;
            __sincosf(fmaf(t, 7.490140565847857e-07f, -3.14159265358979f), &sn, &cs);   // 2 pi / 2^23
            cr += cs;
            ci += sn;
        }
        re.add(cr);
        im.add(ci);
    }
    return make_float2(re.s - re.c, im.s - im.c);
}

// FP32 -> FP64 with integer operations: exact for normal numbers, zero,
// infinities and NaN; FP32 subnormals become signed zero.  For epilogues that
// would otherwise queue one conversion per output on the narrow FP64 pipe.
__device__ __forceinline__ double f32_to_f64_alu(float f) {
    const unsigned int b = __float_as_uint(f);
    const unsigned int e = (b >> 23) & 0xFFu;
    const unsigned long long sign = (unsigned long long)(b >> 31) << 63;
    const unsigned long long ex = (e == 0u) ? 0ull : (e == 0xFFu) ? 0x7FFull : (unsigned long long)(e + 896u);
    const unsigned long long mant = (e == 0u) ? 0ull : (unsigned long long)(b & 0x7FFFFFu) << 29;
    return __longlong_as_double((long long)(sign | (ex << 52) | mant));
}

// Nanoseconds of the GPU's global timer (PTX %globaltimer).
__device__ __forceinline__ unsigned long long gtimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ float u01f(uint32_t x) {          // [0,1)
    return (float)(x >> 8) * (1.0f / 16777216.0f);
}
__device__ __forceinline__ double u01d(uint32_t hi, uint32_t lo) {  // [0,1)
    uint64_t v = ((uint64_t)hi << 21) ^ (uint64_t)(lo >> 11);
    return (double)(v & ((1ull << 53) - 1)) * (1.0 / 9007199254740992.0);
}
// two standard normals from two uniforms (Box-Muller), FP32
__device__ __forceinline__ float2 box_muller(uint32_t a, uint32_t b) {
    float u1 = ((float)(a >> 8) + 0.5f) * (1.0f / 16777216.0f);   // (0,1)
    float u2 = u01f(b);
    float r = sqrtf(-2.0f * __logf(u1));
    float sn, cs;
    __sincosf(6.28318530717958647692f * u2, &sn, &cs);
    return make_float2(r * cs, r * sn);
}

}  // namespace pgb
