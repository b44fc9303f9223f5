// gp.cu -- the Gaussian-process external potential on the device.
//
// GaussianProcessPotential::GP (src/potential.cpp:330-392) with the Matern
// kernel of MaternKernel::K (src/gpkernel.cpp:97-108, include/gpkernel.h:
// 61-72): for an inference point r, normalised as (r - offset) / scale,
//     V(r) = mean_d + std_d (mu + sigma2 sum_k K(r, x_k) w_k),
//     K    = k_nu(|putInBC(x_k - r) / ell|),  w_k = (K^-1 Y)_k.
// The CPU kernel applies the container's boundary conditions to the
// separation; the reference's GPU kernel (potential_gpu.cu:4-54) leaves them
// out and divides by ell instead of multiplying by 1/ell.  This file follows
// the CPU form, so both precisions agree with the reference's CPU path.
//
// FP64 kernel (compiled with -fmad=false): one thread per inference point
// and chunk of training points, streamed through shared memory in index
// order; the chunk sums are added in chunk order.  Chunks exist only to fill
// the GPU when a call has few points: from about 155 k points on there is one
// chunk and every sum has the CPU form's order and rounding (up to exp(),
// which may differ by an ulp from the host's); with several chunks the sum is
// regrouped, a relative change of order 1e-16 of sum_k |K w_k|.
// Mixed kernel: the separations and kernel values in FP32 and the sum in a
// double-float pair (TwoSum), about 1e-7 of sum_k |K w_k| off the FP64 value.
//
// GPHeBenzenePotential::V (src/potential.cpp:5610-5681): points are folded
// into the 30-degree wedge of the ring's symmetry on the device, passed
// through the GP, then switched to the long-range form beyond the core.
#include "pgb_device.cuh"

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

namespace pgb {

struct GpDev {
    double off[3], scale[3], invell[3], pside[3], sideInv[3];
    double standard_mean, standard_std, mu, sigma2;
    int nu2;          // 2 nu: 1, 3 or 5
    int n;            // training points
};

constexpr int kGpBlock = 256;
constexpr int kGpTile = 512;            // training points per shared-memory tile

__device__ __forceinline__ double matern64(int nu2, double r) {
    const double kSqrt3 = 1.7320508075688772935, kSqrt5 = 2.2360679774997896964;
    if (nu2 == 1) return exp(-r);
    if (nu2 == 3) { const double x = kSqrt3 * r; return (1.0 + x) * exp(-x); }
    const double x = kSqrt5 * r;
    return (1.0 + x + x * x / 3.0) * exp(-x);
}

__device__ __forceinline__ float matern32(int nu2, float r) {
    const float kSqrt3 = 1.7320508f, kSqrt5 = 2.2360680f;
    if (nu2 == 1) return expf(-r);
    if (nu2 == 3) { const float x = kSqrt3 * r; return (1.0f + x) * expf(-x); }
    const float x = kSqrt5 * r;
    return (1.0f + x + x * x * (1.0f / 3.0f)) * expf(-x);
}

// Grid: x over blocks of kGpBlock inference points, y over chunks of
// `chunk` training points; each thread sums its chunk in index order and
// writes the partial sum; k_gp*_combine adds the chunks in chunk order.  With
// one chunk the FP64 sum is the CPU form's sequential sum.
__global__ void __launch_bounds__(kGpBlock)
k_gp64(GpDev g, const double4* __restrict__ train, const double* __restrict__ pos, int count,
       int chunk, double* __restrict__ part) {
    __shared__ double4 tile[kGpTile];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int kb = blockIdx.y * chunk, ke = min(g.n, kb + chunk);
    double r0 = 0.0, r1 = 0.0, r2 = 0.0;
    if (i < count) {
        r0 = (pos[3 * (size_t)i] - g.off[0]) / g.scale[0];
        r1 = (pos[3 * (size_t)i + 1] - g.off[1]) / g.scale[1];
        r2 = (pos[3 * (size_t)i + 2] - g.off[2]) / g.scale[2];
    }
    double acc = 0.0;
    for (int k0 = kb; k0 < ke; k0 += kGpTile) {
        const int nt = min(kGpTile, ke - k0);
        __syncthreads();
        for (int k = threadIdx.x; k < nt; k += blockDim.x) tile[k] = train[k0 + k];
        __syncthreads();
        if (i < count) {
            for (int k = 0; k < nt; ++k) {
                const double4 t = tile[k];
                double s0 = t.x - r0, s1 = t.y - r1, s2 = t.z - r2;
                s0 -= g.pside[0] * floor(s0 * g.sideInv[0] + 0.5);
                s1 -= g.pside[1] * floor(s1 * g.sideInv[1] + 0.5);
                s2 -= g.pside[2] * floor(s2 * g.sideInv[2] + 0.5);
                s0 = s0 * g.invell[0]; s1 = s1 * g.invell[1]; s2 = s2 * g.invell[2];
                double d2 = 0.0;
                d2 += s0 * s0; d2 += s1 * s1; d2 += s2 * s2;
                acc += matern64(g.nu2, sqrt(d2)) * t.w;
            }
        }
    }
    if (i < count) part[(size_t)blockIdx.y * count + i] = acc;
}

__global__ void k_gp64_combine(GpDev g, const double* __restrict__ part, int nsplit, int count,
                               double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    double acc = part[i];
    for (int s = 1; s < nsplit; ++s) acc += part[(size_t)s * count + i];
    out[i] = g.standard_mean + g.standard_std * (g.mu + g.sigma2 * acc);
}

__device__ __forceinline__ void two_sum_acc(float& hi, float& lo, float x) {
    const float s = __fadd_rn(hi, x);
    const float bp = __fsub_rn(s, hi);
    const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(x, bp));
    hi = s;
    lo = __fadd_rn(lo, e);
}

__global__ void __launch_bounds__(kGpBlock)
k_gp32(GpDev g, const float4* __restrict__ train, const double* __restrict__ pos, int count,
       int chunk, float2* __restrict__ part) {
    __shared__ float4 tile[kGpTile];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int kb = blockIdx.y * chunk, ke = min(g.n, kb + chunk);
    float r0 = 0.f, r1 = 0.f, r2 = 0.f;
    if (i < count) {
        r0 = (float)((pos[3 * (size_t)i] - g.off[0]) / g.scale[0]);
        r1 = (float)((pos[3 * (size_t)i + 1] - g.off[1]) / g.scale[1]);
        r2 = (float)((pos[3 * (size_t)i + 2] - g.off[2]) / g.scale[2]);
    }
    const float ps0 = (float)g.pside[0], ps1 = (float)g.pside[1], ps2 = (float)g.pside[2];
    const float si0 = (float)g.sideInv[0], si1 = (float)g.sideInv[1], si2 = (float)g.sideInv[2];
    const float il0 = (float)g.invell[0], il1 = (float)g.invell[1], il2 = (float)g.invell[2];
    float hi = 0.f, lo = 0.f;
    for (int k0 = kb; k0 < ke; k0 += kGpTile) {
        const int nt = min(kGpTile, ke - k0);
        __syncthreads();
        for (int k = threadIdx.x; k < nt; k += blockDim.x) tile[k] = train[k0 + k];
        __syncthreads();
        if (i < count) {
            for (int k = 0; k < nt; ++k) {
                const float4 t = tile[k];
                float s0 = t.x - r0, s1 = t.y - r1, s2 = t.z - r2;
                s0 = fmaf(-ps0, floorf(fmaf(s0, si0, 0.5f)), s0) * il0;
                s1 = fmaf(-ps1, floorf(fmaf(s1, si1, 0.5f)), s1) * il1;
                s2 = fmaf(-ps2, floorf(fmaf(s2, si2, 0.5f)), s2) * il2;
                const float d = sqrtf(fmaf(s0, s0, fmaf(s1, s1, s2 * s2)));
                two_sum_acc(hi, lo, matern32(g.nu2, d) * t.w);
            }
        }
    }
    if (i < count) part[(size_t)blockIdx.y * count + i] = make_float2(hi, lo);
}

__global__ void k_gp32_combine(GpDev g, const float2* __restrict__ part, int nsplit, int count,
                               double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    double acc = 0.0;
    for (int s = 0; s < nsplit; ++s) {
        const float2 p = part[(size_t)s * count + i];
        acc += (double)p.x + (double)p.y;
    }
    out[i] = g.standard_mean + g.standard_std * (g.mu + g.sigma2 * acc);
}

// --------------------------------------------------------------------------
// GPHeBenzenePotential: fold, GP, long-range switch
// --------------------------------------------------------------------------
struct Benzene {
    double r0, gama, x1, x2, x3, x4, x5, x6, x7, x8, x9, x10, x11, x12;
};

__device__ __forceinline__ double rad2deg(double a) { return (a * 180.0) / 3.14159265358979323846; }
__device__ __forceinline__ double deg2rad(double a) { return (a * 3.14159265358979323846) / 180.0; }

// the fold of GPHeBenzenePotential::V (potential.cpp:5621-5656); cut = 1
// marks the hard core rho < 3, z < 2
__global__ void k_benzene_fold(const double* __restrict__ pos, int count, double* __restrict__ fold,
                               unsigned char* __restrict__ cut) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const double pi = 3.14159265358979323846;
    const double x = pos[3 * (size_t)i], y = pos[3 * (size_t)i + 1];
    double z = pos[3 * (size_t)i + 2];
    double finx = 0.0, finy = 0.0;
    if (z <= 0.0) z = -z;
    double angle = round(rad2deg(atan2(y, x)) * 10000.0) / 10000.0;
    if (angle < 0.0) angle = 180.0 + (180.0 + angle);
    if (angle <= 30.0) {
        finx = x; finy = y;
    } else {
        double rotateangle = fmod(angle, 60.0) - angle;
        if ((angle + rotateangle) > 30.0) {
            rotateangle = deg2rad(rotateangle);
            const double rx = cos(rotateangle) * x - sin(rotateangle) * y;
            const double ry = sin(rotateangle) * x + cos(rotateangle) * y;
            finx = cos(pi / 3.0) * rx + sin(pi / 3.0) * ry;
            finy = sin(pi / 3.0) * rx - cos(pi / 3.0) * ry;
        } else {
            rotateangle = deg2rad(rotateangle);
            finx = cos(rotateangle) * x - sin(rotateangle) * y;
            finy = sin(rotateangle) * x + cos(rotateangle) * y;
        }
    }
    const double rho = sqrt(finx * finx + finy * finy);
    cut[i] = (rho < 3.0 && z < 2.0) ? 1 : 0;
    fold[3 * (size_t)i] = finx; fold[3 * (size_t)i + 1] = finy; fold[3 * (size_t)i + 2] = z;
}

// GPHeBenzenePotential::long_range (include/potential.h:2455-2480)
__device__ double benzene_long_range(const Benzene& b, double x, double y, double z) {
    const double rnorm = sqrt(x * x + y * y + z * z);
    const double ph0 = atan2(y, x);
    const double th0 = acos(z / rnorm);
    const double tt = cos(th0);
    const double fi = ph0;
    const double normm1 = sqrt(5.0) / 5.0;
    const double normm2 = sqrt(13.0) / 13.0;
    const double normm3 = 0.1792151994e-4;
    const double p1 = -b.x1 / pow(rnorm, 6) - b.x2 / pow(rnorm, 8) - b.x3 / pow(rnorm, 10) - b.x4 / pow(rnorm, 12);
    const double p2 = -normm1 * (1.5 * tt * tt - 0.5) *
                      (b.x5 / pow(rnorm, 6) + b.x6 / pow(rnorm, 8) + b.x7 / pow(rnorm, 10) + b.x8 / pow(rnorm, 12));
    const double p3 = -normm2 * (3.0 / 8.0 + 35.0 / 8.0 * pow(tt, 4) - 15.0 / 4.0 * tt * tt);
    const double p4 = (b.x9 / pow(rnorm, 8) + b.x10 / pow(rnorm, 10) + b.x11 / pow(rnorm, 12));
    const double p5 = -normm3 * 10395.0 * pow(1 - tt * tt, 3) * cos(6 * fi) * b.x12 / pow(rnorm, 10);
    return p1 + p2 + p3 * p4 + p5;
}

__global__ void k_benzene_combine(Benzene b, const double* __restrict__ fold,
                                  const unsigned char* __restrict__ cut, const double* __restrict__ gp,
                                  int count, double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    if (cut[i]) { out[i] = 10000.0; return; }
    const double finx = fold[3 * (size_t)i], finy = fold[3 * (size_t)i + 1], z = fold[3 * (size_t)i + 2];
    const double rho = sqrt(finx * finx + finy * finy);
    double d2 = 0.0;
    d2 += finx * finx; d2 += finy * finy; d2 += z * z;
    const double rnorm = sqrt(d2);
    const double h_long = 1.0 / (1.0 + exp(-b.gama * (rnorm - b.r0)));
    double value;
    if (rho > 5.0 || z > 6.5)
        value = (1.0 - h_long) * gp[i] + h_long * benzene_long_range(b, finx, finy, z);
    else
        value = gp[i];
    out[i] = value / 0.695;
}

}  // namespace pgb

// --------------------------------------------------------------------------
// host side
// --------------------------------------------------------------------------
using namespace pgb;

struct pgb_gp {
    pgb_gp_params p{};
    GpDev g{};
    cudaStream_t stream = nullptr;
    double4* d_train64 = nullptr;
    float4* d_train32 = nullptr;
    // per-call scratch: positions, values, fold, cut flags (grown on demand)
    void* d_buf = nullptr;
    size_t buf_bytes = 0;
    void* d_part = nullptr;              // per-chunk partial sums
    size_t part_bytes = 0;
    std::string err;
    int fail(int code, const std::string& m) { err = m; return code; }
    int cfail(cudaError_t e, const char* where) {
        err = std::string("CUDA error ") + cudaGetErrorString(e) + " at " + where;
        return e == cudaErrorMemoryAllocation ? PGB_ENOMEM : PGB_ECUDA;
    }
};

namespace {
thread_local std::string g_gperr;

int ensure_buf(pgb_gp* h, size_t bytes) {
    if (bytes <= h->buf_bytes) return PGB_OK;
    if (h->d_buf) { cudaStreamSynchronize(h->stream); cudaFree(h->d_buf); h->d_buf = nullptr; h->buf_bytes = 0; }
    cudaError_t e = cudaMalloc(&h->d_buf, bytes);
    if (e != cudaSuccess) { h->d_buf = nullptr; return h->cfail(e, "cudaMalloc(GP scratch)"); }
    h->buf_bytes = bytes;
    return PGB_OK;
}

// Chunks of training points so that the grid covers the GPU: about four
// CTAs per SM, chunks no shorter than one shared-memory tile.
int gp_splits(const pgb_gp* h, int count) {
    const int bx = (count + kGpBlock - 1) / kGpBlock;
    const int want = (4 * 152 + bx - 1) / bx;
    const int maxs = (h->g.n + kGpTile - 1) / kGpTile;
    return std::max(1, std::min(want, maxs));
}

cudaError_t launch_gp(pgb_gp* h, const double* d_pos, int count, double* d_out) {
    if (count <= 0) return cudaSuccess;
    const int bx = (count + kGpBlock - 1) / kGpBlock;
    const int ns = gp_splits(h, count);
    // chunk: a whole number of tiles, so only the last chunk is short
    const int tiles = (h->g.n + kGpTile - 1) / kGpTile;
    const int chunk = ((tiles + ns - 1) / ns) * kGpTile;
    const int nsplit = (h->g.n + chunk - 1) / chunk;
    const size_t need = (size_t)nsplit * count * sizeof(double2);
    if (need > h->part_bytes) {
        if (h->d_part) { cudaStreamSynchronize(h->stream); cudaFree(h->d_part); h->d_part = nullptr; h->part_bytes = 0; }
        cudaError_t e = cudaMalloc(&h->d_part, need);
        if (e != cudaSuccess) { h->d_part = nullptr; return e; }
        h->part_bytes = need;
    }
    dim3 grid(bx, nsplit);
    if (h->p.precision == PGB_MIXED) {
        k_gp32<<<grid, kGpBlock, 0, h->stream>>>(h->g, h->d_train32, d_pos, count, chunk,
                                                static_cast<float2*>(h->d_part));
        k_gp32_combine<<<bx, kGpBlock, 0, h->stream>>>(h->g, static_cast<const float2*>(h->d_part),
                                                      nsplit, count, d_out);
    } else {
        k_gp64<<<grid, kGpBlock, 0, h->stream>>>(h->g, h->d_train64, d_pos, count, chunk,
                                                static_cast<double*>(h->d_part));
        k_gp64_combine<<<bx, kGpBlock, 0, h->stream>>>(h->g, static_cast<const double*>(h->d_part),
                                                      nsplit, count, d_out);
    }
    return cudaGetLastError();
}

size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }
}  // namespace

extern "C" {

int pgb_gp_create(const pgb_gp_params* p, const double* training, int n, pgb_gp** out) {
    if (!out) return PGB_EINVAL;
    *out = nullptr;
    if (!p || !training || n <= 0) { g_gperr = "gp_create: parameters and training rows required"; return PGB_EINVAL; }
    // MaternKernel::selectKernel (gpkernel.cpp:71-89): nu = 1/2, 3/2 or 5/2
    int nu2 = 0;
    if (std::fabs(p->matern_nu - 0.5) < 1.0e-12) nu2 = 1;
    else if (std::fabs(p->matern_nu - 1.5) < 1.0e-12) nu2 = 3;
    else if (std::fabs(p->matern_nu - 2.5) < 1.0e-12) nu2 = 5;
    if (!nu2) { g_gperr = "gp_create: only nu = 1/2, 3/2 and 5/2 are supported"; return PGB_EINVAL; }
    if (p->precision != PGB_FP64 && p->precision != PGB_MIXED) { g_gperr = "gp_create: precision"; return PGB_EINVAL; }
    for (int d = 0; d < 3; ++d)
        if (!(p->ell[d] > 0.0) || p->norm_scale[d] == 0.0 || !(p->side[d] > 0.0)) {
            g_gperr = "gp_create: ell, norm_scale and side must be non-zero";
            return PGB_EINVAL;
        }
    int dev = 0;
    if (cudaGetDeviceCount(&dev) != cudaSuccess || dev == 0) {
        cudaGetLastError();
        g_gperr = "gp_create: no CUDA device";
        return PGB_ECUDA;
    }
    pgb_gp* h = new pgb_gp();
    h->p = *p;
    GpDev& g = h->g;
    for (int d = 0; d < 3; ++d) {
        g.off[d] = p->norm_offset[d];
        g.scale[d] = p->norm_scale[d];
        g.invell[d] = 1.0 / p->ell[d];
        g.pside[d] = p->periodic[d] ? p->side[d] : 0.0;
        g.sideInv[d] = 1.0 / p->side[d];
    }
    g.standard_mean = p->standard_mean; g.standard_std = p->standard_std;
    g.mu = p->mean; g.sigma2 = p->sigma2; g.nu2 = nu2; g.n = n;
    std::vector<double4> t64((size_t)n);
    std::vector<float4> t32((size_t)n);
    for (int k = 0; k < n; ++k) {
        const double* r = training + 4 * (size_t)k;
        t64[k] = make_double4(r[0], r[1], r[2], r[3]);
        t32[k] = make_float4((float)r[0], (float)r[1], (float)r[2], (float)r[3]);
    }
    cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&h->d_train64, t64.size() * sizeof(double4));
    if (e == cudaSuccess) e = cudaMalloc(&h->d_train32, t32.size() * sizeof(float4));
    if (e == cudaSuccess) e = cudaMemcpy(h->d_train64, t64.data(), t64.size() * sizeof(double4), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(h->d_train32, t32.data(), t32.size() * sizeof(float4), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        g_gperr = std::string("gp_create: ") + cudaGetErrorString(e);
        pgb_gp_destroy(h);
        return e == cudaErrorMemoryAllocation ? PGB_ENOMEM : PGB_ECUDA;
    }
    *out = h;
    return PGB_OK;
}

int pgb_gp_destroy(pgb_gp* h) {
    if (!h) return PGB_OK;
    if (h->stream) cudaStreamSynchronize(h->stream);
    cudaFree(h->d_train64); cudaFree(h->d_train32); cudaFree(h->d_buf); cudaFree(h->d_part);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return PGB_OK;
}

const char* pgb_gp_last_error(const pgb_gp* h) { return h ? h->err.c_str() : g_gperr.c_str(); }
void* pgb_gp_stream(pgb_gp* h) { return h ? (void*)h->stream : nullptr; }

int pgb_gp_eval_device_async(pgb_gp* h, const double* d_pos, double* d_values, int count) {
    if (!h || count < 0 || (count > 0 && (!d_pos || !d_values))) return PGB_EINVAL;
    cudaError_t e = launch_gp(h, d_pos, count, d_values);
    if (e != cudaSuccess) return h->cfail(e, "GP launch");
    return PGB_OK;
}

int pgb_gp_eval(pgb_gp* h, const double* pos, double* values, int count) {
    if (!h || count < 0 || (count > 0 && (!pos || !values))) return PGB_EINVAL;
    if (count == 0) return PGB_OK;
    const size_t pb = (size_t)count * 3 * sizeof(double), vb = (size_t)count * sizeof(double);
    int rc = ensure_buf(h, al256(pb) + vb); if (rc) return rc;
    char* base = static_cast<char*>(h->d_buf);
    double* d_pos = reinterpret_cast<double*>(base);
    double* d_val = reinterpret_cast<double*>(base + al256(pb));
    cudaError_t e = cudaMemcpyAsync(d_pos, pos, pb, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = launch_gp(h, d_pos, count, d_val);
    if (e == cudaSuccess) e = cudaMemcpyAsync(values, d_val, vb, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return h->cfail(e, "GP eval");
    return PGB_OK;
}

int pgb_gp_benzene_v(pgb_gp* h, const double* pos, double* values, int count) {
    if (!h || count < 0 || (count > 0 && (!pos || !values))) return PGB_EINVAL;
    if (count == 0) return PGB_OK;
    // GPHeBenzenePotential constants (include/potential.h:2433-2448)
    Benzene b{5.765366674e+00, 1.671477473e+01, 2.290626821e+05, 4.069217828e+06, 9.542607077e+07, 0.0,
              -4.775615288e+04, -1.263899296e+07, -2.959330054e+08, 0.0, 9.511488779e+05,
              2.551023972e+08, 0.0, 1.883887454e+08};
    const size_t pb = (size_t)count * 3 * sizeof(double), vb = (size_t)count * sizeof(double);
    const size_t o_fold = al256(pb), o_gp = o_fold + al256(pb), o_val = o_gp + al256(vb),
                 o_cut = o_val + al256(vb);
    int rc = ensure_buf(h, o_cut + (size_t)count); if (rc) return rc;
    char* base = static_cast<char*>(h->d_buf);
    double* d_pos = reinterpret_cast<double*>(base);
    double* d_fold = reinterpret_cast<double*>(base + o_fold);
    double* d_gp = reinterpret_cast<double*>(base + o_gp);
    double* d_val = reinterpret_cast<double*>(base + o_val);
    unsigned char* d_cut = reinterpret_cast<unsigned char*>(base + o_cut);
    const int blocks = (count + 255) / 256;
    cudaError_t e = cudaMemcpyAsync(d_pos, pos, pb, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) {
        k_benzene_fold<<<blocks, 256, 0, h->stream>>>(d_pos, count, d_fold, d_cut);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = launch_gp(h, d_fold, count, d_gp);
    if (e == cudaSuccess) {
        k_benzene_combine<<<blocks, 256, 0, h->stream>>>(b, d_fold, d_cut, d_gp, count, d_val);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(values, d_val, vb, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return h->cfail(e, "GP benzene");
    return PGB_OK;
}

}  // extern "C"
