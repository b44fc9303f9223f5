// isf_static.cu -- F(q,tau) for callers that must not allocate device memory.
//
// Some callers cannot call cudaMalloc at the point where they measure: an
// estimator hook that runs inside a host code's fixed memory budget (all
// device memory reserved up front by a pool the caller does not own), or
// code that is only allowed to launch work once its set-up phase is over.
// pgb_isf_static serves them: the caller passes device buffers for the
// worldlines, the q-vectors and the result, and the only scratch -- the
// collective densities rho_q(t) -- lives in the file-scope array below, which
// every GPU that loads this library holds until the process exits.
//
// The array is shared by every call on a device and keeps the last call's
// contents.  Nothing in it has to start at zero: the density kernel writes
// every rho_q(t) entry the correlation later reads.  Calls whose work
// overlaps on the GPU (two streams, two host threads) race on it, so callers
// must order their calls.
//
// The array's device address is looked up once per device (on the first
// call made with that device current) and cached for the life of the
// process.  A cudaDeviceReset, or any other teardown of the device's primary
// context, invalidates the cached address, so the entry point must not be
// called on a device after it has been reset.
#include <cstring>
#include <mutex>
#include <string>

#include "pgb_device.cuh"

namespace pgb {

// At most nq * M = 2^21 densities per call: 16 MiB per device.
constexpr long long kStaticRhoMax = 1LL << 21;
// The correlation keeps one q's M densities in shared memory (8 B each, at
// most 200 KB), and the density grid has one row of blocks per slice.
constexpr int kStaticMaxSlices = 25600;
static __device__ __align__(256) float2 g_static_rho[kStaticRhoMax];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
float2* g_rho_ptr[kMaxDevices] = {nullptr};

// Device address of the static array for the current device, looked up once
// per device with that device current (the first call on a device does it).
cudaError_t static_rho_address(float2** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_mutex);
    if (!g_rho_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_static_rho);
        if (e != cudaSuccess) return e;
        g_rho_ptr[dev] = static_cast<float2*>(p);
    }
    *out = g_rho_ptr[dev];
    return cudaSuccess;
}

// rho_q(t) from AoS FP64 beads [M][Ne][3] (the reference's bead array); the
// same arithmetic as k_rhoq32 in scatter.cu, reading AoS instead of SoA.
constexpr int kBlock = 256;

__global__ void __launch_bounds__(kBlock)
k_rhoq32_aos(const double* __restrict__ beads, int M, int N, int Ne, double3 side,
             double3 sideInv, const double* __restrict__ q, int nq, float2* __restrict__ rho) {
    extern __shared__ float4 su[];
    int4* si = reinterpret_cast<int4*>(su + N);
    const int t = blockIdx.y;
    const double* X = beads + (size_t)t * Ne * 3;
    for (int j = threadIdx.x; j < N; j += blockDim.x) {
        const double ux = X[3 * j] * sideInv.x, uy = X[3 * j + 1] * sideInv.y, uz = X[3 * j + 2] * sideInv.z;
        su[j] = make_float4((float)ux, (float)uy, (float)uz, 0.f);
        si[j] = make_int4(fixed_turns(ux), fixed_turns(uy), fixed_turns(uz), 0);
    }
    __syncthreads();
    const int iq = blockIdx.x * kBlock + threadIdx.x;
    if (iq >= nq) return;
    const double inv2pi = 0.15915494309189533577;
    const double dx = q[3 * iq] * side.x * inv2pi, dy = q[3 * iq + 1] * side.y * inv2pi,
                 dz = q[3 * iq + 2] * side.z * inv2pi;
    const double rx = rint(dx), ry = rint(dy), rz = rint(dz);
    const bool lattice = fabs(dx - rx) < 1e-6 && fabs(dy - ry) < 1e-6 && fabs(dz - rz) < 1e-6 &&
                         fabs(rx) < 1048576.0 && fabs(ry) < 1048576.0 && fabs(rz) < 1048576.0;
    rho[(size_t)iq * M + t] = lattice
        ? rho_partial_lattice(si, N, (int)rx, (int)ry, (int)rz)
        : rho_partial(su, N, (float)dx, (float)dy, (float)dz);
}

}  // namespace
}  // namespace pgb

extern "C" int pgb_isf_static(const double* d_beads, int num_slices, int num_ptcl,
                              int ptcl_extent, const double side[3], const double* d_qvecs,
                              int nq, double* d_isf, void* stream) {
    using namespace pgb;
    if (!d_beads || !side || !d_qvecs || !d_isf || num_slices < 2 || num_ptcl < 1 ||
        ptcl_extent < num_ptcl || nq < 1 || side[0] <= 0 || side[1] <= 0 || side[2] <= 0) {
        set_global_error("isf_static: bad arguments (device buffers, sizes and sides must be valid)");
        return PGB_EINVAL;
    }
    if ((long long)nq * num_slices > kStaticRhoMax) {
        set_global_error("isf_static: nq * num_slices = " + std::to_string((long long)nq * num_slices) +
                         " exceeds the static scratch limit of " + std::to_string(kStaticRhoMax) +
                         " densities (16 MiB); split the q-vectors over several calls");
        return PGB_EINVAL;
    }
    if (num_slices > kStaticMaxSlices) {
        set_global_error("isf_static: num_slices = " + std::to_string(num_slices) + " exceeds " +
                         std::to_string(kStaticMaxSlices) +
                         " (one q's densities must fit in 200 KB of shared memory)");
        return PGB_EINVAL;
    }
    if ((size_t)num_ptcl * (sizeof(float4) + sizeof(int4)) > 200 * 1024) {
        set_global_error("isf_static: num_ptcl = " + std::to_string(num_ptcl) +
                         " exceeds 6400 (one slice's beads must fit in 200 KB of shared memory)");
        return PGB_EINVAL;
    }
    float2* rho = nullptr;
    cudaError_t e = static_rho_address(&rho);
    if (e != cudaSuccess) {
        set_global_error(std::string("isf_static: cudaGetSymbolAddress failed: ") + cudaGetErrorString(e));
        return PGB_ECUDA;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    e = set_smem_limit(k_rhoq32_aos, 200 * 1024);
    if (e != cudaSuccess) {
        set_global_error(std::string("isf_static: cudaFuncSetAttribute failed: ") + cudaGetErrorString(e));
        return PGB_ECUDA;
    }
    dim3 grid((nq + kBlock - 1) / kBlock, num_slices);
    double3 sd = make_double3(side[0], side[1], side[2]);
    double3 si = make_double3(1.0 / side[0], 1.0 / side[1], 1.0 / side[2]);
    k_rhoq32_aos<<<grid, kBlock, (size_t)num_ptcl * (sizeof(float4) + sizeof(int4)), s>>>(
        d_beads, num_slices, num_ptcl, ptcl_extent, sd, si, d_qvecs, nq, rho);
    e = cudaGetLastError();
    if (e == cudaSuccess)
        e = launch_isf_direct32(rho, nq, num_slices, 1.0 / (1.0 * num_ptcl * num_slices), d_isf, s);
    if (e != cudaSuccess) {
        set_global_error(std::string("isf_static: launch failed: ") + cudaGetErrorString(e));
        return PGB_ECUDA;
    }
    return PGB_OK;
}
