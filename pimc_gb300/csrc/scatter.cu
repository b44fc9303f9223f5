// scatter.cu -- rho_q(t) in FP32 and the CUDA-core S(q) / F(q,tau) kernels.
//
// S(q) and F(q,tau) of the reference (estimator.cpp:3705-3737, 3923-3961 and
// gpu_ssf/gpu_isf, estimator_gpu.cu:67-165, 288-380) are pair sums over beads;
// both equal correlations of the collective density
//     rho_q(t) = sum_j exp(i q . r_j(t)):
//     S(q)     = 1/(N M) sum_t |rho_q(t)|^2
//     F(q,tau) = 1/(N M) sum_t Re[rho_q(t) conj(rho_q(t+tau))]
// which turns O(Q M N^2) (S) and O(Q M^2 N^2) (F) into O(Q M N) + O(Q M^2).
#include "pgb_device.cuh"

namespace pgb {

// One CTA = one slice t x 256 q-vectors; each thread owns one q and streams
// the slice's beads from shared memory (broadcast reads).  q . r / 2pi =
// sum_d n_d u_d with n_d = q_d L_d / 2pi and u_d = r_d / L_d.  Lattice q
// (integer n_d) use the fixed-point phase (rho_partial_lattice: three integer
// multiply-adds, no rounding); others the FP32 turn reduction (rho_partial).
// Either way __sincosf sees |angle| <= pi and the special-function pipe does
// only the sine and cosine.
constexpr int kRhoBlock = 256;

// The beads of every slice as fractions of the box, once per call: FP32
// turns for general q and 32-bit fixed-point turns for lattice q.  The FP64
// conversion runs here once per bead instead of once per (bead, q block).
__global__ void k_rho_positions(PathView v, float4* __restrict__ uf, int4* __restrict__ ui) {
    const size_t n = (size_t)v.M * v.Ne;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < n;
         idx += (size_t)gridDim.x * blockDim.x) {
        const size_t t = idx / v.Ne, j = idx - t * v.Ne;
        const double* X = v.pos + t * 3 * v.Ne;
        const double ux = X[j] * v.sideInv[0], uy = X[v.Ne + j] * v.sideInv[1],
                     uz = X[2 * v.Ne + j] * v.sideInv[2];
        uf[idx] = make_float4((float)ux, (float)uy, (float)uz, 0.f);
        ui[idx] = make_int4(fixed_turns(ux), fixed_turns(uy), fixed_turns(uz), 0);
    }
}

// The same conversion restricted to the beads inside a cylinder about the z
// axis, x^2 + y^2 < maxR^2 (include(), estimator.cpp:4309-4311), packed to
// the front of each slice in bead order so that the sums keep one order.
// One CTA per slice; cnt[t] receives the slice's count.
constexpr int kMaskBlock = 256;

__global__ void __launch_bounds__(kMaskBlock)
k_rho_positions_masked(PathView v, double maxR2, float4* __restrict__ uf, int4* __restrict__ ui,
                       int* __restrict__ cnt) {
    __shared__ int warp_base[kMaskBlock / 32 + 1];
    const int t = blockIdx.x;
    const int n = v.nbs[t];
    const double* X = v.pos + (size_t)t * 3 * v.Ne;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int base = 0;
    for (int j0 = 0; j0 < n; j0 += kMaskBlock) {
        const int j = j0 + threadIdx.x;
        bool in = false;
        double x = 0.0, y = 0.0, z = 0.0;
        if (j < n) {
            x = X[j]; y = X[v.Ne + j]; z = X[2 * v.Ne + j];
            in = __dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)) < maxR2;
        }
        const unsigned bal = __ballot_sync(0xffffffffu, in);
        if (lane == 0) warp_base[warp] = __popc(bal);
        __syncthreads();
        if (threadIdx.x == 0) {
            int s = 0;
            for (int w = 0; w < kMaskBlock / 32; ++w) { const int c = warp_base[w]; warp_base[w] = s; s += c; }
            warp_base[kMaskBlock / 32] = s;
        }
        __syncthreads();
        if (in) {
            const size_t o = (size_t)t * v.Ne + base + warp_base[warp] + __popc(bal & ((1u << lane) - 1u));
            const double ux = x * v.sideInv[0], uy = y * v.sideInv[1], uz = z * v.sideInv[2];
            uf[o] = make_float4((float)ux, (float)uy, (float)uz, 0.f);
            ui[o] = make_int4(fixed_turns(ux), fixed_turns(uy), fixed_turns(uz), 0);
        }
        base += warp_base[kMaskBlock / 32];
        __syncthreads();
    }
    if (threadIdx.x == 0) cnt[t] = base;
}

// Each wave vector in turns per box side, n_d = q_d L_d / 2 pi, once per call
// (not once per slice in every CTA): FP32 turns with a lattice flag in w, and
// the integers of lattice vectors (the reference's q lists of lattice type)
// for the exact fixed-point phase.
__global__ void k_rho_qsetup(PathView v, const double* __restrict__ q, int nq,
                             float4* __restrict__ qf, int4* __restrict__ qi) {
    const int iq = blockIdx.x * blockDim.x + threadIdx.x;
    if (iq >= nq) return;
    const double inv2pi = 0.15915494309189533577;
    const double dx = q[3*iq] * v.side[0] * inv2pi, dy = q[3*iq+1] * v.side[1] * inv2pi,
                 dz = q[3*iq+2] * v.side[2] * inv2pi;
    const double rx = rint(dx), ry = rint(dy), rz = rint(dz);
    const bool lattice = fabs(dx - rx) < 1e-6 && fabs(dy - ry) < 1e-6 && fabs(dz - rz) < 1e-6 &&
                         fabs(rx) < 1048576.0 && fabs(ry) < 1048576.0 && fabs(rz) < 1048576.0;
    qf[iq] = make_float4((float)dx, (float)dy, (float)dz, lattice ? 1.f : 0.f);
    qi[iq] = make_int4(lattice ? (int)rx : 0, lattice ? (int)ry : 0, lattice ? (int)rz : 0, 0);
}

__global__ void __launch_bounds__(kRhoBlock)
k_rhoq32(PathView v, const float4* __restrict__ uf, const int4* __restrict__ ui,
         const int* __restrict__ cnt, const float4* __restrict__ qf, const int4* __restrict__ qi,
         int nq, float2* __restrict__ rho) {
    extern __shared__ float4 su[];
    int4* si = reinterpret_cast<int4*>(su + v.Ne);
    const int t = blockIdx.y;
    const int n = cnt ? cnt[t] : v.nbs[t];
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        su[j] = uf[(size_t)t * v.Ne + j];
        si[j] = ui[(size_t)t * v.Ne + j];
    }
    __syncthreads();
    const int iq = blockIdx.x * kRhoBlock + threadIdx.x;
    if (iq >= nq) return;
    // lattice wave vectors take the exact fixed-point phase, any other q the
    // FP32 turn reduction
    const float4 f = qf[iq];
    if (f.w != 0.f) {
        const int4 k = qi[iq];
        rho[(size_t)iq * v.M + t] = rho_partial_lattice(si, n, k.x, k.y, k.z);
    } else {
        rho[(size_t)iq * v.M + t] = rho_partial(su, n, f.x, f.y, f.z);
    }
}

size_t rhoq32_work_bytes(const PathView& v) {
    return (size_t)v.M * v.Ne * (sizeof(float4) + sizeof(int4)) + (size_t)v.M * sizeof(int);
}

cudaError_t launch_rhoq32(const PathView& v, const double* d_q, int nq, float2* d_rho,
                          void* d_work, cudaStream_t s, double maxR2) {
    if (nq <= 0) return cudaSuccess;
    float4* uf = static_cast<float4*>(d_work);
    int4* ui = reinterpret_cast<int4*>(uf + (size_t)v.M * v.Ne);
    int* cnt = nullptr;
    if (maxR2 > 0.0) {
        cnt = reinterpret_cast<int*>(ui + (size_t)v.M * v.Ne);
        k_rho_positions_masked<<<v.M, kMaskBlock, 0, s>>>(v, maxR2, uf, ui, cnt);
    } else {
        const size_t nb = (size_t)v.M * v.Ne;
        const int blocks = (int)std::min<size_t>((nb + 255) / 256, 152 * 16);
        k_rho_positions<<<blocks, 256, 0, s>>>(v, uf, ui);
    }
    dim3 grid((nq + kRhoBlock - 1) / kRhoBlock, v.M);
    size_t smem = (size_t)v.Ne * (sizeof(float4) + sizeof(int4));
    if (smem > 200 * 1024) return cudaErrorInvalidValue;   // one slice must fit in shared memory
    {
        const cudaError_t ae = set_smem_limit(k_rhoq32, 200 * 1024);
        if (ae != cudaSuccess) return ae;
    }
    // the wave-vector table sits in the unused half of the rho region, which
    // is sized for FP64 values (16 B per (q, slice)); M is even, so it starts
    // 16-byte aligned
    float4* qf = reinterpret_cast<float4*>(d_rho + (size_t)nq * v.M);
    int4* qi = reinterpret_cast<int4*>(qf + nq);
    k_rho_qsetup<<<(nq + 255) / 256, 256, 0, s>>>(v, d_q, nq, qf, qi);
    k_rhoq32<<<grid, kRhoBlock, smem, s>>>(v, uf, ui, cnt, qf, qi, nq, d_rho);
    return cudaGetLastError();
}

__global__ void k_ssf_from_rho32(const float2* __restrict__ rho, int nq, int M, double norm,
                                 double* __restrict__ out) {
    __shared__ double red[8];
    int iq = blockIdx.x;
    double acc = 0.0;
    for (int t = threadIdx.x; t < M; t += blockDim.x) {
        float2 r = rho[(size_t)iq * M + t];
        acc += (double)r.x * r.x + (double)r.y * r.y;
    }
    double s = block_sum(acc, red);
    if (threadIdx.x == 0) out[iq] = s * norm;
}

cudaError_t launch_ssf_from_rho32(const float2* d_rho, int nq, int M, double norm,
                                  double* d_out, cudaStream_t s) {
    if (nq <= 0) return cudaSuccess;
    k_ssf_from_rho32<<<nq, 256, 0, s>>>(d_rho, nq, M, norm, d_out);
    return cudaGetLastError();
}

// CUDA-core circular correlation: one CTA per q, rho_q staged in shared
// memory, each thread owns kTauPerThread consecutive tau and slides a
// register window along t (one new shared load per kTauPerThread FMAs pairs).
constexpr int kTauPerThread = 8;

__global__ void k_isf_direct32(const float2* __restrict__ rho, int nq, int M, double norm,
                               double* __restrict__ out) {
    extern __shared__ float2 sr[];
    const int iq = blockIdx.x;
    const int nt = M / 2 + 1;
    for (int t = threadIdx.x; t < M; t += blockDim.x) sr[t] = rho[(size_t)iq * M + t];
    __syncthreads();
    for (int tau0 = threadIdx.x * kTauPerThread; tau0 < nt; tau0 += blockDim.x * kTauPerThread) {
        double acc[kTauPerThread];
        float win_r[kTauPerThread], win_i[kTauPerThread];
        #pragma unroll
        for (int k = 0; k < kTauPerThread; ++k) {
            acc[k] = 0.0;
            int t2 = (tau0 + k) % M;
            win_r[k] = sr[t2].x; win_i[k] = sr[t2].y;
        }
        int t = 0;
        while (t < M) {
            float c[kTauPerThread];
            #pragma unroll
            for (int k = 0; k < kTauPerThread; ++k) c[k] = 0.f;
            int tend = min(M, t + 64);
            for (; t < tend; ++t) {
                float2 a = sr[t];
                #pragma unroll
                for (int k = 0; k < kTauPerThread; ++k) c[k] = fmaf(a.x, win_r[k], fmaf(a.y, win_i[k], c[k]));
                #pragma unroll
                for (int k = 0; k < kTauPerThread - 1; ++k) { win_r[k] = win_r[k+1]; win_i[k] = win_i[k+1]; }
                int tn = (t + 1 + tau0 + kTauPerThread - 1) % M;
                win_r[kTauPerThread - 1] = sr[tn].x; win_i[kTauPerThread - 1] = sr[tn].y;
            }
            #pragma unroll
            for (int k = 0; k < kTauPerThread; ++k) acc[k] += c[k];
        }
        #pragma unroll
        for (int k = 0; k < kTauPerThread; ++k)
            if (tau0 + k < nt) out[(size_t)iq * nt + tau0 + k] = acc[k] * norm;
    }
}

cudaError_t launch_isf_direct32(const float2* d_rho, int nq, int M, double norm, double* d_out,
                                cudaStream_t s) {
    if (nq <= 0) return cudaSuccess;
    int nt = M / 2 + 1;
    int threads = (nt + kTauPerThread - 1) / kTauPerThread;
    threads = ((threads + 31) / 32) * 32;
    if (threads > 256) threads = 256;
    const size_t smem = (size_t)M * sizeof(float2);
    if (smem > 200 * 1024) return cudaErrorInvalidValue;    // one q's densities in shared memory
    if (smem > 48 * 1024) {
        const cudaError_t ae = set_smem_limit(k_isf_direct32, 200 * 1024);
        if (ae != cudaSuccess) return ae;
    }
    k_isf_direct32<<<nq, threads, smem, s>>>(d_rho, nq, M, norm, d_out);
    return cudaGetLastError();
}

}  // namespace pgb
