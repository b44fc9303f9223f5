// walkers.cu -- many independent canonical walkers advanced in one kernel.
//
// One CTA owns one walker for the whole launch (a persistent CTA: it runs
// `sweeps` Monte Carlo steps back to back), so walkers never wait on each
// other and no inter-CTA synchronisation exists.  CTAs are issued in order of
// decreasing cost (N^2 M) so the largest chains start first.
//
// Moves follow the reference semantics (src/move.cpp):
//   * staging (StagingMove::attemptMove, move.cpp:1315-1412; positions from
//     MoveBase::newStagingPosition, move.cpp:263-292): a random particle, a
//     random start slice, stage length 2 + U{0..Mbar-2} (variable updates, the
//     reference default) and a single Metropolis test on the potential action
//     change of the moved beads;
//   * centre of mass (CenterOfMassMove::attemptMove, move.cpp:1124-1262): a
//     uniform shift of a whole closed worldline, comDelta = 0.04 lambda_dB.
// A step makes numUpdates = max(100, ceil(N M / Mbar)) moves (pimc.cpp:62-65)
// and then samples the thermodynamic energy (EnergyEstimator, primitive
// action, estimator.cpp:940-1029).
//
// Precision: pair potentials in FP32 (analytic Aziz), per-thread Kahan sums
// folded to FP64 across the CTA; the acceptance exp(-dU) test is FP64.
// Random numbers come from Philox4x32-10 keyed by (seed, walker).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "pgb_device.cuh"

namespace pgb {

constexpr int kMaxStage = 64;        // Mbar <= 64

struct WalkerMeta {
    int N, M, mbar, num_updates;
    long long off;                   // float4 offset of the walker's slab
    float L, Linv;
    float sig2lt;                    // sqrt(2 lambda tau)
    float com_delta;
    double tailV;                    // N^2/V * tailV(rc = L)
};

struct WalkerAcc {
    double esum, esumsq;
    long long samples, bead_updates;
    long long att[2], acc[2];
};

__device__ __forceinline__ uint4 wrand(uint64_t seed, int w, uint32_t c0, uint32_t c1,
                                       uint32_t c2, uint32_t c3) {
    uint2 key = make_uint2((uint32_t)seed ^ (uint32_t)w * 0x9E3779B9u,
                           (uint32_t)(seed >> 32) + (uint32_t)w);
    return philox4x32(make_uint4(c0, c1, c2, c3), key);
}

__device__ __forceinline__ float put_inside(float x, float L, float Linv) {
    return fmaf(-L, floorf(fmaf(x, Linv, 0.5f)), x);
}

// Thermodynamic energy per particle of one walker, all threads of the CTA.
__device__ double walker_energy(const WalkerMeta& m, const float4* __restrict__ P,
                                const AzizF& az, double tau, double lambda, double* red) {
    const int N = m.N, M = m.M;
    KahanF pot, kin;
    const int half = (N - 1) / 2;
    const bool even = (N % 2) == 0;
    for (int idx = threadIdx.x; idx < M * N; idx += blockDim.x) {
        int t = idx / N, i = idx - t * N;
        float4 ri = P[(size_t)t * N + i];
        // each unordered pair once: partners i+1..i+half (cyclic), plus i+N/2
        // for the first N/2 particles when N is even
        int cnt = half + ((even && i < N / 2) ? 1 : 0);
        for (int d = 1; d <= cnt; ++d) {
            int j = i + d; if (j >= N) j -= N;
            float4 rj = P[(size_t)t * N + j];
            float dx = min_image32(ri.x - rj.x, m.L, m.Linv);
            float dy = min_image32(ri.y - rj.y, m.L, m.Linv);
            float dz = min_image32(ri.z - rj.z, m.L, m.Linv);
            pot.add(aziz_v32(fmaf(dx, dx, fmaf(dy, dy, dz * dz)), az));
        }
        int tn = (t + 1 == M) ? 0 : t + 1;
        float4 rn = P[(size_t)tn * N + i];
        float vx = min_image32(rn.x - ri.x, m.L, m.Linv);
        float vy = min_image32(rn.y - ri.y, m.L, m.Linv);
        float vz = min_image32(rn.z - ri.z, m.L, m.Linv);
        kin.add(fmaf(vx, vx, fmaf(vy, vy, vz * vz)));
    }
    double V = block_sum(pot.value(), red);
    double K2 = block_sum(kin.value(), red);
    double totK = 1.5 * N / tau - K2 * ((0.25 / (lambda * tau)) / (tau * M));
    double totV = V / M + m.tailV;
    return (totK + totV) / N;
}

template <int TPW>
__global__ void __launch_bounds__(TPW)
k_walkers_run(const WalkerMeta* __restrict__ meta, const int* __restrict__ order,
              float4* __restrict__ pos, WalkerAcc* __restrict__ accs,
              unsigned long long* __restrict__ ctr, int sweeps, int measure, AzizF az,
              double tau, double lambda, float p_com, int var_updates, uint64_t seed) {
    __shared__ float4 s_new[kMaxStage];
    __shared__ float4 s_old[kMaxStage];
    __shared__ float s_z[kMaxStage][3];
    __shared__ double red[TPW / 32];
    __shared__ int s_acc;
    const int w = order[blockIdx.x];
    const WalkerMeta m = meta[w];
    float4* P = pos + m.off;
    const int N = m.N, M = m.M, tid = threadIdx.x;
    unsigned long long sweep0 = ctr[w];
    double esum = 0.0, esumsq = 0.0;
    long long nsamp = 0, nbu = 0, att0 = 0, att1 = 0, acc0 = 0, acc1 = 0;

    for (int sw = 0; sw < sweeps; ++sw) {
        const unsigned long long gs = sweep0 + sw;
        for (int u = 0; u < m.num_updates; ++u) {
            // every thread draws the same move description
            uint4 r0 = wrand(seed, w, (uint32_t)u, (uint32_t)gs, (uint32_t)(gs >> 32), 0u);
            const bool com = u01f(r0.x) < p_com;
            const int i = (int)(((unsigned long long)r0.z * (unsigned)N) >> 32);
            double dV;
            int nmove;
            if (!com) {
                const int s0 = (int)(((unsigned long long)r0.y * (unsigned)M) >> 32);
                const int len = var_updates
                    ? 2 + (int)(((unsigned long long)r0.w * (unsigned)(m.mbar - 1)) >> 32)
                    : m.mbar;
                nmove = len - 1;
                // normals for the stage: 3 per moved bead
                for (int k = tid; k < nmove; k += TPW) {
                    uint4 a = wrand(seed, w, (uint32_t)u, (uint32_t)gs, (uint32_t)(gs >> 32), 1u + k);
                    float2 z01 = box_muller(a.x, a.y);
                    float2 z2 = box_muller(a.z, a.w);
                    s_z[k][0] = z01.x; s_z[k][1] = z01.y; s_z[k][2] = z2.x;
                }
                for (int k = tid; k < nmove; k += TPW) {
                    int sl = s0 + 1 + k; if (sl >= M) sl -= M;
                    s_old[k] = P[(size_t)sl * N + i];
                }
                __syncthreads();
                if (tid < 3) {
                    // newStagingPosition (move.cpp:263-292), one dimension per thread
                    const float* e0 = reinterpret_cast<const float*>(&P[(size_t)s0 * N + i]);
                    int se = s0 + len; if (se >= M) se -= M;
                    const float* ee = reinterpret_cast<const float*>(&P[(size_t)se * N + i]);
                    float xp = e0[tid], xe = ee[tid];
                    for (int k = 0; k < nmove; ++k) {
                        float f1 = (float)(len - k - 1);
                        float f2 = 1.0f / (float)(len - k);
                        float sg = m.sig2lt * sqrtf(f1 * f2);
                        float mid = fmaf(min_image32(xe - xp, m.L, m.Linv), f2, xp);
                        float x = put_inside(fmaf(sg, s_z[k][tid], mid), m.L, m.Linv);
                        reinterpret_cast<float*>(&s_new[k])[tid] = x;
                        xp = x;
                    }
                }
                __syncthreads();
                KahanF acc;
                const int npairs = nmove * N;
                for (int idx = tid; idx < npairs; idx += TPW) {
                    int k = idx / N, j = idx - k * N;
                    if (j == i) continue;
                    int sl = s0 + 1 + k; if (sl >= M) sl -= M;
                    float4 pj = P[(size_t)sl * N + j];
                    float4 a = s_new[k], b = s_old[k];
                    float ax = min_image32(a.x - pj.x, m.L, m.Linv);
                    float ay = min_image32(a.y - pj.y, m.L, m.Linv);
                    float az_ = min_image32(a.z - pj.z, m.L, m.Linv);
                    float bx = min_image32(b.x - pj.x, m.L, m.Linv);
                    float by = min_image32(b.y - pj.y, m.L, m.Linv);
                    float bz = min_image32(b.z - pj.z, m.L, m.Linv);
                    float vn = aziz_v32(fmaf(ax, ax, fmaf(ay, ay, az_ * az_)), az);
                    float vo = aziz_v32(fmaf(bx, bx, fmaf(by, by, bz * bz)), az);
                    acc.add(vn - vo);
                }
                dV = block_sum(acc.value(), red);
                if (tid == 0) {
                    uint4 ra = wrand(seed, w, (uint32_t)u, (uint32_t)gs, (uint32_t)(gs >> 32), 0xFFFFu);
                    double x = u01d(ra.x, ra.y);
                    s_acc = (x < exp(-(tau * dV))) ? 1 : 0;
                }
                __syncthreads();
                const int ok = s_acc;
                if (ok)
                    for (int k = tid; k < nmove; k += TPW) {
                        int sl = s0 + 1 + k; if (sl >= M) sl -= M;
                        P[(size_t)sl * N + i] = s_new[k];
                    }
                att1 += 1; acc1 += ok;
                __syncthreads();
            } else {
                // centre-of-mass shift of the whole closed worldline of particle i
                nmove = M;
                const float sx = m.com_delta * (u01f(r0.y) - 0.5f);
                const float sy = m.com_delta * (u01f(r0.w) - 0.5f);
                uint4 r1 = wrand(seed, w, (uint32_t)u, (uint32_t)gs, (uint32_t)(gs >> 32), 0xFFFEu);
                const float sz = m.com_delta * (u01f(r1.x) - 0.5f);
                KahanF acc;
                const int npairs = M * N;
                for (int idx = tid; idx < npairs; idx += TPW) {
                    int t = idx / N, j = idx - t * N;
                    if (j == i) continue;
                    float4 pi = P[(size_t)t * N + i];
                    float4 pj = P[(size_t)t * N + j];
                    float bx = min_image32(pi.x - pj.x, m.L, m.Linv);
                    float by = min_image32(pi.y - pj.y, m.L, m.Linv);
                    float bz = min_image32(pi.z - pj.z, m.L, m.Linv);
                    float ax = min_image32(bx + sx, m.L, m.Linv);
                    float ay = min_image32(by + sy, m.L, m.Linv);
                    float az_ = min_image32(bz + sz, m.L, m.Linv);
                    float vn = aziz_v32(fmaf(ax, ax, fmaf(ay, ay, az_ * az_)), az);
                    float vo = aziz_v32(fmaf(bx, bx, fmaf(by, by, bz * bz)), az);
                    acc.add(vn - vo);
                }
                dV = block_sum(acc.value(), red);
                if (tid == 0) {
                    double x = u01d(r1.y, r1.z);
                    s_acc = (x < exp(-(tau * dV))) ? 1 : 0;
                }
                __syncthreads();
                const int ok = s_acc;
                if (ok)
                    for (int t = tid; t < M; t += TPW) {
                        float4 pi = P[(size_t)t * N + i];
                        pi.x = put_inside(pi.x + sx, m.L, m.Linv);
                        pi.y = put_inside(pi.y + sy, m.L, m.Linv);
                        pi.z = put_inside(pi.z + sz, m.L, m.Linv);
                        P[(size_t)t * N + i] = pi;
                    }
                att0 += 1; acc0 += ok;
                __syncthreads();
            }
            nbu += nmove;
        }
        if (measure > 0 && ((gs + 1) % (unsigned long long)measure) == 0) {
            double e = walker_energy(m, P, az, tau, lambda, red);
            esum += e; esumsq += e * e; nsamp += 1;
            __syncthreads();
        }
    }
    if (tid == 0) {
        WalkerAcc& A = accs[w];
        A.esum += esum; A.esumsq += esumsq; A.samples += nsamp; A.bead_updates += nbu;
        A.att[0] += att0; A.att[1] += att1; A.acc[0] += acc0; A.acc[1] += acc1;
        ctr[w] = sweep0 + sweeps;
    }
}

__global__ void k_walkers_init(const WalkerMeta* __restrict__ meta, float4* __restrict__ pos,
                               uint64_t seed) {
    const int w = blockIdx.x;
    const WalkerMeta m = meta[w];
    float4* P = pos + m.off;
    for (int i = threadIdx.x; i < m.N; i += blockDim.x) {
        uint4 a = wrand(seed, w, (uint32_t)i, 0u, 0u, 0xA0000000u);
        float cx = m.L * (u01f(a.x) - 0.5f), cy = m.L * (u01f(a.y) - 0.5f), cz = m.L * (u01f(a.z) - 0.5f);
        for (int t = 0; t < m.M; ++t) {
            uint4 b = wrand(seed, w, (uint32_t)i, (uint32_t)t, 0u, 0xB0000000u);
            float2 z01 = box_muller(b.x, b.y);
            float2 z2 = box_muller(b.z, b.w);
            P[(size_t)t * m.N + i] = make_float4(put_inside(fmaf(m.sig2lt, z01.x, cx), m.L, m.Linv),
                                                 put_inside(fmaf(m.sig2lt, z01.y, cy), m.L, m.Linv),
                                                 put_inside(fmaf(m.sig2lt, z2.x, cz), m.L, m.Linv), 0.f);
        }
    }
}

// Energy per particle of every walker (measurement only, no moves).
__global__ void k_walkers_energy32(const WalkerMeta* __restrict__ meta, const float4* __restrict__ pos,
                                   AzizF az, double tau, double lambda, double* __restrict__ out) {
    __shared__ double red[8];
    const int w = blockIdx.x;
    const WalkerMeta m = meta[w];
    double e = walker_energy(m, pos + m.off, az, tau, lambda, red);
    if (threadIdx.x == 0) out[w] = e;
}

// FP64 analytic Aziz (potential.cpp:1821-1838) for the plain-form comparison
__device__ double aziz_v64(double r, const AzizParams& a) {
    double x = r / a.rm;
    double Urep = a.A * exp(-a.alpha * x + a.beta * x * x);
    double ix2 = 1.0 / (x * x);
    double ix6 = ix2 * ix2 * ix2;
    double ix8 = ix6 * ix2;
    double ix10 = ix8 * ix2;
    double F = (x < a.D) ? exp(-(a.D / x - 1.0) * (a.D / x - 1.0)) : 1.0;
    return a.epsilon * (Urep - (a.C6 * ix6 + a.C8 * ix8 + a.C10 * ix10) * F);
}

__global__ void k_walkers_energy64(const WalkerMeta* __restrict__ meta, const float4* __restrict__ pos,
                                   AzizParams az, double tau, double lambda, double* __restrict__ out) {
    __shared__ double red[8];
    const int w = blockIdx.x;
    const WalkerMeta m = meta[w];
    const float4* P = pos + m.off;
    const int N = m.N, M = m.M;
    const double L = m.L, Li = 1.0 / L;
    double pot = 0.0, kin = 0.0;
    for (int idx = threadIdx.x; idx < M * N; idx += blockDim.x) {
        int t = idx / N, i = idx - t * N;
        float4 ri = P[(size_t)t * N + i];
        for (int j = i + 1; j < N; ++j) {
            float4 rj = P[(size_t)t * N + j];
            double dx = (double)ri.x - rj.x, dy = (double)ri.y - rj.y, dz = (double)ri.z - rj.z;
            dx -= L * floor(dx * Li + 0.5); dy -= L * floor(dy * Li + 0.5); dz -= L * floor(dz * Li + 0.5);
            pot += aziz_v64(sqrt(dx * dx + dy * dy + dz * dz), az);
        }
        int tn = (t + 1 == M) ? 0 : t + 1;
        float4 rn = P[(size_t)tn * N + i];
        double vx = (double)rn.x - ri.x, vy = (double)rn.y - ri.y, vz = (double)rn.z - ri.z;
        vx -= L * floor(vx * Li + 0.5); vy -= L * floor(vy * Li + 0.5); vz -= L * floor(vz * Li + 0.5);
        kin += vx * vx + vy * vy + vz * vz;
    }
    double V = block_sum(pot, red);
    double K2 = block_sum(kin, red);
    double totK = 1.5 * N / tau - K2 * ((0.25 / (lambda * tau)) / (tau * M));
    if (threadIdx.x == 0) out[w] = (totK + V / M + m.tailV) / N;
}

}  // namespace pgb

using namespace pgb;

struct pgb_walkers {
    int W = 0;
    std::vector<int> N, M, mbar;
    std::vector<double> T, L;
    double tau = 0, lambda = 0, p_com = 0;
    uint64_t seed = 0;
    int var_updates = 1, tpw = 0;
    AzizParams az{};
    std::vector<WalkerMeta> meta;
    std::vector<int> order;
    long long total_beads = 0;
    WalkerMeta* d_meta = nullptr;
    int* d_order = nullptr;
    float4* d_pos = nullptr;
    WalkerAcc* d_acc = nullptr;
    unsigned long long* d_ctr = nullptr;
    double* d_en = nullptr;
    double* d_stage = nullptr;
    cudaStream_t stream = nullptr;
    long long launches = 0;
    std::string err;
    int fail(int code, const std::string& m) { err = m; return code; }
    int cfail(cudaError_t e, const char* where) {
        err = std::string("CUDA error ") + cudaGetErrorString(e) + " at " + where;
        return e == cudaErrorMemoryAllocation ? PGB_ENOMEM : PGB_ECUDA;
    }
};

namespace {
thread_local std::string g_werr;

cudaError_t launch_run(pgb_walkers* h, int tpw, int sweeps, int measure) {
    AzizF af = make_aziz_f(h->az);
    switch (tpw) {
    case 64:
        k_walkers_run<64><<<h->W, 64, 0, h->stream>>>(h->d_meta, h->d_order, h->d_pos, h->d_acc, h->d_ctr,
            sweeps, measure, af, h->tau, h->lambda, (float)h->p_com, h->var_updates, h->seed);
        break;
    case 256:
        k_walkers_run<256><<<h->W, 256, 0, h->stream>>>(h->d_meta, h->d_order, h->d_pos, h->d_acc, h->d_ctr,
            sweeps, measure, af, h->tau, h->lambda, (float)h->p_com, h->var_updates, h->seed);
        break;
    default:
        k_walkers_run<128><<<h->W, 128, 0, h->stream>>>(h->d_meta, h->d_order, h->d_pos, h->d_acc, h->d_ctr,
            sweeps, measure, af, h->tau, h->lambda, (float)h->p_com, h->var_updates, h->seed);
        break;
    }
    h->launches += 1;
    return cudaGetLastError();
}

// Pick threads per walker by timing one sweep of each candidate on a copy of
// the state (positions, counters and accumulators are restored afterwards).
int autotune(pgb_walkers* h) {
    size_t pb = (size_t)h->total_beads * sizeof(float4);
    float4* save = nullptr;
    unsigned long long* save_ctr = nullptr;
    cudaError_t e = cudaMalloc(&save, pb);
    if (e != cudaSuccess) return h->cfail(e, "cudaMalloc(autotune)");
    e = cudaMalloc(&save_ctr, h->W * sizeof(unsigned long long));
    if (e != cudaSuccess) { cudaFree(save); return h->cfail(e, "cudaMalloc(autotune)"); }
    cudaMemcpyAsync(save, h->d_pos, pb, cudaMemcpyDeviceToDevice, h->stream);
    cudaMemcpyAsync(save_ctr, h->d_ctr, h->W * sizeof(unsigned long long), cudaMemcpyDeviceToDevice, h->stream);
    cudaEvent_t a, b;
    cudaEventCreate(&a); cudaEventCreate(&b);
    const int cand[3] = {64, 128, 256};
    float best = 1e30f; int best_t = 128;
    for (int c = 0; c < 3; ++c) {
        cudaMemcpyAsync(h->d_pos, save, pb, cudaMemcpyDeviceToDevice, h->stream);
        cudaMemcpyAsync(h->d_ctr, save_ctr, h->W * sizeof(unsigned long long), cudaMemcpyDeviceToDevice, h->stream);
        cudaEventRecord(a, h->stream);
        e = launch_run(h, cand[c], 1, 0);
        cudaEventRecord(b, h->stream);
        if (e == cudaSuccess) e = cudaEventSynchronize(b);
        if (e != cudaSuccess) break;
        float ms = 0; cudaEventElapsedTime(&ms, a, b);
        if (ms < best) { best = ms; best_t = cand[c]; }
    }
    cudaMemcpyAsync(h->d_pos, save, pb, cudaMemcpyDeviceToDevice, h->stream);
    cudaMemcpyAsync(h->d_ctr, save_ctr, h->W * sizeof(unsigned long long), cudaMemcpyDeviceToDevice, h->stream);
    cudaMemsetAsync(h->d_acc, 0, h->W * sizeof(WalkerAcc), h->stream);
    cudaError_t e2 = cudaStreamSynchronize(h->stream);
    cudaEventDestroy(a); cudaEventDestroy(b);
    cudaFree(save); cudaFree(save_ctr);
    if (e != cudaSuccess) return h->cfail(e, "autotune run");
    if (e2 != cudaSuccess) return h->cfail(e2, "autotune restore");
    h->tpw = best_t;
    return PGB_OK;
}
}  // namespace

extern "C" {

const char* pgb_walkers_last_error(const pgb_walkers* h) { return h ? h->err.c_str() : g_werr.c_str(); }

int pgb_walkers_create(const pgb_walkers_params* p, pgb_walkers** out) {
    if (!p || !out || p->num_walkers <= 0 || !p->num_ptcl || !p->num_slices || !p->temperature ||
        !p->side || !p->mbar || p->tau <= 0 || p->lambda <= 0) {
        g_werr = "walkers_create: bad arguments"; return PGB_EINVAL;
    }
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { g_werr = "no CUDA device available"; return PGB_ECUDA; }
    if (p->threads_per_walker != 0 && p->threads_per_walker != 64 && p->threads_per_walker != 128 &&
        p->threads_per_walker != 256) { g_werr = "threads_per_walker must be 0, 64, 128 or 256"; return PGB_EINVAL; }
    pgb_walkers* h = new pgb_walkers();
    h->W = p->num_walkers;
    h->tau = p->tau; h->lambda = p->lambda; h->p_com = p->p_com; h->seed = p->seed;
    h->var_updates = p->var_updates; h->tpw = p->threads_per_walker;
    h->az = aziz_params(p->aziz_year);
    long long off = 0;
    for (int w = 0; w < h->W; ++w) {
        int N = p->num_ptcl[w], M = p->num_slices[w], mb = p->mbar[w];
        double L = p->side[w], T = p->temperature[w];
        if (N < 2 || N > 4096 || M < 4 || M % 2 || mb < 2 || mb > kMaxStage || mb >= M || L <= 0 || T <= 0) {
            g_werr = "walker " + std::to_string(w) + ": need 2<=N<=4096, even M>=4, 2<=Mbar<=64, Mbar<M, L>0, T>0";
            delete h; return PGB_EINVAL;
        }
        h->N.push_back(N); h->M.push_back(M); h->mbar.push_back(mb); h->L.push_back(L); h->T.push_back(T);
        WalkerMeta m{};
        m.N = N; m.M = M; m.mbar = mb;
        int nu = (int)std::ceil(1.0 * N * M / (1.0 * mb));
        m.num_updates = nu < 100 ? 100 : nu;
        m.off = off;
        m.L = (float)L; m.Linv = (float)(1.0 / L);
        m.sig2lt = (float)std::sqrt(2.0 * p->lambda * p->tau);
        m.com_delta = (float)(0.04 * 2.0 * std::sqrt(M_PI * p->lambda / T));
        double rmorc = h->az.rm / L;
        double t2 = h->az.C6 * std::pow(rmorc, 3.0) / 3.0, t3 = h->az.C8 * std::pow(rmorc, 5.0) / 5.0,
               t4 = h->az.C10 * std::pow(rmorc, 7.0) / 7.0;
        double tailV = 2.0 * M_PI * h->az.epsilon * (-h->az.rm * h->az.rm * h->az.rm * (t2 + t3 + t4));
        m.tailV = (1.0 * N * N / (L * L * L)) * tailV;
        h->meta.push_back(m);
        off += (long long)N * M;
    }
    h->total_beads = off;
    h->order.resize(h->W);
    std::iota(h->order.begin(), h->order.end(), 0);
    std::stable_sort(h->order.begin(), h->order.end(), [&](int a, int b) {
        double ca = (double)h->N[a] * h->N[a] * h->M[a], cb = (double)h->N[b] * h->N[b] * h->M[b];
        return ca > cb;
    });
    cudaError_t e;
    do {
        if ((e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking)) != cudaSuccess) break;
        if ((e = cudaMalloc(&h->d_meta, h->W * sizeof(WalkerMeta))) != cudaSuccess) break;
        if ((e = cudaMalloc(&h->d_order, h->W * sizeof(int))) != cudaSuccess) break;
        if ((e = cudaMalloc(&h->d_pos, (size_t)off * sizeof(float4))) != cudaSuccess) break;
        if ((e = cudaMalloc(&h->d_acc, h->W * sizeof(WalkerAcc))) != cudaSuccess) break;
        if ((e = cudaMalloc(&h->d_ctr, h->W * sizeof(unsigned long long))) != cudaSuccess) break;
        if ((e = cudaMalloc(&h->d_en, h->W * sizeof(double))) != cudaSuccess) break;
        if ((e = cudaMemcpyAsync(h->d_meta, h->meta.data(), h->W * sizeof(WalkerMeta), cudaMemcpyHostToDevice, h->stream)) != cudaSuccess) break;
        if ((e = cudaMemcpyAsync(h->d_order, h->order.data(), h->W * sizeof(int), cudaMemcpyHostToDevice, h->stream)) != cudaSuccess) break;
        if ((e = cudaMemsetAsync(h->d_acc, 0, h->W * sizeof(WalkerAcc), h->stream)) != cudaSuccess) break;
        if ((e = cudaMemsetAsync(h->d_ctr, 0, h->W * sizeof(unsigned long long), h->stream)) != cudaSuccess) break;
        if ((e = cudaMemsetAsync(h->d_pos, 0, (size_t)off * sizeof(float4), h->stream)) != cudaSuccess) break;
        e = cudaStreamSynchronize(h->stream);
    } while (0);
    if (e != cudaSuccess) {
        g_werr = std::string("walkers_create: ") + cudaGetErrorString(e);
        int code = e == cudaErrorMemoryAllocation ? PGB_ENOMEM : PGB_ECUDA;
        pgb_walkers_destroy(h);
        return code;
    }
    *out = h;
    return PGB_OK;
}

int pgb_walkers_destroy(pgb_walkers* h) {
    if (!h) return PGB_OK;
    if (h->stream) cudaStreamSynchronize(h->stream);
    cudaFree(h->d_meta); cudaFree(h->d_order); cudaFree(h->d_pos); cudaFree(h->d_acc);
    cudaFree(h->d_ctr); cudaFree(h->d_en); cudaFree(h->d_stage);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return PGB_OK;
}

void* pgb_walkers_stream(pgb_walkers* h) { return h ? (void*)h->stream : nullptr; }
long long pgb_walkers_launch_count(pgb_walkers* h) { return h ? h->launches : 0; }
int pgb_walkers_threads(pgb_walkers* h) { return h ? h->tpw : 0; }

int pgb_walkers_init(pgb_walkers* h) {
    if (!h) return PGB_EINVAL;
    k_walkers_init<<<h->W, 128, 0, h->stream>>>(h->d_meta, h->d_pos, h->seed);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemsetAsync(h->d_ctr, 0, h->W * sizeof(unsigned long long), h->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(h->d_acc, 0, h->W * sizeof(WalkerAcc), h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return h->cfail(e, "walkers init");
    h->launches += 1;
    if (h->tpw == 0) return autotune(h);
    return PGB_OK;
}

int pgb_walkers_set_positions(pgb_walkers* h, int w, const double* pos) {
    if (!h || !pos || w < 0 || w >= h->W) return PGB_EINVAL;
    const WalkerMeta& m = h->meta[w];
    std::vector<float4> tmp((size_t)m.N * m.M);
    for (size_t i = 0; i < tmp.size(); ++i)
        tmp[i] = make_float4((float)pos[3*i], (float)pos[3*i+1], (float)pos[3*i+2], 0.f);
    cudaError_t e = cudaMemcpyAsync(h->d_pos + m.off, tmp.data(), tmp.size() * sizeof(float4),
                                    cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return h->cfail(e, "walkers set positions");
    return PGB_OK;
}

int pgb_walkers_get_positions(pgb_walkers* h, int w, double* pos) {
    if (!h || !pos || w < 0 || w >= h->W) return PGB_EINVAL;
    const WalkerMeta& m = h->meta[w];
    std::vector<float4> tmp((size_t)m.N * m.M);
    cudaError_t e = cudaMemcpyAsync(tmp.data(), h->d_pos + m.off, tmp.size() * sizeof(float4),
                                    cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return h->cfail(e, "walkers get positions");
    for (size_t i = 0; i < tmp.size(); ++i) { pos[3*i] = tmp[i].x; pos[3*i+1] = tmp[i].y; pos[3*i+2] = tmp[i].z; }
    return PGB_OK;
}

__global__ void k_walkers_from64(const double* __restrict__ src, float4* __restrict__ dst, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        dst[i] = make_float4((float)src[3 * i], (float)src[3 * i + 1], (float)src[3 * i + 2], 0.f);
}

size_t pgb_walkers_state_bytes(pgb_walkers* h) { return h ? (size_t)h->total_beads * 3 * sizeof(double) : 0; }

int pgb_walkers_set_all_positions(pgb_walkers* h, const double* pos) {
    if (!h || !pos) return PGB_EINVAL;
    size_t bytes = (size_t)h->total_beads * 3 * sizeof(double);
    if (!h->d_stage) {
        cudaError_t e = cudaMalloc(&h->d_stage, bytes);
        if (e != cudaSuccess) return h->cfail(e, "cudaMalloc(stage)");
    }
    cudaError_t e = cudaMemcpyAsync(h->d_stage, pos, bytes, cudaMemcpyHostToDevice, h->stream);
    if (e != cudaSuccess) return h->cfail(e, "walkers upload");
    int blocks = 152 * 8;
    k_walkers_from64<<<blocks, 256, 0, h->stream>>>(h->d_stage, h->d_pos, h->total_beads);
    e = cudaGetLastError();
    if (e != cudaSuccess) return h->cfail(e, "walkers upload convert");
    h->launches += 1;
    return PGB_OK;
}

int pgb_walkers_run_async(pgb_walkers* h, int sweeps, int measure) {
    if (!h || sweeps < 0 || measure < 0) return PGB_EINVAL;
    if (h->tpw == 0) h->tpw = 128;
    // bounded launches: at most 64 sweeps per kernel
    int left = sweeps;
    while (left > 0) {
        int chunk = left > 64 ? 64 : left;
        cudaError_t e = launch_run(h, h->tpw, chunk, measure);
        if (e != cudaSuccess) return h->cfail(e, "walkers run launch");
        left -= chunk;
    }
    return PGB_OK;
}

int pgb_walkers_sync(pgb_walkers* h) {
    if (!h) return PGB_EINVAL;
    cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return h->cfail(e, "walkers sync");
    return PGB_OK;
}

int pgb_walkers_stats(pgb_walkers* h, pgb_walker_stats* out) {
    if (!h || !out) return PGB_EINVAL;
    std::vector<WalkerAcc> a(h->W);
    cudaError_t e = cudaMemcpyAsync(a.data(), h->d_acc, h->W * sizeof(WalkerAcc), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return h->cfail(e, "walkers stats");
    for (int w = 0; w < h->W; ++w) {
        out[w].energy_sum = a[w].esum; out[w].energy_sumsq = a[w].esumsq;
        out[w].samples = a[w].samples; out[w].bead_updates = a[w].bead_updates;
        for (int k = 0; k < 2; ++k) { out[w].attempted[k] = a[w].att[k]; out[w].accepted[k] = a[w].acc[k]; }
    }
    return PGB_OK;
}

int pgb_walkers_reset_stats(pgb_walkers* h) {
    if (!h) return PGB_EINVAL;
    cudaError_t e = cudaMemsetAsync(h->d_acc, 0, h->W * sizeof(WalkerAcc), h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return h->cfail(e, "walkers reset stats");
    return PGB_OK;
}

int pgb_walkers_energy(pgb_walkers* h, int precision, double* out) {
    if (!h || !out) return PGB_EINVAL;
    if (precision == PGB_FP64)
        k_walkers_energy64<<<h->W, 256, 0, h->stream>>>(h->d_meta, h->d_pos, h->az, h->tau, h->lambda, h->d_en);
    else
        k_walkers_energy32<<<h->W, 256, 0, h->stream>>>(h->d_meta, h->d_pos, make_aziz_f(h->az), h->tau, h->lambda, h->d_en);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, h->d_en, h->W * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return h->cfail(e, "walkers energy");
    h->launches += 1;
    return PGB_OK;
}

}  // extern "C"
