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
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <map>
#include <numeric>
#include <string>
#include <vector>

#include "pgb_device.cuh"

namespace pgb {

constexpr int kMaxStage = 64;        // Mbar <= 64

struct WalkerMeta {
    int N, M, mbar, num_updates;
    long long off;                   // float4 offset of the walker's slab
    unsigned long long key;          // Philox key of the walker's streams
    int max_sweeps;                  // sweeps this walker may still make (per launch cap)
    int pad_;
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

// Streams are keyed per walker (WalkerMeta::key), so a walker's trajectory
// does not depend on its slot or on the other walkers in the launch.
__device__ __forceinline__ uint4 wrand(unsigned long long key, uint32_t c0, uint32_t c1,
                                       uint32_t c2, uint32_t c3) {
    return philox4x32(make_uint4(c0, c1, c2, c3), make_uint2((uint32_t)key, (uint32_t)(key >> 32)));
}

inline unsigned long long walker_key(uint64_t seed, int w) {
    return (((unsigned long long)((uint32_t)(seed >> 32) + (uint32_t)w)) << 32) |
           (unsigned long long)((uint32_t)seed ^ ((uint32_t)w * 0x9E3779B9u));
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

    for (int sw = 0; sw < min(sweeps, m.max_sweeps); ++sw) {
        const unsigned long long gs = sweep0 + sw;
        for (int u = 0; u < m.num_updates; ++u) {
            // every thread draws the same move description
            uint4 r0 = wrand(m.key, (uint32_t)u, (uint32_t)gs, (uint32_t)(gs >> 32), 0u);
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
                    uint4 a = wrand(m.key, (uint32_t)u, (uint32_t)gs, (uint32_t)(gs >> 32), 1u + k);
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
                    uint4 ra = wrand(m.key, (uint32_t)u, (uint32_t)gs, (uint32_t)(gs >> 32), 0xFFFFu);
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
                uint4 r1 = wrand(m.key, (uint32_t)u, (uint32_t)gs, (uint32_t)(gs >> 32), 0xFFFEu);
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
        ctr[w] = sweep0 + min(sweeps, m.max_sweeps);
    }
}

// ---------------------------------------------------------------------------
// Packed-team schedule.  Each walker gets a team of 1, 2, 4 or 8 warps, sized
// to its per-move pair count (about 2 N Mbar/2 pairs), and up to 8 warps of
// teams share one 256-thread CTA.  A team synchronises on its own named
// barrier (bar.sync id, count) -- or __syncwarp for one-warp teams -- so small
// walkers never wait on large ones.  The staging path is drawn as a Brownian
// bridge built by one warp with shuffle scans (the same free-particle
// distribution as the sequential staging construction, move.cpp:263-292).
// ---------------------------------------------------------------------------
// Metropolis test of the FP64 log acceptance ratio a = -tau dV against a
// uniform x in [0,1): accept when a >= 0 or x < exp(a).  An FP32 screen on
// a - log(x) decides every case farther than 1e-3 from the boundary (the
// screen's own error is at most about 1e-5 there, as |a| <= 37), and
// the exact FP64 comparison decides the rest, so the outcome is that of the
// FP64 test.
__device__ __forceinline__ bool metropolis(double dV, double tau, uint32_t hi, uint32_t lo) {
    const double x = u01d(hi, lo);
    const double a = -(tau * dV);
    if (a >= 0.0) return true;
    if (x > 0.0) {
        // FP32 screen; exact FP64 test only near the boundary
        const float d = (float)a - __logf((float)x);
        if (d > 1e-3f) return true;
        if (d < -1e-3f) return false;
    }
    return x < exp(a);
}

// The same test split in two so that the part that depends only on the
// draw (x and an FP32 log x) runs before the pair sums end.  The screen then
// takes the team total as its (hi, lo) FP32 pair: a32 = -tau (hi + lo) is
// within about 1e-5 of a wherever |a| <= 37, far inside the 1e-3 band; the
// band and x = 0 go to the exact FP64 comparison, so the outcome equals
// metropolis() on dV = (double)hi + (double)lo.
struct MetroDraw {
    double x;
    float lx;
};

__device__ __forceinline__ MetroDraw metropolis_draw(uint32_t hi, uint32_t lo) {
    MetroDraw d;
    d.x = u01d(hi, lo);
    d.lx = (d.x > 0.0) ? __logf((float)d.x) : 0.f;
    return d;
}

__device__ __forceinline__ bool metropolis_ff(float hi, float lo, double tau, float tauf,
                                              const MetroDraw& d) {
    if (d.x > 0.0) {
        const float diff = -(tauf * (hi + lo)) - d.lx;
        if (diff > 1e-3f) return true;
        if (diff < -1e-3f) return false;
    }
    const double a = -(tau * ((double)hi + (double)lo));
    return a >= 0.0 || d.x < exp(a);
}

constexpr int kTeamCta = 256;

__device__ __forceinline__ void team_sync(int slot, int nthreads) {
    if (nthreads == 32) __syncwarp();
    else asm volatile("bar.sync %0, %1;" :: "r"(slot + 1), "r"(nthreads) : "memory");
}

__device__ __forceinline__ float warp_scan_incl(float x, int lane) {
    #pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        float y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    return x;
}

template <int MINB>
__global__ void __launch_bounds__(kTeamCta, MINB)
k_walkers_team(const WalkerMeta* __restrict__ meta, const int4* __restrict__ teams,
               float4* __restrict__ pos, WalkerAcc* __restrict__ accs,
               unsigned long long* __restrict__ ctr, int sweeps, int measure, AzizF az,
               double tau, double lambda, float p_com, int var_updates, uint64_t seed,
               unsigned long long budget_ns, int* __restrict__ upos) {
    __shared__ float4 s_new[8][2][kMaxStage];
    __shared__ float4 s_old[8][2][kMaxStage];
    __shared__ double s_red[8][8];
    __shared__ int s_acc[8];
    __shared__ int s_stop[8];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int4 tm = make_int4(-1, 0, 0, 0);
    #pragma unroll
    for (int k = 0; k < 8; ++k) {
        int4 t = teams[blockIdx.x * 8 + k];
        if (t.w && warp >= t.y && warp < t.y + t.z) tm = t;
    }
    if (tm.x < 0) return;                       // warp not in any team
    const int w = tm.x, slot = tm.y, nw = tm.z, T = nw * 32;
    const int tt = threadIdx.x - slot * 32;     // thread index in the team
    const int wi = warp - slot;                 // warp index in the team
    const WalkerMeta m = meta[w];
    float4* P = pos + m.off;
    const int N = m.N, M = m.M;
    double* red = s_red[slot];
    const unsigned long long sweep0 = ctr[w];
    double esum = 0.0, esumsq = 0.0;
    long long nsamp = 0, nbu = 0, att0 = 0, att1 = 0, acc0 = 0, acc1 = 0;
    int buf = 0;
    // pair-loop mapping: G threads per partner j when the team has at least N
    // threads (thread tt -> j = tt % N, moved beads k = tt / N, +G, ...), else
    // one thread per partner and a loop over partners
    const int G = (T >= N) ? T / N : 1;
    const int j0 = (T >= N) ? ((tt < G * N) ? tt % N : N) : tt;
    const int kb0 = (T >= N) ? tt / N : 0;
    const int jstep = (T >= N) ? N : T;
    // Resumable rounds (upos != null): the walker continues from move upos[w]
    // of sweep ctr[w], and with budget_ns > 0 the team stops after the first
    // move that ends later than budget_ns after the team started.  Draws are
    // indexed by (sweep, move), so a chain is the same however its moves are
    // split over launches, and each energy sample is added to the
    // accumulator in sample order.
    const unsigned long long t_start = (tt == 0 && budget_ns) ? gtimer_ns() : 0ull;
    const int nsw = min(sweeps, m.max_sweeps);
    int u = upos ? upos[w] : 0;
    int sw = 0;
    while (sw < nsw) {
        const unsigned long long gs = sweep0 + sw;
        const uint32_t g0 = (uint32_t)gs, g1 = (uint32_t)(gs >> 32);
        int stop = 0;
        for (; u < m.num_updates; ++u) {
            uint4 r0 = wrand(m.key, (uint32_t)u, g0, g1, 0u);
            const bool com = u01f(r0.x) < p_com;
            const int i = (int)(((unsigned long long)r0.z * (unsigned)N) >> 32);
            if (!com) {
                const int s0 = (int)(((unsigned long long)r0.y * (unsigned)M) >> 32);
                const int len = var_updates
                    ? 2 + (int)(((unsigned long long)r0.w * (unsigned)(m.mbar - 1)) >> 32)
                    : m.mbar;
                const int nmove = len - 1;
                float4* sn = s_new[slot][buf];
                float4* so = s_old[slot][buf];
                if (wi == 0) {
                    // Brownian bridge between the fixed beads at s0 and s0+len:
                    // W_j = sum_{i<=j} sigma z_i, x_j = x0 + (j/len)(xe - x0) + W_j - (j/len) W_len
                    int se = s0 + len; if (se >= M) se -= M;
                    const float4 x0 = P[(size_t)s0 * N + i], xe = P[(size_t)se * N + i];
                    float4 ob0 = make_float4(0, 0, 0, 0), ob1 = ob0;
                    {
                        int sl = s0 + 1 + lane; if (sl >= M) sl -= M;
                        if (lane < nmove) ob0 = P[(size_t)sl * N + i];
                        sl = s0 + 33 + lane; if (sl >= M) sl -= M;
                        if (lane + 32 < nmove) ob1 = P[(size_t)sl * N + i];
                    }
                    float a1x = 0.f, a1y = 0.f, a1z = 0.f, a2x = 0.f, a2y = 0.f, a2z = 0.f;
                    const int j1 = lane + 1, j2 = lane + 33;
                    if (j1 <= len) {
                        uint4 a = wrand(m.key, (uint32_t)u, g0, g1, (uint32_t)j1);
                        float2 z01 = box_muller(a.x, a.y), z2 = box_muller(a.z, a.w);
                        a1x = m.sig2lt * z01.x; a1y = m.sig2lt * z01.y; a1z = m.sig2lt * z2.x;
                    }
                    if (j2 <= len) {
                        uint4 a = wrand(m.key, (uint32_t)u, g0, g1, (uint32_t)j2);
                        float2 z01 = box_muller(a.x, a.y), z2 = box_muller(a.z, a.w);
                        a2x = m.sig2lt * z01.x; a2y = m.sig2lt * z01.y; a2z = m.sig2lt * z2.x;
                    }
                    float W1x = warp_scan_incl(a1x, lane), W1y = warp_scan_incl(a1y, lane),
                          W1z = warp_scan_incl(a1z, lane);
                    float W2x = warp_scan_incl(a2x, lane) + __shfl_sync(0xffffffffu, W1x, 31);
                    float W2y = warp_scan_incl(a2y, lane) + __shfl_sync(0xffffffffu, W1y, 31);
                    float W2z = warp_scan_incl(a2z, lane) + __shfl_sync(0xffffffffu, W1z, 31);
                    const int src = (len <= 32) ? len - 1 : len - 33;
                    float Lx = __shfl_sync(0xffffffffu, len <= 32 ? W1x : W2x, src);
                    float Ly = __shfl_sync(0xffffffffu, len <= 32 ? W1y : W2y, src);
                    float Lz = __shfl_sync(0xffffffffu, len <= 32 ? W1z : W2z, src);
                    const float dx = min_image32(xe.x - x0.x, m.L, m.Linv);
                    const float dy = min_image32(xe.y - x0.y, m.L, m.Linv);
                    const float dz = min_image32(xe.z - x0.z, m.L, m.Linv);
                    const float il = 1.0f / (float)len;
                    #pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const int k = lane + 32 * h;            // bead k <-> j = k + 1
                        if (k < nmove) {
                            const float f = (float)(k + 1) * il;
                            const float Wx = h ? W2x : W1x, Wy = h ? W2y : W1y, Wz = h ? W2z : W1z;
                            so[k] = h ? ob1 : ob0;
                            sn[k] = make_float4(put_inside(x0.x + fmaf(f, dx - Lx, Wx), m.L, m.Linv),
                                                put_inside(x0.y + fmaf(f, dy - Ly, Wy), m.L, m.Linv),
                                                put_inside(x0.z + fmaf(f, dz - Lz, Wz), m.L, m.Linv), 0.f);
                        }
                    }
                }
                team_sync(slot, T);
                KahanF acc;
                // thread <-> partner j (G threads per partner share the moved beads)
                for (int j = j0; j < N; j += jstep) {
                    if (j == i) continue;
                    #pragma unroll 4
                    for (int k = kb0; k < nmove; k += G) {
                        int sl = s0 + 1 + k; if (sl >= M) sl -= M;
                        const float4 pj = P[(size_t)sl * N + j];
                        const float4 a = sn[k], b = so[k];
                        const float ax = min_image32(a.x - pj.x, m.L, m.Linv);
                        const float ay = min_image32(a.y - pj.y, m.L, m.Linv);
                        const float az_ = min_image32(a.z - pj.z, m.L, m.Linv);
                        const float bx = min_image32(b.x - pj.x, m.L, m.Linv);
                        const float by = min_image32(b.y - pj.y, m.L, m.Linv);
                        const float bz = min_image32(b.z - pj.z, m.L, m.Linv);
                        const float vn = aziz_v32(fmaf(ax, ax, fmaf(ay, ay, az_ * az_)), az);
                        const float vo = aziz_v32(fmaf(bx, bx, fmaf(by, by, bz * bz)), az);
                        acc.add(vn - vo);
                    }
                }
                double part = warp_sum_ff(acc);
                if (lane == 0) red[wi] = part;
                team_sync(slot, T);
                if (tt == 0) {
                    double dV = 0.0;
                    for (int q = 0; q < nw; ++q) dV += red[q];
                    uint4 ra = wrand(m.key, (uint32_t)u, g0, g1, 0xFFFFu);
                    s_acc[slot] = metropolis(dV, tau, ra.x, ra.y) ? 1 : 0;
                    s_stop[slot] = (budget_ns && gtimer_ns() - t_start > budget_ns) ? 1 : 0;
                }
                team_sync(slot, T);
                const int ok = s_acc[slot];
                stop = s_stop[slot];
                if (wi == 0 && ok) {
                    for (int k2 = lane; k2 < nmove; k2 += 32) {
                        int sl = s0 + 1 + k2; if (sl >= M) sl -= M;
                        P[(size_t)sl * N + i] = sn[k2];
                    }
                    __syncwarp();
                }
                att1 += 1; acc1 += ok; nbu += nmove;
                buf ^= 1;
            } else {
                const float sx = m.com_delta * (u01f(r0.y) - 0.5f);
                const float sy = m.com_delta * (u01f(r0.w) - 0.5f);
                const uint4 r1 = wrand(m.key, (uint32_t)u, g0, g1, 0xFFFEu);
                const float sz = m.com_delta * (u01f(r1.x) - 0.5f);
                KahanF acc;
                for (int j = j0; j < N; j += jstep) {
                    if (j == i) continue;
                    #pragma unroll 4
                    for (int t = kb0; t < M; t += G) {
                        const float4 pi = P[(size_t)t * N + i];
                        const float4 pj = P[(size_t)t * N + j];
                        const float bx = min_image32(pi.x - pj.x, m.L, m.Linv);
                        const float by = min_image32(pi.y - pj.y, m.L, m.Linv);
                        const float bz = min_image32(pi.z - pj.z, m.L, m.Linv);
                        const float ax = min_image32(bx + sx, m.L, m.Linv);
                        const float ay = min_image32(by + sy, m.L, m.Linv);
                        const float az_ = min_image32(bz + sz, m.L, m.Linv);
                        const float vn = aziz_v32(fmaf(ax, ax, fmaf(ay, ay, az_ * az_)), az);
                        const float vo = aziz_v32(fmaf(bx, bx, fmaf(by, by, bz * bz)), az);
                        acc.add(vn - vo);
                    }
                }
                double part = warp_sum_ff(acc);
                if (lane == 0) red[wi] = part;
                team_sync(slot, T);
                if (tt == 0) {
                    double dV = 0.0;
                    for (int q = 0; q < nw; ++q) dV += red[q];
                    s_acc[slot] = metropolis(dV, tau, r1.y, r1.z) ? 1 : 0;
                    s_stop[slot] = (budget_ns && gtimer_ns() - t_start > budget_ns) ? 1 : 0;
                }
                team_sync(slot, T);
                const int ok = s_acc[slot];
                stop = s_stop[slot];
                if (ok)
                    for (int t2 = tt; t2 < M; t2 += T) {
                        float4 pi = P[(size_t)t2 * N + i];
                        pi.x = put_inside(pi.x + sx, m.L, m.Linv);
                        pi.y = put_inside(pi.y + sy, m.L, m.Linv);
                        pi.z = put_inside(pi.z + sz, m.L, m.Linv);
                        P[(size_t)t2 * N + i] = pi;
                    }
                team_sync(slot, T);
                att0 += 1; acc0 += ok; nbu += M;
            }
            if (stop) { ++u; break; }
        }
        if (u < m.num_updates) break;               // stopped inside the sweep
        if (measure > 0 && ((gs + 1) % (unsigned long long)measure) == 0) {
            team_sync(slot, T);
            KahanF pot, kin;
            const int half = (N - 1) / 2;
            const bool even = (N % 2) == 0;
            for (int idx = tt; idx < M * N; idx += T) {
                const int t = idx / N, ii = idx - t * N;
                const float4 ri = P[(size_t)t * N + ii];
                const int cnt = half + ((even && ii < N / 2) ? 1 : 0);
                for (int d = 1; d <= cnt; ++d) {
                    int jj = ii + d; if (jj >= N) jj -= N;
                    const float4 rj = P[(size_t)t * N + jj];
                    const float dx = min_image32(ri.x - rj.x, m.L, m.Linv);
                    const float dy = min_image32(ri.y - rj.y, m.L, m.Linv);
                    const float dz = min_image32(ri.z - rj.z, m.L, m.Linv);
                    pot.add(aziz_v32(fmaf(dx, dx, fmaf(dy, dy, dz * dz)), az));
                }
                const int tn = (t + 1 == M) ? 0 : t + 1;
                const float4 rn = P[(size_t)tn * N + ii];
                const float vx = min_image32(rn.x - ri.x, m.L, m.Linv);
                const float vy = min_image32(rn.y - ri.y, m.L, m.Linv);
                const float vz = min_image32(rn.z - ri.z, m.L, m.Linv);
                kin.add(fmaf(vx, vx, fmaf(vy, vy, vz * vz)));
            }
            double pv = warp_sum(pot.value()), kv = warp_sum(kin.value());
            if (lane == 0) { red[wi] = pv; }
            team_sync(slot, T);
            double V = 0.0;
            if (tt == 0) for (int q = 0; q < nw; ++q) V += red[q];
            team_sync(slot, T);
            if (lane == 0) red[wi] = kv;
            team_sync(slot, T);
            if (tt == 0) {
                double K2 = 0.0;
                for (int q = 0; q < nw; ++q) K2 += red[q];
                const double totK = 1.5 * N / tau - K2 * ((0.25 / (lambda * tau)) / (tau * M));
                const double e = (totK + V / M + m.tailV) / N;
                if (upos) {
                    WalkerAcc& A = accs[w];
                    A.esum += e; A.esumsq += e * e; A.samples += 1;
                } else {
                    esum += e; esumsq += e * e; nsamp += 1;
                }
            }
            team_sync(slot, T);
        }
        ++sw;
        u = 0;
        if (stop) break;
    }
    if (tt == 0) {
        WalkerAcc& A = accs[w];
        A.esum += esum; A.esumsq += esumsq; A.samples += nsamp; A.bead_updates += nbu;
        A.att[0] += att0; A.att[1] += att1; A.acc[0] += acc0; A.acc[1] += acc1;
        ctr[w] = sweep0 + sw;
        if (upos) upos[w] = u;
    }
}

// ---------------------------------------------------------------------------
// Time-window schedule.  Staging moves whose closed segments [s0, s0+len] lie
// in disjoint imaginary-time windows touch disjoint sets of beads and read no
// bead another one writes, so they commute: applying them at once equals
// applying them one after another.  A walker with M slices gets P =
// min(8, M / (Mbar + 1)) warps; every round draws a random offset phi, cuts
// the slices into P windows of S = M / P slices starting at phi, and each warp
// makes one complete staging move inside its window (bridge, pair sums,
// Metropolis test, write-back) with warp-level synchronisation only.  The
// selection of particle, window position and stage length never depends on
// the configuration, so every move keeps the staging acceptance
// min(1, exp(-dU)) and detailed balance; a sweep makes the same number of
// staging and centre-of-mass moves as the sequential loop in expectation.
// ---------------------------------------------------------------------------

template <int MINB>
__global__ void __launch_bounds__(kTeamCta, MINB)
k_walkers_windows(const WalkerMeta* __restrict__ meta, const int4* __restrict__ teams,
                  float4* __restrict__ pos, WalkerAcc* __restrict__ accs,
                  unsigned long long* __restrict__ ctr, int sweeps, int measure, AzizF az,
                  double tau, double lambda, float p_com, int var_updates, uint64_t seed) {
    __shared__ float4 s_new[8][kMaxStage];
    __shared__ float4 s_old[8][kMaxStage];
    __shared__ double s_red[8][8];
    __shared__ int s_acc[8];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int4 tm = make_int4(-1, 0, 0, 0);
    #pragma unroll
    for (int k = 0; k < 8; ++k) {
        int4 t = teams[blockIdx.x * 8 + k];
        if (t.w && warp >= t.y && warp < t.y + t.z) tm = t;
    }
    if (tm.x < 0) return;
    const int w = tm.x, slot = tm.y, P = tm.z, T = P * 32;
    float4* so = s_old[warp];
    const int tt = threadIdx.x - slot * 32, wi = warp - slot;
    const WalkerMeta m = meta[w];
    float4* Pp = pos + m.off;
    const int N = m.N, M = m.M;
    const int S = M / P;                         // window length (>= Mbar + 1)
    float4* sn = s_new[warp];
    double* red = s_red[slot];
    const unsigned long long sweep0 = ctr[w];
    double esum = 0.0, esumsq = 0.0;
    long long nsamp = 0, nbu = 0, nbu_com = 0, att0 = 0, att1 = 0, acc0 = 0, acc1 = 0;

    for (int sw = 0; sw < min(sweeps, m.max_sweeps); ++sw) {
        const unsigned long long gs = sweep0 + sw;
        const uint32_t g0 = (uint32_t)gs, g1 = (uint32_t)(gs >> 32);
        // split of the sweep's numUpdates moves into staging and COM moves
        const uint4 rs = wrand(m.key, 0xC0000000u, g0, g1, 0u);
        const float ncom_f = p_com * (float)m.num_updates;
        const int n_com = (int)ncom_f + ((u01f(rs.x) < ncom_f - floorf(ncom_f)) ? 1 : 0);
        const int n_stage = m.num_updates - n_com;
        const int rounds = (n_stage + P - 1) / P;
        for (int r = 0; r < rounds; ++r) {
            const uint4 rphi = wrand(m.key, 0x80000000u | (uint32_t)r, g0, g1, 0u);
            const int phi = (int)(((unsigned long long)rphi.x * (unsigned)M) >> 32);
            const bool active = (r * P + wi) < n_stage;
            if (active) {
                const uint32_t c0 = (uint32_t)r | ((uint32_t)wi << 24);
                const uint4 r0 = wrand(m.key, c0, g0, g1, 0u);
                const int i = (int)(((unsigned long long)r0.z * (unsigned)N) >> 32);
                const int len = var_updates
                    ? 2 + (int)(((unsigned long long)r0.w * (unsigned)(m.mbar - 1)) >> 32)
                    : m.mbar;
                const int nmove = len - 1;
                const int span = S - len;                                  // >= 1
                int s0 = phi + wi * S + (int)(((unsigned long long)r0.y * (unsigned)span) >> 32);
                s0 %= M;
                // bridge (as in the team schedule), this warp only
                int se = s0 + len; if (se >= M) se -= M;
                const float4 x0 = Pp[(size_t)s0 * N + i], xe = Pp[(size_t)se * N + i];
                float4 ob0 = make_float4(0, 0, 0, 0), ob1 = ob0;
                {
                    int sl = s0 + 1 + lane; if (sl >= M) sl -= M;
                    if (lane < nmove) ob0 = Pp[(size_t)sl * N + i];
                    sl = s0 + 33 + lane; if (sl >= M) sl -= M;
                    if (lane + 32 < nmove) ob1 = Pp[(size_t)sl * N + i];
                }
                float a1x = 0.f, a1y = 0.f, a1z = 0.f, a2x = 0.f, a2y = 0.f, a2z = 0.f;
                if (lane + 1 <= len) {
                    const uint4 a = wrand(m.key, c0, g0, g1, (uint32_t)(lane + 1));
                    const float2 z01 = box_muller(a.x, a.y), z2 = box_muller(a.z, a.w);
                    a1x = m.sig2lt * z01.x; a1y = m.sig2lt * z01.y; a1z = m.sig2lt * z2.x;
                }
                if (lane + 33 <= len) {
                    const uint4 a = wrand(m.key, c0, g0, g1, (uint32_t)(lane + 33));
                    const float2 z01 = box_muller(a.x, a.y), z2 = box_muller(a.z, a.w);
                    a2x = m.sig2lt * z01.x; a2y = m.sig2lt * z01.y; a2z = m.sig2lt * z2.x;
                }
                const float W1x = warp_scan_incl(a1x, lane), W1y = warp_scan_incl(a1y, lane),
                            W1z = warp_scan_incl(a1z, lane);
                const float W2x = warp_scan_incl(a2x, lane) + __shfl_sync(0xffffffffu, W1x, 31);
                const float W2y = warp_scan_incl(a2y, lane) + __shfl_sync(0xffffffffu, W1y, 31);
                const float W2z = warp_scan_incl(a2z, lane) + __shfl_sync(0xffffffffu, W1z, 31);
                const int src = (len <= 32) ? len - 1 : len - 33;
                const float Lx = __shfl_sync(0xffffffffu, len <= 32 ? W1x : W2x, src);
                const float Ly = __shfl_sync(0xffffffffu, len <= 32 ? W1y : W2y, src);
                const float Lz = __shfl_sync(0xffffffffu, len <= 32 ? W1z : W2z, src);
                const float dx = min_image32(xe.x - x0.x, m.L, m.Linv);
                const float dy = min_image32(xe.y - x0.y, m.L, m.Linv);
                const float dz = min_image32(xe.z - x0.z, m.L, m.Linv);
                const float il = 1.0f / (float)len;
                float4 mine0 = make_float4(0, 0, 0, 0), mine1 = mine0;
                #pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int k = lane + 32 * h;
                    if (k < nmove) {
                        const float f = (float)(k + 1) * il;
                        const float Wx = h ? W2x : W1x, Wy = h ? W2y : W1y, Wz = h ? W2z : W1z;
                        const float4 nv = make_float4(put_inside(x0.x + fmaf(f, dx - Lx, Wx), m.L, m.Linv),
                                                      put_inside(x0.y + fmaf(f, dy - Ly, Wy), m.L, m.Linv),
                                                      put_inside(x0.z + fmaf(f, dz - Lz, Wz), m.L, m.Linv), 0.f);
                        sn[k] = nv;
                        so[k] = h ? ob1 : ob0;
                        if (h) mine1 = nv; else mine0 = nv;
                    }
                }
                __syncwarp();
                // pair sums: lane <-> partner j, loop over moved beads k
                KahanF acc;
                for (int j = lane; j < N; j += 32) {
                    if (j == i) continue;
                    #pragma unroll 4
                    for (int k = 0; k < nmove; ++k) {
                        int sl = s0 + 1 + k; if (sl >= M) sl -= M;
                        const float4 pj = Pp[(size_t)sl * N + j];
                        const float4 a = sn[k], b = so[k];
                        const float ax = min_image32(a.x - pj.x, m.L, m.Linv);
                        const float ay = min_image32(a.y - pj.y, m.L, m.Linv);
                        const float az_ = min_image32(a.z - pj.z, m.L, m.Linv);
                        const float bx = min_image32(b.x - pj.x, m.L, m.Linv);
                        const float by = min_image32(b.y - pj.y, m.L, m.Linv);
                        const float bz = min_image32(b.z - pj.z, m.L, m.Linv);
                        acc.add(aziz_v32(fmaf(ax, ax, fmaf(ay, ay, az_ * az_)), az) -
                                aziz_v32(fmaf(bx, bx, fmaf(by, by, bz * bz)), az));
                    }
                }
                const double dV = warp_sum_ff(acc);
                int ok = 0;
                if (lane == 0) {
                    const uint4 ra = wrand(m.key, c0, g0, g1, 0xFFFFu);
                    ok = metropolis(dV, tau, ra.x, ra.y) ? 1 : 0;
                }
                ok = __shfl_sync(0xffffffffu, ok, 0);
                if (ok) {
                    for (int k = lane; k < nmove; k += 32) {
                        int sl = s0 + 1 + k; if (sl >= M) sl -= M;
                        Pp[(size_t)sl * N + i] = (k < 32) ? mine0 : mine1;
                    }
                }
                att1 += 1; acc1 += ok; nbu += nmove;
            }
            team_sync(slot, T);
        }
        // centre-of-mass moves, whole team
        for (int c = 0; c < n_com; ++c) {
            const uint4 r0 = wrand(m.key, 0x40000000u | (uint32_t)c, g0, g1, 0u);
            const int i = (int)(((unsigned long long)r0.z * (unsigned)N) >> 32);
            const float sx = m.com_delta * (u01f(r0.y) - 0.5f);
            const float sy = m.com_delta * (u01f(r0.w) - 0.5f);
            const float sz = m.com_delta * (u01f(r0.x) - 0.5f);
            KahanF acc;
            for (int idx = tt; idx < M * N; idx += T) {
                const int t = idx / N, j = idx - t * N;
                if (j == i) continue;
                const float4 pi = Pp[(size_t)t * N + i];
                const float4 pj = Pp[(size_t)t * N + j];
                const float bx = min_image32(pi.x - pj.x, m.L, m.Linv);
                const float by = min_image32(pi.y - pj.y, m.L, m.Linv);
                const float bz = min_image32(pi.z - pj.z, m.L, m.Linv);
                const float ax = min_image32(bx + sx, m.L, m.Linv);
                const float ay = min_image32(by + sy, m.L, m.Linv);
                const float az_ = min_image32(bz + sz, m.L, m.Linv);
                acc.add(aziz_v32(fmaf(ax, ax, fmaf(ay, ay, az_ * az_)), az) -
                        aziz_v32(fmaf(bx, bx, fmaf(by, by, bz * bz)), az));
            }
            const double part = warp_sum_ff(acc);
            if (lane == 0) red[wi] = part;
            team_sync(slot, T);
            if (tt == 0) {
                double dV = 0.0;
                for (int q = 0; q < P; ++q) dV += red[q];
                const uint4 ra = wrand(m.key, 0x40000000u | (uint32_t)c, g0, g1, 0xFFFEu);
                s_acc[slot] = metropolis(dV, tau, ra.x, ra.y) ? 1 : 0;
            }
            team_sync(slot, T);
            const int ok = s_acc[slot];
            if (ok)
                for (int t = tt; t < M; t += T) {
                    float4 pi = Pp[(size_t)t * N + i];
                    pi.x = put_inside(pi.x + sx, m.L, m.Linv);
                    pi.y = put_inside(pi.y + sy, m.L, m.Linv);
                    pi.z = put_inside(pi.z + sz, m.L, m.Linv);
                    Pp[(size_t)t * N + i] = pi;
                }
            team_sync(slot, T);
            att0 += 1; acc0 += ok; nbu_com += M;
        }
        if (measure > 0 && ((gs + 1) % (unsigned long long)measure) == 0) {
            KahanF pot, kin;
            const int half = (N - 1) / 2;
            const bool even = (N % 2) == 0;
            for (int idx = tt; idx < M * N; idx += T) {
                const int t = idx / N, ii = idx - t * N;
                const float4 ri = Pp[(size_t)t * N + ii];
                const int cnt = half + ((even && ii < N / 2) ? 1 : 0);
                for (int d = 1; d <= cnt; ++d) {
                    int jj = ii + d; if (jj >= N) jj -= N;
                    const float4 rj = Pp[(size_t)t * N + jj];
                    const float dx = min_image32(ri.x - rj.x, m.L, m.Linv);
                    const float dy = min_image32(ri.y - rj.y, m.L, m.Linv);
                    const float dz = min_image32(ri.z - rj.z, m.L, m.Linv);
                    pot.add(aziz_v32(fmaf(dx, dx, fmaf(dy, dy, dz * dz)), az));
                }
                const int tn = (t + 1 == M) ? 0 : t + 1;
                const float4 rn = Pp[(size_t)tn * N + ii];
                const float vx = min_image32(rn.x - ri.x, m.L, m.Linv);
                const float vy = min_image32(rn.y - ri.y, m.L, m.Linv);
                const float vz = min_image32(rn.z - ri.z, m.L, m.Linv);
                kin.add(fmaf(vx, vx, fmaf(vy, vy, vz * vz)));
            }
            const double pv = warp_sum(pot.value()), kv = warp_sum(kin.value());
            if (lane == 0) red[wi] = pv;
            team_sync(slot, T);
            double V = 0.0;
            if (tt == 0) for (int q = 0; q < P; ++q) V += red[q];
            team_sync(slot, T);
            if (lane == 0) red[wi] = kv;
            team_sync(slot, T);
            if (tt == 0) {
                double K2 = 0.0;
                for (int q = 0; q < P; ++q) K2 += red[q];
                const double totK = 1.5 * N / tau - K2 * ((0.25 / (lambda * tau)) / (tau * M));
                const double e = (totK + V / M + m.tailV) / N;
                esum += e; esumsq += e * e; nsamp += 1;
            }
            team_sync(slot, T);
        }
    }
    if (tt == 0) {
        WalkerAcc& A = accs[w];
        A.esum += esum; A.esumsq += esumsq; A.samples += nsamp;
        A.att[0] += att0; A.acc[0] += acc0;
        atomicAdd(reinterpret_cast<unsigned long long*>(&A.bead_updates), (unsigned long long)nbu_com);
        ctr[w] = sweep0 + min(sweeps, m.max_sweeps);
    }
    // staging counters are per warp (each warp moves in its own window)
    if (lane == 0) {
        atomicAdd(reinterpret_cast<unsigned long long*>(&accs[w].att[1]), (unsigned long long)att1);
        atomicAdd(reinterpret_cast<unsigned long long*>(&accs[w].acc[1]), (unsigned long long)acc1);
        atomicAdd(reinterpret_cast<unsigned long long*>(&accs[w].bead_updates), (unsigned long long)nbu);
    }
}

// ---------------------------------------------------------------------------
// TMA-staged team schedule.  Same teams as the packed-team schedule, but the
// rows of the walker slab a move needs -- the moved slices for staging, the
// slices in chunks of Mbar for centre-of-mass moves and energy samples -- are
// copied into the team's shared-memory buffer with one or two bulk copies
// (cp.async.bulk, completion on an mbarrier) issued by one thread as soon as
// the move is drawn.  The copy overlaps the bridge construction; the pair
// sums then read only shared memory.  Every wait is bounded: a copy that does
// not land within the limit sets the walker's error word and the team exits
// together.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}"
                 :: "r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 :: "r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}" : "=r"(ok) : "r"(smem_u32(bar)), "r"(parity) : "memory");
    return ok != 0;
}
__device__ __forceinline__ void fence_proxy_async_global() {
    asm volatile("fence.proxy.async.global;" ::: "memory");
}

constexpr long long kWaitLimit = 1LL << 22;   // try_wait polls before giving up

// Copy rows [r0, r0 + nrows) (mod M) of a walker slab into buf; returns bytes.
__device__ __forceinline__ uint32_t issue_rows(float4* buf, const float4* P, int N, int M, int r0,
                                               int nrows, uint64_t* bar) {
    const int first = min(nrows, M - r0);
    const uint32_t b1 = (uint32_t)first * N * 16u, b2 = (uint32_t)(nrows - first) * N * 16u;
    mbar_expect_tx(bar, b1 + b2);
    bulk_load(buf, P + (size_t)r0 * N, b1, bar);
    if (b2) bulk_load(buf + (size_t)first * N, P, b2, bar);
    return b1 + b2;
}

// Bounded wait by every team thread; returns false (team-wide) on timeout.
__device__ __forceinline__ bool team_wait(uint64_t* bar, uint32_t parity, int slot, int T,
                                          int* s_fail, int* err_word) {
    long long n = 0;
    bool ok = true;
    while (!mbar_try_wait(bar, parity)) {
        if (++n > kWaitLimit) { ok = false; break; }
    }
    if (!ok) { atomicExch(s_fail, 1); if (err_word) atomicExch(err_word, 1); }
    team_sync(slot, T);
    return *(volatile int*)s_fail == 0;
}

// Energy samples: bead ii's pairs with its cnt successors (cyclic) on one
// buffered slice row.  Two interleaved Kahan sums let consecutive pair
// evaluations overlap; they are folded into `pot` at the end.
__device__ __forceinline__ void row_potential(const float4* __restrict__ row, int ii, int cnt, int N,
                                              float4 ri, const WalkerMeta& m, const AzizF& az,
                                              KahanF& pot) {
    KahanF pa, pb;
    int d = 1;
    for (; d + 1 <= cnt; d += 2) {
        int j1 = ii + d; if (j1 >= N) j1 -= N;
        int j2 = j1 + 1; if (j2 >= N) j2 -= N;
        const float4 r1 = row[j1], r2 = row[j2];
        const float ax = min_image32(ri.x - r1.x, m.L, m.Linv);
        const float ay = min_image32(ri.y - r1.y, m.L, m.Linv);
        const float az_ = min_image32(ri.z - r1.z, m.L, m.Linv);
        const float bx = min_image32(ri.x - r2.x, m.L, m.Linv);
        const float by = min_image32(ri.y - r2.y, m.L, m.Linv);
        const float bz = min_image32(ri.z - r2.z, m.L, m.Linv);
        pa.add(aziz_v32(fmaf(ax, ax, fmaf(ay, ay, az_ * az_)), az));
        pb.add(aziz_v32(fmaf(bx, bx, fmaf(by, by, bz * bz)), az));
    }
    if (d <= cnt) {
        int j1 = ii + d; if (j1 >= N) j1 -= N;
        const float4 r1 = row[j1];
        const float ax = min_image32(ri.x - r1.x, m.L, m.Linv);
        const float ay = min_image32(ri.y - r1.y, m.L, m.Linv);
        const float az_ = min_image32(ri.z - r1.z, m.L, m.Linv);
        pa.add(aziz_v32(fmaf(ax, ax, fmaf(ay, ay, az_ * az_)), az));
    }
    pot.add(pa.s - pa.c);
    pot.add(pb.s - pb.c);
}

template <int MINB>
__global__ void __launch_bounds__(kTeamCta, MINB)
k_walkers_tma(const WalkerMeta* __restrict__ meta, const int4* __restrict__ teams,
              float4* __restrict__ pos, WalkerAcc* __restrict__ accs,
              unsigned long long* __restrict__ ctr, int* __restrict__ err, int sweeps, int measure,
              AzizF az, double tau, double lambda, float p_com, int var_updates, uint64_t seed) {
    extern __shared__ float4 dyn[];
    __shared__ float4 s_new[8][kMaxStage];
    __shared__ double s_red[8][8];
    __shared__ float2 s_ff[8][8];
    __shared__ int s_acc[8];
    __shared__ int s_fail[8];
    __shared__ __align__(8) uint64_t s_bar[8];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int4 tm = make_int4(-1, 0, 0, 0);
    #pragma unroll
    for (int k = 0; k < 8; ++k) {
        int4 t = teams[blockIdx.x * 8 + k];
        if (t.w && warp >= t.y && warp < t.y + t.z) tm = t;
    }
    if (tm.x < 0) return;
    const int w = tm.x, slot = tm.y, nw = tm.z, T = nw * 32;
    const int tt = threadIdx.x - slot * 32, wi = warp - slot;
    const WalkerMeta m = meta[w];
    float4* P = pos + m.off;
    float4* buf = dyn + (tm.w - 1);              // team buffer: Mbar rows of N beads
    const int N = m.N, M = m.M, C = m.mbar;
    double* red = s_red[slot];
    float4* sn = s_new[slot];
    uint64_t* bar = &s_bar[slot];
    int* fail = &s_fail[slot];
    if (tt == 0) { mbar_init(bar, 1); *fail = 0; }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    team_sync(slot, T);
    uint32_t phase = 0;
    const unsigned long long sweep0 = ctr[w];
    double esum = 0.0, esumsq = 0.0;
    long long nsamp = 0, nbu = 0, att0 = 0, att1 = 0, acc0 = 0, acc1 = 0;
    const int G = (T >= N) ? T / N : 1;
    const int j0 = (T >= N) ? ((tt < G * N) ? tt % N : N) : tt;
    const int kb0 = (T >= N) ? tt / N : 0;
    const int jstep = (T >= N) ? N : T;

    for (int sw = 0; sw < min(sweeps, m.max_sweeps); ++sw) {
        const unsigned long long gs = sweep0 + sw;
        const uint32_t g0 = (uint32_t)gs, g1 = (uint32_t)(gs >> 32);
        for (int u = 0; u < m.num_updates; ++u) {
            const uint4 r0 = wrand(m.key, (uint32_t)u, g0, g1, 0u);
            const bool com = u01f(r0.x) < p_com;
            const int i = (int)(((unsigned long long)r0.z * (unsigned)N) >> 32);
            if (!com) {
                const int s0 = (int)(((unsigned long long)r0.y * (unsigned)M) >> 32);
                const int len = var_updates
                    ? 2 + (int)(((unsigned long long)r0.w * (unsigned)(m.mbar - 1)) >> 32)
                    : m.mbar;
                const int nmove = len - 1;
                int rs = s0 + 1; if (rs >= M) rs -= M;
                if (tt == 0) issue_rows(buf, P, N, M, rs, nmove, bar);
                if (wi == 0) {
                    int se = s0 + len; if (se >= M) se -= M;
                    const float4 x0 = P[(size_t)s0 * N + i], xe = P[(size_t)se * N + i];
                    float a1x = 0.f, a1y = 0.f, a1z = 0.f, a2x = 0.f, a2y = 0.f, a2z = 0.f;
                    if (lane + 1 <= len) {
                        const uint4 a = wrand(m.key, (uint32_t)u, g0, g1, (uint32_t)(lane + 1));
                        const float2 z01 = box_muller(a.x, a.y), z2 = box_muller(a.z, a.w);
                        a1x = m.sig2lt * z01.x; a1y = m.sig2lt * z01.y; a1z = m.sig2lt * z2.x;
                    }
                    if (lane + 33 <= len) {
                        const uint4 a = wrand(m.key, (uint32_t)u, g0, g1, (uint32_t)(lane + 33));
                        const float2 z01 = box_muller(a.x, a.y), z2 = box_muller(a.z, a.w);
                        a2x = m.sig2lt * z01.x; a2y = m.sig2lt * z01.y; a2z = m.sig2lt * z2.x;
                    }
                    const float W1x = warp_scan_incl(a1x, lane), W1y = warp_scan_incl(a1y, lane),
                                W1z = warp_scan_incl(a1z, lane);
                    const float W2x = warp_scan_incl(a2x, lane) + __shfl_sync(0xffffffffu, W1x, 31);
                    const float W2y = warp_scan_incl(a2y, lane) + __shfl_sync(0xffffffffu, W1y, 31);
                    const float W2z = warp_scan_incl(a2z, lane) + __shfl_sync(0xffffffffu, W1z, 31);
                    const int src = (len <= 32) ? len - 1 : len - 33;
                    const float Lx = __shfl_sync(0xffffffffu, len <= 32 ? W1x : W2x, src);
                    const float Ly = __shfl_sync(0xffffffffu, len <= 32 ? W1y : W2y, src);
                    const float Lz = __shfl_sync(0xffffffffu, len <= 32 ? W1z : W2z, src);
                    const float dx = min_image32(xe.x - x0.x, m.L, m.Linv);
                    const float dy = min_image32(xe.y - x0.y, m.L, m.Linv);
                    const float dz = min_image32(xe.z - x0.z, m.L, m.Linv);
                    const float il = 1.0f / (float)len;
                    #pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const int k = lane + 32 * h;
                        if (k < nmove) {
                            const float f = (float)(k + 1) * il;
                            const float Wx = h ? W2x : W1x, Wy = h ? W2y : W1y, Wz = h ? W2z : W1z;
                            sn[k] = make_float4(put_inside(x0.x + fmaf(f, dx - Lx, Wx), m.L, m.Linv),
                                                put_inside(x0.y + fmaf(f, dy - Ly, Wy), m.L, m.Linv),
                                                put_inside(x0.z + fmaf(f, dz - Lz, Wz), m.L, m.Linv), 0.f);
                        }
                    }
                }
                if (!team_wait(bar, phase, slot, T, fail, err + w)) return;
                phase ^= 1;
                KahanF acc;
                for (int j = j0; j < N; j += jstep) {
                    if (j == i) continue;
                    #pragma unroll 4
                    for (int k = kb0; k < nmove; k += G) {
                        const float4 pj = buf[k * N + j];
                        const float4 a = sn[k], b = buf[k * N + i];
                        const float ax = min_image32(a.x - pj.x, m.L, m.Linv);
                        const float ay = min_image32(a.y - pj.y, m.L, m.Linv);
                        const float az_ = min_image32(a.z - pj.z, m.L, m.Linv);
                        const float bx = min_image32(b.x - pj.x, m.L, m.Linv);
                        const float by = min_image32(b.y - pj.y, m.L, m.Linv);
                        const float bz = min_image32(b.z - pj.z, m.L, m.Linv);
                        acc.add(aziz_v32(fmaf(ax, ax, fmaf(ay, ay, az_ * az_)), az) -
                                aziz_v32(fmaf(bx, bx, fmaf(by, by, bz * bz)), az));
                    }
                }
                // the team total as a (hi, lo) pair: per-warp sums, then one
                // butterfly over the warps (the pipelined schedule does the same)
                const float2 part = warp_ff(acc);
                if (lane == 0) s_ff[slot][wi] = part;
                team_sync(slot, T);
                if (wi == 0) {
                    const float2 v = ff_butterfly(lane < nw ? s_ff[slot][lane].x : 0.f,
                                                  lane < nw ? s_ff[slot][lane].y : 0.f);
                    if (lane == 0) {
                        const uint4 ra = wrand(m.key, (uint32_t)u, g0, g1, 0xFFFFu);
                        s_acc[slot] = metropolis((double)v.x + (double)v.y, tau, ra.x, ra.y) ? 1 : 0;
                    }
                }
                team_sync(slot, T);
                const int ok = s_acc[slot];
                if (wi == 0) {
                    if (ok) {
                        for (int k = lane; k < nmove; k += 32) {
                            int sl = s0 + 1 + k; if (sl >= M) sl -= M;
                            P[(size_t)sl * N + i] = sn[k];
                        }
                        fence_proxy_async_global();
                    }
                    __syncwarp();
                }
                att1 += 1; acc1 += ok; nbu += nmove;
            } else {
                const float sx = m.com_delta * (u01f(r0.y) - 0.5f);
                const float sy = m.com_delta * (u01f(r0.w) - 0.5f);
                const uint4 r1 = wrand(m.key, (uint32_t)u, g0, g1, 0xFFFEu);
                const float sz = m.com_delta * (u01f(r1.x) - 0.5f);
                KahanF acc;
                for (int c0 = 0; c0 < M; c0 += C) {
                    const int nr = min(C, M - c0);
                    if (tt == 0) issue_rows(buf, P, N, M, c0, nr, bar);
                    if (!team_wait(bar, phase, slot, T, fail, err + w)) return;
                    phase ^= 1;
                    for (int j = j0; j < N; j += jstep) {
                        if (j == i) continue;
                        #pragma unroll 4
                        for (int t = kb0; t < nr; t += G) {
                            const float4 pi = buf[t * N + i], pj = buf[t * N + j];
                            const float bx = min_image32(pi.x - pj.x, m.L, m.Linv);
                            const float by = min_image32(pi.y - pj.y, m.L, m.Linv);
                            const float bz = min_image32(pi.z - pj.z, m.L, m.Linv);
                            const float ax = min_image32(bx + sx, m.L, m.Linv);
                            const float ay = min_image32(by + sy, m.L, m.Linv);
                            const float az_ = min_image32(bz + sz, m.L, m.Linv);
                            acc.add(aziz_v32(fmaf(ax, ax, fmaf(ay, ay, az_ * az_)), az) -
                                    aziz_v32(fmaf(bx, bx, fmaf(by, by, bz * bz)), az));
                        }
                    }
                    team_sync(slot, T);            // buffer free for the next chunk
                }
                const float2 part = warp_ff(acc);
                if (lane == 0) s_ff[slot][wi] = part;
                team_sync(slot, T);
                if (wi == 0) {
                    const float2 v = ff_butterfly(lane < nw ? s_ff[slot][lane].x : 0.f,
                                                  lane < nw ? s_ff[slot][lane].y : 0.f);
                    if (lane == 0) s_acc[slot] = metropolis((double)v.x + (double)v.y, tau, r1.y, r1.z) ? 1 : 0;
                }
                team_sync(slot, T);
                const int ok = s_acc[slot];
                if (ok) {
                    for (int t2 = tt; t2 < M; t2 += T) {
                        float4 pi = P[(size_t)t2 * N + i];
                        pi.x = put_inside(pi.x + sx, m.L, m.Linv);
                        pi.y = put_inside(pi.y + sy, m.L, m.Linv);
                        pi.z = put_inside(pi.z + sz, m.L, m.Linv);
                        P[(size_t)t2 * N + i] = pi;
                    }
                    fence_proxy_async_global();
                }
                team_sync(slot, T);
                att0 += 1; acc0 += ok; nbu += M;
            }
        }
        if (measure > 0 && ((gs + 1) % (unsigned long long)measure) == 0) {
            KahanF pot, kin;
            const int half = (N - 1) / 2;
            const bool even = (N % 2) == 0;
            for (int c0 = 0; c0 < M; c0 += C) {
                const int nr = min(C, M - c0);
                if (tt == 0) issue_rows(buf, P, N, M, c0, nr, bar);
                if (!team_wait(bar, phase, slot, T, fail, err + w)) return;
                phase ^= 1;
                for (int idx = tt; idx < nr * N; idx += T) {
                    const int t = idx / N, ii = idx - t * N;
                    const float4 ri = buf[t * N + ii];
                    const int cnt = half + ((even && ii < N / 2) ? 1 : 0);
                    row_potential(buf + (size_t)t * N, ii, cnt, N, ri, m, az, pot);
                }
                team_sync(slot, T);
            }
            for (int idx = tt; idx < M * N; idx += T) {
                const int t = idx / N, ii = idx - t * N;
                const int tn = (t + 1 == M) ? 0 : t + 1;
                const float4 ri = P[(size_t)t * N + ii], rn = P[(size_t)tn * N + ii];
                const float vx = min_image32(rn.x - ri.x, m.L, m.Linv);
                const float vy = min_image32(rn.y - ri.y, m.L, m.Linv);
                const float vz = min_image32(rn.z - ri.z, m.L, m.Linv);
                kin.add(fmaf(vx, vx, fmaf(vy, vy, vz * vz)));
            }
            const double pv = warp_sum(pot.value()), kv = warp_sum(kin.value());
            if (lane == 0) red[wi] = pv;
            team_sync(slot, T);
            double V = 0.0;
            if (tt == 0) for (int q = 0; q < nw; ++q) V += red[q];
            team_sync(slot, T);
            if (lane == 0) red[wi] = kv;
            team_sync(slot, T);
            if (tt == 0) {
                double K2 = 0.0;
                for (int q = 0; q < nw; ++q) K2 += red[q];
                const double totK = 1.5 * N / tau - K2 * ((0.25 / (lambda * tau)) / (tau * M));
                const double e = (totK + V / M + m.tailV) / N;
                esum += e; esumsq += e * e; nsamp += 1;
            }
            team_sync(slot, T);
        }
    }
    if (tt == 0) {
        WalkerAcc& A = accs[w];
        A.esum += esum; A.esumsq += esumsq; A.samples += nsamp; A.bead_updates += nbu;
        A.att[0] += att0; A.att[1] += att1; A.acc[0] += acc0; A.acc[1] += acc1;
        ctr[w] = sweep0 + min(sweeps, m.max_sweeps);
    }
}

// ---------------------------------------------------------------------------
// Pipelined TMA schedule.  Teams of up to CTA/32 warps; each team owns two
// shared-memory buffers of Mbar + 1 slab rows and two sets of bridge
// increments.  Move descriptions come from the counter-based generator, so
// the next staging move is known before the current one is decided: its rows
// (both fixed ends and the moved slices) are copied into the other buffer and
// its Gaussian increments drawn while the current move sums its pairs.  If
// the current move is accepted and shares beads with the prefetched rows, the
// deciding warp's write-back also patches the prefetched copy (after its copy
// has landed), so every move reads the configuration its predecessor left.
// A staging move costs two team barriers: one after the bridge, one before
// the decision; warp 0 alone decides, writes back and patches while the other
// warps wait at the next move's first barrier.  Centre-of-mass moves and
// energy samples stream the slab through the two buffers in Mbar-row chunks.
// ---------------------------------------------------------------------------
struct MoveDesc {
    int com, i, s0, len, nmove;
    float sx, sy;
};

__device__ __forceinline__ MoveDesc draw_move(int u, uint32_t g0, uint32_t g1,
                                              const WalkerMeta& m, float p_com, int var_updates) {
    MoveDesc d;
    const uint4 r0 = wrand(m.key, (uint32_t)u, g0, g1, 0u);
    d.com = u01f(r0.x) < p_com;
    d.i = (int)(((unsigned long long)r0.z * (unsigned)m.N) >> 32);
    d.s0 = (int)(((unsigned long long)r0.y * (unsigned)m.M) >> 32);
    d.len = var_updates ? 2 + (int)(((unsigned long long)r0.w * (unsigned)(m.mbar - 1)) >> 32) : m.mbar;
    d.nmove = d.len - 1;
    d.sx = m.com_delta * (u01f(r0.y) - 0.5f);
    d.sy = m.com_delta * (u01f(r0.w) - 0.5f);
    return d;
}

// Gaussian increments sigma z of the Brownian bridge of staging move u
// (beads k + 1 = 1 .. len), the same draws and arithmetic as the bridge of
// the one-warp construction, spread over the team's threads.
__device__ __forceinline__ void stage_increments(float4* inc, const WalkerMeta& m, int u, uint32_t g0,
                                                 uint32_t g1, int len, int tt, int T) {
    for (int k = tt; k < len; k += T) {
        const uint4 a = wrand(m.key, (uint32_t)u, g0, g1, (uint32_t)(k + 1));
        const float2 z01 = box_muller(a.x, a.y), z2 = box_muller(a.z, a.w);
        inc[k] = make_float4(m.sig2lt * z01.x, m.sig2lt * z01.y, m.sig2lt * z2.x, 0.f);
    }
}

template <int CTA, int MINB>
__global__ void __launch_bounds__(CTA, MINB)
k_walkers_pipe(const WalkerMeta* __restrict__ meta, const int4* __restrict__ teams,
               float4* __restrict__ pos, WalkerAcc* __restrict__ accs,
               unsigned long long* __restrict__ ctr, int* __restrict__ err, int sweeps, int measure,
               AzizF az, double tau, double lambda, float p_com, int var_updates, uint64_t seed) {
    constexpr int NW = CTA / 32;
    extern __shared__ float4 dyn[];
    __shared__ float4 s_new[NW][kMaxStage];
    __shared__ float2 s_ff[NW][NW];
    __shared__ double s_red[NW][NW];
    __shared__ int s_acc[NW];
    __shared__ int s_fail[NW];
    __shared__ __align__(8) uint64_t s_bar[NW][2];
    // move descriptors: one warp draws them and the team reads them, a ring
    // of three per team (move u + 2 is written while u + 1 is being read)
    __shared__ MoveDesc s_mv[NW][3];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int4 tm = make_int4(-1, 0, 0, 0);
    for (int k = 0; k < NW; ++k) {
        int4 t = teams[blockIdx.x * NW + k];
        if (t.w && warp >= t.y && warp < t.y + t.z) tm = t;
    }
    if (tm.x < 0) return;
    const int w = tm.x, slot = tm.y, nw = tm.z, T = nw * 32;
    const int tt = threadIdx.x - slot * 32, wi = warp - slot;
    const WalkerMeta m = meta[w];
    float4* P = pos + m.off;
    const int N = m.N, M = m.M, C = m.mbar, R = C + 1;
    // two row buffers of Mbar + 1 slab rows, then two sets of bridge increments
    float4* const B0 = dyn + (tm.w - 1);
    float4* const B1 = B0 + (size_t)R * N;
    float4* const I0 = B1 + (size_t)R * N;
    float4* const I1 = I0 + kMaxStage;
    uint64_t* const bar0 = &s_bar[slot][0];
    uint64_t* const bar1 = &s_bar[slot][1];
    auto Bsel = [&](int x) { return x ? B1 : B0; };
    auto barsel = [&](int x) { return x ? bar1 : bar0; };
    auto Isel = [&](int x) { return x ? I1 : I0; };
    double* red = s_red[slot];
    float2* ffr = s_ff[slot];
    float4* sn = s_new[slot];
    int* fail = &s_fail[slot];
    if (tt == 0) { mbar_init(bar0, 1); mbar_init(bar1, 1); *fail = 0; }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    team_sync(slot, T);
    uint32_t ph0 = 0u, ph1 = 0u;
    auto phsel = [&](int x) { return x ? ph1 : ph0; };
    auto phflip = [&](int x) { if (x) ph1 ^= 1u; else ph0 ^= 1u; };
    const unsigned long long sweep0 = ctr[w];
    double esum = 0.0, esumsq = 0.0;
    long long nsamp = 0, nbu = 0, att0 = 0, att1 = 0, acc0 = 0, acc1 = 0;
    const int G = (T >= N) ? T / N : 1;
    const int j0 = (T >= N) ? ((tt < G * N) ? tt % N : N) : tt;
    const int kb0 = (T >= N) ? tt / N : 0;
    const int jstep = (T >= N) ? N : T;
    int cur = 0;
    // bounded wait for a copy this team issued and will not read (error path)
    auto drain = [&](int b) {
        long long n = 0;
        while (!mbar_try_wait(barsel(b), phsel(b)))
            if (++n > kWaitLimit) break;
    };

    for (int sw = 0; sw < min(sweeps, m.max_sweeps); ++sw) {
        const unsigned long long gs = sweep0 + sw;
        const uint32_t g0 = (uint32_t)gs, g1 = (uint32_t)(gs >> 32);
        bool have = false;                        // rows of the current move already in Bsel(cur)
        // warp 0 alone runs the generator for the move descriptors; the other
        // warps read them from shared memory once a barrier has ordered them
        MoveDesc D, Dn;
        if (wi == 0) {
            D = draw_move(0, g0, g1, m, p_com, var_updates);
            Dn = (m.num_updates > 1) ? draw_move(1, g0, g1, m, p_com, var_updates) : D;
            if (lane == 0) { s_mv[slot][0] = D; s_mv[slot][1] = Dn; }
        }
        team_sync(slot, T);
        if (wi != 0) { D = s_mv[slot][0]; Dn = s_mv[slot][1]; }
        // the bridge increments of a staging move depend on the draws alone:
        // those of move u + 1 are made while move u sums its pairs
        if (!D.com) stage_increments(Isel(0), m, 0, g0, g1, D.len, tt, T);
        team_sync(slot, T);
        for (int u = 0; u < m.num_updates; ++u) {
            const bool last = (u + 1 == m.num_updates);
            const bool has_nn = (u + 2 < m.num_updates);
            if (!D.com) {
                bool pre = !last && !Dn.com;             // exact in warp 0, which issues the copies
                const int i = D.i, s0 = D.s0, len = D.len, nmove = D.nmove;
                // rows s0 .. s0 + len: the two fixed ends and the moved slices
                if (tt == 0) {
                    if (!have) issue_rows(Bsel(cur), P, N, M, s0, len + 1, barsel(cur));
                    if (pre) issue_rows(Bsel(cur ^ 1), P, N, M, Dn.s0, Dn.len + 1, barsel(cur ^ 1));
                }
                const float4* buf = Bsel(cur);
                if (wi == 0) {
                    // one warp waits for the rows and builds the Brownian bridge
                    // W_j = sum_{i<=j} sigma z_i, x_j = x0 + (j/len)(xe - x0) + W_j - (j/len) W_len
                    long long nwait = 0;
                    bool landed = true;
                    while (!mbar_try_wait(barsel(cur), phsel(cur)))
                        if (++nwait > kWaitLimit) { landed = false; break; }
                    landed = __all_sync(0xffffffffu, landed);
                    if (!landed) {
                        if (lane == 0) { atomicExch(fail, 1); atomicExch(err + w, 1); }
                    } else {
                        const float4 x0 = buf[i], xe = buf[(size_t)len * N + i];
                        const float4* inc = Isel(u & 1);
                        const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
                        const float4 i1 = (lane < len) ? inc[lane] : zero;
                        const float4 i2 = (lane + 32 < len) ? inc[lane + 32] : zero;
                        const float W1x = warp_scan_incl(i1.x, lane), W1y = warp_scan_incl(i1.y, lane),
                                    W1z = warp_scan_incl(i1.z, lane);
                        const float W2x = warp_scan_incl(i2.x, lane) + __shfl_sync(0xffffffffu, W1x, 31);
                        const float W2y = warp_scan_incl(i2.y, lane) + __shfl_sync(0xffffffffu, W1y, 31);
                        const float W2z = warp_scan_incl(i2.z, lane) + __shfl_sync(0xffffffffu, W1z, 31);
                        const int src = (len <= 32) ? len - 1 : len - 33;
                        const float Lx = __shfl_sync(0xffffffffu, len <= 32 ? W1x : W2x, src);
                        const float Ly = __shfl_sync(0xffffffffu, len <= 32 ? W1y : W2y, src);
                        const float Lz = __shfl_sync(0xffffffffu, len <= 32 ? W1z : W2z, src);
                        const float dx = min_image32(xe.x - x0.x, m.L, m.Linv);
                        const float dy = min_image32(xe.y - x0.y, m.L, m.Linv);
                        const float dz = min_image32(xe.z - x0.z, m.L, m.Linv);
                        const float il = 1.0f / (float)len;
                        #pragma unroll
                        for (int h = 0; h < 2; ++h) {
                            const int k = lane + 32 * h;
                            if (k < nmove) {
                                const float f = (float)(k + 1) * il;
                                const float Wx = h ? W2x : W1x, Wy = h ? W2y : W1y, Wz = h ? W2z : W1z;
                                sn[k] = make_float4(put_inside(x0.x + fmaf(f, dx - Lx, Wx), m.L, m.Linv),
                                                    put_inside(x0.y + fmaf(f, dy - Ly, Wy), m.L, m.Linv),
                                                    put_inside(x0.z + fmaf(f, dz - Lz, Wz), m.L, m.Linv), 0.f);
                            }
                        }
                    }
                }
                phflip(cur);
                team_sync(slot, T);
                // move u + 1 was written by warp 0 during move u - 1 (or at the
                // start of the sweep); the barrier above orders it
                if (wi != 0) Dn = s_mv[slot][(u + 1) % 3];
                pre = !last && !Dn.com;
                if (*(volatile int*)fail) {
                    if (tt == 0 && pre) drain(cur ^ 1);
                    return;
                }
                // while the pairs are summed: the next move's increments, the
                // move after it (drawn by the team's last warp, which waits at
                // the barriers rather than leading the critical path), and this
                // move's acceptance draw
                if (pre) stage_increments(Isel((u + 1) & 1), m, u + 1, g0, g1, Dn.len, tt, T);
                MoveDesc Dnn = Dn;
                if (wi == nw - 1 && has_nn) {
                    Dnn = draw_move(u + 2, g0, g1, m, p_com, var_updates);
                    if (lane == 0) s_mv[slot][(u + 2) % 3] = Dnn;
                }
                MetroDraw md{0.0, 0.f};
                if (tt == 0) {
                    const uint4 ra = wrand(m.key, (uint32_t)u, g0, g1, 0xFFFFu);
                    md = metropolis_draw(ra.x, ra.y);
                }
                KahanF acc;
                for (int j = j0; j < N; j += jstep) {
                    if (j == i) continue;
                    #pragma unroll 4
                    for (int k = kb0; k < nmove; k += G) {
                        const float4 pj = buf[(size_t)(k + 1) * N + j];
                        const float4 a = sn[k], b = buf[(size_t)(k + 1) * N + i];
                        const float ax = min_image32(a.x - pj.x, m.L, m.Linv);
                        const float ay = min_image32(a.y - pj.y, m.L, m.Linv);
                        const float az_ = min_image32(a.z - pj.z, m.L, m.Linv);
                        const float bx = min_image32(b.x - pj.x, m.L, m.Linv);
                        const float by = min_image32(b.y - pj.y, m.L, m.Linv);
                        const float bz = min_image32(b.z - pj.z, m.L, m.Linv);
                        acc.add(aziz_v32(fmaf(ax, ax, fmaf(ay, ay, az_ * az_)), az) -
                                aziz_v32(fmaf(bx, bx, fmaf(by, by, bz * bz)), az));
                    }
                }
                const float2 part = warp_ff(acc);
                if (lane == 0) ffr[wi] = part;
                team_sync(slot, T);
                if (wi == 0) {
                    // the decision, the write-back and the patch belong to one warp;
                    // the others go on to the next move's barrier
                    if (has_nn && nw > 1) Dnn = s_mv[slot][(u + 2) % 3];
                    const float2 v = ff_butterfly(lane < nw ? ffr[lane].x : 0.f, lane < nw ? ffr[lane].y : 0.f);
                    int ok = 0;
                    if (lane == 0) {
                        ok = metropolis_ff(v.x, v.y, tau, (float)tau, md) ? 1 : 0;
                        att1 += 1; acc1 += ok; nbu += nmove;
                    }
                    ok = __shfl_sync(0xffffffffu, ok, 0);
                    if (ok) {
                        for (int k = lane; k < nmove; k += 32) {
                            int sl = s0 + 1 + k; if (sl >= M) sl -= M;
                            P[(size_t)sl * N + i] = sn[k];
                        }
                        fence_proxy_async_global();
                        if (pre) {
                            // the prefetched rows must have landed before they are patched
                            long long n = 0;
                            bool landed = true;
                            while (!mbar_try_wait(barsel(cur ^ 1), phsel(cur ^ 1)))
                                if (++n > kWaitLimit) { landed = false; break; }
                            landed = __all_sync(0xffffffffu, landed);
                            if (!landed) {
                                if (lane == 0) { atomicExch(fail, 1); atomicExch(err + w, 1); }
                            } else {
                                float4* nb = Bsel(cur ^ 1);
                                for (int k = lane; k < nmove; k += 32) {
                                    int sl = s0 + 1 + k; if (sl >= M) sl -= M;
                                    int q = sl - Dn.s0; if (q < 0) q += M;
                                    if (q <= Dn.len) nb[(size_t)q * N + i] = sn[k];
                                }
                                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                            }
                        }
                    }
                    __syncwarp();
                }
                if (pre) { cur ^= 1; have = true; } else { have = false; }
                D = Dn;
                Dn = Dnn;
            } else {
                const int i = D.i;
                const float sx = D.sx, sy = D.sy;
                const uint4 r1 = wrand(m.key, (uint32_t)u, g0, g1, 0xFFFEu);
                const float sz = m.com_delta * (u01f(r1.x) - 0.5f);
                MoveDesc Dnn = Dn;
                if (wi == nw - 1 && has_nn) {
                    Dnn = draw_move(u + 2, g0, g1, m, p_com, var_updates);
                    if (lane == 0) s_mv[slot][(u + 2) % 3] = Dnn;
                }
                KahanF acc;
                int b = cur;
                if (tt == 0) issue_rows(Bsel(b), P, N, M, 0, min(C, M), barsel(b));
                for (int c0 = 0; c0 < M; c0 += C) {
                    const int nr = min(C, M - c0), nb0 = c0 + C;
                    if (nb0 < M && tt == 0) issue_rows(Bsel(b ^ 1), P, N, M, nb0, min(C, M - nb0), barsel(b ^ 1));
                    if (!team_wait(barsel(b), phsel(b), slot, T, fail, err + w)) {
                        if (tt == 0 && nb0 < M) drain(b ^ 1);
                        return;
                    }
                    phflip(b);
                    const float4* buf = Bsel(b);
                    for (int j = j0; j < N; j += jstep) {
                        if (j == i) continue;
                        #pragma unroll 4
                        for (int t = kb0; t < nr; t += G) {
                            const float4 pi = buf[t * N + i], pj = buf[t * N + j];
                            const float bx = min_image32(pi.x - pj.x, m.L, m.Linv);
                            const float by = min_image32(pi.y - pj.y, m.L, m.Linv);
                            const float bz = min_image32(pi.z - pj.z, m.L, m.Linv);
                            const float ax = min_image32(bx + sx, m.L, m.Linv);
                            const float ay = min_image32(by + sy, m.L, m.Linv);
                            const float az_ = min_image32(bz + sz, m.L, m.Linv);
                            acc.add(aziz_v32(fmaf(ax, ax, fmaf(ay, ay, az_ * az_)), az) -
                                    aziz_v32(fmaf(bx, bx, fmaf(by, by, bz * bz)), az));
                        }
                    }
                    team_sync(slot, T);
                    b ^= 1;
                }
                cur = b;
                const float2 part = warp_ff(acc);
                if (lane == 0) ffr[wi] = part;
                team_sync(slot, T);
                if (wi == 0) {
                    const float2 v = ff_butterfly(lane < nw ? ffr[lane].x : 0.f, lane < nw ? ffr[lane].y : 0.f);
                    if (lane == 0) s_acc[slot] = metropolis((double)v.x + (double)v.y, tau, r1.y, r1.z) ? 1 : 0;
                }
                team_sync(slot, T);
                const int ok = s_acc[slot];
                // move u + 1 (written during move u - 1 or at the sweep start)
                // and its bridge increments, before this move's last barrier;
                // warp 0 also takes move u + 2
                if (wi != 0) Dn = s_mv[slot][(u + 1) % 3];
                if (wi == 0 && has_nn && nw > 1) Dnn = s_mv[slot][(u + 2) % 3];
                if (!last && !Dn.com) stage_increments(Isel((u + 1) & 1), m, u + 1, g0, g1, Dn.len, tt, T);
                if (ok) {
                    for (int t2 = tt; t2 < M; t2 += T) {
                        float4 pi = P[(size_t)t2 * N + i];
                        pi.x = put_inside(pi.x + sx, m.L, m.Linv);
                        pi.y = put_inside(pi.y + sy, m.L, m.Linv);
                        pi.z = put_inside(pi.z + sz, m.L, m.Linv);
                        P[(size_t)t2 * N + i] = pi;
                    }
                    fence_proxy_async_global();
                }
                team_sync(slot, T);
                att0 += 1; acc0 += ok; nbu += M;
                have = false;
                D = Dn;
                Dn = Dnn;
            }
        }
        if (measure > 0 && ((gs + 1) % (unsigned long long)measure) == 0) {
            KahanF pot, kin;
            const int half = (N - 1) / 2;
            const bool even = (N % 2) == 0;
            int b = cur;
            if (tt == 0) issue_rows(Bsel(b), P, N, M, 0, min(C, M), barsel(b));
            for (int c0 = 0; c0 < M; c0 += C) {
                const int nr = min(C, M - c0), nb0 = c0 + C;
                if (nb0 < M && tt == 0) issue_rows(Bsel(b ^ 1), P, N, M, nb0, min(C, M - nb0), barsel(b ^ 1));
                if (!team_wait(barsel(b), phsel(b), slot, T, fail, err + w)) return;
                phflip(b);
                const float4* buf = Bsel(b);
                for (int idx = tt; idx < nr * N; idx += T) {
                    const int t = idx / N, ii = idx - t * N;
                    const float4 ri = buf[t * N + ii];
                    const int cnt = half + ((even && ii < N / 2) ? 1 : 0);
                    row_potential(buf + (size_t)t * N, ii, cnt, N, ri, m, az, pot);
                }
                team_sync(slot, T);
                b ^= 1;
            }
            cur = b;
            for (int idx = tt; idx < M * N; idx += T) {
                const int t = idx / N, ii = idx - t * N;
                const int tn = (t + 1 == M) ? 0 : t + 1;
                const float4 ri = P[(size_t)t * N + ii], rn = P[(size_t)tn * N + ii];
                const float vx = min_image32(rn.x - ri.x, m.L, m.Linv);
                const float vy = min_image32(rn.y - ri.y, m.L, m.Linv);
                const float vz = min_image32(rn.z - ri.z, m.L, m.Linv);
                kin.add(fmaf(vx, vx, fmaf(vy, vy, vz * vz)));
            }
            const double pv = warp_sum(pot.value()), kv = warp_sum(kin.value());
            if (lane == 0) red[wi] = pv;
            team_sync(slot, T);
            double V = 0.0;
            if (tt == 0) for (int q = 0; q < nw; ++q) V += red[q];
            team_sync(slot, T);
            if (lane == 0) red[wi] = kv;
            team_sync(slot, T);
            if (tt == 0) {
                double K2 = 0.0;
                for (int q = 0; q < nw; ++q) K2 += red[q];
                const double totK = 1.5 * N / tau - K2 * ((0.25 / (lambda * tau)) / (tau * M));
                const double e = (totK + V / M + m.tailV) / N;
                esum += e; esumsq += e * e; nsamp += 1;
            }
            team_sync(slot, T);
        }
    }
    if (tt == 0) {
        WalkerAcc& A = accs[w];
        A.esum += esum; A.esumsq += esumsq; A.samples += nsamp; A.bead_updates += nbu;
        A.att[0] += att0; A.att[1] += att1; A.acc[0] += acc0; A.acc[1] += acc1;
        ctr[w] = sweep0 + min(sweeps, m.max_sweeps);
    }
}

// ---------------------------------------------------------------------------
// Grouped schedule.  Consecutive staging moves whose closed imaginary-time
// intervals [s0, s0 + len] (mod M) are pairwise disjoint read and write
// disjoint rows of the slab, so they commute: making them at once gives the
// chain of making them one after the other.  From move u on, a team takes the
// longest run of up to GMAX such moves whose rows (len + 1 each) fit its
// shared-memory row pool of 2 (Mbar + 1) rows, splits into 1, 2 or 4
// sub-teams and gives each one move: its rows, bridge, pair sums and
// decision.  A run of one is made by the whole team.  Centre-of-mass moves
// and energy samples use the whole team as in the pipelined schedule.  One
// sub-team's serial work (copy wait, bridge, decision, write-back) overlaps
// the others' pair sums.
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool stage_disjoint(const MoveDesc& a, const MoveDesc& b, int M) {
    int d1 = b.s0 - a.s0; if (d1 < 0) d1 += M;
    int d2 = a.s0 - b.s0; if (d2 < 0) d2 += M;
    return d1 > a.len && d2 > b.len;
}

// named barrier of sub-team g of a team starting at warp `slot`: ids
// slot + 2 .. slot + 5 lie inside the team's own range slot + 1 .. slot + nw
// whenever a sub-team has two or more warps (one-warp sub-teams use
// __syncwarp)
__device__ __forceinline__ void sub_sync(int slot, int g, int HT) {
    if (HT == 32) __syncwarp();
    else asm volatile("bar.sync %0, %1;" :: "r"(slot + 2 + g), "r"(HT) : "memory");
}

template <int CTA, int MINB, int GMAX>
__global__ void __launch_bounds__(CTA, MINB)
k_walkers_group(const WalkerMeta* __restrict__ meta, const int4* __restrict__ teams,
                float4* __restrict__ pos, WalkerAcc* __restrict__ accs,
                unsigned long long* __restrict__ ctr, int* __restrict__ err, int sweeps, int measure,
                AzizF az, double tau, double lambda, float p_com, int var_updates, uint64_t seed) {
    constexpr int NW = CTA / 32;
    extern __shared__ float4 dyn[];
    __shared__ float4 s_new[NW][kMaxStage];
    __shared__ float2 s_ff[NW][NW];
    __shared__ double s_red[NW][NW];
    __shared__ int s_acc[NW];
    __shared__ int s_fail[NW];
    __shared__ __align__(8) uint64_t s_bar[NW][4];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int4 tm = make_int4(-1, 0, 0, 0);
    for (int k = 0; k < NW; ++k) {
        int4 t = teams[blockIdx.x * NW + k];
        if (t.w && warp >= t.y && warp < t.y + t.z) tm = t;
    }
    if (tm.x < 0) return;
    const int w = tm.x, slot = tm.y, nw = tm.z, T = nw * 32;
    const int tt = threadIdx.x - slot * 32, wi = warp - slot;
    const WalkerMeta m = meta[w];
    float4* P = pos + m.off;
    const int N = m.N, M = m.M, C = m.mbar, R = C + 1;
    // row pool of 2 (Mbar + 1) rows (the centre-of-mass and energy chunks use
    // its halves B0, B1), then GMAX sets of bridge increments
    float4* const B0 = dyn + (tm.w - 1);
    float4* const B1 = B0 + (size_t)R * N;
    float4* const Ibase = B1 + (size_t)R * N;
    auto Bsel = [&](int x) { return x ? B1 : B0; };
    auto barsel = [&](int x) { return &s_bar[slot][x]; };
    double* red = s_red[slot];
    int* fail = &s_fail[slot];
    if (tt == 0) {
        for (int g = 0; g < 4; ++g) mbar_init(&s_bar[slot][g], 1);
        *fail = 0;
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    team_sync(slot, T);
    uint32_t phase = 0u;                          // bit g: parity of barrier g
    auto phsel = [&](int x) { return (phase >> x) & 1u; };
    auto phflip = [&](int x) { phase ^= 1u << x; };
    const unsigned long long sweep0 = ctr[w];
    double esum = 0.0, esumsq = 0.0;
    long long nsamp = 0, nbu = 0, att0 = 0, att1 = 0, acc0 = 0, acc1 = 0;
    const int Gt = (T >= N) ? T / N : 1;
    const int j0t = (T >= N) ? ((tt < Gt * N) ? tt % N : N) : tt;
    const int kb0t = (T >= N) ? tt / N : 0;
    const int jstept = (T >= N) ? N : T;
    auto drain = [&](int b) {
        long long n = 0;
        while (!mbar_try_wait(barsel(b), phsel(b)))
            if (++n > kWaitLimit) break;
    };

    for (int sw = 0; sw < min(sweeps, m.max_sweeps); ++sw) {
        const unsigned long long gs = sweep0 + sw;
        const uint32_t g0 = (uint32_t)gs, g1 = (uint32_t)(gs >> 32);
        int u = 0;
        while (u < m.num_updates) {
            const MoveDesc D0 = draw_move(u, g0, g1, m, p_com, var_updates);
            if (!D0.com) {
                // the run of pairwise commuting staging moves that starts at u
                int gs0[GMAX], glen[GMAX];
                gs0[0] = D0.s0; glen[0] = D0.len;
                int ng = 1, rows = D0.len + 1;
                while (ng < GMAX && ng < nw && u + ng < m.num_updates) {
                    const MoveDesc Dc = draw_move(u + ng, g0, g1, m, p_com, var_updates);
                    if (Dc.com || rows + Dc.len + 1 > 2 * R) break;
                    bool ok = true;
                    for (int q = 0; q < ng; ++q) {
                        MoveDesc Dq; Dq.s0 = gs0[q]; Dq.len = glen[q];
                        ok = ok && stage_disjoint(Dq, Dc, M);
                    }
                    if (!ok) break;
                    gs0[ng] = Dc.s0; glen[ng] = Dc.len;
                    rows += Dc.len + 1;
                    ++ng;
                }
                const int gsize = (ng == 1) ? 1 : (ng == 2) ? 2 : 4;
                const int qw = nw / gsize;                 // warps per sub-team
                const int sg = wi / qw;                    // this thread's sub-team
                const bool active = sg < ng;
                const int HT = qw * 32;
                const int ht = tt - sg * HT, wih = wi - sg * qw;
                int off = 0;
                for (int q = 0; q < ng; ++q) if (q < sg) off += glen[q] + 1;
                const int uh = u + sg;
                const MoveDesc D = active ? draw_move(uh, g0, g1, m, p_com, var_updates) : D0;
                const int i = D.i, s0 = D.s0, len = D.len, nmove = D.nmove;
                float4* const buf = B0 + (size_t)off * N;
                float4* const inc = Ibase + sg * kMaxStage;
                float4* const sn = s_new[slot + sg * qw];
                float2* const ffr = s_ff[slot + sg * qw];
                uint64_t* const bar = &s_bar[slot][active ? sg : 0];
                auto gsync = [&]() { if (gsize == 1) team_sync(slot, T); else sub_sync(slot, sg, HT); };
                MetroDraw md{0.0, 0.f};
                if (active) {
                    // rows s0 .. s0 + len, increments and the acceptance draw
                    if (ht == 0) issue_rows(buf, P, N, M, s0, len + 1, bar);
                    stage_increments(inc, m, uh, g0, g1, len, ht, HT);
                    if (ht == 0) {
                        const uint4 ra = wrand(m.key, (uint32_t)uh, g0, g1, 0xFFFFu);
                        md = metropolis_draw(ra.x, ra.y);
                    }
                    gsync();
                    if (wih == 0) {
                        long long nwait = 0;
                        bool landed = true;
                        while (!mbar_try_wait(bar, phsel(sg)))
                            if (++nwait > kWaitLimit) { landed = false; break; }
                        landed = __all_sync(0xffffffffu, landed);
                        if (!landed) {
                            // one more bounded wait for the copy before the team leaves
                            if (lane == 0) {
                                atomicExch(fail, 1); atomicExch(err + w, 1);
                                long long n2 = 0;
                                while (!mbar_try_wait(bar, phsel(sg)))
                                    if (++n2 > kWaitLimit) break;
                            }
                        } else {
                            const float4 x0 = buf[i], xe = buf[(size_t)len * N + i];
                            const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
                            const float4 i1 = (lane < len) ? inc[lane] : zero;
                            const float4 i2 = (lane + 32 < len) ? inc[lane + 32] : zero;
                            const float W1x = warp_scan_incl(i1.x, lane), W1y = warp_scan_incl(i1.y, lane),
                                        W1z = warp_scan_incl(i1.z, lane);
                            const float W2x = warp_scan_incl(i2.x, lane) + __shfl_sync(0xffffffffu, W1x, 31);
                            const float W2y = warp_scan_incl(i2.y, lane) + __shfl_sync(0xffffffffu, W1y, 31);
                            const float W2z = warp_scan_incl(i2.z, lane) + __shfl_sync(0xffffffffu, W1z, 31);
                            const int src = (len <= 32) ? len - 1 : len - 33;
                            const float Lx = __shfl_sync(0xffffffffu, len <= 32 ? W1x : W2x, src);
                            const float Ly = __shfl_sync(0xffffffffu, len <= 32 ? W1y : W2y, src);
                            const float Lz = __shfl_sync(0xffffffffu, len <= 32 ? W1z : W2z, src);
                            const float dx = min_image32(xe.x - x0.x, m.L, m.Linv);
                            const float dy = min_image32(xe.y - x0.y, m.L, m.Linv);
                            const float dz = min_image32(xe.z - x0.z, m.L, m.Linv);
                            const float il = 1.0f / (float)len;
                            #pragma unroll
                            for (int hh = 0; hh < 2; ++hh) {
                                const int k = lane + 32 * hh;
                                if (k < nmove) {
                                    const float f = (float)(k + 1) * il;
                                    const float Wx = hh ? W2x : W1x, Wy = hh ? W2y : W1y, Wz = hh ? W2z : W1z;
                                    sn[k] = make_float4(put_inside(x0.x + fmaf(f, dx - Lx, Wx), m.L, m.Linv),
                                                        put_inside(x0.y + fmaf(f, dy - Ly, Wy), m.L, m.Linv),
                                                        put_inside(x0.z + fmaf(f, dz - Lz, Wz), m.L, m.Linv), 0.f);
                                }
                            }
                        }
                    }
                    gsync();
                    if (!*(volatile int*)fail) {
                        const int G = (HT >= N) ? HT / N : 1;
                        const int j0 = (HT >= N) ? ((ht < G * N) ? ht % N : N) : ht;
                        const int kb0 = (HT >= N) ? ht / N : 0;
                        const int jstep = (HT >= N) ? N : HT;
                        KahanF acc;
                        for (int j = j0; j < N; j += jstep) {
                            if (j == i) continue;
                            #pragma unroll 4
                            for (int k = kb0; k < nmove; k += G) {
                                const float4 pj = buf[(size_t)(k + 1) * N + j];
                                const float4 a = sn[k], b = buf[(size_t)(k + 1) * N + i];
                                const float ax = min_image32(a.x - pj.x, m.L, m.Linv);
                                const float ay = min_image32(a.y - pj.y, m.L, m.Linv);
                                const float az_ = min_image32(a.z - pj.z, m.L, m.Linv);
                                const float bx = min_image32(b.x - pj.x, m.L, m.Linv);
                                const float by = min_image32(b.y - pj.y, m.L, m.Linv);
                                const float bz = min_image32(b.z - pj.z, m.L, m.Linv);
                                acc.add(aziz_v32(fmaf(ax, ax, fmaf(ay, ay, az_ * az_)), az) -
                                        aziz_v32(fmaf(bx, bx, fmaf(by, by, bz * bz)), az));
                            }
                        }
                        const float2 part = warp_ff(acc);
                        if (lane == 0) ffr[wih] = part;
                        gsync();
                        if (wih == 0) {
                            const float2 v = ff_butterfly(lane < qw ? ffr[lane].x : 0.f,
                                                          lane < qw ? ffr[lane].y : 0.f);
                            int ok = 0;
                            if (lane == 0) {
                                ok = metropolis_ff(v.x, v.y, tau, (float)tau, md) ? 1 : 0;
                                att1 += 1; acc1 += ok; nbu += nmove;
                            }
                            ok = __shfl_sync(0xffffffffu, ok, 0);
                            if (ok) {
                                for (int k = lane; k < nmove; k += 32) {
                                    int sl = s0 + 1 + k; if (sl >= M) sl -= M;
                                    P[(size_t)sl * N + i] = sn[k];
                                }
                                fence_proxy_async_global();
                            }
                            __syncwarp();
                        }
                    }
                }
                for (int q = 0; q < ng; ++q) phflip(q);
                // every move written back (and visible to later copies) before
                // the pool and the slab rows are reused
                team_sync(slot, T);
                if (*(volatile int*)fail) return;
                u += ng;
            } else {
                const int i = D0.i;
                const float sx = D0.sx, sy = D0.sy;
                const uint4 r1 = wrand(m.key, (uint32_t)u, g0, g1, 0xFFFEu);
                const float sz = m.com_delta * (u01f(r1.x) - 0.5f);
                KahanF acc;
                int b = 0;
                if (tt == 0) issue_rows(Bsel(b), P, N, M, 0, min(C, M), barsel(b));
                for (int c0 = 0; c0 < M; c0 += C) {
                    const int nr = min(C, M - c0), nb0 = c0 + C;
                    if (nb0 < M && tt == 0) issue_rows(Bsel(b ^ 1), P, N, M, nb0, min(C, M - nb0), barsel(b ^ 1));
                    if (!team_wait(barsel(b), phsel(b), slot, T, fail, err + w)) {
                        if (tt == 0 && nb0 < M) drain(b ^ 1);
                        return;
                    }
                    phflip(b);
                    const float4* buf = Bsel(b);
                    for (int j = j0t; j < N; j += jstept) {
                        if (j == i) continue;
                        #pragma unroll 4
                        for (int t = kb0t; t < nr; t += Gt) {
                            const float4 pi = buf[t * N + i], pj = buf[t * N + j];
                            const float bx = min_image32(pi.x - pj.x, m.L, m.Linv);
                            const float by = min_image32(pi.y - pj.y, m.L, m.Linv);
                            const float bz = min_image32(pi.z - pj.z, m.L, m.Linv);
                            const float ax = min_image32(bx + sx, m.L, m.Linv);
                            const float ay = min_image32(by + sy, m.L, m.Linv);
                            const float az_ = min_image32(bz + sz, m.L, m.Linv);
                            acc.add(aziz_v32(fmaf(ax, ax, fmaf(ay, ay, az_ * az_)), az) -
                                    aziz_v32(fmaf(bx, bx, fmaf(by, by, bz * bz)), az));
                        }
                    }
                    team_sync(slot, T);
                    b ^= 1;
                }
                const float2 part = warp_ff(acc);
                if (lane == 0) s_ff[slot][wi] = part;
                team_sync(slot, T);
                if (wi == 0) {
                    const float2 v = ff_butterfly(lane < nw ? s_ff[slot][lane].x : 0.f,
                                                  lane < nw ? s_ff[slot][lane].y : 0.f);
                    if (lane == 0) s_acc[slot] = metropolis((double)v.x + (double)v.y, tau, r1.y, r1.z) ? 1 : 0;
                }
                team_sync(slot, T);
                const int ok = s_acc[slot];
                if (ok) {
                    for (int t2 = tt; t2 < M; t2 += T) {
                        float4 pi = P[(size_t)t2 * N + i];
                        pi.x = put_inside(pi.x + sx, m.L, m.Linv);
                        pi.y = put_inside(pi.y + sy, m.L, m.Linv);
                        pi.z = put_inside(pi.z + sz, m.L, m.Linv);
                        P[(size_t)t2 * N + i] = pi;
                    }
                    fence_proxy_async_global();
                }
                team_sync(slot, T);
                if (tt == 0) { att0 += 1; acc0 += ok; nbu += M; }
                u += 1;
            }
        }
        if (measure > 0 && ((gs + 1) % (unsigned long long)measure) == 0) {
            KahanF pot, kin;
            const int half = (N - 1) / 2;
            const bool even = (N % 2) == 0;
            int b = 0;
            if (tt == 0) issue_rows(Bsel(b), P, N, M, 0, min(C, M), barsel(b));
            for (int c0 = 0; c0 < M; c0 += C) {
                const int nr = min(C, M - c0), nb0 = c0 + C;
                if (nb0 < M && tt == 0) issue_rows(Bsel(b ^ 1), P, N, M, nb0, min(C, M - nb0), barsel(b ^ 1));
                if (!team_wait(barsel(b), phsel(b), slot, T, fail, err + w)) {
                    if (tt == 0 && nb0 < M) drain(b ^ 1);
                    return;
                }
                phflip(b);
                const float4* buf = Bsel(b);
                for (int idx = tt; idx < nr * N; idx += T) {
                    const int t = idx / N, ii = idx - t * N;
                    const float4 ri = buf[t * N + ii];
                    const int cnt = half + ((even && ii < N / 2) ? 1 : 0);
                    row_potential(buf + (size_t)t * N, ii, cnt, N, ri, m, az, pot);
                }
                team_sync(slot, T);
                b ^= 1;
            }
            for (int idx = tt; idx < M * N; idx += T) {
                const int t = idx / N, ii = idx - t * N;
                const int tn = (t + 1 == M) ? 0 : t + 1;
                const float4 ri = P[(size_t)t * N + ii], rn = P[(size_t)tn * N + ii];
                const float vx = min_image32(rn.x - ri.x, m.L, m.Linv);
                const float vy = min_image32(rn.y - ri.y, m.L, m.Linv);
                const float vz = min_image32(rn.z - ri.z, m.L, m.Linv);
                kin.add(fmaf(vx, vx, fmaf(vy, vy, vz * vz)));
            }
            const double pv = warp_sum(pot.value()), kv = warp_sum(kin.value());
            if (lane == 0) red[wi] = pv;
            team_sync(slot, T);
            double V = 0.0;
            if (tt == 0) for (int q = 0; q < nw; ++q) V += red[q];
            team_sync(slot, T);
            if (lane == 0) red[wi] = kv;
            team_sync(slot, T);
            if (tt == 0) {
                double K2 = 0.0;
                for (int q = 0; q < nw; ++q) K2 += red[q];
                const double totK = 1.5 * N / tau - K2 * ((0.25 / (lambda * tau)) / (tau * M));
                const double e = (totK + V / M + m.tailV) / N;
                esum += e; esumsq += e * e; nsamp += 1;
            }
            team_sync(slot, T);
        }
    }
    if (tt == 0) {
        WalkerAcc& A = accs[w];
        A.esum += esum; A.esumsq += esumsq; A.samples += nsamp;
        A.att[0] += att0; A.acc[0] += acc0;
        ctr[w] = sweep0 + min(sweeps, m.max_sweeps);
    }
    // staging counters live with the deciding thread of each sub-team
    if (att1 || nbu) {
        atomicAdd(reinterpret_cast<unsigned long long*>(&accs[w].att[1]), (unsigned long long)att1);
        atomicAdd(reinterpret_cast<unsigned long long*>(&accs[w].acc[1]), (unsigned long long)acc1);
        atomicAdd(reinterpret_cast<unsigned long long*>(&accs[w].bead_updates), (unsigned long long)nbu);
    }
}

__global__ void k_walkers_init(const WalkerMeta* __restrict__ meta, float4* __restrict__ pos,
                               const int* __restrict__ list) {
    const int w = list ? list[blockIdx.x] : blockIdx.x;
    const WalkerMeta m = meta[w];
    float4* P = pos + m.off;
    for (int i = threadIdx.x; i < m.N; i += blockDim.x) {
        uint4 a = wrand(m.key, (uint32_t)i, 0u, 0u, 0xA0000000u);
        float cx = m.L * (u01f(a.x) - 0.5f), cy = m.L * (u01f(a.y) - 0.5f), cz = m.L * (u01f(a.z) - 0.5f);
        for (int t = 0; t < m.M; ++t) {
            uint4 b = wrand(m.key, (uint32_t)i, (uint32_t)t, 0u, 0xB0000000u);
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
    // host uploads: two FP64 staging buffers filled on their own stream, so
    // the copy of the next state overlaps the sweep on the library stream
    double* d_stage[2] = {nullptr, nullptr};
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev_copied[2] = {nullptr, nullptr}, ev_free[2] = {nullptr, nullptr};
    int stage_idx = 0;
    int* d_err = nullptr;                 // per-walker error word (bounded waits)
    // packed-team schedules, one per pairs-per-thread target
    // 0-2 team targets, 3 windows, 4-6 TMA targets, 7-10 pipelined (256/8, 256/16, 512/8, 512/16)
    int4* d_teams[16] = {nullptr};
    int team_ctas[16] = {0};
    size_t team_smem[16] = {0};
    // autotuner record: schedule and one-sweep time of each candidate
    std::vector<int> tune_sched;
    std::vector<float> tune_ms;
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

// Schedules: 64/128/256 = one CTA of that many threads per walker;
// 1004/1008/1016 = packed teams sized for about 4/8/16 pair evaluations per
// thread per staging move.
constexpr int kTeamScheds[3] = {1004, 1008, 1016};

// Team warps per walker (1, 2, 4 or 8) and their packing into 8-warp CTAs:
// walkers sorted by team size, then by cost N^2 M; CTAs issued by decreasing
// cost so the longest chains start first.
// Pack walkers with tw[w] warps each into 8-warp CTAs (first fit, walkers
// sorted by team size then cost); CTAs are issued by decreasing cost.
// with_buffers: each team gets nbuf buffers of (Mbar + extra_rows) slab rows
// and extra_f4 more float4 of shared memory
cudaError_t pack_teams(pgb_walkers* h, int k, const std::vector<int>& tw, bool with_buffers = false,
                       int cta_warps = 8, int nbuf = 1, size_t smem_budget = 160 * 1024,
                       int extra_rows = 0, int extra_f4 = 0) {
    std::vector<int> idx(h->W);
    std::iota(idx.begin(), idx.end(), 0);
    std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) {
        if (tw[a] != tw[b]) return tw[a] > tw[b];
        return (double)h->N[a] * h->N[a] * h->M[a] > (double)h->N[b] * h->N[b] * h->M[b];
    });
    std::vector<std::vector<int4>> ctas;
    std::vector<int> used;
    std::vector<double> cost;
    std::vector<size_t> bytes;
    for (int w : idx) {
        const size_t need = with_buffers
            ? ((size_t)nbuf * (h->mbar[w] + extra_rows) * h->N[w] + extra_f4) * sizeof(float4) : 0;
        if (need > smem_budget) return cudaErrorInvalidValue;
        int c = -1;
        for (int q = (int)ctas.size() - 1; q >= 0 && q >= (int)ctas.size() - 4; --q)
            if (used[q] + tw[w] <= cta_warps && bytes[q] + need <= smem_budget) { c = q; break; }
        if (c < 0) {
            ctas.emplace_back(); used.push_back(0); cost.push_back(0.0); bytes.push_back(0);
            c = (int)ctas.size() - 1;
        }
        ctas[c].push_back(make_int4(w, used[c], tw[w], 1));
        cost[c] = std::max(cost[c], (double)h->N[w] * h->N[w] * h->M[w] / tw[w]);
        used[c] += tw[w];
        bytes[c] += need;
    }
    std::vector<int> order(ctas.size());
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost[a] > cost[b]; });
    std::vector<int4> flat(ctas.size() * cta_warps, make_int4(-1, 0, 0, 0));
    size_t max_smem = 0;
    for (size_t c = 0; c < order.size(); ++c) {
        size_t off = 0;     // float4 units
        for (size_t e = 0; e < ctas[order[c]].size(); ++e) {
            int4 t = ctas[order[c]][e];
            if (with_buffers) {
                t.w = (int)off + 1;
                off += (size_t)nbuf * (h->mbar[t.x] + extra_rows) * h->N[t.x] + extra_f4;
            }
            flat[c * cta_warps + e] = t;
        }
        max_smem = std::max(max_smem, off * sizeof(float4));
    }
    h->team_smem[k] = max_smem;
    cudaError_t e = cudaMalloc(&h->d_teams[k], flat.size() * sizeof(int4));
    if (e != cudaSuccess) return e;
    e = cudaMemcpy(h->d_teams[k], flat.data(), flat.size() * sizeof(int4), cudaMemcpyHostToDevice);
    h->team_ctas[k] = (int)ctas.size();
    return e;
}

// Team warps per walker (1, 2, 4 or 8) for the packed-team schedule, sized
// for about ppt pair evaluations per thread per staging move.
cudaError_t build_teams(pgb_walkers* h, int k) {
    if (h->d_teams[k]) return cudaSuccess;
    const int ppt = kTeamScheds[k] % 1000;
    std::vector<int> tw(h->W);
    for (int w = 0; w < h->W; ++w) {
        double pairs = (double)h->mbar[w] / 2.0 * h->N[w] * 2.0;     // old + new
        int need = (int)std::ceil(pairs / (32.0 * ppt));
        int t = 1;
        while (t < need && t < 8) t <<= 1;
        tw[w] = t;
    }
    return pack_teams(h, k, tw);
}

// TMA-staged teams: same sizing as build_teams, plus a shared-memory buffer
// of Mbar rows per walker.
cudaError_t build_tma_teams(pgb_walkers* h, int ppt) {
    const int k = 4 + ((ppt == 4) ? 0 : (ppt == 16) ? 2 : 1);
    if (h->d_teams[k]) return cudaSuccess;
    std::vector<int> tw(h->W);
    for (int w = 0; w < h->W; ++w) {
        double pairs = (double)h->mbar[w] / 2.0 * h->N[w] * 2.0;
        int need = (int)std::ceil(pairs / (32.0 * ppt));
        int t = 1;
        while (t < need && t < 8) t <<= 1;
        tw[w] = t;
    }
    return pack_teams(h, k, tw, true);
}

// Pipelined TMA teams: cta = 256 (teams of <= 8 warps, 2 CTAs per SM) or
// 512 (<= 16 warps, 1 CTA per SM); two buffers of Mbar rows per walker.
cudaError_t build_pipe_teams(pgb_walkers* h, int k, int cta, int ppt, int nsets = 2) {
    if (h->d_teams[k]) return cudaSuccess;
    const int cap = cta / 32;
    std::vector<int> tw(h->W);
    double wmax = 0.0;
    for (int w = 0; w < h->W; ++w) wmax = std::max(wmax, (double)h->N[w] * h->N[w] * h->M[w]);
    for (int w = 0; w < h->W; ++w) {
        int need;
        if (ppt == 0) {
            // balanced: warps in proportion to the walker's cost N^2 M, so every
            // chain needs about the same time as the largest one with `cap` warps
            need = (int)std::ceil(cap * (double)h->N[w] * h->N[w] * h->M[w] / wmax);
        } else {
            double pairs = (double)h->mbar[w] / 2.0 * h->N[w] * 2.0;
            need = (int)std::ceil(pairs / (32.0 * ppt));
        }
        int t = 1;
        while (t < need && t < cap) t <<= 1;
        tw[w] = t;
    }
    // two buffers of Mbar + 1 rows and nsets sets of kMaxStage bridge increments
    return pack_teams(h, k, tw, true, cap, 2, cta == 512 ? 200 * 1024 : 100 * 1024, 1, nsets * kMaxStage);
}

// One warp per imaginary-time window: P = min(8, M / (Mbar + 1)) windows.
cudaError_t build_windows(pgb_walkers* h) {
    if (h->d_teams[3]) return cudaSuccess;
    std::vector<int> tw(h->W);
    for (int w = 0; w < h->W; ++w) tw[w] = std::max(1, std::min(8, h->M[w] / (h->mbar[w] + 1)));
    return pack_teams(h, 3, tw);
}

cudaError_t launch_run(pgb_walkers* h, int sched, int sweeps, int measure) {
    AzizF af = make_aziz_f(h->az);
    if (sched >= 7000) {
        // 7xxx: runs of up to two commuting moves, 8xxx: up to four
        const int ppt = sched % 1000;
        const int k = 13 + (ppt == 0 ? 0 : ppt == 8 ? 1 : 2);
        cudaError_t e = build_pipe_teams(h, k, 512, ppt, 4);
        if (e != cudaSuccess) return e;
        e = set_smem_limit(k_walkers_group<512, 1, 2>, 200 * 1024);
        if (e == cudaSuccess) e = set_smem_limit(k_walkers_group<512, 1, 4>, 200 * 1024);
        if (e != cudaSuccess) return e;
        if (sched >= 8000)
            k_walkers_group<512, 1, 4><<<h->team_ctas[k], 512, h->team_smem[k], h->stream>>>(h->d_meta,
                h->d_teams[k], h->d_pos, h->d_acc, h->d_ctr, h->d_err, sweeps, measure, af, h->tau,
                h->lambda, (float)h->p_com, h->var_updates, h->seed);
        else
            k_walkers_group<512, 1, 2><<<h->team_ctas[k], 512, h->team_smem[k], h->stream>>>(h->d_meta,
                h->d_teams[k], h->d_pos, h->d_acc, h->d_ctr, h->d_err, sweeps, measure, af, h->tau,
                h->lambda, (float)h->p_com, h->var_updates, h->seed);
        h->launches += 1;
        return cudaGetLastError();
    }
    if (sched >= 5000) {
        const int ppt = sched % 1000;
        const int cta = (sched >= 6000) ? 512 : 256;
        const int k = (ppt == 0) ? (cta == 512 ? 12 : 11) : 7 + (cta == 512 ? 2 : 0) + (ppt == 16 ? 1 : 0);
        cudaError_t e = build_pipe_teams(h, k, cta, ppt);
        if (e != cudaSuccess) return e;
        e = set_smem_limit(k_walkers_pipe<256, 2>, 100 * 1024);
        if (e == cudaSuccess) e = set_smem_limit(k_walkers_pipe<512, 1>, 200 * 1024);
        if (e != cudaSuccess) return e;
        if (cta == 512)
            k_walkers_pipe<512, 1><<<h->team_ctas[k], 512, h->team_smem[k], h->stream>>>(h->d_meta,
                h->d_teams[k], h->d_pos, h->d_acc, h->d_ctr, h->d_err, sweeps, measure, af, h->tau,
                h->lambda, (float)h->p_com, h->var_updates, h->seed);
        else
            k_walkers_pipe<256, 2><<<h->team_ctas[k], 256, h->team_smem[k], h->stream>>>(h->d_meta,
                h->d_teams[k], h->d_pos, h->d_acc, h->d_ctr, h->d_err, sweeps, measure, af, h->tau,
                h->lambda, (float)h->p_com, h->var_updates, h->seed);
        h->launches += 1;
        return cudaGetLastError();
    }
    if (sched >= 4000) {
        const int ppt = sched % 1000;
        const int k = 4 + ((ppt == 4) ? 0 : (ppt == 16) ? 2 : 1);
        cudaError_t e = build_tma_teams(h, ppt);
        if (e != cudaSuccess) return e;
        e = set_smem_limit(k_walkers_tma<2>, 160 * 1024);
        if (e != cudaSuccess) return e;
        if (h->team_smem[k] > 160 * 1024) return cudaErrorInvalidValue;
        k_walkers_tma<2><<<h->team_ctas[k], kTeamCta, h->team_smem[k], h->stream>>>(h->d_meta,
            h->d_teams[k], h->d_pos, h->d_acc, h->d_ctr, h->d_err, sweeps, measure, af, h->tau,
            h->lambda, (float)h->p_com, h->var_updates, h->seed);
        h->launches += 1;
        return cudaGetLastError();
    }
    if (sched >= 3000) {
        cudaError_t e = build_windows(h);
        if (e != cudaSuccess) return e;
        if (sched == 3002)
            k_walkers_windows<2><<<h->team_ctas[3], kTeamCta, 0, h->stream>>>(h->d_meta, h->d_teams[3],
                h->d_pos, h->d_acc, h->d_ctr, sweeps, measure, af, h->tau, h->lambda,
                (float)h->p_com, h->var_updates, h->seed);
        else
            k_walkers_windows<3><<<h->team_ctas[3], kTeamCta, 0, h->stream>>>(h->d_meta, h->d_teams[3],
                h->d_pos, h->d_acc, h->d_ctr, sweeps, measure, af, h->tau, h->lambda,
                (float)h->p_com, h->var_updates, h->seed);
        h->launches += 1;
        return cudaGetLastError();
    }
    if (sched > 1000) {
        // 1xxx: 3 CTAs per SM (80 registers), 2xxx: 2 CTAs per SM (128 registers)
        const int ppt = sched % 1000;
        int k = (ppt == 4) ? 0 : (ppt == 16) ? 2 : 1;
        cudaError_t e = build_teams(h, k);
        if (e != cudaSuccess) return e;
        if (sched >= 2000)
            k_walkers_team<2><<<h->team_ctas[k], kTeamCta, 0, h->stream>>>(h->d_meta, h->d_teams[k],
                h->d_pos, h->d_acc, h->d_ctr, sweeps, measure, af, h->tau, h->lambda,
                (float)h->p_com, h->var_updates, h->seed, 0ull, nullptr);
        else
            k_walkers_team<3><<<h->team_ctas[k], kTeamCta, 0, h->stream>>>(h->d_meta, h->d_teams[k],
                h->d_pos, h->d_acc, h->d_ctr, sweeps, measure, af, h->tau, h->lambda,
                (float)h->p_com, h->var_updates, h->seed, 0ull, nullptr);
        h->launches += 1;
        return cudaGetLastError();
    }
    switch (sched) {
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
    const int cand[15] = {2008, 4008, 5000, 5008, 5016, 6000, 6008, 6016, 3002, 7000, 7008, 7016,
                          8000, 8008, 8016};
    float best = 1e30f; int best_t = 6000;
    for (int c = 0; c < 15; ++c) {
        cudaMemcpyAsync(h->d_pos, save, pb, cudaMemcpyDeviceToDevice, h->stream);
        cudaMemcpyAsync(h->d_ctr, save_ctr, h->W * sizeof(unsigned long long), cudaMemcpyDeviceToDevice, h->stream);
        cudaEventRecord(a, h->stream);
        e = launch_run(h, cand[c], 1, 1);          // one sweep with its energy sample
        cudaEventRecord(b, h->stream);
        if (e != cudaSuccess) {
            // a schedule that does not fit this workload (e.g. shared memory) is skipped
            cudaGetLastError();
            e = cudaEventSynchronize(b);
            if (e != cudaSuccess) break;
            continue;
        }
        e = cudaEventSynchronize(b);
        if (e != cudaSuccess) break;
        float ms = 0; cudaEventElapsedTime(&ms, a, b);
        h->tune_sched.push_back(cand[c]);
        h->tune_ms.push_back(ms);
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
    {
        const int t = p->threads_per_walker;
        const bool team = (t / 1000 == 1 || t / 1000 == 2) && (t % 1000 == 4 || t % 1000 == 8 || t % 1000 == 16);
        const bool win = (t == 3002 || t == 3003 || t == 4004 || t == 4008 || t == 4016 ||
                          t == 5000 || t == 5008 || t == 5016 || t == 6000 || t == 6008 || t == 6016 ||
                          t == 7000 || t == 7008 || t == 7016 || t == 8000 || t == 8008 || t == 8016);
        if (!(t == 0 || t == 64 || t == 128 || t == 256 || team || win)) {
            g_werr = "threads_per_walker must be 0 (autotune), 64/128/256 (one CTA per walker), "
                     "1004/1008/1016 / 2004/2008/2016 (packed teams, 4/8/16 pairs per thread, "
                     "3 or 2 CTAs per SM), 3002/3003 (time windows, 2 or 3 CTAs per SM) or "
                     "4004/4008/4016 (packed teams with TMA-staged rows) or 5000/5008/5016/6000/6008/"
                     "6016 (pipelined TMA teams in 256/512-thread CTAs; x000 = cost-balanced teams) "
                     "or 7000/7008/7016 (up to two commuting moves at once in sub-teams) or "
                     "8000/8008/8016 (up to four)";
            return PGB_EINVAL;
        }
    }
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
        m.key = walker_key(p->seed, w);
        m.max_sweeps = 0x7fffffff;
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
        if ((e = cudaMalloc(&h->d_err, h->W * sizeof(int))) != cudaSuccess) break;
        if ((e = cudaMemsetAsync(h->d_err, 0, h->W * sizeof(int), h->stream)) != cudaSuccess) break;
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
    if (h->copy_stream) cudaStreamSynchronize(h->copy_stream);
    cudaFree(h->d_ctr); cudaFree(h->d_en); cudaFree(h->d_stage[0]); cudaFree(h->d_stage[1]);
    for (int k = 0; k < 16; ++k) cudaFree(h->d_teams[k]);
    cudaFree(h->d_err);
    for (int b = 0; b < 2; ++b) {
        if (h->ev_copied[b]) cudaEventDestroy(h->ev_copied[b]);
        if (h->ev_free[b]) cudaEventDestroy(h->ev_free[b]);
    }
    if (h->copy_stream) cudaStreamDestroy(h->copy_stream);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return PGB_OK;
}

void* pgb_walkers_stream(pgb_walkers* h) { return h ? (void*)h->stream : nullptr; }
long long pgb_walkers_launch_count(pgb_walkers* h) { return h ? h->launches : 0; }
int pgb_walkers_threads(pgb_walkers* h) { return h ? h->tpw : 0; }

int pgb_walkers_tuning(pgb_walkers* h, int* scheds, float* ms, int cap) {
    if (!h) return 0;
    int n = (int)h->tune_sched.size();
    for (int i = 0; i < n && i < cap; ++i) {
        if (scheds) scheds[i] = h->tune_sched[i];
        if (ms) ms[i] = h->tune_ms[i];
    }
    return n;
}

int pgb_walkers_init(pgb_walkers* h) {
    if (!h) return PGB_EINVAL;
    k_walkers_init<<<h->W, 128, 0, h->stream>>>(h->d_meta, h->d_pos, nullptr);
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

int pgb_walkers_get_all_positions(pgb_walkers* h, double* pos) {
    if (!h || !pos) return PGB_EINVAL;
    std::vector<float4> tmp((size_t)h->total_beads);
    cudaError_t e = cudaMemcpyAsync(tmp.data(), h->d_pos, tmp.size() * sizeof(float4),
                                    cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return h->cfail(e, "walkers get all positions");
    for (size_t i = 0; i < tmp.size(); ++i) { pos[3*i] = tmp[i].x; pos[3*i+1] = tmp[i].y; pos[3*i+2] = tmp[i].z; }
    return PGB_OK;
}

int pgb_walkers_get_sweeps(pgb_walkers* h, unsigned long long* sweeps) {
    if (!h || !sweeps) return PGB_EINVAL;
    cudaError_t e = cudaMemcpyAsync(sweeps, h->d_ctr, h->W * sizeof(unsigned long long),
                                    cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return h->cfail(e, "walkers get sweeps");
    return PGB_OK;
}

int pgb_walkers_set_sweeps(pgb_walkers* h, const unsigned long long* sweeps) {
    if (!h || !sweeps) return PGB_EINVAL;
    cudaError_t e = cudaMemcpyAsync(h->d_ctr, sweeps, h->W * sizeof(unsigned long long),
                                    cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return h->cfail(e, "walkers set sweeps");
    return PGB_OK;
}

int pgb_walkers_set_all_positions(pgb_walkers* h, const double* pos) {
    if (!h || !pos) return PGB_EINVAL;
    size_t bytes = (size_t)h->total_beads * 3 * sizeof(double);
    cudaError_t e = cudaSuccess;
    if (!h->copy_stream) {
        if ((e = cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking)) != cudaSuccess)
            return h->cfail(e, "copy stream");
        for (int b = 0; b < 2; ++b) {
            if ((e = cudaEventCreateWithFlags(&h->ev_copied[b], cudaEventDisableTiming)) != cudaSuccess ||
                (e = cudaEventCreateWithFlags(&h->ev_free[b], cudaEventDisableTiming)) != cudaSuccess)
                return h->cfail(e, "upload events");
        }
    }
    const int b = h->stage_idx;
    if (!h->d_stage[b]) {
        if ((e = cudaMalloc(&h->d_stage[b], bytes)) != cudaSuccess) return h->cfail(e, "cudaMalloc(stage)");
        // a fresh buffer has no reader yet
        if ((e = cudaEventRecord(h->ev_free[b], h->stream)) != cudaSuccess) return h->cfail(e, "upload event");
    }
    // copy on the copy stream once the conversion that last read this buffer
    // is done; convert on the library stream once the copy has landed
    if ((e = cudaStreamWaitEvent(h->copy_stream, h->ev_free[b], 0)) != cudaSuccess) return h->cfail(e, "upload wait");
    if ((e = cudaMemcpyAsync(h->d_stage[b], pos, bytes, cudaMemcpyHostToDevice, h->copy_stream)) != cudaSuccess)
        return h->cfail(e, "walkers upload");
    if ((e = cudaEventRecord(h->ev_copied[b], h->copy_stream)) != cudaSuccess) return h->cfail(e, "upload event");
    if ((e = cudaStreamWaitEvent(h->stream, h->ev_copied[b], 0)) != cudaSuccess) return h->cfail(e, "upload wait");
    int blocks = 152 * 8;
    k_walkers_from64<<<blocks, 256, 0, h->stream>>>(h->d_stage[b], h->d_pos, h->total_beads);
    if ((e = cudaGetLastError()) != cudaSuccess) return h->cfail(e, "walkers upload convert");
    if ((e = cudaEventRecord(h->ev_free[b], h->stream)) != cudaSuccess) return h->cfail(e, "upload event");
    h->stage_idx ^= 1;
    h->launches += 1;
    return PGB_OK;
}

int pgb_walkers_run_async(pgb_walkers* h, int sweeps, int measure) {
    if (!h || sweeps < 0 || measure < 0) return PGB_EINVAL;
    if (h->tpw == 0) h->tpw = 6000;
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
    std::vector<int> flags(h->W);
    e = cudaMemcpy(flags.data(), h->d_err, h->W * sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return h->cfail(e, "walkers error words");
    for (int w = 0; w < h->W; ++w)
        if (flags[w]) return h->fail(PGB_ETIMEOUT, "walker " + std::to_string(w) +
                                     ": a staged copy did not complete within the wait limit");
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

// ===========================================================================
// Serving: continuous batching of simulation jobs.
//
// Jobs (N, T, mu, density, sweeps, seed, arrival time) are submitted as they
// come.  Each round the server (1) moves arrived jobs into a FIFO queue,
// (2) admits queued jobs while their worldline slab fits the HBM budget and a
// slot is free, initialises them on the device, (3) advances every active job
// in ONE launch of the packed-team kernel (jobs of all sizes share the
// launch): for `round_seconds` of device time, stopping between two moves and
// resuming there next round, or by a cost-scaled number of sweeps, never past
// the end of the job's current bin, (4) reads the per-job accumulators, emits
// an estimator bin (mean E/N over `bin_sweeps` sweeps) whenever a job
// completes one, and retires finished jobs, freeing their memory and slot for
// the next round.  A job's random streams are keyed by its own seed and
// indexed by (sweep, move), its team size depends only on its own N and Mbar,
// and its energy samples are summed in sample order, so its results are the
// same alone and in any mix, however its moves fall into rounds.
// ===========================================================================
namespace {

struct ServerJob {
    pgb_job_spec spec;
    int state = 0;                 // 0 submitted, 1 queued, 2 active, 3 done
    double t_admit = -1, t_first_bin = -1, t_done = -1;
    int slot = -1, N = 0, M = 0, mbar = 0;
    long long off = -1, beads = 0;
    long long sweeps_done = 0, samples_bin_start = 0;
    double esum_bin_start = 0.0;
    int bins = 0;
    int sweeps_per_round = 1;      // from the job's own cost only
    WalkerMeta meta{};
};

}  // namespace

struct pgb_server {
    pgb_server_params p{};
    AzizParams az{};
    cudaStream_t stream = nullptr;
    float4* d_arena = nullptr;
    long long arena_beads = 0;
    std::map<long long, long long> free_blocks;      // offset -> length (beads)
    int max_slots = 0;
    WalkerMeta* d_meta = nullptr;
    WalkerAcc* d_acc = nullptr;
    unsigned long long* d_ctr = nullptr;
    int* d_upos = nullptr;                           // next move inside the current sweep
    int* d_err = nullptr;
    int4* d_teams = nullptr;
    int teams_cap = 0;
    int* d_list = nullptr;
    std::vector<WalkerMeta> h_meta;
    std::vector<int> free_slots;
    std::vector<int> slot_job;
    std::vector<ServerJob> jobs;
    std::deque<int> queue;
    std::vector<pgb_bin> bins;
    std::chrono::steady_clock::time_point t0;
    long long bead_updates = 0, rounds = 0;
    std::string err;
    int fail(int code, const std::string& m) { err = m; return code; }
    int cfail(cudaError_t e, const char* where) {
        err = std::string("CUDA error ") + cudaGetErrorString(e) + " at " + where;
        return e == cudaErrorMemoryAllocation ? PGB_ENOMEM : PGB_ECUDA;
    }
    double now() const { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); }
    long long alloc(long long n) {
        for (auto it = free_blocks.begin(); it != free_blocks.end(); ++it) {
            if (it->second >= n) {
                long long off = it->first, len = it->second;
                free_blocks.erase(it);
                if (len > n) free_blocks[off + n] = len - n;
                return off;
            }
        }
        return -1;
    }
    void release(long long off, long long n) {
        auto it = free_blocks.emplace(off, n).first;
        auto nx = std::next(it);
        if (nx != free_blocks.end() && it->first + it->second == nx->first) {
            it->second += nx->second; free_blocks.erase(nx);
        }
        if (it != free_blocks.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) { pv->second += it->second; free_blocks.erase(it); }
        }
    }
};

namespace {
thread_local std::string g_serr;
}

extern "C" {

const char* pgb_server_last_error(const pgb_server* s) { return s ? s->err.c_str() : g_serr.c_str(); }

int pgb_server_create(const pgb_server_params* p, pgb_server** out) {
    if (!p || !out || p->hbm_budget_bytes < 1e6 || p->max_active <= 0 || p->sweeps_per_round <= 0 ||
        p->bin_sweeps <= 0 || p->tau <= 0 || p->lambda <= 0 || !(p->round_seconds >= 0.0) ||
        p->round_seconds > 10.0) {
        g_serr = "server_create: need budget >= 1 MB, max_active > 0, sweeps_per_round > 0, "
                 "bin_sweeps > 0, 0 <= round_seconds <= 10";
        return PGB_EINVAL;
    }
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { g_serr = "no CUDA device available"; return PGB_ECUDA; }
    pgb_server* s = new pgb_server();
    s->p = *p;
    s->az = aziz_params(p->aziz_year);
    s->max_slots = p->max_active;
    s->arena_beads = (long long)(p->hbm_budget_bytes / sizeof(float4));
    s->t0 = std::chrono::steady_clock::now();
    cudaError_t e;
    do {
        if ((e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking)) != cudaSuccess) break;
        if ((e = cudaMalloc(&s->d_arena, (size_t)s->arena_beads * sizeof(float4))) != cudaSuccess) break;
        if ((e = cudaMalloc(&s->d_meta, s->max_slots * sizeof(WalkerMeta))) != cudaSuccess) break;
        if ((e = cudaMalloc(&s->d_acc, s->max_slots * sizeof(WalkerAcc))) != cudaSuccess) break;
        if ((e = cudaMalloc(&s->d_ctr, s->max_slots * sizeof(unsigned long long))) != cudaSuccess) break;
        if ((e = cudaMalloc(&s->d_upos, s->max_slots * sizeof(int))) != cudaSuccess) break;
        if ((e = cudaMalloc(&s->d_err, s->max_slots * sizeof(int))) != cudaSuccess) break;
        if ((e = cudaMalloc(&s->d_list, s->max_slots * sizeof(int))) != cudaSuccess) break;
        if ((e = cudaMemsetAsync(s->d_err, 0, s->max_slots * sizeof(int), s->stream)) != cudaSuccess) break;
        e = cudaStreamSynchronize(s->stream);
    } while (0);
    if (e != cudaSuccess) {
        g_serr = std::string("server_create: ") + cudaGetErrorString(e);
        pgb_server_destroy(s);
        return e == cudaErrorMemoryAllocation ? PGB_ENOMEM : PGB_ECUDA;
    }
    s->free_blocks[0] = s->arena_beads;
    s->h_meta.assign(s->max_slots, WalkerMeta{});
    s->slot_job.assign(s->max_slots, -1);
    for (int k = s->max_slots - 1; k >= 0; --k) s->free_slots.push_back(k);
    *out = s;
    return PGB_OK;
}

int pgb_server_destroy(pgb_server* s) {
    if (!s) return PGB_OK;
    if (s->stream) cudaStreamSynchronize(s->stream);
    cudaFree(s->d_arena); cudaFree(s->d_meta); cudaFree(s->d_acc); cudaFree(s->d_ctr);
    cudaFree(s->d_upos); cudaFree(s->d_err); cudaFree(s->d_teams); cudaFree(s->d_list);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return PGB_OK;
}

double pgb_server_clock(pgb_server* s) { return s ? s->now() : 0.0; }
long long pgb_server_bead_updates(pgb_server* s) { return s ? s->bead_updates : 0; }

int pgb_server_submit(pgb_server* s, const pgb_job_spec* j, int* job_id) {
    if (!s || !j) return PGB_EINVAL;
    if (j->n < 2 || j->n > 4096 || j->temperature <= 0 || j->density <= 0 || j->sweeps <= 0)
        return s->fail(PGB_EINVAL, "job: need 2 <= n <= 4096, temperature > 0, density > 0, sweeps > 0");
    ServerJob job;
    job.spec = *j;
    job.N = j->n;
    const double L = std::pow(1.0 * j->n / j->density, 1.0 / 3.0);
    // even M from T and tau (setup.cpp:995-1003), Mbar from setup.cpp:1079-1104
    job.M = 2 * (int)std::lround(1.0 / (2.0 * j->temperature * s->p.tau));
    if (job.M < 4) return s->fail(PGB_EINVAL, "job: temperature too high for tau (fewer than 4 slices)");
    const double ell = std::pow(1.0 * j->n / (L * L * L), -1.0 / 3.0);
    int mb = (int)(ell * ell / (16 * s->p.lambda * s->p.tau));
    if (mb < 2) mb = 2; else if (mb > job.M) mb = job.M / 2;
    if (mb % 2) mb++;
    if (mb >= job.M) mb = job.M - 2;
    if (mb > kMaxStage) mb = kMaxStage;
    job.mbar = mb;
    job.beads = (long long)job.N * job.M;
    if (job.beads > s->arena_beads)
        return s->fail(PGB_EINVAL, "job: worldline slab larger than the whole HBM budget");
    WalkerMeta& m = job.meta;
    m.N = job.N; m.M = job.M; m.mbar = job.mbar;
    const int nu = (int)std::ceil(1.0 * job.N * job.M / (1.0 * job.mbar));
    m.num_updates = nu < 100 ? 100 : nu;
    m.L = (float)L; m.Linv = (float)(1.0 / L);
    m.sig2lt = (float)std::sqrt(2.0 * s->p.lambda * s->p.tau);
    const double T = 1.0 / (job.M * s->p.tau);
    m.com_delta = (float)(0.04 * 2.0 * std::sqrt(M_PI * s->p.lambda / T));
    const double rmorc = s->az.rm / L;
    const double tV = 2.0 * M_PI * s->az.epsilon *
        (-s->az.rm * s->az.rm * s->az.rm * (s->az.C6 * std::pow(rmorc, 3.0) / 3.0 +
                                            s->az.C8 * std::pow(rmorc, 5.0) / 5.0 +
                                            s->az.C10 * std::pow(rmorc, 7.0) / 7.0));
    m.tailV = (1.0 * job.N * job.N / (L * L * L)) * tV;
    m.key = (unsigned long long)j->seed * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull;
    m.max_sweeps = 0;
    // sweeps per round in inverse proportion to the job's cost N^2 M (a
    // 64-particle, 125-slice job makes sweeps_per_round), so one large job
    // does not stretch every round
    {
        const double ref = 64.0 * 64.0 * 125.0, cost = (double)job.N * job.N * job.M;
        job.sweeps_per_round = (int)std::max(1.0, std::min((double)s->p.sweeps_per_round,
                                                           std::floor(s->p.sweeps_per_round * ref / cost)));
    }
    const int id = (int)s->jobs.size();
    s->jobs.push_back(job);
    if (job_id) *job_id = id;
    return PGB_OK;
}

int pgb_server_step(pgb_server* s, int* n_active, int* n_queued) {
    if (!s) return PGB_EINVAL;
    const double now = s->now();
    for (size_t k = 0; k < s->jobs.size(); ++k)
        if (s->jobs[k].state == 0 && s->jobs[k].spec.arrival <= now) { s->jobs[k].state = 1; s->queue.push_back((int)k); }
    // admission: FIFO while a slot and slab memory are free
    std::vector<int> admitted;
    while (!s->queue.empty() && !s->free_slots.empty()) {
        ServerJob& job = s->jobs[s->queue.front()];
        const long long off = s->alloc(job.beads);
        if (off < 0) break;
        job.off = off;
        job.slot = s->free_slots.back();
        s->free_slots.pop_back();
        job.state = 2;
        job.t_admit = now;
        job.meta.off = off;
        s->slot_job[job.slot] = s->queue.front();
        s->h_meta[job.slot] = job.meta;
        admitted.push_back(job.slot);
        s->queue.pop_front();
    }
    std::vector<int> active;
    for (int k = 0; k < s->max_slots; ++k)
        if (s->slot_job[k] >= 0) {
            ServerJob& job = s->jobs[s->slot_job[k]];
            // never past the job's end or its current bin, so every bin holds
            // exactly bin_sweeps samples (the last one the remainder)
            const long long left = job.spec.sweeps - job.sweeps_done;
            const long long bin_left = s->p.bin_sweeps - (job.sweeps_done - job.samples_bin_start);
            long long cap = std::min(left, bin_left);
            if (s->p.round_seconds <= 0.0) cap = std::min<long long>(cap, job.sweeps_per_round);
            s->h_meta[k].max_sweeps = (int)std::max<long long>(cap, 1);
            active.push_back(k);
        } else {
            s->h_meta[k].max_sweeps = 0;
        }
    cudaError_t e = cudaMemcpyAsync(s->d_meta, s->h_meta.data(), s->max_slots * sizeof(WalkerMeta),
                                    cudaMemcpyHostToDevice, s->stream);
    if (e != cudaSuccess) return s->cfail(e, "server meta upload");
    if (!admitted.empty()) {
        for (int k : admitted) {
            cudaMemsetAsync(s->d_acc + k, 0, sizeof(WalkerAcc), s->stream);
            cudaMemsetAsync(s->d_ctr + k, 0, sizeof(unsigned long long), s->stream);
            cudaMemsetAsync(s->d_upos + k, 0, sizeof(int), s->stream);
        }
        e = cudaMemcpyAsync(s->d_list, admitted.data(), admitted.size() * sizeof(int),
                            cudaMemcpyHostToDevice, s->stream);
        if (e != cudaSuccess) return s->cfail(e, "server admit list");
        k_walkers_init<<<(int)admitted.size(), 128, 0, s->stream>>>(s->d_meta, s->d_arena, s->d_list);
        if ((e = cudaGetLastError()) != cudaSuccess) return s->cfail(e, "server init launch");
    }
    if (!active.empty()) {
        // team sizes from each job's own per-move pair count (8 pairs per thread)
        std::vector<int> idx = active;
        std::vector<int> tw(s->max_slots, 1);
        for (int k : active) {
            const WalkerMeta& m = s->h_meta[k];
            const double pairs = (double)m.mbar / 2.0 * m.N * 2.0;
            const int need = (int)std::ceil(pairs / (32.0 * 8));
            int t = 1;
            while (t < need && t < 8) t <<= 1;
            tw[k] = t;
        }
        std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) {
            if (tw[a] != tw[b]) return tw[a] > tw[b];
            const WalkerMeta &x = s->h_meta[a], &y = s->h_meta[b];
            return (double)x.N * x.N * x.M > (double)y.N * y.N * y.M;
        });
        std::vector<int4> flat;
        int used = 8;
        for (int k : idx) {
            if (used + tw[k] > 8) { flat.resize(flat.size() + 8, make_int4(-1, 0, 0, 0)); used = 0; }
            // place the team descriptor in the next free entry of this CTA
            int e8 = 0;
            while (flat[flat.size() - 8 + e8].w) ++e8;
            flat[flat.size() - 8 + e8] = make_int4(k, used, tw[k], 1);
            used += tw[k];
        }
        const int nctas = (int)(flat.size() / 8);
        if ((int)flat.size() > s->teams_cap) {
            cudaFree(s->d_teams);
            s->teams_cap = (int)flat.size() * 2;
            if ((e = cudaMalloc(&s->d_teams, s->teams_cap * sizeof(int4))) != cudaSuccess)
                return s->cfail(e, "server teams");
        }
        if ((e = cudaMemcpyAsync(s->d_teams, flat.data(), flat.size() * sizeof(int4),
                                 cudaMemcpyHostToDevice, s->stream)) != cudaSuccess)
            return s->cfail(e, "server teams upload");
        const bool timed = s->p.round_seconds > 0.0;
        k_walkers_team<2><<<nctas, kTeamCta, 0, s->stream>>>(s->d_meta, s->d_teams, s->d_arena,
            s->d_acc, s->d_ctr, timed ? (1 << 30) : s->p.sweeps_per_round, 1, make_aziz_f(s->az),
            s->p.tau, s->p.lambda, (float)s->p.p_com, 1, 0,
            timed ? (unsigned long long)(s->p.round_seconds * 1e9) : 0ull, s->d_upos);
        if ((e = cudaGetLastError()) != cudaSuccess) return s->cfail(e, "server round launch");
    }
    std::vector<WalkerAcc> acc(s->max_slots);
    e = cudaMemcpyAsync(acc.data(), s->d_acc, s->max_slots * sizeof(WalkerAcc), cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return s->cfail(e, "server round");
    s->rounds += 1;
    const double t_end = s->now();
    for (int k : active) {
        ServerJob& job = s->jobs[s->slot_job[k]];
        const long long before = job.sweeps_done;
        job.sweeps_done = acc[k].samples;       // one energy sample per sweep
        (void)before;
        const bool finished = job.sweeps_done >= job.spec.sweeps;
        while (acc[k].samples - job.samples_bin_start >= s->p.bin_sweeps ||
               (finished && acc[k].samples > job.samples_bin_start)) {
            pgb_bin b;
            b.job = s->slot_job[k];
            b.bin = job.bins;
            b.samples = acc[k].samples - job.samples_bin_start;
            b.energy_per_particle = (acc[k].esum - job.esum_bin_start) / (double)b.samples;
            b.time = t_end;
            s->bins.push_back(b);
            if (job.bins == 0) job.t_first_bin = t_end;
            job.bins += 1;
            job.samples_bin_start = acc[k].samples;
            job.esum_bin_start = acc[k].esum;
        }
        if (finished) {
            job.state = 3;
            job.t_done = t_end;
            s->bead_updates += acc[k].bead_updates;
            s->release(job.off, job.beads);
            s->free_slots.push_back(k);
            s->slot_job[k] = -1;
        }
    }
    // bead updates of active jobs so far are counted when they retire; add the
    // running total of still-active jobs for throughput reports
    if (n_active) { int c = 0; for (int k = 0; k < s->max_slots; ++k) c += (s->slot_job[k] >= 0); *n_active = c; }
    if (n_queued) *n_queued = (int)s->queue.size();
    return PGB_OK;
}

int pgb_server_poll_bins(pgb_server* s, pgb_bin* out, int cap, int* n) {
    if (!s || !n) return PGB_EINVAL;
    const int k = std::min<int>(cap, (int)s->bins.size());
    if (out) for (int i = 0; i < k; ++i) out[i] = s->bins[i];
    s->bins.erase(s->bins.begin(), s->bins.begin() + k);
    *n = k;
    return PGB_OK;
}

int pgb_server_job_info(pgb_server* s, int id, pgb_job_info* out) {
    if (!s || !out || id < 0 || id >= (int)s->jobs.size()) return PGB_EINVAL;
    const ServerJob& j = s->jobs[id];
    out->state = j.state; out->arrival = j.spec.arrival; out->admitted = j.t_admit;
    out->first_bin = j.t_first_bin; out->completed = j.t_done; out->sweeps_done = j.sweeps_done;
    out->n = j.N; out->m = j.M; out->bytes = (size_t)j.beads * sizeof(float4);
    return PGB_OK;
}

int pgb_server_active_bead_updates(pgb_server* s, long long* total) {
    if (!s || !total) return PGB_EINVAL;
    std::vector<WalkerAcc> acc(s->max_slots);
    cudaError_t e = cudaMemcpy(acc.data(), s->d_acc, s->max_slots * sizeof(WalkerAcc), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return s->cfail(e, "server accumulators");
    long long t = s->bead_updates;
    for (int k = 0; k < s->max_slots; ++k) if (s->slot_job[k] >= 0) t += acc[k].bead_updates;
    *total = t;
    return PGB_OK;
}

}  // extern "C"
