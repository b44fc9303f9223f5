// mixed_kernels.cu -- FP32 pair evaluation with FP64 accumulation.
//
// Pair potentials and gradients are the analytic Aziz form in FP32 (no
// table), read from the float4 position mirror; each thread accumulates its
// pairs with Kahan compensation and the block folds the partial sums in FP64.
#include "pgb_device.cuh"

namespace pgb {

__global__ void k_pos32_from64(PathView v, float4* __restrict__ out) {
    size_t n = (size_t)v.M * v.Ne;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        size_t s = i / v.Ne, p = i % v.Ne;
        const double* X = v.pos + s * 3 * v.Ne;
        out[i] = make_float4((float)X[p], (float)X[v.Ne + p], (float)X[2 * v.Ne + p], 0.f);
    }
}

cudaError_t launch_pos32_from64(const PathView& v, float4* d_pos32, cudaStream_t s) {
    size_t n = (size_t)v.M * v.Ne;
    int blocks = (int)((n + 255) / 256);
    if (blocks > 152 * 8) blocks = 152 * 8;
    if (blocks < 1) return cudaSuccess;
    k_pos32_from64<<<blocks, 256, 0, s>>>(v, d_pos32);
    return cudaGetLastError();
}

// d^2V/dr^2 in FP32 (potential.cpp:1877-1907 with d2F of potential.h:976-983)
__device__ __forceinline__ float aziz_d2v32(float r2, const AzizF& a) {
    float rinv = rsqrtf(r2);
    float x = r2 * rinv * a.rminv;
    float ix = rinv * a.rm;
    float ix2 = ix * ix;
    float ix6 = ix2 * ix2 * ix2;
    float e = __expf(x * fmaf(a.beta, x, -a.alpha));
    float ab = fmaf(-2.0f * a.beta, x, a.alpha);
    float T1 = a.A * fmaf(ab, ab, 2.0f * a.beta) * e;
    float t = fmaxf(fmaf(a.D, ix, -1.0f), 0.0f);
    float F = __expf(-t * t);
    float p0 = ix6 * fmaf(ix2, fmaf(ix2, a.C10, a.C8), a.C6);
    float p1 = ix * ix6 * fmaf(ix2, fmaf(ix2, 10.0f * a.C10, 8.0f * a.C8), 6.0f * a.C6);
    float p2 = ix2 * ix6 * fmaf(ix2, fmaf(ix2, 110.0f * a.C10, 72.0f * a.C8), 42.0f * a.C6);
    float dF = 2.0f * a.D * ix2 * t * F;
    float Dix = a.D * ix;
    float d2F = (x < a.D) ? 2.0f * a.D * ix2 * ix * (2.0f * Dix * Dix * Dix - 4.0f * Dix * Dix - Dix + 2.0f) * F : 0.0f;
    return a.eps_rm * a.rminv * (T1 - p2 * F + 2.0f * p1 * dF - p0 * d2F);
}

constexpr int kBeadBlock32 = 256;

__global__ void __launch_bounds__(kBeadBlock32)
k_bead_actions32(PathView v, AzizF az, const int2* __restrict__ beads, int k, int shift,
                 int mode, double tau, double lambda, double vf0, double vf1, double gf0,
                 double gf1, const double* __restrict__ over, double* __restrict__ out,
                 const float4* __restrict__ fall) {
    extern __shared__ float4 lpos[];
    int* lidx = reinterpret_cast<int*>(lpos + v.Ne);
    __shared__ double red[kBeadBlock32 / 32];
    __shared__ int wcount[kBeadBlock32 / 32];
    __shared__ int s_total;
    const int Ne = v.Ne;
    const int b = blockIdx.x;
    const int s = beads[b].x, p = beads[b].y;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    if (s < 0 || s >= v.M || p < 0 || p >= Ne || !v.on[(size_t)s * Ne + p]) {
        if (tid == 0) out[b] = 0.0;
        return;
    }
    const int eo = s % 2;
    const double vf = eo ? vf1 : vf0, gf = eo ? gf1 : gf0;
    const double t = (double)shift * tau;
    const bool need_v = (mode != PGB_ACTION_CORR);
    const bool need_c = (mode == PGB_ACTION_CORR) ? (gf > kEPS)
                      : (mode == PGB_ACTION_FULL) ? (shift == 1 && gf > kEPS) : false;
    const float L0 = (float)v.side[0], L1 = (float)v.side[1], L2 = (float)v.side[2];
    const float I0 = (float)v.sideInv[0], I1 = (float)v.sideInv[1], I2 = (float)v.sideInv[2];
    const float rc2 = (float)v.rc2;
    const float4* P = v.pos32 + (size_t)s * Ne;
    const float4 r1 = over ? make_float4((float)over[3 * b], (float)over[3 * b + 1],
                                         (float)over[3 * b + 2], 0.f)
                           : P[p];
    const int st1 = bead_state(v, s, p);
    if (tid == 0) s_total = 0;
    __syncthreads();
    KahanF vs;
    for (int base = 0; base < Ne; base += kBeadBlock32) {
        int j = base + tid;
        bool in = false;
        float4 rj = make_float4(0, 0, 0, 0);
        if (j < Ne && j != p && v.on[(size_t)s * Ne + j]) {
            rj = P[j];
            float dx = min_image32(rj.x - r1.x, L0, I0);
            float dy = min_image32(rj.y - r1.y, L1, I1);
            float dz = min_image32(rj.z - r1.z, L2, I2);
            float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
            if (r2 < rc2) {
                in = true;
                if (need_v) vs.add((float)pair_factor(st1, bead_state(v, s, j)) * aziz_v32(r2, az));
            }
        }
        unsigned m = __ballot_sync(0xffffffffu, in);
        if (lane == 0) wcount[w] = __popc(m);
        __syncthreads();
        int off = s_total;
        for (int i = 0; i < w; ++i) off += wcount[i];
        if (in) {
            const int slot_ = off + __popc(m & ((1u << lane) - 1u));
            lpos[slot_] = rj;
            lidx[slot_] = j;
        }
        __syncthreads();
        if (tid == 0) { int tot = 0; for (int i = 0; i < kBeadBlock32 / 32; ++i) tot += wcount[i]; s_total += tot; }
        __syncthreads();
    }
    const int nlist = s_total;
    double Vnn = need_v ? block_sum(vs.value(), red) : 0.0;
    double corr_g = 0.0;
    if (need_c && fall) {
        // Every active same-slice bead is in the list (rc covers the box), so
        // the inner sum of gradVnnSquared, F3(b2) = sum over b3 != p, b2 of
        // gradV(r_b2 - r_b3), does not depend on where p is: it is the slice
        // force on b2 less p's own term at p's current position.  O(n) per bead.
        const float4 rpo = P[p];
        KahanF ts;
        float f1x = 0.f, f1y = 0.f, f1z = 0.f;
        const float4* Fs = fall + (size_t)s * Ne;
        for (int n = tid; n < nlist; n += kBeadBlock32) {
            const float4 r2v = lpos[n];
            const float dx = min_image32(r2v.x - r1.x, L0, I0);
            const float dy = min_image32(r2v.y - r1.y, L1, I1);
            const float dz = min_image32(r2v.z - r1.z, L2, I2);
            const float g = aziz_g32(fmaf(dx, dx, fmaf(dy, dy, dz * dz)), az);
            const float F2x = g * dx, F2y = g * dy, F2z = g * dz;
            f1x -= F2x; f1y -= F2y; f1z -= F2z;
            float Fox = F2x, Foy = F2y, Foz = F2z;
            if (over) {
                const float ox = min_image32(r2v.x - rpo.x, L0, I0);
                const float oy = min_image32(r2v.y - rpo.y, L1, I1);
                const float oz = min_image32(r2v.z - rpo.z, L2, I2);
                const float go = aziz_g32(fmaf(ox, ox, fmaf(oy, oy, oz * oz)), az);
                Fox = go * ox; Foy = go * oy; Foz = go * oz;
            }
            const float4 fa = Fs[lidx[n]];
            const float F3x = fa.x - Fox, F3y = fa.y - Foy, F3z = fa.z - Foz;
            const float d22 = fmaf(F2x, F2x, fmaf(F2y, F2y, F2z * F2z));
            const float d23 = fmaf(F2x, F3x, fmaf(F2y, F3y, F2z * F3z));
            ts.add(fmaf(2.0f, d23, d22));
        }
        double T = block_sum(ts.value(), red);
        double Fx = block_sum((double)f1x, red), Fy = block_sum((double)f1y, red),
               Fz = block_sum((double)f1z, red);
        corr_g = T + (Fx * Fx + Fy * Fy + Fz * Fz);
    } else if (need_c) {
        KahanF ts;
        float f1x = 0.f, f1y = 0.f, f1z = 0.f;
        for (int n = tid; n < nlist; n += kBeadBlock32) {
            float4 r2v = lpos[n];
            float dx = min_image32(r2v.x - r1.x, L0, I0);
            float dy = min_image32(r2v.y - r1.y, L1, I1);
            float dz = min_image32(r2v.z - r1.z, L2, I2);
            float g = aziz_g32(fmaf(dx, dx, fmaf(dy, dy, dz * dz)), az);
            float F2x = g * dx, F2y = g * dy, F2z = g * dz;
            f1x -= F2x; f1y -= F2y; f1z -= F2z;
            float F3x = 0.f, F3y = 0.f, F3z = 0.f;
            for (int m2 = 0; m2 < nlist; ++m2) {
                if (m2 == n) continue;
                float4 r3 = lpos[m2];
                float ex = min_image32(r2v.x - r3.x, L0, I0);
                float ey = min_image32(r2v.y - r3.y, L1, I1);
                float ez = min_image32(r2v.z - r3.z, L2, I2);
                float g3 = aziz_g32(fmaf(ex, ex, fmaf(ey, ey, ez * ez)), az);
                F3x = fmaf(g3, ex, F3x); F3y = fmaf(g3, ey, F3y); F3z = fmaf(g3, ez, F3z);
            }
            float d22 = fmaf(F2x, F2x, fmaf(F2y, F2y, F2z * F2z));
            float d23 = fmaf(F2x, F3x, fmaf(F2y, F3y, F2z * F3z));
            ts.add(fmaf(2.0f, d23, d22));
        }
        double T = block_sum(ts.value(), red);
        double Fx = block_sum((double)f1x, red), Fy = block_sum((double)f1y, red),
               Fz = block_sum((double)f1z, red);
        corr_g = T + (Fx * Fx + Fy * Fy + Fz * Fz);
    }
    if (tid == 0) {
        double bareU = vf * t * Vnn;
        double corU = need_c ? gf * t * t * t * lambda * corr_g : 0.0;
        out[b] = (mode == PGB_ACTION_BARE) ? bareU : (mode == PGB_ACTION_CORR) ? corU : bareU + corU;
    }
}

cudaError_t launch_bead_actions32(const PathView& v, AzizParams a, const int2* d_beads, int k,
                                  int shift, int mode, double tau, double lambda,
                                  const double vf[2], const double gf[2], const double* d_over,
                                  double* d_out, cudaStream_t s, const float4* d_force) {
    if (k <= 0) return cudaSuccess;
    size_t smem = (size_t)v.Ne * (sizeof(float4) + sizeof(int));
    if (smem > 200 * 1024) return cudaErrorInvalidValue;     // one slice's list in shared memory
    {
        const cudaError_t ae = set_smem_limit(k_bead_actions32, 200 * 1024);
        if (ae != cudaSuccess) return ae;
    }
    k_bead_actions32<<<k, kBeadBlock32, smem, s>>>(v, make_aziz_f(a), d_beads, k, shift, mode,
                                                   tau, lambda, vf[0], vf[1], gf[0], gf[1], d_over,
                                                   d_out, d_force);
    return cudaGetLastError();
}

// One warp per bead when every active same-slice bead is in the list (the
// cutoff covers the box): no list compaction, and the GSF correction in O(n)
// from the cached slice forces `fall` (see k_bead_actions32).  With `delta`
// set and trial positions given, the warp evaluates the bead at its trial and
// at its current position and writes U(trial) - U(current): one launch per
// batch of trial moves.  Each warp takes kBeadsPerWarp beads in turn and
// leaves its FP32 (hi, lo) sums in shared memory; the FP64 assembly of the
// actions then runs one bead per lane, so the narrow FP64 pipe sees a full
// warp per instruction instead of one lane.
constexpr int kWarpBeadBlock = 256;
constexpr int kBeadsPerWarp = 4;
constexpr int kBeadsPerBlock = (kWarpBeadBlock / 32) * kBeadsPerWarp;   // 32

__device__ __forceinline__ float pair_factor32(int st1, int st2) {
    if (st1 == 2 && st2 == 2) return 1.0f;
    if (st1 == 0 && st2 == 0) return 0.0f;
    return 0.5f;
}

__global__ void __launch_bounds__(kWarpBeadBlock)
k_bead_actions32_full(PathView v, AzizF az, const int2* __restrict__ beads, int k, int shift,
                      int mode, double tau, double lambda, double vf0, double vf1, double gf0,
                      double gf1, const double* __restrict__ over, const float4* __restrict__ fall,
                      int delta, double* __restrict__ out) {
    // per bead of the block: Vn Vo Tn To Fnx Fny Fnz Fox Foy Foz as (hi, lo)
    __shared__ float2 s_part[kBeadsPerBlock][10];
    __shared__ int s_state[kBeadsPerBlock];      // 0 inactive or out of range, 1 active
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int Ne = v.Ne;
    const bool both = delta && over;             // also the current position
    const float L0 = (float)v.side[0], L1 = (float)v.side[1], L2 = (float)v.side[2];
    const float I0 = (float)v.sideInv[0], I1 = (float)v.sideInv[1], I2 = (float)v.sideInv[2];
    for (int r = 0; r < kBeadsPerWarp; ++r) {
        const int lb = warp * kBeadsPerWarp + r;           // bead within the block
        const int b = blockIdx.x * kBeadsPerBlock + lb;
        if (b >= k) { if (lane == 0) s_state[lb] = 0; continue; }
        const int s = beads[b].x, p = beads[b].y;
        if (s < 0 || s >= v.M || p < 0 || p >= Ne || !v.on[(size_t)s * Ne + p]) {
            if (lane == 0) s_state[lb] = 0;
            continue;
        }
        const int eo = s % 2;
        const double gf = eo ? gf1 : gf0;
        const bool need_v = (mode != PGB_ACTION_CORR);
        const bool need_c = (mode == PGB_ACTION_CORR) ? (gf > kEPS)
                          : (mode == PGB_ACTION_FULL) ? (shift == 1 && gf > kEPS) : false;
        const float4* P = v.pos32 + (size_t)s * Ne;
        const float4* Fs = fall + (size_t)s * Ne;
        const float4 rpo = P[p];
        const float4 r1 = over ? make_float4((float)over[3 * b], (float)over[3 * b + 1],
                                             (float)over[3 * b + 2], 0.f) : rpo;
        const int st1 = bead_state(v, s, p);
        KahanF vn, vo, tn, to;
        float fnx = 0.f, fny = 0.f, fnz = 0.f, fox = 0.f, foy = 0.f, foz = 0.f;
        for (int j = lane; j < Ne; j += 32) {
            if (j == p || !v.on[(size_t)s * Ne + j]) continue;
            const float4 rj = P[j];
            const float dx = min_image32(rj.x - r1.x, L0, I0);
            const float dy = min_image32(rj.y - r1.y, L1, I1);
            const float dz = min_image32(rj.z - r1.z, L2, I2);
            const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
            const float fac = pair_factor32(st1, bead_state(v, s, j));
            float ox = dx, oy = dy, oz = dz, ro2 = r2;
            if (over) {
                ox = min_image32(rj.x - rpo.x, L0, I0);
                oy = min_image32(rj.y - rpo.y, L1, I1);
                oz = min_image32(rj.z - rpo.z, L2, I2);
                ro2 = fmaf(ox, ox, fmaf(oy, oy, oz * oz));
            }
            if (need_v) {
                vn.add(fac * aziz_v32(r2, az));
                if (both) vo.add(fac * aziz_v32(ro2, az));
            }
            if (need_c) {
                const float g = aziz_g32(r2, az);
                const float F2x = g * dx, F2y = g * dy, F2z = g * dz;
                float Fox = F2x, Foy = F2y, Foz = F2z;
                if (over) {
                    const float go = aziz_g32(ro2, az);
                    Fox = go * ox; Foy = go * oy; Foz = go * oz;
                }
                const float4 fa = Fs[j];
                // F3: the slice force on j less the term of p at its current position
                const float F3x = fa.x - Fox, F3y = fa.y - Foy, F3z = fa.z - Foz;
                fnx -= F2x; fny -= F2y; fnz -= F2z;
                tn.add(fmaf(2.0f, fmaf(F2x, F3x, fmaf(F2y, F3y, F2z * F3z)),
                            fmaf(F2x, F2x, fmaf(F2y, F2y, F2z * F2z))));
                if (both) {
                    fox -= Fox; foy -= Foy; foz -= Foz;
                    to.add(fmaf(2.0f, fmaf(Fox, F3x, fmaf(Foy, F3y, Foz * F3z)),
                                fmaf(Fox, Fox, fmaf(Foy, Foy, Foz * Foz))));
                }
            }
        }
        const float2 parts[10] = {warp_ff(vn), warp_ff(vo), warp_ff(tn), warp_ff(to),
                                  ff_butterfly(fnx, 0.f), ff_butterfly(fny, 0.f), ff_butterfly(fnz, 0.f),
                                  ff_butterfly(fox, 0.f), ff_butterfly(foy, 0.f), ff_butterfly(foz, 0.f)};
        if (lane == 0) {
            #pragma unroll
            for (int q = 0; q < 10; ++q) s_part[lb][q] = parts[q];
            s_state[lb] = 1;
        }
    }
    __syncthreads();
    if (warp == 0) {
        // one bead of the block per lane: the FP64 assembly of its action(s)
        const int b = blockIdx.x * kBeadsPerBlock + lane;
        if (b < k) {
            double res = 0.0;
            if (s_state[lane]) {
                const int s = beads[b].x;
                const int eo = s % 2;
                const double vf = eo ? vf1 : vf0, gf = eo ? gf1 : gf0;
                const double t = (double)shift * tau;
                const bool need_v = (mode != PGB_ACTION_CORR);
                const bool need_c = (mode == PGB_ACTION_CORR) ? (gf > kEPS)
                                  : (mode == PGB_ACTION_FULL) ? (shift == 1 && gf > kEPS) : false;
                const float2* q = s_part[lane];
                auto dd = [](float2 x) { return (double)x.x + (double)x.y; };
                auto action = [&](double V, double T, double fx, double fy, double fz) {
                    const double bareU = vf * t * V;
                    const double corU = need_c ? gf * t * t * t * lambda * (T + (fx * fx + fy * fy + fz * fz)) : 0.0;
                    return (mode == PGB_ACTION_BARE) ? bareU : (mode == PGB_ACTION_CORR) ? corU : bareU + corU;
                };
                res = action(need_v ? dd(q[0]) : 0.0, dd(q[2]), dd(q[4]), dd(q[5]), dd(q[6]));
                if (both)
                    res -= action(need_v ? dd(q[1]) : 0.0, dd(q[3]), dd(q[7]), dd(q[8]), dd(q[9]));
            }
            out[b] = res;
        }
    }
}

cudaError_t launch_bead_actions32_full(const PathView& v, AzizParams a, const int2* d_beads, int k,
                                       int shift, int mode, double tau, double lambda,
                                       const double vf[2], const double gf[2], const double* d_over,
                                       const float4* d_force, int delta, double* d_out,
                                       cudaStream_t s) {
    if (k <= 0) return cudaSuccess;
    k_bead_actions32_full<<<(k + kBeadsPerBlock - 1) / kBeadsPerBlock, kWarpBeadBlock, 0, s>>>(
        v, make_aziz_f(a), d_beads, k, shift, mode, tau, lambda, vf[0], vf[1], gf[0], gf[1],
        d_over, d_force, delta, d_out);
    return cudaGetLastError();
}

// Same-slice forces of every active bead: F[t][b] = sum over active b3 != b
// of gradV(r_b - r_b3), FP32 with Kahan sums per component.  One CTA per
// slice, O(N^2).
constexpr int kForceBlock = 256;

__global__ void __launch_bounds__(kForceBlock)
k_slice_forces32(PathView v, AzizF az, float4* __restrict__ force) {
    extern __shared__ float4 sp[];
    const int s = blockIdx.x, Ne = v.Ne;
    const float L0 = (float)v.side[0], L1 = (float)v.side[1], L2 = (float)v.side[2];
    const float I0 = (float)v.sideInv[0], I1 = (float)v.sideInv[1], I2 = (float)v.sideInv[2];
    for (int j = threadIdx.x; j < Ne; j += blockDim.x) {
        float4 r = v.pos32[(size_t)s * Ne + j];
        r.w = v.on[(size_t)s * Ne + j] ? 1.f : 0.f;
        sp[j] = r;
    }
    __syncthreads();
    for (int b = threadIdx.x; b < Ne; b += blockDim.x) {
        const float4 rb = sp[b];
        KahanF fx, fy, fz;
        if (rb.w != 0.f) {
            for (int b3 = 0; b3 < Ne; ++b3) {
                const float4 r3 = sp[b3];
                if (b3 == b || r3.w == 0.f) continue;
                const float ex = min_image32(rb.x - r3.x, L0, I0);
                const float ey = min_image32(rb.y - r3.y, L1, I1);
                const float ez = min_image32(rb.z - r3.z, L2, I2);
                const float g = aziz_g32(fmaf(ex, ex, fmaf(ey, ey, ez * ez)), az);
                fx.add(g * ex); fy.add(g * ey); fz.add(g * ez);
            }
        }
        force[(size_t)s * Ne + b] = make_float4(fx.s - fx.c, fy.s - fy.c, fz.s - fz.c, 0.f);
    }
}

cudaError_t launch_slice_forces32(const PathView& v, AzizParams a, float4* d_force, cudaStream_t s) {
    size_t smem = (size_t)v.Ne * sizeof(float4);
    if (smem > 200 * 1024) return cudaErrorInvalidValue;
    {
        const cudaError_t ae = set_smem_limit(k_slice_forces32, 200 * 1024);
        if (ae != cudaSuccess) return ae;
    }
    k_slice_forces32<<<v.M, kForceBlock, smem, s>>>(v, make_aziz_f(a), d_force);
    return cudaGetLastError();
}

// Mixed-precision per-slice estimator terms; same outputs and layout as
// k_slice_terms64 (vint, g2, r1, r2, d1, d2, kin, xch).
constexpr int kSliceBlock32 = 128;

__global__ void __launch_bounds__(kSliceBlock32)
k_slice_terms32(PathView v, AzizF az, int window, double* __restrict__ terms) {
    extern __shared__ float4 sp[];
    __shared__ double red[kSliceBlock32 / 32];
    const int s = blockIdx.x, Ne = v.Ne, n = v.nbs[s];
    const float L0 = (float)v.side[0], L1 = (float)v.side[1], L2 = (float)v.side[2];
    const float I0 = (float)v.sideInv[0], I1 = (float)v.sideInv[1], I2 = (float)v.sideInv[2];
    for (int j = threadIdx.x; j < n; j += blockDim.x) sp[j] = v.pos32[(size_t)s * Ne + j];
    __syncthreads();
    KahanF a_vint, a_g2, a_r1, a_r2, a_d1, a_d2, a_kin, a_xch;
    for (int b1 = threadIdx.x; b1 < n; b1 += blockDim.x) {
        float4 r1 = sp[b1];
        int st1 = bead_state(v, s, b1);
        float Fx = 0.f, Fy = 0.f, Fz = 0.f;
        float T00 = 0.f, T01 = 0.f, T02 = 0.f, T11 = 0.f, T12 = 0.f, T22 = 0.f;
        for (int b2 = 0; b2 < n; ++b2) {
            if (b2 == b1) continue;
            float4 r2 = sp[b2];
            float dx = min_image32(r1.x - r2.x, L0, I0);
            float dy = min_image32(r1.y - r2.y, L1, I1);
            float dz = min_image32(r1.z - r2.z, L2, I2);
            float rr = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
            float V, g;
            aziz_vg32(rr, az, V, g);
            Fx = fmaf(g, dx, Fx); Fy = fmaf(g, dy, Fy); Fz = fmaf(g, dz, Fz);
            if (b2 > b1) a_vint.add((float)pair_factor(st1, bead_state(v, s, b2)) * V);
            // T-matrix: (d2V/r^2 - |dV|/r^3) r r^T + |dV|/r I
            float rinv = rsqrtf(rr);
            float dV = fabsf(g) * rr * rinv;
            float d2V = aziz_d2v32(rr, az);
            float c1 = (d2V - dV * rinv) * rinv * rinv;
            float c0 = dV * rinv;
            T00 = fmaf(c1, dx * dx, T00 + c0); T11 = fmaf(c1, dy * dy, T11 + c0);
            T22 = fmaf(c1, dz * dz, T22 + c0);
            T01 = fmaf(c1, dx * dy, T01); T02 = fmaf(c1, dx * dz, T02); T12 = fmaf(c1, dy * dz, T12);
        }
        a_g2.add(fmaf(Fx, Fx, fmaf(Fy, Fy, Fz * Fz)));
        a_r1.add(fmaf(Fx, r1.x, fmaf(Fy, r1.y, Fz * r1.z)));
        float TFx = fmaf(T00, Fx, fmaf(T01, Fy, T02 * Fz));
        float TFy = fmaf(T01, Fx, fmaf(T11, Fy, T12 * Fz));
        float TFz = fmaf(T02, Fx, fmaf(T12, Fy, T22 * Fz));
        a_r2.add(fmaf(TFx, r1.x, fmaf(TFy, r1.y, TFz * r1.z)));
        if (window > 0) {
            float mx = 0, my = 0, mz = 0, lx = 0, ly = 0, lz = 0, cx = 0, cy = 0, cz = 0;
            int2 cn = make_int2(s, b1), cp = cn;
            float4 pn = r1, pp = r1;
            for (int gm = 0; gm < window; ++gm) {
                if (gm > 0) {
                    cn = v.next[(size_t)cn.x * Ne + cn.y];
                    cp = v.prev[(size_t)cp.x * Ne + cp.y];
                }
                float4 qn = v.pos32[(size_t)cn.x * Ne + cn.y], qp = v.pos32[(size_t)cp.x * Ne + cp.y];
                mx += min_image32(qn.x - pn.x, L0, I0); my += min_image32(qn.y - pn.y, L1, I1);
                mz += min_image32(qn.z - pn.z, L2, I2);
                lx += min_image32(qp.x - pp.x, L0, I0); ly += min_image32(qp.y - pp.y, L1, I1);
                lz += min_image32(qp.z - pp.z, L2, I2);
                cx += (r1.x + mx) + (r1.x + lx); cy += (r1.y + my) + (r1.y + ly);
                cz += (r1.z + mz) + (r1.z + lz);
                pn = qn; pp = qp;
            }
            float den = 1.0f / (2.0f * window);
            float dlx = min_image32(r1.x - cx * den, L0, I0);
            float dly = min_image32(r1.y - cy * den, L1, I1);
            float dlz = min_image32(r1.z - cz * den, L2, I2);
            a_d1.add(fmaf(Fx, dlx, fmaf(Fy, dly, Fz * dlz)));
            a_d2.add(fmaf(TFx, dlx, fmaf(TFy, dly, TFz * dlz)));
            float v1x = 0, v1y = 0, v1z = 0;
            int2 c2 = make_int2(s, b1);
            float4 po = r1;
            for (int gm = 1; gm <= window; ++gm) {
                c2 = v.next[(size_t)c2.x * Ne + c2.y];
                float4 q = v.pos32[(size_t)c2.x * Ne + c2.y];
                v1x += min_image32(q.x - po.x, L0, I0); v1y += min_image32(q.y - po.y, L1, I1);
                v1z += min_image32(q.z - po.z, L2, I2);
                po = q;
            }
            int2 nx = v.next[(size_t)s * Ne + b1];
            float v2x = 0, v2y = 0, v2z = 0;
            if (!(nx.x == kXXX && nx.y == kXXX)) {
                float4 q = v.pos32[(size_t)nx.x * Ne + nx.y];
                v2x = min_image32(q.x - r1.x, L0, I0); v2y = min_image32(q.y - r1.y, L1, I1);
                v2z = min_image32(q.z - r1.z, L2, I2);
            }
            a_xch.add(fmaf(v1x, v2x, fmaf(v1y, v2y, v1z * v2z)));
        }
        int2 nx = v.next[(size_t)s * Ne + b1];
        if (!(nx.x == kXXX && nx.y == kXXX)) {
            float4 q = v.pos32[(size_t)nx.x * Ne + nx.y];
            float ax = min_image32(q.x - r1.x, L0, I0), ay = min_image32(q.y - r1.y, L1, I1);
            float az_ = min_image32(q.z - r1.z, L2, I2);
            a_kin.add(fmaf(ax, ax, fmaf(ay, ay, az_ * az_)));
        }
    }
    double vals[8] = {a_vint.value(), a_g2.value(), a_r1.value(), a_r2.value(),
                      a_d1.value(), a_d2.value(), a_kin.value(), a_xch.value()};
    #pragma unroll
    for (int q = 0; q < 8; ++q) {
        double t = block_sum(vals[q], red);
        if (threadIdx.x == 0) terms[(size_t)q * v.M + s] = t;
    }
}

cudaError_t launch_slice_terms32(const PathView& v, AzizParams a, int window, double* d_terms,
                                 cudaStream_t s) {
    size_t smem = (size_t)v.Ne * sizeof(float4);
    {
        const cudaError_t ae = set_smem_limit(k_slice_terms32, 200 * 1024);
        if (ae != cudaSuccess) return ae;
    }
    k_slice_terms32<<<v.M, kSliceBlock32, smem, s>>>(v, make_aziz_f(a), window, d_terms);
    return cudaGetLastError();
}

}  // namespace pgb
