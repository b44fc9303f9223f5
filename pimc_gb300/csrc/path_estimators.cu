// path_estimators.cu -- the path-wide estimators adjacent to the hot path:
// pair correlation g(r), winding-number superfluid fraction and permutation
// cycles (estimator.cpp:2000-2074, 2735-2781, 3181-3246).  FP64, compiled
// with -fmad=false so that every separation, and therefore every histogram
// bin, is the one the reference computes.
#include "pgb_device.cuh"

namespace pgb {

constexpr int kPcfBins = 50;                 // NPCFSEP, include/common.h:85
constexpr int kEstBlock = 256;

// Separation histogram of the pairs b1 < b2 of slices [t0, t1) with
// ActionBase::updateSepHist's binning (action.cpp:216-224):
// nR = int(|r_b2 - r_b1| / dSep).  One CTA per slice.  The slice is staged
// in shared memory as FP32; each pair's bin is first found in FP32 and, only
// when the FP32 quotient lies within kEdge of a bin edge, recomputed from the
// FP64 positions exactly as the reference does, so every count is the
// reference's.  Error of the FP32 quotient x = |r| / dSep: a position
// (|r_d| <= L/2) rounds by at most 2^-24 L, the difference, the minimum image
// and the sum of squares add a few such roundings, so |r| is off by at most
// about 2^-20 L; with dSep = sqrt(3) L / 100 that is 100 / (sqrt(3) 2^20)
// = 5.5e-5 of a bin for any box, plus 3e-6 from 1/dSep: below 6e-5, a third
// of kEdge.  The FP64 recomputation then runs for about 4e-4 of the pairs:
// one FP64 warp instruction costs the issue of sixteen FP32 ones on this
// GPU, so the edge is kept narrow.  Counts go to per-warp shared
// histograms, so the result is order-free.
constexpr float kEdge = 2.0e-4f;
constexpr int kSepWarps = kEstBlock / 32;

__global__ void __launch_bounds__(kEstBlock)
k_sep_hist(PathView v, int t0, double dSep, unsigned long long* __restrict__ hist) {
    extern __shared__ float4 sp[];                       // [n] slice positions, FP32
    __shared__ unsigned int sh[kSepWarps][kPcfBins];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int b = threadIdx.x; b < kSepWarps * kPcfBins; b += blockDim.x) (&sh[0][0])[b] = 0u;
    const int t = t0 + blockIdx.x;
    const int n = v.nbs[t];
    const double* X = v.pos + (size_t)t * 3 * v.Ne;
    for (int j = threadIdx.x; j < n; j += blockDim.x)
        sp[j] = make_float4((float)X[j], (float)X[v.Ne + j], (float)X[2 * v.Ne + j], 0.f);
    __syncthreads();
    const float Lx = (float)v.side[0], Ly = (float)v.side[1], Lz = (float)v.side[2];
    const float Lix = (float)v.sideInv[0], Liy = (float)v.sideInv[1], Liz = (float)v.sideInv[2];
    const float invSep = (float)(1.0 / dSep);
    const float edge = kEdge;
    for (int b1 = warp; b1 < n - 1; b1 += kSepWarps) {
        const float4 r1 = sp[b1];
        for (int b2 = b1 + 1 + lane; b2 < n; b2 += 32) {
            const float4 r2 = sp[b2];
            float dx = r2.x - r1.x, dy = r2.y - r1.y, dz = r2.z - r1.z;
            dx -= Lx * rint_add(dx * Lix);
            dy -= Ly * rint_add(dy * Liy);
            dz -= Lz * rint_add(dz * Liz);
            const float x = sqrtf(dx * dx + dy * dy + dz * dz) * invSep;
            // floor(x) without float/int conversions: adding 2^23 rounded
            // down leaves floor(x) in the mantissa bits, for 0 <= x < 2^22
            const float xf = __fadd_rd(x, 8388608.0f);
            int nR = __float_as_int(xf) - 0x4B000000;
            const float f = x - __fsub_rn(xf, 8388608.0f);
            if (f < edge || f > 1.0f - edge) {
                const double3 d = sep64(v, t, b2, b1);
                nR = (int)(sqrt(d.x * d.x + d.y * d.y + d.z * d.z) / dSep);
            }
            if (nR >= 0 && nR < kPcfBins) atomicAdd(&sh[warp][nR], 1u);
        }
    }
    __syncthreads();
    for (int b = threadIdx.x; b < kPcfBins; b += blockDim.x) {
        unsigned long long c = 0;
        for (int w = 0; w < kSepWarps; ++w) c += sh[w][b];
        if (c) atomicAdd(&hist[b], c);
    }
}

cudaError_t launch_sep_hist(const PathView& v, int slice, unsigned long long* d_hist, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(d_hist, 0, kPcfBins * sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    const double dSep = 0.5 * sqrt(3.0) * v.side[2] / (1.0 * kPcfBins);   // action.cpp:192
    const int t0 = slice >= 0 ? slice : 0, nt = slice >= 0 ? 1 : v.M;
    const size_t smem = (size_t)v.Ne * sizeof(float4);
    if (smem > 200 * 1024) return cudaErrorInvalidValue;   // one slice in shared memory
    {
        const cudaError_t ae = set_smem_limit(k_sep_hist, 200 * 1024);
        if (ae != cudaSuccess) return ae;
    }
    k_sep_hist<<<nt, kEstBlock, smem, s>>>(v, t0, dSep, d_hist);
    return cudaGetLastError();
}

// Winding and area sums of SuperfluidFractionEstimator::accumulate
// (estimator.cpp:2008-2036): W = sum of getVelocity over the active beads
// (path.h:189-203), Az and I from each bead and its next one.  Partial sums
// per CTA in a fixed order, then one CTA adds the partials in order, so the
// result does not depend on scheduling.
__global__ void __launch_bounds__(kEstBlock)
k_winding_partials(PathView v, double* __restrict__ part) {
    __shared__ double red[5][kEstBlock];
    double w0 = 0.0, w1 = 0.0, w2 = 0.0, az = 0.0, in = 0.0;
    const long long nb = (long long)v.M * v.Ne;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < nb;
         idx += (long long)gridDim.x * blockDim.x) {
        const int t = (int)(idx / v.Ne), p = (int)(idx - (long long)t * v.Ne);
        if (p >= v.nbs[t]) continue;
        const int2 nx = v.next[(size_t)t * v.Ne + p];
        if (nx.x < 0) continue;                              // getVelocity = 0, no area term
        const double* X = v.pos + (size_t)t * 3 * v.Ne;
        const double* Y = v.pos + (size_t)nx.x * 3 * v.Ne;
        const double p1x = X[p], p1y = X[v.Ne + p], p1z = X[2 * v.Ne + p];
        const double p2x = Y[nx.y], p2y = Y[v.Ne + nx.y], p2z = Y[2 * v.Ne + nx.y];
        w0 += min_image(p2x - p1x, v.side[0], v.sideInv[0]);
        w1 += min_image(p2y - p1y, v.side[1], v.sideInv[1]);
        w2 += min_image(p2z - p1z, v.side[2], v.sideInv[2]);
        az += p1x * p2y - p2x * p1y;
        in += p1x * p2x + p1y * p2y;
    }
    red[0][threadIdx.x] = w0; red[1][threadIdx.x] = w1; red[2][threadIdx.x] = w2;
    red[3][threadIdx.x] = az; red[4][threadIdx.x] = in;
    __syncthreads();
    for (int o = kEstBlock / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o)
            for (int k = 0; k < 5; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x < 5) part[(size_t)blockIdx.x * 5 + threadIdx.x] = red[threadIdx.x][0];
}

__global__ void k_winding_total(const double* __restrict__ part, int nblocks, double* __restrict__ out5) {
    if (threadIdx.x < 5) {
        double s = 0.0;
        for (int b = 0; b < nblocks; ++b) s += part[(size_t)b * 5 + threadIdx.x];
        out5[threadIdx.x] = s;
    }
}

constexpr int kWindBlocks = 152;

size_t winding_work_bytes() { return (size_t)kWindBlocks * 5 * sizeof(double) + 5 * sizeof(double); }

cudaError_t launch_winding(const PathView& v, double* d_work, double* d_out5, cudaStream_t s) {
    k_winding_partials<<<kWindBlocks, kEstBlock, 0, s>>>(v, d_work);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_winding_total<<<1, 32, 0, s>>>(d_work, kWindBlocks, d_out5);
    return cudaGetLastError();
}

// Cycle lengths of PermutationCycleEstimator::accumulate
// (estimator.cpp:2735-2781): one thread per active bead of slice 0 walks
// its worldline through the next links.  The reference counts a cycle at
// its first slice-0 bead in index order, i.e. at the smallest one, so each
// thread counts its cycle only if it met no smaller slice-0 bead.  A walk
// is bounded by M * Ne steps (a longer one is not a cycle: -1).
__global__ void k_cycles(PathView v, int* __restrict__ len_out) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    const int nw = v.nbs[0];
    if (n >= nw) return;
    const long long limit = (long long)v.M * v.Ne;
    int2 b = make_int2(0, n);
    long long wl = 0;
    bool smallest = true, closed = false;
    do {
        ++wl;
        if (b.x == 0 && b.y < n) smallest = false;
        b = v.next[(size_t)b.x * v.Ne + b.y];
        if (b.x < 0) break;                                  // open worldline
        if (b.x == 0 && b.y == n) { closed = true; break; }
    } while (wl <= limit);
    len_out[n] = (closed && smallest) ? (int)wl : (closed ? 0 : -1);
}

cudaError_t launch_cycles(const PathView& v, int nw, int* d_len, cudaStream_t s) {
    if (nw <= 0) return cudaSuccess;
    k_cycles<<<(nw + 127) / 128, 128, 0, s>>>(v, d_len);
    return cudaGetLastError();
}

// Beads of slice 0 inside the cylinder x^2 + y^2 < maxR2: num1DParticles
// (estimator.cpp:4318-4327), one CTA, a fixed-order count.
__global__ void k_count_inside(PathView v, double maxR2, int* __restrict__ out) {
    __shared__ int red[kEstBlock];
    int c = 0;
    const int n = v.nbs[0];
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        const double x = v.pos[j], y = v.pos[v.Ne + j];
        c += (x * x + y * y < maxR2) ? 1 : 0;
    }
    red[threadIdx.x] = c;
    __syncthreads();
    for (int o = kEstBlock / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[0] = red[0];
}

cudaError_t launch_count_inside(const PathView& v, double maxR2, int* d_out, cudaStream_t s) {
    k_count_inside<<<1, kEstBlock, 0, s>>>(v, maxR2, d_out);
    return cudaGetLastError();
}

}  // namespace pgb
