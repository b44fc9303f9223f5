// fp64_kernels.cu -- the FP64 "plain form" kernels.
//
// Compiled with -fmad=false: every multiply and add rounds once, in the order
// the reference writes it, so each pair term equals the oracle's bit for bit
// and totals differ only through summation order (parallel reductions).
#include "pgb_device.cuh"

namespace pgb {

// ---------------------------------------------------------------------------
// Aziz functions for the tables (src/potential.cpp:1821-1907 and the F, dF,
// d2F helpers of include/potential.h:963-983).
// ---------------------------------------------------------------------------
struct AzizD {
    double rm, A, epsilon, alpha, beta, D, C6, C8, C10;
    __device__ double F(double x) const { return (x < D ? exp(-(D/x - 1.0)*(D/x - 1.0)) : 1.0); }
    __device__ double dF(double x) const {
        double ix = 1.0/x;
        double r = 2.0*D*ix*ix*(D*ix-1.0)*exp(-(D*ix - 1.0)*(D*ix - 1.0));
        return (x < D ? r : 0.0);
    }
    __device__ double d2F(double x) const {
        double ix = 1.0/x;
        double r = 2.0*D*ix*ix*ix*( 2.0*D*D*D*ix*ix*ix - 4.0*D*D*ix*ix
                - D*ix + 2.0) * exp(-(D*ix - 1.0)*(D*ix - 1.0));
        return (x < D ? r : 0.0);
    }
    __device__ double V(double r) const {
        double x = r / rm;
        double Urep = A * exp(-alpha*x + beta*x*x);
        if (x < kEPS) return 0.0;
        else if (x < 0.01) return (epsilon * Urep);
        double ix2 = 1.0 / (x * x);
        double ix6 = ix2 * ix2 * ix2;
        double ix8 = ix6 * ix2;
        double ix10 = ix8 * ix2;
        double Uatt = -( C6*ix6 + C8*ix8 + C10*ix10 ) * F(x);
        return ( epsilon * (Urep + Uatt) );
    }
    __device__ double dVdr(double r) const {
        double x = r / rm;
        double T1 = A * (-alpha + 2.0*beta*x) * exp(-alpha*x + beta*x*x);
        if (x < kEPS) return 0.0;
        else if (x < 0.01) return ( ( epsilon / rm ) * T1 );
        double ix = 1.0 / x;
        double ix2 = ix*ix;
        double ix6 = ix2 * ix2 * ix2;
        double ix7 = ix6 * ix;
        double ix8 = ix6 * ix2;
        double ix9 = ix8 * ix;
        double ix10 = ix8 * ix2;
        double ix11 = ix10 * ix;
        double T2 = ( 6.0*C6*ix7 + 8.0*C8*ix9 + 10.0*C10*ix11 ) * F(x);
        double T3 = -( C6*ix6 + C8*ix8 + C10*ix10 ) * dF(x);
        return ( ( epsilon / rm ) * (T1 + T2 + T3) );
    }
    __device__ double d2Vdr2(double r) const {
        double x = r / rm;
        double abFactor2 = (alpha - 2.0*beta*x)*(alpha-2.0*beta*x);
        double T1 = A * (2*beta + abFactor2) * exp(-alpha*x + beta*x*x);
        if (x < kEPS) return 0.0;
        else if (x < 0.01) return ( ( epsilon / rm ) * T1 );
        double ix = 1.0 / x;
        double ix2 = ix*ix;
        double ix6 = ix2 * ix2 * ix2;
        double ix7 = ix6 * ix;
        double ix8 = ix6 * ix2;
        double ix9 = ix8 * ix;
        double ix10 = ix8 * ix2;
        double ix11 = ix10 * ix;
        double ix12 = ix11 * ix;
        double T2 = - ( 42.0*C6*ix8 + 72.0*C8*ix10 + 110.0*C10*ix12 ) * F(x);
        double T3 = 2.0*( 6.0*C6*ix7 + 8.0*C8*ix9 + 10.0*C10*ix11 ) * dF(x);
        double T4 = - ( C6*ix6 + C8*ix8 + C10*ix10 ) * d2F(x);
        return ( ( epsilon / (rm*rm) ) * (T1 + T2 + T3 + T4) );
    }
};

__global__ void k_build_tables(const double* __restrict__ r, int n, AzizD az,
                               double* tV, double* tdV, double* td2V) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double x = r[i];
        tV[i] = az.V(x);
        tdV[i] = az.dVdr(x);
        td2V[i] = az.d2Vdr2(x);
    }
}

cudaError_t launch_build_tables(const double* d_r, int n, AzizParams a,
                                double* tV, double* tdV, double* td2V, cudaStream_t s) {
    AzizD az{a.rm, a.A, a.epsilon, a.alpha, a.beta, a.D, a.C6, a.C8, a.C10};
    int blocks = (n + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    if (blocks < 1) blocks = 1;
    k_build_tables<<<blocks, 256, 0, s>>>(d_r, n, az, tV, tdV, td2V);
    return cudaGetLastError();
}

// PotentialBase::V(const dVec*, double*, int) and gradV/grad2V, batched.
__global__ void k_potential_batch64(PathView v, const double* __restrict__ sep,
                                    double* out, int n, int what) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double3 d = make_double3(sep[3*i], sep[3*i+1], sep[3*i+2]);
        if (what == 0) out[i] = V64(v, d);
        else if (what == 1) { double3 g = gradV64(v, d); out[3*i] = g.x; out[3*i+1] = g.y; out[3*i+2] = g.z; }
        else out[i] = grad2V64(v, d);
    }
}

cudaError_t launch_potential_batch64(const PathView& v, const double* d_sep,
                                     double* d_out, int n, int what, cudaStream_t s) {
    int blocks = (n + 255) / 256;
    if (blocks > 152 * 8) blocks = 152 * 8;
    if (blocks < 1) blocks = 1;
    k_potential_batch64<<<blocks, 256, 0, s>>>(v, d_sep, d_out, n, what);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Per-bead potential action, one CTA per bead.
//
// Phase 1 builds the LookupTable interaction list of the bead (every active
// bead of the same slice, other than itself, with |r2 - r1|^2 < rc^2;
// lookuptable.cpp:464-516) in particle order, and sums Vnn
// (action.cpp:1044-1060).  Phase 2 evaluates gradVnnSquared
// (action.cpp:1282-1337): one thread per list member b2 accumulates
// F3 = sum_{b3 in list, b3 != b2} gradV(r2 - r3) from shared memory.
// ---------------------------------------------------------------------------
constexpr int kBeadBlock = 256;

__global__ void __launch_bounds__(kBeadBlock)
k_bead_actions64(PathView v, const int2* __restrict__ beads, int k, int shift, int mode,
                 double tau, double lambda, double vf0, double vf1, double gf0,
                 double gf1, const double* __restrict__ over, double* __restrict__ out) {
    extern __shared__ double smem[];
    const int Ne = v.Ne;
    double* lx = smem;
    double* ly = lx + Ne;
    double* lz = ly + Ne;
    int* lid = reinterpret_cast<int*>(lz + Ne);
    __shared__ double red[kBeadBlock / 32];
    __shared__ int wcount[kBeadBlock / 32];
    __shared__ int s_total;

    const int b = blockIdx.x;
    const int s = beads[b].x, p = beads[b].y;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    if (s < 0 || s >= v.M || p < 0 || p >= Ne || !v.on[(size_t)s * Ne + p]) {
        if (tid == 0) out[b] = 0.0;
        return;
    }
    const int eo = s % 2;
    const double vf = eo ? vf1 : vf0;
    const double gf = eo ? gf1 : gf0;
    const double t = (double)shift * tau;
    const bool need_v = (mode != PGB_ACTION_CORR);
    const bool need_c = (mode == PGB_ACTION_CORR) ? (gf > kEPS)
                      : (mode == PGB_ACTION_FULL) ? (shift == 1 && gf > kEPS) : false;

    const double* X = v.pos + (size_t)s * 3 * Ne;
    // `over` (trial positions) replaces the bead's stored position
    const double x1 = over ? over[3 * b] : X[p];
    const double y1 = over ? over[3 * b + 1] : X[Ne + p];
    const double z1 = over ? over[3 * b + 2] : X[2 * Ne + p];
    const int st1 = bead_state(v, s, p);
    if (tid == 0) s_total = 0;
    __syncthreads();

    double vsum = 0.0;
    for (int base = 0; base < Ne; base += kBeadBlock) {
        int j = base + tid;
        bool in = false;
        double dx = 0, dy = 0, dz = 0;
        if (j < Ne && j != p && v.on[(size_t)s * Ne + j]) {
            // LookupTable stores sep = getSeparation(bead2, bead1) = r2 - r1
            dx = min_image(X[j] - x1, v.side[0], v.sideInv[0]);
            dy = min_image(X[Ne + j] - y1, v.side[1], v.sideInv[1]);
            dz = min_image(X[2 * Ne + j] - z1, v.side[2], v.sideInv[2]);
            double3 d = make_double3(dx, dy, dz);
            if (dot3(d, d) < v.rc2) {
                in = true;
                if (need_v) vsum += pair_factor(st1, bead_state(v, s, j)) * V64(v, d);
            }
        }
        unsigned m = __ballot_sync(0xffffffffu, in);
        if (lane == 0) wcount[w] = __popc(m);
        __syncthreads();
        int off = s_total;
        for (int i = 0; i < w; ++i) off += wcount[i];
        if (in) {
            int pos = off + __popc(m & ((1u << lane) - 1u));
            lx[pos] = X[j]; ly[pos] = X[Ne + j]; lz[pos] = X[2 * Ne + j];
            lid[pos] = j;
        }
        __syncthreads();
        if (tid == 0) { int tot = 0; for (int i = 0; i < kBeadBlock / 32; ++i) tot += wcount[i]; s_total += tot; }
        __syncthreads();
    }
    const int nlist = s_total;
    double Vnn = 0.0;
    if (need_v) Vnn = 0.0 + block_sum(vsum, red);   // totVext (0, free) + totVint

    double corr_g = 0.0;
    if (need_c) {
        double tsum = 0.0, f1x = 0.0, f1y = 0.0, f1z = 0.0;
        for (int n = tid; n < nlist; n += kBeadBlock) {
            double x2 = lx[n], y2 = ly[n], z2 = lz[n];
            double3 d12 = make_double3(min_image(x2 - x1, v.side[0], v.sideInv[0]),
                                       min_image(y2 - y1, v.side[1], v.sideInv[1]),
                                       min_image(z2 - z1, v.side[2], v.sideInv[2]));
            double3 F2 = gradV64(v, d12);
            f1x -= F2.x; f1y -= F2.y; f1z -= F2.z;
            double3 F3 = make_double3(0.0, 0.0, 0.0);
            for (int m2 = 0; m2 < nlist; ++m2) {
                if (m2 == n) continue;
                double3 d23 = make_double3(min_image(x2 - lx[m2], v.side[0], v.sideInv[0]),
                                           min_image(y2 - ly[m2], v.side[1], v.sideInv[1]),
                                           min_image(z2 - lz[m2], v.side[2], v.sideInv[2]));
                double3 g = gradV64(v, d23);
                F3.x += g.x; F3.y += g.y; F3.z += g.z;
            }
            double3 Z = make_double3(0.0, 0.0, 0.0);
            tsum += dot3(F2, F2) + 2.0 * dot3(Z, F2) + 2.0 * dot3(F2, F3);
        }
        double T = block_sum(tsum, red);
        double Fx = block_sum(f1x, red), Fy = block_sum(f1y, red), Fz = block_sum(f1z, red);
        double3 Fint1 = make_double3(Fx, Fy, Fz);
        double3 Z = make_double3(0.0, 0.0, 0.0);
        corr_g = T + (dot3(Z, Z) + 2.0 * dot3(Z, Fint1) + dot3(Fint1, Fint1));
    }
    if (tid == 0) {
        double bareU = vf * t * Vnn;
        double corU = need_c ? gf * t * t * t * lambda * corr_g : 0.0;
        double U;
        if (mode == PGB_ACTION_BARE) U = bareU;
        else if (mode == PGB_ACTION_CORR) U = corU;
        else U = bareU + corU;
        out[b] = U;
    }
}

cudaError_t launch_bead_actions64(const PathView& v, const int2* d_beads, int k, int shift,
                                  int mode, double tau, double lambda, const double vf[2],
                                  const double gf[2], const double* d_over, double* d_out,
                                  cudaStream_t s) {
    if (k <= 0) return cudaSuccess;
    size_t smem = (size_t)v.Ne * (3 * sizeof(double) + sizeof(int));
    {
        const cudaError_t ae = set_smem_limit(k_bead_actions64, 200 * 1024);
        if (ae != cudaSuccess) return ae;
    }
    k_bead_actions64<<<k, kBeadBlock, smem, s>>>(v, d_beads, k, shift, mode, tau, lambda,
                                                 vf[0], vf[1], gf[0], gf[1], d_over, d_out);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Per-slice terms of the estimators, one CTA per slice, one thread per bead
// b1 < numBeadsAtSlice (looping when there are more beads than threads).
//   vint: LocalAction::V(slice)            action.cpp:902-947 (i<j, sep r2-r1)
//   g2:   gradVSquared(slice)              action.cpp:1188-1223
//   r1,d1: rDOTgradUterm1/deltadotgradUterm1 sums (action.cpp:1446,1588)
//   r2,d2: T-matrix terms of rDOTgradUterm2/deltadotgradUterm2 (1503,1700)
//   kin:  sum |getVelocity|^2                path.h:189-203
//   xch:  sum (r_{t+W}-r_t).(r_{t+1}-r_t)     estimator.cpp:1138-1152
// Output layout: terms[q * M + t] for q = 0..7 in the order above.
// ---------------------------------------------------------------------------
constexpr int kSliceBlock = 128;

__device__ __forceinline__ double3 pos64(const PathView& v, int s, int p) {
    const double* X = v.pos + (size_t)s * 3 * v.Ne;
    return make_double3(X[p], X[v.Ne + p], X[2 * v.Ne + p]);
}
__device__ __forceinline__ double3 sepb(const PathView& v, int2 a, int2 b) {
    double3 ra = pos64(v, a.x, a.y), rb = pos64(v, b.x, b.y);
    return make_double3(min_image(ra.x - rb.x, v.side[0], v.sideInv[0]),
                        min_image(ra.y - rb.y, v.side[1], v.sideInv[1]),
                        min_image(ra.z - rb.z, v.side[2], v.sideInv[2]));
}
__device__ __forceinline__ double3 velocity64(const PathView& v, int s, int p) {
    int2 n = v.next[(size_t)s * v.Ne + p];
    if (n.x == kXXX && n.y == kXXX) return make_double3(0.0, 0.0, 0.0);
    return sepb(v, n, make_int2(s, p));
}

__global__ void __launch_bounds__(kSliceBlock)
k_slice_terms64(PathView v, int window, int want_tmat, double* __restrict__ terms) {
    extern __shared__ double sm[];
    const int s = blockIdx.x;
    const int Ne = v.Ne;
    const int n = v.nbs[s];
    double* sx = sm;
    double* sy = sx + Ne;
    double* sz = sy + Ne;
    __shared__ double red[kSliceBlock / 32];
    const double* X = v.pos + (size_t)s * 3 * Ne;
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        sx[j] = X[j]; sy[j] = X[Ne + j]; sz[j] = X[2 * Ne + j];
    }
    __syncthreads();

    double a_vint = 0, a_g2 = 0, a_r1 = 0, a_r2 = 0, a_d1 = 0, a_d2 = 0, a_kin = 0, a_xch = 0;
    for (int b1 = threadIdx.x; b1 < n; b1 += blockDim.x) {
        const double x1 = sx[b1], y1 = sy[b1], z1 = sz[b1];
        const int st1 = bead_state(v, s, b1);
        double3 F = make_double3(0.0, 0.0, 0.0);
        double T[3][3] = {{0,0,0},{0,0,0},{0,0,0}};
        for (int b2 = 0; b2 < n; ++b2) {
            if (b2 == b1) continue;
            double3 rD = make_double3(min_image(x1 - sx[b2], v.side[0], v.sideInv[0]),
                                      min_image(y1 - sy[b2], v.side[1], v.sideInv[1]),
                                      min_image(z1 - sz[b2], v.side[2], v.sideInv[2]));
            double3 g = gradV64(v, rD);
            F.x += g.x; F.y += g.y; F.z += g.z;
            if (want_tmat) {
                double rmag = sqrt(dot3(rD, rD));
                double dVi = sqrt(dot3(g, g));
                double g2Vi = grad2V64(v, rD);
                double dV = dVi + 0.0;
                double d2V = g2Vi + 0.0;
                double r3 = pow(rmag, 3);
                double rr[3] = {rD.x, rD.y, rD.z};
                #pragma unroll
                for (int a = 0; a < 3; ++a)
                    #pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        T[a][c] += rr[a]*rr[c]*d2V/(rmag*rmag) - rr[a]*rr[c]*dV/r3;
                        if (a == c) T[a][c] += dV/rmag;
                    }
            }
            if (b2 > b1) {
                // V(slice) uses sep = getSeparation(bead2, bead1) = r2 - r1
                double3 d21 = make_double3(min_image(sx[b2] - x1, v.side[0], v.sideInv[0]),
                                           min_image(sy[b2] - y1, v.side[1], v.sideInv[1]),
                                           min_image(sz[b2] - z1, v.side[2], v.sideInv[2]));
                a_vint += pair_factor(st1, bead_state(v, s, b2)) * V64(v, d21);
            }
        }
        double3 r1v = make_double3(x1, y1, z1);
        a_g2 += dot3(F, F);
        a_r1 += dot3(F, r1v);
        double3 TF = make_double3(0.0, 0.0, 0.0);
        if (want_tmat) {
            double ip0 = 0.0; ip0 += T[0][0]*F.x; ip0 += T[0][1]*F.y; ip0 += T[0][2]*F.z;
            double ip1 = 0.0; ip1 += T[1][0]*F.x; ip1 += T[1][1]*F.y; ip1 += T[1][2]*F.z;
            double ip2 = 0.0; ip2 += T[2][0]*F.x; ip2 += T[2][1]*F.y; ip2 += T[2][2]*F.z;
            TF = make_double3(0.0 + ip0, 0.0 + ip1, 0.0 + ip2);
            a_r2 += dot3(TF, r1v);
        }
        // centroid deviation delta (action.cpp:1625-1645)
        if (window > 0) {
            double3 rm_ = make_double3(0,0,0), rl_ = make_double3(0,0,0), com = make_double3(0,0,0);
            int2 bn = make_int2(s, b1), bp = make_int2(s, b1);
            int2 nOld = bn, pOld = bp;
            for (int gm = 0; gm < window; ++gm) {
                // next(bead1, gamma) / prev(bead1, gamma)
                int2 cn = make_int2(s, b1), cp = make_int2(s, b1);
                for (int q = 0; q < gm; ++q) cn = v.next[(size_t)cn.x * Ne + cn.y];
                for (int q = 0; q < gm; ++q) cp = v.prev[(size_t)cp.x * Ne + cp.y];
                double3 a = sepb(v, cn, nOld), c = sepb(v, cp, pOld);
                rm_.x += a.x; rm_.y += a.y; rm_.z += a.z;
                rl_.x += c.x; rl_.y += c.y; rl_.z += c.z;
                com.x += (x1 + rm_.x) + (x1 + rl_.x);
                com.y += (y1 + rm_.y) + (y1 + rl_.y);
                com.z += (z1 + rm_.z) + (z1 + rl_.z);
                nOld = cn; pOld = cp;
            }
            double den = 2.0 * window;
            double3 dl = make_double3(min_image(x1 - com.x / den, v.side[0], v.sideInv[0]),
                                      min_image(y1 - com.y / den, v.side[1], v.sideInv[1]),
                                      min_image(z1 - com.z / den, v.side[2], v.sideInv[2]));
            a_d1 += dot3(F, dl);
            if (want_tmat) a_d2 += dot3(TF, dl);
            // virial exchange term: vel1 = sum_{g=1..W} sep(next^g, next^{g-1})
            double3 vel1 = make_double3(0,0,0);
            int2 o = make_int2(s, b1), c2 = o;
            for (int gm = 1; gm <= window; ++gm) {
                c2 = v.next[(size_t)c2.x * Ne + c2.y];
                double3 a = sepb(v, c2, o);
                vel1.x += a.x; vel1.y += a.y; vel1.z += a.z;
                o = c2;
            }
            double3 vel2 = velocity64(v, s, b1);
            a_xch += dot3(vel1, vel2);
        }
        double3 vel = velocity64(v, s, b1);
        a_kin += dot3(vel, vel);
    }
    double vals[8] = {a_vint, a_g2, a_r1, a_r2, a_d1, a_d2, a_kin, a_xch};
    #pragma unroll
    for (int q = 0; q < 8; ++q) {
        double t = block_sum(vals[q], red);
        if (threadIdx.x == 0) terms[(size_t)q * v.M + s] = t;
    }
}

cudaError_t launch_slice_terms64(const PathView& v, int window, int want_tmat,
                                 double* d_terms, cudaStream_t s) {
    size_t smem = (size_t)v.Ne * 3 * sizeof(double);
    {
        const cudaError_t ae = set_smem_limit(k_slice_terms64, 200 * 1024);
        if (ae != cudaSuccess) return ae;
    }
    k_slice_terms64<<<v.M, kSliceBlock, smem, s>>>(v, window, want_tmat, d_terms);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// rho_q(t) = sum_j exp(i q . r_j(t)) in FP64 (raw positions, as gpu_isf uses
// raw bead coordinates).  One warp per (q, t).
// ---------------------------------------------------------------------------
__global__ void k_rhoq64(PathView v, const double* __restrict__ q, int nq, double maxR2,
                         double* __restrict__ rho) {
    int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    int total = nq * v.M;
    if (gw >= total) return;
    int iq = gw / v.M, t = gw % v.M;
    double qx = q[3*iq], qy = q[3*iq+1], qz = q[3*iq+2];
    const double* X = v.pos + (size_t)t * 3 * v.Ne;
    int n = v.nbs[t];
    double re = 0.0, im = 0.0;
    for (int j = lane; j < n; j += 32) {
        // cylinder restriction: only beads with x^2 + y^2 < maxR^2
        if (maxR2 > 0.0 && !(X[j] * X[j] + X[v.Ne + j] * X[v.Ne + j] < maxR2)) continue;
        double ph = 0.0;
        ph += qx * X[j]; ph += qy * X[v.Ne + j]; ph += qz * X[2 * v.Ne + j];
        double sn, cs;
        sincos(ph, &sn, &cs);
        re += cs; im += sn;
    }
    re = warp_sum(re); im = warp_sum(im);
    if (lane == 0) { rho[2 * (size_t)gw] = re; rho[2 * (size_t)gw + 1] = im; }
}

cudaError_t launch_rhoq64(const PathView& v, const double* d_q, int nq, double* d_rho,
                          cudaStream_t s, double maxR2) {
    long long warps = (long long)nq * v.M;
    int blocks = (int)((warps * 32 + 255) / 256);
    if (blocks < 1) return cudaSuccess;
    k_rhoq64<<<blocks, 256, 0, s>>>(v, d_q, nq, maxR2, d_rho);
    return cudaGetLastError();
}

// F(q,tau) = norm * sum_t Re(rho_t conj(rho_{t+tau})), tau in [0, M/2]
__global__ void k_isf_direct64(const double* __restrict__ rho, int nq, int M, double norm,
                               double* __restrict__ out) {
    int nt = M / 2 + 1;
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= (long long)nq * nt) return;
    int iq = (int)(i / nt), tau = (int)(i % nt);
    const double* r = rho + (size_t)iq * M * 2;
    double acc = 0.0;
    for (int t = 0; t < M; ++t) {
        int t2 = t + tau; if (t2 >= M) t2 -= M;
        acc += r[2*t] * r[2*t2] + r[2*t+1] * r[2*t2+1];
    }
    out[i] = acc * norm;
}

cudaError_t launch_isf_direct64(const double* d_rho, int nq, int M, double norm,
                                double* d_out, cudaStream_t s) {
    long long n = (long long)nq * (M / 2 + 1);
    int blocks = (int)((n + 255) / 256);
    if (blocks < 1) return cudaSuccess;
    k_isf_direct64<<<blocks, 256, 0, s>>>(d_rho, nq, M, norm, d_out);
    return cudaGetLastError();
}

__global__ void k_ssf_from_rho64(const double* __restrict__ rho, int nq, int M, double norm,
                                 double* __restrict__ out) {
    int iq = blockIdx.x;
    __shared__ double red[8];
    double acc = 0.0;
    for (int t = threadIdx.x; t < M; t += blockDim.x) {
        double a = rho[((size_t)iq * M + t) * 2], b = rho[((size_t)iq * M + t) * 2 + 1];
        acc += a * a + b * b;
    }
    double s = block_sum(acc, red);
    if (threadIdx.x == 0) out[iq] = s * norm;
}

cudaError_t launch_ssf_from_rho64(const double* d_rho, int nq, int M, double norm,
                                  double* d_out, cudaStream_t s) {
    if (nq <= 0) return cudaSuccess;
    k_ssf_from_rho64<<<nq, 256, 0, s>>>(d_rho, nq, M, norm, d_out);
    return cudaGetLastError();
}

}  // namespace pgb
