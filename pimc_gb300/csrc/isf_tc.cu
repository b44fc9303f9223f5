// isf_tc.cu -- F(q,tau) slice correlation on the 5th-generation tensor cores.
//
// F(q,tau) = 1/(N M) sum_t Re[rho_q(t) conj(rho_q(t+tau))] is a circular
// correlation along imaginary time.  With X_q(w) = sum_t rho_q(t) e^{-2 pi i w t/M}
// (Wiener-Khinchin)
//     F(q,tau) = 1/(N M) * 1/M sum_w |X_q(w)|^2 cos(2 pi w tau / M),
// i.e. two GEMMs against fixed matrices:
//   GEMM 1  [Q x 2M] (Re rho | Im rho)  x  [2M x 2M] DFT  -> (Re X, Im X) interleaved,
//           epilogue P = (Re X)^2 + (Im X)^2            [Q x M]
//   GEMM 2  [Q x M] P  x  [M x (M/2+1)] cosines        -> F(q,tau)
// Both run as split-BF16 products, A = Ah + Al, B = Bh + Bl,
// A B ~ Ah Bh + Ah Bl + Al Bh, accumulated in FP32 in tensor memory.
//
// Kernel: one CTA of 128 threads per 128 x 256 output tile.  The prep
// kernels write every operand in tile order: the 64-wide K chunk of a tile is
// one contiguous block already in the canonical K-major core-matrix layout
// without swizzle (8 x 16-byte core matrices; LBO = 128 B between core
// matrices along K, SBO = 1024 B between 8-row groups), so one bulk copy
// (cp.async.bulk, completion counted on an mbarrier) moves it into shared
// memory.  Warp 0 lane 0 produces chunks into a two-stage ring, warp 1 lane 0
// issues the tcgen05.mma.kind::f16 instructions (M = 128, N = 256, K = 16)
// and releases each stage with tcgen05.commit; every wait is bounded.  The
// accumulator (128 lanes x 256 FP32 columns of TMEM) is read back with
// tcgen05.ld by all four warps.
#include <cuda_bf16.h>
#include <atomic>
#include <cstdint>

#include "pgb_device.cuh"

namespace pgb {

namespace {

constexpr int kTM = 128;          // rows per tile
constexpr int kTN = 256;          // columns per tile (TMEM columns)
constexpr int kTK = 64;           // K per staged chunk
constexpr int kThreads = 128;
constexpr uint32_t kTileA = kTM * kTK * 2;     // bytes of one bf16 A chunk
constexpr uint32_t kTileB = kTN * kTK * 2;     // bytes of one bf16 B chunk
constexpr int kStages = 2;
constexpr uint32_t kStageBytes = 2 * kTileA + 2 * kTileB;     // Ah, Al, Bh, Bl of one chunk
constexpr uint32_t kSmem = kStages * kStageBytes + 1024;
constexpr long long kMmaWaitLimit = 1LL << 24;
constexpr unsigned long long kWaitNs = 1000000000ull;   // one second of wall clock per wait

// Element index of (r, k) in a tile-ordered [rows x K] bf16 operand whose
// tiles are TR rows x 64 K: tile (r / TR, k / 64) is one contiguous block of
// TR * 64 elements in core-matrix order (8-row groups of 1024 B, 16-byte core
// rows, 128 B between core matrices along K).
__host__ __device__ __forceinline__ size_t tiled_index(int r, int k, int K, int TR) {
    const int rt = r / TR, rr = r - rt * TR, kc = k >> 6, kk = k & 63;
    return ((size_t)rt * (size_t)(K >> 6) + (size_t)kc) * (size_t)(TR * 64) +
           (size_t)((rr >> 3) * 512 + (kk >> 3) * 64 + (rr & 7) * 8 + (kk & 7));
}

__device__ __forceinline__ uint32_t su32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);          // start address
    d |= (uint64_t)(128u >> 4) << 16;                  // leading-dimension byte offset (K)
    d |= (uint64_t)(1024u >> 4) << 32;                 // stride-dimension byte offset (M/N)
    d |= (uint64_t)1 << 46;                            // descriptor version for tcgen05
    return d;                                          // base offset 0, no swizzle
}

// kind::f16 instruction descriptor: D = F32, A = B = BF16, both K-major,
// N = 256, M = 128
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kTN >> 3) << 17) |
                            ((uint32_t)(kTM >> 4) << 24);

__device__ __forceinline__ void mma_bf16(uint32_t tmem, uint64_t ad, uint64_t bd, uint32_t acc) {
    asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
                 :: "r"(tmem), "l"(ad), "l"(bd), "r"(kIdesc), "r"(acc) : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                 :: "r"(su32(bar)) : "memory");
}

__device__ __forceinline__ bool bar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}" : "=r"(ok) : "r"(su32(bar)), "r"(parity) : "memory");
    return ok != 0;
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
    uint32_t r[32];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 "
                 "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                 "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),
                   "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]),
                   "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]),
                   "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
                   "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]),
                   "=r"(r[30]), "=r"(r[31])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    #pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void bar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(su32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void bar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}"
                 :: "r"(su32(bar)), "r"(bytes) : "memory");
}


__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 :: "r"(su32(dst)), "l"(src), "r"(bytes), "r"(su32(bar)) : "memory");
}

__device__ __forceinline__ unsigned long long wall_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// a wait on an mbarrier phase that gives up after kMmaWaitLimit polls or
// kWaitNs of wall clock, whichever comes first (false: the phase did not
// complete)
__device__ __forceinline__ bool bar_wait_bounded(uint64_t* bar, uint32_t parity) {
    const unsigned long long t0 = wall_ns();
    long long n = 0;
    while (!bar_try_wait(bar, parity)) {
        if (++n > kMmaWaitLimit) return false;
        if ((n & 255) == 0 && wall_ns() - t0 > kWaitNs) return false;
    }
    return true;
}

// Split-BF16 GEMM  C[rows x cols] = A[rows x K] B[K x cols]; A and B^T
// [cols x K] tile-ordered (tiled_index with TR = 128 and 256), hi/lo parts.
// mode 0: interleaved (re, im) columns -> P[row][col/2] = re^2 + im^2
// mode 1: out[row][col] = scale * C  (FP64), for row < rows_valid, col < cols_valid
// stall_last: a test of the bounded waits.  The producer stops before the
// last chunk (no arrival, no copy), so the MMA thread's wait for that chunk
// runs out; every copy issued has been consumed, the CTA writes no output,
// sets *err, frees its TMEM and returns.
__global__ void __launch_bounds__(kThreads, 1)
k_gemm_split_bf16(const __nv_bfloat16* __restrict__ Ah, const __nv_bfloat16* __restrict__ Al,
                  const __nv_bfloat16* __restrict__ Bh, const __nv_bfloat16* __restrict__ Bl,
                  int K, int mode, float* __restrict__ P, int ldp, double* __restrict__ out,
                  int ldo, int rows_valid, int cols_valid, double scale, int* __restrict__ err,
                  int stall_last) {
    extern __shared__ __align__(1024) unsigned char smem[];
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + kStages * kStageBytes);
    uint64_t* empty = full + kStages;
    uint64_t* done = empty + kStages;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
    int* s_fail = reinterpret_cast<int*>(tmem_slot + 1);
    int* s_count = s_fail + 1;                 // [0] chunks issued, [1] chunks consumed
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int row0 = blockIdx.y * kTM, col0 = blockIdx.x * kTN;
    const int nk = K / kTK;
    const char* gAh = reinterpret_cast<const char*>(Ah) + (size_t)blockIdx.y * nk * kTileA;
    const char* gAl = reinterpret_cast<const char*>(Al) + (size_t)blockIdx.y * nk * kTileA;
    const char* gBh = reinterpret_cast<const char*>(Bh) + (size_t)blockIdx.x * nk * kTileB;
    const char* gBl = reinterpret_cast<const char*>(Bl) + (size_t)blockIdx.x * nk * kTileB;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     :: "r"(su32(tmem_slot)), "r"((uint32_t)kTN) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 32) {
        for (int st = 0; st < kStages; ++st) { bar_init(full + st, 1); bar_init(empty + st, 1); }
        bar_init(done, 1);
        *s_fail = 0;
        s_count[0] = s_count[1] = 0;
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            // producer: chunk c goes to stage c % kStages once the MMAs that
            // read the chunk before it there have completed
            int c = 0;
            for (; c < nk; ++c) {
                const int st = c % kStages;
                if (stall_last && c == nk - 1) break;
                if (c >= kStages && !bar_wait_bounded(empty + st, (uint32_t)((c / kStages - 1) & 1))) {
                    atomicExch(s_fail, 1);
                    break;
                }
                unsigned char* sA = smem + (size_t)st * kStageBytes;
                bar_expect_tx(full + st, kStageBytes);
                bulk_g2s(sA, gAh + (size_t)c * kTileA, kTileA, full + st);
                bulk_g2s(sA + kTileA, gAl + (size_t)c * kTileA, kTileA, full + st);
                bulk_g2s(sA + 2 * kTileA, gBh + (size_t)c * kTileB, kTileB, full + st);
                bulk_g2s(sA + 2 * kTileA + kTileB, gBl + (size_t)c * kTileB, kTileB, full + st);
            }
            s_count[0] = c;
        }
        __syncwarp();
    } else if (warp == 1) {
        if (lane == 0) {
            int c = 0;
            for (; c < nk; ++c) {
                const int st = c % kStages;
                if (!bar_wait_bounded(full + st, (uint32_t)((c / kStages) & 1))) {
                    atomicExch(s_fail, 1);
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t base = su32(smem + (size_t)st * kStageBytes);
                #pragma unroll
                for (int ks = 0; ks < kTK / 16; ++ks) {
                    const uint32_t ko = (uint32_t)(2 * ks) * 128u;
                    const uint64_t ah = smem_desc(base + ko), al = smem_desc(base + kTileA + ko);
                    const uint64_t bh = smem_desc(base + 2 * kTileA + ko);
                    const uint64_t bl = smem_desc(base + 2 * kTileA + kTileB + ko);
                    mma_bf16(tmem, ah, bh, (c > 0 || ks > 0) ? 1u : 0u);
                    mma_bf16(tmem, ah, bl, 1u);
                    mma_bf16(tmem, al, bh, 1u);
                }
                mma_commit(empty + st);        // the stage is free once these MMAs are done
            }
            s_count[1] = c;
            mma_commit(done);                  // tracks every MMA this thread issued
        }
        __syncwarp();
    }
    // everyone, once the producer and the MMA thread have stopped issuing:
    // the accumulator is complete (or the pipeline gave up)
    __syncthreads();
    const bool landed = bar_wait_bounded(done, 0u);
    if (!landed) atomicExch(s_fail, 1);
    __syncthreads();
    if (tid == 0) {
        // copies issued but never consumed must land before the CTA exits
        for (int c = s_count[1]; c < s_count[0]; ++c)
            if (!bar_wait_bounded(full + (c % kStages), (uint32_t)((c / kStages) & 1))) break;
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const bool ok = (*(volatile int*)s_fail == 0);
    if (!ok && tid == 0 && err) atomicExch(err, 1);
    if (ok) {
        const float scalef = (float)scale;
        // epilogue: warp w owns TMEM lanes 32w..32w+31 (rows)
        const int r = 32 * warp + lane;
        const int row = row0 + r;
        float v[32];
        for (int cc = 0; cc < kTN / 32; ++cc) {
            tmem_ld32(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(32 * cc), v);
            if (mode == 0) {
                const int w0 = (col0 + 32 * cc) >> 1;
                if (row < rows_valid) {
                    #pragma unroll
                    for (int j = 0; j < 16; ++j)
                        P[(size_t)row * ldp + w0 + j] = fmaf(v[2 * j], v[2 * j], v[2 * j + 1] * v[2 * j + 1]);
                }
            } else {
                // FP32 scale, FP64 result formed on the integer pipes
                if (row < rows_valid) {
                    #pragma unroll
                    for (int j = 0; j < 32; ++j) {
                        const int col = col0 + 32 * cc + j;
                        if (col < cols_valid) out[(size_t)row * ldo + col] = f32_to_f64_alu(scalef * v[j]);
                    }
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;"
                     :: "r"(tmem), "r"((uint32_t)kTN) : "memory");
}

__device__ __forceinline__ void split_bf16(float x, __nv_bfloat16& h, __nv_bfloat16& l) {
    h = __float2bfloat16_rn(x);
    l = __float2bfloat16_rn(x - __bfloat162float(h));
}

// A1 = (Re rho | Im rho), rows >= nq are zero
__global__ void k_prep_rho(const float2* __restrict__ rho, int nq, int M, int qpad,
                           __nv_bfloat16* Ah, __nv_bfloat16* Al) {
    const long long n = (long long)qpad * 2 * M;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const int q = (int)(i / (2 * M)), k = (int)(i % (2 * M));
        float x = 0.f;
        if (q < nq) { const float2 r = rho[(size_t)q * M + (k % M)]; x = (k < M) ? r.x : r.y; }
        const size_t o = tiled_index(q, k, 2 * M, kTM);
        split_bf16(x, Ah[o], Al[o]);
    }
}

// B1^T [2M cols][2M K]: col 2w -> Re X(w), col 2w+1 -> Im X(w)
__global__ void k_prep_dft(int M, __nv_bfloat16* Bh, __nv_bfloat16* Bl) {
    const long long n = (long long)4 * M * M;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(i / (2 * M)), k = (int)(i % (2 * M));
        const int w = c >> 1, t = k % M;
        const long long ph = ((long long)t * w) % M;
        double sn, cs;
        sincospi(2.0 * (double)ph / (double)M, &sn, &cs);
        double val;
        if ((c & 1) == 0) val = (k < M) ? cs : sn;      // Re X = sum Re(rho) cos + Im(rho) sin
        else              val = (k < M) ? -sn : cs;     // Im X = sum -Re(rho) sin + Im(rho) cos
        const size_t o = tiled_index(c, k, 2 * M, kTN);
        split_bf16((float)val, Bh[o], Bl[o]);
    }
}

// A2 = P [qpad x M] (row-major) -> tile order
__global__ void k_prep_p(const float* __restrict__ P, int qpad, int M, __nv_bfloat16* Ah,
                         __nv_bfloat16* Al) {
    const long long n = (long long)qpad * M;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const int q = (int)(i / M), w = (int)(i % M);
        const size_t o = tiled_index(q, w, M, kTM);
        split_bf16(P[i], Ah[o], Al[o]);
    }
}

// B2^T [colpad][M]: col tau -> cos(2 pi w tau / M), zero beyond M/2
__global__ void k_prep_cos(int M, int colpad, __nv_bfloat16* Bh, __nv_bfloat16* Bl) {
    const long long n = (long long)colpad * M;
    const int nt = M / 2 + 1;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const int tau = (int)(i / M), w = (int)(i % M);
        double val = 0.0;
        if (tau < nt) {
            const long long ph = ((long long)tau * w) % M;
            val = cospi(2.0 * (double)ph / (double)M);
        }
        const size_t o = tiled_index(tau, w, M, kTN);
        split_bf16((float)val, Bh[o], Bl[o]);
    }
}

inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// per-call scratch: the split rho matrix, P and its split, the error flag
struct Layout {
    int qpad, colpad2;
    size_t a1, p, a2, err, total;
};

Layout layout(int nq, int M) {
    Layout L;
    L.qpad = ((nq + kTM - 1) / kTM) * kTM;
    L.colpad2 = ((M / 2 + 1 + kTN - 1) / kTN) * kTN;
    size_t off = 0;
    L.a1 = off; off = align256(off + (size_t)L.qpad * 2 * M * 2 * sizeof(__nv_bfloat16));
    L.p = off;  off = align256(off + (size_t)L.qpad * M * sizeof(float));
    L.a2 = off; off = align256(off + (size_t)L.qpad * M * 2 * sizeof(__nv_bfloat16));
    L.err = off; off = align256(off + sizeof(int));
    L.total = off;
    return L;
}

// fixed matrices of one M: the DFT (B1) and the cosines (B2), each split
struct Tables {
    int colpad2;
    size_t b1, b2, total;
};

Tables tables(int M) {
    Tables T;
    T.colpad2 = ((M / 2 + 1 + kTN - 1) / kTN) * kTN;
    size_t off = 0;
    T.b1 = off; off = align256(off + (size_t)4 * M * M * 2 * sizeof(__nv_bfloat16));
    T.b2 = off; off = align256(off + (size_t)T.colpad2 * M * 2 * sizeof(__nv_bfloat16));
    T.total = off;
    return T;
}

}  // namespace

// the bounded-wait test switch (pgb_test_isf_tc_stall)
std::atomic<int> g_stall_test{0};

void isf_tc_set_stall_test(int on) { g_stall_test.store(on ? 1 : 0); }

size_t isf_tc_error_offset(int nq, int M) { return layout(nq, M).err; }

bool isf_tc_supported(int M) { return M >= 128 && M <= 2048 && (M % 128) == 0; }

size_t isf_tc_scratch_bytes(int nq, int M) { return layout(nq, M).total; }

size_t isf_tc_table_bytes(int M) { return tables(M).total; }

// The DFT and cosine matrices depend on M alone: a context builds them once
// (FP64 sincospi, then split to BF16 pairs) and every F(q,tau) reuses them.
cudaError_t isf_tc_build_tables(int M, void* d_tables, cudaStream_t s) {
    if (!isf_tc_supported(M)) return cudaErrorInvalidValue;
    const Tables T = tables(M);
    char* base = static_cast<char*>(d_tables);
    auto* b1h = reinterpret_cast<__nv_bfloat16*>(base + T.b1);
    auto* b1l = b1h + (size_t)4 * M * M;
    auto* b2h = reinterpret_cast<__nv_bfloat16*>(base + T.b2);
    auto* b2l = b2h + (size_t)T.colpad2 * M;
    k_prep_dft<<<152 * 4, 256, 0, s>>>(M, b1h, b1l);
    k_prep_cos<<<152 * 2, 256, 0, s>>>(M, T.colpad2, b2h, b2l);
    return cudaGetLastError();
}

cudaError_t launch_isf_tc(const float2* d_rho, int nq, int M, double norm, double* d_out,
                          void* d_scratch, const void* d_tables, cudaStream_t s) {
    if (!isf_tc_supported(M) || nq <= 0 || !d_tables) return cudaErrorInvalidValue;
    const int stall = g_stall_test.load();
    const Layout L = layout(nq, M);
    const Tables T = tables(M);
    char* base = static_cast<char*>(d_scratch);
    auto* a1h = reinterpret_cast<__nv_bfloat16*>(base + L.a1);
    auto* a1l = a1h + (size_t)L.qpad * 2 * M;
    const char* tb = static_cast<const char*>(d_tables);
    auto* b1h = reinterpret_cast<const __nv_bfloat16*>(tb + T.b1);
    auto* b1l = b1h + (size_t)4 * M * M;
    auto* P = reinterpret_cast<float*>(base + L.p);
    auto* a2h = reinterpret_cast<__nv_bfloat16*>(base + L.a2);
    auto* a2l = a2h + (size_t)L.qpad * M;
    auto* b2h = reinterpret_cast<const __nv_bfloat16*>(tb + T.b2);
    auto* b2l = b2h + (size_t)T.colpad2 * M;
    int* err = reinterpret_cast<int*>(base + L.err);
    {
        const cudaError_t ae = set_smem_limit(k_gemm_split_bf16, (int)kSmem);
        if (ae != cudaSuccess) return ae;
    }
    cudaMemsetAsync(err, 0, sizeof(int), s);
    k_prep_rho<<<152 * 4, 256, 0, s>>>(d_rho, nq, M, L.qpad, a1h, a1l);
    // GEMM 1: [qpad x 2M] x [2M x 2M] -> P [qpad x M]
    dim3 g1(2 * M / kTN, L.qpad / kTM);
    k_gemm_split_bf16<<<g1, kThreads, kSmem, s>>>(a1h, a1l, b1h, b1l, 2 * M, 0, P, M, nullptr, 0,
                                                  L.qpad, 2 * M, 0.0, err, stall);
    k_prep_p<<<152 * 4, 256, 0, s>>>(P, L.qpad, M, a2h, a2l);
    // GEMM 2: [qpad x M] x [M x colpad2] -> F [nq x (M/2+1)]
    dim3 g2(L.colpad2 / kTN, L.qpad / kTM);
    k_gemm_split_bf16<<<g2, kThreads, kSmem, s>>>(a2h, a2l, b2h, b2l, M, 1, nullptr, 0, d_out,
                                                  M / 2 + 1, nq, M / 2 + 1, norm / (double)M, err, 0);
    return cudaGetLastError();
}

}  // namespace pgb
