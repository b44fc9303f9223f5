// pgb_internal.h -- shared host/device definitions of the GB300 hot-path
// library.  Host code only sees plain pointers; kernels take a PathView.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "pimc_gb300.h"

namespace pgb {

constexpr double kEPS = 1.0e-7;   // include/common.h:89 (EPS)
constexpr int kXXX = -1;          // include/common.h:93 (XXX)

// Aziz HFD-HE2 parameters (src/potential.cpp:1749-1788)
struct AzizParams {
    double rm, A, epsilon, alpha, beta, D, C6, C8, C10;
};
AzizParams aziz_params(int year);
// message returned by pgb_last_error(NULL) on this host thread
void set_global_error(const std::string& msg);
// Raise func's dynamic shared-memory limit to bytes on the current device.
// The attribute belongs to the device's context, so it is set once per
// (kernel, device) pair, under a process-wide lock, and its return code is
// passed back; a failure is not recorded, so the next call tries again.
cudaError_t set_smem_limit(const void* func, int bytes);
template <class F>
cudaError_t set_smem_limit(F* func, int bytes) { return set_smem_limit(reinterpret_cast<const void*>(func), bytes); }
// Prefer a shared-memory carveout of `percent` (0..100) of the SM's unified
// L1/shared storage for func on the current device, once per (kernel, device)
cudaError_t set_carveout(const void* func, int percent);
template <class F>
cudaError_t set_carveout(F* func, int percent) { return set_carveout(reinterpret_cast<const void*>(func), percent); }

// Read-only view of one path handed to kernels by value.
struct PathView {
    int M, Ne;
    double side[3], sideInv[3];
    double rc2;
    // FP64 positions, slice-major SoA: x at pos[(s*3+0)*Ne + p]
    const double* pos;
    const float4* pos32;        // FP32 mirror [M][Ne] (w unused)
    const int2* next;           // [M][Ne] (slice, ptcl)
    const int2* prev;
    const uint8_t* on;          // [M][Ne]
    const int* nbs;             // numBeadsAtSlice [M]
    int worm[8];                // head, tail, special1, special2
    // FP64 direct-lookup tables
    const double* tV;
    const double* tdV;
    const double* td2V;
    double dr;
    int tableLength;
};

struct Ctx {
    pgb_params p{};
    AzizParams az{};
    cudaStream_t stream = nullptr;
    std::string err;
    int M = 0, Ne = 0;
    // tables
    double dr = 0, tailV = 0, maxSep = 0;
    int tableLength = 0;
    double *d_tV = nullptr, *d_tdV = nullptr, *d_td2V = nullptr;
    // path
    double* d_pos = nullptr;      // SoA [M][3][Ne]
    float4* d_pos32 = nullptr;
    int2 *d_next = nullptr, *d_prev = nullptr;
    uint8_t* d_on = nullptr;
    int* d_nbs = nullptr;
    std::vector<int> h_nbs;
    std::vector<int32_t> h_next, h_prev;   // host copies for range walks
    std::vector<uint8_t> h_on;
    int worm[8] = {-1,-1,-1,-1,-1,-1,-1,-1};
    int numBeadsOn = 0;
    bool loaded = false;
    // scratch (grown on demand)
    void* d_scratch = nullptr; size_t scratch_bytes = 0;
    void* d_tc_tables = nullptr;   // split-BF16 DFT and cosine matrices of this M (built once)
    float4* d_force32 = nullptr;   // per-bead same-slice forces of the current configuration
    bool force_valid = false;      // cleared by every position change
    void* h_pinned = nullptr; size_t pinned_bytes = 0;
    // plain-form worm state: the LookupTable's per-slice lists of a single
    // grid box (their order decides swap pivots) and the Worm scalars
    std::vector<std::vector<int>> lk_hash;
    std::vector<int> lk_label;
    bool lk_valid = false;
    bool w_diag = true;
    int w_gap = -1, w_length = 0;
    double w_sep[3] = {0.0, 0.0, 0.0};
    // plain-form generator state (MT19937)
    std::vector<uint32_t> mt_state;
    int mt_left = 0, mt_pos = 0;
    bool mt_seeded = false;

    PathView view() const;
    int fail(int code, const std::string& msg) { err = msg; return code; }
    int cuda_fail(cudaError_t e, const char* where);
    int ensure_scratch(size_t bytes);
    int ensure_pinned(size_t bytes);
};

// Write the listed beads (linear index s*Ne + p) from the host mirrors
// (h_next, h_prev, h_on; positions from pos_aos [M][Ne][3]) and numBeadsAtSlice
// to the device; synchronous.
int upload_beads(Ctx& c, const int* lin, int k, const double* pos_aos);

#define PGB_CUDA(ctx, call)                                              \
    do {                                                                 \
        cudaError_t e__ = (call);                                        \
        if (e__ != cudaSuccess) return (ctx)->cuda_fail(e__, #call);     \
    } while (0)

// ---- kernel launchers (implemented in the .cu files) ----
// fp64_kernels.cu (compiled with -fmad=false: IEEE mul/add, no fusion)
cudaError_t launch_build_tables(const double* d_r, int n, AzizParams az,
                                double* tV, double* tdV, double* td2V,
                                cudaStream_t s);
cudaError_t launch_potential_batch64(const PathView& v, const double* d_sep,
                                     double* d_out, int n, int what,
                                     cudaStream_t s);
cudaError_t launch_bead_actions64(const PathView& v, const int2* d_beads, int k,
                                  int shift, int mode, double tau, double lambda,
                                  const double vf[2], const double gf[2],
                                  const double* d_over, double* d_out, cudaStream_t s);
cudaError_t launch_slice_terms64(const PathView& v, int window, int want_tmat,
                                 double* d_terms /* [8][M] */, cudaStream_t s);
// maxR2 > 0: only beads with x^2 + y^2 < maxR2 (cylinder estimators)
cudaError_t launch_rhoq64(const PathView& v, const double* d_q, int nq,
                          double* d_rho /* [q][M][2] */, cudaStream_t s, double maxR2 = 0.0);
cudaError_t launch_isf_direct64(const double* d_rho, int nq, int M, double norm,
                                double* d_out, cudaStream_t s);
// mixed_kernels.cu (FP32 pairs, FP64 accumulation)
cudaError_t launch_bead_actions32(const PathView& v, AzizParams az,
                                  const int2* d_beads, int k, int shift, int mode,
                                  double tau, double lambda, const double vf[2],
                                  const double gf[2], const double* d_over, double* d_out,
                                  cudaStream_t s, const float4* d_force = nullptr);
// one warp per bead, every active same-slice bead in the list; delta = 1 with
// d_over writes U(trial) - U(current)
cudaError_t launch_bead_actions32_full(const PathView& v, AzizParams az, const int2* d_beads, int k,
                                       int shift, int mode, double tau, double lambda,
                                       const double vf[2], const double gf[2], const double* d_over,
                                       const float4* d_force, int delta, double* d_out,
                                       cudaStream_t s);
// F[t][b] = sum over active b3 != b of gradV(r_b - r_b3) on slice t, FP32 [M][Ne]
cudaError_t launch_slice_forces32(const PathView& v, AzizParams az, float4* d_force, cudaStream_t s);
cudaError_t launch_slice_terms32(const PathView& v, AzizParams az, int window,
                                 double* d_terms, cudaStream_t s);
cudaError_t launch_pos32_from64(const PathView& v, float4* d_pos32,
                                cudaStream_t s);
// scatter.cu
// d_work: rhoq32_work_bytes(v) of scratch for the slices as box fractions;
// d_rho must hold nq*M*16 bytes (the second half keeps the wave-vector table)
size_t rhoq32_work_bytes(const PathView& v);
cudaError_t launch_rhoq32(const PathView& v, const double* d_q, int nq,
                          float2* d_rho /* [q][M] */, void* d_work, cudaStream_t s,
                          double maxR2 = 0.0);
cudaError_t launch_ssf_from_rho32(const float2* d_rho, int nq, int M,
                                  double norm, double* d_out, cudaStream_t s);
cudaError_t launch_ssf_from_rho64(const double* d_rho, int nq, int M,
                                  double norm, double* d_out, cudaStream_t s);
cudaError_t launch_isf_direct32(const float2* d_rho, int nq, int M, double norm,
                                double* d_out, cudaStream_t s);
// path_estimators.cu (g(r), winding, permutation cycles; FP64, -fmad=false)
cudaError_t launch_sep_hist(const PathView& v, int slice, unsigned long long* d_hist, cudaStream_t s);
size_t winding_work_bytes();
cudaError_t launch_winding(const PathView& v, double* d_work, double* d_out5, cudaStream_t s);
cudaError_t launch_cycles(const PathView& v, int nw, int* d_len, cudaStream_t s);
// slice-0 beads with x^2 + y^2 < maxR2 (one int)
cudaError_t launch_count_inside(const PathView& v, double maxR2, int* d_out, cudaStream_t s);
// isf_tc.cu (tcgen05 split-BF16 DFT correlation)
size_t isf_tc_scratch_bytes(int nq, int M);
size_t isf_tc_table_bytes(int M);
cudaError_t isf_tc_build_tables(int M, void* d_tables, cudaStream_t s);
cudaError_t launch_isf_tc(const float2* d_rho, int nq, int M, double norm,
                          double* d_out, void* d_scratch, const void* d_tables, cudaStream_t s);
bool isf_tc_supported(int M);
// the pipeline's error word (int, 0 or 1) at this offset of the scratch
size_t isf_tc_error_offset(int nq, int M);
// test switch: the first GEMM of later calls stalls before its last chunk
void isf_tc_set_stall_test(int on);

}  // namespace pgb

struct pgb_ctx { pgb::Ctx c; };
