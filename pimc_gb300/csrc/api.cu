// api.cu -- host side of the C ABI: context, tables, worldline mirror,
// actions and estimator assembly.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "pgb_device.cuh"

namespace pgb {

AzizParams aziz_params(int year) {
    // src/potential.cpp:1749-1788
    if (year == 1987)
        return {2.9673, 1.8443101E5, 10.948, 10.43329537, -2.27965105, 1.4826,
                1.36745214, 0.42123807, 0.17473318};
    if (year == 1995)
        return {2.9683, 1.86924404E5, 10.956, 10.5717543, -2.07758779, 1.438,
                1.35186623, 0.4149514, 0.17151143};
    return {2.9673, 0.5448504E6, 10.8, 13.353384, 0.0, 1.241314, 1.3732412, 0.4253785, 0.1781};
}

PathView Ctx::view() const {
    PathView v;
    v.M = M; v.Ne = Ne;
    for (int i = 0; i < 3; ++i) { v.side[i] = p.side[i]; v.sideInv[i] = 1.0 / p.side[i]; }
    v.rc2 = p.rc * p.rc;
    v.pos = d_pos; v.pos32 = d_pos32; v.next = d_next; v.prev = d_prev; v.on = d_on;
    v.nbs = d_nbs;
    for (int i = 0; i < 8; ++i) v.worm[i] = worm[i];
    v.tV = d_tV; v.tdV = d_tdV; v.td2V = d_td2V; v.dr = dr; v.tableLength = tableLength;
    return v;
}

int Ctx::cuda_fail(cudaError_t e, const char* where) {
    err = std::string("CUDA error ") + cudaGetErrorString(e) + " at " + where;
    return e == cudaErrorMemoryAllocation ? PGB_ENOMEM : PGB_ECUDA;
}

int Ctx::ensure_scratch(size_t bytes) {
    if (bytes <= scratch_bytes) return PGB_OK;
    if (d_scratch) cudaFree(d_scratch);
    d_scratch = nullptr; scratch_bytes = 0;
    size_t b = std::max(bytes, (size_t)1 << 20);
    cudaError_t e = cudaMalloc(&d_scratch, b);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(scratch)");
    scratch_bytes = b;
    return PGB_OK;
}

int Ctx::ensure_pinned(size_t bytes) {
    if (bytes <= pinned_bytes) return PGB_OK;
    if (h_pinned) cudaFreeHost(h_pinned);
    h_pinned = nullptr; pinned_bytes = 0;
    size_t b = std::max(bytes, (size_t)1 << 20);
    cudaError_t e = cudaMallocHost(&h_pinned, b);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMallocHost(staging)");
    pinned_bytes = b;
    return PGB_OK;
}

// scatter (bead, position) updates into the SoA FP64 array and FP32 mirror
__global__ void k_update_beads(double* pos, float4* pos32, int Ne, const int2* beads,
                               const double* p, int k) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k) return;
    int2 b = beads[i];
    double* X = pos + (size_t)b.x * 3 * Ne;
    X[b.y] = p[3*i]; X[Ne + b.y] = p[3*i+1]; X[2 * Ne + b.y] = p[3*i+2];
    pos32[(size_t)b.x * Ne + b.y] = make_float4((float)p[3*i], (float)p[3*i+1], (float)p[3*i+2], 0.f);
}

// full bead records (position, links, active flag) into the device path
struct BeadRec { int s, p, ns, np, ps, pp, on, pad; double x, y, z; };
__global__ void k_set_beads(double* pos, float4* pos32, int2* nxt, int2* prv, uint8_t* on, int Ne,
                            const BeadRec* r, int k) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k) return;
    const BeadRec b = r[i];
    double* X = pos + (size_t)b.s * 3 * Ne;
    X[b.p] = b.x; X[Ne + b.p] = b.y; X[2 * Ne + b.p] = b.z;
    const size_t j = (size_t)b.s * Ne + b.p;
    pos32[j] = make_float4((float)b.x, (float)b.y, (float)b.z, 0.f);
    nxt[j] = make_int2(b.ns, b.np);
    prv[j] = make_int2(b.ps, b.pp);
    on[j] = (uint8_t)b.on;
}

// AoS [M][Ne][3] FP64 (the reference's bead array) -> SoA [M][3][Ne] and the
// float4 mirror, one bead per thread
__global__ void k_positions_from_aos(const double* __restrict__ aos, double* __restrict__ pos,
                                     float4* __restrict__ pos32, int M, int Ne) {
    const size_t n = (size_t)M * Ne;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        const size_t s = i / Ne, p = i - s * Ne;
        const double x = aos[3 * i], y = aos[3 * i + 1], z = aos[3 * i + 2];
        double* X = pos + s * 3 * Ne;
        X[p] = x; X[Ne + p] = y; X[2 * Ne + p] = z;
        pos32[i] = make_float4((float)x, (float)y, (float)z, 0.f);
    }
}

}  // namespace pgb

using namespace pgb;

namespace {

thread_local std::string g_last_error;

int check_ctx(pgb_ctx* c) { return c ? PGB_OK : PGB_EINVAL; }

int need_path(Ctx& c) {
    if (!c.loaded) return c.fail(PGB_ESTATE, "no path loaded (call pgb_load_path first)");
    return PGB_OK;
}

// True when the cutoff takes in every minimum-image separation, so that each
// bead's list is its whole slice (the reference default rc = L does).
bool full_list(const Ctx& c) {
    const double far2 = 0.25 * (c.p.side[0] * c.p.side[0] + c.p.side[1] * c.p.side[1] +
                                c.p.side[2] * c.p.side[2]);
    return c.p.rc * c.p.rc > far2;
}

// Same-slice forces for the O(n) gradient correction of the mixed form with
// full lists.  Returns the forces (valid until the next position change), or
// nullptr when the action has no gradient term or the lists are cut.
const float4* slice_forces(Ctx& c, int* rc) {
    *rc = PGB_OK;
    if (c.p.precision != PGB_MIXED) return nullptr;
    if (!(c.p.gradvfactor[0] > kEPS || c.p.gradvfactor[1] > kEPS)) return nullptr;
    if (!full_list(c)) return nullptr;
    if (!c.d_force32) {
        cudaError_t e = cudaMalloc(&c.d_force32, (size_t)c.M * c.Ne * sizeof(float4));
        if (e != cudaSuccess) { c.d_force32 = nullptr; *rc = c.cuda_fail(e, "cudaMalloc(slice forces)"); return nullptr; }
    }
    if (!c.force_valid) {
        cudaError_t e = launch_slice_forces32(c.view(), c.az, c.d_force32, c.stream);
        if (e != cudaSuccess) { *rc = c.cuda_fail(e, "slice forces launch"); return nullptr; }
        c.force_valid = true;
    }
    return c.d_force32;
}

// per-slice terms, internal layout [9][M]: vint g2 r1 r2 d1 d2 kin xch kinprev
int compute_terms(Ctx& c, std::vector<double>& h, bool want_tmat) {
    int rc = need_path(c); if (rc) return rc;
    size_t bytes = (size_t)8 * c.M * sizeof(double);
    rc = c.ensure_scratch(bytes); if (rc) return rc;
    double* d = static_cast<double*>(c.d_scratch);
    PathView v = c.view();
    int window = c.p.virial_window > 0 ? c.p.virial_window : 5;
    cudaError_t e = (c.p.precision == PGB_MIXED)
        ? launch_slice_terms32(v, c.az, window, d, c.stream)
        : launch_slice_terms64(v, window, want_tmat ? 1 : 0, d, c.stream);
    if (e != cudaSuccess) return c.cuda_fail(e, "slice terms launch");
    h.assign((size_t)8 * c.M, 0.0);
    PGB_CUDA(&c, cudaMemcpyAsync(h.data(), d, bytes, cudaMemcpyDeviceToHost, c.stream));
    PGB_CUDA(&c, cudaStreamSynchronize(c.stream));
    return PGB_OK;
}

}  // namespace

void pgb::set_global_error(const std::string& msg) { g_last_error = msg; }

cudaError_t pgb::set_carveout(const void* func, int percent) {
    static std::mutex mu;
    static std::map<std::pair<const void*, int>, int> done;   // (kernel, device) -> percent set
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lk(mu);
    auto it = done.find({func, dev});
    if (it != done.end() && it->second == percent) return cudaSuccess;
    e = cudaFuncSetAttribute(func, cudaFuncAttributePreferredSharedMemoryCarveout, percent);
    if (e != cudaSuccess) return e;
    done[{func, dev}] = percent;
    return cudaSuccess;
}

cudaError_t pgb::set_smem_limit(const void* func, int bytes) {
    static std::mutex mu;
    static std::map<std::pair<const void*, int>, int> done;   // (kernel, device) -> bytes set
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lk(mu);
    auto it = done.find({func, dev});
    if (it != done.end() && it->second >= bytes) return cudaSuccess;
    e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e != cudaSuccess) return e;
    done[{func, dev}] = bytes;
    return cudaSuccess;
}

extern "C" {

const char* pgb_last_error(const pgb_ctx* ctx) {
    if (ctx) return ctx->c.err.c_str();
    return g_last_error.c_str();
}

int pgb_device_info(char* name, int cap, int* sm_count, int* cc) {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        g_last_error = "no CUDA device available";
        return PGB_ECUDA;
    }
    cudaDeviceProp prop;
    e = cudaGetDeviceProperties(&prop, 0);
    if (e != cudaSuccess) { g_last_error = cudaGetErrorString(e); return PGB_ECUDA; }
    if (name && cap > 0) { std::strncpy(name, prop.name, cap - 1); name[cap - 1] = 0; }
    if (sm_count) *sm_count = prop.multiProcessorCount;
    if (cc) *cc = prop.major * 10 + prop.minor;
    return PGB_OK;
}

int pgb_create(const pgb_params* p, pgb_ctx** out) {
    if (!p || !out) { g_last_error = "null argument"; return PGB_EINVAL; }
    *out = nullptr;
    if (p->num_slices <= 0 || p->num_ptcl_ext <= 0 || p->tau <= 0 || p->lambda <= 0 ||
        p->rc <= 0 || p->side[0] <= 0 || p->side[1] <= 0 || p->side[2] <= 0) {
        g_last_error = "invalid parameters (sizes, tau, lambda, rc and sides must be > 0)";
        return PGB_EINVAL;
    }
    if (p->precision != PGB_FP64 && p->precision != PGB_MIXED) {
        g_last_error = "precision must be PGB_FP64 or PGB_MIXED"; return PGB_EINVAL;
    }
    if (p->num_ptcl_ext > 8192) { g_last_error = "num_ptcl_ext > 8192 not supported"; return PGB_EINVAL; }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        g_last_error = "no CUDA device available"; return PGB_ECUDA;
    }
    pgb_ctx* h = new pgb_ctx();
    Ctx& c = h->c;
    c.p = *p;
    c.M = p->num_slices; c.Ne = p->num_ptcl_ext;
    c.az = aziz_params(p->aziz_year);
    cudaError_t e = cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) { g_last_error = cudaGetErrorString(e); delete h; return PGB_ECUDA; }
    // table sizes (potential.cpp:1793-1796, container.cpp:100-103)
    double hx = p->side[0] / 2.0, hy = p->side[1] / 2.0, hz = p->side[2] / 2.0;
    double d2 = 0.0; d2 += hx * hx; d2 += hy * hy; d2 += hz * hz;
    c.maxSep = std::sqrt(d2);
    c.dr = (1.0E-6) * c.az.rm;
    c.tableLength = int(c.maxSep / c.dr);
    // tail correction (potential.cpp:1801-1806)
    double rmorc = c.az.rm / p->rc;
    double t2 = c.az.C6 * std::pow(rmorc, 3.0) / 3.0;
    double t3 = c.az.C8 * std::pow(rmorc, 5.0) / 5.0;
    double t4 = c.az.C10 * std::pow(rmorc, 7.0) / 7.0;
    c.tailV = 2.0 * M_PI * c.az.epsilon * (-c.az.rm * c.az.rm * c.az.rm * (t2 + t3 + t4));
    int rc = PGB_OK;
    size_t tb = (size_t)c.tableLength * sizeof(double);
    size_t nb = (size_t)c.M * c.Ne;
    do {
        if ((e = cudaMalloc(&c.d_tV, tb)) != cudaSuccess) break;
        if ((e = cudaMalloc(&c.d_tdV, tb)) != cudaSuccess) break;
        if ((e = cudaMalloc(&c.d_td2V, tb)) != cudaSuccess) break;
        if ((e = cudaMalloc(&c.d_pos, nb * 3 * sizeof(double))) != cudaSuccess) break;
        if ((e = cudaMalloc(&c.d_pos32, nb * sizeof(float4))) != cudaSuccess) break;
        if ((e = cudaMalloc(&c.d_next, nb * sizeof(int2))) != cudaSuccess) break;
        if ((e = cudaMalloc(&c.d_prev, nb * sizeof(int2))) != cudaSuccess) break;
        if ((e = cudaMalloc(&c.d_on, nb)) != cudaSuccess) break;
        if ((e = cudaMalloc(&c.d_nbs, c.M * sizeof(int))) != cudaSuccess) break;
    } while (0);
    if (e != cudaSuccess) { rc = c.cuda_fail(e, "cudaMalloc(context)"); g_last_error = c.err; pgb_destroy(h); return rc; }
    // The table abscissae accumulate r += dr sequentially (potential.h:176-183);
    // that sequence is formed here and the V, dV/dr, d2V/dr2 values are
    // evaluated on the device.
    rc = c.ensure_pinned(tb);
    if (rc) { g_last_error = c.err; pgb_destroy(h); return rc; }
    double* r = static_cast<double*>(c.h_pinned);
    double acc = 0.0;
    for (int n = 0; n < c.tableLength; ++n) { r[n] = acc; acc += c.dr; }
    rc = c.ensure_scratch(tb);
    if (rc) { g_last_error = c.err; pgb_destroy(h); return rc; }
    e = cudaMemcpyAsync(c.d_scratch, r, tb, cudaMemcpyHostToDevice, c.stream);
    if (e == cudaSuccess)
        e = launch_build_tables(static_cast<double*>(c.d_scratch), c.tableLength, c.az,
                                c.d_tV, c.d_tdV, c.d_td2V, c.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
    if (e != cudaSuccess) { rc = c.cuda_fail(e, "table build"); g_last_error = c.err; pgb_destroy(h); return rc; }
    c.h_nbs.assign(c.M, 0);
    *out = h;
    return PGB_OK;
}

int pgb_destroy(pgb_ctx* h) {
    if (!h) return PGB_OK;
    Ctx& c = h->c;
    if (c.stream) cudaStreamSynchronize(c.stream);
    cudaFree(c.d_tV); cudaFree(c.d_tdV); cudaFree(c.d_td2V);
    cudaFree(c.d_pos); cudaFree(c.d_pos32); cudaFree(c.d_next); cudaFree(c.d_prev);
    cudaFree(c.d_on); cudaFree(c.d_nbs);
    if (c.d_scratch) cudaFree(c.d_scratch);
    if (c.d_tc_tables) cudaFree(c.d_tc_tables);
    if (c.d_force32) cudaFree(c.d_force32);
    if (c.h_pinned) cudaFreeHost(c.h_pinned);
    if (c.stream) cudaStreamDestroy(c.stream);
    delete h;
    return PGB_OK;
}

void* pgb_stream(pgb_ctx* h) { return h ? (void*)h->c.stream : nullptr; }

int pgb_table_info(pgb_ctx* h, int* length, double* dr, double* tailV) {
    if (check_ctx(h)) return PGB_EINVAL;
    if (length) *length = h->c.tableLength;
    if (dr) *dr = h->c.dr;
    if (tailV) *tailV = h->c.tailV;
    return PGB_OK;
}

int pgb_copy_tables(pgb_ctx* h, double* V, double* dV, double* d2V) {
    if (check_ctx(h)) return PGB_EINVAL;
    Ctx& c = h->c;
    size_t tb = (size_t)c.tableLength * sizeof(double);
    if (V) PGB_CUDA(&c, cudaMemcpyAsync(V, c.d_tV, tb, cudaMemcpyDeviceToHost, c.stream));
    if (dV) PGB_CUDA(&c, cudaMemcpyAsync(dV, c.d_tdV, tb, cudaMemcpyDeviceToHost, c.stream));
    if (d2V) PGB_CUDA(&c, cudaMemcpyAsync(d2V, c.d_td2V, tb, cudaMemcpyDeviceToHost, c.stream));
    PGB_CUDA(&c, cudaStreamSynchronize(c.stream));
    return PGB_OK;
}

static int potential_batch(pgb_ctx* h, const double* sep, double* out, int n, int what) {
    if (check_ctx(h) || (n > 0 && (!sep || !out)) || n < 0) {
        if (h) h->c.err = "potential batch: bad arguments (count must be non-negative)";
        return PGB_EINVAL;
    }
    if (n == 0) return PGB_OK;
    Ctx& c = h->c;
    int outw = (what == 1) ? 3 : 1;
    size_t in_b = (size_t)n * 3 * sizeof(double), out_b = (size_t)n * outw * sizeof(double);
    int rc = c.ensure_scratch(in_b + out_b); if (rc) return rc;
    double* d_in = static_cast<double*>(c.d_scratch);
    double* d_out = d_in + (size_t)n * 3;
    PGB_CUDA(&c, cudaMemcpyAsync(d_in, sep, in_b, cudaMemcpyHostToDevice, c.stream));
    PGB_CUDA(&c, launch_potential_batch64(c.view(), d_in, d_out, n, what, c.stream));
    PGB_CUDA(&c, cudaMemcpyAsync(out, d_out, out_b, cudaMemcpyDeviceToHost, c.stream));
    PGB_CUDA(&c, cudaStreamSynchronize(c.stream));
    return PGB_OK;
}

int pgb_potential_batch(pgb_ctx* h, const double* sep, double* out, int n) { return potential_batch(h, sep, out, n, 0); }
int pgb_gradv_batch(pgb_ctx* h, const double* sep, double* out3, int n) { return potential_batch(h, sep, out3, n, 1); }
int pgb_grad2v_batch(pgb_ctx* h, const double* sep, double* out, int n) { return potential_batch(h, sep, out, n, 2); }

int pgb_load_path(pgb_ctx* h, const double* pos, const int32_t* next, const int32_t* prev,
                  const uint8_t* on, const int32_t* worm8) {
    if (check_ctx(h) || !pos || !next || !prev || !on) {
        if (h) h->c.err = "load_path: null array";
        return PGB_EINVAL;
    }
    Ctx& c = h->c;
    size_t nb = (size_t)c.M * c.Ne;
    for (size_t i = 0; i < nb * 2; i += 2) {
        int s = next[i], p = next[i + 1];
        if (!((s == kXXX && p == kXXX) || (s >= 0 && s < c.M && p >= 0 && p < c.Ne)))
            return c.fail(PGB_EINVAL, "load_path: next link out of range");
        s = prev[i]; p = prev[i + 1];
        if (!((s == kXXX && p == kXXX) || (s >= 0 && s < c.M && p >= 0 && p < c.Ne)))
            return c.fail(PGB_EINVAL, "load_path: prev link out of range");
    }
    int rc = c.ensure_pinned(nb * 3 * sizeof(double)); if (rc) return rc;
    double* soa = static_cast<double*>(c.h_pinned);
    for (int s = 0; s < c.M; ++s)
        for (int p = 0; p < c.Ne; ++p)
            for (int d = 0; d < 3; ++d)
                soa[((size_t)s * 3 + d) * c.Ne + p] = pos[((size_t)s * c.Ne + p) * 3 + d];
    PGB_CUDA(&c, cudaMemcpyAsync(c.d_pos, soa, nb * 3 * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    PGB_CUDA(&c, cudaStreamSynchronize(c.stream));
    c.h_next.assign(next, next + nb * 2);
    c.h_prev.assign(prev, prev + nb * 2);
    c.h_on.assign(on, on + nb);
    PGB_CUDA(&c, cudaMemcpyAsync(c.d_next, c.h_next.data(), nb * sizeof(int2), cudaMemcpyHostToDevice, c.stream));
    PGB_CUDA(&c, cudaMemcpyAsync(c.d_prev, c.h_prev.data(), nb * sizeof(int2), cudaMemcpyHostToDevice, c.stream));
    PGB_CUDA(&c, cudaMemcpyAsync(c.d_on, c.h_on.data(), nb, cudaMemcpyHostToDevice, c.stream));
    c.numBeadsOn = 0;
    for (int s = 0; s < c.M; ++s) {
        int cnt = 0;
        for (int p = 0; p < c.Ne; ++p) cnt += c.h_on[(size_t)s * c.Ne + p] ? 1 : 0;
        c.h_nbs[s] = cnt;
        c.numBeadsOn += cnt;
    }
    PGB_CUDA(&c, cudaMemcpyAsync(c.d_nbs, c.h_nbs.data(), c.M * sizeof(int), cudaMemcpyHostToDevice, c.stream));
    for (int i = 0; i < 8; ++i) c.worm[i] = worm8 ? worm8[i] : kXXX;
    PGB_CUDA(&c, launch_pos32_from64(c.view(), c.d_pos32, c.stream));
    PGB_CUDA(&c, cudaStreamSynchronize(c.stream));
    c.loaded = true;
    c.force_valid = false;
    c.lk_valid = false;
    return PGB_OK;
}

int pgb_update_positions(pgb_ctx* h, const double* pos) {
    if (check_ctx(h) || !pos) return PGB_EINVAL;
    Ctx& c = h->c;
    int rc = need_path(c); if (rc) return rc;
    const size_t nb = (size_t)c.M * c.Ne, bytes = nb * 3 * sizeof(double);
    rc = c.ensure_scratch(bytes); if (rc) return rc;
    PGB_CUDA(&c, cudaMemcpyAsync(c.d_scratch, pos, bytes, cudaMemcpyHostToDevice, c.stream));
    const int blocks = (int)std::min<size_t>((nb + 255) / 256, 152 * 16);
    k_positions_from_aos<<<blocks, 256, 0, c.stream>>>(static_cast<const double*>(c.d_scratch), c.d_pos,
                                                       c.d_pos32, c.M, c.Ne);
    PGB_CUDA(&c, cudaGetLastError());
    c.force_valid = false;
    return PGB_OK;
}

int pgb_load_positions_device_async(pgb_ctx* h, const double* d_pos) {
    if (check_ctx(h) || !d_pos) return PGB_EINVAL;
    Ctx& c = h->c;
    size_t nb = (size_t)c.M * c.Ne;
    PGB_CUDA(&c, cudaMemcpyAsync(c.d_pos, d_pos, nb * 3 * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
    PGB_CUDA(&c, launch_pos32_from64(c.view(), c.d_pos32, c.stream));
    c.force_valid = false;
    return PGB_OK;
}

int pgb_update_beads(pgb_ctx* h, const int32_t* beads, const double* pos, int k) {
    if (check_ctx(h) || k < 0 || (k > 0 && (!beads || !pos))) return PGB_EINVAL;
    Ctx& c = h->c;
    int rc = need_path(c); if (rc) return rc;
    if (k == 0) return PGB_OK;
    for (int i = 0; i < k; ++i)
        if (beads[2*i] < 0 || beads[2*i] >= c.M || beads[2*i+1] < 0 || beads[2*i+1] >= c.Ne)
            return c.fail(PGB_EINVAL, "update_beads: bead out of range");
    size_t bb = (size_t)k * sizeof(int2), pb = (size_t)k * 3 * sizeof(double);
    rc = c.ensure_scratch(bb + pb + 64); if (rc) return rc;
    rc = c.ensure_pinned(bb + pb + 64); if (rc) return rc;
    char* hp = static_cast<char*>(c.h_pinned);
    std::memcpy(hp, beads, bb);
    std::memcpy(hp + bb, pos, pb);
    char* dp = static_cast<char*>(c.d_scratch);
    PGB_CUDA(&c, cudaMemcpyAsync(dp, hp, bb + pb, cudaMemcpyHostToDevice, c.stream));
    k_update_beads<<<(k + 127) / 128, 128, 0, c.stream>>>(c.d_pos, c.d_pos32, c.Ne,
        reinterpret_cast<const int2*>(dp), reinterpret_cast<const double*>(dp + bb), k);
    PGB_CUDA(&c, cudaGetLastError());
    PGB_CUDA(&c, cudaStreamSynchronize(c.stream));
    c.force_valid = false;
    return PGB_OK;
}

int pgb_set_beads(pgb_ctx* h, const int32_t* beads, const double* pos, const int32_t* next,
                  const int32_t* prev, const uint8_t* on, int k) {
    if (check_ctx(h) || k < 0 || (k > 0 && (!beads || !pos || !next || !prev || !on))) return PGB_EINVAL;
    Ctx& c = h->c;
    int rc = need_path(c); if (rc) return rc;
    auto okb = [&](int s, int p) { return (s == kXXX && p == kXXX) || (s >= 0 && s < c.M && p >= 0 && p < c.Ne); };
    for (int i = 0; i < k; ++i)
        if (beads[2*i] < 0 || beads[2*i] >= c.M || beads[2*i+1] < 0 || beads[2*i+1] >= c.Ne ||
            !okb(next[2*i], next[2*i+1]) || !okb(prev[2*i], prev[2*i+1]))
            return c.fail(PGB_EINVAL, "set_beads: bead or link out of range");
    std::vector<int> lin((size_t)k);
    std::vector<double> aos((size_t)c.M * c.Ne * 3, 0.0);
    // numBeadsAtSlice: the active beads of a slice must stay packed at its
    // front; checked on a copy so that a refused update changes nothing
    std::vector<uint8_t> on2 = c.h_on;
    for (int i = 0; i < k; ++i) on2[(size_t)beads[2*i] * c.Ne + beads[2*i+1]] = on[i] ? 1 : 0;
    std::vector<int> nbs2(c.M);
    int total = 0;
    for (int s = 0; s < c.M; ++s) {
        int cnt = 0;
        for (int p = 0; p < c.Ne; ++p) cnt += on2[(size_t)s * c.Ne + p] ? 1 : 0;
        for (int p = 0; p < c.Ne; ++p)
            if ((p < cnt) != (on2[(size_t)s * c.Ne + p] != 0))
                return c.fail(PGB_ESTATE, "set_beads: active beads of a slice must be packed at its front");
        nbs2[s] = cnt;
        total += cnt;
    }
    for (int i = 0; i < k; ++i) {
        const size_t j = (size_t)beads[2*i] * c.Ne + beads[2*i+1];
        lin[i] = (int)j;
        c.h_next[2*j] = next[2*i]; c.h_next[2*j+1] = next[2*i+1];
        c.h_prev[2*j] = prev[2*i]; c.h_prev[2*j+1] = prev[2*i+1];
        for (int d = 0; d < 3; ++d) aos[3*j + d] = pos[3*i + d];
    }
    c.h_on.swap(on2);
    c.h_nbs = nbs2;
    c.numBeadsOn = total;
    c.lk_valid = false;
    return upload_beads(c, lin.data(), k, aos.data());
}

int pgb_set_worm(pgb_ctx* h, const int32_t* worm8) {
    if (check_ctx(h) || !worm8) return PGB_EINVAL;
    Ctx& c = h->c;
    for (int i = 0; i < 8; i += 2)
        if (!((worm8[i] == kXXX && worm8[i+1] == kXXX) ||
              (worm8[i] >= 0 && worm8[i] < c.M && worm8[i+1] >= 0 && worm8[i+1] < c.Ne)))
            return c.fail(PGB_EINVAL, "set_worm: locator out of range");
    for (int i = 0; i < 8; ++i) c.worm[i] = worm8[i];
    c.lk_valid = false;
    c.force_valid = false;
    return PGB_OK;
}

int pgb_get_path(pgb_ctx* h, int32_t* next, int32_t* prev, uint8_t* on, int32_t* worm8) {
    if (check_ctx(h) || !next || !prev || !on || !worm8) return PGB_EINVAL;
    Ctx& c = h->c;
    int rc = need_path(c); if (rc) return rc;
    const size_t nb = (size_t)c.M * c.Ne;
    std::memcpy(next, c.h_next.data(), nb * 2 * sizeof(int32_t));
    std::memcpy(prev, c.h_prev.data(), nb * 2 * sizeof(int32_t));
    std::memcpy(on, c.h_on.data(), nb);
    for (int i = 0; i < 8; ++i) worm8[i] = c.worm[i];
    return PGB_OK;
}

int pgb_get_positions(pgb_ctx* h, double* pos) {
    if (check_ctx(h) || !pos) return PGB_EINVAL;
    Ctx& c = h->c;
    size_t nb = (size_t)c.M * c.Ne;
    int rc = c.ensure_pinned(nb * 3 * sizeof(double)); if (rc) return rc;
    double* soa = static_cast<double*>(c.h_pinned);
    PGB_CUDA(&c, cudaMemcpyAsync(soa, c.d_pos, nb * 3 * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    PGB_CUDA(&c, cudaStreamSynchronize(c.stream));
    for (int s = 0; s < c.M; ++s)
        for (int p = 0; p < c.Ne; ++p)
            for (int d = 0; d < 3; ++d)
                pos[((size_t)s * c.Ne + p) * 3 + d] = soa[((size_t)s * 3 + d) * c.Ne + p];
    return PGB_OK;
}

int pgb_bead_actions(pgb_ctx* h, const int32_t* beads, int k, int shift, int mode,
                     double* out_per_bead, double* out_sum) {
    if (check_ctx(h)) return PGB_EINVAL;
    Ctx& c = h->c;
    if (k < 0 || (k > 0 && !beads) || shift < 1 || mode < 0 || mode > 2)
        return c.fail(PGB_EINVAL, "bead_actions: bad arguments");
    int rc = need_path(c); if (rc) return rc;
    if (k == 0) { if (out_sum) *out_sum = 0.0; return PGB_OK; }
    for (int i = 0; i < k; ++i)
        if (beads[2*i] < 0 || beads[2*i] >= c.M || beads[2*i+1] < 0 || beads[2*i+1] >= c.Ne)
            return c.fail(PGB_EINVAL, "bead_actions: bead out of range");
    size_t bb = (size_t)k * sizeof(int2), ob = (size_t)k * sizeof(double);
    rc = c.ensure_scratch(bb + ob + 64); if (rc) return rc;
    rc = c.ensure_pinned(bb + ob + 64); if (rc) return rc;
    char* hp = static_cast<char*>(c.h_pinned);
    std::memcpy(hp, beads, bb);
    char* dp = static_cast<char*>(c.d_scratch);
    int2* d_b = reinterpret_cast<int2*>(dp);
    double* d_o = reinterpret_cast<double*>(dp + ((bb + 15) & ~(size_t)15));
    PGB_CUDA(&c, cudaMemcpyAsync(dp, hp, bb, cudaMemcpyHostToDevice, c.stream));
    PathView v = c.view();
    const float4* fall = slice_forces(c, &rc);
    if (rc) return rc;
    cudaError_t e = (c.p.precision != PGB_MIXED)
        ? launch_bead_actions64(v, d_b, k, shift, mode, c.p.tau, c.p.lambda,
                                c.p.vfactor, c.p.gradvfactor, nullptr, d_o, c.stream)
        : full_list(c)
        ? launch_bead_actions32_full(v, c.az, d_b, k, shift, mode, c.p.tau, c.p.lambda,
                                     c.p.vfactor, c.p.gradvfactor, nullptr, fall, 0, d_o, c.stream)
        : launch_bead_actions32(v, c.az, d_b, k, shift, mode, c.p.tau, c.p.lambda,
                                c.p.vfactor, c.p.gradvfactor, nullptr, d_o, c.stream, fall);
    if (e != cudaSuccess) return c.cuda_fail(e, "bead actions launch");
    double* ho = reinterpret_cast<double*>(hp + ((bb + 15) & ~(size_t)15));
    PGB_CUDA(&c, cudaMemcpyAsync(ho, d_o, ob, cudaMemcpyDeviceToHost, c.stream));
    PGB_CUDA(&c, cudaStreamSynchronize(c.stream));
    double tot = 0.0;
    for (int i = 0; i < k; ++i) tot += ho[i];
    if (out_per_bead) std::memcpy(out_per_bead, ho, ob);
    if (out_sum) *out_sum = tot;
    return PGB_OK;
}

int pgb_range_action(pgb_ctx* h, int s0, int p0, int s1, int p1, int shift, double* out) {
    if (check_ctx(h) || !out) return PGB_EINVAL;
    Ctx& c = h->c;
    int rc = need_path(c); if (rc) return rc;
    if (s0 < 0 || s0 >= c.M || p0 < 0 || p0 >= c.Ne || s1 < 0 || s1 >= c.M || p1 < 0 || p1 >= c.Ne)
        return c.fail(PGB_EINVAL, "range_action: bead out of range");
    // walk next links from start to end inclusive (action.cpp:532-541)
    size_t ie = ((size_t)s1 * c.Ne + p1) * 2;
    int stop_s = c.h_next[ie], stop_p = c.h_next[ie + 1];
    std::vector<int32_t> list;
    int s = s0, p = p0;
    long long guard = 0, lim = (long long)c.M * c.Ne + 1;
    do {
        if (s < 0 || p < 0) return c.fail(PGB_EINVAL, "range_action: broken link inside range");
        if (c.h_on[(size_t)s * c.Ne + p]) { list.push_back(s); list.push_back(p); }
        size_t i = ((size_t)s * c.Ne + p) * 2;
        s = c.h_next[i]; p = c.h_next[i + 1];
        if (++guard > lim) return c.fail(PGB_EINVAL, "range_action: end bead not reachable");
    } while (!(s == stop_s && p == stop_p));
    return pgb_bead_actions(h, list.data(), (int)list.size() / 2, shift, PGB_ACTION_FULL, nullptr, out);
}

int pgb_full_action(pgb_ctx* h, double* out) {
    if (check_ctx(h) || !out) return PGB_EINVAL;
    Ctx& c = h->c;
    std::vector<double> t;
    int rc = compute_terms(c, t, false); if (rc) return rc;
    double totU = 0.0, tt = c.p.tau;
    for (int s = 0; s < c.M; ++s) {
        int eo = s % 2;
        totU += c.p.vfactor[eo] * tt * (0.0 + 0.0 + t[s]);
        if (c.p.gradvfactor[eo] > kEPS)
            totU += c.p.gradvfactor[eo] * tt * tt * tt * c.p.lambda * t[(size_t)c.M + s];
    }
    *out = totU;
    return PGB_OK;
}

int pgb_kinetic_action(pgb_ctx* h, double* out) {
    if (check_ctx(h) || !out) return PGB_EINVAL;
    Ctx& c = h->c;
    std::vector<double> t;
    int rc = compute_terms(c, t, false); if (rc) return rc;
    // each link is counted from both of its beads (action.cpp:306-323)
    double totK = 0.0;
    for (int s = 0; s < c.M; ++s) totK += 2.0 * t[(size_t)6 * c.M + s];
    *out = totK / (4.0 * c.p.lambda * c.p.tau);
    return PGB_OK;
}

int pgb_slice_terms_compute(pgb_ctx* h, pgb_slice_terms* o) {
    if (check_ctx(h) || !o) return PGB_EINVAL;
    Ctx& c = h->c;
    std::vector<double> t;
    bool tm = (o->r2 || o->d2);
    int rc = compute_terms(c, t, tm); if (rc) return rc;
    double* dst[8] = {o->vint, o->g2, o->r1, o->r2, o->d1, o->d2, o->kin, o->xch};
    for (int q = 0; q < 8; ++q)
        if (dst[q]) std::memcpy(dst[q], t.data() + (size_t)q * c.M, c.M * sizeof(double));
    return PGB_OK;
}

// EnergyEstimator::accumulate (estimator.cpp:940-1029) from per-slice sums.
int pgb_energy(pgb_ctx* h, double out[9]) {
    if (check_ctx(h) || !out) return PGB_EINVAL;
    Ctx& c = h->c;
    std::vector<double> t;
    int rc = compute_terms(c, t, false); if (rc) return rc;
    const int M = c.M;
    const double tau = c.p.tau, lambda = c.p.lambda;
    const double* vint = t.data();
    const double* g2 = t.data() + M;
    const double* kin = t.data() + 6 * (size_t)M;
    int numParticles = c.numBeadsOn / M;
    double volume = c.p.side[0] * c.p.side[1] * c.p.side[2];
    double tailV = (1.0 * numParticles * numParticles / volume) * c.tailV;
    double kinNorm = (0.25 / (lambda * tau)) / (tau * M);
    double classicalKinetic = (0.5 * 3 / tau) * numParticles;
    double totK = 0.0;
    for (int s = 0; s < M; ++s) totK -= kin[s];
    totK *= kinNorm;
    double t1 = 0.0, t2 = 0.0, vop0 = 0.0, vop1 = 0.0;
    int period = c.p.period > 0 ? c.p.period : 1;
    for (int s = 0; s < M; ++s) {
        int eo = s % 2;
        double dl = (c.p.gradvfactor[eo] > kEPS) ? c.p.gradvfactor[eo] * tau * tau * tau * g2[s] : 0.0;
        double dt = c.p.vfactor[eo] * (0.0 + 0.0 + vint[s]);
        if (c.p.gradvfactor[eo] > kEPS) dt += 3.0 * c.p.gradvfactor[eo] * tau * tau * lambda * g2[s];
        t1 += 1.0 * dl;
        t2 += 1.0 * dt;
        if (!(s % period)) { vop0 += 1.0 * 0.0; vop1 += 1.0 * vint[s]; }
    }
    t1 *= lambda / (tau * M);
    t2 /= 1.0 * M;
    int nper = M / period;
    vop0 /= nper; vop1 /= nper;
    totK += (classicalKinetic + t1);
    double totV = t2 - t1 + tailV;
    vop1 += tailV;
    out[0] = totK; out[1] = totV; out[2] = vop0; out[3] = vop1;
    out[4] = totK + totV; out[5] = totK + totV - c.p.mu * numParticles;
    if (numParticles > 0) {
        out[6] = totK / (1.0 * numParticles); out[7] = totV / (1.0 * numParticles);
        out[8] = (totK + totV) / (1.0 * numParticles);
    } else out[6] = out[7] = out[8] = 0.0;
    return PGB_OK;
}

// VirialEnergyEstimator::accumulate (estimator.cpp:1086-1252)
int pgb_virial(pgb_ctx* h, int quirk, double est[19]) {
    if (check_ctx(h) || !est) return PGB_EINVAL;
    Ctx& c = h->c;
    std::vector<double> t;
    int rc = compute_terms(c, t, true); if (rc) return rc;
    const int M = c.M;
    const double* vint = t.data();
    const double* g2 = t.data() + M;
    const double* r1 = t.data() + 2 * (size_t)M;
    const double* r2 = t.data() + 3 * (size_t)M;
    const double* d1 = t.data() + 4 * (size_t)M;
    const double* d2 = t.data() + 5 * (size_t)M;
    const double* kin = t.data() + 6 * (size_t)M;
    const double* xch = t.data() + 7 * (size_t)M;
    const double tau = c.p.tau, lambda = c.p.lambda;
    const double* VF = c.p.vfactor;
    const double* gF = c.p.gradvfactor;
    for (int i = 0; i < 19; ++i) est[i] = 0.0;
    int numParticles = c.numBeadsOn / M;
    double beta = 1.0 * M * tau;
    int W = c.p.virial_window > 0 ? c.p.virial_window : 5;
    double volume = c.p.side[0] * c.p.side[1] * c.p.side[2];
    double tailV = (1.0 * numParticles * numParticles / volume) * c.tailV;
    double thermTerm1 = (0.5 * 3 / tau) * numParticles;
    double T1 = 0.5 * 3 * numParticles / (1.0 * W * tau);
    double exchangeNorm = 1.0 / (4.0 * W * std::pow(tau, 2) * lambda * M);
    double Pressure = 3 * numParticles;
    double T2 = 0.0, thermE = 0.0;
    for (int s = 0; s < M; ++s) { T2 -= xch[s]; thermE -= kin[s]; }
    double P2 = thermE;
    T2 *= exchangeNorm;
    P2 /= (2.0 * lambda * tau * M);
    Pressure += P2;
    double T3 = 0.0, T4 = 0.0, T5 = 0.0, virKinTerm = 0.0, totVop = 0.0, P3 = 0.0;
    for (int s = 0; s < M; ++s) {
        int eo = s % 2;
        bool cor = gF[eo] > kEPS;
        double t3 = std::pow(tau, 3);
        T3 += VF[eo] * tau * d1[s];
        T4 += cor ? d2[s] * (2.0 * gF[eo] * t3 * lambda) : 0.0;
        double dt = VF[eo] * (0.0 + 0.0 + vint[s]);
        if (cor) dt += 3.0 * gF[eo] * tau * tau * lambda * g2[s];
        T5 += dt;
        virKinTerm += cor ? (0.0 + g2[s]) * (gF[eo] * t3 * lambda) : 0.0;
        if (eo == 0) totVop += (0.0 + 0.0 + vint[s]);
        P3 += VF[eo] * tau * r1[s] + (cor ? r2[s] * (2.0 * gF[eo] * t3 * lambda) : 0.0);
    }
    P3 *= (1.0 / (2.0 * M));
    Pressure -= P3;
    Pressure /= (3 * tau * volume);
    totVop /= (0.5 * M);
    totVop += tailV;
    T3 /= (2.0 * beta);
    T4 /= (1.0 * beta);
    T5 /= (1.0 * M);
    virKinTerm /= (0.5 * beta);
    thermE *= (0.25 / (lambda * tau)) / (tau * M);
    thermE += thermTerm1;
    thermE += T5;
    thermE += tailV;
    double totEcv = T1 + T2 + T3 + T4 + T5 + tailV;
    double Kcv = T1 + T2 + T3 + T4 + virKinTerm;
    double dEdB = (-1.0 * T1 - 2.0 * T2 + 2.0 * T4) / tau;
    for (int s = 0; s < M; s++) {
        int eo = s % 2;
        double d2U = 0.0;
        if (gF[eo] > kEPS) d2U += 6.0 * gF[eo] * tau * lambda * g2[s];
        dEdB += d2U / (1.0 * M);
    }
    dEdB *= beta * beta / (1.0 * M);
    est[0] += totEcv - totVop;
    est[1] += Kcv;
    est[2] += totVop;
    est[3] += totEcv - Kcv;
    est[4] += totEcv;
    est[5] += totEcv - c.p.mu * numParticles;
    if (numParticles > 0) {
        est[6] += (totEcv - totVop) / (1.0 * numParticles);
        est[7] += Kcv / (1.0 * numParticles);
        est[8] += totVop / (1.0 * numParticles);
        est[9] += (totEcv - Kcv) / (1.0 * numParticles);
        est[10] += totEcv / (1.0 * numParticles);
    }
    est[11] += totEcv * thermE * beta * beta;
    est[12] += totEcv * beta;
    est[13] += dEdB;
    est[14] += totEcv * thermE * beta * beta * totEcv * beta;
    // estimator.cpp:1244 writes estIndex["cVCov2"]; the map has no such key, so
    // operator[] inserts index 0 and the term is added into K_op.
    est[quirk ? 0 : 15] += totEcv * beta * dEdB;
    est[16] += totEcv * thermE * beta * beta * dEdB;
    est[17] += thermE;
    est[18] += Pressure;
    return PGB_OK;
}

// EstimatorBase::getQVectors (estimator.cpp:439-570)
int pgb_qvectors(const char* type, const char* input, const double side[3], double* qout,
                 int cap, int* count) {
    if (!type || !input || !side || !count) { g_last_error = "qvectors: null argument"; return PGB_EINVAL; }
    std::string inputType(type), in(input);
    std::vector<std::array<double,3>> qv;
    std::istringstream iss(in);
    std::vector<std::string> tok;
    std::string w;
    while (iss >> w) tok.push_back(w);
    auto norm = [](const std::array<double,3>& q) { double r = 0.0; for (int i = 0; i < 3; ++i) r += q[i]*q[i]; return std::sqrt(r); };
    try {
        if (inputType == "int" || inputType == "float") {
            if (tok.empty() || tok.size() % 3) { g_last_error = "qvectors: need a multiple of 3 components"; return PGB_EINVAL; }
            for (size_t i = 0; i + 2 < tok.size(); i += 3) {
                std::array<double,3> q;
                for (int j = 0; j < 3; ++j)
                    q[j] = (inputType == "int") ? (2.0 * M_PI / side[j]) * std::stoi(tok[i + j])
                                                : (double)std::stof(tok[i + j]);
                qv.push_back(q);
            }
        } else if (inputType == "max_int" || inputType == "max_float") {
            if (tok.size() < 3) { g_last_error = "qvectors: need 3 components"; return PGB_EINVAL; }
            int qmi[3], qi[3];
            std::array<double,3> qmax{}, q{};
            for (int i = 0; i < 3; ++i) {
                if (inputType == "max_int") { qmi[i] = std::abs(std::stoi(tok[i])); qmax[i] = qmi[i] * 2.0 * M_PI / side[i]; }
                else qmax[i] = std::stof(tok[i]);
            }
            double qmm = norm(qmax);
            if (inputType == "max_float")
                for (int i = 0; i < 3; ++i) qmi[i] = 1 + static_cast<int>(qmm * side[i] / 2.0 / M_PI);
            int n_q = 1;
            for (int i = 0; i < 3; ++i) { n_q *= 2 * qmi[i] + 1; qi[i] = -qmi[i]; q[i] = qi[i] * 2.0 * M_PI / side[i]; }
            if (norm(q) <= qmm) qv.push_back(q);
            int pos = 2, cnt = 0;
            while (cnt < n_q - 1) {
                if (qi[pos] == qmi[pos]) { qi[pos] = -qmi[pos]; pos -= 1; }
                else {
                    qi[pos] += 1;
                    for (int i = 0; i < 3; ++i) q[i] = qi[i] * 2.0 * M_PI / side[i];
                    if (norm(q) <= qmm) qv.push_back(q);
                    cnt += 1; pos = 2;
                }
            }
        } else if (inputType == "file_int" || inputType == "file_float") {
            FILE* f = std::fopen(in.c_str(), "r");
            if (!f) { g_last_error = "qvectors: cannot open " + in; return PGB_EINVAL; }
            char line[4096];
            while (std::fgets(line, sizeof line, f)) {
                std::istringstream ls(line);
                std::array<double,3> q;
                if (inputType == "file_int") {
                    int a[3];
                    if (!(ls >> a[0] >> a[1] >> a[2])) continue;
                    for (int i = 0; i < 3; ++i) q[i] = (2.0 * M_PI / side[i]) * a[i];
                } else {
                    float a[3];
                    if (!(ls >> a[0] >> a[1] >> a[2])) continue;
                    for (int i = 0; i < 3; ++i) q[i] = a[i];
                }
                qv.push_back(q);
            }
            std::fclose(f);
        } else {
            g_last_error = "qvectors: unknown wavevector type " + inputType; return PGB_EINVAL;
        }
    } catch (...) {
        g_last_error = "qvectors: cannot parse input"; return PGB_EINVAL;
    }
    *count = (int)qv.size();
    if (qout)
        for (int i = 0; i < (int)qv.size() && i < cap; ++i)
            for (int j = 0; j < 3; ++j) qout[3 * i + j] = qv[i][j];
    return PGB_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Structure factors
// ---------------------------------------------------------------------------
namespace {

// work layout: rho_q (room for FP64 values), then for the FP32 path the slices
// as box fractions, then the tensor-core scratch
size_t rho_region(const Ctx& c, int nq) {
    return ((size_t)nq * c.M * 2 * sizeof(double) + 255) & ~(size_t)255;
}
size_t posbuf_region(const Ctx& c) {
    return (c.p.precision == PGB_MIXED) ? ((rhoq32_work_bytes(c.view()) + 255) & ~(size_t)255) : 0;
}
int scatter_common(Ctx& c, const double* d_q, int nq, int what, int mode, double* d_out,
                   void* d_work, double maxR2 = 0.0) {
    // what: 0 ssf, 1 isf, 2 rho (FP64 values); maxR2 > 0 restricts the
    // densities to the beads inside the cylinder x^2 + y^2 < maxR2 and leaves
    // S(q) unnormalised by N (its per-sample sum over slices / M)
    PathView v = c.view();
    int N = c.numBeadsOn / c.M;
    if (N <= 0 && maxR2 <= 0.0) return c.fail(PGB_ESTATE, "structure factor needs at least one particle");
    double norm = maxR2 > 0.0 ? 1.0 / (1.0 * c.M) : 1.0 / (1.0 * N * c.M);
    cudaError_t e;
    if (c.p.precision == PGB_FP64 || what == 2) {
        double* d_rho = static_cast<double*>(d_work);
        e = launch_rhoq64(v, d_q, nq, d_rho, c.stream, maxR2);
        if (e == cudaSuccess) {
            if (what == 0) e = launch_ssf_from_rho64(d_rho, nq, c.M, norm, d_out, c.stream);
            else if (what == 1) e = launch_isf_direct64(d_rho, nq, c.M, norm, d_out, c.stream);
            else e = cudaMemcpyAsync(d_out, d_rho, (size_t)nq * c.M * 2 * sizeof(double),
                                     cudaMemcpyDeviceToDevice, c.stream);
        }
    } else {
        float2* d_rho = static_cast<float2*>(d_work);
        void* posbuf = static_cast<char*>(d_work) + rho_region(c, nq);
        e = launch_rhoq32(v, d_q, nq, d_rho, posbuf, c.stream, maxR2);
        if (e == cudaSuccess) {
            if (what == 0) e = launch_ssf_from_rho32(d_rho, nq, c.M, norm, d_out, c.stream);
            else if (mode == 1) {
                if (!isf_tc_supported(c.M))
                    return c.fail(PGB_EINVAL, "tensor-core F(q,tau) needs M a multiple of 128 and <= 2048");
                if (!c.d_tc_tables) {
                    e = cudaMalloc(&c.d_tc_tables, isf_tc_table_bytes(c.M));
                    if (e != cudaSuccess) { c.d_tc_tables = nullptr; return c.cuda_fail(e, "cudaMalloc(F(q,tau) tables)"); }
                    e = isf_tc_build_tables(c.M, c.d_tc_tables, c.stream);
                    if (e != cudaSuccess) return c.cuda_fail(e, "F(q,tau) tables");
                }
                void* tc = static_cast<char*>(d_work) + rho_region(c, nq) + posbuf_region(c);
                e = launch_isf_tc(d_rho, nq, c.M, norm, d_out, tc, c.d_tc_tables, c.stream);
            } else e = launch_isf_direct32(d_rho, nq, c.M, norm, d_out, c.stream);
        }
    }
    if (e != cudaSuccess) return c.cuda_fail(e, "structure factor launch");
    return PGB_OK;
}

size_t scatter_work_bytes(const Ctx& c, int nq, int what, int mode) {
    size_t extra = (c.p.precision == PGB_MIXED && what == 1 && mode == 1)
                       ? isf_tc_scratch_bytes(nq, c.M) : 0;
    return rho_region(c, nq) + posbuf_region(c) + extra;
}

int scatter_host(pgb_ctx* h, const double* q, int nq, int what, int mode, double* out) {
    if (!h || !q || !out || nq < 0) return PGB_EINVAL;
    Ctx& c = h->c;
    int rc = need_path(c); if (rc) return rc;
    if (nq == 0) return PGB_OK;
    if (mode != 0 && mode != 1) return c.fail(PGB_EINVAL, "isf mode must be 0 or 1");
    size_t nout = (what == 0) ? (size_t)nq : (what == 1) ? (size_t)nq * (c.M / 2 + 1)
                                                         : (size_t)nq * c.M * 2;
    size_t qb = (size_t)nq * 3 * sizeof(double);
    size_t ob = nout * sizeof(double);
    size_t wb = scatter_work_bytes(c, nq, what, mode);
    size_t off_o = (qb + 255) & ~(size_t)255;
    size_t off_w = (off_o + ob + 255) & ~(size_t)255;
    rc = c.ensure_scratch(off_w + wb); if (rc) return rc;
    char* base = static_cast<char*>(c.d_scratch);
    PGB_CUDA(&c, cudaMemcpyAsync(base, q, qb, cudaMemcpyHostToDevice, c.stream));
    rc = scatter_common(c, reinterpret_cast<double*>(base), nq, what, mode,
                        reinterpret_cast<double*>(base + off_o), base + off_w);
    if (rc) return rc;
    PGB_CUDA(&c, cudaMemcpyAsync(out, base + off_o, ob, cudaMemcpyDeviceToHost, c.stream));
    const bool tc = c.p.precision == PGB_MIXED && what == 1 && mode == 1;
    int tc_err = 0;
    if (tc) {
        // the tensor-core pipeline's error word: a bounded wait ran out
        const char* w = base + off_w + rho_region(c, nq) + posbuf_region(c);
        PGB_CUDA(&c, cudaMemcpyAsync(&tc_err, w + isf_tc_error_offset(nq, c.M), sizeof(int),
                                     cudaMemcpyDeviceToHost, c.stream));
    }
    PGB_CUDA(&c, cudaStreamSynchronize(c.stream));
    if (tc_err)
        return c.fail(PGB_ETIMEOUT, "F(q,tau): a tensor-core pipeline wait ran out (a staged copy or "
                                    "the MMAs did not complete within the wait limit)");
    return PGB_OK;
}

}  // namespace

extern "C" {

int pgb_ssf(pgb_ctx* h, const double* q, int nq, double* out) { return scatter_host(h, q, nq, 0, 0, out); }

int pgb_ssf_cylinder(pgb_ctx* h, const double* q, int nq, double maxR, double* out,
                     int* num_inside0) {
    if (!h || nq < 0 || !(maxR > 0.0) || (nq > 0 && (!q || !out))) return PGB_EINVAL;
    Ctx& c = h->c;
    int rc = need_path(c); if (rc) return rc;
    const double maxR2 = maxR * maxR;
    size_t qb = (size_t)nq * 3 * sizeof(double), ob = (size_t)nq * sizeof(double);
    size_t off_o = (qb + 255) & ~(size_t)255;
    size_t off_c = (off_o + ob + 255) & ~(size_t)255;
    size_t off_w = off_c + 256;
    rc = c.ensure_scratch(off_w + scatter_work_bytes(c, nq, 0, 0)); if (rc) return rc;
    char* base = static_cast<char*>(c.d_scratch);
    int* d_cnt = reinterpret_cast<int*>(base + off_c);
    PGB_CUDA(&c, launch_count_inside(c.view(), maxR2, d_cnt, c.stream));
    if (nq > 0) {
        PGB_CUDA(&c, cudaMemcpyAsync(base, q, qb, cudaMemcpyHostToDevice, c.stream));
        rc = scatter_common(c, reinterpret_cast<double*>(base), nq, 0, 0,
                            reinterpret_cast<double*>(base + off_o), base + off_w, maxR2);
        if (rc) return rc;
        PGB_CUDA(&c, cudaMemcpyAsync(out, base + off_o, ob, cudaMemcpyDeviceToHost, c.stream));
    }
    int n0 = 0;
    PGB_CUDA(&c, cudaMemcpyAsync(&n0, d_cnt, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    PGB_CUDA(&c, cudaStreamSynchronize(c.stream));
    if (num_inside0) *num_inside0 = n0;
    return PGB_OK;
}

int pgb_qvectors_shells(double dq, double qmax, int sphere, double* qvecs, int* shell, int cap,
                        int* count) {
    if (!count || !(dq > 0.0) || qmax < 0.0 || (cap > 0 && (!qvecs || !shell))) return PGB_EINVAL;
    // EstimatorBase::getQVectors2 (estimator.cpp:762-824): magnitudes
    // cq = 0, dq, 2 dq, ... (accumulated) up to qmax + EPS; q = 0 alone; then
    // (0, 0, cq) and, for the sphere, the (theta, phi) grid of 24 steps over
    // the first octant
    const double kEps = 1.0e-7, kPi = 3.14159265358979323846;
    int n = 0, nshell = 0;
    auto put = [&](double x, double y, double z) {
        if (n < cap) { qvecs[3*n] = x; qvecs[3*n+1] = y; qvecs[3*n+2] = z; shell[n] = nshell; }
        ++n;
    };
    for (double cq = 0.0; cq <= qmax + kEps; cq += dq) {
        if (std::fabs(cq) < kEps) put(0.0, 0.0, 0.0);
        else {
            put(0.0, 0.0, cq);
            const int numTheta = 24;
            const double dtheta = sphere ? 0.5 * kPi / numTheta : kPi;
            for (double theta = dtheta; theta <= 0.5 * kPi + kEps; theta += dtheta) {
                const double dphi = dtheta / std::sin(theta);
                for (double phi = 0.0; phi <= 0.5 * kPi + kEps; phi += dphi)
                    put(cq * std::sin(theta) * std::cos(phi), cq * std::sin(theta) * std::sin(phi),
                        cq * std::cos(theta));
            }
        }
        ++nshell;
    }
    *count = n;
    return PGB_OK;
}
int pgb_isf(pgb_ctx* h, const double* q, int nq, int mode, double* out) { return scatter_host(h, q, nq, 1, mode, out); }
int pgb_rhoq(pgb_ctx* h, const double* q, int nq, double* out) { return scatter_host(h, q, nq, 2, 0, out); }

void pgb_test_isf_tc_stall(int on) { isf_tc_set_stall_test(on); }

int pgb_isf_device_async(pgb_ctx* h, const double* d_q, int nq, int mode, double* d_out) {
    if (!h || !d_q || !d_out || nq <= 0) return PGB_EINVAL;
    Ctx& c = h->c;
    int rc = need_path(c); if (rc) return rc;
    if (mode != 0 && mode != 1) return c.fail(PGB_EINVAL, "isf mode must be 0 or 1");
    rc = c.ensure_scratch(scatter_work_bytes(c, nq, 1, mode)); if (rc) return rc;
    return scatter_common(c, d_q, nq, 1, mode, d_out, c.d_scratch);
}

int pgb_ssf_device_async(pgb_ctx* h, const double* d_q, int nq, double* d_out) {
    if (!h || !d_q || !d_out || nq <= 0) return PGB_EINVAL;
    Ctx& c = h->c;
    int rc = need_path(c); if (rc) return rc;
    rc = c.ensure_scratch(scatter_work_bytes(c, nq, 0, 0)); if (rc) return rc;
    return scatter_common(c, d_q, nq, 0, 0, d_out, c.d_scratch);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Trial displacements: for each (bead, trial position) the change of the
// bead's potential action if only that bead moved there -- the quantity every
// single-bead Metropolis test needs (potentialAction(bead) after minus
// before, action.cpp:487-514), for many independent trials in one launch.
// ---------------------------------------------------------------------------
namespace pgb {
__global__ void k_delta(const double* __restrict__ a, const double* __restrict__ b, double* out, int k) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < k) out[i] = a[i] - b[i];
}
}  // namespace pgb

namespace {
int trial_launch(Ctx& c, const int2* d_b, const double* d_pos, int k, int shift, int mode,
                 double* d_new, double* d_old, double* d_delta) {
    PathView v = c.view();
    cudaError_t e;
    if (c.p.precision == PGB_MIXED && full_list(c)) {
        // one fused launch: U(trial) - U(current) per trial
        int rc = PGB_OK;
        const float4* fall = slice_forces(c, &rc);
        if (rc) return rc;
        e = launch_bead_actions32_full(v, c.az, d_b, k, shift, mode, c.p.tau, c.p.lambda,
                                       c.p.vfactor, c.p.gradvfactor, d_pos, fall, 1, d_delta, c.stream);
        if (e != cudaSuccess) return c.cuda_fail(e, "trial actions launch");
        return PGB_OK;
    }
    if (c.p.precision == PGB_MIXED) {
        e = launch_bead_actions32(v, c.az, d_b, k, shift, mode, c.p.tau, c.p.lambda, c.p.vfactor,
                                  c.p.gradvfactor, d_pos, d_new, c.stream);
        if (e == cudaSuccess)
            e = launch_bead_actions32(v, c.az, d_b, k, shift, mode, c.p.tau, c.p.lambda, c.p.vfactor,
                                      c.p.gradvfactor, nullptr, d_old, c.stream);
    } else {
        e = launch_bead_actions64(v, d_b, k, shift, mode, c.p.tau, c.p.lambda, c.p.vfactor,
                                  c.p.gradvfactor, d_pos, d_new, c.stream);
        if (e == cudaSuccess)
            e = launch_bead_actions64(v, d_b, k, shift, mode, c.p.tau, c.p.lambda, c.p.vfactor,
                                      c.p.gradvfactor, nullptr, d_old, c.stream);
    }
    if (e == cudaSuccess) {
        pgb::k_delta<<<(k + 255) / 256, 256, 0, c.stream>>>(d_new, d_old, d_delta, k);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) return c.cuda_fail(e, "trial actions launch");
    return PGB_OK;
}
}  // namespace

extern "C" {

int pgb_trial_actions(pgb_ctx* h, const int32_t* beads, const double* pos, int k, int shift,
                      int mode, double* out_delta) {
    if (!h || k < 0 || (k > 0 && (!beads || !pos || !out_delta)) || shift < 1 || mode < 0 || mode > 2)
        return PGB_EINVAL;
    Ctx& c = h->c;
    int rc = need_path(c); if (rc) return rc;
    if (k == 0) return PGB_OK;
    for (int i = 0; i < k; ++i)
        if (beads[2*i] < 0 || beads[2*i] >= c.M || beads[2*i+1] < 0 || beads[2*i+1] >= c.Ne)
            return c.fail(PGB_EINVAL, "trial_actions: bead out of range");
    size_t bb = ((size_t)k * sizeof(int2) + 255) & ~(size_t)255;
    size_t pb = ((size_t)k * 3 * sizeof(double) + 255) & ~(size_t)255;
    size_t ob = ((size_t)k * sizeof(double) + 255) & ~(size_t)255;
    rc = c.ensure_scratch(bb + pb + 3 * ob); if (rc) return rc;
    char* d = static_cast<char*>(c.d_scratch);
    PGB_CUDA(&c, cudaMemcpyAsync(d, beads, (size_t)k * sizeof(int2), cudaMemcpyHostToDevice, c.stream));
    PGB_CUDA(&c, cudaMemcpyAsync(d + bb, pos, (size_t)k * 3 * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    double* d_new = reinterpret_cast<double*>(d + bb + pb);
    double* d_old = reinterpret_cast<double*>(d + bb + pb + ob);
    double* d_del = reinterpret_cast<double*>(d + bb + pb + 2 * ob);
    rc = trial_launch(c, reinterpret_cast<int2*>(d), reinterpret_cast<double*>(d + bb), k, shift, mode,
                      d_new, d_old, d_del);
    if (rc) return rc;
    PGB_CUDA(&c, cudaMemcpyAsync(out_delta, d_del, (size_t)k * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    PGB_CUDA(&c, cudaStreamSynchronize(c.stream));
    return PGB_OK;
}

int pgb_trial_actions_device_async(pgb_ctx* h, const int32_t* d_beads, const double* d_pos, int k,
                                   int shift, int mode, double* d_delta, double* d_work) {
    if (!h || !d_beads || !d_pos || !d_delta || !d_work || k <= 0 || shift < 1 || mode < 0 || mode > 2)
        return PGB_EINVAL;
    Ctx& c = h->c;
    int rc = need_path(c); if (rc) return rc;
    return trial_launch(c, reinterpret_cast<const int2*>(d_beads), d_pos, k, shift, mode, d_work,
                        d_work + k, d_delta);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Adjacent path-wide estimators: g(r), superfluid fraction, permutation cycles
// ---------------------------------------------------------------------------
extern "C" {

int pgb_pair_correlation(pgb_ctx* h, int slice, double* out50) {
    if (check_ctx(h) || !out50) return PGB_EINVAL;
    Ctx& c = h->c;
    int rc = need_path(c); if (rc) return rc;
    if (slice >= c.M) return c.fail(PGB_EINVAL, "pair_correlation: slice out of range");
    rc = c.ensure_scratch(64 * sizeof(unsigned long long)); if (rc) return rc;
    auto* d_hist = static_cast<unsigned long long*>(c.d_scratch);
    PGB_CUDA(&c, launch_sep_hist(c.view(), slice, d_hist, c.stream));
    unsigned long long hist[50];
    PGB_CUDA(&c, cudaMemcpyAsync(hist, d_hist, sizeof(hist), cudaMemcpyDeviceToHost, c.stream));
    PGB_CUDA(&c, cudaStreamSynchronize(c.stream));
    // PairCorrelationEstimator: constructor norm (estimator.cpp:3187-3223) and
    // accumulate (estimator.cpp:3238-3246), 3D periodic box
    const int N = c.numBeadsOn / c.M;
    double tot = 0.0;
    for (int n = 0; n < 50; ++n) tot += 1.0 * (double)hist[n];
    const double lnorm = 1.0 * (N - 1) / (1.0 * N);
    const double dR = 0.5 * std::sqrt(3.0) * c.p.side[2] / (1.0 * 50);
    const double volume = c.p.side[0] * c.p.side[1] * c.p.side[2];
    const double gNorm = 3.0 / (2.0 * M_PI);
    for (int n = 0; n < 50; ++n) {
        const double dV = std::pow((n + 1) * dR, 3.0) - std::pow(n * dR, 3.0);
        const double norm = 0.5 * (gNorm * volume) / dV;
        out50[n] = ((N > 1) && (tot > 0.0)) ? lnorm * (1.0 * (double)hist[n] / tot) * norm : 0.0;
    }
    return PGB_OK;
}

int pgb_superfluid(pgb_ctx* h, double* out26) {
    if (check_ctx(h) || !out26) return PGB_EINVAL;
    Ctx& c = h->c;
    int rc = need_path(c); if (rc) return rc;
    rc = c.ensure_scratch(winding_work_bytes()); if (rc) return rc;
    double* d_work = static_cast<double*>(c.d_scratch);
    double* d_out = d_work + (winding_work_bytes() / sizeof(double) - 5);
    PGB_CUDA(&c, launch_winding(c.view(), d_work, d_out, c.stream));
    double s5[5];
    PGB_CUDA(&c, cudaMemcpyAsync(s5, d_out, sizeof(s5), cudaMemcpyDeviceToHost, c.stream));
    PGB_CUDA(&c, cudaStreamSynchronize(c.stream));
    // SuperfluidFractionEstimator::accumulate, estimator.cpp:2000-2074
    double W[3] = {s5[0], s5[1], s5[2]};
    const double Az = s5[3], I = s5[4];
    for (int i = 0; i < 26; ++i) out26[i] = 0.0;
    const int N = c.numBeadsOn / c.M;
    if (N > 0) {
        out26[0] = (W[0] * W[0] + W[1] * W[1] + W[2] * W[2]) / (1.0 * N);
        out26[25] = Az * Az / I;
    }
    for (int d = 0; d < 3; ++d) W[d] *= 1.0 / c.p.side[d];
    for (int d = 0; d < 3; ++d) out26[1 + d] = W[d] * W[d];
    int n = 0;
    for (int p = -10; p <= 10; ++p) {
        if (std::fabs(W[2] - 1.0 * p) < 0.2) out26[4 + n] = 1.0;
        ++n;
    }
    return PGB_OK;
}

int pgb_permutation_cycles(pgb_ctx* h, double* out40) {
    if (check_ctx(h) || !out40) return PGB_EINVAL;
    Ctx& c = h->c;
    int rc = need_path(c); if (rc) return rc;
    const int nw = c.h_nbs.empty() ? 0 : c.h_nbs[0];
    for (int i = 0; i < 40; ++i) out40[i] = 0.0;
    if (nw == 0) return PGB_OK;
    rc = c.ensure_scratch((size_t)nw * sizeof(int)); if (rc) return rc;
    int* d_len = static_cast<int*>(c.d_scratch);
    PGB_CUDA(&c, launch_cycles(c.view(), nw, d_len, c.stream));
    std::vector<int> len(nw);
    PGB_CUDA(&c, cudaMemcpyAsync(len.data(), d_len, nw * sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    PGB_CUDA(&c, cudaStreamSynchronize(c.stream));
    // PermutationCycleEstimator::accumulate, estimator.cpp:2735-2781
    const int N = c.numBeadsOn / c.M;
    const double cycleNorm = N > 0 ? 1.0 / (1.0 * N) : 0.0;
    for (int i = 0; i < nw; ++i) {
        if (len[i] < 0) return c.fail(PGB_ESTATE, "permutation_cycles: the path has an open worldline");
        const int cycleNum = len[i] / c.M;
        if (cycleNum > 0 && cycleNum <= 40) out40[cycleNum - 1] += 1.0 * cycleNum * cycleNorm;
    }
    return PGB_OK;
}

}  // extern "C"

namespace pgb {
int upload_beads(Ctx& c, const int* lin, int k, const double* pos_aos) {
    if (k > 0) {
        const size_t rb = (size_t)k * sizeof(BeadRec);
        int rc = c.ensure_scratch(rb + 64); if (rc) return rc;
        rc = c.ensure_pinned(rb + 64); if (rc) return rc;
        BeadRec* hr = static_cast<BeadRec*>(c.h_pinned);
        for (int i = 0; i < k; ++i) {
            const size_t j = (size_t)lin[i];
            BeadRec r;
            r.s = (int)(j / c.Ne); r.p = (int)(j % c.Ne);
            r.ns = c.h_next[2*j]; r.np = c.h_next[2*j+1];
            r.ps = c.h_prev[2*j]; r.pp = c.h_prev[2*j+1];
            r.on = c.h_on[j]; r.pad = 0;
            r.x = pos_aos[3*j]; r.y = pos_aos[3*j+1]; r.z = pos_aos[3*j+2];
            hr[i] = r;
        }
        PGB_CUDA(&c, cudaMemcpyAsync(c.d_scratch, hr, rb, cudaMemcpyHostToDevice, c.stream));
        k_set_beads<<<(k + 127) / 128, 128, 0, c.stream>>>(c.d_pos, c.d_pos32, c.d_next, c.d_prev, c.d_on,
                                                           c.Ne, static_cast<const BeadRec*>(c.d_scratch), k);
        PGB_CUDA(&c, cudaGetLastError());
    }
    PGB_CUDA(&c, cudaMemcpyAsync(c.d_nbs, c.h_nbs.data(), c.M * sizeof(int), cudaMemcpyHostToDevice, c.stream));
    PGB_CUDA(&c, cudaStreamSynchronize(c.stream));
    c.force_valid = false;
    return PGB_OK;
}
}  // namespace pgb
