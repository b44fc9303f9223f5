// worm_walkers.cu -- device-resident worm-algorithm walkers.
//
// Each walker (an independent grand-canonical or windowed canonical He-4
// path) runs the reference's PIMC step entirely on the device: the default
// move list (centre of mass, bisection or staging, open, close, insert,
// remove, advance/recede head and tail, swap head and tail) with the
// reference's attempt probabilities and diagonal/off-diagonal selection
// (src/pimc.cpp:120-208, src/constants.cpp:191-205), the move semantics of
// src/move.cpp:1124-1707, 1710-3826, the Path bookkeeping of
// src/path.cpp:205-420 and the Worm state of src/worm.cpp:52-118.  The
// plain form (plain_moves.cu) runs the same moves from the host with FP64
// device actions and matches the compiled reference step for step; these
// walkers draw from a Philox stream per walker and evaluate the primitive
// action in FP32 pair sums reduced in double-float, so they agree with it
// statistically.
//
// Execution model: a small walker is one warp; a walker of N0 >= 32 is a
// team of two or four warps (kTeamMinN, kTeam4MinN).  The move logic runs
// redundantly and uniformly in all 32 lanes of the walker's first warp
// (every lane draws the same random numbers and makes the same decisions);
// scalar state (worm locators, gap, length, counters) lives in registers,
// identical in every lane; array writes (positions, links, numBeadsAtSlice)
// are made by lane 0, or lane-parallel for independent beads, and published
// with __syncwarp; a team's other warps take their share of every range
// action, per-bead action and energy sample.  Links store the partner
// particle only: next(t, p) is on slice t + 1 and prev on t - 1.
//
// Latency, not throughput, bounds a walker: a move is a chain of dependent
// link loads, pair sums and warp reductions.  So (1) a move walks its range
// once and caches the beads in shared memory (chain[]), and the actions,
// saves, restores and centre-of-mass shifts index that cache; (2) the pair
// terms of a lane have no branches (absent partners add zero), so its four
// partner terms schedule together, and a team splits a range by beads, so
// several beads' load chains are in flight; (3) position chains (staging
// bridges, free-particle walks) are scans over the lanes, and a worm move's
// run of new beads is placed at once and evaluated in doubling chunks; (4)
// the heavy helpers are not inlined: one copy of each serves all twelve
// moves, which keeps the kernel's code small for the instruction caches;
// (5) the largest walkers are launched first; (6) a move's normal deviates
// come from the lanes together (normals()), from the same words as serial
// draws.
//
// Differences from the reference, all documented where they occur:
//  * the swap pivot is drawn from the pivot slice's beads in index order
//    (the reference walks its LookupTable hash, whose order depends on the
//    history of insertions and deletions): the same distribution;
//  * the Aziz potential is the FP32 analytic form with the reference's
//    hard-core branch (repulsive term only below x = r/rm = 0.01);
//  * a slice that outgrows the bead-array capacity stops the walker with an
//    error (the reference grows its arrays).
#include "pgb_device.cuh"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <deque>
#include <limits>
#include <map>
#include <random>
#include <string>
#include <vector>

namespace pgb {

struct WWMeta {
    long long off;          // first bead of this walker in the bead arrays
    int M, Ne, N0, mbar;
    int blev;               // bisection levels b (constants.cpp:116-120)
    int diag_move;          // diagonal move: 0 bisection (the reference's default), 1 staging
    int num_updates;
    int window;             // canonical window half-width, -1 none
    float L, Linv;
    double tau, lambda, mu, C, volume, tailV0, sqrt2LambdaTau, sqrtLambdaTau, comDelta;
    uint2 key;
};

struct WWState {
    int head[2], tail[2], sp1[2], sp2[2];
    int gap, length, diag, numBeadsOn;
    float sep[3];
    int err;
    unsigned long long ctr;          // sweeps completed: the random stream's sweep index
    // a sweep stopped part-way by the time budget: moves made in it and the
    // random stream's position (draw-block counter and word index)
    int upd, rbidx;
    unsigned long long rctr;
    // an energy sample stopped part-way: the next slice and the sums so far
    int epending, eslice;
    double epot, ekin;
};

struct WB { int t, p; };

__device__ __forceinline__ bool isXW(WB b) { return b.t < 0; }
__device__ __forceinline__ bool eqW(WB a, WB b) { return a.t == b.t && a.p == b.p; }

enum { WM_COM = 0, WM_DIAG, WM_OPEN, WM_CLOSE, WM_INSERT, WM_REMOVE, WM_AH, WM_RH, WM_AT, WM_RT,
       WM_SH, WM_ST, WM_N };
enum { WERR_FULL = 1, WERR_LINK = 2, WERR_LOOP = 3 };

// A CTA holds kCtaWarps warps: kCtaWarps small walkers of one warp each, two
// walkers of kTeamMinN <= N0 < kTeam4MinN served by teams of two warps, or
// one walker of N0 >= kTeam4MinN served by a team of all four.  In a team,
// its first warp runs the move logic as a single-warp walker does, and every
// pair sum (a move's range or bead action) and every energy sample is split
// over the team's warps: the first warp posts the job in shared memory, the
// team meets at its own named barrier, each warp sums its share of the beads
// (or slices), and after a second barrier the first warp adds the shares in
// warp order.  A large walker's chain of dependent moves stays on one warp;
// its pair work, most of its instructions, runs on the team.
constexpr int kCtaWarps = 4;
constexpr int kTeamMinN = 32;
constexpr int kTeam4MinN = 64;
constexpr int kTeamMinBeads = 4;     // shorter range actions of a team walker stay on its warp 0
constexpr int kRunCap = 128;         // per-bead shares a team warp keeps (a worm move's run <= Mbar + 1)
constexpr int kOrigCap = 72;         // saved positions per move (Mbar - 1 <= 63)
constexpr int kMaxWind = 27;         // (2 maxWind + 1)^3 with maxWind = 1
constexpr int kChainCap = 1024;      // beads of one move's range cached per walker (M < 1024)
// A bisection's per-level bead lists are gathered into chain[kListOff ..]: the
// move's own range holds at most 2^b + 1 <= 65 beads (Mbar <= 64), below it.
constexpr int kListOff = 512;

// the shared-memory mailbox of a team: the posted job and each warp's share
struct TeamJob {
    int op;                          // 0 stop, 1 range action, 2 energy sums, 3 per-bead actions
    int a, b;                        // chain offset and count, or slices [a, b)
    WB head, tail, sp1, sp2;         // the worm state that sets the pair factors
    float hi[kCtaWarps], lo[kCtaWarps];      // each warp's (double-float) share
    float khi[kCtaWarps], klo[kCtaWarps];    // each warp's kinetic share (energy)
    int bad[kCtaWarps];                      // a warp met a locator outside the arrays
};
// named barrier `id` (1 + the team's place in its CTA: 1 or 2) over the
// team's threads; constant ids, so the kernel reserves three barriers
__device__ __forceinline__ void team_sync(int id, int nthreads) {
    if (id == 1) asm volatile("bar.sync 1, %0;" ::"r"(nthreads) : "memory");
    else asm volatile("bar.sync 2, %0;" ::"r"(nthreads) : "memory");
}

// Aziz V with the reference's hard-core branch (potential.cpp:1821-1843):
// below x = 0.01 the attractive part is dropped
__device__ __forceinline__ float aziz_v32_core(float r2, const AzizF& a) {
    const float x = sqrtf(r2) * a.rminv;
    if (x < 0.01f) return a.eps * a.A * __expf(x * fmaf(a.beta, x, -a.alpha));
    return aziz_v32(r2, a);
}
// the same without branches, so that the pair terms of a lane schedule
// together: below x = 0.01 the attractive terms are selected away
__device__ __forceinline__ float aziz_v32_sel(float r2, const AzizF& a) {
    const float rinv = rsqrtf(r2);
    const float x = r2 * rinv * a.rminv;
    const float ix = rinv * a.rm;
    const float ix2 = ix * ix;
    const float ix6 = ix2 * ix2 * ix2;
    const bool core = x < 0.01f;
    const float poly = core ? 0.0f : ix6 * fmaf(ix2, fmaf(ix2, a.C10, a.C8), a.C6);
    const float urep = a.A * __expf(x * fmaf(a.beta, x, -a.alpha));
    const float t = fmaxf(fmaf(a.D, ix, -1.0f), 0.0f);
    const float F = core ? 0.0f : __expf(-t * t);
    return a.eps * fmaf(-poly, F, urep);
}

struct WormWalker {
    WWMeta m;
    AzizF az;
    float4* pos;
    int* nxt;
    int* prv;
    int* nbs;
    int* chain;                      // shared: the beads of the current move's range, packed
    float* znorm;                    // shared: a move's normal deviates, 3 (Mbar - 1) at most
    int lane;
    int team = 1;                    // warps serving this walker (1, 2 or kCtaWarps)
    int bar = 1;                     // the team's named barrier
    int wk = 0;                      // this warp's place in the team
    TeamJob* job = nullptr;          // the team's mailbox
    float2* tpart = nullptr;         // shared: a team's per-bead sums, kRunCap at most
    float4* qbuf = nullptr;          // shared: a move's new bead positions, kOrigCap at most
    double* acts = nullptr;          // shared: a move's per-bead actions (aliases znorm)
    // uniform scalar state
    WB head, tail, sp1, sp2;
    int gap, length, diag, numBeadsOn;
    float sep[3];
    int err;
    // Philox stream: key per walker, one counter per draw block of four
    unsigned long long ctr;
    uint4 buf;
    int bidx;
    pgb_worm_walker_stats* acc;

    // ---- random numbers (MTRand's conversions on Philox words) ----
    // the next draw block (one copy of the Philox rounds for every call site)
    __device__ __noinline__ void refill() {
        buf = philox4x32(make_uint4((uint32_t)ctr, (uint32_t)(ctr >> 32), 0x574F524Du, 0u), m.key);
        ++ctr;
        bidx = 0;
    }
    __device__ uint32_t u32() {
        if (bidx == 4) refill();
        const int i = bidx++;
        return i == 0 ? buf.x : i == 1 ? buf.y : i == 2 ? buf.z : buf.w;
    }
    __device__ uint32_t randInt(uint32_t n) {
        uint32_t used = n;
        used |= used >> 1; used |= used >> 2; used |= used >> 4; used |= used >> 8; used |= used >> 16;
        uint32_t i;
        int guard = 0;
        do { i = u32() & used; } while (i > n && ++guard < 1000);
        return i > n ? n : i;
    }
    // FP32 deviates: the walkers agree with the reference statistically, and
    // FP64 transcendentals are slow on this GPU
    __device__ float rand() { return (float)u32() * 2.3283064365386963e-10f; }
    __device__ float randExc() { return (float)(u32() >> 8) * 5.9604644775390625e-08f; }
    // polar-method deviate z; randNorm(mean, sd) is mean + z * sd
    __device__ __noinline__ float randNormZ() {
        float x, y, r;
        int guard = 0;
        do {
            x = 2.0f * rand() - 1.0f;
            y = 2.0f * rand() - 1.0f;
            r = __fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y));    // no contraction: normals() rounds alike
        }
        while ((r >= 1.0f || r == 0.0f) && ++guard < 1000);
        if (r >= 1.0f || r == 0.0f) return 0.0f;
        return x * sqrtf(-2.0f * logf(r) / r);
    }
    __device__ float randNorm(float mean, float sd) { return mean + randNormZ() * sd; }
    // the next cnt deviates that cnt calls of randNormZ() would return, made
    // by the lanes together from the same words: lane l tests attempt
    // a = base + l on words 2a and 2a + 1, the accepted attempts in order
    // give the deviates, and the stream then moves past the last attempt
    // used, exactly where the serial draws would leave it
    // (the stream position is read into registers once: the walker's own
    // copy lives in local memory)
    __device__ __noinline__ void normals(int cnt, float* out) {
        const int rem = 4 - bidx;
        const int bi = bidx;
        const uint4 bf = buf;
        const unsigned long long c0 = ctr;
        const uint2 key = m.key;
        const int ln = lane;
        auto word = [&](long long i) -> uint32_t {
            if (i < rem) {
                const int q = bi + (int)i;
                return q == 0 ? bf.x : q == 1 ? bf.y : q == 2 ? bf.z : bf.w;
            }
            const long long j = i - rem;
            const unsigned long long c = c0 + (unsigned long long)(j >> 2);
            const uint4 w = philox4x32(make_uint4((uint32_t)c, (uint32_t)(c >> 32), 0x574F524Du, 0u), key);
            const int q = (int)(j & 3);
            return q == 0 ? w.x : q == 1 ? w.y : q == 2 ? w.z : w.w;
        };
        int have = 0;
        long long base = 0, used = 0;
        for (int round = 0; have < cnt && round < 64; ++round, base += 32) {
            const long long a = base + ln;
            const float x = 2.0f * ((float)word(2 * a) * 2.3283064365386963e-10f) - 1.0f;
            const float y = 2.0f * ((float)word(2 * a + 1) * 2.3283064365386963e-10f) - 1.0f;
            const float r = __fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y));
            const bool ok = !(r >= 1.0f || r == 0.0f);
            const unsigned mask = __ballot_sync(0xffffffffu, ok);
            const int rank = __popc(mask & ((1u << ln) - 1u));
            if (ok && have + rank < cnt) out[have + rank] = x * sqrtf(-2.0f * logf(r) / r);
            const unsigned last = __ballot_sync(0xffffffffu, ok && rank == cnt - have - 1);
            if (last) used = 2 * (base + __ffs(last));
            have += __popc(mask);
        }
        if (have < cnt) {                           // never in practice: 2048 attempts
            for (int i = have + ln; i < cnt; i += 32) out[i] = 0.0f;
            used = 2 * base;
        }
        if (used <= rem) {
            bidx += (int)used;
        } else {
            const long long wb = used - rem, nb = (wb + 3) >> 2;
            const unsigned long long c = c0 + (unsigned long long)(nb - 1);
            buf = philox4x32(make_uint4((uint32_t)c, (uint32_t)(c >> 32), 0x574F524Du, 0u), key);
            ctr = c + 1;
            bidx = (int)(wb - 4 * (nb - 1));
        }
        __syncwarp();
    }

    // ---- path access ----
    // Positions are slice-major ([M][Ne]: a slice's beads contiguous, for the
    // pair sums); links are particle-major ([Ne][M]: one particle index's
    // beads contiguous), so that a walk along a worldline, which mostly keeps
    // its particle index from slice to slice, reads one cache line every 32
    // links instead of one line every link.
    __device__ size_t li(WB b) const { return (size_t)b.t * m.Ne + b.p; }
    __device__ size_t lk(WB b) const { return (size_t)b.p * m.M + b.t; }
    __device__ bool valid(WB b) const { return b.t >= 0 && b.t < m.M && b.p >= 0 && b.p < m.Ne; }
    __device__ WB next(WB b) {
        if (!valid(b)) { err = WERR_LINK; return {-1, -1}; }
        const int p = nxt[lk(b)];
        if (p < 0) return {-1, -1};
        if (p >= m.Ne) { err = WERR_LINK; return {-1, -1}; }
        return {b.t + 1 == m.M ? 0 : b.t + 1, p};
    }
    __device__ WB prev(WB b) {
        if (!valid(b)) { err = WERR_LINK; return {-1, -1}; }
        const int p = prv[lk(b)];
        if (p < 0) return {-1, -1};
        if (p >= m.Ne) { err = WERR_LINK; return {-1, -1}; }
        return {b.t == 0 ? m.M - 1 : b.t - 1, p};
    }
    // The link arrays and extents in registers for the walks along worldlines
    // (next/prev with the same checks, a bad locator or link reported in
    // `bad`): a walk reads one link a step and stores each bead to the move
    // cache, after which the walker's own copy of these fields would be read
    // again from local memory.
    struct LinkWalk {
        const int* nx;
        const int* pv;
        int M, Ne;
        __device__ WB next(WB b, bool& bad) const {
            if (b.t < 0 || b.t >= M || b.p < 0 || b.p >= Ne) { bad = true; return {-1, -1}; }
            const int p = nx[(size_t)b.p * M + b.t];
            if (p < 0) return {-1, -1};
            if (p >= Ne) { bad = true; return {-1, -1}; }
            return {b.t + 1 == M ? 0 : b.t + 1, p};
        }
        __device__ WB prev(WB b, bool& bad) const {
            if (b.t < 0 || b.t >= M || b.p < 0 || b.p >= Ne) { bad = true; return {-1, -1}; }
            const int p = pv[(size_t)b.p * M + b.t];
            if (p < 0) return {-1, -1};
            if (p >= Ne) { bad = true; return {-1, -1}; }
            return {b.t == 0 ? M - 1 : b.t - 1, p};
        }
    };
    __device__ LinkWalk links() const { return LinkWalk{nxt, prv, m.M, m.Ne}; }
    __device__ WB nextN(WB b, int n) { for (int i = 0; i < n && !isXW(b); ++i) b = next(b); return b; }
    __device__ WB prevN(WB b, int n) { for (int i = 0; i < n && !isXW(b); ++i) b = prev(b); return b; }
    // every access checks its bead: a bad locator sets the error word and
    // touches no memory
    __device__ float4 P(WB b) {
        if (!valid(b)) { err = WERR_LINK; return make_float4(0.f, 0.f, 0.f, 0.f); }
        return pos[li(b)];
    }
    __device__ void setP(WB b, float x, float y, float z) {
        if (!valid(b)) { err = WERR_LINK; return; }
        if (lane == 0) pos[li(b)] = make_float4(x, y, z, 0.f);
        __syncwarp();
    }
    // links: the partner's particle index (slice implied)
    __device__ void setNext(WB b, WB v) {
        if (!valid(b)) { err = WERR_LINK; return; }
        if (lane == 0) nxt[lk(b)] = isXW(v) ? -1 : v.p;
        __syncwarp();
    }
    __device__ void setPrev(WB b, WB v) {
        if (!valid(b)) { err = WERR_LINK; return; }
        if (lane == 0) prv[lk(b)] = isXW(v) ? -1 : v.p;
        __syncwarp();
    }
    __device__ int nb(int t) const { return nbs[t]; }
    __device__ void setNb(int t, int v) { __syncwarp(); if (lane == 0) nbs[t] = v; __syncwarp(); }

    // Worm::getState / factor (worm.h:110-118, worm.cpp:108-118)
    __device__ int state(WB b) const {
        if (eqW(b, head) || eqW(b, tail)) return 2;
        if (eqW(b, sp1) || eqW(b, sp2)) return 1;
        return 0;
    }
    __device__ static float factor(int s1, int s2) {
        if (s1 == 0 && s2 == 0) return 1.f;
        if (s1 == 2 && s2 == 2) return 0.f;
        return 0.5f;
    }
    __device__ float putInBC(float x) const { return x - m.L * floorf(x * m.Linv + 0.5f); }

    // ---- pair sums ----
    // A bead is packed as slice << 12 | particle (Ne <= 4096, M < kChainCap).
    __device__ static int pack(WB b) { return (b.t << 12) | b.p; }
    __device__ static WB unpack(int c) { return {c >> 12, c & 4095}; }
    __device__ size_t at(int c) const { return (size_t)(c >> 12) * m.Ne + (c & 4095); }

    // The fields a pair sum reads, copied once per call into registers: the
    // walker itself lives in local memory around the helpers that are not
    // inlined, and reading it there per pair would cost a load each time.
    // The out-of-line pair loops (teamShare, teamBeadShares, energyShare)
    // take it by value, so it arrives in their registers; by reference it
    // would sit in the caller's local memory and every bead would reload it.
    struct PairCtx {
        const float4* pos;
        const int* nbs;
        int Ne, M;
        float L, Linv;
        AzizF az;
        WB head, tail, sp1, sp2;
        int lane;
        __device__ int state(WB b) const {
            if (eqW(b, head) || eqW(b, tail)) return 2;
            if (eqW(b, sp1) || eqW(b, sp2)) return 1;
            return 0;
        }
    };
    __device__ PairCtx pairCtx() const {
        PairCtx c;
        c.pos = pos; c.nbs = nbs; c.Ne = m.Ne; c.M = m.M; c.L = m.L; c.Linv = m.Linv; c.az = az;
        c.head = head; c.tail = tail; c.sp1 = sp1; c.sp2 = sp2; c.lane = lane;
        return c;
    }
    // one bead's loads, all independent of one another: its slice's bead
    // count, its own position and the first 128 same-slice positions
    // (issued for every index below Ne, used below the count); false for a
    // locator outside the walker's arrays, which then loads bead (0, 0)
    // with no partners
    struct BeadLoad { WB b; int n; float4 rb; float4 r[4]; };
    __device__ static bool loadBead(const PairCtx& c, int code, BeadLoad& L) {
        L.b = unpack(code);
        const bool ok = L.b.t < c.M && L.b.p < c.Ne;
        if (!ok) L.b = WB{0, 0};
        const float4* row = c.pos + (size_t)L.b.t * c.Ne;
        L.n = ok ? c.nbs[L.b.t] : 0;
        L.rb = row[L.b.p];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int j = 32 * u + c.lane;
            L.r[u] = j < c.Ne ? row[j] : L.rb;
        }
        return ok;
    }
    // one pair term, without branches: a partner that is absent (j at or
    // beyond the count, or the bead itself) adds zero.  With Plain set the
    // slice holds no worm or special bead and every factor is one.
    template <bool Plain>
    __device__ static void pairTerm(const PairCtx& c, WB b, int s1, int j, int n, float4 rb, float4 rj,
                                    KahanF& k) {
        const bool ok = j < n && j != b.p;
        const float f = ok ? (Plain ? 1.0f : factor(s1, c.state(WB{b.t, j}))) : 0.0f;
        const float dx = min_image32(rj.x - rb.x, c.L, c.Linv);
        const float dy = min_image32(rj.y - rb.y, c.L, c.Linv);
        const float dz = min_image32(rj.z - rb.z, c.L, c.Linv);
        const float r2 = ok ? fmaf(dx, dx, fmaf(dy, dy, dz * dz)) : 1.0f;
        k.add(f * aziz_v32_sel(r2, c.az));
    }
    template <bool Plain>
    __device__ static void pairsOf(const PairCtx& c, const BeadLoad& L, int s1, KahanF& k) {
#pragma unroll
        for (int u = 0; u < 4; ++u) pairTerm<Plain>(c, L.b, s1, 32 * u + c.lane, L.n, L.rb, L.r[u], k);
        const float4* row = c.pos + (size_t)L.b.t * c.Ne;
        for (int j0 = 128; j0 < L.n; j0 += 128) {
            float4 r[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int j = j0 + 32 * u + c.lane;
                r[u] = j < L.n ? row[j] : L.rb;
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) pairTerm<Plain>(c, L.b, s1, j0 + 32 * u + c.lane, L.n, L.rb, r[u], k);
        }
    }
    // tau-less pair terms of a loaded bead with its active same-slice
    // partners, added to the lane's running sum in ascending partner order
    __device__ static void pairsLoaded(const PairCtx& c, const BeadLoad& L, KahanF& k) {
        const int s1 = c.state(L.b);
        const int t = L.b.t;
        if (s1 == 0 && c.head.t != t && c.tail.t != t && c.sp1.t != t && c.sp2.t != t) pairsOf<true>(c, L, s1, k);
        else pairsOf<false>(c, L, s1, k);
    }
    // One warp's share of a team's range action: the beads chain[c0 + wk],
    // chain[c0 + wk + T], ..., each with all its partners as the single-warp
    // form sums them (the next bead of the share loading meanwhile).  The
    // four warps walk four beads at a time, so a range costs about a quarter
    // of the dependent load chain of one warp walking it.  Returns the
    // warp's (double-float) sum; ok false for a locator outside the walker's
    // arrays.
    __device__ __noinline__ static float2 teamShare(const PairCtx c, const int* ch, int c0, int cnt, int wk, int T,
                                                    bool& ok) {
        KahanF k;
        if (wk < cnt) {
            BeadLoad cur, nx;
            ok &= loadBead(c, ch[c0 + wk], cur);
            for (int i = wk; i < cnt; i += T) {
                if (i + T < cnt) ok &= loadBead(c, ch[c0 + i + T], nx);
                if (cur.b.p < cur.n) pairsLoaded(c, cur, k);
                cur = nx;
            }
        }
        return warp_ff(k);
    }
    // warp 0 of a team: post a job, take its own share, collect the others'
    __device__ void teamPost(int op, int a, int b) {
        if (lane == 0) {
            job->op = op; job->a = a; job->b = b;
            job->head = head; job->tail = tail; job->sp1 = sp1; job->sp2 = sp2;
        }
        team_sync(bar, 32 * team);
    }
    __device__ double teamCollect(float2 mine, bool ok) {
        if (lane == 0) { job->hi[0] = mine.x; job->lo[0] = mine.y; job->bad[0] = ok ? 0 : 1; }
        team_sync(bar, 32 * team);
        double s = 0.0;
        int bad = 0;
        for (int q = 0; q < team; ++q) { s += (double)job->hi[q] + (double)job->lo[q]; bad |= job->bad[q]; }
        if (bad) err = WERR_LINK;
        return s;
    }
    // potentialAction over chain[c0 .. c0 + cnt - 1]: the lanes keep one
    // running sum over the whole range and reduce once (a team: each warp
    // over its share of the partners)
    __device__ __noinline__ double chainAction(int c0, int cnt) {
        // short ranges (a single bead's action in the worm moves) stay on
        // warp 0: the team's two barriers and mailbox cost more than the
        // few pair terms a lane would give away
        if (team > 1 && cnt >= kTeamMinBeads) {
            teamPost(1, c0, cnt);
            bool ok = true;
            const float2 mine = teamShare(pairCtx(), chain, c0, cnt, 0, team, ok);
            return m.tau * teamCollect(mine, ok);
        }
        // one warp: the team form with a team of one (one copy of the pair
        // loop in the kernel's code)
        bool ok = true;
        const float2 r = teamShare(pairCtx(), chain, c0, cnt, 0, 1, ok);
        if (!ok) err = WERR_LINK;
        return m.tau * ((double)r.x + (double)r.y);
    }
    // One warp's share of a team's per-bead actions: the beads of its
    // teamShare share, each reduced on its own and written to part[i] by
    // lane 0
    __device__ __noinline__ static void teamBeadShares(const PairCtx c, const int* ch, int c0, int cnt, int wk,
                                                       int T, bool& ok, float2* part) {
        if (wk >= cnt) return;
        BeadLoad cur, nx;
        ok &= loadBead(c, ch[c0 + wk], cur);
        for (int i = wk; i < cnt; i += T) {
            if (i + T < cnt) ok &= loadBead(c, ch[c0 + i + T], nx);
            KahanF k;
            if (cur.b.p < cur.n) pairsLoaded(c, cur, k);
            const float2 r = warp_ff(k);
            if (c.lane == 0) part[i] = r;
            cur = nx;
        }
    }
    // The bare potential action of each bead chain[c0 .. c0 + cnt - 1]
    // (barePotentialAction, action.cpp:628-645, primitive) with the walker's
    // current worm state, into out[0 .. cnt - 1] (shared): the worm moves'
    // beads evaluated together, their Metropolis tests made afterwards in
    // the reference's order.  A bead's value equals bare() of that bead; the
    // next bead's loads are in flight while a bead's terms are summed.
    __device__ __noinline__ void beadActions(int c0, int cnt, double* out) {
        if (team > 1 && cnt >= kTeamMinBeads && cnt <= kRunCap) {
            teamPost(3, c0, cnt);
            bool ok = true;
            teamBeadShares(pairCtx(), chain, c0, cnt, 0, team, ok, tpart);
            if (lane == 0) job->bad[0] = ok ? 0 : 1;
            team_sync(bar, 32 * team);
            int bad = 0;
            for (int q = 0; q < team; ++q) bad |= job->bad[q];
            if (bad) err = WERR_LINK;
            for (int i = lane; i < cnt; i += 32) out[i] = m.tau * ((double)tpart[i].x + (double)tpart[i].y);
            __syncwarp();
            return;
        }
        // one warp: the team form with a team of one, each bead's (double-
        // float) sum written over its own output slot and widened there
        bool ok = true;
        float2* part = reinterpret_cast<float2*>(out);
        teamBeadShares(pairCtx(), chain, c0, cnt, 0, 1, ok, part);
        if (!ok) err = WERR_LINK;
        __syncwarp();
        for (int i = lane; i < cnt; i += 32) {
            const float2 r = part[i];
            out[i] = m.tau * ((double)r.x + (double)r.y);
        }
        __syncwarp();
    }
    // LocalAction::barePotentialAction(bead), primitive action (VF = 1):
    // tau * sum over the other active beads of the slice of factor * V, as
    // a one-bead range in the cache's last slot (no move's range reaches it:
    // a range holds at most M < kChainCap beads)
    __device__ double bare(WB b) {
        if (!valid(b)) { err = WERR_LINK; return 0.0; }
        if (lane == 0) chain[kChainCap - 1] = pack(b);
        __syncwarp();
        return chainAction(kChainCap - 1, 1);
    }
    // the primitive action has no gradient correction (gradVFactor = 0)
    __device__ double corrRange(WB, WB) { return 0.0; }

    // ---- Path bookkeeping (path.cpp:205-420) ----
    __device__ __noinline__ WB addBead(int slice, float x, float y, float z) {
        const int k = nb(slice);
        if (k >= m.Ne) { err = WERR_FULL; return {-1, -1}; }
        WB last{slice, k};
        setNb(slice, k + 1);
        ++numBeadsOn;
        setNext(last, {-1, -1}); setPrev(last, {-1, -1});
        setP(last, x, y, z);
        return last;
    }
    __device__ WB addNextBead(WB pb, float x, float y, float z) {
        const int slice = pb.t + 1 == m.M ? 0 : pb.t + 1;
        WB b = addBead(slice, x, y, z);
        if (err) return b;
        setNext(pb, b); setPrev(b, pb);
        return b;
    }
    __device__ WB addPrevBead(WB nb_, float x, float y, float z) {
        const int slice = nb_.t == 0 ? m.M - 1 : nb_.t - 1;
        WB b = addBead(slice, x, y, z);
        if (err) return b;
        setPrev(nb_, b); setNext(b, nb_);
        return b;
    }
    __device__ __noinline__ void delBead(WB b) {
        if (!valid(b)) { err = WERR_LINK; return; }
        const int k = nb(b.t) - 1;
        setNb(b.t, k);
        const WB last{b.t, k};
        const WB n = next(b), p = prev(b);
        if (!isXW(n)) setPrev(n, {-1, -1});
        if (!isXW(p)) setNext(p, {-1, -1});
        if (b.p < k) {
            const float4 r = P(last);
            const WB ln = next(last), lp = prev(last);
            setP(b, r.x, r.y, r.z);
            setPrev(b, lp); setNext(b, ln);
            if (!isXW(ln)) setPrev(ln, b);
            if (!isXW(lp)) setNext(lp, b);
            if (eqW(head, last)) head = b;
            if (eqW(tail, last)) tail = b;
            if (eqW(sp1, last)) sp1 = b;
            if (eqW(sp2, last)) sp2 = b;
        }
        setNext(last, {-1, -1}); setPrev(last, {-1, -1});
        --numBeadsOn;
    }
    // A run of cnt new beads on the slices after (dir = +1) or before
    // (dir = -1) bead `from`, linked in a chain from it, at positions q[0 ..
    // cnt - 1]: what cnt calls of addNextBead / addPrevBead (path.cpp:266-300)
    // leave, made one lane a bead (the slices are distinct, cnt < M).  Bead k
    // goes to the end of its slice; the run's locators land in chain[c0 + 1 ..
    // c0 + cnt] and chain[c0] = from.  A slice without room stops the walker
    // (WERR_FULL) with nothing added.
    __device__ __noinline__ bool appendRun(WB from, int cnt, int dir, const float4* q, int c0) {
        if (!valid(from) || cnt < 1 || cnt >= m.M) { err = WERR_LINK; return false; }
        bool full = false;
        for (int k = lane; k < cnt; k += 32) {
            int t = from.t + dir * (k + 1);
            t = ((t % m.M) + m.M) % m.M;
            const int slot = nbs[t];
            full |= slot >= m.Ne;
            chain[c0 + 1 + k] = pack(WB{t, slot < m.Ne ? slot : 0});
        }
        if (lane == 0) chain[c0] = pack(from);
        if (__any_sync(0xffffffffu, full)) { err = WERR_FULL; return false; }
        __syncwarp();
        for (int k = lane; k < cnt; k += 32) {
            const WB b = unpack(chain[c0 + 1 + k]);
            const WB before = unpack(chain[c0 + k]);
            const int after = k + 1 < cnt ? unpack(chain[c0 + 2 + k]).p : -1;
            nbs[b.t] = b.p + 1;
            pos[li(b)] = q[k];
            if (dir > 0) { prv[lk(b)] = before.p; nxt[lk(b)] = after; }
            else { nxt[lk(b)] = before.p; prv[lk(b)] = after; }
        }
        if (lane == 0) {
            const int first = unpack(chain[c0 + 1]).p;
            if (dir > 0) nxt[lk(from)] = first;
            else prv[lk(from)] = first;
        }
        numBeadsOn += cnt;
        __syncwarp();
        return true;
    }
    // the undo of appendRun(from, cnt, dir, ., c0) with the run's locators
    // still in chain[c0 .. c0 + cnt]: each bead of the run is the last of its
    // slice, so the cnt delBead calls (path.cpp:318-368) that remove it move
    // no other bead; they drop the slice counts and the run's links, and
    // unlink `from`
    __device__ void dropRun(int cnt, int dir, int c0) {
        for (int k = lane; k < cnt; k += 32) {
            const WB b = unpack(chain[c0 + 1 + k]);
            nbs[b.t] = b.p;
            nxt[lk(b)] = -1; prv[lk(b)] = -1;
        }
        if (lane == 0) {
            const WB from = unpack(chain[c0]);
            if (dir > 0) nxt[lk(from)] = -1;
            else prv[lk(from)] = -1;
        }
        numBeadsOn -= cnt;
        __syncwarp();
    }
    // positions of a free-particle walk of cnt beads from r0 (newFreeParticle
    // position, move.cpp:183-203: each bead a Gaussian step of sqrt(2 lambda
    // tau) from the previous), into qbuf; the 3 cnt deviates come from the
    // lanes together, the same words serial draws would use.  The walk is a
    // prefix sum of the steps over the lanes in unwrapped coordinates, each
    // bead put in the box afterwards: the positions the serial walk (which
    // wraps every step) gives, up to rounding.
    __device__ __noinline__ void freeWalk(float4 r0, int cnt) {
        normals(3 * cnt, znorm);
        const float sg = (float)m.sqrt2LambdaTau;
        float ux = r0.x, uy = r0.y, uz = r0.z;
        for (int base = 0; base < cnt; base += 32) {
            const int k = base + lane;
            float dx = 0.f, dy = 0.f, dz = 0.f;
            if (k < cnt) { dx = znorm[3 * k] * sg; dy = znorm[3 * k + 1] * sg; dz = znorm[3 * k + 2] * sg; }
            for (int o = 1; o < 32; o <<= 1) {
                const float px = __shfl_up_sync(0xffffffffu, dx, o), py = __shfl_up_sync(0xffffffffu, dy, o),
                            pz = __shfl_up_sync(0xffffffffu, dz, o);
                if (lane >= o) { dx += px; dy += py; dz += pz; }
            }
            const float vx = ux + dx, vy = uy + dy, vz = uz + dz;
            if (k < cnt) qbuf[k] = make_float4(putInBC(vx), putInBC(vy), putInBC(vz), 0.f);
            const int last = min(cnt - base, 32) - 1;
            ux = __shfl_sync(0xffffffffu, vx, last);
            uy = __shfl_sync(0xffffffffu, vy, last);
            uz = __shfl_sync(0xffffffffu, vz, last);
        }
        __syncwarp();
    }
    __device__ WB delBeadGetNext(WB b) { WB n = next(b); delBead(b); return n; }
    __device__ WB delBeadGetPrev(WB b) { WB p = prev(b); delBead(b); return p; }

    // ---- Worm (worm.cpp:52-101, worm.h:68-81) ----
    __device__ void wormReset() {
        gap = -1; length = 0; sep[0] = sep[1] = sep[2] = 0.f;
        head = tail = sp1 = sp2 = WB{-1, -1};
    }
    __device__ __noinline__ void wormUpdate(WB nh, WB nt) {
        head = nh; tail = nt;
        gap = nt.t - nh.t;
        if (gap < 0) gap += m.M;
        // Worm::update (worm.cpp:52-101) counts the worm's beads by walking it
        // from tail to head.  The moves only compare that length with Mbar
        // (remove needs length <= Mbar; advance tail and recede head need it
        // above their step, which is at most Mbar), so the walk stops after
        // Mbar + 1 links and a longer worm counts as Mbar + 1: the same
        // decisions without chasing up to N M dependent links.
        WB b = nt;
        length = 0;
        const int cap = m.mbar + 1;
        const LinkWalk lw = links();
        bool bad = false;
        do {
            ++length;
            b = lw.next(b, bad);
            if (isXW(b)) { err = WERR_LOOP; break; }
        } while (!eqW(b, nh) && length < cap);
        const float4 rt = P(nt), rh = P(nh);
        sep[0] = putInBC(rt.x - rh.x);
        sep[1] = putInBC(rt.y - rh.y);
        sep[2] = putInBC(rt.z - rh.z);
        setNext(nh, {-1, -1}); setPrev(nt, {-1, -1});
        sp1 = sp2 = WB{-1, -1};
    }
    __device__ bool tooCostly(double sx, double sy, double sz, int g) const {
        if (g == 0) return true;
        return ((sx * sx + sy * sy + sz * sz) * (0.25 / (m.lambda * m.tau)) / (1.0 * g)) > 4.0;
    }
    __device__ double ensembleWeight(int d) const {
        if (m.window >= 0) {
            const int nbp = numBeadsOn + d, nb0 = m.N0 * m.M, w = m.M * m.window;
            if (nbp > nb0 + w || nbp < nb0 - w) return 0.0;
        }
        return 1.0;
    }

    // ---- sampling helpers (move.cpp:183-488) ----
    // ActionBase::rho0 (action.cpp:254-260) is evaluated in FP32 inline where
    // used: (4 pi lambda L tau)^(-3/2) exp(-d^2 / (4 lambda L tau))
    __device__ static int3 winding(int n) {
        // MoveBase ctor (move.cpp:88-108) with maxWind = 1
        int3 w;
        w.x = (n / 9) % 3; w.x -= (w.x > 1) * 3;
        w.y = (n / 3) % 3; w.y -= (w.y > 1) * 3;
        w.z = n % 3; w.z -= (w.z > 1) * 3;
        return w;
    }
    // sampleWindingSector (move.cpp:362-397)
    __device__ __noinline__ int3 sampleWinding(WB sb, WB eb, int L, double& totald) {
        // lane n < 27 weighs winding sector n; a scan over the lanes gives the
        // cumulative weights in sector order
        const float4 pe = P(eb), ps = P(sb);
        const float Lb = m.L;
        const float den = (float)(4.0 * m.lambda * L * m.tau);
        const float g = rsqrtf(3.14159265358979f * den);
        const float g3 = g * g * g;
        const int ln = lane;
        const float vx = pe.x - ps.x, vy = pe.y - ps.y, vz = pe.z - ps.z;
        float v = 0.0f;
        if (ln < kMaxWind) {
            const int3 w = winding(ln);
            const float ax = vx + w.x * Lb, ay = vy + w.y * Lb, az_ = vz + w.z * Lb;
            v = g3 * expf(-(ax * ax + ay * ay + az_ * az_) / den);
        }
        for (int o = 1; o < 32; o <<= 1) {
            const float u = __shfl_up_sync(0xffffffffu, v, o);
            if (ln >= o) v += u;
        }
        const float total = __shfl_sync(0xffffffffu, v, kMaxWind - 1);
        totald = total;
        const float x = rand();
        const unsigned h = __ballot_sync(0xffffffffu, ln < kMaxWind && v / total >= x);
        const int idx = h ? __ffs(h) - 1 : kMaxWind - 1;
        return winding(idx);
    }
    // cnt <= 2 kOrigCap new staging positions (newStagingPosition with the
    // winding sector, move.cpp:301-338) from `start` towards e over a range
    // of L links, into out[0 .. cnt - 1] (shared), made by the lanes together.
    // Bead k is r_k = (1 - f_k) r_{k-1} + f_k (e + L_box wind) + sigma_k z_k
    // with f_k = 1 / (L - k); the sector's shifts, which the serial form
    // applies whenever a bead leaves the box, move r_{k-1} and the target by
    // the same amount and cancel, so the chain is an affine recurrence in
    // unwrapped coordinates: a scan of the lanes' maps (A, B): u -> A u + B,
    // each bead put in the box afterwards and the sector left where the
    // serial wraps leave it.  The same positions up to rounding.
    __device__ __noinline__ void stagePositions(int cnt, float4 start, float4 e, int L, int3& wind, float4* out) {
        normals(3 * cnt, znorm);
        const float Lb = m.L;
        const float sg0 = (float)m.sqrt2LambdaTau;
        const float Ex = e.x + Lb * wind.x, Ey = e.y + Lb * wind.y, Ez = e.z + Lb * wind.z;
        float ux = start.x, uy = start.y, uz = start.z;
        for (int base = 0; base < cnt; base += 32) {
            const int k = base + lane;
            float A = 1.0f, bx = 0.0f, by = 0.0f, bz = 0.0f;
            if (k < cnt) {
                const float f1 = 1.0f * (L - k - 1), f2 = 1.0f / (1.0f * (L - k));
                const float sg = sg0 * sqrtf(f1 * f2);
                A = 1.0f - f2;
                bx = fmaf(znorm[3 * k], sg, Ex * f2);
                by = fmaf(znorm[3 * k + 1], sg, Ey * f2);
                bz = fmaf(znorm[3 * k + 2], sg, Ez * f2);
            }
            // inclusive scan: the earlier lanes' map applied first
            for (int o = 1; o < 32; o <<= 1) {
                const float pa = __shfl_up_sync(0xffffffffu, A, o);
                const float px = __shfl_up_sync(0xffffffffu, bx, o), py = __shfl_up_sync(0xffffffffu, by, o),
                            pz = __shfl_up_sync(0xffffffffu, bz, o);
                if (lane >= o) { bx = fmaf(A, px, bx); by = fmaf(A, py, by); bz = fmaf(A, pz, bz); A *= pa; }
            }
            const float vx = fmaf(A, ux, bx), vy = fmaf(A, uy, by), vz = fmaf(A, uz, bz);
            if (k < cnt) out[k] = make_float4(putInBC(vx), putInBC(vy), putInBC(vz), 0.f);
            const int last = min(cnt - base, 32) - 1;
            ux = __shfl_sync(0xffffffffu, vx, last);
            uy = __shfl_sync(0xffffffffu, vy, last);
            uz = __shfl_sync(0xffffffffu, vz, last);
        }
        if (cnt > 0) {
            wind.x -= (int)rintf((ux - putInBC(ux)) * m.Linv);
            wind.y -= (int)rintf((uy - putInBC(uy)) * m.Linv);
            wind.z -= (int)rintf((uz - putInBC(uz)) * m.Linv);
        }
        __syncwarp();
    }
    // new staging positions for chain[1 .. cnt] from chain[0]'s position
    // towards e (through qbuf), written lane-parallel
    __device__ void stageChain(int cnt, float4 start, float4 e, int L, int3& wind) {
        stagePositions(cnt, start, e, L, wind, qbuf);
        for (int i = lane; i < cnt; i += 32) pos[at(chain[i + 1])] = qbuf[i];
        __syncwarp();
    }
    // save / restore chain[1 .. cnt] positions, lane-parallel
    __device__ void saveChain(int cnt, float4* orig) {
        for (int i = lane; i < cnt; i += 32) orig[i] = pos[at(chain[i + 1])];
        __syncwarp();
    }
    __device__ void restoreChain(int cnt, const float4* orig) {
        __syncwarp();
        for (int i = lane; i < cnt; i += 32) pos[at(chain[i + 1])] = orig[i];
        __syncwarp();
    }
    __device__ __noinline__ void freePos(WB nbd, float& x, float& y, float& z) {
        const float4 p = P(nbd);
        const float sg = (float)m.sqrt2LambdaTau;
        x = putInBC(randNorm(p.x, sg));
        y = putInBC(randNorm(p.y, sg));
        z = putInBC(randNorm(p.z, sg));
    }
    // a NaN difference rejects
    __device__ bool metro(double dA) { return rand() < expf(-(float)dA); }
    __device__ int randLen() { return 2 * (1 + (int)randInt((uint32_t)(m.mbar / 2 - 1))); }
    __device__ int trueN() const { return numBeadsOn / m.M; }

    // ---- diagonal moves ----
    // CenterOfMassMove (move.cpp:1124-1262).  The worldline through a
    // random bead of slice 0 is cached in chain[c0 .. c0 + wl - 1]: for a
    // closed single-particle loop by one walk back from that bead (its
    // k-th predecessor lands at M - k), for the worm's segment by a walk
    // back to its start and one forward; ranges longer than M beads are not
    // moved, as in the reference.
    __device__ int com(bool& accepted) {
        accepted = false;
        if (numBeadsOn == 0 || nb(0) == 0) return 0;
        const WB first{0, (int)randInt((uint32_t)(nb(0) - 1))};
        WB b = first;
        int back = 0;
        bool closed = false;
        const LinkWalk lw = links();
        bool bad = false;
        for (;;) {
            const WB pb = lw.prev(b, bad);
            if (bad) { err = WERR_LINK; return 0; }
            if (isXW(pb)) break;
            if (eqW(pb, first)) { closed = true; break; }
            if (back + 1 >= m.M) return 0;
            ++back;
            b = pb;
            if (lane == 0) chain[m.M - back] = pack(b);
        }
        int c0 = 0, wl = 0;
        if (closed) {
            c0 = m.M - back - 1;
            wl = back + 1;
            if (lane == 0) chain[c0] = pack(first);
        } else {
            for (WB s = b;;) {
                if (wl >= m.M) return 0;
                if (lane == 0) chain[wl] = pack(s);
                ++wl;
                const WB ns = lw.next(s, bad);
                if (bad) { err = WERR_LINK; return 0; }
                if (isXW(ns)) break;
                s = ns;
            }
        }
        __syncwarp();
        acc->attempted[WM_COM]++;
        float sh[3];
        for (int i = 0; i < 3; ++i) sh[i] = (float)m.comDelta * (-0.5f + rand());
        const double oldA = chainAction(c0, wl);
        shiftChain(c0, wl, sh[0], sh[1], sh[2]);
        const double newA = chainAction(c0, wl);
        if (metro(newA - oldA)) { accepted = true; acc->accepted[WM_COM]++; }
        else shiftChain(c0, wl, -sh[0], -sh[1], -sh[2]);
        return wl;
    }
    __device__ void shiftChain(int c0, int cnt, float sx, float sy, float sz) {
        for (int i = lane; i < cnt; i += 32) {
            const size_t q = at(chain[c0 + i]);
            const float4 r = pos[q];
            pos[q] = make_float4(putInBC(r.x + sx), putInBC(r.y + sy), putInBC(r.z + sz), 0.f);
        }
        __syncwarp();
    }
    // StagingMove (move.cpp:1315-1412) with winding sectors: chain[0] is the
    // start bead, chain[L] the end bead, chain[1 .. L-1] are restaged
    __device__ int staging(bool& accepted, float4* orig) {
        accepted = false;
        if (numBeadsOn == 0 || trueN() == 0) return 0;
        WB sb;
        sb.t = (int)randInt((uint32_t)(m.M - 1));
        if (nb(sb.t) == 0) return 0;
        sb.p = (int)randInt((uint32_t)(nb(sb.t) - 1));
        const int L = 2 + (int)randInt((uint32_t)(m.mbar - 2));
        WB b = sb;
        const LinkWalk lw = links();
        const int* cnts = nbs;
        bool bad = false;
        for (int k = 0; k < L; ++k) {
            if (b.p >= cnts[b.t]) return 0;
            const WB nb_ = lw.next(b, bad);
            if (bad) { err = WERR_LINK; return 0; }
            if (isXW(nb_)) return 0;
            if (lane == 0) chain[k] = pack(b);
            b = nb_;
        }
        if (lane == 0) chain[L] = pack(b);
        __syncwarp();
        const WB eb = b;
        acc->attempted[WM_DIAG]++;
        double tot;
        int3 wind = sampleWinding(sb, eb, L, tot);
        if (L - 1 > kOrigCap) { err = WERR_LOOP; return 0; }
        const double oldA = chainAction(0, L);
        saveChain(L - 1, orig);
        stageChain(L - 1, P(sb), P(eb), L, wind);
        const double newA = chainAction(0, L);
        if (metro(newA - oldA)) { accepted = true; acc->accepted[WM_DIAG]++; }
        else restoreChain(L - 1, orig);
        return L - 1;
    }

    // BisectionMove (move.cpp:1484-1666), local-action branch: chain[0] is
    // the start bead, chain[2^l] the end bead, chain[1 .. 2^l - 1] are moved.
    // Level l (shift s = 2^(l-1)) places the beads at offsets s, 3s, 5s, ...
    // about the midpoint of their neighbours at -s and +s, which are fixed
    // ends or beads placed at earlier levels, so the lanes place them
    // together (the deviates of all levels made at the start by normals(),
    // in the reference's level and bead order).  The
    // level's action is the list action of those beads at tau() = s tau
    // (primitive: no correction); level 1 adds the beads of the earlier
    // levels in their new and old positions; each level is tested against
    // exp(-dA + dA_previous level) and a rejection restores every bead moved
    // so far.  Returns the beads proposed, as the oracle counts them.
    __device__ void gatherStride(int first, int stride, int cnt) {
        for (int i = lane; i < cnt; i += 32) chain[kListOff + i] = chain[first + stride * i];
        __syncwarp();
    }
    __device__ int bisection(bool& accepted, float4* orig, float4* newp) {
        accepted = false;
        if (numBeadsOn == 0) return 0;
        const int numLevels = 1 + (int)randInt((uint32_t)(m.blev - 1));   // variable length (varUpdates)
        const int numActive = (1 << numLevels) - 1;
        if (trueN() == 0) return 0;
        WB sb;
        sb.t = (int)randInt((uint32_t)(m.M - 1));
        if (nb(sb.t) == 0) return 0;
        sb.p = (int)randInt((uint32_t)(nb(sb.t) - 1));
        if (numActive > kOrigCap) { err = WERR_LOOP; return 0; }
        WB b = sb;
        const LinkWalk lw = links();
        const int* cnts = nbs;
        bool bad = false;
        for (int k = 0; k <= numActive; ++k) {
            if (b.p >= cnts[b.t]) return 0;
            const WB nx = lw.next(b, bad);
            if (bad) { err = WERR_LINK; return 0; }
            if (isXW(nx)) return 0;
            if (lane == 0) chain[k] = pack(b);
            b = nx;
        }
        if (lane == 0) chain[numActive + 1] = pack(b);
        __syncwarp();
        acc->attempted[WM_DIAG]++;
        saveChain(numActive, orig);                     // orig[j - 1]: bead at offset j
        const float sgBase = (float)m.sqrtLambdaTau;
        // the normal deviates of every level at once, level by level in the
        // reference's order (a level rejected early leaves the later levels'
        // deviates unused: independent draws, the same distribution)
        normals(3 * numActive, znorm);
        int zoff = 0;
        double oldDelta = 0.0;
        int moved = 0;
        for (int level = numLevels; level > 0; --level) {
            const int s = 1 << (level - 1);
            const int cnt = 1 << (numLevels - level);  // offsets s (2i + 1), i < cnt
            gatherStride(s, 2 * s, cnt);
            double oldA = s * chainAction(kListOff, cnt);
            const float sg = sgBase * sqrtf((float)s);
            const float* z = znorm + 3 * zoff;
            zoff += cnt;
            for (int i = lane; i < cnt; i += 32) {
                const int j = s * (2 * i + 1);
                const float4 pp = pos[at(chain[j - s])], pn = pos[at(chain[j + s])];
                // newBisectionPosition (move.cpp:467-488): midpoint of the
                // neighbours at -s and +s, then a Gaussian kick, then inside
                const float mx = fmaf(0.5f, min_image32(pn.x - pp.x, m.L, m.Linv), pp.x);
                const float my = fmaf(0.5f, min_image32(pn.y - pp.y, m.L, m.Linv), pp.y);
                const float mz = fmaf(0.5f, min_image32(pn.z - pp.z, m.L, m.Linv), pp.z);
                const float4 q = make_float4(putInBC(fmaf(z[3 * i], sg, mx)), putInBC(fmaf(z[3 * i + 1], sg, my)),
                                             putInBC(fmaf(z[3 * i + 2], sg, mz)), 0.f);
                newp[j - 1] = q;
                pos[at(chain[j])] = q;
            }
            __syncwarp();
            moved += cnt;
            double newA = s * chainAction(kListOff, cnt);
            if (level == 1 && numActive > 1) {
                // the beads of the earlier levels: offsets 2, 4, .., numActive - 1
                const int pc = (numActive - 1) / 2;
                gatherStride(2, 2, pc);
                newA += chainAction(kListOff, pc);
                for (int i = lane; i < pc; i += 32) pos[at(chain[2 * (i + 1)])] = orig[2 * i + 1];
                __syncwarp();
                oldA += chainAction(kListOff, pc);
                for (int i = lane; i < pc; i += 32) pos[at(chain[2 * (i + 1)])] = newp[2 * i + 1];
                __syncwarp();
            }
            const double dA = newA - oldA;
            if (metro(dA - oldDelta)) {
                if (level == 1) { accepted = true; acc->accepted[WM_DIAG]++; }
            } else {
                // undoMove (move.cpp:1694-1707): every bead moved so far, the
                // offsets that are multiples of s
                for (int j = lane + 1; j <= numActive; j += 32)
                    if (j % s == 0) pos[at(chain[j])] = orig[j - 1];
                __syncwarp();
                break;
            }
            oldDelta = dA;
        }
        return moved;
    }

    // ---- worm moves (move.cpp:1736-3826), local-action branches ----
    // The worm moves below propose or remove a run of beads and test them one
    // at a time in the reference's order, rejecting at the first failure
    // (move.cpp:1736-3185).  Here the run's beads are placed first (new beads
    // one lane a bead, appendRun), their bare actions evaluated together
    // (beadActions), and then the same sequence of Metropolis tests reads the
    // stored values.  The beads of a run sit on distinct slices and the pair
    // action couples only beads of one slice, so a bead's action is the one
    // the sequential form would find; the worm state is set as the reference
    // sets it while the beads are evaluated.  A new run's normal deviates are
    // all drawn before its uniform ones: a different order of independent
    // draws, the same distribution.

    // the beads from `a` along next (dir > 0) or prev links to `b` inclusive,
    // into chain[0 ..]; returns their number (b not reached: the walk's end,
    // with err set for a broken link)
    __device__ int collectRun(WB a, WB b, int dir) {
        int cnt = 0;
        WB x = a;
        const LinkWalk lw = links();
        const int cap = m.mbar + 1;
        bool bad = false;
        for (int g = 0; g <= cap; ++g) {
            if (isXW(x)) { err = WERR_LINK; break; }
            if (lane == 0) chain[cnt] = pack(x);
            ++cnt;
            if (eqW(x, b)) break;
            x = dir > 0 ? lw.next(x, bad) : lw.prev(x, bad);
        }
        __syncwarp();
        return cnt;
    }
    // acts[k] for chain[k], evaluated a chunk at a time once the tests reach
    // it: the first chunk one bead (kTeamMinBeads for a team), each next one
    // twice as long, so that a run rejected at its first beads costs about
    // what the sequential form costs and a long accepted run is evaluated in
    // a few batches
    __device__ void actsUpTo(int k, int total, int& ev, int& chunk) {
        if (k < ev) return;
        const int n = min(chunk, total - ev);
        beadActions(ev, n, acts + ev);
        ev += n;
        chunk = min(2 * chunk, kRunCap);
    }
    __device__ int firstChunk() const { return team > 1 ? kTeamMinBeads : 1; }
    // removal-type test over the beads chain[0 .. cnt - 1]: -(U_k - f_k
    // shift), f = 1/2 at both ends and 1 between; true when every bead is
    // accepted
    __device__ bool removalTests(int cnt, double actionShift, double corr) {
        int ev = 0, chunk = firstChunk();
        for (int k = 0; k < cnt; ++k) {
            actsUpTo(k, cnt, ev, chunk);
            acc->bead_updates++;
            double dA = -(acts[k] - ((k == 0 || k == cnt - 1) ? 0.5 : 1.0) * actionShift);
            if (k == cnt - 1) dA -= corr;
            if (!metro(dA)) return false;
        }
        return true;
    }
    // insertion-type test over the beads chain[0 .. cnt]: U_k - f_k shift,
    // f = 1/2 at both ends and 1 between.  With `endRef` set, the last bead
    // `end` becomes that worm end (*endRef = end) before its action is taken,
    // as the reference sets the new head or tail before its test; chain[cnt]
    // is then not read.
    __device__ bool insertionTests(int cnt, double actionShift, double corr, WB* endRef, WB end) {
        int ev = 0, chunk = firstChunk();
        const int total = endRef ? cnt : cnt + 1;
        for (int k = 0; k <= cnt; ++k) {
            double u;
            if (k == cnt && endRef) {
                *endRef = end;
                u = bare(end);
            } else {
                actsUpTo(k, total, ev, chunk);
                u = acts[k];
            }
            acc->bead_updates++;
            double dA = u - ((k == 0 || k == cnt) ? 0.5 : 1.0) * actionShift;
            if (k == cnt) dA += corr;
            if (!metro(dA)) return false;
        }
        return true;
    }

    __device__ int open() {
        if (numBeadsOn == 0 || trueN() == 0) return -1;
        const int gapLength = randLen();
        WB hb, tb;
        hb.t = 2 * (int)randInt((uint32_t)(m.M / 2 - 1));
        if (nb(hb.t) == 0) return -1;
        hb.p = (int)randInt((uint32_t)(nb(hb.t) - 1));
        tb = nextN(hb, gapLength);
        if (isXW(tb)) return -1;
        double totalrho0;
        const int3 wind = sampleWinding(hb, tb, gapLength, totalrho0);
        const float4 pt = P(tb), ph = P(hb);
        const double sx = (double)((pt.x - ph.x) + wind.x * m.L);
        const double sy = (double)((pt.y - ph.y) + wind.y * m.L);
        const double sz = (double)((pt.z - ph.z) + wind.z * m.L);
        if (tooCostly(sx, sy, sz, gapLength)) return -1;
        double norm = (m.C * m.mbar * numBeadsOn) / totalrho0;
        norm *= 0.15 / 0.4;
        norm *= ensembleWeight(-gapLength + 1);
        const double muShift = gapLength * m.mu * m.tau;
        acc->attempted[WM_OPEN]++;
        sp1 = hb; sp2 = tb;
        const double actionShift = (-log(norm) + muShift) / gapLength;
        // hb, the gap's beads and tb: removed but the ends
        const int cnt = collectRun(hb, tb, +1);
        if (err) return -2;
        if (removalTests(cnt, actionShift, corrRange(hb, tb))) {
            acc->accepted[WM_OPEN]++;
            WB b = next(hb);
            for (int g = 0; g <= m.M && !eqW(b, tb) && !isXW(b); ++g) b = delBeadGetNext(b);
            wormUpdate(hb, tb);
            diag = 0;
            return 1;
        }
        wormReset(); diag = 1;
        return 0;
    }
    // the undo of a close whose nnew staging beads are chain[1 .. nnew]
    __device__ void closeUndo(int nnew) {
        if (nnew > 0) dropRun(nnew, +1, 0);
        setNext(head, {-1, -1}); setPrev(tail, {-1, -1});
        diag = 0;
    }
    __device__ int close() {
        if (numBeadsOn == 0) return -1;
        if (gap > m.mbar || gap == 0 || tooCostly(sep[0], sep[1], sep[2], gap)) return -1;
        acc->attempted[WM_CLOSE]++;
        const int g0 = gap;
        double totalrho0;
        int3 wind = sampleWinding(head, tail, g0, totalrho0);
        double norm = totalrho0 / (m.C * m.mbar * (numBeadsOn + g0 - 1));
        norm *= 0.4 / 0.15;
        norm *= ensembleWeight(g0 - 1);
        const double muShift = g0 * m.mu * m.tau;
        const double actionShift = (log(norm) + muShift) / g0;
        // the g0 - 1 staging positions from the head towards the tail
        // (newStagingPosition with the winding sector, move.cpp:301-338)
        const int nnew = g0 - 1;
        if (nnew > 0) {
            stagePositions(nnew, P(head), P(tail), g0, wind, qbuf);
            if (!appendRun(head, nnew, +1, qbuf, 0)) return -2;
        } else {
            if (lane == 0) chain[0] = pack(head);
            __syncwarp();
        }
        const WB last = unpack(chain[nnew]);
        setNext(last, tail); setPrev(tail, last);
        if (lane == 0) chain[g0] = pack(tail);
        __syncwarp();
        // head, the new beads and the tail
        if (insertionTests(g0, actionShift, corrRange(head, tail), nullptr, tail)) {
            acc->accepted[WM_CLOSE]++; wormReset(); diag = 1; return 1;
        }
        closeUndo(nnew);
        return 0;
    }
    // the undo of an insert: the run of wl beads after tb, then tb
    __device__ void insertUndo(WB tb, int wl) {
        dropRun(wl, +1, 0);
        delBead(tb);
        wormReset(); diag = 1;
    }
    __device__ int insert() {
        const int wl = randLen();
        acc->attempted[WM_INSERT]++;
        double norm = m.C * m.mbar * m.M * m.volume;
        const double muShift = wl * m.tau * m.mu;
        norm *= 0.15 / 0.4;
        norm *= ensembleWeight(wl);
        if (norm < 2.220446049250313e-16) return 0;
        const int slice = 2 * (int)randInt((uint32_t)(m.M / 2 - 1));
        const float x0 = m.L * (-0.5f + randExc()), y0 = m.L * (-0.5f + randExc()), z0 = m.L * (-0.5f + randExc());
        const WB tb = addBead(slice, x0, y0, z0);
        if (err) return -2;
        sp2 = tb;
        const double actionShift = (log(norm) + muShift) / wl;
        // the new worldline: tb, wl - 1 beads, the head
        freeWalk(make_float4(x0, y0, z0, 0.f), wl);
        if (!appendRun(tb, wl, +1, qbuf, 0)) return -2;
        const WB hb = unpack(chain[wl]);
        // tb, the intermediate beads and the head (sp1 = hb before its test)
        if (insertionTests(wl, actionShift, corrRange(tb, hb), &sp1, hb)) {
            acc->accepted[WM_INSERT]++; wormUpdate(hb, tb); diag = 0; return 1;
        }
        insertUndo(tb, wl);
        return 0;
    }
    __device__ int remove() {
        if (length > m.mbar || length < 1) return -1;
        acc->attempted[WM_REMOVE]++;
        double norm = 1.0 / (m.C * m.mbar * m.M * m.volume);
        const double muShift = length * m.mu * m.tau;
        norm *= 0.4 / 0.15;
        norm *= ensembleWeight(-length);
        if (norm < 2.220446049250313e-16) return 0;
        const double actionShift = (-log(norm) + muShift) / length;
        // the worm from the head back to the tail
        const int cnt = collectRun(head, tail, -1);
        if (err) return -2;
        if (removalTests(cnt, actionShift, corrRange(tail, head))) {
            acc->accepted[WM_REMOVE]++;
            WB b = head;
            for (int g = 0; g <= m.M * m.Ne && !isXW(b); ++g) b = delBeadGetPrev(b);
            wormReset(); diag = 1;
            return 1;
        }
        diag = 0;
        return 0;
    }
    __device__ void ahUndo(int al) {
        head = sp1;
        dropRun(al, +1, 0);
        diag = 0;
        sp1 = WB{-1, -1};
    }
    __device__ int advanceHead() {
        if (numBeadsOn == 0) return -1;
        const int al = randLen();
        acc->attempted[WM_AH]++;
        const double muShift = al * m.tau * m.mu;
        double norm = 1.0;
        norm *= ensembleWeight(al);
        sp1 = head; head = WB{-1, -1};
        const double actionShift = (log(norm) + muShift) / al;
        // the old head and al new beads, the last the new head
        freeWalk(P(sp1), al);
        if (!appendRun(sp1, al, +1, qbuf, 0)) return -2;
        const WB hb = unpack(chain[al]);
        // the old head, the intermediate beads and the new head, set before
        // its test (potentialAction(head): primitive)
        if (insertionTests(al, actionShift, corrRange(sp1, hb), &head, hb)) {
            acc->accepted[WM_AH]++; wormUpdate(hb, tail); diag = 0; return 1;
        }
        ahUndo(al);
        return 0;
    }
    __device__ int advanceTail() {
        if (numBeadsOn == 0) return -1;
        const int al = randLen();
        if (!(al < length)) return -1;
        const WB tb = nextN(tail, al);
        if (isXW(tb)) return -1;
        const double muShift = al * m.tau * m.mu;
        double norm = 1.0;
        norm *= ensembleWeight(-al);
        acc->attempted[WM_AT]++;
        sp1 = tb;
        const double actionShift = (-log(norm) + muShift) / al;
        // the tail and the beads up to tb: removed but tb
        const int cnt = collectRun(tail, tb, +1);
        if (err) return -2;
        if (removalTests(cnt, actionShift, corrRange(tail, tb))) {
            acc->accepted[WM_AT]++;
            WB b = prev(tb);
            for (int g = 0; g <= m.M * m.Ne && !isXW(b); ++g) b = delBeadGetPrev(b);
            wormUpdate(head, tb);
            diag = 0;
            return 1;
        }
        diag = 0; sp1 = WB{-1, -1};
        return 0;
    }
    __device__ int recedeHead() {
        if (numBeadsOn == 0) return -1;
        const int rl = randLen();
        if (!(rl < length)) return -1;
        const WB hb = prevN(head, rl);
        if (isXW(hb)) return -1;
        const double muShift = rl * m.tau * m.mu;
        double norm = 1.0;
        norm *= ensembleWeight(-rl);
        acc->attempted[WM_RH]++;
        sp1 = hb;
        const double actionShift = (-log(norm) + muShift) / rl;
        // the head and the beads back to hb: removed but hb
        const int cnt = collectRun(head, hb, -1);
        if (err) return -2;
        if (removalTests(cnt, actionShift, corrRange(sp1, head))) {
            acc->accepted[WM_RH]++;
            WB b = next(hb);
            for (int g = 0; g <= m.M * m.Ne && !isXW(b); ++g) b = delBeadGetNext(b);
            wormUpdate(hb, tail);
            diag = 0;
            return 1;
        }
        diag = 0; sp1 = WB{-1, -1};
        return 0;
    }
    __device__ void rtUndo(int rl) {
        tail = sp1;
        dropRun(rl, -1, 0);
        diag = 0;
        sp1 = WB{-1, -1};
    }
    __device__ int recedeTail() {
        if (numBeadsOn == 0) return -1;
        const int rl = randLen();
        acc->attempted[WM_RT]++;
        const double muShift = rl * m.tau * m.mu;
        double norm = 1.0;
        norm *= ensembleWeight(rl);
        sp1 = tail; tail = WB{-1, -1};
        const double actionShift = (log(norm) + muShift) / rl;
        // the old tail and rl new beads before it, the last the new tail
        freeWalk(P(sp1), rl);
        if (!appendRun(sp1, rl, -1, qbuf, 0)) return -2;
        const WB tb = unpack(chain[rl]);
        // the old tail, the intermediate beads and the new tail, set before
        // its test
        if (insertionTests(rl, actionShift, corrRange(tb, sp1), &tail, tb)) {
            acc->accepted[WM_RT]++; wormUpdate(head, tb); diag = 0; return 1;
        }
        rtUndo(rl);
        return 0;
    }
    // SwapMoveBase::getNorm + selectPivotBead (move.cpp:3212-3338) over the
    // pivot slice's beads in index order.  Lane w (< 27) accumulates the
    // weight of winding sector w summed over the slice; Sigma is the total.
    // With x >= 0 the pivot is the first (sector, bead) in the reference's
    // order (bead fastest, sector slowest) whose cumulative weight reaches
    // x * Sigma: the sector by a scan over the lanes' sector sums, the bead
    // by a scan inside that sector.
    // rho0 of one sector as the product of its three axis factors, the form
    // the sector sums use
    __device__ static float rho0Shifted(float4 pf, float4 pb, int3 wv, int sign, float g3, float nden, float L) {
        const float ax = (pf.x - pb.x) + (float)(sign * wv.x) * L, ay = (pf.y - pb.y) + (float)(sign * wv.y) * L,
                    az_ = (pf.z - pb.z) + (float)(sign * wv.z) * L;
        return g3 * expf(ax * ax * nden) * expf(ay * ay * nden) * expf(az_ * az_ * nden);
    }
    __device__ __noinline__ double towerNorm(WB b, int pivotSlice, int sign, float x, WB& pivot, int3& wind) {
        const int nL = nb(pivotSlice);
        const float4 pb = P(b);
        const float4* row = pos + (size_t)pivotSlice * m.Ne;
        const float den = (float)(4.0 * m.lambda * m.mbar * m.tau);
        const float g = rsqrtf(3.14159265358979f * den);
        const float g3 = g * g * g;
        const float L = m.L;
        const int ln = lane;
        const float nden = -1.0f / den;
        // each lane's share of the 27 sector weights (32 slots, the last five
        // zero), summed over its beads
        float acc[32];
#pragma unroll
        for (int w = 0; w < 32; ++w) acc[w] = 0.0f;
        for (int n0 = 0; n0 < nL; n0 += 128) {
            float4 pf[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int n = n0 + 32 * u + ln;
                pf[u] = n < nL ? row[n] : pb;
            }
            // rho0 factorises over the axes: three shifts per axis (component
            // 0, +1, -1 of the winding vector) give the 27 sector weights as
            // products, 9 exponentials a bead instead of 27
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const bool ok = n0 + 32 * u + ln < nL;
                const float dx = pf[u].x - pb.x, dy = pf[u].y - pb.y, dz = pf[u].z - pb.z;
                float ex[3], ey[3], ez[3];
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const float sh = (float)(sign * (k == 2 ? -1 : k)) * L;
                    const float ax = dx + sh, ay = dy + sh, az_ = dz + sh;
                    ex[k] = ok ? g3 * expf(ax * ax * nden) : 0.0f;
                    ey[k] = expf(ay * ay * nden);
                    ez[k] = expf(az_ * az_ * nden);
                }
#pragma unroll
                for (int w = 0; w < kMaxWind; ++w) acc[w] = fmaf(ex[(w / 9) % 3] * ey[(w / 3) % 3], ez[w % 3], acc[w]);
            }
        }
        // sector totals over the lanes by recursive halving: at each step a
        // lane keeps the half of its slots that its partner lane does not,
        // adding the partner's copy of them; lane w ends with sector w's total
        // (31 shuffles instead of 27 five-step reductions)
#pragma unroll
        for (int h = 16; h >= 1; h >>= 1) {
            const bool upper = (ln & h) != 0;
#pragma unroll
            for (int i = 0; i < h; ++i) {
                const float send = upper ? acc[i] : acc[i + h];
                const float keep = upper ? acc[i + h] : acc[i];
                acc[i] = keep + __shfl_xor_sync(0xffffffffu, send, h);
            }
        }
        const float mine = ln < kMaxWind ? acc[0] : 0.0f;   // ln w: sector w's weight
        // inclusive scan of the sector sums over lanes 0..26
        float cum = ln < kMaxWind ? mine : 0.0f;
        for (int o = 1; o < 32; o <<= 1) {
            const float u = __shfl_up_sync(0xffffffffu, cum, o);
            if (ln >= o) cum += u;
        }
        const float sum = __shfl_sync(0xffffffffu, cum, kMaxWind - 1);
        if (x >= 0.0f) {
            const float target = x * sum;
            const unsigned hs = __ballot_sync(0xffffffffu, ln < kMaxWind && cum >= target);
            const int ws = hs ? __ffs(hs) - 1 : kMaxWind - 1;
            const float before = __shfl_sync(0xffffffffu, cum - mine, ws);
            const int3 wv = winding(ws);
            float carry = before;
            int found = nL - 1;
            for (int base = 0; base < nL; base += 32) {
                const int n = base + ln;
                float v = n < nL ? rho0Shifted(row[n], pb, wv, sign, g3, nden, L) : 0.0f;
                for (int o = 1; o < 32; o <<= 1) {
                    const float u = __shfl_up_sync(0xffffffffu, v, o);
                    if (ln >= o) v += u;
                }
                const unsigned h = __ballot_sync(0xffffffffu, n < nL && carry + v >= target);
                if (h) { found = base + __ffs(h) - 1; break; }
                carry += __shfl_sync(0xffffffffu, v, 31);
            }
            pivot = WB{pivotSlice, found};
            wind = wv;
        }
        return (double)sum;
    }
    // SwapHeadMove (move.cpp:3388-3622): chain[0 .. Mbar] runs from the swap
    // bead to the pivot; after relinking chain[0] is the old head
    __device__ int swapHead(float4* orig) {
        if (numBeadsOn == 0 || diag) return -1;
        const int swapLength = m.mbar;
        int pivotSlice = head.t + swapLength;
        if (pivotSlice >= m.M) pivotSlice -= m.M;
        if (nb(pivotSlice) == 0) return -1;
        WB pivot; int3 wind;
        const double SigmaHead = towerNorm(head, pivotSlice, 1, rand(), pivot, wind);
        WB b = pivot;
        const LinkWalk lw = links();
        bool bad = false;
        for (int k = 0; k < swapLength; k++) {
            if (eqW(b, tail) || isXW(b)) { if (bad) err = WERR_LINK; return -1; }
            if (lane == 0) chain[swapLength - k] = pack(b);
            b = lw.prev(b, bad);
        }
        if (bad) err = WERR_LINK;
        const WB swp = b;
        if (isXW(swp) || eqW(tail, swp)) return -1;
        if (lane == 0) chain[0] = pack(swp);
        __syncwarp();
        acc->attempted[WM_SH]++;
        WB dummy; int3 dw;
        const double SigmaSwap = towerNorm(swp, pivotSlice, 1, -1.0f, dummy, dw);
        const float PNorm = (float)fmin(SigmaHead / SigmaSwap, 1.0);
        if (rand() < PNorm) {
            const int nm = swapLength - 1;
            sp1 = swp; sp2 = pivot;
            saveChain(nm, orig);
            const double oldA = chainAction(0, swapLength + 1);
            const WB nextSwap = next(swp);
            setNext(head, nextSwap);
            setNext(swp, {-1, -1});
            setPrev(nextSwap, head);
            sp1 = head;
            head = swp;
            if (lane == 0) chain[0] = pack(sp1);
            stageChain(nm, P(sp1), P(pivot), swapLength, wind);
            acc->bead_updates += nm;
            const double newA = chainAction(0, swapLength + 1);
            if (metro(newA - oldA)) { acc->accepted[WM_SH]++; wormUpdate(swp, tail); return 1; }
            head = sp1;
            setNext(head, {-1, -1});
            setNext(swp, nextSwap);
            setPrev(nextSwap, swp);
            restoreChain(nm, orig);
            diag = 0;
            sp1 = sp2 = WB{-1, -1};
            return 0;
        }
        return 0;
    }
    // SwapTailMove (move.cpp:3624-3826): chain[0 .. Mbar] runs from the
    // pivot to the swap bead; after relinking chain[Mbar] is the old tail
    __device__ int swapTail(float4* orig) {
        if (numBeadsOn == 0 || diag) return -1;
        const int swapLength = m.mbar;
        int pivotSlice = tail.t - swapLength;
        if (pivotSlice < 0) pivotSlice += m.M;
        if (nb(pivotSlice) == 0) return -1;
        WB pivot; int3 wind;
        const double SigmaTail = towerNorm(tail, pivotSlice, -1, rand(), pivot, wind);
        WB b = pivot;
        const LinkWalk lw = links();
        bool bad = false;
        for (int k = 0; k < swapLength; k++) {
            if (eqW(b, head) || isXW(b)) { if (bad) err = WERR_LINK; return -1; }
            if (lane == 0) chain[k] = pack(b);
            b = lw.next(b, bad);
        }
        if (bad) err = WERR_LINK;
        const WB swp = b;
        if (isXW(swp) || eqW(head, swp)) return -1;
        if (lane == 0) chain[swapLength] = pack(swp);
        __syncwarp();
        acc->attempted[WM_ST]++;
        WB dummy; int3 dw;
        const double SigmaSwap = towerNorm(swp, pivotSlice, 1, -1.0f, dummy, dw);
        const float PNorm = (float)fmin(SigmaTail / SigmaSwap, 1.0);
        if (rand() < PNorm) {
            const int nm = swapLength - 1;
            sp1 = swp; sp2 = pivot;
            saveChain(nm, orig);
            const double oldA = chainAction(0, swapLength + 1);
            const WB prevSwap = prev(swp);
            setPrev(tail, prevSwap);
            setPrev(swp, {-1, -1});
            setNext(prevSwap, tail);
            sp1 = tail;
            tail = swp;
            const WB s1 = sp1;
            if (lane == 0) chain[swapLength] = pack(s1);
            stageChain(nm, P(pivot), P(s1), swapLength, wind);
            acc->bead_updates += nm;
            const double newA = chainAction(0, swapLength + 1);
            if (metro(newA - oldA)) { acc->accepted[WM_ST]++; wormUpdate(head, swp); return 1; }
            tail = s1;
            setPrev(tail, {-1, -1});
            setPrev(swp, prevSwap);
            setNext(prevSwap, swp);
            restoreChain(nm, orig);
            sp1 = sp2 = WB{-1, -1};
            diag = 0;
            return 0;
        }
        return 0;
    }

    // EnergyEstimator (estimator.cpp:940-1029), primitive action, E/N of a
    // closed configuration: kinetic term over every bead's next link,
    // potential over the pairs of every slice, the rc = L tail
    // the sums of the primitive energy over slices [t0, t1): the pair
    // potential of every slice (row i against the partners j > i, four
    // partners a lane at a time without branches) and every bead's squared
    // link to the next slice
    // (a team: warp wk sums the slices t0 + wk, t0 + wk + T, ..., and warp 0
    // adds the warps' sums in warp order)
    __device__ __noinline__ double2 energySums(int t0, int t1) {
        if (team > 1) {
            teamPost(2, t0, t1);
            float2 p, k;
            energyShare(pairCtx(), nxt, t0, t1, team, p, k);
            if (lane == 0) { job->hi[0] = p.x; job->lo[0] = p.y; job->khi[0] = k.x; job->klo[0] = k.y; }
            team_sync(bar, 32 * team);
            double pot = 0.0, kin = 0.0;
            for (int q = 0; q < team; ++q) {
                pot += (double)job->hi[q] + (double)job->lo[q];
                kin += (double)job->khi[q] + (double)job->klo[q];
            }
            return make_double2(pot, kin);
        }
        float2 p, k;
        energyShare(pairCtx(), nxt, t0, t1, 1, p, k);
        return make_double2((double)p.x + (double)p.y, (double)k.x + (double)k.y);
    }
    // the energy sums of slices t0, t0 + step, ... below t1 by one warp:
    // (pot, kin) as double-float pairs
    __device__ __noinline__ static void energyShare(const PairCtx c, const int* nx_, int t0, int t1, int step,
                                                    float2& pot_out, float2& kin_out) {
        KahanF pot, kin;
        for (int t = t0; t < t1; t += step) {
            const int n = c.nbs[t];
            const int tn = t + 1 == c.M ? 0 : t + 1;
            const float4* row = c.pos + (size_t)t * c.Ne;
            for (int i = c.lane; i < n; i += 32) {
                const int pn = nx_[(size_t)i * c.M + t];
                if (pn >= 0 && pn < c.Ne) {
                    const float4 ri = row[i], rn = c.pos[(size_t)tn * c.Ne + pn];
                    const float vx = min_image32(rn.x - ri.x, c.L, c.Linv);
                    const float vy = min_image32(rn.y - ri.y, c.L, c.Linv);
                    const float vz = min_image32(rn.z - ri.z, c.L, c.Linv);
                    kin.add(fmaf(vx, vx, fmaf(vy, vy, vz * vz)));
                }
            }
            for (int i = 0; i + 1 < n; ++i) {
                const float4 ri = row[i];
                for (int j0 = i + 1; j0 < n; j0 += 128) {
                    float4 r[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const int j = j0 + 32 * u + c.lane;
                        r[u] = j < n ? row[j] : ri;
                    }
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const bool ok = j0 + 32 * u + c.lane < n;
                        const float dx = min_image32(ri.x - r[u].x, c.L, c.Linv);
                        const float dy = min_image32(ri.y - r[u].y, c.L, c.Linv);
                        const float dz = min_image32(ri.z - r[u].z, c.L, c.Linv);
                        const float r2 = ok ? fmaf(dx, dx, fmaf(dy, dy, dz * dz)) : 1.0f;
                        pot.add(ok ? aziz_v32_sel(r2, c.az) : 0.0f);
                    }
                }
            }
        }
        pot_out = warp_ff(pot);
        kin_out = warp_ff(kin);
    }
    // EnergyEstimator's E/N from the sums over all slices
    __device__ double energyFrom(double V, double K2, int& N) const {
        N = numBeadsOn / m.M;
        if (N <= 0) return 0.0;
        const double totK = 1.5 * N / m.tau - K2 * ((0.25 / (m.lambda * m.tau)) / (m.tau * m.M));
        const double totV = V / m.M + (1.0 * N * N / m.volume) * m.tailV0;
        return (totK + totV) / N;
    }
};


// One walker's launch: run by the single warp of a small walker, or by warp 0
// of a team (team > 1, job the team's mailbox).  limit[w] caps the walker's
// completed sweeps; with budget_ns > 0 a walker stops between two moves (the
// clock read before each) once that much device time has passed, and the
// next launch resumes the sweep there.
//
// diag_only: diagonal pre-equilibration in the manner of
// PathIntegralMonteCarlo::equilStepDiagonal (pimc.cpp:216-300): only
// centre-of-mass and diagonal moves, no worm moves and no energy sample.
// Unlike the reference (centre of mass 1 %, the configured diagonal move, an
// adaptive centre-of-mass step) it makes 5 % centre-of-mass moves and
// staging moves: from seeded worldlines with overlapping particles these
// relax in tens of steps where bisection needs hundreds.
__device__ __noinline__ void run_walker(int w, int team, int bar, TeamJob* job, const WWMeta* __restrict__ meta,
                                        float4* __restrict__ pos, int* __restrict__ nxt, int* __restrict__ prv,
                                        int* __restrict__ nbs, const long long* __restrict__ nbs_off,
                                        WWState* __restrict__ states, pgb_worm_walker_stats* __restrict__ stats,
                                        const AzizF& az, int sweeps, const int* __restrict__ limit,
                                        unsigned long long budget_ns, int diag_only, float4* s_orig,
                                        float4* s_newp, int* s_chain, double* s_scr, double* s_cum,
                                        float2* tpart) {
    WormWalker ww;
    ww.m = meta[w];
    ww.az = az;
    ww.lane = threadIdx.x & 31;
    ww.pos = pos + ww.m.off;
    ww.nxt = nxt + ww.m.off;
    ww.prv = prv + ww.m.off;
    ww.nbs = nbs + nbs_off[w];
    ww.acc = &stats[w];
    ww.chain = s_chain;
    ww.znorm = reinterpret_cast<float*>(s_scr);  // a move's deviates, then its per-bead actions
    ww.acts = s_scr;
    ww.qbuf = s_newp;
    ww.team = team;
    ww.bar = bar;
    ww.wk = 0;
    ww.job = job;
    ww.tpart = tpart;
    const WWState st = states[w];
    if (st.err) return;
    ww.head = WB{st.head[0], st.head[1]}; ww.tail = WB{st.tail[0], st.tail[1]};
    ww.sp1 = WB{st.sp1[0], st.sp1[1]}; ww.sp2 = WB{st.sp2[0], st.sp2[1]};
    ww.gap = st.gap; ww.length = st.length; ww.diag = st.diag; ww.numBeadsOn = st.numBeadsOn;
    ww.sep[0] = st.sep[0]; ww.sep[1] = st.sep[1]; ww.sep[2] = st.sep[2];
    ww.err = 0;
    ww.ctr = 0; ww.bidx = 4;
    // per-walker counters accumulate in a register copy, lane 0 writes back
    pgb_worm_walker_stats local = stats[w];
    ww.acc = &local;
    // cumulative probabilities over the default move list (pimc.cpp:120-152),
    // one copy per warp in shared memory
    double* cumD = s_cum;
    double* cumO = s_cum + WM_N;
    if (ww.lane == 0 && diag_only) {
        for (int i = 0; i < WM_N; ++i) cumD[i] = cumO[i] = 1.0 + 1e-7;
        cumD[WM_COM] = cumO[WM_COM] = 0.05;
    } else if (ww.lane == 0) {
        const double prob[WM_N] = {0.01, 0.19, 0.4, 0.15, 0.4, 0.15, 0.075, 0.075, 0.075, 0.075, 0.1, 0.1};
        const int onDiag[WM_N] = {1, 1, 1, 0, 1, 0, 0, 0, 0, 0, 0, 0};
        double cd = 0.0, co = 0.0;
        for (int i = 0; i < WM_N; ++i) {
            if (onDiag[i]) cd += prob[i];
            cumD[i] = cd;
            if (!onDiag[i] || i < 2) co += prob[i];
            cumO[i] = co;
        }
        cumD[WM_N - 1] = 1.0 + 1e-7;
        cumO[WM_N - 1] = 1.0 + 1e-7;
    }
    __syncwarp();
    float4* orig = s_orig;
    const int lim = limit ? min(sweeps, limit[w]) : sweeps;
    const unsigned long long t0 = __shfl_sync(0xffffffffu, gtimer_ns(), 0);
    // the walker's random stream is indexed by (sweep, draw): each sweep
    // starts at counter sweep << 32, and a sweep stopped part-way resumes at
    // the saved move and draw, so where launches split a run does not change
    // the draws
    unsigned long long sweep_no = st.ctr;
    int u0 = st.upd;
    if (u0 > 0) {
        ww.ctr = st.rctr;
        ww.bidx = st.rbidx;
        if (ww.bidx < 4) {
            const unsigned long long c = ww.ctr - 1;
            ww.buf = philox4x32(make_uint4((uint32_t)c, (uint32_t)(c >> 32), 0x574F524Du, 0u), ww.m.key);
        }
    }
    // an energy sample in progress resumes at its next slice (its sweep's
    // moves are done)
    int eslice = st.epending ? st.eslice : -1;
    double epot = st.epending ? st.epot : 0.0, ekin = st.epending ? st.ekin : 0.0;
    auto out_of_time = [&]() {
        // lane 0's clock for every lane: the decision must be uniform
        if (!budget_ns) return false;
        const unsigned long long now = __shfl_sync(0xffffffffu, gtimer_ns(), 0);
        return now - t0 > budget_ns;
    };
    bool stopped = false;
    for (int sw = 0; sw < lim && !ww.err; ++sw) {
        if (eslice < 0) {
            if (u0 == 0) {
                ww.ctr = sweep_no << 32;
                ww.bidx = 4;
            }
            int u = u0;
            for (; u < ww.m.num_updates && !ww.err; ++u) {
                if (out_of_time()) { stopped = true; break; }
                const double x = ww.rand();
                const double* cum = ww.diag ? cumD : cumO;
                int index = WM_N - 1;
                for (int i = 0; i < WM_N; ++i) if (cum[i] >= x) { index = i; break; }
                bool acc = false;
                int moved = 0;
                switch (index) {
                    case WM_COM: moved = ww.com(acc); local.bead_updates += moved; break;
                    case WM_DIAG:
                        moved = (ww.m.diag_move == 1 || diag_only) ? ww.staging(acc, orig)
                                                                   : ww.bisection(acc, orig, s_newp);
                        local.bead_updates += moved;
                        break;
                    case WM_OPEN: ww.open(); break;
                    case WM_CLOSE: ww.close(); break;
                    case WM_INSERT: ww.insert(); break;
                    case WM_REMOVE: ww.remove(); break;
                    case WM_AH: ww.advanceHead(); break;
                    case WM_RH: ww.recedeHead(); break;
                    case WM_AT: ww.advanceTail(); break;
                    case WM_RT: ww.recedeTail(); break;
                    case WM_SH: ww.swapHead(orig); break;
                    case WM_ST: ww.swapTail(orig); break;
                }
            }
            if (stopped || ww.err) { u0 = u; break; }
            u0 = 0;
            if (ww.diag && !diag_only) { eslice = 0; epot = 0.0; ekin = 0.0; }
        }
        if (eslice >= 0) {
            // the energy sample in chunks of 8 slices, the budget checked
            // between chunks; the chunk sums add in slice order, so where a
            // launch stops does not change the sample
            while (eslice < ww.m.M && !ww.err) {
                if (out_of_time()) { stopped = true; break; }
                const int t1 = min(eslice + 8, ww.m.M);
                const double2 r = ww.energySums(eslice, t1);
                epot += r.x;
                ekin += r.y;
                eslice = t1;
            }
            if (stopped || ww.err) break;
            int N;
            const double e = ww.energyFrom(epot, ekin, N);
            local.samples += 1;
            local.energy_sum += e;
            local.energy_sumsq += e * e;
            local.n_sum += N;
            local.n_sumsq += 1.0 * N * N;
            eslice = -1;
        }
        ++sweep_no;
        local.sweeps += 1;
    }
    __syncwarp();
    if (ww.lane == 0) {
        WWState o;
        o.head[0] = ww.head.t; o.head[1] = ww.head.p; o.tail[0] = ww.tail.t; o.tail[1] = ww.tail.p;
        o.sp1[0] = ww.sp1.t; o.sp1[1] = ww.sp1.p; o.sp2[0] = ww.sp2.t; o.sp2[1] = ww.sp2.p;
        o.gap = ww.gap; o.length = ww.length; o.diag = ww.diag; o.numBeadsOn = ww.numBeadsOn;
        o.sep[0] = ww.sep[0]; o.sep[1] = ww.sep[1]; o.sep[2] = ww.sep[2];
        o.err = ww.err; o.ctr = sweep_no;
        o.upd = u0; o.rctr = ww.ctr; o.rbidx = ww.bidx;
        o.epending = eslice >= 0; o.eslice = eslice < 0 ? 0 : eslice; o.epot = epot; o.ekin = ekin;
        states[w] = o;
        local.error = ww.err;
        stats[w] = local;
    }
}


// the helper warps of a team of T warps (this one the wk-th) meeting at
// named barrier `bar`: take the share that the team's first warp posts until
// it posts the stop
__device__ __noinline__ void team_helper(int w, int wk, int T, int bar, const WWMeta* __restrict__ meta,
                                         float4* __restrict__ pos,
                                         int* __restrict__ nxt, int* __restrict__ nbs,
                                         const long long* __restrict__ nbs_off, const AzizF& az, int* chain,
                                         TeamJob* job, float2* tpart) {
    WormWalker ww;
    ww.m = meta[w];
    ww.az = az;
    ww.lane = threadIdx.x & 31;
    ww.pos = pos + ww.m.off;
    ww.nxt = nxt + ww.m.off;
    ww.nbs = nbs + nbs_off[w];
    ww.chain = chain;
    for (;;) {
        team_sync(bar, 32 * T);
        const int op = job->op;
        if (op == 0) break;
        ww.head = job->head; ww.tail = job->tail; ww.sp1 = job->sp1; ww.sp2 = job->sp2;
        const WormWalker::PairCtx c = ww.pairCtx();
        if (op == 1) {
            bool ok = true;
            const float2 r = WormWalker::teamShare(c, chain, job->a, job->b, wk, T, ok);
            if (ww.lane == 0) { job->hi[wk] = r.x; job->lo[wk] = r.y; job->bad[wk] = ok ? 0 : 1; }
        } else if (op == 3) {
            bool ok = true;
            WormWalker::teamBeadShares(c, chain, job->a, job->b, wk, T, ok, tpart);
            if (ww.lane == 0) job->bad[wk] = ok ? 0 : 1;
        } else {
            float2 p, k;
            WormWalker::energyShare(c, ww.nxt, job->a + wk, job->b, T, p, k);
            if (ww.lane == 0) { job->hi[wk] = p.x; job->lo[wk] = p.y; job->khi[wk] = k.x; job->klo[wk] = k.y; }
        }
        team_sync(bar, 32 * T);
    }
}

// plan[4 b .. 4 b + 3] lists the walkers of CTA b: up to four small walkers
// (-1 for an empty place); or one large walker and kPlanTeam in the second
// place, served by the CTA's four warps as a team; or two walkers in the
// first and third places (the third -1 when there is one) and kPlanPair in
// the second, each served by a team of two warps
constexpr int kPlanTeam = -2;
constexpr int kPlanPair = -3;

__global__ void __launch_bounds__(kCtaWarps * 32)
k_worm_walkers(const WWMeta* __restrict__ meta, float4* __restrict__ pos, int* __restrict__ nxt,
               int* __restrict__ prv, int* __restrict__ nbs, const long long* __restrict__ nbs_off,
               WWState* __restrict__ states, pgb_worm_walker_stats* __restrict__ stats,
               AzizF az, int sweeps, const int* __restrict__ plan, const int* __restrict__ limit,
               unsigned long long budget_ns, int diag_only) {
    __shared__ float4 s_orig[kCtaWarps][kOrigCap];
    __shared__ float4 s_newp[kCtaWarps][kOrigCap];
    __shared__ int s_chain[kCtaWarps][kChainCap];
    __shared__ double s_scr[kCtaWarps][3 * kOrigCap / 2];
    __shared__ double s_cum[kCtaWarps][2 * WM_N];
    __shared__ TeamJob s_job[2];
    const int warp = threadIdx.x >> 5;
    const int* pl = plan + kCtaWarps * blockIdx.x;
    if (pl[1] == kPlanTeam || pl[1] == kPlanPair) {
        const int T = pl[1] == kPlanTeam ? kCtaWarps : 2;
        const int g = warp / T;                 // the team's place in the CTA
        const int first = g * T;                // its first warp
        const int w = pl[2 * g];
        if (w < 0) return;                      // an empty pair place: no barrier is used
        const int bar = 1 + g;
        // a team uses its first warp's buffers; its second warp's chain cache
        // holds the team's per-bead shares
        float2* tpart = reinterpret_cast<float2*>(s_chain[first + 1]);
        if (warp == first) {
            run_walker(w, T, bar, &s_job[g], meta, pos, nxt, prv, nbs, nbs_off, states, stats, az, sweeps, limit,
                       budget_ns, diag_only, s_orig[first], s_newp[first], s_chain[first], s_scr[first],
                       s_cum[first], tpart);
            // every path out of run_walker ends here: release the helpers
            if ((threadIdx.x & 31) == 0) s_job[g].op = 0;
            team_sync(bar, 32 * T);
        } else {
            team_helper(w, warp - first, T, bar, meta, pos, nxt, nbs, nbs_off, az, s_chain[first], &s_job[g],
                        tpart);
        }
        return;
    }
    const int w = pl[warp];
    if (w < 0) return;
    run_walker(w, 1, 1, nullptr, meta, pos, nxt, prv, nbs, nbs_off, states, stats, az, sweeps, limit, budget_ns,
               diag_only, s_orig[warp], s_newp[warp], s_chain[warp], s_scr[warp], s_cum[warp], nullptr);
}

// an admitted job's seeded closed worldlines: particle i's centre uniform in
// the box (Philox block (i, 0)), each of its beads jittered by sigma per
// coordinate (Box-Muller on block (i, t + 1)) and put back in the box,
// identity links, N0 beads on every slice; the unused capacity cleared
__global__ void k_seed_worldlines(float4* __restrict__ pos, int* __restrict__ nxt, int* __restrict__ prv,
                                  int* __restrict__ nbs, int M, int Ne, int N0, float L, float sigma, uint2 key) {
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= (long long)M * Ne) return;
    const int t = (int)(k / Ne), i = (int)(k - (long long)t * Ne);
    if (i < N0) {
        const uint4 c = philox4x32(make_uint4((uint32_t)i, 0u, 0x43454E54u, 0u), key);
        const uint4 g = philox4x32(make_uint4((uint32_t)i, (uint32_t)(t + 1), 0x4A495454u, 0u), key);
        const float2 n01 = box_muller(g.x, g.y), n23 = box_muller(g.z, g.w);
        float r[3] = {L * (u01f(c.x) - 0.5f) + sigma * n01.x, L * (u01f(c.y) - 0.5f) + sigma * n01.y,
                      L * (u01f(c.z) - 0.5f) + sigma * n23.x};
        for (int d = 0; d < 3; ++d) r[d] -= L * floorf(r[d] / L + 0.5f);
        pos[k] = make_float4(r[0], r[1], r[2], 0.f);
        nxt[(size_t)i * M + t] = i;          // links particle-major
        prv[(size_t)i * M + t] = i;
    } else {
        pos[k] = make_float4(0.f, 0.f, 0.f, 0.f);
        nxt[(size_t)i * M + t] = -1;
        prv[(size_t)i * M + t] = -1;
    }
    if (i == 0) nbs[t] = N0;
}

// one warp: walker w's bare potential action of each listed bead, by the
// walkers' own pair sums (FP32 terms, Kahan lanes, double-float warp
// reduction), for checking them against the FP64 oracle on the walker's
// current path.  A bead that is not active on its slice gives 0 with the
// worm factors of the walker's worm state, as the moves evaluate it.
__global__ void k_worm_bead_actions(const WWMeta* __restrict__ meta, float4* pos, int* nxt, int* prv, int* nbs,
                                    const long long* __restrict__ nbs_off, const WWState* __restrict__ states,
                                    AzizF az, int w, const int2* __restrict__ beads, int k, double* out) {
    __shared__ int s_chain[kChainCap];
    WormWalker ww;
    ww.m = meta[w];
    ww.az = az;
    ww.lane = threadIdx.x & 31;
    ww.pos = pos + ww.m.off;
    ww.nxt = nxt + ww.m.off;
    ww.prv = prv + ww.m.off;
    ww.nbs = nbs + nbs_off[w];
    ww.chain = s_chain;
    const WWState st = states[w];
    ww.head = WB{st.head[0], st.head[1]}; ww.tail = WB{st.tail[0], st.tail[1]};
    ww.sp1 = WB{st.sp1[0], st.sp1[1]}; ww.sp2 = WB{st.sp2[0], st.sp2[1]};
    ww.err = 0;
    for (int i = 0; i < k; ++i) {
        const WB b{beads[i].x, beads[i].y};
        const bool on = ww.valid(b) && b.p < ww.nbs[b.t];
        const double v = on ? ww.bare(b) : 0.0;
        if (ww.lane == 0) out[i] = v;
    }
}

// one warp: the serial and the lane-parallel normal deviates from the same
// stream position
__global__ void k_normals_check(uint2 key, int skip, int count, float* serial, float* parallel, int* state) {
    __shared__ float s_out[3 * kOrigCap];
    WormWalker a;
    a.m = WWMeta{};
    a.m.key = key;
    a.lane = threadIdx.x & 31;
    a.ctr = 0; a.bidx = 4;
    for (int i = 0; i < skip; ++i) a.u32();
    WormWalker b = a;
    for (int i = 0; i < count; ++i) {
        const float z = a.randNormZ();
        if (a.lane == 0) serial[i] = z;
    }
    b.normals(count, s_out);
    for (int i = a.lane; i < count; i += 32) parallel[i] = s_out[i];
    if (a.lane == 0) {
        state[0] = (int)(uint32_t)a.ctr; state[1] = (int)(uint32_t)(a.ctr >> 32); state[2] = a.bidx;
        state[3] = (int)(uint32_t)b.ctr; state[4] = (int)(uint32_t)(b.ctr >> 32); state[5] = b.bidx;
    }
}

}  // namespace pgb

// --------------------------------------------------------------------------
// host side
// --------------------------------------------------------------------------
using namespace pgb;

// The CTAs of a launch over walkers listed largest first: a walker of
// N0 >= kTeam4MinN gets a CTA of its own, served by a team of four warps;
// walkers of kTeamMinN <= N0 < kTeam4MinN share CTAs two to one, each served
// by a team of two; the others share CTAs four to one; each kind in the
// same order.  A walker's schedule depends only on its own N0, so its chain
// does not depend on which walkers run beside it.
static int build_plan(const std::vector<int>& order, const std::vector<WWMeta>& meta, std::vector<int>& plan) {
    plan.clear();
    std::vector<int> small;
    int pending = -1;                           // a pair walker waiting for its partner
    for (int w : order) {
        if (meta[w].N0 >= kTeam4MinN) plan.insert(plan.end(), {w, kPlanTeam, -1, -1});
        else if (meta[w].N0 >= kTeamMinN) {
            if (pending < 0) pending = w;
            else { plan.insert(plan.end(), {pending, kPlanPair, w, -1}); pending = -1; }
        } else small.push_back(w);
    }
    if (pending >= 0) plan.insert(plan.end(), {pending, kPlanPair, -1, -1});
    for (size_t i = 0; i < small.size(); i += kCtaWarps)
        for (int k = 0; k < kCtaWarps; ++k) plan.push_back(i + k < small.size() ? small[i + k] : -1);
    return (int)(plan.size() / kCtaWarps);
}

// bisection levels b of ConstantParameters::initConstants
// (constants.cpp:116-120): ceil(log2 Mbar), lowered while 2^b >= M
static int bisection_levels(int mbar, int M) {
    int b = (int)std::ceil(std::log(1.0 * mbar) / std::log(2.0) - 1.0e-7);
    while (b > 1 && (1 << b) >= M) --b;
    return b < 1 ? 1 : b;
}

struct pgb_worm_walkers {
    int W = 0;
    std::vector<WWMeta> meta;
    std::vector<long long> nbs_off;
    long long total_beads = 0, total_slices = 0;
    WWMeta* d_meta = nullptr;
    float4* d_pos = nullptr;
    int *d_nxt = nullptr, *d_prv = nullptr, *d_nbs = nullptr;
    long long* d_nbs_off = nullptr;
    WWState* d_state = nullptr;
    pgb_worm_walker_stats* d_stats = nullptr;
    int* d_plan = nullptr;           // the launch's CTAs (build_plan), the largest walkers first
    int n_cta = 0;
    AzizF az{};
    cudaStream_t stream = nullptr;
    long long launches = 0;          // kernels this handle has launched
    std::string err;
    int cfail(cudaError_t e, const char* where) {
        err = std::string("CUDA error ") + cudaGetErrorString(e) + " at " + where;
        return e == cudaErrorMemoryAllocation ? PGB_ENOMEM : PGB_ECUDA;
    }
};

namespace {
thread_local std::string g_wwerr;
}

extern "C" {

const char* pgb_worm_walkers_last_error(const pgb_worm_walkers* h) { return h ? h->err.c_str() : g_wwerr.c_str(); }

int pgb_worm_walkers_destroy(pgb_worm_walkers* h) {
    if (!h) return PGB_OK;
    if (h->stream) cudaStreamSynchronize(h->stream);
    cudaFree(h->d_meta); cudaFree(h->d_pos); cudaFree(h->d_nxt); cudaFree(h->d_prv); cudaFree(h->d_nbs);
    cudaFree(h->d_nbs_off); cudaFree(h->d_state); cudaFree(h->d_stats); cudaFree(h->d_plan);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return PGB_OK;
}

int pgb_worm_walkers_create(const pgb_worm_walkers_params* p, pgb_worm_walkers** out) {
    if (!out) return PGB_EINVAL;
    *out = nullptr;
    if (!p || p->num_walkers <= 0 || !p->num_ptcl || !p->num_slices || !p->side || !p->mbar ||
        !p->capacity || !(p->tau > 0) || !(p->lambda > 0) || !(p->worm_constant > 0)) {
        g_wwerr = "worm_walkers_create: walker arrays, tau, lambda and C0 are required";
        return PGB_EINVAL;
    }
    int dev = 0;
    if (cudaGetDeviceCount(&dev) != cudaSuccess || dev == 0) {
        cudaGetLastError();
        g_wwerr = "worm_walkers_create: no CUDA device";
        return PGB_ECUDA;
    }
    pgb_worm_walkers* h = new pgb_worm_walkers();
    h->W = p->num_walkers;
    const AzizParams ap = aziz_params(p->aziz_year ? p->aziz_year : 1979);
    h->az = make_aziz_f(ap);
    long long off = 0, soff = 0;
    for (int w = 0; w < h->W; ++w) {
        const int N = p->num_ptcl[w], M = p->num_slices[w], mb = p->mbar[w], ne = p->capacity[w];
        const double L = p->side[w];
        if (N < 1 || M < 4 || M % 2 || M >= kChainCap || mb < 2 || mb % 2 || mb >= M || mb > 64 || ne < N ||
            ne > 4096 || !(L > 0)) {
            g_wwerr = "worm walker " + std::to_string(w) + ": need N >= 1, even 4 <= M < 1024, "
                      "even 2 <= Mbar < M, Mbar <= 64, N <= capacity <= 4096, L > 0";
            pgb_worm_walkers_destroy(h);
            return PGB_EINVAL;
        }
        WWMeta m{};
        m.off = off; m.M = M; m.Ne = ne; m.N0 = N; m.mbar = mb;
        m.blev = bisection_levels(mb, M);
        m.diag_move = p->diagonal_move == 1 ? 1 : 0;
        int nu = (int)std::ceil(std::max(N, 1) * M / (1.0 * mb));
        m.num_updates = nu < 100 ? 100 : nu;
        m.window = p->window;
        m.L = (float)L; m.Linv = (float)(1.0 / L);
        m.tau = p->tau; m.lambda = p->lambda; m.mu = p->mu ? p->mu[w] : 0.0;
        m.volume = L * L * L;
        const double c0 = p->worm_constants ? p->worm_constants[w] : p->worm_constant;
        if (!(c0 > 0)) {
            g_wwerr = "worm walker " + std::to_string(w) + ": the worm constant must be positive";
            pgb_worm_walkers_destroy(h);
            return PGB_EINVAL;
        }
        m.C = c0 / (1.0 * mb * M * m.volume);
        const double rmorc = ap.rm / L;
        const double t2 = ap.C6 * std::pow(rmorc, 3.0) / 3.0, t3 = ap.C8 * std::pow(rmorc, 5.0) / 5.0,
                     t4 = ap.C10 * std::pow(rmorc, 7.0) / 7.0;
        m.tailV0 = 2.0 * M_PI * ap.epsilon * (-ap.rm * ap.rm * ap.rm * (t2 + t3 + t4));
        m.sqrtLambdaTau = std::sqrt(p->lambda * p->tau);
        m.sqrt2LambdaTau = std::sqrt(2.0) * m.sqrtLambdaTau;
        const double T = 1.0 / (M * p->tau);
        m.comDelta = 0.04 * 2.0 * std::sqrt(M_PI * p->lambda / T);
        const uint64_t s = p->seed * 0x9E3779B97F4A7C15ull + (uint64_t)w * 0xBF58476D1CE4E5B9ull + 0x94D049BB133111EBull;
        m.key = make_uint2((uint32_t)s, (uint32_t)(s >> 32));
        h->meta.push_back(m);
        h->nbs_off.push_back(soff);
        off += (long long)M * ne;
        soff += M;
    }
    h->total_beads = off; h->total_slices = soff;
    cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&h->d_meta, h->W * sizeof(WWMeta));
    if (e == cudaSuccess) e = cudaMalloc(&h->d_pos, off * sizeof(float4));
    if (e == cudaSuccess) e = cudaMalloc(&h->d_nxt, off * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&h->d_prv, off * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&h->d_nbs, soff * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&h->d_nbs_off, h->W * sizeof(long long));
    if (e == cudaSuccess) e = cudaMalloc(&h->d_state, h->W * sizeof(WWState));
    if (e == cudaSuccess) e = cudaMalloc(&h->d_stats, h->W * sizeof(pgb_worm_walker_stats));
    if (e == cudaSuccess) e = cudaMalloc(&h->d_plan, (size_t)kCtaWarps * h->W * sizeof(int));
    if (e == cudaSuccess) {
        // the sweep lasts as long as the largest walker needs: start the
        // largest first so that they spread over the SMs
        std::vector<int> order(h->W);
        for (int w = 0; w < h->W; ++w) order[w] = w;
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
            const double ca = 1.0 * h->meta[a].N0 * h->meta[a].N0 * h->meta[a].M;
            const double cb = 1.0 * h->meta[b].N0 * h->meta[b].N0 * h->meta[b].M;
            return ca > cb;
        });
        std::vector<int> plan;
        h->n_cta = build_plan(order, h->meta, plan);
        e = cudaMemcpy(h->d_plan, plan.data(), plan.size() * sizeof(int), cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess) e = cudaMemcpy(h->d_meta, h->meta.data(), h->W * sizeof(WWMeta), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(h->d_nbs_off, h->nbs_off.data(), h->W * sizeof(long long), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(h->d_stats, 0, h->W * sizeof(pgb_worm_walker_stats));
    if (e == cudaSuccess) e = cudaMemset(h->d_nbs, 0, soff * sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(h->d_nxt, 0xff, off * sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(h->d_prv, 0xff, off * sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(h->d_pos, 0, off * sizeof(float4));
    if (e != cudaSuccess) {
        g_wwerr = std::string("worm_walkers_create: ") + cudaGetErrorString(e);
        pgb_worm_walkers_destroy(h);
        return e == cudaErrorMemoryAllocation ? PGB_ENOMEM : PGB_ECUDA;
    }
    // every walker starts empty and diagonal until a configuration is loaded
    std::vector<WWState> st((size_t)h->W);
    for (auto& s : st) {
        s = WWState{};
        for (int i = 0; i < 2; ++i) s.head[i] = s.tail[i] = s.sp1[i] = s.sp2[i] = -1;
        s.gap = -1; s.diag = 1;
    }
    e = cudaMemcpy(h->d_state, st.data(), st.size() * sizeof(WWState), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) { int rc = h->cfail(e, "worm walker state"); g_wwerr = h->err; pgb_worm_walkers_destroy(h); return rc; }
    *out = h;
    return PGB_OK;
}

int pgb_worm_walkers_load(pgb_worm_walkers* h, int w, const double* pos) {
    if (!h || !pos || w < 0 || w >= h->W) return PGB_EINVAL;
    const WWMeta& m = h->meta[w];
    const int N = m.N0, M = m.M, ne = m.Ne;
    // closed worldlines on the identity permutation, beads 0..N-1 of every slice
    std::vector<float4> p((size_t)M * ne, make_float4(0.f, 0.f, 0.f, 0.f));
    std::vector<int> nx((size_t)M * ne, -1), pv((size_t)M * ne, -1), nb(M, N);
    for (int t = 0; t < M; ++t)
        for (int i = 0; i < N; ++i) {
            const double* r = pos + ((size_t)t * N + i) * 3;
            p[(size_t)t * ne + i] = make_float4((float)r[0], (float)r[1], (float)r[2], 0.f);
            nx[(size_t)i * M + t] = i;                 // links particle-major
            pv[(size_t)i * M + t] = i;
        }
    WWState s{};
    for (int i = 0; i < 2; ++i) s.head[i] = s.tail[i] = s.sp1[i] = s.sp2[i] = -1;
    s.gap = -1; s.length = 0; s.diag = 1; s.numBeadsOn = N * M; s.err = 0; s.ctr = 0;
    cudaError_t e = cudaMemcpy(h->d_pos + m.off, p.data(), p.size() * sizeof(float4), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(h->d_nxt + m.off, nx.data(), nx.size() * sizeof(int), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(h->d_prv + m.off, pv.data(), pv.size() * sizeof(int), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(h->d_nbs + h->nbs_off[w], nb.data(), nb.size() * sizeof(int), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(h->d_state + w, &s, sizeof(WWState), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(h->d_stats + w, 0, sizeof(pgb_worm_walker_stats));
    if (e != cudaSuccess) return h->cfail(e, "worm walker load");
    return PGB_OK;
}

// The walkers' state lives in local memory around the helpers that are not
// inlined, and a large walker's positions (up to a megabyte) and links stream
// through L1, so the kernel trades shared memory for L1: a carveout of 25 %
// (two 30 KB CTAs an SM) measured fastest on the 1024-walker workload (27 ms
// a step against 31 ms at 50 %, 35 ms at the smallest that fits one CTA,
// 45 ms at 100 %).
constexpr int kWWCarveoutPercent = 25;
static cudaError_t ww_prefer_l1() { return set_carveout(k_worm_walkers, kWWCarveoutPercent); }

static int ww_launch(pgb_worm_walkers* h, int sweeps, int diag_only) {
    if (!h || sweeps < 0) return PGB_EINVAL;
    if (sweeps == 0) return PGB_OK;
    {
        const cudaError_t ce = ww_prefer_l1();
        if (ce != cudaSuccess) return h->cfail(ce, "worm walkers carveout");
    }
    k_worm_walkers<<<h->n_cta, kCtaWarps * 32, 0, h->stream>>>(h->d_meta, h->d_pos, h->d_nxt, h->d_prv, h->d_nbs,
                                                               h->d_nbs_off, h->d_state, h->d_stats, h->az,
                                                               sweeps, h->d_plan, nullptr, 0ull, diag_only);
    ++h->launches;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return h->cfail(e, "worm walkers run");
    return PGB_OK;
}

int pgb_worm_walkers_run_async(pgb_worm_walkers* h, int sweeps) { return ww_launch(h, sweeps, 0); }

int pgb_worm_walkers_equilibrate(pgb_worm_walkers* h, int sweeps) {
    const int rc = ww_launch(h, sweeps, 1);
    if (rc != PGB_OK || sweeps == 0) return rc;
    cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return h->cfail(e, "worm walkers equilibrate");
    return PGB_OK;
}

int pgb_worm_walkers_run(pgb_worm_walkers* h, int sweeps) {
    const int rc = pgb_worm_walkers_run_async(h, sweeps);
    if (rc != PGB_OK || sweeps == 0) return rc;
    cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return h->cfail(e, "worm walkers run");
    return PGB_OK;
}

void* pgb_worm_walkers_stream(pgb_worm_walkers* h) { return h ? (void*)h->stream : nullptr; }

long long pgb_worm_walkers_launch_count(pgb_worm_walkers* h) { return h ? h->launches : 0; }

int pgb_worm_walkers_seed(pgb_worm_walkers* h, uint64_t seed) {
    if (!h) return PGB_EINVAL;
    cudaError_t e = cudaSuccess;
    std::vector<WWState> st((size_t)h->W);
    for (int w = 0; w < h->W && e == cudaSuccess; ++w) {
        const WWMeta& m = h->meta[w];
        const long long nbe = (long long)m.M * m.Ne;
        const uint64_t ws = seed * 0x9E3779B97F4A7C15ull + (uint64_t)w * 0xD1B54A32D192ED03ull + 0x8CB92BA72F3D8DD7ull;
        k_seed_worldlines<<<(unsigned)((nbe + 255) / 256), 256, 0, h->stream>>>(
            h->d_pos + m.off, h->d_nxt + m.off, h->d_prv + m.off, h->d_nbs + h->nbs_off[w], m.M, m.Ne, m.N0,
            m.L, (float)m.sqrt2LambdaTau, make_uint2((uint32_t)ws, (uint32_t)(ws >> 32)));
        ++h->launches;
        e = cudaGetLastError();
        WWState& s = st[w];
        s = WWState{};
        for (int i = 0; i < 2; ++i) s.head[i] = s.tail[i] = s.sp1[i] = s.sp2[i] = -1;
        s.gap = -1; s.diag = 1; s.numBeadsOn = m.N0 * m.M;
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(h->d_state, st.data(), st.size() * sizeof(WWState), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(h->d_stats, 0, h->W * sizeof(pgb_worm_walker_stats), h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return h->cfail(e, "worm walkers seed");
    return PGB_OK;
}

// The whole device state as one image: positions (float4 per bead), next and
// prev links, bead counts per slice, and the per-walker worm records.
static size_t ww_image_parts(const pgb_worm_walkers* h, size_t part[5]) {
    part[0] = (size_t)h->total_beads * sizeof(float4);
    part[1] = part[2] = (size_t)h->total_beads * sizeof(int);
    part[3] = (size_t)h->total_slices * sizeof(int);
    part[4] = (size_t)h->W * sizeof(WWState);
    return part[0] + part[1] + part[2] + part[3] + part[4];
}

long long pgb_worm_walkers_state_bytes(pgb_worm_walkers* h) {
    if (!h) return 0;
    size_t part[5];
    return (long long)ww_image_parts(h, part);
}

int pgb_worm_walkers_get_state(pgb_worm_walkers* h, void* image) {
    if (!h || !image) return PGB_EINVAL;
    size_t part[5];
    ww_image_parts(h, part);
    char* q = static_cast<char*>(image);
    void* src[5] = {h->d_pos, h->d_nxt, h->d_prv, h->d_nbs, h->d_state};
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < 5 && e == cudaSuccess; ++i) {
        e = cudaMemcpyAsync(q, src[i], part[i], cudaMemcpyDeviceToHost, h->stream);
        q += part[i];
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return h->cfail(e, "worm walkers get state");
    return PGB_OK;
}

int pgb_worm_walkers_set_state_async(pgb_worm_walkers* h, const void* image) {
    if (!h || !image) return PGB_EINVAL;
    size_t part[5];
    ww_image_parts(h, part);
    const char* q = static_cast<const char*>(image);
    void* dst[5] = {h->d_pos, h->d_nxt, h->d_prv, h->d_nbs, h->d_state};
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < 5 && e == cudaSuccess; ++i) {
        e = cudaMemcpyAsync(dst[i], q, part[i], cudaMemcpyHostToDevice, h->stream);
        q += part[i];
    }
    if (e != cudaSuccess) return h->cfail(e, "worm walkers set state");
    return PGB_OK;
}

int pgb_worm_walkers_stats_async(pgb_worm_walkers* h, pgb_worm_walker_stats* out) {
    if (!h || !out) return PGB_EINVAL;
    cudaError_t e = cudaMemcpyAsync(out, h->d_stats, h->W * sizeof(pgb_worm_walker_stats), cudaMemcpyDeviceToHost, h->stream);
    if (e != cudaSuccess) return h->cfail(e, "worm walker stats");
    return PGB_OK;
}

int pgb_worm_walkers_bead_actions(pgb_worm_walkers* h, int w, const int32_t* beads, int k, double* out) {
    if (!h || w < 0 || w >= h->W || !beads || !out || k < 0) return PGB_EINVAL;
    if (k == 0) return PGB_OK;
    const WWMeta& m = h->meta[w];
    for (int i = 0; i < k; ++i)
        if (beads[2 * i] < 0 || beads[2 * i] >= m.M || beads[2 * i + 1] < 0 || beads[2 * i + 1] >= m.Ne) {
            h->err = "worm_walkers_bead_actions: bead outside the walker's arrays";
            return PGB_EINVAL;
        }
    int2* d_b = nullptr;
    double* d_o = nullptr;
    cudaError_t e = cudaMalloc(&d_b, k * sizeof(int2));
    if (e == cudaSuccess) e = cudaMalloc(&d_o, k * sizeof(double));
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_b, beads, k * sizeof(int2), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) {
        k_worm_bead_actions<<<1, 32, 0, h->stream>>>(h->d_meta, h->d_pos, h->d_nxt, h->d_prv, h->d_nbs,
                                                     h->d_nbs_off, h->d_state, h->az, w, d_b, k, d_o);
        ++h->launches;
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, d_o, k * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    cudaFree(d_b);
    cudaFree(d_o);
    if (e != cudaSuccess) return h->cfail(e, "worm walker bead actions");
    return PGB_OK;
}

int pgb_worm_walkers_synchronize(pgb_worm_walkers* h) {
    if (!h) return PGB_EINVAL;
    cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return h->cfail(e, "worm walkers synchronize");
    return PGB_OK;
}

int pgb_worm_walkers_reset_stats(pgb_worm_walkers* h) {
    if (!h) return PGB_EINVAL;
    // keep the error words: a stopped walker stays stopped
    std::vector<pgb_worm_walker_stats> st((size_t)h->W);
    cudaError_t e = cudaMemcpy(st.data(), h->d_stats, st.size() * sizeof(pgb_worm_walker_stats), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return h->cfail(e, "worm walker stats");
    for (auto& x : st) { const int er = x.error; x = pgb_worm_walker_stats{}; x.error = er; }
    e = cudaMemcpy(h->d_stats, st.data(), st.size() * sizeof(pgb_worm_walker_stats), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return h->cfail(e, "worm walker stats");
    return PGB_OK;
}

int pgb_worm_walkers_stats(pgb_worm_walkers* h, pgb_worm_walker_stats* out) {
    if (!h || !out) return PGB_EINVAL;
    cudaError_t e = cudaMemcpy(out, h->d_stats, h->W * sizeof(pgb_worm_walker_stats), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return h->cfail(e, "worm walker stats");
    return PGB_OK;
}

int pgb_worm_walkers_get_path(pgb_worm_walkers* h, int w, double* pos, int32_t* next, int32_t* prev,
                              uint8_t* on, int32_t* worm8) {
    if (!h || w < 0 || w >= h->W || !pos || !next || !prev || !on || !worm8) return PGB_EINVAL;
    const WWMeta& m = h->meta[w];
    const int M = m.M, ne = m.Ne;
    std::vector<float4> p((size_t)M * ne);
    std::vector<int> nx((size_t)M * ne), pv((size_t)M * ne), nb(M);
    WWState s;
    cudaError_t e = cudaMemcpy(p.data(), h->d_pos + m.off, p.size() * sizeof(float4), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(nx.data(), h->d_nxt + m.off, nx.size() * sizeof(int), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(pv.data(), h->d_prv + m.off, pv.size() * sizeof(int), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(nb.data(), h->d_nbs + h->nbs_off[w], nb.size() * sizeof(int), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&s, h->d_state + w, sizeof(WWState), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return h->cfail(e, "worm walker path");
    for (int t = 0; t < M; ++t)
        for (int q = 0; q < ne; ++q) {
            const size_t j = (size_t)t * ne + q;
            pos[3 * j] = p[j].x; pos[3 * j + 1] = p[j].y; pos[3 * j + 2] = p[j].z;
            const bool act = q < nb[t];
            on[j] = act ? 1 : 0;
            const int tn = t + 1 == M ? 0 : t + 1, tp = t == 0 ? M - 1 : t - 1;
            const size_t k = (size_t)q * M + t;        // links particle-major
            next[2 * j] = (act && nx[k] >= 0) ? tn : -1; next[2 * j + 1] = (act && nx[k] >= 0) ? nx[k] : -1;
            prev[2 * j] = (act && pv[k] >= 0) ? tp : -1; prev[2 * j + 1] = (act && pv[k] >= 0) ? pv[k] : -1;
        }
    const int wv[8] = {s.head[0], s.head[1], s.tail[0], s.tail[1], s.sp1[0], s.sp1[1], s.sp2[0], s.sp2[1]};
    for (int i = 0; i < 8; ++i) worm8[i] = wv[i];
    return PGB_OK;
}

}  // extern "C"

// --------------------------------------------------------------------------
// Grand-canonical job server over the worm walkers: the canonical server's
// interface (jobs arrive, are admitted when their arrays fit the HBM budget,
// run together in shared launches, stream estimator bins back), with every
// job a device worm walker at its own chemical potential.
// --------------------------------------------------------------------------
namespace {

struct WPool {
    std::map<long long, long long> free_blocks;      // offset -> length
    void init(long long n) { free_blocks.clear(); if (n > 0) free_blocks[0] = n; }
    long long alloc(long long n) {
        for (auto it = free_blocks.begin(); it != free_blocks.end(); ++it)
            if (it->second >= n) {
                const long long off = it->first, len = it->second;
                free_blocks.erase(it);
                if (len > n) free_blocks[off + n] = len - n;
                return off;
            }
        return -1;
    }
    void release(long long off, long long n) {
        auto it = free_blocks.emplace(off, n).first;
        auto nx = std::next(it);
        if (nx != free_blocks.end() && it->first + it->second == nx->first) { it->second += nx->second; free_blocks.erase(nx); }
        if (it != free_blocks.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) { pv->second += it->second; free_blocks.erase(it); }
        }
    }
};

struct WServerJob {
    pgb_job_spec spec{};
    int state = 0;
    double t_admit = -1, t_first = -1, t_done = -1;
    long long sweeps_done = 0, bin_start = 0, samples0 = 0;
    double esum0 = 0.0;
    int bins = 0;
    int M = 0, N0 = 0, Ne = 0, mbar = 0;
    double L = 0;
    int slot = -1;
    long long bead_off = -1, slice_off = -1;
    size_t bytes = 0;
};

thread_local std::string g_wserr;

}  // namespace

struct pgb_worm_server {
    pgb_server_params p{};
    AzizParams ap{};
    AzizF az{};
    int diag_move = 0;               // 0 bisection, 1 staging
    int max_slots = 0;
    std::vector<int> slot_job, free_slots;
    std::vector<WServerJob> jobs;
    std::deque<int> queue;
    std::vector<pgb_bin> bins;
    WPool beads, slices;
    long long n_beads = 0, n_slices = 0;
    float4* d_pos = nullptr;
    int *d_nxt = nullptr, *d_prv = nullptr, *d_nbs = nullptr;
    WWMeta* d_meta = nullptr;
    WWState* d_state = nullptr;
    pgb_worm_walker_stats* d_stats = nullptr;
    long long* d_nbs_off = nullptr;
    int *d_plan = nullptr, *d_limit = nullptr;
    std::vector<WWMeta> h_meta;
    std::vector<long long> h_nbs_off;
    std::vector<int> h_limit;
    std::vector<int> h_plan;         // the round's CTAs (build_plan)
    cudaStream_t stream = nullptr;
    std::chrono::steady_clock::time_point t0;
    long long bead_updates = 0;
    std::string err;
    int fail(int code, const std::string& m) { err = m; return code; }
    int cfail(cudaError_t e, const char* where) {
        err = std::string("CUDA error ") + cudaGetErrorString(e) + " at " + where;
        return e == cudaErrorMemoryAllocation ? PGB_ENOMEM : PGB_ECUDA;
    }
    double now() const { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); }
};

extern "C" {

const char* pgb_worm_server_last_error(const pgb_worm_server* s) { return s ? s->err.c_str() : g_wserr.c_str(); }

int pgb_worm_server_destroy(pgb_worm_server* s) {
    if (!s) return PGB_OK;
    if (s->stream) cudaStreamSynchronize(s->stream);
    cudaFree(s->d_pos); cudaFree(s->d_nxt); cudaFree(s->d_prv); cudaFree(s->d_nbs);
    cudaFree(s->d_meta); cudaFree(s->d_state); cudaFree(s->d_stats); cudaFree(s->d_nbs_off);
    cudaFree(s->d_plan); cudaFree(s->d_limit);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return PGB_OK;
}

int pgb_worm_server_create(const pgb_server_params* p, pgb_worm_server** out) {
    if (!out) return PGB_EINVAL;
    *out = nullptr;
    if (!p || p->hbm_budget_bytes < 1e6 || p->max_active <= 0 || p->sweeps_per_round <= 0 ||
        p->bin_sweeps <= 0 || p->tau <= 0 || p->lambda <= 0 || !(p->round_seconds >= 0.0) ||
        p->round_seconds > 10.0) {
        g_wserr = "worm_server_create: need budget >= 1 MB, max_active > 0, sweeps_per_round > 0, "
                  "bin_sweeps > 0, 0 <= round_seconds <= 10";
        return PGB_EINVAL;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { cudaGetLastError(); g_wserr = "no CUDA device available"; return PGB_ECUDA; }
    pgb_worm_server* s = new pgb_worm_server();
    s->p = *p;
    s->ap = aziz_params(p->aziz_year ? p->aziz_year : 1979);
    s->az = make_aziz_f(s->ap);
    s->diag_move = p->diagonal_move == 1 ? 1 : 0;
    s->max_slots = p->max_active;
    // the budget: bead arrays (24 B a bead), slice counters sized from them
    s->n_beads = (long long)(p->hbm_budget_bytes / 24.0);
    s->n_slices = s->n_beads / 8 + 1;
    s->beads.init(s->n_beads); s->slices.init(s->n_slices);
    s->slot_job.assign(s->max_slots, -1);
    for (int k = s->max_slots - 1; k >= 0; --k) s->free_slots.push_back(k);
    s->h_meta.assign(s->max_slots, WWMeta{});
    s->h_nbs_off.assign(s->max_slots, 0);
    s->h_limit.assign(s->max_slots, 0);
    s->t0 = std::chrono::steady_clock::now();
    cudaError_t e;
    do {
        if ((e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking)) != cudaSuccess) break;
        if ((e = cudaMalloc(&s->d_pos, s->n_beads * sizeof(float4))) != cudaSuccess) break;
        if ((e = cudaMalloc(&s->d_nxt, s->n_beads * sizeof(int))) != cudaSuccess) break;
        if ((e = cudaMalloc(&s->d_prv, s->n_beads * sizeof(int))) != cudaSuccess) break;
        if ((e = cudaMalloc(&s->d_nbs, s->n_slices * sizeof(int))) != cudaSuccess) break;
        if ((e = cudaMalloc(&s->d_meta, s->max_slots * sizeof(WWMeta))) != cudaSuccess) break;
        if ((e = cudaMalloc(&s->d_state, s->max_slots * sizeof(WWState))) != cudaSuccess) break;
        if ((e = cudaMalloc(&s->d_stats, s->max_slots * sizeof(pgb_worm_walker_stats))) != cudaSuccess) break;
        if ((e = cudaMalloc(&s->d_nbs_off, s->max_slots * sizeof(long long))) != cudaSuccess) break;
        if ((e = cudaMalloc(&s->d_plan, (size_t)kCtaWarps * s->max_slots * sizeof(int))) != cudaSuccess) break;
        if ((e = cudaMalloc(&s->d_limit, s->max_slots * sizeof(int))) != cudaSuccess) break;
    } while (0);
    if (e != cudaSuccess) {
        g_wserr = std::string("worm_server_create: ") + cudaGetErrorString(e);
        pgb_worm_server_destroy(s);
        return e == cudaErrorMemoryAllocation ? PGB_ENOMEM : PGB_ECUDA;
    }
    *out = s;
    return PGB_OK;
}

int pgb_worm_server_submit(pgb_worm_server* s, const pgb_job_spec* j, int* job_id) {
    if (!s || !j) return PGB_EINVAL;
    if (j->n < 1 || j->n > 2000 || j->temperature <= 0 || j->density <= 0 || j->sweeps <= 0)
        return s->fail(PGB_EINVAL, "job: need 1 <= n <= 2000, temperature > 0, density > 0, sweeps > 0");
    WServerJob job;
    job.spec = *j;
    job.N0 = j->n;
    int M = (int)std::lround(1.0 / (j->temperature * s->p.tau));
    if (M % 2) M += 1;
    if (M < 4) M = 4;
    job.M = M;
    job.L = std::cbrt(j->n / j->density);
    // Mbar (setup.cpp:1079-1104), even, at most 64 and below M
    const double ell = std::pow(1.0 * j->n / (job.L * job.L * job.L), -1.0 / 3.0);
    int mb = (int)(ell * ell / (16.0 * s->p.lambda * s->p.tau));
    if (mb < 2) mb = 2; else if (mb > M) mb = M / 2;
    if (mb % 2) mb += 1;
    mb = std::min(mb, 64);
    if (mb >= M) mb = (M / 2) % 2 ? M / 2 - 1 : M / 2;
    if (mb < 2) mb = 2;
    job.mbar = mb;
    job.Ne = 2 * j->n + 8;
    job.bytes = (size_t)M * job.Ne * 24 + (size_t)M * 4;
    if (job.Ne > 4096) return s->fail(PGB_EINVAL, "job: n too large for one walker");
    if (job.M >= kChainCap) return s->fail(PGB_EINVAL, "job: temperature too low for one walker (M < 1024)");
    s->jobs.push_back(job);
    if (job_id) *job_id = (int)s->jobs.size() - 1;
    return PGB_OK;
}

int pgb_worm_server_step(pgb_worm_server* s, int* n_active, int* n_queued) {
    if (!s) return PGB_EINVAL;
    const double now = s->now();
    for (size_t k = 0; k < s->jobs.size(); ++k)
        if (s->jobs[k].state == 0 && s->jobs[k].spec.arrival <= now) { s->jobs[k].state = 1; s->queue.push_back((int)k); }
    cudaError_t e = cudaSuccess;
    // admission: FIFO while a slot and both pools have room
    while (!s->queue.empty() && !s->free_slots.empty()) {
        WServerJob& job = s->jobs[s->queue.front()];
        const long long nb = (long long)job.M * job.Ne, ns = job.M;
        const long long bo = s->beads.alloc(nb);
        if (bo < 0) break;
        const long long so = s->slices.alloc(ns);
        if (so < 0) { s->beads.release(bo, nb); break; }
        job.bead_off = bo; job.slice_off = so;
        job.slot = s->free_slots.back();
        s->free_slots.pop_back();
        job.state = 2;
        job.t_admit = now;
        const int k = job.slot;
        s->slot_job[k] = s->queue.front();
        s->queue.pop_front();
        WWMeta m{};
        m.off = bo; m.M = job.M; m.Ne = job.Ne; m.N0 = job.N0; m.mbar = job.mbar;
        m.blev = bisection_levels(job.mbar, job.M);
        m.diag_move = s->diag_move;
        int nu = (int)std::ceil(std::max(job.N0, 1) * job.M / (1.0 * job.mbar));
        m.num_updates = nu < 100 ? 100 : nu;
        m.window = -1;                        // grand canonical
        m.L = (float)job.L; m.Linv = (float)(1.0 / job.L);
        m.tau = s->p.tau; m.lambda = s->p.lambda; m.mu = job.spec.mu;
        m.volume = job.L * job.L * job.L;
        m.C = 1.0 / (1.0 * job.mbar * job.M * m.volume);      // worm constant C0 = 1
        const double rmorc = s->ap.rm / job.L;
        const double t2 = s->ap.C6 * std::pow(rmorc, 3.0) / 3.0, t3 = s->ap.C8 * std::pow(rmorc, 5.0) / 5.0,
                     t4 = s->ap.C10 * std::pow(rmorc, 7.0) / 7.0;
        m.tailV0 = 2.0 * M_PI * s->ap.epsilon * (-s->ap.rm * s->ap.rm * s->ap.rm * (t2 + t3 + t4));
        m.sqrtLambdaTau = std::sqrt(s->p.lambda * s->p.tau);
        m.sqrt2LambdaTau = std::sqrt(2.0) * m.sqrtLambdaTau;
        const double T = 1.0 / (job.M * s->p.tau);
        m.comDelta = 0.04 * 2.0 * std::sqrt(M_PI * s->p.lambda / T);
        const uint64_t sd = job.spec.seed * 0x9E3779B97F4A7C15ull + 0x94D049BB133111EBull;
        m.key = make_uint2((uint32_t)sd, (uint32_t)(sd >> 32));
        s->h_meta[k] = m;
        s->h_nbs_off[k] = so;
        // the job's seeded worldlines are made on the device; its constants,
        // slice offset and initial state are uploaded once (pageable copies
        // return once the source is staged)
        const long long nbe = (long long)job.M * job.Ne;
        const uint64_t ws = job.spec.seed * 0xD1B54A32D192ED03ull + 0x8CB92BA72F3D8DD7ull;
        k_seed_worldlines<<<(unsigned)((nbe + 255) / 256), 256, 0, s->stream>>>(
            s->d_pos + bo, s->d_nxt + bo, s->d_prv + bo, s->d_nbs + so, job.M, job.Ne, job.N0, (float)job.L,
            (float)std::sqrt(2.0 * s->p.lambda * s->p.tau), make_uint2((uint32_t)ws, (uint32_t)(ws >> 32)));
        if (e == cudaSuccess) e = cudaGetLastError();
        WWState st{};
        for (int i = 0; i < 2; ++i) st.head[i] = st.tail[i] = st.sp1[i] = st.sp2[i] = -1;
        st.gap = -1; st.diag = 1; st.numBeadsOn = job.N0 * job.M;
        if (e == cudaSuccess) e = cudaMemcpyAsync(s->d_state + k, &st, sizeof(WWState), cudaMemcpyHostToDevice, s->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(s->d_meta + k, &s->h_meta[k], sizeof(WWMeta), cudaMemcpyHostToDevice, s->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(s->d_nbs_off + k, &s->h_nbs_off[k], sizeof(long long), cudaMemcpyHostToDevice, s->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(s->d_stats + k, 0, sizeof(pgb_worm_walker_stats), s->stream);
        if (e != cudaSuccess) return s->cfail(e, "worm server admit");
    }
    std::vector<int> active;
    for (int k = 0; k < s->max_slots; ++k) {
        if (s->slot_job[k] < 0) { s->h_limit[k] = 0; continue; }
        WServerJob& job = s->jobs[s->slot_job[k]];
        // never past the job's end or its current bin
        const long long left = job.spec.sweeps - job.sweeps_done;
        const long long bin_left = s->p.bin_sweeps - (job.sweeps_done - job.bin_start);
        long long cap = std::min(left, bin_left);
        if (s->p.round_seconds <= 0.0) cap = std::min<long long>(cap, s->p.sweeps_per_round);
        s->h_limit[k] = (int)std::max<long long>(cap, 1);
        active.push_back(k);
    }
    std::stable_sort(active.begin(), active.end(), [&](int a, int b) {
        const WWMeta& ma = s->h_meta[a];
        const WWMeta& mb = s->h_meta[b];
        return 1.0 * ma.N0 * ma.N0 * ma.M > 1.0 * mb.N0 * mb.N0 * mb.M;
    });
    if (e == cudaSuccess) e = cudaMemcpyAsync(s->d_limit, s->h_limit.data(), s->max_slots * sizeof(int), cudaMemcpyHostToDevice, s->stream);
    const int n_cta = active.empty() ? 0 : build_plan(active, s->h_meta, s->h_plan);
    if (e == cudaSuccess && n_cta > 0)
        e = cudaMemcpyAsync(s->d_plan, s->h_plan.data(), s->h_plan.size() * sizeof(int), cudaMemcpyHostToDevice,
                            s->stream);
    if (e != cudaSuccess) return s->cfail(e, "worm server upload");
    if (n_cta > 0) {
        const bool timed = s->p.round_seconds > 0.0;
        if ((e = ww_prefer_l1()) != cudaSuccess) return s->cfail(e, "worm server carveout");
        k_worm_walkers<<<n_cta, kCtaWarps * 32, 0, s->stream>>>(
            s->d_meta, s->d_pos, s->d_nxt, s->d_prv, s->d_nbs, s->d_nbs_off, s->d_state, s->d_stats,
            s->az, timed ? (1 << 30) : s->p.sweeps_per_round,
            s->d_plan, s->d_limit, timed ? (unsigned long long)(s->p.round_seconds * 1e9) : 0ull, 0);
        if ((e = cudaGetLastError()) != cudaSuccess) return s->cfail(e, "worm server launch");
    }
    std::vector<pgb_worm_walker_stats> st(s->max_slots);
    e = cudaMemcpyAsync(st.data(), s->d_stats, s->max_slots * sizeof(pgb_worm_walker_stats), cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return s->cfail(e, "worm server round");
    const double t_end = s->now();
    for (int k : active) {
        const int jid = s->slot_job[k];
        WServerJob& job = s->jobs[jid];
        const pgb_worm_walker_stats& a = st[k];
        job.sweeps_done = a.sweeps;
        const bool failed = a.error != 0;
        const bool finished = failed || job.sweeps_done >= job.spec.sweeps;
        if (job.sweeps_done - job.bin_start >= s->p.bin_sweeps || (finished && job.sweeps_done > job.bin_start)) {
            pgb_bin b;
            b.job = jid;
            b.bin = job.bins++;
            b.samples = a.samples - job.samples0;
            b.energy_per_particle = b.samples > 0 ? (a.energy_sum - job.esum0) / (double)b.samples
                                                  : std::numeric_limits<double>::quiet_NaN();
            b.time = t_end;
            s->bins.push_back(b);
            if (job.t_first < 0) job.t_first = t_end;
            job.bin_start = job.sweeps_done;
            job.samples0 = a.samples;
            job.esum0 = a.energy_sum;
        }
        if (finished) {
            job.state = failed ? 4 : 3;
            job.t_done = t_end;
            s->bead_updates += a.bead_updates;
            s->beads.release(job.bead_off, (long long)job.M * job.Ne);
            s->slices.release(job.slice_off, job.M);
            s->slot_job[k] = -1;
            s->free_slots.push_back(k);
            job.slot = -1;
        }
    }
    int na = 0;
    for (int k = 0; k < s->max_slots; ++k) na += s->slot_job[k] >= 0;
    if (n_active) *n_active = na;
    if (n_queued) *n_queued = (int)s->queue.size();
    return PGB_OK;
}

int pgb_worm_server_poll_bins(pgb_worm_server* s, pgb_bin* out, int cap, int* n) {
    if (!s || !n || cap < 0 || (cap > 0 && !out)) return PGB_EINVAL;
    const int k = std::min<int>(cap, (int)s->bins.size());
    for (int i = 0; i < k; ++i) out[i] = s->bins[i];
    s->bins.erase(s->bins.begin(), s->bins.begin() + k);
    *n = k;
    return PGB_OK;
}

int pgb_worm_server_job_info(pgb_worm_server* s, int jid, pgb_job_info* out) {
    if (!s || !out || jid < 0 || jid >= (int)s->jobs.size()) return PGB_EINVAL;
    const WServerJob& j = s->jobs[jid];
    out->state = j.state;
    out->arrival = j.spec.arrival;
    out->admitted = j.t_admit;
    out->first_bin = j.t_first;
    out->completed = j.t_done;
    out->sweeps_done = j.sweeps_done;
    out->n = j.N0;
    out->m = j.M;
    out->bytes = j.bytes;
    return PGB_OK;
}

double pgb_worm_server_clock(pgb_worm_server* s) { return s ? s->now() : 0.0; }

int pgb_worm_server_active_bead_updates(pgb_worm_server* s, long long* total) {
    if (!s || !total) return PGB_EINVAL;
    std::vector<pgb_worm_walker_stats> st(s->max_slots);
    cudaError_t e = cudaMemcpyAsync(st.data(), s->d_stats, s->max_slots * sizeof(pgb_worm_walker_stats), cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return s->cfail(e, "worm server stats");
    long long t = s->bead_updates;
    for (int k = 0; k < s->max_slots; ++k) if (s->slot_job[k] >= 0) t += st[k].bead_updates;
    *total = t;
    return PGB_OK;
}

}  // extern "C"

extern "C" int pgb_worm_normals_check(uint64_t seed, int skip, int count, float* serial, float* parallel,
                                      int32_t state[6]) {
    using namespace pgb;
    if (!serial || !parallel || !state || count < 1 || count > 3 * kOrigCap || skip < 0 || skip > 1000000)
        return PGB_EINVAL;
    const uint64_t sd = seed * 0x9E3779B97F4A7C15ull + 0x94D049BB133111EBull;
    float *d_s = nullptr, *d_p = nullptr;
    int* d_st = nullptr;
    cudaError_t e = cudaMalloc(&d_s, count * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&d_p, count * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&d_st, 6 * sizeof(int));
    if (e == cudaSuccess) {
        k_normals_check<<<1, 32>>>(make_uint2((uint32_t)sd, (uint32_t)(sd >> 32)), skip, count, d_s, d_p, d_st);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(serial, d_s, count * sizeof(float), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(parallel, d_p, count * sizeof(float), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(state, d_st, 6 * sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(d_s); cudaFree(d_p); cudaFree(d_st);
    return e == cudaSuccess ? PGB_OK : PGB_ECUDA;
}
