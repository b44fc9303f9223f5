// plain_moves.cu -- the plain form: the reference's diagonal move loop driven
// from the host, one FP64 device action evaluation per Metropolis decision.
//
// Move semantics and random-number consumption follow src/move.cpp
// (CenterOfMassMove 1124-1262, StagingMove 1315-1412 with the winding-sector
// sampling of MoveBase 301-397, BisectionMove 1484-1707) and the step driver
// of src/pimc.cpp:189-208, 724-741, so a run with the same MT19937 seed makes
// the same accept/reject decisions as the reference CPU path.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <vector>

#include "pgb_internal.h"

namespace {

using pgb::Ctx;
using dVec = std::array<double, 3>;
using Bead = std::array<int, 2>;
constexpr double EPS = 1.0e-7;
constexpr int XXX = -1;

// MT19937 with the conversions of include/MersenneTwister.h:290-367
struct MT {
    uint32_t* st; int* left; int* pos;
    static constexpr int N = 624, Mm = 397;
    static uint32_t twist(uint32_t m, uint32_t s0, uint32_t s1) {
        return m ^ (((s0 & 0x80000000u) | (s1 & 0x7fffffffu)) >> 1) ^ ((s1 & 1u) ? 0x9908b0dfu : 0u);
    }
    void reload() {
        int i = 0;
        for (; i < N - Mm; ++i) st[i] = twist(st[i + Mm], st[i], st[i + 1]);
        for (; i < N - 1; ++i) st[i] = twist(st[i + Mm - N], st[i], st[i + 1]);
        st[N - 1] = twist(st[Mm - 1], st[N - 1], st[0]);
        *left = N; *pos = 0;
    }
    uint32_t randInt() {
        if (*left == 0) reload();
        --*left;
        uint32_t y = st[(*pos)++];
        y ^= (y >> 11); y ^= (y << 7) & 0x9d2c5680u; y ^= (y << 15) & 0xefc60000u;
        return y ^ (y >> 18);
    }
    uint32_t randInt(uint32_t n) {
        uint32_t used = n;
        used |= used >> 1; used |= used >> 2; used |= used >> 4; used |= used >> 8; used |= used >> 16;
        uint32_t i;
        do { i = randInt() & used; } while (i > n);
        return i;
    }
    double rand() { return double(randInt()) * (1.0 / 4294967295.0); }
    double randNorm(double mean, double sd) {
        double x, y, r;
        do { x = 2.0 * rand() - 1.0; y = 2.0 * rand() - 1.0; r = x * x + y * y; }
        while (r >= 1.0 || r == 0.0);
        double s = std::sqrt(-2.0 * std::log(r) / r);
        return mean + x * s * sd;
    }
};

struct Plain {
    Ctx& c;
    MT R;
    pgb_move_params mp;
    pgb_move_stats st{};
    std::vector<double> pos;    // host mirror AoS [M][Ne][3]
    double sqrtLambdaTau, sqrt2LambdaTau, comDelta;
    int b, numWind;
    std::vector<std::array<int,3>> winding;
    std::vector<double> cumrho0;
    int shift = 1;
    int err = PGB_OK;

    Plain(Ctx& cc, const pgb_move_params& p) : c(cc), mp(p) {
        R.st = c.mt_state.data(); R.left = &c.mt_left; R.pos = &c.mt_pos;
        sqrtLambdaTau = std::sqrt(c.p.lambda * c.p.tau);
        sqrt2LambdaTau = std::sqrt(2.0) * sqrtLambdaTau;
        comDelta = 0.04 * 2.0 * std::sqrt(M_PI * c.p.lambda / mp.temperature);
        b = int(std::ceil(std::log(1.0 * mp.mbar) / std::log(2.0) - EPS));
        while ((int)std::floor(std::pow(2.0, 1.0 * b) + EPS) >= c.M) b--;
        int mw = mp.max_wind;
        numWind = 1;
        for (int i = 0; i < 3; ++i) numWind *= (2 * mw + 1);
        for (int n = 0; n < numWind; n++) {
            std::array<int,3> w{0, 0, 0};
            for (int i = 0; i < 3; i++) {
                int scale = 1;
                for (int j = i + 1; j < 3; j++) scale *= (2 * mw + 1);
                w[i] = (n / scale) % (2 * mw + 1);
                w[i] -= (w[i] > mw) * (2 * mw + 1);
            }
            winding.push_back(w);
        }
        cumrho0.resize(numWind);
    }
    void putInBC(dVec& r) const {
        for (int i = 0; i < 3; ++i) r[i] -= c.p.side[i] * std::floor(r[i] * (1.0 / c.p.side[i]) + 0.5);
    }
    dVec P(Bead bd) const { const double* q = &pos[((size_t)bd[0] * c.Ne + bd[1]) * 3]; return {q[0], q[1], q[2]}; }
    Bead next(Bead bd) const { size_t i = ((size_t)bd[0] * c.Ne + bd[1]) * 2; return {c.h_next[i], c.h_next[i + 1]}; }
    Bead prev(Bead bd) const { size_t i = ((size_t)bd[0] * c.Ne + bd[1]) * 2; return {c.h_prev[i], c.h_prev[i + 1]}; }
    Bead nextN(Bead bd, int n) const { for (int i = 0; i < n; ++i) bd = next(bd); return bd; }
    Bead prevN(Bead bd, int n) const { for (int i = 0; i < n; ++i) bd = prev(bd); return bd; }
    bool on(Bead bd) const { return c.h_on[(size_t)bd[0] * c.Ne + bd[1]] != 0; }
    static bool isX(Bead bd) { return bd[0] == XXX && bd[1] == XXX; }
    dVec sep(Bead a, Bead bb) const { dVec d; dVec ra = P(a), rb = P(bb); for (int i = 0; i < 3; ++i) d[i] = ra[i] - rb[i]; putInBC(d); return d; }

    // device updates of a set of beads (host mirror first)
    void set(const std::vector<Bead>& beads, const std::vector<dVec>& p) {
        if (beads.empty() || err) return;
        std::vector<int32_t> bl; std::vector<double> pl;
        for (size_t i = 0; i < beads.size(); ++i) {
            bl.push_back(beads[i][0]); bl.push_back(beads[i][1]);
            for (int d = 0; d < 3; ++d) { pl.push_back(p[i][d]); pos[((size_t)beads[i][0] * c.Ne + beads[i][1]) * 3 + d] = p[i][d]; }
        }
        err = pgb_update_beads(reinterpret_cast<pgb_ctx*>(&c), bl.data(), pl.data(), (int)beads.size());
    }
    double action_list(const std::vector<Bead>& beads) {
        if (err) return 0.0;
        std::vector<int32_t> bl;
        for (auto& bd : beads) if (on(bd)) { bl.push_back(bd[0]); bl.push_back(bd[1]); }
        double tot = 0.0;
        err = pgb_bead_actions(reinterpret_cast<pgb_ctx*>(&c), bl.data(), (int)bl.size() / 2, shift,
                               PGB_ACTION_FULL, nullptr, &tot);
        return tot;
    }
    double action_range(Bead s, Bead e) {
        std::vector<Bead> l;
        Bead bd = s, stop = next(e);
        do { l.push_back(bd); bd = next(bd); } while (!(bd == stop));
        return action_list(l);
    }
    double rho0(const dVec& vel, int Mx) {
        double n = std::pow(4.0 * M_PI * c.p.lambda * Mx * c.p.tau, -0.5 * 3);
        double d = 0.0; for (int i = 0; i < 3; ++i) d += vel[i] * vel[i];
        return n * std::exp(-d / (4.0 * c.p.lambda * Mx * c.p.tau));
    }
    std::array<int,3> sampleWinding(Bead sb, Bead eb, int L) {
        dVec pe = P(eb), ps = P(sb), vel;
        for (int i = 0; i < 3; ++i) vel[i] = pe[i] - ps[i];
        cumrho0[0] = rho0(vel, L);
        double total = cumrho0[0];
        for (int n = 1; n < numWind; n++) {
            dVec vw; for (int i = 0; i < 3; ++i) vw[i] = vel[i] + winding[n][i] * c.p.side[i];
            double cr = rho0(vw, L);
            total += cr;
            cumrho0[n] = cumrho0[n - 1] + cr;
        }
        for (auto& x : cumrho0) x /= total;
        int idx = int(std::lower_bound(cumrho0.begin(), cumrho0.end(), R.rand()) - cumrho0.begin());
        if (idx >= numWind) idx = numWind - 1;
        return winding[idx];
    }
    dVec stagingPos(Bead nb, Bead eb, int L, int k, std::array<int,3>& wind) {
        double f1 = 1.0 * (L - k - 1), f2 = 1.0 / (1.0 * (L - k));
        double sg = sqrt2LambdaTau * std::sqrt(f1 * f2);
        dVec np = P(nb), e = P(eb), r;
        for (int i = 0; i < 3; ++i) r[i] = (e[i] + c.p.side[i] * wind[i]) - np[i];
        for (int i = 0; i < 3; ++i) r[i] *= f2;
        for (int i = 0; i < 3; ++i) r[i] += np[i];
        for (int i = 0; i < 3; ++i) r[i] = R.randNorm(r[i], sg);
        for (int i = 0; i < 3; ++i) {
            while (r[i] < -0.5 * c.p.side[i]) { wind[i]++; r[i] += c.p.side[i]; }
            while (r[i] >= 0.5 * c.p.side[i]) { wind[i]--; r[i] -= c.p.side[i]; }
        }
        putInBC(r);
        return r;
    }
    dVec bisectionPos(Bead bd, int ls) {
        double delta = sqrtLambdaTau * std::sqrt(1.0 * ls);
        Bead nB = prevN(bd, ls), nx = nextN(bd, ls);
        dVec r = sep(nx, nB), pn = P(nB);
        for (int i = 0; i < 3; ++i) r[i] *= 0.5;
        for (int i = 0; i < 3; ++i) r[i] += pn[i];
        for (int i = 0; i < 3; ++i) r[i] = R.randNorm(r[i], delta);
        putInBC(r);
        return r;
    }
    int com(bool& acc) {
        acc = false;
        if (c.numBeadsOn == 0 || c.h_nbs[0] == 0) return 0;
        Bead first{0, (int)R.randInt((uint32_t)(c.h_nbs[0] - 1))};
        Bead sb = first, eb;
        if (!isX(prev(sb))) { do { sb = prev(sb); } while (!(prev(sb) == first) && !isX(prev(sb))); }
        if (prev(sb) == first) { sb = first; eb = prev(sb); }
        else { eb = first; if (!isX(next(eb))) { do { eb = next(eb); } while (!isX(next(eb))); } }
        std::vector<Bead> wl;
        Bead bd = sb, stop = next(eb);
        do { wl.push_back(bd); bd = next(bd); } while (!(bd == stop));
        if ((int)wl.size() > c.M) return 0;
        st.attempted[0]++;
        dVec sh;
        for (int i = 0; i < 3; ++i) sh[i] = comDelta * (-0.5 + R.rand());
        double oldA = action_list(wl);
        std::vector<dVec> np;
        for (auto& w : wl) { dVec p = P(w); for (int i = 0; i < 3; ++i) p[i] = p[i] + sh[i]; putInBC(p); np.push_back(p); }
        set(wl, np);
        double newA = action_list(wl);
        if (R.rand() < std::exp(-(newA - oldA))) { acc = true; st.accepted[0]++; }
        else {
            std::vector<dVec> rp;
            for (auto& w : wl) { dVec p = P(w); for (int i = 0; i < 3; ++i) p[i] = p[i] - sh[i]; putInBC(p); rp.push_back(p); }
            set(wl, rp);
        }
        return (int)wl.size();
    }
    int staging(bool& acc) {
        acc = false;
        if (c.numBeadsOn == 0 || c.numBeadsOn / c.M == 0) return 0;
        Bead sb;
        sb[0] = (int)R.randInt((uint32_t)(c.M - 1));
        if (c.h_nbs[sb[0]] == 0) return 0;
        sb[1] = (int)R.randInt((uint32_t)(c.h_nbs[sb[0]] - 1));
        int L = mp.mbar;
        if (mp.var_updates) L = 2 + (int)R.randInt((uint32_t)(mp.mbar - 2));
        Bead bd = sb;
        for (int k = 0; k < L; ++k) { if (!on(bd) || isX(next(bd))) return 0; bd = next(bd); }
        Bead eb = bd;
        st.attempted[1]++;
        auto wind = sampleWinding(sb, eb, L);
        Bead pe = prev(eb);
        double oldA = action_range(sb, pe);
        std::vector<Bead> moved; std::vector<dVec> orig, np;
        bd = sb;
        int k = 0;
        do {
            bd = next(bd);
            orig.push_back(P(bd));
            dVec p = stagingPos(prev(bd), eb, L, k, wind);
            // the next proposal uses this bead's new position (path.updateBead)
            for (int d = 0; d < 3; ++d) pos[((size_t)bd[0] * c.Ne + bd[1]) * 3 + d] = p[d];
            moved.push_back(bd); np.push_back(p);
            ++k;
        } while (!(bd == pe));
        set(moved, np);
        double newA = action_range(sb, pe);
        if (R.rand() < std::exp(-(newA - oldA))) { acc = true; st.accepted[1]++; }
        else set(moved, orig);
        return L - 1;
    }
    int bisection(bool& acc) {
        acc = false;
        if (c.numBeadsOn == 0) return 0;
        int nl = b;
        if (mp.var_updates) nl = 1 + (int)R.randInt((uint32_t)(b - 1));
        int nact = (int)std::floor(std::pow(2.0, 1.0 * nl) + EPS) - 1;
        if (c.numBeadsOn / c.M == 0) return 0;
        Bead sb;
        sb[0] = (int)R.randInt((uint32_t)(c.M - 1));
        if (c.h_nbs[sb[0]] == 0) return 0;
        sb[1] = (int)R.randInt((uint32_t)(c.h_nbs[sb[0]] - 1));
        Bead bb = sb;
        for (int k = 0; k < nact + 1; ++k) { if (!on(bb) || isX(next(bb))) return 0; bb = next(bb); }
        Bead eb = bb;
        st.attempted[2]++;
        int nmax = (int)std::floor(std::pow(2.0, 1.0 * b) + EPS) - 1;
        std::vector<char> inc(nmax, 1);
        std::vector<dVec> origPos(nmax), newPos(nmax);
        double oldDelta = 0.0;
        int moved = 0;
        for (int level = nl; level > 0; level--) {
            int sh = (int)std::floor(std::pow(2.0, 1.0 * (level - 1)) + EPS);
            shift = sh;
            double oldA = 0.0, newA = 0.0;
            std::vector<Bead> incl, prevLev; std::vector<int> incIdx, prevIdx;
            Bead bi = nextN(sb, sh);
            int k = 1;
            do {
                int n = k * sh - 1;
                if (inc[n]) { origPos[n] = P(bi); incl.push_back(bi); incIdx.push_back(n); }
                else if (level == 1) { prevLev.push_back(bi); prevIdx.push_back(n); }
                ++k; bi = nextN(bi, sh);
            } while (!(bi == eb));
            oldA += action_list(incl);
            std::vector<dVec> np;
            for (size_t i = 0; i < incl.size(); ++i) {
                int n = incIdx[i];
                newPos[n] = bisectionPos(incl[i], sh);
                for (int d = 0; d < 3; ++d) pos[((size_t)incl[i][0] * c.Ne + incl[i][1]) * 3 + d] = newPos[n][d];
                inc[n] = 0;
                np.push_back(newPos[n]);
            }
            set(incl, np);
            moved += (int)incl.size();
            newA += action_list(incl);
            if (level == 1 && !prevLev.empty()) {
                newA += action_list(prevLev);
                std::vector<dVec> op, nq;
                for (size_t i = 0; i < prevLev.size(); ++i) { op.push_back(origPos[prevIdx[i]]); nq.push_back(newPos[prevIdx[i]]); }
                set(prevLev, op);
                oldA += action_list(prevLev);
                set(prevLev, nq);
            }
            double dA = newA - oldA;
            if (R.rand() < std::exp(-dA + oldDelta)) {
                if (level == 1) { acc = true; st.accepted[2]++; shift = 1; }
            } else {
                std::vector<Bead> rb; std::vector<dVec> rp;
                Bead bk = sb; int kk = 0;
                do { bk = next(bk); if (!inc[kk]) { rb.push_back(bk); rp.push_back(origPos[kk]); } ++kk; }
                while (!(bk == prev(eb)));
                set(rb, rp);
                shift = 1;
                break;
            }
            oldDelta = dA;
        }
        shift = 1;
        return moved;
    }
};

}  // namespace

extern "C" {

int pgb_plain_seed(pgb_ctx* h, uint32_t seed) {
    if (!h) return PGB_EINVAL;
    Ctx& c = h->c;
    c.mt_state.assign(624, 0);
    c.mt_state[0] = seed;
    for (int i = 1; i < 624; ++i)
        c.mt_state[i] = 1812433253u * (c.mt_state[i - 1] ^ (c.mt_state[i - 1] >> 30)) + (uint32_t)i;
    MT m; m.st = c.mt_state.data(); m.left = &c.mt_left; m.pos = &c.mt_pos;
    m.reload();
    c.mt_seeded = true;
    return PGB_OK;
}

int pgb_plain_get_rng(pgb_ctx* h, uint32_t* out625) {
    if (!h || !out625) return PGB_EINVAL;
    Ctx& c = h->c;
    if (!c.mt_seeded) return c.fail(PGB_ESTATE, "plain_get_rng: the generator was never seeded");
    // MTRand::save (MersenneTwister.h): the 624 state words, then `left`
    for (int i = 0; i < 624; ++i) out625[i] = c.mt_state[i];
    out625[624] = (uint32_t)c.mt_left;
    return PGB_OK;
}

int pgb_plain_set_rng(pgb_ctx* h, const uint32_t* in625) {
    if (!h || !in625) return PGB_EINVAL;
    Ctx& c = h->c;
    if (in625[624] > 624u) return c.fail(PGB_EINVAL, "plain_set_rng: `left` must be 0..624");
    // MTRand::load: pNext = &state[N - left]
    c.mt_state.assign(in625, in625 + 624);
    c.mt_left = (int)in625[624];
    c.mt_pos = 624 - c.mt_left;
    c.mt_seeded = true;
    return PGB_OK;
}

int pgb_plain_run(pgb_ctx* h, const pgb_move_params* mp, int nsteps, int32_t* trace, int trace_cap,
                  int* trace_len, double* energies, pgb_move_stats* stats) {
    if (!h || !mp || nsteps < 0) return PGB_EINVAL;
    Ctx& c = h->c;
    if (!c.loaded) return c.fail(PGB_ESTATE, "plain_run: no path loaded");
    if (!c.mt_seeded) return c.fail(PGB_ESTATE, "plain_run: call pgb_plain_seed first");
    if (mp->mbar < 2 || mp->mbar >= c.M || mp->temperature <= 0)
        return c.fail(PGB_EINVAL, "plain_run: need 2 <= mbar < M and temperature > 0");
    Plain pl(c, *mp);
    pl.pos.assign((size_t)c.M * c.Ne * 3, 0.0);
    int rc = pgb_get_positions(h, pl.pos.data());
    if (rc) return rc;
    int N0 = c.numBeadsOn / c.M;
    int nu = mp->num_updates;
    if (nu <= 0) { nu = int(std::ceil(std::max(N0, 1) * c.M / (1.0 * mp->mbar))); if (nu < 100) nu = 100; }
    double cum[2] = {mp->p_com, 1.0 + EPS};
    int ntr = 0;
    for (int step = 0; step < nsteps; ++step) {
        for (int n = 0; n < nu; ++n) {
            double x = pl.R.rand();
            int index = int(std::lower_bound(cum, cum + 2, x) - cum);
            bool acc = false;
            int moved, code;
            if (index == 0) { moved = pl.com(acc); code = 0; }
            else if (mp->diagonal_move == 1) { moved = pl.staging(acc); code = 1; }
            else { moved = pl.bisection(acc); code = 2; }
            if (pl.err) return pl.err;
            pl.st.bead_updates += moved;
            if (trace && ntr < trace_cap && moved > 0) { trace[2 * ntr] = code; trace[2 * ntr + 1] = acc ? 1 : 0; ++ntr; }
        }
        if (energies) {
            double e[9];
            rc = pgb_energy(h, e);
            if (rc) return rc;
            energies[step] = e[8];
        }
    }
    if (trace_len) *trace_len = ntr;
    if (stats) *stats = pl.st;
    return PGB_OK;
}

}  // extern "C"
