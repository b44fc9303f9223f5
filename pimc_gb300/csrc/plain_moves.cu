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
#include <limits>
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
    double randExc() { return double(randInt()) * (1.0 / 4294967296.0); }
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
        flush();
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

    // ---------------------------------------------------------------------
    // Worm-algorithm moves (src/move.cpp:1710-3826) on the host mirrors with
    // FP64 device actions.  Path/LookupTable/Worm bookkeeping as in
    // src/path.cpp:205-420, src/lookuptable.cpp:314-458, src/worm.cpp:52-118;
    // every changed bead is written to the device before the next action.
    // ---------------------------------------------------------------------
    std::vector<int> dirty;
    std::vector<char> isDirty;
    bool full = false, broken = false;
    pgb_worm_params wp{};
    double Cw = 0.0;
    int numBeads0 = 0;
    double prob[12] = {0.01, 0.19, 0.4, 0.15, 0.4, 0.15, 0.075, 0.075, 0.075, 0.075, 0.1, 0.1};
    pgb_worm_stats wst{};
    std::vector<double> cumulant;
    int sizeCDF = 0;
    std::vector<Bead> fullList;
    std::vector<dVec> originalPos;

    size_t lin(Bead b) const { return (size_t)b[0] * c.Ne + b[1]; }
    void touch(Bead b) {
        if (isDirty.empty()) isDirty.assign((size_t)c.M * c.Ne, 0);
        size_t j = lin(b);
        if (!isDirty[j]) { isDirty[j] = 1; dirty.push_back((int)j); }
    }
    void flush() {
        if (err) return;
        if (dirty.empty()) return;
        err = pgb::upload_beads(c, dirty.data(), (int)dirty.size(), pos.data());
        for (int j : dirty) isDirty[j] = 0;
        dirty.clear();
    }
    void setNextB(Bead b, Bead v) { size_t i = lin(b) * 2; c.h_next[i] = v[0]; c.h_next[i + 1] = v[1]; touch(b); }
    void setPrevB(Bead b, Bead v) { size_t i = lin(b) * 2; c.h_prev[i] = v[0]; c.h_prev[i + 1] = v[1]; touch(b); }
    void setPos(Bead b, const dVec& p) { for (int d = 0; d < 3; ++d) pos[lin(b) * 3 + d] = p[d]; touch(b); }
    Bead W(int k) const { return {c.worm[2 * k], c.worm[2 * k + 1]}; }
    void setW(int k, Bead b) { c.worm[2 * k] = b[0]; c.worm[2 * k + 1] = b[1]; }
    Bead head() const { return W(0); }
    Bead tail() const { return W(1); }
    Bead sp1() const { return W(2); }

    // LookupTable with one grid box: per-slice lists in the reference's order
    void lookupInit() {
        c.lk_hash.assign(c.M, std::vector<int>());
        c.lk_label.assign((size_t)c.M * c.Ne, XXX);
        for (int t = 0; t < c.M; ++t)
            for (int p = 0; p < c.Ne; ++p)
                if (c.h_on[(size_t)t * c.Ne + p]) {
                    c.lk_label[(size_t)t * c.Ne + p] = (int)c.lk_hash[t].size();
                    c.lk_hash[t].push_back(p);
                }
        // Worm scalars of the loaded path (Worm::update without unlinking)
        if (c.worm[0] == XXX) { c.w_diag = true; c.w_gap = XXX; c.w_length = 0; c.w_sep[0] = c.w_sep[1] = c.w_sep[2] = 0.0; }
        else {
            c.w_diag = false;
            c.w_gap = c.worm[2] - c.worm[0];
            if (c.w_gap < 0) c.w_gap += c.M;
            Bead b = tail();
            int len = 0;
            const long long limit = (long long)c.M * c.Ne + 1;
            while (true) {
                ++len;
                if (b == head()) break;
                b = next(b);
                if (isX(b) || len > limit) { broken = true; break; }
            }
            c.w_length = len - 1;
            dVec d = sep(tail(), head());
            for (int i = 0; i < 3; ++i) c.w_sep[i] = d[i];
        }
        c.lk_valid = true;
    }
    void lookupAdd(Bead b) { c.lk_label[lin(b)] = (int)c.lk_hash[b[0]].size(); c.lk_hash[b[0]].push_back(b[1]); }
    void lookupDel(Bead b) {
        auto& h = c.lk_hash[b[0]];
        const int l = c.lk_label[lin(b)], last = (int)h.size() - 1;
        if (l < last) { const int moved = h[last]; h[l] = moved; c.lk_label[(size_t)b[0] * c.Ne + moved] = l; }
        h.pop_back();
        c.lk_label[lin(b)] = XXX;
    }
    // Path::addBead: a full slice is an error here (the reference grows Ne)
    Bead addBead(int slice, const dVec& p) {
        Bead last{slice, c.h_nbs[slice]};
        if (last[1] >= c.Ne) { full = true; return {XXX, XXX}; }
        c.h_on[lin(last)] = 1;
        ++c.numBeadsOn;
        ++c.h_nbs[slice];
        setNextB(last, {XXX, XXX}); setPrevB(last, {XXX, XXX});
        setPos(last, p);
        lookupAdd(last);
        return last;
    }
    Bead addNextBead(Bead pb, const dVec& p) {
        int slice = pb[0] + 1;
        if (slice >= c.M) slice -= c.M;
        Bead b = addBead(slice, p);
        if (full) return b;
        setNextB(pb, b); setPrevB(b, pb);
        return b;
    }
    Bead addPrevBead(Bead nb, const dVec& p) {
        int slice = nb[0] - 1;
        if (slice < 0) slice += c.M;
        Bead b = addBead(slice, p);
        if (full) return b;
        setPrevB(nb, b); setNextB(b, nb);
        return b;
    }
    void delBead(Bead b) {
        lookupDel(b);
        --c.h_nbs[b[0]];
        Bead last{b[0], c.h_nbs[b[0]]};
        if (!isX(next(b))) setPrevB(next(b), {XXX, XXX});
        if (!isX(prev(b))) setNextB(prev(b), {XXX, XXX});
        if (b[1] < c.h_nbs[b[0]]) {
            lookupDel(last);
            lookupAdd(b);
            setPos(b, P(last));
            setPrevB(b, prev(last));
            setNextB(b, next(last));
            if (!isX(next(last))) setPrevB(next(last), b);
            if (!isX(prev(last))) setNextB(prev(last), b);
            for (int k = 0; k < 4; ++k) if (W(k) == last) setW(k, b);
        }
        setNextB(last, {XXX, XXX}); setPrevB(last, {XXX, XXX});
        c.h_on[lin(last)] = 0;
        touch(last);
        --c.numBeadsOn;
    }
    Bead delBeadGetNext(Bead b) { Bead n = next(b); delBead(b); return n; }
    Bead delBeadGetPrev(Bead b) { Bead p = prev(b); delBead(b); return p; }
    void wormReset() {
        c.w_gap = XXX; c.w_length = 0; c.w_sep[0] = c.w_sep[1] = c.w_sep[2] = 0.0;
        for (int k = 0; k < 4; ++k) setW(k, {XXX, XXX});
    }
    void wormUpdate(Bead nh, Bead nt) {
        setW(0, nh); setW(1, nt);
        c.w_gap = nt[0] - nh[0];
        if (c.w_gap < 0) c.w_gap += c.M;
        Bead b = nt;
        c.w_length = 0;
        const long long limit = (long long)c.M * c.Ne + 1;
        do {
            ++c.w_length;
            b = next(b);
            if (isX(b) || c.w_length > limit) { broken = true; break; }
        } while (!(b == nh));
        dVec d = sep(nt, nh);
        for (int i = 0; i < 3; ++i) c.w_sep[i] = d[i];
        setNextB(nh, {XXX, XXX}); setPrevB(nt, {XXX, XXX});
        setW(2, {XXX, XXX}); setW(3, {XXX, XXX});
    }
    bool tooCostly(const dVec& s, int g) const {
        if (g == 0) return true;
        double d = 0.0; for (int i = 0; i < 3; ++i) d += s[i] * s[i];
        return (d * (0.25 / (c.p.lambda * c.p.tau)) / (1.0 * g)) > 4.0;
    }
    double ensembleWeight(int dn) {
        const bool window = wp.window >= 0, gauss = wp.gaussian_sd > 0.0;
        if (window || gauss) {
            int nb = c.numBeadsOn, nbp = nb + dn;
            if (window) {
                int w = c.M * wp.window;
                if (nbp > numBeads0 + w || nbp < numBeads0 - w) return 0.0;
            }
            if (gauss) {
                double sb = c.M * wp.gaussian_sd;
                double xp = 1.0 * (nbp - numBeads0) * (nbp - numBeads0) / (2.0 * sb * sb);
                double x = 1.0 * (nb - numBeads0) * (nb - numBeads0) / (2.0 * sb * sb);
                return std::exp(-xp + x);
            }
            return 1.0;
        }
        return 1.0;
    }
    // one bead's action on the device (after the pending writes)
    double beadAction(Bead b, int mode) {
        flush();
        if (err) return 0.0;
        int32_t bl[2] = {b[0], b[1]};
        double per = 0.0, tot = 0.0;
        err = pgb_bead_actions(reinterpret_cast<pgb_ctx*>(&c), bl, 1, 1, mode, &per, &tot);
        return per;
    }
    double bare(Bead b) { return beadAction(b, PGB_ACTION_BARE); }
    double fullBead(Bead b) { return beadAction(b, PGB_ACTION_FULL); }
    // potentialActionCorrection(start, end): per bead along next links, in order
    double corrRange(Bead s, Bead e) {
        flush();
        if (err) return 0.0;
        std::vector<int32_t> bl;
        Bead b = s, stop = next(e);
        do { if (on(b)) { bl.push_back(b[0]); bl.push_back(b[1]); } b = next(b); } while (!(b == stop));
        std::vector<double> per(bl.size() / 2 + 1, 0.0);
        double tot = 0.0;
        err = pgb_bead_actions(reinterpret_cast<pgb_ctx*>(&c), bl.data(), (int)bl.size() / 2, 1,
                               PGB_ACTION_CORR, per.data(), &tot);
        double cr = 0.0;
        for (size_t i = 0; i < bl.size() / 2; ++i) cr += per[i];
        return cr;
    }
    double fullRange(Bead s, Bead e) {
        flush();
        if (err) return 0.0;
        std::vector<int32_t> bl;
        Bead b = s, stop = next(e);
        do { if (on(b)) { bl.push_back(b[0]); bl.push_back(b[1]); } b = next(b); } while (!(b == stop));
        std::vector<double> per(bl.size() / 2 + 1, 0.0);
        double tot = 0.0;
        err = pgb_bead_actions(reinterpret_cast<pgb_ctx*>(&c), bl.data(), (int)bl.size() / 2, 1,
                               PGB_ACTION_FULL, per.data(), &tot);
        double u = 0.0;
        for (size_t i = 0; i < bl.size() / 2; ++i) u += per[i];
        return u;
    }
    dVec freePos(Bead n) {
        dVec r, p = P(n);
        for (int i = 0; i < 3; ++i) r[i] = R.randNorm(p[i], sqrt2LambdaTau);
        putInBC(r);
        return r;
    }
    dVec randPosition() {
        dVec r;
        for (int i = 0; i < 3; ++i) r[i] = c.p.side[i] * (-0.5 + R.randExc());
        return r;
    }
    std::array<int,3> sampleWindingT(Bead sb, Bead eb, int L, double& total) {
        dVec pe = P(eb), ps = P(sb), vel;
        for (int i = 0; i < 3; ++i) vel[i] = pe[i] - ps[i];
        cumrho0[0] = rho0(vel, L);
        total = cumrho0[0];
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
    int Mbar() const { return wp.mbar; }
    int randLen() { return 2 * (1 + (int)R.randInt((uint32_t)(Mbar() / 2 - 1))); }
    bool metro(double dA) { return R.rand() < std::exp(-dA); }
    int trueN() const { return c.numBeadsOn / c.M; }

    int wOpen() {
        if (c.numBeadsOn == 0 || trueN() == 0) return -1;
        const int gapLength = randLen();
        Bead hb, tb;
        hb[0] = 2 * (int)R.randInt((uint32_t)(c.M / 2 - 1));
        hb[1] = (int)R.randInt((uint32_t)(c.h_nbs[hb[0]] - 1));
        tb = nextN(hb, gapLength);
        double totalrho0;
        auto wind = sampleWindingT(hb, tb, gapLength, totalrho0);
        dVec pt = P(tb), ph = P(hb), sp;
        for (int i = 0; i < 3; ++i) sp[i] = (pt[i] - ph[i]) + wind[i] * c.p.side[i];
        if (tooCostly(sp, gapLength)) return -1;
        double norm = (Cw * Mbar() * c.numBeadsOn) / totalrho0;
        norm *= prob[3] / prob[2];
        norm *= ensembleWeight(-gapLength + 1);
        const double muShift = gapLength * wp.mu * c.p.tau;
        wst.attempted[2]++;
        setW(2, hb); setW(3, tb);
        const double actionShift = (-std::log(norm) + muShift) / gapLength;
        double factor = 0.5;
        Bead b = hb;
        do {
            wst.bead_updates++;
            double dA = -(bare(b) - factor * actionShift);
            if (!metro(dA)) { wormReset(); c.w_diag = true; return 0; }
            factor = 1.0;
            b = next(b);
        } while (!(b == tb));
        wst.bead_updates++;
        double dA = -(bare(tb) - 0.5 * actionShift);
        dA -= corrRange(hb, tb);
        if (metro(dA)) {
            wst.accepted[2]++;
            b = next(hb);
            while (!(b == tb)) b = delBeadGetNext(b);
            wormUpdate(hb, tb);
            c.w_diag = false;
            return 1;
        }
        wormReset(); c.w_diag = true;
        return 0;
    }
    void closeUndo() {
        Bead b = next(head());
        while (!(b == tail()) && !isX(b)) b = delBeadGetNext(b);
        setNextB(head(), {XXX, XXX}); setPrevB(tail(), {XXX, XXX});
        c.w_diag = false;
    }
    int wClose() {
        if (c.numBeadsOn == 0) return -1;
        dVec ws{c.w_sep[0], c.w_sep[1], c.w_sep[2]};
        if (c.w_gap > Mbar() || c.w_gap == 0 || tooCostly(ws, c.w_gap)) return -1;
        wst.attempted[3]++;
        const int gap = c.w_gap;
        double totalrho0;
        auto wind = sampleWindingT(head(), tail(), gap, totalrho0);
        double norm = totalrho0 / (Cw * Mbar() * (c.numBeadsOn + gap - 1));
        norm *= prob[2] / prob[3];
        norm *= ensembleWeight(gap - 1);
        const double muShift = gap * wp.mu * c.p.tau;
        const double actionShift = (std::log(norm) + muShift) / gap;
        Bead b = head();
        wst.bead_updates++;
        double dA = bare(b) - 0.5 * actionShift;
        if (!metro(dA)) { closeUndo(); return 0; }
        for (int k = 0; k < gap - 1; k++) {
            dVec p = stagingPos(b, tail(), gap, k, wind);
            b = addNextBead(b, p);
            if (full) return -2;
            wst.bead_updates++;
            dA = bare(b) - actionShift;
            if (!metro(dA)) { closeUndo(); return 0; }
        }
        setNextB(b, tail()); setPrevB(tail(), b);
        wst.bead_updates++;
        dA = bare(tail()) - 0.5 * actionShift;
        dA += corrRange(head(), tail());
        if (metro(dA)) { wst.accepted[3]++; wormReset(); c.w_diag = true; return 1; }
        closeUndo();
        return 0;
    }
    void insertUndo(Bead tb) {
        Bead b = tb;
        do { b = delBeadGetNext(b); } while (!isX(b));
        wormReset(); c.w_diag = true;
    }
    int wInsert() {
        const int wormLength = randLen();
        wst.attempted[4]++;
        double norm = Cw * Mbar() * c.M * (c.p.side[0] * c.p.side[1] * c.p.side[2]);
        const double muShift = wormLength * c.p.tau * wp.mu;
        norm *= prob[5] / prob[4];
        norm *= ensembleWeight(wormLength);
        if (norm < std::numeric_limits<double>::epsilon()) return 0;
        const int slice = 2 * (int)R.randInt((uint32_t)(c.M / 2 - 1));
        dVec rp = randPosition();
        Bead tb = addBead(slice, rp);
        if (full) return -2;
        setW(3, tb);
        const double actionShift = (std::log(norm) + muShift) / wormLength;
        Bead b = tb;
        wst.bead_updates++;
        double dA = bare(b) - 0.5 * actionShift;
        if (!metro(dA)) { insertUndo(tb); return 0; }
        for (int k = 1; k < wormLength; k++) {
            dVec p = freePos(b);
            b = addNextBead(b, p);
            if (full) return -2;
            wst.bead_updates++;
            dA = bare(b) - actionShift;
            if (!metro(dA)) { insertUndo(tb); return 0; }
        }
        dVec p = freePos(b);
        Bead hb = addNextBead(b, p);
        if (full) return -2;
        setW(2, hb);
        wst.bead_updates++;
        dA = bare(hb) - 0.5 * actionShift;
        dA += corrRange(tb, hb);
        if (metro(dA)) { wst.accepted[4]++; wormUpdate(hb, tb); c.w_diag = false; return 1; }
        insertUndo(tb);
        return 0;
    }
    int wRemove() {
        if (c.w_length > Mbar() || c.w_length < 1) return -1;
        wst.attempted[5]++;
        double norm = 1.0 / (Cw * Mbar() * c.M * (c.p.side[0] * c.p.side[1] * c.p.side[2]));
        const double muShift = c.w_length * wp.mu * c.p.tau;
        norm *= prob[4] / prob[5];
        norm *= ensembleWeight(-c.w_length);
        if (norm < std::numeric_limits<double>::epsilon()) return 0;
        const double actionShift = (-std::log(norm) + muShift) / c.w_length;
        Bead b = head();
        double factor = 0.5;
        do {
            wst.bead_updates++;
            double dA = -(bare(b) - factor * actionShift);
            if (!metro(dA)) { c.w_diag = false; return 0; }
            factor = 1.0;
            b = prev(b);
        } while (!(b == tail()));
        wst.bead_updates++;
        double dA = -(bare(tail()) - 0.5 * actionShift);
        dA -= corrRange(tail(), head());
        if (metro(dA)) {
            wst.accepted[5]++;
            b = head();
            do { b = delBeadGetPrev(b); } while (!isX(b));
            wormReset(); c.w_diag = true;
            return 1;
        }
        c.w_diag = false;
        return 0;
    }
    void ahUndo() {
        setW(0, sp1());
        Bead b = next(head());
        while (!isX(b)) b = delBeadGetNext(b);
        setNextB(head(), {XXX, XXX});
        c.w_diag = false;
        setW(2, {XXX, XXX});
    }
    int wAdvanceHead() {
        if (c.numBeadsOn == 0) return -1;
        const int al = randLen();
        wst.attempted[6]++;
        const double muShift = al * c.p.tau * wp.mu;
        double norm = prob[7] / prob[6];
        norm *= ensembleWeight(al);
        setW(2, head()); setW(0, {XXX, XXX});
        const double actionShift = (std::log(norm) + muShift) / al;
        Bead b = sp1();
        wst.bead_updates++;
        double dA = bare(b) - 0.5 * actionShift;
        if (!metro(dA)) { ahUndo(); return 0; }
        for (int k = 0; k < al - 1; k++) {
            dVec p = freePos(b);
            b = addNextBead(b, p);
            if (full) return -2;
            wst.bead_updates++;
            dA = bare(b) - actionShift;
            if (!metro(dA)) { ahUndo(); return 0; }
        }
        dVec p = freePos(b);
        Bead hb = addNextBead(b, p);
        if (full) return -2;
        setW(0, hb);
        wst.bead_updates++;
        dA = fullBead(hb) - 0.5 * actionShift;
        dA += corrRange(sp1(), head());
        if (metro(dA)) { wst.accepted[6]++; wormUpdate(hb, tail()); c.w_diag = false; return 1; }
        ahUndo();
        return 0;
    }
    int wAdvanceTail() {
        if (c.numBeadsOn == 0) return -1;
        const int al = randLen();
        if (!(al < c.w_length)) return -1;
        Bead tb = nextN(tail(), al);
        const double muShift = al * c.p.tau * wp.mu;
        double norm = prob[9] / prob[8];
        norm *= ensembleWeight(-al);
        wst.attempted[8]++;
        setW(2, tb);
        const double actionShift = (-std::log(norm) + muShift) / al;
        double factor = 0.5;
        Bead b = tail();
        do {
            wst.bead_updates++;
            double dA = -(bare(b) - factor * actionShift);
            if (!metro(dA)) { c.w_diag = false; setW(2, {XXX, XXX}); return 0; }
            factor = 1.0;
            b = next(b);
        } while (!(b == tb));
        wst.bead_updates++;
        double dA = -(bare(b) - 0.5 * actionShift);
        dA -= corrRange(tail(), tb);
        if (metro(dA)) {
            wst.accepted[8]++;
            b = prev(tb);
            do { b = delBeadGetPrev(b); } while (!isX(b));
            wormUpdate(head(), tb);
            c.w_diag = false;
            return 1;
        }
        c.w_diag = false; setW(2, {XXX, XXX});
        return 0;
    }
    int wRecedeHead() {
        if (c.numBeadsOn == 0) return -1;
        const int rl = randLen();
        if (!(rl < c.w_length)) return -1;
        Bead hb = prevN(head(), rl);
        const double muShift = rl * c.p.tau * wp.mu;
        double norm = prob[6] / prob[7];
        norm *= ensembleWeight(-rl);
        wst.attempted[7]++;
        setW(2, hb);
        const double actionShift = (-std::log(norm) + muShift) / rl;
        double factor = 0.5;
        Bead b = head();
        do {
            wst.bead_updates++;
            double dA = -(bare(b) - factor * actionShift);
            if (!metro(dA)) { c.w_diag = false; setW(2, {XXX, XXX}); return 0; }
            factor = 1.0;
            b = prev(b);
        } while (!(b == hb));
        wst.bead_updates++;
        double dA = -(bare(hb) - 0.5 * actionShift);
        dA -= corrRange(sp1(), head());
        if (metro(dA)) {
            wst.accepted[7]++;
            b = next(hb);
            do { b = delBeadGetNext(b); } while (!isX(b));
            wormUpdate(hb, tail());
            c.w_diag = false;
            return 1;
        }
        c.w_diag = false; setW(2, {XXX, XXX});
        return 0;
    }
    void rtUndo() {
        setW(1, sp1());
        Bead b = prev(tail());
        while (!isX(b)) b = delBeadGetPrev(b);
        setPrevB(tail(), {XXX, XXX});
        c.w_diag = false;
        setW(2, {XXX, XXX});
    }
    int wRecedeTail() {
        if (c.numBeadsOn == 0) return -1;
        const int rl = randLen();
        wst.attempted[9]++;
        const double muShift = rl * c.p.tau * wp.mu;
        double norm = prob[8] / prob[9];
        norm *= ensembleWeight(rl);
        setW(2, tail()); setW(1, {XXX, XXX});
        const double actionShift = (std::log(norm) + muShift) / rl;
        Bead b = sp1();
        wst.bead_updates++;
        double dA = bare(b) - 0.5 * actionShift;
        if (!metro(dA)) { rtUndo(); return 0; }
        for (int k = 0; k < rl - 1; k++) {
            dVec p = freePos(b);
            b = addPrevBead(b, p);
            if (full) return -2;
            wst.bead_updates++;
            dA = bare(b) - actionShift;
            if (!metro(dA)) { rtUndo(); return 0; }
        }
        dVec p = freePos(b);
        Bead tb = addPrevBead(b, p);
        if (full) return -2;
        setW(1, tb);
        wst.bead_updates++;
        dA = bare(tb) - 0.5 * actionShift;
        dA += corrRange(tb, sp1());
        if (metro(dA)) { wst.accepted[9]++; wormUpdate(head(), tb); c.w_diag = false; return 1; }
        rtUndo();
        return 0;
    }
    // SwapMoveBase::getNorm / selectPivotBead (move.cpp:3223-3330)
    double getNorm(Bead b, int sign) {
        const int nL = (int)fullList.size();
        sizeCDF = nL * numWind;
        if ((int)cumulant.size() < sizeCDF) cumulant.assign(sizeCDF, 0.0);
        const int L = Mbar();
        int index = 0;
        dVec pb = P(b);
        auto sepTo = [&](Bead f) { dVec pf = P(f), d; for (int i = 0; i < 3; ++i) d[i] = pf[i] - pb[i]; return d; };
        dVec sp = sepTo(fullList[0]);
        double Sigma = rho0(sp, L);
        cumulant[index++] = Sigma;
        for (int n = 1; n < nL; n++) {
            sp = sepTo(fullList[n]);
            double cr = rho0(sp, L);
            Sigma += cr;
            cumulant[index] = cumulant[index - 1] + cr;
            ++index;
        }
        for (int w = 1; w < numWind; w++) {
            for (int n = 0; n < nL; n++) {
                sp = sepTo(fullList[n]);
                for (int i = 0; i < 3; ++i) sp[i] = sp[i] + (sign * winding[w][i]) * c.p.side[i];
                double cr = rho0(sp, L);
                Sigma += cr;
                cumulant[index] = cumulant[index - 1] + cr;
                ++index;
            }
        }
        for (int n = 0; n < sizeCDF; n++) cumulant[n] /= Sigma;
        return Sigma;
    }
    Bead selectPivot(std::array<int,3>& wind) {
        const double x = R.rand();
        const int index = int(std::lower_bound(cumulant.begin(), cumulant.begin() + sizeCDF, x) - cumulant.begin());
        const int nL = (int)fullList.size();
        const int w = (index / nL) % numWind;
        const int p = index % nL;
        wind = winding[w];
        return fullList[p];
    }
    void fillList(int slice) {
        fullList.clear();
        for (int p : c.lk_hash[slice]) fullList.push_back({slice, p});
    }
    int wSwapHead() {
        if (c.numBeadsOn == 0) return -1;
        if (c.w_diag) return -1;
        const int swapLength = Mbar();
        int pivotSlice = c.worm[0] + swapLength;
        if (pivotSlice >= c.M) pivotSlice -= c.M;
        fillList(pivotSlice);
        if (fullList.empty()) return -1;
        const double SigmaHead = getNorm(head(), 1);
        std::array<int,3> wind{0, 0, 0};
        Bead pivot = selectPivot(wind);
        Bead b = pivot;
        for (int k = 0; k < swapLength; k++) {
            if (b == tail()) return -1;
            b = prev(b);
        }
        Bead swp = b;
        if (tail() == swp) return -1;
        wst.attempted[10]++;
        const double SigmaSwap = getNorm(swp, 1);
        const double PNorm = std::min(SigmaHead / SigmaSwap, 1.0);
        if (R.rand() < PNorm) {
            setW(2, swp); setW(3, pivot);
            originalPos.clear();
            b = swp;
            do {
                if (!(b == swp) && !(b == pivot)) originalPos.push_back(P(b));
                b = next(b);
            } while (!(b == next(pivot)));
            const double oldAction = fullRange(swp, pivot);
            Bead nextSwap = next(swp);
            setNextB(head(), nextSwap);
            setNextB(swp, {XXX, XXX});
            setPrevB(nextSwap, head());
            setW(2, head());
            setW(0, swp);
            const Bead s1 = sp1();
            b = s1;
            int k = 0;
            do {
                if (!(b == s1) && !(b == pivot)) {
                    dVec p = stagingPos(prev(b), pivot, swapLength, k, wind);
                    setPos(b, p);
                    ++k;
                    wst.bead_updates++;
                }
                b = next(b);
            } while (!(b == next(pivot)));
            const double newAction = fullRange(s1, pivot);
            if (metro(newAction - oldAction)) { wst.accepted[10]++; wormUpdate(swp, tail()); return 1; }
            setW(0, s1);
            setNextB(head(), {XXX, XXX});
            setNextB(swp, nextSwap);
            setPrevB(nextSwap, swp);
            b = next(swp);
            k = 0;
            do { setPos(b, originalPos[k]); ++k; b = next(b); } while (!(b == pivot));
            c.w_diag = false;
            setW(2, {XXX, XXX}); setW(3, {XXX, XXX});
            return 0;
        }
        return 0;
    }
    int wSwapTail() {
        if (c.numBeadsOn == 0) return -1;
        if (c.w_diag) return -1;
        const int swapLength = Mbar();
        int pivotSlice = c.worm[2] - swapLength;
        if (pivotSlice < 0) pivotSlice += c.M;
        fillList(pivotSlice);
        if (fullList.empty()) return -1;
        const double SigmaTail = getNorm(tail(), -1);
        std::array<int,3> wind{0, 0, 0};
        Bead pivot = selectPivot(wind);
        Bead b = pivot;
        for (int k = 0; k < swapLength; k++) {
            if (b == head()) return -1;
            b = next(b);
        }
        Bead swp = b;
        if (head() == swp) return -1;
        wst.attempted[11]++;
        const double SigmaSwap = getNorm(swp, 1);
        const double PNorm = std::min(SigmaTail / SigmaSwap, 1.0);
        if (R.rand() < PNorm) {
            setW(2, swp); setW(3, pivot);
            originalPos.clear();
            b = pivot;
            do {
                if (!(b == swp) && !(b == pivot)) originalPos.push_back(P(b));
                b = next(b);
            } while (!(b == next(swp)));
            const double oldAction = fullRange(pivot, swp);
            Bead prevSwap = prev(swp);
            setPrevB(tail(), prevSwap);
            setPrevB(swp, {XXX, XXX});
            setNextB(prevSwap, tail());
            setW(2, tail());
            setW(1, swp);
            const Bead s1 = sp1();
            int k = 0;
            b = pivot;
            do {
                if (!(b == s1) && !(b == pivot)) {
                    dVec p = stagingPos(prev(b), s1, swapLength, k, wind);
                    setPos(b, p);
                    ++k;
                    wst.bead_updates++;
                }
                b = next(b);
            } while (!(b == next(s1)));
            const double newAction = fullRange(pivot, s1);
            if (metro(newAction - oldAction)) { wst.accepted[11]++; wormUpdate(head(), swp); return 1; }
            setW(1, s1);
            setPrevB(tail(), {XXX, XXX});
            setPrevB(swp, prevSwap);
            setNextB(prevSwap, swp);
            b = next(pivot);
            k = 0;
            do { setPos(b, originalPos[k]); ++k; b = next(b); } while (!(b == swp));
            setW(2, {XXX, XXX}); setW(3, {XXX, XXX});
            c.w_diag = false;
            return 0;
        }
        return 0;
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

extern "C" int pgb_plain_worm_run(pgb_ctx* h, const pgb_worm_params* wp, int nsteps, int32_t* trace,
                                  int trace_cap, int* trace_len, double* energies, int* nparticles,
                                  pgb_worm_stats* stats) {
    if (!h || !wp || nsteps < 0) return PGB_EINVAL;
    Ctx& c = h->c;
    if (!c.loaded) return c.fail(PGB_ESTATE, "plain_worm_run: no path loaded");
    if (!c.mt_seeded) return c.fail(PGB_ESTATE, "plain_worm_run: call pgb_plain_seed first");
    if (wp->mbar < 2 || wp->mbar >= c.M || (wp->mbar % 2) || wp->temperature <= 0 || c.M % 2 ||
        wp->worm_constant <= 0 || wp->initial_num_particles < 0)
        return c.fail(PGB_EINVAL, "plain_worm_run: need even 2 <= mbar < M, even M, T > 0, C0 > 0, N0 >= 0");
    // the swap moves draw pivots from the LookupTable's single grid box,
    // which the reference has when the cutoff exceeds half of every side
    for (int d = 0; d < 3; ++d)
        if (!(c.p.rc > 0.5 * c.p.side[d]))
            return c.fail(PGB_EINVAL, "plain_worm_run: needs rc > L/2 (one LookupTable grid box)");
    pgb_move_params mp{};
    mp.mbar = wp->mbar; mp.diagonal_move = wp->diagonal_move; mp.var_updates = wp->var_updates;
    mp.max_wind = wp->max_wind; mp.temperature = wp->temperature; mp.p_com = 0.0; mp.num_updates = 0;
    Plain pl(c, mp);
    pl.wp = *wp;
    pl.Cw = wp->worm_constant / (1.0 * wp->mbar * c.M * (c.p.side[0] * c.p.side[1] * c.p.side[2]));
    pl.numBeads0 = wp->initial_num_particles * c.M;
    pl.pos.assign((size_t)c.M * c.Ne * 3, 0.0);
    int rc = pgb_get_positions(h, pl.pos.data());
    if (rc) return rc;
    if (!c.lk_valid) pl.lookupInit();
    if (pl.broken) return c.fail(PGB_ESTATE, "plain_worm_run: the loaded worm does not connect tail to head");
    // pimc.cpp:120-152: cumulative probabilities over the default move list;
    // com and the diagonal move act on any configuration, open and insert on
    // diagonal ones, the rest on off-diagonal ones
    const int onDiag[12] = {1, 1, 1, 0, 1, 0, 0, 0, 0, 0, 0, 0};
    const int onOff[12] = {1, 1, 0, 1, 0, 1, 1, 1, 1, 1, 1, 1};
    double cumDiag[12], cumOff[12], cd = 0.0, co = 0.0;
    for (int i = 0; i < 12; ++i) {
        if (onDiag[i]) cd += pl.prob[i];
        cumDiag[i] = cd;
        if (onOff[i]) co += pl.prob[i];
        cumOff[i] = co;
    }
    cumDiag[11] = 1.0 + EPS;
    cumOff[11] = 1.0 + EPS;
    int nu = wp->num_updates;
    if (nu <= 0) { nu = int(std::ceil(std::max(wp->initial_num_particles, 1) * c.M / (1.0 * wp->mbar))); if (nu < 100) nu = 100; }
    int ntr = 0;
    for (int step = 0; step < nsteps; ++step) {
        for (int n = 0; n < nu; ++n) {
            const double x = pl.R.rand();
            const double* cum = c.w_diag ? cumDiag : cumOff;
            const int index = int(std::lower_bound(cum, cum + 12, x) - cum);
            int r = -1;
            bool acc = false;
            switch (index) {
                case 0: { int m = pl.com(acc); r = m > 0 ? (acc ? 1 : 0) : -1; pl.wst.bead_updates += m;
                          if (m > 0) { pl.wst.attempted[0]++; if (acc) pl.wst.accepted[0]++; } break; }
                case 1: { int m = wp->diagonal_move == 1 ? pl.staging(acc) : pl.bisection(acc);
                          r = m > 0 ? (acc ? 1 : 0) : -1; pl.wst.bead_updates += m;
                          if (m > 0) { pl.wst.attempted[1]++; if (acc) pl.wst.accepted[1]++; } break; }
                case 2: r = pl.wOpen(); break;
                case 3: r = pl.wClose(); break;
                case 4: r = pl.wInsert(); break;
                case 5: r = pl.wRemove(); break;
                case 6: r = pl.wAdvanceHead(); break;
                case 7: r = pl.wRecedeHead(); break;
                case 8: r = pl.wAdvanceTail(); break;
                case 9: r = pl.wRecedeTail(); break;
                case 10: r = pl.wSwapHead(); break;
                case 11: r = pl.wSwapTail(); break;
            }
            if (pl.err) return pl.err;
            if (r == -2 || pl.full) {
                pl.flush();
                return c.fail(PGB_ENOMEM, "plain_worm_run: a slice outgrew the bead-array extent Ne");
            }
            if (pl.broken) return c.fail(PGB_ESTATE, "plain_worm_run: worm length walk did not reach the head");
            if (r >= 0 && trace && ntr < trace_cap) { trace[2 * ntr] = index; trace[2 * ntr + 1] = r; ++ntr; }
        }
        pl.flush();
        if (pl.err) return pl.err;
        if (energies) {
            if (c.w_diag) {
                double e[9];
                rc = pgb_energy(h, e);
                if (rc) return rc;
                energies[step] = e[8];
            } else energies[step] = std::nan("");
        }
        if (nparticles) nparticles[step] = c.numBeadsOn / c.M;
    }
    pl.flush();
    if (pl.err) return pl.err;
    pl.wst.diagonal = c.w_diag ? 1 : 0;
    if (trace_len) *trace_len = ntr;
    if (stats) *stats = pl.wst;
    return PGB_OK;
}
