/*
 * pimc_oracle.cpp -- FP64 CPU restatement of the reference WA-PIMC hot path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker).  Loaded by tests/, by
 * __graft_entry__.smoke() and by the CPU-baseline legs of bench.py; never by
 * the product library.  Every routine cites the reference file:line whose
 * behaviour it restates; loops keep the reference's summation order so that
 * FP64 results agree with a same-order FP64 evaluation to rounding.
 *
 * Built with -ffp-contract=off so that a*b+c is never fused: the results are
 * then the same on x86-64 and on aarch64 hosts, and the product's FP64 kernels
 * (built with -fmad=false) can be compared pair by pair.
 *
 * Parity unpinned: the reference cannot be compiled in this image (Boost and
 * <mdspan> are missing) and ships no golden vectors; see pimc_oracle.h.
 */
#include "pimc_oracle.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <chrono>
#include <iomanip>
#include <iostream>
#include <sstream>
#include <string>
#include <thread>
#include <vector>
#include <atomic>

namespace {

constexpr double EPS = 1.0e-7;   // include/common.h:89
constexpr int XXX = -1;          // include/common.h:93

using dVec = std::array<double, 3>;
using dMat = std::array<std::array<double, 3>, 3>;

inline double dot(const dVec& a, const dVec& b) {
    // include/array_math.h:210-216: result starts at 0 and accumulates in order
    double r = 0.0;
    for (int i = 0; i < 3; ++i) r += a[i] * b[i];
    return r;
}
inline dVec sub(const dVec& a, const dVec& b) { return {a[0]-b[0], a[1]-b[1], a[2]-b[2]}; }
inline dVec add(const dVec& a, const dVec& b) { return {a[0]+b[0], a[1]+b[1], a[2]+b[2]}; }
inline dVec scal(double s, const dVec& a) { return {s*a[0], s*a[1], s*a[2]}; }
inline void addto(dVec& a, const dVec& b) { a[0]+=b[0]; a[1]+=b[1]; a[2]+=b[2]; }
inline void subfrom(dVec& a, const dVec& b) { a[0]-=b[0]; a[1]-=b[1]; a[2]-=b[2]; }

// ---------------------------------------------------------------------------
// MT19937 as used by the reference (include/MersenneTwister.h:170-367).  This
// is the published Matsumoto-Nishimura generator with init_genrand seeding;
// rand() scales by 1/(2^32-1), randExc by 1/2^32, randInt(n) masks and
// rejects, randNorm is the polar Box-Muller form that drops the 2nd variate.
// ---------------------------------------------------------------------------
struct MT {
    static constexpr int N = 624, Mm = 397;
    uint32_t st[N];
    int left = 0, pos = 0;
    explicit MT(uint32_t seed) {
        st[0] = seed;
        for (int i = 1; i < N; ++i)
            st[i] = 1812433253u * (st[i-1] ^ (st[i-1] >> 30)) + (uint32_t)i;
        reload();
    }
    static uint32_t twist(uint32_t m, uint32_t s0, uint32_t s1) {
        uint32_t mix = (s0 & 0x80000000u) | (s1 & 0x7fffffffu);
        return m ^ (mix >> 1) ^ ((s1 & 1u) ? 0x9908b0dfu : 0u);
    }
    void reload() {
        int i = 0;
        for (; i < N - Mm; ++i) st[i] = twist(st[i + Mm], st[i], st[i + 1]);
        for (; i < N - 1; ++i) st[i] = twist(st[i + Mm - N], st[i], st[i + 1]);
        st[N - 1] = twist(st[Mm - 1], st[N - 1], st[0]);
        left = N; pos = 0;
    }
    uint32_t randInt() {
        if (left == 0) reload();
        --left;
        uint32_t y = st[pos++];
        y ^= (y >> 11);
        y ^= (y << 7) & 0x9d2c5680u;
        y ^= (y << 15) & 0xefc60000u;
        return y ^ (y >> 18);
    }
    uint32_t randInt(uint32_t n) {
        uint32_t used = n;
        used |= used >> 1; used |= used >> 2; used |= used >> 4;
        used |= used >> 8; used |= used >> 16;
        uint32_t i;
        do { i = randInt() & used; } while (i > n);
        return i;
    }
    double rand() { return double(randInt()) * (1.0 / 4294967295.0); }
    double randExc() { return double(randInt()) * (1.0 / 4294967296.0); }
    double randNorm(double mean, double stddev) {
        double x, y, r;
        do {
            x = 2.0 * rand() - 1.0;
            y = 2.0 * rand() - 1.0;
            r = x * x + y * y;
        } while (r >= 1.0 || r == 0.0);
        double s = std::sqrt(-2.0 * std::log(r) / r);
        return mean + x * s * stddev;
    }
};

// ---------------------------------------------------------------------------
// Aziz HFD-HE2 potential and its direct-lookup tables.
// Parameters: src/potential.cpp:1749-1788.  Functions: potential.cpp:1821-1907
// and include/potential.h:963-983 (F, dF, d2F).  Table: potential.h:163-183
// (r accumulated by r += dr, not k*dr), lookup potential.h:249-260.
// ---------------------------------------------------------------------------
struct AzizTables { std::vector<double> V, dV, d2V; };

struct Aziz {
    double rm, A, epsilon, alpha, beta, D, C6, C8, C10;
    double dr = 0; int tableLength = 0;
    // The tables of one parameter year: entry n is the value at the n-th
    // point of the r += dr grid, which does not depend on the table's length,
    // so every system of that year shares the longest table built so far and
    // reads only its own first tableLength entries.
    std::shared_ptr<const AzizTables> tab;
    double tailV = 0;

    void set_year(int year) {
        if (year == 1987) {
            epsilon = 10.948; rm = 2.9673; D = 1.4826; alpha = 10.43329537;
            beta = -2.27965105; C6 = 1.36745214; C8 = 0.42123807;
            C10 = 0.17473318; A = 1.8443101E5;
        } else if (year == 1995) {
            epsilon = 10.956; rm = 2.9683; D = 1.438; alpha = 10.5717543;
            beta = -2.07758779; C6 = 1.35186623; C8 = 0.4149514;
            C10 = 0.17151143; A = 1.86924404E5;
        } else {
            epsilon = 10.8; rm = 2.9673; D = 1.241314; alpha = 13.353384;
            beta = 0.0; C6 = 1.3732412; C8 = 0.4253785; C10 = 0.1781;
            A = 0.5448504E6;
        }
    }
    double F(double x) const { return (x < D ? std::exp(-(D/x - 1.0)*(D/x - 1.0)) : 1.0); }
    double dF(double x) const {
        double ix = 1.0/x;
        double r = 2.0*D*ix*ix*(D*ix-1.0)*std::exp(-(D*ix - 1.0)*(D*ix - 1.0));
        return (x < D ? r : 0.0);
    }
    double d2F(double x) const {
        double ix = 1.0/x;
        double r = 2.0*D*ix*ix*ix*( 2.0*D*D*D*ix*ix*ix - 4.0*D*D*ix*ix
                - D*ix + 2.0) * std::exp(-(D*ix - 1.0)*(D*ix - 1.0));
        return (x < D ? r : 0.0);
    }
    double valueV(double r) const {
        double x = r / rm;
        double Urep = A * std::exp(-alpha*x + beta*x*x);
        if (x < EPS) return 0.0;
        else if (x < 0.01) return (epsilon * Urep);
        double ix2 = 1.0 / (x * x);
        double ix6 = ix2 * ix2 * ix2;
        double ix8 = ix6 * ix2;
        double ix10 = ix8 * ix2;
        double Uatt = -( C6*ix6 + C8*ix8 + C10*ix10 ) * F(x);
        return ( epsilon * (Urep + Uatt) );
    }
    double valuedVdr(double r) const {
        double x = r / rm;
        double T1 = A * (-alpha + 2.0*beta*x) * std::exp(-alpha*x + beta*x*x);
        if (x < EPS) return 0.0;
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
    double valued2Vdr2(double r) const {
        double x = r / rm;
        double abFactor2 = (alpha - 2.0*beta*x)*(alpha-2.0*beta*x);
        double T1 = A * (2*beta + abFactor2) * std::exp(-alpha*x + beta*x*x);
        if (x < EPS) return 0.0;
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
    void init(int year, double maxSep, double rc, bool build_tables = true) {
        set_year(year);
        // potential.cpp:1795-1796 -> potential.h:163-183
        dr = (1.0E-6)*rm;
        tableLength = int(maxSep/dr);
        if (build_tables) {
            static std::mutex mu;
            static std::map<int, std::shared_ptr<const AzizTables>> cache;
            std::lock_guard<std::mutex> lk(mu);
            auto& c = cache[year];
            if (!c || (int)c->V.size() < tableLength) {
                auto t = std::make_shared<AzizTables>();
                t->V.assign(tableLength, 0.0); t->dV.assign(tableLength, 0.0); t->d2V.assign(tableLength, 0.0);
                double r = 0;
                for (int n = 0; n < tableLength; n++) {
                    t->V[n] = valueV(r);
                    t->dV[n] = valuedVdr(r);
                    t->d2V[n] = valued2Vdr2(r);
                    r += dr;
                }
                c = t;
            }
            tab = c;
        }
        // tail correction, potential.cpp:1801-1806
        double rmorc = rm / rc;
        double t2 = C6*std::pow(rmorc,3.0)/3.0;
        double t3 = C8*std::pow(rmorc,5.0)/5.0;
        double t4 = C10*std::pow(rmorc,7.0)/7.0;
        tailV = 2.0*M_PI*epsilon*(-rm*rm*rm*(t2+t3+t4));
    }
    // TabulatedPotential::direct, potential.h:249-260 (extremal values are 0)
    double direct(const std::vector<double>& T, double r) const {
        int k = int(r/dr);
        if (k <= 0) return 0.0;
        if (k >= tableLength) return 0.0;
        return T[k];
    }
    // AzizPotential::V/gradV/grad2V, potential.h:985-1017
    double V(const dVec& r) const { return direct(tab->V, std::sqrt(dot(r, r))); }
    dVec gradV(const dVec& r) const {
        double rnorm = std::sqrt(dot(r, r));
        double g = direct(tab->dV, rnorm) / rnorm;
        return {g*r[0], g*r[1], g*r[2]};
    }
    double grad2V(const dVec& r) const { return direct(tab->d2V, std::sqrt(dot(r, r))); }
};

enum BeadState { HEADTAIL = 0, SPECIAL = 1, NONE = 2 };

struct Sys {
    // Container (include/container.h:50-54, src/container.cpp:84-113)
    dVec side, sideInv, pSide;
    double volume;
    // constants
    int M, Ne;
    double tau, lambda, rc, rc2, mu;
    double VF[2], gF[2];
    int virialWindow;
    int shift = 1;
    Aziz pot;
    // Path (include/path.h:164-165) + Worm (include/worm.h)
    std::vector<double> pos;          // [M][Ne][3]
    std::vector<int> nxt, prv;        // [M][Ne][2]
    std::vector<uint8_t> on;          // [M][Ne]
    std::vector<int> nbs;             // numBeadsAtSlice
    int head[2], tail[2], sp1[2], sp2[2];
    int numBeadsOn = 0;
    std::vector<int> sepHist;         // action.h:109, 50 bins
    // worm-move state: LookupTable slice lists (one grid box), Worm scalars
    std::vector<std::vector<int>> hash;
    std::vector<int> label;
    bool diag = true;                 // Worm::isConfigDiagonal
    int gap = XXX, length = 0;
    dVec wsep{0.0, 0.0, 0.0};
    bool full = false, broken = false;
    double dSep;
    // scratch interaction list (LookupTable::beadList/beadSep)
    std::vector<int> list; std::vector<dVec> lsep;

    void putInBC(dVec& r) const {
        for (int i = 0; i < 3; ++i) r[i] -= pSide[i] * std::floor(r[i] * sideInv[i] + 0.5);
    }
    dVec P(int s, int p) const { const double* q = &pos[((size_t)s*Ne + p)*3]; return {q[0], q[1], q[2]}; }
    void setP(int s, int p, const dVec& v) { double* q = &pos[((size_t)s*Ne + p)*3]; q[0]=v[0]; q[1]=v[1]; q[2]=v[2]; }
    // Path::getSeparation(bead1,bead2) = r1 - r2 in BC (path.h:179-184)
    dVec sep(int s1, int p1, int s2, int p2) const { dVec d = sub(P(s1,p1), P(s2,p2)); putInBC(d); return d; }
    std::array<int,2> next(int s, int p) const { size_t i = ((size_t)s*Ne+p)*2; return {nxt[i], nxt[i+1]}; }
    std::array<int,2> prev(int s, int p) const { size_t i = ((size_t)s*Ne+p)*2; return {prv[i], prv[i+1]}; }
    std::array<int,2> nextN(std::array<int,2> b, int n) const { for (int m = 0; m < n; ++m) b = next(b[0], b[1]); return b; }
    std::array<int,2> prevN(std::array<int,2> b, int n) const { for (int m = 0; m < n; ++m) b = prev(b[0], b[1]); return b; }
    bool beadOn(int s, int p) const { return on[(size_t)s*Ne + p] != 0; }
    // Worm::getState, worm.h:110-118
    BeadState state(int s, int p) const {
        if ((s == head[0] && p == head[1]) || (s == tail[0] && p == tail[1])) return HEADTAIL;
        if ((s == sp1[0] && p == sp1[1]) || (s == sp2[0] && p == sp2[1])) return SPECIAL;
        return NONE;
    }
    // Worm::factor(state1, bead2), worm.cpp:108-118
    double factor(BeadState s1, int s, int p) const {
        BeadState s2 = state(s, p);
        if (s1 == NONE && s2 == NONE) return 1.0;
        if (s1 == HEADTAIL && s2 == HEADTAIL) return 0.0;
        return 0.5;
    }
    double t() const { return shift * tau; }   // ActionBase::tau(), action.h:136
    dVec velocity(int s, int p) const {        // Path::getVelocity, path.h:189-203
        if (s == XXX || p == XXX) return {0,0,0};
        auto n = next(s, p);
        if (n[0] == XXX && n[1] == XXX) return {0,0,0};
        dVec v = sub(P(n[0], n[1]), P(s, p));
        putInBC(v);
        return v;
    }
    int trueNumParticles() const { return numBeadsOn / M; }

    // LookupTable::updateInteractionList (src/lookuptable.cpp:464-516).  The
    // grid only accelerates the search: the list is every active bead on the
    // same slice, other than bead1, with |r2 - r1|^2 < rc^2 (minimum image).
    void interactionList(int s, int p) {
        list.clear(); lsep.clear();
        for (int q = 0; q < Ne; ++q) {
            if (q == p || !beadOn(s, q)) continue;
            dVec d = sep(s, q, s, p);
            if (dot(d, d) < rc2) { list.push_back(q); lsep.push_back(d); }
        }
    }
    // LocalAction::Vnn(bead, Vext), action.cpp:1044-1060 (free external: Vext = 0)
    double Vnn(int s, int p) {
        if (!beadOn(s, p)) return 0.0;
        double totVext = 0.0;
        double totVint = 0.0;
        interactionList(s, p);
        BeadState st1 = state(s, p);
        for (size_t n = 0; n < list.size(); ++n)
            totVint += factor(st1, s, list[n]) * pot.V(lsep[n]);
        return totVext + totVint;
    }
    // LocalAction::gradVnnSquared, action.cpp:1282-1337 (uses the current list)
    double gradVnnSquared(int s, int p) {
        double totF2 = 0.0;
        if (beadOn(s, p)) {
            dVec Fext1{0,0,0}, Fext2{0,0,0};
            dVec Fint1{0,0,0}, Fint2, Fint3;
            for (size_t n = 0; n < list.size(); ++n) {
                int b2 = list[n];
                Fint2 = pot.gradV(lsep[n]);
                subfrom(Fint1, Fint2);
                Fint3 = {0,0,0};
                for (size_t m = 0; m < list.size(); ++m) {
                    int b3 = list[m];
                    if (b3 != b2 && b3 != p) addto(Fint3, pot.gradV(sep(s, b2, s, b3)));
                }
                totF2 += dot(Fint2,Fint2) + 2.0*dot(Fext2,Fint2) + 2.0*dot(Fint2,Fint3);
            }
            totF2 += dot(Fext1,Fext1) + 2.0 * dot(Fext1,Fint1) + dot(Fint1,Fint1);
        }
        return totF2;
    }
    // LocalAction::potentialAction(bead), action.cpp:487-514
    double potentialAction(int s, int p) {
        int eo = s % 2;
        double bareU = VF[eo]*t()*Vnn(s, p);
        double corU = 0.0;
        if (shift == 1 && gF[eo] > EPS)
            corU = gF[eo]*t()*t()*t()*lambda*gradVnnSquared(s, p);
        return bareU + corU;
    }
    // list/range forms, action.cpp:522-620: only active beads contribute
    double actionOfActive(int s, int p) {
        int eo = s % 2;
        double bareU = VF[eo]*t()*Vnn(s, p);
        double corU = 0.0;
        if (shift == 1 && gF[eo] > EPS)
            corU = gF[eo]*t()*t()*t()*lambda*gradVnnSquared(s, p);
        return bareU + corU;
    }
    double potentialActionRange(std::array<int,2> start, std::array<int,2> end) {
        std::vector<std::array<int,2>> act;
        auto b = start;
        auto stop = next(end[0], end[1]);
        do {
            if (beadOn(b[0], b[1])) act.push_back(b);
            b = next(b[0], b[1]);
        } while (!(b == stop));
        double totU = 0.0;
        for (auto& a : act) totU += actionOfActive(a[0], a[1]);
        return totU;
    }
    double potentialActionList(const std::vector<std::array<int,2>>& beads) {
        double totU = 0.0;
        for (auto& a : beads)
            if (beadOn(a[0], a[1])) totU += actionOfActive(a[0], a[1]);
        return totU;
    }
    double barePotentialAction(int s, int p) { return VF[s%2]*t()*Vnn(s, p); }
    // potentialActionCorrection(bead), action.cpp:696-712
    double potentialActionCorrection(int s, int p) {
        int eo = s % 2;
        if (gF[eo] > EPS) {
            interactionList(s, p);
            return gF[eo]*t()*t()*t()*lambda*gradVnnSquared(s, p);
        }
        return 0.0;
    }
    void updateSepHist(const dVec& d) {      // action.cpp:216-224
        int nR = int(std::sqrt(dot(d, d))/dSep);
        if (nR >= 0 && nR < 50) ++sepHist[nR];
    }
    // LocalAction::V(slice), action.cpp:902-947
    std::array<double,2> Vslice(int s) {
        double totVint = 0.0, totVext = 0.0;
        int n = nbs[s];
        std::fill(sepHist.begin(), sepHist.end(), 0);
        for (int b1 = 0; b1 < n; ++b1) {
            BeadState st1 = state(s, b1);
            for (int b2 = b1 + 1; b2 < n; ++b2) {
                dVec d = sep(s, b2, s, b1);
                updateSepHist(d);
                totVint += factor(st1, s, b2) * pot.V(d);
            }
        }
        return {totVext, totVint};
    }
    // gradVSquared(slice), action.cpp:1188-1223
    double gradVSquaredSlice(int s) {
        double totF2 = 0.0;
        int n = nbs[s];
        for (int b1 = 0; b1 < n; ++b1) {
            dVec F{0,0,0};
            for (int b2 = 0; b2 < n; ++b2)
                if (b2 != b1) addto(F, pot.gradV(sep(s, b1, s, b2)));
            addto(F, dVec{0,0,0});
            totF2 += dot(F, F);
        }
        return totF2;
    }
    // gradVSquared(bead), action.cpp:1126-1180 (all beads of the slice)
    double gradVSquaredBead(int s, int p) {
        double totF2 = 0.0;
        if (!beadOn(s, p)) return 0.0;
        int n = nbs[s];
        dVec Fext1{0,0,0}, Fext2{0,0,0}, Fint1{0,0,0}, Fint2, Fint3;
        for (int b2 = 0; b2 < n; ++b2) {
            if (b2 == p) continue;
            Fint2 = pot.gradV(sep(s, b2, s, p));
            subfrom(Fint1, Fint2);
            Fint3 = {0,0,0};
            for (int b3 = 0; b3 < n; ++b3)
                if (b3 != b2 && b3 != p) addto(Fint3, pot.gradV(sep(s, b2, s, b3)));
            totF2 += dot(Fint2,Fint2) + 2.0*dot(Fext2,Fint2) + 2.0*dot(Fint2,Fint3);
        }
        totF2 += dot(Fext1,Fext1) + 2.0 * dot(Fext1,Fint1) + dot(Fint1,Fint1);
        return totF2;
    }
    // full path potential action, action.cpp:456-472
    double potentialActionFull() {
        double totU = 0.0;
        for (int s = 0; s < M; ++s) {
            int eo = s % 2;
            auto v = Vslice(s);
            totU += VF[eo]*t()*(0.0 + v[0] + v[1]);
            if (gF[eo] > EPS)
                totU += gF[eo] * t() * t() * t() * lambda * gradVSquaredSlice(s);
        }
        return totU;
    }
    // kinetic action of the whole path, action.cpp:306-369
    double kineticActionFull() {
        double totK = 0.0;
        for (int s = 0; s < M; ++s) {
            for (int p = 0; p < nbs[s]; ++p) {
                double k = 0.0;
                auto pr = prev(s, p);
                dVec v = velocity(pr[0], pr[1]);
                k += dot(v, v);
                v = velocity(s, p);
                k += dot(v, v);
                totK += k / (4.0*lambda*t());
            }
        }
        return totK;
    }
    // action.cpp:751-806
    double derivTau(int s) {
        int eo = s % 2;
        auto v = Vslice(s);
        double dU = VF[eo]*(0.0 + v[0] + v[1]);
        if (gF[eo] > EPS)
            dU += 3.0 * gF[eo] * t() * t() * lambda * gradVSquaredSlice(s);
        return dU;
    }
    double secondDerivTau(int s) {
        int eo = s % 2;
        double d2U = 0.0;
        if (gF[eo] > EPS) d2U += 6.0 * gF[eo] * t() * lambda * gradVSquaredSlice(s);
        return d2U;
    }
    double derivLambda(int s) {
        int eo = s % 2;
        if (gF[eo] > EPS) return gF[eo] * t() * t() * t() * gradVSquaredSlice(s);
        return 0.0;
    }
    // rDOTgradUterm1, action.cpp:1446-1478
    double rdotgradU1(int s) {
        int eo = s % 2, n = nbs[s];
        double rDotgV = 0.0;
        for (int b1 = 0; b1 < n; ++b1) {
            dVec gVi{0,0,0};
            for (int b2 = 0; b2 < n; ++b2)
                if (b2 != b1) addto(gVi, pot.gradV(sep(s, b1, s, b2)));
            dVec gV = add(dVec{0,0,0}, gVi);
            rDotgV += dot(gV, P(s, b1));
        }
        return VF[eo]*tau*rDotgV;
    }
    // T-matrix contraction shared by rDOTgradUterm2 / deltadotgradUterm2
    // (action.cpp:1503-1560, 1700-1745): returns T_i * gV_i for bead b1.
    dVec tmatGV(int s, int b1) {
        int n = nbs[s];
        dVec gV{0,0,0};
        dMat tMat{};
        dVec gVdotT{0,0,0};
        dVec gVe{0,0,0};
        double dVe = std::sqrt(dot(gVe,gVe));
        double g2Ve = 0.0;
        addto(gV, gVe);
        for (int b2 = 0; b2 < n; ++b2) {
            dVec rDiff = sep(s, b1, s, b2);
            double rmag = std::sqrt(dot(rDiff,rDiff));
            if (b2 != b1) {
                dVec gVi = pot.gradV(rDiff);
                double dVi = std::sqrt(dot(gVi,gVi));
                double g2Vi = pot.grad2V(rDiff);
                double dV = dVi + dVe;
                double d2V = g2Vi + g2Ve;
                for (int a = 0; a < 3; a++) {
                    for (int b = 0; b < 3; b++) {
                        tMat[a][b] += rDiff[a]*rDiff[b]*d2V/(rmag*rmag)
                            - rDiff[a]*rDiff[b]*dV/std::pow(rmag,3);
                        if (a == b) tMat[a][b] += dV/rmag;
                    }
                }
                addto(gV, gVi);
            }
        }
        // apply_matrix_vector_product, include/common.h:187-200
        for (int row = 0; row < 3; ++row) {
            double ip = 0.0;
            for (int c = 0; c < 3; ++c) ip += tMat[row][c] * gV[c];
            gVdotT[row] += ip;
        }
        return gVdotT;
    }
    double rdotgradU2(int s) {
        int eo = s % 2, n = nbs[s];
        double term2 = 0.0;
        if (gF[eo] > EPS) {
            for (int b1 = 0; b1 < n; ++b1) term2 += dot(tmatGV(s, b1), P(s, b1));
            term2 *= (2.0 * gF[eo] * std::pow(t(),3) * lambda);
        }
        return term2;
    }
    // centroid deviation used by deltadotgradUterm1/2, action.cpp:1625-1645
    dVec delta(int s, int b1) {
        dVec runTotMore{0,0,0}, runTotLess{0,0,0}, COM{0,0,0};
        dVec pos1 = P(s, b1);
        std::array<int,2> bead1{s, b1}, nOld = bead1, pOld = bead1;
        for (int g = 0; g < virialWindow; g++) {
            auto bn = nextN(bead1, g);
            auto bp = prevN(bead1, g);
            addto(runTotMore, sep(bn[0], bn[1], nOld[0], nOld[1]));
            addto(runTotLess, sep(bp[0], bp[1], pOld[0], pOld[1]));
            addto(COM, add(add(pos1, runTotMore), add(pos1, runTotLess)));
            nOld = bn; pOld = bp;
        }
        double den = 2.0*virialWindow;
        COM = {COM[0]/den, COM[1]/den, COM[2]/den};
        dVec d = sub(pos1, COM);
        putInBC(d);
        return d;
    }
    double deltadotgradU1(int s) {
        int eo = s % 2, n = nbs[s];
        double rDotgV = 0.0;
        for (int b1 = 0; b1 < n; ++b1) {
            dVec gVi{0,0,0}, gVe{0,0,0}, gV{0,0,0};
            for (int b2 = 0; b2 < n; ++b2)
                if (b2 != b1) addto(gVi, pot.gradV(sep(s, b1, s, b2)));
            addto(gVe, dVec{0,0,0});
            dVec d = delta(s, b1);
            addto(gV, add(gVe, gVi));
            rDotgV += dot(gV, d);
        }
        return VF[eo]*tau*rDotgV;
    }
    double deltadotgradU2(int s) {
        int eo = s % 2, n = nbs[s];
        double term2 = 0.0;
        if (gF[eo] > EPS) {
            for (int b1 = 0; b1 < n; ++b1) {
                dVec gT = tmatGV(s, b1);
                term2 += dot(gT, delta(s, b1));
            }
            term2 *= (2.0 * gF[eo] * std::pow(t(),3) * lambda);
        }
        return term2;
    }
    double virialKinCorr(int s) {   // action.cpp:1786-1803
        int eo = s % 2;
        double vKC = 0.0;
        if (gF[eo] > EPS) {
            vKC += gradVSquaredSlice(s);
            vKC *= gF[eo] * std::pow(t(),3) * lambda;
        }
        return vKC;
    }

    // EnergyEstimator::accumulate, estimator.cpp:940-1029 (PIMC slices,
    // sliceFactor = 1)
    void energy(double out[9]) {
        double totK = 0.0, totV = 0.0;
        double totVop[2] = {0.0, 0.0};
        int numParticles = trueNumParticles();
        int numTimeSlices = M;
        double tailV = (1.0*numParticles*numParticles/volume) * pot.tailV;
        double fourLambdaTauInv = 0.25 / (lambda * tau);
        double kinNorm = fourLambdaTauInv / (tau * numTimeSlices);
        double classicalKinetic = (0.5 * 3 / tau) * numParticles;
        for (int s = 0; s < M; ++s)
            for (int p = 0; p < nbs[s]; ++p) { dVec v = velocity(s, p); totK -= dot(v, v); }
        totK *= kinNorm;
        double t1 = 0.0, t2 = 0.0;
        int period = (gF[0] > EPS || gF[1] > EPS || VF[0] != VF[1]) ? 2 : 1;
        for (int s = 0; s < M; ++s) {
            t1 += 1.0*derivLambda(s);
            t2 += 1.0*derivTau(s);
            if (!(s % period)) {
                auto v = Vslice(s);
                totVop[0] += 1.0*v[0];
                totVop[1] += 1.0*v[1];
            }
        }
        t1 *= lambda/(tau*numTimeSlices);
        t2 /= 1.0*numTimeSlices;
        int nper = numTimeSlices/period;
        totVop[0] /= nper; totVop[1] /= nper;
        totK += (classicalKinetic + t1);
        totV = t2 - t1 + tailV;
        totVop[1] += tailV;
        out[0] = totK; out[1] = totV; out[2] = totVop[0]; out[3] = totVop[1];
        out[4] = totK + totV; out[5] = totK + totV - mu*numParticles;
        if (numParticles > 0) {
            out[6] = totK/(1.0*numParticles); out[7] = totV/(1.0*numParticles);
            out[8] = (totK + totV)/(1.0*numParticles);
        } else { out[6] = out[7] = out[8] = 0.0; }
    }

    // VirialEnergyEstimator::accumulate, estimator.cpp:1086-1252
    void virial(int quirk, double est[19]) {
        for (int i = 0; i < 19; ++i) est[i] = 0.0;
        double totVop = 0.0, thermE = 0.0, totEcv = 0.0, Kcv = 0.0;
        double T2 = 0.0, T3 = 0.0, T4 = 0.0, virKinTerm = 0.0;
        int numParticles = trueNumParticles();
        int numTimeSlices = M;
        double beta = 1.0*numTimeSlices*tau;
        int W = virialWindow;
        double tailV = (1.0*numParticles*numParticles/volume) * pot.tailV;
        double thermTerm1 = (0.5 * 3 / tau) * numParticles;
        double T1 = 0.5 * 3 * numParticles / (1.0*W*tau);
        double exchangeNorm = 1.0/(4.0*W*std::pow(tau,2)*lambda*numTimeSlices);
        double Pressure = 3*numParticles;
        double P2 = 0.0, P3 = 0.0;
        for (int s = 0; s < M; ++s) {
            for (int p = 0; p < nbs[s]; ++p) {
                std::array<int,2> b1{s, p};
                dVec vel2 = velocity(s, p);
                auto nOld = b1;
                dVec vel1{0,0,0};
                for (int g = 1; g <= W; g++) {
                    auto bn = nextN(b1, g);
                    addto(vel1, sep(bn[0], bn[1], nOld[0], nOld[1]));
                    nOld = bn;
                }
                T2 -= dot(vel1, vel2);
                thermE -= dot(vel2, vel2);
            }
        }
        P2 = thermE;
        T2 *= exchangeNorm;
        P2 /= (2.0*lambda*tau*numTimeSlices);
        Pressure += P2;
        double T5 = 0.0;
        for (int s = 0; s < M; ++s) {
            int eo = s % 2;
            T3 += deltadotgradU1(s);
            T4 += deltadotgradU2(s);
            T5 += derivTau(s);
            virKinTerm += virialKinCorr(s);
            if (eo == 0) { auto v = Vslice(s); totVop += (0.0 + v[0] + v[1]); }
            P3 += rdotgradU1(s) + rdotgradU2(s);
        }
        P3 *= (1.0/(2.0*numTimeSlices));
        Pressure -= P3;
        Pressure /= (3*tau*volume);
        totVop /= (0.5 * numTimeSlices);
        totVop += tailV;
        T3 /= (2.0*beta);
        T4 /= (1.0*beta);
        T5 /= (1.0*numTimeSlices);
        virKinTerm /= (0.5*beta);
        thermE *= (0.25 / (lambda * tau)) / (tau * numTimeSlices);
        thermE += thermTerm1;
        thermE += T5;
        thermE += tailV;
        totEcv = T1 + T2 + T3 + T4 + T5 + tailV;
        Kcv = T1 + T2 + T3 + T4 + virKinTerm;
        double dEdB = (-1.0*T1 - 2.0*T2 + 2.0*T4)/tau;
        for (int s = 0; s < M; s++) dEdB += secondDerivTau(s)/(1.0*numTimeSlices);
        dEdB *= beta*beta/(1.0*numTimeSlices);
        est[0] += totEcv - totVop;
        est[1] += Kcv;
        est[2] += totVop;
        est[3] += totEcv - Kcv;
        est[4] += totEcv;
        est[5] += totEcv - mu*numParticles;
        if (numParticles > 0) {
            est[6] += (totEcv - totVop)/(1.0*numParticles);
            est[7] += Kcv/(1.0*numParticles);
            est[8] += totVop/(1.0*numParticles);
            est[9] += (totEcv - Kcv)/(1.0*numParticles);
            est[10] += totEcv/(1.0*numParticles);
        }
        est[11] += totEcv*thermE*beta*beta;
        est[12] += totEcv*beta;
        est[13] += dEdB;
        est[14] += totEcv*thermE*beta*beta*totEcv*beta;
        // estimator.cpp:1244 indexes the map with "cVCov2", a key that does not
        // exist: operator[] inserts it with index 0, so the term lands in K_op.
        est[quirk ? 0 : 15] += totEcv*beta*dEdB;
        est[16] += totEcv*thermE*beta*beta*dEdB;
        est[17] += thermE;
        est[18] += Pressure;
    }
};

Sys* make_sys(const orc_params* p, bool tables = true) {
    Sys* s = new Sys();
    for (int i = 0; i < 3; ++i) {
        s->side[i] = p->side[i];
        s->sideInv[i] = 1.0 / p->side[i];
        s->pSide[i] = p->side[i];
    }
    s->volume = s->side[0] * s->side[1] * s->side[2];
    s->M = p->num_slices; s->Ne = p->num_ptcl_ext;
    s->tau = p->tau; s->lambda = p->lambda; s->rc = p->rc; s->rc2 = p->rc * p->rc;
    s->mu = p->mu;
    s->VF[0] = p->vfactor[0]; s->VF[1] = p->vfactor[1];
    s->gF[0] = p->gradvfactor[0]; s->gF[1] = p->gradvfactor[1];
    s->virialWindow = p->virial_window > 0 ? p->virial_window : 5;
    // Prism::maxSep = |side/2| (src/container.cpp:103)
    dVec h = {s->side[0]/2.0, s->side[1]/2.0, s->side[2]/2.0};
    double maxSep = std::sqrt(dot(h, h));
    s->pot.init(p->aziz_year, maxSep, p->rc, tables);
    s->sepHist.assign(50, 0);
    s->dSep = 0.5*std::sqrt(3.0)*s->side[2] / 50.0;
    size_t nb = (size_t)s->M * s->Ne;
    s->pos.assign(nb*3, 0.0);
    s->nxt.assign(nb*2, XXX); s->prv.assign(nb*2, XXX);
    s->on.assign(nb, 0); s->nbs.assign(s->M, 0);
    for (int i = 0; i < 2; ++i) s->head[i] = s->tail[i] = s->sp1[i] = s->sp2[i] = XXX;
    return s;
}

void recount(Sys* s) {
    s->numBeadsOn = 0;
    for (int sl = 0; sl < s->M; ++sl) {
        int c = 0;
        for (int p = 0; p < s->Ne; ++p) if (s->beadOn(sl, p)) ++c;
        s->nbs[sl] = c;
        s->numBeadsOn += c;
    }
}

// ---------------------------------------------------------------------------
// Diagonal moves (src/move.cpp) and the step driver (src/pimc.cpp:724-786).
// ---------------------------------------------------------------------------
struct Mover {
    Sys& S; MT& R; orc_move_params mp;
    double sqrtLambdaTau, sqrt2LambdaTau, comDelta;
    int b;                         // bisection levels (constants.cpp:116-120)
    int numWind;
    std::vector<std::array<int,3>> winding;
    std::vector<double> cumrho0;
    orc_move_stats st{};

    Mover(Sys& s, MT& r, const orc_move_params& p) : S(s), R(r), mp(p) {
        sqrtLambdaTau = std::sqrt(S.lambda * S.tau);
        sqrt2LambdaTau = std::sqrt(2.0)*sqrtLambdaTau;
        double dB = 2.0*std::sqrt(M_PI * S.lambda / mp.temperature);
        comDelta = 0.04*dB;                                   // constants.cpp:165
        b = int(std::ceil(std::log(1.0*mp.mbar) / std::log(2.0) - EPS));
        while ((int)std::floor(std::pow(2.0, 1.0*b) + EPS) >= S.M) b--;
        int mw = mp.max_wind;
        numWind = 1;
        for (int i = 0; i < 3; ++i) numWind *= (2*mw + 1);
        // MoveBase ctor, move.cpp:88-108; the stable_sort that follows compares
        // w1 with itself (move.cpp:112-125) and therefore keeps this order.
        for (int n = 0; n < numWind; n++) {
            std::array<int,3> w{0,0,0};
            for (int i = 0; i < 3; i++) {
                int scale = 1;
                for (int j = i+1; j < 3; j++) scale *= (2*mw + 1);
                w[i] = (n/scale) % (2*mw + 1);
                w[i] -= (w[i] > mw)*(2*mw + 1);
            }
            winding.push_back(w);
        }
        cumrho0.resize(numWind);
    }
    // ActionBase::rho0(vel, M), action.cpp:254-260
    double rho0(const dVec& vel, int Mx) {
        double rho0Norm = std::pow(4.0*M_PI*S.lambda*Mx*S.tau, -0.5*3);
        return rho0Norm * std::exp(-dot(vel,vel) / (4.0*S.lambda*Mx*S.tau));
    }
    // MoveBase::sampleWindingSector, move.cpp:362-397
    std::array<int,3> sampleWinding(std::array<int,2> sb, std::array<int,2> eb, int stageLength) {
        dVec vel = sub(S.P(eb[0], eb[1]), S.P(sb[0], sb[1]));
        cumrho0[0] = rho0(vel, stageLength);
        double total = cumrho0[0];
        for (int n = 1; n < numWind; n++) {
            dVec velW = vel;
            for (int i = 0; i < 3; ++i) velW[i] = vel[i] + winding[n][i]*S.side[i];
            double c = rho0(velW, stageLength);
            total += c;
            cumrho0[n] = cumrho0[n-1] + c;
        }
        for (auto& c : cumrho0) c /= total;
        int index = int(std::lower_bound(cumrho0.begin(), cumrho0.end(), R.rand()) - cumrho0.begin());
        if (index >= numWind) index = numWind - 1;
        return winding[index];
    }
    // MoveBase::newStagingPosition (winding form), move.cpp:301-338
    dVec newStagingPosition(std::array<int,2> nb, std::array<int,2> eb, int stageLength, int k, std::array<int,3>& wind) {
        double f1 = 1.0 * (stageLength - k - 1);
        double f2 = 1.0 / (1.0*(stageLength - k));
        double sqrtLambdaKTau = sqrt2LambdaTau * std::sqrt(f1 * f2);
        dVec neighborPos = S.P(nb[0], nb[1]);
        dVec e = S.P(eb[0], eb[1]);
        dVec r;
        for (int i = 0; i < 3; ++i) r[i] = (e[i] + S.side[i]*wind[i]) - neighborPos[i];
        for (int i = 0; i < 3; ++i) r[i] *= f2;
        for (int i = 0; i < 3; ++i) r[i] += neighborPos[i];
        for (int i = 0; i < 3; i++) r[i] = R.randNorm(r[i], sqrtLambdaKTau);
        for (int i = 0; i < 3; i++) {
            while (r[i] < -0.5*S.side[i]) { wind[i]++; r[i] += S.side[i]; }
            while (r[i] >= 0.5*S.side[i]) { wind[i]--; r[i] -= S.side[i]; }
        }
        S.putInBC(r);
        return r;
    }
    // MoveBase::newBisectionPosition, move.cpp:467-488
    dVec newBisectionPosition(std::array<int,2> bead, int lshift) {
        double delta = sqrtLambdaTau*std::sqrt(1.0*lshift);
        auto nB = S.prevN(bead, lshift);
        auto nx = S.nextN(bead, lshift);
        dVec r = S.sep(nx[0], nx[1], nB[0], nB[1]);
        for (int i = 0; i < 3; ++i) r[i] *= 0.5;
        dVec pn = S.P(nB[0], nB[1]);
        for (int i = 0; i < 3; ++i) r[i] += pn[i];
        for (int i = 0; i < 3; i++) r[i] = R.randNorm(r[i], delta);
        S.putInBC(r);
        return r;
    }
    // CenterOfMassMove::attemptMove, move.cpp:1124-1262
    int com(bool& accepted) {
        accepted = false;
        if (S.numBeadsOn == 0) return 0;
        int startSlice = 0;
        if (S.nbs[startSlice] == 0) return 0;
        std::array<int,2> first{startSlice, (int)R.randInt((uint32_t)(S.nbs[startSlice]-1))};
        std::array<int,2> sb = first, eb;
        auto isX = [](std::array<int,2> a) { return a[0] == XXX && a[1] == XXX; };
        if (!isX(S.prev(sb[0], sb[1]))) {
            do { sb = S.prev(sb[0], sb[1]); }
            while (!(S.prev(sb[0], sb[1]) == first) && !isX(S.prev(sb[0], sb[1])));
        }
        if (S.prev(sb[0], sb[1]) == first) { sb = first; eb = S.prev(sb[0], sb[1]); }
        else {
            eb = first;
            if (!isX(S.next(eb[0], eb[1]))) {
                do { eb = S.next(eb[0], eb[1]); } while (!isX(S.next(eb[0], eb[1])));
            }
        }
        int wlLength = 0;
        auto b = sb;
        auto stop = S.next(eb[0], eb[1]);
        do { ++wlLength; b = S.next(b[0], b[1]); } while (!(b == stop));
        if (wlLength > S.M) return 0;
        st.attempted[0]++;
        dVec shiftv;
        for (int i = 0; i < 3; i++) shiftv[i] = comDelta*(-0.5 + R.rand());
        double oldA = S.potentialActionRange(sb, eb);
        b = sb;
        do {
            dVec p = add(S.P(b[0], b[1]), shiftv);
            S.putInBC(p);
            S.setP(b[0], b[1], p);
            b = S.next(b[0], b[1]);
        } while (!(b == stop));
        double newA = S.potentialActionRange(sb, eb);
        if (R.rand() < std::exp(-(newA - oldA))) { accepted = true; st.accepted[0]++; }
        else {
            b = sb;
            do {
                dVec p = sub(S.P(b[0], b[1]), shiftv);
                S.putInBC(p);
                S.setP(b[0], b[1], p);
                b = S.next(b[0], b[1]);
            } while (!(b == stop));
        }
        return wlLength;
    }
    // StagingMove::attemptMove, move.cpp:1315-1412
    int staging(bool& accepted) {
        accepted = false;
        if (S.numBeadsOn == 0) return 0;
        if (S.trueNumParticles() == 0) return 0;
        std::array<int,2> sb;
        sb[0] = (int)R.randInt((uint32_t)(S.M - 1));
        if (S.nbs[sb[0]] == 0) return 0;
        sb[1] = (int)R.randInt((uint32_t)(S.nbs[sb[0]] - 1));
        int stageLength = mp.mbar;
        if (mp.var_updates) stageLength = 2 + (int)R.randInt((uint32_t)(mp.mbar - 2));
        auto b = sb;
        for (int k = 0; k < stageLength; k++) {
            auto nx = S.next(b[0], b[1]);
            if (!S.beadOn(b[0], b[1]) || (nx[0] == XXX && nx[1] == XXX)) return 0;
            b = nx;
        }
        std::array<int,2> eb = b;
        st.attempted[1]++;
        auto wind = sampleWinding(sb, eb, stageLength);
        auto pe = S.prev(eb[0], eb[1]);
        double oldA = S.potentialActionRange(sb, pe);
        std::vector<dVec> orig;
        b = sb;
        int k = 0;
        do {
            b = S.next(b[0], b[1]);
            orig.push_back(S.P(b[0], b[1]));
            auto pb = S.prev(b[0], b[1]);
            dVec np = newStagingPosition(pb, eb, stageLength, k, wind);
            S.setP(b[0], b[1], np);
            ++k;
        } while (!(b == S.prev(eb[0], eb[1])));
        double newA = S.potentialActionRange(sb, pe);
        if (R.rand() < std::exp(-(newA - oldA))) { accepted = true; st.accepted[1]++; }
        else {
            b = sb; k = 0;
            do { b = S.next(b[0], b[1]); S.setP(b[0], b[1], orig[k]); ++k; }
            while (!(b == S.prev(eb[0], eb[1])));
        }
        return stageLength - 1;
    }
    // BisectionMove::attemptMove (local action), move.cpp:1484-1666
    int bisection(bool& accepted) {
        accepted = false;
        if (S.numBeadsOn == 0) return 0;
        int numLevels = b;
        if (mp.var_updates) numLevels = 1 + (int)R.randInt((uint32_t)(b - 1));
        int numActive = (int)std::floor(std::pow(2.0, 1.0*numLevels) + EPS) - 1;
        if (S.trueNumParticles() == 0) return 0;
        std::array<int,2> sb;
        sb[0] = (int)R.randInt((uint32_t)(S.M - 1));
        if (S.nbs[sb[0]] == 0) return 0;
        sb[1] = (int)R.randInt((uint32_t)(S.nbs[sb[0]] - 1));
        auto bb = sb;
        for (int k = 0; k < numActive + 1; k++) {
            auto nx = S.next(bb[0], bb[1]);
            if (!S.beadOn(bb[0], bb[1]) || (nx[0] == XXX && nx[1] == XXX)) return 0;
            bb = nx;
        }
        std::array<int,2> eb = bb;
        st.attempted[2]++;
        int nmax = (int)std::floor(std::pow(2.0, 1.0*b) + EPS) - 1;
        std::vector<char> include(nmax, 1);
        std::vector<dVec> origPos(nmax), newPos(nmax);
        double oldDelta = 0.0;
        int moved = 0;
        for (int level = numLevels; level > 0; level--) {
            int shift = (int)std::floor(std::pow(2.0, 1.0*(level-1)) + EPS);
            S.shift = shift;
            double oldA = 0.0, newA = 0.0;
            std::vector<std::array<int,2>> inc, prevLev;
            std::vector<int> incIdx, prevIdx;
            auto bi = S.nextN(sb, shift);
            int k = 1;
            do {
                int n = k*shift - 1;
                if (include[n]) { origPos[n] = S.P(bi[0], bi[1]); inc.push_back(bi); incIdx.push_back(n); }
                else if (level == 1) { prevLev.push_back(bi); prevIdx.push_back(n); }
                ++k;
                bi = S.nextN(bi, shift);
            } while (!(bi == eb));
            oldA += S.potentialActionList(inc);
            for (size_t i = 0; i < inc.size(); ++i) {
                int n = incIdx[i];
                newPos[n] = newBisectionPosition(inc[i], shift);
                S.setP(inc[i][0], inc[i][1], newPos[n]);
                include[n] = 0;
            }
            moved += (int)inc.size();
            newA += S.potentialActionList(inc);
            if (level == 1) {
                newA += S.potentialActionList(prevLev);
                for (size_t i = 0; i < prevLev.size(); ++i) S.setP(prevLev[i][0], prevLev[i][1], origPos[prevIdx[i]]);
                oldA += S.potentialActionList(prevLev);
                for (size_t i = 0; i < prevLev.size(); ++i) S.setP(prevLev[i][0], prevLev[i][1], newPos[prevIdx[i]]);
            }
            double dA = newA - oldA;
            if (R.rand() < std::exp(-dA + oldDelta)) {
                if (level == 1) { accepted = true; st.accepted[2]++; S.shift = 1; }
            } else {
                auto bk = sb;
                int kk = 0;
                do {
                    bk = S.next(bk[0], bk[1]);
                    if (!include[kk]) S.setP(bk[0], bk[1], origPos[kk]);
                    ++kk;
                } while (!(bk == S.prev(eb[0], eb[1])));
                S.shift = 1;
                break;
            }
            oldDelta = dA;
        }
        S.shift = 1;
        return moved;
    }
};

int run_steps(Sys* s, MT* mt, const orc_move_params* mp, int nsteps,
              int32_t* trace, int trace_cap, double* energies, orc_move_stats* stats) {
    Mover mv(*s, *mt, *mp);
    int N0 = s->trueNumParticles();
    int numUpdates = mp->num_updates;
    if (numUpdates <= 0) {
        numUpdates = int(std::ceil(std::max(N0, 1)*s->M / (1.0*mp->mbar)));
        if (numUpdates < 100) numUpdates = 100;
    }
    // cumulative probabilities, pimc.cpp:120-152 (last entry forced to 1+EPS)
    double cum[2] = {mp->p_com, 1.0 + EPS};
    int ntr = 0;
    for (int step = 0; step < nsteps; ++step) {
        for (int n = 0; n < numUpdates; ++n) {
            double x = mt->rand();
            int index = int(std::lower_bound(cum, cum + 2, x) - cum);
            bool acc = false;
            int moved, code;
            if (index == 0) { moved = mv.com(acc); code = 0; }
            else if (mp->diagonal_move == 1) { moved = mv.staging(acc); code = 1; }
            else { moved = mv.bisection(acc); code = 2; }
            mv.st.bead_updates += moved;
            if (trace && ntr < trace_cap && moved > 0) {
                trace[2*ntr] = code; trace[2*ntr+1] = acc ? 1 : 0; ++ntr;
            }
        }
        if (energies) { double e[9]; s->energy(e); energies[step] = e[8]; }
    }
    if (stats) *stats = mv.st;
    return ntr;
}

#include "pimc_oracle_worm.inc"

// Worm scalars of a loaded path (Worm::update without the unlinking)
void worm_from_load(Sys& S) {
    S.full = S.broken = false;
    if (S.head[0] == XXX) { S.diag = true; S.gap = XXX; S.length = 0; S.wsep = {0.0, 0.0, 0.0}; return; }
    S.diag = false;
    S.gap = S.tail[0] - S.head[0];
    if (S.gap < 0) S.gap += S.M;
    Bead b{S.tail[0], S.tail[1]};
    S.length = 0;
    const long long limit = (long long)S.M * S.Ne + 1;
    while (true) {
        ++S.length;
        if (b[0] == S.head[0] && b[1] == S.head[1]) break;
        b = S.next(b[0], b[1]);
        if (isXB(b) || S.length > limit) { S.broken = true; break; }
    }
    --S.length;   // the loop above counts the head once more than Worm::update
    S.wsep = S.sep(S.tail[0], S.tail[1], S.head[0], S.head[1]);
}

}  // namespace

struct orc_sys { Sys* s; };
struct orc_mt { MT m; explicit orc_mt(uint32_t seed) : m(seed) {} };

extern "C" {

void orc_aziz_values(int year, double r, double out3[3]) {
    Aziz a; a.set_year(year);
    out3[0] = a.valueV(r); out3[1] = a.valuedVdr(r); out3[2] = a.valued2Vdr2(r);
}

orc_sys* orc_create(const orc_params* p) { return new orc_sys{make_sys(p)}; }
void orc_destroy(orc_sys* s) { if (s) { delete s->s; delete s; } }
int orc_table_length(orc_sys* s) { return s->s->pot.tableLength; }
double orc_table_dr(orc_sys* s) { return s->s->pot.dr; }
double orc_tailV(orc_sys* s) { return s->s->pot.tailV; }
void orc_copy_tables(orc_sys* s, double* V, double* dV, double* d2V) {
    auto& p = s->s->pot;
    if (V) std::memcpy(V, p.tab->V.data(), sizeof(double)*p.tableLength);
    if (dV) std::memcpy(dV, p.tab->dV.data(), sizeof(double)*p.tableLength);
    if (d2V) std::memcpy(d2V, p.tab->d2V.data(), sizeof(double)*p.tableLength);
}
double orc_V(orc_sys* s, const double sep[3]) { return s->s->pot.V({sep[0], sep[1], sep[2]}); }
void orc_gradV(orc_sys* s, const double sep[3], double out[3]) {
    dVec g = s->s->pot.gradV({sep[0], sep[1], sep[2]});
    out[0] = g[0]; out[1] = g[1]; out[2] = g[2];
}
double orc_grad2V(orc_sys* s, const double sep[3]) { return s->s->pot.grad2V({sep[0], sep[1], sep[2]}); }

void orc_load_path(orc_sys* h, const double* pos, const int32_t* next,
                   const int32_t* prev, const uint8_t* on, const int32_t* worm8) {
    Sys* s = h->s;
    size_t nb = (size_t)s->M * s->Ne;
    std::memcpy(s->pos.data(), pos, nb*3*sizeof(double));
    for (size_t i = 0; i < nb*2; ++i) { s->nxt[i] = next[i]; s->prv[i] = prev[i]; }
    std::memcpy(s->on.data(), on, nb);
    s->head[0] = worm8[0]; s->head[1] = worm8[1];
    s->tail[0] = worm8[2]; s->tail[1] = worm8[3];
    s->sp1[0] = worm8[4]; s->sp1[1] = worm8[5];
    s->sp2[0] = worm8[6]; s->sp2[1] = worm8[7];
    recount(s);
    reset_lookup(*s);
    worm_from_load(*s);
}
void orc_get_positions(orc_sys* h, double* pos) {
    std::memcpy(pos, h->s->pos.data(), h->s->pos.size()*sizeof(double));
}
void orc_update_bead(orc_sys* h, int slice, int ptcl, const double p[3]) {
    h->s->setP(slice, ptcl, {p[0], p[1], p[2]});
}
void orc_set_shift(orc_sys* h, int shift) { h->s->shift = shift; }

double orc_potential_action_bead(orc_sys* h, int s, int p) { return h->s->potentialAction(s, p); }
double orc_bare_potential_action(orc_sys* h, int s, int p) { return h->s->barePotentialAction(s, p); }
double orc_potential_action_correction(orc_sys* h, int s, int p) { return h->s->potentialActionCorrection(s, p); }
double orc_potential_action_range(orc_sys* h, int s0, int p0, int s1, int p1) {
    return h->s->potentialActionRange({s0, p0}, {s1, p1});
}
double orc_potential_action_list(orc_sys* h, const int32_t* beads, int k) {
    std::vector<std::array<int,2>> v;
    for (int i = 0; i < k; ++i) v.push_back({beads[2*i], beads[2*i+1]});
    return h->s->potentialActionList(v);
}
double orc_potential_action_full(orc_sys* h) { return h->s->potentialActionFull(); }
double orc_kinetic_action_full(orc_sys* h) { return h->s->kineticActionFull(); }
double orc_Vnn(orc_sys* h, int s, int p) { return h->s->Vnn(s, p); }
double orc_gradVnnSquared(orc_sys* h, int s, int p) { h->s->interactionList(s, p); return h->s->gradVnnSquared(s, p); }
void orc_V_slice(orc_sys* h, int s, double out2[2]) { auto v = h->s->Vslice(s); out2[0] = v[0]; out2[1] = v[1]; }
double orc_gradVSquared_slice(orc_sys* h, int s) { return h->s->gradVSquaredSlice(s); }
double orc_gradVSquared_bead(orc_sys* h, int s, int p) { return h->s->gradVSquaredBead(s, p); }
double orc_deriv_tau(orc_sys* h, int s) { return h->s->derivTau(s); }
double orc_deriv_lambda(orc_sys* h, int s) { return h->s->derivLambda(s); }
double orc_second_deriv_tau(orc_sys* h, int s) { return h->s->secondDerivTau(s); }
double orc_rdotgradU1(orc_sys* h, int s) { return h->s->rdotgradU1(s); }
double orc_rdotgradU2(orc_sys* h, int s) { return h->s->rdotgradU2(s); }
double orc_deltadotgradU1(orc_sys* h, int s) { return h->s->deltadotgradU1(s); }
double orc_deltadotgradU2(orc_sys* h, int s) { return h->s->deltadotgradU2(s); }
double orc_virial_kin_corr(orc_sys* h, int s) { return h->s->virialKinCorr(s); }

void orc_energy(orc_sys* h, double out9[9]) { h->s->energy(out9); }
void orc_virial(orc_sys* h, int quirk, double out19[19]) { h->s->virial(quirk, out19); }

// EstimatorBase::getQVectors, src/estimator.cpp:439-570
int orc_qvectors(const char* type, const char* input, const double side[3], double* qout, int cap) {
    std::string inputType(type), in(input);
    std::vector<dVec> qValues;
    std::istringstream iss(in);
    std::vector<std::string> tokens;
    std::string tok;
    while (iss >> tok) tokens.push_back(tok);
    if (inputType == "int" || inputType == "float") {
        for (size_t i = 0; i + 2 < tokens.size(); i += 3) {
            dVec q;
            for (int j = 0; j < 3; ++j) {
                if (inputType == "int") q[j] = (2.0 * M_PI / side[j]) * std::stoi(tokens[i + j]);
                else q[j] = std::stof(tokens[i + j]);
            }
            qValues.push_back(q);
        }
    }
    if (inputType == "max_int" || inputType == "max_float") {
        std::array<int,3> qmi{}, qi{};
        dVec qmax{};
        for (int i = 0; i < 3; ++i) {
            if (inputType == "max_int") {
                qmi[i] = std::abs(std::stoi(tokens[i]));
                qmax[i] = qmi[i] * 2.0 * M_PI / side[i];
            } else {
                qmax[i] = std::stof(tokens[i]);
            }
        }
        double qmagmax = std::sqrt(dot(qmax, qmax));
        if (inputType == "max_float")
            for (int i = 0; i < 3; ++i) qmi[i] = 1 + static_cast<int>(qmagmax * side[i] / 2.0 / M_PI);
        int n_q = 1;
        dVec q;
        for (int i = 0; i < 3; ++i) {
            n_q *= 2 * qmi[i] + 1;
            qi[i] = -qmi[i];
            q[i] = qi[i] * 2.0 * M_PI / side[i];
        }
        if (std::sqrt(dot(q, q)) <= qmagmax) qValues.push_back(q);
        int pos = 2, count = 0;
        while (count < n_q - 1) {
            if (qi[pos] == qmi[pos]) { qi[pos] = -qmi[pos]; pos -= 1; }
            else {
                qi[pos] += 1;
                for (int i = 0; i < 3; ++i) q[i] = qi[i] * 2.0 * M_PI / side[i];
                if (std::sqrt(dot(q, q)) <= qmagmax) qValues.push_back(q);
                count += 1;
                pos = 2;
            }
        }
    }
    if (inputType == "file_int" || inputType == "file_float") {
        FILE* f = std::fopen(in.c_str(), "r");
        if (f) {
            char line[4096];
            while (std::fgets(line, sizeof line, f)) {
                std::istringstream ls(line);
                dVec q;
                if (inputType == "file_int") {
                    int a[3];
                    if (!(ls >> a[0] >> a[1] >> a[2])) continue;
                    for (int i = 0; i < 3; ++i) q[i] = (2.0 * M_PI / side[i]) * a[i];
                } else {
                    float a[3];
                    if (!(ls >> a[0] >> a[1] >> a[2])) continue;
                    for (int i = 0; i < 3; ++i) q[i] = a[i];
                }
                qValues.push_back(q);
            }
            std::fclose(f);
        }
    }
    int n = (int)qValues.size();
    for (int i = 0; i < n && i < cap; ++i) for (int j = 0; j < 3; ++j) qout[3*i+j] = qValues[i][j];
    return n;
}

// StaticStructureFactorEstimator::accumulate, estimator.cpp:3705-3737
void orc_ssf_pairwise(orc_sys* h, const double* q, int nq, double* out) {
    Sys* s = h->s;
    int N = s->trueNumParticles();
    for (int iq = 0; iq < nq; ++iq) {
        dVec qv{q[3*iq], q[3*iq+1], q[3*iq+2]};
        double sf = 0.0;
        for (int t = 0; t < s->M; ++t) {
            for (int b1 = 0; b1 < s->nbs[t]; ++b1) {
                sf += 1.0;
                for (int b2 = b1 + 1; b2 < s->nbs[t]; ++b2)
                    sf += 2*std::cos(dot(s->sep(t, b1, t, b2), qv));
            }
        }
        out[iq] = (sf / N) * (1.0 / s->M);
    }
}

// CylinderStaticStructureFactorEstimator::accumulate (estimator.cpp:5415-5458)
// with include() (4309-4311) and num1DParticles (4318-4327): per q the
// sum over slices of 1 per included bead plus 2 cos(q . sep) per included
// pair i < j, sep = Path::getSeparation.  Returned divided by M only (the
// caller applies 1/num1D or 1/N); *n0 = num1DParticles.
void orc_ssf_cylinder(orc_sys* h, const double* q, int nq, double maxR, double* out, int* n0) {
    Sys* s = h->s;
    auto include = [&](const dVec& r) { return r[0] * r[0] + r[1] * r[1] < maxR * maxR; };
    int tot = 0;
    for (int p = 0; p < s->nbs[0]; ++p)
        if (include(s->P(0, p))) ++tot;
    *n0 = tot;
    for (int iq = 0; iq < nq; ++iq) {
        dVec qv{q[3*iq], q[3*iq+1], q[3*iq+2]};
        double sf = 0.0;
        for (int t = 0; t < s->M; ++t)
            for (int b1 = 0; b1 < s->nbs[t]; ++b1) {
                if (!include(s->P(t, b1))) continue;
                sf += 1.0;
                for (int b2 = b1 + 1; b2 < s->nbs[t]; ++b2)
                    if (include(s->P(t, b2))) sf += 2 * std::cos(dot(s->sep(t, b1, t, b2), qv));
            }
        out[iq] = sf * (1.0 / s->M);
    }
}

// EstimatorBase::getQVectors2 (estimator.cpp:762-824)
int orc_qvectors_shells(double dq, double qmax, int sphere, double* qv, int* shell, int cap) {
    const double kEps = 1.0e-7;
    int n = 0, ns = 0;
    for (double cq = 0.0; cq <= qmax + kEps; cq += dq, ++ns) {
        std::vector<dVec> v;
        if (std::abs(cq) < kEps) v.push_back(dVec{0.0, 0.0, 0.0});
        else {
            v.push_back(dVec{0.0, 0.0, cq});
            const int numTheta = 24;
            const double dtheta = sphere ? 0.5 * M_PI / numTheta : M_PI;
            for (double theta = dtheta; theta <= 0.5 * M_PI + kEps; theta += dtheta) {
                const double dphi = dtheta / std::sin(theta);
                for (double phi = 0.0; phi <= 0.5 * M_PI + kEps; phi += dphi)
                    v.push_back(dVec{cq * std::sin(theta) * std::cos(phi),
                                     cq * std::sin(theta) * std::sin(phi), cq * std::cos(theta)});
            }
        }
        for (const dVec& x : v) {
            if (n < cap) { qv[3*n] = x[0]; qv[3*n+1] = x[1]; qv[3*n+2] = x[2]; shell[n] = ns; }
            ++n;
        }
    }
    return n;
}

void orc_rhoq(orc_sys* h, const double* q, int nq, double* out) {
    Sys* s = h->s;
    for (int iq = 0; iq < nq; ++iq) {
        dVec qv{q[3*iq], q[3*iq+1], q[3*iq+2]};
        for (int t = 0; t < s->M; ++t) {
            double re = 0.0, im = 0.0;
            for (int p = 0; p < s->nbs[t]; ++p) {
                double ph = dot(qv, s->P(t, p));
                re += std::cos(ph); im += std::sin(ph);
            }
            out[((size_t)iq*s->M + t)*2] = re;
            out[((size_t)iq*s->M + t)*2 + 1] = im;
        }
    }
}

void orc_ssf_rhoq(orc_sys* h, const double* q, int nq, double* out) {
    Sys* s = h->s;
    int N = s->trueNumParticles();
    std::vector<double> rho((size_t)s->M * 2);
    for (int iq = 0; iq < nq; ++iq) {
        orc_rhoq(h, q + 3*iq, 1, rho.data());
        double acc = 0.0;
        for (int t = 0; t < s->M; ++t) acc += rho[2*t]*rho[2*t] + rho[2*t+1]*rho[2*t+1];
        out[iq] = acc / (1.0*N*s->M);
    }
}

// IntermediateScatteringFunctionEstimator::accumulate, estimator.cpp:3923-3961
void orc_isf_cpu_form(orc_sys* h, const double* q, int nq, double* out) {
    Sys* s = h->s;
    int N = s->trueNumParticles(), M = s->M;
    for (int i = 0; i < nq; ++i) {
        dVec qv{q[3*i], q[3*i+1], q[3*i+2]};
        for (int tau = 0; tau < M; ++tau) out[(size_t)i*M + tau] = 0.0;
        for (int t1 = 0; t1 < M; ++t1) {
            for (int ts = 0; ts < M; ++ts) {
                int t2 = (t1 + ts) % M;
                for (int b1 = 0; b1 < s->nbs[t1]; ++b1) {
                    double lq1 = dot(qv, s->P(t1, b1));
                    for (int b2 = 0; b2 < s->nbs[t2]; ++b2) {
                        double lq2 = dot(qv, s->P(t2, b2));
                        out[(size_t)i*M + ts] += (std::cos(lq1)*std::cos(lq2) + std::sin(lq1)*std::sin(lq2));
                    }
                }
            }
        }
        for (int tau = 0; tau < M; ++tau) out[(size_t)i*M + tau] = (out[(size_t)i*M + tau]/N) * (1.0/M);
    }
}

// gpu_isf<false> (src/estimator_gpu.cu:67-165) with the host norm of 0.5
// (estimator.cpp:4029): value = (1/(N M)) sum_{t,i,j} cos(q.(r_j(t+tau)-r_i(t)))
void orc_isf_gpu_form(orc_sys* h, const double* q, int nq, double* out) {
    Sys* s = h->s;
    int M = s->M, N = s->trueNumParticles();
    int nt = M/2 + 1;
    double inorm = 1.0/(1.0*N*M);
    for (int i = 0; i < nq; ++i) {
        for (int tau = 0; tau < nt; ++tau) {
            double acc = 0.0;
            for (int m1 = 0; m1 < M; ++m1) {
                int m2 = (m1 + tau) % M;
                for (int n1 = 0; n1 < N; ++n1) for (int n2 = 0; n2 < N; ++n2) {
                    dVec r1 = s->P(m1, n1), r2 = s->P(m2, n2);
                    double qs = 0.0;
                    for (int k = 0; k < 3; ++k) qs += q[3*i+k]*(r2[k] - r1[k]);
                    acc += std::cos(qs);
                }
            }
            out[(size_t)i*nt + tau] = 0.5*(2.0*acc*inorm);
        }
    }
}

void orc_isf_rhoq(orc_sys* h, const double* q, int nq, int nthreads, double* out) {
    Sys* s = h->s;
    int M = s->M, N = s->trueNumParticles();
    int nt = M/2 + 1;
    if (nthreads < 1) nthreads = 1;
    std::atomic<int> nextq(0);
    auto work = [&]() {
        std::vector<double> rho((size_t)M*2);
        for (;;) {
            int i = nextq.fetch_add(1);
            if (i >= nq) break;
            orc_rhoq(h, q + 3*i, 1, rho.data());
            for (int tau = 0; tau < nt; ++tau) {
                double acc = 0.0;
                for (int t = 0; t < M; ++t) {
                    int t2 = (t + tau) % M;
                    acc += rho[2*t]*rho[2*t2] + rho[2*t+1]*rho[2*t2+1];
                }
                out[(size_t)i*nt + tau] = acc / (1.0*N*M);
            }
        }
    };
    std::vector<std::thread> th;
    for (int k = 0; k < nthreads; ++k) th.emplace_back(work);
    for (auto& x : th) x.join();
}

orc_mt* orc_mt_create(uint32_t seed) { return new orc_mt(seed); }
void orc_mt_destroy(orc_mt* m) { delete m; }
uint32_t orc_mt_randint(orc_mt* m) { return m->m.randInt(); }
uint32_t orc_mt_randint_n(orc_mt* m, uint32_t n) { return m->m.randInt(n); }
double orc_mt_rand(orc_mt* m) { return m->m.rand(); }
double orc_mt_randexc(orc_mt* m) { return m->m.randExc(); }
double orc_mt_randnorm(orc_mt* m, double mean, double sd) { return m->m.randNorm(mean, sd); }
// MTRand::save / load (MersenneTwister.h): the 624 words, then `left`; the
// next word read is state[N - left]
void orc_mt_save(orc_mt* m, uint32_t* out625) {
    for (int i = 0; i < MT::N; ++i) out625[i] = m->m.st[i];
    out625[MT::N] = (uint32_t)m->m.left;
}
void orc_mt_load(orc_mt* m, const uint32_t* in625) {
    for (int i = 0; i < MT::N; ++i) m->m.st[i] = in625[i];
    m->m.left = (int)in625[MT::N];
    m->m.pos = MT::N - m->m.left;
}

int orc_run_steps(orc_sys* h, orc_mt* mt, const orc_move_params* mp, int nsteps,
                  int32_t* trace, int trace_cap, double* energies, orc_move_stats* stats) {
    return run_steps(h->s, &mt->m, mp, nsteps, trace, trace_cap, energies, stats);
}

}  // extern "C"

// Seeded closed worldlines (the benchmark inputs): particle i's centre
// uniform in the box, each bead jittered by N(0, 2 lambda tau) per coordinate
// and put back in the box, identity permutation, N beads on every slice.
static void seed_worldlines(Sys* s, MT& mt, int N) {
    const double sig = std::sqrt(2.0*s->lambda*s->tau);
    for (int i = 0; i < N; ++i) {
        dVec c;
        for (int d = 0; d < 3; ++d) c[d] = s->side[d]*(-0.5 + mt.randExc());
        for (int t = 0; t < s->M; ++t) {
            dVec r;
            for (int d = 0; d < 3; ++d) r[d] = mt.randNorm(c[d], sig);
            s->putInBC(r);
            s->setP(t, i, r);
            size_t k = ((size_t)t*s->Ne + i);
            s->on[k] = 1;
            s->nxt[2*k] = (t + 1) % s->M; s->nxt[2*k+1] = i;
            s->prv[2*k] = (t - 1 + s->M) % s->M; s->prv[2*k+1] = i;
        }
    }
    recount(s);
}

// setup.cpp:1079-1104 with the free-particle density estimate: Mbar from the
// interparticle spacing, even, at least 2, at most M/2 when it exceeds M
static int default_mbar(int N, double L, double lambda, double tau, int M) {
    double ell = std::pow(1.0*N/(L*L*L), -1.0/3.0);
    int mbar = int(ell*ell/(16*lambda*tau));
    if (mbar < 2) mbar = 2; else if (mbar > M) mbar = M/2;
    if (mbar % 2) mbar++;
    return mbar;
}

// Runs `work(w)` for w in order[0 .. W) on nthreads threads, each thread
// taking the next walker when it finishes one.  Returns wall seconds.
template <class F>
static double run_pool(const std::vector<int>& order, int nthreads, F&& work) {
    std::atomic<int> next(0);
    auto t0 = std::chrono::steady_clock::now();
    std::vector<std::thread> th;
    for (int k = 0; k < nthreads; ++k)
        th.emplace_back([&]() {
            for (;;) {
                int i = next.fetch_add(1);
                if (i >= (int)order.size()) break;
                work(order[i]);
            }
        });
    for (auto& x : th) x.join();
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

// Walkers in decreasing N^2 M (largest first keeps the pool's tail short).
static std::vector<int> largest_first(int W, const int* N, const int* M) {
    std::vector<int> order(W);
    for (int w = 0; w < W; ++w) order[w] = w;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        return 1.0*N[a]*N[a]*M[a] > 1.0*N[b]*N[b]*M[b];
    });
    return order;
}

extern "C" {

double orc_walkers_cpu(int W, const int* N, const int* M, const double* T,
                       const double* L, const uint32_t* seeds, double tau,
                       double lambda, int nequil, int nsteps, int nthreads,
                       double* mean_en, long long* bead_updates, double* setup_seconds) {
    if (nthreads < 1) nthreads = 1;
    std::vector<Sys*> sys(W, nullptr);
    std::vector<MT> mts;
    mts.reserve(W);
    for (int w = 0; w < W; ++w) mts.emplace_back(seeds[w]);
    std::vector<orc_move_params> mps(W);
    const std::vector<int> order = largest_first(W, N, M);
    // set-up, untimed: the system (tables shared), seeded worldlines and the
    // unsampled steps; PathIntegralMonteCarlo::step (pimc.cpp:724) is the
    // timed unit, as in the reference's own timing of a run
    const double t_setup = run_pool(order, nthreads, [&](int w) {
        orc_params p{};
        p.side[0] = p.side[1] = p.side[2] = L[w];
        p.num_slices = M[w]; p.num_ptcl_ext = N[w];
        p.tau = tau; p.lambda = lambda; p.rc = L[w];
        p.vfactor[0] = p.vfactor[1] = 1.0;
        p.gradvfactor[0] = p.gradvfactor[1] = 0.0;
        p.aziz_year = 1979; p.virial_window = 5; p.mu = 0.0;
        Sys* s = make_sys(&p);
        seed_worldlines(s, mts[w], N[w]);
        orc_move_params& mp = mps[w];
        mp = orc_move_params{};
        mp.mbar = default_mbar(N[w], L[w], lambda, tau, M[w]);
        mp.diagonal_move = 1; mp.var_updates = 1; mp.max_wind = 1;
        mp.temperature = T[w]; mp.p_com = 0.05; mp.num_updates = 0;
        orc_move_stats st{};
        if (nequil > 0) run_steps(s, &mts[w], &mp, nequil, nullptr, 0, nullptr, &st);
        sys[w] = s;
    });
    if (setup_seconds) *setup_seconds = t_setup;
    const double t_run = run_pool(order, nthreads, [&](int w) {
        std::vector<double> en(nsteps);
        orc_move_stats st{};
        run_steps(sys[w], &mts[w], &mps[w], nsteps, nullptr, 0, en.data(), &st);
        double acc = 0.0;
        for (double e : en) acc += e;
        if (mean_en) mean_en[w] = nsteps ? acc / nsteps : 0.0;
        if (bead_updates) bead_updates[w] = st.bead_updates;
    });
    for (Sys* s : sys) delete s;
    return t_run;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Adjacent path-wide estimators (the ranked-next rows of the hot-path table).
// ---------------------------------------------------------------------------
extern "C" {

// PairCorrelationEstimator (estimator.cpp:3181-3246) over the separation
// histogram that LocalAction::V(slice) fills (action.cpp:902-947 with
// ActionBase::updateSepHist, action.cpp:216-224): bins of
// dSep = 0.5 sqrt(3) L_z / NPCFSEP (action.cpp:192), pairs b1 < b2 of a
// slice, |r_b2 - r_b1| (minimum image).  V(slice) clears the histogram, so
// the reference's estimator sees the slice of the last V(slice) call;
// slice >= 0 reproduces that, slice < 0 sums every slice.  Output: one
// accumulate() increment already multiplied by the constructor's norm(n),
// i.e. g(r_n) of this sample.
void orc_pair_correlation(orc_sys* h, int slice, double* out50) {
    Sys* s = h->s;
    const int NPCF = 50;                       // NPCFSEP, include/common.h:85
    const double dSep = 0.5 * std::sqrt(3.0) * s->side[2] / (1.0 * NPCF);
    const double dR = 0.5 * std::sqrt(3.0) * s->side[2] / (1.0 * NPCF);   // periodic in all 3
    std::vector<long long> hist(NPCF, 0);
    const int t0 = slice >= 0 ? slice : 0, t1 = slice >= 0 ? slice + 1 : s->M;
    for (int t = t0; t < t1; ++t)
        for (int b1 = 0; b1 < s->nbs[t]; ++b1)
            for (int b2 = b1 + 1; b2 < s->nbs[t]; ++b2) {
                dVec d = s->sep(t, b2, t, b1);
                int nR = int(std::sqrt(dot(d, d)) / dSep);
                if (nR >= 0 && nR < NPCF) ++hist[nR];
            }
    const int N = s->trueNumParticles();
    double tot = 0.0;
    for (int n = 0; n < NPCF; ++n) tot += 1.0 * hist[n];
    const double lnorm = 1.0 * (N - 1) / (1.0 * N);
    const double volume = s->side[0] * s->side[1] * s->side[2];
    const double gNorm = 3.0 / (2.0 * M_PI);
    for (int n = 0; n < NPCF; ++n) {
        const double dV = std::pow((n + 1) * dR, 3.0) - std::pow(n * dR, 3.0);
        const double norm = 0.5 * (gNorm * volume) / dV;
        out50[n] = ((N > 1) && (tot > 0.0)) ? lnorm * (1.0 * hist[n] / tot) * norm : 0.0;
    }
}

// SuperfluidFractionEstimator::accumulate (estimator.cpp:2000-2074), one
// increment of its 26 columns: W^2/N, W_x^2, W_y^2, W_z^2 (W in box units),
// P(w) for w = -10..10 (|W_z/L - w| < 0.2), Az^2/I; the norms W2Norm =
// T/(2 * 3 * lambda) and ANorm = T M/(2 lambda) are left to the caller
// (estimator.cpp:1976-1980), as the reference applies them per bin.
void orc_superfluid(orc_sys* h, double* out26) {
    Sys* s = h->s;
    dVec W{0, 0, 0};
    double Az = 0.0, I = 0.0;
    for (int t = 0; t < s->M; ++t)
        for (int p = 0; p < s->nbs[t]; ++p) {
            dVec v = s->velocity(t, p);
            for (int d = 0; d < 3; ++d) W[d] += v[d];
            auto nx = s->next(t, p);
            if (nx[0] < 0) continue;                // no next bead: a worm end
            dVec p1 = s->P(t, p);
            dVec p2 = s->P(nx[0], nx[1]);
            Az += p1[0] * p2[1] - p2[0] * p1[1];
            I += p1[0] * p2[0] + p1[1] * p2[1];
        }
    for (int i = 0; i < 26; ++i) out26[i] = 0.0;
    const int N = s->trueNumParticles();
    if (N > 0) {
        out26[0] = dot(W, W) / (1.0 * N);
        out26[25] = Az * Az / I;
    }
    for (int d = 0; d < 3; ++d) W[d] *= s->sideInv[d];
    for (int d = 0; d < 3; ++d) out26[1 + d] = W[d] * W[d];
    int n = 0;
    for (int p = -10; p <= 10; ++p) {
        if (std::fabs(W[2] - 1.0 * p) < 0.2) out26[4 + n] = 1.0;
        ++n;
    }
}

// PermutationCycleEstimator::accumulate (estimator.cpp:2735-2781): every
// worldline through slice 0, counted once, adds cycleNum/N to the entry of
// its cycle length (up to 40).  Closed paths only.
void orc_permutation_cycles(orc_sys* h, double* out40) {
    Sys* s = h->s;
    for (int i = 0; i < 40; ++i) out40[i] = 0.0;
    const int N = s->trueNumParticles();
    const double cycleNorm = N > 0 ? 1.0 / (1.0 * N) : 0.0;
    const int nw = s->nbs[0];
    std::vector<char> doBead(nw, 1);
    for (int n = 0; n < nw; ++n) {
        if (!doBead[n]) continue;
        std::array<int,2> b{0, n};
        int wl = 0;
        do {
            ++wl;
            if (b[0] == 0 && b[1] < nw) doBead[b[1]] = 0;
            b = s->next(b[0], b[1]);
        } while (!(b[0] == 0 && b[1] == n) && wl <= s->M * s->Ne);
        const int cycleNum = wl / s->M;
        if (cycleNum > 0 && cycleNum <= 40) out40[cycleNum - 1] += 1.0 * cycleNum * cycleNorm;
    }
}

}  // extern "C"

// ---------------------------------------------------------------------------
// state-file text through std::ostream, the formatting the reference uses
// ---------------------------------------------------------------------------
namespace {
template <class Cell>
void stream_array2(std::ostream& os, int rows, int cols, Cell cell) {
    os << "(" << 0 << "," << rows - 1 << ") x (" << 0 << "," << cols - 1 << ")\n";
    os << "[ ";
    for (int i = 0; i < rows; ++i) {
        for (int j = 0; j < cols; ++j) { cell(os, i, j); os << " "; }
        if (i < rows - 1) os << "\n  ";
    }
    os << "]" << std::endl;
}
}  // namespace

extern "C" long orc_format_state(const double* pos, const int32_t* next, const int32_t* prev,
                                 const uint8_t* on, int M, int Ne, const long long* counts,
                                 int ncounts, const uint32_t* rng625, char* out, long cap) {
    std::ostringstream os;
    os << Ne << std::endl;
    char line[64];
    for (int k = 0; k < ncounts; ++k) {
        std::snprintf(line, sizeof line, "%16lld\t%16lld\n", counts[2 * k], counts[2 * k + 1]);
        os << line;
    }
    os << std::setprecision(16);
    stream_array2(os, M, Ne, [&](std::ostream& o, int i, int j) {
        const double* r = pos + ((size_t)i * Ne + j) * 3;
        o << "(" << r[0] << "," << r[1] << "," << r[2] << ")";
    });
    os << std::endl;
    stream_array2(os, M, Ne, [&](std::ostream& o, int i, int j) {
        const int32_t* l = next + ((size_t)i * Ne + j) * 2;
        o << "(" << l[0] << "," << l[1] << ")";
    });
    os << std::endl;
    stream_array2(os, M, Ne, [&](std::ostream& o, int i, int j) {
        const int32_t* l = prev + ((size_t)i * Ne + j) * 2;
        o << "(" << l[0] << "," << l[1] << ")";
    });
    os << std::endl;
    stream_array2(os, M, Ne, [&](std::ostream& o, int i, int j) {
        o << (unsigned int)on[(size_t)i * Ne + j];
    });
    os << std::endl;
    for (int i = 0; i < 625; ++i) os << rng625[i] << " ";
    os << std::endl;
    const std::string s = os.str();
    if (out && cap > (long)s.size()) { std::memcpy(out, s.data(), s.size()); out[s.size()] = 0; }
    return (long)s.size();
}

// ---------------------------------------------------------------------------
// Gaussian-process potential (CPU form of the reference)
// ---------------------------------------------------------------------------
namespace {
double orc_matern(double nu, double r) {
    const double kSqrt3 = 1.7320508075688772935, kSqrt5 = 2.2360679774997896964;
    if (std::abs(nu - 0.5) < 1.0e-12) return std::exp(-r);
    if (std::abs(nu - 1.5) < 1.0e-12) { const double x = kSqrt3 * r; return (1.0 + x) * std::exp(-x); }
    const double x = kSqrt5 * r;
    return (1.0 + x + x * x / 3.0) * std::exp(-x);
}

// GaussianProcessPotential::GP(const dVec&) (potential.cpp:330-344)
double orc_gp_one(const orc_gp_params* p, const double* tr, int n, const double* q) {
    dVec r, invell, pside, sideInv;
    for (int d = 0; d < 3; ++d) {
        r[d] = (q[d] - p->norm_offset[d]) / p->norm_scale[d];
        invell[d] = 1.0 / p->ell[d];
        pside[d] = p->periodic[d] ? p->side[d] : 0.0;
        sideInv[d] = 1.0 / p->side[d];
    }
    double kernelDot = 0.0;
    for (int k = 0; k < n; ++k) {
        // MaternKernel::K(r, trainX(k)): sep = trainX - r, putInBC, * 1/ell
        dVec sep;
        for (int d = 0; d < 3; ++d) sep[d] = tr[4 * (size_t)k + d] - r[d];
        for (int d = 0; d < 3; ++d) sep[d] -= pside[d] * std::floor(sep[d] * sideInv[d] + 0.5);
        for (int d = 0; d < 3; ++d) sep[d] = sep[d] * invell[d];
        double d2 = 0.0;
        for (int d = 0; d < 3; ++d) d2 += sep[d] * sep[d];
        kernelDot += orc_matern(p->matern_nu, std::sqrt(d2)) * tr[4 * (size_t)k + 3];
    }
    return p->standard_mean + p->standard_std * (p->mean + p->sigma2 * kernelDot);
}
}  // namespace

extern "C" void orc_gp_eval(const orc_gp_params* p, const double* training, int n,
                            const double* pos, int count, double* out) {
    for (int i = 0; i < count; ++i) out[i] = orc_gp_one(p, training, n, pos + 3 * (size_t)i);
}

// GPHeBenzenePotential::V(const dVec*, double*, int) and long_range
// (potential.cpp:5610-5681, include/potential.h:2433-2480)
extern "C" void orc_gp_benzene(const orc_gp_params* p, const double* training, int n,
                               const double* pos, int count, double* out) {
    const double r0 = 5.765366674e+00, gama = 1.671477473e+01;
    const double x1 = 2.290626821e+05, x2 = 4.069217828e+06, x3 = 9.542607077e+07, x4 = 0.0;
    const double x5 = -4.775615288e+04, x6 = -1.263899296e+07, x7 = -2.959330054e+08, x8 = 0.0;
    const double x9 = 9.511488779e+05, x10 = 2.551023972e+08, x11 = 0.0, x12 = 1.883887454e+08;
    auto rad2deg = [](double a) { return (a * 180.0) / M_PI; };
    auto deg2rad = [](double a) { return (a * M_PI) / 180.0; };
    for (int i = 0; i < count; ++i) {
        const double x = pos[3 * (size_t)i], y = pos[3 * (size_t)i + 1];
        double z = pos[3 * (size_t)i + 2];
        double finx = 0.0, finy = 0.0;
        if (z <= 0.0) z = -z;
        const double pi = M_PI;
        double angle = std::round(rad2deg(std::atan2(y, x)) * 10000.0) / 10000.0;
        if (angle < 0.0) angle = 180.0 + (180.0 + angle);
        if (angle <= 30.0) { finx = x; finy = y; }
        else {
            double rot = std::fmod(angle, 60.0) - angle;
            if ((angle + rot) > 30.0) {
                rot = deg2rad(rot);
                const double rx = std::cos(rot) * x - std::sin(rot) * y;
                const double ry = std::sin(rot) * x + std::cos(rot) * y;
                finx = std::cos(pi / 3.0) * rx + std::sin(pi / 3.0) * ry;
                finy = std::sin(pi / 3.0) * rx - std::cos(pi / 3.0) * ry;
            } else {
                rot = deg2rad(rot);
                finx = std::cos(rot) * x - std::sin(rot) * y;
                finy = std::sin(rot) * x + std::cos(rot) * y;
            }
        }
        const double rho = std::sqrt(finx * finx + finy * finy);
        if (rho < 3.0 && z < 2.0) { out[i] = 10000.0; continue; }
        const double q[3] = {finx, finy, z};
        const double gpv = orc_gp_one(p, training, n, q);
        double d2 = 0.0;
        d2 += finx * finx; d2 += finy * finy; d2 += z * z;
        const double rnorm = std::sqrt(d2);
        const double h_long = 1.0 / (1.0 + std::exp(-gama * (rnorm - r0)));
        double value;
        if (rho > 5.0 || z > 6.5) {
            const double ph0 = std::atan2(finy, finx), th0 = std::acos(z / rnorm);
            const double tt = std::cos(th0), fi = ph0;
            const double normm1 = std::sqrt(5.0) / 5.0, normm2 = std::sqrt(13.0) / 13.0;
            const double normm3 = 0.1792151994e-4;
            const double p1 = -x1 / std::pow(rnorm, 6) - x2 / std::pow(rnorm, 8) - x3 / std::pow(rnorm, 10) - x4 / std::pow(rnorm, 12);
            const double p2 = -normm1 * (1.5 * tt * tt - 0.5) *
                              (x5 / std::pow(rnorm, 6) + x6 / std::pow(rnorm, 8) + x7 / std::pow(rnorm, 10) + x8 / std::pow(rnorm, 12));
            const double p3 = -normm2 * (3.0 / 8.0 + 35.0 / 8.0 * std::pow(tt, 4) - 15.0 / 4.0 * tt * tt);
            const double p4 = (x9 / std::pow(rnorm, 8) + x10 / std::pow(rnorm, 10) + x11 / std::pow(rnorm, 12));
            const double p5 = -normm3 * 10395.0 * std::pow(1 - tt * tt, 3) * std::cos(6 * fi) * x12 / std::pow(rnorm, 10);
            value = (1.0 - h_long) * gpv + h_long * (p1 + p2 + p3 * p4 + p5);
        } else value = gpv;
        out[i] = value / 0.695;
    }
}

extern "C" int orc_run_worm_steps(orc_sys* h, orc_mt* mt, const orc_worm_params* wp, int nsteps,
                                  int32_t* trace, int trace_cap, double* energies,
                                  int* nparticles, orc_worm_stats* stats) {
    if (h->s->hash.size() != (size_t)h->s->M) reset_lookup(*h->s);
    return run_worm_steps(h->s, &mt->m, wp, nsteps, trace, trace_cap, energies, nparticles, stats);
}

// CPU baseline of the device worm walkers: W independent paths run by the
// worm engine above with the reference's default move list, each its own
// system (bead extent 2 N + 8 per slice, the walkers' capacity) and
// MT19937(seeds[w]).  Set-up (system, shared tables, seeded worldlines) and
// npre diagonal pre-equilibration steps and the first nequil steps are
// untimed; nsteps steps of every walker are timed (C0[w] the walker's worm
// constant, NULL for 1)
// on nthreads threads, walkers taken largest first.  Returns the timed wall
// seconds; fills per-walker bead updates of the timed steps, the mean E/N
// over the timed steps that ended diagonal (NaN if none) and the set-up
// seconds.  A walker whose slice outgrows its extent stops (bead_updates of
// the steps it made are kept) and is counted in *failed.
extern "C" double orc_worm_walkers_cpu(int W, const int* N, const int* M, const double* L,
                                       const int* mbar, const double* C0, const uint32_t* seeds,
                                       double tau, double lambda, int window, int diagonal_move, int npre, int nequil,
                                       int nsteps, int nthreads, double* mean_en,
                                       long long* bead_updates, double* setup_seconds, int* failed) {
    if (nthreads < 1) nthreads = 1;
    std::vector<Sys*> sys(W, nullptr);
    std::vector<MT> mts;
    mts.reserve(W);
    for (int w = 0; w < W; ++w) mts.emplace_back(seeds[w]);
    std::vector<orc_worm_params> wps(W);
    std::atomic<int> nfail(0);
    const std::vector<int> order = largest_first(W, N, M);
    const double t_setup = run_pool(order, nthreads, [&](int w) {
        orc_params p{};
        p.side[0] = p.side[1] = p.side[2] = L[w];
        p.num_slices = M[w]; p.num_ptcl_ext = 2 * N[w] + 8;
        p.tau = tau; p.lambda = lambda; p.rc = L[w];
        p.vfactor[0] = p.vfactor[1] = 1.0;
        p.gradvfactor[0] = p.gradvfactor[1] = 0.0;
        p.aziz_year = 1979; p.virial_window = 5; p.mu = 0.0;
        Sys* s = make_sys(&p);
        seed_worldlines(s, mts[w], N[w]);
        reset_lookup(*s);
        orc_worm_params& wp = wps[w];
        wp = orc_worm_params{};
        wp.mbar = mbar[w]; wp.diagonal_move = diagonal_move; wp.var_updates = 1; wp.max_wind = 1;
        wp.temperature = 1.0 / (M[w] * tau); wp.mu = 0.0; wp.worm_constant = C0 ? C0[w] : 1.0;
        wp.window = window; wp.gaussian_sd = 0.0; wp.num_updates = 0;
        wp.initial_num_particles = N[w];
        if (npre > 0) run_diag_steps(s, &mts[w], &wp, npre);
        if (nequil > 0 && run_worm_steps(s, &mts[w], &wp, nequil, nullptr, 0, nullptr, nullptr, nullptr) < 0) {
            ++nfail;
            delete s;
            s = nullptr;
        }
        sys[w] = s;
    });
    if (setup_seconds) *setup_seconds = t_setup;
    const double t_run = run_pool(order, nthreads, [&](int w) {
        if (bead_updates) bead_updates[w] = 0;
        if (mean_en) mean_en[w] = std::nan("");
        if (!sys[w]) return;
        std::vector<double> en(nsteps);
        orc_worm_stats st{};
        if (run_worm_steps(sys[w], &mts[w], &wps[w], nsteps, nullptr, 0, en.data(), nullptr, &st) < 0) ++nfail;
        double acc = 0.0;
        int cnt = 0;
        for (double e : en) if (e == e) { acc += e; ++cnt; }
        if (mean_en && cnt) mean_en[w] = acc / cnt;
        if (bead_updates) bead_updates[w] = st.bead_updates;
    });
    for (Sys* s : sys) delete s;
    if (failed) *failed = nfail.load();
    return t_run;
}

extern "C" void orc_get_path(orc_sys* h, int32_t* next, int32_t* prev, uint8_t* on, int32_t* worm8,
                             int32_t* nbs) {
    Sys* s = h->s;
    size_t nb = (size_t)s->M * s->Ne;
    for (size_t i = 0; i < nb * 2; ++i) { next[i] = s->nxt[i]; prev[i] = s->prv[i]; }
    std::memcpy(on, s->on.data(), nb);
    const int w[8] = {s->head[0], s->head[1], s->tail[0], s->tail[1], s->sp1[0], s->sp1[1], s->sp2[0], s->sp2[1]};
    for (int i = 0; i < 8; ++i) worm8[i] = w[i];
    for (int t = 0; t < s->M; ++t) nbs[t] = s->nbs[t];
}
