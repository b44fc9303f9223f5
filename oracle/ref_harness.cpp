// ref_harness.cpp -- test infrastructure: a C ABI over the reference's own
// sources, compiled unchanged from the reference tree by oracle/Makefile.ref
// into oracle/_ref/libpimc_ref.so.  It builds one reference system the way
// the reference's driver does (src/pdrive.cpp:60-170: constants, Prism,
// LookupTable, Aziz and free potentials, Path, ConstantWaveFunction,
// LocalAction, the default PIMC move list, PathIntegralMonteCarlo) from a
// parameter record instead of a command line, loads worldline positions, and
// exposes the calls the oracle restates: potential values, per-bead and
// full-path actions, the energy, virial, S(q) and F(q,tau) estimators'
// accumulate(), and PathIntegralMonteCarlo::step() with the per-move counts
// and the resulting path.  Only the tests and the fixture scripts load it:
// it pins the oracle to the reference, nothing in the product uses it.
//
// One system at a time: the reference keeps its parameters in a process-wide
// singleton (constants()).
#include "common.h"
#include "constants.h"
#include "container.h"
#include "lookuptable.h"
#include "path.h"
#include "potential.h"
#include "wavefunction.h"
#include "action.h"
#include "move.h"
#include "estimator.h"
#include "pimc.h"
#include "MersenneTwister.h"

#include <cstdint>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

namespace {

// read access to an estimator's accumulators; acc() is one
// EstimatorBase::sample() (frequency 1: it accumulates when the path is
// closed and, in the canonical ensemble, holds N0 particles)
template <class E>
struct Open : E {
    using E::E;
    bool acc() { this->sample(); return this->getNumAccumulated() > 0; }
    double value(int k) const { return this->estimator(k); }
    double normf(int k) const { return this->norm(k); }
    int count() const { return this->numEst; }
};

// the table length of the Aziz lookup tables (a protected member)
struct OpenAziz : AzizPotential {
    using AzizPotential::AzizPotential;
    int length() const { return tableLength; }
};

struct RefSys {
    Prism* box = nullptr;
    LookupTable* lookup = nullptr;
    OpenAziz* aziz = nullptr;
    FreePotential* ext = nullptr;
    ConstantWaveFunction* wf = nullptr;
    LocalAction* action = nullptr;
    MTRand* random = nullptr;
    boost::ptr_vector<Path> paths;
    boost::ptr_vector<move_vector> moves;
    boost::ptr_vector<estimator_vector> estimators;
    PathIntegralMonteCarlo* pimc = nullptr;
    Path* path = nullptr;
    int M = 0, N = 0;
    ~RefSys() {
        delete pimc;
        moves.clear();
        estimators.clear();
        delete action;
        delete wf;
        paths.clear();
        delete aziz;
        delete ext;
        delete lookup;
        delete box;
        delete random;
    }
};

std::string g_err;

}  // namespace

extern "C" {

typedef struct {
    double side, temperature, lambda, rc, mu, worm_constant;
    int num_slices, num_ptcl, mbar;
    int window;          // canonical window half-width (-1: none)
    int canonical;       // 1: canonical ensemble (--canonical)
    int gsf;             // 1: GSF action, 0: primitive
    int staging;         // 1: staging replaces bisection as the diagonal move
    int virial_window;
    int aziz_year;
    uint32_t seed;       // MTRand seed
    const char* wavevector;       // q list for S(q)/F(q,tau), NULL for none
    const char* wavevector_type;  // "int", "float", "max_int", "max_float", ...
} ref_params;

const char* ref_last_error() { return g_err.c_str(); }

// pos: [M][N][3], the first N beads of every slice on closed identity worldlines
void* ref_create(const ref_params* p, const double* pos) {
    try {
        const double L = p->side;
        po::variables_map vm;
        vm.set("label", std::string("ref"));
        vm.set("start_with_state", std::string(""));
        if (p->canonical) vm.set("canonical", true);
        if (p->window >= 0) vm.set("window", p->window);
        vm.set("max_winding", 1);
        vm.set("update_length", p->mbar);
        vm.set("number_time_slices", p->num_slices);
        vm.set("temperature", p->temperature);
        vm.set("imaginary_time_length", 1.0 / p->temperature);
        vm.set("chemical_potential", p->mu);
        vm.set("mass", 24.24 / p->lambda);
        vm.set("potential_cutoff", p->rc);
        vm.set("worm_constant", p->worm_constant);
        vm.set("carbon_carbon_dist", 1.42);
        vm.set("volume", L * L * L);
        vm.set("side", dVec{L, L, L});
        vm.set("number_eq_steps", (uint32)1);
        vm.set("bin_size", (uint32)100);
        vm.set("graphenelut3d_file_prefix", std::string(""));
        vm.set("virial_window", p->virial_window > 0 ? p->virial_window : 5);
        vm.set("number_particles", p->num_ptcl);
        vm.set("number_broken", 0);
        vm.set("end_factor", 1.0);
        vm.set("number_paths", 1);
        vm.set("action", std::string(p->gsf ? "gsf" : "primitive"));
        if (p->wavevector && p->wavevector_type) {
            vm.set("wavevector", std::string(p->wavevector));
            vm.set("wavevector_type", std::string(p->wavevector_type));
        }
        constants()->initConstants(vm);

        auto* s = new RefSys();
        s->M = p->num_slices;
        s->N = p->num_ptcl;
        s->random = new MTRand(p->seed);
        s->box = new Prism(dVec{L, L, L});
        s->lookup = new LookupTable(s->box, s->M, s->N);
        s->aziz = new OpenAziz(p->aziz_year ? p->aziz_year : 1979, s->box);
        s->ext = new FreePotential();
        DynamicArray<dVec, 1> initialPos(s->N);
        for (int i = 0; i < s->N; ++i)
            initialPos(i) = dVec{pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
        s->paths.push_back(new Path(s->box, *s->lookup, s->M, initialPos, 0));
        s->path = &s->paths.front();
        for (int t = 0; t < s->M; ++t)
            for (int i = 0; i < s->N; ++i) {
                const double* r = pos + ((size_t)t * s->N + i) * 3;
                s->path->updateBead(beadLocator{t, i}, dVec{r[0], r[1], r[2]});
            }
        s->wf = new ConstantWaveFunction(*s->path, *s->lookup);
        // Setup::action (setup.cpp:1216-1266)
        std::array<double, 2> VF{1.0, 1.0}, gF{0.0, 0.0};
        int period = 1;
        if (p->gsf) { VF = {2.0 / 3.0, 4.0 / 3.0}; gF = {0.0, 2.0 / 9.0}; period = 2; }
        s->action = new LocalAction(*s->path, *s->lookup, s->ext, s->aziz, s->wf, VF, gF, true,
                                    p->gsf ? "gsf" : "primitive", 1.0, period);
        // the default PIMC move list (setup.cpp:467-471), in that order
        auto* mv = new move_vector();
        Path& path = *s->path;
        mv->push_back(new CenterOfMassMove(path, s->action, *s->random));
        if (p->staging) mv->push_back(new StagingMove(path, s->action, *s->random));
        else mv->push_back(new BisectionMove(path, s->action, *s->random));
        mv->push_back(new OpenMove(path, s->action, *s->random));
        mv->push_back(new CloseMove(path, s->action, *s->random));
        mv->push_back(new InsertMove(path, s->action, *s->random));
        mv->push_back(new RemoveMove(path, s->action, *s->random));
        mv->push_back(new AdvanceHeadMove(path, s->action, *s->random));
        mv->push_back(new RecedeHeadMove(path, s->action, *s->random));
        mv->push_back(new AdvanceTailMove(path, s->action, *s->random));
        mv->push_back(new RecedeTailMove(path, s->action, *s->random));
        mv->push_back(new SwapHeadMove(path, s->action, *s->random));
        mv->push_back(new SwapTailMove(path, s->action, *s->random));
        s->moves.push_back(mv);
        s->estimators.push_back(new estimator_vector());
        s->pimc = new PathIntegralMonteCarlo(s->paths, *s->random, s->moves, s->estimators, false);
        return s;
    } catch (const std::exception& e) {
        g_err = e.what();
        return nullptr;
    }
}

void ref_destroy(void* h) { delete static_cast<RefSys*>(h); }

int ref_table_length(void* h) { return static_cast<RefSys*>(h)->aziz->length(); }
double ref_tail_v(void* h) { return static_cast<RefSys*>(h)->aziz->tailV; }
// AzizPotential::V / gradV / grad2V (potential.h:985-1017) at separations sep[n][3]
void ref_potential(void* h, const double* sep, int n, double* V, double* gradV, double* grad2V) {
    auto* s = static_cast<RefSys*>(h);
    for (int k = 0; k < n; ++k) {
        const dVec r{sep[3 * k], sep[3 * k + 1], sep[3 * k + 2]};
        if (V) V[k] = s->aziz->V(r);
        if (gradV) { const dVec g = s->aziz->gradV(r); for (int d = 0; d < 3; ++d) gradV[3 * k + d] = g[d]; }
        if (grad2V) grad2V[k] = s->aziz->grad2V(r);
    }
}
void ref_set_shift(void* h, int shift) { static_cast<RefSys*>(h)->action->setShift(shift); }
double ref_potential_action_bead(void* h, int t, int p) {
    return static_cast<RefSys*>(h)->action->potentialAction(beadLocator{t, p});
}
double ref_bare_potential_action(void* h, int t, int p) {
    return static_cast<RefSys*>(h)->action->barePotentialAction(beadLocator{t, p});
}
double ref_potential_action_correction(void* h, int t, int p) {
    return static_cast<RefSys*>(h)->action->potentialActionCorrection(beadLocator{t, p});
}
double ref_potential_action_full(void* h) { return static_cast<RefSys*>(h)->action->potentialAction(); }
double ref_kinetic_action(void* h) { return static_cast<RefSys*>(h)->action->kineticAction(); }
// move one bead (Path::updateBead, path.cpp:197-200)
void ref_update_bead(void* h, int t, int p, const double* r) {
    static_cast<RefSys*>(h)->path->updateBead(beadLocator{t, p}, dVec{r[0], r[1], r[2]});
}

// one sample of an estimator on the current (closed) path: out[k] =
// estimator(k) * norm(k), the row output() would write after one sample.
// kind: 0 energy (9 columns), 1 virial (19), 2 S(q) (num_q), 3 F(q,tau)
// (num_q * M).  Returns the number of columns, or -1.
int ref_estimator(void* h, int kind, double* out, int cap) {
    auto* s = static_cast<RefSys*>(h);
    const double maxR = 0.5 * s->box->side[NDIM - 1];
    try {
        auto run = [&](auto& e) {
            if (!e.acc()) { g_err = "the estimator did not sample this configuration"; return -1; }
            const int n = e.count();
            for (int k = 0; k < n && k < cap; ++k) out[k] = e.value(k) * e.normf(k);
            return n;
        };
        switch (kind) {
            case 0: { Open<EnergyEstimator> e(*s->path, s->action, *s->random, maxR); return run(e); }
            case 1: { Open<VirialEnergyEstimator> e(*s->path, s->action, *s->random, maxR); return run(e); }
            case 2: { Open<StaticStructureFactorEstimator> e(*s->path, s->action, *s->random, maxR); return run(e); }
            case 3: { Open<IntermediateScatteringFunctionEstimator> e(*s->path, s->action, *s->random, maxR); return run(e); }
        }
    } catch (const std::exception& e) {
        g_err = e.what();
    }
    return -1;
}

// PathIntegralMonteCarlo::step (pimc.cpp:724-786) nsteps times; returns the
// number of steps that ended with a closed (diagonal) configuration
int ref_run_steps(void* h, int nsteps, double* energies) {
    auto* s = static_cast<RefSys*>(h);
    int closed = 0;
    for (int k = 0; k < nsteps; ++k) {
        s->pimc->step();
        const bool diag = s->path->worm.isConfigDiagonal;
        closed += diag ? 1 : 0;
        if (energies) {
            if (diag) {
                Open<EnergyEstimator> e(*s->path, s->action, *s->random, 0.5 * s->box->side[NDIM - 1]);
                energies[k] = e.acc() ? e.value(8) * e.normf(8) : std::nan("");
            } else {
                energies[k] = std::nan("");
            }
        }
    }
    return closed;
}

// per-move attempted/accepted counts in the move-list order
void ref_move_stats(void* h, long long* attempted, long long* accepted) {
    auto* s = static_cast<RefSys*>(h);
    int k = 0;
    for (auto& m : s->moves.front()) {
        attempted[k] = m.getNumAttempted();
        accepted[k] = m.getNumAccepted();
        ++k;
    }
}

// the bead-array extent (grows as worm moves add beads)
int ref_extent(void* h) { return static_cast<RefSys*>(h)->path->getNumParticles(); }

// positions [M][ne][3], links [M][ne][2], active flags [M][ne], worm
// locators head, tail, special1, special2 [8], beads per slice [M]
void ref_get_path(void* h, int ne, double* pos, int32_t* next, int32_t* prev, uint8_t* on,
                  int32_t* worm8, int32_t* nbs) {
    auto* s = static_cast<RefSys*>(h);
    Path& P = *s->path;
    const int ext = P.getNumParticles();
    for (int t = 0; t < s->M; ++t) {
        nbs[t] = P.numBeadsAtSlice(t);
        for (int q = 0; q < ne; ++q) {
            const size_t j = (size_t)t * ne + q;
            if (q < ext) {
                const beadLocator b{t, q};
                const dVec r = P(t, q);
                const beadLocator n = P.next(b), pv = P.prev(b);
                for (int d = 0; d < 3; ++d) pos[3 * j + d] = r[d];
                next[2 * j] = n[0]; next[2 * j + 1] = n[1];
                prev[2 * j] = pv[0]; prev[2 * j + 1] = pv[1];
                on[j] = P.worm.beadOn(b) ? 1 : 0;
            } else {
                for (int d = 0; d < 3; ++d) pos[3 * j + d] = 0.0;
                next[2 * j] = next[2 * j + 1] = prev[2 * j] = prev[2 * j + 1] = XXX;
                on[j] = 0;
            }
        }
    }
    const beadLocator w[4] = {P.worm.head, P.worm.tail, P.worm.special1, P.worm.special2};
    for (int i = 0; i < 4; ++i) { worm8[2 * i] = w[i][0]; worm8[2 * i + 1] = w[i][1]; }
}

// the generator's state in MTRand::save's layout (625 words)
void ref_rng_state(void* h, uint32_t* out625) {
    auto* s = static_cast<RefSys*>(h);
    MTRand::uint32 buf[MTRand::SAVE];
    s->random->save(buf);
    for (int i = 0; i < MTRand::SAVE; ++i) out625[i] = buf[i];
}

}  // extern "C"
