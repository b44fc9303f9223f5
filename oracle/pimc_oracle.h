/*
 * pimc_oracle.h -- C interface of the FP64 CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GB300 hot
 * path: it restates, in plain C++ and FP64, the reference WA-PIMC CPU code
 * for the pair action (Aziz table, LookupTable cutoff semantics, LocalAction),
 * the path-wide estimators (thermodynamic / virial energy, S(q), F(q,tau)),
 * the MT19937 generator and the diagonal moves (centre of mass, staging,
 * bisection).  Only tests/, __graft_entry__.smoke() and the CPU-baseline legs
 * of bench.py load it.  The product library (pimc_gb300) never links it.
 *
 * Parity status: the reference cannot be built in this image (it needs Boost
 * and <mdspan>), and it ships no golden vectors, so this restatement is
 * "parity unpinned": it is checked against the reference's own invariants
 * (batched-vs-scalar potential check, checkMove full-vs-local action
 * identity, pairwise-vs-rho_q structure factors) rather than against outputs
 * of the reference binary.
 *
 * Conventions: beads are addressed as (slice, ptcl); positions are AoS FP64
 * [M][Ne][3]; links are [M][Ne][2] int32 (slice, ptcl), -1 for "no link";
 * worm locators are int32[8] = head, tail, special1, special2.
 */
#ifndef PIMC_ORACLE_H
#define PIMC_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_sys orc_sys;

typedef struct {
    double side[3];        /* box sides (periodic prism) */
    int    num_slices;     /* M */
    int    num_ptcl_ext;   /* Ne, array extent */
    double tau;            /* imaginary time step */
    double lambda;         /* hbar^2/2m in K A^2 */
    double rc;             /* interaction cutoff (reference default: box side) */
    double vfactor[2];     /* even/odd potential factors */
    double gradvfactor[2]; /* even/odd |grad V|^2 factors */
    int    aziz_year;      /* 1979, 1987 or 1995 */
    int    virial_window;  /* centroid virial window (reference default 5) */
    double mu;             /* chemical potential (for E_mu columns) */
} orc_params;

/* ---- Aziz potential (src/potential.cpp:1741-1907) ---- */
void   orc_aziz_values(int year, double r, double out3[3]);

/* ---- system ---- */
orc_sys* orc_create(const orc_params* p);
void     orc_destroy(orc_sys* s);
int      orc_table_length(orc_sys* s);
double   orc_table_dr(orc_sys* s);
double   orc_tailV(orc_sys* s);
void     orc_copy_tables(orc_sys* s, double* V, double* dV, double* d2V);
double   orc_V(orc_sys* s, const double sep[3]);
void     orc_gradV(orc_sys* s, const double sep[3], double out[3]);
double   orc_grad2V(orc_sys* s, const double sep[3]);
void     orc_load_path(orc_sys* s, const double* pos, const int32_t* next,
                       const int32_t* prev, const uint8_t* on,
                       const int32_t* worm8);
void     orc_get_positions(orc_sys* s, double* pos);
void     orc_update_bead(orc_sys* s, int slice, int ptcl, const double pos[3]);
void     orc_set_shift(orc_sys* s, int shift);

/* ---- action (src/action.cpp) ---- */
double orc_potential_action_bead(orc_sys* s, int slice, int ptcl);
double orc_bare_potential_action(orc_sys* s, int slice, int ptcl);
double orc_potential_action_correction(orc_sys* s, int slice, int ptcl);
double orc_potential_action_range(orc_sys* s, int s0, int p0, int s1, int p1);
double orc_potential_action_list(orc_sys* s, const int32_t* beads, int k);
double orc_potential_action_full(orc_sys* s);
double orc_kinetic_action_full(orc_sys* s);
double orc_Vnn(orc_sys* s, int slice, int ptcl);
double orc_gradVnnSquared(orc_sys* s, int slice, int ptcl);
void   orc_V_slice(orc_sys* s, int slice, double out2[2]);
double orc_gradVSquared_slice(orc_sys* s, int slice);
double orc_gradVSquared_bead(orc_sys* s, int slice, int ptcl);
double orc_deriv_tau(orc_sys* s, int slice);
double orc_deriv_lambda(orc_sys* s, int slice);
double orc_second_deriv_tau(orc_sys* s, int slice);
double orc_rdotgradU1(orc_sys* s, int slice);
double orc_rdotgradU2(orc_sys* s, int slice);
double orc_deltadotgradU1(orc_sys* s, int slice);
double orc_deltadotgradU2(orc_sys* s, int slice);
double orc_virial_kin_corr(orc_sys* s, int slice);

/* ---- estimators (src/estimator.cpp) ---- */
/* one accumulate() of EnergyEstimator: K,V,V_ext,V_int,E,E_mu,K/N,V/N,E/N */
void orc_energy(orc_sys* s, double out9[9]);
/* one accumulate() of VirialEnergyEstimator (19 columns); cvcov2_quirk=1
 * reproduces the reference's misspelt "cVCov2" key (adds into column 0). */
void orc_virial(orc_sys* s, int cvcov2_quirk, double out19[19]);
/* q-vector list (EstimatorBase::getQVectors); returns count, fills up to cap */
int  orc_qvectors(const char* type, const char* input, const double side[3],
                  double* q, int cap);
/* g(r): one PairCorrelationEstimator sample (50 bins) times its norm; slice
 * >= 0 uses that slice's histogram (the reference's V(slice) side effect),
 * slice < 0 every slice */
void orc_pair_correlation(orc_sys* s, int slice, double* out50);
/* one SuperfluidFractionEstimator increment (26 columns, norms not applied) */
void orc_superfluid(orc_sys* s, double* out26);
/* one PermutationCycleEstimator increment (40 columns) */
void orc_permutation_cycles(orc_sys* s, double* out40);
/* The state-file text of PathIntegralMonteCarlo::saveState's text branch
 * (pimc.cpp:923-1000) written with C++ iostreams as the reference does:
 * counts as "%16d\t%16d" lines (ncounts pairs, the first being the totals),
 * then beads at setprecision(16), nextLink, prevLink, worm beads in the
 * DynamicArray stream format (common.h:245-274) and 625 generator words.
 * Returns the text length; the text is copied to out when cap allows. */
long orc_format_state(const double* pos, const int32_t* next, const int32_t* prev,
                      const uint8_t* on, int M, int Ne, const long long* counts, int ncounts,
                      const uint32_t* rng625, char* out, long cap);
/* S(q) pairwise CPU form, per-sample value already normalised by 1/(N M) */
void orc_ssf_pairwise(orc_sys* s, const double* q, int nq, double* out);
/* S(q) by rho_q in FP64 */
void orc_ssf_rhoq(orc_sys* s, const double* q, int nq, double* out);
/* F(q,tau): reference CPU form, tau in [0,M), layout [q][M] */
void orc_isf_cpu_form(orc_sys* s, const double* q, int nq, double* out);
/* F(q,tau): reference GPU form (raw q.(r_j - r_i) sum), tau in [0,M/2], layout [q][M/2+1] */
void orc_isf_gpu_form(orc_sys* s, const double* q, int nq, double* out);
/* F(q,tau) by rho_q in FP64, tau in [0,M/2], layout [q][M/2+1]; nthreads>=1 */
void orc_isf_rhoq(orc_sys* s, const double* q, int nq, int nthreads, double* out);
/* cylinder S(q) (CylinderStaticStructureFactorEstimator), sum over slices / M
 * of the included beads' pair cosines; *n0 = num1DParticles */
void orc_ssf_cylinder(orc_sys* s, const double* q, int nq, double maxR, double* out, int* n0);
/* getQVectors2 shells; returns the count, fills at most cap */
int orc_qvectors_shells(double dq, double qmax, int sphere, double* q, int* shell, int cap);
/* Gaussian-process potential: GaussianProcessPotential::GP with
 * MaternKernel::K (potential.cpp:330-344, gpkernel.cpp:97-108), and
 * GPHeBenzenePotential::V batch (potential.cpp:5610-5681) */
typedef struct {
    double matern_nu, ell[3], norm_offset[3], norm_scale[3];
    double standard_mean, standard_std, mean, sigma2, side[3];
    int periodic[3];
} orc_gp_params;
void orc_gp_eval(const orc_gp_params* p, const double* training, int n, const double* pos,
                 int count, double* out);
void orc_gp_benzene(const orc_gp_params* p, const double* training, int n, const double* pos,
                    int count, double* out);
/* rho_q(t) FP64, layout [q][M][2] */
void orc_rhoq(orc_sys* s, const double* q, int nq, double* out);

/* ---- MT19937 (include/MersenneTwister.h) ---- */
typedef struct orc_mt orc_mt;
orc_mt*  orc_mt_create(uint32_t seed);
void     orc_mt_destroy(orc_mt* m);
uint32_t orc_mt_randint(orc_mt* m);
uint32_t orc_mt_randint_n(orc_mt* m, uint32_t n);
double   orc_mt_rand(orc_mt* m);
double   orc_mt_randexc(orc_mt* m);
double   orc_mt_randnorm(orc_mt* m, double mean, double sd);
void     orc_mt_save(orc_mt* m, uint32_t* out625);          /* MTRand::save layout */
void     orc_mt_load(orc_mt* m, const uint32_t* in625);

/* ---- diagonal moves + driver (src/move.cpp, src/pimc.cpp) ---- */
typedef struct {
    int    mbar;          /* update length Mbar (even) */
    int    diagonal_move; /* 0 = bisection, 1 = staging */
    int    var_updates;   /* reference default: 1 (see constants.cpp:96) */
    int    max_wind;      /* winding sectors sampled by staging, default 1 */
    double temperature;   /* for comDelta = 0.04 * lambda_dB */
    double p_com;         /* probability of a centre-of-mass move */
    int    num_updates;   /* moves per step; <=0 -> max(100, ceil(N M / Mbar)) */
} orc_move_params;

typedef struct {
    long long attempted[3];   /* com, staging, bisection */
    long long accepted[3];
    long long bead_updates;   /* beads proposed and Metropolis-tested */
} orc_move_stats;

/* Run nsteps MC steps on the loaded path using MT19937(seed-state owned by
 * mt).  If trace != NULL, each attempted move appends (move, accepted) pairs
 * as int32 [2] up to trace_cap entries; returns number of trace entries.
 * energies (may be NULL) receives E/N of each step's energy sample. */
int orc_run_steps(orc_sys* s, orc_mt* mt, const orc_move_params* mp, int nsteps,
                  int32_t* trace, int trace_cap, double* energies,
                  orc_move_stats* stats);

/* The worm-algorithm step driver over the reference's default PIMC move list
 * (com, diagonal, open, close, insert, remove, advance head, recede head,
 * advance tail, recede tail, swap head, swap tail; setup.cpp:466-470) with its
 * attempt probabilities (constants.cpp:191-205).  Trace entries are (move
 * index in that list, accepted) for every attempted move; energies[step] is
 * E/N of the step's sample or NaN when the step ends off-diagonal;
 * nparticles[step] = active beads / M.  Returns the trace length, -2 when a
 * slice outgrows the bead-array extent Ne, -3 on a broken worm. */
typedef struct {
    int    mbar, diagonal_move, var_updates, max_wind;
    double temperature, mu, worm_constant;   /* C0 */
    int    window;                           /* canonical window half-width, -1 none */
    double gaussian_sd;                      /* canonical Gaussian weight, <= 0 none */
    int    num_updates;                      /* <= 0: the reference's default */
    int    initial_num_particles;            /* N0 */
} orc_worm_params;
typedef struct {
    long long attempted[12];
    long long accepted[12];
    long long bead_updates;
    int diagonal;
} orc_worm_stats;
int orc_run_worm_steps(orc_sys* s, orc_mt* mt, const orc_worm_params* wp, int nsteps,
                       int32_t* trace, int trace_cap, double* energies, int* nparticles,
                       orc_worm_stats* stats);
/* links [M][Ne][2], on [M][Ne], worm locators [8], numBeadsAtSlice [M] */
void orc_get_path(orc_sys* s, int32_t* next, int32_t* prev, uint8_t* on, int32_t* worm8, int32_t* nbs);

/* CPU baseline: run W independent canonical walkers (each its own system,
 * MT19937 seed seeds[w]) for nsteps each, on nthreads threads.  Each walker
 * w has N[w] particles, M[w] slices, temperature T[w], box side L[w];
 * initial worldlines are generated by the oracle's lattice-free generator
 * from the same seed.  Set-up and the first nequil steps are untimed
 * (*setup_seconds receives their wall time); the nsteps sampled steps of
 * every walker are timed, walkers taken largest first by the threads.
 * Returns the timed wall seconds; fills per-walker mean E/N over the nsteps
 * sampled steps and the bead-update counts of the sampled steps. */
double orc_walkers_cpu(int W, const int* N, const int* M, const double* T,
                       const double* L, const uint32_t* seeds, double tau,
                       double lambda, int nequil, int nsteps, int nthreads,
                       double* mean_en, long long* bead_updates, double* setup_seconds);
/* The same for the worm engine (orc_run_worm_steps' move list), bead extent
 * 2 N + 8 per slice, canonical window `window` (-1: grand canonical at
 * mu = 0), diagonal_move 1 staging / 0 bisection.  mean_en[w] averages the
 * timed steps that end diagonal (NaN if none); *failed counts walkers that
 * outgrew their extent.  C0[w] is walker w's worm constant (NULL: 1).  npre
 * diagonal pre-equilibration steps (centre of mass with probability 0.05,
 * else staging) come first, untimed. */
double orc_worm_walkers_cpu(int W, const int* N, const int* M, const double* L,
                            const int* mbar, const double* C0, const uint32_t* seeds, double tau,
                            double lambda, int window, int diagonal_move, int npre, int nequil,
                            int nsteps, int nthreads, double* mean_en,
                            long long* bead_updates, double* setup_seconds, int* failed);

#ifdef __cplusplus
}
#endif
#endif
