/*
 * pimc_gb300.h -- C ABI of the GB300-native WA-PIMC hot path.
 *
 * The library owns its device memory and one CUDA stream per context.  Every
 * entry point returns 0 on success or a negative PGB_E* code; the message of
 * the last failure is available from pgb_last_error().  No entry point aborts,
 * throws across the ABI or falls back to a CPU path: when the CUDA device or
 * the kernels are unavailable the call fails with PGB_ECUDA.
 *
 * Each group below names the reference interface it replaces (file:line in
 * the DelMaestroGroup/pimc tree).  Arrays follow the reference's own layouts:
 *   positions  AoS FP64 [M][Ne][3]     (Path::beads, include/path.h:164)
 *   links      int32   [M][Ne][2]      (Path::nextLink/prevLink, path.h:165)
 *   on flags   uint8   [M][Ne]         (Worm::beads, include/worm.h:153)
 *   beads      int32   [k][2]          (beadLocator = {slice, ptcl})
 *   worm       int32   [8]             head, tail, special1, special2
 * A context is used from one host thread at a time; calls on one context are
 * serialised on its stream and are synchronous from the caller's view unless
 * the name says "_async".
 */
#ifndef PIMC_GB300_H
#define PIMC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PGB_OK        0
#define PGB_EINVAL   -1   /* bad argument or size */
#define PGB_ECUDA    -2   /* CUDA runtime / launch failure or no device */
#define PGB_ENOMEM   -3   /* device allocation refused */
#define PGB_ESTATE   -4   /* call out of order (e.g. no path loaded) */
#define PGB_ETIMEOUT -5   /* a bounded device wait ran out */

/* precision of the pair sums */
#define PGB_FP64   0      /* plain form: FP64 direct-lookup Aziz tables */
#define PGB_MIXED  1      /* FP32 analytic Aziz pairs, FP64 accumulation */

/* modes of pgb_bead_actions */
#define PGB_ACTION_FULL 0 /* LocalAction::potentialAction(bead)     action.cpp:487 */
#define PGB_ACTION_BARE 1 /* LocalAction::barePotentialAction(bead) action.cpp:628 */
#define PGB_ACTION_CORR 2 /* LocalAction::potentialActionCorrection action.cpp:696 */

typedef struct pgb_ctx pgb_ctx;

/* Physical and numerical parameters of one path (constants.cpp:120-166,
 * setup.cpp:1216-1266, container.cpp:84-113). */
typedef struct {
    double side[3];         /* periodic box sides, A */
    int    num_slices;      /* M (the reference forces it even) */
    int    num_ptcl_ext;    /* Ne, bead-array extent per slice */
    double tau;             /* imaginary time step, 1/K */
    double lambda;          /* hbar^2/2m, K A^2 (24.24/mass) */
    double rc;              /* cutoff; LookupTable list uses |sep|^2 < rc^2 */
    double vfactor[2];      /* even/odd VFactor (primitive 1,1; gsf 2/3,4/3) */
    double gradvfactor[2];  /* even/odd gradVFactor (gsf 0,2/9) */
    int    period;          /* action period (1 primitive, 2 gsf) */
    int    aziz_year;       /* 1979 (HFDHE2), 1987 or 1995 */
    int    virial_window;   /* centroid virial window, reference default 5 */
    int    precision;       /* PGB_FP64 or PGB_MIXED */
    double mu;              /* chemical potential for E_mu columns */
} pgb_params;

/* ---- context: replaces the construction in pdrive.cpp:84-150 ---------- */
int         pgb_create(const pgb_params* p, pgb_ctx** out);
int         pgb_destroy(pgb_ctx* ctx);
const char* pgb_last_error(const pgb_ctx* ctx);   /* ctx may be NULL */
int         pgb_device_info(char* name, int cap, int* sm_count, int* cc);

/* ---- Aziz potential: AzizPotential (potential.h:933-1017,
 *      potential.cpp:1741-1907).  Tables are built on the device from the
 *      host-accumulated r_k = r_{k-1} + dr sequence (potential.h:176-183). -- */
int pgb_table_info(pgb_ctx* ctx, int* length, double* dr, double* tailV);
int pgb_copy_tables(pgb_ctx* ctx, double* V, double* dV, double* d2V);
/* PotentialBase::V(const dVec*, double*, int), potential.h:86 / potential.cpp:127:
 * batched V(sep) for n separation vectors (AoS [n][3]). */
int pgb_potential_batch(pgb_ctx* ctx, const double* sep, double* out, int n);
/* gradV (potential.h:997) and grad2V (potential.h:1010) batched */
int pgb_gradv_batch(pgb_ctx* ctx, const double* sep, double* out3, int n);
int pgb_grad2v_batch(pgb_ctx* ctx, const double* sep, double* out, int n);

/* ---- worldline state: Path/Worm/LookupTable updates (path.cpp:197-420,
 *      lookuptable.cpp:314-458).  The device mirror must follow every bead
 *      change the caller makes, as the reference mutates before it asks.
 *      worm8 may be NULL: no worm (all eight locators XXX = -1). -------- */
int pgb_load_path(pgb_ctx* ctx, const double* pos, const int32_t* next,
                  const int32_t* prev, const uint8_t* on, const int32_t* worm8);
int pgb_update_beads(pgb_ctx* ctx, const int32_t* beads, const double* pos, int k);
/* New positions for every bead (AoS FP64 [M][Ne][3]) with links, on flags and
 * worm unchanged: one host-to-device copy and an on-device transpose, as the
 * reference's GPU estimators copy Path::beads before each sample
 * (estimator.cpp:3846).  Asynchronous on the context stream; pos must stay
 * unchanged until the next synchronous call. */
int pgb_update_positions(pgb_ctx* ctx, const double* pos);
int pgb_get_positions(pgb_ctx* ctx, double* pos);
/* Mirror of Path::addBead / delBead / makeLink / breakLink / updateBead
 * (path.cpp:197-420): k full bead records (slice, ptcl), position, next and
 * prev links, active flag.  The active beads of every slice must stay packed
 * at its front, as the reference's left-packed arrays keep them
 * (PGB_ESTATE otherwise); numBeadsAtSlice follows. */
int pgb_set_beads(pgb_ctx* ctx, const int32_t* beads, const double* pos, const int32_t* next,
                  const int32_t* prev, const uint8_t* on, int k);
/* The worm locators head, tail, special1, special2 (Worm::head ... special2) */
int pgb_set_worm(pgb_ctx* ctx, const int32_t worm8[8]);
/* The host mirror of the links, active flags and worm locators */
int pgb_get_path(pgb_ctx* ctx, int32_t* next, int32_t* prev, uint8_t* on, int32_t worm8[8]);

/* ---- potential action: LocalAction (action.cpp:456-740) --------------
 * Per-bead U_b for k beads at imaginary-time shift `shift` (bisection level
 * spacing, ActionBase::setShift action.h:119).  out_per_bead may be NULL;
 * out_sum receives the sum over beads in list order (ActionBase list and
 * range forms, action.cpp:384-405, 572-620).  Inactive beads give 0. */
int pgb_bead_actions(pgb_ctx* ctx, const int32_t* beads, int k, int shift,
                     int mode, double* out_per_bead, double* out_sum);
/* Trial displacements: delta[i] = U_b(pos[i]) - U_b(current) for bead i alone
 * moved to pos[i] (AoS [k][3]); the trials are independent of one another.
 * This is the quantity of every single-bead Metropolis test
 * (potentialAction(bead) after minus before, action.cpp:487-514). */
int pgb_trial_actions(pgb_ctx* ctx, const int32_t* beads, const double* pos, int k,
                      int shift, int mode, double* out_delta);
/* the same on device buffers, asynchronous on the context stream; d_work
 * holds 2k doubles */
int pgb_trial_actions_device_async(pgb_ctx* ctx, const int32_t* d_beads, const double* d_pos,
                                   int k, int shift, int mode, double* d_delta, double* d_work);
/* potentialAction(startBead, endBead), action.cpp:522-570: follows next links */
int pgb_range_action(pgb_ctx* ctx, int s0, int p0, int s1, int p1, int shift,
                     double* out);
/* potentialAction() over the whole path, action.cpp:456-472 */
int pgb_full_action(pgb_ctx* ctx, double* out);
/* kineticAction(), action.cpp:345-369 */
int pgb_kinetic_action(pgb_ctx* ctx, double* out);

/* Per-slice sums behind the estimator-facing ActionBase virtuals
 * (action.cpp:751-806, 902-947, 1188-1223, 1446-1803).  Arrays of length M:
 *  vint[t]  sum_{i<j} factor V(r_j - r_i)              (V(slice)[1])
 *  g2[t]    sum_i |sum_{j!=i} gradV(r_i - r_j)|^2      (gradVSquared(slice))
 *  r1[t]    sum_i gradV_i . r_i                        (rDOTgradUterm1 / (VF tau))
 *  r2[t]    sum_i (T_i gradV_i) . r_i                  (rDOTgradUterm2 / (2 gF tau^3 lambda))
 *  d1[t]    sum_i gradV_i . delta_i                    (deltaDOTgradUterm1 / (VF tau))
 *  d2[t]    sum_i (T_i gradV_i) . delta_i              (deltaDOTgradUterm2 / (...))
 *  kin[t]   sum_i |r_{t+1} - r_t|^2 on the next link    (getVelocity, path.h:189)
 *  xch[t]   sum_i (r_{t+W} - r_t) . (r_{t+1} - r_t)      (virial T2 term)
 * Any pointer may be NULL.  r2/d2 need the T-matrix and are computed only
 * when non-NULL. */
typedef struct {
    double *vint, *g2, *r1, *r2, *d1, *d2, *kin, *xch;
} pgb_slice_terms;
int pgb_slice_terms_compute(pgb_ctx* ctx, pgb_slice_terms* out);

/* ---- estimators (estimator.cpp:917-1252, 3661-4236) -------------------
 * One accumulate() of EnergyEstimator: K, V, V_ext, V_int, E, E_mu, K/N,
 * V/N, E/N (estimator.cpp:940-1029). */
int pgb_energy(pgb_ctx* ctx, double out9[9]);
/* One accumulate() of VirialEnergyEstimator, 19 columns
 * (estimator.cpp:1086-1252).  cvcov2_quirk = 1 keeps the reference's
 * misspelt "cVCov2" key, which adds totEcv*beta*dEdB into column 0. */
int pgb_virial(pgb_ctx* ctx, int cvcov2_quirk, double out19[19]);
/* EstimatorBase::getQVectors (estimator.cpp:439-570).  Returns the number
 * of q-vectors through *count; fills at most cap of them into q[3*i]. */
int pgb_qvectors(const char* type, const char* input, const double side[3],
                 double* q, int cap, int* count);
/* S(q): StaticStructureFactor(GPU)Estimator::accumulate
 * (estimator.cpp:3705-3737, 3824-3861), per-sample value already divided by
 * N M (the reference's norm 1/M applied), via rho_q. */
int pgb_ssf(pgb_ctx* ctx, const double* q, int nq, double* out);
/* Cylinder S(q): the beads inside x^2 + y^2 < maxR^2 only (include(),
 * estimator.cpp:4309-4311).  out[k] = (1/M) sum_t sum_{i,j inside}
 * cos(q_k . (r_j(t) - r_i(t))) -- what the cylinder GPU estimator's kernel
 * (gpu_ssf_cyl, estimator_gpu.cu:169-285) is meant to sum, with its sum
 * accumulated across the loop and its radius test the right way round -- and
 * *num_inside0 = num1DParticles (estimator.cpp:4318-4327).  The CPU
 * estimator's sample is out / num_inside0 per shell vector
 * (estimator.cpp:5415-5458), the GPU estimator's out / N.  nq = 0 (q and
 * out may be NULL) only counts. */
int pgb_ssf_cylinder(pgb_ctx* ctx, const double* q, int nq, double maxR, double* out,
                     int* num_inside0);
/* EstimatorBase::getQVectors2 (estimator.cpp:762-824): the shell q-vectors
 * of magnitudes 0, dq, 2dq, ... <= qmax; sphere = 0 is the "line" geometry
 * (one vector along z per shell), 1 the octant grid.  shell[i] is the
 * vector's shell index.  *count = total; at most cap are written. */
int pgb_qvectors_shells(double dq, double qmax, int sphere, double* q, int* shell, int cap,
                        int* count);
/* F(q,tau): IntermediateScatteringFunctionEstimatorGpu::accumulate
 * (estimator.cpp:4063-4100, gpu_isf estimator_gpu.cu:67-165): layout
 * [q][M/2+1], value (1/(N M)) sum_{t,i,j} cos(q.(r_j(t+tau) - r_i(t))).
 * mode 0: CUDA-core correlation; mode 1: tensor-core (tcgen05, split-BF16)
 * DFT correlation.  PGB_FP64 contexts always use the FP64 direct form.
 * Every wait of the tensor-core pipeline is bounded (about a second); one
 * that runs out makes the call return PGB_ETIMEOUT, the context usable. */
int pgb_isf(pgb_ctx* ctx, const double* q, int nq, int mode, double* out);
/* Test of the bounded waits (no counterpart in the reference): with on != 0
 * the first tensor-core GEMM of every later pgb_isf (mode 1, PGB_MIXED)
 * stops issuing before its last K chunk, so a wait runs out and the call
 * returns PGB_ETIMEOUT; on = 0 restores normal operation.  Process-wide. */
void pgb_test_isf_tc_stall(int on);
/* The adjacent path-wide estimators, one accumulate() each (FP64):
 * g(r): PairCorrelationEstimator (estimator.cpp:3181-3246), 50 bins of
 *   0.5 sqrt(3) L_z / 50, the sample already times the estimator's norm;
 *   slice >= 0 takes that slice's separation histogram, as the reference's
 *   LocalAction::V(slice) leaves it (action.cpp:902-947), slice < 0 all of
 *   them.
 * superfluid: SuperfluidFractionEstimator (estimator.cpp:2000-2074), 26
 *   columns W^2/N, W_x^2, W_y^2, W_z^2, P(-10..10), Az^2/I; the per-bin norms
 *   T/(6 lambda) and T M/(2 lambda) are the caller's, as in the reference.
 * permutation cycles: PermutationCycleEstimator (estimator.cpp:2735-2781), 40
 *   columns; PGB_ESTATE if a worldline through slice 0 does not close. */
int pgb_pair_correlation(pgb_ctx* ctx, int slice, double out50[50]);
int pgb_superfluid(pgb_ctx* ctx, double out26[26]);
int pgb_permutation_cycles(pgb_ctx* ctx, double out40[40]);
/* rho_q(t) of the loaded path, layout [q][M][2] (FP64 values) */
int pgb_rhoq(pgb_ctx* ctx, const double* q, int nq, double* out);

/* ---- device-resident variants for timing: inputs already in device
 *      memory, results left on the device (no host copies, no syncs; the
 *      tensor-core pipeline's timeout word is checked by pgb_isf only). ---- */
int pgb_isf_device_async(pgb_ctx* ctx, const double* d_q, int nq, int mode,
                         double* d_out);
int pgb_ssf_device_async(pgb_ctx* ctx, const double* d_q, int nq, double* d_out);
int pgb_load_positions_device_async(pgb_ctx* ctx, const double* d_pos);
void* pgb_stream(pgb_ctx* ctx);   /* the context's cudaStream_t */

/* F(q,tau) that allocates nothing, for callers that cannot call cudaMalloc
 * when they measure (their device memory is reserved up front by a pool they
 * do not own, or they may only launch work once set-up is over).  No
 * counterpart in the reference.  The caller passes device buffers: d_beads,
 * AoS FP64 [num_slices][ptcl_extent][3] of which the first num_ptcl beads per
 * slice are used; d_qvecs [nq][3]; d_isf [nq][num_slices/2+1], the same values
 * as pgb_isf mode 0 on a PGB_MIXED context.  The densities rho_q(t) go to a
 * static 16 MiB device array held by every GPU that loads the library, so
 * nq * num_slices must not exceed 2^21, num_slices 25600 and num_ptcl 6400
 * (PGB_EINVAL otherwise, with the limit in the message).  Work is queued on
 * `stream` (a cudaStream_t, NULL for the default stream) and the call returns
 * without waiting.  The first call on a device looks up the array's device
 * address with that device current and caches it; make that first call
 * before any stream capture, and do not call the entry point on a device
 * after cudaDeviceReset (the cached address is then stale).  Calls share the
 * array: calls that overlap on the GPU race, so order them.  Errors are
 * reported by pgb_last_error(NULL). */
int pgb_isf_static(const double* d_beads, int num_slices, int num_ptcl,
                   int ptcl_extent, const double side[3], const double* d_qvecs,
                   int nq, double* d_isf, void* stream);

/* ---- batched walkers: many independent canonical chains in one
 *      persistent kernel (no reference counterpart; replaces running many
 *      pimc.e processes with offset seeds, setup.cpp:921-923). ---------- */
typedef struct pgb_walkers pgb_walkers;
typedef struct {
    int           num_walkers;
    const int*    num_ptcl;     /* N_w */
    const int*    num_slices;   /* M_w (even) */
    const double* temperature;  /* T_w = 1/(M_w tau) */
    const double* side;         /* cube side L_w */
    const int*    mbar;         /* staging length Mbar_w (even, >= 2) */
    double        tau, lambda;
    double        p_com;        /* centre-of-mass move probability */
    uint64_t      seed;         /* Philox key; walker w uses stream w */
    int           aziz_year;
    int           threads_per_walker; /* schedule (pgb_walkers_threads); 0: autotune */
    int           var_updates;  /* 1: stage length 2 + U{0..Mbar-2} */
} pgb_walkers_params;

typedef struct {
    double    energy_sum;      /* sum of E/N samples */
    double    energy_sumsq;
    long long samples;
    long long bead_updates;
    long long attempted[2];    /* com, staging */
    long long accepted[2];
} pgb_walker_stats;

int pgb_walkers_create(const pgb_walkers_params* p, pgb_walkers** out);
int pgb_walkers_destroy(pgb_walkers* w);
/* Initialise worldlines on the device (uniform + N(0, 2 lambda tau) jitter,
 * identity permutation) from the Philox streams. */
int pgb_walkers_init(pgb_walkers* w);
/* Upload one walker's positions (AoS FP64 [M][N][3]) */
int pgb_walkers_set_positions(pgb_walkers* w, int walker, const double* pos);
int pgb_walkers_get_positions(pgb_walkers* w, int walker, double* pos);
/* Upload every walker's positions at once from one host buffer: walker w's
 * AoS FP64 [M_w][N_w][3] block follows walker w-1's (total sum M_w N_w 3
 * doubles).  Pinned host memory gives the full C2C copy bandwidth.  The copy
 * runs on a second stream into one of two staging buffers, so it overlaps
 * work already queued (the previous sweep); the new state takes effect in
 * stream order.  The host buffer must stay unchanged until the next
 * synchronizing call (pgb_walkers_sync, pgb_walkers_stats). */
int pgb_walkers_set_all_positions(pgb_walkers* w, const double* pos);
/* every walker's positions into one host buffer (the layout of
 * pgb_walkers_set_all_positions; the device FP32 values, exact in FP64) */
int pgb_walkers_get_all_positions(pgb_walkers* w, double* pos);
/* sweeps made per walker: with the positions, all a walker's chain needs to
 * resume exactly (its draws are indexed by walker, sweep and move) */
int pgb_walkers_get_sweeps(pgb_walkers* w, unsigned long long* sweeps);
int pgb_walkers_set_sweeps(pgb_walkers* w, const unsigned long long* sweeps);
/* bytes of the host buffer pgb_walkers_set_all_positions reads */
size_t pgb_walkers_state_bytes(pgb_walkers* w);
/* Run `sweeps` MC steps for every walker (numUpdates moves per step,
 * pimc.cpp:62-65, then one energy sample), asynchronously on the stream. */
int pgb_walkers_run_async(pgb_walkers* w, int sweeps, int measure);
/* waits for the stream; PGB_ETIMEOUT if a walker's bounded device wait ran
 * out (the walker's chain stopped; its state is left as it was) */
int pgb_walkers_sync(pgb_walkers* w);
int pgb_walkers_stats(pgb_walkers* w, pgb_walker_stats* per_walker);
int pgb_walkers_reset_stats(pgb_walkers* w);
/* launches of walker kernels issued so far */
long long pgb_walkers_launch_count(pgb_walkers* w);
/* schedule chosen by the autotuner (or set): 64/128/256 = one CTA of that
 * size per walker; 1004/1008/1016 (2004/2008/2016) = walkers packed as thread
 * teams of 1-8 warps into 256-thread CTAs sized for 4/8/16 pair evaluations
 * per thread per move, 3 (2) CTAs per SM; 3003 (3002) = one warp per
 * imaginary-time window, up to min(8, M/(Mbar+1)) concurrent staging moves
 * per walker on disjoint windows, 3 (2) CTAs per SM; 4004/4008/4016 = packed
 * teams whose slab rows are staged in shared memory by bulk copies;
 * 5008/5016 (6008/6016) = the same with the next move's rows prefetched into
 * a second buffer, 256 (512)-thread CTAs, teams of up to 8 (16) warps;
 * 5000 (6000) = the same with team warps proportional to each walker's cost
 * N^2 M, the costliest walker getting all 8 (16); 7000/7008/7016 = teams
 * sized as 6000/6008/6016 that split into sub-teams to make a run of up to
 * two (8000/8008/8016: four) consecutive staging moves at once when their
 * imaginary-time intervals are pairwise disjoint (such moves commute, so the
 * chain is that of making them in turn) */
int pgb_walkers_threads(pgb_walkers* w);
/* the autotuner's record: schedules tried and one-sweep time (ms) of each;
 * returns the number of candidates, fills at most cap */
int pgb_walkers_tuning(pgb_walkers* w, int* scheds, float* ms, int cap);
/* Energy per particle (thermodynamic estimator, primitive action) of each
 * walker's current configuration, FP64 pair sums (plain form) or mixed. */
int pgb_walkers_energy(pgb_walkers* w, int precision, double* en_per_walker);
void* pgb_walkers_stream(pgb_walkers* w);
const char* pgb_walkers_last_error(const pgb_walkers* w);

/* ---- serving: continuous batching of simulation jobs (no reference
 *      counterpart; replaces queueing independent pimc.e runs).  Jobs are
 *      canonical chains of the batched-walker engine (staging + centre-of-mass
 *      moves, energy sampled every sweep); mu is carried for the E_mu column
 *      only. ------------------------------------------------------------- */
typedef struct pgb_server pgb_server;
typedef struct {
    double hbm_budget_bytes;   /* device memory for worldline slabs */
    int    max_active;         /* jobs on the device at once */
    int    sweeps_per_round;   /* sweeps per round of a 64-particle, 125-slice job;
                                  a job of cost N^2 M makes this times 64^2 125/(N^2 M),
                                  at least 1 and at most sweeps_per_round */
    int    bin_sweeps;         /* sweeps per estimator bin (the last bin holds the remainder) */
    double tau, lambda;
    double p_com;
    int    aziz_year;
    double round_seconds;      /* > 0: every job runs for this much device time per round,
                                  stopping and resuming between moves (sweeps_per_round
                                  then unused); 0: sweeps_per_round as above */
    int    diagonal_move;      /* worm server: 0 bisection (the reference's default),
                                  1 staging; unused by the canonical server */
} pgb_server_params;
typedef struct {
    int       n;               /* particles N0 */
    double    temperature;     /* K; M = even round(1/(T tau)) */
    double    mu;              /* chemical potential (reported, canonical run) */
    double    density;         /* initial box: L = (n/density)^(1/3) */
    long long sweeps;          /* Monte Carlo steps to run */
    uint64_t  seed;            /* the job's own random streams */
    double    arrival;         /* server-clock seconds at which the job arrives */
} pgb_job_spec;
typedef struct {
    int       job, bin;
    double    energy_per_particle;  /* mean E/N over the bin */
    long long samples;
    double    time;            /* server clock when the bin became available */
} pgb_bin;
typedef struct {
    int       state;           /* 0 submitted, 1 queued, 2 on the device, 3 done,
                                  4 stopped by a walker error (worm server: the job's
                                  bead capacity 2 n + 8 per slice ran out) */
    double    arrival, admitted, first_bin, completed;  /* -1 when not yet */
    long long sweeps_done;
    int       n, m;
    size_t    bytes;           /* device footprint of the worldline slab */
} pgb_job_info;

int         pgb_server_create(const pgb_server_params* p, pgb_server** out);
int         pgb_server_destroy(pgb_server* s);
int         pgb_server_submit(pgb_server* s, const pgb_job_spec* job, int* job_id);
/* one round: admit arrived jobs that fit, advance every active job, emit bins,
 * retire finished jobs */
int         pgb_server_step(pgb_server* s, int* n_active, int* n_queued);
int         pgb_server_poll_bins(pgb_server* s, pgb_bin* out, int cap, int* n);
int         pgb_server_job_info(pgb_server* s, int job, pgb_job_info* out);
double      pgb_server_clock(pgb_server* s);
long long   pgb_server_bead_updates(pgb_server* s);   /* of retired jobs */
int         pgb_server_active_bead_updates(pgb_server* s, long long* total);
const char* pgb_server_last_error(const pgb_server* s);

/* ---- plain form: the reference move loop driven from the host with one
 *      FP64 device action call per move (move.cpp:1124-1707 semantics,
 *      MT19937 stream as include/MersenneTwister.h). --------------------- */
typedef struct {
    int    mbar;
    int    diagonal_move;   /* 0 bisection, 1 staging */
    int    var_updates;
    int    max_wind;
    double temperature;
    double p_com;
    int    num_updates;     /* <= 0: max(100, ceil(N M / Mbar)) */
} pgb_move_params;

typedef struct {
    long long attempted[3]; /* com, staging, bisection */
    long long accepted[3];
    long long bead_updates;
} pgb_move_stats;

/* Seed the context's MT19937 stream (MTRand(seed), MersenneTwister.h:170-206) */
int pgb_plain_seed(pgb_ctx* ctx, uint32_t seed);
/* The stream's state in MTRand::save layout (MersenneTwister.h:125-126): 624
 * state words then `left`; the state file's generator line
 * (pimc.cpp:966-971).  Setting it resumes the stream exactly. */
int pgb_plain_get_rng(pgb_ctx* ctx, uint32_t out625[625]);
int pgb_plain_set_rng(pgb_ctx* ctx, const uint32_t in625[625]);
/* Run nsteps PathIntegralMonteCarlo::step() loops (pimc.cpp:724-741) of
 * centre-of-mass + diagonal moves on the loaded closed path, continuing the
 * context's MT19937 stream.  trace (optional) receives (move, accepted) int32
 * pairs of attempted moves (0 com, 1 staging, 2 bisection); energies
 * (optional) receives E/N of each step's EnergyEstimator sample. */
int pgb_plain_run(pgb_ctx* ctx, const pgb_move_params* mp, int nsteps,
                  int32_t* trace, int trace_cap, int* trace_len,
                  double* energies, pgb_move_stats* stats);

/* The worm algorithm in the plain form: PathIntegralMonteCarlo::step() over
 * the reference's default PIMC move list (com, diagonal, open, close, insert,
 * remove, advance head, recede head, advance tail, recede tail, swap head,
 * swap tail; setup.cpp:466-470) with its attempt probabilities
 * (constants.cpp:191-205) and diagonal/off-diagonal selection
 * (pimc.cpp:120-208).  Moves run on the host in the reference's order of
 * random numbers; every action is an FP64 device evaluation on the device
 * mirror, which each path change updates (pgb_set_beads' path).  The worm
 * state and the LookupTable order persist across calls until the next
 * pgb_load_path.  Needs rc > L/2 (one LookupTable grid box, from which the
 * swap moves draw their pivot) and a bead-array extent Ne with room for the
 * particle-number fluctuations (PGB_ENOMEM when a slice outgrows it; the
 * reference grows its arrays instead).
 * trace: (move index in the list above, accepted) per attempted move;
 * energies[step]: E/N, NaN when the step ends off-diagonal;
 * nparticles[step]: active beads / M. */
typedef struct {
    int    mbar, diagonal_move, var_updates, max_wind;
    double temperature, mu;
    double worm_constant;          /* C0 (worm_constant, default 1) */
    int    window;                 /* canonical particle window half-width, -1 none */
    double gaussian_sd;            /* canonical Gaussian weight width, <= 0 none */
    int    num_updates;            /* <= 0: ceil(max(N0,1) M / Mbar), at least 100 */
    int    initial_num_particles;  /* N0 */
} pgb_worm_params;
typedef struct {
    long long attempted[12];
    long long accepted[12];
    long long bead_updates;
    int diagonal;                  /* 1 when the run ended on a closed configuration */
} pgb_worm_stats;
int pgb_plain_worm_run(pgb_ctx* ctx, const pgb_worm_params* wp, int nsteps, int32_t* trace,
                       int trace_cap, int* trace_len, double* energies, int* nparticles,
                       pgb_worm_stats* stats);

/* ---- Device-resident worm walkers -----------------------------------------
 * Independent worm-algorithm paths (grand canonical, or canonical with a
 * particle window), one warp per walker below N0 = 32 and a team of two
 * (N0 < 64) or four warps above, advanced by whole PIMC steps on the
 * device: the reference's default move list with its attempt probabilities
 * (the same moves as pgb_plain_worm_run), primitive action, FP32 Aziz pairs
 * reduced in double-float, a Philox stream per walker.  They agree with the
 * plain form and the oracle statistically, not draw for draw.  Walker w has
 * num_ptcl[w] initial particles, num_slices[w] (even) slices of width tau,
 * box side side[w], chemical potential mu[w] (NULL: 0), update length
 * mbar[w] (even, <= 64) and room for capacity[w] beads per slice.
 * The swap moves draw their pivot from the pivot slice's beads in index
 * order (the reference uses its LookupTable order: the same distribution). */
typedef struct pgb_worm_walkers pgb_worm_walkers;
typedef struct {
    int           num_walkers;
    const int*    num_ptcl;
    const int*    num_slices;
    const double* side;
    const double* mu;
    const int*    mbar;
    const int*    capacity;
    double        tau, lambda;
    double        worm_constant;   /* C0 */
    int           window;          /* canonical window half-width, -1 none */
    uint64_t      seed;
    int           aziz_year;       /* 1979 (default) */
    int           diagonal_move;   /* 0 bisection (the reference's default), 1 staging */
    const double* worm_constants;  /* per-walker C0; NULL: worm_constant for every walker */
} pgb_worm_walkers_params;
typedef struct {
    double    energy_sum, energy_sumsq;   /* E/N of the closed configurations */
    double    n_sum, n_sumsq;             /* particle number of the same samples */
    long long samples;                    /* steps that ended closed */
    long long attempted[12];              /* the move list of pgb_plain_worm_run */
    long long accepted[12];
    long long bead_updates;
    long long sweeps;                     /* PIMC steps made */
    int       error;                      /* 1 slice full, 2 bad link, 3 runaway walk */
    int       pad;
} pgb_worm_walker_stats;
int pgb_worm_walkers_create(const pgb_worm_walkers_params* p, pgb_worm_walkers** out);
int pgb_worm_walkers_destroy(pgb_worm_walkers* w);
const char* pgb_worm_walkers_last_error(const pgb_worm_walkers* w);
/* closed worldlines on the identity permutation from positions [M][N][3] */
int pgb_worm_walkers_load(pgb_worm_walkers* w, int walker, const double* pos);
/* advance every walker by `sweeps` PIMC steps (synchronous) */
int pgb_worm_walkers_run(pgb_worm_walkers* w, int sweeps);
/* the same queued on the walkers' stream, returning without waiting */
int pgb_worm_walkers_run_async(pgb_worm_walkers* w, int sweeps);
/* diagonal pre-equilibration (after PathIntegralMonteCarlo::equilStepDiagonal,
 * pimc.cpp:216-300): `sweeps` steps of centre-of-mass (probability 0.05) and
 * staging moves only, no worm moves, no energy samples; synchronous */
int pgb_worm_walkers_equilibrate(pgb_worm_walkers* w, int sweeps);
int pgb_worm_walkers_synchronize(pgb_worm_walkers* w);
void* pgb_worm_walkers_stream(pgb_worm_walkers* w);   /* the cudaStream_t */
long long pgb_worm_walkers_launch_count(pgb_worm_walkers* w);
/* every walker from seeded closed worldlines made on the device: particle
 * i's centre uniform in the box, each bead jittered by N(0, 2 lambda tau) per
 * coordinate, identity links, N beads per slice; the statistics cleared */
int pgb_worm_walkers_seed(pgb_worm_walkers* w, uint64_t seed);
/* The whole device state as one host image of pgb_worm_walkers_state_bytes
 * bytes (positions, links, bead counts, worm records), for checkpoints and
 * for callers that keep the worldlines on the host between steps.  get waits
 * for the copy; set_async queues it on the walkers' stream (the image must
 * stay valid until the stream reaches it; pinned memory for full speed). */
long long pgb_worm_walkers_state_bytes(pgb_worm_walkers* w);
int pgb_worm_walkers_get_state(pgb_worm_walkers* w, void* image);
int pgb_worm_walkers_set_state_async(pgb_worm_walkers* w, const void* image);
/* statistics copy queued on the walkers' stream (synchronize before reading) */
int pgb_worm_walkers_stats_async(pgb_worm_walkers* w, pgb_worm_walker_stats* per_walker);
/* LocalAction::barePotentialAction (action.cpp:628-645, primitive action) of
 * beads [k][2] (slice, particle) of walker `walker`'s current path, computed
 * by the walkers' own FP32 pair sums, for checking them against FP64 */
int pgb_worm_walkers_bead_actions(pgb_worm_walkers* w, int walker, const int32_t* beads, int k,
                                  double* out);
int pgb_worm_walkers_stats(pgb_worm_walkers* w, pgb_worm_walker_stats* per_walker);
int pgb_worm_walkers_reset_stats(pgb_worm_walkers* w);
/* one walker's arrays in the layouts of pgb_load_path ([M][capacity]) */
int pgb_worm_walkers_get_path(pgb_worm_walkers* w, int walker, double* pos, int32_t* next,
                              int32_t* prev, uint8_t* on, int32_t worm8[8]);
/* Self-check of the walkers' random streams: from the stream of `seed`
 * advanced by `skip` words, `count` (<= 192) normal deviates drawn one at a
 * time (serial[]) and made by the 32 lanes together (parallel[]), and the
 * stream position after each (state[0..2] serial counter low, high, word
 * index; state[3..5] the same after the parallel form).  The two agree bit
 * for bit. */
int pgb_worm_normals_check(uint64_t seed, int skip, int count, float* serial, float* parallel,
                           int32_t state[6]);

/* Grand-canonical job server: pgb_server_*'s interface and semantics (the
 * same parameter, job, bin and job-info records) with every job a device worm
 * walker at its own chemical potential mu (worm constant C0 = 1, no window).
 * A job's bins depend only on its spec: the same alone and in any mix. */
typedef struct pgb_worm_server pgb_worm_server;
int         pgb_worm_server_create(const pgb_server_params* p, pgb_worm_server** out);
int         pgb_worm_server_destroy(pgb_worm_server* s);
int         pgb_worm_server_submit(pgb_worm_server* s, const pgb_job_spec* job, int* job_id);
int         pgb_worm_server_step(pgb_worm_server* s, int* n_active, int* n_queued);
int         pgb_worm_server_poll_bins(pgb_worm_server* s, pgb_bin* out, int cap, int* n);
int         pgb_worm_server_job_info(pgb_worm_server* s, int job, pgb_job_info* out);
double      pgb_worm_server_clock(pgb_worm_server* s);
int         pgb_worm_server_active_bead_updates(pgb_worm_server* s, long long* total);
const char* pgb_worm_server_last_error(const pgb_worm_server* s);

/* ---- Gaussian-process external potential ----------------------------------
 * GaussianProcessPotential (include/potential.h:287-323, src/potential.cpp:
 * 244-392) with the Matern kernel (include/gpkernel.h:48-72): the fields are
 * the reference's gp parameter keys (kernel.maternNu, kernel.ell,
 * data.normOffset, data.normScale, data.standardMean, data.standardStd,
 * kernel.mean, kernel.sigma2) plus the container (sides, periodic flags),
 * whose boundary conditions the CPU kernel applies to each separation.
 * Training rows are x, y, z, (K^-1 Y): the first four doubles of each row of
 * the reference's binary training file. */
typedef struct pgb_gp pgb_gp;
typedef struct {
    double matern_nu;          /* 0.5, 1.5 or 2.5 */
    double ell[3];
    double norm_offset[3];
    double norm_scale[3];
    double standard_mean, standard_std;
    double mean;               /* kernel.mean (mu) */
    double sigma2;
    double side[3];
    int    periodic[3];
    int    precision;          /* PGB_FP64: the CPU form bit for bit up to exp();
                                  PGB_MIXED: FP32 kernel values, compensated sum */
} pgb_gp_params;
int pgb_gp_create(const pgb_gp_params* p, const double* training /* [n][4] */, int n,
                  pgb_gp** out);
int pgb_gp_destroy(pgb_gp* gp);
const char* pgb_gp_last_error(const pgb_gp* gp);   /* gp may be NULL */
void* pgb_gp_stream(pgb_gp* gp);
/* GaussianProcessPotential::GP(const dVec*, double*, int), positions AoS */
int pgb_gp_eval(pgb_gp* gp, const double* pos, double* values, int count);
int pgb_gp_eval_device_async(pgb_gp* gp, const double* d_pos, double* d_values, int count);
/* GPHeBenzenePotential::V(const dVec*, double*, int) (src/potential.cpp:
 * 5610-5681): symmetry fold, hard core 10000 K, GP, long-range switch */
int pgb_gp_benzene_v(pgb_gp* gp, const double* pos, double* values, int count);

#ifdef __cplusplus
}
#endif
#endif
