/*
 * pimc_gb300.hpp -- header-only C++ mirror of the reference's plugin classes
 * for the pair action and the path-wide estimators, over the C ABI of
 * pimc_gb300.h.
 *
 * Each class keeps the reference's member names, argument meanings and return
 * values so that a caller written against the reference reads the same:
 *
 *   pgb::AzizPotential   PotentialBase / AzizPotential   include/potential.h:83-109, 933-1017
 *   pgb::Path            the device mirror of Path + Worm  include/path.h:150-200
 *   pgb::LocalAction     ActionBase / LocalAction          include/action.h:30-254
 *   pgb::EnergyEstimator, pgb::VirialEnergyEstimator,
 *   pgb::StaticStructureFactorEstimator,
 *   pgb::IntermediateScatteringFunctionEstimator
 *                        EstimatorBase and its subclasses  include/estimator.h:32-141
 *
 * Errors: every C call that returns a negative PGB_E* code raises pgb::Error
 * (a std::runtime_error carrying the code and the library's message).  The
 * library has no CPU fallback, so without a usable CUDA device the first call
 * (the Context constructor) throws with code PGB_ECUDA.
 */
#ifndef PIMC_GB300_HPP
#define PIMC_GB300_HPP

#include "pimc_gb300.h"

#include <array>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <ostream>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace pgb {

/* beadLocator = {slice, particle} (include/common.h: TinyVector<int,2>) */
using beadLocator = std::array<int, 2>;
using dVec = std::array<double, 3>;

class Error : public std::runtime_error {
 public:
  Error(int code, const std::string& what) : std::runtime_error(what), code_(code) {}
  int code() const { return code_; }
 private:
  int code_;
};

inline void check(int rc, const pgb_ctx* ctx) {
  if (rc != PGB_OK) {
    const char* m = pgb_last_error(ctx);
    throw Error(rc, std::string("pimc_gb300: ") + (m ? m : "error ") + " (code " +
                        std::to_string(rc) + ")");
  }
}
/* the same with the message of another handle */
inline void check(int rc, const pgb_ctx*, const char* msg) {
  if (rc != PGB_OK)
    throw Error(rc, std::string("pimc_gb300: ") + (msg ? msg : "error ") + " (code " +
                        std::to_string(rc) + ")");
}

/* The LocalAction factors of Setup::action (src/setup.cpp:1216-1266):
 * primitive VFactor {1,1}, gradVFactor {0,0}, period 1;
 * gsf VFactor {2/3,4/3}, gradVFactor {2 alpha/9, 2 (1-alpha)/9} with the
 * reference's alpha = 0, i.e. {0, 2/9}, period 2. */
struct Params : pgb_params {
  Params() : pgb_params{} {
    vfactor[0] = vfactor[1] = 1.0;
    period = 1;
    aziz_year = 1979;
    virial_window = 5;
    precision = PGB_FP64;
  }
  static Params primitive(double side, int M, int N, double tau, double lambda) {
    Params p;
    p.side[0] = p.side[1] = p.side[2] = side;
    p.num_slices = M;
    p.num_ptcl_ext = N;
    p.tau = tau;
    p.lambda = lambda;
    p.rc = side;
    return p;
  }
  static Params gsf(double side, int M, int N, double tau, double lambda) {
    Params p = primitive(side, M, N, tau, lambda);
    p.vfactor[0] = 2.0 / 3.0;
    p.vfactor[1] = 4.0 / 3.0;
    p.gradvfactor[0] = 0.0;
    p.gradvfactor[1] = 2.0 / 9.0;
    p.period = 2;
    return p;
  }
};

/* One device context: the path's mirror, its Aziz tables and its stream.
 * Move-only; every mutation made through it bumps epoch() so that cached
 * per-slice terms know when to recompute. */
class Context {
 public:
  explicit Context(const pgb_params& p) : p_(p) { pgb::check(pgb_create(&p_, &h_), nullptr); }
  ~Context() {
    if (h_) pgb_destroy(h_);
  }
  Context(const Context&) = delete;
  Context& operator=(const Context&) = delete;
  Context(Context&& o) noexcept : h_(o.h_), p_(o.p_), epoch_(o.epoch_) { o.h_ = nullptr; }
  Context& operator=(Context&& o) noexcept {
    std::swap(h_, o.h_);
    std::swap(p_, o.p_);
    std::swap(epoch_, o.epoch_);
    return *this;
  }
  pgb_ctx* get() const { return h_; }
  const pgb_params& params() const { return p_; }
  uint64_t epoch() const { return epoch_; }
  void touch() { ++epoch_; }
  void check(int rc) const { pgb::check(rc, h_); }
  /* MTRand::save / load (MersenneTwister.h) of the plain form's generator:
   * 624 state words then `left`, the state file's last line */
  void saveRandom(uint32_t out[625]) const { check(pgb_plain_get_rng(h_, out)); }
  void loadRandom(const uint32_t in[625]) { check(pgb_plain_set_rng(h_, in)); }

 private:
  pgb_ctx* h_ = nullptr;
  pgb_params p_;
  uint64_t epoch_ = 0;
};

/* AzizPotential (include/potential.h:933-1017): the tabulated HFDHE2 pair
 * potential, evaluated on the device.  V(dVec) etc. are one-pair calls kept
 * for parity with the reference; batch through V(const dVec*, double*, int). */
class AzizPotential {
 public:
  explicit AzizPotential(Context& ctx) : ctx_(&ctx) {
    int len;
    double dr;
    ctx_->check(pgb_table_info(ctx_->get(), &len, &dr, &tailV));
  }
  double V(const dVec& sep) const {
    double v;
    ctx_->check(pgb_potential_batch(ctx_->get(), sep.data(), &v, 1));
    return v;
  }
  /* PotentialBase::V(const dVec*, double*, int) (potential.h:86) */
  void V(const dVec* sep, double* out, int n) const {
    ctx_->check(pgb_potential_batch(ctx_->get(), sep->data(), out, n));
  }
  dVec gradV(const dVec& sep) const {
    dVec g;
    ctx_->check(pgb_gradv_batch(ctx_->get(), sep.data(), g.data(), 1));
    return g;
  }
  void gradV(const dVec* sep, dVec* out, int n) const {
    ctx_->check(pgb_gradv_batch(ctx_->get(), sep->data(), out->data(), n));
  }
  double grad2V(const dVec& sep) const {
    double v;
    ctx_->check(pgb_grad2v_batch(ctx_->get(), sep.data(), &v, 1));
    return v;
  }
  double tailV = 0.0;  /* PotentialBase::tailV */

 private:
  Context* ctx_;
};

/* The device mirror of Path (include/path.h): beads, links and worm state.
 * The reference mutates its own Path first and then asks the action; the
 * mirror must see the same mutations (Path::updateBead, src/path.cpp:197-200). */
class Path {
 public:
  explicit Path(Context& ctx) : ctx_(&ctx) {}
  /* positions AoS [M][Ne][3]; next/prev [M][Ne][2]; on [M][Ne]; worm8 = head,
   * tail, special1, special2 (Path::nextLink/prevLink, Worm::beads).  With
   * next/prev/on left null the path is closed, every bead on, and particle p
   * of slice t links to particle p of slices t +- 1 (the identity
   * permutation of Path's constructor, src/path.cpp:50-75). */
  void load(const double* pos, const int32_t* next = nullptr, const int32_t* prev = nullptr,
            const uint8_t* on = nullptr, const int32_t* worm8 = nullptr) {
    const pgb_params& p = ctx_->params();
    const int M = p.num_slices, N = p.num_ptcl_ext;
    std::vector<int32_t> nx, pv;
    std::vector<uint8_t> o;
    if (!next || !prev) {
      nx.resize((size_t)M * N * 2);
      pv.resize((size_t)M * N * 2);
      for (int t = 0; t < M; ++t)
        for (int i = 0; i < N; ++i) {
          const size_t k = 2 * ((size_t)t * N + i);
          nx[k] = (t + 1) % M;
          nx[k + 1] = i;
          pv[k] = (t + M - 1) % M;
          pv[k + 1] = i;
        }
      next = nx.data();
      prev = pv.data();
    }
    if (!on) {
      o.assign((size_t)M * N, 1);
      on = o.data();
    }
    ctx_->check(pgb_load_path(ctx_->get(), pos, next, prev, on, worm8));
    ctx_->touch();
  }
  void updateBead(const beadLocator& b, const dVec& pos) {
    const int32_t bl[2] = {b[0], b[1]};
    ctx_->check(pgb_update_beads(ctx_->get(), bl, pos.data(), 1));
    ctx_->touch();
  }
  void updateBeads(const std::vector<beadLocator>& beads, const std::vector<dVec>& pos) {
    if (beads.size() != pos.size()) throw Error(PGB_EINVAL, "pimc_gb300: beads/pos size mismatch");
    std::vector<int32_t> bl(2 * beads.size());
    for (size_t i = 0; i < beads.size(); ++i) {
      bl[2 * i] = beads[i][0];
      bl[2 * i + 1] = beads[i][1];
    }
    ctx_->check(pgb_update_beads(ctx_->get(), bl.data(), pos.empty() ? nullptr : pos[0].data(),
                                 (int)beads.size()));
    ctx_->touch();
  }
  std::vector<double> positions() const {
    const pgb_params& p = ctx_->params();
    std::vector<double> out((size_t)p.num_slices * p.num_ptcl_ext * 3);
    ctx_->check(pgb_get_positions(ctx_->get(), out.data()));
    return out;
  }

 private:
  Context* ctx_;
};

/* ActionBase / LocalAction (include/action.h:30-254, src/action.cpp:345-1803).
 * The per-slice estimator-facing virtuals are filled by one device call per
 * configuration (pgb_slice_terms_compute) and then indexed by slice. */
class LocalAction {
 public:
  explicit LocalAction(Context& ctx) : ctx_(&ctx) {}

  void setShift(int s) { shift_ = s; }
  int getShift() const { return shift_; }
  /* ActionBase::tau(): shift * tau (action.h:107) */
  double tau() const { return shift_ * ctx_->params().tau; }

  /* potentialAction() over the whole path, action.cpp:456-472 */
  double potentialAction() const {
    double u;
    ctx_->check(pgb_full_action(ctx_->get(), &u));
    return u;
  }
  /* potentialAction(bead), action.cpp:487-514 */
  double potentialAction(const beadLocator& b) const { return one(b, PGB_ACTION_FULL); }
  /* potentialAction(startBead, endBead), action.cpp:522-570 */
  double potentialAction(const beadLocator& b0, const beadLocator& b1) const {
    double u;
    ctx_->check(pgb_range_action(ctx_->get(), b0[0], b0[1], b1[0], b1[1], shift_, &u));
    return u;
  }
  /* potentialAction(vector<beadLocator>), action.cpp:572-620 */
  double potentialAction(const std::vector<beadLocator>& beads) const {
    std::vector<int32_t> bl = flat(beads);
    double u = 0.0;
    ctx_->check(pgb_bead_actions(ctx_->get(), bl.data(), (int)beads.size(), shift_,
                                 PGB_ACTION_FULL, nullptr, &u));
    return u;
  }
  /* barePotentialAction(bead), action.cpp:628-690 */
  double barePotentialAction(const beadLocator& b) const { return one(b, PGB_ACTION_BARE); }
  /* barePotentialAction(vector, vector<double>&): one value per bead */
  void barePotentialAction(const std::vector<beadLocator>& beads, std::vector<double>& out) const {
    std::vector<int32_t> bl = flat(beads);
    out.assign(beads.size(), 0.0);
    double sum;
    ctx_->check(pgb_bead_actions(ctx_->get(), bl.data(), (int)beads.size(), shift_,
                                 PGB_ACTION_BARE, out.data(), &sum));
  }
  /* potentialActionCorrection(bead), action.cpp:696-720 */
  double potentialActionCorrection(const beadLocator& b) const { return one(b, PGB_ACTION_CORR); }
  /* kineticAction(), action.cpp:345-369 */
  double kineticAction() const {
    double k;
    ctx_->check(pgb_kinetic_action(ctx_->get(), &k));
    return k;
  }
  /* delta U_b for each bead moved alone to pos[i]: the difference a
   * single-bead Metropolis test takes (potentialAction(bead) after - before) */
  std::vector<double> trialActions(const std::vector<beadLocator>& beads,
                                   const std::vector<dVec>& pos) const {
    if (beads.size() != pos.size()) throw Error(PGB_EINVAL, "pimc_gb300: beads/pos size mismatch");
    std::vector<int32_t> bl = flat(beads);
    std::vector<double> out(beads.size());
    ctx_->check(pgb_trial_actions(ctx_->get(), bl.data(), pos.empty() ? nullptr : pos[0].data(),
                                  (int)beads.size(), shift_, PGB_ACTION_FULL, out.data()));
    return out;
  }

  /* ---- per-slice virtuals (shift 1, as the estimators call them) ---- */
  /* V(slice) = {V_ext, V_int}, action.cpp:902-947 (no external potential) */
  std::array<double, 2> V(int slice) { return {0.0, terms().vint[idx(slice)]}; }
  /* gradVSquared(slice), action.cpp:1188-1223 */
  double gradVSquared(int slice) { return terms().g2[idx(slice)]; }
  /* derivPotentialActionTau(slice), action.cpp:751-766 */
  double derivPotentialActionTau(int slice) {
    const pgb_params& p = ctx_->params();
    const int eo = slice % 2;
    const double t = p.tau;
    double dU = p.vfactor[eo] * terms().vint[idx(slice)];
    if (p.gradvfactor[eo] > kEps) dU += 3.0 * p.gradvfactor[eo] * t * t * p.lambda * gradVSquared(slice);
    return dU;
  }
  /* secondderivPotentialActionTau(slice), action.cpp:776-788 */
  double secondderivPotentialActionTau(int slice) {
    const pgb_params& p = ctx_->params();
    const int eo = slice % 2;
    if (p.gradvfactor[eo] > kEps) return 6.0 * p.gradvfactor[eo] * p.tau * p.lambda * gradVSquared(slice);
    return 0.0;
  }
  /* derivPotentialActionLambda(slice), action.cpp:798-806 */
  double derivPotentialActionLambda(int slice) {
    const pgb_params& p = ctx_->params();
    const int eo = slice % 2;
    if (p.gradvfactor[eo] > kEps) return p.gradvfactor[eo] * p.tau * p.tau * p.tau * gradVSquared(slice);
    return 0.0;
  }
  /* rDOTgradUterm1/2 (action.cpp:1446-1573) and deltaDOTgradUterm1/2
   * (action.cpp:1588-1782) */
  double rDOTgradUterm1(int slice) { return term1(slice, terms().r1); }
  double rDOTgradUterm2(int slice) { return term2(slice, terms().r2); }
  double deltaDOTgradUterm1(int slice) { return term1(slice, terms().d1); }
  double deltaDOTgradUterm2(int slice) { return term2(slice, terms().d2); }
  /* virKinCorr(slice) = virialKinCorrection, action.cpp:1786-1803 */
  double virKinCorr(int slice) {
    const pgb_params& p = ctx_->params();
    const int eo = slice % 2;
    if (p.gradvfactor[eo] > kEps)
      return gradVSquared(slice) * p.gradvfactor[eo] * p.tau * p.tau * p.tau * p.lambda;
    return 0.0;
  }

 private:
  static constexpr double kEps = 1.0e-7;  /* EPS of the reference's common.h */
  struct Terms {
    std::vector<double> vint, g2, r1, r2, d1, d2;
  };
  const Terms& terms() {
    if (!cached_ || epoch_ != ctx_->epoch()) {
      const int M = ctx_->params().num_slices;
      for (auto* v : {&t_.vint, &t_.g2, &t_.r1, &t_.r2, &t_.d1, &t_.d2}) v->assign(M, 0.0);
      pgb_slice_terms st{};
      st.vint = t_.vint.data();
      st.g2 = t_.g2.data();
      st.r1 = t_.r1.data();
      st.r2 = t_.r2.data();
      st.d1 = t_.d1.data();
      st.d2 = t_.d2.data();
      ctx_->check(pgb_slice_terms_compute(ctx_->get(), &st));
      epoch_ = ctx_->epoch();
      cached_ = true;
    }
    return t_;
  }
  int idx(int slice) const {
    const int M = ctx_->params().num_slices;
    if (slice < 0 || slice >= M) throw Error(PGB_EINVAL, "pimc_gb300: slice out of range");
    return slice;
  }
  double term1(int slice, const std::vector<double>& v) const {
    const pgb_params& p = ctx_->params();
    return p.vfactor[slice % 2] * p.tau * v[idx(slice)];
  }
  double term2(int slice, const std::vector<double>& v) const {
    const pgb_params& p = ctx_->params();
    const int eo = slice % 2;
    if (!(p.gradvfactor[eo] > kEps)) return 0.0;
    return 2.0 * p.gradvfactor[eo] * p.tau * p.tau * p.tau * p.lambda * v[idx(slice)];
  }
  double one(const beadLocator& b, int mode) const {
    const int32_t bl[2] = {b[0], b[1]};
    double u = 0.0;
    ctx_->check(pgb_bead_actions(ctx_->get(), bl, 1, shift_, mode, nullptr, &u));
    return u;
  }
  static std::vector<int32_t> flat(const std::vector<beadLocator>& beads) {
    std::vector<int32_t> bl(2 * beads.size());
    for (size_t i = 0; i < beads.size(); ++i) {
      bl[2 * i] = beads[i][0];
      bl[2 * i + 1] = beads[i][1];
    }
    return bl;
  }

  Context* ctx_;
  int shift_ = 1;
  Terms t_;
  uint64_t epoch_ = 0;
  bool cached_ = false;
};

/* GaussianProcessPotential (include/potential.h:287-323) and the
 * GPHeBenzenePotential external potential built on it
 * (include/potential.h:2413-2450): GP(positions, values, count) and
 * V(positions, values, count) over batches, on the device. */
class GaussianProcessPotential {
 public:
  GaussianProcessPotential(const pgb_gp_params& p, const double* training, int n) {
    const int rc = pgb_gp_create(&p, training, n, &h_);
    pgb::check(rc, nullptr, pgb_gp_last_error(nullptr));
  }
  ~GaussianProcessPotential() {
    if (h_) pgb_gp_destroy(h_);
  }
  GaussianProcessPotential(const GaussianProcessPotential&) = delete;
  GaussianProcessPotential& operator=(const GaussianProcessPotential&) = delete;
  double GP(const dVec& r) {
    double v = 0.0;
    GP(&r, &v, 1);
    return v;
  }
  void GP(const dVec* positions, double* values, int count) {
    const int rc = pgb_gp_eval(h_, count ? positions[0].data() : nullptr, values, count);
    pgb::check(rc, nullptr, pgb_gp_last_error(h_));
  }
  /* GPHeBenzenePotential::V */
  void benzeneV(const dVec* positions, double* values, int count) {
    const int rc = pgb_gp_benzene_v(h_, count ? positions[0].data() : nullptr, values, count);
    pgb::check(rc, nullptr, pgb_gp_last_error(h_));
  }
  pgb_gp* get() const { return h_; }

 private:
  pgb_gp* h_ = nullptr;
};

/* EstimatorBase (include/estimator.h:32-141): sample() accumulates every
 * `frequency` calls; getEstimator(i) is the running average
 * estimator(i) / numAccumulated that output() writes. */
class EstimatorBase {
 public:
  EstimatorBase(Context& ctx, int ncols, int frequency = 1)
      : ctx_(&ctx), est_(ncols, 0.0), norm_(ncols, 1.0), freq_(frequency < 1 ? 1 : frequency) {}
  virtual ~EstimatorBase() = default;
  virtual std::string getName() const { return "base"; }
  void sample() {
    if (numSampled_++ % freq_ == 0 && ready()) {
      accumulate();
      ++numAccumulated_;
      ++totNumAccumulated_;
    }
  }
  void reset() {
    est_.assign(est_.size(), 0.0);
    numAccumulated_ = 0;
  }
  long long numAccumulated() const { return numAccumulated_; }
  double getEstimator(int i) const {
    return numAccumulated_ ? est_.at(i) / (double)numAccumulated_ : 0.0;
  }
  const std::vector<double>& sums() const { return est_; }
  long long getNumSampled() const { return numSampled_; }
  long long getTotNumAccumulated() const { return totNumAccumulated_; }
  /* EstimatorBase::restart (estimator.cpp:333-337) */
  void restart(long long numSampled, long long totNumAccumulated) {
    numSampled_ = numSampled;
    totNumAccumulated_ = totNumAccumulated;
    reset();
  }
  /* EstimatorBase::output (estimator.cpp:348-363): the bin average
   * estimator * norm / numAccumulated as "%16.8E" columns, then reset */
  void output(std::ostream& os, bool endLine = true) {
    char buf[32];
    for (size_t n = 0; n < est_.size(); ++n) {
      const double v = numAccumulated_ ? est_[n] * (norm_[n] / (1.0 * numAccumulated_)) : 0.0;
      std::snprintf(buf, sizeof buf, "%16.8E", v);
      os << buf;
    }
    if (endLine) os << "\n";
    reset();
  }
  const std::vector<double>& norm() const { return norm_; }

 protected:
  virtual void accumulate() = 0;
  /* whether this sample counts (the cylinder estimators skip samples with
   * no particle inside their radius, estimator.cpp:5464-5471) */
  virtual bool ready() { return true; }
  Context* ctx_;
  std::vector<double> est_;
  std::vector<double> norm_;
  long long totNumAccumulated_ = 0;

 private:
  int freq_;
  long long numSampled_ = 0, numAccumulated_ = 0;
};

/* EnergyEstimator (estimator.cpp:917-1029): K, V, V_ext, V_int, E, E_mu,
 * K/N, V/N, E/N */
class EnergyEstimator : public EstimatorBase {
 public:
  explicit EnergyEstimator(Context& ctx, int frequency = 1) : EstimatorBase(ctx, 9, frequency) {}
  std::string getName() const override { return "energy"; }

 protected:
  void accumulate() override {
    double v[9];
    ctx_->check(pgb_energy(ctx_->get(), v));
    for (int i = 0; i < 9; ++i) est_[i] += v[i];
  }
};

/* VirialEnergyEstimator (estimator.cpp:1045-1252), 19 columns; the
 * reference's cVCov2 behaviour is kept unless told otherwise */
class VirialEnergyEstimator : public EstimatorBase {
 public:
  explicit VirialEnergyEstimator(Context& ctx, int frequency = 1, bool cvcov2_quirk = true)
      : EstimatorBase(ctx, 19, frequency), quirk_(cvcov2_quirk) {}
  std::string getName() const override { return "virial"; }

 protected:
  void accumulate() override {
    double v[19];
    ctx_->check(pgb_virial(ctx_->get(), quirk_ ? 1 : 0, v));
    for (int i = 0; i < 19; ++i) est_[i] += v[i];
  }

 private:
  bool quirk_;
};

/* PairCorrelationEstimator (estimator.cpp:3181-3246): g(r) over 50 bins of
 * 0.5 sqrt(3) L_z / 50 from the separation histogram of all slices; the
 * library returns each sample with the estimator's norm applied */
class PairCorrelationEstimator : public EstimatorBase {
 public:
  explicit PairCorrelationEstimator(Context& ctx, int frequency = 1) : EstimatorBase(ctx, 50, frequency) {}
  std::string getName() const override { return "pair correlation function"; }

 protected:
  void accumulate() override {
    double g[50];
    ctx_->check(pgb_pair_correlation(ctx_->get(), -1, g));
    for (int n = 0; n < 50; ++n) est_[n] += g[n];
  }
};

/* SuperfluidFractionEstimator (estimator.cpp:1963-2074): W^2/N, W_x^2,
 * W_y^2, W_z^2, P(-10..10), Az^2/I with norms T/(2*3*lambda) and
 * T M/(2 lambda) on the first and last columns */
class SuperfluidFractionEstimator : public EstimatorBase {
 public:
  SuperfluidFractionEstimator(Context& ctx, double temperature, int frequency = 1)
      : EstimatorBase(ctx, 26, frequency) {
    const pgb_params& p = ctx.params();
    norm_[0] = temperature / (2.0 * 3.0 * p.lambda);
    norm_[25] = 0.5 * temperature * p.num_slices / p.lambda;
  }
  std::string getName() const override { return "superfluid fraction"; }

 protected:
  void accumulate() override {
    double v[26];
    ctx_->check(pgb_superfluid(ctx_->get(), v));
    for (int i = 0; i < 26; ++i) est_[i] += v[i];
  }
};

/* PermutationCycleEstimator (estimator.cpp:2700-2781): 40 cycle lengths */
class PermutationCycleEstimator : public EstimatorBase {
 public:
  explicit PermutationCycleEstimator(Context& ctx, int frequency = 1) : EstimatorBase(ctx, 40, frequency) {}
  std::string getName() const override { return "permutation cycle"; }

 protected:
  void accumulate() override {
    double v[40];
    ctx_->check(pgb_permutation_cycles(ctx_->get(), v));
    for (int i = 0; i < 40; ++i) est_[i] += v[i];
  }
};

/* CylinderStaticStructureFactorEstimator (estimator.cpp:5363-5471): the
 * "line" shells q = (0, 0, n 2 pi / L_z), |q| <= 4; per sample the included
 * beads' sum / num1DParticles, norm 1/M per shell vector count; samples with
 * no particle inside maxR are skipped */
class CylinderStaticStructureFactorEstimator : public EstimatorBase {
 public:
  CylinderStaticStructureFactorEstimator(Context& ctx, double maxR, int frequency = 1)
      : EstimatorBase(ctx, shellCount(ctx), frequency), maxR_(maxR) {
    const double dq = 2.0 * 3.14159265358979323846 / ctx.params().side[2];
    int n = 0;
    check(pgb_qvectors_shells(dq, 4.0, 0, nullptr, nullptr, 0, &n), nullptr);
    q_.resize((size_t)n);
    shell_.resize((size_t)n);
    if (n) check(pgb_qvectors_shells(dq, 4.0, 0, q_[0].data(), shell_.data(), n, &n), nullptr);
    std::vector<int> per(est_.size(), 0);
    for (int s : shell_) ++per[(size_t)s];
    for (size_t k = 0; k < est_.size(); ++k)
      norm_[k] = (1.0 / ctx.params().num_slices) / (per[k] > 0 ? per[k] : 1);
    tmp_.resize(q_.size());
  }
  std::string getName() const override { return "cylinder static structure factor"; }

 protected:
  bool ready() override {
    int n0 = 0;
    ctx_->check(pgb_ssf_cylinder(ctx_->get(), nullptr, 0, maxR_, nullptr, &n0));
    return n0 > 0;
  }
  void accumulate() override {
    int n0 = 0;
    ctx_->check(pgb_ssf_cylinder(ctx_->get(), q_[0].data(), (int)q_.size(), maxR_, tmp_.data(), &n0));
    // the device value is already divided by M; the norm divides by M again
    // in the reference's order, so undo it here
    for (size_t i = 0; i < q_.size(); ++i)
      est_[(size_t)shell_[i]] += tmp_[i] * ctx_->params().num_slices / n0;
  }

 private:
  static int shellCount(const Context& ctx) {
    const double dq = 2.0 * 3.14159265358979323846 / ctx.params().side[2];
    int n = 0;
    check(pgb_qvectors_shells(dq, 4.0, 0, nullptr, nullptr, 0, &n), nullptr);
    std::vector<dVec> q((size_t)n);
    std::vector<int> sh((size_t)n);
    if (n) check(pgb_qvectors_shells(dq, 4.0, 0, q[0].data(), sh.data(), n, &n), nullptr);
    return n ? sh.back() + 1 : 0;
  }
  double maxR_;
  std::vector<dVec> q_;
  std::vector<int> shell_;
  std::vector<double> tmp_;
};

/* CylinderStaticStructureFactorGPUEstimator (estimator.cpp:5486-5613,
 * gpu_ssf_cyl estimator_gpu.cu:169-285): user q-vectors, per sample the
 * included beads' sum over ordered pairs / (N M); numParticles is
 * Path::getTrueNumParticles (every worldline by default) */
class CylinderStaticStructureFactorGPUEstimator : public EstimatorBase {
 public:
  CylinderStaticStructureFactorGPUEstimator(Context& ctx, std::vector<dVec> q, double maxR,
                                            int frequency = 1, int numParticles = -1)
      : EstimatorBase(ctx, (int)q.size(), frequency), q_(std::move(q)), maxR_(maxR),
        N_(numParticles < 0 ? ctx.params().num_ptcl_ext : numParticles), tmp_(q_.size()) {}
  std::string getName() const override { return "cylinder static structure factor gpu"; }

 protected:
  bool ready() override {
    int n0 = 0;
    ctx_->check(pgb_ssf_cylinder(ctx_->get(), nullptr, 0, maxR_, nullptr, &n0));
    return n0 > 0;
  }
  void accumulate() override {
    if (q_.empty()) return;
    int n0 = 0;
    ctx_->check(pgb_ssf_cylinder(ctx_->get(), q_[0].data(), (int)q_.size(), maxR_, tmp_.data(), &n0));
    for (size_t i = 0; i < q_.size(); ++i) est_[i] += tmp_[i] / N_;
  }

 private:
  std::vector<dVec> q_;
  double maxR_;
  int N_;
  std::vector<double> tmp_;
};

/* EstimatorBase::getQVectors (estimator.cpp:439-570) */
inline std::vector<dVec> getQVectors(const std::string& type, const std::string& input,
                                     const double side[3]) {
  int count = 0;
  check(pgb_qvectors(type.c_str(), input.c_str(), side, nullptr, 0, &count), nullptr);
  std::vector<dVec> q((size_t)count);
  if (count) check(pgb_qvectors(type.c_str(), input.c_str(), side, q[0].data(), count, &count), nullptr);
  return q;
}

/* StaticStructureFactor(GPU)Estimator (estimator.cpp:3661-3861): one column
 * per q, already normalised per sample */
class StaticStructureFactorEstimator : public EstimatorBase {
 public:
  StaticStructureFactorEstimator(Context& ctx, std::vector<dVec> q, int frequency = 1)
      : EstimatorBase(ctx, (int)q.size(), frequency), q_(std::move(q)), tmp_(q_.size()) {}
  std::string getName() const override { return "ssf"; }

 protected:
  void accumulate() override {
    if (q_.empty()) return;
    ctx_->check(pgb_ssf(ctx_->get(), q_[0].data(), (int)q_.size(), tmp_.data()));
    for (size_t i = 0; i < q_.size(); ++i) est_[i] += tmp_[i];
  }

 private:
  std::vector<dVec> q_;
  std::vector<double> tmp_;
};

/* IntermediateScatteringFunctionEstimatorGpu (estimator.cpp:3973-4236):
 * layout [q][M/2+1].  mode 0: CUDA-core correlation; 1: tensor cores. */
class IntermediateScatteringFunctionEstimator : public EstimatorBase {
 public:
  IntermediateScatteringFunctionEstimator(Context& ctx, std::vector<dVec> q, int mode = 0,
                                          int frequency = 1)
      : EstimatorBase(ctx, (int)q.size() * (ctx.params().num_slices / 2 + 1), frequency),
        q_(std::move(q)), mode_(mode), tmp_(est_.size()) {}
  std::string getName() const override { return "isf"; }

 protected:
  void accumulate() override {
    if (q_.empty()) return;
    ctx_->check(pgb_isf(ctx_->get(), q_[0].data(), (int)q_.size(), mode_, tmp_.data()));
    for (size_t i = 0; i < tmp_.size(); ++i) est_[i] += tmp_[i];
  }

 private:
  std::vector<dVec> q_;
  int mode_;
  std::vector<double> tmp_;
};

}  // namespace pgb

#endif
