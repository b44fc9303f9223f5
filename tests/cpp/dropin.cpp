// C++ drop-in test of include/pimc_gb300.hpp: the plugin-class mirror is used
// the way the reference's PathIntegralMonteCarlo uses LocalAction and its
// estimators, and every value is compared with the CPU oracle on the same
// worldlines.
//
//   dropin nodevice   -- expects the Context constructor to throw
//                        pgb::Error(PGB_ECUDA): the library has no CPU path
//   dropin parity     -- GSF action, N=24, M=16: per-bead, list, range, bare,
//                        correction, full and kinetic actions; the per-slice
//                        derivatives and virial terms; the energy, virial and
//                        S(q) estimators; all within 1e-12 (relative, floor 1)
#include "pimc_gb300.hpp"
#include "pimc_oracle.h"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <sstream>
#include <vector>

static int g_fail = 0;
static double g_worst = 0.0;

static void cmp(const char* what, double got, double want, double tol = 1e-12) {
  const double err = std::fabs(got - want) / std::fmax(1.0, std::fabs(want));
  if (err > g_worst) g_worst = err;
  if (!(err <= tol)) {
    std::printf("MISMATCH %s: got %.17g want %.17g (rel %.3g)\n", what, got, want, err);
    ++g_fail;
  }
}

static void check_rng(pgb::Context& ctx) {
  ctx.check(pgb_plain_seed(ctx.get(), 4242u));
  uint32_t got[625], want[625];
  ctx.saveRandom(got);
  orc_mt* mt = orc_mt_create(4242u);
  for (int k = 0; k < 1000; ++k) orc_mt_randint(mt);
  orc_mt_save(mt, want);
  ctx.loadRandom(want);
  uint32_t back[625];
  ctx.saveRandom(back);
  int bad = got[624] != 624u;
  for (int i = 0; i < 625; ++i) bad += back[i] != want[i];
  orc_mt_destroy(mt);
  if (bad) {
    std::printf("MISMATCH generator state save/load (%d words)\n", bad);
    ++g_fail;
  }
}

int main(int argc, char** argv) {
  std::setvbuf(stdout, nullptr, _IONBF, 0);
  const char* mode = argc > 1 ? argv[1] : "parity";
  const int N = 24, M = 16;
  const double lam = 24.24 / 4.000264, tau = 0.025, L = std::cbrt(N / 0.02186);
  pgb::Params p = pgb::Params::gsf(L, M, N, tau, lam);

  if (!std::strcmp(mode, "nodevice")) {
    try {
      pgb::Context ctx(p);
    } catch (const pgb::Error& e) {
      std::printf("threw code %d: %s\n", e.code(), e.what());
      return e.code() == PGB_ECUDA ? 0 : 1;
    }
    std::printf("no exception without a device\n");
    return 1;
  }

  // seeded worldlines: uniform particle centres, Gaussian jitter per bead
  std::mt19937_64 rng(20261203);
  std::uniform_real_distribution<double> u(-0.5 * L, 0.5 * L);
  std::normal_distribution<double> g(0.0, std::sqrt(2.0 * lam * tau));
  std::vector<double> pos((size_t)M * N * 3);
  for (int i = 0; i < N; ++i) {
    const double c[3] = {u(rng), u(rng), u(rng)};
    for (int t = 0; t < M; ++t)
      for (int d = 0; d < 3; ++d) {
        double x = c[d] + g(rng);
        x -= L * std::floor(x / L + 0.5);
        pos[3 * ((size_t)t * N + i) + d] = x;
      }
  }
  std::vector<int32_t> next((size_t)M * N * 2), prev((size_t)M * N * 2);
  std::vector<uint8_t> on((size_t)M * N, 1);
  for (int t = 0; t < M; ++t)
    for (int i = 0; i < N; ++i) {
      const size_t k = 2 * ((size_t)t * N + i);
      next[k] = (t + 1) % M, next[k + 1] = i;
      prev[k] = (t + M - 1) % M, prev[k + 1] = i;
    }

  orc_params op{};
  for (int d = 0; d < 3; ++d) op.side[d] = L;
  op.num_slices = M, op.num_ptcl_ext = N, op.tau = tau, op.lambda = lam, op.rc = L;
  op.vfactor[0] = p.vfactor[0], op.vfactor[1] = p.vfactor[1];
  op.gradvfactor[0] = p.gradvfactor[0], op.gradvfactor[1] = p.gradvfactor[1];
  op.aziz_year = 1979, op.virial_window = p.virial_window, op.mu = 0.0;
  orc_sys* o = orc_create(&op);
  const int32_t no_worm[8] = {-1, -1, -1, -1, -1, -1, -1, -1};
  orc_load_path(o, pos.data(), next.data(), prev.data(), on.data(), no_worm);

  pgb::Context ctx(p);
  pgb::Path path(ctx);
  path.load(pos.data());  // identity links filled by the mirror
  pgb::LocalAction act(ctx);
  pgb::AzizPotential pot(ctx);
  cmp("tailV", pot.tailV, orc_tailV(o));

  char name[96];
  // pair potential on a few separations
  for (double r : {2.2, 2.9637, 3.5, 6.0}) {
    const pgb::dVec s = {r / std::sqrt(3.0), r / std::sqrt(3.0), r / std::sqrt(3.0)};
    std::snprintf(name, sizeof name, "V(%g)", r);
    cmp(name, pot.V(s), orc_V(o, s.data()));
  }

  // per-bead forms at shifts 1 and 2
  for (int shift : {1, 2}) {
    act.setShift(shift);
    orc_set_shift(o, shift);
    for (int t = 0; t < M; t += 3)
      for (int i = 0; i < N; i += 5) {
        std::snprintf(name, sizeof name, "U(%d,%d) shift %d", t, i, shift);
        cmp(name, act.potentialAction({t, i}), orc_potential_action_bead(o, t, i));
        std::snprintf(name, sizeof name, "Ubare(%d,%d) shift %d", t, i, shift);
        cmp(name, act.barePotentialAction({t, i}), orc_bare_potential_action(o, t, i));
        std::snprintf(name, sizeof name, "Ucorr(%d,%d) shift %d", t, i, shift);
        cmp(name, act.potentialActionCorrection({t, i}), orc_potential_action_correction(o, t, i));
      }
  }
  act.setShift(1);
  orc_set_shift(o, 1);
  cmp("U(range 2:3 -> 9:3)", act.potentialAction(pgb::beadLocator{2, 3}, pgb::beadLocator{9, 3}),
      orc_potential_action_range(o, 2, 3, 9, 3));
  std::vector<pgb::beadLocator> list = {{0, 0}, {1, 5}, {7, 11}, {15, 23}};
  std::vector<int32_t> flat;
  for (auto& b : list) flat.push_back(b[0]), flat.push_back(b[1]);
  cmp("U(list)", act.potentialAction(list), orc_potential_action_list(o, flat.data(), (int)list.size()));
  std::vector<double> bare;
  act.barePotentialAction(list, bare);
  for (size_t k = 0; k < list.size(); ++k)
    cmp("Ubare(list)", bare[k], orc_bare_potential_action(o, list[k][0], list[k][1]));
  cmp("U(full)", act.potentialAction(), orc_potential_action_full(o));
  cmp("K(full)", act.kineticAction(), orc_kinetic_action_full(o));

  for (int t = 0; t < M; ++t) {
    double v2[2];
    orc_V_slice(o, t, v2);
    std::snprintf(name, sizeof name, "V(slice %d)", t);
    cmp(name, act.V(t)[1], v2[1]);
    cmp("gradVSquared", act.gradVSquared(t), orc_gradVSquared_slice(o, t));
    cmp("dU/dtau", act.derivPotentialActionTau(t), orc_deriv_tau(o, t));
    cmp("d2U/dtau2", act.secondderivPotentialActionTau(t), orc_second_deriv_tau(o, t));
    cmp("dU/dlambda", act.derivPotentialActionLambda(t), orc_deriv_lambda(o, t));
    cmp("rDOTgradU1", act.rDOTgradUterm1(t), orc_rdotgradU1(o, t));
    cmp("rDOTgradU2", act.rDOTgradUterm2(t), orc_rdotgradU2(o, t));
    cmp("deltaDOTgradU1", act.deltaDOTgradUterm1(t), orc_deltadotgradU1(o, t));
    cmp("deltaDOTgradU2", act.deltaDOTgradUterm2(t), orc_deltadotgradU2(o, t));
    cmp("virKinCorr", act.virKinCorr(t), orc_virial_kin_corr(o, t));
  }

  // a bead moved through the mirror: the cached slice terms follow
  const pgb::dVec moved = {0.1, -0.2, 0.3};
  path.updateBead({5, 7}, moved);
  orc_update_bead(o, 5, 7, moved.data());
  cmp("U(5,7) after move", act.potentialAction({5, 7}), orc_potential_action_bead(o, 5, 7));
  cmp("dU/dtau(5) after move", act.derivPotentialActionTau(5), orc_deriv_tau(o, 5));
  const std::vector<double> back = path.positions();
  for (int d = 0; d < 3; ++d) cmp("positions()", back[3 * (5 * N + 7) + d], moved[d], 0.0);

  // estimators: two samples of the same configuration average to one
  pgb::EnergyEstimator en(ctx);
  pgb::VirialEnergyEstimator vir(ctx);
  en.sample();
  en.sample();
  vir.sample();
  double e9[9], v19[19];
  orc_energy(o, e9);
  orc_virial(o, 1, v19);
  for (int i = 0; i < 9; ++i) cmp("energy column", en.getEstimator(i), e9[i]);
  for (int i = 0; i < 19; ++i) cmp("virial column", vir.getEstimator(i), v19[i], 1e-11);

  const double side[3] = {L, L, L};
  std::vector<pgb::dVec> q = pgb::getQVectors("max_float", "3 0 0", side);
  std::vector<double> qflat;
  for (auto& v : q) qflat.insert(qflat.end(), v.begin(), v.end());
  std::vector<double> want(q.size());
  orc_ssf_pairwise(o, qflat.data(), (int)q.size(), want.data());
  pgb::StaticStructureFactorEstimator ssf(ctx, q);
  ssf.sample();
  for (size_t k = 0; k < q.size(); ++k) cmp("S(q)", ssf.getEstimator((int)k), want[k], 1e-10);

  // adjacent path-wide estimators, their norms and the bin row format
  pgb::PairCorrelationEstimator pcf(ctx);
  pgb::SuperfluidFractionEstimator sfe(ctx, 1.0 / (M * tau));
  pgb::PermutationCycleEstimator pce(ctx);
  pcf.sample();
  sfe.sample();
  pce.sample();
  double g50[50], s26[26], c40[40];
  orc_pair_correlation(o, -1, g50);
  orc_superfluid(o, s26);
  orc_permutation_cycles(o, c40);
  for (int n = 0; n < 50; ++n) cmp("g(r) bin", pcf.getEstimator(n), g50[n], 1e-14);
  for (int i = 0; i < 26; ++i) cmp("superfluid column", sfe.getEstimator(i), s26[i]);
  for (int i = 0; i < 40; ++i) cmp("cycle column", pce.getEstimator(i), c40[i], 0.0);
  {
    // the first column is W^2/N times T/(6 lambda); W of closed paths is
    // zero up to rounding, so take the library's own value for the format
    const double w0 = sfe.getEstimator(0), a25 = sfe.getEstimator(25);
    std::ostringstream row;
    sfe.output(row);
    char want0[40];
    std::snprintf(want0, sizeof want0, "%16.8E", w0 * ((1.0 / (M * tau)) / (6.0 * lam)));
    cmp("Area_rho_s column", sfe.norm()[25], 0.5 * (1.0 / (M * tau)) * M / lam, 1e-15);
    (void)a25;
    const std::string r = row.str();
    if (r.size() != 26 * 16 + 1 || r.compare(0, 16, want0) != 0 || sfe.numAccumulated() != 0 ||
        sfe.getTotNumAccumulated() != 1) {
      std::printf("MISMATCH superfluid row '%s' (want first column '%s')\n", r.c_str(), want0);
      ++g_fail;
    }
  }

  // cylinder S(q): the CPU estimator's shells against the oracle's pair loop,
  // the GPU estimator with every bead inside against the prism S(q)
  {
    const double R = 0.3 * L;
    pgb::CylinderStaticStructureFactorEstimator cyl(ctx, R);
    cyl.sample();
    const int ns = (int)cyl.sums().size();
    std::vector<double> qz((size_t)ns * 3, 0.0), want_c((size_t)ns);
    int qn = 0;
    std::vector<int> sh((size_t)ns);
    pgb_qvectors_shells(2.0 * 3.14159265358979323846 / L, 4.0, 0, qz.data(), sh.data(), ns, &qn);
    int n0 = 0;
    orc_ssf_cylinder(o, qz.data(), ns, R, want_c.data(), &n0);
    if (qn != ns || n0 <= 0 || cyl.numAccumulated() != 1) {
      std::printf("MISMATCH cylinder shells %d/%d, inside %d\n", qn, ns, n0);
      ++g_fail;
    }
    for (int k = 0; k < ns; ++k)
      cmp("cylinder S(q) shell", cyl.getEstimator(k) * cyl.norm()[k], want_c[k] / n0, 1e-10);
    pgb::CylinderStaticStructureFactorGPUEstimator cylg(ctx, q, 2.0 * L);
    cylg.sample();
    for (size_t k = 0; k < q.size(); ++k)
      cmp("cylinder S(q), all inside", cylg.getEstimator((int)k), ssf.getEstimator((int)k), 1e-11);
  }

  // the plain form's generator state is MTRand::save's image
  check_rng(ctx);

  // an out-of-range slice is an error, not a read past the arrays
  bool threw = false;
  try {
    act.gradVSquared(M);
  } catch (const pgb::Error& e) {
    threw = e.code() == PGB_EINVAL;
  }
  if (!threw) {
    std::printf("MISMATCH out-of-range slice did not raise PGB_EINVAL\n");
    ++g_fail;
  }

  orc_destroy(o);
  std::printf("q-vectors %zu, worst relative error %.3g, mismatches %d\n", q.size(), g_worst, g_fail);
  return g_fail ? 1 : 0;
}
