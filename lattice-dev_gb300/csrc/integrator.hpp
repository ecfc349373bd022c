// integrator.hpp -- expansion of an integrator call into the reference's exact
// sequence of Hamiltonian pieces.
//
// symp2/4/6/8 -> symp_o2step -> Hamiltonian_Split, restated from
// Pseudospec/openmp_dev/evolve_spectral.f90:129-227 and
// hamiltonian_conformal.f90:50-81 (PSEUDOSPEC order) and
// Discrete/Bubble-Collisions/evolve.f90:98-223,225-240 (DEFROST order).
// The engine then executes the op list, fusing where it can.
#pragma once
#include <cmath>
#include <vector>

#include "engine.hpp"

namespace lat {

struct Op {
  char t;    // 'D' fields kinetic (drift), 'K' gradient+potential (kick),
             // 'G' gravity / metric kinetic, 'M' metric kinetic without expansion (clock only)
  double h;
};

struct Emitter {
  int nterms;           // 2 (Minkowski, PSEUDOSPEC) or 3
  bool defrost;         // DEFROST order: 1 = metric, 2 = drift, 3 = kick
  bool conformal;
  std::vector<Op>* ops;
  double* tg;           // tglobal(1:3), advanced per Hamiltonian piece

  int split(double dt, int hamind) {
    if (hamind < 1 || hamind > nterms) return set_error(LAT_ERR_ARG, "Undefined Hamiltonian term");
    tg[hamind - 1] += dt;
    if (defrost) {
      if (hamind == 1) ops->push_back({conformal ? 'G' : 'M', dt});
      else if (hamind == 2) ops->push_back({'D', dt});
      else ops->push_back({'K', dt});
    } else {
      if (hamind == 1) ops->push_back({'D', dt});
      else if (hamind == nterms) ops->push_back({'K', dt});
      else ops->push_back({'G', dt});
    }
    return LAT_OK;
  }

  int o2step(double dt, double w1, double w2) {
    int s;
    for (int i = 2; i <= nterms - 1; ++i)
      if ((s = split(w1 * dt / 2.0, i))) return s;
    if ((s = split(w1 * dt, nterms))) return s;
    for (int i = nterms - 1; i >= 2; --i)
      if ((s = split(w1 * dt / 2.0, i))) return s;
    return split((w1 + w2) * dt / 2.0, 1);
  }

  int symp(int order, double dt, int nsteps) {
    int s;
#define LAT_TRY(x) \
  if ((s = (x))) return s
    if (nsteps < 1) return set_error(LAT_ERR_ARG, "nsteps < 1");
    if (order == 2) {
      LAT_TRY(split(dt / 2.0, 1));
      for (int j = 1; j <= nsteps - 1; ++j) LAT_TRY(o2step(dt, 1.0, 1.0));
      return o2step(dt, 1.0, 0.0);
    }
    if (order == 4) {
      const double w1 = 1.0 / (2.0 - std::pow(2.0, 1.0 / 3.0));
      const double w0 = 1.0 - 2.0 * w1;
      LAT_TRY(split(w1 * dt / 2.0, 1));
      for (int j = 1; j <= nsteps; ++j) {
        LAT_TRY(o2step(dt, w1, w0));
        LAT_TRY(o2step(dt, w0, w1));
        LAT_TRY(o2step(dt, w1, j == nsteps ? 0.0 : w1));
      }
      return LAT_OK;
    }
    if (order == 6) {
      // the DEFROST tree's w1 literal has one digit fewer (evolve.f90:159)
      const double w3 = 0.784513610477560, w2 = 0.235573213359357;
      const double w1 = defrost ? -1.17767998417887 : -1.177679984177887;
      const double w0 = 1.0 - 2.0 * (w1 + w2 + w3);
      LAT_TRY(split(w3 * dt / 2.0, 1));
      for (int j = 1; j <= nsteps; ++j) {
        LAT_TRY(o2step(dt, w3, w2)); LAT_TRY(o2step(dt, w2, w1)); LAT_TRY(o2step(dt, w1, w0));
        LAT_TRY(o2step(dt, w0, w1)); LAT_TRY(o2step(dt, w1, w2)); LAT_TRY(o2step(dt, w2, w3));
        LAT_TRY(o2step(dt, w3, j == nsteps ? 0.0 : w3));
      }
      return LAT_OK;
    }
    if (order == 8) {
      if (defrost) return set_error(LAT_ERR_UNSUPPORTED, "the DEFROST symp8 has no coefficients (evolve.f90:180-188)");
      const double w[8] = {0, 0.74167036435061295344822780, -0.40910082580003159399730010,
                           0.19075471029623837995387626, -0.57386247111608226665638733,
                           0.29906418130365592384446354, 0.33462491824529818378495798,
                           0.31529309239676659663205666};
      const double w0 = 1.0 - 2.0 * (w[1] + w[2] + w[3] + w[4] + w[5] + w[6] + w[7]);
      const double W[8] = {w0, w[1], w[2], w[3], w[4], w[5], w[6], w[7]};
      LAT_TRY(split(W[7] * dt / 2.0, 1));
      for (int j = 1; j <= nsteps; ++j) {
        for (int i = 7; i >= 1; --i) LAT_TRY(o2step(dt, W[i], W[i - 1]));
        for (int i = 0; i <= 6; ++i) LAT_TRY(o2step(dt, W[i], W[i + 1]));
        LAT_TRY(o2step(dt, W[7], j == nsteps ? 0.0 : W[7]));
      }
      return LAT_OK;
    }
#undef LAT_TRY
    return set_error(LAT_ERR_ARG, "order must be 2, 4, 6 or 8");
  }
};

}  // namespace lat
