// oracle.cpp -- CPU FP64 restatement of the reference lattice hot path.
//
// TEST INFRASTRUCTURE ONLY.  The GPU engine's results are compared with this
// library's: only the tests, __graft_entry__.smoke() and bench.py's
// CPU-baseline leg load it.  The engine never calls it and has no CPU fallback.
//
// Parity status: the reference is Fortran built against FFTW and MPI; neither
// a Fortran compiler nor FFTW exists in the development environment, and the
// reference ships no tests, golden vectors or fixtures.  Parity against the
// reference binary is therefore UNPINNED.  The restatement is pinned instead
// by analytic known-answer tests (plane-wave Laplacian symbols, exact shell
// mode counts, free-field leapfrog dispersion, integrator order, energy-form
// identities) and by numpy.fft cross-checks of its FFT.
//
// Every routine follows the reference loop it restates, cited file:line
// relative to the reference project root.  Semantics kept exactly:
//  - -r8: every real and literal is FP64 (Pseudospec/openmp_dev/Makefile:80);
//  - symp_o2step with merged half-drifts and the split orders of
//    Pseudospec/openmp_dev/hamiltonian_conformal.f90:50-81 (PSEUDOSPEC) and
//    Discrete/Bubble-Collisions/evolve.f90:98-113,225-240 (DEFROST);
//  - the unnormalised FFT Laplacian followed by /N, fftw_mod.f90:177-207;
//  - the STENCIL macro, Discrete/Bubble-Collisions/macros.h:31-44;
//  - spectrum_3d / crossspec_3d (analysis_spec.f90:59-178) and spectrum_bin
//    (Discrete/Bubble-Collisions/analysis.f90:193-223) binning.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../include/lattice.h"
#include "fft.hpp"

using orc::cplx;

namespace {

thread_local std::string g_err;
int fail(int code, const std::string& msg) { g_err = msg; return code; }

inline int64_t idx3(int x, int y, int z, int nx, int ny) {
  return ((int64_t)z * ny + y) * nx + x;
}
inline int wrap(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }
// folded frequency index, as `if (k<=nn) kk=k-1 else kk=n+1-k` with 1-based k
inline int fold(int i0, int n) { return i0 <= n / 2 ? i0 : n - i0; }

struct Orc {
  lat_config cfg{};
  int nx = 0, ny = 0, nz = 0, nf = 0;
  int64_t N = 0, M = 0;
  double dx = 0, dkx = 0, dky = 0, dkz = 0;
  double c[5] = {0, 0, 0, 0, 0};  // c0,c1,c2,c3,cc
  std::vector<double> fld, fldp;   // [f][z][y][x]
  std::vector<double> u, pu;       // GW [6][z][y][x]
  std::vector<double> pu_next;     // GW kick scratch [6][z][y][x]
  std::vector<double> lap;         // scratch
  std::vector<cplx> Fk;            // scratch
  double a = 1.0, ap = 0.0;
  double tglobal[3] = {0, 0, 0};
  orc::Fft3dReal* fft = nullptr;
};

// ------------------------------------------------------------------ model
// potential / modeldv: hamiltonian_minkowski.f90:161-186 (phi^4),
// Pseudospec/mpi_dev/hamiltonian_conformal_rksplit.f90:220-237 (two field),
// Discrete/Bubble-Collisions/model.f90:117,156 (double well, V not 2V).
double potential(const Orc& o, const double* f) {
  const double* p = o.cfg.model_params;
  switch (o.cfg.model) {
    case LAT_MODEL_PHI4: return 0.25 * p[0] * f[0] * f[0] * f[0] * f[0];
    case LAT_MODEL_PHI4_G2:
      return 0.25 * p[0] * f[0] * f[0] * f[0] * f[0] + 0.5 * p[1] * f[0] * f[0] * f[1] * f[1];
    case LAT_MODEL_DOUBLE_WELL: {
      double s = f[0] * f[0] - 1.0;
      return 0.25 * s * s - p[0] * (f[0] + 1.0);
    }
    case LAT_MODEL_FREE: {
      double v = 0;
      for (int l = 0; l < o.nf; ++l) v += 0.5 * p[0] * f[l] * f[l];
      return v;
    }
  }
  return 0;
}
double modeldv(const Orc& o, const double* f, int l) {
  const double* p = o.cfg.model_params;
  switch (o.cfg.model) {
    case LAT_MODEL_PHI4: return l == 0 ? p[0] * f[0] * f[0] * f[0] : 0.0;
    case LAT_MODEL_PHI4_G2:
      return l == 0 ? p[0] * f[0] * f[0] * f[0] + p[1] * f[0] * f[1] * f[1]
                    : p[1] * f[0] * f[0] * f[1];
    case LAT_MODEL_DOUBLE_WELL: return l == 0 ? (f[0] * f[0] - 1.0) * f[0] - p[0] : 0.0;
    case LAT_MODEL_FREE: return p[0] * f[l];
  }
  return 0;
}

inline void site_fields(const Orc& o, int64_t s, double* f) {
  for (int l = 0; l < o.nf; ++l) f[l] = o.fld[l * o.N + s];
}

// ---------------------------------------------------------------- stencils
// STENCIL(c, LAPLACE): c0 RANK0 + c1 RANK1 + c2 RANK2 + c3 RANK3 in the macro's
// term order, Discrete/Bubble-Collisions/macros.h:31-34.
double stencil_sum(const Orc& o, const double* g, int x, int y, int z) {
  const int nx = o.nx, ny = o.ny, nz = o.nz;
  auto at = [&](int dx_, int dy_, int dz_) {
    return g[idx3(wrap(x + dx_, nx), wrap(y + dy_, ny), wrap(z + dz_, nz), nx, ny)];
  };
  double r0 = at(0, 0, 0);
  double r1 = at(-1, 0, 0) + at(1, 0, 0) + at(0, -1, 0) + at(0, 1, 0) + at(0, 0, -1) + at(0, 0, 1);
  double r2 = 0, r3 = 0;
  if (o.c[2] != 0.0)
    r2 = at(-1, -1, 0) + at(1, -1, 0) + at(-1, 1, 0) + at(1, 1, 0) + at(-1, 0, -1) + at(1, 0, -1) +
         at(-1, 0, 1) + at(1, 0, 1) + at(0, -1, -1) + at(0, 1, -1) + at(0, -1, 1) + at(0, 1, 1);
  if (o.c[3] != 0.0)
    r3 = at(-1, -1, -1) + at(1, -1, -1) + at(-1, 1, -1) + at(1, 1, -1) + at(-1, -1, 1) +
         at(1, -1, 1) + at(-1, 1, 1) + at(1, 1, 1);
  return o.c[0] * r0 + o.c[1] * r1 + o.c[2] * r2 + o.c[3] * r3;
}
// STENCIL(c, GRAD2): sum over the stencil of c_r (g(x+r)-g(x))^2,
// Discrete/Bubble-Collisions/macros.h:28 with homlat.f90:65-90.
double stencil_grad2(const Orc& o, const double* g, int x, int y, int z) {
  const int nx = o.nx, ny = o.ny, nz = o.nz;
  const double g0 = g[idx3(x, y, z, nx, ny)];
  auto d2 = [&](int dx_, int dy_, int dz_) {
    double d = g[idx3(wrap(x + dx_, nx), wrap(y + dy_, ny), wrap(z + dz_, nz), nx, ny)] - g0;
    return d * d;
  };
  double r1 = d2(-1, 0, 0) + d2(1, 0, 0) + d2(0, -1, 0) + d2(0, 1, 0) + d2(0, 0, -1) + d2(0, 0, 1);
  double r2 = 0, r3 = 0;
  if (o.c[2] != 0.0)
    r2 = d2(-1, -1, 0) + d2(1, -1, 0) + d2(-1, 1, 0) + d2(1, 1, 0) + d2(-1, 0, -1) + d2(1, 0, -1) +
         d2(-1, 0, 1) + d2(1, 0, 1) + d2(0, -1, -1) + d2(0, 1, -1) + d2(0, -1, 1) + d2(0, 1, 1);
  if (o.c[3] != 0.0)
    r3 = d2(-1, -1, -1) + d2(1, -1, -1) + d2(-1, 1, -1) + d2(1, 1, -1) + d2(-1, -1, 1) +
         d2(1, -1, 1) + d2(-1, 1, 1) + d2(1, 1, 1);
  return o.c[1] * r1 + o.c[2] * r2 + o.c[3] * r3;
}

// Laplacian of g into out with the configured operator (no 1/a^2 factor).
// Spectral: laplacian_3d, fftw_mod.f90:177-207 -- r2c, multiply by
// -(ii^2 dk^2 + jj^2 dk^2 + kk^2 dk^2) with folded indices, c2r, divide by N.
void laplacian(Orc& o, const double* g, double* out) {
  if (o.cfg.laplacian == LAT_LAP_SPECTRAL) {
    o.fft->r2c(g, o.Fk.data());
    const int hx = o.nx / 2 + 1;
#pragma omp parallel for schedule(static)
    for (int z = 0; z < o.nz; ++z) {
      int kk = fold(z, o.nz);
      for (int y = 0; y < o.ny; ++y) {
        int jj = fold(y, o.ny);
        for (int x = 0; x < hx; ++x) {
          double rad2 = (double)x * x * o.dkx * o.dkx + (double)jj * jj * o.dky * o.dky +
                        (double)kk * kk * o.dkz * o.dkz;
          o.Fk[((int64_t)z * o.ny + y) * hx + x] *= -rad2;
        }
      }
    }
    o.fft->c2r(o.Fk.data(), out);
    const double inv = 1.0 / (double)o.nx / (double)o.ny / (double)o.nz;
#pragma omp parallel for schedule(static)
    for (int64_t s = 0; s < o.N; ++s) out[s] *= inv;
    return;
  }
  const double elap = 1.0 / (o.dx * o.dx) / o.c[4];
#pragma omp parallel for schedule(static)
  for (int z = 0; z < o.nz; ++z)
    for (int y = 0; y < o.ny; ++y)
      for (int x = 0; x < o.nx; ++x) out[idx3(x, y, z, o.nx, o.ny)] = stencil_sum(o, g, x, y, z) * elap;
}

bool conformal(const Orc& o) { return o.cfg.background == LAT_BG_CONFORMAL; }

// --------------------------------------------------------- Hamiltonian pieces
// Hamiltonian_fields_kin: Minkowski hamiltonian_minkowski.f90:86-100,
// conformal hamiltonian_conformal.f90:92-118.
void fields_kin(Orc& o, double dt) {
  if (!conformal(o)) {
    const int64_t T = o.nf * o.N;
#pragma omp parallel for schedule(static)
    for (int64_t s = 0; s < T; ++s) o.fld[s] += dt * o.fldp[s];
    if (o.cfg.gw) {
      const int64_t G = 6 * o.N;
#pragma omp parallel for schedule(static)
      for (int64_t s = 0; s < G; ++s) o.u[s] += dt * o.pu[s];
    }
    return;
  }
  const double a2 = o.a * o.a;
  double KE2 = 0;
  const int64_t T = o.nf * o.N;
#pragma omp parallel for schedule(static) reduction(+ : KE2)
  for (int64_t s = 0; s < T; ++s) {
    o.fld[s] = o.fld[s] + dt * o.fldp[s] / a2;
    KE2 += o.fldp[s] * o.fldp[s];
  }
  KE2 = KE2 / (double)o.N;
  o.ap = o.ap + dt * KE2 / (o.a * o.a * o.a);
}

// Hamiltonian_grav_kinetic, hamiltonian_conformal.f90:86-90 (also the
// DEFROST Hamiltonian_metric_kin, Discrete/Bubble-Collisions/evolve.f90:497-500).
void grav_kin(Orc& o, double dt) { o.a = o.a - dt * o.ap / 6.0; }

// GW source d_i phi d_j phi with central differences, all six components at
// one site in the order 11,22,33,12,13,23 (the reference's gw_source_* are
// empty stubs, grav-waves/evolve-gw.f90:21-36).  Each component sums the
// fields in order, so the result does not depend on how many are computed.
const int kGwI[6] = {0, 1, 2, 0, 0, 1};
const int kGwJ[6] = {0, 1, 2, 1, 2, 2};
void gw_sources(const Orc& o, int x, int y, int z, double* src) {
  const double inv2dx = 1.0 / (2.0 * o.dx);
  for (int cc = 0; cc < 6; ++cc) src[cc] = 0;
  for (int l = 0; l < o.nf; ++l) {
    const double* g = &o.fld[l * o.N];
    double d[3];
    d[0] = (g[idx3(wrap(x + 1, o.nx), y, z, o.nx, o.ny)] - g[idx3(wrap(x - 1, o.nx), y, z, o.nx, o.ny)]) * inv2dx;
    d[1] = (g[idx3(x, wrap(y + 1, o.ny), z, o.nx, o.ny)] - g[idx3(x, wrap(y - 1, o.ny), z, o.nx, o.ny)]) * inv2dx;
    d[2] = (g[idx3(x, y, wrap(z + 1, o.nz), o.nx, o.ny)] - g[idx3(x, y, wrap(z - 1, o.nz), o.nx, o.ny)]) * inv2dx;
    for (int cc = 0; cc < 6; ++cc) src[cc] += d[kGwI[cc]] * d[kGwJ[cc]];
  }
}

// Hamiltonian_fields_grad_pot: spectral hamiltonian_conformal.f90:128-174
// (Minkowski hamiltonian_minkowski.f90:111-136); FD conformal
// hamiltonian_conformal.f90:176-196; FD Minkowski
// Discrete/Bubble-Collisions/evolve.f90:255-281.
void fields_grad_pot(Orc& o, double dt) {
  const bool conf = conformal(o);
  const double a = conf ? o.a : 1.0;
  const double a2 = a * a, a4 = a2 * a2;
  double GE2 = 0, PE = 0;
  // the GW kick reads phi before the field kick changes pi (phi is unchanged by a kick)
  if (o.cfg.gw) {
    const double elap = 1.0 / (o.dx * o.dx) / o.c[4];
    const double kap = o.cfg.gw_coupling;
    std::vector<double>& newpu = o.pu_next;
    newpu.resize(6 * o.N);
#pragma omp parallel for schedule(static)
    for (int z = 0; z < o.nz; ++z)
      for (int y = 0; y < o.ny; ++y)
        for (int x = 0; x < o.nx; ++x) {
          const int64_t s = idx3(x, y, z, o.nx, o.ny);
          double src[6];
          gw_sources(o, x, y, z, src);
          for (int cc = 0; cc < 6; ++cc) {
            double lu = stencil_sum(o, &o.u[cc * o.N], x, y, z) * elap;
            newpu[cc * o.N + s] = o.pu[cc * o.N + s] + dt * (lu + kap * src[cc]);
          }
        }
    o.pu.swap(newpu);
  }
  for (int l = 0; l < o.nf; ++l) {
    laplacian(o, &o.fld[l * o.N], o.lap.data());
    double ge = 0;
#pragma omp parallel for schedule(static) reduction(+ : ge)
    for (int64_t s = 0; s < o.N; ++s) {
      double f[4];
      site_fields(o, s, f);
      const double lp = o.lap[s];
      if (o.cfg.laplacian == LAT_LAP_SPECTRAL) {
        o.fldp[l * o.N + s] = o.fldp[l * o.N + s] + dt * (a2 * lp - a4 * modeldv(o, f, l));
        ge -= f[l] * lp;
      } else {
        // the FD kick folds 1/a^2 into the Laplacian: fldp += a^4 dt (lap/a^2 - V')
        const double lpa = lp / a2;
        o.fldp[l * o.N + s] = o.fldp[l * o.N + s] + a4 * dt * (lpa - modeldv(o, f, l));
        ge -= f[l] * lpa;
      }
    }
    GE2 += ge;
  }
  if (!conf) return;
#pragma omp parallel for schedule(static) reduction(+ : PE)
  for (int64_t s = 0; s < o.N; ++s) {
    double f[4];
    site_fields(o, s, f);
    PE += potential(o, f);
  }
  if (o.cfg.laplacian == LAT_LAP_SPECTRAL) GE2 = GE2 / a2;  // hamiltonian_conformal.f90:172
  PE = PE / (double)o.N;
  GE2 = GE2 / (double)o.N;
  o.ap = o.ap - a * a * a * (GE2 + 4.0 * PE) * dt;
}

int n_terms(const Orc& o) {
  if (o.cfg.split_order == LAT_SPLIT_DEFROST) return 3;
  return conformal(o) ? 3 : 2;
}

// Hamiltonian_Split(dt, hamind)
int split(Orc& o, double dt, int hamind) {
  if (hamind < 1 || hamind > n_terms(o)) return fail(LAT_ERR_ARG, "Undefined Hamiltonian term");
  o.tglobal[hamind - 1] += dt;
  if (o.cfg.split_order == LAT_SPLIT_DEFROST) {
    if (hamind == 1) { if (conformal(o)) grav_kin(o, dt); }
    else if (hamind == 2) fields_kin(o, dt);
    else fields_grad_pot(o, dt);
    return LAT_OK;
  }
  if (hamind == 1) fields_kin(o, dt);
  else if (hamind == n_terms(o)) fields_grad_pot(o, dt);
  else grav_kin(o, dt);
  return LAT_OK;
}

// symp_o2step, hamiltonian_conformal.f90:50-64
void o2step(Orc& o, double dt, double w1, double w2) {
  const int nt = n_terms(o);
  for (int i = 2; i <= nt - 1; ++i) split(o, w1 * dt / 2.0, i);
  split(o, w1 * dt, nt);
  for (int i = nt - 1; i >= 2; --i) split(o, w1 * dt / 2.0, i);
  split(o, (w1 + w2) * dt / 2.0, 1);
}

// symp2/4/6/8: Pseudospec/openmp_dev/evolve_spectral.f90:129-227 (PSEUDOSPEC
// order) and Discrete/Bubble-Collisions/evolve.f90:118-223 (DEFROST order,
// whose symp6 w1 literal has one digit fewer and whose symp8 weights are 0).
int symp(Orc& o, int order, double dt, int nsteps) {
  const bool df = o.cfg.split_order == LAT_SPLIT_DEFROST;
  if (nsteps < 1) return fail(LAT_ERR_ARG, "nsteps < 1");
  if (order == 2) {
    split(o, dt / 2.0, 1);
    for (int j = 1; j <= nsteps - 1; ++j) o2step(o, dt, 1.0, 1.0);
    o2step(o, dt, 1.0, 0.0);
    return LAT_OK;
  }
  if (order == 4) {
    const double w1 = 1.0 / (2.0 - std::pow(2.0, 1.0 / 3.0));
    const double w0 = 1.0 - 2.0 * w1;
    split(o, w1 * dt / 2.0, 1);
    for (int j = 1; j <= nsteps; ++j) {
      o2step(o, dt, w1, w0);
      o2step(o, dt, w0, w1);
      o2step(o, dt, w1, j == nsteps ? 0.0 : w1);
    }
    return LAT_OK;
  }
  if (order == 6) {
    const double w3 = 0.784513610477560, w2 = 0.235573213359357;
    const double w1 = df ? -1.17767998417887 : -1.177679984177887;
    const double w0 = 1.0 - 2.0 * (w1 + w2 + w3);
    split(o, w3 * dt / 2.0, 1);
    for (int j = 1; j <= nsteps; ++j) {
      o2step(o, dt, w3, w2); o2step(o, dt, w2, w1); o2step(o, dt, w1, w0);
      o2step(o, dt, w0, w1); o2step(o, dt, w1, w2); o2step(o, dt, w2, w3);
      o2step(o, dt, w3, j == nsteps ? 0.0 : w3);
    }
    return LAT_OK;
  }
  if (order == 8) {
    if (df) return fail(LAT_ERR_UNSUPPORTED, "DEFROST symp8 has no coefficients (evolve.f90:180-188)");
    const double w[8] = {0, 0.74167036435061295344822780, -0.40910082580003159399730010,
                         0.19075471029623837995387626, -0.57386247111608226665638733,
                         0.29906418130365592384446354, 0.33462491824529818378495798,
                         0.31529309239676659663205666};
    double w0 = 1.0 - 2.0 * (w[1] + w[2] + w[3] + w[4] + w[5] + w[6] + w[7]);
    double W[8] = {w0, w[1], w[2], w[3], w[4], w[5], w[6], w[7]};
    split(o, W[7] * dt / 2.0, 1);
    for (int j = 1; j <= nsteps; ++j) {
      for (int i = 7; i >= 1; --i) o2step(o, dt, W[i], W[i - 1]);
      for (int i = 0; i <= 6; ++i) o2step(o, dt, W[i], W[i + 1]);
      o2step(o, dt, W[7], j == nsteps ? 0.0 : W[7]);
    }
    return LAT_OK;
  }
  return fail(LAT_ERR_ARG, "order must be 2, 4, 6 or 8");
}

// ---------------------------------------------------------------- energies
// dump_rho, evolve_spectral.f90:305-415; homlat.f90:65-188.
void energies(Orc& o, double* out) {
  const bool conf = conformal(o);
  const double a = conf ? o.a : 1.0;
  double KE = 0, PE = 0, GE = 0, GG = 0, m0 = 0, m1 = 0;
  const int64_t T = o.nf * o.N;
#pragma omp parallel for schedule(static) reduction(+ : KE)
  for (int64_t s = 0; s < T; ++s) KE += o.fldp[s] * o.fldp[s];
#pragma omp parallel for schedule(static) reduction(+ : PE, m0, m1)
  for (int64_t s = 0; s < o.N; ++s) {
    double f[4] = {0, 0, 0, 0};
    site_fields(o, s, f);
    PE += potential(o, f);
    m0 += f[0];
    if (o.nf > 1) m1 += f[1];
  }
  for (int l = 0; l < o.nf; ++l) {
    const double* g = &o.fld[l * o.N];
    laplacian(o, g, o.lap.data());
    double ge = 0;
#pragma omp parallel for schedule(static) reduction(+ : ge)
    for (int64_t s = 0; s < o.N; ++s) ge -= g[s] * o.lap[s];
    GE += ge;
    if (o.cfg.laplacian != LAT_LAP_SPECTRAL) {
      double gg = 0;
#pragma omp parallel for schedule(static) reduction(+ : gg)
      for (int z = 0; z < o.nz; ++z)
        for (int y = 0; y < o.ny; ++y)
          for (int x = 0; x < o.nx; ++x) gg += stencil_grad2(o, g, x, y, z);
      GG += gg;
    }
  }
  const double Nd = (double)o.N;
  const double knorm = conf ? 1.0 / std::pow(a, 6) : 1.0;
  out[LAT_E_KE] = 0.5 * KE * knorm / Nd;
  out[LAT_E_GE_LAP] = 0.5 * GE / Nd / (a * a);
  out[LAT_E_GE_GRAD] = o.cfg.laplacian == LAT_LAP_SPECTRAL
                           ? out[LAT_E_GE_LAP]
                           : 0.25 / (a * o.dx) / (a * o.dx) / o.c[4] * GG / Nd;
  out[LAT_E_PE] = PE / Nd;
  out[LAT_E_RHO] = out[LAT_E_KE] + out[LAT_E_GE_LAP] + out[LAT_E_PE];
  double H = conf ? -o.ap / 6.0 / (a * a) : 0.0;
  out[LAT_E_GRAV] = -3.0 * H * H;
  out[LAT_E_RESIDUAL] = (out[LAT_E_RHO] + out[LAT_E_GRAV]) / out[LAT_E_RHO];
  out[LAT_E_A] = a;
  out[LAT_E_AP] = conf ? o.ap : 0.0;
  out[LAT_E_MEAN0] = m0 / Nd;
  out[LAT_E_MEAN1] = m1 / Nd;
  out[LAT_E_GW] = 0;
  if (o.cfg.gw) {
    double eg = 0;
    for (int cc = 0; cc < 6; ++cc) {
      const double wt = cc < 3 ? 1.0 : 2.0;
      laplacian(o, &o.u[cc * o.N], o.lap.data());
      double k = 0, g = 0;
#pragma omp parallel for schedule(static) reduction(+ : k, g)
      for (int64_t s = 0; s < o.N; ++s) {
        k += o.pu[cc * o.N + s] * o.pu[cc * o.N + s];
        g -= o.u[cc * o.N + s] * o.lap[s];
      }
      eg += wt * 0.5 * (k + g);
    }
    out[LAT_E_GW] = eg / Nd;
  }
}

// calc_metric, hamiltonian_conformal.f90:263-304
void calc_metric(Orc& o) {
  double e[LAT_NENERGY];
  energies(o, e);
  o.ap = -std::sqrt(o.a * o.a * o.a * o.a * 12.0 * e[LAT_E_RHO]);
}

// ----------------------------------------------------------------- spectra
int nbins_ref(const Orc& o) {
  int ns = (o.nx / 2 + 1) * (o.nx / 2 + 1) + (o.ny / 2 + 1) * (o.ny / 2 + 1) + (o.nz / 2 + 1) * (o.nz / 2 + 1);
  return (int)std::floor(std::sqrt((double)ns + 1.0));  // analysis_spec.f90:55-56
}

// Binning of a half spectrum: the reference loops i = 1..n1 over the full x
// range with folded ii and reads Fk(ii+1,j,k), which visits each interior kx
// plane twice (analysis_spec.f90:87-99).  `val(x,y,z)` gives the summand.
template <class F>
void bin_half(const Orc& o, int mode, int nbins, double* S, double* W, F val) {
  std::vector<double> s(nbins + 2, 0.0), w(nbins + 2, 0.0);
  const int hx = o.nx / 2 + 1;
  for (int z = 0; z < o.nz; ++z) {
    int kk = fold(z, o.nz);
    for (int y = 0; y < o.ny; ++y) {
      int jj = fold(y, o.ny);
      for (int i = 0; i < o.nx; ++i) {
        int ii = fold(i, o.nx);
        (void)hx;
        const double v = val(ii, y, z);
        const double p = std::sqrt((double)(ii * ii + jj * jj + kk * kk));
        const int l = (int)std::floor(p);
        if (mode == LAT_SPEC_WEIGHTED) {
          const double d0 = (double)l - p, d1 = (double)(l + 1) - p;
          const double c0 = (1.0 - d0 * d0) * (1.0 - d0 * d0);
          const double c1 = (1.0 - d1 * d1) * (1.0 - d1 * d1);
          if (l < nbins) { s[l] += c0 * v; w[l] += c0; }
          if (l + 1 < nbins) { s[l + 1] += c1 * v; w[l + 1] += c1; }
        } else {
          if (l < nbins) { s[l] += v; w[l] += 1.0; }
        }
      }
    }
  }
  for (int l = 0; l < nbins; ++l) {
    S[l] = w[l] != 0.0 ? s[l] / w[l] : s[l];
    W[l] = w[l];
  }
}

const double* spec_src(const Orc& o, int what, int field) {
  return what == LAT_SPEC_FLD ? &o.fld[field * o.N] : &o.fldp[field * o.N];
}

}  // namespace

// =================================================================== C ABI
extern "C" {

typedef struct Orc orc_t;

const char* orc_last_error(void) { return g_err.c_str(); }

int orc_create(orc_t** out, const lat_config* cfg) {
  if (!out || !cfg) return fail(LAT_ERR_ARG, "null argument");
  if (cfg->nx < 2 || cfg->ny < 2 || cfg->nz < 2 || cfg->nfld < 1 || cfg->nfld > 4 || cfg->len <= 0)
    return fail(LAT_ERR_ARG, "bad lattice shape");
  if (cfg->model == LAT_MODEL_PHI4_G2 && cfg->nfld != 2) return fail(LAT_ERR_ARG, "two-field model needs nfld = 2");
  if (cfg->gw && (cfg->laplacian == LAT_LAP_SPECTRAL || cfg->background != LAT_BG_MINKOWSKI))
    return fail(LAT_ERR_UNSUPPORTED, "GW evolution needs an FD stencil and Minkowski background");
  Orc* o = new Orc();
  o->cfg = *cfg;
  o->nx = cfg->nx; o->ny = cfg->ny; o->nz = cfg->nz; o->nf = cfg->nfld;
  o->N = (int64_t)o->nx * o->ny * o->nz;
  o->M = (int64_t)(o->nx / 2 + 1) * o->ny * o->nz;
  o->dx = cfg->len / cfg->nx;
  const double twopi = 6.2831853071795864769252867665590;
  o->dkx = twopi / (o->nx * o->dx);
  o->dky = twopi / (o->ny * o->dx);
  o->dkz = twopi / (o->nz * o->dx);
  bool zero = true;
  for (int i = 0; i < 5; ++i) zero = zero && cfg->stencil[i] == 0.0;
  if (zero) {
    if (cfg->laplacian == LAT_LAP_FD7) { o->c[0] = -6; o->c[1] = 1; o->c[2] = 0; o->c[3] = 0; o->c[4] = 1; }
    else { o->c[0] = -128; o->c[1] = 14; o->c[2] = 3; o->c[3] = 1; o->c[4] = 30; }
  } else {
    for (int i = 0; i < 5; ++i) o->c[i] = cfg->stencil[i];
  }
  o->fld.assign(o->nf * o->N, 0.0);
  o->fldp.assign(o->nf * o->N, 0.0);
  if (cfg->gw) { o->u.assign(6 * o->N, 0.0); o->pu.assign(6 * o->N, 0.0); }
  o->lap.assign(o->N, 0.0);
  o->Fk.assign(o->M, cplx(0, 0));
  o->fft = new orc::Fft3dReal(o->nx, o->ny, o->nz);
  *out = o;
  return LAT_OK;
}

int orc_destroy(orc_t* o) {
  if (!o) return LAT_OK;
  delete o->fft;
  delete o;
  return LAT_OK;
}

// state in SoA [field][z][y][x] (not the Fortran AoS layout)
int orc_set_state(orc_t* o, const double* fld, const double* fldp) {
  if (fld) std::memcpy(o->fld.data(), fld, sizeof(double) * o->nf * o->N);
  if (fldp) std::memcpy(o->fldp.data(), fldp, sizeof(double) * o->nf * o->N);
  return LAT_OK;
}
int orc_get_state(orc_t* o, double* fld, double* fldp) {
  if (fld) std::memcpy(fld, o->fld.data(), sizeof(double) * o->nf * o->N);
  if (fldp) std::memcpy(fldp, o->fldp.data(), sizeof(double) * o->nf * o->N);
  return LAT_OK;
}
int orc_gw_set(orc_t* o, const double* u, const double* pu) {
  if (!o->cfg.gw) return fail(LAT_ERR_STATE, "no GW arrays");
  if (u) std::memcpy(o->u.data(), u, sizeof(double) * 6 * o->N);
  if (pu) std::memcpy(o->pu.data(), pu, sizeof(double) * 6 * o->N);
  return LAT_OK;
}
int orc_gw_get(orc_t* o, double* u, double* pu) {
  if (!o->cfg.gw) return fail(LAT_ERR_STATE, "no GW arrays");
  if (u) std::memcpy(u, o->u.data(), sizeof(double) * 6 * o->N);
  if (pu) std::memcpy(pu, o->pu.data(), sizeof(double) * 6 * o->N);
  return LAT_OK;
}

int orc_set_scale_factor(orc_t* o, double a, double ap) { o->a = a; o->ap = ap; return LAT_OK; }
int orc_get_scale_factor(orc_t* o, double* a, double* ap) { *a = o->a; *ap = o->ap; return LAT_OK; }
int orc_get_time(orc_t* o, double* t) { for (int i = 0; i < 3; ++i) t[i] = o->tglobal[i]; return LAT_OK; }
int orc_calc_metric(orc_t* o) { calc_metric(*o); return LAT_OK; }

int orc_split(orc_t* o, double dt, int32_t hamind) { return split(*o, dt, hamind); }
int orc_o2step(orc_t* o, double dt, double w1, double w2) { o2step(*o, dt, w1, w2); return LAT_OK; }
int orc_symp(orc_t* o, int32_t order, double dt, int32_t nsteps) { return symp(*o, order, dt, nsteps); }

int orc_laplacian(orc_t* o, int32_t field, double* out) {
  if (field < 0 || field >= o->nf) return fail(LAT_ERR_ARG, "bad field");
  laplacian(*o, &o->fld[field * o->N], out);
  return LAT_OK;
}
int orc_energies(orc_t* o, double* out) { energies(*o, out); return LAT_OK; }

// LOG.out's rhoball (Discrete/Bubble-Collisions/iofile.f90:523-567): over
// the sites with ((i - n/2)^2 + (j - n/2)^2 + (k - n/2)^2) dx^2 < r2
// (1-based indices) the sums of (sum_f fldp_f)^2, STENCIL(c, GRAD2) summed
// over the fields, and V, into out[0..2].
int orc_rho_ball_sums(orc_t* o, double r2, double* out) {
  double T = 0, G = 0, V = 0;
  for (int z = 0; z < o->nz; ++z)
    for (int y = 0; y < o->ny; ++y)
      for (int x = 0; x < o->nx; ++x) {
        const double bx = x + 1 - o->nx / 2, by = y + 1 - o->ny / 2, bz = z + 1 - o->nz / 2;
        if ((bx * bx + by * by + bz * bz) * o->dx * o->dx >= r2) continue;
        const int64_t s = idx3(x, y, z, o->nx, o->ny);
        double psum = 0, f[8];
        for (int l = 0; l < o->nf; ++l) {
          psum += o->fldp[l * o->N + s];
          G += stencil_grad2(*o, &o->fld[l * o->N], x, y, z);
        }
        T += psum * psum;
        site_fields(*o, s, f);
        V += potential(*o, f);
      }
  out[0] = T;
  out[1] = G;
  out[2] = V;
  return LAT_OK;
}
int orc_spectrum_nbins(orc_t* o, int32_t* ns) { *ns = nbins_ref(*o); return LAT_OK; }

int orc_spectrum(orc_t* o, int32_t what, int32_t field, int32_t mode, int32_t nbins, double* S, double* W) {
  if (field < 0 || field >= o->nf || nbins < 1) return fail(LAT_ERR_ARG, "bad spectrum args");
  o->fft->r2c(spec_src(*o, what, field), o->Fk.data());
  const int hx = o->nx / 2 + 1;
  const cplx* F = o->Fk.data();
  bin_half(*o, mode, nbins, S, W, [&](int ii, int y, int z) {
    return std::norm(F[((int64_t)z * o->ny + y) * hx + ii]);
  });
  return LAT_OK;
}

int orc_crossspec(orc_t* o, int32_t what1, int32_t f1, int32_t what2, int32_t f2, int32_t nbins,
                  double* Sre, double* Sim) {
  std::vector<cplx> F1(o->M);
  o->fft->r2c(spec_src(*o, what1, f1), F1.data());
  o->fft->r2c(spec_src(*o, what2, f2), o->Fk.data());
  const int hx = o->nx / 2 + 1;
  std::vector<double> W(nbins);
  const cplx* F2 = o->Fk.data();
  auto at = [&](int ii, int y, int z) { return ((int64_t)z * o->ny + y) * hx + ii; };
  bin_half(*o, LAT_SPEC_WEIGHTED, nbins, Sre, W.data(), [&](int ii, int y, int z) {
    return (F1[at(ii, y, z)] * std::conj(F2[at(ii, y, z)])).real();
  });
  bin_half(*o, LAT_SPEC_WEIGHTED, nbins, Sim, W.data(), [&](int ii, int y, int z) {
    return (F1[at(ii, y, z)] * std::conj(F2[at(ii, y, z)])).imag();
  });
  return LAT_OK;
}

// TT-projected GW spectrum of pi_ij with the lattice momentum of the central
// difference, k_i = sin(2 pi n_i / N_i)/dx; Lambda = P pi P - P tr(P pi)/2.
int orc_gw_spectrum(orc_t* o, int32_t nbins, double* S, double* W) {
  if (!o->cfg.gw) return fail(LAT_ERR_STATE, "no GW arrays");
  std::vector<std::vector<cplx>> F(6, std::vector<cplx>(o->M));
  for (int cc = 0; cc < 6; ++cc) o->fft->r2c(&o->pu[cc * o->N], F[cc].data());
  const int hx = o->nx / 2 + 1;
  const double twopi = 6.2831853071795864769252867665590;
  bin_half(*o, LAT_SPEC_COUNT, nbins, S, W, [&](int ii, int y, int z) {
    int64_t m = ((int64_t)z * o->ny + y) * hx + ii;
    double k[3] = {std::sin(twopi * ii / o->nx) / o->dx, std::sin(twopi * y / o->ny) / o->dx,
                   std::sin(twopi * z / o->nz) / o->dx};
    double k2 = k[0] * k[0] + k[1] * k[1] + k[2] * k[2];
    if (k2 == 0.0) return 0.0;
    double P[3][3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) P[i][j] = (i == j ? 1.0 : 0.0) - k[i] * k[j] / k2;
    cplx h[3][3];
    const int map[3][3] = {{0, 3, 4}, {3, 1, 5}, {4, 5, 2}};
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) h[i][j] = F[map[i][j]][m];
    cplx PhP[3][3];
    cplx tr = 0;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        cplx acc = 0;
        for (int l = 0; l < 3; ++l)
          for (int mm = 0; mm < 3; ++mm) acc += P[i][l] * h[l][mm] * P[mm][j];
        PhP[i][j] = acc;
      }
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) tr += P[i][j] * h[j][i];
    double sum = 0;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) sum += std::norm(PhP[i][j] - 0.5 * P[i][j] * tr);
    return sum;
  });
  return LAT_OK;
}

// ------------------------------------------------------ initial conditions
// Counter-based draw shared with the engine: splitmix64 finaliser chained over
// (seed, field, mode index), uniforms in (0,1], Box-Muller.
static inline uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
static inline double u01(uint64_t r) { return ((double)(r >> 11) + 1.0) * (1.0 / 9007199254740992.0); }

int orc_mode_gauss(uint64_t seed, int32_t field, int64_t mode, double* g) {
  uint64_t key = mix64(mix64(mix64(seed) ^ (uint64_t)field) ^ (uint64_t)mode);
  double u1 = u01(mix64(key ^ 1ULL)), u2 = u01(mix64(key ^ 2ULL));
  double r = std::sqrt(-2.0 * std::log(u1));
  double th = 6.2831853071795864769252867665590 * u2;
  g[0] = r * std::cos(th);
  g[1] = r * std::sin(th);
  return LAT_OK;
}

int orc_init_vacuum(orc_t* o, uint64_t seed, const double* fld0, const double* dfld0, const double* m2eff,
                    double amp, double kcut_frac) {
  const int hx = o->nx / 2 + 1;
  const double twopi = 6.2831853071795864769252867665590;
  const double V = o->nx * o->dx * o->ny * o->dx * o->nz * o->dx;
  const double Nd = (double)o->N;
  const double kcut = kcut_frac * (twopi / 2.0) / o->dx;
  std::vector<cplx> Fp(o->M);
  for (int l = 0; l < o->nf; ++l) {
#pragma omp parallel for schedule(static)
    for (int z = 0; z < o->nz; ++z)
      for (int y = 0; y < o->ny; ++y)
        for (int x = 0; x < hx; ++x) {
          int64_t m = ((int64_t)z * o->ny + y) * hx + x;
          int jj = fold(y, o->ny), kk = fold(z, o->nz);
          double k2 = (double)x * x * o->dkx * o->dkx + (double)jj * jj * o->dky * o->dky +
                      (double)kk * kk * o->dkz * o->dkz;
          cplx F(0, 0), P(0, 0);
          double kmag = std::sqrt(k2);
          if (k2 > 0.0 && kmag <= kcut) {
            double w = std::sqrt(k2 + m2eff[l]);
            double sig = std::sqrt(amp * Nd * Nd / (2.0 * V * w));
            // Hermitian partner inside the kx = 0 and kx = nx/2 planes
            bool selfplane = (x == 0) || (2 * x == o->nx);
            int64_t mp = ((int64_t)((o->nz - z) % o->nz) * o->ny + (o->ny - y) % o->ny) * hx + x;
            double g[2];
            // pi_k = -i w F_k for the drawing member of a pair (a wave travelling
            // along +k); its Hermitian partner carries the conjugate, +i w F, and a
            // self-conjugate mode (a standing wave) gets no momentum.
            if (selfplane && mp == m) {
              orc_mode_gauss(seed, l, m, g);
              F = cplx(sig * g[0], 0.0);
              P = cplx(0, 0);
            } else if (selfplane && mp < m) {
              orc_mode_gauss(seed, l, mp, g);
              F = std::conj(cplx(sig * g[0], sig * g[1]) * std::sqrt(0.5));
              P = cplx(0, w) * F;
            } else {
              orc_mode_gauss(seed, l, m, g);
              F = cplx(sig * g[0], sig * g[1]) * std::sqrt(0.5);
              P = cplx(0, -w) * F;
            }
          }
          o->Fk[m] = F;
          Fp[m] = P;
        }
    double* f = &o->fld[l * o->N];
    double* p = &o->fldp[l * o->N];
    o->fft->c2r(o->Fk.data(), f);
    o->fft->c2r(Fp.data(), p);
#pragma omp parallel for schedule(static)
    for (int64_t s = 0; s < o->N; ++s) {
      f[s] = fld0[l] + f[s] / Nd;
      p[s] = dfld0[l] + p[s] / Nd;
    }
  }
  return LAT_OK;
}

// The reference's sample(gamma, m2eff) (Pseudospec/openmp_dev/evolve_spectral.f90:
// 421-506): a radial profile ker(k) = k (k^2 + m2eff)^gamma exp(-(k/kcut)^2) on
// an oversampled grid (os = 16, nos = n os^2 points, dk/(2 os) apart), its
// DST-II (FFTW RODFT10: Y_k = 2 sum_j X_j sin(pi (j + 1/2)(k + 1)/nos), here
// summed directly), scaled by norm / k, interpolated linearly onto the
// radius |(i, j, k) - nn| os of every site about the grid centre
// nn = n/2 + 1 (1-based), transformed (r2c), every half-spectrum mode times
// Box-Muller noise sqrt(-2 ln a) e^{2 pi i p}, and transformed back
// (unnormalised).  The noise is the counter-based draw of orc_mode_gauss on
// stream 0x5300 + 2 field + (0 field, 1 momentum) (Fortran's random_number
// cannot be reproduced); the kx = 0 and kx = nx/2 planes are projected onto
// their Hermitian part before the inverse transform (a c2r of non-Hermitian
// input is FFT-library defined).  Cubic lattices; norm uses mpl.
static void sample_field(orc_t* o, uint64_t seed, int stream, double gamma, double m2eff, double mpl, double* out) {
  const int n = o->nx, os = 16, nos = n * os * os, nn = n / 2 + 1, hx = n / 2 + 1;
  const double twopi = 6.2831853071795864769252867665590, pi = twopi / 2;
  const double dx = o->dx, dk = twopi / (n * dx), dxos = dx / os, dkos = dk / (2.0 * os);
  const double kcut = (double)nn * dk / 2.0;
  const double nvol = (double)n * n * n;
  const double norm = 0.5 / (nvol * std::sqrt(twopi * dk * dk * dk) * mpl) * (dkos / dxos);
  std::vector<double> X(nos), ker(nos);
  for (int j = 0; j < nos; ++j) {
    const double kk = (j + 0.5) * dkos;
    X[j] = kk * std::pow(kk * kk + m2eff, gamma) * std::exp(-(kk / kcut) * (kk / kcut));
  }
#pragma omp parallel for schedule(static)
  for (int k = 0; k < nos; ++k) {
    double y = 0.0;
    // angle pi (2j + 1)(k + 1) / (2 nos), reduced modulo 2 pi in integers
    for (int j = 0; j < nos; ++j)
      y += X[j] * std::sin(pi * (double)(((int64_t)(2 * j + 1) * (k + 1)) % (4 * (int64_t)nos)) / (2.0 * nos));
    ker[k] = norm * (2.0 * y) / (k + 1);  // ker(k + 1) of the 1-based profile
  }
  std::vector<double> f(o->N);
#pragma omp parallel for schedule(static)
  for (int z = 0; z < n; ++z)
    for (int y = 0; y < n; ++y)
      for (int x = 0; x < n; ++x) {
        const double di = x + 1 - nn, dj = y + 1 - nn, dz = z + 1 - nn;
        const double kk = std::sqrt(di * di + dj * dj + dz * dz) * os;
        const int l = (int)std::floor(kk);
        f[idx3(x, y, z, n, n)] = l > 0 ? ker[l - 1] + (kk - l) * (ker[l] - ker[l - 1]) : (4.0 * ker[0] - ker[1]) / 3.0;
      }
  std::vector<cplx> F(o->M);
  o->fft->r2c(f.data(), F.data());
  for (int64_t m = 0; m < o->M; ++m) {
    double g[2];
    orc_mode_gauss(seed, stream, m, g);
    F[m] *= cplx(g[0], g[1]);
  }
  for (int z = 0; z < n; ++z)
    for (int y = 0; y < n; ++y)
      for (int x = 0; x < hx; x += (n / 2 > 0 ? n / 2 : 1)) {
        if (x != 0 && 2 * x != n) continue;
        const int64_t m = ((int64_t)z * n + y) * hx + x;
        const int64_t mp = ((int64_t)((n - z) % n) * n + (n - y) % n) * hx + x;
        if (mp < m) continue;
        const cplx h = 0.5 * (F[m] + std::conj(F[mp]));
        F[m] = h;
        F[mp] = std::conj(h);
      }
  o->fft->c2r(F.data(), out);
}

int orc_init_sample(orc_t* o, uint64_t seed, const double* fld0, const double* dfld0, double m2eff, double mpl) {
  if (o->nx != o->ny || o->nx != o->nz) return LAT_ERR_UNSUPPORTED;
  for (int l = 0; l < o->nf; ++l) {
    double* f = &o->fld[l * o->N];
    double* p = &o->fldp[l * o->N];
    sample_field(o, seed, 0x5300 + 2 * l, -0.25, m2eff, mpl, f);
    sample_field(o, seed, 0x5300 + 2 * l + 1, 0.25, m2eff, mpl, p);
    for (int64_t s = 0; s < o->N; ++s) {
      f[s] += fld0[l];
      p[s] += dfld0[l];
    }
  }
  return LAT_OK;
}

int orc_init_bubbles(orc_t* o, int32_t nbub, const double* centres, double radius, double width) {
#pragma omp parallel for schedule(static)
  for (int z = 0; z < o->nz; ++z)
    for (int y = 0; y < o->ny; ++y)
      for (int x = 0; x < o->nx; ++x) {
        double v = -1.0;
        for (int b = 0; b < nbub; ++b) {
          double rx = x * o->dx - centres[3 * b], ry = y * o->dx - centres[3 * b + 1],
                 rz = z * o->dx - centres[3 * b + 2];
          double r = std::sqrt(rx * rx + ry * ry + rz * rz);
          v += 1.0 - std::tanh((r - radius) / width);
        }
        int64_t s = idx3(x, y, z, o->nx, o->ny);
        o->fld[s] = v;
        for (int l = 1; l < o->nf; ++l) o->fld[l * o->N + s] = 0.0;
        for (int l = 0; l < o->nf; ++l) o->fldp[l * o->N + s] = 0.0;
      }
  return LAT_OK;
}

// ------------------------------------------------------- bare transforms
int orc_fft_r2c_3d(int32_t nx, int32_t ny, int32_t nz, const double* f, double* F_interleaved) {
  orc::Fft3dReal t(nx, ny, nz);
  t.r2c(f, reinterpret_cast<cplx*>(F_interleaved));
  return LAT_OK;
}
int orc_fft_c2r_3d(int32_t nx, int32_t ny, int32_t nz, double* F_interleaved, double* f) {
  orc::Fft3dReal t(nx, ny, nz);
  t.c2r(reinterpret_cast<cplx*>(F_interleaved), f);
  return LAT_OK;
}

}  // extern "C"
