// k_spec.cu -- pointwise kick / drift passes and the k-space multiply.
//
// Restates, for the spectral Laplacian,
//   Hamiltonian_fields_kin      Pseudospec/openmp_dev/hamiltonian_conformal.f90:92-118
//   Hamiltonian_grav_kinetic    hamiltonian_conformal.f90:86-90
//   Hamiltonian_fields_grad_pot hamiltonian_conformal.f90:128-174,203-205
//   laplacian_3d k-space loop   Pseudospec/openmp_dev/fftw_mod.f90:192-201
// (Minkowski: hamiltonian_minkowski.f90:86-136).
//
// Fusion.  symp_o2step applies  G(h/2) K(h) G(h/2) D(h')  per substep.  The
// kick's Friedmann update needs GE2 = -sum phi lap / a^2 and PE = sum V(phi),
// both functions of phi alone: GE2 comes from the k-space pass by Parseval
// (sum_x phi lap = -(1/N) sum_k k^2 |F_k|^2) and PE from the previous drift
// pass.  Every block of the fused pass therefore knows a, ysclp before and
// after the kick and the drift coefficient h'/a^2 before it starts, and kick
// and drift run as ONE sweep over HBM.  The drift's KE2 and the new PE are
// reduced deterministically and the last block applies the ysclp update.
#include <algorithm>

#include "engine.hpp"

namespace lat {

namespace {

template <typename R> struct Vec4;
template <> struct Vec4<float> {
  float v[4];
  __device__ __forceinline__ void load(const float* p) {
    float4 t = __ldcs(reinterpret_cast<const float4*>(p));
    v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
  }
  __device__ __forceinline__ void store(float* p) const {
    __stcs(reinterpret_cast<float4*>(p), make_float4(v[0], v[1], v[2], v[3]));
  }
};
template <> struct Vec4<double> {
  double v[4];
  __device__ __forceinline__ void load(const double* p) {
    double2 a = __ldcs(reinterpret_cast<const double2*>(p));
    double2 b = __ldcs(reinterpret_cast<const double2*>(p) + 1);
    v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
  }
  __device__ __forceinline__ void store(double* p) const {
    __stcs(reinterpret_cast<double2*>(p), make_double2(v[0], v[1]));
    __stcs(reinterpret_cast<double2*>(p) + 1, make_double2(v[2], v[3]));
  }
};

struct Coef {
  double a0, ap0, a1, ap1, a2;
  double ck, cv, cd;
  double cc[2];  // closure force coefficients (fused kick+drift with a correction)
};

// Scalar chain of one pass, identical in every block.
__device__ __forceinline__ Coef coefs(const PwArgs& a, bool conf) {
  Coef c{};
  if (!conf) {
    c.ck = a.hk; c.cv = a.hk; c.cd = a.hd;
    return c;
  }
  const DevScalars* sc = a.sc;
  c.a0 = __ldcg(&sc->a);
  c.ap0 = __ldcg(&sc->ap);
  if (a.mode == PW_KD) {
    c.a1 = c.a0 - a.hg * c.ap0 / 6.0;                        // G(h/2)
    const double GE2 = __ldcg(&sc->ge2) / (c.a1 * c.a1) / a.Nd;
    const double PE = __ldcg(&sc->pe);
    c.ap1 = c.ap0 - c.a1 * c.a1 * c.a1 * (GE2 + 4.0 * PE) * a.hk;  // K(h) scalar part
    c.a2 = c.a1 - a.hg * c.ap1 / 6.0;                        // G(h/2)
    c.ck = a.hk * c.a1 * c.a1;
    c.cv = a.hk * c.a1 * c.a1 * c.a1 * c.a1;
    c.cd = a.hd / (c.a2 * c.a2);
  } else if (a.mode == PW_DRIFT) {
    c.cd = a.hd / (c.a0 * c.a0);
  } else {
    c.ck = a.hk * c.a0 * c.a0;
    c.cv = a.hk * c.a0 * c.a0 * c.a0 * c.a0;
  }
  return c;
}

// CORR (fused kick+drift of two fields only): the kick adds the learned
// closure's force hk (a1^4 or a1) corr[s][f] / corr_ts[f] after its own
// update and before the drift, as the separate closure kick would
template <typename R, bool KAHAN, int NF, bool CONF, int MODE, bool GWD, bool CORR = false>
__global__ void __launch_bounds__(256) pw_kernel(PwArgs a) {
  static_assert(!CORR || (MODE == PW_KD && NF == 2), "the closure force enters the fused kick of two fields");
  // the FP64 scalar chain once per block (its divisions would load the FP64
  // pipe with every thread's copy), shared through shared memory
  __shared__ Coef co_sh;
  if (CONF || CORR) {
    if (threadIdx.x == 0) {
      Coef c = coefs(a, CONF);
      if (CORR) {
        const double av = CONF ? c.a1 : 1.0;  // a = 1 in Minkowski
        const double f = a.corr_units ? av : av * av * av * av;
        c.cc[0] = a.hk * f / a.corr_ts[0];
        c.cc[1] = a.hk * f / a.corr_ts[1];
      }
      co_sh = c;
    }
    __syncthreads();
  }
  const Coef co = (CONF || CORR) ? co_sh : coefs(a, false);
  const R ck = (R)co.ck, cv = (R)co.cv, cd = (R)co.cd;
  const R cc[2] = {(R)co.cc[0], (R)co.cc[1]};
  const float* __restrict__ corr = a.corr;
  const int64_t N = a.N;
  R* phi = static_cast<R*>(a.phi);
  R* phic = static_cast<R*>(a.phic);
  R* pi = static_cast<R*>(a.pi);
  const R* lap = static_cast<const R*>(a.lap);
  using Acc = typename AccOf<R>::type;
  Acc acc_ke, acc_pe, acc_ge;

  auto site = [&](R (&f)[NF], R (&c)[NF], R (&p)[NF], const R (&lp)[NF], const R (&dl)[NF]) {
    if (MODE == PW_KD || MODE == PW_KICK) {
      R dv[NF];
      model_dv<R, NF>(a.model, f, dv);
#pragma unroll
      for (int l = 0; l < NF; ++l) {
        if (CONF && MODE == PW_KICK) acc_ge.add(-f[l] * lp[l]);
        p[l] = p[l] + (ck * lp[l] - cv * dv[l]);
        if (CORR) p[l] += cc[l] * dl[l];
      }
      if (CONF && MODE == PW_KICK) acc_pe.add(model_v<R, NF>(a.model, f));
    }
    if (MODE == PW_KD || MODE == PW_DRIFT) {
#pragma unroll
      for (int l = 0; l < NF; ++l) {
        if constexpr (KAHAN) kahan_add(f[l], c[l], cd * p[l]);
        else f[l] = f[l] + cd * p[l];
        if (CONF) acc_ke.add(p[l] * p[l]);
      }
      if (CONF) acc_pe.add(model_v<R, NF>(a.model, f));
    }
  };

  const int64_t nvec = N / 4;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < nvec; v += stride) {
    const int64_t s0 = v * 4;
    Vec4<R> F[NF], C[NF], P[NF], L[NF];
#pragma unroll
    for (int l = 0; l < NF; ++l) {
      F[l].load(phi + l * N + s0);
      if (KAHAN && MODE != PW_KICK) C[l].load(phic + l * N + s0);
      P[l].load(pi + l * N + s0);
      if (MODE != PW_DRIFT) L[l].load(lap + l * N + s0);
    }
    float4 D[2];  // closure force of the 4 sites, [site][field]
    if (CORR) {
      D[0] = __ldcs(reinterpret_cast<const float4*>(corr + 2 * s0));
      D[1] = __ldcs(reinterpret_cast<const float4*>(corr + 2 * s0) + 1);
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      R f[NF], c[NF], p[NF], lp[NF], dl[NF];
#pragma unroll
      for (int l = 0; l < NF; ++l) {
        f[l] = F[l].v[j];
        c[l] = (KAHAN && MODE != PW_KICK) ? C[l].v[j] : R(0);
        p[l] = P[l].v[j];
        lp[l] = MODE != PW_DRIFT ? L[l].v[j] : R(0);
        dl[l] = R(0);
      }
      if (CORR) {
        const float4 d = D[j / 2];
        dl[0] = (R)((j & 1) ? d.z : d.x);
        dl[NF - 1] = (R)((j & 1) ? d.w : d.y);
      }
      site(f, c, p, lp, dl);
#pragma unroll
      for (int l = 0; l < NF; ++l) {
        F[l].v[j] = f[l];
        C[l].v[j] = c[l];
        P[l].v[j] = p[l];
      }
    }
#pragma unroll
    for (int l = 0; l < NF; ++l) {
      if (MODE != PW_KICK) F[l].store(phi + l * N + s0);
      if (KAHAN && MODE != PW_KICK) C[l].store(phic + l * N + s0);
      if (MODE != PW_DRIFT) P[l].store(pi + l * N + s0);
    }
  }
  // tail (N not a multiple of 4)
  for (int64_t s = nvec * 4 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < N; s += stride) {
    R f[NF], c[NF], p[NF], lp[NF], dl[NF];
#pragma unroll
    for (int l = 0; l < NF; ++l) {
      f[l] = phi[l * N + s];
      c[l] = (KAHAN && MODE != PW_KICK) ? phic[l * N + s] : R(0);
      p[l] = pi[l * N + s];
      lp[l] = MODE != PW_DRIFT ? lap[l * N + s] : R(0);
      dl[l] = CORR ? (R)corr[2 * s + l] : R(0);
    }
    site(f, c, p, lp, dl);
#pragma unroll
    for (int l = 0; l < NF; ++l) {
      if (MODE != PW_KICK) phi[l * N + s] = f[l];
      if (KAHAN && MODE != PW_KICK) phic[l * N + s] = c[l];
      if (MODE != PW_DRIFT) pi[l * N + s] = p[l];
    }
  }
  if (GWD) {  // u_ij += h' pu_ij (Minkowski drift of the strain, grav-waves/evolve-gw.f90:38-44)
    R* u = static_cast<R*>(a.u);
    const R* pu = static_cast<const R*>(a.pu);
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < 6 * N; s += stride)
      u[s] = u[s] + cd * pu[s];
  }

  if (CONF) {
    const typename Acc::Red v[3] = {acc_ke.red(), acc_pe.red(), acc_ge.red()};
    double tot[3];
    if (grid_reduce<3>(v, a.rb, tot)) {
      DevScalars* sc = a.sc;
      if (bad(tot[0]) || bad(tot[1]) || bad(tot[2])) sc->err |= 1u;
      if (MODE == PW_KD) {
        sc->a = co.a2;
        sc->ap = co.ap1 + a.hd * (tot[0] / a.Nd) / (co.a2 * co.a2 * co.a2);
        sc->pe = tot[1] / a.Nd;
        sc->ke2 = tot[0];
      } else if (MODE == PW_DRIFT) {
        if (a.defer) {  // a z-slab: the sums of all slabs complete the update on the host
          sc->red[13] = tot[0];
          sc->red[14] = tot[1];
        } else {
          sc->ap = co.ap0 + a.hd * (tot[0] / a.Nd) / (co.a0 * co.a0 * co.a0);
          sc->pe = tot[1] / a.Nd;
          sc->ke2 = tot[0];
        }
      } else {
        const double GE2 = tot[2] / (co.a0 * co.a0) / a.Nd;
        const double PE = tot[1] / a.Nd;
        sc->ap = co.ap0 - co.a0 * co.a0 * co.a0 * (GE2 + 4.0 * PE) * a.hk;
        sc->pe = PE;
      }
    }
  }
}

// grid-stride launches: at most one block per `block` work items, so a small
// lattice does not launch (and reduce over) idle blocks
inline int clamp_grid(int grid, int64_t items, int block) {
  const int64_t need = (items + block - 1) / block;
  return (int)std::max<int64_t>(1, std::min<int64_t>(grid, need));
}

template <typename R, bool KAHAN, int NF, bool CONF>
int pw_go(const PwArgs& a, cudaStream_t s) {
  const bool gw = a.u != nullptr;
  const int grid = clamp_grid(a.grid, gw ? 6 * a.N : (a.N + 3) / 4, a.block);
  switch (a.mode) {
    case PW_KD:
      if constexpr (NF == 2) {
        if (a.corr) {
          pw_kernel<R, KAHAN, NF, CONF, PW_KD, false, true><<<grid, a.block, 0, s>>>(a);
          break;
        }
      } else {
        if (a.corr) return set_error(LAT_ERR_UNSUPPORTED, "the closure force needs two fields");
      }
      pw_kernel<R, KAHAN, NF, CONF, PW_KD, false><<<grid, a.block, 0, s>>>(a);
      break;
    case PW_DRIFT:
      if (gw) pw_kernel<R, KAHAN, NF, CONF, PW_DRIFT, true><<<grid, a.block, 0, s>>>(a);
      else pw_kernel<R, KAHAN, NF, CONF, PW_DRIFT, false><<<grid, a.block, 0, s>>>(a);
      break;
    case PW_KICK: pw_kernel<R, KAHAN, NF, CONF, PW_KICK, false><<<grid, a.block, 0, s>>>(a); break;
    default: return set_error(LAT_ERR_ARG, "bad pointwise mode");
  }
  if (g_launch_counter) ++*g_launch_counter;
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? LAT_OK : cuda_fail(e, "pointwise launch");
}

template <typename R, bool KAHAN, int NF>
int pw_nf(const PwArgs& a, cudaStream_t s) {
  return a.conf ? pw_go<R, KAHAN, NF, true>(a, s) : pw_go<R, KAHAN, NF, false>(a, s);
}

// ----------------------------------------------------------- k-space pass
template <typename R, typename C>
__global__ void __launch_bounds__(256) kmul_kernel(KmulArgs a) {
  C* F = static_cast<C*>(a.Fk);
  const int hx = a.nx / 2 + 1;
  const int64_t M = (int64_t)hx * a.ny * a.nz;
  const int64_t tot = M * a.nf;
  const R dkx2 = (R)a.dkx2, dky2 = (R)a.dky2, dkz2 = (R)a.dkz2, invN = (R)a.invN;
  using Acc = typename AccOf<R>::type;
  Acc acc;
  // 32-bit index arithmetic: nf * M < 2^31 is checked at handle creation
  const unsigned int stride = gridDim.x * blockDim.x;
  const unsigned int Mu = (unsigned int)M, hxu = (unsigned int)hx, nyu = (unsigned int)a.ny;
  for (unsigned int m = blockIdx.x * blockDim.x + threadIdx.x; m < (unsigned int)tot; m += stride) {
    const unsigned int mm = m % Mu;
    const int x = (int)(mm % hxu);
    const unsigned int r = mm / hxu;
    const int y = (int)(r % nyu), z = (int)(r / nyu);
    const int jj = fold_idx(y, a.ny), kk = fold_idx(z, a.nz);
    const R k2 = (R)(x * x) * dkx2 + (R)(jj * jj) * dky2 + (R)(kk * kk) * dkz2;
    C v = F[m];
    if (a.store_ge2) {
      const R w = (x == 0 || 2 * x == a.nx) ? R(1) : R(2);
      acc.add(w * k2 * (v.x * v.x + v.y * v.y));
    }
    const R sc = -k2 * invN;
    v.x *= sc;
    v.y *= sc;
    F[m] = v;
  }
  if (a.store_ge2) {
    const typename Acc::Red v[1] = {acc.red()};
    double t[1];
    if (grid_reduce<1>(v, a.rb, t)) {
      a.sc->ge2 = t[0] * a.invN;
      if (bad(t[0])) a.sc->err |= 1u;
    }
  }
}

__global__ void grav_kernel(DevScalars* sc, double h) { sc->a = sc->a - h * sc->ap / 6.0; }

__global__ void state_reset_kernel(DevScalars* sc) {
  sc->err = 0u;
  for (int i = 0; i < 4; ++i)
    if (!isfinite(sc->mean[i])) sc->mean[i] = 0.0;
  if (!isfinite(sc->ke_cur)) sc->ke_cur = 0.0;
}

// The first kernel of a streamed call: sum pi^2 over all fields (FP32
// momenta, n a multiple of 4) into sc->ke_cur; with phi, the lattice means of
// the two fields' phi_hi (q4 float4 per field) into sc->mean, the shifts of
// the call's first kick (after an upload, an initial condition or steps on
// another path the last kick's means are stale, and a shift far from the mean
// leaves the FP32 passes a large constant to transform: a one-time error of
// 1e-6 in the momenta of the 128^3 preheating lattice); and the coefficients
// of the call's first kick into sc->co.
__global__ void pi2_kernel(const float4* __restrict__ pi, int64_t n4, const float4* __restrict__ phi, int64_t q4,
                           DevScalars* sc, RedBuf rb, KickW first, double Nd) {
  // launched with programmatic serialization (the wait returns at once when
  // nothing precedes it programmatically)
  asm volatile("griddepcontrol.wait;\n" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
  KSum s, ma, mb;
  const int64_t i0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, step = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = i0; i < n4; i += step) {
    const float4 v = __ldcs(pi + i);
    s.add((v.x * v.x + v.y * v.y) + (v.z * v.z + v.w * v.w));
  }
  if (phi) {
    for (int64_t i = i0; i < q4; i += step) {
      const float4 v = __ldcg(phi + i);
      ma.add((v.x + v.y) + (v.z + v.w));
    }
    for (int64_t i = i0; i < q4; i += step) {
      const float4 v = __ldcg(phi + q4 + i);
      mb.add((v.x + v.y) + (v.z + v.w));
    }
  }
  const FF vals[3] = {s.red(), ma.red(), mb.red()};
  double tot[3];
  if (grid_reduce<3>(vals, rb, tot)) {
    sc->ke_cur = tot[0];
    if (bad(tot[0])) sc->err |= 1u;
    if (phi) {
      sc->mean[0] = tot[1] / Nd;
      sc->mean[1] = tot[2] / Nd;
      if (bad(tot[1]) || bad(tot[2])) sc->err |= 1u;
    }
    if (first.valid) kick_coefs_of(sc->a, sc->ap, tot[0], first.hd, first.hk, first.hg, Nd, sc->co);
  }
}

}  // namespace

int launch_pointwise(const PwArgs& a, int precision, cudaStream_t s) {
  if (a.nf == 1) return precision == LAT_FP64 ? pw_nf<double, false, 1>(a, s) : pw_nf<float, true, 1>(a, s);
  if (a.nf == 2) return precision == LAT_FP64 ? pw_nf<double, false, 2>(a, s) : pw_nf<float, true, 2>(a, s);
  return set_error(LAT_ERR_UNSUPPORTED, "pointwise passes support nfld = 1 or 2");
}

int launch_kmul(const KmulArgs& a, int precision, cudaStream_t s) {
  const int grid = clamp_grid(a.grid, ((int64_t)a.nx / 2 + 1) * a.ny * a.nz * a.nf, a.block);
  if (precision == LAT_FP64) kmul_kernel<double, double2><<<grid, a.block, 0, s>>>(a);
  else kmul_kernel<float, float2><<<grid, a.block, 0, s>>>(a);
  if (g_launch_counter) ++*g_launch_counter;
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? LAT_OK : cuda_fail(e, "kmul launch");
}

// One block: the lattice sums of a kick of the streamed separable passes in
// block order, then the scalar chain of the kick (hamiltonian_conformal.f90:
// 86-174): the drift's ysclp += hd KE2/a^3, a1 = a - hg ysclp/6, the kick's
// ysclp -= a1^3 (GE2/a1^2 + 4 PE) hk, a = a1 - hg ysclp/6; and the lattice
// means, the shifts of the next kick; and the FP32 coefficients of the next
// kick of the call (kick_coefs_of), which its three passes load.  The chain
// runs in one thread between pass Z and the next pass X, so its quotients
// use one reciprocal per scale factor (a0, a1) and products by 1/N and 1/6.
__global__ void __launch_bounds__(256) sep_finalize_kernel(SepFinArgs f) {
  // warp w < 7 sums value w of the seven (pass X: pe, GEx, sum phi_A, sum
  // phi_B; Y: GEy; Z: GEz, sum pi^2) over the blocks, all loads of a lane in
  // flight at once; the order of every sum is fixed
  __shared__ double tot[8];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  // a programmatic dependent of pass Z: its partials are read after the wait
  asm volatile("griddepcontrol.wait;\n" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
  if (wid < 7) {
    const int p = wid < 4 ? 0 : (wid == 4 ? 1 : 2);
    const int nv = p == 0 ? 4 : (p == 1 ? 1 : 2), i = p == 0 ? wid : (p == 1 ? 0 : wid - 5);
    const int nb = p == 0 ? f.gx : (p == 1 ? f.gy : f.gz);
    const double* src = f.part + (p == 0 ? SEP_PART_X : (p == 1 ? SEP_PART_Y : SEP_PART_Z)) + i;
    double v[16];
#pragma unroll
    for (int r = 0; r < 16; ++r) {
      const int b = lane + 32 * r;
      v[r] = b < nb ? __ldcg(src + (size_t)b * nv) : 0.0;
    }
    double x = 0.0;
    for (int b = lane + 32 * 16; b < nb; b += 32) x += __ldcg(src + (size_t)b * nv);  // more than 512 blocks
#pragma unroll
    for (int r = 0; r < 16; ++r) x += v[r];
    x = warp_sum(x);
    if (lane == 0) tot[wid] = x;
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  // tot: pe, GEx, sum phi_A, sum phi_B, GEy, GEz, sum pi^2
  DevScalars* w = f.sc;
  w->mean[0] = tot[2] / f.Nd;
  w->mean[1] = tot[3] / f.Nd;
  w->gsum[0] = tot[1];
  w->gsum[1] = tot[4];
  w->gsum[2] = tot[5];
  if (f.conf) {
    const double a0 = w->a, ke = w->ke_cur, iN = 1.0 / f.Nd, hg6 = f.hg * (1.0 / 6.0);
    const double r0 = 1.0 / a0;
    const double ap0 = w->ap + f.hd * ke * iN * (r0 * r0 * r0);
    const double a1 = a0 - hg6 * ap0;
    const double r1 = 1.0 / a1;
    const double GE2 = (tot[1] + tot[4] + tot[5]) * iN * (r1 * r1);
    const double PE = tot[0] * iN;
    const double ap1 = ap0 - a1 * a1 * a1 * (GE2 + 4.0 * PE) * f.hk;
    const double a2 = a1 - hg6 * ap1;
    w->pe = PE;
    if (f.hd != 0.0) w->ke2 = ke;
    w->ap = ap1;
    w->a = a2;
    w->ke_cur = tot[6];
    if (f.next.valid) kick_coefs_of(a2, ap1, tot[6], f.next.hd, f.next.hk, f.next.hg, f.Nd, w->co);
    if (bad(PE) || bad(GE2) || bad(tot[6])) w->err |= 1u;
  }
  if (bad(tot[2]) || bad(tot[3])) w->err |= 1u;
}

int launch_sep_finalize(const SepFinArgs& f, cudaStream_t s) {
  cudaError_t e = launch_pdl(sep_finalize_kernel, dim3(1), dim3(256), 0, s, f);
  if (e != cudaSuccess) return cuda_fail(e, "separable finalize launch");
  if (g_launch_counter) ++*g_launch_counter;
  e = cudaGetLastError();
  return e == cudaSuccess ? LAT_OK : cuda_fail(e, "separable finalize launch");
}

int launch_pi2_sum(const void* pi, int64_t n, DevScalars* sc, RedBuf rb, int grid, cudaStream_t s, KickW first,
                   double Nd, const void* phi, int64_t nsite) {
  if (n % 4 || (phi && nsite % 4)) return set_error(LAT_ERR_STATE, "momenta sum: length not a multiple of 4");
  cudaError_t e = launch_pdl(pi2_kernel, dim3(grid), dim3(256), 0, s, static_cast<const float4*>(pi), n / 4,
                             static_cast<const float4*>(phi), phi ? nsite / 4 : int64_t{0}, sc, rb, first, Nd);
  if (e != cudaSuccess) return cuda_fail(e, "momenta sum launch");
  if (g_launch_counter) ++*g_launch_counter;
  e = cudaGetLastError();
  return e == cudaSuccess ? LAT_OK : cuda_fail(e, "momenta sum launch");
}

int launch_state_reset(DevScalars* sc, cudaStream_t s) {
  state_reset_kernel<<<1, 1, 0, s>>>(sc);
  if (g_launch_counter) ++*g_launch_counter;
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? LAT_OK : cuda_fail(e, "state reset launch");
}

int launch_grav(DevScalars* sc, double h, cudaStream_t s) {
  grav_kernel<<<1, 1, 0, s>>>(sc, h);
  if (g_launch_counter) ++*g_launch_counter;
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? LAT_OK : cuda_fail(e, "grav launch");
}

}  // namespace lat
