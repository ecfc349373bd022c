// k_out.cu -- layout conversion, spectra, energies and initial conditions.
#include "engine.hpp"

namespace lat {

namespace {

// ------------------------------------------------------------ layouts
// Fortran fld(nfld, i, j, k) (field fastest) <-> device [field][z][y][x].
template <typename R, bool KAHAN>
// fs: element stride between fields of the SoA side (N, or the plane count
// of a z-slab's storage times the plane size when N covers its interior)
__global__ void aos2soa_kernel(const double* __restrict__ aos, int nf, int64_t N, int64_t fs, R* hi, R* c) {
  const int64_t tot = N * nf;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < tot; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = t / nf;
    const int f = (int)(t - s * nf);
    const double v = aos[t];
    const R h = (R)v;
    hi[f * fs + s] = h;
    if (KAHAN && c) c[f * fs + s] = (R)((double)h - v);
  }
}
template <typename R, bool KAHAN>
__global__ void soa2aos_kernel(const R* hi, const R* c, int nf, int64_t N, int64_t fs, double* __restrict__ aos) {
  const int64_t tot = N * nf;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < tot; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = t / nf;
    const int f = (int)(t - s * nf);
    double v = (double)hi[f * fs + s];
    if (KAHAN && c) v -= (double)c[f * fs + s];
    aos[t] = v;
  }
}
template <typename R, bool KAHAN>
__global__ void to64_kernel(const R* hi, const R* c, int64_t n, double* out) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    double v = (double)hi[t];
    if (KAHAN && c) v -= (double)c[t];
    out[t] = v;
  }
}
template <typename R, bool KAHAN>
__global__ void from64_kernel(const double* in, int64_t n, R* hi, R* c) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    const double v = in[t];
    const R h = (R)v;
    hi[t] = h;
    if (KAHAN && c) c[t] = (R)((double)h - v);
  }
}

inline int grid_for(int64_t n) {
  int64_t g = (n + 255) / 256;
  return (int)(g > 4096 ? 4096 : (g < 1 ? 1 : g));
}
inline int done(const char* what) {
  if (g_launch_counter) ++*g_launch_counter;
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? LAT_OK : cuda_fail(e, what);
}

// ------------------------------------------------------------ spectra
// Array grid reduction: every block adds its shared bins to partials[block],
// the last block sums the rows in block order.
__device__ void bins_grid_reduce(const double* shb, int nval, double* partials, double* out,
                                 unsigned int* counter) {
  __shared__ int am_last;
  const int bid = blockIdx.x;
  for (int i = threadIdx.x; i < nval; i += blockDim.x) partials[(size_t)bid * nval + i] = shb[i];
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned int t = atomicAdd(counter, 1u);
    am_last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!am_last) return;
  __threadfence();
  for (int i = threadIdx.x; i < nval; i += blockDim.x) {
    double s = 0.0;
    for (int b = 0; b < (int)gridDim.x; ++b) s += __ldcg(&partials[(size_t)b * nval + i]);
    out[i] = s;
  }
  if (threadIdx.x == 0) *counter = 0u;
}

// Binning of spectrum_3d (analysis_spec.f90:86-99) / spectrum_bin
// (Discrete/Bubble-Collisions/analysis.f90:203-214).  The reference loops over
// the full x range with folded ii, i.e. Hermitian weight 2 on interior kx
// planes.  Shell index l = floor(sqrt(ii^2+jj^2+kk^2)) is taken exactly in
// integers; the smooth weights use the correctly rounded FP64 sqrt and
// uncontracted FP64 arithmetic so they are bit-identical to the host's.
template <typename R, typename C>
__global__ void __launch_bounds__(256) spec_kernel(SpecArgs a) {
  extern __shared__ double shb[];  // [3][nbins]
  const int nb = a.nbins;
  for (int i = threadIdx.x; i < 3 * nb; i += blockDim.x) shb[i] = 0.0;
  __syncthreads();
  const C* F1 = static_cast<const C*>(a.F1);
  const C* F2 = static_cast<const C*>(a.F2);
  const unsigned int hx = a.nx / 2 + 1, ny = a.ny;
  const unsigned int M = hx * ny * (unsigned int)a.nz;
  for (unsigned int m = blockIdx.x * blockDim.x + threadIdx.x; m < M; m += gridDim.x * blockDim.x) {
    const int x = (int)(m % hx);
    const unsigned int r = m / hx;
    const int y = (int)(r % ny), z = (int)(r / ny);
    const int jj = fold_idx(y, a.ny), kk = fold_idx(z, a.nz);
    const double wx = (x == 0 || 2 * x == a.nx) ? 1.0 : 2.0;
    const int m2 = x * x + jj * jj + kk * kk;
    const int l = isqrt_exact(m2);
    const C f1 = F1[m];
    double v, vi = 0.0;
    if (a.mode == 2) {
      const C f2 = F2[m];
      v = (double)f1.x * (double)f2.x + (double)f1.y * (double)f2.y;   // Re(F1 conj F2)
      vi = (double)f1.y * (double)f2.x - (double)f1.x * (double)f2.y;  // Im(F1 conj F2)
    } else {
      v = (double)f1.x * (double)f1.x + (double)f1.y * (double)f1.y;
    }
    if (a.mode == LAT_SPEC_COUNT) {
      if (l < nb) {
        atomicAdd(&shb[l], wx * v);
        atomicAdd(&shb[nb + l], wx);
      }
    } else {
      const double p = sqrt((double)m2);
      const double d0 = __dsub_rn((double)l, p), d1 = __dsub_rn((double)(l + 1), p);
      const double e0 = __dsub_rn(1.0, __dmul_rn(d0, d0)), e1 = __dsub_rn(1.0, __dmul_rn(d1, d1));
      const double c0 = __dmul_rn(e0, e0), c1 = __dmul_rn(e1, e1);
      if (l < nb) {
        atomicAdd(&shb[l], wx * c0 * v);
        atomicAdd(&shb[nb + l], wx * c0);
        if (a.mode == 2) atomicAdd(&shb[2 * nb + l], wx * c0 * vi);
      }
      if (l + 1 < nb) {
        atomicAdd(&shb[l + 1], wx * c1 * v);
        atomicAdd(&shb[nb + l + 1], wx * c1);
        if (a.mode == 2) atomicAdd(&shb[2 * nb + l + 1], wx * c1 * vi);
      }
    }
  }
  __syncthreads();
  bins_grid_reduce(shb, 3 * nb, a.partials, a.out, a.counter);
}

// TT projection of the six pi_ij with the lattice momentum of the central
// difference, k_i = sin(2 pi n_i / N_i)/dx:  P = 1 - k k^T/k^2,
// pi^TT = P pi P - P tr(P pi)/2;  sum_ij |pi^TT_ij|^2 binned like spectrum_bin.
template <typename R, typename C>
__global__ void __launch_bounds__(256) gwspec_kernel(GwSpecArgs a) {
  extern __shared__ double shb[];  // [2][nbins]
  const int nb = a.nbins;
  for (int i = threadIdx.x; i < 2 * nb; i += blockDim.x) shb[i] = 0.0;
  __syncthreads();
  const unsigned int hx = a.nx / 2 + 1, ny = a.ny;
  const unsigned int M = hx * ny * (unsigned int)a.nz;
  const double twopi = 6.283185307179586476925286766559;
  for (unsigned int m = blockIdx.x * blockDim.x + threadIdx.x; m < M; m += gridDim.x * blockDim.x) {
    const int x = (int)(m % hx);
    const unsigned int r = m / hx;
    const int y = (int)(r % ny), z = (int)(r / ny);
    const int jj = fold_idx(y, a.ny), kk = fold_idx(z, a.nz);
    const double wx = (x == 0 || 2 * x == a.nx) ? 1.0 : 2.0;
    const int l = isqrt_exact(x * x + jj * jj + kk * kk);
    if (l >= nb) continue;
    double k[3] = {sin(twopi * x / a.nx) / a.dx, sin(twopi * y / a.ny) / a.dx, sin(twopi * z / a.nz) / a.dx};
    const double k2 = k[0] * k[0] + k[1] * k[1] + k[2] * k[2];
    double sum = 0.0;
    if (k2 > 0.0) {
      double P[3][3];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) P[i][j] = (i == j ? 1.0 : 0.0) - k[i] * k[j] / k2;
      const int map[3][3] = {{0, 3, 4}, {3, 1, 5}, {4, 5, 2}};
      double hr[3][3], hi[3][3];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          const C v = static_cast<const C*>(a.F[map[i][j]])[m];
          hr[i][j] = (double)v.x;
          hi[i][j] = (double)v.y;
        }
      double Ar[3][3], Ai[3][3];  // A = P h
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          double sr = 0, si = 0;
#pragma unroll
          for (int l2 = 0; l2 < 3; ++l2) { sr += P[i][l2] * hr[l2][j]; si += P[i][l2] * hi[l2][j]; }
          Ar[i][j] = sr; Ai[i][j] = si;
        }
      double trr = Ar[0][0] + Ar[1][1] + Ar[2][2], tri = Ai[0][0] + Ai[1][1] + Ai[2][2];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          double sr = 0, si = 0;
#pragma unroll
          for (int l2 = 0; l2 < 3; ++l2) { sr += Ar[i][l2] * P[l2][j]; si += Ai[i][l2] * P[l2][j]; }
          sr -= 0.5 * P[i][j] * trr;
          si -= 0.5 * P[i][j] * tri;
          sum += sr * sr + si * si;
        }
    }
    atomicAdd(&shb[l], wx * sum);
    atomicAdd(&shb[nb + l], wx);
  }
  __syncthreads();
  bins_grid_reduce(shb, 2 * nb, a.partials, a.out, a.counter);
}

// ------------------------------------------------------------ energies
template <typename R, bool KAHAN, int NF>
__global__ void __launch_bounds__(256) energy_kernel(EnergyArgs a) {
  const int nx = a.nx, ny = a.ny, nz = a.nz;
  const int64_t N = (int64_t)nx * ny * nz;
  const R* phi = static_cast<const R*>(a.phi);
  const R* pi = static_cast<const R*>(a.pi);
  const R* u = static_cast<const R*>(a.u);
  const R* pu = static_cast<const R*>(a.pu);
  using Acc = typename AccOf<R>::type;
  Acc s[11];
  const R c0 = (R)a.c[0], c1 = (R)a.c[1], c2 = (R)a.c[2], c3 = (R)a.c[3];
  int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool ranged = a.t_hi > 0;  // a z-slab: only its interior sites
  const int64_t tend = ranged ? a.t_hi : N;
  if (ranged) t0 += a.t_lo;
  if constexpr (sizeof(R) == 4) {
    // spectral, no GW arrays: four sites per thread and step (float4 loads),
    // one compensated add per sum and four sites
    if (!ranged && !a.fd && !u && N % 4 == 0) {  // every field's array starts 16-byte aligned
      const int64_t n4 = N / 4;
      for (int64_t v = t0; v < n4; v += (int64_t)gridDim.x * blockDim.x) {
        float4 fq[NF], pq[NF];
#pragma unroll
        for (int l = 0; l < NF; ++l) {
          fq[l] = __ldcs(reinterpret_cast<const float4*>(phi + l * N) + v);
          pq[l] = __ldcs(reinterpret_cast<const float4*>(pi + l * N) + v);
        }
        R ke = 0, pe = 0, m0 = 0, m1 = 0;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          R f[NF];
#pragma unroll
          for (int l = 0; l < NF; ++l) {
            const float4 F4 = fq[l], P4 = pq[l];
            f[l] = j == 0 ? F4.x : (j == 1 ? F4.y : (j == 2 ? F4.z : F4.w));
            const R p = j == 0 ? P4.x : (j == 1 ? P4.y : (j == 2 ? P4.z : P4.w));
            ke += p * p;
          }
          pe += model_v<R, NF>(a.model, f);
          m0 += f[0];
          if (NF > 1) m1 += f[NF > 1 ? 1 : 0];
        }
        s[0].add(ke);
        s[1].add(pe);
        s[2].add(m0);
        if (NF > 1) s[3].add(m1);
      }
      t0 = N;  // no tail
    }
  }
  for (int64_t t = t0; t < tend; t += (int64_t)gridDim.x * blockDim.x) {
    R f[NF];
#pragma unroll
    for (int l = 0; l < NF; ++l) {
      f[l] = phi[l * N + t];
      const R p = pi[l * N + t];
      s[0].add(p * p);
    }
    s[1].add(model_v<R, NF>(a.model, f));
    s[2].add(f[0]);
    if (NF > 1) s[3].add(f[NF > 1 ? 1 : 0]);
    if (a.fd || u) {
      const int x = (int)(t % nx), y = (int)((t / nx) % ny), z = (int)(t / ((int64_t)nx * ny));
      auto wrapi = [](int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); };
      auto stencil = [&](const R* g, R& lapsum, R& grad2) {
        const R g0 = g[t];
        R r1 = 0, r2 = 0, r3 = 0, q1 = 0, q2 = 0, q3 = 0;
        for (int dz = -1; dz <= 1; ++dz)
          for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
              const int rank = (dx != 0) + (dy != 0) + (dz != 0);
              if (rank == 0) continue;
              const R v = g[((int64_t)wrapi(z + dz, nz) * ny + wrapi(y + dy, ny)) * nx + wrapi(x + dx, nx)];
              const R d = v - g0;
              if (rank == 1) { r1 += v; q1 += d * d; }
              else if (rank == 2) { r2 += v; q2 += d * d; }
              else { r3 += v; q3 += d * d; }
            }
        lapsum = c0 * g0 + c1 * r1 + c2 * r2 + c3 * r3;
        grad2 = c1 * q1 + c2 * q2 + c3 * q3;
      };
      if (a.fd) {
        R g2sum = 0;
#pragma unroll
        for (int l = 0; l < NF; ++l) {
          R ls, g2;
          stencil(phi + l * N, ls, g2);
          s[4].add(-f[l] * ls);
          s[5].add(g2);
          g2sum += g2;
        }
        if (a.ball_r2 > 0.0) {  // 1-based indices about n/2 (iofile.f90:552)
          const double bx = x + 1 - nx / 2, by = y + 1 - ny / 2, bz = z + 1 - nz / 2;
          if ((bx * bx + by * by + bz * bz) * a.dx * a.dx < a.ball_r2) {
            R psum = 0;
#pragma unroll
            for (int l = 0; l < NF; ++l) psum += pi[l * N + t];
            s[8].add(psum * psum);
            s[9].add(g2sum);
            s[10].add(model_v<R, NF>(a.model, f));
          }
        }
      }
      if (u) {
        for (int g = 0; g < 6; ++g) {
          const R w = g < 3 ? R(1) : R(2);
          const R p = pu[g * N + t];
          s[6].add(w * p * p);
          R ls, g2;
          stencil(u + g * N, ls, g2);
          s[7].add(-w * u[g * N + t] * ls);
        }
      }
    }
  }
  typename Acc::Red v[11];
  double tot[11];
#pragma unroll
  for (int i = 0; i < 11; ++i) v[i] = s[i].red();
  if (grid_reduce<11>(v, a.rb, tot)) {
    for (int i = 0; i < 11; ++i) {
      a.sc->red[i < 8 ? i : i + 1] = tot[i];  // red[8] is the spectral Parseval sum
      if (bad(tot[i])) a.sc->err |= 1u;
    }
  }
}

// sum over the half spectra of all fields of w k^2 |F_k|^2 (w = 2 for the
// modes whose conjugate partner is not stored): one warp per row (y, z,
// field) of nx/2+1 modes, the row's y and z part of k^2 computed once, the
// terms in the field precision, compensated sums per lane.
template <typename R, typename C>
__global__ void __launch_bounds__(256) parseval_kernel(const C* F, int nx, int ny, int nz, int nf, double dkx2,
                                                       double dky2, double dkz2, DevScalars* sc, int slot,
                                                       RedBuf rb) {
  const int hx = nx / 2 + 1;
  const int64_t rows = (int64_t)ny * nz * nf;
  const int lane = threadIdx.x & 31;
  const int64_t warp0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  using Acc = typename AccOf<R>::type;
  Acc acc;
  for (int64_t row = warp0; row < rows; row += nwarps) {
    const int64_t rr = row % ((int64_t)ny * nz);
    const int y = (int)(rr % ny), z = (int)(rr / ny);
    const int jj = fold_idx(y, ny), kk = fold_idx(z, nz);
    const R kyz = (R)((double)(jj * jj) * dky2 + (double)(kk * kk) * dkz2);
    const C* Fr = F + row * hx;
    for (int x = lane; x < hx; x += 32) {
      const C v = Fr[x];
      const R w = (x == 0 || 2 * x == nx) ? R(1) : R(2);
      const R k2 = (R)(x * x) * (R)dkx2 + kyz;
      acc.add(w * k2 * (v.x * v.x + v.y * v.y));
    }
  }
  const typename Acc::Red vv[1] = {acc.red()};
  double t[1];
  if (grid_reduce<1>(vv, rb, t)) sc->red[slot] = t[0];
}

// -------------------------------------------------- initial conditions
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
__device__ __forceinline__ double u01(uint64_t r) { return ((double)(r >> 11) + 1.0) * (1.0 / 9007199254740992.0); }
__device__ __forceinline__ double2 mode_gauss(uint64_t seed, int field, int64_t mode) {
  const uint64_t key = mix64(mix64(mix64(seed) ^ (uint64_t)field) ^ (uint64_t)mode);
  const double u1 = u01(mix64(key ^ 1ULL)), u2 = u01(mix64(key ^ 2ULL));
  const double r = sqrt(-2.0 * log(u1));
  const double th = 6.2831853071795864769252867665590 * u2;
  return make_double2(r * cos(th), r * sin(th));
}

// Same draw as the oracle's orc_init_vacuum: Hermitian partners inside the
// kx = 0 and kx = nx/2 planes share one draw (the lower mode index draws).
__global__ void vacuum_kernel(VacArgs a) {
  const int hx = a.nx / 2 + 1;
  const int64_t M = (int64_t)hx * a.ny * a.nz;
  for (int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; m < M; m += (int64_t)gridDim.x * blockDim.x) {
    const int x = (int)(m % hx);
    const int64_t r = m / hx;
    const int y = (int)(r % a.ny), z = (int)(r / a.ny);
    const int jj = fold_idx(y, a.ny), kk = fold_idx(z, a.nz);
    const double k2 = (double)x * x * a.dkx * a.dkx + (double)jj * jj * a.dky * a.dky + (double)kk * kk * a.dkz * a.dkz;
    double2 F = make_double2(0, 0), P = make_double2(0, 0);
    if (k2 > 0.0 && sqrt(k2) <= a.kcut) {
      const double w = sqrt(k2 + a.m2);
      const double sig = sqrt(a.sig_pref / w);
      const bool selfplane = (x == 0) || (2 * x == a.nx);
      const int64_t mp = ((int64_t)((a.nz - z) % a.nz) * a.ny + (a.ny - y) % a.ny) * hx + x;
      const double h = 0.70710678118654752440084436210485;
      // pi_k = -i w F_k for the drawing member of a pair (a wave travelling along
      // +k); the Hermitian partner carries +i w F, a self-conjugate mode none.
      if (selfplane && mp == m) {
        double2 g = mode_gauss(a.seed, a.field, m);
        F = make_double2(sig * g.x, 0.0);
      } else if (selfplane && mp < m) {
        double2 g = mode_gauss(a.seed, a.field, mp);
        F = make_double2(sig * g.x * h, -(sig * g.y * h));
        P = make_double2(-w * F.y, w * F.x);  // +i w F
      } else {
        double2 g = mode_gauss(a.seed, a.field, m);
        F = make_double2(sig * g.x * h, sig * g.y * h);
        P = make_double2(w * F.y, -w * F.x);  // -i w F
      }
    }
    a.Fphi[m] = F;
    a.Fpi[m] = P;
  }
}

// ------------------------------------------- the reference's sample() IC
// (Pseudospec/openmp_dev/evolve_spectral.f90:421-506).  The DST-II of the
// oversampled radial profile, Y_k = 2 sum_j X_j sin(pi (2j+1)(k+1) / (2 nos)),
// is the imaginary part of one complex FFT of length 4 nos of the odd
// embedding z[2j+1] = X_j, z[4 nos - 2j - 1] = -X_j: Y_k = -Im Z_{k+1}.
__global__ void sample_dst_in_kernel(double2* z, int nos, double dkos, double m2, double gamma, double kcut) {
  const int64_t L4 = 4LL * nos;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < L4; t += (int64_t)gridDim.x * blockDim.x) {
    double v = 0.0;
    if (t & 1) {
      const bool lower = t < 2LL * nos;
      const int64_t j = lower ? (t - 1) / 2 : (L4 - t - 1) / 2;
      const double kk = (j + 0.5) * dkos;
      const double x = kk * pow(kk * kk + m2, gamma) * exp(-(kk / kcut) * (kk / kcut));
      v = lower ? x : -x;
    }
    z[t] = make_double2(v, 0.0);
  }
}

// ker[k] = norm Y_k / (k + 1): the 1-based profile ker(k + 1)
__global__ void sample_dst_out_kernel(const double2* Z, int nos, double norm, double* ker) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nos; t += gridDim.x * blockDim.x)
    ker[t] = norm * (-Z[t + 1].y) / (t + 1);
}

// the profile interpolated at |(i, j, k) - nn| os (1-based indices, nn = n/2 + 1)
__global__ void sample_kernel3d(const double* ker, int n, double* f) {
  const int64_t N = (int64_t)n * n * n;
  const int nn = n / 2 + 1, os = 16;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < N; t += (int64_t)gridDim.x * blockDim.x) {
    const int x = (int)(t % n), y = (int)((t / n) % n), z = (int)(t / ((int64_t)n * n));
    const double di = x + 1 - nn, dj = y + 1 - nn, dz = z + 1 - nn;
    const double kk = sqrt(di * di + dj * dj + dz * dz) * os;
    const int l = (int)floor(kk);
    f[t] = l > 0 ? ker[l - 1] + (kk - l) * (ker[l] - ker[l - 1]) : (4.0 * ker[0] - ker[1]) / 3.0;
  }
}

// every half-spectrum mode times the Box-Muller noise of its counter-based draw
__global__ void sample_noise_kernel(double2* F, int64_t M, uint64_t seed, int stream) {
  for (int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; m < M; m += (int64_t)gridDim.x * blockDim.x) {
    const double2 g = mode_gauss(seed, stream, m), v = F[m];
    F[m] = make_double2(v.x * g.x - v.y * g.y, v.x * g.y + v.y * g.x);
  }
}

// the kx = 0 and kx = n/2 planes projected onto their Hermitian part
__global__ void sample_hermitize_kernel(double2* F, int n) {
  const int hx = n / 2 + 1;
  const int64_t P = 2LL * n * n;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < P; t += (int64_t)gridDim.x * blockDim.x) {
    const int x = (t < (int64_t)n * n) ? 0 : n / 2;
    const int64_t r = t % ((int64_t)n * n);
    const int y = (int)(r % n), z = (int)(r / n);
    const int64_t m = ((int64_t)z * n + y) * hx + x;
    const int64_t mp = ((int64_t)((n - z) % n) * n + (n - y) % n) * hx + x;
    if (mp < m) continue;
    const double2 a = F[m], b = F[mp];
    const double2 h = make_double2(0.5 * (a.x + b.x), 0.5 * (a.y - b.y));
    F[m] = h;
    F[mp] = make_double2(h.x, -h.y);
  }
}

// STENCIL(c,LAPLACE) with pre-scaled coefficients lc = c/(cc dx^2), FP64.
__global__ void fd_lap64_kernel(const double* g, double* out, int nx, int ny, int nz, double l0, double l1, double l2,
                                double l3) {
  const int64_t N = (int64_t)nx * ny * nz;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < N; t += (int64_t)gridDim.x * blockDim.x) {
    const int x = (int)(t % nx), y = (int)((t / nx) % ny), z = (int)(t / ((int64_t)nx * ny));
    double r1 = 0, r2 = 0, r3 = 0;
    for (int dz = -1; dz <= 1; ++dz)
      for (int dy = -1; dy <= 1; ++dy)
        for (int dx = -1; dx <= 1; ++dx) {
          const int rank = (dx != 0) + (dy != 0) + (dz != 0);
          if (rank == 0) continue;
          const int xx = x + dx < 0 ? x + dx + nx : (x + dx >= nx ? x + dx - nx : x + dx);
          const int yy = y + dy < 0 ? y + dy + ny : (y + dy >= ny ? y + dy - ny : y + dy);
          const int zz = z + dz < 0 ? z + dz + nz : (z + dz >= nz ? z + dz - nz : z + dz);
          const double v = g[((int64_t)zz * ny + yy) * nx + xx];
          if (rank == 1) r1 += v; else if (rank == 2) r2 += v; else r3 += v;
        }
    out[t] = l0 * g[t] + l1 * r1 + l2 * r2 + l3 * r3;
  }
}

__global__ void add_scale_kernel(double* f, int64_t n, double scale, double offset) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
    f[t] = offset + f[t] * scale;
}

__global__ void bubbles_kernel(double* phi, int nx, int ny, int nz, double dx, int nbub, const double* cen,
                               double R, double w) {
  const int64_t N = (int64_t)nx * ny * nz;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < N; t += (int64_t)gridDim.x * blockDim.x) {
    const int x = (int)(t % nx), y = (int)((t / nx) % ny), z = (int)(t / ((int64_t)nx * ny));
    double v = -1.0;
    for (int b = 0; b < nbub; ++b) {
      const double rx = x * dx - cen[3 * b], ry = y * dx - cen[3 * b + 1], rz = z * dx - cen[3 * b + 2];
      const double rr = sqrt(rx * rx + ry * ry + rz * rz);
      v += 1.0 - tanh((rr - R) / w);
    }
    phi[t] = v;
  }
}

// Boosted-wall bubbles of Discrete/Bubble-Collisions/ic_bubble.f90:45-77 with
// the profile and time derivative of init_cond.f90:192-234: centres are
// 1-based site indices, distances are not wrapped, bubbles superpose, and
// phi_false is added at the end.
__global__ void bubbles_boost_kernel(double* phi, double* pi, int nx, int ny, int nz, double dx, int nbub,
                                     const int* cen, double r0, double t0, double pf, double pt) {
  const int64_t N = (int64_t)nx * ny * nz;
  const double step = (pf - pt) / 2.0, ave = (-pf + pt) / 2.0, rt2 = 1.4142135623730951;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < N; t += (int64_t)gridDim.x * blockDim.x) {
    const int x = (int)(t % nx), y = (int)((t / nx) % ny), z = (int)(t / ((int64_t)nx * ny));
    double f = 0.0, d = 0.0;
    for (int b = 0; b < nbub; ++b) {
      const int ii = x + 1 - cen[3 * b], jj = y + 1 - cen[3 * b + 1], kk = z + 1 - cen[3 * b + 2];
      const double rad = sqrt((double)(ii * ii + jj * jj + kk * kk) * dx * dx);
      if (rad * rad > t0 * t0) {
        const double s1 = sqrt(rad * rad - t0 * t0), s = s1 - r0;
        const double ch = cosh(s / rt2);
        f += step * tanh(s / rt2) + ave;
        d += -step * t0 / s1 / rt2 / (ch * ch);
      } else {
        f += pt - pf;
      }
    }
    phi[t] = f + pf;
    pi[t] = d;
  }
}

}  // namespace

int launch_bubbles_boosted(double* phi, double* pi, int nx, int ny, int nz, double dx, int nbub, const int* cen,
                           double r0, double t0, double pf, double pt, cudaStream_t s) {
  bubbles_boost_kernel<<<grid_for((int64_t)nx * ny * nz), 256, 0, s>>>(phi, pi, nx, ny, nz, dx, nbub, cen, r0, t0,
                                                                       pf, pt);
  return done("boosted bubbles");
}

int launch_aos2soa(const double* aos, int nf, int64_t N, int precision, void* hi, void* c, cudaStream_t s,
                   int64_t fstride) {
  const int64_t fs = fstride > 0 ? fstride : N;
  if (precision == LAT_FP64)
    aos2soa_kernel<double, false><<<grid_for(N * nf), 256, 0, s>>>(aos, nf, N, fs, (double*)hi, nullptr);
  else aos2soa_kernel<float, true><<<grid_for(N * nf), 256, 0, s>>>(aos, nf, N, fs, (float*)hi, (float*)c);
  return done("aos2soa");
}
int launch_soa2aos(const void* hi, const void* c, int nf, int64_t N, int precision, double* aos, cudaStream_t s,
                   int64_t fstride) {
  const int64_t fs = fstride > 0 ? fstride : N;
  if (precision == LAT_FP64)
    soa2aos_kernel<double, false><<<grid_for(N * nf), 256, 0, s>>>((const double*)hi, nullptr, nf, N, fs, aos);
  else
    soa2aos_kernel<float, true><<<grid_for(N * nf), 256, 0, s>>>((const float*)hi, (const float*)c, nf, N, fs, aos);
  return done("soa2aos");
}
// Every ds-th site of one field array as FP64 (phi_hi - c for FP32), in the
// lattice order (x fastest): the data of output_cube
// (Discrete/Bubble-Collisions/outputfile.f90:942-1016).
template <typename R, bool KAHAN>
__global__ void cube_kernel(const R* __restrict__ hi, const R* __restrict__ c, int nx, int ny, int nz, int ds,
                            double* __restrict__ out) {
  const int mx = nx / ds, my = ny / ds, mz = nz / ds;
  const int64_t M = (int64_t)mx * my * mz;
  for (int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; o < M; o += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(o % mx), j = (int)((o / mx) % my), k = (int)(o / ((int64_t)mx * my));
    const int64_t s = ((int64_t)k * ds * ny + (int64_t)j * ds) * nx + (int64_t)i * ds;
    out[o] = KAHAN ? (double)hi[s] - (double)c[s] : (double)hi[s];
  }
}

int launch_cube(const void* hi, const void* c, int nx, int ny, int nz, int ds, int precision, double* out,
                cudaStream_t s) {
  const int64_t M = (int64_t)(nx / ds) * (ny / ds) * (nz / ds);
  if (precision == LAT_FP64)
    cube_kernel<double, false><<<grid_for(M), 256, 0, s>>>((const double*)hi, nullptr, nx, ny, nz, ds, out);
  else if (c)
    cube_kernel<float, true><<<grid_for(M), 256, 0, s>>>((const float*)hi, (const float*)c, nx, ny, nz, ds, out);
  else
    cube_kernel<float, false><<<grid_for(M), 256, 0, s>>>((const float*)hi, nullptr, nx, ny, nz, ds, out);
  return done("cube");
}

int launch_to_fp64(const void* hi, const void* c, int64_t n, int precision, double* out, cudaStream_t s) {
  if (precision == LAT_FP64) to64_kernel<double, false><<<grid_for(n), 256, 0, s>>>((const double*)hi, nullptr, n, out);
  else to64_kernel<float, true><<<grid_for(n), 256, 0, s>>>((const float*)hi, (const float*)c, n, out);
  return done("to_fp64");
}
int launch_from_fp64(const double* in, int64_t n, int precision, void* hi, void* c, cudaStream_t s) {
  if (precision == LAT_FP64) from64_kernel<double, false><<<grid_for(n), 256, 0, s>>>(in, n, (double*)hi, nullptr);
  else from64_kernel<float, true><<<grid_for(n), 256, 0, s>>>(in, n, (float*)hi, (float*)c);
  return done("from_fp64");
}

int launch_spectrum(const SpecArgs& a, int precision, cudaStream_t s) {
  const size_t smem = (size_t)3 * a.nbins * sizeof(double);
  if (precision == LAT_FP64) spec_kernel<double, double2><<<a.grid, a.block, smem, s>>>(a);
  else spec_kernel<float, float2><<<a.grid, a.block, smem, s>>>(a);
  return done("spectrum");
}

int launch_gw_spectrum(const GwSpecArgs& a, int precision, cudaStream_t s) {
  const size_t smem = (size_t)2 * a.nbins * sizeof(double);
  if (precision == LAT_FP64) gwspec_kernel<double, double2><<<a.grid, a.block, smem, s>>>(a);
  else gwspec_kernel<float, float2><<<a.grid, a.block, smem, s>>>(a);
  return done("gw spectrum");
}

int launch_energy(const EnergyArgs& a, int precision, cudaStream_t s) {
  if (a.nf == 1) {
    if (precision == LAT_FP64) energy_kernel<double, false, 1><<<a.grid, a.block, 0, s>>>(a);
    else energy_kernel<float, true, 1><<<a.grid, a.block, 0, s>>>(a);
  } else if (a.nf == 2) {
    if (precision == LAT_FP64) energy_kernel<double, false, 2><<<a.grid, a.block, 0, s>>>(a);
    else energy_kernel<float, true, 2><<<a.grid, a.block, 0, s>>>(a);
  } else {
    return set_error(LAT_ERR_UNSUPPORTED, "energies support nfld = 1 or 2");
  }
  return done("energy");
}

int launch_parseval(const void* Fk, int nx, int ny, int nz, int nf, double dkx2, double dky2, double dkz2,
                    DevScalars* sc, int slot, RedBuf rb, int grid, int precision, cudaStream_t s) {
  if (precision == LAT_FP64)
    parseval_kernel<double, double2><<<grid, 256, 0, s>>>((const double2*)Fk, nx, ny, nz, nf, dkx2, dky2, dkz2, sc, slot, rb);
  else
    parseval_kernel<float, float2><<<grid, 256, 0, s>>>((const float2*)Fk, nx, ny, nz, nf, dkx2, dky2, dkz2, sc, slot, rb);
  return done("parseval");
}

int launch_vacuum_modes(const VacArgs& a, cudaStream_t s) {
  const int64_t M = (int64_t)(a.nx / 2 + 1) * a.ny * a.nz;
  vacuum_kernel<<<grid_for(M), 256, 0, s>>>(a);
  return done("vacuum");
}
int launch_fd_laplacian64(const double* in, double* out, int nx, int ny, int nz, const double* lc, cudaStream_t s) {
  fd_lap64_kernel<<<grid_for((int64_t)nx * ny * nz), 256, 0, s>>>(in, out, nx, ny, nz, lc[0], lc[1], lc[2], lc[3]);
  return done("fd laplacian");
}
int launch_sample_steps(int step, const SampleArgs& a, cudaStream_t s) {
  const int blk = 256;
  auto grid = [&](int64_t n) { return (unsigned)std::min<int64_t>((n + blk - 1) / blk, 4096); };
  switch (step) {
    case 0: sample_dst_in_kernel<<<grid(4LL * a.nos), blk, 0, s>>>(a.z, a.nos, a.dkos, a.m2, a.gamma, a.kcut); break;
    case 1: sample_dst_out_kernel<<<grid(a.nos), blk, 0, s>>>(a.z, a.nos, a.norm, a.ker); break;
    case 2: sample_kernel3d<<<grid((int64_t)a.n * a.n * a.n), blk, 0, s>>>(a.ker, a.n, a.f); break;
    case 3: sample_noise_kernel<<<grid(a.M), blk, 0, s>>>(a.F, a.M, a.seed, a.stream); break;
    case 4: sample_hermitize_kernel<<<grid(2LL * a.n * a.n), blk, 0, s>>>(a.F, a.n); break;
    default: return set_error(LAT_ERR_ARG, "sample step");
  }
  if (g_launch_counter) ++*g_launch_counter;
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? LAT_OK : cuda_fail(e, "sample launch");
}

int launch_add_scale(double* f, int64_t n, double scale, double offset, cudaStream_t s) {
  add_scale_kernel<<<grid_for(n), 256, 0, s>>>(f, n, scale, offset);
  return done("add_scale");
}
int launch_bubbles(double* phi, int nx, int ny, int nz, double dx, int nbub, const double* cen, double R, double w,
                   cudaStream_t s) {
  bubbles_kernel<<<grid_for((int64_t)nx * ny * nz), 256, 0, s>>>(phi, nx, ny, nz, dx, nbub, cen, R, w);
  return done("bubbles");
}

}  // namespace lat
