// k_coarse.cu -- sharp-k filtering of a fine lattice onto a coarse one
// (training data of the learned closure; no reference counterpart).
#include <cufft.h>

#include <algorithm>

#include "engine.hpp"

namespace lat {

namespace {

// Coarse half spectrum [nc][nc][nc/2+1] from the fine half spectrum
// [fnz][fny][fnx/2+1]: modes with |k| < nc/2 on every axis, times `scale`;
// the coarse Nyquist planes are zero.
__global__ void truncate_kernel(const double2* __restrict__ Ff, int fnx, int fny, int fnz, double2* __restrict__ Fc,
                                int nc, double scale) {
  const int hc = nc / 2 + 1, hf = fnx / 2 + 1;
  const int64_t total = (int64_t)hc * nc * nc;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(e % hc);
    const int j = (int)((e / hc) % nc);
    const int k = (int)(e / ((int64_t)hc * nc));
    double2 v = make_double2(0.0, 0.0);
    if (i != nc / 2 && j != nc / 2 && k != nc / 2) {
      const int kj = j < nc / 2 ? j : j - nc, kk = k < nc / 2 ? k : k - nc;
      const int fj = kj < 0 ? kj + fny : kj, fk = kk < 0 ? kk + fnz : kk;
      const double2 f = Ff[((int64_t)fk * fny + fj) * hf + i];
      v = make_double2(f.x * scale, f.y * scale);
    }
    Fc[e] = v;
  }
}

// V'_f of every field at every fine site, FP64 from phi_hi - c
template <typename R, int NF>
__global__ void dv_fine_kernel(const R* __restrict__ fld, const R* __restrict__ c, int64_t N, ModelP m,
                               double* __restrict__ out) {
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < N; s += (int64_t)gridDim.x * blockDim.x) {
    double f[NF], dv[NF];
#pragma unroll
    for (int l = 0; l < NF; ++l) f[l] = (double)fld[l * N + s] - (c ? (double)c[l * N + s] : 0.0);
    model_dv<double, NF>(m, f, dv);
#pragma unroll
    for (int l = 0; l < NF; ++l) out[l * N + s] = dv[l];
  }
}

// out[s] = V'_f(phi_c(s)) - filt[s]
template <int NF>
__global__ void delta_kernel(const double* __restrict__ phic, const double* __restrict__ filt, int f, int64_t Nc,
                             ModelP m, double scale, float* __restrict__ out) {
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < Nc; s += (int64_t)gridDim.x * blockDim.x) {
    double p[NF], dv[NF];
#pragma unroll
    for (int l = 0; l < NF; ++l) p[l] = phic[l * Nc + s];
    model_dv<double, NF>(m, p, dv);
    out[s] = (float)((dv[f] - filt[s]) * scale);
  }
}

__global__ void to_f32_kernel(const double* __restrict__ in, int64_t n, double scale, float* __restrict__ out) {
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n; s += (int64_t)gridDim.x * blockDim.x)
    out[s] = (float)(in[s] * scale);
}

unsigned grid_of(int64_t n) { return (unsigned)std::min<int64_t>((n + 255) / 256, 152 * 16); }

int done(const char* where) {
  if (g_launch_counter) ++*g_launch_counter;
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? LAT_OK : cuda_fail(e, where);
}

}  // namespace

int launch_truncate(const double2* Ff, int fnx, int fny, int fnz, double2* Fc, int nc, double scale,
                    cudaStream_t s) {
  truncate_kernel<<<grid_of((int64_t)(nc / 2 + 1) * nc * nc), 256, 0, s>>>(Ff, fnx, fny, fnz, Fc, nc, scale);
  return done("truncate launch");
}

int launch_dv_fine(const void* fld, const void* c, int nf, int64_t N, const ModelP& m, int precision, double* out,
                   cudaStream_t s) {
  if (precision == LAT_FP64) {
    if (nf == 1) dv_fine_kernel<double, 1><<<grid_of(N), 256, 0, s>>>((const double*)fld, nullptr, N, m, out);
    else dv_fine_kernel<double, 2><<<grid_of(N), 256, 0, s>>>((const double*)fld, nullptr, N, m, out);
  } else {
    if (nf == 1) dv_fine_kernel<float, 1><<<grid_of(N), 256, 0, s>>>((const float*)fld, (const float*)c, N, m, out);
    else dv_fine_kernel<float, 2><<<grid_of(N), 256, 0, s>>>((const float*)fld, (const float*)c, N, m, out);
  }
  return done("dv launch");
}

int launch_delta(const double* phic, const double* filt, int f, int nf, int64_t Nc, const ModelP& m, double scale,
                 float* out, cudaStream_t s) {
  if (nf == 1) delta_kernel<1><<<grid_of(Nc), 256, 0, s>>>(phic, filt, f, Nc, m, scale, out);
  else delta_kernel<2><<<grid_of(Nc), 256, 0, s>>>(phic, filt, f, Nc, m, scale, out);
  return done("delta launch");
}

int launch_to_f32(const double* in, int64_t n, double scale, float* out, cudaStream_t s) {
  to_f32_kernel<<<grid_of(n), 256, 0, s>>>(in, n, scale, out);
  return done("f32 launch");
}

}  // namespace lat
