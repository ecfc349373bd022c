// k_noalloc.cu -- binned power spectrum that allocates no memory.
//
// For callers that cannot call cudaMalloc: a Fortran or C driver that has
// handed the whole device to its own fixed memory pool, or a code that must
// not allocate once its time loop has started.  The caller passes the half
// spectrum and an output buffer, both already on the device; the scratch the
// binning needs (per-block partial bins and an arrival counter) lives in the
// fixed file-scope array below.
//
// The array is a static __device__ object: every GPU that loads this library
// holds its 1 MiB (plus a 256-byte header) until the process exits.  Every
// call shares it and it keeps the last call's contents, so calls that overlap
// on the GPU (different streams, or different host threads on one device)
// race on it; callers must order their calls.
//
// Host code must not use the array's name as a device address (in host code
// it names a host-side stand-in).  The first call on a device, with that
// device current, asks the runtime for the array's device address with
// cudaGetSymbolAddress and remembers it; make that first call before any
// stream capture on that device.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <string>

#include "engine.hpp"

namespace lat {
namespace {

constexpr int kNaMaxBins = 512;    // largest nbins accepted
constexpr int kNaMaxBlocks = 128;  // partial rows: one per block
constexpr int kNaHeader = 32;      // doubles reserved for the arrival counter
constexpr int kNaDoubles = kNaHeader + kNaMaxBlocks * 2 * kNaMaxBins;

static __device__ __align__(256) double g_na_scratch[kNaDoubles];

struct NaArgs {
  const void* F;
  int nx, ny, nz, mode, nbins;
  double* scratch;  // device address of g_na_scratch
  double* out;      // [2*nbins]: S/W, W
};

__device__ __forceinline__ int na_fold(int i0, int n) { return i0 <= n / 2 ? i0 : n - i0; }
__device__ __forceinline__ int na_isqrt(int m) {
  int r = (int)sqrtf((float)m);
  while (r * r > m) --r;
  while ((r + 1) * (r + 1) <= m) ++r;
  return r;
}

// Same binning as lat_spectrum: full-x-range Hermitian weights, integer shell
// index, smooth two-bin weights in uncontracted FP64 (spectrum_3d,
// Pseudospec/openmp_dev/analysis_spec.f90:86-101) or integer counts
// (spectrum_bin, Discrete/Bubble-Collisions/analysis.f90:203-221).
template <typename C>
__global__ void __launch_bounds__(256) na_spec_kernel(NaArgs a) {
  extern __shared__ double shb[];  // [2][nbins]
  const int nb = a.nbins;
  for (int i = threadIdx.x; i < 2 * nb; i += blockDim.x) shb[i] = 0.0;
  __syncthreads();
  const C* F = static_cast<const C*>(a.F);
  const unsigned int hx = a.nx / 2 + 1, ny = a.ny;
  const unsigned int M = hx * ny * (unsigned int)a.nz;
  for (unsigned int m = blockIdx.x * blockDim.x + threadIdx.x; m < M; m += gridDim.x * blockDim.x) {
    const int x = (int)(m % hx);
    const unsigned int r = m / hx;
    const int y = (int)(r % ny), z = (int)(r / ny);
    const int jj = na_fold(y, a.ny), kk = na_fold(z, a.nz);
    const double wx = (x == 0 || 2 * x == a.nx) ? 1.0 : 2.0;
    const int m2 = x * x + jj * jj + kk * kk;
    const int l = na_isqrt(m2);
    const C f = F[m];
    const double v = (double)f.x * (double)f.x + (double)f.y * (double)f.y;
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
      }
      if (l + 1 < nb) {
        atomicAdd(&shb[l + 1], wx * c1 * v);
        atomicAdd(&shb[nb + l + 1], wx * c1);
      }
    }
  }
  __syncthreads();
  // partial rows in the static scratch; the last block to arrive sums them in
  // block order, writes S/W and W, and leaves the counter at zero
  double* partials = a.scratch + kNaHeader;
  unsigned int* counter = reinterpret_cast<unsigned int*>(a.scratch);
  __shared__ int am_last;
  for (int i = threadIdx.x; i < 2 * nb; i += blockDim.x) partials[(size_t)blockIdx.x * 2 * nb + i] = shb[i];
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) am_last = (atomicAdd(counter, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!am_last) return;
  __threadfence();
  for (int l = threadIdx.x; l < nb; l += blockDim.x) {
    double s = 0.0, w = 0.0;
    for (int b = 0; b < (int)gridDim.x; ++b) {
      s += __ldcg(&partials[(size_t)b * 2 * nb + l]);
      w += __ldcg(&partials[(size_t)b * 2 * nb + nb + l]);
    }
    a.out[l] = w != 0.0 ? s / w : s;
    a.out[nb + l] = w;
  }
  if (threadIdx.x == 0) *counter = 0u;
}

// Device address of g_na_scratch per device ordinal, looked up by the first
// call on that device and kept for the life of the process (a device reset
// after that call is not supported).
std::mutex g_na_mu;
double* g_na_addr[64] = {};

}  // namespace
}  // namespace lat

using namespace lat;

extern "C" int lat_spectrum_noalloc(const void* Fk_dev, int32_t nx, int32_t ny, int32_t nz, int32_t precision,
                                    int32_t mode, int32_t nbins, double* out_dev, void* stream) {
  if (!Fk_dev || !out_dev) return set_error(LAT_ERR_ARG, "null device pointer");
  if (nx < 2 || ny < 2 || nz < 2) return set_error(LAT_ERR_ARG, "bad lattice shape");
  if ((int64_t)(nx / 2 + 1) * ny * nz >= ((int64_t)1 << 31)) return set_error(LAT_ERR_ARG, "lattice too large");
  if (nbins < 1 || nbins > kNaMaxBins)
    return set_error(LAT_ERR_ARG, "nbins must be 1.." + std::to_string(kNaMaxBins) +
                                      " (the fixed scratch of lat_spectrum_noalloc holds no more)");
  if (mode != LAT_SPEC_WEIGHTED && mode != LAT_SPEC_COUNT) return set_error(LAT_ERR_ARG, "bad spectrum mode");
  if (precision != LAT_FP64 && precision != LAT_FP32_KAHAN) return set_error(LAT_ERR_ARG, "bad precision");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev < 0 || dev >= 64) return set_error(LAT_ERR_ARG, "device ordinal out of range");
  double* scratch;
  {
    std::lock_guard<std::mutex> lk(g_na_mu);
    if (!g_na_addr[dev]) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_na_scratch);
      if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress");
      g_na_addr[dev] = static_cast<double*>(p);
    }
    scratch = g_na_addr[dev];
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // the arrival counter must start at zero.  The last block of every
  // completed launch resets it, but a launch that was aborted (a failed
  // launch, a lost context that was recovered) can leave it set, and a stale
  // count would make a block other than the last one sum the partials: keep
  // this memset.
  e = cudaMemsetAsync(scratch, 0, kNaHeader * sizeof(double), s);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync");
  NaArgs a{};
  a.F = Fk_dev;
  a.nx = nx; a.ny = ny; a.nz = nz;
  a.mode = mode;
  a.nbins = nbins;
  a.scratch = scratch;
  a.out = out_dev;
  const int64_t M = (int64_t)(nx / 2 + 1) * ny * nz;
  int grid = (int)std::min<int64_t>(kNaMaxBlocks, (M + 255) / 256);
  const size_t smem = (size_t)2 * nbins * sizeof(double);
  if (precision == LAT_FP64) na_spec_kernel<double2><<<grid, 256, smem, s>>>(a);
  else na_spec_kernel<float2><<<grid, 256, smem, s>>>(a);
  e = cudaGetLastError();
  return e == cudaSuccess ? LAT_OK : cuda_fail(e, "lat_spectrum_noalloc launch");
}
