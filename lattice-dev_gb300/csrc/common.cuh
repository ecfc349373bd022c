// common.cuh -- shared device helpers of the GB300 lattice engine (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/lattice.h"

namespace lat {

// ------------------------------------------------------------ precision
template <int P> struct Prec;
template <> struct Prec<LAT_FP64> {
  using real = double;
  using cplx = double2;
  static constexpr bool kahan = false;
};
template <> struct Prec<LAT_FP32_KAHAN> {
  using real = float;
  using cplx = float2;
  static constexpr bool kahan = true;
};

// ------------------------------------------------------------- scalars
// FP64 scalar block resident in HBM.  The Friedmann variables and the
// lattice sums that feed them never leave the device during an evolution.
struct DevScalars {
  double a;        // scale factor yscl
  double ap;       // its conjugate momentum ysclp
  double pe;       // <V(phi)> of the current fields (set by the last drift pass)
  double ge2;      // (1/N) sum_k k^2 |F_k|^2 over fields = -sum_x phi lap phi (last k-space pass)
  double ke2;      // sum_x pi^2 of the last drift pass (diagnostic)
  double red[16];  // raw sums of the last stand-alone reduction (energies)
  double gsum[3];  // -sum phi d2_axis(phi) of the separable passes X, Y, Z
  double mean[4];  // lattice means of the fields (spectral shift of the separable passes)
  double ke_cur;   // sum pi^2 of the current momenta, kept by the streamed passes
  float co[4];     // FP32 cd, ck, cv of the next streamed kick (kick_coefs_of), from the kernel before it
  unsigned int err;  // bit 0: NaN/Inf met in a reduction; bit 1: a bounded device wait gave up
  unsigned int pad[3];
};

// The FP32 coefficients of a streamed kick from the FP64 scalar state before
// it (hamiltonian_conformal.f90:86-174): cd = hd/a0^2 for the drift of pass
// X, ck = hk a1^2 and cv = hk a1^4 for the kick, where a1 = a0 - hg ap0/6
// follows the drift's ysclp update ap0 = ap + hd (ke/N)/a0^3.  Evaluated once
// per kick by the single-block kernel before it (k_spec.cu), never in the
// passes: at GB300's FP64 rate the chain's divisions and dependent loads held
// the start of every pass that evaluated it.  One reciprocal of a0 serves
// every quotient, and 1/N, 1/6 fold into products: each FP64 division is a
// dependent chain on the critical path between pass Z and the next pass X.
__device__ __forceinline__ void kick_coefs_of(double a0, double ap, double ke, double hd, double hk, double hg,
                                              double Nd, float* c) {
  const double r = 1.0 / a0, r2 = r * r;
  const double ap0 = ap + hd * ke * (1.0 / Nd) * (r2 * r);
  const double a1 = a0 - (hg * (1.0 / 6.0)) * ap0;
  c[0] = (float)(hd * r2);
  const double k1 = hk * a1 * a1;
  c[1] = (float)k1;
  c[2] = (float)(k1 * a1 * a1);
}

// Programmatic dependent launch: a kernel launched with programmatic stream
// serialization may start while its predecessor in the stream drains.  It
// must call pdl_wait() before it reads anything the predecessor writes
// (wait returns once the predecessor grid has completed and its memory is
// visible; without a programmatic predecessor it returns at once).  Every
// kernel of such a chain calls pdl_trigger() only after its own pdl_wait(),
// so a kernel's successor never starts before the kernel's own predecessor
// has completed: anything written two kernels back may be read before the
// wait.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory"); }

// Reduction scratch: one partial row per block plus an arrival counter.
struct RedBuf {
  double* partials;       // [max_blocks * 16]
  unsigned int* counter;  // single word, left at zero after every kernel
};

// Model parameters as both precisions (the kernels pick by R).
struct ModelP {
  int model;
  double p[4];
};

// ---------------------------------------------------------- reductions
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// Float-float value hi + lo: the warp-level partial sums of compensated FP32
// accumulators.  GB300 runs FP64 at a small fraction of its FP32 rate, so a
// warp's 31 additions run on the FP32 pipes (relative error ~2^-47) and only
// the warp's total is converted to FP64.
struct FF {
  float hi, lo;
};
// Knuth's TwoSum: s + e == a + b exactly (round-to-nearest, no reassociation)
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bv = s - a;
  e = (a - (s - bv)) + (b - bv);
}
__device__ __forceinline__ FF ff_add(FF a, FF b) {
  float s, e, hi, lo;
  two_sum(a.hi, b.hi, s, e);
  e += a.lo + b.lo;
  two_sum(s, e, hi, lo);  // renormalise
  return FF{hi, lo};
}
__device__ __forceinline__ double warp_sum(FF v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const FF w{__shfl_down_sync(0xffffffffu, v.hi, o), __shfl_down_sync(0xffffffffu, v.lo, o)};
    v = ff_add(v, w);
  }
  return (double)v.hi + (double)v.lo;
}

// Compensated FP32 accumulator: per-thread partial sums stay in FP32 while
// keeping ~FP64 accuracy; red() hands the sum s - c to the reductions as a
// float-float value.
struct KSum {
  using Red = FF;
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float x) {
    float y = x - c;
    float t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __device__ __forceinline__ double val() const { return (double)s - (double)c; }
  __device__ __forceinline__ FF red() const { return FF{s, -c}; }
};
struct DSum {
  using Red = double;
  double s = 0.0;
  __device__ __forceinline__ void add(double x) { s += x; }
  __device__ __forceinline__ double val() const { return s; }
  __device__ __forceinline__ double red() const { return s; }
};
template <typename R> struct AccOf;
template <> struct AccOf<float> { using type = KSum; };
template <> struct AccOf<double> { using type = DSum; };

// Deterministic grid reduction of NV values (doubles, or float-float warp
// inputs): block partials are written in block order and the last block to
// arrive sums them in a fixed order, so two identical launches give
// bit-identical totals.  Returns true in thread 0 of the last block, with
// `total` filled; the counter is reset for the next launch (graph replays
// reuse it).  All threads of every block must call it.
template <int NV, typename T>
__device__ __forceinline__ bool grid_reduce(const T (&v)[NV], const RedBuf rb, double (&total)[NV]) {
  __shared__ double sh[NV][32];
  __shared__ int am_last;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nthreads = blockDim.x * blockDim.y * blockDim.z;
  const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int lane2 = tid & 31, wid2 = tid >> 5, nw = (nthreads + 31) >> 5;
  (void)lane; (void)wid;
  const int bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
  const int nblk = gridDim.x * gridDim.y * gridDim.z;
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    double x = warp_sum(v[i]);
    if (lane2 == 0) sh[i][wid2] = x;
  }
  __syncthreads();
  if (wid2 == 0) {
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      double x = lane2 < nw ? sh[i][lane2] : 0.0;
      x = warp_sum(x);
      if (lane2 == 0) rb.partials[(size_t)bid * NV + i] = x;
    }
    if (lane2 == 0) {
      __threadfence();
      unsigned int t = atomicAdd(rb.counter, 1u);
      am_last = (t == (unsigned int)nblk - 1u);
    }
  }
  __syncthreads();
  if (!am_last) return false;
  __threadfence();
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    double x = 0.0;
    for (int b = tid; b < nblk; b += nthreads) x += __ldcg(&rb.partials[(size_t)b * NV + i]);
    x = warp_sum(x);
    __syncthreads();
    if (lane2 == 0) sh[i][wid2] = x;
  }
  __syncthreads();
  if (tid != 0) return false;
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    double s = 0.0;
    for (int w = 0; w < nw; ++w) s += sh[i][w];
    total[i] = s;
  }
  *rb.counter = 0u;
  return true;
}

// Block sums of NV doubles written to out[blockIdx.x * NV + i] by thread 0:
// the partials of a reduction that a later kernel completes in block order
// (no fence or arrival counter in the pass).  All threads must call it.
template <int NV, typename T>
__device__ __forceinline__ void block_partials(const T (&v)[NV], double* out) {
  __shared__ double sh[NV][32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    const double x = warp_sum(v[i]);
    if (lane == 0) sh[i][wid] = x;
  }
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      const double x = warp_sum(lane < nw ? sh[i][lane] : 0.0);
      if (lane == 0) out[(size_t)blockIdx.x * NV + i] = x;
    }
  }
}

__device__ __forceinline__ bool bad(double x) { return !(x - x == 0.0); }

// ---------------------------------------------------------------- models
// potential / modeldv of the reference models (V, not DEFROST's 2V).
template <typename R, int NF>
__device__ __forceinline__ void model_dv(const ModelP& m, const R (&f)[NF], R (&dv)[NF]) {
  const R p0 = (R)m.p[0], p1 = (R)m.p[1];
  switch (m.model) {
    case LAT_MODEL_PHI4:
      dv[0] = p0 * f[0] * f[0] * f[0];
#pragma unroll
      for (int l = 1; l < NF; ++l) dv[l] = R(0);
      break;
    case LAT_MODEL_PHI4_G2:
      if constexpr (NF >= 2) {
        dv[0] = p0 * f[0] * f[0] * f[0] + p1 * f[0] * f[1] * f[1];
        dv[1] = p1 * f[0] * f[0] * f[1];
      } else {
        dv[0] = p0 * f[0] * f[0] * f[0];
      }
      break;
    case LAT_MODEL_DOUBLE_WELL:
      dv[0] = (f[0] * f[0] - R(1)) * f[0] - p0;
#pragma unroll
      for (int l = 1; l < NF; ++l) dv[l] = R(0);
      break;
    default:  // LAT_MODEL_FREE
#pragma unroll
      for (int l = 0; l < NF; ++l) dv[l] = p0 * f[l];
      break;
  }
}
template <typename R, int NF>
__device__ __forceinline__ R model_v(const ModelP& m, const R (&f)[NF]) {
  const R p0 = (R)m.p[0], p1 = (R)m.p[1];
  switch (m.model) {
    case LAT_MODEL_PHI4: return R(0.25) * p0 * f[0] * f[0] * f[0] * f[0];
    case LAT_MODEL_PHI4_G2:
      if constexpr (NF >= 2)
        return R(0.25) * p0 * f[0] * f[0] * f[0] * f[0] + R(0.5) * p1 * f[0] * f[0] * f[1] * f[1];
      else
        return R(0.25) * p0 * f[0] * f[0] * f[0] * f[0];
    case LAT_MODEL_DOUBLE_WELL: {
      R s = f[0] * f[0] - R(1);
      return R(0.25) * s * s - p0 * (f[0] + R(1));
    }
    default: {
      R v = R(0);
#pragma unroll
      for (int l = 0; l < NF; ++l) v += R(0.5) * p0 * f[l] * f[l];
      return v;
    }
  }
}

// Kahan-compensated drift x += inc, true value = x - c.
__device__ __forceinline__ void kahan_add(float& x, float& c, float inc) {
  float y = inc - c;
  float t = x + y;
  c = (t - x) - y;
  x = t;
}

// folded frequency |k| index of a DFT index i0 in [0,n)
__device__ __forceinline__ int fold_idx(int i0, int n) { return i0 <= n / 2 ? i0 : n - i0; }

// exact floor(sqrt(m)) for 0 <= m < 2^31
__device__ __forceinline__ int isqrt_exact(int m) {
  int r = (int)sqrtf((float)m);
  while (r * r > m) --r;
  while ((r + 1) * (r + 1) <= m) ++r;
  return r;
}

}  // namespace lat
