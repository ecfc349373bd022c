// ensemble.cu -- batched ensembles of independent lattices of uneven size.
//
// No reference counterpart: the reference runs one lattice per job (one PBS
// submission per seed, Pseudospec/openmp_dev/submit_defrost).  Here all runs
// live in one set of concatenated arrays, grouped by size class:
//
//   fld/fldc/fldp/lap : [class][run][z][y][x]   (sites)
//   Fk                : [class][run][z][y][n/2+1] (half spectra)
//
// A pass over the ensemble is ONE persistent launch whose blocks stride over a
// segment table (one segment per size class, each with its own step sizes and
// wavenumber scale), so every run advances in the same launch whatever its
// size; the only other launches are one batched cuFFT plan per size class.
// A whole symp call is captured once in a CUDA graph and replayed.
// Spectral Laplacian, Minkowski background, one field.
#include <cufft.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "engine.hpp"
#include "integrator.hpp"

namespace lat {

namespace {

constexpr int kMaxSeg = 8;

struct EnsSeg {
  long long v0, v1;  // [v0, v1) in units of 4 sites (pointwise) or complex entries (kmul)
  double ck, cd;     // kick and drift coefficients of this class for the current op
  int n;             // lattice side
  double dk2;        // (2 pi / L)^2
  double invN;
};
struct EnsArgs {
  EnsSeg seg[kMaxSeg];
  int nseg;
  int mode;  // 0 = kick+drift, 1 = drift
  void* phi;
  void* phic;
  void* pi;
  const void* lap;
  void* Fk;
  ModelP model;
};

template <typename R> struct V4;
template <> struct V4<float> {
  using T = float4;
  static __device__ __forceinline__ void ld(const float* p, float (&v)[4]) {
    float4 t = __ldcs(reinterpret_cast<const float4*>(p));
    v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
  }
  static __device__ __forceinline__ void st(float* p, const float (&v)[4]) {
    __stcs(reinterpret_cast<float4*>(p), make_float4(v[0], v[1], v[2], v[3]));
  }
};
template <> struct V4<double> {
  static __device__ __forceinline__ void ld(const double* p, double (&v)[4]) {
    double2 a = __ldcs(reinterpret_cast<const double2*>(p)), b = __ldcs(reinterpret_cast<const double2*>(p) + 1);
    v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
  }
  static __device__ __forceinline__ void st(double* p, const double (&v)[4]) {
    __stcs(reinterpret_cast<double2*>(p), make_double2(v[0], v[1]));
    __stcs(reinterpret_cast<double2*>(p) + 1, make_double2(v[2], v[3]));
  }
};

// Persistent kick+drift (or drift) over every run of every size class.
template <typename R, bool KAHAN, int MODE>
__global__ void __launch_bounds__(256) ens_pw_kernel(EnsArgs a) {
  R* phi = static_cast<R*>(a.phi);
  R* phic = static_cast<R*>(a.phic);
  R* pi = static_cast<R*>(a.pi);
  const R* lap = static_cast<const R*>(a.lap);
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long total = a.seg[a.nseg - 1].v1;
  int s = 0;
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < total; v += stride) {
    while (v >= a.seg[s].v1) ++s;
    const R ck = (R)a.seg[s].ck, cd = (R)a.seg[s].cd;
    const long long o = v * 4;
    R f[4], c[4], p[4], l[4];
    V4<R>::ld(phi + o, f);
    if (KAHAN) V4<R>::ld(phic + o, c);
    V4<R>::ld(pi + o, p);
    if (MODE == 0) V4<R>::ld(lap + o, l);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      if (MODE == 0) {
        R ff[1] = {f[j]}, dv[1];
        model_dv<R, 1>(a.model, ff, dv);
        p[j] = p[j] + ck * (l[j] - dv[0]);
      }
      if constexpr (KAHAN) kahan_add(f[j], c[j], cd * p[j]);
      else f[j] = f[j] + cd * p[j];
    }
    V4<R>::st(phi + o, f);
    if (KAHAN) V4<R>::st(phic + o, c);
    if (MODE == 0) V4<R>::st(pi + o, p);
  }
}

// Persistent k-space multiply F *= -k^2/N over every run's half spectrum.
template <typename R, typename C>
__global__ void __launch_bounds__(256) ens_kmul_kernel(EnsArgs a) {
  C* F = static_cast<C*>(a.Fk);
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long total = a.seg[a.nseg - 1].v1;
  int s = 0;
  for (long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x; m < total; m += stride) {
    while (m >= a.seg[s].v1) ++s;
    const int n = a.seg[s].n;
    const unsigned int hx = n / 2 + 1;
    const unsigned int M = hx * (unsigned int)n * (unsigned int)n;
    const unsigned int mm = (unsigned int)((m - a.seg[s].v0) % M);
    const int x = (int)(mm % hx);
    const unsigned int r = mm / hx;
    const int y = (int)(r % (unsigned int)n), z = (int)(r / (unsigned int)n);
    const int jj = fold_idx(y, n), kk = fold_idx(z, n);
    const R scl = -(R)(x * x + jj * jj + kk * kk) * (R)a.seg[s].dk2 * (R)a.seg[s].invN;
    C v = F[m];
    v.x *= scl;
    v.y *= scl;
    F[m] = v;
  }
}

// phi at site 0 of every run of a class: the first pass X's shifts
__global__ void run_shift_init_kernel(const float* __restrict__ phi, int64_t nsite, int runs,
                                      float* __restrict__ shift_b) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < runs) shift_b[r] = phi[(int64_t)r * nsite];
}

struct EnsGraph {
  int order;
  double dto;
  int nsteps;
  int64_t kernels;
  cudaGraphExec_t exec;
};

}  // namespace
}  // namespace lat

using namespace lat;

struct lat_ens_s {
  lat_config base{};
  int prec = LAT_FP32_KAHAN;
  size_t rsz = 4, csz = 8;
  int dev = 0, nsm = 152;
  cudaStream_t stream = nullptr;
  struct Cls {
    int n = 0, count = 0;
    int64_t site_off = 0, fk_off = 0;  // elements
    cufftHandle r2c = 0, c2r = 0, r2c1 = 0, z2d1 = 0;
    bool have = false;
    double dx = 0, dk = 0;
    float2* tw = nullptr;     // W_n^j (streamed separable passes)
    float* shift = nullptr;   // [2][count] zs shift per run: written by pass X / pass Z
    // the class's streamed passes run on their own stream, forked from and
    // joined to the ensemble's stream around every kick (graph branches)
    cudaStream_t side = nullptr;
    cudaEvent_t done = nullptr;
    // tensor maps of passes Y and Z (zs and momenta of the class's pairs),
    // encoded once: the class's arrays never move
    CUtensorMap tm_zs[2] = {}, tm_pi[2] = {};
    bool tm_ok[2] = {false, false};
  };
  std::vector<Cls> cls;
  std::vector<int> run_cls;
  std::vector<int64_t> run_off, run_fk;
  int64_t Ntot = 0, Mtot = 0;
  void *phi = nullptr, *phic = nullptr, *pi = nullptr, *lap = nullptr, *Fk = nullptr;
  void* work = nullptr;
  size_t work_size = 0;
  DevScalars* sc = nullptr;
  RedBuf rb{};
  double* spec_part = nullptr;
  double* spec_out = nullptr;
  unsigned int* spec_counter = nullptr;
  int grid = 0, block = 256;
  bool sep_ok = false;  // every class can run the streamed separable passes (pairs of runs)
  bool sep = false;     // and they are in use (else cuFFT per class)
  int64_t launches = 0;
  std::vector<EnsGraph> graphs;
  cudaEvent_t marks[16] = {};
  cudaEvent_t fork = nullptr;  // start of a kick on the ensemble's stream
};

namespace {

#define ECK(x)                                                  \
  do {                                                          \
    cudaError_t e_ = (x);                                       \
    if (e_ != cudaSuccess) return cuda_fail(e_, #x);            \
  } while (0)
#define ECF(x)                                                                              \
  do {                                                                                      \
    cufftResult r_ = (x);                                                                   \
    if (r_ != CUFFT_SUCCESS) return set_error(LAT_ERR_CUDA, std::string(#x) + ": cuFFT error"); \
  } while (0)
#define ERET(x)                \
  do {                         \
    int s_ = (x);              \
    if (s_ != LAT_OK) return s_; \
  } while (0)

struct EGuard {
  explicit EGuard(lat_ens_s* e) {
    g_launch_counter = &e->launches;
    cudaSetDevice(e->dev);
  }
  ~EGuard() { g_launch_counter = nullptr; }
};

int plan(lat_ens_s* e, cufftHandle* p, int n, int batch, cufftType t) {
  ECF(cufftCreate(p));
  ECF(cufftSetAutoAllocation(*p, 0));
  int dims[3] = {n, n, n};
  const long long N = (long long)n * n * n, M = (long long)(n / 2 + 1) * n * n;
  const bool r2c = (t == CUFFT_R2C || t == CUFFT_D2Z);
  size_t ws = 0;
  ECF(cufftMakePlanMany(*p, 3, dims, nullptr, 1, (int)(r2c ? N : M), nullptr, 1, (int)(r2c ? M : N), t, batch, &ws));
  if (ws > e->work_size) {
    if (e->work) cudaFree(e->work);
    ECK(cudaMalloc(&e->work, ws));
    e->work_size = ws;
    for (auto& c : e->cls)
      if (c.have) {
        cufftSetWorkArea(c.r2c, e->work);
        cufftSetWorkArea(c.c2r, e->work);
        cufftSetWorkArea(c.r2c1, e->work);
        cufftSetWorkArea(c.z2d1, e->work);
      }
  }
  ECF(cufftSetWorkArea(*p, e->work));
  ECF(cufftSetStream(*p, e->stream));
  return LAT_OK;
}

EnsArgs base_args(lat_ens_s* e) {
  EnsArgs a{};
  a.nseg = (int)e->cls.size();
  a.phi = e->phi;
  a.phic = e->phic;
  a.pi = e->pi;
  a.lap = e->lap;
  a.Fk = e->Fk;
  a.model.model = e->base.model;
  for (int i = 0; i < 4; ++i) a.model.p[i] = e->base.model_params[i];
  return a;
}

int launch_ens_pw(lat_ens_s* e, EnsArgs a) {
  int64_t v = 0;
  for (int i = 0; i < a.nseg; ++i) {
    const int64_t n3 = (int64_t)e->cls[i].n * e->cls[i].n * e->cls[i].n * e->cls[i].count;
    a.seg[i].v0 = v / 4;
    v += n3;
    a.seg[i].v1 = v / 4;
  }
  if (e->prec == LAT_FP64) {
    if (a.mode == 0) ens_pw_kernel<double, false, 0><<<e->grid, e->block, 0, e->stream>>>(a);
    else ens_pw_kernel<double, false, 1><<<e->grid, e->block, 0, e->stream>>>(a);
  } else {
    if (a.mode == 0) ens_pw_kernel<float, true, 0><<<e->grid, e->block, 0, e->stream>>>(a);
    else ens_pw_kernel<float, true, 1><<<e->grid, e->block, 0, e->stream>>>(a);
  }
  ++e->launches;
  cudaError_t er = cudaGetLastError();
  return er == cudaSuccess ? LAT_OK : cuda_fail(er, "ensemble pass");
}

int launch_ens_kmul(lat_ens_s* e) {
  EnsArgs a = base_args(e);
  int64_t m = 0;
  for (int i = 0; i < a.nseg; ++i) {
    const auto& c = e->cls[i];
    a.seg[i].v0 = m;
    m += (int64_t)(c.n / 2 + 1) * c.n * c.n * c.count;
    a.seg[i].v1 = m;
    a.seg[i].n = c.n;
    a.seg[i].dk2 = c.dk * c.dk;
    a.seg[i].invN = 1.0 / ((double)c.n * c.n * c.n);
  }
  if (e->prec == LAT_FP64) ens_kmul_kernel<double, double2><<<e->grid, e->block, 0, e->stream>>>(a);
  else ens_kmul_kernel<float, float2><<<e->grid, e->block, 0, e->stream>>>(a);
  ++e->launches;
  cudaError_t er = cudaGetLastError();
  return er == cudaSuccess ? LAT_OK : cuda_fail(er, "ensemble k-space pass");
}

int ens_fft(lat_ens_s* e, bool forward) {
  for (auto& c : e->cls) {
    char* f = (char*)(forward ? e->phi : e->lap) + (size_t)c.site_off * e->rsz;
    char* k = (char*)e->Fk + (size_t)c.fk_off * e->csz;
    cufftResult r;
    if (e->prec == LAT_FP64)
      r = forward ? cufftExecD2Z(c.r2c, (cufftDoubleReal*)f, (cufftDoubleComplex*)k)
                  : cufftExecZ2D(c.c2r, (cufftDoubleComplex*)k, (cufftDoubleReal*)f);
    else
      r = forward ? cufftExecR2C(c.r2c, (cufftReal*)f, (cufftComplex*)k) : cufftExecC2R(c.c2r, (cufftComplex*)k, (cufftReal*)f);
    if (r != CUFFT_SUCCESS) return set_error(LAT_ERR_CUDA, "ensemble cuFFT exec");
  }
  return LAT_OK;
}

// One streamed separable pass (k_sep_stream.cuh) over every pair of runs of
// class c: in place, kick weight hk and preceding drift hd in units of dt.
int ens_sep_pass(lat_ens_s* e, lat_ens_s::Cls& c, int axis, double hk, double hd, double dto) {
  const int64_t n = c.n, n3 = n * n * n;
  const double dt = dto * c.dx;
  SepArgs a{};
  a.nx = a.ny = a.nz = c.n;
  a.nf = 1;
  float* f = (float*)e->phi + c.site_off;
  float* fc = (float*)e->phic + c.site_off;
  float* p = (float*)e->pi + c.site_off;
  float* z = (float*)e->lap + c.site_off;
  a.phi = a.phi_out = f;
  a.phic = a.phic_out = fc;
  a.pi = a.pi_out = p;
  a.lap = a.lap_out = z;
  a.twN = c.tw;
  a.dk2 = c.dk * c.dk;
  a.model.model = e->base.model;
  for (int i = 0; i < 4; ++i) a.model.p[i] = e->base.model_params[i];
  a.hk = hk * dt;
  a.hd = hd * dt;
  a.Nd = (double)n3;
  a.conf = 0;
  a.pair_lines = n * n;
  a.nlines = (int64_t)(c.count / 2) * a.pair_lines;
  a.nsm = e->nsm;
  a.stream = 1;
  a.runs = 1;
  a.shift_a = c.shift;
  a.shift_b = c.shift + c.count;
  a.sc = e->sc;
  a.rb = e->rb;
  if (axis > 0) {  // Y, Z: TMA tiles
    if (!c.tm_ok[axis - 1]) {
      ERET(encode_stream_tmaps(a, axis, sep_runs_lines(c.n, axis), c.n));
      c.tm_zs[axis - 1] = a.tm_zs;
      c.tm_pi[axis - 1] = a.tm_pi;
      c.tm_ok[axis - 1] = true;
    }
    a.tm_zs = c.tm_zs[axis - 1];
    a.tm_pi = c.tm_pi[axis - 1];
  }
  return launch_sep_runs(a, c.n, axis, c.side ? c.side : e->stream);
}

int ens_pw_args(lat_ens_s* e, int mode, double hk, double hd, double dto);

// The op list on the streamed passes: every kick is the passes X (carrying
// the preceding drift), Y and Z, per size class; the last drift is the
// pointwise pass.  Minkowski lists only ((D) (K D+)*).
int ens_exec_sep(lat_ens_s* e, const std::vector<Op>& ops, double dto) {
  struct Grp { double hk, hd; };
  std::vector<Grp> grp;
  double lead = 0;
  size_t i = 0;
  while (i < ops.size() && ops[i].t == 'D') lead += ops[i++].h;
  while (i < ops.size()) {
    if (ops[i].t != 'K') return set_error(LAT_ERR_STATE, "ensemble op list: kick expected");
    Grp g{ops[i++].h, 0.0};
    while (i < ops.size() && ops[i].t == 'D') g.hd += ops[i++].h;
    grp.push_back(g);
  }
  if (!grp.empty())
    for (auto& c : e->cls) {
      run_shift_init_kernel<<<(c.count + 127) / 128, 128, 0, e->stream>>>((const float*)e->phi + c.site_off,
                                                                          (int64_t)c.n * c.n * c.n, c.count,
                                                                          c.shift + c.count);
      ++e->launches;
      ECK(cudaGetLastError());
    }
  double pending = lead;
  // the size classes share no device state on these passes: every kick
  // forks one branch per class (X, Y, Z of its pairs of runs) and joins them,
  // so one class's pass tails overlap the others' passes
  const bool branches = e->fork && e->cls.size() > 1;
  for (const Grp& g : grp) {
    if (branches) ECK(cudaEventRecord(e->fork, e->stream));
    for (auto& c : e->cls) {
      if (branches) ECK(cudaStreamWaitEvent(c.side, e->fork, 0));
      ERET(ens_sep_pass(e, c, 0, g.hk, pending, dto));
      ERET(ens_sep_pass(e, c, 1, g.hk, 0.0, dto));
      ERET(ens_sep_pass(e, c, 2, g.hk, 0.0, dto));
      if (branches) ECK(cudaEventRecord(c.done, c.side));
    }
    if (branches)
      for (auto& c : e->cls) ECK(cudaStreamWaitEvent(e->stream, c.done, 0));
    pending = g.hd;
  }
  if (pending != 0.0) ERET(ens_pw_args(e, 1, 0.0, pending, dto));
  return LAT_OK;
}

int ens_pw_args(lat_ens_s* e, int mode, double hk, double hd, double dto) {
  EnsArgs a = base_args(e);
  a.mode = mode;
  for (int i = 0; i < a.nseg; ++i) {
    const double dt = dto * e->cls[i].dx;  // dt = (dt/dx) dx per size class
    a.seg[i].ck = hk * dt;
    a.seg[i].cd = hd * dt;
  }
  return launch_ens_pw(e, a);
}

int ens_exec(lat_ens_s* e, const std::vector<Op>& ops, double dto) {
  if (e->sep) return ens_exec_sep(e, ops, dto);
  auto pw = [&](int mode, double hk, double hd) { return ens_pw_args(e, mode, hk, hd, dto); };
  size_t i = 0;
  while (i < ops.size()) {
    if (ops[i].t == 'K' && i + 1 < ops.size() && ops[i + 1].t == 'D') {
      double hd = 0;
      size_t j = i + 1;
      while (j < ops.size() && ops[j].t == 'D') hd += ops[j++].h;
      ERET(ens_fft(e, true));
      ERET(launch_ens_kmul(e));
      ERET(ens_fft(e, false));
      ERET(pw(0, ops[i].h, hd));
      i = j;
    } else if (ops[i].t == 'D') {
      double hd = 0;
      size_t j = i;
      while (j < ops.size() && ops[j].t == 'D') hd += ops[j++].h;
      ERET(pw(1, 0.0, hd));
      i = j;
    } else if (ops[i].t == 'K') {
      // a kick with no drift after it: kick-drift with a zero drift
      ERET(ens_fft(e, true));
      ERET(launch_ens_kmul(e));
      ERET(ens_fft(e, false));
      ERET(pw(0, ops[i].h, 0.0));
      ++i;
    } else {
      ++i;
    }
  }
  return LAT_OK;
}

// per-run views for the output paths
int run_ptrs(lat_ens_s* e, int run, char** f, char** c, char** p, const lat_ens_s::Cls** cl) {
  if (run < 0 || run >= (int)e->run_cls.size()) return set_error(LAT_ERR_ARG, "bad run index");
  *cl = &e->cls[e->run_cls[run]];
  const size_t off = (size_t)e->run_off[run] * e->rsz;
  *f = (char*)e->phi + off;
  *c = e->phic ? (char*)e->phic + off : nullptr;
  *p = (char*)e->pi + off;
  return LAT_OK;
}

}  // namespace

extern "C" {

int lat_ens_destroy(lat_ens_t* e) {
  if (!e) return LAT_OK;
  cudaSetDevice(e->dev);
  if (e->stream) cudaStreamSynchronize(e->stream);
  for (auto& m : e->marks)
    if (m) cudaEventDestroy(m);
  for (auto& g : e->graphs) cudaGraphExecDestroy(g.exec);
  for (auto& c : e->cls) {
    if (c.have) {
      cufftDestroy(c.r2c); cufftDestroy(c.c2r); cufftDestroy(c.r2c1); cufftDestroy(c.z2d1);
    }
    if (c.tw) cudaFree(c.tw);
    if (c.shift) cudaFree(c.shift);
    if (c.side) cudaStreamDestroy(c.side);
    if (c.done) cudaEventDestroy(c.done);
  }
  if (e->fork) cudaEventDestroy(e->fork);
  void* bufs[] = {e->phi, e->phic, e->pi, e->lap, e->Fk, e->work, e->sc, e->rb.partials, e->rb.counter,
                  e->spec_part, e->spec_out, e->spec_counter};
  for (void* b : bufs)
    if (b) cudaFree(b);
  if (e->stream) cudaStreamDestroy(e->stream);
  delete e;
  return LAT_OK;
}

int lat_ens_create(lat_ens_t** out, const lat_config* base, int32_t nruns, const int32_t* sizes) {
  if (!out || !base || !sizes || nruns < 1) return set_error(LAT_ERR_ARG, "bad ensemble arguments");
  *out = nullptr;
  if (base->laplacian != LAT_LAP_SPECTRAL || base->background != LAT_BG_MINKOWSKI || base->nfld != 1 || base->gw)
    return set_error(LAT_ERR_UNSUPPORTED, "ensembles: one field, spectral Laplacian, Minkowski background");
  if (base->precision != LAT_FP64 && base->precision != LAT_FP32_KAHAN) return set_error(LAT_ERR_ARG, "bad precision");
  lat_ens_s* e = new lat_ens_s();
  e->base = *base;
  e->prec = base->precision;
  e->rsz = e->prec == LAT_FP64 ? 8 : 4;
  e->csz = 2 * e->rsz;
  e->dev = base->device;
  EGuard g(e);
  auto bail = [&](int code) { lat_ens_destroy(e); return code; };
  std::vector<int> uniq;
  for (int r = 0; r < nruns; ++r) {
    if (sizes[r] < 4 || sizes[r] % 2) return bail(set_error(LAT_ERR_ARG, "ensemble sizes must be even and >= 4"));
    if (std::find(uniq.begin(), uniq.end(), sizes[r]) == uniq.end()) uniq.push_back(sizes[r]);
  }
  if ((int)uniq.size() > kMaxSeg) return bail(set_error(LAT_ERR_UNSUPPORTED, "at most 8 distinct sizes"));
  std::sort(uniq.begin(), uniq.end());
  const double twopi = 6.2831853071795864769252867665590;
  for (int n : uniq) {
    lat_ens_s::Cls c;
    c.n = n;
    c.dx = base->len / n;
    c.dk = twopi / base->len;
    e->cls.push_back(c);
  }
  e->run_cls.resize(nruns);
  for (int r = 0; r < nruns; ++r)
    e->run_cls[r] = (int)(std::find(uniq.begin(), uniq.end(), sizes[r]) - uniq.begin());
  // class-major layout; runs keep their order inside a class
  int64_t so = 0, fo = 0;
  e->run_off.assign(nruns, 0);
  e->run_fk.assign(nruns, 0);
  for (size_t ci = 0; ci < e->cls.size(); ++ci) {
    auto& c = e->cls[ci];
    c.site_off = so;
    c.fk_off = fo;
    const int64_t n3 = (int64_t)c.n * c.n * c.n, m = (int64_t)(c.n / 2 + 1) * c.n * c.n;
    for (int r = 0; r < nruns; ++r)
      if (e->run_cls[r] == (int)ci) {
        e->run_off[r] = so;
        e->run_fk[r] = fo;
        so += n3;
        fo += m;
        ++c.count;
      }
  }
  e->Ntot = so;
  e->Mtot = fo;
  cudaError_t er = cudaSetDevice(e->dev);
  if (er != cudaSuccess) return bail(cuda_fail(er, "cudaSetDevice"));
  int nsm = 0;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, e->dev);
  e->nsm = nsm > 0 ? nsm : 152;
  e->grid = e->nsm * 4;
  if ((er = cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking)) != cudaSuccess) return bail(cuda_fail(er, "stream"));
  auto alloc = [&](void** p, size_t bytes) -> int {
    cudaError_t ee = cudaMalloc(p, bytes);
    if (ee != cudaSuccess) return set_error(LAT_ERR_ALLOC, std::string("cudaMalloc: ") + cudaGetErrorString(ee));
    cudaMemsetAsync(*p, 0, bytes, e->stream);
    return LAT_OK;
  };
  int st;
  if ((st = alloc(&e->phi, e->Ntot * e->rsz))) return bail(st);
  if (e->prec == LAT_FP32_KAHAN && (st = alloc(&e->phic, e->Ntot * e->rsz))) return bail(st);
  if ((st = alloc(&e->pi, e->Ntot * e->rsz))) return bail(st);
  if ((st = alloc(&e->lap, e->Ntot * e->rsz))) return bail(st);
  if ((st = alloc(&e->Fk, e->Mtot * e->csz))) return bail(st);
  if ((st = alloc((void**)&e->sc, sizeof(DevScalars)))) return bail(st);
  if ((st = alloc((void**)&e->rb.partials, (size_t)8192 * 16 * sizeof(double)))) return bail(st);
  if ((st = alloc((void**)&e->rb.counter, 64))) return bail(st);
  if ((st = alloc((void**)&e->spec_part, (size_t)e->nsm * 2 * 3 * 2048 * sizeof(double)))) return bail(st);
  if ((st = alloc((void**)&e->spec_out, (size_t)3 * 2048 * sizeof(double)))) return bail(st);
  if ((st = alloc((void**)&e->spec_counter, 64))) return bail(st);
  const bool d = e->prec == LAT_FP64;
  for (auto& c : e->cls) {
    if ((st = plan(e, &c.r2c, c.n, c.count, d ? CUFFT_D2Z : CUFFT_R2C))) return bail(st);
    if ((st = plan(e, &c.c2r, c.n, c.count, d ? CUFFT_Z2D : CUFFT_C2R))) return bail(st);
    if ((st = plan(e, &c.r2c1, c.n, 1, d ? CUFFT_D2Z : CUFFT_R2C))) return bail(st);
    if ((st = plan(e, &c.z2d1, c.n, 1, CUFFT_Z2D))) return bail(st);
    c.have = true;
  }
  // the streamed separable passes: FP32, every class of a supported side with
  // an even run count, every pass in whole tiles (LAT_ENS_CUFFT=1: cuFFT)
  const char* force_fft = getenv("LAT_ENS_CUFFT");
  e->sep_ok = e->prec == LAT_FP32_KAHAN && !(force_fft && force_fft[0] == '1');
  for (auto& c : e->cls) {
    const int64_t n = c.n;
    const int lx = sep_runs_lines(c.n, 0), ly = sep_runs_lines(c.n, 1), lz = sep_runs_lines(c.n, 2);
    if (!lx || !ly || !lz || c.count % 2 || (n * n) % lx || (n * n) % ly || (n * n) % lz || n % ly || n % lz)
      e->sep_ok = false;
  }
  if (e->sep_ok) {
    if ((er = cudaEventCreateWithFlags(&e->fork, cudaEventDisableTiming)) != cudaSuccess)
      return bail(cuda_fail(er, "ensemble fork event"));
    for (auto& c : e->cls) {
      if ((er = cudaStreamCreateWithFlags(&c.side, cudaStreamNonBlocking)) != cudaSuccess ||
          (er = cudaEventCreateWithFlags(&c.done, cudaEventDisableTiming)) != cudaSuccess)
        return bail(cuda_fail(er, "ensemble class stream"));
      if ((st = alloc((void**)&c.tw, (size_t)c.n * sizeof(float2)))) return bail(st);
      if ((st = alloc((void**)&c.shift, (size_t)2 * c.count * sizeof(float)))) return bail(st);
      std::vector<float> w(2 * c.n);
      for (int j = 0; j < c.n; ++j) {
        const long double ang = -6.283185307179586476925286766559L * (long double)j / (long double)c.n;
        w[2 * j] = (float)cosl(ang);
        w[2 * j + 1] = (float)sinl(ang);
      }
      if ((er = cudaMemcpyAsync(c.tw, w.data(), w.size() * sizeof(float), cudaMemcpyHostToDevice, e->stream)) !=
          cudaSuccess)
        return bail(cuda_fail(er, "ensemble twiddles"));
      if ((er = cudaStreamSynchronize(e->stream)) != cudaSuccess) return bail(cuda_fail(er, "ensemble twiddles"));
    }
    e->sep = true;
  }
  if ((er = cudaStreamSynchronize(e->stream)) != cudaSuccess) return bail(cuda_fail(er, "ensemble create"));
  *out = e;
  return LAT_OK;
}

int lat_ens_init_vacuum(lat_ens_t* e, const uint64_t* seeds, double fld0, double dfld0, double m2eff, double amp,
                        double kcut_frac) {
  if (!e || !seeds) return set_error(LAT_ERR_ARG, "null argument");
  EGuard g(e);
  int64_t nmax = 0;
  for (auto& c : e->cls) nmax = std::max<int64_t>(nmax, (int64_t)c.n * c.n * c.n);
  double2 *Fa = nullptr, *Fb = nullptr;
  double* tmp = nullptr;
  int rc = LAT_OK;
  if (cudaMalloc(&Fa, sizeof(double2) * nmax) != cudaSuccess || cudaMalloc(&Fb, sizeof(double2) * nmax) != cudaSuccess ||
      cudaMalloc(&tmp, sizeof(double) * nmax) != cudaSuccess)
    rc = set_error(LAT_ERR_ALLOC, "ensemble vacuum scratch");
  const double twopi = 6.2831853071795864769252867665590;
  for (int r = 0; r < (int)e->run_cls.size() && rc == LAT_OK; ++r) {
    char *f, *c, *p;
    const lat_ens_s::Cls* cl;
    if ((rc = run_ptrs(e, r, &f, &c, &p, &cl))) break;
    const int n = cl->n;
    const double Nd = (double)n * n * n, V = e->base.len * e->base.len * e->base.len;
    VacArgs va{};
    va.nx = va.ny = va.nz = n;
    va.seed = seeds[r];
    va.field = 0;
    va.dkx = va.dky = va.dkz = cl->dk;
    va.sig_pref = amp * Nd * Nd / (2.0 * V);
    va.m2 = m2eff;
    va.kcut = kcut_frac * (twopi / 2.0) / cl->dx;
    va.Fphi = Fa;
    va.Fpi = Fb;
    if ((rc = launch_vacuum_modes(va, e->stream))) break;
    if (cufftExecZ2D(cl->z2d1, (cufftDoubleComplex*)Fa, tmp) != CUFFT_SUCCESS) { rc = set_error(LAT_ERR_CUDA, "z2d"); break; }
    if ((rc = launch_add_scale(tmp, (int64_t)Nd, 1.0 / Nd, fld0, e->stream))) break;
    if ((rc = launch_from_fp64(tmp, (int64_t)Nd, e->prec, f, c, e->stream))) break;
    if (cufftExecZ2D(cl->z2d1, (cufftDoubleComplex*)Fb, tmp) != CUFFT_SUCCESS) { rc = set_error(LAT_ERR_CUDA, "z2d"); break; }
    if ((rc = launch_add_scale(tmp, (int64_t)Nd, 1.0 / Nd, dfld0, e->stream))) break;
    if ((rc = launch_from_fp64(tmp, (int64_t)Nd, e->prec, p, nullptr, e->stream))) break;
  }
  cudaStreamSynchronize(e->stream);
  if (Fa) cudaFree(Fa);
  if (Fb) cudaFree(Fb);
  if (tmp) cudaFree(tmp);
  return rc;
}

namespace {
int ens_symp(lat_ens_t* e, int32_t order, double dt_over_dx, int32_t nsteps, bool run);
}

int lat_ens_symp(lat_ens_t* e, int32_t order, double dt_over_dx, int32_t nsteps) {
  if (!e) return set_error(LAT_ERR_ARG, "null handle");
  EGuard g(e);
  return ens_symp(e, order, dt_over_dx, nsteps, true);
}

int lat_ens_prepare(lat_ens_t* e, int32_t order, double dt_over_dx, int32_t nsteps) {
  if (!e) return set_error(LAT_ERR_ARG, "null handle");
  EGuard g(e);
  return ens_symp(e, order, dt_over_dx, nsteps, false);
}

int lat_ens_mark(lat_ens_t* e, int32_t slot) {
  if (!e || slot < 0 || slot >= 16) return set_error(LAT_ERR_ARG, "bad mark slot");
  EGuard g(e);
  if (!e->marks[slot]) ECK(cudaEventCreate(&e->marks[slot]));
  ECK(cudaEventRecord(e->marks[slot], e->stream));
  return LAT_OK;
}

int lat_ens_mark_elapsed(lat_ens_t* e, int32_t a, int32_t b, double* ms) {
  if (!e || !ms || a < 0 || b < 0 || a >= 16 || b >= 16 || !e->marks[a] || !e->marks[b])
    return set_error(LAT_ERR_ARG, "bad mark slots");
  EGuard g(e);
  ECK(cudaEventSynchronize(e->marks[b]));
  float t = 0;
  ECK(cudaEventElapsedTime(&t, e->marks[a], e->marks[b]));
  *ms = t;
  return LAT_OK;
}

int lat_ens_launch_count(const lat_ens_t* e, int64_t* count) {
  if (!e || !count) return set_error(LAT_ERR_ARG, "null argument");
  *count = e->launches;
  return LAT_OK;
}

int lat_ens_sep_streamed(const lat_ens_t* e, int32_t* on) {
  if (!e || !on) return set_error(LAT_ERR_ARG, "null argument");
  *on = e->sep ? 1 : 0;
  return LAT_OK;
}

int lat_ens_tuning_get(const lat_ens_t* e, int32_t out[2]) {
  if (!e || !out) return set_error(LAT_ERR_ARG, "null argument");
  out[0] = e->block;
  out[1] = e->grid / e->nsm;
  return LAT_OK;
}

int lat_ens_autotune(lat_ens_t* e, const char* cache_path) {
  if (!e) return set_error(LAT_ERR_ARG, "null handle");
  EGuard g(e);
  std::string key = std::string("ens:") + (e->prec == LAT_FP64 ? "fp64" : "fp32k") + ":" + std::to_string(e->nsm);
  for (size_t r = 0; r < e->run_cls.size(); ++r) key += ":" + std::to_string(e->cls[e->run_cls[r]].n);
  if (cache_path) {  // a cached choice for this exact ensemble
    FILE* fp = fopen(cache_path, "r");
    if (fp) {
      char line[4096];
      const std::string pat = "\"key\": \"" + key + "\"";
      int blk = 0, bps = 0, sep = 0;
      bool found = false;
      while (fgets(line, sizeof(line), fp)) {
        if (!strstr(line, pat.c_str())) continue;
        const char* q = strstr(line, "\"block\":");
        if (q && sscanf(q, "\"block\": %d, \"bps\": %d, \"sep\": %d", &blk, &bps, &sep) == 3) found = true;
      }
      fclose(fp);
      if (found && blk > 0 && bps > 0) {
        e->block = blk;
        e->grid = e->nsm * bps;
        e->sep = e->sep_ok && sep != 0;
        for (auto& ge : e->graphs) cudaGraphExecDestroy(ge.exec);
        e->graphs.clear();
        return LAT_OK;
      }
    }
  }
  // candidates run real passes: save and restore the state
  const size_t fb = (size_t)e->Ntot * e->rsz;
  void* saved[3] = {nullptr, nullptr, nullptr};
  void* live[3] = {e->phi, e->phic, e->pi};
  for (int i = 0; i < 3; ++i)
    if (live[i]) {
      ECK(cudaMalloc(&saved[i], fb));
      ECK(cudaMemcpyAsync(saved[i], live[i], fb, cudaMemcpyDeviceToDevice, e->stream));
    }
  std::vector<Op> ops;
  double tg[3] = {0, 0, 0};
  Emitter em{2, false, false, &ops, tg};
  int st = em.symp(2, 1.0, 2);
  cudaEvent_t a = nullptr, b = nullptr;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  float best = 1e30f, tsep = 1e30f;
  int bblk = e->block, bgrid = e->grid;
  if (e->sep_ok && st == LAT_OK) {  // the streamed separable passes
    e->sep = true;
    st = ens_exec(e, ops, 1e-4);  // warm-up
    cudaEventRecord(a, e->stream);
    for (int r = 0; r < 3 && st == LAT_OK; ++r) st = ens_exec(e, ops, 1e-4);
    cudaEventRecord(b, e->stream);
    cudaEventSynchronize(b);
    cudaEventElapsedTime(&tsep, a, b);
  }
  e->sep = false;  // the cuFFT path with its pointwise shapes
  for (int blk : {128, 256})  // the persistent passes are built for at most 256 threads
    for (int bps : {1, 2, 4, 8}) {
      if (st != LAT_OK) break;
      e->block = blk;
      e->grid = e->nsm * bps;
      st = ens_exec(e, ops, 1e-4);  // warm-up
      cudaEventRecord(a, e->stream);
      for (int r = 0; r < 3 && st == LAT_OK; ++r) st = ens_exec(e, ops, 1e-4);
      cudaEventRecord(b, e->stream);
      cudaEventSynchronize(b);
      float ms = 0;
      cudaEventElapsedTime(&ms, a, b);
      if (st == LAT_OK && ms < best) { best = ms; bblk = blk; bgrid = e->grid; }
    }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  e->block = bblk;
  e->grid = bgrid;
  e->sep = e->sep_ok && tsep < best;
  for (int i = 0; i < 3; ++i)
    if (saved[i]) cudaMemcpyAsync(live[i], saved[i], fb, cudaMemcpyDeviceToDevice, e->stream);
  cudaStreamSynchronize(e->stream);
  for (void* p : saved)
    if (p) cudaFree(p);
  for (auto& ge : e->graphs) cudaGraphExecDestroy(ge.exec);
  e->graphs.clear();
  if (st != LAT_OK) return st;
  if (cache_path) {
    FILE* fp = fopen(cache_path, "a");
    if (fp) {
      fprintf(fp, "{\"key\": \"%s\", \"block\": %d, \"bps\": %d, \"sep\": %d}\n", key.c_str(), e->block,
              e->grid / e->nsm, e->sep ? 1 : 0);
      fclose(fp);
    }
  }
  return LAT_OK;
}

}  // extern "C"

namespace {
int ens_symp(lat_ens_t* e, int32_t order, double dt_over_dx, int32_t nsteps, bool run) {
  std::vector<Op> ops;
  double tg[3] = {0, 0, 0};
  Emitter em{2, false, false, &ops, tg};
  ERET(em.symp(order, 1.0, nsteps));  // unit step: every h scales with each class's dt
  for (auto& ge : e->graphs)
    if (ge.order == order && ge.dto == dt_over_dx && ge.nsteps == nsteps) {
      if (!run) return LAT_OK;
      ECK(cudaGraphLaunch(ge.exec, e->stream));
      e->launches += ge.kernels;
      return LAT_OK;
    }
  EnsGraph ge{order, dt_over_dx, nsteps, 0, nullptr};
  const int64_t before = e->launches;
  ECK(cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeRelaxed));
  int st = ens_exec(e, ops, dt_over_dx);
  cudaGraph_t graph = nullptr;
  cudaError_t er = cudaStreamEndCapture(e->stream, &graph);
  if (st != LAT_OK) {
    if (graph) cudaGraphDestroy(graph);
    return st;
  }
  if (er != cudaSuccess) return cuda_fail(er, "ensemble graph capture");
  ge.kernels = e->launches - before;
  er = cudaGraphInstantiate(&ge.exec, graph, 0);
  cudaGraphDestroy(graph);
  if (er != cudaSuccess) return cuda_fail(er, "ensemble graph instantiate");
  if (e->graphs.size() >= 8) {
    cudaGraphExecDestroy(e->graphs.front().exec);
    e->graphs.erase(e->graphs.begin());
  }
  e->graphs.push_back(ge);
  if (!run) {
    e->launches = before;
    return LAT_OK;
  }
  ECK(cudaGraphLaunch(ge.exec, e->stream));
  return LAT_OK;
}
}  // namespace

extern "C" {

int lat_ens_sync(lat_ens_t* e) {
  if (!e) return set_error(LAT_ERR_ARG, "null handle");
  EGuard g(e);
  ECK(cudaStreamSynchronize(e->stream));
  return LAT_OK;
}

int lat_ens_energies(lat_ens_t* e, double* out) {
  if (!e || !out) return set_error(LAT_ERR_ARG, "null argument");
  EGuard g(e);
  for (int r = 0; r < (int)e->run_cls.size(); ++r) {
    char *f, *c, *p;
    const lat_ens_s::Cls* cl;
    ERET(run_ptrs(e, r, &f, &c, &p, &cl));
    const int n = cl->n;
    EnergyArgs ea{};
    ea.nx = ea.ny = ea.nz = n;
    ea.nf = 1;
    ea.phi = f; ea.phic = c; ea.pi = p;
    ea.fd = 0;
    ea.model.model = e->base.model;
    for (int i = 0; i < 4; ++i) ea.model.p[i] = e->base.model_params[i];
    ea.sc = e->sc;
    ea.rb = e->rb;
    ea.grid = e->nsm * 4;
    ea.block = 256;
    ERET(launch_energy(ea, e->prec, e->stream));
    cufftResult fr = e->prec == LAT_FP64
                         ? cufftExecD2Z(cl->r2c1, (cufftDoubleReal*)f, (cufftDoubleComplex*)e->Fk)
                         : cufftExecR2C(cl->r2c1, (cufftReal*)f, (cufftComplex*)e->Fk);
    if (fr != CUFFT_SUCCESS) return set_error(LAT_ERR_CUDA, "ensemble energy FFT");
    ERET(launch_parseval(e->Fk, n, n, n, 1, cl->dk * cl->dk, cl->dk * cl->dk, cl->dk * cl->dk, e->sc, 8, e->rb,
                         e->nsm * 4, e->prec, e->stream));
    DevScalars s;
    ECK(cudaMemcpyAsync(&s, e->sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, e->stream));
    ECK(cudaStreamSynchronize(e->stream));
    const double Nd = (double)n * n * n;
    double* o = out + (size_t)r * LAT_NENERGY;
    o[LAT_E_KE] = 0.5 * s.red[0] / Nd;
    o[LAT_E_GE_LAP] = 0.5 * (s.red[8] / Nd) / Nd;
    o[LAT_E_GE_GRAD] = o[LAT_E_GE_LAP];
    o[LAT_E_PE] = s.red[1] / Nd;
    o[LAT_E_RHO] = o[LAT_E_KE] + o[LAT_E_GE_LAP] + o[LAT_E_PE];
    o[LAT_E_GRAV] = 0.0;
    o[LAT_E_RESIDUAL] = 1.0;
    o[LAT_E_A] = 1.0;
    o[LAT_E_AP] = 0.0;
    o[LAT_E_MEAN0] = s.red[2] / Nd;
    o[LAT_E_MEAN1] = 0.0;
    o[LAT_E_GW] = 0.0;
  }
  return LAT_OK;
}

int lat_ens_spectrum(lat_ens_t* e, int32_t run, int32_t nbins, double* S, double* W) {
  if (!e || !S || !W || nbins < 1 || nbins > 2048) return set_error(LAT_ERR_ARG, "bad spectrum arguments");
  EGuard g(e);
  char *f, *c, *p;
  const lat_ens_s::Cls* cl;
  ERET(run_ptrs(e, run, &f, &c, &p, &cl));
  cufftResult fr = e->prec == LAT_FP64 ? cufftExecD2Z(cl->r2c1, (cufftDoubleReal*)f, (cufftDoubleComplex*)e->Fk)
                                       : cufftExecR2C(cl->r2c1, (cufftReal*)f, (cufftComplex*)e->Fk);
  if (fr != CUFFT_SUCCESS) return set_error(LAT_ERR_CUDA, "ensemble spectrum FFT");
  SpecArgs sa{};
  sa.nx = sa.ny = sa.nz = cl->n;
  sa.F1 = e->Fk;
  sa.mode = LAT_SPEC_WEIGHTED;
  sa.nbins = nbins;
  sa.partials = e->spec_part;
  sa.out = e->spec_out;
  sa.counter = e->spec_counter;
  sa.grid = e->nsm * 2;
  sa.block = 256;
  ERET(launch_spectrum(sa, e->prec, e->stream));
  std::vector<double> o(3 * nbins);
  ECK(cudaMemcpyAsync(o.data(), e->spec_out, sizeof(double) * 3 * nbins, cudaMemcpyDeviceToHost, e->stream));
  ECK(cudaStreamSynchronize(e->stream));
  for (int l = 0; l < nbins; ++l) {
    W[l] = o[nbins + l];
    S[l] = W[l] != 0.0 ? o[l] / W[l] : o[l];
  }
  return LAT_OK;
}

int lat_ens_download(lat_ens_t* e, int32_t run, double* fld, double* fldp) {
  if (!e) return set_error(LAT_ERR_ARG, "null handle");
  EGuard g(e);
  char *f, *c, *p;
  const lat_ens_s::Cls* cl;
  ERET(run_ptrs(e, run, &f, &c, &p, &cl));
  const int64_t n3 = (int64_t)cl->n * cl->n * cl->n;
  double* tmp = nullptr;
  ECK(cudaMalloc(&tmp, sizeof(double) * n3));
  int rc = LAT_OK;
  if (fld) {
    rc = launch_to_fp64(f, c, n3, e->prec, tmp, e->stream);
    if (rc == LAT_OK && cudaMemcpyAsync(fld, tmp, sizeof(double) * n3, cudaMemcpyDeviceToHost, e->stream) != cudaSuccess)
      rc = set_error(LAT_ERR_CUDA, "download");
    cudaStreamSynchronize(e->stream);
  }
  if (fldp && rc == LAT_OK) {
    rc = launch_to_fp64(p, nullptr, n3, e->prec, tmp, e->stream);
    if (rc == LAT_OK && cudaMemcpyAsync(fldp, tmp, sizeof(double) * n3, cudaMemcpyDeviceToHost, e->stream) != cudaSuccess)
      rc = set_error(LAT_ERR_CUDA, "download");
    cudaStreamSynchronize(e->stream);
  }
  cudaFree(tmp);
  return rc;
}

}  // extern "C"
