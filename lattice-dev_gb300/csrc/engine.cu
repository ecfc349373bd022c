// engine.cu -- host side of the GB300 lattice engine and its C ABI.
//
// The reference keeps the lattice in Fortran module globals and advances it
// with symp{2,4,6,8} -> symp_o2step -> Hamiltonian_Split
// (Pseudospec/openmp_dev/evolve_spectral.f90:129-227,
//  hamiltonian_conformal.f90:50-81).  Here a handle owns the lattice in HBM.
// An integrator call is first expanded into the reference's exact sequence
// of Hamiltonian pieces (an op list: D = fields kinetic, K = gradient +
// potential, G = gravity/metric kinetic), then executed with fusion:
//   PSEUDOSPEC conformal, spectral:  G K G D      -> one k-space pass + one sweep
//   Minkowski (both split orders):   K D [D ...]  -> one sweep (drifts merged)
// and every remaining op as its own kernel (FD conformal, DEFROST conformal,
// lat_split, lat_o2step), so the fused path and the plain path can be
// checked against each other and against the CPU oracle.
#include <cufft.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "engine.hpp"
#include "integrator.hpp"
#include "net.hpp"

namespace lat {

thread_local int64_t* g_launch_counter = nullptr;
static thread_local std::string t_err;

int set_error(int code, const std::string& msg) {
  t_err = msg;
  return code;
}
int cuda_fail(cudaError_t e, const char* where) {
  return set_error(LAT_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}
static int cufft_fail(cufftResult r, const char* where) {
  return set_error(LAT_ERR_CUDA, std::string(where) + ": cuFFT error " + std::to_string((int)r));
}

}  // namespace lat

using namespace lat;

#define CK(x)                                             \
  do {                                                    \
    cudaError_t e_ = (x);                                 \
    if (e_ != cudaSuccess) return cuda_fail(e_, #x);      \
  } while (0)
#define CF(x)                                             \
  do {                                                    \
    cufftResult r_ = (x);                                 \
    if (r_ != CUFFT_SUCCESS) return cufft_fail(r_, #x);   \
  } while (0)
#define RET(x)                                            \
  do {                                                    \
    int s_ = (x);                                         \
    if (s_ != LAT_OK) return s_;                          \
  } while (0)

namespace {

struct GraphEntry {
  int order;
  double dt;
  int nsteps;
  int cur, ucur;
  int cur_after, ucur_after;
  void *fldc, *fldp;              // current compensation / momentum buffers at capture
  void *fldc_after, *fldp_after;  // and after the captured call
  uint64_t cl_key;                 // attached closure network (0: none), its cadence and units
  int cl_every, cl_units;
  int64_t kernels;
  cudaGraphExec_t exec;
};

}  // namespace

struct lat_s {
  lat_config cfg{};
  int nx = 0, ny = 0, nz = 0, nf = 0;
  int64_t N = 0, M = 0;
  double dx = 0, dkx = 0, dky = 0, dkz = 0;
  double c[5] = {0, 0, 0, 0, 0};
  int prec = LAT_FP64;
  size_t rsz = 8, csz = 16;
  int dev = 0, nsm = 152;
  cudaStream_t stream = nullptr;

  void* fld[2] = {nullptr, nullptr};
  int cur = 0;
  void* fldc = nullptr;      // current Kahan compensation buffer
  void* fldp = nullptr;      // current momentum buffer
  void* lap = nullptr;
  void* fldc_alt = nullptr;  // second buffers the separable passes write to
  void* fldp_alt = nullptr;
  void* lap_alt = nullptr;
  void* Fk = nullptr;  // max(nf,2) * M complex
  void* u[2] = {nullptr, nullptr};
  int ucur = 0;
  void* pu = nullptr;
  void* Fk6 = nullptr;

  DevScalars* sc = nullptr;
  RedBuf rb{};
  int64_t red_cap = 0;  // blocks the partial buffer holds
  double* spec_part = nullptr;
  double* spec_out = nullptr;
  unsigned int* spec_counter = nullptr;
  int spec_grid = 0;
  double* stage = nullptr;  // nf*N doubles
  size_t stage_elems = 0;

  cufftHandle p_r2c = 0, p_c2r = 0, p_r2c1 = 0, p_c2r1 = 0, p_r2c6 = 0;
  bool have_r2c = false, have_c2r = false, have_r2c1 = false, have_c2r1 = false, have_r2c6 = false;
  void* fft_work = nullptr;
  size_t fft_work_size = 0;

  double tglobal[3] = {0, 0, 0};

  cufftHandle p_d2z1 = 0;          // FP64 transform for spectra of FP32 fields
  bool have_d2z1 = false;
  void* Fk64 = nullptr;            // 2 * M double2

  bool sep_ok = false;            // separable spectral passes available for these sizes
  bool sep = false;               // and in use
  bool sep_stream = true;         // streamed passes where available (LAT_SEP_CLASSIC=1: off)
  void* tw[3] = {nullptr, nullptr, nullptr};  // W_N^j per axis, field precision

  int fd_ty = 8, fd_zc = 32;
  int pw_grid = 0, pw_block = 256;

  bool timing = false;
  struct Ev { cudaEvent_t a, b; int cls; };
  std::vector<Ev> ev_pool;
  size_t ev_used = 0;
  double t_ms[LAT_NKCLASS] = {0};
  int64_t t_n[LAT_NKCLASS] = {0};
  int64_t launches = 0;

  cudaEvent_t marks[16] = {};
  bool use_graphs = true;
  std::vector<GraphEntry> graphs;

  // learned closure (lat_closure_attach)
  lat_net_s* cl_net = nullptr;
  int cl_every = 1;
  int cl_units = 0;  // 1: the network sees (a phi, pi / a) and predicts a^3 Delta
  double cl_tscale[2] = {1, 1};
  net::InferBufs cl_b{};
  // the network runs on a side stream beside the kick's transforms (it reads
  // the same fields, writes only cl_b), joined before the fused kick+drift
  cudaStream_t cl_stream = nullptr;
  cudaEvent_t cl_fork = nullptr, cl_join = nullptr;

  // z-slab of a global lattice (lat_slab_create): storage plane 0 is the
  // ghost of global plane z0-1, planes 1..nz_loc hold global planes
  // z0..z1-1, plane nz_loc+1 is the ghost of z1.  Kicks and reductions
  // cover the interior; the ghost planes are filled through the halo hook
  // before every kick, and the lattice sums go through the sum hook.
  bool slab = false;
  int slab_z0 = 0, slab_nzg = 0, nz_loc = 0;
  double slab_nd = 0;  // sites of the global lattice
  lat_halo_fn slab_halo = nullptr;
  lat_sum_fn slab_sum = nullptr;
  void* slab_user = nullptr;

  // tensor maps of the streamed passes Y and Z, encoded for the zs and
  // momentum buffers they were made with
  CUtensorMap sep_tm_zs[2] = {}, sep_tm_pi[2] = {};
  const void* sep_tm_for[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
};

namespace {

struct ApiGuard {
  int64_t* prev;
  explicit ApiGuard(lat_s* h) : prev(g_launch_counter) {
    if (h) {
      g_launch_counter = &h->launches;
      cudaSetDevice(h->dev);
    }
  }
  ~ApiGuard() { g_launch_counter = prev; }  // a hook may call back into the library
};

// The site count of the lattice sums: the global lattice for a z-slab.
double nd_of(const lat_s* h) { return h->slab ? h->slab_nd : (double)h->N; }

// ---------------------------------------------------------------- timing
int harvest(lat_s* h) {
  if (h->ev_used == 0) return LAT_OK;
  CK(cudaStreamSynchronize(h->stream));
  for (size_t i = 0; i < h->ev_used; ++i) {
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, h->ev_pool[i].a, h->ev_pool[i].b));
    h->t_ms[h->ev_pool[i].cls] += ms;
    h->t_n[h->ev_pool[i].cls] += 1;
  }
  h->ev_used = 0;
  return LAT_OK;
}

struct Timed {
  lat_s* h;
  size_t idx = (size_t)-1;
  Timed(lat_s* hh, int cls) : h(hh) {
    if (!h->timing) return;
    if (h->ev_used == h->ev_pool.size()) {
      if (harvest(h) != LAT_OK) return;
    }
    idx = h->ev_used++;
    h->ev_pool[idx].cls = cls;
    cudaEventRecord(h->ev_pool[idx].a, h->stream);
  }
  ~Timed() {
    if (idx != (size_t)-1) cudaEventRecord(h->ev_pool[idx].b, h->stream);
  }
};

// ------------------------------------------------------------- helpers
bool getenv_flag(const char* name) {
  const char* v = getenv(name);
  return v && v[0] == '1';
}
bool conformal(const lat_s* h) { return h->cfg.background == LAT_BG_CONFORMAL; }
bool spectral(const lat_s* h) { return h->cfg.laplacian == LAT_LAP_SPECTRAL; }
int n_terms(const lat_s* h) {
  if (h->cfg.split_order == LAT_SPLIT_DEFROST) return 3;
  return conformal(h) ? 3 : 2;
}

ModelP model_of(const lat_s* h) {
  ModelP m;
  m.model = h->cfg.model;
  for (int i = 0; i < 4; ++i) m.p[i] = h->cfg.model_params[i];
  return m;
}

int fft_exec_r2c(lat_s* h, cufftHandle p, const void* in, void* out) {
  Timed t(h, LAT_K_FFT_R2C);  // a library launch: not counted among the engine's kernels
  if (h->prec == LAT_FP64) CF(cufftExecD2Z(p, (cufftDoubleReal*)in, (cufftDoubleComplex*)out));
  else CF(cufftExecR2C(p, (cufftReal*)in, (cufftComplex*)out));
  return LAT_OK;
}
int fft_exec_c2r(lat_s* h, cufftHandle p, void* in, void* out) {
  Timed t(h, LAT_K_FFT_C2R);
  if (h->prec == LAT_FP64) CF(cufftExecZ2D(p, (cufftDoubleComplex*)in, (cufftDoubleReal*)out));
  else CF(cufftExecC2R(p, (cufftComplex*)in, (cufftReal*)out));
  return LAT_OK;
}

int make_plan(lat_s* h, cufftHandle* p, bool* have, bool r2c, int batch) {
  if (*have) return LAT_OK;
  CF(cufftCreate(p));
  CF(cufftSetAutoAllocation(*p, 0));
  int n[3] = {h->nz, h->ny, h->nx};
  size_t ws = 0;
  cufftType t;
  if (h->prec == LAT_FP64) t = r2c ? CUFFT_D2Z : CUFFT_Z2D;
  else t = r2c ? CUFFT_R2C : CUFFT_C2R;
  long long idist = r2c ? h->N : h->M, odist = r2c ? h->M : h->N;
  CF(cufftMakePlanMany(*p, 3, n, nullptr, 1, (int)idist, nullptr, 1, (int)odist, t, batch, &ws));
  (void)idist; (void)odist;
  if (ws > h->fft_work_size) {
    if (h->fft_work) cudaFree(h->fft_work);
    h->fft_work = nullptr;
    CK(cudaMalloc(&h->fft_work, ws));
    h->fft_work_size = ws;
    // re-point every existing plan at the new work area
    if (h->have_r2c) CF(cufftSetWorkArea(h->p_r2c, h->fft_work));
    if (h->have_c2r) CF(cufftSetWorkArea(h->p_c2r, h->fft_work));
    if (h->have_r2c1) CF(cufftSetWorkArea(h->p_r2c1, h->fft_work));
    if (h->have_c2r1) CF(cufftSetWorkArea(h->p_c2r1, h->fft_work));
    if (h->have_r2c6) CF(cufftSetWorkArea(h->p_r2c6, h->fft_work));
  }
  CF(cufftSetWorkArea(*p, h->fft_work));
  CF(cufftSetStream(*p, h->stream));
  *have = true;
  return LAT_OK;
}

RedBuf red(lat_s* h) { return h->rb; }

PwArgs pw_base(lat_s* h) {
  PwArgs a{};
  a.N = h->N;
  a.nf = h->nf;
  a.phi = h->fld[h->cur];
  a.phic = h->fldc;
  a.pi = h->fldp;
  a.lap = h->lap;
  a.u = nullptr;
  a.pu = nullptr;
  a.model = model_of(h);
  a.Nd = nd_of(h);
  a.conf = conformal(h) ? 1 : 0;
  a.sc = h->sc;
  a.rb = red(h);
  a.grid = h->pw_grid;
  a.block = h->pw_block;
  return a;
}

FdArgs fd_base(lat_s* h) {
  FdArgs a{};
  a.nx = h->nx; a.ny = h->ny; a.nz = h->nz; a.nf = h->nf;
  a.phi_in = h->fld[h->cur];
  a.phi_out = nullptr;
  a.phic = h->fldc;
  a.pi = h->fldp;
  a.u_in = h->cfg.gw ? h->u[h->ucur] : nullptr;
  a.u_out = nullptr;
  a.pu = h->pu;
  const double e = 1.0 / (h->dx * h->dx) / h->c[4];
  for (int i = 0; i < 4; ++i) a.lc[i] = h->c[i] * e;
  a.seven = (h->c[2] == 0.0 && h->c[3] == 0.0) ? 1 : 0;
  a.model = model_of(h);
  a.kappa = h->cfg.gw_coupling;
  a.inv2dx = 1.0 / (2.0 * h->dx);
  a.conf = 0;
  a.Nd = nd_of(h);
  a.sc = h->sc;
  a.rb = red(h);
  a.ty = h->fd_ty;
  a.zc = h->fd_zc;
  if (h->slab) {  // the interior planes; the ghosts are the neighbours' boundary planes
    a.zlo = 1;
    a.zhi = 1 + h->nz_loc;
  }
  return a;
}

// spectral Laplacian of all fields into h->lap (kmul optionally stores ge2)
int spectral_lap(lat_s* h, bool store_ge2) {
  RET(fft_exec_r2c(h, h->p_r2c, h->fld[h->cur], h->Fk));
  {
    Timed t(h, LAT_K_KMUL);
    KmulArgs k{};
    k.nx = h->nx; k.ny = h->ny; k.nz = h->nz; k.nf = h->nf;
    k.Fk = h->Fk;
    k.dkx2 = h->dkx * h->dkx; k.dky2 = h->dky * h->dky; k.dkz2 = h->dkz * h->dkz;
    k.invN = 1.0 / (double)h->N;
    k.store_ge2 = store_ge2 ? 1 : 0;
    k.sc = h->sc;
    k.rb = red(h);
    k.grid = h->pw_grid;
    k.block = 256;
    RET(launch_kmul(k, h->prec, h->stream));
  }
  return fft_exec_c2r(h, h->p_c2r, h->Fk, h->lap);
}

// ------------------------------------------------------------ op lists
Emitter emitter(lat_s* h, std::vector<Op>* ops, double* tg) {
  return Emitter{n_terms(h), h->cfg.split_order == LAT_SPLIT_DEFROST, conformal(h), ops, tg};
}

// ----------------------------------------------------------- execution
int exec_drift(lat_s* h, double hd) {
  Timed t(h, LAT_K_DRIFT);
  PwArgs a = pw_base(h);
  a.mode = PW_DRIFT;
  a.hd = hd;
  if (h->cfg.gw) { a.u = h->u[h->ucur]; a.pu = h->pu; }
  return launch_pointwise(a, h->prec, h->stream);
}

int exec_kick(lat_s* h, double hk) {
  if (spectral(h)) {
    RET(spectral_lap(h, false));
    Timed t(h, LAT_K_KICK);
    PwArgs a = pw_base(h);
    a.mode = PW_KICK;
    a.hk = hk;
    return launch_pointwise(a, h->prec, h->stream);
  }
  Timed t(h, LAT_K_KICK);
  FdArgs a = fd_base(h);
  a.hk = hk;
  a.hd = 0;
  a.conf = conformal(h) ? 1 : 0;
  return launch_fd(a, h->prec, h->stream, nullptr);
}

int exec_grav(lat_s* h, double hg) {
  Timed t(h, LAT_K_OTHER);
  return launch_grav(h->sc, hg, h->stream);
}

// corr: the attached closure's force enters the kick (spectral lattices);
// join: an event of work on another stream the kick+drift waits for (after
// the transforms of the Laplacian)
int exec_kd(lat_s* h, double hk, double hg, double hd, bool corr = false, cudaEvent_t join = nullptr) {
  if (spectral(h)) {
    RET(spectral_lap(h, conformal(h)));
    if (join) CK(cudaStreamWaitEvent(h->stream, join, 0));
    Timed t(h, LAT_K_KICKDRIFT);
    PwArgs a = pw_base(h);
    a.mode = PW_KD;
    a.hk = hk; a.hg = hg; a.hd = hd;
    if (corr) {
      a.corr = h->cl_b.out;
      a.corr_ts[0] = h->cl_tscale[0];
      a.corr_ts[1] = h->cl_tscale[1];
      a.corr_units = h->cl_units;
    }
    return launch_pointwise(a, h->prec, h->stream);
  }
  if (corr) return set_error(LAT_ERR_STATE, "fused closure kick on a finite-difference lattice");
  // FD Minkowski: stencil kick + drift into the other buffer
  Timed t(h, LAT_K_KICKDRIFT);
  FdArgs a = fd_base(h);
  a.phi_out = h->fld[1 - h->cur];
  if (h->cfg.gw) a.u_out = h->u[1 - h->ucur];
  a.hk = hk;
  a.hd = hd;
  RET(launch_fd(a, h->prec, h->stream, nullptr));
  h->cur = 1 - h->cur;
  if (h->cfg.gw) h->ucur = 1 - h->ucur;
  return LAT_OK;
}

// ------------------------------------------------------------- z-slabs
int read_scalars(lat_s* h, DevScalars* out);

// Fill the ghost planes through the caller's hook; the stream's work so far
// has completed when the hook packs the boundary planes.
int slab_exchange(lat_s* h) {
  if (!h->slab_halo) return set_error(LAT_ERR_STATE, "z-slab handle without a halo hook (lat_slab_set_hooks)");
  CK(cudaStreamSynchronize(h->stream));
  if (h->slab_halo(h->slab_user, h) != 0) return set_error(LAT_ERR_STATE, "z-slab halo hook failed");
  return LAT_OK;
}

// Replace v[0..n) by its sum over all slabs through the caller's hook.
int slab_allreduce(lat_s* h, double* v, int n) {
  if (!h->slab_sum) return set_error(LAT_ERR_STATE, "z-slab handle without a sum hook (lat_slab_set_hooks)");
  if (h->slab_sum(h->slab_user, v, n) != 0) return set_error(LAT_ERR_STATE, "z-slab sum hook failed");
  return LAT_OK;
}

// Conformal z-slab: complete the ysclp update of a drift or of a kick from
// the slab's lattice sums (left in sc->red[13..14] by the deferred kernel)
// summed over all slabs, with the kernels' own arithmetic:
// Hamiltonian_fields_kin, ysclp += dt (KE2/N)/a^3, and
// Hamiltonian_fields_grad_pot (FD), ysclp -= a^3 (GE2/a^2/N + 4 PE/N) dt
// (Pseudospec/openmp_dev/hamiltonian_conformal.f90:92-118,176-205).
int slab_friedmann(lat_s* h, bool kick, double step) {
  DevScalars s;
  RET(read_scalars(h, &s));
  if (s.err & 1u) return set_error(LAT_ERR_NAN, "NaN/Inf in a lattice reduction");
  double v[2] = {s.red[13], s.red[14]};
  RET(slab_allreduce(h, v, 2));
  const double Nd = h->slab_nd;
  double ap, pe = 0;
  if (!kick) {
    ap = s.ap + step * (v[0] / Nd) / (s.a * s.a * s.a);
  } else {
    const double GE2 = v[0] / (s.a * s.a) / Nd;
    pe = v[1] / Nd;
    ap = s.ap - s.a * s.a * s.a * (GE2 + 4.0 * pe) * step;
    CK(cudaMemcpyAsync(&h->sc->pe, &pe, sizeof(double), cudaMemcpyHostToDevice, h->stream));
  }
  CK(cudaMemcpyAsync(&h->sc->ap, &ap, sizeof(double), cudaMemcpyHostToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));  // the host values above are copied before they go out of scope
  return LAT_OK;
}

// The op list of a z-slab, eagerly: every kick after a halo exchange,
// stencil kicks on the interior planes, drifts over the whole storage (the
// ghosts' momenta stay zero, so their drift changes nothing), the Friedmann
// updates of a conformal background from the sums of all slabs.
int exec_slab(lat_s* h, const std::vector<Op>& ops) {
  const bool conf = conformal(h);
  for (const Op& o : ops) {
    switch (o.t) {
      case 'D': {
        PwArgs a = pw_base(h);
        a.mode = PW_DRIFT;
        a.hd = o.h;
        a.defer = conf ? 1 : 0;
        if (h->cfg.gw) { a.u = h->u[h->ucur]; a.pu = h->pu; }
        RET(launch_pointwise(a, h->prec, h->stream));
        if (conf) RET(slab_friedmann(h, false, o.h));
        break;
      }
      case 'K': {
        RET(slab_exchange(h));
        FdArgs a = fd_base(h);
        a.hk = o.h;
        a.hd = 0;
        a.conf = conf ? 1 : 0;
        a.defer = conf ? 1 : 0;
        RET(launch_fd(a, h->prec, h->stream, nullptr));
        if (conf) RET(slab_friedmann(h, true, o.h));
        break;
      }
      case 'G': RET(exec_grav(h, o.h)); break;
      default: break;  // 'M' in Minkowski: clock only
    }
  }
  return LAT_OK;
}

int exec_plain(lat_s* h, const std::vector<Op>& ops) {
  if (h->slab) return exec_slab(h, ops);
  for (const Op& o : ops) {
    switch (o.t) {
      case 'D': RET(exec_drift(h, o.h)); break;
      case 'K': RET(exec_kick(h, o.h)); break;
      case 'G': RET(exec_grav(h, o.h)); break;
      default: break;  // 'M' in Minkowski: clock only
    }
  }
  return LAT_OK;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the driver library).
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn encode_tiled_fn() {
  static EncodeTiledFn fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<EncodeTiledFn>(p);
  }();
  return fn;
}

}  // namespace

int lat::encode_stream_tmaps(SepArgs& a, int axis, int lines, int n) {
  EncodeTiledFn enc = encode_tiled_fn();
  if (!enc) return set_error(LAT_ERR_CUDA, "cuTensorMapEncodeTiled entry point unavailable");
  const cuuint64_t nx = (cuuint64_t)a.nx, ny = (cuuint64_t)a.ny, nz = (cuuint64_t)a.nz, Ns = nx * ny * nz;
  const cuuint64_t pairs = a.runs ? (cuuint64_t)(a.nlines / a.pair_lines) : 1;
  const cuuint32_t L = (cuuint32_t)lines, N = (cuuint32_t)n;
  const cuuint32_t one[5] = {1, 1, 1, 1, 1};
  // zs: lines A and B interleaved, float2 per site, addressed as floats; a
  // pair's array follows the previous pair's
  const cuuint64_t zdim[4] = {2 * nx, ny, nz, pairs};
  const cuuint64_t zstr[3] = {2 * nx * 4, 2 * nx * ny * 4, 2 * Ns * 4};
  const cuuint32_t zbox[4] = {2 * L, axis == 1 ? N : 1u, axis == 2 ? N : 1u, 1};
  CUresult r = enc(&a.tm_zs, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, const_cast<void*>(a.lap), zdim, zstr, zbox, one,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return set_error(LAT_ERR_CUDA, "tensor map of zs: error " + std::to_string((int)r));
  // momenta of lines A and B (the two fields, or the two runs of a pair), Ns sites apart
  const cuuint64_t pdim[5] = {nx, ny, nz, 2, pairs};
  const cuuint64_t pstr[4] = {nx * 4, nx * ny * 4, Ns * 4, 2 * Ns * 4};
  const cuuint32_t pbox[5] = {L, axis == 1 ? N : 1u, axis == 2 ? N : 1u, 2, 1};
  r = enc(&a.tm_pi, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 5, a.pi_out, pdim, pstr, pbox, one,
          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return set_error(LAT_ERR_CUDA, "tensor map of the momenta: error " + std::to_string((int)r));
  return LAT_OK;
}

namespace {

// One separable spectral pass (k_sep.cuh) along `axis`.
int sep_pass(lat_s* h, int axis, double hk, double hg, double hd, int* grid_out = nullptr) {
  static const int kcls[3] = {LAT_K_SEP_X, LAT_K_SEP_Y, LAT_K_SEP_Z};
  Timed t(h, kcls[axis]);
  SepArgs a{};
  a.grid_out = grid_out;
  a.nx = h->nx; a.ny = h->ny; a.nz = h->nz; a.nf = h->nf;
  a.phi = h->fld[h->cur];
  a.phic = h->fldc;
  a.pi = h->fldp;
  a.phi_out = h->fld[1 - h->cur];
  a.phic_out = h->fldc_alt;
  a.pi_out = h->fldp_alt;
  if (h->sep_stream) {  // in place (every tile is updated by the block that read it); lap holds zs
    a.phi_out = h->fld[h->cur];
    a.phic_out = h->fldc;
    a.pi_out = h->fldp;
    a.lap = h->lap;
    a.lap_out = h->lap;
  } else {
    a.lap = axis == 2 ? h->lap_alt : h->lap;
    a.lap_out = axis == 0 ? h->lap : h->lap_alt;
  }
  a.twN = h->tw[axis];
  if (!h->sep_ok || !a.twN || !a.phi || !a.phi_out || !a.pi || !a.pi_out || !a.lap || !a.lap_out ||
      (h->prec == LAT_FP32_KAHAN && (!a.phic || !a.phic_out)))
    return set_error(LAT_ERR_STATE, "separable pass buffers missing");
  const int n = axis == 0 ? h->nx : (axis == 1 ? h->ny : h->nz);
  const double dk = axis == 0 ? h->dkx : (axis == 1 ? h->dky : h->dkz);
  a.dk2 = dk * dk;
  a.model = model_of(h);
  a.hk = hk; a.hg = hg; a.hd = hd;
  a.Nd = (double)h->N;
  a.conf = conformal(h) ? 1 : 0;
  const int64_t pairs = h->nf == 2 ? 1 : 2;
  a.nlines = axis == 0 ? (int64_t)h->ny * h->nz / pairs
                       : (axis == 1 ? (int64_t)h->nx * h->nz / pairs : (int64_t)h->nx * h->ny / pairs);
  a.sc = h->sc;
  a.rb = red(h);
  a.nsm = h->nsm;
  a.stream = h->sep_stream ? 1 : 0;
  a.runs = 0;                // the two fields of this lattice form one pair
  a.pair_lines = a.nlines;
  if (h->sep_stream && axis > 0) {  // passes Y and Z move their tiles by TMA
    const int k = axis - 1;
    if (h->sep_tm_for[k][0] != a.lap || h->sep_tm_for[k][1] != a.pi_out) {
      const int lines = n == 128 ? sep_stream_lines_128(axis) : sep_stream_lines_256(axis);
      RET(encode_stream_tmaps(a, axis, lines, n));
      h->sep_tm_zs[k] = a.tm_zs;
      h->sep_tm_pi[k] = a.tm_pi;
      h->sep_tm_for[k][0] = a.lap;
      h->sep_tm_for[k][1] = a.pi_out;
    }
    a.tm_zs = h->sep_tm_zs[k];
    a.tm_pi = h->sep_tm_pi[k];
  }
  int st;
  switch (n) {
    case 16: st = launch_sep_16(a, h->prec, axis, h->stream); break;
    case 32: st = launch_sep_32(a, h->prec, axis, h->stream); break;
    case 64: st = launch_sep_64(a, h->prec, axis, h->stream); break;
    case 128: st = launch_sep_128(a, h->prec, axis, h->stream); break;
    case 256: st = launch_sep_256(a, h->prec, axis, h->stream); break;
    case 512: st = launch_sep_512(a, h->prec, axis, h->stream); break;
    default: return set_error(LAT_ERR_UNSUPPORTED, "separable pass length");
  }
  if (st != LAT_OK || h->sep_stream) return st;
  if (axis == 0) {  // drifted fields now live in the second buffers
    h->cur = 1 - h->cur;
    std::swap(h->fldc, h->fldc_alt);
  } else if (axis == 2) {  // kicked momenta
    std::swap(h->fldp, h->fldp_alt);
  }
  return LAT_OK;
}

// Separable spectral execution of an op list: every kick becomes the passes
// X (carrying the preceding drift), Y and Z (the kick); the last drift runs
// stand-alone.  Returns LAT_ERR_UNSUPPORTED (nothing launched) when the list
// is not D (G K G D | K D+)* shaped.
int exec_sep(lat_s* h, const std::vector<Op>& ops) {
  const bool conf = conformal(h);
  struct Grp { double hk, hg, hd; };
  std::vector<Grp> grp;
  double lead = 0;
  size_t i = 0;
  while (i < ops.size() && ops[i].t == 'D') {
    lead += ops[i++].h;
    if (conf) break;
  }
  while (i < ops.size()) {
    if (conf) {
      if (i + 3 < ops.size() && ops[i].t == 'G' && ops[i + 1].t == 'K' && ops[i + 2].t == 'G' && ops[i + 3].t == 'D' &&
          ops[i].h == ops[i + 2].h) {
        grp.push_back({ops[i + 1].h, ops[i].h, ops[i + 3].h});
        i += 4;
        continue;
      }
    } else if (ops[i].t == 'K' && i + 1 < ops.size() && ops[i + 1].t == 'D') {
      Grp g{ops[i].h, 0.0, 0.0};
      ++i;
      while (i < ops.size() && ops[i].t == 'D') g.hd += ops[i++].h;
      grp.push_back(g);
      continue;
    }
    return LAT_ERR_UNSUPPORTED;
  }
  double pending = lead;
  if (h->sep_stream && !grp.empty()) {
    // the fields' means (the first kick's shifts) and, expanding, sum pi^2 and
    // the coefficients of the first kick
    Timed t(h, LAT_K_OTHER);
    RET(launch_pi2_sum(h->fldp, (int64_t)h->nf * h->N, h->sc, red(h), 2 * h->nsm, h->stream,
                       KickW{grp[0].hk, grp[0].hg, lead, conf ? 1 : 0}, (double)h->N, h->fld[h->cur], h->N));
  }
  for (size_t gi = 0; gi < grp.size(); ++gi) {
    const Grp& g = grp[gi];
    if (h->sep_stream) {
      // every streamed pass takes the kick's weights and pass X's drift (the
      // scalar block keeps the pre-kick state until the finalize after Z)
      SepFinArgs f{};
      RET(sep_pass(h, 0, g.hk, g.hg, pending, &f.gx));
      RET(sep_pass(h, 1, g.hk, g.hg, pending, &f.gy));
      RET(sep_pass(h, 2, g.hk, g.hg, pending, &f.gz));
      f.sc = h->sc;
      f.part = red(h).partials;
      f.hk = g.hk;
      f.hg = g.hg;
      f.hd = pending;
      f.Nd = (double)h->N;
      f.conf = conf ? 1 : 0;
      // the next kick takes this group's drift in its pass X
      if (conf && gi + 1 < grp.size()) f.next = KickW{grp[gi + 1].hk, grp[gi + 1].hg, g.hd, 1};
      if (!conf) f.gy = f.gz = 0;  // a static background writes no Y, Z partials
      if (4 * f.gx > SEP_PART_Y || f.gy > SEP_PART_Z - SEP_PART_Y || (SEP_PART_Z + 2 * f.gz) > 16 * h->red_cap)
        return set_error(LAT_ERR_STATE, "streamed separable passes: partial sums exceed the reduction buffer");
      Timed t(h, LAT_K_OTHER);
      RET(launch_sep_finalize(f, h->stream));
    } else {
      RET(sep_pass(h, 0, 0.0, 0.0, pending));
      RET(sep_pass(h, 1, 0.0, 0.0, 0.0));
      RET(sep_pass(h, 2, g.hk, g.hg, 0.0));
    }
    pending = g.hd;
  }
  if (pending != 0.0) RET(exec_drift(h, pending));
  return LAT_OK;
}

// Op list with the closure: the network evaluated on the fields before the
// first of every cl_every kicks, and its force correction added after each
// kick (the kick itself is unchanged).  On a spectral lattice the groups of
// exec_fused (K D... in Minkowski, G K G D in conformal) run as the fused
// kick+drift with the correction inside, the network evaluated before the
// group with the scale factor after its first gravity half-step; every other
// op runs on its own, a kick followed by the separate correction kernel.
int exec_closure(lat_s* h, const std::vector<Op>& ops) {
  net::out_scale(h->cl_net, h->cl_tscale);  // the network's current normalisation
  const bool conf = conformal(h);
  const bool fuse = spectral(h) && !(conf && h->cfg.split_order == LAT_SPLIT_DEFROST);
  const int fp64 = h->prec == LAT_FP64 ? 1 : 0;
  int kicks = 0;
  auto run_net = [&](double hg, cudaStream_t s) -> int {
    const size_t fb = (size_t)h->N * h->rsz;
    const void* ch[4] = {h->fld[h->cur], (const char*)h->fld[h->cur] + fb, h->fldp, (const char*)h->fldp + fb};
    return net::infer(h->cl_net, ch, fp64, h->nx, h->ny, h->nz, h->cl_units ? h->sc : nullptr, hg, h->cl_b, s);
  };
  auto infer = [&](double hg) -> int {  // before the kick with index `kicks`, in order
    if (kicks++ % h->cl_every) return LAT_OK;
    Timed t(h, LAT_K_OTHER);
    return run_net(hg, h->stream);
  };
  // before a fused group: the network on the side stream, forked here; the
  // event the group's kick+drift joins (null: nothing to join)
  auto infer_side = [&](double hg, cudaEvent_t* join) -> int {
    *join = nullptr;
    if (h->timing || !h->cl_stream) return infer(hg);  // timed launches stay in order
    if (kicks++ % h->cl_every) return LAT_OK;
    CK(cudaEventRecord(h->cl_fork, h->stream));
    CK(cudaStreamWaitEvent(h->cl_stream, h->cl_fork, 0));
    RET(run_net(hg, h->cl_stream));
    CK(cudaEventRecord(h->cl_join, h->cl_stream));
    *join = h->cl_join;
    return LAT_OK;
  };
  size_t i = 0;
  while (i < ops.size()) {
    if (fuse && !conf && ops[i].t == 'K' && i + 1 < ops.size() && ops[i + 1].t == 'D') {
      double hd = 0;
      size_t j = i + 1;
      while (j < ops.size() && ops[j].t == 'D') hd += ops[j++].h;
      cudaEvent_t join;
      RET(infer_side(0.0, &join));
      RET(exec_kd(h, ops[i].h, 0.0, hd, true, join));
      i = j;
      continue;
    }
    if (fuse && conf && ops[i].t == 'G' && i + 3 < ops.size() && ops[i + 1].t == 'K' && ops[i + 2].t == 'G' &&
        ops[i + 3].t == 'D' && ops[i].h == ops[i + 2].h) {
      cudaEvent_t join;
      RET(infer_side(ops[i].h, &join));
      RET(exec_kd(h, ops[i + 1].h, ops[i].h, ops[i + 3].h, true, join));
      i += 4;
      continue;
    }
    const Op& o = ops[i++];
    switch (o.t) {
      case 'D': RET(exec_drift(h, o.h)); break;
      case 'G': RET(exec_grav(h, o.h)); break;
      case 'K': {
        RET(infer(0.0));
        RET(exec_kick(h, o.h));
        Timed t(h, LAT_K_OTHER);
        net::CorrArgs c{};
        c.pi = h->fldp;
        c.out = h->cl_b.out;
        c.tscale[0] = h->cl_tscale[0];
        c.tscale[1] = h->cl_tscale[1];
        c.hk = o.h;
        c.conf = conf ? 1 : 0;
        c.units = h->cl_units;
        c.sc = h->sc;
        c.N = h->N;
        RET(net::corr_kick(c, fp64, h->nsm, h->stream));
        break;
      }
      default: break;
    }
  }
  return LAT_OK;
}

int exec_fused(lat_s* h, const std::vector<Op>& in) {
  std::vector<Op> ops;
  for (const Op& o : in)
    if (o.t != 'M') ops.push_back(o);
  if (h->cl_net) return exec_closure(h, ops);
  const bool conf = conformal(h);
  if (h->sep && (!conf || h->cfg.split_order == LAT_SPLIT_PSEUDOSPEC)) {
    const int st = exec_sep(h, ops);
    if (st != LAT_ERR_UNSUPPORTED) return st;
  }
  if (conf && !spectral(h)) return exec_plain(h, ops);
  if (conf && h->cfg.split_order == LAT_SPLIT_DEFROST) return exec_plain(h, ops);
  size_t i = 0;
  while (i < ops.size()) {
    if (!conf && ops[i].t == 'K' && i + 1 < ops.size() && ops[i + 1].t == 'D') {
      double hd = 0;
      size_t j = i + 1;
      while (j < ops.size() && ops[j].t == 'D') hd += ops[j++].h;
      RET(exec_kd(h, ops[i].h, 0.0, hd));
      i = j;
      continue;
    }
    if (conf && ops[i].t == 'G' && i + 3 < ops.size() && ops[i + 1].t == 'K' && ops[i + 2].t == 'G' &&
        ops[i + 3].t == 'D' && ops[i].h == ops[i + 2].h) {
      RET(exec_kd(h, ops[i + 1].h, ops[i].h, ops[i + 3].h));
      i += 4;
      continue;
    }
    if (ops[i].t == 'D' && !conf) {  // leading drift(s)
      double hd = 0;
      size_t j = i;
      while (j < ops.size() && ops[j].t == 'D') hd += ops[j++].h;
      RET(exec_drift(h, hd));
      i = j;
      continue;
    }
    std::vector<Op> one(1, ops[i]);
    RET(exec_plain(h, one));
    ++i;
  }
  return LAT_OK;
}

int ensure_stage(lat_s* h, size_t elems) {
  if (h->stage_elems >= elems) return LAT_OK;
  if (h->stage) cudaFree(h->stage);
  h->stage = nullptr;
  CK(cudaMalloc(&h->stage, elems * sizeof(double)));
  h->stage_elems = elems;
  return LAT_OK;
}

// Host Fortran array (nfld, 1-lo:n+hi, ...) <-> unpadded AoS staging.
int copy_aos(lat_s* h, double* host, int lo, int hi, bool to_device) {
  const int nf = h->nf;
  const size_t row = (size_t)nf * h->nx * sizeof(double);
  if (lo == 0 && hi == 0) {
    const size_t bytes = (size_t)nf * h->N * sizeof(double);
    if (to_device) CK(cudaMemcpyAsync(h->stage, host, bytes, cudaMemcpyHostToDevice, h->stream));
    else CK(cudaMemcpyAsync(host, h->stage, bytes, cudaMemcpyDeviceToHost, h->stream));
    return LAT_OK;
  }
  const int64_t px = h->nx + lo + hi, py = h->ny + lo + hi;
  for (int z = 0; z < h->nz; ++z) {
    double* hp = host + (int64_t)nf * (lo + px * (lo + py * (int64_t)(z + lo)));
    double* dp = h->stage + (int64_t)nf * h->nx * h->ny * z;
    if (to_device)
      CK(cudaMemcpy2DAsync(dp, row, hp, (size_t)nf * px * sizeof(double), row, h->ny, cudaMemcpyHostToDevice, h->stream));
    else
      CK(cudaMemcpy2DAsync(hp, (size_t)nf * px * sizeof(double), dp, row, row, h->ny, cudaMemcpyDeviceToHost, h->stream));
  }
  return LAT_OK;
}

// Device address of a host array the GPU reads and writes in place (pinned
// and mapped: cudaHostAlloc, lat_host_alloc, cudaHostRegister), else null.
// Unpadded Fortran arrays at such addresses are converted by one kernel that
// reads or writes host memory over the CPU-GPU link, with no staging copy;
// LAT_NO_DIRECT_HOST=1 forces the staged copies.
double* mapped_host(const void* host) {
  if (getenv_flag("LAT_NO_DIRECT_HOST")) return nullptr;
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, host) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (at.type != cudaMemoryTypeHost || !at.devicePointer) return nullptr;
  return static_cast<double*>(at.devicePointer);
}

int read_scalars(lat_s* h, DevScalars* out) {
  CK(cudaMemcpyAsync(out, h->sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return LAT_OK;
}

// ball_r2 > 0 (FD lattices): also the sums of LOG.out's rhoball into ball[3]
int compute_energies(lat_s* h, double* out, double ball_r2 = 0.0, double* ball = nullptr) {
  if (h->slab) {  // the gradient sums read the ghost planes; no ball sums
    if (ball) return set_error(LAT_ERR_UNSUPPORTED, "not available on a z-slab handle");
    RET(slab_exchange(h));
  }
  EnergyArgs e{};
  e.ball_r2 = spectral(h) ? 0.0 : ball_r2;
  if (h->slab) {
    const int64_t plane = (int64_t)h->nx * h->ny;
    e.t_lo = plane;
    e.t_hi = plane * (1 + h->nz_loc);
  }
  e.dx = h->dx;
  e.nx = h->nx; e.ny = h->ny; e.nz = h->nz; e.nf = h->nf;
  e.phi = h->fld[h->cur];
  e.phic = h->fldc;
  e.pi = h->fldp;
  e.u = h->cfg.gw ? h->u[h->ucur] : nullptr;
  e.pu = h->cfg.gw ? h->pu : nullptr;
  e.fd = spectral(h) ? 0 : 1;
  for (int i = 0; i < 4; ++i) e.c[i] = h->c[i];
  e.model = model_of(h);
  e.sc = h->sc;
  e.rb = red(h);
  e.grid = h->pw_grid;
  e.block = 256;
  {
    Timed t(h, LAT_K_OTHER);
    RET(launch_energy(e, h->prec, h->stream));
  }
  if (spectral(h)) {
    RET(fft_exec_r2c(h, h->p_r2c, h->fld[h->cur], h->Fk));
    Timed t(h, LAT_K_OTHER);
    RET(launch_parseval(h->Fk, h->nx, h->ny, h->nz, h->nf, h->dkx * h->dkx, h->dky * h->dky, h->dkz * h->dkz,
                        h->sc, 8, red(h), h->pw_grid, h->prec, h->stream));
  }
  DevScalars s;
  RET(read_scalars(h, &s));
  if (s.err & 2u) return set_error(LAT_ERR_TIMEOUT, "a tensor copy of a streamed pass was not completed in time");
  if (s.err & 1u) return set_error(LAT_ERR_NAN, "NaN/Inf in a lattice reduction");
  if (h->slab) RET(slab_allreduce(h, s.red, 8));  // KE, PE, means, the FD gradient sums and GW sums
  const bool conf = conformal(h);
  const double a = conf ? s.a : 1.0;
  const double Nd = nd_of(h);
  const double knorm = conf ? 1.0 / std::pow(a, 6) : 1.0;
  const double elap = 1.0 / (h->dx * h->dx) / h->c[4];
  double ge_raw;  // -sum phi lap phi
  if (spectral(h)) ge_raw = s.red[8] / Nd;
  else ge_raw = s.red[4] * elap;
  out[LAT_E_KE] = 0.5 * s.red[0] * knorm / Nd;
  out[LAT_E_GE_LAP] = 0.5 * ge_raw / Nd / (a * a);
  out[LAT_E_GE_GRAD] = spectral(h) ? out[LAT_E_GE_LAP] : 0.25 / (a * h->dx) / (a * h->dx) / h->c[4] * s.red[5] / Nd;
  out[LAT_E_PE] = s.red[1] / Nd;
  out[LAT_E_RHO] = out[LAT_E_KE] + out[LAT_E_GE_LAP] + out[LAT_E_PE];
  const double H = conf ? -s.ap / 6.0 / (a * a) : 0.0;
  out[LAT_E_GRAV] = -3.0 * H * H;
  out[LAT_E_RESIDUAL] = (out[LAT_E_RHO] + out[LAT_E_GRAV]) / out[LAT_E_RHO];
  out[LAT_E_A] = a;
  out[LAT_E_AP] = conf ? s.ap : 0.0;
  out[LAT_E_MEAN0] = s.red[2] / Nd;
  out[LAT_E_MEAN1] = s.red[3] / Nd;
  out[LAT_E_GW] = h->cfg.gw ? 0.5 * (s.red[6] + s.red[7] * elap) / Nd : 0.0;
  if (ball) {
    ball[0] = s.red[9];
    ball[1] = s.red[10];
    ball[2] = s.red[11];
  }
  return LAT_OK;
}

int free_graphs(lat_s* h) {
  for (auto& g : h->graphs) cudaGraphExecDestroy(g.exec);
  h->graphs.clear();
  return LAT_OK;
}

int src_ptr(lat_s* h, int what, int field, const void** p) {
  if (field < 0 || field >= h->nf) return set_error(LAT_ERR_ARG, "bad field index");
  const char* base;
  if (what == LAT_SPEC_FLD) base = (const char*)h->fld[h->cur];
  else if (what == LAT_SPEC_FLDP) base = (const char*)h->fldp;
  else return set_error(LAT_ERR_ARG, "bad spectrum source");
  *p = base + (size_t)field * h->N * h->rsz;
  return LAT_OK;
}

int run_spectrum(lat_s* h, const void* F1, const void* F2, int mode, int nbins, double* hostout, int prec) {
  SpecArgs s{};
  s.nx = h->nx; s.ny = h->ny; s.nz = h->nz;
  s.F1 = F1; s.F2 = F2; s.mode = mode; s.nbins = nbins;
  s.partials = h->spec_part;
  s.out = h->spec_out;
  s.counter = h->spec_counter;
  s.grid = h->spec_grid;
  s.block = 256;
  {
    Timed t(h, LAT_K_OTHER);
    RET(launch_spectrum(s, prec, h->stream));
  }
  CK(cudaMemcpyAsync(hostout, h->spec_out, sizeof(double) * 3 * nbins, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return LAT_OK;
}

const int kMaxBins = 2048;

// Half spectrum of one field or momentum array for the output routines.  An
// FP32 field is transformed in FP64 from phi_hi - c, so a field sitting near
// a large mean keeps the digits of its fluctuation (an FP32 transform of
// phi_hi alone would not).  Returns the precision of the spectrum written.
int output_spectrum(lat_s* h, int what, int field, int slot, void** Fout, int* prec) {
  const void* src = nullptr;
  RET(src_ptr(h, what, field, &src));
  if (h->prec == LAT_FP64) {
    void* F = (char*)h->Fk + (size_t)slot * h->M * h->csz;
    RET(fft_exec_r2c(h, h->p_r2c1, src, F));
    *Fout = F;
    *prec = LAT_FP64;
    return LAT_OK;
  }
  if (!h->Fk64) CK(cudaMalloc(&h->Fk64, (size_t)2 * h->M * sizeof(double2)));
  if (!h->have_d2z1) {
    CF(cufftCreate(&h->p_d2z1));
    int n[3] = {h->nz, h->ny, h->nx};
    size_t ws = 0;
    CF(cufftMakePlanMany(h->p_d2z1, 3, n, nullptr, 1, 0, nullptr, 1, 0, CUFFT_D2Z, 1, &ws));
    CF(cufftSetStream(h->p_d2z1, h->stream));
    h->have_d2z1 = true;
  }
  RET(ensure_stage(h, (size_t)std::max(h->nf, 2) * h->N));
  const void* comp = (what == LAT_SPEC_FLD && h->fldc) ? (const char*)h->fldc + (size_t)field * h->N * h->rsz : nullptr;
  double* tmp = h->stage + (size_t)slot * h->N;
  RET(launch_to_fp64(src, comp, h->N, h->prec, tmp, h->stream));
  void* F = (double2*)h->Fk64 + (size_t)slot * h->M;
  {
    Timed t(h, LAT_K_FFT_R2C);
    CF(cufftExecD2Z(h->p_d2z1, tmp, (cufftDoubleComplex*)F));
  }
  *Fout = F;
  *prec = LAT_FP64;
  return LAT_OK;
}

}  // namespace

namespace {
// lat_symp through the handle's graph cache.  run = false builds and caches
// the graph of the call without launching it (the handle's state is left
// as it was).
int symp_graph(lat_s* h, int32_t order, double dt, int32_t nsteps, bool run) {
  std::vector<Op> ops;
  double tg[3] = {h->tglobal[0], h->tglobal[1], h->tglobal[2]};
  Emitter em = emitter(h, &ops, tg);
  RET(em.symp(order, dt, nsteps));
  if (h->slab) {  // the hooks run on the host between the kernels: no graphs
    if (!run) return LAT_OK;
    RET(exec_slab(h, ops));
    std::memcpy(h->tglobal, tg, sizeof(tg));
    return LAT_OK;
  }
  const bool graphs = h->use_graphs && !h->timing;
  // a graph holds the closure's buffers and its normalisation by value: it
  // matches only the same network, normalisation, cadence and units
  const uint64_t cl_key = h->cl_net ? net::net_key(h->cl_net) : 0;
  const int cl_every = h->cl_net ? h->cl_every : 0, cl_units = h->cl_net ? h->cl_units : 0;
  if (!graphs) {
    if (!run) return LAT_OK;
    RET(exec_fused(h, ops));
    std::memcpy(h->tglobal, tg, sizeof(tg));
    return LAT_OK;
  }
  for (auto& ge : h->graphs) {
    if (ge.order == order && ge.dt == dt && ge.nsteps == nsteps && ge.cur == h->cur && ge.ucur == h->ucur &&
        ge.fldc == h->fldc && ge.fldp == h->fldp && ge.cl_key == cl_key && ge.cl_every == cl_every &&
        ge.cl_units == cl_units) {
      if (!run) return LAT_OK;
      CK(cudaGraphLaunch(ge.exec, h->stream));
      h->launches += ge.kernels;
      h->cur = ge.cur_after;
      h->ucur = ge.ucur_after;
      if (h->fldc != ge.fldc_after) std::swap(h->fldc, h->fldc_alt);
      if (h->fldp != ge.fldp_after) std::swap(h->fldp, h->fldp_alt);
      std::memcpy(h->tglobal, tg, sizeof(tg));
      return LAT_OK;
    }
  }
  GraphEntry ge{};
  ge.order = order; ge.dt = dt; ge.nsteps = nsteps; ge.cur = h->cur; ge.ucur = h->ucur;
  ge.cl_key = cl_key; ge.cl_every = cl_every; ge.cl_units = cl_units;
  ge.fldc = h->fldc; ge.fldp = h->fldp;
  void* const c_alt0 = h->fldc_alt;
  void* const p_alt0 = h->fldp_alt;
  const int64_t before = h->launches;
  auto rewind = [&]() {  // pointer state before the capture
    h->cur = ge.cur; h->ucur = ge.ucur;
    h->fldc = ge.fldc; h->fldc_alt = c_alt0;
    h->fldp = ge.fldp; h->fldp_alt = p_alt0;
  };
  CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeRelaxed));
  int st = exec_fused(h, ops);
  cudaGraph_t graph = nullptr;
  cudaError_t e = cudaStreamEndCapture(h->stream, &graph);
  if (st != LAT_OK) {
    if (graph) cudaGraphDestroy(graph);
    rewind();
    h->launches = before;
    return st;
  }
  if (e != cudaSuccess) {
    rewind();
    h->launches = before;
    return cuda_fail(e, "graph capture");
  }
  ge.kernels = h->launches - before;
  ge.cur_after = h->cur;
  ge.ucur_after = h->ucur;
  ge.fldc_after = h->fldc;
  ge.fldp_after = h->fldp;
  e = cudaGraphInstantiate(&ge.exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) {
    rewind();
    h->launches = before;
    return cuda_fail(e, "graph instantiate");
  }
  if (h->graphs.size() >= 8) {
    cudaGraphExecDestroy(h->graphs.front().exec);
    h->graphs.erase(h->graphs.begin());
  }
  h->graphs.push_back(ge);
  if (!run) {  // nothing ran: the handle keeps its state
    rewind();
    h->launches = before;
    return LAT_OK;
  }
  CK(cudaGraphLaunch(ge.exec, h->stream));
  std::memcpy(h->tglobal, tg, sizeof(tg));
  return LAT_OK;
}
}  // namespace

// ====================================================================== C ABI
extern "C" {

const char* lat_last_error(void) { return t_err.c_str(); }
const char* lat_version(void) { return "lattice-gb300 0.1 (sm_103a)"; }

int lat_destroy(lat_t* h) {
  if (!h) return LAT_OK;
  cudaSetDevice(h->dev);
  if (h->stream) cudaStreamSynchronize(h->stream);
  if (h->cl_stream) cudaStreamSynchronize(h->cl_stream);
  free_graphs(h);
  if (h->cl_net) net::net_attach_ref(h->cl_net, -1);
  if (h->cl_fork) cudaEventDestroy(h->cl_fork);
  if (h->cl_join) cudaEventDestroy(h->cl_join);
  if (h->cl_stream) cudaStreamDestroy(h->cl_stream);
  for (void* t : h->tw)
    if (t) cudaFree(t);
  {
    void* cb[] = {h->cl_b.a0, h->cl_b.a1, h->cl_b.a2, h->cl_b.out};
    for (void* b : cb)
      if (b) cudaFree(b);
  }
  if (h->Fk64) cudaFree(h->Fk64);
  if (h->have_d2z1) cufftDestroy(h->p_d2z1);
  void* bufs[] = {h->fld[0], h->fld[1], h->fldc, h->fldp, h->lap, h->fldc_alt, h->fldp_alt, h->lap_alt, h->Fk,
                  h->u[0], h->u[1], h->pu, h->Fk6,
                  h->sc, h->rb.partials, h->rb.counter, h->spec_part, h->spec_out, h->spec_counter, h->stage,
                  h->fft_work};
  for (void* b : bufs)
    if (b) cudaFree(b);
  if (h->have_r2c) cufftDestroy(h->p_r2c);
  if (h->have_c2r) cufftDestroy(h->p_c2r);
  if (h->have_r2c1) cufftDestroy(h->p_r2c1);
  if (h->have_c2r1) cufftDestroy(h->p_c2r1);
  if (h->have_r2c6) cufftDestroy(h->p_r2c6);
  for (auto& e : h->ev_pool) { cudaEventDestroy(e.a); cudaEventDestroy(e.b); }
  for (auto& m : h->marks)
    if (m) cudaEventDestroy(m);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return LAT_OK;
}

int lat_create(lat_t** out, const lat_config* cfg) {
  if (!out || !cfg) return set_error(LAT_ERR_ARG, "null argument");
  *out = nullptr;
  if (cfg->nx < 2 || cfg->ny < 2 || cfg->nz < 2 || !(cfg->len > 0)) return set_error(LAT_ERR_ARG, "bad lattice shape");
  if (cfg->nfld < 1 || cfg->nfld > 2) return set_error(LAT_ERR_UNSUPPORTED, "nfld must be 1 or 2");
  if (cfg->laplacian != LAT_LAP_SPECTRAL && cfg->laplacian != LAT_LAP_FD7 && cfg->laplacian != LAT_LAP_FD27)
    return set_error(LAT_ERR_ARG, "bad laplacian");
  if (cfg->background != LAT_BG_MINKOWSKI && cfg->background != LAT_BG_CONFORMAL)
    return set_error(LAT_ERR_ARG, "bad background");
  if (cfg->precision != LAT_FP64 && cfg->precision != LAT_FP32_KAHAN) return set_error(LAT_ERR_ARG, "bad precision");
  if (cfg->split_order != LAT_SPLIT_PSEUDOSPEC && cfg->split_order != LAT_SPLIT_DEFROST)
    return set_error(LAT_ERR_ARG, "bad split order");
  if (cfg->model < LAT_MODEL_PHI4 || cfg->model > LAT_MODEL_FREE) return set_error(LAT_ERR_ARG, "bad model");
  if (cfg->model == LAT_MODEL_PHI4_G2 && cfg->nfld != 2) return set_error(LAT_ERR_ARG, "two-field model needs nfld = 2");
  if (cfg->gw && (cfg->laplacian == LAT_LAP_SPECTRAL || cfg->background != LAT_BG_MINKOWSKI))
    return set_error(LAT_ERR_UNSUPPORTED, "GW evolution needs an FD stencil and Minkowski background");
  const int64_t N = (int64_t)cfg->nx * cfg->ny * cfg->nz;
  const int64_t M = (int64_t)(cfg->nx / 2 + 1) * cfg->ny * cfg->nz;
  if (6 * M >= ((int64_t)1 << 31) || 6 * N >= ((int64_t)1 << 33)) return set_error(LAT_ERR_ARG, "lattice too large");

  lat_s* h = new lat_s();
  h->cfg = *cfg;
  h->nx = cfg->nx; h->ny = cfg->ny; h->nz = cfg->nz; h->nf = cfg->nfld;
  h->N = N; h->M = M;
  h->dx = cfg->len / cfg->nx;
  const double twopi = 6.2831853071795864769252867665590;
  h->dkx = twopi / (h->nx * h->dx);
  h->dky = twopi / (h->ny * h->dx);
  h->dkz = twopi / (h->nz * h->dx);
  bool zero = true;
  for (int i = 0; i < 5; ++i) zero = zero && cfg->stencil[i] == 0.0;
  if (zero) {
    if (cfg->laplacian == LAT_LAP_FD7) { h->c[0] = -6; h->c[1] = 1; h->c[2] = 0; h->c[3] = 0; h->c[4] = 1; }
    else { h->c[0] = -128; h->c[1] = 14; h->c[2] = 3; h->c[3] = 1; h->c[4] = 30; }
  } else {
    for (int i = 0; i < 5; ++i) h->c[i] = cfg->stencil[i];
  }
  h->prec = cfg->precision;
  h->rsz = h->prec == LAT_FP64 ? 8 : 4;
  h->csz = 2 * h->rsz;
  h->dev = cfg->device;
  ApiGuard g(h);
  auto bail = [&](int code) { lat_destroy(h); return code; };
  cudaError_t e = cudaSetDevice(h->dev);
  if (e != cudaSuccess) return bail(cuda_fail(e, "cudaSetDevice"));
  int nsm = 0;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, h->dev);
  h->nsm = nsm > 0 ? nsm : 152;
  if ((e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking)) != cudaSuccess)
    return bail(cuda_fail(e, "stream"));

  auto alloc = [&](void** p, size_t bytes) -> int {
    cudaError_t ee = cudaMalloc(p, bytes);
    if (ee != cudaSuccess) return set_error(LAT_ERR_ALLOC, std::string("cudaMalloc: ") + cudaGetErrorString(ee));
    cudaMemsetAsync(*p, 0, bytes, h->stream);
    return LAT_OK;
  };
  const size_t fb = (size_t)h->nf * N * h->rsz;
  int st;
  if ((st = alloc(&h->fld[0], fb))) return bail(st);
  if (!spectral(h) && (st = alloc(&h->fld[1], fb))) return bail(st);
  if (h->prec == LAT_FP32_KAHAN && (st = alloc(&h->fldc, fb))) return bail(st);
  if ((st = alloc(&h->fldp, fb))) return bail(st);
  if ((st = alloc(&h->lap, fb))) return bail(st);
  if ((st = alloc(&h->Fk, (size_t)std::max(h->nf, 2) * M * h->csz))) return bail(st);
  if (cfg->gw) {
    const size_t gb = (size_t)6 * N * h->rsz;
    if ((st = alloc(&h->u[0], gb))) return bail(st);
    if ((st = alloc(&h->u[1], gb))) return bail(st);
    if ((st = alloc(&h->pu, gb))) return bail(st);
  }
  if ((st = alloc((void**)&h->sc, sizeof(DevScalars)))) return bail(st);
  DevScalars s0{};
  s0.a = 1.0;
  cudaMemcpyAsync(h->sc, &s0, sizeof(DevScalars), cudaMemcpyHostToDevice, h->stream);

  // pointwise grid: a few resident blocks per SM, all blocks alive at once
  h->pw_block = 256;
  h->pw_grid = h->nsm * 4;
  int64_t maxb = std::max<int64_t>(h->pw_grid, 4096);
  for (int ty : {2, 4, 8, 16})
    for (int zc : {2, 4, 8, 16, 32, 64}) maxb = std::max<int64_t>(maxb, fd_max_blocks(h->nx, h->ny, h->nz, ty, zc));
  h->red_cap = maxb;
  if ((st = alloc((void**)&h->rb.partials, (size_t)maxb * 16 * sizeof(double)))) return bail(st);
  if ((st = alloc((void**)&h->rb.counter, 64))) return bail(st);
  h->spec_grid = h->nsm * 2;
  if ((st = alloc((void**)&h->spec_part, (size_t)h->spec_grid * 3 * kMaxBins * sizeof(double)))) return bail(st);
  if ((st = alloc((void**)&h->spec_out, (size_t)3 * kMaxBins * sizeof(double)))) return bail(st);
  if ((st = alloc((void**)&h->spec_counter, 64))) return bail(st);
  h->fd_ty = 8;
  h->fd_zc = std::min(32, h->nz);

  if ((st = make_plan(h, &h->p_r2c1, &h->have_r2c1, true, 1))) return bail(st);
  if ((st = make_plan(h, &h->p_c2r1, &h->have_c2r1, false, 1))) return bail(st);
  if (spectral(h)) {
    if ((st = make_plan(h, &h->p_r2c, &h->have_r2c, true, h->nf))) return bail(st);
    if ((st = make_plan(h, &h->p_c2r, &h->have_c2r, false, h->nf))) return bail(st);
  }
  if (spectral(h)) {
    auto pow2ok = [](int n) { return n >= 16 && n <= 512 && (n & (n - 1)) == 0; };
    auto cols = [&](int n) {  // x-columns per block of a y or z pass of length n
      switch (n) {
        case 16: return sep_columns_16(h->prec, h->nf);
        case 32: return sep_columns_32(h->prec, h->nf);
        case 64: return sep_columns_64(h->prec, h->nf);
        case 128: return sep_columns_128(h->prec, h->nf);
        case 256: return sep_columns_256(h->prec, h->nf);
        default: return sep_columns_512(h->prec, h->nf);
      }
    };
    h->sep_ok = pow2ok(h->nx) && pow2ok(h->ny) && pow2ok(h->nz);
    // the passes need whole column blocks and (one field) an even number of x-rows
    if (h->sep_ok) h->sep_ok = h->nx % cols(h->ny) == 0 && h->nx % cols(h->nz) == 0;
    if (cfg->spectral_impl == LAT_SPEC_IMPL_SEPARABLE && !h->sep_ok)
      return bail(set_error(LAT_ERR_UNSUPPORTED, "separable spectral passes need power-of-two sides 16..512"));
    h->sep = h->sep_ok && cfg->spectral_impl == LAT_SPEC_IMPL_SEPARABLE && !getenv_flag("LAT_NO_SEPARABLE");
    // two FP32 fields on lines of 128 or 256 points whose passes all form
    // whole tiles: the streamed passes (LAT_SEP_CLASSIC=1 keeps the others)
    auto stream_lines = [](int n, int axis) {
      return n == 128 ? sep_stream_lines_128(axis) : (n == 256 ? sep_stream_lines_256(axis) : 0);
    };
    const int lx = stream_lines(h->nx, 0), ly = stream_lines(h->ny, 1), lz = stream_lines(h->nz, 2);
    h->sep_stream = h->sep_ok && h->prec == LAT_FP32_KAHAN && h->nf == 2 && lx && ly && lz &&
                    ((int64_t)h->ny * h->nz) % lx == 0 && h->nx % ly == 0 && h->nx % lz == 0 &&
                    !getenv_flag("LAT_SEP_CLASSIC");
    if (h->sep_ok) {
      if ((st = alloc(&h->fld[1], fb))) return bail(st);
      if (h->prec == LAT_FP32_KAHAN && (st = alloc(&h->fldc_alt, fb))) return bail(st);
      if ((st = alloc(&h->fldp_alt, fb))) return bail(st);
      if ((st = alloc(&h->lap_alt, fb))) return bail(st);
    }
    if (h->sep_ok) {  // the autotuner may switch an AUTO handle to the passes later
      const int dims[3] = {h->nx, h->ny, h->nz};
      for (int ax = 0; ax < 3; ++ax) {
        const int n = dims[ax];
        std::vector<double> w64(2 * n);
        std::vector<float> w32(2 * n);
        for (int j = 0; j < n; ++j) {
          const long double ang = -6.283185307179586476925286766559L * (long double)j / (long double)n;
          w64[2 * j] = (double)cosl(ang);
          w64[2 * j + 1] = (double)sinl(ang);
          w32[2 * j] = (float)w64[2 * j];
          w32[2 * j + 1] = (float)w64[2 * j + 1];
        }
        if ((st = alloc(&h->tw[ax], (size_t)n * h->csz))) return bail(st);
        const void* src = h->prec == LAT_FP64 ? (const void*)w64.data() : (const void*)w32.data();
        if ((e = cudaMemcpyAsync(h->tw[ax], src, (size_t)n * h->csz, cudaMemcpyHostToDevice, h->stream)) != cudaSuccess)
          return bail(cuda_fail(e, "twiddle upload"));
        if ((e = cudaStreamSynchronize(h->stream)) != cudaSuccess) return bail(cuda_fail(e, "twiddle upload"));
      }
    }
  }
  h->ev_pool.resize(4096);
  for (auto& ev : h->ev_pool) {
    cudaEventCreate(&ev.a);
    cudaEventCreate(&ev.b);
  }
  if ((e = cudaStreamSynchronize(h->stream)) != cudaSuccess) return bail(cuda_fail(e, "create sync"));
  h->use_graphs = !getenv_flag("LAT_NO_GRAPHS");
  *out = h;
  return LAT_OK;
}

int lat_get_config(const lat_t* h, lat_config* cfg) {
  if (!h || !cfg) return set_error(LAT_ERR_ARG, "null argument");
  *cfg = h->cfg;
  return LAT_OK;
}

// The NaN flag of the scalar block is sticky until the fields are replaced:
// every call that uploads or draws a new state clears it (and drops
// non-finite shifts carried over from the old state), so a handle that
// reported LAT_ERR_NAN is usable again after a fresh upload.
static int clear_nan_flag(lat_t* h) { return launch_state_reset(h->sc, h->stream); }

// Interior planes of a z-slab <-> unpadded Fortran-layout host arrays
// fld(nfld, nx, ny, nz_loc) (pad: the sum of the caller's padding, which
// must be zero).
static int slab_copy(lat_t* h, double* fld, int pad_f, double* fldp, int pad_p, bool up) {
  if (pad_f || pad_p) return set_error(LAT_ERR_UNSUPPORTED, "z-slab arrays take no ghost padding");
  const int64_t plane = (int64_t)h->nx * h->ny, Ni = plane * h->nz_loc;
  const size_t bytes = sizeof(double) * (size_t)h->nf * Ni;
  for (int which = 0; which < 2; ++which) {
    double* host = which == 0 ? fld : fldp;
    if (!host) continue;
    char* hi = static_cast<char*>(which == 0 ? h->fld[h->cur] : h->fldp) + (size_t)plane * h->rsz;
    char* c = (which == 0 && h->fldc) ? static_cast<char*>(h->fldc) + (size_t)plane * h->rsz : nullptr;
    if (up) {
      CK(cudaMemcpyAsync(h->stage, host, bytes, cudaMemcpyHostToDevice, h->stream));
      RET(launch_aos2soa(h->stage, h->nf, Ni, h->prec, hi, c, h->stream, h->N));
    } else {
      RET(launch_soa2aos(hi, c, h->nf, Ni, h->prec, h->stage, h->stream, h->N));
      CK(cudaMemcpyAsync(host, h->stage, bytes, cudaMemcpyDeviceToHost, h->stream));
    }
    CK(cudaStreamSynchronize(h->stream));
  }
  return LAT_OK;
}

int lat_upload(lat_t* h, const double* fld, int32_t fld_lo, int32_t fld_hi, const double* fldp, int32_t fldp_lo,
               int32_t fldp_hi) {
  if (!h) return set_error(LAT_ERR_ARG, "null handle");
  if (fld_lo < 0 || fld_hi < 0 || fldp_lo < 0 || fldp_hi < 0) return set_error(LAT_ERR_ARG, "negative padding");
  ApiGuard g(h);
  RET(clear_nan_flag(h));
  RET(ensure_stage(h, (size_t)h->nf * h->N));
  if (h->slab) return slab_copy(h, const_cast<double*>(fld), fld_lo + fld_hi, const_cast<double*>(fldp),
                                fldp_lo + fldp_hi, true);
  if (fld) {
    const double* d = (fld_lo == 0 && fld_hi == 0) ? mapped_host(fld) : nullptr;
    if (!d) {
      RET(copy_aos(h, const_cast<double*>(fld), fld_lo, fld_hi, true));
      d = h->stage;
    }
    RET(launch_aos2soa(d, h->nf, h->N, h->prec, h->fld[h->cur], h->fldc, h->stream));
  }
  if (fldp) {
    const double* d = (fldp_lo == 0 && fldp_hi == 0) ? mapped_host(fldp) : nullptr;
    if (!d) {
      RET(copy_aos(h, const_cast<double*>(fldp), fldp_lo, fldp_hi, true));
      d = h->stage;
    }
    RET(launch_aos2soa(d, h->nf, h->N, h->prec, h->fldp, nullptr, h->stream));  // momenta: no compensation
  }
  CK(cudaStreamSynchronize(h->stream));
  return LAT_OK;
}

int lat_download(lat_t* h, double* fld, int32_t fld_lo, int32_t fld_hi, double* fldp, int32_t fldp_lo,
                 int32_t fldp_hi) {
  if (!h) return set_error(LAT_ERR_ARG, "null handle");
  if (fld_lo < 0 || fld_hi < 0 || fldp_lo < 0 || fldp_hi < 0) return set_error(LAT_ERR_ARG, "negative padding");
  ApiGuard g(h);
  RET(ensure_stage(h, (size_t)h->nf * h->N));
  if (h->slab) return slab_copy(h, fld, fld_lo + fld_hi, fldp, fldp_lo + fldp_hi, false);
  if (fld) {
    double* d = (fld_lo == 0 && fld_hi == 0) ? mapped_host(fld) : nullptr;
    RET(launch_soa2aos(h->fld[h->cur], h->fldc, h->nf, h->N, h->prec, d ? d : h->stage, h->stream));
    if (!d) RET(copy_aos(h, fld, fld_lo, fld_hi, false));
  }
  if (fldp) {
    double* d = (fldp_lo == 0 && fldp_hi == 0) ? mapped_host(fldp) : nullptr;
    RET(launch_soa2aos(h->fldp, nullptr, h->nf, h->N, h->prec, d ? d : h->stage, h->stream));
    if (!d) RET(copy_aos(h, fldp, fldp_lo, fldp_hi, false));
  }
  CK(cudaStreamSynchronize(h->stream));
  return LAT_OK;
}

int lat_set_scale_factor(lat_t* h, double a, double ap) {
  if (!h) return set_error(LAT_ERR_ARG, "null handle");
  ApiGuard g(h);
  DevScalars s;
  RET(read_scalars(h, &s));
  s.a = a;
  s.ap = ap;
  CK(cudaMemcpyAsync(h->sc, &s, sizeof(DevScalars), cudaMemcpyHostToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return LAT_OK;
}

int lat_get_scale_factor(lat_t* h, double* a, double* ap) {
  if (!h || !a || !ap) return set_error(LAT_ERR_ARG, "null argument");
  ApiGuard g(h);
  DevScalars s;
  RET(read_scalars(h, &s));
  *a = conformal(h) ? s.a : 1.0;
  *ap = conformal(h) ? s.ap : 0.0;
  return LAT_OK;
}

int lat_energies(lat_t* h, double out[LAT_NENERGY]) {
  if (!h || !out) return set_error(LAT_ERR_ARG, "null argument");
  ApiGuard g(h);
  return compute_energies(h, out);
}

int lat_calc_metric(lat_t* h) {
  if (!h) return set_error(LAT_ERR_ARG, "null handle");
  ApiGuard g(h);
  double e[LAT_NENERGY];
  RET(compute_energies(h, e));
  DevScalars s;
  RET(read_scalars(h, &s));
  s.ap = -std::sqrt(s.a * s.a * s.a * s.a * 12.0 * e[LAT_E_RHO]);
  CK(cudaMemcpyAsync(h->sc, &s, sizeof(DevScalars), cudaMemcpyHostToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return LAT_OK;
}

int lat_split(lat_t* h, double dt, int32_t hamind) {
  if (!h) return set_error(LAT_ERR_ARG, "null handle");
  ApiGuard g(h);
  std::vector<Op> ops;
  Emitter em = emitter(h, &ops, h->tglobal);
  RET(em.split(dt, hamind));
  return exec_plain(h, ops);
}

int lat_o2step(lat_t* h, double dt, double w1, double w2) {
  if (!h) return set_error(LAT_ERR_ARG, "null handle");
  ApiGuard g(h);
  std::vector<Op> ops;
  Emitter em = emitter(h, &ops, h->tglobal);
  RET(em.o2step(dt, w1, w2));
  return exec_plain(h, ops);
}

int lat_symp(lat_t* h, int32_t order, double dt, int32_t nsteps) {
  if (!h) return set_error(LAT_ERR_ARG, "null handle");
  ApiGuard g(h);
  return symp_graph(h, order, dt, nsteps, true);
}

int lat_symp_prepare(lat_t* h, int32_t order, double dt, int32_t nsteps) {
  if (!h) return set_error(LAT_ERR_ARG, "null handle");
  ApiGuard g(h);
  return symp_graph(h, order, dt, nsteps, false);
}

int lat_get_time(lat_t* h, double tglobal[3]) {
  if (!h || !tglobal) return set_error(LAT_ERR_ARG, "null argument");
  for (int i = 0; i < 3; ++i) tglobal[i] = h->tglobal[i];
  return LAT_OK;
}

int lat_sync(lat_t* h) {
  if (!h) return set_error(LAT_ERR_ARG, "null handle");
  ApiGuard g(h);
  CK(cudaStreamSynchronize(h->stream));
  unsigned int err = 0;
  CK(cudaMemcpy(&err, &h->sc->err, sizeof(unsigned int), cudaMemcpyDeviceToHost));
  if (err & 2u) return set_error(LAT_ERR_TIMEOUT, "a tensor copy of a streamed pass was not completed in time");
  if (err & 1u) return set_error(LAT_ERR_NAN, "NaN/Inf in a lattice reduction");
  if (h->cl_net) {
    int cerr = 0;
    CK(cudaMemcpy(&cerr, net::net_err(h->cl_net), sizeof(int), cudaMemcpyDeviceToHost));
    if (cerr) return set_error(LAT_ERR_TIMEOUT, "closure convolution: a tensor-core wait gave up");
  }
  return LAT_OK;
}

int lat_laplacian(lat_t* h, int32_t field, double* out) {
  if (h && h->slab) return set_error(LAT_ERR_UNSUPPORTED, "not available on a z-slab handle");
  if (!h || !out) return set_error(LAT_ERR_ARG, "null argument");
  if (field < 0 || field >= h->nf) return set_error(LAT_ERR_ARG, "bad field index");
  ApiGuard g(h);
  RET(ensure_stage(h, (size_t)h->nf * h->N));
  const char* src = (const char*)h->fld[h->cur] + (size_t)field * h->N * h->rsz;
  if (spectral(h)) {
    RET(fft_exec_r2c(h, h->p_r2c1, src, h->Fk));
    KmulArgs k{};
    k.nx = h->nx; k.ny = h->ny; k.nz = h->nz; k.nf = 1;
    k.Fk = h->Fk;
    k.dkx2 = h->dkx * h->dkx; k.dky2 = h->dky * h->dky; k.dkz2 = h->dkz * h->dkz;
    k.invN = 1.0 / (double)h->N;
    k.store_ge2 = 0;
    k.sc = h->sc; k.rb = red(h); k.grid = h->pw_grid; k.block = 256;
    RET(launch_kmul(k, h->prec, h->stream));
    RET(fft_exec_c2r(h, h->p_c2r1, h->Fk, h->lap));
    RET(launch_to_fp64(h->lap, nullptr, h->N, h->prec, h->stage, h->stream));
  } else {
    // stencil Laplacian through a kick of zero size would not expose lap; use
    // the energy-style direct stencil: out = (c0 g + c1 R1 + c2 R2 + c3 R3)/(cc dx^2)
    RET(launch_to_fp64(src, nullptr, h->N, h->prec, h->stage, h->stream));
    const double e = 1.0 / (h->dx * h->dx) / h->c[4];
    double lc[4] = {h->c[0] * e, h->c[1] * e, h->c[2] * e, h->c[3] * e};
    double* tmp = (double*)h->lap;  // FP64 needs N doubles: lap holds nf*N reals >= N doubles only in FP64
    if (h->prec != LAT_FP64) {
      RET(ensure_stage(h, (size_t)std::max(2, h->nf) * h->N));
      tmp = h->stage + h->N;
    }
    RET(launch_fd_laplacian64(h->stage, tmp, h->nx, h->ny, h->nz, lc, h->stream));
    CK(cudaMemcpyAsync(out, tmp, sizeof(double) * h->N, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return LAT_OK;
  }
  CK(cudaMemcpyAsync(out, h->stage, sizeof(double) * h->N, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return LAT_OK;
}

int lat_spectrum_nbins(const lat_t* h, int32_t* ns) {
  if (!h || !ns) return set_error(LAT_ERR_ARG, "null argument");
  int s = (h->nx / 2 + 1) * (h->nx / 2 + 1) + (h->ny / 2 + 1) * (h->ny / 2 + 1) + (h->nz / 2 + 1) * (h->nz / 2 + 1);
  *ns = (int)std::floor(std::sqrt((double)s + 1.0));
  return LAT_OK;
}

int lat_spectrum(lat_t* h, int32_t what, int32_t field, int32_t mode, int32_t nbins, double* S, double* W) {
  if (h && h->slab) return set_error(LAT_ERR_UNSUPPORTED, "not available on a z-slab handle");
  if (!h || !S || !W) return set_error(LAT_ERR_ARG, "null argument");
  if (nbins < 1 || nbins > kMaxBins) return set_error(LAT_ERR_ARG, "nbins out of range");
  if (mode != LAT_SPEC_WEIGHTED && mode != LAT_SPEC_COUNT) return set_error(LAT_ERR_ARG, "bad spectrum mode");
  ApiGuard g(h);
  void* F;
  int sp;
  RET(output_spectrum(h, what, field, 0, &F, &sp));
  std::vector<double> o(3 * nbins);
  RET(run_spectrum(h, F, nullptr, mode, nbins, o.data(), sp));
  for (int l = 0; l < nbins; ++l) {
    W[l] = o[nbins + l];
    S[l] = W[l] != 0.0 ? o[l] / W[l] : o[l];
  }
  return LAT_OK;
}

int lat_crossspec(lat_t* h, int32_t what1, int32_t field1, int32_t what2, int32_t field2, int32_t nbins,
                  double* S_re, double* S_im) {
  if (h && h->slab) return set_error(LAT_ERR_UNSUPPORTED, "not available on a z-slab handle");
  if (!h || !S_re || !S_im) return set_error(LAT_ERR_ARG, "null argument");
  if (nbins < 1 || nbins > kMaxBins) return set_error(LAT_ERR_ARG, "nbins out of range");
  ApiGuard g(h);
  void *F1, *F2;
  int sp;
  RET(output_spectrum(h, what1, field1, 0, &F1, &sp));
  RET(output_spectrum(h, what2, field2, 1, &F2, &sp));
  std::vector<double> o(3 * nbins);
  RET(run_spectrum(h, F1, F2, 2, nbins, o.data(), sp));
  for (int l = 0; l < nbins; ++l) {
    const double w = o[nbins + l];
    S_re[l] = w != 0.0 ? o[l] / w : o[l];
    S_im[l] = w != 0.0 ? o[2 * nbins + l] / w : o[2 * nbins + l];
  }
  return LAT_OK;
}

int lat_gw_spectrum(lat_t* h, int32_t nbins, double* S, double* W) {
  if (h && h->slab) return set_error(LAT_ERR_UNSUPPORTED, "not available on a z-slab handle");
  if (!h || !S || !W) return set_error(LAT_ERR_ARG, "null argument");
  if (!h->cfg.gw) return set_error(LAT_ERR_STATE, "handle has no GW arrays");
  if (nbins < 1 || nbins > kMaxBins) return set_error(LAT_ERR_ARG, "nbins out of range");
  ApiGuard g(h);
  if (!h->Fk6) CK(cudaMalloc(&h->Fk6, (size_t)6 * h->M * h->csz));
  RET(make_plan(h, &h->p_r2c6, &h->have_r2c6, true, 6));
  RET(fft_exec_r2c(h, h->p_r2c6, h->pu, h->Fk6));
  GwSpecArgs a{};
  a.nx = h->nx; a.ny = h->ny; a.nz = h->nz;
  for (int c = 0; c < 6; ++c) a.F[c] = (const char*)h->Fk6 + (size_t)c * h->M * h->csz;
  a.dx = h->dx;
  a.nbins = nbins;
  a.partials = h->spec_part;
  a.out = h->spec_out;
  a.counter = h->spec_counter;
  a.grid = h->spec_grid;
  a.block = 256;
  {
    Timed t(h, LAT_K_OTHER);
    RET(launch_gw_spectrum(a, h->prec, h->stream));
  }
  std::vector<double> o(2 * nbins);
  CK(cudaMemcpyAsync(o.data(), h->spec_out, sizeof(double) * 2 * nbins, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  for (int l = 0; l < nbins; ++l) {
    W[l] = o[nbins + l];
    S[l] = W[l] != 0.0 ? o[l] / W[l] : o[l];
  }
  return LAT_OK;
}

// GW strains and momenta of a z-slab's interior planes, [6][nz_loc][ny][nx].
static int slab_gw_copy(lat_t* h, double* u, double* pu, bool up) {
  const int64_t plane = (int64_t)h->nx * h->ny, Ni = plane * h->nz_loc;
  for (int which = 0; which < 2; ++which) {
    double* host = which == 0 ? u : pu;
    if (!host) continue;
    char* base = static_cast<char*>(which == 0 ? h->u[h->ucur] : h->pu);
    if (up) CK(cudaMemcpyAsync(h->stage, host, sizeof(double) * 6 * Ni, cudaMemcpyHostToDevice, h->stream));
    for (int gc = 0; gc < 6; ++gc) {
      char* dev = base + ((size_t)gc * h->N + plane) * h->rsz;
      if (up) RET(launch_from_fp64(h->stage + gc * Ni, Ni, h->prec, dev, nullptr, h->stream));
      else RET(launch_to_fp64(dev, nullptr, Ni, h->prec, h->stage + gc * Ni, h->stream));
    }
    if (!up) CK(cudaMemcpyAsync(host, h->stage, sizeof(double) * 6 * Ni, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
  }
  return LAT_OK;
}

int lat_gw_download(lat_t* h, double* u, double* pu) {
  if (!h) return set_error(LAT_ERR_ARG, "null handle");
  if (!h->cfg.gw) return set_error(LAT_ERR_STATE, "handle has no GW arrays");
  ApiGuard g(h);
  RET(ensure_stage(h, (size_t)6 * h->N));
  if (h->slab) return slab_gw_copy(h, u, pu, false);
  if (u) {
    RET(launch_to_fp64(h->u[h->ucur], nullptr, 6 * h->N, h->prec, h->stage, h->stream));
    CK(cudaMemcpyAsync(u, h->stage, sizeof(double) * 6 * h->N, cudaMemcpyDeviceToHost, h->stream));
  }
  CK(cudaStreamSynchronize(h->stream));
  if (pu) {
    RET(launch_to_fp64(h->pu, nullptr, 6 * h->N, h->prec, h->stage, h->stream));
    CK(cudaMemcpyAsync(pu, h->stage, sizeof(double) * 6 * h->N, cudaMemcpyDeviceToHost, h->stream));
  }
  CK(cudaStreamSynchronize(h->stream));
  return LAT_OK;
}

int lat_gw_upload(lat_t* h, const double* u, const double* pu) {
  if (!h) return set_error(LAT_ERR_ARG, "null handle");
  if (!h->cfg.gw) return set_error(LAT_ERR_STATE, "handle has no GW arrays");
  ApiGuard g(h);
  RET(clear_nan_flag(h));
  RET(ensure_stage(h, (size_t)6 * h->N));
  if (h->slab) return slab_gw_copy(h, const_cast<double*>(u), const_cast<double*>(pu), true);
  if (u) {
    CK(cudaMemcpyAsync(h->stage, u, sizeof(double) * 6 * h->N, cudaMemcpyHostToDevice, h->stream));
    RET(launch_from_fp64(h->stage, 6 * h->N, h->prec, h->u[h->ucur], nullptr, h->stream));
  }
  if (pu) {
    CK(cudaMemcpyAsync(h->stage, pu, sizeof(double) * 6 * h->N, cudaMemcpyHostToDevice, h->stream));
    RET(launch_from_fp64(h->stage, 6 * h->N, h->prec, h->pu, nullptr, h->stream));
  }
  CK(cudaStreamSynchronize(h->stream));
  return LAT_OK;
}

int lat_init_vacuum(lat_t* h, uint64_t seed, const double* fld0, const double* dfld0, const double* m2eff,
                    double amp, double kcut_frac) {
  if (h && h->slab) return set_error(LAT_ERR_UNSUPPORTED, "not available on a z-slab handle");
  if (!h || !fld0 || !dfld0 || !m2eff) return set_error(LAT_ERR_ARG, "null argument");
  ApiGuard g(h);
  RET(clear_nan_flag(h));
  const double twopi = 6.2831853071795864769252867665590;
  const double V = (h->nx * h->dx) * (h->ny * h->dx) * (h->nz * h->dx);
  const double Nd = (double)h->N;
  double2 *Fa = nullptr, *Fb = nullptr;
  double* tmp = nullptr;
  cufftHandle p;
  CF(cufftCreate(&p));
  int n[3] = {h->nz, h->ny, h->nx};
  size_t ws = 0;
  int rc = LAT_OK;
  do {
    if (cudaMalloc(&Fa, sizeof(double2) * h->M) != cudaSuccess || cudaMalloc(&Fb, sizeof(double2) * h->M) != cudaSuccess ||
        cudaMalloc(&tmp, sizeof(double) * h->N) != cudaSuccess) {
      rc = set_error(LAT_ERR_ALLOC, "vacuum scratch");
      break;
    }
    if (cufftMakePlanMany(p, 3, n, nullptr, 1, 0, nullptr, 1, 0, CUFFT_Z2D, 1, &ws) != CUFFT_SUCCESS ||
        cufftSetStream(p, h->stream) != CUFFT_SUCCESS) {
      rc = set_error(LAT_ERR_CUDA, "vacuum plan");
      break;
    }
    for (int l = 0; l < h->nf && rc == LAT_OK; ++l) {
      VacArgs va{};
      va.nx = h->nx; va.ny = h->ny; va.nz = h->nz;
      va.seed = seed;
      va.field = l;
      va.dkx = h->dkx; va.dky = h->dky; va.dkz = h->dkz;
      va.sig_pref = amp * Nd * Nd / (2.0 * V);
      va.m2 = m2eff[l];
      va.kcut = kcut_frac * (twopi / 2.0) / h->dx;
      va.Fphi = Fa;
      va.Fpi = Fb;
      if ((rc = launch_vacuum_modes(va, h->stream))) break;
      char* fdst = (char*)h->fld[h->cur] + (size_t)l * h->N * h->rsz;
      char* cdst = h->fldc ? (char*)h->fldc + (size_t)l * h->N * h->rsz : nullptr;
      char* pdst = (char*)h->fldp + (size_t)l * h->N * h->rsz;
      if (cufftExecZ2D(p, (cufftDoubleComplex*)Fa, tmp) != CUFFT_SUCCESS) { rc = set_error(LAT_ERR_CUDA, "vacuum z2d"); break; }
      if ((rc = launch_add_scale(tmp, h->N, 1.0 / Nd, fld0[l], h->stream))) break;
      if ((rc = launch_from_fp64(tmp, h->N, h->prec, fdst, cdst, h->stream))) break;
      if (cufftExecZ2D(p, (cufftDoubleComplex*)Fb, tmp) != CUFFT_SUCCESS) { rc = set_error(LAT_ERR_CUDA, "vacuum z2d"); break; }
      if ((rc = launch_add_scale(tmp, h->N, 1.0 / Nd, dfld0[l], h->stream))) break;
      if ((rc = launch_from_fp64(tmp, h->N, h->prec, pdst, nullptr, h->stream))) break;
    }
    if (rc == LAT_OK && cudaStreamSynchronize(h->stream) != cudaSuccess) rc = set_error(LAT_ERR_CUDA, "vacuum sync");
  } while (0);
  cudaStreamSynchronize(h->stream);
  cufftDestroy(p);
  if (Fa) cudaFree(Fa);
  if (Fb) cudaFree(Fb);
  if (tmp) cudaFree(tmp);
  return rc;
}

int lat_init_sample(lat_t* h, uint64_t seed, const double* fld0, const double* dfld0, double m2eff, double mpl) {
  if (h && h->slab) return set_error(LAT_ERR_UNSUPPORTED, "not available on a z-slab handle");
  if (!h || !fld0 || !dfld0 || !(mpl != 0.0)) return set_error(LAT_ERR_ARG, "null or zero argument");
  if (h->nx != h->ny || h->nx != h->nz) return set_error(LAT_ERR_UNSUPPORTED, "sample: cubic lattices");
  ApiGuard g(h);
  RET(clear_nan_flag(h));
  const int n = h->nx, os = 16, nos = n * os * os;
  const double twopi = 6.2831853071795864769252867665590;
  const double dk = twopi / (n * h->dx), dxos = h->dx / os, dkos = dk / (2.0 * os);
  SampleArgs sa{};
  sa.n = n;
  sa.nos = nos;
  sa.dkos = dkos;
  sa.m2 = m2eff;
  sa.kcut = (double)(n / 2 + 1) * dk / 2.0;
  sa.norm = 0.5 / ((double)n * n * n * std::sqrt(twopi * dk * dk * dk) * mpl) * (dkos / dxos);
  sa.M = h->M;
  sa.seed = seed;
  cufftHandle p1 = 0, p3 = 0, p3i = 0;
  bool have1 = false, have3 = false, have3i = false;
  int rc = LAT_OK;
  do {
    if (cudaMalloc(&sa.z, sizeof(double2) * 4 * (size_t)nos) != cudaSuccess ||
        cudaMalloc(&sa.ker, sizeof(double) * nos) != cudaSuccess ||
        cudaMalloc(&sa.f, sizeof(double) * h->N) != cudaSuccess ||
        cudaMalloc(&sa.F, sizeof(double2) * h->M) != cudaSuccess) {
      rc = set_error(LAT_ERR_ALLOC, "sample scratch");
      break;
    }
    int dims[3] = {n, n, n};
    size_t ws = 0;
    bool ok = (have1 = cufftCreate(&p1) == CUFFT_SUCCESS) &&
              cufftMakePlan1d(p1, 4 * nos, CUFFT_Z2Z, 1, &ws) == CUFFT_SUCCESS &&
              cufftSetStream(p1, h->stream) == CUFFT_SUCCESS;
    ok = ok && (have3 = cufftCreate(&p3) == CUFFT_SUCCESS) &&
         cufftMakePlanMany(p3, 3, dims, nullptr, 1, 0, nullptr, 1, 0, CUFFT_D2Z, 1, &ws) == CUFFT_SUCCESS &&
         cufftSetStream(p3, h->stream) == CUFFT_SUCCESS;
    ok = ok && (have3i = cufftCreate(&p3i) == CUFFT_SUCCESS) &&
         cufftMakePlanMany(p3i, 3, dims, nullptr, 1, 0, nullptr, 1, 0, CUFFT_Z2D, 1, &ws) == CUFFT_SUCCESS &&
         cufftSetStream(p3i, h->stream) == CUFFT_SUCCESS;
    if (!ok) {
      rc = set_error(LAT_ERR_CUDA, "sample plans");
      break;
    }
    for (int l = 0; l < h->nf && rc == LAT_OK; ++l) {
      for (int kind = 0; kind < 2 && rc == LAT_OK; ++kind) {
        sa.gamma = kind == 0 ? -0.25 : 0.25;
        sa.stream = 0x5300 + 2 * l + kind;
        if ((rc = launch_sample_steps(0, sa, h->stream))) break;
        if (cufftExecZ2Z(p1, (cufftDoubleComplex*)sa.z, (cufftDoubleComplex*)sa.z, CUFFT_FORWARD) != CUFFT_SUCCESS) {
          rc = set_error(LAT_ERR_CUDA, "sample dst");
          break;
        }
        if ((rc = launch_sample_steps(1, sa, h->stream))) break;
        if ((rc = launch_sample_steps(2, sa, h->stream))) break;
        if (cufftExecD2Z(p3, sa.f, (cufftDoubleComplex*)sa.F) != CUFFT_SUCCESS) {
          rc = set_error(LAT_ERR_CUDA, "sample d2z");
          break;
        }
        if ((rc = launch_sample_steps(3, sa, h->stream))) break;
        if ((rc = launch_sample_steps(4, sa, h->stream))) break;
        if (cufftExecZ2D(p3i, (cufftDoubleComplex*)sa.F, sa.f) != CUFFT_SUCCESS) {
          rc = set_error(LAT_ERR_CUDA, "sample z2d");
          break;
        }
        if ((rc = launch_add_scale(sa.f, h->N, 1.0, kind == 0 ? fld0[l] : dfld0[l], h->stream))) break;
        char* dst = (char*)(kind == 0 ? h->fld[h->cur] : h->fldp) + (size_t)l * h->N * h->rsz;
        char* cdst = (kind == 0 && h->fldc) ? (char*)h->fldc + (size_t)l * h->N * h->rsz : nullptr;
        rc = launch_from_fp64(sa.f, h->N, h->prec, dst, cdst, h->stream);
      }
    }
    if (rc == LAT_OK && cudaStreamSynchronize(h->stream) != cudaSuccess) rc = set_error(LAT_ERR_CUDA, "sample sync");
  } while (0);
  cudaStreamSynchronize(h->stream);
  if (have1) cufftDestroy(p1);
  if (have3) cufftDestroy(p3);
  if (have3i) cufftDestroy(p3i);
  void* bufs[] = {sa.z, sa.ker, sa.f, sa.F};
  for (void* b : bufs)
    if (b) cudaFree(b);
  return rc;
}

int lat_init_bubbles(lat_t* h, int32_t nbub, const double* centres, double radius, double width) {
  if (h && h->slab) return set_error(LAT_ERR_UNSUPPORTED, "not available on a z-slab handle");
  if (!h || (nbub > 0 && !centres) || nbub < 0 || nbub > 64 || !(width > 0)) return set_error(LAT_ERR_ARG, "bad bubble arguments");
  ApiGuard g(h);
  RET(clear_nan_flag(h));
  RET(ensure_stage(h, (size_t)h->nf * h->N + 3 * 64));
  double* cen = h->stage + (size_t)h->nf * h->N;
  if (nbub > 0) CK(cudaMemcpyAsync(cen, centres, sizeof(double) * 3 * nbub, cudaMemcpyHostToDevice, h->stream));
  RET(launch_bubbles(h->stage, h->nx, h->ny, h->nz, h->dx, nbub, cen, radius, width, h->stream));
  RET(launch_from_fp64(h->stage, h->N, h->prec, h->fld[h->cur], h->fldc, h->stream));
  const size_t fb = (size_t)h->N * h->rsz;
  for (int l = 1; l < h->nf; ++l) {
    CK(cudaMemsetAsync((char*)h->fld[h->cur] + l * fb, 0, fb, h->stream));
    if (h->fldc) CK(cudaMemsetAsync((char*)h->fldc + l * fb, 0, fb, h->stream));
  }
  CK(cudaMemsetAsync(h->fldp, 0, h->nf * fb, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return LAT_OK;
}

int lat_init_bubbles_boosted(lat_t* h, int32_t nbub, const int32_t* centres, double r0, double t0,
                             double phi_false, double phi_true) {
  if (h && h->slab) return set_error(LAT_ERR_UNSUPPORTED, "not available on a z-slab handle");
  if (!h || (nbub > 0 && !centres) || nbub < 0 || nbub > 64 || !(r0 >= 0) || !(t0 >= 0))
    return set_error(LAT_ERR_ARG, "bad bubble arguments");
  ApiGuard g(h);
  RET(clear_nan_flag(h));
  RET(ensure_stage(h, (size_t)std::max(h->nf, 2) * h->N + 3 * 64));
  double* phi = h->stage;
  double* pi = h->stage + h->N;
  int* cen = reinterpret_cast<int*>(h->stage + (size_t)std::max(h->nf, 2) * h->N);
  if (nbub > 0) CK(cudaMemcpyAsync(cen, centres, sizeof(int32_t) * 3 * nbub, cudaMemcpyHostToDevice, h->stream));
  RET(launch_bubbles_boosted(phi, pi, h->nx, h->ny, h->nz, h->dx, nbub, cen, r0, t0, phi_false, phi_true,
                             h->stream));
  const size_t fb = (size_t)h->N * h->rsz;
  RET(launch_from_fp64(phi, h->N, h->prec, h->fld[h->cur], h->fldc, h->stream));
  RET(launch_from_fp64(pi, h->N, h->prec, h->fldp, nullptr, h->stream));
  for (int l = 1; l < h->nf; ++l) {
    CK(cudaMemsetAsync((char*)h->fld[h->cur] + l * fb, 0, fb, h->stream));
    if (h->fldc) CK(cudaMemsetAsync((char*)h->fldc + l * fb, 0, fb, h->stream));
    CK(cudaMemsetAsync((char*)h->fldp + l * fb, 0, fb, h->stream));
  }
  CK(cudaStreamSynchronize(h->stream));
  return LAT_OK;
}

int lat_checkpoint_write(lat_t* h, const char* dir, double time, int32_t frame) {
  if (h && h->slab) return set_error(LAT_ERR_UNSUPPORTED, "not available on a z-slab handle");
  if (!h || !dir) return set_error(LAT_ERR_ARG, "null argument");
  std::vector<double> f((size_t)h->nf * h->N), p((size_t)h->nf * h->N);
  RET(lat_download(h, f.data(), 0, 0, p.data(), 0, 0));
  double a, ap;
  RET(lat_get_scale_factor(h, &a, &ap));
  for (int l = 0; l < h->nf; ++l) {
    for (int which = 0; which < 2; ++which) {
      std::string path = std::string(dir) + (which == 0 ? "/fld_" : "/fldp_") + std::to_string(l + 1) + ".raw";
      FILE* fp = fopen(path.c_str(), "wb");
      if (!fp) return set_error(LAT_ERR_IO, "cannot write " + path);
      const std::vector<double>& src = which == 0 ? f : p;
      std::vector<double> one(h->N);
      for (int64_t s = 0; s < h->N; ++s) one[s] = src[s * h->nf + l];
      size_t nw = fwrite(one.data(), sizeof(double), h->N, fp);
      fclose(fp);
      if ((int64_t)nw != h->N) return set_error(LAT_ERR_IO, "short write " + path);
    }
  }
  std::string path = std::string(dir) + "/checkpt.dat";
  FILE* fp = fopen(path.c_str(), "w");
  if (!fp) return set_error(LAT_ERR_IO, "cannot write " + path);
  fprintf(fp, " %.17g %.17g\n %.17g\n %d\n", a, ap, time, frame);
  fclose(fp);
  return LAT_OK;
}

int lat_checkpoint_read(lat_t* h, const char* dir, double* time, int32_t* frame) {
  if (h && h->slab) return set_error(LAT_ERR_UNSUPPORTED, "not available on a z-slab handle");
  if (!h || !dir) return set_error(LAT_ERR_ARG, "null argument");
  std::vector<double> f((size_t)h->nf * h->N), p((size_t)h->nf * h->N);
  for (int l = 0; l < h->nf; ++l) {
    for (int which = 0; which < 2; ++which) {
      std::string path = std::string(dir) + (which == 0 ? "/fld_" : "/fldp_") + std::to_string(l + 1) + ".raw";
      FILE* fp = fopen(path.c_str(), "rb");
      if (!fp) return set_error(LAT_ERR_IO, "cannot read " + path);
      std::vector<double> one(h->N);
      size_t nr = fread(one.data(), sizeof(double), h->N, fp);
      fclose(fp);
      if ((int64_t)nr != h->N) return set_error(LAT_ERR_IO, "short or corrupt file " + path);
      std::vector<double>& dst = which == 0 ? f : p;
      for (int64_t s = 0; s < h->N; ++s) dst[s * h->nf + l] = one[s];
    }
  }
  std::string path = std::string(dir) + "/checkpt.dat";
  FILE* fp = fopen(path.c_str(), "r");
  if (!fp) return set_error(LAT_ERR_IO, "cannot read " + path);
  double a = 0, ap = 0, t = 0;
  int fr = 0;
  int got = fscanf(fp, "%lf %lf %lf %d", &a, &ap, &t, &fr);
  fclose(fp);
  if (got != 4) return set_error(LAT_ERR_IO, "corrupt checkpt.dat header");
  RET(lat_upload(h, f.data(), 0, 0, p.data(), 0, 0));
  RET(lat_set_scale_factor(h, a, ap));
  if (time) *time = t;
  if (frame) *frame = fr;
  return LAT_OK;
}

int lat_timing_enable(lat_t* h, int32_t on) {
  if (!h) return set_error(LAT_ERR_ARG, "null handle");
  h->timing = on != 0;
  return LAT_OK;
}
int lat_timing_read(lat_t* h, int32_t kclass, double* total_ms, int64_t* launches) {
  if (!h || kclass < 0 || kclass >= LAT_NKCLASS) return set_error(LAT_ERR_ARG, "bad timing class");
  ApiGuard g(h);
  RET(harvest(h));
  if (total_ms) *total_ms = h->t_ms[kclass];
  if (launches) *launches = h->t_n[kclass];
  return LAT_OK;
}
int lat_timing_reset(lat_t* h) {
  if (!h) return set_error(LAT_ERR_ARG, "null handle");
  ApiGuard g(h);
  RET(harvest(h));
  for (int i = 0; i < LAT_NKCLASS; ++i) { h->t_ms[i] = 0; h->t_n[i] = 0; }
  return LAT_OK;
}
int lat_mark(lat_t* h, int32_t slot) {
  if (!h || slot < 0 || slot >= 16) return set_error(LAT_ERR_ARG, "bad mark slot");
  ApiGuard g(h);
  if (!h->marks[slot]) CK(cudaEventCreate(&h->marks[slot]));
  CK(cudaEventRecord(h->marks[slot], h->stream));
  return LAT_OK;
}
int lat_mark_elapsed(lat_t* h, int32_t a, int32_t b, double* ms) {
  if (!h || !ms || a < 0 || a >= 16 || b < 0 || b >= 16 || !h->marks[a] || !h->marks[b])
    return set_error(LAT_ERR_ARG, "bad mark slots");
  ApiGuard g(h);
  CK(cudaEventSynchronize(h->marks[b]));
  float f = 0;
  CK(cudaEventElapsedTime(&f, h->marks[a], h->marks[b]));
  *ms = f;
  return LAT_OK;
}
int lat_launch_count(const lat_t* h, int64_t* count) {
  if (!h || !count) return set_error(LAT_ERR_ARG, "null argument");
  *count = h->launches;
  return LAT_OK;
}
int lat_device_ptr(lat_t* h, int32_t what, void** ptr) {
  if (!h || !ptr) return set_error(LAT_ERR_ARG, "null argument");
  switch (what) {
    case 0: *ptr = h->fld[h->cur]; break;
    case 1: *ptr = h->fldp; break;
    case 2: *ptr = h->fldc; break;
    case 3: *ptr = h->sc; break;
    default: return set_error(LAT_ERR_ARG, "bad pointer selector");
  }
  return LAT_OK;
}
int lat_host_alloc(void** ptr, size_t bytes) {
  if (!ptr) return set_error(LAT_ERR_ARG, "null argument");
  cudaError_t e = cudaHostAlloc(ptr, bytes, cudaHostAllocDefault);
  return e == cudaSuccess ? LAT_OK : set_error(LAT_ERR_ALLOC, cudaGetErrorString(e));
}
int lat_host_free(void* ptr) {
  if (ptr) cudaFreeHost(ptr);
  return LAT_OK;
}

int lat_dev_alloc(int32_t device, void** ptr, size_t bytes) {
  if (!ptr) return set_error(LAT_ERR_ARG, "null argument");
  cudaSetDevice(device);
  cudaError_t e = cudaMalloc(ptr, bytes);
  return e == cudaSuccess ? LAT_OK : set_error(LAT_ERR_ALLOC, cudaGetErrorString(e));
}
int lat_dev_free(void* ptr) {
  if (ptr) cudaFree(ptr);
  return LAT_OK;
}
int lat_memcpy(void* dst, const void* src, size_t bytes, int32_t kind) {
  if ((!dst || !src) && bytes) return set_error(LAT_ERR_ARG, "null argument");
  if (kind < 0 || kind > 2) return set_error(LAT_ERR_ARG, "kind: 0 host to device, 1 device to host, 2 device to device");
  const cudaMemcpyKind k[3] = {cudaMemcpyHostToDevice, cudaMemcpyDeviceToHost, cudaMemcpyDeviceToDevice};
  cudaError_t e = cudaMemcpy(dst, src, bytes, k[kind]);
  return e == cudaSuccess ? LAT_OK : cuda_fail(e, "lat_memcpy");
}

int lat_laplacian_3d(int32_t n1, int32_t n2, int32_t n3, double* f, double dk) {
  if (!f || n1 < 2 || n2 < 2 || n3 < 2 || !(dk > 0)) return set_error(LAT_ERR_ARG, "bad laplacian_3d arguments");
  lat_config c{};
  c.nx = n1; c.ny = n2; c.nz = n3; c.nfld = 1;
  c.len = 6.2831853071795864769252867665590 / dk;
  c.laplacian = LAT_LAP_SPECTRAL;
  c.background = LAT_BG_MINKOWSKI;
  c.precision = LAT_FP64;
  c.model = LAT_MODEL_FREE;
  lat_t* h = nullptr;
  RET(lat_create(&h, &c));
  h->dkx = h->dky = h->dkz = dk;  // one dk for every axis, fftw_mod.f90:195
  int st = lat_upload(h, f, 0, 0, nullptr, 0, 0);
  if (st == LAT_OK) st = lat_laplacian(h, 0, f);
  lat_destroy(h);
  return st;
}

int lat_spectrum_3d(int32_t n1, int32_t n2, int32_t n3, const double* f, int32_t mode, int32_t nbins, double* S,
                    double* W) {
  if (!f || n1 < 2 || n2 < 2 || n3 < 2) return set_error(LAT_ERR_ARG, "bad spectrum_3d arguments");
  lat_config c{};
  c.nx = n1; c.ny = n2; c.nz = n3; c.nfld = 1;
  c.len = 1.0;
  c.laplacian = LAT_LAP_SPECTRAL;
  c.background = LAT_BG_MINKOWSKI;
  c.precision = LAT_FP64;
  c.model = LAT_MODEL_FREE;
  lat_t* h = nullptr;
  RET(lat_create(&h, &c));
  int st = lat_upload(h, f, 0, 0, nullptr, 0, 0);
  if (st == LAT_OK) st = lat_spectrum(h, LAT_SPEC_FLD, 0, mode, nbins, S, W);
  lat_destroy(h);
  return st;
}

// ------------------------------------------------------------- autotune
namespace {

std::string tune_key(lat_s* h) {
  cudaDeviceProp prop{};
  cudaGetDeviceProperties(&prop, h->dev);
  char buf[512];
  snprintf(buf, sizeof(buf), "%s|sm%d%d|p%d|lap%d|bg%d|nf%d|gw%d|%dx%dx%d|impl%d", prop.name, prop.major, prop.minor,
           h->prec, h->cfg.laplacian, h->cfg.background, h->nf, h->cfg.gw, h->nx, h->ny, h->nz,
           h->cfg.spectral_impl);
  return buf;
}

bool tune_lookup(const char* path, const std::string& key, int v[5]) {
  if (!path) return false;
  FILE* fp = fopen(path, "r");
  if (!fp) return false;
  char line[1024];
  bool found = false;
  const std::string pat = "\"key\": \"" + key + "\"";
  while (fgets(line, sizeof(line), fp)) {
    if (!strstr(line, pat.c_str())) continue;
    int a, b, c, d, e = 0;
    const char* q = strstr(line, "\"ty\":");
    if (q && sscanf(q, "\"ty\": %d, \"zc\": %d, \"pw_block\": %d, \"pw_bps\": %d, \"sep\": %d", &a, &b, &c, &d,
                    &e) >= 4) {
      v[0] = a; v[1] = b; v[2] = c; v[3] = d; v[4] = e;
      found = true;
    }
  }
  fclose(fp);
  return found;
}

// device time of `reps` executions of one representative pass
int time_pass(lat_s* h, int reps, float* ms) {
  cudaEvent_t a, b;
  CK(cudaEventCreate(&a));
  CK(cudaEventCreate(&b));
  int st = LAT_OK;
  const double hk = 1e-3, hg = 5e-4, hd = 1e-3;
  for (int w = 0; w < 2 && st == LAT_OK; ++w) {  // w = 0 warms up
    cudaEventRecord(a, h->stream);
    for (int r = 0; r < reps && st == LAT_OK; ++r) {
      if (spectral(h) || !conformal(h)) st = exec_kd(h, hk, conformal(h) ? hg : 0.0, hd);
      else st = exec_kick(h, hk);
    }
    cudaEventRecord(b, h->stream);
  }
  if (st == LAT_OK) {
    cudaEventSynchronize(b);
    cudaEventElapsedTime(ms, a, b);
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return st;
}

}  // namespace

int lat_autotune(lat_t* h, const char* cache_path) {
  if (h && h->slab) return set_error(LAT_ERR_UNSUPPORTED, "not available on a z-slab handle");
  if (!h) return set_error(LAT_ERR_ARG, "null handle");
  ApiGuard g(h);
  const std::string key = tune_key(h);
  int v[5] = {0, 0, 0, 0, 0};
  if (tune_lookup(cache_path, key, v)) {
    h->fd_ty = v[0]; h->fd_zc = std::min(v[1], h->nz); h->pw_block = v[2]; h->pw_grid = h->nsm * v[3];
    if (h->sep_ok && h->cfg.spectral_impl == LAT_SPEC_IMPL_AUTO) h->sep = v[4] != 0;
    free_graphs(h);
    return LAT_OK;
  }
  // save the state: candidates run real passes on this lattice
  const size_t fb = (size_t)h->nf * h->N * h->rsz, gb = (size_t)6 * h->N * h->rsz;
  std::vector<void*> saved;
  auto save = [&](void* src, size_t bytes) -> int {
    void* d = nullptr;
    if (!src) { saved.push_back(nullptr); return LAT_OK; }
    CK(cudaMalloc(&d, bytes));
    CK(cudaMemcpyAsync(d, src, bytes, cudaMemcpyDeviceToDevice, h->stream));
    saved.push_back(d);
    return LAT_OK;
  };
  const int cur0 = h->cur, ucur0 = h->ucur;
  void* const c0 = h->fldc;
  void* const c0a = h->fldc_alt;
  void* const p0 = h->fldp;
  void* const p0a = h->fldp_alt;
  RET(save(h->fld[h->cur], fb));
  RET(save(h->fldc, fb));
  RET(save(h->fldp, fb));
  RET(save(h->cfg.gw ? h->u[h->ucur] : nullptr, gb));
  RET(save(h->cfg.gw ? h->pu : nullptr, gb));
  RET(save(h->sc, sizeof(DevScalars)));
  const bool was_timing = h->timing;
  h->timing = false;
  int st = LAT_OK;
  float best = 1e30f;
  int bty = h->fd_ty, bzc = h->fd_zc, bpb = h->pw_block, bbps = h->pw_grid / h->nsm;
  const int reps = h->N >= (1 << 22) ? 3 : 10;
  if (!spectral(h)) {
    for (int ty : {2, 4, 8, 16})
      for (int zc : {2, 4, 8, 16, 32, 64}) {  // short z-chunks: enough blocks on small lattices
        if (st != LAT_OK) break;
        if (zc > h->nz && zc != 8) continue;
        h->fd_ty = ty;
        h->fd_zc = std::min(zc, h->nz);
        float ms = 0;
        st = time_pass(h, reps, &ms);
        if (st == LAT_OK && ms < best) { best = ms; bty = ty; bzc = h->fd_zc; }
      }
    h->fd_ty = bty;
    h->fd_zc = bzc;
  }
  best = 1e30f;
  for (int pb : {128, 256})
    for (int bps : {1, 2, 4, 8}) {
      if (st != LAT_OK) break;
      if ((int64_t)h->nsm * bps > h->red_cap) continue;
      h->pw_block = pb;
      h->pw_grid = h->nsm * bps;
      float ms = 0;
      if (!spectral(h) && !conformal(h)) {  // FD Minkowski: the pointwise drift is the only pointwise pass
        cudaEvent_t a, b;
        cudaEventCreate(&a);
        cudaEventCreate(&b);
        exec_drift(h, 1e-3);
        cudaEventRecord(a, h->stream);
        for (int r = 0; r < reps; ++r) st = exec_drift(h, 1e-3);
        cudaEventRecord(b, h->stream);
        cudaEventSynchronize(b);
        cudaEventElapsedTime(&ms, a, b);
        cudaEventDestroy(a);
        cudaEventDestroy(b);
      } else {
        st = time_pass(h, reps, &ms);
      }
      if (st == LAT_OK && ms < best) { best = ms; bpb = pb; bbps = bps; }
    }
  h->pw_block = bpb;
  h->pw_grid = h->nsm * bbps;
  // spectral Laplacian: cuFFT path against the separable passes, one substep each
  if (st == LAT_OK && h->sep_ok && h->cfg.spectral_impl == LAT_SPEC_IMPL_AUTO) {
    std::vector<Op> ops;
    double tg[3] = {0, 0, 0};
    Emitter em = emitter(h, &ops, tg);
    st = em.symp(2, 1e-3, 2);
    float tms[2] = {0, 0};
    for (int impl = 0; impl < 2 && st == LAT_OK; ++impl) {
      h->sep = impl == 1;
      cudaEvent_t a, b;
      cudaEventCreate(&a);
      cudaEventCreate(&b);
      st = exec_fused(h, ops);  // warm-up
      cudaEventRecord(a, h->stream);
      for (int r = 0; r < reps && st == LAT_OK; ++r) st = exec_fused(h, ops);
      cudaEventRecord(b, h->stream);
      cudaEventSynchronize(b);
      cudaEventElapsedTime(&tms[impl], a, b);
      cudaEventDestroy(a);
      cudaEventDestroy(b);
    }
    h->sep = tms[1] < tms[0];
  }
  h->timing = was_timing;
  // restore
  h->cur = cur0;
  h->ucur = ucur0;
  h->fldc = c0; h->fldc_alt = c0a;
  h->fldp = p0; h->fldp_alt = p0a;
  void* dst[6] = {h->fld[h->cur], h->fldc, h->fldp, h->cfg.gw ? h->u[h->ucur] : nullptr,
                  h->cfg.gw ? h->pu : nullptr, h->sc};
  size_t sz[6] = {fb, fb, fb, gb, gb, sizeof(DevScalars)};
  for (int i = 0; i < 6; ++i)
    if (saved[i]) cudaMemcpyAsync(dst[i], saved[i], sz[i], cudaMemcpyDeviceToDevice, h->stream);
  CK(cudaStreamSynchronize(h->stream));
  for (void* p : saved)
    if (p) cudaFree(p);
  free_graphs(h);
  if (st != LAT_OK) return st;
  if (cache_path) {
    FILE* fp = fopen(cache_path, "a");
    if (fp) {
      fprintf(fp, "{\"key\": \"%s\", \"ty\": %d, \"zc\": %d, \"pw_block\": %d, \"pw_bps\": %d, \"sep\": %d}\n",
              key.c_str(), h->fd_ty, h->fd_zc, h->pw_block, h->pw_grid / h->nsm, h->sep ? 1 : 0);
      fclose(fp);
    }
  }
  return LAT_OK;
}

int lat_closure_attach(lat_t* h, lat_net_t* net, int32_t every, int32_t units) {
  if (h && h->slab) return set_error(LAT_ERR_UNSUPPORTED, "not available on a z-slab handle");
  if (!h) return set_error(LAT_ERR_ARG, "null handle");
  ApiGuard g(h);
  CK(cudaStreamSynchronize(h->stream));
  // cached graphs stay: their key holds the closure state they were captured with
  if (!net) {
    if (h->cl_net) net::net_attach_ref(h->cl_net, -1);
    h->cl_net = nullptr;
    return LAT_OK;
  }
  if (h->nf != 2) return set_error(LAT_ERR_UNSUPPORTED, "the closure network takes two fields");
  if (h->nx % 16 || h->ny % 8) return set_error(LAT_ERR_UNSUPPORTED, "closure lattice: nx % 16 == 0, ny % 8 == 0");
  if (every < 1) return set_error(LAT_ERR_ARG, "every must be >= 1");
  if (units != LAT_UNITS_PROGRAM && units != LAT_UNITS_CONFORMAL) return set_error(LAT_ERR_ARG, "units: 0 or 1");
  if (net::net_device(net) != h->dev) return set_error(LAT_ERR_ARG, "network and lattice on different devices");
  if (!h->cl_stream) {
    CK(cudaStreamCreateWithFlags(&h->cl_stream, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&h->cl_fork, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&h->cl_join, cudaEventDisableTiming));
  }
  if (!h->cl_b.a0) {
    CK(cudaMalloc(&h->cl_b.a0, (size_t)h->N * net::C_IN * 2));
    CK(cudaMalloc(&h->cl_b.a1, (size_t)h->N * net::C_HID * 2));
    CK(cudaMalloc(&h->cl_b.a2, (size_t)h->N * net::C_HID * 2));
    CK(cudaMalloc(&h->cl_b.out, (size_t)h->N * 2 * sizeof(float)));
  }
  if (h->cl_net) net::net_attach_ref(h->cl_net, -1);
  net::net_attach_ref(net, +1);
  h->cl_net = net;
  h->cl_every = every;
  h->cl_units = conformal(h) ? units : LAT_UNITS_PROGRAM;  // a = 1 in Minkowski
  net::out_scale(net, h->cl_tscale);
  return LAT_OK;
}

int lat_coarsen(lat_t* h, int32_t nc, int32_t units, float* out) {
  if (h && h->slab) return set_error(LAT_ERR_UNSUPPORTED, "not available on a z-slab handle");
  if (!h || !out) return set_error(LAT_ERR_ARG, "null argument");
  ApiGuard g(h);
  if (units != LAT_UNITS_PROGRAM && units != LAT_UNITS_CONFORMAL) return set_error(LAT_ERR_ARG, "units: 0 or 1");
  double av = 1.0;  // conformal units: fields times a, momenta over a, Delta times a^3
  if (units == LAT_UNITS_CONFORMAL && conformal(h)) {
    DevScalars scal{};
    RET(read_scalars(h, &scal));
    av = scal.a;
  }
  if (nc < 4 || nc % 2 || nc > h->nx || nc > h->ny || nc > h->nz)
    return set_error(LAT_ERR_ARG, "coarse side: even, at least 4, at most the fine sides");
  if (h->nx % 2) return set_error(LAT_ERR_ARG, "fine nx must be even");
  const int64_t Nc = (int64_t)nc * nc * nc, Mc = (int64_t)(nc / 2 + 1) * nc * nc;
  const int nf = h->nf;
  RET(ensure_stage(h, (size_t)std::max(nf, 2) * h->N));
  if (!h->Fk64) CK(cudaMalloc(&h->Fk64, (size_t)2 * h->M * sizeof(double2)));
  if (h->prec != LAT_FP64 && !h->have_d2z1) {
    CF(cufftCreate(&h->p_d2z1));
    int n[3] = {h->nz, h->ny, h->nx};
    size_t ws = 0;
    CF(cufftMakePlanMany(h->p_d2z1, 3, n, nullptr, 1, 0, nullptr, 1, 0, CUFFT_D2Z, 1, &ws));
    CF(cufftSetStream(h->p_d2z1, h->stream));
    h->have_d2z1 = true;
  }
  double2* Fc = nullptr;
  double *phic = nullptr, *tmp = nullptr;
  cufftHandle pc = 0;
  bool have_pc = false;
  int st = LAT_OK;
  auto fine_fft = [&](const double* in) -> int {  // fine FP64 real -> Fk64
    if (h->prec == LAT_FP64) return fft_exec_r2c(h, h->p_r2c1, in, h->Fk64);
    CF(cufftExecD2Z(h->p_d2z1, const_cast<double*>(in), (cufftDoubleComplex*)h->Fk64));
    return LAT_OK;
  };
  auto filter = [&](const double* in, double* dst) -> int {  // fine real -> coarse real (FP64)
    RET(fine_fft(in));
    RET(launch_truncate((const double2*)h->Fk64, h->nx, h->ny, h->nz, Fc, nc, 1.0 / (double)h->N, h->stream));
    CF(cufftExecZ2D(pc, (cufftDoubleComplex*)Fc, dst));
    return LAT_OK;
  };
  auto body = [&]() -> int {
    CK(cudaMalloc(&Fc, (size_t)Mc * sizeof(double2)));
    CK(cudaMalloc(&phic, (size_t)nf * Nc * sizeof(double)));
    CK(cudaMalloc(&tmp, (size_t)Nc * sizeof(double)));
    CF(cufftPlan3d(&pc, nc, nc, nc, CUFFT_Z2D));
    have_pc = true;
    CF(cufftSetStream(pc, h->stream));
    double* fine = h->stage;
    const size_t fb = (size_t)h->N * h->rsz;
    for (int f = 0; f < nf; ++f) {  // filtered fields (kept in FP64 for Delta)
      const void* comp = h->fldc ? (const char*)h->fldc + f * fb : nullptr;
      RET(launch_to_fp64((const char*)h->fld[h->cur] + f * fb, comp, h->N, h->prec, fine, h->stream));
      RET(filter(fine, phic + f * Nc));
      RET(launch_to_f32(phic + f * Nc, Nc, av, out + (int64_t)f * Nc, h->stream));
    }
    for (int f = 0; f < nf; ++f) {  // filtered momenta
      RET(launch_to_fp64((const char*)h->fldp + f * fb, nullptr, h->N, h->prec, fine, h->stream));
      RET(filter(fine, tmp));
      RET(launch_to_f32(tmp, Nc, 1.0 / av, out + (int64_t)(nf + f) * Nc, h->stream));
    }
    RET(launch_dv_fine(h->fld[h->cur], h->fldc, nf, h->N, model_of(h), h->prec, fine, h->stream));
    for (int f = 0; f < nf; ++f) {  // Delta_f = V'_f(F phi) - F V'_f(phi)
      RET(filter(fine + (size_t)f * h->N, tmp));
      RET(launch_delta(phic, tmp, f, nf, Nc, model_of(h), av * av * av, out + (int64_t)(2 * nf + f) * Nc, h->stream));
    }
    CK(cudaStreamSynchronize(h->stream));
    return LAT_OK;
  };
  st = body();
  cudaStreamSynchronize(h->stream);
  if (have_pc) cufftDestroy(pc);
  if (Fc) cudaFree(Fc);
  if (phic) cudaFree(phic);
  if (tmp) cudaFree(tmp);
  return st;
}

// One Fortran ES22.15 field followed by the 2X of the reference's
// '(30(ES22.15,2X))' records.
static void put_es(FILE* fp, double v) { fprintf(fp, "%22.15E  ", v); }

int lat_write_energy_line(lat_t* h, const char* path, double time) {
  if (!h || !path) return set_error(LAT_ERR_ARG, "null argument");
  double e[LAT_NENERGY];
  RET(lat_energies(h, e));
  ApiGuard g(h);
  FILE* fp = fopen(path, "a");
  if (!fp) return set_error(LAT_ERR_IO, std::string("cannot open ") + path);
  const double a = e[LAT_E_A], ap = e[LAT_E_AP];
  const double cols[11] = {time, a, e[LAT_E_RHO], e[LAT_E_KE], e[LAT_E_PE], e[LAT_E_GE_LAP], e[LAT_E_GRAV],
                           (e[LAT_E_RHO] + e[LAT_E_GRAV]) / e[LAT_E_RHO], -ap * ap / 12.0 / (a * a * a * a),
                           e[LAT_E_MEAN0], e[LAT_E_MEAN1]};
  const int n = h->nf >= 2 ? 11 : 10;
  for (int i = 0; i < n; ++i) put_es(fp, cols[i]);
  fputc('\n', fp);
  const bool ok = fclose(fp) == 0;
  return ok ? LAT_OK : set_error(LAT_ERR_IO, std::string("write failed: ") + path);
}

int lat_write_log_line(lat_t* h, const char* path, double time) {
  if (h && h->slab) return set_error(LAT_ERR_UNSUPPORTED, "not available on a z-slab handle");
  if (!h || !path) return set_error(LAT_ERR_ARG, "null argument");
  ApiGuard g(h);
  if (spectral(h)) return set_error(LAT_ERR_UNSUPPORTED, "LOG.out: finite-difference lattices");
  double e[LAT_NENERGY], ball[3];
  RET(compute_energies(h, e, 45.0, ball));  // ballrad = 5 3^2 (iofile.f90:527)
  const double a = e[LAT_E_A], ap = e[LAT_E_AP];
  const double H = conformal(h) ? -ap / 6.0 / (a * a) : 0.0;
  // get_energy_coeffs (homlat.f90:34-46): ekin (sum pi)^2 + egrad GRAD2 + epot modelv
  const double ekin = 0.5 / std::pow(a, 6), egrad = 0.25 / (a * h->dx) / (a * h->dx) / h->c[4];
  const double rhoball = ekin * ball[0] + egrad * ball[1] + ball[2];
  const double ke = e[LAT_E_KE], pe = e[LAT_E_PE], ge = e[LAT_E_GE_GRAD], gel = e[LAT_E_GE_LAP];
  const double grav = e[LAT_E_GRAV];
  FILE* fp = fopen(path, "a");
  if (!fp) return set_error(LAT_ERR_IO, std::string("cannot open ") + path);
  if (ftell(fp) == 0)
    fputs("# t  a  H  <rho>  rhoball  KE  PE  GE  GE(lap)  -3H^2  H_total\n", fp);
  const double cols[11] = {time, a, H, ke + ge + pe, rhoball, ke, pe, ge, gel, grav, ge + ke + pe + grav};
  for (double v : cols) put_es(fp, v);
  fputc('\n', fp);
  const bool ok = fclose(fp) == 0;
  return ok ? LAT_OK : set_error(LAT_ERR_IO, std::string("write failed: ") + path);
}

int lat_write_spectrum_block(lat_t* h, const char* path) {
  if (h && h->slab) return set_error(LAT_ERR_UNSUPPORTED, "not available on a z-slab handle");
  if (!h || !path) return set_error(LAT_ERR_ARG, "null argument");
  int32_t ns = 0;
  RET(lat_spectrum_nbins(h, &ns));
  std::vector<double> S1(ns), S2(ns), Cr(ns), Ci(ns), W(ns);
  RET(lat_spectrum(h, LAT_SPEC_FLD, 0, LAT_SPEC_WEIGHTED, ns, S1.data(), W.data()));
  RET(lat_spectrum(h, LAT_SPEC_FLDP, 0, LAT_SPEC_WEIGHTED, ns, S2.data(), W.data()));
  RET(lat_crossspec(h, LAT_SPEC_FLDP, 0, LAT_SPEC_FLD, 0, ns, Cr.data(), Ci.data()));
  FILE* fp = fopen(path, "a");
  if (!fp) return set_error(LAT_ERR_IO, std::string("cannot open ") + path);
  const int ncols = 2 * h->nf + 2;  // the reference fills the first four
  for (int i = 0; i < ns; ++i) {
    put_es(fp, i * h->dkx);
    const double v[4] = {S1[i], S2[i], Cr[i], Ci[i]};
    for (int c = 0; c < ncols; ++c) put_es(fp, c < 4 ? v[c] : 0.0);
    fputc('\n', fp);
  }
  fputc('\n', fp);
  const bool ok = fclose(fp) == 0;
  return ok ? LAT_OK : set_error(LAT_ERR_IO, std::string("write failed: ") + path);
}

int lat_write_cube(lat_t* h, int32_t what, int32_t field, int32_t ds, const char* dir, const char* name,
                   int32_t frame, double time) {
  if (h && h->slab) return set_error(LAT_ERR_UNSUPPORTED, "not available on a z-slab handle");
  if (!h || !dir || !name) return set_error(LAT_ERR_ARG, "null argument");
  if (ds < 1 || h->nx % ds || h->ny % ds || h->nz % ds) return set_error(LAT_ERR_ARG, "sides must be multiples of ds");
  if (frame < 0 || frame > 99999) return set_error(LAT_ERR_ARG, "frame: 0..99999");
  ApiGuard g(h);
  const void* src = nullptr;
  RET(src_ptr(h, what, field, &src));
  const void* c = nullptr;
  if (what == LAT_SPEC_FLD && h->prec == LAT_FP32_KAHAN)
    c = (const char*)h->fldc + (size_t)field * h->N * h->rsz;
  const int mx = h->nx / ds, my = h->ny / ds, mz = h->nz / ds;
  const size_t M = (size_t)mx * my * mz;
  RET(ensure_stage(h, M));
  RET(launch_cube(src, c, h->nx, h->ny, h->nz, ds, h->prec, h->stage, h->stream));
  std::vector<double> buf(M);
  CK(cudaMemcpyAsync(buf.data(), h->stage, M * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  char base[64];
  snprintf(base, sizeof(base), "-%05d", (int)frame);
  const std::string raw_name = std::string(name) + base + ".raw";
  const std::string raw = std::string(dir) + "/" + raw_name;
  const std::string bov = std::string(dir) + "/" + name + base + ".bov";
  FILE* fp = fopen(raw.c_str(), "wb");
  if (!fp) return set_error(LAT_ERR_IO, "cannot open " + raw);
  const bool okr = fwrite(buf.data(), sizeof(double), M, fp) == M;
  if (fclose(fp) != 0 || !okr) return set_error(LAT_ERR_IO, "write failed: " + raw);
  fp = fopen(bov.c_str(), "w");
  if (!fp) return set_error(LAT_ERR_IO, "cannot open " + bov);
  fprintf(fp, "TIME:        %25.16E\n", time);
  fprintf(fp, "VARIABLE:    %s\n", name);
  fprintf(fp, "BRICK_ORIGIN:%25.16E%25.16E%25.16E\n", 0.0, 0.0, 0.0);
  fprintf(fp, "BRICK_SIZE:  %25.16E%25.16E%25.16E\n", h->nx * h->dx, h->ny * h->dx, h->nz * h->dx);
  fprintf(fp, "DATA_FILE:   %s\n", raw_name.c_str());
  fprintf(fp, "DATA_SIZE:   %5d%5d%5d\n", mx, my, mz);
  fprintf(fp, "DATA_FORMAT: DOUBLE\n");
  fprintf(fp, "DATA_ENDIAN: LITTLE\n");
  fprintf(fp, "CENTERING:   zonal\n");
  if (fclose(fp) != 0) return set_error(LAT_ERR_IO, "write failed: " + bov);
  return LAT_OK;
}

int lat_sep_streamed(const lat_t* h, int32_t* on) {
  if (!h || !on) return set_error(LAT_ERR_ARG, "null argument");
  *on = h->sep_ok && h->sep_stream ? 1 : 0;
  return LAT_OK;
}

int lat_tuning_get(const lat_t* h, int32_t out[6]) {
  if (!h || !out) return set_error(LAT_ERR_ARG, "null argument");
  out[0] = 32; out[1] = h->fd_ty; out[2] = h->fd_zc; out[3] = h->pw_block; out[4] = h->pw_grid / h->nsm;
  out[5] = h->sep ? LAT_SPEC_IMPL_SEPARABLE : LAT_SPEC_IMPL_CUFFT;
  return LAT_OK;
}

}  // extern "C"

// ------------------------------------------------------------ z-slabs
int lat_slab_create(lat_t** out, const lat_config* gcfg, int32_t z0, int32_t z1) {
  if (!out || !gcfg) return set_error(LAT_ERR_ARG, "null argument");
  *out = nullptr;
  if (gcfg->laplacian == LAT_LAP_SPECTRAL)
    return set_error(LAT_ERR_UNSUPPORTED,
                     "z-slabs need a finite-difference stencil (no distributed transform for the spectral Laplacian)");
  if (z0 < 0 || z1 <= z0 || z1 > gcfg->nz) return set_error(LAT_ERR_ARG, "slab planes outside [0, nz)");
  lat_config c = *gcfg;
  c.nz = (z1 - z0) + 2;  // the interior and one ghost plane on each side
  c.spectral_impl = LAT_SPEC_IMPL_AUTO;
  lat_t* h = nullptr;
  RET(lat_create(&h, &c));
  h->slab = true;
  h->slab_z0 = z0;
  h->slab_nzg = gcfg->nz;
  h->nz_loc = z1 - z0;
  h->slab_nd = (double)gcfg->nx * gcfg->ny * gcfg->nz;
  h->use_graphs = false;
  *out = h;
  return LAT_OK;
}

int lat_slab_set_hooks(lat_t* h, lat_halo_fn halo, lat_sum_fn sum, void* user) {
  if (!h) return set_error(LAT_ERR_ARG, "null handle");
  if (!h->slab) return set_error(LAT_ERR_STATE, "not a z-slab handle");
  h->slab_halo = halo;
  h->slab_sum = sum;
  h->slab_user = user;
  return LAT_OK;
}

int lat_slab_halo_bytes(const lat_t* h, size_t* bytes) {
  if (!h || !bytes) return set_error(LAT_ERR_ARG, "null argument");
  if (!h->slab) return set_error(LAT_ERR_STATE, "not a z-slab handle");
  *bytes = (size_t)(h->nf + (h->cfg.gw ? 6 : 0)) * h->nx * h->ny * h->rsz;
  return LAT_OK;
}

int lat_slab_halo(lat_t* h, int32_t op, void* dev_buf) {
  if (!h || !dev_buf) return set_error(LAT_ERR_ARG, "null argument");
  if (!h->slab) return set_error(LAT_ERR_STATE, "not a z-slab handle");
  if (op < 0 || op > 3) return set_error(LAT_ERR_ARG, "halo op must be 0..3");
  ApiGuard g(h);
  const size_t pb = (size_t)h->nx * h->ny * h->rsz;  // bytes of one plane of one array
  const int pl = op == 0 ? 1 : (op == 1 ? h->nz_loc : (op == 2 ? 0 : h->nz_loc + 1));
  const int narr = h->nf + (h->cfg.gw ? 6 : 0);
  for (int k = 0; k < narr; ++k) {
    char* base = k < h->nf ? static_cast<char*>(h->fld[h->cur]) + (size_t)k * h->N * h->rsz
                           : static_cast<char*>(h->u[h->ucur]) + (size_t)(k - h->nf) * h->N * h->rsz;
    char* dev = base + (size_t)pl * pb;
    char* buf = static_cast<char*>(dev_buf) + (size_t)k * pb;
    if (op < 2) CK(cudaMemcpyAsync(buf, dev, pb, cudaMemcpyDeviceToDevice, h->stream));
    else CK(cudaMemcpyAsync(dev, buf, pb, cudaMemcpyDeviceToDevice, h->stream));
  }
  CK(cudaStreamSynchronize(h->stream));
  return LAT_OK;
}
