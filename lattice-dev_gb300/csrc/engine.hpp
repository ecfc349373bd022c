// engine.hpp -- host-side structures of the GB300 lattice engine and the
// launchers each kernel translation unit exports.
#pragma once
#include <cuda.h>  // CUtensorMap (tensor-memory-access descriptors; encoded through the runtime's driver entry point)
#include <cuda_runtime.h>
#include <cufft.h>

#include <string>
#include <vector>

#include "common.cuh"

namespace lat {

// Set the thread's error message and return `code`.
int set_error(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* where);

// Launch `k` as a programmatic dependent of the previous kernel in stream s
// (programmatic stream serialization): it may start while that kernel
// drains and must order its reads of the predecessor's outputs with
// griddepcontrol.wait.  Stream capture records the dependency as a
// programmatic graph edge.
template <typename K, typename... Args>
cudaError_t launch_pdl(K k, dim3 grid, dim3 block, size_t smem, cudaStream_t s, const Args&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k, args...);
}

// ------------------------------------------------------------ FD passes
// One tiled stencil pass: kick (and optionally drift) of the fields and,
// with gw, of the six u_ij.  Tiles of 32 x ty sites march along z in chunks
// of zc planes; the 3x3 in-plane neighbourhood of each plane is staged in
// shared memory and the three-plane window is kept in registers.
struct FdArgs {
  int nx, ny, nz, nf;
  const void* phi_in;  // fields read by the stencil
  void* phi_out;       // drifted fields (fused pass), nullptr for kick only
  void* phic;          // Kahan compensation (FP32 only), updated in place
  void* pi;            // momenta, updated in place
  const void* u_in;    // GW strain read by the stencil (nullptr: no GW)
  void* u_out;         // drifted strain (fused pass)
  void* pu;            // GW momenta
  double lc[4];        // stencil coefficients c_r / (cc dx^2)
  int seven;           // 7-point stencil (c2 = c3 = 0)
  ModelP model;
  double hk, hd;       // kick and drift sizes
  double kappa, inv2dx;
  int conf;            // conformal kick: a from the scalar block, GE2/PE reductions, ysclp update
  double Nd;
  DevScalars* sc;
  RedBuf rb;
  int ty, zc;          // tile: 32 x ty threads, zc planes per block
  int vec;             // set by the launcher: 16-byte staging of the tile rows (FP32, nx % 32 == 0)
  // planes [zlo, zhi) are updated and reduced (zhi = 0: all nz planes); a
  // z-slab keeps ghost planes 0 and nz-1, filled by the halo exchange
  int zlo, zhi;
  int defer;           // conformal kick: store the lattice sums in sc->red[13..14], leave ysclp to the host
};
int launch_fd(const FdArgs& a, int precision, cudaStream_t s, int* nblocks_out);
int fd_max_blocks(int nx, int ny, int nz, int ty, int zc);

// ------------------------------------------------------ pointwise passes
enum PwMode { PW_KD = 0, PW_DRIFT = 1, PW_KICK = 2 };
struct PwArgs {
  int64_t N;
  int nf;
  void* phi;          // fields, updated in place by drifts
  void* phic;         // Kahan compensation (FP32)
  void* pi;
  const void* lap;    // Laplacian (spectral, already divided by N) for kicks
  void* u;            // GW strain (drift only), nullptr if none
  const void* pu;
  ModelP model;
  double hk, hg, hd;  // kick, gravity half-kick and drift sizes
  double Nd;
  int conf;
  int mode;           // PwMode
  DevScalars* sc;
  RedBuf rb;
  int grid, block;
  // learned-closure force of the kick (fused kick+drift with two fields):
  // pi_f += hk (a^4 or a) corr[s][f] / corr_ts[f], a after the first
  // gravity half-step; null: none
  const float* corr;
  double corr_ts[2];
  int corr_units;  // 0: a^4 (program units), 1: a (conformal units)
  int defer;       // conformal drift: store sum pi^2 and sum V in sc->red[13..14], leave ysclp to the host
};
int launch_pointwise(const PwArgs& a, int precision, cudaStream_t s);

// Separable spectral passes (k_sep.cuh): one launch per axis per kick.
struct SepArgs {
  int nx, ny, nz, nf;
  const void* phi;   // inputs
  const void* phic;
  const void* pi;
  const void* lap;
  void* phi_out;     // outputs: every updated array goes to its second buffer
  void* phic_out;
  void* pi_out;
  void* lap_out;
  const void* twN;  // W_N^j, j < N, of this axis, in the field precision
  double dk2;       // (2 pi / (n dx))^2 of this axis
  ModelP model;
  double hk, hg, hd;
  double Nd;
  int conf;
  int64_t nlines;   // complex lines of this pass
  int nsm;          // SMs of the device (grid of the streamed passes)
  int stream;       // 1: the streamed passes of k_sep_stream.cuh (other buffer roles)
  // streamed passes over pairs of independent one-field runs (ensembles):
  // run 2i is line A and run 2i+1 line B, A and B nx*ny*nz apart, pairs
  // 2*nx*ny*nz apart; nlines = pairs * pair_lines.  Minkowski only.
  int runs;                 // 1: pairs of runs, 0: the two fields of one lattice (pair_lines = nlines)
  int64_t pair_lines;       // lines of one pair along this pass
  float* shift_a;           // [2 * pairs] shift of zs per run: written by pass X, read by pass Z
  float* shift_b;           // [2 * pairs] phi at site 0 of each run: written by pass Z, read by pass X
  int* grid_out;            // host: receives the grid of a streamed pass (or null)
  DevScalars* sc;
  RedBuf rb;
  // streamed passes Y and Z: tensor maps of zs (float, dims {2 nx, ny, nz,
  // pairs}, box {2 LINES, N, 1, 1} for Y and {2 LINES, 1, N, 1} for Z) and of
  // the momenta (dims {nx, ny, nz, 2 lines, pairs}, box {LINES, N, 1, 2, 1}
  // or {LINES, 1, N, 2, 1}); a tile is one TMA load of each
  CUtensorMap tm_zs;
  CUtensorMap tm_pi;
};
// Encode the two tensor maps of a streamed pass along `axis` (1 or 2) with
// `lines` x-columns per tile and line length n.
int encode_stream_tmaps(SepArgs& a, int axis, int lines, int n);
int launch_sep_16(const SepArgs& a, int precision, int axis, cudaStream_t s);
int launch_sep_32(const SepArgs& a, int precision, int axis, cudaStream_t s);
int launch_sep_64(const SepArgs& a, int precision, int axis, cudaStream_t s);
int launch_sep_128(const SepArgs& a, int precision, int axis, cudaStream_t s);
int launch_sep_256(const SepArgs& a, int precision, int axis, cudaStream_t s);
int launch_sep_512(const SepArgs& a, int precision, int axis, cudaStream_t s);
int sep_stream_lines_128(int axis);  // lines per tile of the streamed passes (k_sep_stream.cuh)
int sep_stream_lines_256(int axis);
// streamed passes over pairs of one-field runs (ensembles), lines of n = 64,
// 96, 128, 192 or 256 points (k_sep_<n>.cu)
int launch_sep_runs_64(const SepArgs& a, int axis, cudaStream_t s);
int launch_sep_runs_96(const SepArgs& a, int axis, cudaStream_t s);
int launch_sep_runs_128(const SepArgs& a, int axis, cudaStream_t s);
int launch_sep_runs_192(const SepArgs& a, int axis, cudaStream_t s);
int launch_sep_runs_256(const SepArgs& a, int axis, cudaStream_t s);
int sep_runs_lines_64(int axis);
int sep_runs_lines_96(int axis);
int sep_runs_lines_128(int axis);
int sep_runs_lines_192(int axis);
int sep_runs_lines_256(int axis);
// lines per tile of the pass along `axis` for lines of n points; 0: n not supported
inline int sep_runs_lines(int n, int axis) {
  switch (n) {
    case 64: return sep_runs_lines_64(axis);
    case 96: return sep_runs_lines_96(axis);
    case 128: return sep_runs_lines_128(axis);
    case 192: return sep_runs_lines_192(axis);
    case 256: return sep_runs_lines_256(axis);
    default: return 0;
  }
}
inline int launch_sep_runs(const SepArgs& a, int n, int axis, cudaStream_t s) {
  switch (n) {
    case 64: return launch_sep_runs_64(a, axis, s);
    case 96: return launch_sep_runs_96(a, axis, s);
    case 128: return launch_sep_runs_128(a, axis, s);
    case 192: return launch_sep_runs_192(a, axis, s);
    case 256: return launch_sep_runs_256(a, axis, s);
    default: return set_error(LAT_ERR_UNSUPPORTED, "streamed separable passes: line length");
  }
}
// A streamed kick's weights (valid = 0: no kick follows in this call).
struct KickW {
  double hk, hg, hd;
  int valid;
};
// sum pi^2 into sc->ke_cur; with phi (two FP32 fields of nsite sites) the
// fields' means into sc->mean; with first.valid the first kick's coefficients
// into sc->co
int launch_pi2_sum(const void* pi, int64_t n, DevScalars* sc, RedBuf rb, int grid, cudaStream_t s,
                   KickW first = KickW{0.0, 0.0, 0.0, 0}, double Nd = 1.0, const void* phi = nullptr,
                   int64_t nsite = 0);
// Partials of the streamed passes of one kick in the reduction buffer: pass X
// [grid][pe, GEx, sum phi_A, sum phi_B] at SEP_PART_X, pass Y [grid][GEy],
// pass Z [grid][GEz, sum pi^2]; completed after pass Z by launch_sep_finalize.
constexpr int SEP_PART_X = 0, SEP_PART_Y = 8192, SEP_PART_Z = 12288;
struct SepFinArgs {
  DevScalars* sc;
  const double* part;  // the reduction buffer
  int gx, gy, gz;      // blocks of the three passes
  double hk, hg, hd;   // the kick, its grav-kinetic halves and the drift of pass X
  double Nd;
  int conf;
  KickW next;          // the next kick of the call, whose coefficients the finalize leaves in sc->co
};
int launch_sep_finalize(const SepFinArgs& f, cudaStream_t s);
int sep_columns_16(int precision, int nf);
int sep_columns_32(int precision, int nf);
int sep_columns_64(int precision, int nf);
int sep_columns_128(int precision, int nf);
int sep_columns_256(int precision, int nf);
int sep_columns_512(int precision, int nf);

// k-space multiply F *= -k^2/N with the Parseval sum of k^2|F|^2 (Hermitian
// weights) into sc->ge2 when store_ge2 is set.
struct KmulArgs {
  int nx, ny, nz, nf;
  void* Fk;
  double dkx2, dky2, dkz2, invN;
  int store_ge2;
  DevScalars* sc;
  RedBuf rb;
  int grid, block;
};
int launch_kmul(const KmulArgs& a, int precision, cudaStream_t s);
// a -= h * ap / 6 on the device (Hamiltonian_grav_kinetic)
int launch_grav(DevScalars* sc, double h, cudaStream_t s);
// New state in the handle: clear the NaN flag; non-finite carried shifts and
// sums of the previous state become 0 (any finite shift is exact).
int launch_state_reset(DevScalars* sc, cudaStream_t s);

// ------------------------------------------------------- output kernels
// fstride: elements between the fields of the SoA arrays (default N)
int launch_aos2soa(const double* aos, int nf, int64_t N, int precision, void* hi, void* c,
                   cudaStream_t s, int64_t fstride = 0);
int launch_soa2aos(const void* hi, const void* c, int nf, int64_t N, int precision, double* aos,
                   cudaStream_t s, int64_t fstride = 0);
int launch_to_fp64(const void* hi, const void* c, int64_t n, int precision, double* out, cudaStream_t s);
int launch_cube(const void* hi, const void* c, int nx, int ny, int nz, int ds, int precision, double* out,
                cudaStream_t s);
int launch_from_fp64(const double* in, int64_t n, int precision, void* hi, void* c, cudaStream_t s);

struct SpecArgs {
  int nx, ny, nz;
  const void* F1;  // half spectrum [z][y][nx/2+1]
  const void* F2;  // second spectrum for the cross spectrum (nullptr otherwise)
  int mode;        // LAT_SPEC_WEIGHTED / LAT_SPEC_COUNT / 2 = cross (weighted)
  int nbins;
  double* partials;   // [grid][3*nbins]
  double* out;        // [3*nbins]: S (or S_re), W, S_im
  unsigned int* counter;
  int grid, block;
};
int launch_spectrum(const SpecArgs& a, int precision, cudaStream_t s);

struct GwSpecArgs {
  int nx, ny, nz;
  const void* F[6];
  double dx;
  int nbins;
  double* partials;
  double* out;  // [2*nbins]
  unsigned int* counter;
  int grid, block;
};
int launch_gw_spectrum(const GwSpecArgs& a, int precision, cudaStream_t s);

// Energies: raw lattice sums into sc->red:
// [0] sum pi^2, [1] sum V, [2] sum phi_1, [3] sum phi_2, [4] -sum phi L phi (FD),
// [5] sum STENCIL(c,GRAD2) (FD), [6] sum pu^2, [7] -sum u L u (GW, weighted)
struct EnergyArgs {
  int nx, ny, nz, nf;
  const void* phi;
  const void* phic;
  const void* pi;
  const void* u;
  const void* pu;
  int fd;  // FD sums [4],[5],[7]
  double c[4];  // raw stencil coefficients c0..c3
  // FD only, ball_r2 > 0: over the sites with |(x, y, z) + 1 - n/2|^2 dx^2 <
  // ball_r2 (LOG.out's rhoball), sum (sum_f pi_f)^2, the stencil's gradient
  // squared and V into red[9], red[10], red[11]
  double ball_r2, dx;
  ModelP model;
  DevScalars* sc;
  RedBuf rb;
  int grid, block;
  int64_t t_lo, t_hi;  // sites [t_lo, t_hi) are summed (t_hi = 0: all); a z-slab sums its interior planes
};
int launch_energy(const EnergyArgs& a, int precision, cudaStream_t s);
// sum over the half spectrum of w k^2 |F|^2 (Parseval) into sc->red[slot]
int launch_parseval(const void* Fk, int nx, int ny, int nz, int nf, double dkx2, double dky2,
                    double dkz2, DevScalars* sc, int slot, RedBuf rb, int grid, int precision,
                    cudaStream_t s);

struct VacArgs {
  int nx, ny, nz;
  uint64_t seed;
  int field;
  double dkx, dky, dkz, sig_pref;  // sig = sqrt(sig_pref / w)
  double m2, kcut;
  double2* Fphi;
  double2* Fpi;
};
int launch_vacuum_modes(const VacArgs& a, cudaStream_t s);
int launch_fd_laplacian64(const double* in, double* out, int nx, int ny, int nz, const double* lc, cudaStream_t s);
int launch_add_scale(double* f, int64_t n, double scale, double offset, cudaStream_t s);
// the reference's sample() IC, step by step (k_out.cu): 0 DST input, 1 DST
// output (after the host's 4 nos FFT of z), 2 radial kernel on the lattice,
// 3 noise (after the r2c of f into F), 4 Hermitian kx = 0, n/2 planes
struct SampleArgs {
  int n, nos;
  double dkos, m2, gamma, kcut, norm;
  double2* z;   // 4 nos
  double* ker;  // nos
  double* f;    // n^3
  double2* F;   // (n/2 + 1) n^2
  int64_t M;
  uint64_t seed;
  int stream;
};
int launch_sample_steps(int step, const SampleArgs& a, cudaStream_t s);
int launch_bubbles(double* phi, int nx, int ny, int nz, double dx, int nbub, const double* centres_dev,
                   double radius, double width, cudaStream_t s);
int launch_bubbles_boosted(double* phi, double* pi, int nx, int ny, int nz, double dx, int nbub, const int* cen,
                           double r0, double t0, double pf, double pt, cudaStream_t s);

// ------------------------------------------- coarsening (k_coarse.cu)
int launch_truncate(const double2* Ff, int fnx, int fny, int fnz, double2* Fc, int nc, double scale, cudaStream_t s);
int launch_dv_fine(const void* fld, const void* c, int nf, int64_t N, const ModelP& m, int precision, double* out,
                   cudaStream_t s);
int launch_delta(const double* phic, const double* filt, int f, int nf, int64_t Nc, const ModelP& m, double scale,
                 float* out, cudaStream_t s);
int launch_to_f32(const double* in, int64_t n, double scale, float* out, cudaStream_t s);

// bookkeeping of launches for the kernel-launch census
extern thread_local int64_t* g_launch_counter;

}  // namespace lat
