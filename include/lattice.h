/*
 * lattice.h -- C ABI of the GB300 lattice engine.
 *
 * The engine evolves interacting scalar fields on a periodic 3D lattice with
 * the symplectic kick-drift (leapfrog / Yoshida) scheme of the Fortran lattice
 * codes, on one sm_103a GPU.  Every entry point below replaces one Fortran
 * module procedure of the reference; the replaced routine is cited beside it
 * (paths are relative to the reference project root).  A Fortran driver binds
 * these through iso_c_binding; Python binds them through ctypes.
 *
 * Conventions (all entry points):
 *  - return an int status (LAT_OK == 0); nothing aborts the process;
 *    lat_last_error() gives a one-line message for the calling thread;
 *  - LAT_ERR_NAN: a lattice reduction met NaN/Inf; lat_sync, lat_energies
 *    and the calls that read the scalar block report it until a call that
 *    replaces the fields (lat_upload, lat_gw_upload, lat_init_*,
 *    lat_checkpoint_read) clears it;
 *  - a handle owns its device memory and one CUDA stream; handles are not
 *    thread-safe, distinct handles may be used from distinct threads;
 *  - the caller owns every host array; host field arrays use the Fortran
 *    layout fld(nfld, i, j, k) with the field index fastest and optional
 *    ghost padding (lo/hi sites per side), as in the reference drivers;
 *  - fields stay resident in HBM between calls; copies happen only in
 *    upload / download / output calls.
 */
#ifndef LATTICE_GB300_H
#define LATTICE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
enum lat_status {
  LAT_OK = 0,
  LAT_ERR_ARG = 1,         /* bad argument / configuration                 */
  LAT_ERR_CUDA = 2,        /* CUDA runtime or cuFFT error                  */
  LAT_ERR_TIMEOUT = 3,     /* a bounded device wait gave up                */
  LAT_ERR_NAN = 4,         /* NaN/Inf in an FP64 reduction                 */
  LAT_ERR_ALLOC = 5,       /* device or host allocation failed             */
  LAT_ERR_STATE = 6,       /* call not valid in the handle's state         */
  LAT_ERR_IO = 7,          /* checkpoint file error                        */
  LAT_ERR_UNSUPPORTED = 8  /* valid request the engine does not implement   */
};

/* ---------------------------------------------------------- configuration */
enum lat_laplacian {
  LAT_LAP_SPECTRAL = 1,  /* FFT Laplacian, Pseudospec/openmp_dev/fftw_mod.f90:177-207 */
  LAT_LAP_FD7 = 7,       /* 7-point stencil, Discrete/Bubble-Collisions/params.f90:116 */
  LAT_LAP_FD27 = 27      /* 27-point stencil, Discrete/Bubble-Collisions/params.f90:119, macros.h:31-44 */
};

enum lat_background {
  LAT_BG_MINKOWSKI = 0,  /* Pseudospec/openmp_dev/hamiltonian_minkowski.f90 */
  LAT_BG_CONFORMAL = 1   /* Pseudospec/openmp_dev/hamiltonian_conformal.f90 (self-consistent a) */
};

enum lat_precision {
  LAT_FP64 = 0,          /* plain FP64 fields (the reference's -r8)        */
  LAT_FP32_KAHAN = 1     /* FP32 fields, Kahan-compensated drift, FP64 reductions */
};

/* Order of the Hamiltonian pieces inside symp_o2step.
 *  PSEUDOSPEC: 1 = fields kinetic (drift), 2 = gravity kinetic (conformal
 *    only), last = gradient+potential (kick);
 *    Pseudospec/openmp_dev/hamiltonian_conformal.f90:50-81.
 *  DEFROST: 1 = metric kinetic, 2 = fields kinetic, 3 = gradient+potential;
 *    Discrete/Bubble-Collisions/evolve.f90:98-113,225-240. */
enum lat_split_order { LAT_SPLIT_PSEUDOSPEC = 0, LAT_SPLIT_DEFROST = 1 };

enum lat_model {
  LAT_MODEL_PHI4 = 0,        /* V = lam/4 phi^4 (params[0]=lam); hamiltonian_minkowski.f90:161-186 */
  LAT_MODEL_PHI4_G2 = 1,     /* V = lam/4 phi^4 + g2/2 phi^2 chi^2 (params: lam, g2), nfld = 2;
                                Pseudospec/mpi_dev/hamiltonian_conformal_rksplit.f90:220-237 */
  LAT_MODEL_DOUBLE_WELL = 2, /* V = (phi^2-1)^2/4 - del (phi+1) (params[0]=del);
                                Discrete/Bubble-Collisions/model.f90:96-165 */
  LAT_MODEL_FREE = 3         /* V = sum_f m2/2 phi_f^2 (params[0]=m2), known-answer model */
};

typedef struct lat_config {
  int32_t nx, ny, nz;        /* lattice sites per side (x fastest)          */
  int32_t nfld;              /* number of real scalar fields                */
  double len;                /* box side along x; dx = len/nx, dk = 2 pi/(n dx) */
  int32_t laplacian;         /* enum lat_laplacian                          */
  int32_t background;        /* enum lat_background                         */
  int32_t precision;         /* enum lat_precision                          */
  int32_t split_order;       /* enum lat_split_order                        */
  int32_t model;             /* enum lat_model                              */
  int32_t gw;                /* 1: evolve the six u_ij and pi_ij (FD, Minkowski) */
  double model_params[4];
  double stencil[5];         /* (c0,c1,c2,c3,cc); all zero = default of the chosen stencil */
  double gw_coupling;        /* kappa in pi_ij' = lap u_ij + kappa d_i phi d_j phi */
  int32_t device;            /* CUDA ordinal                                */
  int32_t spectral_impl;     /* enum lat_spectral_impl                      */
  int32_t reserved[6];
} lat_config;

/* How a spectral kick computes its Laplacian.  CUFFT: 3D R2C, -k^2/N multiply
 * and C2R (any size).  SEPARABLE: three passes of in-register 1D transforms,
 * one per axis (sides 16..512, powers of two), which also transform the FP32
 * field with its Kahan compensation.  AUTO: cuFFT until lat_autotune times
 * both on the handle's lattice and keeps the faster. */
enum lat_spectral_impl { LAT_SPEC_IMPL_AUTO = 0, LAT_SPEC_IMPL_CUFFT = 1, LAT_SPEC_IMPL_SEPARABLE = 2 };

typedef struct lat_s lat_t;

/* ---------------------------------------------------------------- errors */
const char* lat_last_error(void);
const char* lat_version(void);

/* ---------------------------------------------------------------- handle */
/* Allocates fields, FFT plans and scratch.  Replaces the module-global
 * arrays and plans of Pseudospec/openmp_dev/hamiltonian_conformal.f90:22-38
 * and initialize_arrays, evolve_spectral.f90:107-127. */
int lat_create(lat_t** out, const lat_config* cfg);
int lat_destroy(lat_t* h);
int lat_get_config(const lat_t* h, lat_config* cfg);

/* Host <-> device copies of the state in the Fortran layout
 * fld(nfld, 1-lo : n+hi, ...) (ghost sites are ignored on upload and left
 * untouched on download).  Pseudospec: fld lo=hi=1, fldp lo=hi=0
 * (hamiltonian_conformal.f90:22-23); DEFROST: lo=2, hi=3
 * (Discrete/Bubble-Collisions/latpar.f90:78-80). */
int lat_upload(lat_t* h, const double* fld, int32_t fld_lo, int32_t fld_hi,
               const double* fldp, int32_t fldp_lo, int32_t fldp_hi);
int lat_download(lat_t* h, double* fld, int32_t fld_lo, int32_t fld_hi,
                 double* fldp, int32_t fldp_lo, int32_t fldp_hi);

/* Scale factor yscl and its conjugate momentum ysclp (conformal only).
 * get_scale_factor / get_hubble, hamiltonian_conformal.f90:242-250. */
int lat_set_scale_factor(lat_t* h, double a, double ap);
int lat_get_scale_factor(lat_t* h, double* a, double* ap);
/* Friedmann constraint: ysclp = -sqrt(12 a^4 rho). calc_metric,
 * hamiltonian_conformal.f90:263-304. */
int lat_calc_metric(lat_t* h);

/* ------------------------------------------------------------ integrator */
/* symp2/4/6/8 (order 2,4,6,8), Pseudospec/openmp_dev/evolve_spectral.f90:129-227
 * and Discrete/Bubble-Collisions/evolve.f90:118-223.  The whole call runs
 * asynchronously on the handle's stream without host synchronisation. */
int lat_symp(lat_t* h, int32_t order, double dt, int32_t nsteps);
/* Builds and caches the CUDA graph that lat_symp(h, order, dt, nsteps) would
 * replay from the handle's current buffers, without running it (no
 * reference counterpart: it moves graph capture out of a timed call). */
int lat_symp_prepare(lat_t* h, int32_t order, double dt, int32_t nsteps);
/* symp_o2step(dt,w1,w2), hamiltonian_conformal.f90:50-64. */
int lat_o2step(lat_t* h, double dt, double w1, double w2);
/* Hamiltonian_Split(dt, hamind), hamiltonian_conformal.f90:66-81 and
 * Discrete/Bubble-Collisions/evolve.f90:225-240. */
int lat_split(lat_t* h, double dt, int32_t hamind);
/* Substep clocks tglobal(1:3), Discrete/Bubble-Collisions/evolve.f90:39. */
int lat_get_time(lat_t* h, double tglobal[3]);
/* Blocks until the handle's stream is idle; reports device-side errors. */
int lat_sync(lat_t* h);

/* -------------------------------------------------------------- Laplacian */
/* Laplacian of field `field` (0-based) with the configured operator, written
 * to out(nx,ny,nz).  laplacian_3d, Pseudospec/openmp_dev/fftw_mod.f90:177-207;
 * FD: STENCIL(c,LAPLACE)/(cc dx^2), Discrete/Bubble-Collisions/evolve.f90:271-281. */
int lat_laplacian(lat_t* h, int32_t field, double* out);
/* Stand-alone laplacian_3d(n1,n2,n3,f,Fk,dk,planf,planb): f(n1,n2,n3) is
 * replaced by its spectral Laplacian, FP64 (fftw_mod.f90:177-207). */
int lat_laplacian_3d(int32_t n1, int32_t n2, int32_t n3, double* f, double dk);

/* ------------------------------------------------------------- energies */
enum lat_energy_index {
  LAT_E_KE = 0,        /* 1/2 <pi^2> / a^6                       */
  LAT_E_GE_LAP = 1,    /* -1/2 <phi lap phi> / a^2               */
  LAT_E_GE_GRAD = 2,   /* 1/2 <(grad phi)^2> / a^2 (stencil form) */
  LAT_E_PE = 3,        /* <V>                                     */
  LAT_E_RHO = 4,       /* KE + GE_LAP + PE                        */
  LAT_E_GRAV = 5,      /* -3 H^2, H = -ysclp/(6 a^2)              */
  LAT_E_RESIDUAL = 6,  /* (rho + grav)/rho                        */
  LAT_E_A = 7,
  LAT_E_AP = 8,
  LAT_E_MEAN0 = 9,     /* <phi_1>                                 */
  LAT_E_MEAN1 = 10,    /* <phi_2> (0 for one field)               */
  LAT_E_GW = 11,       /* 1/2 <pi_ij pi_ij> + 1/2 <grad u_ij . grad u_ij> (gw only) */
  LAT_NENERGY = 12
};
/* dump_rho, Pseudospec/openmp_dev/evolve_spectral.f90:305-415; homlat
 * grad_en / grad_en_wlap / pot_en / kinetic_en,
 * Discrete/Bubble-Collisions/homlat.f90:65-188. */
int lat_energies(lat_t* h, double out[LAT_NENERGY]);

/* --------------------------------------------------------------- spectra */
enum lat_spec_what { LAT_SPEC_FLD = 0, LAT_SPEC_FLDP = 1 };
enum lat_spec_mode {
  LAT_SPEC_WEIGHTED = 0,  /* two-bin smooth weights, spectrum_3d, Pseudospec/openmp_dev/analysis_spec.f90:59-102 */
  LAT_SPEC_COUNT = 1      /* floor(|n|)+1 with integer counts, spectrum_bin, Discrete/Bubble-Collisions/analysis.f90:193-223 */
};
/* Number of bins of spectrum_3d: floor(sqrt((nx/2+1)^2+(ny/2+1)^2+(nz/2+1)^2+1)),
 * init_spectrum_3d, analysis_spec.f90:48-57. */
int lat_spectrum_nbins(const lat_t* h, int32_t* ns);
/* S(l) = sum_k c |F_k|^2 / W(l) with the unnormalised forward DFT F_k of
 * the chosen array; W is the weight sum (WEIGHTED) or the integer mode count
 * (COUNT, stored exactly in the doubles).  Bins beyond ns come back zero. */
int lat_spectrum(lat_t* h, int32_t what, int32_t field, int32_t mode,
                 int32_t nbins, double* S, double* W);
/* crossspec_3d(Fk1,Fk2,S_real,S_imag), analysis_spec.f90:145-178. */
int lat_crossspec(lat_t* h, int32_t what1, int32_t field1, int32_t what2,
                  int32_t field2, int32_t nbins, double* S_re, double* S_im);
/* Stand-alone spectrum_3d(S,f,Fk,plan) of a host array f(n1,n2,n3). */
int lat_spectrum_3d(int32_t n1, int32_t n2, int32_t n3, const double* f,
                    int32_t mode, int32_t nbins, double* S, double* W);
/* Binning of a half spectrum already on the device, allocating nothing.
 * No counterpart in the reference: it serves callers that cannot call
 * cudaMalloc -- a driver that has given the whole device to its own fixed
 * memory pool, or a code that must not allocate once its time loop runs.
 * Fk_dev: half spectrum [nz][ny][nx/2+1] of complex FP64 (precision
 * LAT_FP64) or FP32 (LAT_FP32_KAHAN), as written by lat_spectrum's R2C;
 * out_dev: 2*nbins doubles on the device, S(l) = sum c|F|^2 / W(l) then W(l);
 * mode as lat_spectrum; stream: a cudaStream_t or NULL for the default stream.
 * Scratch is a fixed 1 MiB static device array that every GPU loading this
 * library keeps until exit; nbins above 512 is rejected with LAT_ERR_ARG.
 * All calls share that scratch: calls that overlap on the GPU race, so order
 * them.  The first call on a device looks up the scratch's device address
 * (with that device current) and keeps it for the life of the process; make
 * it before any stream capture.  A device reset (cudaDeviceReset, or a
 * destroyed and recreated primary context) after that first call is not
 * supported: the kept address would no longer be valid. */
int lat_spectrum_noalloc(const void* Fk_dev, int32_t nx, int32_t ny, int32_t nz,
                         int32_t precision, int32_t mode, int32_t nbins,
                         double* out_dev, void* stream);

/* ---------------------------------------------------- gravitational waves */
/* TT-projected GW spectrum: sum over modes of sum_ij |Lambda_ij,lm pi_lm(k)|^2
 * per integer shell (spectrum_bin binning), divided by the count W.
 * Storage hij/pi_hij, grav-waves/data-gw.f90:14-40; drift h += pi dt,
 * grav-waves/evolve-gw.f90:38-44; the projector is the empty stub of
 * grav-waves/gw-projectors.f90:13-26. */
int lat_gw_spectrum(lat_t* h, int32_t nbins, double* S, double* W);
/* u_ij / pi_ij host copies, component order 11,22,33,12,13,23, each (nx,ny,nz). */
int lat_gw_download(lat_t* h, double* u, double* pu);
int lat_gw_upload(lat_t* h, const double* u, const double* pu);

/* ---------------------------------------------------- initial conditions */
/* Vacuum fluctuations drawn mode by mode in k space with a counter-based
 * generator keyed by (seed, field, mode) so that CPU and GPU draw identical
 * fields: <|F_k|^2> = amp N^2 / (2 V w_k), w_k = sqrt(k^2 + m2eff[f]),
 * pi_k = -i w_k F_k (a wave travelling along +k; the Hermitian partner of a
 * drawn mode inside the kx = 0 and kx = nx/2 planes carries +i w_k F_k and a
 * self-conjugate mode none), |k| > kcut_frac * pi/dx and k = 0 zeroed; then
 * fld = fld0[f] + IDFT(F)/N, fldp = dfld0[f] + IDFT(pi_k)/N.  Replaces
 * init_fields/sample, Pseudospec/openmp_dev/evolve_spectral.f90:262-303,421-506
 * (whose draw depends on the compiler's random_number). */
int lat_init_vacuum(lat_t* h, uint64_t seed, const double* fld0,
                    const double* dfld0, const double* m2eff, double amp,
                    double kcut_frac);
/* The reference's own generator, sample(gamma, m2eff) of
 * Pseudospec/openmp_dev/evolve_spectral.f90:421-506 as init_fields calls it
 * (:294-299): per field f, fld = fld0[f] + sample(-1/4, m2eff) and
 * fldp = dfld0[f] + sample(+1/4, m2eff), independent noise.  sample builds
 * the radial profile k (k^2 + m2eff)^gamma exp(-(k/kcut)^2) (kcut = (n/2+1)
 * dk/2) on an oversampled grid (16^2 points per lattice site along a side),
 * takes its DST-II (FFTW's RODFT10), scales it by norm/k with
 * norm = 0.5 / (n^3 sqrt(2 pi dk^3) mpl) (dkos/dxos), interpolates it onto
 * every site's distance from the grid centre, multiplies each half-spectrum
 * mode of its transform by Box-Muller noise sqrt(-2 ln a) e^{2 pi i p} and
 * transforms back (unnormalised).  The noise is the counter-based draw of
 * lat_init_vacuum keyed by (seed, 0x5300 + 2 f + {0 field, 1 momentum},
 * mode) in place of the compiler's random_number, and the kx = 0 and
 * kx = nx/2 planes are projected onto their Hermitian part before the
 * inverse transform (a c2r of non-Hermitian input is FFT-library defined).
 * Cubic lattices (LAT_ERR_UNSUPPORTED otherwise); mpl is the reference's
 * mpl parameter (1e7/3 in hamiltonian_minkowski.f90:9). */
int lat_init_sample(lat_t* h, uint64_t seed, const double* fld0,
                    const double* dfld0, double m2eff, double mpl);
/* Thin-wall bubbles phi = -1 + sum_b [1 - tanh((r_b - R)/width)], zero momentum;
 * centres in lattice units of length (x,y,z per bubble).  Replaces
 * init_fields/initbubble, Discrete/Bubble-Collisions/ic_bubble.f90:17-123. */
int lat_init_bubbles(lat_t* h, int32_t nbub, const double* centres,
                     double radius, double width);
/* Expanding-wall bubbles exactly as init_fields / initbubble build them
 * (Discrete/Bubble-Collisions/ic_bubble.f90:17-77 with the profile and
 * derivative of init_cond.f90:192-234): for each bubble centred at the
 * 1-based site (cx, cy, cz), with r the unwrapped distance and
 * step = (phi_false - phi_true)/2, ave = (phi_true - phi_false)/2:
 *   r > t0:  phi += step tanh(s/sqrt2) + ave,  s = sqrt(r^2 - t0^2) - r0,
 *            pi  += -step t0 / (sqrt(r^2 - t0^2) sqrt2) / cosh^2(s/sqrt2);
 *   else:    phi += phi_true - phi_false;
 * then phi += phi_false.  Other fields are zero. */
int lat_init_bubbles_boosted(lat_t* h, int32_t nbub, const int32_t* centres, double r0, double t0,
                             double phi_false, double phi_true);

/* -------------------------------------------------------------- checkpoint */
/* Raw native-double checkpoint fld_<i>.raw / fldp_<i>.raw (interior only,
 * x fastest) plus checkpt.dat "yscl ysclp / time / outframenum";
 * make_check_pt / read_check_pt, Discrete/Bubble-Collisions/scafld.f90:227-287
 * and driver.f90:71-91,117-129.  `dir` must exist. */
int lat_checkpoint_write(lat_t* h, const char* dir, double time, int32_t frame);
int lat_checkpoint_read(lat_t* h, const char* dir, double* time, int32_t* frame);

/* ------------------------------------------------------------ output files */
/* Appends one record to an energy file in the column layout of dump_rho
 * (Pseudospec/openmp_dev/evolve_spectral.f90:402-405, energy_spec.out):
 * time, a, rho, KE, PE, GE, -3H^2, (rho - 3H^2)/rho, -ysclp^2/(12 a^4),
 * <phi_1>, <phi_2> (the last for two or more fields), each as Fortran
 * ES22.15 followed by two spaces. */
int lat_write_energy_line(lat_t* h, const char* path, double time);
/* One record of the DEFROST tree's LOG.out (output_log_file,
 * Discrete/Bubble-Collisions/iofile.f90:614-630), appended to `path` in the
 * format of lat_write_energy_line, after a one-line header when the file is
 * empty: t, a, H, <rho> = KE + GE + PE (scalar_en), rhoball, KE, PE,
 * GE (grad_en), GE (grad_en_wlap), -3H^2 (grav_en), KE + GE + PE - 3H^2
 * (hamiltonian).  rhoball (iofile.f90:523-567) sums ekin (sum_f pi_f)^2 +
 * egrad GRAD2 + V over the sites with |(i, j, k) - n/2|^2 dx^2 < 45 (1-based
 * indices), ekin = 1/(2 a^6), egrad = 1/(4 (a dx)^2 cc).  Finite-difference
 * lattices (LAT_ERR_UNSUPPORTED otherwise). */
int lat_write_log_line(lat_t* h, const char* path, double time);
/* Appends one block to a spectrum file as make_output writes it
 * (evolve_spectral.f90:525-549, spectrum.out): for each of the ns bins,
 * (i-1) dk, P(phi_1), P(pi_1), Re and Im of the pi_1 x conj(phi_1) cross
 * spectrum, then zeros up to 2 nfld + 2 columns (columns the reference
 * leaves unset), then an empty line. */
int lat_write_spectrum_block(lat_t* h, const char* path);
/* output_cube (Discrete/Bubble-Collisions/outputfile.f90:942-1016): writes
 * every ds-th site of field `field` (what = LAT_SPEC_FLD) or of its momentum
 * (LAT_SPEC_FLDP) as FP64 little-endian, x fastest, to
 * <dir>/<name>-<frame, 5 digits>.raw, and the VisIt brick-of-values header
 * <dir>/<name>-<frame>.bov (TIME, VARIABLE, BRICK_ORIGIN, BRICK_SIZE = n dx,
 * DATA_FILE, DATA_SIZE = n / ds, DATA_FORMAT DOUBLE, DATA_ENDIAN LITTLE,
 * CENTERING zonal).  Every side must be a multiple of ds. */
int lat_write_cube(lat_t* h, int32_t what, int32_t field, int32_t ds, const char* dir, const char* name,
                   int32_t frame, double time);

/* ------------------------------------------------------------- ensembles */
/* A batch of independent runs of one model on lattices of uneven size,
 * advanced together: per-size batched FFT plans and one persistent launch
 * per pass over a (run, tile) work list, the whole step captured in a CUDA
 * graph.  Spectral Laplacian, Minkowski, FP32-Kahan or FP64.  No reference
 * counterpart (the reference runs one lattice per job). */
typedef struct lat_ens_s lat_ens_t;
int lat_ens_create(lat_ens_t** out, const lat_config* base, int32_t nruns,
                   const int32_t* sizes /* n per run, cubic */);
int lat_ens_destroy(lat_ens_t* e);
int lat_ens_init_vacuum(lat_ens_t* e, const uint64_t* seeds, double fld0,
                        double dfld0, double m2eff, double amp, double kcut_frac);
int lat_ens_symp(lat_ens_t* e, int32_t order, double dt_over_dx, int32_t nsteps);
int lat_ens_energies(lat_ens_t* e, double* out /* nruns x LAT_NENERGY */);
int lat_ens_spectrum(lat_ens_t* e, int32_t run, int32_t nbins, double* S, double* W);
int lat_ens_download(lat_ens_t* e, int32_t run, double* fld, double* fldp);
int lat_ens_sync(lat_ens_t* e);
/* Graph of lat_ens_symp(e, order, dt_over_dx, nsteps) built without running it. */
int lat_ens_prepare(lat_ens_t* e, int32_t order, double dt_over_dx, int32_t nsteps);
/* CUDA events on the ensemble's stream (slots 0..15) and the device time between two. */
int lat_ens_mark(lat_ens_t* e, int32_t slot);
int lat_ens_mark_elapsed(lat_ens_t* e, int32_t slot_a, int32_t slot_b, double* ms);
int lat_ens_launch_count(const lat_ens_t* e, int64_t* count);
/* Times the persistent passes' block size and blocks per SM on this ensemble
 * and, where every size class admits them, the streamed separable passes
 * against the per-class cuFFT path (state saved and restored); keeps the
 * fastest and caches it in cache_path (JSON lines keyed by precision, SM count
 * and the run sizes); NULL: no cache. */
int lat_ens_autotune(lat_ens_t* e, const char* cache_path);
/* out[0] threads per block, out[1] blocks per SM of the persistent passes */
int lat_ens_tuning_get(const lat_ens_t* e, int32_t out[2]);
/* 1 when the ensemble's kicks run on the streamed separable passes: FP32,
 * every size class 64, 96, 128, 192 or 256 with an even number of runs, two
 * runs of a class forming one complex line (the default when admitted;
 * LAT_ENS_CUFFT=1 in the environment at creation keeps cuFFT), else 0. */
int lat_ens_sep_streamed(const lat_ens_t* e, int32_t* on);

/* ------------------------------------------------- learned subgrid closure */
/* No reference counterpart.  A coarse lattice evolved with a kick corrected
 * by a small network: three periodic 3x3x3 convolutions 4 -> 32 -> 32 -> 2
 * channels with GELU (tanh form) after the first two, BF16 weights and activations,
 * FP32 accumulation on the tensor cores, FP32 master weights and Adam state.
 * Inputs are the coarse (phi, chi, pi_phi, pi_chi) of a two-field lattice,
 * normalised as (x - in_shift) * in_scale; the output o_f gives the force
 * correction Delta_f = o_f / out_scale_f and the kick uses V'_f - Delta_f:
 *   pi_f += dt (a^2 lap phi_f - a^4 (V'_f - Delta_f)).
 * Training data come from lat_coarsen of fine runs: one sample is six
 * FP32 arrays [6][nz][ny][nx] (phi, chi, pi_phi, pi_chi, Delta_phi,
 * Delta_chi) and sample s of a batch starts at data + idx[s] * stride.
 * Lattices: nx a multiple of 16, ny a multiple of 8. */
typedef struct lat_net_s lat_net_t;
/* Variables the network sees on a conformal lattice.  PROGRAM: phi, pi and
 * Delta as evolved.  CONFORMAL: a phi, pi / a and a^3 Delta, which for the
 * quartic models make the data stationary in the radiation era (the kick
 * then adds hk a (a^3 Delta)).  Minkowski lattices ignore the choice. */
enum lat_closure_units { LAT_UNITS_PROGRAM = 0, LAT_UNITS_CONFORMAL = 1 };
int64_t lat_net_nparams(void);
int lat_net_create(lat_net_t** out, int32_t device, uint64_t seed);
/* refused (LAT_ERR_STATE) while the network is attached to a lattice */
int lat_net_destroy(lat_net_t* n);
/* flat FP32 parameters: W1[27][8][32] b1[32] W2[27][32][32] b2[32]
 * W3[27][32][8] b3[8]; tap = (dz+1)*9 + (dy+1)*3 + (dx+1) for the input
 * offset (dx, dy, dz); padded channels (inputs 4..7, outputs 2..7) are zero */
int lat_net_get_params(lat_net_t* n, float* out, int64_t count);
int lat_net_set_params(lat_net_t* n, const float* in, int64_t count);
int lat_net_set_norm(lat_net_t* n, const double in_shift[4], const double in_scale[4],
                     const double out_scale[2]);
int lat_net_get_norm(const lat_net_t* n, double in_shift[4], double in_scale[4], double out_scale[2]);
/* network output (normalised units) of nidx samples into out_dev [nidx][N][2] */
int lat_net_forward(lat_net_t* n, const float* data_dev, int64_t stride, const int32_t* idx,
                    int32_t nidx, int32_t nx, int32_t ny, int32_t nz, float* out_dev);
/* mean squared error of the batch against out_scale * Delta and its gradient
 * with respect to the flat parameters (grad_host may be NULL); no update */
int lat_net_grad(lat_net_t* n, const float* data_dev, int64_t stride, const int32_t* idx,
                 int32_t nidx, int32_t nx, int32_t ny, int32_t nz, double* loss, float* grad_host);
/* one Adam step (beta 0.9, 0.999, eps 1e-8) on the batch; returns the loss before the step */
int lat_net_train_step(lat_net_t* n, const float* data_dev, int64_t stride, const int32_t* idx,
                       int32_t nidx, int32_t nx, int32_t ny, int32_t nz, double lr, double* loss);
int64_t lat_net_launch_count(const lat_net_t* n);
/* Device time (CUDA events on the network's stream, after one warm-up) of
 * one forward pass over an nx x ny x nz lattice, averaged over `reps`:
 * ms[0] input packing, ms[1..3] the three convolutions. */
int lat_net_time_forward(lat_net_t* n, int32_t nx, int32_t ny, int32_t nz, int32_t reps, double ms[4]);
/* Attach (net != NULL) or detach (NULL) a closure to a two-field lattice.
 * lat_symp then evaluates the network on the current fields before the
 * first of every `every` kicks of a call (every >= 1) and applies the
 * correction after each kick; `units` is a lat_closure_units value and must
 * match the data the network was trained on.  The normalisation is read at
 * attach time. */
int lat_closure_attach(lat_t* h, lat_net_t* net, int32_t every, int32_t units);
/* Sharp-k filter of a fine lattice onto a coarse nc^3 lattice of the same
 * box: modes |k_i| < nc/2 (per axis, coarse Nyquist planes dropped) are kept,
 * in FP64.  Writes FP32 [3 nf][nc^3]: the filtered fields, the filtered
 * momenta, and Delta_f = V'_f(F phi) - F V'_f(phi) (the force the coarse
 * kick misses) into out_dev, in the variables `units` selects. */
int lat_coarsen(lat_t* fine, int32_t nc, int32_t units, float* out_dev);

/* ------------------------------------------------------ z-slab decomposition */
/* A handle for the z-planes [z0, z1) of a global periodic lattice, one per
 * rank of a decomposed run: the MPI slab split of the reference, where each
 * rank owns a range of planes, exchanges one ghost plane with each z
 * neighbour before every FD kick and all-reduces the lattice sums of the
 * Friedmann update (Pseudospec/mpi_dev/hamiltonian_minkowski.f90:297-342,
 * hamiltonian_conformal.f90:112-114,198-201; the DEFROST tree's wrap_field
 * for z, Discrete/Bubble-Collisions/scafld.f90:120-192).  Finite-difference
 * stencils only (7 or 27 points, GW strains included); the spectral
 * Laplacian's distributed transform is not built (lat_slab_create refuses
 * it with LAT_ERR_UNSUPPORTED).  Field arrays of lat_upload/lat_download and
 * lat_gw_upload/lat_gw_download on a slab hold its nz_loc = z1 - z0 interior
 * planes, unpadded.  The caller moves the data between ranks (MPI, NCCL,
 * torch.distributed): two hooks are called from inside lat_symp, lat_split,
 * lat_o2step, lat_energies and lat_calc_metric, which then run without CUDA
 * graphs:
 *   halo(user, h): fill both ghost planes of h, e.g. lat_slab_halo packs of
 *     the boundary planes sent to the z neighbours and unpacks of what they
 *     sent; called before every kick and every energy reduction;
 *   sum(user, v, n): replace the n doubles of v by their sum over all
 *     slabs (MPI_Allreduce); called for the lattice sums of every
 *     conformal drift and kick and of lat_energies.
 * A hook returns 0 on success; any other value stops the call with
 * LAT_ERR_STATE.  Without hooks the evolution calls return LAT_ERR_STATE.
 * Spectra, Laplacian, initial-condition, checkpoint, output-cube, LOG.out,
 * autotune and closure calls return LAT_ERR_UNSUPPORTED on a slab handle. */
typedef int (*lat_halo_fn)(void* user, lat_t* h);
typedef int (*lat_sum_fn)(void* user, double* v, int32_t n);
int lat_slab_create(lat_t** out, const lat_config* global_cfg, int32_t z0, int32_t z1);
int lat_slab_set_hooks(lat_t* h, lat_halo_fn halo, lat_sum_fn sum, void* user);
/* Bytes of one halo message: one z-plane of every field (FP32 lattices: the
 * high words phi_hi the stencil reads) and of the six GW strains, in the
 * handle's precision, [array][y][x]. */
int lat_slab_halo_bytes(const lat_t* h, size_t* bytes);
/* op 0 / 1: copy the lowest / highest interior plane (global z0 / z1-1)
 * into dev_buf; op 2 / 3: fill the lower / upper ghost plane (global z0-1 /
 * z1) from dev_buf.  dev_buf is device memory of lat_slab_halo_bytes; the
 * call returns when the copy has completed. */
int lat_slab_halo(lat_t* h, int32_t op, void* dev_buf);

/* ---------------------------------------------------------- measurement */
/* Kernel classes timed with CUDA events on the handle's stream when
 * timing is enabled (one event pair per launch). */
enum lat_kclass {
  LAT_K_KICKDRIFT = 0,   /* fused kick+drift pass (FD stencil or spectral pointwise) */
  LAT_K_DRIFT = 1,
  LAT_K_KICK = 2,
  LAT_K_KMUL = 3,        /* k-space -k^2/N multiply (+ Parseval reduction) */
  LAT_K_FFT_R2C = 4,     /* cuFFT forward */
  LAT_K_FFT_C2R = 5,     /* cuFFT inverse */
  LAT_K_GW = 6,          /* GW kick+drift */
  LAT_K_OTHER = 7,
  LAT_K_SEP_X = 8,       /* separable spectral pass X: drift + d2/dx2 */
  LAT_K_SEP_Y = 9,       /* separable spectral pass Y: + d2/dy2 */
  LAT_K_SEP_Z = 10,      /* separable spectral pass Z: + d2/dz2 and kick */
  LAT_NKCLASS = 11
};
int lat_timing_enable(lat_t* h, int32_t on);
/* total milliseconds and launch count of one class since the last reset */
int lat_timing_read(lat_t* h, int32_t kclass, double* total_ms, int64_t* launches);
int lat_timing_reset(lat_t* h);
/* Records CUDA event `slot` (0..15) on the handle's stream; lat_mark_elapsed
 * waits for both events and returns the device time between them. */
int lat_mark(lat_t* h, int32_t slot);
int lat_mark_elapsed(lat_t* h, int32_t slot_a, int32_t slot_b, double* ms);
/* number of engine kernels launched on this handle since creation */
int lat_launch_count(const lat_t* h, int64_t* count);
/* Device pointers of the state, for zero-copy harnesses.  what: 0 = fld,
 * 1 = fldp, 2 = Kahan compensation of fld (FP32 only), 3 = scalar block.
 * Element type is double (FP64) or float (FP32_KAHAN), layout [field][z][y][x]. */
int lat_device_ptr(lat_t* h, int32_t what, void** ptr);
/* Pinned host memory for staging (cudaHostAlloc / cudaFreeHost). */
int lat_host_alloc(void** ptr, size_t bytes);
int lat_host_free(void* ptr);
/* Device memory for data sets (closure training samples) and a synchronous
 * copy; kind 0 host to device, 1 device to host, 2 device to device. */
int lat_dev_alloc(int32_t device, void** ptr, size_t bytes);
int lat_dev_free(void* ptr);
int lat_memcpy(void* dst, const void* src, size_t bytes, int32_t kind);

/* -------------------------------------------------------------- autotune */
/* Times the candidate tile shapes / block schedules of this handle's kernels
 * on its own lattice (state is saved and restored) and keeps the fastest;
 * results are cached in `cache_path` (JSON lines) keyed by size, precision,
 * stencil and device, and reused when present.  cache_path may be NULL. */
int lat_autotune(lat_t* h, const char* cache_path);
/* The choice in use: FD tile tx, ty, zchunk; pointwise block threads, blocks
 * per SM; spectral path (LAT_SPEC_IMPL_CUFFT or LAT_SPEC_IMPL_SEPARABLE). */
int lat_tuning_get(const lat_t* h, int32_t out[6]);
/* 1 when the handle's separable passes are the streamed kind (two FP32
 * fields, every side 128 or 256: the kick accumulates in the momenta pass by
 * pass and no Laplacian array is kept), else 0. */
int lat_sep_streamed(const lat_t* h, int32_t* on);

#ifdef __cplusplus
}
#endif
#endif /* LATTICE_GB300_H */
