// fft.hpp -- FP64 mixed-radix FFT for the CPU oracle (test infrastructure
// only; the engine uses cuFFT).  Unnormalised transforms with FFTW's sign
// conventions: forward e^{-2 pi i k x / n}, backward e^{+2 pi i k x / n}.
// The 3D real transforms follow fftw_plan_dft_r2c_3d(nz,ny,nx,...) as used by
// Pseudospec/openmp_dev/evolve_spectral.f90:110-111: the array is f[z][y][x]
// (x fastest) and the halved axis is x, giving F[z][y][nx/2+1].
#pragma once
#include <complex>
#include <vector>
#include <cstdint>

namespace orc {

using cplx = std::complex<double>;

// One 1D complex transform length with its radix factorisation and twiddles.
class Fft1d {
 public:
  explicit Fft1d(int n = 1);
  int size() const { return n_; }
  // In-place transform of `data` (contiguous); `work` must hold n entries.
  void exec(cplx* data, cplx* work, int sign) const;

 private:
  void rec(const cplx* in, cplx* out, int n, int stride, int fi, int sign) const;
  int n_;
  std::vector<int> factors_;
  std::vector<cplx> tw_;  // e^{-2 pi i j / n}, j = 0..n-1
};

// 3D real <-> half-complex transforms over f[nz][ny][nx] (x fastest).
class Fft3dReal {
 public:
  Fft3dReal(int nx, int ny, int nz);
  int nx() const { return nx_; }
  int ny() const { return ny_; }
  int nz() const { return nz_; }
  int64_t nreal() const { return (int64_t)nx_ * ny_ * nz_; }
  int64_t ncplx() const { return (int64_t)(nx_ / 2 + 1) * ny_ * nz_; }
  // F = sum_x f(x) e^{-i k x}; f is not modified.
  void r2c(const double* f, cplx* F) const;
  // f = sum_k F(k) e^{+i k x} (unnormalised); F is destroyed.
  void c2r(cplx* F, double* f) const;

 private:
  void lines_yz(cplx* F, int sign) const;
  int nx_, ny_, nz_;
  Fft1d fx_, fy_, fz_;
};

}  // namespace orc
