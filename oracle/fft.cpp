// fft.cpp -- FP64 mixed-radix FFT for the CPU oracle (test infrastructure).
// Recursive decimation in time over the factorisation of n (radix 4, 2, 3, 5,
// then any remaining prime by direct summation).  Real 3D transforms pack two
// real x-rows into one complex transform.
#include "fft.hpp"

#include <cmath>
#include <cstring>

namespace orc {

static const double kTwoPi = 6.283185307179586476925286766559;

Fft1d::Fft1d(int n) : n_(n) {
  int m = n;
  while (m % 4 == 0) { factors_.push_back(4); m /= 4; }
  while (m % 2 == 0) { factors_.push_back(2); m /= 2; }
  for (int p = 3; m > 1; p += 2) {
    while (m % p == 0) { factors_.push_back(p); m /= p; }
  }
  tw_.resize(n);
  for (int j = 0; j < n; ++j) {
    // angle reduced to the first octant-free form for accuracy
    long double ang = -(long double)kTwoPi * (long double)j / (long double)n;
    tw_[j] = cplx((double)std::cos(ang), (double)std::sin(ang));
  }
}

void Fft1d::rec(const cplx* in, cplx* out, int n, int stride, int fi,
                int sign) const {
  if (n == 1) { out[0] = in[0]; return; }
  const int p = factors_[fi];
  const int m = n / p;
  for (int q = 0; q < p; ++q) rec(in + (int64_t)q * stride, out + q * m, m, stride * p, fi + 1, sign);
  const int tstep = n_ / n;  // W_n^j = tw_[j * tstep]
  auto W = [&](int64_t j) -> cplx {
    cplx w = tw_[(j * tstep) % n_];
    return sign > 0 ? std::conj(w) : w;
  };
  if (p == 2) {
    for (int k = 0; k < m; ++k) {
      cplx a = out[k], b = out[k + m] * W(k);
      out[k] = a + b;
      out[k + m] = a - b;
    }
    return;
  }
  if (p == 4) {
    const cplx mi = sign > 0 ? cplx(0, 1) : cplx(0, -1);  // W_4^1
    for (int k = 0; k < m; ++k) {
      cplx t0 = out[k];
      cplx t1 = out[k + m] * W(k);
      cplx t2 = out[k + 2 * m] * W(2 * k);
      cplx t3 = out[k + 3 * m] * W(3 * k);
      cplx s02 = t0 + t2, d02 = t0 - t2, s13 = t1 + t3, d13 = (t1 - t3) * mi;
      out[k] = s02 + s13;
      out[k + m] = d02 + d13;
      out[k + 2 * m] = s02 - s13;
      out[k + 3 * m] = d02 - d13;
    }
    return;
  }
  std::vector<cplx> t(p), r(p);
  const int pstep = n_ / p;  // W_p^j = tw_[j * pstep]
  for (int k = 0; k < m; ++k) {
    for (int q = 0; q < p; ++q) t[q] = out[k + q * m] * W((int64_t)q * k);
    for (int s = 0; s < p; ++s) {
      cplx acc = 0;
      for (int q = 0; q < p; ++q) {
        cplx w = tw_[((int64_t)((q * s) % p) * pstep) % n_];
        acc += t[q] * (sign > 0 ? std::conj(w) : w);
      }
      r[s] = acc;
    }
    for (int s = 0; s < p; ++s) out[k + s * m] = r[s];
  }
}

void Fft1d::exec(cplx* data, cplx* work, int sign) const {
  if (n_ == 1) return;
  rec(data, work, n_, 1, 0, sign);
  std::memcpy((void*)data, (const void*)work, sizeof(cplx) * n_);
}

Fft3dReal::Fft3dReal(int nx, int ny, int nz)
    : nx_(nx), ny_(ny), nz_(nz), fx_(nx), fy_(ny), fz_(nz) {}

void Fft3dReal::lines_yz(cplx* F, int sign) const {
  const int hx = nx_ / 2 + 1;
  const int B = 8;
  // y lines: for each z and block of kx
  const int nblk = (hx + B - 1) / B;
#pragma omp parallel
  {
    std::vector<cplx> buf((size_t)B * (ny_ > nz_ ? ny_ : nz_)), work(ny_ > nz_ ? ny_ : nz_);
#pragma omp for schedule(static)
    for (int64_t t = 0; t < (int64_t)nz_ * nblk; ++t) {
      int z = (int)(t / nblk), kb = (int)(t % nblk) * B;
      int nb = hx - kb < B ? hx - kb : B;
      cplx* base = F + (int64_t)z * ny_ * hx;
      for (int y = 0; y < ny_; ++y)
        for (int b = 0; b < nb; ++b) buf[(size_t)b * ny_ + y] = base[(int64_t)y * hx + kb + b];
      for (int b = 0; b < nb; ++b) fy_.exec(&buf[(size_t)b * ny_], work.data(), sign);
      for (int y = 0; y < ny_; ++y)
        for (int b = 0; b < nb; ++b) base[(int64_t)y * hx + kb + b] = buf[(size_t)b * ny_ + y];
    }
#pragma omp for schedule(static)
    for (int64_t t = 0; t < (int64_t)ny_ * nblk; ++t) {
      int y = (int)(t / nblk), kb = (int)(t % nblk) * B;
      int nb = hx - kb < B ? hx - kb : B;
      const int64_t zs = (int64_t)ny_ * hx;
      cplx* base = F + (int64_t)y * hx + kb;
      for (int z = 0; z < nz_; ++z)
        for (int b = 0; b < nb; ++b) buf[(size_t)b * nz_ + z] = base[z * zs + b];
      for (int b = 0; b < nb; ++b) fz_.exec(&buf[(size_t)b * nz_], work.data(), sign);
      for (int z = 0; z < nz_; ++z)
        for (int b = 0; b < nb; ++b) base[z * zs + b] = buf[(size_t)b * nz_ + z];
    }
  }
}

void Fft3dReal::r2c(const double* f, cplx* F) const {
  const int hx = nx_ / 2 + 1;
  const int64_t nrows = (int64_t)ny_ * nz_;
  const int64_t npairs = (nrows + 1) / 2;
#pragma omp parallel
  {
    std::vector<cplx> z(nx_), work(nx_);
#pragma omp for schedule(static)
    for (int64_t pr = 0; pr < npairs; ++pr) {
      int64_t r1 = 2 * pr, r2 = r1 + 1;
      const double* a = f + r1 * nx_;
      const double* b = r2 < nrows ? f + r2 * nx_ : nullptr;
      for (int x = 0; x < nx_; ++x) z[x] = cplx(a[x], b ? b[x] : 0.0);
      fx_.exec(z.data(), work.data(), -1);
      cplx* o1 = F + r1 * hx;
      cplx* o2 = b ? F + r2 * hx : nullptr;
      for (int k = 0; k < hx; ++k) {
        cplx zk = z[k], zm = std::conj(z[(nx_ - k) % nx_]);
        o1[k] = 0.5 * (zk + zm);
        if (o2) o2[k] = cplx(0, -0.5) * (zk - zm);
      }
    }
  }
  lines_yz(F, -1);
}

void Fft3dReal::c2r(cplx* F, double* f) const {
  const int hx = nx_ / 2 + 1;
  lines_yz(F, +1);
  const int64_t nrows = (int64_t)ny_ * nz_;
  const int64_t npairs = (nrows + 1) / 2;
#pragma omp parallel
  {
    std::vector<cplx> z(nx_), work(nx_);
#pragma omp for schedule(static)
    for (int64_t pr = 0; pr < npairs; ++pr) {
      int64_t r1 = 2 * pr, r2 = r1 + 1;
      cplx* x1 = F + r1 * hx;
      cplx* x2 = r2 < nrows ? F + r2 * hx : nullptr;
      // the DC and Nyquist bins of a real row are real (FFTW ignores their imaginary parts)
      auto X1 = [&](int k) {
        cplx v = x1[k];
        if (k == 0 || 2 * k == nx_) v = cplx(v.real(), 0.0);
        return v;
      };
      auto X2 = [&](int k) {
        if (!x2) return cplx(0, 0);
        cplx v = x2[k];
        if (k == 0 || 2 * k == nx_) v = cplx(v.real(), 0.0);
        return v;
      };
      for (int k = 0; k < hx; ++k) z[k] = X1(k) + cplx(0, 1) * X2(k);
      for (int k = hx; k < nx_; ++k) z[k] = std::conj(X1(nx_ - k)) + cplx(0, 1) * std::conj(X2(nx_ - k));
      fx_.exec(z.data(), work.data(), +1);
      double* a = f + r1 * nx_;
      for (int x = 0; x < nx_; ++x) a[x] = z[x].real();
      if (x2) {
        double* b = f + r2 * nx_;
        for (int x = 0; x < nx_; ++x) b[x] = z[x].imag();
      }
    }
  }
}

}  // namespace orc
