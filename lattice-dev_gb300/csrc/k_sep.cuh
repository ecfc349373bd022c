// k_sep.cuh -- separable spectral Laplacian passes (sm_103a).
//
// The spectral Laplacian of laplacian_3d (Pseudospec/openmp_dev/fftw_mod.f90:
// 177-207: r2c, multiply by -(ii^2+jj^2+kk^2) dk^2, c2r, divide by N) is a
// sum of three one-dimensional spectral second derivatives, because the
// multiplier -|k|^2 = -kx^2 - ky^2 - kz^2 separates and the 3D DFT is a
// product of 1D DFTs.  Each 1D term is a transform along one lattice line,
// so it runs inside one thread block, in registers, with no global
// transposes and no k-space array in HBM:
//
//   pass X: drift (Kahan) of phi, then lap  = d2x(phi)      [+ KE2, PE, GEx]
//   pass Y:                             lap += d2y(phi)      [+ GEy]
//   pass Z:                     kick with lap + d2z(phi)     [+ GEz, Friedmann]
//
// Two real lines share one complex transform: since the multiplier is real and
// even, IDFT(H DFT(A + iB)) = d2(A) + i d2(B).  With two fields the pair is
// the two fields at the same sites (so the coupled potential sees both); with
// one field it is two neighbouring lines.
//
// Line transforms of N = P Q points use P threads with Q points each:
// a Q-point DFT in registers, twiddles W_N^{t kq}, a transpose through shared
// memory, P-point DFTs, the multiplier -(f dk)^2/N, and the mirror image back
// to the original layout.  The per-axis Parseval sum (f dk)^2 |Z_k|^2 / N is
// taken where the spectrum sits in registers; it equals -sum phi d2(phi), so
// GE2 = GEx + GEy + GEz as in hamiltonian_conformal.f90:146,172.
//
// The transform input is (phi_hi - mean) - c: the lattice mean (a constant,
// which the multiplier removes exactly) is taken off so rounding scales with
// the fluctuation, and the Kahan compensation c restores the bits the FP32
// field lost.
#pragma once
#include <utility>

#include "engine.hpp"
#include "twiddles.h"

namespace lat {
namespace sep {

template <int N> struct Split;
template <> struct Split<16> { static constexpr int P = 4, Q = 4; };
template <> struct Split<32> { static constexpr int P = 4, Q = 8; };
template <> struct Split<64> { static constexpr int P = 8, Q = 8; };
template <> struct Split<128> { static constexpr int P = 8, Q = 16; };
template <> struct Split<256> { static constexpr int P = 16, Q = 16; };
template <> struct Split<512> { static constexpr int P = 16, Q = 32; };
template <> struct Split<96> { static constexpr int P = 8, Q = 12; };   // Q = 3 x 4 (dft12); 12 rows over 8 threads
template <> struct Split<192> { static constexpr int P = 16, Q = 12; };  // Q = 3 x 4 (dft12); 12 rows over 16 threads

template <typename R> struct Cx;
template <> struct Cx<float> {
  using T = float2;
  static __device__ __forceinline__ float2 tw(int j) { return make_float2(c_tw64f[j][0], c_tw64f[j][1]); }
  static __device__ __forceinline__ float2 tw24(int j) { return make_float2(c_tw24f[j][0], c_tw24f[j][1]); }
};
template <> struct Cx<double> {
  using T = double2;
  static __device__ __forceinline__ double2 tw(int j) { return make_double2(c_tw64[j][0], c_tw64[j][1]); }
  static __device__ __forceinline__ double2 tw24(int j) { return make_double2(c_tw24[j][0], c_tw24[j][1]); }
};

template <typename C> __device__ __forceinline__ C cmul(C a, C b) {
  C r;
  r.x = a.x * b.x - a.y * b.y;
  r.y = a.x * b.y + a.y * b.x;
  return r;
}
template <typename C> __device__ __forceinline__ C cmulc(C a, C b) {  // a * conj(b)
  C r;
  r.x = a.x * b.x + a.y * b.y;
  r.y = a.y * b.x - a.x * b.y;
  return r;
}

__device__ __forceinline__ constexpr int brev(int i, int R) {
  int r = 0;
  for (int b = 1; b < R; b <<= 1) {
    r = (r << 1) | (i & 1);
    i >>= 1;
  }
  return r;
}

template <int R, int I> struct BrevC { static constexpr int value = brev(I, R); };

template <int R, int I, typename T>
__device__ __forceinline__ void brev_swap(T (&re)[R], T (&im)[R]) {
  constexpr int J = BrevC<R, I>::value;
  if constexpr (J > I) {
    const T a = re[I], b = im[I];
    re[I] = re[J];
    im[I] = im[J];
    re[J] = a;
    im[J] = b;
  }
}
template <int R, typename T, int... I>
__device__ __forceinline__ void bitrev_perm(T (&re)[R], T (&im)[R], std::integer_sequence<int, I...>) {
  (brev_swap<R, I>(re, im), ...);
}

// One radix-2 stage (butterflies of length LEN) of the in-register DFT, then
// the next stage; every loop bound is a template constant so the whole
// transform unrolls into straight-line register code.
template <int R, bool INV, typename Rt, int LEN>
__device__ __forceinline__ void dft_stage(Rt (&re)[R], Rt (&im)[R]) {
  constexpr int HALF = LEN / 2;
#pragma unroll
  for (int i = 0; i < R; i += LEN) {
#pragma unroll
    for (int k = 0; k < HALF; ++k) {
      const Rt ar = re[i + k], ai = im[i + k];
      Rt br = re[i + k + HALF], bi = im[i + k + HALF];
      if (k != 0) {
        if (4 * k == LEN) {  // W = -i (forward) or +i (inverse)
          const Rt tr = br;
          if (INV) { br = -bi; bi = tr; }
          else { br = bi; bi = -tr; }
        } else {
          const auto w = Cx<Rt>::tw(k * (64 / LEN));
          const Rt tr = br;
          if (INV) {  // b * conj(w)
            br = tr * w.x + bi * w.y;
            bi = bi * w.x - tr * w.y;
          } else {    // b * w
            br = tr * w.x - bi * w.y;
            bi = tr * w.y + bi * w.x;
          }
        }
      }
      re[i + k] = ar + br;
      im[i + k] = ai + bi;
      re[i + k + HALF] = ar - br;
      im[i + k + HALF] = ai - bi;
    }
  }
  if constexpr (LEN < R) dft_stage<R, INV, Rt, 2 * LEN>(re, im);
}

template <int R, bool INV, typename Rt>
__device__ __forceinline__ void dft3m(Rt (&re)[R], Rt (&im)[R]);
template <bool INV, typename Rt>
__device__ __forceinline__ void dft16r4(Rt (&re)[16], Rt (&im)[16]);

// In-register DFT on separate real and imaginary arrays, natural order in and
// out: radix 4 for R = 16, radix 2 for the other powers of two up to 64
// points (W_len^k from the constant table), and R = 12 = 3 x 4 and
// 24 = 3 x 8.
template <int R, bool INV, typename Rt>
__device__ __forceinline__ void dft(Rt (&re)[R], Rt (&im)[R]) {
  if constexpr (R == 24 || R == 12) {
    dft3m<R, INV, Rt>(re, im);
  } else if constexpr (R == 16) {
    dft16r4<INV, Rt>(re, im);
  } else {
    static_assert(R >= 2 && R <= 64 && (R & (R - 1)) == 0, "register DFT length must be a power of two <= 64 or 24");
    bitrev_perm<R>(re, im, std::make_integer_sequence<int, R>{});
    dft_stage<R, INV, Rt, 2>(re, im);
  }
}

// 4-point DFT of (a, b, c, d) in place: y0 = (a + c) + (b + d),
// y2 = (a + c) - (b + d), y1,3 = (a - c) -+ i (b - d) forward (+- inverse).
template <bool INV, typename Rt>
__device__ __forceinline__ void dft4_at(Rt (&re)[16], Rt (&im)[16], int i0, int i1, int i2, int i3) {
  const Rt sr = re[i0] + re[i2], si = im[i0] + im[i2];
  const Rt dr = re[i0] - re[i2], di = im[i0] - im[i2];
  const Rt tr = re[i1] + re[i3], ti = im[i1] + im[i3];
  const Rt ur = re[i1] - re[i3], ui = im[i1] - im[i3];
  re[i0] = sr + tr;
  im[i0] = si + ti;
  re[i2] = sr - tr;
  im[i2] = si - ti;
  if (INV) {  // y1 = d + i u, y3 = d - i u
    re[i1] = dr - ui;
    im[i1] = di + ur;
    re[i3] = dr + ui;
    im[i3] = di - ur;
  } else {    // y1 = d - i u, y3 = d + i u
    re[i1] = dr + ui;
    im[i1] = di - ur;
    re[i3] = dr - ui;
    im[i3] = di + ur;
  }
}

// 16-point DFT by decimation in time over 4 (radix 4): the four 4-point DFTs
// A_n2[k1] of x[4 n1 + n2], twiddles W_16^{n2 k1} (W_64^{4 n2 k1} from the
// constant table; W_16^4 = -i is a swap), then 4-point DFTs over n2 give
// X[k1 + 4 k2].  160 real additions and multiplications against 168 for
// four radix-2 stages.
template <bool INV, typename Rt>
__device__ __forceinline__ void dft16r4(Rt (&re)[16], Rt (&im)[16]) {
#pragma unroll
  for (int n2 = 0; n2 < 4; ++n2) dft4_at<INV, Rt>(re, im, n2, n2 + 4, n2 + 8, n2 + 12);  // A_n2[k1] at 4 k1 + n2
#pragma unroll
  for (int n2 = 1; n2 < 4; ++n2) {
#pragma unroll
    for (int k1 = 1; k1 < 4; ++k1) {
      const int j = 4 * k1 + n2, m = n2 * k1;
      const Rt xr = re[j], xi = im[j];
      if (m == 4) {  // W_16^4 = -i (forward), +i (inverse)
        if (INV) { re[j] = -xi; im[j] = xr; }
        else { re[j] = xi; im[j] = -xr; }
      } else {
        const auto w = Cx<Rt>::tw(4 * m);
        if (INV) {  // times conj(w)
          re[j] = xr * w.x + xi * w.y;
          im[j] = xi * w.x - xr * w.y;
        } else {
          re[j] = xr * w.x - xi * w.y;
          im[j] = xr * w.y + xi * w.x;
        }
      }
    }
  }
  // X[k1 + 4 k2] = sum over n2 of B_n2[k1] W_4^{n2 k2}: 4-point DFTs across
  // n2 of the values at 4 k1 + n2, written back in natural order
  Rt orr[16], oi[16];
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1) {
    dft4_at<INV, Rt>(re, im, 4 * k1, 4 * k1 + 1, 4 * k1 + 2, 4 * k1 + 3);
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) {
      orr[k1 + 4 * k2] = re[4 * k1 + k2];
      oi[k1 + 4 * k2] = im[4 * k1 + k2];
    }
  }
#pragma unroll
  for (int k = 0; k < 16; ++k) {
    re[k] = orr[k];
    im[k] = oi[k];
  }
}

// 3M-point DFT (M = 4 or 8) by decimation in time over 3: the three M-point
// DFTs of the subsequences x[3 n1 + n2] (Y_n2[k1]), twiddles
// W_3M^{n2 k1} = W_24^{(8/M) n2 k1}, then 3-point DFTs over n2 give
// X[k1 + M k2].  The 3-point DFT with w = exp(-+2 pi i / 3):
// X0 = a + s, X1,2 = a - s/2 -+ i (sqrt(3)/2) d, s = b + c, d = b - c.
template <int R, bool INV, typename Rt>
__device__ __forceinline__ void dft3m(Rt (&re)[R], Rt (&im)[R]) {
  static_assert(R == 24 || R == 12, "dft3m takes 12 or 24 points");
  constexpr int M = R / 3, TS = 8 / M;
  Rt ar[3][M], ai[3][M];
#pragma unroll
  for (int n2 = 0; n2 < 3; ++n2) {
#pragma unroll
    for (int n1 = 0; n1 < M; ++n1) {
      ar[n2][n1] = re[3 * n1 + n2];
      ai[n2][n1] = im[3 * n1 + n2];
    }
    dft<M, INV, Rt>(ar[n2], ai[n2]);
  }
#pragma unroll
  for (int n2 = 1; n2 < 3; ++n2) {
#pragma unroll
    for (int k1 = 1; k1 < M; ++k1) {
      const auto w = Cx<Rt>::tw24(TS * n2 * k1);
      const Rt xr = ar[n2][k1], xi = ai[n2][k1];
      if (INV) {  // times conj(w)
        ar[n2][k1] = xr * w.x + xi * w.y;
        ai[n2][k1] = xi * w.x - xr * w.y;
      } else {
        ar[n2][k1] = xr * w.x - xi * w.y;
        ai[n2][k1] = xr * w.y + xi * w.x;
      }
    }
  }
  const Rt h3 = (Rt)0.8660254037844386;  // sqrt(3)/2
#pragma unroll
  for (int k1 = 0; k1 < M; ++k1) {
    const Rt sr = ar[1][k1] + ar[2][k1], si = ai[1][k1] + ai[2][k1];
    const Rt dr = (ar[1][k1] - ar[2][k1]) * h3, di = (ai[1][k1] - ai[2][k1]) * h3;
    const Rt tr = ar[0][k1] - (Rt)0.5 * sr, ti = ai[0][k1] - (Rt)0.5 * si;
    re[k1] = ar[0][k1] + sr;
    im[k1] = ai[0][k1] + si;
    if (INV) {  // X1 = t + i m, X2 = t - i m
      re[k1 + M] = tr - di;
      im[k1 + M] = ti + dr;
      re[k1 + 2 * M] = tr + di;
      im[k1 + 2 * M] = ti - dr;
    } else {    // X1 = t - i m, X2 = t + i m
      re[k1 + M] = tr + di;
      im[k1 + M] = ti - dr;
      re[k1 + 2 * M] = tr - di;
      im[k1 + 2 * M] = ti + dr;
    }
  }
}

// Spectral second derivative of the complex line held as (re, im)[q] =
// line[t + P q] by the P threads t of the line; returns the derivative in the
// same layout and adds (f dk)^2 |Z_k|^2 / N to `ge`.  sl: this line's
// [Q][P+1] shared slice (complex); twN: W_N^j in shared memory.  Every thread
// of the block must call it.
template <int N, typename R, typename C, typename Acc>
__device__ __forceinline__ void d2_line(R (&re)[Split<N>::Q], R (&im)[Split<N>::Q], int t, C* sl, const C* twN, R dk2,
                                        Acc& ge) {
  constexpr int P = Split<N>::P, Q = Split<N>::Q, G = Q / P, S = P + 1;
  static_assert(Q % P == 0, "the one-tile passes need Q a multiple of P");
  dft<Q, false, R>(re, im);
#pragma unroll
  for (int kq = 0; kq < Q; ++kq) {
    const C w = twN[(t * kq) & (N - 1)];
    const R xr = re[kq], xi = im[kq];
    C o;
    o.x = xr * w.x - xi * w.y;
    o.y = xr * w.y + xi * w.x;
    sl[kq * S + t] = o;
  }
  __syncthreads();
  R ur[G][P], ui[G][P];
#pragma unroll
  for (int g = 0; g < G; ++g) {
    const int kq = t + g * P;
#pragma unroll
    for (int tt = 0; tt < P; ++tt) {
      const C z = sl[kq * S + tt];
      ur[g][tt] = z.x;
      ui[g][tt] = z.y;
    }
    dft<P, false, R>(ur[g], ui[g]);
    R gpart = R(0);  // this thread's P modes, folded into `ge` once
#pragma unroll
    for (int kp = 0; kp < P; ++kp) {
      const int k = kq + Q * kp;
      const int f = k <= N / 2 ? k : k - N;
      const R f2 = (R)(f * f) * dk2;  // (f dk)^2
      const R zr = ur[g][kp], zi = ui[g][kp];
      gpart += f2 * (zr * zr + zi * zi);
      const R h = -f2 * (R)(1.0 / N);
      ur[g][kp] = zr * h;
      ui[g][kp] = zi * h;
    }
    ge.add(gpart * (R)(1.0 / N));
    dft<P, true, R>(ur[g], ui[g]);
  }
  // no barrier here: rows kq = t + g P are read and rewritten by thread t
  // alone; the next barrier orders them before the column reads
#pragma unroll
  for (int g = 0; g < G; ++g) {
    const int kq = t + g * P;
#pragma unroll
    for (int mp = 0; mp < P; ++mp) {
      const C w = twN[(mp * kq) & (N - 1)];
      const R xr = ur[g][mp], xi = ui[g][mp];
      C o;  // times conj(W_N^{mp kq})
      o.x = xr * w.x + xi * w.y;
      o.y = xi * w.x - xr * w.y;
      sl[kq * S + mp] = o;
    }
  }
  __syncthreads();
#pragma unroll
  for (int kq = 0; kq < Q; ++kq) {
    const C z = sl[kq * S + t];
    re[kq] = z.x;
    im[kq] = z.y;
  }
  dft<Q, true, R>(re, im);
}

// Offsets of the two real lines (A, B) of complex line l along AXIS and the
// stride between successive points.
template <int AXIS, int NF>
__device__ __forceinline__ void line_map(int64_t l, int nx, int ny, int64_t Nsite, int64_t& offA, int64_t& offB,
                                         int64_t& stride) {
  if (AXIS == 0) {
    stride = 1;
    if (NF == 2) { offA = l * nx; offB = Nsite + offA; }
    else { offA = 2 * l * nx; offB = offA + nx; }
  } else {
    const int64_t plane = (int64_t)nx * ny;
    stride = AXIS == 1 ? nx : plane;
    int64_t x, o;
    if (NF == 2) { x = l % nx; o = l / nx; }
    else { x = 2 * (l % (nx / 2)); o = l / (nx / 2); }
    offA = (AXIS == 1 ? o * plane : o * nx) + x;
    offB = NF == 2 ? Nsite + offA : offA + 1;
  }
}

}  // namespace sep

enum SepPass { SEP_X = 0, SEP_Y = 1, SEP_Z = 2 };

namespace sep {

__device__ __forceinline__ void cp16(void* smem, const void* gmem) {
  const unsigned int sa = (unsigned int)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// Tile geometry of a pass: 256 threads, LINES = 256/P complex lines per
// block.  The FFT scratch of one line is padded so that the lines sharing a
// warp start in different shared-memory banks.
template <typename R, int NF, int AXIS, int N>
struct Tile {
  static constexpr int P = Split<N>::P, Q = Split<N>::Q, S = P + 1;
  static constexpr int THREADS = 256;
  static constexpr int LINES = THREADS / P;
  static constexpr int W = NF == 2 ? LINES : 2 * LINES;  // real x-columns per block (AXIS 1, 2)
  static constexpr int CW = 2 * (int)sizeof(R) / 4;      // 32-bit words per complex
  // lanes of one line inside a warp and the words one access of that line spans
  static constexpr int LANES = AXIS == 0 ? P : 32 / LINES;
  static constexpr int line_words = LANES * CW >= 32 ? 0 : LANES * CW;
  static constexpr int lstride_for(int pad) {
    return ((Q * S + pad) * CW) % 32 == line_words ? Q * S + pad : lstride_for(pad + 1);
  }
  static constexpr int LSTRIDE = lstride_for(0);
  // arrays read only after the transform (Y: lap; Z: lap, pi) are copied
  // into shared memory asynchronously at block entry
  static constexpr int NA = AXIS == 1 ? 1 : (AXIS == 2 ? 2 : 0);
  static constexpr int ATILE = 2 * LINES * N;  // reals per staged array
  static constexpr int SMEM = (N + LINES * LSTRIDE) * 2 * (int)sizeof(R) + NA * ATILE * (int)sizeof(R);
};

// One pass of the separable spectral kick-drift; AXIS selects the pass:
// 0 = drift + d2x, 1 = d2y, 2 = d2z + kick.  Every array a pass updates is
// written to a second buffer (phi, c, pi and lap ping-pong), so no pointer a
// thread loads from is ever stored to: with restrict-qualified pointers the
// compiler issues all of a thread's loads before the transform, and 256
// threads per block keep enough warps resident to hide HBM latency.
template <typename R, int NF, int AXIS, int N, bool KAHAN>
__global__ void __launch_bounds__(256) sep_kernel(SepArgs a) {
  using C = typename Cx<R>::T;
  using T = Tile<R, NF, AXIS, N>;
  constexpr int P = T::P, Q = T::Q, LINES = T::LINES;
  extern __shared__ __align__(128) unsigned char smraw[];
  C* twN = reinterpret_cast<C*>(smraw);
  C* fft = twN + N;
  R* astage = reinterpret_cast<R*>(fft + LINES * T::LSTRIDE);  // [NA][ATILE]
  const int tid = threadIdx.x;
  const int t = AXIS == 0 ? tid % P : tid / LINES;
  const int li = AXIS == 0 ? tid / P : tid % LINES;
  if constexpr (AXIS != 0) {
    // the block's lines are W adjacent x-columns at one z (AXIS 1) or y (AXIS 2)
    constexpr int W = T::W, VEC = 16 / (int)sizeof(R), CPR = W / VEC;
    static_assert(W % VEC == 0, "staged rows must hold whole 16-byte copies");
    const int64_t l0 = (int64_t)blockIdx.x * LINES;
    const int64_t per = NF == 2 ? a.nx : a.nx / 2;  // lines per plane
    const int64_t x0 = NF == 2 ? l0 % per : 2 * (l0 % per), o = l0 / per;
    const int64_t plane_ = (int64_t)a.nx * a.ny;
    const int64_t base = (AXIS == 1 ? o * plane_ : o * a.nx) + x0;
    const int64_t stride = AXIS == 1 ? a.nx : plane_;
    const int64_t Ns = plane_ * a.nz;
    const R* src[2] = {static_cast<const R*>(a.lap), static_cast<const R*>(a.pi)};
    constexpr int chunks = (NF == 2 ? 2 : 1) * N * CPR;
#pragma unroll
    for (int k = 0; k < T::NA; ++k) {
      for (int i = tid; i < chunks; i += T::THREADS) {
        const int f = i / (N * CPR), rem = i % (N * CPR);
        const int pos = rem / CPR, cidx = rem % CPR;
        cp16(astage + (size_t)k * T::ATILE + (size_t)f * N * W + (size_t)pos * W + cidx * VEC,
             src[k] + (int64_t)f * Ns + base + (int64_t)pos * stride + cidx * VEC);
      }
    }
    cp_commit();
  }
  // staged post-transform value (array k, real line A/B, position)
  auto staged = [&](int k, int ab, int pos) -> R {
    const R* sm = astage + (size_t)k * T::ATILE;
    if (NF == 2) return sm[(size_t)ab * N * T::W + (size_t)pos * T::W + li];
    return sm[(size_t)pos * T::W + 2 * li + ab];
  };
  for (int j = tid; j < N; j += T::THREADS) twN[j] = static_cast<const C*>(a.twN)[j];
  C* sl = fft + li * T::LSTRIDE;
  const int64_t Nsite = (int64_t)a.nx * a.ny * a.nz;
  const int64_t l = (int64_t)blockIdx.x * LINES + li;
  const bool valid = l < a.nlines;
  int64_t offA = 0, offB = 0, st = 1;
  if (valid) line_map<AXIS, NF>(l, a.nx, a.ny, Nsite, offA, offB, st);
  const R* __restrict__ phi = static_cast<const R*>(a.phi);
  const R* __restrict__ phic = static_cast<const R*>(a.phic);
  const R* __restrict__ pi = static_cast<const R*>(a.pi);
  R* __restrict__ phi_o = static_cast<R*>(a.phi_out);
  R* __restrict__ phic_o = static_cast<R*>(a.phic_out);
  R* __restrict__ pi_o = static_cast<R*>(a.pi_out);
  R* __restrict__ lap_o = static_cast<R*>(a.lap_out);
  const DevScalars* sc = a.sc;
  const R shA = (R)__ldcg(&sc->mean[0]);
  const R shB = (R)__ldcg(&sc->mean[NF == 2 ? 1 : 0]);
  const R dk2 = (R)a.dk2;
  using Acc = typename AccOf<R>::type;
  Acc ge;
  R vr[Q], vi[Q];

  if constexpr (AXIS == 0) {
    double a0 = 1.0;
    R cd = (R)a.hd;
    if (a.conf) {
      a0 = __ldcg(&sc->a);
      cd = (R)(a.hd / (a0 * a0));
    }
    const bool drift = a.hd != 0.0;
    Acc ke, pe, mA, mB;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      const int64_t pos = t + P * q;
      R zr = R(0), zi = R(0);
      if (valid) {
        const int64_t sA = offA + pos * st, sB = offB + pos * st;
        R fA = phi[sA], fB = phi[sB];
        R cA = R(0), cB = R(0);
        if (KAHAN) { cA = phic[sA]; cB = phic[sB]; }
        if (drift) {
          const R pA = pi[sA], pB = pi[sB];
          if constexpr (KAHAN) {
            kahan_add(fA, cA, cd * pA);
            kahan_add(fB, cB, cd * pB);
          } else {
            fA = fA + cd * pA;
            fB = fB + cd * pB;
          }
          if (a.conf) ke.add(pA * pA + pB * pB);
        }
        phi_o[sA] = fA;
        phi_o[sB] = fB;
        if (KAHAN) {
          phic_o[sA] = cA;
          phic_o[sB] = cB;
        }
        if (a.conf) {
          if constexpr (NF == 2) {
            R ff[2] = {fA, fB};
            pe.add(model_v<R, 2>(a.model, ff));
          } else {
            R f1[1] = {fA}, f2[1] = {fB};
            pe.add(model_v<R, 1>(a.model, f1) + model_v<R, 1>(a.model, f2));
          }
        }
        mA.add(fA);
        mB.add(fB);
        zr = (fA - shA) - cA;
        zi = (fB - shB) - cB;
      }
      vr[q] = zr;
      vi[q] = zi;
    }
    __syncthreads();  // twiddle table
    d2_line<N, R, C>(vr, vi, t, sl, twN, dk2, ge);
    if (valid) {
#pragma unroll
      for (int q = 0; q < Q; ++q) {
        const int64_t pos = t + P * q;
        lap_o[offA + pos * st] = vr[q];
        lap_o[offB + pos * st] = vi[q];
      }
    }
    const typename Acc::Red vals[5] = {ke.red(), pe.red(), ge.red(), mA.red(), mB.red()};
    double tot[5];
    if (grid_reduce<5>(vals, a.rb, tot)) {
      DevScalars* w = a.sc;
      if (a.conf) {
        w->ap = w->ap + a.hd * (tot[0] / a.Nd) / (a0 * a0 * a0);
        w->pe = tot[1] / a.Nd;
        if (drift) w->ke2 = tot[0];
      }
      w->gsum[0] = tot[2];
      if (NF == 2) {
        w->mean[0] = tot[3] / a.Nd;
        w->mean[1] = tot[4] / a.Nd;
      } else {
        w->mean[0] = (tot[3] + tot[4]) / a.Nd;
      }
      if (bad(tot[0]) || bad(tot[1]) || bad(tot[2])) w->err |= 1u;
    }
  } else {
    R hA[Q], hB[Q];  // Z: phi - c of the sites, for the potential
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      const int64_t pos = t + P * q;
      R zr = R(0), zi = R(0);
      if (valid) {
        const int64_t sA = offA + pos * st, sB = offB + pos * st;
        const R fA = phi[sA], fB = phi[sB];
        R cA = R(0), cB = R(0);
        if (KAHAN) { cA = phic[sA]; cB = phic[sB]; }
        zr = (fA - shA) - cA;
        zi = (fB - shB) - cB;
        if (AXIS == 2) {
          hA[q] = fA - cA;
          hB[q] = fB - cB;
        }
      }
      vr[q] = zr;
      vi[q] = zi;
    }
    __syncthreads();  // twiddle table
    d2_line<N, R, C>(vr, vi, t, sl, twN, dk2, ge);
    cp_wait_all();  // the staged lap (and pi)
    __syncthreads();
    if constexpr (AXIS == 1) {
      if (valid) {
#pragma unroll
        for (int q = 0; q < Q; ++q) {
          const int pos = t + P * q;
          lap_o[offA + (int64_t)pos * st] = staged(0, 0, pos) + vr[q];
          lap_o[offB + (int64_t)pos * st] = staged(0, 1, pos) + vi[q];
        }
      }
      if (a.conf) {
        const typename Acc::Red vals[1] = {ge.red()};
        double tot[1];
        if (grid_reduce<1>(vals, a.rb, tot)) a.sc->gsum[1] = tot[0];
      }
    } else {
      double a0 = 1.0, ap0 = 0.0, a1 = 1.0;
      R ck = (R)a.hk, cv = (R)a.hk;
      if (a.conf) {
        a0 = __ldcg(&sc->a);
        ap0 = __ldcg(&sc->ap);
        a1 = a0 - a.hg * ap0 / 6.0;  // Hamiltonian_grav_kinetic before the kick
        ck = (R)(a.hk * a1 * a1);
        cv = (R)(a.hk * a1 * a1 * a1 * a1);
      }
      if (valid) {
#pragma unroll
        for (int q = 0; q < Q; ++q) {
          const int pos = t + P * q;
          const int64_t sA = offA + (int64_t)pos * st, sB = offB + (int64_t)pos * st;
          const R lA = staged(0, 0, pos) + vr[q], lB = staged(0, 1, pos) + vi[q];
          R dvA, dvB;
          if constexpr (NF == 2) {
            R ff[2] = {hA[q], hB[q]}, dv[2];
            model_dv<R, 2>(a.model, ff, dv);
            dvA = dv[0];
            dvB = dv[1];
          } else {
            R f1[1] = {hA[q]}, f2[1] = {hB[q]}, d1[1], d2[1];
            model_dv<R, 1>(a.model, f1, d1);
            model_dv<R, 1>(a.model, f2, d2);
            dvA = d1[0];
            dvB = d2[0];
          }
          pi_o[sA] = staged(1, 0, pos) + (ck * lA - cv * dvA);
          pi_o[sB] = staged(1, 1, pos) + (ck * lB - cv * dvB);
        }
      }
      if (a.conf) {
        const typename Acc::Red vals[1] = {ge.red()};
        double tot[1];
        if (grid_reduce<1>(vals, a.rb, tot)) {
          DevScalars* w = a.sc;
          const double GE2 = (w->gsum[0] + w->gsum[1] + tot[0]) / (a1 * a1) / a.Nd;
          const double PE = w->pe;
          const double ap1 = ap0 - a1 * a1 * a1 * (GE2 + 4.0 * PE) * a.hk;  // kick's ysclp update
          w->gsum[2] = tot[0];
          w->ap = ap1;
          w->a = a1 - a.hg * ap1 / 6.0;  // second Hamiltonian_grav_kinetic
          if (bad(GE2)) w->err |= 1u;
        }
      }
    }
  }
}

template <typename R, int NF, int AXIS, int N, bool KAHAN>
int sep_go(const SepArgs& a, cudaStream_t s) {
  using T = Tile<R, NF, AXIS, N>;
  const size_t smem = T::SMEM;
  auto k = sep_kernel<R, NF, AXIS, N, KAHAN>;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_fail(e, "separable pass smem attribute");
  }
  if (AXIS != 0 && a.nx % T::W) return set_error(LAT_ERR_STATE, "separable pass: nx not a multiple of the column block");
  const int64_t grid = (a.nlines + T::LINES - 1) / T::LINES;
  k<<<(unsigned int)grid, T::THREADS, smem, s>>>(a);
  if (g_launch_counter) ++*g_launch_counter;
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? LAT_OK : cuda_fail(e, "separable pass launch");
}

template <int N>
int sep_dispatch(const SepArgs& a, int precision, int axis, cudaStream_t s) {
#define LAT_SEP_AX(R, NF, K)                                    \
  switch (axis) {                                                \
    case 0: return sep_go<R, NF, 0, N, K>(a, s);                \
    case 1: return sep_go<R, NF, 1, N, K>(a, s);                \
    default: return sep_go<R, NF, 2, N, K>(a, s);               \
  }
  if (precision == LAT_FP64) {
    if (a.nf == 1) { LAT_SEP_AX(double, 1, false) }
    else { LAT_SEP_AX(double, 2, false) }
  } else {
    if (a.nf == 1) { LAT_SEP_AX(float, 1, true) }
    else { LAT_SEP_AX(float, 2, true) }
  }
#undef LAT_SEP_AX
}

// real x-columns one block of a y or z pass covers (nx must be a multiple)
template <int N>
int sep_columns(int precision, int nf) {
  if (precision == LAT_FP64) return nf == 2 ? Tile<double, 2, 2, N>::W : Tile<double, 1, 2, N>::W;
  return nf == 2 ? Tile<float, 2, 2, N>::W : Tile<float, 1, 2, N>::W;
}

// number of complex lines of a pass along `axis`
inline int64_t sep_lines(int axis, int nf, int nx, int ny, int nz) {
  const int64_t pairs = nf == 2 ? 1 : 2;
  if (axis == 0) return (int64_t)ny * nz / pairs;
  if (axis == 1) return (int64_t)nx * nz / pairs;
  return (int64_t)nx * ny / pairs;
}

}  // namespace sep

}  // namespace lat
