// k_sep_stream.cuh -- streamed separable spectral passes for two FP32 fields.
//
// Same arithmetic as sep_kernel (k_sep.cuh: passes X, Y, Z of the spectral
// Laplacian of laplacian_3d, Pseudospec/openmp_dev/fftw_mod.f90:177-207, with
// the drift and kick of hamiltonian_conformal.f90:92-174 fused in), organised
// for latency hiding instead of occupancy:
//
// * one persistent block of 256 threads per SM walks its share of the tiles
//   (LINES complex lines each);
// * every input of a tile is copied into shared memory by cp.async, issued
//   one or two tiles ahead, so HBM reads stay in flight while the block runs
//   the line transforms of the current tile;
// * a tile's early inputs (the transform input; in X also the momenta of the
//   drift) and late inputs (Y: lap; Z: lap and pi, used after the transform)
//   are separate loads in a ring of slots, and the slot whose early inputs
//   were just read serves as the transform's transpose scratch before it is
//   refilled.
//
// The ring keeps a fixed number of cp.async groups in flight (an empty group
// is committed past the last tile), so every wait is wait_group(SLOTS - 1).
#pragma once
#include "k_sep.cuh"

namespace lat {
namespace sep {

template <int K> __device__ __forceinline__ void cp_wait_keep() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(K) : "memory");
}

template <int AXIS, int N>
struct STile {
  static constexpr int P = Split<N>::P, Q = Split<N>::Q;
  static constexpr int THREADS = 256, LINES = THREADS / P;
  // X: one staged row per line (padded by P floats so the 32/P lines of a
  // warp start in different banks); Y, Z: one row of LINES x-columns per
  // position along the line
  static constexpr int RS = AXIS == 0 ? N + P : LINES;
  static constexpr int ROWS = AXIS == 0 ? LINES : N;
  static constexpr int ARR = ROWS * RS;  // floats per staged array
  static constexpr int N_EARLY = AXIS == 0 ? 6 : 4;  // X: phi, c, pi of both fields; Y, Z: phi, c
  static constexpr int N_LATE = AXIS == 0 ? 0 : (AXIS == 1 ? 2 : 4);  // Y: lap; Z: lap, pi
  static constexpr int LPT = N_LATE ? 2 : 1;  // loads per tile
  static constexpr int SLOTS = LPT == 1 ? 2 : 3;
  static constexpr int SLOT = N_EARLY * ARR;  // floats per slot
  static constexpr int LSTRIDE = Tile<float, 2, AXIS, N>::LSTRIDE;
  static constexpr int SMEM = SLOTS * SLOT * 4 + N * 8;
  static_assert(LINES * LSTRIDE * 8 <= SLOT * 4, "transform scratch must fit in a slot");
  static_assert(RS % 4 == 0 && (AXIS != 0 || N % 4 == 0), "staged rows must hold whole 16-byte copies");
  static_assert(SMEM <= 220 * 1024, "ring must fit in shared memory");
};

// Copy one load of tile `tile` (part 0: early inputs, 1: late inputs) into a
// slot with 16-byte cp.async copies spread over the block.  Every array of a
// load is 64 Q copies; thread tid always copies chunk tid % CPR of rows
// tid / CPR + j * (THREADS / CPR), so its addresses are one base per array
// plus compile-time steps.
template <int AXIS, int N>
__device__ __forceinline__ void stage_load(const SepArgs& a, float* dst, int64_t tile, int part, int tid) {
  using T = STile<AXIS, N>;
  constexpr int CPR = (AXIS == 0 ? N : T::RS) / 4;  // 16-byte chunks per staged row
  constexpr int PER = T::ROWS * CPR, STEPS = PER / T::THREADS, RPJ = T::THREADS / CPR;
  static_assert(PER % T::THREADS == 0 && T::THREADS % CPR == 0, "copies must tile the block");
  const int64_t Ns = (int64_t)a.nx * a.ny * a.nz;
  const int row0 = tid / CPR, ch = tid % CPR;
  const int64_t l0 = tile * T::LINES;
  int64_t src0, stride;
  if constexpr (AXIS == 0) {
    src0 = (l0 + row0) * a.nx + ch * 4;  // rows = lines l0 .. l0 + LINES - 1
    stride = a.nx;
  } else {
    const int64_t plane = (int64_t)a.nx * a.ny;
    const int64_t x0 = l0 % a.nx, o = l0 / a.nx;
    stride = AXIS == 1 ? a.nx : plane;
    src0 = (AXIS == 1 ? o * plane : o * a.nx) + x0 + row0 * stride + ch * 4;
  }
  const int64_t jstep = RPJ * stride;
  float* d0 = dst + row0 * T::RS + ch * 4;
  // arrays: X [field][phi, c, pi]; early [field][phi, c]; late Y [field][lap], late Z [field][lap, pi]
  constexpr int NA = AXIS == 0 ? 6 : (T::N_EARLY > T::N_LATE ? T::N_EARLY : T::N_LATE);
  const int narr = AXIS == 0 ? 6 : (part == 0 ? T::N_EARLY : T::N_LATE);
  const int per_f = AXIS == 0 ? 3 : (part == 0 ? 2 : T::N_LATE / 2);
#pragma unroll
  for (int arr = 0; arr < NA; ++arr) {
    if (arr < narr) {
      const int f = arr / per_f, k = arr % per_f;
      const void* sp = AXIS == 0 ? (k == 0 ? a.phi : (k == 1 ? a.phic : a.pi))
                                 : (part == 0 ? (k == 0 ? a.phi : a.phic) : (k == 0 ? a.lap : a.pi));
      const float* src = static_cast<const float*>(sp) + f * Ns + src0;
      float* d = d0 + arr * T::ARR;
#pragma unroll
      for (int j = 0; j < STEPS; ++j) cp16(d + j * RPJ * T::RS, src + j * jstep);
    }
  }
}

template <int AXIS, int N>
__global__ void __launch_bounds__(256, 1) sep_stream_kernel(const __grid_constant__ SepArgs a) {
  using T = STile<AXIS, N>;
  constexpr int P = T::P, Q = T::Q, LINES = T::LINES, S = T::SLOTS, LPT = T::LPT;
  extern __shared__ __align__(16) unsigned char smraw[];
  float* slots = reinterpret_cast<float*>(smraw);
  float2* twN = reinterpret_cast<float2*>(slots + S * T::SLOT);
  const int tid = threadIdx.x;
  const int t = AXIS == 0 ? tid % P : tid / LINES;
  const int li = AXIS == 0 ? tid / P : tid % LINES;
  const int64_t ntiles = a.nlines / LINES;
  const int64_t my = ntiles > (int64_t)blockIdx.x ? (ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
  auto issue = [&](int64_t k) {
    const int64_t j = k / LPT;
    if (j < my) stage_load<AXIS, N>(a, slots + (k % S) * T::SLOT, (int64_t)blockIdx.x + j * gridDim.x,
                                    (int)(k % LPT), tid);
    cp_commit();
  };
#pragma unroll
  for (int k = 0; k < S; ++k) issue(k);
  for (int j = tid; j < N; j += T::THREADS) twN[j] = static_cast<const float2*>(a.twN)[j];

  const int64_t Nsite = (int64_t)a.nx * a.ny * a.nz;
  const int64_t plane = (int64_t)a.nx * a.ny;
  float* __restrict__ phi_o = static_cast<float*>(a.phi_out);
  float* __restrict__ phic_o = static_cast<float*>(a.phic_out);
  float* __restrict__ pi_o = static_cast<float*>(a.pi_out);
  float* __restrict__ lap_o = static_cast<float*>(a.lap_out);
  const DevScalars* sc = a.sc;
  const float shA = (float)__ldcg(&sc->mean[0]);
  const float shB = (float)__ldcg(&sc->mean[1]);
  const float dk2 = (float)a.dk2;
  KSum ge, ke, pe, mA, mB;
  // X: drift coefficient; Z: kick coefficients after Hamiltonian_grav_kinetic
  double a0 = 1.0, ap0 = 0.0, a1 = 1.0;
  float cd = (float)a.hd, ck = (float)a.hk, cv = (float)a.hk;
  const bool drift = a.hd != 0.0;
  if (a.conf) {
    a0 = __ldcg(&sc->a);
    ap0 = __ldcg(&sc->ap);
    if (AXIS == 0) cd = (float)(a.hd / (a0 * a0));
    if (AXIS == 2) {
      a1 = a0 - a.hg * ap0 / 6.0;
      ck = (float)(a.hk * a1 * a1);
      cv = (float)(a.hk * a1 * a1 * a1 * a1);
    }
  }

  for (int64_t j = 0; j < my; ++j) {
    const int64_t k = j * LPT;
    const int64_t l = ((int64_t)blockIdx.x + j * gridDim.x) * LINES + li;
    float* es = slots + (k % S) * T::SLOT;
    cp_wait_keep<S - 1>();
    __syncthreads();
    float vr[Q], vi[Q];
    float hA[AXIS == 2 ? Q : 1], hB[AXIS == 2 ? Q : 1];
    int64_t offA, st;
    if constexpr (AXIS == 0) {
      offA = l * a.nx;
      st = 1;
    } else {
      const int64_t x = l % a.nx, o = l / a.nx;
      offA = (AXIS == 1 ? o * plane : o * a.nx) + x;
      st = AXIS == 1 ? a.nx : plane;
    }
    const int64_t offB = Nsite + offA;
    auto at = [&](const float* sl, int arr, int pos) -> float {
      return AXIS == 0 ? sl[arr * T::ARR + li * T::RS + pos] : sl[arr * T::ARR + pos * T::RS + li];
    };
    float kes = 0.f, pes = 0.f, mAs = 0.f, mBs = 0.f;  // this line's sums, folded into KSum once
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      const int pos = t + P * q;
      if constexpr (AXIS == 0) {
        float fA = at(es, 0, pos), cA = at(es, 1, pos);
        float fB = at(es, 3, pos), cB = at(es, 4, pos);
        if (drift) {
          const float pA = at(es, 2, pos), pB = at(es, 5, pos);
          kahan_add(fA, cA, cd * pA);
          kahan_add(fB, cB, cd * pB);
          if (a.conf) kes += pA * pA + pB * pB;
        }
        phi_o[offA + pos] = fA;
        phi_o[offB + pos] = fB;
        phic_o[offA + pos] = cA;
        phic_o[offB + pos] = cB;
        if (a.conf) {
          float ff[2] = {fA, fB};
          pes += model_v<float, 2>(a.model, ff);
        }
        mAs += fA;
        mBs += fB;
        vr[q] = (fA - shA) - cA;
        vi[q] = (fB - shB) - cB;
      } else {
        const float fA = at(es, 0, pos), cA = at(es, 1, pos);
        const float fB = at(es, 2, pos), cB = at(es, 3, pos);
        vr[q] = (fA - shA) - cA;
        vi[q] = (fB - shB) - cB;
        if constexpr (AXIS == 2) {
          hA[q] = fA - cA;
          hB[q] = fB - cB;
        }
      }
    }
    if constexpr (AXIS == 0) {
      ke.add(kes);
      pe.add(pes);
      mA.add(mAs);
      mB.add(mBs);
    }
    __syncthreads();  // the slot becomes the transform scratch
    d2_line<N, float, float2>(vr, vi, t, reinterpret_cast<float2*>(es) + li * T::LSTRIDE, twN, dk2, ge);
    __syncthreads();
    issue(k + S);  // refill the slot
    if constexpr (AXIS == 0) {
#pragma unroll
      for (int q = 0; q < Q; ++q) {
        const int pos = t + P * q;
        lap_o[offA + pos] = vr[q];
        lap_o[offB + pos] = vi[q];
      }
    } else {
      const float* ls = slots + ((k + 1) % S) * T::SLOT;
      cp_wait_keep<S - 1>();
      __syncthreads();
#pragma unroll
      for (int q = 0; q < Q; ++q) {
        const int pos = t + P * q;
        const int64_t sA = offA + (int64_t)pos * st, sB = offB + (int64_t)pos * st;
        if constexpr (AXIS == 1) {
          lap_o[sA] = at(ls, 0, pos) + vr[q];
          lap_o[sB] = at(ls, 1, pos) + vi[q];
        } else {
          const float lA = at(ls, 0, pos) + vr[q], lB = at(ls, 2, pos) + vi[q];
          float ff[2] = {hA[q], hB[q]}, dv[2];
          model_dv<float, 2>(a.model, ff, dv);
          pi_o[sA] = at(ls, 1, pos) + (ck * lA - cv * dv[0]);
          pi_o[sB] = at(ls, 3, pos) + (ck * lB - cv * dv[1]);
        }
      }
      __syncthreads();
      issue(k + 1 + S);
    }
  }
  cp_wait_all();

  if constexpr (AXIS == 0) {
    double vals[5] = {ke.val(), pe.val(), ge.val(), mA.val(), mB.val()}, tot[5];
    if (grid_reduce<5>(vals, a.rb, tot)) {
      DevScalars* w = a.sc;
      if (a.conf) {
        w->ap = w->ap + a.hd * (tot[0] / a.Nd) / (a0 * a0 * a0);
        w->pe = tot[1] / a.Nd;
        if (drift) w->ke2 = tot[0];
      }
      w->gsum[0] = tot[2];
      w->mean[0] = tot[3] / a.Nd;
      w->mean[1] = tot[4] / a.Nd;
      if (bad(tot[0]) || bad(tot[1]) || bad(tot[2])) w->err |= 1u;
    }
  } else if constexpr (AXIS == 1) {
    if (a.conf) {
      double vals[1] = {ge.val()}, tot[1];
      if (grid_reduce<1>(vals, a.rb, tot)) a.sc->gsum[1] = tot[0];
    }
  } else {
    if (a.conf) {
      double vals[1] = {ge.val()}, tot[1];
      if (grid_reduce<1>(vals, a.rb, tot)) {
        DevScalars* w = a.sc;
        const double GE2 = (w->gsum[0] + w->gsum[1] + tot[0]) / (a1 * a1) / a.Nd;
        const double ap1 = ap0 - a1 * a1 * a1 * (GE2 + 4.0 * w->pe) * a.hk;
        w->gsum[2] = tot[0];
        w->ap = ap1;
        w->a = a1 - a.hg * ap1 / 6.0;
        if (bad(GE2)) w->err |= 1u;
      }
    }
  }
}

// Launch of the streamed pass: one block per SM (fewer when there are fewer
// tiles).  Returns LAT_ERR_UNSUPPORTED (nothing launched) when the lines do
// not form whole tiles.
template <int AXIS, int N>
int sep_stream_go(const SepArgs& a, cudaStream_t s) {
  using T = STile<AXIS, N>;
  if (a.nf != 2 || a.nlines % T::LINES || (AXIS != 0 && a.nx % T::LINES)) return LAT_ERR_UNSUPPORTED;
  auto k = sep_stream_kernel<AXIS, N>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, T::SMEM);
  if (e != cudaSuccess) return cuda_fail(e, "streamed separable pass smem attribute");
  const int64_t ntiles = a.nlines / T::LINES;
  const int grid = (int)(ntiles < a.nsm ? ntiles : a.nsm);
  k<<<grid, T::THREADS, T::SMEM, s>>>(a);
  if (g_launch_counter) ++*g_launch_counter;
  e = cudaGetLastError();
  return e == cudaSuccess ? LAT_OK : cuda_fail(e, "streamed separable pass launch");
}

template <int N>
int sep_stream_dispatch(const SepArgs& a, int axis, cudaStream_t s) {
  switch (axis) {
    case 0: return sep_stream_go<0, N>(a, s);
    case 1: return sep_stream_go<1, N>(a, s);
    default: return sep_stream_go<2, N>(a, s);
  }
}

}  // namespace sep
}  // namespace lat
