// k_sep_stream.cuh -- streamed separable spectral passes for pairs of FP32 lines.
//
// The spectral Laplacian of laplacian_3d (Pseudospec/openmp_dev/fftw_mod.f90:
// 177-207) is the sum of one-dimensional second derivatives along x, y and z
// (k_sep.cuh).  For two FP32 fields (or, in ensembles, two independent
// one-field runs of one size) the engine runs the three passes of a drift +
// kick in this form, line A and line B forming one complex line:
//
//   pass X: drift of phi (Kahan), z = (phi - shift) - c written as the FP32
//           array zs (lines A and B interleaved),
//           pi += ck d2x(z) - cv V'(z + shift)               [PE, GEx, means]
//   pass Y: pi += ck d2y(zs)                                 [GEy]
//   pass Z: pi += ck d2z(zs)                                 [GEz, sum pi^2]
//
// with ck = hk a1^2, cv = hk a1^4, a1 = a - hg ysclp / 6 after the drift's
// ysclp += hd sum(pi^2)/N / a^3 (hamiltonian_conformal.f90:86-174).  The
// potential force belongs to the pass that holds the drifted fields in
// registers (X, whose loads leave issue slots free); evaluated in pass Z it
// cost that pass 32 registers of z + shift and 9 us of its 78 us at 256^3.
// The momenta accumulate the kick pass by pass, so no Laplacian array is kept:
// per line and kick the passes move 28 + 12 + 12 bytes per site.  Pass X
// needs ck before it has seen all momenta, so sum pi^2 comes from the pass Z
// of the previous kick (or one reduction before the first pass X of a call,
// which also takes the fields' means: the first kick's shifts).
// The passes only write per-block partial sums; one single-block kernel after
// pass Z (launch_sep_finalize) completes them in block order and advances
// the scale factor, so no pass ends on a grid-wide arrival counter and the
// scalar block holds the pre-kick state for all three passes.
// Two fields use the lattice means as shifts; pairs of runs (Minkowski) use
// each run's phi at site 0 as it was after the previous kick.
//
// Blocks are persistent.  A block reads the inputs of its tile from shared
// memory into registers, refills the slot with the next tile's inputs at
// once, and runs the line transforms in a separate scratch, so the next
// tile's HBM reads are in flight during the transforms.  Pass X: 128 threads
// per block; every warp stages (cp.async) and transforms its own lines with
// warp barriers only.  Passes Y, Z: 32 x-columns per block (128-byte rows of
// momenta: at 16 columns the strided 64-byte rows ran both passes 4-6%
// slower), with a second slot for the momenta, which are needed only after
// the transform; each slot is filled by one TMA tensor copy (zs: a 4D box,
// the momenta of both lines: one 5D box) issued by one thread and counted on
// an mbarrier.  Every
// update of a tile is written by the block that read it, so the passes also
// run in place.
//
// The two-field chain X, Y, Z, finalize (pairs of runs: Y, Z) is launched
// with programmatic dependent launch: each pass starts while its predecessor drains and waits
// (griddepcontrol.wait) only before reading what the predecessor writes.
// Pass X stages its whole first tile early (phi and c were last written by
// the previous pass X, the momenta by the previous pass Z, both complete
// before its predecessor let it start), pass Z its first zs tile and that
// tile's transform (zs comes from pass X; pass Y writes only the momenta).
// Y and Z wait on each slot's mbarrier per thread and take four block
// barriers per tile (two release the slots, two order the transposes).
// The passes load the
// kick's FP32 coefficients (cd, ck, cv: kick_coefs_of) from the scalar block,
// where the single-block kernel before pass X (the previous kick's finalize,
// or the momentum sum that starts a call) left them: at GB300's FP64 rate the
// coefficient chain, evaluated per thread, had cost pass Z 13 us of its 92 us
// at 256^3, and evaluated once per warp (X) or block (Y, Z) it still held
// each pass's start, 23.5 us per Yoshida-4 step.
#pragma once
#include "k_sep.cuh"

namespace lat {
namespace sep {

template <int K> __device__ __forceinline__ void cp_wait_keep() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(K) : "memory");
}

// Spectral second derivative of one complex line, as d2_line (k_sep.cuh) but
// with per-block tables instead of per-point index arithmetic:
// tf[kq * P + t] = W_N^{t kq} and ti[mp * Q + kq] = W_N^{mp kq} (the same
// table when P == Q), fk[k] = -(f dk)^2 / N for wavenumber index k.  Every table
// read is the thread's base plus a compile-time offset.  WARP: the P threads
// of every line sit in one warp, so the transposes need only warp barriers.
// GE: add the axis' Parseval sum (f dk)^2 |Z_k|^2 / N to `ge` (only an
// expanding background needs it).
template <int N, bool WARP, bool GE, typename Acc>
__device__ __forceinline__ void d2_line_tab(float (&re)[Split<N>::Q], float (&im)[Split<N>::Q], int t, float2* sl,
                                            const float2* tf, const float2* ti, const float* fk, Acc& ge) {
  // G rows kq = t + g P of the transposed line per thread; when P does not
  // divide Q (96 = 8 x 12, 192 = 16 x 12) the last row group covers only
  // kq < Q and the threads past it sit out the middle phase
  constexpr int P = Split<N>::P, Q = Split<N>::Q, G = (Q + P - 1) / P, S = P + 1;
  auto sync = [] {
    if (WARP) __syncwarp();
    else __syncthreads();
  };
  dft<Q, false, float>(re, im);
  const float2* tft = tf + t;
  sl[t] = make_float2(re[0], im[0]);  // kq = 0: W_N^0 = 1 on every thread
#pragma unroll
  for (int kq = 1; kq < Q; ++kq) {
    const float2 w = tft[kq * P];
    const float xr = re[kq], xi = im[kq];
    sl[kq * S + t] = make_float2(xr * w.x - xi * w.y, xr * w.y + xi * w.x);
  }
  sync();
  float ur[G][P], ui[G][P];
#pragma unroll
  for (int g = 0; g < G; ++g) {
    const int kq = t + g * P;
    if (Q % P != 0 && kq >= Q) break;  // (uniform per thread: the last group)
#pragma unroll
    for (int tt = 0; tt < P; ++tt) {
      const float2 z = sl[kq * S + tt];
      ur[g][tt] = z.x;
      ui[g][tt] = z.y;
    }
    dft<P, false, float>(ur[g], ui[g]);
    const float* fkk = fk + kq;  // k = kq + Q kp; fk holds -(f dk)^2 / N
    float gp[4] = {0.f, 0.f, 0.f, 0.f};  // four independent partial sums
#pragma unroll
    for (int kp = 0; kp < P; ++kp) {
      const float h = fkk[Q * kp];
      const float zr = ur[g][kp], zi = ui[g][kp];
      if (GE) gp[kp % 4] += h * (zr * zr + zi * zi);
      ur[g][kp] = zr * h;
      ui[g][kp] = zi * h;
    }
    if (GE) ge.add(-((gp[0] + gp[1]) + (gp[2] + gp[3])));
    dft<P, true, float>(ur[g], ui[g]);
  }
  // no barrier here: rows kq = t + g P are read and rewritten by thread t
  // alone; the next barrier orders them before the column reads
#pragma unroll
  for (int g = 0; g < G; ++g) {
    const int kq = t + g * P;
    if (Q % P != 0 && kq >= Q) break;
    const float2* tik = ti + kq;
    sl[kq * S] = make_float2(ur[g][0], ui[g][0]);  // mp = 0: W_N^0 = 1 on every thread
#pragma unroll
    for (int mp = 1; mp < P; ++mp) {
      const float2 w = tik[mp * Q];
      const float xr = ur[g][mp], xi = ui[g][mp];
      sl[kq * S + mp] = make_float2(xr * w.x + xi * w.y, xi * w.x - xr * w.y);  // times conj(W_N^{mp kq})
    }
  }
  sync();
#pragma unroll
  for (int kq = 0; kq < Q; ++kq) {
    const float2 z = sl[kq * S + t];
    re[kq] = z.x;
    im[kq] = z.y;
  }
  dft<Q, true, float>(re, im);
}

// Build the tables of d2_line_tab from W_N^j (global) in shared memory:
// tf, ti as above, fk[k] = -(f dk)^2 / N.
template <int N>
__device__ __forceinline__ void build_tables(const float2* twN, float dk2, float2* tf, float2* ti, float* fk, int tid,
                                             int nthreads) {
  constexpr int P = Split<N>::P, Q = Split<N>::Q;
  for (int j = tid; j < P * Q; j += nthreads) {
    tf[j] = twN[((j % P) * (j / P)) % N];
    if (P != Q) ti[j] = twN[((j / Q) * (j % Q)) % N];
  }
  for (int k = tid; k < N; k += nthreads) {  // the multiplier of the second derivative, with the 1/N
    const int f = k <= N / 2 ? k : k - N;
    fk[k] = -((float)(f * f) * dk2) * (1.0f / N);
  }
}

template <int AXIS, int N>
struct STile {
  static constexpr int P = Split<N>::P, Q = Split<N>::Q;
  static constexpr int LINES_YZ = 32;  // x-columns of a Y, Z tile (128-byte rows of momenta)
  static constexpr int THREADS = AXIS == 0 ? 128 : P * LINES_YZ, LINES = THREADS / P;
  // X: one staged row per line (padded by P floats so the 32/P lines of a
  // warp start in different banks); Y, Z: one row of LINES x-columns per
  // position along the line
  static constexpr int RS = AXIS == 0 ? N + P : LINES;
  static constexpr int ROWS = AXIS == 0 ? LINES : N;
  static constexpr int ARR = ROWS * RS;               // floats per staged array
  static constexpr int N_EARLY = AXIS == 0 ? 6 : 2;   // X: phi, c, pi of both lines; Y, Z: zs (float2 rows)
  static constexpr int N_LATE = AXIS == 0 ? 0 : 2;    // Y, Z: pi of both lines
  // transpose scratch per line, in complex: Q rows of P + 1, padded so the
  // lines a warp touches at once start in different banks
  static constexpr int LANES = AXIS == 0 ? P : (32 / LINES > 0 ? 32 / LINES : 1);
  static constexpr int LINE_WORDS = LANES * 2 >= 32 ? 0 : LANES * 2;
  static constexpr int lstride_for(int pad) {
    return ((Q * (P + 1) + pad) * 2) % 32 == LINE_WORDS ? Q * (P + 1) + pad : lstride_for(pad + 1);
  }
  static constexpr int LSTRIDE = lstride_for(0);
  static constexpr int E_OFF = 0, L_OFF = N_EARLY * ARR, S_OFF = L_OFF + N_LATE * ARR;  // floats
  static constexpr int TF_OFF = S_OFF + LINES * LSTRIDE * 2;  // twiddle tables W_N^{t kq}, W_N^{mp kq}
  static constexpr int TI_OFF = P == Q ? TF_OFF : TF_OFF + 2 * N;
  static constexpr int FK_OFF = TI_OFF + 2 * N;                   // (f dk)^2
  static constexpr int SMEM = (FK_OFF + N) * 4;
  // blocks per SM: dynamic and static (block partials) shared memory plus
  // the 1 KB the SM reserves per block, within 228 KB; at most 3
  static constexpr int PER_BLOCK = SMEM + 1300 + 1024;
  static constexpr int MINB = (228 * 1024) / PER_BLOCK > 3 ? 3 : (228 * 1024) / PER_BLOCK;
  static_assert(MINB >= 1, "a block must fit in shared memory");
  static_assert(RS % 4 == 0 && N % 4 == 0, "staged rows must hold whole 16-byte copies");
};


// ------------------------------------------------ tensor memory access (TMA)
// One thread issues a tile copy described by a tensor map; completion is
// counted in bytes on an mbarrier that every consumer waits on.
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait for the phase of `parity`: false if it did not complete
// within the limit (the caller records the timeout and leaves).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  for (uint32_t i = 0; i < (1u << 22); ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1, int c2,
                                            int c3) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
      "[%6];\n" ::"r"(smem_u32(dst)),
      "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tma_load_5d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1, int c2,
                                            int c3, int c4) {
  asm volatile(
      "cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, %6}], "
      "[%7];\n" ::"r"(smem_u32(dst)),
      "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(smem_u32(bar))
      : "memory");
}
// order this thread's generic-proxy shared-memory accesses before later
// async-proxy (TMA) accesses of the same memory
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

// First-line geometry of a tile: the pair it belongs to and the offset of
// line A's first site.  Two fields: one pair (pair_lines = nlines).
template <int AXIS>
__device__ __forceinline__ int64_t tile_base(const SepArgs& a, int64_t l0, int64_t& pair) {
  // 32-bit index arithmetic (the dispatch checks nlines < 2^31): 64-bit
  // divisions by the runtime extents cost more than a tile's addressing
  const uint32_t l = (uint32_t)l0;
  uint32_t p = 0, r = l;
  if (a.runs) {
    const uint32_t pl = (uint32_t)a.pair_lines;
    p = l / pl;
    r = l - p * pl;
  }
  pair = p;
  const int64_t Ns = (int64_t)a.nx * a.ny * a.nz;
  const int64_t pbase = (int64_t)p * 2 * Ns;
  if constexpr (AXIS == 0) return pbase + (int64_t)r * a.nx;
  const uint32_t nx = (uint32_t)a.nx;
  const uint32_t o = r / nx, x0 = r - o * nx;
  return pbase + (AXIS == 1 ? (int64_t)o * a.nx * a.ny : (int64_t)o * a.nx) + x0;
}

// Pass X staging by one warp: the rows of its own 32/P lines of tile `tile`
// (6 arrays: [line A, B][phi, c, pi]), so the warp waits only for its copies.
template <int N>
__device__ __forceinline__ void stage_rows_x(const SepArgs& a, float* dst, int64_t tile, int warp, int lane) {
  using T = STile<0, N>;
  constexpr int LPW = 32 / T::P, CPR = N / 4;  // lines per warp, 16-byte chunks per row
  const int64_t Ns = (int64_t)a.nx * a.ny * a.nz;
  int64_t pair;
  const int64_t r0 = tile_base<0>(a, tile * T::LINES + warp * LPW, pair);  // first site of the warp's rows
  float* d0 = dst + warp * LPW * T::RS;
#pragma unroll
  for (int arr = 0; arr < 6; ++arr) {
    const int f = arr / 3, k = arr % 3;
    const void* sp = k == 0 ? a.phi : (k == 1 ? a.phic : a.pi);
    const float* src = static_cast<const float*>(sp) + f * Ns + r0;
#pragma unroll
    for (int i = lane; i < LPW * CPR; i += 32) {
      const int r = i / CPR, c = i % CPR;
      cp16(d0 + arr * T::ARR + r * T::RS + c * 4, src + (int64_t)r * a.nx + c * 4);
    }
  }
}

// Pass X: drift, zs, the potential force and the x part of the kick.
// MODEL >= 0: the potential fixed at compile time; -1: read from the arguments.
template <int N, bool RUNS, bool CONF, int MODEL = -1>
__global__ void __launch_bounds__(STile<0, N>::THREADS, STile<0, N>::MINB)
    sep_stream_x(const __grid_constant__ SepArgs a) {
  using T = STile<0, N>;
  constexpr int P = T::P, Q = T::Q, LINES = T::LINES;
  extern __shared__ __align__(128) unsigned char smraw[];
  float* sm = reinterpret_cast<float*>(smraw);
  float* es = sm + T::E_OFF;
  float2* scr = reinterpret_cast<float2*>(sm + T::S_OFF);
  float2* tf = reinterpret_cast<float2*>(sm + T::TF_OFF);
  float2* ti = reinterpret_cast<float2*>(sm + T::TI_OFF);
  float* fk = sm + T::FK_OFF;
  const int tid = threadIdx.x, t = tid % P, li = tid / P, warp = tid / 32, lane = tid % 32;
  const int64_t ntiles = a.nlines / LINES;
  const int64_t my = ntiles > (int64_t)blockIdx.x ? (ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
  if constexpr (!RUNS) {
    // launched as a programmatic dependent of the previous kick's finalize
    // (or of the momentum sum that starts a call), which lets this pass start
    // only after its own wait for the kernel before it: phi and c (last
    // written by the previous pass X) and the momenta (previous pass Z) are
    // complete, so the whole first tile is staged while the predecessor
    // runs; the scalar block it writes is read after the wait
    if (my > 0) stage_rows_x<N>(a, es, blockIdx.x, warp, lane);
    cp_commit();
    build_tables<N>(static_cast<const float2*>(a.twN), (float)a.dk2, tf, ti, fk, tid, T::THREADS);
    pdl_wait();
    pdl_trigger();
  } else {
    if (my > 0) stage_rows_x<N>(a, es, blockIdx.x, warp, lane);
    cp_commit();
    build_tables<N>(static_cast<const float2*>(a.twN), (float)a.dk2, tf, ti, fk, tid, T::THREADS);
  }
  __syncthreads();  // tables; from here on every warp runs its own lines

  const int64_t Nsite = (int64_t)a.nx * a.ny * a.nz;
  float* __restrict__ phi_o = static_cast<float*>(a.phi_out);
  float* __restrict__ phic_o = static_cast<float*>(a.phic_out);
  float* __restrict__ pi_o = static_cast<float*>(a.pi_out);
  float* __restrict__ zs_o = static_cast<float*>(a.lap_out);
  const DevScalars* sc = a.sc;
  // the scalar block holds the pre-kick state until launch_sep_finalize runs
  // after pass Z; only the FP32 coefficients live through the tile loop
  float shAf = 0.f, shBf = 0.f;
  if (!RUNS) {
    shAf = (float)__ldcg(&sc->mean[0]);
    shBf = (float)__ldcg(&sc->mean[1]);
  }
  const bool drift = a.hd != 0.0;
  float cd = (float)a.hd, ck = (float)a.hk, cv = (float)a.hk;
  if (CONF) {  // the kick's coefficients, left by the kernel before it (read after the wait above)
    cd = __ldcg(&sc->co[0]);
    ck = __ldcg(&sc->co[1]);
    cv = __ldcg(&sc->co[2]);
  }
  ModelP mp = a.model;
  if constexpr (MODEL >= 0) mp.model = MODEL;
  KSum ge, pe, mA, mB;
  // pairs of runs: each run's shift is its phi at site 0 after the previous
  // kick (shift_b), loaded one tile ahead; the block holding a pair's first
  // tile passes it on to pass Z (shift_a)
  float nshA = 0.f, nshB = 0.f;
  if (RUNS && my > 0) {
    const int64_t p0 = (int64_t)blockIdx.x * LINES / a.pair_lines;
    nshA = __ldcg(a.shift_b + 2 * p0);
    nshB = __ldcg(a.shift_b + 2 * p0 + 1);
  }
  for (int64_t j = 0; j < my; ++j) {
    int64_t pair;
    const int64_t l0 = ((int64_t)blockIdx.x + j * gridDim.x) * LINES;
    const int64_t offA = tile_base<0>(a, l0 + li, pair);
    const int64_t offB = Nsite + offA;
    float2* zs2 = reinterpret_cast<float2*>(zs_o) + (offA - pair * Nsite);  // both lines, interleaved
    float shA = shAf, shB = shBf;
    if (RUNS) {
      shA = nshA;
      shB = nshB;
      if (tid == 0 && l0 % a.pair_lines == 0) {
        a.shift_a[2 * pair] = shA;
        a.shift_a[2 * pair + 1] = shB;
      }
      if (j + 1 < my) {
        const int64_t pn = (l0 + (int64_t)gridDim.x * LINES) / a.pair_lines;
        nshA = __ldcg(a.shift_b + 2 * pn);
        nshB = __ldcg(a.shift_b + 2 * pn + 1);
      }
    }
    cp_wait_keep<0>();
    __syncwarp();
    float vr[Q], vi[Q], pA[Q], pB[Q];
    // this line's sums in four independent partials each, folded into KSum once
    float pes[4] = {0.f, 0.f, 0.f, 0.f}, mAs[4] = {0.f, 0.f, 0.f, 0.f}, mBs[4] = {0.f, 0.f, 0.f, 0.f};
    const float* row = es + li * T::RS;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      const int pos = t + P * q;
      float fA = row[pos], cA = row[T::ARR + pos];
      float fB = row[3 * T::ARR + pos], cB = row[4 * T::ARR + pos];
      pA[q] = row[2 * T::ARR + pos];
      pB[q] = row[5 * T::ARR + pos];
      if (drift) {
        kahan_add(fA, cA, cd * pA[q]);
        kahan_add(fB, cB, cd * pB[q]);
      }
      phi_o[offA + pos] = fA;
      phi_o[offB + pos] = fB;
      phic_o[offA + pos] = cA;
      phic_o[offB + pos] = cB;
      if (!RUNS) {
        if (CONF) {
          float ff[2] = {fA, fB};
          pes[q % 4] += model_v<float, 2>(mp, ff);
        }
        mAs[q % 4] += fA;
        mBs[q % 4] += fB;
      }
      vr[q] = (fA - shA) - cA;
      vi[q] = (fB - shB) - cB;
      zs2[pos] = make_float2(vr[q], vi[q]);
      // the potential force at the drifted, compensated fields (zs + shift)
      float dA, dB;
      if constexpr (RUNS) {  // two independent runs: each its own potential
        float fa[1] = {vr[q] + shA}, fb[1] = {vi[q] + shB}, da[1], db[1];
        model_dv<float, 1>(mp, fa, da);
        model_dv<float, 1>(mp, fb, db);
        dA = da[0];
        dB = db[0];
      } else {
        float ff[2] = {vr[q] + shA, vi[q] + shB}, dv[2];
        model_dv<float, 2>(mp, ff, dv);
        dA = dv[0];
        dB = dv[1];
      }
      pA[q] = pA[q] - cv * dA;
      pB[q] = pB[q] - cv * dB;
    }
    if (!RUNS) {
      pe.add((pes[0] + pes[1]) + (pes[2] + pes[3]));
      mA.add((mAs[0] + mAs[1]) + (mAs[2] + mAs[3]));
      mB.add((mBs[0] + mBs[1]) + (mBs[2] + mBs[3]));
    }
    __syncwarp();  // the warp's rows are free: stage its rows of the next tile
    if (j + 1 < my) stage_rows_x<N>(a, es, (int64_t)blockIdx.x + (j + 1) * gridDim.x, warp, lane);
    cp_commit();
    d2_line_tab<N, true, CONF>(vr, vi, t, scr + li * T::LSTRIDE, tf, ti, fk, ge);
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      const int pos = t + P * q;
      pi_o[offA + pos] = pA[q] + ck * vr[q];
      pi_o[offB + pos] = pB[q] + ck * vi[q];
    }
  }
  cp_wait_all();
  if (RUNS) return;
  // this block's sums; launch_sep_finalize completes them after pass Z
  const FF vals[4] = {pe.red(), ge.red(), mA.red(), mB.red()};
  block_partials<4>(vals, a.rb.partials + SEP_PART_X);
}

// Passes Y (AXIS 1: the y part of the kick) and Z (AXIS 2: the z part, which
// completes the kick; its ysclp update follows in launch_sep_finalize; the
// potential force was added by pass X, whose fields are in registers).  A tile's zs rows (64 KB at 256 points) and both
// lines' momentum rows arrive by one TMA tensor copy each (zs: a 4D box,
// the momenta of lines A and B: one 5D box; the last dimension is the pair
// of runs, 1 for the two fields of a lattice), counted on an mbarrier per
// slot, issued by one thread; the
// updated momenta are stored from registers (128-byte rows per warp), so the
// momentum slot takes the next tile as soon as every thread has read it (a
// tensor store from the slot would hold the next copy until the store had
// read the slot, and every warp waited for that at the next barrier).  Launched as
// programmatic dependents: pass Y (after pass X, which writes zs and the
// momenta) waits before its first copy; pass Z (after pass Y, which writes
// only the momenta) loads and transforms its first zs tile while Y drains.
// A bounded mbarrier wait that gives up sets bit 1 of the scalar block's
// error word (reported as LAT_ERR_TIMEOUT) and the block leaves.
// RUNS: pairs of one-field runs, each line with its own shift (the run's phi
// at site 0 after the previous kick); pass Z hands the new site-0 values
// (zs + the shift pass X took) to the next pass X.
template <int AXIS, int N, bool RUNS, bool CONF>
__global__ void __launch_bounds__(STile<AXIS, N>::THREADS, STile<AXIS, N>::MINB)
    sep_stream_yz_tma(const __grid_constant__ SepArgs a) {
  using T = STile<AXIS, N>;
  constexpr int P = T::P, Q = T::Q, LINES = T::LINES;
  constexpr uint32_t ZS_BYTES = 2u * LINES * N * 4u;  // box {2 LINES, N} floats
  constexpr uint32_t PI_BYTES = 2u * LINES * N * 4u;  // box {LINES, N, 2 fields} floats
  static_assert(T::E_OFF == 0 && (T::L_OFF * 4) % 128 == 0, "TMA slots must be 128-byte aligned");
  extern __shared__ __align__(128) unsigned char smraw[];
  __shared__ __align__(8) uint64_t bar[2];  // [0]: zs slot, [1]: momentum slot
  // the dynamic region starts after the static variables: the slots begin at
  // its first 128-byte boundary (the launch adds 128 bytes)
  unsigned char* base = smraw + ((128u - (smem_u32(smraw) & 127u)) & 127u);
  float* sm = reinterpret_cast<float*>(base);
  float* es = sm + T::E_OFF;
  float* ls = sm + T::L_OFF;
  float2* scr = reinterpret_cast<float2*>(sm + T::S_OFF);
  float2* tf = reinterpret_cast<float2*>(sm + T::TF_OFF);
  float2* ti = reinterpret_cast<float2*>(sm + T::TI_OFF);
  float* fk = sm + T::FK_OFF;
  const int tid = threadIdx.x, t = tid / LINES, li = tid % LINES;
  const int64_t ntiles = a.nlines / LINES;
  const int my = ntiles > (int64_t)blockIdx.x ? (int)((ntiles - 1 - blockIdx.x) / gridDim.x + 1) : 0;
  // tile -> (pair, first x-column, plane index along the other axis): the
  // lines of pass Y are (x, z), those of pass Z (x, y)
  auto coords = [&](int tile, int& pr, int& x0, int& o) {
    uint32_t r = (uint32_t)tile * LINES;
    pr = 0;
    if (RUNS) {
      const uint32_t pl = (uint32_t)a.pair_lines;
      pr = (int)(r / pl);
      r -= (uint32_t)pr * pl;
    }
    const uint32_t nx = (uint32_t)a.nx;
    o = (int)(r / nx);
    x0 = (int)(r - (uint32_t)o * nx);
  };
  auto load_zs = [&](int tile) {
    int pr, x0, o;
    coords(tile, pr, x0, o);
    mbar_expect_tx(&bar[0], ZS_BYTES);
    if (AXIS == 1) tma_load_4d(es, &a.tm_zs, &bar[0], 2 * x0, 0, o, pr);
    else tma_load_4d(es, &a.tm_zs, &bar[0], 2 * x0, o, 0, pr);
  };
  auto load_pi = [&](int tile) {
    int pr, x0, o;
    coords(tile, pr, x0, o);
    mbar_expect_tx(&bar[1], PI_BYTES);
    if (AXIS == 1) tma_load_5d(ls, &a.tm_pi, &bar[1], x0, 0, o, 0, pr);
    else tma_load_5d(ls, &a.tm_pi, &bar[1], x0, o, 0, 0, pr);
  };
  const int64_t Nsite = (int64_t)a.nx * a.ny * a.nz;
  const int64_t st = AXIS == 1 ? a.nx : (int64_t)a.nx * a.ny;
  float* __restrict__ pi_o = static_cast<float*>(a.pi_out);

  if (smem_u32(base) & 127u) {  // tensor copies need 128-byte aligned slots: refuse, never misaddress
    if (tid == 0) atomicOr(&a.sc->err, 2u);
    return;
  }
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_init_fence();
  }
  __syncthreads();
  if constexpr (AXIS == 1) {
    build_tables<N>(static_cast<const float2*>(a.twN), (float)a.dk2, tf, ti, fk, tid, T::THREADS);
    pdl_wait();
    pdl_trigger();
    if (tid == 0 && my > 0) {
      load_zs(blockIdx.x);
      load_pi(blockIdx.x);
    }
  } else {
    if (tid == 0 && my > 0) load_zs(blockIdx.x);  // zs was written two kernels back (pass X)
    build_tables<N>(static_cast<const float2*>(a.twN), (float)a.dk2, tf, ti, fk, tid, T::THREADS);
  }
  const DevScalars* sc = a.sc;  // written by the finalize three kernels back
  float ck = (float)a.hk;  // static background
  if (CONF) ck = __ldcg(&sc->co[1]);  // expanding: the kick's coefficient, left by the kernel before pass X
  KSum ge, ke;
  int fail = 0;
  for (int j = 0; j < my; ++j) {
    const int tile = (int)blockIdx.x + j * (int)gridDim.x;
    const uint32_t ph = (uint32_t)(j & 1);
    int pr, x0, o;
    coords(tile, pr, x0, o);
    // every thread waits on the slot's barrier itself; the barrier that
    // releases the slot also makes a timeout the whole block's decision
    fail = !mbar_wait(&bar[0], ph);
    float vr[Q], vi[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      const int pos = t + P * q;
      const float2 z = reinterpret_cast<const float2*>(es)[pos * T::RS + li];
      vr[q] = z.x;
      vi[q] = z.y;
    }
    if constexpr (RUNS && AXIS == 2) {
      if (t == 0 && li == 0 && ((uint32_t)tile * LINES) % (uint32_t)a.pair_lines == 0) {
        // site 0 of both runs of the pair (zs + the shift pass X took): the
        // next pass X's shifts
        a.shift_b[2 * pr] = vr[0] + __ldcg(a.shift_a + 2 * pr);
        a.shift_b[2 * pr + 1] = vi[0] + __ldcg(a.shift_a + 2 * pr + 1);
      }
    }
    if (__syncthreads_or(fail)) break;  // every thread has its zs: the slot takes the next tile
    if (tid == 0 && j + 1 < my) {
      fence_proxy_async();
      load_zs(tile + (int)gridDim.x);
    }
    d2_line_tab<N, false, CONF>(vr, vi, t, scr + li * T::LSTRIDE, tf, ti, fk, ge);
    if (AXIS == 2 && j == 0) {  // pass Y has completed: its momenta may be read
      pdl_wait();
      pdl_trigger();
      if (tid == 0) load_pi(tile);
    }
    fail = !mbar_wait(&bar[1], ph);
    const int64_t offA = (int64_t)pr * 2 * Nsite + (AXIS == 1 ? (int64_t)o * a.nx * a.ny : (int64_t)o * a.nx) + x0 + li;
    const int64_t offB = Nsite + offA;
    float kes[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      const int pos = t + P * q;
      const float* pa = ls + pos * T::RS + li;
      float pA = pa[0], pB = pa[T::ARR];
      pA = pA + ck * vr[q];
      pB = pB + ck * vi[q];
      if (AXIS == 2 && CONF) kes[q % 4] += pA * pA + pB * pB;
      pi_o[offA + (int64_t)pos * st] = pA;
      pi_o[offB + (int64_t)pos * st] = pB;
    }
    if (AXIS == 2 && CONF) ke.add((kes[0] + kes[1]) + (kes[2] + kes[3]));
    if (__syncthreads_or(fail)) break;  // every thread has read its momenta: the slot takes the next tile
    if (tid == 0 && j + 1 < my) {
      fence_proxy_async();
      load_pi(tile + (int)gridDim.x);
    }
  }
  if (fail) {
    // a copy never completed: record it, give the copies in flight a
    // bounded wait, and leave without partial sums
    if (tid == 0) {
      atomicOr(&a.sc->err, 2u);
      mbar_wait(&bar[0], 0u);
      mbar_wait(&bar[0], 1u);
      mbar_wait(&bar[1], 0u);
      mbar_wait(&bar[1], 1u);
    }
    return;
  }
  if constexpr (!CONF) return;
  if constexpr (AXIS == 1) {
    const FF vals[1] = {ge.red()};
    block_partials<1>(vals, a.rb.partials + SEP_PART_Y);
  } else {
    const FF vals[2] = {ge.red(), ke.red()};
    block_partials<2>(vals, a.rb.partials + SEP_PART_Z);
  }
}

// pdl: launch as a programmatic dependent of the previous kernel in the
// stream (the two-field passes, which order their reads by pdl_wait)
template <typename K>
int stream_launch(K k, int smem, int threads, int minb, int64_t ntiles, const SepArgs& a, cudaStream_t s,
                  bool pdl = false) {
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return cuda_fail(e, "streamed separable pass smem attribute");
  const int64_t cap = (int64_t)minb * a.nsm;
  const int grid = (int)(ntiles < cap ? ntiles : cap);
  if (a.grid_out) *a.grid_out = grid;  // host side: the blocks whose partials the finalize sums
  if (pdl) {
    e = launch_pdl(k, dim3(grid), dim3(threads), (size_t)smem, s, a);
    if (e != cudaSuccess) return cuda_fail(e, "streamed separable pass launch");
  } else {
    k<<<grid, threads, smem, s>>>(a);
  }
  if (g_launch_counter) ++*g_launch_counter;
  e = cudaGetLastError();
  return e == cudaSuccess ? LAT_OK : cuda_fail(e, "streamed separable pass launch");
}

// Lines per block tile of the streamed pass along `axis` (the host checks
// that every pass of a lattice forms whole tiles before choosing them).
template <int N>
int stream_lines(int axis) {
  return axis == 0 ? STile<0, N>::LINES : (axis == 1 ? STile<1, N>::LINES : STile<2, N>::LINES);
}

template <int N, bool RUNS>
int sep_stream_dispatch(const SepArgs& a, int axis, cudaStream_t s) {
  const int lines = stream_lines<N>(axis);
  if (a.pair_lines <= 0 || a.nlines <= 0 || a.nlines >= (int64_t{1} << 31) || a.nlines % a.pair_lines ||
      a.pair_lines % lines ||
      (axis != 0 && a.nx % lines) || (!RUNS && (a.nf != 2 || a.nlines != a.pair_lines)) ||
      (RUNS && (a.conf || !a.shift_a || !a.shift_b)))
    return set_error(LAT_ERR_STATE, "streamed separable pass: lines do not form whole tiles");
  const int64_t ntiles = a.nlines / lines;
  // X, Y, Z (and the two-field finalize) launch as programmatic dependents;
  // the pairs-of-runs pass X follows an event join, so it launches plainly
  using TY = STile<1, N>;
  using TZ = STile<2, N>;
  if constexpr (!RUNS) {
    if (a.conf) {
      switch (axis) {
        case 0:
          if (a.model.model == LAT_MODEL_PHI4_G2)  // the headline model: the potential folds at compile time
            return stream_launch(sep_stream_x<N, false, true, LAT_MODEL_PHI4_G2>, STile<0, N>::SMEM,
                                 STile<0, N>::THREADS, STile<0, N>::MINB, ntiles, a, s, true);
          return stream_launch(sep_stream_x<N, false, true>, STile<0, N>::SMEM, STile<0, N>::THREADS,
                               STile<0, N>::MINB, ntiles, a, s, true);
        case 1: return stream_launch(sep_stream_yz_tma<1, N, false, true>, TY::SMEM + 128, TY::THREADS, TY::MINB,
                                     ntiles, a, s, true);
        default:
          return stream_launch(sep_stream_yz_tma<2, N, false, true>, TZ::SMEM + 128, TZ::THREADS, TZ::MINB, ntiles,
                               a, s, true);
      }
    }
  }
  switch (axis) {
    case 0: return stream_launch(sep_stream_x<N, RUNS, false>, STile<0, N>::SMEM, STile<0, N>::THREADS,
                                 STile<0, N>::MINB, ntiles, a, s, !RUNS);
    case 1: return stream_launch(sep_stream_yz_tma<1, N, RUNS, false>, TY::SMEM + 128, TY::THREADS, TY::MINB, ntiles,
                                 a, s, true);
    default: return stream_launch(sep_stream_yz_tma<2, N, RUNS, false>, TZ::SMEM + 128, TZ::THREADS, TZ::MINB, ntiles,
                                  a, s, true);
  }
}

}  // namespace sep
}  // namespace lat
