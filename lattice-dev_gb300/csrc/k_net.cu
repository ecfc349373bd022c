// k_net.cu -- BF16 kernels of the learned subgrid closure (sm_103a).
//
// The closure network is three periodic 3x3x3 convolutions, 4 -> 32 -> 32 -> 2
// channels, GELU after the first two.  Activations are stored channels-last
// ([lattice][z][y][x][C], C padded to 8 or 32) in BF16; every product
// accumulates in FP32 on the tensor cores (mma.sync m16n8k16 / m16n8k8 with
// BF16 operands); the master weights and the optimiser state are FP32.
//
// A convolution is an implicit GEMM: output sites x output channels, summed
// over 27 taps x input channels.  A block stages its tile's input halo and
// all 27 weight taps in shared memory and walks the taps with ldmatrix; the
// same kernel runs the backward data pass with the taps mirrored and the
// weights transposed.  The weight gradient is a GEMM over sites: per block
// partial sums, reduced over blocks in a fixed order (deterministic).
#include <cuda_bf16.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <type_traits>

#include "common.cuh"
#include "gelu.cuh"
#include "net.hpp"

namespace lat {
namespace net {

namespace {

constexpr int TX = 16, TY = 8, HX = TX + 2, HY = TY + 2, HZ = 3, HSITES = HX * HY * HZ;
constexpr int TSITES = TX * TY;

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void cp16(void* s, const void* g) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(smem_u32(s)), "l"(g) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }
template <int K> __device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(K) : "memory");
}

__device__ __forceinline__ void ldsm_x4(uint32_t (&r)[4], const void* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(smem_u32(p)));
}
__device__ __forceinline__ void ldsm_x2(uint32_t (&r)[2], const void* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0,%1}, [%2];\n"
               : "=r"(r[0]), "=r"(r[1])
               : "r"(smem_u32(p)));
}
__device__ __forceinline__ void ldsm_x4_t(uint32_t (&r)[4], const void* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(smem_u32(p)));
}
__device__ __forceinline__ void ldsm_x2_t(uint32_t (&r)[2], const void* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x2.trans.shared.b16 {%0,%1}, [%2];\n"
               : "=r"(r[0]), "=r"(r[1])
               : "r"(smem_u32(p)));
}
// D = A(16x16, row) B(16x8, col) + D, BF16 in, FP32 accumulate
__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}
// D = A(16x8, row) B(8x8, col) + D
__device__ __forceinline__ void mma1688(float (&d)[4], const uint32_t (&a)[2], uint32_t b0) {
  asm volatile("mma.sync.aligned.m16n8k8.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5}, {%6}, {%0,%1,%2,%3};\n"
               : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
               : "r"(a[0]), "r"(a[1]), "r"(b0));
}

__device__ __forceinline__ float gelu(float z) { return gelu_t(z); }
__device__ __forceinline__ float gelu_d(float z) { return gelu_t_d(z); }

// padded shared-memory row (elements) of a site with C channels: 80-byte rows
// for 32 channels keep the 8 rows of an ldmatrix in distinct banks
template <int C> struct Row { static constexpr int S = C == 32 ? 40 : 8; };

// Stage the (TZ=1) x TY x TX tile's halo of a channels-last lattice
// [nz][ny][nx][C] into shared memory rows of Row<C>::S elements.
template <int C>
__device__ __forceinline__ void load_halo(__nv_bfloat16* sm, const __nv_bfloat16* src, int nx, int ny, int nz,
                                          int x0, int y0, int z0) {
  constexpr int CH = C / 8;  // 16-byte chunks per site
  for (int i = threadIdx.x; i < HSITES * CH; i += blockDim.x) {
    const int s = i / CH, c = i % CH;
    const int hx = s % HX, hy = (s / HX) % HY, hz = s / (HX * HY);
    int x = x0 + hx - 1, y = y0 + hy - 1, z = z0 + hz - 1;
    x = x < 0 ? x + nx : (x >= nx ? x - nx : x);
    y = y < 0 ? y + ny : (y >= ny ? y - ny : y);
    z = z < 0 ? z + nz : (z >= nz ? z - nz : z);
    const int64_t g = (((int64_t)z * ny + y) * nx + x) * C + c * 8;
    cp16(sm + s * Row<C>::S + c * 8, src + g);
  }
}

// ---------------------------------------------------------------- conv
// out[s][n] = epi( sum_tap sum_k in[s + off(tap)][k] * W[tap][n][k] )
// EPI_GELU:   z = acc + b; zout = z (optional); out = gelu(z)        (BF16)
// EPI_LINEAR: out = acc + b, first two channels, FP32 [s][2]
// EPI_BWD:    out = acc * gelu'(zin[s][n])                            (BF16)
template <int CA, int CB, int EPI, bool STORE_Z>
__global__ void __launch_bounds__(128) conv_kernel(ConvArgs a) {
  constexpr int SA = Row<CA>::S, SW = Row<CA>::S;
  constexpr int NT = CB / 8;  // n-tiles of 8 output channels
  extern __shared__ __align__(16) unsigned char smraw[];
  __nv_bfloat16* wsm = reinterpret_cast<__nv_bfloat16*>(smraw);  // [27][CB][SW]
  __nv_bfloat16* hsm = wsm + 27 * CB * SW;                        // [HSITES][SA]
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int g = lane >> 2, t4 = lane & 3;
  // weights once per block
  {
    constexpr int CH = CA / 8;
    const __nv_bfloat16* W = a.w;
    for (int i = tid; i < 27 * CB * CH; i += blockDim.x) {
      const int row = i / CH, c = i % CH;
      cp16(wsm + row * SW + c * 8, W + (int64_t)row * CA + c * 8);
    }
    cp_commit();
  }
  float bias[NT][2];
#pragma unroll
  for (int nt = 0; nt < NT; ++nt) {
    bias[nt][0] = a.bias ? a.bias[nt * 8 + 2 * t4] : 0.f;
    bias[nt][1] = a.bias ? a.bias[nt * 8 + 2 * t4 + 1] : 0.f;
  }
  const int tiles_x = a.nx / TX, tiles_y = a.ny / TY;
  const int64_t tiles_per = (int64_t)tiles_x * tiles_y * a.nz;
  const int64_t ntiles = tiles_per * a.nlat;
  const int64_t Nsite = (int64_t)a.nx * a.ny * a.nz;
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int64_t lat_i = tile / tiles_per;
    int64_t r = tile % tiles_per;
    const int tx = (int)(r % tiles_x);
    r /= tiles_x;
    const int ty = (int)(r % tiles_y);
    const int z0 = (int)(r / tiles_y);
    const int x0 = tx * TX, y0 = ty * TY;
    const __nv_bfloat16* src = a.in + lat_i * Nsite * CA;
    __syncthreads();  // previous tile's reads of the halo are done
    load_halo<CA>(hsm, src, a.nx, a.ny, a.nz, x0, y0, z0);
    cp_commit();
    cp_wait_all();
    __syncthreads();

    float acc[2][NT][4];
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
      for (int nt = 0; nt < NT; ++nt)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[mt][nt][q] = 0.f;

#pragma unroll 1
    for (int tap = 0; tap < 27; ++tap) {
      const int dz = tap / 9, dy = (tap / 3) % 3, dx = tap % 3;  // halo offsets 0..2
      const __nv_bfloat16* wt = wsm + tap * CB * SW;
      if constexpr (CA == 32) {
#pragma unroll
        for (int kk = 0; kk < 2; ++kk) {
          // B fragments for all n-tiles of this k-step
          uint32_t b[NT][2];
          if constexpr (NT >= 2) {
#pragma unroll
            for (int np = 0; np < NT / 2; ++np) {
              const int idx = lane >> 3, rr = lane & 7;
              const int n = np * 16 + rr + 8 * (idx >> 1), k = kk * 16 + 8 * (idx & 1);
              uint32_t q[4];
              ldsm_x4(q, wt + n * SW + k);
              b[2 * np][0] = q[0]; b[2 * np][1] = q[1];
              b[2 * np + 1][0] = q[2]; b[2 * np + 1][1] = q[3];
            }
          } else {
            const int idx = (lane >> 3) & 1, rr = lane & 7;
            uint32_t q[2];
            ldsm_x2(q, wt + rr * SW + kk * 16 + 8 * idx);
            b[0][0] = q[0]; b[0][1] = q[1];
          }
#pragma unroll
          for (int mt = 0; mt < 2; ++mt) {
            const int yy = 2 * warp + mt;  // tile row of this m-tile
            const int idx = lane >> 3, rr = lane & 7;
            const int xs = rr + 8 * (idx & 1);
            const int hs = (dz * HY + (yy + dy)) * HX + (xs + dx);
            uint32_t af[4];
            ldsm_x4(af, hsm + hs * SA + kk * 16 + 8 * (idx >> 1));
#pragma unroll
            for (int nt = 0; nt < NT; ++nt) mma16816(acc[mt][nt], af, b[nt][0], b[nt][1]);
          }
        }
      } else {  // CA == 8: one k8 step per tap
        uint32_t b[NT];
        if constexpr (NT == 4) {
          const int idx = lane >> 3, rr = lane & 7;
          uint32_t q[4];
          ldsm_x4(q, wt + (idx * 8 + rr) * SW);
          b[0] = q[0]; b[1] = q[1]; b[2] = q[2]; b[3] = q[3];
        } else {
          ldsm_x1(b[0], wt + (lane & 7) * SW);
        }
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
          const int yy = 2 * warp + mt;
          const int xs = (lane & 7) + 8 * ((lane >> 3) & 1);
          const int hs = (dz * HY + (yy + dy)) * HX + (xs + dx);
          uint32_t af[2];
          ldsm_x2(af, hsm + hs * SA);
#pragma unroll
          for (int nt = 0; nt < NT; ++nt) mma1688(acc[mt][nt], af, b[nt]);
        }
      }
    }
    // epilogue: rows g and g+8 of each m-tile are x = g, g + 8
    const int64_t obase = lat_i * Nsite;
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
      const int y = y0 + 2 * warp + mt;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int x = x0 + g + 8 * h;
        const int64_t s = obase + ((int64_t)z0 * a.ny + y) * a.nx + x;
#pragma unroll
        for (int nt = 0; nt < NT; ++nt) {
          const int n = nt * 8 + 2 * t4;
          float v0 = acc[mt][nt][2 * h], v1 = acc[mt][nt][2 * h + 1];
          if constexpr (EPI == EPI_GELU) {
            v0 += bias[nt][0];
            v1 += bias[nt][1];
            if constexpr (STORE_Z)
              *reinterpret_cast<__nv_bfloat162*>(a.zout + s * CB + n) = __floats2bfloat162_rn(v0, v1);
            *reinterpret_cast<__nv_bfloat162*>(a.out + s * CB + n) = __floats2bfloat162_rn(gelu(v0), gelu(v1));
          } else if constexpr (EPI == EPI_LINEAR) {
            if (nt == 0 && t4 == 0)
              *reinterpret_cast<float2*>(a.outf + s * 2) = make_float2(v0 + bias[0][0], v1 + bias[0][1]);
          } else {
            const __nv_bfloat162 zz = *reinterpret_cast<const __nv_bfloat162*>(a.zin + s * CB + n);
            const float z0f = __bfloat162float(zz.x), z1f = __bfloat162float(zz.y);
            *reinterpret_cast<__nv_bfloat162*>(a.out + s * CB + n) =
                __floats2bfloat162_rn(v0 * gelu_d(z0f), v1 * gelu_d(z1f));
          }
        }
      }
    }
  }
}

// ----------------------------------------------------- output layer, 32 -> 2
// The direct form above re-reads 27 taps x 32 input channels of the halo
// (1.7 KB per site) for only two output channels.  Here the weights stay in
// the MMA's A fragments and the input sites are its N side: for a staged
// input plane and tap row dz, D[(tap, co)][site'] = sum_ci W[tap][co][ci]
// x[site'][ci] for the 9 (dy, dx) taps x 2 outputs (18 rows of two m16
// tiles), over every staged site (the item's TYO output rows plus one halo
// row on either side, whole x-rows of NXO sites, so the x halo is the row
// itself).  D goes to shared memory; each thread then adds, for its output
// site, the 9 D values of its neighbours in a fixed order.
//
// An item marches through zc output planes: input plane zA - 1 + j is staged
// once (its successor's copies in flight meanwhile) and serves output planes
// j (tap row 0), j - 1 (row 1) and j - 2 (row 2), which completes; three
// rotating accumulators per thread hold the planes in progress.  D is
// double-buffered when two blocks per SM still fit, so the sums of one tap
// row overlap the MMAs of the next.  Input rows are 64 bytes, 16-byte chunks
// swizzled by (site >> 1) & 3 so the 8 rows of an ldmatrix fall in distinct
// banks.
template <int NXO, int TYO>
struct OutGeom {
  static constexpr int HR = TYO + 2, NS = HR * NXO;    // staged rows and sites per plane
  static constexpr int DS = NS + 8;                    // D row stride (floats): 64-bit stores conflict-free
  static constexpr int XIN = NS * 64;                  // bytes per staged plane
  static constexpr int DB = 18 * DS * 4;               // bytes per D buffer
  static constexpr int NDB = 2 * XIN + 2 * DB <= 110 * 1024 ? 2 : 1;
  static constexpr int SMEM = 2 * XIN + NDB * DB;
  static_assert((NS / 8) % 8 == 0, "n-tiles divide evenly over 8 warps");
  static_assert(TYO * NXO == 256, "one output site per thread");
};

__device__ __forceinline__ int swz(int site, int chunk) { return site * 64 + ((chunk ^ ((site >> 1) & 3)) << 4); }

template <int NXO, int TYO>
__global__ void __launch_bounds__(256) out_conv_kernel(ConvArgs a, int zc) {
  using G = OutGeom<NXO, TYO>;
  extern __shared__ __align__(16) unsigned char smraw[];
  unsigned char* xin = smraw;                                   // [2][NS] x 64 bytes (swizzled)
  float* dsm = reinterpret_cast<float*>(smraw + 2 * G::XIN);   // [NDB][18][DS]
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, g = lane >> 2, t4 = lane & 3;
  // A fragments: [dz][m tile][k step]; row R = 2 (3 dy + dx) + co of m tile R / 16, zero beyond 18
  uint32_t af[3][2][2][4];
#pragma unroll
  for (int dz = 0; dz < 3; ++dz)
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
      for (int ks = 0; ks < 2; ++ks)
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          const int R = 16 * mt + g + ((r & 1) ? 8 : 0);
          const int k = 16 * ks + 2 * t4 + ((r & 2) ? 8 : 0);
          uint32_t v = 0;
          if (R < 18) {
            const int tap = dz * 9 + R / 2, co = R % 2;
            v = *reinterpret_cast<const uint32_t*>(a.w + ((int64_t)tap * 8 + co) * 32 + k);
          }
          af[dz][mt][ks][r] = v;
        }
  const float b0 = a.bias ? a.bias[0] : 0.f, b1 = a.bias ? a.bias[1] : 0.f;
  const int64_t Nsite = (int64_t)a.nx * a.ny * a.nz;
  const int tiles_y = a.ny / TYO, zchunks = (a.nz + zc - 1) / zc;
  const int64_t items_per = (int64_t)tiles_y * zchunks, nitems = items_per * a.nlat;
  const int ox = tid % NXO, oy = tid / NXO;  // this thread's output site within the item

  auto stage = [&](int buf, const __nv_bfloat16* src, int y0, int z) {
    z = z < 0 ? z + a.nz : (z >= a.nz ? z - a.nz : z);
    unsigned char* dst = xin + buf * G::XIN;
    for (int i = tid; i < G::NS * 4; i += 256) {
      const int site = i >> 2, c = i & 3;
      const int hy = site / NXO, x = site % NXO;
      int y = y0 - 1 + hy;
      y = y < 0 ? y + a.ny : (y >= a.ny ? y - a.ny : y);
      cp16(dst + swz(site, c), src + (((int64_t)z * a.ny + y) * NXO + x) * 32 + c * 8);
    }
    cp_commit();
  };
  // D of tap row DZ for every staged site of plane buffer xb into D buffer db
  auto mma_row = [&](auto dzc, const unsigned char* xb, float* db) {
    constexpr int DZ = decltype(dzc)::value;
#pragma unroll 1
    for (int nt = warp; nt < G::NS / 8; nt += 8) {
      uint32_t b[4];
      ldsm_x4(b, xb + swz(nt * 8 + (lane & 7), lane >> 3));
      float d0[4] = {0.f, 0.f, 0.f, 0.f}, d1[4] = {0.f, 0.f, 0.f, 0.f};
      mma16816(d0, af[DZ][0][0], b[0], b[1]);
      mma16816(d0, af[DZ][0][1], b[2], b[3]);
      mma16816(d1, af[DZ][1][0], b[0], b[1]);
      mma16816(d1, af[DZ][1][1], b[2], b[3]);
      const int col = nt * 8 + 2 * t4;
      *reinterpret_cast<float2*>(db + g * G::DS + col) = make_float2(d0[0], d0[1]);
      *reinterpret_cast<float2*>(db + (g + 8) * G::DS + col) = make_float2(d0[2], d0[3]);
      if (g < 2) *reinterpret_cast<float2*>(db + (16 + g) * G::DS + col) = make_float2(d1[0], d1[1]);
    }
  };
  // this thread's output site: the 9 (dy, dx) taps of D buffer db, in a fixed order
  auto gather = [&](const float* db, float& c0, float& c1) {
#pragma unroll
    for (int dy = 0; dy < 3; ++dy) {
#pragma unroll
      for (int dx = 0; dx < 3; ++dx) {
        int hx = ox + dx - 1;
        hx = hx < 0 ? hx + NXO : (hx >= NXO ? hx - NXO : hx);
        const int site = (oy + dy) * NXO + hx, R = 2 * (3 * dy + dx);
        c0 += db[R * G::DS + site];
        c1 += db[(R + 1) * G::DS + site];
      }
    }
  };

  int pb = 0;  // D buffer of the next MMA pass
  for (int64_t item = blockIdx.x; item < nitems; item += gridDim.x) {
    const int64_t li = item / items_per;
    const int64_t rr = item % items_per;
    const int y0 = (int)(rr % tiles_y) * TYO, zA = (int)(rr / tiles_y) * zc;
    const int nzs = min(zc, a.nz - zA);
    const __nv_bfloat16* src = a.in + li * Nsite * 32;
    float* outp = a.outf + (li * Nsite + (int64_t)(y0 + oy) * NXO + ox) * 2;
    // accumulators of output planes j (n), j - 1 (m), j - 2 (l) relative to zA
    float n0 = 0.f, n1 = 0.f, m0 = 0.f, m1 = 0.f, l0 = 0.f, l1 = 0.f;
    stage(0, src, y0, zA - 1);
#pragma unroll 1
    for (int j = 0; j <= nzs + 1; ++j) {
      if (j <= nzs) {
        stage((j + 1) & 1, src, y0, zA + j);
        cp_async_wait<1>();
      } else {
        cp_wait_all();
      }
      __syncthreads();  // plane j landed; the previous plane's last sums are done
      const unsigned char* xb = xin + (j & 1) * G::XIN;
      float* dA = dsm + pb * (G::NDB - 1) * 18 * G::DS;         // D buffers of this plane's passes
      float* dB = dsm + (pb ^ 1) * (G::NDB - 1) * 18 * G::DS;
      const bool r0 = j < nzs, r1 = j >= 1 && j - 1 < nzs, r2 = j >= 2;  // output planes j, j-1, j-2 exist
      // tap row 0 -> plane j, row 1 -> plane j - 1, row 2 -> plane j - 2 (uniform branches)
      if (r0) mma_row(std::integral_constant<int, 0>{}, xb, dA);
      __syncthreads();
      if (r0) gather(dA, n0, n1);
      if (G::NDB == 1) __syncthreads();
      if (r1) mma_row(std::integral_constant<int, 1>{}, xb, dB);
      __syncthreads();
      if (r1) gather(dB, m0, m1);
      if (G::NDB == 1) __syncthreads();
      if (r2) mma_row(std::integral_constant<int, 2>{}, xb, dA);
      __syncthreads();
      if (r2) {
        gather(dA, l0, l1);
        *reinterpret_cast<float2*>(outp + (int64_t)(zA + j - 2) * a.ny * NXO * 2) = make_float2(l0 + b0, l1 + b1);
      }
      pb ^= 1;  // the next plane's first pass writes the buffer this plane's row 1 used
      l0 = m0, l1 = m1, m0 = n0, m1 = n1, n0 = 0.f, n1 = 0.f;
    }
  }
  cp_wait_all();
}

// ------------------------------------------------------- weight gradient
// part[blk][tap][i][o] = sum over the block's sites s of X[s + off(tap)][i] * D[s][o]
// (X: CX channels, halo-shifted; D: CD channels).  The GEMM's M side is the
// 32-channel operand.  part_b[blk][o] = sum_s D[s][o].
template <int CX, int CD>
__global__ void __launch_bounds__(288) wgrad_kernel(WgradArgs a) {
  constexpr bool MX = CX == 32;  // M = X channels (else M = D channels)
  constexpr int CN = MX ? CD : CX;
  constexpr int NT = CN / 8;
  constexpr int SX = Row<CX>::S, SD = Row<CD>::S;
  extern __shared__ __align__(16) unsigned char smraw[];
  __nv_bfloat16* xs = reinterpret_cast<__nv_bfloat16*>(smraw);  // [HSITES][SX]
  __nv_bfloat16* ds = xs + HSITES * SX;                           // [TSITES][SD]
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;  // 9 warps
  const int g = lane >> 2, t4 = lane & 3;
  float acc[3][2][NT][4];
#pragma unroll
  for (int j = 0; j < 3; ++j)
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
      for (int nt = 0; nt < NT; ++nt)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[j][mt][nt][q] = 0.f;
  float bsum = 0.f;  // thread tid < CD: channel tid of D

  const int tiles_x = a.nx / TX, tiles_y = a.ny / TY;
  const int64_t tiles_per = (int64_t)tiles_x * tiles_y * a.nz;
  const int64_t ntiles = tiles_per * a.nlat;
  const int64_t Nsite = (int64_t)a.nx * a.ny * a.nz;
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int64_t lat_i = tile / tiles_per;
    int64_t r = tile % tiles_per;
    const int tx = (int)(r % tiles_x);
    r /= tiles_x;
    const int ty = (int)(r % tiles_y);
    const int z0 = (int)(r / tiles_y);
    const int x0 = tx * TX, y0 = ty * TY;
    __syncthreads();
    load_halo<CX>(xs, a.x + lat_i * Nsite * CX, a.nx, a.ny, a.nz, x0, y0, z0);
    {
      constexpr int CH = CD / 8;
      const __nv_bfloat16* D = a.d + lat_i * Nsite * CD;
      for (int i = tid; i < TSITES * CH; i += blockDim.x) {
        const int s = i / CH, c = i % CH;
        const int xx = s % TX, yy = s / TX;
        cp16(ds + s * SD + c * 8, D + (((int64_t)z0 * a.ny + y0 + yy) * a.nx + x0 + xx) * CD + c * 8);
      }
    }
    cp_commit();
    cp_wait_all();
    __syncthreads();
    if (tid < CD)
      for (int s = 0; s < TSITES; ++s) bsum += __bfloat162float(ds[s * SD + tid]);

#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const int tap = warp + 9 * j;
      const int dz = tap / 9, dy = (tap / 3) % 3, dx = tap % 3;
#pragma unroll 1
      for (int ky = 0; ky < TY; ++ky) {  // 16 sites of tile row ky per k-step
        // shifted X rows: halo site of tile site (xx, ky) moved by the tap
        auto xrow = [&](int xx) { return ((dz * HY) + (ky + dy)) * HX + (xx + dx); };
        auto drow = [&](int xx) { return ky * TX + xx; };
        const int idx = lane >> 3, rr = lane & 7;
        // M operand (2 m-tiles of 16 channels): ldmatrix.trans of [site][chan]
        uint32_t am[2][4];
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
          const int site = rr + 8 * (idx >> 1), ch = mt * 16 + 8 * (idx & 1);
          if constexpr (MX) ldsm_x4_t(am[mt], xs + xrow(site) * SX + ch);
          else ldsm_x4_t(am[mt], ds + drow(site) * SD + ch);
        }
        // N operand (NT n-tiles of 8 channels)
        uint32_t bn[NT][2];
        if constexpr (NT >= 2) {
#pragma unroll
          for (int np = 0; np < NT / 2; ++np) {
            const int site = rr + 8 * (idx & 1), ch = np * 16 + 8 * (idx >> 1);
            uint32_t q[4];
            if constexpr (MX) ldsm_x4_t(q, ds + drow(site) * SD + ch);
            else ldsm_x4_t(q, xs + xrow(site) * SX + ch);
            bn[2 * np][0] = q[0]; bn[2 * np][1] = q[1];
            bn[2 * np + 1][0] = q[2]; bn[2 * np + 1][1] = q[3];
          }
        } else {
          const int site = rr + 8 * (idx & 1);
          uint32_t q[2];
          if constexpr (MX) ldsm_x2_t(q, ds + drow(site) * SD);
          else ldsm_x2_t(q, xs + xrow(site) * SX);
          bn[0][0] = q[0]; bn[0][1] = q[1];
        }
#pragma unroll
        for (int mt = 0; mt < 2; ++mt)
#pragma unroll
          for (int nt = 0; nt < NT; ++nt) mma16816(acc[j][mt][nt], am[mt], bn[nt][0], bn[nt][1]);
      }
    }
  }
  // partials in [tap][x-chan][d-chan] order
  float* part = a.part + (int64_t)blockIdx.x * 27 * CX * CD;
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    const int tap = warp + 9 * j;
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
      for (int nt = 0; nt < NT; ++nt)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int m = mt * 16 + g + 8 * (q >> 1), n = nt * 8 + 2 * t4 + (q & 1);
          const int i = MX ? m : n, o = MX ? n : m;
          part[(tap * CX + i) * CD + o] = acc[j][mt][nt][q];
        }
  }
  if (tid < CD) a.part_b[(int64_t)blockIdx.x * CD + tid] = bsum;
}

// grad[e] = sum over blocks of part[blk][e], blocks in index order
__global__ void reduce_parts_kernel(const float* __restrict__ part, int nblk, int64_t per, float* __restrict__ out) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < per; e += (int64_t)gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int b = 0; b < nblk; ++b) s += part[(int64_t)b * per + e];
    out[e] = s;
  }
}

// ------------------------------------------------------------ pointwise
// channels-last BF16 input [lat][site][8] from four FP32/FP64 channel arrays,
// normalised: (x u - shift) * scale = x (u scale) - shift scale in FP32 (the
// result is rounded to BF16); channels 4..7 are zero.  The unit factors u
// (a, 1/a) and the affine coefficients are formed once per block.
template <typename R>
__global__ void pack_kernel(PackArgs a) {
  __shared__ float mul_sh[4], add_sh[4];
  if (threadIdx.x == 0) {
    double u[4] = {1.0, 1.0, 1.0, 1.0};
    if (a.sc) {
      // the scale factor the kick sees: after a pending gravity half-step
      // (the same expression as the gravity kernel's)
      const double av = a.hg != 0.0 ? __ldcg(&a.sc->a) - a.hg * __ldcg(&a.sc->ap) / 6.0 : __ldcg(&a.sc->a);
      u[0] = u[1] = av;
      u[2] = u[3] = 1.0 / av;
    }
    for (int c = 0; c < 4; ++c) {
      mul_sh[c] = (float)(u[c] * a.scale[c]);
      add_sh[c] = (float)(-a.shift[c] * a.scale[c]);
    }
  }
  __syncthreads();
  float mul[4], add[4];
#pragma unroll
  for (int c = 0; c < 4; ++c) mul[c] = mul_sh[c], add[c] = add_sh[c];
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t l = 0; l < a.nlat; ++l) {
    const int64_t base = a.idx ? (int64_t)a.idx[l] * a.lat_stride : l * a.lat_stride;
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < a.N; s += stride) {
      __align__(16) __nv_bfloat16 v[8];
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const R* p = static_cast<const R*>(a.ch[c]);
        v[c] = __float2bfloat16_rn(fmaf((float)p[base + s], mul[c], add[c]));
      }
#pragma unroll
      for (int c = 4; c < 8; ++c) v[c] = __float2bfloat16_rn(0.f);
      *reinterpret_cast<uint4*>(a.out + (l * a.N + s) * 8) = *reinterpret_cast<const uint4*>(v);
    }
  }
}

// MSE against the scaled targets; dout = 2 (out - t) / count in BF16 [site][8]
__global__ void loss_kernel(LossArgs a) {
  const int64_t total = a.nlat * a.N;
  double local = 0.0;
  const double inv = 1.0 / (2.0 * (double)total);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t l = i / a.N, s = i % a.N;
    const int64_t base = (int64_t)a.idx[l] * a.lat_stride;
    const float2 o = *reinterpret_cast<const float2*>(a.out + i * 2);
    const float t0 = (float)(a.t0[base + s] * a.tscale[0]), t1 = (float)(a.t1[base + s] * a.tscale[1]);
    const float e0 = o.x - t0, e1 = o.y - t1;
    local += (double)e0 * e0 + (double)e1 * e1;
    __align__(16) __nv_bfloat16 v[8];
    v[0] = __float2bfloat16_rn((float)(2.0 * inv) * e0);
    v[1] = __float2bfloat16_rn((float)(2.0 * inv) * e1);
#pragma unroll
    for (int c = 2; c < 8; ++c) v[c] = __float2bfloat16_rn(0.f);
    *reinterpret_cast<uint4*>(a.dout + i * 8) = *reinterpret_cast<const uint4*>(v);
  }
  // block sum into part[blockIdx]
  __shared__ double ws[32];
  local = warp_sum(local);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = local;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < (blockDim.x >> 5) ? ws[threadIdx.x] : 0.0;
    v = warp_sum(v);
    if (threadIdx.x == 0) a.part[blockIdx.x] = v * inv;
  }
}

__global__ void sum_kernel(const double* __restrict__ part, int n, double* __restrict__ out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += part[i];
    *out = s;
  }
}

// Adam step on the flat FP32 parameters (bias-corrected)
__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ gr, float* __restrict__ m,
                            float* __restrict__ v, int64_t n, float lr, float b1, float b2, float eps, float c1,
                            float c2) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float g = gr[i];
    const float mi = b1 * m[i] + (1.f - b1) * g;
    const float vi = b2 * v[i] + (1.f - b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

// BF16 copies of one layer's weights W[tap][i][o] (FP32):
//   fwd[tap][o][i] = W[tap][i][o];   bwd[tap][i][o] = W[26 - tap][i][o]
__global__ void repack_kernel(const float* __restrict__ W, int ci, int co, __nv_bfloat16* __restrict__ fwd,
                              __nv_bfloat16* __restrict__ bwd) {
  const int n = 27 * ci * co;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
    const int tap = e / (ci * co), r = e % (ci * co), i = r / co, o = r % co;
    fwd[(tap * co + o) * ci + i] = __float2bfloat16_rn(W[e]);
    if (bwd) bwd[((26 - tap) * ci + i) * co + o] = __float2bfloat16_rn(W[e]);
  }
}

// closure kick: pi_f += hk a^4 Delta_f with Delta_f = out[s][f] / tscale[f] (units 0) or
// a^3 Delta_f = out[s][f] / tscale[f] (units 1); a = 1 in Minkowski
template <typename R>
__global__ void corr_kick_kernel(CorrArgs a) {
  __shared__ double c_sh[2];  // the coefficients once per block (FP64 divisions)
  if (threadIdx.x == 0) {
    double av = 1.0;
    if (a.conf) av = __ldcg(&a.sc->a);
    const double f = a.units ? av : av * av * av * av;  // a^4 Delta = a (a^3 Delta)
    c_sh[0] = a.hk * f / a.tscale[0];
    c_sh[1] = a.hk * f / a.tscale[1];
  }
  __syncthreads();
  const R c0 = (R)c_sh[0], c1 = (R)c_sh[1];
  R* p0 = static_cast<R*>(a.pi);
  R* p1 = p0 + a.N;
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < a.N; s += (int64_t)gridDim.x * blockDim.x) {
    const float2 o = *reinterpret_cast<const float2*>(a.out + s * 2);
    p0[s] += c0 * (R)o.x;
    p1[s] += c1 * (R)o.y;
  }
}

template <int CA, int CB, int EPI, bool SZ>
int conv_go(const ConvArgs& a, int nsm, cudaStream_t s) {
  constexpr size_t smem = (size_t)(27 * CB * Row<CA>::S + HSITES * Row<CA>::S) * 2;
  auto k = conv_kernel<CA, CB, EPI, SZ>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return cuda_fail(e, "conv smem attribute");
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, 128, smem);
  if (per_sm < 1) per_sm = 1;
  const int64_t ntiles = (int64_t)(a.nx / TX) * (a.ny / TY) * a.nz * a.nlat;
  const int64_t grid = std::min<int64_t>(ntiles, (int64_t)nsm * per_sm);
  k<<<(unsigned)grid, 128, smem, s>>>(a);
  if (g_launch_counter) ++*g_launch_counter;
  e = cudaGetLastError();
  return e == cudaSuccess ? LAT_OK : cuda_fail(e, "conv launch");
}

template <int NXO, int TYO>
int out_conv_go(const ConvArgs& a, int nsm, cudaStream_t s) {
  constexpr int smem = OutGeom<NXO, TYO>::SMEM;
  auto k = out_conv_kernel<NXO, TYO>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return cuda_fail(e, "output conv smem attribute");
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, 256, smem);
  if (per_sm < 1) per_sm = 1;
  // output planes per item: the fewest rounds of items over the resident
  // blocks, counting an item's two extra input planes
  const int64_t slots = (int64_t)nsm * per_sm, items_xy = (int64_t)(a.ny / TYO) * a.nlat;
  int zc = 16;
  int64_t best = -1;
  for (int c = 16; c >= 2; c /= 2) {
    const int64_t items = items_xy * ((a.nz + c - 1) / c);
    const int64_t cost = ((items + slots - 1) / slots) * (std::min(c, a.nz) + 2);
    if (best < 0 || cost < best) best = cost, zc = c;
  }
  const int64_t nitems = items_xy * ((a.nz + zc - 1) / zc);
  const int64_t grid = std::min<int64_t>(nitems, slots);
  k<<<(unsigned)grid, 256, smem, s>>>(a, zc);
  if (g_launch_counter) ++*g_launch_counter;
  e = cudaGetLastError();
  return e == cudaSuccess ? LAT_OK : cuda_fail(e, "output conv launch");
}

}  // namespace

int conv(const ConvArgs& a, int ca, int cb, int epi, int nsm, cudaStream_t s) {
  if (a.nx % TX || a.ny % TY || a.nz < 1) return set_error(LAT_ERR_ARG, "closure lattice: nx % 16, ny % 8");
  static const bool no_tc = [] {
    const char* v = getenv("LAT_NO_TCGEN05");
    return v && v[0] && v[0] != '0';
  }();
  if (!no_tc && a.err && conv_tc_ok(ca, cb, epi, a.nx, a.ny)) return conv_tc(a, ca, epi, nsm, a.err, s);
  const bool sz = a.zout != nullptr;
  if (ca == 8 && cb == 32 && epi == EPI_GELU) return sz ? conv_go<8, 32, EPI_GELU, true>(a, nsm, s)
                                                        : conv_go<8, 32, EPI_GELU, false>(a, nsm, s);
  if (ca == 32 && cb == 32 && epi == EPI_GELU) return sz ? conv_go<32, 32, EPI_GELU, true>(a, nsm, s)
                                                         : conv_go<32, 32, EPI_GELU, false>(a, nsm, s);
  if (ca == 32 && cb == 8 && epi == EPI_LINEAR) {
    // whole x-rows of 64 or 128 sites: the weights-stationary kernel
    if (a.nx == 64 && a.ny % 4 == 0) return out_conv_go<64, 4>(a, nsm, s);
    if (a.nx == 128 && a.ny % 2 == 0) return out_conv_go<128, 2>(a, nsm, s);
    return conv_go<32, 8, EPI_LINEAR, false>(a, nsm, s);
  }
  if (ca == 8 && cb == 32 && epi == EPI_BWD) return conv_go<8, 32, EPI_BWD, false>(a, nsm, s);
  if (ca == 32 && cb == 32 && epi == EPI_BWD) return conv_go<32, 32, EPI_BWD, false>(a, nsm, s);
  return set_error(LAT_ERR_UNSUPPORTED, "conv shape");
}

int wgrad_blocks(int nsm) { return nsm; }

int wgrad(const WgradArgs& a, int cx, int cd, int nblk, float* dW, float* db, cudaStream_t s) {
  if (a.nx % TX || a.ny % TY) return set_error(LAT_ERR_ARG, "closure lattice: nx % 16, ny % 8");
  size_t smem = 0;
  cudaError_t e;
  auto go = [&](auto kern, int CX, int CD) -> int {
    smem = (size_t)(HSITES * (CX == 32 ? 40 : 8) + TSITES * (CD == 32 ? 40 : 8)) * 2;
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_fail(e, "wgrad smem attribute");
    kern<<<nblk, 288, smem, s>>>(a);
    if (g_launch_counter) ++*g_launch_counter;
    e = cudaGetLastError();
    return e == cudaSuccess ? LAT_OK : cuda_fail(e, "wgrad launch");
  };
  int st;
  if (cx == 32 && cd == 8) st = go(wgrad_kernel<32, 8>, 32, 8);
  else if (cx == 32 && cd == 32) st = go(wgrad_kernel<32, 32>, 32, 32);
  else if (cx == 8 && cd == 32) st = go(wgrad_kernel<8, 32>, 8, 32);
  else return set_error(LAT_ERR_UNSUPPORTED, "wgrad shape");
  if (st != LAT_OK) return st;
  const int64_t per = 27LL * cx * cd;
  reduce_parts_kernel<<<(unsigned)((per + 255) / 256), 256, 0, s>>>(a.part, nblk, per, dW);
  reduce_parts_kernel<<<1, 256, 0, s>>>(a.part_b, nblk, cd, db);
  if (g_launch_counter) *g_launch_counter += 2;
  e = cudaGetLastError();
  return e == cudaSuccess ? LAT_OK : cuda_fail(e, "wgrad reduce launch");
}

int pack(const PackArgs& a, int fp64, int nsm, cudaStream_t s) {
  const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>((a.N + 255) / 256, (int64_t)nsm * 8));
  if (fp64) pack_kernel<double><<<grid, 256, 0, s>>>(a);
  else pack_kernel<float><<<grid, 256, 0, s>>>(a);
  if (g_launch_counter) ++*g_launch_counter;
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? LAT_OK : cuda_fail(e, "pack launch");
}

int loss(const LossArgs& a, int nblk, double* out, cudaStream_t s) {
  loss_kernel<<<nblk, 256, 0, s>>>(a);
  sum_kernel<<<1, 32, 0, s>>>(a.part, nblk, out);
  if (g_launch_counter) *g_launch_counter += 2;
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? LAT_OK : cuda_fail(e, "loss launch");
}

int adam(float* p, const float* g, float* m, float* v, int64_t n, double lr, int64_t step, cudaStream_t s) {
  const double b1 = 0.9, b2 = 0.999;
  const float c1 = (float)(1.0 - pow(b1, (double)step)), c2 = (float)(1.0 - pow(b2, (double)step));
  adam_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(p, g, m, v, n, (float)lr, (float)b1, (float)b2, 1e-8f, c1,
                                                           c2);
  if (g_launch_counter) ++*g_launch_counter;
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? LAT_OK : cuda_fail(e, "adam launch");
}

int repack(const float* W, int ci, int co, __nv_bfloat16* fwd, __nv_bfloat16* bwd, cudaStream_t s) {
  repack_kernel<<<(27 * ci * co + 255) / 256, 256, 0, s>>>(W, ci, co, fwd, bwd);
  if (g_launch_counter) ++*g_launch_counter;
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? LAT_OK : cuda_fail(e, "repack launch");
}

int corr_kick(const CorrArgs& a, int fp64, int nsm, cudaStream_t s) {
  const unsigned grid = (unsigned)std::min<int64_t>((a.N + 255) / 256, (int64_t)nsm * 8);
  if (fp64) corr_kick_kernel<double><<<grid, 256, 0, s>>>(a);
  else corr_kick_kernel<float><<<grid, 256, 0, s>>>(a);
  if (g_launch_counter) ++*g_launch_counter;
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? LAT_OK : cuda_fail(e, "closure kick launch");
}

}  // namespace net
}  // namespace lat
