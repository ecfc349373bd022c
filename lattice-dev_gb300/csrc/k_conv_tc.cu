// k_conv_tc.cu -- the closure's 3x3x3 convolutions with 32 output channels
// (32 -> 32, and 4 padded to 8 -> 32) on the 5th-generation tensor cores
// (tcgen05.mma, accumulators in tensor memory).
//
// Work item: 256 output sites -- two M tiles of 128 sites -- marching through
// zc z-planes.  An M tile is one 128-site x-row (XW = 128) or two 64-site
// x-rows (XW = 64).  Output plane z needs input planes z-1, z, z+1; the block
// keeps a ring of four halo planes in shared memory, so each step loads one
// new plane.
//
// Per step, for each M tile: M = 128 sites, N = 32 output channels, K = 27
// taps x 32 input channels = 54 tcgen05.mma (M128 N32 K16, BF16 in, FP32
// out) issued by one thread.  Both operands come from shared memory through
// matrix descriptors in the no-swizzle K-major layout (8-row x 16-byte core
// matrices):
//   A: the 128 rows of one tap are 128 consecutive x of the halo; the tap's
//      x offset is a 16-byte shift.  XW = 128 stores each halo row as 130
//      consecutive x (core matrices 128 B apart).  XW = 64 stores it in
//      groups of 10 positions per 8 sites (x 8g-1 .. 8g+8, core matrices
//      160 B apart), so that a 16-byte shift stays inside a group and the
//      16 core matrices of two consecutive rows sit at one stride;
//   B: the weights [tap 27][channel chunk][out 32][8], staged once.
// Accumulators are double-buffered in TMEM (2 x 64 columns): a ninth warp
// issues the MMAs of step j while eight warps read back step j-1
// (tcgen05.ld; warp w owns TMEM lanes 32 (w mod 4) .. and columns
// 16 (w / 4) ..) for the epilogue (bias + GELU, or times GELU' for the
// backward data pass) and the next plane's copies are in flight.
//
// Every wait is bounded: a warp that gives up raises a shared abort flag that
// the whole block reads after its next barrier; the block then sets the error
// word, waits (bounded) for its own MMAs, frees its TMEM and returns.
#include <cuda_bf16.h>
#include <stdint.h>

#include <algorithm>

#include "gelu.cuh"
#include "net.hpp"

namespace lat {
namespace net {

namespace {

constexpr int TCR = 2;            // M tiles per step
constexpr int ZC_MAX = 16;        // z-planes per item, at most
constexpr int CM_BYTES = 128;     // one core matrix: 8 rows x 16 bytes
constexpr int NSLOT = 4;          // ring of halo planes
constexpr int B_CHUNK = 32 * 16;  // bytes per 8-channel chunk of the 32 output rows of B
constexpr int TMEM_COLS = 128;    // 2 buffers x 2 M tiles x 32 fp32 columns

// shared-memory geometry for CA input channels (32, or 8 = 4 padded) and
// x-rows of XW sites (128 or 64)
template <int CA, int XW>
struct TcGeom {
  static constexpr int CH = CA / 8;                 // 16-byte channel chunks per site
  static constexpr int RPT = 128 / XW;              // y-rows per M tile
  static constexpr int IR = TCR * RPT;              // y-rows per item
  // CA 8 stages one more halo row: the partner rows of the third tap row
  // (finite data, multiplied by zero weights)
  static constexpr int HY = IR + 2 + (CA == 8 ? 1 : 0);
  static constexpr bool GROUPED = XW < 128;
  static constexpr int POS = GROUPED ? XW / 8 * 10 : XW + 2;     // 16-byte positions per halo row and chunk
  static constexpr int SBO = GROUPED ? 160 : CM_BYTES;           // between core matrices along M
  static constexpr int ROW = GROUPED ? POS * 16 : CH * POS * 16;  // between halo y-rows
  static constexpr int CHK = GROUPED ? HY * POS * 16 : POS * 16;  // between channel chunks (K)
  static constexpr int A_PLANE = HY * CH * POS * 16;
  static constexpr int A_BYTES = NSLOT * A_PLANE;
  static constexpr int B_TAP = CH * B_CHUNK;        // 2 KB (CA 32) or 512 B (CA 8) per tap
  // CA 8: a zero chunk after the 27 taps partners the third tap row of a plane
  static constexpr int B_BYTES = 27 * B_TAP + (CA == 8 ? B_CHUNK : 0);
  static constexpr int SMEM = B_BYTES + A_BYTES + 64;  // + two mbarriers and the TMEM address
  static_assert(!GROUPED || (XW / 8) * SBO == ROW, "the core matrices of an M tile sit at one stride");
  static_assert(SMEM <= 227 * 1024, "shared memory per block");
};
constexpr int THREADS = 288;   // warps 0-7: copies and epilogue; warp 8: MMA issue
constexpr int WORKERS = 256;
constexpr uint32_t kSpinLimit = 1u << 20;

__device__ __forceinline__ uint32_t su32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void cp16(uint32_t saddr, const void* g) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(saddr), "l"(g) : "memory");
}

// shared-memory matrix descriptor, no swizzle, K-major
__device__ __forceinline__ uint64_t mdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version of this tensor-core generation
  return d;                // base offset 0, absolute LBO mode 0, layout SWIZZLE_NONE (0)
}

// instruction descriptor: kind::f16, A and B BF16, D FP32, both K-major, M = 128, N = 32
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((32u >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(kIdesc), "r"(acc));
}

__device__ __forceinline__ bool mbar_try(uint32_t addr, uint32_t phase) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(addr), "r"(phase)
      : "memory");
  return ok != 0;
}


// copies of halo plane z (periodic) of an item into ring slot `slot`
template <int CA, int XW>
__device__ __forceinline__ void load_plane(uint32_t a_s, int slot, const __nv_bfloat16* src, const ConvArgs& a,
                                           int x0, int y0, int z) {
  using G = TcGeom<CA, XW>;
  z = z < 0 ? z + a.nz : (z >= a.nz ? z - a.nz : z);
  const uint32_t base = a_s + slot * G::A_PLANE;
  if (threadIdx.x >= WORKERS) return;  // the MMA warp issues no copies
  for (int i = threadIdx.x; i < G::HY * G::POS * G::CH; i += WORKERS) {
    const int c = i % G::CH;
    const int s = i / G::CH;
    const int p = s % G::POS, hy = s / G::POS;
    // position p of a halo row holds x0 + hx - 1
    const int hx = G::GROUPED ? 8 * (p / 10) + p % 10 : p;
    int x = x0 + hx - 1, y = y0 + hy - 1;
    x = x < 0 ? x + a.nx : (x >= a.nx ? x - a.nx : x);
    y = y < 0 ? y + a.ny : (y >= a.ny ? y - a.ny : y);
    cp16(base + hy * G::ROW + c * G::CHK + p * 16, src + (((int64_t)z * a.ny + y) * a.nx + x) * CA + c * 8);
  }
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}

template <int CA, int XW, int EPI, bool STORE_Z>
__global__ void __launch_bounds__(THREADS, 1) conv_tc_kernel(ConvArgs a, int zc, int* err) {
  using G = TcGeom<CA, XW>;
  constexpr int CHK = G::CHK, ROW = G::ROW, SBO = G::SBO, A_PLANE = G::A_PLANE, B_TAP = G::B_TAP;
  constexpr int RPT = G::RPT, IR = G::IR;
  constexpr int B_BYTES = G::B_BYTES, A_BYTES = G::A_BYTES;
  extern __shared__ __align__(1024) unsigned char sm[];
  uint64_t* mbar = reinterpret_cast<uint64_t*>(sm + B_BYTES + A_BYTES);  // [2]
  uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + B_BYTES + A_BYTES + 32);
  volatile int* abort = reinterpret_cast<volatile int*>(sm + B_BYTES + A_BYTES + 48);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t b_s = su32(sm), a_s = su32(sm + B_BYTES);
  const uint32_t mb[2] = {su32(mbar), su32(mbar + 1)};

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(su32(tslot)),
                 "r"(TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
  }
  if (tid == 0) {
    *abort = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(mb[0]));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(mb[1]));
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  // weights [tap][co][ci] (global) -> [tap][ci chunk][co][8] (shared)
  for (int i = tid; i < 27 * 32 * G::CH; i += THREADS) {
    const int tap = i / (32 * G::CH), r = i % (32 * G::CH), n = r / G::CH, c = r % G::CH;
    cp16(b_s + tap * B_TAP + c * B_CHUNK + n * 16, a.w + ((int64_t)tap * 32 + n) * CA + c * 8);
  }
  if constexpr (CA == 8)  // the zero chunk (made visible to the tensor core by the fence of step 0)
    for (int i = tid; i < B_CHUNK / 16; i += THREADS)
      *reinterpret_cast<uint4*>(sm + 27 * B_TAP + i * 16) = make_uint4(0, 0, 0, 0);
  asm volatile("cp.async.commit_group;\n" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = *tslot;

  // epilogue geometry: warp w -> TMEM lanes 32 (w & 3) (sites), columns 16 (w >> 2) (channels)
  const int quarter = warp & 3, half = warp >> 2;
  float2 bias[8];
#pragma unroll
  for (int n = 0; n < 8; ++n)
    bias[n] = (EPI == EPI_GELU && a.bias && warp < 8) ? make_float2(a.bias[16 * half + 2 * n], a.bias[16 * half + 2 * n + 1])
                                                       : make_float2(0.f, 0.f);

  const int tiles_x = a.nx / XW, tiles_y = a.ny / IR, zchunks = (a.nz + zc - 1) / zc;
  const int64_t items_per = (int64_t)tiles_x * tiles_y * zchunks;
  const int64_t nitems = items_per * a.nlat;
  const int64_t Nsite = (int64_t)a.nx * a.ny * a.nz;
  uint32_t phase[2] = {0, 0};
  int pending[2] = {0, 0};  // commits not yet waited for, per TMEM buffer
  bool failed = false;

  auto epilogue = [&](int buf, int64_t lat_base, int x0, int y0, int z) {
    const int m = 32 * quarter + lane;  // TMEM lane = row of the M tile
    const int x = x0 + m % XW;
#pragma unroll 1
    for (int r = 0; r < TCR; ++r) {
      uint32_t v[16];
      const uint32_t taddr = tmem + ((uint32_t)(32 * quarter) << 16) + buf * 64 + r * 32 + 16 * half;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
            "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
      const int64_t s = lat_base + ((int64_t)z * a.ny + (y0 + r * RPT + m / XW)) * a.nx + x;
      __align__(16) __nv_bfloat162 o[8];
      if constexpr (EPI == EPI_GELU) {
        __align__(16) __nv_bfloat162 zz[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const float2 zf = __fadd2_rn(make_float2(__uint_as_float(v[2 * j]), __uint_as_float(v[2 * j + 1])), bias[j]);
          zz[j] = __float22bfloat162_rn(zf);
          o[j] = __float22bfloat162_rn(gelu_t2(zf));
        }
        if constexpr (STORE_Z) {
          uint4* zp = reinterpret_cast<uint4*>(a.zout + s * 32 + 16 * half);
          zp[0] = reinterpret_cast<const uint4*>(zz)[0];
          zp[1] = reinterpret_cast<const uint4*>(zz)[1];
        }
      } else {  // EPI_BWD: times GELU'(z) of the layer's stored pre-activation
        __align__(16) __nv_bfloat162 zz[8];
        const uint4* zp = reinterpret_cast<const uint4*>(a.zin + s * 32 + 16 * half);
        reinterpret_cast<uint4*>(zz)[0] = zp[0];
        reinterpret_cast<uint4*>(zz)[1] = zp[1];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const float2 g = gelu_t_d2(__bfloat1622float2(zz[j]));
          o[j] = __float22bfloat162_rn(
              __fmul2_rn(make_float2(__uint_as_float(v[2 * j]), __uint_as_float(v[2 * j + 1])), g));
        }
      }
      uint4* op = reinterpret_cast<uint4*>(a.out + s * 32 + 16 * half);
      op[0] = reinterpret_cast<const uint4*>(o)[0];
      op[1] = reinterpret_cast<const uint4*>(o)[1];
    }
  };

  for (int64_t item = blockIdx.x; item < nitems && !failed; item += gridDim.x) {
    const int64_t li = item / items_per;
    int64_t rr = item % items_per;
    const int tx = (int)(rr % tiles_x);
    rr /= tiles_x;
    const int ty = (int)(rr % tiles_y);
    const int tz = (int)(rr / tiles_y);
    const int x0 = tx * XW, y0 = ty * IR, zA = tz * zc;
    const int nzs = min(zc, a.nz - zA);
    const __nv_bfloat16* src = a.in + li * Nsite * CA;
    const int64_t lat_base = li * Nsite;
    // planes q = -1, 0, 1 of the item (q = z - zA) into slots (q + 1) & 3
    load_plane<CA, XW>(a_s, 0, src, a, x0, y0, zA - 1);
    load_plane<CA, XW>(a_s, 1, src, a, x0, y0, zA);
    load_plane<CA, XW>(a_s, 2, src, a, x0, y0, zA + 1);
#pragma unroll 1
    for (int j = 0; j <= nzs; ++j) {
      const int buf = j & 1;
      if (j < nzs) {
        // planes j-1 .. j+1 have landed (only they are outstanding here)
        asm volatile("cp.async.wait_group 0;\n" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
        __syncthreads();
        if (*abort) {  // read after the barrier: every thread sees the same value
          failed = true;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        if (warp == 8 && lane == 0) {
          // descriptors are affine in the start address: one base per operand and
          // plane slot, compile-time offsets for the taps (the start-address field
          // never carries: shared addresses stay below 256 KB)
#pragma unroll
          for (int r = 0; r < TCR; ++r) {
            const uint32_t d = tmem + buf * 64 + r * 32;
            if constexpr (CA == 32) {
              const uint64_t bd0 = mdesc(b_s, B_CHUNK, CM_BYTES);
              uint64_t ad0[3];
#pragma unroll
              for (int dz = 0; dz < 3; ++dz)
                ad0[dz] = mdesc(a_s + ((j + dz) & 3) * A_PLANE + r * RPT * ROW, CHK, SBO);
#pragma unroll
              for (int tap = 0; tap < 27; ++tap) {
                const int dz = tap / 9, dy = (tap / 3) % 3, dx = tap % 3;
#pragma unroll
                for (int k = 0; k < 2; ++k) {
                  const uint64_t ad = ad0[dz] + (uint64_t)((dy * ROW + dx * 16 + 2 * k * CHK) >> 4);
                  const uint64_t bd = bd0 + (uint64_t)((tap * B_TAP + 2 * k * B_CHUNK) >> 4);
                  mma_bf16(d, ad, bd, (tap | k) ? 1u : 0u);
                }
              }
            } else {
              // 8 channels per tap: one K16 step takes the taps (dy 0, dx) and
              // (dy 1, dx) of a plane, the second 8-channel core matrix of A and
              // B one halo row and three taps further (LBO); the taps (dy 2, dx)
              // pair with the row below (finite data) times the zero chunk of B
#pragma unroll
              for (int dz = 0; dz < 3; ++dz) {
                const uint32_t abase = a_s + ((j + dz) & 3) * A_PLANE + r * RPT * ROW;
#pragma unroll
                for (int p = 0; p < 6; ++p) {
                  const int dx = p % 3, dy = p < 3 ? 0 : 2;
                  const int tap0 = dz * 9 + dy * 3 + dx;
                  const uint32_t lbo_b = p < 3 ? (uint32_t)(3 * B_TAP) : (uint32_t)((27 - tap0) * B_TAP);
                  const uint64_t ad = mdesc(abase + dy * ROW + dx * 16, ROW, SBO);
                  const uint64_t bd = mdesc(b_s + tap0 * B_TAP, lbo_b, CM_BYTES);
                  mma_bf16(d, ad, bd, (dz | p) ? 1u : 0u);
                }
              }
            }
          }
          asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                           mb[buf])
                       : "memory");
        }
        pending[buf] = 1;
      }
      if (j >= 1) {
        const int pb = (j - 1) & 1;
        // bounded wait, agreed within the warp (tcgen05.ld is warp-collective);
        // the MMA warp goes straight to the barrier
        uint32_t spins = 0;
        int to = 0;
        while (warp < 8 && !mbar_try(mb[pb], phase[pb])) {
          if (++spins > kSpinLimit) {
            to = 1;
            break;
          }
        }
        if (warp == 8) {
          // no TMEM reads, no copies
        } else if (__any_sync(0xffffffffu, to)) {
          if (lane == 0) *abort = 1;
        } else {
          phase[pb] ^= 1u;
          pending[pb] = 0;
          // the slot of plane j-2 is free: prefetch plane j+2 behind the epilogue
          if (j + 2 <= nzs) load_plane<CA, XW>(a_s, (j + 3) & 3, src, a, x0, y0, zA + j + 2);
          asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
          epilogue(pb, lat_base, x0, y0, zA + j - 1);
        }
        // TMEM buffer pb is read before MMA(j + 1) overwrites it
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
        __syncthreads();
        if (*abort) {
          failed = true;
          break;
        }
      } else if (2 <= nzs) {
        // j == 0: slot 3 is free; prefetch plane 2
        load_plane<CA, XW>(a_s, 3, src, a, x0, y0, zA + 2);
      }
    }
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    __syncthreads();
  }
  if (failed) {
    if (tid == 0) atomicOr(err, 1);
    // MMAs of a buffer that was not waited for may still be running (the
    // worker warps track the phases; the MMA warp does not wait)
    for (int b = 0; b < 2 && warp < 8; ++b) {
      if (!pending[b]) continue;
      uint32_t spins = 0;
      while (!mbar_try(mb[b], phase[b]) && ++spins < kSpinLimit) {
      }
    }
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TMEM_COLS));
  }
}

// x-row width of the item layout for an nx-wide lattice (0: no layout fits)
int tc_xw(int nx, int ny) {
  if (nx % 128 == 0 && ny % TcGeom<32, 128>::IR == 0) return 128;
  if (nx % 64 == 0 && ny % TcGeom<32, 64>::IR == 0) return 64;
  return 0;
}

// z-planes per item: the fewest rounds of items over the SMs, counting the
// item's pipeline fill (three plane copies, no epilogue) as one step
int tc_zc(int64_t items_xy, int nz, int nsm) {
  int best = ZC_MAX;
  int64_t best_cost = -1;
  for (int zc = ZC_MAX; zc >= 4; zc /= 2) {
    const int64_t items = items_xy * ((nz + zc - 1) / zc);
    const int64_t cost = ((items + nsm - 1) / nsm) * (std::min(zc, nz) + 1);
    if (best_cost < 0 || cost < best_cost) best_cost = cost, best = zc;
  }
  return best;
}

template <int XW>
int conv_tc_go(const ConvArgs& a, int ca, int epi, int nsm, int* err, cudaStream_t s) {
  const bool sz = a.zout != nullptr;
  const int64_t items_xy = (int64_t)(a.nx / XW) * (a.ny / TcGeom<32, XW>::IR) * a.nlat;
  const int zc = tc_zc(items_xy, a.nz, nsm);
  auto go = [&](auto kern, int smem) -> int {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return cuda_fail(e, "tcgen05 conv smem attribute");
    const int64_t nitems = items_xy * ((a.nz + zc - 1) / zc);
    const unsigned grid = (unsigned)std::min<int64_t>(nitems, (int64_t)nsm);
    kern<<<grid, THREADS, smem, s>>>(a, zc, err);
    if (g_launch_counter) ++*g_launch_counter;
    e = cudaGetLastError();
    return e == cudaSuccess ? LAT_OK : cuda_fail(e, "tcgen05 conv launch");
  };
  if (ca == 8) {
    constexpr int sm8 = TcGeom<8, XW>::SMEM;
    if (epi == EPI_BWD) return go(conv_tc_kernel<8, XW, EPI_BWD, false>, sm8);
    return sz ? go(conv_tc_kernel<8, XW, EPI_GELU, true>, sm8) : go(conv_tc_kernel<8, XW, EPI_GELU, false>, sm8);
  }
  constexpr int sm32 = TcGeom<32, XW>::SMEM;
  if (epi == EPI_GELU)
    return sz ? go(conv_tc_kernel<32, XW, EPI_GELU, true>, sm32) : go(conv_tc_kernel<32, XW, EPI_GELU, false>, sm32);
  return go(conv_tc_kernel<32, XW, EPI_BWD, false>, sm32);
}

}  // namespace

bool conv_tc_ok(int ca, int cb, int epi, int nx, int ny) {
  if (!tc_xw(nx, ny) || cb != 32 || epi == EPI_LINEAR) return false;
  return ca == 32 || ca == 8;
}

int conv_tc(const ConvArgs& a, int ca, int epi, int nsm, int* err, cudaStream_t s) {
  const int xw = tc_xw(a.nx, a.ny);
  if (xw == 128) return conv_tc_go<128>(a, ca, epi, nsm, err, s);
  if (xw == 64) return conv_tc_go<64>(a, ca, epi, nsm, err, s);
  return set_error(LAT_ERR_ARG, "tcgen05 conv: nx % 64");
}

}  // namespace net
}  // namespace lat
