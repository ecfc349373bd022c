// k_fd.cu -- finite-difference kick / kick+drift passes (sm_103a).
//
// Restates Hamiltonian_fields_grad_pot + Hamiltonian_fields_kin of
// Discrete/Bubble-Collisions/evolve.f90:244-281 (Minkowski) and
// Pseudospec/openmp_dev/hamiltonian_conformal.f90:176-205 (conformal) with the
// STENCIL macro of Discrete/Bubble-Collisions/macros.h:31-44.  Periodic wrap is
// index arithmetic on the staged tile: no ghost copies (wrap_field,
// scafld.f90:120-192) are made.
//
// Decomposition of the 27-point operator: for every plane keep per site
//   c  = centre, s1 = sum of the 4 in-plane face neighbours,
//   s2 = sum of the 4 in-plane corner neighbours;
// then  RANK1 = s1(z) + c(z-1) + c(z+1),  RANK2 = s2(z) + s1(z-1) + s1(z+1),
//       RANK3 = s2(z-1) + s2(z+1).
// Each plane is staged once in shared memory (9 reads per site) and the
// (c,s1,s2) of planes z-1, z, z+1 live in registers while the tile marches in z.
// FP32 lattices whose rows are whole tiles stage the 32 interior values of a
// row with 16-byte copies into rows of 40 (interior at column 4, halo at 3
// and 36) and the two halo values with 4-byte copies; otherwise every value
// is a 4-byte copy into rows of 34.
#include "engine.hpp"

namespace lat {

namespace {

__device__ __forceinline__ int pmod(int i, int n) {
  int r = i % n;
  return r < 0 ? r + n : r;
}

__device__ __forceinline__ void cp_async_elem(void* smem, const void* gmem, int bytes) {
  const unsigned int sa = (unsigned int)__cvta_generic_to_shared(smem);
  if (bytes == 8) asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gmem) : "memory");
  else asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned int sa = (unsigned int)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int G> __device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(G) : "memory");
}

constexpr int kFdMaxSlots = 4;  // halo'd plane elements one thread stages per plane (covers ty >= 2)

template <typename R, bool KAHAN, int NF, bool GW, bool SEVEN, int MODE>
__global__ void __launch_bounds__(512) fd_kernel(FdArgs a) {
  // launched as a programmatic dependent: every array may have been written
  // by the previous pass, so nothing is read before the wait; the next pass
  // (usually the next step's) launches while this one runs
  pdl_wait();
  pdl_trigger();
  constexpr int NC = NF + (GW ? 6 : 0);
  constexpr int TX = 32;
  const int TY = blockDim.y;
  const bool vec = a.vec != 0;
  const int Wd = vec ? 40 : TX + 2, XO = vec ? 4 : 1, PL = Wd * (TY + 2);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  R* sm = reinterpret_cast<R*>(smem_raw);  // [3][NC][PL]: ring of planes z-1, z, z+1 (and the one in flight)

  const int nx = a.nx, ny = a.ny, nz = a.nz;
  const int64_t N = (int64_t)nx * ny * nz;
  const int64_t plane = (int64_t)nx * ny;
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int tid = tx + TX * ty, nthr = TX * TY;
  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
  const int zend = a.zhi > 0 ? a.zhi : nz;  // planes [a.zlo, zend) are computed
  const int z0 = a.zlo + blockIdx.z * a.zc;
  const int z1 = min(z0 + a.zc, zend);
  const int x = x0 + tx, y = y0 + ty;
  const bool active = (x < nx) && (y < ny);

  const R* phi = static_cast<const R*>(a.phi_in);
  const R* uin = static_cast<const R*>(a.u_in);

  // in-plane offsets (periodic wrap) of the tile elements this thread stages;
  // the same for every plane, so the wrap arithmetic runs once per block
  int slot_off[kFdMaxSlots];
  int nslot = 0;
  // 16-byte staging: thread tid copies interior chunk tid (8 per row) or, after
  // those, one halo value (2 per row); v_kind 1 / 2 / 0 (none)
  int v_kind = 0, v_dst = 0, v_src = 0;
  if (vec) {
    const int nch = 8 * (TY + 2);
    if (tid < nch) {
      const int r = tid >> 3, ch = tid & 7;
      v_kind = 1;
      v_dst = r * Wd + 4 + 4 * ch;
      v_src = pmod(y0 + r - 1, ny) * nx + x0 + 4 * ch;
    } else if (tid < nch + 2 * (TY + 2)) {
      const int h = tid - nch, r = h >> 1, side = h & 1;
      v_kind = 2;
      v_dst = r * Wd + (side ? 36 : 3);
      v_src = pmod(y0 + r - 1, ny) * nx + pmod(side ? x0 + TX : x0 - 1, nx);
    }
  } else {
#pragma unroll
    for (int k = 0; k < kFdMaxSlots; ++k) {
      const int i = tid + k * nthr;
      slot_off[k] = 0;
      if (i < PL) {
        const int r = i / Wd, cc = i - r * Wd;
        const int gx = pmod(x0 + cc - 1, nx), gy = pmod(y0 + r - 1, ny);
        slot_off[k] = gy * nx + gx;
        nslot = k + 1;
      }
    }
  }
  // issue the asynchronous copy of plane z into ring buffer b
  auto load_plane = [&](int z, int b) {
    const int64_t zo = (int64_t)pmod(z, nz) * plane;
    if (vec) {
      if (v_kind) {
#pragma unroll
        for (int c = 0; c < NC; ++c) {
          const R* src = (c < NF ? phi + (int64_t)c * N : uin + (int64_t)(c - NF) * N) + zo + v_src;
          R* dst = sm + (b * NC + c) * PL + v_dst;
          if (v_kind == 1) cp_async16(dst, src);
          else cp_async_elem(dst, src, (int)sizeof(R));
        }
      }
      cp_async_commit();
      return;
    }
#pragma unroll
    for (int k = 0; k < kFdMaxSlots; ++k) {
      if (k < nslot) {
        const int i = tid + k * nthr;
#pragma unroll
        for (int c = 0; c < NC; ++c) {
          const R* src = c < NF ? phi + (int64_t)c * N : uin + (int64_t)(c - NF) * N;
          cp_async_elem(sm + (b * NC + c) * PL + i, src + zo + slot_off[k], (int)sizeof(R));
        }
      }
    }
    cp_async_commit();
  };

  R wc[NC][3], ws1[NC][3], ws2[NC][3];
  R gxw[NF][2], gyw[NF][2];  // in-plane phi differences of planes z (slot 0) and z+1 (slot 1)
  const int ctr = (ty + 1) * Wd + (tx + XO);

  auto fill = [&](int b, int slot) {
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      const R* p = sm + (b * NC + c) * PL;
      wc[c][slot] = p[ctr];
      ws1[c][slot] = (p[ctr - 1] + p[ctr + 1]) + (p[ctr - Wd] + p[ctr + Wd]);
      if (!SEVEN) ws2[c][slot] = (p[ctr - Wd - 1] + p[ctr - Wd + 1]) + (p[ctr + Wd - 1] + p[ctr + Wd + 1]);
      else ws2[c][slot] = R(0);
    }
    if (GW) {
#pragma unroll
      for (int f = 0; f < NF; ++f) {
        const R* p = sm + (b * NC + f) * PL;
        gxw[f][slot == 2 ? 1 : 0] = p[ctr + 1] - p[ctr - 1];
        gyw[f][slot == 2 ? 1 : 0] = p[ctr + Wd] - p[ctr - Wd];
      }
    }
  };

  const R l0 = (R)a.lc[0], l1 = (R)a.lc[1], l2 = (R)a.lc[2], l3 = (R)a.lc[3];
  R ck = (R)a.hk, cv = (R)a.hk;
  const R cd = (R)a.hd;
  double a_conf = 1.0;
  if (MODE == 2) {
    a_conf = a.sc->a;
    ck = (R)(a.hk * a_conf * a_conf);
    cv = (R)(a.hk * a_conf * a_conf * a_conf * a_conf);
  }
  const R kap = (R)a.kappa, i2 = (R)a.inv2dx;
  using Acc = typename AccOf<R>::type;
  Acc acc_ge, acc_pe;

  // ring: plane p (counted from z0-1) lives in buffer p % 3; two planes are in
  // flight ahead of the one being filled
  load_plane(z0 - 1, 0);
  load_plane(z0, 1);
  load_plane(z0 + 1, 2);
  cp_async_wait<2>();
  __syncthreads();
  fill(0, 0);
  cp_async_wait<1>();
  __syncthreads();
  fill(1, 1);

  R* pi = static_cast<R*>(a.pi);
  R* phio = static_cast<R*>(a.phi_out);
  R* phic = static_cast<R*>(a.phic);
  R* pu = static_cast<R*>(a.pu);
  R* uo = static_cast<R*>(a.u_out);

  for (int z = z0; z < z1; ++z) {
    const int bnext = (z - z0 + 2) % 3;  // buffer of plane z+1
    const int64_t s = ((int64_t)z * ny + y) * nx + x;
    // this site's pointwise state, requested before the wait so that it lands
    // while the plane ring catches up
    R piv[NF], cpv[NF], puv[GW ? 6 : 1];
    if (active) {
#pragma unroll
      for (int l = 0; l < NF; ++l) {
        piv[l] = pi[(int64_t)l * N + s];
        cpv[l] = (KAHAN && MODE == 0) ? phic[(int64_t)l * N + s] : R(0);
      }
      if (GW) {
#pragma unroll
        for (int g = 0; g < 6; ++g) puv[g] = pu[(int64_t)g * N + s];
      }
    }
    // plane z+2 goes into the buffer of plane z-1, read two iterations ago
    if (z + 1 < z1) load_plane(z + 2, (z - z0 + 3) % 3);
    else cp_async_commit();  // keep one group per iteration
    cp_async_wait<1>();
    __syncthreads();
    fill(bnext, 2);
    if (active) {
      R lap[NC];
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        R r1 = ws1[c][1] + (wc[c][0] + wc[c][2]);
        R v = l0 * wc[c][1] + l1 * r1;
        if (!SEVEN) {
          R r2 = ws2[c][1] + (ws1[c][0] + ws1[c][2]);
          R r3 = ws2[c][0] + ws2[c][2];
          v += l2 * r2 + l3 * r3;
        }
        lap[c] = v;
      }
      R f[NF], dv[NF];
#pragma unroll
      for (int l = 0; l < NF; ++l) f[l] = wc[l][1];
      model_dv<R, NF>(a.model, f, dv);
#pragma unroll
      for (int l = 0; l < NF; ++l) {
        const int64_t sl = (int64_t)l * N + s;
        const R pn = piv[l] + (ck * lap[l] - cv * dv[l]);
        pi[sl] = pn;
        if (MODE == 0) {
          if constexpr (KAHAN) {
            R xv = f[l], cc = cpv[l];
            kahan_add(xv, cc, cd * pn);
            phio[sl] = xv;
            phic[sl] = cc;
          } else {
            phio[sl] = f[l] + cd * pn;
          }
        }
        if (MODE == 2) acc_ge.add(-f[l] * lap[l]);
      }
      if (MODE == 2) acc_pe.add(model_v<R, NF>(a.model, f));
      if (GW) {
        R dxp[NF], dyp[NF], dzp[NF];
#pragma unroll
        for (int l = 0; l < NF; ++l) {
          dxp[l] = gxw[l][0] * i2;
          dyp[l] = gyw[l][0] * i2;
          dzp[l] = (wc[l][2] - wc[l][0]) * i2;
        }
#pragma unroll
        for (int g = 0; g < 6; ++g) {
          R src = R(0);
#pragma unroll
          for (int l = 0; l < NF; ++l) {
            const R di = g == 0 || g == 3 || g == 4 ? dxp[l] : (g == 1 || g == 5 ? dyp[l] : dzp[l]);
            const R dj = g == 0 ? dxp[l] : (g == 1 || g == 3 ? dyp[l] : dzp[l]);
            src += di * dj;
          }
          const int64_t sg = (int64_t)g * N + s;
          const R pn = puv[g] + ck * (lap[NF + g] + kap * src);
          pu[sg] = pn;
          if (MODE == 0) uo[sg] = wc[NF + g][1] + cd * pn;
        }
      }
    }
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      wc[c][0] = wc[c][1]; wc[c][1] = wc[c][2];
      ws1[c][0] = ws1[c][1]; ws1[c][1] = ws1[c][2];
      ws2[c][0] = ws2[c][1]; ws2[c][1] = ws2[c][2];
    }
    if (GW) {
#pragma unroll
      for (int l = 0; l < NF; ++l) { gxw[l][0] = gxw[l][1]; gyw[l][0] = gyw[l][1]; }
    }
  }

  if (MODE == 2) {
    const typename Acc::Red v[2] = {acc_ge.red(), acc_pe.red()};
    double tot[2];
    if (grid_reduce<2>(v, a.rb, tot)) {
      DevScalars* sc = a.sc;
      if (a.defer) {  // a z-slab: the sums of all slabs complete the update on the host
        sc->red[13] = tot[0];
        sc->red[14] = tot[1];
        if (bad(tot[0]) || bad(tot[1])) sc->err |= 1u;
      } else {
        const double ac = sc->a;
        const double GE2 = tot[0] / (ac * ac) / a.Nd;
        const double PE = tot[1] / a.Nd;
        if (bad(GE2) || bad(PE)) sc->err |= 1u;
        sc->ap = sc->ap - ac * ac * ac * (GE2 + 4.0 * PE) * a.hk;
        sc->pe = PE;
      }
    }
  }
}

// FP32 lattices whose rows are multiples of 64 sites: the same pass with two
// x-sites per thread (tiles of 64 x TY sites).  A staged row is read as one
// 8-byte value (x, x+1) and two 4-byte values (x-1, x+2), six reads that
// serve both sites' 3 x 3 neighbourhoods; momenta, strains and outputs move
// as float2.  The z-window keeps, per array and site, two rolling partial
// sums instead of nine values (c, s1, s2 of three planes): when plane q
// arrives with (c, s1, s2), the Laplacian of plane q-1 completes with
// l1 c + l2 s1 + l3 s2, plane q starts from that same term plus
// l0 c + l1 s1 + l2 s2, and plane q+1 starts from l1 c + l2 s1 + l3 s2.
constexpr int kFd2Wd = 72;  // staged row: halo at 3, interior 4..67 (16-byte aligned), halo at 68

__device__ __forceinline__ void fd2_row(const float* row, int tx, float& l, float2& m, float& r) {
  m = *reinterpret_cast<const float2*>(row + 4 + 2 * tx);
  l = row[3 + 2 * tx];
  r = row[6 + 2 * tx];
}

template <bool KAHAN, int NF, bool GW, bool SEVEN, int MODE>
__global__ void __launch_bounds__(256) fd2_kernel(FdArgs a) {
  pdl_wait();  // a programmatic dependent, as fd_kernel
  pdl_trigger();
  using R = float;
  constexpr int NC = NF + (GW ? 6 : 0);
  constexpr int Wd = kFd2Wd;
  const int TY = blockDim.y;
  const int PL = Wd * (TY + 2);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  R* sm = reinterpret_cast<R*>(smem_raw);  // [3][NC][PL]: ring of planes

  const int nx = a.nx, ny = a.ny, nz = a.nz;
  const int64_t N = (int64_t)nx * ny * nz;
  const int64_t plane = (int64_t)nx * ny;
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int tid = tx + 32 * ty, nthr = 32 * TY;
  const int x0 = blockIdx.x * 64, y0 = blockIdx.y * TY;
  const int zend = a.zhi > 0 ? a.zhi : nz;
  const int z0 = a.zlo + blockIdx.z * a.zc;
  const int z1 = min(z0 + a.zc, zend);
  const int x = x0 + 2 * tx, y = y0 + ty;
  const bool active = y < ny;

  const R* phi = static_cast<const R*>(a.phi_in);
  const R* uin = static_cast<const R*>(a.u_in);

  // staging: per plane and array (TY + 2) rows of 16 interior 16-byte chunks
  // and 2 halo values; thread tid takes copies tid, tid + nthr, ...
  constexpr int kSlots = 3;
  int s_kind[kSlots], s_dst[kSlots], s_src[kSlots];
  const int ncopy = 18 * (TY + 2);
#pragma unroll
  for (int k = 0; k < kSlots; ++k) {
    const int i = tid + k * nthr;
    s_kind[k] = 0;
    s_dst[k] = 0;
    s_src[k] = 0;
    if (i < ncopy) {
      const int r = i / 18, c = i - 18 * r;
      const int gy = pmod(y0 + r - 1, ny);
      if (c < 16) {
        s_kind[k] = 1;
        s_dst[k] = r * Wd + 4 + 4 * c;
        s_src[k] = gy * nx + x0 + 4 * c;
      } else {
        s_kind[k] = 2;
        s_dst[k] = r * Wd + (c == 16 ? 3 : 68);
        s_src[k] = gy * nx + (c == 16 ? pmod(x0 - 1, nx) : pmod(x0 + 64, nx));
      }
    }
  }
  auto load_plane = [&](int z, int b) {
    const int64_t zo = (int64_t)pmod(z, nz) * plane;
#pragma unroll
    for (int k = 0; k < kSlots; ++k) {
      if (s_kind[k]) {
#pragma unroll
        for (int c = 0; c < NC; ++c) {
          const R* src = (c < NF ? phi + (int64_t)c * N : uin + (int64_t)(c - NF) * N) + zo + s_src[k];
          R* dst = sm + (b * NC + c) * PL + s_dst[k];
          if (s_kind[k] == 1) cp_async16(dst, src);
          else cp_async_elem(dst, src, 4);
        }
      }
    }
    cp_async_commit();
  };

  const R l0 = (R)a.lc[0], l1 = (R)a.lc[1], l2 = (R)a.lc[2], l3 = (R)a.lc[3];
  R ck = (R)a.hk, cv = (R)a.hk;
  const R cd = (R)a.hd;
  if (MODE == 2) {
    const double ac = a.sc->a;
    ck = (R)(a.hk * ac * ac);
    cv = (R)(a.hk * ac * ac * ac * ac);
  }
  const R kap = (R)a.kappa, i2 = (R)a.inv2dx;
  using Acc = typename AccOf<R>::type;
  Acc acc_ge, acc_pe;

  // rolling sums per array and site: P = Laplacian of the next output plane
  // so far, Q = the start of the plane after it
  R P[NC][2], Q[NC][2];
  R fc[NF][2][3];             // field values of planes z-1, z, z+1 (GW z-derivative, potential)
  R gx[NF][2], gy[NF][2];     // in-plane field differences of the output plane (GW)
  R uc[GW ? 6 : 1][2];        // strain of the output plane (drift)
  R ngx[NF][2], ngy[NF][2];

  // the values of plane buffer b: centre, s1, s2 of both sites for array c,
  // folded into the rolling sums by `take`
  auto read3 = [&](int b, int c, R (&cc)[2], R (&s1)[2], R (&s2)[2], R (&dx)[2], R (&dy)[2]) {
    const R* base = sm + (b * NC + c) * PL;
    float lu, ru, lm, rm, ld, rd;
    float2 mu, mm, md;
    fd2_row(base + ty * Wd, tx, lu, mu, ru);        // y - 1
    fd2_row(base + (ty + 1) * Wd, tx, lm, mm, rm);  // y
    fd2_row(base + (ty + 2) * Wd, tx, ld, md, rd);  // y + 1
    cc[0] = mm.x;
    cc[1] = mm.y;
    s1[0] = (lm + mm.y) + (mu.x + md.x);
    s1[1] = (mm.x + rm) + (mu.y + md.y);
    if (!SEVEN) {
      s2[0] = (lu + mu.y) + (ld + md.y);
      s2[1] = (mu.x + ru) + (md.x + rd);
    } else {
      s2[0] = s2[1] = R(0);
    }
    dx[0] = mm.y - lm;
    dx[1] = rm - mm.x;
    dy[0] = md.x - mu.x;
    dy[1] = md.y - mu.y;
  };

  load_plane(z0 - 1, 0);
  load_plane(z0, 1);
  load_plane(z0 + 1, 2);
  cp_async_wait<2>();
  __syncthreads();
#pragma unroll
  for (int c = 0; c < NC; ++c) {  // plane z0 - 1: the start of P
    R cc[2], s1[2], s2[2], dx[2], dy[2];
    read3(0, c, cc, s1, s2, dx, dy);
#pragma unroll
    for (int j = 0; j < 2; ++j) P[c][j] = l1 * cc[j] + l2 * s1[j] + l3 * s2[j];
    if (c < NF) {
      fc[c][0][0] = cc[0];
      fc[c][1][0] = cc[1];
    }
  }
  cp_async_wait<1>();
  __syncthreads();
#pragma unroll
  for (int c = 0; c < NC; ++c) {  // plane z0: its own term into P, the start of Q
    R cc[2], s1[2], s2[2], dx[2], dy[2];
    read3(1, c, cc, s1, s2, dx, dy);
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      P[c][j] += l0 * cc[j] + l1 * s1[j] + l2 * s2[j];
      Q[c][j] = l1 * cc[j] + l2 * s1[j] + l3 * s2[j];
    }
    if (c < NF) {
      fc[c][0][1] = cc[0];
      fc[c][1][1] = cc[1];
      gx[c][0] = dx[0]; gx[c][1] = dx[1];
      gy[c][0] = dy[0]; gy[c][1] = dy[1];
    } else if (GW) {
      uc[c - NF][0] = cc[0];
      uc[c - NF][1] = cc[1];
    }
  }

  R* pi = static_cast<R*>(a.pi);
  R* phio = static_cast<R*>(a.phi_out);
  R* phic = static_cast<R*>(a.phic);
  R* pu = static_cast<R*>(a.pu);
  R* uo = static_cast<R*>(a.u_out);

  for (int z = z0; z < z1; ++z) {
    const int bnext = (z - z0 + 2) % 3;  // buffer of plane z+1
    const int64_t s = ((int64_t)z * ny + y) * nx + x;
    float2 piv[NF], cpv[NF], puv[GW ? 6 : 1];
    if (active) {
#pragma unroll
      for (int l = 0; l < NF; ++l) {
        piv[l] = *reinterpret_cast<const float2*>(pi + (int64_t)l * N + s);
        cpv[l] = (KAHAN && MODE == 0) ? *reinterpret_cast<const float2*>(phic + (int64_t)l * N + s)
                                      : make_float2(0.f, 0.f);
      }
      if (GW) {
#pragma unroll
        for (int g = 0; g < 6; ++g) puv[g] = *reinterpret_cast<const float2*>(pu + (int64_t)g * N + s);
      }
    }
    if (z + 1 < z1) load_plane(z + 2, (z - z0 + 3) % 3);
    else cp_async_commit();
    cp_async_wait<1>();
    __syncthreads();
    R lap[NC][2];
#pragma unroll
    for (int c = 0; c < NC; ++c) {  // plane z+1 completes the Laplacian of plane z
      R cc[2], s1[2], s2[2], dx[2], dy[2];
      read3(bnext, c, cc, s1, s2, dx, dy);
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const R t = l1 * cc[j] + l2 * s1[j] + l3 * s2[j];
        lap[c][j] = P[c][j] + t;
        P[c][j] = Q[c][j] + (l0 * cc[j] + l1 * s1[j] + l2 * s2[j]);
        Q[c][j] = t;
      }
      if (c < NF) {
        fc[c][0][2] = cc[0];
        fc[c][1][2] = cc[1];
        ngx[c][0] = dx[0]; ngx[c][1] = dx[1];
        ngy[c][0] = dy[0]; ngy[c][1] = dy[1];
      }
    }
    if (active) {
      float2 pn2[NF];
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        R f[NF], dv[NF];
#pragma unroll
        for (int l = 0; l < NF; ++l) f[l] = fc[l][j][1];
        model_dv<R, NF>(a.model, f, dv);
#pragma unroll
        for (int l = 0; l < NF; ++l) {
          const R pv = j == 0 ? piv[l].x : piv[l].y;
          const R pn = pv + (ck * lap[l][j] - cv * dv[l]);
          if (j == 0) pn2[l].x = pn; else pn2[l].y = pn;
          if (MODE == 2) acc_ge.add(-f[l] * lap[l][j]);
        }
        if (MODE == 2) acc_pe.add(model_v<R, NF>(a.model, f));
      }
#pragma unroll
      for (int l = 0; l < NF; ++l) {
        const int64_t sl = (int64_t)l * N + s;
        *reinterpret_cast<float2*>(pi + sl) = pn2[l];
        if (MODE == 0) {
          float2 xo, co;
          if constexpr (KAHAN) {
            R xv = fc[l][0][1], cc = cpv[l].x;
            kahan_add(xv, cc, cd * pn2[l].x);
            xo.x = xv; co.x = cc;
            xv = fc[l][1][1]; cc = cpv[l].y;
            kahan_add(xv, cc, cd * pn2[l].y);
            xo.y = xv; co.y = cc;
            *reinterpret_cast<float2*>(phic + sl) = co;
          } else {
            xo.x = fc[l][0][1] + cd * pn2[l].x;
            xo.y = fc[l][1][1] + cd * pn2[l].y;
          }
          *reinterpret_cast<float2*>(phio + sl) = xo;
        }
      }
      if (GW) {
#pragma unroll
        for (int g = 0; g < 6; ++g) {
          float2 pg, ug;
#pragma unroll
          for (int j = 0; j < 2; ++j) {
            R src = R(0);
#pragma unroll
            for (int l = 0; l < NF; ++l) {
              const R dxp = gx[l][j] * i2, dyp = gy[l][j] * i2, dzp = (fc[l][j][2] - fc[l][j][0]) * i2;
              const R di = g == 0 || g == 3 || g == 4 ? dxp : (g == 1 || g == 5 ? dyp : dzp);
              const R dj = g == 0 ? dxp : (g == 1 || g == 3 ? dyp : dzp);
              src += di * dj;
            }
            const R pv = j == 0 ? puv[g].x : puv[g].y;
            const R pn = pv + ck * (lap[NF + g][j] + kap * src);
            if (j == 0) { pg.x = pn; ug.x = uc[g][0] + cd * pn; }
            else { pg.y = pn; ug.y = uc[g][1] + cd * pn; }
          }
          const int64_t sg = (int64_t)g * N + s;
          *reinterpret_cast<float2*>(pu + sg) = pg;
          if (MODE == 0) *reinterpret_cast<float2*>(uo + sg) = ug;
        }
      }
    }
    // the window moves one plane up
#pragma unroll
    for (int l = 0; l < NF; ++l) {
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        fc[l][j][0] = fc[l][j][1];
        fc[l][j][1] = fc[l][j][2];
        gx[l][j] = ngx[l][j];
        gy[l][j] = ngy[l][j];
      }
    }
    if (GW) {  // strain of the next output plane, from the buffer just read
#pragma unroll
      for (int g = 0; g < 6; ++g) {
        const R* base = sm + (bnext * NC + NF + g) * PL + (ty + 1) * Wd + 4 + 2 * tx;
        const float2 v = *reinterpret_cast<const float2*>(base);
        uc[g][0] = v.x;
        uc[g][1] = v.y;
      }
    }
  }

  if (MODE == 2) {
    const typename Acc::Red v[2] = {acc_ge.red(), acc_pe.red()};
    double tot[2];
    if (grid_reduce<2>(v, a.rb, tot)) {
      DevScalars* sc = a.sc;
      if (a.defer) {
        sc->red[13] = tot[0];
        sc->red[14] = tot[1];
        if (bad(tot[0]) || bad(tot[1])) sc->err |= 1u;
      } else {
        const double ac = sc->a;
        const double GE2 = tot[0] / (ac * ac) / a.Nd;
        const double PE = tot[1] / a.Nd;
        if (bad(GE2) || bad(PE)) sc->err |= 1u;
        sc->ap = sc->ap - ac * ac * ac * (GE2 + 4.0 * PE) * a.hk;
        sc->pe = PE;
      }
    }
  }
}

template <bool KAHAN, int NF, bool GW, bool SEVEN, int MODE>
int go2(const FdArgs& a, cudaStream_t s, int* nb) {
  constexpr int NC = NF + (GW ? 6 : 0);
  const int nzc = (a.zhi > 0 ? a.zhi : a.nz) - a.zlo;
  if (a.zlo < 0 || nzc < 1 || a.zlo + nzc > a.nz) return set_error(LAT_ERR_ARG, "FD plane range");
  if (a.ty < 1 || a.ty > 8) return set_error(LAT_ERR_ARG, "FD tile of two sites per thread: 1 <= ty <= 8");
  dim3 block(32, a.ty);
  dim3 grid(a.nx / 64, (a.ny + a.ty - 1) / a.ty, (nzc + a.zc - 1) / a.zc);
  const size_t smem = (size_t)3 * NC * kFd2Wd * (a.ty + 2) * sizeof(float);
  auto k = fd2_kernel<KAHAN, NF, GW, SEVEN, MODE>;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_fail(e, "fd2 smem attribute");
  }
  cudaError_t e = launch_pdl(k, grid, block, smem, s, a);
  if (e != cudaSuccess) return cuda_fail(e, "fd2 kernel launch");
  if (nb) *nb = grid.x * grid.y * grid.z;
  if (g_launch_counter) ++*g_launch_counter;
  e = cudaGetLastError();
  return e == cudaSuccess ? LAT_OK : cuda_fail(e, "fd2 kernel launch");
}

template <typename R, bool KAHAN, int NF, bool GW, bool SEVEN, int MODE>
int go(const FdArgs& a0, cudaStream_t s, int* nb) {
  constexpr int NC = NF + (GW ? 6 : 0);
  FdArgs a = a0;
  a.vec = (sizeof(R) == 4 && a.nx % 32 == 0) ? 1 : 0;  // whole 32-value rows, 16-byte aligned
  const int wd = a.vec ? 40 : 34;
  dim3 block(32, a.ty);
  const int nzc = (a.zhi > 0 ? a.zhi : a.nz) - a.zlo;  // planes computed
  if (a.zlo < 0 || nzc < 1 || a.zlo + nzc > a.nz) return set_error(LAT_ERR_ARG, "FD plane range");
  dim3 grid((a.nx + 31) / 32, (a.ny + a.ty - 1) / a.ty, (nzc + a.zc - 1) / a.zc);
  size_t smem = (size_t)3 * NC * wd * (a.ty + 2) * sizeof(R);
  if (a.ty < 1 || (!a.vec && 34 * (a.ty + 2) > kFdMaxSlots * 32 * a.ty))
    return set_error(LAT_ERR_ARG, "FD tile too narrow");
  auto k = fd_kernel<R, KAHAN, NF, GW, SEVEN, MODE>;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_fail(e, "fd smem attribute");
  }
  cudaError_t e = launch_pdl(k, grid, block, smem, s, a);
  if (e != cudaSuccess) return cuda_fail(e, "fd kernel launch");
  if (nb) *nb = grid.x * grid.y * grid.z;
  if (g_launch_counter) ++*g_launch_counter;
  e = cudaGetLastError();
  return e == cudaSuccess ? LAT_OK : cuda_fail(e, "fd kernel launch");
}

template <typename R, bool KAHAN, int NF>
int go_nf(const FdArgs& a, cudaStream_t s, int* nb) {
  const bool gw = a.u_in != nullptr;
  const int mode = a.conf ? 2 : (a.phi_out ? 0 : 1);
  if (gw && mode == 2) return set_error(LAT_ERR_UNSUPPORTED, "GW with conformal FD kick");
  // FP32 rows of whole 64-site tiles: two sites per thread (fd2_kernel)
  const bool two = sizeof(R) == 4 && a.nx % 64 == 0 && a.ty <= 8;  // up to 256 threads of <= 255 registers
#define LAT_FD_CASE(GWV, SEV)                                                          \
  if (mode == 0) return two ? go2<KAHAN, NF, GWV, SEV, 0>(a, s, nb) : go<R, KAHAN, NF, GWV, SEV, 0>(a, s, nb); \
  if (mode == 1) return two ? go2<KAHAN, NF, GWV, SEV, 1>(a, s, nb) : go<R, KAHAN, NF, GWV, SEV, 1>(a, s, nb);
  if (gw) {
    if (a.seven) { LAT_FD_CASE(true, true) } else { LAT_FD_CASE(true, false) }
  } else {
    if (a.seven) {
      LAT_FD_CASE(false, true)
      return two ? go2<KAHAN, NF, false, true, 2>(a, s, nb) : go<R, KAHAN, NF, false, true, 2>(a, s, nb);
    } else {
      LAT_FD_CASE(false, false)
      return two ? go2<KAHAN, NF, false, false, 2>(a, s, nb) : go<R, KAHAN, NF, false, false, 2>(a, s, nb);
    }
  }
#undef LAT_FD_CASE
  return set_error(LAT_ERR_ARG, "bad FD mode");
}

}  // namespace

int fd_max_blocks(int nx, int ny, int nz, int ty, int zc) {
  return ((nx + 31) / 32) * ((ny + ty - 1) / ty) * ((nz + zc - 1) / zc);
}

int launch_fd(const FdArgs& a, int precision, cudaStream_t s, int* nb) {
  if (a.nf == 1) {
    if (precision == LAT_FP64) return go_nf<double, false, 1>(a, s, nb);
    return go_nf<float, true, 1>(a, s, nb);
  }
  if (a.nf == 2) {
    if (precision == LAT_FP64) return go_nf<double, false, 2>(a, s, nb);
    return go_nf<float, true, 2>(a, s, nb);
  }
  return set_error(LAT_ERR_UNSUPPORTED, "FD passes support nfld = 1 or 2");
}

}  // namespace lat
