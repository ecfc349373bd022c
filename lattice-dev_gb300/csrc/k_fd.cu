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
  k<<<grid, block, smem, s>>>(a);
  if (nb) *nb = grid.x * grid.y * grid.z;
  if (g_launch_counter) ++*g_launch_counter;
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? LAT_OK : cuda_fail(e, "fd kernel launch");
}

template <typename R, bool KAHAN, int NF>
int go_nf(const FdArgs& a, cudaStream_t s, int* nb) {
  const bool gw = a.u_in != nullptr;
  const int mode = a.conf ? 2 : (a.phi_out ? 0 : 1);
  if (gw && mode == 2) return set_error(LAT_ERR_UNSUPPORTED, "GW with conformal FD kick");
#define LAT_FD_CASE(GWV, SEV)                                          \
  if (mode == 0) return go<R, KAHAN, NF, GWV, SEV, 0>(a, s, nb);       \
  if (mode == 1) return go<R, KAHAN, NF, GWV, SEV, 1>(a, s, nb);
  if (gw) {
    if (a.seven) { LAT_FD_CASE(true, true) } else { LAT_FD_CASE(true, false) }
  } else {
    if (a.seven) {
      LAT_FD_CASE(false, true)
      return go<R, KAHAN, NF, false, true, 2>(a, s, nb);
    } else {
      LAT_FD_CASE(false, false)
      return go<R, KAHAN, NF, false, false, 2>(a, s, nb);
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
