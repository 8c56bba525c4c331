// Persistent collocate / integrate kernels of the GB300 grid backend,
// orthorhombic cells (CP2K: src/grid/ref/grid_ref_collint.h:30-327).
//
// Work unit: one task (a pair of primitive Gaussians on one grid level) per
// warp.  Warps pull tasks from a queue ordered by decreasing predicted cost
// with one atomic per task; there is no CTA-wide synchronisation.
//
// The cube is traversed separably, mapped onto the warp: lane <-> x index of
// the cube (sub-warps exactly as wide as the cube, so narrow cubes process
// several rows at once), planes k and rows j sequential.  Per plane the z
// factor is folded into the coefficients (C_xy), per lane the x factor
// (q[ly]); the per-point work is lp+1 fused multiply-adds:
//   collocate:  rho(x,y,z) += sum_ly q[ly](x) * pol_y[ly](y)   (FP64 red)
//   integrate:  w[ly] += V(x,y,z) * pol_y[ly](y) per lane; folded with z per
//               plane and with x + a shared-memory transpose per task.
// Arithmetic type N: double (FP64 path), float (FP32 path) or dfloat (mixed
// path: FP32 pipes, ~48-bit significands).  The grid accumulation is FP64
// atomics in L2 for every N; dfloat adds its low words into an FP32 side grid
// that is folded into the FP64 grid at the end.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <type_traits>

#include "gb300_internal.h"
#include "numeric.cuh"

namespace gb300 {

namespace {

constexpr unsigned FULL = 0xffffffffu;

template <int LPB, typename T> constexpr int padded() {
  return sizeof(T) == 4 ? ((LPB + 1 + 3) & ~3) : ((LPB + 1 + 1) & ~1);
}

// Per-warp shared memory of the orthorhombic kernels.
template <typename N, int LPB> struct OrthoSmem {
  using T = typename Num<N>::T;
  static constexpr int P = LPB + 1;
  static constexpr int PP = padded<LPB, T>();
  static __host__ __device__ constexpr int red_stride() {
    return ((P * (P + 1)) / 2 + P) | 1;
  }
  // collocate: tables, coefficients, C_xy, periodic maps
  static __host__ __device__ size_t bytes_coll(int wmax) {
    size_t b = sizeof(T) * (3 * (size_t)wmax * PP + ntri(LPB) * P + ntri(LPB));
    b += sizeof(int) * 3 * (size_t)wmax;
    b += 64; // alignment slack
    return (b + 15) & ~size_t(15);
  }
  // collocate over point lists: as bytes_coll plus the per-plane x folds
  // q[x][ly] of every x of the cube
  static __host__ __device__ size_t bytes_coll_pl(int wmax) {
    return bytes_coll(wmax) + ((sizeof(T) * (size_t)wmax * PP + 15) & ~size_t(15));
  }
  // integrate: tables (reused as the x-fold transpose), maps, accumulator
  static __host__ __device__ size_t pol_words_int(int wmax) {
    const size_t a = 3 * (size_t)wmax * PP, r = 32 * (size_t)red_stride();
    return a > r ? a : r;
  }
  static __host__ __device__ size_t bytes_int(int wmax) {
    size_t b = sizeof(T) * pol_words_int(wmax);
    b += sizeof(int) * 3 * (size_t)wmax;
    b += sizeof(double) * ncoset(LPB);
    b += 64;
    return (b + 15) & ~size_t(15);
  }
};

// Copy an aligned table row of PP elements into registers with 16-byte loads.
template <typename T, int PP>
__device__ __forceinline__ void load_row(const T *src, T (&dst)[PP]) {
  static_assert((PP * sizeof(T)) % 16 == 0, "row not 16-byte sized");
  const float4 *s = reinterpret_cast<const float4 *>(src);
  float4 *d = reinterpret_cast<float4 *>(dst);
#pragma unroll
  for (int i = 0; i < (int)(PP * sizeof(T) / 16); i++)
    d[i] = s[i];
}

// The 1-D tables from the Gaussian along each line by the multiplicative
// recurrence of grid_ref_collint.h:262-293, run in dfloat by 6 lanes (3
// directions x 2 sides of c = 0) from exponentials the host evaluated in FP64:
// seed[dir] = {e(0), f_up(0), f_down(0), q, h, -roff} with
// e(c) = exp(-z (c h - r)^2), e(c +- 1) = e(c) f(c), f(c +- 1) = f(c) q.
// Stored as dfloat, or (T = float) rounded to FP32: an FP32 table whose
// relative error does not grow with the exponent z x^2, unlike expf of a
// rounded argument.
template <typename T, int LPB, int PP>
__device__ __forceinline__ void seeded_tables(int w, int cmax, int lp, T *pol, int lane,
                                              const float2 *seed) {
  if (lane < 6) {
    const int dir = lane >> 1, up = lane & 1;
    const float2 *sd = seed + 6 * dir;
    dfloat ec = dfloat{sd[0].x, sd[0].y};
    dfloat f = up ? dfloat{sd[1].x, sd[1].y} : dfloat{sd[2].x, sd[2].y};
    const dfloat q = dfloat{sd[3].x, sd[3].y};
    const dfloat hd = dfloat{sd[4].x, sd[4].y}, rd = dfloat{sd[5].x, sd[5].y};
    const int cend = up ? cmax + 1 : -cmax;
    for (int cc = 0;; cc += up ? 1 : -1) {
      if (up || cc != 0) { // c = 0 is written by the up-going lane
        const dfloat x = df_fma1(rd, hd, (float)cc);
        dfloat v = ec;
        T *p = pol + (size_t)(dir * w + cc + cmax) * PP;
#pragma unroll
        for (int l = 0; l <= LPB; l++) {
          if (l > lp)
            break;
          if constexpr (std::is_same<T, float>::value)
            p[l] = v.h;
          else
            p[l] = v;
          v = df_mul(v, x);
        }
      }
      if (cc == cend)
        break;
      ec = df_mul(ec, f);
      f = df_mul(f, q);
    }
  }
}

// 1-D factors pol[dir][c][l] = x_c^l exp(-zetp x_c^2), x_c = c*h - roff,
// c in [-cmax, cmax+1]; and the periodic maps map[dir][c]
// (grid_ref_collint.h:259-304).
template <typename N, int LPB>
__device__ __forceinline__ void fill_ortho_tables(const TaskDesc &d, const LevelDesc &L,
                                                  int cmax, int lp,
                                                  typename Num<N>::T *pol, int *map,
                                                  int lane, const float2 *seed) {
  using T = typename Num<N>::T;
  constexpr int PP = OrthoSmem<N, LPB>::PP;
  const int w = 2 * cmax + 2;
  for (int e = lane; e < 3 * w; e += 32) {
    const int dir = e / w, c = e - dir * w, cc = c - cmax;
    map[dir * w + c] = imod(d.center[dir] + cc - L.shift[dir], L.npts_global[dir]);
  }
  if constexpr (std::is_same<T, double>::value) {
    // FP64: direct evaluation
    for (int e = lane; e < 3 * w; e += 32) {
      const int dir = e / w, c = e - dir * w, cc = c - cmax;
      const double x = (double)cc * L.dh[dir * 4] - d.roff[dir];
      double v = exp(-d.zetp * x * x);
      T *p = pol + (size_t)(dir * w + c) * PP;
#pragma unroll
      for (int l = 0; l <= LPB; l++) {
        if (l > lp)
          break;
        p[l] = v;
        v *= x;
      }
    }
  } else if constexpr (std::is_same<T, float>::value) {
    if (seed) { // rounded from the double-float recurrence below
      seeded_tables<T, LPB, PP>(w, cmax, lp, pol, lane, seed);
      return;
    }
    for (int e = lane; e < 3 * w; e += 32) {
      const int dir = e / w, c = e - dir * w, cc = c - cmax;
      const float x = fmaf((float)cc, (float)L.dh[dir * 4], -(float)d.roff[dir]);
      float v = expf(-(float)d.zetp * x * x);
      T *p = pol + (size_t)(dir * w + c) * PP;
#pragma unroll
      for (int l = 0; l <= LPB; l++) {
        if (l > lp)
          break;
        p[l] = v;
        v *= x;
      }
    }
  } else {
    seeded_tables<T, LPB, PP>(w, cmax, lp, pol, lane, seed);
  }
}

// Recurrence seeds of task t for fill_ortho_tables: the double-float kernels
// always use them; the FP32 kernels only on the outside rows of a split task,
// whose exponents z x^2 are large (elsewhere expf is as accurate and cheaper)
template <typename N>
__device__ __forceinline__ const float2 *table_seed(const GridArgs &a, int t) {
  if constexpr (std::is_same<N, float>::value)
    return a.core_side == 2 ? a.seeds + (size_t)t * 18 : nullptr;
  else
    return a.seeds + (size_t)t * 18;
}

// number of (ly, lx) pairs before row ly in a triangle of degree m
__device__ __forceinline__ int tri_idx(int ly, int lx, int m) {
  return ly * (m + 1) - (ly * (ly - 1)) / 2 + lx;
}

// grid write of one collocated value
template <typename N>
__device__ __forceinline__ void grid_add(double *g, float *glo, size_t i,
                                         typename Num<N>::T v) {
  if constexpr (std::is_same<N, dfloat>::value) {
    atomicAdd(g + i, f2d_grid(v.h));
    atomicAdd(glo + i, v.l);
  } else if constexpr (std::is_same<N, float>::value) {
    atomicAdd(g + i, f2d_grid(v));
  } else {
    atomicAdd(g + i, v);
  }
}

// grid read for integrate
template <typename N>
__device__ __forceinline__ typename Num<N>::T grid_get(const void *g, size_t i, int stride = 1) {
  if constexpr (std::is_same<N, dfloat>::value) {
    const float2 v = __ldg(reinterpret_cast<const float2 *>(g) + i);
    return dfloat{v.x, v.y};
  } else if constexpr (std::is_same<N, float>::value) {
    return __ldg(reinterpret_cast<const float *>(g) + i * stride);
  } else {
    return __ldg(reinterpret_cast<const typename Num<N>::T *>(g) + i);
  }
}

// cube geometry shared by the two kernels
struct CubeGeo {
  int K, cmax, w, x_lo, x_hi, SW, G, sub, grp, NX;
  const int16_t *tab;
  const int16_t *jx; // [K][NX] last row index per (plane, x)
  int lb2;
};

__device__ __forceinline__ CubeGeo cube_geo(const SphereHdr &H, const int16_t *sph_tab, int lane) {
  CubeGeo g;
  g.tab = sph_tab + H.off;
  g.jx = g.tab + H.jxo;
  g.NX = 1 - H.lb[0];
  g.K = 1 - H.lb[2];
  g.lb2 = H.lb[2];
  g.cmax = H.cmax;
  g.w = 2 * H.cmax + 2;
  g.x_lo = H.lb[0];
  g.x_hi = 1 - H.lb[0];
  const int width = g.x_hi - g.x_lo + 1;
  g.SW = width < 32 ? width : 32;
  g.G = 32 / g.SW;
  g.sub = lane % g.SW;
  g.grp = lane / g.SW; // lanes with grp >= G are idle
  return g;
}

// ------------------------------------------------------------------------
// collocate, orthorhombic
// ------------------------------------------------------------------------
// SPLIT: the launch runs one side of split tasks (a.core_side), whose rows
// are limited per plane; a template flag, so that whole-task launches keep
// the plain row loop (this kernel is bound by instruction issue)
template <typename N, int LPB, bool SPLIT = false>
__global__ void __launch_bounds__(128) collocate_ortho(GridArgs a, int wmax) {
  using T = typename Num<N>::T;
  using M = Num<N>;
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr int P = LPB + 1;
  constexpr int PP = OrthoSmem<N, LPB>::PP;
  const int lane = threadIdx.x & 31;
  unsigned char *ws = smem + (threadIdx.x >> 5) * OrthoSmem<N, LPB>::bytes_coll(wmax);
  T *pol = (T *)ws;
  T *coef = pol + 3 * (size_t)wmax * PP;
  T *cxy = coef + ntri(LPB) * P;
  int *map = (int *)(cxy + ntri(LPB));
  const T *coefs = (const T *)a.coef;

  for (;;) {
    int qi = 0;
    if (lane == 0)
      qi = atomicAdd(a.counter, 1);
    qi = __shfl_sync(FULL, qi, 0);
    if (qi >= a.nqueue)
      break;
    const WorkItem w = work_item(a, qi);
    const int t = w.t;
    const long long t0 = clock64();
    const TaskDesc d = a.tasks[t];
    const LevelDesc &L = a.levels.lv[d.level];
    const int lp = d.la_max + a.d.la_max + d.lb_max + a.d.lb_max;
    const CubeGeo cg = cube_geo(a.sph[d.sphere], a.sph_tab, lane);
    const int k_lo = cg.lb2 + w.k0, k_hi = min(1 - cg.lb2, cg.lb2 + w.k0 + w.nk - 1);
    if (cg.w > wmax || lp > LPB) { // the host sized the work arrays; never expected
      if (lane == 0)
        atomicOr(a.error, 1);
      continue;
    }
    const int ntr = ntri(lp);
    // coefficients regrouped as coef[(ly, lx)][lz], zero beyond lz = lp-ly-lx,
    // so that the per-plane z fold is a plain loop
    for (int r = lane; r < ntr * P; r += 32) {
      const int e = r / P, lz = r - e * P;
      int ly = 0, rem = e;
      while (rem > lp - ly) {
        rem -= lp - ly + 1;
        ly++;
      }
      const int lx = rem;
      T v = M::zero();
      if (lz <= lp - ly - lx) {
        const size_t ci = (size_t)a.coef_off[t] + cidx(lz, ly, lx, lp);
        if constexpr (std::is_same<T, float>::value)
          v = ((const float *)a.coef)[ci * a.coef_stride];
        else
          v = coefs[ci];
      }
      coef[r] = v;
    }
    fill_ortho_tables<N, LPB>(d, L, cg.cmax, lp, pol, map, lane, table_seed<N>(a, t));
    __syncwarp();

    double *grid = a.grids[d.level];
    float *glo = a.grids_lo[d.level];
    const size_t nx = L.npts_local[0], nxy = nx * L.npts_local[1];
    const bool lane_on = cg.grp < cg.G;
    const float r2 = SPLIT ? a.core_r2[t] : kCoreAll;

    for (int xc = cg.x_lo; xc <= cg.x_hi; xc += cg.SW) {
      const int cx = xc + cg.sub;
      const bool xin = lane_on && cx <= cg.x_hi;
      T px[PP];
      load_row<T, PP>(pol + (size_t)((xin ? cx : cg.x_lo) + cg.cmax) * PP, px);
      const int ig = map[(xin ? cx : cg.x_lo) + cg.cmax];

      for (int k = k_lo; k <= k_hi; k++) {
        const int kk = k <= 0 ? -k : k - 1;
        const int js = cg.tab[kk];
        // C_xy[ly][lx] = sum_lz C_xyz[lz][ly][lx] pol_z[lz](k)
        const T *pz = pol + (size_t)(2 * cg.w + k + cg.cmax) * PP;
        for (int e = lane; e < ntr; e += 32) {
          const T *cr = coef + e * P;
          T s = M::zero();
#pragma unroll
          for (int lz = 0; lz < P; lz++)
            if (lz <= lp)
              s = M::fma_acc(s, cr[lz], pz[lz]);
          cxy[e] = M::norm(s);
        }
        __syncwarp();
        // q[ly] = sum_lx C_xy[ly][lx] pol_x[lx](x_lane)
        T q[P];
#pragma unroll
        for (int ly = 0; ly < P; ly++) {
          T s = M::zero();
          if (ly <= lp) {
            const T *row = cxy + tri_idx(ly, 0, lp);
#pragma unroll
            for (int lx = 0; lx < P; lx++)
              if (lx <= lp - ly)
                s = M::fma_acc(s, row[lx], px[lx]);
          }
          q[ly] = M::norm(s);
        }
        __syncwarp();
        const size_t zoff = (size_t)map[2 * cg.w + k + cg.cmax] * nxy;
        // rows of this lane's x on the plane: j in [jlo, jhi]
        const int JJ = xin ? (int)cg.jx[kk * cg.NX + (cx <= 0 ? -cx : cx - 1)] : -1;
        int jlo = -JJ, jhi = JJ + 1, xlo = 1, xhi = 0; // rows [xlo, xhi] left out
        const int jend = 1 - js;
        if constexpr (SPLIT) { // the rows inside the cylinder, or those outside
          int clo, chi;
          core_rows(r2, d, L, k, clo, chi);
          if (a.core_side == 1) {
            jlo = max(jlo, clo);
            jhi = min(jhi, chi);
          } else {
            xlo = clo;
            xhi = chi;
          }
        }
        for (int j = js + cg.grp; j <= jend; j += 2 * cg.G) {
          const int j2 = j + cg.G;
          bool in1 = j >= jlo && j <= jhi;
          bool in2 = j2 >= jlo && j2 <= jhi;
          if constexpr (SPLIT) {
            in1 = in1 && (j < xlo || j > xhi);
            in2 = in2 && (j2 < xlo || j2 > xhi);
          }
          if (!(in1 || in2))
            continue;
          const int j2c = j2 <= jend ? j2 : jend;
          T p1[PP], p2[PP];
          load_row<T, PP>(pol + (size_t)(cg.w + j + cg.cmax) * PP, p1);
          load_row<T, PP>(pol + (size_t)(cg.w + j2c + cg.cmax) * PP, p2);
          T v1 = M::zero(), v2 = M::zero();
#pragma unroll
          for (int ly = 0; ly < P; ly++)
            if (ly <= lp) {
              v1 = M::fma_acc(v1, q[ly], p1[ly]);
              v2 = M::fma_acc(v2, q[ly], p2[ly]);
            }
          if (in1)
            grid_add<N>(grid, glo, zoff + (size_t)map[cg.w + j + cg.cmax] * nx + ig, v1);
          if (in2)
            grid_add<N>(grid, glo, zoff + (size_t)map[cg.w + j2c + cg.cmax] * nx + ig, v2);
        }
      }
    }
    if (a.task_cycles && lane == 0)
      atomicAdd((unsigned long long *)&a.task_cycles[t], (unsigned long long)(clock64() - t0));
    __syncwarp();
  }
}

// ------------------------------------------------------------------------
// collocate, orthorhombic, over the sphere's point lists
// ------------------------------------------------------------------------
// Same arithmetic as collocate_ortho, different lane mapping: per plane the
// warp first folds x into a table q[x][ly] for every x of the cube, then
// walks the plane's points in row-major order, 32 consecutive points per
// warp step (two steps per iteration), so every lane has work whatever the
// cube width and the shape of the plane's disc.  The points come from a
// host-built list per sphere (shared by all tasks of that sphere, so it
// stays in L1/L2); consecutive lanes hit consecutive x of a row, keeping the
// grid atomics coalesced.
template <typename N, int LPB>
__global__ void __launch_bounds__(128) collocate_ortho_pl(GridArgs a, int wmax) {
  using T = typename Num<N>::T;
  using M = Num<N>;
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr int P = LPB + 1;
  constexpr int PP = OrthoSmem<N, LPB>::PP;
  const int lane = threadIdx.x & 31;
  unsigned char *ws = smem + (threadIdx.x >> 5) * OrthoSmem<N, LPB>::bytes_coll_pl(wmax);
  T *pol = (T *)ws;
  T *qt = pol + 3 * (size_t)wmax * PP;
  T *coef = qt + (size_t)wmax * PP;
  T *cxy = coef + ntri(LPB) * P;
  int *map = (int *)(cxy + ntri(LPB));
  const T *coefs = (const T *)a.coef;

  for (;;) {
    int qi = 0;
    if (lane == 0)
      qi = atomicAdd(a.counter, 1);
    qi = __shfl_sync(FULL, qi, 0);
    if (qi >= a.nqueue)
      break;
    const WorkItem w = work_item(a, qi);
    const int t = w.t;
    const long long t0 = clock64();
    const TaskDesc d = a.tasks[t];
    const LevelDesc &L = a.levels.lv[d.level];
    const int lp = d.la_max + a.d.la_max + d.lb_max + a.d.lb_max;
    const SphereHdr &H = a.sph[d.sphere];
    const CubeGeo cg = cube_geo(H, a.sph_tab, lane);
    const int k_lo = cg.lb2 + w.k0, k_hi = min(1 - cg.lb2, cg.lb2 + w.k0 + w.nk - 1);
    if (cg.w > wmax || lp > LPB || H.plo < 0) { // the host sized the work arrays
      if (lane == 0)
        atomicOr(a.error, 1);
      continue;
    }
    const int ntr = ntri(lp);
    // coefficients regrouped as coef[(ly, lx)][lz], zero beyond lz = lp-ly-lx,
    // so that the per-plane z fold is a plain loop
    for (int r = lane; r < ntr * P; r += 32) {
      const int e = r / P, lz = r - e * P;
      int ly = 0, rem = e;
      while (rem > lp - ly) {
        rem -= lp - ly + 1;
        ly++;
      }
      const int lx = rem;
      T v = M::zero();
      if (lz <= lp - ly - lx) {
        const size_t ci = (size_t)a.coef_off[t] + cidx(lz, ly, lx, lp);
        if constexpr (std::is_same<T, float>::value)
          v = ((const float *)a.coef)[ci * a.coef_stride];
        else
          v = coefs[ci];
      }
      coef[r] = v;
    }
    fill_ortho_tables<N, LPB>(d, L, cg.cmax, lp, pol, map, lane, table_seed<N>(a, t));
    __syncwarp();

    double *grid = a.grids[d.level];
    float *glo = a.grids_lo[d.level];
    const size_t nx = L.npts_local[0], nxy = nx * L.npts_local[1];
    const int *ploff = a.sph_ploff + H.plo;

    const float r2 = a.core_side ? a.core_r2[t] : kCoreAll;
    for (int k = k_lo; k <= k_hi; k++) {
      const int kk = k <= 0 ? -k : k - 1;
      const int n = ploff[kk + 1] - ploff[kk];
      // the plane's points [f0, f1) and [g0, g1): all of them, or (split
      // task) the rows inside the cylinder, or the rows outside it, which are
      // contiguous ranges of the row-major list
      int f0 = 0, f1 = n, g0 = n, g1 = n;
      if (a.core_side) {
        int clo, chi;
        core_rows(r2, d, L, k, clo, chi);
        const int js = cg.tab[kk], row0 = cg.tab[cg.K + kk];
        int before = 0, inside = 0;
        for (int j = js + lane; j <= 1 - js; j += 32) {
          const int jj = j <= 0 ? -j : j - 1;
          const int len = 2 - 2 * cg.tab[2 * cg.K + row0 + jj];
          if (j < clo)
            before += len;
          else if (j <= chi)
            inside += len;
        }
        before = __reduce_add_sync(FULL, before);
        inside = __reduce_add_sync(FULL, inside);
        if (a.core_side == 1) {
          f0 = before;
          f1 = before + inside;
        } else {
          f1 = before;
          g0 = before + inside;
        }
        if (f1 <= f0 && g1 <= g0)
          continue; // nothing of this plane on this side
      }
      // C_xy[ly][lx] = sum_lz C_xyz[lz][ly][lx] pol_z[lz](k)
      const T *pz = pol + (size_t)(2 * cg.w + k + cg.cmax) * PP;
      for (int e = lane; e < ntr; e += 32) {
        const T *cr = coef + e * P;
        T s = M::zero();
#pragma unroll
        for (int lz = 0; lz < P; lz++)
          if (lz <= lp)
            s = M::fma_acc(s, cr[lz], pz[lz]);
        cxy[e] = M::norm(s);
      }
      __syncwarp();
      // q[c][ly] = sum_lx C_xy[ly][lx] pol_x[lx](c), every x of the cube
      for (int c = lane; c < cg.w; c += 32) {
        T px[PP];
        load_row<T, PP>(pol + (size_t)c * PP, px);
        T *qr = qt + (size_t)c * PP;
#pragma unroll
        for (int ly = 0; ly < P; ly++) {
          T s = M::zero();
          if (ly <= lp) {
            const T *row = cxy + tri_idx(ly, 0, lp);
#pragma unroll
            for (int lx = 0; lx < P; lx++)
              if (lx <= lp - ly)
                s = M::fma_acc(s, row[lx], px[lx]);
          }
          qr[ly] = M::norm(s);
        }
      }
      __syncwarp();
      const size_t zoff = (size_t)map[2 * cg.w + k + cg.cmax] * nxy;
      const int *pts = a.sph_pts + ploff[kk];
      for (int rg = 0; rg < 2; rg++) {
       const int fe = rg ? g1 : f1;
       for (int f = (rg ? g0 : f0) + lane; f < fe; f += 64) {
        const int f2 = f + 32;
        const bool two = f2 < fe;
        const int pk1 = __ldg(pts + f);
        const int pk2 = two ? __ldg(pts + f2) : pk1;
        const int x1 = (int)(short)(pk1 & 0xffff), j1 = pk1 >> 16;
        const int x2 = (int)(short)(pk2 & 0xffff), j2 = pk2 >> 16;
        T q1[PP], q2[PP], p1[PP], p2[PP];
        load_row<T, PP>(qt + (size_t)(x1 + cg.cmax) * PP, q1);
        load_row<T, PP>(pol + (size_t)(cg.w + j1 + cg.cmax) * PP, p1);
        load_row<T, PP>(qt + (size_t)(x2 + cg.cmax) * PP, q2);
        load_row<T, PP>(pol + (size_t)(cg.w + j2 + cg.cmax) * PP, p2);
        T v1 = M::zero(), v2 = M::zero();
#pragma unroll
        for (int ly = 0; ly < P; ly++)
          if (ly <= lp) {
            v1 = M::fma_acc(v1, q1[ly], p1[ly]);
            v2 = M::fma_acc(v2, q2[ly], p2[ly]);
          }
        grid_add<N>(grid, glo,
                    zoff + (size_t)map[cg.w + j1 + cg.cmax] * nx + map[x1 + cg.cmax], v1);
        if (two)
          grid_add<N>(grid, glo,
                      zoff + (size_t)map[cg.w + j2 + cg.cmax] * nx + map[x2 + cg.cmax], v2);
       }
      }
      __syncwarp();
    }
    if (a.task_cycles && lane == 0)
      atomicAdd((unsigned long long *)&a.task_cycles[t], (unsigned long long)(clock64() - t0));
    __syncwarp();
  }
}

// ------------------------------------------------------------------------
// integrate, orthorhombic (adjoint of collocate_ortho)
// ------------------------------------------------------------------------
template <typename N, int LPB>
__global__ void __launch_bounds__(128, LPB <= 4 ? 5 : 1) integrate_ortho(GridArgs a, int wmax) {
  using T = typename Num<N>::T;
  using M = Num<N>;
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr int P = LPB + 1;
  constexpr int PP = OrthoSmem<N, LPB>::PP;
  constexpr int NYZ = (LPB + 1) * (LPB + 2) / 2;
  const int lane = threadIdx.x & 31;
  unsigned char *ws = smem + (threadIdx.x >> 5) * OrthoSmem<N, LPB>::bytes_int(wmax);
  T *pol = (T *)ws;
  T *red = pol; // the x fold of the last x-chunk overwrites the tables
  int *map = (int *)(pol + OrthoSmem<N, LPB>::pol_words_int(wmax));
  double *acc = (double *)(((uintptr_t)(map + 3 * wmax) + 15) & ~uintptr_t(15));
  double *out = (double *)a.coef_out;

  for (;;) {
    int qi = 0;
    if (lane == 0)
      qi = atomicAdd(a.counter, 1);
    qi = __shfl_sync(FULL, qi, 0);
    if (qi >= a.nqueue)
      break;
    const WorkItem w = work_item(a, qi);
    const int t = w.t;
    const long long t0 = clock64();
    const TaskDesc d = a.tasks[t];
    const LevelDesc &L = a.levels.lv[d.level];
    const int lp = d.la_max + a.d.la_max + d.lb_max + a.d.lb_max;
    const CubeGeo cg = cube_geo(a.sph[d.sphere], a.sph_tab, lane);
    const int k_lo = cg.lb2 + w.k0, k_hi = min(1 - cg.lb2, cg.lb2 + w.k0 + w.nk - 1);
    if (cg.w > wmax || lp > LPB) {
      if (lane == 0)
        atomicOr(a.error, 1);
      continue;
    }
    const int nco = ncoset(lp);
    for (int e = lane; e < nco; e += 32)
      acc[e] = 0.0;
    fill_ortho_tables<N, LPB>(d, L, cg.cmax, lp, pol, map, lane, table_seed<N>(a, t));
    __syncwarp();

    const float r2 = a.core_side ? a.core_r2[t] : kCoreAll;
    const void *grid = a.grids_in[d.level];
    const int gstride = a.grid_stride;
    const size_t nx = L.npts_local[0], nxy = nx * L.npts_local[1];
    // lanes: x chunks of sub-warps, rows of a plane split over the groups
    // of a chunk; the sphere's plan (cubes up to 32 wide) sizes the chunks
    // and gives central chunks, whose columns are longer, more groups
    const int ip = a.sph[d.sphere].iplan;
    int sub = cg.sub, phase = cg.grp, nph = cg.G, xstep = cg.SW, cbase = 0;
    bool on = cg.grp < cg.G;
    if (ip) {
      const int sw = ip & 63, nc = (ip >> 6) & 7, gi = lane / sw;
      sub = lane % sw;
      on = false;
      for (int c = 0, base = 0; c < nc; c++) {
        const int nn = (ip >> (9 + 5 * c)) & 31;
        if (!on && gi < base + nn) {
          phase = gi - base;
          nph = nn;
          cbase = c * sw;
          on = true;
        }
        base += nn;
      }
      xstep = cg.x_hi - cg.x_lo + 1; // one pass covers every chunk
    }

    for (int xc = cg.x_lo; xc <= cg.x_hi; xc += xstep) {
      const int cx = xc + cbase + sub;
      const bool xin = on && cx <= cg.x_hi;
      const int ig = map[(xin ? cx : cg.x_lo) + cg.cmax];
      T ayz[NYZ]; // [lz][ly], lz + ly <= LPB
#pragma unroll
      for (int e = 0; e < NYZ; e++)
        ayz[e] = M::zero();

      for (int k = k_lo; k <= k_hi; k++) {
        const int kk = k <= 0 ? -k : k - 1;
        const int js = cg.tab[kk];
        const size_t zoff = (size_t)map[2 * cg.w + k + cg.cmax] * nxy;
        T wy[P];
#pragma unroll
        for (int l = 0; l < P; l++)
          wy[l] = M::zero();
        // this lane's rows of the plane: j in [jlo, jhi] (jhi <= 1 - js), every
        // G-th row from its group's phase, R rows per step; the grid values
        // of the next step are loaded before this step's arithmetic
        const int JJ = xin ? (int)cg.jx[kk * cg.NX + (cx <= 0 ? -cx : cx - 1)] : -1;
        int jlo = -JJ, jhi = JJ + 1, jlo2 = 1, jhi2 = 0;
        if (a.core_side) { // split task: the rows inside, or the two runs outside
          int clo, chi;
          core_rows(r2, d, L, k, clo, chi);
          if (a.core_side == 1) {
            jlo = max(jlo, clo);
            jhi = min(jhi, chi);
          } else {
            jlo2 = max(jlo, chi + 1);
            jhi2 = jhi;
            jhi = min(jhi, clo - 1);
          }
        }
        const int G = nph;
        const size_t base = zoff + ig;
        auto fetch = [&](int jj, bool ok) -> T {
          return ok ? grid_get<N>(grid, base + (size_t)map[cg.w + jj + cg.cmax] * nx, gstride)
                    : M::zero();
        };
        // R rows per step (4 in FP32, whose arithmetic is too short to hide
        // the L2 latency of 2 loads in flight; 2 otherwise)
        constexpr int R = std::is_same<N, float>::value ? 4 : 2;
        for (int sg = 0; sg < 2; sg++) {
          const int slo = sg ? jlo2 : jlo, shi = sg ? jhi2 : jhi;
          if (slo > shi)
            continue;
          int j = js + phase;
          if (j < slo)
            j += ((slo - j + G - 1) / G) * G;
          bool has[R];
          T v[R];
#pragma unroll
          for (int r = 0; r < R; r++) {
            has[r] = j + r * G <= shi;
            v[r] = fetch(j + r * G, has[r]);
          }
          while (has[0]) {
            const int jn = j + R * G;
            bool hn[R];
            T vn[R];
#pragma unroll
            for (int r = 0; r < R; r++) {
              hn[r] = jn + r * G <= shi;
              vn[r] = fetch(jn + r * G, hn[r]);
            }
#pragma unroll
            for (int r = 0; r < R; r++) {
              T pr[PP];
              load_row<T, PP>(pol + (size_t)(cg.w + (has[r] ? j + r * G : j) + cg.cmax) * PP, pr);
#pragma unroll
              for (int ly = 0; ly < P; ly++)
                if (ly <= lp)
                  wy[ly] = M::fma_acc(wy[ly], v[r], pr[ly]);
            }
            j = jn;
#pragma unroll
            for (int r = 0; r < R; r++) {
              has[r] = hn[r];
              v[r] = vn[r];
            }
          }
        }
#pragma unroll
        for (int l = 0; l < P; l++)
          wy[l] = M::norm(wy[l]);
        T pz[PP];
        load_row<T, PP>(pol + (size_t)(2 * cg.w + k + cg.cmax) * PP, pz);
#pragma unroll
        for (int lz = 0; lz < P; lz++) {
          if (lz > lp)
            break;
#pragma unroll
          for (int ly = 0; ly < P; ly++)
            if (ly <= lp - lz)
              ayz[lz * P - (lz * (lz - 1)) / 2 + ly] =
                  M::fma_acc(ayz[lz * P - (lz * (lz - 1)) / 2 + ly], wy[ly], pz[lz]);
        }
      }
      // x fold and reduction over the warp through shared memory:
      // C_xyz[lz][ly][lx] += sum_lanes ayz[lz][ly] * pol_x[lx]
      {
        constexpr int RS = OrthoSmem<N, LPB>::red_stride();
        T *rl = red + lane * RS;
        T px[PP];
        load_row<T, PP>(pol + (size_t)((xin ? cx : cg.x_lo) + cg.cmax) * PP, px);
        __syncwarp(); // every lane holds its pol_x before the tables are overwritten
#pragma unroll
        for (int e = 0; e < NYZ; e++)
          rl[e] = M::norm(ayz[e]);
#pragma unroll
        for (int l = 0; l < P; l++)
          rl[NYZ + l] = (xin && l <= lp) ? px[l] : M::zero();
        __syncwarp();
        for (int e = lane; e < nco; e += 32) {
          int lz, ly, lx;
          decode_cidx(e, lp, lz, ly, lx);
          const int yz = lz * P - (lz * (lz - 1)) / 2 + ly;
          T s = M::zero();
#pragma unroll 8
          for (int r = 0; r < 32; r++)
            s = M::fma_acc(s, red[r * RS + yz], red[r * RS + NYZ + lx]);
          acc[e] += M::to_double(s);
        }
        __syncwarp();
        if (xc + xstep <= cg.x_hi) { // another x-chunk follows: rebuild the tables
          fill_ortho_tables<N, LPB>(d, L, cg.cmax, lp, pol, map, lane, table_seed<N>(a, t));
          __syncwarp();
        }
      }
    }
    __syncwarp();
    double *dst = out + a.coef_off[t];
    for (int e = lane; e < nco; e += 32)
      if (a.items || a.accum) // parts of one task add up (the buffer is zeroed)
        atomicAdd(dst + e, acc[e]);
      else
        dst[e] = acc[e];
    if (a.task_cycles && lane == 0)
      atomicAdd((unsigned long long *)&a.task_cycles[t], (unsigned long long)(clock64() - t0));
    __syncwarp();
  }
}

// ------------------------------------------------------------------------
// integrate, orthorhombic, FP32 class, on the tensor cores
// ------------------------------------------------------------------------
// The first contraction of the integrate is a dense matrix product per
// task: T1[(k, j)][lx] = sum_x V(x, j, k) pol_x[lx](x) over the rows (k, j)
// of the sphere (plane by plane) and the cube's x range, V zero outside the
// sphere (the reference's point set, grid_ref_collint.h:144-151).  One warp
// runs it as mma.sync m16n8k8 TF32 tiles (16 rows x 8 x per step, n = 8
// covers lx <= 7), each operand split into a TF32 high and low part and
// three products accumulated in FP32 (high*high + high*low + low*high), which
// keeps about 21 bits of every product.  The rows are folded with
// pol_y(j) pol_z(k) on the CUDA cores and reduced over the warp once per
// task.
template <int LPB> struct TcSmem {
  static constexpr int PP = 8; // padded<LPB, float>() for LPB <= 7
  static __host__ __device__ size_t bytes(int wmax) {
    size_t b = sizeof(float) * 3 * (size_t)wmax * PP; // pol x, y, z
    b += sizeof(float2) * (size_t)wmax * 8;          // pol_x split hi / lo
    b += sizeof(int) * 3 * (size_t)wmax;             // periodic maps
    b += sizeof(int) * 4 * ((size_t)wmax + 4);       // per plane: first row, row map
    b += 64;
    return (b + 15) & ~size_t(15);
  }
};

__device__ __forceinline__ unsigned f2tf32(float x) {
  unsigned r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ void mma_tf32(float (&c)[4], const unsigned (&a)[4], unsigned b0,
                                         unsigned b1) {
  asm volatile("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 "
               "{%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, {%0, %1, %2, %3};"
               : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
               : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

template <int LPB>
__global__ void __launch_bounds__(128) integrate_ortho_tc(GridArgs a, int wmax) {
  static_assert(LPB <= 7, "one n8 tile holds lx <= 7");
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr int P = LPB + 1;
  constexpr int PP = TcSmem<LPB>::PP;
  constexpr int NT = (P * (P + 1)) / 2; // (ly, lz) pairs with ly + lz <= LPB
  const int lane = threadIdx.x & 31, grp = lane >> 2, tq = lane & 3;
  unsigned char *ws = smem + (threadIdx.x >> 5) * TcSmem<LPB>::bytes(wmax);
  float *pol = (float *)ws;
  float2 *pxs = (float2 *)(pol + 3 * (size_t)wmax * PP);
  int *map = (int *)(pxs + (size_t)wmax * 8);
  int *starts = map + 3 * wmax;
  int *prow = starts + wmax + 4; // per plane: j of row 0, skip at row, rows skipped
  double *out = (double *)a.coef_out;

  for (;;) {
    int qi = 0;
    if (lane == 0)
      qi = atomicAdd(a.counter, 1);
    qi = __shfl_sync(FULL, qi, 0);
    if (qi >= a.nqueue)
      break;
    const WorkItem w = work_item(a, qi);
    const int t = w.t;
    const long long t0 = clock64();
    const TaskDesc d = a.tasks[t];
    const LevelDesc &L = a.levels.lv[d.level];
    const int lp = d.la_max + a.d.la_max + d.lb_max + a.d.lb_max;
    const CubeGeo cg = cube_geo(a.sph[d.sphere], a.sph_tab, lane);
    const int k_lo = cg.lb2 + w.k0, k_hi = min(1 - cg.lb2, cg.lb2 + w.k0 + w.nk - 1);
    if (cg.w > wmax || lp > LPB || k_hi - k_lo + 1 > wmax + 2) {
      if (lane == 0)
        atomicOr(a.error, 1);
      continue;
    }
    fill_ortho_tables<float, LPB>(d, L, cg.cmax, lp, pol, map, lane, table_seed<float>(a, t));
    __syncwarp();
    // pol_x split into TF32 high and low parts, lx >= P (or > lp) zero
    for (int e = lane; e < cg.w * 8; e += 32) {
      const int c = e >> 3, l = e & 7;
      const float v = (l <= lp) ? pol[(size_t)c * PP + l] : 0.f;
      const unsigned hi = f2tf32(v);
      const unsigned lo = f2tf32(v - __uint_as_float(hi));
      pxs[e] = make_float2(__uint_as_float(hi), __uint_as_float(lo));
    }
    // the rows of every plane k_lo .. k_hi (j in [js, 1 - js]; of a split
    // task the rows inside or outside the cylinder) numbered plane after
    // plane: row i of plane p is j = prow[3p] + i (+ prow[3p + 2] from
    // i = prow[3p + 1] on, stepping over the inside rows)
    const int np = k_hi - k_lo + 1;
    const float r2 = a.core_side ? a.core_r2[t] : kCoreAll;
    {
      int carry = 0;
      for (int p0 = 0; p0 < np; p0 += 32) {
        const int p = p0 + lane;
        int cnt = 0;
        if (p < np) {
          const int k = k_lo + p, kk = k <= 0 ? -k : k - 1, js = cg.tab[kk];
          int j0 = js, at = 1 << 20, skip = 0;
          cnt = 2 - 2 * js;
          if (a.core_side) {
            int clo, chi;
            core_rows(r2, d, L, k, clo, chi);
            const int ilo = max(clo, js), ihi = min(chi, 1 - js);
            const int inside = max(0, ihi - ilo + 1);
            if (a.core_side == 1) {
              j0 = ilo;
              cnt = inside;
            } else {
              at = min(max(clo - js, 0), cnt);
              skip = inside;
              cnt -= inside;
            }
          }
          prow[3 * p] = j0;
          prow[3 * p + 1] = at;
          prow[3 * p + 2] = skip;
        }
        int incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int y = __shfl_up_sync(FULL, incl, o);
          if (lane >= o)
            incl += y;
        }
        if (p < np)
          starts[p] = carry + incl - cnt;
        carry += __shfl_sync(FULL, incl, 31);
      }
      if (lane == 0)
        starts[np] = carry;
    }
    __syncwarp();
    const int R = starts[np];
    const float *grid = (const float *)a.grids_in[d.level];
    const size_t nx = L.npts_local[0], nxy = nx * L.npts_local[1];
    const int K = 1 - cg.lb2;
    float acc[2][NT];
#pragma unroll
    for (int s2 = 0; s2 < 2; s2++)
#pragma unroll
      for (int e = 0; e < NT; e++)
        acc[s2][e] = 0.f;
    // x indices of the grid: linear over the cube's x range unless the cube
    // wraps around the periodic grid there (then through the map)
    const int mx0 = map[cg.cmax];
    const bool linx = map[cg.x_hi + cg.cmax] - map[cg.x_lo + cg.cmax] == cg.x_hi - cg.x_lo;
    int pc = 0; // plane cursor (rows only grow)
    for (int rb = 0; rb < R; rb += 16) {
      // the two rows of this lane in the tile; rows past the end get an
      // empty x range [1 << 28, 1 << 28 - 1] for the unsigned range test
      int kr[2], jr[2], xs[2], xe[2];
      const float *rowp[2];
      bool rv[2];
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const int r = rb + grp + 8 * h;
        rv[h] = r < R;
        kr[h] = k_lo;
        jr[h] = 0;
        xs[h] = 1 << 28;
        xe[h] = (1 << 28) - 1;
        rowp[h] = grid;
        if (rv[h]) {
          int p = pc;
          while (starts[p + 1] <= r)
            p++;
          if (h == 0)
            pc = p;
          const int k = k_lo + p, kk = k <= 0 ? -k : k - 1;
          const int i = r - starts[p];
          const int j = prow[3 * p] + i + (i >= prow[3 * p + 1] ? prow[3 * p + 2] : 0);
          const int jj = j <= 0 ? -j : j - 1;
          const int ist = cg.tab[2 * K + cg.tab[K + kk] + jj];
          kr[h] = k;
          jr[h] = j;
          xs[h] = ist;
          xe[h] = 1 - ist;
          rowp[h] = grid + (size_t)map[2 * cg.w + k + cg.cmax] * nxy +
                    (size_t)map[cg.w + j + cg.cmax] * nx;
        }
      }
      float c[4] = {0.f, 0.f, 0.f, 0.f};
      // the tile's x range: the union of its rows' ranges (short rows of the
      // sphere's outer planes need fewer steps than the cube's width)
      int xmn = 1 << 20, xmx = -(1 << 20);
#pragma unroll
      for (int h = 0; h < 2; h++)
        if (rv[h]) {
          xmn = min(xmn, xs[h]);
          xmx = max(xmx, xe[h]);
        }
      // the row look-ups above diverge; mma.sync.aligned needs the whole warp
      // converged (the reductions reconverge it)
      xmn = max(__reduce_min_sync(FULL, xmn), cg.x_lo);
      xmx = min(__reduce_max_sync(FULL, xmx), cg.x_hi);
      // x steps counted up front: written as a loop on xb <= x_hi, this
      // kernel ran a single step under nvcc 13.0 (measured, lp <= 6 tasks of
      // 12 and more x points)
      const int nxs = xmx >= xmn ? (xmx - xmn + 8) >> 3 : 0;
#pragma unroll 1
      for (int xs8 = 0; xs8 < nxs; xs8++) {
        const int xb = xmn + 8 * xs8;
        float av[4];
        float2 bv[2];
#pragma unroll
        for (int s2 = 0; s2 < 2; s2++) {
          const int x = xb + tq + 4 * s2;
          const bool xin = x <= xmx;
          int mx = mx0 + x;
          if (!linx) // warp-uniform
            mx = xin ? map[x + cg.cmax] : 0;
          bv[s2] = xin ? pxs[(x + cg.cmax) * 8 + grp] : make_float2(0.f, 0.f);
#pragma unroll
          for (int h = 0; h < 2; h++) { // x in [xs, xe]: the row's points (xe <= xmx)
            const bool in = (unsigned)(x - xs[h]) <= (unsigned)(xe[h] - xs[h]);
            av[h + 2 * s2] = in ? __ldg(rowp[h] + mx) : 0.f;
          }
        }
        // TF32 high part by truncation (the low 13 bits cleared), low part
        // the exact remainder (the tensor cores read its top 19 bits)
        unsigned ahi[4], alo[4];
#pragma unroll
        for (int i = 0; i < 4; i++) {
          ahi[i] = __float_as_uint(av[i]) & 0xffffe000u;
          alo[i] = __float_as_uint(av[i] - __uint_as_float(ahi[i]));
        }
        const unsigned b0h = __float_as_uint(bv[0].x), b1h = __float_as_uint(bv[1].x);
        const unsigned b0l = __float_as_uint(bv[0].y), b1l = __float_as_uint(bv[1].y);
        __syncwarp();
        mma_tf32(c, alo, b0h, b1h);
        mma_tf32(c, ahi, b0l, b1l);
        mma_tf32(c, ahi, b0h, b1h);
      }
      // fold the rows: acc[s][(ly, lz)] += T1[row][lx = 2 tq + s] pol_y[ly](j) pol_z[lz](k)
#pragma unroll
      for (int h = 0; h < 2; h++) {
        if (!rv[h])
          continue;
        const float *py = pol + (size_t)(cg.w + jr[h] + cg.cmax) * PP;
        const float *pz = pol + (size_t)(2 * cg.w + kr[h] + cg.cmax) * PP;
#pragma unroll
        for (int s2 = 0; s2 < 2; s2++) {
          const int lx = 2 * tq + s2;
          if (lx > lp)
            continue;
          const float v = c[2 * h + s2];
          int e = 0;
#pragma unroll
          for (int ly = 0; ly < P; ly++) {
            const float u = v * py[ly];
#pragma unroll
            for (int lz = 0; lz < P - ly; lz++, e++)
              if (lx + ly + lz <= lp)
                acc[s2][e] = fmaf(u, pz[lz], acc[s2][e]);
          }
        }
      }
    }
    // sum over the 8 lanes that share tq (the row groups)
    __syncwarp();
#pragma unroll
    for (int s2 = 0; s2 < 2; s2++)
#pragma unroll
      for (int e = 0; e < NT; e++) {
        float v = acc[s2][e];
        v += __shfl_xor_sync(FULL, v, 4);
        v += __shfl_xor_sync(FULL, v, 8);
        v += __shfl_xor_sync(FULL, v, 16);
        acc[s2][e] = v;
      }
    if (grp == 0) {
      double *dst = out + a.coef_off[t];
#pragma unroll
      for (int s2 = 0; s2 < 2; s2++) {
        const int lx = 2 * tq + s2;
        if (lx > lp)
          continue;
        int e = 0;
#pragma unroll
        for (int ly = 0; ly < P; ly++)
#pragma unroll
          for (int lz = 0; lz < P - ly; lz++, e++)
            if (lx + ly + lz <= lp) {
              const double v = f2d_exact(acc[s2][e]);
              const int ci = cidx(lz, ly, lx, lp);
              if (a.items || a.accum) // parts of one task add up (the buffer is zeroed)
                atomicAdd(dst + ci, v);
              else
                dst[ci] = v;
            }
      }
    }
    if (a.task_cycles && lane == 0)
      atomicAdd((unsigned long long *)&a.task_cycles[t], (unsigned long long)(clock64() - t0));
    __syncwarp();
  }
}

// ------------------------------------------------------------------------
// collocate, orthorhombic, FP32 class, on the tensor cores
// ------------------------------------------------------------------------
// With the x factor folded into the coefficients once per task,
//   Q[x][(ly, lz)] = sum_lx C_xyz[lz][ly][lx] pol_x[lx](x),
// every value of the cube is a product over the (ly, lz) pairs:
//   rho[x][(j, k)] = sum_(ly,lz) Q[x][(ly, lz)] pol_y[ly](j) pol_z[lz](k).
// One warp per task runs it as mma.sync m16n8k8 TF32 tiles: 16 x of the cube
// (M) by 8 rows (j, k) of the sphere (N; the rows of all planes numbered one
// after another, as in integrate_ortho_tc), the pairs (K, two steps of 8 for
// lp <= 4, ntri(lp) <= 16).  Both operands are split into TF32 high and low
// parts and three products accumulated in FP32 (about 21 bits per product).
// Each lane adds its four results that lie inside the sphere (the
// reference's point set, grid_ref_collint.h:144-151) to the FP64 grid;
// points of a tile outside the sphere cost only tensor-core work.  Split
// tasks (core_side) take their rows inside or outside the cylinder.
template <int LPB> struct TcCollSmem {
  static constexpr int PP = 8;
  static constexpr int NPR = (ntri(LPB) + 7) & ~7; // pairs, padded to k8 steps
  static __host__ __device__ size_t bytes(int wmax) {
    size_t b = sizeof(float) * 3 * (size_t)wmax * PP;      // pol x, y, z
    b += sizeof(float2) * (size_t)wmax * NPR;              // Q[x][pair] hi / lo
    b += sizeof(float) * ((ncoset(LPB) + 3) & ~3);         // C_xyz of the task
    b += sizeof(int) * 3 * (size_t)wmax;                   // periodic maps
    b += sizeof(int) * 4 * ((size_t)wmax + 4);             // per plane: first row, row map
    b += 64;
    return (b + 15) & ~size_t(15);
  }
};

template <int LPB>
__global__ void __launch_bounds__(128) collocate_ortho_tc(GridArgs a, int wmax) {
  static_assert(ntri(LPB) <= 32, "pairs fit four k8 steps");
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr int PP = TcCollSmem<LPB>::PP;
  constexpr int NPR = TcCollSmem<LPB>::NPR;
  constexpr int KS = NPR / 8; // k8 steps
  const int lane = threadIdx.x & 31, grp = lane >> 2, tq = lane & 3;
  unsigned char *ws = smem + (threadIdx.x >> 5) * TcCollSmem<LPB>::bytes(wmax);
  float *pol = (float *)ws;
  float2 *qs = (float2 *)(pol + 3 * (size_t)wmax * PP);
  float *cx = (float *)(qs + (size_t)wmax * NPR);
  int *map = (int *)(cx + ((ncoset(LPB) + 3) & ~3));
  int *starts = map + 3 * wmax;
  int *prow = starts + wmax + 4;

  for (;;) {
    int qi = 0;
    if (lane == 0)
      qi = atomicAdd(a.counter, 1);
    qi = __shfl_sync(FULL, qi, 0);
    if (qi >= a.nqueue)
      break;
    const WorkItem w = work_item(a, qi);
    const int t = w.t;
    const long long t0 = clock64();
    const TaskDesc d = a.tasks[t];
    const LevelDesc &L = a.levels.lv[d.level];
    const int lp = d.la_max + a.d.la_max + d.lb_max + a.d.lb_max;
    const CubeGeo cg = cube_geo(a.sph[d.sphere], a.sph_tab, lane);
    const int k_lo = cg.lb2 + w.k0, k_hi = min(1 - cg.lb2, cg.lb2 + w.k0 + w.nk - 1);
    if (cg.w > wmax || lp > LPB || k_hi - k_lo + 1 > wmax + 2) {
      if (lane == 0) // the host sized the work arrays; never expected
        atomicOr(a.error, 1);
      continue;
    }
    const int nco = ncoset(lp), npr = ntri(lp);
    for (int e = lane; e < nco; e += 32)
      cx[e] = ((const float *)a.coef)[((size_t)a.coef_off[t] + e) * a.coef_stride];
    fill_ortho_tables<float, LPB>(d, L, cg.cmax, lp, pol, map, lane, table_seed<float>(a, t));
    __syncwarp();
    // Q[x][pair] for every x of the cube, pairs (ly, lz) with ly + lz <= lp in
    // the order of lz, then ly; padded pairs zero
    for (int e = lane; e < cg.w * NPR; e += 32) {
      const int c = e / NPR, pr = e - c * NPR;
      float v = 0.f;
      if (pr < npr) {
        int lz = 0, rem = pr;
        while (rem > lp - lz) {
          rem -= lp - lz + 1;
          lz++;
        }
        const int ly = rem;
        const float *px = pol + (size_t)c * PP;
#pragma unroll
        for (int lx = 0; lx <= LPB; lx++)
          if (lx <= lp - ly - lz)
            v = fmaf(cx[cidx(lz, ly, lx, lp)], px[lx], v);
      }
      const unsigned hi = f2tf32(v);
      qs[e] = make_float2(__uint_as_float(hi), __uint_as_float(f2tf32(v - __uint_as_float(hi))));
    }
    // the rows of planes k_lo .. k_hi (split tasks: inside or outside the
    // cylinder) numbered plane after plane, as in integrate_ortho_tc
    const int np = k_hi - k_lo + 1;
    const float r2 = a.core_side ? a.core_r2[t] : kCoreAll;
    {
      int carry = 0;
      for (int p0 = 0; p0 < np; p0 += 32) {
        const int p = p0 + lane;
        int cnt = 0;
        if (p < np) {
          const int k = k_lo + p, kk = k <= 0 ? -k : k - 1, js = cg.tab[kk];
          int j0 = js, at = 1 << 20, skip = 0;
          cnt = 2 - 2 * js;
          if (a.core_side) {
            int clo, chi;
            core_rows(r2, d, L, k, clo, chi);
            const int ilo = max(clo, js), ihi = min(chi, 1 - js);
            const int inside = max(0, ihi - ilo + 1);
            if (a.core_side == 1) {
              j0 = ilo;
              cnt = inside;
            } else {
              at = min(max(clo - js, 0), cnt);
              skip = inside;
              cnt -= inside;
            }
          }
          prow[3 * p] = j0;
          prow[3 * p + 1] = at;
          prow[3 * p + 2] = skip;
        }
        int incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int y = __shfl_up_sync(FULL, incl, o);
          if (lane >= o)
            incl += y;
        }
        if (p < np)
          starts[p] = carry + incl - cnt;
        carry += __shfl_sync(FULL, incl, 31);
      }
      if (lane == 0)
        starts[np] = carry;
    }
    __syncwarp();
    const int R = starts[np];
    // this lane's B pairs: 8 s + tq and 8 s + tq + 4 of every k8 step s
    int ply[2 * KS], plz[2 * KS];
#pragma unroll
    for (int i = 0; i < 2 * KS; i++) {
      const int pr = 8 * (i >> 1) + tq + 4 * (i & 1);
      int lz = 0, rem = pr;
      while (rem > lp - lz && lz <= lp) {
        rem -= lp - lz + 1;
        lz++;
      }
      ply[i] = pr < npr ? rem : -1;
      plz[i] = lz;
    }
    double *grid = a.grids[d.level];
    const size_t nx = L.npts_local[0], nxy = nx * L.npts_local[1];
    const int K = cg.K;
    const int nxt = (cg.x_hi - cg.x_lo + 16) >> 4; // x tiles, counted up front
    // row r of the numbering -> plane k, row j, cursor pc over the planes
    auto row_of = [&](int r, int &pc, int &k, int &j) {
      int p = pc;
      while (starts[p + 1] <= r)
        p++;
      pc = p;
      const int i = r - starts[p];
      k = k_lo + p;
      j = prow[3 * p] + i + (i >= prow[3 * p + 1] ? prow[3 * p + 2] : 0);
    };
    int pcb = 0, pco = 0;
    const int nrt = (R + 7) >> 3;
#pragma unroll 1
    for (int rt = 0; rt < nrt; rt++) {
      // B: pol_y[ly](j) pol_z[lz](k) of row 8 rt + grp for this lane's pairs
      unsigned bh[2 * KS], bl[2 * KS];
      {
        const int r = 8 * rt + grp;
        float pyz[2 * KS];
        if (r < R) {
          int k, j;
          row_of(r, pcb, k, j);
          const float *py = pol + (size_t)(cg.w + j + cg.cmax) * PP;
          const float *pz = pol + (size_t)(2 * cg.w + k + cg.cmax) * PP;
#pragma unroll
          for (int i = 0; i < 2 * KS; i++)
            pyz[i] = ply[i] >= 0 ? py[ply[i]] * pz[plz[i]] : 0.f;
        } else {
#pragma unroll
          for (int i = 0; i < 2 * KS; i++)
            pyz[i] = 0.f;
        }
#pragma unroll
        for (int i = 0; i < 2 * KS; i++) {
          bh[i] = f2tf32(pyz[i]);
          bl[i] = f2tf32(pyz[i] - __uint_as_float(bh[i]));
        }
      }
      // outputs of this lane: rows 8 rt + 2 tq + h
      int xs[2], xe[2];
      size_t roff[2];
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const int r = 8 * rt + 2 * tq + h;
        xs[h] = 1;
        xe[h] = 0;
        roff[h] = 0;
        if (r < R) {
          int k, j;
          row_of(r, pco, k, j);
          const int kk = k <= 0 ? -k : k - 1, jj = j <= 0 ? -j : j - 1;
          const int ist = cg.tab[2 * K + cg.tab[K + kk] + jj];
          xs[h] = ist;
          xe[h] = 1 - ist;
          roff[h] = (size_t)map[2 * cg.w + k + cg.cmax] * nxy +
                    (size_t)map[cg.w + j + cg.cmax] * nx;
        }
      }
      __syncwarp(); // the look-ups above diverge; mma.sync needs the whole warp
#pragma unroll 1
      for (int xt = 0; xt < nxt; xt++) {
        const int xa = cg.x_lo + 16 * xt + grp, xc = xa + 8;
        const bool in0 = xa <= cg.x_hi, in1 = xc <= cg.x_hi;
        float c[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int s8 = 0; s8 < KS; s8++) {
          const float2 z2 = make_float2(0.f, 0.f);
          const int p0 = 8 * s8 + tq;
          const float2 q00 = in0 ? qs[(size_t)(xa + cg.cmax) * NPR + p0] : z2;
          const float2 q01 = in0 ? qs[(size_t)(xa + cg.cmax) * NPR + p0 + 4] : z2;
          const float2 q10 = in1 ? qs[(size_t)(xc + cg.cmax) * NPR + p0] : z2;
          const float2 q11 = in1 ? qs[(size_t)(xc + cg.cmax) * NPR + p0 + 4] : z2;
          const unsigned ahi[4] = {__float_as_uint(q00.x), __float_as_uint(q10.x),
                                   __float_as_uint(q01.x), __float_as_uint(q11.x)};
          const unsigned alo[4] = {__float_as_uint(q00.y), __float_as_uint(q10.y),
                                   __float_as_uint(q01.y), __float_as_uint(q11.y)};
          mma_tf32(c, alo, bh[2 * s8], bh[2 * s8 + 1]);
          mma_tf32(c, ahi, bl[2 * s8], bl[2 * s8 + 1]);
          mma_tf32(c, ahi, bh[2 * s8], bh[2 * s8 + 1]);
        }
        const int mx0 = in0 ? map[xa + cg.cmax] : 0, mx1 = in1 ? map[xc + cg.cmax] : 0;
        // c0 (xa, row 2tq), c1 (xa, row 2tq+1), c2 (xc, 2tq), c3 (xc, 2tq+1)
#pragma unroll
        for (int i = 0; i < 4; i++) {
          const int h = i & 1, x = i < 2 ? xa : xc;
          if (x >= xs[h] && x <= xe[h])
            atomicAdd(grid + roff[h] + (i < 2 ? mx0 : mx1), f2d_grid(c[i]));
        }
        __syncwarp();
      }
    }
    if (a.task_cycles && lane == 0)
      atomicAdd((unsigned long long *)&a.task_cycles[t], (unsigned long long)(clock64() - t0));
    __syncwarp();
  }
}

} // namespace

// ------------------------------------------------------------------------
// launch wrappers
// ------------------------------------------------------------------------
template <typename N, int LPB>
static void launch_ortho_t(const GridArgs &a, bool collocate, int wmax, LaunchCfg &cfg,
                           cudaStream_t s) {
  // split tasks' sides: the row walk has an FP32 instance for them, the
  // other arithmetics take the point lists
  const bool split = a.core_side != 0;
  const bool pl = collocate && (cfg.variant == 1 || (split && !std::is_same<N, float>::value));
  const size_t per_warp = pl ? OrthoSmem<N, LPB>::bytes_coll_pl(wmax)
                          : collocate ? OrthoSmem<N, LPB>::bytes_coll(wmax)
                                      : OrthoSmem<N, LPB>::bytes_int(wmax);
  int nw = warps_for(per_warp);
  if (nw < 1)
    return launch_error("orthorhombic grid kernel: cube too large for shared memory");
  if (cfg.warps > 0 && cfg.warps < nw)
    nw = cfg.warps;
  const size_t smem = nw * per_warp;
  const bool rw_split = collocate && !pl && split; // FP32 only, see above
  const void *k = pl         ? (const void *)collocate_ortho_pl<N, LPB>
                  : rw_split ? (const void *)collocate_ortho<N, LPB, std::is_same<N, float>::value>
                  : collocate ? (const void *)collocate_ortho<N, LPB>
                              : (const void *)integrate_ortho<N, LPB>;
  set_smem((const void *)k, smem);
  const int nb = cfg.blocks > 0 ? cfg.blocks : cfg_blocks(cfg, persistent_blocks(k, 32 * nw, smem));
  cfg.warps = nw;
  cfg.blocks = nb;
  if (pl)
    collocate_ortho_pl<N, LPB><<<nb, 32 * nw, smem, s>>>(a, wmax);
  else if (rw_split)
    collocate_ortho<N, LPB, std::is_same<N, float>::value><<<nb, 32 * nw, smem, s>>>(a, wmax);
  else if (collocate)
    collocate_ortho<N, LPB><<<nb, 32 * nw, smem, s>>>(a, wmax);
  else
    integrate_ortho<N, LPB><<<nb, 32 * nw, smem, s>>>(a, wmax);
  count_launch();
}

template <int LPB>
static void launch_ortho_tc(const GridArgs &a, int wmax, LaunchCfg &cfg, cudaStream_t s) {
  const size_t per_warp = TcSmem<LPB>::bytes(wmax);
  int nw = warps_for(per_warp);
  if (nw < 1)
    return launch_error("orthorhombic grid kernel: cube too large for shared memory");
  if (cfg.warps > 0 && cfg.warps < nw)
    nw = cfg.warps;
  const size_t smem = nw * per_warp;
  const void *k = (const void *)integrate_ortho_tc<LPB>;
  set_smem(k, smem);
  const int nb = cfg.blocks > 0 ? cfg.blocks : cfg_blocks(cfg, persistent_blocks(k, 32 * nw, smem));
  cfg.warps = nw;
  cfg.blocks = nb;
  integrate_ortho_tc<LPB><<<nb, 32 * nw, smem, s>>>(a, wmax);
  count_launch();
}

template <int LPB>
static void launch_coll_tc(const GridArgs &a, int wmax, LaunchCfg &cfg, cudaStream_t s) {
  const size_t per_warp = TcCollSmem<LPB>::bytes(wmax);
  int nw = warps_for(per_warp);
  if (nw < 1)
    return launch_error("orthorhombic grid kernel: cube too large for shared memory");
  if (cfg.warps > 0 && cfg.warps < nw)
    nw = cfg.warps;
  const size_t smem = nw * per_warp;
  const void *k = (const void *)collocate_ortho_tc<LPB>;
  set_smem(k, smem);
  const int nb = cfg.blocks > 0 ? cfg.blocks : cfg_blocks(cfg, persistent_blocks(k, 32 * nw, smem));
  cfg.warps = nw;
  cfg.blocks = nb;
  collocate_ortho_tc<LPB><<<nb, 32 * nw, smem, s>>>(a, wmax);
  count_launch();
}

template <int LPB>
static void launch_ortho_lp(const GridArgs &a, int arith, bool collocate, int wmax,
                            LaunchCfg &cfg, cudaStream_t s) {
  if constexpr (LPB <= 6) {
    if (!collocate && arith == ARITH_FP32 && cfg.tensor)
      return launch_ortho_tc<LPB>(a, wmax, cfg, s);
    if (collocate && arith == ARITH_FP32 && cfg.tensor_coll)
      return launch_coll_tc<LPB>(a, wmax, cfg, s);
  }
  if (arith == ARITH_FP64)
    launch_ortho_t<double, LPB>(a, collocate, wmax, cfg, s);
  else if (arith == ARITH_FP32)
    launch_ortho_t<float, LPB>(a, collocate, wmax, cfg, s);
  else
    launch_ortho_t<dfloat, LPB>(a, collocate, wmax, cfg, s);
}

static void launch_grid(const GridArgs &a, int arith, bool general, bool collocate, int bucket,
                        int extent, LaunchCfg &cfg, cudaStream_t s) {
  if (general) {
    if (collocate)
      launch_collocate_general_impl(a, arith, kBucketLp[bucket], extent, cfg, s);
    else
      launch_integrate_general_impl(a, arith, kBucketLp[bucket], extent, cfg, s);
    return;
  }
  switch (kBucketLp[bucket]) {
  case 4: launch_ortho_lp<4>(a, arith, collocate, extent, cfg, s); break;
  case 6: launch_ortho_lp<6>(a, arith, collocate, extent, cfg, s); break;
  case 9: launch_ortho_lp<9>(a, arith, collocate, extent, cfg, s); break;
  case 12: launch_ortho_lp<12>(a, arith, collocate, extent, cfg, s); break;
  case 16: launch_ortho_lp<16>(a, arith, collocate, extent, cfg, s); break;
  }
}

template <typename N, int LPB>
static size_t ortho_per_warp(bool collocate, int variant, int wmax) {
  return collocate && variant == 1 ? OrthoSmem<N, LPB>::bytes_coll_pl(wmax)
         : collocate               ? OrthoSmem<N, LPB>::bytes_coll(wmax)
                                   : OrthoSmem<N, LPB>::bytes_int(wmax);
}

template <int LPB>
static size_t ortho_per_warp_lp(int arith, bool collocate, int variant, int wmax) {
  if (arith == ARITH_FP64)
    return ortho_per_warp<double, LPB>(collocate, variant, wmax);
  if (arith == ARITH_FP32)
    return ortho_per_warp<float, LPB>(collocate, variant, wmax);
  return ortho_per_warp<dfloat, LPB>(collocate, variant, wmax);
}

bool grid_launch_fits(int arith, bool general, bool collocate, int bucket, int extent,
                      int variant, int iwidth) {
  if (bucket < 0 || bucket >= kNumBuckets || extent < 1)
    return false;
  if (general)
    return general_launch_fits(arith, collocate, kBucketLp[bucket], extent, variant, iwidth);
  size_t pw = 0;
  switch (kBucketLp[bucket]) {
  case 4: pw = ortho_per_warp_lp<4>(arith, collocate, variant, extent); break;
  case 6: pw = ortho_per_warp_lp<6>(arith, collocate, variant, extent); break;
  case 9: pw = ortho_per_warp_lp<9>(arith, collocate, variant, extent); break;
  case 12: pw = ortho_per_warp_lp<12>(arith, collocate, variant, extent); break;
  case 16: pw = ortho_per_warp_lp<16>(arith, collocate, variant, extent); break;
  }
  return warps_for(pw) >= 1;
}

void launch_collocate(const GridArgs &a, int arith, bool general, int bucket, int extent,
                      LaunchCfg &cfg, cudaStream_t s) {
  launch_grid(a, arith, general, true, bucket, extent, cfg, s);
}

void launch_integrate(const GridArgs &a, int arith, bool general, int bucket, int extent,
                      LaunchCfg &cfg, cudaStream_t s) {
  launch_grid(a, arith, general, false, bucket, extent, cfg, s);
}

// ------------------------------------------------------------------------
// grid conversions around the mixed paths
// ------------------------------------------------------------------------
__global__ void grid_split_kernel(const double *__restrict__ src, void *__restrict__ dst,
                                  size_t n, int arith, float *__restrict__ hi) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const double v = src[i];
    if (arith == ARITH_FP32) {
      ((float *)dst)[i] = (float)v;
    } else {
      const float h = (float)v;
      ((float2 *)dst)[i] = make_float2(h, (float)(v - (double)h));
      if (hi) // dense high words for the mixed mode's FP32 tasks
        hi[i] = h;
    }
  }
}

__global__ void grid_fold_lo_kernel(double *__restrict__ g, const float *__restrict__ lo,
                                    size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    g[i] += (double)lo[i];
}

static int grid_blocks(size_t n) {
  size_t nb = (n + 255) / 256;
  return (int)(nb > 152 * 16 ? 152 * 16 : (nb ? nb : 1));
}

void launch_grid_split(const double *src, void *dst, size_t n, int arith, cudaStream_t s,
                       float *hi) {
  if (n == 0)
    return;
  grid_split_kernel<<<grid_blocks(n), 256, 0, s>>>(src, dst, n, arith, hi);
  count_launch();
}

void launch_grid_fold_lo(double *g, const float *lo, size_t n, cudaStream_t s) {
  if (n == 0)
    return;
  grid_fold_lo_kernel<<<grid_blocks(n), 256, 0, s>>>(g, lo, n);
  count_launch();
}

} // namespace gb300
