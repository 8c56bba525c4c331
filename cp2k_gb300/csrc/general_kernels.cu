// Collocate / integrate kernels for non-orthorhombic cells and border-masked
// tasks (CP2K's "general" path, src/grid/ref/grid_ref_collint.h:333-794).
//
// The polynomial lives in lattice-index coordinates (C_ijk, produced by the
// coefficient kernel from C_xyz), the point set is the index box around the
// sphere with per-row bounds from a quadratic in i (grid_ref_collint.h:
// 424-463).  Those bounds are computed in FP64 with explicitly rounded
// operations (no FMA contraction) so the visited points are exactly the
// reference's.  Mapping onto the warp as in the orthorhombic kernels: lane <->
// i, planes k and rows j sequential, per-point lp+1 FMAs; collocation also
// has a point-list form (collocate_general_pl) whose lanes take consecutive
// points of a plane.  Large boxes arrive as several work items, each a
// range of planes.
//
// Gaussian: FP64 path uses the reference's three pair factors (Mathieu's
// split, grid_ref_collint.h:358-367): e_ki per lane and plane, e_jk per row
// (precomputed per plane in shared memory), e_ij by a multiplicative
// recurrence along j.  FP32 path evaluates exp(-zetp r^2) per point from
// cube-local Cartesian offsets.  The double-float path (mixed mode) evaluates
// it per point in dfloat (df_exp_neg), see collocate_general_df.
#include <cuda_runtime.h>

#include <climits>
#include <cmath>
#include <type_traits>

#include "gb300_internal.h"
#include "numeric.cuh"

namespace gb300 {

namespace {

constexpr unsigned FULL = 0xffffffffu;

template <typename T> __device__ __forceinline__ T wsum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
    v += __shfl_xor_sync(FULL, v, o);
  return v;
}

template <typename T, int LPB> struct GenSmem {
  static constexpr int P = LPB + 1;
  // the integrate fold passes KC (kl, jl) rows at a time
  static constexpr int NKJ = (P * (P + 1)) / 2;
  static constexpr int KC = NKJ < 32 ? NKJ : 32;
  static __host__ __device__ constexpr int red_stride() { return (KC + P) | 1; }
  // the e_jk table of the FP64 Gaussian (none in the FP32 / dfloat kernels)
  static __host__ __device__ constexpr int ejk_words(int nj) {
    return std::is_same<T, double>::value ? nj : 0;
  }
  static __host__ __device__ size_t bytes(int nj) {
    size_t b = sizeof(double) * ncoset(LPB) + sizeof(double) * (size_t)ejk_words(nj); // acc, ejk
    b += sizeof(T) * (ncoset(LPB) + ntri(LPB));                            // coef, cij
    b += sizeof(T) * 32 * (size_t)red_stride();                            // fold
    b += sizeof(int2) * (size_t)nj;                                         // row bounds
    b += 32;                                                                // alignment slack
    return (b + 15) & ~size_t(15);
  }
};

struct GenTask {
  double gp[3];
  int imin[3], imax[3];
  int bnd[3][2];
  double h[9];  // dh
  double hh[3]; // |h0|^2, |h1|^2, |h2|^2
  double h01, h12, h20;
};

__device__ __forceinline__ void gen_setup(const TaskDesc &d, const LevelDesc &L, GenTask &g) {
  for (int i = 0; i < 3; i++) {
    g.gp[i] = d.roff[i];
    g.imin[i] = d.center[i];
    g.imax[i] = d.imax[i];
    g.bnd[i][0] = 0;
    g.bnd[i][1] = L.npts_local[i] - 1;
    if (d.border_mask & (1 << (2 * i)))
      g.bnd[i][0] += L.border_width[i];
    if (d.border_mask & (1 << (2 * i + 1)))
      g.bnd[i][1] -= L.border_width[i];
  }
  for (int i = 0; i < 9; i++)
    g.h[i] = L.dh[i];
  for (int a = 0; a < 3; a++)
    g.hh[a] = g.h[a * 3] * g.h[a * 3] + g.h[a * 3 + 1] * g.h[a * 3 + 1] +
              g.h[a * 3 + 2] * g.h[a * 3 + 2];
  auto dot = [&](int a, int b) {
    return g.h[a * 3] * g.h[b * 3] + g.h[a * 3 + 1] * g.h[b * 3 + 1] + g.h[a * 3 + 2] * g.h[b * 3 + 2];
  };
  g.h01 = dot(0, 1);
  g.h12 = dot(1, 2);
  g.h20 = dot(2, 0);
}

// grid index along dir for lattice index c, or -1 when outside the bounds
__device__ __forceinline__ int gmap(int c, int dir, const GenTask &g, const LevelDesc &L) {
  const int v = imod(c - L.shift[dir], L.npts_global[dir]);
  return (g.bnd[dir][0] <= v && v <= g.bnd[dir][1]) ? v : -1;
}

// Row bounds of (j, k) exactly as grid_ref_collint.h:431-463 evaluates them.
__device__ __forceinline__ int2 row_bounds(int j, int k, const GenTask &g, double radius) {
  double a = 0.0, b = 0.0, c = 0.0;
#pragma unroll
  for (int i = 0; i < 3; i++) {
    const double t0 = __dmul_rn(-g.gp[0], g.h[0 * 3 + i]);
    const double t1 = __dmul_rn(__dsub_rn((double)j, g.gp[1]), g.h[1 * 3 + i]);
    const double t2 = __dmul_rn(__dsub_rn((double)k, g.gp[2]), g.h[2 * 3 + i]);
    const double v = __dadd_rn(__dadd_rn(t0, t1), t2);
    a = __dadd_rn(a, __dmul_rn(g.h[i], g.h[i]));
    b = __dadd_rn(b, __dmul_rn(__dmul_rn(2.0, v), g.h[i]));
    c = __dadd_rn(c, __dmul_rn(v, v));
  }
  const double disc = __dsub_rn(__dmul_rn(b, b),
                                __dmul_rn(__dmul_rn(4.0, a), __dsub_rn(c, __dmul_rn(radius, radius))));
  if (!(0.0 < disc))
    return make_int2(1, 0);
  const double sq = __dsqrt_rn(disc);
  const double inv2a = __ddiv_rn(1.0, __dmul_rn(2.0, a));
  return make_int2((int)ceil(__dmul_rn(__dsub_rn(-b, sq), inv2a)),
                   (int)floor(__dmul_rn(__dadd_rn(-b, sq), inv2a)));
}

// The same bounds from a double-float evaluation, when that evaluation
// decides them: it carries an error bound (first order, with generous
// constants; eps below covers the dfloat arithmetic, the rounding of the
// inputs and the reference's own FP64 rounding) and answers only when the
// sign of the discriminant and both roots' floor/ceil are certain under it.
// Otherwise the caller falls back to row_bounds.  This keeps the visited
// points identical while moving the per-row work off the FP64 pipe.
struct RowFast {
  dfloat base[3], h0[3], h1[3], h2[3]; // v_c = base_c + j h1_c + k h2_c
  dfloat a4, inv2a, r2;                // 4 |h0|^2, 1 / (2 |h0|^2), radius^2
  float a, habs0;                      // |h0|^2, sum_c |h0_c|
};

__device__ __forceinline__ void row_fast_setup(const GenTask &g, double radius, RowFast &f) {
  double a = 0.0;
  float habs0 = 0.f;
  for (int c = 0; c < 3; c++) {
    f.base[c] = df_make(-g.gp[0] * g.h[c] - g.gp[1] * g.h[3 + c] - g.gp[2] * g.h[6 + c]);
    f.h0[c] = df_make(g.h[c]);
    f.h1[c] = df_make(g.h[3 + c]);
    f.h2[c] = df_make(g.h[6 + c]);
    a += g.h[c] * g.h[c];
    habs0 += fabsf((float)g.h[c]);
  }
  f.a4 = df_make(4.0 * a);
  f.inv2a = df_make(1.0 / (2.0 * a));
  f.r2 = df_make(radius * radius);
  f.a = (float)a;
  f.habs0 = habs0;
}

// true with the bounds in rb when decided, false when the caller must use
// the FP64 evaluation
__device__ __forceinline__ bool row_bounds_fast(int j, int k, const RowFast &f, int2 &rb) {
  constexpr float eps = 1.0e-12f;
  const float fj = (float)j, fk = (float)k;
  dfloat b{0.f, 0.f}, c{-f.r2.h, -f.r2.l};
  float vs = 0.f, vv = 0.f;
#pragma unroll
  for (int i = 0; i < 3; i++) {
    const dfloat v = df_fma1(df_fma1(f.base[i], f.h1[i], fj), f.h2[i], fk);
    vs += fabsf(f.base[i].h) + fabsf(fj * f.h1[i].h) + fabsf(fk * f.h2[i].h);
    vv += v.h * v.h;
    b = df_fma(b, v, f.h0[i]);
    c = df_fma(c, v, v);
  }
  b = dfloat{2.f * b.h, 2.f * b.l};
  const dfloat disc = df_fma(df_mul(dfloat{-f.a4.h, -f.a4.l}, c), b, b);
  const float ab = fabsf(b.h), r2 = f.r2.h;
  const float db = eps * (2.f * vs * f.habs0 + ab);
  const float dc = eps * (2.f * vs * vs + vv + r2);
  const float dd = 2.f * ab * db + f.a4.h * dc + eps * (ab * ab + f.a4.h * (vv + r2));
  if (disc.h <= -2.f * dd) {
    rb = make_int2(1, 0);
    return true;
  }
  if (disc.h <= 2.f * dd)
    return false;
  // dfloat square root: one Newton step from the FP32 root
  const float s0 = sqrtf(disc.h);
  const float corr = (fmaf(-s0, s0, disc.h) + disc.l) * (0.5f / s0);
  const dfloat sq = df_two_sum(s0, corr);
  const float ds = dd / sqrtf(disc.h - dd) + eps * s0;
  const float dx = (db + ds + eps * (ab + s0)) * f.inv2a.h;
  const dfloat nb{-b.h, -b.l};
  const dfloat x1 = df_mul(df_add(nb, dfloat{-sq.h, -sq.l}), f.inv2a);
  const dfloat x2 = df_mul(df_add(nb, sq), f.inv2a);
  const float m1 = 2.f * dx + eps * fabsf(x1.h) + fabsf(x1.l);
  const float m2 = 2.f * dx + eps * fabsf(x2.h) + fabsf(x2.l);
  if (fabsf(x1.h - rintf(x1.h)) <= m1 || fabsf(x2.h - rintf(x2.h)) <= m2)
    return false;
  rb = make_int2((int)ceilf(x1.h), (int)floorf(x2.h));
  return true;
}

// Per-plane preparation shared by collocate and integrate: row bounds (and
// for FP64 the e_jk factors) for every j of the box.
template <typename T>
__device__ __forceinline__ void plane_rows(int k, const GenTask &g, const LevelDesc &L,
                                           double radius, double zetp, int2 *rows,
                                           double *ejk, int lane, const RowFast &f) {
  const int nj = g.imax[1] - g.imin[1] + 1;
  const double dk = (double)k - g.gp[2];
  for (int r = lane; r < nj; r += 32) {
    const int j = g.imin[1] + r;
    int2 rb = make_int2(1, 0);
    if (gmap(j, 1, g, L) >= 0 && !row_bounds_fast(j, k, f, rb))
      rb = row_bounds(j, k, g, radius);
    rows[r] = rb;
    if constexpr (std::is_same<T, double>::value) {
      const double dj = (double)j - g.gp[1];
      ejk[r] = exp(-zetp * (dj * dj * g.hh[1] + 2.0 * dj * dk * g.h12));
    }
  }
}

template <typename T, int LPB>
__global__ void __launch_bounds__(128) collocate_general(GridArgs a, int njmax) {
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr int P = LPB + 1;
  const int lane = threadIdx.x & 31;
  unsigned char *ws = smem + (threadIdx.x >> 5) * GenSmem<T, LPB>::bytes(njmax);
  double *ejk = (double *)ws + ncoset(LPB);
  T *coef = (T *)(ejk + GenSmem<T, LPB>::ejk_words(njmax));
  T *cij = coef + ncoset(LPB);
  T *red = cij + ntri(LPB);
  int2 *rows = (int2 *)(((uintptr_t)(red + 32 * GenSmem<T, LPB>::red_stride()) + 7) & ~uintptr_t(7));
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
    GenTask g;
    gen_setup(d, L, g);
    const int k_lo = g.imin[2] + w.k0, k_hi = min(g.imax[2], g.imin[2] + w.k0 + w.nk - 1);
    RowFast rowf;
    row_fast_setup(g, d.radius, rowf);
    const int lp = d.la_max + a.d.la_max + d.lb_max + a.d.lb_max;
    const int nj = g.imax[1] - g.imin[1] + 1;
    if (nj > njmax || lp > LPB) {
      if (lane == 0)
        atomicOr(a.error, 1);
      continue;
    }
    const int nco = ncoset(lp), ntr = ntri(lp);
    if (sizeof(T) == 4 && a.coef_stride == 2) {
      // FP32 task of the mixed mode: the high words of the dfloat coefficients
      const float *csrc = (const float *)a.coef + 2 * (size_t)a.coef_off[t];
      for (int e = lane; e < nco; e += 32)
        coef[e] = (T)csrc[2 * e];
    } else {
      const T *csrc = coefs + a.coef_off[t];
      for (int e = lane; e < nco; e += 32)
        coef[e] = csrc[e];
    }
    double *grid = a.grids[d.level];
    const size_t nx = L.npts_local[0], nxy = nx * L.npts_local[1];
    const int width = g.imax[0] - g.imin[0] + 1;
    const int SW = width <= 8 ? 8 : (width <= 16 ? 16 : 32);
    const int G = 32 / SW, sub = lane % SW, grp = lane / SW;
    const double zetp = d.zetp;
    const float fj0 = (float)((double)g.imin[1] - g.gp[1]);

    for (int xc = g.imin[0]; xc <= g.imax[0]; xc += SW) {
      const int i = xc + sub;
      const bool xin = i <= g.imax[0];
      const int ig = xin ? gmap(i, 0, g, L) : -1;
      const double di = (double)i - g.gp[0];
      T px[P];
      {
        T p = T(1);
#pragma unroll
        for (int l = 0; l < P; l++) {
          px[l] = p;
          p *= (T)di;
        }
      }
      // FP64: e_ij(i, j) = exp(-zetp (di^2 |h0|^2 + 2 di dj h0.h1)) along j
      const double dj_first = (double)(g.imin[1] + grp) - g.gp[1];
      const double eij0 = (sizeof(T) == 8)
                              ? exp(-zetp * (di * di * g.hh[0] + 2.0 * di * dj_first * g.h01))
                              : 0.0;
      const double eij_step = (sizeof(T) == 8) ? exp(-zetp * 2.0 * di * g.h01 * G) : 0.0;
      // FP32: cube-local Cartesian offset of the lane's i
      float rx[3];
#pragma unroll
      for (int c = 0; c < 3; c++)
        rx[c] = (float)(di * g.h[c]);

      for (int k = k_lo; k <= k_hi; k++) {
        const int kg = gmap(k, 2, g, L);
        if (kg < 0)
          continue;
        const double dk = (double)k - g.gp[2];
        plane_rows<T>(k, g, L, d.radius, zetp, rows, ejk, lane, rowf);
        // C_ij = sum_kl C_ijk dk^kl
        for (int e = lane; e < ntr; e += 32) {
          int jl = 0, rem = e;
          while (rem > lp - jl) {
            rem -= lp - jl + 1;
            jl++;
          }
          const int il = rem;
          T s = 0, pk = T(1);
          for (int kl = 0; kl <= lp - jl - il; kl++) {
            s += coef[cidx(kl, jl, il, lp)] * pk;
            pk *= (T)dk;
          }
          cij[e] = s;
        }
        __syncwarp();
        T q[P];
#pragma unroll
        for (int jl = 0; jl < P; jl++) {
          T s = 0;
          if (jl <= lp) {
            const T *row = cij + jl * (lp + 1) - (jl * (jl - 1)) / 2;
#pragma unroll
            for (int il = 0; il < P; il++)
              if (il <= lp - jl)
                s += row[il] * px[il];
          }
          q[jl] = s;
        }
        const double eki = (sizeof(T) == 8)
                               ? exp(-zetp * (dk * dk * g.hh[2] + 2.0 * dk * di * g.h20))
                               : 0.0;
        float rk[3];
#pragma unroll
        for (int c = 0; c < 3; c++)
          rk[c] = rx[c] + (float)(dk * g.h[6 + c]);
        double eij = eij0;
        double *gplane = grid + (size_t)kg * nxy;
        for (int j0 = g.imin[1]; j0 <= g.imax[1]; j0 += G, eij *= eij_step) {
          const int j = j0 + grp;
          if (j > g.imax[1] || ig < 0)
            continue;
          const int2 rb = rows[j - g.imin[1]];
          if (i < rb.x || i > rb.y)
            continue;
          const int jg = gmap(j, 1, g, L); // >= 0 since rb non-empty
          const float djf = (float)(j - g.imin[1]) + fj0;
          T gauss;
          if (sizeof(T) == 8) {
            gauss = (T)(eij * ejk[j - g.imin[1]] * eki);
          } else {
            float r2 = 0.f;
#pragma unroll
            for (int c = 0; c < 3; c++) {
              const float rc = fmaf(djf, (float)g.h[3 + c], rk[c]);
              r2 = fmaf(rc, rc, r2);
            }
            gauss = (T)expf(-(float)zetp * r2);
          }
          T v = 0, pj = T(1);
          const T djt = (sizeof(T) == 8) ? (T)((double)j - g.gp[1]) : (T)djf;
#pragma unroll
          for (int jl = 0; jl < P; jl++) {
            if (jl <= lp)
              v += q[jl] * pj;
            pj *= djt;
          }
          if constexpr (sizeof(T) == 8)
            atomicAdd(gplane + (size_t)jg * nx + ig, (double)(v * gauss));
          else // integer-pipe conversion: the FP64 pipe is the scarce one
            atomicAdd(gplane + (size_t)jg * nx + ig, f2d_grid((float)(v * gauss)));
        }
        __syncwarp();
      }
    }
    if (a.task_cycles && lane == 0) // summed over the task's work items
      atomicAdd((unsigned long long *)&a.task_cycles[t], (unsigned long long)(clock64() - t0));
    __syncwarp();
  }
}

template <typename T, int LPB>
__global__ void __launch_bounds__(128) integrate_general(GridArgs a, int njmax) {
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr int P = LPB + 1;
  constexpr int NKJ = (LPB + 1) * (LPB + 2) / 2;
  const int lane = threadIdx.x & 31;
  unsigned char *ws = smem + (threadIdx.x >> 5) * GenSmem<T, LPB>::bytes(njmax);
  double *acc = (double *)ws;
  double *ejk = acc + ncoset(LPB);
  T *coef = (T *)(ejk + GenSmem<T, LPB>::ejk_words(njmax));
  T *cij = coef + ncoset(LPB);
  T *red = cij + ntri(LPB);
  int2 *rows = (int2 *)(((uintptr_t)(red + 32 * GenSmem<T, LPB>::red_stride()) + 7) & ~uintptr_t(7));
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
    GenTask g;
    gen_setup(d, L, g);
    const int k_lo = g.imin[2] + w.k0, k_hi = min(g.imax[2], g.imin[2] + w.k0 + w.nk - 1);
    RowFast rowf;
    row_fast_setup(g, d.radius, rowf);
    const int lp = d.la_max + a.d.la_max + d.lb_max + a.d.lb_max;
    const int nj = g.imax[1] - g.imin[1] + 1;
    if (nj > njmax || lp > LPB) {
      if (lane == 0)
        atomicOr(a.error, 1);
      continue;
    }
    const int nco = ncoset(lp);
    for (int e = lane; e < nco; e += 32)
      acc[e] = 0.0;
    __syncwarp();
    const T *grid = (const T *)a.grids_in[d.level];
    const int gs = sizeof(T) == 4 ? a.grid_stride : 1;
    const size_t nx = L.npts_local[0], nxy = nx * L.npts_local[1];
    const int width = g.imax[0] - g.imin[0] + 1;
    const int SW = width <= 8 ? 8 : (width <= 16 ? 16 : 32);
    const int G = 32 / SW, sub = lane % SW, grp = lane / SW;
    const double zetp = d.zetp;
    const float fj0 = (float)((double)g.imin[1] - g.gp[1]);

    for (int xc = g.imin[0]; xc <= g.imax[0]; xc += SW) {
      const int i = xc + sub;
      const bool xin = i <= g.imax[0];
      const int ig = xin ? gmap(i, 0, g, L) : -1;
      const double di = (double)i - g.gp[0];
      const double dj_first = (double)(g.imin[1] + grp) - g.gp[1];
      const double eij0 = (sizeof(T) == 8)
                              ? exp(-zetp * (di * di * g.hh[0] + 2.0 * di * dj_first * g.h01))
                              : 0.0;
      const double eij_step = (sizeof(T) == 8) ? exp(-zetp * 2.0 * di * g.h01 * G) : 0.0;
      float rx[3];
#pragma unroll
      for (int c = 0; c < 3; c++)
        rx[c] = (float)(di * g.h[c]);
      T akj[NKJ];
#pragma unroll
      for (int e = 0; e < NKJ; e++)
        akj[e] = T(0);

      for (int k = k_lo; k <= k_hi; k++) {
        const int kg = gmap(k, 2, g, L);
        if (kg < 0)
          continue;
        const double dk = (double)k - g.gp[2];
        plane_rows<T>(k, g, L, d.radius, zetp, rows, ejk, lane, rowf);
        __syncwarp();
        const double eki = (sizeof(T) == 8)
                               ? exp(-zetp * (dk * dk * g.hh[2] + 2.0 * dk * di * g.h20))
                               : 0.0;
        float rk[3];
#pragma unroll
        for (int c = 0; c < 3; c++)
          rk[c] = rx[c] + (float)(dk * g.h[6 + c]);
        T wj[P];
#pragma unroll
        for (int l = 0; l < P; l++)
          wj[l] = T(0);
        double eij = eij0;
        // FP32 tasks of the mixed mode read the high words of the (hi, lo) grid
        const T *gplane = grid + (size_t)kg * nxy * gs;
        for (int j0 = g.imin[1]; j0 <= g.imax[1]; j0 += G, eij *= eij_step) {
          const int j = j0 + grp;
          if (j > g.imax[1] || ig < 0)
            continue;
          const int2 rb = rows[j - g.imin[1]];
          if (i < rb.x || i > rb.y)
            continue;
          const int jg = gmap(j, 1, g, L);
          const float djf = (float)(j - g.imin[1]) + fj0;
          T gauss;
          if (sizeof(T) == 8) {
            gauss = (T)(eij * ejk[j - g.imin[1]] * eki);
          } else {
            float r2 = 0.f;
#pragma unroll
            for (int c = 0; c < 3; c++) {
              const float rc = fmaf(djf, (float)g.h[3 + c], rk[c]);
              r2 = fmaf(rc, rc, r2);
            }
            gauss = (T)expf(-(float)zetp * r2);
          }
          const T vg = __ldg(gplane + ((size_t)jg * nx + ig) * gs) * gauss;
          const T djt = (sizeof(T) == 8) ? (T)((double)j - g.gp[1]) : (T)djf;
          T pj = T(1);
#pragma unroll
          for (int jl = 0; jl < P; jl++) {
            if (jl <= lp)
              wj[jl] += vg * pj;
            pj *= djt;
          }
        }
        __syncwarp();
        T pk = T(1);
#pragma unroll
        for (int kl = 0; kl < P; kl++) {
          if (kl > lp)
            break;
#pragma unroll
          for (int jl = 0; jl < P; jl++)
            if (jl <= lp - kl)
              akj[kl * P - (kl * (kl - 1)) / 2 + jl] += wj[jl] * pk;
          pk *= (T)dk;
        }
      }
      // fold i and reduce over the warp through shared memory, KC rows of
      // akj per pass
      {
        constexpr int KC = GenSmem<T, LPB>::KC, RS = GenSmem<T, LPB>::red_stride();
        T *rl = red + lane * RS;
        T pi = xin ? T(1) : T(0);
#pragma unroll
        for (int l = 0; l < P; l++) {
          rl[KC + l] = pi;
          pi *= (T)di;
        }
#pragma unroll
        for (int c0 = 0; c0 < NKJ; c0 += KC) {
#pragma unroll
          for (int c = 0; c < KC; c++)
            if (c0 + c < NKJ)
              rl[c] = akj[c0 + c];
          __syncwarp();
          for (int e = lane; e < nco; e += 32) {
            int kl, jl, il;
            decode_cidx(e, lp, kl, jl, il);
            const int kj = kl * P - (kl * (kl - 1)) / 2 + jl - c0;
            if (kj < 0 || kj >= KC)
              continue;
            T s = T(0);
#pragma unroll 8
            for (int r = 0; r < 32; r++)
              s += red[r * RS + kj] * red[r * RS + KC + il];
            acc[e] += (double)s;
          }
          __syncwarp();
        }
      }
    }
    __syncwarp();
    double *dst = out + a.coef_off[t];
    for (int e = lane; e < nco; e += 32) {
      if (a.items || a.accum) // parts of one task add up (the buffer is zeroed)
        atomicAdd(dst + e, acc[e]);
      else
        dst[e] = acc[e];
    }
    if (a.task_cycles && lane == 0) // summed over the task's work items
      atomicAdd((unsigned long long *)&a.task_cycles[t], (unsigned long long)(clock64() - t0));
    __syncwarp();
  }
}

// ------------------------------------------------------------------------
// double-float (mixed mode) general kernels
//
// Same point set and polynomial as above, in dfloat arithmetic on the FP32
// pipes. The Gaussian is evaluated per point by df_exp_neg, from the
// exponent in completed-square form along the lane's j line:
//   zetp |r_ik + dj h1|^2 = A u^2 + x_perp,   u = dj - dj*,  A = zetp |h1|^2,
// where r_ik = di h0 + dk h2, dj* = -(r_ik . h1) / |h1|^2 and x_perp =
// zetp |r_ik|^2 - A dj*^2 >= 0. Both terms are non-negative, so the exponent
// carries no cancellation. The FP64 work left is per lane and plane (the
// line constants) and per row (the row bounds).
// ------------------------------------------------------------------------

// 2^(-j/64), j = 0..63, as dfloat pairs (the table of df_exp_neg)
__device__ __forceinline__ void fill_exp2_table(float2 *tab) {
  for (int j = threadIdx.x; j < 64; j += blockDim.x) {
    const double v = exp2(-(double)j / 64.0);
    const float h = (float)v;
    tab[j] = make_float2(h, (float)(v - (double)h));
  }
  __syncthreads();
}

struct DfLine {
  dfloat c0; // dj - dj* at the box's first row
  dfloat xp; // x_perp
};

__device__ __forceinline__ DfLine df_line(double di, double dk, const GenTask &g, double zetp,
                                          double inv_hh1, double fj0) {
  double rc[3];
#pragma unroll
  for (int c = 0; c < 3; c++)
    rc[c] = di * g.h[c] + dk * g.h[6 + c];
  const double rh = rc[0] * g.h[3] + rc[1] * g.h[4] + rc[2] * g.h[5];
  const double rr = rc[0] * rc[0] + rc[1] * rc[1] + rc[2] * rc[2];
  const double djs = -rh * inv_hh1;
  return DfLine{df_make(fj0 - djs), df_make(fmax(zetp * (rr - rh * rh * inv_hh1), 0.0))};
}

// Gaussian at row offset rf (rows from the box's first row) of the line
__device__ __forceinline__ dfloat df_gauss(const DfLine &L, dfloat A, float rf, const float2 *tab) {
  const dfloat u = df_add1(L.c0, rf);
  return df_exp_neg(df_fma(L.xp, df_mul(A, u), u), tab);
}

template <int LPB>
__global__ void __launch_bounds__(128) collocate_general_df(GridArgs a, int njmax) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ float2 tab[64];
  fill_exp2_table(tab);
  constexpr int P = LPB + 1;
  using S = GenSmem<dfloat, LPB>;
  const int lane = threadIdx.x & 31;
  unsigned char *ws = smem + (threadIdx.x >> 5) * S::bytes(njmax);
  double *ejk = (double *)ws + ncoset(LPB);
  dfloat *coef = (dfloat *)(ejk + S::ejk_words(njmax));
  dfloat *cij = coef + ncoset(LPB);
  dfloat *red = cij + ntri(LPB);
  int2 *rows = (int2 *)(((uintptr_t)(red + 32 * S::red_stride()) + 7) & ~uintptr_t(7));
  const dfloat *coefs = (const dfloat *)a.coef;

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
    GenTask g;
    gen_setup(d, L, g);
    const int k_lo = g.imin[2] + w.k0, k_hi = min(g.imax[2], g.imin[2] + w.k0 + w.nk - 1);
    RowFast rowf;
    row_fast_setup(g, d.radius, rowf);
    const int lp = d.la_max + a.d.la_max + d.lb_max + a.d.lb_max;
    const int nj = g.imax[1] - g.imin[1] + 1;
    if (nj > njmax || lp > LPB) {
      if (lane == 0)
        atomicOr(a.error, 1);
      continue;
    }
    const int nco = ncoset(lp), ntr = ntri(lp);
    for (int e = lane; e < nco; e += 32)
      coef[e] = coefs[a.coef_off[t] + e];
    double *grid = a.grids[d.level];
    float *glo = a.grids_lo[d.level];
    const size_t nx = L.npts_local[0], nxy = nx * L.npts_local[1];
    const int width = g.imax[0] - g.imin[0] + 1;
    const int SW = width <= 8 ? 8 : (width <= 16 ? 16 : 32);
    const int G = 32 / SW, sub = lane % SW, grp = lane / SW;
    const double zetp = d.zetp, inv_hh1 = 1.0 / g.hh[1];
    const double fj0 = (double)g.imin[1] - g.gp[1];
    const dfloat A = df_make(zetp * g.hh[1]), dj0 = df_make(fj0);

    for (int xc = g.imin[0]; xc <= g.imax[0]; xc += SW) {
      const int i = xc + sub;
      const bool xin = i <= g.imax[0];
      const int ig = xin ? gmap(i, 0, g, L) : -1;
      const double di = (double)i - g.gp[0];
      dfloat px[P];
      {
        const dfloat dd = df_make(di);
        dfloat p{1.f, 0.f};
#pragma unroll
        for (int l = 0; l < P; l++) {
          px[l] = p;
          p = df_mul(p, dd);
        }
      }
      for (int k = k_lo; k <= k_hi; k++) {
        const int kg = gmap(k, 2, g, L);
        if (kg < 0)
          continue;
        const double dk = (double)k - g.gp[2];
        plane_rows<dfloat>(k, g, L, d.radius, zetp, rows, ejk, lane, rowf);
        // C_ij = sum_kl C_ijk dk^kl (Horner in kl)
        const dfloat dkd = df_make(dk);
        for (int e = lane; e < ntr; e += 32) {
          int jl = 0, rem = e;
          while (rem > lp - jl) {
            rem -= lp - jl + 1;
            jl++;
          }
          const int il = rem;
          dfloat s{0.f, 0.f};
          for (int kl = lp - jl - il; kl >= 0; kl--)
            s = df_fma(coef[cidx(kl, jl, il, lp)], s, dkd);
          cij[e] = s;
        }
        __syncwarp();
        dfloat q[P];
#pragma unroll
        for (int jl = 0; jl < P; jl++) {
          dfloat s{0.f, 0.f};
          if (jl <= lp) {
            const dfloat *row = cij + jl * (lp + 1) - (jl * (jl - 1)) / 2;
#pragma unroll
            for (int il = 0; il < P; il++)
              if (il <= lp - jl)
                s = df_fma_acc(s, row[il], px[il]);
          }
          q[jl] = df_norm(s);
        }
        const DfLine line = df_line(di, dk, g, zetp, inv_hh1, fj0);
        double *gplane = grid + (size_t)kg * nxy;
        float *lplane = glo + (size_t)kg * nxy;
        for (int j0 = g.imin[1]; j0 <= g.imax[1]; j0 += G) {
          const int j = j0 + grp;
          if (j > g.imax[1] || ig < 0)
            continue;
          const int2 rb = rows[j - g.imin[1]];
          if (i < rb.x || i > rb.y)
            continue;
          const int jg = gmap(j, 1, g, L); // >= 0 since rb non-empty
          const float rf = (float)(j - g.imin[1]);
          const dfloat gauss = df_gauss(line, A, rf, tab);
          const dfloat dj = df_add1(dj0, rf);
          dfloat v{0.f, 0.f};
#pragma unroll
          for (int jl = P - 1; jl >= 0; jl--)
            if (jl <= lp)
              v = df_fma(q[jl], v, dj);
          const dfloat val = df_mul(v, gauss);
          const size_t idx = (size_t)jg * nx + ig;
          atomicAdd(gplane + idx, f2d_grid(val.h));
          atomicAdd(lplane + idx, val.l);
        }
        __syncwarp();
      }
    }
    if (a.task_cycles && lane == 0) // summed over the task's work items
      atomicAdd((unsigned long long *)&a.task_cycles[t], (unsigned long long)(clock64() - t0));
    __syncwarp();
  }
}

// acc + b without renormalisation (the sum of a long run is renormalised once)
__device__ __forceinline__ dfloat df_acc(dfloat acc, dfloat b) {
  const float s = acc.h + b.h;
  const float bb = s - acc.h;
  return dfloat{s, ((acc.h - (s - bb)) + (b.h - bb)) + (acc.l + b.l)};
}

// binomial coefficients up to the largest contraction order
struct BinomD {
  double v[GB300_LP_MAX + 1][GB300_LP_MAX + 1];
};
constexpr BinomD make_binom_d() {
  BinomD t{};
  for (int n = 0; n <= GB300_LP_MAX; n++) {
    t.v[n][0] = 1.0;
    for (int k = 1; k <= n; k++)
      t.v[n][k] = t.v[n][k - 1] * (n - k + 1) / k;
  }
  return t;
}
__constant__ BinomD kBinomD = make_binom_d();

// acc[cidx(kl, jl, il, lp)] holds sum w (i - r_i)^il (j - r_j)^jl (k - r_k)^kl
// over the task's points; replaced in place by the same sums about the
// centre c (c - r within half a grid step, so the binomial sums carry no
// cancellation).  One warp, lanes over the lines of each axis.
__device__ void shift_moments(double *acc, int lp, const double *c, const int *r, int lane) {
  for (int ax = 0; ax < 3; ax++) { // 0: i, 1: j, 2: k
    const double s = (double)r[ax] - c[ax]; // (x - c) = (x - r) + (r - c)
    double sp[GB300_LP_MAX + 1];
    sp[0] = 1.0;
    for (int n = 1; n <= lp; n++)
      sp[n] = sp[n - 1] * s;
    const int nlines = ntri(lp);
    for (int q = lane; q < nlines; q += 32) {
      // the line's two fixed exponents (u, v), u + v <= lp
      int u = 0, rem = q;
      while (rem > lp - u) {
        rem -= lp - u + 1;
        u++;
      }
      const int v = rem, L = lp - u - v;
      auto at = [&](int m) -> double & {
        return ax == 0 ? acc[cidx(u, v, m, lp)]
                       : (ax == 1 ? acc[cidx(u, m, v, lp)] : acc[cidx(m, u, v, lp)]);
      };
      for (int n = L; n >= 0; n--) {
        double sum = 0.0;
        for (int m = 0; m <= n; m++)
          sum = fma(kBinomD.v[n][m] * sp[n - m], at(m), sum);
        at(n) = sum;
      }
    }
    __syncwarp();
  }
}

template <int LPB>
__global__ void __launch_bounds__(128) integrate_general_df(GridArgs a, int njmax) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ float2 tab[64];
  fill_exp2_table(tab);
  constexpr int P = LPB + 1;
  constexpr int NKJ = (LPB + 1) * (LPB + 2) / 2;
  using S = GenSmem<dfloat, LPB>;
  const int lane = threadIdx.x & 31;
  unsigned char *ws = smem + (threadIdx.x >> 5) * S::bytes(njmax);
  double *acc = (double *)ws;
  double *ejk = acc + ncoset(LPB);
  dfloat *red = (dfloat *)(ejk + S::ejk_words(njmax)) + ncoset(LPB) + ntri(LPB);
  int2 *rows = (int2 *)(((uintptr_t)(red + 32 * S::red_stride()) + 7) & ~uintptr_t(7));
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
    GenTask g;
    gen_setup(d, L, g);
    const int k_lo = g.imin[2] + w.k0, k_hi = min(g.imax[2], g.imin[2] + w.k0 + w.nk - 1);
    RowFast rowf;
    row_fast_setup(g, d.radius, rowf);
    const int lp = d.la_max + a.d.la_max + d.lb_max + a.d.lb_max;
    const int nj = g.imax[1] - g.imin[1] + 1;
    if (nj > njmax || lp > LPB) {
      if (lane == 0)
        atomicOr(a.error, 1);
      continue;
    }
    const int nco = ncoset(lp);
    for (int e = lane; e < nco; e += 32)
      acc[e] = 0.0;
    __syncwarp();
    // the (hi, lo) float pairs of the split grid
    const float2 *grid = (const float2 *)a.grids_in[d.level];
    const size_t nx = L.npts_local[0], nxy = nx * L.npts_local[1];
    const int width = g.imax[0] - g.imin[0] + 1;
    const int SW = width <= 8 ? 8 : (width <= 16 ? 16 : 32);
    const int G = 32 / SW, sub = lane % SW, grp = lane / SW;
    const double zetp = d.zetp, inv_hh1 = 1.0 / g.hh[1];
    const double fj0 = (double)g.imin[1] - g.gp[1];
    const dfloat A = df_make(zetp * g.hh[1]);
    // the moments are taken about the grid point nearest the Gaussian's
    // centre, so that every power is of an exact small integer offset, and
    // shifted to the centre at the end
    int cref[3];
#pragma unroll
    for (int c = 0; c < 3; c++)
      cref[c] = (int)rint(g.gp[c]);

    for (int xc = g.imin[0]; xc <= g.imax[0]; xc += SW) {
      const int i = xc + sub;
      const bool xin = i <= g.imax[0];
      const int ig = xin ? gmap(i, 0, g, L) : -1;
      const double di = (double)i - g.gp[0];
      dfloat akj[NKJ];
#pragma unroll
      for (int e = 0; e < NKJ; e++)
        akj[e] = dfloat{0.f, 0.f};

      for (int k = k_lo; k <= k_hi; k++) {
        const int kg = gmap(k, 2, g, L);
        if (kg < 0)
          continue;
        const double dk = (double)k - g.gp[2];
        plane_rows<dfloat>(k, g, L, d.radius, zetp, rows, ejk, lane, rowf);
        __syncwarp();
        const DfLine line = df_line(di, dk, g, zetp, inv_hh1, fj0);
        dfloat wj[P];
#pragma unroll
        for (int l = 0; l < P; l++)
          wj[l] = dfloat{0.f, 0.f};
        const float2 *gplane = grid + (size_t)kg * nxy;
        for (int j0 = g.imin[1]; j0 <= g.imax[1]; j0 += G) {
          const int j = j0 + grp;
          if (j > g.imax[1] || ig < 0)
            continue;
          const int2 rb = rows[j - g.imin[1]];
          if (i < rb.x || i > rb.y)
            continue;
          const int jg = gmap(j, 1, g, L);
          const float rf = (float)(j - g.imin[1]);
          const float2 gv = __ldg(gplane + (size_t)jg * nx + ig);
          dfloat pj = df_mul(dfloat{gv.x, gv.y}, df_gauss(line, A, rf, tab));
          const float dj = (float)(j - cref[1]);
#pragma unroll
          for (int jl = 0; jl < P; jl++) {
            if (jl <= lp)
              wj[jl] = df_acc(wj[jl], pj);
            if (jl < P - 1)
              pj = df_mul1(pj, dj);
          }
        }
        __syncwarp();
        const float dkd = (float)(k - cref[2]);
        dfloat pk{1.f, 0.f};
#pragma unroll
        for (int kl = 0; kl < P; kl++) {
          if (kl > lp)
            break;
#pragma unroll
          for (int jl = 0; jl < P; jl++)
            if (jl <= lp - kl) {
              dfloat &x = akj[kl * P - (kl * (kl - 1)) / 2 + jl];
              x = df_fma_acc(x, df_norm(wj[jl]), pk);
            }
          pk = df_norm(df_mul1(pk, dkd));
        }
      }
      // fold i and reduce over the warp through shared memory, KC rows of
      // akj per pass
      {
        constexpr int KC = S::KC, RS = S::red_stride();
        dfloat *rl = red + lane * RS;
        const float dd = (float)(i - cref[0]);
        dfloat pi = xin ? dfloat{1.f, 0.f} : dfloat{0.f, 0.f};
#pragma unroll
        for (int l = 0; l < P; l++) {
          rl[KC + l] = pi;
          pi = df_norm(df_mul1(pi, dd));
        }
#pragma unroll
        for (int c0 = 0; c0 < NKJ; c0 += KC) {
#pragma unroll
          for (int c = 0; c < KC; c++)
            if (c0 + c < NKJ)
              rl[c] = df_norm(akj[c0 + c]);
          __syncwarp();
          for (int e = lane; e < nco; e += 32) {
            int kl, jl, il;
            decode_cidx(e, lp, kl, jl, il);
            const int kj = kl * P - (kl * (kl - 1)) / 2 + jl - c0;
            if (kj < 0 || kj >= KC)
              continue;
            dfloat s{0.f, 0.f};
#pragma unroll 8
            for (int r = 0; r < 32; r++)
              s = df_fma_acc(s, red[r * RS + kj], red[r * RS + KC + il]);
            acc[e] += to_double(df_norm(s));
          }
          __syncwarp();
        }
      }
    }
    __syncwarp();
    // moments about the reference point -> moments about the centre:
    // (x - c)^n = sum_m C(n, m) (x - r)^m (r - c)^(n - m), axis by axis
    shift_moments(acc, lp, g.gp, cref, lane);
    double *dst = out + a.coef_off[t];
    for (int e = lane; e < nco; e += 32) {
      if (a.items || a.accum) // parts of one task add up (the buffer is zeroed)
        atomicAdd(dst + e, acc[e]);
      else
        dst[e] = acc[e];
    }
    if (a.task_cycles && lane == 0) // summed over the task's work items
      atomicAdd((unsigned long long *)&a.task_cycles[t], (unsigned long long)(clock64() - t0));
    __syncwarp();
  }
}

// ------------------------------------------------------------------------
// point-list collocation, general path (FP32 and double-float)
//
// The kernels above bind lanes to i and walk the box's rows: lanes whose i
// lies outside the sphere's row idle, and the sphere fills about half of
// the box.  Here the warp first builds, per plane, the clipped i-range of
// every row and their prefix offsets, and per i of the box the x-folded
// polynomial Q[i][jl] = sum_il C_ij[jl][il] di^il and the Gaussian's line
// constants; then it walks the plane's points in row-major order, 32
// consecutive points per step.  Same points and arithmetic as
// collocate_general_df / collocate_general<float>.
// ------------------------------------------------------------------------
template <typename T, int LPB> struct PlSmem {
  static constexpr int P = LPB + 1;
  static __host__ __device__ size_t bytes(int nj, int iw) {
    size_t b = sizeof(T) * (ncoset(LPB) + ntri(LPB) + (size_t)iw * P); // coef, cij, Q
    b = (b + 15) & ~size_t(15);
    b += sizeof(float4) * (size_t)iw;                                   // line constants
    b += sizeof(int) * (size_t)iw;                                      // grid index of i
    b = (b + 7) & ~size_t(7);
    b += sizeof(int2) * (size_t)nj + sizeof(int) * (2 * (size_t)nj + 1); // rows, jg, offsets
    return (b + 15) & ~size_t(15);
  }
};

template <typename T, int LPB>
__global__ void __launch_bounds__(128) collocate_general_pl(GridArgs a, int njmax) {
  constexpr bool DF = std::is_same<T, dfloat>::value;
  using M = Num<T>;
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ float2 tab[64];
  fill_exp2_table(tab);
  constexpr int P = LPB + 1;
  const int iw = a.iwidth;
  const int lane = threadIdx.x & 31;
  unsigned char *ws = smem + (threadIdx.x >> 5) * PlSmem<T, LPB>::bytes(njmax, iw);
  T *coef = (T *)ws;
  T *cij = coef + ncoset(LPB);
  T *Q = cij + ntri(LPB); // [iw][P]
  float4 *lin = (float4 *)(((uintptr_t)(Q + (size_t)iw * P) + 15) & ~uintptr_t(15));
  int *igx = (int *)(lin + iw);
  int2 *rows = (int2 *)(((uintptr_t)(igx + iw) + 7) & ~uintptr_t(7));
  int *jgr = (int *)(rows + njmax);
  int *off = jgr + njmax; // [njmax + 1]

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
    GenTask g;
    gen_setup(d, L, g);
    RowFast rowf;
    row_fast_setup(g, d.radius, rowf);
    const int k_lo = g.imin[2] + w.k0, k_hi = min(g.imax[2], g.imin[2] + w.k0 + w.nk - 1);
    const int lp = d.la_max + a.d.la_max + d.lb_max + a.d.lb_max;
    const int nj = g.imax[1] - g.imin[1] + 1;
    const int width = g.imax[0] - g.imin[0] + 1;
    if (nj > njmax || lp > LPB || width > iw) {
      if (lane == 0)
        atomicOr(a.error, 1);
      continue;
    }
    const int nco = ncoset(lp), ntr = ntri(lp);
    if constexpr (DF) {
      const dfloat *csrc = (const dfloat *)a.coef + a.coef_off[t];
      for (int e = lane; e < nco; e += 32)
        coef[e] = csrc[e];
    } else if (a.coef_stride == 2) { // FP32 class of the mixed mode: high words
      const float *csrc = (const float *)a.coef + 2 * (size_t)a.coef_off[t];
      for (int e = lane; e < nco; e += 32)
        coef[e] = csrc[2 * e];
    } else {
      const float *csrc = (const float *)a.coef + a.coef_off[t];
      for (int e = lane; e < nco; e += 32)
        coef[e] = csrc[e];
    }
    for (int x = lane; x < width; x += 32)
      igx[x] = gmap(g.imin[0] + x, 0, g, L);
    double *grid = a.grids[d.level];
    float *glo = a.grids_lo[d.level];
    const size_t nx = L.npts_local[0], nxy = nx * L.npts_local[1];
    const double zetp = d.zetp, inv_hh1 = 1.0 / g.hh[1];
    const double fj0 = (double)g.imin[1] - g.gp[1];
    const dfloat A = df_make(zetp * g.hh[1]), dj0 = df_make(fj0);
    const float fj0f = (float)fj0, zetpf = (float)zetp;
    const float h1f[3] = {(float)g.h[3], (float)g.h[4], (float)g.h[5]};

    for (int k = k_lo; k <= k_hi; k++) {
      const int kg = gmap(k, 2, g, L);
      if (kg < 0)
        continue;
      const double dk = (double)k - g.gp[2];
      plane_rows<T>(k, g, L, d.radius, zetp, rows, nullptr, lane, rowf);
      __syncwarp();
      // clipped i-range per row, the row's grid index, exclusive offsets
      int total = 0;
      for (int r0 = 0; r0 < nj; r0 += 32) {
        const int r = r0 + lane;
        int len = 0;
        if (r < nj) {
          const int2 rb = rows[r];
          const int i0 = max(rb.x, g.imin[0]), i1 = min(rb.y, g.imax[0]);
          len = max(0, i1 - i0 + 1);
          rows[r] = make_int2(i0, i1);
          jgr[r] = len > 0 ? gmap(g.imin[1] + r, 1, g, L) : -1;
        }
        int inc = len;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int y = __shfl_up_sync(FULL, inc, o);
          if (lane >= o)
            inc += y;
        }
        if (r < nj)
          off[r] = total + inc - len;
        total += __shfl_sync(FULL, inc, 31);
      }
      if (lane == 0)
        off[nj] = total;
      // C_ij = sum_kl C_ijk dk^kl (Horner in kl)
      const T dkt = M::from(dk);
      for (int e = lane; e < ntr; e += 32) {
        int jl = 0, rem = e;
        while (rem > lp - jl) {
          rem -= lp - jl + 1;
          jl++;
        }
        const int il = rem;
        T s = M::zero();
        for (int kl = lp - jl - il; kl >= 0; kl--)
          s = M::fma(coef[cidx(kl, jl, il, lp)], s, dkt);
        cij[e] = s;
      }
      __syncwarp();
      // per i of the box: Q[i][jl] and the Gaussian's line constants
      for (int x = lane; x < width; x += 32) {
        const double di = (double)(g.imin[0] + x) - g.gp[0];
        T px[P];
        {
          const T dd = M::from(di);
          T p = T(1);
#pragma unroll
          for (int l = 0; l < P; l++) {
            px[l] = p;
            p = M::mul(p, dd);
          }
        }
#pragma unroll
        for (int jl = 0; jl < P; jl++) {
          T s = M::zero();
          if (jl <= lp) {
            const T *row = cij + jl * (lp + 1) - (jl * (jl - 1)) / 2;
#pragma unroll
            for (int il = 0; il < P; il++)
              if (il <= lp - jl)
                s = M::fma_acc(s, row[il], px[il]);
          }
          Q[(size_t)x * P + jl] = M::norm(s);
        }
        if constexpr (DF) {
          const DfLine ln = df_line(di, dk, g, zetp, inv_hh1, fj0);
          lin[x] = make_float4(ln.c0.h, ln.c0.l, ln.xp.h, ln.xp.l);
        } else {
          float rk[3];
#pragma unroll
          for (int c = 0; c < 3; c++)
            rk[c] = (float)(di * g.h[c]) + (float)(dk * g.h[6 + c]);
          lin[x] = make_float4(rk[0], rk[1], rk[2], 0.f);
        }
      }
      __syncwarp();
      double *gplane = grid + (size_t)kg * nxy;
      int r = 0;
      for (int p0 = 0; p0 < total; p0 += 32) {
        const int p = p0 + lane;
        if (p >= total)
          continue;
        while (off[r + 1] <= p)
          r++;
        const int i = rows[r].x + (p - off[r]);
        const int x = i - g.imin[0];
        const int ig = igx[x];
        if (ig < 0)
          continue;
        const T *q = Q + (size_t)x * P;
        const float4 lv = lin[x];
        const float rf = (float)r;
        const size_t idx = (size_t)jgr[r] * nx + ig;
        if constexpr (DF) {
          const dfloat gauss = df_gauss(DfLine{dfloat{lv.x, lv.y}, dfloat{lv.z, lv.w}}, A, rf, tab);
          const dfloat dj = df_add1(dj0, rf);
          dfloat v{0.f, 0.f};
#pragma unroll
          for (int jl = P - 1; jl >= 0; jl--)
            if (jl <= lp)
              v = df_fma(q[jl], v, dj);
          const dfloat val = df_mul(v, gauss);
          atomicAdd(gplane + idx, f2d_grid(val.h));
          atomicAdd(glo + (size_t)kg * nxy + idx, val.l);
        } else {
          const float djf = rf + fj0f;
          float r2 = 0.f;
          const float rk[3] = {lv.x, lv.y, lv.z};
#pragma unroll
          for (int c = 0; c < 3; c++) {
            const float rc = fmaf(djf, h1f[c], rk[c]);
            r2 = fmaf(rc, rc, r2);
          }
          float v = 0.f;
#pragma unroll
          for (int jl = P - 1; jl >= 0; jl--)
            if (jl <= lp)
              v = fmaf(v, djf, q[jl]);
          atomicAdd(gplane + idx, f2d_grid(v * expf(-zetpf * r2)));
        }
      }
      __syncwarp();
    }
    if (a.task_cycles && lane == 0) // summed over the task's work items
      atomicAdd((unsigned long long *)&a.task_cycles[t], (unsigned long long)(clock64() - t0));
    __syncwarp();
  }
}

template <typename T, int LPB>
const void *gen_kernel(bool collocate) {
  if constexpr (std::is_same<T, dfloat>::value)
    return collocate ? (const void *)collocate_general_df<LPB>
                     : (const void *)integrate_general_df<LPB>;
  else
    return collocate ? (const void *)collocate_general<T, LPB>
                     : (const void *)integrate_general<T, LPB>;
}

template <typename T, int LPB>
void launch_gen(const GridArgs &a, bool collocate, int njmax, LaunchCfg &cfg, cudaStream_t s) {
  // variant 1: point-list collocation (FP32 and double-float)
  constexpr bool can_pl = !std::is_same<T, double>::value;
  const bool pl = can_pl && collocate && cfg.variant == 1;
  const size_t per_warp =
      pl ? PlSmem<T, LPB>::bytes(njmax, a.iwidth) : GenSmem<T, LPB>::bytes(njmax);
  int nw = warps_for(per_warp);
  if (nw < 1)
    return launch_error("general path: box too large for shared memory");
  if (cfg.warps > 0 && cfg.warps < nw)
    nw = cfg.warps;
  const size_t smem = nw * per_warp;
  if constexpr (can_pl) {
    if (pl) {
      const void *k = (const void *)collocate_general_pl<T, LPB>;
      set_smem(k, smem);
      const int nb =
          cfg.blocks > 0 ? cfg.blocks : cfg_blocks(cfg, persistent_blocks(k, 32 * nw, smem));
      cfg.warps = nw;
      cfg.blocks = nb;
      collocate_general_pl<T, LPB><<<nb, 32 * nw, smem, s>>>(a, njmax);
      count_launch();
      return;
    }
  }
  const void *k = gen_kernel<T, LPB>(collocate);
  set_smem(k, smem);
  const int nb = cfg.blocks > 0 ? cfg.blocks : cfg_blocks(cfg, persistent_blocks(k, 32 * nw, smem));
  cfg.warps = nw;
  cfg.blocks = nb;
  if constexpr (std::is_same<T, dfloat>::value) {
    if (collocate)
      collocate_general_df<LPB><<<nb, 32 * nw, smem, s>>>(a, njmax);
    else
      integrate_general_df<LPB><<<nb, 32 * nw, smem, s>>>(a, njmax);
  } else {
    if (collocate)
      collocate_general<T, LPB><<<nb, 32 * nw, smem, s>>>(a, njmax);
    else
      integrate_general<T, LPB><<<nb, 32 * nw, smem, s>>>(a, njmax);
  }
  count_launch();
}

void launch_gen_any(const GridArgs &a, bool collocate, int arith, int lpb, int njmax,
                    LaunchCfg &cfg, cudaStream_t s) {
  switch (lpb) {
#define GB_CASE(LP)                                                            \
  case LP:                                                                     \
    if (arith == ARITH_FP32)                                                   \
      launch_gen<float, LP>(a, collocate, njmax, cfg, s);                      \
    else if (arith == ARITH_MIXED)                                             \
      launch_gen<dfloat, LP>(a, collocate, njmax, cfg, s);                     \
    else                                                                       \
      launch_gen<double, LP>(a, collocate, njmax, cfg, s);                     \
    break;
    GB_CASE(4) GB_CASE(6) GB_CASE(9) GB_CASE(12) GB_CASE(16)
#undef GB_CASE
  }
}

template <typename T, int LPB>
size_t gen_per_warp(bool collocate, int njmax, int variant, int iwidth) {
  constexpr bool can_pl = !std::is_same<T, double>::value;
  return can_pl && collocate && variant == 1 ? PlSmem<T, LPB>::bytes(njmax, iwidth)
                                             : GenSmem<T, LPB>::bytes(njmax);
}

} // namespace

bool general_launch_fits(int arith, bool collocate, int lpb, int njmax, int variant, int iwidth) {
  size_t pw = 0;
  switch (lpb) {
#define GB_CASE(LP)                                                            \
  case LP:                                                                     \
    pw = arith == ARITH_FP32    ? gen_per_warp<float, LP>(collocate, njmax, variant, iwidth)  \
         : arith == ARITH_MIXED ? gen_per_warp<dfloat, LP>(collocate, njmax, variant, iwidth) \
                                : gen_per_warp<double, LP>(collocate, njmax, variant, iwidth); \
    break;
    GB_CASE(4) GB_CASE(6) GB_CASE(9) GB_CASE(12) GB_CASE(16)
#undef GB_CASE
  default: return false;
  }
  return warps_for(pw) >= 1;
}

void launch_collocate_general_impl(const GridArgs &a, int arith, int lpb, int njmax,
                                   LaunchCfg &cfg, cudaStream_t s) {
  launch_gen_any(a, true, arith, lpb, njmax, cfg, s);
}

void launch_integrate_general_impl(const GridArgs &a, int arith, int lpb, int njmax,
                                   LaunchCfg &cfg, cudaStream_t s) {
  launch_gen_any(a, false, arith, lpb, njmax, cfg, s);
}

} // namespace gb300
