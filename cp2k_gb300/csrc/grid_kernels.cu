// Persistent collocate / integrate kernels of the GB300 grid backend.
//
// Work unit: one task (a pair of primitive Gaussians on one grid level) per
// warp.  Warps pull tasks from a queue (descending predicted cost) with one
// atomic per task; no CTA-wide synchronisation.
//
// Inside a task the cube is traversed separably, as CP2K's reference loops do
// (src/grid/ref/grid_ref_collint.h:30-327 orthorhombic, :333-794 general), but
// mapped onto the warp: lane <-> x index of the cube (sub-warps of 8/16 lanes
// for narrow cubes take several rows at once), planes k sequential, rows j
// sequential.  Per plane the z factor is folded into the coefficients
// (C_xy), per lane the x factor (q[ly]), so the per-point work is lp+1 FMAs:
//   collocate:  rho(x,y,z) += sum_ly q[ly](x) * pol_y[ly](y)  -> FP64 red to HBM
//   integrate:  w[ly] += V(x,y,z) * pol_y[ly](y)  (per lane), folded with z
//               per plane and with x + a warp reduction per task.
// The grid is touched with coalesced row segments; the collocate adds are
// FP64 atomics executed in L2 (the FP64 accumulation of the mixed path).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>

#include "gb300_internal.h"

namespace gb300 {

namespace {

constexpr unsigned FULL = 0xffffffffu;

template <typename T> __device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
    v += __shfl_xor_sync(FULL, v, o);
  return v;
}

template <typename T> struct Math;
template <> struct Math<double> {
  static __device__ __forceinline__ double gauss(double zetp, double x) {
    return exp(-zetp * x * x);
  }
};
template <> struct Math<float> {
  static __device__ __forceinline__ float gauss(float zetp, float x) {
    return expf(-zetp * x * x);
  }
};

// Per-warp shared memory of the orthorhombic kernels.
template <typename T, int LPB> struct OrthoSmem {
  static constexpr int P = LPB + 1;
  // per lane: [lz][ly] partial sums and pol_x, padded to an odd word count
  static __host__ __device__ constexpr int red_stride() {
    return ((P * (P + 1)) / 2 + P) | 1;
  }
  static __host__ __device__ size_t bytes(int wmax) {
    size_t b = sizeof(T) * (3 * (size_t)wmax * P + ncoset(LPB) + ntri(LPB));
    b += sizeof(int) * 3 * (size_t)wmax;
    b += sizeof(double) * ncoset(LPB); // integrate accumulator
    b += sizeof(T) * 32 * (size_t)red_stride(); // integrate x-fold transpose
    b += 32;                                     // alignment slack
    return (b + 15) & ~size_t(15);
  }
};

// 1-D factors pol[dir][c][l] = (x_c)^l exp(-zetp x_c^2), x_c = c*h - roff,
// c in [-cmax, cmax+1]; and the periodic maps map[dir][c] (REF's map[],
// grid_ref_collint.h:296-304).
template <typename T, int LPB>
__device__ __forceinline__ void fill_ortho_tables(const TaskDesc &d, const LevelDesc &L,
                                                  int cmax, int lp, T *pol, int *map,
                                                  int lane) {
  const int w = 2 * cmax + 2;
  for (int e = lane; e < 3 * w; e += 32) {
    const int dir = e / w, c = e - dir * w, cc = c - cmax;
    const double h = L.dh[dir * 4];
    T x;
    if (sizeof(T) == 8)
      x = (T)((double)cc * h - d.roff[dir]);
    else
      x = (T)fmaf((float)cc, (float)h, -(float)d.roff[dir]);
    T v = Math<T>::gauss((T)d.zetp, x);
    T *p = pol + (size_t)(dir * w + c) * (LPB + 1);
#pragma unroll
    for (int l = 0; l <= LPB; l++) {
      if (l > lp)
        break;
      p[l] = v;
      v *= x;
    }
    map[dir * w + c] = imod(d.center[dir] + cc - L.shift[dir], L.npts_global[dir]);
  }
}

// tri index of (ly, lx), lx + ly <= m
__device__ __forceinline__ int tri_idx(int ly, int lx, int m) {
  return ly * (m + 1) - (ly * (ly - 1)) / 2 + lx;
}

// ------------------------------------------------------------------------
// collocate, orthorhombic
// ------------------------------------------------------------------------
template <typename T, int LPB>
__global__ void __launch_bounds__(128)
    collocate_ortho(GridArgs a, int wmax) {
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr int P = LPB + 1;
  const int lane = threadIdx.x & 31;
  unsigned char *ws = smem + (threadIdx.x >> 5) * OrthoSmem<T, LPB>::bytes(wmax);
  T *pol = (T *)ws;
  T *coef = pol + 3 * (size_t)wmax * P;
  T *cxy = coef + ncoset(LPB);
  int *map = (int *)(cxy + ntri(LPB));
  const T *coefs = (const T *)a.coef;

  for (;;) {
    int qi = 0;
    if (lane == 0)
      qi = atomicAdd(a.counter, 1);
    qi = __shfl_sync(FULL, qi, 0);
    if (qi >= a.nqueue)
      break;
    const int t = a.queue[qi];
    const long long t0 = clock64();
    const TaskDesc d = a.tasks[t];
    const LevelDesc &L = a.levels.lv[d.level];
    const int lp = d.la_max + a.d.la_max + d.lb_max + a.d.lb_max;
    const SphereHdr H = a.sph[d.sphere];
    const int16_t *tab = a.sph_tab + H.off;
    const int K = 1 - H.lb[2];
    const int cmax = H.cmax, w = 2 * cmax + 2;
    if (w > wmax || lp > LPB) { // host sized the smem; never expected
      if (lane == 0)
        atomicOr(a.error, 1);
      continue;
    }
    const int nco = ncoset(lp);
    const T *csrc = coefs + a.coef_off[t];
    for (int e = lane; e < nco; e += 32)
      coef[e] = csrc[e];
    fill_ortho_tables<T, LPB>(d, L, cmax, lp, pol, map, lane);
    __syncwarp();

    double *grid = a.grids[d.level];
    const size_t nx = L.npts_local[0], nxy = nx * L.npts_local[1];
    const int x_lo = H.lb[0], x_hi = 1 - H.lb[0], width = x_hi - x_lo + 1;
    const int SW = width <= 8 ? 8 : (width <= 16 ? 16 : 32);
    const int G = 32 / SW, sub = lane % SW, grp = lane / SW;
    const int ntr = ntri(lp);

    for (int xc = x_lo; xc <= x_hi; xc += SW) {
      const int cx = xc + sub;
      const bool xin = cx <= x_hi;
      T px[P];
      const T *pxs = pol + (size_t)(cx + cmax) * P;
#pragma unroll
      for (int l = 0; l < P; l++)
        px[l] = (xin && l <= lp) ? pxs[l] : T(0);
      const int ig = xin ? map[cx + cmax] : 0;

      for (int k = H.lb[2]; k <= 1 - H.lb[2]; k++) {
        const int kk = k <= 0 ? -k : k - 1;
        const int js = tab[kk];
        const int16_t *irow = tab + 2 * K + tab[K + kk];
        // C_xy[ly][lx] = sum_lz C_xyz[lz][ly][lx] pol_z[lz](k)
        const T *pz = pol + (size_t)(2 * w + k + cmax) * P;
        for (int e = lane; e < ntr; e += 32) {
          int ly = 0, rem = e;
          while (rem > lp - ly) {
            rem -= lp - ly + 1;
            ly++;
          }
          const int lx = rem;
          T s = 0;
          for (int lz = 0; lz <= lp - ly - lx; lz++)
            s += coef[cidx(lz, ly, lx, lp)] * pz[lz];
          cxy[e] = s;
        }
        __syncwarp();
        // q[ly] = sum_lx C_xy[ly][lx] pol_x[lx](x_lane)
        T q[P];
#pragma unroll
        for (int ly = 0; ly < P; ly++) {
          T s = 0;
          if (ly <= lp) {
            const T *row = cxy + tri_idx(ly, 0, lp);
#pragma unroll
            for (int lx = 0; lx < P; lx++)
              if (lx <= lp - ly)
                s += row[lx] * px[lx];
          }
          q[ly] = s;
        }
        __syncwarp();
        double *gplane = grid + (size_t)map[2 * w + k + cmax] * nxy;
        for (int j0 = js; j0 <= 1 - js; j0 += G) {
          const int j = j0 + grp;
          if (!xin || j > 1 - js)
            continue;
          const int is = irow[j <= 0 ? -j : j - 1];
          if (cx < is || cx > 1 - is)
            continue;
          const T *py = pol + (size_t)(w + j + cmax) * P;
          T v = 0;
#pragma unroll
          for (int ly = 0; ly < P; ly++)
            if (ly <= lp)
              v += q[ly] * py[ly];
          atomicAdd(gplane + (size_t)map[w + j + cmax] * nx + ig, (double)v);
        }
      }
    }
    if (a.task_cycles && lane == 0)
      a.task_cycles[t] = clock64() - t0;
    __syncwarp();
  }
}

// ------------------------------------------------------------------------
// integrate, orthorhombic (adjoint of collocate_ortho)
// ------------------------------------------------------------------------
template <typename T, int LPB>
__global__ void __launch_bounds__(128)
    integrate_ortho(GridArgs a, int wmax) {
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr int P = LPB + 1;
  constexpr int NYZ = (LPB + 1) * (LPB + 2) / 2;
  const int lane = threadIdx.x & 31;
  unsigned char *ws = smem + (threadIdx.x >> 5) * OrthoSmem<T, LPB>::bytes(wmax);
  T *pol = (T *)ws;
  T *coef = pol + 3 * (size_t)wmax * P;
  T *cxy = coef + ncoset(LPB);
  int *map = (int *)(cxy + ntri(LPB));
  double *acc = (double *)(((uintptr_t)(map + 3 * wmax) + 7) & ~uintptr_t(7));
  T *red = (T *)(acc + ncoset(LPB));
  double *out = (double *)a.coef_out;

  for (;;) {
    int qi = 0;
    if (lane == 0)
      qi = atomicAdd(a.counter, 1);
    qi = __shfl_sync(FULL, qi, 0);
    if (qi >= a.nqueue)
      break;
    const int t = a.queue[qi];
    const long long t0 = clock64();
    const TaskDesc d = a.tasks[t];
    const LevelDesc &L = a.levels.lv[d.level];
    const int lp = d.la_max + a.d.la_max + d.lb_max + a.d.lb_max;
    const SphereHdr H = a.sph[d.sphere];
    const int16_t *tab = a.sph_tab + H.off;
    const int K = 1 - H.lb[2];
    const int cmax = H.cmax, w = 2 * cmax + 2;
    if (w > wmax || lp > LPB) {
      if (lane == 0)
        atomicOr(a.error, 1);
      continue;
    }
    const int nco = ncoset(lp);
    for (int e = lane; e < nco; e += 32)
      acc[e] = 0.0;
    fill_ortho_tables<T, LPB>(d, L, cmax, lp, pol, map, lane);
    __syncwarp();

    const T *grid = (const T *)a.grids_in[d.level];
    const size_t nx = L.npts_local[0], nxy = nx * L.npts_local[1];
    const int x_lo = H.lb[0], x_hi = 1 - H.lb[0], width = x_hi - x_lo + 1;
    const int SW = width <= 8 ? 8 : (width <= 16 ? 16 : 32);
    const int G = 32 / SW, sub = lane % SW, grp = lane / SW;

    for (int xc = x_lo; xc <= x_hi; xc += SW) {
      const int cx = xc + sub;
      const bool xin = cx <= x_hi;
      const int ig = xin ? map[cx + cmax] : 0;
      T ayz[NYZ]; // [lz][ly], lz + ly <= LPB
#pragma unroll
      for (int e = 0; e < NYZ; e++)
        ayz[e] = T(0);

      for (int k = H.lb[2]; k <= 1 - H.lb[2]; k++) {
        const int kk = k <= 0 ? -k : k - 1;
        const int js = tab[kk];
        const int16_t *irow = tab + 2 * K + tab[K + kk];
        const T *gplane = grid + (size_t)map[2 * w + k + cmax] * nxy;
        T wy[P];
#pragma unroll
        for (int l = 0; l < P; l++)
          wy[l] = T(0);
        for (int j0 = js; j0 <= 1 - js; j0 += G) {
          const int j = j0 + grp;
          if (!xin || j > 1 - js)
            continue;
          const int is = irow[j <= 0 ? -j : j - 1];
          if (cx < is || cx > 1 - is)
            continue;
          const T v = __ldg(gplane + (size_t)map[w + j + cmax] * nx + ig);
          const T *py = pol + (size_t)(w + j + cmax) * P;
#pragma unroll
          for (int ly = 0; ly < P; ly++)
            if (ly <= lp)
              wy[ly] += v * py[ly];
        }
        const T *pz = pol + (size_t)(2 * w + k + cmax) * P;
#pragma unroll
        for (int lz = 0; lz < P; lz++) {
          if (lz > lp)
            break;
          const T z = pz[lz];
#pragma unroll
          for (int ly = 0; ly < P; ly++)
            if (ly <= lp - lz)
              ayz[lz * P - (lz * (lz - 1)) / 2 + ly] += wy[ly] * z;
        }
      }
      // x fold and reduction over the warp through shared memory:
      // C_xyz[lz][ly][lx] += sum_lanes ayz[lz][ly] * pol_x[lx]
      {
        constexpr int RS = OrthoSmem<T, LPB>::red_stride();
        T *rl = red + lane * RS;
        const T *pxs = pol + (size_t)(cx + cmax) * P;
#pragma unroll
        for (int e = 0; e < NYZ; e++)
          rl[e] = ayz[e];
#pragma unroll
        for (int l = 0; l < P; l++)
          rl[NYZ + l] = (xin && l <= lp) ? pxs[l] : T(0);
        __syncwarp();
        for (int e = lane; e < nco; e += 32) {
          int lz, ly, lx;
          decode_cidx(e, lp, lz, ly, lx);
          const int yz = lz * P - (lz * (lz - 1)) / 2 + ly;
          T s = T(0);
#pragma unroll 8
          for (int r = 0; r < 32; r++)
            s += red[r * RS + yz] * red[r * RS + NYZ + lx];
          acc[e] += (double)s;
        }
        __syncwarp();
      }
    }
    __syncwarp();
    double *dst = out + a.coef_off[t];
    for (int e = lane; e < nco; e += 32)
      dst[e] = acc[e];
    if (a.task_cycles && lane == 0)
      a.task_cycles[t] = clock64() - t0;
    __syncwarp();
  }
}

} // namespace

// ------------------------------------------------------------------------
// launch wrappers
// ------------------------------------------------------------------------
template <typename T, int LPB>
static void launch_coll_t(const GridArgs &a, bool general, int wmax, int nblocks,
                          cudaStream_t s) {
  const size_t per_warp = OrthoSmem<T, LPB>::bytes(wmax);
  const int nw = warps_for(per_warp);
  const size_t smem = nw * per_warp;
  if (general) {
    launch_collocate_general_impl(a, sizeof(T) == 4, LPB, wmax, nblocks, s);
    return;
  }
  if (nw < 1)
    return launch_error("collocate: cube too large for shared memory");
  auto k = collocate_ortho<T, LPB>;
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (nblocks <= 0)
    nblocks = persistent_blocks((const void *)k, 32 * nw, smem);
  k<<<nblocks, 32 * nw, smem, s>>>(a, wmax);
  count_launch();
}

template <typename T, int LPB>
static void launch_int_t(const GridArgs &a, bool general, int wmax, int nblocks,
                         cudaStream_t s) {
  const size_t per_warp = OrthoSmem<T, LPB>::bytes(wmax);
  const int nw = warps_for(per_warp);
  const size_t smem = nw * per_warp;
  if (general) {
    launch_integrate_general_impl(a, sizeof(T) == 4, LPB, wmax, nblocks, s);
    return;
  }
  if (nw < 1)
    return launch_error("integrate: cube too large for shared memory");
  auto k = integrate_ortho<T, LPB>;
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (nblocks <= 0)
    nblocks = persistent_blocks((const void *)k, 32 * nw, smem);
  k<<<nblocks, 32 * nw, smem, s>>>(a, wmax);
  count_launch();
}

size_t ortho_smem_per_warp(bool fp32, int bucket, int wmax) {
  const int lpb = kBucketLp[bucket];
#define GB_CASE(LP)                                                            \
  if (lpb == LP)                                                               \
    return fp32 ? OrthoSmem<float, LP>::bytes(wmax) : OrthoSmem<double, LP>::bytes(wmax);
  GB_CASE(4) GB_CASE(6) GB_CASE(9) GB_CASE(16)
#undef GB_CASE
  return 0;
}

void launch_collocate(const GridArgs &a, bool fp32, bool general, int bucket,
                      int wmax, int nblocks, cudaStream_t s) {
  switch (kBucketLp[bucket]) {
#define GB_CASE(LP)                                                            \
  case LP:                                                                     \
    if (fp32)                                                                  \
      launch_coll_t<float, LP>(a, general, wmax, nblocks, s);                  \
    else                                                                       \
      launch_coll_t<double, LP>(a, general, wmax, nblocks, s);                 \
    break;
    GB_CASE(4) GB_CASE(6) GB_CASE(9) GB_CASE(16)
#undef GB_CASE
  }
}

void launch_integrate(const GridArgs &a, bool fp32, bool general, int bucket,
                      int wmax, int nblocks, cudaStream_t s) {
  switch (kBucketLp[bucket]) {
#define GB_CASE(LP)                                                            \
  case LP:                                                                     \
    if (fp32)                                                                  \
      launch_int_t<float, LP>(a, general, wmax, nblocks, s);                   \
    else                                                                       \
      launch_int_t<double, LP>(a, general, wmax, nblocks, s);                  \
    break;
    GB_CASE(4) GB_CASE(6) GB_CASE(9) GB_CASE(16)
#undef GB_CASE
  }
}

// FP64 -> FP32 copy of a potential grid for the mixed integrate path.
__global__ void grid_to_fp32_kernel(const double *__restrict__ src,
                                    float *__restrict__ dst, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    dst[i] = (float)src[i];
}

void launch_grid_to_fp32(const double *src, float *dst, size_t n, cudaStream_t s) {
  if (n == 0)
    return;
  int nb = (int)((n + 255) / 256);
  if (nb > 152 * 16)
    nb = 152 * 16;
  grid_to_fp32_kernel<<<nb, 256, 0, s>>>(src, dst, n);
  count_launch();
}

} // namespace gb300
