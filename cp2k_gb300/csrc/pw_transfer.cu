// Multigrid transfer between the realspace level grids and the plane-wave
// grid, and the periodic Hartree solve between them, kept on the device, so
// that collocate -> FFT -> Poisson -> integrate stays in HBM (CP2K:
// src/pw_env/rs_pw_interface.F:64-136 density_rs2pw and :151-228
// potential_pw2rs with the default pw_interp, replicated grids;
// src/pw/pw_poisson_types.F:316-320 the periodic influence function 4 pi /
// |G|^2 and src/pw/pw_poisson_methods.F:363-367 the Hartree energy; the
// reference's GPU FFT helpers are src/pw/gpu/pw_gpu_kernels.cu).
//
// Conventions of the reference's pw layer, restated:
//   * a grid of n points per direction holds the frequencies -n/2 .. n/2 - 1
//     in every direction (src/pw/pw_grid_info.F:247-254), all of them (no
//     spherical cutoff on these grids);
//   * realspace -> G space divides by the number of points, G space ->
//     realspace does not (src/pw/fft_tools.F:394-397);
//   * a coarse level's coefficients add into the finest level's at the same
//     frequency (pw_axpy on grids that reference each other,
//     src/pw/pw_methods.F:748-925), and the finest level's coefficients at a
//     coarse level's frequencies are that level's coefficients (pw_copy);
//   * potential_pw2rs scales a coarse level's real-space values by
//     dvol(level) / dvol(finest) = N(finest) / N(level).
//
// Data layout: every grid x fastest, [nz][ny][nx] (the collocate / integrate
// grids); G-space arrays are the full complex boxes [nz][ny][nx] of
// double2 (re, im) in FFT order.  Three-dimensional complex FFTs in FP64
// (cuFFT), plans and work arrays owned by the handle.
#include <cuda_runtime.h>
#include <cufft.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "gb300_internal.h"
#include "grid_gb300.h"

#define GB300_API extern "C" __attribute__((visibility("default")))

namespace gb300 {
namespace {

[[noreturn]] void pw_fail(const char *what, int code) {
  fprintf(stderr, "grid_gb300 error: plane-wave transfer: %s (%d)\n", what, code);
  abort();
}
#define CKC(x)                                                                 \
  do {                                                                         \
    cudaError_t e_ = (x);                                                      \
    if (e_ != cudaSuccess)                                                     \
      pw_fail(#x, (int)e_);                                                    \
  } while (0)
#define CKF(x)                                                                 \
  do {                                                                         \
    cufftResult r_ = (x);                                                      \
    if (r_ != CUFFT_SUCCESS)                                                   \
      pw_fail(#x, (int)r_);                                                    \
  } while (0)

// array index of frequency f on a grid of n points, and the reverse
__device__ __forceinline__ int freq_of(int a, int n) { return a < (n + 1) / 2 ? a : a - n; }
__device__ __forceinline__ int index_of(int f, int n) { return f >= 0 ? f : f + n; }

struct Box {
  int n[3]; // x, y, z
};

// re(c[i]) = g[i], im = 0
__global__ void real_to_complex(const double *__restrict__ g, double2 *__restrict__ c, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    c[i] = make_double2(g[i], 0.0);
}

// g[i] = scale * re(c[i])
__global__ void complex_to_real(const double2 *__restrict__ c, double *__restrict__ g, size_t n,
                                double scale) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    g[i] = scale * c[i].x;
}

// fine[f] (+)= scale * coarse[f] for every frequency f of the coarse box
__global__ void spectrum_pad(const double2 *__restrict__ coarse, Box cb, double2 *__restrict__ fine,
                             Box fb, double scale, int accumulate) {
  const size_t n = (size_t)cb.n[0] * cb.n[1] * cb.n[2];
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const int ax = (int)(i % cb.n[0]), ay = (int)((i / cb.n[0]) % cb.n[1]),
              az = (int)(i / ((size_t)cb.n[0] * cb.n[1]));
    const int fx = index_of(freq_of(ax, cb.n[0]), fb.n[0]);
    const int fy = index_of(freq_of(ay, cb.n[1]), fb.n[1]);
    const int fz = index_of(freq_of(az, cb.n[2]), fb.n[2]);
    const size_t j = ((size_t)fz * fb.n[1] + fy) * fb.n[0] + fx;
    const double2 v = coarse[i];
    if (accumulate) {
      fine[j].x += scale * v.x;
      fine[j].y += scale * v.y;
    } else {
      fine[j] = make_double2(scale * v.x, scale * v.y);
    }
  }
}

// coarse[f] = scale * fine[f] for every frequency f of the coarse box
__global__ void spectrum_cut(const double2 *__restrict__ fine, Box fb, double2 *__restrict__ coarse,
                             Box cb, double scale) {
  const size_t n = (size_t)cb.n[0] * cb.n[1] * cb.n[2];
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const int ax = (int)(i % cb.n[0]), ay = (int)((i / cb.n[0]) % cb.n[1]),
              az = (int)(i / ((size_t)cb.n[0] * cb.n[1]));
    const int fx = index_of(freq_of(ax, cb.n[0]), fb.n[0]);
    const int fy = index_of(freq_of(ay, cb.n[1]), fb.n[1]);
    const int fz = index_of(freq_of(az, cb.n[2]), fb.n[2]);
    const double2 v = fine[((size_t)fz * fb.n[1] + fy) * fb.n[0] + fx];
    coarse[i] = make_double2(scale * v.x, scale * v.y);
  }
}

// out = the spectrum of Re(inverse transform of v): (v(f) + conj(v(-f))) / 2,
// -f taken on the same grid (the Nyquist frequency -n/2 is its own partner)
__global__ void hermitian_part(const double2 *__restrict__ v, double2 *__restrict__ out, Box b) {
  const size_t n = (size_t)b.n[0] * b.n[1] * b.n[2];
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const int ax = (int)(i % b.n[0]), ay = (int)((i / b.n[0]) % b.n[1]),
              az = (int)(i / ((size_t)b.n[0] * b.n[1]));
    const int px = index_of(-freq_of(ax, b.n[0]), b.n[0]) % b.n[0];
    const int py = index_of(-freq_of(ay, b.n[1]), b.n[1]) % b.n[1];
    const int pz = index_of(-freq_of(az, b.n[2]), b.n[2]) % b.n[2];
    const double2 a = v[i], c = v[((size_t)pz * b.n[1] + py) * b.n[0] + px];
    out[i] = make_double2(0.5 * (a.x + c.x), 0.5 * (a.y - c.y));
  }
}

// 2 pi times the reciprocal vectors b_d (rows), b_d . a_e = delta_de
struct Recip {
  double b[3][3];
};

// v(G) = 4 pi rho(G) / |G|^2, zero at G = 0; the sum of |rho(G)|^2 4 pi /
// |G|^2 into esum (when given), by block partial sums
__global__ void poisson_kernel(const double2 *rho, double2 *v, Box bx, // may alias
                               Recip r, double *esum) {
  __shared__ double part[8];
  const size_t n = (size_t)bx.n[0] * bx.n[1] * bx.n[2];
  double local = 0.0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const int ax = (int)(i % bx.n[0]), ay = (int)((i / bx.n[0]) % bx.n[1]),
              az = (int)(i / ((size_t)bx.n[0] * bx.n[1]));
    const double f[3] = {(double)freq_of(ax, bx.n[0]), (double)freq_of(ay, bx.n[1]),
                         (double)freq_of(az, bx.n[2])};
    double g2 = 0.0;
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const double gc = f[0] * r.b[0][c] + f[1] * r.b[1][c] + f[2] * r.b[2][c];
      g2 += gc * gc;
    }
    const double2 p = rho[i];
    const double k = g2 > 0.0 ? 4.0 * M_PI / g2 : 0.0;
    v[i] = make_double2(k * p.x, k * p.y);
    local += k * (p.x * p.x + p.y * p.y);
  }
  if (!esum)
    return;
  for (int o = 16; o > 0; o >>= 1)
    local += __shfl_xor_sync(0xffffffffu, local, o);
  if ((threadIdx.x & 31) == 0)
    part[threadIdx.x >> 5] = local;
  __syncthreads();
  if (threadIdx.x == 0) {
    double sacc = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++)
      sacc += part[w];
    atomicAdd(esum, sacc);
  }
}

int blocks_for(size_t n) {
  const size_t b = (n + 255) / 256;
  return (int)(b < 152 * 8 ? (b ? b : 1) : 152 * 8);
}

} // namespace
} // namespace gb300

using namespace gb300;

struct grid_gb300_pw_transfer {
  int nlevels = 0;
  double *d_esum = nullptr;      // Hartree energy sum of the Poisson solve
  std::vector<Box> box;          // per level
  std::vector<size_t> npts;      // per level
  std::vector<cufftHandle> plan; // per level, Z2Z
  std::vector<double2 *> work;   // per level, one complex box
};

GB300_API void grid_gb300_pw_create(const int nlevels, const int *npts,
                                    grid_gb300_pw_transfer **handle) {
  if (nlevels < 1 || nlevels > GB300_MAX_LEVELS)
    pw_fail("number of levels out of range", nlevels);
  grid_gb300_pw_transfer *h = new grid_gb300_pw_transfer();
  h->nlevels = nlevels;
  for (int l = 0; l < nlevels; l++) {
    Box b;
    for (int d = 0; d < 3; d++) {
      b.n[d] = npts[3 * l + d];
      if (b.n[d] < 1 || b.n[d] > npts[d])
        pw_fail("level grids must be non-empty and no larger than the first (finest)", l);
    }
    h->box.push_back(b);
    h->npts.push_back((size_t)b.n[0] * b.n[1] * b.n[2]);
    cufftHandle p;
    CKF(cufftPlan3d(&p, b.n[2], b.n[1], b.n[0], CUFFT_Z2Z));
    h->plan.push_back(p);
    double2 *w = nullptr;
    CKC(cudaMalloc((void **)&w, sizeof(double2) * h->npts.back()));
    h->work.push_back(w);
  }
  *handle = h;
}

GB300_API void grid_gb300_pw_free(grid_gb300_pw_transfer *h) {
  if (!h)
    return;
  for (size_t l = 0; l < h->plan.size(); l++) {
    cufftDestroy(h->plan[l]);
    cudaFree(h->work[l]);
  }
  if (h->d_esum)
    cudaFree(h->d_esum);
  delete h;
}

GB300_API void grid_gb300_pw_density_rs2pw(grid_gb300_pw_transfer *h,
                                           const double *const *rs_grids, double *rho,
                                           void *rho_gspace, void *stream) {
  cudaStream_t s = (cudaStream_t)stream;
  const int L = h->nlevels;
  double2 *fine = rho_gspace ? (double2 *)rho_gspace : h->work[0];
  // the finest level first: its spectrum starts the sum
  for (int l = 0; l < L; l++) {
    CKF(cufftSetStream(h->plan[l], s));
    double2 *w = h->work[l];
    real_to_complex<<<blocks_for(h->npts[l]), 256, 0, s>>>(rs_grids[l], w, h->npts[l]);
    CKF(cufftExecZ2Z(h->plan[l], (cufftDoubleComplex *)w, (cufftDoubleComplex *)w,
                     CUFFT_FORWARD));
    spectrum_pad<<<blocks_for(h->npts[l]), 256, 0, s>>>(w, h->box[l], fine, h->box[0],
                                                         1.0 / (double)h->npts[l], l > 0);
    count_launch(2);
  }
  if (rho) {
    // G space -> realspace on the finest grid (no scale); the sum stays in
    // rho_gspace when the caller asked for it
    double2 *w = h->work[0];
    if (fine != w)
      CKC(cudaMemcpyAsync(w, fine, sizeof(double2) * h->npts[0], cudaMemcpyDeviceToDevice, s));
    CKF(cufftExecZ2Z(h->plan[0], (cufftDoubleComplex *)w, (cufftDoubleComplex *)w,
                     CUFFT_INVERSE));
    complex_to_real<<<blocks_for(h->npts[0]), 256, 0, s>>>(w, rho, h->npts[0], 1.0);
    count_launch();
  }
  CKC(cudaGetLastError());
}

GB300_API void grid_gb300_pw_potential_pw2rs(grid_gb300_pw_transfer *h, const double *v_rspace,
                                             double *const *rs_grids, void *stream) {
  cudaStream_t s = (cudaStream_t)stream;
  const int L = h->nlevels;
  // the finest level is the potential itself (pw_copy)
  CKC(cudaMemcpyAsync(rs_grids[0], v_rspace, sizeof(double) * h->npts[0],
                      cudaMemcpyDeviceToDevice, s));
  if (L == 1)
    return;
  double2 *f = h->work[0];
  CKF(cufftSetStream(h->plan[0], s));
  real_to_complex<<<blocks_for(h->npts[0]), 256, 0, s>>>(v_rspace, f, h->npts[0]);
  CKF(cufftExecZ2Z(h->plan[0], (cufftDoubleComplex *)f, (cufftDoubleComplex *)f, CUFFT_FORWARD));
  count_launch();
  for (int l = 1; l < L; l++) {
    CKF(cufftSetStream(h->plan[l], s));
    double2 *w = h->work[l];
    spectrum_cut<<<blocks_for(h->npts[l]), 256, 0, s>>>(f, h->box[0], w, h->box[l],
                                                         1.0 / (double)h->npts[0]);
    CKF(cufftExecZ2Z(h->plan[l], (cufftDoubleComplex *)w, (cufftDoubleComplex *)w,
                     CUFFT_INVERSE));
    complex_to_real<<<blocks_for(h->npts[l]), 256, 0, s>>>(
        w, rs_grids[l], h->npts[l], (double)h->npts[0] / (double)h->npts[l]);
    count_launch(2);
  }
  CKC(cudaGetLastError());
}

GB300_API void grid_gb300_pw_potential_g2rs(grid_gb300_pw_transfer *h, const void *v_gspace,
                                            double *const *rs_grids, void *stream) {
  cudaStream_t s = (cudaStream_t)stream;
  const int L = h->nlevels;
  // the spectrum of the real potential on the finest grid (what
  // potential_pw2rs's forward transform of it would give)
  double2 *w0 = h->work[0];
  hermitian_part<<<blocks_for(h->npts[0]), 256, 0, s>>>((const double2 *)v_gspace, w0, h->box[0]);
  count_launch();
  // coarser levels first (they read w0): the coefficients at their
  // frequencies, as potential_pw2rs
  for (int l = 1; l < L; l++) {
    CKF(cufftSetStream(h->plan[l], s));
    double2 *w = h->work[l];
    spectrum_cut<<<blocks_for(h->npts[l]), 256, 0, s>>>(w0, h->box[0], w, h->box[l], 1.0);
    CKF(cufftExecZ2Z(h->plan[l], (cufftDoubleComplex *)w, (cufftDoubleComplex *)w,
                     CUFFT_INVERSE));
    complex_to_real<<<blocks_for(h->npts[l]), 256, 0, s>>>(
        w, rs_grids[l], h->npts[l], (double)h->npts[0] / (double)h->npts[l]);
    count_launch(2);
  }
  // the finest level: back to real space (no scale)
  CKF(cufftSetStream(h->plan[0], s));
  CKF(cufftExecZ2Z(h->plan[0], (cufftDoubleComplex *)w0, (cufftDoubleComplex *)w0,
                   CUFFT_INVERSE));
  complex_to_real<<<blocks_for(h->npts[0]), 256, 0, s>>>(w0, rs_grids[0], h->npts[0], 1.0);
  count_launch();
  CKC(cudaGetLastError());
}

GB300_API void grid_gb300_pw_poisson(grid_gb300_pw_transfer *h, const double *dh,
                                     const void *rho_gspace, void *v_gspace, double *v_rspace,
                                     double *energy, void *stream) {
  cudaStream_t s = (cudaStream_t)stream;
  const Box &b = h->box[0];
  // hmat: columns are the cell vectors a_d = n_d dh[d][:]
  double hm[3][3];
  for (int c = 0; c < 3; c++)
    for (int d = 0; d < 3; d++)
      hm[c][d] = b.n[d] * dh[3 * d + c];
  const double det = hm[0][0] * (hm[1][1] * hm[2][2] - hm[1][2] * hm[2][1]) -
                     hm[0][1] * (hm[1][0] * hm[2][2] - hm[1][2] * hm[2][0]) +
                     hm[0][2] * (hm[1][0] * hm[2][1] - hm[1][1] * hm[2][0]);
  if (!(fabs(det) > 0.0))
    pw_fail("Poisson solve: singular cell", 0);
  // inverse by cofactors: inv[e][c] = cof[c][e] / det; 2 pi b_e = 2 pi inv[e][:]
  Recip r;
  for (int e = 0; e < 3; e++)
    for (int c = 0; c < 3; c++) {
      const int c1 = (c + 1) % 3, c2 = (c + 2) % 3, e1 = (e + 1) % 3, e2 = (e + 2) % 3;
      const double cof = hm[c1][e1] * hm[c2][e2] - hm[c1][e2] * hm[c2][e1];
      r.b[e][c] = 2.0 * M_PI * cof / det;
    }
  if (energy) {
    if (!h->d_esum)
      CKC(cudaMalloc((void **)&h->d_esum, sizeof(double)));
    CKC(cudaMemsetAsync(h->d_esum, 0, sizeof(double), s));
  }
  poisson_kernel<<<blocks_for(h->npts[0]), 256, 0, s>>>(
      (const double2 *)rho_gspace, (double2 *)v_gspace, b, r, energy ? h->d_esum : nullptr);
  count_launch();
  CKC(cudaGetLastError());
  if (v_rspace) { // G space -> realspace on the finest grid (no scale)
    double2 *w = h->work[0];
    CKF(cufftSetStream(h->plan[0], s));
    CKC(cudaMemcpyAsync(w, v_gspace, sizeof(double2) * h->npts[0], cudaMemcpyDeviceToDevice, s));
    CKF(cufftExecZ2Z(h->plan[0], (cufftDoubleComplex *)w, (cufftDoubleComplex *)w,
                     CUFFT_INVERSE));
    complex_to_real<<<blocks_for(h->npts[0]), 256, 0, s>>>(w, v_rspace, h->npts[0], 1.0);
    count_launch();
    CKC(cudaGetLastError());
  }
  if (energy) {
    double sum = 0.0;
    CKC(cudaMemcpyAsync(&sum, h->d_esum, sizeof(double), cudaMemcpyDeviceToHost, s));
    CKC(cudaStreamSynchronize(s));
    *energy = 0.5 * fabs(det) * sum;
  }
}

