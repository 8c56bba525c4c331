// Allocation-free single-task collocation.
//
// Some callers cannot allocate device memory while they run: a program that
// reserved all of the GPU's memory for its own pool at start-up and hands out
// pieces of that arena only, and drivers that forbid cudaMalloc/cudaFree after
// initialisation because those calls can synchronise the whole device and
// stall every other stream.  grid_gb300_collocate_pgf_product_static lets them
// collocate one primitive pair with device buffers they already own: every
// piece of per-call scratch (the task descriptor, sphere bounds, polynomial
// coefficients, work counters) lives in one file-scope __device__ array of
// fixed size, kStaticScratchBytes, that every GPU which loads this library
// holds until the process exits.
//
// The array is shared by all calls: each call overwrites what the previous
// one left (the work counter and error word are reset by the call itself),
// and two calls whose kernels overlap on the GPU (different streams without
// ordering) race on it.  The first call on a device resolves the array's
// device address with cudaGetSymbolAddress and keeps it.
//
// Errors are found on the host before anything is copied or launched: the
// scratch layout, the coefficient kernel's and the grid kernel's shared-
// memory budgets.  The grid kernel's own per-task size check (an error word
// in the scratch array) cannot trigger for a launch planned from this one
// task, and it is not read back, which would need a synchronisation.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "gb300_internal.h"
#include "grid_gb300.h"

#define GB300_API extern "C" __attribute__((visibility("default")))

namespace gb300 {

static constexpr size_t kStaticScratchBytes = 256 * 1024;
static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

namespace {

std::mutex g_mu;
void *g_addr[64] = {}; // device address of g_static_scratch per device ordinal
// the last error of a call, per calling host thread
thread_local char g_err[256] = "";

int set_error(const char *msg) {
  snprintf(g_err, sizeof(g_err), "%s", msg);
  return 1;
}

// once per device, with that device current
int scratch_address(void **out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
    return set_error("no current CUDA device");
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_addr[dev]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess || !p)
      return set_error("cudaGetSymbolAddress of the static scratch array failed");
    g_addr[dev] = p;
  }
  *out = g_addr[dev];
  return 0;
}

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

LDiffs ldiffs_of(int f, bool *ok) {
  *ok = true;
  if (f == GRID_FUNC_AB)
    return LDiffs{0, 0, 0, 0};
  if (f >= 411 && f <= 433 && f % 10 >= 1 && f % 10 <= 3)
    return LDiffs{1, -1, 2, -1};
  if ((f >= 701 && f <= 703) || (f >= 801 && f <= 803))
    return LDiffs{2, -2, 2, -2};
  if (f == 200 || (f >= 301 && f <= 303) || (f >= 501 && f <= 503) || (f >= 601 && f <= 603) ||
      (f >= 901 && f <= 906) || (f >= 1001 && f <= 1003))
    return LDiffs{1, -1, 1, -1};
  *ok = false;
  return LDiffs{0, 0, 0, 0};
}

} // namespace
} // namespace gb300

using namespace gb300;

GB300_API const char *grid_gb300_static_scratch_error(void) { return g_err; }

GB300_API size_t grid_gb300_static_scratch_bytes(void) { return kStaticScratchBytes; }

GB300_API int grid_gb300_collocate_pgf_product_static(
    const bool orthorhombic, const int border_mask, const int func, const int la_max,
    const int la_min, const int lb_max, const int lb_min, const double zeta, const double zetb,
    const double rscale, const double *dh, const double *dh_inv, const double *ra,
    const double *rab, const int *npts_global, const int *npts_local, const int *shift_local,
    const int *border_width, const double radius, const int o1, const int o2, const int n1,
    const int n2, const double *pab, double *grid, void *stream) {
  (void)n2;
  bool ok = true;
  const LDiffs dl = ldiffs_of(func, &ok);
  if (!ok)
    return set_error("unknown grid_func");
  if (la_max < 0 || lb_max < 0 || la_max > GB300_LMAX || lb_max > GB300_LMAX || la_min < 0 ||
      lb_min < 0 || la_min > la_max || lb_min > lb_max)
    return set_error("angular momenta out of range");
  const int lp = la_max + dl.la_max + lb_max + dl.lb_max;
  if (bucket_of(lp) < 0)
    return set_error("contraction order exceeds the supported maximum");
  void *base = nullptr;
  if (scratch_address(&base))
    return 1;

  // ---- level and geometry, with the reference's FP64 expressions
  //      (src/grid/ref/grid_ref_collint.h:207-245, 609-640, 917-947)
  LevelSet levels{};
  levels.nlevels = 1;
  LevelDesc &L = levels.lv[0];
  for (int i = 0; i < 3; i++) {
    L.npts_global[i] = npts_global[i];
    L.npts_local[i] = npts_local[i];
    L.shift[i] = shift_local[i];
    L.border_width[i] = border_width[i];
  }
  L.dh_max = 0.0;
  for (int i = 0; i < 9; i++) {
    L.dh[i] = dh[i];
    L.dh_inv[i] = dh_inv[i];
    L.dh_max = fmax(L.dh_max, fabs(dh[i]));
  }
  if (2.0 * radius < L.dh_max)
    return 0; // maps onto no grid point (grid_ref_collint.h:928-937)

  TaskDesc d;
  memset(&d, 0, sizeof(d));
  d.la_max = (int8_t)la_max;
  d.la_min = (int8_t)la_min;
  d.lb_max = (int8_t)lb_max;
  d.lb_min = (int8_t)lb_min;
  d.o1 = (int16_t)o1;
  d.o2 = (int16_t)o2;
  d.border_mask = (uint8_t)border_mask;
  d.radius = radius;
  d.zeta = zeta;
  d.zetb = zetb;
  d.iatom = 0;
  d.jatom = 1;
  const double zetp = zeta + zetb, f = zetb / zetp;
  const double rab2 = rab[0] * rab[0] + rab[1] * rab[1] + rab[2] * rab[2];
  d.zetp = zetp;
  // the coefficient kernel multiplies by 2 for iatom != jatom
  d.prefexp = 0.5 * rscale * exp(-zeta * f * rab2);
  for (int k = 0; k < 3; k++) {
    d.rab[k] = rab[k];
    d.rp[k] = ra[k] + f * rab[k];
  }
  std::vector<int16_t> tab;
  SphereHdr sph{};
  int extent = 1;
  const bool general = !(orthorhombic && border_mask == 0);
  if (!general) {
    for (int k = 0; k < 3; k++) {
      double s_ = 0.0;
      for (int j = 0; j < 3; j++)
        s_ += L.dh_inv[j * 3 + k] * d.rp[j];
      d.center[k] = (int)floor(s_);
      d.roff[k] = d.rp[k] - ((double)d.center[k]) * L.dh[k * 4];
    }
    const double drmin = fmin(L.dh[0], fmin(L.dh[4], L.dh[8]));
    const double nrad = fmax(1.0, ceil(d.radius / drmin));
    // size of the sphere table before building it: [K] + [K] + rows + [K][NX]
    double ext[3];
    for (int i = 0; i < 3; i++)
      ext[i] = 1.0 - ceil(-1e-8 - drmin * nrad * L.dh_inv[i * 4]);
    const double tab_bytes = 2.0 * ext[2] * (2.0 + ext[1] + ext[0]);
    if (!(tab_bytes < 0.5 * (double)kStaticScratchBytes))
      return set_error("task needs more scratch than the static array holds "
                       "(grid_gb300_static_scratch_bytes)");
    long long np = 0;
    build_sphere(L, drmin * nrad, sph, tab, np);
    for (int k = 0; k < 3; k++)
      if (L.npts_global[k] != L.npts_local[k]) {
        const int off = imod(d.center[k] + sph.lb[k] - L.shift[k], L.npts_global[k]) - sph.lb[k];
        if (!(off + 1 - sph.lb[k] < L.npts_local[k] && off + sph.lb[k] >= 0))
          return set_error("cube does not fit into the local grid");
      }
    extent = 2 * sph.cmax + 2;
  } else {
    d.flags |= TF_GENERAL;
    for (int k = 0; k < 3; k++) {
      double g = 0.0;
      for (int j = 0; j < 3; j++)
        g += L.dh_inv[j * 3 + k] * d.rp[j];
      d.roff[k] = g;
      d.center[k] = INT32_MAX;
      d.imax[k] = INT32_MIN;
    }
    for (int a = -1; a <= 1; a++)
      for (int b = -1; b <= 1; b++)
        for (int c = -1; c <= 1; c++) {
          const double x = d.rp[0] + a * d.radius, y = d.rp[1] + b * d.radius,
                       z = d.rp[2] + c * d.radius;
          for (int k = 0; k < 3; k++) {
            const double r = L.dh_inv[0 * 3 + k] * x + L.dh_inv[1 * 3 + k] * y +
                             L.dh_inv[2 * 3 + k] * z;
            d.center[k] = d.center[k] < (int)floor(r) ? d.center[k] : (int)floor(r);
            d.imax[k] = d.imax[k] > (int)ceil(r) ? d.imax[k] : (int)ceil(r);
          }
        }
    extent = d.imax[1] - d.center[1] + 1;
  }
  SubblockDesc sb;
  memset(&sb, 0, sizeof(sb));
  sb.cart_offset = 0;
  sb.ncoa = n1; // pab is [n2][n1]
  sb.ncob = n2;
  sb.ntasks = 1;

  // ---- layout of the scratch array
  const int nco = ncoset(lp);
  size_t off = 0;
  const size_t o_task = off;
  off = align256(off + sizeof(TaskDesc));
  const size_t o_sub = off;
  off = align256(off + sizeof(SubblockDesc));
  const size_t o_ints = off; // coef_off, queue, counter, error
  off = align256(off + 4 * sizeof(int));
  const size_t o_atoms = off;
  off = align256(off + 6 * sizeof(double));
  const size_t o_levels = off;
  off = align256(off + sizeof(LevelSet));
  std::vector<double> dhtab;
  build_dh_table(levels, dhtab);
  const size_t o_dhtab = off;
  off = align256(off + dhtab.size() * sizeof(double));
  const size_t o_sph = off;
  off = align256(off + sizeof(SphereHdr));
  const size_t o_tab = off;
  off = align256(off + tab.size() * sizeof(int16_t) + 2);
  const size_t o_seeds = off;
  off = align256(off + 18 * sizeof(float2));
  const size_t o_coef = off;
  off = align256(off + (size_t)nco * sizeof(double));
  if (off > kStaticScratchBytes)
    return set_error("task needs more scratch than the static array holds "
                     "(grid_gb300_static_scratch_bytes)");
  const int coef_w = (int)coef_words(la_max + dl.la_max, lb_max + dl.lb_max);
  if (!coefficients_fit(coef_w))
    return set_error("angular momenta too large for the coefficient kernel's shared memory");
  if (!grid_launch_fits(ARITH_FP64, general, true, bucket_of(lp), extent, 0, 0))
    return set_error(general ? "general path: box too large for shared memory"
                             : "orthorhombic path: cube too large for shared memory");

  std::vector<unsigned char> host(o_coef, 0);
  memcpy(&host[o_task], &d, sizeof(d));
  memcpy(&host[o_sub], &sb, sizeof(sb));
  const int ints[4] = {0, 0, 0, 0}; // coef_off, queue[0], counter, error
  memcpy(&host[o_ints], ints, sizeof(ints));
  const double atoms[6] = {ra[0], ra[1], ra[2], ra[0] + rab[0], ra[1] + rab[1], ra[2] + rab[2]};
  memcpy(&host[o_atoms], atoms, sizeof(atoms));
  memcpy(&host[o_levels], &levels, sizeof(levels));
  memcpy(&host[o_dhtab], dhtab.data(), dhtab.size() * sizeof(double));
  sph.off = 0;
  memcpy(&host[o_sph], &sph, sizeof(sph));
  if (!tab.empty())
    memcpy(&host[o_tab], tab.data(), tab.size() * sizeof(int16_t));
  cudaStream_t s = (cudaStream_t)stream;
  unsigned char *dev = (unsigned char *)base;
  if (cudaMemcpyAsync(dev, host.data(), host.size(), cudaMemcpyHostToDevice, s) != cudaSuccess)
    return set_error("copy of the task into the static scratch array failed");

  int *ints_d = (int *)(dev + o_ints);
  CoefArgs co{};
  co.tasks = (const TaskDesc *)(dev + o_task);
  co.subs = (const SubblockDesc *)(dev + o_sub);
  co.coef_off = ints_d + 0;
  co.atom_pos = (const double *)(dev + o_atoms);
  co.pab_cart = pab;
  co.coef = dev + o_coef;
  co.ntasks = 1;
  co.func = func;
  co.d = dl;
  co.levels = (const LevelSet *)(dev + o_levels);
  co.dhtab = (const double *)(dev + o_dhtab);
  launch_coefficients(co, ARITH_FP64, coef_w, s);
  if (const char *m = take_launch_error())
    return set_error(m);
  if (cudaGetLastError() != cudaSuccess)
    return set_error("coefficient kernel launch failed");

  GridArgs ga{};
  ga.tasks = (const TaskDesc *)(dev + o_task);
  ga.queue = ints_d + 1;
  ga.nqueue = 1;
  ga.counter = ints_d + 2;
  ga.error = ints_d + 3;
  ga.coef_off = ints_d + 0;
  ga.coef = dev + o_coef;
  ga.sph = (const SphereHdr *)(dev + o_sph);
  ga.sph_tab = (const int16_t *)(dev + o_tab);
  ga.seeds = (const float2 *)(dev + o_seeds);
  ga.grids[0] = grid;
  ga.levels = levels;
  ga.d = dl;
  ga.coef_stride = 1;
  ga.grid_stride = 1;
  launch_collocate(ga, ARITH_FP64, general, bucket_of(lp), extent, 1, s);
  if (const char *m = take_launch_error())
    return set_error(m);
  if (cudaGetLastError() != cudaSuccess)
    return set_error("grid kernel launch failed");
  return 0;
}
