// Single-task collocate / integrate of CP2K's grid API on host buffers:
// grid_cpu_collocate_pgf_product and grid_cpu_integrate_pgf_product
// (src/grid/cpu/grid_cpu_collocate.h, grid_cpu_integrate.h), which CP2K's
// Fortran binds by name (src/grid/grid_api.F:145, 318) for the tasks it
// handles one at a time.  The work runs on the GPU with the task-list
// kernels, one task per call: the task's geometry with the reference's FP64
// expressions on the host (src/grid/ref/grid_ref_collint.h:207-245,
// 583-640, 917-947), the block and the whole grid copied to the device and
// back (the caller's arrays are accumulated into, as the reference does),
// FP64 arithmetic.  Calls are synchronous and serialised by a mutex; the
// device buffers grow to the largest call and are kept until exit.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "gb300_internal.h"
#include "grid_gb300.h"

#define GB300_API extern "C" __attribute__((visibility("default")))

namespace gb300 {
namespace {

[[noreturn]] void pgf_fail(const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  fprintf(stderr, "grid_gb300 error: %s\n", buf);
  abort(); // CP2K's own backends assert (src/grid/grid_task_list.c:131-133)
}
#define CKP(x)                                                                 \
  do {                                                                         \
    cudaError_t e_ = (x);                                                      \
    if (e_ != cudaSuccess)                                                     \
      pgf_fail("%s failed: %s", #x, cudaGetErrorString(e_));                   \
  } while (0)

// device buffers of the single-task calls, grown on demand
struct PgfBuffers {
  std::mutex mu;
  cudaStream_t s = nullptr;
  void *scratch = nullptr; // task, level, sphere table, seeds, counters, coefficients
  size_t scratch_cap = 0;
  double *grid = nullptr;
  size_t grid_cap = 0;
  double *blk = nullptr; // pab, hab, hdab, hadb, a_hdab, forces, virials
  size_t blk_cap = 0;
};
PgfBuffers g_pgf;

template <typename T> void grow(T **p, size_t *cap, size_t bytes) {
  if (*cap >= bytes)
    return;
  if (*p)
    CKP(cudaFree(*p));
  CKP(cudaMalloc((void **)p, bytes));
  *cap = bytes;
}

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// grid_prepare_pab.h / grid_process_vab.h shifts of a collocation
LDiffs collocate_ldiffs(int f) {
  if (f == GRID_FUNC_AB)
    return LDiffs{0, 0, 0, 0};
  if (f >= 411 && f <= 433 && f % 10 >= 1 && f % 10 <= 3)
    return LDiffs{1, -1, 2, -1};
  if ((f >= 701 && f <= 703) || (f >= 801 && f <= 803))
    return LDiffs{2, -2, 2, -2};
  if (f == 200 || (f >= 301 && f <= 303) || (f >= 501 && f <= 503) || (f >= 601 && f <= 603) ||
      (f >= 901 && f <= 906) || (f >= 1001 && f <= 1003))
    return LDiffs{1, -1, 1, -1};
  pgf_fail("unknown grid_func %d", f);
}

// one task's descriptor, level, sphere table and layout in the scratch
struct PgfTask {
  TaskDesc d;
  LevelSet levels;
  SphereHdr sph;
  std::vector<int16_t> tab;
  std::vector<double> dhtab;
  bool general = false;
  int extent = 1;
  bool skip = false;
};

void pgf_task(bool orthorhombic, int border_mask, int la_max, int la_min, int lb_max, int lb_min,
              double zeta, double zetb, double rscale, const double *dh, const double *dh_inv,
              const double *ra, const double *rab, const int *npts_global,
              const int *npts_local, const int *shift_local, const int *border_width,
              double radius, int o1, int o2, PgfTask &p) {
  if (la_max < 0 || lb_max < 0 || la_max > GB300_LMAX || lb_max > GB300_LMAX || la_min < 0 ||
      lb_min < 0 || la_min > la_max || lb_min > lb_max)
    pgf_fail("single task: angular momenta out of range");
  p.levels.nlevels = 1;
  LevelDesc &L = p.levels.lv[0];
  for (int i = 0; i < 3; i++) {
    L.npts_global[i] = npts_global[i];
    L.npts_local[i] = npts_local[i];
    L.shift[i] = shift_local[i];
    L.border_width[i] = border_width[i];
    if (npts_local[i] < 1 || npts_global[i] < 1)
      pgf_fail("single task: empty grid");
  }
  L.dh_max = 0.0;
  for (int i = 0; i < 9; i++) {
    L.dh[i] = dh[i];
    L.dh_inv[i] = dh_inv[i];
    L.dh_max = fmax(L.dh_max, fabs(dh[i]));
  }
  if (2.0 * radius < L.dh_max) { // maps onto no grid point (grid_ref_collint.h:928-937)
    p.skip = true;
    return;
  }
  TaskDesc &d = p.d;
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
  d.prefexp = rscale * exp(-zeta * f * rab2);
  for (int k = 0; k < 3; k++) {
    d.rab[k] = rab[k];
    d.rp[k] = ra[k] + f * rab[k];
  }
  p.general = !(orthorhombic && border_mask == 0);
  if (!p.general) {
    for (int k = 0; k < 3; k++) {
      double s_ = 0.0;
      for (int j = 0; j < 3; j++)
        s_ += L.dh_inv[j * 3 + k] * d.rp[j];
      d.center[k] = (int)floor(s_);
      d.roff[k] = d.rp[k] - ((double)d.center[k]) * L.dh[k * 4];
    }
    const double drmin = fmin(L.dh[0], fmin(L.dh[4], L.dh[8]));
    const double nrad = fmax(1.0, ceil(d.radius / drmin));
    if (nrad > 32767.0)
      pgf_fail("single task: radius spans more than 32767 grid steps");
    long long np = 0;
    build_sphere(L, drmin * nrad, p.sph, p.tab, np);
    for (int k = 0; k < 3; k++)
      if (L.npts_global[k] != L.npts_local[k]) { // grid_ref_collint.h:247-255
        const int off = imod(d.center[k] + p.sph.lb[k] - L.shift[k], L.npts_global[k]) -
                        p.sph.lb[k];
        if (!(off + 1 - p.sph.lb[k] < L.npts_local[k] && off + p.sph.lb[k] >= 0))
          pgf_fail("single task: cube does not fit into the local grid");
      }
    p.extent = 2 * p.sph.cmax + 2;
  } else {
    d.flags |= TF_GENERAL;
    for (int k = 0; k < 3; k++) {
      double gk = 0.0;
      for (int j = 0; j < 3; j++)
        gk += L.dh_inv[j * 3 + k] * d.rp[j];
      d.roff[k] = gk;
      d.center[k] = INT32_MAX;
      d.imax[k] = INT32_MIN;
    }
    for (int a = -1; a <= 1; a++) // the 27 corners (grid_ref_collint.h:624-640)
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
    p.extent = d.imax[1] - d.center[1] + 1;
  }
  build_dh_table(p.levels, p.dhtab);
}

// scratch layout of one task (offsets in bytes)
struct PgfLayout {
  size_t task, sub, ints, atoms, levels, dhtab, sph, tab, seeds, coef, total;
};
PgfLayout pgf_layout(const PgfTask &p, int nco) {
  PgfLayout o{};
  size_t off = 0;
  o.task = off;
  off = align256(off + sizeof(TaskDesc));
  o.sub = off;
  off = align256(off + sizeof(SubblockDesc));
  o.ints = off; // coef_off, queue[0], counter, error
  off = align256(off + 4 * sizeof(int));
  o.atoms = off;
  off = align256(off + 6 * sizeof(double));
  o.levels = off;
  off = align256(off + sizeof(LevelSet));
  o.dhtab = off;
  off = align256(off + p.dhtab.size() * sizeof(double));
  o.sph = off;
  off = align256(off + sizeof(SphereHdr));
  o.tab = off;
  off = align256(off + p.tab.size() * sizeof(int16_t) + 2);
  o.seeds = off;
  off = align256(off + 18 * sizeof(float2));
  o.coef = off;
  off = align256(off + (size_t)nco * sizeof(double));
  o.total = off;
  return o;
}

// the host image of the scratch up to the coefficients
std::vector<unsigned char> pgf_image(const PgfTask &p, const PgfLayout &o, const double *ra,
                                     const double *rab, int n1, int n2) {
  std::vector<unsigned char> host(o.coef, 0);
  memcpy(&host[o.task], &p.d, sizeof(TaskDesc));
  SubblockDesc sb;
  memset(&sb, 0, sizeof(sb));
  sb.ncoa = n1; // the block is [n2][n1]
  sb.ncob = n2;
  sb.ntasks = 1;
  memcpy(&host[o.sub], &sb, sizeof(sb));
  const double atoms[6] = {ra[0], ra[1], ra[2], ra[0] + rab[0], ra[1] + rab[1], ra[2] + rab[2]};
  memcpy(&host[o.atoms], atoms, sizeof(atoms));
  memcpy(&host[o.levels], &p.levels, sizeof(LevelSet));
  if (!p.dhtab.empty())
    memcpy(&host[o.dhtab], p.dhtab.data(), p.dhtab.size() * sizeof(double));
  SphereHdr sph = p.sph;
  sph.off = 0;
  memcpy(&host[o.sph], &sph, sizeof(sph));
  if (!p.tab.empty())
    memcpy(&host[o.tab], p.tab.data(), p.tab.size() * sizeof(int16_t));
  return host;
}

void check_launch() {
  if (const char *m = take_launch_error())
    pgf_fail("single task: %s", m);
  CKP(cudaGetLastError());
}

} // namespace
} // namespace gb300

using namespace gb300;

GB300_API void grid_cpu_collocate_pgf_product(
    const bool orthorhombic, const int border_mask, const enum grid_func func, const int la_max,
    const int la_min, const int lb_max, const int lb_min, const double zeta, const double zetb,
    const double rscale, const double *dh, const double *dh_inv, const double *ra,
    const double *rab, const int *npts_global, const int *npts_local, const int *shift_local,
    const int *border_width, const double radius, const int o1, const int o2, const int n1,
    const int n2, const double *pab, double *grid) {
  const LDiffs dl = collocate_ldiffs(func);
  PgfTask p;
  // the coefficient kernel multiplies by 2 for iatom != jatom
  pgf_task(orthorhombic, border_mask, la_max, la_min, lb_max, lb_min, zeta, zetb, 0.5 * rscale,
           dh, dh_inv, ra, rab, npts_global, npts_local, shift_local, border_width, radius, o1,
           o2, p);
  if (p.skip)
    return;
  const int lp = la_max + dl.la_max + lb_max + dl.lb_max;
  if (bucket_of(lp) < 0)
    pgf_fail("single task: contraction order %d exceeds the supported maximum", lp);
  const int coef_w = (int)coef_words(la_max + dl.la_max, lb_max + dl.lb_max);
  if (!coefficients_fit(coef_w) ||
      !grid_launch_fits(ARITH_FP64, p.general, true, bucket_of(lp), p.extent, 0, 0))
    pgf_fail("single task: too large for the kernels' shared memory");
  const PgfLayout o = pgf_layout(p, ncoset(lp));
  const size_t ngrid = (size_t)npts_local[0] * npts_local[1] * npts_local[2];
  std::lock_guard<std::mutex> lk(g_pgf.mu);
  if (!g_pgf.s)
    CKP(cudaStreamCreateWithFlags(&g_pgf.s, cudaStreamNonBlocking));
  cudaStream_t s = g_pgf.s;
  grow(&g_pgf.scratch, &g_pgf.scratch_cap, o.total);
  grow(&g_pgf.grid, &g_pgf.grid_cap, sizeof(double) * ngrid);
  grow(&g_pgf.blk, &g_pgf.blk_cap, sizeof(double) * (size_t)n1 * n2);
  const std::vector<unsigned char> host = pgf_image(p, o, ra, rab, n1, n2);
  unsigned char *dev = (unsigned char *)g_pgf.scratch;
  CKP(cudaMemcpyAsync(dev, host.data(), host.size(), cudaMemcpyHostToDevice, s));
  CKP(cudaMemcpyAsync(g_pgf.blk, pab, sizeof(double) * (size_t)n1 * n2, cudaMemcpyHostToDevice,
                      s));
  CKP(cudaMemcpyAsync(g_pgf.grid, grid, sizeof(double) * ngrid, cudaMemcpyHostToDevice, s));
  int *ints = (int *)(dev + o.ints);
  CoefArgs co{};
  co.tasks = (const TaskDesc *)(dev + o.task);
  co.subs = (const SubblockDesc *)(dev + o.sub);
  co.coef_off = ints + 0;
  co.atom_pos = (const double *)(dev + o.atoms);
  co.pab_cart = g_pgf.blk;
  co.coef = dev + o.coef;
  co.ntasks = 1;
  co.func = func;
  co.d = dl;
  co.levels = (const LevelSet *)(dev + o.levels);
  co.dhtab = (const double *)(dev + o.dhtab);
  launch_coefficients(co, ARITH_FP64, coef_w, s);
  check_launch();
  GridArgs ga{};
  ga.tasks = co.tasks;
  ga.queue = ints + 1;
  ga.nqueue = 1;
  ga.counter = ints + 2;
  ga.error = ints + 3;
  ga.coef_off = ints + 0;
  ga.coef = dev + o.coef;
  ga.sph = (const SphereHdr *)(dev + o.sph);
  ga.sph_tab = (const int16_t *)(dev + o.tab);
  ga.seeds = (const float2 *)(dev + o.seeds);
  ga.grids[0] = g_pgf.grid;
  ga.levels = p.levels;
  ga.d = dl;
  ga.coef_stride = 1;
  ga.grid_stride = 1;
  launch_collocate(ga, ARITH_FP64, p.general, bucket_of(lp), p.extent, 1, s);
  check_launch();
  CKP(cudaMemcpyAsync(grid, g_pgf.grid, sizeof(double) * ngrid, cudaMemcpyDeviceToHost, s));
  int err = 0;
  CKP(cudaMemcpyAsync(&err, ints + 3, sizeof(int), cudaMemcpyDeviceToHost, s));
  CKP(cudaStreamSynchronize(s));
  if (err)
    pgf_fail("single task: the collocate kernel reported a work item beyond its plan");
}

GB300_API void grid_cpu_integrate_pgf_product(
    const bool orthorhombic, const bool compute_tau, const int border_mask, const int la_max,
    const int la_min, const int lb_max, const int lb_min, const double zeta, const double zetb,
    const double *dh, const double *dh_inv, const double *ra, const double *rab,
    const int *npts_global, const int *npts_local, const int *shift_local,
    const int *border_width, const double radius, const int o1, const int o2, const int n1,
    const int n2, const double *grid, double *hab, const double *pab, double *forces,
    double *virials, double *hdab, double *hadb, double *a_hdab) {
  // grid_ref_integrate.c:56-64
  const bool calc_f = forces != nullptr || hdab != nullptr;
  const bool calc_v = virials != nullptr || a_hdab != nullptr;
  if (calc_v && !calc_f)
    pgf_fail("single task: virials require forces");
  if ((forces || virials) && !pab)
    pgf_fail("single task: forces and virials require pab");
  if (compute_tau && (hdab || hadb || a_hdab))
    pgf_fail("single task: derivative blocks are not available with compute_tau");
  LDiffs dl{0, 0, 0, 0};
  if (calc_f || calc_v) {
    dl.la_max += 1;
    dl.la_min -= 1;
    dl.lb_min -= 1;
  }
  if (calc_v) {
    dl.la_max += 1;
    dl.lb_max += 1;
  }
  if (compute_tau) {
    dl.la_max += 1;
    dl.lb_max += 1;
    dl.la_min -= 1;
    dl.lb_min -= 1;
  }
  PgfTask p;
  pgf_task(orthorhombic, border_mask, la_max, la_min, lb_max, lb_min, zeta, zetb, 1.0, dh,
           dh_inv, ra, rab, npts_global, npts_local, shift_local, border_width, radius, o1, o2,
           p);
  if (p.skip)
    return;
  const int lp = la_max + dl.la_max + lb_max + dl.lb_max;
  if (bucket_of(lp) < 0)
    pgf_fail("single task: contraction order %d exceeds the supported maximum", lp);
  const int words = (int)coef_words(la_max + dl.la_max, lb_max + dl.lb_max);
  if ((size_t)words * 8 > kSmemBudget ||
      !grid_launch_fits(ARITH_FP64, p.general, false, bucket_of(lp), p.extent, 0, 0))
    pgf_fail("single task: too large for the kernels' shared memory");
  const PgfLayout o = pgf_layout(p, ncoset(lp));
  const size_t ngrid = (size_t)npts_local[0] * npts_local[1] * npts_local[2];
  const size_t nblk = (size_t)n1 * n2;
  // device block area: pab, hab, hdab, hadb, a_hdab, forces (6), virials (18)
  const size_t o_pab = 0, o_hab = nblk, o_hd = 2 * nblk, o_ha = 5 * nblk, o_ahd = 8 * nblk,
               o_f = 17 * nblk, o_v = o_f + 6, n_all = o_v + 18;
  std::lock_guard<std::mutex> lk(g_pgf.mu);
  if (!g_pgf.s)
    CKP(cudaStreamCreateWithFlags(&g_pgf.s, cudaStreamNonBlocking));
  cudaStream_t s = g_pgf.s;
  grow(&g_pgf.scratch, &g_pgf.scratch_cap, o.total);
  grow(&g_pgf.grid, &g_pgf.grid_cap, sizeof(double) * ngrid);
  grow(&g_pgf.blk, &g_pgf.blk_cap, sizeof(double) * n_all);
  const std::vector<unsigned char> host = pgf_image(p, o, ra, rab, n1, n2);
  unsigned char *dev = (unsigned char *)g_pgf.scratch;
  double *blk = g_pgf.blk;
  CKP(cudaMemcpyAsync(dev, host.data(), host.size(), cudaMemcpyHostToDevice, s));
  CKP(cudaMemcpyAsync(g_pgf.grid, grid, sizeof(double) * ngrid, cudaMemcpyHostToDevice, s));
  // the outputs are accumulated into: the caller's values go in first
  auto in = [&](size_t off, const double *h, size_t n) {
    if (h)
      CKP(cudaMemcpyAsync(blk + off, h, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  };
  in(o_pab, pab, nblk);
  in(o_hab, hab, nblk);
  in(o_hd, hdab, 3 * nblk);
  in(o_ha, hadb, 3 * nblk);
  in(o_ahd, a_hdab, 9 * nblk);
  in(o_f, forces, 6);
  in(o_v, virials, 18);
  int *ints = (int *)(dev + o.ints);
  GridArgs ga{};
  ga.tasks = (const TaskDesc *)(dev + o.task);
  ga.queue = ints + 1;
  ga.nqueue = 1;
  ga.counter = ints + 2;
  ga.error = ints + 3;
  ga.coef_off = ints + 0;
  ga.coef_out = (double *)(dev + o.coef);
  ga.sph = (const SphereHdr *)(dev + o.sph);
  ga.sph_tab = (const int16_t *)(dev + o.tab);
  ga.seeds = (const float2 *)(dev + o.seeds);
  ga.grids_in[0] = g_pgf.grid;
  ga.levels = p.levels;
  ga.d = dl;
  ga.coef_stride = 1;
  ga.grid_stride = 1;
  launch_integrate(ga, ARITH_FP64, p.general, bucket_of(lp), p.extent, 1, s);
  check_launch();
  PgfPostArgs pa{};
  pa.task = ga.tasks;
  pa.atom_pos = (const double *)(dev + o.atoms);
  pa.coef = (const double *)(dev + o.coef);
  pa.dhtab = (const double *)(dev + o.dhtab);
  pa.d = dl;
  pa.compute_tau = compute_tau ? 1 : 0;
  pa.n1 = n1;
  pa.pab = pab ? blk + o_pab : nullptr;
  pa.hab = blk + o_hab;
  pa.forces = forces ? blk + o_f : nullptr;
  pa.virials = virials ? blk + o_v : nullptr;
  pa.hdab = hdab ? blk + o_hd : nullptr;
  pa.hadb = hadb ? blk + o_ha : nullptr;
  pa.a_hdab = a_hdab ? blk + o_ahd : nullptr;
  pa.words = words;
  launch_pgf_post(pa, s);
  check_launch();
  auto out = [&](size_t off, double *h, size_t n) {
    if (h)
      CKP(cudaMemcpyAsync(h, blk + off, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  };
  out(o_hab, hab, nblk);
  out(o_hd, hdab, 3 * nblk);
  out(o_ha, hadb, 3 * nblk);
  out(o_ahd, a_hdab, 9 * nblk);
  out(o_f, forces, 6);
  out(o_v, virials, 18);
  int err = 0;
  CKP(cudaMemcpyAsync(&err, ints + 3, sizeof(int), cudaMemcpyDeviceToHost, s));
  CKP(cudaStreamSynchronize(s));
  if (err)
    pgf_fail("single task: the integrate kernel reported a work item beyond its plan");
}
