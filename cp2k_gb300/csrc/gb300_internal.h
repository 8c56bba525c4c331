// Internal definitions shared by the GB300 grid backend's translation units.
//
// Data layout in HBM (one task list):
//   TaskDesc[ntasks]      geometry + indices of every task, sorted by
//                         (block, iset, jset, level) so the per-subblock
//                         kernels walk contiguous runs; 176 B per task.
//   SubblockDesc[nsub]    one per (block, iset, jset): offsets into the
//                         spherical pab/hab buffer and the Cartesian scratch.
//   sphere tables         int16 row bounds per (level, discretised radius),
//                         built on the host with the reference's FP64
//                         expressions (src/grid/ref/grid_ref_collint.h:
//                         139-151, 44-52, 237-245).
//   queues                per (path, lp bucket) the task order taken by the
//                         persistent grid kernels.
//   coefficients          per task the C_xyz (ortho) or C_ijk (general)
//                         polynomial, compact: lz outer, ly, lx inner.
#pragma once

#include <cstddef>
#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

#define GB300_MAX_LEVELS 8
#define GB300_LMAX 8    // largest l of a set this backend accepts
#define GB300_LP_MAX 16 // la + lb after every angular-momentum shift

namespace gb300 {

// arithmetic of the per-point work (values of enum grid_gb300_precision)
enum Arith : int { ARITH_FP64 = 0, ARITH_MIXED = 1, ARITH_FP32 = 2 };

enum TaskFlags : uint8_t {
  TF_SKIP = 1,    // 2*radius < dh_max: maps onto no grid point
  TF_GENERAL = 2, // non-orthorhombic cell or border_mask != 0
};

struct __align__(16) TaskDesc {
  double rp[3];       // Gaussian product centre
  double zetp;        // zeta + zetb
  double zeta, zetb;  //
  double prefexp;     // exp(-zeta*zetb/zetp*|rab|^2)  (rscale applied later)
  double radius;      //
  double roff[3];     // ortho: rp - centre*dh ; general: gp = dh_inv^T rp
  double rab[3];      //
  int center[3];      // ortho: cube centre ; general: index_min
  int imax[3];        // general: index_max
  int level;          // 0-based
  int sphere;         // ortho: sphere-table index
  int subblock;       // SubblockDesc index
  int iatom, jatom;   // 0-based
  int orig;           // position in the caller's list
  int16_t o1, o2;     // first Cartesian index of ipgf / jpgf in the subblock
  int8_t la_max, la_min, lb_max, lb_min;
  uint8_t flags;
  uint8_t border_mask;
  uint8_t pad_[6];
};
static_assert(sizeof(TaskDesc) == 176, "TaskDesc layout");

struct SubblockDesc {
  int block_offset;  // spherical block in pab/hab buffers
  int cart_offset;   // Cartesian pab/hab scratch
  int ncoa, ncob;    // Cartesian sizes (npgf * ncoset(lmax))
  int nsgf_seta, nsgf_setb;
  int sgfa, sgfb;    // first spherical function of the set (0-based)
  int nsgfa, nsgfb;  // spherical size of the whole atom basis
  int maxcoa, maxcob;
  int sphia, sphib;  // offsets of sphi rows sgfa / sgfb in the device sphi
  int transpose;     // iatom <= jatom: block stored [sgfb][sgfa]
  int identity;      // both contractions are identities (copy instead of gemm)
  int iatom, jatom;
  int first_task, ntasks;
};

struct SphereHdr {
  int lb[3];
  int cmax;
  int off; // into the int16 table: [K] jstart, [K] row offsets, istart rows
  int jxo; // relative offset of the [K][1-lb[0]] table of last row index per x
  int plo; // point lists: index of this sphere's plane offsets in sph_ploff (-1: none)
  // integrate lane plan for cubes up to 32 wide (0: none): x-chunk width sw
  // (bits 0-5), number of chunks nc (bits 6-8), row groups per chunk n[c]
  // (5 bits each from bit 9)
  int iplan;
};

struct LevelDesc {
  int npts_global[3];
  int npts_local[3];
  int shift[3];
  int border_width[3];
  double dh[9];
  double dh_inv[9];
  double dh_max;
};

struct LevelSet {
  int nlevels;
  LevelDesc lv[GB300_MAX_LEVELS];
};

// l-range changes of the collocated / integrated C_ab relative to the basis
struct LDiffs {
  int la_max, la_min, lb_max, lb_min;
};

__host__ __device__ constexpr int ncoset(int l) {
  return l < 0 ? 0 : (l + 1) * (l + 2) * (l + 3) / 6;
}
__host__ __device__ inline int coset(int lx, int ly, int lz) {
  const int l = lx + ly + lz;
  return l == 0 ? 0 : ncoset(l - 1) + ((l - lx) * (l - lx + 1)) / 2 + lz;
}
// number of (a, b) with a + b <= m
__host__ __device__ constexpr int ntri(int m) { return m < 0 ? 0 : (m + 1) * (m + 2) / 2; }
// compact index of x^lx y^ly z^lz in a polynomial of degree <= lp
__host__ __device__ inline int cidx(int lz, int ly, int lx, int lp) {
  const int m = lp - lz;
  return ncoset(lp) - ncoset(m) + ly * (m + 1) - (ly * (ly - 1)) / 2 + lx;
}
__host__ __device__ inline int imod(int a, int m) { return ((a % m) + m) % m; }
// inverse of cidx
__host__ __device__ inline void decode_cidx(int e, int lp, int &lz, int &ly, int &lx) {
  lz = 0;
  int rem = e;
  while (rem >= ntri(lp - lz)) {
    rem -= ntri(lp - lz);
    lz++;
  }
  const int m = lp - lz;
  ly = 0;
  while (rem > m - ly) {
    rem -= m - ly + 1;
    ly++;
  }
  lx = rem;
}

// -------------------------------------------------------------------------
// kernel entry points (launch wrappers), implemented in the .cu files
// -------------------------------------------------------------------------
struct CoefArgs {
  const TaskDesc *tasks;
  const SubblockDesc *subs;
  const int *coef_off;  // per task offset into the coefficient buffer
  const double *atom_pos;
  const double *pab_cart; // Cartesian pab scratch (FP64)
  void *coef;             // T*
  int ntasks;
  int func;
  LDiffs d;
  const LevelSet *levels; // device copy
  const double *dhtab;     // general-path transform table (build_dh_table), FP64
  const float *dhtab_f;    // the same in FP32 (FP32 kernels)
  const float2 *dhtab_df;  // the same as double-float pairs (mixed kernels)
  const int *order;        // if set, only these tasks (norder of them)
  int norder;
  int transform;           // C_ab -> C_xyz: see uses_staged()
};

struct GridArgs {
  const TaskDesc *tasks;
  const int *queue;
  const int2 *items;      // general path: (task, first plane | planes << 16), or null
  int iwidth;             // general path: widest box of the queue in i
  int nqueue;             // tasks, or work items when items is set
  int *counter;           // work counter, zeroed before launch
  const int *coef_off;
  const void *coef;       // T* (collocate) ; double* out (integrate)
  void *coef_out;
  const SphereHdr *sph;
  const int16_t *sph_tab;
  const int *sph_pts;   // packed (x, j) of every point of a sphere plane, row-major
  const int *sph_ploff; // per sphere plane kk: start of its points in sph_pts
  double *grids[GB300_MAX_LEVELS];         // collocate targets
  float *grids_lo[GB300_MAX_LEVELS];       // collocate low words (mixed path)
  const void *grids_in[GB300_MAX_LEVELS];  // integrate sources (per arith)
  LevelSet levels;
  LDiffs d;
  int coef_stride;   // FP32 kernels: floats per stored coefficient (2: dfloat buffer)
  int grid_stride;   // FP32 integrate: floats per grid point (2: hi/lo pairs)
  int nwarps_total;
  const float2 *seeds;    // mixed path: per task [3][6] dfloat recurrence seeds
  long long *task_cycles; // optional per-task timings (clock64)
  int *error;             // device error word
  // mixed mode, orthorhombic tasks split by rows: per task the squared radius
  // (bohr^2) of the cylinder around the Gaussian's x axis whose rows (j, k)
  // run in double-float; the rows outside run in FP32 in a shell queue.
  // kCoreAll: every row is inside; negative: none is.  Null with core_side 0.
  const float *core_r2;
  int core_side; // 0: every row of the task; 1: rows inside; 2: rows outside
  int accum;     // integrate: add into the (zeroed) coefficient buffer
};

constexpr float kCoreAll = 3.0e38f;

#ifdef __CUDACC__
// Rows j of cube plane k inside the cylinder y^2 + z^2 <= r2 around the
// Gaussian product's x axis (y = j dh_y - roff_y, z = k dh_z - roff_z):
// [lo, hi], empty when lo > hi.  Every kernel that runs one side of a split
// task calls this function; it uses round-to-nearest FP32 operations only
// (no contraction), so the double-float and the FP32 side agree on every row.
__device__ __forceinline__ void core_rows(float r2, const TaskDesc &d, const LevelDesc &L, int k,
                                          int &lo, int &hi) {
  if (r2 >= kCoreAll) {
    lo = -(1 << 20);
    hi = 1 << 20;
    return;
  }
  const float z = __fsub_rn(__fmul_rn((float)k, (float)L.dh[8]), (float)d.roff[2]);
  const float rem = __fsub_rn(r2, __fmul_rn(z, z));
  if (!(rem >= 0.f)) {
    lo = 1;
    hi = 0;
    return;
  }
  const float s = __fsqrt_rn(rem), ry = (float)d.roff[1], iy = (float)L.dh_inv[4];
  lo = (int)ceilf(__fmul_rn(__fsub_rn(ry, s), iy));
  hi = (int)floorf(__fmul_rn(__fadd_rn(ry, s), iy));
}
#endif

struct PostArgs {
  const TaskDesc *tasks;
  const SubblockDesc *subs;
  const int *coef_off;
  const double *coef;     // integrated C_xyz / C_ijk (FP64)
  const double *pab_cart; // for forces / virial
  double *hab_cart;       // accumulated Cartesian hab scratch
  const double *atom_pos;
  double *forces;         // [natoms][3] or null
  double *virial;         // [9] or null
  int ntasks;
  int compute_tau;
  LDiffs d;
  const LevelSet *levels;
  const double *dhtab;     // general-path transform table (build_dh_table), FP64
  const float *dhtab_f;    // the same in FP32
  const float2 *dhtab_df;  // the same as double-float pairs
  const int *order;        // if set, only these tasks (norder of them)
  int norder;
  int transform;           // C_xyz -> C_ab: see uses_staged()
};

// single-task integrate (grid_cpu_integrate_pgf_product): one task's post
// processing, every output accumulated (FP64; all pointers device memory)
struct PgfPostArgs {
  const TaskDesc *task;
  const double *atom_pos; // ra[3]
  const double *coef;     // integrated C_xyz (C_ijk on the general path)
  const double *dhtab;    // general-path transform table
  LDiffs d;               // the integrate shifts
  int compute_tau;
  int n1;                 // leading dimension of the [n2][n1] blocks
  const double *pab;      // or null
  double *hab;
  double *forces;         // [2][3] or null
  double *virials;        // [2][3][3] or null
  double *hdab, *hadb;    // [n2][n1][3] or null
  double *a_hdab;         // [n2][n1][3][3] or null
  int words;              // shared-memory doubles (coef_words)
};
void launch_pgf_post(const PgfPostArgs &a, cudaStream_t s);

struct ContractArgs {
  const SubblockDesc *subs;
  int nsubs;
  const double *sphi;
  const double *blocks; // spherical pab (decontract) ; hab out (contract)
  double *blocks_out;
  double *cart;         // Cartesian scratch
  int words;            // per-warp shared-memory doubles (largest work array)
};
// Per-group shared memory of the coefficient / post kernels in 8-byte words:
// cab [n2][n1] (FP64, then the working type in place), alpha, cxyz, cijk.
__host__ __device__ inline size_t coef_smem_words(int n1, int n2, int la, int lb, int lp) {
  return (size_t)n1 * n2 + 3 * (size_t)(la + 1) * (lb + 1) * (lp + 1) +
         2 * (size_t)ncoset(lp) + 8;
}
// the staged transforms' T1 and T2, after those
__host__ __device__ inline size_t staged_words(int la, int lb, int lp) {
  return (size_t)ntri(la) * ntri(lb) * (lp + 1) + (size_t)(la + 1) * (lb + 1) * ntri(lp);
}
// C_ab <-> C_xyz transform of a task with (shifted) angular momenta la, lb
// in the coefficient kernel (forward) or the post kernel (adjoint): the
// staged per-direction contractions (true) or the direct gather.
// variant 0: direct, 1: staged, -1: staged forward where la or lb >= 3 and
// direct in the adjoint (whose outputs, the C_ab entries, each gather only
// their own non-zero terms); staged only where its scratch fits one CTA's
// shared memory (200 KB).
__host__ __device__ inline bool uses_staged(int variant, int la, int lb, bool forward) {
  const int lp = la + lb;
  if (coef_smem_words(ncoset(la), ncoset(lb), la, lb, lp) + staged_words(la, lb, lp) >
      (size_t)(200 * 1024 / 8))
    return false;
  return variant == 1 || (variant < 0 && forward && (la >= 3 || lb >= 3));
}
// per-group shared-memory words of the coefficient / post kernels for a task
size_t coef_words(int la, int lb, bool staged = false);

void launch_decontract(const ContractArgs &a, cudaStream_t s);
void launch_contract_hab(const ContractArgs &a, cudaStream_t s);
// mixed mode, one work queue at a time: the queue's tasks (a.order) in the
// working type of their class, `work` = ARITH_FP32 (float), ARITH_MIXED
// (double-float) or ARITH_FP64 (general-path tasks); coefficients are stored
// as double-float pairs, general-path ones in FP64
void launch_coefficients_mixed(const CoefArgs &a, int work, int max_smem_words, cudaStream_t s);
void launch_post_mixed(const PostArgs &a, int work, int max_smem_words, cudaStream_t s);
void launch_coefficients(const CoefArgs &a, int arith, int max_smem_words,
                         cudaStream_t s);
// `extent` is the largest cube width (2*cmax+2) of the queue for the
// orthorhombic kernels and the largest j-range of the box for the general ones;
// it sizes the per-warp shared memory (4 warps per CTA).
// Launch shape of a persistent grid kernel: inputs (0 = automatic) and, on
// return, the shape used.
struct LaunchCfg {
  int warps = 0;  // warps per CTA (capped by the shared-memory budget)
  int blocks = 0; // CTAs (automatic: all that fit on the GPU at once)
  int occupancy = 100; // automatic CTA count: this percentage of all that fit
  int variant = 0;     // collocate, orthorhombic: 0 row walk, 1 point list
  int tensor = 0;      // integrate, orthorhombic, FP32, lp <= 6: tensor-core kernel
  int tensor_coll = 0; // collocate, orthorhombic, FP32, lp <= 6: tensor-core kernel
};
inline int cfg_blocks(const LaunchCfg &c, int persistent) {
  if (c.blocks > 0)
    return c.blocks;
  const int nb = persistent * (c.occupancy > 0 ? c.occupancy : 100) / 100;
  return nb > 0 ? nb : 1;
}
void launch_collocate(const GridArgs &a, int arith, bool general, int bucket,
                      int extent, LaunchCfg &cfg, cudaStream_t s);
void launch_integrate(const GridArgs &a, int arith, bool general, int bucket,
                      int extent, LaunchCfg &cfg, cudaStream_t s);
inline void launch_collocate(const GridArgs &a, int arith, bool general, int bucket,
                             int extent, int nblocks, cudaStream_t s) {
  LaunchCfg c;
  c.blocks = nblocks;
  launch_collocate(a, arith, general, bucket, extent, c, s);
}
inline void launch_integrate(const GridArgs &a, int arith, bool general, int bucket,
                             int extent, int nblocks, cudaStream_t s) {
  LaunchCfg c;
  c.blocks = nblocks;
  launch_integrate(a, arith, general, bucket, extent, c, s);
}
// Host-side checks that a launch of the grid kernels (`iwidth`: the general
// point-list kernel's box width) or of the coefficient kernel fits the
// shared-memory budget; the launch wrappers refuse what does not fit through
// launch_error().
bool grid_launch_fits(int arith, bool general, bool collocate, int bucket, int extent,
                      int variant, int iwidth);
bool general_launch_fits(int arith, bool collocate, int lpb, int njmax, int variant,
                         int iwidth);
bool coefficients_fit(int words_per_group);
// general path: FP64 for ARITH_FP64 and ARITH_MIXED, FP32 for ARITH_FP32
void launch_collocate_general_impl(const GridArgs &a, int arith, int lpb,
                                   int njmax, LaunchCfg &cfg, cudaStream_t s);
void launch_integrate_general_impl(const GridArgs &a, int arith, int lpb,
                                   int njmax, LaunchCfg &cfg, cudaStream_t s);
constexpr int kWarpsPerCta = 4;
constexpr size_t kSmemBudget = 200 * 1024; // dynamic shared memory per CTA
// warps per CTA so that per-warp regions fit the budget (0: does not fit)
inline int warps_for(size_t per_warp) {
  int w = (int)(kSmemBudget / (per_warp ? per_warp : 1));
  return w > kWarpsPerCta ? kWarpsPerCta : w;
}
void launch_post(const PostArgs &a, int arith, int max_smem_words,
                 cudaStream_t s);
// V grid -> float (ARITH_FP32) or float2 hi/lo pairs (ARITH_MIXED)
void launch_grid_split(const double *src, void *dst, size_t n, int arith,
                       cudaStream_t s, float *hi = nullptr);
// g += (double)lo
void launch_grid_fold_lo(double *g, const float *lo, size_t n, cudaStream_t s);

// lp bucket limits of the templated grid kernels
constexpr int kNumBuckets = 5;
constexpr int kBucketLp[kNumBuckets] = {4, 6, 9, 12, 16};
inline int bucket_of(int lp) {
  for (int b = 0; b < kNumBuckets; b++)
    if (lp <= kBucketLp[b])
      return b;
  return -1;
}

// Sphere bounds of one (level, discretised radius) appended to `tab`
// (api.cu); npoints receives the number of grid points the cube visits.
void build_sphere(const LevelDesc &L, double disr, SphereHdr &h,
                  std::vector<int16_t> &tab, long long &npoints);

// Point lists of a sphere (for the point-list collocate kernel): the points
// (x, j) of every plane kk in row-major order (j, then x), packed as
// (x & 0xffff) | (j << 16), appended to `pts`; the K + 1 plane offsets go to
// `ploff` and h.plo receives their index.
void build_sphere_points(SphereHdr &h, const std::vector<int16_t> &tab, std::vector<int> &pts,
                         std::vector<int> &ploff);

// Table for the general path's C_xyz <-> C_ijk transform: per level the
// pivoted factorisation M = P^T L D U of M[c][d] = dh[d][c] as kLatTab
// values: pi(0..2), L10, L20, L21, D0, D1, D2, U02, U12, U01
constexpr int kLatTab = 12;
#ifdef __CUDACC__
// one work item of a grid launch: a task, or a range of its planes (k0 planes
// past the first, nk of them)
struct WorkItem {
  int t, k0, nk;
};
__device__ __forceinline__ WorkItem work_item(const GridArgs &a, int qi) {
  if (a.items) {
    const int2 it = a.items[qi];
    return WorkItem{it.x, it.y & 0xffff, it.y >> 16};
  }
  return WorkItem{a.queue[qi], 0, 1 << 20};
}
#endif

// splitting of large general-path boxes into plane ranges (work items)
constexpr long long kSlicePoints = 16384;
constexpr int kSlicePlanes = 4;
// orthorhombic tasks: split past twice the queue's share per resident warp
constexpr double kNominalWarps = 152.0 * 16.0;
constexpr long long kOrthoSliceMin = 4096;
inline size_t dh_table_size(int nlevels) { return (size_t)nlevels * kLatTab; }
void build_dh_table(const LevelSet &ls, std::vector<double> &tab);

// counts launches for grid_gb300_kernel_launches()
void count_launch(int n = 1);
// records a launch-configuration error; the host call fails after the launch
// sequence (reported like a device error)
void launch_error(const char *msg);
// returns and clears the message recorded by launch_error (nullptr if none)
const char *take_launch_error();

// learned cost model (mlp_kernels.cu)
int mlp_nparams();
int mlp_tiles(int n);
void launch_mlp_loss_grad(const float *P, const float *X, const float *T, int n, float *loss,
                          float *grad, float *work, cudaStream_t s);
void launch_mlp_adam(float *P, const float *grad, float *m, float *v, int step, float lr,
                     float beta1, float beta2, float eps, cudaStream_t s);
void launch_mlp_predict(const float *P, const float *X, int n, const float *norm, float *Y,
                        cudaStream_t s);

// raises a kernel's dynamic shared-memory limit to at least smem (cached)
void set_smem(const void *kernel, size_t smem);

// persistent grid size: CTAs that fit on all SMs at once for this kernel
int persistent_blocks(const void *kernel, int threads, size_t smem);

} // namespace gb300
