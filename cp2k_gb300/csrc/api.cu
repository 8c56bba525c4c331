// Host side of the GB300 grid backend: the C ABI of include/grid_gb300.h.
//
// Task-list creation does, once per geometry and in FP64 on the host, what
// CP2K's reference computes per task inside its loops (the Gaussian product
// centre and prefactor, the cube centre, the discretised radius and its
// sphere bounds, the general-path index box: src/grid/ref/grid_ref_collint.h:
// 207-245, 583-640, 917-947), sorts the tasks into per-subblock runs and into
// cost-ordered work queues, and uploads everything into device-resident
// arrays.  Collocate / integrate calls then only move pab/hab/grids and
// launch kernels.  Host code is compiled with -ffp-contract=off so the
// discrete decisions (floor/ceil of FP64 expressions) match the reference's
// ISO-C build bit for bit on x86-64 and aarch64.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <thread>
#include <array>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <numeric>
#include <string>
#include <tuple>
#include <vector>

#include "gb300_internal.h"
#include "grid_gb300.h"

#define GB300_API extern "C" __attribute__((visibility("default")))

namespace gb300 {

static std::atomic<long long> g_launches{0};
void count_launch(int n) { g_launches += n; }
static std::atomic<const char *> g_launch_error{nullptr};
void launch_error(const char *msg) { g_launch_error = msg; }
const char *take_launch_error() { return g_launch_error.exchange(nullptr); }

static std::mutex g_err_mu;
static char g_last_error[512] = "";

[[noreturn]] static void fail(const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  {
    std::lock_guard<std::mutex> lk(g_err_mu);
    snprintf(g_last_error, sizeof(g_last_error), "%s", buf);
  }
  fprintf(stderr, "grid_gb300 error: %s\n", buf);
  abort();
}

#define CK(x)                                                                  \
  do {                                                                         \
    cudaError_t e_ = (x);                                                      \
    if (e_ != cudaSuccess)                                                     \
      fail("%s failed: %s (%s:%d)", #x, cudaGetErrorString(e_), __FILE__,     \
           __LINE__);                                                          \
  } while (0)

void set_smem(const void *kernel, size_t smem) {
  static std::mutex mu;
  static std::map<std::pair<int, const void *>, size_t> done;
  int dev = 0;
  CK(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(mu);
  size_t &cur = done[std::make_pair(dev, kernel)];
  if (smem > cur) { // the attribute call is slow; make it once per size increase
    CK(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    cur = smem;
  }
}

int persistent_blocks(const void *kernel, int threads, size_t smem) {
  static std::mutex mu;
  static std::map<std::pair<const void *, size_t>, int> cache;
  std::lock_guard<std::mutex> lk(mu);
  auto key = std::make_pair(kernel, smem);
  auto it = cache.find(key);
  if (it != cache.end())
    return it->second;
  int dev = 0, nsm = 0, per_sm = 0;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem));
  if (per_sm < 1)
    fail("kernel does not fit on an SM (%zu B shared memory)", smem);
  const int nb = nsm * per_sm;
  cache[key] = nb;
  return nb;
}

} // namespace gb300

using namespace gb300;

// ===========================================================================
// offload buffers (src/offload/offload_buffer.c)
// ===========================================================================
GB300_API void offload_create_buffer(const int length, offload_buffer **buffer) {
  const size_t bytes = (size_t)(length > 0 ? length : 1) * sizeof(double);
  offload_buffer *b = *buffer;
  if (b != nullptr) {
    if (b->size >= (size_t)length * sizeof(double)) {
      b->size = (size_t)length * sizeof(double);
      return; // reuse, as the reference does
    }
    offload_free_buffer(b);
  }
  b = (offload_buffer *)malloc(sizeof(offload_buffer));
  if (!b)
    fail("out of host memory");
  b->size = (size_t)length * sizeof(double);
  CK(cudaMallocHost((void **)&b->host_buffer, bytes));
  CK(cudaMalloc((void **)&b->device_buffer, bytes));
  *buffer = b;
}

GB300_API void offload_free_buffer(offload_buffer *buffer) {
  if (!buffer)
    return;
  CK(cudaFreeHost(buffer->host_buffer));
  CK(cudaFree(buffer->device_buffer));
  free(buffer);
}

GB300_API double *offload_get_buffer_host_pointer(offload_buffer *buffer) {
  return buffer ? buffer->host_buffer : nullptr;
}

// ===========================================================================
// basis sets (src/grid/common/grid_basis_set.c:19-86)
// ===========================================================================
GB300_API void grid_create_basis_set(const int nset, const int nsgf, const int maxco,
                                     const int maxpgf, const int *lmin, const int *lmax,
                                     const int *npgf, const int *nsgf_set,
                                     const int *first_sgf, const double *sphi,
                                     const double *zet, grid_basis_set **basis_set) {
  grid_basis_set *b = (grid_basis_set *)malloc(sizeof(grid_basis_set));
  if (!b)
    fail("out of host memory");
  b->nset = nset;
  b->nsgf = nsgf;
  b->maxco = maxco;
  b->maxpgf = maxpgf;
  auto dup_i = [&](const int *src) {
    int *p = (int *)malloc(sizeof(int) * (nset > 0 ? nset : 1));
    if (nset > 0)
      memcpy(p, src, sizeof(int) * nset);
    return p;
  };
  b->lmin = dup_i(lmin);
  b->lmax = dup_i(lmax);
  b->npgf = dup_i(npgf);
  b->nsgf_set = dup_i(nsgf_set);
  b->first_sgf = dup_i(first_sgf);
  const size_t ns = (size_t)nsgf * maxco, nz = (size_t)nset * maxpgf;
  b->sphi = (double *)malloc(sizeof(double) * (ns ? ns : 1));
  b->zet = (double *)malloc(sizeof(double) * (nz ? nz : 1));
  if (ns)
    memcpy(b->sphi, sphi, sizeof(double) * ns);
  if (nz)
    memcpy(b->zet, zet, sizeof(double) * nz);
  for (int i = 0; i < nset; i++)
    if (b->lmax[i] > GB300_LMAX || b->lmin[i] < 0 || b->lmin[i] > b->lmax[i])
      fail("basis set: unsupported angular momentum range [%d, %d]", b->lmin[i], b->lmax[i]);
  *basis_set = b;
}

GB300_API void grid_free_basis_set(grid_basis_set *b) {
  if (!b)
    return;
  free(b->lmin);
  free(b->lmax);
  free(b->npgf);
  free(b->nsgf_set);
  free(b->first_sgf);
  free(b->sphi);
  free(b->zet);
  free(b);
}

// ===========================================================================
// library config (src/grid/common/grid_library.c)
// ===========================================================================
static grid_library_config g_config = {GRID_BACKEND_AUTO, false, false};
static long long g_counters[2][4][GB300_LP_MAX + 1];
static bool g_initialized = false;

GB300_API void grid_library_init(void) {
  if (g_initialized)
    return;
  memset(g_counters, 0, sizeof(g_counters));
  g_initialized = true;
}

GB300_API void grid_library_finalize(void) { g_initialized = false; }

GB300_API void grid_library_set_config(const enum grid_backend backend, const bool validate,
                                       const bool apply_cutoff) {
  g_config.backend = backend;
  g_config.validate = validate;
  g_config.apply_cutoff = apply_cutoff;
}

GB300_API grid_library_config grid_library_get_config(void) { return g_config; }

GB300_API void grid_library_counter_add(const int lp, const enum grid_backend backend,
                                        const enum grid_library_kernel kernel,
                                        const int increment) {
  (void)backend;
  if (lp < 0 || lp > GB300_LP_MAX || kernel < 0 || kernel > 3)
    return;
  __atomic_fetch_add(&g_counters[0][kernel][lp], (long long)increment, __ATOMIC_RELAXED);
}

GB300_API void grid_library_print_stats(const int fortran_comm,
                                        void (*print_func)(const char *, int, int),
                                        const int output_unit) {
  (void)fortran_comm;
  static const char *names[4] = {"collocate ortho", "integrate ortho", "collocate general",
                                 "integrate general"};
  char line[160];
  snprintf(line, sizeof(line), "\n %-26s %6s %16s\n", "GB300 GRID KERNEL", "LP", "COUNT");
  print_func(line, (int)strlen(line), output_unit);
  for (int k = 0; k < 4; k++)
    for (int lp = 0; lp <= GB300_LP_MAX; lp++)
      if (g_counters[0][k][lp]) {
        snprintf(line, sizeof(line), " %-26s %6d %16lld\n", names[k], lp, g_counters[0][k][lp]);
        print_func(line, (int)strlen(line), output_unit);
      }
}

GB300_API long long grid_gb300_kernel_launches(void) { return g_launches.load(); }

GB300_API const char *grid_gb300_last_error(void) { return g_last_error; }

// ===========================================================================
// task lists
// ===========================================================================
namespace gb300 {

// Copy chunks of the host-buffer calls: subblock ranges in block order,
// chunk c holding subblocks [sub_lo[c], sub_lo[c+1]) and the block-buffer
// elements [el_lo[c], el_lo[c+1]) (which partition the buffer).
struct CopyChunks {
  int n = 1;
  std::vector<int> sub_lo;
  std::vector<long long> el_lo;
};
constexpr int kMaxQueues = 256;          // queue launches per call (work counters)
constexpr int kQueueKeys = 2 * kNumBuckets * 2 * 2; // (general, bucket, class, size)

struct Queue {
  int *d_idx = nullptr;
  int n = 0;
  // general path: grid work items (task, first plane | planes << 16), large
  // boxes split by planes over several warps; null when no task is split
  int2 *d_items = nullptr;
  int nitems = 0;
  int iwidth = 0; // general path: widest box in i
  int extent = 0; // ortho: max cube width; general: max j-range
  int general = 0, bucket = 0;
  int fp32 = 0; // mixed path: this queue runs in plain FP32
  int side = 0; // row split: 0 whole tasks, 1 rows inside the cylinder, 2 rows outside
  int key = 0;          // (general, bucket, FP32 class, size class)
  int base = 0;         // key of the tuned launch shapes
  int chunk = 0;        // host-buffer calls: the copy chunk whose tasks it holds
  long long points = 0; // grid points the queue's tasks visit
  double flops = 0.0;   // 2 (lp+1) points summed over the tasks
};

// per-launch CUDA-event timing of the grid kernels (opt-in)
struct LaunchRecord {
  grid_gb300_launch_info info;
  int key = 0;
  cudaEvent_t a = nullptr, b = nullptr;
};

// cube widths up to this share one work queue; wider cubes get their own so
// that the common small cubes run with small per-warp tables (more warps);
// the autotuner may move the split per task list
constexpr int kSmallExtent = 34;

struct Mode { // everything that depends on the l shifts of a call
  LDiffs d;
  std::vector<int> coef_off; // per task (block order)
  int *d_coef_off = nullptr;
  size_t coef_total = 0;
  std::vector<Queue> queues; // launch order
  int *d_qidx = nullptr;     // every queue's task indices (queues point into it)
  int2 *d_qitems = nullptr;  // every split queue's work items
  // what the queues depend on: l shifts, precision, derivative factor, copy
  // chunks (not the phase)
  std::tuple<int, int, int, int> qsig{-1, -1, -1, -1};
  // host-buffer calls (nch > 1): per copy chunk and FP32 class (mixed mode)
  // the tasks whose coefficients (collocate) or post-processing (integrate)
  // depend on that chunk of pab / hab
  std::vector<int *> d_chunk_idx; // [chunk * 2 + class]
  std::vector<int> chunk_n;
  int coef_words = 0;      // per-warp shared memory words of coefficient/post
  int transform = -1;      // transform variant the words were sized for
  int sched_version = -1;
  // mixed mode row split: per task squared cylinder radius (kCoreAll: whole
  // task in its class), on the device for the kernels
  std::vector<float> core_r2;
  float *d_core_r2 = nullptr;
  bool row_split = false; // some task runs split
};

struct TaskList {
  // row-split radii and outside shares per (l shifts, derivative factor,
  // threshold), shared by the modes that need the same ones
  std::map<std::tuple<int, int, int, double>, std::pair<std::vector<float>, std::vector<double>>>
      core_cache;
  bool empty = false;
  bool ortho = true;
  int ntasks = 0, nlevels = 0, natoms = 0, nkinds = 0, nblocks = 0;
  long long buffer_len = 0;
  int precision = GRID_GB300_FP64;
  int schedule = GRID_GB300_SCHEDULE_SIZE;
  int sched_version = 0;
  LevelSet levels{};
  std::vector<TaskDesc> tasks; // block order
  std::vector<SubblockDesc> subs;
  std::vector<SphereHdr> sph;
  std::vector<int16_t> sph_tab;
  std::vector<int> sph_pts, sph_ploff; // point lists of the spheres
  std::vector<long long> points; // per task (block order)
  std::vector<float> model_cost; // per task, empty unless a model was applied
  double model_bin = 0.2;        // width of the log-time bins of the model schedule
  std::vector<float> features;   // per task [6]: cost-model inputs (block order)
  bool task_timing = false;      // record clock64 cycles per task
  bool launch_timing = false;    // record CUDA events around every grid launch
  bool capturing = false;        // inside grid_gb300_capture_step: no timing events
  long long gen = 0;             // bumped whenever a device array the kernels use moves
  std::vector<LaunchRecord> launches; // of the last call
  std::vector<cudaEvent_t> event_pool;
  std::map<std::tuple<int, int, int>, LaunchCfg> tuned; // (precision, phase, queue key) -> shape
  int small_extent[3] = {kSmallExtent, kSmallExtent, kSmallExtent}; // per precision
  int coll_variant = -1; // orthorhombic collocate lanes: 0 row walk, 1 point list, -1 by arith
  int transform_variant = -1; // C_ab <-> C_xyz: 0 direct, 1 staged, -1 by l (uses_staged)
  std::vector<double> gbound;    // per task bound of |contribution| for |P| <= 1
  float2 *d_seeds = nullptr;
  double mixed_threshold = 0.3;  // mixed path: tasks with gbound <= this run FP32
  std::vector<int> npts_local;   // [nlevels][3]
  size_t cart_total = 0;
  int contract_words = 1;
  // device
  TaskDesc *d_tasks = nullptr;
  SubblockDesc *d_subs = nullptr;
  SphereHdr *d_sph = nullptr;
  int16_t *d_sph_tab = nullptr;
  int *d_sph_pts = nullptr, *d_sph_ploff = nullptr;
  double *d_dhtab = nullptr;
  float *d_dhtab_f = nullptr;
  float2 *d_dhtab_df = nullptr;
  double *d_atom_pos = nullptr;
  double *d_sphi = nullptr;
  LevelSet *d_levels = nullptr;
  double *d_pab_cart = nullptr, *d_hab_cart = nullptr;
  void *d_coef = nullptr; // collocate coefficients
  size_t coef_cap = 0;
  double *d_coef_int = nullptr; // integrated coefficients
  size_t coef_int_cap = 0;
  void *d_gridsplit[GB300_MAX_LEVELS] = {}; // integrate: V as float / float2
  float *d_gridhi[GB300_MAX_LEVELS] = {};    // mixed integrate: V high words, dense
  float *d_gridlo[GB300_MAX_LEVELS] = {};   // collocate: low words (mixed)
  double *d_forces = nullptr, *d_virial = nullptr;
  int *d_counters = nullptr; // one per queue launch (kMaxQueues)
  // host-buffer calls: pab / hab copies in pieces that overlap the kernels
  int copy_chunks = 3;
  CopyChunks chunks;
  int chunks_for = -1; // copy_chunks the chunks were computed for
  cudaStream_t copy_stream = nullptr;
  std::vector<cudaEvent_t> copy_ev;
  // the independent grid launches of a phase alternate over this many
  // streams, so that one launch's tail overlaps the next one's start
  int queue_streams = 2;
  // orthorhombic, FP32 class, lp <= 6: the tensor-core kernels
  int tc_integrate = 1;
  int tc_collocate = 0; // measured slower than the CUDA-core collocation
  // mixed mode: the outer rows of orthorhombic double-float tasks in FP32
  int row_split = 1;
  cudaStream_t aux_stream = nullptr;
  cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
  int *d_error = nullptr;
  long long *d_cycles = nullptr;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[5] = {};
  double timings[4] = {0, 0, 0, 0};
  std::map<int, Mode> modes;
};

static int mode_key(const LDiffs &d) {
  return ((d.la_max + 4) << 12) | ((d.la_min + 4) << 8) | ((d.lb_max + 4) << 4) | (d.lb_min + 4);
}

// grid_prepare_pab.h:447-517
static LDiffs func_ldiffs(int f) {
  LDiffs d{0, 0, 0, 0};
  if (f == GRID_FUNC_AB)
    return d;
  if (f >= 411 && f <= 433 && f % 10 >= 1 && f % 10 <= 3)
    return LDiffs{1, -1, 2, -1};
  if ((f >= 701 && f <= 703) || (f >= 801 && f <= 803))
    return LDiffs{2, -2, 2, -2};
  if (f == 200 || (f >= 301 && f <= 303) || (f >= 501 && f <= 503) || (f >= 601 && f <= 603) ||
      (f >= 901 && f <= 906) || (f >= 1001 && f <= 1003))
    return LDiffs{1, -1, 1, -1};
  fail("unknown grid_func %d", f);
}

// grid_process_vab.h:222-251
static LDiffs integrate_ldiffs(bool forces, bool virial, bool tau) {
  LDiffs d{0, 0, 0, 0};
  if (forces || virial) {
    d.la_max += 1;
    d.la_min -= 1;
    d.lb_min -= 1;
  }
  if (virial) {
    d.la_max += 1;
    d.lb_max += 1;
  }
  if (tau) {
    d.la_max += 1;
    d.lb_max += 1;
    d.la_min -= 1;
    d.lb_min -= 1;
  }
  return d;
}

// Sphere bounds of one (level, discretised radius), with the reference's
// expressions (grid_ref_collint.h:237-245, 139-151, 44-52).
void build_sphere(const LevelDesc &L, double disr, SphereHdr &h, std::vector<int16_t> &tab,
                  long long &npoints) {
  h.plo = -1;
  for (int i = 0; i < 3; i++)
    h.lb[i] = (int)ceil(-1e-8 - disr * L.dh_inv[i * 4]);
  h.cmax = std::max(std::max(1 - h.lb[0], 1 - h.lb[1]), 1 - h.lb[2]);
  h.off = (int)tab.size();
  const int K = 1 - h.lb[2], NX = 1 - h.lb[0];
  std::vector<int> js(K), rows;
  std::vector<int16_t> is;
  npoints = 0;
  for (int kk = 0; kk < K; kk++) {
    const int k1 = -kk;
    const int kd = (2 * k1 - 1) / 2;
    const double kr = kd * L.dh[8];
    const double kremain = disr * disr - kr * kr;
    const int jstart = (int)ceil(-1e-8 - sqrt(fmax(0.0, kremain)) * L.dh_inv[4]);
    js[kk] = jstart;
    rows.push_back((int)is.size());
    for (int jj = 0; jj <= -jstart; jj++) {
      const int j1 = -jj;
      const int jd = (2 * j1 - 1) / 2;
      const double jr = jd * L.dh[4];
      const double jremain = kremain - jr * jr;
      const int istart = (int)ceil(-1e-8 - sqrt(fmax(0.0, jremain)) * L.dh_inv[0]);
      is.push_back((int16_t)istart);
      npoints += 4LL * (2 - 2 * istart); // rows j1, j2 of planes k1, k2
    }
  }
  // last row index JJ per (plane, x): x with distance index ii lies on rows
  // j in [-JJ, JJ + 1] (row jj holds x iff istart(kk, jj) <= -ii; istart
  // grows with jj), -1 if no row of the plane holds x.
  std::vector<int16_t> jx((size_t)K * NX, -1);
  for (int kk = 0; kk < K; kk++)
    for (int ii = 0; ii < NX; ii++) {
      int last = -1;
      for (int jj = 0; jj <= -js[kk]; jj++)
        if (is[rows[kk] + jj] <= -ii)
          last = jj;
      jx[(size_t)kk * NX + ii] = (int16_t)last;
    }
  // integrate lane plan: split the x range into nc chunks of sw lanes and
  // give each chunk n[c] row groups (floor(32 / sw) groups in all), so that
  // lanes of short edge columns are not idle while central columns finish;
  // cost = sum over planes of the slowest group's rows, minimised over nc
  h.iplan = 0;
  {
    const int W = 2 * NX; // x in [lb0, 1 - lb0]
    if (W <= 32) {
      auto len = [&](int kk, int x) { // rows of column x on plane kk
        const int ii = x <= 0 ? -x : x - 1;
        return 2 * (jx[(size_t)kk * NX + ii] + 1);
      };
      long long best = -1;
      for (int nc = 1; nc <= 4; nc++) {
        const int sw = (W + nc - 1) / nc, gt = 32 / sw;
        if (gt < nc || (nc > 1 && (nc - 1) * sw >= W))
          continue;
        int n[4] = {1, 1, 1, 1};
        auto cost = [&](const int *nn) {
          long long c = 0;
          for (int kk = 0; kk < K; kk++) {
            int m = 0;
            for (int ci = 0; ci < nc; ci++) {
              int ml = 0;
              for (int x = h.lb[0] + ci * sw; x < h.lb[0] + (ci + 1) * sw && x <= 1 - h.lb[0]; x++)
                ml = std::max(ml, len(kk, x));
              m = std::max(m, (ml + nn[ci] - 1) / nn[ci]);
            }
            c += m;
          }
          return c;
        };
        for (int extra = gt - nc; extra > 0; extra--) { // greedy: where it helps most
          int bc = 0;
          long long bv = -1;
          for (int ci = 0; ci < nc; ci++) {
            n[ci]++;
            const long long v = cost(n);
            n[ci]--;
            if (bv < 0 || v < bv) {
              bv = v;
              bc = ci;
            }
          }
          n[bc]++;
        }
        const long long c = cost(n);
        if (best < 0 || c < best) {
          best = c;
          h.iplan = sw | (nc << 6);
          for (int ci = 0; ci < nc; ci++)
            h.iplan |= n[ci] << (9 + 5 * ci);
        }
      }
    }
  }
  for (int kk = 0; kk < K; kk++)
    tab.push_back((int16_t)js[kk]);
  for (int kk = 0; kk < K; kk++)
    tab.push_back((int16_t)rows[kk]);
  if (is.size() + jx.size() + 2 * (size_t)K > 32767)
    fail("sphere table exceeds int16 offsets");
  tab.insert(tab.end(), is.begin(), is.end());
  h.jxo = 2 * K + (int)is.size();
  tab.insert(tab.end(), jx.begin(), jx.end());
}

// LU factorisation with partial pivoting of M[c][d] = dh[d][c] per level:
// P M = L D U with L unit lower, U unit upper, (P x)_i = x_pi(i)
void build_dh_table(const LevelSet &ls, std::vector<double> &tab) {
  tab.assign(dh_table_size(ls.nlevels), 0.0);
  for (int l = 0; l < ls.nlevels; l++) {
    double A[3][3];
    int pi[3] = {0, 1, 2};
    for (int c = 0; c < 3; c++)
      for (int d = 0; d < 3; d++)
        A[c][d] = ls.lv[l].dh[3 * d + c];
    for (int k = 0; k < 3; k++) {
      int p = k;
      for (int i = k + 1; i < 3; i++)
        if (std::fabs(A[i][k]) > std::fabs(A[p][k]))
          p = i;
      if (A[p][k] == 0.0)
        fail("singular grid spacing matrix on level %d", l);
      std::swap(A[k], A[p]);
      std::swap(pi[k], pi[p]);
      for (int i = k + 1; i < 3; i++) {
        A[i][k] /= A[k][k];
        for (int j = k + 1; j < 3; j++)
          A[i][j] -= A[i][k] * A[k][j];
      }
    }
    double *t = &tab[(size_t)l * kLatTab];
    for (int i = 0; i < 3; i++) {
      t[i] = pi[i];
      t[6 + i] = A[i][i];
    }
    t[3] = A[1][0];
    t[4] = A[2][0];
    t[5] = A[2][1];
    t[9] = A[0][2] / A[0][0];
    t[10] = A[1][2] / A[1][1];
    t[11] = A[0][1] / A[0][0];
  }
}

void build_sphere_points(SphereHdr &h, const std::vector<int16_t> &tab, std::vector<int> &pts,
                         std::vector<int> &ploff) {
  const int K = 1 - h.lb[2];
  const int16_t *t = tab.data() + h.off;
  h.plo = (int)ploff.size();
  for (int kk = 0; kk < K; kk++) {
    ploff.push_back((int)pts.size());
    const int js = t[kk], row0 = t[K + kk];
    for (int j = js; j <= 1 - js; j++) {
      const int jj = j <= 0 ? -j : j - 1;
      const int i0 = t[2 * K + row0 + jj];
      for (int x = i0; x <= 1 - i0; x++)
        pts.push_back((int)((unsigned)(x & 0xffff) | ((unsigned)j << 16)));
    }
  }
  ploff.push_back((int)pts.size());
  if (pts.size() > (size_t)INT32_MAX)
    fail("sphere point lists exceed int offsets");
}

// Upper bound of |a Gaussian-product contribution| to any point for
// Cartesian density-matrix elements |P_ab| <= 1: the prefactor times the sum,
// over the Cartesian pairs (a, b) of the task's sets, of the product over the
// three directions of B[a_d][b_d] = sum_n |alpha_n| max_x |x^n exp(-zetp x^2)|
// with alpha the binomial expansion of (x-A)^i (x-B)^j about P and
// max_x |x^n exp(-z x^2)| = (n / (2 e z))^(n/2).  Used to pick FP32 or
// double-float per task.
static double contribution_bound(const TaskDesc &d, const double *ra) {
  const int la = d.la_max, lb = d.lb_max;
  // binomial coefficients, once
  static const auto binom = [] {
    std::array<std::array<double, GB300_LMAX + 1>, GB300_LMAX + 1> c{};
    for (int n = 0; n <= GB300_LMAX; n++) {
      c[n][0] = 1.0;
      for (int k = 1; k <= n; k++)
        c[n][k] = c[n - 1][k - 1] + (k <= n - 1 ? c[n - 1][k] : 0.0);
    }
    return c;
  }();
  double m[2 * GB300_LMAX + 2];
  for (int n = 0; n <= la + lb; n++)
    m[n] = n == 0 ? 1.0 : pow(n / (2.0 * M_E * d.zetp), 0.5 * n);
  double B[3][GB300_LMAX + 1][GB300_LMAX + 1];
  for (int dir = 0; dir < 3; dir++) {
    const double pa = d.rp[dir] - ra[dir], pb = d.rp[dir] - (ra[dir] + d.rab[dir]);
    double ppa[GB300_LMAX + 1], ppb[GB300_LMAX + 1];
    ppa[0] = ppb[0] = 1.0;
    for (int k = 1; k <= GB300_LMAX; k++) {
      ppa[k] = ppa[k - 1] * pa;
      ppb[k] = ppb[k - 1] * pb;
    }
    for (int xa = 0; xa <= la; xa++)
      for (int xb = 0; xb <= lb; xb++) {
        double al[2 * GB300_LMAX + 2] = {0};
        for (int k = 0; k <= xa; k++) {
          const double wa = binom[xa][k] * ppa[k];
          for (int q = 0; q <= xb; q++)
            al[xa - k + xb - q] += wa * binom[xb][q] * ppb[q];
        }
        double s = 0.0;
        for (int n = 0; n <= xa + xb; n++)
          s += fabs(al[n]) * m[n];
        B[dir][xa][xb] = s;
      }
  }
  double g = 0.0;
  for (int l1 = d.la_min; l1 <= la; l1++)
    for (int ax = 0; ax <= l1; ax++)
      for (int ay = 0; ay <= l1 - ax; ay++) {
        const int az = l1 - ax - ay;
        for (int l2 = d.lb_min; l2 <= lb; l2++)
          for (int bx = 0; bx <= l2; bx++)
            for (int by = 0; by <= l2 - bx; by++) {
              const int bz = l2 - bx - by;
              g += B[0][ax][bx] * B[1][ay][by] * B[2][az][bz];
            }
      }
  return g * d.prefexp * ((d.iatom == d.jatom) ? 1.0 : 2.0);
}

// Row split of a double-float task (mixed mode, orthorhombic cubes).  A row
// (j, k) of the cube at distance rho = sqrt(y^2 + z^2) from the Gaussian
// product's x axis holds contributions of at most
//   f(rho) = prefactor sum_(a,b) B_x[a_x][b_x] sum_n C_n rho^n exp(-zetp rho^2)
// for |P_ab| <= 1: B_x is contribution_bound's x factor (maximum over x) and
// C_n collects the products of the y and z binomial expansions, with
// |y|^p |z|^q <= rho^(p+q).  Past rho0 = sqrt(nmax / (2 zetp)) every term
// decreases, so the rows with rho >= rc, f(rc) <= tau, obey the FP32 class's
// bound and run in FP32; the rows inside stay double-float.  Returns rc^2
// (bohr^2) and the share of the sphere's points outside, or kCoreAll when
// that share is under a half (the second pass over the task repeats its
// table set-up and plane folds; measured on the 512-atom workload, shares
// from a tenth up split nearly the same tasks and time the same).
// The outside rows obey the bound tau / kShellMargin rather than tau: their
// FP32 rounding errors are correlated within a task (one set of rounded
// coefficients and table values), unlike those of many small FP32-class
// tasks.  Measured on the 512-atom workload (mixed step, Tr(V rho) error per
// atom against the oracle; the errors do not fall monotonically): margin 1
// gives 7.0e-10 Ha, 1.5 gives 7.2e-10, 2 gives 8.3e-11, 3 gives 2.8e-10,
// against the 1e-8 target; the step takes 18.83, 18.85, 19.01 and 19.11 ms
// (rho 5.7e-8 throughout).  Earlier, with every task whole, 1.1e-10.
constexpr double kShellMargin = 1.5;

static float core_radius2(const TaskDesc &d, int dla, int dlb, double tau, double *outside) {
  *outside = 0.0;
  // the call's l shifts (derivatives) raise the polynomial degree of the
  // rows' values: the bound runs over the shifted l ranges
  if (d.la_max + dla > GB300_LMAX || d.lb_max + dlb > GB300_LMAX)
    return kCoreAll; // past the tables below: keep the task whole
  const int la = d.la_max + dla, lb = d.lb_max + dlb;
  const int la_min = std::max(d.la_min - dla, 0), lb_min = std::max(d.lb_min - dlb, 0);
  const int nn = la + lb + 1;
  double bin[GB300_LMAX + 1][GB300_LMAX + 1] = {};
  for (int n = 0; n <= GB300_LMAX; n++) {
    bin[n][0] = 1.0;
    for (int k = 1; k <= n; k++)
      bin[n][k] = bin[n - 1][k - 1] + (k <= n - 1 ? bin[n - 1][k] : 0.0);
  }
  double m[2 * GB300_LMAX + 2];
  for (int n = 0; n < nn; n++)
    m[n] = n == 0 ? 1.0 : pow(n / (2.0 * M_E * d.zetp), 0.5 * n);
  // |binomial expansion| of (x - A)^xa (x - B)^xb about P, per direction
  static thread_local double al[3][GB300_LMAX + 1][GB300_LMAX + 1][2 * GB300_LMAX + 2];
  for (int dir = 0; dir < 3; dir++) {
    const double pa = d.zetb / d.zetp * d.rab[dir], pb = pa - d.rab[dir];
    double ppa[GB300_LMAX + 1], ppb[GB300_LMAX + 1];
    ppa[0] = ppb[0] = 1.0;
    for (int k = 1; k <= std::max(la, lb); k++) {
      ppa[k] = ppa[k - 1] * pa;
      ppb[k] = ppb[k - 1] * pb;
    }
    for (int xa = 0; xa <= la; xa++)
      for (int xb = 0; xb <= lb; xb++) {
        double *c = al[dir][xa][xb];
        for (int n = 0; n < nn; n++)
          c[n] = 0.0;
        for (int k = 0; k <= xa; k++)
          for (int q = 0; q <= xb; q++)
            c[xa - k + xb - q] += bin[xa][k] * ppa[k] * bin[xb][q] * ppb[q];
        for (int n = 0; n < nn; n++)
          c[n] = fabs(c[n]);
      }
  }
  double C[4 * GB300_LMAX + 2] = {};
  for (int l1 = la_min; l1 <= la; l1++)
    for (int ax = 0; ax <= l1; ax++)
      for (int ay = 0; ay <= l1 - ax; ay++) {
        const int az = l1 - ax - ay;
        for (int l2 = lb_min; l2 <= lb; l2++)
          for (int bx = 0; bx <= l2; bx++)
            for (int by = 0; by <= l2 - bx; by++) {
              const int bz = l2 - bx - by;
              const double *cx = al[0][ax][bx], *cy = al[1][ay][by], *cz = al[2][az][bz];
              double Bx = 0.0;
              for (int n = 0; n <= ax + bx; n++)
                Bx += cx[n] * m[n];
              for (int p = 0; p <= ay + by; p++)
                for (int q = 0; q <= az + bz; q++)
                  C[p + q] += Bx * cy[p] * cz[q];
            }
      }
  int nmax = 0;
  for (int n = 0; n < 2 * nn; n++)
    if (C[n] > 0.0)
      nmax = n;
  const double pref = d.prefexp * ((d.iatom == d.jatom) ? 1.0 : 2.0);
  auto f = [&](double r) {
    double poly = 0.0;
    for (int n = nmax; n >= 0; n--)
      poly = poly * r + C[n];
    return pref * poly * exp(-d.zetp * r * r);
  };
  const double R = d.radius, r0 = sqrt(nmax / (2.0 * d.zetp));
  if (r0 >= R || f(R) > tau)
    return kCoreAll;
  double lo = r0, hi = R;
  if (f(r0) > tau) {
    // 26 halvings leave hi within 2^-26 R above the crossing (the radius is
    // kept as a float, rounded up)
    for (int it = 0; it < 26; it++) {
      const double mid = 0.5 * (lo + hi);
      (f(mid) > tau ? lo : hi) = mid;
    }
  } else {
    hi = r0;
  }
  const double share = pow(std::max(0.0, 1.0 - hi * hi / (R * R)), 1.5);
  if (share < 0.5)
    return kCoreAll;
  *outside = share;
  return nextafterf((float)(hi * hi), kCoreAll);
}

template <typename T> static T *dalloc_copy(const std::vector<T> &v) {
  T *p = nullptr;
  const size_t n = v.empty() ? 1 : v.size();
  CK(cudaMalloc((void **)&p, sizeof(T) * n));
  if (!v.empty())
    CK(cudaMemcpy(p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice));
  return p;
}

static void free_device(TaskList *t) {
  void *ptrs[] = {t->d_seeds, t->d_tasks, t->d_subs, t->d_sph, t->d_sph_tab, t->d_sph_pts,
                  t->d_sph_ploff, t->d_dhtab, t->d_dhtab_f, t->d_dhtab_df, t->d_atom_pos,
                  t->d_sphi,
                  t->d_levels, t->d_pab_cart, t->d_hab_cart, t->d_coef, t->d_coef_int,
                  t->d_forces, t->d_virial, t->d_counters, t->d_error, t->d_cycles};
  for (void *p : ptrs)
    if (p)
      cudaFree(p);
  for (int l = 0; l < GB300_MAX_LEVELS; l++) {
    if (t->d_gridsplit[l])
      cudaFree(t->d_gridsplit[l]);
    if (t->d_gridhi[l])
      cudaFree(t->d_gridhi[l]);
    if (t->d_gridlo[l])
      cudaFree(t->d_gridlo[l]);
  }
  for (auto &kv : t->modes) {
    if (kv.second.d_coef_off)
      cudaFree(kv.second.d_coef_off);
    for (int *p : kv.second.d_chunk_idx)
      if (p)
        cudaFree(p);
    if (kv.second.d_qidx)
      cudaFree(kv.second.d_qidx);
    if (kv.second.d_qitems)
      cudaFree(kv.second.d_qitems);
    if (kv.second.d_core_r2)
      cudaFree(kv.second.d_core_r2);
  }
  for (auto &e : t->ev)
    if (e)
      cudaEventDestroy(e);
  for (auto &e : t->event_pool)
    cudaEventDestroy(e);
  if (t->stream)
    cudaStreamDestroy(t->stream);
  for (auto &e : t->copy_ev)
    cudaEventDestroy(e);
  if (t->copy_stream)
    cudaStreamDestroy(t->copy_stream);
  if (t->fork_ev)
    cudaEventDestroy(t->fork_ev);
  if (t->join_ev)
    cudaEventDestroy(t->join_ev);
  if (t->aux_stream)
    cudaStreamDestroy(t->aux_stream);
}

static bool sphi_is_identity(const grid_basis_set *b, int iset) {
  const int nco = b->npgf[iset] * ncoset(b->lmax[iset]);
  if (b->nsgf_set[iset] != nco)
    return false;
  const int s0 = b->first_sgf[iset] - 1;
  for (int r = 0; r < nco; r++)
    for (int c = 0; c < nco; c++)
      if (b->sphi[(size_t)(s0 + r) * b->maxco + c] != (r == c ? 1.0 : 0.0))
        return false;
  return true;
}

// GRID_GB300_HOST_TIMING set: the host phases of task-list creation and of
// the work-queue construction, in ms since the start of the call, on stderr
struct HostPhases {
  bool on;
  const char *what;
  std::chrono::steady_clock::time_point t0;
  explicit HostPhases(const char *w)
      : on(getenv("GRID_GB300_HOST_TIMING") != nullptr), what(w),
        t0(std::chrono::steady_clock::now()) {}
  void mark(const char *phase) const {
    if (on)
      fprintf(stderr, "grid_gb300 host %s: %s %.2f ms\n", what, phase,
              std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0)
                  .count());
  }
};

// host threads for the preparation (GRID_GB300_HOST_THREADS fixes it)
static int host_threads() {
  int nt = (int)std::max(1u, std::min(std::thread::hardware_concurrency(), 64u));
  if (const char *e = getenv("GRID_GB300_HOST_THREADS")) // testing: fix the thread count
    nt = std::max(1, std::min(atoi(e), 64));
  return nt;
}

// Runs body(i) for i in [0, n) on the host's cores, in contiguous chunks.
template <typename F> static void parallel_for(int n, const F &body) {
  const int nt = host_threads();
  const int chunks = n < 4096 ? 1 : nt;
  if (chunks == 1) {
    for (int i = 0; i < n; i++)
      body(i);
    return;
  }
  std::vector<std::thread> th;
  for (int c = 0; c < chunks; c++)
    th.emplace_back([&, c] {
      const int i0 = (int)((long long)n * c / chunks), i1 = (int)((long long)n * (c + 1) / chunks);
      for (int i = i0; i < i1; i++)
        body(i);
    });
  for (auto &x : th)
    x.join();
}

// Runs body(i) for i in [0, n) on the host's cores, items taken one at a
// time (for few items of uneven cost).
template <typename F> static void parallel_items(int n, const F &body) {
  const int nt = std::min(host_threads(), n);
  if (nt <= 1) {
    for (int i = 0; i < n; i++)
      body(i);
    return;
  }
  std::atomic<int> next{0};
  std::vector<std::thread> th;
  for (int c = 0; c < nt; c++)
    th.emplace_back([&] {
      for (int i = next++; i < n; i = next++)
        body(i);
    });
  for (auto &x : th)
    x.join();
}

// std::sort on the host's cores: chunks sorted in parallel, then merged
// pairwise in rounds.  With a comparator that orders no two elements equal
// the result is that of std::sort, whatever the number of threads.
template <typename T, typename C> static void parallel_sort(std::vector<T> &v, C comp) {
  const size_t n = v.size();
  int nt = host_threads();
  while (nt > 1 && n / (size_t)nt < 16384)
    nt /= 2;
  if (nt <= 1) {
    std::sort(v.begin(), v.end(), comp);
    return;
  }
  std::vector<size_t> b(nt + 1);
  for (int c = 0; c <= nt; c++)
    b[c] = n * (size_t)c / (size_t)nt;
  {
    std::vector<std::thread> th;
    for (int c = 0; c < nt; c++)
      th.emplace_back([&, c] { std::sort(v.begin() + b[c], v.begin() + b[c + 1], comp); });
    for (auto &x : th)
      x.join();
  }
  std::vector<T> tmp(n);
  std::vector<T> *src = &v, *dst = &tmp;
  for (int w = 1; w < nt; w *= 2) {
    std::vector<std::thread> th;
    for (int c = 0; c < nt; c += 2 * w)
      th.emplace_back([&, c] {
        const size_t lo = b[c], mid = b[std::min(c + w, nt)], hi = b[std::min(c + 2 * w, nt)];
        std::merge(src->begin() + lo, src->begin() + mid, src->begin() + mid,
                   src->begin() + hi, dst->begin() + lo, comp);
      });
    for (auto &x : th)
      x.join();
    std::swap(src, dst);
  }
  if (src != &v)
    v.swap(*src);
}

// The FP64 seeds of the double-float Gaussian recurrences of every
// orthorhombic task (zeros for skipped and general-path tasks), per
// direction exp(-z r^2), exp(-z h (h - 2r)), exp(-z h (h + 2r)),
// exp(-2 z h^2), h, -r as (high, low) float pairs, from the task's
// descriptor and its level's spacing (the recurrences of grid_kernels.cu)
__global__ void seeds_kernel(const TaskDesc *__restrict__ tasks, int ntasks,
                             const LevelSet *__restrict__ levels, float2 *__restrict__ seeds) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < ntasks; t += gridDim.x * blockDim.x) {
    const TaskDesc &d = tasks[t];
    float2 *o = seeds + (size_t)t * 18;
    if (d.flags & (TF_SKIP | TF_GENERAL)) {
      for (int q = 0; q < 18; q++)
        o[q] = make_float2(0.f, 0.f);
      continue;
    }
    const LevelDesc &L = levels->lv[d.level];
    for (int dir = 0; dir < 3; dir++) {
      const double h = L.dh[dir * 4], r = d.roff[dir], z = d.zetp;
      const double v[6] = {exp(__dmul_rn(__dmul_rn(-z, r), r)),
                           exp(__dmul_rn(__dmul_rn(-z, h), __dsub_rn(h, __dmul_rn(2.0, r)))),
                           exp(__dmul_rn(__dmul_rn(-z, h), __dadd_rn(h, __dmul_rn(2.0, r)))),
                           exp(__dmul_rn(__dmul_rn(__dmul_rn(-2.0, z), h), h)), h, -r};
      for (int q = 0; q < 6; q++) {
        const float hi = __double2float_rn(v[q]);
        o[dir * 6 + q] = make_float2(hi, __double2float_rn(v[q] - (double)hi));
      }
    }
  }
}

static TaskList *create(bool ortho, int ntasks, int nlevels, int natoms, int nkinds,
                        int nblocks, const int *block_offsets, const double *atom_positions,
                        const int *atom_kinds, const grid_basis_set **basis_sets,
                        const int *level_list, const int *iatom_list, const int *jatom_list,
                        const int *iset_list, const int *jset_list, const int *ipgf_list,
                        const int *jpgf_list, const int *border_mask_list,
                        const int *block_num_list, const double *radius_list,
                        const double *rab_list, const int *npts_global, const int *npts_local,
                        const int *shift_local, const int *border_width, const double *dh,
                        const double *dh_inv, bool host_only = false) {
  const HostPhases hp("create");
  TaskList *t = new TaskList();
  t->ortho = ortho;
  t->ntasks = ntasks;
  t->nlevels = nlevels;
  t->natoms = natoms;
  t->nkinds = nkinds;
  t->nblocks = nblocks;
  if (nlevels > GB300_MAX_LEVELS)
    fail("at most %d grid levels are supported (got %d)", GB300_MAX_LEVELS, nlevels);
  t->npts_local.assign(npts_local, npts_local + 3 * std::max(nlevels, 0));
  if (ntasks == 0 || nblocks == 0 || nlevels == 0) {
    t->empty = true;
    return t;
  }
  // ---- levels
  t->levels.nlevels = nlevels;
  for (int l = 0; l < nlevels; l++) {
    LevelDesc &L = t->levels.lv[l];
    for (int i = 0; i < 3; i++) {
      L.npts_global[i] = npts_global[3 * l + i];
      L.npts_local[i] = npts_local[3 * l + i];
      L.shift[i] = shift_local[3 * l + i];
      L.border_width[i] = border_width[3 * l + i];
      if (L.npts_global[i] < 1 || L.npts_local[i] < 1)
        fail("level %d: empty grid", l);
    }
    L.dh_max = 0.0;
    for (int i = 0; i < 9; i++) {
      L.dh[i] = dh[9 * l + i];
      L.dh_inv[i] = dh_inv[9 * l + i];
      L.dh_max = fmax(L.dh_max, fabs(L.dh[i]));
    }
  }
  // ---- basis data on device: concatenated sphi per kind
  std::vector<long long> sphi_off(nkinds);
  std::vector<double> sphi_all;
  for (int k = 0; k < nkinds; k++) {
    const grid_basis_set *b = basis_sets[k];
    sphi_off[k] = (long long)sphi_all.size();
    sphi_all.insert(sphi_all.end(), b->sphi, b->sphi + (size_t)b->nsgf * b->maxco);
  }
  // ---- block order
  std::vector<int> order(ntasks);
  std::iota(order.begin(), order.end(), 0);
  for (int i = 0; i < ntasks; i++) {
    const int lev = level_list[i], ia = iatom_list[i], ja = jatom_list[i], bn = block_num_list[i];
    if (lev < 1 || lev > nlevels || ia < 1 || ia > natoms || ja < 1 || ja > natoms || bn < 1 ||
        bn > nblocks)
      fail("task %d: index out of range (level %d, atoms %d/%d, block %d)", i, lev, ia, ja, bn);
    const grid_basis_set *bi = basis_sets[atom_kinds[ia - 1] - 1];
    const grid_basis_set *bj = basis_sets[atom_kinds[ja - 1] - 1];
    if (iset_list[i] < 1 || iset_list[i] > bi->nset || jset_list[i] < 1 || jset_list[i] > bj->nset ||
        ipgf_list[i] < 1 || ipgf_list[i] > bi->npgf[iset_list[i] - 1] || jpgf_list[i] < 1 ||
        jpgf_list[i] > bj->npgf[jset_list[i] - 1])
      fail("task %d: set/pgf index out of range", i);
    if (!(radius_list[i] >= 0.0) || !std::isfinite(radius_list[i]))
      fail("task %d: invalid radius %g", i, radius_list[i]);
  }
  hp.mark("validated");
  // stable order by (block, iset, jset, level): sort packed keys with the
  // input index as the last key
  {
    struct Key {
      int block, iset, jset, level, i;
    };
    std::vector<Key> keys(ntasks);
    bool by_block = true; // input already in block order (as the generators make it)
    for (int i = 0; i < ntasks; i++) {
      keys[i] = Key{block_num_list[i], iset_list[i], jset_list[i], level_list[i], i};
      by_block = by_block && (i == 0 || block_num_list[i] >= block_num_list[i - 1]);
    }
    const auto less = [](const Key &a, const Key &b) {
      if (a.block != b.block)
        return a.block < b.block;
      if (a.iset != b.iset)
        return a.iset < b.iset;
      if (a.jset != b.jset)
        return a.jset < b.jset;
      if (a.level != b.level)
        return a.level < b.level;
      return a.i < b.i;
    };
    if (by_block) { // each block's run on its own, in parallel
      std::vector<int> run = {0};
      for (int i = 1; i < ntasks; i++)
        if (keys[i].block != keys[i - 1].block)
          run.push_back(i);
      run.push_back(ntasks);
      parallel_for((int)run.size() - 1, [&](int r) {
        std::sort(keys.begin() + run[r], keys.begin() + run[r + 1], less);
      });
    } else {
      parallel_sort(keys, less);
    }
    for (int i = 0; i < ntasks; i++)
      order[i] = keys[i].i;
  }
  hp.mark("sorted");
  // ---- tasks, subblocks, sphere tables
  t->tasks.resize(ntasks);
  t->points.assign(ntasks, 0);
  t->gbound.assign(ntasks, 0.0);

  t->features.assign((size_t)ntasks * 6, 0.f);
  // cell skew of the finest level's cell (0 for orthorhombic cells)
  double skew = 0.0;
  {
    const double *h = dh; // rows: step vectors
    const double det = h[0] * (h[4] * h[8] - h[5] * h[7]) - h[1] * (h[3] * h[8] - h[5] * h[6]) +
                       h[2] * (h[3] * h[7] - h[4] * h[6]);
    double norms = 1.0;
    for (int r = 0; r < 3; r++)
      norms *= sqrt(h[3 * r] * h[3 * r] + h[3 * r + 1] * h[3 * r + 1] + h[3 * r + 2] * h[3 * r + 2]);
    skew = norms > 0.0 ? 1.0 - fabs(det) / norms : 0.0;
  }
  // Phase 1, in parallel over the tasks: everything a task needs that does
  // not depend on the shared sphere tables (geometry, seeds, general-path
  // boxes and point counts, class bounds, most features).
  std::vector<long long> nrad_of(ntasks, -1); // ortho tasks: discretised radius
  parallel_for(ntasks, [&](int s) {
    const int i = order[s];
    TaskDesc &d = t->tasks[s];
    memset(&d, 0, sizeof(d));
    const int lev = level_list[i] - 1, ia = iatom_list[i] - 1, ja = jatom_list[i] - 1;
    const int iset = iset_list[i] - 1, jset = jset_list[i] - 1;
    const grid_basis_set *bi = basis_sets[atom_kinds[ia] - 1];
    const grid_basis_set *bj = basis_sets[atom_kinds[ja] - 1];
    const LevelDesc &L = t->levels.lv[lev];
    d.level = lev;
    d.iatom = ia;
    d.jatom = ja;
    d.orig = i;
    d.la_max = (int8_t)bi->lmax[iset];
    d.la_min = (int8_t)bi->lmin[iset];
    d.lb_max = (int8_t)bj->lmax[jset];
    d.lb_min = (int8_t)bj->lmin[jset];
    d.o1 = (int16_t)((ipgf_list[i] - 1) * ncoset(bi->lmax[iset]));
    d.o2 = (int16_t)((jpgf_list[i] - 1) * ncoset(bj->lmax[jset]));
    d.border_mask = (uint8_t)border_mask_list[i];
    d.radius = radius_list[i];
    const double zeta = bi->zet[iset * bi->maxpgf + ipgf_list[i] - 1];
    const double zetb = bj->zet[jset * bj->maxpgf + jpgf_list[i] - 1];
    d.zeta = zeta;
    d.zetb = zetb;
    // cab_to_grid (grid_ref_collint.h:917-947)
    const double zetp = zeta + zetb, f = zetb / zetp;
    const double *rab = &rab_list[3 * i], *ra = &atom_positions[3 * ia];
    const double rab2 = rab[0] * rab[0] + rab[1] * rab[1] + rab[2] * rab[2];
    d.zetp = zetp;
    d.prefexp = exp(-zeta * f * rab2);
    for (int k = 0; k < 3; k++) {
      d.rab[k] = rab[k];
      d.rp[k] = ra[k] + f * rab[k];
    }
    if (2.0 * d.radius < L.dh_max) {
      d.flags |= TF_SKIP;
    } else if (ortho && d.border_mask == 0) {
      // ortho_cxyz_to_grid (grid_ref_collint.h:207-245)
      for (int k = 0; k < 3; k++) {
        double s_ = 0.0;
        for (int j = 0; j < 3; j++)
          s_ += L.dh_inv[j * 3 + k] * d.rp[j];
        d.center[k] = (int)floor(s_);
        d.roff[k] = d.rp[k] - ((double)d.center[k]) * L.dh[k * 4];
      }
      const double drmin = fmin(L.dh[0], fmin(L.dh[4], L.dh[8]));
      // clamped before the cast; radii past the int16 tables fail later
      nrad_of[s] = (long long)fmin(fmax(1.0, ceil(d.radius / drmin)), 1e9);
      // the FP64 seeds of its double-float Gaussian recurrences are
      // computed on the device after the upload (seeds_kernel)
    } else {
      // general_cijk_to_grid (grid_ref_collint.h:609-640)
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
              d.center[k] = std::min(d.center[k], (int)floor(r));
              d.imax[k] = std::max(d.imax[k], (int)ceil(r));
            }
          }
      // points: rows of the box (host count, same expressions as the kernel)
      long long np = 0;
      const int w = d.imax[0] - d.center[0] + 1;
      (void)w;
      for (int k = d.center[2]; k <= d.imax[2]; k++)
        for (int j = d.center[1]; j <= d.imax[1]; j++) {
          double qa = 0, qb = 0, qc = 0;
          for (int c = 0; c < 3; c++) {
            const double v = (0 - d.roff[0]) * L.dh[c] + (j - d.roff[1]) * L.dh[3 + c] +
                             (k - d.roff[2]) * L.dh[6 + c];
            qa += L.dh[c] * L.dh[c];
            qb += 2.0 * v * L.dh[c];
            qc += v * v;
          }
          const double disc = qb * qb - 4.0 * qa * (qc - d.radius * d.radius);
          if (0.0 < disc) {
            const double sq = sqrt(disc), inv2a = 1.0 / (2.0 * qa);
            const int lo = (int)ceil((-qb - sq) * inv2a), hi = (int)floor((-qb + sq) * inv2a);
            if (hi >= lo)
              np += hi - lo + 1;
          }
        }
      t->points[s] = np;
    }
    t->gbound[s] = contribution_bound(d, atom_positions + 3 * ia);
    float *fe = &t->features[(size_t)s * 6];
    fe[0] = (float)d.la_max;
    fe[1] = (float)d.lb_max;
    fe[2] = (float)(zeta + zetb);
    if (d.flags & TF_SKIP)
      fe[3] = 0.f;
    else if (d.flags & TF_GENERAL)
      fe[3] = 0.5f * (float)std::max(d.imax[0] - d.center[0],
                                     std::max(d.imax[1] - d.center[1], d.imax[2] - d.center[2]));
    fe[4] = (float)L.dh_max;
    fe[5] = (float)skew;
  });
  hp.mark("per-task geometry");
  // Phase 2, in task order: the sphere tables of the orthorhombic tasks
  // (shared, built on first use) and the subblocks.
  std::vector<std::vector<char>> sphi_identity(nkinds); // per kind and set
  for (int kd = 0; kd < nkinds; kd++)
    for (int st = 0; st < basis_sets[kd]->nset; st++)
      sphi_identity[kd].push_back(sphi_is_identity(basis_sets[kd], st) ? 1 : 0);
  std::vector<std::vector<int>> sphere_of(nlevels); // [level][nrad] -> sphere, or -1
  std::vector<long long> sphere_points;
  {
    // the spheres in order of first use, then built in parallel and joined
    std::vector<std::pair<int, int>> uniq; // (level, nrad)
    for (int s = 0; s < ntasks; s++) {
      if (nrad_of[s] < 0)
        continue;
      const int lev = t->tasks[s].level;
      const long long nrad = nrad_of[s];
      // the sphere tables hold int16 offsets: radii past 32767 grid steps
      // cannot be tabulated (and must not size this lookup)
      if (nrad > 32767)
        fail("task %d: radius %g spans more than 32767 grid steps of level %d", order[s],
             radius_list[order[s]], lev);
      std::vector<int> &known = sphere_of[lev];
      if ((long long)known.size() <= nrad)
        known.resize((size_t)nrad + 1, -1);
      if (known[nrad] < 0) {
        known[nrad] = (int)uniq.size();
        uniq.emplace_back(lev, (int)nrad);
      }
    }
    const int U = (int)uniq.size();
    std::vector<SphereHdr> hdr(U);
    std::vector<std::vector<int16_t>> tabs(U);
    std::vector<std::vector<int>> pts(U), plo(U);
    sphere_points.assign(U, 0);
    hp.mark("spheres listed");
    parallel_items(U, [&](int u) {
      const LevelDesc &L = t->levels.lv[uniq[u].first];
      const double drmin = fmin(L.dh[0], fmin(L.dh[4], L.dh[8]));
      build_sphere(L, drmin * (double)uniq[u].second, hdr[u], tabs[u], sphere_points[u]);
      build_sphere_points(hdr[u], tabs[u], pts[u], plo[u]);
    });
    for (int u = 0; u < U; u++) {
      SphereHdr h = hdr[u];
      h.off += (int)t->sph_tab.size();
      h.plo += (int)t->sph_ploff.size();
      const long long base = (long long)t->sph_pts.size();
      if (base + (long long)pts[u].size() > (long long)INT32_MAX)
        fail("sphere point lists exceed int offsets");
      t->sph_tab.insert(t->sph_tab.end(), tabs[u].begin(), tabs[u].end());
      for (int e : plo[u])
        t->sph_ploff.push_back((int)(e + base));
      t->sph_pts.insert(t->sph_pts.end(), pts[u].begin(), pts[u].end());
      t->sph.push_back(h);
    }
  }
  hp.mark("spheres built");
  // per task, in parallel: its sphere, point count and whether it starts a
  // subblock (a new (block, iset, jset) in the sorted order)
  std::vector<char> new_sub(ntasks, 0);
  parallel_for(ntasks, [&](int s) {
    const int i = order[s];
    TaskDesc &d = t->tasks[s];
    const int lev = d.level;
    const LevelDesc &L = t->levels.lv[lev];
    if (nrad_of[s] >= 0) {
      d.sphere = sphere_of[lev][nrad_of[s]];
      const SphereHdr &h = t->sph[d.sphere];
      for (int k = 0; k < 3; k++)
        if (L.npts_global[k] != L.npts_local[k]) { // grid_ref_collint.h:247-255
          const int off = imod(d.center[k] + h.lb[k] - L.shift[k], L.npts_global[k]) - h.lb[k];
          if (!(off + 1 - h.lb[k] < L.npts_local[k] && off + h.lb[k] >= 0))
            fail("task %d: cube does not fit into the local grid of level %d", i, lev);
        }
      t->points[s] = sphere_points[d.sphere];
      t->features[(size_t)s * 6 + 3] = (float)h.cmax;
    }
    const int p = s > 0 ? order[s - 1] : -1;
    new_sub[s] = s == 0 || block_num_list[p] != block_num_list[i] || iset_list[p] != iset_list[i] ||
                 jset_list[p] != jset_list[i];
  });
  hp.mark("tasks placed");
  // the subblocks: their descriptors in parallel, then the Cartesian scratch
  // offsets (a running sum) and the buffer and scratch maxima in order
  std::vector<int> sub_first;
  for (int s = 0; s < ntasks; s++)
    if (new_sub[s])
      sub_first.push_back(s);
  const int nsub = (int)sub_first.size();
  t->subs.assign(nsub, SubblockDesc{});
  std::vector<long long> block_end(nsub);
  parallel_for(nsub, [&](int u) {
    const int s = sub_first[u];
    const int i = order[s];
    const TaskDesc &d = t->tasks[s];
    const int ia = d.iatom, ja = d.jatom;
    const int iset = iset_list[i] - 1, jset = jset_list[i] - 1;
    const grid_basis_set *bi = basis_sets[atom_kinds[ia] - 1];
    const grid_basis_set *bj = basis_sets[atom_kinds[ja] - 1];
    const int bn = block_num_list[i] - 1;
    SubblockDesc &sb = t->subs[u];
    memset(&sb, 0, sizeof(sb));
    sb.block_offset = block_offsets[bn];
    sb.ncoa = bi->npgf[iset] * ncoset(bi->lmax[iset]);
    sb.ncob = bj->npgf[jset] * ncoset(bj->lmax[jset]);
    sb.nsgf_seta = bi->nsgf_set[iset];
    sb.nsgf_setb = bj->nsgf_set[jset];
    sb.sgfa = bi->first_sgf[iset] - 1;
    sb.sgfb = bj->first_sgf[jset] - 1;
    sb.nsgfa = bi->nsgf;
    sb.nsgfb = bj->nsgf;
    sb.maxcoa = bi->maxco;
    sb.maxcob = bj->maxco;
    sb.sphia = (int)(sphi_off[atom_kinds[ia] - 1] + (long long)sb.sgfa * bi->maxco);
    sb.sphib = (int)(sphi_off[atom_kinds[ja] - 1] + (long long)sb.sgfb * bj->maxco);
    sb.transpose = ia <= ja;
    sb.identity = sphi_identity[atom_kinds[ia] - 1][iset] && sphi_identity[atom_kinds[ja] - 1][jset];
    sb.iatom = ia;
    sb.jatom = ja;
    sb.first_task = s;
    block_end[u] = (long long)block_offsets[bn] + (long long)bi->nsgf * bj->nsgf;
  });
  long long maxbuf = 0;
  for (int u = 0; u < nsub; u++) {
    SubblockDesc &sb = t->subs[u];
    sb.cart_offset = (int)t->cart_total;
    t->cart_total += (size_t)sb.ncoa * sb.ncob;
    if (t->cart_total > (size_t)INT32_MAX)
      fail("Cartesian scratch exceeds int offsets");
    t->contract_words = std::max(t->contract_words, sb.nsgf_setb * sb.ncoa);
    maxbuf = std::max(maxbuf, block_end[u]);
  }
  sub_first.push_back(ntasks);
  parallel_for((int)t->subs.size(), [&](int u) {
    t->subs[u].ntasks = sub_first[u + 1] - sub_first[u];
    for (int s = sub_first[u]; s < sub_first[u + 1]; s++)
      t->tasks[s].subblock = u;
  });
  t->buffer_len = maxbuf;
  hp.mark("spheres and subblocks");
  if (host_only) // grid_gb300_host_digest: the host preparation alone
    return t;
  // ---- upload
  CK(cudaStreamCreateWithFlags(&t->stream, cudaStreamNonBlocking));
  for (auto &e : t->ev)
    CK(cudaEventCreate(&e));
  t->d_tasks = dalloc_copy(t->tasks);
  CK(cudaMalloc((void **)&t->d_seeds, sizeof(float2) * 18 * (size_t)ntasks));
  t->d_subs = dalloc_copy(t->subs);
  t->d_sph = dalloc_copy(t->sph);
  t->d_sph_tab = dalloc_copy(t->sph_tab);
  t->d_sph_pts = dalloc_copy(t->sph_pts);
  {
    std::vector<double> dt;
    build_dh_table(t->levels, dt);
    t->d_dhtab = dalloc_copy(dt);
    std::vector<float> df(dt.size());
    std::vector<float2> dd(dt.size());
    for (size_t k = 0; k < dt.size(); k++) {
      df[k] = (float)dt[k];
      dd[k] = make_float2(df[k], (float)(dt[k] - (double)df[k]));
    }
    t->d_dhtab_f = dalloc_copy(df);
    t->d_dhtab_df = dalloc_copy(dd);
  }
  t->d_sph_ploff = dalloc_copy(t->sph_ploff);
  t->d_atom_pos = dalloc_copy(std::vector<double>(atom_positions, atom_positions + 3 * natoms));
  t->d_sphi = dalloc_copy(sphi_all);
  CK(cudaMalloc((void **)&t->d_levels, sizeof(LevelSet)));
  CK(cudaMemcpy(t->d_levels, &t->levels, sizeof(LevelSet), cudaMemcpyHostToDevice));
  seeds_kernel<<<(unsigned)std::min<long long>((ntasks + 255) / 256, 152LL * 16), 256, 0,
                 t->stream>>>(t->d_tasks, ntasks, t->d_levels, t->d_seeds);
  count_launch();
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(t->stream));
  CK(cudaMalloc((void **)&t->d_pab_cart, sizeof(double) * std::max<size_t>(t->cart_total, 1)));
  CK(cudaMalloc((void **)&t->d_hab_cart, sizeof(double) * std::max<size_t>(t->cart_total, 1)));
  CK(cudaMalloc((void **)&t->d_forces, sizeof(double) * 3 * std::max(natoms, 1)));
  CK(cudaMalloc((void **)&t->d_virial, sizeof(double) * 9));
  CK(cudaMalloc((void **)&t->d_counters, sizeof(int) * kMaxQueues));
  CK(cudaMalloc((void **)&t->d_error, sizeof(int)));
  CK(cudaMemset(t->d_error, 0, sizeof(int)));
  hp.mark("uploaded");
  return t;
}

} // namespace gb300

namespace gb300 {

// frees a mode's work queues and their device arrays
static void release_queues(Mode &m) {
  if (m.d_core_r2)
    cudaFree(m.d_core_r2);
  m.d_core_r2 = nullptr;
  if (m.d_qidx)
    cudaFree(m.d_qidx);
  if (m.d_qitems)
    cudaFree(m.d_qitems);
  m.d_qidx = nullptr;
  m.d_qitems = nullptr;
  m.queues.clear();
  for (int *p : m.d_chunk_idx)
    if (p)
      cudaFree(p);
  m.d_chunk_idx.clear();
  m.chunk_n.clear();
  m.core_r2.clear();
  m.row_split = false;
}

// phase 0 collocate, 1 integrate, 2 integrate with tau
static Mode &get_mode(TaskList *t, const LDiffs &d, int phase, int nch = 1) {
  // one mode per (l shifts, precision, phase, copy chunks): switching the
  // precision back and forth reuses the queues built for each; with nch > 1
  // (host-buffer calls, t->chunks) every queue holds the tasks of one chunk
  const int key = ((mode_key(d) * 4 + t->precision) * 3 + phase) * 8 + nch;
  // derivatives of the Gaussians (derivative densities; the gradients of tau;
  // the forces and virial of an integration) multiply the contributions by up
  // to (2 zeta + l + 1) per unit of angular-momentum shift, with cancellation
  // in the sums; the FP32 class then uses the bound scaled by that factor
  const int dshift = phase == 0 ? d.la_max + d.lb_max : phase == 2 ? 2 : d.la_max;
  auto it = t->modes.find(key);
  if (it != t->modes.end() && it->second.sched_version == t->sched_version)
    return it->second;
  const HostPhases hp("work queues");
  Mode &m = t->modes[key];
  m.d = d;
  if (m.d_coef_off == nullptr) {
    m.coef_off.resize(t->ntasks);
    size_t off = 0;
    for (int s = 0; s < t->ntasks; s++) {
      const TaskDesc &k = t->tasks[s];
      const int la = k.la_max + d.la_max, lb = k.lb_max + d.lb_max;
      m.coef_off[s] = (int)off;
      if (!(k.flags & TF_SKIP))
        off += ncoset(la + lb);
      if (off > (size_t)INT32_MAX)
        fail("coefficient buffer exceeds int offsets");
    }
    m.coef_total = off;
    m.d_coef_off = dalloc_copy(m.coef_off);
  }
  {
    // shared memory of the coefficient / post kernels (depends on the
    // transform variant, so it is redone whenever the mode is rebuilt)
    // per (la, lb): the words depend on the task's l only
    int words = 4;
    bool seen[GB300_LMAX + 8][GB300_LMAX + 8] = {};
    for (int s = 0; s < t->ntasks; s++) {
      const TaskDesc &k = t->tasks[s];
      if (k.flags & TF_SKIP)
        continue;
      const int la = k.la_max + d.la_max, lb = k.lb_max + d.lb_max;
      if (seen[la][lb])
        continue;
      seen[la][lb] = true;
      // collocate: the coefficient kernel (forward); integrate: the post kernel
      words = std::max(words, (int)coef_words(la, lb, uses_staged(t->transform_variant, la, lb,
                                                                  phase == 0)));
    }
    m.coef_words = words;
    m.transform = t->transform_variant;
  }
  m.qsig = std::make_tuple(mode_key(d), t->precision, dshift, nch);
  // a mode of the other phase built under the same settings has the same
  // queues: copy them on the device instead of building them again
  for (auto &kv : t->modes) {
    const Mode &o = kv.second;
    if (&o == &m || o.sched_version != t->sched_version || o.qsig != m.qsig || !o.d_qidx)
      continue;
    release_queues(m);
    m.core_r2 = o.core_r2;
    m.row_split = o.row_split;
    m.d_core_r2 = o.row_split ? dalloc_copy(m.core_r2) : nullptr;
    size_t nidx = 0, nitems = 0;
    for (const Queue &q : o.queues) {
      nidx += (size_t)q.n;
      nitems += q.d_items ? (size_t)q.nitems : 0;
    }
    CK(cudaMalloc((void **)&m.d_qidx, sizeof(int) * std::max<size_t>(nidx, 1)));
    CK(cudaMemcpy(m.d_qidx, o.d_qidx, sizeof(int) * nidx, cudaMemcpyDeviceToDevice));
    if (nitems) {
      CK(cudaMalloc((void **)&m.d_qitems, sizeof(int2) * nitems));
      CK(cudaMemcpy(m.d_qitems, o.d_qitems, sizeof(int2) * nitems, cudaMemcpyDeviceToDevice));
    }
    m.queues = o.queues;
    for (Queue &q : m.queues) {
      q.d_idx = m.d_qidx + (q.d_idx - o.d_qidx);
      q.d_items = q.d_items ? m.d_qitems + (q.d_items - o.d_qitems) : nullptr;
    }
    m.chunk_n = o.chunk_n;
    for (size_t c = 0; c < o.d_chunk_idx.size(); c++) {
      int *p = nullptr;
      if (o.d_chunk_idx[c]) {
        CK(cudaMalloc((void **)&p, sizeof(int) * (size_t)o.chunk_n[c]));
        CK(cudaMemcpy(p, o.d_chunk_idx[c], sizeof(int) * (size_t)o.chunk_n[c],
                      cudaMemcpyDeviceToDevice));
      }
      m.d_chunk_idx.push_back(p);
    }
    m.sched_version = t->sched_version;
    t->gen++;
    hp.mark("queues copied from the other phase");
    return m;
  }
  // row split (mixed mode, orthorhombic double-float tasks): the radius of
  // the double-float core per task, with the class test's derivative factor
  const bool split_rows = t->precision == GRID_GB300_MIXED && t->row_split;
  // the radii depend on the l shifts, the derivative factor and the
  // threshold only: a collocation and an integration without forces share
  // them, so they are kept per list
  const auto core_key = std::make_tuple(d.la_max, d.lb_max, dshift, t->mixed_threshold);
  auto cached = split_rows ? t->core_cache.find(core_key) : t->core_cache.end();
  const bool have_core = cached != t->core_cache.end();
  if (have_core) {
    m.core_r2 = cached->second.first;
  } else {
    m.core_r2.assign(t->ntasks, kCoreAll);
  }
  std::vector<double> outside =
      have_core ? cached->second.second : std::vector<double>(t->ntasks, 0.0);
  if (split_rows && !have_core)
    parallel_for(t->ntasks, [&](int s) {
      const TaskDesc &k = t->tasks[s];
      // general-path tasks stay whole: their kernels' cost is dominated by
      // per-row set-up (the ellipsoid's row bounds), which a second pass
      // repeats (measured on the triclinic workload: collocation 5.9 ms
      // whole, 7.4 ms split)
      if ((k.flags & (TF_SKIP | TF_GENERAL)) != 0)
        return;
      double fac = 1.0;
      if (dshift > 0)
        fac = pow(2.0 * std::max(k.zeta, k.zetb) + std::max(k.la_max, k.lb_max) + 1.0, dshift);
      if (t->gbound[s] * fac <= t->mixed_threshold)
        return; // FP32 class already
      m.core_r2[s] = core_radius2(k, d.la_max, d.lb_max, t->mixed_threshold / (fac * kShellMargin),
                                  &outside[s]);
    });
  if (split_rows && !have_core)
    t->core_cache[core_key] = std::make_pair(m.core_r2, outside);
  hp.mark("coefficient offsets, row split radii");
  m.row_split = false;
  // work queues: (general, lp bucket, FP32 class, size class), descending
  // cost; the outside rows of split tasks in shell queues keyed from
  // kQueueKeys on
  std::map<int, std::vector<std::pair<double, int>>> items;
  std::vector<char> task_cls(t->ntasks, -1); // FP32 class, -1: skipped
  std::vector<int> task_key(t->ntasks, -1);
  std::vector<double> task_cost(t->ntasks, 0.0);
  // what the queue build reads per task, in compact arrays (the queues visit
  // the tasks in cost order): lp, cube width or j range, i range, planes
  std::vector<int> task_lp(t->ntasks, 0), task_ext(t->ntasks, 0), task_iw(t->ntasks, 0),
      task_nk(t->ntasks, 0);
  parallel_for(t->ntasks, [&](int s) {
    const TaskDesc &k = t->tasks[s];
    if (k.flags & TF_SKIP)
      return;
    const int lp = k.la_max + d.la_max + k.lb_max + d.lb_max;
    const int b = bucket_of(lp);
    if (b < 0)
      fail("contraction order lp=%d exceeds %d", lp, GB300_LP_MAX);
    const int g = (k.flags & TF_GENERAL) ? 1 : 0;
    double gb = t->gbound[s];
    if (dshift > 0)
      gb *= pow(2.0 * std::max(k.zeta, k.zetb) + std::max(k.la_max, k.lb_max) + 1.0, dshift);
    const int cls = (t->precision == GRID_GB300_MIXED && gb <= t->mixed_threshold) ? 1 : 0;
    const int ext = g == 0 ? 2 * t->sph[k.sphere].cmax + 2 : k.imax[1] - k.center[1] + 1;
    const int sz = ext <= t->small_extent[t->precision] ? 0 : 1;
    double cost;
    if (t->schedule == GRID_GB300_SCHEDULE_INPUT)
      cost = -(double)k.orig;
    else if (t->schedule == GRID_GB300_SCHEDULE_MODEL && !t->model_cost.empty()) {
      // predicted log time, quantised into bins; inside a bin the size order
      // keeps tasks of one sphere together (their point lists stay in cache)
      const double size = (double)t->points[s] * (lp + 1) + 64.0 * (lp + 1) * (lp + 2);
      const double bin = t->model_bin > 0.0 ? floor(t->model_cost[s] / t->model_bin)
                                            : (double)t->model_cost[s];
      cost = t->model_bin > 0.0 ? bin + size / (size + 1.0e12) : bin;
    } else
      cost = (double)t->points[s] * (lp + 1) + 64.0 * (lp + 1) * (lp + 2);
    task_cls[s] = (char)cls;
    task_key[s] = ((g * kNumBuckets + b) * 2 + cls) * 2 + sz;
    task_cost[s] = cost;
    task_lp[s] = lp;
    task_ext[s] = ext;
    task_iw[s] = g ? k.imax[0] - k.center[0] + 1 : 0;
    task_nk[s] = g ? k.imax[2] - k.center[2] + 1 : 2 - 2 * t->sph[k.sphere].lb[2];
  });
  {
    // filled per thread over contiguous task ranges, then joined: the
    // queue sort below orders its items totally, so the join order is free
    const int nt = std::max(1, std::min(host_threads(), t->ntasks / 4096 + 1));
    std::vector<std::map<int, std::vector<std::pair<double, int>>>> part(nt);
    std::vector<char> split_any(nt, 0);
    std::vector<std::thread> th;
    for (int c = 0; c < nt; c++)
      th.emplace_back([&, c] {
        const int s0 = (int)((long long)t->ntasks * c / nt);
        const int s1 = (int)((long long)t->ntasks * (c + 1) / nt);
        auto &its = part[c];
        for (int s = s0; s < s1; s++) {
          const int key = task_key[s];
          if (key < 0)
            continue;
          const double cost = task_cost[s];
          if (m.core_r2[s] < kCoreAll) {
            const double out = outside[s];
            its[key].push_back({cost * (1.0 - out), s});
            its[kQueueKeys + key + 2].push_back({cost * out, s}); // FP32 class bit set
            split_any[c] = 1;
          } else {
            its[key].push_back({cost, s});
          }
        }
      });
    for (auto &x : th)
      x.join();
    for (int c = 0; c < nt; c++) {
      for (auto &kv : part[c]) {
        auto &dst = items[kv.first];
        dst.insert(dst.end(), kv.second.begin(), kv.second.end());
      }
      m.row_split = m.row_split || split_any[c];
    }
  }
  hp.mark("classes and costs");
  {
    const bool split_any = m.row_split;
    std::vector<float> r2;
    r2.swap(m.core_r2);
    release_queues(m);
    m.core_r2.swap(r2);
    m.row_split = split_any;
  }
  m.d_core_r2 = m.row_split ? dalloc_copy(m.core_r2) : nullptr;
  if (nch > 1) {
    // tasks are in subblock order: chunk c's tasks are those of its subblocks
    for (int c = 0; c < nch; c++) {
      const int sa = t->chunks.sub_lo[c], sb = t->chunks.sub_lo[c + 1];
      const int t0 = sa < (int)t->subs.size() ? t->subs[sa].first_task : t->ntasks;
      const int t1 = sb < (int)t->subs.size() ? t->subs[sb].first_task : t->ntasks;
      for (int cls = 0; cls < 2; cls++) {
        std::vector<int> idx;
        for (int s = t0; s < t1; s++)
          if (task_cls[s] == cls)
            idx.push_back(s);
        m.chunk_n.push_back((int)idx.size());
        m.d_chunk_idx.push_back(idx.empty() ? nullptr : dalloc_copy(idx));
      }
    }
  }
  // host-buffer calls: each copy chunk gets queues of its own tasks, so that
  // a chunk's grid kernels run while the next chunk is copied
  std::vector<int> chunk_of;
  if (nch > 1) {
    chunk_of.assign(t->ntasks, 0);
    for (int c = 0; c < nch; c++) {
      const int sa = t->chunks.sub_lo[c], sb = t->chunks.sub_lo[c + 1];
      const int t0 = sa < (int)t->subs.size() ? t->subs[sa].first_task : t->ntasks;
      const int t1 = sb < (int)t->subs.size() ? t->subs[sb].first_task : t->ntasks;
      for (int s = t0; s < t1; s++)
        chunk_of[s] = c;
    }
  }
  // heavier classes first: large cubes, then the arithmetic of the mode, FP32 last
  std::vector<int> keys;
  for (auto &kv : items)
    keys.push_back(kv.first);
  std::stable_sort(keys.begin(), keys.end(), [](int x, int y) {
    const int cx = (x >> 1) & 1, cy = (y >> 1) & 1, sx = x & 1, sy = y & 1;
    if (cx != cy)
      return cx < cy;
    if (sx != sy)
      return sx > sy;
    return x < y;
  });
  hp.mark("chunk lists");
  // descending cost; ties in task order (the lists are filled in task order,
  // so this is their stable sort by cost)
  for (auto &kv : items)
    parallel_sort(kv.second, [](const std::pair<double, int> &x,
                                const std::pair<double, int> &y) {
      return x.first > y.first || (x.first == y.first && x.second < y.second);
    });
  hp.mark("queue items sorted");
  // the queues in launch order, each built on its own thread; their task
  // indices and work items then go to the device in one piece each
  struct QueueBuild {
    Queue q;
    std::vector<std::pair<double, int>> v;
    std::vector<int> idx;
    std::vector<int2> items;
  };
  std::vector<QueueBuild> qb;
  for (int qc = 0; qc < (nch > 1 ? nch : 1); qc++)
    for (int key : keys) {
      QueueBuild b;
      if (nch > 1) {
        for (const auto &e : items[key])
          if (chunk_of[e.second] == qc)
            b.v.push_back(e);
        if (b.v.empty())
          continue;
      } else {
        b.v.swap(items[key]);
      }
      b.q.chunk = qc;
      b.q.key = key;
      qb.push_back(std::move(b));
    }
  parallel_items((int)qb.size(), [&](int n) {
    QueueBuild &b = qb[n];
    Queue &q = b.q;
    const int key = q.key;
    const std::vector<std::pair<double, int>> &v = b.v;
    q.base = key; // shell queues tune apart from the FP32 class's
    const int kb = key % kQueueKeys;
    q.general = kb / (2 * 2 * kNumBuckets);
    q.bucket = (kb / 4) % kNumBuckets;
    q.fp32 = (kb >> 1) & 1;
    std::vector<int> &idx = b.idx;
    idx.resize(v.size());
    int ext = 1;
    for (size_t i = 0; i < v.size(); i++) {
      const int ts = v[i].second;
      idx[i] = ts;
      long long pts = t->points[ts]; // of the task's points in this queue
      if (m.core_r2[ts] < kCoreAll) { // estimated split, the two parts adding up
        q.side = key >= kQueueKeys ? 2 : 1;
        const long long in = llround((1.0 - outside[ts]) * (double)pts);
        pts = key >= kQueueKeys ? pts - in : in;
      }
      q.points += pts;
      q.flops += 2.0 * (task_lp[ts] + 1) * (double)pts;
      ext = std::max(ext, task_ext[ts]);
      if (q.general)
        q.iwidth = std::max(q.iwidth, task_iw[ts]);
    }
    q.n = (int)idx.size();
    q.extent = ext;
    // Large tasks are split by planes into several work items, so that a
    // few of them do not keep single warps busy while the GPU idles.
    // General path: boxes of more than kSlicePoints points, in items of at
    // least kSlicePlanes planes.  Orthorhombic path: tasks of more than
    // twice the queue's balanced share per resident warp, in items of half
    // that share (at least kOrthoSliceMin points and two planes).
    const double share = (double)q.points / kNominalWarps;
    const long long target = std::max<long long>(kOrthoSliceMin, (long long)(0.5 * share));
    std::vector<int2> &wi = b.items;
    bool split = false;
    for (int s : idx) {
      const int nk = task_nk[s];
      int ns;
      if (q.general) {
        const long long by_pts = (t->points[s] + kSlicePoints - 1) / kSlicePoints;
        ns = (int)std::max<long long>(
            1, std::min<long long>(by_pts, (nk + kSlicePlanes - 1) / kSlicePlanes));
      } else {
        ns = 1;
        if (t->points[s] > 2 * target)
          ns = (int)std::min<long long>(nk / 2, (t->points[s] + target - 1) / target);
        ns = std::max(ns, 1);
      }
      split |= ns > 1;
      for (int c = 0; c < ns; c++) {
        const int k0 = (int)((long long)nk * c / ns), k1 = (int)((long long)nk * (c + 1) / ns);
        wi.push_back(make_int2(s, k0 | ((k1 - k0) << 16)));
      }
    }
    if (split)
      q.nitems = (int)wi.size();
    else
      wi.clear();
  });
  {
    size_t nidx = 0, nitems = 0;
    for (const QueueBuild &b : qb) {
      nidx += b.idx.size();
      nitems += b.items.size();
    }
    std::vector<int> all_idx;
    std::vector<int2> all_items;
    all_idx.reserve(nidx);
    all_items.reserve(nitems);
    for (const QueueBuild &b : qb) {
      all_idx.insert(all_idx.end(), b.idx.begin(), b.idx.end());
      all_items.insert(all_items.end(), b.items.begin(), b.items.end());
    }
    m.d_qidx = dalloc_copy(all_idx);
    m.d_qitems = nitems ? dalloc_copy(all_items) : nullptr;
    size_t oi = 0, ow = 0;
    for (QueueBuild &b : qb) {
      b.q.d_idx = m.d_qidx + oi;
      oi += b.idx.size();
      b.q.d_items = nullptr;
      if (b.q.nitems > 0) {
        b.q.d_items = m.d_qitems + ow;
        ow += b.items.size();
      }
      m.queues.push_back(b.q);
    }
  }
  m.sched_version = t->sched_version;
  t->gen++;
  hp.mark("queues sorted, split and uploaded");
  return m;
}

// returns 1 when the buffer was (re)allocated
static int ensure(void **p, size_t *cap, size_t bytes) {
  if (*cap >= bytes && *p)
    return 0;
  if (*p)
    CK(cudaFree(*p));
  CK(cudaMalloc(p, std::max<size_t>(bytes, 16)));
  *cap = bytes;
  return 1;
}

static void check_device_error(TaskList *t) {
  if (const char *m = take_launch_error())
    fail("%s", m);
  int err = 0;
  CK(cudaMemcpy(&err, t->d_error, sizeof(int), cudaMemcpyDeviceToHost));
  if (err)
    fail("grid kernel reported error code %d (work item exceeded its shared-memory sizing)", err);
}

static double ev_ms(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  return ms;
}

static void read_timings(TaskList *t) {
  CK(cudaEventSynchronize(t->ev[3]));
  t->timings[0] = ev_ms(t->ev[0], t->ev[1]);
  t->timings[1] = ev_ms(t->ev[1], t->ev[2]);
  t->timings[2] = ev_ms(t->ev[2], t->ev[3]);
  t->timings[3] = ev_ms(t->ev[0], t->ev[3]);
}

static void record_phase(TaskList *t, int i, cudaStream_t s) {
  if (!t->capturing)
    CK(cudaEventRecord(t->ev[i], s));
}

static cudaEvent_t pool_event(TaskList *t, size_t i) {
  while (t->event_pool.size() <= i) {
    cudaEvent_t e;
    CK(cudaEventCreate(&e));
    t->event_pool.push_back(e);
  }
  return t->event_pool[i];
}

// one persistent grid-kernel launch of a work queue, with its tuned launch
// shape and (optionally) CUDA events around it
static void grid_launch(TaskList *t, const Queue &q, int phase, int arith, const GridArgs &ga,
                        cudaStream_t s) {
  LaunchCfg cfg;
  // automatic: on the orthorhombic path the point-list kernel pays off where
  // the per-point arithmetic is expensive (FP64, double-float), the row walk
  // for plain FP32; on the general path (box around the sphere) the point
  // list wins in every arithmetic that has one (FP32, double-float)
  cfg.variant = t->coll_variant >= 0 ? t->coll_variant : ((q.general || arith != ARITH_FP32) ? 1 : 0);
  auto it = t->tuned.find(std::make_tuple(t->precision, phase, q.base));
  if (it != t->tuned.end())
    cfg = it->second;
  cfg.tensor = t->tc_integrate;
  // the tensor-core collocation keeps about 21 bits per product: the mixed
  // mode's FP32 class (contributions bounded by the threshold) takes it,
  // plain FP32 mode keeps the CUDA-core kernels' 24
  cfg.tensor_coll = t->tc_collocate && t->precision == GRID_GB300_MIXED;
  LaunchRecord rec;
  const bool timed = t->launch_timing && !t->capturing;
  if (timed) {
    rec.a = pool_event(t, 2 * t->launches.size());
    rec.b = pool_event(t, 2 * t->launches.size() + 1);
    CK(cudaEventRecord(rec.a, s));
  }
  if (phase == 0)
    launch_collocate(ga, arith, q.general == 1, q.bucket, q.extent, cfg, s);
  else
    launch_integrate(ga, arith, q.general == 1, q.bucket, q.extent, cfg, s);
  if (timed) {
    CK(cudaEventRecord(rec.b, s));
    grid_gb300_launch_info &in = rec.info;
    in.phase = phase;
    in.precision = arith;
    in.general = q.general;
    in.lp_bucket = kBucketLp[q.bucket];
    in.ntasks = q.n;
    in.work_items = q.d_items ? q.nitems : q.n;
    in.warps_per_block = cfg.warps;
    in.blocks = cfg.blocks;
    in.points = q.points;
    in.flops = q.flops;
    in.ms = 0.0;
    rec.key = q.base;
    t->launches.push_back(rec);
  }
}

// Grid launches of one phase are independent (each its own tasks and work
// counter; the grids take atomic adds): with two queue streams they
// alternate between the caller's stream and an auxiliary one, forked from
// and joined back into the caller's stream around the phase.  Per-launch
// timing keeps them on one stream.
static bool two_queue_streams(const TaskList *t) {
  return t->queue_streams > 1 && !t->launch_timing;
}
static void fork_queues(TaskList *t, cudaStream_t s) {
  if (!two_queue_streams(t))
    return;
  if (!t->aux_stream) {
    CK(cudaStreamCreateWithFlags(&t->aux_stream, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&t->fork_ev, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&t->join_ev, cudaEventDisableTiming));
  }
  CK(cudaEventRecord(t->fork_ev, s));
  CK(cudaStreamWaitEvent(t->aux_stream, t->fork_ev, 0));
}
static cudaStream_t queue_stream(const TaskList *t, cudaStream_t s, int i) {
  return (two_queue_streams(t) && (i & 1)) ? t->aux_stream : s;
}
static void join_queues(TaskList *t, cudaStream_t s) {
  if (!two_queue_streams(t))
    return;
  CK(cudaEventRecord(t->join_ev, t->aux_stream));
  CK(cudaStreamWaitEvent(s, t->join_ev, 0));
}

static void begin_call(TaskList *t, cudaStream_t s) {
  if (!t->capturing)
    t->launches.clear();
  if (t->task_timing) {
    if (!t->d_cycles) {
      CK(cudaMalloc((void **)&t->d_cycles, sizeof(long long) * std::max(t->ntasks, 1)));
      t->gen++;
    }
    CK(cudaMemsetAsync(t->d_cycles, 0, sizeof(long long) * std::max(t->ntasks, 1), s));
  }
}

// Host-buffer calls: the copies of one call run on the list's copy stream in
// the pieces of a CopyChunks, overlapping the kernels of earlier pieces.
struct HostCopy {
  const CopyChunks *ch = nullptr;
  cudaStream_t cs = nullptr;       // copy stream
  const cudaEvent_t *ready = nullptr;  // collocate: pab chunk c is on the device
  const cudaEvent_t *vready = nullptr; // integrate: V of level l is on the device
  cudaEvent_t pab_ready = nullptr;     // integrate: pab (forces / virial) is on the device
  const cudaEvent_t *done = nullptr;   // integrate: hab chunk c is final on the device
  double *hab_host = nullptr;          // integrate: where hab chunk c goes
};

static void run_collocate(TaskList *t, int func, const double *pab, double *const *grids,
                          cudaStream_t s, const HostCopy *hc = nullptr) {
  const LDiffs d = func_ldiffs(func);
  const int nch = hc ? hc->ch->n : 1;
  Mode &m = get_mode(t, d, 0, nch);
  const int arith = t->precision;
  t->gen += ensure(&t->d_coef, &t->coef_cap, m.coef_total * (arith == ARITH_FP32 ? 4 : 8));
  begin_call(t, s);
  record_phase(t, 0, s);
  // the grids are overwritten (grid_ref_task_list.c:418-424)
  for (int l = 0; l < t->nlevels; l++) {
    const int *n = &t->npts_local[3 * l];
    const size_t np = (size_t)n[0] * n[1] * n[2];
    CK(cudaMemsetAsync(grids[l], 0, sizeof(double) * np, s));
    if (arith == ARITH_MIXED) {
      if (!t->d_gridlo[l]) {
        CK(cudaMalloc((void **)&t->d_gridlo[l], sizeof(float) * np));
        t->gen++;
      }
      CK(cudaMemsetAsync(t->d_gridlo[l], 0, sizeof(float) * np, s));
    }
  }
  CK(cudaMemsetAsync(t->d_counters, 0, sizeof(int) * kMaxQueues, s));
  CoefArgs co{};
  co.tasks = t->d_tasks;
  co.subs = t->d_subs;
  co.coef_off = m.d_coef_off;
  co.atom_pos = t->d_atom_pos;
  co.pab_cart = t->d_pab_cart;
  co.coef = t->d_coef;
  co.ntasks = t->ntasks;
  co.func = func;
  co.d = d;
  co.levels = t->d_levels;
  co.dhtab = t->d_dhtab;
  co.dhtab_f = t->d_dhtab_f;
  co.dhtab_df = t->d_dhtab_df;
  co.transform = m.transform;
  GridArgs ga{};
  ga.coef_stride = 1;
  ga.grid_stride = 1;
  ga.tasks = t->d_tasks;
  ga.coef_off = m.d_coef_off;
  ga.coef = t->d_coef;
  ga.sph = t->d_sph;
  ga.sph_tab = t->d_sph_tab;
  ga.sph_pts = t->d_sph_pts;
  ga.sph_ploff = t->d_sph_ploff;
  for (int l = 0; l < t->nlevels; l++) {
    ga.grids[l] = grids[l];
    ga.grids_lo[l] = t->d_gridlo[l];
  }
  ga.levels = t->levels;
  ga.d = d;
  ga.task_cycles = t->task_timing ? t->d_cycles : nullptr;
  ga.seeds = t->d_seeds;
  ga.error = t->d_error;
  int qi = 0;
  auto launch_queues = [&](int chunk) {
    fork_queues(t, s);
    for (const Queue &q : m.queues) {
      if (chunk >= 0 && q.chunk != chunk)
        continue;
      ga.queue = q.d_idx;
      ga.items = q.d_items;
      ga.iwidth = q.iwidth;
      ga.nqueue = q.d_items ? q.nitems : q.n;
      if (qi >= kMaxQueues)
        fail("more than %d work queues in one call", kMaxQueues);
      ga.counter = t->d_counters + qi++;
      // FP32 queues read the high words of the coefficient slots (shell
      // queues: of the split tasks' double-float coefficients)
      ga.coef_stride = q.fp32 ? 2 : 1;
      ga.core_side = q.side;
      ga.core_r2 = q.side ? m.d_core_r2 : nullptr;
      grid_launch(t, q, 0, q.fp32 ? (int)ARITH_FP32 : arith, ga, queue_stream(t, s, qi));
      if (q.side != 2)
        grid_library_counter_add(kBucketLp[q.bucket], GRID_BACKEND_GB300,
                                 q.general ? GRID_COLLOCATE_GENERAL : GRID_COLLOCATE_ORTHO, q.n);
    }
    join_queues(t, s);
  };
  // pab -> Cartesian -> coefficients, piece by piece where the host-buffer
  // call copies pab in pieces (each waits for its piece only); there each
  // piece's grid kernels follow its coefficients, while the next piece is
  // still being copied
  for (int c = 0; c < nch; c++) {
    int s0 = 0, ns = (int)t->subs.size();
    if (hc) { // this piece of pab is on the device
      CK(cudaStreamWaitEvent(s, hc->ready[c], 0));
      s0 = hc->ch->sub_lo[c];
      ns = hc->ch->sub_lo[c + 1] - s0;
    }
    ContractArgs ca{t->d_subs + s0, ns, t->d_sphi, pab, nullptr, t->d_pab_cart,
                    t->contract_words};
    launch_decontract(ca, s);
    if (nch > 1) {
      for (int cls = 0; cls < 2; cls++) {
        co.order = m.d_chunk_idx[2 * c + cls];
        co.norder = m.chunk_n[2 * c + cls];
        if (co.norder == 0)
          continue;
        if (arith == ARITH_MIXED)
          launch_coefficients_mixed(co, cls ? (int)ARITH_FP32 : (int)ARITH_MIXED, m.coef_words,
                                    s);
        else
          launch_coefficients(co, arith, m.coef_words, s);
      }
    } else if (arith == ARITH_MIXED) {
      // one launch per work queue, each in the working type of its class: the
      // kernels stay small (instruction cache) and need no per-task branch
      for (const Queue &q : m.queues) {
        if (q.side == 2) // the core queue computes a split task's coefficients
          continue;
        co.order = q.d_idx;
        co.norder = q.n;
        launch_coefficients_mixed(co, q.fp32 ? (int)ARITH_FP32 : (int)ARITH_MIXED, m.coef_words,
                                  s);
      }
    } else {
      launch_coefficients(co, arith, m.coef_words, s);
    }
    if (c == 0)
      record_phase(t, 1, s);
    if (nch > 1)
      launch_queues(c);
  }
  if (nch == 1)
    launch_queues(-1);
  if (arith == ARITH_MIXED)
    for (int l = 0; l < t->nlevels; l++) {
      const int *n = &t->npts_local[3 * l];
      launch_grid_fold_lo(grids[l], t->d_gridlo[l], (size_t)n[0] * n[1] * n[2], s);
    }
  CK(cudaGetLastError());
  record_phase(t, 2, s);
  record_phase(t, 3, s);
}

static void run_integrate(TaskList *t, bool tau, const double *pab, const double *const *grids,
                          double *hab, double *forces, double *virial, cudaStream_t s,
                          const HostCopy *hc = nullptr) {
  const LDiffs d = integrate_ldiffs(forces != nullptr, virial != nullptr, tau);
  const int nch = hc ? hc->ch->n : 1;
  Mode &m = get_mode(t, d, tau ? 2 : 1, nch);
  const int arith = t->precision;
  const bool need_pab = forces != nullptr || virial != nullptr;
  t->gen += ensure((void **)&t->d_coef_int, &t->coef_int_cap, m.coef_total * 8);
  begin_call(t, s);
  record_phase(t, 0, s);
  if (arith != ARITH_FP64)
    for (int l = 0; l < t->nlevels; l++) {
      const int *n = &t->npts_local[3 * l];
      const size_t np = (size_t)n[0] * n[1] * n[2];
      if (!t->d_gridsplit[l]) {
        CK(cudaMalloc(&t->d_gridsplit[l], sizeof(float2) * np));
        t->gen++;
      }
      if (arith == ARITH_MIXED && !t->d_gridhi[l]) {
        CK(cudaMalloc((void **)&t->d_gridhi[l], sizeof(float) * np));
        t->gen++;
      }
      if (hc)
        CK(cudaStreamWaitEvent(s, hc->vready[l], 0));
      launch_grid_split(grids[l], t->d_gridsplit[l], np, arith, s,
                        arith == ARITH_MIXED ? t->d_gridhi[l] : nullptr);
    }
  else if (hc)
    for (int l = 0; l < t->nlevels; l++)
      CK(cudaStreamWaitEvent(s, hc->vready[l], 0));
  if (need_pab) {
    if (hc)
      CK(cudaStreamWaitEvent(s, hc->pab_ready, 0));
    ContractArgs ca{t->d_subs, (int)t->subs.size(), t->d_sphi, pab, nullptr, t->d_pab_cart,
                    t->contract_words};
    launch_decontract(ca, s);
  }
  CK(cudaMemsetAsync(t->d_counters, 0, sizeof(int) * kMaxQueues, s));
  // split general tasks add their planes' partial coefficients
  bool any_split = m.row_split; // split tasks: both sides add their coefficients
  for (const Queue &q : m.queues)
    any_split |= q.d_items != nullptr;
  if (any_split)
    CK(cudaMemsetAsync(t->d_coef_int, 0, m.coef_total * 8, s));
  CK(cudaMemsetAsync(t->d_hab_cart, 0, sizeof(double) * std::max<size_t>(t->cart_total, 1), s));
  if (forces)
    CK(cudaMemsetAsync(forces, 0, sizeof(double) * 3 * t->natoms, s));
  if (virial)
    CK(cudaMemsetAsync(virial, 0, sizeof(double) * 9, s));
  // hab is overwritten (grid_ref_task_list.c:672-678)
  CK(cudaMemsetAsync(hab, 0, sizeof(double) * (size_t)t->buffer_len, s));
  record_phase(t, 1, s);
  GridArgs ga{};
  ga.coef_stride = 1;
  ga.grid_stride = 1;
  ga.tasks = t->d_tasks;
  ga.coef_off = m.d_coef_off;
  ga.coef_out = t->d_coef_int;
  ga.sph = t->d_sph;
  ga.sph_tab = t->d_sph_tab;
  ga.sph_pts = t->d_sph_pts;
  ga.sph_ploff = t->d_sph_ploff;
  ga.levels = t->levels;
  ga.d = d;
  ga.task_cycles = t->task_timing ? t->d_cycles : nullptr;
  ga.seeds = t->d_seeds;
  ga.error = t->d_error;
  PostArgs pa{t->d_tasks, t->d_subs, m.d_coef_off, t->d_coef_int,
              need_pab ? t->d_pab_cart : nullptr, t->d_hab_cart, t->d_atom_pos, forces, virial,
              t->ntasks, tau ? 1 : 0, d, t->d_levels, t->d_dhtab, t->d_dhtab_f, t->d_dhtab_df,
              nullptr, 0, m.transform};
  int qi = 0;
  auto launch_queues = [&](int chunk) {
    fork_queues(t, s);
    for (const Queue &q : m.queues) {
      if (chunk >= 0 && q.chunk != chunk)
        continue;
      ga.queue = q.d_idx;
      ga.items = q.d_items;
      ga.iwidth = q.iwidth;
      ga.nqueue = q.d_items ? q.nitems : q.n;
      if (qi >= kMaxQueues)
        fail("more than %d work queues in one call", kMaxQueues);
      ga.counter = t->d_counters + qi++;
      ga.grid_stride = 1;
      ga.core_side = q.side;
      ga.core_r2 = q.side ? m.d_core_r2 : nullptr;
      ga.accum = q.side != 0;
      // FP64: the grid; mixed: float2 pairs for the double-float class, dense
      // high words for the FP32 class
      for (int l = 0; l < t->nlevels; l++)
        ga.grids_in[l] = arith == ARITH_FP64                  ? (const void *)grids[l]
                         : (arith == ARITH_MIXED && q.fp32) ? (const void *)t->d_gridhi[l]
                                                            : (const void *)t->d_gridsplit[l];
      grid_launch(t, q, 1, q.fp32 ? (int)ARITH_FP32 : arith, ga, queue_stream(t, s, qi));
      if (q.side != 2)
        grid_library_counter_add(kBucketLp[q.bucket], GRID_BACKEND_GB300,
                                 q.general ? GRID_INTEGRATE_GENERAL : GRID_INTEGRATE_ORTHO, q.n);
    }
    join_queues(t, s);
  };
  if (nch == 1) {
    launch_queues(-1);
    record_phase(t, 2, s);
  }
  // integrated coefficients -> hab (forces, virial), piece by piece where the
  // host-buffer call copies hab out in pieces: the largest piece first, so
  // that the copy left after the last kernel is the smallest one; there each
  // piece's grid kernels run first, so that its copy overlaps the next
  // piece's grid kernels
  for (int ci = nch - 1; ci >= 0; ci--) {
    if (nch > 1) {
      launch_queues(ci);
      if (ci == nch - 1)
        record_phase(t, 2, s);
    }
    if (nch > 1) {
      for (int cls = 0; cls < 2; cls++) {
        pa.order = m.d_chunk_idx[2 * ci + cls];
        pa.norder = m.chunk_n[2 * ci + cls];
        if (pa.norder == 0)
          continue;
        if (arith == ARITH_MIXED)
          launch_post_mixed(pa, cls ? (int)ARITH_FP32 : (int)ARITH_MIXED, m.coef_words, s);
        else
          launch_post(pa, arith, m.coef_words, s);
      }
    } else if (arith == ARITH_MIXED) {
      for (const Queue &q : m.queues) {
        if (q.side == 2) // posted with the task's core queue
          continue;
        pa.order = q.d_idx;
        pa.norder = q.n;
        launch_post_mixed(pa, q.fp32 ? (int)ARITH_FP32 : (int)ARITH_MIXED, m.coef_words, s);
      }
    } else {
      launch_post(pa, arith, m.coef_words, s);
    }
    int s0 = 0, ns = (int)t->subs.size();
    if (hc) {
      s0 = hc->ch->sub_lo[ci];
      ns = hc->ch->sub_lo[ci + 1] - s0;
    }
    ContractArgs cb{t->d_subs + s0, ns, t->d_sphi, nullptr, hab, t->d_hab_cart,
                    t->contract_words};
    launch_contract_hab(cb, s);
    if (hc) { // this piece of hab is final: copy it out behind the next kernels
      CK(cudaEventRecord(hc->done[ci], s));
      CK(cudaStreamWaitEvent(hc->cs, hc->done[ci], 0));
      const long long e0 = hc->ch->el_lo[ci], e1 = hc->ch->el_lo[ci + 1];
      if (e1 > e0)
        CK(cudaMemcpyAsync(hc->hab_host + e0, hab + e0, sizeof(double) * (size_t)(e1 - e0),
                           cudaMemcpyDeviceToHost, hc->cs));
    }
  }
  CK(cudaGetLastError());
  record_phase(t, 3, s);
}

static TaskList *TL(const void *p) {
  if (!p)
    fail("null task list");
  return (TaskList *)p;
}

} // namespace gb300

// ===========================================================================
// backend-level entry points
// ===========================================================================
GB300_API void grid_gb300_create_task_list(
    const bool orthorhombic, const int ntasks, const int nlevels, const int natoms,
    const int nkinds, const int nblocks, const int *block_offsets, const double *atom_positions,
    const int *atom_kinds, const grid_basis_set **basis_sets, const int *level_list,
    const int *iatom_list, const int *jatom_list, const int *iset_list, const int *jset_list,
    const int *ipgf_list, const int *jpgf_list, const int *border_mask_list,
    const int *block_num_list, const double *radius_list, const double *rab_list,
    const int *npts_global, const int *npts_local, const int *shift_local,
    const int *border_width, const double *dh, const double *dh_inv,
    grid_gb300_task_list **task_list) {
  // Re-creation through an existing handle (CP2K does this at every change
  // of geometry, src/grid/grid_task_list.c:42-63) keeps the caller's
  // settings: precision, schedule, mixed threshold, collocate variant, model
  // bin width, tuned launch shapes and timing switches.  Per-task data (model
  // predictions, timings) belong to the old geometry and are dropped; the
  // learned schedule falls back to the size order until a model is applied.
  struct Kept {
    int precision, schedule, coll_variant, transform_variant, copy_chunks, queue_streams,
        tc_integrate, tc_collocate, row_split;
    double mixed_threshold, model_bin;
    int small_extent[3];
    std::map<std::tuple<int, int, int>, LaunchCfg> tuned;
    bool launch_timing, task_timing;
  };
  std::unique_ptr<Kept> kept;
  if (*task_list) {
    const TaskList *o = TL(*task_list);
    kept.reset(new Kept{o->precision, o->schedule, o->coll_variant, o->transform_variant,
                        o->copy_chunks, o->queue_streams, o->tc_integrate, o->tc_collocate,
                        o->row_split,
                        o->mixed_threshold,
                        o->model_bin, {o->small_extent[0], o->small_extent[1],
                                       o->small_extent[2]},
                        o->tuned, o->launch_timing, o->task_timing});
    grid_gb300_free_task_list(*task_list);
  }
  TaskList *t = create(orthorhombic, ntasks, nlevels, natoms, nkinds, nblocks, block_offsets,
                       atom_positions, atom_kinds, basis_sets, level_list, iatom_list,
                       jatom_list, iset_list, jset_list, ipgf_list, jpgf_list,
                       border_mask_list, block_num_list, radius_list, rab_list, npts_global,
                       npts_local, shift_local, border_width, dh, dh_inv);
  t->precision = GRID_GB300_FP64;
  t->schedule = GRID_GB300_SCHEDULE_SIZE;
  if (kept) {
    t->precision = kept->precision;
    t->schedule = kept->schedule;
    t->coll_variant = kept->coll_variant;
    t->transform_variant = kept->transform_variant;
    t->copy_chunks = kept->copy_chunks;
    t->queue_streams = kept->queue_streams;
    t->tc_integrate = kept->tc_integrate;
    t->tc_collocate = kept->tc_collocate;
    t->row_split = kept->row_split;
    t->mixed_threshold = kept->mixed_threshold;
    t->model_bin = kept->model_bin;
    for (int i = 0; i < 3; i++)
      t->small_extent[i] = kept->small_extent[i];
    t->tuned = kept->tuned;
    t->launch_timing = kept->launch_timing;
    t->task_timing = kept->task_timing;
  }
  *task_list = t;
}

// FNV-1a over the bytes of a vector of plain structs
template <typename V> static unsigned long long fnv_bytes(const V &v) {
  unsigned long long h = 1469598103934665603ull;
  const unsigned char *p = (const unsigned char *)v.data();
  for (size_t i = 0; i < v.size() * sizeof(v[0]); i++) {
    h ^= p[i];
    h *= 1099511628211ull;
  }
  return h;
}

GB300_API double grid_gb300_row_split_radius2(int la_min, int la_max, int lb_min, int lb_max,
                                              double zeta, double zetb, const double *rab,
                                              double radius, int same_atom, int dla, int dlb,
                                              double tau, double *outside) {
  if (la_min < 0 || la_max < la_min || lb_min < 0 || lb_max < lb_min || la_max > GB300_LMAX ||
      lb_max > GB300_LMAX || !(zeta > 0.0) || !(zetb > 0.0) || !(radius > 0.0) || dla < 0 ||
      dlb < 0)
    fail("grid_gb300_row_split_radius2: invalid arguments");
  TaskDesc d{};
  d.la_min = (int8_t)la_min;
  d.la_max = (int8_t)la_max;
  d.lb_min = (int8_t)lb_min;
  d.lb_max = (int8_t)lb_max;
  d.zeta = zeta;
  d.zetb = zetb;
  d.zetp = zeta + zetb;
  double r2 = 0.0;
  for (int i = 0; i < 3; i++) {
    d.rab[i] = rab[i];
    r2 += rab[i] * rab[i];
  }
  d.prefexp = exp(-zeta * zetb / d.zetp * r2);
  d.radius = radius;
  d.iatom = 0;
  d.jatom = same_atom ? 0 : 1;
  double out = 0.0;
  const float c2 = core_radius2(d, dla, dlb, tau, &out);
  if (outside)
    *outside = out;
  return (double)c2;
}

GB300_API void grid_gb300_host_digest(
    const bool orthorhombic, const int ntasks, const int nlevels, const int natoms,
    const int nkinds, const int nblocks, const int *block_offsets, const double *atom_positions,
    const int *atom_kinds, const grid_basis_set **basis_sets, const int *level_list,
    const int *iatom_list, const int *jatom_list, const int *iset_list, const int *jset_list,
    const int *ipgf_list, const int *jpgf_list, const int *border_mask_list,
    const int *block_num_list, const double *radius_list, const double *rab_list,
    const int *npts_global, const int *npts_local, const int *shift_local,
    const int *border_width, const double *dh, const double *dh_inv,
    unsigned long long digest[12]) {
  TaskList *t = create(orthorhombic, ntasks, nlevels, natoms, nkinds, nblocks, block_offsets,
                       atom_positions, atom_kinds, basis_sets, level_list, iatom_list,
                       jatom_list, iset_list, jset_list, ipgf_list, jpgf_list,
                       border_mask_list, block_num_list, radius_list, rab_list, npts_global,
                       npts_local, shift_local, border_width, dh, dh_inv, true);
  digest[0] = fnv_bytes(t->tasks);
  digest[1] = 0; // the seeds are computed on the device
  digest[2] = fnv_bytes(t->gbound);
  digest[3] = fnv_bytes(t->features);
  digest[4] = fnv_bytes(t->points);
  digest[5] = fnv_bytes(t->subs);
  digest[6] = fnv_bytes(t->sph);
  digest[7] = fnv_bytes(t->sph_tab);
  digest[8] = fnv_bytes(t->sph_pts);
  digest[9] = fnv_bytes(t->sph_ploff);
  digest[10] = (unsigned long long)t->cart_total;
  unsigned long long n32 = 0;
  for (double g : t->gbound)
    n32 += g <= 0.3;
  digest[11] = n32;
  delete t;
}

GB300_API void grid_gb300_free_task_list(grid_gb300_task_list *task_list) {
  if (!task_list)
    return;
  TaskList *t = TL(task_list);
  free_device(t);
  delete t;
}

GB300_API void grid_gb300_collocate_device_async(const grid_gb300_task_list *task_list, int func,
                                                 const double *pab_blocks, double *const *grids,
                                                 void *stream) {
  TaskList *t = TL(task_list);
  cudaStream_t s = (cudaStream_t)stream;
  if (t->empty) {
    for (int l = 0; l < t->nlevels; l++) {
      const int *n = &t->npts_local[3 * l];
      CK(cudaMemsetAsync(grids[l], 0, sizeof(double) * (size_t)n[0] * n[1] * n[2], s));
    }
    return;
  }
  run_collocate(t, func, pab_blocks, grids, s);
}

GB300_API void grid_gb300_integrate_device_async(const grid_gb300_task_list *task_list,
                                                 bool compute_tau, const double *pab_blocks,
                                                 const double *const *grids, double *hab_blocks,
                                                 double *forces, double *virial, void *stream) {
  TaskList *t = TL(task_list);
  cudaStream_t s = (cudaStream_t)stream;
  if ((forces || virial) && !pab_blocks)
    fail("forces and virial require pab_blocks");
  if (t->empty) {
    if (t->buffer_len)
      CK(cudaMemsetAsync(hab_blocks, 0, sizeof(double) * t->buffer_len, s));
    if (forces)
      CK(cudaMemsetAsync(forces, 0, sizeof(double) * 3 * t->natoms, s));
    if (virial)
      CK(cudaMemsetAsync(virial, 0, sizeof(double) * 9, s));
    return;
  }
  run_integrate(t, compute_tau, pab_blocks, grids, hab_blocks, forces, virial, s);
}

// Copy chunks of the host-buffer calls: t->copy_chunks pieces whose sizes
// grow 1 : 2 : 4 ... in block order, cut at block starts.  One piece where
// the blocks' ranges in the buffer are not in subblock order.
static const CopyChunks &get_chunks(TaskList *t) {
  if (t->chunks_for == t->copy_chunks)
    return t->chunks;
  const int nsubs = (int)t->subs.size();
  CopyChunks c;
  c.sub_lo = {0, nsubs};
  c.el_lo = {0, t->buffer_len};
  const int want = std::max(1, std::min(t->copy_chunks, 7));
  bool ok = nsubs > 0 && t->buffer_len > 0;
  std::vector<long long> bstart(nsubs);
  long long prev_end = 0;
  for (int i = 0; i < nsubs && ok; i++) {
    const SubblockDesc &sb = t->subs[i];
    bstart[i] = sb.block_offset;
    if (i > 0 && sb.block_offset == t->subs[i - 1].block_offset)
      continue; // another subblock of the same block
    if (sb.block_offset < prev_end)
      ok = false;
    prev_end = (long long)sb.block_offset + (long long)sb.nsgfa * sb.nsgfb;
  }
  if (ok && want > 1) {
    std::vector<int> sub_lo = {0};
    std::vector<long long> el_lo = {0};
    const double denom = (double)((1 << want) - 1);
    for (int k = 1; k < want; k++) {
      const long long target = (long long)((double)((1 << k) - 1) / denom * t->buffer_len);
      int i = sub_lo.back() + 1;
      while (i < nsubs && (bstart[i] < target || bstart[i] == bstart[i - 1]))
        i++;
      if (i >= nsubs)
        break;
      sub_lo.push_back(i);
      el_lo.push_back(bstart[i]);
    }
    sub_lo.push_back(nsubs);
    el_lo.push_back(t->buffer_len);
    c.sub_lo = sub_lo;
    c.el_lo = el_lo;
  }
  c.n = (int)c.sub_lo.size() - 1;
  t->chunks = c;
  t->chunks_for = t->copy_chunks;
  return t->chunks;
}

// the copy stream and `n` timing-free events of a host-buffer call
static cudaEvent_t *copy_events(TaskList *t, size_t n) {
  if (!t->copy_stream)
    CK(cudaStreamCreateWithFlags(&t->copy_stream, cudaStreamNonBlocking));
  while (t->copy_ev.size() < n) {
    cudaEvent_t e;
    CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    t->copy_ev.push_back(e);
  }
  return t->copy_ev.data();
}

GB300_API void grid_gb300_collocate_task_list(const grid_gb300_task_list *task_list,
                                              const enum grid_func func, const int nlevels,
                                              const offload_buffer *pab_blocks,
                                              offload_buffer **grids) {
  TaskList *t = TL(task_list);
  if (nlevels != t->nlevels)
    fail("collocate: nlevels %d does not match the task list (%d)", nlevels, t->nlevels);
  if (t->empty) {
    for (int l = 0; l < nlevels; l++)
      memset(grids[l]->host_buffer, 0, grids[l]->size);
    return;
  }
  cudaStream_t s = t->stream;
  double *g[GB300_MAX_LEVELS];
  for (int l = 0; l < nlevels; l++)
    g[l] = grids[l]->device_buffer;
  const CopyChunks &ch = get_chunks(t);
  if (ch.n > 1 && (long long)(pab_blocks->size / sizeof(double)) >= t->buffer_len) {
    // pab in pieces on the copy stream; piece c's kernels start once it landed
    cudaEvent_t *ev = copy_events(t, (size_t)ch.n + 1);
    CK(cudaEventRecord(ev[ch.n], s)); // earlier work on the list's stream is done
    CK(cudaStreamWaitEvent(t->copy_stream, ev[ch.n], 0));
    for (int c = 0; c < ch.n; c++) {
      const long long e0 = ch.el_lo[c], e1 = ch.el_lo[c + 1];
      if (e1 > e0)
        CK(cudaMemcpyAsync(pab_blocks->device_buffer + e0, pab_blocks->host_buffer + e0,
                           sizeof(double) * (size_t)(e1 - e0), cudaMemcpyHostToDevice,
                           t->copy_stream));
      CK(cudaEventRecord(ev[c], t->copy_stream));
    }
    HostCopy hc;
    hc.ch = &ch;
    hc.cs = t->copy_stream;
    hc.ready = ev;
    run_collocate(t, func, pab_blocks->device_buffer, g, s, &hc);
  } else {
    CK(cudaMemcpyAsync(pab_blocks->device_buffer, pab_blocks->host_buffer, pab_blocks->size,
                       cudaMemcpyHostToDevice, s));
    run_collocate(t, func, pab_blocks->device_buffer, g, s);
  }
  for (int l = 0; l < nlevels; l++)
    CK(cudaMemcpyAsync(grids[l]->host_buffer, grids[l]->device_buffer, grids[l]->size,
                       cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  read_timings(t);
  check_device_error(t);
}

GB300_API void grid_gb300_integrate_task_list(const grid_gb300_task_list *task_list,
                                              const bool compute_tau, const int nlevels,
                                              const offload_buffer *pab_blocks,
                                              const offload_buffer **grids,
                                              offload_buffer *hab_blocks, double *forces,
                                              double *virial) {
  TaskList *t = TL(task_list);
  if (nlevels != t->nlevels)
    fail("integrate: nlevels %d does not match the task list (%d)", nlevels, t->nlevels);
  if ((forces || virial) && !pab_blocks)
    fail("forces and virial require pab_blocks");
  if (t->empty) {
    memset(hab_blocks->host_buffer, 0, hab_blocks->size);
    if (forces)
      memset(forces, 0, sizeof(double) * 3 * t->natoms);
    if (virial)
      memset(virial, 0, sizeof(double) * 9);
    return;
  }
  if ((long long)(hab_blocks->size / sizeof(double)) < t->buffer_len)
    fail("integrate: hab buffer holds %zu doubles, the task list needs %lld",
         hab_blocks->size / sizeof(double), t->buffer_len);
  cudaStream_t s = t->stream;
  const double *g[GB300_MAX_LEVELS];
  for (int l = 0; l < nlevels; l++)
    g[l] = grids[l]->device_buffer;
  const bool need_pab = pab_blocks && (forces || virial);
  const CopyChunks &ch = get_chunks(t);
  if (ch.n > 1) {
    // V levels and pab in on the copy stream, hab out in pieces behind the
    // kernels of the next piece
    cudaEvent_t *ev = copy_events(t, (size_t)(2 * ch.n + nlevels + 2));
    cudaEvent_t *vready = ev, *done = ev + nlevels, start = ev[nlevels + ch.n],
                pab_ready = ev[nlevels + ch.n + 1];
    CK(cudaEventRecord(start, s));
    CK(cudaStreamWaitEvent(t->copy_stream, start, 0));
    for (int l = 0; l < nlevels; l++) {
      CK(cudaMemcpyAsync(grids[l]->device_buffer, grids[l]->host_buffer, grids[l]->size,
                         cudaMemcpyHostToDevice, t->copy_stream));
      CK(cudaEventRecord(vready[l], t->copy_stream));
    }
    if (need_pab)
      CK(cudaMemcpyAsync(pab_blocks->device_buffer, pab_blocks->host_buffer, pab_blocks->size,
                         cudaMemcpyHostToDevice, t->copy_stream));
    CK(cudaEventRecord(pab_ready, t->copy_stream));
    HostCopy hc;
    hc.ch = &ch;
    hc.cs = t->copy_stream;
    hc.vready = vready;
    hc.pab_ready = pab_ready;
    hc.done = done;
    hc.hab_host = hab_blocks->host_buffer;
    run_integrate(t, compute_tau, pab_blocks ? pab_blocks->device_buffer : nullptr, g,
                  hab_blocks->device_buffer, forces ? t->d_forces : nullptr,
                  virial ? t->d_virial : nullptr, s, &hc);
    // the reference zeroes the whole hab buffer; past the task list's blocks
    // nothing is computed
    if (hab_blocks->size > sizeof(double) * (size_t)t->buffer_len)
      memset(hab_blocks->host_buffer + t->buffer_len, 0,
             hab_blocks->size - sizeof(double) * (size_t)t->buffer_len);
  } else {
    for (int l = 0; l < nlevels; l++)
      CK(cudaMemcpyAsync(grids[l]->device_buffer, grids[l]->host_buffer, grids[l]->size,
                         cudaMemcpyHostToDevice, s));
    if (need_pab)
      CK(cudaMemcpyAsync(pab_blocks->device_buffer, pab_blocks->host_buffer, pab_blocks->size,
                         cudaMemcpyHostToDevice, s));
    run_integrate(t, compute_tau, pab_blocks ? pab_blocks->device_buffer : nullptr, g,
                  hab_blocks->device_buffer, forces ? t->d_forces : nullptr,
                  virial ? t->d_virial : nullptr, s);
    CK(cudaMemcpyAsync(hab_blocks->host_buffer, hab_blocks->device_buffer,
                       sizeof(double) * (size_t)t->buffer_len, cudaMemcpyDeviceToHost, s));
    if (hab_blocks->size > sizeof(double) * (size_t)t->buffer_len)
      memset(hab_blocks->host_buffer + t->buffer_len, 0,
             hab_blocks->size - sizeof(double) * (size_t)t->buffer_len);
  }
  if (forces)
    CK(cudaMemcpyAsync(forces, t->d_forces, sizeof(double) * 3 * t->natoms,
                       cudaMemcpyDeviceToHost, s));
  if (virial)
    CK(cudaMemcpyAsync(virial, t->d_virial, sizeof(double) * 9, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (t->copy_stream)
    CK(cudaStreamSynchronize(t->copy_stream));
  read_timings(t);
  check_device_error(t);
}

// ===========================================================================
// CP2K task-list surface (src/grid/grid_task_list.c)
// ===========================================================================
struct TopList {
  int nlevels = 0;
  int natoms = 0;
  std::vector<int> npts_local;
  grid_gb300_task_list *impl = nullptr;
};

GB300_API void grid_create_task_list(
    const bool orthorhombic, const int ntasks, const int nlevels, const int natoms,
    const int nkinds, const int nblocks, const int *block_offsets, const double *atom_positions,
    const int *atom_kinds, const grid_basis_set **basis_sets, const int *level_list,
    const int *iatom_list, const int *jatom_list, const int *iset_list, const int *jset_list,
    const int *ipgf_list, const int *jpgf_list, const int *border_mask_list,
    const int *block_num_list, const double *radius_list, const double *rab_list,
    const int *npts_global, const int *npts_local, const int *shift_local,
    const int *border_width, const double *dh, const double *dh_inv,
    grid_task_list **task_list) {
  const int be = g_config.backend;
  if (be != GRID_BACKEND_AUTO && be != GRID_BACKEND_GPU && be != GRID_BACKEND_GB300)
    fail("grid backend %d is provided by CP2K's own grid library, not by this one", be);
  TopList *tl = (TopList *)*task_list;
  const bool fresh = !tl;
  if (!tl)
    tl = new TopList();
  tl->nlevels = nlevels;
  tl->natoms = natoms;
  tl->npts_local.assign(npts_local, npts_local + 3 * std::max(nlevels, 0));
  grid_gb300_create_task_list(orthorhombic, ntasks, nlevels, natoms, nkinds, nblocks,
                              block_offsets, atom_positions, atom_kinds, basis_sets, level_list,
                              iatom_list, jatom_list, iset_list, jset_list, ipgf_list,
                              jpgf_list, border_mask_list, block_num_list, radius_list,
                              rab_list, npts_global, npts_local, shift_local, border_width, dh,
                              dh_inv, &tl->impl);
  if (fresh) {
    // CP2K passes no precision: a new list takes it from the environment
    if (const char *e = getenv("GRID_GB300_PRECISION")) {
      const std::string v(e);
      if (v == "fp64" || v == "FP64")
        grid_gb300_set_precision(tl->impl, GRID_GB300_FP64);
      else if (v == "mixed" || v == "MIXED")
        grid_gb300_set_precision(tl->impl, GRID_GB300_MIXED);
      else if (v == "fp32" || v == "FP32")
        grid_gb300_set_precision(tl->impl, GRID_GB300_FP32);
      else
        fail("GRID_GB300_PRECISION=%s: expected fp64, mixed or fp32", e);
    }
    if (const char *e = getenv("GRID_GB300_MIXED_THRESHOLD")) {
      char *end = nullptr;
      const double v = strtod(e, &end);
      if (end == e || *end != '\0' || !(v >= 0.0))
        fail("GRID_GB300_MIXED_THRESHOLD=%s: expected a number >= 0", e);
      grid_gb300_set_mixed_threshold(tl->impl, v);
    }
  }
  *task_list = tl;
}

GB300_API grid_gb300_task_list *grid_gb300_backend_handle(const grid_task_list *task_list) {
  return task_list ? ((const TopList *)task_list)->impl : nullptr;
}

GB300_API void grid_free_task_list(grid_task_list *task_list) {
  if (!task_list)
    return;
  TopList *tl = (TopList *)task_list;
  grid_gb300_free_task_list(tl->impl);
  delete tl;
}

static void check_npts(const TopList *tl, int nlevels, const int *npts_local) {
  if (nlevels != tl->nlevels)
    fail("nlevels %d does not match the task list (%d)", nlevels, tl->nlevels);
  for (int i = 0; i < 3 * nlevels; i++)
    if (npts_local[i] != tl->npts_local[i])
      fail("npts_local of level %d does not match the task list", i / 3);
}

GB300_API void grid_collocate_task_list(const grid_task_list *task_list,
                                        const enum grid_func func, const int nlevels,
                                        const int *npts_local, const offload_buffer *pab_blocks,
                                        offload_buffer **grids) {
  const TopList *tl = (const TopList *)task_list;
  if (!tl)
    return;
  check_npts(tl, nlevels, npts_local);
  grid_gb300_collocate_task_list(tl->impl, func, nlevels, pab_blocks, grids);
}

GB300_API void grid_integrate_task_list(const grid_task_list *task_list, const bool compute_tau,
                                        const int natoms, const int nlevels,
                                        const int *npts_local, const offload_buffer *pab_blocks,
                                        const offload_buffer **grids, offload_buffer *hab_blocks,
                                        double *forces, double *virial) {
  const TopList *tl = (const TopList *)task_list;
  if (!tl)
    return;
  check_npts(tl, nlevels, npts_local);
  if (natoms != tl->natoms)
    fail("natoms %d does not match the task list (%d)", natoms, tl->natoms);
  grid_gb300_integrate_task_list(tl->impl, compute_tau, nlevels, pab_blocks, grids, hab_blocks,
                                 forces, virial);
}

// ===========================================================================
// extensions
// ===========================================================================
GB300_API void grid_gb300_set_precision(const grid_gb300_task_list *task_list, int precision) {
  if (precision != GRID_GB300_FP64 && precision != GRID_GB300_MIXED &&
      precision != GRID_GB300_FP32)
    fail("unknown precision mode %d", precision);
  TaskList *t = TL(task_list);
  // queues are kept per precision (get_mode); nothing to rebuild here
  t->precision = precision;
}

GB300_API int grid_gb300_get_precision(const grid_gb300_task_list *task_list) {
  return TL(task_list)->precision;
}

GB300_API void grid_gb300_set_mixed_threshold(const grid_gb300_task_list *task_list,
                                              double threshold) {
  TaskList *t = TL(task_list);
  if (!(threshold >= 0.0))
    fail("mixed threshold must be >= 0");
  if (t->mixed_threshold != threshold) {
    t->mixed_threshold = threshold;
    t->sched_version++;
  }
}

GB300_API void grid_gb300_mixed_split(const grid_gb300_task_list *task_list, double *frac_tasks,
                                      double *frac_points) {
  const TaskList *t = TL(task_list);
  double nt = 0, nf = 0, pt = 0, pf = 0;
  for (size_t s = 0; s < t->tasks.size(); s++) {
    if (t->tasks[s].flags & TF_SKIP)
      continue;
    nt += 1;
    pt += (double)t->points[s];
    if (t->gbound[s] <= t->mixed_threshold) {
      nf += 1;
      pf += (double)t->points[s];
    }
  }
  if (frac_tasks)
    *frac_tasks = nt ? nf / nt : 0.0;
  if (frac_points)
    *frac_points = pt ? pf / pt : 0.0;
}

GB300_API void grid_gb300_row_split_stats(const grid_gb300_task_list *task_list,
                                          double *frac_tasks_split, double *frac_points_fp32) {
  const TaskList *t = TL(task_list);
  std::vector<double> out(t->tasks.size(), 0.0);
  std::vector<char> cls(t->tasks.size(), -1);
  parallel_for((int)t->tasks.size(), [&](int s) {
    const TaskDesc &k = t->tasks[s];
    if (k.flags & TF_SKIP)
      return;
    if (t->gbound[s] <= t->mixed_threshold) {
      cls[s] = 1;
      return;
    }
    cls[s] = 0;
    if (t->row_split && !(k.flags & TF_GENERAL) &&
        core_radius2(k, 0, 0, t->mixed_threshold / kShellMargin, &out[s]) >= kCoreAll)
      out[s] = 0.0;
  });
  double nt = 0, ns = 0, pt = 0, pf = 0;
  for (size_t s = 0; s < t->tasks.size(); s++) {
    if (cls[s] < 0)
      continue;
    nt += 1;
    pt += (double)t->points[s];
    if (cls[s] == 1)
      pf += (double)t->points[s];
    else if (out[s] > 0.0) {
      ns += 1;
      pf += out[s] * (double)t->points[s];
    }
  }
  if (frac_tasks_split)
    *frac_tasks_split = nt ? ns / nt : 0.0;
  if (frac_points_fp32)
    *frac_points_fp32 = pt ? pf / pt : 0.0;
}

GB300_API void grid_gb300_set_schedule(const grid_gb300_task_list *task_list, int schedule) {
  if (schedule < GRID_GB300_SCHEDULE_SIZE || schedule > GRID_GB300_SCHEDULE_INPUT)
    fail("unknown schedule %d", schedule);
  TaskList *t = TL(task_list);
  if (t->schedule != schedule) {
    t->schedule = schedule;
    t->sched_version++;
  }
}

GB300_API void grid_gb300_task_list_info(const grid_gb300_task_list *task_list, int *ntasks,
                                         int *nlevels, int *natoms, long long *buffer_len) {
  const TaskList *t = TL(task_list);
  if (ntasks)
    *ntasks = t->ntasks;
  if (nlevels)
    *nlevels = t->nlevels;
  if (natoms)
    *natoms = t->natoms;
  if (buffer_len)
    *buffer_len = t->buffer_len;
}

GB300_API void grid_gb300_task_sizes(const grid_gb300_task_list *task_list, long long *points,
                                     int *lp) {
  const TaskList *t = TL(task_list);
  for (int s = 0; s < (int)t->tasks.size(); s++) {
    const TaskDesc &k = t->tasks[s];
    if (points)
      points[k.orig] = (k.flags & TF_SKIP) ? 0 : t->points[s];
    if (lp)
      lp[k.orig] = k.la_max + k.lb_max;
  }
}

// ---------------------------------------------------------------------------
// CUDA-graph capture of one SCF step
// ---------------------------------------------------------------------------
namespace gb300 {
struct StepGraph {
  TaskList *t = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  long long kernels = 0;
  long long gen = 0;
  int sched_version = 0, precision = 0;
  bool task_timing = false;
};
} // namespace gb300

GB300_API grid_gb300_step_graph *grid_gb300_capture_step(
    const grid_gb300_task_list *task_list, int func, const double *pab_blocks,
    double *const *rho_grids, bool compute_tau, const double *const *v_grids, double *hab_blocks,
    double *forces, double *virial, void *stream) {
  TaskList *t = TL(task_list);
  cudaStream_t s = (cudaStream_t)stream;
  if (!s)
    fail("capture_step: needs a created stream (the legacy default stream cannot be captured)");
  // one plain run: creates the work queues and the lazily allocated arrays
  // so that the captured sequence allocates nothing
  grid_gb300_collocate_device_async(task_list, func, pab_blocks, rho_grids, stream);
  grid_gb300_integrate_device_async(task_list, compute_tau, pab_blocks, v_grids, hab_blocks,
                                    forces, virial, stream);
  CK(cudaStreamSynchronize(s));
  check_device_error(t);
  StepGraph *g = new StepGraph;
  g->t = t;
  g->gen = t->gen;
  const long long k0 = grid_gb300_kernel_launches();
  t->capturing = true;
  CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  grid_gb300_collocate_device_async(task_list, func, pab_blocks, rho_grids, stream);
  grid_gb300_integrate_device_async(task_list, compute_tau, pab_blocks, v_grids, hab_blocks,
                                    forces, virial, stream);
  const cudaError_t e = cudaStreamEndCapture(s, &g->graph);
  t->capturing = false;
  if (e != cudaSuccess)
    fail("capture_step: stream capture failed: %s", cudaGetErrorString(e));
  if (t->gen != g->gen)
    fail("capture_step: device arrays moved during capture");
  g->kernels = grid_gb300_kernel_launches() - k0;
  g_launches -= g->kernels; // capturing launches nothing
  CK(cudaGraphInstantiate(&g->exec, g->graph, 0));
  g->sched_version = t->sched_version;
  g->precision = t->precision;
  g->task_timing = t->task_timing;
  return (grid_gb300_step_graph *)g;
}

GB300_API void grid_gb300_step_graph_launch(grid_gb300_step_graph *graph, void *stream) {
  StepGraph *g = (StepGraph *)graph;
  if (!g)
    fail("null step graph");
  const TaskList *t = g->t;
  if (t->gen != g->gen || t->sched_version != g->sched_version ||
      t->precision != g->precision || t->task_timing != g->task_timing)
    fail("step graph: the task list changed since capture (precision, schedule, timing or "
         "buffers); capture again");
  CK(cudaGraphLaunch(g->exec, (cudaStream_t)stream));
  count_launch((int)g->kernels);
}

GB300_API void grid_gb300_step_graph_wait(grid_gb300_step_graph *graph, void *stream) {
  StepGraph *g = (StepGraph *)graph;
  if (!g)
    fail("null step graph");
  CK(cudaStreamSynchronize((cudaStream_t)stream));
  check_device_error(g->t);
}

GB300_API long long grid_gb300_step_graph_kernels(const grid_gb300_step_graph *graph) {
  return graph ? ((const StepGraph *)graph)->kernels : 0;
}

GB300_API void grid_gb300_step_graph_free(grid_gb300_step_graph *graph) {
  StepGraph *g = (StepGraph *)graph;
  if (!g)
    return;
  if (g->exec)
    cudaGraphExecDestroy(g->exec);
  if (g->graph)
    cudaGraphDestroy(g->graph);
  delete g;
}

// ---------------------------------------------------------------------------
// autotuner: size-class split and per-queue launch shapes, by measurement
// ---------------------------------------------------------------------------
namespace gb300 {
// one SCF step with per-launch events; returns the summed grid-kernel time
// and appends (phase, key, ms) of every grid launch
static double tune_step(TaskList *t, int func, const double *pab, double *const *rho,
                        const double *const *v, double *hab, cudaStream_t s,
                        std::vector<std::tuple<int, int, double>> *out) {
  double total = 0.0;
  for (int phase = 0; phase < 2; phase++) {
    if (phase == 0)
      run_collocate(t, func, pab, rho, s);
    else
      run_integrate(t, false, pab, v, hab, nullptr, nullptr, s);
    CK(cudaStreamSynchronize(s));
    check_device_error(t);
    for (LaunchRecord &r : t->launches) {
      const double ms = ev_ms(r.a, r.b);
      total += ms;
      if (out)
        out->emplace_back(phase, r.key, ms);
    }
  }
  return total;
}
} // namespace gb300

GB300_API double grid_gb300_autotune(const grid_gb300_task_list *task_list, int func,
                                     const double *pab_blocks, double *const *rho_grids,
                                     const double *const *v_grids, double *hab_blocks,
                                     void *stream) {
  TaskList *t = TL(task_list);
  if (t->empty)
    return 0.0;
  cudaStream_t s = (cudaStream_t)stream;
  const bool lt = t->launch_timing;
  t->launch_timing = true;
  const int prec = t->precision;
  for (auto it = t->tuned.begin(); it != t->tuned.end();)
    it = std::get<0>(it->first) == prec ? t->tuned.erase(it) : std::next(it);
  // 1. work split: the cube width that separates the small- and large-cube
  //    queues (best of two timed steps each, after one warm-up step)
  const int splits[] = {26, 34, 42, 66};
  int best_split = t->small_extent[prec];
  double best = 1e300;
  for (int e : splits) {
    t->small_extent[prec] = e;
    t->sched_version++;
    tune_step(t, func, pab_blocks, rho_grids, v_grids, hab_blocks, s, nullptr);
    double ms = 1e300;
    for (int r = 0; r < 2; r++)
      ms = std::min(ms, tune_step(t, func, pab_blocks, rho_grids, v_grids, hab_blocks, s, nullptr));
    if (ms < best) {
      best = ms;
      best_split = e;
    }
  }
  t->small_extent[prec] = best_split;
  t->sched_version++;
  tune_step(t, func, pab_blocks, rho_grids, v_grids, hab_blocks, s, nullptr);
  // 2. launch shape of every queue: warps per CTA x share of the resident CTAs
  struct Cand {
    int warps, occ, variant;
  };
  const Cand cands[] = {{4, 100, 0}, {2, 100, 0}, {1, 100, 0}, {4, 75, 0},
                        {4, 50, 0},  {4, 100, 1}, {2, 100, 1}, {1, 100, 1}};
  std::map<std::pair<int, int>, std::pair<double, int>> pick; // (phase,key) -> (ms, cand)
  for (int c = 0; c < (int)(sizeof(cands) / sizeof(cands[0])); c++) {
    for (const auto &kv : t->modes)
      for (const Queue &q : kv.second.queues)
        for (int phase = 0; phase < 2; phase++) {
          LaunchCfg cfg;
          cfg.warps = cands[c].warps;
          cfg.occupancy = cands[c].occ;
          cfg.variant = cands[c].variant;
          t->tuned[std::make_tuple(prec, phase, q.base)] = cfg;
        }
    std::map<std::pair<int, int>, double> ms;
    for (int r = 0; r < 2; r++) {
      std::vector<std::tuple<int, int, double>> rec;
      tune_step(t, func, pab_blocks, rho_grids, v_grids, hab_blocks, s, &rec);
      for (auto &x : rec) {
        auto key = std::make_pair(std::get<0>(x), std::get<1>(x));
        auto f = ms.find(key);
        ms[key] = f == ms.end() ? std::get<2>(x) : std::min(f->second, std::get<2>(x));
      }
    }
    for (auto &kv : ms) {
      auto f = pick.find(kv.first);
      if (f == pick.end() || kv.second < f->second.first)
        pick[kv.first] = {kv.second, c};
    }
  }
  double total = 0.0;
  for (auto &kv : pick) {
    LaunchCfg cfg;
    cfg.warps = cands[kv.second.second].warps;
    cfg.occupancy = cands[kv.second.second].occ;
    cfg.variant = cands[kv.second.second].variant;
    t->tuned[std::make_tuple(prec, kv.first.first, kv.first.second)] = cfg;
    total += kv.second.first;
  }
  t->launch_timing = lt;
  t->launches.clear();
  t->gen++;
  return total;
}

GB300_API void grid_gb300_set_collocate_variant(const grid_gb300_task_list *task_list,
                                                int variant) {
  if (variant < -1 || variant > 1)
    fail("unknown collocate variant %d", variant);
  TaskList *t = TL(task_list);
  t->coll_variant = variant;
  t->tuned.clear();
  t->gen++;
}

GB300_API void grid_gb300_set_tensor_integrate(const grid_gb300_task_list *task_list,
                                               int enable) {
  TaskList *t = TL(task_list);
  t->tc_integrate = enable ? 1 : 0;
  t->gen++; // captured graphs hold the other kernel
}

GB300_API void grid_gb300_set_tensor_collocate(const grid_gb300_task_list *task_list,
                                               int enable) {
  TaskList *t = TL(task_list);
  t->tc_collocate = enable ? 1 : 0;
  t->gen++; // captured graphs hold the other kernel
}

GB300_API void grid_gb300_set_row_split(const grid_gb300_task_list *task_list, int enable) {
  TaskList *t = TL(task_list);
  t->row_split = enable ? 1 : 0;
  t->sched_version++; // the work queues change
}

GB300_API void grid_gb300_set_queue_streams(const grid_gb300_task_list *task_list, int n) {
  if (n < 1 || n > 2)
    fail("queue streams must be 1 or 2, got %d", n);
  TL(task_list)->queue_streams = n;
}

GB300_API void grid_gb300_set_copy_chunks(const grid_gb300_task_list *task_list, int chunks) {
  if (chunks < 1 || chunks > 7)
    fail("copy chunks must be in 1..7, got %d", chunks);
  TL(task_list)->copy_chunks = chunks;
}

GB300_API void grid_gb300_set_transform_variant(const grid_gb300_task_list *task_list,
                                               int variant) {
  if (variant < -1 || variant > 1)
    fail("unknown transform variant %d", variant);
  TaskList *t = TL(task_list);
  if (t->transform_variant != variant) {
    t->transform_variant = variant;
    t->sched_version++; // the modes' shared-memory sizes depend on it
  }
}

GB300_API void grid_gb300_set_model_bin_width(const grid_gb300_task_list *task_list,
                                              double width) {
  if (!(width >= 0.0))
    fail("model bin width must be >= 0");
  TaskList *t = TL(task_list);
  t->model_bin = width;
  t->sched_version++;
}

GB300_API int grid_gb300_tuned_split(const grid_gb300_task_list *task_list) {
  const TaskList *t = TL(task_list);
  return t->small_extent[t->precision];
}

GB300_API void grid_gb300_set_launch_timing(const grid_gb300_task_list *task_list, int enable) {
  TL(task_list)->launch_timing = enable != 0;
}

GB300_API int grid_gb300_launch_timings(const grid_gb300_task_list *task_list, int max,
                                        grid_gb300_launch_info *info) {
  TaskList *t = TL(task_list);
  const int n = (int)t->launches.size();
  for (int i = 0; i < n && i < max; i++) {
    LaunchRecord &r = t->launches[i];
    CK(cudaEventSynchronize(r.b));
    r.info.ms = ev_ms(r.a, r.b);
    info[i] = r.info;
  }
  return n;
}

GB300_API void grid_gb300_set_task_timing(const grid_gb300_task_list *task_list, int enable) {
  TL(task_list)->task_timing = enable != 0;
}

GB300_API void grid_gb300_task_cycles(const grid_gb300_task_list *task_list, long long *cycles) {
  TaskList *t = TL(task_list);
  if (t->empty)
    return;
  if (!t->d_cycles) {
    memset(cycles, 0, sizeof(long long) * t->ntasks);
    return;
  }
  CK(cudaDeviceSynchronize());
  std::vector<long long> c(t->ntasks);
  CK(cudaMemcpy(c.data(), t->d_cycles, sizeof(long long) * t->ntasks, cudaMemcpyDeviceToHost));
  for (int s = 0; s < t->ntasks; s++)
    cycles[t->tasks[s].orig] = c[s];
}

GB300_API void grid_gb300_task_features(const grid_gb300_task_list *task_list, float *features) {
  TaskList *t = TL(task_list);
  if (t->empty)
    return;
  for (int s = 0; s < t->ntasks; s++)
    memcpy(features + (size_t)t->tasks[s].orig * 6, &t->features[(size_t)s * 6], 6 * sizeof(float));
}

GB300_API int grid_gb300_cost_model_nparams(void) { return mlp_nparams(); }

GB300_API size_t grid_gb300_cost_model_work_floats(int n) {
  return (size_t)mlp_tiles(n) * (mlp_nparams() + 1);
}

GB300_API void grid_gb300_cost_model_loss_grad(const float *params, const float *x, const float *t_,
                                               int n, float *loss, float *grad, float *work,
                                               void *stream) {
  if (n < 1)
    fail("cost model: no training samples");
  launch_mlp_loss_grad(params, x, t_, n, loss, grad, work, (cudaStream_t)stream);
  CK(cudaGetLastError());
}

GB300_API void grid_gb300_cost_model_adam(float *params, const float *grad, float *m, float *v,
                                          int step, float lr, float beta1, float beta2, float eps,
                                          void *stream) {
  if (step < 1)
    fail("cost model: Adam steps count from 1");
  launch_mlp_adam(params, grad, m, v, step, lr, beta1, beta2, eps, (cudaStream_t)stream);
  CK(cudaGetLastError());
}

GB300_API void grid_gb300_cost_model_predict(const float *params, const float *x, int n,
                                             const float *norm, float *y, void *stream) {
  launch_mlp_predict(params, x, n, norm, y, (cudaStream_t)stream);
  CK(cudaGetLastError());
}

GB300_API void grid_gb300_apply_cost_model(const grid_gb300_task_list *task_list,
                                           const float *params, const float *norm, void *stream) {
  TaskList *t = TL(task_list);
  if (t->empty)
    return;
  const cudaStream_t s = (cudaStream_t)stream;
  float *d_x = nullptr, *d_y = nullptr;
  CK(cudaMalloc((void **)&d_x, sizeof(float) * t->features.size()));
  CK(cudaMalloc((void **)&d_y, sizeof(float) * t->ntasks));
  CK(cudaMemcpyAsync(d_x, t->features.data(), sizeof(float) * t->features.size(),
                     cudaMemcpyHostToDevice, s));
  launch_mlp_predict(params, d_x, t->ntasks, norm, d_y, s);
  t->model_cost.resize(t->ntasks);
  CK(cudaMemcpyAsync(t->model_cost.data(), d_y, sizeof(float) * t->ntasks,
                     cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  CK(cudaFree(d_x));
  CK(cudaFree(d_y));
  for (float &c : t->model_cost)
    if (!std::isfinite(c))
      fail("cost model: non-finite prediction");
  t->sched_version++;
}

GB300_API void grid_gb300_last_timings(const grid_gb300_task_list *task_list,
                                       double timings_ms[4]) {
  TaskList *t = TL(task_list);
  if (!t->empty)
    read_timings(t);
  for (int i = 0; i < 4; i++)
    timings_ms[i] = t->timings[i];
}
