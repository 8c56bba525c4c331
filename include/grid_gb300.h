/*
 * C ABI of the GB300 grid backend (libgb300grid.so).
 *
 * Two layers, both plain C (no CUDA or torch types in any signature):
 *
 *  1. The CP2K grid library surface, symbol for symbol, so that Quickstep's
 *     Fortran binding (src/grid/grid_api.F) can call this library unchanged:
 *     offload buffers, basis sets, task lists, library config.  AUTO, GPU and
 *     the new GB300 backend value all run on this backend; REF/CPU/DGEMM are
 *     served by CP2K's own library and are rejected here with an error.
 *
 *  2. The backend-level entry points grid_gb300_* with the signatures of
 *     CP2K's per-backend functions (src/grid/gpu/grid_gpu_task_list.h:25-54),
 *     which CP2K's dispatcher (src/grid/grid_task_list.c:93-134, 199-223,
 *     324-350) binds from a new `case GRID_BACKEND_GB300:`.  Extensions for
 *     device-resident buffers, precision and schedule follow them.
 *
 * Errors: the CP2K surface has no status codes (it aborts, see
 * src/grid/grid_task_list.c:131-133); this library does the same on misuse
 * after printing a message, and additionally records the message for
 * grid_gb300_last_error().  Calls are synchronous unless named *_async.
 */
#ifndef GRID_GB300_H
#define GRID_GB300_H

#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- src/offload/offload_buffer.h:16-20 -------------------------------- */
typedef struct {
  size_t size;          /* bytes */
  double *host_buffer;  /* pinned host memory */
  double *device_buffer;
} offload_buffer;

/* Replaces offload_create_buffer (src/offload/offload_buffer.h:26). */
void offload_create_buffer(const int length, offload_buffer **buffer);
/* Replaces offload_free_buffer (src/offload/offload_buffer.h:32). */
void offload_free_buffer(offload_buffer *buffer);
/* Replaces offload_get_buffer_host_pointer (src/offload/offload_buffer.h:38). */
double *offload_get_buffer_host_pointer(offload_buffer *buffer);

/* ---- src/grid/common/grid_constants.h:10-54 ---------------------------- */
enum grid_func {
  GRID_FUNC_AB = 100,
  GRID_FUNC_DADB = 200,
  GRID_FUNC_ADBmDAB_X = 301,
  GRID_FUNC_ADBmDAB_Y = 302,
  GRID_FUNC_ADBmDAB_Z = 303,
  GRID_FUNC_ARDBmDARB_XX = 411,
  GRID_FUNC_ARDBmDARB_XY = 412,
  GRID_FUNC_ARDBmDARB_XZ = 413,
  GRID_FUNC_ARDBmDARB_YX = 421,
  GRID_FUNC_ARDBmDARB_YY = 422,
  GRID_FUNC_ARDBmDARB_YZ = 423,
  GRID_FUNC_ARDBmDARB_ZX = 431,
  GRID_FUNC_ARDBmDARB_ZY = 432,
  GRID_FUNC_ARDBmDARB_ZZ = 433,
  GRID_FUNC_DABpADB_X = 501,
  GRID_FUNC_DABpADB_Y = 502,
  GRID_FUNC_DABpADB_Z = 503,
  GRID_FUNC_DX = 601,
  GRID_FUNC_DY = 602,
  GRID_FUNC_DZ = 603,
  GRID_FUNC_DXDY = 701,
  GRID_FUNC_DYDZ = 702,
  GRID_FUNC_DZDX = 703,
  GRID_FUNC_DXDX = 801,
  GRID_FUNC_DYDY = 802,
  GRID_FUNC_DZDZ = 803,
  GRID_FUNC_DAB_X = 901,
  GRID_FUNC_DAB_Y = 902,
  GRID_FUNC_DAB_Z = 903,
  GRID_FUNC_ADB_X = 904,
  GRID_FUNC_ADB_Y = 905,
  GRID_FUNC_ADB_Z = 906,
  GRID_FUNC_CORE_X = 1001,
  GRID_FUNC_CORE_Y = 1002,
  GRID_FUNC_CORE_Z = 1003,
};

enum grid_backend {
  GRID_BACKEND_AUTO = 10,
  GRID_BACKEND_REF = 11,
  GRID_BACKEND_CPU = 12,
  GRID_BACKEND_DGEMM = 13,
  GRID_BACKEND_GPU = 14,
  GRID_BACKEND_GB300 = 15, /* new: this library */
};

/* ---- src/grid/common/grid_basis_set.h:14-64 ---------------------------- */
typedef struct {
  int nset;
  int nsgf;
  int maxco;
  int maxpgf;
  int *lmin;
  int *lmax;
  int *npgf;
  int *nsgf_set;
  int *first_sgf;
  double *sphi; /* [nsgf][maxco] */
  double *zet;  /* [nset][maxpgf] */
} grid_basis_set;

/* Replaces grid_create_basis_set (src/grid/common/grid_basis_set.h:52). */
void grid_create_basis_set(const int nset, const int nsgf, const int maxco,
                           const int maxpgf, const int *lmin, const int *lmax,
                           const int *npgf, const int *nsgf_set,
                           const int *first_sgf, const double *sphi,
                           const double *zet, grid_basis_set **basis_set);
/* Replaces grid_free_basis_set (src/grid/common/grid_basis_set.h:64). */
void grid_free_basis_set(grid_basis_set *basis_set);

/* ---- src/grid/common/grid_library.h:22-85 ------------------------------ */
typedef struct {
  enum grid_backend backend;
  bool validate;
  bool apply_cutoff;
} grid_library_config;

enum grid_library_kernel {
  GRID_COLLOCATE_ORTHO = 0,
  GRID_INTEGRATE_ORTHO = 1,
  GRID_COLLOCATE_GENERAL = 2,
  GRID_INTEGRATE_GENERAL = 3,
};

/* Replaces grid_library_init (src/grid/common/grid_library.h:25). */
void grid_library_init(void);
/* Replaces grid_library_finalize (src/grid/common/grid_library.h:31). */
void grid_library_finalize(void);
/* Replaces grid_library_set_config (src/grid/common/grid_library.h:47).
 * validate=true is accepted and recorded; the shadow REF run it asks for is
 * not linked into this library (no CPU path here) -- parity against REF is
 * checked by the test-suite instead. */
void grid_library_set_config(const enum grid_backend backend,
                             const bool validate, const bool apply_cutoff);
/* Replaces grid_library_get_config (src/grid/common/grid_library.h:53). */
grid_library_config grid_library_get_config(void);
/* Replaces grid_library_print_stats (src/grid/common/grid_library.h:59). */
void grid_library_print_stats(const int fortran_comm,
                              void (*print_func)(const char *, int, int),
                              const int output_unit);
/* Replaces grid_library_counter_add (src/grid/common/grid_library.h:81). */
void grid_library_counter_add(const int lp, const enum grid_backend backend,
                              const enum grid_library_kernel kernel,
                              const int increment);

/* ---- src/grid/grid_task_list.h:16-126 ---------------------------------- */
typedef void grid_task_list;

/* Replaces grid_create_task_list (src/grid/grid_task_list.h:59-72).
 * Arrays are C row-major: atom_positions[natoms][3], rab_list[ntasks][3],
 * npts_*[nlevels][3], dh/dh_inv[nlevels][3][3].  Task lists are 1-based.
 * A new list computes in FP64 unless the environment sets
 * GRID_GB300_PRECISION=fp64|mixed|fp32 (and GRID_GB300_MIXED_THRESHOLD, see
 * grid_gb300_set_mixed_threshold); re-creation keeps the list's settings. */
void grid_create_task_list(
    const bool orthorhombic, const int ntasks, const int nlevels,
    const int natoms, const int nkinds, const int nblocks,
    const int *block_offsets, const double *atom_positions,
    const int *atom_kinds, const grid_basis_set **basis_sets,
    const int *level_list, const int *iatom_list, const int *jatom_list,
    const int *iset_list, const int *jset_list, const int *ipgf_list,
    const int *jpgf_list, const int *border_mask_list,
    const int *block_num_list, const double *radius_list,
    const double *rab_list, const int *npts_global, const int *npts_local,
    const int *shift_local, const int *border_width, const double *dh,
    const double *dh_inv, grid_task_list **task_list);

/* Replaces grid_free_task_list (src/grid/grid_task_list.h:78). */
void grid_free_task_list(grid_task_list *task_list);

/* Replaces grid_collocate_task_list (src/grid/grid_task_list.h:95-99).
 * Grids are overwritten (host_buffer of each grid on return). */
void grid_collocate_task_list(const grid_task_list *task_list,
                              const enum grid_func func, const int nlevels,
                              const int *npts_local,
                              const offload_buffer *pab_blocks,
                              offload_buffer **grids);

/* Replaces grid_integrate_task_list (src/grid/grid_task_list.h:122-126).
 * hab, forces[natoms][3] and virial[3][3] are overwritten; forces and virial
 * may be NULL and require pab_blocks when given. */
void grid_integrate_task_list(const grid_task_list *task_list,
                              const bool compute_tau, const int natoms,
                              const int nlevels, const int *npts_local,
                              const offload_buffer *pab_blocks,
                              const offload_buffer **grids,
                              offload_buffer *hab_blocks, double *forces,
                              double *virial);

/* ---- backend level (src/grid/gpu/grid_gpu_task_list.h:25-54) ----------- */
typedef void grid_gb300_task_list;

/* Replaces grid_gpu_create_task_list (src/grid/gpu/grid_gpu_task_list.h:25). */
void grid_gb300_create_task_list(
    const bool orthorhombic, const int ntasks, const int nlevels,
    const int natoms, const int nkinds, const int nblocks,
    const int *block_offsets, const double *atom_positions,
    const int *atom_kinds, const grid_basis_set **basis_sets,
    const int *level_list, const int *iatom_list, const int *jatom_list,
    const int *iset_list, const int *jset_list, const int *ipgf_list,
    const int *jpgf_list, const int *border_mask_list,
    const int *block_num_list, const double *radius_list,
    const double *rab_list, const int *npts_global, const int *npts_local,
    const int *shift_local, const int *border_width, const double *dh,
    const double *dh_inv, grid_gb300_task_list **task_list);

/* Replaces grid_gpu_free_task_list (src/grid/gpu/grid_gpu_task_list.h:40). */
void grid_gb300_free_task_list(grid_gb300_task_list *task_list);

/* Replaces grid_gpu_collocate_task_list (grid_gpu_task_list.h:46-49). */
void grid_gb300_collocate_task_list(const grid_gb300_task_list *task_list,
                                    const enum grid_func func,
                                    const int nlevels,
                                    const offload_buffer *pab_blocks,
                                    offload_buffer **grids);

/* Replaces grid_gpu_integrate_task_list (grid_gpu_task_list.h:50-54).
 * forces is [natoms][3], virial [3][3]; either may be NULL. */
void grid_gb300_integrate_task_list(const grid_gb300_task_list *task_list,
                                    const bool compute_tau, const int nlevels,
                                    const offload_buffer *pab_blocks,
                                    const offload_buffer **grids,
                                    offload_buffer *hab_blocks, double *forces,
                                    double *virial);

/* ---- extensions (no counterpart in CP2K) ------------------------------ */

/* Arithmetic of the grid kernels:
 *  GRID_GB300_FP64  -- everything in FP64 (parity 1e-12 with REF);
 *  GRID_GB300_MIXED -- per-point polynomial x Gaussian on the FP32 pipes in
 *                      compensated double-float arithmetic (pairs of FP32
 *                      values, ~48-bit significands); FP64 prefactors,
 *                      geometry and C_ab <-> C_xyz transforms, FP64
 *                      accumulation into the grid and hab/forces/virial;
 *  GRID_GB300_FP32  -- plain FP32 per-point work and transforms, FP64
 *                      accumulation (fastest, ~1e-7 of max |rho|). */
enum grid_gb300_precision {
  GRID_GB300_FP64 = 0,
  GRID_GB300_MIXED = 1,
  GRID_GB300_FP32 = 2,
};

/* Order in which the persistent kernels take tasks:
 *  GRID_GB300_SCHEDULE_SIZE  -- descending analytic size (points x (lp+1));
 *  GRID_GB300_SCHEDULE_MODEL -- descending cost predicted by the loaded MLP
 *                               cost model (falls back to SIZE without one);
 *  GRID_GB300_SCHEDULE_INPUT -- list order as given (no reordering). */
enum grid_gb300_schedule {
  GRID_GB300_SCHEDULE_SIZE = 0,
  GRID_GB300_SCHEDULE_MODEL = 1,
  GRID_GB300_SCHEDULE_INPUT = 2,
};

void grid_gb300_set_precision(const grid_gb300_task_list *task_list,
                              int precision);
int grid_gb300_get_precision(const grid_gb300_task_list *task_list);
void grid_gb300_set_schedule(const grid_gb300_task_list *task_list,
                             int schedule);

/* Mixed path: tasks whose contribution bound (Gaussian-product prefactor x
 * polynomial maxima, for density-matrix elements of magnitude <= 1) is at
 * most `threshold` run in plain FP32, the others in double-float
 * (orthorhombic kernels) or FP64 (general kernels).  0 runs no task in plain
 * FP32.  Default 0.3. */
void grid_gb300_set_mixed_threshold(const grid_gb300_task_list *task_list,
                                    double threshold);
/* Share of the tasks (and of their grid points) that the mixed path
 * currently runs in plain FP32. */
void grid_gb300_mixed_split(const grid_gb300_task_list *task_list,
                            double *frac_tasks, double *frac_points);

/* Device-resident variants: pab/hab/grid pointers are device addresses
 * (FP64), grids[level] laid out x-fastest as npts_local.  The work is
 * enqueued on `stream` (a cudaStream_t passed as void*, NULL = the legacy
 * default stream); *_async return without synchronising. */
void grid_gb300_collocate_device_async(const grid_gb300_task_list *task_list,
                                       int func, const double *pab_blocks,
                                       double *const *grids, void *stream);
void grid_gb300_integrate_device_async(const grid_gb300_task_list *task_list,
                                       bool compute_tau,
                                       const double *pab_blocks,
                                       const double *const *grids,
                                       double *hab_blocks, double *forces,
                                       double *virial, void *stream);

/* The backend-level handle behind a task list made by grid_create_task_list,
 * for calling the grid_gb300_* extensions on it. */
grid_gb300_task_list *grid_gb300_backend_handle(const grid_task_list *task_list);

/* Number of tasks, levels, atoms and the pab/hab buffer length (doubles)
 * recorded at creation; any pointer may be NULL. */
void grid_gb300_task_list_info(const grid_gb300_task_list *task_list,
                               int *ntasks, int *nlevels, int *natoms,
                               long long *buffer_len);

/* Per-task analytic sizes in the caller's task order: grid points visited
 * and contraction order lp for collocation with func GRID_FUNC_AB. */
void grid_gb300_task_sizes(const grid_gb300_task_list *task_list,
                           long long *points, int *lp);

/* Kernel timing of the last call on this task list (milliseconds, CUDA
 * events on the launching stream; waits for that call to finish):
 * [0] coefficient kernels, [1] grid kernels, [2] post-processing,
 * [3] total device time. */
void grid_gb300_last_timings(const grid_gb300_task_list *task_list,
                             double timings_ms[4]);

/* Number of kernels this library launched on the device since load. */
long long grid_gb300_kernel_launches(void);

/* Autotuner: for the current precision, times SCF steps (collocate(func) +
 * integrate hab, device buffers, on `stream`) over the cube width that splits
 * small- from large-cube work queues (26, 34, 42, 66) and then, per work
 * queue, over launch shapes (warps per CTA 1/2/4, 50-100 % of the resident
 * CTAs, both collocate lane mappings), and keeps the fastest.  Results of later calls are unchanged up to
 * the order of floating-point atomic additions.  Returns the summed
 * grid-kernel time (ms) of the chosen shapes. */
double grid_gb300_autotune(const grid_gb300_task_list *task_list, int func,
                           const double *pab_blocks, double *const *rho_grids,
                           const double *const *v_grids, double *hab_blocks,
                           void *stream);
/* Lane mapping of the orthorhombic collocate kernel: 0 walks the rows of
 * each sphere plane with lanes bound to x; 1 walks the plane's points in
 * row-major order from a per-sphere point list, so that all lanes have work;
 * -1 (default) uses 1 for FP64 and double-float launches and 0 for plain
 * FP32 ones.  Same arithmetic; clears autotuned shapes. */
void grid_gb300_set_collocate_variant(const grid_gb300_task_list *task_list,
                                      int variant);
/* Cube width separating the small- and large-cube queues at the current
 * precision (default 34). */
int grid_gb300_tuned_split(const grid_gb300_task_list *task_list);
/* Host-buffer calls (grid_gb300_collocate_task_list / _integrate_task_list
 * and the CP2K surface) move pab in and hab out in `chunks` pieces (1..7,
 * default 3) on a copy stream, sizes growing 1 : 2 : 4 in block order, so
 * that the copies overlap the kernels of other pieces.  No counterpart in
 * CP2K (src/grid/gpu/grid_gpu_context.cu:509, 528, 645 copy whole buffers). */
void grid_gb300_set_copy_chunks(const grid_gb300_task_list *task_list, int chunks);
/* The grid-kernel launches of a collocate or integrate (one per work queue,
 * independent of each other) alternate over n streams (1 or 2, default 2):
 * the caller's stream and an auxiliary one forked from and joined back into
 * it, so that the tail of one launch overlaps the start of the next.  With
 * per-launch timing on they stay on one stream.  No counterpart in CP2K. */
void grid_gb300_set_queue_streams(const grid_gb300_task_list *task_list, int n);
/* Integration of the FP32 class (mixed mode) and of FP32 mode, orthorhombic
 * tasks with lp <= 6: 1 (default) runs the first contraction, over the x
 * points of each row of the sphere, as TF32 tensor-core matrix products
 * (mma.sync m16n8k8, operands split into high and low TF32 parts, three
 * products, about 21 bits per product); 0 runs the CUDA-core kernel.  No
 * counterpart in CP2K. */
void grid_gb300_set_tensor_integrate(const grid_gb300_task_list *task_list, int enable);
/* 1: in the mixed mode, FP32-class orthorhombic collocation with lp <= 6 on
 * the tensor cores (16 x by 8 rows of the sphere per mma.sync m16n8k8 tile,
 * the (ly, lz) pairs as the contraction, operands split as above, about 21
 * bits per product); 0 (default) runs the CUDA-core kernels, which are
 * faster on the measured workloads.  Plain FP32 mode always runs the
 * CUDA-core kernels.  No counterpart in CP2K. */
void grid_gb300_set_tensor_collocate(const grid_gb300_task_list *task_list, int enable);
/* Mixed mode: 1 (default) splits every orthorhombic double-float task by
 * rows.  The rows (j, k) farther from the Gaussian product's x axis than the
 * radius where the task's contribution bound falls to a third of the mixed
 * threshold run in FP32 (a second, FP32 pass over the task), the rows inside
 * stay double-float; 0 keeps every task whole in its class.  General-path
 * tasks stay whole.  No counterpart in CP2K. */
void grid_gb300_set_row_split(const grid_gb300_task_list *task_list, int enable);
/* The row split of a density collocation (no derivatives) in the mixed mode
 * at the current threshold: the share of tasks split, and the share of grid
 * points computed in FP32 (FP32-class tasks plus the outside rows of split
 * tasks, the latter estimated from the cylinder's volume share). */
void grid_gb300_row_split_stats(const grid_gb300_task_list *task_list,
                                double *frac_tasks_split, double *frac_points_fp32);
/* The row split's core for one primitive pair (host only, no GPU; for tests
 * and tuning): the squared radius (bohr^2) of the cylinder around the
 * Gaussian product's x axis outside which every row's contributions are at
 * most tau for density-matrix entries of magnitude <= 1 (the factor 2 of
 * pairs of different atoms included), with the l ranges raised by dla, dlb
 * (the derivatives of a call); *outside receives the share of the sphere's
 * points outside it.  Returns 3e38 when the pair stays whole.  Aborts on
 * invalid arguments. */
double grid_gb300_row_split_radius2(int la_min, int la_max, int lb_min, int lb_max,
                                    double zeta, double zetb, const double *rab,
                                    double radius, int same_atom, int dla, int dlb,
                                    double tau, double *outside);
/* C_ab <-> C_xyz change of basis of the coefficient and post kernels: 0 the
 * direct gather over all (a, b) pairs, 1 the staged per-direction
 * contractions (x, then y, then z), -1 (default) staged in the coefficient
 * kernel where la or lb >= 3 and direct in the post kernel.
 * No counterpart in CP2K (src/grid/ref/grid_ref_collint.h:827-911 runs the
 * direct loops); both give the same results up to rounding. */
void grid_gb300_set_transform_variant(const grid_gb300_task_list *task_list, int variant);

/* CUDA-graph capture of one SCF step on device buffers: collocate(func)
 * into rho_grids, then integrate v_grids into hab (forces / virial optional,
 * as for grid_gb300_integrate_device_async).  The capture first runs the step
 * once on `stream` (a created cudaStream_t as void*; the legacy default
 * stream cannot be captured) so that every work array exists, then records
 * the step's kernels and memsets as one graph.  A launch replays the step
 * with the same pointers; it fails if the task list's precision, schedule,
 * timing switches or internal arrays changed since capture.  Launches are
 * asynchronous; grid_gb300_step_graph_wait synchronises the stream and checks
 * the kernels' error word. */
typedef void grid_gb300_step_graph;
grid_gb300_step_graph *grid_gb300_capture_step(
    const grid_gb300_task_list *task_list, int func, const double *pab_blocks,
    double *const *rho_grids, bool compute_tau, const double *const *v_grids,
    double *hab_blocks, double *forces, double *virial, void *stream);
void grid_gb300_step_graph_launch(grid_gb300_step_graph *graph, void *stream);
void grid_gb300_step_graph_wait(grid_gb300_step_graph *graph, void *stream);
long long grid_gb300_step_graph_kernels(const grid_gb300_step_graph *graph);
void grid_gb300_step_graph_free(grid_gb300_step_graph *graph);

/* Per-launch timing of the grid kernels (off by default).  When enabled,
 * every collocate/integrate call records CUDA events around each grid-kernel
 * launch; grid_gb300_launch_timings waits for the last call and copies up to
 * `max` records, returning how many launches that call made. */
typedef struct {
  int phase;          /* 0 collocate, 1 integrate */
  int precision;      /* arithmetic of the launch: GRID_GB300_FP64 / _MIXED
                         (double-float) / _FP32 */
  int general;        /* 1: general (non-orthorhombic or border) kernel */
  int lp_bucket;      /* lp limit of the kernel instance (4, 6, 9, 12, 16) */
  int ntasks;         /* tasks in the launch */
  int warps_per_block;
  int blocks;
  long long points;   /* grid points the tasks visit */
  double flops;       /* sum over tasks of 2 (lp+1) points */
  double ms;          /* CUDA-event duration on the launching stream */
  int work_items;     /* work items: the tasks, counting a large task split
                         into plane ranges once per range */
} grid_gb300_launch_info;
void grid_gb300_set_launch_timing(const grid_gb300_task_list *task_list,
                                  int enable);
int grid_gb300_launch_timings(const grid_gb300_task_list *task_list, int max,
                              grid_gb300_launch_info *info);

/* ---- learned task-cost model ------------------------------------------
 * A 6 -> 64 -> 64 -> 1 MLP (SiLU, FP32) predicting log(task time) from the
 * task features below; its prediction orders the work queues under
 * GRID_GB300_SCHEDULE_MODEL.  Parameters are one flat FP32 device array of
 * grid_gb300_cost_model_nparams() words:
 *   W1[64][6] b1[64] W2[64][64] b2[64] w3[64] b3.
 * All pointers below are device pointers; work is enqueued on `stream`. */
int grid_gb300_cost_model_nparams(void);

/* Task features in the caller's task order, [ntasks][6] host floats:
 * la_max, lb_max, zeta_a + zeta_b, cube radius (grid points), level grid
 * spacing (bohr), cell skew (1 - |det h| / (|a| |b| |c|)). */
void grid_gb300_task_features(const grid_gb300_task_list *task_list,
                              float *features);

/* Per-task timing (off by default): when enabled, the grid kernels record
 * the clock64() cycles each task took; grid_gb300_task_cycles copies the
 * cycles of the last call in the caller's task order (0 for tasks that were
 * skipped). */
void grid_gb300_set_task_timing(const grid_gb300_task_list *task_list,
                                int enable);
void grid_gb300_task_cycles(const grid_gb300_task_list *task_list,
                            long long *cycles);

/* Training: loss = mean squared error of the prediction for the n samples
 * x[n][6] (standardised features) against targets t[n]; writes the loss
 * (one float) and its gradient (nparams floats).  `work` must hold
 * grid_gb300_cost_model_work_floats(n) floats.  Deterministic. */
size_t grid_gb300_cost_model_work_floats(int n);
void grid_gb300_cost_model_loss_grad(const float *params, const float *x,
                                     const float *t, int n, float *loss,
                                     float *grad, float *work, void *stream);
/* One Adam step (step counts from 1). */
void grid_gb300_cost_model_adam(float *params, const float *grad, float *m,
                                float *v, int step, float lr, float beta1,
                                float beta2, float eps, void *stream);
/* Inference: y[s] for raw features x[n][6] standardised on the fly by
 * norm = {mean[6], scale[6]} (NULL: none). */
void grid_gb300_cost_model_predict(const float *params, const float *x, int n,
                                   const float *norm, float *y, void *stream);
/* GRID_GB300_SCHEDULE_MODEL orders each queue by the predicted log time
 * quantised into bins of this width (default 0.2), and by the analytic size
 * inside a bin, which keeps tasks of one sphere together; 0 orders by the raw
 * prediction. */
void grid_gb300_set_model_bin_width(const grid_gb300_task_list *task_list,
                                    double width);
/* Predicts the cost of every task of the list with the given parameters
 * and normalisation (device pointers) and uses it for
 * GRID_GB300_SCHEDULE_MODEL.  Synchronises `stream`. */
void grid_gb300_apply_cost_model(const grid_gb300_task_list *task_list,
                                 const float *params, const float *norm,
                                 void *stream);

/* ---- single tasks (src/grid/grid_api.F:145, 318 bind these by name) ------
 * grid_cpu_collocate_pgf_product (src/grid/cpu/grid_cpu_collocate.h) and
 * grid_cpu_integrate_pgf_product (src/grid/cpu/grid_cpu_integrate.h): one
 * primitive pair on host buffers, same arguments and meaning; the work runs
 * on the GPU in FP64 (the block and the whole grid go to the device and
 * back; every output is accumulated into, as the reference does).  pab, hab:
 * [n2][n1]; forces [2][3] and virials [2][3][3] of atoms a and b; hdab,
 * hadb [n2][n1][3] and a_hdab [n2][n1][3][3] (not with compute_tau).
 * Synchronous; calls from several threads are serialised. */
void grid_cpu_collocate_pgf_product(
    const bool orthorhombic, const int border_mask, const enum grid_func func,
    const int la_max, const int la_min, const int lb_max, const int lb_min,
    const double zeta, const double zetb, const double rscale, const double *dh,
    const double *dh_inv, const double *ra, const double *rab, const int *npts_global,
    const int *npts_local, const int *shift_local, const int *border_width,
    const double radius, const int o1, const int o2, const int n1, const int n2,
    const double *pab, double *grid);
void grid_cpu_integrate_pgf_product(
    const bool orthorhombic, const bool compute_tau, const int border_mask, const int la_max,
    const int la_min, const int lb_max, const int lb_min, const double zeta, const double zetb,
    const double *dh, const double *dh_inv, const double *ra, const double *rab,
    const int *npts_global, const int *npts_local, const int *shift_local,
    const int *border_width, const double radius, const int o1, const int o2, const int n1,
    const int n2, const double *grid, double *hab, const double *pab, double *forces,
    double *virials, double *hdab, double *hadb, double *a_hdab);

/* Allocation-free collocation of one primitive pair, for callers that
 * cannot allocate device memory at call time (a program that gave the GPU's
 * memory to its own fixed arena at start-up, drivers that forbid cudaMalloc
 * after initialisation because it can synchronise the whole device).
 * No counterpart in CP2K; the arguments mean what they mean for
 * grid_cpu_collocate_pgf_product (src/grid/cpu/grid_cpu_collocate.h), with
 * pab ([n2][n1]) and grid (npts_local, x fastest; collocated values are
 * added) given as device pointers and the work enqueued on `stream`
 * (cudaStream_t as void*).  FP64 arithmetic.
 * All per-call scratch lives in one static __device__ array of
 * grid_gb300_static_scratch_bytes() bytes held by every GPU that loads the
 * library; no device memory is allocated.  Calls share that array: calls
 * whose kernels overlap on the GPU race, calls on one stream are ordered.
 * The first call on a device looks up the array's address and should come
 * before any stream capture.  Returns 0, or nonzero with a message in
 * grid_gb300_static_scratch_error() (the calling thread's last message) when
 * the task needs more scratch than the array holds, its cube or box exceeds
 * the kernels' shared memory, or an argument is out of range; these checks
 * run on the host before anything is copied or launched. */
int grid_gb300_collocate_pgf_product_static(
    const bool orthorhombic, const int border_mask, const int func,
    const int la_max, const int la_min, const int lb_max, const int lb_min,
    const double zeta, const double zetb, const double rscale,
    const double *dh, const double *dh_inv, const double *ra,
    const double *rab, const int *npts_global, const int *npts_local,
    const int *shift_local, const int *border_width, const double radius,
    const int o1, const int o2, const int n1, const int n2,
    const double *pab, double *grid, void *stream);
size_t grid_gb300_static_scratch_bytes(void);
const char *grid_gb300_static_scratch_error(void);

/* ---- plane-wave transfer of the multigrid levels (device resident) -------
 * The steps either side of collocate / integrate in a Quickstep SCF cycle:
 * density_rs2pw (src/pw_env/rs_pw_interface.F:64-136) and potential_pw2rs
 * (:151-228) with the default interpolation (pw_interp) on replicated grids,
 * so that rho -> plane-wave grid -> potential -> level grids stays in device
 * memory.  npts: [nlevels][3] (x, y, z) points per level, finest first; all
 * arrays device pointers, grids x fastest ([nz][ny][nx]); G-space arrays the
 * full complex box of the finest level (re, im pairs of doubles) in FFT
 * order, coefficients normalised by the number of points as the reference's
 * forward transform does.  Work is enqueued on `stream`. */
typedef struct grid_gb300_pw_transfer grid_gb300_pw_transfer;
void grid_gb300_pw_create(const int nlevels, const int *npts, grid_gb300_pw_transfer **handle);
void grid_gb300_pw_free(grid_gb300_pw_transfer *handle);
/* rho (finest grid, may be NULL) and rho_gspace (may be NULL) from the
 * collocated level grids: the sum over levels of their spectra on the
 * finest grid's frequencies, transformed back to real space. */
void grid_gb300_pw_density_rs2pw(grid_gb300_pw_transfer *handle, const double *const *rs_grids,
                                 double *rho, void *rho_gspace, void *stream);
/* The potential on every level grid from the potential on the finest grid:
 * the finest level copies it, coarser levels take its coefficients at their
 * frequencies, transform back and scale by dvol(level) / dvol(finest). */
void grid_gb300_pw_potential_pw2rs(grid_gb300_pw_transfer *handle, const double *v_rspace,
                                   double *const *rs_grids, void *stream);
/* potential_pw2rs from the finest grid's G-space coefficients (the layout
 * of rho_gspace above, e.g. grid_gb300_pw_poisson's v_gspace): the same
 * level grids without the forward transform of the finest grid. */
void grid_gb300_pw_potential_g2rs(grid_gb300_pw_transfer *handle, const void *v_gspace,
                                  double *const *rs_grids, void *stream);
/* Periodic Hartree solve on the finest grid's G-space box (the layout of
 * rho_gspace above): v(G) = 4 pi rho(G) / |G|^2, v(0) = 0, with G = 2 pi
 * sum_d f_d b_d over the grid's frequencies and b_d the reciprocal vectors
 * of the cell whose vectors are a_d = n_d dh[d][:] (dh: the finest level's
 * spacing matrix, row d the step along lattice vector d; n_d its points)
 * (src/pw/pw_poisson_types.F:316-320, PERIODIC3D).  rho_gspace and v_gspace
 * may be the same buffer.  v_rspace (may be NULL) receives v on the finest
 * grid in real space, ready for grid_gb300_pw_potential_pw2rs.  energy
 * (host, may be NULL) receives the Hartree energy 0.5 Omega sum
 * conj(rho(G)) v(G) (src/pw/pw_poisson_methods.F:363-367); asking for it
 * synchronises the stream. */
void grid_gb300_pw_poisson(grid_gb300_pw_transfer *handle, const double *dh,
                           const void *rho_gspace, void *v_gspace, double *v_rspace,
                           double *energy, void *stream);

/* ---- task-list generation and block packing on the device ---------------
 * Replaces, for one geometry, the work of Quickstep's generate_qs_task_list
 * (src/task_list_methods.F:117-501; task_list_inner_loop :652-719,
 * compute_pgf_properties :738-800, the API arrays :507-618): every atom pair
 * i <= j and periodic image n (-nimages[d] .. nimages[d] along cell vector d;
 * for i == j image 0 and one of each +/- n pair) with |rab| <= rmax, every
 * primitive pair (iset, ipgf, jset, jpgf) whose Gaussian-product prefactor
 * exp(-zeta zetb / zetp |rab|^2) exceeds eps, in that order; the level of
 * gaussian_gridlevel (src/pw_env/gaussian_gridlevels.F:147-167, cutoff[] in
 * the units of zetp * rel_cutoff, finest first); the radius of
 * exp_radius_very_extended (src/aobasis/ao_util.F:207-290); one block per
 * atom pair with tasks, numbered in pair order, at offset sum nsgf(i)
 * nsgf(j) of the blocks before it.  The basis is uploaded once; runs take
 * new positions (a moved geometry) and leave the arrays of
 * grid_create_task_list (1-based indices, rab [ntasks][3]) in device memory.
 * Sets and primitives: set_lmax and set_npgf hold every kind's sets, kind
 * after kind ([sum nset]); zet [sum nset][maxpgf].  Cell rows are the cell
 * vectors (bohr).  Invalid arguments abort with a message. */
typedef void grid_gb300_task_generator;
void grid_gb300_taskgen_create(
    const int natoms, const int nkinds, const int *atom_kinds, const int *nset,
    const int *nsgf, const int *set_lmax, const int *set_npgf, const int maxpgf,
    const double *zet, const double *cell, const int *nimages, const double rmax,
    const double eps, const int nlevels, const double *cutoff, const double rel_cutoff,
    grid_gb300_task_generator **generator);
void grid_gb300_taskgen_free(grid_gb300_task_generator *generator);
/* Screen primitive pairs by the basis radii as Quickstep does
 * (task_list_methods.F:673-696: set_radius(a) + kind_radius(b),
 * set_radius(a) + set_radius(b), pgf_radius(a) + set_radius(b),
 * pgf_radius(a) + pgf_radius(b) against |rab|, loop order iset, jset, ipgf,
 * jpgf) instead of by the prefactor: pgf_radius [sum nset][maxpgf],
 * set_radius [sum nset], kind_radius [nkinds], the basis set's radii
 * (qs_interactions.F:472-492). */
void grid_gb300_taskgen_set_radius_screen(grid_gb300_task_generator *generator,
                                          const double *pgf_radius, const double *set_radius,
                                          const double *kind_radius);
/* Generates the task list for atom_positions ([natoms][3], bohr; a device
 * pointer when on_device != 0, else host); returns the task and block counts
 * and the pab buffer length (doubles).  Synchronises the stream. */
void grid_gb300_taskgen_run(grid_gb300_task_generator *generator,
                            const double *atom_positions, const int on_device,
                            void *stream, int *ntasks, int *nblocks,
                            long long *buffer_size);
/* Device pointers of the last run's arrays (valid until the next run or
 * free); any argument may be NULL. */
void grid_gb300_taskgen_arrays(const grid_gb300_task_generator *generator,
                               int **level, int **iatom, int **jatom, int **iset,
                               int **jset, int **ipgf, int **jpgf, int **border_mask,
                               int **block_num, double **radius, double **rab,
                               int **block_offsets);
/* The same arrays copied to host memory (caller-sized: ntasks, 3 ntasks for
 * rab, nblocks for block_offsets); any argument may be NULL. */
void grid_gb300_taskgen_copy(const grid_gb300_task_generator *generator, int *level,
                             int *iatom, int *jatom, int *iset, int *jset, int *ipgf,
                             int *jpgf, int *border_mask, int *block_num, double *radius,
                             double *rab, int *block_offsets);
/* grid_gb300_create_task_list on the last run's arrays and positions (a
 * non-NULL *task_list is re-created in place, keeping its settings). */
void grid_gb300_taskgen_create_task_list(
    grid_gb300_task_generator *generator, const bool orthorhombic, const int nlevels,
    const grid_basis_set **basis_sets, const int *npts_global, const int *npts_local,
    const int *shift_local, const int *border_width, const double *dh, const double *dh_inv,
    grid_gb300_task_list **task_list);
/* rs_pack_buffer (src/task_list_methods.F:2593-2619) on device memory: block
 * b, sizes[b] doubles at src + src_offsets[b], is copied to dst +
 * dst_offsets[b] (the task list's block offsets).  Enqueued on `stream`. */
void grid_gb300_pack_blocks(const long long nblocks, const long long *src_offsets,
                            const int *dst_offsets, const int *sizes, const double *src,
                            double *dst, void *stream);
/* rs_unpack_buffer (:2625-2674): blocks[block_offsets[b] + k] +=
 * buffer[buffer_offsets[b] + k] for k < sizes[b].  The target blocks must
 * not overlap (one entry per block, as in the reference's atom-pair list). */
void grid_gb300_unpack_blocks(const long long nblocks, const int *buffer_offsets,
                              const long long *block_offsets, const int *sizes,
                              const double *buffer, double *blocks, void *stream);
/* dbcsr_get_block_p for many blocks at once: offsets[q] = key_offsets[k] for
 * the key k with (key_rows[k], key_cols[k]) == (rows[q], cols[q]), keys
 * sorted by row, then column; -1 where absent.  Returns the number of
 * absent blocks (the reference asserts found); synchronises the stream.
 * All arrays are device pointers. */
long long grid_gb300_find_blocks(const long long nkeys, const int *key_rows,
                                 const int *key_cols, const long long *key_offsets,
                                 const long long nquery, const int *rows, const int *cols,
                                 long long *offsets, void *stream);

/* Last error message recorded by the library ("" if none). */
const char *grid_gb300_last_error(void);

/* ---- testing ---------------------------------------------------------------
 * Runs the host-side preparation of grid_gb300_create_task_list (ordering,
 * per-task geometry, class bounds, features, sphere tables, subblocks)
 * without touching the GPU, and returns FNV-1a hashes of the prepared
 * arrays: digest[0..9] tasks, 0 (the recurrence seeds are computed on the
 * device), class bounds, features, point
 * counts, subblocks, sphere headers, sphere tables, sphere points, point
 * offsets; digest[10] the Cartesian scratch size; digest[11] the number of
 * tasks whose class bound is <= 0.3.  The preparation runs on the host's
 * cores; GRID_GB300_HOST_THREADS fixes their number. */
void grid_gb300_host_digest(
    const bool orthorhombic, const int ntasks, const int nlevels, const int natoms,
    const int nkinds, const int nblocks, const int *block_offsets, const double *atom_positions,
    const int *atom_kinds, const grid_basis_set **basis_sets, const int *level_list,
    const int *iatom_list, const int *jatom_list, const int *iset_list, const int *jset_list,
    const int *ipgf_list, const int *jpgf_list, const int *border_mask_list,
    const int *block_num_list, const double *radius_list, const double *rab_list,
    const int *npts_global, const int *npts_local, const int *shift_local,
    const int *border_width, const double *dh, const double *dh_inv,
    unsigned long long digest[12]);

#ifdef __cplusplus
}
#endif

#endif /* GRID_GB300_H */
