/*
 * TEST INFRASTRUCTURE -- the CPU oracle.  Not product code: only tests/,
 * __graft_entry__.smoke() and bench.py's cpu_baseline / reference legs may
 * load it, and only as the checker or the timed CPU baseline.
 *
 * A plain-C, FP64 restatement of CP2K's REF grid backend
 * (src/grid/ref/grid_ref_task_list.c, grid_ref_collint.h,
 * grid_ref_collocate.c, grid_ref_integrate.c, common/grid_prepare_pab.h,
 * common/grid_process_vab.h).  Parity of this restatement is pinned by the
 * tests against the reference's sample_tasks .task golden vectors and
 * against the reference library itself (oracle/_ref) on synthetic task lists.
 */
#ifndef GRID_ORACLE_H
#define GRID_ORACLE_H

#include <stdbool.h>
#include <stddef.h>

/* Same field layout as the reference's grid_basis_set
 * (src/grid/common/grid_basis_set.h:14-26). */
typedef struct {
  int nset, nsgf, maxco, maxpgf;
  int *lmin, *lmax, *npgf, *nsgf_set, *first_sgf;
  double *sphi; /* [nsgf][maxco] */
  double *zet;  /* [nset][maxpgf] */
} oracle_basis;

void oracle_create_basis_set(int nset, int nsgf, int maxco, int maxpgf,
                             const int *lmin, const int *lmax, const int *npgf,
                             const int *nsgf_set, const int *first_sgf,
                             const double *sphi, const double *zet,
                             oracle_basis **out);
void oracle_free_basis_set(oracle_basis *b);

/* Arguments as grid_create_task_list (src/grid/grid_task_list.h:59-72):
 * 1-based task lists, row-major [n][3] / [n][3][3] arrays. */
void oracle_create_task_list(
    bool orthorhombic, int ntasks, int nlevels, int natoms, int nkinds,
    int nblocks, const int *block_offsets, const double *atom_positions,
    const int *atom_kinds, const oracle_basis *const *basis_sets,
    const int *level_list, const int *iatom_list, const int *jatom_list,
    const int *iset_list, const int *jset_list, const int *ipgf_list,
    const int *jpgf_list, const int *border_mask_list,
    const int *block_num_list, const double *radius_list,
    const double *rab_list, const int *npts_global, const int *npts_local,
    const int *shift_local, const int *border_width, const double *dh,
    const double *dh_inv, void **task_list);
void oracle_free_task_list(void *task_list);

/* grid_collocate_task_list semantics: grids are overwritten. */
void oracle_collocate_task_list(const void *task_list, int func, int nlevels,
                                const double *pab_blocks, double **grids);

/* grid_integrate_task_list semantics: hab (hab_len doubles), forces
 * [natoms][3] and virial [3][3] are overwritten; forces/virial may be NULL. */
void oracle_integrate_task_list(const void *task_list, bool compute_tau,
                                int natoms, int nlevels,
                                const double *pab_blocks,
                                const double *const *grids, double *hab_blocks,
                                size_t hab_len, double *forces,
                                double *virial);

/* Single-task entry points with the argument meaning of
 * grid_ref_collocate_pgf_product / grid_ref_integrate_pgf_product
 * (src/grid/ref/grid_ref_collocate.h, grid_ref_integrate.h).
 * pab/hab are [n2][n1]; forces [2][3]; virials [2][3][3]; hdab, hadb
 * [n2][n1][3] and a_hdab [n2][n1][3][3] (may be NULL). */
void oracle_collocate_pgf_product(
    bool orthorhombic, int border_mask, int func, int la_max, int la_min,
    int lb_max, int lb_min, double zeta, double zetb, double rscale,
    const double *dh, const double *dh_inv, const double *ra,
    const double *rab, const int *npts_global, const int *npts_local,
    const int *shift_local, const int *border_width, double radius, int o1,
    int o2, int n1, int n2, const double *pab, double *grid);

void oracle_integrate_pgf_product(
    bool orthorhombic, bool compute_tau, int border_mask, int la_max,
    int la_min, int lb_max, int lb_min, double zeta, double zetb,
    const double *dh, const double *dh_inv, const double *ra,
    const double *rab, const int *npts_global, const int *npts_local,
    const int *shift_local, const int *border_width, double radius, int o1,
    int o2, int n1, int n2, const double *grid, double *hab,
    const double *pab, double *forces, double *virials, double *hdab,
    double *hadb, double *a_hdab);

/* Number of grid points the oracle's loops visit for every task of the list
 * (in the caller's task order), with the cube-to-grid contraction order lp
 * that collocation with func uses.  Used for the algorithmic FLOP count.
 * Returns the total. */
long long oracle_count_task_points(const void *task_list, int func,
                                   long long *points_out, int *lp_out);

#endif
