/*
 * Synthetic GPW task-list generator.
 *
 * Produces exactly the argument arrays of grid_create_task_list for a seeded
 * random system, restating how CP2K's Quickstep builds them:
 *   - pair screening per (iset, jset, ipgf, jpgf) by the Gaussian-product
 *     prefactor exp(-zeta*zetb/zetp * |rab|^2) > eps
 *     (task_list_methods.F:652-719, task_list_inner_loop);
 *   - the task radius from exp_radius_very_extended (aobasis/ao_util.F:207-290)
 *     and exp_radius (ao_util.F:95-180), with the same single-precision
 *     exponential and interval contraction;
 *   - the grid level from gaussian_gridlevel (pw_env/gaussian_gridlevels.F:
 *     147-167): the coarsest level whose cutoff still covers zetp*rel_cutoff;
 *   - one matrix block per atom pair (i <= j); periodic images are encoded in
 *     rab (task_list_methods.F:507-618).
 * Every atom is its own kind (own exponents), so the task shapes are uneven.
 * Host-only C, portable (x86-64 and aarch64).
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define WL_MAX_LEVELS 8
#define WL_MAX_ELEM 2
#define WL_MAX_SETS 4

typedef struct {
  uint64_t seed;
  int natoms;
  double cell[3][3]; /* rows: cell vectors, bohr */
  int nlevels;
  int npts[WL_MAX_LEVELS][3];
  double cutoff[WL_MAX_LEVELS]; /* finest first */
  double rel_cutoff;
  double eps;
  int nelem;
  double elem_fraction[WL_MAX_ELEM]; /* share of atoms, first element first */
  int nsets[WL_MAX_ELEM];
  int set_lmax[WL_MAX_ELEM][WL_MAX_SETS];
  double zet_min, zet_max;
  int random_sphi; /* 0: identity contraction, 1: random orthonormal rows */
  int npgf[WL_MAX_ELEM]; /* primitives per set */
  /* 0: primitive pairs screened by prefactor > eps (the benchmark
   * workloads); 1: by the basis radii as Quickstep does
   * (task_list_methods.F:673-696), in its loop order iset, jset, ipgf,
   * jpgf, with the radii of qs_interactions.F:472-492 (every shell
   * coefficient 1, threshold eps_pgf_orb) */
  int screen;
  double eps_pgf_orb;
} wl_params;

typedef struct {
  int natoms, nkinds, ntasks, nblocks, nlevels;
  long long buffer_size;
  double *atom_positions; /* [natoms][3] */
  int *atom_kinds;        /* [natoms] (1-based) */
  /* per kind basis */
  int *nset, *nsgf, *maxco, *maxpgf; /* [nkinds] */
  int *set_off;                      /* [nkinds] offset into set arrays */
  int *lmin, *lmax, *npgf, *nsgf_set, *first_sgf; /* [sum nset] */
  int *sphi_off;                     /* [nkinds] offset into sphi */
  double *sphi;                      /* concatenated [nsgf][maxco] */
  double *zet;                       /* [sum nset][maxpgf_all] */
  int maxpgf_all;
  int *block_offsets;                /* [nblocks] */
  int *level, *iatom, *jatom, *iset, *jset, *ipgf, *jpgf, *border_mask,
      *block_num;                    /* [ntasks] */
  double *radius, *rab;              /* [ntasks], [ntasks][3] */
  double dh[WL_MAX_LEVELS][3][3], dh_inv[WL_MAX_LEVELS][3][3];
  int nimg[3];  /* periodic images searched per cell vector: -nimg..nimg */
  double rmax;  /* pair distance cut (bohr) */
  /* basis radii (screen 1): [sum nset][maxpgf_all], [sum nset], [nkinds] */
  double *rpgf, *set_radius, *kind_radius;
} wl_out;

/* --------------------------------------------------------------- random -- */
static uint64_t sm64(uint64_t *s) {
  uint64_t z = (*s += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
static double urand(uint64_t *s) { return (double)(sm64(s) >> 11) * 0x1.0p-53; }

static inline int ncoset(int l) { return l < 0 ? 0 : (l + 1) * (l + 2) * (l + 3) / 6; }

/* ---------------------------------------------------- radius (ao_util.F) -- */
static double g_eval(double d, double a, double r, int l) {
  return d * (double)expf((float)(-a * r * r)) * pow(r, l);
}

static double exp_radius(int l, double alpha, double threshold, double prefactor,
                         double epsabs, double rlow) {
  const int itermax = 5000;
  const double contract[2] = {(double)0.38f, (double)0.62f};
  const double a = fabs(alpha), t = fabs(threshold);
  double radius = rlow;
  if (prefactor == 0.0)
    return radius;
  double r = fmax(sqrt(0.5 * (double)l / a), radius);
  const double d = fabs(prefactor);
  double g = d;
  if (l != 0)
    g = g_eval(d, a, r, l);
  if (g < t)
    return radius;
  radius = r * 2.0 + 1.0;
  int i;
  for (i = 1; i <= itermax; i++) {
    if (g_eval(d, a, radius, l) < t)
      break;
    r = radius;
    radius = r * 2.0 + 1.0;
  }
  double dr = 0.0;
  for (i = i + 1; i <= itermax; i++) {
    const double rd = radius - r;
    if (rd < epsabs || rd == dr)
      return radius;
    double s[2];
    for (int j = 0; j < 2; j++)
      s[j] = r + rd * contract[j];
    for (int j = 0; j < 2; j++) {
      if (g_eval(d, a, s[j], l) < t) {
        radius = s[j];
        break;
      }
      r = s[j];
    }
    dr = rd;
  }
  return radius;
}

static double exp_radius_very_extended(int la_max, int lb_max, const double ra[3],
                                       const double rb[3], const double rp[3],
                                       double zetp, double eps, double prefactor) {
  double rad_a = 0.0, rad_b = 0.0;
  for (int d = 0; d < 3; d++) {
    rad_a += (ra[d] - rp[d]) * (ra[d] - rp[d]);
    rad_b += (rb[d] - rp[d]) * (rb[d] - rp[d]);
  }
  rad_a = sqrt(rad_a);
  rad_b = sqrt(rad_b);
  double poly[64] = {0};
  for (int lxa = 0; lxa <= la_max; lxa++)
    for (int lxb = 0; lxb <= lb_max; lxb++) {
      double coef[64] = {0};
      double bini = 1.0, s1 = 1.0;
      for (int i = 0; i <= lxa; i++) {
        double binj = 1.0, s2 = 1.0;
        for (int j = 0; j <= lxb; j++) {
          coef[lxa + lxb - i - j] += bini * binj * s1 * s2;
          binj = (binj * (lxb - j)) / (j + 1);
          s2 *= rad_b;
        }
        bini = (bini * (lxa - i)) / (i + 1);
        s1 *= rad_a;
      }
      for (int i = 0; i <= lxa + lxb; i++)
        poly[i] = fmax(poly[i], coef[i]);
    }
  double radius = 0.0;
  for (int i = 0; i <= la_max + lb_max; i++)
    radius = fmax(radius, exp_radius(i, zetp, eps, poly[i] * prefactor, 1.0e-2, radius));
  return radius;
}

static int grid_level(const wl_params *p, double zetp) {
  int lev = 1;
  const double need = fabs(zetp) * p->rel_cutoff;
  for (int i = 1; i <= p->nlevels; i++)
    if (p->cutoff[i - 1] + 1e-6 >= need)
      lev = i;
  return lev;
}

static void inv3(const double m[3][3], double r[3][3]) {
  const double det = m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]) -
                     m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0]) +
                     m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
  r[0][0] = (m[1][1] * m[2][2] - m[1][2] * m[2][1]) / det;
  r[0][1] = (m[0][2] * m[2][1] - m[0][1] * m[2][2]) / det;
  r[0][2] = (m[0][1] * m[1][2] - m[0][2] * m[1][1]) / det;
  r[1][0] = (m[1][2] * m[2][0] - m[1][0] * m[2][2]) / det;
  r[1][1] = (m[0][0] * m[2][2] - m[0][2] * m[2][0]) / det;
  r[1][2] = (m[0][2] * m[1][0] - m[0][0] * m[1][2]) / det;
  r[2][0] = (m[1][0] * m[2][1] - m[1][1] * m[2][0]) / det;
  r[2][1] = (m[0][1] * m[2][0] - m[0][0] * m[2][1]) / det;
  r[2][2] = (m[0][0] * m[1][1] - m[0][1] * m[1][0]) / det;
}

/* growable int/double arrays for the task lists */
typedef struct {
  void *p;
  size_t n, cap, elem;
} vec;
static void vpush(vec *v, const void *x) {
  if (v->n == v->cap) {
    v->cap = v->cap ? 2 * v->cap : 4096;
    v->p = realloc(v->p, v->cap * v->elem);
    if (!v->p) {
      fprintf(stderr, "workload: out of memory\n");
      abort();
    }
  }
  memcpy((char *)v->p + v->n * v->elem, x, v->elem);
  v->n++;
}

/* Random orthogonal n x n matrix (Gram-Schmidt on uniform entries). */
static void random_orthogonal(int n, uint64_t *s, double *q) {
  for (int i = 0; i < n * n; i++)
    q[i] = 2.0 * urand(s) - 1.0;
  for (int r = 0; r < n; r++) {
    for (int k = 0; k < r; k++) {
      double dot = 0.0;
      for (int c = 0; c < n; c++)
        dot += q[r * n + c] * q[k * n + c];
      for (int c = 0; c < n; c++)
        q[r * n + c] -= dot * q[k * n + c];
    }
    double nrm = 0.0;
    for (int c = 0; c < n; c++)
      nrm += q[r * n + c] * q[r * n + c];
    nrm = sqrt(nrm);
    for (int c = 0; c < n; c++)
      q[r * n + c] /= nrm;
  }
}

/* The task arrays for the atom positions in o->atom_positions: every atom
 * pair i <= j, every periodic image within rmax, every primitive pair that
 * passes the prefactor screen, in that order.  Replaces any earlier arrays. */
static void build_tasks(wl_out *o, const wl_params *p) {
  const int na = o->natoms;
  const int maxpgf_all = o->maxpgf_all;
  void *old[] = {o->block_offsets, o->level, o->iatom, o->jatom, o->iset, o->jset,
                 o->ipgf, o->jpgf, o->border_mask, o->block_num, o->radius, o->rab};
  for (size_t q = 0; q < sizeof(old) / sizeof(old[0]); q++)
    free(old[q]);
  /* image range from the most diffuse possible product (screen 0), or
   * from the largest sum of two kind radii (screen 1) */
  const double ln_eps = log(1.0 / p->eps);
  double rmax = sqrt(ln_eps / (0.5 * p->zet_min));
  if (p->screen == 1) {
    double kr = 0.0;
    for (int k = 0; k < o->nkinds; k++)
      kr = fmax(kr, o->kind_radius[k]);
    rmax = 2.0 * kr;
  }
  double cinv[3][3];
  inv3(p->cell, cinv);
  int nimg[3];
  for (int d = 0; d < 3; d++) {
    const double h = sqrt(cinv[0][d] * cinv[0][d] + cinv[1][d] * cinv[1][d] +
                          cinv[2][d] * cinv[2][d]);
    nimg[d] = (int)ceil(rmax * h) + 1;
    o->nimg[d] = nimg[d];
  }
  o->rmax = rmax;
  vec vi[9], vr = {0, 0, 0, sizeof(double)}, vrab = {0, 0, 0, 3 * sizeof(double)},
             vblk = {0, 0, 0, sizeof(int)};
  for (int q = 0; q < 9; q++) {
    vi[q].p = NULL;
    vi[q].n = vi[q].cap = 0;
    vi[q].elem = sizeof(int);
  }
  long long offset = 0;
  int nblocks = 0;
  for (int i = 0; i < na; i++) {
    const double *ra = &o->atom_positions[3 * i];
    for (int j = i; j < na; j++) {
      const double *rj = &o->atom_positions[3 * j];
      int block = 0;
      for (int n0i = -nimg[0]; n0i <= nimg[0]; n0i++)
        for (int n1i = -nimg[1]; n1i <= nimg[1]; n1i++)
          for (int n2i = -nimg[2]; n2i <= nimg[2]; n2i++) {
            if (i == j) { /* same atom: image 0 and one of each +/- pair */
              const int lex = n0i != 0 ? n0i : (n1i != 0 ? n1i : n2i);
              if (lex < 0)
                continue;
            }
            double rab[3];
            for (int d = 0; d < 3; d++)
              rab[d] = rj[d] - ra[d] + n0i * p->cell[0][d] + n1i * p->cell[1][d] +
                       n2i * p->cell[2][d];
            const double rab2 = rab[0] * rab[0] + rab[1] * rab[1] + rab[2] * rab[2];
            if (rab2 > rmax * rmax)
              continue;
            if (p->screen == 1) {
              /* task_list_inner_loop (task_list_methods.F:673-696) */
              const double dab = sqrt(rab2);
              const double krb = o->kind_radius[j];
              for (int is = 0; is < o->nset[i]; is++) {
                const int gi = o->set_off[i] + is;
                if (o->set_radius[gi] + krb < dab)
                  continue;
                for (int js = 0; js < o->nset[j]; js++) {
                  const int gj = o->set_off[j] + js;
                  if (o->set_radius[gi] + o->set_radius[gj] < dab)
                    continue;
                  for (int ip = 0; ip < o->npgf[gi]; ip++) {
                    const double rpa = o->rpgf[(size_t)gi * maxpgf_all + ip];
                    if (rpa + o->set_radius[gj] < dab)
                      continue;
                    const double za = o->zet[(size_t)gi * maxpgf_all + ip];
                    for (int jp = 0; jp < o->npgf[gj]; jp++) {
                      if (rpa + o->rpgf[(size_t)gj * maxpgf_all + jp] < dab)
                        continue;
                      const double zb = o->zet[(size_t)gj * maxpgf_all + jp];
                      const double zetp = za + zb, f = zb / zetp;
                      const double pref = exp(-za * f * rab2);
                      double rp[3], rb[3];
                      for (int d = 0; d < 3; d++) {
                        rp[d] = ra[d] + f * rab[d];
                        rb[d] = ra[d] + rab[d];
                      }
                      const double radius = exp_radius_very_extended(
                          o->lmax[gi], o->lmax[gj], ra, rb, rp, zetp, p->eps, pref);
                      if (!block) {
                        block = ++nblocks;
                        const int off = (int)offset;
                        vpush(&vblk, &off);
                        offset += (long long)o->nsgf[i] * o->nsgf[j];
                      }
                      const int v[9] = {grid_level(p, zetp), i + 1, j + 1, is + 1, js + 1,
                                        ip + 1, jp + 1, 0, block};
                      for (int q = 0; q < 9; q++)
                        vpush(&vi[q], &v[q]);
                      vpush(&vr, &radius);
                      vpush(&vrab, rab);
                    }
                  }
                }
              }
              continue;
            }
            for (int is = 0; is < o->nset[i]; is++)
            for (int ip = 0; ip < o->npgf[o->set_off[i] + is]; ip++) {
              const int gi = o->set_off[i] + is;
              const double za = o->zet[(size_t)gi * maxpgf_all + ip];
              for (int js = 0; js < o->nset[j]; js++)
              for (int jp = 0; jp < o->npgf[o->set_off[j] + js]; jp++) {
                const int gj = o->set_off[j] + js;
                const double zb = o->zet[(size_t)gj * maxpgf_all + jp];
                const double zetp = za + zb, f = zb / zetp;
                const double pref = exp(-za * f * rab2);
                if (!(pref > p->eps))
                  continue;
                double rp[3], rb[3];
                for (int d = 0; d < 3; d++) {
                  rp[d] = ra[d] + f * rab[d];
                  rb[d] = ra[d] + rab[d];
                }
                const double radius = exp_radius_very_extended(
                    o->lmax[gi], o->lmax[gj], ra, rb, rp, zetp, p->eps, pref);
                if (!block) {
                  block = ++nblocks;
                  const int off = (int)offset;
                  vpush(&vblk, &off);
                  offset += (long long)o->nsgf[i] * o->nsgf[j];
                }
                const int v[9] = {grid_level(p, zetp), i + 1, j + 1, is + 1, js + 1,
                                  ip + 1, jp + 1, 0, block};
                for (int q = 0; q < 9; q++)
                  vpush(&vi[q], &v[q]);
                vpush(&vr, &radius);
                vpush(&vrab, rab);
              }
            }
          }
    }
  }
  if (offset > 2147483647LL) {
    fprintf(stderr, "workload: block buffer exceeds int offsets\n");
    abort();
  }
  o->ntasks = (int)vr.n;
  o->nblocks = nblocks;
  o->buffer_size = offset;
  o->block_offsets = vblk.p;
  int **dst[9] = {&o->level, &o->iatom, &o->jatom, &o->iset, &o->jset,
                  &o->ipgf, &o->jpgf, &o->border_mask, &o->block_num};
  for (int q = 0; q < 9; q++)
    *dst[q] = vi[q].p;
  o->radius = vr.p;
  o->rab = vrab.p;
}

wl_out *wl_generate(const wl_params *p) {
  if (p->nlevels < 1 || p->nlevels > WL_MAX_LEVELS || p->nelem < 1 ||
      p->nelem > WL_MAX_ELEM || p->natoms < 1)
    return NULL;
  uint64_t s = p->seed;
  wl_out *o = calloc(1, sizeof(wl_out));
  const int na = p->natoms;
  o->natoms = na;
  o->nkinds = na; /* one kind per atom */
  o->nlevels = p->nlevels;
  /* element of each atom: the first round(f0*natoms) atoms are element 0 */
  int *elem = malloc(sizeof(int) * na);
  const int n0 = p->nelem == 1 ? na : (int)floor(p->elem_fraction[0] * na + 0.5);
  for (int i = 0; i < na; i++)
    elem[i] = (i < n0) ? 0 : 1;
  /* positions: uniform fractional coordinates */
  o->atom_positions = malloc(sizeof(double) * 3 * na);
  o->atom_kinds = malloc(sizeof(int) * na);
  for (int i = 0; i < na; i++) {
    double f[3];
    for (int d = 0; d < 3; d++)
      f[d] = urand(&s);
    for (int d = 0; d < 3; d++)
      o->atom_positions[3 * i + d] =
          f[0] * p->cell[0][d] + f[1] * p->cell[1][d] + f[2] * p->cell[2][d];
    o->atom_kinds[i] = i + 1;
  }
  /* basis sets */
  int totsets = 0;
  for (int i = 0; i < na; i++)
    totsets += p->nsets[elem[i]];
  o->nset = malloc(sizeof(int) * na);
  o->nsgf = malloc(sizeof(int) * na);
  o->maxco = malloc(sizeof(int) * na);
  o->maxpgf = malloc(sizeof(int) * na);
  o->set_off = malloc(sizeof(int) * na);
  o->sphi_off = malloc(sizeof(int) * na);
  o->lmin = malloc(sizeof(int) * totsets);
  o->lmax = malloc(sizeof(int) * totsets);
  o->npgf = malloc(sizeof(int) * totsets);
  o->nsgf_set = malloc(sizeof(int) * totsets);
  o->first_sgf = malloc(sizeof(int) * totsets);
  int maxpgf_all = 1;
  for (int e = 0; e < p->nelem; e++)
    if (p->npgf[e] > maxpgf_all)
      maxpgf_all = p->npgf[e];
  o->maxpgf_all = maxpgf_all;
  o->zet = calloc((size_t)totsets * maxpgf_all, sizeof(double));
  long long sphi_total = 0;
  int so = 0;
  const double lzmin = log(p->zet_min), lzmax = log(p->zet_max);
  for (int i = 0; i < na; i++) {
    const int e = elem[i];
    o->nset[i] = p->nsets[e];
    o->set_off[i] = so;
    int nsgf = 0, maxco = 0;
    const int np = p->npgf[e] > 0 ? p->npgf[e] : 1;
    for (int k = 0; k < p->nsets[e]; k++) {
      const int L = p->set_lmax[e][k];
      const int nsf = p->random_sphi ? ncoset(L) : np * ncoset(L);
      o->lmin[so + k] = 0;
      o->lmax[so + k] = L;
      o->npgf[so + k] = np;
      o->nsgf_set[so + k] = nsf;
      o->first_sgf[so + k] = nsgf + 1;
      for (int q = 0; q < np; q++)
        o->zet[(size_t)(so + k) * maxpgf_all + q] = exp(lzmin + urand(&s) * (lzmax - lzmin));
      nsgf += nsf;
      if (np * ncoset(L) > maxco)
        maxco = np * ncoset(L);
    }
    o->nsgf[i] = nsgf;
    o->maxco[i] = maxco;
    o->maxpgf[i] = maxpgf_all;
    o->sphi_off[i] = (int)sphi_total;
    sphi_total += (long long)nsgf * maxco;
    so += p->nsets[e];
  }
  o->sphi = calloc(sphi_total, sizeof(double));
  for (int i = 0; i < na; i++) {
    double *sp = &o->sphi[o->sphi_off[i]];
    for (int k = 0; k < o->nset[i]; k++) {
      const int n = o->nsgf_set[o->set_off[i] + k], r0 = o->first_sgf[o->set_off[i] + k] - 1;
      if (p->random_sphi) {
        /* n contracted functions over npgf*n Cartesian primitives:
         * rows of a random orthogonal matrix of that width */
        const int m = o->npgf[o->set_off[i] + k] * n;
        double *q = malloc(sizeof(double) * m * m);
        random_orthogonal(m, &s, q);
        for (int r = 0; r < n; r++)
          for (int c = 0; c < m; c++)
            sp[(size_t)(r0 + r) * o->maxco[i] + c] = q[r * m + c];
        free(q);
      } else {
        for (int r = 0; r < n; r++)
          sp[(size_t)(r0 + r) * o->maxco[i] + r] = 1.0;
      }
    }
  }
  /* basis radii (qs_interactions.F:472-492): per primitive the largest
   * exp_radius over the set's shells l = 0..lmax, coefficient 1, threshold
   * eps_pgf_orb, absolute accuracy 1e-12 (exp_radius without epsabs) */
  o->rpgf = calloc((size_t)totsets * maxpgf_all, sizeof(double));
  o->set_radius = calloc((size_t)totsets, sizeof(double));
  o->kind_radius = calloc((size_t)na, sizeof(double));
  {
    const double epo = p->eps_pgf_orb > 0.0 ? p->eps_pgf_orb : 1.0e-5;
    for (int i = 0; i < na; i++) {
      double kr = 0.0;
      for (int k = 0; k < o->nset[i]; k++) {
        const int gs = o->set_off[i] + k;
        double sr = 0.0;
        for (int q = 0; q < o->npgf[gs]; q++) {
          const double z = o->zet[(size_t)gs * maxpgf_all + q];
          double r = 0.0;
          for (int l = o->lmin[gs]; l <= o->lmax[gs]; l++)
            r = fmax(r, exp_radius(l, z, epo, 1.0, 1.0e-12, r));
          o->rpgf[(size_t)gs * maxpgf_all + q] = r;
          sr = fmax(sr, r);
        }
        o->set_radius[gs] = sr;
        kr = fmax(kr, sr);
      }
      o->kind_radius[i] = kr;
    }
  }
  /* grid levels */
  for (int l = 0; l < p->nlevels; l++) {
    for (int a = 0; a < 3; a++)
      for (int b = 0; b < 3; b++)
        o->dh[l][a][b] = p->cell[a][b] / p->npts[l][a];
    inv3(o->dh[l], o->dh_inv[l]);
  }
  build_tasks(o, p);
  free(elem);
  return o;
}

/* Rebuild the task arrays of o for new atom positions ([natoms][3], bohr),
 * keeping its basis sets: the task list of a moved geometry. */
int wl_retask(wl_out *o, const wl_params *p, const double *positions) {
  if (!o || !p || !positions || p->natoms != o->natoms)
    return 1;
  memcpy(o->atom_positions, positions, sizeof(double) * 3 * (size_t)o->natoms);
  build_tasks(o, p);
  return 0;
}

void wl_free(wl_out *o) {
  if (!o)
    return;
  void *ptrs[] = {o->atom_positions, o->atom_kinds, o->nset, o->nsgf, o->maxco,
                  o->maxpgf, o->set_off, o->lmin, o->lmax, o->npgf, o->nsgf_set,
                  o->first_sgf, o->sphi_off, o->sphi, o->zet, o->block_offsets,
                  o->level, o->iatom, o->jatom, o->iset, o->jset, o->ipgf, o->jpgf,
                  o->border_mask, o->block_num, o->radius, o->rab, o->rpgf, o->set_radius,
                  o->kind_radius};
  for (size_t i = 0; i < sizeof(ptrs) / sizeof(ptrs[0]); i++)
    free(ptrs[i]);
  free(o);
}
