/*
 * TEST INFRASTRUCTURE -- the CPU oracle (see grid_oracle.h).
 *
 * FP64 restatement of CP2K's REF grid backend.  Every routine names the
 * reference file:line whose algorithm it follows.  The point sets visited on
 * the grid (discretised radius, sphere bounds, quadratic row bounds, periodic
 * maps) are reproduced operation for operation, because a single missing or
 * extra grid point would break 1e-12 parity; arithmetic that only affects
 * rounding is written in this file's own way.  Built with -ffp-contract=off so
 * that bound computations round exactly as the reference's ISO-C build does.
 */
#include "grid_oracle.h"

#include <limits.h>
#include <math.h>
#include <omp.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------ */
/* Cartesian-orbital indexing (src/grid/common/grid_common.h:56-102).        */
/* ------------------------------------------------------------------------ */
static inline int ncoset(int l) { return l < 0 ? 0 : (l + 1) * (l + 2) * (l + 3) / 6; }

static inline int coset(int lx, int ly, int lz) {
  const int l = lx + ly + lz;
  if (l == 0)
    return 0;
  return ncoset(l - 1) + ((l - lx) * (l - lx + 1)) / 2 + lz;
}

static inline int imod(int a, int m) { return ((a % m) + m) % m; }
static inline int imax(int a, int b) { return a > b ? a : b; }
static inline int imin(int a, int b) { return a < b ? a : b; }

static double factorial(int n) {
  double f = 1.0;
  for (int i = 2; i <= n; i++)
    f *= (double)i;
  return f;
}

typedef struct {
  int l[3];
} orb;

static inline orb o_up(int d, orb a) {
  a.l[d] += 1;
  return a;
}
static inline orb o_dn(int d, orb a) {
  a.l[d] = a.l[d] > 0 ? a.l[d] - 1 : 0;
  return a;
}
static inline int o_idx(orb a) { return coset(a.l[0], a.l[1], a.l[2]); }

/* ------------------------------------------------------------------------ */
/* Basis sets (src/grid/common/grid_basis_set.c:19-73).                      */
/* ------------------------------------------------------------------------ */
static void *xmalloc(size_t n) {
  void *p = malloc(n ? n : 1);
  if (!p) {
    fprintf(stderr, "oracle: out of memory\n");
    abort();
  }
  return p;
}

void oracle_create_basis_set(int nset, int nsgf, int maxco, int maxpgf,
                             const int *lmin, const int *lmax, const int *npgf,
                             const int *nsgf_set, const int *first_sgf,
                             const double *sphi, const double *zet,
                             oracle_basis **out) {
  oracle_basis *b = xmalloc(sizeof(*b));
  b->nset = nset;
  b->nsgf = nsgf;
  b->maxco = maxco;
  b->maxpgf = maxpgf;
  int **dst[5] = {&b->lmin, &b->lmax, &b->npgf, &b->nsgf_set, &b->first_sgf};
  const int *src[5] = {lmin, lmax, npgf, nsgf_set, first_sgf};
  for (int i = 0; i < 5; i++) {
    *dst[i] = xmalloc(sizeof(int) * nset);
    memcpy(*dst[i], src[i], sizeof(int) * nset);
  }
  b->sphi = xmalloc(sizeof(double) * nsgf * maxco);
  memcpy(b->sphi, sphi, sizeof(double) * nsgf * maxco);
  b->zet = xmalloc(sizeof(double) * nset * maxpgf);
  memcpy(b->zet, zet, sizeof(double) * nset * maxpgf);
  *out = b;
}

void oracle_free_basis_set(oracle_basis *b) {
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

/* ------------------------------------------------------------------------ */
/* P_ab -> C_ab for every grid_func (src/grid/common/grid_prepare_pab.h).    */
/* ------------------------------------------------------------------------ */
typedef struct {
  double *c; /* [ncoset(lb)][ncoset(la)] */
  int n1;    /* leading dimension = ncoset(la_max_cab) */
} cabw;

static inline void cadd(cabw *w, orb a, orb b, double v) {
  w->c[o_idx(b) * w->n1 + o_idx(a)] += v;
}

/* Values of enum grid_func (src/grid/common/grid_constants.h:10-46). */
enum {
  F_AB = 100, F_DADB = 200,
  F_ADBmDAB_X = 301, F_ADBmDAB_Z = 303,
  F_ARDBmDARB_XX = 411, F_ARDBmDARB_ZZ = 433,
  F_DABpADB_X = 501, F_DABpADB_Z = 503,
  F_DX = 601, F_DZ = 603,
  F_DXDY = 701, F_DZDX = 703,
  F_DXDX = 801, F_DZDZ = 803,
  F_DAB_X = 901, F_DAB_Z = 903, F_ADB_X = 904, F_ADB_Z = 906,
  F_CORE_X = 1001, F_CORE_Z = 1003
};

static int func_known(int f) {
  return f == F_AB || f == F_DADB || (f >= F_ADBmDAB_X && f <= F_ADBmDAB_Z) ||
         (f >= 411 && f <= 413) || (f >= 421 && f <= 423) ||
         (f >= 431 && f <= 433) || (f >= F_DABpADB_X && f <= F_DABpADB_Z) ||
         (f >= F_DX && f <= F_DZ) || (f >= F_DXDY && f <= F_DZDX) ||
         (f >= F_DXDX && f <= F_DZDZ) || (f >= F_DAB_X && f <= F_ADB_Z) ||
         (f >= F_CORE_X && f <= F_CORE_Z);
}

/* Angular-momentum range changes of each func
 * (src/grid/common/grid_prepare_pab.h:447-517). */
static void func_ldiffs(int f, int *la_min_d, int *la_max_d, int *lb_min_d,
                        int *lb_max_d) {
  if (!func_known(f)) {
    fprintf(stderr, "oracle: unknown grid_func %d\n", f);
    abort();
  }
  int amax = 0, amin = 0, bmax = 0, bmin = 0;
  if (f == F_AB) {
  } else if (f >= 411 && f <= 433) {
    amax = 1; amin = -1; bmax = 2; bmin = -1;
  } else if ((f >= F_DXDY && f <= F_DZDX) || (f >= F_DXDX && f <= F_DZDZ)) {
    amax = 2; amin = -2; bmax = 2; bmin = -2;
  } else {
    amax = 1; amin = -1; bmax = 1; bmin = -1;
  }
  *la_min_d = amin; *la_max_d = amax; *lb_min_d = bmin; *lb_max_d = bmax;
}

/* d_{i1} d_{i2} acting on b (grid_prepare_pab.h:151-173, oneterm_dijdij). */
static void term_dij_b(int pair, double fa, orb a, orb b, double zetb, cabw *w) {
  static const int P1[3] = {0, 1, 2}, P2[3] = {1, 2, 0};
  const int i1 = P1[pair], i2 = P2[pair];
  cadd(w, a, o_dn(i1, o_dn(i2, b)), b.l[i1] * b.l[i2] * fa);
  cadd(w, a, o_up(i1, o_dn(i2, b)), -2.0 * zetb * b.l[i2] * fa);
  cadd(w, a, o_dn(i1, o_up(i2, b)), -2.0 * zetb * b.l[i1] * fa);
  cadd(w, a, o_up(i1, o_up(i2, b)), 4.0 * zetb * zetb * fa);
}

/* d_i d_i acting on b (grid_prepare_pab.h:196-204, oneterm_diidii). */
static void term_dii_b(int d, double fa, orb a, orb b, double zetb, cabw *w) {
  cadd(w, a, o_dn(d, o_dn(d, b)), b.l[d] * (b.l[d] - 1) * fa);
  cadd(w, a, b, -2.0 * zetb * (2 * b.l[d] + 1) * fa);
  cadd(w, a, o_up(d, o_up(d, b)), 4.0 * zetb * zetb * fa);
}

/* One (a, b) element of P mapped into C (grid_prepare_pab.h:26-430). */
static void prep_one(int f, orb a, orb b, double za, double zb, double p,
                     cabw *w) {
  if (f == F_AB) {
    cadd(w, a, b, p);
  } else if (f == F_DADB) {
    for (int i = 0; i < 3; i++) {
      cadd(w, o_dn(i, a), o_dn(i, b), 0.5 * a.l[i] * b.l[i] * p);
      cadd(w, o_dn(i, a), o_up(i, b), -1.0 * a.l[i] * zb * p);
      cadd(w, o_up(i, a), o_dn(i, b), -1.0 * za * b.l[i] * p);
      cadd(w, o_up(i, a), o_up(i, b), 2.0 * za * zb * p);
    }
  } else if (f >= F_ADBmDAB_X && f <= F_ADBmDAB_Z) {
    const int d = f - F_ADBmDAB_X;
    cadd(w, a, o_dn(d, b), b.l[d] * p);
    cadd(w, a, o_up(d, b), -2.0 * zb * p);
    cadd(w, o_dn(d, a), b, -a.l[d] * p);
    cadd(w, o_up(d, a), b, 2.0 * za * p);
  } else if (f >= 411 && f <= 433) {
    const int d = f / 10 - 41, r = f % 10 - 1;
    const orb br = o_up(r, b);
    cadd(w, a, o_dn(d, br), b.l[d] * p);
    cadd(w, a, o_up(d, br), -2.0 * zb * p);
    cadd(w, o_dn(d, a), br, -a.l[d] * p);
    cadd(w, o_up(d, a), br, 2.0 * za * p);
  } else if (f >= F_DABpADB_X && f <= F_DABpADB_Z) {
    const int d = f - F_DABpADB_X;
    cadd(w, a, o_dn(d, b), b.l[d] * p);
    cadd(w, a, o_up(d, b), -2.0 * zb * p);
    cadd(w, o_dn(d, a), b, a.l[d] * p);
    cadd(w, o_up(d, a), b, -2.0 * za * p);
  } else if (f >= F_DAB_X && f <= F_DAB_Z) {
    const int d = f - F_DAB_X;
    cadd(w, o_dn(d, a), b, -a.l[d] * p);
    cadd(w, o_up(d, a), b, 2.0 * za * p);
  } else if (f >= F_ADB_X && f <= F_ADB_Z) {
    const int d = f - F_ADB_X;
    cadd(w, a, o_dn(d, b), -b.l[d] * p);
    cadd(w, a, o_up(d, b), 2.0 * zb * p);
  } else if (f >= F_CORE_X && f <= F_CORE_Z) {
    const int d = f - F_CORE_X;
    cadd(w, o_up(d, a), b, 2.0 * za * p);
  } else if (f >= F_DX && f <= F_DZ) {
    const int d = f - F_DX;
    cadd(w, o_dn(d, a), o_dn(d, b), a.l[d] * b.l[d] * p);
    cadd(w, o_dn(d, a), o_up(d, b), -2.0 * a.l[d] * zb * p);
    cadd(w, o_up(d, a), o_dn(d, b), -2.0 * za * b.l[d] * p);
    cadd(w, o_up(d, a), o_up(d, b), 4.0 * za * zb * p);
  } else if (f >= F_DXDY && f <= F_DZDX) {
    static const int D1[3] = {0, 1, 2}, D2[3] = {1, 2, 0};
    const int pair = f - F_DXDY, d1 = D1[pair], d2 = D2[pair];
    term_dij_b(pair, a.l[d1] * a.l[d2] * p, o_dn(d1, o_dn(d2, a)), b, zb, w);
    term_dij_b(pair, -2.0 * za * a.l[d2] * p, o_up(d1, o_dn(d2, a)), b, zb, w);
    term_dij_b(pair, -2.0 * za * a.l[d1] * p, o_dn(d1, o_up(d2, a)), b, zb, w);
    term_dij_b(pair, 4.0 * za * za * p, o_up(d1, o_up(d2, a)), b, zb, w);
  } else if (f >= F_DXDX && f <= F_DZDZ) {
    const int d = f - F_DXDX;
    term_dii_b(d, a.l[d] * (a.l[d] - 1) * p, o_dn(d, o_dn(d, a)), b, zb, w);
    term_dii_b(d, -2.0 * za * (2 * a.l[d] + 1) * p, a, b, zb, w);
    term_dii_b(d, 4.0 * za * za * p, o_up(d, o_up(d, a)), b, zb, w);
  }
}

/* Whole P sub-block -> C (src/grid/ref/grid_ref_prepare_pab.c:54-82). */
static void prepare_cab(int f, int o1, int o2, int la_max, int la_min,
                        int lb_max, int lb_min, double za, double zb, int n1,
                        const double *pab, int n1_cab, double *cab) {
  cabw w = {cab, n1_cab};
  for (int la = la_min; la <= la_max; la++)
    for (int ax = 0; ax <= la; ax++)
      for (int ay = 0; ay <= la - ax; ay++) {
        const orb a = {{ax, ay, la - ax - ay}};
        for (int lb = lb_min; lb <= lb_max; lb++)
          for (int bx = 0; bx <= lb; bx++)
            for (int by = 0; by <= lb - bx; by++) {
              const orb b = {{bx, by, lb - bx - by}};
              const double p = pab[(size_t)(o2 + o_idx(b)) * n1 + o1 + o_idx(a)];
              prep_one(f, a, b, za, zb, p, &w);
            }
      }
}

/* ------------------------------------------------------------------------ */
/* C_ab <-> C_xyz about the product centre rp                               */
/* (src/grid/ref/grid_ref_collint.h:827-911).  cxyz is dense [lp+1]^3,       */
/* index [lzp][lyp][lxp].  forward=1: collocate (cab -> cxyz);               */
/* forward=0: integrate adjoint (cxyz -> cab, accumulated).                  */
/* ------------------------------------------------------------------------ */
static void cab_cxyz(int forward, int la_max, int la_min, int lb_max,
                     int lb_min, double prefactor, const double ra[3],
                     const double rb[3], const double rp[3], double *cab,
                     double *cxyz) {
  const int lp = la_max + lb_max, lp1 = lp + 1;
  const int na = la_max + 1, nb = lb_max + 1;
  /* alpha[d][lxb][lxa][l]: coefficient of (x-p)^l in (x-a)^lxa (x-b)^lxb */
  double *alpha = calloc((size_t)3 * nb * na * lp1, sizeof(double));
#define ALPHA(d, b, a, l) alpha[(((size_t)(d) * nb + (b)) * na + (a)) * lp1 + (l)]
  for (int d = 0; d < 3; d++) {
    const double pa = rp[d] - ra[d], pb = rp[d] - rb[d];
    for (int xa = 0; xa <= la_max; xa++)
      for (int xb = 0; xb <= lb_max; xb++) {
        double ca = 1.0, powa = 1.0;
        for (int k = 0; k <= xa; k++) {
          double cb = 1.0, powb = 1.0;
          for (int m = 0; m <= xb; m++) {
            ALPHA(d, xb, xa, xa - k + xb - m) += ca * cb * powa * powb;
            cb = cb * (double)(xb - m) / (double)(m + 1);
            powb *= pb;
          }
          ca = ca * (double)(xa - k) / (double)(k + 1);
          powa *= pa;
        }
      }
  }
  const int n1 = ncoset(la_max);
  for (int za = 0; za <= la_max; za++)
    for (int zb = 0; zb <= lb_max; zb++)
      for (int ya = 0; ya <= la_max - za; ya++)
        for (int yb = 0; yb <= lb_max - zb; yb++)
          for (int xa = imax(la_min - za - ya, 0); xa <= la_max - za - ya; xa++)
            for (int xb = imax(lb_min - zb - yb, 0); xb <= lb_max - zb - yb; xb++) {
              double *c = &cab[(size_t)coset(xb, yb, zb) * n1 + coset(xa, ya, za)];
              double acc = 0.0;
              for (int pz = 0; pz <= za + zb; pz++)
                for (int py = 0; py <= ya + yb; py++)
                  for (int px = 0; px <= xa + xb; px++) {
                    const double w = ALPHA(0, xb, xa, px) * ALPHA(1, yb, ya, py) *
                                     ALPHA(2, zb, za, pz) * prefactor;
                    double *cx = &cxyz[((size_t)pz * lp1 + py) * lp1 + px];
                    if (forward)
                      *cx += (*c) * w;
                    else
                      acc += (*cx) * w;
                  }
              if (!forward)
                *c += acc;
            }
#undef ALPHA
  free(alpha);
}

/* ------------------------------------------------------------------------ */
/* Orthorhombic cube <-> grid (src/grid/ref/grid_ref_collint.h:30-327).     */
/* ------------------------------------------------------------------------ */
static inline int ceil_bound(double remain, double hinv) {
  /* grid_ref_collint.h:49,147 -- identical expression, no contraction */
  return (int)ceil(-1e-8 - sqrt(fmax(0.0, remain)) * hinv);
}

static long long ortho_cube(int collocate, int lp, double zetp,
                            const double dh[9], const double dh_inv[9],
                            const double rp[3], const int npts_global[3],
                            const int npts_local[3], const int shift_local[3],
                            double radius, double *cxyz, double *grid,
                            int count_only) {
  const int lp1 = lp + 1;
  int center[3];
  for (int i = 0; i < 3; i++) {
    double s = 0.0;
    for (int j = 0; j < 3; j++)
      s += dh_inv[j * 3 + i] * rp[j];
    center[i] = (int)floor(s);
  }
  double roff[3];
  for (int i = 0; i < 3; i++)
    roff[i] = rp[i] - ((double)center[i]) * dh[i * 4];
  const double drmin = fmin(dh[0], fmin(dh[4], dh[8]));
  const double disr = drmin * fmax(1.0, ceil(radius / drmin));
  int lb[3];
  for (int i = 0; i < 3; i++) {
    lb[i] = (int)ceil(-1e-8 - disr * dh_inv[i * 4]);
    if (npts_global[i] != npts_local[i]) {
      const int off = imod(center[i] + lb[i] - shift_local[i], npts_global[i]) - lb[i];
      if (!(off + 1 - lb[i] < npts_local[i] && off + lb[i] >= 0)) {
        fprintf(stderr, "oracle: cube does not fit into the local grid\n");
        abort();
      }
    }
  }
  const int cmax = imax(imax(1 - lb[0], 1 - lb[1]), 1 - lb[2]);
  const int w = 2 * cmax + 1;
  const size_t stride = (size_t)npts_local[1] * npts_local[0];
  long long npoints = 0;
  double *pol = NULL, *cxy = NULL, *cx = NULL;
  int *map = NULL;
  if (!count_only) {
    pol = malloc(sizeof(double) * 3 * lp1 * w); /* [d][l][c+cmax] */
    map = malloc(sizeof(int) * 3 * w);
    for (int d = 0; d < 3; d++) {
      const double h = dh[d * 4];
      for (int c = lb[d]; c <= 1 - lb[d]; c++) {
        const double x = c * h - roff[d];
        double v = exp(-zetp * x * x);
        for (int l = 0; l <= lp; l++) {
          pol[((size_t)d * lp1 + l) * w + c + cmax] = v;
          v *= x;
        }
      }
      for (int c = -cmax; c <= cmax; c++)
        map[d * w + c + cmax] = imod(center[d] + c - shift_local[d], npts_global[d]);
    }
    cxy = malloc(sizeof(double) * lp1 * lp1 * 2); /* [ly][lx][k1/k2] */
    cx = malloc(sizeof(double) * lp1 * 4);        /* [lx][(k,j) pair]  */
  }
#define POL(d, l, c) pol[((size_t)(d) * lp1 + (l)) * w + (c) + cmax]
  for (int k1 = lb[2]; k1 <= 0; k1++) {
    const int k2 = 1 - k1;
    const int kd = (2 * k1 - 1) / 2;
    const double kr = kd * dh[8];
    const double kremain = disr * disr - kr * kr;
    const int jstart = ceil_bound(kremain, dh_inv[4]);
    if (!count_only) {
      memset(cxy, 0, sizeof(double) * lp1 * lp1 * 2);
      if (collocate)
        for (int lz = 0; lz <= lp; lz++)
          for (int ly = 0; ly <= lp - lz; ly++)
            for (int lx = 0; lx <= lp - lz - ly; lx++) {
              const double c = cxyz[((size_t)lz * lp1 + ly) * lp1 + lx];
              cxy[(ly * lp1 + lx) * 2 + 0] += c * POL(2, lz, k1);
              cxy[(ly * lp1 + lx) * 2 + 1] += c * POL(2, lz, k2);
            }
    }
    for (int j1 = jstart; j1 <= 0; j1++) {
      const int j2 = 1 - j1;
      const int jd = (2 * j1 - 1) / 2;
      const double jr = jd * dh[4];
      const double jremain = kremain - jr * jr;
      const int istart = ceil_bound(jremain, dh_inv[0]);
      const int iend = 1 - istart;
      npoints += 4LL * (iend - istart + 1);
      if (count_only)
        continue;
      const size_t kg1 = map[2 * w + k1 + cmax], kg2 = map[2 * w + k2 + cmax];
      const size_t jg1 = map[1 * w + j1 + cmax], jg2 = map[1 * w + j2 + cmax];
      const size_t base[4] = {kg1 * stride + jg1 * npts_local[0],
                              kg2 * stride + jg1 * npts_local[0],
                              kg1 * stride + jg2 * npts_local[0],
                              kg2 * stride + jg2 * npts_local[0]};
      memset(cx, 0, sizeof(double) * lp1 * 4);
      if (collocate) {
        for (int ly = 0; ly <= lp; ly++)
          for (int lx = 0; lx <= lp - ly; lx++) {
            const double p1 = POL(1, ly, j1), p2 = POL(1, ly, j2);
            const double *c = &cxy[(ly * lp1 + lx) * 2];
            cx[lx * 4 + 0] += c[0] * p1;
            cx[lx * 4 + 1] += c[1] * p1;
            cx[lx * 4 + 2] += c[0] * p2;
            cx[lx * 4 + 3] += c[1] * p2;
          }
        for (int i = istart; i <= iend; i++) {
          const size_t ig = map[i + cmax];
          double s[4] = {0.0, 0.0, 0.0, 0.0};
          for (int lx = 0; lx <= lp; lx++) {
            const double p = POL(0, lx, i);
            for (int q = 0; q < 4; q++)
              s[q] += cx[lx * 4 + q] * p;
          }
          for (int q = 0; q < 4; q++)
            grid[base[q] + ig] += s[q];
        }
      } else {
        for (int i = istart; i <= iend; i++) {
          const size_t ig = map[i + cmax];
          double g[4];
          for (int q = 0; q < 4; q++)
            g[q] = grid[base[q] + ig];
          for (int lx = 0; lx <= lp; lx++) {
            const double p = POL(0, lx, i);
            for (int q = 0; q < 4; q++)
              cx[lx * 4 + q] += g[q] * p;
          }
        }
        for (int ly = 0; ly <= lp; ly++)
          for (int lx = 0; lx <= lp - ly; lx++) {
            const double p1 = POL(1, ly, j1), p2 = POL(1, ly, j2);
            double *c = &cxy[(ly * lp1 + lx) * 2];
            c[0] += cx[lx * 4 + 0] * p1 + cx[lx * 4 + 2] * p2;
            c[1] += cx[lx * 4 + 1] * p1 + cx[lx * 4 + 3] * p2;
          }
      }
    }
    if (!count_only && !collocate)
      for (int lz = 0; lz <= lp; lz++)
        for (int ly = 0; ly <= lp - lz; ly++)
          for (int lx = 0; lx <= lp - lz - ly; lx++)
            cxyz[((size_t)lz * lp1 + ly) * lp1 + lx] +=
                cxy[(ly * lp1 + lx) * 2 + 0] * POL(2, lz, k1) +
                cxy[(ly * lp1 + lx) * 2 + 1] * POL(2, lz, k2);
  }
#undef POL
  free(pol);
  free(map);
  free(cxy);
  free(cx);
  return npoints;
}

/* ------------------------------------------------------------------------ */
/* General (non-orthorhombic or border-masked) cube <-> grid                 */
/* (src/grid/ref/grid_ref_collint.h:333-794).                                */
/* ------------------------------------------------------------------------ */

/* cxyz[lz][ly][lx] <-> cijk[kl][jl][il] through the multinomial expansion of
 * x = sum_d u_d dh[d][0] etc. (grid_ref_collint.h:698-762).  forward=1 maps
 * cxyz -> cijk (collocate), forward=0 the adjoint (integrate). */
static void cxyz_cijk(int forward, int lp, const double dh[9], double *cxyz,
                      double *cijk) {
  const int lp1 = lp + 1;
  /* hp[n][d][c] = dh[d][c]^n */
  double *hp = malloc(sizeof(double) * lp1 * 9);
  for (int c = 0; c < 9; c++) {
    hp[c] = 1.0;
    for (int n = 1; n <= lp; n++)
      hp[n * 9 + c] = hp[(n - 1) * 9 + c] * dh[c];
  }
  for (int lx = 0; lx <= lp; lx++)
    for (int ly = 0; ly <= lp - lx; ly++)
      for (int lz = 0; lz <= lp - lx - ly; lz++) {
        double *cc = &cxyz[((size_t)lz * lp1 + ly) * lp1 + lx];
        const double fl = factorial(lx) * factorial(ly) * factorial(lz);
        double acc = 0.0;
        /* split each Cartesian power over the three lattice directions */
        for (int ix = 0; ix <= lx; ix++)
          for (int jx = 0; jx <= lx - ix; jx++) {
            const int kx = lx - ix - jx;
            const double wx = hp[ix * 9 + 0] * hp[jx * 9 + 3] * hp[kx * 9 + 6] /
                              (factorial(ix) * factorial(jx) * factorial(kx));
            for (int iy = 0; iy <= ly; iy++)
              for (int jy = 0; jy <= ly - iy; jy++) {
                const int ky = ly - iy - jy;
                const double wy = hp[iy * 9 + 1] * hp[jy * 9 + 4] * hp[ky * 9 + 7] /
                                  (factorial(iy) * factorial(jy) * factorial(ky));
                for (int iz = 0; iz <= lz; iz++)
                  for (int jz = 0; jz <= lz - iz; jz++) {
                    const int kz = lz - iz - jz;
                    const double wz = hp[iz * 9 + 2] * hp[jz * 9 + 5] *
                                      hp[kz * 9 + 8] /
                                      (factorial(iz) * factorial(jz) * factorial(kz));
                    const int il = ix + iy + iz, jl = jx + jy + jz, kl = kx + ky + kz;
                    double *ck = &cijk[((size_t)kl * lp1 + jl) * lp1 + il];
                    const double wgt = wx * wy * wz * fl;
                    if (forward)
                      *ck += (*cc) * wgt;
                    else
                      acc += (*ck) * wgt;
                  }
              }
          }
        if (!forward)
          *cc += acc;
      }
  free(hp);
}

static long long general_cube(int collocate, int border_mask, int lp,
                              double zetp, const double dh[9],
                              const double dh_inv[9], const double rp[3],
                              const int npts_global[3], const int npts_local[3],
                              const int shift_local[3],
                              const int border_width[3], double radius,
                              double *cijk, double *grid, int count_only) {
  const int lp1 = lp + 1;
  int bnd[3][2];
  for (int d = 0; d < 3; d++) {
    bnd[d][0] = 0;
    bnd[d][1] = npts_local[d] - 1;
    if (border_mask & (1 << (2 * d)))
      bnd[d][0] += border_width[d];
    if (border_mask & (1 << (2 * d + 1)))
      bnd[d][1] -= border_width[d];
  }
  double gp[3] = {0.0, 0.0, 0.0};
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      gp[i] += dh_inv[j * 3 + i] * rp[j];
  int imn[3] = {INT_MAX, INT_MAX, INT_MAX}, imx[3] = {INT_MIN, INT_MIN, INT_MIN};
  for (int a = -1; a <= 1; a++)
    for (int b = -1; b <= 1; b++)
      for (int c = -1; c <= 1; c++) {
        const double x = rp[0] + a * radius, y = rp[1] + b * radius,
                     z = rp[2] + c * radius;
        for (int d = 0; d < 3; d++) {
          const double r = dh_inv[0 * 3 + d] * x + dh_inv[1 * 3 + d] * y +
                           dh_inv[2 * 3 + d] * z;
          imn[d] = imin(imn[d], (int)floor(r));
          imx[d] = imax(imx[d], (int)ceil(r));
        }
      }
  const int n[3] = {imx[0] - imn[0] + 1, imx[1] - imn[1] + 1, imx[2] - imn[2] + 1};
  int *map[3];
  for (int d = 0; d < 3; d++) {
    map[d] = malloc(sizeof(int) * n[d]);
    for (int c = imn[d]; c <= imx[d]; c++) {
      const int g = imod(c - shift_local[d], npts_global[d]);
      map[d][c - imn[d]] = (bnd[d][0] <= g && g <= bnd[d][1]) ? g : INT_MIN;
    }
  }
  /* Pair tables (grid_ref_collint.h:535-576): e_ab[a][b] =
   * exp(-zetp (da^2 h_aa + 2 da db h_ab)) for the lattice direction pairs
   * (0,1), (1,2), (2,0); their product is exp(-zetp r^2). */
  double *e[3] = {NULL, NULL, NULL};
  static const int PA[3] = {0, 1, 2}, PB[3] = {1, 2, 0};
  if (!count_only)
    for (int t = 0; t < 3; t++) {
      const int A = PA[t], B = PB[t];
      double haa = 0.0, hab = 0.0;
      for (int c = 0; c < 3; c++) {
        haa += dh[A * 3 + c] * dh[A * 3 + c];
        hab += dh[A * 3 + c] * dh[B * 3 + c];
      }
      e[t] = malloc(sizeof(double) * n[A] * n[B]);
      for (int a = 0; a < n[A]; a++) {
        const double da = (a + imn[A]) - gp[A];
        for (int b = 0; b < n[B]; b++) {
          const double db = (b + imn[B]) - gp[B];
          e[t][(size_t)a * n[B] + b] = exp(-zetp * (da * da * haa + 2.0 * da * db * hab));
        }
      }
    }
  const size_t stride = (size_t)npts_local[1] * npts_local[0];
  double *cij = count_only ? NULL : malloc(sizeof(double) * lp1 * lp1);
  double *ci = count_only ? NULL : malloc(sizeof(double) * lp1);
  long long npoints = 0;
  for (int k = imn[2]; k <= imx[2]; k++) {
    const int kg = map[2][k - imn[2]];
    if (kg < bnd[2][0] || bnd[2][1] < kg)
      continue;
    const double dk = k - gp[2];
    if (!count_only) {
      memset(cij, 0, sizeof(double) * lp1 * lp1);
      if (collocate) {
        double pk = 1.0;
        for (int kl = 0; kl <= lp; kl++) {
          for (int jl = 0; jl <= lp - kl; jl++)
            for (int il = 0; il <= lp - kl - jl; il++)
              cij[jl * lp1 + il] += cijk[((size_t)kl * lp1 + jl) * lp1 + il] * pk;
          pk *= dk;
        }
      }
    }
    for (int j = imn[1]; j <= imx[1]; j++) {
      const int jg = map[1][j - imn[1]];
      if (jg < 0)
        continue;
      const double dj = j - gp[1];
      /* quadratic row bounds, grid_ref_collint.h:424-463 (same operations) */
      double qa = 0.0, qb = 0.0, qc = 0.0;
      for (int c = 0; c < 3; c++) {
        const double v = (0 - gp[0]) * dh[0 * 3 + c] + (j - gp[1]) * dh[1 * 3 + c] +
                         (k - gp[2]) * dh[2 * 3 + c];
        qa += dh[0 * 3 + c] * dh[0 * 3 + c];
        qb += 2.0 * v * dh[0 * 3 + c];
        qc += v * v;
      }
      const double disc = qb * qb - 4.0 * qa * (qc - radius * radius);
      if (!(0.0 < disc))
        continue;
      const double sq = sqrt(disc), inv2a = 1.0 / (2.0 * qa);
      const int ismin = (int)ceil((-qb - sq) * inv2a);
      const int ismax = (int)floor((-qb + sq) * inv2a);
      if (count_only) {
        for (int i = ismin; i <= ismax; i++)
          npoints += (map[0][i - imn[0]] >= 0);
        continue;
      }
      memset(ci, 0, sizeof(double) * lp1);
      if (collocate) {
        double pj = 1.0;
        for (int jl = 0; jl <= lp; jl++) {
          for (int il = 0; il <= lp - jl; il++)
            ci[il] += cij[jl * lp1 + il] * pj;
          pj *= dj;
        }
      }
      const size_t base = (size_t)kg * stride + (size_t)jg * npts_local[0];
      const double ejk = e[1][(size_t)(j - imn[1]) * n[2] + (k - imn[2])];
      for (int i = ismin; i <= ismax; i++) {
        const int ig = map[0][i - imn[0]];
        if (ig < 0)
          continue;
        npoints++;
        const double di = i - gp[0];
        const double gauss = e[0][(size_t)(i - imn[0]) * n[1] + (j - imn[1])] * ejk *
                             e[2][(size_t)(k - imn[2]) * n[0] + (i - imn[0])];
        double pw = gauss;
        if (collocate) {
          double s = 0.0;
          for (int il = 0; il <= lp; il++) {
            s += ci[il] * pw;
            pw *= di;
          }
          grid[base + ig] += s;
        } else {
          const double g = grid[base + ig];
          for (int il = 0; il <= lp; il++) {
            ci[il] += g * pw;
            pw *= di;
          }
        }
      }
      if (!collocate) {
        double pj = 1.0;
        for (int jl = 0; jl <= lp; jl++) {
          for (int il = 0; il <= lp - jl; il++)
            cij[jl * lp1 + il] += ci[il] * pj;
          pj *= dj;
        }
      }
    }
    if (!count_only && !collocate) {
      double pk = 1.0;
      for (int kl = 0; kl <= lp; kl++) {
        for (int jl = 0; jl <= lp - kl; jl++)
          for (int il = 0; il <= lp - kl - jl; il++)
            cijk[((size_t)kl * lp1 + jl) * lp1 + il] += cij[jl * lp1 + il] * pk;
        pk *= dk;
      }
    }
  }
  for (int d = 0; d < 3; d++)
    free(map[d]);
  for (int t = 0; t < 3; t++)
    free(e[t]);
  free(cij);
  free(ci);
  return npoints;
}

/* ------------------------------------------------------------------------ */
/* cab <-> grid for one primitive pair (grid_ref_collint.h:917-965).         */
/* Returns the number of grid points visited.                                */
/* ------------------------------------------------------------------------ */
static long long cab_grid(int collocate, bool ortho, int border_mask,
                          int la_max, int la_min, int lb_max, int lb_min,
                          double zeta, double zetb, double rscale,
                          const double dh[9], const double dh_inv[9],
                          const double ra[3], const double rab[3],
                          const int npts_global[3], const int npts_local[3],
                          const int shift_local[3], const int border_width[3],
                          double radius, double *cab, double *grid,
                          int count_only) {
  double dh_max = 0.0;
  for (int i = 0; i < 9; i++)
    dh_max = fmax(dh_max, fabs(dh[i]));
  if (2.0 * radius < dh_max)
    return 0; /* too small to be mapped onto this grid */
  const double zetp = zeta + zetb, f = zetb / zetp;
  const double rab2 = rab[0] * rab[0] + rab[1] * rab[1] + rab[2] * rab[2];
  const double prefactor = rscale * exp(-zeta * f * rab2);
  double rp[3], rb[3];
  for (int i = 0; i < 3; i++) {
    rp[i] = ra[i] + f * rab[i];
    rb[i] = ra[i] + rab[i];
  }
  const int lp = la_max + lb_max, lp1 = lp + 1;
  const bool use_ortho = ortho && border_mask == 0;
  double *cxyz = NULL, *cijk = NULL;
  if (!count_only) {
    cxyz = calloc((size_t)lp1 * lp1 * lp1, sizeof(double));
    cijk = calloc((size_t)lp1 * lp1 * lp1, sizeof(double));
    if (collocate) {
      cab_cxyz(1, la_max, la_min, lb_max, lb_min, prefactor, ra, rb, rp, cab, cxyz);
      if (!use_ortho)
        cxyz_cijk(1, lp, dh, cxyz, cijk);
    }
  }
  long long np;
  if (use_ortho)
    np = ortho_cube(collocate, lp, zetp, dh, dh_inv, rp, npts_global, npts_local,
                    shift_local, radius, cxyz, grid, count_only);
  else
    np = general_cube(collocate, border_mask, lp, zetp, dh, dh_inv, rp,
                      npts_global, npts_local, shift_local, border_width, radius,
                      cijk, grid, count_only);
  if (!count_only) {
    if (!collocate) {
      if (!use_ortho)
        cxyz_cijk(0, lp, dh, cxyz, cijk);
      cab_cxyz(0, la_max, la_min, lb_max, lb_min, prefactor, ra, rb, rp, cab, cxyz);
    }
    free(cxyz);
    free(cijk);
  }
  return np;
}

/* ------------------------------------------------------------------------ */
/* Single-task entry points (src/grid/ref/grid_ref_collocate.c:19-49,       */
/* grid_ref_integrate.c:44-152) and the integrate post-processing            */
/* (src/grid/common/grid_process_vab.h:29-251).                              */
/* ------------------------------------------------------------------------ */
void oracle_collocate_pgf_product(
    bool orthorhombic, int border_mask, int func, int la_max, int la_min,
    int lb_max, int lb_min, double zeta, double zetb, double rscale,
    const double *dh, const double *dh_inv, const double *ra,
    const double *rab, const int *npts_global, const int *npts_local,
    const int *shift_local, const int *border_width, double radius, int o1,
    int o2, int n1, int n2, const double *pab, double *grid) {
  (void)n2;
  int amin_d, amax_d, bmin_d, bmax_d;
  func_ldiffs(func, &amin_d, &amax_d, &bmin_d, &bmax_d);
  const int la_min_c = imax(la_min + amin_d, 0), lb_min_c = imax(lb_min + bmin_d, 0);
  const int la_max_c = la_max + amax_d, lb_max_c = lb_max + bmax_d;
  const int n1c = ncoset(la_max_c), n2c = ncoset(lb_max_c);
  double *cab = calloc((size_t)n1c * n2c, sizeof(double));
  prepare_cab(func, o1, o2, la_max, la_min, lb_max, lb_min, zeta, zetb, n1, pab,
              n1c, cab);
  cab_grid(1, orthorhombic, border_mask, la_max_c, la_min_c, lb_max_c, lb_min_c,
           zeta, zetb, rscale, dh, dh_inv, ra, rab, npts_global, npts_local,
           shift_local, border_width, radius, cab, grid, 0);
  free(cab);
}

typedef struct {
  const double *c;
  int m1;
  double za, zb;
  const double *rab;
} vabctx;

static inline double cg(const vabctx *x, orb a, orb b) {
  return x->c[o_idx(b) * x->m1 + o_idx(a)];
}

enum { V_HAB, V_FA, V_FB, V_VA, V_VB };

/* The non-tau forms (grid_process_vab.h:29-43, 67-78, 103-107, 135-145). */
static double vab_plain(const vabctx *x, int kind, int i, int j, orb a, orb b) {
  switch (kind) {
  case V_HAB:
    return cg(x, a, b);
  case V_FA:
    return 2.0 * x->za * cg(x, o_up(i, a), b) - a.l[i] * cg(x, o_dn(i, a), b);
  case V_FB:
    return 2.0 * x->zb * (cg(x, o_up(i, a), b) - x->rab[i] * cg(x, a, b)) -
           b.l[i] * cg(x, a, o_dn(i, b));
  case V_VA:
    return 2.0 * x->za * cg(x, o_up(i, o_up(j, a)), b) -
           a.l[j] * cg(x, o_up(i, o_dn(j, a)), b);
  default: /* V_VB */
    return 2.0 * x->zb *
               (cg(x, o_up(i, o_up(j, a)), b) - cg(x, o_up(i, a), b) * x->rab[j] -
                cg(x, o_up(j, a), b) * x->rab[i] + cg(x, a, b) * x->rab[j] * x->rab[i]) -
           b.l[j] * cg(x, a, o_up(i, o_dn(j, b)));
  }
}

/* <nabla a| . |nabla b> combination used when compute_tau is set
 * (grid_process_vab.h:45-62 and the matching blocks for each quantity). */
static double vab(const vabctx *x, bool tau, int kind, int i, int j, orb a, orb b) {
  if (!tau)
    return vab_plain(x, kind, i, j, a, b);
  double s = 0.0;
  for (int k = 0; k < 3; k++) {
    s += 0.5 * a.l[k] * b.l[k] * vab_plain(x, kind, i, j, o_dn(k, a), o_dn(k, b));
    s -= x->za * b.l[k] * vab_plain(x, kind, i, j, o_up(k, a), o_dn(k, b));
    s -= a.l[k] * x->zb * vab_plain(x, kind, i, j, o_dn(k, a), o_up(k, b));
    s += 2.0 * x->za * x->zb * vab_plain(x, kind, i, j, o_up(k, a), o_up(k, b));
  }
  return s;
}

void oracle_integrate_pgf_product(
    bool orthorhombic, bool compute_tau, int border_mask, int la_max,
    int la_min, int lb_max, int lb_min, double zeta, double zetb,
    const double *dh, const double *dh_inv, const double *ra,
    const double *rab, const int *npts_global, const int *npts_local,
    const int *shift_local, const int *border_width, double radius, int o1,
    int o2, int n1, int n2, const double *grid, double *hab,
    const double *pab, double *forces, double *virials, double *hdab,
    double *hadb, double *a_hdab) {
  (void)n2;
  /* grid_ref_integrate.c:56-57: the derivative blocks need the same shifts */
  const bool do_f = forces != NULL || hdab != NULL || hadb != NULL,
             do_v = virials != NULL || a_hdab != NULL;
  /* process_get_ldiffs, grid_process_vab.h:222-251 */
  int amax_d = 0, amin_d = 0, bmax_d = 0, bmin_d = 0;
  if (do_f || do_v) {
    amax_d += 1; amin_d -= 1; bmin_d -= 1;
  }
  if (do_v) {
    amax_d += 1; bmax_d += 1;
  }
  if (compute_tau) {
    amax_d += 1; bmax_d += 1; amin_d -= 1; bmin_d -= 1;
  }
  const int la_max_l = la_max + amax_d, lb_max_l = lb_max + bmax_d;
  const int la_min_l = imax(0, la_min + amin_d), lb_min_l = imax(0, lb_min + bmin_d);
  const int m1 = ncoset(la_max_l), m2 = ncoset(lb_max_l);
  double *cab = calloc((size_t)m1 * m2, sizeof(double));
  cab_grid(0, orthorhombic, border_mask, la_max_l, la_min_l, lb_max_l, lb_min_l,
           zeta, zetb, 1.0, dh, dh_inv, ra, rab, npts_global, npts_local,
           shift_local, border_width, radius, cab, (double *)grid, 0);
  const vabctx x = {cab, m1, zeta, zetb, rab};
  for (int la = la_min; la <= la_max; la++)
    for (int ax = 0; ax <= la; ax++)
      for (int ay = 0; ay <= la - ax; ay++) {
        const orb a = {{ax, ay, la - ax - ay}};
        for (int lb = lb_min; lb <= lb_max; lb++)
          for (int bx = 0; bx <= lb; bx++)
            for (int by = 0; by <= lb - bx; by++) {
              const orb b = {{bx, by, lb - bx - by}};
              const size_t e = (size_t)(o2 + o_idx(b)) * n1 + o1 + o_idx(a);
              hab[e] += vab(&x, compute_tau, V_HAB, 0, 0, a, b);
              /* grid_ref_integrate.c:121-145 (no tau) */
              for (int i = 0; i < 3; i++) {
                if (hdab != NULL)
                  hdab[e * 3 + i] += vab(&x, false, V_FA, i, 0, a, b);
                if (hadb != NULL)
                  hadb[e * 3 + i] += vab(&x, false, V_FB, i, 0, a, b);
                if (a_hdab != NULL)
                  for (int j = 0; j < 3; j++)
                    a_hdab[(e * 3 + i) * 3 + j] += vab(&x, false, V_VA, i, j, a, b);
              }
              if (forces != NULL) {
                const double p = pab[e];
                for (int i = 0; i < 3; i++) {
                  forces[i] += p * vab(&x, compute_tau, V_FA, i, 0, a, b);
                  forces[3 + i] += p * vab(&x, compute_tau, V_FB, i, 0, a, b);
                }
              }
              if (virials != NULL) {
                const double p = pab[e];
                for (int i = 0; i < 3; i++)
                  for (int j = 0; j < 3; j++) {
                    virials[i * 3 + j] += p * vab(&x, compute_tau, V_VA, i, j, a, b);
                    virials[9 + i * 3 + j] += p * vab(&x, compute_tau, V_VB, i, j, a, b);
                  }
              }
            }
      }
  free(cab);
}

/* ------------------------------------------------------------------------ */
/* Task lists (src/grid/ref/grid_ref_task_list.c:26-691).                    */
/* ------------------------------------------------------------------------ */
typedef struct {
  int level, iatom, jatom, iset, jset, ipgf, jpgf, border_mask, block_num;
  double radius, rab[3];
  int orig; /* position in the caller's list, for stable ordering */
} otask;

typedef struct {
  bool ortho;
  int ntasks, nlevels, natoms, nkinds, nblocks, maxco;
  int *block_offsets, *atom_kinds;
  double *atom_positions;
  const oracle_basis **basis;
  otask *tasks;
  int *npts_global, *npts_local, *shift_local, *border_width; /* [nlevels][3] */
  double *dh, *dh_inv;                                         /* [nlevels][9] */
  int *first, *last; /* [nlevels][nblocks] */
} otasklist;

static int cmp_task(const void *pa, const void *pb) {
  /* (level, block_num, iset, jset) as grid_ref_task_list.c:26-37, ties by
   * input position so that the order is deterministic */
  const otask *a = pa, *b = pb;
  if (a->level != b->level) return a->level - b->level;
  if (a->block_num != b->block_num) return a->block_num - b->block_num;
  if (a->iset != b->iset) return a->iset - b->iset;
  if (a->jset != b->jset) return a->jset - b->jset;
  return a->orig - b->orig;
}

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
    const double *dh_inv, void **out) {
  otasklist *t = xmalloc(sizeof(*t));
  t->ortho = orthorhombic;
  t->ntasks = ntasks;
  t->nlevels = nlevels;
  t->natoms = natoms;
  t->nkinds = nkinds;
  t->nblocks = nblocks;
  t->block_offsets = xmalloc(sizeof(int) * nblocks);
  memcpy(t->block_offsets, block_offsets, sizeof(int) * nblocks);
  t->atom_kinds = xmalloc(sizeof(int) * natoms);
  memcpy(t->atom_kinds, atom_kinds, sizeof(int) * natoms);
  t->atom_positions = xmalloc(sizeof(double) * 3 * natoms);
  memcpy(t->atom_positions, atom_positions, sizeof(double) * 3 * natoms);
  t->basis = xmalloc(sizeof(void *) * nkinds);
  memcpy(t->basis, basis_sets, sizeof(void *) * nkinds);
  t->tasks = xmalloc(sizeof(otask) * ntasks);
  for (int i = 0; i < ntasks; i++) {
    otask *k = &t->tasks[i];
    k->level = level_list[i];
    k->iatom = iatom_list[i];
    k->jatom = jatom_list[i];
    k->iset = iset_list[i];
    k->jset = jset_list[i];
    k->ipgf = ipgf_list[i];
    k->jpgf = jpgf_list[i];
    k->border_mask = border_mask_list[i];
    k->block_num = block_num_list[i];
    k->radius = radius_list[i];
    for (int d = 0; d < 3; d++)
      k->rab[d] = rab_list[3 * i + d];
    k->orig = i;
  }
  qsort(t->tasks, ntasks, sizeof(otask), cmp_task);
  int *lv[4] = {NULL, NULL, NULL, NULL};
  const int *src[4] = {npts_global, npts_local, shift_local, border_width};
  for (int q = 0; q < 4; q++) {
    lv[q] = xmalloc(sizeof(int) * 3 * nlevels);
    memcpy(lv[q], src[q], sizeof(int) * 3 * nlevels);
  }
  t->npts_global = lv[0];
  t->npts_local = lv[1];
  t->shift_local = lv[2];
  t->border_width = lv[3];
  t->dh = xmalloc(sizeof(double) * 9 * nlevels);
  memcpy(t->dh, dh, sizeof(double) * 9 * nlevels);
  t->dh_inv = xmalloc(sizeof(double) * 9 * nlevels);
  memcpy(t->dh_inv, dh_inv, sizeof(double) * 9 * nlevels);
  const size_t nlb = (size_t)nlevels * nblocks;
  t->first = xmalloc(sizeof(int) * nlb);
  t->last = xmalloc(sizeof(int) * nlb);
  for (size_t i = 0; i < nlb; i++) {
    t->first[i] = 0;
    t->last[i] = -1;
  }
  for (int i = 0; i < ntasks; i++) {
    const size_t key = (size_t)(t->tasks[i].level - 1) * nblocks + t->tasks[i].block_num - 1;
    if (i == 0 || t->tasks[i - 1].level != t->tasks[i].level ||
        t->tasks[i - 1].block_num != t->tasks[i].block_num)
      t->first[key] = i;
    t->last[key] = i;
  }
  t->maxco = 1;
  for (int k = 0; k < nkinds; k++)
    t->maxco = imax(t->maxco, basis_sets[k]->maxco);
  *out = t;
}

void oracle_free_task_list(void *p) {
  otasklist *t = p;
  if (!t)
    return;
  free(t->block_offsets);
  free(t->atom_kinds);
  free(t->atom_positions);
  free(t->basis);
  free(t->tasks);
  free(t->npts_global);
  free(t->npts_local);
  free(t->shift_local);
  free(t->border_width);
  free(t->dh);
  free(t->dh_inv);
  free(t->first);
  free(t->last);
  free(t);
}

typedef struct {
  int ncoa, ncob, ncoseta, ncosetb, nsgf_seta, nsgf_setb, nsgfa, nsgfb, sgfa,
      sgfb, maxcoa, maxcob;
} subdims;

static subdims sub_dims(const oracle_basis *ib, const oracle_basis *jb, int iset,
                        int jset) {
  subdims s;
  s.ncoseta = ncoset(ib->lmax[iset]);
  s.ncosetb = ncoset(jb->lmax[jset]);
  s.ncoa = ib->npgf[iset] * s.ncoseta;
  s.ncob = jb->npgf[jset] * s.ncosetb;
  s.nsgf_seta = ib->nsgf_set[iset];
  s.nsgf_setb = jb->nsgf_set[jset];
  s.nsgfa = ib->nsgf;
  s.nsgfb = jb->nsgf;
  s.sgfa = ib->first_sgf[iset] - 1;
  s.sgfb = jb->first_sgf[jset] - 1;
  s.maxcoa = ib->maxco;
  s.maxcob = jb->maxco;
  return s;
}

/* Spherical sub-block -> Cartesian pab[ncob][ncoa]
 * (grid_ref_task_list.c:237-271; the block is stored [sgfb][sgfa] when
 * iatom <= jatom, else [sgfa][sgfb]). */
static void load_pab(const oracle_basis *ib, const oracle_basis *jb, int iset,
                     int jset, bool transpose, const double *block, double *pab) {
  const subdims s = sub_dims(ib, jb, iset, jset);
  double *work = xmalloc(sizeof(double) * s.nsgf_setb * s.ncoa);
  for (int sb = 0; sb < s.nsgf_setb; sb++)
    for (int ca = 0; ca < s.ncoa; ca++) {
      double acc = 0.0;
      for (int sa = 0; sa < s.nsgf_seta; sa++) {
        const double p = transpose
                             ? block[(size_t)(s.sgfb + sb) * s.nsgfa + s.sgfa + sa]
                             : block[(size_t)(s.sgfa + sa) * s.nsgfb + s.sgfb + sb];
        acc += p * ib->sphi[(size_t)(s.sgfa + sa) * s.maxcoa + ca];
      }
      work[sb * s.ncoa + ca] = acc;
    }
  for (int cb = 0; cb < s.ncob; cb++)
    for (int ca = 0; ca < s.ncoa; ca++) {
      double acc = 0.0;
      for (int sb = 0; sb < s.nsgf_setb; sb++)
        acc += jb->sphi[(size_t)(s.sgfb + sb) * s.maxcob + cb] * work[sb * s.ncoa + ca];
      pab[cb * s.ncoa + ca] = acc;
    }
  free(work);
}

/* Cartesian hab[ncob][ncoa] -> accumulated into the spherical sub-block
 * (grid_ref_task_list.c:462-499). */
static void store_hab(const oracle_basis *ib, const oracle_basis *jb, int iset,
                      int jset, bool transpose, const double *hab, double *block) {
  const subdims s = sub_dims(ib, jb, iset, jset);
  double *work = xmalloc(sizeof(double) * s.nsgf_setb * s.ncoa);
  for (int sb = 0; sb < s.nsgf_setb; sb++)
    for (int ca = 0; ca < s.ncoa; ca++) {
      double acc = 0.0;
      for (int cb = 0; cb < s.ncob; cb++)
        acc += jb->sphi[(size_t)(s.sgfb + sb) * s.maxcob + cb] * hab[cb * s.ncoa + ca];
      work[sb * s.ncoa + ca] = acc;
    }
  for (int sb = 0; sb < s.nsgf_setb; sb++)
    for (int sa = 0; sa < s.nsgf_seta; sa++) {
      double acc = 0.0;
      for (int ca = 0; ca < s.ncoa; ca++)
        acc += work[sb * s.ncoa + ca] * ib->sphi[(size_t)(s.sgfa + sa) * s.maxcoa + ca];
      if (transpose)
        block[(size_t)(s.sgfb + sb) * s.nsgfa + s.sgfa + sa] += acc;
      else
        block[(size_t)(s.sgfa + sa) * s.nsgfb + s.sgfb + sb] += acc;
    }
  free(work);
}

void oracle_collocate_task_list(const void *p, int func, int nlevels,
                                const double *pab_blocks, double **grids) {
  const otasklist *t = p;
  if (nlevels != t->nlevels) {
    fprintf(stderr, "oracle: nlevels mismatch\n");
    abort();
  }
  for (int level = 0; level < t->nlevels; level++) {
    const int *ng = &t->npts_global[3 * level], *nl = &t->npts_local[3 * level];
    const size_t npts = (size_t)nl[0] * nl[1] * nl[2];
    const double *dh = &t->dh[9 * level], *dhi = &t->dh_inv[9 * level];
    const int nthreads = omp_get_max_threads();
    double **tl = xmalloc(sizeof(double *) * nthreads);
#pragma omp parallel num_threads(nthreads)
    {
      const int me = omp_get_thread_num();
      tl[me] = calloc(npts, sizeof(double));
      double *pab = xmalloc(sizeof(double) * t->maxco * t->maxco);
#pragma omp for schedule(dynamic, 1)
      for (int blk = 0; blk < t->nblocks; blk++) {
        const size_t key = (size_t)level * t->nblocks + blk;
        int cur_iset = -1, cur_jset = -1;
        for (int it = t->first[key]; it <= t->last[key]; it++) {
          const otask *k = &t->tasks[it];
          const int ia = k->iatom - 1, ja = k->jatom - 1;
          const oracle_basis *ib = t->basis[t->atom_kinds[ia] - 1];
          const oracle_basis *jb = t->basis[t->atom_kinds[ja] - 1];
          const int iset = k->iset - 1, jset = k->jset - 1;
          const subdims s = sub_dims(ib, jb, iset, jset);
          if (iset != cur_iset || jset != cur_jset) {
            load_pab(ib, jb, iset, jset, ia <= ja,
                     &pab_blocks[t->block_offsets[k->block_num - 1]], pab);
            cur_iset = iset;
            cur_jset = jset;
          }
          oracle_collocate_pgf_product(
              t->ortho, k->border_mask, func, ib->lmax[iset], ib->lmin[iset],
              jb->lmax[jset], jb->lmin[jset],
              ib->zet[iset * ib->maxpgf + k->ipgf - 1],
              jb->zet[jset * jb->maxpgf + k->jpgf - 1], (ia == ja) ? 1.0 : 2.0,
              dh, dhi, &t->atom_positions[3 * ia], k->rab, ng, nl,
              &t->shift_local[3 * level], &t->border_width[3 * level], k->radius,
              (k->ipgf - 1) * s.ncoseta, (k->jpgf - 1) * s.ncosetb, s.ncoa, s.ncob,
              pab, tl[me]);
        }
      }
      free(pab);
      /* sum the thread-local grids, each thread owning a slice of points */
#pragma omp for schedule(static)
      for (size_t i = 0; i < npts; i++) {
        double acc = 0.0;
        for (int q = 0; q < nthreads; q++)
          acc += tl[q][i];
        grids[level][i] = acc;
      }
    }
    for (int q = 0; q < nthreads; q++)
      free(tl[q]);
    free(tl);
  }
}

void oracle_integrate_task_list(const void *p, bool compute_tau, int natoms,
                                int nlevels, const double *pab_blocks,
                                const double *const *grids, double *hab_blocks,
                                size_t hab_len, double *forces, double *virial) {
  const otasklist *t = p;
  if (nlevels != t->nlevels || natoms != t->natoms) {
    fprintf(stderr, "oracle: nlevels/natoms mismatch\n");
    abort();
  }
  memset(hab_blocks, 0, sizeof(double) * hab_len);
  if (forces)
    memset(forces, 0, sizeof(double) * 3 * natoms);
  if (virial)
    memset(virial, 0, sizeof(double) * 9);
  const bool need_pab = forces != NULL || virial != NULL;
  for (int level = 0; level < t->nlevels; level++) {
    const int *ng = &t->npts_global[3 * level], *nl = &t->npts_local[3 * level];
    const double *dh = &t->dh[9 * level], *dhi = &t->dh_inv[9 * level];
#pragma omp parallel
    {
      double *pab = xmalloc(sizeof(double) * t->maxco * t->maxco);
      double *hab = xmalloc(sizeof(double) * t->maxco * t->maxco);
#pragma omp for schedule(dynamic, 1)
      for (int blk = 0; blk < t->nblocks; blk++) {
        const size_t key = (size_t)level * t->nblocks + blk;
        if (t->first[key] > t->last[key])
          continue;
        const otask *k0 = &t->tasks[t->first[key]];
        const int ia = k0->iatom - 1, ja = k0->jatom - 1;
        const oracle_basis *ib = t->basis[t->atom_kinds[ia] - 1];
        const oracle_basis *jb = t->basis[t->atom_kinds[ja] - 1];
        double *block = &hab_blocks[t->block_offsets[blk]];
        const double *pblock = need_pab ? &pab_blocks[t->block_offsets[blk]] : NULL;
        double f[6] = {0}, v[18] = {0};
        int it = t->first[key];
        while (it <= t->last[key]) {
          /* one run of tasks sharing (iset, jset) */
          const int iset = t->tasks[it].iset - 1, jset = t->tasks[it].jset - 1;
          const subdims s = sub_dims(ib, jb, iset, jset);
          if (need_pab)
            load_pab(ib, jb, iset, jset, ia <= ja, pblock, pab);
          memset(hab, 0, sizeof(double) * s.ncoa * s.ncob);
          for (; it <= t->last[key] && t->tasks[it].iset - 1 == iset &&
                 t->tasks[it].jset - 1 == jset;
               it++) {
            const otask *k = &t->tasks[it];
            oracle_integrate_pgf_product(
                t->ortho, compute_tau, k->border_mask, ib->lmax[iset],
                ib->lmin[iset], jb->lmax[jset], jb->lmin[jset],
                ib->zet[iset * ib->maxpgf + k->ipgf - 1],
                jb->zet[jset * jb->maxpgf + k->jpgf - 1], dh, dhi,
                &t->atom_positions[3 * ia], k->rab, ng, nl,
                &t->shift_local[3 * level], &t->border_width[3 * level],
                k->radius, (k->ipgf - 1) * s.ncoseta, (k->jpgf - 1) * s.ncosetb,
                s.ncoa, s.ncob, grids[level], hab, need_pab ? pab : NULL,
                forces ? f : NULL, virial ? v : NULL, NULL, NULL, NULL);
          }
          store_hab(ib, jb, iset, jset, ia <= ja, hab, block);
        }
        /* off-diagonal blocks count twice (grid_ref_task_list.c:625) */
        const double scale = (ia == ja) ? 1.0 : 2.0;
        if (forces) {
#pragma omp critical(oracle_forces)
          for (int d = 0; d < 3; d++) {
            forces[3 * ia + d] += scale * f[d];
            forces[3 * ja + d] += scale * f[3 + d];
          }
        }
        if (virial) {
#pragma omp critical(oracle_virial)
          for (int q = 0; q < 9; q++)
            virial[q] += scale * (v[q] + v[9 + q]);
        }
      }
      free(pab);
      free(hab);
    }
  }
}

long long oracle_count_task_points(const void *p, int func, long long *points_out,
                                   int *lp_out) {
  const otasklist *t = p;
  int amin_d, amax_d, bmin_d, bmax_d;
  func_ldiffs(func, &amin_d, &amax_d, &bmin_d, &bmax_d);
  long long total = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : total)
  for (int it = 0; it < t->ntasks; it++) {
    const otask *k = &t->tasks[it];
    const int level = k->level - 1, ia = k->iatom - 1, ja = k->jatom - 1;
    const oracle_basis *ib = t->basis[t->atom_kinds[ia] - 1];
    const oracle_basis *jb = t->basis[t->atom_kinds[ja] - 1];
    const int iset = k->iset - 1, jset = k->jset - 1;
    const int la = ib->lmax[iset] + amax_d, lb = jb->lmax[jset] + bmax_d;
    const long long np = cab_grid(
        1, t->ortho, k->border_mask, la, 0, lb, 0,
        ib->zet[iset * ib->maxpgf + k->ipgf - 1],
        jb->zet[jset * jb->maxpgf + k->jpgf - 1], 1.0, &t->dh[9 * level],
        &t->dh_inv[9 * level], &t->atom_positions[3 * ia], k->rab,
        &t->npts_global[3 * level], &t->npts_local[3 * level],
        &t->shift_local[3 * level], &t->border_width[3 * level], k->radius,
        NULL, NULL, 1);
    if (points_out)
      points_out[k->orig] = np;
    if (lp_out)
      lp_out[k->orig] = la + lb;
    total += np;
  }
  return total;
}
