// Per-task and per-subblock small dense transforms of the GB300 backend.
//
//  decontract   spherical P sub-block -> Cartesian pab           (per subblock)
//               (src/grid/ref/grid_ref_task_list.c:237-271, load_pab)
//  coefficients pab -> C_ab (grid_func) -> C_xyz about rp (-> C_ijk for the
//               general path)                                     (per task)
//               (common/grid_prepare_pab.h, ref/grid_ref_collint.h:698-911)
//  post         integrated C_xyz (C_ijk) -> C_ab -> hab, forces, virial
//               (ref/grid_ref_integrate.c:44-152, common/grid_process_vab.h)
//  contract_hab Cartesian hab -> spherical block, accumulated     (per subblock)
//               (src/grid/ref/grid_ref_task_list.c:462-499, store_hab)
//
// One warp per task / subblock, operands staged in shared memory.  The
// per-task work is templated on the arithmetic type: FP64 for the plain path,
// FP32 for the mixed path (accumulation into hab / forces / virial stays FP64
// atomics in both).
#include <cuda_runtime.h>

#include <cstdio>
#include <type_traits>

#include <algorithm>
#include <cstdint>
#include <vector>

#include "gb300_internal.h"
#include "numeric.cuh"

namespace gb300 {

namespace {

constexpr unsigned FULL = 0xffffffffu;

struct Orb {
  int l[3];
};
__device__ __forceinline__ Orb up(int d, Orb a) {
  a.l[d] += 1;
  return a;
}
__device__ __forceinline__ Orb dn(int d, Orb a) {
  a.l[d] = a.l[d] > 0 ? a.l[d] - 1 : 0;
  return a;
}
__device__ __forceinline__ int oidx(Orb a) { return coset(a.l[0], a.l[1], a.l[2]); }

// orbital of Cartesian index i within shell l (inverse of coset)
__device__ __forceinline__ Orb orb_of(int l, int i) {
  // coset ordering inside a shell: lx descending, then lz ascending
  int lx = l;
  int base = 0;
  while (i >= base + (l - lx + 1)) {
    base += l - lx + 1;
    lx--;
  }
  const int lz = i - base;
  Orb o;
  o.l[0] = lx;
  o.l[2] = lz;
  o.l[1] = l - lx - lz;
  return o;
}

// ------------------------------------------------------------------------
// grid_func: P_ab -> C_ab  (grid_prepare_pab.h:26-430)
// ------------------------------------------------------------------------
template <typename T> struct CabW {
  T *c;
  int n1;
  __device__ __forceinline__ void add(Orb a, Orb b, T v) const {
    if (v != T(0))
      atomicAdd(&c[oidx(b) * n1 + oidx(a)], v);
  }
  __device__ __forceinline__ void set(Orb a, Orb b, T v) const { c[oidx(b) * n1 + oidx(a)] = v; }
};

template <typename T>
__device__ void term_dij_b(int pair, T fa, Orb a, Orb b, T zb, const CabW<T> &w) {
  const int i1 = pair, i2 = (pair + 1) % 3;
  w.add(a, dn(i1, dn(i2, b)), T(b.l[i1] * b.l[i2]) * fa);
  w.add(a, up(i1, dn(i2, b)), T(-2) * zb * T(b.l[i2]) * fa);
  w.add(a, dn(i1, up(i2, b)), T(-2) * zb * T(b.l[i1]) * fa);
  w.add(a, up(i1, up(i2, b)), T(4) * zb * zb * fa);
}

template <typename T>
__device__ void term_dii_b(int d, T fa, Orb a, Orb b, T zb, const CabW<T> &w) {
  w.add(a, dn(d, dn(d, b)), T(b.l[d] * (b.l[d] - 1)) * fa);
  w.add(a, b, T(-2) * zb * T(2 * b.l[d] + 1) * fa);
  w.add(a, up(d, up(d, b)), T(4) * zb * zb * fa);
}

template <typename T>
__device__ void prep_one(int f, Orb a, Orb b, T za, T zb, T p, const CabW<T> &w) {
  if (f == 100) {
    w.set(a, b, p); // each (a, b) owns its entry
  } else if (f == 200) {
    for (int i = 0; i < 3; i++) {
      w.add(dn(i, a), dn(i, b), T(0.5) * T(a.l[i] * b.l[i]) * p);
      w.add(dn(i, a), up(i, b), -T(a.l[i]) * zb * p);
      w.add(up(i, a), dn(i, b), -za * T(b.l[i]) * p);
      w.add(up(i, a), up(i, b), T(2) * za * zb * p);
    }
  } else if (f >= 301 && f <= 303) {
    const int d = f - 301;
    w.add(a, dn(d, b), T(b.l[d]) * p);
    w.add(a, up(d, b), T(-2) * zb * p);
    w.add(dn(d, a), b, -T(a.l[d]) * p);
    w.add(up(d, a), b, T(2) * za * p);
  } else if (f >= 411 && f <= 433) {
    const int d = f / 10 - 41, r = f % 10 - 1;
    const Orb br = up(r, b);
    w.add(a, dn(d, br), T(b.l[d]) * p);
    w.add(a, up(d, br), T(-2) * zb * p);
    w.add(dn(d, a), br, -T(a.l[d]) * p);
    w.add(up(d, a), br, T(2) * za * p);
  } else if (f >= 501 && f <= 503) {
    const int d = f - 501;
    w.add(a, dn(d, b), T(b.l[d]) * p);
    w.add(a, up(d, b), T(-2) * zb * p);
    w.add(dn(d, a), b, T(a.l[d]) * p);
    w.add(up(d, a), b, T(-2) * za * p);
  } else if (f >= 901 && f <= 903) {
    const int d = f - 901;
    w.add(dn(d, a), b, -T(a.l[d]) * p);
    w.add(up(d, a), b, T(2) * za * p);
  } else if (f >= 904 && f <= 906) {
    const int d = f - 904;
    w.add(a, dn(d, b), -T(b.l[d]) * p);
    w.add(a, up(d, b), T(2) * zb * p);
  } else if (f >= 1001 && f <= 1003) {
    const int d = f - 1001;
    w.add(up(d, a), b, T(2) * za * p);
  } else if (f >= 601 && f <= 603) {
    const int d = f - 601;
    w.add(dn(d, a), dn(d, b), T(a.l[d] * b.l[d]) * p);
    w.add(dn(d, a), up(d, b), T(-2) * T(a.l[d]) * zb * p);
    w.add(up(d, a), dn(d, b), T(-2) * za * T(b.l[d]) * p);
    w.add(up(d, a), up(d, b), T(4) * za * zb * p);
  } else if (f >= 701 && f <= 703) {
    const int pair = f - 701, d1 = pair, d2 = (pair + 1) % 3;
    term_dij_b<T>(pair, T(a.l[d1] * a.l[d2]) * p, dn(d1, dn(d2, a)), b, zb, w);
    term_dij_b<T>(pair, T(-2) * za * T(a.l[d2]) * p, up(d1, dn(d2, a)), b, zb, w);
    term_dij_b<T>(pair, T(-2) * za * T(a.l[d1]) * p, dn(d1, up(d2, a)), b, zb, w);
    term_dij_b<T>(pair, T(4) * za * za * p, up(d1, up(d2, a)), b, zb, w);
  } else if (f >= 801 && f <= 803) {
    const int d = f - 801;
    term_dii_b<T>(d, T(a.l[d] * (a.l[d] - 1)) * p, dn(d, dn(d, a)), b, zb, w);
    term_dii_b<T>(d, T(-2) * za * T(2 * a.l[d] + 1) * p, a, b, zb, w);
    term_dii_b<T>(d, T(4) * za * za * p, up(d, up(d, a)), b, zb, w);
  }
}

// A group of lanes working on one task: the whole warp, or half of it for
// small tasks (two tasks per warp keep more lanes busy).
struct Grp {
  int lane, n;   // lane within the group, group size (16, 32, or the CTA)
  unsigned mask; // the group's lanes in the warp (groups up to 32 lanes)
  __device__ __forceinline__ void sync() const {
    if (n > 32)
      __syncthreads(); // the group is the whole CTA
    else
      __syncwarp(mask);
  }
};

// Group layout of a CTA: gsize 16 (two tasks per warp), 32 (one per warp) or
// blockDim.x (one large task per CTA, 128 or 256 threads).
struct GrpLayout {
  Grp g;
  int gid, ngroups, slot; // first task, stride, shared-memory slot in the CTA
};
__device__ __forceinline__ GrpLayout grp_layout(int gsize) {
  const int tid = threadIdx.x, per_cta = blockDim.x / gsize, gi = tid / gsize;
  const int sub = (tid & 31) / (gsize < 32 ? gsize : 32);
  const unsigned mask = gsize >= 32 ? 0xffffffffu : ((1u << gsize) - 1) << (sub * gsize);
  return GrpLayout{Grp{tid % gsize, gsize, mask}, (int)blockIdx.x * per_cta + gi,
                   (int)gridDim.x * per_cta, gi};
}

// ------------------------------------------------------------------------
// Binomial expansion tables alpha[dir][lxb][lxa][l]: coefficient of (x-p)^l
// in (x-a)^lxa (x-b)^lxb  (grid_ref_collint.h:838-861)
// ------------------------------------------------------------------------
__constant__ float c_binom[GB300_LP_MAX + 1][GB300_LP_MAX + 1];

// Entry orders of the transforms' per-lane loops, per (la, lb) with la, lb
// < kOrdL: lanes of a warp take consecutive entries, and their loops have
// very different trip counts (1 to ~10^3 terms), so the entries are sorted
// by their number of terms, longest first; neighbouring lanes then run
// loops of similar length.  Kind 0: the C_ab entries (a, b) of the post
// kernel, index ib * ncoset(la) + ia, (a_x + b_x + 1)(a_y + b_y + 1)
// (a_z + b_z + 1) terms.  Kind 1: the C_xyz outputs p (cidx order) of the
// coefficient kernel, #{(a, b): a + b >= p componentwise} terms.
constexpr int kOrdL = 9;
constexpr int kOrderWords = 495 * 495 + kOrdL * kOrdL * 969;
__device__ uint16_t g_order[kOrderWords];
__constant__ int c_order_off[2][kOrdL][kOrdL];

__device__ __forceinline__ const uint16_t *entry_order(int kind, int la, int lb) {
  return (la < kOrdL && lb < kOrdL) ? g_order + c_order_off[kind][la][lb] : nullptr;
}

// Term lists of the C_ab -> C_xyz gather for la, lb < kTermL: for output e
// (cidx order) the terms g_terms[g_tstart[e] .. g_tstart[e + 1]), each the
// C_ab index (x low 16 bits), the alpha offsets of z (x high 16 bits), x
// (y low) and y (y high) in the [3][lb + 1][la + 1][lp + 1] alpha table.
// The gather then costs a packed load and four shared-memory loads per term
// instead of the index arithmetic of the nested loops.  The terms keep the
// loops' order and the products their factor order, so the sums follow
// cab_cxyz_term's rounding (the mixed mode's energy error moved from 1e-10
// to 9e-10 Ha/atom with a different term order).
constexpr int kTermL = 4;
constexpr int kTermWords = 40000, kTStartWords = kTermL * kTermL * 100;
__device__ uint2 g_terms[kTermWords];
__device__ int g_tstart[kTStartWords];
__constant__ int c_tstart_off[kTermL][kTermL];


template <typename T>
__device__ void fill_alpha(T *alpha, int la, int lb, int lp, const double ra[3],
                           const double rb[3], const double rp[3], const Grp &g) {
  const int na = la + 1, nb = lb + 1, P = lp + 1;
  for (int e = g.lane; e < 3 * na * nb * P; e += g.n)
    alpha[e] = T(0);
  g.sync();
  for (int e = g.lane; e < 3 * na * nb; e += g.n) {
    const int d = e / (na * nb), r = e % (na * nb), xb = r / na, xa = r % na;
    const T pa = T(rp[d] - ra[d]), pb = T(rp[d] - rb[d]);
    T *al = alpha + ((size_t)(d * nb + xb) * na + xa) * P;
    T powa = T(1);
    for (int k = 0; k <= xa; k++) {
      const T wa = T(c_binom[xa][k]) * powa;
      T powb = T(1);
      for (int m = 0; m <= xb; m++) {
        al[xa - k + xb - m] += wa * T(c_binom[xb][m]) * powb;
        powb *= pb;
      }
      powa *= pa;
    }
  }
  g.sync();
}

// sum over C_ab entries of one C_xyz monomial (or the adjoint), gathering
// only pairs whose alpha products are structurally non-zero.
template <typename T>
__device__ T cab_cxyz_term(const T *cab, int n1, const T *alpha, int la, int lb,
                           int lp, int px, int py, int pz) {
  const int na = la + 1, nb = lb + 1, P = lp + 1;
  auto A = [&](int d, int xb, int xa, int l) {
    return alpha[((size_t)(d * nb + xb) * na + xa) * P + l];
  };
  // loop bounds visit only the pairs with a_d + b_d >= p_d
  T s = T(0);
  for (int az = 0; az <= la; az++)
    for (int bz = max(0, pz - az); bz <= lb; bz++) {
      const T wz = A(2, bz, az, pz);
      for (int ay = 0; ay <= la - az; ay++)
        for (int by = max(0, py - ay); by <= lb - bz; by++) {
          const T wyz = wz * A(1, by, ay, py);
          for (int ax = 0; ax <= la - az - ay; ax++)
            for (int bx = max(0, px - ax); bx <= lb - bz - by; bx++)
              s += wyz * A(0, bx, ax, px) * cab[coset(bx, by, bz) * n1 + coset(ax, ay, az)];
        }
    }
  return s;
}

// C_ab entry (a, b) from C_xyz (integrate adjoint of the above).  The
// (px, py, pz) terms run as one flat loop with carries, so lanes whose
// entries have equally many terms (the entry order sorts them so) keep the
// same control flow whatever the shape of their index ranges.
template <typename T>
__device__ T cxyz_cab_term(const T *cxyz, const T *alpha, int la, int lb, int lp, Orb a,
                           Orb b) {
  const int na = la + 1, nb = lb + 1, P = lp + 1;
  const T *ax = alpha + ((size_t)(0 * nb + b.l[0]) * na + a.l[0]) * P;
  const T *ay = alpha + ((size_t)(1 * nb + b.l[1]) * na + a.l[1]) * P;
  const T *az = alpha + ((size_t)(2 * nb + b.l[2]) * na + a.l[2]) * P;
  const int nx = a.l[0] + b.l[0] + 1, ny = a.l[1] + b.l[1] + 1, nz = a.l[2] + b.l[2] + 1;
  const int n = nx * ny * nz;
  // the x terms of a C_xyz row as a running dot product (one fused
  // multiply-add per term), folded in with alpha_y alpha_z at the row's end
  using M = Num<T>;
  int px = 0, py = 0, pz = 0, row = cidx(0, 0, 0, lp);
  T wyz = M::norm(ay[0] * az[0]);
  T s = M::zero(), d = M::zero();
  for (int t = 0; t < n; t++) {
    d = M::fma_acc(d, ax[px], cxyz[row + px]);
    if (++px == nx) {
      s = M::fma_acc(s, wyz, M::norm(d));
      d = M::zero();
      px = 0;
      if (++py == ny) {
        py = 0;
        ++pz;
      }
      if (pz < nz) {
        wyz = M::norm(ay[py] * az[pz]);
        row = cidx(pz, py, 0, lp);
      }
    }
  }
  return M::norm(s);
}

// General path: C_xyz (Cartesian, about P) <-> C_ijk (lattice indices).
// The polynomial p(r) in Cartesian offsets becomes q(u) = p(M u) in lattice
// offsets, M[c][d] = dh[d][c] (grid_ref_collint.h:698-762 expands every
// monomial into the product of three multinomials).  Here M is factorised on
// the host, per level, with partial pivoting, M = P^T L D U, and the change of
// variables runs as eight elementary substitutions, each a gather over the
// coefficient vector (one output per lane, no atomics):
//   permutation  x = P^T y         q[e] = p[l] with l[pi(i)] = e[i]
//   shear        y_r = z_r + b z_c  q[e] = sum_k C(e_r + k, k) b^k p[e + k (^r - ^c)]
//   scaling      y_r = d_r z_r      q[e] = p[e] d_0^e_0 d_1^e_1 d_2^e_2
// in the order P^T, L = S(1,0) S(2,0) S(2,1), D, U = S(0,2) S(1,2) S(0,1).
// A shear costs ncoset(lp) (mean exponent + 1) terms, against the
// O(lp^6) terms of the full multinomial expansion.  Integrate applies the
// transposed steps in reverse order.  The table (build_dh_table) holds per
// level: pi (3 entries), L10, L20, L21, D0, D1, D2, U02, U12, U01, in the
// arithmetic type T of the kernel.
template <typename T> __device__ __forceinline__ const T *dh_tab(const double *d, const float *f,
                                                                 const float2 *df);
template <> __device__ __forceinline__ const double *dh_tab<double>(const double *d, const float *,
                                                                    const float2 *) {
  return d;
}
template <> __device__ __forceinline__ const float *dh_tab<float>(const double *, const float *f,
                                                                  const float2 *) {
  return f;
}
template <> __device__ __forceinline__ const dfloat *dh_tab<dfloat>(const double *, const float *,
                                                                    const float2 *df) {
  return reinterpret_cast<const dfloat *>(df);
}

__device__ __forceinline__ int pick3(int i, int a, int b, int c) {
  return i == 0 ? a : (i == 1 ? b : c);
}

// shear y_r = z_r + b z_c (adjoint: its transpose) from in to out
template <typename T>
__device__ void lat_shear(const T *in, T *out, int lp, int r, int c, T b, bool adjoint,
                          const Grp &g) {
  using M = Num<T>;
  const int n = ncoset(lp);
  // source exponents move by k (d0, d1, d2) per term
  const int s = adjoint ? -1 : 1;
  const int d0 = s * ((r == 0) - (c == 0)), d1 = s * ((r == 1) - (c == 1)),
            d2 = s * ((r == 2) - (c == 2));
  for (int e = g.lane; e < n; e += g.n) {
    int l2, l1, l0;
    decode_cidx(e, lp, l2, l1, l0);
    const int lr = pick3(r, l0, l1, l2);
    const int kmax = adjoint ? lr : pick3(c, l0, l1, l2);
    T acc = M::zero(), pw = T(1);
    for (int k = 0; k <= kmax; k++) {
      const float cb = adjoint ? c_binom[lr][k] : c_binom[lr + k][k];
      acc = M::fma_acc(acc, M::mul(pw, T(cb)),
                       in[cidx(l2 + k * d2, l1 + k * d1, l0 + k * d0, lp)]);
      pw = M::mul(pw, b);
    }
    out[e] = M::norm(acc);
  }
}

template <typename T>
__device__ void lat_scale(const T *in, T *out, int lp, const T *dd, const Grp &g) {
  using M = Num<T>;
  const int n = ncoset(lp);
  for (int e = g.lane; e < n; e += g.n) {
    int l2, l1, l0;
    decode_cidx(e, lp, l2, l1, l0);
    T v = in[e];
    for (int k = 0; k < l0; k++)
      v = M::mul(v, dd[0]);
    for (int k = 0; k < l1; k++)
      v = M::mul(v, dd[1]);
    for (int k = 0; k < l2; k++)
      v = M::mul(v, dd[2]);
    out[e] = v;
  }
}

// permutation (forward: q[e] = p[l], l[pi(i)] = e[i]; adjoint: its inverse)
template <typename T>
__device__ void lat_perm(const T *in, T *out, int lp, const int pi[3], bool adjoint,
                         const Grp &g) {
  const int n = ncoset(lp);
  for (int e = g.lane; e < n; e += g.n) {
    int e2, e1, e0;
    decode_cidx(e, lp, e2, e1, e0);
    int l0, l1, l2;
    if (!adjoint) {
      // l[pi(i)] = e[i]
      l0 = pick3(pi[0] == 0 ? 0 : (pi[1] == 0 ? 1 : 2), e0, e1, e2);
      l1 = pick3(pi[0] == 1 ? 0 : (pi[1] == 1 ? 1 : 2), e0, e1, e2);
      l2 = pick3(pi[0] == 2 ? 0 : (pi[1] == 2 ? 1 : 2), e0, e1, e2);
    } else {
      // l[i] = e[pi(i)]
      l0 = pick3(pi[0], e0, e1, e2);
      l1 = pick3(pi[1], e0, e1, e2);
      l2 = pick3(pi[2], e0, e1, e2);
    }
    out[e] = in[cidx(l2, l1, l0, lp)];
  }
}

// C_ijk (forward) or C_xyz (adjoint) from the vector in a; b is scratch of
// the same size.  Returns the buffer holding the result (a or b).
template <typename T>
__device__ T *lattice_transform(const T *tab, int level, int lp, bool adjoint, T *a, T *b,
                                const Grp &g) {
  const T *t = tab + (size_t)level * kLatTab;
  const int pi[3] = {(int)Num<T>::to_double(t[0]), (int)Num<T>::to_double(t[1]),
                     (int)Num<T>::to_double(t[2])};
  // forward steps: perm, S(1,0,L10), S(2,0,L20), S(2,1,L21), D, S(0,2,U02),
  // S(1,2,U12), S(0,1,U01)
  const int sr[6] = {1, 2, 2, 0, 1, 0}, sc[6] = {0, 0, 1, 2, 2, 1};
  const int sb[6] = {3, 4, 5, 9, 10, 11};
  T *x = a, *y = b;
  auto swap = [&]() {
    T *tmp = x;
    x = y;
    y = tmp;
    g.sync();
  };
  if (!adjoint) {
    lat_perm<T>(x, y, lp, pi, false, g);
    swap();
    for (int s = 0; s < 6; s++) {
      if (s == 3) {
        lat_scale<T>(x, y, lp, t + 6, g);
        swap();
      }
      lat_shear<T>(x, y, lp, sr[s], sc[s], t[sb[s]], false, g);
      swap();
    }
  } else {
    for (int s = 5; s >= 0; s--) {
      lat_shear<T>(x, y, lp, sr[s], sc[s], t[sb[s]], true, g);
      swap();
      if (s == 3) {
        lat_scale<T>(x, y, lp, t + 6, g);
        swap();
      }
    }
    lat_perm<T>(x, y, lp, pi, true, g);
    swap();
  }
  return x;
}



// Decode the Cartesian index i (0 .. ncoset(lmax)-1) into an orbital.
__device__ __forceinline__ Orb orb_of_index(int i) {
  int l = 0;
  while (ncoset(l) <= i)
    l++;
  return orb_of(l, i - ncoset(l - 1));
}

// ------------------------------------------------------------------------
// Staged transforms: the C_ab <-> C_xyz change of basis one direction at a
// time.  C_xyz[p] = sum_{a,b} C_ab[a,b] prod_d alpha_d[b_d][a_d][p_d] is
// evaluated as three small contractions, x, then y, then z:
//   T1[(ay,az),(by,bz)][px] = sum_{ax,bx} C_ab[a,b] alpha_x[bx][ax][px]
//   T2[az][bz][(px,py)]     = sum_{ay,by} T1[(ay,az),(by,bz)][px] alpha_y[by][ay][py]
//   C_xyz[(px,py,pz)]        = sum_{az,bz} T2[az][bz][(px,py)] alpha_z[bz][az][pz]
// and the integrate adjoint in reverse (z, y, x).  A direct gather costs
// each output prod_d (a_d + b_d + 1)-style sums over all (a, b) pairs; the
// stages cost about a quarter of that at la = lb = 4 (the reference's own
// cab_to_cxyz, grid_ref_collint.h:827-911, runs the nested loops directly).
// Index helpers: pairs (u, v) with u + v <= L in the order of u + v, then v.
// ------------------------------------------------------------------------
__device__ __forceinline__ int pidx(int u, int v) {
  const int s = u + v;
  return (s * (s + 1)) / 2 + v;
}
__device__ __forceinline__ void pdecode(int i, int &u, int &v) {
  int s = 0;
  while (((s + 1) * (s + 2)) / 2 <= i)
    s++;
  v = i - (s * (s + 1)) / 2;
  u = s - v;
}

template <typename T>
__device__ void cab_to_cxyz_staged(const T *cab, int n1, const T *alpha, int la, int lb, int lp,
                                   T *t1, T *t2, T *cxyz, T pref, const uint16_t *ord,
                                   const Grp &g) {
  using M = Num<T>;
  const int na = la + 1, nb = lb + 1, P = lp + 1, npa = ntri(la), npb = ntri(lb),
            nt = ntri(lp);
  auto A = [&](int d, int xb, int xa) { return alpha + ((size_t)(d * nb + xb) * na + xa) * P; };
  // x: T1[(ay,az),(by,bz)][px]
  for (int e = g.lane; e < npa * npb * P; e += g.n) {
    const int px = e % P, r = e / P, ipb = r % npb, ipa = r / npb;
    int ay, az, by, bz;
    pdecode(ipa, ay, az);
    pdecode(ipb, by, bz);
    const int ra = la - ay - az, rb = lb - by - bz;
    T acc = M::zero();
    if (px <= ra + rb)
      for (int ax = 0; ax <= ra; ax++)
        for (int bx = px > ax ? px - ax : 0; bx <= rb; bx++)
          acc = M::fma_acc(acc, A(0, bx, ax)[px],
                           cab[coset(bx, by, bz) * n1 + coset(ax, ay, az)]);
    t1[e] = M::norm(acc);
  }
  g.sync();
  // y: T2[az][bz][(px,py)]
  for (int e = g.lane; e < na * nb * nt; e += g.n) {
    const int it = e % nt, r = e / nt, bz = r % nb, az = r / nb;
    int px, py;
    pdecode(it, px, py);
    T acc = M::zero();
    if (px + py <= (la - az) + (lb - bz))
      for (int ay = 0; ay <= la - az; ay++)
        for (int by = py > ay ? py - ay : 0; by <= lb - bz; by++)
          if (px <= (la - ay - az) + (lb - by - bz))
            acc = M::fma_acc(acc, A(1, by, ay)[py],
                             t1[((size_t)pidx(ay, az) * npb + pidx(by, bz)) * P + px]);
    t2[e] = M::norm(acc);
  }
  g.sync();
  // z: C_xyz
  for (int i = g.lane; i < ncoset(lp); i += g.n) {
    const int e = ord ? ord[i] : i;
    int pz, py, px;
    decode_cidx(e, lp, pz, py, px);
    T acc = M::zero();
    for (int az = 0; az <= la; az++)
      for (int bz = pz > az ? pz - az : 0; bz <= lb; bz++)
        if (px + py <= (la - az) + (lb - bz))
          acc = M::fma_acc(acc, A(2, bz, az)[pz], t2[(size_t)(az * nb + bz) * nt + pidx(px, py)]);
    cxyz[e] = M::mul(M::norm(acc), pref);
  }
}

template <typename T>
__device__ void cxyz_to_cab_staged(const T *cxyz, const T *alpha, int la, int lb, int lp,
                                   T *t1, T *t2, T *cab, int m1, T pref, const Grp &g) {
  using M = Num<T>;
  const int na = la + 1, nb = lb + 1, P = lp + 1, npa = ntri(la), npb = ntri(lb),
            nt = ntri(lp);
  auto A = [&](int d, int xb, int xa) { return alpha + ((size_t)(d * nb + xb) * na + xa) * P; };
  // z: T2[az][bz][(px,py)] = sum_pz alpha_z C_xyz
  for (int e = g.lane; e < na * nb * nt; e += g.n) {
    const int it = e % nt, r = e / nt, bz = r % nb, az = r / nb;
    int px, py;
    pdecode(it, px, py);
    T acc = M::zero();
    if (px + py <= (la - az) + (lb - bz)) {
      const T *al = A(2, bz, az);
      const int pzmax = az + bz < lp - px - py ? az + bz : lp - px - py;
      for (int pz = 0; pz <= pzmax; pz++)
        acc = M::fma_acc(acc, al[pz], cxyz[cidx(pz, py, px, lp)]);
    }
    t2[e] = M::norm(acc);
  }
  g.sync();
  // y: T1[(ay,az),(by,bz)][px] = sum_py alpha_y T2
  for (int e = g.lane; e < npa * npb * P; e += g.n) {
    const int px = e % P, r = e / P, ipb = r % npb, ipa = r / npb;
    int ay, az, by, bz;
    pdecode(ipa, ay, az);
    pdecode(ipb, by, bz);
    T acc = M::zero();
    if (px <= (la - ay - az) + (lb - by - bz)) {
      const T *al = A(1, by, ay);
      const T *src = t2 + (size_t)(az * nb + bz) * nt;
      for (int py = 0; py <= ay + by; py++)
        acc = M::fma_acc(acc, al[py], src[pidx(px, py)]);
    }
    t1[e] = M::norm(acc);
  }
  g.sync();
  // x: C_ab[a,b] = sum_px alpha_x T1
  const int m2 = ncoset(lb);
  for (int e = g.lane; e < m1 * m2; e += g.n) {
    const Orb oa = orb_of_index(e % m1), ob = orb_of_index(e / m1);
    const T *al = A(0, ob.l[0], oa.l[0]);
    const T *src =
        t1 + ((size_t)pidx(oa.l[1], oa.l[2]) * npb + pidx(ob.l[1], ob.l[2])) * P;
    T acc = M::zero();
    for (int px = 0; px <= oa.l[0] + ob.l[0]; px++)
      acc = M::fma_acc(acc, al[px], src[px]);
    cab[e] = M::mul(M::norm(acc), pref);
  }
}

// store of one coefficient in the grid kernels' arithmetic
template <typename Tout, typename U>
__device__ __forceinline__ void store_coef(void *out, size_t i, U v) {
  if constexpr (std::is_same<Tout, dfloat>::value) {
    if constexpr (std::is_same<U, dfloat>::value)
      ((dfloat *)out)[i] = v;
    else if constexpr (std::is_same<U, float>::value)
      ((dfloat *)out)[i] = dfloat{v, 0.f};
    else
      ((dfloat *)out)[i] = df_make(to_double(v));
  } else if constexpr (std::is_same<Tout, float>::value && std::is_same<U, float>::value) {
    ((float *)out)[i] = v;
  } else {
    ((Tout *)out)[i] = (Tout)to_double(v);
  }
}

// ------------------------------------------------------------------------
// coefficients of one task (one warp): P_ab -> C_ab -> C_xyz (-> C_ijk)
// ------------------------------------------------------------------------
template <typename U, typename Tout>
__device__ void coef_task(const CoefArgs &a, int t, const TaskDesc &d, double *ws, const Grp &g) {
  const SubblockDesc sb = a.subs[d.subblock];
  const int la_max = d.la_max + a.d.la_max, lb_max = d.lb_max + a.d.lb_max;
  const int lp = la_max + lb_max;
  const int n1 = ncoset(la_max), n2 = ncoset(lb_max);
  double *cabd = ws;
  U *cab = (U *)cabd; // converted in place after the FP64 accumulation
  U *alpha = (U *)(cabd + (size_t)n1 * n2);
  U *cxyz = (U *)((double *)alpha + 3 * (size_t)(la_max + 1) * (lb_max + 1) * (lp + 1));
  U *cijk = (U *)((double *)cxyz + ncoset(lp));
  for (int e = g.lane; e < n1 * n2; e += g.n)
    cabd[e] = 0.0;
  g.sync();
  // P_ab -> C_ab in FP64 (grid_prepare_pab.h; a few operations per element)
  const CabW<double> w{cabd, n1};
  const double *pab = a.pab_cart + sb.cart_offset;
  const int na = ncoset(d.la_max) - ncoset(d.la_min - 1);
  const int nb = ncoset(d.lb_max) - ncoset(d.lb_min - 1);
  for (int e = g.lane; e < na * nb; e += g.n) {
    const int ia = ncoset(d.la_min - 1) + e % na, ib = ncoset(d.lb_min - 1) + e / na;
    const double p = pab[(size_t)(d.o2 + ib) * sb.ncoa + d.o1 + ia];
    prep_one<double>(a.func, orb_of_index(ia), orb_of_index(ib), d.zeta, d.zetb, p, w);
  }
  g.sync();
  if constexpr (sizeof(U) == sizeof(double)) {
    for (int e = g.lane; e < n1 * n2; e += g.n) { // each lane rewrites only its own slots
      const double v = cabd[e];
      cab[e] = U(v);
    }
  } else {
    // 4-byte U, in ascending chunks of g.n elements: the values of chunk k
    // land in doubles below (k+1) g.n / 2, all of which were read by then
    for (int base = 0; base < n1 * n2; base += g.n) {
      const int e = base + g.lane;
      const double v = e < n1 * n2 ? cabd[e] : 0.0;
      g.sync();
      if (e < n1 * n2)
        cab[e] = U(v);
    }
  }
  g.sync();
  const double *ra = a.atom_pos + 3 * d.iatom;
  double rb[3];
  for (int i = 0; i < 3; i++)
    rb[i] = ra[i] + d.rab[i];
  fill_alpha<U>(alpha, la_max, lb_max, lp, ra, rb, d.rp, g);
  const U pref = U(d.prefexp * ((d.iatom == d.jatom) ? 1.0 : 2.0));
  const int nco = ncoset(lp);
  const bool general = d.flags & TF_GENERAL;
  // (at low lp the outputs' term counts differ little and the plain order
  // keeps the stores contiguous)
  const uint16_t *ord = lp >= 6 ? entry_order(1, la_max, lb_max) : nullptr;
  if (uses_staged(a.transform, la_max, lb_max, true)) {
    U *t1 = (U *)((double *)cijk + nco);
    U *t2 = (U *)((double *)t1 + (size_t)ntri(la_max) * ntri(lb_max) * (lp + 1));
    cab_to_cxyz_staged<U>(cab, n1, alpha, la_max, lb_max, lp, t1, t2, cxyz, pref, ord, g);
    g.sync();
    const U *cl = general ? lattice_transform<U>(dh_tab<U>(a.dhtab, a.dhtab_f, a.dhtab_df),
                                                 d.level, lp, false, cxyz, cijk, g)
                          : cxyz;
    for (int e = g.lane; e < nco; e += g.n)
      store_coef<Tout, U>(a.coef, (size_t)a.coef_off[t] + e, cl[e]);
    g.sync();
    return;
  }
  for (int i = g.lane; i < nco; i += g.n) {
    const int e = ord ? ord[i] : i;
    int pz, py, px;
    decode_cidx(e, lp, pz, py, px);
    U v;
    if (la_max < kTermL && lb_max < kTermL) {
      const int *ts = g_tstart + c_tstart_off[la_max][lb_max];
      U acc = U(0);
      for (int q = ts[e]; q < ts[e + 1]; q++) {
        const uint2 w = g_terms[q];
        acc += alpha[w.x >> 16] * alpha[w.y >> 16] * alpha[w.y & 0xffffu] * cab[w.x & 0xffffu];
      }
      v = acc * pref;
    } else {
      v = cab_cxyz_term<U>(cab, n1, alpha, la_max, lb_max, lp, px, py, pz) * pref;
    }
    if (general)
      cxyz[e] = v;
    else
      store_coef<Tout, U>(a.coef, (size_t)a.coef_off[t] + e, v);
  }
  if (general) {
    g.sync();
    const U *cl = lattice_transform<U>(dh_tab<U>(a.dhtab, a.dhtab_f, a.dhtab_df), d.level, lp,
                                       false, cxyz, cijk, g);
    for (int e = g.lane; e < nco; e += g.n)
      store_coef<Tout, U>(a.coef, (size_t)a.coef_off[t] + e, cl[e]);
  }
  g.sync();
}

// U: working type of the tasks (the mixed mode launches one kernel per work
// queue, each in the type of its class)
template <typename U, typename Tout>
__global__ void __launch_bounds__(256) coefficients_kernel(CoefArgs a, int words_per_group,
                                                           int gsize) {
  extern __shared__ __align__(16) unsigned char smem[];
  const GrpLayout gl = grp_layout(gsize);
  const Grp &g = gl.g;
  const int gid = gl.gid, ngroups = gl.ngroups;
  double *ws = (double *)smem + (size_t)gl.slot * words_per_group;
  const int nt = a.order ? a.norder : a.ntasks;
  for (int i = gid; i < nt; i += ngroups) {
    const int t = a.order ? a.order[i] : i;
    const TaskDesc d = a.tasks[t];
    if (d.flags & TF_SKIP)
      continue;
    coef_task<U, Tout>(a, t, d, ws, g);
  }
}

// ------------------------------------------------------------------------
// post: integrated C_xyz -> C_ab -> hab / forces / virial (one warp per task)
// ------------------------------------------------------------------------
// Cartesian orbitals by coset index with neighbour tables, so that the
// derivative terms of the post kernel look their orbitals up instead of
// recomputing coset indices: g_orb_lxyz[i] = lx | ly << 4 | lz << 8,
// g_orb_up[d][i] the index of the orbital + 1_d, g_orb_dn[d][i] of the
// orbital - 1_d (the orbital itself where its d component is 0, as dn()).
constexpr int kOrbL = 12;                                     // orbitals with l < kOrbL
constexpr int kOrbN = kOrbL * (kOrbL + 1) * (kOrbL + 2) / 6; // their number
__device__ uint16_t g_orb_lxyz[kOrbN];
__device__ uint16_t g_orb_up[3][kOrbN];
__device__ uint16_t g_orb_dn[3][kOrbN];
struct OI {
  int i;
};
__device__ __forceinline__ int ocomp(OI a, int d) {
  return (__ldg(&g_orb_lxyz[a.i]) >> (4 * d)) & 15;
}
__device__ __forceinline__ OI oup(int d, OI a) { return OI{__ldg(&g_orb_up[d][a.i])}; }
__device__ __forceinline__ OI odn(int d, OI a) { return OI{__ldg(&g_orb_dn[d][a.i])}; }

template <typename T> struct VabCtx {
  const T *c;
  int m1;
  T za, zb;
  T rab[3];
  __device__ __forceinline__ T g(OI a, OI b) const { return c[b.i * m1 + a.i]; }
};

enum { V_HAB, V_FA, V_FB, V_VA, V_VB };

template <typename T>
__device__ T vab_plain(const VabCtx<T> &x, int kind, int i, int j, OI a, OI b) {
  switch (kind) {
  case V_HAB:
    return x.g(a, b);
  case V_FA:
    return T(2) * x.za * x.g(oup(i, a), b) - T(ocomp(a, i)) * x.g(odn(i, a), b);
  case V_FB:
    return T(2) * x.zb * (x.g(oup(i, a), b) - x.rab[i] * x.g(a, b)) -
           T(ocomp(b, i)) * x.g(a, odn(i, b));
  case V_VA:
    return T(2) * x.za * x.g(oup(i, oup(j, a)), b) - T(ocomp(a, j)) * x.g(oup(i, odn(j, a)), b);
  default:
    return T(2) * x.zb *
               (x.g(oup(i, oup(j, a)), b) - x.g(oup(i, a), b) * x.rab[j] -
                x.g(oup(j, a), b) * x.rab[i] + x.g(a, b) * x.rab[j] * x.rab[i]) -
           T(ocomp(b, j)) * x.g(a, oup(i, odn(j, b)));
  }
}

template <typename T>
__device__ T vab(const VabCtx<T> &x, bool tau, int kind, int i, int j, OI a, OI b) {
  if (!tau)
    return vab_plain(x, kind, i, j, a, b);
  T s = T(0);
  for (int k = 0; k < 3; k++) {
    const int ak = ocomp(a, k), bk = ocomp(b, k);
    s += T(0.5) * T(ak * bk) * vab_plain(x, kind, i, j, odn(k, a), odn(k, b));
    s -= x.za * T(bk) * vab_plain(x, kind, i, j, oup(k, a), odn(k, b));
    s -= T(ak) * x.zb * vab_plain(x, kind, i, j, odn(k, a), oup(k, b));
    s += T(2) * x.za * x.zb * vab_plain(x, kind, i, j, oup(k, a), oup(k, b));
  }
  return s;
}

template <typename U>
__device__ void post_task(const PostArgs &a, int t, const TaskDesc &d, double *ws, const Grp &g,
                          double f[6], double v[9]) {
  const SubblockDesc sb = a.subs[d.subblock];
  const int la_max = d.la_max + a.d.la_max, lb_max = d.lb_max + a.d.lb_max;
  const int lp = la_max + lb_max;
  const int m1 = ncoset(la_max), m2 = ncoset(lb_max);
  U *cab = (U *)ws;
  U *alpha = (U *)(ws + (size_t)m1 * m2);
  U *cxyz = (U *)((double *)alpha + 3 * (size_t)(la_max + 1) * (lb_max + 1) * (lp + 1));
  U *cijk = (U *)((double *)cxyz + ncoset(lp));
  const int nco = ncoset(lp);
  const double *src = a.coef + a.coef_off[t];
  const bool general = d.flags & TF_GENERAL;
  for (int e = g.lane; e < nco; e += g.n) {
    if (general)
      cijk[e] = U(src[e]);
    else
      cxyz[e] = U(src[e]);
  }
  g.sync();
  const U *cx = general ? lattice_transform<U>(dh_tab<U>(a.dhtab, a.dhtab_f, a.dhtab_df),
                                               d.level, lp, true, cijk, cxyz, g)
                        : cxyz;
  const double *ra = a.atom_pos + 3 * d.iatom;
  double rb[3];
  for (int i = 0; i < 3; i++)
    rb[i] = ra[i] + d.rab[i];
  fill_alpha<U>(alpha, la_max, lb_max, lp, ra, rb, d.rp, g);
  const U pref = U(d.prefexp);
  if (uses_staged(a.transform, la_max, lb_max, false)) {
    U *t1 = (U *)((double *)cijk + nco);
    U *t2 = (U *)((double *)t1 + (size_t)ntri(la_max) * ntri(lb_max) * (lp + 1));
    cxyz_to_cab_staged<U>(cx, alpha, la_max, lb_max, lp, t1, t2, cab, m1, pref, g);
  } else {
    const uint16_t *ord = entry_order(0, la_max, lb_max);
    for (int i = g.lane; i < m1 * m2; i += g.n) {
      const int e = ord ? ord[i] : i;
      const Orb oa = orb_of_index(e % m1), ob = orb_of_index(e / m1);
      cab[e] = cxyz_cab_term<U>(cx, alpha, la_max, lb_max, lp, oa, ob) * pref;
    }
  }
  g.sync();
  VabCtx<U> x{cab, m1, U(d.zeta), U(d.zetb), {U(d.rab[0]), U(d.rab[1]), U(d.rab[2])}};
  const bool tau = a.compute_tau;
  const int na = ncoset(d.la_max) - ncoset(d.la_min - 1);
  const int nb = ncoset(d.lb_max) - ncoset(d.lb_min - 1);
  const double *pab = a.pab_cart ? a.pab_cart + sb.cart_offset : nullptr;
  double *hab = a.hab_cart + sb.cart_offset;
  // With tau, forces and virial are linear in the density matrix: the tau
  // shifts move onto it once (P', below), and the plain formulas then run
  // once per entry of P' instead of twelve times per pair.  P' lives in the
  // alpha / C_xyz / C_ijk area, free once C_ab is built.
  const int n1p = ncoset(d.la_max + 1), n2p = ncoset(d.lb_max + 1);
  const bool tau_fv = tau && (a.forces || a.virial) &&
                      (size_t)n1p * n2p <= 3 * (size_t)(la_max + 1) * (lb_max + 1) * (lp + 1) +
                                               2 * (size_t)ncoset(lp);
  // forces and virial accumulate per lane in the working type (the FP64 pipe
  // is the scarce unit on GB300) and reach FP64 once per task
  using M = Num<U>;
  U fu[6], vu[9];
  for (int i = 0; i < 6; i++)
    fu[i] = M::zero();
  for (int i = 0; i < 9; i++)
    vu[i] = M::zero();
  for (int e = g.lane; e < na * nb; e += g.n) {
    const int ia = ncoset(d.la_min - 1) + e % na, ib = ncoset(d.lb_min - 1) + e / na;
    const OI oa{ia}, ob{ib};
    const size_t el = (size_t)(d.o2 + ib) * sb.ncoa + d.o1 + ia;
    atomicAdd(&hab[el], to_double(vab<U>(x, tau, V_HAB, 0, 0, oa, ob)));
    if ((a.forces || a.virial) && !tau_fv) {
      const U p = M::from(pab[el]);
      if (a.forces)
        for (int i = 0; i < 3; i++) {
          fu[i] = M::fma_acc(fu[i], p, vab<U>(x, tau, V_FA, i, 0, oa, ob));
          fu[3 + i] = M::fma_acc(fu[3 + i], p, vab<U>(x, tau, V_FB, i, 0, oa, ob));
        }
      if (a.virial)
        for (int i = 0; i < 3; i++)
          for (int j = 0; j < 3; j++)
            vu[i * 3 + j] = M::fma_acc(vu[i * 3 + j], p,
                                       M::add(vab<U>(x, tau, V_VA, i, j, oa, ob),
                                              vab<U>(x, tau, V_VB, i, j, oa, ob)));
    }
  }
  if (tau_fv) {
    // P'(a', b') = sum_k of the four tau terms' weights times P at the
    // shifted pair that maps onto (a', b'):
    //   0.5 (a'_k + 1)(b'_k + 1) P(a' + 1_k, b' + 1_k)
    //   - zeta_a (b'_k + 1) P(a' - 1_k, b' + 1_k)      (a'_k >= 1)
    //   - zeta_b (a'_k + 1) P(a' + 1_k, b' - 1_k)      (b'_k >= 1)
    //   + 2 zeta_a zeta_b P(a' - 1_k, b' - 1_k)        (a'_k, b'_k >= 1)
    // with P zero outside the task's block (the inverse of vab's tau sum).
    double *pp = (double *)alpha;
    const int ia0 = ncoset(d.la_min - 1), ia1 = ncoset(d.la_max);
    const int ib0 = ncoset(d.lb_min - 1), ib1 = ncoset(d.lb_max);
    auto P = [&](Orb oa, Orb ob) -> double {
      const int ia = oidx(oa), ib = oidx(ob);
      if (ia < ia0 || ia >= ia1 || ib < ib0 || ib >= ib1)
        return 0.0;
      return pab[(size_t)(d.o2 + ib) * sb.ncoa + d.o1 + ia];
    };
    g.sync(); // every lane is done with alpha and C_xyz
    for (int e = g.lane; e < n1p * n2p; e += g.n) {
      const Orb oa = orb_of_index(e % n1p), ob = orb_of_index(e / n1p);
      double s = 0.0;
      for (int k = 0; k < 3; k++) {
        const double ak = oa.l[k], bk = ob.l[k];
        s += 0.5 * (ak + 1.0) * (bk + 1.0) * P(up(k, oa), up(k, ob));
        if (oa.l[k] >= 1)
          s -= d.zeta * (bk + 1.0) * P(dn(k, oa), up(k, ob));
        if (ob.l[k] >= 1)
          s -= d.zetb * (ak + 1.0) * P(up(k, oa), dn(k, ob));
        if (oa.l[k] >= 1 && ob.l[k] >= 1)
          s += 2.0 * d.zeta * d.zetb * P(dn(k, oa), dn(k, ob));
      }
      pp[e] = s;
    }
    g.sync();
    for (int e = g.lane; e < n1p * n2p; e += g.n) {
      const double pd = pp[e];
      if (pd == 0.0)
        continue;
      const U p = M::from(pd);
      const OI oa{e % n1p}, ob{e / n1p};
      if (a.forces)
        for (int i = 0; i < 3; i++) {
          fu[i] = M::fma_acc(fu[i], p, vab_plain<U>(x, V_FA, i, 0, oa, ob));
          fu[3 + i] = M::fma_acc(fu[3 + i], p, vab_plain<U>(x, V_FB, i, 0, oa, ob));
        }
      if (a.virial)
        for (int i = 0; i < 3; i++)
          for (int j = 0; j < 3; j++)
            vu[i * 3 + j] = M::fma_acc(vu[i * 3 + j], p,
                                       M::add(vab_plain<U>(x, V_VA, i, j, oa, ob),
                                              vab_plain<U>(x, V_VB, i, j, oa, ob)));
    }
  }
  if (a.forces)
    for (int i = 0; i < 6; i++)
      f[i] += to_double(M::norm(fu[i]));
  if (a.virial)
    for (int i = 0; i < 9; i++)
      v[i] += to_double(M::norm(vu[i]));
  g.sync();
}

template <typename U>
__global__ void __launch_bounds__(256) post_kernel(PostArgs a, int words_per_group, int gsize) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ double vir_cta[9];
  const int lane = threadIdx.x & 31;
  const GrpLayout gl = grp_layout(gsize);
  const Grp &g = gl.g;
  const int gid = gl.gid, ngroups = gl.ngroups;
  const int wsz = gsize < 32 ? gsize : 32; // lanes of a group within one warp
  double *ws = (double *)smem + (size_t)gl.slot * words_per_group;
  if (threadIdx.x < 9)
    vir_cta[threadIdx.x] = 0.0;
  __syncthreads();
  const int nt = a.order ? a.norder : a.ntasks;
  for (int i = gid; i < nt; i += ngroups) {
    const int t = a.order ? a.order[i] : i;
    const TaskDesc d = a.tasks[t];
    if (d.flags & TF_SKIP)
      continue;
    double f[6] = {0, 0, 0, 0, 0, 0}, v[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    post_task<U>(a, t, d, ws, g, f, v);
    const double scale = (d.iatom == d.jatom) ? 1.0 : 2.0;
    // sums over each warp's part of the group (xor offsets below the part
    // size stay inside it); the first lane of each part adds its sum
    if (a.forces) {
      for (int i = 0; i < 6; i++) {
        double s = f[i];
        for (int o = wsz / 2; o > 0; o >>= 1)
          s += __shfl_xor_sync(g.mask, s, o);
        f[i] = s;
      }
      if (lane % wsz == 0)
        for (int i = 0; i < 3; i++) {
          atomicAdd(&a.forces[3 * d.iatom + i], scale * f[i]);
          atomicAdd(&a.forces[3 * d.jatom + i], scale * f[3 + i]);
        }
    }
    if (a.virial) {
      for (int i = 0; i < 9; i++) {
        double s = v[i];
        for (int o = wsz / 2; o > 0; o >>= 1)
          s += __shfl_xor_sync(g.mask, s, o);
        v[i] = s;
      }
      if (lane % wsz == 0)
        for (int i = 0; i < 9; i++)
          atomicAdd(&vir_cta[i], scale * v[i]);
    }
  }
  __syncthreads();
  if (a.virial && threadIdx.x < 9)
    atomicAdd(&a.virial[threadIdx.x], vir_cta[threadIdx.x]);
}

// ------------------------------------------------------------------------
// post of one task of the single-task integrate (FP64, one CTA): C_xyz ->
// C_ab -> hab, the forces and virials of atoms a and b separately, and the
// derivative blocks hdab, hadb, a_hdab, all accumulated into the caller's
// arrays (src/grid/ref/grid_ref_integrate.c:81-145)
// ------------------------------------------------------------------------
__global__ void __launch_bounds__(128) pgf_post_kernel(PgfPostArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ double red[27];
  const Grp g{(int)threadIdx.x, (int)blockDim.x, 0xffffffffu};
  const TaskDesc d = *a.task;
  const int la_max = d.la_max + a.d.la_max, lb_max = d.lb_max + a.d.lb_max;
  const int lp = la_max + lb_max;
  const int m1 = ncoset(la_max), m2 = ncoset(lb_max), nco = ncoset(lp);
  double *ws = (double *)smem;
  double *cab = ws;
  double *alpha = ws + (size_t)m1 * m2;
  double *cxyz = alpha + 3 * (size_t)(la_max + 1) * (lb_max + 1) * (lp + 1);
  double *cijk = cxyz + nco;
  const bool general = d.flags & TF_GENERAL;
  for (int e = g.lane; e < nco; e += g.n)
    (general ? cijk : cxyz)[e] = a.coef[e];
  if (threadIdx.x < 27)
    red[threadIdx.x] = 0.0;
  g.sync();
  const double *cx = general ? lattice_transform<double>(a.dhtab, d.level, lp, true, cijk, cxyz, g)
                             : cxyz;
  double rb[3];
  for (int i = 0; i < 3; i++)
    rb[i] = a.atom_pos[i] + d.rab[i];
  fill_alpha<double>(alpha, la_max, lb_max, lp, a.atom_pos, rb, d.rp, g);
  for (int e = g.lane; e < m1 * m2; e += g.n)
    cab[e] = cxyz_cab_term<double>(cx, alpha, la_max, lb_max, lp, orb_of_index(e % m1),
                                   orb_of_index(e / m1)) *
             d.prefexp;
  g.sync();
  const VabCtx<double> x{cab, m1, d.zeta, d.zetb, {d.rab[0], d.rab[1], d.rab[2]}};
  const bool tau = a.compute_tau;
  const int na = ncoset(d.la_max) - ncoset(d.la_min - 1);
  const int nb = ncoset(d.lb_max) - ncoset(d.lb_min - 1);
  double acc[27]; // forces a, b; virials a, b
  for (int i = 0; i < 27; i++)
    acc[i] = 0.0;
  for (int e = g.lane; e < na * nb; e += g.n) {
    const int ia = ncoset(d.la_min - 1) + e % na, ib = ncoset(d.lb_min - 1) + e / na;
    const OI oa{ia}, ob{ib};
    const size_t el = (size_t)(d.o2 + ib) * a.n1 + d.o1 + ia;
    a.hab[el] += vab<double>(x, tau, V_HAB, 0, 0, oa, ob);
    const double p = a.pab ? a.pab[el] : 0.0;
    for (int i = 0; i < 3; i++) {
      if (a.forces) {
        acc[i] += p * vab<double>(x, tau, V_FA, i, 0, oa, ob);
        acc[3 + i] += p * vab<double>(x, tau, V_FB, i, 0, oa, ob);
      }
      if (a.virials)
        for (int j = 0; j < 3; j++) {
          acc[6 + i * 3 + j] += p * vab<double>(x, tau, V_VA, i, j, oa, ob);
          acc[15 + i * 3 + j] += p * vab<double>(x, tau, V_VB, i, j, oa, ob);
        }
      if (a.hdab)
        a.hdab[el * 3 + i] += vab_plain<double>(x, V_FA, i, 0, oa, ob);
      if (a.hadb)
        a.hadb[el * 3 + i] += vab_plain<double>(x, V_FB, i, 0, oa, ob);
      if (a.a_hdab)
        for (int j = 0; j < 3; j++)
          a.a_hdab[(el * 3 + i) * 3 + j] += vab_plain<double>(x, V_VA, i, j, oa, ob);
    }
  }
  for (int i = 0; i < 27; i++) {
    double v = acc[i];
    for (int o = 16; o > 0; o >>= 1)
      v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0)
      atomicAdd(&red[i], v);
  }
  __syncthreads();
  if (threadIdx.x < 6 && a.forces)
    a.forces[threadIdx.x] += red[threadIdx.x];
  if (threadIdx.x < 18 && a.virials)
    a.virials[threadIdx.x] += red[6 + threadIdx.x];
}

// ------------------------------------------------------------------------
// decontract / contract: one warp per subblock, FP64
// ------------------------------------------------------------------------
__global__ void __launch_bounds__(128) decontract_kernel(ContractArgs a, int words_per_warp) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int lane = threadIdx.x & 31;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  double *work = (double *)smem + (size_t)(threadIdx.x >> 5) * words_per_warp;
  for (int s = gw; s < a.nsubs; s += nwarps) {
    const SubblockDesc sb = a.subs[s];
    const double *blk = a.blocks + sb.block_offset;
    double *out = a.cart + sb.cart_offset;
    auto P = [&](int sbi, int sai) {
      return sb.transpose ? blk[(size_t)(sb.sgfb + sbi) * sb.nsgfa + sb.sgfa + sai]
                          : blk[(size_t)(sb.sgfa + sai) * sb.nsgfb + sb.sgfb + sbi];
    };
    if (sb.identity) {
      for (int e = lane; e < sb.ncoa * sb.ncob; e += 32)
        out[e] = P(e / sb.ncoa, e % sb.ncoa);
    } else {
      // work[sb][ca] = sum_sa P[sb][sa] sphi_a[sa][ca]
      for (int e = lane; e < sb.nsgf_setb * sb.ncoa; e += 32) {
        const int r = e / sb.ncoa, ca = e % sb.ncoa;
        double acc = 0.0;
        for (int sa = 0; sa < sb.nsgf_seta; sa++)
          acc += P(r, sa) * a.sphi[sb.sphia + (size_t)sa * sb.maxcoa + ca];
        work[e] = acc;
      }
      __syncwarp();
      for (int e = lane; e < sb.ncob * sb.ncoa; e += 32) {
        const int cb = e / sb.ncoa, ca = e % sb.ncoa;
        double acc = 0.0;
        for (int r = 0; r < sb.nsgf_setb; r++)
          acc += a.sphi[sb.sphib + (size_t)r * sb.maxcob + cb] * work[r * sb.ncoa + ca];
        out[e] = acc;
      }
      __syncwarp();
    }
  }
}

__global__ void __launch_bounds__(128) contract_hab_kernel(ContractArgs a, int words_per_warp) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int lane = threadIdx.x & 31;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  double *work = (double *)smem + (size_t)(threadIdx.x >> 5) * words_per_warp;
  for (int s = gw; s < a.nsubs; s += nwarps) {
    const SubblockDesc sb = a.subs[s];
    double *blk = a.blocks_out + sb.block_offset;
    const double *hab = a.cart + sb.cart_offset;
    auto H = [&](int sbi, int sai) -> double & {
      return sb.transpose ? blk[(size_t)(sb.sgfb + sbi) * sb.nsgfa + sb.sgfa + sai]
                          : blk[(size_t)(sb.sgfa + sai) * sb.nsgfb + sb.sgfb + sbi];
    };
    if (sb.identity) {
      for (int e = lane; e < sb.ncoa * sb.ncob; e += 32)
        H(e / sb.ncoa, e % sb.ncoa) += hab[e];
    } else {
      // work[sb][ca] = sum_cb sphi_b[sb][cb] hab[cb][ca]
      for (int e = lane; e < sb.nsgf_setb * sb.ncoa; e += 32) {
        const int r = e / sb.ncoa, ca = e % sb.ncoa;
        double acc = 0.0;
        for (int cb = 0; cb < sb.ncob; cb++)
          acc += a.sphi[sb.sphib + (size_t)r * sb.maxcob + cb] * hab[(size_t)cb * sb.ncoa + ca];
        work[e] = acc;
      }
      __syncwarp();
      for (int e = lane; e < sb.nsgf_setb * sb.nsgf_seta; e += 32) {
        const int r = e / sb.nsgf_seta, sa = e % sb.nsgf_seta;
        double acc = 0.0;
        for (int ca = 0; ca < sb.ncoa; ca++)
          acc += work[r * sb.ncoa + ca] * a.sphi[sb.sphia + (size_t)sa * sb.maxcoa + ca];
        H(r, sa) += acc;
      }
      __syncwarp();
    }
  }
}

int grid_size_for(int nwarps_needed, int warps_per_cta = 4) {
  int nb = (nwarps_needed + warps_per_cta - 1) / warps_per_cta;
  if (nb > 152 * 32)
    nb = 152 * 32;
  return nb < 1 ? 1 : nb;
}

} // namespace

static void upload_orders() {
  std::vector<uint16_t> tab;
  std::vector<int> off(2 * kOrdL * kOrdL);
  std::vector<int> ox, oy, oz; // orbital of Cartesian index
  for (int l = 0; l < kOrdL; l++)
    for (int lx = l; lx >= 0; lx--)
      for (int lz = 0; lz <= l - lx; lz++) {
        ox.push_back(lx);
        oy.push_back(l - lx - lz);
        oz.push_back(lz);
      }
  for (size_t i = 0; i < ox.size(); i++)
    if (coset(ox[i], oy[i], oz[i]) != (int)i)
      return launch_error("entry orders: orbital order mismatch");
  {
    // orbital tables of the post kernel's derivative terms
    static uint16_t lxyz[kOrbN], upt[3][kOrbN], dnt[3][kOrbN];
    int i = 0;
    for (int l = 0; l < kOrbL; l++)
      for (int lx = l; lx >= 0; lx--)
        for (int lz = 0; lz <= l - lx; lz++, i++) {
          const int c[3] = {lx, l - lx - lz, lz};
          lxyz[i] = (uint16_t)(c[0] | (c[1] << 4) | (c[2] << 8));
          for (int d = 0; d < 3; d++) {
            int u[3] = {c[0], c[1], c[2]}, w[3] = {c[0], c[1], c[2]};
            u[d] += 1;
            w[d] = w[d] > 0 ? w[d] - 1 : 0;
            upt[d][i] = (uint16_t)coset(u[0], u[1], u[2]);
            dnt[d][i] = (uint16_t)coset(w[0], w[1], w[2]);
          }
        }
    if (i != kOrbN)
      return launch_error("orbital tables: size mismatch");
    cudaMemcpyToSymbol(g_orb_lxyz, lxyz, sizeof(lxyz));
    cudaMemcpyToSymbol(g_orb_up, upt, sizeof(upt));
    cudaMemcpyToSymbol(g_orb_dn, dnt, sizeof(dnt));
  }
  std::vector<std::pair<long long, int>> v;
  auto push_sorted = [&]() {
    std::stable_sort(v.begin(), v.end(), [](const std::pair<long long, int> &x,
                                            const std::pair<long long, int> &y) {
      return x.first > y.first;
    });
    for (auto &p : v)
      tab.push_back((uint16_t)p.second);
  };
  for (int la = 0; la < kOrdL; la++)
    for (int lb = 0; lb < kOrdL; lb++) {
      const int m1 = ncoset(la), m2 = ncoset(lb), lp = la + lb;
      off[(0 * kOrdL + la) * kOrdL + lb] = (int)tab.size();
      v.clear();
      for (int ib = 0; ib < m2; ib++)
        for (int ia = 0; ia < m1; ia++)
          v.push_back({(long long)(ox[ia] + ox[ib] + 1) * (oy[ia] + oy[ib] + 1) *
                           (oz[ia] + oz[ib] + 1),
                       ib * m1 + ia});
      push_sorted();
      off[(1 * kOrdL + la) * kOrdL + lb] = (int)tab.size();
      v.clear();
      for (int e = 0; e < ncoset(lp); e++) {
        int pz, py, px;
        decode_cidx(e, lp, pz, py, px);
        long long n = 0;
        for (int ia = 0; ia < m1; ia++) {
          const int q = std::max(px - ox[ia], 0) + std::max(py - oy[ia], 0) +
                        std::max(pz - oz[ia], 0);
          n += ncoset(lb - q);
        }
        v.push_back({n, e});
      }
      push_sorted();
    }
  if (tab.size() > (size_t)kOrderWords)
    return launch_error("entry orders: table exceeds its size");
  // term lists of the C_ab -> C_xyz gather
  std::vector<uint2> terms;
  std::vector<int> tstart;
  int toff[kTermL][kTermL];
  for (int la = 0; la < kTermL; la++)
    for (int lb = 0; lb < kTermL; lb++) {
      const int m1 = ncoset(la), m2 = ncoset(lb), lp = la + lb, P = lp + 1;
      const int na = la + 1, nb = lb + 1;
      toff[la][lb] = (int)tstart.size();
      auto aoff = [&](int d, int xb, int xa, int l) { return ((d * nb + xb) * na + xa) * P + l; };
      for (int e = 0; e < ncoset(lp); e++) {
        int pz, py, px;
        decode_cidx(e, lp, pz, py, px);
        tstart.push_back((int)terms.size());
        // the order of cab_cxyz_term's loops
        for (int az = 0; az <= la; az++)
          for (int bz = std::max(0, pz - az); bz <= lb; bz++)
            for (int ay = 0; ay <= la - az; ay++)
              for (int by = std::max(0, py - ay); by <= lb - bz; by++)
                for (int ax = 0; ax <= la - az - ay; ax++)
                  for (int bx = std::max(0, px - ax); bx <= lb - bz - by; bx++) {
                    const unsigned ci = (unsigned)(coset(bx, by, bz) * m1 + coset(ax, ay, az));
                    const unsigned azo = (unsigned)aoff(2, bz, az, pz);
                    const unsigned axo = (unsigned)aoff(0, bx, ax, px);
                    const unsigned ayo = (unsigned)aoff(1, by, ay, py);
                    terms.push_back(make_uint2(ci | (azo << 16), axo | (ayo << 16)));
                  }
      }
      tstart.push_back((int)terms.size());
    }
  if (terms.size() > (size_t)kTermWords || tstart.size() > (size_t)kTStartWords)
    return launch_error("term lists: table exceeds its size");
  cudaMemcpyToSymbol(g_terms, terms.data(), terms.size() * sizeof(uint2));
  cudaMemcpyToSymbol(g_tstart, tstart.data(), tstart.size() * sizeof(int));
  cudaMemcpyToSymbol(c_tstart_off, toff, sizeof(toff));
  cudaMemcpyToSymbol(g_order, tab.data(), tab.size() * sizeof(uint16_t));
  cudaMemcpyToSymbol(c_order_off, off.data(), off.size() * sizeof(int));
}

static void upload_binomials() {
  static bool done = false;
  if (done)
    return;
  upload_orders();
  float b[GB300_LP_MAX + 1][GB300_LP_MAX + 1] = {};
  for (int n = 0; n <= GB300_LP_MAX; n++) {
    b[n][0] = 1.f;
    for (int k = 1; k <= n; k++)
      b[n][k] = b[n - 1][k - 1] + (k <= n - 1 ? b[n - 1][k] : 0.f);
  }
  cudaMemcpyToSymbol(c_binom, b, sizeof(b));
  done = true;
}

void launch_decontract(const ContractArgs &a, cudaStream_t s) {
  if (a.nsubs == 0)
    return;
  const size_t per_warp = sizeof(double) * (size_t)a.words;
  const int nw = warps_for(per_warp);
  if (nw < 1)
    return launch_error("decontraction: sub-block too large for shared memory");
  const size_t smem = nw * per_warp;
  set_smem((const void *)decontract_kernel, smem);
  decontract_kernel<<<grid_size_for(a.nsubs, nw), 32 * nw, smem, s>>>(a, a.words);
  count_launch();
}

void launch_contract_hab(const ContractArgs &a, cudaStream_t s) {
  if (a.nsubs == 0)
    return;
  const size_t per_warp = sizeof(double) * (size_t)a.words;
  const int nw = warps_for(per_warp);
  if (nw < 1)
    return launch_error("contraction: sub-block too large for shared memory");
  const size_t smem = nw * per_warp;
  set_smem((const void *)contract_hab_kernel, smem);
  contract_hab_kernel<<<grid_size_for(a.nsubs, nw), 32 * nw, smem, s>>>(a, a.words);
  count_launch();
}

// two tasks per warp (groups of 16 lanes) while the per-task work is small;
// one task per 4-warp CTA when its shared memory would leave an SM with few
// warps (high angular momenta)
constexpr int kSmallTaskWords = 1024, kLargeTaskWords = 4096;

struct GroupLaunch {
  int gsize, threads, grid;
  size_t smem;
};
// large_threads: the CTA of a large task; 256 where the kernel's registers
// still let that many warps reside (more warps for an issue-bound kernel),
// else 128
static GroupLaunch group_launch(int words_per_group, int ntasks, int large_threads = 256) {
  GroupLaunch L{};
  if (words_per_group > kLargeTaskWords) {
    L.gsize = L.threads = large_threads;
    L.smem = (size_t)words_per_group * 8;
    L.grid = std::max(1, std::min(ntasks, 152 * 32));
    return L;
  }
  L.gsize = words_per_group <= kSmallTaskWords ? 16 : 32;
  const size_t per_warp = (size_t)words_per_group * 8 * (32 / L.gsize);
  const int nw = warps_for(per_warp);
  L.threads = 32 * nw;
  L.smem = nw * per_warp;
  L.grid = nw < 1 ? 0 : grid_size_for(ntasks, nw);
  return L;
}

template <typename U, typename Tout>
static void launch_coef_t(const CoefArgs &a, int words_per_group, cudaStream_t s) {
  const GroupLaunch L = group_launch(words_per_group, a.order ? a.norder : a.ntasks);
  if (L.grid < 1 || L.smem > kSmemBudget)
    return launch_error("coefficients: angular momenta too large for shared memory");
  auto k = coefficients_kernel<U, Tout>;
  set_smem((const void *)k, L.smem);
  k<<<L.grid, L.threads, L.smem, s>>>(a, words_per_group, L.gsize);
  count_launch();
}

void launch_coefficients_mixed(const CoefArgs &a, int work, int words_per_warp, cudaStream_t s) {
  if ((a.order ? a.norder : a.ntasks) == 0)
    return;
  upload_binomials();
  if (work == ARITH_FP32)
    launch_coef_t<float, dfloat>(a, words_per_warp, s);
  else if (work == ARITH_FP64)
    launch_coef_t<double, dfloat>(a, words_per_warp, s);
  else
    launch_coef_t<dfloat, dfloat>(a, words_per_warp, s);
}

void launch_coefficients(const CoefArgs &a, int arith, int words_per_warp, cudaStream_t s) {
  if (a.ntasks == 0)
    return;
  upload_binomials();
  if (arith == ARITH_FP32)
    launch_coef_t<float, float>(a, words_per_warp, s);
  else if (arith == ARITH_MIXED)
    launch_coef_t<dfloat, dfloat>(a, words_per_warp, s);
  else
    launch_coef_t<double, double>(a, words_per_warp, s);
}

template <typename U>
static void launch_post_t(const PostArgs &a, int words_per_group, cudaStream_t s) {
  // the FP32 and FP64 post kernels take 120-128 registers: 256-thread CTAs
  // would not add resident warps (measured slower); the double-float one
  // takes 80
  const GroupLaunch L = group_launch(words_per_group, a.order ? a.norder : a.ntasks,
                                     std::is_same<U, dfloat>::value ? 256 : 128);
  if (L.grid < 1 || L.smem > kSmemBudget)
    return launch_error("post-processing: angular momenta too large for shared memory");
  auto k = post_kernel<U>;
  set_smem((const void *)k, L.smem);
  k<<<L.grid, L.threads, L.smem, s>>>(a, words_per_group, L.gsize);
  count_launch();
}

void launch_post_mixed(const PostArgs &a, int work, int words_per_warp, cudaStream_t s) {
  if ((a.order ? a.norder : a.ntasks) == 0)
    return;
  upload_binomials();
  if (work == ARITH_FP32)
    launch_post_t<float>(a, words_per_warp, s);
  else if (work == ARITH_FP64)
    launch_post_t<double>(a, words_per_warp, s);
  else
    launch_post_t<dfloat>(a, words_per_warp, s);
}

void launch_post(const PostArgs &a, int arith, int words_per_warp, cudaStream_t s) {
  if (a.ntasks == 0)
    return;
  upload_binomials();
  if (arith == ARITH_FP32)
    launch_post_t<float>(a, words_per_warp, s);
  else if (arith == ARITH_MIXED)
    launch_post_t<dfloat>(a, words_per_warp, s);
  else
    launch_post_t<double>(a, words_per_warp, s);
}

bool coefficients_fit(int words_per_group) {
  const GroupLaunch L = group_launch(words_per_group, 1);
  return L.grid >= 1 && L.smem <= kSmemBudget;
}

void launch_pgf_post(const PgfPostArgs &a, cudaStream_t s) {
  upload_binomials();
  const size_t smem = sizeof(double) * (size_t)a.words;
  if (smem > kSmemBudget)
    return launch_error("single-task post-processing: angular momenta too large for shared memory");
  set_smem((const void *)pgf_post_kernel, smem);
  pgf_post_kernel<<<1, 128, smem, s>>>(a);
  count_launch();
}

size_t coef_words(int la, int lb, bool staged) {
  return coef_smem_words(ncoset(la), ncoset(lb), la, lb, la + lb) +
         (staged ? staged_words(la, lb, la + lb) : 0);
}

} // namespace gb300
