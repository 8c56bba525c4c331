// Task-list generation and density-matrix block packing on the device.
//
// Generation builds, for one geometry, the argument arrays of
// grid_create_task_list the way Quickstep does
// (src/task_list_methods.F:117-501 generate_qs_task_list, :652-719
// task_list_inner_loop, :738-800 compute_pgf_properties, block numbering and
// buffer offsets :507-618), with the screening of the synthetic workloads:
//   * every atom pair i <= j and every periodic image n within the pair
//     distance cut rmax (for i == j only image 0 and one image of each +/- n
//     pair);
//   * every primitive pair (iset, ipgf, jset, jpgf), in that order, whose
//     Gaussian-product prefactor exp(-zeta zetb / zetp |rab|^2) exceeds eps;
//     or, after grid_gb300_taskgen_set_radius_screen, Quickstep's own
//     screening by the basis radii (set radius + kind radius, set + set,
//     primitive + set, primitive + primitive against |rab|,
//     task_list_methods.F:673-696), in its order iset, jset, ipgf, jpgf;
//   * the grid level of gaussian_gridlevel (src/pw_env/gaussian_gridlevels.F:
//     147-167): the coarsest level whose cutoff covers zetp * rel_cutoff;
//   * the radius of exp_radius_very_extended (src/aobasis/ao_util.F:207-290)
//     over exp_radius (:95-180): single-precision exponential, doubling then
//     interval contraction by 0.38 / 0.62, absolute accuracy 1e-2;
//   * one block per atom pair with tasks, numbered in pair order, its buffer
//     offset the running sum of nsgf(i) * nsgf(j).
// The host generator (csrc/workload.c) runs the same loops in C; every array
// made here equals its array element for element.  Every comparison that
// decides the outcome (distance cut, prefactor screen, the bisection's
// g(r) < threshold) is first taken in single precision, with a margin above
// the rounding of both sides (GB300's FP64 rate is a small fraction of its
// FP32 rate); inside the margin the exact double expression decides, in the
// host code's order with explicitly rounded operations (no contraction into
// FMAs), the single-precision exponential as exp in double rounded once to
// float (the correctly rounded value but for inputs within 2^-29 of a
// rounding boundary), and integer powers by repeated multiplication
// (Fortran's r**l).  The values written (rab, radius) are always exact
// double results.
//
// Kernels: one thread per atom pair counts the tasks of its images (only the
// images whose lattice box can reach the distance cut are visited); a
// three-phase scan turns the counts into task offsets and block numbers; one
// thread per block writes its tasks in order; one thread per task finds the
// radius.  Two synchronisations per run read back the totals.
//
// Packing is rs_pack_buffer / rs_unpack_buffer (src/task_list_methods.F:
// 2593-2674) on device memory: blocks gathered from a block store into the
// pab buffer at the task list's block offsets, and hab slices added back;
// block lookup by (row, col) replaces dbcsr_get_block_p.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "gb300_internal.h"
#include "grid_gb300.h"

#define GB300_API extern "C" __attribute__((visibility("default")))

namespace gb300 {
namespace {

[[noreturn]] void tg_fail(const char *what, int code) {
  fprintf(stderr, "grid_gb300 error: task generation: %s (%d)\n", what, code);
  abort();
}
#define CKT(x)                                                                 \
  do {                                                                         \
    cudaError_t e_ = (x);                                                      \
    if (e_ != cudaSuccess)                                                     \
      tg_fail(#x, (int)e_);                                                    \
  } while (0)

constexpr int kTgMaxLevels = 16;
constexpr int kTgMaxL = 12;             // la + lb <= 2 * kTgMaxL
constexpr int kTgPoly = 2 * kTgMaxL + 1; // polynomial coefficients per task
constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

struct TgParams {
  int natoms;
  long long npairs;
  int nimg[3];
  double cell[3][3];
  double rmax, eps, rel_cutoff;
  int nlevels;
  double cutoff[kTgMaxLevels];
  int maxpgf;
  // single-precision copies for the screening decisions
  float cellf[3][3], cellnorm[3], rmaxf, leps;
  float cinvf[3][3], hf[3];  // inverse cell; column norms (reciprocal lengths)
  const float *zetf;   // [nsets][maxpgf]
  // basis-radius screening (Quickstep's task_list_inner_loop), when set
  int screen;
  const double *rpgf;        // [nsets][maxpgf]
  const double *set_radius;  // [nsets]
  const double *kind_radius; // [nkinds]
  const double *pos;   // [natoms][3]
  const int *kind;     // [natoms], 0-based
  const int *set_off;  // [nkinds]
  const int *nset;     // [nkinds]
  const int *nsgf;     // [nkinds]
  const int *lmax;     // [nsets]
  const int *npgf;     // [nsets]
  const double *zet;   // [nsets][maxpgf]
};

struct BinomTable {
  double v[kTgMaxL + 1][kTgMaxL + 1];
};
constexpr BinomTable make_binom() {
  BinomTable t{};
  for (int n = 0; n <= kTgMaxL; n++) {
    t.v[n][0] = 1.0;
    for (int k = 1; k <= n; k++)
      t.v[n][k] = t.v[n][k - 1] * (n - k + 1) / k;
  }
  return t;
}
__constant__ BinomTable kBinom = make_binom();

struct TgOut {
  int *level, *iatom, *jatom, *iset, *jset, *ipgf, *jpgf, *border_mask, *block_num;
  double *radius, *rab;
  int *block_offsets;
};

// IEEE double operations that are never fused
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }

// pair index p -> (i, j), i <= j; row i starts at i n - i (i - 1) / 2
__device__ __forceinline__ long long row_start(long long i, long long n) {
  return i * n - i * (i - 1) / 2;
}
__device__ void pair_of(long long p, int n, int &i, int &j) {
  // estimate in single precision, then exact integer corrections
  const float b = 2.0f * n + 1.0f;
  long long r = (long long)((b - sqrtf(fmaxf(b * b - 8.0f * (float)p, 0.0f))) * 0.5f);
  r = r < 0 ? 0 : (r > n - 1 ? n - 1 : r);
  while (r > 0 && row_start(r, n) > p)
    r--;
  while (r < n - 1 && row_start(r + 1, n) <= p)
    r++;
  i = (int)r;
  j = (int)(r + (p - row_start(r, n)));
}

// rab of image n and |rab|^2, in the host code's order of operations
__device__ __forceinline__ double image_rab(const TgParams &P, const double ra[3],
                                           const double rj[3], const int n[3], double rab[3]) {
#pragma unroll
  for (int d = 0; d < 3; d++)
    rab[d] = dadd(dadd(dadd(dsub(rj[d], ra[d]), dmul((double)n[0], P.cell[0][d])),
                       dmul((double)n[1], P.cell[1][d])),
                  dmul((double)n[2], P.cell[2][d]));
  return dadd(dadd(dmul(rab[0], rab[0]), dmul(rab[1], rab[1])), dmul(rab[2], rab[2]));
}

// Decisions are taken in single precision where a margin of 1e-3 (in the
// exponent) covers every rounding of both sides, and by the exact double
// expression inside that band: the outcome is the host's.
constexpr float kMargin = 1e-3f;

// exp(-za zb / (za + zb) rab2) > eps
__device__ __forceinline__ bool passes(const TgParams &P, double za, double zb, float zaf,
                                       float zbf, double rab2, float rab2f) {
  const float y = -zaf * (zbf / (zaf + zbf)) * rab2f;
  const float diff = y - P.leps;
  if (diff > kMargin)
    return true;
  if (diff < -kMargin)
    return false;
  const double zetp = dadd(za, zb), f = ddiv(zb, zetp);
  const double pref = exp(dmul(dmul(-za, f), rab2));
  return pref > P.eps;
}

// Quickstep's screening of one atom pair (task_list_methods.F:673-696):
// sets and primitives whose radii reach |rab|, in the loop order iset, jset,
// ipgf, jpgf; f(iset, jset, ipgf, jpgf) for each pair that is kept
template <class F>
__device__ __forceinline__ void radius_screen(const TgParams &P, int ki, int kj, double rab2,
                                              F &&f) {
  const double dab = __dsqrt_rn(rab2);
  const double krb = P.kind_radius[kj];
  const int si0 = P.set_off[ki], sj0 = P.set_off[kj];
  for (int is = 0; is < P.nset[ki]; is++) {
    const double sra = P.set_radius[si0 + is];
    if (dadd(sra, krb) < dab)
      continue;
    for (int js = 0; js < P.nset[kj]; js++) {
      const double srb = P.set_radius[sj0 + js];
      if (dadd(sra, srb) < dab)
        continue;
      for (int ip = 0; ip < P.npgf[si0 + is]; ip++) {
        const double rpa = P.rpgf[(size_t)(si0 + is) * P.maxpgf + ip];
        if (dadd(rpa, srb) < dab)
          continue;
        for (int jp = 0; jp < P.npgf[sj0 + js]; jp++)
          if (!(dadd(rpa, P.rpgf[(size_t)(sj0 + js) * P.maxpgf + jp]) < dab))
            f(is, js, ip, jp);
      }
    }
  }
}

// tasks of one image of the pair (ki, kj): primitive pairs that pass
__device__ int image_tasks(const TgParams &P, int ki, int kj, double rab2) {
  int c = 0;
  if (P.screen) {
    radius_screen(P, ki, kj, rab2, [&](int, int, int, int) { c++; });
    return c;
  }
  const float rab2f = __double2float_rn(rab2);
  const int si0 = P.set_off[ki], sj0 = P.set_off[kj];
  for (int is = 0; is < P.nset[ki]; is++)
    for (int ip = 0; ip < P.npgf[si0 + is]; ip++) {
      const size_t ia = (size_t)(si0 + is) * P.maxpgf + ip;
      const double za = P.zet[ia];
      const float zaf = P.zetf[ia];
      for (int js = 0; js < P.nset[kj]; js++)
        for (int jp = 0; jp < P.npgf[sj0 + js]; jp++) {
          const size_t ib = (size_t)(sj0 + js) * P.maxpgf + jp;
          c += passes(P, za, P.zet[ib], zaf, P.zetf[ib], rab2, rab2f);
        }
    }
  return c;
}

// an atom pair's positions: exact, and their difference in single precision
struct PairPos {
  double ra[3], rj[3];
  float df[3];
};
__device__ __forceinline__ PairPos pair_pos(const TgParams &P, int i, int j) {
  PairPos q;
#pragma unroll
  for (int d = 0; d < 3; d++) {
    q.ra[d] = P.pos[3 * i + d];
    q.rj[d] = P.pos[3 * j + d];
    q.df[d] = __double2float_rn(dsub(q.rj[d], q.ra[d]));
  }
  return q;
}

// The images n of pair (i, j) within the distance cut, in the host's order
// (n0, n1, n2 lexicographic; for i == j image 0 and the images whose first
// non-zero index is positive), f(n, rab, rab2) for each.  Only the box of
// lattice coordinates that can reach the cut is searched:
// |u_k + n_k| <= rmax |b_k| with u the pair's difference in lattice
// coordinates and b_k the reciprocal vectors, widened above the rounding of
// the single-precision bounds.  Each candidate is tried against the cut in
// single precision with a margin, then exactly.
template <class F>
__device__ __forceinline__ void for_images(const TgParams &P, int i, int j, const PairPos &q,
                                           F &&f) {
  int lo[3], hi[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const float u = q.df[0] * P.cinvf[0][k] + q.df[1] * P.cinvf[1][k] + q.df[2] * P.cinvf[2][k];
    const float w = P.rmaxf * P.hf[k];
    const float m = 1e-4f + 1e-6f * (fabsf(u) + w);
    const float nk = (float)P.nimg[k];
    lo[k] = (int)fminf(fmaxf(ceilf(-u - w - m), -nk), nk + 1.0f);
    hi[k] = (int)fminf(fmaxf(floorf(-u + w + m), -nk - 1.0f), nk);
  }
  const double rmax2 = dmul(P.rmax, P.rmax);
  for (int n0 = lo[0]; n0 <= hi[0]; n0++)
    for (int n1 = lo[1]; n1 <= hi[1]; n1++)
      for (int n2 = lo[2]; n2 <= hi[2]; n2++) {
        const int n[3] = {n0, n1, n2};
        if (i == j) {
          const int lex = n0 != 0 ? n0 : (n1 != 0 ? n1 : n2);
          if (lex < 0)
            continue;
        }
        float rf2 = 0.0f;
#pragma unroll
        for (int d = 0; d < 3; d++) {
          const float x = q.df[d] + (float)n0 * P.cellf[0][d] + (float)n1 * P.cellf[1][d] +
                          (float)n2 * P.cellf[2][d];
          rf2 += x * x;
        }
        const float span = P.rmaxf + fabsf(q.df[0]) + fabsf(q.df[1]) + fabsf(q.df[2]) +
                           fabsf((float)n0) * P.cellnorm[0] + fabsf((float)n1) * P.cellnorm[1] +
                           fabsf((float)n2) * P.cellnorm[2];
        const float lim = P.rmaxf + 1e-5f * span + 1e-6f;
        if (rf2 > lim * lim)
          continue;
        double rab[3];
        const double rab2 = image_rab(P, q.ra, q.rj, n, rab);
        if (rab2 > rmax2)
          continue;
        f(rab, rab2);
      }
}

// one thread per atom pair: number of tasks over its images
__global__ void __launch_bounds__(256) pair_count_kernel(TgParams P, int *__restrict__ cnt) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < P.npairs;
       p += (long long)gridDim.x * blockDim.x) {
    int i, j;
    pair_of(p, P.natoms, i, j);
    const PairPos q = pair_pos(P, i, j);
    const int ki = P.kind[i], kj = P.kind[j];
    int c = 0;
    for_images(P, i, j, q, [&](const double *, double rab2) { c += image_tasks(P, ki, kj, rab2); });
    cnt[p] = c;
  }
}

// ---------------------------------------------------------------- scan --
struct V2 {
  long long a, b;
};
__device__ __forceinline__ V2 operator+(V2 x, V2 y) { return {x.a + y.a, x.b + y.b}; }

__device__ __forceinline__ V2 warp_incl(V2 v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    V2 u;
    u.a = __shfl_up_sync(0xffffffffu, v.a, o);
    u.b = __shfl_up_sync(0xffffffffu, v.b, o);
    if (lane >= o)
      v = v + u;
  }
  return v;
}

// exclusive scan across the CTA of one value per thread; total in *tot
__device__ V2 cta_excl(V2 v, V2 *tot) {
  __shared__ V2 wsum[kScanThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const V2 inc = warp_incl(v);
  if (lane == 31)
    wsum[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    V2 s = lane < kScanThreads / 32 ? wsum[lane] : V2{0, 0};
    s = warp_incl(s);
    if (lane < kScanThreads / 32)
      wsum[lane] = s;
  }
  __syncthreads();
  V2 base = warp > 0 ? wsum[warp - 1] : V2{0, 0};
  *tot = wsum[kScanThreads / 32 - 1];
  __syncthreads();
  V2 e = base + inc;
  e.a -= v.a;
  e.b -= v.b;
  return e;
}

// values scanned: pair tasks and "has tasks"; block sizes
struct PairIn {
  const int *cnt;
  __device__ V2 operator()(long long p) const {
    const int c = cnt[p];
    return {c, c > 0};
  }
};
struct BlockIn {
  const int *size;
  __device__ V2 operator()(long long b) const { return {size[b], 0}; }
};

// per pair with tasks: its block's pair, first task and size
struct PairOut {
  const int *cnt;
  const int *kind;
  const int *nsgf;
  int natoms;
  int *pair_i, *pair_j;
  long long *task0;
  int *size;
  __device__ void operator()(long long p, V2 excl) const {
    if (cnt[p] == 0)
      return;
    int i, j;
    pair_of(p, natoms, i, j);
    const long long b = excl.b;
    pair_i[b] = i;
    pair_j[b] = j;
    task0[b] = excl.a;
    size[b] = nsgf[kind[i]] * nsgf[kind[j]];
  }
};
struct BlockOut {
  int *offsets;
  __device__ void operator()(long long b, V2 excl) const {
    offsets[b] = excl.a <= INT_MAX ? (int)excl.a : -1;
  }
};

template <class In>
__global__ void __launch_bounds__(kScanThreads) scan_tiles(In in, long long n, V2 *partial) {
  const long long t0 = blockIdx.x * (long long)kScanTile;
  V2 s{0, 0};
  for (int k = threadIdx.x; k < kScanTile; k += kScanThreads) {
    const long long idx = t0 + k;
    if (idx < n)
      s = s + in(idx);
  }
  V2 tot;
  cta_excl(s, &tot);
  if (threadIdx.x == 0)
    partial[blockIdx.x] = tot;
}

// one CTA: exclusive scan of the tile totals; grand total at partial[ntiles]
__global__ void __launch_bounds__(kScanThreads) scan_partials(V2 *partial, long long ntiles) {
  V2 carry{0, 0};
  for (long long c0 = 0; c0 < ntiles; c0 += kScanThreads) {
    const long long idx = c0 + threadIdx.x;
    const V2 v = idx < ntiles ? partial[idx] : V2{0, 0};
    V2 tot;
    const V2 e = cta_excl(v, &tot);
    if (idx < ntiles)
      partial[idx] = carry + e;
    carry = carry + tot;
  }
  if (threadIdx.x == 0)
    partial[ntiles] = carry;
}

template <class In, class Out>
__global__ void __launch_bounds__(kScanThreads) scan_apply(In in, Out out, long long n,
                                                           const V2 *partial) {
  const long long t0 = blockIdx.x * (long long)kScanTile + (long long)threadIdx.x * kScanItems;
  V2 v[kScanItems], s{0, 0};
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    v[k] = t0 + k < n ? in(t0 + k) : V2{0, 0};
    s = s + v[k];
  }
  V2 tot;
  V2 e = cta_excl(s, &tot) + partial[blockIdx.x];
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    if (t0 + k < n)
      out(t0 + k, e);
    e = e + v[k];
  }
}

// ------------------------------------------------------------- tasks --
__device__ int grid_level(const TgParams &P, double zetp) {
  int lev = 1;
  const double need = dmul(fabs(zetp), P.rel_cutoff);
  for (int l = 1; l <= P.nlevels; l++)
    if (dadd(P.cutoff[l - 1], 1e-6) >= need)
      lev = l;
  return lev;
}

// one thread per block: the tasks of the block's pair, images in order
__global__ void __launch_bounds__(256)
    fill_tasks_kernel(TgParams P, long long nblocks, const int *__restrict__ pair_i,
                      const int *__restrict__ pair_j, const long long *__restrict__ task0,
                      TgOut o) {
  for (long long b = blockIdx.x * (long long)blockDim.x + threadIdx.x; b < nblocks;
       b += (long long)gridDim.x * blockDim.x) {
    const int i = pair_i[b], j = pair_j[b];
    const int ki = P.kind[i], kj = P.kind[j];
    const PairPos q = pair_pos(P, i, j);
    long long t = task0[b];
    const int si0 = P.set_off[ki], sj0 = P.set_off[kj];
    for_images(P, i, j, q, [&](const double *rab, double rab2) {
      auto write = [&](int is, int js, int ip, int jp, double za, double zb) {
        o.level[t] = grid_level(P, dadd(za, zb));
        o.iatom[t] = i + 1;
        o.jatom[t] = j + 1;
        o.iset[t] = is + 1;
        o.jset[t] = js + 1;
        o.ipgf[t] = ip + 1;
        o.jpgf[t] = jp + 1;
        o.border_mask[t] = 0;
        o.block_num[t] = (int)b + 1;
        o.rab[3 * t] = rab[0];
        o.rab[3 * t + 1] = rab[1];
        o.rab[3 * t + 2] = rab[2];
        t++;
      };
      if (P.screen) {
        radius_screen(P, ki, kj, rab2, [&](int is, int js, int ip, int jp) {
          write(is, js, ip, jp, P.zet[(size_t)(si0 + is) * P.maxpgf + ip],
                P.zet[(size_t)(sj0 + js) * P.maxpgf + jp]);
        });
        return;
      }
      const float rab2f = __double2float_rn(rab2);
      for (int is = 0; is < P.nset[ki]; is++)
        for (int ip = 0; ip < P.npgf[si0 + is]; ip++) {
          const size_t ia = (size_t)(si0 + is) * P.maxpgf + ip;
          const double za = P.zet[ia];
          const float zaf = P.zetf[ia];
          for (int js = 0; js < P.nset[kj]; js++)
            for (int jp = 0; jp < P.npgf[sj0 + js]; jp++) {
              const size_t ib = (size_t)(sj0 + js) * P.maxpgf + jp;
              const double zb = P.zet[ib];
              if (!passes(P, za, zb, zaf, P.zetf[ib], rab2, rab2f))
                continue;
              write(is, js, ip, jp, za, zb);
            }
        }
    });
  }
}

// d exp(-a r^2) r^l, the exponential in single precision
__device__ __forceinline__ double g_eval(double d, double a, double r, int l) {
  const float x = __double2float_rn(dmul(dmul(-a, r), r));
  const double e = (double)__double2float_rn(exp((double)x));
  double pw = 1.0;
  for (int k = 0; k < l; k++)
    pw = dmul(pw, r);
  return dmul(dmul(d, e), pw);
}

__device__ __forceinline__ float log_of(double v) {
  const float f = __double2float_rn(v);
  return (f > 1e-30f && f < 1e30f) ? logf(f) : __double2float_rn(log(v));
}

// g_eval(d, a, r, l) < t: in single precision on the logarithms, ln d - a r^2
// + l ln r against ln t, where the margin decides; else g_eval itself.  Below
// exp(-87) the single-precision exponential is subnormal or zero, so there the
// comparison uses e^-87 as an upper bound and defers to g_eval otherwise.
struct Below {
  double d, a, t;
  int l;
  float af, ld, lt;
  __device__ bool operator()(double r) const {
    const float rf = __double2float_rn(r);
    const float x = -af * rf * rf;
    const float xe = fmaxf(x, -87.0f);
    const float diff = ld + xe + (l ? (float)l * logf(rf) : 0.0f) - lt;
    if (diff < -kMargin)
      return true;
    if (x > -87.0f && diff > kMargin)
      return false;
    return g_eval(d, a, r, l) < t;
  }
};

// smallest radius past which d exp(-a r^2) r^l stays below t (ao_util.F:95-180)
__device__ double exp_radius(int l, double alpha, double threshold, double prefactor,
                             double epsabs, double rlow) {
  const int itermax = 5000;
  const double contract[2] = {(double)0.38f, (double)0.62f};
  const double a = fabs(alpha), t = fabs(threshold);
  double radius = rlow;
  if (prefactor == 0.0)
    return radius;
  double r = fmax(__dsqrt_rn(ddiv(dmul(0.5, (double)l), a)), radius);
  const double d = fabs(prefactor);
  const Below below{d, a, t, l, __double2float_rn(a), log_of(d), log_of(t)};
  if (l != 0 ? below(r) : d < t)
    return radius;
  radius = dadd(dmul(r, 2.0), 1.0);
  int i;
  for (i = 1; i <= itermax; i++) {
    if (below(radius))
      break;
    r = radius;
    radius = dadd(dmul(r, 2.0), 1.0);
  }
  double dr = 0.0;
  for (i = i + 1; i <= itermax; i++) {
    const double rd = dsub(radius, r);
    if (rd < epsabs || rd == dr)
      return radius;
    // the two contraction points of [r, radius), the second only when the
    // first is above
    const double r0 = r;
    const double s0 = dadd(r0, dmul(rd, contract[0]));
    if (below(s0)) {
      radius = s0;
    } else {
      r = s0;
      const double s1 = dadd(r0, dmul(rd, contract[1]));
      if (below(s1))
        radius = s1;
      else
        r = s1;
    }
    dr = rd;
  }
  return radius;
}

// one thread per task: the radius of exp_radius_very_extended (ao_util.F:207-290)
__global__ void __launch_bounds__(128) radius_kernel(TgParams P, long long ntasks, TgOut o) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < ntasks;
       t += (long long)gridDim.x * blockDim.x) {
    const int i = o.iatom[t] - 1, j = o.jatom[t] - 1;
    const int gi = P.set_off[P.kind[i]] + o.iset[t] - 1;
    const int gj = P.set_off[P.kind[j]] + o.jset[t] - 1;
    const double za = P.zet[(size_t)gi * P.maxpgf + o.ipgf[t] - 1];
    const double zb = P.zet[(size_t)gj * P.maxpgf + o.jpgf[t] - 1];
    const double rab[3] = {o.rab[3 * t], o.rab[3 * t + 1], o.rab[3 * t + 2]};
    const double rab2 = dadd(dadd(dmul(rab[0], rab[0]), dmul(rab[1], rab[1])), dmul(rab[2], rab[2]));
    const double zetp = dadd(za, zb), f = ddiv(zb, zetp);
    const double pref = exp(dmul(dmul(-za, f), rab2));
    const double ra[3] = {P.pos[3 * i], P.pos[3 * i + 1], P.pos[3 * i + 2]};
    double rad_a = 0.0, rad_b = 0.0;
#pragma unroll
    for (int d = 0; d < 3; d++) {
      const double rp = dadd(ra[d], dmul(f, rab[d]));
      const double rb = dadd(ra[d], rab[d]);
      const double ea = dsub(ra[d], rp), eb = dsub(rb, rp);
      rad_a = dadd(rad_a, dmul(ea, ea));
      rad_b = dadd(rad_b, dmul(eb, eb));
    }
    rad_a = __dsqrt_rn(rad_a);
    rad_b = __dsqrt_rn(rad_b);
    const int la = P.lmax[gi], lb = P.lmax[gj];
    // the powers rad^i and the binomials of the host's recurrences (there
    // s1 = s1 rad from 1, and bin (n - i) / (i + 1), whose every step is an
    // exact integer, i.e. the binomial coefficients of the table)
    double pa[kTgMaxL + 1], pb[kTgMaxL + 1];
    pa[0] = pb[0] = 1.0;
    for (int k = 1; k <= la; k++)
      pa[k] = dmul(pa[k - 1], rad_a);
    for (int k = 1; k <= lb; k++)
      pb[k] = dmul(pb[k - 1], rad_b);
    double poly[kTgPoly];
    for (int k = 0; k <= la + lb; k++)
      poly[k] = 0.0;
    for (int lxa = 0; lxa <= la; lxa++)
      for (int lxb = 0; lxb <= lb; lxb++) {
        double coef[kTgPoly];
        for (int k = 0; k <= lxa + lxb; k++)
          coef[k] = 0.0;
        for (int ii = 0; ii <= lxa; ii++)
          for (int jj = 0; jj <= lxb; jj++) {
            const int k = lxa + lxb - ii - jj;
            const double bb = dmul(kBinom.v[lxa][ii], kBinom.v[lxb][jj]);
            coef[k] = dadd(coef[k], dmul(dmul(bb, pa[ii]), pb[jj]));
          }
        for (int k = 0; k <= lxa + lxb; k++)
          poly[k] = fmax(poly[k], coef[k]);
      }
    double radius = 0.0;
    for (int k = 0; k <= la + lb; k++)
      radius = fmax(radius, exp_radius(k, zetp, P.eps, dmul(poly[k], pref), 1.0e-2, radius));
    o.radius[t] = radius;
  }
}

// ------------------------------------------------------------ packing --
// one warp per block: dst[dst_off + k] = src[src_off + k]
__global__ void __launch_bounds__(256)
    pack_kernel(long long n, const long long *__restrict__ src_off,
                const int *__restrict__ dst_off, const int *__restrict__ size,
                const double *__restrict__ src, double *__restrict__ dst) {
  const int lane = threadIdx.x & 31;
  const long long w0 = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long b = w0; b < n; b += nw) {
    const double *s = src + src_off[b];
    double *d = dst + dst_off[b];
    const int m = size[b];
    int k = lane;
    for (; k + 96 < m; k += 128) {
      const double v0 = __ldg(s + k), v1 = __ldg(s + k + 32), v2 = __ldg(s + k + 64),
                   v3 = __ldg(s + k + 96);
      d[k] = v0;
      d[k + 32] = v1;
      d[k + 64] = v2;
      d[k + 96] = v3;
    }
    for (; k < m; k += 32)
      d[k] = __ldg(s + k);
  }
}

// one warp per block: blocks[blk_off + k] += buffer[buf_off + k]
__global__ void __launch_bounds__(256)
    unpack_kernel(long long n, const int *__restrict__ buf_off,
                  const long long *__restrict__ blk_off, const int *__restrict__ size,
                  const double *__restrict__ buf, double *__restrict__ blocks) {
  const int lane = threadIdx.x & 31;
  const long long w0 = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long b = w0; b < n; b += nw) {
    const double *s = buf + buf_off[b];
    double *d = blocks + blk_off[b];
    const int m = size[b];
    int k = lane;
    for (; k + 96 < m; k += 128) {
      const double v0 = __ldg(s + k), v1 = __ldg(s + k + 32), v2 = __ldg(s + k + 64),
                   v3 = __ldg(s + k + 96);
      const double u0 = d[k], u1 = d[k + 32], u2 = d[k + 64], u3 = d[k + 96];
      d[k] = u0 + v0;
      d[k + 32] = u1 + v1;
      d[k + 64] = u2 + v2;
      d[k + 96] = u3 + v3;
    }
    for (; k < m; k += 32)
      d[k] = d[k] + __ldg(s + k);
  }
}

// one thread per query: binary search of (row, col) in keys sorted by row
// then column; -1 and a count of misses when absent
__global__ void find_blocks_kernel(long long nkeys, const int *__restrict__ key_row,
                                   const int *__restrict__ key_col,
                                   const long long *__restrict__ key_off, long long nq,
                                   const int *__restrict__ row, const int *__restrict__ col,
                                   long long *__restrict__ off, unsigned long long *missing) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < nq;
       q += (long long)gridDim.x * blockDim.x) {
    const long long want = ((long long)row[q] << 32) | (unsigned)col[q];
    long long lo = 0, hi = nkeys;
    while (lo < hi) {
      const long long mid = (lo + hi) >> 1;
      const long long k = ((long long)key_row[mid] << 32) | (unsigned)key_col[mid];
      if (k < want)
        lo = mid + 1;
      else
        hi = mid;
    }
    if (lo < nkeys && key_row[lo] == row[q] && key_col[lo] == col[q]) {
      off[q] = key_off[lo];
    } else {
      off[q] = -1;
      atomicAdd(missing, 1ull);
    }
  }
}

int warp_grid(long long nwarps) {
  const long long cap = 152LL * 16;
  const long long blocks = (nwarps + 7) / 8;
  return (int)std::max(1LL, std::min(blocks, cap));
}

int thread_grid(long long n) {
  const long long cap = 152LL * 32;
  return (int)std::max(1LL, std::min((n + 255) / 256, cap));
}

template <class T> void grow(T *&p, size_t &cap, size_t n) {
  if (n <= cap)
    return;
  if (p)
    CKT(cudaFree(p));
  const size_t c = std::max(n, cap + cap / 2);
  CKT(cudaMalloc((void **)&p, c * sizeof(T)));
  cap = c;
}

} // namespace

struct TaskGenerator {
  TgParams P{};
  int nkinds = 0;
  std::vector<int> h_kind1; // atom kinds, 1-based
  std::vector<double> h_pos;
  // device basis and positions
  int *d_kind = nullptr, *d_set_off = nullptr, *d_nset = nullptr, *d_nsgf = nullptr;
  int *d_lmax = nullptr, *d_npgf = nullptr;
  double *d_zet = nullptr, *d_pos = nullptr;
  float *d_zetf = nullptr;
  double *d_rpgf = nullptr, *d_set_radius = nullptr, *d_kind_radius = nullptr;
  int nsets = 0;
  // work
  int *d_cnt = nullptr;
  size_t cap_cnt = 0;
  V2 *d_partial = nullptr;
  size_t cap_partial = 0;
  int *d_pair_i = nullptr, *d_pair_j = nullptr, *d_size = nullptr;
  long long *d_task0 = nullptr;
  size_t cap_blk = 0, cap_blk2 = 0, cap_blk3 = 0, cap_blk4 = 0;
  // outputs
  int *d_i32[9] = {};
  size_t cap_i32[9] = {};
  double *d_radius = nullptr, *d_rab = nullptr;
  size_t cap_radius = 0, cap_rab = 0;
  int *d_block_offsets = nullptr;
  size_t cap_boff = 0;
  V2 *h_tot = nullptr; // pinned
  int ntasks = 0, nblocks = 0;
  long long buffer_size = 0;
  bool have = false;
  // host copies for task-list creation
  std::vector<int> h_i32[9];
  std::vector<double> h_radius, h_rab;
  std::vector<int> h_block_offsets;

  TgOut out() {
    TgOut o;
    o.level = d_i32[0];
    o.iatom = d_i32[1];
    o.jatom = d_i32[2];
    o.iset = d_i32[3];
    o.jset = d_i32[4];
    o.ipgf = d_i32[5];
    o.jpgf = d_i32[6];
    o.border_mask = d_i32[7];
    o.block_num = d_i32[8];
    o.radius = d_radius;
    o.rab = d_rab;
    o.block_offsets = d_block_offsets;
    return o;
  }
};

template <class In, class Out>
static V2 run_scan(TaskGenerator *g, In in, Out out, long long n, cudaStream_t s) {
  const long long ntiles = std::max(1LL, (n + kScanTile - 1) / kScanTile);
  grow(g->d_partial, g->cap_partial, (size_t)ntiles + 1);
  scan_tiles<<<(unsigned)ntiles, kScanThreads, 0, s>>>(in, n, g->d_partial);
  scan_partials<<<1, kScanThreads, 0, s>>>(g->d_partial, ntiles);
  scan_apply<<<(unsigned)ntiles, kScanThreads, 0, s>>>(in, out, n, g->d_partial);
  count_launch(3);
  CKT(cudaGetLastError());
  CKT(cudaMemcpyAsync(g->h_tot, g->d_partial + ntiles, sizeof(V2), cudaMemcpyDeviceToHost, s));
  CKT(cudaStreamSynchronize(s));
  return *g->h_tot;
}

} // namespace gb300

using gb300::TaskGenerator;

GB300_API void grid_gb300_taskgen_create(
    const int natoms, const int nkinds, const int *atom_kinds, const int *nset,
    const int *nsgf, const int *set_lmax, const int *set_npgf, const int maxpgf,
    const double *zet, const double *cell, const int *nimages, const double rmax,
    const double eps, const int nlevels, const double *cutoff, const double rel_cutoff,
    grid_gb300_task_generator **generator) {
  using namespace gb300;
  if (!generator)
    tg_fail("null generator handle", 0);
  if (natoms < 1 || nkinds < 1 || maxpgf < 1 || nlevels < 1 || nlevels > kTgMaxLevels)
    tg_fail("invalid sizes (natoms, nkinds, maxpgf, nlevels)", nlevels);
  if (!(eps > 0.0) || !(rmax >= 0.0) || !(rel_cutoff > 0.0))
    tg_fail("eps and rel_cutoff must be positive, rmax not negative", 0);
  for (int d = 0; d < 3; d++)
    if (nimages[d] < 0 || nimages[d] > 64)
      tg_fail("image range outside 0..64", nimages[d]);
  std::vector<int> kind0(natoms), set_off(nkinds);
  int nsets = 0;
  for (int k = 0; k < nkinds; k++) {
    if (nset[k] < 0 || nsgf[k] < 0)
      tg_fail("negative set or function count", k);
    set_off[k] = nsets;
    nsets += nset[k];
  }
  for (int a = 0; a < natoms; a++) {
    if (atom_kinds[a] < 1 || atom_kinds[a] > nkinds)
      tg_fail("atom kind out of range", a);
    kind0[a] = atom_kinds[a] - 1;
  }
  for (int s = 0; s < nsets; s++) {
    if (set_lmax[s] < 0 || set_lmax[s] > kTgMaxL)
      tg_fail("set lmax outside 0..12", set_lmax[s]);
    if (set_npgf[s] < 0 || set_npgf[s] > maxpgf)
      tg_fail("set primitive count outside 0..maxpgf", set_npgf[s]);
  }
  auto *g = new TaskGenerator();
  g->nkinds = nkinds;
  g->nsets = nsets;
  g->h_kind1.assign(atom_kinds, atom_kinds + natoms);
  TgParams &P = g->P;
  P.natoms = natoms;
  P.npairs = (long long)natoms * (natoms + 1) / 2;
  for (int d = 0; d < 3; d++)
    P.nimg[d] = nimages[d];
  for (int a = 0; a < 3; a++)
    for (int b = 0; b < 3; b++)
      P.cell[a][b] = cell[3 * a + b];
  P.rmax = rmax;
  P.eps = eps;
  P.rel_cutoff = rel_cutoff;
  P.nlevels = nlevels;
  for (int l = 0; l < nlevels; l++)
    P.cutoff[l] = cutoff[l];
  P.maxpgf = maxpgf;
  for (int a = 0; a < 3; a++) {
    double nrm = 0.0;
    for (int b = 0; b < 3; b++) {
      P.cellf[a][b] = (float)cell[3 * a + b];
      nrm += cell[3 * a + b] * cell[3 * a + b];
    }
    P.cellnorm[a] = (float)std::sqrt(nrm);
  }
  {
    // inverse of the cell (rows: cell vectors), for the image boxes
    const double *m = cell;
    const double det = m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) +
                       m[2] * (m[3] * m[7] - m[4] * m[6]);
    if (!(std::fabs(det) > 0.0))
      tg_fail("singular cell", 0);
    double inv[3][3];
    for (int r = 0; r < 3; r++)
      for (int c = 0; c < 3; c++) {
        // cofactor of (c, r) over det
        const int r1 = (c + 1) % 3, r2 = (c + 2) % 3, c1 = (r + 1) % 3, c2 = (r + 2) % 3;
        inv[r][c] = (m[3 * r1 + c1] * m[3 * r2 + c2] - m[3 * r1 + c2] * m[3 * r2 + c1]) / det;
      }
    for (int k = 0; k < 3; k++) {
      double h = 0.0;
      for (int r = 0; r < 3; r++) {
        P.cinvf[r][k] = (float)inv[r][k];
        h += inv[r][k] * inv[r][k];
      }
      P.hf[k] = (float)std::sqrt(h);
    }
  }
  P.rmaxf = (float)rmax;
  P.leps = (float)std::log(eps);
  std::vector<float> zetf((size_t)nsets * maxpgf);
  for (size_t q = 0; q < zetf.size(); q++)
    zetf[q] = (float)zet[q];
  auto up = [](auto *&dst, const auto *src, size_t n) {
    CKT(cudaMalloc((void **)&dst, std::max<size_t>(n, 1) * sizeof(*src)));
    if (n)
      CKT(cudaMemcpy(dst, src, n * sizeof(*src), cudaMemcpyHostToDevice));
  };
  up(g->d_kind, kind0.data(), natoms);
  up(g->d_set_off, set_off.data(), nkinds);
  up(g->d_nset, nset, nkinds);
  up(g->d_nsgf, nsgf, nkinds);
  up(g->d_lmax, set_lmax, nsets);
  up(g->d_npgf, set_npgf, nsets);
  up(g->d_zet, zet, (size_t)nsets * maxpgf);
  up(g->d_zetf, zetf.data(), zetf.size());
  CKT(cudaMalloc((void **)&g->d_pos, sizeof(double) * 3 * natoms));
  CKT(cudaMallocHost((void **)&g->h_tot, sizeof(V2)));
  P.pos = g->d_pos;
  P.kind = g->d_kind;
  P.set_off = g->d_set_off;
  P.nset = g->d_nset;
  P.nsgf = g->d_nsgf;
  P.lmax = g->d_lmax;
  P.npgf = g->d_npgf;
  P.zet = g->d_zet;
  P.zetf = g->d_zetf;
  *generator = g;
}

GB300_API void grid_gb300_taskgen_set_radius_screen(grid_gb300_task_generator *generator,
                                                   const double *pgf_radius,
                                                   const double *set_radius,
                                                   const double *kind_radius) {
  using namespace gb300;
  auto *g = (TaskGenerator *)generator;
  if (!g || !pgf_radius || !set_radius || !kind_radius)
    tg_fail("null generator or radii", 0);
  const size_t npr = (size_t)g->nsets * g->P.maxpgf;
  for (size_t q = 0; q < npr; q++)
    if (!(pgf_radius[q] >= 0.0))
      tg_fail("negative or invalid primitive radius", (int)q);
  auto up = [](double *&dst, const double *src, size_t n) {
    if (!dst)
      CKT(cudaMalloc((void **)&dst, std::max<size_t>(n, 1) * sizeof(double)));
    if (n)
      CKT(cudaMemcpy(dst, src, n * sizeof(double), cudaMemcpyHostToDevice));
  };
  up(g->d_rpgf, pgf_radius, npr);
  up(g->d_set_radius, set_radius, (size_t)g->nsets);
  up(g->d_kind_radius, kind_radius, (size_t)g->nkinds);
  g->P.rpgf = g->d_rpgf;
  g->P.set_radius = g->d_set_radius;
  g->P.kind_radius = g->d_kind_radius;
  g->P.screen = 1;
}

GB300_API void grid_gb300_taskgen_free(grid_gb300_task_generator *generator) {
  using namespace gb300;
  auto *g = (TaskGenerator *)generator;
  if (!g)
    return;
  void *d[] = {g->d_kind, g->d_set_off, g->d_nset, g->d_nsgf, g->d_lmax, g->d_npgf,
               g->d_zet, g->d_zetf, g->d_rpgf, g->d_set_radius, g->d_kind_radius, g->d_pos,
               g->d_cnt, g->d_partial, g->d_pair_i, g->d_pair_j,
               g->d_size, g->d_task0, g->d_radius, g->d_rab, g->d_block_offsets};
  for (void *p : d)
    if (p)
      cudaFree(p);
  for (int q = 0; q < 9; q++)
    if (g->d_i32[q])
      cudaFree(g->d_i32[q]);
  if (g->h_tot)
    cudaFreeHost(g->h_tot);
  delete g;
}

GB300_API void grid_gb300_taskgen_run(grid_gb300_task_generator *generator,
                                      const double *atom_positions, const int on_device,
                                      void *stream, int *ntasks, int *nblocks,
                                      long long *buffer_size) {
  using namespace gb300;
  auto *g = (TaskGenerator *)generator;
  if (!g || !atom_positions)
    tg_fail("null generator or positions", 0);
  cudaStream_t s = (cudaStream_t)stream;
  TgParams &P = g->P;
  const size_t pos_bytes = sizeof(double) * 3 * P.natoms;
  if (on_device) {
    CKT(cudaMemcpyAsync(g->d_pos, atom_positions, pos_bytes, cudaMemcpyDeviceToDevice, s));
    g->h_pos.clear();
  } else {
    g->h_pos.assign(atom_positions, atom_positions + 3 * P.natoms);
    CKT(cudaMemcpyAsync(g->d_pos, g->h_pos.data(), pos_bytes, cudaMemcpyHostToDevice, s));
  }
  // 1. tasks per atom pair
  grow(g->d_cnt, g->cap_cnt, (size_t)P.npairs);
  pair_count_kernel<<<thread_grid(P.npairs), 256, 0, s>>>(P, g->d_cnt);
  count_launch();
  CKT(cudaGetLastError());
  // 2. task offsets and block numbers of the pairs with tasks
  grow(g->d_pair_i, g->cap_blk, (size_t)P.npairs);
  grow(g->d_pair_j, g->cap_blk2, (size_t)P.npairs);
  grow(g->d_task0, g->cap_blk3, (size_t)P.npairs);
  grow(g->d_size, g->cap_blk4, (size_t)P.npairs);
  PairOut po{g->d_cnt, g->d_kind, g->d_nsgf, P.natoms, g->d_pair_i, g->d_pair_j, g->d_task0,
             g->d_size};
  const V2 tot = run_scan(g, PairIn{g->d_cnt}, po, P.npairs, s);
  if (tot.a > INT_MAX)
    tg_fail("more than 2^31 - 1 tasks", 0);
  g->ntasks = (int)tot.a;
  g->nblocks = (int)tot.b;
  // 3. block offsets
  grow(g->d_block_offsets, g->cap_boff, (size_t)g->nblocks);
  const V2 btot = run_scan(g, BlockIn{g->d_size}, BlockOut{g->d_block_offsets}, g->nblocks, s);
  if (btot.a > INT_MAX)
    tg_fail("block buffer exceeds int offsets", 0);
  g->buffer_size = btot.a;
  // 4. tasks, then radii
  for (int q = 0; q < 9; q++)
    grow(g->d_i32[q], g->cap_i32[q], (size_t)g->ntasks);
  grow(g->d_radius, g->cap_radius, (size_t)g->ntasks);
  grow(g->d_rab, g->cap_rab, (size_t)g->ntasks * 3);
  const TgOut o = g->out();
  if (g->nblocks > 0) {
    fill_tasks_kernel<<<thread_grid(g->nblocks), 256, 0, s>>>(P, g->nblocks, g->d_pair_i,
                                                            g->d_pair_j, g->d_task0, o);
    count_launch();
  }
  if (g->ntasks > 0) {
    const int blocks = (int)std::min<long long>((g->ntasks + 127) / 128, 152LL * 64);
    radius_kernel<<<blocks, 128, 0, s>>>(P, g->ntasks, o);
    count_launch();
  }
  CKT(cudaGetLastError());
  CKT(cudaStreamSynchronize(s));
  g->have = true;
  if (ntasks)
    *ntasks = g->ntasks;
  if (nblocks)
    *nblocks = g->nblocks;
  if (buffer_size)
    *buffer_size = g->buffer_size;
}

GB300_API void grid_gb300_taskgen_arrays(const grid_gb300_task_generator *generator,
                                         int **level, int **iatom, int **jatom, int **iset,
                                         int **jset, int **ipgf, int **jpgf, int **border_mask,
                                         int **block_num, double **radius, double **rab,
                                         int **block_offsets) {
  using namespace gb300;
  auto *g = (TaskGenerator *)generator;
  if (!g || !g->have)
    tg_fail("no generated task list", 0);
  int **dst[9] = {level, iatom, jatom, iset, jset, ipgf, jpgf, border_mask, block_num};
  for (int q = 0; q < 9; q++)
    if (dst[q])
      *dst[q] = g->d_i32[q];
  if (radius)
    *radius = g->d_radius;
  if (rab)
    *rab = g->d_rab;
  if (block_offsets)
    *block_offsets = g->d_block_offsets;
}

GB300_API void grid_gb300_taskgen_copy(const grid_gb300_task_generator *generator, int *level,
                                       int *iatom, int *jatom, int *iset, int *jset, int *ipgf,
                                       int *jpgf, int *border_mask, int *block_num,
                                       double *radius, double *rab, int *block_offsets) {
  using namespace gb300;
  auto *g = (TaskGenerator *)generator;
  if (!g || !g->have)
    tg_fail("no generated task list", 0);
  int *dst[9] = {level, iatom, jatom, iset, jset, ipgf, jpgf, border_mask, block_num};
  const size_t nt = (size_t)g->ntasks;
  for (int q = 0; q < 9; q++)
    if (dst[q] && nt)
      CKT(cudaMemcpy(dst[q], g->d_i32[q], nt * sizeof(int), cudaMemcpyDeviceToHost));
  if (radius && nt)
    CKT(cudaMemcpy(radius, g->d_radius, nt * sizeof(double), cudaMemcpyDeviceToHost));
  if (rab && nt)
    CKT(cudaMemcpy(rab, g->d_rab, 3 * nt * sizeof(double), cudaMemcpyDeviceToHost));
  if (block_offsets && g->nblocks)
    CKT(cudaMemcpy(block_offsets, g->d_block_offsets, (size_t)g->nblocks * sizeof(int),
                   cudaMemcpyDeviceToHost));
}

GB300_API void grid_gb300_taskgen_create_task_list(
    grid_gb300_task_generator *generator, const bool orthorhombic, const int nlevels,
    const grid_basis_set **basis_sets, const int *npts_global, const int *npts_local,
    const int *shift_local, const int *border_width, const double *dh, const double *dh_inv,
    grid_gb300_task_list **task_list) {
  using namespace gb300;
  auto *g = (TaskGenerator *)generator;
  if (!g || !g->have)
    tg_fail("no generated task list", 0);
  if (nlevels != g->P.nlevels)
    tg_fail("level count differs from the generator's", nlevels);
  if (g->h_pos.empty()) {
    g->h_pos.resize(3 * (size_t)g->P.natoms);
    CKT(cudaMemcpy(g->h_pos.data(), g->d_pos, g->h_pos.size() * sizeof(double),
                   cudaMemcpyDeviceToHost));
  }
  const size_t nt = (size_t)g->ntasks;
  for (int q = 0; q < 9; q++)
    g->h_i32[q].resize(std::max<size_t>(nt, 1));
  g->h_radius.resize(std::max<size_t>(nt, 1));
  g->h_rab.resize(std::max<size_t>(3 * nt, 1));
  g->h_block_offsets.resize(std::max(g->nblocks, 1));
  grid_gb300_taskgen_copy(g, g->h_i32[0].data(), g->h_i32[1].data(), g->h_i32[2].data(),
                          g->h_i32[3].data(), g->h_i32[4].data(), g->h_i32[5].data(),
                          g->h_i32[6].data(), g->h_i32[7].data(), g->h_i32[8].data(),
                          g->h_radius.data(), g->h_rab.data(), g->h_block_offsets.data());
  grid_gb300_create_task_list(
      orthorhombic, g->ntasks, nlevels, g->P.natoms, g->nkinds, g->nblocks,
      g->h_block_offsets.data(), g->h_pos.data(), g->h_kind1.data(), basis_sets,
      g->h_i32[0].data(), g->h_i32[1].data(), g->h_i32[2].data(), g->h_i32[3].data(),
      g->h_i32[4].data(), g->h_i32[5].data(), g->h_i32[6].data(), g->h_i32[7].data(),
      g->h_i32[8].data(), g->h_radius.data(), g->h_rab.data(), npts_global, npts_local,
      shift_local, border_width, dh, dh_inv, task_list);
}

GB300_API void grid_gb300_pack_blocks(const long long nblocks, const long long *src_offsets,
                                      const int *dst_offsets, const int *sizes,
                                      const double *src, double *dst, void *stream) {
  using namespace gb300;
  if (nblocks <= 0)
    return;
  pack_kernel<<<warp_grid(nblocks), 256, 0, (cudaStream_t)stream>>>(
      nblocks, src_offsets, dst_offsets, sizes, src, dst);
  count_launch();
  CKT(cudaGetLastError());
}

GB300_API void grid_gb300_unpack_blocks(const long long nblocks, const int *buffer_offsets,
                                        const long long *block_offsets, const int *sizes,
                                        const double *buffer, double *blocks, void *stream) {
  using namespace gb300;
  if (nblocks <= 0)
    return;
  unpack_kernel<<<warp_grid(nblocks), 256, 0, (cudaStream_t)stream>>>(
      nblocks, buffer_offsets, block_offsets, sizes, buffer, blocks);
  count_launch();
  CKT(cudaGetLastError());
}

GB300_API long long grid_gb300_find_blocks(const long long nkeys, const int *key_rows,
                                           const int *key_cols, const long long *key_offsets,
                                           const long long nquery, const int *rows,
                                           const int *cols, long long *offsets, void *stream) {
  using namespace gb300;
  if (nquery <= 0)
    return 0;
  cudaStream_t s = (cudaStream_t)stream;
  unsigned long long *d_miss = nullptr, h_miss = 0;
  CKT(cudaMallocAsync((void **)&d_miss, sizeof(unsigned long long), s));
  CKT(cudaMemsetAsync(d_miss, 0, sizeof(unsigned long long), s));
  const int blocks = (int)std::min<long long>((nquery + 255) / 256, 152LL * 16);
  find_blocks_kernel<<<blocks, 256, 0, s>>>(nkeys, key_rows, key_cols, key_offsets, nquery, rows,
                                            cols, offsets, d_miss);
  count_launch();
  CKT(cudaGetLastError());
  CKT(cudaMemcpyAsync(&h_miss, d_miss, sizeof(h_miss), cudaMemcpyDeviceToHost, s));
  CKT(cudaFreeAsync(d_miss, s));
  CKT(cudaStreamSynchronize(s));
  return (long long)h_miss;
}
