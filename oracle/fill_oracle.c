/*
 * fill_oracle.c -- CPU restatement of the reference's ghost fill.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle the CUDA engine is checked
 * against and the CPU baseline bench.py times; nothing in the product calls
 * it.  Parity is pinned by the reference's own known-answer and property
 * tests restated in tests/ (exact weights, polynomial exactness, every ghost
 * written once, periodic = tiling bit for bit, interiors untouched, parity
 * at reflecting faces, outflow = nearest owned point).  The reference itself
 * (Julia) cannot run here, and it stores no golden vectors.
 *
 * What it restates, over a schedule already flattened into the
 * tam_schedule_desc arrays (include/treeamr_cuda.h):
 *   - stencil_sum            src/ghosts.jl:75-118  (m_1 innermost, weight
 *                            product ((w_1*w_2)*w_3), acc from +0, no FMA),
 *                            in both of its forms (src/ghosts.jl:28-56): the
 *                            CPU's, where a dimension whose weight column has
 *                            a single nonzero weight (src/schedule.jl:83-86)
 *                            takes that one tap, and the device's full sum
 *   - copy_load              src/ghosts.jl:127-128 (+0 + x)
 *   - scaled                 src/ghosts.jl:369-370 (x*f + 0)
 *   - transfer_kernel!       src/ghosts.jl:372-402
 *   - run_phase! (CPU form)  src/ghosts.jl:572-593: the owned blocks split
 *                            into contiguous chunks, one per thread
 *                            (src/threading.jl:50-70 equalsplit), each thread
 *                            running its share of every group of the stage
 *   - exchange_ghosts!       src/ghosts.jl:1099-1160: stages in tag order
 *   - RotatedSource          src/ghosts.jl:183-244: a turned group's source
 *                            read through its axis map and variable table
 *   - bounded_sum,           src/ghosts.jl:291-361: the bounded operators'
 *     bracket_clamp_sum      kernels, with Julia's min and max
 *   - the adjoint (transpose) of the same linear map, stage by stage in
 *     reverse, in scatter form: a new capability with no reference
 *     counterpart, so its oracle is the linear algebra of the forward.
 *
 * Build: see oracle/build.py.  Compiled with -ffp-contract=off so that no
 * multiply-add is fused on any host architecture.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "treeamr_cuda.h"

/* contiguous chunk c of n blocks split k ways (src/threading.jl:58-70) */
static void equalsplit(int64_t n, int k, int c, int64_t *lo, int64_t *hi) {
  int64_t q = n / k, r = n % k;
  *lo = c * q + (c < r ? c : r);
  *hi = *lo + q + (c < r ? 1 : 0);
}

/* first index in [lo, hi) of the non-decreasing list with list[i] >= x */
static int64_t lower_bound(const int32_t *list, int64_t lo, int64_t hi, int64_t x) {
  while (lo < hi) {
    int64_t mid = lo + (hi - lo) / 2;
    if (list[mid] < x)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo;
}

/* Julia's min and max of two floats (NaN-propagating, -0 below +0), which the
 * bounded operators' extremes follow (src/ghosts.jl:291-361), and minmod and
 * the monotonized central slope (src/ghosts.jl:291-292). */
#define DEFINE_BOUNDED_HELPERS(T, SUFFIX, ABS)                                                  \
  static inline T jmin_##SUFFIX(T x, T y) {                                                    \
    const int c = (y < x) || (signbit(y) && !signbit(x));                                       \
    return c ? (isnan(x) ? x : y) : (isnan(y) ? y : x);                                         \
  }                                                                                             \
  static inline T jmax_##SUFFIX(T x, T y) {                                                    \
    const int c = (y > x) || (!signbit(y) && signbit(x));                                       \
    return c ? (isnan(x) ? x : y) : (isnan(y) ? y : x);                                         \
  }                                                                                             \
  static inline T minmod_##SUFFIX(T a, T b) {                                                  \
    return (a > 0 && b > 0) ? jmin_##SUFFIX(a, b)                                               \
           : (a < 0 && b < 0) ? jmax_##SUFFIX(a, b) : (T)0;                                     \
  }                                                                                             \
  static inline T mc_##SUFFIX(T a, T b) {                                                      \
    return minmod_##SUFFIX((T)2 * a, minmod_##SUFFIX((T)2 * b, (a + b) / (T)2));                \
  }                                                                                             \
  static inline T abs_##SUFFIX(T x) { return ABS(x); }

DEFINE_BOUNDED_HELPERS(double, f64, fabs)
DEFINE_BOUNDED_HELPERS(float, f32, fabsf)

#define DEFINE_ORACLE(T, SUFFIX)                                                                \
  static void run_transfers_##SUFFIX(const tam_schedule_desc *d, const tam_group *g,            \
                                     int64_t t0, int64_t t1, T *work, const T *alt,            \
                                     int32_t nvars, const T *factors, const int32_t *rotvars,  \
                                     int one_tap) {                                             \
    const int D = d->ndim;                                                                      \
    int n[3] = {1, 1, 1}, o[3] = {1, 1, 1}, tf[3] = {0, 0, 0};                                  \
    int64_t S[3] = {1, 1, 1};                                                                   \
    int unit = 1;                                                                               \
    for (int k = 0; k < D; ++k) {                                                               \
      n[k] = g->stencil[k].ntarget;                                                             \
      o[k] = g->stencil[k].order;                                                               \
      tf[k] = g->stencil[k].targetfirst - 1;                                                    \
      S[k] = d->stored[k];                                                                      \
      unit = unit && g->stencil[k].unit;                                                        \
    }                                                                                           \
    const T *W = (const T *)d->weights;                                                         \
    const int64_t s2 = S[0], s3 = S[0] * S[1], vs = S[0] * S[1] * S[2];                         \
    const int64_t bs = vs * nvars;                                                              \
    /* the source's strides per virtual dimension: the identity, or a turned  \
       group's axis map (RotatedSource, src/ghosts.jl:183-244) */              \
    /* the real array's extent along e is S[perm[e]]: the set's own, or an    \
       odd orientation's partner with the seam's dimensions swapped */        \
    int64_t vst[3] = {1, s2, s3}, c0 = 0;                                                       \
    const T *from = work;                                                                       \
    if (g->orientation) {                                                                       \
      int64_t R[3] = {1, 1, 1};                                                                 \
      for (int e = 0; e < D; ++e) R[e] = S[(g->axes >> (2 * e)) & 3];                          \
      const int64_t rst[3] = {1, R[0], R[0] * R[1]};                                            \
      for (int e = 0; e < D; ++e) {                                                             \
        const int p = (g->axes >> (2 * e)) & 3, f = (g->axes >> (8 + e)) & 1;                  \
        vst[p] = f ? -rst[e] : rst[e];                                                          \
        if (f) c0 += rst[e] * (R[e] - 1);                                                       \
      }                                                                                         \
      if (g->orientation & 1) from = alt;                                                       \
    }                                                                                           \
    for (int64_t t = t0; t < t1; ++t) {                                                         \
      const int64_t tb = d->targetblocks[g->first + t] - 1;                                     \
      const int64_t sb = d->sourceblocks[g->first + t] - 1;                                     \
      for (int v = 0; v < nvars; ++v)                                                           \
        for (int i3 = 0; i3 < n[2]; ++i3)                                                       \
          for (int i2 = 0; i2 < n[1]; ++i2)                                                     \
            for (int i1 = 0; i1 < n[0]; ++i1) {                                                 \
              int idx[3] = {i1, i2, i3};                                                        \
              int64_t base[3] = {0, 0, 0};                                                      \
              const T *wc[3] = {0, 0, 0};                                                       \
              int lo[3] = {0, 0, 0}, hi[3] = {1, 1, 1};                                         \
              for (int k = 0; k < D; ++k) {                                                     \
                base[k] = d->srcstart[g->stencil[k].srcstart + idx[k]] - 1;                     \
                wc[k] = W + g->stencil[k].weights + (int64_t)o[k] * idx[k];                     \
                hi[k] = o[k];                                                                   \
                int nonzero = 0, row = 0;                                                       \
                for (int m = 0; m < o[k]; ++m)                                                  \
                  if (wc[k][m] != (T)0) {                                                       \
                    ++nonzero;                                                                  \
                    row = m;                                                                    \
                  }                                                                             \
                if (one_tap && nonzero == 1) {                                                  \
                  lo[k] = row;                                                                  \
                  hi[k] = row + 1;                                                              \
                }                                                                               \
              }                                                                                 \
              const int sv = g->orientation ? rotvars[v + (int64_t)nvars * g->orientation] - 1  \
                                            : v;                                                \
              const T *src = from + sb * bs + sv * vs + c0 + base[0] * vst[0] +                 \
                             base[1] * vst[1] + base[2] * vst[2];                               \
              T acc = (T)0;                                                                     \
              if (g->bounded == 1) {                                                            \
                /* bounded_sum (src/ghosts.jl:296-310): the parent at the      \
                   window's middle row and its face neighbours */              \
                const int64_t *st = vst;                                                        \
                int64_t o0 = 0;                                                                 \
                for (int k = 0; k < D; ++k) o0 += st[k];                                        \
                const T u = src[o0];                                                            \
                T lov[3], hiv[3], sl[3], M = u, m = u, dl = 0, S = 0;                           \
                for (int k = 0; k < D; ++k) {                                                   \
                  lov[k] = src[o0 - st[k]];                                                     \
                  hiv[k] = src[o0 + st[k]];                                                     \
                  sl[k] = mc_##SUFFIX(hiv[k] - u, u - lov[k]);                                  \
                }                                                                               \
                for (int k = 0; k < D; ++k) M = jmax_##SUFFIX(M, lov[k]);                       \
                for (int k = 0; k < D; ++k) M = jmax_##SUFFIX(M, hiv[k]);                       \
                for (int k = 0; k < D; ++k) m = jmin_##SUFFIX(m, lov[k]);                       \
                for (int k = 0; k < D; ++k) m = jmin_##SUFFIX(m, hiv[k]);                       \
                for (int k = D - 1; k >= 0; --k) { /* right folds */                          \
                  const T sg = wc[k][2] > wc[k][0] ? sl[k] : -sl[k];                            \
                  dl = k == D - 1 ? sg : sg + dl;                                               \
                  S = k == D - 1 ? abs_##SUFFIX(sl[k]) : abs_##SUFFIX(sl[k]) + S;               \
                }                                                                               \
                dl = dl / (T)4;                                                                 \
                S = S / (T)4;                                                                   \
                T phi = 1;                                                                      \
                if (S > 0) phi = jmin_##SUFFIX(jmin_##SUFFIX((T)1, (M - u) / S), (u - m) / S);  \
                acc = (u + phi * dl) + (T)0 * (M - m);                                          \
              } else if (g->bounded == 2) {                                                     \
                /* bracket_clamp_sum (src/ghosts.jl:323-361): the full sum     \
                   clamped into the points of nonzero linear weight */         \
                int p[3] = {1, 1, 1};                                                           \
                for (int k = 0; k < D; ++k) p[k] = o[k] / 2;                                    \
                T blo = (T)INFINITY, bhi = -(T)INFINITY;                                        \
                for (int m3 = 0; m3 < p[2]; ++m3)                                               \
                  for (int m2 = 0; m2 < p[1]; ++m2)                                             \
                    for (int m1 = 0; m1 < p[0]; ++m1) {                                         \
                      T wp = wc[0][m1];                                                         \
                      if (D >= 2) wp = wp * wc[1][m2];                                          \
                      if (D >= 3) wp = wp * wc[2][m3];                                          \
                      const T u = src[m1 * vst[0] + m2 * vst[1] + m3 * vst[2]];                 \
                      T term = wp * u;                                                          \
                      acc = acc + term;                                                         \
                      const int in = wc[0][p[0] + m1] != (T)0 &&                                \
                                     (D < 2 || wc[1][p[1] + m2] != (T)0) &&                     \
                                     (D < 3 || wc[2][p[2] + m3] != (T)0);                       \
                      if (in) {                                                                 \
                        blo = jmin_##SUFFIX(blo, u);                                            \
                        bhi = jmax_##SUFFIX(bhi, u);                                            \
                      }                                                                         \
                    }                                                                           \
                const T cl = acc > bhi ? bhi : acc < blo ? blo : acc;                           \
                acc = cl + (T)0 * (bhi - blo);                                                  \
              } else if (unit) {                                                                \
                acc = (T)0 + src[0];                                                            \
              } else {                                                                          \
                for (int m3 = lo[2]; m3 < hi[2]; ++m3)                                          \
                  for (int m2 = lo[1]; m2 < hi[1]; ++m2)                                        \
                    for (int m1 = lo[0]; m1 < hi[0]; ++m1) {                                    \
                      T wp = wc[0][m1];                                                         \
                      if (D >= 2) wp = wp * wc[1][m2];                                          \
                      if (D >= 3) wp = wp * wc[2][m3];                                          \
                      T term = wp * src[m1 * vst[0] + m2 * vst[1] + m3 * vst[2]];               \
                      acc = acc + term;                                                         \
                    }                                                                           \
              }                                                                                 \
              T x = acc;                                                                        \
              if (g->factorcol) {                                                               \
                T f = factors[v + (int64_t)nvars * (g->factorcol - 1)];                         \
                x = x * f + (T)0;                                                               \
              }                                                                                 \
              work[tb * bs + v * vs + (tf[0] + i1) + (int64_t)(tf[1] + i2) * s2 +               \
                   (int64_t)(tf[2] + i3) * s3] = x;                                             \
            }                                                                                   \
    }                                                                                           \
  }                                                                                             \
                                                                                                \
  static void run_stage_##SUFFIX(const tam_schedule_desc *d, int32_t tag, T *work,             \
                                 const T *alt, int32_t nvars, const T *factors,                 \
                                 const int32_t *rotvars, int nthreads, int one_tap) {           \
    _Pragma("omp parallel num_threads(nthreads)") {                                             \
      int c = 0, k = 1;                                                                         \
      ORACLE_THREAD_IDS(c, k);                                                                  \
      int64_t lo, hi;                                                                           \
      equalsplit(d->nblocks, k, c, &lo, &hi);                                                   \
      for (int32_t gi = 0; gi < d->ngroups; ++gi) {                                             \
        const tam_group *g = &d->groups[gi];                                                    \
        if (g->stage != tag) continue;                                                          \
        const int32_t *owners = d->targetblocks + g->first;                                     \
        int64_t a = lower_bound(owners, 0, g->ntransfers, lo + 1);                              \
        int64_t b = lower_bound(owners, 0, g->ntransfers, hi + 1);                              \
        if (a < b)                                                                              \
          run_transfers_##SUFFIX(d, g, a, b, work, alt, nvars, factors, rotvars, one_tap);      \
      }                                                                                         \
    }                                                                                           \
  }

#ifdef _OPENMP
#define ORACLE_THREAD_IDS(c, k) \
  do {                          \
    c = omp_get_thread_num();   \
    k = omp_get_num_threads();  \
  } while (0)
#else
#define ORACLE_THREAD_IDS(c, k) \
  do {                          \
    c = 0;                      \
    k = 1;                      \
  } while (0)
#endif

DEFINE_ORACLE(double, f64)
DEFINE_ORACLE(float, f32)

static int collect_tags(const tam_schedule_desc *d, int32_t *tags, int cap) {
  int n = 0;
  for (int32_t gi = 0; gi < d->ngroups; ++gi) {
    int32_t t = d->groups[gi].stage, seen = 0;
    for (int j = 0; j < n; ++j) seen |= tags[j] == t;
    if (!seen && n < cap) tags[n++] = t;
  }
  for (int i = 1; i < n; ++i)
    for (int j = i; j > 0 && tags[j - 1] > tags[j]; --j) {
      int32_t x = tags[j];
      tags[j] = tags[j - 1];
      tags[j - 1] = x;
    }
  return n;
}

/* The serial-forest fill: every stage tag in [first, last], in order.
 * one_tap = 1: the CPU form of the sum, 0: the device form.  A turned group
 * (across a seam) reads variable rotvars[v + nvars r] - 1 (nvars x 4,
 * column-major, 1-based) of `alt` for an odd orientation r, of `work` for an
 * even one; `rotvars` may be NULL when the schedule has no turned group. */
int oracle_fill_turned(const tam_schedule_desc *d, void *work, const void *alt, int32_t nvars,
                       const void *factors, const int32_t *rotvars, int32_t first,
                       int32_t last, int nthreads, int one_tap) {
  if (!d || !work || nvars < 1) return -1;
  if (nthreads < 1) nthreads = 1;
  if (!alt) alt = work;
  for (int32_t gi = 0; gi < d->ngroups; ++gi)
    if (d->groups[gi].orientation && !rotvars) return -1;
  int32_t tags[128];
  int nt = collect_tags(d, tags, 128);
  for (int i = 0; i < nt; ++i) {
    if (tags[i] < first || tags[i] > last) continue;
    if (d->dtype == TAM_F64)
      run_stage_f64(d, tags[i], (double *)work, (const double *)alt, nvars,
                    (const double *)factors, rotvars, nthreads, one_tap);
    else
      run_stage_f32(d, tags[i], (float *)work, (const float *)alt, nvars,
                    (const float *)factors, rotvars, nthreads, one_tap);
  }
  return 0;
}

int oracle_fill(const tam_schedule_desc *d, void *work, int32_t nvars, const void *factors,
                int32_t first, int32_t last, int nthreads, int one_tap) {
  return oracle_fill_turned(d, work, work, nvars, factors, NULL, first, last, nthreads,
                            one_tap);
}

/* The transpose of the fill, in scatter form, serial.  Stage s is
 * x <- (I - E_s) x + E_s A_s x, with E_s the projection on its targets and
 * A_s reading the stage's sources as they were before it; its transpose is
 * y <- (I - E_s) y + A_s^T E_s y.  A stage may read its own targets (stage P
 * scales each wall-plane point in place), so the targets' adjoints are read
 * first (pass 0), the targets zeroed (pass 1), and then the values read
 * scattered onto their sources with the transfer's weights (pass 2).
 * Stages run in reverse tag order. */
#define DEFINE_ADJOINT(T, SUFFIX)                                                               \
  static int adjoint_stage_##SUFFIX(const tam_schedule_desc *d, int32_t tag, T *y,            \
                                     T *yalt, int32_t nvars, const T *factors,                  \
                                     const int32_t *rotvars) {                                  \
    const int D = d->ndim;                                                                      \
    int64_t S[3] = {1, 1, 1};                                                                   \
    for (int k = 0; k < D; ++k) S[k] = d->stored[k];                                            \
    const int64_t s2 = S[0], s3 = S[0] * S[1], vs = S[0] * S[1] * S[2], bs = vs * nvars;        \
    const T *W = (const T *)d->weights;                                                         \
    int64_t ntarget = 0;                                                                        \
    for (int32_t gi = 0; gi < d->ngroups; ++gi) {                                               \
      const tam_group *g = &d->groups[gi];                                                      \
      if (g->stage != tag) continue;                                                            \
      int64_t box = g->ntransfers * nvars;                                                      \
      for (int k = 0; k < D; ++k) box *= g->stencil[k].ntarget;                                 \
      ntarget += box;                                                                           \
    }                                                                                           \
    T *snap = (T *)malloc((size_t)(ntarget > 0 ? ntarget : 1) * sizeof(T));                    \
    if (!snap) return -1;                                                                       \
    for (int pass = 0; pass < 3; ++pass) {                                                      \
      int64_t k_snap = 0;                                                                       \
      for (int32_t gi = 0; gi < d->ngroups; ++gi) {                                             \
        const tam_group *g = &d->groups[gi];                                                    \
        if (g->stage != tag) continue;                                                          \
        int n[3] = {1, 1, 1}, o[3] = {1, 1, 1}, tf[3] = {0, 0, 0};                              \
        for (int k = 0; k < D; ++k) {                                                           \
          n[k] = g->stencil[k].ntarget;                                                         \
          o[k] = g->stencil[k].order;                                                           \
          tf[k] = g->stencil[k].targetfirst - 1;                                                \
        }                                                                                       \
        /* a turned group scatters onto its real source: for an odd turn the  \
           array yalt (a RotationPair's partner, or y itself for a set        \
           symmetric in the seam's plane), whose extent along e is           \
           R_e = S[perm[e]] (the same block and variable strides) */          \
        int64_t vst[3] = {1, s2, s3}, c0 = 0;                                                   \
        T *from = (g->orientation & 1) ? yalt : y;                                              \
        if (g->orientation) {                                                                   \
          int64_t R[3] = {1, 1, 1};                                                             \
          for (int e = 0; e < D; ++e) R[e] = S[(g->axes >> (2 * e)) & 3];                       \
          const int64_t rst[3] = {1, R[0], R[0] * R[1]};                                        \
          for (int e = 0; e < D; ++e) {                                                         \
            const int p = (g->axes >> (2 * e)) & 3, f = (g->axes >> (8 + e)) & 1;              \
            vst[p] = f ? -rst[e] : rst[e];                                                      \
            if (f) c0 += rst[e] * (R[e] - 1);                                                   \
          }                                                                                     \
        }                                                                                       \
        for (int64_t t = 0; t < g->ntransfers; ++t) {                                           \
          const int64_t tb = d->targetblocks[g->first + t] - 1;                                 \
          const int64_t sb = d->sourceblocks[g->first + t] - 1;                                 \
          for (int v = 0; v < nvars; ++v)                                                       \
            for (int i3 = 0; i3 < n[2]; ++i3)                                                   \
              for (int i2 = 0; i2 < n[1]; ++i2)                                                 \
                for (int i1 = 0; i1 < n[0]; ++i1) {                                             \
                  T *yt = y + tb * bs + v * vs + (tf[0] + i1) + (int64_t)(tf[1] + i2) * s2 +    \
                          (int64_t)(tf[2] + i3) * s3;                                           \
                  if (pass == 0) {                                                              \
                    snap[k_snap++] = *yt;                                                       \
                    continue;                                                                   \
                  }                                                                             \
                  if (pass == 1) {                                                              \
                    *yt = (T)0;                                                                 \
                    continue;                                                                   \
                  }                                                                             \
                  T a = snap[k_snap++];                                                         \
                  if (g->factorcol) a = a * factors[v + (int64_t)nvars * (g->factorcol - 1)];   \
                  int idx[3] = {i1, i2, i3};                                                    \
                  int64_t base[3] = {0, 0, 0};                                                  \
                  const T *wc[3] = {0, 0, 0};                                                   \
                  for (int k = 0; k < D; ++k) {                                                 \
                    base[k] = d->srcstart[g->stencil[k].srcstart + idx[k]] - 1;                 \
                    wc[k] = W + g->stencil[k].weights + (int64_t)o[k] * idx[k];                 \
                  }                                                                             \
                  const int sv =                                                                \
                      g->orientation ? rotvars[v + (int64_t)nvars * g->orientation] - 1 : v;    \
                  T *ys = from + sb * bs + sv * vs + c0 + base[0] * vst[0] +                    \
                          base[1] * vst[1] + base[2] * vst[2];                                  \
                  for (int m3 = 0; m3 < o[2]; ++m3)                                             \
                    for (int m2 = 0; m2 < o[1]; ++m2)                                           \
                      for (int m1 = 0; m1 < o[0]; ++m1) {                                       \
                        T wp = wc[0][m1];                                                       \
                        if (D >= 2) wp = wp * wc[1][m2];                                        \
                        if (D >= 3) wp = wp * wc[2][m3];                                        \
                        ys[m1 * vst[0] + m2 * vst[1] + m3 * vst[2]] += wp * a;                  \
                      }                                                                         \
                }                                                                               \
        }                                                                                       \
      }                                                                                         \
    }                                                                                           \
    free(snap);                                                                                 \
    return 0;                                                                                   \
  }

DEFINE_ADJOINT(double, f64)
DEFINE_ADJOINT(float, f32)

/* The transpose of oracle_fill_turned with `alt`: odd turns scatter onto
 * yalt (a RotationPair's partner cotangent, in the partner's layout).  For
 * the pair's whole fill a caller runs, tag by tag from the last, the second
 * member's stage and then the first's, each with the other's cotangent. */
int oracle_fill_adjoint_pair(const tam_schedule_desc *d, void *y, void *yalt, int32_t nvars,
                             const void *factors, const int32_t *rotvars, int32_t first,
                             int32_t last) {
  if (!d || !y || !yalt || nvars < 1) return -1;
  for (int32_t gi = 0; gi < d->ngroups; ++gi)
    if (d->groups[gi].orientation && !rotvars) return -1;
  int32_t tags[128];
  int nt = collect_tags(d, tags, 128);
  for (int i = nt - 1; i >= 0; --i) {
    if (tags[i] < first || tags[i] > last) continue;
    const int rc =
        d->dtype == TAM_F64
            ? adjoint_stage_f64(d, tags[i], (double *)y, (double *)yalt, nvars,
                                (const double *)factors, rotvars)
            : adjoint_stage_f32(d, tags[i], (float *)y, (float *)yalt, nvars,
                                (const float *)factors, rotvars);
    if (rc != 0) return rc;
  }
  return 0;
}

/* rotvars: the variable table of turned groups (NULL without any); a turned
 * group must keep the stored extents (a set symmetric in the seam's plane) */
int oracle_fill_adjoint_turned(const tam_schedule_desc *d, void *y, int32_t nvars,
                               const void *factors, const int32_t *rotvars, int32_t first,
                               int32_t last) {
  if (!d || !y || nvars < 1) return -1;
  for (int32_t gi = 0; gi < d->ngroups; ++gi) {
    const tam_group *g = &d->groups[gi];
    if (!g->orientation) continue;
    if (!rotvars) return -1;
    for (int e = 0; e < d->ndim; ++e)
      if (d->stored[(g->axes >> (2 * e)) & 3] != d->stored[e]) return -1;
  }
  return oracle_fill_adjoint_pair(d, y, y, nvars, factors, rotvars, first, last);
}

int oracle_fill_adjoint(const tam_schedule_desc *d, void *y, int32_t nvars, const void *factors,
                        int32_t first, int32_t last) {
  return oracle_fill_adjoint_turned(d, y, nvars, factors, NULL, first, last);
}
