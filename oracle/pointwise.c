/* The point-by-point ghost fill: TEST INFRASTRUCTURE ONLY.
 *
 * A second oracle of the ghost fill that uses no GhostSchedule.  For every
 * stored point of every block it derives from the forest's geometry alone
 * where the value comes from and computes it:
 *
 *   - the direction of the ghost region the point lies in, and, past a
 *     reflecting or outflow face, its mirror or clamped image and the parity
 *     factor (mirror_sources!, mirror_rows, clamp_rows, parityfactors:
 *     src/schedule.jl:2237-2297, 1337-1395; src/storage.jl:536-555);
 *   - the leaf covering the adjacent node by a lookup of the leaf set: the
 *     same level (a copy, src/schedule.jl:960-965), one level coarser (a
 *     prolongation, src/schedule.jl:1047-1079, with the window clamped into
 *     the coarse block's stored range) or finer (a restriction from the child
 *     covering the point, src/schedule.jl:1002-1025: injection along a
 *     vertex-like dimension, the order-p window clamped into the child's own
 *     range along a cell-like one);
 *   - for a vertex-centred set, the value of a point that several blocks
 *     hold (their closed boxes share it): the copy on the finest level
 *     holding it, there the one with the greatest class tuple, dimension 1
 *     first (piece_primary, src/schedule.jl:1911-1924), projected by
 *     (1 + sigma)/2 on a reflecting wall plane (stage P,
 *     src/schedule.jl:2605-2633); a ghost point that a block of the ghost's
 *     level holds takes that value (ghost_plane_parts, stage 0);
 *   - the stage order: own points first (stages P and 0), then every ghost
 *     that reads own points only (phase 1), then the prolongations by target
 *     level, coarsest first (src/ghosts.jl:1099-1160).
 *
 * The arithmetic is the reference's transfer_kernel! (src/ghosts.jl:58-128,
 * 363-402): acc = +0, acc += ((w_1 w_2) w_3) u with m_1 innermost and no
 * fused multiply-add (built with -ffp-contract=off), a copy +0 + u, a factor
 * x f + 0; the full sum over every tap (the reference's device form; on
 * finite data the same bits as its CPU form).  The weights are given by the
 * caller per window offset, computed there in exact rationals and rounded
 * once.
 *
 * Supported: brick forests of 1 to 3 dimensions, every dimension cell-like
 * or every one vertex-like, periodic, reflecting and outflow faces (no outer
 * faces left to a boundary hook, no seams).  The caller passes the leaves
 * (level and anchor, the node's integer coordinates at its level over the
 * whole brick) in the field data's block order. */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define PW_REFLECT 1
#define PW_OUTFLOW 2

typedef struct {
  int32_t D, N, p, vertex;
  int32_t G[3], S[3];
  int32_t roots[3];
  int32_t periodic[3];
  int32_t face[3][2];  /* past a non-periodic face: PW_REFLECT or PW_OUTFLOW */
  int64_t nblocks;
  int32_t nvars;
  const int32_t *level;    /* [nblocks] */
  const int64_t *anchor;   /* [nblocks * 3] */
  const int32_t *sigma;    /* [nvars * 3]: +1 even, -1 odd, per dimension */
} pw_mesh;

/* ---- the leaf set: open addressing on (level, anchor) ---------------------- */
typedef struct {
  int64_t size;
  int64_t *slot; /* block index or -1 */
  const pw_mesh *m;
} pw_table;

static uint64_t pw_hash(int lvl, const int64_t a[3]) {
  uint64_t h = 1469598103934665603ull ^ (uint64_t)lvl;
  for (int d = 0; d < 3; ++d) {
    h ^= (uint64_t)a[d] + 0x9E3779B97F4A7C15ull + (h << 6) + (h >> 2);
    h *= 1099511628211ull;
  }
  return h;
}

static int pw_table_init(pw_table *t, const pw_mesh *m) {
  int64_t size = 16;
  while (size < 4 * m->nblocks) size <<= 1;
  t->size = size;
  t->m = m;
  t->slot = (int64_t *)malloc(sizeof(int64_t) * size);
  if (!t->slot) return -1;
  for (int64_t i = 0; i < size; ++i) t->slot[i] = -1;
  for (int64_t b = 0; b < m->nblocks; ++b) {
    uint64_t h = pw_hash(m->level[b], m->anchor + 3 * b) & (uint64_t)(size - 1);
    while (t->slot[h] >= 0) h = (h + 1) & (uint64_t)(size - 1);
    t->slot[h] = b;
  }
  return 0;
}

/* The leaf at level `lvl` with anchor `a` (each coordinate wrapped where the
 * dimension is periodic), or -1; -2 when `a` lies outside a non-periodic
 * brick. */
static int64_t pw_find(const pw_table *t, int lvl, const int64_t a_in[3]) {
  const pw_mesh *m = t->m;
  int64_t a[3] = {0, 0, 0};
  for (int d = 0; d < m->D; ++d) {
    const int64_t n = (int64_t)m->roots[d] << lvl;
    a[d] = a_in[d];
    if (a[d] < 0 || a[d] >= n) {
      if (!m->periodic[d]) return -2;
      a[d] = ((a[d] % n) + n) % n;
    }
  }
  uint64_t h = pw_hash(lvl, a) & (uint64_t)(t->size - 1);
  for (;;) {
    const int64_t b = t->slot[h];
    if (b < 0) return -1;
    if (m->level[b] == lvl && m->anchor[3 * b] == a[0] && m->anchor[3 * b + 1] == a[1] &&
        m->anchor[3 * b + 2] == a[2])
      return b;
    h = (h + 1) & (uint64_t)(t->size - 1);
  }
}

static int64_t floordiv(int64_t a, int64_t b) {
  int64_t q = a / b;
  if ((a % b != 0) && ((a < 0) != (b < 0))) --q;
  return q;
}
static int64_t ceildiv(int64_t a, int64_t b) { return -floordiv(-a, b); }
static int64_t clampi(int64_t x, int64_t lo, int64_t hi) { return x < lo ? lo : x > hi ? hi : x; }

/* Where a point's value comes from. */
enum { SRC_OWN = 0, SRC_COPY = 1, SRC_SUM = 2 };
typedef struct {
  int kind;
  int64_t block;    /* the source block */
  int64_t at[3];    /* SRC_COPY: 0-based stored index in the source; SRC_SUM: window start */
  int32_t widx[3];  /* SRC_SUM: per dimension the weight row (4 * offset in the window) */
  int32_t order[3]; /* SRC_SUM: taps per dimension */
  int32_t fstate[3];/* per dimension: 0, 1 mirrored, 3 clamped */
  int32_t stage;    /* 0: phase 1 (reads own points), L >= 1: prolongation into level L */
} pw_src;

/* The primary copy of the vertex point of block b at 0-based own offsets
 * i[d] in 0..N: (holder block, its 0-based stored index).  Finest level
 * first (at most one finer than b under 2:1 balance), then the greatest
 * class tuple, dimension 1 most significant. */
static int64_t pw_primary(const pw_table *t, int64_t b, const int64_t i[3], int64_t at[3]) {
  const pw_mesh *m = t->m;
  const int L = m->level[b];
  for (int up = 1; up >= 0; --up) {
    const int lvl = L + up;
    int64_t Y[3] = {0, 0, 0};
    for (int d = 0; d < m->D; ++d) Y[d] = (m->anchor[3 * b + d] * m->N + i[d]) << up;
    int64_t best = -1, bestkey = -1;
    int64_t bestat[3] = {0, 0, 0};
    const int ncomb = 1 << m->D;
    for (int comb = 0; comb < ncomb; ++comb) {
      int64_t a[3] = {0, 0, 0};
      int64_t key = 0;
      int ok = 1;
      int64_t loc[3] = {0, 0, 0};
      for (int d = 0; d < m->D; ++d) {
        const int hi = (comb >> d) & 1;
        const int onplane = (Y[d] % m->N) == 0;
        int cls;
        if (onplane) {
          a[d] = hi ? Y[d] / m->N : Y[d] / m->N - 1;  /* hi: the block above, class 0 */
          cls = hi ? 0 : 2;
        } else {
          if (hi) { ok = 0; break; }
          a[d] = floordiv(Y[d], m->N);
          cls = 1;
        }
        loc[d] = Y[d] - a[d] * m->N + m->G[d];
        key = key * 3 + cls;
      }
      if (!ok) continue;
      int64_t aw[3] = {a[0], a[1], a[2]};
      const int64_t h = pw_find(t, lvl, aw);
      if (h < 0) continue;
      /* loc is the point's offset in the block whether or not the anchor
       * wrapped: a wrap moves the point and the anchor together */
      if (key > bestkey) {
        bestkey = key;
        best = h;
        for (int d = 0; d < 3; ++d) bestat[d] = loc[d];
      }
    }
    if (best >= 0) {
      for (int d = 0; d < 3; ++d) at[d] = bestat[d];
      return best;
    }
  }
  return -1;
}

/* The source of the stored point j (0-based) of block b. */
static int pw_source(const pw_table *t, int64_t b, const int64_t j[3], pw_src *s) {
  const pw_mesh *m = t->m;
  const int D = m->D, N = m->N, p = m->p, c = m->vertex;
  const int L = m->level[b];
  const int64_t *a = m->anchor + 3 * b;
  int delta[3] = {0, 0, 0};
  int64_t js[3] = {j[0], j[1], j[2]};  /* the image's 1-based stored index */
  int any = 0;
  memset(s, 0, sizeof(*s));
  for (int d = 0; d < D; ++d) {
    const int64_t jj = j[d] + 1;
    const int G = m->G[d];
    delta[d] = jj <= G ? -1 : jj > G + N + c ? 1 : 0;
    js[d] = jj;
    if (!delta[d]) continue;
    any = 1;
    const int64_t nn = a[d] + delta[d];
    const int64_t n = (int64_t)m->roots[d] << L;
    if ((nn < 0 || nn >= n) && !m->periodic[d]) {
      const int kind = m->face[d][delta[d] > 0];
      if (kind == PW_REFLECT) {
        js[d] = delta[d] < 0 ? 2 * G + 1 + c - jj : 2 * (G + N) + 1 + c - jj;
        s->fstate[d] = 1;
      } else if (kind == PW_OUTFLOW) {
        js[d] = delta[d] < 0 ? G + 1 : G + N + c;
        s->fstate[d] = 3;
      } else {
        return -1;  /* an outer face: the boundary hook's, not supported */
      }
      delta[d] = 0;
    }
  }
  if (!any) {
    s->kind = SRC_OWN;
    return 0;
  }
  int nz = 0;
  for (int d = 0; d < D; ++d) nz |= delta[d] != 0;
  if (!nz) {  /* the block's own point: a mirror or a clamp onto itself */
    s->kind = SRC_COPY;
    s->block = b;
    for (int d = 0; d < 3; ++d) s->at[d] = d < D ? js[d] - 1 : 0;
    s->stage = 0;
    return 0;
  }
  int64_t nb[3] = {0, 0, 0};
  for (int d = 0; d < D; ++d) nb[d] = a[d] + delta[d];
  int64_t same = pw_find(t, L, nb);
  if (same >= 0) {  /* a copy across the face, edge or corner */
    s->kind = SRC_COPY;
    s->block = same;
    for (int d = 0; d < 3; ++d) s->at[d] = d < D ? js[d] - (int64_t)N * delta[d] - 1 : 0;
    s->stage = 0;
    return 0;
  }
  int64_t par[3] = {0, 0, 0};
  for (int d = 0; d < D; ++d) par[d] = floordiv(nb[d], 2);
  const int64_t coarse = L > 0 ? pw_find(t, L - 1, par) : -1;
  if (coarse >= 0) {
    if (c == 1) {
      /* a point that a block of this level holds is that block's own */
      int64_t X[3] = {0, 0, 0}, cand[3][2];
      int nc[3] = {1, 1, 1};
      for (int d = 0; d < D; ++d) {
        X[d] = a[d] * N + (js[d] - m->G[d] - 1);
        if (X[d] % N == 0) {
          cand[d][0] = X[d] / N - 1;
          cand[d][1] = X[d] / N;
          nc[d] = 2;
        } else {
          cand[d][0] = floordiv(X[d], N);
        }
      }
      for (int k2 = 0; k2 < (D >= 3 ? nc[2] : 1); ++k2)
        for (int k1 = 0; k1 < (D >= 2 ? nc[1] : 1); ++k1)
          for (int k0 = 0; k0 < nc[0]; ++k0) {
            const int kk[3] = {k0, k1, k2};
            int64_t an[3] = {0, 0, 0};
            for (int d = 0; d < D; ++d) an[d] = cand[d][kk[d]];
            const int64_t h = pw_find(t, L, an);
            if (h < 0) continue;
            s->kind = SRC_COPY;
            s->block = h;
            for (int d = 0; d < 3; ++d)
              s->at[d] = d < D ? X[d] - an[d] * N + m->G[d] : 0;
            s->stage = 0;
            return 0;
          }
    }
    /* prolongation from the coarser leaf, in its stored frame */
    s->kind = SRC_SUM;
    s->block = coarse;
    s->stage = L;
    for (int d = 0; d < 3; ++d) {
      if (d >= D) {
        s->at[d] = 0;
        s->order[d] = 1;
        s->widx[d] = 0;
        continue;
      }
      const int G = m->G[d], Sd = m->S[d];
      const int od = (int)(a[d] & 1);
      const int sd = (delta[d] == 1 && od == 1) ? 1 : (delta[d] == -1 && od == 0) ? -1 : 0;
      const int64_t phi = (int64_t)od * N + js[d] - G - 1;
      const int64_t origin = -(int64_t)N * sd + G + 1;
      int64_t lo, four_x;
      if (c == 1) {
        lo = clampi(floordiv(phi, 2) - p / 2 + 1 + origin, 1, Sd - p + 1);
        four_x = 2 * phi + 4 * origin;
      } else {
        lo = clampi(ceildiv(phi, 2) - p / 2 + origin, 1, Sd - p + 1);
        four_x = 2 * phi - 1 + 4 * origin;
      }
      const int64_t w = four_x - 4 * lo;
      if (w < 0 || w > 4 * (p - 1)) return -3;  /* would extrapolate */
      s->at[d] = lo - 1;
      s->order[d] = p;
      s->widx[d] = (int32_t)w;
    }
    return 0;
  }
  /* finer: the child of the adjacent node covering the point */
  int64_t child[3] = {0, 0, 0};
  int od[3] = {0, 0, 0};
  for (int d = 0; d < D; ++d) {
    if (delta[d] == 1) od[d] = 0;
    else if (delta[d] == -1) od[d] = 1;
    else {
      const int64_t q = js[d] - m->G[d] - 1;
      od[d] = c == 1 ? q > N / 2 : q >= N / 2;
    }
    child[d] = 2 * nb[d] + od[d];
  }
  const int64_t fine = pw_find(t, L + 1, child);
  if (fine < 0) return -4;  /* not a 2:1 balanced forest */
  s->block = fine;
  s->stage = 0;
  if (c == 1) {
    s->kind = SRC_COPY;
    for (int d = 0; d < 3; ++d) {
      if (d >= D) { s->at[d] = 0; continue; }
      const int G = m->G[d];
      s->at[d] = G + 2 * (js[d] - (int64_t)N * delta[d] - G - 1 - (int64_t)od[d] * (N / 2));
    }
    return 0;
  }
  s->kind = SRC_SUM;
  for (int d = 0; d < 3; ++d) {
    if (d >= D) {
      s->at[d] = 0;
      s->order[d] = 1;
      s->widx[d] = 0;
      continue;
    }
    const int G = m->G[d];
    const int64_t q = js[d] - (int64_t)N * delta[d] - G - 1;
    const int64_t f0 = G + 1 + 2 * (q - (int64_t)od[d] * (N / 2));
    const int64_t lo = clampi(f0 - p / 2 + 1, G + 1, G + N - p + 1);
    s->at[d] = lo - 1;
    s->order[d] = p;
    s->widx[d] = (int32_t)(4 * (f0 - lo) + 2);
  }
  return 0;
}

/* ---- the fill, per element type ------------------------------------------ */
#define PW_DEFINE(T, NAME)                                                                   \
  static T NAME##_factor(const pw_mesh *m, const int32_t fstate[3], int v) {               \
    T f = (T)1;                                                                            \
    for (int d = 0; d < m->D; ++d)                                                         \
      if (fstate[d] == 1) f = f * (T)m->sigma[3 * v + d];                                  \
    return f;                                                                              \
  }                                                                                        \
  static void NAME##_point(const pw_table *t, const T *wtab, const T *src, T *dst,         \
                           int64_t b, const int64_t j[3], const pw_src *s) {               \
    const pw_mesh *m = t->m;                                                               \
    const int64_t S1 = m->S[0], S2 = m->S[1], S3 = m->S[2];                                \
    const int64_t vol = S1 * S2 * S3;                                                      \
    const int64_t toff = (j[2] * S2 + j[1]) * S1 + j[0];                                   \
    int mirrored = 0;                                                                      \
    for (int d = 0; d < m->D; ++d) mirrored |= s->fstate[d] != 0;                          \
    for (int v = 0; v < m->nvars; ++v) {                                                   \
      const T *sp = src + (s->block * m->nvars + v) * vol;                                 \
      T x;                                                                                 \
      if (s->kind == SRC_COPY) {                                                           \
        x = (T)0 + sp[(s->at[2] * S2 + s->at[1]) * S1 + s->at[0]];                         \
      } else {                                                                             \
        const T *w1 = wtab + (int64_t)s->widx[0] * m->p;                                   \
        const T *w2 = wtab + (int64_t)s->widx[1] * m->p;                                   \
        const T *w3 = wtab + (int64_t)s->widx[2] * m->p;                                   \
        T acc = (T)0;                                                                      \
        for (int m3 = 0; m3 < s->order[2]; ++m3)                                           \
          for (int m2 = 0; m2 < s->order[1]; ++m2)                                         \
            for (int m1 = 0; m1 < s->order[0]; ++m1) {                                     \
              T wp = w1[m1];                                                               \
              if (m->D >= 2) wp = wp * w2[m2];                                             \
              if (m->D >= 3) wp = wp * w3[m3];                                             \
              const T u = sp[((s->at[2] + m3) * S2 + s->at[1] + m2) * S1 + s->at[0] + m1]; \
              acc = acc + wp * u;                                                          \
            }                                                                              \
        x = acc;                                                                           \
      }                                                                                    \
      if (mirrored) x = x * NAME##_factor(m, s->fstate, v) + (T)0;                         \
      dst[(b * m->nvars + v) * vol + toff] = x;                                            \
    }                                                                                      \
  }                                                                                        \
  static int NAME##_fill(const pw_mesh *m, const T *wtab, const T *in, T *out, int nthreads) { \
    pw_table t;                                                                            \
    if (pw_table_init(&t, m)) return -10;                                                  \
    const int64_t S1 = m->S[0], S2 = m->S[1], S3 = m->S[2];                                \
    const int64_t vol = S1 * S2 * S3;                                                      \
    int maxlevel = 0;                                                                      \
    for (int64_t b = 0; b < m->nblocks; ++b)                                               \
      if (m->level[b] > maxlevel) maxlevel = m->level[b];                                  \
    int status = 0;                                                                        \
    /* own points: stages P and 0 for a vertex-centred set */                              \
    _Pragma("omp parallel for schedule(dynamic, 4) num_threads(nthreads)")                 \
    for (int64_t b = 0; b < m->nblocks; ++b) {                                             \
      for (int64_t i2 = 0; i2 < S3; ++i2)                                                  \
        for (int64_t i1 = 0; i1 < S2; ++i1)                                                \
          for (int64_t i0 = 0; i0 < S1; ++i0) {                                            \
            const int64_t j[3] = {i0, i1, i2};                                             \
            int own = 1, face = 0;                                                         \
            int64_t io[3] = {0, 0, 0};                                                     \
            for (int d = 0; d < m->D; ++d) {                                               \
              io[d] = j[d] - m->G[d];                                                      \
              if (io[d] < 0 || io[d] > m->N + m->vertex - 1) own = 0;                      \
              if (m->vertex && (io[d] == 0 || io[d] == m->N)) face = 1;                    \
            }                                                                              \
            if (!own) continue;                                                            \
            const int64_t toff = (i2 * S2 + i1) * S1 + i0;                                 \
            if (!face) {                                                                   \
              for (int v = 0; v < m->nvars; ++v)                                           \
                out[(b * m->nvars + v) * vol + toff] = in[(b * m->nvars + v) * vol + toff]; \
              continue;                                                                    \
            }                                                                              \
            int64_t at[3];                                                                 \
            const int64_t h = pw_primary(&t, b, io, at);                                   \
            if (h < 0) {                                                                   \
              status = -5;                                                                 \
              continue;                                                                    \
            }                                                                              \
            const int primary = h == b && at[0] == i0 && at[1] == i1 && at[2] == i2;       \
            int32_t wall[3] = {0, 0, 0};                                                   \
            int onwall = 0;                                                                \
            for (int d = 0; d < m->D; ++d) {                                               \
              if (m->periodic[d]) continue;                                                \
              const int64_t X = m->anchor[3 * b + d] * m->N + io[d];                       \
              const int64_t top = ((int64_t)m->roots[d] << m->level[b]) * m->N;            \
              if ((X == 0 && m->face[d][0] == PW_REFLECT) ||                               \
                  (X == top && m->face[d][1] == PW_REFLECT)) {                             \
                wall[d] = 1;                                                               \
                onwall = 1;                                                                \
              }                                                                            \
            }                                                                              \
            const int64_t hoff = (at[2] * S2 + at[1]) * S1 + at[0];                        \
            for (int v = 0; v < m->nvars; ++v) {                                           \
              T x = in[(h * m->nvars + v) * vol + hoff];                                   \
              if (onwall) {                                                                \
                T f = (T)1;                                                                \
                for (int d = 0; d < m->D; ++d)                                             \
                  if (wall[d]) f = f * (T)((1 + m->sigma[3 * v + d]) / 2);                 \
                x = x * f + (T)0;                                                          \
              }                                                                            \
              if (!primary) x = (T)0 + x;                                                  \
              out[(b * m->nvars + v) * vol + toff] = x;                                    \
            }                                                                              \
          }                                                                                \
    }                                                                                      \
    if (status) {                                                                          \
      free(t.slot);                                                                        \
      return status;                                                                       \
    }                                                                                      \
    /* phase 1, then the prolongations into each level, coarsest first */                 \
    for (int stage = 0; stage <= maxlevel; ++stage) {                                      \
      _Pragma("omp parallel for schedule(dynamic, 4) num_threads(nthreads)")               \
      for (int64_t b = 0; b < m->nblocks; ++b) {                                           \
        if (stage > 0 && m->level[b] != stage) continue;                                   \
        for (int64_t i2 = 0; i2 < S3; ++i2)                                                \
          for (int64_t i1 = 0; i1 < S2; ++i1)                                              \
            for (int64_t i0 = 0; i0 < S1; ++i0) {                                          \
              const int64_t j[3] = {i0, i1, i2};                                           \
              pw_src s;                                                                    \
              const int rc = pw_source(&t, b, j, &s);                                      \
              if (rc) {                                                                    \
                status = rc;                                                               \
                continue;                                                                  \
              }                                                                            \
              if (s.kind == SRC_OWN || s.stage != stage) continue;                         \
              NAME##_point(&t, wtab, out, out, b, j, &s);                                  \
            }                                                                              \
      }                                                                                    \
    }                                                                                      \
    free(t.slot);                                                                          \
    return status;                                                                         \
  }

PW_DEFINE(double, pw_f64)
PW_DEFINE(float, pw_f32)

/* Fills `out` (every block's stored points, column-major per block and
 * variable, blocks in the leaves' order) from the own points of `in`.
 * `wtab` holds, for each window offset 4 * (x - lo) in 0..4(p-1), the p
 * weights of the order-p Lagrange interpolant at x, in the element type.
 * Returns 0, or a negative code: -1 an outer face, -3 a window that would
 * extrapolate, -4 a forest that is not 2:1 balanced, -5 a shared point no
 * block holds, -10 no memory. */
int pw_fill(const pw_mesh *m, int dtype_bytes, const void *wtab, const void *in, void *out,
            int nthreads) {
  if (!m || m->D < 1 || m->D > 3 || m->p < 1) return -9;
  if (dtype_bytes == 8)
    return pw_f64_fill(m, (const double *)wtab, (const double *)in, (double *)out, nthreads);
  return pw_f32_fill(m, (const float *)wtab, (const float *)in, (float *)out, nthreads);
}
