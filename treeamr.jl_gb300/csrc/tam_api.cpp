// Host side of libtreeamr_cuda.so: descriptor validation, upload, tiling
// and the stage loop of a fill.  See include/treeamr_cuda.h for the ABI.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "tam_internal.h"
#include "treeamr_cuda.h"

namespace {

std::mutex g_err_mutex;
std::string g_err;  // errors with no context

int fail(tam_ctx *ctx, int code, const std::string &msg) {
  if (ctx) {
    ctx->err = msg;
  } else {
    std::lock_guard<std::mutex> lock(g_err_mutex);
    g_err = msg;
  }
  return code;
}

}  // namespace

namespace tam {
int record_error(tam_ctx *ctx, int code, const std::string &msg) { return fail(ctx, code, msg); }
}  // namespace tam

namespace {

int cuda_fail(tam_ctx *ctx, cudaError_t e, const char *what) {
  cudaGetLastError();  // clear a sticky-free error so the next call starts clean
  return fail(ctx, TAM_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// Runs the body with the context's device current and puts the caller's
// device back afterwards.
class DeviceGuard {
 public:
  explicit DeviceGuard(int device) {
    ok_ = cudaGetDevice(&prev_) == cudaSuccess;
    if (ok_ && prev_ != device) ok_ = cudaSetDevice(device) == cudaSuccess;
  }
  ~DeviceGuard() {
    int cur = -1;
    if (cudaGetDevice(&cur) == cudaSuccess && cur != prev_) cudaSetDevice(prev_);
  }
  bool ok() const { return ok_; }

 private:
  int prev_ = 0;
  bool ok_ = false;
};

template <typename T>
cudaError_t upload(T **dst, const T *src, size_t n) {
  *dst = nullptr;
  if (n == 0) n = 1;  // a valid pointer even for an empty pool
  cudaError_t e = cudaMalloc((void **)dst, n * sizeof(T));
  if (e != cudaSuccess) return e;
  if (src) return cudaMemcpy(*dst, src, n * sizeof(T), cudaMemcpyHostToDevice);
  return cudaMemset(*dst, 0, n * sizeof(T));
}

void free_sched_device(tam_sched *s) {
  cudaFree(s->d_groups);
  cudaFree(s->d_tb);
  cudaFree(s->d_sb);
  cudaFree(s->d_srcstart);
  cudaFree(s->d_weights);
  cudaFree(s->d_tiles);
  cudaFree(s->d_ptiles);
  cudaFree(s->d_cls);
  cudaFree(s->d_wtab);
  cudaFree(s->d_wshort);
  cudaFree(s->d_staged);
  cudaFree(s->d_csingle);
  cudaFree(s->d_perm);
  cudaFree(s->d_err);
  cudaFree(s->d_solos);
  tam::side_destroy(s->side);
  s->d_ptiles = nullptr;
  s->d_groups = nullptr;
  s->d_tb = s->d_sb = s->d_srcstart = nullptr;
  s->d_weights = nullptr;
  s->d_tiles = nullptr;
  s->d_cls = nullptr;
  s->d_wtab = nullptr;
  s->d_wshort = nullptr;
  s->d_staged = nullptr;
  s->d_csingle = s->d_perm = nullptr;
  s->d_err = nullptr;
  s->d_solos = nullptr;
}

// Every check that makes a fill memory-safe: indices into the pools, block
// indices, and each stencil's target rows and source windows inside the
// stored extent.
int validate(tam_ctx *ctx, const tam_schedule_desc *d, int64_t nsource) {
  char buf[256];
  if (!d) return fail(ctx, TAM_EINVAL, "schedule descriptor is NULL");
  if (d->abi_version != TAM_ABI_VERSION) {
    snprintf(buf, sizeof buf, "descriptor ABI version %d, library %d", d->abi_version,
             TAM_ABI_VERSION);
    return fail(ctx, TAM_EINVAL, buf);
  }
  if (d->ndim < 1 || d->ndim > 3) return fail(ctx, TAM_EINVAL, "ndim must be 1, 2 or 3");
  if (d->dtype != TAM_F32 && d->dtype != TAM_F64)
    return fail(ctx, TAM_EINVAL, "dtype must be TAM_F32 or TAM_F64");
  if (d->nblocks < 0 || d->nblocks > INT32_MAX) return fail(ctx, TAM_EINVAL, "bad nblocks");
  if (d->ngroups < 0) return fail(ctx, TAM_EINVAL, "bad ngroups");
  if (d->ngroups > 0 && !d->groups) return fail(ctx, TAM_EINVAL, "groups is NULL");
  if (d->ntransfers < 0 || d->ntransfers > INT32_MAX)
    return fail(ctx, TAM_EINVAL, "bad ntransfers");
  if (d->ntransfers > 0 && (!d->targetblocks || !d->sourceblocks))
    return fail(ctx, TAM_EINVAL, "block lists are NULL");
  if (d->nsrcstart < 0 || (d->nsrcstart > 0 && !d->srcstart))
    return fail(ctx, TAM_EINVAL, "bad srcstart pool");
  if (d->nweights < 0 || (d->nweights > 0 && !d->weights))
    return fail(ctx, TAM_EINVAL, "bad weight pool");
  int64_t maxcols = 1;
  for (int k = 0; k < d->ndim; ++k) maxcols *= 3;
  if (d->nfactorcols != maxcols && d->nfactorcols != 4 * maxcols)
    return fail(ctx, TAM_EINVAL, "nfactorcols must be 3^D, or 4 * 3^D over a seam");
  maxcols = d->nfactorcols;
  int64_t vol = 1;
  for (int k = 0; k < d->ndim; ++k) {
    if (d->stored[k] < 1) return fail(ctx, TAM_EINVAL, "stored extents must be positive");
    vol = std::min<int64_t>(vol * d->stored[k], (int64_t)INT32_MAX + 1);
  }
  // the kernels address within a block's variable in 32 bits
  if (vol > INT32_MAX) return fail(ctx, TAM_EUNSUPPORTED, "a block of 2^31 points or more");
  if (nsource < 0 || nsource > INT32_MAX) return fail(ctx, TAM_EINVAL, "bad source block count");
  for (int64_t t = 0; t < d->ntransfers; ++t) {
    if (d->targetblocks[t] < 1 || d->targetblocks[t] > d->nblocks ||
        d->sourceblocks[t] < 1 || d->sourceblocks[t] > nsource) {
      snprintf(buf, sizeof buf,
               "transfer %lld names a block outside 1:%lld (targets) or 1:%lld (sources)",
               (long long)t, (long long)d->nblocks, (long long)nsource);
      return fail(ctx, TAM_EINVAL, buf);
    }
  }
  for (int32_t gi = 0; gi < d->ngroups; ++gi) {
    const tam_group &g = d->groups[gi];
    if (g.kind < TAM_COPY || g.kind > TAM_PROLONG) return fail(ctx, TAM_EINVAL, "bad group kind");
    if (g.bounded < 0 || g.bounded > 2)
      return fail(ctx, TAM_EINVAL, "a group's bound must be 0, 1 or 2");
    if (g.factorcol < 0 || g.factorcol > maxcols)
      return fail(ctx, TAM_EINVAL, "factor column outside the table");
    if (g.first < 0 || g.ntransfers < 0 || g.first + g.ntransfers > d->ntransfers)
      return fail(ctx, TAM_EINVAL, "group block range outside the block lists");
    if (g.stage < TAM_STAGE_SELFIMAGE || g.stage > 2 + 64)
      return fail(ctx, TAM_EINVAL, "bad stage tag");
    if (g.orientation < 0 || g.orientation > 3)
      return fail(ctx, TAM_EINVAL, "a group's orientation must be 0..3");
    if (g.orientation == 0 && g.axes != 0)
      return fail(ctx, TAM_EINVAL, "an ordinary group has the identity axis map (axes = 0)");
    if (g.orientation != 0) {
      // the axis map: a permutation of the dimensions.  The real array has
      // stored extent S[perm[e]] along e (the schedule's own layout for a set
      // symmetric in the seam's plane, the partner's swapped one for an odd
      // orientation of a RotationPair), so a virtual index inside the stored
      // box reads a real one inside the real array's box
      int seen = 0;
      for (int e = 0; e < 3; ++e) {
        const int p = (g.axes >> (2 * e)) & 3, f = (g.axes >> (8 + e)) & 1;
        if (e >= d->ndim) {
          if (p != 0 || f != 0)
            return fail(ctx, TAM_EINVAL, "axis map entries beyond ndim must be zero");
          continue;
        }
        if (p >= d->ndim || (seen >> p) & 1)
          return fail(ctx, TAM_EINVAL, "a turned group's axis map is not a permutation");
        seen |= 1 << p;
        if ((g.orientation & 1) == 0 && d->stored[p] != d->stored[e])
          return fail(ctx, TAM_EINVAL,
                      "an even orientation reads the set's own array, so its axis map must "
                      "keep the stored extents");
      }
      if ((g.axes & ~0x73F) != 0)
        return fail(ctx, TAM_EINVAL, "stray bits in a turned group's axis map");
    }
    for (int k = 0; k < d->ndim; ++k) {
      const tam_stencil &s = g.stencil[k];
      const int S = d->stored[k];
      if (s.ntarget < 1 || s.order < 1 || s.order > 16) {
        snprintf(buf, sizeof buf, "group %d dim %d: ntarget %d order %d", gi, k + 1, s.ntarget,
                 s.order);
        return fail(ctx, TAM_EINVAL, buf);
      }
      if (g.bounded == 1 && (s.order != 3 || s.unit))
        return fail(ctx, TAM_EINVAL,
                    "a bounded conservative group has order-3 stencils in every dimension");
      if (g.bounded == 2 && (s.order % 2 || s.unit))
        return fail(ctx, TAM_EINVAL,
                    "a bounded point-value group's stencils stack two sets of weights");
      // the source window: a stacked point-value stencil reads half its rows
      const int win = g.bounded == 2 ? s.order / 2 : s.order;
      if (s.targetfirst < 1 || s.targetfirst + s.ntarget - 1 > S)
        return fail(ctx, TAM_EINVAL, "target rows outside the stored extent");
      if (s.srcstart < 0 || s.srcstart + s.ntarget > d->nsrcstart)
        return fail(ctx, TAM_EINVAL, "srcstart offset outside the pool");
      if (s.weights < 0 || s.weights + (int64_t)s.order * s.ntarget > d->nweights)
        return fail(ctx, TAM_EINVAL, "weight offset outside the pool");
      for (int i = 0; i < s.ntarget; ++i) {
        const int32_t b = d->srcstart[s.srcstart + i];
        if (b < 1 || b + win - 1 > S) {
          snprintf(buf, sizeof buf,
                   "group %d dim %d row %d: source window %d:%d outside 1:%d", gi, k + 1, i + 1,
                   b, b + win - 1, S);
          return fail(ctx, TAM_EINVAL, buf);
        }
      }
    }
  }
  return TAM_OK;
}

// The weight products of a uniform-order group: per dimension the distinct
// weight columns ("classes") and each row's class, then for every class
// combination the P^D products ((w_1*w_2)*w_3) rounded in T in that order
// (src/ghosts.jl:58-74), which is what the reference forms per tap.  Only the
// operand order matters for the bits: each product is one IEEE multiply.
template <typename T>
void build_product_table(const tam_schedule_desc *d, const tam_group &h, tam::DevGroup &g,
                         std::vector<int32_t> &cls, std::vector<unsigned char> &wtab) {
  const T *W = (const T *)d->weights;
  const int P = h.stencil[0].order;
  std::vector<std::vector<const T *>> columns(3);
  for (int k = 0; k < 3; ++k) {
    g.cls[k] = (int64_t)cls.size();
    if (k >= d->ndim) {
      g.C[k] = 1;
      cls.push_back(0);
      continue;
    }
    const tam_stencil &st = h.stencil[k];
    for (int i = 0; i < st.ntarget; ++i) {
      const T *col = W + st.weights + (int64_t)P * i;
      int found = -1;
      for (size_t c = 0; c < columns[k].size(); ++c)
        if (memcmp(columns[k][c], col, sizeof(T) * P) == 0) {
          found = (int)c;
          break;
        }
      if (found < 0) {
        found = (int)columns[k].size();
        columns[k].push_back(col);
      }
      cls.push_back(found);
    }
    g.C[k] = (int32_t)columns[k].size();
  }
  const int P2 = d->ndim >= 2 ? P : 1, P3 = d->ndim >= 3 ? P : 1;
  size_t off = wtab.size();
  // element-aligned start
  while (off % sizeof(T)) ++off;
  g.wtab = (int64_t)(off / sizeof(T));
  const int64_t count = (int64_t)g.C[0] * g.C[1] * g.C[2] * P * P2 * P3;
  wtab.resize(off + count * sizeof(T));
  T *out = (T *)(wtab.data() + off);
  int64_t n = 0;
  const T one = T(1);
  for (int c3 = 0; c3 < g.C[2]; ++c3)
    for (int c2 = 0; c2 < g.C[1]; ++c2)
      for (int c1 = 0; c1 < g.C[0]; ++c1)
        for (int m3 = 0; m3 < P3; ++m3)
          for (int m2 = 0; m2 < P2; ++m2)
            for (int m1 = 0; m1 < P; ++m1) {
              const T w1 = columns[0][c1][m1];
              const T w2 = d->ndim >= 2 ? columns[1][c2][m2] : one;
              const T w3 = d->ndim >= 3 ? columns[2][c3][m3] : one;
              volatile T p = w1;  // one rounding per multiply, in T, left to right
              if (d->ndim >= 2) p = p * w2;
              if (d->ndim >= 3) p = p * w3;
              out[n++] = p;
            }
  // Float64 products whose significands fit 24 bits take the integer-pipe
  // multiply (mul_short in tam_kernels.cuh); it needs normal nonzero weights.
  g.shortw = 0;
  if (sizeof(T) == 8) {
    bool ok = true;
    for (int64_t i = 0; i < count && ok; ++i) {
      uint64_t b;
      memcpy(&b, &out[i], 8);
      const uint64_t e = (b >> 52) & 0x7FF;
      // a zero product is allowed: the multiply flags it and the point takes
      // the FP64 pipe, and the one-tap form never reaches it
      ok = (b << 1) == 0 || (e >= 1 && e <= 2046 && (b & ((1ull << 29) - 1)) == 0);
    }
    g.shortw = ok ? 1 : 0;
  }
}

// The one-tap skip of the reference's CPU fill (src/ghosts.jl:28-56,
// src/schedule.jl:83-86 single_rows): per dimension and target row, the row
// of the column's only nonzero weight, or -1.  Where any row of the group has
// one, `perm` lists the box points ordered (stably) by the set of dimensions
// that skip, so that the lanes of a warp mostly share their trip counts.
template <typename T>
void build_singles(const tam_schedule_desc *d, const tam_group &h, tam::DevGroup &g,
                   std::vector<int32_t> &csingle, std::vector<int32_t> &perm) {
  const T *W = (const T *)d->weights;
  bool any = false;
  for (int k = 0; k < 3; ++k) {
    g.csingle[k] = (int64_t)csingle.size();
    if (k >= d->ndim) {
      csingle.push_back(-1);
      continue;
    }
    const tam_stencil &st = h.stencil[k];
    for (int i = 0; i < st.ntarget; ++i) {
      const T *col = W + st.weights + (int64_t)st.order * i;
      int row = -1, nonzero = 0;
      for (int m = 0; m < st.order; ++m)
        if (col[m] != T(0)) {
          ++nonzero;
          row = m;
        }
      const int single = nonzero == 1 ? row : -1;
      any = any || (single >= 0 && st.order > 1);
      csingle.push_back(single);
    }
  }
  g.perm = -1;
  if (!any) return;
  g.perm = (int64_t)perm.size();
  std::vector<std::pair<int, int>> order;
  order.reserve((size_t)g.n[0] * g.n[1] * g.n[2]);
  for (int i3 = 0; i3 < g.n[2]; ++i3)
    for (int i2 = 0; i2 < g.n[1]; ++i2)
      for (int i1 = 0; i1 < g.n[0]; ++i1) {
        const int idx[3] = {i1, i2, i3};
        int mask = 0;
        for (int k = 0; k < d->ndim; ++k)
          if (csingle[g.csingle[k] + idx[k]] >= 0) mask |= 1 << k;
        order.push_back({mask, i1 + g.n[0] * (i2 + g.n[1] * i3)});
      }
  std::stable_sort(order.begin(), order.end(),
                   [](const std::pair<int, int> &a, const std::pair<int, int> &b) {
                     return a.first < b.first;
                   });
  for (const auto &o : order) perm.push_back(o.second);
}

tam::SchedArgs sched_args(const tam_sched *s) {
  return tam::SchedArgs{s->d_groups, s->d_tb,     s->d_sb,        s->d_srcstart,
                        s->d_weights, s->d_cls,   s->d_wtab,      s->shape.int_mul,
                        nullptr,      s->d_csingle, s->d_perm,    s->shape.one_tap,
                        s->shape.copy_points, s->d_wshort, s->shape.pair_vars,
                        s->shape.copy_share * s->ctx->nsm, s->shape.soft_add};
}

// The order in which the fused launches visit target blocks: with
// TAM_OPT_BLOCK_ORDER 1, a reverse Cuthill-McKee numbering of the graph whose
// edges are the schedule's transfers (breadth first from a block of least
// degree, each block's neighbours in increasing degree, the whole reversed),
// so that blocks that exchange ghosts are visited close together in time and
// the sectors they share -- a block's faces are one transfer's source and
// another's target -- stay in L2 between the two; otherwise the blocks' own
// (curve) order.  rank[b] for 1-based block b - 1.
std::vector<int32_t> block_rank(const tam_sched *s) {
  const int64_t n = s->nblocks;
  std::vector<int32_t> rank(n);
  for (int64_t b = 0; b < n; ++b) rank[b] = (int32_t)b;
  if (s->shape.block_order != 1 || s->nsource != s->nblocks || n < 2) return rank;
  std::vector<std::vector<int32_t>> adj(n);
  for (size_t t = 0; t < s->h_tb.size(); ++t) {
    const int32_t a = s->h_tb[t] - 1, c = s->h_sb[t] - 1;
    if (a == c) continue;
    adj[a].push_back(c);
    adj[c].push_back(a);
  }
  for (auto &l : adj) {
    std::sort(l.begin(), l.end());
    l.erase(std::unique(l.begin(), l.end()), l.end());
  }
  auto deg_less = [&](int32_t x, int32_t y) {
    return adj[x].size() != adj[y].size() ? adj[x].size() < adj[y].size() : x < y;
  };
  for (auto &l : adj) std::sort(l.begin(), l.end(), deg_less);
  std::vector<int32_t> order;
  order.reserve(n);
  std::vector<char> seen(n, 0);
  std::vector<int32_t> by_degree(n);
  for (int64_t b = 0; b < n; ++b) by_degree[b] = (int32_t)b;
  std::sort(by_degree.begin(), by_degree.end(), deg_less);
  for (int32_t start : by_degree) {  // every connected component
    if (seen[start]) continue;
    size_t head = order.size();
    order.push_back(start);
    seen[start] = 1;
    while (head < order.size()) {
      const int32_t v = order[head++];
      for (int32_t w : adj[v])
        if (!seen[w]) {
          seen[w] = 1;
          order.push_back(w);
        }
    }
  }
  for (int64_t i = 0; i < n; ++i) rank[order[n - 1 - i]] = (int32_t)i;
  return rank;
}

// The fused tiles of every stage: each stage's transfers ordered by target
// block (in block_rank's order), then group, each cut into runs of
// `tile_items` box points; the
// stencil tiles cut where their points' path through the kernel changes and
// ordered by it, each path's tiles in that order (tam::StencilRuns), with
// the path's key in `keys` (0 for a copy tile).
void tiles_of(tam_sched *s, std::vector<tam::Stage> &list, const std::vector<int32_t> &rank,
              tam::StencilRuns &runs, std::vector<tam::Tile> &tiles,
              std::vector<uint16_t> &keys, std::vector<tam::Tile> &staged) {
  const int ti = s->shape.tile_items, tst = s->shape.stencil_items();
  for (tam::Stage &st : list) {
    st.tile0 = (int64_t)tiles.size();
    struct Entry {
      int32_t tblock, group, transfer, sblock;
    };
    std::vector<Entry> entries;
    for (int32_t gi : st.groups) {
      const tam::DevGroup &g = s->groups[gi];
      if (g.turned) continue;  // a turned group has a launch of its own
      for (int64_t t = 0; t < g.ntransfers; ++t)
        entries.push_back({rank[s->h_tb[g.first + t] - 1], gi, (int32_t)(g.first + t),
                           s->h_sb[g.first + t] - 1});
    }
    // by target block, or (TAM_OPT_BLOCK_ORDER 2) by source block first: the
    // transfers that read one block's edges then run together, and its
    // sectors come from DRAM once; 3: the copies by target block and the
    // stencils, whose source windows several targets share, by source
    auto by = [](bool source) {
      return [source](const Entry &a, const Entry &b) {
        if (source && a.sblock != b.sblock) return a.sblock < b.sblock;
        return a.tblock != b.tblock ? a.tblock < b.tblock : a.group < b.group;
      };
    };
    std::stable_sort(entries.begin(), entries.end(), by(s->shape.block_order == 2));
    std::vector<Entry> sentries = entries;
    if (s->shape.block_order == 3) std::stable_sort(sentries.begin(), sentries.end(), by(true));
    // unit copies first (the light kernel; those without a factor column
    // first of all), then the stencils
    for (int pass = 0; pass < 2; ++pass) {
      for (const Entry &e : entries) {
        const tam::DevGroup &g = s->groups[e.group];
        if (tile_pass(g) != pass) continue;
        const int box = g.n[0] * g.n[1] * g.n[2];
        for (int i0 = 0; i0 < box; i0 += ti) {
          tiles.push_back({e.group, e.transfer, i0, std::min(ti, box - i0)});
          keys.push_back(0);
        }
      }
      if (pass == 0) st.ncopy0 = (int64_t)tiles.size() - st.tile0;
      if (pass == 1) st.ncopy = (int64_t)tiles.size() - st.tile0;
    }
    std::vector<tam::Tile> sten;
    std::vector<uint16_t> skeys;
    for (const Entry &e : sentries) {
      const tam::DevGroup &g = s->groups[e.group];
      if (tile_pass(g) != 2) continue;
      if (!s->shape.path_tiles) {  // by target block alone: one key
        const int box = g.n[0] * g.n[1] * g.n[2];
        for (int i0 = 0; i0 < box; i0 += tst) {
          sten.push_back({e.group, e.transfer, i0, std::min(tst, box - i0)});
          skeys.push_back(0);
        }
        continue;
      }
      if (!runs.cache.count(e.group))
        tam::StencilRuns::of(g, s->h_pool_csingle.data(), s->h_pool_perm.data(), s->D,
                             runs.cache[e.group]);
      runs.tiles(e.group, e.transfer, tst, sten, skeys);
    }
    // with TAM_OPT_STAGED, a staged group's tiles go last: the stencil kernel
    // leaves them to the staged kernel, which takes the group's transfers
    // whole (the tiles still list every target, for the adjoint's zeroing)
    const bool staging = s->shape.staged != 0;
    auto is_staged = [&](size_t i) { return staging && s->groups[sten[i].group].staged; };
    std::vector<size_t> order(sten.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](size_t x, size_t y) {
      const bool sx = is_staged(x), sy = is_staged(y);
      return sx != sy ? sy : skeys[x] < skeys[y];
    });
    st.nsten = 0;
    for (size_t i : order) {
      tiles.push_back(sten[i]);
      keys.push_back(skeys[i]);
      if (!is_staged(i)) ++st.nsten;
    }
    st.ntiles = (int64_t)tiles.size() - st.tile0;
    st.staged0 = (int64_t)staged.size();
    st.staged_window = 0;
    if (staging)
      for (const Entry &e : entries) {
        const tam::DevGroup &g = s->groups[e.group];
        if (tile_pass(g) == 2 && g.staged) {
          staged.push_back({e.group, e.transfer, 0, g.n[0] * g.n[1] * g.n[2]});
          st.staged_window =
              std::max<int64_t>(st.staged_window, (int64_t)g.wn[0] * g.wn[1] * g.wn[2]);
        }
      }
    st.nstaged = (int64_t)staged.size() - st.staged0;
  }
}

// The tiles of every stage, then of every stage group, in one array, and
// their staged transfers in `staged`.
std::vector<tam::Tile> build_tiles(tam_sched *s, std::vector<uint16_t> &keys,
                                   std::vector<tam::Tile> &staged) {
  std::vector<tam::Tile> tiles;
  keys.clear();
  staged.clear();
  tam::StencilRuns runs;
  const std::vector<int32_t> rank = block_rank(s);
  tiles_of(s, s->stages, rank, runs, tiles, keys, staged);
  tiles_of(s, s->merged, rank, runs, tiles, keys, staged);
  if (staged.empty()) staged.push_back({0, 0, 0, 0});  // a valid pool even when unused
  return tiles;
}

// Packed tiles of every stage, then of every stage group.
std::vector<tam::PTile> pack_all(tam_sched *s, const std::vector<tam::Tile> &tiles,
                                 const std::vector<uint16_t> &keys) {
  std::vector<tam::PTile> out =
      tam::pack_stages(s->stages, tiles, s->shape.tile_items, &keys, s->shape.stencil_items());
  std::vector<tam::PTile> more =
      tam::pack_stages(s->merged, tiles, s->shape.tile_items, &keys, s->shape.stencil_items());
  for (tam::Stage &m : s->merged) m.ptile0 += (int64_t)out.size();
  out.insert(out.end(), more.begin(), more.end());
  return out;
}

// The stage groups (src/schedule.jl:2735-2931, stage_groups): after phase 1,
// a prolongation stage joins the group of the stage below it when its tag is
// the next one, none of its groups is turned or bounded (those run in
// launches of their own), and none of its points conflicts with a stage
// already in the group: nothing it reads or writes is written by one of
// them, and nothing it writes is read by one.  Per block, every group's
// target box is a write and its source window (the srcstart range widened
// by the order) a read.  Running a group's stages as one launch pair is
// then the same as running them one after another.
void build_stage_groups(tam_sched *s) {
  s->merged.clear();
  s->merged_at.assign(s->stages.size(), -1);
  if (s->nsource != s->nblocks) return;  // a regrid reads another array
  struct Box {
    int32_t lo[3], hi[3];
  };
  auto meets = [](const Box &a, const Box &b) {
    for (int d = 0; d < 3; ++d)
      if (std::max(a.lo[d], b.lo[d]) > std::min(a.hi[d], b.hi[d])) return false;
    return true;
  };
  std::vector<std::vector<Box>> writes(s->nblocks), reads(s->nblocks);
  std::vector<int32_t> touched;
  struct Access {
    int32_t block;
    Box box;
    bool write;
  };
  auto access_of = [&](const tam::Stage &st, std::vector<Access> &out, bool &eligible) {
    out.clear();
    eligible = true;
    for (int32_t gi : st.groups) {
      const tam_group &h = s->host_groups[gi];
      if (h.orientation != 0 || h.bounded != 0) eligible = false;
      Box w{{0, 0, 0}, {0, 0, 0}}, r{{0, 0, 0}, {0, 0, 0}};
      for (int d = 0; d < s->D; ++d) {
        const tam_stencil &sd = h.stencil[d];
        w.lo[d] = sd.targetfirst;
        w.hi[d] = sd.targetfirst + sd.ntarget - 1;
        int32_t lo = INT32_MAX, hi = INT32_MIN;
        for (int i = 0; i < sd.ntarget; ++i) {
          const int32_t v = s->h_srcstart[sd.srcstart + i];
          lo = std::min(lo, v);
          hi = std::max(hi, v);
        }
        r.lo[d] = lo;
        r.hi[d] = hi + sd.order - 1;
      }
      for (int64_t t = h.first; t < h.first + h.ntransfers; ++t) {
        out.push_back({s->h_tb[t] - 1, w, true});
        out.push_back({s->h_sb[t] - 1, r, false});
      }
    }
  };
  std::vector<Access> acc;
  size_t open = SIZE_MAX;  // first stage of the group being formed
  for (size_t i = 0; i < s->stages.size(); ++i) {
    const tam::Stage &st = s->stages[i];
    bool eligible = false;
    if (st.tag > 1) access_of(st, acc, eligible);
    bool joins = eligible && open != SIZE_MAX && st.tag == s->stages[i - 1].tag + 1;
    if (joins) {
      for (const Access &a : acc) {
        for (const Box &b : writes[a.block])
          if (meets(a.box, b)) joins = false;
        if (a.write)
          for (const Box &b : reads[a.block])
            if (meets(a.box, b)) joins = false;
        if (!joins) break;
      }
    }
    if (!joins) {
      // a new group starts here (or none, for an ineligible stage)
      for (int32_t b : touched) {
        writes[b].clear();
        reads[b].clear();
      }
      touched.clear();
      open = eligible ? i : SIZE_MAX;
    }
    if (eligible) {
      for (const Access &a : acc) {
        (a.write ? writes : reads)[a.block].push_back(a.box);
        touched.push_back(a.block);
      }
      if (joins) {
        if (s->merged_at[open] < 0) {
          tam::Stage m;
          m.tag = s->stages[open].tag;
          m.groups = s->stages[open].groups;
          m.span = 1;
          s->merged_at[open] = (int32_t)s->merged.size();
          s->merged.push_back(m);
        }
        tam::Stage &m = s->merged[s->merged_at[open]];
        m.groups.insert(m.groups.end(), st.groups.begin(), st.groups.end());
        m.span += 1;
        m.last_tag = st.tag;
      }
    }
  }
}

// The solo groups of every stage (SoloGroup): turned or bounded.  A turned
// group's axis map is folded into signed strides of the real array, whose
// stored extent along e is R_e = S[perm[e]].  Virtual stored index k
// (1-based) along virtual dimension perm[e] reads real index k, or
// R_e + 1 - k where flip[e], along e; with j = k - 1 the real offset is
//   sum_e stride_e * (flip[e] ? R_e - 1 - j : j),   stride = (1, R_0, R_0 R_1),
// so vs[perm[e]] = +-stride_e and c0 = sum over flipped e of stride_e (R_e - 1).
// An untouched group (a bounded one off the seam) has the identity.
void build_solos(tam_sched *s) {
  s->h_solos.clear();
  for (tam::Stage &st : s->stages) {
    st.solo0 = (int64_t)s->h_solos.size();
    for (int32_t gi : st.groups) {
      const tam_group &h = s->host_groups[gi];
      if (h.orientation == 0 && h.bounded == 0) continue;
      tam::SoloGroup t{};
      t.group = gi;
      t.col = h.orientation;
      t.odd = h.orientation & 1;
      t.bounded = h.bounded;
      // the axis map; an unturned (bounded) group reads in place: the identity
      int perm[3] = {0, 1, 2}, flip[3] = {0, 0, 0};
      if (h.orientation != 0)
        for (int e = 0; e < s->D; ++e) {
          perm[e] = (h.axes >> (2 * e)) & 3;
          flip[e] = (h.axes >> (8 + e)) & 1;
        }
      int R[3] = {1, 1, 1};
      for (int e = 0; e < s->D; ++e) R[e] = s->S[perm[e]];
      const int64_t stride[3] = {1, R[0], (int64_t)R[0] * R[1]};
      t.vs[0] = 1;
      t.vs[1] = stride[1];
      t.vs[2] = stride[2];
      t.c0 = 0;
      for (int e = 0; e < s->D; ++e) {
        t.vs[perm[e]] = flip[e] ? -stride[e] : stride[e];
        if (flip[e]) t.c0 += stride[e] * (R[e] - 1);
      }
      s->h_solos.push_back(t);
    }
    st.nsolo = (int64_t)s->h_solos.size() - st.solo0;
  }
}

}  // namespace

namespace tam {

cudaError_t fill_one_stage(tam_sched *s, void *work, int nvars, const void *factors,
                           int32_t tag, cudaStream_t stream) {
  const SchedArgs args = sched_args(s);
  for (const Stage &stage : s->stages) {
    if (stage.tag != tag) continue;
    if (stage.nsolo > 0) return cudaErrorNotSupported;  // no turned or bounded group here
    cudaError_t e = launch_fused_stage(s->dtype, s->D, s->d_tiles, s->d_ptiles, stage, args,
                                       work, factors, nvars, s->S, s->shape.threads, stream,
                                       &s->side, nullptr, s->d_staged);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace tam

extern "C" {

int tam_abi_version(void) { return TAM_ABI_VERSION; }

int tam_init(int device, tam_ctx **out) {
  if (!out) return fail(nullptr, TAM_EINVAL, "tam_init: out is NULL");
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaGetDeviceCount");
  if (device < 0 || device >= n) return fail(nullptr, TAM_EINVAL, "no such CUDA device");
  tam_ctx *ctx = new (std::nothrow) tam_ctx;
  if (!ctx) return fail(nullptr, TAM_ENOMEM, "out of host memory");
  ctx->device = device;
  e = cudaDeviceGetAttribute(&ctx->nsm, cudaDevAttrMultiProcessorCount, device);
  if (e != cudaSuccess) {
    delete ctx;
    return cuda_fail(nullptr, e, "cudaDeviceGetAttribute");
  }
  *out = ctx;
  return TAM_OK;
}

void tam_free(tam_ctx *ctx) { delete ctx; }

int tam_last_error(const tam_ctx *ctx, char *buf, size_t n) {
  if (!buf || n == 0) return TAM_EINVAL;
  std::string msg;
  if (ctx) {
    msg = ctx->err;
  } else {
    std::lock_guard<std::mutex> lock(g_err_mutex);
    msg = g_err;
  }
  size_t k = std::min(n - 1, msg.size());
  memcpy(buf, msg.data(), k);
  buf[k] = 0;
  return TAM_OK;
}

static int schedule_upload(tam_ctx *ctx, const tam_schedule_desc *d, int64_t nsource,
                           tam_sched **out);

int tam_schedule_upload(tam_ctx *ctx, const tam_schedule_desc *d, tam_sched **out) {
  if (!ctx || !out || !d) return fail(ctx, TAM_EINVAL, "tam_schedule_upload: NULL argument");
  return schedule_upload(ctx, d, d->nblocks, out);
}

int tam_regrid_upload(tam_ctx *ctx, const tam_schedule_desc *d, int64_t old_nblocks,
                      tam_sched **out) {
  if (!ctx || !out || !d) return fail(ctx, TAM_EINVAL, "tam_regrid_upload: NULL argument");
  return schedule_upload(ctx, d, old_nblocks, out);
}

static int schedule_upload(tam_ctx *ctx, const tam_schedule_desc *d, int64_t nsource,
                           tam_sched **out) {
  *out = nullptr;
  int rc = validate(ctx, d, nsource);
  if (rc != TAM_OK) return rc;
  DeviceGuard guard(ctx->device);
  if (!guard.ok()) return fail(ctx, TAM_ECUDA, "cannot make the context's device current");

  tam_sched *s = new (std::nothrow) tam_sched;
  if (!s) return fail(ctx, TAM_ENOMEM, "out of host memory");
  s->ctx = ctx;
  s->D = d->ndim;
  s->dtype = d->dtype;
  for (int k = 0; k < 3; ++k) s->S[k] = k < d->ndim ? d->stored[k] : 1;
  s->nblocks = d->nblocks;
  s->nsource = nsource;
  s->nfactorcols = d->nfactorcols;
  s->ntransfers = d->ntransfers;
  s->host_groups.assign(d->groups, d->groups + d->ngroups);

  // Device groups, with a unit pad entry (srcstart 1, weight 1) for the
  // dimensions beyond D.
  std::vector<int32_t> srcstart(d->srcstart, d->srcstart + d->nsrcstart);
  const int64_t pad_ss = (int64_t)srcstart.size();
  srcstart.push_back(1);
  const size_t esz = d->dtype == TAM_F64 ? 8 : 4;
  std::vector<unsigned char> weights((size_t)(d->nweights + 1) * esz);
  if (d->nweights) memcpy(weights.data(), d->weights, (size_t)d->nweights * esz);
  const int64_t pad_w = d->nweights;
  if (d->dtype == TAM_F64) {
    double one = 1.0;
    memcpy(weights.data() + pad_w * esz, &one, esz);
  } else {
    float one = 1.0f;
    memcpy(weights.data() + pad_w * esz, &one, esz);
  }

  s->groups.resize(d->ngroups);
  std::vector<int32_t> cls;
  std::vector<unsigned char> wtab;
  std::vector<int32_t> csingle(1, -1), perm(1, 0);  // a valid pool even when unused
  for (int32_t gi = 0; gi < d->ngroups; ++gi) {
    const tam_group &h = d->groups[gi];
    tam::DevGroup &g = s->groups[gi];
    memset(&g, 0, sizeof g);
    bool unit = true, uniform = true;
    int p0 = h.stencil[0].order;
    for (int k = 0; k < 3; ++k) {
      if (k < d->ndim) {
        const tam_stencil &st = h.stencil[k];
        g.n[k] = st.ntarget;
        g.tf[k] = st.targetfirst - 1;
        g.order[k] = st.order;
        g.ss[k] = st.srcstart;
        g.w[k] = st.weights;
        unit = unit && st.unit;
        uniform = uniform && st.order == p0;
      } else {
        g.n[k] = 1;
        g.tf[k] = 0;
        g.order[k] = 1;
        g.ss[k] = pad_ss;
        g.w[k] = pad_w;
      }
    }
    g.unit = unit ? 1 : 0;
    g.factorcol = h.factorcol;
    g.pclass = unit ? 0 : (uniform && (p0 == 2 || p0 == 3 || p0 == 4 || p0 == 6)) ? p0 : -1;
    g.first = h.first;
    g.ntransfers = h.ntransfers;
    g.turned = (h.orientation != 0 || h.bounded != 0) ? 1 : 0;
    if (h.orientation != 0) s->needs_rotvars = true;
    if (h.bounded != 0) s->has_bounded = true;
    if (h.factorcol != 0) s->needs_factors = true;
    s->points += (int64_t)g.n[0] * g.n[1] * g.n[2] * g.ntransfers;
    // the division-free box decomposition
    {
      const uint64_t n1 = (uint64_t)g.n[0], n12 = n1 * (uint64_t)g.n[1];
      const uint64_t box = n12 * (uint64_t)g.n[2];
      g.mag1 = g.mag12 = 0;
      if (box * n1 < (1ull << 32) && box * n12 < (1ull << 32)) {
        g.mag1 = (uint32_t)(((1ull << 32) + n1 - 1) / n1);
        g.mag12 = (uint32_t)(((1ull << 32) + n12 - 1) / n12);
        if (n1 == 1) g.mag1 = 0;    // 2^32 does not fit: divide
        if (n12 == 1) g.mag12 = 0;
      }
    }
    // affine unit copies
    g.affine = 0;
    if (g.pclass == 0) {
      bool aff = true;
      for (int k = 0; k < 3; ++k) {
        const int32_t *ssk = srcstart.data() + g.ss[k];
        const int n = g.n[k];
        const int32_t step = n > 1 ? ssk[1] - ssk[0] : 0;
        aff = aff && step >= -1 && step <= 1;
        for (int i = 1; i < n && aff; ++i) aff = ssk[i] - ssk[0] == step * i;
        g.cs0[k] = ssk[0] - 1;
        g.cstep[k] = step;
      }
      g.affine = aff ? 1 : 0;
    }
    for (int k = 0; k < 3; ++k) g.C[k] = 1;
    for (int k = 0; k < 3; ++k) g.csingle[k] = 0;
    g.perm = -1;
    if (g.pclass > 1) {
      if (d->dtype == TAM_F64)
        build_product_table<double>(d, h, g, cls, wtab);
      else
        build_product_table<float>(d, h, g, cls, wtab);
    }
    if (g.pclass != 0) {
      if (d->dtype == TAM_F64)
        build_singles<double>(d, h, g, csingle, perm);
      else
        build_singles<float>(d, h, g, csingle, perm);
    }
    // the source window, and whether the staged kernel takes the group
    int64_t wvol = 1;
    for (int k = 0; k < 3; ++k) {
      g.wlo[k] = 0;
      g.wn[k] = 1;
      if (k >= d->ndim) continue;
      const tam_stencil &sd = h.stencil[k];
      int32_t lo = INT32_MAX, hi = INT32_MIN;
      for (int i = 0; i < sd.ntarget; ++i) {
        lo = std::min(lo, d->srcstart[sd.srcstart + i]);
        hi = std::max(hi, d->srcstart[sd.srcstart + i]);
      }
      if (sd.ntarget > 0) {
        g.wlo[k] = lo - 1;
        g.wn[k] = hi - lo + sd.order;
      }
      wvol *= g.wn[k];
    }
    const int64_t box = (int64_t)g.n[0] * g.n[1] * g.n[2];
    g.staged = g.pclass != 0 && h.orientation == 0 && h.bounded == 0 &&
               box >= tam::kStagedMinBox &&
               wvol * (d->dtype == TAM_F64 ? 8 : 4) <= tam::kStagedBytes;
  }

  // Stages in tag order, and the fused tiles of each: ordered by target
  // block, then group, then box position.
  std::map<int32_t, std::vector<int32_t>> bytag;
  for (int32_t gi = 0; gi < d->ngroups; ++gi) bytag[d->groups[gi].stage].push_back(gi);
  for (auto &kv : bytag) {
    tam::Stage st;
    st.tag = kv.first;
    st.groups = kv.second;
    s->stages.push_back(st);
  }
  s->h_tb.assign(d->targetblocks, d->targetblocks + d->ntransfers);
  s->h_sb.assign(d->sourceblocks, d->sourceblocks + d->ntransfers);
  s->h_srcstart.assign(d->srcstart, d->srcstart + d->nsrcstart);
  s->h_pool_csingle = std::move(csingle);
  s->h_pool_perm = std::move(perm);
  // Float64 stencils are bound by the FP64 pipe, which a divergent warp
  // wastes; Float32 ones by memory, which the blocks' order serves best
  s->shape.path_tiles = d->dtype == TAM_F64 ? 1 : 0;
  build_stage_groups(s);
  std::vector<uint16_t> keys;
  std::vector<tam::Tile> staged;
  std::vector<tam::Tile> tiles = build_tiles(s, keys, staged);
  std::vector<tam::PTile> ptiles = pack_all(s, tiles, keys);
  build_solos(s);
  std::vector<uint64_t> wshort;
  if (d->dtype == TAM_F64) wshort = tam::short_weights(wtab);
  if (wshort.empty()) wshort.push_back(0);

  cudaError_t e;
  if ((e = tam::side_create(s->side)) != cudaSuccess ||
      (e = upload(&s->d_solos, s->h_solos.data(), s->h_solos.size())) != cudaSuccess ||
      (e = upload(&s->d_ptiles, ptiles.data(), ptiles.size())) != cudaSuccess ||
      (e = upload(&s->d_groups, s->groups.data(), s->groups.size())) != cudaSuccess ||
      (e = upload(&s->d_tb, d->targetblocks, (size_t)d->ntransfers)) != cudaSuccess ||
      (e = upload(&s->d_sb, d->sourceblocks, (size_t)d->ntransfers)) != cudaSuccess ||
      (e = upload(&s->d_srcstart, srcstart.data(), srcstart.size())) != cudaSuccess ||
      (e = upload((unsigned char **)&s->d_weights, weights.data(), weights.size())) !=
          cudaSuccess ||
      (e = upload(&s->d_tiles, tiles.data(), tiles.size())) != cudaSuccess ||
      (e = upload(&s->d_staged, staged.data(), staged.size())) != cudaSuccess ||
      (e = upload(&s->d_cls, cls.data(), cls.size())) != cudaSuccess ||
      (e = upload((unsigned char **)&s->d_wtab, wtab.data(), wtab.size())) != cudaSuccess ||
      (e = upload(&s->d_wshort, wshort.data(), wshort.size())) != cudaSuccess ||
      (e = upload(&s->d_csingle, s->h_pool_csingle.data(), s->h_pool_csingle.size())) !=
          cudaSuccess ||
      (e = upload(&s->d_perm, s->h_pool_perm.data(), s->h_pool_perm.size())) != cudaSuccess ||
      (e = upload(&s->d_err, (const int32_t *)nullptr, 1)) != cudaSuccess) {
    free_sched_device(s);
    delete s;
    return e == cudaErrorMemoryAllocation ? fail(ctx, TAM_ENOMEM, "device allocation failed")
                                          : cuda_fail(ctx, e, "schedule upload");
  }
  // host copies of the pools, for a batch of forests (tam_batch_create)
  s->h_pool_srcstart = std::move(srcstart);
  s->h_pool_weights = std::move(weights);
  s->h_pool_cls = std::move(cls);
  s->h_pool_wtab = std::move(wtab);
  *out = s;
  return TAM_OK;
}

void tam_schedule_free(tam_sched *s) {
  if (!s) return;
  DeviceGuard guard(s->ctx->device);
  tam::adjoint_free(s);
  free_sched_device(s);
  delete s;
}

// Whether odd turns read another array than the set's own: a RotationPair
// member, whose layout is not symmetric in the seam's plane.
static bool reads_partner(const tam_sched *s) {
  for (const tam_group &h : s->host_groups) {
    if (!(h.orientation & 1)) continue;
    for (int e = 0; e < s->D; ++e)
      if (s->S[(h.axes >> (2 * e)) & 3] != s->S[e]) return true;
  }
  return false;
}

static int adjoint_ready(tam_sched *s) {
  if (s->adj.ready) return TAM_OK;
  if (s->has_bounded)
    return fail(s->ctx, TAM_EUNSUPPORTED,
                "a schedule with bounded operators is not linear, so it has no adjoint");
  std::string err;
  int rc = tam::adjoint_prepare(s, err);
  if (rc != TAM_OK) return fail(s->ctx, rc, err);
  return TAM_OK;
}

int tam_adjoint_scratch_bytes(tam_sched *s, int32_t nvars, size_t *bytes) {
  if (!s || !bytes || nvars < 1) return fail(s ? s->ctx : nullptr, TAM_EINVAL,
                                             "tam_adjoint_scratch_bytes: bad argument");
  DeviceGuard guard(s->ctx->device);
  int rc = adjoint_ready(s);
  if (rc != TAM_OK) return rc;
  *bytes = (size_t)s->adj.scratch_points * nvars * (s->dtype == TAM_F64 ? 8 : 4);
  return TAM_OK;
}

static int check_fill_args(tam_sched *s, void *work, int32_t nvars, int64_t nblocks,
                           const void *factors);
static int owned_adjoint(tam_sched *s, void *y, void *alt, int32_t nvars, int64_t nblocks,
                         const void *factors, const int32_t *rotvars, int32_t first_stage,
                         int32_t last_stage, void *stream);

// A turned group's transpose adds onto the array its forward fill read: the
// set's own, or for odd turns of a RotationPair member the partner's.
static int check_partner(tam_sched *s, const void *alt) {
  if (!alt && reads_partner(s))
    return fail(s->ctx, TAM_EUNSUPPORTED,
                "this is a RotationPair member (a layout not symmetric in the seam's plane): "
                "its adjoint adds onto the partner's array, so use tam_fill_adjoint_alt");
  return TAM_OK;
}

// The adjoint with the caller's scratch (which may be NULL only when the
// schedule needs none).
static int adjoint_with(tam_sched *s, void *y, void *alt, int32_t nvars, int64_t nblocks,
                        const void *factors, const int32_t *rotvars, int32_t first_stage,
                        int32_t last_stage, void *scratch, size_t scratch_bytes, void *stream) {
  int rc = check_fill_args(s, y, nvars, nblocks, factors);
  if (rc != TAM_OK) return rc;
  rc = check_partner(s, alt);
  if (rc != TAM_OK) return rc;
  if (s->needs_rotvars && !rotvars)
    return fail(s->ctx, TAM_EINVAL,
                "this schedule turns ghosts across a rotating seam, but no variable table was "
                "given: use tam_fill_adjoint_ex");
  DeviceGuard guard(s->ctx->device);
  if (!guard.ok()) return fail(s->ctx, TAM_ECUDA, "cannot make the context's device current");
  rc = adjoint_ready(s);
  if (rc != TAM_OK) return rc;
  const size_t need = (size_t)s->adj.scratch_points * nvars * (s->dtype == TAM_F64 ? 8 : 4);
  if (need > 0 && (!scratch || scratch_bytes < need))
    return fail(s->ctx, TAM_EINVAL, "adjoint scratch smaller than tam_adjoint_scratch_bytes");
  cudaError_t e = tam::adjoint_run(s, y, alt, nvars, factors, rotvars, first_stage, last_stage,
                                   scratch, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(s->ctx, e, "adjoint launch");
  return TAM_OK;
}

int tam_fill_adjoint_scratch(tam_sched *s, void *y, int32_t nvars, int64_t nblocks,
                             const void *factors, int32_t first_stage, int32_t last_stage,
                             void *scratch, size_t scratch_bytes, void *stream) {
  return adjoint_with(s, y, nullptr, nvars, nblocks, factors, nullptr, first_stage, last_stage,
                      scratch, scratch_bytes, stream);
}

int tam_fill_adjoint_ex(tam_sched *s, void *y, int32_t nvars, int64_t nblocks,
                        const void *factors, const int32_t *rotvars, int32_t first_stage,
                        int32_t last_stage, void *scratch, size_t scratch_bytes, void *stream) {
  return tam_fill_adjoint_alt(s, y, nullptr, nvars, nblocks, factors, rotvars, first_stage,
                              last_stage, scratch, scratch_bytes, stream);
}

int tam_fill_adjoint_alt(tam_sched *s, void *y, void *alt_y, int32_t nvars, int64_t nblocks,
                         const void *factors, const int32_t *rotvars, int32_t first_stage,
                         int32_t last_stage, void *scratch, size_t scratch_bytes, void *stream) {
  if (!scratch) {
    int rc = check_fill_args(s, y, nvars, nblocks, factors);
    if (rc != TAM_OK) return rc;
    return owned_adjoint(s, y, alt_y, nvars, nblocks, factors, rotvars, first_stage,
                         last_stage, stream);
  }
  return adjoint_with(s, y, alt_y, nvars, nblocks, factors, rotvars, first_stage, last_stage,
                      scratch, scratch_bytes, stream);
}

int tam_fill_adjoint(tam_sched *s, void *y, int32_t nvars, int64_t nblocks, const void *factors,
                     int32_t first_stage, int32_t last_stage, void *stream) {
  return tam_fill_adjoint_ex(s, y, nvars, nblocks, factors, nullptr, first_stage, last_stage,
                             nullptr, 0, stream);
}

// The adjoint with the library's own scratch, grown on demand.
static int owned_adjoint(tam_sched *s, void *y, void *alt, int32_t nvars, int64_t nblocks,
                         const void *factors, const int32_t *rotvars, int32_t first_stage,
                         int32_t last_stage, void *stream) {
  int rc0 = check_partner(s, alt);
  if (rc0 != TAM_OK) return rc0;
  if (s->needs_rotvars && !rotvars)
    return fail(s->ctx, TAM_EINVAL,
                "this schedule turns ghosts across a rotating seam, but no variable table was "
                "given: use tam_fill_adjoint_ex");
  DeviceGuard guard(s->ctx->device);
  if (!guard.ok()) return fail(s->ctx, TAM_ECUDA, "cannot make the context's device current");
  int rc = adjoint_ready(s);
  if (rc != TAM_OK) return rc;
  const size_t need = (size_t)s->adj.scratch_points * nvars * (s->dtype == TAM_F64 ? 8 : 4);
  if (need > s->adj_scratch_bytes) {
    // grown only between fills: wait for any fill still using the old one
    cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(s->ctx, e, "adjoint scratch");
    cudaFree(s->adj_scratch);
    s->adj_scratch = nullptr;
    s->adj_scratch_bytes = 0;
    e = cudaMalloc(&s->adj_scratch, need);
    if (e != cudaSuccess) return fail(s->ctx, TAM_ENOMEM, "adjoint scratch allocation failed");
    s->adj_scratch_bytes = need;
  }
  return adjoint_with(s, y, alt, nvars, nblocks, factors, rotvars, first_stage, last_stage,
                      s->adj_scratch, s->adj_scratch_bytes, stream);
}

int tam_schedule_stage_groups(const tam_sched *s, int32_t *groups, int32_t *stages_in_groups) {
  if (!s) return fail(nullptr, TAM_EINVAL, "tam_schedule_stage_groups: NULL schedule");
  int32_t n = 0;
  for (const tam::Stage &m : s->merged) n += m.span;
  if (groups) *groups = (int32_t)s->merged.size();
  if (stages_in_groups) *stages_in_groups = n;
  return TAM_OK;
}

int tam_schedule_info(const tam_sched *s, int64_t *ngroups, int64_t *ntransfers, int64_t *points,
                      int32_t *nstages) {
  if (!s) return fail(nullptr, TAM_EINVAL, "tam_schedule_info: NULL schedule");
  if (ngroups) *ngroups = (int64_t)s->groups.size();
  if (ntransfers) *ntransfers = s->ntransfers;
  if (points) *points = s->points;
  if (nstages) *nstages = (int32_t)s->stages.size();
  return TAM_OK;
}

static int check_fill_args(tam_sched *s, void *work, int32_t nvars, int64_t nblocks,
                           const void *factors) {
  if (!s) return fail(nullptr, TAM_EINVAL, "fill: NULL schedule");
  tam_ctx *ctx = s->ctx;
  if (!work) return fail(ctx, TAM_EINVAL, "fill: work is NULL");
  if (nvars < 1) return fail(ctx, TAM_EINVAL, "fill: nvars must be positive");
  if (nblocks != s->nblocks)
    return fail(ctx, TAM_ELAYOUT, "fill: the field set's block count differs from the schedule's");
  if (s->needs_factors && !factors)
    return fail(ctx, TAM_EINVAL,
                "this schedule mirrors ghosts across a reflecting face, but no factor table "
                "was given (src/ghosts.jl:426-429)");
  return TAM_OK;
}

int tam_fill(tam_sched *s, void *work, int32_t nvars, int64_t nblocks, const void *factors,
             int32_t first_stage, int32_t last_stage, void *stream) {
  return tam_fill_ex(s, work, nullptr, nvars, nblocks, factors, nullptr, first_stage,
                     last_stage, TAM_METHOD_FUSED, stream);
}

int tam_fill_ex(tam_sched *s, void *work, const void *alt_work, int32_t nvars, int64_t nblocks,
                const void *factors, const int32_t *rotvars, int32_t first_stage,
                int32_t last_stage, int32_t method, void *stream) {
  int rc = check_fill_args(s, work, nvars, nblocks, factors);
  if (rc != TAM_OK) return rc;
  if (method != TAM_METHOD_FUSED && method != TAM_METHOD_PLAIN)
    return fail(s->ctx, TAM_EINVAL, "method must be TAM_METHOD_FUSED or TAM_METHOD_PLAIN");
  if (s->needs_rotvars && !rotvars)
    return fail(s->ctx, TAM_EINVAL,
                "this schedule turns ghosts across a rotating seam, but no variable table was "
                "given to turn them with (src/ghosts.jl:431-434)");
  DeviceGuard guard(s->ctx->device);
  if (!guard.ok()) return fail(s->ctx, TAM_ECUDA, "cannot make the context's device current");
  cudaStream_t st = (cudaStream_t)stream;
  tam::SchedArgs args = sched_args(s);
  if (method == TAM_METHOD_PLAIN) args.one_tap = 0;  // the device form
  for (size_t i = 0; i < s->stages.size(); ++i) {
    const tam::Stage &stage = s->stages[i];
    if (stage.tag < first_stage || stage.tag > last_stage) continue;
    cudaError_t e = cudaSuccess;
    const int32_t mi = s->merged_at.empty() ? -1 : s->merged_at[i];
    if (method == TAM_METHOD_FUSED && s->shape.merge_stages && mi >= 0 &&
        s->merged[mi].last_tag <= last_stage) {
      // a stage group inside the range: one launch pair for all its stages
      const tam::Stage &m = s->merged[mi];
      e = tam::launch_fused_stage(s->dtype, s->D, s->d_tiles, s->d_ptiles, m, args, work,
                                  factors, nvars, s->S, s->shape.threads, st, &s->side, nullptr,
                                  s->d_staged);
      if (e != cudaSuccess) return cuda_fail(s->ctx, e, "fused stage-group launch");
      i += m.span - 1;
      continue;
    }
    if (method == TAM_METHOD_FUSED) {
      e = tam::launch_fused_stage(s->dtype, s->D, s->d_tiles, s->d_ptiles, stage, args, work,
                                  factors, nvars, s->S, s->shape.threads, st, &s->side, nullptr,
                                  s->d_staged);
      if (e != cudaSuccess) return cuda_fail(s->ctx, e, "fused stage launch");
    } else {
      for (int32_t gi : stage.groups) {
        if (s->groups[gi].turned) continue;
        e = tam::launch_plain_group(s->dtype, s->D, s->groups[gi], s->d_groups + gi, args,
                                    work, factors, nvars, s->S, st);
        if (e != cudaSuccess) return cuda_fail(s->ctx, e, "plain group launch");
      }
    }
    if (stage.nsolo > 0) {
      e = tam::launch_solo(s->dtype, s->D, s->d_solos + stage.solo0, stage.nsolo, args, work,
                             alt_work ? alt_work : work, work, factors, rotvars, nvars, s->S,
                             s->d_err, st);
      if (e != cudaSuccess) return cuda_fail(s->ctx, e, "turned group launch");
    }
  }
  return TAM_OK;
}

int tam_fill_host(tam_sched *s, const void *host_in, void *host_out, void *device_work,
                  int32_t nvars, int64_t nblocks, const void *factors, int32_t first_stage,
                  int32_t last_stage, void *stream) {
  if (!host_in || !host_out)
    return fail(s ? s->ctx : nullptr, TAM_EINVAL, "tam_fill_host: NULL host buffer");
  int rc = check_fill_args(s, device_work, nvars, nblocks, factors);
  if (rc != TAM_OK) return rc;
  DeviceGuard guard(s->ctx->device);
  if (!guard.ok()) return fail(s->ctx, TAM_ECUDA, "cannot make the context's device current");
  const size_t bytes = (size_t)nblocks * nvars * s->S[0] * s->S[1] * s->S[2] *
                       (s->dtype == TAM_F64 ? 8 : 4);
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = cudaMemcpyAsync(device_work, host_in, bytes, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return cuda_fail(s->ctx, e, "tam_fill_host upload");
  rc = tam_fill(s, device_work, nvars, nblocks, factors, first_stage, last_stage, stream);
  if (rc != TAM_OK) return rc;
  e = cudaMemcpyAsync(host_out, device_work, bytes, cudaMemcpyDeviceToHost, st);
  if (e != cudaSuccess) return cuda_fail(s->ctx, e, "tam_fill_host download");
  return TAM_OK;
}

int tam_fill_host_own(tam_sched *s, const tam_state_layout *layout, const void *host_in,
                      void *host_out, void *device_work, int32_t nvars, int64_t nblocks,
                      const void *factors, int32_t first_stage, int32_t last_stage,
                      void *stream) {
  if (!host_in || !host_out || !layout)
    return fail(s ? s->ctx : nullptr, TAM_EINVAL, "tam_fill_host_own: NULL argument");
  int rc = check_fill_args(s, device_work, nvars, nblocks, factors);
  if (rc != TAM_OK) return rc;
  if (layout->dtype != s->dtype || layout->ndim != s->D || layout->nvars != nvars ||
      layout->nblocks != nblocks)
    return fail(s->ctx, TAM_ELAYOUT, "tam_fill_host_own: the layout is not the schedule's");
  for (int d = 0; d < s->D; ++d)
    if (layout->stored[d] != s->S[d])
      return fail(s->ctx, TAM_ELAYOUT,
                  "tam_fill_host_own: the layout's stored extents are not the schedule's");
  DeviceGuard guard(s->ctx->device);
  if (!guard.ok()) return fail(s->ctx, TAM_ECUDA, "cannot make the context's device current");
  // the kernel reads host_in through its device mapping: page-locked memory
  cudaPointerAttributes attr;
  cudaError_t e = cudaPointerGetAttributes(&attr, host_in);
  if (e != cudaSuccess || attr.type != cudaMemoryTypeHost || !attr.devicePointer) {
    cudaGetLastError();
    return fail(s->ctx, TAM_EINVAL,
                "tam_fill_host_own: host_in must be page-locked host memory (cudaHostAlloc "
                "or cudaHostRegister), which the upload kernel reads directly");
  }
  rc = tam::own_box_copy(layout, device_work, attr.devicePointer, stream);
  if (rc != TAM_OK) return fail(s->ctx, rc, "tam_fill_host_own: own-point upload");
  rc = tam_fill(s, device_work, nvars, nblocks, factors, first_stage, last_stage, stream);
  if (rc != TAM_OK) return rc;
  const size_t bytes = (size_t)nblocks * nvars * s->S[0] * s->S[1] * s->S[2] *
                       (s->dtype == TAM_F64 ? 8 : 4);
  e = cudaMemcpyAsync(host_out, device_work, bytes, cudaMemcpyDeviceToHost,
                      (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(s->ctx, e, "tam_fill_host_own download");
  return TAM_OK;
}

int tam_regrid_transfer(tam_sched *s, const void *old_work, int64_t old_nblocks,
                        void *new_work, int64_t new_nblocks, int32_t nvars, void *stream) {
  if (!s || !old_work || !new_work)
    return fail(s ? s->ctx : nullptr, TAM_EINVAL, "tam_regrid_transfer: NULL argument");
  if (nvars < 1) return fail(s->ctx, TAM_EINVAL, "tam_regrid_transfer: nvars must be positive");
  if (new_nblocks != s->nblocks || old_nblocks != s->nsource)
    return fail(s->ctx, TAM_ELAYOUT,
                "tam_regrid_transfer: the block counts differ from the transfer's");
  if (s->needs_factors || s->needs_rotvars)
    return fail(s->ctx, TAM_EUNSUPPORTED, "a regrid transfer takes no factor column and no turn");
  if (old_work == new_work)
    return fail(s->ctx, TAM_EINVAL, "tam_regrid_transfer: the old and new arrays must differ");
  DeviceGuard guard(s->ctx->device);
  if (!guard.ok()) return fail(s->ctx, TAM_ECUDA, "cannot make the context's device current");
  cudaStream_t st = (cudaStream_t)stream;
  for (const tam::Stage &stage : s->stages) {
    cudaError_t e = tam::launch_fused_stage(s->dtype, s->D, s->d_tiles, s->d_ptiles, stage,
                                            sched_args(s), new_work, nullptr, nvars, s->S,
                                            s->shape.threads, st, &s->side, old_work,
                                            s->d_staged);
    if (e != cudaSuccess) return cuda_fail(s->ctx, e, "regrid transfer launch");
    if (stage.nsolo > 0) {  // bounded children
      e = tam::launch_solo(s->dtype, s->D, s->d_solos + stage.solo0, stage.nsolo, sched_args(s),
                           old_work, old_work, new_work, nullptr, nullptr, nvars, s->S, s->d_err,
                           st);
      if (e != cudaSuccess) return cuda_fail(s->ctx, e, "regrid transfer launch");
    }
  }
  return TAM_OK;
}

int tam_fill_plain(tam_sched *s, void *work, int32_t nvars, int64_t nblocks, const void *factors,
                   int32_t first_stage, int32_t last_stage, void *stream) {
  return tam_fill_ex(s, work, nullptr, nvars, nblocks, factors, nullptr, first_stage,
                     last_stage, TAM_METHOD_PLAIN, stream);
}

int tam_schedule_set_option(tam_sched *s, int32_t option, int64_t value) {
  if (!s) return fail(nullptr, TAM_EINVAL, "tam_schedule_set_option: NULL schedule");
  switch (option) {
    case TAM_OPT_TILE_ITEMS:
    case TAM_OPT_STENCIL_TILE:
    case TAM_OPT_BLOCK_ORDER:
    case TAM_OPT_PATH_TILES:
    case TAM_OPT_STAGED: {
      int *field = option == TAM_OPT_TILE_ITEMS     ? &s->shape.tile_items
                   : option == TAM_OPT_STENCIL_TILE ? &s->shape.stencil_tile
                   : option == TAM_OPT_BLOCK_ORDER  ? &s->shape.block_order
                   : option == TAM_OPT_PATH_TILES   ? &s->shape.path_tiles
                                                    : &s->shape.staged;
      if (option == TAM_OPT_TILE_ITEMS && (value < 16 || value > 4096))
        return fail(s->ctx, TAM_EINVAL, "tile items must be in 16..4096");
      if (option == TAM_OPT_STENCIL_TILE && value != 0 && (value < 16 || value > 4096))
        return fail(s->ctx, TAM_EINVAL, "stencil tile items are 0 or in 16..4096");
      if (option == TAM_OPT_BLOCK_ORDER && (value < 0 || value > 3))
        return fail(s->ctx, TAM_EINVAL, "block_order is 0..3");
      if ((option == TAM_OPT_PATH_TILES || option == TAM_OPT_STAGED) && value != 0 &&
          value != 1)
        return fail(s->ctx, TAM_EINVAL, "path_tiles and staged are 0 or 1");
      if (value == *field) return TAM_OK;
      DeviceGuard guard(s->ctx->device);
      const int old = *field;
      *field = (int)value;
      std::vector<uint16_t> keys;
      std::vector<tam::Tile> staged;
      std::vector<tam::Tile> tiles = build_tiles(s, keys, staged);
      std::vector<tam::PTile> ptiles = pack_all(s, tiles, keys);
      tam::Tile *d = nullptr, *dst = nullptr;
      tam::PTile *dp = nullptr;
      cudaError_t e = upload(&d, tiles.data(), tiles.size());
      if (e == cudaSuccess) e = upload(&dp, ptiles.data(), ptiles.size());
      if (e == cudaSuccess) e = upload(&dst, staged.data(), staged.size());
      if (e != cudaSuccess) {
        cudaFree(d);
        cudaFree(dp);
        cudaFree(dst);
        *field = old;
        std::vector<tam::Tile> back = build_tiles(s, keys, staged);
        pack_all(s, back, keys);
        return cuda_fail(s->ctx, e, "re-tiling");
      }
      cudaDeviceSynchronize();  // no fill may still read the old tiles
      cudaFree(s->d_tiles);
      cudaFree(s->d_ptiles);
      cudaFree(s->d_staged);
      s->d_tiles = d;
      s->d_ptiles = dp;
      s->d_staged = dst;
      return TAM_OK;
    }
    case TAM_OPT_THREADS:
      if (value < 64 || value > 512 || value % 32)
        return fail(s->ctx, TAM_EINVAL, "threads must be a multiple of 32 in 64..512");
      s->shape.threads = (int)value;
      return TAM_OK;
    case TAM_OPT_INT_MUL:
      if (value != 0 && value != 1) return fail(s->ctx, TAM_EINVAL, "int_mul is 0 or 1");
      s->shape.int_mul = (int)value;
      return TAM_OK;
    case TAM_OPT_ONE_TAP:
      if (value != 0 && value != 1) return fail(s->ctx, TAM_EINVAL, "one_tap is 0 or 1");
      s->shape.one_tap = (int)value;
      return TAM_OK;
    case TAM_OPT_PAIR_VARS:
      if (value != 0 && value != 1) return fail(s->ctx, TAM_EINVAL, "pair_vars is 0 or 1");
      s->shape.pair_vars = (int)value;
      return TAM_OK;
    case TAM_OPT_MERGE_STAGES:
      if (value != 0 && value != 1) return fail(s->ctx, TAM_EINVAL, "merge_stages is 0 or 1");
      s->shape.merge_stages = (int)value;
      return TAM_OK;
    case TAM_OPT_COPY_POINTS:
      if (value != 1 && value != 2 && value != 4)
        return fail(s->ctx, TAM_EINVAL, "copy_points is 1, 2 or 4");
      s->shape.copy_points = (int)value;
      return TAM_OK;
    case TAM_OPT_COPY_SHARE:
      if (value < 0 || value > 32) return fail(s->ctx, TAM_EINVAL, "copy_share is 0..32");
      s->shape.copy_share = (int)value;
      return TAM_OK;
    case TAM_OPT_SOFT_ADD:
      if (value != 0 && value != 1) return fail(s->ctx, TAM_EINVAL, "soft_add is 0 or 1");
      s->shape.soft_add = (int)value;
      return TAM_OK;
    default:
      return fail(s->ctx, TAM_EINVAL, "unknown option");
  }
}

int tam_schedule_get_option(const tam_sched *s, int32_t option, int64_t *value) {
  if (!s || !value) return fail(nullptr, TAM_EINVAL, "tam_schedule_get_option: NULL argument");
  switch (option) {
    case TAM_OPT_TILE_ITEMS: *value = s->shape.tile_items; return TAM_OK;
    case TAM_OPT_THREADS: *value = s->shape.threads; return TAM_OK;
    case TAM_OPT_INT_MUL: *value = s->shape.int_mul; return TAM_OK;
    case TAM_OPT_ONE_TAP: *value = s->shape.one_tap; return TAM_OK;
    case TAM_OPT_COPY_POINTS: *value = s->shape.copy_points; return TAM_OK;
    case TAM_OPT_MERGE_STAGES: *value = s->shape.merge_stages; return TAM_OK;
    case TAM_OPT_STAGED: *value = s->shape.staged; return TAM_OK;
    case TAM_OPT_PAIR_VARS: *value = s->shape.pair_vars; return TAM_OK;
    case TAM_OPT_BLOCK_ORDER: *value = s->shape.block_order; return TAM_OK;
    case TAM_OPT_PATH_TILES: *value = s->shape.path_tiles; return TAM_OK;
    case TAM_OPT_COPY_SHARE: *value = s->shape.copy_share; return TAM_OK;
    case TAM_OPT_SOFT_ADD: *value = s->shape.soft_add; return TAM_OK;
    case TAM_OPT_STENCIL_TILE: *value = s->shape.stencil_tile; return TAM_OK;
    default: return fail(s->ctx, TAM_EINVAL, "unknown option");
  }
}

int tam_selftest(tam_ctx *ctx, int32_t which, int64_t n, uint64_t seed, int64_t *mismatches) {
  if (!ctx || !mismatches || n < 0) return fail(ctx, TAM_EINVAL, "tam_selftest: bad argument");
  if (which != TAM_SELFTEST_MUL && which != TAM_SELFTEST_ADD && which != TAM_SELFTEST_MUL_FULL)
    return fail(ctx, TAM_EINVAL, "tam_selftest: unknown test");
  DeviceGuard guard(ctx->device);
  if (!guard.ok()) return fail(ctx, TAM_ECUDA, "cannot make the context's device current");
  unsigned long long *d = nullptr, h[2] = {0, 0};
  cudaError_t e = cudaMalloc((void **)&d, sizeof h);
  if (e == cudaSuccess) e = cudaMemset(d, 0, sizeof h);
  if (e == cudaSuccess)
    e = which == TAM_SELFTEST_MUL   ? tam::launch_selftest_mul(n, seed, d, 0)
        : which == TAM_SELFTEST_ADD ? tam::launch_selftest_add(n, seed, d, 0)
                                    : tam::launch_selftest_mul_full(n, seed, d, 0);
  if (e == cudaSuccess) e = cudaMemcpy(h, d, sizeof h, cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "tam_selftest");
  *mismatches = (int64_t)h[0];
  return TAM_OK;
}

int tam_device_status(tam_sched *s, void *stream, int32_t *code) {
  if (!s || !code) return fail(nullptr, TAM_EINVAL, "tam_device_status: NULL argument");
  DeviceGuard guard(s->ctx->device);
  cudaStream_t st = (cudaStream_t)stream;
  int32_t h = 0;
  cudaError_t e = cudaMemcpyAsync(&h, s->d_err, sizeof h, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e == cudaSuccess) e = cudaMemsetAsync(s->d_err, 0, sizeof(int32_t), st);
  if (e != cudaSuccess) return cuda_fail(s->ctx, e, "tam_device_status");
  *code = h;
  return TAM_OK;
}

}  // extern "C"
