// Many forests in one launch: the batch of tam_batch_create / tam_batch_fill.
//
// The reference fills one field set at a time (src/ghosts.jl:1783).  A batch
// takes the uploaded schedules of several independent forests -- of any
// sizes and block extents, one element type -- whose field data live at
// given offsets of one arena, concatenates their groups, pools and block
// lists into one schedule-shaped set of device arrays with every group
// tagged with its member, and tiles each stage tag across all members, so
// that a whole stage of every forest is one copy launch and one stencil
// launch.  Members' solo groups (turned across a seam, or bounded) follow
// each stage's fused launches as one solo launch for all members.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <new>
#include <string>
#include <vector>

#include "tam_internal.h"
#include "treeamr_cuda.h"

struct tam_batch {
  tam_ctx *ctx = nullptr;
  int D = 0, dtype = 0;
  std::vector<tam_sched *> members;
  std::vector<tam::Member> layout;     // per member
  std::vector<int64_t> member_points;  // nblocks * prod(S) per member (one variable)
  bool needs_factors = false;
  bool needs_rotvars = false, has_bounded = false;
  std::vector<tam::DevGroup> groups;
  std::vector<int32_t> h_tb;
  std::vector<int32_t> h_csingle, h_perm;  // the concatenated pools, for the tiling
  std::vector<tam::Stage> stages;
  tam::LaunchShape shape;
  tam::DevGroup *d_groups = nullptr;
  int32_t *d_tb = nullptr, *d_sb = nullptr, *d_srcstart = nullptr, *d_cls = nullptr;
  int32_t *d_csingle = nullptr, *d_perm = nullptr;
  void *d_weights = nullptr, *d_wtab = nullptr;
  uint64_t *d_wshort = nullptr;
  tam::Tile *d_tiles = nullptr;
  tam::PTile *d_ptiles = nullptr;
  tam::Tile *d_staged = nullptr;
  tam::Member *d_members = nullptr;
  std::vector<tam::SoloGroup> h_solos;  // by stage tag, members in order
  tam::SoloGroup *d_solos = nullptr;
  int32_t *d_err = nullptr;  // the solo launches' error word
  tam::SideStream side;
  // each member's first group, transfer and weight in the concatenated arrays
  std::vector<int64_t> group_base, transfer_base, weight_base;
  // the batched adjoint, prepared on first use
  tam::AdjPlan adj;
  void *adj_scratch = nullptr;
  size_t adj_scratch_bytes = 0;
};

namespace {

int bfail(tam_ctx *ctx, int code, const std::string &msg) {
  if (ctx) ctx->err = msg;
  return code;
}

struct Guard {
  int prev = 0;
  bool ok = false;
  explicit Guard(int device) {
    ok = cudaGetDevice(&prev) == cudaSuccess;
    if (ok && prev != device) ok = cudaSetDevice(device) == cudaSuccess;
  }
  ~Guard() {
    int cur = -1;
    if (cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
  }
};

template <typename T>
cudaError_t up(T **dst, const T *src, size_t n) {
  *dst = nullptr;
  const size_t m = std::max<size_t>(n, 1);
  cudaError_t e = cudaMalloc((void **)dst, m * sizeof(T));
  if (e != cudaSuccess || n == 0) return e;
  return cudaMemcpy(*dst, src, n * sizeof(T), cudaMemcpyHostToDevice);
}

void free_batch_device(tam_batch *b) {
  cudaFree(b->d_groups);
  cudaFree(b->d_tb);
  cudaFree(b->d_sb);
  cudaFree(b->d_srcstart);
  cudaFree(b->d_cls);
  cudaFree(b->d_weights);
  cudaFree(b->d_wtab);
  cudaFree(b->d_wshort);
  cudaFree(b->d_staged);
  cudaFree(b->d_tiles);
  cudaFree(b->d_ptiles);
  cudaFree(b->d_members);
  cudaFree(b->d_csingle);
  cudaFree(b->d_perm);
  cudaFree(b->d_solos);
  cudaFree(b->d_err);
  tam::adjoint_plan_free(b->adj);
  cudaFree(b->adj_scratch);
  b->adj_scratch = nullptr;
  b->adj_scratch_bytes = 0;
  tam::side_destroy(b->side);
  b->d_ptiles = nullptr;
  b->d_groups = nullptr;
  b->d_tb = b->d_sb = b->d_srcstart = b->d_cls = nullptr;
  b->d_weights = b->d_wtab = nullptr;
  b->d_wshort = nullptr;
  b->d_staged = nullptr;
  b->d_tiles = nullptr;
  b->d_members = nullptr;
  b->d_csingle = b->d_perm = nullptr;
  b->d_solos = nullptr;
  b->d_err = nullptr;
}

// Every stage tag's tiles across all members: per member the transfers by
// target block, unit copies of every member first, then the stencils.
std::vector<tam::Tile> batch_tiles(tam_batch *b, std::vector<uint16_t> &keys,
                                   std::vector<tam::Tile> &staged) {
  std::vector<tam::Tile> tiles;
  keys.clear();
  staged.clear();
  tam::StencilRuns runs;
  const int ti = b->shape.tile_items, tst = b->shape.stencil_items();
  for (tam::Stage &st : b->stages) {
    st.tile0 = (int64_t)tiles.size();
    struct Entry {
      int32_t member, tblock, group, transfer;
    };
    std::vector<Entry> entries;
    for (int32_t gi : st.groups) {
      const tam::DevGroup &g = b->groups[gi];
      if (g.turned) continue;  // a solo group: its own launch
      for (int64_t t = 0; t < g.ntransfers; ++t)
        entries.push_back({g.member, b->h_tb[g.first + t], gi, (int32_t)(g.first + t)});
    }
    std::stable_sort(entries.begin(), entries.end(), [](const Entry &x, const Entry &y) {
      if (x.member != y.member) return x.member < y.member;
      return x.tblock != y.tblock ? x.tblock < y.tblock : x.group < y.group;
    });
    for (int pass = 0; pass < 2; ++pass) {
      for (const Entry &e : entries) {
        const tam::DevGroup &g = b->groups[e.group];
        if (tam::tile_pass(g) != pass) continue;
        const int box = g.n[0] * g.n[1] * g.n[2];
        for (int i0 = 0; i0 < box; i0 += ti) {
          tiles.push_back({e.group, e.transfer, i0, std::min(ti, box - i0)});
          keys.push_back(0);
        }
      }
      if (pass == 0) st.ncopy0 = (int64_t)tiles.size() - st.tile0;
      if (pass == 1) st.ncopy = (int64_t)tiles.size() - st.tile0;
    }
    // the stencils by their path through the kernel (tam::StencilRuns)
    std::vector<tam::Tile> sten;
    std::vector<uint16_t> skeys;
    for (const Entry &e : entries) {
      const tam::DevGroup &g = b->groups[e.group];
      if (tam::tile_pass(g) != 2) continue;
      if (!b->shape.path_tiles) {  // by target block alone: one key
        const int box = g.n[0] * g.n[1] * g.n[2];
        for (int i0 = 0; i0 < box; i0 += tst) {
          sten.push_back({e.group, e.transfer, i0, std::min(tst, box - i0)});
          skeys.push_back(0);
        }
        continue;
      }
      if (!runs.cache.count(e.group))
        tam::StencilRuns::of(g, b->h_csingle.data(), b->h_perm.data(), b->D,
                             runs.cache[e.group]);
      runs.tiles(e.group, e.transfer, tst, sten, skeys);
    }
    // staged groups' tiles last (the staged kernel takes their transfers)
    const bool staging = b->shape.staged != 0;
    auto is_staged = [&](size_t i) { return staging && b->groups[sten[i].group].staged; };
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
        const tam::DevGroup &g = b->groups[e.group];
        if (tam::tile_pass(g) == 2 && g.staged) {
          staged.push_back({e.group, e.transfer, 0, g.n[0] * g.n[1] * g.n[2]});
          st.staged_window =
              std::max<int64_t>(st.staged_window, (int64_t)g.wn[0] * g.wn[1] * g.wn[2]);
        }
      }
    st.nstaged = (int64_t)staged.size() - st.staged0;
  }
  if (staged.empty()) staged.push_back({0, 0, 0, 0});  // a valid pool even when unused
  return tiles;
}

int check_arena(tam_batch *b, int64_t arena_elems, int32_t nvars, const void *factor_arena,
                int64_t factor_elems) {
  if (nvars < 1) return bfail(b->ctx, TAM_EINVAL, "batch fill: nvars must be positive");
  for (size_t m = 0; m < b->members.size(); ++m) {
    const tam::Member &L = b->layout[m];
    const int64_t cols = b->members[m]->nfactorcols;  // 3^D, or 4 * 3^D over a seam
    if (L.work_off < 0 || L.work_off + b->member_points[m] * nvars > arena_elems)
      return bfail(b->ctx, TAM_EINVAL,
                   "batch fill: member " + std::to_string(m) + " lies outside the arena");
    if (b->members[m]->needs_factors &&
        (!factor_arena || L.fac_off < 0 || L.fac_off + cols * nvars > factor_elems))
      return bfail(b->ctx, TAM_EINVAL,
                   "batch fill: member " + std::to_string(m) +
                       " mirrors ghosts and its factor table lies outside the factor arena");
  }
  return TAM_OK;
}

}  // namespace

extern "C" {

int tam_batch_create(tam_ctx *ctx, tam_sched *const *members, int32_t n,
                     const int64_t *work_offsets, const int64_t *factor_offsets,
                     tam_batch **out) {
  if (!ctx || !members || !work_offsets || !out || n < 1)
    return bfail(ctx, TAM_EINVAL, "tam_batch_create: bad argument");
  *out = nullptr;
  const tam_sched *first = members[0];
  if (!first) return bfail(ctx, TAM_EINVAL, "tam_batch_create: NULL member");
  for (int32_t m = 0; m < n; ++m) {
    if (!members[m]) return bfail(ctx, TAM_EINVAL, "tam_batch_create: NULL member");
    if (members[m]->ctx != ctx)
      return bfail(ctx, TAM_EINVAL, "tam_batch_create: a member was uploaded by another context");
    if (members[m]->D != first->D || members[m]->dtype != first->dtype)
      return bfail(ctx, TAM_EINVAL,
                   "tam_batch_create: members differ in dimension or element type");
    // a member's odd turns read its own array: a RotationPair member, whose
    // layout is not symmetric in the seam's plane, reads its partner's
    for (const tam_group &h : members[m]->host_groups) {
      if (!(h.orientation & 1)) continue;
      for (int e = 0; e < members[m]->D; ++e)
        if (members[m]->S[(h.axes >> (2 * e)) & 3] != members[m]->S[e])
          return bfail(ctx, TAM_EUNSUPPORTED,
                       "tam_batch_create: member " + std::to_string(m) +
                           " is a RotationPair member (its layout is not symmetric in the "
                           "seam's plane) and reads its partner's array; fill the pair with "
                           "tam_fill_ex");
    }
  }
  Guard guard(ctx->device);
  if (!guard.ok) return bfail(ctx, TAM_ECUDA, "cannot make the context's device current");
  tam_batch *b = new (std::nothrow) tam_batch;
  if (!b) return bfail(ctx, TAM_ENOMEM, "out of host memory");
  b->ctx = ctx;
  b->D = first->D;
  b->dtype = first->dtype;
  const size_t esz = b->dtype == TAM_F64 ? 8 : 4;
  std::vector<int32_t> tb, sb, srcstart, cls, csingle, perm;
  std::vector<unsigned char> weights, wtab;
  std::map<int32_t, std::vector<int32_t>> bytag;
  for (int32_t m = 0; m < n; ++m) {
    tam_sched *s = members[m];
    b->members.push_back(s);
    tam::Member L;
    memset(&L, 0, sizeof L);
    L.work_off = work_offsets[m];
    L.fac_off = factor_offsets ? factor_offsets[m] : 0;
    for (int k = 0; k < 3; ++k) L.S[k] = s->S[k];
    b->layout.push_back(L);
    b->member_points.push_back(s->nblocks * (int64_t)s->S[0] * s->S[1] * s->S[2]);
    b->needs_factors = b->needs_factors || s->needs_factors;
    b->needs_rotvars = b->needs_rotvars || s->needs_rotvars;
    b->has_bounded = b->has_bounded || s->has_bounded;
    const int64_t g0 = (int64_t)b->groups.size(), t0 = (int64_t)tb.size();
    const int64_t ss0 = (int64_t)srcstart.size(), c0 = (int64_t)cls.size();
    const int64_t cs0 = (int64_t)csingle.size(), p0 = (int64_t)perm.size();
    const int64_t w0 = (int64_t)(weights.size() / esz), wt0 = (int64_t)(wtab.size() / esz);
    b->group_base.push_back(g0);
    b->transfer_base.push_back(t0);
    b->weight_base.push_back(w0);
    for (const tam::DevGroup &h : s->groups) {
      tam::DevGroup g = h;
      for (int k = 0; k < 3; ++k) {
        g.ss[k] += ss0;
        g.w[k] += w0;
        g.cls[k] += c0;
        g.csingle[k] += cs0;
      }
      if (g.perm >= 0) g.perm += p0;
      g.wtab += wt0;
      g.first += t0;
      g.member = m;
      b->groups.push_back(g);
    }
    for (const tam::Stage &st : s->stages)
      for (int32_t gi : st.groups) bytag[st.tag].push_back((int32_t)(g0 + gi));
    tb.insert(tb.end(), s->h_tb.begin(), s->h_tb.end());
    sb.insert(sb.end(), s->h_sb.begin(), s->h_sb.end());
    srcstart.insert(srcstart.end(), s->h_pool_srcstart.begin(), s->h_pool_srcstart.end());
    cls.insert(cls.end(), s->h_pool_cls.begin(), s->h_pool_cls.end());
    csingle.insert(csingle.end(), s->h_pool_csingle.begin(), s->h_pool_csingle.end());
    perm.insert(perm.end(), s->h_pool_perm.begin(), s->h_pool_perm.end());
    weights.insert(weights.end(), s->h_pool_weights.begin(), s->h_pool_weights.end());
    // element-aligned: each member's product table starts on an element
    wtab.resize((wtab.size() + esz - 1) / esz * esz);
    const int64_t wt0b = (int64_t)(wtab.size() / esz);
    if (wt0b != wt0) {
      for (int64_t gi = g0; gi < (int64_t)b->groups.size(); ++gi)
        b->groups[gi].wtab += wt0b - wt0;
    }
    wtab.insert(wtab.end(), s->h_pool_wtab.begin(), s->h_pool_wtab.end());
  }
  if (tb.size() > (size_t)INT32_MAX || b->groups.size() > (size_t)INT32_MAX) {
    delete b;
    return bfail(ctx, TAM_EUNSUPPORTED, "tam_batch_create: more than 2^31 transfers or groups");
  }
  for (auto &kv : bytag) {
    tam::Stage st;
    st.tag = kv.first;
    st.groups = kv.second;
    // the members' solo groups of this tag, their group indices moved to the batch's
    st.solo0 = (int64_t)b->h_solos.size();
    for (int32_t m = 0; m < n; ++m) {
      const tam_sched *s = members[m];
      for (const tam::Stage &ms : s->stages) {
        if (ms.tag != st.tag) continue;
        for (int64_t i = ms.solo0; i < ms.solo0 + ms.nsolo; ++i) {
          tam::SoloGroup t = s->h_solos[i];
          t.group += (int32_t)b->group_base[m];
          b->h_solos.push_back(t);
        }
      }
    }
    st.nsolo = (int64_t)b->h_solos.size() - st.solo0;
    b->stages.push_back(st);
  }
  b->h_tb = tb;
  b->h_csingle = csingle;
  b->h_perm = perm;
  b->shape.path_tiles = b->dtype == TAM_F64 ? 1 : 0;
  std::vector<uint16_t> keys;
  std::vector<tam::Tile> staged;
  std::vector<tam::Tile> tiles = batch_tiles(b, keys, staged);
  std::vector<tam::PTile> ptiles =
      tam::pack_stages(b->stages, tiles, b->shape.tile_items, &keys,
                         b->shape.stencil_items());
  std::vector<uint64_t> wshort;
  if (b->dtype == TAM_F64) wshort = tam::short_weights(wtab);
  if (wshort.empty()) wshort.push_back(0);
  cudaError_t e;
  if ((e = tam::side_create(b->side)) != cudaSuccess ||
      (e = up(&b->d_ptiles, ptiles.data(), ptiles.size())) != cudaSuccess ||
      (e = up(&b->d_groups, b->groups.data(), b->groups.size())) != cudaSuccess ||
      (e = up(&b->d_tb, tb.data(), tb.size())) != cudaSuccess ||
      (e = up(&b->d_sb, sb.data(), sb.size())) != cudaSuccess ||
      (e = up(&b->d_srcstart, srcstart.data(), srcstart.size())) != cudaSuccess ||
      (e = up(&b->d_cls, cls.data(), cls.size())) != cudaSuccess ||
      (e = up(&b->d_csingle, csingle.data(), csingle.size())) != cudaSuccess ||
      (e = up(&b->d_perm, perm.data(), perm.size())) != cudaSuccess ||
      (e = up((unsigned char **)&b->d_weights, weights.data(), weights.size())) != cudaSuccess ||
      (e = up((unsigned char **)&b->d_wtab, wtab.data(), wtab.size())) != cudaSuccess ||
      (e = up(&b->d_wshort, wshort.data(), wshort.size())) != cudaSuccess ||
      (e = up(&b->d_tiles, tiles.data(), tiles.size())) != cudaSuccess ||
      (e = up(&b->d_staged, staged.data(), staged.size())) != cudaSuccess ||
      (e = up(&b->d_members, b->layout.data(), b->layout.size())) != cudaSuccess ||
      (e = up(&b->d_solos, b->h_solos.data(), b->h_solos.size())) != cudaSuccess ||
      (e = cudaMalloc((void **)&b->d_err, sizeof(int32_t))) != cudaSuccess ||
      (e = cudaMemset(b->d_err, 0, sizeof(int32_t))) != cudaSuccess) {
    free_batch_device(b);
    delete b;
    return bfail(ctx, e == cudaErrorMemoryAllocation ? TAM_ENOMEM : TAM_ECUDA,
                 std::string("tam_batch_create: ") + cudaGetErrorString(e));
  }
  *out = b;
  return TAM_OK;
}

void tam_batch_free(tam_batch *b) {
  if (!b) return;
  Guard guard(b->ctx->device);
  free_batch_device(b);
  delete b;
}

int tam_batch_fill(tam_batch *b, void *arena, int64_t arena_elems, int32_t nvars,
                   const void *factor_arena, int64_t factor_elems, int32_t first_stage,
                   int32_t last_stage, void *stream) {
  return tam_batch_fill_ex(b, arena, arena_elems, nvars, factor_arena, factor_elems, nullptr,
                           first_stage, last_stage, stream);
}

int tam_batch_fill_ex(tam_batch *b, void *arena, int64_t arena_elems, int32_t nvars,
                      const void *factor_arena, int64_t factor_elems, const int32_t *rotvars,
                      int32_t first_stage, int32_t last_stage, void *stream) {
  if (!b || !arena) return bfail(b ? b->ctx : nullptr, TAM_EINVAL, "tam_batch_fill: NULL argument");
  int rc = check_arena(b, arena_elems, nvars, factor_arena, factor_elems);
  if (rc != TAM_OK) return rc;
  if (b->needs_rotvars && !rotvars)
    return bfail(b->ctx, TAM_EINVAL,
                 "a member of this batch turns ghosts across a rotating seam, but no variable "
                 "table was given to turn them with: use tam_batch_fill_ex");
  Guard guard(b->ctx->device);
  if (!guard.ok) return bfail(b->ctx, TAM_ECUDA, "cannot make the context's device current");
  const tam::SchedArgs args{b->d_groups,  b->d_tb,      b->d_sb,          b->d_srcstart,
                            b->d_weights, b->d_cls,     b->d_wtab,        b->shape.int_mul,
                            b->d_members, b->d_csingle, b->d_perm,        b->shape.one_tap,
                            b->shape.copy_points, b->d_wshort, b->shape.pair_vars,
                            b->shape.copy_share * b->ctx->nsm, b->shape.soft_add};
  const int S[3] = {1, 1, 1};  // each member's own, from the member table
  for (const tam::Stage &st : b->stages) {
    if (st.tag < first_stage || st.tag > last_stage) continue;
    cudaError_t e = tam::launch_fused_stage(b->dtype, b->D, b->d_tiles, b->d_ptiles, st, args,
                                            arena, factor_arena, nvars, S, b->shape.threads,
                                            (cudaStream_t)stream, &b->side, nullptr,
                                            b->d_staged);
    if (e == cudaSuccess && st.nsolo > 0)
      e = tam::launch_solo(b->dtype, b->D, b->d_solos + st.solo0, st.nsolo, args, arena, arena,
                           arena, factor_arena, rotvars, nvars, S, b->d_err,
                           (cudaStream_t)stream);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return bfail(b->ctx, TAM_ECUDA, std::string("batch stage launch: ") + cudaGetErrorString(e));
    }
  }
  return TAM_OK;
}

int tam_batch_fill_adjoint(tam_batch *b, void *arena, int64_t arena_elems, int32_t nvars,
                           const void *factor_arena, int64_t factor_elems, int32_t first_stage,
                           int32_t last_stage, void *stream) {
  return tam_batch_fill_adjoint_ex(b, arena, arena_elems, nvars, factor_arena, factor_elems,
                                   nullptr, first_stage, last_stage, stream);
}

int tam_batch_fill_adjoint_ex(tam_batch *b, void *arena, int64_t arena_elems, int32_t nvars,
                              const void *factor_arena, int64_t factor_elems,
                              const int32_t *rotvars, int32_t first_stage, int32_t last_stage,
                              void *stream) {
  if (!b || !arena)
    return bfail(b ? b->ctx : nullptr, TAM_EINVAL, "tam_batch_fill_adjoint: NULL argument");
  int rc = check_arena(b, arena_elems, nvars, factor_arena, factor_elems);
  if (rc != TAM_OK) return rc;
  if (b->has_bounded)
    return bfail(b->ctx, TAM_EUNSUPPORTED,
                 "a member of this batch has bounded operators, which are not linear, so the "
                 "batch has no adjoint");
  if (b->needs_rotvars && !rotvars)
    return bfail(b->ctx, TAM_EINVAL,
                 "a member of this batch turns ghosts across a rotating seam, but no variable "
                 "table was given: use tam_batch_fill_adjoint_ex");
  Guard guard(b->ctx->device);
  if (!guard.ok) return bfail(b->ctx, TAM_ECUDA, "cannot make the context's device current");
  if (!b->adj.ready) {
    std::string err;
    rc = tam::adjoint_prepare_batch(b->adj, b->members, b->group_base, b->transfer_base,
                                    b->weight_base, b->stages, err);
    if (rc != TAM_OK) return bfail(b->ctx, rc, "tam_batch_fill_adjoint: " + err);
  }
  const size_t need = (size_t)b->adj.scratch_points * nvars * (b->dtype == TAM_F64 ? 8 : 4);
  if (need > b->adj_scratch_bytes) {
    // grown only between fills: wait for any fill still using the old one
    cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess)
      return bfail(b->ctx, TAM_ECUDA, std::string("batch adjoint: ") + cudaGetErrorString(e));
    cudaFree(b->adj_scratch);
    b->adj_scratch = nullptr;
    b->adj_scratch_bytes = 0;
    if (cudaMalloc(&b->adj_scratch, need) != cudaSuccess) {
      cudaGetLastError();
      return bfail(b->ctx, TAM_ENOMEM, "batch adjoint: scratch allocation failed");
    }
    b->adj_scratch_bytes = need;
  }
  const tam::AdjRun r{b->dtype,   b->D,      b->d_groups, b->d_tb,   b->d_weights,
                      b->d_members, b->d_tiles, &b->stages, {1, 1, 1}, b->d_solos,
                      rotvars,     b->d_err,    arena};
  // stages from the last down to 0 transposed, then stage P forward: it
  // scales each wall-plane point in place, a diagonal map, its own transpose
  const bool p = first_stage <= TAM_STAGE_SELFIMAGE && TAM_STAGE_SELFIMAGE <= last_stage;
  cudaError_t e = tam::adjoint_run_plan(b->adj, r, arena, nvars, factor_arena,
                                        p ? TAM_STAGE_SELFIMAGE + 1 : first_stage, last_stage,
                                        b->adj_scratch, (cudaStream_t)stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return bfail(b->ctx, TAM_ECUDA, std::string("batch adjoint launch: ") + cudaGetErrorString(e));
  }
  if (p)
    return tam_batch_fill_ex(b, arena, arena_elems, nvars, factor_arena, factor_elems, rotvars,
                             TAM_STAGE_SELFIMAGE, TAM_STAGE_SELFIMAGE, stream);
  return TAM_OK;
}

int tam_batch_device_status(tam_batch *b, void *stream, int32_t *code) {
  if (!b || !code) return bfail(b ? b->ctx : nullptr, TAM_EINVAL, "tam_batch_device_status: NULL argument");
  Guard guard(b->ctx->device);
  if (!guard.ok) return bfail(b->ctx, TAM_ECUDA, "cannot make the context's device current");
  cudaStream_t st = (cudaStream_t)stream;
  int32_t h = 0;
  cudaError_t e = cudaMemcpyAsync(&h, b->d_err, sizeof h, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e == cudaSuccess) e = cudaMemsetAsync(b->d_err, 0, sizeof(int32_t), st);
  if (e != cudaSuccess)
    return bfail(b->ctx, TAM_ECUDA, std::string("tam_batch_device_status: ") + cudaGetErrorString(e));
  *code = h;
  return TAM_OK;
}

int tam_batch_set_option(tam_batch *b, int32_t option, int64_t value) {
  if (!b) return TAM_EINVAL;
  if (option == TAM_OPT_TILE_ITEMS || option == TAM_OPT_STENCIL_TILE ||
      option == TAM_OPT_PATH_TILES || option == TAM_OPT_STAGED) {
    int *field = option == TAM_OPT_TILE_ITEMS     ? &b->shape.tile_items
                 : option == TAM_OPT_STENCIL_TILE ? &b->shape.stencil_tile
                 : option == TAM_OPT_PATH_TILES   ? &b->shape.path_tiles
                                                  : &b->shape.staged;
    if (option == TAM_OPT_TILE_ITEMS && (value < 16 || value > 4096))
      return bfail(b->ctx, TAM_EINVAL, "tile items must be in 16..4096");
    if (option == TAM_OPT_STENCIL_TILE && value != 0 && (value < 16 || value > 4096))
      return bfail(b->ctx, TAM_EINVAL, "stencil tile items are 0 or in 16..4096");
    if ((option == TAM_OPT_PATH_TILES || option == TAM_OPT_STAGED) && value != 0 && value != 1)
      return bfail(b->ctx, TAM_EINVAL, "path_tiles and staged are 0 or 1");
    Guard guard(b->ctx->device);
    const int old = *field;
    *field = (int)value;
    std::vector<uint16_t> keys;
    std::vector<tam::Tile> staged;
    std::vector<tam::Tile> tiles = batch_tiles(b, keys, staged);
    std::vector<tam::PTile> ptiles =
        tam::pack_stages(b->stages, tiles, b->shape.tile_items, &keys,
                         b->shape.stencil_items());
    tam::Tile *d = nullptr, *dst = nullptr;
    tam::PTile *dp = nullptr;
    cudaError_t e = up(&d, tiles.data(), tiles.size());
    if (e == cudaSuccess) e = up(&dp, ptiles.data(), ptiles.size());
    if (e == cudaSuccess) e = up(&dst, staged.data(), staged.size());
    if (e != cudaSuccess) {
      cudaFree(d);
      cudaFree(dp);
      cudaFree(dst);
      *field = old;
      std::vector<tam::Tile> back = batch_tiles(b, keys, staged);
      tam::pack_stages(b->stages, back, b->shape.tile_items, &keys, b->shape.stencil_items());
      return bfail(b->ctx, TAM_ECUDA, "re-tiling the batch failed");
    }
    cudaDeviceSynchronize();
    cudaFree(b->d_tiles);
    cudaFree(b->d_ptiles);
    cudaFree(b->d_staged);
    b->d_tiles = d;
    b->d_ptiles = dp;
    b->d_staged = dst;
    return TAM_OK;
  }
  if (option == TAM_OPT_THREADS) {
    if (value < 64 || value > 512 || value % 32)
      return bfail(b->ctx, TAM_EINVAL, "threads must be a multiple of 32 in 64..512");
    b->shape.threads = (int)value;
    return TAM_OK;
  }
  if (option == TAM_OPT_INT_MUL) {
    if (value != 0 && value != 1) return bfail(b->ctx, TAM_EINVAL, "int_mul is 0 or 1");
    b->shape.int_mul = (int)value;
    return TAM_OK;
  }
  if (option == TAM_OPT_ONE_TAP) {
    if (value != 0 && value != 1) return bfail(b->ctx, TAM_EINVAL, "one_tap is 0 or 1");
    b->shape.one_tap = (int)value;
    return TAM_OK;
  }
  if (option == TAM_OPT_PAIR_VARS) {
    if (value != 0 && value != 1) return bfail(b->ctx, TAM_EINVAL, "pair_vars is 0 or 1");
    b->shape.pair_vars = (int)value;
    return TAM_OK;
  }
  if (option == TAM_OPT_COPY_POINTS) {
    if (value != 1 && value != 2 && value != 4)
      return bfail(b->ctx, TAM_EINVAL, "copy_points is 1, 2 or 4");
    b->shape.copy_points = (int)value;
    return TAM_OK;
  }
  if (option == TAM_OPT_COPY_SHARE) {
    if (value < 0 || value > 32) return bfail(b->ctx, TAM_EINVAL, "copy_share is 0..32");
    b->shape.copy_share = (int)value;
    return TAM_OK;
  }
  if (option == TAM_OPT_SOFT_ADD) {
    if (value != 0 && value != 1) return bfail(b->ctx, TAM_EINVAL, "soft_add is 0 or 1");
    b->shape.soft_add = (int)value;
    return TAM_OK;
  }
  return bfail(b->ctx, TAM_EINVAL, "unknown option");
}

}  // extern "C"
