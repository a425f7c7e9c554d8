// Internal types of libtreeamr_cuda.so shared by the host API and the kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <map>
#include <string>
#include <vector>

#include "treeamr_cuda.h"

namespace tam {

// A TransferGroup as the kernels read it: the host descriptor with the
// stored-index offsets made 0-based and unused dimensions padded to one
// row of one unit weight, so a kernel for D < 3 is the D = 3 kernel with
// trip counts of one.
struct DevGroup {
  int32_t n[3];      // target rows per dimension
  int32_t tf[3];     // targetfirst - 1
  int32_t order[3];  // weights per column
  int32_t unit;      // every dimension is a unit copy
  int32_t factorcol; // 0 or the 1-based factor column
  int32_t pclass;    // 0: copy, P > 0: uniform order P, -1: mixed orders
  int64_t ss[3];     // srcstart pool offsets (0-based entries)
  int64_t w[3];      // weight pool offsets
  int64_t first;     // block-list offset
  int64_t ntransfers;
  // Uniform-order groups only: the weight products ((w_1*w_2)*w_3) of every
  // combination of distinct weight columns, rounded in the element type in
  // that order, so a tap costs one multiply and one add and the result is
  // bit-identical to forming the product per tap.  Row i of dimension d has
  // column class cls[d][i]; the products of classes (c1, c2, c3) start at
  // wtab + ((c3 * C2 + c2) * C1 + c1) * P^D, taps m_1 fastest.
  int32_t C[3];      // distinct columns per dimension
  int32_t shortw;    // every product is normal with a significand of <= 24 bits
  int64_t cls[3];    // class-index pool offsets (one int32 per target row)
  int64_t wtab;      // product-table pool offset
  int32_t member;    // the forest of a batch this group belongs to (0 alone)
  int32_t turned;    // a solo group (turned across a seam, or bounded): no tiles
  // The one-tap skip of the reference's CPU fill (src/ghosts.jl:28-56): per
  // dimension, for each column class, the row of its only nonzero weight, or
  // -1 (int32 pool entries at csingle[d] + class).  `perm` (or -1) orders the
  // box points by which dimensions skip, so that a warp's lanes share their
  // trip counts: point `perm[item]` is the item-th a tile takes.
  int64_t csingle[3];
  int64_t perm;
  // Box points to rows without a division: i3 = umulhi(item, mag12),
  // i2 = umulhi(rest, mag1), exact because box * n1 < 2^32 (0: divide).
  uint32_t mag1, mag12;
  // A unit copy whose source rows advance by -1, 0 or +1 a target row in
  // every dimension (a translation, a mirror, a clamp): the source row of
  // target row i is cs0[d] + cstep[d] * i (0-based), no srcstart load.
  int32_t affine;
  int32_t cs0[3];
  int32_t cstep[3];
  // A stencil group's source window, every transfer's the same in its source
  // block: rows wlo[d] .. wlo[d] + wn[d] - 1 (0-based stored indices), the
  // rows its columns read (the staged stencil kernel loads it into shared
  // memory).  staged: the group's transfers run in that kernel.
  int32_t wlo[3];
  int32_t wn[3];
  int32_t staged;
};

// A group the fused tiles do not take, run in a launch of its own after its
// stage's fused launches: a turned group (across a seam), whose real source
// is read at c0 + sum_d vs[d] * j[d] for virtual 0-based stored indices j
// (the axis map folded into signed strides of the real array), target
// variable v from real variable rotvars[v + nvars * col] - 1; or a bounded
// group (`bounded` 1: the bounded conservative prolongation, 2: the
// point-value sum clamped into its bracket), read in place (col 0, the
// array's own strides).
struct SoloGroup {
  int32_t group;    // index into the schedule's groups
  int32_t col;      // the orientation r: the rotvars column (0: not turned)
  int32_t odd;      // reads the alternate array
  int32_t bounded;  // 0, or the group's bound (tam_group.bounded)
  int64_t vs[3];
  int64_t c0;
};

// One forest of a batch (tam_batch_fill): where its field data and factor
// table start in the batch's arenas, in elements, and its stored extents.
struct Member {
  int64_t work_off;
  int64_t fac_off;
  int32_t S[3];
  int32_t pad;
};

// A warp's share of one transfer: box points [item0, item0 + nitems) of
// transfer `transfer` (an index into the block lists) of group `group`.
// Every variable of those points is the same warp's.
struct Tile {
  int32_t group;
  int32_t transfer;
  int32_t item0;
  int32_t nitems;
};

// What a warp of the fused kernels takes: up to 32 consecutive tiles
// (tiles[seg0 .. seg0 + nseg)), nitems box points in all, so that small
// transfers -- an 8-point corner, a 2-point edge of a vertex set -- share a
// warp instead of leaving most of its lanes idle.
struct PTile {
  int32_t seg0;
  int32_t nseg;
  int32_t nitems;
  int32_t pad;
};

// Which of a stage's three runs of tiles a group's transfers go to: unit
// copies without a factor column, unit copies with one, stencils.
inline int tile_pass(const DevGroup &g) {
  return g.pclass != 0 ? 2 : g.factorcol != 0 ? 1 : 0;
}

// The packing: consecutive tiles of [begin, end) joined while they fit in
// `target` points and 32 segments and, with `keys`, share their key.
void pack_tiles(const std::vector<Tile> &tiles, const std::vector<uint16_t> *keys,
                int64_t begin, int64_t end, int target, std::vector<PTile> &out);

struct Stage;
// Every stage's packed tiles (sets the stages' ptile0, npcopy, nptiles).
std::vector<PTile> pack_stages(std::vector<Stage> &stages, const std::vector<Tile> &tiles,
                               int target, const std::vector<uint16_t> *keys = nullptr,
                               int stencil_target = 0);

// A stencil group's box points in tile order cut into runs that take the
// same path through the stencil kernel: the same order class and, in the
// CPU form of the sum, the same set of dimensions that take one tap.  The
// key of a run is ((pclass + 2) << 4) | mask (mask 8: no one-tap rows).
// Tiles cut from runs and packed only with tiles of their key keep every
// lane of a warp on one path: GB300's FP64 pipe spends the same time on a
// warp instruction whatever lanes are off.
struct StencilRuns {
  struct Run {
    int first, n;
    uint16_t key;
  };
  std::map<int32_t, std::vector<Run>> cache;  // by group index
  static void of(const DevGroup &g, const int32_t *csingle, const int32_t *perm, int D,
                 std::vector<Run> &runs);
  // Tiles of at most `ti` points of transfer `transfer` of group `gi`
  // (its runs in `cache`), with their keys.
  void tiles(int32_t gi, int32_t transfer, int ti, std::vector<Tile> &out,
             std::vector<uint16_t> &keys);
};

// A second stream and two events, so a stage's copy and stencil launches run
// side by side (fork and join on the caller's stream; capturable).
struct SideStream {
  cudaStream_t stream = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
  bool ok() const { return stream && fork && join; }
};
cudaError_t side_create(SideStream &s);
void side_destroy(SideStream &s);

struct Stage {
  int32_t tag;
  std::vector<int32_t> groups;  // indices into the schedule's groups
  int64_t tile0 = 0;            // first tile in the schedule's tile array
  int64_t ntiles = 0;           // copy tiles first, then stencil tiles
  int64_t ncopy0 = 0;           // the stage's unit-copy tiles without a factor column,
  int64_t ncopy = 0;            // then all its unit-copy tiles
  int64_t ptile0 = 0;           // first packed tile of the stage
  int64_t npcopy0 = 0;          // packed tiles of the copies without a factor, of
  int64_t npcopy = 0;           // all the copies, then
  int64_t nptiles = 0;          // all packed tiles of the stage
  int64_t solo0 = 0;            // the stage's solo groups: solos[solo0 .. solo0 + nsolo)
  int64_t nsolo = 0;
  int32_t span = 1;             // a stage group: the consecutive stages it runs as one
  int32_t last_tag = 0;         // and the last one's tag
  int64_t staged0 = 0;          // its staged stencil transfers: staged[staged0 ..
  int64_t nstaged = 0;          //   staged0 + nstaged) (tam::Tile, the whole box)
  int64_t staged_window = 0;    // the largest window of them, one variable, in elements
  int64_t nsten = 0;            // stencil tiles the stencil kernel takes (the first
                                //   ones after the copies; the staged ones follow)
  int64_t np4_0 = 0;            // packed tiles [np4_0, np4_0 + np4) of the stage: the
  int64_t np4 = 0;              //   run of uniform order-4 stencils (tiles by path)
};

// The transpose of one group, for the adjoint fill (tam_adjoint.cu): per
// dimension the footprint, the source rows the group's windows cover
// (flo .. flo + fn - 1, 0-based stored indices), and for each footprint row
// the target rows that read it with their weights, in CSR form: entries
// [off[r], off[r+1]) of the entry pool, each (target row, weight index).
struct AdjGroup {
  int32_t flo[3];
  int32_t fn[3];
  int64_t off[3];    // offset into the row-offset pool (fn + 1 entries)
  int64_t fsize;     // footprint points: fn[0] * fn[1] * fn[2]
  // A turned group: its footprint (virtual rows) lands on the real source
  // at tc0 + sum_d tvs[d] * row[d], real variable rotvars[v + nvars * col] - 1
  // (col 0: an ordinary group, the footprint in place).
  int32_t col;
  // A unit copy whose source rows step by +-1 in every dimension of more
  // than one row (a translation or a mirror, not turned): its transpose is
  // the target box read back through the same map, which pass 2 reads in
  // place (pass 1 has nothing to do for it).
  int32_t direct;
  int64_t tvs[3];
  int64_t tc0;
};

// Pass 1's transfers of one size class: list[first .. first + count) of the
// pass-1 transfer list ((transfer, group) pairs), and the shared memory a CTA
// of the class reserves: the boxes (elements) and the transposed stencils
// (entries and row offsets, all three dimensions), the class's maxima.
struct AdjPass1 {
  int64_t first = 0, count = 0;
  int64_t smem_elems = 0, csr_ents = 0, csr_rows = 0;
};

// Shared-memory classes of pass 1, by a transfer's bytes at 8-byte elements:
// a launch per class, so that one large box does not set every CTA's share
// (and with it the CTAs a multiprocessor holds).
constexpr int kAdjClasses = 3;
constexpr int64_t kAdjClassBytes[kAdjClasses - 1] = {12 * 1024, 48 * 1024};

// One stage of the adjoint: its transfers for pass 1 (a CTA each), and the
// source blocks pass 2 reduces into.
struct AdjStage {
  int32_t tag;
  AdjPass1 p1[kAdjClasses];
  int64_t red0 = 0, nred = 0;     // into the reduction block list
  int64_t scratch_points = 0;     // footprint points of the stage (per variable)
};

// Pass 2's work for one source block: the transfers reading it,
// list[first .. first + count), in waves: a transfer's footprint meets no
// other footprint of its wave, and one that meets an earlier transfer's
// (in transfer order) is in a later wave, so every point's adds keep
// transfer order; wend[i] marks the last entry of a wave.
struct AdjReduce {
  int32_t sblock;  // 0-based
  int32_t count;
  int64_t first;
  int32_t turned;  // a turned transfer among them: one CTA takes every variable
  int32_t pad;
};

// The adjoint's arrays on the device (tam_adjoint.cu), for one schedule or a
// batch of forests: transposed stencils per group, per stage the pass-1
// transfers and the pass-2 reduction blocks, and each transfer's scratch box.
struct AdjPlan {
  AdjGroup *groups = nullptr;
  int32_t *off = nullptr;        // CSR row offsets
  void *ent = nullptr;           // CSR entries, int2 (target row, weight index)
  int64_t *scr = nullptr;        // per transfer: scratch offset in points
  void *xfers = nullptr;         // pass-1 transfers, int2 (transfer, group)
  AdjReduce *red = nullptr;      // pass-2 reduction blocks
  void *list = nullptr;          // their transfers, int2 (transfer, group)
  uint8_t *wend = nullptr;       // per list entry: 1 ends a wave
  std::vector<AdjStage> stages;  // one per forward stage, in the same order
  int64_t scratch_points = 0;    // max over stages, per variable
  bool ready = false;
};

struct LaunchShape {
  int tile_items = 128;     // box points per tile
  int threads = 256;        // threads per CTA of the fused kernel
  int int_mul = 0;          // Float64 short-weight multiplies on the integer pipe
  int one_tap = 1;          // the CPU form of the sum (TAM_OPT_ONE_TAP)
  int copy_points = 1;      // points a lane of the copy kernel takes at once (TAM_OPT_COPY_POINTS)
  int block_order = 0;      // 0: the blocks' order, 1: a locality order (TAM_OPT_BLOCK_ORDER)
  int path_tiles = 0;       // stencil tiles grouped by path (TAM_OPT_PATH_TILES)
  int merge_stages = 1;     // stage groups run as one launch pair (TAM_OPT_MERGE_STAGES)
  int staged = 0;           // large stencil boxes from a shared-memory window (TAM_OPT_STAGED)
  int pair_vars = 0;        // Float64 order-4 stencils two variables a lane (TAM_OPT_PAIR_VARS)
  int copy_share = 0;       // copy CTAs a multiprocessor beside the stencils (TAM_OPT_COPY_SHARE)
  int soft_add = 0;         // Float64 order 4: a tap a row added on the integer pipe (TAM_OPT_SOFT_ADD)
  int stencil_tile = 0;     // box points per stencil tile, 0: tile_items (TAM_OPT_STENCIL_TILE)
  int stencil_items() const { return stencil_tile ? stencil_tile : tile_items; }
};

}  // namespace tam

struct tam_ctx {
  int device = 0;
  int nsm = 0;
  std::string err;
};

struct tam_sched {
  tam_ctx *ctx = nullptr;
  int D = 0;
  int dtype = 0;
  int S[3] = {1, 1, 1};
  int64_t nblocks = 0;
  int64_t nsource = 0;        // source blocks: nblocks, or a regrid's old count
  int32_t nfactorcols = 0;
  bool needs_factors = false;
  bool needs_rotvars = false;   // a turned group reads the variable table
  bool has_bounded = false;     // a bounded group: nonlinear, no adjoint
  std::vector<tam::SoloGroup> h_solos;
  std::vector<tam_group> host_groups;
  std::vector<int32_t> h_tb;  // target blocks, for re-tiling
  std::vector<int32_t> h_sb;  // source blocks, for the adjoint's lists
  std::vector<int32_t> h_srcstart;
  // the uploaded pools as the device holds them (with the pad entries)
  std::vector<int32_t> h_pool_srcstart;
  std::vector<unsigned char> h_pool_weights;
  std::vector<int32_t> h_pool_cls;
  std::vector<unsigned char> h_pool_wtab;
  std::vector<int32_t> h_pool_csingle;
  std::vector<int32_t> h_pool_perm;
  std::vector<tam::DevGroup> groups;
  std::vector<tam::Stage> stages;
  // Stage groups: consecutive prolongation stages that may run as one launch
  // pair (no point one writes is read or written by another), each a Stage
  // over the union of their groups, with its own tiles; merged_at[i] is the
  // group starting at stage i, or -1.
  std::vector<tam::Stage> merged;
  std::vector<int32_t> merged_at;
  int64_t ntransfers = 0;
  int64_t points = 0;
  tam::LaunchShape shape;
  // device arrays
  tam::DevGroup *d_groups = nullptr;
  int32_t *d_tb = nullptr;
  int32_t *d_sb = nullptr;
  int32_t *d_srcstart = nullptr;
  void *d_weights = nullptr;
  int32_t *d_cls = nullptr;
  void *d_wtab = nullptr;
  uint64_t *d_wshort = nullptr;
  int32_t *d_csingle = nullptr;
  int32_t *d_perm = nullptr;
  tam::Tile *d_tiles = nullptr;
  tam::PTile *d_ptiles = nullptr;
  tam::Tile *d_staged = nullptr;  // staged stencil transfers, by stage then stage group
  tam::SoloGroup *d_solos = nullptr;
  tam::SideStream side;
  int32_t *d_err = nullptr;
  // the adjoint, prepared on first use (tam_adjoint.cu)
  tam::AdjPlan adj;
  void *adj_scratch = nullptr;          // owned scratch, grown on demand
  size_t adj_scratch_bytes = 0;
};

namespace tam {

// Records `msg` as the last error of `ctx` (or, for a NULL context, as the
// library's last error without a context) and returns `code`.
int record_error(tam_ctx *ctx, int code, const std::string &msg);

// Kernel launchers (tam_kernels.cu).  All asynchronous on `stream`.
// The read-only schedule arrays every kernel gets.
struct SchedArgs {
  const DevGroup *groups;
  const int32_t *tb;
  const int32_t *sb;
  const int32_t *srcstart;
  const void *weights;
  const int32_t *cls;
  const void *wtab;
  int int_mul;
  const Member *members;  // a batch's member table, or null for one schedule
  const int32_t *csingle;  // per group, dimension and target row: the single row or -1
  const int32_t *perm;     // per group with singles: the box points in tile order
  int one_tap;             // take the single rows (the CPU form) in the fused kernels
  int copy_points;         // points a lane of the copy kernel takes at once (1, 2 or 4)
  const void *wshort;      // Float64: the product table's entries as mul_short takes them
  int pair_vars;           // Float64 order-4 stencils: two variables a lane
  int copy_ctas;           // beside stencils: the copy launch first, at most this grid (0: after)
  int soft_add;            // Float64 order 4: a tap a row added on the integer pipe
};

// The Float64 product table `wtab` (doubles) with each entry split as the
// integer-pipe multiply takes it, one uint64 an entry at the same index:
// the low word the significand as an integer in [2^23, 2^24), the high word
// the sign bit and the unbiased exponent plus 8192 (a zero weight: -4096).
std::vector<uint64_t> short_weights(const std::vector<unsigned char> &wtab);

cudaError_t launch_plain_group(int dtype, int D, const DevGroup &g, const DevGroup *d_g,
                               const SchedArgs &a, void *work, const void *factors, int nvars,
                               const int S[3], cudaStream_t stream);

// One stage `st` (or stage group): its packed tiles (from ptiles +
// st.ptile0) [0, npcopy) run the copy kernel (those from npcopy0 on with
// their factor column) and [npcopy, nptiles) the stencil kernel, the run
// [np4_0, np4_0 + np4) of them in its order-4 form, and its staged
// transfers (from staged + st.staged0) the staged kernel; on `stream` and,
// when `side` is given and both copies and stencils are present, the
// stencils on the side stream alongside.  Sources are read from `src` when
// given (a regrid's old array), else from `work`.
cudaError_t launch_fused_stage(int dtype, int D, const Tile *tiles, const PTile *ptiles,
                               const Stage &st, const SchedArgs &a, void *work,
                               const void *factors, int nvars, const int S[3], int threads,
                               cudaStream_t stream, SideStream *side, const void *src,
                               const Tile *staged);

// Shared memory a block of the staged stencil kernel holds, and the largest
// window (in bytes, one variable) a group may have to be staged.
constexpr int kStagedBytes = 48 * 1024;
// A stencil group's transfers go to the staged kernel when each holds this
// many box points or more (smaller ones keep the packed tiles).
constexpr int kStagedMinBox = 64;

// The solo groups turns[0 .. n) of one stage: a flat launch per group
// (blockIdx.y), reading `src` for an even orientation and `alt` for an odd
// one, target variable v from real variable rotvars[v + nvars * r] - 1
// (an entry outside 1:nvars skips the item and records TAM_EINVAL in *err).
cudaError_t launch_solo(int dtype, int D, const SoloGroup *turns, int64_t n,
                          const SchedArgs &a, const void *src, const void *alt, void *work,
                          const void *factors, const int32_t *rotvars, int nvars,
                          const int S[3], int32_t *err, cudaStream_t stream);

// The own boxes of `src` into `dst`, both in the working layout (tam_state.cu).
int own_box_copy(const tam_state_layout *layout, void *dst, const void *src, void *stream);

cudaError_t launch_selftest_mul(int64_t n, uint64_t seed, unsigned long long *mismatches,
                                cudaStream_t stream);
// mul_full against the hardware multiply, the same counts.
cudaError_t launch_selftest_mul_full(int64_t n, uint64_t seed, unsigned long long *mismatches,
                                     cudaStream_t stream);
// add_soft against the hardware add: mismatches[0] the differing results,
// mismatches[1] the pairs the adder hands back to the FP64 pipe.
cudaError_t launch_selftest_add(int64_t n, uint64_t seed, unsigned long long *mismatches,
                                cudaStream_t stream);

// The forward fill of the one stage `tag` of `s` on `work`, its fused
// launches as tam_fill runs them (tam_api.cpp); a stage with turned or
// bounded groups is refused (cudaErrorNotSupported).
cudaError_t fill_one_stage(tam_sched *s, void *work, int nvars, const void *factors,
                           int32_t tag, cudaStream_t stream);

// The adjoint (tam_adjoint.cu).  Stage P (TAM_STAGE_SELFIMAGE) scales each
// point of a reflecting wall plane in place by its variable's factor, a
// diagonal map and so its own transpose: the adjoint runs it forward, since
// the transposed passes (which zero a stage's targets after adding onto its
// sources) assume a stage reads none of its own targets.
int adjoint_prepare(tam_sched *s, std::string &err);
void adjoint_free(tam_sched *s);
// `alt`: the array odd turns read in the forward fill (a RotationPair's
// partner), onto which their transposes add; null: `y` itself.
cudaError_t adjoint_run(tam_sched *s, void *y, void *alt, int nvars, const void *factors,
                        const int32_t *rotvars, int32_t first, int32_t last, void *scratch,
                        cudaStream_t stream);

// A batch's plan from its members' (each member's groups, transfers and
// weights at the given bases of the batch's concatenated arrays; `stages`
// the batch's stages, whose tags the plan's stages follow).
int adjoint_prepare_batch(AdjPlan &plan, const std::vector<tam_sched *> &members,
                          const std::vector<int64_t> &group_base,
                          const std::vector<int64_t> &transfer_base,
                          const std::vector<int64_t> &weight_base,
                          const std::vector<Stage> &stages, std::string &err);
void adjoint_plan_free(AdjPlan &plan);

// The arrays a run of a plan reads beside it.
struct AdjRun {
  int dtype, D;
  const DevGroup *groups;
  const int32_t *tb;
  const void *weights;
  const Member *members;           // a batch's member table, or null
  const Tile *fwd_tiles;           // the forward fill's tiles (the zero pass)
  const std::vector<Stage> *fwd_stages;
  int S[3];                        // stored extents (a batch: each member's own)
  const SoloGroup *turns;          // the solo groups (their targets are zeroed too)
  const int32_t *rotvars;          // the variable table of turned groups, or null
  int32_t *err;                    // error word: a variable table naming no variable
  void *alt;                       // odd turns' sources (a RotationPair's partner), or null
};
cudaError_t adjoint_run_plan(const AdjPlan &plan, const AdjRun &r, void *y, int nvars,
                             const void *factors, int32_t first, int32_t last, void *scratch,
                             cudaStream_t stream);

}  // namespace tam
