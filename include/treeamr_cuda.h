/*
 * treeamr_cuda.h -- C ABI of libtreeamr_cuda.so, the GB300 ghost-fill engine.
 *
 * The reference (TreeAMR.jl) replays a precomputed GhostSchedule of
 * TransferGroups with one KernelAbstractions launch per group
 * (src/ghosts.jl:372-402 transfer_kernel!, :420-521 run_group!,
 * :563-593 run_phase!, :1099-1160 exchange_ghosts!).  This library takes the
 * same schedule, flattened once into the plain arrays below by the host that
 * built it (src/schedule.jl:3075-3292 GhostSchedule, :2970 local_groups), and
 * replays it on one GPU.
 *
 * Conventions, all the reference's own so a Julia caller passes its arrays
 * unchanged:
 *   - work is column-major (S_1, ..., S_D, nvars, nblocks), index 1 fastest
 *     (src/storage.jl:364-472); S_d = N + 2 G_d + c_d.
 *   - block indices and stored indices are 1-based.
 *   - a stencil column i holds `order` weights, weights[w + order*i + m].
 *   - the factor table is nvars x ncols column-major (src/storage.jl:536-551).
 *   - pointers to field data (work, factors) are device pointers owned by the
 *     caller; the library borrows them for the call only.
 *   - every entry point returns TAM_OK (0) or a negative tam_status, never
 *     aborts and never traps; tam_last_error() says why.
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy default).
 */
#ifndef TREEAMR_CUDA_H
#define TREEAMR_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TAM_ABI_VERSION 2
#define TAM_MAX_DIM 3

enum tam_status {
  TAM_OK = 0,
  TAM_EINVAL = -1,        /* an argument or descriptor is malformed        */
  TAM_ECUDA = -2,         /* a CUDA call failed                            */
  TAM_ENOMEM = -3,        /* device allocation failed                      */
  TAM_ELAYOUT = -4,       /* field set does not match the schedule layout  */
  TAM_ETIMEOUT = -5,      /* a bounded device wait gave up                 */
  TAM_EUNSUPPORTED = -6   /* a feature the schedule asks for is not built  */
};

enum tam_dtype { TAM_F32 = 1, TAM_F64 = 2 };
enum tam_kind { TAM_COPY = 1, TAM_RESTRICT = 2, TAM_PROLONG = 3 };

/* Stage tags, ascending in the order a fill runs them
 * (src/schedule.jl:640-642, src/ghosts.jl:1099-1160). */
#define TAM_STAGE_SELFIMAGE (-1) /* stage P: wall-plane projection   */
#define TAM_STAGE_UNIFY 0        /* stage 0: secondaries <- primary  */
#define TAM_STAGE_PHASE1 1       /* copies and restrictions          */
#define TAM_STAGE_PROLONG(l) (2 + (l)) /* prolongations onto level l */
#define TAM_STAGE_ALL_FIRST (-1)
#define TAM_STAGE_ALL_LAST 0x7fffffff

/* One dimension of a transfer: Stencil1D (src/schedule.jl:64-93). */
typedef struct tam_stencil {
  int32_t targetfirst; /* 1-based stored index of the first target row   */
  int32_t ntarget;     /* target rows                                    */
  int32_t order;       /* weights per column                             */
  int32_t unit;        /* 1: one point of weight exactly one (a copy)    */
  int64_t srcstart;    /* offset into srcstart pool: ntarget entries     */
  int64_t weights;     /* offset into weight pool: order*ntarget entries */
} tam_stencil;

/* One TransferGroup (src/schedule.jl:150-197): the transfers
 * (targetblocks[first+t], sourceblocks[first+t]), t < ntransfers. */
typedef struct tam_group {
  int32_t kind;      /* tam_kind                                          */
  int32_t stage;     /* stage tag (transfer_stage, src/schedule.jl:656)   */
  int32_t factorcol; /* 0, or the 1-based factor-table column             */
  /* 0, or how the kernel bounds the result (boundedmode,
   * src/operators.jl:417-441): 1 the bounded conservative prolongation
   * (order-3 stencils, the parent at the window's middle row,
   * src/ghosts.jl:291-310), 2 the point-value sum clamped into its bracket
   * (stencils of 2p rows: the order-p weights, then the linear ones over the
   * same window, src/ghosts.jl:311-361).  A bounded group runs in a launch of
   * its own after its stage's fused launches; a schedule with one has no
   * adjoint. */
  int32_t bounded;
  /* A turned group (across a rotating or half-turn seam, TransferGroup's
   * orientation/perm/flip, src/schedule.jl:150-197, src/ghosts.jl:183-244):
   * orientation r in 1..3 (0: an ordinary group), and its axis map in
   * gather form, `axes` = sum_e perm[e] << 2e  +  flip[e] << (8 + e) with
   * 0-based dimensions: virtual stored index k reads the real point whose
   * index along e is k[perm[e]], or R_e + 1 - k[perm[e]] where flip[e], and
   * variable rotvars[v + nvars * r] (1-based) of the real source, an array
   * of stored extent R_e = S[perm[e]] along e.  An odd orientation reads the
   * alternate array of tam_fill_ex: the set's own when its layout is
   * symmetric in the seam's plane, else its RotationPair partner's, the
   * swapped layout. */
  int32_t orientation;
  int32_t axes;
  int64_t first;     /* offset into the block lists                        */
  int64_t ntransfers;
  tam_stencil stencil[TAM_MAX_DIM]; /* dimensions >= ndim are ignored      */
} tam_group;

/* A whole schedule, as host arrays (read during the call only). */
typedef struct tam_schedule_desc {
  int32_t abi_version;        /* TAM_ABI_VERSION                           */
  int32_t ndim;               /* D in 1..3                                 */
  int32_t dtype;              /* tam_dtype of the weights and of work      */
  int32_t stored[TAM_MAX_DIM];/* S_d                                       */
  int64_t nblocks;
  int32_t ngroups;
  int32_t nfactorcols;        /* 3^D, or 4 * 3^D over a seam (the columns
                                 mirror + 3^D r, src/storage.jl:717-740)   */
  const tam_group *groups;
  int64_t ntransfers;         /* length of both block lists                */
  const int32_t *targetblocks;/* 1-based                                   */
  const int32_t *sourceblocks;/* 1-based                                   */
  int64_t nsrcstart;
  const int32_t *srcstart;    /* 1-based stored indices                    */
  int64_t nweights;
  const void *weights;        /* float or double per dtype                 */
} tam_schedule_desc;

typedef struct tam_ctx tam_ctx;
typedef struct tam_sched tam_sched;

/* Library version: TAM_ABI_VERSION. */
int tam_abi_version(void);

/* Open the library on a CUDA device.  Replaces the reference's backend
 * selection (src/device.jl:1-34 todevice / get_backend). */
int tam_init(int device, tam_ctx **out);
void tam_free(tam_ctx *ctx);

/* The last error message of this context (or of the library when ctx is
 * NULL), NUL-terminated into buf. */
int tam_last_error(const tam_ctx *ctx, char *buf, size_t n);

/* Validate a flattened schedule and upload it once.  Replaces
 * todevice(backend, ::TransferGroup) and local_groups
 * (src/schedule.jl:184-188, 2970-2992).  Every stencil window and block
 * index is checked against the layout here, so no fill can read or write
 * outside `work`. */
int tam_schedule_upload(tam_ctx *ctx, const tam_schedule_desc *desc, tam_sched **out);
void tam_schedule_free(tam_sched *s);

/* Counts of the uploaded schedule: groups, transfers, point-variables per
 * variable written (sum ntransfers * prod ntarget), stages. */
int tam_schedule_info(const tam_sched *s, int64_t *ngroups, int64_t *ntransfers,
                      int64_t *points, int32_t *nstages);

/* The fused fill: every stage tag in [first_stage, last_stage], in order,
 * each stage one batched launch over all its groups' transfers, grouped by
 * target block.  Replaces exchange_ghosts! / run_stages! / run_phase! for a
 * serial forest (src/ghosts.jl:1099-1160, 988-1007, 563-570).  A boundary
 * hook runs between two calls: [-1, 1] then [2, TAM_STAGE_ALL_LAST]
 * (src/ghosts.jl:1134-1136).  `factors` may be NULL when no group has a
 * factor column.  Asynchronous on `stream`. */
int tam_fill(tam_sched *s, void *work, int32_t nvars, int64_t nblocks,
             const void *factors, int32_t first_stage, int32_t last_stage,
             void *stream);

/* tam_fill and tam_fill_plain with what a turned group reads
 * (run_group!'s altsrc and rotvars, src/ghosts.jl:420-490): `rotvars`, a
 * device table of nvars x 4 int32 (column-major, 1-based variables; the
 * field set's variable map per orientation), required when the schedule has
 * a turned group, and `alt_work`, the array an odd orientation reads (a
 * RotationPair's partner; NULL: `work` itself).  `method` is
 * TAM_METHOD_FUSED or TAM_METHOD_PLAIN.  A turned group runs in its own
 * launch after the stage's fused launches. */
#define TAM_METHOD_FUSED 0
#define TAM_METHOD_PLAIN 1
int tam_fill_ex(tam_sched *s, void *work, const void *alt_work, int32_t nvars,
                int64_t nblocks, const void *factors, const int32_t *rotvars,
                int32_t first_stage, int32_t last_stage, int32_t method, void *stream);

/* The fill of a field set whose data live in host memory (the reference's
 * fill_ghosts!, src/ghosts.jl:1783, on host arrays): asynchronous on
 * `stream`, host_in (nblocks * nvars * S1*S2*S3 elements in the layout of
 * tam_fill) is copied into device_work, the stages [first_stage, last_stage]
 * are filled there as tam_fill fills them, and device_work is copied back
 * into host_out (which may be host_in).  Page-locked host buffers let the
 * copies run on the copy engines beside other streams' work: a caller that
 * fills a sequence of field states round-robin over two or three streams,
 * each with its own device buffer, keeps one state's upload, another's fill
 * and a third's download in flight together.  factors is a device pointer,
 * as for tam_fill. */
int tam_fill_host(tam_sched *s, const void *host_in, void *host_out, void *device_work,
                  int32_t nvars, int64_t nblocks, const void *factors, int32_t first_stage,
                  int32_t last_stage, void *stream);

/* The regrid transfer (src/regrid.jl:585-756, 942-955): the serial transfer
 * groups from the leaves before a refinement or coarsening (sources, blocks
 * of the old array) to the leaves after (targets, blocks of the new array),
 * every target the new block's own range: a copy of a kept leaf, a
 * prolongation from the parent of a created one, a restriction from each
 * child of a coarsened one.  tam_regrid_upload takes the descriptor with
 * nblocks the new count and the old count beside it; tam_regrid_transfer
 * reads old_work and writes new_work (distinct arrays of one layout),
 * asynchronous on stream.  The ghosts are left to the next fill. */
int tam_regrid_upload(tam_ctx *ctx, const tam_schedule_desc *desc, int64_t old_nblocks,
                      tam_sched **out);
int tam_regrid_transfer(tam_sched *s, const void *old_work, int64_t old_nblocks,
                        void *new_work, int64_t new_nblocks, int32_t nvars, void *stream);

/* The plain fill: one launch per TransferGroup, one thread per
 * point-variable, as the reference's device path launches transfer_kernel!
 * (src/ghosts.jl:420-521).  Same arguments and results as tam_fill. */
int tam_fill_plain(tam_sched *s, void *work, int32_t nvars, int64_t nblocks,
                   const void *factors, int32_t first_stage, int32_t last_stage,
                   void *stream);

/* The adjoint (transpose) of the fill: y <- A^T y, stages in reverse, in
 * gather form (deterministic, no atomics).  No reference counterpart: the
 * reference has no adjoint; this is the kernel a ChainRulesCore rrule of
 * fill_ghosts! (src/ghosts.jl:1783) would call for its pullback.  For each
 * stage s, y <- (I - E_s) y + A_s^T E_s y with E_s the stage's targets: the
 * ghosts' adjoints are pushed onto the points their values came from, and
 * the ghosts' own adjoints are zeroed.  Stage P, which scales each point of
 * a reflecting wall plane in place by its variable's factor, is diagonal
 * and its own transpose: it runs as in the fill.  Same arguments as tam_fill; `y`
 * has the layout of `work`.  The library allocates its scratch on the
 * first call with a given nvars (so make that call before any stream
 * capture).  A schedule with a turned group (a seam) needs the variable
 * table: use tam_fill_adjoint_ex.  A stencil transfer's transpose runs in
 * one CTA's shared memory (its target box, two intermediate boxes and its
 * transposed stencils); a schedule with a transfer too large for it is
 * refused with TAM_EUNSUPPORTED on the first call.  In 3-D at order 4 the
 * largest is an x-face prolongation (G x N x N points): blocks of N up to 56
 * fit in Float64, up to 80 in Float32. */
int tam_fill_adjoint(tam_sched *s, void *y, int32_t nvars, int64_t nblocks,
                     const void *factors, int32_t first_stage, int32_t last_stage,
                     void *stream);

/* Scratch bytes tam_fill_adjoint_scratch needs for `nvars` variables. */
int tam_adjoint_scratch_bytes(tam_sched *s, int32_t nvars, size_t *bytes);

/* The adjoint with the variable table of a schedule that turns transfers
 * across a seam (the field set's rotvars, as tam_fill_ex takes it; NULL
 * without turned groups), with the caller's scratch, or, when `scratch` is
 * NULL, the library's own.  A turned group's transpose adds onto its real
 * source in the set's own array, so a RotationPair member (a layout not
 * symmetric in the seam's plane) is refused with TAM_EUNSUPPORTED. */
int tam_fill_adjoint_ex(tam_sched *s, void *y, int32_t nvars, int64_t nblocks,
                        const void *factors, const int32_t *rotvars, int32_t first_stage,
                        int32_t last_stage, void *scratch, size_t scratch_bytes,
                        void *stream);

/* The adjoint of tam_fill_ex with `alt_work`: the transposes of odd turns add
 * onto `alt_y` (the partner's cotangent, in the partner's layout), the rest
 * onto `y`.  The adjoint of a RotationPair fill runs, stage tag by stage tag
 * from the last, the second member's stage, then the first's, each with the
 * other's cotangent as `alt_y` (the forward order reversed).  NULL `alt_y`:
 * tam_fill_adjoint_ex. */
int tam_fill_adjoint_alt(tam_sched *s, void *y, void *alt_y, int32_t nvars, int64_t nblocks,
                         const void *factors, const int32_t *rotvars, int32_t first_stage,
                         int32_t last_stage, void *scratch, size_t scratch_bytes,
                         void *stream);

/* tam_fill_adjoint with caller-owned device scratch of at least
 * tam_adjoint_scratch_bytes; allocates nothing per call. */
int tam_fill_adjoint_scratch(tam_sched *s, void *y, int32_t nvars, int64_t nblocks,
                             const void *factors, int32_t first_stage, int32_t last_stage,
                             void *scratch, size_t scratch_bytes, void *stream);

/* tam_fill_adjoint for callers that must not allocate device memory while
 * they run -- a solver inside someone else's memory pool or arena, a code
 * path that must never trigger the synchronisation cudaMalloc/cudaFree
 * imply, or an allocator-free real-time loop.  It has no counterpart in the
 * reference.  Its scratch is a fixed array compiled into the library,
 * TAM_STATIC_SCRATCH_BYTES (64 MiB) on every GPU that loads the library,
 * held until the process exits; a schedule whose adjoint needs more for
 * `nvars` variables (tam_adjoint_scratch_bytes) is refused with
 * TAM_EUNSUPPORTED.  Set-up that does allocate must come first: the
 * schedule's transposed stencils are built by tam_adjoint_scratch_bytes (or
 * a first tam_fill_adjoint), and a schedule without them is refused with
 * TAM_EINVAL.  The first call on each device looks up the array's device
 * address once (cudaGetSymbolAddress); make that first call before any
 * stream capture.  The address is kept for the life of the process: after
 * cudaDeviceReset (or anything else that destroys the device's primary
 * context) the kept address is stale, so a caller that resets a device
 * must not call this entry point on it again.  All calls share the one array and leave their results in
 * it, so calls that overlap on the GPU (two streams, two threads) race and
 * must be serialised by the caller.  Nothing in the array needs to start
 * at zero: each call writes every scratch element before reading it. */
#define TAM_STATIC_SCRATCH_BYTES ((size_t)64 << 20)
int tam_fill_adjoint_static(tam_sched *s, void *y, int32_t nvars, int64_t nblocks,
                            const void *factors, int32_t first_stage, int32_t last_stage,
                            void *stream);

/* A batch: several independent forests filled together, one launch per
 * stage for all of them.  No reference counterpart (the reference fills one
 * field set per call, src/ghosts.jl:1783); this is the multi-forest form of
 * tam_fill for field data laid out in one arena, each member's `work`
 * (column-major, its own S_d and nblocks, `nvars` shared) starting at
 * work_offsets[m] elements and its factor table at factor_offsets[m]
 * (NULL when no member mirrors).  Members share dimension and element type;
 * they stay owned by the caller and must outlive the batch. */
typedef struct tam_batch tam_batch;
int tam_batch_create(tam_ctx *ctx, tam_sched *const *members, int32_t n,
                     const int64_t *work_offsets, const int64_t *factor_offsets,
                     tam_batch **out);
void tam_batch_free(tam_batch *b);
/* Every stage tag in [first_stage, last_stage] of every member; the arena
 * holds arena_elems elements (checked against every member's extent), the
 * factor arena each member's nvars * nfactorcols table.  Members may turn
 * transfers across a seam (a member's odd turns read its own array, so a
 * RotationPair member, whose layout is not symmetric in the seam's plane, is
 * refused by tam_batch_create) or bound them; their solo groups run after
 * each stage's fused launches, one launch for all members. */
int tam_batch_fill(tam_batch *b, void *arena, int64_t arena_elems, int32_t nvars,
                   const void *factor_arena, int64_t factor_elems, int32_t first_stage,
                   int32_t last_stage, void *stream);
/* tam_batch_fill with the variable table of turned transfers (tam_fill_ex's
 * `rotvars`, nvars x 4, shared by every turned member); required when a
 * member turns transfers, may be NULL otherwise. */
int tam_batch_fill_ex(tam_batch *b, void *arena, int64_t arena_elems, int32_t nvars,
                      const void *factor_arena, int64_t factor_elems, const int32_t *rotvars,
                      int32_t first_stage, int32_t last_stage, void *stream);
/* The adjoint of tam_batch_fill, member by member (tam_fill_adjoint); a batch
 * with a bounded member has none (TAM_EUNSUPPORTED). */
int tam_batch_fill_adjoint(tam_batch *b, void *arena, int64_t arena_elems, int32_t nvars,
                           const void *factor_arena, int64_t factor_elems,
                           int32_t first_stage, int32_t last_stage, void *stream);
/* The adjoint of tam_batch_fill_ex. */
int tam_batch_fill_adjoint_ex(tam_batch *b, void *arena, int64_t arena_elems, int32_t nvars,
                              const void *factor_arena, int64_t factor_elems,
                              const int32_t *rotvars, int32_t first_stage, int32_t last_stage,
                              void *stream);
/* tam_device_status for a batch: its solo launches' error word (a variable
 * table naming no variable), read on `stream` and cleared. */
int tam_batch_device_status(tam_batch *b, void *stream, int32_t *code);
/* tam_schedule_set_option for a batch. */
int tam_batch_set_option(tam_batch *b, int32_t option, int64_t value);

/* The second-order wave equation's right-hand side, u_t = v, v_t = lap(u)
 * with the 7-point Laplacian, over every owned point of every listed block
 * (the RHS of the reference's wave test, test/wave.jl:49-110; the
 * application step around the fill, `map_blocks!`, src/state.jl:393).
 * Cell-centred blocks with G >= 1; u is variable 1 of a block and v
 * variable 2.  adjoint = 0: out = f(in) at owned points (out's ghosts are
 * left alone).  adjoint = 1: out = f^T(in) at every stored point.  `blocks`
 * is a device array. */
typedef struct tam_wave_block {
  int64_t off;     /* element offset of the block's variable u            */
  int32_t S[3];    /* stored extents                                      */
  int32_t G;       /* ghost width                                         */
  int32_t N;       /* owned cells per dimension                           */
  int32_t pad;
  double inv_h2;   /* 1 / h^2 of the block's level                        */
} tam_wave_block;
int tam_wave_rhs(int32_t dtype, const tam_wave_block *blocks, int32_t nblocks,
                 int32_t max_points_per_block, const void *in, void *out, int32_t adjoint,
                 void *stream);
/* One stage of classical RK4 around that right-hand side, at every stored
 * point: k = R(x) (zero at ghosts), t_out = y + ct*k (when t_out is not
 * NULL) and acc_out = (acc_in, or y when NULL) + ca*k, so a step's stage
 * states and weighted sum need no stored k.  x's ghosts must be filled; x
 * may not be t_out or acc_out; acc_out may be acc_in. */
int tam_wave_rk4_stage(int32_t dtype, const tam_wave_block *blocks, int32_t nblocks,
                       int32_t max_points_per_block, const void *x, const void *y,
                       void *t_out, const void *acc_in, void *acc_out, double ct, double ca,
                       void *stream);
/* `steps` RK4 steps of the wave equation over a batch of forests as one CUDA
 * graph: per step four tam_batch_fill calls, each followed by one
 * tam_wave_rk4_stage (stage states in `ta` and `tb`, the step's sum in
 * `acc`, the state `y` advanced in place), captured on a private stream of
 * `device` (nothing runs at capture).  tam_graph_launch replays it on a
 * stream; the arrays, the batch and the block table must outlive the graph.
 * The reference replays every launch from the host each step. */
typedef struct tam_graph tam_graph;
int tam_graph_capture_rk4(tam_batch *b, int32_t dtype, const tam_wave_block *blocks,
                          int32_t nblocks, int32_t max_points_per_block, void *y, void *ta,
                          void *tb, void *acc, int64_t arena_elems, int32_t nvars,
                          const void *factor_arena, int64_t factor_elems, double dt,
                          int32_t steps, int32_t device, tam_graph **out);
int tam_graph_launch(tam_graph *g, void *stream);
void tam_graph_free(tam_graph *g);

/* The transpose of a stage's right-hand side with its cotangent formed on
 * the fly: out = R^T (c1*g + c2*xprev) (xprev may be NULL), and when ybar is
 * not NULL, ybar += xprev at every stored point.  out may alias none of g,
 * xprev, ybar; ybar may not alias xprev. */
int tam_wave_rk4_adjoint_stage(int32_t dtype, const tam_wave_block *blocks, int32_t nblocks,
                               int32_t max_points_per_block, const void *g, double c1,
                               const void *xprev, double c2, void *out, void *ybar,
                               void *stream);

/* The cell-wise boundary hook on the device (CellBoundary,
 * src/ghosts.jl:1166-1318) with a built-in function of position: every ghost
 * of every region beyond an outer face gets g(x, v), x formed as
 * nodeposition forms it (fma(T(m), s, lo), src/storage.jl:1008-1017).
 * TAM_BC_CONSTANT: g = coef[v].  TAM_BC_POLYNOMIAL: g = sum over the terms q
 * of ((coef[v*nterms+q] * x1^a) * x2^b) * x3^c, (a, b, c) = exps[q], powers
 * by repeated multiplication, summed in term order from +0, every operation
 * rounded once.  With fn.relative, the relative form (Relative,
 * src/ghosts.jl:1431-1475): g(x_g) + (u(r) - g(x_r)), r the ghost's index
 * with clamps[d] in place of it where clamps[d] != 0, read from work.
 * Regions and coef are device arrays; regions' blocks are 0-based, first
 * 1-based stored indices.  Asynchronous on stream. */
#define TAM_BC_CONSTANT 1
#define TAM_BC_POLYNOMIAL 2
#define TAM_BC_MAX_TERMS 20
typedef struct tam_boundary_region {
  int32_t block;       /* 0-based                                            */
  int32_t first[3];    /* 1-based stored index of the region's first point  */
  int32_t n[3];        /* extent per dimension (1 beyond ndim)              */
  int32_t ghosts[3];   /* the layout's ghost widths G_d                      */
  int32_t stagger[3];  /* c_d: 1 vertex-like, 0 cell-like                    */
  int32_t clamps[3];   /* relative form: the nearest evolved point's stored */
                       /* index along d, or 0 (the ghost's own index)        */
  int32_t pad;
  int64_t base[3];     /* the block's integer base B_d (nodeposition)        */
  double lo[3];        /* the domain's low corner along d, in T              */
  double h;            /* the block's spacing, in T                          */
} tam_boundary_region;
typedef struct tam_boundary_fn {
  int32_t kind;
  int32_t nterms;
  int32_t relative;    /* 1: Relative(g), the ghost is g(x_g) + (u(r) - g(x_r)) */
  int32_t exps[TAM_BC_MAX_TERMS][3];
} tam_boundary_fn;
int tam_boundary_apply(int32_t dtype, const tam_boundary_region *regions, int32_t nregions,
                       tam_boundary_fn fn, const void *coef, void *work, int32_t nvars,
                       const int32_t stored[3], void *stream);

/* The state vector and the working array (src/state.jl:101-160): the
 * state holds every block's own points only, shape (own_1, own_2, own_3,
 * nvars, nblocks) column-major with own_d = N + c_d; own point i_d is stored
 * index ghosts_d + i_d (0-based) of the working array (stored_1, stored_2,
 * stored_3, nvars, nblocks).  Unused dimensions: own = stored = 1, ghosts = 0. */
typedef struct tam_state_layout {
  int32_t dtype;       /* TAM_F32 or TAM_F64                                */
  int32_t ndim;
  int32_t own[3];
  int32_t stored[3];
  int32_t ghosts[3];
  int32_t nvars;
  int64_t nblocks;
} tam_state_layout;
/* scatter!: state -> the working array's own points; ghosts untouched.
 * gather!: the working array's own points -> state.  Device pointers,
 * asynchronous on `stream`; bits are copied, NaN payloads and -0 kept. */
int tam_scatter(const tam_state_layout *layout, const void *state, void *work, void *stream);
int tam_gather(const tam_state_layout *layout, const void *work, void *state, void *stream);

/* A seam's axis projection (stage P's axis part, axis_project!,
 * src/ghosts.jl:599-660, 736-770), run after stage P and before stage 0:
 * each of the `npoints` axis points, at element offset points[i] of its
 * variable 0 in `work` (block * nvars * block_points + its offset in the
 * block), gets for every variable v the mean of its images under the
 * orbit's powers of the set's map, t_r = factors[v + nvars * ncol * r] *
 * work[.. variable rotvars[v + nvars * r] - 1 ..] (t_0 the value itself),
 * summed in pairs a half turn apart: ((t_0 + t_2) + (t_1 + t_3)) / 4 for
 * members = 4 (a quarter turn) or (t_0 + t_2) / 2 for members = 2 (a half
 * turn).  `buffer` (npoints * nvars elements) holds the means, all gathered
 * before any is written.  ncol is 3^D, the factor table's columns per
 * orientation.  A variable table naming no variable gives NaN.  The
 * projection's transpose (for the adjoint fill, between stage 0's transpose
 * and stage P's) is the same call with each column r of the variable table
 * inverted and each factor moved with its variable: rotvars'[w, r] = v and
 * factors'[w, ncol r] = factors[v, ncol r] where rotvars[v, r] = w. */
int tam_axis_project(int32_t dtype, const int64_t *points, int64_t npoints, int32_t members,
                     void *work, int32_t nvars, int64_t block_points, const void *factors,
                     int32_t ncol, const int32_t *rotvars, void *buffer, void *stream);

/* tam_fill_host moving only what the fill reads up: the own points of
 * host_in (the box `layout` describes, ghosts[d] .. ghosts[d] + own[d] - 1
 * along d) are copied into device_work by a kernel that reads host_in
 * through its device mapping (so host_in must be page-locked: cudaHostAlloc
 * or cudaHostRegister), the stages [first_stage, last_stage] are filled,
 * and device_work comes back into host_out whole.  The fill reads own
 * points only, so every point it writes is as tam_fill_host would leave
 * it; a point neither own nor written by the fill (a hook region) comes
 * back as device_work held it.  Asynchronous on `stream`. */
int tam_fill_host_own(tam_sched *s, const tam_state_layout *layout, const void *host_in,
                      void *host_out, void *device_work, int32_t nvars, int64_t nblocks,
                      const void *factors, int32_t first_stage, int32_t last_stage,
                      void *stream);


/* Launch options of the fused fill, per schedule (no reference counterpart:
 * the reference has no tuning; these are what the autotuner sets).  Changing
 * one changes speed only, never a result. */
#define TAM_OPT_TILE_ITEMS 1 /* box points per warp tile, 16..4096           */
#define TAM_OPT_THREADS 2    /* threads per CTA, 64..512, a multiple of 32    */
#define TAM_OPT_INT_MUL 3    /* 1: Float64 stencil multiplies on the integer  */
                             /* pipe (see tam_selftest), 0: FP64 pipe          */
/* The form of the stencil sum (src/ghosts.jl:28-56): 1 (the default) is the
 * reference's CPU form, a dimension whose weight column has one nonzero
 * weight takes that one tap; 0 is its device form, every tap.  The two give
 * the same bits for finite data; they differ only where a NaN or an infinity
 * sits under a zero weight, which the full sum carries into the result.
 * tam_fill_plain always takes the device form. */
#define TAM_OPT_ONE_TAP 4
/* Points a lane of the unit-copy launches takes at once, 1 (the default), 2
 * or 4: each point's every variable is loaded before any is stored, so more
 * points a lane put more loads in flight a warp, for more registers a
 * thread. */
#define TAM_OPT_COPY_POINTS 5
/* The order in which a fill's launches visit target blocks: 0 (the default)
 * the blocks' own order, 1 a reverse Cuthill-McKee order of the graph of
 * the schedule's transfers, which keeps blocks that exchange ghosts close
 * together in time (the sectors they share stay in L2); 2 by source block
 * first (the blocks' own order), then target: the transfers that read one
 * block run together, so each source sector comes from DRAM once; 3 the
 * copies by target block and the stencils by source block. */
#define TAM_OPT_BLOCK_ORDER 6
/* 1: a stage's stencil points grouped by their path through the kernel
 * (the order class and, in the CPU form, the dimensions that take one tap),
 * so that no warp mixes paths; 0: by target block only.  The default is 1
 * for Float64 (the FP64 pipe spends a warp instruction's time whatever
 * lanes are off) and 0 for Float32. */
#define TAM_OPT_PATH_TILES 7
/* 1 (the default): consecutive prolongation stages none of whose points
 * conflict (src/schedule.jl:2735-2931, stage_groups) run as one launch pair
 * when a fill's stage range holds them all; 0: one launch pair a stage. */
#define TAM_OPT_MERGE_STAGES 8
/* The stage groups the schedule found: how many, and how many stages they
 * hold in all (a whole fill runs `nstages - stages_in_groups + groups`
 * launch pairs).  No reference counterpart beyond stage_groups itself. */
int tam_schedule_stage_groups(const tam_sched *s, int32_t *groups, int32_t *stages_in_groups);
/* 1: every stencil transfer of a large box (64 points or more, its source
 * window within 48 KiB a variable) runs in a kernel that stages the window
 * in shared memory, a CTA a transfer, and sums each point's taps from there;
 * 0 (the default): every stencil point reads its taps in place.  The same
 * bits either way. */
#define TAM_OPT_STAGED 9
/* 1: a Float64 order-4 stencil point sums two variables at a time (two
 * independent chains sharing each tap's weight product); 0 (the default):
 * one at a time.  The same bits either way. */
#define TAM_OPT_PAIR_VARS 10
/* How a stage's unit copies share the GPU with its stencils: 0 (the
 * default) the stencil launch first and the copies after it, each with a
 * CTA for every few tiles; n > 0 the copy launch first with n CTAs per
 * multiprocessor, walking its tiles grid-strided, and the stencil launch
 * beside it, whose CTAs fill the rest of every multiprocessor and take over
 * the copies' room as they finish: memory-bound copies and FP64-bound
 * stencils on the same multiprocessors at once.  The same bits either way. */
#define TAM_OPT_COPY_SHARE 11
/* 1: in Float64 order-4 stencils with the integer-pipe multiply, the last
 * tap of every row of four adds on the integer pipe (an exact
 * round-to-nearest adder, tam_selftest 2) instead of the FP64 pipe, which
 * GB300 gives 1/64 of the FP32 rate; the sum keeps the reference's order,
 * so the same bits.  0 (the default): every add on the FP64 pipe. */
#define TAM_OPT_SOFT_ADD 12
/* Box points per warp tile of the stencils, 16..4096, or 0 (the default):
 * TAM_OPT_TILE_ITEMS for copies and stencils alike.  Copies want short
 * tiles (their warps wait on memory), order-4 stencils longer ones. */
#define TAM_OPT_STENCIL_TILE 13
int tam_schedule_set_option(tam_sched *s, int32_t option, int64_t value);
int tam_schedule_get_option(const tam_sched *s, int32_t option, int64_t *value);

/* The launch-option autotuner: times every combination of TAM_OPT_TILE_ITEMS
 * (32 .. 512), TAM_OPT_THREADS (128, 256, 512) and, for Float64,
 * TAM_OPT_INT_MUL (0, 1) on the caller's own field data (which should be
 * representative: zeros, subnormals and specials send the integer-pipe
 * multiplies' points back to the FP64 pipe) (best of `reps`
 * fills after a warm-up, CUDA events on `stream`), then, from the fastest,
 * TAM_OPT_MERGE_STAGES, TAM_OPT_PATH_TILES, TAM_OPT_STAGED,
 * TAM_OPT_PAIR_VARS (Float64), TAM_OPT_BLOCK_ORDER, TAM_OPT_COPY_POINTS and
 * TAM_OPT_COPY_SHARE (0, 1, 2, 4), TAM_OPT_STENCIL_TILE (0, 32, 64, 128) and,
 * for Float64, TAM_OPT_SOFT_ADD one at a time, twice over; leaves the
 * fastest set and returns the first three (the others through
 * tam_schedule_get_option).  The fills overwrite `work`'s ghosts (never an
 * own point).  Synchronizes `stream`; re-tiling allocates, so not inside a
 * stream capture.  The reference has no tuning. */
int tam_autotune(tam_sched *s, void *work, int32_t nvars, int64_t nblocks, const void *factors,
                 int32_t reps, void *stream, int64_t *tile_items, int64_t *threads,
                 int64_t *int_mul, double *best_ms);

/* Read (and clear) the device error word of the schedule's last fills:
 * 0, or a tam_status a kernel recorded.  Synchronizes `stream`. */
int tam_device_status(tam_sched *s, void *stream, int32_t *code);

/* Built-in self-test, no reference counterpart: which = 1 compares the
 * integer-pipe Float64 multiply the fills use for short weight products
 * with the hardware multiply on n pseudo-random pairs (all bit patterns of
 * the data, specials included) and returns the number of results that
 * differ in any bit (NaNs compared as one pattern).  which = 2 compares the
 * integer-pipe Float64 add (TAM_OPT_SOFT_ADD) with the hardware add on n
 * pairs of a running sum (every kind of value) and a product (normal),
 * weighted to equal and adjacent exponents, cancellations and the edges of
 * the normal range, and returns the results that differ in any bit (pairs
 * the adder hands back to the FP64 pipe are not compared).  which = 3
 * compares the integer-pipe multiply of weights of any width (the Float64
 * order-6 products) with the hardware multiply on n pairs of normal
 * factors, exponents across the range and products near its edges.
 * Synchronous. */
#define TAM_SELFTEST_MUL 1
#define TAM_SELFTEST_ADD 2
#define TAM_SELFTEST_MUL_FULL 3
int tam_selftest(tam_ctx *ctx, int32_t which, int64_t n, uint64_t seed, int64_t *mismatches);

#ifdef __cplusplus
}
#endif
#endif /* TREEAMR_CUDA_H */
