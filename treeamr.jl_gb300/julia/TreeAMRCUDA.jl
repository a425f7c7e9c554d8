# TreeAMRCUDA.jl -- the ccall side of libtreeamr_cuda.so for TreeAMR.jl.
#
# A package extension a TreeAMR.jl maintainer adds (it loads with CUDA.jl):
# it flattens each GhostSchedule once into the struct-of-arrays descriptor
# of include/treeamr_cuda.h, uploads it, and routes fill_ghosts! of a
# CuArray field set through tam_fill, with the boundary hook between phase 1
# and the prolongations exactly where exchange_ghosts! runs it
# (src/ghosts.jl:1099-1160).  The adjoint is exposed as a ChainRulesCore
# rrule.  Written against the reference's own types (src/schedule.jl:64-197,
# 820-864; src/storage.jl:364-472); not executed in this repository, which
# has no Julia toolchain.
module TreeAMRCUDA

using TreeAMR
using TreeAMR: GhostSchedule, TransferGroup, Stencil1D, FieldSet, CellBoundary, RotationPair,
               hasrotating
using CUDA
import ChainRulesCore

const LIB = get(ENV, "TREEAMR_CUDA_LIB", joinpath(@__DIR__, "..", "csrc", "_build",
                                                  "libtreeamr_cuda.so"))

const TAM_ABI_VERSION = Int32(2)
const TAM_METHOD_FUSED, TAM_METHOD_PLAIN = Int32(0), Int32(1)
const TAM_F32, TAM_F64 = Int32(1), Int32(2)
const TAM_COPY, TAM_RESTRICT, TAM_PROLONG = Int32(1), Int32(2), Int32(3)
const STAGE_FIRST, STAGE_LAST = Int32(-1), typemax(Int32)

# include/treeamr_cuda.h: tam_stencil, tam_group, tam_schedule_desc
struct TamStencil
    targetfirst::Int32
    ntarget::Int32
    order::Int32
    unit::Int32
    srcstart::Int64
    weights::Int64
end

struct TamGroup
    kind::Int32
    stage::Int32
    factorcol::Int32
    bounded::Int32
    orientation::Int32   # a turned group's orientation (0: none)
    axes::Int32          # its axis map: perm[e] - 1 << 2(e-1), flip[e] << (7 + e)
    first::Int64
    ntransfers::Int64
    stencil::NTuple{3,TamStencil}
end

struct TamScheduleDesc
    abi_version::Int32
    ndim::Int32
    dtype::Int32
    stored::NTuple{3,Int32}
    nblocks::Int64
    ngroups::Int32
    nfactorcols::Int32
    groups::Ptr{TamGroup}
    ntransfers::Int64
    targetblocks::Ptr{Int32}
    sourceblocks::Ptr{Int32}
    nsrcstart::Int64
    srcstart::Ptr{Int32}
    nweights::Int64
    weights::Ptr{Cvoid}
end

function check(rc, ctx, what)
    rc == 0 && return nothing
    buf = Vector{UInt8}(undef, 1024)
    ccall((:tam_last_error, LIB), Cint, (Ptr{Cvoid}, Ptr{UInt8}, Csize_t), ctx, buf, length(buf))
    msg = unsafe_string(pointer(buf))
    rc == -1 ? throw(ArgumentError("$what: $msg")) : error("$what failed ($rc): $msg")
end

const CONTEXTS = Dict{Int,Ptr{Cvoid}}()
function context(dev::Int)
    get!(CONTEXTS, dev) do
        out = Ref{Ptr{Cvoid}}(C_NULL)
        check(ccall((:tam_init, LIB), Cint, (Cint, Ref{Ptr{Cvoid}}), dev, out), C_NULL,
              "tam_init")
        out[]
    end
end

kindcode(k::Symbol) = k === :copy ? TAM_COPY : k === :restrict ? TAM_RESTRICT : TAM_PROLONG

# The stage of a group: the stage tag its key had (src/schedule.jl:656-658),
# recovered from where the schedule filed it.
function stage_groups(s::GhostSchedule)
    out = Tuple{Int32,Any}[]
    foreach(g -> push!(out, (Int32(-1), g)), s.selfimage)
    foreach(g -> push!(out, (Int32(0), g)), s.unify)
    foreach(g -> push!(out, (Int32(1), g)), s.phase1)
    for (l, gs) in zip(s.levels, s.phase2)
        foreach(g -> push!(out, (Int32(2 + l), g)), gs)
    end
    return out
end

# Flatten a host-built schedule (the stencils on the CPU backend) into the
# descriptor's pools, upload it, and keep the handle.
mutable struct DeviceSchedule
    handle::Ptr{Cvoid}
    ctx::Ptr{Cvoid}
    generation::Int
end

function upload(s::GhostSchedule{T,D}, dev::Int=CUDA.device().handle) where {T,D}
    groups = TamGroup[]
    tb, sb, ss = Int32[], Int32[], Int32[]
    ws = T[]
    memo = IdDict{Any,Tuple{Int64,Int64}}()
    for (stage, g) in stage_groups(s)
        sts = ntuple(3) do d
            d > D && return TamStencil(1, 1, 1, 1, 0, 0)
            st = g.stencils[d]
            off = get!(memo, st) do
                o = (Int64(length(ss)), Int64(length(ws)))
                append!(ss, Array(st.srcstart))
                append!(ws, vec(Array(st.weights)))
                o
            end
            TamStencil(st.targetfirst, length(st.srcstart), size(st.weights, 1), st.unit,
                       off[1], off[2])
        end
        # a turned group's axis map (src/ghosts.jl:238-244), 0-based in the ABI
        axes = g.orientation == 0 ? Int32(0) :
               Int32(sum((Int(g.perm[e]) - 1) << (2 * (e - 1)) + Int(g.flip[e]) << (7 + e)
                         for e in 1:D))
        push!(groups, TamGroup(kindcode(g.kind), stage, g.factorcol, g.bounded,
                               g.orientation, axes, length(tb), length(g.targetblocks), sts))
        append!(tb, Array(g.targetblocks))
        append!(sb, Array(g.sourceblocks))
    end
    c = map(x -> x === :vertex ? 1 : 0, s.centering)
    stored = ntuple(d -> d <= D ? Int32(s.forest.N + 2s.G[d] + c[d]) : Int32(1), 3)
    ctx = context(dev)
    out = Ref{Ptr{Cvoid}}(C_NULL)
    GC.@preserve groups tb sb ss ws begin
        desc = TamScheduleDesc(TAM_ABI_VERSION, D, T === Float64 ? TAM_F64 : TAM_F32, stored,
                               nleaves(s.forest), length(groups),
                               (hasrotating(s.forest) ? 4 : 1) * 3^D, pointer(groups),
                               length(tb), pointer(tb), pointer(sb), length(ss), pointer(ss),
                               length(ws), pointer(ws))
        check(ccall((:tam_schedule_upload, LIB), Cint,
                    (Ptr{Cvoid}, Ref{TamScheduleDesc}, Ref{Ptr{Cvoid}}), ctx, desc, out),
              ctx, "tam_schedule_upload")
    end
    ds = DeviceSchedule(out[], ctx, s.generation)
    finalizer(d -> ccall((:tam_schedule_free, LIB), Cvoid, (Ptr{Cvoid},), d.handle), ds)
    return ds
end

const UPLOADS = WeakKeyDict{GhostSchedule,DeviceSchedule}()
device_schedule(s::GhostSchedule) = get!(() -> upload(s), UPLOADS, s)

# Launch options of an uploaded schedule (TAM_OPT_* of include/treeamr_cuda.h):
# they change how a fill is launched, never its bits.  The reference has no
# tuning (its device fill is one launch per group).
const OPTIONS = (tile_items=Int32(1), threads=Int32(2), int_mul=Int32(3), one_tap=Int32(4),
                 copy_points=Int32(5), block_order=Int32(6), path_tiles=Int32(7),
                 merge_stages=Int32(8), staged=Int32(9), pair_vars=Int32(10),
                 copy_share=Int32(11), soft_add=Int32(12), stencil_tile=Int32(13))

function set_option!(schedule::GhostSchedule, name::Symbol, value::Integer)
    ds = device_schedule(schedule)
    check(ccall((:tam_schedule_set_option, LIB), Cint, (Ptr{Cvoid}, Int32, Int64),
                ds.handle, OPTIONS[name], value), ds.ctx, "tam_schedule_set_option")
    return schedule
end

function get_option(schedule::GhostSchedule, name::Symbol)
    ds = device_schedule(schedule)
    out = Ref{Int64}(0)
    check(ccall((:tam_schedule_get_option, LIB), Cint, (Ptr{Cvoid}, Int32, Ref{Int64}),
                ds.handle, OPTIONS[name], out), ds.ctx, "tam_schedule_get_option")
    return out[]
end

# The library's autotuner (tam_autotune) on the caller's own field set, whose
# data should be representative (zeros and specials send the integer-pipe
# multiplies' points back to the FP64 pipe).  Its fills overwrite the ghosts,
# never an own point.  Leaves the fastest options set on the schedule and
# returns them, with the best fill's time in milliseconds.
function autotune!(fs::FieldSet{T,D,R,<:CuArray}, schedule::GhostSchedule;
                   reps::Integer=3) where {T,D,R}
    TreeAMR.check_fill(fs, schedule)
    ds = device_schedule(schedule)
    ti, th, im = Ref{Int64}(0), Ref{Int64}(0), Ref{Int64}(0)
    ms = Ref{Cdouble}(0)
    rc = ccall((:tam_autotune, LIB), Cint,
               (Ptr{Cvoid}, CuPtr{Cvoid}, Int32, Int64, CuPtr{Cvoid}, Int32, Ptr{Cvoid},
                Ref{Int64}, Ref{Int64}, Ref{Int64}, Ref{Cdouble}),
               ds.handle, pointer(fs.work), fs.nvars, size(fs.work, ndims(fs.work)),
               fs.factors === nothing ? CU_NULL : pointer(fs.factors), reps,
               CUDA.stream().handle, ti, th, im, ms)
    check(rc, ds.ctx, "tam_autotune")
    names = keys(OPTIONS)
    return merge(NamedTuple{names}(map(k -> get_option(schedule, k), names)),
                 (best_ms=ms[],))
end

function tam_fill!(fs::FieldSet, ds::DeviceSchedule, first::Int32, last::Int32;
                   plain::Bool=false, factors=fs.factors, rotvars=fs.rotvars, alt=nothing)
    stream = CUDA.stream().handle
    fptr = factors === nothing ? CU_NULL : pointer(factors)
    if rotvars === nothing && alt === nothing
        f = plain ? :tam_fill_plain : :tam_fill
        rc = ccall((f, LIB), Cint,
                   (Ptr{Cvoid}, CuPtr{Cvoid}, Int32, Int64, CuPtr{Cvoid}, Int32, Int32,
                    Ptr{Cvoid}),
                   ds.handle, pointer(fs.work), fs.nvars, size(fs.work, ndims(fs.work)), fptr,
                   first, last, stream)
        return check(rc, ds.ctx, String(f))
    end
    # turned transfers across a seam: the variable table, and for a pair the
    # partner's array (run_group!'s rotvars and altsrc, src/ghosts.jl:420-490)
    rc = ccall((:tam_fill_ex, LIB), Cint,
               (Ptr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, Int32, Int64, CuPtr{Cvoid},
                CuPtr{Int32}, Int32, Int32, Int32, Ptr{Cvoid}),
               ds.handle, pointer(fs.work), alt === nothing ? CU_NULL : pointer(alt),
               fs.nvars, size(fs.work, ndims(fs.work)), fptr,
               rotvars === nothing ? CU_NULL : pointer(rotvars), first, last,
               plain ? TAM_METHOD_PLAIN : TAM_METHOD_FUSED, stream)
    check(rc, ds.ctx, "tam_fill_ex")
end

# fill_ghosts!(pair, (sa, sb)) of CuArray sets (src/ghosts.jl:2117): the two
# schedules' stages merged by (stage, member), each member reading its
# partner's array through the pair's tables; the hooks after phase 1.
function fill_pair!(pair::RotationPair, (sa, sb)::Tuple{GhostSchedule,GhostSchedule};
                    boundary=nothing)
    a, b = pair.a, pair.b
    da, db = device_schedule(sa), device_schedule(sb)
    ha, hb = boundary isa Tuple ? boundary : (boundary, boundary)
    for (lo, hi) in ((STAGE_FIRST, Int32(1)), (Int32(2), STAGE_LAST))
        tags = sort!(unique!(vcat(stage_tags(sa), stage_tags(sb))))
        for t in filter(t -> lo <= t <= hi, tags)
            tam_fill!(a, da, Int32(t), Int32(t); factors=pair.afactors, rotvars=pair.arotvars,
                      alt=b.work)
            tam_fill!(b, db, Int32(t), Int32(t); factors=pair.bfactors, rotvars=pair.brotvars,
                      alt=a.work)
        end
        if lo == STAGE_FIRST
            ha === nothing || TreeAMR.apply_boundary!(a, ha, sa, CUDABackend())
            hb === nothing || TreeAMR.apply_boundary!(b, hb, sb, CUDABackend())
        end
    end
    return pair
end
stage_tags(s::GhostSchedule) = Int32[first(x) for x in stage_groups(s)]

# Stage P's axis part (run_axis!, src/ghosts.jl:757-766) through
# tam_axis_project, between stage P and stage 0: the schedule's axis points
# (a MeanPoints, src/ghosts.jl:677-689) as element offsets of variable 0 in
# the working array, kept per schedule.  `transpose` runs the projection's
# transpose, the same call with each column of the variable table inverted
# and each factor moved with its variable, which the adjoint runs between
# stage 0's transpose and stage P's.
const AXIS_OFFSETS = WeakKeyDict{GhostSchedule,Any}()
function axis_offsets(fs::FieldSet, schedule::GhostSchedule)
    get!(AXIS_OFFSETS, schedule) do
        ax = schedule.axis
        S = size(fs.work)[1:end-2]
        vol = prod(S)
        blocks, points = Array(ax.blocks), Array(ax.points)
        offs = Int64[]
        for i in eachindex(blocks)
            o = 0
            for d in length(S):-1:1
                o = o * S[d] + (points[i][d] - 1)
            end
            push!(offs, (Int64(blocks[i]) - 1) * fs.nvars * vol + o)
        end
        (CuArray(offs), vol)
    end
end
function transposed_tables(fs::FieldSet{T,D}) where {T,D}
    fac, rv = Array(fs.factors), Array(fs.rotvars)
    ncol = 3^D
    ft, rt = zero(fac), similar(rv)
    for r in 0:3, v in 1:fs.nvars
        w = rv[v, r+1]
        rt[w, r+1] = v
        ft[w, ncol*r+1] = fac[v, ncol*r+1]
    end
    return CuArray(ft), CuArray(rt)
end
function run_axis!(A::CuArray{T}, fs::FieldSet{T,D}, schedule::GhostSchedule;
                   transpose::Bool=false) where {T,D}
    schedule.axis === nothing && return nothing
    TreeAMR.turns_variables(fs) || return nothing
    offs, vol = axis_offsets(fs, schedule)
    factors, rotvars = transpose ? transposed_tables(fs) : (fs.factors, fs.rotvars)
    buf = CuArray{T}(undef, length(offs) * fs.nvars)
    members = TreeAMR.ishalfturn(fs.forest) ? Int32(2) : Int32(4)
    rc = ccall((:tam_axis_project, LIB), Cint,
               (Int32, CuPtr{Int64}, Int64, Int32, CuPtr{Cvoid}, Int32, Int64, CuPtr{Cvoid},
                Int32, CuPtr{Int32}, CuPtr{Cvoid}, Ptr{Cvoid}),
               T === Float64 ? TAM_F64 : TAM_F32, pointer(offs), length(offs), members,
               pointer(A), fs.nvars, vol, pointer(factors), Int32(3^D), pointer(rotvars),
               pointer(buf), CUDA.stream().handle)
    rc == 0 || error("tam_axis_project failed ($rc)")
    return nothing
end

# The drop-in: fill_ghosts! of a CuArray field set (src/ghosts.jl:1783),
# after the reference's own checks: stage P, the axis, then the rest, the
# hook after phase 1 (src/ghosts.jl:1111-1136).
function TreeAMR.exchange_ghosts!(fs::FieldSet{T,D,R,<:CuArray}, schedule::GhostSchedule,
                                  boundary, backend) where {T,D,R}
    ds = device_schedule(schedule)
    tam_fill!(fs, ds, STAGE_FIRST, Int32(-1))
    run_axis!(fs.work, fs, schedule)
    if boundary === nothing
        tam_fill!(fs, ds, Int32(0), STAGE_LAST)
    else
        tam_fill!(fs, ds, Int32(0), Int32(1))
        TreeAMR.apply_boundary!(fs, boundary, schedule, backend)
        tam_fill!(fs, ds, Int32(2), STAGE_LAST)
    end
    return fs
end

# unify! of a CuArray field set over a GhostSchedule (src/ghosts.jl:1836-1840,
# unify_arrays!): stage P, the axis, stage 0, after the reference's checks.
# The state-vector form and a UnifySchedule stay on the reference's path.
function TreeAMR.unify!(fs::FieldSet{T,D,R,<:CuArray}, schedule::GhostSchedule) where {T,D,R}
    TreeAMR.check_fill(fs, schedule)
    TreeAMR.check_unpartnered(fs, "unify!")
    ds = device_schedule(schedule)
    tam_fill!(fs, ds, STAGE_FIRST, Int32(-1))
    run_axis!(fs.work, fs, schedule)
    tam_fill!(fs, ds, Int32(0), Int32(0))
    return fs
end

# scatter! / gather! of a device-resident state (src/state.jl:101-160)
# through tam_scatter / tam_gather: one launch each, the state vector read
# or written linearly, the working array in runs of the own x-extent.
struct TamStateLayout
    dtype::Int32
    ndim::Int32
    own::NTuple{3,Int32}
    stored::NTuple{3,Int32}
    ghosts::NTuple{3,Int32}
    nvars::Int32
    nblocks::Int64
end

function state_layout(fs::FieldSet{T,D}) where {T,D}
    own = TreeAMR.ownextents(fs)
    S = size(fs.work)
    return TamStateLayout(T === Float64 ? TAM_F64 : TAM_F32, D,
                          ntuple(d -> d <= D ? Int32(own[d]) : Int32(1), 3),
                          ntuple(d -> d <= D ? Int32(S[d]) : Int32(1), 3),
                          ntuple(d -> d <= D ? Int32(fs.G[d]) : Int32(0), 3),
                          fs.nvars, TreeAMR.nblocks(fs))
end

function TreeAMR.scatter!(fs::FieldSet{T,D,R,<:CuArray}, u::CuVector{T}) where {T,D,R}
    TreeAMR.check_statelength(u, fs)
    rc = ccall((:tam_scatter, LIB), Cint,
               (Ref{TamStateLayout}, CuPtr{Cvoid}, CuPtr{Cvoid}, Ptr{Cvoid}),
               state_layout(fs), pointer(u), pointer(fs.work), CUDA.stream().handle)
    check(rc, C_NULL, "tam_scatter")
    return fs
end

function TreeAMR.gather!(u::CuVector{T}, fs::FieldSet{T,D,R,<:CuArray}) where {T,D,R}
    TreeAMR.check_statelength(u, fs)
    rc = ccall((:tam_gather, LIB), Cint,
               (Ref{TamStateLayout}, CuPtr{Cvoid}, CuPtr{Cvoid}, Ptr{Cvoid}),
               state_layout(fs), pointer(fs.work), pointer(u), CUDA.stream().handle)
    check(rc, C_NULL, "tam_gather")
    return u
end

# y <- A^T y over stages [first, last] (tam_fill_adjoint_alt): with the
# variable table across a seam, and for a pair member the partner's
# cotangent `alt`, onto which odd turns' transposes add.
function tam_fill_adjoint!(y::CuArray, fs::FieldSet, ds::DeviceSchedule, first::Int32,
                           last::Int32; factors=fs.factors, rotvars=fs.rotvars, alt=nothing)
    rc = ccall((:tam_fill_adjoint_alt, LIB), Cint,
               (Ptr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, Int32, Int64, CuPtr{Cvoid},
                CuPtr{Int32}, Int32, Int32, CuPtr{Cvoid}, Csize_t, Ptr{Cvoid}),
               ds.handle, pointer(y), alt === nothing ? CU_NULL : pointer(alt), fs.nvars,
               size(y, ndims(y)), factors === nothing ? CU_NULL : pointer(factors),
               rotvars === nothing ? CU_NULL : pointer(rotvars), first, last, CU_NULL, 0,
               CUDA.stream().handle)
    check(rc, ds.ctx, "tam_fill_adjoint_alt")
end

# y <- A^T y: the pullback of the fill, the axis projection's transpose
# between stage 0's and stage P's.
function fill_ghosts_adjoint!(y::CuArray, fs::FieldSet, schedule::GhostSchedule)
    ds = device_schedule(schedule)
    tam_fill_adjoint!(y, fs, ds, Int32(0), STAGE_LAST)
    run_axis!(y, fs, schedule; transpose=true)
    tam_fill_adjoint!(y, fs, ds, STAGE_FIRST, Int32(-1))
    return y
end

# (ya, yb) <- A^T (ya, yb) for a pair fill without hooks: tag by tag from the
# last, b's stage transpose then a's, each adding onto the other's cotangent.
function fill_pair_adjoint!(ya::CuArray, yb::CuArray, pair::RotationPair,
                            (sa, sb)::Tuple{GhostSchedule,GhostSchedule})
    a, b = pair.a, pair.b
    da, db = device_schedule(sa), device_schedule(sb)
    ta, tb = stage_tags(sa), stage_tags(sb)
    for t in reverse(sort!(unique!(vcat(ta, tb))))
        t in tb && tam_fill_adjoint!(yb, b, db, t, t; factors=pair.bfactors,
                                     rotvars=pair.brotvars, alt=ya)
        t in ta && tam_fill_adjoint!(ya, a, da, t, t; factors=pair.afactors,
                                     rotvars=pair.arotvars, alt=yb)
    end
    return ya, yb
end

# A field set held in host memory, filled on the GPU (tam_fill_host): the
# state is uploaded into a device buffer kept per schedule, filled there and
# downloaded into fs.work, all on the task's stream.  Page-locked host memory
# (CUDA.Mem.pin(fs.work)) lets the copies overlap other streams' work.
const HOST_BUFFERS = WeakKeyDict{GhostSchedule,Any}()
function fill_ghosts_on_gpu!(fs::FieldSet{T,D,R,<:Array}, schedule::GhostSchedule;
                             factors::Union{Nothing,CuArray}=nothing) where {T,D,R}
    TreeAMR.check_fill(fs, schedule)
    ds = device_schedule(schedule)
    buf = get!(() -> CuArray{T}(undef, size(fs.work)), HOST_BUFFERS, schedule)
    fdev = factors === nothing && fs.factors !== nothing ? CuArray(fs.factors) : factors
    GC.@preserve fdev buf begin
        rc = ccall((:tam_fill_host, LIB), Cint,
                   (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, CuPtr{Cvoid}, Int32, Int64, CuPtr{Cvoid},
                    Int32, Int32, Ptr{Cvoid}),
                   ds.handle, pointer(fs.work), pointer(fs.work), pointer(buf), fs.nvars,
                   size(fs.work, ndims(fs.work)), fdev === nothing ? CU_NULL : pointer(fdev),
                   STAGE_FIRST, STAGE_LAST, CUDA.stream().handle)
        check(rc, ds.ctx, "tam_fill_host")
        CUDA.synchronize()
    end
    return fs
end

# A functional form for differentiation: the filled copy of `x`.
function ghost_filled(x::CuArray, fs::FieldSet, schedule::GhostSchedule)
    y = copy(x)
    saved = fs.work
    try
        fs.work .= y
        fill_ghosts!(fs, schedule)
        copyto!(y, fs.work)
    finally
        copyto!(fs.work, saved)
    end
    return y
end

function ChainRulesCore.rrule(::typeof(ghost_filled), x::CuArray, fs::FieldSet,
                              schedule::GhostSchedule)
    y = ghost_filled(x, fs, schedule)
    pullback(ȳ) = (ChainRulesCore.NoTangent(),
                   fill_ghosts_adjoint!(copy(ChainRulesCore.unthunk(ȳ)), fs, schedule),
                   ChainRulesCore.NoTangent(), ChainRulesCore.NoTangent())
    return y, pullback
end

end # module
