"""
    MaviCUDA

Julia binding of libmavi_cuda.so (include/mavi_cuda.h): routes Mavi.jl's step
loop for a `System` to the GPU.

The hook is the reference's device mode (`IntCfg.device`, src/configs.jl:471-475):
a system whose `int_cfg.device isa CUDADevice` gets a GPU step function from
`get_step_function` (src/integration.jl:537-548), and `run_system`
(src/run_system.jl:7-23) works unchanged. State arrays are passed to the
library by pointer: `Vector{SVector{2,Float64}}` is the interleaved
[x1, y1, x2, y2, ...] layout the ABI takes.

The GPU copy of the state is authoritative while stepping; `sync!(system)`
copies it back into `system.state` (done automatically by `run_system` here and
by `gpu_run!`). Indices crossing the ABI are 0-based.

Bulk drivers: for a CUDA system, `run_system` runs all its steps in one
`mavi_step` call and `run_experiment` one call per event (collector save,
checkpoint, final time), copying the state back once per call instead of once
per step; the single-step `gpu_step!` keeps exact per-step semantics for code
that calls the step function itself.
"""
module MaviCUDA

using StaticArrays
import Mavi
using Mavi.Configs: DeviceMode, RectangleCfg, CircleCfg, LinesCfg, RigidWalls, PeriodicWalls,
    SlipperyWalls, PotentialWalls, ManyWalls, ManyGeometries, HarmTruncCfg, LenJonesCfg, SzaboCfg,
    RunTumbleCfg, has_chunks
using Mavi.States: SecondLawState, SelfPropelledState
import Mavi.Rings
const RC = Mavi.Rings.Configs
const RS = Mavi.Rings.Sources

const libmavi = get(ENV, "MAVI_CUDA_LIB", joinpath(@__DIR__, "..", "lib", "libmavi_cuda.so"))

# ---- constants (include/mavi_cuda.h) ---------------------------------------
const MAVI_OK = Cint(0)
const STATE_SECOND_LAW, STATE_SELF_PROPELLED, STATE_RINGS = Int32(0), Int32(1), Int32(2)
const DYN_HARM_TRUNC, DYN_LEN_JONES, DYN_SZABO, DYN_RUN_TUMBLE, DYN_RINGS = Int32.(0:4)
const STEP_NEWTON, STEP_SZABO, STEP_RTP, STEP_RINGS, STEP_OVERDAMPED = Int32.(0:4)
const GEOM_RECTANGLE, GEOM_CIRCLE, GEOM_LINES = Int32.(0:2)
const WALL_RIGID, WALL_PERIODIC, WALL_SLIPPERY, WALL_POTENTIAL = Int32.(0:3)
const PREC_FP64, PREC_MIXED = Int32(0), Int32(1)
const NOISE_DEVICE, NOISE_INJECTED = Int32(0), Int32(1)
const MAX_SPACES, MAX_LINES, MAX_TYPES = 4, 16, 4
const SRC_SOURCE, SRC_SINK = Int32(0), Int32(1)
const SPAWN_POL_FIXED, SPAWN_POL_RANDOM = Int32(0), Int32(1)

# ---- C structs (same field order and types as the header) -------------------
struct CSpace
    wall::Int32; geometry::Int32
    length::Float64; height::Float64; bl_x::Float64; bl_y::Float64
    radius::Float64; cx::Float64; cy::Float64
    num_lines::Int32; has_bbox::Int32
    lines::NTuple{4 * MAX_LINES, Float64}
    bbox_length::Float64; bbox_height::Float64; bbox_bl_x::Float64; bbox_bl_y::Float64
    pot_kind::Int32; pot_mode::Int32
    pot_params::NTuple{4, Float64}
end

struct CRingsCfg
    num_types::Int32; num_rings::Int32; nmax::Int32; _pad0::Int32
    num_particles::NTuple{MAX_TYPES, Int32}
    p0::NTuple{MAX_TYPES, Float64}; relax_time::NTuple{MAX_TYPES, Float64}
    vo::NTuple{MAX_TYPES, Float64}; mobility::NTuple{MAX_TYPES, Float64}
    rot_diff::NTuple{MAX_TYPES, Float64}; k_area::NTuple{MAX_TYPES, Float64}
    k_spring::NTuple{MAX_TYPES, Float64}; l_spring::NTuple{MAX_TYPES, Float64}
    k_bend::NTuple{MAX_TYPES, Float64}
    inter::NTuple{4 * MAX_TYPES * MAX_TYPES, Float64}   # k_rep, k_atr, dist_eq, dist_max matrices
end

struct CDynamicCfg
    kind::Int32; _pad0::Int32
    k_rep::Float64; k_atr::Float64; dist_eq::Float64; dist_max::Float64
    sigma::Float64; epsilon::Float64
    vo::Float64; mobility::Float64; relax_time::Float64; k_adh::Float64; r_eq::Float64
    r_max::Float64; rot_diff::Float64; tumble_rate::Float64
end

struct CReplicaParams
    num_particles::Int64
    state_kind::Int32; step_kind::Int32; num_spaces::Int32
    chunk_cols::Int32; chunk_rows::Int32; _pad0::Int32
    dt::Float64
    spaces::NTuple{MAX_SPACES, CSpace}
    dyn::CDynamicCfg
    rings::CRingsCfg
end

struct CSourceEntry
    kind::Int32; num_boxes::Int32; pol_mode::Int32; geometry::Int32
    pol::Float64; pad::Float64
    length::Float64; height::Float64; bl_x::Float64; bl_y::Float64
    radius::Float64; cx::Float64; cy::Float64
end

struct CSpawnBox
    bl_x::Float64; bl_y::Float64; length::Float64; height::Float64
    num_chunks::Int32; _pad0::Int32
end

struct CInvasion
    invasor::Int32; invaded::Int32; p_id::Int32; _pad0::Int32
end

struct COptions
    precision::Int32; noise_mode::Int32; seed::UInt64
    device::Int32; use_graph::Int32; block_size::Int32; gather_mode::Int32
end

"""
    CUDADevice(; precision=:fp64, device=0, seed=0)

Device mode for `IntCfg(device=CUDADevice())`. `precision = :fp64` runs every
operation in double (the drop-in); `:mixed` runs the pair loop in FP32 on
chunk-relative offsets with FP64 update, wrap and binning.
"""
# gather: the pair pass (MaviOptions.gather_mode): -1 autotuned at creation;
# 0-2 warp-staged / per-chunk / per-column (the same bits); 3-7 mixed-form
# variants (tiles, tiles from a work queue, 2 or 4 lanes, split gather)
Base.@kwdef struct CUDADevice <: DeviceMode
    precision::Symbol = :fp64
    device::Int = 0
    seed::UInt64 = 0
    gather::Int = -1
end

# ---- packing -----------------------------------------------------------------
zspace() = CSpace(0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, ntuple(_ -> 0.0, 4MAX_LINES), 0, 0, 0, 0, 0, 0,
                  (0.0, 0.0, 0.0, 0.0))

function cspace(wall, geom)
    s = zspace()
    wcode = wall isa RigidWalls ? WALL_RIGID : wall isa PeriodicWalls ? WALL_PERIODIC :
            wall isa SlipperyWalls ? WALL_SLIPPERY : wall isa PotentialWalls ? WALL_POTENTIAL :
            error("unsupported wall type $(typeof(wall))")
    pk, pm, pp = Int32(0), Int32(0), (0.0, 0.0, 0.0, 0.0)
    if wall isa PotentialWalls
        p = wall.potential
        pm = Int32(wall.mode isa Mavi.Configs.Outside ? 0 : wall.mode isa Mavi.Configs.Inside ? 1 : 2)
        if p isa HarmTruncCfg
            pk, pp = DYN_HARM_TRUNC, (p.k_rep, p.k_atr, p.dist_eq, p.dist_max)
        else
            pk, pp = DYN_LEN_JONES, (p.sigma, p.epsilon, 0.0, 0.0)
        end
    end
    if geom isa RectangleCfg
        return CSpace(wcode, GEOM_RECTANGLE, geom.length, geom.height, geom.bottom_left[1],
                      geom.bottom_left[2], 0, 0, 0, 0, 0, s.lines, 0, 0, 0, 0, pk, pm, pp)
    elseif geom isa CircleCfg
        return CSpace(wcode, GEOM_CIRCLE, 0, 0, 0, 0, geom.radius, geom.center[1], geom.center[2],
                      0, 0, s.lines, 0, 0, 0, 0, pk, pm, pp)
    elseif geom isa LinesCfg
        n = length(geom.lines)
        n <= MAX_LINES || error("at most $MAX_LINES lines")
        flat = zeros(4MAX_LINES)
        for (k, l) in enumerate(geom.lines)
            flat[4k-3:4k] .= (l.p1[1], l.p1[2], l.p2[1], l.p2[2])
        end
        bb = geom.bbox
        hb = isnothing(bb) ? 0 : 1
        b = isnothing(bb) ? (0.0, 0.0, 0.0, 0.0) : (bb.length, bb.height, bb.bottom_left[1], bb.bottom_left[2])
        return CSpace(wcode, GEOM_LINES, 0, 0, 0, 0, 0, 0, 0, n, hb, Tuple(flat), b..., pk, pm, pp)
    end
    error("unsupported geometry $(typeof(geom))")
end

function cspaces(space_cfg)
    w, g = space_cfg.wall_type, space_cfg.geometry_cfg
    pairs = w isa ManyWalls ? collect(zip(w.list, g.list)) : [(w, g)]
    length(pairs) <= MAX_SPACES || error("at most $MAX_SPACES (wall, geometry) entries")
    sp = [cspace(a, b) for (a, b) in pairs]
    while length(sp) < MAX_SPACES
        push!(sp, zspace())
    end
    return Tuple(sp), Int32(length(pairs))
end

function cdynamic(cfg)
    z = 0.0
    cfg isa HarmTruncCfg && return CDynamicCfg(DYN_HARM_TRUNC, 0, cfg.k_rep, cfg.k_atr, cfg.dist_eq,
                                               cfg.dist_max, z, z, z, 1.0, z, z, z, z, z, z)
    cfg isa LenJonesCfg && return CDynamicCfg(DYN_LEN_JONES, 0, z, z, z, z, cfg.sigma, cfg.epsilon,
                                              z, 1.0, z, z, z, z, z, z)
    cfg isa SzaboCfg && return CDynamicCfg(DYN_SZABO, 0, cfg.k_rep, z, z, z, z, z, cfg.vo, cfg.mobility,
                                           cfg.relax_time, cfg.k_adh, cfg.r_eq, cfg.r_max, cfg.rot_diff, z)
    cfg isa RunTumbleCfg && return CDynamicCfg(DYN_RUN_TUMBLE, 0, z, z, z, z, cfg.sigma, cfg.epsilon,
                                               cfg.vo, 1.0, z, z, z, z, z, cfg.tumble_rate)
    cfg isa RC.RingsCfg && return CDynamicCfg(DYN_RINGS, 0, z, z, z, z, z, z, z, 1.0, z, z, z, z, z, z)
    error("unsupported dynamic config $(typeof(cfg))")
end

# RingsCfg (src/rings/configs.jl:95-163) for the state's rings: per-type
# vectors (a scalar applies to every type) and the InteractionMatrix as four
# row-major MAX_TYPES x MAX_TYPES matrices.
_tup4(v, T) = ntuple(k -> k <= length(v) ? T(v[k]) : zero(T), MAX_TYPES)
function crings(cfg, st)
    nt = cfg.num_types
    nmax, nr = size(st.rings_pos)
    np = st.num_particles
    nps = np isa AbstractVector ? np : fill(np, nt)
    finder = cfg.interaction_finder
    inter(a, b) = finder isa RC.InteractionMatrix ? finder.matrix[a, b] : finder
    flat = zeros(4 * MAX_TYPES * MAX_TYPES)
    for a in 1:nt, b in 1:nt
        it = inter(a, b)
        k = (a - 1) * MAX_TYPES + (b - 1)
        flat[1 + k] = it.k_rep
        flat[1 + MAX_TYPES^2 + k] = it.k_atr
        flat[1 + 2 * MAX_TYPES^2 + k] = it.dist_eq
        flat[1 + 3 * MAX_TYPES^2 + k] = it.dist_max
    end
    pt(x) = _tup4(x isa AbstractVector ? x : fill(x, nt), Float64)
    CRingsCfg(Int32(nt), Int32(nr), Int32(nmax), Int32(0), _tup4(nps, Int32),
              pt(cfg.p0), pt(cfg.relax_time), pt(cfg.vo), pt(cfg.mobility), pt(cfg.rot_diff), pt(cfg.k_area),
              pt(cfg.k_spring), pt(cfg.l_spring), ntuple(_ -> 0.0, MAX_TYPES), Tuple(flat))
end

const ZRINGS = CRingsCfg(0, 0, 0, 0, ntuple(_ -> Int32(0), MAX_TYPES), ntuple(_ -> ntuple(_ -> 0.0, MAX_TYPES), 9)...,
                         ntuple(_ -> 0.0, 4 * MAX_TYPES * MAX_TYPES))

function step_kind(system)
    cfg = system.dynamic_cfg
    cfg isa RC.RingsCfg && return STEP_RINGS
    cfg isa SzaboCfg && return STEP_SZABO
    cfg isa RunTumbleCfg && return STEP_RTP
    return STEP_NEWTON
end

function replica_params(system, kind=step_kind(system))
    st = system.state
    sp, nsp = cspaces(system.space_cfg)
    cc = system.int_cfg.chunks_cfg
    cols, rows = has_chunks(system.int_cfg) ? (Int32(cc.num_cols), Int32(cc.num_rows)) : (Int32(0), Int32(0))
    rings = st isa Rings.RingsState
    sk = rings ? STATE_RINGS : st isa SecondLawState ? STATE_SECOND_LAW : STATE_SELF_PROPELLED
    CReplicaParams(length(st.pos), sk, kind, nsp, cols, rows, 0, system.int_cfg.dt, sp,
                   cdynamic(system.dynamic_cfg), rings ? crings(system.dynamic_cfg, st) : ZRINGS)
end

# pointers of the state arrays the ABI takes (velocities, polarisations)
_vel_ptr(st) = st isa SecondLawState ? pointer(st.vel) : Ptr{SVector{2,Float64}}(C_NULL)
_pol_ptr(st) = st isa SelfPropelledState ? pointer(st.pol_angle) :
               st isa Rings.RingsState ? pointer(st.pol) : Ptr{Float64}(C_NULL)

# ---- handles -------------------------------------------------------------------
mutable struct Handle
    ptr::Ptr{Cvoid}
end

const HANDLES = IdDict{Any, Handle}()

function check(st, what, h=C_NULL)
    st == MAVI_OK && return
    msg = unsafe_string(ccall((:mavi_status_string, libmavi), Cstring, (Cint,), st))
    if h != C_NULL
        buf = zeros(UInt8, 512)
        ccall((:mavi_last_error, libmavi), Cint, (Ptr{Cvoid}, Ptr{UInt8}, Int32), h, buf, 512)
        msg *= ": " * unsafe_string(pointer(buf))
    end
    # the reference raises BoundsError / throws on the same conditions
    error("$what: $msg")
end

function handle!(system)
    haskey(HANDLES, system) && return HANDLES[system].ptr
    dev = system.int_cfg.device
    opt = COptions(dev.precision == :mixed ? PREC_MIXED : PREC_FP64, NOISE_DEVICE, dev.seed,
                   dev.device, 1, 0, dev.gather)
    params = Ref(replica_params(system))
    st = system.state
    vel, pol = _vel_ptr(st), _pol_ptr(st)
    types = st isa Rings.RingsState && !isnothing(st.types) ? Int32.(st.types) : Int32[]
    out = Ref{Ptr{Cvoid}}(C_NULL)
    GC.@preserve st types begin
        check(ccall((:mavi_create, libmavi), Cint,
                    (Ref{COptions}, Int32, Ref{CReplicaParams}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid},
                     Ptr{Int32}, Ref{Ptr{Cvoid}}),
                    opt, 1, params, pointer(st.pos), vel, pol,
                    isempty(types) ? Ptr{Int32}(C_NULL) : pointer(types), out), "mavi_create")
    end
    h = Handle(out[])
    finalizer(x -> ccall((:mavi_destroy, libmavi), Cint, (Ptr{Cvoid},), x.ptr), h)
    HANDLES[system] = h
    # the handle's clock starts at the system's time_info (a loaded system keeps its count)
    check(ccall((:mavi_set_time, libmavi), Cint, (Ptr{Cvoid}, Int32, Int64, Float64),
                h.ptr, 0, system.time_info.num_steps, system.time_info.time), "mavi_set_time", h.ptr)
    st isa Rings.RingsState && configure_sources!(system, h.ptr)
    st isa Rings.RingsState && configure_invasions!(system, h.ptr)
    return h.ptr
end

"The system's InvasionsCfg and ring chunks (RingsIntCfg extra, src/rings/configs.jl:334-350), or nothing."
function _invasions_cfg(system)
    extra = hasproperty(system.int_cfg, :extra) ? system.int_cfg.extra : nothing
    (isnothing(extra) || !hasproperty(extra, :invasions_cfg)) && return nothing
    return extra.invasions_cfg, extra.r_chunks_cfg
end

"""
Invasion detection (update_invasions!, src/rings/integration.jl:511-520)
passed to `mavi_rings_invasions_config`: steps_to_update and the ring-chunk
grid; the handle's creation stands for the system's construction
(`last_check = num_steps`, src/rings/rings.jl:276-284).
"""
function configure_invasions!(system, h)
    cfg = _invasions_cfg(system)
    (isnothing(cfg) || isnothing(cfg[1])) && return
    inv, rc = cfg
    cols, rows = isnothing(rc) ? (0, 0) : (rc.num_cols, rc.num_rows)
    check(ccall((:mavi_rings_invasions_config, libmavi), Cint, (Ptr{Cvoid}, Int32, Int32, Int64, Int32, Int32),
                h, 0, 1, inv.steps_to_update, cols, rows), "mavi_rings_invasions_config", h)
end

"""
Variable rings ids and the system's sources and sinks (VarRingsIds,
src/rings/states.jl:20-40; `system.info.sources`, src/rings/rings.jl:162-186)
passed to `mavi_rings_sources`, from the reference's own `Source` / `Sink`
objects: boxes (`bbox`), spawn points (`bbox_spawn_pos`) and chunk lists
(`checker.ids`) are the ones the reference computed.
"""
function configure_sources!(system, h)
    st = system.state
    ids = st.rings_ids
    ids isa Rings.States.VarRingsIds || return
    mask = Int32.(ids.mask)
    entries, boxes, spawn, rc = CSourceEntry[], CSpawnBox[], Float64[], Int32[]
    srcs = system.info.sources
    for s in (isnothing(srcs) ? () : srcs)
        if s isa RS.Sink
            g = s.cfg.geometry_cfg
            if g isa CircleCfg
                push!(entries, CSourceEntry(SRC_SINK, 0, 0, GEOM_CIRCLE, 0, 0, 0, 0, 0, 0,
                                            g.radius, g.center[1], g.center[2]))
            else
                push!(entries, CSourceEntry(SRC_SINK, 0, 0, GEOM_RECTANGLE, 0, 0, g.length, g.height,
                                            g.bottom_left[1], g.bottom_left[2], 0, 0, 0))
            end
            continue
        end
        random = s.cfg.spawn_pol isa RS.RandomPol
        nb = length(s.bbox)
        push!(entries, CSourceEntry(SRC_SOURCE, nb, random ? SPAWN_POL_RANDOM : SPAWN_POL_FIXED, 0,
                                    random ? 0.0 : Float64(s.cfg.spawn_pol), Float64(s.cfg.pad),
                                    0, 0, 0, 0, 0, 0, 0))
        for i in 1:nb
            b = s.bbox[i]
            lst = s.checker isa RS.ChunksChecker ? s.checker.ids[i] : nothing
            push!(boxes, CSpawnBox(b.bottom_left[1], b.bottom_left[2], b.length, b.height,
                                   isnothing(lst) ? -1 : length(lst), 0))
            for p in s.bbox_spawn_pos[i]
                push!(spawn, p[1], p[2])
            end
            if !isnothing(lst)
                for c in lst
                    push!(rc, Int32(c[1] - 1), Int32(c[2] - 1))
                end
            end
        end
    end
    GC.@preserve mask entries boxes spawn rc check(
        ccall((:mavi_rings_sources, libmavi), Cint,
              (Ptr{Cvoid}, Int32, Ptr{Int32}, Int32, Ptr{CSourceEntry}, Ptr{CSpawnBox}, Ptr{Float64}, Ptr{Int32}),
              h, 0, mask, length(entries), entries, boxes, spawn, rc), "mavi_rings_sources", h)
end

"Copy the GPU state and the time back into `system` (user particle order)."
function sync!(system)
    h = handle!(system)
    st = system.state
    vel, pol = _vel_ptr(st), _pol_ptr(st)
    GC.@preserve st check(ccall((:mavi_download_state, libmavi), Cint,
                                (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}),
                                h, pointer(st.pos), vel, pol), "mavi_download_state", h)
    if st isa Rings.RingsState
        # RingsInfo.areas of the last force evaluation
        check(ccall((:mavi_rings_areas, libmavi), Cint, (Ptr{Cvoid}, Int32, Ptr{Float64}),
                    h, 0, system.info.areas), "mavi_rings_areas", h)
    end
    if st isa Rings.RingsState && st.rings_ids isa Rings.States.VarRingsIds
        ids = st.rings_ids
        nr = length(ids.mask)
        mask, uids, na = zeros(Int32, nr), zeros(Int32, nr), Ref{Int32}(0)
        check(ccall((:mavi_rings_active, libmavi), Cint, (Ptr{Cvoid}, Int32, Ptr{Int32}, Ptr{Int32}, Ref{Int32}),
                    h, 0, mask, uids, na), "mavi_rings_active", h)
        ids.mask .= mask .!= 0
        ids.uids .= uids
        Mavi.States.update_ids!(st)          # ids, p_ids, counts (calc_active_ids!)
    end
    cfg = st isa Rings.RingsState ? _invasions_cfg(system) : nothing
    if !isnothing(cfg) && !isnothing(cfg[1])
        # RingsInfo.invasions: the list in the reference's push order, last_check
        cnt, last = Ref{Int64}(0), Ref{Int64}(0)
        check(ccall((:mavi_rings_invasions, libmavi), Cint,
                    (Ptr{Cvoid}, Int32, Ptr{CInvasion}, Int64, Ref{Int64}, Ref{Int64}),
                    h, 0, C_NULL, 0, cnt, last), "mavi_rings_invasions", h)
        buf = Vector{CInvasion}(undef, cnt[])
        check(ccall((:mavi_rings_invasions, libmavi), Cint,
                    (Ptr{Cvoid}, Int32, Ptr{CInvasion}, Int64, Ref{Int64}, Ref{Int64}),
                    h, 0, buf, cnt[], cnt, last), "mavi_rings_invasions", h)
        info = system.info.invasions
        empty!(info.list)
        for v in buf
            push!(info.list, Rings.Invasion(invasor=Int(v.invasor), invaded=Int(v.invaded), p_id=Int(v.p_id)))
        end
        info.last_check = last[]
    end
    n, t = Ref{Int64}(0), Ref{Float64}(0)
    check(ccall((:mavi_get_time, libmavi), Cint, (Ptr{Cvoid}, Ref{Int64}, Ref{Float64}), h, n, t),
          "mavi_get_time", h)
    system.time_info.num_steps = n[]
    system.time_info.time = t[]
    return system
end

"""
Queue the copy of the GPU state into `system.state` and return
(`mavi_download_state_async`); the arrays are complete after `wait!(system)`.
Independent systems on their own handles overlap one system's copy with the
others' steps.
"""
function download_async!(system)
    h = handle!(system)
    st = system.state
    vel, pol = _vel_ptr(st), _pol_ptr(st)
    check(ccall((:mavi_download_state_async, libmavi), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}),
                h, pointer(st.pos), vel, pol), "mavi_download_state_async", h)
end

"Wait for the system's queued GPU work and copies (`mavi_synchronize`); throws on a device error."
function wait!(system)
    h = handle!(system)
    check(ccall((:mavi_synchronize, libmavi), Cint, (Ptr{Cvoid},), h), "mavi_synchronize", h)
end

"Push `system.state` to the GPU (after the caller edited it on the host)."
function upload!(system)
    h = handle!(system)
    st = system.state
    vel, pol = _vel_ptr(st), _pol_ptr(st)
    GC.@preserve st check(ccall((:mavi_upload_state, libmavi), Cint,
                                (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}),
                                h, pointer(st.pos), vel, pol), "mavi_upload_state", h)
end

"Advance `num_steps` steps on the GPU and copy the state back once."
function gpu_run!(system, num_steps::Integer)
    h = handle!(system)
    check(ccall((:mavi_step, libmavi), Cint, (Ptr{Cvoid}, Int64), h, num_steps), "mavi_step", h)
    sync!(system)
end

"""
One-step GPU step function, the value `get_step_function` returns for a
`CUDADevice` system. It keeps `system.state` current after every step, which
costs a device-to-host copy per step; `gpu_run!` steps in bulk.
"""
gpu_step!(system) = gpu_run!(system, 1)

"Forces of the current state (`calc_forces!` + optionally `calc_walls_forces!`)."
function calc_forces(system; include_walls=false)
    h = handle!(system)
    f = Vector{SVector{2, Float64}}(undef, length(system.state.pos))
    check(ccall((:mavi_calc_forces, libmavi), Cint, (Ptr{Cvoid}, Int32, Ptr{Cvoid}),
                h, include_walls ? 1 : 0, f), "mavi_calc_forces", h)
    return f
end

"Energy series on the device (`mavi_energy_series`): per sample, advance `steps_between` steps and record the
kinetic and potential energy; one copy back at the end, then `sync!`. Returns (ke, pe) vectors."
function energy_series(system, num_samples::Integer, steps_between::Integer; all_pairs=false)
    h = handle!(system)
    ke, pe = zeros(Float64, num_samples), zeros(Float64, num_samples)
    check(ccall((:mavi_energy_series, libmavi), Cint, (Ptr{Cvoid}, Int64, Int64, Int32, Ptr{Float64}, Ptr{Float64}),
                h, num_samples, steps_between, all_pairs ? 1 : 0, ke, pe), "mavi_energy_series", h)
    sync!(system)
    return ke, pe
end

"Pair-distance histogram (`mavi_pair_distribution`) of the current state: `num_bins` counts of
unordered pairs with floor(d / dr) == k, d < r_max, dr = r_max / num_bins."
function pair_distribution(system, r_max::Real, num_bins::Integer)
    h = handle!(system)
    counts = zeros(UInt64, num_bins)
    check(ccall((:mavi_pair_distribution, libmavi), Cint, (Ptr{Cvoid}, Int32, Float64, Int32, Ptr{UInt64}),
                h, 0, r_max, num_bins, counts), "mavi_pair_distribution", h)
    return counts
end

# ---- bulk drivers ------------------------------------------------------------------
# The reference's drivers call the step function once per step (src/run_system.jl:7-23,
# src/experiments.jl:94-144). For a CUDA system the steps between two host-side events
# run in one mavi_step call and the state is copied back once per event, not per step.

const CUDASystem = Mavi.Systems.System{T, ND, NT, S, W, G, D,
                                       <:Mavi.Configs.IntCfg{<:Number, <:Any, CUDADevice}} where {T, ND, NT, S, W, G, D}

"Steps the reference's `while cond(time)` loop takes from `t0` (replays `time += dt`, update_time!,
src/integration.jl:500-503); returns (steps, final time)."
function steps_while(cond, t0::Float64, dt::Float64)
    t, n = t0, 0
    while cond(t)
        t += dt
        n += 1
    end
    return n, t
end

"""
    run_system(system::CUDASystem; tf, num_steps, step_func)

`run_system` (src/run_system.jl:7-23) for a system on the GPU: the number of steps
(`num_steps`, or the steps the reference's `while time < tf` loop takes) runs in one
`mavi_step` call and the state is copied back once. A caller-supplied `step_func`
other than the GPU step runs the reference's loop unchanged.
"""
function Mavi.RunSystem.run_system(system::CUDASystem; tf=nothing, num_steps=nothing, step_func=nothing)
    if !isnothing(step_func) && step_func !== gpu_step!
        if !isnothing(tf)
            while system.time_info.time < tf
                step_func(system)
            end
        else
            for _ in 1:num_steps
                step_func(system)
            end
        end
        return
    end
    n = isnothing(tf) ? num_steps : steps_while(t -> t < tf, system.time_info.time, system.int_cfg.dt)[1]
    n > 0 && gpu_run!(system, n)
    return
end

const EXP = Mavi.Experiments

# Steps until a collector acts, for the collectors whose rule is known; `nothing` for
# any other collector (the experiment then runs one step per call, as the reference).
_steps_to_collect(::EXP.Collector, t0, dt, limit) = nothing
function _steps_to_collect(col::EXP.DelayedCol, t0, dt, limit)
    # collect (src/experiments.jl:435-445): saves when time - last_save_time > delay_time
    last, delay = col.state.last_save_time, col.cfg.delay_time
    n = steps_while(t -> !(t - last > delay), t0, dt)[1]
    return n == 0 ? 1 : min(n, limit)      # already due: the collect after the next step saves
end
function _steps_to_collect(col::EXP.ManyCols, t0, dt, limit)
    n = limit
    for c in values(col.cols)
        k = _steps_to_collect(c, t0, dt, limit)
        isnothing(k) && return nothing
        n = min(n, k)
    end
    return n
end

# check_checkpoint (src/experiments.jl:461-467): acts when time - last_time >= delta_time
_steps_to_checkpoint(::Nothing, ::Nothing, t0, dt, limit) = limit
function _steps_to_checkpoint(cfg::EXP.CheckpointCfg, cp, t0, dt, limit)
    n = steps_while(t -> t - cp.last_time < cfg.delta_time, t0, dt)[1]
    return n == 0 ? 1 : min(n, limit)
end

"""
    run_experiment(experiment::Experiment{<:CUDASystem}, stop_func=nothing; prog_kwargs, check_every=1)

`run_experiment` (src/experiments.jl:94-144) for a system on the GPU. Between two
events (a collector saving, a checkpoint, the final time) the steps run in one
`mavi_step` call; `collect`, `check_checkpoint` and the progress display then run
exactly as in the reference's loop, on the state copied back at that step, and
they see the same times (the host replays `time += dt`). `stop_func` is evaluated
every `check_every` steps (1: every step, the reference's behaviour). A custom
step function other than the GPU step, or a collector whose saving rule is not
known here, runs the reference's loop unchanged.
"""
function EXP.run_experiment(experiment::EXP.Experiment{<:CUDASystem}, stop_func=nothing;
                            prog_kwargs=nothing, check_every::Integer=1)
    system, col, cfg = experiment.system, experiment.col, experiment.cfg
    dt = system.int_cfg.dt
    if experiment.custom_step !== gpu_step! || isnothing(_steps_to_collect(col, system.time_info.time, dt, 1))
        return invoke(EXP.run_experiment, Tuple{EXP.Experiment, Any}, experiment, stop_func;
                      prog_kwargs=prog_kwargs)
    end
    prog_kwargs = isnothing(prog_kwargs) ? () : prog_kwargs
    stop = isnothing(stop_func) ? nothing : stop_func
    EXP.save_system_configs(system, cfg.root)
    EXP.save_experiment_configs(experiment)
    col_path = mkpath(joinpath(cfg.root, EXP.COL_DIRNAME))
    if !isnothing(experiment.checkpoint)
        mkpath(joinpath(cfg.root, EXP.CHECKPOINT_DIRNAME, "1"))
        mkpath(joinpath(cfg.root, EXP.CHECKPOINT_DIRNAME, "2"))
    end
    prog = EXP.ProgContinuos(init=system.time_info.time, final=cfg.tf; prog_kwargs...)
    while system.time_info.time < cfg.tf
        t = system.time_info.time
        limit = steps_while(x -> x < cfg.tf, t, dt)[1]
        isnothing(stop) || (limit = min(limit, check_every))
        n = min(_steps_to_collect(col, t, dt, limit),
                _steps_to_checkpoint(cfg.checkpoint_cfg, experiment.checkpoint, t, dt, limit))
        gpu_run!(system, max(n, 1))
        EXP.collect(col, system)
        EXP.check_checkpoint(cfg.checkpoint_cfg, experiment)
        EXP.show_progress(prog, system.time_info.time)
        if !isnothing(stop) && stop(system)
            break
        end
    end
    EXP.save_data(col, col_path)
    if cfg.save_final_state
        EXP.save_system(system, joinpath(cfg.root, EXP.FINAL_STATE_NAME))
    end
    EXP.show_finish(prog)
    open(joinpath(cfg.root, ".done"), "w") do f
        write(f, "Experiment concluded on $(EXP.Dates.now())\n")
    end
    return
end

# ---- the hook into Mavi.jl -------------------------------------------------------
# get_step_function(::StandardSys, system) (src/integration.jl:539-548) dispatches on
# the dynamic config; a CUDA device mode takes precedence.
function Mavi.Integration.get_step_function(t::Mavi.Systems.StandardSys, system::Mavi.Systems.System{
        T, ND, NT, S, W, G, D, <:Mavi.Configs.IntCfg{<:Number, <:Any, CUDADevice}}) where {T, ND, NT, S, W, G, D}
    return gpu_step!
end

# the rings step (get_step_function(::RingsSys, system), src/rings/integration.jl:545)
function Mavi.Integration.get_step_function(t::Rings.RingsSys, system::Mavi.Systems.System{
        T, ND, NT, S, W, G, D, <:Mavi.Configs.IntCfg{<:Number, <:Any, CUDADevice}}) where {T, ND, NT, S, W, G, D}
    return gpu_step!
end

end # module
