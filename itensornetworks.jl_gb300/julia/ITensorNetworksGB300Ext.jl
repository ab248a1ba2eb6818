# ITensorNetworksGB300Ext -- package extension that routes ITensorNetworks.jl's
# belief-propagation hot path to libgbtn.so (GB300, sm_103a) through ccall.
#
# Load order: `using ITensorNetworks, GB300TensorNetworks` activates this
# extension (weakdep GB300TensorNetworks in ITensorNetworks' Project.toml,
# `[extensions] ITensorNetworksGB300Ext = "GB300TensorNetworks"`).
#
# Its main type is `GB300BeliefPropagationCache <: AbstractBeliefPropagationCache`
# (the interface of src/caches/abstractbeliefpropagationcache.jl:44-69), made by
# `initialize_cache(Algorithm("gb300_bp"), tn)` and so picked up by every
# `alg`+`cache!` entry point of the reference (expect.jl:21-41,
# environment.jl:21-39, contract.jl:41-58, normalize.jl:63-80).  It keeps one
# library plan alive for its whole life: the tensors are uploaded once (again
# only after `bpc[v] = t`), the messages stay on the GPU between `update`,
# `expect`, `logscalar`, `region_scalar`, `rescale` and `normalize`, and a
# host copy of the messages is made only when `messages(bpc)` or
# `environment(bpc, verts)` asks for ITensors.
#
# For a plain BeliefPropagationCache it also adds `update(bpc; alg="gb300_bp", maxiter, tol,
# schedule, edge_sequence, precision)` (the reference's defaults: sequential
# sweeps in default_bp_edge_sequence order, maxiter 1 on trees and required
# otherwise) packs the cache's partitioned tensor network into the
# C-ABI layout (include/gbtn.h), runs the sweeps on the GPU and writes the
# messages back into the cache, so `expect`, `environment`, `scalar`,
# `logscalar`, `inner`, `norm` and `normalize` keep their signatures and read
# converged messages as usual.  Dense Float64, Float32, ComplexF64 and
# ComplexF32 tensors with one site index per vertex and one link per edge are
# supported; other caches raise, as the library has no CPU path.  The default
# precision follows the element type (FP64 for Float64 / ComplexF64, FP32 for
# Float32 / ComplexF32); complex tensors (complex_values = 1) run the FP64,
# FP32 or mixed sweeps, not the BF16 tensor-core one.
#
# It also adds `apply(Algorithm("gb300"), gates, psi; maxdim, cutoff, normalize,
# envs)`, the simple update of src/apply.jl:33-160 on the GPU (FP64 truncated
# SVD), `tebd(Algorithm("gb300"), ℋ, ψ; β, Δβ, maxdim, cutoff)` over it (src/tebd.jl),
# and ChainRulesCore rrules for `bp_energy(psi, ops, coefs)` (the BP two-site
# energy), `bp_logscalar(psi)` and `bp_expect_sum(psi, op)`, whose pullbacks are
# the library's hand-written adjoints (implicit differentiation at the BP fixed
# point; complex tensors too), and for `gb300_apply(gates, psi; ...)` (the real
# simple update through the library's taped adjoint of QR, truncated SVD and
# environment roots, to the input tensors and the gates).
#
# Not executed in the environment this file was written in (no Julia
# toolchain); it documents the binding a maintainer adds.
module ITensorNetworksGB300Ext

using ITensorNetworks: ITensorNetworks, AbstractBeliefPropagationCache, BeliefPropagationCache,
    QuadraticFormNetwork, messages, set_messages, partitioned_tensornetwork, quotientedges, tensornetwork,
    ket_vertex, bra_vertex
using DataGraphs: DataGraphs
using Dictionaries: Dictionary, set!
using ITensors: Op
using ITensors: ITensors, ITensor, Index, inds, commonind, hascommoninds, array, itensor, dag, prime, tags
using LinearAlgebra: LinearAlgebra, norm
using NDTensors: Algorithm, @Algorithm_str
using Graphs: src, dst
using NamedGraphs.PartitionedGraphs: PartitionedGraphs, PartitionedGraph, QuotientEdge, QuotientVertex,
    quotientvertices, quotient_graph, unpartitioned_graph
using GB300TensorNetworks: libgbtn
using ChainRulesCore: ChainRulesCore, NoTangent

const GBTN_OK = Int32(0)

struct GraphDesc
    nv::Int32
    ne::Int32
    edge_u::Ptr{Int32}
    edge_v::Ptr{Int32}
    edge_dim::Ptr{Int32}
    site_dim::Ptr{Int32}
    leg_ptr::Ptr{Int32}
    leg_edge::Ptr{Int32}
    vertex_network::Ptr{Int32}
    n_networks::Int32
    separate_bra::Int32
    complex_values::Int32  # 1: ComplexF64 tensors, interleaved (re, im) in the library's arrays
end

struct BPOpts
    schedule::Int32
    precision::Int32
    maxiter::Int32
    normalize::Int32
    tol::Float64
    edge_sequence::Ptr{Int32}
    edge_sequence_len::Int32
    tol_bf16::Float64
    tol_f32::Float64
    maxiter_bf16::Int32
    maxiter_f32::Int32
    refine_f64::Int32
    refine::Int32       # 0: double-FP32 refinement (default), 1: FP64
    confirm_f64::Int32  # FP64 sweeps after a double-FP32 refinement
end

function check(ctx, code)
    code == GBTN_OK && return nothing
    msg = unsafe_string(ccall((:gbtn_last_error, libgbtn), Cstring, (Ptr{Cvoid},), ctx))
    return error(msg)  # same convention as the reference's error() calls
end

const CTX = Ref{Ptr{Cvoid}}(C_NULL)
function context()
    if CTX[] == C_NULL
        h = Ref{Ptr{Cvoid}}(C_NULL)
        check(C_NULL, ccall((:gbtn_ctx_create, libgbtn), Cint, (Cint, Ref{Ptr{Cvoid}}), 0, h))
        CTX[] = h[]
    end
    return CTX[]
end

# Pack the ket and bra layers of a form-network cache: vertex order =
# partitions, edges = quotient edges (src < dst), legs in each ket tensor's
# index order after the site index.  The bra layer holds dag(phi) (with its
# site and link indices mapped); the library conjugates the bra it is given,
# so it receives phi = conj(bra), in the ket's leg order.  When phi equals the
# ket everywhere (a QuadraticFormNetwork) the plan shares the bra
# (separate_bra = 0), which keeps the tensor-core path; otherwise (inner(phi,
# psi), a BilinearFormNetwork with the identity operator) both layers are
# passed.  Operator tensors are taken to be identities.
function pack(bpc::BeliefPropagationCache)
    pvs = collect(quotientvertices(bpc))
    vid = Dict(pv => i - 1 for (i, pv) in enumerate(pvs))
    pes = collect(quotientedges(bpc))
    tn = tensornetwork(bpc)
    ket(pv) = tn[(parent(pv), "ket")]
    bra(pv) = tn[(parent(pv), "bra")]
    eu = Int32[vid[src(pe)] for pe in pes]
    ev = Int32[vid[dst(pe)] for pe in pes]
    links = [commonind(ket(src(pe)), ket(dst(pe))) for pe in pes]
    blinks = [commonind(bra(src(pe)), bra(dst(pe))) for pe in pes]
    edim = Int32[length(l) for l in links]
    sdim = Int32[]
    leg_ptr = Int32[0]
    leg_edge = Int32[]
    cplx = any(pv -> eltype(ket(pv)) <: Complex || eltype(bra(pv)) <: Complex, pvs)
    data = cplx ? ComplexF64[] : Float64[]
    bdata = similar(data)
    shared = true
    for pv in pvs
        t = ket(pv)
        s = only(filter(i -> !(i in links), inds(t)))
        ls = filter(i -> i in links, collect(inds(t)))
        append!(leg_edge, Int32[findfirst(==(l), links) - 1 for l in ls])
        push!(leg_ptr, length(leg_edge))
        push!(sdim, length(s))
        kv = vec(array(t, s, ls...))  # column-major, site index first
        append!(data, kv)
        tb = bra(pv)
        sb = only(filter(i -> !(i in blinks), inds(tb)))
        lbs = [blinks[findfirst(==(l), links)] for l in ls]  # the bra's links in the ket's leg order
        bv = conj.(vec(array(tb, sb, lbs...)))
        shared &= bv == kv
        append!(bdata, bv)
    end
    # messages keep the tensors' element type (Float32, Float64, ComplexF32, ComplexF64)
    elt = promote_type((eltype(ket(pv)) for pv in pvs)..., (eltype(bra(pv)) for pv in pvs)...)
    return (; pvs, vid, pes, links, eu, ev, edim, sdim, leg_ptr, leg_edge, data, bdata, shared, cplx, elt)
end

function ITensorNetworks.update(alg::Algorithm"gb300_bp", bpc::BeliefPropagationCache)
    p = pack(bpc)
    ctx = context()
    GC.@preserve p begin
        desc = GraphDesc(length(p.pvs), length(p.pes), pointer(p.eu), pointer(p.ev), pointer(p.edim),
            pointer(p.sdim), pointer(p.leg_ptr), pointer(p.leg_edge), C_NULL, 1, p.shared ? 0 : 1,
            p.cplx ? 1 : 0)
        plan = Ref{Ptr{Cvoid}}(C_NULL)
        check(ctx, ccall((:gbtn_plan_create, libgbtn), Cint, (Ptr{Cvoid}, Ref{GraphDesc}, Ref{Ptr{Cvoid}}),
            ctx, desc, plan))
        try
            check(ctx, ccall((:gbtn_set_factors, libgbtn), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Cint),
                plan[], p.data, p.shared ? C_NULL : pointer(p.bdata), 0))
            # the reference's defaults: sequential sweeps in the forest-cover order
            # (default_bp_edge_sequence), maxiter 1 on trees and required otherwise
            sched = Dict("sequential" => 0, "parallel" => 1, "colored" => 2)[get(alg.kwargs, :schedule,
                "sequential")]
            maxiter = get(alg.kwargs, :maxiter, ITensorNetworks.default_bp_maxiter(bpc))
            isnothing(maxiter) && error("You need to specify a number of iterations for BP!")
            seq = Int32[]
            if sched == 0
                de = Dict((p.eu[k], p.ev[k]) => Int32(2 * (k - 1)) for k in eachindex(p.pes))
                for qe in get(alg.kwargs, :edge_sequence, ITensorNetworks.default_bp_edge_sequence(bpc))
                    a, b = Int32(p.vid[src(qe)]), Int32(p.vid[dst(qe)])
                    push!(seq, haskey(de, (a, b)) ? de[(a, b)] : de[(b, a)] + Int32(1))
                end
            end
            single = real(p.elt) === Float32
            prec = Dict("f64" => 0, "f32" => 1, "bf16" => 2, "mixed" => 3, "df32" => 4)[get(alg.kwargs,
                :precision, single ? "f32" : "f64")]
            tol = something(get(alg.kwargs, :tol, nothing), -1.0)
            opts = BPOpts(sched, prec, maxiter, 1, tol, isempty(seq) ? C_NULL : pointer(seq), length(seq),
                0.0, 0.0, 0, 0, 0, 0, 0)
            iters = Ref{Int32}(0)
            diff = Ref{Float64}(0.0)
            GC.@preserve seq check(ctx, ccall((:gbtn_bp_run, libgbtn), Cint,
                (Ptr{Cvoid}, Ref{BPOpts}, Ref{Int32}, Ref{Float64}), plan[], opts, iters, diff))
            nmsg = sum(Int(c)^2 for c in p.edim) * 2
            flat = Vector{eltype(p.data)}(undef, nmsg)
            check(ctx, ccall((:gbtn_get_messages, libgbtn), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Cint),
                plan[], flat, 0))
            # unpack: directed edge 2e = u->v, 2e+1 = v->u; message M[b, a] with
            # b the bra (primed) link and a the ket link
            off = 0
            new = Dict{QuotientEdge, Vector{ITensor}}()
            elt = p.elt
            for (e, pe) in enumerate(p.pes), (dir, qe) in ((0, pe), (1, reverse(pe)))
                c = Int(p.edim[e])
                M = convert(Matrix{elt}, reshape(flat[(off + 1):(off + c * c)], c, c))
                off += c * c
                l = p.links[e]
                new[qe] = [itensor(M, dag(prime(l)), l)]
            end
            bpc = set_messages(bpc, new)
        finally
            ccall((:gbtn_plan_destroy, libgbtn), Cint, (Ptr{Cvoid},), plan[])
        end
    end
    return bpc
end


# ---- the GPU-resident cache ----------------------------------------------------

# One library plan and the host-side maps of a packed form network; the
# finalizer frees the device storage.
mutable struct GB300Plan
    handle::Ptr{Cvoid}
    p::Any          # pack(): vertex and edge maps, leg order, host tensor arrays
    uploaded::Bool  # the device tensors match the cache's
end

function GB300Plan(p)
    ctx = context()
    h = Ref{Ptr{Cvoid}}(C_NULL)
    GC.@preserve p begin
        desc = GraphDesc(length(p.pvs), length(p.pes), pointer(p.eu), pointer(p.ev), pointer(p.edim),
            pointer(p.sdim), pointer(p.leg_ptr), pointer(p.leg_edge), C_NULL, 1, p.shared ? 0 : 1,
            p.cplx ? 1 : 0)
        check(ctx, ccall((:gbtn_plan_create, libgbtn), Cint, (Ptr{Cvoid}, Ref{GraphDesc}, Ref{Ptr{Cvoid}}),
            ctx, desc, h))
    end
    plan = GB300Plan(h[], p, false)
    finalizer(plan) do x
        x.handle == C_NULL || ccall((:gbtn_plan_destroy, libgbtn), Cint, (Ptr{Cvoid},), x.handle)
        x.handle = C_NULL
    end
    return plan
end

"""
    GB300BeliefPropagationCache

A BP cache whose messages live on the GPU (libgbtn plan).  Implements the
reference's cache interface (abstractbeliefpropagationcache.jl:44-69) and is
updated in place: `update` returns the same object.
"""
struct GB300BeliefPropagationCache{V, PV, PTN} <: AbstractBeliefPropagationCache{V, PV}
    partitioned_tensornetwork::PTN
    plan::GB300Plan
    host_messages::Base.RefValue{Any}  # Dictionary mirrored from the device, nothing when stale
end

function GB300BeliefPropagationCache(ptn::PTN, plan::GB300Plan) where {PTN}
    V = eltype(ITensorNetworks.vertices(ptn))
    PV = eltype(quotientvertices(ptn))
    return GB300BeliefPropagationCache{V, PV, PTN}(ptn, plan, Ref{Any}(nothing))
end

ITensorNetworks.partitioned_tensornetwork(bpc::GB300BeliefPropagationCache) = bpc.partitioned_tensornetwork
ITensorNetworks.default_update_alg(::GB300BeliefPropagationCache) = "gb300_bp"
ITensorNetworks.default_message_update_alg(::GB300BeliefPropagationCache) = "contract"
ITensorNetworks.partitions(bpc::GB300BeliefPropagationCache) = quotientvertices(bpc.partitioned_tensornetwork)
PartitionedGraphs.quotientedges(bpc::GB300BeliefPropagationCache) = quotientedges(bpc.partitioned_tensornetwork)
function PartitionedGraphs.partitioned_vertices(bpc::GB300BeliefPropagationCache)
    return PartitionedGraphs.partitioned_vertices(bpc.partitioned_tensornetwork)
end
function ITensorNetworks.default_bp_maxiter(bpc::GB300BeliefPropagationCache)
    return ITensorNetworks.default_bp_maxiter(quotient_graph(bpc.partitioned_tensornetwork))
end
function ITensorNetworks.default_bp_edge_sequence(bpc::GB300BeliefPropagationCache)
    return ITensorNetworks.default_edge_sequence(bpc.partitioned_tensornetwork)
end

# bpc[v] = t (update_factor): the tensor network changes on the host and the
# device copy is refreshed before the next library call.
function DataGraphs.set_vertex_data!(bpc::GB300BeliefPropagationCache, value, vertex)
    DataGraphs.set_vertex_data!(tensornetwork(bpc), value, vertex)
    bpc.plan.uploaded = false
    return bpc
end

# Upload the tensors once, and again only after they changed.
function device_plan(bpc::GB300BeliefPropagationCache)
    plan = bpc.plan
    if !plan.uploaded
        p = pack(bpc)  # the current tensors, same vertex / edge / leg order as the plan
        plan.p = merge(plan.p, (; data=p.data, bdata=p.bdata))
        GC.@preserve p check(context(), ccall((:gbtn_set_factors, libgbtn), Cint,
            (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Cint), plan.handle, p.data,
            plan.p.shared ? C_NULL : pointer(p.bdata), 0))
        plan.uploaded = true
    end
    return plan.handle
end

function ITensorNetworks.initialize_cache(alg::Algorithm"gb300_bp", tn;
                                          partitioned_vertices=ITensorNetworks.default_partitioned_vertices(tn),
                                          messages=nothing)
    ptn = PartitionedGraph(tn, partitioned_vertices)
    bpc = GB300BeliefPropagationCache(ptn, GB300Plan(pack_ptn(ptn)))
    h = device_plan(bpc)
    if isnothing(messages)
        check(context(), ccall((:gbtn_init_messages, libgbtn), Cint, (Ptr{Cvoid}, Cint), h, 0))  # identity
    else
        ITensorNetworks.set_messages!(bpc, messages)
    end
    return bpc
end

function Base.copy(bpc::GB300BeliefPropagationCache)
    ptn = copy(bpc.partitioned_tensornetwork)
    new = GB300BeliefPropagationCache(ptn, GB300Plan(bpc.plan.p))
    flat = device_messages(bpc)
    check(context(), ccall((:gbtn_set_messages, libgbtn), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Cint),
        device_plan(new), flat, 0))
    return new
end

function device_messages(bpc::GB300BeliefPropagationCache)
    p = bpc.plan.p
    flat = Vector{eltype(p.data)}(undef, 2 * sum(Int(c)^2 for c in p.edim; init=0))
    check(context(), ccall((:gbtn_get_messages, libgbtn), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Cint),
        device_plan(bpc), flat, 0))
    return flat
end

# messages(bpc): ITensors made from the device messages (one host copy per
# state; directed edge 2e = u->v, 2e+1 = v->u; M[b, a], b the bra link)
function ITensorNetworks.messages(bpc::GB300BeliefPropagationCache)
    isnothing(bpc.host_messages[]) || return bpc.host_messages[]
    p = bpc.plan.p
    flat = device_messages(bpc)
    out = Dictionary{QuotientEdge, Vector{ITensor}}()
    off = 0
    for (e, pe) in enumerate(p.pes), qe in (pe, reverse(pe))
        c = Int(p.edim[e])
        M = convert(Matrix{p.elt}, reshape(flat[(off + 1):(off + c * c)], c, c))
        off += c * c
        set!(out, qe, [itensor(M, dag(prime(p.links[e])), p.links[e])])
    end
    bpc.host_messages[] = out
    return out
end

function ITensorNetworks.set_messages!(bpc::GB300BeliefPropagationCache, ms)
    p = bpc.plan.p
    flat = similar(p.data, 2 * sum(Int(c)^2 for c in p.edim; init=0))
    off = 0
    for (e, pe) in enumerate(p.pes), qe in (pe, reverse(pe))
        c = Int(p.edim[e])
        flat[(off + 1):(off + c * c)] = vec(array(only(ms[qe]), dag(prime(p.links[e])), p.links[e]))
        off += c * c
    end
    check(context(), ccall((:gbtn_set_messages, libgbtn), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Cint),
        device_plan(bpc), flat, 0))
    bpc.host_messages[] = nothing
    return bpc
end

function ITensorNetworks.set_default_kwargs(alg::Algorithm"gb300_bp", bpc::GB300BeliefPropagationCache)
    maxiter = get(alg.kwargs, :maxiter, ITensorNetworks.default_bp_maxiter(bpc))
    edge_sequence = get(alg.kwargs, :edge_sequence, ITensorNetworks.default_bp_edge_sequence(bpc))
    return Algorithm("gb300_bp"; maxiter, edge_sequence, tol=get(alg.kwargs, :tol, nothing),
        schedule=get(alg.kwargs, :schedule, "sequential"), precision=get(alg.kwargs, :precision, nothing),
        verbose=get(alg.kwargs, :verbose, false))
end

# update(::Algorithm"bp") with the sweeps on the GPU; the cache is updated in
# place and returned (abstractbeliefpropagationcache.jl:313-337)
function ITensorNetworks.update(alg::Algorithm"gb300_bp", bpc::GB300BeliefPropagationCache)
    p = bpc.plan.p
    maxiter = alg.kwargs.maxiter
    isnothing(maxiter) && error("You need to specify a number of iterations for BP!")
    sched = Dict("sequential" => 0, "parallel" => 1, "colored" => 2)[alg.kwargs.schedule]
    seq = Int32[]
    if sched == 0
        de = Dict((p.eu[k], p.ev[k]) => Int32(2 * (k - 1)) for k in eachindex(p.pes))
        for qe in alg.kwargs.edge_sequence
            a, b = Int32(p.vid[src(qe)]), Int32(p.vid[dst(qe)])
            push!(seq, haskey(de, (a, b)) ? de[(a, b)] : de[(b, a)] + Int32(1))
        end
    end
    single = real(p.elt) === Float32
    prec = Dict("f64" => 0, "f32" => 1, "bf16" => 2, "mixed" => 3, "df32" => 4)[something(alg.kwargs.precision,
        single ? "f32" : "f64")]
    tol = something(alg.kwargs.tol, -1.0)
    opts = BPOpts(sched, prec, maxiter, 1, tol, isempty(seq) ? C_NULL : pointer(seq), length(seq),
        0.0, 0.0, 0, 0, 0, 0, 0)
    iters = Ref{Int32}(0)
    diff = Ref{Float64}(0.0)
    GC.@preserve seq check(context(), ccall((:gbtn_bp_run, libgbtn), Cint,
        (Ptr{Cvoid}, Ref{BPOpts}, Ref{Int32}, Ref{Float64}), device_plan(bpc), opts, iters, diff))
    if alg.kwargs.verbose && tol >= 0 && diff[] <= tol
        println("BP converged to desired precision after $(iters[]) iterations.")
    end
    bpc.host_messages[] = nothing
    return bpc
end

function ITensorNetworks.environment(bpc::GB300BeliefPropagationCache, verts::Vector; kwargs...)
    pvs = ITensorNetworks.quotientvertices(bpc, verts)
    ms = ITensorNetworks.incoming_messages(bpc, pvs; kwargs...)
    central = ITensorNetworks.factors(bpc, setdiff(ITensorNetworks.vertices(bpc, pvs), verts))
    return vcat(ms, central)
end

# region scalars from the device: tr(rho_v) per partition, <m_e, m_ebar> per edge
function device_scalars(bpc::GB300BeliefPropagationCache, which::Symbol)
    p = bpc.plan.p
    n = which === :vertex ? length(p.pvs) : length(p.pes)
    out = Vector{p.cplx ? ComplexF64 : Float64}(undef, max(n, 1))
    f = which === :vertex ? :gbtn_vertex_scalars : :gbtn_edge_scalars
    check(context(), ccall((f, libgbtn), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), device_plan(bpc), out))
    return out
end
function ITensorNetworks.region_scalar(bpc::GB300BeliefPropagationCache, pv::QuotientVertex; kwargs...)
    return device_scalars(bpc, :vertex)[bpc.plan.p.vid[pv] + 1]
end
function ITensorNetworks.region_scalar(bpc::GB300BeliefPropagationCache, pe::QuotientEdge; kwargs...)
    p = bpc.plan.p
    k = findfirst(e -> e == pe || e == reverse(pe), p.pes)
    return device_scalars(bpc, :edge)[k]
end
function ITensorNetworks.vertex_scalars(bpc::GB300BeliefPropagationCache, pvs=ITensorNetworks.partitions(bpc);
                                        kwargs...)
    vs = device_scalars(bpc, :vertex)
    return [vs[bpc.plan.p.vid[pv] + 1] for pv in pvs]
end

# logscalar(bpc) (abstractbeliefpropagationcache.jl:397-408), FP64 on the device
function ITensorNetworks.logscalar(bpc::GB300BeliefPropagationCache)
    re, im = Ref{Float64}(0.0), Ref{Float64}(0.0)
    check(context(), ccall((:gbtn_logscalar, libgbtn), Cint, (Ptr{Cvoid}, Ref{Float64}, Ref{Float64}),
        device_plan(bpc), re, im))
    return im[] == 0 ? re[] : complex(re[], im[])
end

# rescale(bpc; verts) = rescale_messages then rescale_partitions
# (abstractbeliefpropagationcache.jl:349-395) on the device; the rescaled
# tensors are read back into the cache's network (normalize.jl:63-80 returns
# its ket network).
function ITensorNetworks.rescale(bpc::GB300BeliefPropagationCache; kwargs...)
    h = device_plan(bpc)
    check(context(), ccall((:gbtn_rescale_messages, libgbtn), Cint, (Ptr{Cvoid},), h))
    check(context(), ccall((:gbtn_rescale_partitions, libgbtn), Cint, (Ptr{Cvoid},), h))
    p = bpc.plan.p
    flat = similar(p.data)
    check(context(), ccall((:gbtn_get_factors, libgbtn), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Cint), h, flat, 0))
    tn = tensornetwork(bpc)
    off = 0
    for (i, pv) in enumerate(p.pvs)
        v = parent(pv)
        t = tn[(v, "ket")]
        s = only(filter(j -> !(j in p.links), inds(t)))
        ls = filter(j -> j in p.links, collect(inds(t)))
        len = length(t)
        knew = itensor(convert(Array{eltype(t)}, reshape(flat[(off + 1):(off + len)], length(s), length.(ls)...)),
            s, ls...)
        off += len
        DataGraphs.set_vertex_data!(tn, knew, (v, "ket"))
        DataGraphs.set_vertex_data!(tn, dag(prime(knew)), (v, "bra"))
    end
    bpc.plan.uploaded = true  # the device already holds these tensors
    bpc.host_messages[] = nothing
    return bpc
end

# expect(alg, psi, ops; cache!) (expect.jl:21-41) with every one-site <O_v> =
# tr(rho_v O)/tr(rho_v) from the device (gbtn_expect1)
function ITensorNetworks.expect(alg::Algorithm"gb300_bp", ψ::ITensorNetworks.AbstractITensorNetwork, ops;
                                (cache!)=nothing, update_cache=isnothing(cache!), cache_update_kwargs=(;),
                                cache_construction_kwargs=(;), kwargs...)
    ψIψ = QuadraticFormNetwork(ψ)
    if isnothing(cache!)
        cache! = Ref(ITensorNetworks.initialize_cache(alg, ψIψ; cache_construction_kwargs...))
    end
    update_cache && (cache![] = ITensorNetworks.update(cache![]; cache_update_kwargs...))
    bpc = cache![]
    p = bpc.plan.p
    out = Float64[]
    for o in (ops isa Op ? [ops] : ops)
        v = only(o.sites)
        i = p.vid[only(filter(pv -> parent(pv) == v, p.pvs))]
        s = ITensorNetworks.siteinds(ψ)[v] |> only
        M = zeros(Float64, sum(Int(d)^2 for d in p.sdim))
        offs = cumsum(vcat(0, Int.(p.sdim) .^ 2))
        for (j, d) in enumerate(p.sdim)  # identity elsewhere; only vertex i is read
            M[(offs[j] + 1):offs[j + 1]] = vec(Matrix{Float64}(LinearAlgebra.I, Int(d), Int(d)))
        end
        M[(offs[i + 1] + 1):offs[i + 2]] = vec(real(array(ITensors.op(o.which_op, s), prime(s), s)))
        res = zeros(Float64, length(p.pvs))
        check(context(), ccall((:gbtn_expect1, libgbtn), Cint, (Ptr{Cvoid}, Ptr{Float64}, Cint, Ptr{Float64}),
            device_plan(bpc), M, 1, res))
        push!(out, res[i + 1])
    end
    return ops isa Op ? only(out) : out
end

# Pack a partitioned form network (one site partition per vertex: its ket,
# operator and bra) in the ABI layout; same as pack(bpc) for a cache.
pack_ptn(ptn) = pack(BeliefPropagationCache(ptn))
pack(bpc::GB300BeliefPropagationCache) = pack_ptn(bpc.partitioned_tensornetwork)

# ---- simple update (apply / tebd) -------------------------------------------

struct GradOpts
    mode::Int32
    maxiter::Int32
    tol::Float64
    unroll::Int32
    checkpoint::Int32
end

# Ket tensors of a plain ITensorNetwork in the ABI layout (vertex order of
# `vertices(psi)`, edges with src < dst, legs in each tensor's index order),
# as ComplexF64 when `cplx` (interleaved pairs in the library) else Float64.
function pack_state(psi; cplx=false)
    vs = collect(ITensorNetworks.vertices(psi))
    vid = Dict(v => i - 1 for (i, v) in enumerate(vs))
    es = collect(ITensorNetworks.edges(psi))
    links = [commonind(psi[ITensorNetworks.src(e)], psi[ITensorNetworks.dst(e)]) for e in es]
    eu = Int32[vid[ITensorNetworks.src(e)] for e in es]
    ev = Int32[vid[ITensorNetworks.dst(e)] for e in es]
    edim = Int32[length(l) for l in links]
    sdim, leg_ptr, leg_edge, sites = Int32[], Int32[0], Int32[], Index[]
    data = cplx ? ComplexF64[] : Float64[]
    for v in vs
        t = psi[v]
        s = only(filter(i -> !(i in links), inds(t)))
        ls = filter(i -> i in links, collect(inds(t)))
        append!(leg_edge, Int32[findfirst(==(l), links) - 1 for l in ls])
        push!(leg_ptr, length(leg_edge))
        push!(sdim, length(s))
        push!(sites, s)
        append!(data, vec(array(t, s, ls...)))
    end
    return (; vs, es, links, eu, ev, edim, sdim, leg_ptr, leg_edge, data, sites)
end

"""
    apply(Algorithm("gb300"), gates, psi; maxdim, cutoff=nothing, normalize=true, envs=nothing, callback)

Two-site `gates` (ITensors acting on the site indices of neighbouring vertices)
applied in order by the GPU simple update, one-site gates contracted into their
site tensor on the host (src/apply.jl:107-116); `callback(; singular_values,
truncation_error)` is called per gate as in src/apply.jl:97-146.  `envs`:
`nothing` (tebd) or a Dict from QuotientEdge to the converged message.
Complex gates (e.g. `op("RandomUnitary", ...)`), states or environments run
the library's complex path (complex_values = 1).
"""
function ITensorNetworks.apply(::Algorithm"gb300", gates::Vector{ITensor}, psi; maxdim, cutoff=nothing,
                               normalize=true, envs=nothing, callback=(; kws...) -> nothing)
    # one-site gates act on their site tensor on the host, as the reference's
    # apply does (src/apply.jl:107-116); the runs of two-site gates between
    # them go to the GPU in order
    if any(g -> length(inds(g)) == 2, gates)
        run = ITensor[]
        flush!(psi) = isempty(run) ? psi :
            ITensorNetworks.apply(Algorithm("gb300"), copy(run), psi; maxdim, cutoff, normalize, envs, callback)
        for g in gates
            if length(inds(g)) == 2
                psi = flush!(psi)
                empty!(run)
                v = only(filter(w -> hascommoninds(g, psi[w]), collect(ITensorNetworks.vertices(psi))))
                t = ITensors.apply(g, psi[v])
                normalize && (t ./= norm(t))
                psi = copy(psi)
                psi[v] = t
            else
                push!(run, g)
            end
        end
        return flush!(psi)
    end
    cplx = any(g -> eltype(g) <: Complex, gates) ||
           any(v -> eltype(psi[v]) <: Complex, ITensorNetworks.vertices(psi)) ||
           (envs !== nothing && any(m -> eltype(only(m)) <: Complex, values(envs)))
    T = cplx ? ComplexF64 : Float64
    p = pack_state(psi; cplx)
    ctx = context()
    chimax = max(maxdim, maximum(p.edim))
    eidx = Int32[]
    gdata = T[]
    for g in gates
        vs = [v for v in p.vs if !isempty(intersect(inds(g), [p.sites[findfirst(==(v), p.vs)]]))]
        su, sv = p.sites[findfirst(==(vs[1]), p.vs)], p.sites[findfirst(==(vs[2]), p.vs)]
        e = findfirst(k -> Set((p.eu[k], p.ev[k])) == Set((findfirst(==(vs[1]), p.vs) - 1,
                                                              findfirst(==(vs[2]), p.vs) - 1)), eachindex(p.eu))
        u_first = p.eu[e] == findfirst(==(vs[1]), p.vs) - 1
        a, b = u_first ? (su, sv) : (sv, su)
        push!(eidx, e - 1)
        append!(gdata, vec(array(g, prime(a), prime(b), a, b)))  # row s'_u + du s'_v, column s_u + du s_v
    end
    GC.@preserve p eidx gdata begin
        desc = GraphDesc(length(p.vs), length(p.es), pointer(p.eu), pointer(p.ev), pointer(p.edim),
            pointer(p.sdim), pointer(p.leg_ptr), pointer(p.leg_edge), C_NULL, 1, 0, cplx ? 1 : 0)
        h = Ref{Ptr{Cvoid}}(C_NULL)
        check(ctx, ccall((:gbtn_su_create, libgbtn), Cint, (Ptr{Cvoid}, Ref{GraphDesc}, Int32, Ref{Ptr{Cvoid}}),
            ctx, desc, chimax, h))
        try
            check(ctx, ccall((:gbtn_su_set_factors, libgbtn), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), h[], p.data))
            envbuf = C_NULL
            if envs !== nothing
                envbuf = zeros(T, 2 * length(p.es) * chimax^2)
                for (k, e) in enumerate(p.es), (dir, qe) in ((0, e), (1, reverse(e)))
                    M = array(only(envs[qe]))
                    c = size(M, 1)
                    o = (2 * (k - 1) + dir) * chimax^2
                    envbuf[(o + 1):(o + c * c)] = vec(M)
                end
            end
            n = length(gates)
            te = zeros(n)
            sv = zeros(n * maxdim)
            check(ctx, ccall((:gbtn_su_apply, libgbtn), Cint,
                (Ptr{Cvoid}, Int32, Ptr{Int32}, Ptr{Cvoid}, Int32, Ptr{Cvoid}, Int32, Float64, Int32,
                 Ptr{Float64}, Ptr{Float64}),
                h[], n, eidx, gdata, 1, envbuf, maxdim, something(cutoff, -1.0), normalize ? 1 : 0, te, sv))
            for j in 1:n
                s = sv[((j - 1) * maxdim + 1):(j * maxdim)]
                callback(; singular_values=s[s .> 0], truncation_error=te[j])
            end
            dims = zeros(Int32, length(p.es))
            check(ctx, ccall((:gbtn_su_edge_dims, libgbtn), Cint, (Ptr{Cvoid}, Ptr{Int32}), h[], dims))
            newlinks = [d == length(l) ? l : Index(Int(d), tags(l)) for (d, l) in zip(dims, p.links)]
            total = sum(Int(p.sdim[i]) * prod(Int(dims[p.leg_edge[q] + 1]) for q in (p.leg_ptr[i] + 1):p.leg_ptr[i + 1];
                                                 init=1) for i in eachindex(p.vs))
            flat = Vector{T}(undef, total)
            check(ctx, ccall((:gbtn_su_get_factors, libgbtn), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Int64),
                h[], flat, cplx ? 2 * total : total))
            psi = copy(psi)
            off = 0
            for (i, v) in enumerate(p.vs)
                ls = [newlinks[p.leg_edge[q] + 1] for q in (p.leg_ptr[i] + 1):p.leg_ptr[i + 1]]
                shp = (Int(p.sdim[i]), length.(ls)...)
                len = prod(shp)
                psi[v] = itensor(reshape(flat[(off + 1):(off + len)], shp), p.sites[i], ls...)
                off += len
            end
            return psi
        finally
            ccall((:gbtn_su_destroy, libgbtn), Cint, (Ptr{Cvoid},), h[])
        end
    end
end

"""
    tebd(Algorithm("gb300"), ℋ, ψ; β, Δβ, maxdim, cutoff, print_frequency=10, ortho=false)

src/tebd.jl:2-31 with the gate list applied by the GPU simple update: the
gates are the caller's ITensors `exp(-Δβ * ℋ; alg=Trotter{2}())`, so they are
the reference's; each of the `Int(β ÷ Δβ)` steps is one
`apply(Algorithm("gb300"), gates, ψ; maxdim, cutoff, normalize=true)`.  The
gates act on the two sites of an edge (on the GPU) or on one site (on the host,
as the reference's apply); `ortho=true` (tree_orthogonalize) is not provided.
"""
function ITensorNetworks.tebd(::Algorithm"gb300", ℋ, ψ; β, Δβ, maxdim, cutoff, print_frequency=10,
                              ortho=false)
    ortho && error("tebd(Algorithm(\"gb300\"), ...; ortho=true): tree_orthogonalize is not provided by libgbtn")
    𝒰 = exp(-Δβ * ℋ; alg=ITensors.Trotter{2}())
    u⃗ = Vector{ITensor}(𝒰, ITensorNetworks.siteinds(ψ))
    all(g -> length(inds(g)) in (2, 4), u⃗) ||
        error("tebd(Algorithm(\"gb300\")): gates act on one site or on the two sites of an edge")
    for step in 1:Int(β ÷ Δβ)
        step % print_frequency == 0 && @show step, (step - 1) * Δβ, β
        ψ = ITensorNetworks.apply(Algorithm("gb300"), u⃗, ψ; maxdim, cutoff, normalize=true)
    end
    return ψ
end

# ---- the simple update with its adjoint (ChainRulesCore) -----------------------

# Owner of a simple-update state and the tape of one taped apply; both are
# released when the pullback that holds it is collected.
mutable struct SUTape
    state::Ptr{Cvoid}
    tape::Ptr{Cvoid}
    function SUTape(state)
        t = new(state, C_NULL)
        finalizer(t) do x
            x.tape != C_NULL && ccall((:gbtn_su_tape_destroy, libgbtn), Cint, (Ptr{Cvoid},), x.tape)
            x.state != C_NULL && ccall((:gbtn_su_destroy, libgbtn), Cint, (Ptr{Cvoid},), x.state)
            x.tape = C_NULL
            x.state = C_NULL
        end
        return t
    end
end

"""
    gb300_apply(gates, psi; maxdim, cutoff=nothing, normalize=true, envs=nothing)

The two-site `gates` (real ITensors on the site indices of neighbouring
vertices) applied in order by the GPU simple update, as
`apply(Algorithm("gb300"), gates, psi; ...)`, differentiable: its rrule pulls
a cotangent of the returned network (a Dict vertex => ITensor with the
returned tensors' indices) back to the input tensors and to the gates, through
the library's taped adjoint (gbtn_su_apply_taped / gbtn_su_tape_vjp).  The
environments are constants.
"""
gb300_apply(gates::Vector{ITensor}, psi; kwargs...) = first(gb300_apply_with_pullback(gates, psi; kwargs...))

function gb300_apply_with_pullback(gates::Vector{ITensor}, psi; maxdim, cutoff=nothing, normalize=true,
                                   envs=nothing)
    all(g -> length(inds(g)) == 4 && eltype(g) <: Real, gates) ||
        error("gb300_apply: real two-site gates only")
    p = pack_state(psi)
    ctx = context()
    chimax = max(maxdim, maximum(p.edim))
    eidx = Int32[]
    gdata = Float64[]
    gsites = Tuple{Index, Index}[]
    for g in gates
        vs = [v for v in p.vs if !isempty(intersect(inds(g), [p.sites[findfirst(==(v), p.vs)]]))]
        iu, iv = findfirst(==(vs[1]), p.vs) - 1, findfirst(==(vs[2]), p.vs) - 1
        e = findfirst(k -> Set((p.eu[k], p.ev[k])) == Set((iu, iv)), eachindex(p.eu))
        a, b = p.eu[e] == iu ? (p.sites[iu + 1], p.sites[iv + 1]) : (p.sites[iv + 1], p.sites[iu + 1])
        push!(eidx, e - 1)
        push!(gsites, (a, b))
        append!(gdata, vec(array(g, prime(a), prime(b), a, b)))
    end
    envbuf = Float64[]
    if envs !== nothing
        envbuf = zeros(2 * length(p.es) * chimax^2)
        for (k, e) in enumerate(p.es), (dir, qe) in ((0, e), (1, reverse(e)))
            M = array(only(envs[qe]))
            c = size(M, 1)
            o = (2 * (k - 1) + dir) * chimax^2
            envbuf[(o + 1):(o + c * c)] = vec(M)
        end
    end
    n = length(gates)
    desc = GraphDesc(length(p.vs), length(p.es), pointer(p.eu), pointer(p.ev), pointer(p.edim),
        pointer(p.sdim), pointer(p.leg_ptr), pointer(p.leg_edge), C_NULL, 1, 0, 0)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    GC.@preserve p begin
        check(ctx, ccall((:gbtn_su_create, libgbtn), Cint, (Ptr{Cvoid}, Ref{GraphDesc}, Int32, Ref{Ptr{Cvoid}}),
            ctx, desc, chimax, h))
    end
    holder = SUTape(h[])
    check(ctx, ccall((:gbtn_su_set_factors, libgbtn), Cint, (Ptr{Cvoid}, Ptr{Float64}), holder.state, p.data))
    tref = Ref{Ptr{Cvoid}}(C_NULL)
    check(ctx, ccall((:gbtn_su_apply_taped, libgbtn), Cint,
        (Ptr{Cvoid}, Int32, Ptr{Int32}, Ptr{Float64}, Int32, Ptr{Float64}, Int32, Float64, Int32,
         Ptr{Float64}, Ptr{Float64}, Ref{Ptr{Cvoid}}),
        holder.state, n, eidx, gdata, 1, envs === nothing ? C_NULL : envbuf, maxdim, something(cutoff, -1.0),
        normalize ? 1 : 0, C_NULL, C_NULL, tref))
    holder.tape = tref[]
    dims = zeros(Int32, length(p.es))
    check(ctx, ccall((:gbtn_su_edge_dims, libgbtn), Cint, (Ptr{Cvoid}, Ptr{Int32}), holder.state, dims))
    newlinks = [d == length(l) ? l : Index(Int(d), tags(l)) for (d, l) in zip(dims, p.links)]
    legs(i, ls) = [ls[p.leg_edge[q] + 1] for q in (p.leg_ptr[i] + 1):p.leg_ptr[i + 1]]
    total = sum(Int(p.sdim[i]) * prod(length.(legs(i, newlinks)); init=1) for i in eachindex(p.vs))
    flat = Vector{Float64}(undef, total)
    check(ctx, ccall((:gbtn_su_get_factors, libgbtn), Cint, (Ptr{Cvoid}, Ptr{Float64}, Int64),
        holder.state, flat, total))
    out = copy(psi)
    off = 0
    for (i, v) in enumerate(p.vs)
        ls = legs(i, newlinks)
        len = Int(p.sdim[i]) * prod(length.(ls); init=1)
        out[v] = itensor(reshape(flat[(off + 1):(off + len)], Int(p.sdim[i]), length.(ls)...), p.sites[i], ls...)
        off += len
    end
    function pullback(dout)
        cot = Float64[]
        for (i, v) in enumerate(p.vs)
            append!(cot, vec(haskey(dout, v) ? array(dout[v], p.sites[i], legs(i, newlinks)...) :
                             zeros(Int(p.sdim[i]), length.(legs(i, newlinks))...)))
        end
        din = zeros(length(p.data))
        gc = zeros(length(gdata))
        check(ctx, ccall((:gbtn_su_tape_vjp, libgbtn), Cint,
            (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
            holder.state, holder.tape, cot, din, gc, C_NULL))
        dpsi = Dict{Any, ITensor}()
        o = 0
        for (i, v) in enumerate(p.vs)
            ls = legs(i, p.links)
            len = Int(p.sdim[i]) * prod(length.(ls); init=1)
            dpsi[v] = itensor(reshape(din[(o + 1):(o + len)], Int(p.sdim[i]), length.(ls)...), p.sites[i], ls...)
            o += len
        end
        dgates = ITensor[]
        og = 0
        for (a, b) in gsites
            da, db = length(a), length(b)
            len = (da * db)^2
            push!(dgates, itensor(reshape(gc[(og + 1):(og + len)], da, db, da, db), prime(a), prime(b), a, b))
            og += len
        end
        return dgates, dpsi
    end
    return out, pullback
end

function ChainRulesCore.rrule(::typeof(gb300_apply), gates::Vector{ITensor}, psi; kwargs...)
    out, pb = gb300_apply_with_pullback(gates, psi; kwargs...)
    function gb300_apply_pullback(dout)
        dgates, dpsi = pb(ChainRulesCore.unthunk(dout))
        return (NoTangent(), dgates, dpsi)
    end
    return out, gb300_apply_pullback
end

# ---- BP energy and its adjoint (ChainRulesCore) ------------------------------

"""
    bp_energy(psi, ops, coefs; maxiter=500)

sum_e sum_t coefs[t] <ops[t] (x) ops[t]>_e with BP reduced density matrices of
the converged (mixed-precision, FP64-refined) messages; ops are d x d matrices.
"""
function bp_energy(psi, ops::Vector{Matrix{Float64}}, coefs::Vector{Float64}; maxiter=500)
    return first(energy_and_grad(psi, ops, coefs; maxiter, want_grad=false))
end

function energy_and_grad(psi, ops, coefs; maxiter=500, want_grad=true)
    p = pack_state(psi)
    ctx = context()
    opbuf = reduce(vcat, vec.(ops))
    GC.@preserve p opbuf begin
        desc = GraphDesc(length(p.vs), length(p.es), pointer(p.eu), pointer(p.ev), pointer(p.edim),
            pointer(p.sdim), pointer(p.leg_ptr), pointer(p.leg_edge), C_NULL, 1, 0, 0)
        plan = Ref{Ptr{Cvoid}}(C_NULL)
        check(ctx, ccall((:gbtn_plan_create, libgbtn), Cint, (Ptr{Cvoid}, Ref{GraphDesc}, Ref{Ptr{Cvoid}}),
            ctx, desc, plan))
        try
            check(ctx, ccall((:gbtn_set_factors, libgbtn), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Cint),
                plan[], p.data, C_NULL, 0))
            opts = BPOpts(1, 3, maxiter, 1, 1e-14, C_NULL, 0, 0.0, 0.0, 0, 0, 0, 0, 0)
            check(ctx, ccall((:gbtn_bp_run, libgbtn), Cint, (Ptr{Cvoid}, Ref{BPOpts}, Ptr{Int32}, Ptr{Float64}),
                plan[], opts, C_NULL, C_NULL))
            E = Ref{Float64}(0.0)
            if !want_grad
                check(ctx, ccall((:gbtn_energy2, libgbtn), Cint, (Ptr{Cvoid}, Int32, Ptr{Float64}, Ptr{Float64},
                    Ref{Float64}), plan[], length(coefs), coefs, opbuf, E))
                return (E[], nothing)
            end
            grad = similar(p.data)
            gopts = GradOpts(0, 500, 1e-12, 0, 0)
            check(ctx, ccall((:gbtn_energy2_grad, libgbtn), Cint,
                (Ptr{Cvoid}, Int32, Ptr{Float64}, Ptr{Float64}, Ref{GradOpts}, Ref{Float64}, Ptr{Float64},
                 Ptr{Int32}, Ptr{Float64}),
                plan[], length(coefs), coefs, opbuf, gopts, E, grad, C_NULL, C_NULL))
            # unpack dE/dA into one ITensor per vertex (same indices as psi[v])
            dpsi = Dict{Any, ITensor}()
            off = 0
            for (i, v) in enumerate(p.vs)
                ls = [p.links[p.leg_edge[q] + 1] for q in (p.leg_ptr[i] + 1):p.leg_ptr[i + 1]]
                shp = (Int(p.sdim[i]), length.(ls)...)
                len = prod(shp)
                dpsi[v] = itensor(reshape(grad[(off + 1):(off + len)], shp), p.sites[i], ls...)
                off += len
            end
            return (E[], dpsi)
        finally
            ccall((:gbtn_plan_destroy, libgbtn), Cint, (Ptr{Cvoid},), plan[])
        end
    end
end

function ChainRulesCore.rrule(::typeof(bp_energy), psi, ops, coefs; maxiter=500)
    E, dpsi = energy_and_grad(psi, ops, coefs; maxiter)
    function bp_energy_pullback(dE)
        return (NoTangent(), Dict(v => dE * t for (v, t) in dpsi), NoTangent(), NoTangent())
    end
    return E, bp_energy_pullback
end

# ---- BP log-norm and one-site expectation values with their adjoints -----------

"""
    bp_logscalar(psi; maxiter=500)

Re logscalar of the BP cache of psi (abstractbeliefpropagationcache.jl:397-408)
at the converged (mixed-precision, refined) messages.
"""
bp_logscalar(psi; maxiter=500) = first(scalar_and_grad(psi, nothing; maxiter, want_grad=false))

"""
    bp_expect_sum(psi, op; maxiter=500)

Re sum_v <op>_v (expect.jl:5-19) with one d x d operator op[s', s] for every site.
"""
bp_expect_sum(psi, op::AbstractMatrix; maxiter=500) = first(scalar_and_grad(psi, op; maxiter, want_grad=false))

# value and gradient (dL/dA as one ITensor per vertex; for complex tensors
# dL/dRe + i dL/dIm, ChainRulesCore's convention) through the fixed point
function scalar_and_grad(psi, op; maxiter=500, want_grad=true)
    cplx = any(v -> eltype(psi[v]) <: Complex, ITensorNetworks.vertices(psi)) || eltype(op) <: Complex
    p = pack_state(psi; cplx)
    ctx = context()
    opbuf = op === nothing ? Float64[] : (cplx ? collect(reinterpret(Float64, vec(ComplexF64.(op)))) : vec(Float64.(op)))
    data = cplx ? reinterpret(Float64, p.data) : p.data
    GC.@preserve p opbuf data begin
        desc = GraphDesc(length(p.vs), length(p.es), pointer(p.eu), pointer(p.ev), pointer(p.edim),
            pointer(p.sdim), pointer(p.leg_ptr), pointer(p.leg_edge), C_NULL, 1, 0, cplx ? 1 : 0)
        plan = Ref{Ptr{Cvoid}}(C_NULL)
        check(ctx, ccall((:gbtn_plan_create, libgbtn), Cint, (Ptr{Cvoid}, Ref{GraphDesc}, Ref{Ptr{Cvoid}}),
            ctx, desc, plan))
        try
            check(ctx, ccall((:gbtn_set_factors, libgbtn), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Cint),
                plan[], data, C_NULL, 0))
            # real tensors: the mixed pipeline; complex ones: FP32 then FP64 sweeps
            opts = BPOpts(1, 3, maxiter, 1, 1e-14, C_NULL, 0, 0.0, 0.0, 0, 0, 0, 0, 0)
            check(ctx, ccall((:gbtn_bp_run, libgbtn), Cint, (Ptr{Cvoid}, Ref{BPOpts}, Ptr{Int32}, Ptr{Float64}),
                plan[], opts, C_NULL, C_NULL))
            val = Ref{Float64}(0.0)
            grad = similar(data)
            gopts = GradOpts(0, 500, 1e-12, 0, 0)
            if op === nothing
                check(ctx, ccall((:gbtn_logscalar_grad, libgbtn), Cint,
                    (Ptr{Cvoid}, Ref{GradOpts}, Ref{Float64}, Ptr{Float64}, Ptr{Int32}, Ptr{Float64}),
                    plan[], gopts, val, grad, C_NULL, C_NULL))
            else
                check(ctx, ccall((:gbtn_expect1_grad, libgbtn), Cint,
                    (Ptr{Cvoid}, Ptr{Float64}, Ref{GradOpts}, Ref{Float64}, Ptr{Float64}, Ptr{Int32}, Ptr{Float64}),
                    plan[], opbuf, gopts, val, grad, C_NULL, C_NULL))
            end
            want_grad || return (val[], nothing)
            g = cplx ? reinterpret(ComplexF64, grad) : grad
            dpsi = Dict{Any, ITensor}()
            off = 0
            for (i, v) in enumerate(p.vs)
                ls = [p.links[p.leg_edge[q] + 1] for q in (p.leg_ptr[i] + 1):p.leg_ptr[i + 1]]
                shp = (Int(p.sdim[i]), length.(ls)...)
                len = prod(shp)
                dpsi[v] = itensor(reshape(g[(off + 1):(off + len)], shp), p.sites[i], ls...)
                off += len
            end
            return (val[], dpsi)
        finally
            ccall((:gbtn_plan_destroy, libgbtn), Cint, (Ptr{Cvoid},), plan[])
        end
    end
end

function ChainRulesCore.rrule(::typeof(bp_logscalar), psi; maxiter=500)
    L, dpsi = scalar_and_grad(psi, nothing; maxiter)
    bp_logscalar_pullback(dL) = (NoTangent(), Dict(v => dL * t for (v, t) in dpsi))
    return L, bp_logscalar_pullback
end

function ChainRulesCore.rrule(::typeof(bp_expect_sum), psi, op; maxiter=500)
    X, dpsi = scalar_and_grad(psi, op; maxiter)
    bp_expect_sum_pullback(dX) = (NoTangent(), Dict(v => dX * t for (v, t) in dpsi), NoTangent())
    return X, bp_expect_sum_pullback
end

end
