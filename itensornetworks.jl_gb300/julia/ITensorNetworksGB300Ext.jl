# ITensorNetworksGB300Ext -- package extension that routes ITensorNetworks.jl's
# belief-propagation hot path to libgbtn.so (GB300, sm_103a) through ccall.
#
# Load order: `using ITensorNetworks, GB300TensorNetworks` activates this
# extension (weakdep GB300TensorNetworks in ITensorNetworks' Project.toml,
# `[extensions] ITensorNetworksGB300Ext = "GB300TensorNetworks"`).
#
# It adds the algorithm "gb300_bp": `update(bpc; alg="gb300_bp", maxiter, tol,
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
# and a ChainRulesCore rrule for `bp_energy(psi, ops, coefs)`, the BP
# two-site energy, whose pullback is the library's hand-written adjoint
# (implicit differentiation at the BP fixed point).
#
# Not executed in the environment this file was written in (no Julia
# toolchain); it documents the binding a maintainer adds.
module ITensorNetworksGB300Ext

using ITensorNetworks: ITensorNetworks, AbstractBeliefPropagationCache, BeliefPropagationCache,
    messages, set_messages, partitioned_tensornetwork, quotientedges, tensornetwork
using ITensors: ITensors, ITensor, Index, inds, commonind, hascommoninds, array, itensor, dag, prime, tags
using LinearAlgebra: norm
using NDTensors: Algorithm, @Algorithm_str
using Graphs: src, dst
using NamedGraphs.PartitionedGraphs: QuotientEdge, quotientvertices
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

end
