# ITensorNetworksGB300Ext -- package extension that routes ITensorNetworks.jl's
# belief-propagation hot path to libgbtn.so (GB300, sm_103a) through ccall.
#
# Load order: `using ITensorNetworks, GB300TensorNetworks` activates this
# extension (weakdep GB300TensorNetworks in ITensorNetworks' Project.toml,
# `[extensions] ITensorNetworksGB300Ext = "GB300TensorNetworks"`).
#
# It adds the algorithm "gb300_bp": `update(bpc; alg="gb300_bp", maxiter, tol,
# schedule, precision)` packs the cache's partitioned tensor network into the
# C-ABI layout (include/gbtn.h), runs the sweeps on the GPU and writes the
# messages back into the cache, so `expect`, `environment`, `scalar`,
# `logscalar`, `inner`, `norm` and `normalize` keep their signatures and read
# converged messages as usual.  Real Float64/Float32 dense tensors with one
# site index per vertex, one link per edge and chi <= 8 are supported; other
# caches fall back to nothing -- they raise, as the library has no CPU path.
#
# Not executed in the environment this file was written in (no Julia
# toolchain); it documents the binding a maintainer adds.
module ITensorNetworksGB300Ext

using ITensorNetworks: ITensorNetworks, AbstractBeliefPropagationCache, BeliefPropagationCache,
    messages, set_messages, partitioned_tensornetwork, quotientedges, tensornetwork
using ITensors: ITensor, Index, inds, commonind, array, itensor, dag, prime
using NDTensors: Algorithm, @Algorithm_str
using NamedGraphs.PartitionedGraphs: QuotientEdge, quotientvertices
using GB300TensorNetworks: libgbtn

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

# Pack the ket layer of a QuadraticFormNetwork cache: vertex order =
# partitions, edges = quotient edges (src < dst), legs in each ket tensor's
# index order after the site index.
function pack(bpc::BeliefPropagationCache)
    pvs = collect(quotientvertices(bpc))
    vid = Dict(pv => i - 1 for (i, pv) in enumerate(pvs))
    pes = collect(quotientedges(bpc))
    tn = tensornetwork(bpc)
    ket(pv) = tn[(parent(pv), "ket")]
    eu = Int32[vid[src(pe)] for pe in pes]
    ev = Int32[vid[dst(pe)] for pe in pes]
    links = [commonind(ket(src(pe)), ket(dst(pe))) for pe in pes]
    edim = Int32[length(l) for l in links]
    sdim = Int32[]
    leg_ptr = Int32[0]
    leg_edge = Int32[]
    data = Float64[]
    for pv in pvs
        t = ket(pv)
        s = only(filter(i -> !(i in links), inds(t)))
        ls = filter(i -> i in links, collect(inds(t)))
        append!(leg_edge, Int32[findfirst(==(l), links) - 1 for l in ls])
        push!(leg_ptr, length(leg_edge))
        push!(sdim, length(s))
        append!(data, vec(array(t, s, ls...)))  # column-major, site index first
    end
    return (; pvs, pes, links, eu, ev, edim, sdim, leg_ptr, leg_edge, data)
end

function ITensorNetworks.update(alg::Algorithm"gb300_bp", bpc::BeliefPropagationCache)
    p = pack(bpc)
    ctx = context()
    GC.@preserve p begin
        desc = GraphDesc(length(p.pvs), length(p.pes), pointer(p.eu), pointer(p.ev), pointer(p.edim),
            pointer(p.sdim), pointer(p.leg_ptr), pointer(p.leg_edge), C_NULL, 1, 0)
        plan = Ref{Ptr{Cvoid}}(C_NULL)
        check(ctx, ccall((:gbtn_plan_create, libgbtn), Cint, (Ptr{Cvoid}, Ref{GraphDesc}, Ref{Ptr{Cvoid}}),
            ctx, desc, plan))
        try
            check(ctx, ccall((:gbtn_set_factors, libgbtn), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Cint),
                plan[], p.data, C_NULL, 0))
            sched = get(alg.kwargs, :schedule, "parallel") == "colored" ? 2 : 1
            prec = Dict("f64" => 0, "f32" => 1, "bf16" => 2, "mixed" => 3)[get(alg.kwargs, :precision, "f64")]
            tol = something(get(alg.kwargs, :tol, nothing), -1.0)
            opts = BPOpts(sched, prec, alg.kwargs.maxiter, 1, tol, C_NULL, 0, 0.0, 0.0, 0, 0, 0)
            iters = Ref{Int32}(0)
            diff = Ref{Float64}(0.0)
            check(ctx, ccall((:gbtn_bp_run, libgbtn), Cint, (Ptr{Cvoid}, Ref{BPOpts}, Ref{Int32}, Ref{Float64}),
                plan[], opts, iters, diff))
            nmsg = sum(Int(c)^2 for c in p.edim) * 2
            flat = Vector{Float64}(undef, nmsg)
            check(ctx, ccall((:gbtn_get_messages, libgbtn), Cint, (Ptr{Cvoid}, Ptr{Float64}, Cint),
                plan[], flat, 0))
            # unpack: directed edge 2e = u->v, 2e+1 = v->u; message M[b, a] with
            # b the bra (primed) link and a the ket link
            off = 0
            new = Dict{QuotientEdge, Vector{ITensor}}()
            for (e, pe) in enumerate(p.pes), (dir, qe) in ((0, pe), (1, reverse(pe)))
                c = Int(p.edim[e])
                M = reshape(flat[(off + 1):(off + c * c)], c, c)
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

end
