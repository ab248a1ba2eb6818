"""BeliefPropagationCache on the GPU and the reference-facing entry points.

Mirrors the interface of ITensorNetworks.jl's BP cache and its users:

* ``BeliefPropagationCache`` / ``initialize_cache`` -- src/caches/beliefpropagationcache.jl:13-35,
  src/initialize_cache.jl:14-28 (identity messages on loopy graphs)
* ``update(bpc; maxiter, tol, edge_sequence, ...)`` -- abstractbeliefpropagationcache.jl:313-337
* ``updated_message`` / ``message_diff`` -- :225-239, :32-36
* ``environment`` -- beliefpropagationcache.jl:100-105
* ``vertex_scalars`` / ``edge_scalars`` / ``logscalar`` / ``scalar`` -- :83-97, :397-412
* ``rescale_messages`` / ``rescale_partitions`` / ``rescale`` -- beliefpropagationcache.jl:121-139,
  abstractbeliefpropagationcache.jl:349-395
* ``expect`` -- src/expect.jl:21-109; ``inner``/``loginner``/``norm_sqr``/``norm`` -- src/inner.jl;
  ``logscalar``/``scalar`` on networks -- src/contract.jl:41-62; ``normalize``/``rescale`` -- src/normalize.jl.

All arithmetic runs in libgbtn on the GPU; this module only moves arrays and
keeps the bookkeeping.  The cache is updated in place and returned, where the
reference returns an updated copy."""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib
from ._lib import check, dptr, iptr
from .network import TensorNetwork, default_edge_sequence


def bp_opts(maxiter, tol, schedule, seq, precision, normalize, mixed):
    """gbtn_bp_opts for one update; ``seq`` (int32, kept alive by the caller)
    is the directed-edge sequence of the sequential schedule, else None;
    ``mixed`` holds the per-phase limits (tol_bf16, tol_f32, maxiter_bf16,
    maxiter_f32, refine_f64, refine, confirm_f64)."""
    o = _lib.BPOpts()
    o.schedule = _lib.SCHED[schedule]
    o.precision = _lib.PRECISION[precision]
    o.maxiter = int(maxiter)
    o.normalize = 1 if normalize else 0
    o.tol = -1.0 if tol is None else float(tol)
    if seq is not None:
        o.edge_sequence = iptr(seq)
        o.edge_sequence_len = len(seq)
    else:
        o.edge_sequence = C.cast(None, C.POINTER(C.c_int32))
        o.edge_sequence_len = 0
    o.tol_bf16 = float(mixed.get("tol_bf16", 0.0))
    o.tol_f32 = float(mixed.get("tol_f32", 0.0))
    o.maxiter_bf16 = int(mixed.get("maxiter_bf16", 0))
    o.maxiter_f32 = int(mixed.get("maxiter_f32", 0))
    o.refine_f64 = int(mixed.get("refine_f64", 0))
    o.refine = _lib.REFINE[mixed.get("refine", "df32")]
    o.confirm_f64 = int(mixed.get("confirm_f64", 0))
    return o


class BeliefPropagationCache:
    def __init__(self, tn: TensorNetwork, messages=None, bra=None, ctx=None):
        if tn.tensors is None:
            raise ValueError("the network has no tensors")
        # the cache's own network object: set_factors and rescale_partitions
        # replace its tensor list, never the caller's (rescale and normalize
        # return new networks, as in the reference)
        tn = tn.shallow_copy()
        self.tn = tn
        self.ctx = ctx or _lib.default_context()
        self.lib = self.ctx.lib
        self.separate_bra = bra is not None
        # complex tensors (ComplexF64): interleaved (re, im) doubles on the device
        self.complex = tn.is_complex or (bra is not None and any(np.iscomplexobj(t) for t in bra))
        self.dtype = np.complex128 if self.complex else np.float64
        # element type the messages are reported in (the reference's messages
        # keep the tensors' eltype: Float32, Float64, ComplexF32, ComplexF64)
        ts = list(tn.tensors) + (list(bra) if bra is not None else [])
        single = all(np.asarray(t).dtype in (np.float32, np.complex64) for t in ts)
        self.elt = np.dtype((np.complex64 if self.complex else np.float32) if single else self.dtype)
        if self.complex and not tn.is_complex:
            tn = tn.copy()
            tn.tensors = [np.asarray(t, dtype=np.complex128) for t in tn.tensors]
            self.tn = tn
        desc, keep = tn.graph_desc(separate_bra=self.separate_bra)
        h = C.c_void_p()
        check(self.ctx.handle, self.lib.gbtn_plan_create(self.ctx.handle, C.byref(desc), C.byref(h)))
        self.handle = h
        nf, nm = C.c_int64(), C.c_int64()
        check(self.ctx.handle, self.lib.gbtn_plan_sizes(h, C.byref(nf), C.byref(nm)))
        self.n_factor, self.n_message = nf.value, nm.value
        self.set_factors(tn.tensors, bra)
        if messages is not None:
            self.set_messages(messages)

    # -- storage ---------------------------------------------------------------
    def _c(self, code):
        check(self.ctx.handle, code)

    def set_factors(self, ket, bra=None):
        k = self.tn.flat([np.asarray(t, dtype=self.dtype) for t in ket])
        if self.separate_bra:
            b = self.tn.flat([np.asarray(t, dtype=self.dtype) for t in bra])
            self._c(self.lib.gbtn_set_factors(self.handle, k.ctypes.data, b.ctypes.data, _lib.HOST))
            self.bra_tensors = [np.asarray(t, dtype=self.dtype) for t in bra]
        else:
            self._c(self.lib.gbtn_set_factors(self.handle, k.ctypes.data, None, _lib.HOST))
        self.tn.tensors = [np.asarray(t, dtype=self.dtype) for t in ket]

    def update_factors(self, factors, bra_factors=None):
        """update_factors(bpc, factors) (abstractbeliefpropagationcache.jl:158-165):
        ``factors`` maps vertices to new site tensors of the same shape (and,
        for a cache with a separate bra, ``bra_factors`` the bra's); the
        messages are kept.  One upload of all tensors.  Unlike the reference,
        which returns a copy, the cache is updated in place and returned."""
        def merged(current, new):
            out = list(current)
            for v, t in dict(new or {}).items():
                t = np.asarray(t)
                if not 0 <= int(v) < self.tn.nv:
                    raise _lib.InvalidArgument(1, f"vertex {v} is not in the network")
                if tuple(t.shape) != tuple(self.tn.shape(int(v))):
                    raise _lib.InvalidArgument(
                        1, f"factor of vertex {v} has shape {tuple(t.shape)}, expected {tuple(self.tn.shape(int(v)))}")
                out[int(v)] = t
            return out
        ket = merged(self.tn.tensors, factors)
        bra = merged(self.bra_tensors, bra_factors) if self.separate_bra else None
        self.set_factors(ket, bra)
        return self

    def update_factor(self, vertex, factor, bra_factor=None):
        """update_factor(bpc, vertex, factor) (:167-171) for one vertex."""
        return self.update_factors({vertex: factor}, None if bra_factor is None else {vertex: bra_factor})

    def factors(self):
        out = np.empty(self.n_factor, dtype=self.dtype)
        self._c(self.lib.gbtn_get_factors(self.handle, out.ctypes.data, _lib.HOST))
        return self.tn.unflat(out)

    def messages(self):
        out = np.empty(max(self.n_message, 1), dtype=self.dtype)
        self._c(self.lib.gbtn_get_messages(self.handle, out.ctypes.data, _lib.HOST))
        return [m.astype(self.elt, copy=False) for m in self.tn.unflat_messages(out)]

    def flat_messages(self):
        """Every message in the ABI layout: directed edges in order, each
        chi x chi column-major."""
        out = np.empty(max(self.n_message, 1), dtype=self.dtype)
        self._c(self.lib.gbtn_get_messages(self.handle, out.ctypes.data, _lib.HOST))
        return out[:self.n_message]

    def edge_diffs(self):
        """message_diff of every directed edge from the last sweep run with a
        tolerance (NaN before the first)."""
        out = np.empty(max(2 * self.tn.ne, 1))
        self._c(self.lib.gbtn_get_edge_diffs(self.handle, out.ctypes.data, _lib.HOST))
        return out[:2 * self.tn.ne]

    def message(self, de):
        return self.messages()[de]

    def set_messages(self, msgs):
        flat = (self.tn.flat_messages(msgs, self.complex) if isinstance(msgs, (list, tuple))
                else np.ascontiguousarray(msgs, dtype=self.dtype))
        self._c(self.lib.gbtn_set_messages(self.handle, flat.ctypes.data, _lib.HOST))

    def init_messages(self, kind="identity"):
        self._c(self.lib.gbtn_init_messages(self.handle, _lib.INIT[kind]))

    # -- message passing -------------------------------------------------------
    def default_maxiter(self):
        """1 on trees, none on loopy graphs (abstractbeliefpropagationcache.jl:38-41)."""
        return 1 if self.tn.is_tree() else None

    def update(self, maxiter=None, tol=None, schedule="sequential", edge_sequence=None, precision="f64",
               normalize=True, verbose=False, **mixed):
        """Run BP sweeps; returns the cache.  ``schedule``: "sequential" (the
        reference default, forest-cover order unless ``edge_sequence`` is
        given), "parallel" (Jacobi) or "colored" (colour-class Gauss-Seidel)."""
        if maxiter is None:
            maxiter = self.default_maxiter()
        if maxiter is None:
            raise _lib.InvalidArgument(1, "You need to specify a number of iterations for BP!")
        seq = None
        if schedule == "sequential":
            if edge_sequence is None:
                if getattr(self, "_default_seq", None) is None:  # the graph is fixed for the cache's life
                    self._default_seq = np.ascontiguousarray(default_edge_sequence(self.tn), dtype=np.int32)
                seq = self._default_seq
            else:
                seq = np.ascontiguousarray(edge_sequence, dtype=np.int32)
        o = bp_opts(maxiter, tol, schedule, seq, precision, normalize, mixed)
        it = np.zeros(self.tn.n_networks, dtype=np.int32)
        md = np.zeros(self.tn.n_networks)
        self._c(self.lib.gbtn_bp_run(self.handle, C.byref(o), iptr(it), dptr(md)))
        self.iterations, self.mean_diff = it, md
        if verbose:
            for n in range(self.tn.n_networks):
                if tol is not None and md[n] <= tol:
                    print(f"BP converged to desired precision after {it[n]} iterations.")
        return self

    def phase_sweeps(self):
        """Sweeps of each phase of the last update (most over the networks):
        {"bf16", "f32", "refine", "f64"}; 0 for a phase that did not run."""
        out = np.zeros(4, dtype=np.int32)
        self._c(self.lib.gbtn_plan_phase_sweeps(self.handle, iptr(out)))
        return dict(zip(("bf16", "f32", "refine", "f64"), (int(x) for x in out)))

    def set_tc_policy(self, policy):
        """Tensor-core routing of the BF16 phase: "auto" (timed on this plan's
        vertices), "all" (every d = 2, degree <= 4, chi <= 8 vertex, padded),
        "native" (degree 4, chi = 8 only) or "off"."""
        self._c(self.lib.gbtn_plan_set_tc_policy(self.handle, _lib.TC_POLICIES[policy]))
        return self

    def set_simt_tuning(self, mode=True):
        """SIMT team width per size class: True = measured (default), False =
        the fixed rule, 32 / 128 / 256 = that width wherever it fits."""
        m = {True: 1, False: 0}.get(mode, mode) if isinstance(mode, bool) else int(mode)
        self._c(self.lib.gbtn_plan_set_simt_tuning(self.handle, m))
        return self

    def simt_teams(self, precision="f64"):
        """{n_bound: team} chosen for an arithmetic ("f64", "f32", "df32",
        "z64", "z32"), n_bound = 2^k for every measured size class."""
        arith = {"f64": 0, "f32": 1, "df32": 2, "z64": 3, "z32": 4}[precision]
        out = np.zeros(32, dtype=np.int32)
        self._c(self.lib.gbtn_plan_simt_teams(self.handle, arith, iptr(out)))
        return {1 << k: int(t) for k, t in enumerate(out) if t}

    def set_graphs(self, on=True):
        """Replay the sweeps of parallel / coloured runs from CUDA graphs."""
        self._c(self.lib.gbtn_plan_set_graphs(self.handle, 1 if on else 0))
        return self

    def tc_split(self):
        """(is_tc per vertex as a bool array, measured ms of the chosen split)."""
        out = np.zeros(max(self.tn.nv, 1), dtype=np.int32)
        ms = C.c_double(0.0)
        self._c(self.lib.gbtn_plan_tc_split(self.handle, iptr(out), C.byref(ms)))
        return out[:self.tn.nv].astype(bool), ms.value

    def updated_message(self, de):
        c = self.tn.edge_dims[de // 2]
        out = np.empty(c * c, dtype=self.dtype)
        self._c(self.lib.gbtn_updated_message(self.handle, int(de), dptr(out.view(np.float64))))
        return out.reshape((c, c), order="F").astype(self.elt, copy=False)

    # -- environments and scalars ---------------------------------------------
    def environment(self, verts):
        """Incoming messages into the partitions of ``verts`` (directed edge id,
        message) and the vertex tensors (beliefpropagationcache.jl:100-105)."""
        vs = set(verts)
        msgs = self.messages()
        incoming = []
        for v in verts:
            for e in self.tn.legs[v]:
                w = self.tn.other(v, e)
                if w in vs:
                    continue
                de = self.tn.directed(e, w)
                incoming.append((de, msgs[de]))
        return incoming, [self.tn.tensors[v] for v in verts]

    def vertex_rdms(self):
        n = sum(d * d for d in self.tn.site_dims)
        out = np.empty(n, dtype=self.dtype)
        self._c(self.lib.gbtn_vertex_rdms(self.handle, dptr(out.view(np.float64))))
        res, off = [], 0
        for d in self.tn.site_dims:
            res.append(out[off:off + d * d].reshape((d, d), order="F"))
            off += d * d
        return res

    def edge_rdms(self, edges=None):
        edges = list(range(self.tn.ne)) if edges is None else list(edges)
        if not edges:
            return []
        es = np.ascontiguousarray(edges, dtype=np.int32)
        Ds = [self.tn.site_dims[self.tn.edges[e][0]] * self.tn.site_dims[self.tn.edges[e][1]] for e in edges]
        out = np.empty(sum(D * D for D in Ds), dtype=self.dtype)
        self._c(self.lib.gbtn_edge_rdms(self.handle, iptr(es), len(edges), dptr(out.view(np.float64))))
        res, off = [], 0
        for D in Ds:
            res.append(out[off:off + D * D].reshape((D, D), order="F"))
            off += D * D
        return res

    def vertex_scalars(self):
        out = np.empty(self.tn.nv, dtype=self.dtype)
        self._c(self.lib.gbtn_vertex_scalars(self.handle, dptr(out.view(np.float64))))
        return out

    def edge_scalars(self):
        out = np.empty(max(self.tn.ne, 1), dtype=self.dtype)
        self._c(self.lib.gbtn_edge_scalars(self.handle, dptr(out.view(np.float64))))
        return out[:self.tn.ne]

    def logscalar(self):
        """Per network log of the BP estimate (a Python complex when negative
        terms appear, -inf when an edge scalar is zero)."""
        re = np.empty(self.tn.n_networks)
        im = np.empty(self.tn.n_networks)
        self._c(self.lib.gbtn_logscalar(self.handle, dptr(re), dptr(im)))
        vals = [complex(r, i) if i != 0.0 else float(r) for r, i in zip(re, im)]
        return vals[0] if self.tn.n_networks == 1 else vals

    def scalar(self):
        ls = self.logscalar()
        f = (lambda x: complex(np.exp(x)) if isinstance(x, complex) else math.exp(x))
        return f(ls) if not isinstance(ls, list) else [f(x) for x in ls]

    def expect(self, op, per_vertex=False):
        """<O_v> per vertex: ``op`` is a d x d matrix O[s', s], a list of them
        (per_vertex), or the name of a real S=1/2 operator ("Sz", "Sx", "S+",
        "S-", "Id") as in the reference's expect(psi, "Sz")."""
        if isinstance(op, str):
            from .opsum import named_operator
            op, per_vertex = named_operator(op, self.tn), False
        out = np.empty(self.tn.nv)
        if per_vertex:
            ops = np.ascontiguousarray(np.concatenate([np.asarray(o, float).reshape(-1, order="F") for o in op]))
        else:
            ops = np.ascontiguousarray(np.asarray(op, float).reshape(-1, order="F"))
        self._c(self.lib.gbtn_expect1(self.handle, dptr(ops), 1 if per_vertex else 0, dptr(out)))
        return out

    def expect2(self, op2, edges=None):
        edges = list(range(self.tn.ne)) if edges is None else list(edges)
        es = np.ascontiguousarray(edges, dtype=np.int32)
        op = np.ascontiguousarray(np.asarray(op2, float).reshape(-1, order="F"))
        out = np.empty(len(edges))
        self._c(self.lib.gbtn_expect2(self.handle, iptr(es), len(edges), dptr(op), dptr(out)))
        return out

    # -- energies and gradients -----------------------------------------------
    def _terms(self, terms):
        """(coefficients, operators in the plan's element type as doubles)."""
        coef = np.ascontiguousarray([float(c) for c, _ in terms])
        ops = np.ascontiguousarray(np.concatenate([np.asarray(o, self.dtype).reshape(-1, order="F") for _, o in terms]))
        return coef, ops.view(np.float64)

    def energy2(self, terms):
        """sum_e sum_t c_t <O_t (x) O_t>_e over every edge (terms = [(c_t, O_t)])."""
        coef, ops = self._terms(terms)
        out = np.empty(self.tn.n_networks)
        self._c(self.lib.gbtn_energy2(self.handle, len(terms), dptr(coef), dptr(ops), dptr(out)))
        return out[0] if self.tn.n_networks == 1 else out

    def energy2_grad(self, terms, mode="implicit", maxiter=500, tol=1e-12, unroll=30, checkpoint=0):
        """(energy, [dE/dA_v]) through the converged messages ("implicit") or
        through `unroll` Jacobi sweeps from identity messages ("unrolled").
        Complex networks: the real part of the energy, and the gradient as
        dE/dRe + i dE/dIm."""
        coef, ops = self._terms(terms)
        o = _lib.GradOpts()
        o.mode = 0 if mode == "implicit" else 1
        o.maxiter, o.tol, o.unroll, o.checkpoint = int(maxiter), float(tol), int(unroll), int(checkpoint)
        e = np.empty(self.tn.n_networks)
        g = np.empty(self.n_factor, dtype=self.dtype)
        it = np.zeros(1, dtype=np.int32)
        res = np.zeros(1)
        self._c(self.lib.gbtn_energy2_grad(self.handle, len(terms), dptr(coef), dptr(ops), C.byref(o), dptr(e),
                                           dptr(g.view(np.float64)), iptr(it), dptr(res)))
        self.adjoint_iterations, self.adjoint_residual = int(it[0]), float(res[0])
        return (e[0] if self.tn.n_networks == 1 else e), self.tn.unflat(g)

    def vjp(self, msg_cot, maxiter=500, tol=1e-12, mode="implicit", unroll=30, checkpoint=0):
        """dL/dA from dL/dm: at the fixed point (mode "implicit", implicit
        differentiation at the messages in the cache) or through `unroll`
        Jacobi sweeps from identity messages (mode "unrolled", checkpointed
        every `checkpoint` sweeps, default sqrt(unroll); those sweeps' final
        messages stay in the cache).  Complex networks: cotangents and
        gradients are dL/dRe + i dL/dIm of a real loss L."""
        mc = (self.tn.flat_messages(msg_cot, self.complex) if isinstance(msg_cot, (list, tuple))
              else np.ascontiguousarray(msg_cot, self.dtype))
        o = _lib.GradOpts()
        o.mode, o.maxiter, o.tol = (0 if mode == "implicit" else 1), int(maxiter), float(tol)
        o.unroll, o.checkpoint = int(unroll), int(checkpoint)
        g = np.empty(self.n_factor, dtype=self.dtype)
        it = np.zeros(1, dtype=np.int32)
        res = np.zeros(1)
        self._c(self.lib.gbtn_bp_vjp(self.handle, dptr(mc.view(np.float64)), C.byref(o), dptr(g.view(np.float64)),
                                     iptr(it), dptr(res)))
        return self.tn.unflat(g)

    def _scalar_grad(self, fn, extra, maxiter, tol):
        o = _lib.GradOpts()
        o.mode, o.maxiter, o.tol = 0, int(maxiter), float(tol)
        val = np.empty(self.tn.n_networks)
        g = np.empty(self.n_factor, dtype=self.dtype)
        it = np.zeros(1, dtype=np.int32)
        res = np.zeros(1)
        self._c(fn(self.handle, *extra, C.byref(o), dptr(val), dptr(g.view(np.float64)), iptr(it), dptr(res)))
        self.grad_iterations, self.grad_residual = int(it[0]), float(res[0])
        return (float(val[0]) if self.tn.n_networks == 1 else val), self.tn.unflat(g)

    def logscalar_grad(self, maxiter=500, tol=1e-12):
        """(Re logscalar, its gradient dA) at the current (converged) messages:
        the direct derivative plus the implicit part through the BP fixed point.
        Quadratic-form networks, real or complex (gradient dL/dRe + i dL/dIm);
        summed over a batch's networks for the gradient, per network for the
        value."""
        return self._scalar_grad(self.lib.gbtn_logscalar_grad, (), maxiter, tol)

    def expect_sum_grad(self, op, maxiter=500, tol=1e-12):
        """(Re sum_v <O_v>, its gradient dA) at the current (converged)
        messages, one d x d operator O[s', s] for every vertex."""
        op = np.ascontiguousarray(np.asarray(op, dtype=self.dtype).reshape(-1, order="F"))
        return self._scalar_grad(self.lib.gbtn_expect1_grad, (dptr(op.view(np.float64)),), maxiter, tol)

    # -- rescaling -------------------------------------------------------------
    def rescale_messages(self):
        self._c(self.lib.gbtn_rescale_messages(self.handle))
        return self

    def rescale_partitions(self):
        self._c(self.lib.gbtn_rescale_partitions(self.handle))
        self.tn.tensors = self.factors()
        return self

    def rescale(self):
        return self.rescale_messages().rescale_partitions()

    def close(self):
        if getattr(self, "handle", None):
            self.lib.gbtn_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# -----------------------------------------------------------------------------
# Module-level functions with the reference's names
# -----------------------------------------------------------------------------

def initialize_cache(tn, messages=None, bra=None, ctx=None):
    """``initialize_cache(Algorithm"bp", QuadraticFormNetwork(tn))``: identity
    messages (trees included; one sweep overwrites them there)."""
    return BeliefPropagationCache(tn, messages=messages, bra=bra, ctx=ctx)


def update(bpc, **kwargs):
    return bpc.update(**kwargs)


def updated_message(bpc, de):
    return bpc.updated_message(de)


def message_diff(a, b):
    """1 - |<a/|a|, b/|b|>|^2 (host-side helper on two message matrices, real
    or complex; abstractbeliefpropagationcache.jl:32-36)."""
    a = np.asarray(a, np.complex128 if np.iscomplexobj(a) or np.iscomplexobj(b) else np.float64)
    b = np.asarray(b, a.dtype)
    return 1.0 - abs(np.vdot(a / np.linalg.norm(a), b / np.linalg.norm(b))) ** 2


def _cache_for(tn, cache, update_cache, cache_update_kwargs, bra=None):
    if cache is None:
        cache = initialize_cache(tn, bra=bra)
        update_cache = True if update_cache is None else update_cache
    elif update_cache is None:
        update_cache = False
    if update_cache:
        cache.update(**(cache_update_kwargs or {}))
    return cache


def expect(psi, op, vertices=None, alg="bp", cache=None, update_cache=None, cache_update_kwargs=None):
    """<psi|O_v|psi>/<psi|psi> on every vertex (expect.jl:58-109); ``op`` is a
    d x d matrix O[s', s] or the name of a real S=1/2 operator ("Sz").  Returns
    a numpy array (or the subset ``vertices``)."""
    if alg != "bp":
        raise ValueError("only alg='bp' runs on the GPU")
    cache = _cache_for(psi, cache, update_cache, cache_update_kwargs)
    out = cache.expect(op)
    return out if vertices is None else out[list(vertices)]


def environment(bpc, verts):
    return bpc.environment(verts)


# Functions of a cache under the reference's names (the reference calls them
# with the cache as first argument; abstractbeliefpropagationcache.jl:83-97,
# 158-175, beliefpropagationcache.jl:107-119).
def messages(bpc):
    return bpc.messages()


def message(bpc, directed_edge):
    return bpc.message(directed_edge)


def vertex_scalars(bpc):
    return bpc.vertex_scalars()


def edge_scalars(bpc):
    return bpc.edge_scalars()


def update_factor(bpc, vertex, factor):
    return bpc.update_factor(vertex, factor)


def incoming_messages(bpc, verts, ignore_edges=()):
    """incoming_messages(bpc, partition_vertices; ignore_edges)
    (abstractbeliefpropagationcache.jl:99-107): the messages on directed edges
    entering ``verts`` from outside, except the directed edges listed in
    ``ignore_edges``, as (directed edge, message) pairs."""
    skip = set(int(d) for d in ignore_edges)
    incoming, _ = bpc.environment(list(verts))
    return [(de, m) for de, m in incoming if de not in skip]


def factors(bpc, verts=None):
    """factors(bpc, verts) (abstractbeliefpropagationcache.jl:75-81): the site
    tensors of ``verts`` (all vertices when None), read back from the device."""
    ts = bpc.factors()
    return ts if verts is None else [ts[int(v)] for v in verts]


def default_bp_maxiter(bpc):
    """1 on a tree, None (maxiter required) on a loopy graph
    (abstractbeliefpropagationcache.jl:38-41)."""
    return bpc.default_maxiter()


def region_scalar(bpc, vertex=None, edge=None):
    """region_scalar(bpc, pv) / region_scalar(bpc, pe) (beliefpropagationcache.jl:107-119):
    the partition scalar of a vertex (its tensors with all incoming messages)
    or the scalar <m_e, m_ebar> of an edge; give exactly one of the two."""
    if (vertex is None) == (edge is None):
        raise ValueError("give a vertex or an edge")
    return bpc.vertex_scalars()[vertex] if edge is None else bpc.edge_scalars()[edge]


def scalar_factors_quotient(bpc):
    """(vertex scalars, edge scalars), the factors of the BP estimate
    prod_v Z_v / prod_e <m_e, m_ebar> (abstractbeliefpropagationcache.jl:95-97)."""
    return bpc.vertex_scalars(), bpc.edge_scalars()


def update_factors(bpc, factors):
    return bpc.update_factors(factors)


def identity_messages(tn):
    """The initial messages of a quadratic form (quadraticformnetwork.jl:96-124):
    the chi x chi identity delta(dag(k'), k) on every directed edge, in
    directed-edge order."""
    return [np.eye(tn.edge_dims[de // 2]) for de in range(2 * tn.ne)]


def logscalar(tn, alg="bp", cache=None, update_cache=None, cache_update_kwargs=None, bra=None):
    """logscalar(alg, tn; cache!, ...) (contract.jl:41-58) on <bra|tn> (bra =
    conj(tn) when not given)."""
    if alg != "bp":
        raise ValueError("only alg='bp' runs on the GPU")
    return _cache_for(tn, cache, update_cache, cache_update_kwargs, bra).logscalar()


def scalar(tn, alg="bp", **kw):
    ls = logscalar(tn, alg=alg, **kw)
    return complex(np.exp(ls)) if isinstance(ls, complex) else math.exp(ls)


def loginner(phi, psi, alg="bp", **kw):
    """log <phi|psi> by BP on the two-layer network (inner.jl:93-149)."""
    return logscalar(psi, alg=alg, bra=phi.tensors, **kw)


def inner(phi, psi, alg="bp", **kw):
    """<phi|psi> by BP (inner.jl:151-160)."""
    ls = loginner(phi, psi, alg=alg, **kw)
    return complex(np.exp(ls)) if isinstance(ls, complex) else math.exp(ls)


def norm_sqr(psi, alg="bp", **kw):
    return scalar(psi, alg=alg, **kw)


def norm(psi, alg="bp", **kw):
    return math.sqrt(abs(float(np.real(norm_sqr(psi, alg=alg, **kw)))))


def rescale(tn, alg="bp", cache=None, update_cache=None, cache_update_kwargs=None):
    """rescale(alg, tn; cache!) (normalize.jl:23-31): every partition scalar 1."""
    cache = _cache_for(tn, cache, update_cache, cache_update_kwargs)
    cache.rescale()
    out = tn.copy()
    out.tensors = cache.factors()
    return out


def normalize(tn, alg="bp", cache=None, update_cache=None, cache_update_kwargs=None):
    """normalize(alg="bp") (normalize.jl:63-80): rescale the messages, then the
    ket/bra partitions, so the BP norm of the returned state is 1."""
    return rescale(tn, alg=alg, cache=cache, update_cache=update_cache, cache_update_kwargs=cache_update_kwargs)
