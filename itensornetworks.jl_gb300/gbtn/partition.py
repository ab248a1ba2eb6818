"""Belief propagation with multi-site partitions (``partitioned_vertices``,
src/caches/beliefpropagationcache.jl:24-35, exercised by
test/test_expect.jl:28-39).

In the reference a partition's message to a neighbouring partition is a tensor
over every (bra, ket) link pair that crosses between the two, and the update
contracts the partition's ket, operator and bra tensors with the incoming
messages.  Fusing the crossing links of each neighbouring pair into one index,
and the partition's site indices into one site index, turns this into ordinary
BP on the coarse network whose vertices are the partitions: the update
contracts the same tensors, the identity initial message is the product of
the per-link identities, and the Frobenius norm and message_diff do not see
the fusion.  The coarse tensors are contracted once here (the partition
contraction the reference repeats in every update); sweeps, environments and
scalars run on the GPU through the ordinary cache, within its limits
(fused site and bond dimensions <= 64; above 8 they run the global-memory
path, so square blocks of four sites at chi = 2 and columns of up to six
sites at d = chi = 2 are in reach).

Fusion order: the sites of a partition in the order given, the first fastest;
the crossing edges of a neighbouring pair by ascending edge id, the first
fastest (column-major, like every other index of the ABI)."""
from __future__ import annotations

import numpy as np

from .network import TensorNetwork


class CoarseGraining:
    """The coarse network of ``tn`` for ``partitions`` (lists of vertices that
    cover every vertex once) and the maps back to the original sites."""

    def __init__(self, tn: TensorNetwork, partitions):
        parts = [[int(v) for v in p] for p in partitions]
        seen = sorted(v for p in parts for v in p)
        if seen != list(range(tn.nv)):
            raise ValueError("partitions must cover every vertex exactly once")
        if any(len(p) == 0 for p in parts):
            raise ValueError("empty partition")
        self.tn = tn
        self.parts = parts
        self.part_of = np.empty(tn.nv, dtype=np.int64)
        for i, p in enumerate(parts):
            self.part_of[p] = i
        crossing = {}
        self.internal = []
        for e, (u, v) in enumerate(tn.edges):
            a, b = int(self.part_of[u]), int(self.part_of[v])
            if a == b:
                self.internal.append(e)
            else:
                crossing.setdefault((min(a, b), max(a, b)), []).append(e)
        self.coarse_pairs = sorted(crossing)
        self.crossing = [sorted(crossing[k]) for k in self.coarse_pairs]  # original edges per coarse edge
        site_dims = [int(np.prod([tn.site_dims[v] for v in p])) for p in parts]
        edge_dims = [int(np.prod([tn.edge_dims[e] for e in es])) for es in self.crossing]
        self.coarse = TensorNetwork(len(parts), self.coarse_pairs, site_dims, edge_dims)
        if tn.tensors is not None:
            self.coarse.tensors = [self._contract(i) for i in range(len(parts))]

    def _contract(self, i):
        """The partition's tensors contracted over its internal edges, indices
        (fused sites, fused crossing legs in the coarse network's leg order)."""
        tn, p = self.tn, self.parts[i]
        label = {}

        def lab(key):
            if key not in label:
                label[key] = len(label)
            return label[key]

        ops = []
        for v in p:
            ops += [np.asarray(tn.tensors[v]), [lab(("s", v))] + [lab(("e", e)) for e in tn.legs[v]]]
        out = [lab(("s", v)) for v in p]
        shape = [self.coarse.site_dims[i]]
        for ce in self.coarse.legs[i]:
            out += [lab(("e", e)) for e in self.crossing[ce]]
            shape.append(self.coarse.edge_dims[ce])
        t = np.einsum(*ops, out, optimize=True)
        return np.ascontiguousarray(t.reshape(shape, order="F"))

    def _contract_vjp(self, i, cot):
        """The adjoint of _contract: dL/d(each site tensor of partition i) from
        dL/d(its coarse tensor), the cotangent contracted with the partition's
        other tensors."""
        tn, p = self.tn, self.parts[i]
        label = {}

        def lab(key):
            if key not in label:
                label[key] = len(label)
            return label[key]

        labs = {v: [lab(("s", v))] + [lab(("e", e)) for e in tn.legs[v]] for v in p}
        out = [lab(("s", v)) for v in p]
        dims = [tn.site_dims[v] for v in p]
        for ce in self.coarse.legs[i]:
            out += [lab(("e", e)) for e in self.crossing[ce]]
            dims += [tn.edge_dims[e] for e in self.crossing[ce]]
        c = np.asarray(cot).reshape(dims, order="F")
        res = {}
        for v in p:
            ops = [c, out]
            for w in p:
                if w != v:
                    ops += [np.asarray(tn.tensors[w]), labs[w]]
            res[v] = np.einsum(*ops, labs[v], optimize=True)
        return res

    def tensor_cotangents(self, coarse_cot):
        """dL/d(original site tensors) from dL/d(coarse tensors)."""
        out = [None] * self.tn.nv
        for i in range(len(self.parts)):
            for v, g in self._contract_vjp(i, coarse_cot[i]).items():
                out[v] = g
        return out

    def fused_operator(self, op):
        """sum_{v in p} 1 (x) .. op_v .. (x) 1 on a partition's fused site index
        (first site fastest), the same for every partition; partitions must
        share their sites' dimensions in order."""
        shapes = {tuple(self.tn.site_dims[v] for v in p) for p in self.parts}
        if len(shapes) != 1:
            raise ValueError("partitions of different site dimensions have no common fused operator")
        ds = next(iter(shapes))
        op = np.asarray(op)
        total = 0
        for j in range(len(ds)):
            m = np.ones((1, 1), dtype=op.dtype)
            for q in reversed(range(len(ds))):
                m = np.kron(m, op if q == j else np.eye(ds[q], dtype=op.dtype))
            total = total + m
        return total

    def site_rdms(self, coarse_rdms):
        """Single-site reduced density matrices of every original vertex from
        the coarse vertices' (fused-site) ones, by partial trace."""
        out = [None] * self.tn.nv
        for i, p in enumerate(self.parts):
            dims = [self.tn.site_dims[v] for v in p]
            k = len(p)
            rho = np.asarray(coarse_rdms[i]).reshape(dims + dims, order="F")
            for j, v in enumerate(p):
                keep = [j, k + j]
                sub = list(range(2 * k))
                for a in range(k):
                    if a != j:
                        sub[k + a] = sub[a]  # trace s'_a = s_a
                res = np.einsum(rho, sub, keep)
                out[v] = res
        return out


class PartitionedBPCache:
    """BeliefPropagationCache over multi-site partitions: update / expect /
    logscalar / scalar with the reference's meaning, computed on the coarse
    network (see the module docstring)."""

    def __init__(self, tn: TensorNetwork, partitions, ctx=None):
        from .cache import BeliefPropagationCache
        if tn.tensors is None:
            raise ValueError("the network has no tensors")
        self.cg = CoarseGraining(tn, partitions)
        self.cache = BeliefPropagationCache(self.cg.coarse, ctx=ctx)

    def update(self, **kw):
        self.cache.update(**kw)
        return self

    @property
    def iterations(self):
        return self.cache.iterations

    def messages(self):
        """Coarse messages: one fused-bra x fused-ket matrix per directed coarse edge."""
        return self.cache.messages()

    def site_rdms(self):
        return self.cg.site_rdms(self.cache.vertex_rdms())

    def expect(self, op):
        """<O_v> for every original vertex, op = d x d matrix O[s', s]."""
        op = np.asarray(op, float)
        out = np.empty(self.cg.tn.nv)
        for v, r in enumerate(self.site_rdms()):
            out[v] = float(np.sum(r * op) / np.trace(r))
        return out

    def logscalar(self):
        return self.cache.logscalar()

    # -- gradients: the coarse plan's hand-written adjoints at its converged
    #    messages, pulled back through the partition contraction
    def logscalar_grad(self, **kw):
        """(Re logscalar, dL/d(site tensors)) at the converged messages."""
        val, G = self.cache.logscalar_grad(**kw)
        return val, self.cg.tensor_cotangents(G)

    def expect_sum_grad(self, op, **kw):
        """(sum_v <op>_v over every original site, its gradient): the coarse
        expectation of the fused operator (partitions of equal site dimensions)."""
        val, G = self.cache.expect_sum_grad(self.cg.fused_operator(op), **kw)
        return val, self.cg.tensor_cotangents(G)

    def scalar(self):
        return self.cache.scalar()

    def close(self):
        self.cache.close()


def partitioned_cache(tn: TensorNetwork, partitions, ctx=None):
    """BeliefPropagationCache(tn; partitioned_vertices) for multi-site partitions."""
    return PartitionedBPCache(tn, partitions, ctx)
