"""Host-side network data model (the role of ITensorNetwork / IndsNetwork,
src/itensornetwork.jl, src/indsnetwork.jl) and edge schedules
(src/edge_sequences.jl).

A :class:`TensorNetwork` is a graph with one dense tensor per vertex.  Vertex
``v`` carries ``A_v[s, l_1, ..., l_k]`` (column-major, site index first, links
in the vertex's leg order), the layout the C ABI takes.  Many independent
networks become one :class:`TensorNetwork` through :func:`disjoint_union`; the
library then runs them side by side with per-network convergence."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib


class TensorNetwork:
    def __init__(self, nv, edges, site_dims, edge_dims, tensors=None, legs=None, vertex_network=None,
                 n_networks=1):
        self.nv = int(nv)
        self.edges = [(int(u), int(v)) for (u, v) in edges]
        self.site_dims = [int(d) for d in site_dims]
        self.edge_dims = [int(c) for c in edge_dims]
        if legs is None:
            # incident edges ordered by neighbour label (NamedGraphs' incident_edges order)
            inc = [[] for _ in range(self.nv)]
            for e, (u, v) in enumerate(self.edges):
                if u == v:
                    raise ValueError("self loops are not allowed")
                inc[u].append((v, e))
                inc[v].append((u, e))
            legs = [[e for (_, e) in sorted(lst)] for lst in inc]
        self.legs = [list(map(int, l)) for l in legs]
        self.vertex_network = None if vertex_network is None else [int(x) for x in vertex_network]
        self.n_networks = int(n_networks)
        self.tensors = tensors

    # -- structure -----------------------------------------------------------
    @property
    def ne(self):
        return len(self.edges)

    def shape(self, v):
        return (self.site_dims[v],) + tuple(self.edge_dims[e] for e in self.legs[v])

    def size(self, v):
        return int(np.prod(self.shape(v)))

    def other(self, v, e):
        u, w = self.edges[e]
        return w if u == v else u

    def directed(self, e, frm):
        return 2 * e if self.edges[e][0] == frm else 2 * e + 1

    def dsrc(self, de):
        u, v = self.edges[de // 2]
        return u if de % 2 == 0 else v

    def network_of(self, v):
        return 0 if self.vertex_network is None else self.vertex_network[v]

    def is_tree(self):
        if self.ne != self.nv - self.n_networks:
            return False
        parent = list(range(self.nv))

        def find(x):
            while parent[x] != x:
                parent[x] = parent[parent[x]]
                x = parent[x]
            return x
        for u, v in self.edges:
            ru, rv = find(u), find(v)
            if ru == rv:
                return False
            parent[ru] = rv
        return True

    # -- storage ---------------------------------------------------------------
    @property
    def is_complex(self):
        """Complex tensors (ComplexF64): the library then stores interleaved
        (re, im) doubles."""
        return self.tensors is not None and any(np.iscomplexobj(t) for t in self.tensors)

    def flat(self, tensors=None):
        ts = self.tensors if tensors is None else tensors
        dt = np.complex128 if any(np.iscomplexobj(t) for t in ts) else np.float64
        return np.ascontiguousarray(np.concatenate([np.asarray(t, dtype=dt).reshape(-1, order="F") for t in ts]))

    def unflat(self, flat):
        out, off = [], 0
        for v in range(self.nv):
            n = self.size(v)
            out.append(np.asarray(flat[off:off + n]).reshape(self.shape(v), order="F").copy())
            off += n
        return out

    def message_sizes(self):
        return [self.edge_dims[de // 2] ** 2 for de in range(2 * self.ne)]

    def unflat_messages(self, flat):
        out, off = [], 0
        for de in range(2 * self.ne):
            c = self.edge_dims[de // 2]
            out.append(np.asarray(flat[off:off + c * c]).reshape((c, c), order="F").copy())
            off += c * c
        return out

    def flat_messages(self, msgs, complex_values=None):
        cplx = any(np.iscomplexobj(m) for m in msgs) if complex_values is None else complex_values
        dt = np.complex128 if cplx else np.float64
        return np.ascontiguousarray(np.concatenate([np.asarray(m, dtype=dt).reshape(-1, order="F") for m in msgs]))

    def graph_desc(self, separate_bra=False):
        """(GraphDesc, keep-alive arrays) for gbtn_plan_create."""
        eu = np.ascontiguousarray([u for u, _ in self.edges] or [0], dtype=np.int32)
        ev = np.ascontiguousarray([v for _, v in self.edges] or [0], dtype=np.int32)
        ed = np.ascontiguousarray(self.edge_dims or [1], dtype=np.int32)
        sd = np.ascontiguousarray(self.site_dims, dtype=np.int32)
        lp = np.zeros(self.nv + 1, dtype=np.int32)
        for v in range(self.nv):
            lp[v + 1] = lp[v] + len(self.legs[v])
        le = np.ascontiguousarray([e for l in self.legs for e in l] or [0], dtype=np.int32)
        keep = [eu, ev, ed, sd, lp, le]
        d = _lib.GraphDesc()
        d.nv, d.ne = self.nv, self.ne
        d.edge_u, d.edge_v, d.edge_dim = _lib.iptr(eu), _lib.iptr(ev), _lib.iptr(ed)
        d.site_dim, d.leg_ptr, d.leg_edge = _lib.iptr(sd), _lib.iptr(lp), _lib.iptr(le)
        if self.vertex_network is not None:
            vn = np.ascontiguousarray(self.vertex_network, dtype=np.int32)
            keep.append(vn)
            d.vertex_network = _lib.iptr(vn)
            d.n_networks = self.n_networks
        else:
            d.vertex_network = C.cast(None, C.POINTER(C.c_int32))
            d.n_networks = 1
        d.separate_bra = 1 if separate_bra else 0
        d.complex_values = 1 if self.is_complex else 0
        return d, keep

    def shallow_copy(self):
        """A new network object sharing the tensor arrays: replacing its tensor
        list leaves this one untouched."""
        ts = None if self.tensors is None else list(self.tensors)
        return TensorNetwork(self.nv, self.edges, self.site_dims, self.edge_dims, ts,
                             [list(l) for l in self.legs], self.vertex_network, self.n_networks)

    def copy(self):
        ts = None if self.tensors is None else [t.copy() for t in self.tensors]
        return TensorNetwork(self.nv, self.edges, self.site_dims, self.edge_dims, ts,
                             [list(l) for l in self.legs], self.vertex_network, self.n_networks)


# -----------------------------------------------------------------------------
# Constructors
# -----------------------------------------------------------------------------

def square_lattice(Lx, Ly, chi=2, d=2, edge_dims=None):
    """Open Lx x Ly grid.  Vertex ``i + Lx*j`` is site (i+1, j+1) of
    ``named_grid((Lx, Ly))``; edges in ascending (src, dst) label order."""
    edges = []
    for j in range(Ly):
        for i in range(Lx):
            p = i + Lx * j
            if i + 1 < Lx:
                edges.append((p, p + 1))
            if j + 1 < Ly:
                edges.append((p, p + Lx))
    edges.sort()
    if edge_dims is None:
        edge_dims = [chi] * len(edges)
    return TensorNetwork(Lx * Ly, edges, [d] * (Lx * Ly), edge_dims)


def random_tensors(tn, seed, unit_norm=False):
    """I.i.d. N(0,1) tensors from numpy's PCG64 stream, drawn in vertex order."""
    rng = np.random.default_rng(seed)
    ts = []
    for v in range(tn.nv):
        shp = tn.shape(v)
        t = rng.standard_normal(int(np.prod(shp))).reshape(shp, order="F")
        if unit_norm:
            t = t / np.linalg.norm(t)
        ts.append(t)
    return ts


def random_network(tn, seed, unit_norm=False):
    out = tn.copy()
    out.tensors = random_tensors(tn, seed, unit_norm)
    return out


def disjoint_union(nets):
    """One TensorNetwork holding several independent networks (a batch)."""
    nv, edges, sd, ed, legs, vnet, ts = 0, [], [], [], [], [], []
    for k, t in enumerate(nets):
        eoff = len(edges)
        edges += [(u + nv, v + nv) for (u, v) in t.edges]
        ed += t.edge_dims
        sd += t.site_dims
        legs += [[e + eoff for e in l] for l in t.legs]
        vnet += [k] * t.nv
        if t.tensors is not None:
            ts += list(t.tensors)
        nv += t.nv
    return TensorNetwork(nv, edges, sd, ed, ts if ts else None, legs, vnet, len(nets))


# -----------------------------------------------------------------------------
# Edge schedules (src/edge_sequences.jl)
# -----------------------------------------------------------------------------

def _forest_cover(tn):
    remaining = list(range(tn.ne))
    forests = []
    while remaining:
        parent = list(range(tn.nv))

        def find(x):
            while parent[x] != x:
                parent[x] = parent[parent[x]]
                x = parent[x]
            return x
        forest, rest = [], []
        for e in remaining:
            u, v = tn.edges[e]
            ru, rv = find(u), find(v)
            if ru != rv:
                parent[ru] = rv
                forest.append(e)
            else:
                rest.append(e)
        forests.append(forest)
        remaining = rest
    return forests


def _post_order(tn, forest, root):
    adj = {}
    for e in forest:
        u, v = tn.edges[e]
        adj.setdefault(u, []).append((v, e))
        adj.setdefault(v, []).append((u, e))
    for k in adj:
        adj[k].sort()
    out, seen = [], {root}
    stack = [(root, None, 0)]
    while stack:
        v, via, i = stack[-1]
        nb = adj.get(v, [])
        while i < len(nb) and nb[i][0] in seen:
            i += 1
        if i == len(nb):
            stack.pop()
            if via is not None:
                out.append(tn.directed(via, v))
            continue
        stack[-1] = (v, via, i + 1)
        w, e = nb[i]
        seen.add(w)
        stack.append((w, e, 0))
    return out, seen


def default_edge_sequence(tn):
    """The ``"forest_cover"`` schedule: edge-disjoint spanning forests built
    greedily in edge order; for each tree (rooted at its smallest vertex) the
    post-order DFS edges towards the root, then their reverses in reverse
    order (edge_sequences.jl:32-47)."""
    seq = []
    for forest in _forest_cover(tn):
        verts = sorted({x for e in forest for x in tn.edges[e]})
        done = set()
        for r in verts:
            if r in done:
                continue
            tree, seen = _post_order(tn, forest, r)
            done |= seen
            seq += tree + [de ^ 1 for de in reversed(tree)]
    return seq


def parallel_edge_sequence(tn):
    """``edge_sequence(Algorithm"parallel")``: every edge, then every reverse."""
    return [2 * e for e in range(tn.ne)] + [2 * e + 1 for e in range(tn.ne)]
