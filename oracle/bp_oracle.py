"""FP64 CPU oracle for the belief-propagation (BP) hot path of ITensorNetworks.jl.

TEST INFRASTRUCTURE ONLY.  This module is the checker: only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg import it.  The
product path (``itensornetworks.jl_gb300/``) never calls it.

It restates, in plain NumPy float64/complex128 arithmetic, the reference
algorithm on the quadratic-form network <psi|psi> (ket A_v, identity operator,
bra conj(A_v) per site partition):

* message update            ``src/caches/abstractbeliefpropagationcache.jl:225-239``
  (incoming messages ``:99-107``; contract, Frobenius-normalise unless zero)
* message diff              ``abstractbeliefpropagationcache.jl:32-36``
* sequential sweep          ``abstractbeliefpropagationcache.jl:272-287``
* parallel (Jacobi) sweep   ``abstractbeliefpropagationcache.jl:294-308`` (every
  group computed from the pre-iteration cache; the reference body raises a
  MethodError at ``:302``, so the intended semantics are restated)
* ``update`` loop           ``abstractbeliefpropagationcache.jl:313-329``
  (convergence when sum(diff)/len(sequence) <= tol)
* identity messages         ``src/formnetworks/quadraticformnetwork.jl:96-124``
* forest-cover edge order   ``src/edge_sequences.jl:32-47``
* environment / expect      ``src/caches/beliefpropagationcache.jl:100-105``,
  exact environment ``src/environment.jl:6-20``,
  ``src/expect.jl:5-19``; two-site RDM ``test/test_belief_propagation.jl:64-91``
* region scalars, logscalar ``beliefpropagationcache.jl:107-119``,
  ``abstractbeliefpropagationcache.jl:397-412``
* rescale / normalize       ``beliefpropagationcache.jl:121-139``,
  ``abstractbeliefpropagationcache.jl:349-395``, ``src/normalize.jl:63-80``
* tebd                      ``src/tebd.jl:2-31`` (Trotter{2} gates, Strang
  splitting), ``test/utils.jl:174-192,239-246`` (Ising model, group_terms)
* simple update (apply)     ``src/apply.jl:9-146`` with ITensors' truncation
  rule restated in :func:`truncate_spectrum`.

Conventions shared with the GPU library (and the C-ABI):

* graph: vertices ``0..nv-1``; undirected edges ``e`` with endpoints
  ``edges[e] = (u, v)``; directed edge ``2e`` is ``u -> v``, ``2e+1`` is ``v -> u``.
* vertex tensor ``A_v`` has shape ``(d_v, chi_{legs[v][0]}, ..., chi_{legs[v][k-1]})``
  stored column-major (site index fastest), as NDTensors' Dense storage.
* a message on directed edge ``u -> v`` is a ``chi x chi`` matrix ``M[b, a]``
  with ``b`` the bra (primed) link and ``a`` the ket link, column-major.

Parity status: pinned against the reference's own self-consistency tests
(BP exact on trees vs. exact contraction, fixed-point residual, zero network,
rescale -> unit scalars, map_eigvals identities).  The reference publishes no
numeric golden vectors and cannot run here (no Julia), so the forest-cover
edge order and the SVD truncation details follow the documented restatements
below ("parity unpinned" for those two items only).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


# ----------------------------------------------------------------------------
# Graph / network data model
# ----------------------------------------------------------------------------

@dataclass
class Graph:
    nv: int
    edges: list  # [(u, v)] undirected, u != v
    site_dims: list  # d_v
    edge_dims: list  # chi_e
    legs: list = field(default=None)  # legs[v] = [edge ids in tensor leg order]

    def __post_init__(self):
        self.edges = [(int(u), int(v)) for (u, v) in self.edges]
        self.site_dims = [int(d) for d in self.site_dims]
        self.edge_dims = [int(c) for c in self.edge_dims]
        if self.legs is None:
            # NamedGraphs' incident_edges order: neighbours in ascending label order.
            inc = [[] for _ in range(self.nv)]
            for e, (u, v) in enumerate(self.edges):
                inc[u].append((v, e))
                inc[v].append((u, e))
            self.legs = [[e for (_, e) in sorted(lst)] for lst in inc]

    @property
    def ne(self):
        return len(self.edges)

    def other(self, v, e):
        u, w = self.edges[e]
        return w if u == v else u

    def directed(self, e, frm):
        """Directed edge id of edge ``e`` leaving vertex ``frm``."""
        return 2 * e if self.edges[e][0] == frm else 2 * e + 1

    def dsrc(self, de):
        u, v = self.edges[de // 2]
        return u if de % 2 == 0 else v

    def ddst(self, de):
        u, v = self.edges[de // 2]
        return v if de % 2 == 0 else u

    def shape(self, v):
        return (self.site_dims[v],) + tuple(self.edge_dims[e] for e in self.legs[v])

    def is_forest(self):
        uf = list(range(self.nv))

        def find(x):
            while uf[x] != x:
                uf[x] = uf[uf[x]]
                x = uf[x]
            return x
        for u, v in self.edges:
            ru, rv = find(u), find(v)
            if ru == rv:
                return False
            uf[ru] = rv
        return True


def square_lattice(Lx, Ly, chi=2, d=2, edge_dims=None):
    """Open-boundary Lx x Ly grid.  Vertex ``i + Lx*j`` is site (i+1, j+1); the
    ordering (first coordinate fastest) and edge order (ascending (src, dst)
    labels) follow NamedGraphs' ``named_grid`` over Graphs' integer labels."""
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
    return Graph(Lx * Ly, edges, [d] * (Lx * Ly), edge_dims)


def random_tree(n, seed, chi=2, d=2):
    """Random labelled tree on n vertices (each vertex i>0 attaches to a random
    earlier vertex)."""
    rng = np.random.default_rng(seed)
    edges = sorted((int(rng.integers(0, i)), i) for i in range(1, n))
    return Graph(n, edges, [d] * n, [chi] * len(edges))


def comb_tree(nx, ny, chi=2, d=2):
    """Comb tree: a spine along the first row, teeth along the second coordinate
    (the shape of NamedGraphs' ``named_comb_tree``)."""
    edges = []
    for j in range(ny):
        for i in range(nx):
            p = i + nx * j
            if j == 0 and i + 1 < nx:
                edges.append((p, p + 1))
            if j + 1 < ny:
                edges.append((p, p + nx))
    edges.sort()
    return Graph(nx * ny, edges, [d] * (nx * ny), [chi] * len(edges))


def random_network(g, seed, dtype=np.float64, unit_norm=False):
    """I.i.d. N(0,1) site tensors from ``numpy.random.Generator(PCG64(seed))``,
    drawn in vertex order, each in column-major flat order."""
    rng = np.random.default_rng(seed)
    ts = []
    for v in range(g.nv):
        shp = g.shape(v)
        n = int(np.prod(shp))
        if np.issubdtype(dtype, np.complexfloating):
            flat = rng.standard_normal(n) + 1j * rng.standard_normal(n)
        else:
            flat = rng.standard_normal(n)
        t = flat.reshape(shp, order="F").astype(dtype)
        if unit_norm:
            t = t / np.linalg.norm(t)
        ts.append(t)
    return ts


def flatten_tensors(ts):
    return np.concatenate([np.asarray(t).reshape(-1, order="F") for t in ts])


def unflatten_tensors(g, flat):
    out, off = [], 0
    for v in range(g.nv):
        shp = g.shape(v)
        n = int(np.prod(shp))
        out.append(np.asarray(flat[off:off + n]).reshape(shp, order="F"))
        off += n
    return out


def flatten_messages(g, msgs):
    return np.concatenate([np.asarray(msgs[de]).reshape(-1, order="F") for de in range(2 * g.ne)])


def unflatten_messages(g, flat):
    out, off = [], 0
    for de in range(2 * g.ne):
        c = g.edge_dims[de // 2]
        out.append(np.asarray(flat[off:off + c * c]).reshape((c, c), order="F"))
        off += c * c
    return out


# ----------------------------------------------------------------------------
# Initial messages and edge sequences
# ----------------------------------------------------------------------------

def identity_messages(g, dtype=np.float64):
    """delta(bra, ket) on every crossing link (quadraticformnetwork.jl:96-124)."""
    return [np.eye(g.edge_dims[de // 2], dtype=dtype) for de in range(2 * g.ne)]


def ones_messages(g, dtype=np.float64):
    """All-ones messages normalised to unit Frobenius norm."""
    out = []
    for de in range(2 * g.ne):
        c = g.edge_dims[de // 2]
        out.append(np.full((c, c), 1.0 / c, dtype=dtype))
    return out


def forest_cover(g):
    """Edge-disjoint spanning forests covering every edge, built greedily in
    ascending edge order (the role of NamedGraphs' ``forest_cover``)."""
    remaining = list(range(g.ne))
    forests = []
    while remaining:
        uf = list(range(g.nv))

        def find(x):
            while uf[x] != x:
                uf[x] = uf[uf[x]]
                x = uf[x]
            return x
        forest, rest = [], []
        for e in remaining:
            u, v = g.edges[e]
            ru, rv = find(u), find(v)
            if ru != rv:
                uf[ru] = rv
                forest.append(e)
            else:
                rest.append(e)
        forests.append(forest)
        remaining = rest
    return forests


def post_order_dfs_edges(g, forest_edges, root):
    """Directed edges (child -> parent) of the tree containing ``root`` in
    post-order of a DFS from ``root`` visiting neighbours in ascending order."""
    adj = {}
    for e in forest_edges:
        u, v = g.edges[e]
        adj.setdefault(u, []).append((v, e))
        adj.setdefault(v, []).append((u, e))
    for k in adj:
        adj[k].sort()
    out, seen = [], {root}
    stack = [(root, None, iter(adj.get(root, [])))]
    while stack:
        v, via, it = stack[-1]
        nxt = None
        for (w, e) in it:
            if w not in seen:
                nxt = (w, e)
                break
        if nxt is None:
            stack.pop()
            if via is not None:
                out.append(g.directed(via, v))  # child v -> parent
            continue
        w, e = nxt
        seen.add(w)
        stack.append((w, e, iter(adj.get(w, []))))
    return out, seen


def default_edge_sequence(g):
    """forest_cover schedule (edge_sequences.jl:32-47): for every tree of every
    forest, its post-order DFS edges towards the root (smallest vertex), then
    the reverses of those edges in reverse order."""
    seq = []
    for forest in forest_cover(g):
        verts = sorted({x for e in forest for x in g.edges[e]})
        done = set()
        for r in verts:
            if r in done:
                continue
            tree_edges, seen = post_order_dfs_edges(g, forest, r)
            done |= seen
            seq += tree_edges + [de ^ 1 for de in reversed(tree_edges)]
    return seq


def parallel_edge_sequence(g):
    """``edge_sequence(Algorithm"parallel")``: all edges, then all reverses."""
    return [2 * e for e in range(g.ne)] + [2 * e + 1 for e in range(g.ne)]


def vertex_colors(g):
    """Greedy proper colouring in vertex order (checkerboard on a grid)."""
    col = [-1] * g.nv
    nbrs = [[] for _ in range(g.nv)]
    for (u, v) in g.edges:
        nbrs[u].append(v)
        nbrs[v].append(u)
    for v in range(g.nv):
        used = {col[w] for w in nbrs[v] if col[w] >= 0}
        c = 0
        while c in used:
            c += 1
        col[v] = c
    return col


# ----------------------------------------------------------------------------
# Message update and sweeps
# ----------------------------------------------------------------------------

def _incoming(g, msgs, v, skip_leg=None):
    """(leg position, message into v) for every leg except ``skip_leg``."""
    out = []
    for p, e in enumerate(g.legs[v]):
        if p == skip_leg:
            continue
        de_in = g.directed(e, g.other(v, e))
        out.append((p, msgs[de_in]))
    return out


def contract_partition(g, A, B, msgs, v, open_leg=None, open_site=False):
    """Contract ket A_v, bra conj(B_v) and incoming messages at vertex v.

    ``open_leg``: leg position left open (result gains [b, a] of that leg).
    ``open_site``: site indices left open (result gains [s', s]).
    Result index order: [s', s] (if open_site) then [b, a] (if open_leg)."""
    a = A[v]
    b = np.conj(B[v])
    k = a.ndim - 1
    S, SP = 0, 1
    ket = [S] + [2 + p for p in range(k)]
    bra = [SP if open_site else S] + [2 + k + p for p in range(k)]
    ops = [a, ket, b, bra]
    for p, m in _incoming(g, msgs, v, skip_leg=open_leg):
        ops += [m, [2 + k + p, 2 + p]]
    out = []
    if open_site:
        out += [SP, S]
    if open_leg is not None:
        out += [2 + k + open_leg, 2 + open_leg]
    return np.einsum(*ops, out, optimize=True)


def updated_message(g, A, B, msgs, de, normalize=True):
    """m_{v->w}: contract incoming messages (except from w) with the partition
    tensors of v, then divide by the Frobenius norm unless it is zero."""
    v = g.dsrc(de)
    e = de // 2
    p = g.legs[v].index(e)
    m = contract_partition(g, A, B, msgs, v, open_leg=p)
    nrm = np.linalg.norm(m)
    if normalize and nrm != 0:
        m = m / nrm
    return m


def message_diff(a, b):
    """1 - |<a/|a|, b/|b|>|^2 (abstractbeliefpropagationcache.jl:32-36)."""
    na = np.linalg.norm(a)
    nb = np.linalg.norm(b)
    with np.errstate(invalid="ignore", divide="ignore"):
        f = abs(np.vdot(a / na, b / nb)) ** 2
    return 1.0 - f


def bp_update(g, A, msgs, *, B=None, maxiter, tol=None, schedule="sequential",
              edge_sequence=None, normalize=True):
    """``update(bpc; maxiter, tol, edge_sequence)``.  Returns
    ``(messages, iterations_run, last_mean_diff)``."""
    if maxiter is None:
        raise ValueError("You need to specify a number of iterations for BP!")
    B = A if B is None else B
    msgs = [m.copy() for m in msgs]
    if edge_sequence is None:
        edge_sequence = (default_edge_sequence(g) if schedule == "sequential"
                         else parallel_edge_sequence(g))
    colors = vertex_colors(g) if schedule == "colored" else None
    it, mean_diff = 0, float("nan")
    for it in range(1, maxiter + 1):
        diff = 0.0
        if schedule == "sequential":
            for de in edge_sequence:
                new = updated_message(g, A, B, msgs, de, normalize)
                if tol is not None:
                    diff += message_diff(new, msgs[de])
                msgs[de] = new
        elif schedule == "parallel":
            new = {de: updated_message(g, A, B, msgs, de, normalize) for de in edge_sequence}
            for de in edge_sequence:
                if tol is not None:
                    diff += message_diff(new[de], msgs[de])
            for de in edge_sequence:
                msgs[de] = new[de]
        elif schedule == "colored":
            for c in range(max(colors) + 1):
                des = [de for de in edge_sequence if colors[g.dsrc(de)] == c]
                new = {de: updated_message(g, A, B, msgs, de, normalize) for de in des}
                for de in des:
                    if tol is not None:
                        diff += message_diff(new[de], msgs[de])
                    msgs[de] = new[de]
        else:
            raise ValueError(schedule)
        # an empty sequence divides 0 by 0: NaN, never <= tol, so the loop runs
        # maxiter no-op iterations (abstractbeliefpropagationcache.jl:320)
        mean_diff = diff / len(edge_sequence) if len(edge_sequence) else float("nan")
        if tol is not None and mean_diff <= tol:
            break
    return msgs, it, mean_diff


# ----------------------------------------------------------------------------
# Environments, scalars, expectation values
# ----------------------------------------------------------------------------

def vertex_rdm(g, A, B, msgs, v):
    """rho_v[s', s] = env contracted with ket (s) and bra (s') at v."""
    return contract_partition(g, A, B, msgs, v, open_site=True)


def vertex_scalar(g, A, B, msgs, v):
    """region_scalar of the partition of v (beliefpropagationcache.jl:107-113)."""
    return np.trace(vertex_rdm(g, A, B, msgs, v))


def edge_scalar(g, msgs, e):
    """region_scalar of a quotient edge: contract(m_e, m_reverse(e))."""
    return np.sum(msgs[2 * e] * msgs[2 * e + 1])


def logscalar(g, A, B, msgs):
    """sum_v log Z_v - sum_e log <m_e, m_ebar> (abstractbeliefpropagationcache.jl:397-408)."""
    num = np.array([vertex_scalar(g, A, B, msgs, v) for v in range(g.nv)])
    den = np.array([edge_scalar(g, msgs, e) for e in range(g.ne)])
    if np.any(np.real(num) < 0):
        num = num.astype(complex)
    if np.any(np.real(den) < 0):
        den = den.astype(complex)
    if np.any(den == 0):
        return -np.inf
    with np.errstate(divide="ignore"):
        return np.sum(np.log(num)) - np.sum(np.log(den))


def expect1(g, A, msgs, op, B=None, vertices=None):
    """<O_v> = tr(rho_v O) / tr(rho_v) with O[s', s] (expect.jl:5-19)."""
    B = A if B is None else B
    vertices = range(g.nv) if vertices is None else vertices
    out = []
    for v in vertices:
        rho = vertex_rdm(g, A, B, msgs, v)
        o = op[v] if isinstance(op, (list, tuple)) else op
        out.append(np.sum(rho * o) / np.trace(rho))
    return np.array(out)


def edge_rdm(g, A, B, msgs, e):
    """Two-site RDM rho[(s'_u, s'_v), (s_u, s_v)] for edge e=(u,v), as the
    reference's test builds it (test_belief_propagation.jl:64-91): incoming
    messages into {u, v} except the two on e, with the ket link and the bra
    link of e contracted directly."""
    u, v = g.edges[e]
    pu = g.legs[u].index(e)
    pv = g.legs[v].index(e)
    Ru = contract_partition(g, A, B, msgs, u, open_leg=pu, open_site=True)  # [s'u, su, b, a]
    Rv = contract_partition(g, A, B, msgs, v, open_leg=pv, open_site=True)  # [s'v, sv, b, a]
    rho = np.einsum("ijba,klba->ikjl", Ru, Rv)  # [s'u, s'v, su, sv]
    du, dv = g.site_dims[u], g.site_dims[v]
    return rho.reshape(du * dv, du * dv, order="F")


def expect2(g, A, msgs, op2, B=None, edges=None):
    """<O_u O_v> on edges from the two-site RDM; ``op2`` is (du*dv)x(du*dv) with
    row index s'_u + du*s'_v and column index s_u + du*s_v."""
    B = A if B is None else B
    edges = range(g.ne) if edges is None else edges
    out = []
    for e in edges:
        rho = edge_rdm(g, A, B, msgs, e)
        out.append(np.sum(rho * op2) / np.trace(rho))
    return np.array(out)


# ----------------------------------------------------------------------------
# Rescaling / normalisation
# ----------------------------------------------------------------------------

def rescale_messages(g, msgs):
    """Per edge: normalise both messages, fix the sign, divide both by
    sqrt(<m_e, m_ebar>) (beliefpropagationcache.jl:121-139)."""
    msgs = [m.copy() for m in msgs]
    for e in range(g.ne):
        me = msgs[2 * e] / np.linalg.norm(msgs[2 * e])
        mer = msgs[2 * e + 1] / np.linalg.norm(msgs[2 * e + 1])
        n = np.sum(me * mer)
        if np.isreal(n):
            s = np.sign(np.real(n))
            me = me * s
            n = n * s
        sf = 1.0 / np.sqrt(n)
        msgs[2 * e] = sf * me
        msgs[2 * e + 1] = sf * mer
    return msgs


def rescale_partitions(g, A, msgs, B=None):
    """Scale each ket (and its bra) so every vertex scalar is 1
    (abstractbeliefpropagationcache.jl:349-379 restricted to the ket and bra
    vertices, normalize.jl:77): divide both tensors by their norms, compute the
    partition scalar z with the divided tensors, take r = z^(-1/2) (principal
    root) and s = sign(z) when z is real (for a complex z: an exactly zero
    imaginary part), else 1.  The reference weights the first vertex of the
    partition by s * (s * r) and the others by s * r; the partition lists the bra
    before the ket, because the form network is disjoint_union(operator, bra,
    ket) (formnetworks/bilinearformnetwork.jl:34-38) and partitions group the
    vertices in that order (abstractformnetwork.jl:89-91).  So the ket takes
    s * r and the bra conj(B_v) takes s * s * r.  With B = None the bra is
    conj(A) and only the kets are returned; with B the rescaled (A, B)."""
    out, outb = [], []
    for v in range(g.nv):
        a = A[v] / np.linalg.norm(A[v])
        b = a if B is None else B[v] / np.linalg.norm(B[v])
        z = np.trace(contract_partition(g, {v: a}, {v: b}, msgs, v, open_site=True))
        real = np.isrealobj(z) or np.imag(z) == 0
        sg = np.sign(np.real(z)) if real else 1.0
        r = z ** -0.5
        out.append(a * (sg * r))
        outb.append(b * np.conj(sg * sg * r))  # the contraction conjugates B
    return out if B is None else (out, outb)


def normalize_bp(g, A, msgs):
    """normalize(alg="bp") after the cache update: rescale messages, then
    partitions (normalize.jl:63-80).  Returns (new site tensors, messages)."""
    msgs = rescale_messages(g, msgs)
    return rescale_partitions(g, A, msgs), msgs


# ----------------------------------------------------------------------------
# tebd(H, psi; beta, dbeta, maxdim, cutoff) with a second-order Trotter product
# ----------------------------------------------------------------------------

# ITensors' "S=1/2" operators in the basis (up, down): S = sigma / 2
SPIN_HALF = {
    "Id": np.eye(2),
    "Sz": np.diag([0.5, -0.5]),
    "Sx": np.array([[0.0, 0.5], [0.5, 0.0]]),
    "Sy": np.array([[0.0, -0.5j], [0.5j, 0.0]]),
    "S+": np.array([[0.0, 1.0], [0.0, 0.0]]),
    "S-": np.array([[0.0, 0.0], [1.0, 0.0]]),
}


def ising_terms(g, J1=-1.0, h=0.0):
    """The Ising model of the reference's tests (test/utils.jl:174-192, J2 = 0):
    J1 Sz Sz on every edge in edge order, then h Sx on every vertex.  Terms are
    (coefficient, [(operator, vertex), ...])."""
    terms = [(J1, [("Sz", u), ("Sz", v)]) for (u, v) in g.edges]
    terms += [(h, [("Sx", v)]) for v in range(g.nv)]
    return terms


def group_terms(terms, g):
    """test/utils.jl:239-246: every term joins the group of the first edge (in
    edge order) holding all its sites; groups keep the order in which their
    edges first appear among the terms.  Returns [(edge, [terms])]."""
    groups = {}
    for t in terms:
        sites = {v for _, v in t[1]}
        e = next(k for k, (u, v) in enumerate(g.edges) if sites <= {u, v})
        groups.setdefault(e, []).append(t)
    return list(groups.items())


def group_matrix(g, e, terms):
    """Sum of the terms as a (du dv) x (du dv) matrix on edge e = (u, v), row
    s'_u + du s'_v (the gate convention of simple_update)."""
    u, v = g.edges[e]
    H = 0
    for c, ops in terms:
        Ou, Ov = np.eye(2), np.eye(2)
        for name, x in ops:  # a product as written: op1 op2 ... on each site
            if x == u:
                Ou = Ou @ SPIN_HALF[name]
            else:
                Ov = Ov @ SPIN_HALF[name]
        H = H + c * np.kron(Ov, Ou)  # row index s'_u + 2 s'_v
    return H


def trotter2_gates(g, groups, dbeta):
    """exp(-dbeta H) as a symmetric second-order Trotter product (Strang
    splitting, the published form of ITensors' Trotter{2}): exp(-dbeta/2 h_k)
    for the groups in order, then in reverse order.  Returns [(edge, gate)]."""
    half = []
    for e, terms in groups:
        h = group_matrix(g, e, terms)
        w, U = np.linalg.eigh(h)  # the terms are Hermitian
        half.append((e, (U * np.exp(-0.5 * dbeta * w)) @ U.conj().T))
    return half + half[::-1]


def tebd(g, A, groups, beta, dbeta, maxdim, cutoff):
    """tebd.jl:2-31 with ortho = false: int(beta / dbeta) (floor) steps, each
    applying the Trotter gates one by one with normalize = true and no
    environments (apply.jl:148-160 -> simple_update_bp without envs).
    Returns (graph with the new bond dimensions, tensors)."""
    g = Graph(g.nv, g.edges, g.site_dims, list(g.edge_dims), [list(l) for l in g.legs])
    A = [a.copy() for a in A]
    seq = trotter2_gates(g, groups, dbeta)
    for _ in range(int(beta // dbeta)):
        for e, gate in seq:
            u, v = g.edges[e]
            pu, pv = g.legs[u].index(e), g.legs[v].index(e)
            Au, Av, _, _ = simple_update(gate, A[u], A[v], pu, pv, {}, {}, maxdim=maxdim, cutoff=cutoff)
            A[u], A[v] = Au / np.linalg.norm(Au), Av / np.linalg.norm(Av)
            g.edge_dims[e] = Au.shape[pu + 1]
    return g, A


# ----------------------------------------------------------------------------
# Exact contraction (small networks only; used to pin BP on trees)
# ----------------------------------------------------------------------------

def exact_rdm1(g, A, v, B=None):
    """Exact rho_v[s', s] of <B|A> by contracting the whole network."""
    B = A if B is None else B
    ops = []
    nid = [0]

    def new():
        nid[0] += 1
        return nid[0]
    ket_link = {e: new() for e in range(g.ne)}
    bra_link = {e: new() for e in range(g.ne)}
    out = None
    for w in range(g.nv):
        s = new()
        if w == v:
            sp = new()
            out = [sp, s]
        else:
            sp = s
        ops += [A[w], [s] + [ket_link[e] for e in g.legs[w]]]
        ops += [np.conj(B[w]), [sp] + [bra_link[e] for e in g.legs[w]]]
    return np.einsum(*ops, out, optimize="greedy")


def exact_environment(g, A, v, B=None):
    """Exact environment of vertex v in <B|A> (environment(qf, [v]; alg =
    "exact"), environment.jl:6-20): every other ket and bra tensor contracted,
    v's links left open.  Index order: v's bra links, then its ket links (leg
    order); the site indices of v meet through the identity operator, which is
    left out."""
    B = A if B is None else B
    nid = [0]

    def new():
        nid[0] += 1
        return nid[0]
    ket_link = {e: new() for e in range(g.ne)}
    bra_link = {e: new() for e in range(g.ne)}
    ops = []
    for w in range(g.nv):
        if w == v:
            continue
        s = new()
        ops += [A[w], [s] + [ket_link[e] for e in g.legs[w]]]
        ops += [np.conj(B[w]), [s] + [bra_link[e] for e in g.legs[w]]]
    out = [bra_link[e] for e in g.legs[v]] + [ket_link[e] for e in g.legs[v]]
    return np.einsum(*ops, out, optimize="greedy")


def exact_scalar(g, A, B=None):
    B = A if B is None else B
    return np.trace(exact_rdm1(g, A, 0, B))


# ----------------------------------------------------------------------------
# Simple update (apply.jl) with ITensors' truncation rule
# ----------------------------------------------------------------------------

def truncate_spectrum(p, maxdim=None, cutoff=None, mindim=1):
    """ITensors/NDTensors truncation of a descending non-negative spectrum p
    (singular values squared): drop from the tail while beyond ``maxdim``,
    then while the discarded weight plus the next value stays within
    ``cutoff * sum(p)`` and more than ``mindim`` values remain.  Returns
    ``(kept, truncerr)`` with truncerr the discarded fraction of sum(p)."""
    p = np.asarray(p, dtype=float).copy()
    n = len(p)
    for i in range(n - 1, -1, -1):
        if p[i] >= 0:
            break
        p[i] = 0.0
    truncerr = 0.0
    if maxdim is not None:
        while n > maxdim:
            truncerr += p[n - 1]
            n -= 1
    scale = float(np.sum(p))
    if scale == 0.0:
        scale = 1.0
    if cutoff is not None:
        while n > mindim and truncerr + p[n - 1] <= cutoff * scale:
            truncerr += p[n - 1]
            n -= 1
    truncerr /= scale
    return max(n, 1), truncerr


def map_eigvals(f, m, cutoff):
    """f applied to the eigenvalues of the Hermitian matrix m (apply.jl:9-25);
    eigenvalues are sorted by descending magnitude and the tail whose summed
    magnitude is within ``cutoff`` of the total is dropped."""
    h = 0.5 * (m + m.conj().T)
    lam, U = np.linalg.eigh(h)
    order = np.argsort(-np.abs(lam), kind="stable")
    lam, U = lam[order], U[:, order]
    n = len(lam)
    tot = float(np.sum(np.abs(lam)))
    tot = tot if tot != 0 else 1.0
    disc = 0.0
    while n > 1 and disc + abs(lam[n - 1]) <= cutoff * tot:
        disc += abs(lam[n - 1])
        n -= 1
    lam, U = lam[:n], U[:, :n]
    return (U * f(lam)) @ U.conj().T


def simple_update(gate, Au, Av, pu, pv, envs_u, envs_v, maxdim=None, cutoff=None,
                  eig_cutoff=None):
    """simple_update_bp (apply.jl:33-95) for a two-site gate on edge (u, v).

    ``Au`` has the shared bond at leg position ``pu`` (1-based among the
    link legs, i.e. tensor axis pu+1), likewise ``Av``/``pv``.  ``envs_u`` maps
    tensor axis -> chi x chi environment message M[b, a] (may be empty).
    ``gate`` is (du*dv) x (du*dv), row s'_u + du*s'_v, column s_u + du*s_v.
    Returns (Au_new, Av_new, singular_values_kept, truncerr)."""
    eps = np.finfo(float).eps
    eig_cut = 10 * eps if eig_cutoff is None else eig_cutoff

    def absorb(T, envs, f):
        for ax, m in envs.items():
            # contract the ket link index of the env (a) with T's leg
            s = map_eigvals(f, m, eig_cut)
            T = np.moveaxis(np.tensordot(T, s, axes=([ax], [1])), -1, ax)
        return T

    def inv_sqrt(x):
        return 1.0 / np.sqrt(x)

    psu = absorb(Au, envs_u, np.sqrt)
    psv = absorb(Av, envs_v, np.sqrt)
    du, dv = Au.shape[0], Av.shape[0]
    au, av = pu + 1, pv + 1
    chi_e = Au.shape[au]
    # QR separating the other link legs (Q) from (site, bond) (R)
    def qr_split(T, ax):
        others = [i for i in range(1, T.ndim) if i != ax]
        Tp = np.transpose(T, others + [0, ax])
        ro = int(np.prod([T.shape[i] for i in others])) if others else 1
        mat = Tp.reshape(ro, T.shape[0] * T.shape[ax], order="F")
        Q, R = np.linalg.qr(mat, mode="reduced")
        return Q, R, others
    Qu, Ru, oth_u = qr_split(psu, au)
    Qv, Rv, oth_v = qr_split(psv, av)
    ru, rv = Ru.shape[0], Rv.shape[0]
    Ru3 = Ru.reshape(ru, du, chi_e, order="F")  # [r_u, s_u, l]
    Rv3 = Rv.reshape(rv, dv, chi_e, order="F")  # [r_v, s_v, l]
    theta = np.einsum("isl,jtl->istj", Ru3, Rv3)  # [r_u, s_u, s_v, r_v]
    G = gate.reshape(du, dv, du, dv, order="F")  # [s'_u, s'_v, s_u, s_v]
    theta = np.einsum("abst,istj->iabj", G, theta)
    mat = theta.reshape(ru * du, dv * rv, order="F")
    U, S, Vh = np.linalg.svd(mat, full_matrices=False)
    n, truncerr = truncate_spectrum(S ** 2, maxdim=maxdim, cutoff=cutoff)
    U, S, Vh = U[:, :n], S[:n], Vh[:n, :]
    sq = np.sqrt(S)
    L = (U * sq).reshape(ru, du, n, order="F")  # [r_u, s_u, k]
    R = (sq[:, None] * Vh).reshape(n, dv, rv, order="F")  # [k, s_v, r_v]

    def rebuild(Q, others, shape, core, ax, envs):
        # Q: [prod(other link dims), r] (column-major); core: [r, s, k].
        oshape = [shape[i] for i in others]
        Qt = Q.reshape(oshape + [Q.shape[1]], order="F")
        T = np.tensordot(Qt, core, axes=([len(oshape)], [0]))  # others..., s, k
        names = list(others) + [0, ax]
        T = np.transpose(T, [names.index(i) for i in range(len(shape))])
        for a_, m in envs.items():
            s_ = map_eigvals(inv_sqrt, m, eig_cut)
            T = np.moveaxis(np.tensordot(T, s_.conj(), axes=([a_], [0])), -1, a_)
        return T
    Au_new = rebuild(Qu, oth_u, Au.shape, L, au, envs_u)
    Rv_core = np.transpose(R, (2, 1, 0))  # [r_v, s_v, k]
    Av_new = rebuild(Qv, oth_v, Av.shape, Rv_core, av, envs_v)
    return Au_new, Av_new, S, truncerr


# ----------------------------------------------------------------------------
# Operators (spin-1/2 and Pauli conventions)
# ----------------------------------------------------------------------------

SZ = np.array([[0.5, 0.0], [0.0, -0.5]])
SX = np.array([[0.0, 0.5], [0.5, 0.0]])
PZ = np.array([[1.0, 0.0], [0.0, -1.0]])
PX = np.array([[0.0, 1.0], [1.0, 0.0]])
PY = np.array([[0.0, -1j], [1j, 0.0]])
ID2 = np.eye(2)


def kron2(a, b):
    """Two-site operator with row index s'_u + du*s'_v: O = b (x) a in numpy's
    kron (first-site index fastest)."""
    return np.kron(b, a)


# ----------------------------------------------------------------------------
# Rounding model of the BF16 tensor-core message update
# ----------------------------------------------------------------------------

def bf16_round(x):
    """Round float64 (or float32) values to the nearest bfloat16 (8 significant
    bits, ties to even), returned as float64.  Exact for the normal range."""
    x = np.asarray(x, dtype=np.float64)
    m, e = np.frexp(x)  # x = m 2^e, 0.5 <= |m| < 1
    return np.ldexp(np.rint(m * 256.0) / 256.0, e)


def tc_bf16_messages(g, A, msgs, v):
    """Outgoing messages of vertex v as the BF16 tensor-core sweep computes
    them (d = 2, degree <= 4, chi <= 8; real tensors, bra = ket): the same
    contraction as :func:`updated_message`, evaluated through the kernel's two
    pairs of two-leg environments with BF16 roundings at the kernel's points --
    site tensor rounded to BF16; incoming messages stored as FP32; Kronecker
    products of two messages formed in FP32 and rounded to BF16; the
    half-contracted tensors T12 / T34 rounded to BF16 before the second
    product.  Sums are taken in float64 (the kernel accumulates in FP32), so
    the result differs from the kernel's by FP32 accumulation error and the
    rare BF16 rounding it flips.  Returns {directed edge: normalised chi x chi
    message}."""
    k = len(g.legs[v])
    assert k <= 4 and g.site_dims[v] == 2
    shape = list(A[v].shape) + [1] * (4 - k)
    Z = bf16_round(np.asarray(A[v], dtype=np.float64).reshape(shape, order="F"))
    M = []
    for p in range(4):
        if p < k:
            e = g.legs[v][p]
            M.append(np.asarray(msgs[g.directed(e, g.other(v, e))], dtype=np.float32))
        else:
            M.append(np.ones((1, 1), dtype=np.float32))

    def kron(Ma, Mb):  # K[b_a, b_b, a_a, a_b] = bf16(fp32(Ma[b_a, a_a] * Mb[b_b, a_b]))
        prod = Ma[:, None, :, None] * Mb[None, :, None, :]  # float32 products
        return bf16_round(prod.astype(np.float32))

    K12, K34 = kron(M[0], M[1]), kron(M[2], M[3])
    T12 = bf16_round(np.einsum("sxyzw,bcxy->szwbc", Z, K12))
    T34 = bf16_round(np.einsum("sxyzw,uvzw->sxyuv", Z, K34))
    G34 = np.einsum("szwbc,sbcuv->zwuv", T12, Z)  # [a3, a4, b3, b4]
    G12 = np.einsum("sxyuv,sbcuv->xybc", T34, Z)  # [a1, a2, b1, b2]
    M64 = [m.astype(np.float64) for m in M]
    outs = [np.einsum("xybc,cy->bx", G12, M64[1]),   # leg 0: [b1, a1]
            np.einsum("xybc,bx->cy", G12, M64[0]),   # leg 1: [b2, a2]
            np.einsum("zwuv,vw->uz", G34, M64[3]),   # leg 2: [b3, a3]
            np.einsum("zwuv,uz->vw", G34, M64[2])]   # leg 3: [b4, a4]
    res = {}
    for p in range(k):
        m = outs[p]
        nrm = np.linalg.norm(m)
        res[g.directed(g.legs[v][p], v)] = m / nrm if nrm != 0 else m
    return res
