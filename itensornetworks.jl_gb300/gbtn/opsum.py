"""Operator sums and imaginary-time TEBD with the reference's signature.

``tebd(H, psi, beta=, dbeta=, maxdim=, cutoff=, print_frequency=, ortho=)``
mirrors src/tebd.jl:2-31: the gates of exp(-dbeta H) as a second-order
Trotter product (ITensors' ``Trotter{2}``: exp(-dbeta/2 h_k) for the terms in
order, then in reverse order), applied ``int(beta // dbeta)`` times by the
GPU simple update with ``normalize = true`` and no environments, which is what
``apply(gates, psi; cutoff, maxdim, normalize = true)`` does for two-site
gates (src/apply.jl:148-160).

``OpSum`` holds ITensors-style terms on spin-1/2 sites ("S=1/2" operators
Sz, Sx, Sy, S+, S-, Id, in the basis (up, down)):
``H += (coefficient, "Sz", u, "Sz", v)`` or ``H += (coefficient, "Sx", v)``.
``group_terms(H, tn)`` merges the terms edge by edge like the reference's
test utility (test/utils.jl:239-246): a term joins the first edge, in edge
order, that holds all its sites.  Ungrouped terms become one gate each, a
one-site term acting on the first edge that holds its site.
"""
from __future__ import annotations

import numpy as np

from . import _lib
from .network import TensorNetwork

SPIN_HALF_OPS = {
    "Id": np.eye(2),
    "Sz": np.diag([0.5, -0.5]),
    "Sx": np.array([[0.0, 0.5], [0.5, 0.0]]),
    "Sy": np.array([[0.0, -0.5j], [0.5j, 0.0]]),
    "S+": np.array([[0.0, 1.0], [0.0, 0.0]]),
    "S-": np.array([[0.0, 0.0], [1.0, 0.0]]),
}


def named_operator(name, tn: TensorNetwork):
    """The matrix O[s', s] of a named S=1/2 operator for expect(psi, "Sz")
    (expect.jl:21-41): every site of ``tn`` must have dimension 2, and the
    operator must be real (the library reports the real part of <O> for a real
    O; "Sy" is imaginary)."""
    if name not in SPIN_HALF_OPS:
        raise ValueError(f"unknown operator {name!r} (S=1/2 sites: {sorted(SPIN_HALF_OPS)})")
    if any(d != 2 for d in tn.site_dims):
        raise ValueError(f"operator {name!r} acts on spin-1/2 sites; this network has site dimensions "
                         f"{sorted(set(tn.site_dims))}")
    op = SPIN_HALF_OPS[name]
    if np.iscomplexobj(op):
        raise ValueError(f"operator {name!r} is complex: pass its matrix to a complex-aware contraction instead")
    return np.asarray(op, dtype=float)


class OpSum:
    """A sum of products of named one-site operators.  Each term is stored as
    (coefficient, ((name, vertex), ...)); ``groups`` (set by group_terms) is a
    list of (edge, [terms]) or None."""

    def __init__(self, terms=None):
        self.terms = [self._parse(t) for t in (terms or [])]
        self.groups = None

    @staticmethod
    def _parse(t):
        t = tuple(t)
        if not t:
            raise ValueError("empty term")
        c, rest = (t[0], t[1:]) if not isinstance(t[0], str) else (1.0, t)
        if len(rest) == 0 or len(rest) % 2:
            raise ValueError(f"a term is (coefficient, name, site, name, site, ...), got {t!r}")
        ops = tuple((str(rest[i]), int(rest[i + 1])) for i in range(0, len(rest), 2))
        for name, _ in ops:
            if name not in SPIN_HALF_OPS:
                raise ValueError(f"unknown operator {name!r} (S=1/2 sites: {sorted(SPIN_HALF_OPS)})")
        return (complex(c) if np.iscomplexobj(c) else float(c), ops)

    def __iadd__(self, t):
        self.terms.append(self._parse(t))
        self.groups = None
        return self

    def __len__(self):
        return len(self.terms)


def _first_edge(tn: TensorNetwork, sites):
    for e, (u, v) in enumerate(tn.edges):
        if sites <= {u, v}:
            return e
    raise ValueError(f"no edge holds the sites {sorted(sites)}: terms act on one site or on the two ends of an edge")


def group_terms(H: OpSum, tn: TensorNetwork) -> OpSum:
    """The terms of H merged per edge (test/utils.jl:239-246): each term joins
    the group of the first edge in edge order holding all its sites; groups
    keep the order in which their edges first appear among the terms."""
    groups = {}
    for t in H.terms:
        groups.setdefault(_first_edge(tn, {v for _, v in t[1]}), []).append(t)
    out = OpSum()
    out.terms = list(H.terms)
    out.groups = list(groups.items())
    return out


def _edge_matrix(tn: TensorNetwork, e, terms):
    """Sum of the terms on edge e = (u, v) as a 4 x 4 matrix in the gate
    convention of the simple update (row s'_u + 2 s'_v); a product of operators
    on one site is taken as written (op1 op2 ...)."""
    u, v = tn.edges[e]
    if tn.site_dims[u] != 2 or tn.site_dims[v] != 2:
        raise ValueError("OpSum operators act on spin-1/2 sites (site dimension 2)")
    h = np.zeros((4, 4), dtype=complex)
    for c, ops in terms:
        ou, ov = np.eye(2, dtype=complex), np.eye(2, dtype=complex)
        for name, x in ops:
            if x == u:
                ou = ou @ SPIN_HALF_OPS[name]
            else:
                ov = ov @ SPIN_HALF_OPS[name]
        h += c * np.kron(ov, ou)
    return h.real.copy() if not np.any(h.imag) else h


def _expm(a):
    from scipy.linalg import expm
    return expm(a)


def trotter2_gates(H: OpSum, tn: TensorNetwork, dbeta):
    """exp(-dbeta H; alg = Trotter{2}()) as [(edge, gate)]: exp(-dbeta/2 h_k)
    over the groups (or single terms) in order, then in reverse order."""
    groups = H.groups if H.groups is not None else [
        (_first_edge(tn, {v for _, v in t[1]}), [t]) for t in H.terms]
    half = [(e, _expm(-0.5 * dbeta * _edge_matrix(tn, e, terms))) for e, terms in groups]
    return half + half[::-1]


def tebd_opsum(H: OpSum, psi: TensorNetwork, *, beta, dbeta, maxdim, cutoff, print_frequency=10, ortho=False,
               ctx=None):
    """tebd(H, psi; beta, dbeta, maxdim, cutoff, print_frequency, ortho)
    (src/tebd.jl:2-31).  Returns the evolved network."""
    from .su import SimpleUpdateState
    if ortho:
        raise _lib.Unsupported(3, "tebd(ortho=true) orthogonalises a tree tensor network (tree_orthogonalize), "
                                  "which this library does not implement")
    seq = trotter2_gates(H, psi, dbeta)
    cplx = psi.is_complex or any(np.iscomplexobj(gt) for _, gt in seq)
    chi_max = max([int(maxdim)] + list(psi.edge_dims))
    st = SimpleUpdateState(psi, chi_max, ctx=ctx, complex_values=cplx)
    edges = [e for e, _ in seq]
    gates = [gt for _, gt in seq]
    nsteps = int(beta // dbeta)
    for step in range(1, nsteps + 1):
        if print_frequency and step % print_frequency == 0:
            print(f"(step, (step - 1) * dbeta, beta) = ({step}, {(step - 1) * dbeta}, {beta})")
        st.apply(gates, edges, maxdim=maxdim, cutoff=cutoff, normalize=True)
    out = st.network()
    st.close()
    return out
