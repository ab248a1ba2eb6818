"""FP64 autograd restatement of the BP energy and its gradient.

TEST INFRASTRUCTURE ONLY (the checker for the library's hand-written
adjoints; only tests/ import it).  The reference has no automatic
differentiation code and cannot run here, so the "gradient through the
reference" is restated as reverse-mode autograd (PyTorch, float64, CPU)
through the same algorithm the oracle follows:

* parallel (Jacobi) message sweeps from identity messages, each message
  contracted and divided by its Frobenius norm
  (src/caches/abstractbeliefpropagationcache.jl:225-239, 294-308);
* the BP energy sum_e <h_e> with <h_e> = tr(rho_e h_e) / tr(rho_e) from the
  two-site BP reduced density matrix (test/test_belief_propagation.jl:64-91).

With enough sweeps to converge, the unrolled gradient equals the gradient
through the fixed point, which the library computes by implicit
differentiation.
"""
from __future__ import annotations

import numpy as np
import torch

import bp_oracle as O

# Heisenberg (J=1, Pauli): XX + YY + ZZ = X(x)X - J(x)J + Z(x)Z with J = [[0,-1],[1,0]]
PX = np.array([[0.0, 1.0], [1.0, 0.0]])
PJ = np.array([[0.0, -1.0], [1.0, 0.0]])
PZ = np.array([[1.0, 0.0], [0.0, -1.0]])
HEISENBERG_TERMS = [(1.0, PX, PX), (-1.0, PJ, PJ), (1.0, PZ, PZ)]


def heisenberg_matrix():
    """4 x 4 two-site operator, row s'_u + 2 s'_v, column s_u + 2 s_v."""
    return sum(c * np.kron(b, a) for c, a, b in HEISENBERG_TERMS)


def _msg(g, A, msgs, de):
    v = g.dsrc(de)
    e = de // 2
    p = g.legs[v].index(e)
    a = A[v]
    k = a.dim() - 1
    ops = [a, [0] + [1 + q for q in range(k)], a, [0] + [1 + k + q for q in range(k)]]
    for q, f in enumerate(g.legs[v]):
        if q == p:
            continue
        ops += [msgs[g.directed(f, g.other(v, f))], [1 + k + q, 1 + q]]
    m = torch.einsum(*ops, [1 + k + p, 1 + p])
    return m / torch.linalg.norm(m)


def sweeps(g, A, T):
    msgs = [torch.eye(g.edge_dims[de // 2], dtype=torch.float64) for de in range(2 * g.ne)]
    for _ in range(T):
        msgs = [_msg(g, A, msgs, de) for de in range(2 * g.ne)]
    return msgs


def energy(g, A, msgs, h=None):
    """sum_e tr(rho_e h) / tr(rho_e) with the BP two-site RDM of every edge."""
    h = torch.tensor(heisenberg_matrix() if h is None else h, dtype=torch.float64)
    tot = 0.0
    for e, (u, v) in enumerate(g.edges):
        halves = []
        for x in (u, v):
            a = A[x]
            k = a.dim() - 1
            p = g.legs[x].index(e)
            ops = [a, [0] + [2 + q for q in range(k)], a, [1] + [2 + k + q for q in range(k)]]
            for q, f in enumerate(g.legs[x]):
                if q == p:
                    continue
                ops += [msgs[g.directed(f, g.other(x, f))], [2 + k + q, 2 + q]]
            halves.append(torch.einsum(*ops, [1, 0, 2 + k + p, 2 + p]))  # [s', s, b, a]
        Ru, Rv = halves
        # [s'_v, s'_u, s_v, s_u] -> row s'_u + 2 s'_v, column s_u + 2 s_v
        rho = torch.einsum("ijba,klba->kilj", Ru, Rv).reshape(4, 4)
        tot = tot + torch.sum(rho * h) / torch.trace(rho)
    return tot


def energy_and_grad(g, A_np, T):
    """(E, [dE/dA_v]) unrolled through T parallel sweeps from identity messages."""
    A = [torch.tensor(a, dtype=torch.float64, requires_grad=True) for a in A_np]
    E = energy(g, A, sweeps(g, A, T))
    E.backward()
    return float(E), [a.grad.numpy() for a in A]


def energy_np(g, A_np, T):
    with torch.no_grad():
        A = [torch.tensor(a, dtype=torch.float64) for a in A_np]
        return float(energy(g, A, sweeps(g, A, T)))


def check_against_oracle(g, A_np, T):
    """The torch restatement agrees with bp_oracle (used by the CPU tests)."""
    with torch.no_grad():
        A = [torch.tensor(a, dtype=torch.float64) for a in A_np]
        m = [x.numpy() for x in sweeps(g, A, T)]
    m_ref, _, _ = O.bp_update(g, A_np, O.identity_messages(g), maxiter=T, schedule="parallel")
    return max(np.max(np.abs(a - b)) for a, b in zip(m, m_ref))
