"""Generate the golden fixtures in this folder from the FP64 oracle.

The reference (Julia) cannot run in this environment and publishes no numeric
vectors, so the fixtures are produced by the oracle, whose correctness is
pinned separately by the reference's own known-answer tests (BP exact on
trees against exact contraction, fixed-point residual, unit scalars after
normalisation; see tests/test_oracle.py).  Each case stores its inputs' seeds
and shapes, the messages after the stated sweeps, <Sz> per site and the BP
log-norm.  Regenerate with ``python tests/golden/make_golden.py``.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent / "oracle"))
import bp_oracle as O  # noqa: E402


def case_c1():
    """4x4 open PEPS, d=2, chi=2, FP64 N(0,1) seed 1, all-ones messages, 20
    sequential forest-cover sweeps."""
    g = O.square_lattice(4, 4, chi=2)
    A = O.random_network(g, 1)
    seq = O.default_edge_sequence(g)
    m, it, md = O.bp_update(g, A, O.ones_messages(g), maxiter=20, schedule="sequential", edge_sequence=seq)
    return dict(Lx=4, Ly=4, chi=2, seed=1, seq=np.array(seq), msgs=O.flatten_messages(g, m),
                sz=O.expect1(g, A, m, O.SZ), logscalar=O.logscalar(g, A, A, m))


def case_grid3():
    """3x3, chi=2, seed 1234, identity messages, update(maxiter=25, tol=eps)."""
    g = O.square_lattice(3, 3, chi=2)
    A = O.random_network(g, 1234)
    m, it, md = O.bp_update(g, A, O.identity_messages(g), maxiter=25, tol=np.finfo(float).eps)
    return dict(Lx=3, Ly=3, chi=2, seed=1234, iters=it, mean_diff=md, msgs=O.flatten_messages(g, m),
                sz=O.expect1(g, A, m, O.SZ), logscalar=O.logscalar(g, A, A, m))


def case_uneven():
    """5x4 grid with bond dims drawn from {2..5} (seed 11), tensors seed 7,
    identity messages, 60 parallel (Jacobi) sweeps; also <SzSz> on all edges."""
    rng = np.random.default_rng(11)
    g0 = O.square_lattice(5, 4, chi=2)
    dims = [int(x) for x in rng.integers(2, 6, size=g0.ne)]
    g = O.square_lattice(5, 4, edge_dims=dims)
    A = O.random_network(g, 7)
    m, it, md = O.bp_update(g, A, O.identity_messages(g), maxiter=60, schedule="parallel", tol=1e-14)
    szsz = O.expect2(g, A, m, O.kron2(O.SZ, O.SZ))
    return dict(Lx=5, Ly=4, dims=np.array(dims), seed=7, iters=it, msgs=O.flatten_messages(g, m),
                sz=O.expect1(g, A, m, O.SZ), szsz=szsz, logscalar=O.logscalar(g, A, A, m))


def case_tree():
    """Random tree on 9 vertices (seed 3), chi=3: BP after one forest-cover
    sweep equals exact contraction (the pin)."""
    g = O.random_tree(9, seed=3, chi=3)
    A = O.random_network(g, 5)
    m, _, _ = O.bp_update(g, A, O.identity_messages(g), maxiter=1)
    exact = []
    for v in range(g.nv):
        r = O.exact_rdm1(g, A, v)
        exact.append(np.sum(r * O.SZ) / np.trace(r))
    return dict(n=9, tree_seed=3, chi=3, seed=5, edges=np.array(g.edges), sz=O.expect1(g, A, m, O.SZ),
                sz_exact=np.array(exact), logscalar=O.logscalar(g, A, A, m),
                log_exact=np.log(O.exact_scalar(g, A)))


def main():
    cases = {"c1": case_c1(), "grid3": case_grid3(), "uneven": case_uneven(), "tree": case_tree()}
    flat = {f"{c}__{k}": np.asarray(v) for c, d in cases.items() for k, v in d.items()}
    np.savez_compressed(HERE / "bp_small.npz", **flat)
    print("wrote", HERE / "bp_small.npz", {k: v.shape for k, v in flat.items()})


if __name__ == "__main__":
    main()
