"""Multi-site partitions (partitioned_vertices, test/test_expect.jl:28-39):
BP over partitions = BP on the coarse network whose vertices are the
partitions, with fused site and crossing-link indices.

CPU tests pin the coarse-graining bookkeeping (bit-exact) and its semantics
with the oracle: BP over column partitions of a grid is exact (the partition
graph is a chain), as the reference's test asserts.  GPU tests run the same
through the library (1e-10 relative against exact contraction; 1e-10 against
the oracle's BP on the coarse network for a loopy partition graph)."""
import numpy as np
import pytest

import bp_oracle as O
import gbtn
from gbtn.partition import CoarseGraining


def grid(L, chi, seed):
    g = O.square_lattice(L, L, chi=chi)
    A = O.random_network(g, seed)
    tn = gbtn.TensorNetwork(g.nv, g.edges, g.site_dims, g.edge_dims, [a.copy() for a in A])
    return tn, g, A


def columns(L):
    # vertex i + L*j is site (i+1, j+1); group by the first coordinate, as the reference's test does
    return [[i + L * j for j in range(L)] for i in range(L)]


def exact_sz_and_norm(g, A):
    """<Sz_v> and <psi|psi> from the state vector (the ket layer contracted once)."""
    ops, lid = [], {e: 20 + e for e in range(g.ne)}
    for v in range(g.nv):
        ops += [A[v], [v] + [lid[e] for e in g.legs[v]]]
    psi = np.einsum(*ops, list(range(g.nv)), optimize=True)
    nrm = float(np.sum(psi * psi))
    sz = []
    for v in range(g.nv):
        p2 = np.moveaxis(psi, v, 0).reshape(2, -1)
        rho = p2 @ p2.T
        sz.append(np.sum(rho * O.SZ) / np.trace(rho))
    return np.array(sz), nrm


def as_graph(tn):
    return O.Graph(tn.nv, tn.edges, tn.site_dims, list(tn.edge_dims), [list(l) for l in tn.legs])


def test_singleton_partitions_reproduce_the_network():
    tn, g, A = grid(3, 2, 1)
    cg = CoarseGraining(tn, [[v] for v in range(tn.nv)])
    assert cg.coarse.edges == tn.edges
    assert cg.coarse.edge_dims == tn.edge_dims and cg.coarse.site_dims == tn.site_dims
    assert cg.coarse.legs == tn.legs
    for a, b in zip(cg.coarse.tensors, tn.tensors):
        np.testing.assert_array_equal(a, b)


def test_column_partitions_structure():
    tn, g, A = grid(3, 2, 2)
    cg = CoarseGraining(tn, columns(3))
    assert cg.coarse.nv == 3 and cg.coarse.edges == [(0, 1), (1, 2)]
    assert cg.coarse.site_dims == [8, 8, 8] and cg.coarse.edge_dims == [8, 8]
    assert [t.shape for t in cg.coarse.tensors] == [(8, 8), (8, 8, 8), (8, 8)]
    # the coarse network contracts to the same <psi|psi>
    gc = as_graph(cg.coarse)
    assert O.exact_scalar(gc, cg.coarse.tensors) == pytest.approx(exact_sz_and_norm(g, A)[1], rel=1e-12)
    with pytest.raises(ValueError):
        CoarseGraining(tn, [[0, 1], [2]])


@pytest.mark.parametrize("L", [2, 3])
def test_column_partitioned_bp_is_exact_oracle(L):
    tn, g, A = grid(L, 2, 10 + L)
    cg = CoarseGraining(tn, columns(L))
    gc = as_graph(cg.coarse)
    m, _, _ = O.bp_update(gc, cg.coarse.tensors, O.identity_messages(gc), maxiter=20, schedule="parallel")
    rdms = cg.site_rdms([O.vertex_rdm(gc, cg.coarse.tensors, cg.coarse.tensors, m, i) for i in range(gc.nv)])
    sz = [np.sum(r * O.SZ) / np.trace(r) for r in rdms]
    exact, nrm = exact_sz_and_norm(g, A)
    np.testing.assert_allclose(sz, exact, rtol=1e-10, atol=1e-12)
    # and the BP norm of the partitioned network is the exact norm
    assert np.exp(O.logscalar(gc, cg.coarse.tensors, cg.coarse.tensors, m)) == pytest.approx(nrm, rel=1e-10)


@pytest.mark.gpu
@pytest.mark.parametrize("L", [2, 3, 4])
def test_column_partitioned_bp_is_exact_gpu(lib_built, L):
    # L = 4: fused site dimension 16 and crossing bonds of dimension 16 run the
    # global-memory path (test/test_expect.jl:28-39 uses columns of the grid)
    tn, g, A = grid(L, 2, 10 + L)
    pc = gbtn.partitioned_cache(tn, columns(L)).update(maxiter=20, schedule="parallel")
    exact, nrm = exact_sz_and_norm(g, A)
    np.testing.assert_allclose(pc.expect(O.SZ), exact, rtol=1e-10, atol=1e-12)
    assert np.exp(pc.logscalar()) == pytest.approx(nrm, rel=1e-10)
    pc.close()


@pytest.mark.gpu
def test_domino_partitions_on_a_loopy_grid_gpu(lib_built):
    # 4x4 grid in 1x2 dominoes: a loopy partition graph, fused bonds of dimension 2 and 4
    L = 4
    tn, g, A = grid(L, 2, 31)
    parts = [[i + L * j, i + 1 + L * j] for j in range(L) for i in range(0, L, 2)]
    pc = gbtn.partitioned_cache(tn, parts).update(maxiter=300, schedule="parallel")
    cg = pc.cg
    gc = as_graph(cg.coarse)
    m, _, _ = O.bp_update(gc, cg.coarse.tensors, O.identity_messages(gc), maxiter=300, schedule="parallel")
    rdms = cg.site_rdms([O.vertex_rdm(gc, cg.coarse.tensors, cg.coarse.tensors, m, i) for i in range(gc.nv)])
    ref = [np.sum(r * O.SZ) / np.trace(r) for r in rdms]
    np.testing.assert_allclose(pc.expect(O.SZ), ref, rtol=1e-10, atol=1e-12)
    pc.close()


@pytest.mark.gpu
def test_square_block_partitions_on_a_loopy_grid_gpu(lib_built):
    # 6x6 grid in 2x2 blocks: a loopy 3x3 partition graph with fused site
    # dimension 16 and crossing bonds of dimension 4, against the oracle's BP
    # on the same coarse network
    L = 6
    tn, g, A = grid(L, 2, 47)
    parts = [[i + L * j, i + 1 + L * j, i + L * (j + 1), i + 1 + L * (j + 1)]
             for j in range(0, L, 2) for i in range(0, L, 2)]
    pc = gbtn.partitioned_cache(tn, parts).update(maxiter=200, schedule="parallel")
    cg = pc.cg
    assert set(cg.coarse.site_dims) == {16} and set(cg.coarse.edge_dims) == {4}
    gc = as_graph(cg.coarse)
    m, _, _ = O.bp_update(gc, cg.coarse.tensors, O.identity_messages(gc), maxiter=200, schedule="parallel")
    rdms = cg.site_rdms([O.vertex_rdm(gc, cg.coarse.tensors, cg.coarse.tensors, m, i) for i in range(gc.nv)])
    ref = [np.sum(r * O.SZ) / np.trace(r) for r in rdms]
    np.testing.assert_allclose(pc.expect(O.SZ), ref, rtol=1e-10, atol=1e-12)
    assert pc.logscalar() == pytest.approx(float(np.real(O.logscalar(gc, cg.coarse.tensors, cg.coarse.tensors, m))),
                                           rel=1e-10)
    pc.close()
