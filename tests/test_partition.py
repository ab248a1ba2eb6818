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


def test_fused_operator_is_the_sum_over_sites():
    """Tr(rho_fused O_fused) = sum_v tr(rho_v op) for the partial traces of the
    fused RDM (CPU: the fusion order, first site fastest)."""
    tn, g, A = grid(4, 2, 3)
    cg = CoarseGraining(tn, [[0, 1, 4, 5], [2, 3, 6, 7], [8, 9, 12, 13], [10, 11, 14, 15]])
    rng = np.random.default_rng(1)
    X = rng.standard_normal((16, 16))
    rho = X @ X.T
    op = np.array([[0.3, 0.2], [0.2, -0.5]])
    fused = cg.fused_operator(op)
    parts_rho = cg.site_rdms([rho] * 4)
    assert np.sum(rho * fused) == pytest.approx(sum(np.sum(parts_rho[v] * op) for v in (0, 1, 4, 5)), rel=1e-12)


@pytest.mark.gpu
def test_partition_gradients_against_finite_differences(lib_built):
    """Gradients on 1x2 domino partitions of a 4x4 grid: the coarse plan's
    adjoints pulled back through the partition contraction, against central
    differences of the oracle's BP on the coarse network (h = 1e-5, 1e-6)."""
    L = 4
    tn, g, A = grid(L, 2, 61)
    A = [a / np.linalg.norm(a) for a in A]
    tn.tensors = [a.copy() for a in A]
    parts = [[i + L * j, i + 1 + L * j] for j in range(L) for i in range(0, L, 2)]
    pc = gbtn.partitioned_cache(tn, parts).update(maxiter=400, schedule="parallel")
    val, G = pc.logscalar_grad(tol=1e-14)
    sval, GS = pc.expect_sum_grad(O.SZ, tol=1e-14)

    def coarse_oracle(ts):
        t = gbtn.TensorNetwork(g.nv, g.edges, g.site_dims, g.edge_dims, ts)
        cg = CoarseGraining(t, parts)
        gc = as_graph(cg.coarse)
        m, _, _ = O.bp_update(gc, cg.coarse.tensors, O.identity_messages(gc), maxiter=400, schedule="parallel")
        return cg, gc, m

    def f_log(ts):
        cg, gc, m = coarse_oracle(ts)
        return float(np.real(O.logscalar(gc, cg.coarse.tensors, cg.coarse.tensors, m)))

    def f_sz(ts):
        cg, gc, m = coarse_oracle(ts)
        rdms = cg.site_rdms([O.vertex_rdm(gc, cg.coarse.tensors, cg.coarse.tensors, m, i) for i in range(gc.nv)])
        return float(sum(np.sum(r * O.SZ) / np.trace(r) for r in rdms))

    assert val == pytest.approx(f_log(A), rel=1e-10)
    assert sval == pytest.approx(f_sz(A), rel=1e-9, abs=1e-12)
    rng = np.random.default_rng(5)
    D = [rng.standard_normal(a.shape) for a in A]
    nrm = np.sqrt(sum(np.sum(d * d) for d in D))
    D = [d / nrm for d in D]
    h = 1e-5
    for f, grad in ((f_log, G), (f_sz, GS)):
        fd = (f([a + h * d for a, d in zip(A, D)]) - f([a - h * d for a, d in zip(A, D)])) / (2 * h)
        an = sum(float(np.sum(x * d)) for x, d in zip(grad, D))
        assert an == pytest.approx(fd, rel=1e-6, abs=1e-10)
    pc.close()


def test_partition_contraction_adjoint_cpu():
    """tensor_cotangents is the adjoint of the partition contraction: for a
    random coarse cotangent W, <W, dT(A)[D]> (central differences of the
    contraction) equals <tensor_cotangents(W), D>, on 2x2 blocks with internal
    and crossing edges."""
    L = 4
    tn, g, A = grid(L, 2, 17)
    parts = [[i + L * j, i + 1 + L * j, i + L * (j + 1), i + 1 + L * (j + 1)] for j in (0, 2) for i in (0, 2)]
    cg = CoarseGraining(tn, parts)
    rng = np.random.default_rng(3)
    W = [rng.standard_normal(t.shape) for t in cg.coarse.tensors]
    G = cg.tensor_cotangents(W)
    assert [x.shape for x in G] == [a.shape for a in A]
    D = [rng.standard_normal(a.shape) for a in A]

    def pairing(ts):
        c = CoarseGraining(gbtn.TensorNetwork(g.nv, g.edges, g.site_dims, g.edge_dims, ts), parts)
        return sum(float(np.sum(w * t)) for w, t in zip(W, c.coarse.tensors))

    h = 1e-3
    fd = (pairing([a + h * d for a, d in zip(A, D)]) - pairing([a - h * d for a, d in zip(A, D)])) / (2 * h)
    an = sum(float(np.sum(x * d)) for x, d in zip(G, D))
    # each coarse tensor is multilinear (degree 4) in its sites, so the central
    # difference carries an O(h^2) term: ~1e-6 relative at h = 1e-3
    assert an == pytest.approx(fd, rel=1e-5)
