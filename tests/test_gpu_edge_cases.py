"""Degenerate and limit shapes against the FP64 oracle: a graph without edges
(BP is a no-op: maxiter iterations, mean diff NaN as the reference's 0/0,
scalars and <Sz> from the vertices alone), an isolated vertex beside a
lattice, bond dimension 1 (product states: BP is exact), site dimension 1
and mixed site dimensions, a degree-8 vertex (the kernels' maximum; BP exact
on the star tree), ragged batches (1-, 2- and many-vertex networks side by
side, per-network convergence), and the shapes the library refuses
(degree 9, a vertex tensor beyond the shared-memory kernels) reported as
GBTN_ERR_UNSUPPORTED.  Messages to 1e-10, observables to 1e-10 relative."""
import numpy as np
import pytest

import bp_oracle as O
import gbtn

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib(lib_built):
    yield


def both(nv, edges, site, chi, seed, legs=None):
    g = O.Graph(nv, edges, site, chi, legs=legs)
    A = O.random_network(g, seed)
    tn = gbtn.TensorNetwork(nv, edges, site, chi, [a.copy() for a in A], legs=[list(l) for l in g.legs])
    return tn, g, A


def exact(g, A):
    """(<Sz_v> for every vertex, <psi|psi>) from the full state vector (small networks)."""
    ops = []
    for v in range(g.nv):
        ops += [A[v], [20 + v] + list(g.legs[v])]
    psi = np.einsum(*ops, [20 + v for v in range(g.nv)], optimize=True)
    p = np.abs(psi) ** 2
    norm = p.sum()
    sz = []
    for v in range(g.nv):
        pv = p.sum(axis=tuple(a for a in range(g.nv) if a != v))
        sz.append(float(np.dot(pv, np.diag(O.SZ))) / norm)
    return np.array(sz), norm


def sz_ops(g):
    return [np.diag(np.linspace(0.5, -0.5, d)) if d > 1 else np.ones((1, 1)) for d in g.site_dims]


def check_messages(bpc, g, ref, tol=1e-10):
    got = bpc.messages()
    assert len(got) == 2 * g.ne
    for de in range(2 * g.ne):
        np.testing.assert_allclose(got[de], ref[de], rtol=0, atol=tol)


@pytest.mark.parametrize("precision", ["f64", "f32", "mixed", "bf16"])
def test_graph_without_edges(precision):
    tn, g, A = both(3, [], [2, 3, 1], [], 4)
    bpc = gbtn.BeliefPropagationCache(tn)
    with pytest.raises(gbtn.InvalidArgument):  # not a tree (three components): maxiter is required
        bpc.update()
    bpc.update(maxiter=5, tol=1e-12, schedule="parallel", precision=precision)
    assert bpc.iterations[0] == 5 and np.isnan(bpc.mean_diff[0])
    bpc.update(maxiter=2, schedule="sequential")
    m = O.identity_messages(g)
    _, it, md = O.bp_update(g, A, m, maxiter=5, tol=1e-12, schedule="parallel")
    assert it == 5 and np.isnan(md)
    np.testing.assert_allclose(bpc.vertex_scalars(), [O.vertex_scalar(g, A, A, m, v) for v in range(g.nv)],
                               rtol=1e-12)
    assert bpc.logscalar() == pytest.approx(O.logscalar(g, A, A, m), rel=1e-12)
    ops = sz_ops(g)
    ref = [np.real(np.sum(O.vertex_rdm(g, A, A, m, v) * ops[v]) / np.trace(O.vertex_rdm(g, A, A, m, v)))
           for v in range(g.nv)]
    np.testing.assert_allclose(bpc.expect(ops, per_vertex=True), ref, rtol=1e-12, atol=1e-14)


def test_isolated_vertex_beside_a_lattice():
    lat = O.square_lattice(3, 3, chi=3)
    tn, g, A = both(10, lat.edges, lat.site_dims + [2], lat.edge_dims, 6)
    bpc = gbtn.BeliefPropagationCache(tn).update(maxiter=30, schedule="parallel")
    ref, _, _ = O.bp_update(g, A, O.identity_messages(g), maxiter=30, schedule="parallel")
    check_messages(bpc, g, ref)
    np.testing.assert_allclose(bpc.expect(O.SZ), O.expect1(g, A, ref, O.SZ), rtol=1e-10, atol=1e-13)
    assert bpc.logscalar() == pytest.approx(O.logscalar(g, A, A, ref), rel=1e-10)


@pytest.mark.parametrize("schedule", ["sequential", "parallel"])
def test_bond_dimension_one_is_exact(schedule):
    lat = O.square_lattice(3, 3, chi=1)
    tn, g, A = both(lat.nv, lat.edges, lat.site_dims, lat.edge_dims, 7)
    bpc = gbtn.BeliefPropagationCache(tn).update(maxiter=3, schedule=schedule)
    sz, norm = exact(g, A)
    np.testing.assert_allclose(bpc.expect(O.SZ), sz, rtol=0, atol=1e-12)
    assert np.exp(bpc.logscalar()) == pytest.approx(norm, rel=1e-11)
    assert all(m.shape == (1, 1) for m in bpc.messages())


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_site_dimension_one_and_mixed_site_dimensions(precision):
    lat = O.square_lattice(4, 3, chi=2)
    site = [1, 2, 3, 4, 1, 2, 3, 8, 2, 1, 5, 2]
    tn, g, A = both(lat.nv, lat.edges, site, lat.edge_dims, 8)
    bpc = gbtn.BeliefPropagationCache(tn).update(maxiter=6, schedule="parallel", precision=precision)
    ref, _, _ = O.bp_update(g, A, O.identity_messages(g), maxiter=6, schedule="parallel")
    check_messages(bpc, g, ref, 1e-10 if precision == "f64" else 1e-5)
    ops = sz_ops(g)
    got = bpc.expect(ops, per_vertex=True)
    want = [np.sum(O.vertex_rdm(g, A, A, ref, v) * ops[v]) / np.trace(O.vertex_rdm(g, A, A, ref, v))
            for v in range(g.nv)]
    np.testing.assert_allclose(got, want, rtol=0, atol=(1e-10 if precision == "f64" else 1e-5))


def test_bf16_refuses_the_sequential_schedule():
    # the tensor-core kernel computes every message of a vertex at once, so
    # BF16 sweeps run in parallel or in colour classes; a sequential request is
    # refused rather than run at another precision (the mixed pipeline runs its
    # FP32 and refinement phases in waves: test_gpu_sequential.py)
    bpc = gbtn.BeliefPropagationCache(gbtn.random_network(gbtn.square_lattice(3, 3, chi=2), 1))
    with pytest.raises(gbtn.Unsupported):
        bpc.update(maxiter=2, schedule="sequential", precision="bf16")


def test_degree_eight_vertex_on_a_star_is_exact():
    edges = [(0, k) for k in range(1, 9)]
    tn, g, A = both(9, edges, [2] * 9, [2] * 8, 9)
    assert max(len(l) for l in tn.legs) == 8
    bpc = gbtn.BeliefPropagationCache(tn).update()  # a tree: one sweep by default
    bpc2 = gbtn.BeliefPropagationCache(tn).update(maxiter=3, schedule="parallel")
    sz, norm = exact(g, A)
    for b in (bpc, bpc2):
        np.testing.assert_allclose(b.expect(O.SZ), sz, rtol=0, atol=1e-12)
        assert np.exp(b.logscalar()) == pytest.approx(norm, rel=1e-11)


def test_ragged_batch_converges_per_network():
    parts = []
    for k, (nv, edges, chi) in enumerate([
            (1, [], []),
            (2, [(0, 1)], [3]),
            (9, O.square_lattice(3, 3).edges, [2] * 12),
            (20, O.square_lattice(5, 4).edges, [3] * 31)]):
        parts.append(both(nv, edges, [2] * nv, chi, 20 + k))
    batch = gbtn.disjoint_union([p[0] for p in parts])
    bpc = gbtn.BeliefPropagationCache(batch).update(maxiter=200, tol=1e-12, schedule="parallel")
    it = bpc.iterations
    got = bpc.messages()
    off = 0
    for n, (tn, g, A) in enumerate(parts):
        ref, rit, rmd = O.bp_update(g, A, O.identity_messages(g), maxiter=200, tol=1e-12, schedule="parallel")
        assert it[n] == rit, (n, it[n], rit)
        if g.ne == 0:
            assert np.isnan(bpc.mean_diff[n]) and np.isnan(rmd)
        for de in range(2 * g.ne):
            np.testing.assert_allclose(got[off + de], ref[de], rtol=0, atol=1e-10)
        off += 2 * g.ne


def test_ragged_batch_on_the_tensor_cores():
    parts = [both(2, [(0, 1)], [2, 2], [5], 30), both(9, O.square_lattice(3, 3).edges, [2] * 9, [8] * 12, 31)]
    batch = gbtn.disjoint_union([p[0] for p in parts])
    bpc = gbtn.BeliefPropagationCache(batch).set_tc_policy("all")
    bpc.update(maxiter=1, schedule="parallel", precision="bf16")
    got = bpc.messages()
    off = 0
    for tn, g, A in parts:
        ref, _, _ = O.bp_update(g, A, O.identity_messages(g), maxiter=1, schedule="parallel")
        for de in range(2 * g.ne):
            np.testing.assert_allclose(got[off + de], ref[de], rtol=0, atol=3e-2)
        off += 2 * g.ne


def test_shapes_beyond_the_kernels_are_unsupported():
    star9 = gbtn.random_network(gbtn.TensorNetwork(10, [(0, k) for k in range(1, 10)], [2] * 10, [2] * 9), 1)
    with pytest.raises(gbtn.Unsupported, match="degree"):
        gbtn.BeliefPropagationCache(star9)
    big = gbtn.random_network(gbtn.square_lattice(2, 2, chi=2, d=65), 2)  # site dimensions run up to 64
    with pytest.raises(gbtn.Unsupported, match="site dimension"):
        gbtn.BeliefPropagationCache(big)
    # a tensor the shared-memory kernels cannot hold runs the global-memory path
    ok = gbtn.random_network(gbtn.square_lattice(3, 3, chi=8, d=4), 2)  # centre: 4 * 8^4 = 16384 entries
    gbtn.BeliefPropagationCache(ok).update(maxiter=2, schedule="parallel").close()
