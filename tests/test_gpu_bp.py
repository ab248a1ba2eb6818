"""GPU parity of the BP hot path against the FP64 oracle, through the C ABI.

Tolerances: FP64 paths 1e-10 relative (1e-12 absolute on unit-norm
messages); FP32 paths 1e-5 absolute on <Sz>; MIXED (FP32 then FP64
refinement) 1e-10 relative on <Sz> after convergence."""
from pathlib import Path

import numpy as np
import pytest

import bp_oracle as O
import build_oracle
import gbtn

pytestmark = pytest.mark.gpu
GOLD = np.load(Path(__file__).parent / "golden" / "bp_small.npz")
EPS = np.finfo(float).eps


@pytest.fixture(scope="module", autouse=True)
def _lib(lib_built):
    yield


def pair(Lx, Ly, seed, chi=2, edge_dims=None, unit_norm=False):
    tn = gbtn.square_lattice(Lx, Ly, chi=chi, edge_dims=edge_dims)
    tn = gbtn.random_network(tn, seed, unit_norm=unit_norm)
    g = O.square_lattice(Lx, Ly, chi=chi, edge_dims=edge_dims)
    A = O.random_network(g, seed, unit_norm=unit_norm)
    np.testing.assert_array_equal(tn.flat(), O.flatten_tensors(A))
    return tn, g, A


def test_c1_sequential_f64_golden():
    tn, g, A = pair(4, 4, int(GOLD["c1__seed"]))
    bpc = gbtn.BeliefPropagationCache(tn)
    bpc.init_messages("ones")
    bpc.update(maxiter=20, schedule="sequential")
    np.testing.assert_allclose(tn.flat_messages(bpc.messages()), GOLD["c1__msgs"], rtol=0, atol=1e-12)
    sz = bpc.expect(O.SZ)
    np.testing.assert_allclose(sz, GOLD["c1__sz"], rtol=1e-10, atol=1e-14)
    np.testing.assert_array_equal(bpc.expect("Sz"), sz)  # expect(psi, "Sz") by name, as the reference
    assert bpc.logscalar() == pytest.approx(float(GOLD["c1__logscalar"]), rel=1e-12)
    assert list(bpc.iterations) == [20]


def test_grid3_converges_like_reference():
    tn, g, A = pair(3, 3, int(GOLD["grid3__seed"]))
    bpc = gbtn.BeliefPropagationCache(tn).update(maxiter=25, tol=EPS)
    assert abs(int(bpc.iterations[0]) - int(GOLD["grid3__iters"])) <= 1
    np.testing.assert_allclose(tn.flat_messages(bpc.messages()), GOLD["grid3__msgs"], atol=1e-12)
    # test_belief_propagation.jl:49-55 on the GPU
    msgs = bpc.messages()
    for de in range(2 * tn.ne):
        assert gbtn.message_diff(bpc.updated_message(de), msgs[de]) < 10 * EPS


def test_uneven_parallel_golden():
    dims = [int(x) for x in GOLD["uneven__dims"]]
    tn, g, A = pair(5, 4, int(GOLD["uneven__seed"]), edge_dims=dims)
    bpc = gbtn.BeliefPropagationCache(tn).update(maxiter=60, tol=1e-14, schedule="parallel")
    np.testing.assert_allclose(tn.flat_messages(bpc.messages()), GOLD["uneven__msgs"], atol=1e-11)
    np.testing.assert_allclose(bpc.expect(O.SZ), GOLD["uneven__sz"], rtol=1e-10, atol=1e-13)
    np.testing.assert_allclose(bpc.expect2(O.kron2(O.SZ, O.SZ)), GOLD["uneven__szsz"], rtol=1e-10, atol=1e-13)
    assert bpc.logscalar() == pytest.approx(float(GOLD["uneven__logscalar"]), rel=1e-11)


def test_tree_bp_equals_exact():
    edges = [tuple(e) for e in GOLD["tree__edges"]]
    n = int(GOLD["tree__n"])
    chi = int(GOLD["tree__chi"])
    tn = gbtn.TensorNetwork(n, edges, [2] * n, [chi] * len(edges))
    g = O.Graph(n, edges, [2] * n, [chi] * len(edges))
    A = O.random_network(g, int(GOLD["tree__seed"]))
    tn.tensors = A
    bpc = gbtn.BeliefPropagationCache(tn).update()  # maxiter defaults to 1 on a tree
    np.testing.assert_allclose(bpc.expect(O.SZ), GOLD["tree__sz_exact"], rtol=1e-10, atol=1e-13)
    assert bpc.logscalar() == pytest.approx(float(GOLD["tree__log_exact"]), rel=1e-11)


def test_inner_bp_exact_on_tree():
    g = O.comb_tree(2, 3, chi=2)
    x = O.random_network(g, 1)
    y = O.random_network(g, 2)
    tx = gbtn.TensorNetwork(g.nv, g.edges, g.site_dims, g.edge_dims, x)
    ty = gbtn.TensorNetwork(g.nv, g.edges, g.site_dims, g.edge_dims, y)
    val = gbtn.inner(tx, ty, cache_update_kwargs=dict(maxiter=1))
    assert val == pytest.approx(O.exact_scalar(g, y, x), rel=1e-10)


@pytest.mark.parametrize("schedule", ["sequential", "parallel", "colored"])
def test_schedules_match_oracle_f64(schedule):
    tn, g, A = pair(5, 3, 21, chi=3)
    bpc = gbtn.BeliefPropagationCache(tn).update(maxiter=7, schedule=schedule)
    m, _, _ = O.bp_update(g, A, O.identity_messages(g), maxiter=7, schedule=schedule)
    np.testing.assert_allclose(tn.flat_messages(bpc.messages()), O.flatten_messages(g, m), atol=1e-12)


def test_f32_and_mixed_paths():
    # tol bounds 1-cos^2 of messages, i.e. message angles only to sqrt(tol); the
    # 1e-10 comparison therefore uses a fixed, fully converged sweep count.
    tn, g, A = pair(6, 6, 3, chi=4, unit_norm=True)
    mc, _, _ = build_oracle.run(g, O.flatten_tensors(A), O.flatten_messages(g, O.identity_messages(g)), "parallel",
                                None, 400, tol=None, nthreads=4)
    ref = O.expect1(g, A, O.unflatten_messages(g, mc), O.SZ)
    scale = np.max(np.abs(ref))
    b32 = gbtn.BeliefPropagationCache(tn).update(maxiter=400, tol=1e-12, schedule="parallel", precision="f32")
    assert np.max(np.abs(b32.expect(O.SZ) - ref)) / scale < 1e-5
    # a few FP64 sweeps from the FP32 fixed point already meet the 1e-6 target ...
    bm = gbtn.BeliefPropagationCache(tn).update(maxiter=400, tol=1e-15, schedule="parallel", precision="mixed",
                                                refine_f64=2)
    assert np.max(np.abs(bm.expect(O.SZ) - ref)) / scale < 1e-6
    # ... and a full FP64 phase reaches the FP64 answer
    bm = gbtn.BeliefPropagationCache(tn).update(maxiter=400, schedule="parallel", precision="mixed")
    assert np.max(np.abs(bm.expect(O.SZ) - ref)) / scale < 1e-10


def test_batched_networks_converge_independently():
    nets, pairs = [], []
    for k, (L, chi) in enumerate([(3, 2), (4, 3), (2, 2), (5, 2)]):
        tn, g, A = pair(L, L, 40 + k, chi=chi)
        nets.append(tn)
        pairs.append((g, A))
    batch = gbtn.disjoint_union(nets)
    bpc = gbtn.BeliefPropagationCache(batch).update(maxiter=80, tol=1e-13, schedule="parallel")
    sz = bpc.expect(O.SZ)
    off = 0
    for k, (g, A) in enumerate(pairs):
        m, it, _ = O.bp_update(g, A, O.identity_messages(g), maxiter=80, tol=1e-13, schedule="parallel")
        assert abs(int(bpc.iterations[k]) - it) <= 1
        np.testing.assert_allclose(sz[off:off + g.nv], O.expect1(g, A, m, O.SZ), atol=1e-9)
        off += g.nv
    ls = bpc.logscalar()
    assert len(ls) == 4


def test_c2_shape_f32_parallel_vs_fp64_oracle():
    # 16x16, d=2, chi=4, unit-norm tensors, FP32 Jacobi, tol 1e-8, <= 50 sweeps
    tn, g, A = pair(16, 16, 2, chi=4, unit_norm=True)
    bpc = gbtn.BeliefPropagationCache(tn).update(maxiter=50, tol=1e-8, schedule="parallel", precision="f32")
    it = int(bpc.iterations[0])
    mc, itc, _ = build_oracle.run(g, O.flatten_tensors(A), O.flatten_messages(g, O.identity_messages(g)), "parallel",
                                  None, it, tol=None, nthreads=4)
    m = O.unflatten_messages(g, mc)
    np.testing.assert_allclose(bpc.expect(O.SZ), O.expect1(g, A, m, O.SZ), atol=1e-5)
    np.testing.assert_allclose(bpc.expect2(O.kron2(O.SZ, O.SZ)), O.expect2(g, A, m, O.kron2(O.SZ, O.SZ)), atol=1e-5)


def test_two_site_rdm_psd_and_matches_oracle():
    tn, g, A = pair(3, 3, 1234)
    bpc = gbtn.BeliefPropagationCache(tn).update(maxiter=25, tol=EPS)
    m, _, _ = O.bp_update(g, A, O.identity_messages(g), maxiter=25, tol=EPS)
    rdms = bpc.edge_rdms()
    for e, r in enumerate(rdms):
        np.testing.assert_allclose(r, O.edge_rdm(g, A, A, m, e), rtol=1e-10, atol=1e-13)
        r = r / np.trace(r)
        assert np.all(np.linalg.eigvalsh(0.5 * (r + r.T)) >= -EPS)


def test_zero_network_logscalar_is_minus_inf():
    tn, g, A = pair(3, 1, 1234)
    tn.tensors[0] = 0 * tn.tensors[0]
    bpc = gbtn.BeliefPropagationCache(tn).update(maxiter=1)
    assert bpc.scalar() == 0.0


def test_rescale_gives_unit_scalars():
    tn, g, A = pair(3, 2, 1234)
    bpc = gbtn.BeliefPropagationCache(tn).update(maxiter=20)
    bpc.rescale()
    np.testing.assert_allclose(bpc.edge_scalars(), 1.0, rtol=1e-12)
    np.testing.assert_allclose(bpc.vertex_scalars(), 1.0, rtol=1e-12)
    assert all(np.array_equal(t, a) for t, a in zip(tn.tensors, A))  # the input network is not rescaled
    psi = gbtn.normalize(tn, cache_update_kwargs=dict(maxiter=20))
    assert all(np.array_equal(t, a) for t, a in zip(tn.tensors, A))
    assert gbtn.scalar(psi, cache_update_kwargs=dict(maxiter=20)) == pytest.approx(1.0, rel=1e-10)


def test_argument_errors_map_to_reference_errors():
    tn, g, A = pair(3, 3, 1)
    bpc = gbtn.BeliefPropagationCache(tn)
    with pytest.raises(gbtn.InvalidArgument, match="number of iterations"):
        bpc.update()
    with pytest.raises(gbtn.InvalidArgument):
        bpc.update(maxiter=2, edge_sequence=[0, 1, 999])
    big = gbtn.random_network(gbtn.square_lattice(2, 2, chi=65), 1)  # bond dimensions run up to 64
    with pytest.raises(gbtn.Unsupported):
        gbtn.BeliefPropagationCache(big)


def test_full_size_fixed_point_properties():
    # 32x32, chi=8, d=2: size-independent checks at the target shape
    tn = gbtn.random_network(gbtn.square_lattice(32, 32, chi=8), 5)
    bpc = gbtn.BeliefPropagationCache(tn).update(maxiter=100, tol=1e-13, schedule="parallel", precision="mixed",
                                                refine_f64=3)
    msgs = bpc.messages()
    for de in (0, 1, 777, 2 * tn.ne - 1):
        m = msgs[de]
        assert np.linalg.norm(m) == pytest.approx(1.0, rel=1e-12)
        # real messages are symmetric in exact arithmetic; the FP32 phase leaves
        # roundoff-level asymmetry that three FP64 sweeps only contract by rho^3
        np.testing.assert_allclose(m, m.T, atol=1e-6)
        assert gbtn.message_diff(bpc.updated_message(de), m) < 1e-10
    sz = bpc.expect(O.SZ)
    assert np.all(np.abs(sz) <= 0.5 + 1e-12)
