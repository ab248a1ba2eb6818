"""Charge-conserving (QN) block-sparse networks on the GPU against the dense
FP64 oracle.

A U(1)-graded network is expanded to dense tensors (zero outside the blocks
that balance each vertex's flux) for the oracle; the library stores and
contracts only the blocks.  BP from identity messages keeps the messages
block-diagonal in the link sectors, so the library's sector-block messages,
expanded, must equal the oracle's dense messages: 1e-12 on unit-norm FP64
messages, 1e-10 relative on <Sz> and the log-scalar.  The reference's QN
regression case (test/test_belief_propagation.jl:103-116: a loopy 4-cycle of
S=1/2 sites, a product state, BP scalar finite and nonzero) is restated."""
import numpy as np
import pytest

import bp_oracle as O
import gbtn

pytestmark = pytest.mark.gpu

UP_DOWN = [(1, 1), (-1, 1)]  # S=1/2 site: charge 2 Sz of |up>, |down>


@pytest.fixture(scope="module", autouse=True)
def _lib(lib_built):
    yield


def oracle_graph(tn):
    return O.Graph(tn.nv, tn.edges, tn.site_dims, tn.edge_dims, tn.legs)


def random_u1_lattice(Lx, Ly, seed):
    tn = gbtn.square_lattice(Lx, Ly, chi=4)
    links = [[(-1, 1), (0, 2), (1, 1)]] * tn.ne
    sites = [UP_DOWN] * tn.nv
    flux = [1 if (v % Lx + v // Lx) % 2 else -1 for v in range(tn.nv)]
    return gbtn.random_qn_network(tn, links, sites, flux, seed, unit_norm=True)


@pytest.mark.parametrize("L", [(3, 3), (4, 4), (5, 3)])
def test_qn_bp_matches_dense_oracle(L):
    q = random_u1_lattice(*L, seed=10 + L[0])
    tn = q.tn
    g = oracle_graph(tn)
    A = tn.tensors
    m, _, _ = O.bp_update(g, A, O.identity_messages(g), maxiter=25, schedule="parallel")
    # the premise: dense BP keeps the messages block-diagonal in the link sectors
    for de in range(2 * g.ne):
        e = de // 2
        for c1, a1, b1 in gbtn.QNNetwork._ranges(q.link_sectors[e]):
            for c2, a2, b2 in gbtn.QNNetwork._ranges(q.link_sectors[e]):
                if c1 != c2:
                    assert np.max(np.abs(m[de][a1:b1, a2:b2])) < 1e-14
    bpc = gbtn.QNBeliefPropagationCache(q)
    assert bpc.n_block_elems < sum(tn.size(v) for v in range(tn.nv))  # only the allowed blocks are stored
    bpc.update(maxiter=25, schedule="parallel")
    got = bpc.messages()
    assert max(float(np.max(np.abs(got[de] - m[de]))) for de in range(2 * g.ne)) <= 1e-12
    sz = bpc.expect(O.SZ)
    ref = O.expect1(g, A, m, O.SZ)
    np.testing.assert_allclose(sz, ref, rtol=1e-10, atol=1e-13)
    assert bpc.logscalar() == pytest.approx(float(np.real(O.logscalar(g, A, A, m))), rel=1e-10)
    # and the dense plan on the expanded tensors agrees
    dense = gbtn.BeliefPropagationCache(tn).update(maxiter=25, schedule="parallel")
    assert max(float(np.max(np.abs(dense.messages()[de] - got[de]))) for de in range(2 * g.ne)) <= 1e-12
    dense.close()
    bpc.close()


def test_qn_convergence_and_diff():
    q = random_u1_lattice(4, 4, seed=3)
    g = oracle_graph(q.tn)
    m, it, md = O.bp_update(g, q.tn.tensors, O.identity_messages(g), maxiter=200, tol=1e-12, schedule="parallel")
    bpc = gbtn.QNBeliefPropagationCache(q).update(maxiter=200, tol=1e-12, schedule="parallel")
    assert abs(bpc.iterations - it) <= 1
    assert max(float(np.max(np.abs(bpc.messages()[de] - m[de]))) for de in range(2 * g.ne)) <= 1e-6
    bpc.close()


def test_qn_graded_loopy_product_state_scalar():
    # test/test_belief_propagation.jl:109-116: a 4-cycle of S=1/2 sites with
    # conserved Sz, the product state up/down by site parity, BP scalar of
    # <psi|psi> from identity messages: finite, nonzero (and exactly 1 here)
    tn = gbtn.square_lattice(2, 2, chi=1)
    up, dn = np.array([1.0, 0.0]), np.array([0.0, 1.0])
    flux, ts = [], []
    for v in range(tn.nv):
        i, j = v % 2, v // 2
        odd = (i + j + 2) % 2 == 1
        ts.append((up if odd else dn).reshape((2,) + (1,) * len(tn.legs[v])))
        flux.append(1 if odd else -1)
    tn.tensors = ts
    q = gbtn.QNNetwork(tn, [[(0, 1)]] * tn.ne, [UP_DOWN] * tn.nv, flux)
    bpc = gbtn.QNBeliefPropagationCache(q).update(maxiter=25)  # the reference's default: sequential
    n2 = bpc.scalar()
    assert np.isfinite(n2) and n2 != 0
    assert n2 == pytest.approx(O.exact_scalar(oracle_graph(tn), ts), rel=1e-12)
    np.testing.assert_allclose(bpc.expect(O.SZ), [0.5 if f > 0 else -0.5 for f in flux], atol=1e-14)
    bpc.close()


def test_qn_refusals():
    tn = gbtn.square_lattice(2, 2, chi=2)
    q = gbtn.random_qn_network(tn, [[(0, 1), (0, 1)]] * tn.ne, [UP_DOWN] * tn.nv, [1, -1, -1, 1], 1)
    with pytest.raises(gbtn.Unsupported, match="distinct charges"):
        gbtn.QNBeliefPropagationCache(q)
    tn9 = gbtn.square_lattice(2, 2, chi=9)
    q9 = gbtn.random_qn_network(tn9, [[(0, 9)]] * tn9.ne, [UP_DOWN] * tn9.nv, [1, 1, 1, 1], 1)
    with pytest.raises(gbtn.Unsupported, match="sector dimensions"):
        gbtn.QNBeliefPropagationCache(q9)


@pytest.mark.parametrize("L", [(3, 3), (4, 3)])
def test_qn_sequential_schedule_matches_the_strict_sequence(L):
    """The reference's default update: the forest-cover edge sequence, each
    message seeing every earlier one.  Three sweeps (far from converged, so
    the order matters) equal the dense oracle's strictly sequential sweeps to
    1e-12, with the mean diff over the sequence; a sequence with repeats and
    a converged run with a tolerance as well."""
    q = random_u1_lattice(*L, seed=30 + L[0])
    tn = q.tn
    g = oracle_graph(tn)
    A = tn.tensors
    seq = list(gbtn.default_edge_sequence(tn))
    m, _, md = O.bp_update(g, A, O.identity_messages(g), maxiter=3, tol=0.0, schedule="sequential", edge_sequence=seq)
    bpc = gbtn.QNBeliefPropagationCache(q).update(maxiter=3, tol=0.0)
    got = bpc.messages()
    assert max(float(np.max(np.abs(got[de] - m[de]))) for de in range(2 * g.ne)) <= 1e-12
    assert bpc.mean_diff == pytest.approx(md, rel=1e-9, abs=1e-15)
    # repeats and gaps in the sequence
    seq2 = seq[: len(seq) // 2] + seq[:3] + seq[len(seq) // 2:][::2]
    m2, _, _ = O.bp_update(g, A, O.identity_messages(g), maxiter=2, schedule="sequential", edge_sequence=seq2)
    bpc.init_messages()
    bpc.update(maxiter=2, edge_sequence=seq2)
    got2 = bpc.messages()
    assert max(float(np.max(np.abs(got2[de] - m2[de]))) for de in range(2 * g.ne)) <= 1e-12
    # to convergence under the tolerance: the oracle's sequential run (Jacobi
    # sweeps may oscillate or settle elsewhere on a loopy graph)
    bpc.init_messages()
    bpc.update(maxiter=200, tol=1e-14)
    ref, it, _ = O.bp_update(g, A, O.identity_messages(g), maxiter=200, tol=1e-14, schedule="sequential",
                             edge_sequence=seq)
    assert abs(bpc.iterations - it) <= 1
    np.testing.assert_allclose(bpc.expect(O.SZ), O.expect1(g, A, ref, O.SZ), rtol=1e-9, atol=1e-12)
    bpc.close()


def max_msg_err(got, ref):
    return max(float(np.max(np.abs(g - r))) for g, r in zip(got, ref))


def test_qn_reduced_precision_sweeps_against_the_oracle():
    """FP32 and double-FP32 parallel sweeps on the blocks: 25 sweeps from
    identity messages against the oracle's FP64 sweeps -- FP32 to 1e-5 on the
    unit-norm messages (a few FP32 roundings per sweep, contracted by BP),
    double-FP32 to 1e-12 (unit roundoff 2^-48 in the products and sums, FP64
    storage)."""
    q = random_u1_lattice(4, 4, seed=3)
    g = oracle_graph(q.tn)
    A = q.tn.tensors
    m, _, _ = O.bp_update(g, A, O.identity_messages(g), maxiter=25, schedule="parallel")
    bpc = gbtn.QNBeliefPropagationCache(q)
    bpc.update(maxiter=25, schedule="parallel", precision="f32")
    assert bpc.phase_sweeps()["f32"] == 25
    assert max_msg_err(bpc.messages(), m) <= 1e-5
    bpc.init_messages()
    bpc.update(maxiter=25, schedule="parallel", precision="df32")
    assert bpc.phase_sweeps()["refine"] == 25
    assert max_msg_err(bpc.messages(), m) <= 1e-12
    bpc.close()


@pytest.mark.parametrize("schedule", ["parallel", "sequential"])
def test_qn_mixed_solve_reaches_the_fp64_fixed_point(schedule):
    """MIXED: FP32 sweeps to their tolerance or noise floor, then double-FP32
    sweeps from there.  With every refinement sweep run (no tolerance) the
    result is the FP64 fixed point of the same schedule: <Sz> to 1e-10
    relative against the oracle run to its rounding floor."""
    q = random_u1_lattice(4, 4, seed=3)
    g = oracle_graph(q.tn)
    A = q.tn.tensors
    seq = list(gbtn.default_edge_sequence(q.tn)) if schedule == "sequential" else None
    ref, _, _ = O.bp_update(g, A, O.identity_messages(g), maxiter=400, schedule=schedule, edge_sequence=seq)
    bpc = gbtn.QNBeliefPropagationCache(q)
    bpc.update(maxiter=150, schedule=schedule, precision="mixed")
    ph = bpc.phase_sweeps()
    assert 0 < ph["f32"] < 150 and ph["refine"] == 150
    np.testing.assert_allclose(bpc.expect(O.SZ), O.expect1(g, A, ref, O.SZ), rtol=1e-10, atol=1e-13)
    assert bpc.logscalar() == pytest.approx(float(np.real(O.logscalar(g, A, A, ref))), rel=1e-10)
    # with a tolerance the refinement stops when the mean diff reaches it
    bpc.init_messages()
    bpc.update(maxiter=150, tol=1e-13, schedule=schedule, precision="mixed", refine="f64")
    assert bpc.mean_diff <= 1e-13 and bpc.phase_sweeps()["refine"] == bpc.iterations < 150
    np.testing.assert_allclose(bpc.expect(O.SZ), O.expect1(g, A, ref, O.SZ), rtol=1e-5, atol=1e-8)
    bpc.close()


def test_qn_precision_refusals():
    q = random_u1_lattice(3, 3, seed=4)
    bpc = gbtn.QNBeliefPropagationCache(q)
    with pytest.raises(gbtn.Unsupported, match="tensor-core"):
        bpc.update(maxiter=3, schedule="parallel", precision="bf16")
    with pytest.raises(gbtn.InvalidArgument):
        bpc.update(maxiter=3, schedule="colored", precision="f32")
    bpc.close()


def test_qn_gradients_are_the_dense_adjoint_on_the_blocks():
    """Gradients of a QN cache: the dense plan's implicit adjoints at the QN
    fixed point, gathered at the allowed blocks (the dense tensors are the
    blocks embedded with zeros, a linear map).  Against central differences of
    the oracle's converged log-norm and energy along directions inside the
    blocks (h = 1e-5, 1e-6 relative), zero outside the blocks."""
    from gbtn.operators import HEISENBERG
    q = random_u1_lattice(3, 3, seed=12)
    g = oracle_graph(q.tn)
    A = q.tn.tensors
    bpc = gbtn.QNBeliefPropagationCache(q).update(maxiter=400, schedule="parallel")
    val, G = bpc.logscalar_grad(tol=1e-14)
    E, GE = bpc.energy2_grad(HEISENBERG, tol=1e-14)
    for v in range(g.nv):
        assert not np.any(G[v][~q.mask(v)]) and not np.any(GE[v][~q.mask(v)])

    def converged(ts):
        m, _, _ = O.bp_update(g, ts, O.identity_messages(g), maxiter=400, schedule="parallel")
        return m

    def f_log(ts):
        return float(np.real(O.logscalar(g, ts, ts, converged(ts))))

    heis = sum(c * np.kron(op, op) for c, op in HEISENBERG)

    def f_energy(ts):
        return float(np.sum(O.expect2(g, ts, converged(ts), heis)))

    assert val == pytest.approx(f_log(A), rel=1e-10)
    assert E == pytest.approx(f_energy(A), rel=1e-9)
    rng = np.random.default_rng(4)
    D = [rng.standard_normal(a.shape) * q.mask(v) for v, a in enumerate(A)]
    nrm = np.sqrt(sum(np.sum(d * d) for d in D))
    D = [d / nrm for d in D]
    h = 1e-5
    for f, grad in ((f_log, G), (f_energy, GE)):
        fd = (f([a + h * d for a, d in zip(A, D)]) - f([a - h * d for a, d in zip(A, D)])) / (2 * h)
        an = sum(float(np.sum(x * d)) for x, d in zip(grad, D))
        assert an == pytest.approx(fd, rel=1e-6, abs=1e-10)
    bpc.close()
