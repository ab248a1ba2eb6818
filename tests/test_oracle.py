"""The FP64 oracle against the reference's own known-answer tests, the golden
fixtures, and the C restatement (CPU only)."""
from pathlib import Path

import numpy as np
import pytest

import bp_oracle as O
import build_oracle

GOLD = np.load(Path(__file__).parent / "golden" / "bp_small.npz")
EPS = np.finfo(float).eps


def exact_sz(g, A):
    out = []
    for v in range(g.nv):
        r = O.exact_rdm1(g, A, v)
        out.append(np.sum(r * O.SZ) / np.trace(r))
    return np.array(out)


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_bp_exact_on_trees(seed):
    # test/test_expect.jl:12-20 and test/test_inner.jl:12-48: BP = exact on a tree
    g = O.random_tree(7, seed=seed, chi=2)
    A = O.random_network(g, 100 + seed)
    m, it, _ = O.bp_update(g, A, O.identity_messages(g), maxiter=1)
    assert it == 1
    np.testing.assert_allclose(O.expect1(g, A, m, O.SZ), exact_sz(g, A), rtol=1e-12, atol=1e-14)
    assert O.logscalar(g, A, A, m) == pytest.approx(np.log(O.exact_scalar(g, A)), rel=1e-12)


def test_bp_exact_on_comb_tree_inner():
    # inner(x, y; alg="bp") == exact on a tree (test_inner.jl:21-38)
    g = O.comb_tree(2, 3, chi=2)
    x = O.random_network(g, 1)
    y = O.random_network(g, 2)
    m, _, _ = O.bp_update(g, y, O.identity_messages(g), B=x, maxiter=1)
    ex = O.exact_scalar(g, y, x)
    ls = O.logscalar(g, y, x, m)
    assert np.exp(ls) == pytest.approx(ex, rel=1e-11)


def test_fixed_point_residual():
    # test_belief_propagation.jl:49-55 on a 3x3 grid, chi=2
    g = O.square_lattice(3, 3, chi=2)
    A = O.random_network(g, 1234)
    m, _, _ = O.bp_update(g, A, O.identity_messages(g), maxiter=25, tol=EPS)
    for de in range(2 * g.ne):
        assert O.message_diff(O.updated_message(g, A, A, m, de), m[de]) < 10 * EPS


def test_two_site_rdm_hermitian_psd():
    # test_belief_propagation.jl:64-91
    g = O.square_lattice(3, 3, chi=2)
    A = O.random_network(g, 1234)
    m, _, _ = O.bp_update(g, A, O.identity_messages(g), maxiter=25, tol=EPS)
    e = g.edges.index((4, 7)) if (4, 7) in g.edges else 0
    rho = O.edge_rdm(g, A, A, m, e)
    rho = rho / np.trace(rho)
    assert rho.shape == (4, 4)
    assert np.max(np.abs(rho - rho.T)) < 10 * EPS
    assert np.all(np.linalg.eigvalsh(rho) >= -EPS)


def test_zero_network_scalar_is_zero():
    # test_belief_propagation.jl:93-99
    g = O.square_lattice(3, 1, chi=2)
    A = O.random_network(g, 1234)
    A[0] = 0 * A[0]
    m, _, _ = O.bp_update(g, A, O.identity_messages(g), maxiter=1)
    assert np.exp(O.logscalar(g, A, A, m)) == 0.0


def test_product_state_bp_exact():
    # test_expect.jl:41-50: product state, BP exact
    g = O.square_lattice(2, 2, chi=1)
    up, dn = np.array([1.0, 0.0]), np.array([0.0, 1.0])
    A = [(up if (v % 2 + v // 2) % 2 else dn).reshape((2,) + (1,) * len(g.legs[v])) for v in range(g.nv)]
    m, _, _ = O.bp_update(g, A, O.identity_messages(g), maxiter=20)
    np.testing.assert_allclose(O.expect1(g, A, m, O.SZ), exact_sz(g, A), atol=1e-14)


def test_normalize_gives_unit_scalars():
    # test_normalize.jl:30-66 (a real state here; the ComplexF32 one runs on the GPU path)
    g = O.square_lattice(3, 2, chi=2)
    A = O.random_network(g, 1234)
    m, _, _ = O.bp_update(g, A, O.identity_messages(g), maxiter=20)
    A2, m2 = O.normalize_bp(g, A, m)
    np.testing.assert_allclose([O.edge_scalar(g, m2, e) for e in range(g.ne)], 1.0, rtol=1e-12)
    np.testing.assert_allclose([O.vertex_scalar(g, A2, A2, m2, v) for v in range(g.nv)], 1.0, rtol=1e-12)
    m3, _, _ = O.bp_update(g, A2, O.identity_messages(g), maxiter=20)
    assert np.exp(O.logscalar(g, A2, A2, m3)) == pytest.approx(1.0, rel=1e-10)


@pytest.mark.parametrize("n", [2, 3, 5, 10])
def test_map_eigvals_identities(n):
    # test_map_eigvals.jl:7-34 (Float64)
    rng = np.random.default_rng(1234)
    X = rng.standard_normal((n, n))
    P = X @ X.T
    s = O.map_eigvals(np.sqrt, P, 0.0)
    np.testing.assert_allclose(s @ s.T, P, rtol=1e-10, atol=1e-10)
    inv = O.map_eigvals(lambda x: 1 / x, P, 0.0)
    np.testing.assert_allclose(inv @ P, np.eye(n), atol=1e-8)
    isq = O.map_eigvals(lambda x: 1 / np.sqrt(x), P, 0.0)
    np.testing.assert_allclose(isq @ s, np.eye(n), atol=1e-8)


def _state(g, A):
    ops, lid = [], {e: 10 + e for e in range(g.ne)}
    for v in range(g.nv):
        ops += [A[v], [v] + [lid[e] for e in g.legs[v]]]
    return np.einsum(*ops, list(range(g.nv)))


def test_simple_update_matches_exact_gate():
    # apply(o, psi) without truncation equals the exact gate application
    g = O.square_lattice(2, 2, chi=2)
    A = O.random_network(g, 7)
    Q, _ = np.linalg.qr(np.random.default_rng(5).standard_normal((4, 4)))
    e = 0
    u, v = g.edges[e]
    pu, pv = g.legs[u].index(e), g.legs[v].index(e)
    m, _, _ = O.bp_update(g, A, O.identity_messages(g), maxiter=30, tol=1e-14)
    envs_u = {1 + p: m[g.directed(f, g.other(u, f))] for p, f in enumerate(g.legs[u]) if f != e}
    envs_v = {1 + p: m[g.directed(f, g.other(v, f))] for p, f in enumerate(g.legs[v]) if f != e}
    for eu, ev in (({}, {}), (envs_u, envs_v)):
        Au, Av, S, te = O.simple_update(Q, A[u], A[v], pu, pv, eu, ev)
        B = list(A)
        B[u], B[v] = Au, Av
        g2 = O.Graph(g.nv, g.edges, g.site_dims, list(g.edge_dims))
        g2.edge_dims[e] = Au.shape[pu + 1]
        exact = np.einsum("abst,stkl->abkl", Q.reshape(2, 2, 2, 2, order="F"), _state(g, A))
        np.testing.assert_allclose(_state(g2, B), exact, atol=1e-12)
        assert te == 0.0


def test_simple_update_truncation_nonzero_error():
    # test_apply.jl:52-63: truncated gate -> truncerr != 0 and fidelity > 0
    g = O.square_lattice(2, 2, chi=2)
    A = O.random_network(g, 1234)
    Q, _ = np.linalg.qr(np.random.default_rng(9).standard_normal((4, 4)))
    e = 0
    u, v = g.edges[e]
    Au, Av, S, te = O.simple_update(Q, A[u], A[v], g.legs[u].index(e), g.legs[v].index(e), {}, {}, maxdim=2)
    assert te > 0 and len(S) == 2
    B = list(A)
    B[u], B[v] = Au, Av
    g2 = O.Graph(g.nv, g.edges, g.site_dims, list(g.edge_dims))
    exact = np.einsum("abst,stkl->abkl", Q.reshape(2, 2, 2, 2, order="F"), _state(g, A))
    f = np.vdot(_state(g2, B), exact)
    assert abs(f) > 0


def test_truncate_spectrum_rule():
    p = np.array([0.5, 0.3, 0.15, 0.04, 0.01])
    assert O.truncate_spectrum(p, maxdim=3)[0] == 3
    n, te = O.truncate_spectrum(p, cutoff=0.02)
    assert n == 4 and te == pytest.approx(0.01)
    n, te = O.truncate_spectrum(p, cutoff=0.05)
    assert n == 3 and te == pytest.approx(0.05)
    assert O.truncate_spectrum(np.zeros(3), cutoff=1e-10)[0] == 1


def test_golden_fixtures_reproduce():
    g = O.square_lattice(4, 4, chi=2)
    A = O.random_network(g, int(GOLD["c1__seed"]))
    assert O.default_edge_sequence(g) == list(GOLD["c1__seq"])
    m, _, _ = O.bp_update(g, A, O.ones_messages(g), maxiter=20, schedule="sequential")
    np.testing.assert_allclose(O.flatten_messages(g, m), GOLD["c1__msgs"], rtol=0, atol=1e-13)
    np.testing.assert_allclose(O.expect1(g, A, m, O.SZ), GOLD["c1__sz"], atol=1e-13)
    # the tree fixture carries its own exactness pin
    np.testing.assert_allclose(GOLD["tree__sz"], GOLD["tree__sz_exact"], atol=1e-12)
    assert float(GOLD["tree__logscalar"]) == pytest.approx(float(GOLD["tree__log_exact"]), rel=1e-12)


def test_schedules_share_the_fixed_point():
    g = O.square_lattice(4, 3, chi=3)
    A = O.random_network(g, 3)
    ref = None
    for sch in ("sequential", "parallel", "colored"):
        m, it, md = O.bp_update(g, A, O.identity_messages(g), maxiter=400, tol=1e-20, schedule=sch)
        sz = O.expect1(g, A, m, O.SZ)
        if ref is None:
            ref = sz
        np.testing.assert_allclose(sz, ref, atol=1e-9)


@pytest.mark.parametrize("schedule", ["sequential", "parallel"])
def test_c_restatement_matches_oracle(schedule):
    rng = np.random.default_rng(4)
    g0 = O.square_lattice(4, 3)
    g = O.square_lattice(4, 3, edge_dims=[int(x) for x in rng.integers(1, 5, size=g0.ne)])
    A = O.random_network(g, 9)
    seq = O.default_edge_sequence(g) if schedule == "sequential" else O.parallel_edge_sequence(g)
    m, it, md = O.bp_update(g, A, O.identity_messages(g), maxiter=15, tol=1e-300, schedule=schedule,
                            edge_sequence=seq)
    mc, itc, mdc = build_oracle.run(g, O.flatten_tensors(A), O.flatten_messages(g, O.identity_messages(g)),
                                    schedule, seq if schedule == "sequential" else None, 15, tol=1e-300, nthreads=2)
    np.testing.assert_allclose(mc, O.flatten_messages(g, m), rtol=1e-12, atol=1e-14)
    assert itc == it


def test_rescale_partitions_with_a_separate_bra_gives_unit_scalars():
    # abstractbeliefpropagationcache.jl:349-379 with ket and bra vertices
    # (the bra first in each partition): every partition scalar becomes 1 --
    # complex tensors with an independent bra (any phase), and real tensors
    # with positive scalars (a negative real scalar has no real square root:
    # the reference raises a DomainError there, the oracle returns NaN)
    for dtype, seed_b in ((np.complex128, 4), (np.float64, 3)):
        g = O.square_lattice(3, 3, chi=2)
        A = O.random_network(g, 3, dtype=dtype)
        B = O.random_network(g, seed_b, dtype=dtype)
        m, _, _ = O.bp_update(g, A, O.identity_messages(g), B=B, maxiter=30, schedule="parallel")
        k, b = O.rescale_partitions(g, A, m, B)
        for v in range(g.nv):
            z = np.trace(O.contract_partition(g, {v: k[v]}, {v: b[v]}, m, v, open_site=True))
            assert abs(z - 1.0) < 1e-12


def test_exact_environment_equals_bp_messages_on_a_tree():
    # environment(qf, [v]; alg="exact") against the BP environment on a tree
    # (test_forms.jl:59-73): the product of the incoming messages, normalised
    g = O.comb_tree(3, 3, chi=2)
    A = O.random_network(g, 7)
    m, _, _ = O.bp_update(g, A, O.identity_messages(g), maxiter=1)
    for v in range(g.nv):
        k = len(g.legs[v])
        ops = []
        for p, e in enumerate(g.legs[v]):
            de = 2 * e if g.edges[e][1] == v else 2 * e + 1
            ops += [m[de], [p, k + p]]
        env_bp = np.einsum(*ops, list(range(2 * k)))
        env_ex = O.exact_environment(g, A, v)
        np.testing.assert_allclose(env_bp / np.linalg.norm(env_bp), env_ex / np.linalg.norm(env_ex),
                                   rtol=0, atol=1e-12)


def test_trotter_tebd_lowers_the_ising_energy():
    # tebd.jl:2-31 on the Ising model of test_tebd.jl (2 x 3, h = 0.1, all up,
    # beta 2, dbeta 0.2, maxdim 2): the energy goes down, towards the exact
    # ground energy, and the Trotter list is a palindrome of half steps
    g = O.square_lattice(2, 3, chi=1)
    terms = O.ising_terms(g, h=0.1)
    groups = O.group_terms(terms, g)
    seq = O.trotter2_gates(g, groups, 0.2)
    assert [e for e, _ in seq] == [e for e, _ in groups] + [e for e, _ in groups][::-1]
    up = np.array([1.0, 0.0])
    A = [up.reshape((2,) + (1,) * len(g.legs[v])) for v in range(g.nv)]

    def energy(gg, T):
        ops = []
        for v in range(gg.nv):
            ops += [T[v], [v] + [20 + e for e in gg.legs[v]]]
        psi = np.einsum(*ops, list(range(gg.nv)), optimize=True)
        psi = psi / np.linalg.norm(psi)
        E = 0.0
        for c, tops in terms:
            phi = psi
            for name, x in reversed(tops):
                phi = np.moveaxis(np.tensordot(O.SPIN_HALF[name], phi, axes=([1], [x])), 0, x)
            E += c * float(np.real(np.vdot(psi, phi)))
        return E
    g2, B = O.tebd(g, A, groups, beta=2.0, dbeta=0.2, maxdim=2, cutoff=1e-8)
    assert max(g2.edge_dims) <= 2
    assert energy(g2, B) < energy(g, A) - 1e-3
