"""Hand-written adjoints of the BP log-norm and of one-site expectation values
against central finite differences of the FP64 oracle.

The value side follows logscalar (abstractbeliefpropagationcache.jl:397-408)
and expect (expect.jl:5-19); the reference has no derivative of either, so the
gradient is pinned by differentiating the oracle numerically: for a unit-norm
direction D per site, (f(A + hD) - f(A - hD)) / 2h with f evaluated at the
oracle's converged BP fixed point (the C restatement of the parallel sweep,
run to its rounding floor).  Central differences with h = 1e-5 carry a
truncation error ~h^2 and a rounding error ~1e-16 |f| / h, both below 1e-9
relative here; the test asks for 1e-6 relative, the tolerance of the energy
gradient's finite-difference test."""
import numpy as np
import pytest

import bp_oracle as O
import build_oracle
import gbtn

pytestmark = pytest.mark.gpu

H = 1e-5
RTOL = 1e-6
SWEEPS = 400  # oracle sweeps: the mean diff reaches its floor well before


@pytest.fixture(scope="module", autouse=True)
def _lib(lib_built):
    yield


def converged(g, A):
    m0 = O.flatten_messages(g, O.identity_messages(g))
    mc, _, _ = build_oracle.run(g, O.flatten_tensors(A), m0, "parallel", None, SWEEPS)
    return O.unflatten_messages(g, mc)


def oracle_logscalar(g, A):
    return float(np.real(O.logscalar(g, A, A, converged(g, A))))


def oracle_expect_sum(g, A, op):
    return float(np.sum(O.expect1(g, A, converged(g, A), op)))


def flat(ts):
    return np.concatenate([np.asarray(t).reshape(-1, order="F") for t in ts])


def directional_fd(f, A, D):
    plus = f([a + H * d for a, d in zip(A, D)])
    minus = f([a - H * d for a, d in zip(A, D)])
    return (plus - minus) / (2 * H)


def unit_directions(A, seed):
    rng = np.random.default_rng(seed)
    return [d / np.linalg.norm(d) for d in (rng.standard_normal(a.shape) for a in A)]


def cache(g, A):
    """Every sweep runs (no tolerance): a mean message diff of 1e-15 still
    leaves ~3e-8 in the messages (the diff is quadratic in the error), which
    the log-norm, stationary at the fixed point, does not see but <O> does."""
    tn = gbtn.TensorNetwork(g.nv, g.edges, g.site_dims, g.edge_dims, [a.copy() for a in A])
    return gbtn.BeliefPropagationCache(tn).update(maxiter=SWEEPS, schedule="parallel")


CASES = {
    "grid4x3_chi2": lambda: O.square_lattice(4, 3, chi=2),
    "grid3x3_uneven": lambda: O.square_lattice(
        3, 3, edge_dims=[int(x) for x in np.random.default_rng(2).integers(1, 5, size=O.square_lattice(3, 3).ne)]),
    "tree8_d3": lambda: O.random_tree(8, 4, chi=3, d=3),
}


@pytest.mark.parametrize("case", list(CASES))
def test_logscalar_gradient_matches_finite_differences(case):
    g = CASES[case]()
    A = O.random_network(g, 21, unit_norm=True)
    bpc = cache(g, A)
    val, G = bpc.logscalar_grad(tol=1e-14)
    assert val == pytest.approx(oracle_logscalar(g, A), rel=1e-11, abs=1e-11)
    assert val == pytest.approx(float(np.real(bpc.logscalar())), rel=1e-12, abs=1e-12)
    for seed in (1, 2):
        D = unit_directions(A, seed)
        fd = directional_fd(lambda ts: oracle_logscalar(g, ts), A, D)
        an = float(np.dot(flat(G), flat(D)))
        assert an == pytest.approx(fd, rel=RTOL, abs=1e-9), (case, seed)
    assert bpc.grad_residual <= 1e-14
    bpc.close()


@pytest.mark.parametrize("case", ["grid4x3_chi2", "tree8_d3"])
def test_expect_sum_gradient_matches_finite_differences(case):
    g = CASES[case]()
    A = O.random_network(g, 22, unit_norm=True)
    d = g.site_dims[0]
    op = np.diag(np.arange(d, dtype=float) - (d - 1) / 2) if d != 2 else O.SZ
    op = op + 0.3 * np.eye(d, k=1)  # not symmetric: the ket and bra slots differ
    bpc = cache(g, A)
    val, G = bpc.expect_sum_grad(op, tol=1e-14)
    assert val == pytest.approx(oracle_expect_sum(g, A, op), rel=1e-10, abs=1e-12)
    for seed in (3, 4):
        D = unit_directions(A, seed)
        fd = directional_fd(lambda ts: oracle_expect_sum(g, ts, op), A, D)
        an = float(np.dot(flat(G), flat(D)))
        assert an == pytest.approx(fd, rel=RTOL, abs=1e-9), (case, seed)
    bpc.close()


def test_batched_gradients_are_per_network():
    """Two networks in one plan: the values per network, the gradient of the
    sum equal to the single-network gradients side by side."""
    g1, g2 = O.square_lattice(3, 3, chi=2), O.square_lattice(2, 4, chi=3)
    A1, A2 = O.random_network(g1, 5, unit_norm=True), O.random_network(g2, 6, unit_norm=True)
    t1 = gbtn.TensorNetwork(g1.nv, g1.edges, g1.site_dims, g1.edge_dims, [a.copy() for a in A1])
    t2 = gbtn.TensorNetwork(g2.nv, g2.edges, g2.site_dims, g2.edge_dims, [a.copy() for a in A2])
    both = gbtn.BeliefPropagationCache(gbtn.disjoint_union([t1, t2])).update(maxiter=SWEEPS, schedule="parallel")
    vals, G = both.logscalar_grad(tol=1e-14)
    v1, G1 = cache(g1, A1).logscalar_grad(tol=1e-14)
    v2, G2 = cache(g2, A2).logscalar_grad(tol=1e-14)
    np.testing.assert_allclose(vals, [v1, v2], rtol=1e-11)
    np.testing.assert_allclose(flat(G), np.concatenate([flat(G1), flat(G2)]), rtol=1e-8, atol=1e-11)
    evals, _ = both.expect_sum_grad(O.SZ, tol=1e-14)
    np.testing.assert_allclose(evals, [oracle_expect_sum(g1, A1, O.SZ), oracle_expect_sum(g2, A2, O.SZ)],
                               rtol=1e-9, atol=1e-12)
    both.close()


def test_scalar_gradients_refused_where_they_have_no_path():
    g = O.square_lattice(2, 2, chi=2)
    gl = O.square_lattice(2, 2, chi=10)
    bl = gbtn.BeliefPropagationCache(gbtn.TensorNetwork(gl.nv, gl.edges, gl.site_dims, gl.edge_dims,
                                                        O.random_network(gl, 1)))
    with pytest.raises(gbtn.Unsupported):
        bl.expect_sum_grad(O.SZ)
    bl.close()
    A = O.random_network(g, 2)
    bs = gbtn.BeliefPropagationCache(gbtn.TensorNetwork(g.nv, g.edges, g.site_dims, g.edge_dims, A),
                                     bra=[a.copy() for a in A])
    with pytest.raises(gbtn.InvalidArgument):
        bs.logscalar_grad()
    bs.close()


# ---- complex tensors -----------------------------------------------------------
# The loss is real (Re logscalar = sum log|D_v| - sum log|z_e|, Re sum <O_v>);
# the gradient G is dL/dRe A + i dL/dIm A, so for a complex direction D,
# (L(A + hD) - L(A - hD)) / 2h = Re <G, D> = Re sum conj(G) D.  The oracle is the
# NumPy restatement in complex arithmetic (the C port is real), run to its
# fixed point; every value here is invariant under the phases of the messages.

CSWEEPS = 250


def converged_c(g, A):
    msgs, _, _ = O.bp_update(g, A, O.identity_messages(g, dtype=np.complex128), maxiter=CSWEEPS, schedule="parallel")
    return msgs


def complex_directions(A, seed):
    rng = np.random.default_rng(seed)
    out = []
    for a in A:
        d = rng.standard_normal(a.shape) + 1j * rng.standard_normal(a.shape)
        out.append(d / np.linalg.norm(d))
    return out


def ccache(g, A):
    tn = gbtn.TensorNetwork(g.nv, g.edges, g.site_dims, g.edge_dims, [a.copy() for a in A])
    return gbtn.BeliefPropagationCache(tn).update(maxiter=CSWEEPS, schedule="parallel")


def re_dot(G, D):
    return float(np.real(np.vdot(flat(G), flat(D))))


@pytest.mark.parametrize("case", ["grid4x3_chi2", "tree8_d3"])
def test_complex_logscalar_gradient_matches_finite_differences(case):
    g = CASES[case]()
    A = O.random_network(g, 31, dtype=np.complex128, unit_norm=True)
    bpc = ccache(g, A)
    val, G = bpc.logscalar_grad(tol=1e-13)
    f = lambda ts: float(np.real(O.logscalar(g, ts, ts, converged_c(g, ts))))
    assert val == pytest.approx(f(A), rel=1e-10, abs=1e-10)
    D = complex_directions(A, 5)
    fd = directional_fd(f, A, D)
    assert re_dot(G, D) == pytest.approx(fd, rel=RTOL, abs=1e-9)
    assert bpc.grad_residual <= 1e-13
    bpc.close()


@pytest.mark.parametrize("case", ["tree8_d3", "grid4x3_chi2"])
def test_complex_expect_gradient_with_a_non_hermitian_operator(case):
    """On the loopy grid one sweep moves every converged message by a phase
    (complex BP does not settle them), which the adjoint accounts for; on the
    tree the messages are exact after a few sweeps."""
    g = CASES[case]()
    A = O.random_network(g, 32, dtype=np.complex128, unit_norm=True)
    rng = np.random.default_rng(9)
    d = g.site_dims[0]
    op = rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d))
    bpc = ccache(g, A)
    val, G = bpc.expect_sum_grad(op, tol=1e-13)
    f = lambda ts: float(np.real(np.sum(O.expect1(g, ts, converged_c(g, ts), op))))
    assert val == pytest.approx(f(A), rel=1e-10, abs=1e-12)
    D = complex_directions(A, 6)
    assert re_dot(G, D) == pytest.approx(directional_fd(f, A, D), rel=RTOL, abs=1e-9)
    bpc.close()


def test_complex_vjp_of_a_phase_invariant_message_functional():
    """L(m) = sum_e log|<m_e, m_ebar>| at the fixed point: its message cotangent
    conj(m_ebar / z_e) (and the reverse) through gbtn_bp_vjp against finite
    differences of the same functional of the oracle's fixed point."""
    g = CASES["grid4x3_chi2"]()
    A = O.random_network(g, 33, dtype=np.complex128, unit_norm=True)
    bpc = ccache(g, A)
    m = bpc.messages()
    cot = []
    for de in range(2 * g.ne):
        other = m[de ^ 1]
        z = np.sum(m[de & ~1] * m[de | 1])
        cot.append(np.conj(other / z))
    G = bpc.vjp(cot, tol=1e-13)

    def f(ts):
        mm = converged_c(g, ts)
        return float(sum(np.log(abs(np.sum(mm[2 * e] * mm[2 * e + 1]))) for e in range(g.ne)))

    D = complex_directions(A, 7)
    assert re_dot(G, D) == pytest.approx(directional_fd(f, A, D), rel=RTOL, abs=1e-9)
    bpc.close()
