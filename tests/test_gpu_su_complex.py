"""Simple update with complex gates and tensors (ComplexF64) against the
oracle's restatement of simple_update_bp (src/apply.jl:33-95), including the
reference's own case (test/test_apply.jl): a random unitary two-site gate on a
real state with simple-BP environments, maxdim = chi, normalize = true, where
the truncation error is nonzero and the fidelity with the exact application
positive.  Gauge-invariant comparisons: kept singular values (1e-10
relative), truncation errors, bond dimensions, and the contracted state up to
a global phase (|<a, b>| = 1 to 1e-9)."""
import numpy as np
import pytest

import bp_oracle as O
import gbtn

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib(lib_built):
    yield


def state(g, A):
    ops = []
    for v in range(g.nv):
        ops += [A[v], [v] + [20 + e for e in g.legs[v]]]
    psi = np.einsum(*ops, list(range(g.nv)), optimize=True)
    return psi / np.linalg.norm(psi)


def overlap(a, b):
    return abs(np.vdot(a.ravel(), b.ravel()))


def random_unitary(seed, n=4):
    rng = np.random.default_rng(seed)
    Z = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    Q, R = np.linalg.qr(Z)
    return Q * (np.diag(R) / np.abs(np.diag(R)))


def oracle_gate(g, A, gate, e, envs=None, maxdim=None, cutoff=None, normalize=True):
    u, v = g.edges[e]
    pu, pv = g.legs[u].index(e), g.legs[v].index(e)
    eu, ev = {}, {}
    if envs is not None:
        eu = {1 + p: envs[g.directed(f, g.other(u, f))] for p, f in enumerate(g.legs[u]) if f != e}
        ev = {1 + p: envs[g.directed(f, g.other(v, f))] for p, f in enumerate(g.legs[v]) if f != e}
    Au, Av, S, te = O.simple_update(gate, A[u], A[v], pu, pv, eu, ev, maxdim=maxdim, cutoff=cutoff)
    if normalize:
        Au, Av = Au / np.linalg.norm(Au), Av / np.linalg.norm(Av)
    B = list(A)
    B[u], B[v] = Au, Av
    g2 = O.Graph(g.nv, g.edges, g.site_dims, list(g.edge_dims), [list(l) for l in g.legs])
    g2.edge_dims[e] = Au.shape[pu + 1]
    return g2, B, S, te


def gpu_net(g, A):
    return gbtn.TensorNetwork(g.nv, g.edges, g.site_dims, g.edge_dims, [a.copy() for a in A])


@pytest.mark.parametrize("e", [1, 5])
def test_random_unitary_on_a_real_state_with_bp_environments(e):
    g = O.square_lattice(3, 3, chi=2)
    A = O.random_network(g, 1234)
    envs = gbtn.BeliefPropagationCache(gpu_net(g, A)).update(maxiter=20).messages()
    U = random_unitary(e)
    g2, B, S, te = oracle_gate(g, A, U, e, envs=envs, maxdim=2, cutoff=None)
    seen = {}
    out = gbtn.apply(U, gpu_net(g, A), e, envs=envs, maxdim=2, normalize=True,
                     callback=lambda **kw: seen.update(kw))
    assert out.is_complex
    np.testing.assert_allclose(seen["singular_values"], S, rtol=1e-10)
    assert seen["truncation_error"] == pytest.approx(te, rel=1e-8, abs=1e-14)
    assert seen["truncation_error"] != 0.0  # the reference's checks: truncation happened ...
    got = state(g2, out.tensors)
    assert overlap(got, state(g2, B)) == pytest.approx(1.0, abs=1e-9)
    exact = state(g, A)  # ... and the truncated state keeps a positive fidelity with the exact one
    ops = [exact, list(range(g.nv))]
    u, v = g.edges[e]
    psi_exact = np.einsum(exact, list(range(g.nv)), U.reshape(2, 2, 2, 2, order="F"), [20, 21, u, v],
                          [20 if k == u else 21 if k == v else k for k in range(g.nv)])
    assert overlap(got, psi_exact / np.linalg.norm(psi_exact)) > 0.0


def test_complex_state_and_gate_sequence_without_environments():
    g = O.square_lattice(3, 3, chi=2)
    A = O.random_network(g, 7, dtype=np.complex128)
    rng = np.random.default_rng(3)
    H = rng.standard_normal((4, 4)) + 1j * rng.standard_normal((4, 4))
    H = H + H.conj().T
    w, V = np.linalg.eigh(H)
    gates = [random_unitary(11), (V * np.exp(-1j * 0.3 * w)) @ V.conj().T, random_unitary(12),
             (V * np.exp(-0.2 * w)) @ V.conj().T]
    order = [0, 5, 7, 2]
    st = gbtn.SimpleUpdateState(gpu_net(g, A), chi_max=4)
    te_g, sv = st.apply(gates, order, maxdim=3, cutoff=1e-12, normalize=True)
    gg, B = g, list(A)
    for k, e in enumerate(order):
        gg, B, S, te = oracle_gate(gg, B, gates[k], e, maxdim=3, cutoff=1e-12)
        np.testing.assert_allclose(sv[k][:len(S)], S, rtol=1e-9)
        assert te_g[k] == pytest.approx(te, rel=1e-7, abs=1e-13)
    assert st.edge_dims() == gg.edge_dims
    assert overlap(state(gg, st.network().tensors), state(gg, B)) == pytest.approx(1.0, abs=1e-9)


@pytest.mark.parametrize("e", [2, 6])
def test_rank_deficient_complex_theta_keeps_exactly_its_rank(e):
    # a product of single-site unitaries on a bond of dimension 4 that carries
    # rank 2: two values kept, the noise columns discarded by the cutoff
    g = O.square_lattice(3, 3, chi=4)
    A = O.random_network(g, 31, dtype=np.complex128)
    u = g.edges[e][0]
    pu = g.legs[u].index(e)
    rng = np.random.default_rng(e)
    P = rng.standard_normal((2, 4)) + 1j * rng.standard_normal((2, 4))
    A[u] = np.moveaxis(np.tensordot(A[u], P.conj().T @ P, axes=([1 + pu], [0])), -1, 1 + pu)
    gate = np.kron(random_unitary(20 + e, 2), random_unitary(30 + e, 2))
    g2, B, S, te = oracle_gate(g, A, gate, e, maxdim=4, cutoff=1e-12)
    assert g2.edge_dims[e] == 2
    st = gbtn.SimpleUpdateState(gpu_net(g, A), chi_max=4)
    te_g, sv = st.apply(gate, [e], maxdim=4, cutoff=1e-12, normalize=True)
    assert st.edge_dims()[e] == 2
    np.testing.assert_allclose(sv[0][:2], S, rtol=1e-10)
    assert te_g[0] == pytest.approx(te, abs=1e-14)
    assert overlap(state(g2, st.network().tensors), state(g2, B)) == pytest.approx(1.0, abs=1e-9)


def test_complex_gates_need_a_complex_state_and_fit_the_kernel():
    g = O.square_lattice(3, 3, chi=2)
    A = O.random_network(g, 2)
    st = gbtn.SimpleUpdateState(gpu_net(g, A), chi_max=4)  # a real state
    with pytest.raises(ValueError):
        st.apply(random_unitary(1), [0], maxdim=2)
    big = O.square_lattice(3, 3, chi=8)  # centre tensor 2 * 8^4 = 8192 complex entries
    Ab = O.random_network(big, 3, dtype=np.complex128)
    stb = gbtn.SimpleUpdateState(gpu_net(big, Ab), chi_max=8)
    with pytest.raises(gbtn.Unsupported):
        stb.apply(random_unitary(2), [big.legs[4][0]], maxdim=8)
