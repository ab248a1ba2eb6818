"""Hand-written adjoints against reverse-mode autograd of the oracle and
against central finite differences (FP64).

Tolerances: the unrolled gradient reproduces autograd through the same T
sweeps to 1e-9 relative; the implicit (fixed-point) gradient matches autograd
unrolled to convergence to 1e-7 relative and a directional central finite
difference (h = 1e-4) to 1e-6 relative."""
import numpy as np
import pytest

import bp_oracle as O
import gbtn
from gbtn.operators import HEISENBERG

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
import bp_autograd as AG  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _lib(lib_built):
    yield


def pair(Lx, Ly, chi, seed):
    g = O.square_lattice(Lx, Ly, chi=chi)
    A = O.random_network(g, seed, unit_norm=True)
    tn = gbtn.TensorNetwork(g.nv, g.edges, g.site_dims, g.edge_dims, [a.copy() for a in A])
    return tn, g, A


def flat(ts):
    return np.concatenate([np.asarray(t).reshape(-1, order="F") for t in ts])


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def test_energy_matches_oracle():
    tn, g, A = pair(4, 3, 3, 2)
    bpc = gbtn.BeliefPropagationCache(tn).update(maxiter=200, tol=1e-15, schedule="parallel")
    m = bpc.messages()
    ref = O.expect2(g, A, m, AG.heisenberg_matrix()).sum()
    assert bpc.energy2(HEISENBERG) == pytest.approx(ref, rel=1e-12)


def test_unrolled_gradient_matches_autograd():
    tn, g, A = pair(3, 3, 2, 7)
    T = 12
    E_ref, G_ref = AG.energy_and_grad(g, A, T)
    bpc = gbtn.BeliefPropagationCache(tn)
    for ck in (0, 1, 5):  # sqrt(T), every sweep, and a ragged last segment
        E, G = bpc.energy2_grad(HEISENBERG, mode="unrolled", unroll=T, checkpoint=ck)
        assert E == pytest.approx(E_ref, rel=1e-12)
        assert rel(flat(G), flat(G_ref)) < 1e-9


def test_implicit_gradient_matches_converged_autograd():
    tn, g, A = pair(4, 3, 2, 11)
    E_ref, G_ref = AG.energy_and_grad(g, A, 120)
    bpc = gbtn.BeliefPropagationCache(tn).update(maxiter=400, schedule="parallel")
    E, G = bpc.energy2_grad(HEISENBERG, mode="implicit", tol=1e-13)
    assert E == pytest.approx(E_ref, rel=1e-10)
    assert rel(flat(G), flat(G_ref)) < 1e-7
    assert bpc.adjoint_residual <= 1e-13


def test_implicit_gradient_vs_finite_differences_8x8_chi3():
    tn, g, A = pair(8, 8, 3, 5)
    bpc = gbtn.BeliefPropagationCache(tn).update(maxiter=500, schedule="parallel")
    E, G = bpc.energy2_grad(HEISENBERG, mode="implicit", tol=1e-13)
    rng = np.random.default_rng(3)
    # unit-norm direction per site, like the tensors: the step is h relative
    D = [d / np.linalg.norm(d) for d in (rng.standard_normal(a.shape) for a in A)]
    h = 1e-4

    def energy_at(ts):
        net = gbtn.TensorNetwork(g.nv, g.edges, g.site_dims, g.edge_dims, ts)
        b = gbtn.BeliefPropagationCache(net).update(maxiter=500, schedule="parallel")
        return b.energy2(HEISENBERG)

    fd = (energy_at([a + h * d for a, d in zip(A, D)]) - energy_at([a - h * d for a, d in zip(A, D)])) / (2 * h)
    an = float(np.dot(flat(G), flat(D)))
    assert an == pytest.approx(fd, rel=1e-6)


def test_vjp_is_linear_and_matches_energy_gradient_split():
    tn, g, A = pair(3, 3, 2, 4)
    bpc = gbtn.BeliefPropagationCache(tn).update(maxiter=300, schedule="parallel")
    rng = np.random.default_rng(8)
    c1 = rng.standard_normal(bpc.n_message)
    c2 = rng.standard_normal(bpc.n_message)
    g1 = flat(bpc.vjp(c1))
    g2 = flat(bpc.vjp(c2))
    g12 = flat(bpc.vjp(2.0 * c1 - 0.5 * c2))
    np.testing.assert_allclose(g12, 2.0 * g1 - 0.5 * g2, rtol=1e-9, atol=1e-12)


def test_torch_autograd_binding():
    from gbtn.autograd import BPEnergy
    tn, g, A = pair(3, 3, 2, 9)
    ts = [torch.tensor(a, requires_grad=True) for a in A]
    E = BPEnergy.apply(tn, HEISENBERG, dict(maxiter=300, schedule="parallel"), *ts)
    E.backward()
    E_ref, G_ref = AG.energy_and_grad(g, A, 150)
    assert float(E) == pytest.approx(E_ref, rel=1e-10)
    assert rel(flat([t.grad.numpy() for t in ts]), flat(G_ref)) < 1e-7


def _complex_energy(g, A, msgs):
    """Re sum_e sum_t c_t <O_t (x) O_t>_e of the oracle (Heisenberg terms)."""
    return float(np.real(sum(c * np.sum(O.expect2(g, A, msgs, np.kron(op, op))) for c, op in HEISENBERG)))


@pytest.mark.parametrize("mode", ["implicit", "unrolled"])
def test_complex_energy_gradient_vs_finite_differences(mode):
    """Complex tensors: E = Re sum of the two-site terms, gradient dE/dRe + i
    dE/dIm; along a complex direction D, (E(A + hD) - E(A - hD)) / 2h =
    Re <G, D>.  Implicit: E at the converged messages (250 oracle sweeps);
    unrolled: E after exactly T sweeps from identity messages."""
    g = O.square_lattice(3, 3, chi=2)
    A = O.random_network(g, 41, dtype=np.complex128, unit_norm=True)
    tn = gbtn.TensorNetwork(g.nv, g.edges, g.site_dims, g.edge_dims, [a.copy() for a in A])
    sweeps = 250 if mode == "implicit" else 12
    bpc = gbtn.BeliefPropagationCache(tn)
    if mode == "implicit":
        bpc.update(maxiter=sweeps, schedule="parallel")
        E, G = bpc.energy2_grad(HEISENBERG, mode="implicit", tol=1e-13)
    else:
        E, G = bpc.energy2_grad(HEISENBERG, mode="unrolled", unroll=sweeps, checkpoint=5)

    def energy_at(ts):
        m, _, _ = O.bp_update(g, ts, O.identity_messages(g, dtype=np.complex128), maxiter=sweeps, schedule="parallel")
        return _complex_energy(g, ts, m)

    assert E == pytest.approx(energy_at(A), rel=1e-10, abs=1e-12)
    rng = np.random.default_rng(12)
    D = []
    for a in A:
        d = rng.standard_normal(a.shape) + 1j * rng.standard_normal(a.shape)
        D.append(d / np.linalg.norm(d))
    h = 1e-5
    fd = (energy_at([a + h * d for a, d in zip(A, D)]) - energy_at([a - h * d for a, d in zip(A, D)])) / (2 * h)
    an = float(np.real(np.vdot(flat(G), flat(D))))
    assert an == pytest.approx(fd, rel=1e-6, abs=1e-9)
    bpc.close()


@pytest.mark.parametrize("ck", [0, 1, 5])
def test_unrolled_message_vjp_matches_autograd(ck):
    """gbtn_bp_vjp in UNROLLED mode: L = sum_de <C_de, m_de> of the messages
    after T Jacobi sweeps from identity messages, dL/dA against reverse-mode
    autograd through the same sweeps of the oracle (1e-9 relative)."""
    tn, g, A = pair(3, 3, 2, 13)
    T = 9
    rng = np.random.default_rng(4)
    Cs = [rng.standard_normal((g.edge_dims[de // 2],) * 2) for de in range(2 * g.ne)]
    At = [torch.tensor(a, dtype=torch.float64, requires_grad=True) for a in A]
    msgs = AG.sweeps(g, At, T)
    L = sum(torch.sum(torch.tensor(c) * m) for c, m in zip(Cs, msgs))
    L.backward()
    G_ref = [a.grad.numpy() for a in At]
    bpc = gbtn.BeliefPropagationCache(tn)
    G = bpc.vjp(Cs, mode="unrolled", unroll=T, checkpoint=ck)
    assert rel(flat(G), flat(G_ref)) < 1e-9
    # the sweeps' final messages are left in the cache
    m_ref = [m.detach().numpy() for m in msgs]
    assert max(float(np.max(np.abs(a - b))) for a, b in zip(bpc.messages(), m_ref)) < 1e-12
    bpc.close()
