"""Hand-written adjoint of the simple update (gbtn_su_apply_vjp) against
central finite differences of the oracle's simple_update_bp restatement
(src/apply.jl:33-95; the reference itself has no derivative).

The factors a gate leaves are gauge dependent (a sign per kept singular
vector, paired across the bond), so the loss is gauge invariant: L = <W, psi>
for a fixed random W and psi the contracted state vector of the network after
the gates.  The test computes dL/d(tensors after the gates) by contracting W
with the other tensors, pulls it back through the GPU adjoint, and compares
the directional derivative <G, D> with (L(A + hD) - L(A - hD)) / 2h of the
oracle for unit directions D (h = 1e-5: truncation ~h^2 and rounding
~1e-16 / h, both below 1e-9 relative here); 1e-6 relative, the tolerance of
the BP gradients' finite-difference tests.  The same for the gate matrices."""
import numpy as np
import pytest

import bp_oracle as O
import gbtn
from test_gpu_su import gpu_net, oracle_gate, random_gate

pytestmark = pytest.mark.gpu

H = 1e-5
RTOL = 1e-6


@pytest.fixture(scope="module", autouse=True)
def _lib(lib_built):
    yield


def psi(g, A):
    ops, lid = [], {e: 20 + e for e in range(g.ne)}
    for v in range(g.nv):
        ops += [A[v], [v] + [lid[e] for e in g.legs[v]]]
    return np.einsum(*ops, list(range(g.nv)), optimize=True)


def psi_cotangents(g, A, W):
    """d<W, psi>/dA_v for every v: W contracted with every other tensor."""
    lid = {e: 20 + e for e in range(g.ne)}
    out = []
    for v in range(g.nv):
        ops = [W, list(range(g.nv))]
        for w in range(g.nv):
            if w != v:
                ops += [A[w], [w] + [lid[e] for e in g.legs[w]]]
        out.append(np.einsum(*ops, [v] + [lid[e] for e in g.legs[v]], optimize=True))
    return out


def oracle_layers(g, A, layers, envs, maxdim, cutoff, normalize):
    """Apply layers[i] = [(edge, gate), ...] in order with the oracle."""
    for layer in layers:
        for e, gate in layer:
            g, A, _, _ = oracle_gate(g, A, gate, e, envs=envs, maxdim=maxdim, cutoff=cutoff, normalize=normalize)
    return g, A


def unit(rng, shapes):
    d = [rng.standard_normal(s) for s in shapes]
    nrm = np.sqrt(sum(np.sum(x * x) for x in d))
    return [x / nrm for x in d]


def check_case(g, A, layers, envs=None, maxdim=3, cutoff=None, normalize=False, seed=0):
    rng = np.random.default_rng(seed)
    g_out, A_out = oracle_layers(g, A, layers, envs, maxdim, cutoff, normalize)
    W = rng.standard_normal(psi(g_out, A_out).shape)
    loss = lambda AA, lay: float(np.sum(W * psi(*oracle_layers(g, AA, lay, envs, maxdim, cutoff, normalize))))

    st = gbtn.SimpleUpdateState(gpu_net(g, A), chi_max=4)
    edges = [e for layer in layers for e, _ in layer]
    gates = [gt for layer in layers for _, gt in layer]
    _, _, pull = st.apply_with_pullback(gates, edges, envs=envs, maxdim=maxdim, cutoff=cutoff, normalize=normalize)
    out = st.network()
    assert list(out.edge_dims) == list(g_out.edge_dims)
    cot = psi_cotangents(g_out, out.tensors, W)
    G, Gg, _ = pull(cot)
    assert [x.shape for x in G] == [a.shape for a in A]
    # the state is where apply left it
    np.testing.assert_array_equal(np.concatenate([t.ravel() for t in st.network().tensors]),
                                  np.concatenate([t.ravel() for t in out.tensors]))
    for s in range(2):
        D = unit(rng, [a.shape for a in A])
        fd = (loss([a + H * d for a, d in zip(A, D)], layers) - loss([a - H * d for a, d in zip(A, D)], layers)) / (2 * H)
        an = sum(float(np.sum(x * d)) for x, d in zip(G, D))
        assert an == pytest.approx(fd, rel=RTOL, abs=1e-9), ("tensors", s)
    # gate cotangents: a direction per gate
    Dg = unit(rng, [gt.shape for gt in gates])

    def shifted(sgn):
        it = iter(Dg)
        return [[(e, gt + sgn * H * next(it)) for e, gt in layer] for layer in layers]
    fd = (loss(A, shifted(1)) - loss(A, shifted(-1))) / (2 * H)
    an = sum(float(np.sum(x * d)) for x, d in zip(Gg, Dg))
    assert an == pytest.approx(fd, rel=RTOL, abs=1e-9), "gates"
    st.close()


@pytest.mark.parametrize("normalize", [False, True])
@pytest.mark.parametrize("e", [0, 5])
def test_single_gate_adjoint(e, normalize):
    """One gate, truncated to maxdim = 3 of up to 8 singular values (the
    discarded ones enter the adjoint), without environments."""
    g = O.square_lattice(3, 3, chi=2)
    A = O.random_network(g, 40 + e)
    check_case(g, A, [[(e, random_gate(e))]], maxdim=3, normalize=normalize, seed=e)


def test_gate_layer_with_bp_environments():
    """A checkerboard layer of vertex-disjoint gates in one batch, with the
    BP messages of the state as (constant) environments, a cutoff and
    normalisation (BP-gauged TEBD, tebd.jl with envs)."""
    g = O.square_lattice(3, 3, chi=2)
    A = O.random_network(g, 7, unit_norm=True)
    envs, _, _ = O.bp_update(g, A, O.identity_messages(g), maxiter=200, schedule="parallel")
    layer = [(e, random_gate(10 + e)) for e in (0, 5, 10, 4)]
    assert len({v for e, _ in layer for v in g.edges[e]}) == 8  # disjoint
    check_case(g, A, [layer], envs=envs, maxdim=3, cutoff=1e-10, normalize=True, seed=3)


def test_pullback_through_a_gate_sequence():
    """Two layers sharing vertices: the pullback restores each batch's saved
    input state and runs the adjoints in reverse."""
    g = O.square_lattice(3, 2, chi=2)
    A = O.random_network(g, 11)
    layers = [[(0, random_gate(1)), (6, random_gate(2))], [(1, random_gate(3))], [(0, random_gate(4))]]
    check_case(g, A, layers, maxdim=4, normalize=True, seed=5)


def test_adjoint_refusals():
    g = O.square_lattice(2, 2, chi=2)
    A = O.random_network(g, 3)
    st = gbtn.SimpleUpdateState(gpu_net(g, A), chi_max=4)
    cot = [np.zeros_like(a) for a in A]
    with pytest.raises(gbtn.InvalidArgument, match="disjoint"):
        st.apply_vjp([random_gate(1), random_gate(2)], [0, 1], g.edge_dims, cot)
    with pytest.raises(gbtn.InvalidArgument):  # a truncation that does not match the gate's
        st.apply_vjp(random_gate(1), [0], [1] + list(g.edge_dims[1:]), cot, maxdim=4)
    st.close()
    gc = O.square_lattice(2, 2, chi=2)
    Ac = O.random_network(gc, 3, dtype=np.complex128)
    sc = gbtn.SimpleUpdateState(gpu_net(gc, Ac), chi_max=4)
    with pytest.raises(gbtn.Unsupported):
        sc.apply_vjp(random_gate(1), [0], gc.edge_dims, [np.zeros_like(a) for a in Ac])
    sc.close()


def test_bp_energy_gradient_through_a_tebd_step():
    """d<H>_BP/dA0 through one Trotter step: A0 -> four checkerboard layers of
    Heisenberg gates exp(-0.1 h) (simple update, maxdim 4, normalised) -> A1
    -> BP energy.  The BP adjoint gives dE/dA1 (implicit, at the converged
    messages), the simple-update pullback carries it to A0; against central
    differences of the oracle (its simple update, then its BP fixed point and
    two-site energy)."""
    torch = pytest.importorskip("torch")  # noqa: F841 (bp_autograd needs it)
    import bp_autograd as AG
    from gbtn.operators import HEISENBERG
    g = O.square_lattice(3, 3, chi=2)
    A = O.random_network(g, 17, unit_norm=True)
    hm = AG.heisenberg_matrix()
    w, U = np.linalg.eigh(hm)
    gate = (U * np.exp(-0.1 * w)) @ U.T
    colours = [[0, 5, 10], [2, 7, 11], [1, 3, 4], [6, 8, 9]]  # checkerboard classes of the 3x3 edges
    for c in colours:
        assert len({v for e in c for v in g.edges[e]}) == 2 * len(c)
    layers = [[(e, gate) for e in c] for c in colours]
    st = gbtn.SimpleUpdateState(gpu_net(g, A), chi_max=4)
    edges = [e for c in colours for e in c]
    _, _, pull = st.apply_with_pullback(gate, edges, maxdim=4, normalize=True)
    net1 = st.network()
    bpc = gbtn.BeliefPropagationCache(net1).update(maxiter=500, schedule="parallel")
    E, G1 = bpc.energy2_grad(HEISENBERG, mode="implicit", tol=1e-13)
    G0, Gg, _ = pull(G1)

    def energy(AA, gt=gate):
        lay = [[(e, gt) for e in c] for c in colours]
        g1, A1 = oracle_layers(g, AA, lay, None, 4, None, True)
        m, _, _ = O.bp_update(g1, A1, O.identity_messages(g1), maxiter=500, schedule="parallel")
        return float(np.sum(O.expect2(g1, A1, m, hm)))

    assert E == pytest.approx(energy(A), rel=1e-10)
    rng = np.random.default_rng(8)
    D = unit(rng, [a.shape for a in A])
    h = 1e-4
    fd = (energy([a + h * d for a, d in zip(A, D)]) - energy([a - h * d for a, d in zip(A, D)])) / (2 * h)
    an = sum(float(np.sum(x * d)) for x, d in zip(G0, D))
    assert an == pytest.approx(fd, rel=RTOL)
    # one shared gate: its cotangent is the sum over its applications
    Dg = rng.standard_normal(gate.shape)
    Dg /= np.linalg.norm(Dg)
    fdg = (energy(A, gate + h * Dg) - energy(A, gate - h * Dg)) / (2 * h)
    assert float(np.sum(Gg.sum(axis=0) * Dg)) == pytest.approx(fdg, rel=RTOL)
    bpc.close()
    st.close()


def test_batch_vjp_equals_the_taped_pullback():
    """gbtn_su_apply_vjp on one batch (host cotangents, explicit post
    dimensions) and the taped pullback give the same cotangents."""
    g = O.square_lattice(3, 3, chi=2)
    A = O.random_network(g, 23)
    edges = [0, 5, 10]
    gates = [random_gate(30 + e) for e in edges]
    envs, _, _ = O.bp_update(g, A, O.identity_messages(g), maxiter=100, schedule="parallel")
    st = gbtn.SimpleUpdateState(gpu_net(g, A), chi_max=4)
    _, _, pull = st.apply_with_pullback(gates, edges, envs=envs, maxdim=3, cutoff=1e-12, normalize=True)
    out = st.network()
    rng = np.random.default_rng(2)
    cot = [rng.standard_normal(t.shape) for t in out.tensors]
    G1, Gg1, E1 = pull(cot)
    st.set_state(gpu_net(g, A))
    G2, Gg2, E2 = st.apply_vjp(gates, edges, out.edge_dims, cot, envs=envs, maxdim=3, cutoff=1e-12, normalize=True)
    for a, b in zip(G1, G2):
        np.testing.assert_allclose(a, b, rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(Gg1, Gg2, rtol=1e-12, atol=1e-14)
    for a, b in zip(E1, E2):
        np.testing.assert_allclose(a, b, rtol=1e-12, atol=1e-14)
    G3, _, _ = pull(cot)  # a tape can be pulled back again
    for a, b in zip(G1, G3):
        np.testing.assert_array_equal(a, b)
    st.close()
    del pull  # the tape outlives nothing it needs


def test_environment_cotangents():
    """dL/d(envs) through the square-root and inverse-square-root environments
    (the eigen-decomposition's divided differences): against central
    differences of the oracle along symmetric directions of every message."""
    g = O.square_lattice(3, 3, chi=2)
    A = O.random_network(g, 9, unit_norm=True)
    envs, _, _ = O.bp_update(g, A, O.identity_messages(g), maxiter=300, schedule="parallel")
    layer = [(e, random_gate(20 + e)) for e in (0, 5, 10, 4)]
    rng = np.random.default_rng(6)
    g_out, A_out = oracle_layers(g, A, [layer], envs, 3, 1e-12, True)
    W = rng.standard_normal(psi(g_out, A_out).shape)
    st = gbtn.SimpleUpdateState(gpu_net(g, A), chi_max=4)
    _, _, pull = st.apply_with_pullback([gt for _, gt in layer], [e for e, _ in layer], envs=envs, maxdim=3,
                                        cutoff=1e-12, normalize=True)
    out = st.network()
    _, _, Eb = pull(psi_cotangents(g_out, out.tensors, W))
    assert len(Eb) == 2 * g.ne
    D = [rng.standard_normal(m.shape) for m in envs]
    D = [(d + d.T) / 2 for d in D]
    nrm = np.sqrt(sum(np.sum(d * d) for d in D))
    D = [d / nrm for d in D]

    def loss(ev):
        return float(np.sum(W * psi(*oracle_layers(g, A, [layer], ev, 3, 1e-12, True))))

    h = 1e-5
    fd = (loss([m + h * d for m, d in zip(envs, D)]) - loss([m - h * d for m, d in zip(envs, D)])) / (2 * h)
    an = sum(float(np.sum(x * d)) for x, d in zip(Eb, D))
    assert an == pytest.approx(fd, rel=RTOL, abs=1e-9)
    st.close()


def test_gradient_through_bp_gauged_gates():
    """BP-gauged simple update (tebd.jl with envs = the BP messages of the
    state): L(A) = <W, psi(apply(gates, A; envs = BP(A)))>.  dL/dA = the
    pullback's tensor cotangent plus the BP fixed point's VJP of its
    environment cotangent (gbtn_bp_vjp); against central differences of the
    oracle's BP and simple update."""
    g = O.square_lattice(3, 3, chi=2)
    A = O.random_network(g, 19, unit_norm=True)
    layer = [(e, random_gate(40 + e)) for e in (1, 3, 4, 10)]
    assert len({v for e, _ in layer for v in g.edges[e]}) == 8
    rng = np.random.default_rng(7)

    def fwd_oracle(AA):
        m, _, _ = O.bp_update(g, AA, O.identity_messages(g), maxiter=400, schedule="parallel")
        return oracle_layers(g, AA, [layer], m, 3, 1e-12, True)

    g_out, A_out = fwd_oracle(A)
    W = rng.standard_normal(psi(g_out, A_out).shape)
    tn = gpu_net(g, A)
    bpc = gbtn.BeliefPropagationCache(tn).update(maxiter=400, schedule="parallel")
    envs = bpc.messages()
    st = gbtn.SimpleUpdateState(tn, chi_max=4)
    _, _, pull = st.apply_with_pullback([gt for _, gt in layer], [e for e, _ in layer], envs=envs, maxdim=3,
                                        cutoff=1e-12, normalize=True)
    out = st.network()
    G, _, Eb = pull(psi_cotangents(g_out, out.tensors, W))
    Gbp = bpc.vjp(Eb, tol=1e-14)
    total = [a + b for a, b in zip(G, Gbp)]
    D = unit(rng, [a.shape for a in A])
    h = 1e-5
    loss = lambda AA: float(np.sum(W * psi(*fwd_oracle(AA))))
    fd = (loss([a + h * d for a, d in zip(A, D)]) - loss([a - h * d for a, d in zip(A, D)])) / (2 * h)
    an = sum(float(np.sum(x * d)) for x, d in zip(total, D))
    assert an == pytest.approx(fd, rel=RTOL, abs=1e-9)
    st.close()
    bpc.close()


@pytest.mark.parametrize("bp_envs,nsteps", [(False, 2), (True, 1)])
def test_tebd_pullback(bp_envs, nsteps):
    """tebd_with_pullback: a checkerboard Trotter evolution (Heisenberg gates
    exp(-0.1 h), maxdim 3, normalised), with BP-gauged environments or
    without, against central differences of the oracle doing the same steps
    (its BP before every class when gauged); the shared per-edge gates'
    cotangents too."""
    torch = pytest.importorskip("torch")  # noqa: F841 (bp_autograd needs it)
    import bp_autograd as AG
    g = O.square_lattice(3, 3, chi=2)
    A = O.random_network(g, 29, unit_norm=True)
    hm = AG.heisenberg_matrix()
    w, U = np.linalg.eigh(hm)
    gate = (U * np.exp(-0.1 * w)) @ U.T
    classes = [[0, 5, 10], [2, 7, 11], [1, 3, 4], [6, 8, 9]]

    def fwd_oracle(AA, gt=gate):
        gg = g
        for _ in range(nsteps):
            for cls in classes:
                envs = None
                if bp_envs:
                    envs, _, _ = O.bp_update(gg, AA, O.identity_messages(gg), maxiter=400, schedule="parallel")
                gg, AA = oracle_layers(gg, AA, [[(e, gt) for e in cls]], envs, 3, None, True)
        return gg, AA

    g_out, A_out = fwd_oracle(A)
    rng = np.random.default_rng(12)
    W = rng.standard_normal(psi(g_out, A_out).shape)
    st, pull = gbtn.tebd_with_pullback(gpu_net(g, A), lambda e: gate, classes, nsteps, maxdim=3, cutoff=None,
                                       chi_max=4, bp_envs=bp_envs, bp_maxiter=400, bp_tol=None)
    out = st.network()
    assert list(out.edge_dims) == list(g_out.edge_dims)
    G, dG = pull(psi_cotangents(g_out, out.tensors, W))
    D = unit(rng, [a.shape for a in A])
    h = 1e-5
    loss = lambda AA, gt=gate: float(np.sum(W * psi(*fwd_oracle(AA, gt))))
    fd = (loss([a + h * d for a, d in zip(A, D)]) - loss([a - h * d for a, d in zip(A, D)])) / (2 * h)
    assert sum(float(np.sum(x * d)) for x, d in zip(G, D)) == pytest.approx(fd, rel=RTOL, abs=1e-9)
    Dg = rng.standard_normal(gate.shape)
    Dg /= np.linalg.norm(Dg)
    fdg = (loss(A, gate + h * Dg) - loss(A, gate - h * Dg)) / (2 * h)
    assert float(np.sum(sum(dG.values()) * Dg)) == pytest.approx(fdg, rel=RTOL, abs=1e-9)
    st.close()
