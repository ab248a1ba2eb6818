"""Simple update (apply / tebd) on the GPU against the oracle's restatement of
simple_update_bp (src/apply.jl:33-95).

The factors of an SVD / QR are gauge dependent, so the comparisons use
gauge-invariant quantities: kept singular values and truncation errors
(1e-10 relative / 1e-12 absolute), bond dimensions (exact) and the contracted
state vector, normalised and up to a global sign (1e-9)."""
import numpy as np
import pytest

import bp_oracle as O
import gbtn

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib(lib_built):
    yield


def state(g, A):
    ops, lid = [], {e: 20 + e for e in range(g.ne)}
    for v in range(g.nv):
        ops += [A[v], [v] + [lid[e] for e in g.legs[v]]]
    psi = np.einsum(*ops, list(range(g.nv)), optimize=True)
    return psi / np.linalg.norm(psi)


def same_up_to_sign(a, b, tol):
    return min(np.max(np.abs(a - b)), np.max(np.abs(a + b))) < tol


def random_gate(seed, dt=0.3):
    rng = np.random.default_rng(seed)
    H = rng.standard_normal((4, 4))
    H = H + H.T
    w, U = np.linalg.eigh(H)
    return (U * np.exp(-dt * w)) @ U.T


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


@pytest.mark.parametrize("e", [0, 3, 7])
def test_single_gate_matches_oracle(e):
    g = O.square_lattice(3, 3, chi=2)
    A = O.random_network(g, 21)
    gate = random_gate(e)
    g2, B, S, te = oracle_gate(g, A, gate, e, maxdim=2, cutoff=1e-12)
    st = gbtn.SimpleUpdateState(gpu_net(g, A), chi_max=4)
    te_g, sv = st.apply(gate, [e], maxdim=2, cutoff=1e-12, normalize=True)
    assert st.edge_dims()[e] == g2.edge_dims[e]
    np.testing.assert_allclose(sv[0][:len(S)], S, rtol=1e-10)
    assert te_g[0] == pytest.approx(te, rel=1e-9, abs=1e-14)
    out = st.network()
    assert same_up_to_sign(state(g2, out.tensors), state(g2, B), 1e-9)


def rank2_bond(g, A, e, seed):
    """Make edge e (dimension 4) carry rank 2: A[u]'s leg on e is projected
    onto a random 2-dimensional subspace."""
    u = g.edges[e][0]
    pu = g.legs[u].index(e)
    P = np.random.default_rng(seed).standard_normal((2, g.edge_dims[e]))
    B = list(A)
    B[u] = np.moveaxis(np.tensordot(A[u], P.T @ P, axes=([1 + pu], [0])), -1, 1 + pu)
    return B


@pytest.mark.parametrize("e", [2, 6])
def test_rank_deficient_theta_keeps_exactly_its_rank(e):
    # a product gate on a bond of rank 2: theta (8 x 8 after the QRs) has rank
    # 2, so maxdim 4 with a relative cutoff keeps two values and discards the
    # six noise columns, which the FP64 Jacobi leaves unrotated among themselves
    g = O.square_lattice(3, 3, chi=4)
    A = rank2_bond(g, O.random_network(g, 77), e, e)
    rng = np.random.default_rng(10 + e)
    gate = np.kron(rng.standard_normal((2, 2)), rng.standard_normal((2, 2)))
    g2, B, S, te = oracle_gate(g, A, gate, e, maxdim=4, cutoff=1e-12)
    assert g2.edge_dims[e] == 2
    st = gbtn.SimpleUpdateState(gpu_net(g, A), chi_max=4)
    te_g, sv = st.apply(gate, [e], maxdim=4, cutoff=1e-12, normalize=True)
    assert st.edge_dims()[e] == 2
    np.testing.assert_allclose(sv[0][:2], S, rtol=1e-10)
    assert np.all(sv[0][2:] == 0.0)
    assert te_g[0] == pytest.approx(te, abs=1e-14)
    assert same_up_to_sign(state(g2, st.network().tensors), state(g2, B), 1e-9)


def test_single_gate_with_bp_environment():
    g = O.square_lattice(3, 3, chi=3)
    A = O.random_network(g, 5)
    bpc = gbtn.BeliefPropagationCache(gpu_net(g, A)).update(maxiter=100, tol=1e-15, schedule="parallel")
    envs = bpc.messages()
    e = 5
    gate = random_gate(3)
    g2, B, S, te = oracle_gate(g, A, gate, e, envs=envs, maxdim=3, cutoff=1e-10)
    st = gbtn.SimpleUpdateState(gpu_net(g, A), chi_max=6)
    te_g, sv = st.apply(gate, [e], envs=envs, maxdim=3, cutoff=1e-10, normalize=True)
    np.testing.assert_allclose(sv[0][:len(S)], S, rtol=1e-9)
    assert te_g[0] == pytest.approx(te, rel=1e-8, abs=1e-14)
    assert same_up_to_sign(state(g2, st.network().tensors), state(g2, B), 1e-8)


def test_tfim_tebd_matches_oracle():
    Lx, Ly, g_field, dt, steps, maxdim = 3, 3, 3.0, 0.05, 4, 4
    g = O.square_lattice(Lx, Ly, chi=1)
    plus = np.array([1.0, 1.0]) / np.sqrt(2)
    A = [plus.reshape((2,) + (1,) * len(g.legs[v])) for v in range(g.nv)]
    z = [len(l) for l in g.legs]
    order = [e for cls in gbtn.checkerboard_edges(Lx, Ly) for e in cls]
    gate_of = lambda e: gbtn.tfim_gate(dt, g_field, z[g.edges[e][0]], z[g.edges[e][1]])
    st = gbtn.SimpleUpdateState(gpu_net(g, A), chi_max=maxdim)
    gg, B = g, list(A)
    for _ in range(steps):
        te_g, _ = st.apply([gate_of(e) for e in order], order, maxdim=maxdim, cutoff=1e-10, normalize=True)
        tes = []
        for e in order:
            gg, B, S, te = oracle_gate(gg, B, gate_of(e), e, maxdim=maxdim, cutoff=1e-10)
            tes.append(te)
        np.testing.assert_allclose(te_g, tes, rtol=1e-6, atol=1e-13)
    assert st.edge_dims() == gg.edge_dims
    assert same_up_to_sign(state(gg, st.network().tensors), state(gg, B), 1e-9)


def test_tfim_20x20_chi8_runs_and_lowers_energy():
    # the shape of the TFIM benchmark (20x20, chi_max 8, cutoff 1e-10), 10 steps
    L, g_field, dt = 20, 3.0, 0.01
    tn = gbtn.square_lattice(L, L, chi=1)
    plus = np.array([1.0, 1.0]) / np.sqrt(2)
    tn.tensors = [plus.reshape((2,) + (1,) * len(tn.legs[v])) for v in range(tn.nv)]
    z = [len(l) for l in tn.legs]
    classes = gbtn.checkerboard_edges(L, L)
    st, te = gbtn.tebd(tn, lambda e: gbtn.tfim_gate(dt, g_field, z[tn.edges[e][0]], z[tn.edges[e][1]]), classes,
                       nsteps=10, maxdim=8, cutoff=1e-10, normalize=True, chi_max=8)
    dims = st.edge_dims()
    assert max(dims) <= 8 and min(dims) >= 1
    net = st.network()
    bpc = gbtn.BeliefPropagationCache(net).update(maxiter=100, tol=1e-12, schedule="parallel")
    x = bpc.expect(O.PX)
    zz = bpc.expect2(np.kron(O.PZ, O.PZ))
    e_site = (-zz.sum() - g_field * x.sum()) / tn.nv
    # the |+> product state has energy -g = -3 per site; imaginary time lowers it
    assert e_site < -3.0
    assert np.all(np.abs(x) <= 1 + 1e-12)


def test_bp_gauged_tebd_matches_oracle():
    # tebd with BP environments refreshed before every colour class, against the
    # oracle's BP fixed point and simple update with envs (apply.jl:33-95)
    Lx, Ly, g_field, dt, steps, maxdim = 3, 3, 3.0, 0.05, 2, 3
    g = O.square_lattice(Lx, Ly, chi=2)
    A = O.random_network(g, 17, unit_norm=True)
    z = [len(l) for l in g.legs]
    classes = gbtn.checkerboard_edges(Lx, Ly)
    gate_of = lambda e: gbtn.tfim_gate(dt, g_field, z[g.edges[e][0]], z[g.edges[e][1]])
    st, te_g = gbtn.tebd(gpu_net(g, A), gate_of, classes, nsteps=steps, maxdim=maxdim, cutoff=1e-12,
                         chi_max=6, bp_envs=True, bp_maxiter=300, bp_tol=None)
    gg, B = g, list(A)
    for _ in range(steps):
        tes = []
        for cls in classes:
            envs, _, _ = O.bp_update(gg, B, O.identity_messages(gg), maxiter=300, schedule="parallel")
            for e in cls:
                gg, B, S, t = oracle_gate(gg, B, gate_of(e), e, envs=envs, maxdim=maxdim, cutoff=1e-12)
                tes.append(t)
    np.testing.assert_allclose(te_g, tes, rtol=1e-6, atol=1e-12)
    assert st.edge_dims() == gg.edge_dims
    assert same_up_to_sign(state(gg, st.network().tensors), state(gg, B), 1e-8)


def test_spin_one_sites_and_the_size_limit():
    """d = 3 sites (spin 1): a gate on the centre bond against the oracle, and
    a gate whose rebuilt site would exceed the kernels' 8192 elements
    (3 x 8^3 x 8 at maxdim 8) refused before any launch, the state untouched."""
    base = O.square_lattice(3, 3, chi=8, d=3)
    dims = list(base.edge_dims)
    dims[3] = 4  # edge (1, 4): the centre site holds 3 x 8^3 x 4 = 6144 elements
    g = O.square_lattice(3, 3, chi=8, d=3, edge_dims=dims)
    A = O.random_network(g, 31, unit_norm=True)
    rng = np.random.default_rng(8)
    H = rng.standard_normal((9, 9))
    H = H + H.T
    w, U = np.linalg.eigh(H)
    gate = (U * np.exp(-0.2 * w)) @ U.T
    st = gbtn.SimpleUpdateState(gpu_net(g, A), chi_max=8)
    before = st.network()
    with pytest.raises(gbtn.Unsupported, match="limits"):
        st.apply(gate, [3], maxdim=8, cutoff=1e-12, normalize=True)
    after = st.network()
    assert list(after.edge_dims) == list(before.edge_dims)
    for a, b in zip(after.tensors, before.tensors):
        np.testing.assert_array_equal(a, b)
    g2, B, S, te = oracle_gate(g, A, gate, 3, maxdim=4, cutoff=1e-12)
    te_g, sv = st.apply(gate, [3], maxdim=4, cutoff=1e-12, normalize=True)
    assert st.edge_dims()[3] == g2.edge_dims[3]
    np.testing.assert_allclose(sv[0][:len(S)], S, rtol=1e-10)
    assert te_g[0] == pytest.approx(te, rel=1e-9, abs=1e-14)
    # the two updated sites contracted over their bond (gauge invariant; the
    # whole state of nine spin-1 sites at bond 8 is too large to contract here)
    out = st.network()
    u, v = g.edges[3]
    pu, pv = g.legs[u].index(3), g.legs[v].index(3)
    two = lambda T: np.tensordot(T[u], T[v], axes=([1 + pu], [1 + pv]))
    np.testing.assert_allclose(two(out.tensors), two(B), rtol=0, atol=1e-10 * np.max(np.abs(two(B))))
    for w in range(g.nv):
        if w not in (u, v):
            np.testing.assert_array_equal(out.tensors[w], A[w])
    st.close()
