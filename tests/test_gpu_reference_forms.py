"""The parts of the reference's test/test_forms.jl that run on the BP path.

* :14-73 -- on a 1 x 4 chain (chi 2) the BP environment of a vertex, after the
  default update (one forest-cover sweep on a tree), equals the exact
  environment up to normalisation.  Restated for the reference's end vertex and
  an interior one: the exact environment of a tree vertex factorises into one
  matrix per leg, which BP's incoming messages must reproduce.
* :75-90 -- a ComplexF64 state on a 3 x 3 comb tree whose vertices carry two,
  one or no site indices (site dimensions 4, 2, 1): the BP scalars of the
  bilinear form <bra|ket> and of <ket|ket> equal the exact contractions (the
  reference compares exact scalars with exact inner products; BP is exact on
  the tree).

Seeded standard-normal tensors stand in for the StableRNG inputs."""
import numpy as np
import pytest

import bp_oracle as O
import gbtn

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib(lib_built):
    yield


def net(g, A):
    return gbtn.TensorNetwork(g.nv, g.edges, g.site_dims, g.edge_dims, [a.copy() for a in A])


@pytest.mark.parametrize("v", [0, 1])
def test_bp_environment_on_a_chain_equals_the_exact_one(v):
    g = O.square_lattice(1, 4, chi=2)
    A = O.random_network(g, 1234)
    bpc = gbtn.BeliefPropagationCache(net(g, A)).update()  # a tree: the default is one sweep
    incoming, tensors = bpc.environment([v])
    # the BP environment: the product of the incoming messages M[b, a], legs in v's order
    by_leg = {g.legs[v].index(de // 2): m for de, m in incoming}
    k = len(g.legs[v])
    ops, out = [], []
    for p in range(k):
        ops += [by_leg[p], [p, k + p]]
    env_bp = np.einsum(*ops, list(range(2 * k)))
    env_ex = O.exact_environment(g, A, v)
    np.testing.assert_allclose(env_bp / np.linalg.norm(env_bp), env_ex / np.linalg.norm(env_ex), rtol=0, atol=1e-12)
    assert np.array_equal(tensors[0], A[v])


def test_nonuniform_site_indices_on_a_comb_tree():
    g0 = O.comb_tree(3, 3, chi=2)
    dims = [4] * g0.nv
    dims[0] = 1  # (1, 1): no site index
    dims[g0.nv - 1] = 2  # (3, 3): one site index
    g = O.Graph(g0.nv, g0.edges, dims, list(g0.edge_dims))
    ket = O.random_network(g, 1234, dtype=np.complex128)
    bra = O.random_network(g, 4321, dtype=np.complex128)
    exact_blf = O.exact_scalar(g, ket, bra)  # <bra|ket>
    got = gbtn.inner(net(g, bra), net(g, ket))
    assert abs(got - exact_blf) <= 1e-10 * abs(exact_blf)
    exact_qf = O.exact_scalar(g, ket)
    got = gbtn.norm_sqr(net(g, ket))
    assert abs(got - exact_qf) <= 1e-10 * abs(exact_qf)
