"""The reference's test/test_normalize.jl restated on the GPU path.

* :17-28 -- a random comb tree (2 x 3, chi 2) rescaled by BP (maxiter 20) has
  exact scalar 1.
* :30-66 -- a ComplexF32 state on a loopy 3 x 2 grid normalised by BP from
  identity messages (maxiter 20, the default sequential schedule): the cache
  keeps ComplexF32 messages, every edge and vertex scalar is 1, and a fresh BP
  scalar of the normalised state is 1.  Julia's isapprox on Float32 values
  means rtol sqrt(eps(Float32)); the ComplexF32 arithmetic is the FP32 path,
  and the FP64 path is checked at 1e-10.

The StableRNG inputs cannot be regenerated without Julia; seeded standard
normal tensors of the same shapes stand in for them."""
import numpy as np
import pytest

import bp_oracle as O
import gbtn

pytestmark = pytest.mark.gpu

RT32 = float(np.sqrt(np.finfo(np.float32).eps))


@pytest.fixture(scope="module", autouse=True)
def _lib(lib_built):
    yield


def net(g, A):
    return gbtn.TensorNetwork(g.nv, g.edges, g.site_dims, g.edge_dims, [a.copy() for a in A])


def test_comb_tree_rescaled_by_bp_has_exact_scalar_one():
    g = O.comb_tree(2, 3, chi=2)
    A = O.random_network(g, 1234)
    out = gbtn.rescale(net(g, A), cache_update_kwargs=dict(maxiter=20))
    assert O.exact_scalar(g, out.tensors) == pytest.approx(1.0, rel=1e-10)


@pytest.mark.parametrize("precision,tol", [("f32", RT32), ("f64", 1e-10)])
def test_loopy_complexf32_state_normalised_by_bp(precision, tol):
    g = O.square_lattice(3, 2, chi=2)
    A = [a.astype(np.complex64) for a in O.random_network(g, 1234, dtype=np.complex128)]
    kw = dict(maxiter=20, precision=precision)
    cache = gbtn.BeliefPropagationCache(net(g, A))
    psi = gbtn.normalize(net(g, A), cache=cache, update_cache=True, cache_update_kwargs=kw)
    assert all(m.dtype == np.complex64 for m in cache.messages())
    np.testing.assert_allclose(cache.edge_scalars(), 1.0, rtol=tol, atol=0)
    np.testing.assert_allclose(cache.vertex_scalars(), 1.0, rtol=tol, atol=0)
    z = gbtn.scalar(psi, cache_update_kwargs=kw)
    assert abs(z - 1.0) <= tol
    # the kets are the oracle's rescale of the same messages (a second cache
    # runs the same deterministic sweeps; its FP64 master copy, not messages(),
    # which rounds to the ComplexF32 element type)
    c2 = gbtn.BeliefPropagationCache(net(g, A)).update(**kw)
    ref = O.normalize_bp(g, [a.astype(np.complex128) for a in A], c2.tn.unflat_messages(c2.flat_messages()))[0]
    for v in range(g.nv):
        np.testing.assert_allclose(psi.tensors[v], ref[v], rtol=0, atol=max(tol, 1e-12) * np.max(np.abs(ref[v])))
