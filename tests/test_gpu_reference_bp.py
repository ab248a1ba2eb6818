"""The reference's belief-propagation test (test/test_belief_propagation.jl)
restated on the GPU for each element type it runs -- Float32, Float64,
ComplexF32, ComplexF64 (FP32 sweeps for the single-precision types, FP64
otherwise):

* a 3x3 grid, S=1/2, chi = 2, identity messages, update(maxiter=25, tol=eps):
  every message satisfies message_diff(updated_message, message) < 10 eps and
  keeps the element type;
* updating a factor in the cache replaces it;
* the trace-normalised two-site RDM of sites (2,2), (2,3) has eigenvalues with
  |imag| <= eps and real part >= -eps;
* a 3x1 chain whose first tensor is zero has scalar 0;
* a loopy 4-cycle product state (the non-QN form of the reference's QN
  regression) has a finite, nonzero scalar."""
import numpy as np
import pytest

import gbtn

pytestmark = pytest.mark.gpu

ELTS = [np.float32, np.float64, np.complex64, np.complex128]


@pytest.fixture(scope="module", autouse=True)
def _lib(lib_built):
    yield


def network(Lx, Ly, chi, elt, seed):
    tn = gbtn.square_lattice(Lx, Ly, chi=chi)
    rng = np.random.default_rng(seed)
    ts = []
    for v in range(tn.nv):
        shape = tn.shape(v)
        x = rng.standard_normal(shape)
        if np.issubdtype(elt, np.complexfloating):
            x = x + 1j * rng.standard_normal(shape)
        ts.append(x.astype(elt))
    tn.tensors = ts
    return tn


def precision(elt):
    return "f32" if elt in (np.float32, np.complex64) else "f64"


@pytest.mark.parametrize("elt", ELTS)
def test_belief_propagation_as_the_reference(elt):
    eps = float(np.finfo(np.dtype(elt).type(0).real.dtype).eps)
    tn = network(3, 3, 2, elt, 1234)
    bpc = gbtn.BeliefPropagationCache(tn)
    bpc.init_messages("identity")
    # updating a factor of the cache (the reference sets ket and dag(prime(ket)) together)
    rng = np.random.default_rng(7)
    new = rng.standard_normal(tn.shape(0))
    if np.iscomplexobj(np.zeros(1, elt)):
        new = new + 1j * rng.standard_normal(tn.shape(0))
    before = bpc.factors()
    gbtn.update_factor(bpc, 0, new.astype(elt))
    after = bpc.factors()
    np.testing.assert_array_equal(after[0], new.astype(elt).astype(bpc.dtype))
    for v in range(1, tn.nv):
        np.testing.assert_array_equal(after[v], before[v])
    bpc.update(maxiter=25, tol=eps, precision=precision(elt))
    msgs = bpc.messages()
    for de in range(2 * tn.ne):
        assert msgs[de].dtype == np.dtype(elt)
        assert gbtn.message_diff(bpc.updated_message(de), msgs[de]) < 10 * eps
    # two-site RDM of (2,2)-(2,3): vertices 4 and 7 of the 3x3 grid
    e = tn.edges.index((4, 7))
    rdm = bpc.edge_rdms([e])[0]
    rdm = rdm / np.trace(rdm)
    assert rdm.shape == (4, 4)
    ev = np.linalg.eigvals(rdm)
    assert np.all(np.abs(ev.imag) <= eps)
    assert np.all(ev.real >= -eps)


@pytest.mark.parametrize("elt", ELTS)
def test_network_evaluating_to_zero(elt):
    tn = network(3, 1, 2, elt, 1234)
    tn.tensors[0] = 0 * tn.tensors[0]
    assert gbtn.scalar(tn, cache_update_kwargs=dict(maxiter=20, precision=precision(elt))) == 0


def test_loopy_product_state_scalar_is_finite_and_nonzero():
    # 4-cycle (a 2x2 periodic grid), S=1/2 product state, alternating up / down
    tn = gbtn.TensorNetwork(4, [(0, 1), (1, 2), (2, 3), (0, 3)], [2] * 4, [1] * 4)
    up, dn = np.array([1.0, 0.0]), np.array([0.0, 1.0])
    tn.tensors = [(up if v % 2 == 0 else dn).reshape(2, 1, 1) for v in range(4)]
    n2 = gbtn.scalar(tn, cache_update_kwargs=dict(maxiter=25))
    assert np.isfinite(n2) and n2 != 0
