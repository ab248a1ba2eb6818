"""Bond dimensions above 8 and large site dimensions (the global-memory path)
against the FP64 oracle.

The reference contracts any bond dimension (updated_message,
abstractbeliefpropagationcache.jl:225-239).  Vertices whose tensors do not
fit the shared-memory kernels -- chi or d above 8, or too many elements --
run the global-memory path (intermediates in HBM, one launch per schedule
step over a wave of vertices).  Tolerances as the FP64 parity tests: 1e-12
absolute on unit-norm FP64 messages (1e-11 for chi = 16, whose tensors sum
2^17 products per entry), 1e-5 for FP32, 1e-12 for double-FP32, 1e-10
relative on <Sz>, scalars and environments."""
import numpy as np
import pytest

import bp_oracle as O
import gbtn

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib(lib_built):
    yield


def net(g, A, complex_values=False):
    return gbtn.TensorNetwork(g.nv, g.edges, g.site_dims, g.edge_dims, [a.copy() for a in A])


def max_err(got, want):
    return max(float(np.max(np.abs(np.asarray(got[de]) - want[de]))) for de in range(len(want)))


CASES = {
    "grid3x3_chi12": lambda: O.square_lattice(3, 3, chi=12),
    "grid3x3_chi16": lambda: O.square_lattice(3, 3, chi=16),
    "grid4x3_chi9": lambda: O.square_lattice(4, 3, chi=9),
    "grid3x3_mixed_chi": lambda: O.square_lattice(3, 3, edge_dims=[8, 10, 3, 16, 2, 9, 8, 12, 4, 11, 5, 7]),
    "chain_d16": lambda: O.Graph(4, [(0, 1), (1, 2), (2, 3)], [16, 12, 10, 16], [3, 5, 3]),
}


@pytest.mark.parametrize("schedule", ["parallel", "colored", "sequential"])
@pytest.mark.parametrize("case", list(CASES))
def test_large_f64_sweeps_match_oracle(case, schedule):
    g = CASES[case]()
    A = O.random_network(g, 3, unit_norm=True)
    m1, _, _ = O.bp_update(g, A, O.identity_messages(g), maxiter=1, schedule="parallel")
    seq = O.default_edge_sequence(g)
    want, _, md = O.bp_update(g, A, m1, maxiter=2, tol=0.0 if schedule != "sequential" else None,
                              schedule=schedule, edge_sequence=seq if schedule == "sequential" else None)
    bpc = gbtn.BeliefPropagationCache(net(g, A))
    bpc.set_messages(m1)
    bpc.update(maxiter=2, tol=0.0 if schedule != "sequential" else None, schedule=schedule,
               edge_sequence=seq if schedule == "sequential" else None)
    tol = 1e-11 if max(g.edge_dims) >= 16 else 1e-12
    assert max_err(bpc.messages(), want) <= tol
    if schedule != "sequential":
        assert float(bpc.mean_diff[0]) == pytest.approx(md, rel=1e-8, abs=1e-15)
    bpc.close()


@pytest.mark.parametrize("precision,tol", [("f32", 1e-5), ("df32", 1e-12)])
def test_large_reduced_precision_sweeps(precision, tol):
    g = CASES["grid3x3_mixed_chi"]()
    A = O.random_network(g, 4, unit_norm=True)
    m1, _, _ = O.bp_update(g, A, O.identity_messages(g), maxiter=1, schedule="parallel")
    want, _, _ = O.bp_update(g, A, m1, maxiter=1, schedule="parallel")
    bpc = gbtn.BeliefPropagationCache(net(g, A))
    bpc.set_messages(m1)
    bpc.update(maxiter=1, schedule="parallel", precision=precision)
    assert max_err(bpc.messages(), want) <= tol
    bpc.close()


def test_large_environments_scalars_and_mixed_pipeline():
    g = CASES["grid3x3_mixed_chi"]()
    A = O.random_network(g, 5)
    m, _, _ = O.bp_update(g, A, O.identity_messages(g), maxiter=60, schedule="parallel")
    bpc = gbtn.BeliefPropagationCache(net(g, A))
    bpc.update(maxiter=60, schedule="parallel")
    sz = bpc.expect(O.SZ)
    ref = O.expect1(g, A, m, O.SZ)
    np.testing.assert_allclose(sz, ref, rtol=0, atol=1e-10 * np.max(np.abs(ref)))
    rd = bpc.vertex_rdms()
    for v in range(g.nv):
        np.testing.assert_allclose(rd[v], O.vertex_rdm(g, A, A, m, v), rtol=1e-10, atol=1e-12 * np.abs(rd[v]).max())
    assert bpc.logscalar() == pytest.approx(float(np.real(O.logscalar(g, A, A, m))), rel=1e-10)
    for de in [0, 5, 2 * g.ne - 1]:
        np.testing.assert_allclose(bpc.updated_message(de), O.updated_message(g, A, A, m, de), atol=1e-12)
    # rescale_messages at chi > 8: unit edge scalars
    bpc.rescale_messages()
    np.testing.assert_allclose(bpc.edge_scalars(), np.ones(g.ne), rtol=1e-12)
    # the mixed pipeline routes these vertices to FP32, then double-FP32
    mix = gbtn.BeliefPropagationCache(net(g, A)).update(maxiter=200, tol=1e-14, schedule="parallel", precision="mixed")
    np.testing.assert_allclose(mix.expect(O.SZ), ref, rtol=0, atol=1e-6 * np.max(np.abs(ref)))
    with pytest.raises(gbtn.Unsupported):
        mix.edge_rdms([0])
    mix.close()
    bpc.close()


def test_large_complex_f64_sweep():
    g = CASES["grid3x3_chi12"]()
    A = O.random_network(g, 6, dtype=np.complex128, unit_norm=True)
    m1, _, _ = O.bp_update(g, A, O.identity_messages(g, dtype=np.complex128), maxiter=1, schedule="parallel")
    want, _, _ = O.bp_update(g, A, m1, maxiter=1, schedule="parallel")
    bpc = gbtn.BeliefPropagationCache(net(g, A))
    bpc.set_messages(m1)
    bpc.update(maxiter=1, schedule="parallel")
    assert max_err(bpc.messages(), want) <= 1e-12
    bpc.close()


def test_refused_beyond_the_large_path():
    with pytest.raises(gbtn.Unsupported, match="bond dimension"):
        gbtn.BeliefPropagationCache(gbtn.random_network(gbtn.square_lattice(2, 2, chi=65), 1))
