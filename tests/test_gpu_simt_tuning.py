"""The measured SIMT team width per size class against the oracle.

Every team width (32 threads per vertex with four vertices per block, 128,
256) computes the same messages up to the rounding of the close reductions,
so each forced width and the measured choice must match the oracle's FP64
Jacobi sweep within the FP64 tolerance of the other parity tests (1e-12 on
unit-norm messages), and FP32 / df32 sweeps within their own (1e-5, 1e-12)."""
import numpy as np
import pytest

import bp_oracle as O
import build_oracle
import gbtn

pytestmark = pytest.mark.gpu

TOL = {"f64": 1e-12, "df32": 1e-12, "f32": 1e-5}


@pytest.fixture(scope="module", autouse=True)
def _lib(lib_built):
    yield


def uneven_case():
    """A 7x6 lattice with bond dimensions 2..8 (vertex sizes from 8 to 8192):
    several size classes on both work lists."""
    rng = np.random.default_rng(5)
    g0 = O.square_lattice(7, 6)
    g = O.square_lattice(7, 6, edge_dims=[int(x) for x in rng.integers(2, 9, size=g0.ne)])
    return g, O.random_network(g, 17)


def sweep_err(g, A, mode, precision):
    m2, _, _ = O.bp_update(g, A, O.identity_messages(g), maxiter=2, schedule="parallel")
    want, _, _ = O.bp_update(g, A, m2, maxiter=1, schedule="parallel")
    tn = gbtn.TensorNetwork(g.nv, g.edges, g.site_dims, g.edge_dims, [a.copy() for a in A])
    bpc = gbtn.BeliefPropagationCache(tn).set_simt_tuning(mode)
    bpc.set_messages(m2)
    bpc.update(maxiter=1, schedule="parallel", precision=precision)
    got = bpc.messages()
    teams = bpc.simt_teams(precision)
    bpc.close()
    return max(float(np.max(np.abs(got[de] - want[de]))) for de in range(2 * g.ne)), teams


@pytest.mark.parametrize("precision", ["f64", "f32", "df32"])
@pytest.mark.parametrize("mode", [False, True, 32, 128, 256])
def test_every_team_width_matches_the_oracle(precision, mode):
    g, A = uneven_case()
    err, teams = sweep_err(g, A, mode, precision)
    assert err <= TOL[precision], f"mode {mode}: {err:.3e}"
    if mode is False:
        assert teams == {}
    else:
        assert teams and set(teams.values()) <= {32, 128, 256}
        if mode in (32, 128, 256):
            assert mode in teams.values()


def test_measured_choice_reaches_the_oracle_fixed_point():
    """200 FP64 sweeps (no tolerance) agree between the fixed rule and the
    measured widths to rounding; the mixed pipeline under either is within its
    1e-6 bound of the oracle's converged <Sz> (a solve stopped at tol 1e-13
    leaves ~3e-7 in the messages, so two such solves differ at ~1e-8)."""
    g, A = uneven_case()
    m0 = O.flatten_messages(g, O.identity_messages(g))
    mc, _, _ = build_oracle.run(g, O.flatten_tensors(A), m0, "parallel", None, 200)
    ref = O.expect1(g, A, O.unflatten_messages(g, mc), O.SZ)
    tn = gbtn.TensorNetwork(g.nv, g.edges, g.site_dims, g.edge_dims, [a.copy() for a in A])
    f64 = {}
    for mode in (False, True):
        bpc = gbtn.BeliefPropagationCache(tn).set_simt_tuning(mode).set_graphs(True)
        bpc.update(maxiter=200, schedule="parallel", precision="f64")
        f64[mode] = bpc.expect(O.SZ)
        bpc.init_messages("identity")
        bpc.update(maxiter=300, tol=1e-13, schedule="parallel", precision="mixed")
        assert np.max(np.abs(bpc.expect(O.SZ) - ref)) / np.max(np.abs(ref)) <= 1e-6
        bpc.close()
    np.testing.assert_allclose(f64[True], f64[False], rtol=0, atol=1e-12)
    np.testing.assert_allclose(f64[True], ref, rtol=0, atol=1e-10)
