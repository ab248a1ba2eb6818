"""Double-FP32 (df32) sweeps against the FP64 oracle.

A df32 value is the unevaluated sum of two floats (about 48 significant
bits); the sweep reads FP64 tensors and messages, contracts in df32 on the
FP32 pipe and normalises and compares messages in FP64.  Tolerances: one
sweep within 1e-12 of the oracle's FP64 sweep on unit-norm messages (df32's
relative rounding is ~1e-14 per operation; a lost low word would show as
~1e-7, the FP32 level), the converged fixed point within 1e-10 relative in
<Sz>, and the mixed pipeline with its default df32 refinement within 1e-10
after a full refinement phase."""
import numpy as np
import pytest

import bp_oracle as O
import build_oracle
import gbtn

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib(lib_built):
    yield


def net(g, A):
    return gbtn.TensorNetwork(g.nv, g.edges, g.site_dims, g.edge_dims, [a.copy() for a in A])


def converged_sz(g, A, sweeps):
    """<Sz> after `sweeps` FP64 parallel sweeps of the oracle's C restatement."""
    m0 = O.flatten_messages(g, O.identity_messages(g))
    mc, _, _ = build_oracle.run(g, O.flatten_tensors(A), m0, "parallel", None, sweeps)
    return O.expect1(g, A, O.unflatten_messages(g, mc), O.SZ)


def max_msg_err(got, want):
    return max(float(np.max(np.abs(got[de] - want[de]))) for de in range(len(want)))


@pytest.mark.parametrize("schedule", ["parallel", "colored"])
@pytest.mark.parametrize("case", ["grid6x6_chi8", "grid5x4_uneven", "tree_deg8_d3"])
def test_one_df32_sweep_matches_fp64_oracle(case, schedule):
    if case == "grid6x6_chi8":
        g = O.square_lattice(6, 6, chi=8)
    elif case == "grid5x4_uneven":
        rng = np.random.default_rng(3)
        g0 = O.square_lattice(5, 4)
        g = O.square_lattice(5, 4, edge_dims=[int(x) for x in rng.integers(1, 9, size=g0.ne)])
    else:
        # a star of degree 8 (bond dims 2-3) with leaves: the degree-8 schedule and d = 3
        edges = [(0, i) for i in range(1, 9)]
        g = O.Graph(9, edges, [3] * 9, [2, 3, 2, 2, 3, 2, 2, 2])
    A = O.random_network(g, 8)
    m2, _, _ = O.bp_update(g, A, O.identity_messages(g), maxiter=2, schedule="parallel")
    want, _, _ = O.bp_update(g, A, m2, maxiter=1, schedule=schedule)
    bpc = gbtn.BeliefPropagationCache(net(g, A))
    bpc.set_messages(m2)
    bpc.update(maxiter=1, schedule=schedule, precision="df32")
    err = max_msg_err(bpc.messages(), want)
    assert err <= 1e-12, f"df32 sweep differs from the FP64 oracle by {err:.3e}"
    bpc.close()


def test_df32_fixed_point_matches_oracle():
    g = O.square_lattice(8, 8, chi=6)
    A = O.random_network(g, 14)
    ref = converged_sz(g, A, 80)
    bpc = gbtn.BeliefPropagationCache(net(g, A)).update(maxiter=80, schedule="parallel", precision="df32")
    sz = bpc.expect(O.SZ)
    assert np.max(np.abs(sz - ref)) / np.max(np.abs(ref)) <= 1e-10
    assert bpc.phase_sweeps() == {"bf16": 0, "f32": 0, "refine": 80, "f64": 0}
    bpc.close()


def test_mixed_default_refinement_is_df32_and_converges():
    g = O.square_lattice(8, 8, chi=8)
    A = O.random_network(g, 15)
    ref = converged_sz(g, A, 80)
    bpc = gbtn.BeliefPropagationCache(net(g, A))
    bpc.update(maxiter=200, schedule="parallel", precision="mixed", refine_f64=60)
    ph = bpc.phase_sweeps()
    assert ph["refine"] == 60 and ph["f64"] == 0  # no tolerance: every refinement sweep runs
    assert 1 <= ph["bf16"] <= 200 and 1 <= ph["f32"] <= 200  # these phases keep their own tolerances
    sz = bpc.expect(O.SZ)
    assert np.max(np.abs(sz - ref)) / np.max(np.abs(ref)) <= 1e-10
    # FP64 confirmation sweeps after the df32 phase, and the FP64 refinement option
    bpc.init_messages("identity")
    bpc.update(maxiter=200, tol=1e-14, schedule="parallel", precision="mixed", confirm_f64=2)
    ph = bpc.phase_sweeps()
    assert 1 <= ph["f64"] <= 2 and ph["refine"] >= 1
    bpc.init_messages("identity")
    bpc.update(maxiter=200, tol=1e-14, schedule="parallel", precision="mixed", refine="f64")
    ph = bpc.phase_sweeps()
    assert ph["refine"] >= 1 and ph["f64"] == 0
    assert np.max(np.abs(bpc.expect(O.SZ) - ref)) / np.max(np.abs(ref)) <= 1e-6
    bpc.close()


def test_df32_refused_where_it_has_no_path():
    g = O.square_lattice(3, 3, chi=2)
    # sequential double-FP32 sweeps on a plan with a vertex of the global-memory path
    gl = O.square_lattice(3, 3, chi=10)
    bpc = gbtn.BeliefPropagationCache(net(gl, O.random_network(gl, 1)))
    with pytest.raises(gbtn.Unsupported):
        bpc.update(maxiter=2, schedule="sequential", precision="df32")
    bpc.close()
    Az = O.random_network(g, 1, dtype=np.complex128)
    bz = gbtn.BeliefPropagationCache(net(g, Az))
    with pytest.raises(gbtn.Unsupported):
        bz.update(maxiter=2, schedule="parallel", precision="df32")
    bz.close()
