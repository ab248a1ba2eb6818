"""The sequential schedule (the reference's default) in waves, against the
oracle's strictly sequential update (abstractbeliefpropagationcache.jl:272-287).

The library cuts the edge sequence into waves of messages that neither read
nor write a message another message of the same wave writes, and runs each
wave as one launch; the result must equal the one-message-at-a-time update:
1e-12 on unit-norm FP64 messages, the per-network iteration count of a
tolerance run within one sweep of the oracle's, and sequences that repeat
directed edges or leave some out handled as the reference handles them."""
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


def max_err(got, want):
    return max(float(np.max(np.abs(np.asarray(got[de]) - want[de]))) for de in range(len(want)))


@pytest.mark.parametrize("precision,tol", [("f64", 1e-12), ("df32", 1e-12), ("f32", 1e-5)])
def test_waves_equal_the_strict_sequence(precision, tol):
    g = O.square_lattice(12, 10, chi=4)
    A = O.random_network(g, 9, unit_norm=True)
    seq = O.default_edge_sequence(g)
    m0 = O.flatten_messages(g, O.identity_messages(g))
    mc, _, _ = build_oracle.run(g, O.flatten_tensors(A), m0, "sequential", seq, 3)
    want = O.unflatten_messages(g, mc)
    bpc = gbtn.BeliefPropagationCache(net(g, A)).update(maxiter=3, schedule="sequential", precision=precision)
    assert max_err(bpc.messages(), want) <= tol
    bpc.close()


def test_waves_on_a_batch_converge_per_network_like_the_oracle():
    gs = [O.square_lattice(6, 6, chi=3), O.square_lattice(9, 4, chi=5), O.random_tree(15, seed=3, chi=4)]
    As = [O.random_network(g, 40 + k) for k, g in enumerate(gs)]
    batch = gbtn.disjoint_union([net(g, A) for g, A in zip(gs, As)])
    bpc = gbtn.BeliefPropagationCache(batch).update(maxiter=200, tol=1e-10, schedule="sequential")
    its = list(bpc.iterations)
    msgs = bpc.messages()
    off_e = 0
    for k, (g, A) in enumerate(zip(gs, As)):
        seq = O.default_edge_sequence(g)
        m, it, _ = O.bp_update(g, A, O.identity_messages(g), maxiter=200, tol=1e-10, schedule="sequential",
                               edge_sequence=seq)
        assert abs(its[k] - it) <= 1, (k, its[k], it)
        got = msgs[2 * off_e:2 * (off_e + g.ne)]
        assert max(float(np.max(np.abs(got[de] - m[de]))) for de in range(2 * g.ne)) <= 1e-6
        off_e += g.ne
    bpc.close()


def test_sequences_with_repeats_and_gaps():
    g = O.square_lattice(4, 4, chi=3)
    A = O.random_network(g, 12, unit_norm=True)
    full = O.default_edge_sequence(g)
    seq = full[:10] + full[:10] + full[20:]  # ten messages twice, some never
    m, it, md = O.bp_update(g, A, O.identity_messages(g), maxiter=2, tol=0.0, schedule="sequential",
                            edge_sequence=seq)
    bpc = gbtn.BeliefPropagationCache(net(g, A)).update(maxiter=2, tol=0.0, schedule="sequential", edge_sequence=seq)
    assert max_err(bpc.messages(), m) <= 1e-12
    assert float(bpc.mean_diff[0]) == pytest.approx(md, rel=1e-9, abs=1e-15)
    bpc.close()


def test_mixed_sequential_pipeline_reaches_the_oracle_fixed_point():
    """MIXED with the reference's default schedule: FP32 waves to their
    tolerance or noise floor, then double-FP32 waves to tol.  The result
    is within 1e-6 relative <Sz> of the oracle's sequential fixed point (the
    mixed pipeline's bound; tol 1e-14 itself leaves ~1e-7), with the phase
    sweeps recorded; refine="f64" and confirm_f64 run their FP64 waves."""
    g = O.square_lattice(6, 6, chi=6)
    A = O.random_network(g, 19)
    seq = list(gbtn.default_edge_sequence(net(g, A)))
    ref_m, _, _ = O.bp_update(g, A, O.identity_messages(g), maxiter=60, schedule="sequential", edge_sequence=seq)
    ref = O.expect1(g, A, ref_m, O.SZ)
    scale = np.max(np.abs(ref))
    bpc = gbtn.BeliefPropagationCache(net(g, A))
    bpc.update(maxiter=200, tol=1e-14, precision="mixed")
    ph = bpc.phase_sweeps()
    assert ph["bf16"] == 0 and ph["f32"] >= 1 and ph["refine"] >= 1 and ph["f64"] == 0
    assert np.max(np.abs(bpc.expect(O.SZ) - ref)) / scale <= 1e-6
    bpc.init_messages("identity")
    bpc.update(maxiter=200, tol=1e-14, precision="mixed", refine="f64")
    assert np.max(np.abs(bpc.expect(O.SZ) - ref)) / scale <= 1e-6
    bpc.init_messages("identity")
    bpc.update(maxiter=200, tol=1e-14, precision="mixed", confirm_f64=1)
    assert bpc.phase_sweeps()["f64"] == 1
    assert np.max(np.abs(bpc.expect(O.SZ) - ref)) / scale <= 1e-6
    with pytest.raises(gbtn.Unsupported):
        bpc.update(maxiter=2, tol=1e-14, precision="bf16")
    bpc.close()
