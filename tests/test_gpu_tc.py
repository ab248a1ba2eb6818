"""BF16 tensor-core (tcgen05) message path against the FP64 oracle.

Tolerances: one BF16 sweep from the same input messages agrees with the FP64
sweep to 3e-2 absolute on unit-norm messages (BF16 keeps 8 significant bits;
a layout or descriptor error shows up as O(0.1-1) differences); messages of
vertices outside the tensor-core class run FP32 and agree to 1e-5.  The mixed
pipeline (BF16 -> FP32 -> FP64) meets <= 1e-6 max relative error in <Sz>
after two FP64 sweeps and 1e-10 after a full FP64 phase."""
import numpy as np
import pytest

import bp_oracle as O
import build_oracle
import gbtn

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib(lib_built):
    yield


def pair(L, seed, chi=8):
    tn = gbtn.random_network(gbtn.square_lattice(L, L, chi=chi), seed)
    g = O.square_lattice(L, L, chi=chi)
    A = O.random_network(g, seed)
    return tn, g, A


def tc_directed_edges(g):
    """Directed edges leaving degree-4, chi=8, d=2 vertices (the tensor-core class)."""
    out = set()
    for v in range(g.nv):
        if len(g.legs[v]) == 4 and all(g.edge_dims[e] == 8 for e in g.legs[v]) and g.site_dims[v] == 2:
            out |= {g.directed(e, v) for e in g.legs[v]}
    return out


def test_one_bf16_sweep_matches_fp64_sweep():
    tn, g, A = pair(6, 3)
    m3, _, _ = O.bp_update(g, A, O.identity_messages(g), maxiter=3, schedule="parallel")
    m4, _, _ = O.bp_update(g, A, m3, maxiter=1, schedule="parallel")
    bpc = gbtn.BeliefPropagationCache(tn)
    bpc.set_messages(m3)
    bpc.update(maxiter=1, schedule="parallel", precision="bf16")
    got = bpc.messages()
    tcset = tc_directed_edges(g)
    assert len(tcset) == 4 * 16
    err_tc = max(np.max(np.abs(got[de] - m4[de])) for de in tcset)
    err_rest = max(np.max(np.abs(got[de] - m4[de])) for de in range(2 * g.ne) if de not in tcset)
    assert err_tc < 3e-2, f"tensor-core messages differ by {err_tc:.3e}"
    assert err_rest < 1e-5, f"SIMT messages differ by {err_rest:.3e}"
    for de in tcset:
        assert np.linalg.norm(got[de]) == pytest.approx(1.0, rel=1e-6)


def test_bf16_colored_schedule_matches_fp64():
    tn, g, A = pair(5, 8)
    m2, _, _ = O.bp_update(g, A, O.identity_messages(g), maxiter=2, schedule="parallel")
    m3, _, _ = O.bp_update(g, A, m2, maxiter=1, schedule="colored")
    bpc = gbtn.BeliefPropagationCache(tn)
    bpc.set_messages(m2)
    bpc.update(maxiter=1, schedule="colored", precision="bf16")
    got = bpc.messages()
    err = max(np.max(np.abs(got[de] - m3[de])) for de in range(2 * g.ne))
    assert err < 3e-2


def test_mixed_pipeline_accuracy_on_32x32_chi8():
    # the target shape: 32x32, d=2, chi=8, N(0,1) tensors
    tn, g, A = pair(32, 11)
    ref = gbtn.BeliefPropagationCache(tn).update(maxiter=300, schedule="parallel", precision="f64")
    sz_ref = ref.expect(O.SZ)
    scale = np.max(np.abs(sz_ref))
    b16 = gbtn.BeliefPropagationCache(tn).update(maxiter=300, tol=1e-7, schedule="parallel", precision="bf16")
    err16 = np.max(np.abs(b16.expect(O.SZ) - sz_ref)) / scale
    assert err16 < 5e-2
    mix = gbtn.BeliefPropagationCache(tn).update(maxiter=300, tol=1e-14, schedule="parallel", precision="mixed",
                                                 refine_f64=2)
    err_mix = np.max(np.abs(mix.expect(O.SZ) - sz_ref)) / scale
    assert err_mix <= 1e-6, f"mixed pipeline max relative <Sz> error {err_mix:.3e}"
    full = gbtn.BeliefPropagationCache(tn).update(maxiter=300, schedule="parallel", precision="mixed")
    assert np.max(np.abs(full.expect(O.SZ) - sz_ref)) / scale < 1e-10


def test_bf16_batch_with_uneven_shapes_and_convergence():
    nets, pairs = [], []
    for k, L in enumerate([4, 6, 3]):
        tn, g, A = pair(L, 60 + k)
        nets.append(tn)
        pairs.append((g, A))
    batch = gbtn.disjoint_union(nets)
    bpc = gbtn.BeliefPropagationCache(batch).update(maxiter=200, tol=1e-15, schedule="parallel", precision="mixed",
                                                    tol_bf16=1e-6)
    sz = bpc.expect(O.SZ)
    off = 0
    for g, A in pairs:
        mc, _, _ = build_oracle.run(g, O.flatten_tensors(A), O.flatten_messages(g, O.identity_messages(g)),
                                    "parallel", None, 400, tol=None, nthreads=4)
        ref = O.expect1(g, A, O.unflatten_messages(g, mc), O.SZ)
        np.testing.assert_allclose(sz[off:off + g.nv], ref, atol=1e-6 * np.max(np.abs(ref)))
        off += g.nv
