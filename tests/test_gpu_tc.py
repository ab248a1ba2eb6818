"""BF16 tensor-core (tcgen05) message path against the FP64 oracle.

Tolerances: one BF16 sweep from the same input messages agrees with the FP64
sweep to 3e-2 absolute on unit-norm messages (BF16 keeps 8 significant bits;
a layout or descriptor error shows up as O(0.1-1) differences; the tighter
check against the oracle's BF16 rounding model is in
test_gpu_oracle_configs.py); messages of
vertices outside the tensor-core class run FP32 and agree to 1e-5.  Vertices
padded to the kernel's shape (boundary legs, bond dimensions below 8, leaves)
meet the same 3e-2 and keep their compact shapes.  The mixed
pipeline (BF16 -> FP32 -> FP64) meets <= 1e-6 max relative error in <Sz>
after two FP64 sweeps and 1e-10 after a full FP64 phase."""
from pathlib import Path

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
    bpc = gbtn.BeliefPropagationCache(tn).set_tc_policy("native")
    bpc.set_messages(m3)
    bpc.update(maxiter=1, schedule="parallel", precision="bf16")
    got = bpc.messages()
    tcset = tc_directed_edges(g)
    is_tc, _ = bpc.tc_split()
    assert {v for v in range(g.nv) if is_tc[v]} == {v for v in range(g.nv) if len(g.legs[v]) == 4}
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
    bpc = gbtn.BeliefPropagationCache(tn).set_tc_policy("all")
    bpc.set_messages(m2)
    bpc.update(maxiter=1, schedule="colored", precision="bf16")
    got = bpc.messages()
    err = max(np.max(np.abs(got[de] - m3[de])) for de in range(2 * g.ne))
    assert err < 3e-2


def test_mixed_pipeline_accuracy_on_32x32_chi8():
    # the target shape: 32x32, d=2, chi=8, N(0,1) tensors (seed 11); the
    # reference <Sz> is the oracle's converged fixed point (C restatement of
    # the reference's sweep, tests/golden/make_large_fixtures.py)
    tn, g, A = pair(32, 11)
    fx = np.load(Path(__file__).resolve().parent / "golden" / "peps32x32_chi8_batch16.npz")
    sz_ref = fx["sz"][11 * 1024:12 * 1024]
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


def uneven(L, seed, lo=2, hi=8, d=2):
    rng = np.random.default_rng(1000 + seed)
    g0 = O.square_lattice(L, L, chi=2, d=d)
    dims = [int(x) for x in rng.integers(lo, hi + 1, size=g0.ne)]
    g = O.square_lattice(L, L, d=d, edge_dims=dims)
    A = O.random_network(g, seed)
    tn = gbtn.TensorNetwork(g.nv, g.edges, g.site_dims, g.edge_dims, [a.copy() for a in A])
    return tn, g, A


def test_padded_boundary_sweep_matches_fp64():
    tn, g, A = pair(6, 5)
    m3, _, _ = O.bp_update(g, A, O.identity_messages(g), maxiter=3, schedule="parallel")
    m4, _, _ = O.bp_update(g, A, m3, maxiter=1, schedule="parallel")
    bpc = gbtn.BeliefPropagationCache(tn).set_tc_policy("all")
    bpc.set_messages(m3)
    bpc.update(maxiter=1, schedule="parallel", precision="bf16")
    is_tc, _ = bpc.tc_split()
    assert is_tc.all()  # corners (2 legs) and edges (3 legs) padded
    got = bpc.messages()
    err = max(np.max(np.abs(got[de] - m4[de])) for de in range(2 * g.ne))
    assert err < 3e-2, f"padded tensor-core messages differ by {err:.3e}"
    for de in range(2 * g.ne):
        assert np.linalg.norm(got[de]) == pytest.approx(1.0, rel=1e-5)


def test_padded_uneven_bond_dims_sweep_and_mixed_fixed_point():
    tn, g, A = uneven(6, 7)
    assert len(set(g.edge_dims)) > 3
    m3, _, _ = O.bp_update(g, A, O.identity_messages(g), maxiter=3, schedule="parallel")
    m4, _, _ = O.bp_update(g, A, m3, maxiter=1, schedule="parallel")
    bpc = gbtn.BeliefPropagationCache(tn).set_tc_policy("all")
    bpc.set_messages(m3)
    bpc.update(maxiter=1, schedule="parallel", precision="bf16")
    got = bpc.messages()
    for de in range(2 * g.ne):
        assert got[de].shape == m4[de].shape
    err = max(np.max(np.abs(got[de] - m4[de])) for de in range(2 * g.ne))
    assert err < 3e-2, f"padded uneven-chi messages differ by {err:.3e}"
    ref = gbtn.BeliefPropagationCache(tn).update(maxiter=400, schedule="parallel", precision="f64")
    sz_ref = ref.expect(O.SZ)
    mix = gbtn.BeliefPropagationCache(tn).set_tc_policy("all").update(maxiter=400, schedule="parallel",
                                                                       precision="mixed")
    np.testing.assert_allclose(mix.expect(O.SZ), sz_ref, rtol=0, atol=1e-10 * np.max(np.abs(sz_ref)))


def test_padded_leaves_on_a_tree():
    # random tree of degree <= 4 (vertex i attaches to an earlier vertex with a free leg)
    rng = np.random.default_rng(4)
    deg, edges = [0] * 24, []
    for i in range(1, 24):
        u = int(rng.choice([w for w in range(i) if deg[w] < 4]))
        edges.append((u, i))
        deg[u] += 1
        deg[i] += 1
    dims = [int(x) for x in rng.integers(2, 9, size=len(edges))]
    g = O.Graph(24, sorted(edges), [2] * 24, dims)
    A = O.random_network(g, 9)
    tn = gbtn.TensorNetwork(g.nv, g.edges, g.site_dims, g.edge_dims, [a.copy() for a in A])
    degs = [len(l) for l in g.legs]
    assert 1 in degs
    bpc = gbtn.BeliefPropagationCache(tn).set_tc_policy("all")
    bpc.update(maxiter=60, schedule="parallel", precision="bf16")
    is_tc, _ = bpc.tc_split()
    assert all(is_tc[v] == (degs[v] <= 4) for v in range(g.nv))
    m, _, _ = O.bp_update(g, A, O.identity_messages(g), maxiter=60, schedule="parallel")
    got = bpc.messages()
    err = max(np.max(np.abs(got[de] - m[de])) for de in range(2 * g.ne))
    assert err < 3e-2
    mix = gbtn.BeliefPropagationCache(tn).set_tc_policy("all").update(maxiter=60, schedule="parallel",
                                                                       precision="mixed")
    ref = O.expect1(g, A, m, O.SZ)
    np.testing.assert_allclose(mix.expect(O.SZ), ref, rtol=0, atol=1e-10 * np.max(np.abs(ref)))


def test_autotuned_split_on_uneven_batch():
    nets, pairs = [], []
    for k, L in enumerate([8, 12, 16]):
        tn, g, A = uneven(L, 20 + k)
        nets.append(tn)
        pairs.append((g, A))
    batch = gbtn.disjoint_union(nets)
    bpc = gbtn.BeliefPropagationCache(batch)
    is_tc, ms = bpc.tc_split()
    assert ms > 0.0
    cand = [batch.site_dims[v] == 2 and len(batch.legs[v]) <= 4 for v in range(batch.nv)]
    assert all(cand[v] for v in range(batch.nv) if is_tc[v])
    bpc.update(maxiter=300, schedule="parallel", precision="mixed")
    sz = bpc.expect(O.SZ)
    off = 0
    for g, A in pairs:
        mc, _, _ = build_oracle.run(g, O.flatten_tensors(A), O.flatten_messages(g, O.identity_messages(g)),
                                    "parallel", None, 400, tol=None, nthreads=4)
        ref = O.expect1(g, A, O.unflatten_messages(g, mc), O.SZ)
        np.testing.assert_allclose(sz[off:off + g.nv], ref, rtol=0, atol=1e-10 * np.max(np.abs(ref)))
        off += g.nv


@pytest.mark.parametrize("precision", ["bf16", "f32", "f64"])
@pytest.mark.parametrize("schedule", ["parallel", "colored"])
def test_graph_replay_matches_direct_launches(precision, schedule):
    # sweeps replayed from a captured CUDA graph give the same messages, bit for
    # bit, as the same sweeps launched one by one (7 sweeps: 1 direct + 3 replays).
    # Both plans take the fixed SIMT team rule: a measured choice is made per plan
    # and may differ between two plans, which changes the rounding.
    tn, g, A = uneven(7, 31)
    runs = []
    for graphs in (False, True):
        bpc = gbtn.BeliefPropagationCache(tn).set_tc_policy("all").set_simt_tuning(False).set_graphs(graphs)
        bpc.update(maxiter=7, schedule=schedule, precision=precision)
        first = bpc.messages()
        bpc.update(maxiter=7, schedule=schedule, precision=precision)  # reuses the cached graph
        runs.append((first, bpc.messages()))
    for k in range(2):
        for de in range(2 * g.ne):
            np.testing.assert_array_equal(runs[0][k][de], runs[1][k][de])


def test_graph_replay_keeps_convergence_bookkeeping():
    tn, g, A = uneven(6, 32)
    out = []
    for graphs in (False, True):
        bpc = gbtn.BeliefPropagationCache(tn).set_simt_tuning(128).set_graphs(graphs)
        bpc.update(maxiter=300, tol=1e-12, schedule="parallel", precision="f64")
        out.append((bpc.iterations, bpc.messages()))
    assert np.array_equal(out[0][0], out[1][0])
    for de in range(2 * g.ne):
        np.testing.assert_array_equal(out[0][1][de], out[1][1][de])


@pytest.mark.parametrize("policy", ["all", "auto"])
def test_new_factors_after_a_bf16_run_rebuild_the_images(policy):
    # set_factors on a plan that already ran BF16 uploads the tensors in pieces
    # and rebuilds the BF16 images as they land; the next sweep must equal a
    # fresh plan's sweep on the new tensors, bit for bit
    tn1, _, _ = uneven(9, 41)
    rng = np.random.default_rng(42)
    tn2 = gbtn.TensorNetwork(tn1.nv, tn1.edges, tn1.site_dims, tn1.edge_dims,
                             [rng.standard_normal(np.shape(t)) for t in tn1.tensors])  # same shapes, new values
    bpc = gbtn.BeliefPropagationCache(tn1).set_tc_policy(policy)
    bpc.update(maxiter=2, schedule="parallel", precision="bf16")
    bpc.set_factors(tn2.tensors)
    bpc.init_messages("identity")
    bpc.update(maxiter=3, schedule="parallel", precision="bf16")
    fresh = gbtn.BeliefPropagationCache(tn2).set_tc_policy(policy)
    fresh.init_messages("identity")
    fresh.update(maxiter=3, schedule="parallel", precision="bf16")
    a, b = bpc.messages(), fresh.messages()
    if policy == "all":
        for de in range(2 * tn2.ne):
            np.testing.assert_array_equal(a[de], b[de])
    else:  # the autotuned split may differ between the two plans; both are BF16-accurate
        for de in range(2 * tn2.ne):
            np.testing.assert_allclose(a[de], b[de], rtol=0, atol=3e-2)
    np.testing.assert_array_equal(np.concatenate([t.ravel() for t in bpc.factors()]),
                                  np.concatenate([np.asarray(t).ravel() for t in tn2.tensors]))


def test_bf16_message_diffs_match_the_fp64_formula():
    # the tensor-core kernel forms message_diff in FP32 as s - s^2/4 with
    # s = |a^ - b^|^2; on the FP32 messages themselves it equals the reference's
    # 1 - <a,b>^2 / (|a|^2 |b|^2) evaluated in FP64 to FP32's relative accuracy
    tn, g, A = uneven(6, 41)
    bpc = gbtn.BeliefPropagationCache(tn).set_tc_policy("all")
    bpc.update(maxiter=3, schedule="parallel", precision="bf16")
    before = bpc.messages()
    bpc.update(maxiter=1, tol=0.0, schedule="parallel", precision="bf16")
    after = bpc.messages()
    got = bpc.edge_diffs()
    want = np.array([O.message_diff(after[de].astype(np.float64), before[de].astype(np.float64))
                     for de in range(2 * g.ne)])
    assert np.all(want > 0)
    np.testing.assert_allclose(got, want, rtol=1e-4, atol=1e-10)
