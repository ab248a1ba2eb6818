"""Complex tensors (ComplexF32 / ComplexF64, test/test_belief_propagation.jl:18-20)
against the oracle, which conjugates the bra and uses the complex inner
product in message_diff.  FP64 path: messages after a fixed number of sweeps
to 1e-10 (every schedule), <Sz> and the complex log-scalar to 1e-10,
exactness on a tree, inner products with a separate bra.  FP32 path (complex
FP32 elements, the ComplexF32 case): messages after a fixed number of sweeps
to 1e-5 (parallel, coloured; 2e-5 after two sequential sweeps, whose updates compound within
a sweep; FP32 keeps 24 significant bits); the mixed pipeline
(complex FP32 sweeps, then FP64 ones to tol) reaches the FP64 fixed point to
1e-10.  Two-site RDMs and <O_u O_v> (1e-10, RDMs compared after trace
normalisation since each message keeps a free phase) and rescale_messages
(1e-12, edge scalars 1) are complex too.  Paths that take real tensors only
report GBTN_ERR_UNSUPPORTED."""
import numpy as np
import pytest

import bp_oracle as O
import gbtn

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib(lib_built):
    yield


def cnet(g, seed):
    A = O.random_network(g, seed, dtype=np.complex128, unit_norm=True)
    tn = gbtn.TensorNetwork(g.nv, g.edges, g.site_dims, g.edge_dims, [a.copy() for a in A])
    return tn, A


@pytest.mark.parametrize("schedule", ["parallel", "colored", "sequential"])
def test_complex_messages_match_oracle(schedule):
    # few sweeps: BP on this random complex network does not converge, and its
    # sequential dynamics amplify rounding differences sweep after sweep
    g = O.square_lattice(4, 4, chi=3)
    tn, A = cnet(g, 3)
    n = 4
    ref, _, _ = O.bp_update(g, A, O.identity_messages(g), maxiter=n, schedule=schedule)
    bpc = gbtn.BeliefPropagationCache(tn).update(maxiter=n, schedule=schedule)
    got = bpc.messages()
    assert all(np.iscomplexobj(m) for m in got)
    err = max(np.max(np.abs(got[de] - ref[de])) for de in range(2 * g.ne))
    assert err < 1e-10, f"{schedule}: {err:.3e}"


def test_complex_expect_logscalar_and_convergence():
    g = O.square_lattice(5, 4, chi=2)
    tn, A = cnet(g, 8)
    # converges (tol bounds 1 - cos^2 of messages) ...
    conv = gbtn.BeliefPropagationCache(tn).update(maxiter=400, tol=1e-14, schedule="parallel")
    assert conv.iterations[0] < 400
    # ... and a fixed, fully converged sweep count is compared at 1e-10
    bpc = gbtn.BeliefPropagationCache(tn).update(maxiter=400, schedule="parallel")
    m, _, _ = O.bp_update(g, A, O.identity_messages(g), maxiter=400, schedule="parallel")
    sz_ref = np.real(O.expect1(g, A, m, O.SZ))
    np.testing.assert_allclose(bpc.expect(O.SZ), sz_ref, rtol=0, atol=1e-10 * np.max(np.abs(sz_ref)))
    ls_ref = O.logscalar(g, A, A, m)
    ls = bpc.logscalar()
    assert complex(ls).real == pytest.approx(np.real(ls_ref), rel=1e-10, abs=1e-10)
    # the imaginary part of a sum of principal logs is defined modulo 2 pi
    dphi = (complex(ls).imag - np.imag(ls_ref)) / (2 * np.pi)
    assert abs(dphi - round(dphi)) < 1e-9
    # Frobenius normalisation leaves the phase of a complex message free: after
    # many sweeps the messages agree up to a phase each, which vertex scalars
    # carry and <Sz> and the log-scalar (each message once in a vertex and once
    # in an edge scalar) do not
    got = bpc.messages()
    for de in range(2 * g.ne):
        assert abs(np.vdot(got[de], m[de])) == pytest.approx(1.0, abs=1e-10)
    z = bpc.vertex_scalars()
    assert np.iscomplexobj(z) and z.shape == (g.nv,)
    np.testing.assert_allclose(np.abs(z), [abs(O.vertex_scalar(g, A, A, m, v)) for v in range(g.nv)], rtol=1e-10)


def test_complex_bp_is_exact_on_a_tree():
    g = O.random_tree(12, 5, chi=3)
    tn, A = cnet(g, 9)
    bpc = gbtn.BeliefPropagationCache(tn).update(maxiter=30, schedule="parallel")
    exact = [np.real(np.sum(O.exact_rdm1(g, A, v) * O.SZ) / np.trace(O.exact_rdm1(g, A, v))) for v in range(g.nv)]
    np.testing.assert_allclose(bpc.expect(O.SZ), exact, rtol=0, atol=1e-10)
    assert np.exp(complex(bpc.logscalar())) == pytest.approx(O.exact_scalar(g, A), rel=1e-9)


def test_complex_inner_with_separate_bra_on_a_tree():
    g = O.random_tree(10, 2, chi=2)
    tn, A = cnet(g, 4)
    _, B = cnet(g, 5)
    phi = gbtn.TensorNetwork(g.nv, g.edges, g.site_dims, g.edge_dims, [b.copy() for b in B])
    val = gbtn.inner(phi, tn, cache_update_kwargs=dict(maxiter=30, schedule="parallel"))
    assert complex(val) == pytest.approx(complex(O.exact_scalar(g, A, B)), rel=1e-9)


@pytest.mark.parametrize("schedule", ["parallel", "colored", "sequential"])
def test_complex_fp32_messages_match_oracle(schedule):
    g = O.square_lattice(4, 4, chi=3)
    tn, A = cnet(g, 3)
    # in a sequential sweep each update feeds the next, and on this
    # non-converging network FP32 rounding grows along the chain: a complex64
    # emulation of the sweep with FP32-level perturbations of the summation
    # order ends 1.5e-5 to 2.6e-3 from the FP64 result after four sweeps,
    # below 2e-7 after one and 4e-6 after two -- so two sweeps, 2e-5
    n = 2 if schedule == "sequential" else 4
    ref, _, _ = O.bp_update(g, A, O.identity_messages(g), maxiter=n, schedule=schedule)
    bpc = gbtn.BeliefPropagationCache(tn).update(maxiter=n, schedule=schedule, precision="f32")
    got = bpc.messages()
    err = max(np.max(np.abs(got[de] - ref[de])) for de in range(2 * g.ne))
    tol = 2e-5 if schedule == "sequential" else 1e-5
    assert err < tol, f"{schedule}: {err:.3e}"
    assert err > 1e-12  # the sweeps really ran in FP32


def test_complex_mixed_reaches_the_fp64_fixed_point():
    g = O.square_lattice(5, 4, chi=2)
    tn, A = cnet(g, 8)
    m, _, _ = O.bp_update(g, A, O.identity_messages(g), maxiter=400, schedule="parallel")
    sz_ref = np.real(O.expect1(g, A, m, O.SZ))
    # FP32 sweeps to their noise floor, then a full FP64 phase: the FP64 fixed point
    bpc = gbtn.BeliefPropagationCache(tn).update(maxiter=400, schedule="parallel", precision="mixed")
    np.testing.assert_allclose(bpc.expect(O.SZ), sz_ref, rtol=0, atol=1e-10 * np.max(np.abs(sz_ref)))
    got = bpc.messages()
    for de in range(2 * g.ne):  # equal up to each message's free phase
        assert abs(np.vdot(got[de], m[de])) == pytest.approx(1.0, abs=1e-10)
    # stopped at tol 1e-14 (message angles ~1e-7): within the 1e-6 bar, like plain FP64 at the same tol
    mix = gbtn.BeliefPropagationCache(tn).update(maxiter=400, tol=1e-14, schedule="parallel", precision="mixed")
    assert mix.iterations[0] < 400 and mix.mean_diff[0] <= 1e-14
    np.testing.assert_allclose(mix.expect(O.SZ), sz_ref, rtol=0, atol=1e-6 * np.max(np.abs(sz_ref)))


def test_complex_bf16_is_unsupported_and_energies_are_real_parts():
    g = O.square_lattice(3, 3, chi=2)
    tn, A = cnet(g, 1)
    bpc = gbtn.BeliefPropagationCache(tn)
    with pytest.raises(gbtn.Unsupported):
        bpc.update(maxiter=2, schedule="parallel", precision="bf16")
    # the two-site energy of a complex network: the real part of the oracle's
    bpc.init_messages("identity")
    bpc.update(maxiter=30, schedule="parallel")
    want = float(np.real(np.sum(O.expect2(g, A, bpc.messages(), np.kron(O.SZ, O.SZ)))))
    assert bpc.energy2([(1.0, O.SZ)]) == pytest.approx(want, rel=1e-10, abs=1e-13)


def test_complex_rescale_partitions_and_normalize_match_the_oracle():
    # normalize(alg="bp") of a complex state: messages rescaled, then every ket
    # divided by its norm and scaled by z^(-1/2) of its partition scalar.  On
    # random complex tensors BP amplifies rounding-level message phases about
    # threefold per sweep, so after 40 sweeps the partition scalars carry O(1)
    # phases; the library moves them onto the (phase-free) messages
    kw = dict(maxiter=40, schedule="parallel")
    g = O.square_lattice(4, 3, chi=2)
    tn, A = cnet(g, 21)
    bpc = gbtn.BeliefPropagationCache(tn).update(**kw)
    msgs = bpc.messages()
    bpc.rescale()
    ref, ref_msgs = O.normalize_bp(g, A, msgs)
    got = bpc.factors()
    for v in range(g.nv):
        np.testing.assert_allclose(got[v], ref[v], rtol=0, atol=1e-12 * np.max(np.abs(ref[v])))
    # every vertex and edge scalar 1, as in the reference's cache
    np.testing.assert_allclose(bpc.vertex_scalars(), 1.0, rtol=0, atol=1e-12)
    np.testing.assert_allclose(bpc.edge_scalars(), 1.0, rtol=0, atol=1e-12)
    # the caller's network is left alone (rescale returns a new one) ...
    assert all(np.array_equal(t, a) for t, a in zip(tn.tensors, A))
    # ... so the module-level normalize runs the same sweeps from the same
    # tensors and returns the same kets, with BP norm 1
    out = gbtn.normalize(tn, cache_update_kwargs=kw)
    for v in range(g.nv):
        np.testing.assert_allclose(out.tensors[v], ref[v], rtol=0, atol=1e-12 * np.max(np.abs(ref[v])))
    n2 = gbtn.norm_sqr(out, cache_update_kwargs=kw)
    assert abs(n2 - 1.0) < 1e-10


def test_complex_rescale_partitions_with_a_separate_bra():
    # <phi|psi> with complex phi != psi: the ket takes s*r and the bra s*s*r,
    # which brings every partition scalar to 1 whatever its phase
    g = O.square_lattice(3, 3, chi=2)
    tn, A = cnet(g, 5)
    _, B = cnet(g, 6)
    bpc = gbtn.BeliefPropagationCache(tn, bra=B).update(maxiter=100, schedule="parallel")
    msgs = bpc.messages()
    bpc.rescale_partitions()
    ref_k, ref_b = O.rescale_partitions(g, A, msgs, B)
    got = bpc.factors()
    for v in range(g.nv):
        np.testing.assert_allclose(got[v], ref_k[v], rtol=0, atol=1e-12 * np.max(np.abs(ref_k[v])))
        z = np.trace(O.contract_partition(g, {v: ref_k[v]}, {v: ref_b[v]}, msgs, v, open_site=True))
        assert abs(z - 1.0) < 1e-12
    np.testing.assert_allclose(bpc.vertex_scalars(), 1.0, rtol=0, atol=1e-12)


def test_complex_two_site_rdms_and_expect2():
    g = O.square_lattice(4, 3, chi=2)
    tn, A = cnet(g, 12)
    bpc = gbtn.BeliefPropagationCache(tn).update(maxiter=200, schedule="parallel")
    m, _, _ = O.bp_update(g, A, O.identity_messages(g), maxiter=200, schedule="parallel")
    rho = bpc.edge_rdms()
    zz = np.kron(O.SZ, O.SZ)
    for e in range(g.ne):
        ref = O.edge_rdm(g, A, A, m, e)
        # each message carries a free phase: compare the normalised RDMs
        r, rr = rho[e] / np.trace(rho[e]), ref / np.trace(ref)
        assert np.iscomplexobj(rho[e])
        np.testing.assert_allclose(r, rr, rtol=0, atol=1e-10)
    got = bpc.expect2(zz)
    ref = np.real(O.expect2(g, A, m, zz))
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-10 * np.max(np.abs(ref)))


def test_complex_rescale_messages_matches_oracle():
    g = O.square_lattice(4, 4, chi=3)
    tn, A = cnet(g, 6)
    bpc = gbtn.BeliefPropagationCache(tn).update(maxiter=3, schedule="parallel")
    before = bpc.messages()
    bpc.rescale_messages()
    got = bpc.messages()
    ref = O.rescale_messages(g, before)
    err = max(np.max(np.abs(got[de] - ref[de])) for de in range(2 * g.ne))
    assert err < 1e-12, err
    # every edge scalar <m_e, m_ebar> (no conjugation) is now 1
    np.testing.assert_allclose(bpc.edge_scalars(), np.ones(g.ne), rtol=0, atol=1e-12)
