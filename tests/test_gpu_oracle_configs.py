"""The benchmark configurations at their full sizes against the FP64 oracle.

Every accuracy figure the bench reports is anchored here to the oracle, not to
the library's own FP64 kernel:

* 16 x 32x32 PEPS, d=2, chi=8 (the headline batch): the mixed pipeline solved
  to tol 1e-14 is within 1e-6 max relative <Sz> error of the oracle's
  converged fixed point on every network; the plain FP64 path after 60 sweeps
  is within 1e-10.
* the 64-network uneven batch (L ~ U{8..32}, chi_e ~ U{2..8}): the same bounds.
* the 20x20 transverse-field Ising simple update, 200 steps, chi_max 8,
  cutoff 1e-10: bond dimensions equal, <X> per site and the energy per site
  within 1e-7, last step's truncation errors within 1e-5 relative.
* one BF16 tensor-core sweep against the oracle's rounding model of that sweep
  (site tensor, Kronecker products and half-contracted tensors in BF16, FP32
  messages): within 1e-3 on unit-norm messages, 30x tighter than the plain
  FP64 comparison allows.

The oracle results at full size come from tests/golden/make_large_fixtures.py
(the C restatement of the reference's sweep and the NumPy simple update)."""
from pathlib import Path

import numpy as np
import pytest

import bp_oracle as O
import gbtn
from gbtn import workloads

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
SZ_MIXED = 1e-6   # max relative <Sz> error of the mixed pipeline (the target's bound)
SZ_FP64 = 1e-10   # plain FP64 path, converged


@pytest.fixture(scope="module", autouse=True)
def _lib(lib_built):
    yield


def per_network_rel_err(sz, ref, sizes):
    out, off = [], 0
    for n in sizes:
        a, b = ref[off:off + n], sz[off:off + n]
        out.append(float(np.max(np.abs(b - a)) / np.max(np.abs(a))))
        off += n
    return np.array(out)


def _batch_case(tn, nets, ref):
    sizes = [n.nv for n in nets]
    bpc = gbtn.BeliefPropagationCache(tn)
    bpc.update(maxiter=300, tol=1e-14, schedule="parallel", precision="mixed")
    err_mix = per_network_rel_err(bpc.expect(O.SZ), ref, sizes)
    bpc.init_messages("identity")
    bpc.update(maxiter=60, schedule="parallel", precision="f64")
    err_64 = per_network_rel_err(bpc.expect(O.SZ), ref, sizes)
    bpc.close()
    return err_mix, err_64


def test_headline_batch_mixed_and_fp64_against_oracle():
    fx = np.load(GOLDEN / "peps32x32_chi8_batch16.npz")
    tn, nets = workloads.peps_batch(16, 32, 8, 2, 0)
    err_mix, err_64 = _batch_case(tn, nets, fx["sz"])
    assert err_mix.max() <= SZ_MIXED, f"mixed: max relative <Sz> error {err_mix.max():.3e}"
    assert err_64.max() <= SZ_FP64, f"fp64: max relative <Sz> error {err_64.max():.3e}"


def test_uneven_batch_mixed_and_fp64_against_oracle():
    fx = np.load(GOLDEN / "uneven64_sz.npz")
    tn, nets = workloads.uneven_batch(64, 7)
    assert [n.nv for n in nets] == list(fx["nv"])
    err_mix, err_64 = _batch_case(tn, nets, fx["sz"])
    assert err_mix.max() <= SZ_MIXED, f"mixed: max relative <Sz> error {err_mix.max():.3e}"
    assert err_64.max() <= SZ_FP64, f"fp64: max relative <Sz> error {err_64.max():.3e}"


def test_tfim_20x20_200_steps_against_oracle():
    fx = np.load(GOLDEN / "tfim20x20_su200.npz")
    L, steps, g_field, dt = int(fx["L"]), int(fx["steps"]), float(fx["g"]), float(fx["dt"])
    chi_max, cutoff = int(fx["chi_max"]), float(fx["cutoff"])
    tn = workloads.plus_state(L)
    order, gates, _ = workloads.tfim_gates(L, g_field, dt)
    st = gbtn.SimpleUpdateState(tn, chi_max)
    te = None
    for _ in range(steps):
        te, _ = st.apply(gates, order, maxdim=chi_max, cutoff=cutoff, normalize=True)
    assert st.edge_dims() == list(fx["edge_dims"])
    np.testing.assert_allclose(te, fx["truncerr_last_step"], rtol=1e-5, atol=1e-14)
    net = st.network()
    st.close()
    bpc = gbtn.BeliefPropagationCache(net).update(maxiter=int(fx["bp_sweeps"]), schedule="parallel")
    x = bpc.expect(O.PX)
    zz = bpc.expect2(np.kron(O.PZ, O.PZ))
    energy = (-zz.sum() - g_field * x.sum()) / net.nv
    np.testing.assert_allclose(x, fx["x"], rtol=0, atol=1e-7)
    assert energy == pytest.approx(float(fx["energy_per_site"]), rel=1e-7)


def _bf16_vs_model(g, A, policy):
    m3, _, _ = O.bp_update(g, A, O.identity_messages(g), maxiter=3, schedule="parallel")
    tn = gbtn.TensorNetwork(g.nv, g.edges, g.site_dims, g.edge_dims, [a.copy() for a in A])
    bpc = gbtn.BeliefPropagationCache(tn).set_tc_policy(policy)
    bpc.set_messages(m3)
    bpc.update(maxiter=1, schedule="parallel", precision="bf16")
    got = bpc.messages()
    is_tc, _ = bpc.tc_split()
    bpc.close()
    err_model, err_fp64 = 0.0, 0.0
    n = 0
    for v in range(g.nv):
        if not is_tc[v]:
            continue
        for de, want in O.tc_bf16_messages(g, A, m3, v).items():
            err_model = max(err_model, float(np.linalg.norm(got[de] - want)))
            err_fp64 = max(err_fp64, float(np.linalg.norm(got[de] - O.updated_message(g, A, A, m3, de))))
            n += 1
    return n, err_model, err_fp64


@pytest.mark.parametrize("case", ["native6x6_chi8", "uneven5x5_chi2to8"])
def test_bf16_sweep_against_the_oracle_rounding_model(case):
    if case == "native6x6_chi8":
        g = O.square_lattice(6, 6, chi=8)
    else:
        rng = np.random.default_rng(41)
        g0 = O.square_lattice(5, 5)
        g = O.square_lattice(5, 5, edge_dims=[int(x) for x in rng.integers(2, 9, size=g0.ne)])
    A = O.random_network(g, 23)
    n, err_model, err_fp64 = _bf16_vs_model(g, A, "all")
    assert n == 2 * g.ne
    assert err_model <= 1e-3, f"BF16 sweep vs rounding model: {err_model:.3e} (vs FP64: {err_fp64:.3e})"
