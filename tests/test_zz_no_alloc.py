"""The allocation-free sweep entry point against the plan-based one and the oracle.

gbtn_bp_sweep_static serves callers that cannot allocate device memory at the
moment they run a BP sweep -- for example a framework that is capturing its
CUDA stream into a graph, or an application that hands the library a fixed
memory budget.  The caller owns every device buffer (allocated here by torch,
which stands in for such a caller); the entry point itself only launches
kernels that keep their scratch in a fixed device array.  Two sweeps in a row
must reproduce the plan-based FP64 parallel sweep (gbtn_bp_run) and the FP64
oracle's Jacobi sweep within the FP64 tolerance of the other parity tests.
This file is collected last so that a failure here cannot hide another test's
result."""
import ctypes as C

import numpy as np
import pytest

import bp_oracle as O
import gbtn
from gbtn import _lib

pytestmark = pytest.mark.gpu

ATOL = 1e-12  # unit-norm FP64 messages, as the other FP64 parity tests


def _device_graph(tn, torch):
    """GraphDesc whose arrays live in caller-owned device memory (tn: a gbtn
    network or an oracle graph; both carry edges, dimensions and legs)."""
    cols = {
        "edge_u": [u for u, _ in tn.edges],
        "edge_v": [v for _, v in tn.edges],
        "edge_dim": tn.edge_dims,
        "site_dim": tn.site_dims,
        "leg_ptr": np.concatenate([[0], np.cumsum([len(l) for l in tn.legs])]).tolist(),
        "leg_edge": [e for l in tn.legs for e in l],
    }
    keep = {k: torch.tensor(v, dtype=torch.int32, device="cuda") for k, v in cols.items()}
    d = _lib.GraphDesc()
    d.nv, d.ne = tn.nv, tn.ne
    for k, t in keep.items():
        setattr(d, k, C.cast(C.c_void_p(t.data_ptr()), C.POINTER(C.c_int32)))
    d.vertex_network = C.cast(None, C.POINTER(C.c_int32))
    d.n_networks, d.separate_bra, d.complex_values = 1, 0, 0
    return d, keep


def _oracle_sweeps(g, tensors, m0, n):
    """n FP64 Jacobi sweeps of the oracle from m0: (messages, mean diff) after each."""
    msgs = O.unflatten_messages(g, m0)
    out = []
    for _ in range(n):
        msgs, _, md = O.bp_update(g, tensors, msgs, maxiter=1, tol=0.0, schedule="parallel")
        out.append((O.flatten_messages(g, msgs), md))
    return out


def _run_static(lib, desc, fac, src, dst, mean, stream_ptr):
    return lib.gbtn_bp_sweep_static(0, C.byref(desc), fac.data_ptr(), src.data_ptr(), dst.data_ptr(),
                                    mean.data_ptr(), stream_ptr)


@pytest.mark.parametrize("on_side_stream", [False, True])
def test_static_sweep_matches_plan_sweep_and_oracle_twice(lib_built, on_side_stream):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(12)
    shape = gbtn.square_lattice(6, 5)
    dims = [int(x) for x in rng.integers(1, 9, size=shape.ne)]
    tn = gbtn.random_network(gbtn.square_lattice(6, 5, edge_dims=dims, d=2), 31)

    # existing entry point: a plan and two FP64 parallel sweeps
    bpc = gbtn.BeliefPropagationCache(tn)
    m0 = tn.flat_messages(bpc.messages())
    ref = []
    for _ in range(2):
        bpc.update(maxiter=1, tol=0.0, schedule="parallel")
        ref.append((tn.flat_messages(bpc.messages()), float(bpc.mean_diff[0])))
    g = O.Graph(tn.nv, tn.edges, tn.site_dims, tn.edge_dims, tn.legs)
    orc = _oracle_sweeps(g, O.unflatten_tensors(g, tn.flat()), m0, 2)

    # allocation-free entry point on caller-owned device buffers
    lib = _lib.load()
    desc, keep = _device_graph(tn, torch)
    fac = torch.tensor(tn.flat(), dtype=torch.float64, device="cuda")
    msg = [torch.tensor(m0, dtype=torch.float64, device="cuda"), torch.zeros(len(m0), dtype=torch.float64, device="cuda")]
    mean = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    side = torch.cuda.Stream() if on_side_stream else None
    if side is not None:
        side.wait_stream(torch.cuda.current_stream())
    for call in range(2):
        src, dst = msg[call % 2], msg[(call + 1) % 2]
        rc = _run_static(lib, desc, fac, src, dst, mean, C.c_void_p(side.cuda_stream) if side else None)
        assert rc == 0
        torch.cuda.synchronize()
        got = dst.cpu().numpy()
        want_msgs, want_mean = ref[call]
        np.testing.assert_allclose(got, want_msgs, rtol=0, atol=ATOL)
        assert float(mean.item()) == pytest.approx(want_mean, rel=1e-10, abs=1e-14)
        orc_msgs, orc_mean = orc[call]
        np.testing.assert_allclose(got, orc_msgs, rtol=0, atol=ATOL)
        assert float(mean.item()) == pytest.approx(orc_mean, rel=1e-9, abs=1e-14)


def test_static_sweep_skips_a_vertex_beyond_the_limits(lib_built):
    """A 3x3 chi=8 lattice whose centre has d = 4: its tensor holds
    4 * 8^4 = 16384 > 8192 elements.  The centre is skipped on the device: its
    outgoing entries of msg_out keep what the buffer held, *mean_diff is NaN,
    and every other vertex's messages equal the oracle's sweep."""
    torch = pytest.importorskip("torch")
    g0 = O.square_lattice(3, 3, chi=8, d=2)
    site = list(g0.site_dims)
    site[4] = 4
    g = O.Graph(g0.nv, g0.edges, site, g0.edge_dims, g0.legs)
    tensors = O.random_network(g, 5, unit_norm=True)
    m0 = O.flatten_messages(g, O.identity_messages(g))
    (want, _), = _oracle_sweeps(g, tensors, m0, 1)

    lib = _lib.load()
    desc, keep = _device_graph(g, torch)

    sentinel = 7.0
    fac = torch.tensor(O.flatten_tensors(tensors), dtype=torch.float64, device="cuda")
    src = torch.tensor(m0, dtype=torch.float64, device="cuda")
    dst = torch.full((len(m0),), sentinel, dtype=torch.float64, device="cuda")
    mean = torch.zeros(1, dtype=torch.float64, device="cuda")
    assert _run_static(lib, desc, fac, src, dst, mean, None) == 0
    torch.cuda.synchronize()
    got = dst.cpu().numpy()
    assert np.isnan(float(mean.item()))
    off = np.concatenate([[0], np.cumsum([g.edge_dims[de // 2] ** 2 for de in range(2 * g.ne)])])
    for de in range(2 * g.ne):
        sl = slice(off[de], off[de + 1])
        if g.dsrc(de) == 4:
            assert np.all(got[sl] == sentinel), de
        else:
            np.testing.assert_allclose(got[sl], want[sl], rtol=0, atol=ATOL)
