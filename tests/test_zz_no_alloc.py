"""The allocation-free sweep entry point against the plan-based one.

gbtn_bp_sweep_static serves callers that cannot allocate device memory at the
moment they run a BP sweep -- for example a framework that is capturing its
CUDA stream into a graph, or an application that hands the library a fixed
memory budget.  The caller owns every device buffer (allocated here by torch,
which stands in for such a caller); the entry point itself only launches
kernels that keep their scratch in a fixed device array.  Two sweeps in a row
must reproduce the plan-based FP64 parallel sweep (gbtn_bp_run) within the
FP64 tolerance of the other parity tests.  This file is collected last so
that a failure here cannot hide another test's result."""
import ctypes as C

import numpy as np
import pytest

import gbtn
from gbtn import _lib

pytestmark = pytest.mark.gpu


def _device_graph(tn, torch):
    """GraphDesc whose arrays live in caller-owned device memory."""
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
    d.n_networks, d.separate_bra = 1, 0
    return d, keep


def test_static_sweep_matches_plan_sweep_twice(lib_built):
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

    # allocation-free entry point on caller-owned device buffers
    lib = _lib.load()
    desc, keep = _device_graph(tn, torch)
    fac = torch.tensor(tn.flat(), dtype=torch.float64, device="cuda")
    msg = [torch.tensor(m0, dtype=torch.float64, device="cuda"), torch.zeros(len(m0), dtype=torch.float64, device="cuda")]
    mean = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    for call in range(2):
        src, dst = msg[call % 2], msg[(call + 1) % 2]
        rc = lib.gbtn_bp_sweep_static(0, C.byref(desc), fac.data_ptr(), src.data_ptr(), dst.data_ptr(),
                                      mean.data_ptr(), None)
        assert rc == 0
        torch.cuda.synchronize()
        want_msgs, want_mean = ref[call]
        np.testing.assert_allclose(dst.cpu().numpy(), want_msgs, rtol=0, atol=1e-12)
        assert float(mean.item()) == pytest.approx(want_mean, rel=1e-10, abs=1e-14)


def test_static_sweep_rejects_sizes_beyond_the_maximum(lib_built):
    lib = _lib.load()
    d = _lib.GraphDesc()
    d.nv, d.ne = 16385, 0  # GBTN_STATIC_MAX_VERTICES + 1; rejected before any device access
    buf = C.c_void_p(1)
    rc = lib.gbtn_bp_sweep_static(0, C.byref(d), buf, buf, buf, buf, None)
    assert rc == 3  # GBTN_ERR_UNSUPPORTED
