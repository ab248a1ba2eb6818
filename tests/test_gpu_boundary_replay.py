"""The Julia extension's call sequence on one plan, replayed through ctypes.

GB300BeliefPropagationCache (julia/ITensorNetworksGB300Ext.jl) keeps one
library plan for its whole life.  A user's `expect(psi, ops; alg="gb300_bp")`,
`logscalar`, `region_scalar` and `normalize(psi; alg="gb300_bp", cache!)`
become, in order: gbtn_plan_create, gbtn_set_factors, gbtn_init_messages,
gbtn_bp_run (sequential, the forest-cover sequence), gbtn_expect1 (one
operator per call, identity elsewhere), gbtn_logscalar, gbtn_vertex_scalars /
gbtn_edge_scalars, gbtn_rescale_messages + gbtn_rescale_partitions +
gbtn_get_factors.  This test makes exactly those calls on one plan, checks
every result against the oracle, and checks through gbtn_plan_counters that
the tensors went up once and no message crossed the host boundary."""
import ctypes as C

import numpy as np
import pytest

import bp_oracle as O
from gbtn import _lib
from gbtn.network import default_edge_sequence

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built(lib_built):
    yield


def counters(lib, plan):
    c = (C.c_int64 * 4)()
    assert lib.gbtn_plan_counters(plan, c) == 0
    return list(c)


def test_julia_call_sequence_on_one_plan():
    import gbtn
    g = O.square_lattice(4, 3, chi=3)
    A = O.random_network(g, 21)
    tn = gbtn.TensorNetwork(g.nv, g.edges, g.site_dims, g.edge_dims, [a.copy() for a in A])
    ctx = gbtn.Context(0)
    lib = ctx.lib
    desc, keep = tn.graph_desc()
    plan = C.c_void_p()
    _lib.check(ctx.handle, lib.gbtn_plan_create(ctx.handle, C.byref(desc), C.byref(plan)))
    try:
        flat = np.ascontiguousarray(tn.flat())
        _lib.check(ctx.handle, lib.gbtn_set_factors(plan, flat.ctypes.data, None, _lib.HOST))  # initialize_cache
        _lib.check(ctx.handle, lib.gbtn_init_messages(plan, 0))                                 # identity messages
        seq = np.ascontiguousarray(default_edge_sequence(tn), dtype=np.int32)                   # update(bpc)
        o = _lib.BPOpts()
        o.schedule, o.precision, o.maxiter, o.normalize, o.tol = 0, 0, 30, 1, -1.0
        o.edge_sequence, o.edge_sequence_len = _lib.iptr(seq), len(seq)
        _lib.check(ctx.handle, lib.gbtn_bp_run(plan, C.byref(o), None, None))
        m, _, _ = O.bp_update(g, A, O.identity_messages(g), maxiter=30, schedule="sequential",
                              edge_sequence=list(seq))
        # expect(psi, [Op("Sz", v) for v]): one call per operator, identity elsewhere
        sz = []
        for v in range(g.nv):
            ops = np.concatenate([(O.SZ if w == v else np.eye(2)).reshape(-1, order="F") for w in range(g.nv)])
            res = np.zeros(g.nv)
            _lib.check(ctx.handle, lib.gbtn_expect1(plan, _lib.dptr(np.ascontiguousarray(ops)), 1, _lib.dptr(res)))
            sz.append(res[v])
        np.testing.assert_allclose(sz, O.expect1(g, A, m, O.SZ), rtol=1e-10, atol=1e-14)
        re, im = np.zeros(1), np.zeros(1)                                                       # logscalar(bpc)
        _lib.check(ctx.handle, lib.gbtn_logscalar(plan, _lib.dptr(re), _lib.dptr(im)))
        ls = O.logscalar(g, A, A, m)
        assert complex(re[0], im[0]) == pytest.approx(complex(ls), rel=1e-10)
        vs, es = np.zeros(g.nv), np.zeros(g.ne)                                                 # region_scalar
        _lib.check(ctx.handle, lib.gbtn_vertex_scalars(plan, _lib.dptr(vs)))
        _lib.check(ctx.handle, lib.gbtn_edge_scalars(plan, _lib.dptr(es)))
        np.testing.assert_allclose(vs, [O.vertex_scalar(g, A, A, m, v) for v in range(g.nv)], rtol=1e-10)
        np.testing.assert_allclose(es, [O.edge_scalar(g, m, e) for e in range(g.ne)], rtol=1e-10)
        assert counters(lib, plan) == [1, 0, 0, 0]  # nothing but the tensors crossed the host boundary
        # normalize(psi; alg, cache!): rescale on the device, kets read back
        _lib.check(ctx.handle, lib.gbtn_rescale_messages(plan))
        _lib.check(ctx.handle, lib.gbtn_rescale_partitions(plan))
        out = np.zeros_like(flat)
        _lib.check(ctx.handle, lib.gbtn_get_factors(plan, out.ctypes.data, _lib.HOST))
        B = O.unflatten_tensors(g, out)
        mr = O.rescale_messages(g, m)
        np.testing.assert_allclose([O.vertex_scalar(g, B, B, mr, v) for v in range(g.nv)], np.ones(g.nv), rtol=1e-9)
        assert counters(lib, plan) == [1, 0, 0, 1]
    finally:
        lib.gbtn_plan_destroy(plan)
        ctx.close()
