"""Failure detection without a GPU fault: the tensor-core kernel's bounded
waits.  gbtn_ctx_test_wait_timeout makes every image copy's mbarrier expect 16
bytes more than the copy delivers, so nothing completes the barrier, the 1 s
bounded wait gives up, each CTA drains its own copies, frees its TMEM and
returns, and the sweep reports GBTN_ERR_TIMEOUT.  The plan and the context stay
usable: the next sweeps equal a fresh plan's bit for bit."""
import time

import numpy as np
import pytest

import gbtn
from gbtn import _lib

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib_built(lib_built):
    yield


def bf16_cache(tn):
    bpc = gbtn.BeliefPropagationCache(tn)
    bpc.set_tc_policy("all")  # every vertex on the tensor-core kernel, no autotuner launches
    return bpc


def test_a_wait_that_runs_out_reports_a_timeout_and_the_context_recovers():
    tn = gbtn.random_network(gbtn.square_lattice(4, 4, chi=8), 3, unit_norm=True)
    bpc = bf16_cache(tn)
    ctx = bpc.ctx
    _lib.check(ctx.handle, ctx.lib.gbtn_ctx_test_wait_timeout(ctx.handle, 1))
    try:
        t0 = time.perf_counter()
        with pytest.raises(gbtn.GBTNError) as err:
            bpc.update(maxiter=1, schedule="parallel", precision="bf16")
        elapsed = time.perf_counter() - t0
    finally:
        _lib.check(ctx.handle, ctx.lib.gbtn_ctx_test_wait_timeout(ctx.handle, 0))
    assert err.value.code == 4  # GBTN_ERR_TIMEOUT
    assert elapsed < 20.0  # one 1 s wait and one 1 s drain per CTA, all CTAs resident at once
    bpc.init_messages("identity")
    bpc.update(maxiter=3, schedule="parallel", precision="bf16")
    ref = bf16_cache(tn)
    ref.update(maxiter=3, schedule="parallel", precision="bf16")
    for a, b in zip(bpc.messages(), ref.messages()):
        np.testing.assert_array_equal(a, b)
