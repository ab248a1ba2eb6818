"""One network split into blocks on the GPU (gbtn.sharded.GpuShard, boundary
messages exchanged between the blocks after every Jacobi sweep) reproduces the
unsplit GPU sweep; the per-edge diffs the split driver's convergence test sums
(gbtn_get_edge_diffs) match the FP64 oracle's message_diff."""
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT / "itensornetworks.jl_gb300"))
sys.path.insert(0, str(ROOT / "oracle"))

import bp_oracle as O  # noqa: E402
import gbtn  # noqa: E402
from gbtn.sharded import GpuShard, ShardPlan, block_owner, run_local  # noqa: E402

pytestmark = pytest.mark.gpu


def _unsplit_gpu(tn, sweeps, tol=None):
    bpc = gbtn.BeliefPropagationCache(tn)
    bpc.init_messages("identity")
    bpc.update(maxiter=sweeps, tol=tol, schedule="parallel", precision="f64")
    return bpc


@pytest.mark.parametrize("device", ["cpu", "cuda"])
@pytest.mark.parametrize("blocks", [(2, 1), (2, 2), (3, 2)])
def test_split_gpu_sweeps_match_unsplit(blocks, device):
    # device "cuda": boundary messages gathered and scattered in device tensors
    # (the NCCL path's data movement) with the library on torch's stream
    L, sweeps = 8, 10
    tn = gbtn.random_network(gbtn.square_lattice(L, L, chi=3), 21)
    owner = block_owner(L, *blocks)
    shards = [GpuShard(ShardPlan(tn, owner, r)) for r in range(blocks[0] * blocks[1])]
    it, _ = run_local(shards, maxiter=sweeps, device=device)
    ref = _unsplit_gpu(tn, sweeps).messages()
    got = {}
    for s in shards:
        got.update(s.plan.global_messages(s.get_messages()))
        s.close()
    assert it == sweeps and sorted(got) == list(range(2 * tn.ne))
    err = max(float(np.max(np.abs(got[de] - ref[de]))) for de in got)
    assert err <= 1e-12, err


@pytest.mark.parametrize("device", ["cpu", "cuda"])
def test_split_gpu_convergence_matches_unsplit(device):
    L, tol = 8, 1e-10
    tn = gbtn.random_network(gbtn.square_lattice(L, L, chi=2), 4)
    shards = [GpuShard(ShardPlan(tn, block_owner(L, 2, 2), r)) for r in range(4)]
    it, mean = run_local(shards, maxiter=200, tol=tol, device=device)
    for s in shards:
        s.close()
    ref = _unsplit_gpu(tn, 200, tol)
    assert it == int(ref.iterations[0]) and it < 200
    assert mean == pytest.approx(float(ref.mean_diff[0]), rel=1e-8, abs=1e-16)


def test_edge_diffs_match_oracle():
    tn = gbtn.random_network(gbtn.square_lattice(5, 4, chi=3), 8)
    bpc = gbtn.BeliefPropagationCache(tn)
    assert np.all(np.isnan(bpc.edge_diffs()))  # no sweep with a tolerance yet
    bpc.init_messages("identity")
    bpc.update(maxiter=3, schedule="parallel", precision="f64")
    old = bpc.messages()
    bpc.update(maxiter=1, tol=0.0, schedule="parallel", precision="f64")
    new = bpc.messages()
    d = bpc.edge_diffs()
    ref = np.array([O.message_diff(new[de], old[de]) for de in range(2 * tn.ne)])
    assert np.max(np.abs(d - ref)) <= 1e-12
    assert abs(d.mean() - float(bpc.mean_diff[0])) <= 1e-14
