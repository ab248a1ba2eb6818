"""One network split across ranks (gbtn.sharded): block bookkeeping, and the
split Jacobi sweep over gloo ranks (world size 2 and 4) reproducing the unsplit
sweep, with the FP64 oracle as each rank's compute.  The same driver on the GPU
is tested in test_gpu_sharded.py."""
import os
import socket
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT / "itensornetworks.jl_gb300"))
sys.path.insert(0, str(ROOT / "oracle"))
sys.path.insert(0, str(ROOT / "tests"))

import bp_oracle as O  # noqa: E402
import gbtn  # noqa: E402
from gbtn.sharded import ShardPlan, block_owner, run_local  # noqa: E402
from sharded_oracle import OracleShard  # noqa: E402

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _network(Lx, Ly, chi, seed):
    return gbtn.random_network(gbtn.square_lattice(Lx, Ly, chi=chi), seed)


def _unsplit(tn, sweeps, tol=None):
    g = O.Graph(tn.nv, tn.edges, tn.site_dims, tn.edge_dims, legs=[list(l) for l in tn.legs])
    return O.bp_update(g, [np.asarray(t) for t in tn.tensors], O.identity_messages(g), maxiter=sweeps, tol=tol,
                       schedule="parallel")


def test_plan_bookkeeping():
    tn = _network(5, 4, 2, 3)
    # 2 x 2 blocks of a 5 x 4 lattice (uneven widths)
    owner = [min(i * 2 // 5, 1) + 2 * min(j * 2 // 4, 1) for j in range(4) for i in range(5)]
    plans = [ShardPlan(tn, owner, r) for r in range(4)]
    owned = sorted(2 * p.gedges[lde // 2] + lde % 2 for p in plans for lde in p.owned_des)
    assert owned == list(range(2 * tn.ne))  # every directed edge computed by exactly one rank
    for p in plans:
        for q, idx in p.send.items():
            assert len(idx) == len(plans[q].recv[p.rank])
        for i, v in enumerate(p.own):  # own tensors keep their global leg order
            assert [p.gedges[le] for le in p.local.legs[i]] == tn.legs[v]
            assert p.local.shape(i) == tn.shape(v)
        for i, g in enumerate(p.ghosts):
            assert p.local.site_dims[len(p.own) + i] == 1


def test_block_owner_covers_lattice():
    own = block_owner(6, 3, 2)
    assert sorted(set(own)) == list(range(6))
    assert own[0] == 0 and own[5] == 2 and own[35] == 5


def test_split_sweep_in_one_process_matches_unsplit():
    tn = _network(6, 6, 2, 11)
    owner = block_owner(6, 2, 2)
    shards = [OracleShard(ShardPlan(tn, owner, r)) for r in range(4)]
    it, mean = run_local(shards, maxiter=7)
    ref, _, _ = _unsplit(tn, 7)
    got = {}
    for s in shards:
        got.update(s.plan.global_messages(s.get_messages()))
    assert sorted(got) == list(range(2 * tn.ne))
    err = max(float(np.max(np.abs(got[de] - ref[de]))) for de in got)
    assert it == 7 and err <= 1e-12, err


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir, blocks, sweeps, tol):
    sys.path.insert(0, str(ROOT / "itensornetworks.jl_gb300"))
    sys.path.insert(0, str(ROOT / "oracle"))
    sys.path.insert(0, str(ROOT / "tests"))
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        import gbtn
        from gbtn.sharded import ShardPlan, block_owner, run_distributed
        from sharded_oracle import OracleShard
        tn = gbtn.random_network(gbtn.square_lattice(6, 6, chi=2), 5)
        shard = OracleShard(ShardPlan(tn, block_owner(6, *blocks), rank))
        it, mean = run_distributed(shard, maxiter=sweeps, tol=tol)
        msgs = shard.plan.global_messages(shard.get_messages())
        des = np.array(sorted(msgs), dtype=np.int64)
        np.savez(os.path.join(out_dir, f"rank{rank}.npz"), it=it, mean=mean, des=des,
                 vals=np.concatenate([msgs[d].reshape(-1, order="F") for d in des]))
        dist.barrier()
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("blocks,sweeps,tol", [((2, 1), 6, None), ((2, 2), 40, 1e-9)])
def test_split_sweep_over_gloo_matches_unsplit(tmp_path, blocks, sweeps, tol):
    world = blocks[0] * blocks[1]
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path), blocks, sweeps, tol), nprocs=world,
                       start_method="spawn")
    tn = _network(6, 6, 2, 5)
    ref, ref_it, ref_mean = _unsplit(tn, sweeps, tol)
    its = set()
    for r in range(world):
        z = np.load(tmp_path / f"rank{r}.npz")
        its.add(int(z["it"]))
        off = 0
        for de in z["des"]:
            c = tn.edge_dims[de // 2]
            m = z["vals"][off:off + c * c].reshape((c, c), order="F")
            off += c * c
            assert np.max(np.abs(m - ref[de])) <= 1e-12
        if tol is not None:
            assert float(z["mean"]) == pytest.approx(ref_mean, rel=1e-9, abs=1e-15)
    assert its == {ref_it}  # every rank stops at the unsplit run's sweep
