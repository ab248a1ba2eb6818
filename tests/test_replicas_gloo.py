"""Replica path of bench.py (one process per GPU, weak scaling, no
data-path collective) on CPU ranks over gloo, world size 2: each rank works
on its own batch, the job's time is the slowest rank's (all-reduce MAX), the
value aggregates every rank's units, and only rank 0 runs the CPU reference
arm."""
import os
import socket
import sys
from pathlib import Path

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(ROOT / "itensornetworks.jl_gb300"))
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        import bench
        import gbtn
        seed = bench.replica_seed(rank)
        tn = gbtn.random_network(gbtn.square_lattice(4, 4, chi=2), seed)
        t_local = 1.0 + 0.5 * rank  # this rank's (fake) ms per step
        t_job = bench.max_over_ranks(t_local, world, "cpu")
        value = bench.aggregate_rate(world, 48, t_job)
        np.savez(os.path.join(out_dir, f"rank{rank}.npz"), seed=seed, first=tn.tensors[0], t_job=t_job,
                 value=value, ref=bench.reference_runs_on(rank))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_replicas_over_gloo(tmp_path):
    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, start_method="spawn")
    r = [np.load(tmp_path / f"rank{k}.npz") for k in range(world)]
    assert int(r[0]["seed"]) != int(r[1]["seed"])
    assert not np.allclose(r[0]["first"], r[1]["first"])  # independent batches
    assert float(r[0]["t_job"]) == float(r[1]["t_job"]) == 1.5  # slowest rank
    assert float(r[0]["value"]) == pytest.approx(2 * 48 / 1.5e-3)
    assert bool(r[0]["ref"]) and not bool(r[1]["ref"])
