"""Benchmark of the BP hot path: belief-propagation message updates per second.

Workload (default): a batch of 16 independent 32x32 open PEPS, d=2, chi=8,
i.i.d. N(0,1) site tensors (seeded), all-edges-at-once (Jacobi) sweeps.  One
step = one sweep over the whole batch = 16 * 3968 directed-edge message
updates.  The chosen path runs the contractions in BF16 on the tensor cores
(FP32 accumulation, FP64 normalisation); the plain FP64 and the FP32 paths
are measured beside it, and the mixed pipeline (BF16 -> FP32 -> FP64
refinement) is timed to convergence against the plain FP64 path with its
<Sz> error.  The BF16 tensor images of the batch take 236 MB, the FP32 copies
486 MB and the FP64 tensors 972 MB -- all larger than L2 (129 MB), so no L2
flush is needed between steps.

Output: one JSON line (rank 0).  ``--impl reference`` times the CPU
restatement of the reference's per-edge update (FP64, all host threads) on a
bounded sample of the same workload."""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "itensornetworks.jl_gb300"))

L, CHI, D, BATCH = 32, 8, 2, 16
MSGS_PER_NET = 4 * L * (L - 1)


def flops_per_sweep(L=L, chi=CHI, d=D):
    """Algorithmic work of one sweep: per directed edge 2*d*prod(chi)*sum(chi)
    over the legs of its source vertex."""
    tot = 0
    for j in range(L):
        for i in range(L):
            k = (i > 0) + (i < L - 1) + (j > 0) + (j < L - 1)
            tot += k * 2 * d * chi ** k * (k * chi)
    return tot


def bytes_per_sweep(elt, L=L, chi=CHI, d=D):
    """Compulsory traffic of one Jacobi sweep: every site tensor read once,
    every message read once and written once."""
    tens = 0
    for j in range(L):
        for i in range(L):
            k = (i > 0) + (i < L - 1) + (j > 0) + (j < L - 1)
            tens += d * chi ** k
    msgs = MSGS_PER_NET * chi * chi
    return tens * elt + msgs * elt * 2


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                self.rows.append(parts)

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            self.proc.wait(timeout=5)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[3 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def make_batch(seed0=0):
    import gbtn
    nets = [gbtn.random_network(gbtn.square_lattice(L, L, chi=CHI, d=D), seed0 + k) for k in range(BATCH)]
    return gbtn.disjoint_union(nets)


def cpu_reference_rate(seconds=10.0, nthreads=0):
    """Messages/s of the C restatement (FP64, OpenMP over directed edges) on
    one 32x32 chi=8 network, Jacobi sweeps, until ``seconds`` elapsed."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import bp_oracle as O
    import build_oracle
    g = O.square_lattice(L, L, chi=CHI, d=D)
    A = O.flatten_tensors(O.random_network(g, 0))
    m0 = O.flatten_messages(g, O.identity_messages(g))
    build_oracle.run(g, A, m0, "parallel", None, 1, nthreads=nthreads)  # warm-up
    sweeps, t0 = 0, time.perf_counter()
    while True:
        build_oracle.run(g, A, m0, "parallel", None, 1, nthreads=nthreads)
        sweeps += 1
        el = time.perf_counter() - t0
        if el >= seconds:
            break
    cores = nthreads or os.cpu_count()
    return sweeps * MSGS_PER_NET / el, cores, f"{sweeps} Jacobi sweeps of one 32x32 chi=8 PEPS ({el:.1f} s)"


# ---- replica plumbing (one process per GPU, no data-path collective) ----------

def replica_env():
    """(rank, world size, local rank) from the torchrun environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def replica_seed(rank):
    """Seed of a rank's batch: every replica works on its own networks."""
    return 1000 * rank


def reference_runs_on(rank):
    """The CPU reference arm runs (and prints) on rank 0 only."""
    return rank == 0


def max_over_ranks(x, world, device):
    """The slowest rank's time (the job's time): all-reduce MAX over ranks."""
    if world > 1:
        import torch
        t = torch.tensor([x], device=device, dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        x = float(t.item())
    return x


def aggregate_rate(world, units_per_rank_step, ms_per_step):
    """Whole-job throughput: the units of every rank / the slowest rank's time."""
    return world * units_per_rank_step / (ms_per_step * 1e-3)


def run_reference(args):
    rank, _, _ = replica_env()
    if not reference_runs_on(rank):
        return
    rates = []
    for _ in range(args.warmup):
        cpu_reference_rate(seconds=0.5)
    for _ in range(args.steps):
        r, cores, sample = cpu_reference_rate(seconds=2.0)
        rates.append(r)
    val = float(np.mean(rates))
    line = {"impl": "reference", "metric": "bp_msg_updates_per_s", "value": val, "unit": "msg-updates/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * BATCH * MSGS_PER_NET / val, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"bp_sweep_{BATCH}x_peps32x32_d2_chi8", "batch": BATCH, "L": L, "chi": CHI, "d": D,
                       "schedule": "parallel", "l2": "inputs larger than L2"},
            "cpu_baseline": {"value": val, "unit": "msg-updates/s", "cores": cores, "kind": "port",
                             "sample": "per step: " + sample},
            "e2e": {"value": val, "unit": "msg-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def batched_uneven_timing(gbtn, ctx, stream, barrier, nnet=64, sweeps=20, seed=7):
    """Batched BP with uneven shapes: nnet independent square PEPS, side
    lengths ~ U{8..32}, per-edge bond dimensions ~ U{2..8}, d = 2, N(0,1)
    tensors, one plan.  Parallel sweeps in BF16 (tensor-core split chosen by
    the autotuner, sweeps replayed from CUDA graphs; also timed without
    graphs) and in plain FP64, msg-updates/s each; then the mixed pipeline and
    plain FP64 to convergence from the same start, max relative error of
    <Sz> per network."""
    import torch
    rng = np.random.default_rng(seed)
    nets = []
    for k in range(nnet):
        Lk = int(rng.integers(8, 33))
        ne = 2 * Lk * (Lk - 1)
        dims = [int(x) for x in rng.integers(2, 9, size=ne)]
        nets.append(gbtn.random_network(gbtn.square_lattice(Lk, Lk, d=2, edge_dims=dims), 5000 + k))
    tn = gbtn.disjoint_union(nets)
    msgs = 2 * tn.ne
    bpc = gbtn.BeliefPropagationCache(tn, ctx=ctx)
    is_tc, tune_ms = bpc.tc_split()

    def ms_per_sweep(precision, graphs, n):
        bpc.set_graphs(graphs)
        bpc.init_messages("identity")
        bpc.update(maxiter=3, schedule="parallel", precision=precision)
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        bpc.update(maxiter=n, schedule="parallel", precision=precision)
        e1.record(stream)
        barrier()
        return e0.elapsed_time(e1) / n

    ms16g = ms_per_sweep("bf16", True, sweeps)
    ms16 = ms_per_sweep("bf16", False, sweeps)
    ms64 = ms_per_sweep("f64", True, max(4, sweeps // 4))
    sz_op = np.array([[0.5, 0.0], [0.0, -0.5]])

    def solve(precision, **kw):
        bpc.set_graphs(True)
        bpc.init_messages("identity")
        barrier()
        t0 = time.perf_counter()
        bpc.update(maxiter=400, tol=1e-14, schedule="parallel", precision=precision, **kw)
        barrier()
        return (time.perf_counter() - t0) * 1e3, bpc.expect(sz_op)

    t64, sz64 = solve("f64")
    tmix, szmix = solve("mixed", refine_f64=2)
    errs, off = [], 0
    for net in nets:
        a, b = sz64[off:off + net.nv], szmix[off:off + net.nv]
        errs.append(float(np.max(np.abs(b - a)) / np.max(np.abs(a))))
        off += net.nv
    out = {"workload": f"bp_batch_{nnet}x_peps_L8-32_chi2-8_d2", "networks": nnet, "vertices": tn.nv,
           "msgs_per_sweep": msgs,
           "bf16_graph_ms_per_sweep": ms16g, "bf16_ms_per_sweep": ms16, "fp64_ms_per_sweep": ms64,
           "bf16_msg_updates_per_s": msgs / (ms16g * 1e-3), "fp64_msg_updates_per_s": msgs / (ms64 * 1e-3),
           "chosen_over_fp64_per_sweep": ms64 / ms16g,
           "tc_split": {"tensor_core_vertices": int(is_tc.sum()), "simt_vertices": int(tn.nv - is_tc.sum()),
                        "tuned_split_ms": tune_ms},
           "time_to_solution": {"tol": 1e-14, "fp64_ms": t64, "mixed_ms": tmix, "speedup": t64 / tmix,
                                "mixed_max_rel_err_sz": max(errs)}}
    bpc.close()
    return out


def gradient_timing(gbtn, ctx, barrier, rank, Lg=12, chig=6, reps=3):
    """Seconds per gradient of the BP Heisenberg energy on an Lg x Lg PEPS."""
    from gbtn.operators import HEISENBERG
    tn = gbtn.random_network(gbtn.square_lattice(Lg, Lg, chi=chig), 77, unit_norm=True)
    bpc = gbtn.BeliefPropagationCache(tn, ctx=ctx)

    def implicit():
        bpc.init_messages("identity")
        bpc.update(maxiter=300, tol=1e-13, schedule="parallel", precision="mixed", refine_f64=3)
        return bpc.energy2_grad(HEISENBERG, mode="implicit", tol=1e-10)

    def unrolled():
        return bpc.energy2_grad(HEISENBERG, mode="unrolled", unroll=30)

    out = {"workload": f"heisenberg_{Lg}x{Lg}_chi{chig}_unit_norm", "unit": "s/grad"}
    for name, fn in (("implicit", implicit), ("unrolled30", unrolled)):
        fn()
        barrier()
        t0 = time.perf_counter()
        for _ in range(reps):
            E, G = fn()
        barrier()
        out[name + "_s"] = (time.perf_counter() - t0) / reps
        out[name + "_energy"] = float(E)
    out["adjoint_iterations"] = bpc.adjoint_iterations
    bpc.close()
    if rank == 0:
        # CPU baseline: reverse-mode autograd (FP64, all host threads) through
        # 30 parallel sweeps of the oracle's restatement, one gradient
        sys.path.insert(0, str(ROOT / "oracle"))
        import bp_autograd
        import bp_oracle as O
        import torch
        g = O.square_lattice(Lg, Lg, chi=chig)
        A = O.random_network(g, 77, unit_norm=True)
        t0 = time.perf_counter()
        bp_autograd.energy_and_grad(g, A, 30)
        out["cpu_autograd_unrolled30_s"] = time.perf_counter() - t0
        out["cpu_threads"] = torch.get_num_threads()
    return out


def simple_update_timing(gbtn, ctx, barrier, rank, Ls=20, steps=200, g_field=3.0, dt=0.01, chi_max=8):
    """TFIM imaginary-time evolution by simple update: H = -sum ZZ - g sum X on an
    Ls x Ls open lattice from |+>, gates exp(-dt h_e) in checkerboard order,
    chi_max 8, cutoff 1e-10, FP64.  Reports gate updates per second and the
    BP-gauged <X> and energy per site of the final state."""
    tn = gbtn.square_lattice(Ls, Ls, chi=1)
    plus = np.array([1.0, 1.0]) / np.sqrt(2)
    tn.tensors = [plus.reshape((2,) + (1,) * len(tn.legs[v])) for v in range(tn.nv)]
    z = [len(l) for l in tn.legs]
    classes = gbtn.checkerboard_edges(Ls, Ls)
    order = [e for c in classes for e in c]
    gates = [gbtn.tfim_gate(dt, g_field, z[tn.edges[e][0]], z[tn.edges[e][1]]) for e in order]
    st = gbtn.SimpleUpdateState(tn, chi_max, ctx=ctx)
    barrier()
    t0 = time.perf_counter()
    for _ in range(steps):
        st.apply(gates, order, maxdim=chi_max, cutoff=1e-10, normalize=True)
    barrier()
    el = time.perf_counter() - t0
    t1 = time.perf_counter()
    st.apply(gates, order, maxdim=chi_max, cutoff=1e-10, normalize=True)
    barrier()
    last_step_s = time.perf_counter() - t1
    net = st.network()
    bpc = gbtn.BeliefPropagationCache(net, ctx=ctx).update(maxiter=200, tol=1e-14, schedule="parallel")
    px = np.array([[0.0, 1.0], [1.0, 0.0]])
    pz = np.array([[1.0, 0.0], [0.0, -1.0]])
    x = bpc.expect(px)
    zz = bpc.expect2(np.kron(pz, pz))
    out = {"workload": f"tfim_{Ls}x{Ls}_g{g_field}_dt{dt}_{steps}steps_chimax{chi_max}_cutoff1e-10",
           "gate_updates_per_s": steps * len(order) / el, "total_s": el,
           "gate_updates_per_s_at_chi8": len(order) / last_step_s,
           "max_bond_dim": max(st.edge_dims()), "x_per_site": float(np.mean(x)),
           "energy_per_site": float((-zz.sum() - g_field * x.sum()) / tn.nv)}
    if rank == 0:
        # CPU baseline: the oracle's FP64 simple update (NumPy/LAPACK) on the
        # gates of one step from the final state
        sys.path.insert(0, str(ROOT / "oracle"))
        import bp_oracle as O
        g = O.Graph(net.nv, net.edges, net.site_dims, list(net.edge_dims), [list(l) for l in net.legs])
        A = [t.copy() for t in net.tensors]
        t0 = time.perf_counter()
        n = 0
        for e, gate in zip(order, gates):
            u, v = g.edges[e]
            pu, pv = g.legs[u].index(e), g.legs[v].index(e)
            Au, Av, S, te = O.simple_update(gate, A[u], A[v], pu, pv, {}, {}, maxdim=chi_max, cutoff=1e-10)
            A[u], A[v] = Au / np.linalg.norm(Au), Av / np.linalg.norm(Av)
            g.edge_dims[e] = Au.shape[pu + 1]
            n += 1
            if time.perf_counter() - t0 > 10.0:
                break
        out["cpu_oracle_gate_updates_per_s_at_chi8"] = n / (time.perf_counter() - t0)
    bpc.close()
    st.close()
    return out


def run_ours(args):
    import ctypes as C

    import torch

    import gbtn
    from gbtn import _lib

    rank, world, local = replica_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    ctx = gbtn.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream)
    tn = make_batch(seed0=replica_seed(rank))
    bpc = gbtn.BeliefPropagationCache(tn, ctx=ctx)
    lib = ctx.lib
    # tensor-core routing of the BF16 phase, chosen by the library's autotuner
    # (timed on these vertices before the warm-up)
    is_tc, tune_ms = bpc.tc_split()

    def run(n, precision, tol=None, **mixed):
        o = _lib.BPOpts()
        o.schedule, o.precision, o.maxiter, o.normalize = 1, _lib.PRECISION[precision], n, 1
        o.tol = -1.0 if tol is None else tol
        o.edge_sequence = C.cast(None, C.POINTER(C.c_int32))
        o.tol_bf16 = mixed.get("tol_bf16", 0.0)
        o.tol_f32 = mixed.get("tol_f32", 0.0)
        o.refine_f64 = mixed.get("refine_f64", 0)
        if tol is None:
            _lib.check(ctx.handle, lib.gbtn_bp_run(bpc.handle, C.byref(o), None, None))
            return None
        it = np.zeros(tn.n_networks, dtype=np.int32)
        md = np.zeros(tn.n_networks)
        _lib.check(ctx.handle, lib.gbtn_bp_run(bpc.handle, C.byref(o), _lib.iptr(it), _lib.dptr(md)))
        return it

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    def max_ranks(x):
        return max_over_ranks(x, world, "cuda")

    def timed(precision, steps, warmup):
        """ms per sweep: W untimed sweeps, then K sweeps between CUDA events."""
        run(warmup, precision)
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        run(steps, precision)
        e1.record(stream)
        barrier()
        return max_ranks(e0.elapsed_time(e1) / steps)

    msgs_step = BATCH * MSGS_PER_NET
    # 1. chosen path: BF16 tensor-core sweeps (clocks sampled during the timed region)
    with ClockSampler(local) as clk:
        ms_bf16 = timed("bf16", args.steps, args.warmup)
    ms_f32 = timed("f32", args.steps, args.warmup)
    ms_f64 = timed("f64", max(2, args.steps // 2), 1)

    # 2. the dominant kernel's own duration, CUDA events around every launch
    ctx.set_profiling(True)
    run(args.steps, "bf16")
    barrier()
    tc_ms, tc_n = ctx.kernel_time(_lib.KCLASS_TENSOR_CORE)
    simt_ms, simt_n = ctx.kernel_time(_lib.KCLASS_SIMT_F32)
    ctx.set_profiling(False)

    # 3. time to solution: plain FP64 vs the mixed pipeline, same start, same tol
    sz_op = np.array([[0.5, 0.0], [0.0, -0.5]])

    def solve(precision, **kw):
        bpc.init_messages("identity")
        barrier()
        t0 = time.perf_counter()
        it = run(args.solve_maxiter, precision, tol=args.solve_tol, **kw)
        barrier()
        return (time.perf_counter() - t0) * 1e3, it

    fp64_ms, fp64_it = solve("f64")
    sz64 = bpc.expect(sz_op)
    mix_ms, mix_it = solve("mixed", refine_f64=2)
    szmix = bpc.expect(sz_op)
    per_net = []
    for k in range(BATCH):
        a = sz64[k * L * L:(k + 1) * L * L]
        b = szmix[k * L * L:(k + 1) * L * L]
        per_net.append(float(np.max(np.abs(b - a)) / np.max(np.abs(a))))

    # 4. end to end through the public API: pinned host tensors -> device, one
    #    BF16 sweep (tensor images rebuilt from the new tensors), all messages back
    n_fac, n_msg = bpc.n_factor, bpc.n_message
    host_fac = torch.from_numpy(tn.flat()).pin_memory()
    host_msg = torch.empty(n_msg, dtype=torch.float64).pin_memory()

    def e2e_step():
        _lib.check(ctx.handle, lib.gbtn_set_factors(bpc.handle, C.c_void_p(host_fac.data_ptr()), None, _lib.HOST))
        bpc.init_messages("identity")
        run(1, "bf16")
        _lib.check(ctx.handle, lib.gbtn_get_messages(bpc.handle, C.c_void_p(host_msg.data_ptr()), _lib.HOST))

    for _ in range(args.warmup):
        e2e_step()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    barrier()
    e2e_ms = max_ranks((time.perf_counter() - t0) * 1e3 / args.steps)

    # 4b. message normalisation / gauge scaling (rescale_messages, an HBM-type
    #     kernel: every message read and written once) on converged messages
    bpc.init_messages("identity")
    run(30, "f64")
    ctx.set_profiling(True)
    for _ in range(args.warmup):
        bpc.rescale_messages()
    ctx.kernel_time(_lib.KCLASS_GAUGE)  # forget the warm-up launches
    for _ in range(args.steps):
        bpc.rescale_messages()
    g_ms, g_n = ctx.kernel_time(_lib.KCLASS_GAUGE)
    ctx.set_profiling(False)
    g_launch_ms = g_ms / max(g_n, 1)
    g_bytes = 2 * n_msg * 8
    hbm_peak = (json.loads((ROOT / "MEASURED_PEAKS.json").read_text()).get("hbm_gbs")
                if (ROOT / "MEASURED_PEAKS.json").exists() else None) or 6800.0
    gauge = {"kernel": "rescale_messages_kernel", "workload": "all messages of the batch (FP64)",
             "launch_ms": g_launch_ms, "launches": g_n, "algorithmic_bytes": g_bytes,
             "achieved_gbs": g_bytes / (g_launch_ms * 1e-3) / 1e9, "peak_gbs": hbm_peak,
             "frac": g_bytes / (g_launch_ms * 1e-3) / 1e9 / hbm_peak}

    # 5. gradient of the BP energy (Heisenberg, 12x12, d=2, chi=6, unit-norm tensors):
    #    mixed-precision BP to convergence + FP64 implicit adjoint, and the
    #    checkpointed 30-sweep unrolled variant; seconds per full dE/dA
    grad = gradient_timing(gbtn, ctx, barrier, rank)
    # 6. simple update (TFIM, 20x20, 200 steps)
    su = simple_update_timing(gbtn, ctx, barrier, rank)
    # 7. batched BP with uneven shapes (64 networks, L 8..32, chi 2..8)
    batched = batched_uneven_timing(gbtn, ctx, stream, barrier)

    value = aggregate_rate(world, msgs_step, ms_bf16)
    # algorithmic flops of one tensor-core launch: every routed vertex's k
    # messages of 2 d prod(chi) sum(chi) each, at its own (unpadded) shape
    tc_v = [v for v in range(tn.nv) if is_tc[v]]
    n_tc = len(tc_v)
    alg_flops_launch = float(sum(len(tn.legs[v]) * 2.0 * tn.size(v) * sum(tn.edge_dims[e] for e in tn.legs[v])
                                 for v in tc_v))
    n_tc_native = sum(1 for v in tc_v if len(tn.legs[v]) == 4)
    mma_flops_vertex = 2 * (2 * 128 * 64 * 64) + 2 * (2 * 64 * 64 * 128)  # GEMM1, GEMM1', GEMM2, GEMM2'
    # compulsory bytes of one launch: every routed vertex's BF16 tensor at its
    # own (unpadded) shape, and each of its incoming and outgoing FP32 messages once
    alg_bytes_launch = float(sum(2 * tn.size(v) + 2 * 4 * sum(tn.edge_dims[e] ** 2 for e in tn.legs[v])
                                 for v in tc_v))
    tc_launch_ms = tc_ms / max(tc_n, 1)
    achieved = alg_flops_launch / (tc_launch_ms * 1e-3) / 1e12
    achieved_gbs = alg_bytes_launch / (tc_launch_ms * 1e-3) / 1e9
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak = peaks.get("bf16_tflops")
    peak_src = "measured burst" if peak else "fallback"
    peak = peak or 1900.0
    hbm_src = "measured" if peaks.get("hbm_gbs") else "fallback"
    # the binding roof: the arithmetic intensity (flops per compulsory byte) is
    # below the ridge point of the two peaks, so HBM caps the kernel first
    intensity = alg_flops_launch / max(alg_bytes_launch, 1.0)
    ridge = peak * 1e12 / (hbm_peak * 1e9)
    bound = "hbm" if intensity < ridge else "tensor"
    traffic = None
    tfile = ROOT / "profiles" / "tc_vertex_kernel_traffic.json"
    if tfile.exists():
        tj = json.loads(tfile.read_text())
        traffic = tj["dram_bytes_per_vertex"] * n_tc
    if rank == 0:
        cpu_val, cores, sample = cpu_reference_rate(seconds=10.0)
        cpu1_val, _, sample1 = cpu_reference_rate(seconds=3.0, nthreads=1)
        line = {
            "metric": "bp_msg_updates_per_s", "value": value, "unit": "msg-updates/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_bf16, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "bf16", "data": "synthetic",
            "config": {"workload": f"bp_sweep_{BATCH}x_peps32x32_d2_chi8", "batch": BATCH, "L": L, "chi": CHI, "d": D,
                       "schedule": "parallel (Jacobi)",
                       "chosen_path": "bf16 tcgen05 contractions (vertices padded to degree 4, chi 8; autotuned split with fp32 simt), fp32 accumulation",
                       "l2": "inputs larger than L2 (bf16 images 236 MB)", "parallelism": f"replicas{world}"},
            "paths_ms_per_sweep": {"bf16_tensor_core": ms_bf16, "f32_simt": ms_f32, "f64_simt": ms_f64},
            "chosen_over_fp64_per_sweep": ms_f64 / ms_bf16,
            "time_to_solution": {
                "tol": args.solve_tol, "fp64_ms": fp64_ms, "fp64_sweeps": int(np.max(fp64_it)),
                "mixed_ms": mix_ms, "mixed_final_fp64_sweeps": int(np.max(mix_it)),
                "speedup": fp64_ms / mix_ms, "mixed_max_rel_err_sz": max(per_net)},
            "roofline": dict(
                {"bound": "hbm", "achieved": achieved_gbs, "peak": hbm_peak, "unit": "GB/s",
                 "frac": achieved_gbs / hbm_peak, "traffic": traffic}
                if bound == "hbm" else
                {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                 "frac": achieved / peak, "traffic": traffic},
                **{"kernel": "tc_vertex_kernel", "launch_ms": tc_launch_ms, "launches": tc_n,
                   "other_kernels_ms_per_sweep": {"simt_f32": simt_ms / max(args.steps, 1)},
                   "units_per_launch": n_tc, "unit_kind": "vertex (all outgoing messages)",
                   "alg_bytes_per_launch": alg_bytes_launch, "alg_bytes_per_unit": alg_bytes_launch / max(n_tc, 1),
                   "alg_flops_per_launch": alg_flops_launch,
                   "alg_flops_per_unit": alg_flops_launch / max(n_tc, 1),
                   "intensity_flop_per_byte": intensity, "ridge_flop_per_byte": ridge,
                   "hbm": {"achieved": achieved_gbs, "peak": hbm_peak, "unit": "GB/s",
                           "frac": achieved_gbs / hbm_peak},
                   "tensor": {"achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                              "mma_issued_tflops": n_tc * mma_flops_vertex / (tc_launch_ms * 1e-3) / 1e12},
                   "tc_split": {"policy": "auto", "tensor_core_vertices": n_tc,
                                "of_which_degree4": n_tc_native, "simt_vertices": tn.nv - n_tc,
                                "tuned_split_ms": tune_ms},
                   "note": (f"algorithmic bytes and flops of the routed vertices at their unpadded shapes / "
                            f"event-timed kernel duration; bound = the roof the intensity meets first "
                            f"({hbm_src} HBM copy bandwidth, {peak_src} bf16 peak); traffic = ncu DRAM "
                            f"bytes per vertex (padded images) x vertices")}),
            "gradient": grad,
            "simple_update": su,
            "batched_uneven": batched,
            "gauge_scaling": gauge,
            "cpu_baseline": {"value": cpu_val, "unit": "msg-updates/s", "cores": cores, "kind": "port",
                             "sample": sample,
                             "single_core": {"value": cpu1_val, "unit": "msg-updates/s", "cores": 1,
                                             "sample": sample1}},
            "e2e": {"value": aggregate_rate(world, msgs_step, e2e_ms), "unit": "msg-updates/s",
                    "h2d_bytes_per_step": n_fac * 8, "d2h_bytes_per_step": n_msg * 8},
            "gpu_launches": int(tc_n + simt_n + 2),
            "clocks": clk.summary(),
        }
        print(json.dumps(line))
    bpc.close()
    ctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--batch", type=int, default=BATCH, help="networks per step (default 16; smaller for profiling)")
    ap.add_argument("--solve-tol", type=float, default=1e-14, help="tol of the time-to-solution runs")
    ap.add_argument("--solve-maxiter", type=int, default=300)
    args = ap.parse_args()
    globals()["BATCH"] = args.batch
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
