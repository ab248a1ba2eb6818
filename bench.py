"""Benchmark of the BP hot path: belief-propagation message updates per second.

Workload (default): a batch of 16 independent 32x32 open PEPS, d=2, chi=8,
i.i.d. N(0,1) site tensors (seeds 0..15), all-edges-at-once (Jacobi) sweeps.
One step = one accuracy-matched solve of the whole batch from identity
messages: the mixed pipeline (BF16 tensor-core sweeps, FP32 sweeps, then
double-FP32 refinement sweeps with FP64 normalisation) until every network's
mean message diff is <= 1e-14.  ``value`` = message updates the solve ran
(sweeps of every phase x 63,488 directed edges) / solve time; the line also
carries the plain FP64 GPU path's time to the same tolerance (the speed-up),
the max relative <Sz> error against the FP64 oracle's converged fixed point
(tests/golden/peps32x32_chi8_batch16.npz), the per-sweep rate of every
arithmetic and each kernel's share of the solve.  The BF16 images of the
batch take 236 MB, the FP64 tensors 972 MB -- larger than L2 (129 MB), so no
L2 flush is needed between steps.

Output: one JSON line (rank 0).  ``--impl reference`` times the C
restatement of the reference's per-edge update (FP64, all host threads) on
FP64 Jacobi sweeps of the same 16-network batch, one sweep per step.
"""
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


FP32_NOMINAL_TFLOPS = 152 * 128 * 2 * 2.07e9 / 1e12  # SMs x FP32 lanes x 2 flops x max SM clock


def executed_flops_per_sweep(L=L, chi=CHI, d=D):
    """Flops the SIMT vertex kernel executes in one sweep: 12 contraction steps
    of 2 n chi at a degree-4 vertex (the shared-prefix schedule; the reference's
    per-message count is 16), the reference's count at the lower-degree
    boundary vertices (an upper bound there, 1 % of the total)."""
    tot = 0
    for j in range(L):
        for i in range(L):
            k = (i > 0) + (i < L - 1) + (j > 0) + (j < L - 1)
            n = d * chi ** k
            tot += (12 if k == 4 else k * k) * 2 * n * chi
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
    from gbtn import workloads
    return workloads.peps_batch(BATCH, L, CHI, D, seed0)[0]


def config_dict(world=1):
    """The workload, identical for both arms."""
    return {"workload": f"bp_solve_{BATCH}x_peps32x32_d2_chi8", "batch": BATCH, "L": L, "chi": CHI, "d": D,
            "schedule": "parallel (Jacobi)", "tol": 1e-14, "init": "identity messages",
            "l2": "inputs larger than L2 (fp64 tensors 972 MB)", "parallelism": f"replicas{world}"}


class CpuReference:
    """The C restatement of the reference's per-edge update (FP64, OpenMP over
    directed edges) on the first `nets` networks of the batch, FP64 Jacobi
    sweeps from identity messages."""

    def __init__(self, nets=None, nthreads=0):
        sys.path.insert(0, str(ROOT / "oracle"))
        import bp_oracle as O
        import build_oracle
        self.run_c = build_oracle.run
        tn = make_batch()
        self.nets = BATCH if nets is None else nets
        nv, ne = self.nets * L * L, self.nets * 2 * L * (L - 1)
        self.g = O.Graph(nv, tn.edges[:ne], tn.site_dims[:nv], tn.edge_dims[:ne], [list(l) for l in tn.legs[:nv]])
        self.A = tn.flat()[:sum(tn.size(v) for v in range(nv))]
        self.m0 = O.flatten_messages(self.g, O.identity_messages(self.g))
        self.nthreads = nthreads
        self.cores = nthreads or os.cpu_count()

    def sweep_s(self):
        t0 = time.perf_counter()
        self.run_c(self.g, self.A, self.m0, "parallel", None, 1, nthreads=self.nthreads)
        return time.perf_counter() - t0

    def rate(self, seconds):
        """msg-updates/s over sweeps until `seconds` elapsed (at least one)."""
        sweeps, el = 0, 0.0
        while sweeps == 0 or el < seconds:
            el += self.sweep_s()
            sweeps += 1
        return (sweeps * self.nets * MSGS_PER_NET / el,
                f"{sweeps} FP64 Jacobi sweeps of {self.nets} 32x32 chi=8 PEPS ({el:.1f} s, {self.cores} threads)")


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
    ref = CpuReference()
    for _ in range(args.warmup):
        ref.sweep_s()
    times = [ref.sweep_s() for _ in range(args.steps)]  # one FP64 sweep of the whole batch per step
    val = BATCH * MSGS_PER_NET * len(times) / sum(times)
    sample = f"per step one FP64 Jacobi sweep of the {BATCH} networks ({np.mean(times):.2f} s, {ref.cores} threads)"
    line = {"impl": "reference", "metric": "bp_msg_updates_per_s", "value": val, "unit": "msg-updates/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * float(np.mean(times)), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": config_dict(args.gpus),
            "cpu_baseline": {"value": val, "unit": "msg-updates/s", "cores": ref.cores, "kind": "port",
                             "sample": sample},
            "e2e": {"value": val, "unit": "msg-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def oracle_sz_error(sz, fixture, sizes):
    """Max over networks of max|<Sz> - oracle| / max|oracle| (the oracle's
    converged fixed point from tests/golden; None when the fixture is absent)."""
    f = ROOT / "tests" / "golden" / fixture
    if not f.exists():
        return None
    ref = np.load(f)["sz"]
    if len(ref) != len(sz):
        return None
    worst, off = 0.0, 0
    for n in sizes:
        a, b = ref[off:off + n], sz[off:off + n]
        worst = max(worst, float(np.max(np.abs(b - a)) / np.max(np.abs(a))))
        off += n
    return worst


def batched_uneven_timing(gbtn, ctx, stream, barrier, nnet=64, sweeps=20, seed=7):
    """Batched BP with uneven shapes: nnet independent square PEPS, side
    lengths ~ U{8..32}, per-edge bond dimensions ~ U{2..8}, d = 2, N(0,1)
    tensors, one plan.  Parallel sweeps in BF16 (tensor-core split chosen by
    the autotuner, sweeps replayed from CUDA graphs), DF32 and plain FP64,
    msg-updates/s each; then the mixed pipeline and plain FP64 to convergence
    from the same start, max relative error of <Sz> per network against the
    FP64 oracle's fixed point (tests/golden/uneven64_sz.npz)."""
    import torch
    from gbtn import workloads
    tn, nets = workloads.uneven_batch(nnet, seed)
    msgs = 2 * tn.ne
    bpc = gbtn.BeliefPropagationCache(tn, ctx=ctx)
    is_tc, tune_ms = bpc.tc_split()

    def ms_per_sweep(precision, n):
        bpc.set_graphs(True)
        bpc.init_messages("identity")
        bpc.update(maxiter=3, schedule="parallel", precision=precision)
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        bpc.update(maxiter=n, schedule="parallel", precision=precision)
        e1.record(stream)
        barrier()
        return e0.elapsed_time(e1) / n

    ms16 = ms_per_sweep("bf16", sweeps)
    msdf = ms_per_sweep("df32", max(4, sweeps // 4))
    ms64 = ms_per_sweep("f64", max(4, sweeps // 4))
    sz_op = np.array([[0.5, 0.0], [0.0, -0.5]])
    sizes = [n.nv for n in nets]

    def solve(precision):
        bpc.set_graphs(True)
        bpc.init_messages("identity")
        barrier()
        t0 = time.perf_counter()
        bpc.update(maxiter=400, tol=1e-14, schedule="parallel", precision=precision)
        barrier()
        return (time.perf_counter() - t0) * 1e3, bpc.expect(sz_op), bpc.phase_sweeps()

    solve("mixed")  # warm-up (graphs captured)
    t64, sz64, ph64 = solve("f64")
    tmix, szmix, phmix = solve("mixed")
    out = {"workload": f"bp_batch_{nnet}x_peps_L8-32_chi2-8_d2", "networks": nnet, "vertices": tn.nv,
           "msgs_per_sweep": msgs,
           "ms_per_sweep": {"bf16": ms16, "df32": msdf, "f64": ms64},
           "bf16_msg_updates_per_s": msgs / (ms16 * 1e-3), "fp64_msg_updates_per_s": msgs / (ms64 * 1e-3),
           "tc_split": {"tensor_core_vertices": int(is_tc.sum()), "simt_vertices": int(tn.nv - is_tc.sum()),
                        "tuned_split_ms": tune_ms},
           "time_to_solution": {"tol": 1e-14, "fp64_ms": t64, "fp64_sweeps": ph64["f64"], "mixed_ms": tmix,
                                "mixed_phase_sweeps": phmix, "speedup": t64 / tmix,
                                "mixed_max_rel_err_sz_vs_oracle": oracle_sz_error(szmix, "uneven64_sz.npz", sizes),
                                "fp64_max_rel_err_sz_vs_oracle": oracle_sz_error(sz64, "uneven64_sz.npz", sizes)}}
    bpc.close()
    return out


def large_bond_timing(gbtn, ctx, stream, barrier, nnet=4, L=8, chi=16, sweeps=4):
    """The global-memory path (bond dimensions 9..64): nnet L x L PEPS with
    chi = 16 on every link, d = 2, N(0,1) tensors; parallel sweeps per
    arithmetic and the time to solution at tol 1e-14 of the mixed pipeline (FP32
    then double-FP32 sweeps: the tensor-core kernel takes chi <= 8) against
    plain FP64.  No oracle fixture exists at this size: the errors are against
    this library's own FP64 solve run 40 sweeps further."""
    import torch
    from gbtn import workloads
    tn, _ = workloads.peps_batch(nnet, L, chi, 2, 900)
    bpc = gbtn.BeliefPropagationCache(tn, ctx=ctx).set_graphs(True)
    msgs = 2 * tn.ne
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def per_sweep(precision):
        bpc.init_messages("identity")
        bpc.update(maxiter=2, schedule="parallel", precision=precision)
        barrier()
        e0.record(stream)
        bpc.update(maxiter=sweeps, schedule="parallel", precision=precision)
        e1.record(stream)
        barrier()
        return e0.elapsed_time(e1) / sweeps

    ms = {p: per_sweep(p) for p in ("f32", "df32", "f64")}
    sz_op = np.array([[0.5, 0.0], [0.0, -0.5]])

    def solve(precision, extra=0):
        bpc.init_messages("identity")
        barrier()
        e0.record(stream)
        bpc.update(maxiter=300, tol=1e-14, schedule="parallel", precision=precision)
        e1.record(stream)
        barrier()
        t = e0.elapsed_time(e1)
        ph = bpc.phase_sweeps()
        if extra:
            bpc.update(maxiter=extra, schedule="parallel", precision="f64")
        return t, bpc.expect(sz_op), ph

    solve("mixed")
    t64, sz64, ph64 = solve("f64")
    _, szref, _ = solve("f64", extra=40)
    tmix, szmix, phmix = solve("mixed")
    rel = lambda a: float(np.max(np.abs(a - szref)) / np.max(np.abs(szref)))
    out = {"workload": f"bp_batch_{nnet}x_peps{L}x{L}_chi{chi}_d2", "msgs_per_sweep": msgs, "ms_per_sweep": ms,
           "msg_updates_per_s": {p: msgs / (v * 1e-3) for p, v in ms.items()},
           "time_to_solution": {"tol": 1e-14, "fp64_ms": t64, "fp64_sweeps": ph64["f64"], "mixed_ms": tmix,
                                "mixed_phase_sweeps": phmix, "speedup": t64 / tmix,
                                "mixed_max_rel_err_sz_vs_fp64_converged": rel(szmix),
                                "fp64_max_rel_err_sz_vs_fp64_converged": rel(sz64)}}
    bpc.close()
    return out


def qn_timing(gbtn, ctx, stream, barrier, L=24, sweeps=10):
    """Charge-conserving (U(1)) block-sparse network: an L x L PEPS with
    S=1/2 sites (charges +-1), links of dimension 8 in sectors of charge
    -1, 0, +1 (dimensions 2, 4, 2), fluxes alternating by site parity, N(0,1)
    entries in the allowed blocks.  FP64 parallel sweeps of the block-sparse
    plan against the dense plan on the same tensors expanded with zeros."""
    import torch
    tn = gbtn.square_lattice(L, L, chi=8)
    links = [[(-1, 2), (0, 4), (1, 2)]] * tn.ne
    flux = [1 if (v % L + v // L) % 2 else -1 for v in range(tn.nv)]
    q = gbtn.random_qn_network(tn, links, [[(1, 1), (-1, 1)]] * tn.nv, flux, 11, unit_norm=True)

    def ms(update):
        update(2)
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        update(sweeps)
        e1.record(stream)
        barrier()
        return e0.elapsed_time(e1) / sweeps

    qc = gbtn.QNBeliefPropagationCache(q, ctx=ctx)
    dc = gbtn.BeliefPropagationCache(q.tn, ctx=ctx)
    ms_qn = ms(lambda n: qc.update(maxiter=n, schedule="parallel"))
    ms_dense = ms(lambda n: dc.update(maxiter=n, schedule="parallel", precision="f64"))
    ms_qn_seq = ms(lambda n: qc.update(maxiter=n))  # the reference's default sequential schedule
    ms_qn32 = ms(lambda n: qc.update(maxiter=n, schedule="parallel", precision="f32"))
    ms_qndf = ms(lambda n: qc.update(maxiter=n, schedule="parallel", precision="df32"))
    qc.init_messages()
    qc.update(maxiter=sweeps + 2, schedule="parallel")
    dc.init_messages("identity")
    dc.update(maxiter=sweeps + 2, schedule="parallel", precision="f64")
    err = max(float(np.max(np.abs(a - b))) for a, b in zip(qc.messages(), dc.messages()))

    # time to solution from identity messages to a mean diff of 1e-13: FP64
    # sweeps against the mixed FP32 -> double-FP32 solve
    def solve(**kw):
        qc.init_messages()
        barrier()
        t0 = time.perf_counter()
        qc.update(maxiter=400, tol=1e-13, schedule="parallel", **kw)
        barrier()
        return 1e3 * (time.perf_counter() - t0), qc.expect(np.diag([0.5, -0.5])), qc.iterations
    solve()
    t64, sz64, it64 = solve()
    solve(precision="mixed")
    tmx, szmx, _ = solve(precision="mixed")
    out = {"workload": f"u1_peps{L}x{L}_chi8_sectors2-4-2_d2", "fp64_ms_per_sweep_block_sparse": ms_qn,
           "fp64_ms_per_sweep_dense": ms_dense, "speedup": ms_dense / ms_qn,
           "fp64_ms_per_sweep_block_sparse_sequential": ms_qn_seq,
           "fp32_ms_per_sweep_block_sparse": ms_qn32, "df32_ms_per_sweep_block_sparse": ms_qndf,
           "time_to_solution_tol1e-13_ms": {"fp64": t64, "fp64_sweeps": it64, "mixed": tmx,
                                            "mixed_phase_sweeps": qc.phase_sweeps(), "speedup": t64 / tmx,
                                            "max_abs_sz_difference": float(np.max(np.abs(szmx - sz64)))},
           "stored_elements_block_sparse": qc.n_block_elems,
           "stored_elements_dense": int(sum(q.tn.size(v) for v in range(tn.nv))),
           "max_message_difference_vs_dense": err}
    qc.close()
    dc.close()
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


FP64_NOMINAL_TFLOPS = 1.25  # GB300 dense FP64 (nominal; no measured FP64 figure is available)


def su_step_flops(net, order):
    """Algorithmic FP64 flops of one simple-update step (every gate of `order` on
    the network's current shapes, no environments): per side the Householder QR
    of the (other legs) x (site, bond) matrix, 2 m c^2 - 2 c^3 / 3 with
    c = d chi_bond; theta = R_u R_v and the gate; the SVD of theta with thin
    U and V by the Golub-Reinsch count 14 m n^2 + 8 n^3 (Golub & Van Loan);
    per side the reflectors applied to the kept columns, 4 m r k."""
    tot = 0.0
    for e in order:
        u, v = net.edges[e]
        ce = net.edge_dims[e]
        sides = []
        for x in (u, v):
            d = net.site_dims[x]
            n = d * int(np.prod([net.edge_dims[q] for q in net.legs[x]]))
            m = n // (d * ce)
            c = d * ce
            r = min(m, c)
            tot += 2.0 * m * c * c - 2.0 * c ** 3 / 3.0
            sides.append((d, m, r))
        (du, mu, ru), (dv, mv, rv) = sides
        mt, nt = ru * du, rv * dv
        tot += 2.0 * mt * nt * ce + 2.0 * mt * nt * du * dv
        big, small = max(mt, nt), min(mt, nt)
        tot += 14.0 * big * small * small + 8.0 * small ** 3
        k = min(small, ce)
        tot += 4.0 * mu * ru * k + 4.0 * mv * rv * k
    return tot


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
    # BP of this near-critical (g = 3) state converges slowly: 2000 FP64 sweeps,
    # as the oracle fixture (<X> moves by < 1e-15 over the last 1000)
    bpc = gbtn.BeliefPropagationCache(net, ctx=ctx).update(maxiter=2000, schedule="parallel")
    px = np.array([[0.0, 1.0], [1.0, 0.0]])
    pz = np.array([[1.0, 0.0], [0.0, -1.0]])
    x = bpc.expect(px)
    zz = bpc.expect2(np.kron(pz, pz))
    step_flops = su_step_flops(net, order)
    fp64 = {"flops_per_step": step_flops, "achieved_tflops": step_flops / last_step_s / 1e12,
            "peak_tflops": FP64_NOMINAL_TFLOPS, "peak_source": "nominal",
            "frac": step_flops / last_step_s / 1e12 / FP64_NOMINAL_TFLOPS,
            "count": "Householder QRs, theta and gate, SVD with thin U/V by the Golub-Reinsch count, "
                     "reflectors applied; the last step's shapes and time"}
    # the adjoint of one step at chi 8 (gbtn_su_apply_vjp per colour class, in
    # reverse, from the saved input of each class): a random cotangent of the
    # tensors after the step pulled back to its input tensors and gates
    # (a first taped step and pullback allocate the state's adjoint scratch;
    # the second pair is timed, as every step of a gradient loop after the first)
    rng = np.random.default_rng(5)
    for rep in range(2):
        barrier()
        t2 = time.perf_counter()
        _, _, pull = st.apply_with_pullback(gates, order, maxdim=chi_max, cutoff=1e-10, normalize=True)
        barrier()
        fwd_ckpt_s = time.perf_counter() - t2
        # column-major, as every gradient the library returns (energy2_grad, ...)
        cot = [rng.standard_normal(t.size).reshape(t.shape, order="F") for t in st.network().tensors]
        barrier()
        t3 = time.perf_counter()
        pull(cot)
        barrier()
        vjp_s = time.perf_counter() - t3
    out = {"workload": f"tfim_{Ls}x{Ls}_g{g_field}_dt{dt}_{steps}steps_chimax{chi_max}_cutoff1e-10",
           "gate_updates_per_s": steps * len(order) / el, "total_s": el,
           "gate_updates_per_s_at_chi8": len(order) / last_step_s, "fp64_roofline": fp64,
           "adjoint_at_chi8": {"step_s": vjp_s, "gate_vjps_per_s": len(order) / vjp_s,
                               "forward_with_checkpoints_s": fwd_ckpt_s,
                               "includes": "cotangents to and from the host; per colour class the saved device "
                                           "snapshot restored, the forward QR/SVD recomputed, the adjoint kernel"},
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
    bpc.set_graphs(True)
    lib = ctx.lib
    # tensor-core routing of the BF16 phase, chosen by the library's autotuner
    # (timed on these vertices before the warm-up)
    is_tc, tune_ms = bpc.tc_split()
    sz_op = np.array([[0.5, 0.0], [0.0, -0.5]])
    msgs_step = BATCH * MSGS_PER_NET
    sizes = [L * L] * BATCH

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    def max_ranks(x):
        return max_over_ranks(x, world, "cuda")

    def solve(precision):
        bpc.init_messages("identity")
        bpc.update(maxiter=args.solve_maxiter, tol=args.solve_tol, schedule="parallel", precision=precision)

    def sweeps_of_last_run():
        ph = bpc.phase_sweeps()
        return ph, sum(ph.values())

    # 1. the step: an accuracy-matched mixed solve of the batch (W warm-up, K timed;
    #    CUDA events on the library's stream, clocks sampled during the timed region)
    for _ in range(args.warmup):
        solve("mixed")
    barrier()
    with ClockSampler(local) as clk:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            solve("mixed")
        e1.record(stream)
        barrier()
    ms_step = max_ranks(e0.elapsed_time(e1) / args.steps)
    phases, sweeps_step = sweeps_of_last_run()
    sz_mixed = bpc.expect(sz_op)
    err_mixed = oracle_sz_error(sz_mixed, "peps32x32_chi8_batch16.npz", sizes) if rank == 0 else None
    updates_step = sweeps_step * msgs_step

    # 2. the plain FP64 GPU path to the same tolerance from the same start
    solve("f64")
    barrier()
    e0.record(stream)
    solve("f64")
    e1.record(stream)
    barrier()
    fp64_ms = max_ranks(e0.elapsed_time(e1))
    fp64_sweeps = bpc.phase_sweeps()["f64"]
    err_fp64 = (oracle_sz_error(bpc.expect(sz_op), "peps32x32_chi8_batch16.npz", sizes) if rank == 0 else None)

    # 3. kernel shares of one mixed solve (CUDA events around every launch)
    ctx.set_profiling(True)
    solve("mixed")
    barrier()
    kcls = {"tc_vertex_kernel (bf16)": _lib.KCLASS_TENSOR_CORE, "bp_vertex_kernel<float>": _lib.KCLASS_SIMT_F32,
            "bp_vertex_kernel<df32>": _lib.KCLASS_SIMT_DF32, "bp_vertex_kernel<double>": _lib.KCLASS_SIMT_F64}
    kt = {name: ctx.kernel_time(k) for name, k in kcls.items()}
    ctx.set_profiling(False)
    k_total = sum(ms for ms, _ in kt.values()) or 1.0
    shares = {name: {"ms": ms, "launches": n, "share_of_kernel_time": ms / k_total} for name, (ms, n) in kt.items()}

    # 4. per-sweep rate of every arithmetic (K sweeps between CUDA events; the
    #    tensor-core kernel's own launch time for its roofline)
    def per_sweep(precision, n):
        bpc.init_messages("identity")
        bpc.update(maxiter=max(3, args.warmup), schedule="parallel", precision=precision)
        barrier()
        e0.record(stream)
        bpc.update(maxiter=n, schedule="parallel", precision=precision)
        e1.record(stream)
        barrier()
        return max_ranks(e0.elapsed_time(e1) / n)

    ms_bf16 = per_sweep("bf16", args.steps)
    ms_f32 = per_sweep("f32", args.steps)
    ms_df32 = per_sweep("df32", max(3, args.steps // 2))
    ms_f64 = per_sweep("f64", max(2, args.steps // 4))

    # the reference's default schedule: sequential sweeps in the forest-cover
    # order, run as waves of independent messages
    def per_sweep_seq(precision, n):
        bpc.init_messages("identity")
        bpc.update(maxiter=2, schedule="sequential", precision=precision)
        barrier()
        e0.record(stream)
        bpc.update(maxiter=n, schedule="sequential", precision=precision)
        e1.record(stream)
        barrier()
        return max_ranks(e0.elapsed_time(e1) / n)

    seq_ms = {p: per_sweep_seq(p, 3) for p in ("f32", "df32", "f64")}

    # time to solution with the sequential schedule (tol as the headline): the
    # mixed pipeline's FP32 and double-FP32 waves against plain FP64 waves
    def solve_seq(precision):
        bpc.init_messages("identity")
        barrier()
        e0.record(stream)
        bpc.update(maxiter=args.solve_maxiter, tol=args.solve_tol, schedule="sequential", precision=precision)
        e1.record(stream)
        barrier()
        return max_ranks(e0.elapsed_time(e1)), bpc.expect(sz_op), bpc.phase_sweeps()

    solve_seq("mixed")
    seq64_ms, seq64_sz, seq64_ph = solve_seq("f64")
    seqmix_ms, seqmix_sz, seqmix_ph = solve_seq("mixed")
    seq_tts = {"tol": args.solve_tol, "fp64_ms": seq64_ms, "fp64_sweeps": seq64_ph["f64"], "mixed_ms": seqmix_ms,
               "mixed_phase_sweeps": seqmix_ph, "speedup": seq64_ms / seqmix_ms,
               "mixed_max_rel_err_sz_vs_oracle": oracle_sz_error(seqmix_sz, "peps32x32_chi8_batch16.npz", sizes)
               if rank == 0 else None,
               "fp64_max_rel_err_sz_vs_oracle": oracle_sz_error(seq64_sz, "peps32x32_chi8_batch16.npz", sizes)
               if rank == 0 else None}
    ctx.set_profiling(True)
    bpc.update(maxiter=args.steps, schedule="parallel", precision="bf16")
    barrier()
    tc_ms, tc_n = ctx.kernel_time(_lib.KCLASS_TENSOR_CORE)
    ctx.kernel_time(_lib.KCLASS_SIMT_F32)
    ctx.set_profiling(False)

    # 5. end to end through the public API: pinned host tensors -> device, the
    #    mixed solve, <Sz> of every site back to the host
    n_fac = bpc.n_factor
    host_fac = torch.from_numpy(tn.flat()).pin_memory()
    host_op = np.ascontiguousarray(sz_op.reshape(-1, order="F"))
    host_sz = np.zeros(tn.nv)

    def e2e_step():
        _lib.check(ctx.handle, lib.gbtn_set_factors(bpc.handle, C.c_void_p(host_fac.data_ptr()), None, _lib.HOST))
        solve("mixed")
        _lib.check(ctx.handle, lib.gbtn_expect1(bpc.handle, _lib.dptr(host_op), 0, _lib.dptr(host_sz)))

    for _ in range(args.warmup):
        e2e_step()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    barrier()
    e2e_ms = max_ranks((time.perf_counter() - t0) * 1e3 / args.steps)

    # 6. message normalisation / gauge scaling (rescale_messages, HBM-type) on converged messages
    ctx.set_profiling(True)
    for _ in range(args.warmup):
        bpc.rescale_messages()
    ctx.kernel_time(_lib.KCLASS_GAUGE)  # forget the warm-up launches
    for _ in range(args.steps):
        bpc.rescale_messages()
    g_ms, g_n = ctx.kernel_time(_lib.KCLASS_GAUGE)
    ctx.set_profiling(False)
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    hbm_peak = peaks.get("hbm_gbs") or 6800.0
    hbm_src = "measured" if peaks.get("hbm_gbs") else "fallback"
    g_launch_ms = g_ms / max(g_n, 1)
    g_bytes = 2 * bpc.n_message * 8
    gauge = {"kernel": "rescale_messages_kernel", "launch_ms": g_launch_ms, "algorithmic_bytes": g_bytes,
             "achieved_gbs": g_bytes / (g_launch_ms * 1e-3) / 1e9, "peak_gbs": hbm_peak,
             "frac": g_bytes / (g_launch_ms * 1e-3) / 1e9 / hbm_peak}

    # 7. the other configurations: gradient (c5), simple update (c4), uneven batch (c3)
    def section(fn, *a):
        """A secondary section; an error is reported in the line instead of
        losing the line (every rank runs the same sections on the same code)."""
        try:
            return fn(*a)
        except Exception as exc:  # noqa: BLE001
            torch.cuda.synchronize()
            return {"error": f"{type(exc).__name__}: {exc}"}

    grad = section(gradient_timing, gbtn, ctx, barrier, rank)
    su = section(simple_update_timing, gbtn, ctx, barrier, rank)
    batched = batched_uneven_timing(gbtn, ctx, stream, barrier)
    qn = section(qn_timing, gbtn, ctx, stream, barrier)
    large = section(large_bond_timing, gbtn, ctx, stream, barrier)

    # roofline of the tensor-core kernel: algorithmic flops and compulsory bytes of
    # the routed vertices at their own (unpadded) shapes / its event-timed launch
    tc_v = [v for v in range(tn.nv) if is_tc[v]]
    n_tc = len(tc_v)
    alg_flops = float(sum(len(tn.legs[v]) * 2.0 * tn.size(v) * sum(tn.edge_dims[e] for e in tn.legs[v])
                          for v in tc_v))
    alg_bytes = float(sum(2 * tn.size(v) + 2 * 4 * sum(tn.edge_dims[e] ** 2 for e in tn.legs[v]) for v in tc_v))
    tc_launch_ms = tc_ms / max(tc_n, 1)
    achieved_tf = alg_flops / (tc_launch_ms * 1e-3) / 1e12
    achieved_gbs = alg_bytes / (tc_launch_ms * 1e-3) / 1e9
    bf16_peak = peaks.get("bf16_tflops") or 1900.0
    bf16_src = "measured burst" if peaks.get("bf16_tflops") else "fallback"
    intensity = alg_flops / max(alg_bytes, 1.0)
    ridge = bf16_peak * 1e12 / (hbm_peak * 1e9)
    traffic = None
    tfile = ROOT / "profiles" / "tc_vertex_kernel_traffic.json"
    if tfile.exists():
        traffic = json.loads(tfile.read_text())["dram_bytes_per_vertex"] * n_tc
    mma_flops_vertex = 2 * (2 * 128 * 64 * 64) + 2 * (2 * 64 * 64 * 128)
    if intensity < ridge:
        roof = {"bound": "hbm", "achieved": achieved_gbs, "peak": hbm_peak, "unit": "GB/s",
                "frac": achieved_gbs / hbm_peak, "traffic": traffic}
    else:
        roof = {"bound": "tensor", "achieved": achieved_tf, "peak": bf16_peak, "unit": "TFLOP/s",
                "frac": achieved_tf / bf16_peak, "traffic": traffic}
    roof.update({"kernel": "tc_vertex_kernel", "launch_ms": tc_launch_ms, "units_per_launch": n_tc,
                 "unit_kind": "vertex", "alg_bytes_per_unit": alg_bytes / max(n_tc, 1),
                 "alg_flops_per_unit": alg_flops / max(n_tc, 1), "intensity": intensity, "ridge": ridge,
                 "tensor_frac": achieved_tf / bf16_peak,
                 "mma_issued_tflops": n_tc * mma_flops_vertex / (tc_launch_ms * 1e-3) / 1e12,
                 "peaks": f"{hbm_src} hbm, {bf16_src} bf16"})
    if rank == 0:
        cpu = CpuReference()
        cpu_val, sample = cpu.rate(10.0)
        cpu1_val, sample1 = CpuReference(nets=1, nthreads=1).rate(3.0)
        value = aggregate_rate(world, updates_step, ms_step)
        line = {
            "metric": "bp_msg_updates_per_s", "value": value, "unit": "msg-updates/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "bf16+f32+df32", "data": "synthetic",
            "config": config_dict(world),
            "time_to_solution": {"tol": args.solve_tol, "mixed_ms": ms_step, "fp64_ms": fp64_ms,
                                 "speedup": fp64_ms / ms_step, "mixed_phase_sweeps": phases,
                                 "fp64_sweeps": fp64_sweeps,
                                 "mixed_max_rel_err_sz_vs_oracle": err_mixed,
                                 "fp64_max_rel_err_sz_vs_oracle": err_fp64},
            # the uneven 64-network batch's accuracy-matched solve, early in the line
            "uneven_time_to_solution": {"workload": batched["workload"], **batched["time_to_solution"]},
            "e2e": {"value": aggregate_rate(world, updates_step, e2e_ms), "unit": "msg-updates/s",
                    "ms_per_step": e2e_ms, "h2d_bytes_per_step": n_fac * 8, "d2h_bytes_per_step": tn.nv * 8},
            # own kernels per timed solve: the message kernels counted above, one
            # convergence reduction per sweep, message conversions and the init
            "gpu_launches": int(sum(n for _, n in kt.values()) + sweeps_step + 4) * args.steps,
            "clocks": clk.summary(),
            "roofline": roof,
            "cpu_baseline": {"value": cpu_val, "unit": "msg-updates/s", "cores": cpu.cores, "kind": "port",
                             "sample": sample,
                             "single_core": {"value": cpu1_val, "cores": 1, "sample": sample1}},
            "chosen_path": ("mixed: bf16 tcgen05 sweeps (fp32 accumulation, autotuned split with fp32 simt), "
                            "fp32 simt sweeps, double-fp32 refinement sweeps; norms and diffs fp64"),
            "value_definition": "message updates the solve ran (every phase's sweeps x 63488) / solve time",
            "fp64_equivalent_msg_updates_per_s": aggregate_rate(world, fp64_sweeps * msgs_step, ms_step),
            "kernel_shares_of_mixed_solve": shares,
            "paths_ms_per_sweep": {"bf16_tensor_core": ms_bf16, "f32_simt": ms_f32, "df32_simt": ms_df32,
                                   "f64_simt": ms_f64},
            # the SIMT kernels that carry the solve, against the nominal FP32 pipe
            # rate (no measured FP32 peak exists for these GPUs); df32 runs ~12
            # FP32 instructions per multiply-add
            "simt_rates": {"executed_gflop_per_sweep": executed_flops_per_sweep() * BATCH / 1e9,
                           "fp32_tflops": executed_flops_per_sweep() * BATCH / (ms_f32 * 1e-3) / 1e12,
                           "fp32_frac_of_nominal": executed_flops_per_sweep() * BATCH / (ms_f32 * 1e-3) / 1e12
                           / FP32_NOMINAL_TFLOPS,
                           "df32_tflops": executed_flops_per_sweep() * BATCH / (ms_df32 * 1e-3) / 1e12,
                           "fp32_nominal_tflops": FP32_NOMINAL_TFLOPS},
            "sequential_schedule": {"ms_per_sweep": seq_ms,
                                    "msg_updates_per_s": {p: msgs_step / (ms * 1e-3) for p, ms in seq_ms.items()},
                                    "time_to_solution": seq_tts},
            "tc_split": {"tensor_core_vertices": n_tc, "simt_vertices": tn.nv - n_tc, "tuned_split_ms": tune_ms},
            "gauge_scaling": gauge,
            "batched_uneven": {k: v for k, v in batched.items() if k != "time_to_solution"},
            "qn_block_sparse": qn,
            "large_bond": large,
            "simple_update": su,
            "gradient": grad,
        }
        print(json.dumps(line))
    bpc.close()
    ctx.close()


def run_sweeps_only(args):
    """A few parallel sweeps of the batch in one arithmetic and nothing else:
    the command the ncu captures of one message kernel run (--sweeps-only).
    The sweeps compute message diffs as the solve does (a tolerance no sweep
    reaches), and take the fixed SIMT team rule so that the launch sequence is
    the same on every run (the measured choice for this batch is the same
    widths: 256 threads for the chi = 8 interior)."""
    import gbtn
    ctx = gbtn.Context(0)
    tn = make_batch()
    bpc = gbtn.BeliefPropagationCache(tn, ctx=ctx).set_simt_tuning(False)
    bpc.update(maxiter=args.warmup + args.steps, tol=1e-300, schedule="parallel", precision=args.sweeps_only)
    bpc.messages()  # waits for the sweeps
    bpc.close()
    ctx.close()


def run_su_pullback(args):
    """Profiling mode (--su-pullback L): the L x L TFIM state of the simple-update
    configuration after `steps` steps at chi 8, then one taped step and its
    pullback (the command of the adjoint kernel's ncu captures)."""
    import torch

    import gbtn
    L, chi = args.su_pullback, 8
    tn = gbtn.square_lattice(L, L, chi=1)
    plus = np.array([1.0, 1.0]) / np.sqrt(2)
    tn.tensors = [plus.reshape((2,) + (1,) * len(tn.legs[v])) for v in range(tn.nv)]
    z = [len(l) for l in tn.legs]
    order = [e for c in gbtn.checkerboard_edges(L, L) for e in c]
    gates = [gbtn.tfim_gate(0.01, 3.0, z[tn.edges[e][0]], z[tn.edges[e][1]]) for e in order]
    st = gbtn.SimpleUpdateState(tn, chi)
    for _ in range(args.steps):
        st.apply(gates, order, maxdim=chi, cutoff=1e-10, normalize=True)
    _, _, pull = st.apply_with_pullback(gates, order, maxdim=chi, cutoff=1e-10, normalize=True)
    rng = np.random.default_rng(1)
    cot = [rng.standard_normal(t.size).reshape(t.shape, order="F") for t in st.network().tensors]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    pull(cot)
    torch.cuda.synchronize()
    print(json.dumps({"su_pullback_lattice": L, "steps_before": args.steps, "max_bond_dim": max(st.edge_dims()),
                      "pullback_s": time.perf_counter() - t0}))
    st.close()


def run_qn_sweeps(args):
    """Profiling mode (--qn-sweeps PRECISION): warmup + steps parallel sweeps of
    the 24 x 24 U(1) block-sparse network of the QN section in one arithmetic
    (the command of the QN block kernel's ncu captures)."""
    import gbtn
    L = 24
    tn = gbtn.square_lattice(L, L, chi=8)
    links = [[(-1, 2), (0, 4), (1, 2)]] * tn.ne
    flux = [1 if (v % L + v // L) % 2 else -1 for v in range(tn.nv)]
    q = gbtn.random_qn_network(tn, links, [[(1, 1), (-1, 1)]] * tn.nv, flux, 11, unit_norm=True)
    qc = gbtn.QNBeliefPropagationCache(q)
    qc.update(maxiter=args.warmup + args.steps, schedule="parallel", precision=args.qn_sweeps)
    print(json.dumps({"qn_sweeps": args.qn_sweeps, "sweeps": args.warmup + args.steps,
                      "blocks": qc.n_blocks, "block_elements": qc.n_block_elems}))
    qc.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--batch", type=int, default=BATCH, help="networks per step (default 16; smaller for profiling)")
    ap.add_argument("--solve-tol", type=float, default=1e-14, help="tol of the time-to-solution runs")
    ap.add_argument("--solve-maxiter", type=int, default=300)
    ap.add_argument("--sweeps-only", default=None, choices=["f64", "f32", "df32", "bf16"],
                    help="only run warmup + steps parallel sweeps in this arithmetic (for profiler captures)")
    ap.add_argument("--su-pullback", type=int, default=0, metavar="L",
                    help="only run one taped simple-update step and its pullback on the L x L TFIM state after "
                         "--steps steps (for profiler captures)")
    ap.add_argument("--qn-sweeps", default=None, choices=["f64", "f32", "df32"],
                    help="only run warmup + steps parallel sweeps of the U(1) block-sparse network (profiler captures)")
    args = ap.parse_args()
    globals()["BATCH"] = args.batch
    if args.sweeps_only:
        run_sweeps_only(args)
    elif args.qn_sweeps:
        run_qn_sweeps(args)
    elif args.su_pullback:
        run_su_pullback(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
