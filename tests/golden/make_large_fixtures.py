"""Oracle fixtures of the benchmark configurations at their full sizes.

The GPU runs of the 32x32 chi=8 batch, the 64-network uneven batch and the
20x20 transverse-field Ising simple update are compared with these FP64
oracle results (tests/test_gpu_oracle_configs.py, and bench.py's error
fields).  They are too slow to recompute inside a GPU test, so they are
generated once here and committed; regenerate with

    python tests/golden/make_large_fixtures.py [peps16|uneven64|tfim20]

* ``peps32x32_chi8_batch16.npz`` -- 16 networks (seeds 0..15, N(0,1), d=2,
  chi=8); the C restatement of the reference's parallel BP sweep
  (oracle/bp_ref.c) runs 60 FP64 sweeps from identity messages, every one of
  them (no convergence test: the mean diff reaches its rounding floor near
  1e-17, where it can turn negative, while the messages still move by ~1e-8;
  <Sz> changes by < 1e-14 after sweep 40); <Sz> per site by the NumPy oracle.
* ``uneven64_sz.npz`` -- the 64 networks of the uneven batch (L ~ U{8..32},
  chi_e ~ U{2..8}, seed 7), 100 FP64 sweeps each, <Sz> per site.
* ``tfim20x20_su200.npz`` -- 200 steps of the NumPy oracle's simple update
  (src/apply.jl:33-95, ITensors' truncation rule) on the 20x20 lattice from
  |+>, gates exp(-0.01 h_e), g = 3, checkerboard order, chi_max 8, cutoff
  1e-10, both tensors normalised after each gate; then 2000 FP64 BP sweeps of
  the final state (near the critical field BP converges slowly: <X> moves by
  < 1e-12 over the last 1000) and <X> per site, <ZZ> per edge, energy per
  site, the bond dimensions and the last step's truncation errors.
"""
from __future__ import annotations

import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT / "oracle"))
sys.path.insert(0, str(ROOT / "itensornetworks.jl_gb300"))
import bp_oracle as O  # noqa: E402
import build_oracle  # noqa: E402
from gbtn import workloads  # noqa: E402  (seeded generators only; no GPU call)


BP_SWEEPS_TFIM = 2000  # BP of the near-critical (g = 3) Ising state converges slowly


def oracle_graph(tn):
    return O.Graph(tn.nv, tn.edges, tn.site_dims, list(tn.edge_dims), [list(l) for l in tn.legs])


def sweep_c(g, A, sweeps):
    """`sweeps` FP64 parallel sweeps of the C restatement from identity
    messages, all of them run (no convergence test), then the mean message
    diff of one more sweep (a tolerance every mean passes stops it there)."""
    m0 = O.flatten_messages(g, O.identity_messages(g))
    flat = O.flatten_tensors(A)
    mc, _, _ = build_oracle.run(g, flat, m0, "parallel", None, sweeps, tol=None)
    mc, _, md = build_oracle.run(g, flat, mc, "parallel", None, 1, tol=1e300)
    return O.unflatten_messages(g, mc), md


def converged_sz(tn, sweeps):
    """<Sz> per site and the last mean diff after `sweeps` FP64 parallel sweeps."""
    g = oracle_graph(tn)
    A = [np.asarray(t, dtype=np.float64) for t in tn.tensors]
    msgs, md = sweep_c(g, A, sweeps)
    return O.expect1(g, A, msgs, O.SZ), md


def make_peps16():
    _, nets = workloads.peps_batch(16, 32, 8, 2, 0)
    sz, md = [], []
    for k, tn in enumerate(nets):
        s, d = converged_sz(tn, 60)
        sz.append(s)
        md.append(d)
        print(f"peps16 network {k}: last mean diff {d:.2e}", flush=True)
    np.savez_compressed(HERE / "peps32x32_chi8_batch16.npz", sz=np.concatenate(sz), mean_diff=np.array(md),
                        seeds=np.arange(16), L=32, chi=8, d=2, sweeps=60)


def make_uneven64():
    _, nets = workloads.uneven_batch(64, 7)
    sz, md, nv = [], [], []
    for k, tn in enumerate(nets):
        s, d = converged_sz(tn, 100)
        sz.append(s)
        md.append(d)
        nv.append(tn.nv)
        print(f"uneven64 network {k} ({tn.nv} sites): last mean diff {d:.2e}", flush=True)
    np.savez_compressed(HERE / "uneven64_sz.npz", sz=np.concatenate(sz), mean_diff=np.array(md), nv=np.array(nv),
                        seed=7, sweeps=100)


def make_tfim20(steps=200, L=20, g_field=3.0, dt=0.01, chi_max=8, cutoff=1e-10):
    tn = workloads.plus_state(L)
    order, gates, _ = workloads.tfim_gates(L, g_field, dt)
    g = oracle_graph(tn)
    A = [t.copy() for t in tn.tensors]
    t0 = time.perf_counter()
    te_last = []
    for step in range(steps):
        te_last = []
        for e, gate in zip(order, gates):
            u, v = g.edges[e]
            pu, pv = g.legs[u].index(e), g.legs[v].index(e)
            Au, Av, S, te = O.simple_update(gate, A[u], A[v], pu, pv, {}, {}, maxdim=chi_max, cutoff=cutoff)
            A[u], A[v] = Au / np.linalg.norm(Au), Av / np.linalg.norm(Av)
            g.edge_dims[e] = Au.shape[pu + 1]
            te_last.append(te)
        if step % 20 == 0:
            print(f"tfim20 step {step}: {time.perf_counter() - t0:.0f} s, max bond {max(g.edge_dims)}", flush=True)
    half, _ = sweep_c(g, A, BP_SWEEPS_TFIM // 2)
    msgs, md = sweep_c(g, A, BP_SWEEPS_TFIM)
    x = O.expect1(g, A, msgs, O.PX)
    print(f"tfim20: <X> change over the last {BP_SWEEPS_TFIM // 2} BP sweeps "
          f"{np.max(np.abs(x - O.expect1(g, A, half, O.PX))):.2e}", flush=True)
    zz = O.expect2(g, A, msgs, np.kron(O.PZ, O.PZ))
    energy = float((-np.sum(zz) - g_field * np.sum(x)) / g.nv)
    print(f"tfim20: <X> {np.mean(x):.10f}, energy/site {energy:.10f}, last BP diff {md:.2e}", flush=True)
    np.savez_compressed(HERE / "tfim20x20_su200.npz", x=x, zz=zz, energy_per_site=energy,
                        edge_dims=np.array(g.edge_dims), truncerr_last_step=np.array(te_last), bp_mean_diff=md,
                        L=L, steps=steps, g=g_field, dt=dt, chi_max=chi_max, cutoff=cutoff, bp_sweeps=BP_SWEEPS_TFIM)


if __name__ == "__main__":
    which = sys.argv[1:] or ["peps16", "uneven64", "tfim20"]
    for w in which:
        t0 = time.perf_counter()
        {"peps16": make_peps16, "uneven64": make_uneven64, "tfim20": make_tfim20}[w]()
        print(f"{w}: {time.perf_counter() - t0:.0f} s", flush=True)
