"""Seeded synthetic networks of the benchmark configurations.

The reference publishes no dataset; its configurations are defined by shape
and distribution only.  These generators draw the site tensors from
``numpy.random.Generator(PCG64(seed))`` (i.i.d. N(0,1), vertex order,
column-major), so the GPU runs, the oracle fixtures and the CPU baseline all
see the same bytes."""
from __future__ import annotations

import numpy as np

from .network import TensorNetwork, disjoint_union, random_network, square_lattice


def peps_batch(batch=16, L=32, chi=8, d=2, seed0=0):
    """``batch`` independent L x L open PEPS with bond dimension chi on every
    edge, network k drawn with seed seed0 + k; returns (union, [networks])."""
    nets = [random_network(square_lattice(L, L, chi=chi, d=d), seed0 + k) for k in range(batch)]
    return disjoint_union(nets), nets


def uneven_batch(nnet=64, seed=7, lo_L=8, hi_L=32, lo_chi=2, hi_chi=8, d=2):
    """Batched BP with uneven shapes: nnet square PEPS, side lengths
    ~ U{lo_L..hi_L}, per-edge bond dimensions ~ U{lo_chi..hi_chi}, N(0,1)
    tensors (network k drawn with seed 5000 + k); returns (union, [networks])."""
    rng = np.random.default_rng(seed)
    nets = []
    for k in range(nnet):
        Lk = int(rng.integers(lo_L, hi_L + 1))
        ne = 2 * Lk * (Lk - 1)
        dims = [int(x) for x in rng.integers(lo_chi, hi_chi + 1, size=ne)]
        nets.append(random_network(square_lattice(Lk, Lk, d=d, edge_dims=dims), 5000 + k))
    return disjoint_union(nets), nets


def plus_state(L) -> TensorNetwork:
    """The L x L product state |+> with bond dimension 1 (the start of the
    transverse-field Ising simple-update run)."""
    tn = square_lattice(L, L, chi=1)
    plus = np.array([1.0, 1.0]) / np.sqrt(2)
    tn.tensors = [plus.reshape((2,) + (1,) * len(tn.legs[v])) for v in range(tn.nv)]
    return tn


def tfim_gates(L, g_field=3.0, dt=0.01):
    """Edges of the L x L lattice in checkerboard order and the gate
    exp(-dt h_e) of each, h_e = -ZZ - g (X/z_u + X/z_v) (field split over the
    z incident edges of every site); returns (order, gates, classes)."""
    from .su import checkerboard_edges, tfim_gate
    tn = square_lattice(L, L, chi=1)
    z = [len(l) for l in tn.legs]
    classes = checkerboard_edges(L, L)
    order = [e for c in classes for e in c]
    gates = [tfim_gate(dt, g_field, z[tn.edges[e][0]], z[tn.edges[e][1]]) for e in order]
    return order, gates, classes
