"""Host-side logic of the gbtn package and the C-ABI library surface (CPU)."""
import ctypes as C
import subprocess

import numpy as np
import pytest

import bp_oracle as O
import gbtn
from gbtn import _lib
from gbtn.network import default_edge_sequence, disjoint_union, parallel_edge_sequence, square_lattice


@pytest.mark.parametrize("L", [(1, 1), (2, 2), (4, 4), (5, 3), (16, 16)])
def test_lattice_bookkeeping_matches_oracle(L):
    tn = square_lattice(*L, chi=3)
    g = O.square_lattice(*L, chi=3)
    assert tn.edges == g.edges
    assert tn.legs == g.legs
    assert [tn.shape(v) for v in range(tn.nv)] == [g.shape(v) for v in range(g.nv)]


@pytest.mark.parametrize("L", [(2, 2), (4, 4), (7, 5), (32, 32)])
def test_edge_sequences_bit_exact(L):
    tn = square_lattice(*L)
    g = O.square_lattice(*L)
    seq = default_edge_sequence(tn)
    assert seq == O.default_edge_sequence(g)
    assert sorted(seq) == list(range(2 * tn.ne))  # every directed edge once per sweep
    assert parallel_edge_sequence(tn) == O.parallel_edge_sequence(g)


def test_tree_sequence_is_collect_then_distribute():
    g = O.random_tree(12, seed=2)
    tn = gbtn.TensorNetwork(g.nv, g.edges, g.site_dims, g.edge_dims)
    seq = default_edge_sequence(tn)
    assert seq == O.default_edge_sequence(g)
    half = len(seq) // 2
    assert seq[half:] == [de ^ 1 for de in reversed(seq[:half])]


def test_disjoint_union_offsets():
    a = gbtn.random_network(square_lattice(2, 2, chi=2), 1)
    b = gbtn.random_network(square_lattice(3, 2, chi=3), 2)
    u = disjoint_union([a, b])
    assert u.nv == 10 and u.ne == a.ne + b.ne and u.n_networks == 2
    assert u.vertex_network == [0] * 4 + [1] * 6
    assert u.edges[a.ne] == (b.edges[0][0] + 4, b.edges[0][1] + 4)
    assert u.legs[4] == [e + a.ne for e in b.legs[0]]
    np.testing.assert_array_equal(u.flat(), np.concatenate([a.flat(), b.flat()]))


def test_graph_desc_arrays():
    tn = square_lattice(3, 2, chi=2)
    d, keep = tn.graph_desc()
    assert d.nv == 6 and d.ne == tn.ne and d.separate_bra == 0
    lp = np.ctypeslib.as_array(d.leg_ptr, shape=(7,))
    assert list(lp) == [0] + list(np.cumsum([len(l) for l in tn.legs]))


def test_flat_roundtrip():
    tn = gbtn.random_network(square_lattice(3, 3, edge_dims=[2, 3, 1, 2, 3, 2, 1, 2, 3, 2, 2, 3]), 5)
    np.testing.assert_array_equal(tn.flat(tn.unflat(tn.flat())), tn.flat())
    msgs = O.identity_messages(O.square_lattice(3, 3, edge_dims=tn.edge_dims))
    np.testing.assert_array_equal(tn.flat_messages(tn.unflat_messages(tn.flat_messages(msgs))), tn.flat_messages(msgs))


def test_struct_layouts(tmp_path):
    """The ctypes mirrors of the ABI structs have the C compiler's sizes and
    field offsets (a C program compiled against include/gbtn.h prints them)."""
    structs = {"gbtn_graph_desc": _lib.GraphDesc, "gbtn_bp_opts": _lib.BPOpts, "gbtn_grad_opts": _lib.GradOpts}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "gbtn.h"', "int main(void) {"]
    for cname, cls in structs.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in cls._fields_:
            lines.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines.append("  return 0;\n}")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", str(_lib.INCLUDE), str(src), "-o", str(exe)], check=True)
    got = {}
    for ln in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines():
        a, b, c = ln.split()
        got[(a, b)] = int(c)
    for cname, cls in structs.items():
        assert got[(cname, "size")] == C.sizeof(cls), cname
        for fname, _ in cls._fields_:
            assert got[(cname, fname)] == getattr(cls, fname).offset, (cname, fname)


def test_library_builds_and_exports_every_declared_symbol(lib_built):
    declared = _lib.declared_symbols()
    assert "gbtn_bp_run" in declared and len(declared) >= 20
    out = subprocess.run(["nm", "-D", "--defined-only", str(lib_built)], capture_output=True, text=True, check=True)
    exported = {ln.split()[-1] for ln in out.stdout.splitlines() if " T " in ln}
    missing = [s for s in declared if s not in exported]
    assert not missing, missing
    lib = _lib.load()
    assert lib.gbtn_abi_version() == 2
    assert set(_lib.SIGNATURES) == set(declared)


def test_no_library_or_no_gpu_fails_loudly(lib_built, tmp_path):
    # the product has no CPU path: a missing libgbtn.so raises on load, and a
    # machine without a usable GPU raises when the context is made
    with pytest.raises(gbtn.LibraryNotBuilt):
        _lib.load(tmp_path / "libgbtn.so")
    import torch
    if not torch.cuda.is_available():
        with pytest.raises(gbtn.GBTNError):
            gbtn.Context(0)


def test_missing_maxiter_on_loopy_graph_raises_before_gpu():
    class Fake(gbtn.BeliefPropagationCache):
        def __init__(self, tn):
            self.tn = tn
    bpc = Fake(gbtn.random_network(square_lattice(3, 3), 1))
    with pytest.raises(gbtn.InvalidArgument, match="number of iterations"):
        bpc.update()


def test_update_factors_and_reference_named_functions():
    # update_factor / update_factors (abstractbeliefpropagationcache.jl:158-171)
    # through a cache double whose upload is recorded instead of run
    class Recording(gbtn.BeliefPropagationCache):
        def __init__(self, tn, bra=None):
            self.tn = tn
            self.separate_bra = bra is not None
            self.dtype = np.float64
            self.bra_tensors = bra
            self.uploads = []

        def set_factors(self, ket, bra=None):
            self.uploads.append((ket, bra))
            self.tn.tensors = ket

    tn = gbtn.random_network(square_lattice(3, 2), 4)
    old = list(tn.tensors)
    bpc = Recording(tn)
    new = np.ones(tn.shape(2))
    assert gbtn.update_factor(bpc, 2, new) is bpc
    ket, bra = bpc.uploads[-1]
    assert bra is None and ket[2] is new and all(ket[v] is old[v] for v in range(tn.nv) if v != 2)
    with pytest.raises(gbtn.InvalidArgument):
        bpc.update_factor(1, np.ones((3, 3)))
    with pytest.raises(gbtn.InvalidArgument):
        bpc.update_factors({tn.nv: new})
    sep = Recording(gbtn.random_network(square_lattice(3, 2), 5), bra=list(old))
    sep.update_factor(0, np.zeros(tn.shape(0)), bra_factor=np.ones(tn.shape(0)))
    ket, bra = sep.uploads[-1]
    assert np.all(ket[0] == 0) and np.all(bra[0] == 1) and bra[1] is old[1]
    ids = gbtn.identity_messages(tn)
    ref = O.identity_messages(O.square_lattice(3, 2))
    assert len(ids) == 2 * tn.ne and all(np.array_equal(a, b) for a, b in zip(ids, ref))


def test_region_scalars_read_the_vertex_and_edge_scalars():
    class Scalars(gbtn.BeliefPropagationCache):
        def __init__(self):
            pass

        def vertex_scalars(self):
            return np.array([2.0, 3.0, 5.0])

        def edge_scalars(self):
            return np.array([7.0, 11.0])

    bpc = Scalars()
    assert gbtn.region_scalar(bpc, vertex=1) == 3.0 and gbtn.region_scalar(bpc, edge=1) == 11.0
    with pytest.raises(ValueError):
        gbtn.region_scalar(bpc)
    vs, es = gbtn.scalar_factors_quotient(bpc)
    assert list(vs) == [2.0, 3.0, 5.0] and list(es) == [7.0, 11.0]


def test_incoming_messages_factors_and_default_maxiter():
    tn = gbtn.random_network(square_lattice(3, 2), 6)

    class Msgs(gbtn.BeliefPropagationCache):
        def __init__(self, tn):
            self.tn = tn

        def messages(self):
            return [np.full((c, c), float(de)) for de, c in
                    ((de, self.tn.edge_dims[de // 2]) for de in range(2 * self.tn.ne))]

        def factors(self):
            return list(self.tn.tensors)

    bpc = Msgs(tn)
    v = 4
    inc = gbtn.incoming_messages(bpc, [v])
    want = sorted(tn.directed(e, tn.other(v, e)) for e in tn.legs[v])
    assert sorted(de for de, _ in inc) == want
    assert all(np.all(m == de) for de, m in inc)
    assert sorted(de for de, _ in gbtn.incoming_messages(bpc, [v], ignore_edges=[want[0]])) == want[1:]
    assert all(a is b for a, b in zip(gbtn.factors(bpc, [1, 3]), [tn.tensors[1], tn.tensors[3]]))
    assert gbtn.default_bp_maxiter(bpc) is None  # a loopy grid: maxiter is required
    assert gbtn.default_bp_maxiter(Msgs(gbtn.random_network(square_lattice(4, 1), 1))) == 1


def test_static_sweep_refusals_before_any_device_access(lib_built):
    """gbtn_bp_sweep_static refuses, on the host and before touching a device,
    more vertices than its fixed scratch holds and a descriptor with separate
    bra tensors (it always contracts the ket with its own conjugate)."""
    lib = _lib.load()
    buf = C.c_void_p(1)
    d = _lib.GraphDesc()
    d.nv, d.ne = 16385, 0  # GBTN_STATIC_MAX_VERTICES + 1
    assert lib.gbtn_bp_sweep_static(0, C.byref(d), buf, buf, buf, buf, None) == 3  # GBTN_ERR_UNSUPPORTED
    d = _lib.GraphDesc()
    d.nv, d.ne, d.separate_bra = 4, 0, 1
    assert lib.gbtn_bp_sweep_static(0, C.byref(d), buf, buf, buf, buf, None) == 3
    d = _lib.GraphDesc()
    d.nv, d.ne, d.complex_values = 4, 0, 1
    assert lib.gbtn_bp_sweep_static(0, C.byref(d), buf, buf, buf, buf, None) == 3
