"""Charge-conserving (QN, U(1)-graded) block-sparse networks on the GPU.

The counterpart of BP on ITensors built with ``conserve_qns = true`` (the
QN-graded loopy case of test/test_belief_propagation.jl:103-116).  Every
index is a list of sectors ``(charge, dim)``, contiguous ranges of the dense
index in the order given; a vertex tensor is nonzero only in the blocks whose
charges balance its flux,

    charge(site sector) + sum_{legs into v} q - sum_{legs out of v} q = flux[v],

where a link's charge q is counted out of ``edges[e][0]`` and into
``edges[e][1]``.  The library stores only those blocks and the diagonal
sector blocks of the messages (which stay block-diagonal under BP), and
contracts block by block (include/gbtn.h, gbtn_qn_*)."""
from __future__ import annotations

import ctypes as C
import itertools

import numpy as np

from . import _lib
from ._lib import check, dptr, iptr
from .cache import bp_opts
from .network import TensorNetwork, default_edge_sequence


def _csr(lists):
    ptr = np.zeros(len(lists) + 1, dtype=np.int32)
    for i, l in enumerate(lists):
        ptr[i + 1] = ptr[i] + len(l)
    flat = [x for l in lists for x in l]
    dims = np.ascontiguousarray([d for _, d in flat] or [1], dtype=np.int32)
    charges = np.ascontiguousarray([c for c, _ in flat] or [0], dtype=np.int32)
    return ptr, dims, charges


class QNNetwork:
    """A U(1)-graded network: the graph of ``tn`` (dense shapes, legs), sector
    lists of every link and site index, and the flux of every vertex.  The
    tensors are held dense (zero outside the allowed blocks)."""

    def __init__(self, tn: TensorNetwork, link_sectors, site_sectors, flux):
        self.tn = tn
        self.link_sectors = [[(int(c), int(d)) for c, d in s] for s in link_sectors]
        self.site_sectors = [[(int(c), int(d)) for c, d in s] for s in site_sectors]
        self.flux = [int(f) for f in flux]
        for e, s in enumerate(self.link_sectors):
            if sum(d for _, d in s) != tn.edge_dims[e]:
                raise ValueError(f"sectors of link {e} do not add up to its dimension")
        for v, s in enumerate(self.site_sectors):
            if sum(d for _, d in s) != tn.site_dims[v]:
                raise ValueError(f"sectors of site {v} do not add up to its dimension")

    # sector ranges of an index
    @staticmethod
    def _ranges(sectors):
        out, o = [], 0
        for c, d in sectors:
            out.append((c, o, o + d))
            o += d
        return out

    def allowed(self, v):
        """Sector tuples (site sector, leg sectors...) of the nonzero blocks of v."""
        tn = self.tn
        legs = tn.legs[v]
        out = []
        choices = [range(len(self.site_sectors[v]))] + [range(len(self.link_sectors[e])) for e in legs]
        for idx in itertools.product(*choices):
            q = self.site_sectors[v][idx[0]][0]
            for p, e in enumerate(legs):
                c = self.link_sectors[e][idx[p + 1]][0]
                q += -c if tn.edges[e][0] == v else c
            if q == self.flux[v]:
                out.append(idx)
        return out

    def mask(self, v):
        """Boolean mask of the nonzero entries of the dense tensor of v."""
        tn = self.tn
        m = np.zeros(tn.shape(v), dtype=bool)
        ranges = [self._ranges(self.site_sectors[v])] + [self._ranges(self.link_sectors[e]) for e in tn.legs[v]]
        for idx in self.allowed(v):
            m[tuple(slice(ranges[i][s][1], ranges[i][s][2]) for i, s in enumerate(idx))] = True
        return m

    def desc(self):
        """(QNDesc, keep-alive arrays) for gbtn_qn_plan_create."""
        ep, ed, ec = _csr(self.link_sectors)
        sp, sd, sc = _csr(self.site_sectors)
        fl = np.ascontiguousarray(self.flux, dtype=np.int32)
        keep = [ep, ed, ec, sp, sd, sc, fl]
        d = _lib.QNDesc()
        d.edge_sec_ptr, d.sec_dim, d.sec_charge = iptr(ep), iptr(ed), iptr(ec)
        d.site_sec_ptr, d.site_sec_dim, d.site_sec_charge = iptr(sp), iptr(sd), iptr(sc)
        d.flux = iptr(fl)
        return d, keep


def random_qn_network(tn: TensorNetwork, link_sectors, site_sectors, flux, seed, unit_norm=False):
    """N(0,1) entries (numpy PCG64(seed), vertex order, column-major) in the
    allowed blocks, zero elsewhere."""
    q = QNNetwork(tn, link_sectors, site_sectors, flux)
    rng = np.random.default_rng(seed)
    ts = []
    for v in range(tn.nv):
        m = q.mask(v)
        vals = rng.standard_normal(int(m.sum()))
        flat = np.zeros(m.size)
        flat[m.reshape(-1, order="F")] = vals
        t = flat.reshape(m.shape, order="F")
        if unit_norm and np.linalg.norm(t) > 0:
            t = t / np.linalg.norm(t)
        ts.append(t)
    q.tn = TensorNetwork(tn.nv, tn.edges, tn.site_dims, tn.edge_dims, ts, tn.legs)
    return q


class QNBeliefPropagationCache:
    """BeliefPropagationCache of a QN network: the nonzero blocks and the
    diagonal message blocks on the GPU, parallel (Jacobi) sweeps, environments
    and logscalar."""

    def __init__(self, qnet: QNNetwork, ctx=None):
        self.ctx = ctx or _lib.default_context()
        self.lib = self.ctx.lib
        self.q = qnet
        tn = qnet.tn
        gd, self._gkeep = tn.graph_desc()
        qd, self._qkeep = qnet.desc()
        h = C.c_void_p()
        check(self.ctx.handle, self.lib.gbtn_qn_plan_create(self.ctx.handle, C.byref(gd), C.byref(qd), C.byref(h)))
        self.handle = h
        nb = np.zeros(1, dtype=np.int32)
        ne_ = C.c_int64()
        nm = C.c_int64()
        check(self.ctx.handle, self.lib.gbtn_qn_plan_sizes(h, iptr(nb), C.byref(ne_), C.byref(nm)))
        self.n_blocks, self.n_block_elems, self.n_message = int(nb[0]), ne_.value, nm.value
        fields = np.zeros(max(self.n_blocks, 1) * 10, dtype=np.int32)
        offs = np.zeros(max(self.n_blocks, 1), dtype=np.int64)
        check(self.ctx.handle, self.lib.gbtn_qn_blocks(h, iptr(fields), offs.ctypes.data_as(C.POINTER(C.c_int64))))
        self.blocks = fields[:10 * self.n_blocks].reshape(self.n_blocks, 10)
        self.block_offsets = offs[:self.n_blocks]
        if tn.tensors is not None:
            self.set_tensors(tn.tensors)

    def _block_slices(self, b):
        v, ss = int(self.blocks[b, 0]), int(self.blocks[b, 1])
        tn = self.q.tn
        sl = [slice(*QNNetwork._ranges(self.q.site_sectors[v])[ss][1:])]
        for p, e in enumerate(tn.legs[v]):
            sk = int(self.blocks[b, 2 + p])
            sl.append(slice(*QNNetwork._ranges(self.q.link_sectors[e])[sk][1:]))
        return v, tuple(sl)

    def pack(self, tensors):
        """The nonzero blocks of dense tensors in the plan's storage order."""
        out = np.zeros(max(self.n_block_elems, 1))
        for b in range(self.n_blocks):
            v, sl = self._block_slices(b)
            blk = np.asarray(tensors[v], dtype=np.float64)[sl]
            o = int(self.block_offsets[b])
            out[o:o + blk.size] = blk.reshape(-1, order="F")
        return out

    def set_tensors(self, tensors):
        data = np.ascontiguousarray(self.pack(tensors))
        check(self.ctx.handle, self.lib.gbtn_qn_set_blocks(self.handle, C.c_void_p(data.ctypes.data), _lib.HOST))
        self._dense = [np.asarray(t, dtype=np.float64) * self.q.mask(v) for v, t in enumerate(tensors)]

    def init_messages(self):
        check(self.ctx.handle, self.lib.gbtn_qn_init_messages(self.handle))
        return self

    def update(self, maxiter=None, tol=None, schedule="sequential", edge_sequence=None, precision="f64",
               normalize=True, **mixed):
        """update(bpc; maxiter, tol, edge_sequence): the reference's default
        sequential schedule (forest-cover order unless ``edge_sequence`` is
        given) or "parallel" (Jacobi) sweeps.  maxiter defaults to 1 on trees
        and is required otherwise, as in the reference.  ``precision``: "f64",
        "f32", "df32" or "mixed" (FP32 sweeps, then double-FP32 refinement to
        tol; ``mixed`` takes the per-phase limits of the dense cache)."""
        if maxiter is None and self.q.tn.is_tree():
            maxiter = 1
        if maxiter is None:
            raise _lib.InvalidArgument(1, "You need to specify a number of iterations for BP!")
        if schedule not in ("parallel", "sequential"):
            raise _lib.InvalidArgument(1, f"unknown schedule {schedule!r}")
        seq = None
        if schedule == "sequential":
            if edge_sequence is None:
                if getattr(self, "_default_seq", None) is None:
                    self._default_seq = np.ascontiguousarray(default_edge_sequence(self.q.tn), dtype=np.int32)
                seq = self._default_seq
            else:
                seq = np.ascontiguousarray(edge_sequence, dtype=np.int32)
        it = np.zeros(1, dtype=np.int32)
        md = np.zeros(1)
        if precision == "f64" and normalize and not mixed:
            t = -1.0 if tol is None else float(tol)
            if seq is None:
                check(self.ctx.handle, self.lib.gbtn_qn_bp_run(self.handle, int(maxiter), t, iptr(it), dptr(md)))
            else:
                check(self.ctx.handle, self.lib.gbtn_qn_bp_run_sequential(self.handle, iptr(seq), len(seq),
                                                                          int(maxiter), t, iptr(it), dptr(md)))
        else:
            o = bp_opts(maxiter, tol, schedule, seq, precision, normalize, mixed)
            check(self.ctx.handle, self.lib.gbtn_qn_bp_run_ex(self.handle, C.byref(o), iptr(it), dptr(md)))
        self.iterations, self.mean_diff = int(it[0]), float(md[0])
        return self

    def phase_sweeps(self):
        """Sweeps of each phase of the last update: {"bf16", "f32", "refine", "f64"}."""
        out = np.zeros(4, dtype=np.int32)
        check(self.ctx.handle, self.lib.gbtn_qn_phase_sweeps(self.handle, iptr(out)))
        return dict(zip(("bf16", "f32", "refine", "f64"), (int(x) for x in out)))

    def messages(self):
        """Dense chi x chi messages per directed edge (block-diagonal)."""
        flat = np.zeros(max(self.n_message, 1))
        check(self.ctx.handle, self.lib.gbtn_qn_get_messages(self.handle, C.c_void_p(flat.ctypes.data), _lib.HOST))
        tn = self.q.tn
        out, o = [], 0
        for de in range(2 * tn.ne):
            e = de // 2
            m = np.zeros((tn.edge_dims[e], tn.edge_dims[e]))
            for _, a, b in QNNetwork._ranges(self.q.link_sectors[e]):
                d = b - a
                m[a:b, a:b] = flat[o:o + d * d].reshape((d, d), order="F")
                o += d * d
            out.append(m)
        return out

    def vertex_rdms(self):
        tn = self.q.tn
        n = sum(d * d for d in tn.site_dims)
        out = np.zeros(n)
        check(self.ctx.handle, self.lib.gbtn_qn_vertex_rdms(self.handle, dptr(out)))
        res, o = [], 0
        for d in tn.site_dims:
            res.append(out[o:o + d * d].reshape((d, d), order="F"))
            o += d * d
        return res

    def expect(self, op):
        """<O_v> = tr(rho_v O) / tr(rho_v) for every vertex (op: d x d, O[s', s])."""
        op = np.asarray(op, float)
        return np.array([float(np.sum(r * op) / np.trace(r)) for r in self.vertex_rdms()])

    def logscalar(self):
        re, im = np.zeros(1), np.zeros(1)
        check(self.ctx.handle, self.lib.gbtn_qn_logscalar(self.handle, dptr(re), dptr(im)))
        return complex(re[0], im[0]) if im[0] != 0.0 else float(re[0])

    def scalar(self):
        ls = self.logscalar()
        return complex(np.exp(ls)) if isinstance(ls, complex) else float(np.exp(ls))

    # -- gradients ------------------------------------------------------------
    # The dense tensors are the blocks embedded with zeros (a linear map E), and
    # dense BP from the block-diagonal messages reproduces this plan's messages,
    # so dL/d(blocks) = E^T dL/d(dense tensors): the dense plan's hand-written
    # adjoints at the QN fixed point, gathered at the allowed blocks.  The
    # gradients come back as dense arrays, zero outside the blocks (pack() gives
    # the block storage).
    def _dense_cache(self):
        from .cache import BeliefPropagationCache
        tn = self.q.tn
        net = TensorNetwork(tn.nv, tn.edges, tn.site_dims, tn.edge_dims, [t.copy() for t in self._dense], tn.legs)
        bpc = BeliefPropagationCache(net, ctx=self.ctx)
        bpc.set_messages(self.messages())
        return bpc

    def _masked(self, G):
        return [np.asarray(g) * self.q.mask(v) for v, g in enumerate(G)]

    def energy2_grad(self, terms, mode="implicit", **kw):
        """(energy, dE/dA) of sum_e sum_t c_t <O_t (x) O_t>_e at the converged
        messages (mode "implicit"), or through unrolled sweeps from identity
        messages (mode "unrolled"), as BeliefPropagationCache.energy2_grad."""
        bpc = self._dense_cache()
        try:
            E, G = bpc.energy2_grad(terms, mode=mode, **kw)
        finally:
            bpc.close()
        return E, self._masked(G)

    def logscalar_grad(self, **kw):
        """(Re logscalar, its gradient) at the converged messages."""
        bpc = self._dense_cache()
        try:
            val, G = bpc.logscalar_grad(**kw)
        finally:
            bpc.close()
        return val, self._masked(G)

    def expect_sum_grad(self, op, **kw):
        """(sum_v <op>_v, its gradient) at the converged messages."""
        bpc = self._dense_cache()
        try:
            val, G = bpc.expect_sum_grad(op, **kw)
        finally:
            bpc.close()
        return val, self._masked(G)

    def close(self):
        if getattr(self, "handle", None):
            self.lib.gbtn_qn_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
