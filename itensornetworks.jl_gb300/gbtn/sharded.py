"""Jacobi belief propagation over one network split across ranks.

A Jacobi sweep (the parallel schedule, src/caches/abstractbeliefpropagationcache.jl:294-308)
computes every message from the previous sweep's messages.  A network whose
vertices are split into blocks, one per rank, therefore sweeps block by block
with one exchange step per sweep: each rank computes the messages leaving its
own vertices, then sends the messages on cut edges (own vertex -> a vertex of
rank q) to rank q, and receives the messages entering its own vertices from
the other side.  The result after k sweeps is the unsplit network's result
after k sweeps.

Local network of a rank: its own vertices in global order, with their tensors
and leg orders, then one ghost vertex per foreign neighbour (site dimension 1,
its legs the cut edges to own vertices in its global leg order, a tensor of
ones).  Local edges are the global edges with an own endpoint, in global order
and orientation, so a local directed edge 2e'+o is global 2e+o.  The local sweep
also computes ghost -> own messages; the received messages overwrite them
before they are used, and they are left out of the convergence sum.

Convergence follows the reference's update loop (:313-329): the mean of
message_diff over every directed edge of the sweep, here summed over each
rank's own directed edges and all-reduced as (sum, count).

:class:`ShardPlan` holds the bookkeeping (plain integers, identical on every
rank), :class:`GpuShard` runs one rank's block through the library, and two
drivers move the boundary messages: :func:`run_local` (every block in one
process, exchange by copies -- one GPU or a test) and :func:`run_distributed`
(one block per process, torch.distributed point-to-point sends and an
all-reduce; NCCL between GPUs, gloo on the host).

Both drivers move boundary messages through torch tensors on an exchange
device.  On a GPU (``device="cuda"``, the default with NCCL) a block's messages
are copied device to device out of the library into one tensor, the entries of
each cut edge are gathered there and sent with NCCL, and the received entries
are scattered back before the copy into the library.  The library runs on
torch's current stream meanwhile, so the copies, gathers, NCCL waits and sweeps
are ordered on one stream and no message crosses the host.  On the host
(gloo, or a test double of a block) the same steps run on CPU tensors."""
from __future__ import annotations

import ctypes as C
from contextlib import contextmanager

import numpy as np

from . import _lib
from .network import TensorNetwork


class ShardPlan:
    """Block ``rank`` of ``tn`` under the vertex owner map ``owner[v]``."""

    def __init__(self, tn: TensorNetwork, owner, rank: int):
        owner = [int(x) for x in owner]
        if len(owner) != tn.nv:
            raise ValueError("owner needs one rank per vertex")
        self.tn, self.owner, self.rank = tn, owner, int(rank)
        own = [v for v in range(tn.nv) if owner[v] == rank]
        if not own:
            raise ValueError(f"rank {rank} owns no vertex")
        gedges = [e for e, (u, v) in enumerate(tn.edges) if owner[u] == rank or owner[v] == rank]
        ghosts = sorted({w for e in gedges for w in tn.edges[e] if owner[w] != rank})
        self.own, self.ghosts, self.gedges = own, ghosts, gedges
        self.lvert = {g: i for i, g in enumerate(own + ghosts)}  # global vertex -> local
        self.ledge = {g: i for i, g in enumerate(gedges)}         # global edge -> local
        ledges = [(self.lvert[u], self.lvert[v]) for (u, v) in (tn.edges[e] for e in gedges)]
        legs = [[self.ledge[e] for e in tn.legs[v]] for v in own]
        legs += [[self.ledge[e] for e in tn.legs[g] if e in self.ledge] for g in ghosts]
        site = [tn.site_dims[v] for v in own] + [1] * len(ghosts)
        chi = [tn.edge_dims[e] for e in gedges]
        tensors = None
        if tn.tensors is not None:
            tensors = [np.asarray(tn.tensors[v]) for v in own]
            for i, g in enumerate(ghosts):
                shape = (1,) + tuple(chi[le] for le in legs[len(own) + i])
                tensors.append(np.ones(shape, dtype=np.asarray(tn.tensors[g]).dtype))
        self.local = TensorNetwork(len(own) + len(ghosts), ledges, site, chi, tensors=tensors, legs=legs)
        # flat offsets of local directed-edge messages (ABI layout)
        sizes = [chi[de // 2] ** 2 for de in range(2 * len(gedges))]
        self.msg_off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
        self.n_message = int(self.msg_off[-1])
        # directed edges (local ids) leaving own vertices: the convergence sum
        self.owned_des = np.array([de for de in range(2 * len(gedges))
                                   if owner[tn.dsrc(2 * gedges[de // 2] + de % 2)] == rank], dtype=np.int64)
        # per neighbour rank: flat entries to send (own -> q) and to receive (q -> own),
        # both in global directed-edge order, so the two sides agree
        send, recv = {}, {}
        for le, e in enumerate(gedges):
            for o in (0, 1):
                gde = 2 * e + o
                src, dst = tn.dsrc(gde), tn.dsrc(gde ^ 1)
                if owner[src] == rank and owner[dst] != rank:
                    send.setdefault(owner[dst], []).append((gde, 2 * le + o))
                elif owner[src] != rank and owner[dst] == rank:
                    recv.setdefault(owner[src], []).append((gde, 2 * le + o))
        self.send = {q: self._entries(sorted(lst)) for q, lst in send.items()}
        self.recv = {q: self._entries(sorted(lst)) for q, lst in recv.items()}
        self.neighbours = sorted(set(self.send) | set(self.recv))

    def _entries(self, pairs):
        """Flat message entries of the local directed edges in ``pairs``."""
        if not pairs:
            return np.zeros(0, dtype=np.int64)
        return np.concatenate([np.arange(self.msg_off[lde], self.msg_off[lde + 1]) for _, lde in pairs])

    def global_messages(self, flat):
        """{global directed edge: message} for every directed edge leaving an own vertex."""
        tn, out = self.tn, {}
        for lde in self.owned_des:
            e, o = self.gedges[lde // 2], lde % 2
            c = tn.edge_dims[e]
            out[2 * e + o] = np.asarray(flat[self.msg_off[lde]:self.msg_off[lde + 1]]).reshape((c, c), order="F")
        return out


class GpuShard:
    """One rank's block on the GPU: FP64 Jacobi sweeps of the local network
    through the library (its messages stay on the device between sweeps;
    boundary messages cross through host buffers)."""

    def __init__(self, plan: ShardPlan, ctx=None):
        from .cache import BeliefPropagationCache
        self.plan = plan
        self.bpc = BeliefPropagationCache(plan.local, ctx=ctx)

    def init_messages(self, kind="identity"):
        self.bpc.init_messages(kind)

    def sweep(self, want_diff):
        """One Jacobi sweep; the local per-directed-edge diffs (or None)."""
        self.bpc.update(maxiter=1, tol=0.0 if want_diff else None, schedule="parallel", precision="f64")
        return self.bpc.edge_diffs() if want_diff else None

    def get_messages(self):
        return self.bpc.flat_messages()

    def set_messages(self, flat):
        self.bpc.set_messages(np.ascontiguousarray(flat))

    # -- device-resident exchange ------------------------------------------------
    def message_count(self):
        return self.bpc.n_message

    def is_complex(self):
        return self.bpc.complex

    def messages_to(self, buf):
        """Copy the block's flat messages into ``buf``, a contiguous CUDA tensor
        of message_count() elements (device to device, on the context's stream)."""
        self.bpc._c(self.bpc.lib.gbtn_get_messages(self.bpc.handle, C.c_void_p(buf.data_ptr()), _lib.DEVICE))

    def messages_from(self, buf):
        self.bpc._c(self.bpc.lib.gbtn_set_messages(self.bpc.handle, C.c_void_p(buf.data_ptr()), _lib.DEVICE))

    @contextmanager
    def on_stream(self, stream_ptr):
        """Run the library on ``stream_ptr`` (a raw cudaStream_t) inside the block."""
        ctx = self.bpc.ctx
        old = ctx.stream
        ctx.set_stream(stream_ptr)
        try:
            yield
        finally:
            ctx.set_stream(old)

    def close(self):
        self.bpc.close()


class _Exchange:
    """A block's messages as one torch tensor on the exchange device, with the
    flat entry indices of its cut edges there."""

    def __init__(self, shard, device):
        import torch
        self.torch = torch
        self.shard = shard
        self.device = device
        plan = shard.plan
        self.on_gpu = device.type == "cuda"
        if self.on_gpu:
            dt = torch.complex128 if shard.is_complex() else torch.float64
            self.buf = torch.empty(max(shard.message_count(), 1), dtype=dt, device=device)
        else:
            self.buf = None
        self.send = {q: torch.as_tensor(np.asarray(i, dtype=np.int64), device=device) for q, i in plan.send.items()}
        self.recv = {q: torch.as_tensor(np.asarray(i, dtype=np.int64), device=device) for q, i in plan.recv.items()}

    def pull(self):
        """The block's current messages into the exchange tensor."""
        if self.on_gpu:
            self.shard.messages_to(self.buf)
        else:
            self.buf = self.torch.from_numpy(np.array(self.shard.get_messages()))
        return self.buf

    def push(self):
        if self.on_gpu:
            self.shard.messages_from(self.buf)
        else:
            self.shard.set_messages(self.buf.numpy())

    def outgoing(self, q):
        return self.buf.index_select(0, self.send[q])

    def incoming(self, q, values):
        self.buf.index_copy_(0, self.recv[q], values)


def _finish_sweep(shard, diffs):
    """(sum, count) of this block's own directed-edge diffs."""
    if diffs is None:
        return 0.0, 0
    d = np.asarray(diffs)[shard.plan.owned_des]
    return float(d.sum()), int(d.size)


def _exchange_device(device):
    import torch
    return torch.device(device) if device is not None else torch.device("cpu")


@contextmanager
def _library_on_torch_stream(shards, device):
    """GPU blocks run on torch's current stream while the exchange uses it."""
    if device.type != "cuda":
        yield
        return
    import torch
    stream = torch.cuda.current_stream(device).cuda_stream
    with _nested([s.on_stream(stream) for s in shards if hasattr(s, "on_stream")]):
        yield


@contextmanager
def _nested(cms):
    if not cms:
        yield
        return
    with cms[0]:
        with _nested(cms[1:]):
            yield


def run_local(shards, maxiter, tol=None, init="identity", device=None):
    """Jacobi sweeps of every block in this process, boundary messages copied
    between the blocks after each sweep (on ``device``: "cpu" by default,
    "cuda" for GPU blocks exchanged on the device).  Returns (sweeps run, last
    mean diff)."""
    if maxiter is None or maxiter < 1:
        raise ValueError("You need to specify a number of iterations for BP!")
    dev = _exchange_device(device)
    ex = {s.plan.rank: _Exchange(s, dev) for s in shards}
    mean = float("nan")
    it = 0
    with _library_on_torch_stream(shards, dev):
        for s in shards:
            s.init_messages(init)
        for it in range(1, maxiter + 1):
            tot, cnt = 0.0, 0
            for s in shards:
                d = s.sweep(tol is not None)
                a, b = _finish_sweep(s, d)
                tot, cnt = tot + a, cnt + b
            for r in ex:  # every block's new messages before any is overwritten (Jacobi)
                ex[r].pull()
            if len(ex) > 1:
                vals = {(r, q): ex[q].outgoing(r) for r in ex for q in ex[r].recv}
                for (r, q), v in vals.items():
                    ex[r].incoming(q, v)
            for r in ex:
                ex[r].push()
            if tol is not None:
                mean = tot / max(cnt, 1)
                if mean <= tol:
                    break
    return it, mean


def run_distributed(shard, maxiter, tol=None, init="identity", group=None, device=None):
    """This process's block, exchanging boundary messages with the blocks of
    the other ranks of ``group`` (torch.distributed point-to-point sends, one
    all-reduce per sweep when ``tol`` is given).  The exchange tensors live on
    ``device``: by default the GPU with NCCL and the host with other backends.
    Returns (sweeps run, last mean diff), identical on every rank."""
    import torch
    import torch.distributed as dist

    if maxiter is None or maxiter < 1:
        raise ValueError("You need to specify a number of iterations for BP!")
    if device is None:
        device = f"cuda:{shard.bpc.ctx.device}" if str(dist.get_backend(group)) == "nccl" else "cpu"
    dev = _exchange_device(device)
    plan = shard.plan
    ex = _Exchange(shard, dev)
    cplx = ex.on_gpu and shard.is_complex()

    def wire(t):  # complex entries travel as (re, im) pairs of doubles
        return torch.view_as_real(t) if cplx else t

    mean = float("nan")
    it = 0
    with _library_on_torch_stream([shard], dev):
        shard.init_messages(init)
        for it in range(1, maxiter + 1):
            d = shard.sweep(tol is not None)
            ex.pull()
            ops, inbox, keep = [], {}, []
            for q in plan.neighbours:
                if q in ex.send:
                    out = ex.outgoing(q)
                    keep.append(out)
                    ops.append(dist.P2POp(dist.isend, wire(out), q, group))
                if q in ex.recv:
                    inbox[q] = torch.empty(len(plan.recv[q]), dtype=ex.buf.dtype, device=dev)
                    ops.append(dist.P2POp(dist.irecv, wire(inbox[q]), q, group))
            if ops:
                for r in dist.batch_isend_irecv(ops):
                    r.wait()
            for q, buf in inbox.items():
                ex.incoming(q, buf)
            ex.push()
            if tol is not None:
                a, b = _finish_sweep(shard, d)
                t = torch.tensor([a, float(b)], dtype=torch.float64, device=dev)
                dist.all_reduce(t, group=group)
                tot, cnt = t.tolist()
                mean = tot / max(cnt, 1.0)
                if mean <= tol:
                    break
    return it, mean


def block_owner(L, blocks_x, blocks_y):
    """Owner map of an L x L square lattice (vertex i + L j) cut into
    blocks_x x blocks_y rectangular blocks, rank = bx + blocks_x * by."""
    own = []
    for j in range(L):
        for i in range(L):
            bx = min(i * blocks_x // L, blocks_x - 1)
            by = min(j * blocks_y // L, blocks_y - 1)
            own.append(bx + blocks_x * by)
    return own
