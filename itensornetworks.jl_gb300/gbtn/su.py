"""Simple update on the GPU: ``apply`` and ``tebd`` (src/apply.jl, src/tebd.jl).

``SimpleUpdateState`` holds a tensor network whose bond dimensions grow up to
``chi_max`` as two-site gates are applied.  Gates are (du*dv) x (du*dv)
matrices acting on an edge (u, v) = network.edges[e], row s'_u + du*s'_v,
column s_u + du*s_v.  Every numerical step (sqrt environments, QR, gate, SVD,
truncation, reassembly) runs in libgbtn in FP64; complex networks (complex
tensors, gates or environments, e.g. random unitaries) run complex FP64."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import check, dptr, iptr
from .network import TensorNetwork


class SimpleUpdateState:
    def __init__(self, tn: TensorNetwork, chi_max: int, ctx=None, complex_values=None):
        if tn.tensors is None:
            raise ValueError("the network has no tensors")
        self.ctx = ctx or _lib.default_context()
        self.lib = self.ctx.lib
        self.tn = tn.copy()
        self.complex = tn.is_complex if complex_values is None else bool(complex_values)
        self.dtype = np.complex128 if self.complex else np.float64
        self.tn.tensors = [np.asarray(t, dtype=self.dtype) for t in self.tn.tensors]
        self.chi_max = int(chi_max)
        desc, keep = self.tn.graph_desc()
        h = C.c_void_p()
        check(self.ctx.handle, self.lib.gbtn_su_create(self.ctx.handle, C.byref(desc), self.chi_max, C.byref(h)))
        self.handle = h
        flat = self.tn.flat()
        check(self.ctx.handle, self.lib.gbtn_su_set_factors(self.handle, dptr(flat.view(np.float64))))

    def edge_dims(self):
        out = np.zeros(max(self.tn.ne, 1), dtype=np.int32)
        check(self.ctx.handle, self.lib.gbtn_su_edge_dims(self.handle, iptr(out)))
        return [int(x) for x in out[:self.tn.ne]]

    def network(self):
        """The current state as a TensorNetwork (current bond dimensions)."""
        dims = self.edge_dims()
        net = TensorNetwork(self.tn.nv, self.tn.edges, self.tn.site_dims, dims, None, self.tn.legs,
                            self.tn.vertex_network, self.tn.n_networks)
        n = sum(net.size(v) for v in range(net.nv))
        out = np.empty(max(n, 1), dtype=self.dtype)
        buf = out.view(np.float64)
        check(self.ctx.handle, self.lib.gbtn_su_get_factors(self.handle, dptr(buf), buf.size))
        net.tensors = net.unflat(out[:n])
        return net

    def _pack(self, gates, envs):
        shared = not isinstance(gates, (list, tuple))
        glist = [gates] if shared else list(gates)
        if not self.complex and (any(np.iscomplexobj(x) for x in glist)
                                 or (envs is not None and any(np.iscomplexobj(m) for m in envs))):
            raise ValueError("complex gates or environments need a complex state (complex_values=True)")
        dt = self.dtype
        g = np.ascontiguousarray(np.concatenate([np.asarray(x, dt).reshape(-1, order="F") for x in glist]))
        env_arr = None
        if envs is not None:
            cm = self.chi_max
            env_arr = np.zeros(2 * self.tn.ne * cm * cm, dtype=dt)
            for de, m in enumerate(envs):
                c = m.shape[0]
                env_arr[de * cm * cm:de * cm * cm + c * c] = np.asarray(m, dt).reshape(-1, order="F")
        return shared, g, env_arr

    def apply(self, gates, edges, envs=None, maxdim=None, cutoff=None, normalize=False):
        """Apply gates[j] on edges[j] in order.  ``gates`` is one matrix (shared)
        or a list.  ``envs``: None or a list of 2*ne message matrices (the BP
        environment).  Returns (truncation errors, kept singular values)."""
        edges = np.ascontiguousarray(edges, dtype=np.int32)
        n = len(edges)
        shared, g, env_arr = self._pack(gates, envs)
        md = int(maxdim) if maxdim else self.chi_max
        te = np.zeros(max(n, 1))
        sv = np.zeros(max(n * md, 1))
        check(self.ctx.handle, self.lib.gbtn_su_apply(
            self.handle, n, iptr(edges), dptr(g.view(np.float64)), 0 if shared else 1,
            None if env_arr is None else dptr(env_arr.view(np.float64)), md,
            -1.0 if cutoff is None else float(cutoff),
            1 if normalize else 0, dptr(te), dptr(sv)))
        return te[:n], sv[:n * md].reshape(n, md)

    def set_state(self, net: TensorNetwork):
        """Replace the bond dimensions and tensors by those of ``net`` (same graph)."""
        dims = np.ascontiguousarray(net.edge_dims, dtype=np.int32)
        if len(dims):
            check(self.ctx.handle, self.lib.gbtn_su_set_edge_dims(self.handle, iptr(dims)))
        flat = np.ascontiguousarray(np.concatenate([np.asarray(t, self.dtype).reshape(-1, order="F")
                                                    for t in net.tensors]))
        check(self.ctx.handle, self.lib.gbtn_su_set_factors(self.handle, dptr(flat.view(np.float64))))

    def apply_vjp(self, gates, edges, post_dims, cot, envs=None, maxdim=None, cutoff=None, normalize=False):
        """Adjoint of ``apply`` for gates on disjoint vertices, at the current
        tensors (the gates' inputs).  ``cot``: per vertex dL/d(tensor after the
        gates) with bond dimensions ``post_dims``.  Returns (dL/d(current
        tensors) per vertex, dL/dG per gate as an (n, D, D) array, dL/d(envs)
        as a list of 2*ne matrices, or None without envs)."""
        if self.complex:
            raise _lib.Unsupported(2, "simple update adjoint: real tensors only")
        edges = np.ascontiguousarray(edges, dtype=np.int32)
        n = len(edges)
        shared, g, env_arr = self._pack(gates, envs)
        post = np.ascontiguousarray(post_dims, dtype=np.int32)
        flat = np.ascontiguousarray(np.concatenate([np.asarray(t, float).reshape(-1, order="F") for t in cot]))
        pre_dims = self.edge_dims()
        pre = TensorNetwork(self.tn.nv, self.tn.edges, self.tn.site_dims, pre_dims, None, self.tn.legs,
                            self.tn.vertex_network, self.tn.n_networks)
        out = np.zeros(max(sum(pre.size(v) for v in range(pre.nv)), 1))
        D = self.tn.site_dims[self.tn.edges[int(edges[0])][0]] * self.tn.site_dims[self.tn.edges[int(edges[0])][1]] \
            if n else 1
        gc = np.zeros(max(n * D * D, 1))
        ec = None if env_arr is None else np.zeros_like(env_arr)
        md = int(maxdim) if maxdim else self.chi_max
        check(self.ctx.handle, self.lib.gbtn_su_apply_vjp(
            self.handle, n, iptr(edges), dptr(g), 0 if shared else 1,
            None if env_arr is None else dptr(env_arr), md, -1.0 if cutoff is None else float(cutoff),
            1 if normalize else 0, iptr(post), dptr(flat), dptr(out), dptr(gc), None if ec is None else dptr(ec)))
        n_el = sum(pre.size(v) for v in range(pre.nv))
        return (pre.unflat(out[:n_el]), gc[:n * D * D].reshape(n, D, D).transpose(0, 2, 1),
                None if ec is None else self._unpack_envs(ec, envs))

    def _unpack_envs(self, arr, envs):
        """The 2*ne environment matrices (their shapes) out of the chi_max^2 slots."""
        cm = self.chi_max
        out = []
        for de, m in enumerate(envs):
            c = np.asarray(m).shape[0]
            out.append(arr[de * cm * cm:de * cm * cm + c * c].reshape(c, c, order="F").copy())
        return out

    def apply_with_pullback(self, gates, edges, envs=None, maxdim=None, cutoff=None, normalize=False):
        """``apply`` that also returns its pullback: (truncation errors, kept
        singular values, pullback), pullback(cot) -> (dL/d(tensors before the
        gates) per vertex, dL/dG per gate (n, D, D), dL/d(envs) as 2*ne
        matrices or None without envs).  The library keeps a tape
        of the state before every batch of consecutive vertex-disjoint gates
        in device memory (gbtn_su_apply_taped); the pullback runs the batches'
        adjoints backwards on the device and leaves the state where ``apply``
        left it.  Real tensors."""
        if self.complex:
            raise _lib.Unsupported(2, "simple update adjoint: real tensors only")
        edges = np.ascontiguousarray(edges, dtype=np.int32)
        n = len(edges)
        shared, g, env_arr = self._pack(gates, envs)
        md = int(maxdim) if maxdim else self.chi_max
        te = np.zeros(max(n, 1))
        sv = np.zeros(max(n * md, 1))
        before = self.network()
        tape = _Tape(self)
        check(self.ctx.handle, self.lib.gbtn_su_apply_taped(
            self.handle, n, iptr(edges), dptr(g), 0 if shared else 1,
            None if env_arr is None else dptr(env_arr), md, -1.0 if cutoff is None else float(cutoff),
            1 if normalize else 0, dptr(te), dptr(sv), C.byref(tape.handle)))
        after_dims = self.edge_dims()
        du = [self.tn.site_dims[self.tn.edges[int(e)][0]] * self.tn.site_dims[self.tn.edges[int(e)][1]] for e in edges]
        D = du[0] if n else 1

        def pullback(cot):
            flat = np.ascontiguousarray(np.concatenate([np.asarray(c, float).reshape(-1, order="F") for c in cot]))
            n_after = sum(int(np.prod(np.asarray(c).shape)) for c in cot)
            want = sum(self.tn.site_dims[v] * int(np.prod([after_dims[e] for e in self.tn.legs[v]]))
                       for v in range(self.tn.nv))
            if n_after != want:
                raise _lib.InvalidArgument(1, "cotangents do not have the shapes the gates left")
            out = np.zeros(max(sum(before.size(v) for v in range(before.nv)), 1))
            gc = np.zeros(max(n * D * D, 1))
            ec = None if env_arr is None else np.zeros_like(env_arr)
            check(self.ctx.handle, self.lib.gbtn_su_tape_vjp(self.handle, tape.handle, dptr(flat), dptr(out), dptr(gc),
                                                             None if ec is None else dptr(ec)))
            n_el = sum(before.size(v) for v in range(before.nv))
            return (before.unflat(out[:n_el]), gc[:n * D * D].reshape(n, D, D).transpose(0, 2, 1),
                    None if ec is None else self._unpack_envs(ec, envs))

        pullback.tape = tape  # freed with the pullback
        return te[:n], sv[:n * md].reshape(n, md), pullback

    def close(self):
        if getattr(self, "handle", None):
            self.lib.gbtn_su_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _Tape:
    """Owner of a gbtn_su_tape."""

    def __init__(self, st):
        self.st = st
        self.handle = C.c_void_p()

    def __del__(self):
        try:
            if self.handle:
                self.st.lib.gbtn_su_tape_destroy(self.handle)
            self.handle = C.c_void_p()
        except Exception:
            pass


def apply(gate, psi: TensorNetwork, edge, envs=None, maxdim=None, cutoff=None, normalize=False, callback=None,
          chi_max=None):
    """apply(o, psi; envs, maxdim, cutoff, normalize, callback) for one two-site
    gate (apply.jl:97-146).  Returns the updated network; ``callback`` receives
    singular_values= and truncation_error= like the reference's callback."""
    cm = chi_max or max([maxdim or 0] + list(psi.edge_dims) + [psi.site_dims[0] * max(psi.edge_dims or [1])])
    cm = min(cm, 8)
    cplx = psi.is_complex or np.iscomplexobj(gate) or (envs is not None and any(np.iscomplexobj(m) for m in envs))
    st = SimpleUpdateState(psi, cm, complex_values=cplx)
    te, sv = st.apply(gate, [edge], envs=envs, maxdim=maxdim or cm, cutoff=cutoff, normalize=normalize)
    if callback is not None:
        k = int(np.count_nonzero(sv[0]))
        callback(singular_values=sv[0][:k], truncation_error=float(te[0]))
    out = st.network()
    st.close()
    return out


# -----------------------------------------------------------------------------
# Transverse-field Ising TEBD (the two-site gates of a first-order, or
# symmetric second-order, checkerboard Trotter step)
# -----------------------------------------------------------------------------

PX = np.array([[0.0, 1.0], [1.0, 0.0]])
PZ = np.array([[1.0, 0.0], [0.0, -1.0]])


def _expm_sym(h, t):
    w, U = np.linalg.eigh(h)
    return (U * np.exp(t * w)) @ U.T


def tfim_bond_hamiltonian(g, z_u, z_v):
    """h_e = -Z(x)Z - g (X(x)I / z_u + I(x)X / z_v): the field of every site is
    split evenly over its z incident edges (row s'_u + 2 s'_v)."""
    I2 = np.eye(2)
    return -np.kron(PZ, PZ) - g * (np.kron(I2, PX) / z_u + np.kron(PX, I2) / z_v)


def tfim_gate(dt, g, z_u, z_v):
    """exp(-dt h_e)."""
    return _expm_sym(tfim_bond_hamiltonian(g, z_u, z_v), -dt)


def checkerboard_edges(Lx, Ly):
    """Edges of square_lattice(Lx, Ly) in four vertex-disjoint colour classes:
    horizontal bonds with even / odd first coordinate, then vertical bonds with
    even / odd second coordinate."""
    from .network import square_lattice
    tn = square_lattice(Lx, Ly)
    classes = [[], [], [], []]
    for e, (u, v) in enumerate(tn.edges):
        i, j = u % Lx, u // Lx
        if v == u + 1:
            classes[i % 2].append(e)
        else:
            classes[2 + j % 2].append(e)
    return classes


def tebd(*args, **kwargs):
    """Two forms.  ``tebd(H, psi, beta=, dbeta=, maxdim=, cutoff=,
    print_frequency=10, ortho=False)`` with an OpSum H is the reference's
    signature (src/tebd.jl:2-31; see gbtn.opsum) and returns the evolved network.
    ``tebd(psi, gate_of_edge, edge_classes, nsteps, maxdim, cutoff, ...)`` runs
    precomputed two-site gates class by class (tebd_gates)."""
    from .opsum import OpSum, tebd_opsum
    if args and isinstance(args[0], OpSum):
        return tebd_opsum(*args, **kwargs)
    return tebd_gates(*args, **kwargs)


def tebd_gates(psi: TensorNetwork, gate_of_edge, edge_classes, nsteps, maxdim, cutoff, normalize=True, chi_max=None,
               state=None, bp_envs=False, bp_maxiter=30, bp_tol=1e-12, bp_precision="f64"):
    """nsteps Trotter steps: every class of vertex-disjoint edges in order
    (tebd.jl:2-31 with a checkerboard gate order).  Returns the final state and
    the truncation errors of the last step.

    bp_envs=True is the BP-gauged variant (apply with envs, test/test_apply.jl:30-35,
    with the cache refreshed inside the loop): before each class the
    current state's BP messages are computed on the GPU (parallel schedule,
    at most bp_maxiter sweeps, tol bp_tol) and its gates use them as
    environments.  Gates of one class touch disjoint vertices, so none of them
    changes a message another one reads; the refresh between classes picks up
    the bond dimensions the previous class changed."""
    st = state or SimpleUpdateState(psi, chi_max or maxdim)
    gates = {e: gate_of_edge(e) for cls in edge_classes for e in cls}
    order = [e for cls in edge_classes for e in cls]
    te = None
    for _ in range(nsteps):
        if not bp_envs:
            te, _ = st.apply([gates[e] for e in order], order, maxdim=maxdim, cutoff=cutoff, normalize=normalize)
            continue
        tes = []
        for cls in edge_classes:
            envs = bp_environments(st, maxiter=bp_maxiter, tol=bp_tol, precision=bp_precision)
            t, _ = st.apply([gates[e] for e in cls], list(cls), envs=envs, maxdim=maxdim, cutoff=cutoff,
                            normalize=normalize)
            tes.append(t)
        te = np.concatenate(tes)
    return st, te


def bp_environments(st: SimpleUpdateState, maxiter=30, tol=1e-12, precision="f64"):
    """Converged BP messages of the state held by ``st`` (one chi x chi matrix
    per directed edge, current bond dimensions), computed on the GPU."""
    from .cache import BeliefPropagationCache
    bpc = BeliefPropagationCache(st.network(), ctx=st.ctx)
    bpc.update(maxiter=maxiter, tol=tol, schedule="parallel", precision=precision)
    msgs = bpc.messages()
    bpc.close()
    return msgs


def tebd_with_pullback(psi: TensorNetwork, gate_of_edge, edge_classes, nsteps, maxdim, cutoff, normalize=True,
                       chi_max=None, bp_envs=False, bp_maxiter=300, bp_tol=1e-13):
    """``tebd_gates`` (real tensors) that also returns its pullback:
    (state, pullback), pullback(cot) -> (dL/d(psi's tensors), {edge: dL/dG}),
    cot = dL/d(the final tensors).  Without bp_envs the whole gate sequence is
    one taped apply.  With bp_envs the environments of every colour class are
    the converged BP messages of the state before it, and the pullback adds
    their path: each class's environment cotangent goes through that state's
    BP fixed point (implicit adjoint, gbtn_bp_vjp) to its tensors.  Memory: one
    device copy of the state per batch of vertex-disjoint gates, and with
    bp_envs one BP plan per class, kept until the pullback is dropped."""
    from .cache import BeliefPropagationCache
    st = SimpleUpdateState(psi, chi_max or maxdim)
    gates = {e: np.asarray(gate_of_edge(e), dtype=float) for cls in edge_classes for e in cls}
    if not bp_envs:
        order = [e for _ in range(nsteps) for cls in edge_classes for e in cls]
        _, _, pull = st.apply_with_pullback([gates[e] for e in order], order, maxdim=maxdim, cutoff=cutoff,
                                            normalize=normalize)

        def pullback(cot):
            g0, gc, _ = pull(cot)
            dg = {e: np.zeros_like(gates[e]) for e in gates}
            for e, m in zip(order, gc):
                dg[e] += m
            return g0, dg
        return st, pullback
    records = []
    for _ in range(nsteps):
        for cls in edge_classes:
            bpc = BeliefPropagationCache(st.network(), ctx=st.ctx)
            bpc.update(maxiter=bp_maxiter, tol=bp_tol, schedule="parallel", precision="f64")
            envs = bpc.messages()
            _, _, pull = st.apply_with_pullback([gates[e] for e in cls], list(cls), envs=envs, maxdim=maxdim,
                                                cutoff=cutoff, normalize=normalize)
            records.append((list(cls), bpc, pull))
    final = st.network()

    def pullback(cot):
        dg = {e: np.zeros_like(gates[e]) for e in gates}
        for cls, bpc, pull in reversed(records):
            cot, gc, denv = pull(cot)
            cot = [a + b for a, b in zip(cot, bpc.vjp(denv, tol=1e-14))]
            for e, m in zip(cls, gc):
                dg[e] += m
        st.set_state(final)
        return cot, dg
    return st, pullback
