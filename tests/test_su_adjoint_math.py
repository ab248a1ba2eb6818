"""The simple update's adjoint, restated in NumPy (CPU), against central
differences of the oracle's simple_update_bp (src/apply.jl:33-95).

The restatement follows the algorithm of the library's adjoint kernels:
- with W_x = Q_x R_x the matricised sites and P_x = Q_x (x) 1_site, the outputs
  are the halves L = P_u U_k sqrt(s_k), R = P_v V_k sqrt(s_k) of the truncated
  SVD of Theta = P_u theta P_v^T, so no QR derivative is needed;
- the cotangents of L and R split into their parts in range(P_x) and
  orthogonal to it;
- the truncated-SVD adjoint (Townsend 2016) runs in range with theta's full
  spectrum: the discarded singular values enter F_ij = 1/(s_j^2 - s_i^2), and
  the discarded vectors carry zero cotangent;
- the orthogonal parts contract with the other site's R only;
- the gate is transposed and the bond contraction goes back to Rbar.
It checks the mathematics the kernels implement, independently of them, on
shapes where the full state stays small (no environments: those add linear
maps the GPU tests cover)."""
import numpy as np
import pytest

import bp_oracle as O


def matricise(T, ax):
    """(other legs) x (site, bond) with the other legs in order, column-major."""
    others = [i for i in range(1, T.ndim) if i != ax]
    Tp = np.transpose(T, others + [0, ax])
    m = int(np.prod([T.shape[i] for i in others])) if others else 1
    return Tp.reshape(m, T.shape[0] * T.shape[ax], order="F"), others


def unmatricise(Wm, shape, others, ax):
    T = Wm.reshape([shape[i] for i in others] + [shape[0], shape[ax]], order="F")
    names = others + [0, ax]
    return np.transpose(T, [names.index(i) for i in range(len(shape))])


def su_forward(gate, Au, Av, pu, pv, maxdim):
    """The oracle's simple update without environments, unnormalised."""
    Bu, Bv, S, _ = O.simple_update(gate, Au, Av, pu, pv, {}, {}, maxdim=maxdim)
    return Bu, Bv


def su_vjp(gate, Au, Av, pu, pv, maxdim, Bu_bar, Bv_bar):
    """dL/dAu, dL/dAv, dL/dgate from dL/d(outputs), as the kernels compute them."""
    du, dv = Au.shape[0], Av.shape[0]
    au, av = pu + 1, pv + 1
    ce = Au.shape[au]
    Wu, ou = matricise(Au, au)
    Wv, ov = matricise(Av, av)
    Qu, Ru = np.linalg.qr(Wu)
    Qv, Rv = np.linalg.qr(Wv)
    ru, rv = Ru.shape[0], Rv.shape[0]
    # theta[(iu, su'), (sv', iv)]: rows iu + ru su', columns sv' + dv iv
    Ru3 = Ru.reshape(ru, du, ce, order="F")
    Rv3 = Rv.reshape(rv, dv, ce, order="F")
    psi = np.einsum("isl,jtl->istj", Ru3, Rv3)                 # [iu, su, sv, iv]
    G4 = gate.reshape(du, dv, du, dv, order="F")               # [su', sv', su, sv]
    th = np.einsum("abst,istj->iabj", G4, psi)                 # [iu, su', sv', iv]
    mt, nt = ru * du, dv * rv
    theta = th.reshape(mt, nt, order="F")
    U, s, Vh = np.linalg.svd(theta, full_matrices=False)
    V = Vh.T
    n = len(s)
    k = O.truncate_spectrum(s ** 2, maxdim=maxdim)[0]
    sq = np.sqrt(s[:k])
    # output cotangents as big-space factors: Lbar[(row, s), b], Rbar[(row, s), b]
    Lb = np.moveaxis(Bu_bar, [*ou, 0, au], range(Bu_bar.ndim)).reshape(-1, du, k, order="F")
    Rb = np.moveaxis(Bv_bar, [*ov, 0, av], range(Bv_bar.ndim)).reshape(-1, dv, k, order="F")
    # range split: Z = Q^T Ybar, perp = Ybar - Q Z
    Zu = np.einsum("rt,rsb->tsb", Qu, Lb)
    Zv = np.einsum("rt,rsb->tsb", Qv, Rb)
    Lperp = Lb - np.einsum("rt,tsb->rsb", Qu, Zu)
    Rperp = Rb - np.einsum("rt,tsb->rsb", Qv, Zv)
    Ub = (Zu * sq).reshape(mt, k, order="F")                   # rows iu + ru su
    Vb = np.transpose(Zv * sq, (1, 0, 2)).reshape(nt, k, order="F")  # rows sv + dv iv
    sbar = (np.sum(U[:, :k] * (Ub / sq), axis=0) + np.sum(V[:, :k] * (Vb / sq), axis=0)) / (2 * sq)
    UtUb = np.zeros((n, n))
    VtVb = np.zeros((n, n))
    UtUb[:, :k] = U.T @ Ub
    VtVb[:, :k] = V.T @ Vb
    J = np.zeros((n, n))
    for p in range(n):
        for q in range(n):
            if p == q:
                J[p, q] = sbar[p] if p < k else 0.0
            elif p < k or q < k:
                F = 1.0 / (s[q] ** 2 - s[p] ** 2)
                J[p, q] = F * ((UtUb[p, q] - UtUb[q, p]) * s[q] + s[p] * (VtVb[p, q] - VtVb[q, p]))
    P1 = (Ub - U @ UtUb[:, :k]) / s[:k]
    P2 = (Vb - V @ VtVb[:, :k]) / s[:k]
    thbar = U @ J @ V.T + P1 @ V[:, :k].T + U[:, :k] @ P2.T
    thb4 = thbar.reshape(ru, du, dv, rv, order="F")            # [iu, su', sv', iv]
    phi = np.einsum("abst,iabj->istj", G4, thb4)               # gate transposed: [iu, su, sv, iv]
    gbar = np.einsum("iabj,istj->abst", thb4, psi).reshape(du * dv, du * dv, order="F")
    Rub = np.einsum("istj,jtl->isl", phi, Rv3).reshape(ru, du * ce, order="F")
    Rvb = np.einsum("istj,isl->jtl", phi, Ru3).reshape(rv, dv * ce, order="F")
    # orthogonal parts: contractions with the other site's R only
    M2 = np.einsum("bjc,jtl->cbtl", V[:, :k].reshape(dv, rv, k, order="F"), Rv3)  # [c, sv', sv, l]
    H2 = np.einsum("abst,cbtl->acsl", G4, M2) / sq[None, :, None, None]   # [su', c, su, l]
    Wub = Qu @ Rub + np.einsum("rac,acsl->rsl", Lperp, H2).reshape(-1, du * ce, order="F")
    M3 = np.einsum("iac,isl->casl", U[:, :k].reshape(ru, du, k, order="F"), Ru3)
    H3 = np.einsum("abst,casl->bctl", G4, M3) / sq[None, :, None, None]   # [sv', c, sv, l]
    Wvb = Qv @ Rvb + np.einsum("rbc,bctl->rtl", Rperp, H3).reshape(-1, dv * ce, order="F")
    return unmatricise(Wub, Au.shape, ou, au), unmatricise(Wvb, Av.shape, ov, av), gbar


@pytest.mark.parametrize("maxdim", [2, 3, 8])
def test_su_adjoint_restatement_matches_finite_differences(maxdim):
    """A gate on the centre bond of a 3x3 lattice (site tensors of degree 3 and
    4): L = <W, Au' ._bond Av'> (gauge invariant), truncated to maxdim of up to
    8 singular values (8 keeps them all: no discarded spectrum)."""
    g = O.square_lattice(3, 3, chi=2)
    A = O.random_network(g, 5)
    e = 5  # (3, 4)
    u, v = g.edges[e]
    pu, pv = g.legs[u].index(e), g.legs[v].index(e)
    rng = np.random.default_rng(maxdim)
    H = rng.standard_normal((4, 4))
    gate = np.eye(4) + 0.3 * (H + H.T)
    Bu, Bv = su_forward(gate, A[u], A[v], pu, pv, maxdim)
    two = lambda X, Y: np.tensordot(X, Y, axes=([pu + 1], [pv + 1]))
    W = rng.standard_normal(two(Bu, Bv).shape)
    loss = lambda Au, Av, gt=gate: float(np.sum(W * two(*su_forward(gt, Au, Av, pu, pv, maxdim))))
    # dL/d(outputs): W contracted with the other output
    nu = Bu.ndim - 1
    Bu_bar = np.tensordot(W, Bv, axes=(list(range(nu, W.ndim)), [i for i in range(Bv.ndim) if i != pv + 1]))
    Bu_bar = np.moveaxis(Bu_bar, -1, pu + 1)
    Bv_bar = np.tensordot(Bu, W, axes=([i for i in range(Bu.ndim) if i != pu + 1], list(range(nu))))
    Bv_bar = np.moveaxis(Bv_bar, 0, pv + 1)
    gu, gv, gg = su_vjp(gate, A[u], A[v], pu, pv, maxdim, Bu_bar, Bv_bar)
    h = 1e-6
    Du, Dv = rng.standard_normal(A[u].shape), rng.standard_normal(A[v].shape)
    fd = (loss(A[u] + h * Du, A[v] + h * Dv) - loss(A[u] - h * Du, A[v] - h * Dv)) / (2 * h)
    assert float(np.sum(gu * Du) + np.sum(gv * Dv)) == pytest.approx(fd, rel=1e-6)
    Dg = rng.standard_normal(gate.shape)
    fdg = (loss(A[u], A[v], gate + h * Dg) - loss(A[u], A[v], gate - h * Dg)) / (2 * h)
    assert float(np.sum(gg * Dg)) == pytest.approx(fdg, rel=1e-6)
