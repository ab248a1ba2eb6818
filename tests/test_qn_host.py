"""Host bookkeeping of U(1)-graded networks (CPU): the nonzero-block masks
balance every vertex's flux, and dense BP of such a network keeps its
messages block-diagonal in the link sectors -- the property the library's
block-sparse storage of messages rests on."""
import numpy as np

import bp_oracle as O
import gbtn


def test_masks_balance_the_flux():
    tn = gbtn.square_lattice(3, 2, chi=3)
    links = [[(-1, 1), (1, 2)]] * tn.ne
    sites = [[(1, 1), (-1, 1)]] * tn.nv
    flux = [1, -1, 1, -1, 1, -1]
    q = gbtn.QNNetwork(tn, links, sites, flux)
    for v in range(tn.nv):
        m = q.mask(v)
        ranges = [gbtn.QNNetwork._ranges(sites[v])] + [gbtn.QNNetwork._ranges(links[e]) for e in tn.legs[v]]
        for idx in np.ndindex(m.shape):
            charge = 0
            for a, i in enumerate(idx):
                c = next(ch for ch, lo, hi in ranges[a] if lo <= i < hi)
                if a == 0:
                    charge += c
                else:
                    e = tn.legs[v][a - 1]
                    charge += -c if tn.edges[e][0] == v else c
            assert m[idx] == (charge == flux[v])


def test_dense_bp_keeps_messages_block_diagonal():
    tn = gbtn.square_lattice(3, 3, chi=4)
    links = [[(-1, 1), (0, 2), (1, 1)]] * tn.ne
    q = gbtn.random_qn_network(tn, links, [[(1, 1), (-1, 1)]] * tn.nv, [1, -1, 1, -1, 1, -1, 1, -1, 1], 2)
    g = O.Graph(tn.nv, tn.edges, tn.site_dims, tn.edge_dims, tn.legs)
    m, _, _ = O.bp_update(g, q.tn.tensors, O.identity_messages(g), maxiter=10, schedule="parallel")
    off = 0.0
    for de in range(2 * g.ne):
        r = gbtn.QNNetwork._ranges(links[de // 2])
        for c1, a1, b1 in r:
            for c2, a2, b2 in r:
                if c1 != c2:
                    off = max(off, float(np.max(np.abs(m[de][a1:b1, a2:b2]))))
    assert off < 1e-14
