"""OpSum host logic (no GPU): term parsing, the reference's group_terms order
(test/utils.jl:239-246) and the second-order Trotter gate list of tebd
(src/tebd.jl:2-31) against the oracle's restatement."""
import numpy as np
import pytest

import bp_oracle as O
import gbtn


def ising(tn, h):
    H = gbtn.OpSum()
    for (u, v) in tn.edges:
        H += (-1.0, "Sz", u, "Sz", v)
    for v in range(tn.nv):
        H += (h, "Sx", v)
    return H


@pytest.mark.parametrize("Lx,Ly", [(2, 3), (3, 3), (4, 2)])
def test_grouping_and_trotter_gates_match_the_oracle(Lx, Ly):
    tn = gbtn.square_lattice(Lx, Ly, chi=1)
    g = O.square_lattice(Lx, Ly, chi=1)
    Hg = gbtn.group_terms(ising(tn, 0.3), tn)
    og = O.group_terms(O.ising_terms(g, h=0.3), g)
    assert [e for e, _ in Hg.groups] == [e for e, _ in og]
    assert [len(t) for _, t in Hg.groups] == [len(t) for _, t in og]
    a, b = gbtn.trotter2_gates(Hg, tn, 0.2), O.trotter2_gates(g, og, 0.2)
    assert [e for e, _ in a] == [e for e, _ in b]
    for (_, x), (_, y) in zip(a, b):
        np.testing.assert_allclose(x, y, rtol=0, atol=1e-14)
    # a palindrome of half steps: the list composes to exp(-dbeta H_edge) per edge when terms commute
    assert len(a) == 2 * len(Hg.groups)


def test_terms_parse_like_opsum_tuples():
    H = gbtn.OpSum()
    H += ("Sz", 0, "Sz", 1)
    H += (0.5j, "S+", 2, "S-", 3)
    assert H.terms[0] == (1.0, (("Sz", 0), ("Sz", 1)))
    assert H.terms[1][0] == 0.5j
    with pytest.raises(ValueError):
        H += (1.0, "Sq", 0)
    with pytest.raises(ValueError):
        H += (1.0, "Sz")
    tn = gbtn.square_lattice(2, 2, chi=1)
    far = gbtn.OpSum([(1.0, "Sz", 0, "Sz", 3)])  # a diagonal pair: no edge holds both sites
    with pytest.raises(ValueError):
        gbtn.group_terms(far, tn)


def test_named_operators_for_expect():
    tn = gbtn.square_lattice(2, 2, chi=1)
    from gbtn.opsum import named_operator
    np.testing.assert_array_equal(named_operator("Sz", tn), np.diag([0.5, -0.5]))
    np.testing.assert_array_equal(named_operator("S+", tn), [[0.0, 1.0], [0.0, 0.0]])  # S+|dn> = |up>: O[up, dn]
    with pytest.raises(ValueError):
        named_operator("Sy", tn)  # imaginary: the library reports real parts of real operators
    with pytest.raises(ValueError):
        named_operator("Sq", tn)
    t3 = gbtn.TensorNetwork(tn.nv, tn.edges, [3, 2, 2, 2], tn.edge_dims)
    with pytest.raises(ValueError):
        named_operator("Sz", t3)


def test_complex_terms_give_the_oracle_gates():
    # Sy is imaginary: an XY model with a field makes complex Hermitian edge
    # terms, and its Trotter gates exp(-dbeta/2 h) are complex
    tn = gbtn.square_lattice(3, 2, chi=1)
    g = O.square_lattice(3, 2, chi=1)
    H = gbtn.OpSum()
    terms = []
    for (u, v) in tn.edges:
        for name in ("Sx", "Sy"):
            H += (0.7, name, u, name, v)
            terms.append((0.7, [(name, u), (name, v)]))
    for v in range(tn.nv):
        H += (0.3, "Sz", v)
        terms.append((0.3, [("Sz", v)]))
    a = gbtn.trotter2_gates(gbtn.group_terms(H, tn), tn, 0.1)
    b = O.trotter2_gates(g, O.group_terms(terms, g), 0.1)
    assert [e for e, _ in a] == [e for e, _ in b]
    for (_, x), (_, y) in zip(a, b):
        np.testing.assert_allclose(x, y, rtol=0, atol=1e-14)
    # Sx Sx + Sy Sy is real (the imaginary parts cancel), so these gates are real
    assert not any(np.iscomplexobj(x) and np.any(np.imag(x)) for _, x in a)
    # S+ S- is real but not Hermitian, Sy Sz is imaginary: the gate (a general
    # matrix exponential, no Hermitian assumption) is complex
    Hc = gbtn.OpSum([(1.0, "S+", 0, "S-", 1), (1.0, "Sy", 0, "Sz", 1)])
    h = gbtn.trotter2_gates(gbtn.group_terms(Hc, tn), tn, 0.2)[0][1]
    assert np.iscomplexobj(h) and np.any(np.imag(h))
