"""The oracle's ASCI-PT2 (asci_pt2_constraint, pt2.hpp:59-565) against its
definition on small spaces: E_PT2 = sum over every determinant Q of the full
space outside the wavefunction of (sum_P C_P <Q|H|P>)^2 / (E0 - <Q|H|Q>),
with exact matrix elements and diagonals (the oracle's fast diagonals agree
to rounding).  Complements the reference's pinned water value
(test_oracle_golden.py).  No GPU."""
import numpy as np
import pytest


def _brute_pt2(H, a, b, C, E0, full_a, full_b):
    inside = set(zip(a.tolist(), b.tolist()))
    e = 0.
    nq = 0
    for qa, qb in zip(full_a.tolist(), full_b.tolist()):
        if (qa, qb) in inside:
            continue
        v = sum(c * H.matrix_element((qa, qb), (pa, pb)) for pa, pb, c in zip(a.tolist(), b.tolist(), C))
        if v == 0.:
            continue
        hqq = H.matrix_element((qa, qb), (qa, qb))
        e += v * v / (E0 - hqq)
        nq += 1
    return e, nq


@pytest.mark.parametrize("norb,na,nb,keep,seed", [(6, 3, 3, 40, 1), (7, 2, 3, 25, 2), (6, 2, 2, 30, 3)])
def test_pt2_matches_definition(oracle, pkg, norb, na, nb, keep, seed):
    T, V, _ = pkg.integrals.synthetic_integrals(norb, 2 * norb, seed)
    H = oracle.Hamiltonian(T, V)
    fa, fb = pkg.determinants.spin_sort(*pkg.determinants.fci_space(norb, na, nb))
    rng = np.random.default_rng(seed)
    sel = np.sort(rng.choice(len(fa), size=keep, replace=False))
    a, b = fa[sel], fb[sel]
    C = rng.standard_normal(keep)
    C /= np.linalg.norm(C)
    E0 = -abs(rng.standard_normal()) - 20.0
    e, n = oracle.asci_pt2(H, a, b, C, E0, pt2_tol=0.0)
    eb, nbq = _brute_pt2(H, a, b, C, E0, fa, fb)
    assert abs(e - eb) < 1e-12 * max(1., abs(eb))
    assert n >= nbq  # accidental zero sums of nonzero terms are still counted by the oracle
