"""The oracle's orbital entropies (form_entropies, sorted_double_loop.hpp:
755-903, entropies.hpp) pinned against their definition: von Neumann entropies
of the one- and two-orbital reduced density matrices built here by explicit
partial traces of the CI vector (determinants ordered alpha block then beta
block, ascending orbital index: the sign convention of MACIS's excitation
signs).  The reference's own entropy tests need SCF integrals that are not
available here; these identities hold for any normalised vector.  No GPU."""
import numpy as np
import pytest


def _brute(n, A, B, C):
    def occ_list(a, b):
        return [(p, 0) for p in range(n) if (a >> p) & 1] + [(p, 1) for p in range(n) if (b >> p) & 1]

    eps = np.finfo(float).eps
    s1 = np.zeros(n)
    for i in range(n):
        p = np.zeros(4)
        for a, b, c in zip(A, B, C):
            p[((int(a) >> i) & 1) + 2 * ((int(b) >> i) & 1)] += c * c
        s1[i] = -sum(x * np.log(x) for x in p if x > eps)
    s2 = np.zeros((n, n))
    for i in range(n):
        for j in range(i + 1, n):
            loc = [(i, 0), (j, 0), (i, 1), (j, 1)]
            envs = {}
            for a, b, c in zip(A, B, C):
                ol = occ_list(int(a), int(b))
                target = [x for x in loc if x in ol] + [x for x in ol if x not in loc]
                pos = [ol.index(x) for x in target]
                inv = sum(1 for u in range(len(pos)) for v in range(u + 1, len(pos)) if pos[u] > pos[v])
                k = sum(1 << t for t, x in enumerate(loc) if x in ol)
                envs.setdefault(tuple(x for x in ol if x not in loc), np.zeros(16))[k] += (-1) ** inv * c
            w = np.linalg.eigvalsh(sum(np.outer(v, v) for v in envs.values()))
            s2[i, j] = s2[j, i] = -sum(x * np.log(x) for x in w if x > eps)
    return s1, s2


@pytest.mark.parametrize("n,na,nb,seed", [(4, 2, 2, 1), (5, 3, 2, 2), (6, 3, 3, 3), (5, 1, 1, 4), (6, 2, 1, 5)])
def test_entropies_match_partial_traces(oracle, pkg, n, na, nb, seed):
    a, b = pkg.determinants.spin_sort(*pkg.determinants.fci_space(n, na, nb))
    rng = np.random.default_rng(seed)
    if seed % 2:  # a selected (incomplete) space
        keep = np.sort(rng.choice(len(a), size=max(2, 2 * len(a) // 3), replace=False))
        a, b = a[keep], b[keep]
    C = rng.standard_normal(len(a))
    C /= np.linalg.norm(C)
    s1, s2, mi = oracle.entropies(n, a, b, C)
    t1, t2 = _brute(n, a, b, C)
    np.testing.assert_allclose(s1, t1, atol=1e-13, rtol=0)
    np.testing.assert_allclose(s2, t2, atol=1e-13, rtol=0)
    np.testing.assert_allclose(mi, s1[:, None] + s1[None, :] - s2 - np.diag(2 * s1), atol=1e-13, rtol=0)


def test_entropies_casci_vector(oracle, pkg, n2_6e6o):
    a, b = pkg.determinants.spin_sort(*pkg.determinants.fci_space(6, 3, 3))
    H = oracle.Hamiltonian(n2_6e6o["T"], n2_6e6o["V"])
    _, X, _ = oracle.build_csr(H, a, b).selected_ci_diag(tol=1e-10)
    s1, s2, mi = oracle.entropies(6, a, b, X)
    t1, t2 = _brute(6, a, b, X)
    assert np.abs(s1 - t1).max() < 1e-12 and np.abs(s2 - t2).max() < 1e-12
    # a single determinant has no entropy
    z1, z2, z3 = oracle.entropies(6, a[:1], b[:1], np.ones(1))
    assert not z1.any() and not z2.any() and not z3.any()
