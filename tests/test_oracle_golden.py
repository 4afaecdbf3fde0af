"""The CPU oracle pinned against the reference's own golden vectors and known
answers (external/macis/tests, external/macis/python/tests).  No GPU."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, load_package


def _h2o_cisd(pkg):
    d = pkg.determinants
    a, b = d.cisd_space(24, *d.canonical_hf(5, 5))
    return d.spin_sort(a, b)


def test_fci_order_matches_generate_combs(oracle, pkg):
    # prev_permutation order == lexicographic combinations
    for n, k in [(6, 3), (8, 4), (10, 3), (12, 6)]:
        assert np.array_equal(oracle.combs(n, k), pkg.determinants.combs(n, k))
    a, b = pkg.determinants.fci_space(6, 3, 2)
    oa, ob = oracle.fci_dets(6, 3, 2)
    assert np.array_equal(a, oa) and np.array_equal(b, ob)
    assert a[0] == 0b111 and b[0] == 0b11  # first string = lowest orbitals (HF)


def test_h2o_cisd_csr_matches_reference_rowptr(oracle, pkg, h2o, known):
    """external/macis/tests/csr_hamiltonian.cxx:46-106: n, nnz and rowptr."""
    a, b = _h2o_cisd(pkg)
    ref = known["h2o_cisd_csr"]
    assert len(a) == ref["n"]
    H = oracle.Hamiltonian(h2o["T"], h2o["V"])
    M = oracle.build_csr(H, a, b, ref["thresh"])
    rp, ci, nz = M.arrays()
    assert M.nnz == ref["nnz"]
    golden = np.load(GOLDEN + "/h2o_ccpvdz_cisd_rowptr.npy")
    assert np.array_equal(rp, golden.astype(np.int64))
    # columns sorted within rows, symmetric pattern
    for i in range(0, len(a), 997):
        cols = ci[rp[i]:rp[i + 1]]
        assert np.all(np.diff(cols) > 0)


def test_h2o_cisd_davidson_energy(oracle, pkg, h2o, known):
    """external/macis/tests/davidson.cxx:44-75."""
    ref = known["h2o_cisd_davidson"]
    d = pkg.determinants
    a, b = d.cisd_space(24, *d.canonical_hf(5, 5))  # reference order (not sorted)
    H = oracle.Hamiltonian(h2o["T"], h2o["V"])
    M = oracle.build_csr(H, a, b, 1e-16)
    E, X, it = M.selected_ci_diag(max_m=ref["max_m"], tol=ref["tol"])
    assert abs(E + h2o["E_core"] - ref["E0_total"]) < ref["atol"]
    assert abs(np.linalg.norm(X) - 1.0) < 1e-12
    assert abs(X @ M.spmv(X) - E) < 1e-12


def test_n2_casci_energy(oracle, pkg, n2_6e6o, known):
    """external/macis/python/tests/test_pymacis.py:114-142 (electronic energy)."""
    ref = known["n2_6e6o_casci"]
    a, b = pkg.determinants.fci_space(6, 3, 3)
    assert len(a) == ref["ndets"]
    H = oracle.Hamiltonian(n2_6e6o["T"], n2_6e6o["V"])
    M = oracle.build_csr(H, a, b)
    E, X, _ = M.selected_ci_diag()
    assert np.isclose(E, ref["E_total"])


def test_o2_rdms_pinned_sums_and_identities(oracle, pkg):
    """external/macis/tests/double_loop.cxx:506-579 (O2 wavefunction, padded
    to 5000 states with empty determinants)."""
    w = np.load(GOLDEN + "/o2_wfn.npz")
    known = {"sum_abs_ordm": 8.0000005763, "sum_abs_trdm": 44.1092472977}
    n = 34
    a = np.zeros(5000, dtype=np.uint64)
    b = np.zeros(5000, dtype=np.uint64)
    C = np.zeros(5000)
    m = len(w["alpha"])
    a[:m], b[:m], C[:m] = w["alpha"], w["beta"], w["coeffs"]
    C /= np.linalg.norm(C)
    R = oracle.rdms_spin_dep(n, a, b, C)
    ordm = R["aa"] + R["bb"]
    trdm = R["aaaa"] + R["bbbb"] + R["aabb"] + R["aabb"].transpose(2, 3, 0, 1)
    assert abs(np.abs(ordm).sum() - known["sum_abs_ordm"]) < 1e-6
    assert abs(np.abs(trdm).sum() - known["sum_abs_trdm"]) < 1e-6
    assert abs(np.trace(ordm) - (int(w["nalpha"]) + int(w["nbeta"]))) < 1e-6
    assert np.allclose(ordm, ordm.T, atol=1e-6)


def test_rdm_energy_identity_cas(oracle, pkg):
    """E = T.(g_a+g_b) + V.(G_aaaa+G_bbbb) + 2 V.G_aabb (double_loop.cxx:215-241)."""
    T, V, _ = pkg.integrals.synthetic_integrals(6, 8, seed=3)
    a, b = pkg.determinants.fci_space(6, 3, 3)
    H = oracle.Hamiltonian(T, V)
    M = oracle.build_csr(H, a, b)
    E, X, _ = M.selected_ci_diag()
    R = oracle.rdms_spin_dep(6, a, b, X)
    E_rdm = (np.sum(T * (R["aa"] + R["bb"])) + np.sum(V * (R["aaaa"] + R["bbbb"]))
             + 2 * np.sum(V * R["aabb"]))
    assert abs(E_rdm - E) < 1e-10


def test_matrix_element_symmetry_and_diag(oracle, pkg):
    T, V, _ = pkg.integrals.synthetic_integrals(8, 16, seed=1)
    assert np.array_equal(V, V.transpose(1, 0, 2, 3)) and np.array_equal(V, V.transpose(2, 3, 0, 1))
    H = oracle.Hamiltonian(T, V)
    a, b = pkg.determinants.fci_space(8, 4, 4)
    M = oracle.build_csr(H, a, b)
    rp, ci, nz = M.arrays()
    # symmetric matrix, 361 elements per row for CAS(8,8)
    assert np.all(np.diff(rp) == 361)
    import scipy.sparse as sp
    A = sp.csr_matrix((nz, ci, rp), shape=(len(a), len(a)))
    assert abs(A - A.T).max() < 1e-14


def test_jacobi_syev(oracle):
    rng = np.random.default_rng(0)
    A = rng.normal(size=(17, 17))
    A = A + A.T
    w, Q = oracle.syev(A)
    wr = np.linalg.eigvalsh(A)
    assert np.allclose(w, wr, atol=1e-12)
    assert np.allclose(Q.T @ A @ Q, np.diag(w), atol=1e-11)


def test_h2o_asci_grow_refine_energies(oracle, pkg, h2o, known):
    """external/macis/tests/asci.cxx:488-574 (Fixed core, ntdets_max 10000)."""
    ref = known["h2o_asci_10k"]
    H = oracle.Hamiltonian(h2o["T"], h2o["V"])
    a0, b0 = pkg.determinants.canonical_hf(5, 5)
    E0 = H.matrix_element((a0, b0), (a0, b0))
    E, a, b, c, Eg = oracle.asci(H, [a0], [b0], [1.0], E0, ntdets_max=ref["ntdets_max"], core_fixed=1)
    assert abs(Eg - ref["E0_grow"]) < 1e-8
    assert abs(E - ref["E0_refine"]) < 1e-8
    assert len(a) == 10000 and abs(c @ c - 1.0) < 1e-12
    # ASCI-PT2 of the refined wavefunction (asci.cxx:556-570); one pass and a
    # hash-partitioned run agree
    ept2, npt2 = oracle.asci_pt2(H, a, b, c, E)
    assert abs(ept2 - ref["EPT2"]) < ref["atol"]
    e4, n4 = oracle.asci_pt2(H, a, b, c, E, pass_max=1 << 23)
    assert n4 == npt2 and abs(e4 - ept2) < 1e-14
    # the reference refuses an unsorted wavefunction (pt2.hpp:79-80)
    with pytest.raises(RuntimeError, match="Sorted"):
        oracle.asci_pt2(H, a[::-1].copy(), b[::-1].copy(), c[::-1].copy(), E)


def test_n2_asci_energy(oracle, pkg, n2_14e18o, known):
    """external/macis/python/tests/test_pymacis.py:158-187."""
    ref = known["n2_14e18o_asci"]
    H = oracle.Hamiltonian(n2_14e18o["T"], n2_14e18o["V"])
    a0, b0 = pkg.determinants.canonical_hf(7, 7)
    E0 = H.matrix_element((a0, b0), (a0, b0))
    E, a, b, c, _ = oracle.asci(H, [a0], [b0], [1.0], E0, ntdets_max=ref["ntdets_max"],
                                grow_factor=ref["grow_factor"], max_refine_iter=ref["max_refine_iter"],
                                ci_max_subspace=ref["max_subspace"])
    assert np.isclose(E, ref["E_total"])
    assert abs(E - ref["E_total"]) < 1e-8
    assert len(a) == ref["ndets"] and np.isclose(np.linalg.norm(c), 1.0)


def test_h2o_casscf_energy(oracle, h2o, known):
    """external/macis/tests/mcscf.cxx:26-66: water cc-pVDZ, 1 inactive +
    CAS(8e,8o), no starting RDMs, E = -76.1114493227 (1e-8)."""
    ref = known["h2o_casscf"]
    E, g, G, iters, conv = oracle.casscf(h2o["T"], h2o["V"], h2o["E_core"], ref["nalpha"], ref["nbeta"],
                                         ref["ninact"], ref["nact"])
    assert conv and iters > 0
    assert abs(E - ref["E_total"]) < ref["atol"]
    assert abs(np.trace(g) - 8.0) < 1e-10


def test_h2o_casscf_from_reference_rdms(oracle, h2o, known):
    """mcscf.cxx:67-79 ("With Guess"): the same CASSCF started from the
    reference's stored CAS(8e,8o) RDMs (ref_data/h2o.ccpvdz.cas88.rdms.bin)
    reaches the same energy."""
    ref = known["h2o_casscf"]
    d = np.load(os.path.join(GOLDEN, "h2o_ccpvdz_cas88_rdms.npz"))
    n = int(d["nact"])
    g0, G0 = d["ordm"].reshape(n, n, order="F"), d["trdm"].reshape((n,) * 4, order="F")
    assert abs(np.trace(g0) - 8.0) < 1e-10
    E, _, _, iters, conv = oracle.casscf(h2o["T"], h2o["V"], h2o["E_core"], ref["nalpha"], ref["nbeta"],
                                         ref["ninact"], ref["nact"], rdm1=g0, rdm2=G0)
    assert conv and abs(E - ref["E_total"]) < ref["atol"]



def test_casscf_building_blocks_match_reference_sums(oracle, h2o, known):
    """external/macis/tests/fock_matrices.cxx:26-256 (tolerance 1e-6): the
    inactive Fock matrix sum and inactive energy for 0 .. 23 inactive
    orbitals; with the stored CAS(8e,8o) RDMs at 1 inactive + 8 active
    orbitals the sums of the active Fock matrix, the auxiliary Q matrix and
    the generalized Fock matrix, and the energy formed from the last."""
    ref = known["h2o_fock_matrices"]
    tol = ref["atol"]
    for ni, (s_ref, e_ref) in enumerate(zip(ref["inactive_sums"], ref["inactive_energies"])):
        Fi, _, _, _, Ei, _ = oracle.mcscf_fock(h2o["T"], h2o["V"], ni, 0)
        assert abs(Fi.sum() - s_ref) < tol, ni
        assert abs(Ei - e_ref) < tol, ni
    d = np.load(os.path.join(GOLDEN, "h2o_ccpvdz_cas88_rdms.npz"))
    n = int(d["nact"])
    assert (ref["ninact"], ref["nact"]) == (1, n)
    g0, G0 = d["ordm"].reshape(n, n, order="F"), d["trdm"].reshape((n,) * 4, order="F")
    _, Fa, Q, F, _, Ef = oracle.mcscf_fock(h2o["T"], h2o["V"], ref["ninact"], n, g0, G0)
    assert abs(Fa.sum() - ref["active_fock_sum"]) < tol
    assert abs(Q.sum() - ref["aux_q_sum"]) < tol
    assert abs(F.sum() - ref["generalized_fock_sum"]) < tol
    assert abs(Ef - ref["E_from_generalized_fock"]) < tol


def test_water_slater_condon_values(oracle, h2o, known):
    """external/macis/tests/double_loop.cxx:22-241 on the water cc-pVDZ
    integrals (tolerance 1e-6): the HF energy, the diagonals of a single, a
    same-spin and an opposite-spin double excitation, Brillouin's theorem for
    every single, the MP2 energy summed from <HF|H|D> over all doubles, and the
    HF RDM energy identities (spin-traced and spin-separated)."""
    ref = known["h2o_double_loop"]
    tol = ref["atol"]
    T, V, n, no = h2o["T"], h2o["V"], h2o["norb"], 5
    H = oracle.Hamiltonian(T, V)
    hf = ((1 << no) - 1, (1 << no) - 1)
    me = lambda bra, ket: H.matrix_element(bra, ket)
    EHF = me(hf, hf)
    assert abs(EHF + h2o["E_core"] - ref["E_HF_total"]) < tol
    s = (hf[0] ^ 1 ^ (1 << no), hf[1])
    assert abs(me(s, s) - ref["E_single_diag"]) < tol
    d_ss = (hf[0] ^ 0b11 ^ (0b11 << no), hf[1])
    assert abs(me(d_ss, d_ss) - ref["E_double_ss_diag"]) < tol
    d_os = (hf[0] ^ 1 ^ (1 << no), hf[1] ^ 0b10 ^ (0b10 << no))
    assert abs(me(d_os, d_os) - ref["E_double_os_diag"]) < tol
    for i in range(no):
        for a in range(no, n):
            for ex in ((hf[0] ^ (1 << i) ^ (1 << a), hf[1]), (hf[0], hf[1] ^ (1 << i) ^ (1 << a))):
                h1, h2 = me(hf, ex), me(ex, hf)
                assert abs(h1) < tol and abs(h1 - h2) < 1e-14
    eps = np.array([T[p, p] + sum(2 * V[p, p, i, i] - V[p, i, i, p] for i in range(no)) for p in range(n)])
    emp2 = 0.0
    vir, occ = range(no, n), range(no)
    for a in vir:
        for b in vir:
            for i in occ:
                for j in occ:
                    den = eps[a] + eps[b] - eps[i] - eps[j]
                    if a < b and i < j:  # same spin, alpha and beta
                        m = (1 << i) ^ (1 << j) ^ (1 << a) ^ (1 << b)
                        for ex in ((hf[0] ^ m, hf[1]), (hf[0], hf[1] ^ m)):
                            h = me(hf, ex)
                            emp2 += h * h / den
                    ex = (hf[0] ^ (1 << i) ^ (1 << a), hf[1] ^ (1 << j) ^ (1 << b))
                    h = me(hf, ex)
                    emp2 += h * h / den
    assert abs(-emp2 - ref["EMP2"]) < tol
    R = oracle.rdms_spin_dep(n, np.array([hf[0]], np.uint64), np.array([hf[1]], np.uint64), np.ones(1))
    E_sep = np.sum(T * (R["aa"] + R["bb"])) + np.sum(V * (R["aaaa"] + R["bbbb"])) + 2 * np.sum(V * R["aabb"])
    G = R["aaaa"] + R["bbbb"] + R["aabb"] + R["aabb"].transpose(2, 3, 0, 1)
    E_tr = np.sum(T * (R["aa"] + R["bb"])) + np.sum(V * G)
    assert abs(E_sep - EHF) < tol and abs(E_tr - EHF) < tol


@pytest.mark.parametrize("na,nb", [(5, 5), (5, 3)])
def test_hf_rdm_structure_34_orbitals(oracle, na, nb):
    """double_loop.cxx:243-298 (closed shell, 5+5) and :430-504 (open shell,
    5+3): the spin-traced RDMs of the HF determinant over 34 orbitals, as
    equalities: Gamma_iikk = n_i n_k / 2 and Gamma_ikki = -(na_i na_k +
    nb_i nb_k) / 2 for i != k, Gamma_iiii = na_i nb_i, gamma = diag(n), every
    other element zero (the reference bounds the same elements: 2 / 1,
    -1 / -0.5 and 1)."""
    n = 34
    A = np.array([(1 << na) - 1], np.uint64)
    B = np.array([(1 << nb) - 1], np.uint64)
    R = oracle.rdms_spin_dep(n, A, B, np.ones(1))
    G = R["aaaa"] + R["bbbb"] + R["aabb"] + R["aabb"].transpose(2, 3, 0, 1)
    g = R["aa"] + R["bb"]
    oa = np.array([1.0 if p < na else 0.0 for p in range(n)])
    ob = np.array([1.0 if p < nb else 0.0 for p in range(n)])
    occ = oa + ob
    Gref = np.zeros((n,) * 4)
    for i in range(n):
        for k in range(n):
            if i == k:
                Gref[i, i, i, i] = oa[i] * ob[i]
            else:
                Gref[i, i, k, k] = 0.5 * occ[i] * occ[k]
                Gref[i, k, k, i] = -0.5 * (oa[i] * oa[k] + ob[i] * ob[k])
    assert np.abs(G - Gref).max() < 1e-14
    assert np.abs(g - np.diag(occ)).max() < 1e-14


def test_davidson_solver_reference_cases(oracle):
    """python/tests/test_davidson_solver.py:17-71: davidson_solver (diagonal
    guess + davidson, tol 1e-8, max_m 20) on a 6 x 6 tridiagonal and the
    two-site Heisenberg model; eigenvalue and |overlap| with the analytic
    eigenvector to the reference's 1e-12."""
    from conftest import davidson_solver_cases
    for name, A, E_ref, v_ref in davidson_solver_cases():
        A.sort_indices()
        M = oracle.csr_from_arrays(A.indptr, A.indices, A.data)
        E, X, _ = M.selected_ci_diag(max_m=20, tol=1e-8)
        assert abs(E - E_ref) < 1e-12 + 1e-12 * abs(E_ref), name
        assert X.shape == v_ref.shape and abs(abs(X @ v_ref) - 1.0) < 1e-12, name
