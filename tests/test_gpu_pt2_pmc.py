"""ASCI-PT2 (qdkgb_asci_pt2) and the projected multi-configuration calculator
on the GPU, against the CPU oracle and the reference's pinned value:

* water cc-pVDZ, 5+5 electrons, ASCI grown and refined to 10,000 determinants
  (Fixed core): E_PT2 = -5.701535028967e-3 (external/macis/tests/asci.cxx:
  556-570, tolerance 1e-8); the GPU and the oracle also agree on the number of
  external determinants and to 1e-12 on E_PT2, in one pass and split into
  passes by a small table bound;
* a complete active space has no external determinant (E_PT2 = 0);
* an unsorted wavefunction is refused, as the reference does (pt2.hpp:79-80);
* PMC (macis_pmc.cpp:42-178) on a determinant subset of N2 CAS(6e,6o) in the
  caller's order: energy = the oracle's H build + Davidson on the same list to
  1e-10, a single determinant gives <D|H|D>, the RDM traces are the electron
  counts."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def capi(pkg):
    pkg.build.build()
    return pkg.capi


@pytest.fixture(scope="module")
def h2o_wfn(oracle, pkg, h2o, known):
    ref = known["h2o_asci_10k"]
    H = oracle.Hamiltonian(h2o["T"], h2o["V"])
    a0, b0 = pkg.determinants.canonical_hf(5, 5)
    E0 = H.matrix_element((a0, b0), (a0, b0))
    E, a, b, c, _ = oracle.asci(H, [a0], [b0], [1.0], E0, ntdets_max=ref["ntdets_max"], core_fixed=1)
    return H, E, a, b, c


def test_pt2_water_matches_reference_and_oracle(capi, oracle, h2o, h2o_wfn, known):
    H, E, a, b, c = h2o_wfn
    e_orc, n_orc = oracle.asci_pt2(H, a, b, c, E)
    with capi.Context(0) as ctx:
        ctx.set_integrals(h2o["T"], h2o["V"])
        e1, n1 = capi.asci_pt2(ctx, a, b, c, E)
        e3, n3 = capi.asci_pt2(ctx, a, b, c, E, max_slots=1 << 22)  # a table of 2^22 slots: four passes
    ref = known["h2o_asci_10k"]
    assert abs(e1 - ref["EPT2"]) < ref["atol"]
    assert n1 == n_orc and abs(e1 - e_orc) < 1e-12
    assert n3 == n1 and abs(e3 - e1) < 1e-12


def test_pt2_complete_space_and_sorted_input(capi, oracle, pkg, n2_6e6o):
    a, b = pkg.determinants.spin_sort(*pkg.determinants.fci_space(6, 3, 3))  # PT2 wants spin order
    H = oracle.Hamiltonian(n2_6e6o["T"], n2_6e6o["V"])
    E, X, _ = oracle.build_csr(H, a, b).selected_ci_diag(tol=1e-10)
    with capi.Context(0) as ctx:
        ctx.set_integrals(n2_6e6o["T"], n2_6e6o["V"])
        e, n = capi.asci_pt2(ctx, a, b, X, E)
        assert e == 0.0 and n == 0
        with pytest.raises(capi.QdkgbError, match="Sorted"):
            capi.asci_pt2(ctx, a[::-1], b[::-1], X[::-1], E)
    # a truncated space has external determinants; GPU = oracle
    sel = np.argsort(-np.abs(X), kind="stable")[:60]
    sel.sort()
    Hs = oracle.build_csr(H, a[sel], b[sel])
    Es, Xs, _ = Hs.selected_ci_diag(max_m=59, tol=1e-10)
    e_orc, n_orc = oracle.asci_pt2(H, a[sel], b[sel], Xs, Es)
    with capi.Context(0) as ctx:
        ctx.set_integrals(n2_6e6o["T"], n2_6e6o["V"])
        e, n = capi.asci_pt2(ctx, a[sel], b[sel], Xs, Es)
    assert n == n_orc and n > 0 and abs(e - e_orc) < 1e-13 and e < 0


def test_pmc_matches_oracle(pkg, oracle, n2_6e6o):
    calc = pkg.calculators
    a, b = pkg.determinants.fci_space(6, 3, 3)
    rng = np.random.default_rng(7)
    sel = rng.choice(len(a), size=150, replace=False)  # the caller's order, unsorted
    cfgs = [pkg.determinants.to_canonical_string(a[i], b[i], 6) for i in sel]
    ham = calc.Hamiltonian(n2_6e6o["T"], n2_6e6o["V"], n2_6e6o["E_core"])
    p = calc.create("projected_multi_configuration_calculator")
    p.settings().set("calculate_one_rdm", True)
    p.settings().set("ci_residual_tolerance", 1e-10)
    E, wfn = p.run(ham, cfgs)
    Ho = oracle.Hamiltonian(n2_6e6o["T"], n2_6e6o["V"])
    Eo, Xo, _ = oracle.build_csr(Ho, a[sel], b[sel]).selected_ci_diag(max_m=149, tol=1e-10)
    assert abs(E - (Eo + n2_6e6o["E_core"])) < 1e-10
    assert wfn.get_configurations() == cfgs
    assert abs(abs(wfn.coefficients @ Xo) - 1.0) < 1e-8  # the same vector, in the caller's order
    assert abs(np.trace(wfn.get_active_one_rdm_spin_traced()) - 6.0) < 1e-10
    # one determinant: <D|H|D> + E_core
    E1, w1 = calc.create("projected_multi_configuration_calculator").run(ham, cfgs[:1])
    assert abs(E1 - (Ho.matrix_element((a[sel[0]], b[sel[0]]), (a[sel[0]], b[sel[0]])) + n2_6e6o["E_core"])) < 1e-12
    assert w1.coefficients.tolist() == [1.0]


@pytest.mark.late
def test_pmc_repeated_configurations(pkg, oracle, n2_6e6o):
    """A configuration list that repeats determinants (test_pmc.py:104-141
    passes "222000" twice): the energy and vector are the lowest eigenpair of
    the matrix MACIS builds for the list as given (the oracle's double loop,
    dense here) and the RDMs are the oracle's form_rdms over the list with the
    returned coefficients; one determinant given twice has 2 <D|H|D>."""
    import scipy.sparse as sp
    calc, det = pkg.calculators, pkg.determinants
    a, b = det.fci_space(6, 3, 3)
    rng = np.random.default_rng(11)
    sel = rng.choice(len(a), 20, replace=False)
    lst = np.concatenate([sel, sel[[2, 5, 5]]])
    rng.shuffle(lst)
    cfgs = [det.to_canonical_string(a[i], b[i], 6) for i in lst]
    ham = calc.Hamiltonian(n2_6e6o["T"], n2_6e6o["V"], n2_6e6o["E_core"])
    H = oracle.Hamiltonian(n2_6e6o["T"], n2_6e6o["V"])
    E_core = n2_6e6o["E_core"]

    def dense(la, lb):
        rp, ci, nz = oracle.build_csr(H, la, lb).arrays()
        return sp.csr_matrix((nz, ci, rp), shape=(len(la),) * 2).toarray()

    p = calc.create("projected_multi_configuration_calculator")
    p.settings().set("calculate_one_rdm", True)
    p.settings().set("calculate_two_rdm", True)
    E, wfn = p.run(ham, cfgs)
    w, X = np.linalg.eigh(dense(a[lst], b[lst]))
    assert wfn.size() == len(cfgs) and wfn.get_configurations() == cfgs
    assert abs(E - (w[0] + E_core)) < 1e-10
    assert abs(abs(wfn.coefficients @ X[:, 0]) - 1.0) < 1e-8
    Ro = oracle.rdms_spin_dep(6, a[lst], b[lst], wfn.coefficients)
    aa, bb = wfn.get_active_one_rdm_spin_dependent()
    aabb, aaaa, bbbb = wfn.get_active_two_rdm_spin_dependent()
    np.testing.assert_allclose(aa, Ro["aa"], atol=1e-10, rtol=0)
    np.testing.assert_allclose(bb, Ro["bb"], atol=1e-10, rtol=0)
    for got, key in ((aabb, "aabb"), (aaaa, "aaaa"), (bbbb, "bbbb")):
        np.testing.assert_allclose(got, 2.0 * Ro[key].ravel(order="F"), atol=1e-10, rtol=0)
    # the reference's three-configuration case, on this active space
    three = ["222000", "22ud00", "222000"]
    E3, w3 = calc.create("projected_multi_configuration_calculator").run(ham, three)
    a3 = np.array([det.from_canonical_string(s)[0] for s in three], np.uint64)
    b3 = np.array([det.from_canonical_string(s)[1] for s in three], np.uint64)
    hf = H.matrix_element((7, 7), (7, 7))
    assert w3.size() == 3 and E3 < hf + E_core
    assert abs(E3 - (np.linalg.eigvalsh(dense(a3, b3))[0] + E_core)) < 1e-10
    E2, w2 = calc.create("projected_multi_configuration_calculator").run(ham, ["222000", "222000"])
    assert abs(E2 - (2 * hf + E_core)) < 1e-10 and w2.size() == 2
