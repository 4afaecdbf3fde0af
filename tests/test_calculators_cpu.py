"""qdk-style plugin surface: registry, settings (names, defaults, bounds,
locking), containers.  No GPU."""
import numpy as np
import pytest


def test_registry_and_defaults(pkg):
    calc = pkg.calculators
    kinds = calc.available()
    assert kinds["multi_configuration_calculator"] == ["gb300_asci", "gb300_cas"]
    assert calc.available("multi_configuration_calculator") == ["gb300_asci", "gb300_cas"]
    c = calc.create("multi_configuration_calculator")
    assert c.name() == "gb300_cas"
    s = c.settings()
    # mc.hpp:34-62 and macis_base.hpp:27-36 defaults
    assert s.get("ci_residual_tolerance") == 1e-6
    assert s.get("max_solver_iterations") == 200
    assert s.get("iterative_solver_dimension_cutoff") == 2000
    assert s.get("calculate_one_rdm") is False and s.get("calculate_two_rdm") is False
    assert s.get("ci_matel_tol") == np.finfo(float).eps
    with pytest.raises(KeyError):
        calc.create("multi_configuration_calculator", "no_such_solver")
    with pytest.raises(KeyError):
        calc.create("no_such_kind", "gb300_cas")


def test_settings_validation_and_lock(pkg):
    c = pkg.calculators.create("multi_configuration_calculator", "gb300_cas")
    s = c.settings()
    with pytest.raises(ValueError):
        s.set("ci_residual_tolerance", 2.0)  # BoundConstraint [0, 1]
    with pytest.raises(ValueError):
        s.set("max_solver_iterations", 0)
    with pytest.raises(TypeError):
        s.set("calculate_one_rdm", 1)
    with pytest.raises(TypeError):
        s.set("precision", 5)
    with pytest.raises(KeyError):
        s.set("not_a_setting", 1)
    s.set("ci_residual_tolerance", 1e-9)
    s.lock()
    with pytest.raises(pkg.calculators.SettingsAreLocked):
        s.set("ci_residual_tolerance", 1e-7)


def test_wavefunction_container(pkg):
    d = pkg.determinants
    a, b = d.fci_space(4, 2, 2)
    C = np.ones(len(a)) / np.sqrt(len(a))
    w = pkg.calculators.Wavefunction(4, a, b, C)
    cfg = w.get_configurations()
    assert cfg[0] == "2200" and len(cfg) == 36
    with pytest.raises(RuntimeError):
        w.get_active_one_rdm_spin_dependent()


def test_hamiltonian_from_fcidump_roundtrip(pkg, tmp_path):
    T, V, _ = pkg.integrals.synthetic_integrals(5, 6, seed=2)
    p = tmp_path / "x.fcidump"
    pkg.integrals.write_fcidump(str(p), T, V, E_core=1.25, nelec=4)
    H = pkg.calculators.Hamiltonian.from_fcidump(str(p))
    assert H.norb == 5 and H.get_core_energy() == 1.25
    assert np.allclose(H.get_one_body_integrals(), T, atol=1e-15)
    assert np.allclose(H.get_two_body_integrals(), V, atol=1e-15)


def test_synthetic_integrals_recipe(pkg):
    T, V, ec = pkg.integrals.synthetic_integrals(12, 24, seed=7)
    assert ec == 0.0 and T.shape == (12, 12) and V.shape == (12,) * 4
    assert np.array_equal(T, T.T)
    for perm in [(1, 0, 2, 3), (0, 1, 3, 2), (2, 3, 0, 1), (3, 2, 1, 0)]:
        assert np.array_equal(V, V.transpose(perm))
    M = V.reshape(144, 144)
    assert np.linalg.eigvalsh(M).min() > -1e-12  # PSD
    assert np.allclose(np.diag(T), -2.0 + 0.25 * np.arange(12))


def test_pmc_plugin_surface(pkg):
    """ProjectedMultiConfigurationCalculator (pmc.hpp:31-150, macis_pmc.cpp:
    42-178): type and default name, settings, and the errors raised before any
    device work."""
    calc = pkg.calculators
    kind = "projected_multi_configuration_calculator"
    assert calc.available(kind) == ["gb300_pmc"]
    c = calc.create(kind)
    assert c.name() == "gb300_pmc" and c.type_name() == kind
    s = c.settings()
    assert s.get("iterative_solver_dimension_cutoff") == 2000 and s.get("ci_matel_tol") == np.finfo(float).eps
    H = calc.Hamiltonian(np.eye(4), np.zeros(4 ** 4))
    with pytest.raises(RuntimeError, match="cannot be empty"):
        c.run(H, [])
    with pytest.raises(RuntimeError, match="orbital capacity"):
        calc.create(kind).run(H, ["220"])
    with pytest.raises(ValueError):
        calc.create(kind).run(H, ["22x0"])
    with pytest.raises(ValueError):
        calc.create(kind).run(H, ["2200u"])  # beyond the active space
    a, b = calc.Gb300Pmc._parse(["2ud0", (0b11, 0b101)], 4)
    assert a.tolist() == [0b011, 0b11] and b.tolist() == [0b101, 0b101]
    # settings are locked once run starts, even when it fails
    with pytest.raises(calc.SettingsAreLocked):
        c.settings().set("ci_residual_tolerance", 1e-9)


def test_asci_pt2_settings(pkg):
    """MacisAsciSettings PT2 / constraint defaults (macis_asci.hpp:59-138 from
    ASCISettings, determinant_search.hpp:113-191)."""
    s = pkg.calculators.create("multi_configuration_calculator", "gb300_asci").settings()
    assert s.get("pt2_tol") == 1e-16
    assert s.get("pt2_reserve_count") == 70000000 and s.get("pt2_bigcon_thresh") == 250
    assert s.get("pt2_prune") is False and s.get("pt2_precompute_eps") is False
    assert s.get("pt2_max_constraint_level") == 5 and s.get("pt2_min_constraint_level") == 0
    assert s.get("constraint_level") == 2 and s.get("pair_size_max") == 500000000
    with pytest.raises(ValueError):
        s.set("pt2_tol", 2.0)


def test_pmc_repeated_list_math(pkg, oracle, n2_6e6o):
    """A PMC list that repeats determinants (test_pmc.py:104-141 passes one):
    the host steps of Gb300Pmc._run_repeated with the oracle standing in for
    the device.  The lowest eigenpair of M^1/2 H M^1/2 over the distinct
    determinants, mapped back, is the lowest eigenpair of the matrix the oracle
    (MACIS's double loop) builds for the list as given; the RDMs of the
    per-determinant sums c equal the oracle's RDMs of C over the list; a
    positive lowest eigenvalue gives 0 with a null vector of H'."""
    import scipy.sparse as sp
    calc, det = pkg.calculators, pkg.determinants
    a, b = det.fci_space(6, 3, 3)
    rng = np.random.default_rng(5)
    sel = rng.choice(len(a), 30, replace=False)
    lst = np.concatenate([sel, sel[[3, 7, 7, 12]]])
    rng.shuffle(lst)
    la, lb = a[lst], b[lst]
    ua, ub, inv, mult = calc.collapse_repeated(la, lb)
    assert len(ua) == 30 and mult.sum() == len(la) and sorted(mult.tolist())[-3:] == [2, 2, 3]
    assert np.array_equal(ua[inv], la) and np.array_equal(ub[inv], lb)
    assert np.array_equal(np.lexsort((ub, ua)), np.arange(30))
    H = oracle.Hamiltonian(n2_6e6o["T"], n2_6e6o["V"])
    rp, ci, nz = oracle.build_csr(H, ua, ub).arrays()
    A = sp.csr_matrix((calc.multiplicity_scaled(rp, ci, nz, mult), ci, rp), shape=(30, 30)).toarray()
    w, Y = np.linalg.eigh(A)
    E, C, c = calc.repeated_list_solution(w[0], Y[:, 0], inv, mult)
    rp2, ci2, nz2 = oracle.build_csr(H, la, lb).arrays()
    Hp = sp.csr_matrix((nz2, ci2, rp2), shape=(len(la),) * 2).toarray()
    w2, X = np.linalg.eigh(Hp)
    assert E == w[0] and abs(E - w2[0]) < 1e-12
    assert abs(C @ C - 1.0) < 1e-12 and abs(abs(C @ X[:, 0]) - 1.0) < 1e-10
    R1 = oracle.rdms_spin_dep(6, la, lb, C)
    R2 = oracle.rdms_spin_dep(6, ua, ub, c)
    assert np.abs(R1["aa"] - R2["aa"]).max() > 1e-3  # the once-counted copies
    calc.add_repeated_pair_terms(R2, 6, ua, ub, C, c, inv)
    for k in R1:
        assert np.abs(R1[k] - R2[k]).max() < 1e-12, k
    # any vector over the list, not only the eigenvector: C arbitrary, c = P^T C
    Cr = rng.standard_normal(len(la))
    cr = np.bincount(inv, weights=Cr)
    R1 = oracle.rdms_spin_dep(6, la, lb, Cr)
    R2 = oracle.rdms_spin_dep(6, ua, ub, cr)
    calc.add_repeated_pair_terms(R2, 6, ua, ub, Cr, cr, inv)
    for k in R1:
        assert np.abs(R1[k] - R2[k]).max() < 1e-12, k
    # one determinant twice: H' = h J, lowest eigenvalue 2h (h < 0) or 0 (h > 0)
    u1a, u1b, inv1, m1 = calc.collapse_repeated(la[[0, 0]], lb[[0, 0]])
    h = H.matrix_element((int(la[0]), int(lb[0])), (int(la[0]), int(lb[0])))
    E1, C1, _ = calc.repeated_list_solution(h * m1[0], np.ones(1), inv1, m1)
    assert E1 == 2 * h and np.allclose(C1, [2 ** -0.5] * 2)
    E0, C0, c0 = calc.repeated_list_solution(0.5, Y[:, 0], inv, mult)
    assert E0 == 0.0 and not np.any(c0) and abs(C0 @ C0 - 1.0) < 1e-15
    assert np.abs(Hp @ C0).max() < 1e-12
    R1 = oracle.rdms_spin_dep(6, la, lb, C0)
    R2 = oracle.rdms_spin_dep(6, ua, ub, c0)
    calc.add_repeated_pair_terms(R2, 6, ua, ub, C0, c0, inv)
    for k in R1:
        assert np.abs(R1[k] - R2[k]).max() < 1e-12, k


@pytest.mark.parametrize("key,value,match", [
    ("grow_factor", 1.0, "grow_factor must be > 1.0"),
    ("min_grow_factor", 1.0, "min_grow_factor must be > 1.0"),
    ("min_grow_factor", 9.0, "min_grow_factor must be <= grow_factor"),
    ("growth_backoff_rate", 1.0, "growth_backoff_rate must be in"),
    ("growth_backoff_rate", 0.0, "growth_backoff_rate must be in"),
    ("growth_recovery_rate", 1.0, "growth_recovery_rate must be > 1.0"),
])
def test_asci_growth_settings_are_checked(pkg, key, value, match):
    """get_asci_settings_ (macis_base.cpp:101-124; test_macis.cpp:1460-1473
    for grow_factor = 1): invalid growth settings raise before any device
    work."""
    calc = pkg.calculators
    c = calc.create("multi_configuration_calculator", "gb300_asci")
    c.settings().set(key, value)
    H = calc.Hamiltonian(np.eye(6), np.zeros(6 ** 4))
    with pytest.raises(RuntimeError, match=match):
        c.run(H, 3, 3)


def test_asci_core_threshold_is_checked(pkg):
    calc = pkg.calculators
    c = calc.create("multi_configuration_calculator", "gb300_asci")
    c.settings().set("core_selection_threshold", 0.0)
    H = calc.Hamiltonian(np.eye(6), np.zeros(6 ** 4))
    with pytest.raises(ValueError, match="core_selection_threshold"):
        c.run(H, 3, 3)
    c2 = calc.create("multi_configuration_calculator", "gb300_asci")
    c2.settings().set("core_selection_threshold", 0.0)
    c2.settings().set("core_selection_strategy", "fixed")
    c2.settings().set("grow_factor", 1.0)  # reaches the growth check: the threshold is not read
    with pytest.raises(RuntimeError, match="grow_factor"):
        c2.run(H, 3, 3)


def test_wavefunction_entropies_from_rdms(pkg, oracle, n2_6e6o):
    """WavefunctionContainer entropy semantics (wavefunction.cpp:556-685):
    with only spin-dependent RDMs, single-orbital entropies come from
    gamma_aa(ii), gamma_bb(ii) and the aabb (ii|ii) element
    (orbital_entropy.hpp:24-37) and equal form_entropies' (the oracle's
    restatement); two-orbital entropies and mutual information follow from
    each other with s1 (off the diagonal; zero on it)."""
    calc, det = pkg.calculators, pkg.determinants
    a, b = det.spin_sort(*det.fci_space(6, 3, 3))
    H = oracle.Hamiltonian(n2_6e6o["T"], n2_6e6o["V"])
    _, X, _ = oracle.build_csr(H, a, b).selected_ci_diag(tol=1e-10)
    s1o, s2o, mio = oracle.entropies(6, a, b, X)
    R = oracle.rdms_spin_dep(6, a, b, X)
    off = ~np.eye(6, dtype=bool)
    w = calc.Wavefunction(6, a, b, X, R)
    assert w.has_single_orbital_entropies()
    assert not w.has_two_orbital_entropies() and not w.has_mutual_information()
    np.testing.assert_allclose(w.get_single_orbital_entropies(), s1o, atol=1e-12, rtol=0)
    with pytest.raises(RuntimeError, match="Two-orbital entropies are not available"):
        w.get_two_orbital_entropies()
    with pytest.raises(RuntimeError, match="Mutual information is not available"):
        w.get_mutual_information()
    w2 = calc.Wavefunction(6, a, b, X, R, {"mi": mio})
    assert w2.has_two_orbital_entropies()
    s2 = w2.get_two_orbital_entropies()
    np.testing.assert_allclose(s2[off], s2o[off], atol=1e-12, rtol=0)
    assert not np.any(np.diag(s2))
    w3 = calc.Wavefunction(6, a, b, X, {k: R[k] for k in ("aa", "bb")}, {"s2": s2o})
    assert not w3.has_single_orbital_entropies() and not w3.has_mutual_information()
    with pytest.raises(RuntimeError, match="Spin-dependent one- and two-body RDMs"):
        w3.get_single_orbital_entropies()
    w4 = calc.Wavefunction(6, a, b, X, None, {"s1": s1o, "s2": s2o})
    np.testing.assert_allclose(w4.get_mutual_information()[off], mio[off], atol=1e-12, rtol=0)
    # a selected space over 12 orbitals with a random vector
    T, V, _ = pkg.integrals.synthetic_integrals(12, 16, 2)
    rng = np.random.default_rng(1)
    sa, sb = det.fci_space(12, 3, 2)
    keep = np.sort(rng.choice(len(sa), 400, replace=False))
    sa, sb = det.spin_sort(sa[keep], sb[keep])
    C = rng.standard_normal(len(sa))
    C /= np.linalg.norm(C)
    s1r, _, _ = oracle.entropies(12, sa, sb, C)
    wr = calc.Wavefunction(12, sa, sb, C, oracle.rdms_spin_dep(12, sa, sb, C))
    np.testing.assert_allclose(wr.get_single_orbital_entropies(), s1r, atol=1e-12, rtol=0)


def test_asci_grow_phase_settings(pkg, monkeypatch):
    """The grow-phase settings of MacisAsciSettings (macis_asci.hpp:93-182,
    determinant_search.hpp:136-198): defaults; H-build variants accepted (the
    same matrix), unknown ones refused; taper_grow_factor, just_singles,
    grow_with_rot and rot_size_start passed to the device driver, the grow's
    orbital rotation recorded on the wavefunction; grow_ci_residual_tolerance runs
    asci_grow at its tolerance and asci_refine at the main one (grow.hpp:73-78),
    checked with a recording stand-in for the device calls."""
    calc = pkg.calculators
    c = calc.create("multi_configuration_calculator", "gb300_asci")
    s = c.settings()
    assert (s.get("grow_ci_residual_tolerance"), s.get("taper_grow_factor"), s.get("just_singles"),
            s.get("grow_with_rot"), s.get("rot_size_start"), s.get("hamiltonian_build_algorithm"),
            s.get("dynamic_bit_masking_num_masks"), s.get("min_patch_overlap")) == (0.0, 0.0, False, False, 1000,
                                                                                    "", 0, 0.3)
    H = calc.Hamiltonian(np.eye(8), np.zeros(8 ** 4))

    def run(**kv):
        x = calc.create("multi_configuration_calculator", "gb300_asci")
        x.settings().set("ntdets_max", 100)
        for k, v in kv.items():
            x.settings().set(k, v)
        return x.run(H, 4, 4)

    with pytest.raises(ValueError, match="hamiltonian_build_algorithm"):
        run(hamiltonian_build_algorithm="magic")

    calls, seen = [], []

    class FakeContext:
        def __init__(self, device):
            pass

        def __enter__(self):
            return self

        def __exit__(self, *a):
            return False

        def set_integrals(self, T, V):
            pass

        def set_dets(self, a, b):
            pass

        def build_hamiltonian(self, thresh):
            pass

        def diagonal(self):
            return np.array([-1.0])

    def fake_asci(ctx, a0, b0, c0, E0, grow, refine, tol, **kw):
        calls.append((grow, refine, tol, E0))
        seen.append((kw["taper_grow_factor"], kw["just_singles"]))
        rots.append((kw["grow_with_rot"], kw["rot_size_start"]))
        return E0 - 0.5, np.array([15], np.uint64), np.array([15], np.uint64), np.ones(1), E0 - 0.25

    rots = []
    U = np.linalg.qr(np.random.default_rng(1).normal(size=(8, 8)))[0]
    monkeypatch.setattr(calc.capi, "Context", FakeContext)
    monkeypatch.setattr(calc.capi, "asci", fake_asci)
    monkeypatch.setattr(calc.capi, "asci_rotation", lambda ctx: U)
    _, w = run(grow_with_rot=True, rot_size_start=50)
    assert rots == [(1, 50)] and np.array_equal(w.info["orbital_rotation"], U)
    calls.clear()
    E, _ = run(hamiltonian_build_algorithm="residue_arrays", min_patch_overlap=0.9)
    assert calls == [(True, True, 1e-6, -1.0)] and E == -1.5
    calls.clear()
    run(grow_ci_residual_tolerance=1e-4)
    assert calls == [(True, False, 1e-4, -1.0), (False, True, 1e-6, -1.5)]
    calls.clear()
    run(grow_ci_residual_tolerance=1e-4, max_refine_iter=0)
    assert calls == [(True, False, 1e-4, -1.0)]
    seen.clear()
    run(taper_grow_factor=1.5)
    assert seen == [(1.5, 0)]
    seen.clear()
    run(just_singles=True)
    assert seen == [(0.0, 1)]


def test_wavefunction_accessors(pkg, oracle, n2_6e6o):
    """StateVectorContainer accessors (state_vector.cpp:171-330, 785-880):
    coefficients by determinant (0 when absent), determinant strings, RDM
    presence flags, and active occupations (a single determinant's own; else
    the descending eigenvalues of the spin-resolved 1-RDMs)."""
    calc, det = pkg.calculators, pkg.determinants
    a, b = det.spin_sort(*det.fci_space(6, 3, 3))
    H = oracle.Hamiltonian(n2_6e6o["T"], n2_6e6o["V"])
    _, X, _ = oracle.build_csr(H, a, b).selected_ci_diag(tol=1e-10)
    R = oracle.rdms_spin_dep(6, a, b, X, want=("aa", "bb"))
    w = calc.Wavefunction(6, a, b, X, R)
    assert w.get_coefficients() is w.coefficients
    assert w.get_active_determinants() == w.get_configurations()
    s0 = w.get_active_determinants()[7]
    assert w.get_coefficient(s0) == X[7] and w.get_coefficient((a[7], b[7])) == X[7]
    assert w.get_coefficient("000222") == X[np.flatnonzero((a == 0b111000) & (b == 0b111000))[0]]
    assert calc.Wavefunction(6, a[:5], b[:5], X[:5]).get_coefficient("000222") == 0.0
    assert w.has_one_rdm_spin_dependent() and w.has_one_rdm_spin_traced() and w.has_active_one_rdm()
    assert not w.has_two_rdm_spin_dependent() and not w.has_two_rdm_spin_traced() and not w.has_active_two_rdm()
    na, nb = w.get_active_orbital_occupations()
    assert np.all(np.diff(na) <= 1e-15) and abs(na.sum() - 3) < 1e-10 and abs(nb.sum() - 3) < 1e-10
    np.testing.assert_allclose(na, np.sort(np.linalg.eigvalsh(R["aa"]))[::-1], atol=1e-14)
    one = calc.Wavefunction(6, np.array([0b001011], np.uint64), np.array([0b000111], np.uint64), np.ones(1))
    oa, ob = one.get_active_orbital_occupations()
    assert oa.tolist() == [1, 1, 0, 1, 0, 0] and ob.tolist() == [1, 1, 1, 0, 0, 0]
    with pytest.raises(RuntimeError, match="1RDM must be available"):
        calc.Wavefunction(6, a, b, X).get_active_orbital_occupations()


def test_pmc_repeated_flow_on_oracle_device(pkg, oracle, n2_6e6o, monkeypatch):
    """Gb300Pmc on lists that repeat determinants, with the oracle answering
    the device calls: the checks of the GPU test (energy and vector = the
    lowest eigenpair of MACIS's matrix for the list as given, RDMs = the
    oracle's form_rdms over the list, one determinant twice = 2 <D|H|D>) hold
    for the host orchestration itself."""
    import scipy.sparse as sp
    from conftest import OracleDevice
    calc, det = pkg.calculators, pkg.determinants
    monkeypatch.setattr(calc.capi, "Context", OracleDevice)
    a, b = det.fci_space(6, 3, 3)
    rng = np.random.default_rng(11)
    sel = rng.choice(len(a), 20, replace=False)
    lst = np.concatenate([sel, sel[[2, 5, 5]]])
    rng.shuffle(lst)
    cfgs = [det.to_canonical_string(a[i], b[i], 6) for i in lst]
    ham = calc.Hamiltonian(n2_6e6o["T"], n2_6e6o["V"], n2_6e6o["E_core"])
    H = oracle.Hamiltonian(n2_6e6o["T"], n2_6e6o["V"])

    def dense(la, lb):
        rp, ci, nz = oracle.build_csr(H, la, lb).arrays()
        return sp.csr_matrix((nz, ci, rp), shape=(len(la),) * 2).toarray()

    p = calc.create("projected_multi_configuration_calculator")
    p.settings().set("calculate_one_rdm", True)
    p.settings().set("calculate_two_rdm", True)
    p.settings().set("calculate_single_orbital_entropies", True)
    E, wfn = p.run(ham, cfgs)
    w, X = np.linalg.eigh(dense(a[lst], b[lst]))
    assert wfn.size() == len(cfgs) and wfn.get_configurations() == cfgs
    assert abs(E - (w[0] + n2_6e6o["E_core"])) < 1e-10
    assert abs(abs(wfn.coefficients @ X[:, 0]) - 1.0) < 1e-8
    Ro = oracle.rdms_spin_dep(6, a[lst], b[lst], wfn.coefficients)
    aa, bb = wfn.get_active_one_rdm_spin_dependent()
    aabb, aaaa, bbbb = wfn.get_active_two_rdm_spin_dependent()
    np.testing.assert_allclose(aa, Ro["aa"], atol=1e-10, rtol=0)
    np.testing.assert_allclose(bb, Ro["bb"], atol=1e-10, rtol=0)
    for got, key in ((aabb, "aabb"), (aaaa, "aaaa"), (bbbb, "bbbb")):
        np.testing.assert_allclose(got, 2.0 * Ro[key].ravel(order="F"), atol=1e-10, rtol=0)
    assert wfn.has_single_orbital_entropies() and len(wfn.get_single_orbital_entropies()) == 6
    E2, w2 = calc.create("projected_multi_configuration_calculator").run(ham, ["222000", "222000"])
    hf = H.matrix_element((7, 7), (7, 7))
    assert abs(E2 - (2 * hf + n2_6e6o["E_core"])) < 1e-10 and w2.size() == 2
    three = ["222000", "22ud00", "222000"]
    E3, w3 = calc.create("projected_multi_configuration_calculator").run(ham, three)
    a3 = np.array([det.from_canonical_string(s)[0] for s in three], np.uint64)
    b3 = np.array([det.from_canonical_string(s)[1] for s in three], np.uint64)
    assert w3.size() == 3 and abs(E3 - (np.linalg.eigvalsh(dense(a3, b3))[0] + n2_6e6o["E_core"])) < 1e-10


def test_list_constrained_settings(pkg):
    """ListConstraint settings (macis_asci.hpp:141-145 for
    core_selection_strategy) refuse other values when set."""
    s = pkg.calculators.create("multi_configuration_calculator", "gb300_asci").settings()
    with pytest.raises(ValueError, match="not one of"):
        s.set("core_selection_strategy", "bogus")
    with pytest.raises(ValueError, match="not one of"):
        s.set("precision", "fp16")
    s.set("core_selection_strategy", "fixed")
    s.set("precision", "mixed")
    assert (s.get("core_selection_strategy"), s.get("precision")) == ("fixed", "mixed")


def test_register_custom_algorithm(pkg, monkeypatch):
    """registry.register (registry.py:496-538): type and name from the
    instance; a taken name raises DuplicateRegistrationError; an unknown type
    raises KeyError."""
    calc = pkg.calculators
    monkeypatch.setattr(calc, "_REGISTRY", {k: dict(v) for k, v in calc._REGISTRY.items()})

    class MyCas(calc.Gb300Cas):
        def name(self):
            return "my_cas"

    calc.register(lambda: MyCas())
    assert "my_cas" in calc.available("multi_configuration_calculator")
    assert isinstance(calc.create("multi_configuration_calculator", "my_cas"), MyCas)
    with pytest.raises(calc.DuplicateRegistrationError):
        calc.register(lambda: MyCas())
    with pytest.raises(calc.DuplicateRegistrationError):
        calc.register(lambda: calc.Gb300Pmc())

    class Odd(calc.Gb300Cas):
        def type_name(self):
            return "no_such_type"

    with pytest.raises(KeyError):
        calc.register(lambda: Odd())


def test_create_with_settings_show_default_unregister(pkg, monkeypatch):
    """registry.create(type, name, **settings), show_default and unregister
    (registry.py:295-372, 593-663)."""
    calc = pkg.calculators
    monkeypatch.setattr(calc, "_REGISTRY", {k: dict(v) for k, v in calc._REGISTRY.items()})
    c = calc.create("multi_configuration_calculator", "gb300_cas", ci_residual_tolerance=1e-9, calculate_one_rdm=True)
    assert c.settings().get("ci_residual_tolerance") == 1e-9 and c.settings().get("calculate_one_rdm") is True
    with pytest.raises(KeyError):
        calc.create("multi_configuration_calculator", "gb300_cas", no_such_setting=1)
    assert calc.show_default() == {"multi_configuration_calculator": "gb300_cas",
                                   "projected_multi_configuration_calculator": "gb300_pmc",
                                   "active_space_selector": "gb300_autocas_eos"}
    assert calc.show_default("active_space_selector") == "gb300_autocas_eos" and calc.show_default("nope") == ""
    calc.unregister("multi_configuration_calculator", "gb300_asci")
    assert calc.available("multi_configuration_calculator") == ["gb300_cas"]
    with pytest.raises(KeyError):
        calc.unregister("multi_configuration_calculator", "gb300_asci")


def test_settings_update_and_inspect(pkg):
    """Settings.update and registry.inspect_settings (registry.py:428-494)."""
    calc = pkg.calculators
    s = calc.create("multi_configuration_calculator", "gb300_asci").settings()
    s.update({"ntdets_max": 500}, grow_factor=4.0)
    assert s.get("ntdets_max") == 500 and s.get("grow_factor") == 4.0
    with pytest.raises(ValueError):
        s.update(grow_factor=0.5)
    rows = {r[0]: r for r in calc.inspect_settings("multi_configuration_calculator", "gb300_asci")}
    assert rows["ntdets_max"][1:3] == ("int", 100000) and rows["ntdets_max"][3] == "Maximum number of determinants"
    assert rows["core_selection_strategy"][4] == ["percentage", "fixed"]
    assert rows["just_singles"][3] is None and rows["just_singles"][4] is None
