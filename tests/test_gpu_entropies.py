"""Orbital entropies and mutual information on the GPU (qdkgb_orbital_entropies,
form_entropies sorted_double_loop.hpp:755-903) against the CPU oracle, whose
restatement is pinned to the partial-trace definition in
test_oracle_entropies.py: a CASCI vector, a random vector on a selected space
of 40 orbitals (the global-accumulation path), the calculator flags
(calculate_single_orbital_entropies, calculate_two_orbital_entropies,
calculate_mutual_information) and a single determinant (no entropy)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def capi(pkg):
    pkg.build.build()
    return pkg.capi


def test_entropies_casci_vector(capi, oracle, pkg, n2_6e6o):
    a, b = pkg.determinants.spin_sort(*pkg.determinants.fci_space(6, 3, 3))
    H = oracle.Hamiltonian(n2_6e6o["T"], n2_6e6o["V"])
    _, X, _ = oracle.build_csr(H, a, b).selected_ci_diag(tol=1e-10)
    o1, o2, om = oracle.entropies(6, a, b, X)
    with capi.Context(0) as ctx:
        ctx.set_integrals(n2_6e6o["T"], n2_6e6o["V"])
        ctx.set_dets(a, b)
        s1, s2, mi = ctx.orbital_entropies(X)
        t1, t2, tm = ctx.orbital_entropies(X, two_orbital=False, mutual_information=False)
        ctx.set_dets(a[:1], b[:1])
        z1, z2, zm = ctx.orbital_entropies(np.ones(1))
    np.testing.assert_allclose(s1, o1, atol=1e-12, rtol=0)
    np.testing.assert_allclose(s2, o2, atol=1e-12, rtol=0)
    np.testing.assert_allclose(mi, om, atol=1e-12, rtol=0)
    assert t2 is None and tm is None and np.abs(t1 - s1).max() < 1e-14
    assert not np.any(z1) and not np.any(z2) and not np.any(zm)


def test_entropies_selected_space_40_orbitals(capi, oracle, pkg):
    n = 40
    T, V, _ = pkg.integrals.synthetic_integrals(n, 2 * n, 11)
    rng = np.random.default_rng(3)
    strings = pkg.determinants.combs(n, 2)
    a = rng.choice(strings, size=80, replace=False)
    b = rng.choice(strings, size=60, replace=False)
    A, B = np.meshgrid(a, b, indexing="ij")
    keep = rng.random(A.size) < 0.5
    A, B = pkg.determinants.spin_sort(A.ravel()[keep].astype(np.uint64), B.ravel()[keep].astype(np.uint64))
    C = rng.standard_normal(len(A))
    C /= np.linalg.norm(C)
    o1, o2, om = oracle.entropies(n, A, B, C)
    with capi.Context(0) as ctx:
        ctx.set_integrals(T, V)
        ctx.set_dets(A, B)
        s1, s2, mi = ctx.orbital_entropies(C)
    np.testing.assert_allclose(s1, o1, atol=1e-12, rtol=0)
    np.testing.assert_allclose(s2, o2, atol=1e-12, rtol=0)
    np.testing.assert_allclose(mi, om, atol=1e-12, rtol=0)


def test_calculator_entropy_flags(pkg, oracle, n2_6e6o):
    calc = pkg.calculators
    c = calc.create("multi_configuration_calculator", "gb300_cas")
    for k in ("calculate_single_orbital_entropies", "calculate_two_orbital_entropies",
              "calculate_mutual_information"):
        c.settings().set(k, True)
    c.settings().set("ci_residual_tolerance", 1e-10)
    ham = calc.Hamiltonian(n2_6e6o["T"], n2_6e6o["V"], n2_6e6o["E_core"])
    _, wfn = c.run(ham, 3, 3)
    o1, o2, om = oracle.entropies(6, wfn.alpha, wfn.beta, wfn.coefficients)
    np.testing.assert_allclose(wfn.get_single_orbital_entropies(), o1, atol=1e-10, rtol=0)
    np.testing.assert_allclose(wfn.get_two_orbital_entropies(), o2, atol=1e-10, rtol=0)
    np.testing.assert_allclose(wfn.get_mutual_information(), om, atol=1e-10, rtol=0)
    c2 = calc.create("multi_configuration_calculator", "gb300_cas")
    _, w2 = c2.run(ham, 3, 3)
    assert not w2.has_single_orbital_entropies()
    with pytest.raises(RuntimeError):
        w2.get_mutual_information()


def test_orbitals_beyond_norb_are_refused(capi, n2_6e6o):
    """a determinant that occupies an orbital >= norb is refused before any
    kernel indexes the integrals or the RDM / entropy arrays with it"""
    with capi.Context(0) as ctx:
        ctx.set_integrals(n2_6e6o["T"], n2_6e6o["V"])
        a = np.array([0b0000111, 0b1000011], dtype=np.uint64)  # orbital 6 of a 6-orbital space
        b = np.array([0b0000111, 0b0000111], dtype=np.uint64)
        ctx.set_dets(a, b)
        with pytest.raises(capi.QdkgbError, match="beyond"):
            ctx.orbital_entropies(np.array([0.6, 0.8]))
        with pytest.raises(capi.QdkgbError, match="beyond"):
            ctx.build_hamiltonian()
        with pytest.raises(capi.QdkgbError, match="beyond"):
            capi.asci_pt2(ctx, a, b, np.array([0.6, 0.8]), -1.0)
