"""The qdk-style surface on the GPU: gb300_cas, davidson_solver, and the
differentiable energy (RDM gradients vs central finite differences)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built(pkg):
    pkg.build.build()


def test_gb300_cas_n2_golden_and_rdms(pkg, oracle, n2_6e6o, known):
    calc = pkg.calculators.create("multi_configuration_calculator", "gb300_cas")
    s = calc.settings()
    s.set("ci_residual_tolerance", 1e-8)
    s.set("calculate_one_rdm", True)
    s.set("calculate_two_rdm", True)
    H = pkg.calculators.Hamiltonian(n2_6e6o["T"], n2_6e6o["V"], n2_6e6o["E_core"])
    E, wfn = calc.run(H, 3, 3)
    assert np.isclose(E - n2_6e6o["E_core"], known["n2_6e6o_casci"]["E_total"])
    assert wfn.size() == 400
    # RDMs against the oracle on the returned vector; energy identity
    R = oracle.rdms_spin_dep(6, wfn.alpha, wfn.beta, wfn.coefficients)
    aa, bb = wfn.get_active_one_rdm_spin_dependent()
    assert np.allclose(aa, R["aa"], atol=1e-12) and np.allclose(bb, R["bb"], atol=1e-12)
    aabb, aaaa, bbbb = wfn.get_active_two_rdm_spin_dependent()
    assert np.allclose(aabb, 2 * R["aabb"].ravel(order="F"), atol=1e-12)
    G = wfn.get_active_two_rdm_spin_traced()
    E_rdm = np.sum(n2_6e6o["T"] * (aa + bb)) + np.sum(n2_6e6o["V"] * G) + n2_6e6o["E_core"]
    assert abs(E_rdm - E) < 1e-9
    with pytest.raises(pkg.calculators.SettingsAreLocked):
        s.set("ci_residual_tolerance", 1e-6)


def test_gb300_cas_mixed_precision_matches_fp64(pkg):
    T, V, _ = pkg.integrals.synthetic_integrals(10, 20, seed=21)
    H = pkg.calculators.Hamiltonian(T, V, 0.5)
    out = {}
    for prec in ("fp64", "mixed"):
        calc = pkg.calculators.create("multi_configuration_calculator", "gb300_cas")
        calc.settings().set("ci_residual_tolerance", 1e-8)
        calc.settings().set("precision", prec)
        out[prec], _ = calc.run(H, 5, 5)
    assert abs(out["fp64"] - out["mixed"]) < 1e-8


def test_davidson_solver_on_scipy_csr(pkg, oracle, h2o, known):
    import scipy.sparse as sp
    d = pkg.determinants
    a, b = d.cisd_space(24, *d.canonical_hf(5, 5))  # the reference test's (unsorted) order
    M = oracle.build_csr(oracle.Hamiltonian(h2o["T"], h2o["V"]), a, b, 1e-16)
    rp, ci, nz = M.arrays()
    A = sp.csr_matrix((nz, ci, rp), shape=(len(a), len(a)))
    E, X = pkg.calculators.davidson_solver(A, tol=1e-8, max_m=15)
    ref = known["h2o_cisd_davidson"]
    assert abs(E + h2o["E_core"] - ref["E0_total"]) < ref["atol"]
    assert abs(np.linalg.norm(X) - 1) < 1e-12
    assert abs(X @ (A @ X) - E) < 1e-10


@pytest.mark.late
def test_davidson_solver_reference_cases(pkg):
    """python/tests/test_davidson_solver.py:17-71 on the GPU: davidson_solver
    with its defaults (tol 1e-8, max_m 20) on the 6 x 6 tridiagonal and the
    two-site Heisenberg model, to the reference's 1e-12."""
    from conftest import davidson_solver_cases
    for name, A, E_ref, v_ref in davidson_solver_cases():
        E, X = pkg.calculators.davidson_solver(A)
        assert abs(E - E_ref) < 1e-12 + 1e-12 * abs(E_ref), name
        assert X.shape == v_ref.shape and abs(abs(X @ v_ref) - 1.0) < 1e-12, name


def test_autograd_rdm_gradients_match_finite_differences(pkg):
    """dE/dh1 = 1-RDM and dE/dV = 2-RDM against central differences (step 1e-5)
    on 20 seeded integral entries, each perturbed over its whole symmetry orbit."""
    import torch
    ag = pkg.autograd
    n, na, nb = 6, 3, 3
    T, V, _ = pkg.integrals.synthetic_integrals(n, 8, seed=4)
    E, gT, gV = ag.rdms_as_gradients(torch.from_numpy(T), torch.from_numpy(V), na, nb, tol=1e-10)
    gT, gV = gT.numpy(), gV.numpy()
    rng = np.random.default_rng(11)
    h = 1e-5

    def energy(Tp, Vp):
        return float(ag.casci_energy(torch.from_numpy(Tp), torch.from_numpy(Vp), na, nb, tol=1e-10))

    for trial in range(20):
        if trial % 4 == 0:
            p, q = rng.integers(0, n, 2)
            orbit = {(p, q), (q, p)}
            dT = np.zeros_like(T)
            for (i, j) in orbit:
                dT[i, j] = 1.0
            fd = (energy(T + h * dT, V) - energy(T - h * dT, V)) / (2 * h)
            an = sum(gT[i, j] for (i, j) in orbit)
        else:
            p, q, r, s = rng.integers(0, n, 4)
            orbit = {(p, q, r, s), (q, p, r, s), (p, q, s, r), (q, p, s, r),
                     (r, s, p, q), (s, r, p, q), (r, s, q, p), (s, r, q, p)}
            dV = np.zeros_like(V)
            for idx in orbit:
                dV[idx] = 1.0
            fd = (energy(T, V + h * dV) - energy(T, V - h * dV)) / (2 * h)
            an = sum(gV[idx] for idx in orbit)
        assert abs(fd - an) < 1e-6, (trial, fd, an)


def test_gb300_asci_calculator_n2(pkg, n2_14e18o, known):
    """The qdk-style ASCI plugin with the pymacis test's settings."""
    ref = known["n2_14e18o_asci"]
    calc = pkg.calculators.create("multi_configuration_calculator", "gb300_asci")
    s = calc.settings()
    s.set("ci_residual_tolerance", 1e-8)
    s.set("ntdets_max", ref["ntdets_max"])
    s.set("grow_factor", float(ref["grow_factor"]))
    s.set("max_refine_iter", ref["max_refine_iter"])
    s.set("calculate_one_rdm", True)
    H = pkg.calculators.Hamiltonian(n2_14e18o["T"], n2_14e18o["V"], n2_14e18o["E_core"])
    E, wfn = calc.run(H, 7, 7)
    assert abs(E - n2_14e18o["E_core"] - ref["E_total"]) < 1e-8
    assert wfn.size() == ref["ndets"]
    aa, bb = wfn.get_active_one_rdm_spin_dependent()
    assert abs(np.trace(aa) - 7) < 1e-8 and abs(np.trace(bb) - 7) < 1e-8


def test_gb300_asci_falls_back_to_cas_for_small_spaces(pkg, n2_6e6o, known):
    calc = pkg.calculators.create("multi_configuration_calculator", "gb300_asci")
    calc.settings().set("ci_residual_tolerance", 1e-8)
    H = pkg.calculators.Hamiltonian(n2_6e6o["T"], n2_6e6o["V"], 0.0)
    E, wfn = calc.run(H, 3, 3)
    assert wfn.size() == 400 and np.isclose(E, known["n2_6e6o_casci"]["E_total"])
