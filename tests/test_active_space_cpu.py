"""The entropy-based active-space selectors that consume this library's
orbital entropies: autoCAS (autocas_active_space.cpp:15-160) and autoCAS-EOS
(entropy_active_space.cpp:14-87), with _sort_entropies_and_indices,
new_orbitals and new_wavefunction (active_space.cpp:46-376).  Host logic on
the CPU, on hand-worked entropy profiles; and on entropies derived from the
oracle's RDMs of an N2 CAS(6e,6o) vector."""
import numpy as np
import pytest


def _wfn(calc, s1, active, inactive, dets=2):
    """A wavefunction over `active` (3 + 3 electrons) carrying the given
    single-orbital entropies; `dets` determinants."""
    n = len(active)
    a = np.array([0b000111, 0b001011][:dets], np.uint64)
    b = np.array([0b000111, 0b000111][:dets], np.uint64)
    c = np.ones(dets) / np.sqrt(dets)
    return calc.Wavefunction(n, a, b, c, None, {"s1": np.asarray(s1, float)}, active_indices=active,
                             inactive_indices=inactive)


# raw entropies at orbitals 2 .. 9; normalised by 1.2 and sorted:
# 1, .917, .833, .792, .758, .167, .0167, .0083 (orbitals 2, 3, 4, 5, 9, 8, 6, 7),
# none on a bin edge
PROFILE = [1.2, 1.1, 1.0, 0.95, 0.02, 0.01, 0.2, 0.91]
ACTIVE = list(range(2, 10))


def test_registry_and_settings(pkg):
    calc = pkg.calculators
    assert calc.available("active_space_selector") == ["gb300_autocas", "gb300_autocas_eos"]
    assert calc.create("active_space_selector").name() == "gb300_autocas_eos"  # active_space.hpp:206
    sel = calc.create("active_space_selector", "gb300_autocas")
    assert sel.type_name() == "active_space_selector"
    s = sel.settings()
    assert (s.get("num_bins"), s.get("min_plateau_size"), s.get("entropy_threshold"),
            s.get("normalize_entropies")) == (100, 10, 0.14, True)
    with pytest.raises(ValueError):
        s.set("num_bins", 1)
    with pytest.raises(ValueError):
        s.set("min_plateau_size", 0)
    e = calc.create("active_space_selector", "gb300_autocas_eos").settings()
    assert (e.get("diff_threshold"), e.get("entropy_threshold"), e.get("normalize_entropies")) == (0.1, 0.14, True)


def test_autocas_plateaus(pkg):
    """Counts of orbitals above the 100 bins: 8 (bin 0), 7 (bin 1), 6 (bins
    2-16), 5 (bins 17-75), 4, 3, 2, 1 (4, 4, 8 and 8 bins).  With plateaus of
    at least 10 bins the larger count, 6, keeps orbitals 2, 3, 4, 5, 9, 8; with
    at least 20 only the 5-run (59 bins) is a plateau; with at least 60 none."""
    calc = pkg.calculators
    w = _wfn(calc, PROFILE, ACTIVE, [0, 1])
    out = calc.create("active_space_selector", "gb300_autocas").run(w)
    assert out.get_active_indices() == [2, 3, 4, 5, 8, 9]
    # aufbau 3 + 3 over orbitals 2 .. 9, truncated: orbitals 2, 3, 4 doubly occupied
    assert out.size() == 1 and int(out.alpha[0]) == 0b000111 and int(out.beta[0]) == 0b000111
    assert out.get_inactive_indices() == [0, 1]
    s = calc.create("active_space_selector", "gb300_autocas")
    s.settings().set("min_plateau_size", 20)
    assert s.select(w) == [2, 3, 4, 5, 9]
    s = calc.create("active_space_selector", "gb300_autocas")
    s.settings().set("min_plateau_size", 60)
    assert s.select(w) == []


def test_autocas_single_reference_and_raw_entropies(pkg):
    calc = pkg.calculators
    small = [0.1, 0.05, 0.02, 0.01, 0.0, 0.0, 0.0, 0.0]  # max 0.1 < 0.14
    out = calc.create("active_space_selector", "gb300_autocas").run(_wfn(calc, small, ACTIVE, [0, 1]))
    assert out.get_active_indices() == [] and out.norb == 0
    assert out.get_inactive_indices() == [0, 1, 2, 3, 4]
    # unnormalised: raw entropies above 1 count in every bin (no plateau change)
    s = calc.create("active_space_selector", "gb300_autocas")
    s.settings().set("normalize_entropies", False)
    raw = [1.5, 1.4, 0.305, 0.295, 0.0, 0.0, 0.0, 0.0]
    # counts: bins 0-29 -> 4, 30 -> 3, 31-99 -> 2: plateaus of 30 and 69 bins
    assert s.select(_wfn(calc, raw, ACTIVE, [])) == [2, 3, 4, 5]


def test_autocas_eos(pkg):
    """Drops above 0.1 after the 5th (.758 -> .167) and 6th (.167 -> .0167)
    sorted entropies, both above 0.14 / 1.2: the larger size, 6, is kept."""
    calc = pkg.calculators
    w = _wfn(calc, PROFILE, ACTIVE, [0, 1], dets=1)
    out = calc.create("active_space_selector", "gb300_autocas_eos").run(w)
    assert out.get_active_indices() == [2, 3, 4, 5, 8, 9]
    # one determinant: its own occupations (0b001011 alpha at positions 0, 1, 3)
    w1 = calc.Wavefunction(8, np.array([0b001011], np.uint64), np.array([0b000111], np.uint64), np.ones(1),
                           None, {"s1": np.asarray(PROFILE)}, active_indices=ACTIVE, inactive_indices=[0, 1])
    o1 = calc.create("active_space_selector", "gb300_autocas_eos").run(w1)
    assert int(o1.alpha[0]) == 0b001011 and int(o1.beta[0]) == 0b000111
    e = calc.create("active_space_selector", "gb300_autocas_eos")
    e.settings().set("diff_threshold", 0.35)
    assert e.select(w) == [2, 3, 4, 5, 9]  # only the .59 drop
    e = calc.create("active_space_selector", "gb300_autocas_eos")
    e.settings().set("entropy_threshold", 0.6)  # .6 / 1.2 = .5: the .167 entry no longer counts
    assert e.select(w) == [2, 3, 4, 5, 9]


def test_errors(pkg):
    calc = pkg.calculators
    bare = calc.Wavefunction(8, np.array([7], np.uint64), np.array([7], np.uint64), np.ones(1))
    with pytest.raises(RuntimeError, match="does not have single orbital entropies"):
        calc.create("active_space_selector", "gb300_autocas").run(bare)
    with pytest.raises(RuntimeError, match="outside of initial active space"):
        calc.selected_active_wavefunction(_wfn(calc, PROFILE, ACTIVE, []), [1, 2])
    with pytest.raises(ValueError):
        calc.Wavefunction(8, np.array([7], np.uint64), np.array([7], np.uint64), np.ones(1), active_indices=[0])


def test_selection_from_rdm_entropies(pkg, oracle, n2_6e6o):
    """On an N2 CAS(6e,6o) vector whose entropies come from the oracle's RDMs
    (the derivation a wavefunction with RDMs uses), both selectors return a
    subset of the active orbitals that holds the highest-entropy ones."""
    calc, det = pkg.calculators, pkg.determinants
    a, b = det.spin_sort(*det.fci_space(6, 3, 3))
    H = oracle.Hamiltonian(n2_6e6o["T"], n2_6e6o["V"])
    _, X, _ = oracle.build_csr(H, a, b).selected_ci_diag(tol=1e-10)
    w = calc.Wavefunction(6, a, b, X, oracle.rdms_spin_dep(6, a, b, X), active_indices=range(4, 10),
                          inactive_indices=[0, 1, 2, 3])
    s1 = w.get_single_orbital_entropies()
    top = 4 + int(np.argmax(s1))
    for name in ("gb300_autocas", "gb300_autocas_eos"):
        sel = calc.create("active_space_selector", name).select(w)
        assert set(sel) <= set(range(4, 10))
        assert not sel or top in sel


def test_cas_then_autocas_flow(pkg, n2_6e6o, monkeypatch):
    """The flow of python/tests/test_active_space.py:38-80 (CASCI with 1- and
    2-RDMs, then each selector on the wavefunction) with the oracle answering
    the device calls: the entropies come from the RDMs, and both selectors
    return sorted subsets of the active orbitals as one-determinant
    wavefunctions."""
    from conftest import OracleDevice
    calc = pkg.calculators
    monkeypatch.setattr(calc.capi, "Context", OracleDevice)
    mc = calc.create("multi_configuration_calculator", "gb300_cas")
    mc.settings().set("calculate_one_rdm", True)
    mc.settings().set("calculate_two_rdm", True)
    ham = calc.Hamiltonian(n2_6e6o["T"], n2_6e6o["V"], n2_6e6o["E_core"])
    _, wfn = mc.run(ham, 3, 3)
    assert wfn.has_single_orbital_entropies() and "s1" not in wfn._ent
    for name in ("gb300_autocas", "gb300_autocas_eos"):
        out = calc.create("active_space_selector", name).run(wfn)
        idx = out.get_active_indices()
        assert idx == sorted(idx) and set(idx) <= set(range(6)) and out.size() == 1
        assert out.norb == len(idx)
