"""The drop-in calculators choose the operator by device memory
(qdkgb_build_operator): the stored Hamiltonian when it fits, else (complete
spaces) the direct sigma.  A capped context forces the switch at a small
shape; CASCI(14e,14o), whose stored matrix (3.98e10 elements) exceeds HBM,
runs through create("multi_configuration_calculator", "gb300_cas").run(H, 7, 7)
and through the differentiable energy, with the RDM gradients checked
against central finite differences (step 1e-5) of the energy on seeded
integral orbits: 20 entries at CASCI(12e,12o), 2 at CASCI(14e,14o)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built(pkg):
    pkg.build.build()


def test_capped_context_switches_to_the_direct_sigma(pkg):
    capi = pkg.capi
    T, V, _ = pkg.integrals.synthetic_integrals(8, 16, seed=77)
    a, b = capi.fci_dets(8, 4, 4)
    with capi.Context(0) as ctx:
        ctx.set_integrals(T, V)
        ctx.set_dets(a, b)
        assert ctx.build_operator(max_m=60) == "slab"
        E_stored, _, _ = ctx.davidson(tol=1e-9, max_m=60)
    with capi.Context(0) as ctx:
        ctx.set_integrals(T, V)
        ctx.set_dets(a, b)
        # room for the Davidson workspace (~5 MB) and the direct sigma's
        # tables, not for the stored matrix (1,768,900 values, 14 MB)
        ctx.set_device_limit(ctx.device_bytes() + 10 * (1 << 20))
        assert ctx.build_operator(max_m=60) == "direct"
        assert ctx.operator_layout()[0] == capi.LAYOUT_DIRECT
        E_direct, _, _ = ctx.davidson(tol=1e-9, max_m=60)
    assert abs(E_direct - E_stored) < 1e-10


def test_gb300_cas_uses_the_direct_sigma_under_a_memory_cap(pkg):
    T, V, _ = pkg.integrals.synthetic_integrals(8, 16, seed=78)
    H = pkg.calculators.Hamiltonian(T, V, 0.25)
    out = {}
    # 24 MiB: room for the Davidson workspace (200 vectors, 16 MB) and the
    # direct sigma, not for it and the stored matrix (14 MB) together
    for cap in (0, 24 << 20):
        calc = pkg.calculators.create("multi_configuration_calculator", "gb300_cas")
        calc.settings().set("device_memory_limit", cap)
        calc.settings().set("calculate_one_rdm", True)
        E, wfn = calc.run(H, 4, 4)
        out[cap] = (E, wfn)
    assert out[0][1].info["operator"] in ("slab", "slab+direct32") and out[24 << 20][1].info["operator"] == "direct"
    assert abs(out[0][0] - out[24 << 20][0]) < 1e-10
    g0 = sum(out[0][1].get_active_one_rdm_spin_dependent())
    g1 = sum(out[24 << 20][1].get_active_one_rdm_spin_dependent())
    assert np.max(np.abs(g0 - g1)) < 1e-7


def _orbit_fd_check(ag, T, V, na, nb, entries, seed, precision, tol=1e-9):
    import torch
    E, gT, gV = ag.rdms_as_gradients(torch.from_numpy(T), torch.from_numpy(V), na, nb, tol=tol, precision=precision)
    gT, gV = gT.numpy(), gV.numpy()
    n = T.shape[0]
    rng = np.random.default_rng(seed)
    h = 1e-5

    def energy(Tp, Vp):
        return float(ag.casci_energy(torch.from_numpy(Tp), torch.from_numpy(Vp), na, nb, tol=tol,
                                     precision=precision))

    for trial in range(entries):
        if trial % 4 == 0:
            p, q = rng.integers(0, n, 2)
            orbit = {(p, q), (q, p)}
            dT = np.zeros_like(T)
            for idx in orbit:
                dT[idx] = 1.0
            fd = (energy(T + h * dT, V) - energy(T - h * dT, V)) / (2 * h)
            an = sum(gT[idx] for idx in orbit)
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
    return E


@pytest.mark.late
def test_autograd_cas12_twenty_entries(pkg):
    T, V, _ = pkg.integrals.synthetic_integrals(12, 24, seed=20261203)
    _orbit_fd_check(pkg.autograd, T, V, 6, 6, 20, seed=12, precision="mixed")


@pytest.mark.late
def test_cas14_through_the_plugin_and_autograd(pkg):
    T, V, _ = pkg.integrals.synthetic_integrals(14, 28, seed=20261203)
    H = pkg.calculators.Hamiltonian(T, V, 0.0)
    calc = pkg.calculators.create("multi_configuration_calculator", "gb300_cas")
    calc.settings().set("calculate_one_rdm", True)
    calc.settings().set("calculate_two_rdm", True)
    calc.settings().set("precision", "mixed")
    E, wfn = calc.run(H, 7, 7)
    assert wfn.info["operator"] == "direct" and wfn.size() == 11778624
    aa, bb = wfn.get_active_one_rdm_spin_dependent()
    G = wfn.get_active_two_rdm_spin_traced()
    E_rdm = np.sum(T * (aa + bb)) + np.sum(V * G)
    assert abs(E_rdm - E) < 1e-8, (E_rdm, E)
    # the differentiable energy reaches the same space; its gradient (the RDMs)
    # against central differences on one one-body and one two-body orbit
    Eg = _orbit_fd_check(pkg.autograd, T, V, 7, 7, 2, seed=14, precision="mixed", tol=1e-8)
    assert abs(float(Eg) - E) < 1e-8
