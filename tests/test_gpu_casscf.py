"""CASSCF (qdkgb_casscf, casscf_diis) on the GPU against the reference's
pinned value: water cc-pVDZ, 1 inactive + 8 active orbitals, 4 + 4 active
electrons, no starting RDMs: E = -76.1114493227 (external/macis/tests/
mcscf.cxx:26-66, tolerance 1e-8).  With every orbital active there is no
rotation and the result is the CASCI (N2 CAS(6e,6o), test_pymacis.py:114-142).
The oracle's CASSCF restatement (pinned on the CPU to the same value) takes the
same optimisation path: same energy, same macro-iteration count (within 2),
the same active 1-RDM."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def capi(pkg):
    pkg.build.build()
    return pkg.capi


def test_casscf_water_matches_reference(capi, oracle, h2o, known):
    ref = known["h2o_casscf"]
    with capi.Context(0) as ctx:
        E, g, G, U, iters, conv = capi.casscf(ctx, h2o["T"], h2o["V"], h2o["E_core"], ref["nalpha"], ref["nbeta"],
                                              ref["ninact"], ref["nact"])
    assert conv and iters > 0
    assert abs(E - ref["E_total"]) < ref["atol"], (E, ref["E_total"])
    # the oracle's restatement takes the same path: same energy and iteration count
    Eo, go, _, it_o, conv_o = oracle.casscf(h2o["T"], h2o["V"], h2o["E_core"], ref["nalpha"], ref["nbeta"],
                                            ref["ninact"], ref["nact"])
    assert conv_o and abs(E - Eo) < 1e-9 and abs(iters - it_o) <= 2
    np.testing.assert_allclose(g, go, atol=1e-6, rtol=0)
    assert abs(np.trace(g) - 8.0) < 1e-10
    assert np.allclose(U.T @ U, np.eye(U.shape[0]), atol=1e-12)
    # restarted in the optimised orbitals with the final RDMs: converged at
    # once (no macro iteration), the energy from those RDMs is the same
    n = U.shape[0]
    T2 = U.T @ h2o["T"] @ U
    V2 = np.einsum("abcd,ap,bq,cr,ds->pqrs", h2o["V"].reshape(n, n, n, n), U, U, U, U, optimize=True)
    with capi.Context(0) as ctx:
        E2, _, _, _, it2, conv2 = capi.casscf(ctx, T2, V2, h2o["E_core"], ref["nalpha"], ref["nbeta"], ref["ninact"],
                                              ref["nact"], rdm1=g, rdm2=G, orb_grad_tol=1e-3)
    assert conv2 and it2 == 0 and abs(E2 - E) < 1e-9


def test_casscf_all_active_is_casci(capi, n2_6e6o, known):
    ref = known["n2_6e6o_casci"]
    with capi.Context(0) as ctx:
        E, g, _, U, iters, conv = capi.casscf(ctx, n2_6e6o["T"], n2_6e6o["V"], n2_6e6o["E_core"], 3, 3, 0, 6)
    assert conv and iters == 0 and np.allclose(U, np.eye(6))
    assert abs(E - n2_6e6o["E_core"] - ref["E_total"]) < 1e-6  # the pinned value is electronic
    with capi.Context(0) as ctx, pytest.raises(capi.QdkgbError):
        capi.casscf(ctx, n2_6e6o["T"], n2_6e6o["V"], 0.0, 3, 3, 2, 6)  # 2 + 6 > 6 orbitals
