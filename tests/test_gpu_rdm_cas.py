"""RDMs of complete (CAS) spaces: the spin-regrouped path (opposite-spin sweep
over alpha transitions, same-spin blocks from the string overlaps) against
the pair walk on the same vector (QDKGB_RDM_PAIR_WALK=1 keeps the pair walk)
and against the oracle's form_rdms_spin_dep, to 1e-12; the reference's
|C_I C_J| <= 1e-16 skip rule on a vector whose products straddle the bound;
and, at CASCI(14e,14o), the RDM energy identity and trace/symmetry rules on
the direct-sigma FP64 ground state."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def capi(pkg):
    pkg.build.build()
    return pkg.capi


@pytest.fixture(scope="module")
def ctx(capi):
    c = capi.Context(0)
    yield c
    c.close()


def _rdms(ctx, C, walk):
    old = os.environ.get("QDKGB_RDM_PAIR_WALK")
    os.environ["QDKGB_RDM_PAIR_WALK"] = "1" if walk else "0"
    try:
        return ctx.rdms_spin_dep(C)
    finally:
        if old is None:
            del os.environ["QDKGB_RDM_PAIR_WALK"]
        else:
            os.environ["QDKGB_RDM_PAIR_WALK"] = old


@pytest.mark.parametrize("norb,na,nb", [(8, 4, 4), (9, 5, 3), (7, 2, 5), (10, 5, 5), (6, 3, 0), (5, 5, 2)])
def test_cas_rdms_match_pair_walk_and_oracle(ctx, pkg, oracle, norb, na, nb):
    T, V, _ = pkg.integrals.synthetic_integrals(norb, 2 * norb, seed=40 + norb + na)
    a, b = pkg.determinants.fci_space(norb, na, nb)
    ctx.set_integrals(T, V)
    ctx.set_dets(a, b)
    C = np.random.default_rng(norb * 7 + nb).normal(size=len(a))
    C /= np.linalg.norm(C)
    R = _rdms(ctx, C, walk=False)
    W = _rdms(ctx, C, walk=True)
    Ro = oracle.rdms_spin_dep(norb, a, b, C)
    for k in ("aa", "bb", "aaaa", "bbbb", "aabb"):
        assert np.max(np.abs(R[k] - W[k])) < 1e-12, k
        assert np.max(np.abs(R[k] - Ro[k])) < 1e-12, k


def test_cas_rdms_skip_rule(ctx, pkg, oracle):
    # coefficients 10^U(-8.6, -7.4): most pair products lie within a decade
    # of 1e-16, so a wrong skip rule changes every block at O(1) relative
    norb, na, nb = 8, 4, 4
    T, V, _ = pkg.integrals.synthetic_integrals(norb, 16, seed=5)
    a, b = pkg.determinants.fci_space(norb, na, nb)
    ctx.set_integrals(T, V)
    ctx.set_dets(a, b)
    rng = np.random.default_rng(11)
    C = np.where(rng.random(len(a)) < 0.5, -1.0, 1.0) * 10 ** rng.uniform(-8.6, -7.4, len(a))
    R = _rdms(ctx, C, walk=False)
    Ro = oracle.rdms_spin_dep(norb, a, b, C)
    for k in ("aa", "bb", "aaaa", "bbbb", "aabb"):
        scale = np.max(np.abs(Ro[k]))
        assert scale > 0
        assert np.max(np.abs(R[k] - Ro[k])) <= 1e-10 * scale, k


@pytest.mark.late
def test_cas12_rdms_of_the_ground_state_match_oracle(ctx, pkg, oracle):
    from conftest import GOLDEN
    d = np.load(os.path.join(GOLDEN, "ref_cas12.npz"))
    T, V = d["T"], d["V"]
    a, b = pkg.determinants.fci_space(12, 6, 6)
    ctx.set_integrals(T, V)
    ctx.set_dets(a, b)
    ctx.build_hamiltonian()
    E, C, _ = ctx.davidson(tol=1e-8)
    R = ctx.rdms_spin_dep(C)
    Ro = oracle.rdms_spin_dep(12, a, b, C)
    for k in ("aa", "bb", "aaaa", "bbbb", "aabb"):
        assert np.max(np.abs(R[k] - Ro[k])) < 1e-12, k
    E_rdm = np.sum(T * (R["aa"] + R["bb"])) + np.sum(V * (R["aaaa"] + R["bbbb"])) + 2 * np.sum(V * R["aabb"])
    assert abs(E_rdm - E) < 1e-10


@pytest.mark.late
def test_cas14_rdm_energy_identity(ctx, pkg):
    T, V, _ = pkg.integrals.synthetic_integrals(14, 28, seed=20261203)
    a, b = pkg.determinants.fci_space(14, 7, 7)
    ctx.set_integrals(T, V)
    ctx.set_dets(a, b)
    ctx.build_direct_sigma()
    E, C, _ = ctx.davidson(tol=1e-8)
    R = ctx.rdms_spin_dep(C)
    E_rdm = np.sum(T * (R["aa"] + R["bb"])) + np.sum(V * (R["aaaa"] + R["bbbb"])) + 2 * np.sum(V * R["aabb"])
    assert abs(E_rdm - E) < 1e-10, (E_rdm, E)
    assert abs(np.trace(R["aa"]) - 7) < 1e-10 and abs(np.trace(R["bb"]) - 7) < 1e-10
    # sum_ik G_aabb[i, i, k, k] = 1/2 n_a n_b, and G_aabb[i, j, k, l] = G_aabb[j, i, l, k]
    assert abs(np.einsum("iikk->", R["aabb"]) - 0.5 * 49) < 1e-9
    assert np.max(np.abs(R["aabb"] - R["aabb"].transpose(1, 0, 3, 2))) < 1e-12
    assert np.max(np.abs(R["aa"] - R["aa"].T)) < 1e-12


def test_spin_traced_rdms_match_reference_form_rdms(ctx, capi):
    """qdkgb_rdms against the reference's own form_rdms (tests/golden/
    ref_cas8.npz, the reference's CI vector), to 1e-12; it accumulates."""
    from conftest import GOLDEN
    d = np.load(os.path.join(GOLDEN, "ref_cas8.npz"))
    a, b = capi.fci_dets(8, 4, 4)
    ctx.set_integrals(d["T"], d["V"])
    ctx.set_dets(a, b)
    o1, o2 = ctx.rdms(d["C"])
    assert np.max(np.abs(o1 - d["rdm_traced1"])) < 1e-12
    assert np.max(np.abs(o2 - d["rdm_traced2"])) < 1e-12


def test_operator_action_block_contract(ctx, capi, pkg, oracle):
    """qdkgb_operator_action: AV = alpha H V + beta AV over a block of
    columns (davidson.hpp:79-90), beta = 0 ignoring AV's contents."""
    T, V, _ = pkg.integrals.synthetic_integrals(8, 16, seed=90)
    a, b = capi.fci_dets(8, 4, 4)
    ctx.set_integrals(T, V)
    ctx.set_dets(a, b)
    ctx.build_hamiltonian()
    M = oracle.build_csr(oracle.Hamiltonian(T, V), a, b)
    rng = np.random.default_rng(3)
    X = rng.normal(size=(len(a), 3))
    Y0 = rng.normal(size=(len(a), 3))
    Y = ctx.operator_action(X, alpha=2.0, AV=Y0, beta=0.5)
    ref = np.stack([2.0 * M.spmv(X[:, j]) + 0.5 * Y0[:, j] for j in range(3)], axis=1)
    assert np.max(np.abs(Y - ref)) < 1e-11 * np.max(np.abs(ref))
    Z = ctx.operator_action(X, AV=np.full((len(a), 3), np.nan), beta=0.0)
    assert np.all(np.isfinite(Z))
    assert np.max(np.abs(Z[:, 1] - M.spmv(X[:, 1]))) < 1e-11 * np.max(np.abs(Z))
