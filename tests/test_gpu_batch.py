"""Batched CASCI (qdkgb_casci_batch) against the CPU oracle: per-instance
energies (mixed form within 1e-8 Eh of the oracle's FP64 Davidson, FP64 form
within 1e-10) and spin-summed 1-RDMs (1e-6 absolute: the vectors agree to the
residual tolerance over the gap), for instances of uneven size and shape."""
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


def _instances(pkg, shapes, seed0):
    out = []
    for i, (norb, na, nb) in enumerate(shapes):
        T, V, _ = pkg.integrals.synthetic_integrals(norb, 2 * norb, seed0 + i)
        out.append((norb, na, nb, T, V))
    return out


def _oracle_ref(oracle, pkg, inst):
    norb, na, nb, T, V = inst
    a, b = pkg.determinants.fci_space(norb, na, nb)
    M = oracle.build_csr(oracle.Hamiltonian(T, V), a, b)
    E, X, _ = M.selected_ci_diag(tol=1e-10)
    R = oracle.rdms_spin_dep(norb, a, b, X)
    return E, R["aa"] + R["bb"]


SHAPES = [(6, 3, 3), (4, 2, 2), (8, 4, 4), (6, 3, 3), (6, 3, 2), (8, 4, 4), (4, 2, 2), (6, 3, 3)]


def test_batch_mixed_matches_oracle(ctx, oracle, pkg, capi):
    inst = _instances(pkg, SHAPES, 100)
    E, R, its, info = capi.casci_batch(ctx, inst, res_tol=1e-8)
    assert info["graph_replays"] > 0
    for i, q in enumerate(inst):
        Eo, Ro = _oracle_ref(oracle, pkg, q)
        assert abs(E[i] - Eo) < 1e-8, (i, E[i], Eo)
        np.testing.assert_allclose(R[i], Ro, atol=1e-6, rtol=0, err_msg=str(i))
        assert abs(np.trace(R[i]) - (q[1] + q[2])) < 1e-10
        assert its[i] > 0


def test_batch_fp64_matches_oracle(ctx, oracle, pkg, capi):
    inst = _instances(pkg, SHAPES[:5], 200)
    E, R, its, info = capi.casci_batch(ctx, inst, res_tol=1e-9, precision=capi.PREC_FP64)
    for i, q in enumerate(inst):
        Eo, Ro = _oracle_ref(oracle, pkg, q)
        assert abs(E[i] - Eo) < 1e-10, (i, E[i], Eo)
        np.testing.assert_allclose(R[i], Ro, atol=1e-6, rtol=0)


def test_batch_graph_replay_is_identical_and_order_independent(ctx, pkg, capi):
    inst = _instances(pkg, SHAPES, 300)
    E1, _, it1, i1 = capi.casci_batch(ctx, inst, want_rdm1=False, use_graph=1)
    E2, _, it2, i2 = capi.casci_batch(ctx, inst, want_rdm1=False, use_graph=0)
    assert i1["graph_replays"] > 0 and i2["graph_replays"] == 0
    assert np.array_equal(E1, E2) and np.array_equal(it1, it2)
    # one instance alone gives the same energy as inside the batch
    for j in (0, 2, 4):
        Ej, _, _, _ = capi.casci_batch(ctx, [inst[j]], want_rdm1=False)
        assert abs(Ej[0] - E1[j]) < 1e-9
    # sub-batches (a tiny memory bound) change nothing but the grouping
    E3, _, _, _ = capi.casci_batch(ctx, inst, want_rdm1=False, max_slab_bytes=1)
    assert np.max(np.abs(E3 - E1)) < 1e-9


def test_batch_single_instance_path_agrees(ctx, pkg, capi):
    inst = _instances(pkg, [(8, 4, 4)], 400)
    E, _, _, _ = capi.casci_batch(ctx, inst, want_rdm1=False, res_tol=1e-9)
    c2 = capi.Context(0)
    try:
        Es, _, _ = c2.casci(inst[0][3], inst[0][4], 4, 4, tol=1e-9)
    finally:
        c2.close()
    assert abs(E[0] - Es) < 1e-9


def test_batch_rejects_bad_input(ctx, pkg, capi):
    inst = _instances(pkg, [(6, 3, 3)], 500)
    with pytest.raises(capi.QdkgbError):
        capi.casci_batch(ctx, [(6, 7, 3, inst[0][3], inst[0][4])])
    with pytest.raises(capi.QdkgbError):
        capi.casci_batch(ctx, inst, max_subspace=1)
    E, _, _, _ = capi.casci_batch(ctx, [], want_rdm1=False)
    assert len(E) == 0
