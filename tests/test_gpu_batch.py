"""Batched CASCI (qdkgb_casci_batch) against the CPU oracle: per-instance
energies (mixed form within 1e-8 Eh of the oracle's FP64 Davidson, FP64 form
within 1e-10) and spin-summed 1-RDMs (1e-6 absolute: the vectors agree to the
residual tolerance over the gap), for instances of uneven size and shape,
through both solvers: the lockstep launch sequence (default) and the
persistent cluster kernel (every cluster size agrees with the lockstep
path)."""
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


@pytest.mark.parametrize("persistent", [1, 0])
def test_batch_mixed_matches_oracle(ctx, oracle, pkg, capi, persistent):
    inst = _instances(pkg, SHAPES, 100)
    E, R, its, info = capi.casci_batch(ctx, inst, res_tol=1e-8, persistent=persistent)
    assert (info["graph_replays"] > 0) == (persistent == 0)
    for i, q in enumerate(inst):
        Eo, Ro = _oracle_ref(oracle, pkg, q)
        assert abs(E[i] - Eo) < 1e-8, (i, E[i], Eo)
        np.testing.assert_allclose(R[i], Ro, atol=1e-6, rtol=0, err_msg=str(i))
        assert abs(np.trace(R[i]) - (q[1] + q[2])) < 1e-10
        assert its[i] > 0


def test_batch_direct_sigma_equals_slab_sigma(ctx, pkg, capi, monkeypatch, oracle):
    """The lockstep solver's new directions through the direct contraction
    (default for complete spaces) or the stored FP32 slab
    (QDKGB_BATCH_DIRECT=0): the same energies and 1-RDMs (the full-precision
    refreshes decide convergence), both at the oracle's."""
    inst = _instances(pkg, [(10, 5, 5), (8, 4, 4), (10, 5, 4), (6, 3, 3), (8, 4, 4)], 800)
    E1, R1, _, _ = capi.casci_batch(ctx, inst, persistent=0)
    monkeypatch.setenv("QDKGB_BATCH_DIRECT", "0")
    E0, R0, _, _ = capi.casci_batch(ctx, inst, persistent=0)
    assert np.max(np.abs(E1 - E0)) < 1e-9
    for i in range(len(inst)):
        np.testing.assert_allclose(R1[i], R0[i], atol=1e-7, rtol=0)
    for j in (0, 2):
        Eo, _ = _oracle_ref(oracle, pkg, inst[j])
        assert abs(E1[j] - Eo) < 1e-8


@pytest.mark.parametrize("persistent", [1, 0])
def test_batch_fp64_matches_oracle(ctx, oracle, pkg, capi, persistent):
    inst = _instances(pkg, SHAPES[:5], 200)
    E, R, its, info = capi.casci_batch(ctx, inst, res_tol=1e-9, precision=capi.PREC_FP64, persistent=persistent)
    for i, q in enumerate(inst):
        Eo, Ro = _oracle_ref(oracle, pkg, q)
        assert abs(E[i] - Eo) < 1e-10, (i, E[i], Eo)
        np.testing.assert_allclose(R[i], Ro, atol=1e-6, rtol=0)


def test_batch_graph_replay_is_identical_and_order_independent(ctx, pkg, capi):
    inst = _instances(pkg, SHAPES, 300)
    E1, _, it1, i1 = capi.casci_batch(ctx, inst, want_rdm1=False, use_graph=1, persistent=0)
    E2, _, it2, i2 = capi.casci_batch(ctx, inst, want_rdm1=False, use_graph=0, persistent=0)
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


def test_persistent_cluster_sizes_agree_with_lockstep(ctx, pkg, capi):
    """Every cluster size of the persistent solver (CTAs per instance) gives
    the lockstep path's energies and 1-RDMs.  The algorithm is the same; the
    reductions run in another order, and the lockstep path's FP32 sigma is
    the vectorised kernel (another rounding of the FP32 products), so the
    mixed form's iteration counts may differ; the FP64 form's agree to one."""
    inst = _instances(pkg, [(8, 4, 4), (8, 4, 4), (8, 4, 3), (6, 3, 3), (8, 4, 4)], 600)
    E0, R0, it0, _ = capi.casci_batch(ctx, inst, persistent=0)
    F0, _, f0, _ = capi.casci_batch(ctx, inst, want_rdm1=False, persistent=0, precision=capi.PREC_FP64)
    for cl in (1, 2, 4):
        E, R, its, _ = capi.casci_batch(ctx, inst, persistent=1, cluster=cl)
        assert np.max(np.abs(E - E0)) < 1e-9, cl
        for i in range(len(inst)):
            np.testing.assert_allclose(R[i], R0[i], atol=1e-7, rtol=0)
        assert np.all(its > 0)
        F, _, f, _ = capi.casci_batch(ctx, inst, want_rdm1=False, persistent=1, cluster=cl,
                                      precision=capi.PREC_FP64)
        assert np.max(np.abs(F - F0)) < 1e-10, cl
        assert np.all(np.abs(f - f0) <= 1), (cl, f, f0)


def test_persistent_autotuner_records_its_choice(pkg, capi, oracle):
    """The first persistent call on a context times the cluster-size
    candidates of each shape (a few iterations of every instance) and keeps
    the fastest (qdkgb_batch_plan); the energies match the oracle."""
    inst = _instances(pkg, [(10, 5, 5)] * 3 + [(6, 3, 3)] * 2, 700)
    with capi.Context(0) as c:
        assert capi.batch_plan(c) == []
        E, _, _, _ = capi.casci_batch(c, inst, want_rdm1=False, persistent=1)
        plan = {p["shape"]: p for p in capi.batch_plan(c)}
        E2, _, _, _ = capi.casci_batch(c, inst, want_rdm1=False, persistent=1)
        assert len(capi.batch_plan(c)) == len(plan)
    p10 = plan[(10, 5, 5)]
    assert len(p10["candidates"]) >= 2 and p10["cluster"] in [q for q, _ in p10["candidates"]]
    assert all(ms > 0 for _, ms in p10["candidates"])
    assert min(p10["candidates"], key=lambda q: q[1])[0] == p10["cluster"]
    assert (6, 3, 3) not in plan  # one candidate only: nothing to time
    assert np.max(np.abs(E - E2)) < 1e-9
    for j in (0, 3):
        Eo, _ = _oracle_ref(oracle, pkg, inst[j])
        assert abs(E[j] - Eo) < 1e-8
