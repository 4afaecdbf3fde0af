"""GPU parity against the CPU oracle and the reference's golden vectors, all
through the C ABI (libqdkgb.so).

Tolerances: determinant lists, CSR row pointers and columns are compared
bit-exact; FP64 matrix elements bit-exact as well (the kernels reproduce the
reference's operation order), with 1e-12 relative as the documented bar;
energies 1e-10 Eh (FP64) and 1e-8 Eh (mixed precision); RDMs 1e-12 absolute.
"""
import numpy as np
import pytest

from conftest import GOLDEN

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


def _cas(pkg, norb, nel, nchol, seed, spacing=0.25):
    T, V, _ = pkg.integrals.synthetic_integrals(norb, nchol, seed, diag_spacing=spacing)
    a, b = pkg.determinants.fci_space(norb, nel // 2, nel // 2)
    return T, V, a, b


def _check_csr(ctx, oracle, T, V, a, b, thresh):
    ctx.set_integrals(T, V)
    ctx.set_dets(a, b)
    nnz = ctx.build_hamiltonian(thresh)
    rp, ci, nz = ctx.get_csr(64)
    M = oracle.build_csr(oracle.Hamiltonian(T, V), a, b, thresh)
    orp, oci, onz = M.arrays()
    assert nnz == M.nnz
    np.testing.assert_array_equal(rp, orp)
    np.testing.assert_array_equal(ci, oci)
    # bit-exact values (the documented bar is 1e-12 relative)
    np.testing.assert_allclose(nz, onz, rtol=1e-12, atol=0)
    assert np.array_equal(nz, onz), "FP64 values differ from the oracle in the last bits"
    np.testing.assert_array_equal(ctx.diagonal(), M.diag())
    return M


def test_cas88_csr_bit_exact(ctx, oracle, pkg):
    T, V, a, b = _cas(pkg, 8, 8, 16, seed=11)
    M = _check_csr(ctx, oracle, T, V, a, b, np.finfo(float).eps)
    assert M.nnz == 4900 * 361


def test_h2o_cisd_csr_golden(ctx, oracle, pkg, h2o, known):
    d = pkg.determinants
    a, b = d.spin_sort(*d.cisd_space(24, *d.canonical_hf(5, 5)))
    M = _check_csr(ctx, oracle, h2o["T"], h2o["V"], a, b, 1e-16)
    rp32, ci32, _ = ctx.get_csr(32)
    golden = np.load(GOLDEN + "/h2o_ccpvdz_cisd_rowptr.npy")
    np.testing.assert_array_equal(rp32, golden)
    assert ctx.nnz == known["h2o_cisd_csr"]["nnz"]


def test_thresh_zero_keeps_structural_zeros(ctx, oracle, pkg, n2_6e6o):
    a, b = pkg.determinants.fci_space(6, 3, 3)
    _check_csr(ctx, oracle, n2_6e6o["T"], n2_6e6o["V"], a, b, 0.0)
    _check_csr(ctx, oracle, n2_6e6o["T"], n2_6e6o["V"], a, b, 1e-6)


def test_uneven_spaces_and_edge_cases(ctx, oracle, pkg):
    T, V, _ = pkg.integrals.synthetic_integrals(10, 12, seed=5)
    # open shell, nalpha != nbeta
    a, b = pkg.determinants.fci_space(10, 4, 2)
    _check_csr(ctx, oracle, T, V, a, b, 1e-14)
    # a selected (ragged) subset sorted by spin_comparator
    rng = np.random.default_rng(0)
    a, b = pkg.determinants.fci_space(10, 3, 3)
    keep = np.sort(rng.choice(len(a), 3000, replace=False))
    sa, sb = pkg.determinants.spin_sort(a[keep], b[keep])
    _check_csr(ctx, oracle, T, V, sa, sb, 1e-14)
    # single determinant
    _check_csr(ctx, oracle, T, V, sa[:1], sb[:1], 1e-14)
    # one electron per spin
    a, b = pkg.determinants.fci_space(10, 1, 1)
    _check_csr(ctx, oracle, T, V, a, b, 1e-14)


def test_build_is_deterministic(ctx, pkg):
    T, V, a, b = _cas(pkg, 8, 8, 16, seed=2)
    ctx.set_integrals(T, V)
    ctx.set_dets(a, b)
    ctx.build_hamiltonian()
    r1 = ctx.get_csr()
    ctx.build_hamiltonian()
    r2 = ctx.get_csr()
    for x, y in zip(r1, r2):
        assert np.array_equal(x, y)


def test_split_storage_and_spmv(ctx, oracle, pkg, capi):
    T, V, a, b = _cas(pkg, 8, 8, 16, seed=4)
    ctx.set_integrals(T, V)
    ctx.set_dets(a, b)
    ctx.build_hamiltonian(storage=capi.H_FP64)
    _, _, nz64 = ctx.get_csr()
    x = np.random.default_rng(1).normal(size=len(a))
    y64 = ctx.spmv(x, capi.PREC_FP64)
    M = oracle.build_csr(oracle.Hamiltonian(T, V), a, b)
    yo = M.spmv(x)
    assert np.max(np.abs(y64 - yo)) <= 1e-12 * np.max(np.abs(yo))
    ctx.build_hamiltonian(storage=capi.H_SPLIT32)
    _, _, nzs = ctx.get_csr()
    assert np.all(np.abs(nzs - nz64) <= 2.0 ** -47 * np.abs(nz64))
    ys = ctx.spmv(x, capi.PREC_FP64)  # hi+lo values, FP64 accumulation
    assert np.max(np.abs(ys - yo)) <= 1e-12 * np.max(np.abs(yo))
    y32 = ctx.spmv(x, capi.PREC_MIXED)  # FP32 values/x/accumulation
    rel = np.max(np.abs(y32 - yo)) / np.max(np.abs(yo))
    assert 1e-9 < rel < 1e-5


def test_davidson_fp64_matches_oracle(ctx, oracle, pkg):
    T, V, a, b = _cas(pkg, 8, 8, 16, seed=7)
    ctx.set_integrals(T, V)
    ctx.set_dets(a, b)
    ctx.build_hamiltonian()
    E, C, info = ctx.davidson(tol=1e-8)
    M = oracle.build_csr(oracle.Hamiltonian(T, V), a, b)
    Eo, Co, ito = M.selected_ci_diag(tol=1e-8)
    assert abs(E - Eo) < 1e-10
    assert abs(abs(C @ Co) - 1.0) < 1e-10
    assert info["residual_norm"] < 1e-8
    assert info["iterations"] == ito  # same algorithm, same iteration count


def test_davidson_h2o_cisd_golden(ctx, pkg, h2o, known):
    ref = known["h2o_cisd_davidson"]
    d = pkg.determinants
    a, b = d.spin_sort(*d.cisd_space(24, *d.canonical_hf(5, 5)))
    ctx.set_integrals(h2o["T"], h2o["V"])
    ctx.set_dets(a, b)
    ctx.build_hamiltonian(1e-16)
    E, C, info = ctx.davidson(max_m=ref["max_m"], tol=ref["tol"])
    assert abs(E + h2o["E_core"] - ref["E0_total"]) < ref["atol"]
    assert abs(np.linalg.norm(C) - 1) < 1e-12


def test_davidson_n2_casci_golden(ctx, pkg, n2_6e6o, known):
    E, C, info = ctx.casci(n2_6e6o["T"], n2_6e6o["V"], 3, 3)
    assert np.isclose(E, known["n2_6e6o_casci"]["E_total"])


@pytest.mark.parametrize("fp32", ["direct", "slab"])
def test_mixed_precision_energy(ctx, oracle, pkg, capi, monkeypatch, fp32):
    """Mixed form on a complete space with either FP32 sigma: the direct
    contraction beside the FP64 slab (default) or the stored FP32 slab copy
    (QDKGB_MIXED_FP32=slab)."""
    T, V, a, b = _cas(pkg, 10, 10, 20, seed=8)
    M = oracle.build_csr(oracle.Hamiltonian(T, V), a, b)
    Eo, _, _ = M.selected_ci_diag(tol=1e-9)
    if fp32 == "slab":
        monkeypatch.setenv("QDKGB_MIXED_FP32", "slab")
    ctx.set_integrals(T, V)
    ctx.set_dets(a, b)
    ctx.build_hamiltonian(storage=capi.H_SPLIT32)
    assert ctx.operator_layout()[0] == (capi.OP_SLAB if fp32 == "slab" else capi.OP_SLAB_DIRECT32)
    E, C, info = ctx.davidson(tol=1e-8, precision=capi.PREC_MIXED)
    assert abs(E - Eo) < 1e-8, (E - Eo, info)
    assert info["residual_norm"] < 1e-8
    assert info["spmv_fp32"] > info["spmv_fp64"]


def test_davidson_not_converged_raises(ctx, pkg, capi):
    T, V, a, b = _cas(pkg, 8, 8, 16, seed=9)
    ctx.set_integrals(T, V)
    ctx.set_dets(a, b)
    ctx.build_hamiltonian()
    with pytest.raises(capi.NotConverged):
        ctx.davidson(max_m=3, tol=1e-12)


def _rdm_check(ctx, oracle, n, a, b, C, atol=1e-12):
    R = ctx.rdms_spin_dep(C)
    Ro = oracle.rdms_spin_dep(n, a, b, C)
    for k in Ro:
        np.testing.assert_allclose(R[k], Ro[k], atol=atol, rtol=0, err_msg=k)
    return R


def test_rdms_match_oracle_cas(ctx, oracle, pkg):
    T, V, a, b = _cas(pkg, 8, 8, 16, seed=12)
    ctx.set_integrals(T, V)
    ctx.set_dets(a, b)
    ctx.build_hamiltonian()
    E, C, _ = ctx.davidson()
    R = _rdm_check(ctx, oracle, 8, a, b, C)
    E_rdm = (np.sum(T * (R["aa"] + R["bb"])) + np.sum(V * (R["aaaa"] + R["bbbb"])) + 2 * np.sum(V * R["aabb"]))
    assert abs(E_rdm - E) < 1e-10


def test_rdms_sliced_tile_norb14(ctx, oracle, pkg):
    # n = 14: the n^4 tile is split over last-index slices
    T, V, _ = pkg.integrals.synthetic_integrals(14, 6, seed=2)
    a, b = pkg.determinants.fci_space(14, 2, 2)
    ctx.set_integrals(T, V)
    ctx.set_dets(a, b)
    C = np.random.default_rng(3).normal(size=len(a))
    C /= np.linalg.norm(C)
    _rdm_check(ctx, oracle, 14, a, b, C)


def test_rdms_o2_wavefunction_golden(ctx, oracle, pkg):
    """external/macis/tests/double_loop.cxx:506-579 through the GPU (n = 34:
    global-memory accumulation path).  The list is sorted by spin_comparator
    (RDMs are invariant under the permutation); the empty padding
    determinants are dropped (the reference skips them)."""
    w = np.load(GOLDEN + "/o2_wfn.npz")
    C = w["coeffs"] / np.linalg.norm(w["coeffs"])
    order = np.lexsort((w["beta"], w["alpha"]))
    a, b, C = w["alpha"][order], w["beta"][order], C[order]
    T = np.zeros((34, 34))
    V = np.zeros((34,) * 4)
    ctx.set_integrals(T, V)
    ctx.set_dets(a, b)
    R = _rdm_check(ctx, oracle, 34, a, b, C)
    ordm = R["aa"] + R["bb"]
    trdm = R["aaaa"] + R["bbbb"] + R["aabb"] + R["aabb"].transpose(2, 3, 0, 1)
    assert abs(np.abs(ordm).sum() - 8.0000005763) < 1e-6
    assert abs(np.abs(trdm).sum() - 44.1092472977) < 1e-6


def test_mixed_precision_stays_in_the_guess_symmetry_sector(ctx, oracle, pkg, capi):
    """Seeded case whose lowest S_z = 0 state is odd under spin flip: the
    reference's FP64 iteration from the closed-shell guess stays in the even
    sector; the mixed solve must land on the same state."""
    T, V, a, b = _cas(pkg, 10, 10, 20, seed=9)
    M = oracle.build_csr(oracle.Hamiltonian(T, V), a, b)
    Eo, _, _ = M.selected_ci_diag(tol=1e-9)
    ctx.set_integrals(T, V)
    ctx.set_dets(a, b)
    ctx.build_hamiltonian(storage=capi.H_SPLIT32)
    E, C, info = ctx.davidson(tol=1e-8, precision=capi.PREC_MIXED)
    assert abs(E - Eo) < 1e-8, (E, Eo)


def test_operator_layouts(ctx, oracle, pkg, capi):
    """Complete spaces are held in the slab layout (values only) and export
    the reference's CSR bit-exactly; a threshold that drops most elements
    turns the slab into CSR; selected spaces and direct sigma report theirs."""
    T, V, a, b = _cas(pkg, 8, 8, 16, seed=13)
    ctx.set_integrals(T, V)
    ctx.set_dets(a, b)
    ctx.build_hamiltonian(np.finfo(float).eps)
    lay, stored = ctx.operator_layout()
    assert lay == capi.OP_SLAB and stored == len(a) * 361 == ctx.nnz
    # most elements below the threshold: CSR, still identical to the oracle
    big = float(np.quantile(np.abs(oracle.build_csr(oracle.Hamiltonian(T, V), a, b).arrays()[2]), 0.7))
    _check_csr(ctx, oracle, T, V, a, b, big)
    assert ctx.operator_layout()[0] == capi.OP_CSR
    # a few elements dropped: slab with zeros, CSR export identical
    small = float(np.quantile(np.abs(oracle.build_csr(oracle.Hamiltonian(T, V), a, b).arrays()[2]), 0.1))
    _check_csr(ctx, oracle, T, V, a, b, small)
    assert ctx.operator_layout()[0] == capi.OP_SLAB
    x = np.random.default_rng(4).normal(size=len(a))
    M = oracle.build_csr(oracle.Hamiltonian(T, V), a, b, small)
    yo = M.spmv(x)
    assert np.max(np.abs(ctx.spmv(x, capi.PREC_FP64) - yo)) <= 1e-12 * np.max(np.abs(yo))
    # a selected (non-product) space uses CSR
    rng = np.random.default_rng(1)
    keep = np.sort(rng.choice(len(a), 1000, replace=False))
    sa, sb = pkg.determinants.spin_sort(a[keep], b[keep])
    ctx.set_dets(sa, sb)
    ctx.build_hamiltonian()
    assert ctx.operator_layout()[0] == capi.OP_CSR
    ctx.set_dets(a, b)
    ctx.build_direct_sigma()
    assert ctx.operator_layout()[0] == capi.OP_DIRECT


def test_casci_reuses_the_complete_space(ctx, oracle, pkg):
    """Repeated qdkgb_casci calls of one shape keep the determinant space;
    new integrals, a different shape or an explicit set_dets rebuild what
    they must."""
    for seed, (norb, na) in [(21, (8, 4)), (22, (8, 4)), (23, (6, 3)), (24, (8, 4))]:
        T, V, _ = pkg.integrals.synthetic_integrals(norb, 2 * norb, seed)
        a, b = pkg.determinants.fci_space(norb, na, na)
        Eo, _, _ = oracle.build_csr(oracle.Hamiltonian(T, V), a, b).selected_ci_diag(tol=1e-10)
        E, C, _ = ctx.casci(T, V, na, na, tol=1e-9)
        assert abs(E - Eo) < 1e-9, (seed, E, Eo)
        if seed == 22:
            # a selected list in between must not be mistaken for the space
            ctx.set_dets(a[:100], b[:100])


@pytest.mark.late
def test_device_limit_gives_oom_and_the_context_recovers(pkg, oracle):
    """Failure detection with the capped allocator (qdkgb_set_device_limit):
    a Hamiltonian build that needs more device memory than the cap fails with
    QDKGB_ERR_OOM before reaching the device; with the cap lifted the same
    context builds and solves to the oracle's energy."""
    capi = pkg.capi
    T, V, _ = pkg.integrals.synthetic_integrals(8, 16, 21)
    a, b = capi.fci_dets(8, 4, 4)
    with capi.Context(0) as ctx:
        ctx.set_integrals(T, V)
        ctx.set_dets(a, b)
        ctx.set_device_limit(ctx.device_bytes() + 4096)
        with pytest.raises(capi.QdkgbError) as ei:
            ctx.build_hamiltonian()
        assert ei.value.code == capi.ERR_OOM and "limit" in str(ei.value)
        ctx.set_device_limit(0)
        ctx.build_hamiltonian()
        E, _, _ = ctx.davidson(tol=1e-10)
    Eo, _, _ = oracle.build_csr(oracle.Hamiltonian(T, V), a, b).selected_ci_diag(tol=1e-10)
    assert abs(E - Eo) < 1e-10


def test_tma_fed_fp32_sigma_equals_register_fed(pkg, monkeypatch):
    """The FP32 slab sigma kernels (register-fed four, eight and sixteen
    positions deep; TMA-fed: bulk copies of the slab rows into a
    shared-memory ring) sum every row in the same order, so on the same plan
    (QDKGB_SIGMA32_KERNEL pins the kernel and the planner's default segments)
    they give the same FP32 sigma bit for bit; left to itself the autotuner
    times every kernel on every candidate plan and keeps the fastest pair."""
    capi = pkg.capi
    pkg.build.build()
    T, V, _ = pkg.integrals.synthetic_integrals(10, 20, seed=31)
    a, b = capi.fci_dets(10, 5, 5)
    x = np.random.default_rng(5).normal(size=len(a)).astype(np.float32)
    out = {}
    monkeypatch.setenv("QDKGB_MIXED_FP32", "slab")  # the stored FP32 copy
    for kern in capi.SIGMA32_KERNELS + (None,):
        if kern:
            monkeypatch.setenv("QDKGB_SIGMA32_KERNEL", kern)
        else:
            monkeypatch.delenv("QDKGB_SIGMA32_KERNEL", raising=False)
        with capi.Context(0) as ctx:
            ctx.set_integrals(T, V)
            ctx.set_dets(a, b)
            ctx.build_hamiltonian(storage=capi.H_SPLIT32)
            y = ctx.spmv(x, precision=capi.PREC_MIXED)
            seg, cand, used, kms = ctx.sigma_plan(capi.PREC_MIXED, with_kernel=True)
            out[kern] = (np.asarray(y, dtype=np.float32), used, cand, kms, seg)
    for k in capi.SIGMA32_KERNELS:
        assert out[k][1] == k and out[k][4] == out["register"][4]
        assert np.array_equal(out["register"][0].view(np.uint32), out[k][0].view(np.uint32)), k
    _, used, cand, kms, seg = out[None]
    assert len(cand) >= 1
    for k in capi.SIGMA32_KERNELS:
        assert len(kms[k]) == len(cand) and all(np.isfinite(t) and t > 0 for t in kms[k]), k
    best = min(min(v) for v in kms.values())
    chosen = [t for (s, _), t in zip(cand, kms[used]) if s == seg]
    assert abs(min(chosen) - best) < 1e-12
    assert np.max(np.abs(out[None][0] - out["register"][0])) <= 1e-5 * np.max(np.abs(out["register"][0]))
