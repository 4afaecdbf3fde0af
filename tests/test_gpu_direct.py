"""Direct (recompute-on-the-fly) sigma for complete spaces vs the CSR sigma
and the oracle.  Tolerances: FP64 sigma 1e-12 relative (the single-excitation
sum is split in two parts, so not bit-exact), FP32 sigma ~1e-6 relative,
energies 1e-10 Eh (FP64) / 1e-8 Eh (mixed)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(pkg):
    pkg.build.build()
    c = pkg.capi.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("norb,na,nb,seed", [(8, 4, 4, 1), (10, 4, 3, 2), (9, 2, 5, 3), (6, 1, 1, 4)])
def test_direct_sigma_matches_csr(ctx, pkg, norb, na, nb, seed):
    capi = pkg.capi
    T, V, _ = pkg.integrals.synthetic_integrals(norb, 10, seed)
    a, b = capi.fci_dets(norb, na, nb)
    ctx.set_integrals(T, V)
    ctx.set_dets(a, b)
    ctx.build_hamiltonian(0.0)  # keep every structural element
    x = np.random.default_rng(seed).normal(size=len(a))
    y_csr = ctx.spmv(x, capi.PREC_FP64)
    D_csr = ctx.diagonal()
    ctx.build_direct_sigma()
    y64 = ctx.spmv(x, capi.PREC_FP64)
    y32 = ctx.spmv(x, capi.PREC_MIXED)
    scale = np.max(np.abs(y_csr))
    assert np.max(np.abs(y64 - y_csr)) <= 1e-12 * scale
    rel32 = np.max(np.abs(y32 - y_csr)) / scale
    assert rel32 < 1e-5
    assert np.allclose(ctx.diagonal(), D_csr, rtol=0, atol=1e-14 * np.max(np.abs(D_csr)))
    with pytest.raises(capi.QdkgbError):
        ctx.get_csr()


@pytest.mark.parametrize("norb,na,nb,seed", [(12, 3, 3, 11), (12, 3, 4, 12), (11, 5, 5, 13), (7, 3, 2, 14)])
def test_direct_fp32_contraction_matches_walk(ctx, pkg, monkeypatch, norb, na, nb, seed):
    """The FP32 opposite-spin term as a per-alpha-string contraction (the
    default) and as the element-wise walk (QDKGB_DIRECT_MM=0) both agree
    with the CSR sigma to FP32 accuracy; shapes with more than one chunk of
    beta strings, more than one pass of pair indices (n >= 12) and unequal
    string sets."""
    capi = pkg.capi
    T, V, _ = pkg.integrals.synthetic_integrals(norb, 2 * norb, seed)
    a, b = capi.fci_dets(norb, na, nb)
    ctx.set_integrals(T, V)
    ctx.set_dets(a, b)
    ctx.build_hamiltonian(0.0)
    x = np.random.default_rng(seed).normal(size=len(a))
    y_csr = ctx.spmv(x, capi.PREC_FP64)
    scale = np.max(np.abs(y_csr))
    ys = {}
    for mm in ("1", "0"):
        monkeypatch.setenv("QDKGB_DIRECT_MM", mm)
        ctx.build_direct_sigma()
        ys[mm] = ctx.spmv(x, capi.PREC_MIXED)
        assert np.max(np.abs(ys[mm] - y_csr)) / scale < 1e-5, mm
    y2 = ctx.spmv(x, capi.PREC_MIXED)
    assert np.array_equal(y2, ys["0"])
    monkeypatch.setenv("QDKGB_DIRECT_MM", "1")
    ctx.build_direct_sigma()
    assert np.array_equal(ctx.spmv(x, capi.PREC_MIXED), ys["1"])  # reproducible


@pytest.mark.parametrize("norb,na,nb,seed", [(12, 3, 3, 21), (11, 5, 4, 22), (8, 4, 4, 23)])
def test_direct_fp32_dense_same_spin_matches_csr(ctx, pkg, monkeypatch, norb, na, nb, seed):
    """The same-spin string-only part of the contraction form as two dense
    FP32 products (QDKGB_DIRECT_DENSE=1) and as the element-wise kernels
    (=0) both agree with the CSR sigma; the structure is kept across builds
    of one space and the values follow new integrals."""
    capi = pkg.capi
    a, b = capi.fci_dets(norb, na, nb)
    ctx.set_dets(a, b)
    x = np.random.default_rng(seed).normal(size=len(a))
    for k, s2 in enumerate((seed, seed + 100)):
        T, V, _ = pkg.integrals.synthetic_integrals(norb, 2 * norb, s2)
        ctx.set_integrals(T, V)
        ctx.build_hamiltonian(0.0)
        y_csr = ctx.spmv(x, capi.PREC_FP64)
        scale = np.max(np.abs(y_csr))
        for dense in ("1", "0"):
            monkeypatch.setenv("QDKGB_DIRECT_DENSE", dense)
            ctx.build_direct_sigma()
            y32 = ctx.spmv(x, capi.PREC_MIXED)
            assert np.max(np.abs(y32 - y_csr)) / scale < 1e-5, (k, dense)
            y64 = ctx.spmv(x, capi.PREC_FP64)
            assert np.max(np.abs(y64 - y_csr)) <= 1e-12 * scale, (k, dense)
    monkeypatch.delenv("QDKGB_DIRECT_DENSE")
    ctx.build_direct_sigma()  # the first FP32 sigma times both forms and keeps one
    y32 = ctx.spmv(x, capi.PREC_MIXED)
    assert np.max(np.abs(y32 - y_csr)) / scale < 1e-5


@pytest.mark.parametrize("norb,na,nb,seed", [(6, 3, 3, 31), (10, 5, 4, 32), (12, 3, 3, 33)])
def test_tensor_core_same_spin_products(ctx, pkg, monkeypatch, norb, na, nb, seed):
    """The dense same-spin products on the tensor cores (tcgen05 TF32 x 3,
    the default; QDKGB_DIRECT_TC=0 the FMA pipe) agree with the CSR sigma to
    FP32 accuracy and with the FMA-pipe products to rounding; shapes with
    partial 128 x 64 tiles and K blocks."""
    capi = pkg.capi
    T, V, _ = pkg.integrals.synthetic_integrals(norb, 2 * norb, seed)
    a, b = capi.fci_dets(norb, na, nb)
    ctx.set_integrals(T, V)
    ctx.set_dets(a, b)
    ctx.build_hamiltonian(0.0)
    x = np.random.default_rng(seed).normal(size=len(a))
    y_csr = ctx.spmv(x, capi.PREC_FP64)
    scale = np.max(np.abs(y_csr))
    monkeypatch.setenv("QDKGB_DIRECT_DENSE", "1")
    ys = {}
    for tc in ("0", "1"):
        monkeypatch.setenv("QDKGB_DIRECT_TC", tc)
        ctx.build_direct_sigma()
        ys[tc] = ctx.spmv(x, capi.PREC_MIXED)
        assert np.all(np.isfinite(ys[tc])), tc
        assert np.max(np.abs(ys[tc] - y_csr)) / scale < 1e-5, tc
    assert np.max(np.abs(ys["1"] - ys["0"])) / scale < 1e-5
    monkeypatch.delenv("QDKGB_DIRECT_TC")


def test_direct_davidson_fp64_and_mixed(ctx, pkg, oracle):
    capi = pkg.capi
    T, V, _ = pkg.integrals.synthetic_integrals(10, 20, seed=9)
    a, b = capi.fci_dets(10, 5, 5)
    M = oracle.build_csr(oracle.Hamiltonian(T, V), a, b)
    Eo, Co, _ = M.selected_ci_diag(tol=1e-9)
    ctx.set_integrals(T, V)
    ctx.set_dets(a, b)
    ctx.build_direct_sigma()
    E64, C64, info64 = ctx.davidson(tol=1e-8, precision=capi.PREC_FP64)
    assert abs(E64 - Eo) < 1e-10
    E32, C32, info32 = ctx.davidson(tol=1e-8, precision=capi.PREC_MIXED)
    assert abs(E32 - Eo) < 1e-8
    assert info32["residual_norm"] < 1e-8
    # RDMs of the direct-sigma vector through the pair walk, vs the oracle
    R = ctx.rdms_spin_dep(C64, want=("aa", "bb"))
    Ro = oracle.rdms_spin_dep(10, a, b, C64, want=("aa", "bb"))
    assert np.max(np.abs(R["aa"] - Ro["aa"])) < 1e-12


def test_direct_rejects_incomplete_space(ctx, pkg):
    capi = pkg.capi
    T, V, _ = pkg.integrals.synthetic_integrals(8, 10, 5)
    a, b = capi.fci_dets(8, 3, 3)
    ctx.set_integrals(T, V)
    ctx.set_dets(a[:-7], b[:-7])
    with pytest.raises(capi.QdkgbError) as ei:
        ctx.build_direct_sigma()
    assert ei.value.code == capi.ERR_UNSUPPORTED
