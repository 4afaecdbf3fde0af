"""Parity at the benchmark configurations' own sizes, against fixtures made by
the reference's own MACIS code (tests/golden/ref_*.npz, written by
make_ref_golden.py from the unmodified reference sources).

* CASCI(8e,8o) (4,900 determinants): the CSR (int64 row pointers and columns,
  FP64 values) is bit-identical to make_csr_hamiltonian<int64_t>'s, in both
  storage layouts; E(FP64) within 1e-10 Eh of the reference's Davidson with the
  same iteration count; E(mixed) within 1e-8 Eh; RDMs of the GPU vector
  within 1e-12 of the oracle's and 1e-8 of the reference's (the reference's
  RDMs are of its own vector, equal to ours to the residual tolerance).
* CASCI(12e,12o) (853,776 determinants, 1,553,018,544 elements): the CSR
  digests are compared block by block (qdkgb_get_csr64_rows), E(FP64) within
  1e-10 Eh with the same iteration count, E(mixed) within 1e-8 Eh, sample rows
  equal element for element, 1-RDMs within 1e-8.
* The batched configuration's norb = 10 instances (63,504 determinants):
  energies within 1e-8 Eh and 1-RDMs within 1e-6 (the batched tolerance).
* ASCI over 40 orbitals (8 + 8 electrons, Fixed core 10,000, grow factor 8)
  grown to 200,000 determinants: the selected determinant set equals the
  reference's (digest of the list sorted by (alpha, beta)) and E within 1e-8 Eh.
"""
import hashlib
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = [pytest.mark.gpu, pytest.mark.late]

EPS = float(np.finfo(np.float64).eps)


def _fixture(name):
    p = os.path.join(GOLDEN, name)
    if not os.path.exists(p):
        pytest.fail("missing fixture %s (make_ref_golden.py)" % name)
    return np.load(p)


@pytest.fixture(scope="module")
def capi(pkg):
    pkg.build.build()
    return pkg.capi


def _sha(a):
    return hashlib.sha256(memoryview(np.ascontiguousarray(a)).cast("B")).hexdigest()


def _csr_digests(ctx, n, block=65536):
    """SHA-256 of the global int64 row pointers, int64 columns and FP64
    values, accumulated over row blocks so the host holds one block at a time."""
    hr, hc, hv = hashlib.sha256(), hashlib.sha256(), hashlib.sha256()
    off = 0
    for r0 in range(0, n, block):
        r1 = min(n, r0 + block)
        rp, ci, nz = ctx.get_csr_rows(r0, r1)
        hr.update(memoryview(np.ascontiguousarray(rp[:-1] + off)).cast("B"))
        hc.update(memoryview(ci).cast("B"))
        hv.update(memoryview(nz).cast("B"))
        off += int(rp[-1])
    hr.update(memoryview(np.array([off], np.int64)).cast("B"))
    return hr.hexdigest(), hc.hexdigest(), hv.hexdigest(), off


def test_cas8_config_matches_reference(capi, pkg, oracle):
    d = _fixture("ref_cas8.npz")
    norb, na, nb = int(d["norb"]), int(d["nalpha"]), int(d["nbeta"])
    a, b = capi.fci_dets(norb, na, nb)
    assert _sha(a) == str(d["sha_alpha"]) and _sha(b) == str(d["sha_beta"])
    with capi.Context(0) as ctx:
        ctx.set_integrals(d["T"], d["V"])
        ctx.set_dets(a, b)
        for storage in (capi.H_FP64, capi.H_SPLIT32):
            nnz = ctx.build_hamiltonian(storage=storage)
            assert nnz == int(d["nnz"])
            rp, ci, nz = ctx.get_csr(64)
            assert _sha(rp) == str(d["sha_rowptr"]) and _sha(ci) == str(d["sha_colind"])
            if storage == capi.H_FP64:
                assert _sha(nz) == str(d["sha_nzval"])
            # the block getter gives the same digests
            assert _csr_digests(ctx, len(a), block=777)[:2] == (str(d["sha_rowptr"]), str(d["sha_colind"]))
        ctx.build_hamiltonian(storage=capi.H_FP64)
        E, C, info = ctx.davidson(tol=1e-8)
        assert abs(E - float(d["E"])) < 1e-10, (E, float(d["E"]))
        assert info["iterations"] == int(d["iterations"])
        R = ctx.rdms_spin_dep(C)
        ctx.build_hamiltonian(storage=capi.H_SPLIT32)
        Em, _, _ = ctx.davidson(tol=1e-8, precision=capi.PREC_MIXED)
        assert abs(Em - float(d["E"])) < 1e-8
    Ro = oracle.rdms_spin_dep(norb, a, b, C)
    for k in ("aa", "bb", "aaaa", "bbbb", "aabb"):
        assert np.max(np.abs(R[k] - Ro[k])) < 1e-12, k
        assert np.max(np.abs(R[k] - d["rdm_" + k])) < 1e-8, k


def test_cas12_config_matches_reference(capi):
    d = _fixture("ref_cas12.npz")
    norb, na, nb = int(d["norb"]), int(d["nalpha"]), int(d["nbeta"])
    a, b = capi.fci_dets(norb, na, nb)
    assert _sha(a) == str(d["sha_alpha"]) and _sha(b) == str(d["sha_beta"])
    with capi.Context(0) as ctx:
        ctx.set_integrals(d["T"], d["V"])
        ctx.set_dets(a, b)
        nnz = ctx.build_hamiltonian(storage=capi.H_FP64)
        assert nnz == int(d["nnz"])
        hr, hc, hv, total = _csr_digests(ctx, len(a))
        assert total == int(d["nnz"])
        assert (hr, hc, hv) == (str(d["sha_rowptr"]), str(d["sha_colind"]), str(d["sha_nzval"]))
        for r in d["sample_rows"]:
            rp, ci, nz = ctx.get_csr_rows(int(r), int(r) + 1)
            assert np.array_equal(ci, d["row%d_colind" % r]) and np.array_equal(nz, d["row%d_nzval" % r])
        E, C, info = ctx.davidson(tol=1e-8)
        assert abs(E - float(d["E"])) < 1e-10, (E, float(d["E"]))
        assert info["iterations"] == int(d["iterations"])
        R = ctx.rdms_spin_dep(C, want=("aa", "bb"))
        assert np.max(np.abs(R["aa"] - d["rdm_aa"])) < 1e-8
        assert np.max(np.abs(R["bb"] - d["rdm_bb"])) < 1e-8
        ctx.build_hamiltonian(storage=capi.H_SPLIT32)
        Em, _, _ = ctx.davidson(tol=1e-8, precision=capi.PREC_MIXED)
        assert abs(Em - float(d["E"])) < 1e-8, (Em, float(d["E"]))


def test_batch_norb10_instances_match_reference(capi):
    d = _fixture("ref_batch10.npz")
    inst = [(10, 5, 5, d["T%d" % i], d["V%d" % i]) for i in d["index"]]
    with capi.Context(0) as ctx:
        E, R, its, _ = capi.casci_batch(ctx, inst, res_tol=1e-8)
    for j in range(len(inst)):
        assert abs(E[j] - d["E"][j]) < 1e-8, (j, E[j], d["E"][j])
        np.testing.assert_allclose(R[j], d["rdm_aa"][j] + d["rdm_bb"][j], atol=1e-6, rtol=0)


def test_asci40_selected_set_matches_reference(capi, pkg):
    from conftest import unpack_eri
    d = _fixture("ref_asci40.npz")
    norb = int(d["norb"])
    a0, b0 = pkg.determinants.canonical_hf(int(d["nalpha"]), int(d["nbeta"]))
    with capi.Context(0) as ctx:
        ctx.set_integrals(d["T"], unpack_eri(d["V_packed"], norb))
        ctx.set_dets(np.array([a0], np.uint64), np.array([b0], np.uint64))
        ctx.build_hamiltonian()
        E0 = float(ctx.diagonal()[0])
        _, a, b, c, Eg = capi.asci(ctx, [a0], [b0], [1.0], E0, grow=True, refine=False,
                                   ntdets_max=int(d["ntdets_max"]), core_selection_fixed=1, ncdets_max=10000,
                                   grow_factor=8)
    assert len(a) == int(d["ndets"])
    order = np.lexsort((b, a))
    sa, sb = a[order], b[order]
    assert np.array_equal(sa[:512], d["head_alpha"]) and np.array_equal(sb[:512], d["head_beta"])
    assert np.array_equal(sa[-512:], d["tail_alpha"]) and np.array_equal(sb[-512:], d["tail_beta"])
    assert (_sha(sa), _sha(sb)) == (str(d["sha_sorted_alpha"]), str(d["sha_sorted_beta"]))
    assert abs(Eg - float(d["E_grow"])) < 1e-8, (Eg, float(d["E_grow"]))
    assert norb == 40
