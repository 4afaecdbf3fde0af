"""The oracle restatement against fixtures made by the reference's own MACIS
code at the benchmark configurations' sizes (tests/golden/ref_*.npz, written
by make_ref_golden.py from the unmodified reference sources): the CSR of
CASCI(8e,8o) bit-identical (SHA-256 of the int64 row pointers and columns and
the FP64 values), the Davidson energy within 1e-10 Eh with the same iteration
count, the RDMs within 1e-12, and the batched configuration's norb = 10
instances' energies within 1e-10 Eh."""
import hashlib
import os

import numpy as np

from conftest import GOLDEN


def _sha(a):
    return hashlib.sha256(memoryview(np.ascontiguousarray(a)).cast("B")).hexdigest()


def test_cas8_oracle_matches_reference(oracle):
    d = np.load(os.path.join(GOLDEN, "ref_cas8.npz"))
    norb, na, nb = int(d["norb"]), int(d["nalpha"]), int(d["nbeta"])
    a, b = oracle.fci_dets(norb, na, nb)
    assert _sha(a) == str(d["sha_alpha"]) and _sha(b) == str(d["sha_beta"])
    M = oracle.build_csr(oracle.Hamiltonian(d["T"], d["V"]), a, b)
    rp, ci, nz = M.arrays()
    assert M.nnz == int(d["nnz"])
    assert (_sha(rp), _sha(ci), _sha(nz)) == (str(d["sha_rowptr"]), str(d["sha_colind"]), str(d["sha_nzval"]))
    for r in d["sample_rows"]:
        assert np.array_equal(ci[rp[r]:rp[r + 1]], d["row%d_colind" % r])
        assert np.array_equal(nz[rp[r]:rp[r + 1]], d["row%d_nzval" % r])
    E, C, it = M.selected_ci_diag(tol=1e-8)
    assert abs(E - float(d["E"])) < 1e-10 and it == int(d["iterations"])
    R = oracle.rdms_spin_dep(norb, a, b, d["C"])
    for k in ("aa", "bb", "aaaa", "bbbb", "aabb"):
        assert np.max(np.abs(R[k] - d["rdm_" + k])) < 1e-12, k
    # the spin-traced RDMs of form_rdms are the sums of the spin blocks
    g = R["aa"] + R["bb"]
    assert np.max(np.abs(g - d["rdm_traced1"])) < 1e-12
    G = R["aaaa"] + R["bbbb"] + R["aabb"] + np.transpose(R["aabb"], (2, 3, 0, 1))
    assert np.max(np.abs(G - d["rdm_traced2"])) < 1e-12
    # lobpcgxx's lowest root is the Davidson root
    assert abs(float(d["lobpcg_evals"][0]) - float(d["E"])) < 1e-8
    assert float(d["lobpcg_evals"][1]) > float(d["lobpcg_evals"][0])


def test_batch_norb10_oracle_matches_reference(oracle):
    d = np.load(os.path.join(GOLDEN, "ref_batch10.npz"))
    a, b = oracle.fci_dets(10, 5, 5)
    for j, i in enumerate(d["index"]):
        M = oracle.build_csr(oracle.Hamiltonian(d["T%d" % i], d["V%d" % i]), a, b)
        E, C, _ = M.selected_ci_diag(tol=1e-8)
        assert abs(E - d["E"][j]) < 1e-10, (j, E, d["E"][j])
        R = oracle.rdms_spin_dep(10, a, b, C, want=("aa", "bb"))
        assert np.max(np.abs(R["aa"] - d["rdm_aa"][j])) < 1e-9
