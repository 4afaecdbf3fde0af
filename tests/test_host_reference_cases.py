"""The library's host-side determinant and FCIDUMP handling against the
reference's own unit tests (CPU only):

* external/macis/tests/sd_operations.cxx: the canonical HF determinant,
  occupied / virtual lists, single and double excitations of one spin string
  and of both, the CIS and CISD spaces, the FCI space order and the
  canonical-string conversions (determinant lists in tests/golden/
  sd_operations.json, read out of that file by make_golden.py);
* external/macis/tests/fcidump.cxx: header, core energy and the one- and
  two-body sums of the water cc-pVDZ FCIDUMP as read by
  ``integrals_from_lines``, the canonical orbital energies (the diagonal of
  the oracle's inactive Fock matrix with 5 occupied orbitals) and the MP2
  energy formed from them (tolerance 1e-6)."""
import json
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def sd_ref():
    with open(os.path.join(GOLDEN, "sd_operations.json")) as f:
        return json.load(f)


def pack(alpha, beta, half):
    """MACIS's single-bitset form wfn_t<2*half>: alpha low, beta high."""
    return [int(a) | (int(b) << half) for a, b in zip(np.atleast_1d(alpha), np.atleast_1d(beta))]


def test_canonical_hf_and_occ_vir(pkg):
    det = pkg.determinants
    a, b = det.canonical_hf(4, 2)
    assert pack(a, b, 16) == [0x0003000F]  # wfn_t<32>
    occ, vir = det._occ_vir(12, 0xAF)
    assert occ == [0, 1, 2, 3, 5, 7] and vir == [4, 6, 8, 9, 10, 11]


def test_single_spin_excitations(pkg, sd_ref):
    det = pkg.determinants
    hf = int(det.canonical_hf(4, 0)[0])
    assert sorted(det._singles(8, hf)) == sorted(sd_ref["singles_single_spin"])
    assert sorted(det._doubles(8, hf)) == sorted(sd_ref["doubles_single_spin"])


def test_cis_and_cisd_spaces(pkg, sd_ref):
    """CISD of the 8-orbital HF(4,4) determinant = HF + the reference's both-spin
    singles + its both-spin doubles; the singles part alone with HF is the
    reference's CIS space."""
    det = pkg.determinants
    a0, b0 = det.canonical_hf(4, 4)
    a, b = det.cisd_space(8, a0, b0)
    packed = pack(a, b, 32)
    hf = pack(a0, b0, 32)[0]
    singles, doubles = sd_ref["singles_both_spins"], sd_ref["doubles_both_spins"]
    assert len(packed) == len(set(packed)) == 1 + len(singles) + len(doubles)
    assert sorted(packed) == sorted([hf] + singles + doubles)
    ns = len(singles)
    assert packed[0] == hf and sorted(packed[1:1 + ns]) == sorted(singles)


def test_fci_order(pkg, sd_ref):
    det = pkg.determinants
    assert [int(x) for x in det.combs(4, 2)] == sd_ref["fci_combs_4_2"]
    a, b = det.fci_space(4, 2, 2)
    assert pack(a, b, 32) == sd_ref["fci_space_4_2_2"]


def test_canonical_strings(pkg):
    det = pkg.determinants
    a, b = det.canonical_hf(2, 2)
    a, b = int(a) ^ (1 << 3), int(b) ^ (1 << 4)  # .flip(3).flip(4 + 32)
    full = "220ud" + "0" * 27
    assert det.to_canonical_string(a, b, 32) == full
    for s in (full, "220ud"):
        fa, fb = det.from_canonical_string(s)
        assert (int(fa), int(fb)) == (a, b)


def test_water_fcidump(pkg, oracle, h2o, known):
    ref = known["h2o_fcidump"]
    tol = ref["atol"]
    assert (h2o["norb"], h2o["nelec"], h2o["ms2"]) == (ref["norb"], ref["nelec"], ref["ms2"])
    assert abs(h2o["E_core"] - ref["E_core"]) < tol
    assert abs(h2o["T"].sum() - ref["T_sum"]) < tol
    assert abs(h2o["V"].sum() - ref["V_sum"]) < tol
    n, no = ref["norb"], ref["nocc"]
    Fi = oracle.mcscf_fock(h2o["T"], h2o["V"], no, 0)[0]
    eps = np.diag(Fi)
    np.testing.assert_allclose(eps, ref["eps"], atol=tol, rtol=0)
    V = h2o["V"]
    o, v = slice(0, no), slice(no, n)
    dir_ = V[v, o, v, o]  # (ai|bj) as [a, i, b, j]
    exh = dir_.transpose(2, 1, 0, 3)  # (bi|aj)
    den = eps[v][:, None, None, None] + eps[v][None, None, :, None] - eps[o][None, :, None, None] \
        - eps[o][None, None, None, :]
    emp2 = -np.sum(dir_ * (2 * dir_ - exh) / den)
    assert abs(emp2 - ref["EMP2"]) < tol


def test_macis_wavefunction_files(pkg, tmp_path):
    """read_wavefunction / write_wavefunction (wavefunction_io.hpp:40-116) on
    the reference's O2 wavefunction (tests/golden/o2_wfn.npz holds its
    determinants and coefficients): written and read back exactly, with the
    reference's header and line layout."""
    det = pkg.determinants
    d = np.load(os.path.join(GOLDEN, "o2_wfn.npz"))
    p = tmp_path / "o2.wfn.dat"
    det.write_wavefunction(str(p), int(d["norb"]), d["alpha"], d["beta"], d["coeffs"])
    lines = p.read_text().splitlines()
    assert lines[0] == "%d %d %d %d" % (len(d["coeffs"]), int(d["norb"]), int(d["nalpha"]), int(d["nbeta"]))
    assert len(lines[1]) == 30 + 1 + int(d["norb"]) + 1 and "e" in lines[1][:30]
    a, b, c, norb, na, nb = det.read_wavefunction(str(p))
    assert (norb, na, nb) == (int(d["norb"]), int(d["nalpha"]), int(d["nbeta"]))
    assert np.array_equal(a, d["alpha"]) and np.array_equal(b, d["beta"]) and np.array_equal(c, d["coeffs"])
    w = pkg.calculators.Wavefunction.from_macis_file(str(p))
    assert w.norb == int(d["norb"]) and np.array_equal(w.coefficients, d["coeffs"])
    w.to_macis_file(str(tmp_path / "again.dat"))
    assert (tmp_path / "again.dat").read_text() == p.read_text()
    # wavefunction_io.hpp:99-102: unequal lengths throw, an empty wavefunction writes nothing
    with pytest.raises(RuntimeError, match="Invalid Wave Function Dimensions"):
        det.write_wavefunction(str(tmp_path / "bad.dat"), 4, d["alpha"][:3], d["beta"][:3], d["coeffs"][:2])
    det.write_wavefunction(str(tmp_path / "empty.dat"), 4, [], [], [])
    assert not (tmp_path / "empty.dat").exists() and not (tmp_path / "bad.dat").exists()


def test_macis_rdm_files(pkg, tmp_path):
    """read_rdms_binary / write_rdms_binary (fcidump.cxx:486-558) on the
    reference's water CAS(8e,8o) RDMs (tests/golden/h2o_ccpvdz_cas88_rdms.npz):
    the file is an int32 norb and the column-major RDMs; written and read back
    exactly; a wrong norb is refused."""
    ints = pkg.integrals
    d = np.load(os.path.join(GOLDEN, "h2o_ccpvdz_cas88_rdms.npz"))
    n = int(d["nact"])
    g0, G0 = d["ordm"].reshape(n, n, order="F"), d["trdm"].reshape((n,) * 4, order="F")
    p = tmp_path / "rdms.bin"
    ints.write_rdms_binary(str(p), g0, G0)
    raw = p.read_bytes()
    assert len(raw) == 4 + 8 * (n ** 2 + n ** 4)
    assert raw[:4] == np.array([n], np.int32).tobytes() and raw[4:4 + 8 * n * n] == d["ordm"].tobytes()
    g, G = ints.read_rdms_binary(str(p), n)
    assert np.array_equal(g, g0) and np.array_equal(G, G0)
    with pytest.raises(RuntimeError, match="NORB"):
        ints.read_rdms_binary(str(p), n + 1)
