"""Regenerate the golden fixtures in this folder from the reference checkout.

Run where the reference checkout exists, giving its path:

    python tests/golden/make_golden.py REFERENCE_CHECKOUT

It copies the reference's own test inputs and known answers for the CI hot
path into compact numpy files, so that the tests never read the reference at
run time:

* FCIDUMP integral lines (index quadruples + values) of
  - external/macis/tests/ref_data/h2o.ccpvdz.fci.dat (water cc-pVDZ, 24 orbitals)
  - external/macis/python/tests/data/n2_selected_6e6o.hamiltonian.fcidump
  - external/macis/python/tests/data/n2_full_14e18o.hamiltonian.fcidump
* the CSR row-pointer golden of the water CISD Hamiltonian
  (external/macis/tests/ref_data/h2o.ccpvdz.cisd.rowptr.bin, int32)
* the O2 CI wavefunction external/macis/tests/ref_data/o2.wfn.dat
* the water CAS(8e,8o) active RDMs external/macis/tests/ref_data/
  h2o.ccpvdz.cas88.rdms.bin (int32 norb, then the column-major 1-RDM and
  2-RDM; read_rdms_binary, src/macis/fcidump.cxx:487-527)
* known_answers.json: the energies / sums the reference tests pin, with the
  file:line each one comes from;
* sd_operations.json: the determinant lists of external/macis/tests/
  sd_operations.cxx (singles, doubles and the FCI space of small strings, in
  MACIS's packed wfn_t<64> form: alpha in bits 0-31, beta in bits 32-63).
"""
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def parse_fcidump_lines(path):
    text = open(path).read()
    m = re.search(r"&END|^\s*/\s*$", text, re.M | re.I)
    head, body = text[:m.start()], text[m.end():]
    hdr = {k: int(re.search(k + r"\s*=\s*(-?\d+)", head, re.I).group(1)) for k in ("NORB", "NELEC")}
    ms2 = re.search(r"MS2\s*=\s*(-?\d+)", head, re.I)
    rows = np.loadtxt(body.splitlines(), ndmin=2)
    return dict(norb=hdr["NORB"], nelec=hdr["NELEC"], ms2=int(ms2.group(1)) if ms2 else 0,
                idx=rows[:, 1:5].astype(np.int8), vals=rows[:, 0].astype(np.float64))


def parse_wfn_list(text, anchor, name):
    """The integer list ``name = { ... };`` that follows ``anchor`` in a C++
    test source (hex and 0b literals)."""
    start = text.index(anchor)
    m = re.search(re.escape(name) + r"\s*=\s*\{(.*?)\};", text[start:], re.S)
    return [int(tok, 0) for tok in re.findall(r"0[xXbB][0-9a-fA-F]+", m.group(1))]


def main(ref):
    macis = os.path.join(ref, "external", "macis")
    dumps = {
        "h2o_ccpvdz": os.path.join(macis, "tests", "ref_data", "h2o.ccpvdz.fci.dat"),
        "n2_6e6o": os.path.join(macis, "python", "tests", "data", "n2_selected_6e6o.hamiltonian.fcidump"),
        "n2_14e18o": os.path.join(macis, "python", "tests", "data", "n2_full_14e18o.hamiltonian.fcidump"),
    }
    for name, path in dumps.items():
        d = parse_fcidump_lines(path)
        np.savez_compressed(os.path.join(HERE, name + "_fcidump.npz"), **d)

    rp = np.fromfile(os.path.join(macis, "tests", "ref_data", "h2o.ccpvdz.cisd.rowptr.bin"), dtype=np.int32)
    np.save(os.path.join(HERE, "h2o_ccpvdz_cisd_rowptr.npy"), rp)

    lines = open(os.path.join(macis, "tests", "ref_data", "o2.wfn.dat")).read().splitlines()
    nstate, norb, na, nb = (int(x) for x in lines[0].split())
    coeffs, strs = [], []
    for ln in lines[1:]:
        if ln.strip():
            c, s = ln.split()
            coeffs.append(float(c))
            strs.append(s)
    alpha = np.array([sum(1 << i for i, ch in enumerate(s) if ch in "2u") for s in strs], dtype=np.uint64)
    beta = np.array([sum(1 << i for i, ch in enumerate(s) if ch in "2d") for s in strs], dtype=np.uint64)
    np.savez_compressed(os.path.join(HERE, "o2_wfn.npz"), alpha=alpha, beta=beta, coeffs=np.array(coeffs),
                        norb=norb, nalpha=na, nbeta=nb)

    raw = open(os.path.join(macis, "tests", "ref_data", "h2o.ccpvdz.cas88.rdms.bin"), "rb").read()
    nact = int(np.frombuffer(raw[:4], dtype=np.int32)[0])
    vals = np.frombuffer(raw[4:], dtype=np.float64)
    np.savez_compressed(os.path.join(HERE, "h2o_ccpvdz_cas88_rdms.npz"), nact=nact,
                        ordm=vals[:nact ** 2].copy(), trdm=vals[nact ** 2:nact ** 2 + nact ** 4].copy())

    sd = open(os.path.join(macis, "tests", "sd_operations.cxx")).read()
    sd_lists = {
        "singles_single_spin": parse_wfn_list(sd, 'SECTION("Singles")', "ref_singles"),
        "singles_both_spins": parse_wfn_list(sd, 'SECTION("Both Spin")', "ref_singles"),
        "doubles_single_spin": parse_wfn_list(sd, 'SECTION("Doubles")', "ref_doubles"),
        "doubles_both_spins": parse_wfn_list(sd, 'SECTION("Both Spins")', "ref_doubles"),
        "fci_combs_4_2": parse_wfn_list(sd, 'SECTION("FCI")', "ref_combs"),
        "fci_space_4_2_2": parse_wfn_list(sd, 'SECTION("FCI")', "ref_dets"),
        "source": "external/macis/tests/sd_operations.cxx:45-249",
    }
    with open(os.path.join(HERE, "sd_operations.json"), "w") as f:
        json.dump(sd_lists, f, indent=0)

    known = {
        "h2o_cisd_csr": {"n": 12636, "nnz": 3517816, "thresh": 1e-16,
                         "source": "external/macis/tests/csr_hamiltonian.cxx:46-77"},
        "h2o_cisd_davidson": {"E0_total": -7.623197835987e01, "max_m": 15, "tol": 1e-8, "atol": 1e-8,
                              "source": "external/macis/tests/davidson.cxx:44-58"},
        "n2_6e6o_casci": {"E_total": -9.155573e00, "ndets": 400, "nalpha": 3, "nbeta": 3,
                          "source": "external/macis/python/tests/test_pymacis.py:114-142"},
        "n2_14e18o_asci": {"E_total": -1.205187165264e02, "ndets": 2000, "grow_factor": 2,
                           "ntdets_max": 2000, "max_refine_iter": 15, "max_subspace": 1000,
                           "source": "external/macis/python/tests/test_pymacis.py:158-187"},
        "h2o_asci_10k": {"E0_grow": -8.542926580489e01, "E0_refine": -8.542926585527e01, "ntdets_max": 10000,
                         "EPT2": -5.701535028967e-03, "atol": 1e-8,
                         "source": "external/macis/tests/asci.cxx:488-574 (EPT2: :556-570)"},
        "h2o_casscf": {"E_total": -7.61114493227e01, "ninact": 1, "nact": 8, "nalpha": 4, "nbeta": 4, "atol": 1e-8,
                       "source": "external/macis/tests/mcscf.cxx:26-66"},
        "h2o_fock_matrices": {
            "inactive_sums": [
                -1.0954327626528054e+02, -7.9049334675325397e+01, -5.5421794916425746e+01, -3.2896413433510098e+01,
                -9.6790625410977995e+00, 1.3541890926738670e+01, 2.8118988584004747e+01, 4.2282474623774370e+01,
                6.1330877241905775e+01, 8.0462280904553381e+01, 1.0115739942244966e+02, 1.2234906887017347e+02,
                1.4193737383338043e+02, 1.6158815460036422e+02, 1.8055391956530423e+02, 1.9946376174456546e+02,
                2.2023047024882104e+02, 2.3908456464316561e+02, 2.6013779050396846e+02, 2.8151944194600628e+02,
                3.0499216988942629e+02, 3.2832856341497029e+02, 3.5190406182710450e+02, 3.7494850617879558e+02],
            "inactive_energies": [
                0.0000000000000000e+00, -6.1315494224913593e+01, -7.2212778636226929e+01, -7.9040381402513631e+01,
                -8.3471297093533877e+01, -8.5217981091537155e+01, -8.4546001263510988e+01, -8.2730095439120404e+01,
                -7.8127776664404351e+01, -7.1592548154010231e+01, -6.2930084392284229e+01, -5.2096342927325999e+01,
                -3.9855391765969998e+01, -2.5412026151032496e+01, -8.6447385900261242e+00, 9.9027251048627019e+00,
                3.0946082901947307e+01, 5.3450370843339400e+01, 8.0911983168177073e+01, 1.1078946373217127e+02,
                1.4537422212238749e+02, 1.8291223010717863e+02, 2.2328918072756994e+02, 2.6673925924545023e+02],
            "ninact": 1, "nact": 8, "active_fock_sum": 9.2434393637673907e+01, "aux_q_sum": 2.609524939005e+01,
            "generalized_fock_sum": -4.7465630072124384e+01, "E_from_generalized_fock": -8.5250440649419417e+01,
            "atol": 1e-6, "source": "external/macis/tests/fock_matrices.cxx:26-256"},
        "h2o_fcidump": {
            "norb": 24, "nelec": 10, "ms2": 0, "E_core": 9.191200742618042, "T_sum": -1.095432762653e+02,
            "V_sum": 2.701609068389e+02, "nocc": 5,
            "eps": [-20.5504959651472, -1.33652308180416, -0.699084807015877, -0.566535827115135,
                    -0.493126779151562, 0.185508268977809, 0.25620321890592, 0.78902083505165,
                    0.854064342891826, 1.16354210561965, 1.20037835222836, 1.25333579878846,
                    1.44452900701373, 1.4762147730592, 1.67453827449385, 1.86734472965445,
                    1.93460967763627, 2.4520550848955, 2.48955724627828, 3.28543361094139,
                    3.33853354817945, 3.5101570353257, 3.86543012937399, 4.14719831587618],
            "EMP2": -0.203989305096243, "atol": 1e-6, "source": "external/macis/tests/fcidump.cxx:18-112"},
        "h2o_double_loop": {"E_HF_total": -76.0267803489191, "E_single_diag": -6.488097259228e+01,
                            "E_double_ss_diag": -6.314093508151e+01, "E_double_os_diag": -6.304547887231e+01,
                            "EMP2": -0.203989305096243, "atol": 1e-6,
                            "source": "external/macis/tests/double_loop.cxx:22-241"},
        "o2_rdms": {"n_dets_padded": 5000, "sum_abs_ordm": 8.0000005763, "sum_abs_trdm": 44.1092472977,
                    "atol": 1e-6, "source": "external/macis/tests/double_loop.cxx:506-579"},
    }
    with open(os.path.join(HERE, "known_answers.json"), "w") as f:
        json.dump(known, f, indent=1)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(__doc__)
    main(sys.argv[1])
