"""Determinant lists in MACIS order, as (alpha, beta) uint64 spin-string pairs.

MACIS stores a determinant as ``std::bitset<N>`` with the alpha string in the
low N/2 bits and the beta string in the high N/2 bits
(``include/macis/wfn/raw_bitset.hpp:55-106``).  This library keeps the two
spin strings as separate uint64 arrays (bit i = spatial orbital i), which
covers every ``wfn_t<N>`` up to N = 128 (64 orbitals per spin).
"""
import itertools

import numpy as np


def combs(nbits, nset):
    """generate_combs (``include/macis/sd_operations.hpp:305-323``): strings of
    ``nset`` bits out of ``nbits`` in std::prev_permutation order, starting
    from the lowest orbitals.  Equivalent order: lexicographically descending
    occupation vectors v[0..nbits), i.e. combinations of positions in
    lexicographic order."""
    out = []
    for pos in itertools.combinations(range(nbits), nset):
        s = 0
        for p in pos:
            s |= 1 << p
        out.append(s)
    return np.array(out, dtype=np.uint64)


def fci_space(norb, na, nb):
    """generate_hilbert_space (``sd_operations.hpp:333-351``): alpha-major
    product of the alpha and beta string lists."""
    a = combs(norb, na)
    b = combs(norb, nb)
    return np.repeat(a, len(b)), np.tile(b, len(a))


def canonical_hf(na, nb):
    """canonical_hf_determinant (``raw_bitset.hpp:183-188``)."""
    return np.uint64((1 << na) - 1), np.uint64((1 << nb) - 1)


def _occ_vir(norb, s):
    occ = [i for i in range(norb) if (s >> i) & 1]
    vir = [i for i in range(norb) if not (s >> i) & 1]
    return occ, vir


def _singles(norb, s):
    # append_singles (sd_operations.hpp:60-77): virtual outer, occupied inner
    occ, vir = _occ_vir(norb, s)
    return [(s ^ (1 << o)) | (1 << v) for v in vir for o in occ]


def _doubles(norb, s):
    # append_doubles (sd_operations.hpp:89-110): a < b virtual, i < j occupied
    occ, vir = _occ_vir(norb, s)
    out = []
    for ia, a in enumerate(vir):
        for i_, i in enumerate(occ):
            for b in vir[ia + 1:]:
                for j in occ[i_ + 1:]:
                    out.append((s ^ (1 << i) ^ (1 << j)) | (1 << a) | (1 << b))
    return out


def cisd_space(norb, ref_alpha, ref_beta):
    """generate_cisd_hilbert_space (``sd_operations.hpp:265-275`` with
    generate_singles_doubles_spin ``:213-262``): reference, alpha singles,
    beta singles, alpha doubles, beta doubles, alpha x beta singles."""
    a, b = int(ref_alpha), int(ref_beta)
    sa, sb = _singles(norb, a), _singles(norb, b)
    da, db = _doubles(norb, a), _doubles(norb, b)
    dets = [(a, b)]
    dets += [(x, b) for x in sa]
    dets += [(a, y) for y in sb]
    dets += [(x, b) for x in da]
    dets += [(a, y) for y in db]
    dets += [(x, y) for x in sa for y in sb]
    arr = np.array(dets, dtype=np.uint64)
    return arr[:, 0].copy(), arr[:, 1].copy()


def spin_sort(alpha, beta):
    """std::sort by spin_comparator (``raw_bitset.hpp:119-141``): alpha string
    first, then beta, both compared as unsigned integers."""
    order = np.lexsort((beta, alpha))
    return alpha[order], beta[order]


def to_canonical_string(alpha, beta, norb):
    """'2' doubly occupied, 'u' alpha only, 'd' beta only, '0' empty
    (``sd_operations.hpp:480-510``)."""
    out = []
    for i in range(norb):
        ua, ub = (int(alpha) >> i) & 1, (int(beta) >> i) & 1
        out.append("2" if ua and ub else "u" if ua else "d" if ub else "0")
    return "".join(out)


def from_canonical_string(s):
    a = b = 0
    for i, ch in enumerate(s):
        if ch in "2u":
            a |= 1 << i
        if ch in "2d":
            b |= 1 << i
    return np.uint64(a), np.uint64(b)


def read_wavefunction(path):
    """read_wavefunction (include/macis/wavefunction_io.hpp:40-93): the
    header "nstates norb nalpha nbeta", then one "coefficient canonical-string"
    line per determinant.  Returns (alpha, beta, coeffs, norb, nalpha, nbeta)."""
    with open(path) as f:
        head = f.readline().split()
        if len(head) < 4:
            raise ValueError("wavefunction file header must hold nstates norb nalpha nbeta")
        _, norb, na, nb = (int(x) for x in head[:4])
        a, b, c = [], [], []
        for line in f:
            parts = line.split()
            if not parts:
                continue
            x, y = from_canonical_string(parts[1])
            a.append(x)
            b.append(y)
            c.append(float(parts[0]))
    return (np.array(a, dtype=np.uint64), np.array(b, dtype=np.uint64), np.array(c, dtype=np.float64), norb, na,
            nb)


def write_wavefunction(path, norb, alpha, beta, coeffs):
    """write_wavefunction (wavefunction_io.hpp:95-116): unequal determinant and
    coefficient counts raise "Invalid Wave Function Dimensions", an empty
    wavefunction writes no file; otherwise the header from the
    first determinant's electron counts, then each coefficient in scientific
    notation with 16 digits (30 wide) and the determinant's canonical string."""
    alpha = np.asarray(alpha, dtype=np.uint64)
    beta = np.asarray(beta, dtype=np.uint64)
    coeffs = np.asarray(coeffs, dtype=np.float64)
    if not (len(alpha) == len(beta) == len(coeffs)):
        raise RuntimeError("Invalid Wave Function Dimensions")
    if len(alpha) == 0:
        return  # the reference writes nothing (not even a header) for an empty wavefunction
    with open(path, "w") as f:
        f.write("%d %d %d %d\n" % (len(coeffs), norb, int(alpha[0]).bit_count(), int(beta[0]).bit_count()))
        for x, y, c in zip(alpha, beta, coeffs):
            f.write("%30.16e %s \n" % (c, to_canonical_string(x, y, norb)))
