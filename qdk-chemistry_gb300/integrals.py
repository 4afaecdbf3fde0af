"""Integral inputs for the CI path: seeded synthetic integrals and FCIDUMP I/O.

Layout convention (the one MACIS reads, ``include/macis/types.hpp:33-56``):
``T[p, q]`` and ``V[p, q, r, s]`` are returned as numpy arrays whose
*column-major* flattening is the buffer handed to the library
(``V(p,q,r,s) = buf[p + n q + n^2 r + n^3 s]``).  Because every integral set
produced here is exactly 8-fold symmetric, the row-major buffer qdk stores
(``canonical_four_center.cpp:148-153``) is bit-identical to it.
"""
import re

import numpy as np


def _sym_pair_index(n):
    p, q = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    return np.maximum(p, q) * n + np.minimum(p, q)


def symmetrize_eri(M, n):
    """Exact 8-fold symmetrisation of an (n^2 x n^2) matrix M[pq, rs]: every
    element takes the value of its canonical representative, so V(pq|rs),
    V(qp|rs), V(rs|pq), ... are bitwise equal."""
    idx = _sym_pair_index(n).ravel()
    Mc = M[np.ix_(idx, idx)]
    a = idx[:, None]
    b = idx[None, :]
    Mc = np.where(a >= b, Mc, Mc.T)
    return Mc.reshape(n, n, n, n)


def synthetic_integrals(norb, n_chol, seed, diag_spacing=0.25, offdiag_sigma=0.05, chol_sigma=0.1):
    """Seeded synthetic real integrals (PCG64 via numpy.default_rng).

    h1 = diag(-2.0 + diag_spacing * p) + symmetric off-diagonal N(0, offdiag_sigma^2);
    V_pqrs = sum_Q L_Q,pq L_Q,rs over ``n_chol`` symmetric L_Q with entries
    N(0, chol_sigma^2).  V is positive semi-definite as an (pq, rs) matrix and
    exactly 8-fold symmetric.  Core energy is 0.
    Returns (T, V, E_core).
    """
    n = int(norb)
    rng = np.random.default_rng(seed)
    off = np.triu(rng.normal(0.0, offdiag_sigma, (n, n)), 1)
    T = off + off.T + np.diag(-2.0 + diag_spacing * np.arange(n))
    L = rng.normal(0.0, chol_sigma, (n_chol, n, n))
    L = np.triu(L) + np.transpose(np.triu(L, 1), (0, 2, 1))
    Lm = L.reshape(n_chol, n * n)
    M = Lm.T @ Lm
    V = symmetrize_eri(M, n)
    return np.ascontiguousarray(T), np.ascontiguousarray(V), 0.0


# ----------------------------------------------------------------- FCIDUMP
def read_fcidump(path_or_text, is_text=False):
    """Parse an FCIDUMP file.

    Follows MACIS's reader (``src/macis/fcidump.cxx``): header up to ``&END``;
    every later line is ``value p q r s`` (1-based); all four indices non-zero
    is a two-body line expanded over the 8 index permutations (``:420-428``),
    all zero is the core energy, anything else a one-body line stored at
    T(p,q) and T(q,p) (``:345-350``).
    Returns dict(norb, nelec, ms2, T, V, E_core).
    """
    text = path_or_text if is_text else open(path_or_text).read()
    m = re.search(r"&END|^\s*/\s*$", text, re.M | re.I)
    if m is None:
        raise ValueError("FCIDUMP header terminator (&END) not found")
    head, body = text[:m.start()], text[m.end():]
    hdr = {}
    for key in ("NORB", "NELEC", "MS2"):
        m = re.search(key + r"\s*=\s*(-?\d+)", head, re.IGNORECASE)
        if m:
            hdr[key] = int(m.group(1))
    rows = np.loadtxt(body.splitlines(), ndmin=2)
    vals = rows[:, 0]
    idx = rows[:, 1:5].astype(np.int64)
    return integrals_from_lines(hdr["NORB"], idx, vals, hdr.get("NELEC"), hdr.get("MS2", 0))


def integrals_from_lines(norb, idx, vals, nelec=None, ms2=0):
    """Dense T, V from FCIDUMP lines (idx: [L,4] 1-based, vals: [L])."""
    n = int(norb)
    T = np.zeros((n, n))
    V = np.zeros((n, n, n, n))
    E_core = 0.0
    idx = np.asarray(idx, dtype=np.int64)
    vals = np.asarray(vals, dtype=np.float64)
    two = np.all(idx != 0, axis=1)
    core = np.all(idx == 0, axis=1)
    one = ~two & ~core
    # lines are applied in file order, as the reference reader does
    for (p, q, r, s), v in zip(idx[two] - 1, vals[two]):
        V[p, q, r, s] = V[p, q, s, r] = V[q, p, r, s] = V[q, p, s, r] = v
        V[r, s, p, q] = V[s, r, p, q] = V[r, s, q, p] = V[s, r, q, p] = v
    for (p, q), v in zip(idx[one][:, :2] - 1, vals[one]):
        T[p, q] = T[q, p] = v
    if np.any(core):
        E_core = float(vals[core][-1])
    return dict(norb=n, nelec=nelec, ms2=ms2, T=T, V=V, E_core=E_core)


def write_fcidump(path, T, V, E_core=0.0, nelec=0, ms2=0, thresh=1e-16):
    """Write an FCIDUMP with the canonical (8-fold unique) two-body lines."""
    n = T.shape[0]
    lines = ["&FCI NORB=%d, NELEC=%d, MS2=%d," % (n, nelec, ms2),
             "ORBSYM=" + ",".join(["1"] * n) + ",", "ISYM=1,", "&END"]
    for p in range(n):
        for q in range(p + 1):
            for r in range(n):
                for s in range(r + 1):
                    if p * n + q < r * n + s:
                        continue
                    v = V[p, q, r, s]
                    if abs(v) > thresh:
                        lines.append("%.16e %d %d %d %d" % (v, p + 1, q + 1, r + 1, s + 1))
    for p in range(n):
        for q in range(p + 1):
            if abs(T[p, q]) > thresh:
                lines.append("%.16e %d %d 0 0" % (T[p, q], p + 1, q + 1))
    lines.append("%.16e 0 0 0 0" % E_core)
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def read_rdms_binary(path, norb=None):
    """read_rdms_binary (src/macis/fcidump.cxx:486-530): an int norb, then the
    column-major 1-RDM (norb^2 doubles) and 2-RDM (norb^4 doubles).  Returns
    (1-RDM [p, q], 2-RDM [p, q, r, s]) indexed as MACIS's (p, q) / (p, q, r, s);
    a norb that differs from the file's raises RuntimeError."""
    raw = open(path, "rb").read()
    n = int(np.frombuffer(raw[:4], dtype=np.int32)[0])
    if norb is not None and n != int(norb):
        raise RuntimeError("NORB in RDM file doesn't match %d %d" % (int(norb), n))
    vals = np.frombuffer(raw[4:], dtype=np.float64)
    if len(vals) < n * n + n ** 4:
        raise ValueError("RDM file holds %d values, %d expected" % (len(vals), n * n + n ** 4))
    g = vals[:n * n].reshape((n, n), order="F").copy()
    G = vals[n * n:n * n + n ** 4].reshape((n,) * 4, order="F").copy()
    return g, G


def write_rdms_binary(path, ordm, trdm):
    """write_rdms_binary (src/macis/fcidump.cxx:532-558): the layout
    read_rdms_binary reads."""
    g = np.asarray(ordm, dtype=np.float64)
    n = g.shape[0]
    G = np.asarray(trdm, dtype=np.float64).reshape((n,) * 4)
    with open(path, "wb") as f:
        f.write(np.array([n], dtype=np.int32).tobytes())
        f.write(g.ravel(order="F").tobytes())
        f.write(G.ravel(order="F").tobytes())
