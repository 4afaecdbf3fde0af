"""ctypes binding of the CPU oracle (test infrastructure only; see __init__)."""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "macis_oracle.cpp")
_OUT_DIR = os.path.join(_HERE, "_build")
_LIB_PATH = os.path.join(_OUT_DIR, "libmacis_oracle.so")
_lib = None

_u64p = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")


def build(force=False):
    """Compile the oracle with g++ (OpenMP, no FMA contraction)."""
    os.makedirs(_OUT_DIR, exist_ok=True)
    if (not force and os.path.exists(_LIB_PATH)
            and os.path.getmtime(_LIB_PATH) >= os.path.getmtime(_SRC)):
        return _LIB_PATH
    cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-fPIC", "-shared",
           "-ffp-contract=off", _SRC, "-o", _LIB_PATH + ".tmp"]
    subprocess.check_call(cmd)
    os.replace(_LIB_PATH + ".tmp", _LIB_PATH)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        vp, i64, f64, ci = ctypes.c_void_p, ctypes.c_int64, ctypes.c_double, ctypes.c_int
        L.orc_last_error.restype = ctypes.c_char_p
        L.orc_num_threads.restype = ci
        L.orc_combs.restype = i64
        L.orc_combs.argtypes = [ci, ci, ctypes.c_void_p]
        L.orc_ham_create.restype = vp
        L.orc_ham_create.argtypes = [ci, _f64p, _f64p]
        L.orc_ham_destroy.argtypes = [vp]
        L.orc_ham_intermediates.argtypes = [vp, _f64p, _f64p, _f64p, _f64p]
        L.orc_matrix_element.restype = f64
        L.orc_matrix_element.argtypes = [vp, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64]
        L.orc_csr_build.restype = vp
        L.orc_csr_build.argtypes = [vp, _u64p, _u64p, i64, f64]
        L.orc_csr_from_arrays.restype = vp
        L.orc_csr_from_arrays.argtypes = [i64, _i64p, _i64p, _f64p]
        L.orc_csr_nnz.restype = i64
        L.orc_csr_nnz.argtypes = [vp]
        L.orc_csr_copy.argtypes = [vp, _i64p, _i64p, _f64p]
        L.orc_csr_destroy.argtypes = [vp]
        L.orc_csr_spmv.argtypes = [vp, _f64p, _f64p]
        L.orc_csr_diag.argtypes = [vp, _f64p]
        L.orc_selected_ci_diag.restype = ci
        L.orc_selected_ci_diag.argtypes = [vp, i64, f64, _f64p, ctypes.POINTER(f64), ctypes.POINTER(i64)]
        L.orc_syev.argtypes = [ci, _f64p, _f64p]
        L.orc_rdms_spin_dep.argtypes = [ci, _u64p, _u64p, i64, _f64p] + [ctypes.c_void_p] * 5
        L.orc_sdl_sample.restype = i64
        L.orc_sdl_sample.argtypes = [vp, _u64p, _u64p, i64, f64, i64, i64]
        L.orc_csr_build_rows.restype = vp
        L.orc_csr_build_rows.argtypes = [vp, _u64p, _u64p, i64, f64, i64, i64]
        L.orc_csr_spmv_block.argtypes = [vp, _f64p, _f64p]
        L.orc_asci.restype = i64
        L.orc_asci.argtypes = [vp, _f64p, i64, _u64p, _u64p, _f64p, f64, ci, ci, i64, _u64p, _u64p, _f64p,
                               ctypes.POINTER(f64), ctypes.POINTER(f64), ctypes.c_void_p]
        L.orc_asci_grow_requests.restype = i64
        L.orc_asci_grow_requests.argtypes = [vp, _f64p, i64, _u64p, _u64p, _f64p, f64, i64, _i64p]
        L.orc_asci_iter.restype = i64
        L.orc_asci_iter.argtypes = [vp, _f64p, i64, _u64p, _u64p, _f64p, f64, i64, i64, _u64p, _u64p, _f64p,
                                    ctypes.POINTER(f64)]
        L.orc_asci_search.restype = i64
        L.orc_asci_search.argtypes = [vp, _f64p, i64, _u64p, _u64p, _f64p, f64, i64, i64, _u64p, _u64p]
        L.orc_mcscf_fock.restype = None
        L.orc_mcscf_fock.argtypes = [ci, ci, ci, _f64p, _f64p, _f64p, _f64p, _f64p, _f64p, _f64p, _f64p,
                                     ctypes.POINTER(f64), ctypes.POINTER(f64)]
        L.orc_casscf.restype = ci
        L.orc_casscf.argtypes = [_f64p, ci, ci, ci, ci, ci, f64, _f64p, _f64p, _f64p, _f64p, ctypes.POINTER(f64),
                                 ctypes.POINTER(i64), ctypes.POINTER(ci)]
        L.orc_entropies.restype = ci
        L.orc_entropies.argtypes = [ci, _u64p, _u64p, i64, _f64p, _f64p, _f64p, _f64p]
        L.orc_asci_pt2.restype = ci
        L.orc_asci_pt2.argtypes = [vp, i64, _u64p, _u64p, _f64p, f64, f64, i64, ctypes.POINTER(f64),
                                   ctypes.POINTER(i64)]
        _lib = L
    return _lib


def num_threads():
    return lib().orc_num_threads()


def combs(nbits, nset):
    """generate_combs order (prev_permutation from the lowest orbitals)."""
    L = lib()
    cnt = L.orc_combs(nbits, nset, None)
    out = np.zeros(cnt, dtype=np.uint64)
    L.orc_combs(nbits, nset, out.ctypes.data)
    return out


def fci_dets(norb, na, nb):
    """generate_hilbert_space: alpha-major product of the two string lists."""
    a = combs(norb, na)
    b = combs(norb, nb)
    return np.repeat(a, len(b)), np.tile(b, len(a))


class Hamiltonian:
    """Integrals + MACIS intermediates (HamiltonianGeneratorBase)."""

    def __init__(self, T, V):
        self.n = int(T.shape[0])
        # column-major buffers as MACIS reads them
        self._T = np.ascontiguousarray(np.asarray(T, dtype=np.float64).ravel(order="F"))
        self._V = np.ascontiguousarray(np.asarray(V, dtype=np.float64).ravel(order="F"))
        self._h = lib().orc_ham_create(self.n, self._T, self._V)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_ham_destroy(self._h)
            self._h = None

    def intermediates(self):
        n = self.n
        G = np.zeros(n ** 3)
        Vr = np.zeros(n ** 3)
        G2 = np.zeros(n ** 2)
        V2 = np.zeros(n ** 2)
        lib().orc_ham_intermediates(self._h, G, Vr, G2, V2)
        return G, Vr, G2, V2

    def matrix_element(self, bra, ket):
        return lib().orc_matrix_element(self._h, int(bra[0]), int(bra[1]), int(ket[0]), int(ket[1]))


class Csr:
    def __init__(self, handle, n):
        self._m = handle
        self.n = n

    def __del__(self):
        if getattr(self, "_m", None):
            lib().orc_csr_destroy(self._m)
            self._m = None

    @property
    def nnz(self):
        return lib().orc_csr_nnz(self._m)

    def arrays(self):
        nnz = self.nnz
        rp = np.zeros(self.n + 1, dtype=np.int64)
        ci = np.zeros(nnz, dtype=np.int64)
        nz = np.zeros(nnz, dtype=np.float64)
        lib().orc_csr_copy(self._m, rp, ci, nz)
        return rp, ci, nz

    def spmv(self, x):
        y = np.zeros(self.n)
        lib().orc_csr_spmv(self._m, np.ascontiguousarray(x, dtype=np.float64), y)
        return y

    def diag(self):
        d = np.zeros(self.n)
        lib().orc_csr_diag(self._m, d)
        return d

    def selected_ci_diag(self, max_m=200, tol=1e-8, X=None):
        """Returns (E, X, iterations); raises on non-convergence."""
        X = np.zeros(self.n) if X is None else np.array(X, dtype=np.float64)
        E = ctypes.c_double()
        it = ctypes.c_int64()
        rc = lib().orc_selected_ci_diag(self._m, max_m, tol, X, ctypes.byref(E), ctypes.byref(it))
        if rc == 1:
            raise RuntimeError("Davidson Did Not Converge!")
        if rc != 0:
            raise RuntimeError(lib().orc_last_error().decode())
        return E.value, X, it.value


def csr_from_arrays(rowptr, colind, values):
    """A caller's CSR matrix as an oracle operator (davidson_solver.cpp:60-64);
    its selected_ci_diag() is davidson_solver's diagonal guess + davidson."""
    rp = np.ascontiguousarray(rowptr, dtype=np.int64)
    ci = np.ascontiguousarray(colind, dtype=np.int64)
    nz = np.ascontiguousarray(values, dtype=np.float64)
    n = len(rp) - 1
    return Csr(lib().orc_csr_from_arrays(n, rp, ci, nz), n)


def build_csr(ham, alpha, beta, thresh=np.finfo(np.float64).eps):
    alpha = np.ascontiguousarray(alpha, dtype=np.uint64)
    beta = np.ascontiguousarray(beta, dtype=np.uint64)
    h = lib().orc_csr_build(ham._h, alpha, beta, len(alpha), float(thresh))
    if not h:
        raise RuntimeError(lib().orc_last_error().decode())
    return Csr(h, len(alpha))


def syev(A):
    A = np.array(A, dtype=np.float64, order="F")
    k = A.shape[0]
    buf = np.ascontiguousarray(A.ravel(order="F"))
    w = np.zeros(k)
    lib().orc_syev(k, buf, w)
    return w, buf.reshape((k, k), order="F")


def rdms_spin_dep(norb, alpha, beta, C, want=("aa", "bb", "aaaa", "bbbb", "aabb")):
    """form_rdms_spin_dep: returns dict of column-major-filled arrays shaped
    (n,n) / (n,n,n,n) indexed as [p,q] / [p,q,r,s] = MACIS (p,q,r,s)."""
    n = norb
    out = {}
    ptrs = []
    for k in ("aa", "bb", "aaaa", "bbbb", "aabb"):
        if k in want:
            buf = np.zeros(n ** (2 if len(k) == 2 else 4))
            out[k] = buf
            ptrs.append(buf.ctypes.data)
        else:
            ptrs.append(None)
    lib().orc_rdms_spin_dep(n, np.ascontiguousarray(alpha, dtype=np.uint64),
                            np.ascontiguousarray(beta, dtype=np.uint64), len(alpha),
                            np.ascontiguousarray(C, dtype=np.float64), *ptrs)
    res = {}
    for k, buf in out.items():
        shape = (n, n) if len(k) == 2 else (n, n, n, n)
        res[k] = buf.reshape(shape, order="F")
    return res


def sdl_sample(ham, alpha, beta, thresh, stride, offset=0):
    """Reference SDL count+fill work for every stride-th bra alpha group
    (timing sample of the CPU H build).  Returns elements produced."""
    alpha = np.ascontiguousarray(alpha, dtype=np.uint64)
    beta = np.ascontiguousarray(beta, dtype=np.uint64)
    return lib().orc_sdl_sample(ham._h, alpha, beta, len(alpha), float(thresh), int(stride), int(offset))


class CsrRows(Csr):
    def spmv_block(self, x):
        y = np.zeros(self.n)
        lib().orc_csr_spmv_block(self._m, np.ascontiguousarray(x, dtype=np.float64), y)
        return y


def build_rows(ham, alpha, beta, r0, r1, thresh=np.finfo(np.float64).eps):
    """CSR rows [r0, r1) against all kets (reference non-symmetric SDL)."""
    alpha = np.ascontiguousarray(alpha, dtype=np.uint64)
    beta = np.ascontiguousarray(beta, dtype=np.uint64)
    h = lib().orc_csr_build_rows(ham._h, alpha, beta, len(alpha), float(thresh), int(r0), int(r1))
    if not h:
        raise RuntimeError(lib().orc_last_error().decode())
    return CsrRows(h, r1 - r0)


ASCI_DEFAULTS = dict(ntdets_max=100000, ntdets_min=100, ncdets_max=100, core_fixed=0, core_threshold=0.95,
                     h_el_tol=1e-8, rv_prune_tol=1e-8, grow_factor=8.0, min_grow_factor=1.01, backoff=0.5,
                     recovery=1.1, max_refine_iter=6, refine_energy_tol=1e-6, warm_start=1,
                     min_warm_start_overlap=0.5, ci_res_tol=1e-8, ci_max_subspace=200,
                     ci_matel_tol=float(np.finfo(np.float64).eps), taper_grow_factor=0.0, just_singles=0,
                     grow_with_rot=0, rot_size_start=1000)
_ASCI_ORDER = list(ASCI_DEFAULTS)


def _asci_settings(**kw):
    d = dict(ASCI_DEFAULTS)
    for k, v in kw.items():
        if k not in d:
            raise KeyError(k)
        d[k] = v
    return np.array([float(d[k]) for k in _ASCI_ORDER])


def asci(ham, alpha0, beta0, c0, E0, grow=True, refine=True, rotation=None, **settings):
    """asci_grow then asci_refine (MACIS semantics); returns
    (E, alpha, beta, C, E_after_grow).  With grow_with_rot the integrals are
    rotated to natural orbitals during the grow (on a copy: ham is left as
    it is); rotation, an n x n array when given, receives the accumulated
    rotation (the identity without one)."""
    s = _asci_settings(**settings)
    cap = int(max(s[0] * 4, 16))
    oa = np.zeros(cap, dtype=np.uint64)
    ob = np.zeros(cap, dtype=np.uint64)
    oc = np.zeros(cap)
    E = ctypes.c_double()
    Eg = ctypes.c_double()
    rot = np.zeros(ham.n * ham.n)
    n = lib().orc_asci(ham._h, s, len(alpha0), np.ascontiguousarray(alpha0, dtype=np.uint64),
                       np.ascontiguousarray(beta0, dtype=np.uint64), np.ascontiguousarray(c0, dtype=np.float64),
                       float(E0), int(grow), int(refine), cap, oa, ob, oc, ctypes.byref(E), ctypes.byref(Eg),
                       rot.ctypes.data)
    if n < 0:
        raise RuntimeError(lib().orc_last_error().decode())
    if rotation is not None:
        rotation[...] = rot.reshape((ham.n, ham.n), order="F")
    return E.value, oa[:n].copy(), ob[:n].copy(), oc[:n].copy(), Eg.value


def asci_grow_requests(ham, alpha0, beta0, c0, E0, **settings):
    """asci_grow alone; per asci_iter, (determinants requested, reached)."""
    s = _asci_settings(**settings)
    req = np.zeros(256, dtype=np.int64)
    n = lib().orc_asci_grow_requests(ham._h, s, len(alpha0), np.ascontiguousarray(alpha0, dtype=np.uint64),
                                     np.ascontiguousarray(beta0, dtype=np.uint64),
                                     np.ascontiguousarray(c0, dtype=np.float64), float(E0), len(req), req)
    if n < 0:
        raise RuntimeError(lib().orc_last_error().decode())
    r = req[:min(n, len(req))].tolist()
    return list(zip(r[0::2], r[1::2]))


def asci_iter(ham, alpha, beta, c, E0, ndets_max, **settings):
    """One asci_iter (iteration.hpp:50-226): search for up to ndets_max
    determinants around the core of (alpha, beta, c), then diagonalise;
    returns (E, alpha, beta, C)."""
    s = _asci_settings(**settings)
    cap = int(max(ndets_max * 4, len(alpha)) + 16)
    oa = np.zeros(cap, dtype=np.uint64)
    ob = np.zeros(cap, dtype=np.uint64)
    oc = np.zeros(cap)
    E = ctypes.c_double()
    n = lib().orc_asci_iter(ham._h, s, len(alpha), np.ascontiguousarray(alpha, dtype=np.uint64),
                            np.ascontiguousarray(beta, dtype=np.uint64), np.ascontiguousarray(c, dtype=np.float64),
                            float(E0), int(ndets_max), cap, oa, ob, oc, ctypes.byref(E))
    if n < 0:
        raise RuntimeError(lib().orc_last_error().decode())
    return E.value, oa[:n].copy(), ob[:n].copy(), oc[:n].copy()


def asci_search(ham, alpha, beta, c, E0, ndets_max, **settings):
    """One asci_search step on a core (sorted by spin_comparator)."""
    s = _asci_settings(**settings)
    cap = int(ndets_max * 4 + len(alpha) + 16)
    oa = np.zeros(cap, dtype=np.uint64)
    ob = np.zeros(cap, dtype=np.uint64)
    n = lib().orc_asci_search(ham._h, s, len(alpha), np.ascontiguousarray(alpha, dtype=np.uint64),
                              np.ascontiguousarray(beta, dtype=np.uint64), np.ascontiguousarray(c, dtype=np.float64),
                              float(E0), int(ndets_max), cap, oa, ob)
    if n < 0:
        raise RuntimeError(lib().orc_last_error().decode())
    return oa[:n].copy(), ob[:n].copy()


def asci_pt2(ham, alpha, beta, c, E0, pt2_tol=1e-16, pass_max=0):
    """asci_pt2_constraint (pt2.hpp:59-565) on a wavefunction sorted by
    spin_comparator; returns (E_PT2, number of external determinants)."""
    e = ctypes.c_double()
    npt = ctypes.c_int64()
    rc = lib().orc_asci_pt2(ham._h, len(alpha), np.ascontiguousarray(alpha, dtype=np.uint64),
                            np.ascontiguousarray(beta, dtype=np.uint64), np.ascontiguousarray(c, dtype=np.float64),
                            float(E0), float(pt2_tol), int(pass_max), ctypes.byref(e), ctypes.byref(npt))
    if rc != 0:
        raise RuntimeError(lib().orc_last_error().decode())
    return e.value, npt.value


def entropies(norb, alpha, beta, C):
    """form_entropies (sorted_double_loop.hpp:755-903, entropies.hpp):
    (single-orbital entropies (n), two-orbital entropies (n x n), mutual
    information (n x n))."""
    n = int(norb)
    s1 = np.zeros(n)
    s2 = np.zeros((n, n))
    mi = np.zeros((n, n))
    rc = lib().orc_entropies(n, np.ascontiguousarray(alpha, dtype=np.uint64), np.ascontiguousarray(beta, dtype=np.uint64),
                             len(alpha), np.ascontiguousarray(C, dtype=np.float64), s1, s2, mi)
    if rc != 0:
        raise RuntimeError(lib().orc_last_error().decode())
    return s1, s2, mi


MCSCF_DEFAULTS = dict(max_macro_iter=100, max_orbital_step=0.5, orb_grad_tol=5e-6, enable_diis=1, diis_start_iter=3,
                      diis_nkeep=10, ci_res_tol=1e-8, ci_max_subspace=200,
                      ci_matel_tol=float(np.finfo(np.float64).eps))


def casscf(T, V, E_core, nalpha, nbeta, ninact, nact, rdm1=None, rdm2=None, **settings):
    """casscf_diis (mcscf.hpp:54-60, mcscf_impl.hpp:25-262) from full
    molecular-orbital integrals, optionally from starting active RDMs (used
    when their trace is the electron count); returns (E, 1-RDM, 2-RDM, macro
    iterations, converged)."""
    d = dict(MCSCF_DEFAULTS)
    for k, v in settings.items():
        if k not in d:
            raise KeyError(k)
        d[k] = v
    s = np.array([float(d[k]) for k in MCSCF_DEFAULTS])
    T = np.asarray(T, dtype=np.float64)
    n = T.shape[0]
    Tb = np.ascontiguousarray(T.ravel(order="F"))
    Vb = np.ascontiguousarray(np.asarray(V, dtype=np.float64).reshape(n, n, n, n).ravel(order="F"))
    A1 = np.zeros(nact * nact) if rdm1 is None else np.array(np.asarray(rdm1, dtype=np.float64).ravel(order="F"))
    A2 = np.zeros(nact ** 4) if rdm2 is None else np.array(np.asarray(rdm2, dtype=np.float64).ravel(order="F"))
    E = ctypes.c_double()
    it = ctypes.c_int64()
    conv = ctypes.c_int()
    rc = lib().orc_casscf(s, int(nalpha), int(nbeta), n, int(ninact), int(nact), float(E_core), Tb, Vb, A1, A2,
                          ctypes.byref(E), ctypes.byref(it), ctypes.byref(conv))
    if rc != 0:
        raise RuntimeError(lib().orc_last_error().decode())
    return E.value, A1.reshape(nact, nact, order="F"), A2.reshape((nact,) * 4, order="F"), it.value, bool(conv.value)


def mcscf_fock(T, V, ninact, nact, rdm1=None, rdm2=None):
    """The fock_matrices.cxx building blocks at one orbital partition:
    (Fi, Fa, Q, F, inactive energy, energy from F); Fa / Q / F and the last
    energy need the active RDMs."""
    T = np.asarray(T, dtype=np.float64)
    n = T.shape[0]
    Tb = np.ascontiguousarray(T.ravel(order="F"))
    Vb = np.ascontiguousarray(np.asarray(V, dtype=np.float64).reshape(n, n, n, n).ravel(order="F"))
    na = int(nact)
    A1 = np.zeros(max(na * na, 1)) if rdm1 is None else np.ascontiguousarray(np.asarray(rdm1).ravel(order="F"))
    A2 = np.zeros(max(na ** 4, 1)) if rdm2 is None else np.ascontiguousarray(np.asarray(rdm2).ravel(order="F"))
    Fi, Fa, F = np.zeros(n * n), np.zeros(n * n), np.zeros(n * n)
    Q = np.zeros(max(na * n, 1))
    Ei, Ef = ctypes.c_double(), ctypes.c_double()
    lib().orc_mcscf_fock(n, int(ninact), na if rdm1 is not None else 0, Tb, Vb, A1, A2, Fi, Fa, Q, F,
                         ctypes.byref(Ei), ctypes.byref(Ef))
    m = lambda x: x.reshape(n, n, order="F")
    return m(Fi), m(Fa), Q[:na * n].reshape(na, n, order="F"), m(F), Ei.value, Ef.value
