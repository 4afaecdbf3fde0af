"""ctypes binding of oracle/_ref/libmacis_ref.so: the reference's own MACIS
code (unmodified headers and base.cxx, compiled by oracle/build_ref.sh with
the shims in oracle/ref_shims).  Test infrastructure only: it produces the
golden fixtures in tests/golden (make_ref_golden.py) and pins the oracle
restatement.  It needs the reference checkout to build, so it is available
in the container that holds the reference, not on machines without it.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "_ref", "libmacis_ref.so")
_lib = None

_u64p = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")


def reference_dir():
    """The reference checkout, from the QDK_REFERENCE environment variable."""
    d = os.environ.get("QDK_REFERENCE")
    if not d:
        raise RuntimeError("set QDK_REFERENCE to the reference checkout to build the reference's MACIS")
    return d


def build(force=False):
    if force or not os.path.exists(_LIB):
        subprocess.check_call(["sh", os.path.join(_HERE, "build_ref.sh"), reference_dir()])
    return _LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB)
        vp, i64, f64, ci = ctypes.c_void_p, ctypes.c_int64, ctypes.c_double, ctypes.c_int
        P = ctypes.POINTER
        L.ref_last_error.restype = ctypes.c_char_p
        L.ref_fci_dets.argtypes = [ci, ci, ci, P(i64), vp, vp]
        L.ref_build_csr.argtypes = [ci, _f64p, _f64p, i64, _u64p, _u64p, f64, P(vp)]
        L.ref_csr_info.argtypes = [vp, P(i64), P(i64), P(vp), P(vp), P(vp)]
        L.ref_csr_free.argtypes = [vp]
        L.ref_selected_ci_diag.argtypes = [vp, i64, f64, _f64p, P(f64), P(i64), P(i64)]
        L.ref_spmv.argtypes = [vp, _f64p, _f64p]
        L.ref_rdms_spin_dep.argtypes = [ci, _f64p, _f64p, i64, _u64p, _u64p, _f64p, vp, vp, vp, vp, vp]
        L.ref_rdms.argtypes = [ci, _f64p, _f64p, i64, _u64p, _u64p, _f64p, vp, vp]
        L.ref_lobpcg.argtypes = [vp, i64, i64, f64, i64, _f64p, _f64p, _f64p]
        L.ref_asci.restype = i64
        L.ref_asci.argtypes = [ci, _f64p, _f64p, _f64p, i64, _u64p, _u64p, _f64p, f64, ci, ci, i64, _u64p, _u64p,
                               _f64p, P(f64), P(f64)]
        _lib = L
    return _lib


def _check(rc):
    if rc != 0:
        raise RuntimeError("MACIS: " + lib().ref_last_error().decode())


def fci_dets(norb, na, nb):
    n = ctypes.c_int64()
    _check(lib().ref_fci_dets(norb, na, nb, ctypes.byref(n), None, None))
    a = np.zeros(n.value, np.uint64)
    b = np.zeros(n.value, np.uint64)
    _check(lib().ref_fci_dets(norb, na, nb, ctypes.byref(n), a.ctypes.data, b.ctypes.data))
    return a, b


class Csr:
    """sparsexx::csr_matrix<double, int64_t> made by make_csr_hamiltonian."""

    def __init__(self, norb, T, V, alpha, beta, thresh):
        self._T = np.asfortranarray(T, np.float64).ravel(order="F").copy()
        self._V = np.asarray(V, np.float64).ravel(order="F").copy()
        h = ctypes.c_void_p()
        _check(lib().ref_build_csr(norb, self._T, self._V, len(alpha), np.ascontiguousarray(alpha, np.uint64),
                                   np.ascontiguousarray(beta, np.uint64), thresh, ctypes.byref(h)))
        self.h = h

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.ref_csr_free(self.h)
            self.h = None

    def views(self):
        """(rowptr, colind, nzval) as zero-copy views of the reference's vectors."""
        m, nnz = ctypes.c_int64(), ctypes.c_int64()
        rp, ci, nz = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
        lib().ref_csr_info(self.h, ctypes.byref(m), ctypes.byref(nnz), ctypes.byref(rp), ctypes.byref(ci),
                           ctypes.byref(nz))
        mk = lambda p, n, t: np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(t)), shape=(n,))
        return mk(rp.value, m.value + 1, ctypes.c_int64), mk(ci.value, nnz.value, ctypes.c_int64), \
            mk(nz.value, nnz.value, ctypes.c_double)

    @property
    def n(self):
        return len(self.views()[0]) - 1

    def selected_ci_diag(self, max_m=200, tol=1e-8, guess=None):
        C = np.zeros(self.n) if guess is None else np.array(guess, np.float64)
        E, it, calls = ctypes.c_double(), ctypes.c_int64(), ctypes.c_int64()
        _check(lib().ref_selected_ci_diag(self.h, max_m, tol, C, ctypes.byref(E), ctypes.byref(it),
                                          ctypes.byref(calls)))
        return E.value, C, {"iterations": it.value, "sigma_calls": calls.value}

    def spmv(self, x):
        y = np.zeros(self.n)
        _check(lib().ref_spmv(self.h, np.ascontiguousarray(x, np.float64), y))
        return y

    def lobpcg(self, X, nroots, tol=1e-8, max_iter=500):
        # lobpcgxx's Rayleigh-Ritz assumes an orthonormal basis, so the
        # starting block is orthonormalised here (its callers do the same)
        X = np.asfortranarray(np.linalg.qr(np.asarray(X, np.float64))[0])
        k = X.shape[1]
        Xf = X.ravel(order="F").copy()
        ev, res = np.zeros(nroots), np.zeros(nroots)
        _check(lib().ref_lobpcg(self.h, k, nroots, tol, max_iter, Xf, ev, res))
        return ev, Xf.reshape((self.n, k), order="F")[:, :nroots], res


def rdms_spin_dep(norb, T, V, alpha, beta, C):
    """form_rdms_spin_dep over the whole list (accumulates into zeros)."""
    n = norb
    out = {k: np.zeros((n,) * (2 if len(k) == 2 else 4), order="F") for k in ("aa", "bb", "aaaa", "bbbb", "aabb")}
    Tf = np.asarray(T, np.float64).ravel(order="F").copy()
    Vf = np.asarray(V, np.float64).ravel(order="F").copy()
    _check(lib().ref_rdms_spin_dep(norb, Tf, Vf, len(alpha), np.ascontiguousarray(alpha, np.uint64),
                                   np.ascontiguousarray(beta, np.uint64), np.ascontiguousarray(C, np.float64),
                                   *[out[k].ctypes.data for k in ("aa", "bb", "aaaa", "bbbb", "aabb")]))
    return out


def rdms(norb, T, V, alpha, beta, C):
    """form_rdms (spin-traced) over the whole list."""
    n = norb
    o1 = np.zeros((n, n), order="F")
    o2 = np.zeros((n,) * 4, order="F")
    Tf = np.asarray(T, np.float64).ravel(order="F").copy()
    Vf = np.asarray(V, np.float64).ravel(order="F").copy()
    _check(lib().ref_rdms(norb, Tf, Vf, len(alpha), np.ascontiguousarray(alpha, np.uint64),
                          np.ascontiguousarray(beta, np.uint64), np.ascontiguousarray(C, np.float64),
                          o1.ctypes.data, o2.ctypes.data))
    return o1, o2


def asci(norb, T, V, alpha0, beta0, c0, E0, grow=True, refine=True, **settings):
    """The reference's asci_grow then asci_refine (wfn_t<128>); settings by the
    oracle's names (oracle.ASCI_DEFAULTS).  Returns (E, alpha, beta, C,
    E_after_grow)."""
    from . import oracle as _orc
    s = _orc._asci_settings(**settings)
    cap = int(max(s[0] * 4, 16))
    oa, ob, oc = np.zeros(cap, np.uint64), np.zeros(cap, np.uint64), np.zeros(cap)
    E, Eg = ctypes.c_double(), ctypes.c_double()
    Tf = np.asarray(T, np.float64).ravel(order="F").copy()
    Vf = np.asarray(V, np.float64).ravel(order="F").copy()
    n = lib().ref_asci(norb, Tf, Vf, s, len(alpha0), np.ascontiguousarray(alpha0, np.uint64),
                       np.ascontiguousarray(beta0, np.uint64), np.ascontiguousarray(c0, np.float64), float(E0),
                       int(grow), int(refine), cap, oa, ob, oc, ctypes.byref(E), ctypes.byref(Eg))
    if n < 0:
        raise RuntimeError("MACIS: " + lib().ref_last_error().decode())
    return E.value, oa[:n].copy(), ob[:n].copy(), oc[:n].copy(), Eg.value
