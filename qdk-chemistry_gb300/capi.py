"""ctypes binding of libqdkgb.so (the C ABI in include/qdkgb.h).

This is the same binding a qdk-chemistry maintainer would add on the Python
side of the boundary.  The library is required: importing this module on a
machine without the built library raises, and every call that needs the GPU
raises the library's own error when no CUDA device is present.  There is no
CPU fallback.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libqdkgb.so")

OK = 0
ERR_INVALID = 1
ERR_CUDA = 2
ERR_OOM = 3
ERR_NOT_CONVERGED = 4
ERR_UNSUPPORTED = 5
ERR_STATE = 6

LAYOUT_COLMAJOR = 0
LAYOUT_ROWMAJOR = 1
# operator layouts (qdkgb_operator_layout, qdkgb_build_operator)
LAYOUT_NONE, LAYOUT_CSR, LAYOUT_SLAB, LAYOUT_DIRECT, LAYOUT_SLAB_DIRECT32 = 0, 1, 2, 3, 4
LAYOUT_NAMES = {1: "csr", 2: "slab", 3: "direct", 4: "slab+direct32"}
H_FP64 = 0
H_SPLIT32 = 1
PREC_FP64 = 0
PREC_MIXED = 1
OP_NONE, OP_CSR, OP_SLAB, OP_DIRECT, OP_SLAB_DIRECT32 = 0, 1, 2, 3, 4

EXPORTED = [
    "qdkgb_create", "qdkgb_destroy", "qdkgb_last_error", "qdkgb_set_stream", "qdkgb_device_bytes",
    "qdkgb_set_device_limit", "qdkgb_operator_layout", "qdkgb_problem_size", "qdkgb_direct_plan",
    "qdkgb_set_integrals", "qdkgb_fci_dets", "qdkgb_set_dets", "qdkgb_build_hamiltonian", "qdkgb_get_csr32",
    "qdkgb_get_csr64", "qdkgb_get_csr32_rows", "qdkgb_get_csr64_rows", "qdkgb_diagonal", "qdkgb_spmv", "qdkgb_spmv_device", "qdkgb_davidson_default_settings",
    "qdkgb_davidson", "qdkgb_rdms_spin_dep", "qdkgb_orbital_entropies", "qdkgb_casci",
    "qdkgb_mcscf_default_settings", "qdkgb_casscf", "qdkgb_version", "qdkgb_kernel_launches",
    "qdkgb_sigma_split_noalloc", "qdkgb_set_csr", "qdkgb_build_direct_sigma", "qdkgb_build_operator",
    "qdkgb_operator_action", "qdkgb_rdms", "qdkgb_asci_phase_times", "qdkgb_sigma_plan",
    "qdkgb_asci_default_settings", "qdkgb_asci_search", "qdkgb_asci", "qdkgb_asci_pt2",
    "qdkgb_batch_default_settings", "qdkgb_casci_batch", "qdkgb_batch_plan", "qdkgb_asci_rotation",
]


# the FP32 sigma kernels of the autotuner (qdkgb_sigma_plan), by index
SIGMA32_KERNELS = ("register", "tma", "register8", "register16")


class QdkgbError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("qdkgb error %d: %s" % (code, msg))
        self.code = code


class NotConverged(QdkgbError):
    pass


class DavidsonSettings(ctypes.Structure):
    _fields_ = [("max_m", ctypes.c_int64), ("res_tol", ctypes.c_double), ("precision", ctypes.c_int),
                ("use_guess", ctypes.c_int), ("min_abs_denominator", ctypes.c_double), ("nroots", ctypes.c_int)]


class McscfSettings(ctypes.Structure):
    """qdkgb_mcscf_settings (MCSCFSettings, mcscf.hpp:22-52)."""
    _fields_ = [("max_macro_iter", ctypes.c_int64), ("max_orbital_step", ctypes.c_double),
                ("orb_grad_tol", ctypes.c_double), ("enable_diis", ctypes.c_int), ("diis_start_iter", ctypes.c_int64),
                ("diis_nkeep", ctypes.c_int64), ("ci_res_tol", ctypes.c_double), ("ci_max_subspace", ctypes.c_int64),
                ("ci_matel_tol", ctypes.c_double)]


class AsciSettings(ctypes.Structure):
    _fields_ = [("ntdets_max", ctypes.c_int64), ("ntdets_min", ctypes.c_int64), ("ncdets_max", ctypes.c_int64),
                ("core_selection_fixed", ctypes.c_int), ("core_selection_threshold", ctypes.c_double),
                ("h_el_tol", ctypes.c_double), ("rv_prune_tol", ctypes.c_double), ("grow_factor", ctypes.c_double),
                ("min_grow_factor", ctypes.c_double), ("growth_backoff_rate", ctypes.c_double),
                ("growth_recovery_rate", ctypes.c_double), ("max_refine_iter", ctypes.c_int64),
                ("refine_energy_tol", ctypes.c_double), ("warm_start", ctypes.c_int),
                ("min_warm_start_overlap", ctypes.c_double), ("taper_grow_factor", ctypes.c_double),
                ("just_singles", ctypes.c_int), ("min_patch_overlap", ctypes.c_double),
                ("grow_with_rot", ctypes.c_int), ("rot_size_start", ctypes.c_int64)]


class CasInstance(ctypes.Structure):
    _fields_ = [("norb", ctypes.c_int), ("nalpha", ctypes.c_int), ("nbeta", ctypes.c_int),
                ("T", ctypes.c_void_p), ("V", ctypes.c_void_p)]


class BatchSettings(ctypes.Structure):
    _fields_ = [("res_tol", ctypes.c_double), ("precision", ctypes.c_int), ("max_subspace", ctypes.c_int),
                ("max_cycles", ctypes.c_int), ("matel_tol", ctypes.c_double),
                ("min_abs_denominator", ctypes.c_double), ("use_graph", ctypes.c_int),
                ("max_slab_bytes", ctypes.c_int64), ("persistent", ctypes.c_int), ("cluster", ctypes.c_int)]


class BatchInfo(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int), ("graph_replays", ctypes.c_int), ("seconds", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class DavidsonInfo(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int64), ("spmv_fp64", ctypes.c_int64), ("spmv_fp32", ctypes.c_int64),
                ("restarts", ctypes.c_int64), ("residual_norm", ctypes.c_double), ("seconds", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None


def lib():
    """Load the library (it must have been built: python qdk-chemistry_gb300/build.py)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError("libqdkgb.so is not built (%s); run qdk-chemistry_gb300/build.py" % LIB_PATH)
    L = ctypes.CDLL(LIB_PATH)
    vp, i64, ci, dp = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_double
    P = ctypes.POINTER
    L.qdkgb_create.argtypes = [P(vp), ci]
    L.qdkgb_destroy.argtypes = [vp]
    L.qdkgb_last_error.argtypes = [vp]
    L.qdkgb_last_error.restype = ctypes.c_char_p
    L.qdkgb_set_stream.argtypes = [vp, vp]
    L.qdkgb_device_bytes.argtypes = [vp, P(i64)]
    L.qdkgb_set_device_limit.argtypes = [vp, i64]
    L.qdkgb_operator_layout.argtypes = [vp, P(ctypes.c_int), P(i64)]
    L.qdkgb_direct_plan.argtypes = [vp, P(ctypes.c_int), P(ctypes.c_int), P(ctypes.c_double)]
    L.qdkgb_problem_size.argtypes = [vp, P(i64), P(i64)]
    L.qdkgb_set_integrals.argtypes = [vp, ci, vp, vp, ci]
    L.qdkgb_fci_dets.argtypes = [ci, ci, ci, vp, vp, P(i64)]
    L.qdkgb_set_dets.argtypes = [vp, i64, vp, vp]
    L.qdkgb_build_hamiltonian.argtypes = [vp, dp, ci, P(i64)]
    L.qdkgb_get_csr32.argtypes = [vp, vp, vp, vp]
    L.qdkgb_get_csr64.argtypes = [vp, vp, vp, vp]
    L.qdkgb_get_csr32_rows.argtypes = [vp, i64, i64, vp, vp, vp]
    L.qdkgb_build_operator.argtypes = [vp, dp, ci, ci, P(ci), P(i64)]
    L.qdkgb_operator_action.argtypes = [vp, i64, dp, vp, i64, dp, vp, i64]
    L.qdkgb_rdms.argtypes = [vp, vp, vp, vp]
    L.qdkgb_asci_phase_times.argtypes = [vp, vp, P(i64), P(i64)]
    L.qdkgb_batch_plan.argtypes = [vp, ci, P(ci), vp, vp, vp, vp, vp]
    L.qdkgb_asci_rotation.argtypes = [vp, vp]
    L.qdkgb_sigma_plan.argtypes = [vp, ci, P(ci), P(ci), vp, vp, P(ci), vp]
    L.qdkgb_get_csr64_rows.argtypes = [vp, i64, i64, vp, vp, vp]
    L.qdkgb_diagonal.argtypes = [vp, vp]
    L.qdkgb_set_csr.argtypes = [vp, i64, vp, vp, vp]
    L.qdkgb_build_direct_sigma.argtypes = [vp]
    L.qdkgb_asci_default_settings.argtypes = [P(AsciSettings)]
    L.qdkgb_asci_default_settings.restype = None
    L.qdkgb_mcscf_default_settings.argtypes = [P(McscfSettings)]
    L.qdkgb_mcscf_default_settings.restype = None
    L.qdkgb_casscf.argtypes = [vp, P(McscfSettings), ci, ci, ci, ci, ci, dp, vp, vp, vp, vp, P(dp), vp, P(i64), P(ci)]
    L.qdkgb_asci_search.argtypes = [vp, P(AsciSettings), i64, vp, vp, vp, dp, i64, i64, vp, vp, P(i64)]
    L.qdkgb_asci_pt2.argtypes = [vp, i64, vp, vp, vp, dp, dp, i64, P(dp), P(i64)]
    L.qdkgb_asci.argtypes = [vp, P(AsciSettings), P(DavidsonSettings), dp, i64, vp, vp, vp, dp, ci, ci, i64, vp, vp, vp,
                             P(i64), P(dp), P(dp)]
    L.qdkgb_spmv.argtypes = [vp, ci, vp, vp]
    L.qdkgb_spmv_device.argtypes = [vp, ci, vp, vp]
    L.qdkgb_davidson_default_settings.argtypes = [P(DavidsonSettings)]
    L.qdkgb_davidson_default_settings.restype = None
    L.qdkgb_davidson.argtypes = [vp, P(DavidsonSettings), P(dp), vp, P(DavidsonInfo)]
    L.qdkgb_rdms_spin_dep.argtypes = [vp, vp, vp, vp, vp, vp, vp]
    L.qdkgb_orbital_entropies.argtypes = [vp, vp, vp, vp, vp]
    L.qdkgb_casci.argtypes = [vp, ci, ci, ci, vp, vp, ci, P(DavidsonSettings), dp, P(dp), vp, P(DavidsonInfo)]
    L.qdkgb_version.restype = ctypes.c_char_p
    L.qdkgb_kernel_launches.restype = ctypes.c_int64
    L.qdkgb_sigma_split_noalloc.argtypes = [i64, vp, vp, vp, vp, vp, vp, vp]
    L.qdkgb_batch_default_settings.argtypes = [P(BatchSettings)]
    L.qdkgb_casci_batch.argtypes = [vp, ci, P(CasInstance), P(BatchSettings), vp, vp, vp, P(BatchInfo)]
    _lib = L
    return L


def _ptr(a):
    return None if a is None else a.ctypes.data


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def fci_dets(norb, nalpha, nbeta):
    """All determinants in MACIS order (generate_hilbert_space)."""
    n = ctypes.c_int64()
    rc = lib().qdkgb_fci_dets(norb, nalpha, nbeta, None, None, ctypes.byref(n))
    if rc:
        raise QdkgbError(rc, "invalid FCI space")
    a = np.zeros(n.value, dtype=np.uint64)
    b = np.zeros(n.value, dtype=np.uint64)
    rc = lib().qdkgb_fci_dets(norb, nalpha, nbeta, _ptr(a), _ptr(b), ctypes.byref(n))
    if rc:
        raise QdkgbError(rc, "fci_dets failed")
    return a, b


def kernel_launches():
    """Kernel launches issued by the library in this process."""
    return lib().qdkgb_kernel_launches()


NOALLOC_MAX_ROWS = 1 << 20


def sigma_split_noalloc(n, rowptr_ptr, colind_ptr, hi_ptr, lo_ptr, x_ptr, y_ptr, stream_ptr=None):
    """Allocation-free full-precision sigma on caller-owned device arrays
    (qdkgb_sigma_split_noalloc); raises on a non-zero status."""
    rc = lib().qdkgb_sigma_split_noalloc(n, rowptr_ptr, colind_ptr, hi_ptr, lo_ptr, x_ptr, y_ptr, stream_ptr)
    if rc:
        raise QdkgbError(rc, lib().qdkgb_last_error(None).decode())


def default_asci_settings(**kw):
    s = AsciSettings()
    lib().qdkgb_asci_default_settings(ctypes.byref(s))
    for k, v in kw.items():
        if not hasattr(s, k):
            raise KeyError(k)
        setattr(s, k, v)
    return s


def default_mcscf_settings(**kw):
    s = McscfSettings()
    lib().qdkgb_mcscf_default_settings(ctypes.byref(s))
    for k, v in kw.items():
        if not hasattr(s, k):
            raise KeyError(k)
        setattr(s, k, v)
    return s


def casscf(ctx, T, V, E_core, nalpha, nbeta, ninact, nact, rdm1=None, rdm2=None, **settings):
    """CASSCF (qdkgb_casscf, casscf_diis mcscf.hpp:54-60) from full molecular-
    orbital integrals T (n x n) and V (n^4, (pq|rs)); starts from the given
    spin-traced active RDMs when their trace is the electron count.  Returns
    (total energy, 1-RDM (nact x nact), 2-RDM (nact^4), orbital rotation U,
    macro iterations, converged)."""
    T = np.asarray(T, dtype=np.float64)
    n = T.shape[0]
    Tb = _f64(T.ravel(order="F"))
    Vb = _f64(np.asarray(V, dtype=np.float64).reshape(n, n, n, n).ravel(order="F"))
    s = default_mcscf_settings(**settings)
    A1 = np.zeros(nact * nact) if rdm1 is None else _f64(np.asarray(rdm1, dtype=np.float64).ravel(order="F")).copy()
    A2 = np.zeros(nact ** 4) if rdm2 is None else _f64(np.asarray(rdm2, dtype=np.float64).ravel(order="F")).copy()
    U = np.zeros(n * n)
    E = ctypes.c_double()
    it = ctypes.c_int64()
    conv = ctypes.c_int()
    ctx._check(lib().qdkgb_casscf(ctx.handle, ctypes.byref(s), int(nalpha), int(nbeta), n, int(ninact), int(nact),
                                  float(E_core), _ptr(Tb), _ptr(Vb), _ptr(A1), _ptr(A2), ctypes.byref(E), _ptr(U),
                                  ctypes.byref(it), ctypes.byref(conv)))
    return (E.value, A1.reshape(nact, nact, order="F"), A2.reshape((nact,) * 4, order="F"),
            U.reshape(n, n, order="F"), it.value, bool(conv.value))


def default_davidson_settings():
    s = DavidsonSettings()
    lib().qdkgb_davidson_default_settings(ctypes.byref(s))
    return s


class Context:
    """One GPU context: integrals, determinant space, device CSR, solver workspace."""

    def __init__(self, device=0):
        L = lib()
        h = ctypes.c_void_p()
        rc = L.qdkgb_create(ctypes.byref(h), device)
        if rc:
            raise QdkgbError(rc, "qdkgb_create failed (no usable CUDA device?)")
        self._h = h
        self.norb = None

    def close(self):
        if getattr(self, "_h", None):
            lib().qdkgb_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc):
        if rc:
            msg = lib().qdkgb_last_error(self._h).decode()
            if rc == ERR_NOT_CONVERGED:
                raise NotConverged(rc, msg)
            raise QdkgbError(rc, msg)

    def _sizes(self):
        nd, nnz = ctypes.c_int64(), ctypes.c_int64()
        self._check(lib().qdkgb_problem_size(self._h, ctypes.byref(nd), ctypes.byref(nnz)))
        return nd.value, nnz.value

    @property
    def ndets(self):
        """Dimension of the operator (qdkgb_problem_size): the current list's
        determinant count, or the rows of a caller's CSR."""
        return self._sizes()[0]

    @property
    def nnz(self):
        """CSR elements of the built operator as the getters export them."""
        return self._sizes()[1]

    @property
    def handle(self):
        return self._h

    def device_bytes(self):
        b = ctypes.c_int64()
        self._check(lib().qdkgb_device_bytes(self._h, ctypes.byref(b)))
        return b.value

    def set_device_limit(self, nbytes):
        """Cap the device memory the context may hold (0: no cap); a larger
        allocation raises QdkgbError(ERR_OOM) and the context stays usable."""
        self._check(lib().qdkgb_set_device_limit(self._h, int(nbytes)))

    def operator_layout(self):
        """(layout, stored elements): OP_CSR, OP_SLAB (complete space, values
        only), OP_SLAB_DIRECT32 (the FP64 slab, and the direct contraction
        for the mixed form's FP32 sigma) or OP_DIRECT (no stored matrix);
        OP_NONE before a build."""
        lay = ctypes.c_int()
        st = ctypes.c_int64()
        self._check(lib().qdkgb_operator_layout(self._h, ctypes.byref(lay), ctypes.byref(st)))
        return lay.value, st.value

    def set_stream(self, stream_ptr):
        self._check(lib().qdkgb_set_stream(self._h, stream_ptr))

    def set_integrals(self, T, V, layout=LAYOUT_COLMAJOR):
        """T, V as numpy arrays indexed [p,q] / [p,q,r,s]; passed column-major."""
        T = np.asarray(T, dtype=np.float64)
        V = np.asarray(V, dtype=np.float64)
        n = T.shape[0]
        if layout == LAYOUT_COLMAJOR:
            Tb = _f64(T.ravel(order="F"))
            Vb = _f64(V.ravel(order="F"))
        else:
            Tb = _f64(T.ravel(order="C"))
            Vb = _f64(V.ravel(order="C"))
        self._check(lib().qdkgb_set_integrals(self._h, n, _ptr(Tb), _ptr(Vb), layout))
        self.norb = n

    def set_dets(self, alpha, beta):
        alpha = np.ascontiguousarray(alpha, dtype=np.uint64)
        beta = np.ascontiguousarray(beta, dtype=np.uint64)
        self._check(lib().qdkgb_set_dets(self._h, len(alpha), _ptr(alpha), _ptr(beta)))

    def build_hamiltonian(self, thresh=np.finfo(np.float64).eps, storage=H_FP64):
        nnz = ctypes.c_int64()
        self._check(lib().qdkgb_build_hamiltonian(self._h, float(thresh), storage, ctypes.byref(nnz)))
        return nnz.value

    def build_operator(self, thresh=np.finfo(np.float64).eps, storage=H_FP64, max_m=200):
        """The stored Hamiltonian when it fits on the device, else (complete
        spaces) the direct sigma (qdkgb_build_operator); returns the layout
        name ("slab", "slab+direct32", "csr" or "direct")."""
        lay = ctypes.c_int()
        nnz = ctypes.c_int64()
        self._check(lib().qdkgb_build_operator(self._h, float(thresh), int(storage), int(max_m), ctypes.byref(lay),
                                               ctypes.byref(nnz)))
        return LAYOUT_NAMES[lay.value]

    def direct_plan(self):
        """The direct sigma's FP32 form (qdkgb_direct_plan): {"contraction":
        "walk" / "fma" / "tensor", "dense": None (not yet timed) / bool,
        "same_spin_ms": (element-wise, dense), "contraction_ms": (FMA,
        tensor cores)}."""
        mm, dense = ctypes.c_int(), ctypes.c_int()
        ms = (ctypes.c_double * 4)()
        self._check(lib().qdkgb_direct_plan(self._h, ctypes.byref(mm), ctypes.byref(dense), ms))
        return {"contraction": ("walk", "fma", "tensor")[mm.value],
                "dense": None if dense.value < 0 else bool(dense.value),
                "same_spin_ms": (ms[0], ms[1]), "contraction_ms": (ms[2], ms[3])}

    def build_direct_sigma(self):
        """Recompute-on-the-fly sigma for a complete space (no CSR stored)."""
        self._check(lib().qdkgb_build_direct_sigma(self._h))

    def get_csr(self, index_bits=64):
        n, nnz = self._sizes()
        it = np.int64 if index_bits == 64 else np.int32
        rp = np.zeros(n + 1, dtype=it)
        ci = np.zeros(nnz, dtype=it)
        nz = np.zeros(nnz, dtype=np.float64)
        fn = lib().qdkgb_get_csr64 if index_bits == 64 else lib().qdkgb_get_csr32
        self._check(fn(self._h, _ptr(rp), _ptr(ci), _ptr(nz)))
        return rp, ci, nz

    def get_csr_rows(self, row_begin, row_end, index_bits=64):
        """Rows [row_begin, row_end) of the CSR as a bra block: (rowptr from 0,
        global colind, values)."""
        it = np.int64 if index_bits == 64 else np.int32
        fn = lib().qdkgb_get_csr64_rows if index_bits == 64 else lib().qdkgb_get_csr32_rows
        rp = np.zeros(row_end - row_begin + 1, dtype=it)
        self._check(fn(self._h, row_begin, row_end, _ptr(rp), None, None))
        ci = np.zeros(int(rp[-1]), dtype=it)
        nz = np.zeros(int(rp[-1]), dtype=np.float64)
        self._check(fn(self._h, row_begin, row_end, _ptr(rp), _ptr(ci), _ptr(nz)))
        return rp, ci, nz

    def set_csr(self, rowptr, colind, values):
        """Use a caller's CSR matrix (0-based) as the device operator."""
        rp = np.ascontiguousarray(rowptr, dtype=np.int64)
        ci = np.ascontiguousarray(colind, dtype=np.int64)
        nz = _f64(values)
        n = len(rp) - 1
        self._check(lib().qdkgb_set_csr(self._h, n, _ptr(rp), _ptr(ci), _ptr(nz)))

    def diagonal(self):
        d = np.zeros(self.ndets)
        self._check(lib().qdkgb_diagonal(self._h, _ptr(d)))
        return d

    def spmv(self, x, precision=PREC_FP64):
        x = _f64(x)
        y = np.zeros(self.ndets)
        self._check(lib().qdkgb_spmv(self._h, precision, _ptr(x), _ptr(y)))
        return y

    def spmv_device(self, x_ptr, y_ptr, precision=PREC_FP64):
        self._check(lib().qdkgb_spmv_device(self._h, precision, x_ptr, y_ptr))

    def davidson(self, max_m=200, tol=1e-8, precision=PREC_FP64, guess=None, want_vector=True, nroots=1):
        """Lowest root (E, C, info); with nroots > 1 the block Davidson:
        (energies (nroots), C (ndets x nroots), info)."""
        s = default_davidson_settings()
        s.max_m = max_m
        s.res_tol = tol
        s.precision = precision
        s.nroots = nroots
        if nroots > 1:
            C = np.zeros(self.ndets * nroots) if (want_vector or guess is not None) else None
            if guess is not None:
                C[:] = np.asarray(guess, dtype=np.float64).ravel(order="F")
            s.use_guess = 0 if guess is None else 1
            E = np.zeros(nroots)
            info = DavidsonInfo()
            self._check(lib().qdkgb_davidson(self._h, ctypes.byref(s), E.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                             _ptr(C), ctypes.byref(info)))
            return E, (C.reshape((self.ndets, nroots), order="F") if C is not None else None), info.as_dict()
        C = np.zeros(self.ndets) if guess is None else _f64(guess).copy()
        if not want_vector and guess is None:
            C = None
        s.use_guess = 0 if guess is None else 1
        E = ctypes.c_double()
        info = DavidsonInfo()
        self._check(lib().qdkgb_davidson(self._h, ctypes.byref(s), ctypes.byref(E), _ptr(C), ctypes.byref(info)))
        return E.value, C, info.as_dict()

    def rdms_spin_dep(self, C, want=("aa", "bb", "aaaa", "bbbb", "aabb")):
        n = self.norb
        C = _f64(C)
        bufs = {}
        ptrs = []
        for k in ("aa", "bb", "aaaa", "bbbb", "aabb"):
            if k in want:
                bufs[k] = np.zeros(n ** (2 if len(k) == 2 else 4))
                ptrs.append(_ptr(bufs[k]))
            else:
                ptrs.append(None)
        self._check(lib().qdkgb_rdms_spin_dep(self._h, _ptr(C), *ptrs))
        return {k: v.reshape((n, n) if len(k) == 2 else (n, n, n, n), order="F") for k, v in bufs.items()}

    def sigma_plan(self, precision=PREC_MIXED, with_kernel=False):
        """(segments in use, [(candidate segments, mean ms), ...]) of the
        complete-space sigma's autotuner (qdkgb_sigma_plan); with_kernel adds
        the FP32 kernel in use (a name of SIGMA32_KERNELS) and every kernel's
        ms per candidate ({name: [ms, ...]}, NaN where not timed)."""
        seg = ctypes.c_int()
        n = ctypes.c_int(32)
        ker = ctypes.c_int()
        cs = np.zeros(32, dtype=np.int32)
        cm = np.zeros(32)
        km = np.zeros(4 * 32)
        self._check(lib().qdkgb_sigma_plan(self._h, precision, ctypes.byref(seg), ctypes.byref(n), cs.ctypes.data,
                                           cm.ctypes.data, ctypes.byref(ker), km.ctypes.data))
        m = min(n.value, 32)
        out = (seg.value, [(int(cs[i]), float(cm[i])) for i in range(m)])
        if with_kernel:
            out = out + (SIGMA32_KERNELS[ker.value],
                         {SIGMA32_KERNELS[k]: [float(km[32 * k + i]) for i in range(m)] for k in range(4)})
        return out

    def operator_action(self, V, alpha=1.0, AV=None, beta=0.0):
        """AV = alpha H V + beta AV for the columns of V (ndets x m), the
        reference's operator_action block contract (qdkgb_operator_action)."""
        Vf = np.asfortranarray(np.asarray(V, dtype=np.float64).reshape(self.ndets, -1))
        m = Vf.shape[1]
        out = np.zeros((self.ndets, m), order="F") if AV is None else np.asfortranarray(
            np.array(AV, dtype=np.float64).reshape(self.ndets, m))
        self._check(lib().qdkgb_operator_action(self._h, m, float(alpha), Vf.ctypes.data, self.ndets, float(beta),
                                                out.ctypes.data, self.ndets))
        return out

    def rdms(self, C):
        """Spin-traced (1-RDM, 2-RDM) of form_rdms (qdkgb_rdms)."""
        n = self.norb
        o1 = np.zeros(n * n)
        o2 = np.zeros(n ** 4)
        self._check(lib().qdkgb_rdms(self._h, _ptr(_f64(C)), _ptr(o1), _ptr(o2)))
        return o1.reshape((n, n), order="F"), o2.reshape((n, n, n, n), order="F")

    def orbital_entropies(self, C, two_orbital=True, mutual_information=True):
        """(single-orbital entropies (n), two-orbital entropies (n x n) or None,
        mutual information (n x n) or None) of C over the current determinants
        (qdkgb_orbital_entropies)."""
        n = self.norb
        C = _f64(C)
        s1 = np.zeros(n)
        s2 = np.zeros((n, n)) if two_orbital else None
        mi = np.zeros((n, n)) if mutual_information else None
        self._check(lib().qdkgb_orbital_entropies(self._h, _ptr(C), _ptr(s1), _ptr(s2) if s2 is not None else None,
                                                  _ptr(mi) if mi is not None else None))
        return s1, s2, mi

    def casci(self, T, V, nalpha, nbeta, max_m=200, tol=1e-8, precision=PREC_FP64, matel_tol=np.finfo(float).eps,
              want_vector=True):
        T = np.asarray(T, dtype=np.float64)
        V = np.asarray(V, dtype=np.float64)
        n = T.shape[0]
        Tb = _f64(T.ravel(order="F"))
        Vb = _f64(V.ravel(order="F"))
        s = default_davidson_settings()
        s.max_m = max_m
        s.res_tol = tol
        s.precision = precision
        nd = ctypes.c_int64()
        lib().qdkgb_fci_dets(n, nalpha, nbeta, None, None, ctypes.byref(nd))
        C = np.zeros(nd.value) if want_vector else None
        E = ctypes.c_double()
        info = DavidsonInfo()
        self._check(lib().qdkgb_casci(self._h, n, nalpha, nbeta, _ptr(Tb), _ptr(Vb), LAYOUT_COLMAJOR,
                                      ctypes.byref(s), float(matel_tol), ctypes.byref(E), _ptr(C),
                                      ctypes.byref(info)))
        self.norb = n
        return E.value, C, info.as_dict()


def _asci_ctx_check(ctx, rc):
    ctx._check(rc)


def asci_search(ctx, core_alpha, core_beta, core_coeff, E0, ndets_max, **settings):
    """One GPU determinant search (qdkgb_asci_search)."""
    s = default_asci_settings(**settings)
    ca = np.ascontiguousarray(core_alpha, dtype=np.uint64)
    cb = np.ascontiguousarray(core_beta, dtype=np.uint64)
    cc = _f64(core_coeff)
    n = ctypes.c_int64()
    ctx._check(lib().qdkgb_asci_search(ctx.handle, ctypes.byref(s), len(ca), _ptr(ca), _ptr(cb), _ptr(cc), float(E0),
                                       int(ndets_max), 0, None, None, ctypes.byref(n)))
    oa = np.zeros(n.value, dtype=np.uint64)
    ob = np.zeros(n.value, dtype=np.uint64)
    ctx._check(lib().qdkgb_asci_search(ctx.handle, ctypes.byref(s), len(ca), _ptr(ca), _ptr(cb), _ptr(cc), float(E0),
                                       int(ndets_max), n.value, _ptr(oa), _ptr(ob), ctypes.byref(n)))
    return oa, ob


def asci_pt2(ctx, alpha, beta, coeff, E0, pt2_tol=1e-16, max_slots=0):
    """ASCI-PT2 on the GPU (qdkgb_asci_pt2, asci_pt2_constraint pt2.hpp:59-565)
    for a wavefunction sorted by spin_comparator; integrals must be set.
    max_slots bounds the target table (0: by free memory; smaller tables
    split the target space into passes).  Returns (E_PT2, number of external
    determinants)."""
    a = np.ascontiguousarray(alpha, dtype=np.uint64)
    b = np.ascontiguousarray(beta, dtype=np.uint64)
    c = _f64(coeff)
    if not (len(a) == len(b) == len(c)):
        raise ValueError("alpha, beta and coeff must have the same length")
    e = ctypes.c_double()
    n = ctypes.c_int64()
    ctx._check(lib().qdkgb_asci_pt2(ctx.handle, len(a), _ptr(a), _ptr(b), _ptr(c), float(E0), float(pt2_tol),
                                    int(max_slots), ctypes.byref(e), ctypes.byref(n)))
    return e.value, n.value


def asci(ctx, alpha0, beta0, c0, E0, grow=True, refine=True, tol=1e-8, max_m=200, precision=PREC_FP64,
         matel_tol=np.finfo(float).eps, **settings):
    """asci_grow + asci_refine on the GPU (qdkgb_asci); integrals must be set.
    Returns (E, alpha, beta, C, E_after_grow)."""
    s = default_asci_settings(**settings)
    ci = default_davidson_settings()
    ci.res_tol = tol
    ci.max_m = max_m
    ci.precision = precision
    a0 = np.ascontiguousarray(alpha0, dtype=np.uint64)
    b0 = np.ascontiguousarray(beta0, dtype=np.uint64)
    c0 = _f64(c0)
    cap = int(max(s.ntdets_max * 4, 16))
    oa = np.zeros(cap, dtype=np.uint64)
    ob = np.zeros(cap, dtype=np.uint64)
    oc = np.zeros(cap)
    n = ctypes.c_int64()
    E = ctypes.c_double()
    Eg = ctypes.c_double()
    ctx._check(lib().qdkgb_asci(ctx.handle, ctypes.byref(s), ctypes.byref(ci), float(matel_tol), len(a0), _ptr(a0),
                                _ptr(b0), _ptr(c0), float(E0), int(grow), int(refine), cap, _ptr(oa), _ptr(ob),
                                _ptr(oc), ctypes.byref(n), ctypes.byref(E), ctypes.byref(Eg)))
    m = min(n.value, cap)
    return E.value, oa[:m].copy(), ob[:m].copy(), oc[:m].copy(), Eg.value


def asci_rotation(ctx):
    """The last asci call's accumulated natural-orbital rotation (norb x norb,
    columns = the final orbitals over the given ones; the identity without
    grow_with_rot) (qdkgb_asci_rotation)."""
    n = int(ctx.norb)
    U = np.zeros(n * n)
    ctx._check(lib().qdkgb_asci_rotation(ctx.handle, _ptr(U)))
    return U.reshape((n, n), order="F")


def asci_phase_times(ctx):
    """Seconds of the last asci call by phase (search, determinant space,
    H build, Davidson), its asci_iter count and how many of its Hamiltonians
    were patched from the previous one (qdkgb_asci_phase_times)."""
    t = np.zeros(4)
    it, pb = ctypes.c_int64(), ctypes.c_int64()
    ctx._check(lib().qdkgb_asci_phase_times(ctx.handle, _ptr(t), ctypes.byref(it), ctypes.byref(pb)))
    return {"search_s": t[0], "det_space_s": t[1], "hbuild_s": t[2], "davidson_s": t[3], "iterations": it.value,
            "patched_builds": pb.value}


def batch_plan(ctx, cap=16):
    """The persistent batched solver's tuning record (qdkgb_batch_plan): per
    tuned shape, its (norb, nalpha, nbeta), the cluster size in use and the
    timed candidates as (cluster size, ms)."""
    n = ctypes.c_int()
    shape = np.zeros(3 * cap, dtype=np.int32)
    cl = np.zeros(cap, dtype=np.int32)
    nc = np.zeros(cap, dtype=np.int32)
    cc = np.zeros(4 * cap, dtype=np.int32)
    cm = np.zeros(4 * cap)
    ctx._check(lib().qdkgb_batch_plan(ctx.handle, cap, ctypes.byref(n), _ptr(shape), _ptr(cl), _ptr(nc), _ptr(cc),
                                      _ptr(cm)))
    out = []
    for i in range(min(n.value, cap)):
        out.append({"shape": tuple(int(v) for v in shape[3 * i:3 * i + 3]), "cluster": int(cl[i]),
                    "candidates": [(int(cc[4 * i + j]), float(cm[4 * i + j])) for j in range(int(nc[i]))]})
    return out


def default_batch_settings(**kw):
    s = BatchSettings()
    lib().qdkgb_batch_default_settings(ctypes.byref(s))
    for k, v in kw.items():
        if not hasattr(s, k):
            raise KeyError(k)
        setattr(s, k, v)
    return s


def casci_batch(ctx, instances, want_rdm1=True, **settings):
    """Batched CASCI (qdkgb_casci_batch).  instances: sequence of
    (norb, nalpha, nbeta, T, V) with T[p, q] and V[p, q, r, s] numpy arrays.
    Returns (energies, [1-RDM per instance or None], iterations, info)."""
    s = default_batch_settings(**settings)
    n = len(instances)
    arr = (CasInstance * max(n, 1))()
    keep = []
    for i, (norb, na, nb, T, V) in enumerate(instances):
        Tb = _f64(np.asarray(T, dtype=np.float64).ravel(order="F"))
        Vb = _f64(np.asarray(V, dtype=np.float64).ravel(order="F"))
        keep += [Tb, Vb]
        arr[i] = CasInstance(int(norb), int(na), int(nb), Tb.ctypes.data, Vb.ctypes.data)
    E = np.zeros(n)
    its = np.zeros(n, dtype=np.int32)
    offs = np.concatenate([[0], np.cumsum([int(x[0]) ** 2 for x in instances])]).astype(np.int64)
    R = np.zeros(int(offs[-1])) if want_rdm1 else None
    info = BatchInfo()
    ctx._check(lib().qdkgb_casci_batch(ctx.handle, n, arr, ctypes.byref(s), _ptr(E), _ptr(R), _ptr(its),
                                       ctypes.byref(info)))
    rdms = None
    if want_rdm1:
        rdms = [R[offs[i]:offs[i + 1]].reshape(int(instances[i][0]), int(instances[i][0])) for i in range(n)]
    return E, rdms, its, info.as_dict()
