import importlib.util
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built sm_103a library")
    config.addinivalue_line("markers", "late: tests of the newest entry points, run after the others")


def pytest_collection_modifyitems(config, items):
    """Tests marked late run after the rest (before test_zz_no_alloc.py, which
    is collected last on purpose), so that under -x a failure in one of them
    leaves every other result in place."""
    def rank(item):
        if item.nodeid.startswith("tests/test_zz_") or "/test_zz_" in item.nodeid:
            return 2
        return 1 if item.get_closest_marker("late") else 0
    items[:] = sorted(items, key=rank)


def load_package():
    """Import the package directory ``qdk-chemistry_gb300`` as ``qdk_chemistry_gb300``."""
    name = "qdk_chemistry_gb300"
    if name in sys.modules:
        return sys.modules[name]
    pkg_dir = os.path.join(ROOT, "qdk-chemistry_gb300")
    spec = importlib.util.spec_from_file_location(name, os.path.join(pkg_dir, "__init__.py"),
                                                  submodule_search_locations=[pkg_dir])
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="session")
def pkg():
    return load_package()


@pytest.fixture(scope="session")
def oracle():
    import oracle as orc
    orc.build()
    return orc


@pytest.fixture(scope="session")
def known():
    with open(os.path.join(GOLDEN, "known_answers.json")) as f:
        return json.load(f)


def _pair_k(n):
    p, q = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    hi, lo = np.maximum(p, q), np.minimum(p, q)
    return hi * (hi + 1) // 2 + lo


def pack_eri(V):
    """The unique elements of an 8-fold symmetric V[p, q, r, s] (canonical
    pairs pq >= rs of canonical orbital pairs p >= q), exactly."""
    n = V.shape[0]
    k = _pair_k(n)
    P = n * (n + 1) // 2
    out = np.zeros(P * (P + 1) // 2)
    K1 = k[:, :, None, None]
    K2 = k[None, None, :, :]
    hi, lo = np.maximum(K1, K2), np.minimum(K1, K2)
    out[(hi * (hi + 1) // 2 + lo).ravel()] = np.asarray(V).ravel()
    return out


def unpack_eri(packed, n):
    """Inverse of pack_eri: the full n^4 array (bitwise equal to the packed V)."""
    k = _pair_k(n)
    K1 = k[:, :, None, None]
    K2 = k[None, None, :, :]
    hi, lo = np.maximum(K1, K2), np.minimum(K1, K2)
    return np.ascontiguousarray(packed[hi * (hi + 1) // 2 + lo])


def load_fcidump(name):
    pkg = load_package()
    d = np.load(os.path.join(GOLDEN, name + "_fcidump.npz"))
    return pkg.integrals.integrals_from_lines(int(d["norb"]), d["idx"], d["vals"], int(d["nelec"]), int(d["ms2"]))


@pytest.fixture(scope="session")
def h2o():
    return load_fcidump("h2o_ccpvdz")


@pytest.fixture(scope="session")
def n2_6e6o():
    return load_fcidump("n2_6e6o")


@pytest.fixture(scope="session")
def n2_14e18o():
    return load_fcidump("n2_14e18o")


def davidson_solver_cases():
    """The two analytic cases of python/tests/test_davidson_solver.py:17-71 as
    (name, CSR matrix, lowest eigenvalue, its eigenvector): the 6 x 6
    tridiagonal (2 on the diagonal, -1 beside it; 2 - 2 cos(pi/7), v_i =
    sin(i pi/7)) and the two-site Heisenberg XX + YY + ZZ (-3, the singlet)."""
    import scipy.sparse as sp
    tri = 2.0 * np.eye(6) - np.eye(6, k=1) - np.eye(6, k=-1)
    v = np.sin(np.arange(1, 7) * np.pi / 7)
    heis = np.array([[1.0, 0, 0, 0], [0, -1, 2, 0], [0, 2, -1, 0], [0, 0, 0, 1]])
    return [("tridiagonal6", sp.csr_matrix(tri), 2 - 2 * np.cos(np.pi / 7), v / np.linalg.norm(v)),
            ("heisenberg2", sp.csr_matrix(heis), -3.0, np.array([0.0, 1.0, -1.0, 0.0]) / np.sqrt(2))]


class OracleDevice:
    """A test-only stand-in for capi.Context whose calls are answered by the
    oracle: it runs the calculators' host orchestration end to end on the
    CPU (the device numerics are covered by the GPU tests)."""

    def __init__(self, device=0):
        import oracle
        self.o = oracle
        self.M = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False

    def set_integrals(self, T, V):
        self.n = T.shape[0]
        self.H = self.o.Hamiltonian(T, V)

    def set_dets(self, a, b):
        self.a, self.b = np.asarray(a, np.uint64), np.asarray(b, np.uint64)
        self.ndets = len(self.a)

    def build_hamiltonian(self, thresh=np.finfo(np.float64).eps, storage=0):
        self.M = self.o.build_csr(self.H, self.a, self.b, thresh)
        return self.M.nnz

    def build_operator(self, thresh=np.finfo(np.float64).eps, storage=0, max_m=200):
        self.build_hamiltonian(thresh, storage)
        return "csr"

    def set_device_limit(self, nbytes):
        pass

    def get_csr(self, index_bits=64):
        return self.M.arrays()

    def set_csr(self, rp, ci, nz):
        self.M = self.o.csr_from_arrays(rp, ci, nz)
        self.ndets = len(rp) - 1

    def diagonal(self):
        return self.M.diag()

    def davidson(self, max_m=200, tol=1e-8, precision=0, guess=None, want_vector=True):
        E, X, it = self.M.selected_ci_diag(max_m=max_m, tol=tol)
        return E, X, {"iterations": it}

    def rdms_spin_dep(self, C, want=("aa", "bb", "aaaa", "bbbb", "aabb")):
        return self.o.rdms_spin_dep(self.n, self.a, self.b, C, want=want)

    def orbital_entropies(self, C, two_orbital=True, mutual_information=True):
        s1, s2, mi = self.o.entropies(self.n, self.a, self.b, C)
        return s1, (s2 if two_orbital else None), (mi if mutual_information else None)

