"""qdk-chemistry's multi-configuration plugin surface, backed by the GB300 core.

Mirrors, with the same names, defaults and error behaviour:
* the algorithm registry: ``create(type, name, **settings)``,
  ``available(...)``, ``register(generator)``, ``unregister(...)``,
  ``show_default(...)`` (python/src/qdk_chemistry/algorithms/registry.py:
  295-663, cpp/include/qdk/chemistry/algorithms/algorithm.hpp:242-369);
* ``MultiConfigurationSettings`` + the MACIS settings
  (cpp/include/qdk/chemistry/algorithms/mc.hpp:26-62,
  cpp/src/qdk/chemistry/algorithms/microsoft/macis_base.hpp:27-36): typed
  defaults, bound checks, locked once ``run`` starts (``SettingsAreLocked``);
* ``MultiConfigurationCalculator.run(hamiltonian, n_alpha, n_beta) ->
  (total energy, Wavefunction)`` (mc.hpp:87-172), the CASCI plugin
  (macis_cas.cpp:35-148) and the ASCI plugin (macis_asci.cpp:44-234);
* ``ProjectedMultiConfigurationCalculator.run(hamiltonian, configurations)``
  (pmc.hpp:31-150) and the PMC plugin (macis_pmc.cpp:42-178);
* the entropy-based active-space selectors over the wavefunction's
  entropies (autocas_active_space.cpp, entropy_active_space.cpp);
* ``davidson_solver(csr, tol=1e-8, max_m=20) -> (eigenvalue, eigenvector)``
  (python/src/pybind11/algorithms/davidson_solver.cpp:56-108).
All computation runs in libqdkgb.so on the GPU.
"""
import numpy as np

from . import capi, determinants, integrals


class SettingsAreLocked(RuntimeError):
    pass


class DuplicateRegistrationError(RuntimeError):
    pass


class Settings:
    """Typed settings with defaults and optional constraints (data::Settings):
    a (lo, hi) tuple bounds a number (BoundConstraint), a list names the
    allowed values (ListConstraint)."""

    def __init__(self):
        self._values = {}
        self._types = {}
        self._bounds = {}
        self._doc = {}
        self._locked = False

    def set_default(self, key, typ, value, doc="", bounds=None):
        self._types[key] = typ
        self._values[key] = typ(value)
        self._bounds[key] = bounds
        self._doc[key] = doc

    def set(self, key, value):
        if self._locked:
            raise SettingsAreLocked("settings are locked (the algorithm has run)")
        if key not in self._types:
            raise KeyError("unknown setting '%s'" % key)
        typ = self._types[key]
        if typ is bool and not isinstance(value, (bool, np.bool_)):
            raise TypeError("setting '%s' expects bool" % key)
        if typ in (int, float) and isinstance(value, bool):
            raise TypeError("setting '%s' expects %s" % (key, typ.__name__))
        if typ is str and not isinstance(value, str):
            raise TypeError("setting '%s' expects str" % key)
        v = typ(value)
        b = self._bounds.get(key)
        if isinstance(b, list):
            if v not in b:
                raise ValueError("setting '%s' = %r not one of %r" % (key, v, b))
        elif b is not None:
            lo, hi = b
            if not (lo <= v <= hi):
                raise ValueError("setting '%s' = %r outside [%r, %r]" % (key, v, lo, hi))
        self._values[key] = v

    def get(self, key):
        return self._values[key]

    def get_or_default(self, key, default):
        return self._values.get(key, default)

    def update(self, values=None, **kw):
        """Set several settings at once (each checked as by set)."""
        for key, value in dict(values or {}, **kw).items():
            self.set(key, value)

    def get_expected_python_type(self, key):
        return self._types[key].__name__

    def has_description(self, key):
        return bool(self._doc.get(key))

    def get_description(self, key):
        return self._doc[key]

    def has_limits(self, key):
        return self._bounds.get(key) is not None

    def get_limits(self, key):
        return self._bounds[key]

    def has(self, key):
        return key in self._values

    def keys(self):
        return list(self._values)

    def lock(self):
        self._locked = True

    def locked(self):
        return self._locked

    def to_dict(self):
        return dict(self._values)


class MultiConfigurationSettings(Settings):
    """mc.hpp:34-62 defaults."""

    def __init__(self):
        super().__init__()
        self.set_default("calculate_one_rdm", bool, False)
        self.set_default("calculate_two_rdm", bool, False)
        self.set_default("calculate_single_orbital_entropies", bool, False)
        self.set_default("calculate_two_orbital_entropies", bool, False)
        self.set_default("calculate_mutual_information", bool, False)
        self.set_default("ci_residual_tolerance", float, 1.0e-6, "CI residual convergence tolerance", (0.0, 1.0))
        self.set_default("max_solver_iterations", int, 200, "Maximum number of Davidson iterations", (1, 2 ** 63 - 1))
        self.set_default("iterative_solver_dimension_cutoff", int, 2000,
                         "Matrix size cutoff for using iterative eigensolver", (1, 2 ** 63 - 1))


class Gb300Settings(MultiConfigurationSettings):
    """MacisSettings (macis_base.hpp:27-36) plus the GPU controls."""

    def __init__(self):
        super().__init__()
        self.set_default("ci_matel_tol", float, np.finfo(np.float64).eps,
                         "Hamiltonian matrix element sparsification threshold", (0.0, 1.0))
        self.set_default("precision", str, "fp64", "fp64 or mixed (FP32 sigma with FP64 defect correction)",
                         ["fp64", "mixed"])
        self.set_default("device", int, 0, "CUDA device ordinal", (0, 1024))
        self.set_default("device_memory_limit", int, 0,
                         "cap on the device bytes the calculation may hold (0: none); when the stored "
                         "Hamiltonian would not fit, complete spaces use the direct sigma", (0, 1 << 62))


class Hamiltonian:
    """Active-space Hamiltonian: one-body T (n x n), two-body V (n^4, (pq|rs)),
    core energy (data::Hamiltonian's get_one_body_integrals /
    get_two_body_integrals / get_core_energy)."""

    def __init__(self, one_body, two_body, core_energy=0.0):
        self._T = np.asarray(one_body, dtype=np.float64)
        n = self._T.shape[0]
        V = np.asarray(two_body, dtype=np.float64)
        self._V = V.reshape(n, n, n, n)
        self._ecore = float(core_energy)

    @classmethod
    def from_fcidump(cls, path):
        d = integrals.read_fcidump(path)
        return cls(d["T"], d["V"], d["E_core"])

    @property
    def norb(self):
        return self._T.shape[0]

    def get_one_body_integrals(self):
        return self._T

    def get_two_body_integrals(self):
        return self._V

    def get_core_energy(self):
        return self._ecore


def single_orbital_entropies(occ_alpha, occ_beta, double_occ):
    """-sum w ln w over the one-orbital RDM eigenvalues (empty, alpha only,
    beta only, double: 1 - na - nb + d, na - d, nb - d, d), zero weights
    skipped (orbital_entropy.hpp:24-37, Boguslawski & Tecmer 2015)."""
    na = np.asarray(occ_alpha, dtype=np.float64)
    nb = np.asarray(occ_beta, dtype=np.float64)
    d = np.asarray(double_occ, dtype=np.float64)
    out = np.zeros(na.shape)
    for w in (1.0 - na - nb + d, na - d, nb - d, d):
        pos = w > 0.0
        out[pos] -= w[pos] * np.log(w[pos])
    return out


class Wavefunction:
    """Determinants + CI coefficients (+ optional RDMs), the StateVectorContainer
    the reference builds (macis_base.hpp:134-283).  The spin-resolved two-body
    RDMs carry the reference's factor 2 (macis_base.hpp:203-212)."""

    def __init__(self, norb, alpha, beta, coeffs, rdms=None, entropies=None, active_indices=None,
                 inactive_indices=None):
        self.norb = norb
        # the molecular-orbital indices of the active orbitals (0 .. norb-1
        # unless given) and of the doubly occupied inactive ones
        self.active_indices = list(range(norb)) if active_indices is None else [int(i) for i in active_indices]
        self.inactive_indices = [] if inactive_indices is None else [int(i) for i in inactive_indices]
        if len(self.active_indices) != norb:
            raise ValueError("active_indices must name norb orbitals")
        self.alpha = np.asarray(alpha, dtype=np.uint64)
        self.beta = np.asarray(beta, dtype=np.uint64)
        self.coefficients = np.asarray(coeffs, dtype=np.float64)
        self._rdms = dict(rdms or {})
        self._ent = dict(entropies or {})

    def size(self):
        return len(self.coefficients)

    def get_active_indices(self):
        return list(self.active_indices)

    def get_inactive_indices(self):
        return list(self.inactive_indices)

    def get_active_num_electrons(self):
        return (int(self.alpha[0]).bit_count(), int(self.beta[0]).bit_count()) if len(self.alpha) else (0, 0)

    def get_total_num_electrons(self):
        na, nb = self.get_active_num_electrons()
        return na + len(self.inactive_indices), nb + len(self.inactive_indices)

    # the StateVectorContainer accessors (state_vector.cpp:171-330, 785-880)
    def get_coefficients(self):
        return self.coefficients

    def to_macis_file(self, path):
        """MACIS's text wavefunction (write_wavefunction, wavefunction_io.hpp:95-116)."""
        determinants.write_wavefunction(path, self.norb, self.alpha, self.beta, self.coefficients)

    @classmethod
    def from_macis_file(cls, path):
        a, b, c, norb, _, _ = determinants.read_wavefunction(path)
        return cls(norb, a, b, c)

    def get_active_determinants(self):
        return self.get_configurations()

    def get_coefficient(self, configuration):
        """The coefficient of a determinant (canonical string or (alpha, beta)
        pair); 0 for one absent from the expansion."""
        if not len(self.alpha):
            raise RuntimeError("No determinants available")
        if isinstance(configuration, str):
            a, b = determinants.from_canonical_string(configuration)
        else:
            a, b = configuration
        hit = np.flatnonzero((self.alpha == np.uint64(a)) & (self.beta == np.uint64(b)))
        return float(self.coefficients[hit[0]]) if len(hit) else 0.0

    def get_active_orbital_occupations(self):
        """(alpha, beta) occupations of the active orbitals: those of the
        determinant for a single one, else the eigenvalues of the spin-resolved
        1-RDMs in descending order."""
        if not len(self.alpha):
            raise RuntimeError("No determinants available")
        if self.size() == 1:
            bits = np.arange(self.norb, dtype=np.uint64)
            occ = lambda s: ((np.uint64(s) >> bits) & np.uint64(1)).astype(np.float64)
            return occ(self.alpha[0]), occ(self.beta[0])
        if not self.has_one_rdm():
            raise RuntimeError("1RDM must be available to compute orbital occupations")
        aa, bb = self.get_active_one_rdm_spin_dependent()
        return np.linalg.eigvalsh(aa)[::-1].copy(), np.linalg.eigvalsh(bb)[::-1].copy()

    def has_one_rdm_spin_dependent(self):
        return self.has_one_rdm()

    def has_one_rdm_spin_traced(self):
        return self.has_one_rdm()

    def has_active_one_rdm(self):
        return self.has_one_rdm()

    def has_two_rdm_spin_dependent(self):
        return self.has_two_rdm()

    def has_two_rdm_spin_traced(self):
        return self.has_two_rdm()

    def has_active_two_rdm(self):
        return self.has_two_rdm()

    def get_configurations(self):
        return [determinants.to_canonical_string(a, b, self.norb) for a, b in zip(self.alpha, self.beta)]

    def has_one_rdm(self):
        return "aa" in self._rdms

    def has_two_rdm(self):
        return "aaaa" in self._rdms

    def get_active_one_rdm_spin_dependent(self):
        if not self.has_one_rdm():
            raise RuntimeError("one-body RDM was not requested (calculate_one_rdm)")
        return self._rdms["aa"], self._rdms["bb"]

    def get_active_one_rdm_spin_traced(self):
        aa, bb = self.get_active_one_rdm_spin_dependent()
        return aa + bb

    def get_active_two_rdm_spin_dependent(self):
        """(aabb, aaaa, bbbb), flattened column-major, times 2 as qdk stores them."""
        if not self.has_two_rdm():
            raise RuntimeError("two-body RDM was not requested (calculate_two_rdm)")
        f = lambda t: 2.0 * t.ravel(order="F")
        return f(self._rdms["aabb"]), f(self._rdms["aaaa"]), f(self._rdms["bbbb"])

    # Entropies follow WavefunctionContainer (cpp/src/qdk/chemistry/data/
    # wavefunction.cpp:556-685): stored values first; otherwise single-orbital
    # entropies come from the spin-dependent 1- and 2-RDMs, and two-orbital
    # entropies and mutual information from each other with s1.
    def has_single_orbital_entropies(self):
        return "s1" in self._ent or (self.has_one_rdm() and self.has_two_rdm())

    def has_two_orbital_entropies(self):
        return "s2" in self._ent or ("mi" in self._ent and self.has_single_orbital_entropies())

    def has_mutual_information(self):
        return "mi" in self._ent or ("s2" in self._ent and self.has_single_orbital_entropies())

    def get_single_orbital_entropies(self):
        if "s1" in self._ent:
            return self._ent["s1"]
        if not (self.has_one_rdm() and self.has_two_rdm()):
            raise RuntimeError("Spin-dependent one- and two-body RDMs must be set to evaluate "
                               "single-orbital entropies")
        i = np.arange(self.norb)
        # the qdk-normalised aabb element (ii|ii) is <n_ia n_ib> (twice the
        # stored half-convention block)
        s1 = single_orbital_entropies(self._rdms["aa"][i, i], self._rdms["bb"][i, i],
                                      2.0 * self._rdms["aabb"][i, i, i, i])
        self._ent["s1"] = s1
        return s1

    def get_two_orbital_entropies(self):
        if "s2" in self._ent:
            return self._ent["s2"]
        if "mi" in self._ent and self.has_single_orbital_entropies():
            s1 = self.get_single_orbital_entropies()
            s2 = s1[:, None] + s1[None, :] - self._ent["mi"]
            np.fill_diagonal(s2, 0.0)
            self._ent["s2"] = s2
            return s2
        raise RuntimeError("Two-orbital entropies are not available. Provide them at construction time, or "
                           "provide both single-orbital entropies (or RDMs) and mutual information.")

    def get_mutual_information(self):
        if "mi" in self._ent:
            return self._ent["mi"]
        if "s2" in self._ent and self.has_single_orbital_entropies():
            s1 = self.get_single_orbital_entropies()
            mi = s1[:, None] + s1[None, :] - self._ent["s2"]
            np.fill_diagonal(mi, 0.0)
            self._ent["mi"] = mi
            return mi
        raise RuntimeError("Mutual information is not available. Provide it at construction time, or provide "
                           "both single-orbital entropies (or RDMs) and two-orbital entropies.")

    def get_active_two_rdm_spin_traced(self):
        """MACIS spin-traced 2-RDM (E = T.g + V.G): aaaa + bbbb + aabb + aabb^T(rs,pq)."""
        if not self.has_two_rdm():
            raise RuntimeError("two-body RDM was not requested (calculate_two_rdm)")
        r = self._rdms
        return r["aaaa"] + r["bbbb"] + r["aabb"] + r["aabb"].transpose(2, 3, 0, 1)


class MultiConfigurationCalculator:
    """Algorithm::run locks the settings, then calls _run_impl (algorithm.hpp:67-70)."""

    def __init__(self):
        self._settings = self._make_settings()

    def _make_settings(self):
        return Gb300Settings()

    def settings(self):
        return self._settings

    def name(self):
        raise NotImplementedError

    def type_name(self):
        return "multi_configuration_calculator"

    def run(self, hamiltonian, n_alpha, n_beta):
        self._settings.lock()
        return self._run_impl(hamiltonian, int(n_alpha), int(n_beta))

    def _run_impl(self, hamiltonian, n_alpha, n_beta):
        raise NotImplementedError

    # shared by the CI plugins
    def _check_unsupported(self):
        pass

    def _entropies(self, ctx, C):
        """Orbital entropies / mutual information of C over the context's
        determinants when the settings ask for them (form_entropies)."""
        s = self._settings
        w1 = s.get("calculate_single_orbital_entropies")
        w2 = s.get("calculate_two_orbital_entropies")
        wm = s.get("calculate_mutual_information")
        if not (w1 or w2 or wm):
            return None
        s1, s2, mi = ctx.orbital_entropies(C, two_orbital=w2, mutual_information=wm)
        out = {"s1": s1}
        if w2:
            out["s2"] = s2
        if wm:
            out["mi"] = mi
        return out

    def _davidson_limits(self, n):
        """(residual tolerance, subspace size) for an n-dimensional problem."""
        s = self._settings
        tol = s.get("ci_residual_tolerance")
        max_m = s.get("max_solver_iterations")
        if n <= s.get("iterative_solver_dimension_cutoff"):
            # the reference diagonalises small spaces densely (macis_cas.cpp:89-101);
            # here the same Davidson runs to a tight residual (an exact eigenpair
            # up to rounding) with room for the whole space
            tol = min(tol, 1e-10)
            max_m = max(2, min(n, 254))
        return tol, min(max_m, 254)

    def _solve(self, ctx, hamiltonian, a, b):
        """H build + Davidson (+ RDMs) on a determinant list; returns (E_total, Wavefunction)."""
        s = self._settings
        prec = s.get("precision")
        if prec not in ("fp64", "mixed"):
            raise ValueError("precision must be 'fp64' or 'mixed'")
        mixed = prec == "mixed"
        ctx.set_dets(a, b)
        tol, max_m = self._davidson_limits(len(a))
        # the stored matrix when it fits on the device, else (complete spaces,
        # e.g. CAS(14e,14o)) the direct sigma
        layout = ctx.build_operator(s.get("ci_matel_tol"), capi.H_SPLIT32 if mixed else capi.H_FP64, max_m)
        E, C, info = ctx.davidson(max_m=max_m, tol=tol, precision=capi.PREC_MIXED if mixed else capi.PREC_FP64)
        info["operator"] = layout
        rdms = None
        want = []
        if s.get("calculate_one_rdm"):
            want += ["aa", "bb"]
        if s.get("calculate_two_rdm"):
            want += ["aaaa", "bbbb", "aabb"]
        if want:
            rdms = ctx.rdms_spin_dep(C, want=tuple(want))
        wfn = Wavefunction(hamiltonian.norb, a, b, C, rdms, self._entropies(ctx, C))
        wfn.info = info
        return E + hamiltonian.get_core_energy(), wfn


class Gb300Cas(MultiConfigurationCalculator):
    """CASCI over the full (n_alpha, n_beta) space (MacisCas, macis_cas.cpp:120-148)."""

    def name(self):
        return "gb300_cas"

    def _run_impl(self, hamiltonian, n_alpha, n_beta):
        self._check_unsupported()
        n = hamiltonian.norb
        if not (0 <= n_alpha <= n and 0 <= n_beta <= n):
            raise ValueError("electron counts must lie in [0, norb]")
        if n > 64:
            raise ValueError("at most 64 active orbitals per spin")
        a, b = capi.fci_dets(n, n_alpha, n_beta)
        with capi.Context(self._settings.get("device")) as ctx:
            if self._settings.get("device_memory_limit"):
                ctx.set_device_limit(self._settings.get("device_memory_limit"))
            ctx.set_integrals(hamiltonian.get_one_body_integrals(), hamiltonian.get_two_body_integrals())
            return self._solve(ctx, hamiltonian, a, b)


def check_growth_settings(grow_factor, min_grow_factor, backoff_rate, recovery_rate):
    """The growth settings as get_asci_settings_ checks them before any work
    (cpp/src/qdk/chemistry/algorithms/microsoft/macis_base.cpp:101-124)."""
    if not grow_factor > 1.0:
        raise RuntimeError("grow_factor must be > 1.0, got %f" % grow_factor)
    if not min_grow_factor > 1.0:
        raise RuntimeError("min_grow_factor must be > 1.0, got %f" % min_grow_factor)
    if min_grow_factor > grow_factor:
        raise RuntimeError("min_grow_factor must be <= grow_factor")
    if not 0.0 < backoff_rate < 1.0:
        raise RuntimeError("growth_backoff_rate must be in (0, 1), got %f" % backoff_rate)
    if not recovery_rate > 1.0:
        raise RuntimeError("growth_recovery_rate must be > 1.0, got %f" % recovery_rate)


class Gb300AsciSettings(Gb300Settings):
    """MacisAsciSettings names and defaults (macis_asci.hpp:36-189, from
    ASCISettings, determinant_search.hpp:95-199)."""

    def __init__(self):
        super().__init__()
        self.set_default("ntdets_max", int, 100000, "Maximum number of determinants", (1, 2 ** 63 - 1))
        self.set_default("ntdets_min", int, 100, "Minimum number of determinants", (1, 2 ** 63 - 1))
        self.set_default("ncdets_max", int, 100, "Maximum number of core determinants", (1, 2 ** 63 - 1))
        self.set_default("search_matel_tol", float, 1e-8, "ASCI search matrix element threshold", (0.0, 1.0))
        self.set_default("rv_prune_tol", float, 1e-8, "ASCI score pruning threshold", (0.0, 1.0))
        self.set_default("refine_energy_tol", float, 1e-6, "refinement energy tolerance", (0.0, 1.0))
        self.set_default("grow_factor", float, 8.0, "growth factor", (1.0, 1e6))
        self.set_default("min_grow_factor", float, 1.01, "minimum growth factor", (1.0, 1e6))
        self.set_default("growth_backoff_rate", float, 0.5, "grow factor backoff", (0.0, 1.0))
        self.set_default("growth_recovery_rate", float, 1.1, "grow factor recovery", (1.0, 1e6))
        self.set_default("max_refine_iter", int, 6, "maximum refinement iterations", (0, 2 ** 63 - 1))
        self.set_default("core_selection_strategy", str, "percentage", "'percentage' or 'fixed'",
                         ["percentage", "fixed"])
        self.set_default("core_selection_threshold", float, 0.95, "core weight fraction", (0.0, 1.0))
        self.set_default("warm_start_davidson", bool, True)
        self.set_default("min_warm_start_overlap", float, 0.5, "", (0.0, 1.0))
        # ASCI-PT2 (asci_pt2, pt2.hpp:59-565): pt2_tol drops single contributions
        # |c <Q|H|P>| below it.  The reference's work-split knobs (constraint
        # levels, big-constraint threshold, reserve and prune of its pair
        # buffers, next-value batching) are accepted with their defaults; the
        # GPU search and PT2 split the target space by a hash instead.
        big = 2 ** 63 - 1
        self.set_default("pt2_tol", float, 1e-16, "PT2 correction tolerance", (0.0, 1.0))
        self.set_default("pt2_reserve_count", int, 70000000, "Reserve count for PT2 calculations", (0, big))
        self.set_default("pt2_prune", bool, False)
        self.set_default("pt2_precompute_eps", bool, False)
        self.set_default("pt2_precompute_idx", bool, False)
        self.set_default("pt2_print_progress", bool, False)
        self.set_default("pt2_bigcon_thresh", int, 250, "Threshold for using bigcon PT2 algorithm", (0, big))
        self.set_default("pair_size_max", int, 500000000, "Maximum number of ASCI contribution pairs", (1, big))
        self.set_default("nxtval_bcount_thresh", int, 1000, "Threshold for next value batch count", (1, big))
        self.set_default("nxtval_bcount_inc", int, 10, "Increment for next value batch count", (1, big))
        self.set_default("constraint_level", int, 2, "Constraint level for excitation generation", (0, big))
        self.set_default("pt2_max_constraint_level", int, 5, "Maximum constraint level for PT2", (0, big))
        self.set_default("pt2_min_constraint_level", int, 0, "Minimum constraint level for PT2", (0, big))
        self.set_default("pt2_constraint_refine_force", int, 0, "Force constraint refinement for PT2", (0, big))
        # grow-phase controls (determinant_search.hpp:136-198, macis_asci.hpp:93-182)
        self.set_default("grow_ci_residual_tolerance", float, 0.0,
                         "CI residual tolerance during grow phase (0 = use refine tolerance)", (0.0, 1.0))
        self.set_default("taper_grow_factor", float, 0.0,
                         "Growth factor for final expansion near ntdets_max (0 = disabled)", (0.0, 1e6))
        self.set_default("just_singles", bool, False)
        self.set_default("grow_with_rot", bool, False)
        self.set_default("rot_size_start", int, 1000, "Starting size for rotations", (1, big))
        # H-build variants of the reference (the same matrix; one GPU build here)
        self.set_default("hamiltonian_build_algorithm", str, "",
                         "'' or 'sorted_double_loop' (default), 'residue_arrays', 'dynamic_bit_masking'")
        self.set_default("dynamic_bit_masking_num_masks", int, 0, "Number of bit masks (0 = generator default)",
                         (0, big))
        self.set_default("min_patch_overlap", float, 0.3, "Minimum determinant overlap for incremental H build",
                         (0.0, 1.0))


class Gb300Asci(MultiConfigurationCalculator):
    """Selected CI grown by ASCI (MacisAsci, macis_asci.cpp:44-234): the full
    space when ntdets_max exceeds its dimension, otherwise asci_grow from the
    Hartree-Fock determinant then asci_refine (when max_refine_iter > 0)."""

    def _make_settings(self):
        return Gb300AsciSettings()

    def name(self):
        return "gb300_asci"

    def _run_impl(self, hamiltonian, n_alpha, n_beta):
        self._check_unsupported()
        s = self._settings
        n = hamiltonian.norb
        if not (0 <= n_alpha <= n and 0 <= n_beta <= n):
            raise ValueError("electron counts must lie in [0, norb]")
        strategy = s.get("core_selection_strategy").lower()
        if strategy not in ("percentage", "fixed"):
            raise ValueError("Invalid core_selection_strategy: '%s'. Valid options are 'fixed' or 'percentage'."
                             % strategy)
        check_growth_settings(s.get("grow_factor"), s.get("min_grow_factor"), s.get("growth_backoff_rate"),
                              s.get("growth_recovery_rate"))
        thr = s.get("core_selection_threshold")
        if strategy == "percentage" and not (np.finfo(np.float64).eps <= thr <= 1.0):
            raise ValueError("core_selection_threshold must be in [epsilon, 1.0], got %f" % thr)
        if s.get("hamiltonian_build_algorithm") not in ("", "sorted_double_loop", "residue_arrays",
                                                        "dynamic_bit_masking"):
            raise ValueError("Unknown hamiltonian_build_algorithm: '%s'" % s.get("hamiltonian_build_algorithm"))
        # the reference's H-build variants give the same matrix as the one GPU
        # build, so that setting is accepted as it is
        from math import comb
        if s.get("ntdets_max") > comb(n, n_alpha) * comb(n, n_beta):
            return Gb300Cas._run_impl(self, hamiltonian, n_alpha, n_beta)
        prec = s.get("precision")
        with capi.Context(s.get("device")) as ctx:
            ctx.set_integrals(hamiltonian.get_one_body_integrals(), hamiltonian.get_two_body_integrals())
            a0, b0 = determinants.canonical_hf(n_alpha, n_beta)
            ctx.set_dets([a0], [b0])
            # E0 = <HF|H|HF> (macis_asci.cpp:159-163)
            ctx.build_hamiltonian(0.0)
            E0 = float(ctx.diagonal()[0])
            kw = dict(
                max_m=min(s.get("max_solver_iterations"), 254),
                precision=capi.PREC_MIXED if prec == "mixed" else capi.PREC_FP64, matel_tol=s.get("ci_matel_tol"),
                ntdets_max=s.get("ntdets_max"), ntdets_min=s.get("ntdets_min"), ncdets_max=s.get("ncdets_max"),
                core_selection_fixed=1 if strategy == "fixed" else 0,
                core_selection_threshold=s.get("core_selection_threshold"), h_el_tol=s.get("search_matel_tol"),
                rv_prune_tol=s.get("rv_prune_tol"), grow_factor=s.get("grow_factor"),
                min_grow_factor=s.get("min_grow_factor"), growth_backoff_rate=s.get("growth_backoff_rate"),
                growth_recovery_rate=s.get("growth_recovery_rate"), max_refine_iter=s.get("max_refine_iter"),
                refine_energy_tol=s.get("refine_energy_tol"), warm_start=int(s.get("warm_start_davidson")),
                min_warm_start_overlap=s.get("min_warm_start_overlap"), taper_grow_factor=s.get("taper_grow_factor"),
                just_singles=int(s.get("just_singles")), min_patch_overlap=s.get("min_patch_overlap"),
                grow_with_rot=int(s.get("grow_with_rot")), rot_size_start=s.get("rot_size_start"))
            tol = s.get("ci_residual_tolerance")
            grow_tol = s.get("grow_ci_residual_tolerance")
            refine = s.get("max_refine_iter") > 0
            if grow_tol > 0.0:
                # asci_grow with its own CI tolerance (grow.hpp:73-78), then
                # asci_refine with the main one
                E, a, b, C, _ = capi.asci(ctx, [a0], [b0], [1.0], E0, grow=True, refine=False, tol=grow_tol, **kw)
                rot = capi.asci_rotation(ctx)
                if refine:
                    E, a, b, C, _ = capi.asci(ctx, a, b, C, E, grow=False, refine=True, tol=tol, **kw)
            else:
                E, a, b, C, _ = capi.asci(ctx, [a0], [b0], [1.0], E0, grow=True, refine=refine, tol=tol, **kw)
                rot = capi.asci_rotation(ctx)
            rdms = None
            want = []
            if s.get("calculate_one_rdm"):
                want += ["aa", "bb"]
            if s.get("calculate_two_rdm"):
                want += ["aaaa", "bbbb", "aabb"]
            ent = None
            if want or any(s.get(k) for k in ("calculate_single_orbital_entropies",
                                               "calculate_two_orbital_entropies", "calculate_mutual_information")):
                ctx.set_dets(a, b)
                if want:
                    rdms = ctx.rdms_spin_dep(C, want=tuple(want))
                ent = self._entropies(ctx, C)
        wfn = Wavefunction(n, a, b, C, rdms, ent)
        if s.get("grow_with_rot"):
            # the determinants, coefficients and RDMs refer to the natural
            # orbitals of the grow (columns over the given active orbitals),
            # as the reference's generator holds them after asci_grow
            wfn.info = dict(getattr(wfn, "info", None) or {}, orbital_rotation=rot)
        return E + hamiltonian.get_core_energy(), wfn


class ProjectedMultiConfigurationCalculator(MultiConfigurationCalculator):
    """run(hamiltonian, configurations) -> (total energy, Wavefunction): the
    projected multi-configuration calculator (pmc.hpp:31-150): the CI problem
    on a caller's determinant list."""

    def type_name(self):
        return "projected_multi_configuration_calculator"

    def run(self, hamiltonian, configurations):
        self._settings.lock()
        return self._run_impl(hamiltonian, configurations)


def collapse_repeated(alpha, beta):
    """The distinct determinants of a list in spin order (spin_comparator,
    raw_bitset.hpp:119-141), the index of each list position among them, and
    the multiplicity of each."""
    alpha = np.asarray(alpha, dtype=np.uint64)
    beta = np.asarray(beta, dtype=np.uint64)
    order = np.lexsort((beta, alpha))
    sa, sb = alpha[order], beta[order]
    first = np.ones(len(sa), dtype=bool)
    first[1:] = (sa[1:] != sa[:-1]) | (sb[1:] != sb[:-1])
    group = np.cumsum(first) - 1
    inverse = np.empty(len(sa), dtype=np.int64)
    inverse[order] = group
    return sa[first], sb[first], inverse, np.bincount(group)


def multiplicity_scaled(rowptr, colind, values, mult):
    """The values of M^1/2 H M^1/2 for a CSR H over distinct determinants and
    their multiplicities M."""
    w = np.sqrt(np.asarray(mult, dtype=np.float64))
    rows = np.repeat(np.arange(len(rowptr) - 1), np.diff(rowptr))
    return values * w[rows] * w[np.asarray(colind)]


def repeated_list_solution(E, y, inverse, mult):
    """The lowest eigenpair of a repeated list's matrix H' = P H P^T from the
    lowest eigenpair (E, y) of M^1/2 H M^1/2: (E, C = P M^-1/2 y) when E <= 0,
    else (0, the difference of the first repeated pair over sqrt 2); with
    c = P^T C = M^1/2 y (zero for the latter), the sum of C over the copies of
    each distinct determinant.  Returns (E', C, c)."""
    mult = np.asarray(mult)
    if E > 0.0:
        k = int(np.flatnonzero(mult[inverse] > 1)[0])
        pair = np.flatnonzero(inverse == inverse[k])[:2]
        C = np.zeros(len(inverse))
        C[pair] = np.array([1.0, -1.0]) / np.sqrt(2.0)
        return 0.0, C, np.zeros(len(mult))
    w = np.sqrt(mult.astype(np.float64))
    return E, y[inverse] / w[inverse], y * w


def add_repeated_pair_terms(rdms, norb, alpha_u, beta_u, C, c, inverse):
    """form_rdms over a list with repeats (sorted_double_loop.hpp:560-620)
    visits each unordered pair of list positions once: two copies k < l of a
    determinant add its diagonal contribution (rdms.hpp:439-516) once with
    C_k C_l, where a pair of different determinants adds both orderings.  The
    result is the RDMs of c = P^T C plus, for each distinct determinant u,
    delta_u = (sum_{k in u} C_k^2 - c_u^2) / 2 times the RDMs of u alone
    (gamma = diag(n), Gamma_ppqq = n_p n_q / 2, minus n_p n_q / 2 at pqqp
    within a spin).  Adds that second part to the blocks present in rdms."""
    s_u = np.bincount(inverse, weights=np.asarray(C) ** 2, minlength=len(c))
    delta = 0.5 * (s_u - np.asarray(c) ** 2)
    keep = np.abs(delta) > 0.0
    if not np.any(keep):
        return
    bits = np.arange(norb, dtype=np.uint64)
    na = ((alpha_u[keep][:, None] >> bits) & np.uint64(1)).astype(np.float64)
    nb = ((beta_u[keep][:, None] >> bits) & np.uint64(1)).astype(np.float64)
    d = delta[keep]
    i = np.arange(norb)
    P, Q = i[:, None], i[None, :]
    if "aa" in rdms:
        rdms["aa"][i, i] += d @ na
    if "bb" in rdms:
        rdms["bb"][i, i] += d @ nb
    for key, occ in (("aaaa", na), ("bbbb", nb)):
        if key in rdms:
            M = 0.5 * (occ.T * d) @ occ
            rdms[key][P, P, Q, Q] += M
            rdms[key][P, Q, Q, P] -= M
    if "aabb" in rdms:
        rdms["aabb"][P, P, Q, Q] += 0.5 * (nb.T * d) @ na


class Gb300Pmc(ProjectedMultiConfigurationCalculator):
    """MacisPmc (macis_pmc.cpp:42-178): H build and Davidson on the given
    configurations, in their order (canonical strings '2', 'u', 'd', '0' per
    orbital, or (alpha, beta) bit-string pairs); one determinant gives <D|H|D>.
    The list is solved in spin order and the coefficients come back in the
    caller's order (the eigenpair does not depend on the order).  A list that
    repeats determinants gets the reference's answer for the list as given
    (see ``_run_repeated``).
    With calculate_one_rdm / calculate_two_rdm the wavefunction carries the
    RDMs (the reference forms the spin-traced ones, macis_pmc.cpp:126-161; here
    the spin-resolved blocks are kept and the traced views derive from them)."""

    def name(self):
        return "gb300_pmc"

    @staticmethod
    def _parse(configurations, norb):
        a, b = [], []
        for cfg in configurations:
            if isinstance(cfg, str):
                if set(cfg) - set("2ud0"):
                    raise ValueError("configuration '%s': characters must be '2', 'u', 'd' or '0'" % cfg)
                if len(cfg) < norb:
                    raise RuntimeError("Configuration orbital capacity does not match Hamiltonian active space.")
                x, y = determinants.from_canonical_string(cfg[:norb])
                if any(ch not in "0" for ch in cfg[norb:]):
                    raise ValueError("configuration '%s' occupies orbitals beyond the active space" % cfg)
            else:
                x, y = int(cfg[0]), int(cfg[1])
                if norb < 64 and ((x >> norb) or (y >> norb)):
                    raise ValueError("configuration occupies orbitals beyond the active space")
            a.append(x)
            b.append(y)
        return np.array(a, dtype=np.uint64), np.array(b, dtype=np.uint64)

    def _run_impl(self, hamiltonian, configurations):
        self._check_unsupported()
        configurations = list(configurations)
        if not configurations:
            raise RuntimeError("Configuration basis cannot be empty")
        n = hamiltonian.norb
        if n > 64:
            raise ValueError("at most 64 active orbitals per spin")
        a, b = self._parse(configurations, n)
        ua, ub, inverse, mult = collapse_repeated(a, b)
        if len(ua) < len(a):
            return self._run_repeated(hamiltonian, a, b, ua, ub, inverse, mult)
        with capi.Context(self._settings.get("device")) as ctx:
            ctx.set_integrals(hamiltonian.get_one_body_integrals(), hamiltonian.get_two_body_integrals())
            if len(a) == 1:
                # a single determinant: E = <D|H|D>, C = [1] (macis_pmc.cpp:93-96)
                ctx.set_dets(a, b)
                ctx.build_hamiltonian(0.0)
                E = float(ctx.diagonal()[0])
                C = np.ones(1)
                rdms = None
                want = self._rdm_blocks()
                if want:
                    rdms = ctx.rdms_spin_dep(C, want=want)
                return E + hamiltonian.get_core_energy(), Wavefunction(n, a, b, C, rdms, self._entropies(ctx, C))
            # solved on the spin-sorted list (the layout the H build groups by
            # alpha string), the CI vector returned in the caller's order
            order = np.lexsort((b, a))
            E, ws = self._solve(ctx, hamiltonian, a[order], b[order])
            C = np.empty_like(ws.coefficients)
            C[order] = ws.coefficients
            wfn = Wavefunction(n, a, b, C, ws._rdms, ws._ent)
            wfn.info = ws.info
            return E, wfn

    def _run_repeated(self, hamiltonian, a, b, ua, ub, inverse, mult):
        """A list that names some determinant more than once.  MacisPmc solves
        the matrix of the list as given (macis_pmc.cpp:93-116), in which two
        copies of a determinant couple by its diagonal element
        (sorted_double_loop.hpp:296-323): H' = P H P^T, P mapping each list
        position to its distinct determinant.  The eigenpairs of H' with a
        nonzero eigenvalue are those of A = M^1/2 H M^1/2 (M: the
        multiplicities), mapped back as C = P M^-1/2 y; the others have
        eigenvalue 0.  A is solved on the device (H build on the distinct
        determinants in spin order, multiplicity scaling, Davidson in FP64); if
        its lowest eigenvalue is positive the lowest of H' is 0, with the
        difference of the first repeated pair as the vector.  The RDMs of C
        over the list (form_rdms, macis_pmc.cpp:126-161) are formed on the
        device for c = P^T C = M^1/2 y over the distinct determinants, plus the
        once-counted pairs of copies (add_repeated_pair_terms); entropies are
        formed from the state c / |c|."""
        s = self._settings
        n = hamiltonian.norb
        with capi.Context(s.get("device")) as ctx:
            ctx.set_integrals(hamiltonian.get_one_body_integrals(), hamiltonian.get_two_body_integrals())
            ctx.set_dets(ua, ub)
            ctx.build_hamiltonian(s.get("ci_matel_tol"), capi.H_FP64)
            info = None
            if len(ua) == 1:
                E, y = float(ctx.diagonal()[0]) * float(mult[0]), np.ones(1)
            else:
                rp, ci, nz = ctx.get_csr()
                ctx.set_csr(rp, ci, multiplicity_scaled(rp, ci, nz, mult))
                tol, max_m = self._davidson_limits(len(ua))
                E, y, info = ctx.davidson(max_m=max_m, tol=tol, precision=capi.PREC_FP64)
            E, C, c = repeated_list_solution(E, y, inverse, mult)
            want = self._rdm_blocks()
            rdms = None
            if want:
                rdms = ctx.rdms_spin_dep(c, want=want)
                add_repeated_pair_terms(rdms, n, ua, ub, C, c, inverse)
            nc = float(np.linalg.norm(c))
            ent = self._entropies(ctx, c / nc) if nc > 0.0 else None
        wfn = Wavefunction(n, a, b, C, rdms, ent)
        wfn.info = info
        return E + hamiltonian.get_core_energy(), wfn

    def _rdm_blocks(self):
        s = self._settings
        want = []
        if s.get("calculate_one_rdm"):
            want += ["aa", "bb"]
        if s.get("calculate_two_rdm"):
            want += ["aaaa", "bbbb", "aabb"]
        return tuple(want)


class ActiveSpaceSelector:
    """run(wavefunction) -> Wavefunction over the selected active orbitals
    (active_space.hpp); Algorithm::run locks the settings first."""

    def __init__(self):
        self._settings = self._make_settings()

    def settings(self):
        return self._settings

    def type_name(self):
        return "active_space_selector"

    def run(self, wavefunction):
        self._settings.lock()
        return self._run_impl(wavefunction)


class AutocasSettings(Settings):
    """AutocasActiveSpaceSettings (autocas_active_space.hpp:37-56)."""

    def __init__(self):
        super().__init__()
        self.set_default("num_bins", int, 100, "Number of bins for entropy discretization", (2, 2 ** 63 - 1))
        self.set_default("min_plateau_size", int, 10, "Minimum size of entropy plateau to be considered",
                         (1, 2 ** 63 - 1))
        self.set_default("entropy_threshold", float, 0.14,
                         "Minimum absolute entropy value the plateau has to be above")
        self.set_default("normalize_entropies", bool, True)


class AutocasEosSettings(Settings):
    """AutocasEosActiveSpaceSettings (entropy_active_space.hpp:40-46)."""

    def __init__(self):
        super().__init__()
        self.set_default("normalize_entropies", bool, True)
        self.set_default("diff_threshold", float, 0.1)
        self.set_default("entropy_threshold", float, 0.14)


def sorted_entropies_and_indices(wavefunction, normalize):
    """_sort_entropies_and_indices (active_space.cpp:46-117): the single-orbital
    entropies of the wavefunction's active orbitals in descending order with
    their orbital indices, normalised by the largest when asked (and that
    largest is above machine epsilon).  Returns (max entropy, indices,
    sorted entropies)."""
    if not wavefunction.has_single_orbital_entropies():
        raise RuntimeError("Wavefunction does not have single orbital entropies.")
    s1 = np.asarray(wavefunction.get_single_orbital_entropies(), dtype=np.float64)
    idx = wavefunction.get_active_indices()
    if len(s1) != len(idx):
        raise RuntimeError("Entropy size does not match number of active space orbitals.")
    order = np.argsort(-s1, kind="stable")
    ent = s1[order]
    indices = [idx[i] for i in order]
    mx = float(ent.max()) if len(ent) else 0.0
    if normalize and mx > np.finfo(np.float64).eps:
        ent = ent / mx
    return mx, indices, ent


def selected_active_wavefunction(wavefunction, selected):
    """new_orbitals + new_wavefunction (active_space.cpp:119-376) for a
    restricted wavefunction: the selected orbitals (sorted) must lie in its
    active space; the result holds one determinant over them, that of a
    one-determinant wavefunction or else the aufbau determinant of the active
    electrons, with the occupations of the selected orbitals
    (_extract_active_orbitals :281-321); the inactive orbitals are the lowest
    nelec/2 not selected (_get_inactive_space_indices :220-239)."""
    selected = sorted(int(i) for i in selected)
    old = wavefunction.get_active_indices()
    for i in selected:
        if i not in old:
            raise RuntimeError("Selected orbital (index: %d) is outside of initial active space." % i)
    na, nb = wavefunction.get_active_num_electrons()
    if wavefunction.size() == 1:
        da, db = int(wavefunction.alpha[0]), int(wavefunction.beta[0])
    else:
        da, db = (1 << na) - 1, (1 << nb) - 1
    a = b = 0
    for k, i in enumerate(selected):
        p = old.index(i)
        a |= ((da >> p) & 1) << k
        b |= ((db >> p) & 1) << k
    ta, tb = wavefunction.get_total_num_electrons()
    inactive = [i for i in range((ta + tb) // 2) if i not in selected]
    return Wavefunction(len(selected), np.array([a], np.uint64), np.array([b], np.uint64), np.ones(1),
                        active_indices=selected, inactive_indices=inactive)


class Gb300Autocas(ActiveSpaceSelector):
    """AutocasActiveSpaceSelector (autocas_active_space.cpp:15-160): bins the
    (normalised) single-orbital entropies, finds plateaus of equal "orbitals
    above the bin" counts at least min_plateau_size bins long, and keeps the
    orbitals counted at the start of the largest one; no orbital is kept when
    the largest raw entropy is below entropy_threshold."""

    def _make_settings(self):
        return AutocasSettings()

    def name(self):
        return "gb300_autocas"

    def select(self, wavefunction):
        s = self._settings
        mx, indices, ent = sorted_entropies_and_indices(wavefunction, s.get("normalize_entropies"))
        if mx < s.get("entropy_threshold"):
            return []
        nbins = s.get("num_bins")
        bins = np.arange(nbins) * (1.0 / nbins)
        above = [int(np.count_nonzero(ent > t)) for t in bins]
        plateaus, start = [], 0
        for i in range(1, nbins):
            if above[i] != above[i - 1]:
                if i - start >= s.get("min_plateau_size"):
                    plateaus.append(start)
                start = i
        if nbins - start >= s.get("min_plateau_size"):
            plateaus.append(start)
        sizes = [above[p] for p in plateaus if above[p] > 0]
        return sorted(indices[:max(sizes) if sizes else 0])

    def _run_impl(self, wavefunction):
        return selected_active_wavefunction(wavefunction, self.select(wavefunction))


class Gb300AutocasEos(ActiveSpaceSelector):
    """AutocasEosActiveSpaceSelector (entropy_active_space.cpp:14-87): keeps
    the largest k whose k-th sorted (normalised) entropy lies above
    entropy_threshold (normalised by the largest entropy when asked) and drops
    to the next one by more than diff_threshold."""

    def _make_settings(self):
        return AutocasEosSettings()

    def name(self):
        return "gb300_autocas_eos"

    def select(self, wavefunction):
        s = self._settings
        norm = s.get("normalize_entropies")
        mx, indices, ent = sorted_entropies_and_indices(wavefunction, norm)
        thr = s.get("entropy_threshold")
        if norm:
            with np.errstate(divide="ignore", invalid="ignore"):
                thr = np.float64(thr) / np.float64(mx)
        diff = ent[:-1] - ent[1:]
        sizes = [i + 1 for i in range(len(diff)) if ent[i] > thr and diff[i] > s.get("diff_threshold")]
        return sorted(indices[:max(sizes) if sizes else 0])

    def _run_impl(self, wavefunction):
        return selected_active_wavefunction(wavefunction, self.select(wavefunction))


_REGISTRY = {"multi_configuration_calculator": {"gb300_cas": Gb300Cas, "gb300_asci": Gb300Asci},
             "projected_multi_configuration_calculator": {"gb300_pmc": Gb300Pmc},
             "active_space_selector": {"gb300_autocas": Gb300Autocas, "gb300_autocas_eos": Gb300AutocasEos}}
_DEFAULT = {"multi_configuration_calculator": "gb300_cas",
            "projected_multi_configuration_calculator": "gb300_pmc",
            "active_space_selector": "gb300_autocas_eos"}


def register(generator):
    """register (python/src/qdk_chemistry/algorithms/registry.py:496-538,
    register_instance algorithm.hpp:310): the algorithm type and name come from
    an instance; a name already taken raises DuplicateRegistrationError, an
    unknown type KeyError."""
    inst = generator()
    kind = inst.type_name()
    if kind not in _REGISTRY:
        raise KeyError("Algorithm type '%s' is not registered. Available algorithm types: %s"
                       % (kind, ", ".join(sorted(_REGISTRY))))
    if inst.name() in _REGISTRY[kind]:
        raise DuplicateRegistrationError("'%s' is already registered as a %s" % (inst.name(), kind))
    _REGISTRY[kind][inst.name()] = generator


def available(kind=None):
    """The registered names of one algorithm type, or a dict over all types
    (registry.py available)."""
    if kind is None:
        return {k: sorted(v) for k, v in _REGISTRY.items()}
    return sorted(_REGISTRY.get(kind, {}))


def create(kind, name=None, **settings):
    """create(kind, name, **settings) (registry.py:295-372): the default name
    of the type when none is given (mc.hpp:213, pmc.hpp:186,
    active_space.hpp:206), then the keyword settings applied."""
    if kind not in _REGISTRY:
        raise KeyError("unknown algorithm type '%s'" % kind)
    name = name or _DEFAULT.get(kind)
    if name not in _REGISTRY[kind]:
        raise KeyError("no '%s' named '%s' (available: %s)" % (kind, name, ", ".join(available(kind))))
    alg = _REGISTRY[kind][name]()
    for key, value in settings.items():
        alg.settings().set(key, value)
    return alg


def inspect_settings(kind, name):
    """The settings schema of one implementation (registry.py:428-494): a
    (name, python type, default, description or None, limits or None) tuple
    per setting."""
    s = create(kind, name).settings()
    return [(k, s.get_expected_python_type(k), s.get(k), s.get_description(k) if s.has_description(k) else None,
             s.get_limits(k) if s.has_limits(k) else None) for k in s.keys()]


def show_default(kind=None):
    """The default name of one algorithm type ('' for an unknown one), or a
    dict over all types (registry.py:593-632)."""
    if kind is None:
        return dict(_DEFAULT)
    return _DEFAULT.get(kind, "")


def unregister(kind, name):
    """Remove a registered implementation (registry.py:635-663)."""
    if kind not in _REGISTRY or name not in _REGISTRY[kind]:
        raise KeyError("no '%s' named '%s' is registered" % (kind, name))
    del _REGISTRY[kind][name]


def davidson_solver(csr_matrix, tol=1e-8, max_m=20, device=0):
    """Lowest eigenpair of a symmetric scipy CSR matrix on the GPU
    (davidson_solver.cpp:60-107: diagonal guess, macis::davidson)."""
    A = csr_matrix.tocsr()
    A.sort_indices()
    with capi.Context(device) as ctx:
        ctx.set_csr(A.indptr, A.indices, A.data)
        E, X, _ = ctx.davidson(max_m=max_m, tol=tol)
    return E, X
