"""C ABI checks that need no GPU: the library builds/loads, exports every
function declared in include/qdkgb.h, host-only entry points work, and the
device entry points fail with a status code (not a crash) without a GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def _declared():
    text = open(os.path.join(ROOT, "include", "qdkgb.h")).read()
    return sorted(set(re.findall(r"\b(qdkgb_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def capi(pkg):
    pkg.build.build()
    return pkg.capi


def test_exports_every_declared_symbol(capi):
    L = capi.lib()
    declared = _declared()
    assert len(declared) >= 19
    for name in declared:
        assert hasattr(L, name), name
    assert set(capi.EXPORTED) <= set(declared)
    assert b"sm_103a" in L.qdkgb_version()


def test_fci_dets_host_order(capi, oracle):
    for n, na, nb in [(6, 3, 3), (8, 4, 3), (12, 6, 6), (40, 1, 1)]:
        a, b = capi.fci_dets(n, na, nb)
        oa, ob = oracle.fci_dets(n, na, nb)
        assert np.array_equal(a, oa) and np.array_equal(b, ob)


def test_fci_dets_rejects_bad_arguments(capi):
    n = ctypes.c_int64()
    assert capi.lib().qdkgb_fci_dets(0, 1, 1, None, None, ctypes.byref(n)) == capi.ERR_INVALID
    assert capi.lib().qdkgb_fci_dets(8, 9, 1, None, None, ctypes.byref(n)) == capi.ERR_INVALID
    assert capi.lib().qdkgb_fci_dets(65, 1, 1, None, None, ctypes.byref(n)) == capi.ERR_INVALID


def test_null_context_is_an_error_not_a_crash(capi):
    L = capi.lib()
    assert L.qdkgb_set_dets(None, 1, None, None) == capi.ERR_INVALID
    assert L.qdkgb_build_hamiltonian(None, 0.0, 0, None) == capi.ERR_INVALID
    assert L.qdkgb_set_device_limit(None, 1 << 20) == capi.ERR_INVALID
    assert L.qdkgb_destroy(None) == capi.OK


def test_noalloc_rejects_rows_beyond_the_limit(capi):
    # the size check of the allocation-free sigma runs before any pointer is
    # touched or any CUDA call is made, so it is checked without a GPU
    with pytest.raises(capi.QdkgbError) as ei:
        capi.sigma_split_noalloc(capi.NOALLOC_MAX_ROWS + 1, 16, 16, 16, 16, 16, 16)
    assert ei.value.code == capi.ERR_INVALID
    assert "QDKGB_NOALLOC_MAX_ROWS" in str(ei.value)
    with pytest.raises(capi.QdkgbError) as ei:
        capi.sigma_split_noalloc(-1, 16, 16, 16, 16, 16, 16)
    assert ei.value.code == capi.ERR_INVALID


def test_create_without_gpu_reports_status(capi):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    rc = capi.lib().qdkgb_create(ctypes.byref(h), 0)
    assert rc != capi.OK and not h.value


def test_default_settings_mirror_reference(capi):
    s = capi.default_davidson_settings()
    # ci_max_subspace / max_solver_iterations 200, ci_res_tol 1e-8, clamp 1e-12
    assert s.max_m == 200 and s.res_tol == 1e-8 and s.min_abs_denominator == 1e-12


def test_mcscf_and_pt2_defaults(pkg):
    """qdkgb_mcscf_default_settings = MCSCFSettings (external/macis/include/
    macis/mcscf/mcscf.hpp:22-52); host-only, no device needed."""
    capi = pkg.capi
    s = capi.default_mcscf_settings()
    assert s.max_macro_iter == 100 and s.max_orbital_step == 0.5 and s.orb_grad_tol == 5e-6
    assert s.enable_diis == 1 and s.diis_start_iter == 3 and s.diis_nkeep == 10
    assert s.ci_res_tol == 1e-8 and s.ci_max_subspace == 200 and s.ci_matel_tol == np.finfo(float).eps
    s2 = capi.default_mcscf_settings(orb_grad_tol=1e-7)
    assert s2.orb_grad_tol == 1e-7
    with pytest.raises(KeyError):
        capi.default_mcscf_settings(no_such_setting=1)


def test_settings_struct_layouts_match(pkg):
    """Each C default-settings call writes exactly the ctypes mirror: called on
    a buffer longer than the mirror and filled with a sentinel byte, it leaves
    the tail untouched, and every ASCI field reads back its default
    (qdkgb_asci_default_settings)."""
    capi = pkg.capi
    L = capi.lib()
    for cls, fn in ((capi.AsciSettings, L.qdkgb_asci_default_settings),
                    (capi.DavidsonSettings, L.qdkgb_davidson_default_settings),
                    (capi.McscfSettings, L.qdkgb_mcscf_default_settings),
                    (capi.BatchSettings, L.qdkgb_batch_default_settings)):
        n = ctypes.sizeof(cls)
        buf = (ctypes.c_ubyte * (n + 64))(*([0xAB] * (n + 64)))
        fn(ctypes.cast(buf, ctypes.POINTER(cls)))
        assert bytes(buf[n:]) == b"\xab" * 64, cls.__name__
    s = capi.default_asci_settings()
    want = dict(ntdets_max=100000, ntdets_min=100, ncdets_max=100, core_selection_fixed=0,
                core_selection_threshold=0.95, h_el_tol=1e-8, rv_prune_tol=1e-8, grow_factor=8.0,
                min_grow_factor=1.01, growth_backoff_rate=0.5, growth_recovery_rate=1.1, max_refine_iter=6,
                refine_energy_tol=1e-6, warm_start=1, min_warm_start_overlap=0.5, taper_grow_factor=0.0,
                just_singles=0, min_patch_overlap=0.3, grow_with_rot=0, rot_size_start=1000)
    assert [f for f, _ in capi.AsciSettings._fields_] == list(want)
    assert {k: getattr(s, k) for k in want} == want
