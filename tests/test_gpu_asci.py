"""GPU ASCI (search, grow, refine) against the oracle and the reference's
golden energies.  Selected determinant sets are compared as sets, bit-exact;
energies to 1e-8 Eh (the reference's davidson_tolerance)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(pkg):
    pkg.build.build()
    c = pkg.capi.Context(0)
    yield c
    c.close()


def _as_set(a, b):
    return set(zip(a.tolist(), b.tolist()))


def test_asci_search_selected_set_matches_oracle(ctx, pkg, oracle, h2o):
    """One search step from a water wavefunction of 800 determinants (core =
    the 100 largest), asking for 6400: the GPU set equals the oracle's set."""
    H = oracle.Hamiltonian(h2o["T"], h2o["V"])
    a0, b0 = pkg.determinants.canonical_hf(5, 5)
    E0 = H.matrix_element((a0, b0), (a0, b0))
    E, a, b, c, _ = oracle.asci(H, [a0], [b0], [1.0], E0, ntdets_max=800, core_fixed=1, max_refine_iter=0,
                                refine=False)
    order = np.argsort(-np.abs(c), kind="stable")[:100]
    ca, cb, cc = a[order], b[order], c[order]
    srt = np.lexsort((cb, ca))
    ca, cb, cc = ca[srt], cb[srt], cc[srt]
    oa, ob = oracle.asci_search(H, ca, cb, cc, E, 6400)
    ctx.set_integrals(h2o["T"], h2o["V"])
    ga, gb = pkg.capi.asci_search(ctx, ca, cb, cc, E, 6400)
    assert len(ga) == len(oa) == 6400
    assert _as_set(ga, gb) == _as_set(oa, ob)


def test_asci_water_10k_golden(ctx, pkg, oracle, h2o, known):
    """external/macis/tests/asci.cxx:488-574 on the GPU path."""
    ref = known["h2o_asci_10k"]
    H = oracle.Hamiltonian(h2o["T"], h2o["V"])
    a0, b0 = pkg.determinants.canonical_hf(5, 5)
    E0 = H.matrix_element((a0, b0), (a0, b0))
    ctx.set_integrals(h2o["T"], h2o["V"])
    E, a, b, c, Eg = pkg.capi.asci(ctx, [a0], [b0], [1.0], E0, ntdets_max=10000, core_selection_fixed=1)
    assert abs(Eg - ref["E0_grow"]) < 1e-8
    assert abs(E - ref["E0_refine"]) < 1e-8
    assert len(a) == 10000 and abs(c @ c - 1) < 1e-12
    Eo, oa, ob, oc, _ = oracle.asci(H, [a0], [b0], [1.0], E0, ntdets_max=10000, core_fixed=1)
    assert _as_set(a, b) == _as_set(oa, ob)


def test_asci_n2_golden(ctx, pkg, oracle, n2_14e18o, known):
    """external/macis/python/tests/test_pymacis.py:158-187 on the GPU path."""
    ref = known["n2_14e18o_asci"]
    H = oracle.Hamiltonian(n2_14e18o["T"], n2_14e18o["V"])
    a0, b0 = pkg.determinants.canonical_hf(7, 7)
    E0 = H.matrix_element((a0, b0), (a0, b0))
    ctx.set_integrals(n2_14e18o["T"], n2_14e18o["V"])
    E, a, b, c, _ = pkg.capi.asci(ctx, [a0], [b0], [1.0], E0, ntdets_max=ref["ntdets_max"],
                                  grow_factor=ref["grow_factor"], max_refine_iter=ref["max_refine_iter"], max_m=254)
    assert abs(E - ref["E_total"]) < 1e-8
    assert len(a) == ref["ndets"]


@pytest.mark.late
def test_asci_just_singles_and_taper_match_oracle(ctx, pkg, oracle, h2o):
    """The search's just_singles (determinant_search.hpp:274-296) and the
    grow's taper_grow_factor (grow.hpp:97-107) on the GPU against the oracle:
    a singles-only search from a 100-determinant water core asked for more
    determinants than exist (no cut-off, so no tie at a boundary) gives the
    oracle's set; a tapered grow to 1000 determinants reaches the oracle's
    energy (1e-6: a borderline tie may differ in one determinant)."""
    H = oracle.Hamiltonian(h2o["T"], h2o["V"])
    a0, b0 = pkg.determinants.canonical_hf(5, 5)
    E0 = H.matrix_element((a0, b0), (a0, b0))
    E, a, b, c, _ = oracle.asci(H, [a0], [b0], [1.0], E0, ntdets_max=100, core_fixed=1, refine=False)
    srt = np.lexsort((b, a))
    ca, cb, cc = a[srt], b[srt], c[srt]
    oa, ob = oracle.asci_search(H, ca, cb, cc, E, 10 ** 6, just_singles=1)
    ctx.set_integrals(h2o["T"], h2o["V"])
    ga, gb = pkg.capi.asci_search(ctx, ca, cb, cc, E, 10 ** 6, just_singles=1)
    assert len(oa) < 10 ** 6 and _as_set(ga, gb) == _as_set(oa, ob)
    Eg, ta, _, tc, _ = pkg.capi.asci(ctx, [a0], [b0], [1.0], E0, refine=False, ntdets_max=1000,
                                     core_selection_fixed=1, taper_grow_factor=1.1)
    Eo, oa, _, _, _ = oracle.asci(H, [a0], [b0], [1.0], E0, refine=False, ntdets_max=1000, core_fixed=1,
                                  taper_grow_factor=1.1)
    assert len(ta) >= 1000 and abs(tc @ tc - 1) < 1e-12 and abs(Eg - Eo) < 1e-6


def test_asci_grow_repeats_bit_for_bit(pkg):
    """Two grows from the same start on the same context select the same
    determinants in the same order with bit-identical coefficients and
    energy: the search's sums and diagonals do not depend on the order in
    which its atomics land.  The phase timer reports every phase."""
    import os

    from conftest import GOLDEN, unpack_eri
    capi = pkg.capi
    d = np.load(os.path.join(GOLDEN, "ref_asci40.npz"))
    norb = int(d["norb"])
    a0, b0 = pkg.determinants.canonical_hf(int(d["nalpha"]), int(d["nbeta"]))
    runs = []
    with capi.Context(0) as ctx:
        ctx.set_integrals(d["T"], unpack_eri(d["V_packed"], norb))
        ctx.set_dets(np.array([a0], np.uint64), np.array([b0], np.uint64))
        ctx.build_hamiltonian()
        E0 = float(ctx.diagonal()[0])
        for _ in range(2):
            _, a, b, c, Eg = capi.asci(ctx, [a0], [b0], [1.0], E0, grow=True, refine=False, ntdets_max=50000,
                                       core_selection_fixed=1, ncdets_max=10000, grow_factor=8)
            runs.append((a, b, c, Eg, capi.asci_phase_times(ctx)))
    (a1, b1, c1, E1, t1), (a2, b2, c2, E2, _) = runs
    assert np.array_equal(a1, a2) and np.array_equal(b1, b2)
    assert np.array_equal(c1.view(np.uint64), c2.view(np.uint64)) and E1 == E2
    assert t1["iterations"] > 0 and all(t1[k] > 0 for k in ("search_s", "det_space_s", "hbuild_s", "davidson_s"))


def test_asci_patched_hamiltonian_equals_full_rebuild(pkg, monkeypatch):
    """The ASCI iterations patch the previous iteration's Hamiltonian (new
    rows and long kept rows walked, the new rows' elements transposed into
    the kept rows, the kept rows merged with their renumbered old rows).  The
    patched CSR equals a rebuild of the same list element for element, and a
    grow followed by refine iterations gives bit-identical determinants,
    coefficients, energies and final matrices with every Hamiltonian rebuilt
    (QDKGB_ASCI_FULL_BUILD=1).  The 40-orbital space's reference determinant
    has rows longer than the merge buffer, so the long-row walk is covered."""
    import os

    from conftest import GOLDEN, unpack_eri
    pkg.build.build()
    capi = pkg.capi
    d = np.load(os.path.join(GOLDEN, "ref_asci40.npz"))
    norb = int(d["norb"])
    a0, b0 = pkg.determinants.canonical_hf(int(d["nalpha"]), int(d["nbeta"]))
    out = {}
    for full in (False, True):
        monkeypatch.setenv("QDKGB_ASCI_FULL_BUILD", "1" if full else "0")
        with capi.Context(0) as ctx:
            ctx.set_integrals(d["T"], unpack_eri(d["V_packed"], norb))
            ctx.set_dets(np.array([a0], np.uint64), np.array([b0], np.uint64))
            ctx.build_hamiltonian()
            E0 = float(ctx.diagonal()[0])
            _, a, b, c, Eg = capi.asci(ctx, [a0], [b0], [1.0], E0, grow=True, refine=False, ntdets_max=30000,
                                       core_selection_fixed=1, ncdets_max=3000, grow_factor=2)
            tg = capi.asci_phase_times(ctx)
            grown = ctx.get_csr(64)
            ctx.set_dets(a, b)
            ctx.build_hamiltonian()
            rebuilt = ctx.get_csr(64)
            for x, y in zip(grown, rebuilt):
                assert np.array_equal(x.view(np.uint64) if x.dtype == np.float64 else x,
                                      y.view(np.uint64) if y.dtype == np.float64 else y)
            with pytest.raises(capi.NotConverged):
                capi.asci(ctx, a, b, c, Eg, grow=False, refine=True, core_selection_fixed=1, ncdets_max=3000,
                          ntdets_max=30000, max_refine_iter=3, refine_energy_tol=1e-14)
            tr = capi.asci_phase_times(ctx)
            out[full] = (a, b, c, Eg, ctx.get_csr(64), tg, tr)
    (a1, b1, c1, E1, H1, tg1, tr1), (a2, b2, c2, E2, H2, tg2, tr2) = out[False], out[True]
    assert tg1["patched_builds"] > 0 and tr1["patched_builds"] > 0
    assert tg2["patched_builds"] == 0 and tr2["patched_builds"] == 0
    assert np.array_equal(a1, a2) and np.array_equal(b1, b2)
    assert np.array_equal(c1.view(np.uint64), c2.view(np.uint64)) and E1 == E2
    for x, y in zip(H1, H2):
        assert np.array_equal(x.view(np.uint64) if x.dtype == np.float64 else x,
                              y.view(np.uint64) if y.dtype == np.float64 else y)


def test_grow_with_rotation_matches_oracle(pkg, oracle, h2o):
    """Natural-orbital rotation during the grow (grow_with_rot,
    grow.hpp:163-252) on the GPU against the oracle's restatement on water:
    the same selected determinants, energies within 1e-8 Eh, rotations equal
    up to the sign of each orbital; the context keeps the rotated integrals,
    and the rotation is the identity without grow_with_rot."""
    pkg.build.build()
    capi = pkg.capi
    H = oracle.Hamiltonian(h2o["T"], h2o["V"])
    n = H.n
    E_hf = H.matrix_element((31, 31), (31, 31))
    kw = dict(ntdets_max=400, core_selection_fixed=1, ncdets_max=50, grow_factor=2.0, grow_with_rot=1,
              rot_size_start=100)
    Uo = np.zeros((n, n))
    Eo, oa, ob, oc, Ego = oracle.asci(H, [31], [31], [1.0], E_hf, grow=True, refine=False, rotation=Uo,
                                      ntdets_max=400, core_fixed=1, ncdets_max=50, grow_factor=2.0,
                                      grow_with_rot=1, rot_size_start=100)
    with capi.Context(0) as ctx:
        ctx.set_integrals(h2o["T"], h2o["V"])
        Eg, ga, gb, gc, Egg = capi.asci(ctx, [31], [31], [1.0], E_hf, grow=True, refine=False, **kw)
        Ug = capi.asci_rotation(ctx)
        assert abs(Egg - Ego) < 1e-8 and abs(Eg - Eo) < 1e-8
        assert _as_set(ga, gb) == _as_set(oa, ob)
        overlap = np.abs(Ug.T @ Uo)
        assert np.max(np.abs(overlap - np.eye(n))) < 1e-6
        capi.asci(ctx, [31], [31], [1.0], E_hf, grow=True, refine=False, ntdets_max=100,
                  core_selection_fixed=1, ncdets_max=50)
        assert np.array_equal(capi.asci_rotation(ctx), np.eye(n))
