"""Golden fixtures made by the reference's own MACIS code at the sizes of the
benchmark configurations (test infrastructure).

The reference is compiled from its unmodified sources by oracle/build_ref.sh
(project-written API shims for BLAS++/LAPACK++, mdspan and spdlog in
oracle/ref_shims) and called through oracle/macis_ref.py.  Run it where the
reference checkout exists, giving its path:

    python tests/golden/make_ref_golden.py REFERENCE_CHECKOUT [cas8 cas12 batch asci40 ...]

Each fixture stores the integrals it was made from (so that machines whose
BLAS rounds the synthetic recipe differently still test the same matrix), the
reference's results, and SHA-256 digests of the reference's CSR arrays
(int64 row pointers and columns, FP64 values) for bit-exact comparisons of
matrices too large to commit:

* ref_cas8.npz   - CASCI(8e,8o), 16 Cholesky vectors (the CPU-runnable
  configuration): CSR digests, E and Davidson iterations, the CI vector,
  spin-resolved and spin-traced RDMs, the two lowest roots by lobpcgxx.
* ref_cas12.npz  - CASCI(12e,12o), 24 Cholesky vectors (the headline
  configuration, 853,776 determinants, 1,553,018,544 elements): CSR digests,
  E, iterations, a sample of rows, the 1-RDMs.
* ref_batch10.npz - the first norb = 10 instances of the 512-instance batch:
  E and 1-RDMs.
* ref_asci40.npz - ASCI over 40 orbitals, 8 + 8 electrons, Fixed core 10,000,
  grow factor 8 (diagonal spacing 0.1, 80 Cholesky vectors), grown to
  200,000 determinants: E and the selected set (SHA-256 of the list sorted by
  (alpha, beta), plus its first and last 512 entries).  V is stored as its
  unique elements (conftest.pack_eri).
"""
import hashlib
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

SEED = 20261203          # the benchmark's integral seed
BATCH_SEED = 20261204    # the batched configuration's seed
EPS = float(np.finfo(np.float64).eps)


def digest(arr):
    return hashlib.sha256(memoryview(np.ascontiguousarray(arr)).cast("B")).hexdigest()


def _pkg():
    from conftest import load_package
    return load_package()


def cas_fixture(R, name, norb, nel, nchol, seed, rdm2=True, lobpcg=False, sample_rows=()):
    pkg = _pkg()
    T, V, _ = pkg.integrals.synthetic_integrals(norb, nchol, seed)
    a, b = R.fci_dets(norb, nel // 2, nel // 2)
    t0 = time.time()
    M = R.Csr(norb, T, V, a, b, EPS)
    rp, ci, nz = M.views()
    t_build = time.time() - t0
    out = dict(T=T, V=V, norb=norb, nalpha=nel // 2, nbeta=nel // 2, nchol=nchol, seed=seed, ndets=len(a),
               nnz=len(nz), sha_rowptr=digest(rp), sha_colind=digest(ci), sha_nzval=digest(nz),
               sha_alpha=digest(a), sha_beta=digest(b))
    rows = [r for r in sample_rows if r < len(a)]
    out["sample_rows"] = np.array(rows, np.int64)
    for r in rows:
        out["row%d_colind" % r] = ci[rp[r]:rp[r + 1]].copy()
        out["row%d_nzval" % r] = nz[rp[r]:rp[r + 1]].copy()
    t0 = time.time()
    E, C, info = M.selected_ci_diag(max_m=200, tol=1e-8)
    t_dav = time.time() - t0
    out.update(E=E, iterations=info["iterations"], sigma_calls=info["sigma_calls"])
    if len(a) <= 100000:
        out["C"] = C
    if lobpcg:
        rng = np.random.default_rng(7)
        X = rng.normal(size=(len(a), 4))
        ev, Xr, res = M.lobpcg(X, 2, tol=1e-9, max_iter=2000)
        out.update(lobpcg_evals=ev, lobpcg_res=res)
    del M
    t0 = time.time()
    if rdm2:
        r = R.rdms_spin_dep(norb, T, V, a, b, C)
        for k, v in r.items():
            out["rdm_" + k] = v
        o1, o2 = R.rdms(norb, T, V, a, b, C)
        out.update(rdm_traced1=o1, rdm_traced2=o2)
    else:
        r = R.rdms_spin_dep(norb, T, V, a, b, C)
        out.update(rdm_aa=r["aa"], rdm_bb=r["bb"])
        out["rdm_aabb_norm"] = float(np.linalg.norm(r["aabb"]))
        out["rdm_aaaa_norm"] = float(np.linalg.norm(r["aaaa"]))
    t_rdm = time.time() - t0
    out["seconds"] = np.array([t_build, t_dav, t_rdm])
    path = os.path.join(HERE, name)
    np.savez_compressed(path, **out)
    print("%s: ndets %d nnz %d E %.12f iters %d (build %.1f s, Davidson %.1f s, RDMs %.1f s)"
          % (name, len(a), len(nz), E, info["iterations"], t_build, t_dav, t_rdm))


def batch_fixture(R, count=3):
    pkg = _pkg()
    rng = np.random.default_rng(BATCH_SEED)
    norbs = rng.choice((6, 8, 10), size=512)
    picked = [i for i, no in enumerate(norbs) if no == 10][:count]
    out = dict(index=np.array(picked, np.int64))
    E, aa, bb = [], [], []
    for i in picked:
        T, V, _ = pkg.integrals.synthetic_integrals(10, 20, BATCH_SEED + 1 + i)
        a, b = R.fci_dets(10, 5, 5)
        M = R.Csr(10, T, V, a, b, EPS)
        e, C, _ = M.selected_ci_diag(max_m=200, tol=1e-8)
        r = R.rdms_spin_dep(10, T, V, a, b, C)
        E.append(e)
        aa.append(r["aa"])
        bb.append(r["bb"])
        out["T%d" % i], out["V%d" % i] = T, V
    out.update(E=np.array(E), rdm_aa=np.array(aa), rdm_bb=np.array(bb))
    np.savez_compressed(os.path.join(HERE, "ref_batch10.npz"), **out)
    print("ref_batch10: instances %s E %s" % (picked, E))


def asci_fixture(R, ndets=200000):
    pkg = _pkg()
    norb, nel, nchol = 40, 16, 80
    T, V, _ = pkg.integrals.synthetic_integrals(norb, nchol, SEED, diag_spacing=0.1)
    a0, b0 = pkg.determinants.canonical_hf(nel // 2, nel // 2)
    import oracle
    E0 = oracle.Hamiltonian(T, V).matrix_element((a0, b0), (a0, b0))
    t0 = time.time()
    E, a, b, c, Eg = R.asci(norb, T, V, [a0], [b0], [1.0], E0, grow=True, refine=False, ntdets_max=ndets,
                            core_fixed=1, ncdets_max=10000, grow_factor=8)
    dt = time.time() - t0
    from conftest import pack_eri, unpack_eri
    Vp = pack_eri(V)
    assert np.array_equal(unpack_eri(Vp, norb), V)
    order = np.lexsort((b, a))  # sorted by (alpha, beta)
    sa, sb = a[order], b[order]
    out = dict(T=T, V_packed=Vp, norb=norb, nalpha=nel // 2, nbeta=nel // 2, ntdets_max=ndets, E_grow=Eg,
               ndets=len(a), sha_sorted_alpha=digest(sa), sha_sorted_beta=digest(sb), head_alpha=sa[:512],
               head_beta=sb[:512], tail_alpha=sa[-512:], tail_beta=sb[-512:], seconds=dt)
    np.savez_compressed(os.path.join(HERE, "ref_asci40.npz"), **out)
    print("ref_asci40: %d determinants E %.12f (%.1f s)" % (len(a), Eg, dt))


def main(argv):
    if len(argv) < 2:
        sys.exit(__doc__)
    os.environ["QDK_REFERENCE"] = argv[1]
    import oracle.macis_ref as R
    R.build(force=True)
    which = argv[2:] or ["cas8", "batch", "asci40", "cas12"]
    if "cas8" in which:
        cas_fixture(R, "ref_cas8.npz", 8, 8, 16, SEED, rdm2=True, lobpcg=True, sample_rows=(0, 1, 2450, 4899))
    if "batch" in which:
        batch_fixture(R)
    if "asci40" in which:
        asci_fixture(R)
    if "cas12" in which:
        cas_fixture(R, "ref_cas12.npz", 12, 12, 24, SEED, rdm2=False,
                    sample_rows=(0, 1, 924, 426888, 853775))


if __name__ == "__main__":
    main(sys.argv)
