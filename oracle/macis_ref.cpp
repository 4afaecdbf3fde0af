// Test infrastructure only (never linked into the product): a C-ABI driver
// around the reference's own MACIS code, compiled from the unmodified
// reference headers by oracle/build_ref.sh against the project-written
// shims in oracle/ref_shims.  It exists to produce golden fixtures from the
// reference itself (tests/golden/make_ref_golden.py) and to pin the oracle
// restatement (oracle/macis_oracle.cpp) against it.
//
// Every entry point calls the reference's functions:
//   generate_hilbert_space            include/macis/sd_operations.hpp:333-351
//   make_csr_hamiltonian<int64_t>     include/macis/csr_hamiltonian.hpp:41-55
//     (SortedDoubleLoopHamiltonianGenerator, sorted_double_loop.hpp:86-451)
//   extract_diagonal_elements + diagonal_guess + davidson, the body of
//     serial_selected_ci_diag         include/macis/solvers/selected_ci_diag.hpp:111-158
//   form_rdms_spin_dep / form_rdms    sorted_double_loop.hpp:512-753
//   asci_grow / asci_refine           include/macis/asci/grow.hpp, refine.hpp
//   lobpcgxx::lobpcg                  src/lobpcgxx/include/lobpcgxx/lobpcg.hpp
#include <macis/asci/grow.hpp>
#include <macis/asci/refine.hpp>
#include <macis/csr_hamiltonian.hpp>
#include <macis/hamiltonian_generator/sorted_double_loop.hpp>
#include <macis/mcscf/mcscf.hpp>
#include <macis/sd_operations.hpp>
#include <macis/solvers/davidson.hpp>
#include <macis/solvers/selected_ci_diag.hpp>
#include <lobpcgxx/lobpcg.hpp>

#include <cstdint>
#include <cstring>
#include <exception>
#include <string>
#include <vector>

namespace {
thread_local std::string g_err;

using csr64 = sparsexx::csr_matrix<double, int64_t>;

// determinants cross this boundary as (alpha, beta) uint64 pairs; MACIS keeps
// them in one bitset<N> with alpha in the low N/2 bits (raw_bitset.hpp:55-106)
template <size_t N>
std::vector<macis::wfn_t<N>> to_bitsets(int64_t n, const uint64_t* a, const uint64_t* b) {
  std::vector<macis::wfn_t<N>> d(n);
  for (int64_t i = 0; i < n; ++i) {
    macis::wfn_t<N> x;
    for (size_t k = 0; k < 64 && k < N / 2; ++k) {
      if ((a[i] >> k) & 1ull) x.set(k);
      if ((b[i] >> k) & 1ull) x.set(k + N / 2);
    }
    d[i] = x;
  }
  return d;
}
template <size_t N>
void from_bitsets(const std::vector<macis::wfn_t<N>>& d, uint64_t* a, uint64_t* b) {
  for (size_t i = 0; i < d.size(); ++i) {
    uint64_t x = 0, y = 0;
    for (size_t k = 0; k < 64 && k < N / 2; ++k) {
      if (d[i][k]) x |= 1ull << k;
      if (d[i][k + N / 2]) y |= 1ull << k;
    }
    a[i] = x;
    b[i] = y;
  }
}

template <typename F>
int guarded(F&& f) {
  try {
    f();
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return 1;
  } catch (...) {
    g_err = "unknown exception";
    return 1;
  }
}

// counts operator applications so the Davidson iteration count is visible
struct CountingOp {
  const macis::SparseMatrixOperator<csr64>& op;
  mutable int64_t calls = 0;
  void operator_action(size_t m, double alpha, const double* V, size_t LDV, double beta, double* AV,
                       size_t LDAV) const {
    ++calls;
    op.operator_action(m, alpha, V, LDV, beta, AV, LDAV);
  }
};

template <size_t N>
csr64* build_csr_n(int norb, double* T, double* V, int64_t n, const uint64_t* a, const uint64_t* b,
                   double thresh) {
  using gen_t = macis::SortedDoubleLoopHamiltonianGenerator<macis::wfn_t<N>>;
  gen_t gen(macis::matrix_span<double>(T, norb, norb), macis::rank4_span<double>(V, norb, norb, norb, norb));
  auto dets = to_bitsets<N>(n, a, b);
  return new csr64(macis::make_csr_hamiltonian<int64_t>(dets.begin(), dets.end(), gen, thresh));
}

template <size_t N>
void rdms_n(int norb, double* T, double* V, int64_t n, const uint64_t* a, const uint64_t* b, const double* C,
            double* aa, double* bb, double* aaaa, double* bbbb, double* aabb) {
  using gen_t = macis::SortedDoubleLoopHamiltonianGenerator<macis::wfn_t<N>>;
  gen_t gen(macis::matrix_span<double>(T, norb, norb), macis::rank4_span<double>(V, norb, norb, norb, norb));
  auto dets = to_bitsets<N>(n, a, b);
  const size_t no = norb;
  gen.form_rdms_spin_dep(dets.begin(), dets.end(), dets.begin(), dets.end(), const_cast<double*>(C),
                         macis::matrix_span<double>(aa, no, no), macis::matrix_span<double>(bb, no, no),
                         macis::rank4_span<double>(aaaa, no, no, no, no),
                         macis::rank4_span<double>(bbbb, no, no, no, no),
                         macis::rank4_span<double>(aabb, no, no, no, no));
}

template <size_t N>
void rdms_traced_n(int norb, double* T, double* V, int64_t n, const uint64_t* a, const uint64_t* b, const double* C,
                   double* ordm, double* trdm) {
  using gen_t = macis::SortedDoubleLoopHamiltonianGenerator<macis::wfn_t<N>>;
  gen_t gen(macis::matrix_span<double>(T, norb, norb), macis::rank4_span<double>(V, norb, norb, norb, norb));
  auto dets = to_bitsets<N>(n, a, b);
  const size_t no = norb;
  gen.form_rdms(dets.begin(), dets.end(), dets.begin(), dets.end(), const_cast<double*>(C),
                macis::matrix_span<double>(ordm, no, no), macis::rank4_span<double>(trdm, no, no, no, no));
}
}  // namespace

extern "C" {

const char* ref_last_error() { return g_err.c_str(); }

int ref_fci_dets(int norb, int na, int nb, int64_t* n, uint64_t* a, uint64_t* b) {
  return guarded([&] {
    auto d = macis::generate_hilbert_space<macis::wfn_t<64>>(norb, na, nb);
    if (a && b) from_bitsets<64>(d, a, b);
    *n = (int64_t)d.size();
  });
}

// norb <= 32 uses wfn_t<64> (alpha in the low 32 bits), larger wfn_t<128>,
// as the reference's calculators pick the bitset width
int ref_build_csr(int norb, double* T, double* V, int64_t n, const uint64_t* a, const uint64_t* b, double thresh,
                  void** handle) {
  return guarded([&] {
    *handle = norb <= 32 ? (void*)build_csr_n<64>(norb, T, V, n, a, b, thresh)
                         : (void*)build_csr_n<128>(norb, T, V, n, a, b, thresh);
  });
}

int ref_csr_info(void* h, int64_t* m, int64_t* nnz, const int64_t** rowptr, const int64_t** colind,
                 const double** nzval) {
  auto* H = (csr64*)h;
  *m = (int64_t)H->m();
  *nnz = (int64_t)H->nnz();
  *rowptr = H->rowptr().data();
  *colind = H->colind().data();
  *nzval = H->nzval().data();
  return 0;
}

void ref_csr_free(void* h) { delete (csr64*)h; }

// serial_selected_ci_diag's steps (diagonal, identity guess unless C holds a
// usable guess, SparseMatrixOperator, davidson), with the operator counted
int ref_selected_ci_diag(void* h, int64_t max_m, double tol, double* C, double* E, int64_t* iters,
                         int64_t* sigma_calls) {
  return guarded([&] {
    auto& H = *(csr64*)h;
    const int64_t N = (int64_t)H.m();
    std::vector<double> Cv(C, C + N);
    auto D = sparsexx::extract_diagonal_elements(H);
    double max_c = 0;
    for (double c : Cv) max_c = std::max(max_c, std::abs(c));
    if (!(max_c > 1.0 / N)) macis::diagonal_guess(N, H, Cv.data());
    macis::SparseMatrixOperator<csr64> op(H);
    CountingOp cop{op};
    auto [niter, e] = macis::davidson(N, max_m, cop, D.data(), tol, Cv.data());
    std::copy(Cv.begin(), Cv.end(), C);
    *E = e;
    *iters = (int64_t)niter;
    *sigma_calls = cop.calls;
  });
}

int ref_spmv(void* h, const double* x, double* y) {
  return guarded([&] {
    auto& H = *(csr64*)h;
    macis::SparseMatrixOperator<csr64> op(H);
    op.operator_action(1, 1.0, x, H.m(), 0.0, y, H.m());
  });
}

int ref_rdms_spin_dep(int norb, double* T, double* V, int64_t n, const uint64_t* a, const uint64_t* b,
                      const double* C, double* aa, double* bb, double* aaaa, double* bbbb, double* aabb) {
  return guarded([&] {
    if (norb <= 32)
      rdms_n<64>(norb, T, V, n, a, b, C, aa, bb, aaaa, bbbb, aabb);
    else
      rdms_n<128>(norb, T, V, n, a, b, C, aa, bb, aaaa, bbbb, aabb);
  });
}

int ref_rdms(int norb, double* T, double* V, int64_t n, const uint64_t* a, const uint64_t* b, const double* C,
             double* ordm, double* trdm) {
  return guarded([&] {
    if (norb <= 32)
      rdms_traced_n<64>(norb, T, V, n, a, b, C, ordm, trdm);
    else
      rdms_traced_n<128>(norb, T, V, n, a, b, C, ordm, trdm);
  });
}

// lobpcgxx::lobpcg on the CSR (the reference's multi-root solver), nroots
// lowest eigenpairs from the given starting block X (N x k, column major)
int ref_lobpcg(void* h, int64_t k, int64_t nroots, double tol, int64_t max_iter, double* X, double* evals,
               double* res) {
  return guarded([&] {
    auto& H = *(csr64*)h;
    const int64_t N = (int64_t)H.m();
    lobpcgxx::lobpcg_settings settings;
    settings.conv_tol = tol;
    settings.maxiter = max_iter;
    settings.print_iter = false;
    lobpcgxx::lobpcg_operator<double> op([&](int64_t n, int64_t kk, const double* x, int64_t ldx, double* y,
                                             int64_t ldy) {
      sparsexx::spblas::gespmbv(kk, 1.0, H, x, ldx, 0.0, y, ldy);
      (void)n;
    });
    std::vector<double> lam(k), r(k);
    lobpcgxx::lobpcg_convergence<double> conv;
    lobpcgxx::lobpcg(settings, N, k, nroots, op, lam.data(), X, N, r.data(), conv);
    for (int64_t i = 0; i < nroots; ++i) {
      evals[i] = lam[i];
      res[i] = r[i];
    }
  });
}

// asci_grow then asci_refine on wfn_t<128> (norb <= 64), with the oracle's
// settings vector (oracle.py ASCI_DEFAULTS order) mapped onto the reference's
// ASCISettings / MCSCFSettings; returns the determinant count (<= cap
// written), or -1 with the reason in ref_last_error
int64_t ref_asci(int norb, double* T, double* V, const double* set, int64_t n0, const uint64_t* a0,
                 const uint64_t* b0, const double* c0, double E0, int do_grow, int do_refine, int64_t cap,
                 uint64_t* out_a, uint64_t* out_b, double* out_c, double* E_out, double* E_grow_out) {
  int64_t nret = -1;
  int rc = guarded([&] {
    macis::ASCISettings S;
    macis::MCSCFSettings M;
    S.ntdets_max = (size_t)set[0];
    S.ntdets_min = (size_t)set[1];
    S.ncdets_max = (size_t)set[2];
    S.core_selection_strategy =
        set[3] != 0 ? macis::CoreSelectionStrategy::Fixed : macis::CoreSelectionStrategy::Percentage;
    S.core_selection_threshold = set[4];
    S.h_el_tol = set[5];
    S.rv_prune_tol = set[6];
    S.grow_factor = set[7];
    S.min_grow_factor = set[8];
    S.growth_backoff_rate = set[9];
    S.growth_recovery_rate = set[10];
    S.max_refine_iter = (size_t)set[11];
    S.refine_energy_tol = set[12];
    S.warm_start_davidson = set[13] != 0;
    S.min_warm_start_overlap = set[14];
    M.ci_res_tol = set[15];
    M.ci_max_subspace = (size_t)set[16];
    M.ci_matel_tol = set[17];
    S.taper_grow_factor = set[18];
    S.just_singles = set[19] != 0;
    using gen_t = macis::SortedDoubleLoopHamiltonianGenerator<macis::wfn_t<128>>;
    gen_t gen(macis::matrix_span<double>(T, norb, norb), macis::rank4_span<double>(V, norb, norb, norb, norb));
    auto wfn = to_bitsets<128>(n0, a0, b0);
    std::vector<double> X(c0, c0 + n0);
    double E = E0;
    if (do_grow) std::tie(E, wfn, X) = macis::asci_grow<128, int64_t>(S, M, E, wfn, X, gen, norb);
    if (E_grow_out) *E_grow_out = E;
    if (do_refine) std::tie(E, wfn, X) = macis::asci_refine<128, int64_t>(S, M, E, wfn, X, gen, norb);
    *E_out = E;
    nret = (int64_t)wfn.size();
    std::vector<uint64_t> a(wfn.size()), b(wfn.size());
    from_bitsets<128>(wfn, a.data(), b.data());
    for (int64_t i = 0; i < std::min(nret, cap); ++i) {
      out_a[i] = a[i];
      out_b[i] = b[i];
      out_c[i] = X[i];
    }
  });
  return rc ? -1 : nret;
}

}  // extern "C"
