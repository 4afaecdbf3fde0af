// CPU oracle for the selected-CI / CASCI hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file restates, in plain C++ with OpenMP, the
// algorithms of MACIS (external/macis in microsoft/qdk-chemistry) that the GPU
// library replaces.  Only the tests, the smoke check and the CPU-baseline legs
// of the benchmark may load it; the product library never links or calls it.
//
// The MACIS headers themselves cannot be compiled here: they need BLAS++,
// LAPACK++, Kokkos mdspan, spdlog and CMake-generated config headers, none of
// which is present.  So every function below follows the cited reference lines
// step by step, on uint64 spin strings instead of std::bitset.
//
// Conventions (as in MACIS):
//   * T(p,q) = T[p + n*q]; V(p,q,r,s) = V[p + n*q + n^2*r + n^3*s] (column-major).
//   * A determinant is (alpha string, beta string); bit i set = orbital i occupied.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <stdexcept>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

inline int popc(uint64_t x) { return __builtin_popcountll(x); }
// macis::ffs: 1-based index of the lowest set bit, 0 if none
// (external/macis/include/macis/bitset_operations.hpp:240-263).
inline uint32_t ffs1(uint64_t x) { return x ? (uint32_t)__builtin_ctzll(x) + 1u : 0u; }
// macis::full_mask<N>(i): bits [0, i) set (bitset_operations.hpp:230-238).
inline uint64_t full_mask(uint32_t i) { return i >= 64 ? ~0ull : ((1ull << i) - 1ull); }

// sd_operations.hpp:27-30
inline uint32_t first_occupied_flipped(uint64_t state, uint64_t ex) { return ffs1(state & ex) - 1u; }

// sd_operations.hpp:40-50: parity of the occupied orbitals strictly between p and q.
inline double single_excitation_sign(uint64_t state, uint32_t p, uint32_t q) {
  uint64_t mask;
  if (p > q)
    mask = state & (full_mask(p) ^ full_mask(q + 1));
  else
    mask = state & (full_mask(q) ^ full_mask(p + 1));
  return (popc(mask) % 2) ? -1. : 1.;
}

struct Single {
  uint32_t o, v;
  double sign;
};
// sd_operations.hpp:394-402
inline Single single_excitation_sign_indices(uint64_t bra, uint64_t ket, uint64_t ex) {
  uint32_t o1 = first_occupied_flipped(ket, ex);
  uint32_t v1 = first_occupied_flipped(bra, ex);
  double s = single_excitation_sign(ket, v1, o1);
  return {o1, v1, s};
}
struct Double {
  uint32_t o1, v1, o2, v2;
  double sign;
};
// sd_operations.hpp:413-425: apply the first single to the ket, then repeat.
inline Double doubles_sign_indices(uint64_t bra, uint64_t ket, uint64_t ex) {
  Single a = single_excitation_sign_indices(bra, ket, ex);
  ket ^= (1ull << a.o) | (1ull << a.v);
  ex ^= (1ull << a.o) | (1ull << a.v);
  Single b = single_excitation_sign_indices(bra, ket, ex);
  return {a.o, a.v, b.o, b.v, a.sign * b.sign};
}

inline void bits_to_indices(uint64_t x, std::vector<uint32_t>& out) {
  out.clear();
  while (x) {
    out.push_back((uint32_t)__builtin_ctzll(x));
    x &= x - 1;
  }
}

// HamiltonianGeneratorBase: integrals + intermediates
// (src/macis/hamiltonian_generator/base.ipp:27-77).
struct Ham {
  int n = 0;
  std::vector<double> T, V, G_red, V_red, G2_red, V2_red;
  double t(uint32_t p, uint32_t q) const { return T[p + (size_t)n * q]; }
  double v(uint32_t p, uint32_t q, uint32_t r, uint32_t s) const {
    return V[p + (size_t)n * (q + (size_t)n * (r + (size_t)n * s))];
  }
  void init(int n_, const double* T_, const double* V_) {
    n = n_;
    size_t n2 = (size_t)n * n, n3 = n2 * n, n4 = n3 * n;
    T.assign(T_, T_ + n2);
    V.assign(V_, V_ + n4);
    G_red.assign(n3, 0.);
    V_red.assign(n3, 0.);
    G2_red.assign(n2, 0.);
    V2_red.assign(n2, 0.);
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i)
        for (int k = 0; k < n; ++k) {
          G_red[k + n * (i + (size_t)n * j)] = v(k, k, i, j) - v(k, j, i, k);
          V_red[k + n * (i + (size_t)n * j)] = v(k, k, i, j);
        }
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        G2_red[i + (size_t)n * j] = 0.5 * (v(i, i, j, j) - v(i, j, j, i));
        V2_red[i + (size_t)n * j] = v(i, i, j, j);
      }
  }

  // matrix_elements.hpp:113-121
  double me_4(uint64_t bra, uint64_t ket, uint64_t ex) const {
    Double d = doubles_sign_indices(bra, ket, ex);
    double g = v(d.v1, d.o1, d.v2, d.o2) - v(d.v1, d.o2, d.v2, d.o1);
    return d.sign * g;
  }
  // matrix_elements.hpp:140-151
  double me_22(uint64_t ba, uint64_t ka, uint64_t exa, uint64_t bb, uint64_t kb, uint64_t exb) const {
    Single a = single_excitation_sign_indices(ba, ka, exa);
    Single b = single_excitation_sign_indices(bb, kb, exb);
    double sign = a.sign * b.sign;
    return sign * v(a.v, a.o, b.v, b.o);
  }
  // matrix_elements.hpp:169-189
  double me_2(uint64_t bra, uint64_t ket, uint64_t ex, const std::vector<uint32_t>& occ_same,
              const std::vector<uint32_t>& occ_other) const {
    Single s = single_excitation_sign_indices(bra, ket, ex);
    double h = t(s.v, s.o);
    const double* g = &G_red[(size_t)n * (s.v + (size_t)n * s.o)];
    for (auto p : occ_same) h += g[p];
    const double* vr = &V_red[(size_t)n * (s.v + (size_t)n * s.o)];
    for (auto p : occ_other) h += vr[p];
    return s.sign * h;
  }
  // matrix_elements.hpp:203-230
  double me_diag(const std::vector<uint32_t>& oa, const std::vector<uint32_t>& ob) const {
    double h = 0;
    for (auto p : oa) h += t(p, p);
    for (auto p : ob) h += t(p, p);
    for (auto q : oa)
      for (auto p : oa) h += G2_red[p + (size_t)n * q];
    for (auto q : ob)
      for (auto p : ob) h += G2_red[p + (size_t)n * q];
    for (auto q : ob)
      for (auto p : oa) h += V2_red[p + (size_t)n * q];
    return h;
  }
  // matrix_elements.hpp:65-97
  double me(uint64_t ba, uint64_t bb, uint64_t ka, uint64_t kb) const {
    uint64_t exa = ba ^ ka, exb = bb ^ kb;
    int ca = popc(exa), cb = popc(exb);
    if (ca + cb > 4) return 0.;
    std::vector<uint32_t> oa, ob;
    bits_to_indices(ba, oa);
    bits_to_indices(bb, ob);
    if (ca == 4) return me_4(ba, ka, exa);
    if (cb == 4) return me_4(bb, kb, exb);
    if (ca == 2 && cb == 2) return me_22(ba, ka, exa, bb, kb, exb);
    if (ca == 2) return me_2(ba, ka, exa, oa, ob);
    if (cb == 2) return me_2(bb, kb, exb, ob, oa);
    return me_diag(oa, ob);
  }
};

struct Csr {
  int64_t n = 0;
  std::vector<int64_t> rowptr, colind;
  std::vector<double> nzval;
};

// get_unique_alpha (sd_operations.hpp:449-468) plus the offsets scan of
// sorted_double_loop.hpp:105-132.
void unique_alpha(const uint64_t* alpha, int64_t nd, std::vector<uint64_t>& ua, std::vector<int64_t>& off) {
  ua.clear();
  off.clear();
  if (nd == 0) {
    off.push_back(0);
    return;
  }
  ua.push_back(alpha[0]);
  off.push_back(0);
  for (int64_t i = 1; i < nd; ++i)
    if (alpha[i] != ua.back()) {
      ua.push_back(alpha[i]);
      off.push_back(i);
    }
  off.push_back(nd);
}

// SortedDoubleLoopHamiltonianGenerator::make_csr_hamiltonian_block_ for the
// symmetric case (bra list == ket list),
// include/macis/hamiltonian_generator/sorted_double_loop.hpp:86-451:
// count pass (137-225), scan (230-234), fill with atomic slot capture and the
// mirrored entry (254-360), per-row column sort (369-410), and
// threshold_parallel (|h| > thresh kept, csr_matrix.hpp:317-372).
Csr* build_csr_sdl(const Ham& H, const uint64_t* alpha, const uint64_t* beta, int64_t nd, double thresh) {
  std::vector<uint64_t> ua;
  std::vector<int64_t> off;
  unique_alpha(alpha, nd, ua, off);
  const int64_t nu = (int64_t)ua.size();
  std::vector<int64_t> row_nnz(nd, 0);

#pragma omp parallel
  {
    std::vector<int64_t> local(nd, 0);
#pragma omp for schedule(dynamic)
    for (int64_t ib = 0; ib < nu; ++ib) {
      if (!ua[ib]) continue;
      const uint64_t ba = ua[ib];
      for (int64_t ik = ib; ik < nu; ++ik) {
        if (!ua[ik]) continue;
        const uint64_t ka = ua[ik];
        const uint64_t exa = ba ^ ka;
        const int ca = popc(exa);
        if (ca > 4) continue;
        if (ca == 4) {
          double h4 = H.me_4(ba, ka, exa);
          if (std::abs(h4) < thresh) continue;
        }
        for (int64_t i = off[ib]; i < off[ib + 1]; ++i) {
          const uint64_t bb = beta[i];
          for (int64_t j = off[ik]; j < off[ik + 1]; ++j) {
            if (j < i) continue;
            const uint64_t kb = beta[j];
            const uint64_t exb = bb ^ kb;
            const int cb = popc(exb);
            if (ca + cb > 4) continue;
            if (cb == 4) {
              double h4 = H.me_4(bb, kb, exb);
              if (std::abs(h4) < thresh) continue;
            }
            local[i]++;
            if (i != j) local[j]++;
          }
        }
      }
    }
    for (int64_t i = 0; i < nd; ++i)
      if (local[i]) {
#pragma omp atomic
        row_nnz[i] += local[i];
      }
  }

  Csr* M = new Csr;
  M->n = nd;
  M->rowptr.assign(nd + 1, 0);
  for (int64_t i = 0; i < nd; ++i) M->rowptr[i + 1] = M->rowptr[i] + row_nnz[i];
  const int64_t nnz = M->rowptr[nd];
  M->colind.assign(nnz, 0);
  M->nzval.assign(nnz, 0.);
  std::vector<int64_t> slot(M->rowptr.begin(), M->rowptr.end() - 1);

#pragma omp parallel
  {
    std::vector<uint32_t> oa, ob;
#pragma omp for schedule(dynamic)
    for (int64_t ib = 0; ib < nu; ++ib) {
      if (!ua[ib]) continue;
      const uint64_t ba = ua[ib];
      bits_to_indices(ba, oa);
      for (int64_t ik = ib; ik < nu; ++ik) {
        if (!ua[ik]) continue;
        const uint64_t ka = ua[ik];
        const uint64_t exa = ba ^ ka;
        const int ca = popc(exa);
        if (ca > 4) continue;
        for (int64_t i = off[ib]; i < off[ib + 1]; ++i) {
          const uint64_t bb = beta[i];
          bits_to_indices(bb, ob);
          for (int64_t j = off[ik]; j < off[ik + 1]; ++j) {
            if (j < i) continue;
            const uint64_t kb = beta[j];
            const uint64_t exb = bb ^ kb;
            const int cb = popc(exb);
            if (ca + cb > 4) continue;
            double h;
            if (ca == 4) {
              h = H.me_4(ba, ka, exa);
              if (std::abs(h) < thresh) continue;
            } else if (cb == 4) {
              h = H.me_4(bb, kb, exb);
              if (std::abs(h) < thresh) continue;
            } else if (ca == 2) {
              h = (cb == 2) ? H.me_22(ba, ka, exa, bb, kb, exb) : H.me_2(ba, ka, exa, oa, ob);
            } else if (cb == 2) {
              h = H.me_2(bb, kb, exb, ob, oa);
            } else {
              h = H.me_diag(oa, ob);
            }
            int64_t s;
#pragma omp atomic capture
            s = slot[i]++;
            M->colind[s] = j;
            M->nzval[s] = h;
            if (i != j) {
              int64_t s2;
#pragma omp atomic capture
              s2 = slot[j]++;
              M->colind[s2] = i;
              M->nzval[s2] = h;
            }
          }
        }
      }
    }
  }

  // per-row column sort
#pragma omp parallel
  {
    std::vector<int64_t> idx, cols;
    std::vector<double> vals;
#pragma omp for schedule(dynamic)
    for (int64_t i = 0; i < nd; ++i) {
      int64_t st = M->rowptr[i], en = M->rowptr[i + 1];
      int64_t sz = en - st;
      if (sz <= 1) continue;
      idx.resize(sz);
      std::iota(idx.begin(), idx.end(), 0);
      std::sort(idx.begin(), idx.end(), [&](int64_t a, int64_t b) { return M->colind[st + a] < M->colind[st + b]; });
      cols.resize(sz);
      vals.resize(sz);
      for (int64_t k = 0; k < sz; ++k) {
        cols[k] = M->colind[st + idx[k]];
        vals[k] = M->nzval[st + idx[k]];
      }
      std::copy(cols.begin(), cols.end(), M->colind.begin() + st);
      std::copy(vals.begin(), vals.end(), M->nzval.begin() + st);
    }
  }

  // threshold_parallel (csr_matrix.hpp:317-372): keep |h| > thresh.
  if (thresh > 0.0) {
    std::vector<int64_t> nrp(nd + 1, 0);
    int64_t w = 0;
    for (int64_t i = 0; i < nd; ++i) {
      for (int64_t k = M->rowptr[i]; k < M->rowptr[i + 1]; ++k)
        if (std::abs(M->nzval[k]) > thresh) {
          M->nzval[w] = M->nzval[k];
          M->colind[w] = M->colind[k];
          ++w;
        }
      nrp[i + 1] = w;
    }
    M->rowptr = std::move(nrp);
    M->nzval.resize(w);
    M->colind.resize(w);
  }
  return M;
}

// sparsexx::spblas::gespmbv with K=1, alpha=1, beta=0 (spblas/spmbv.hpp:49-85).
void spmv(const Csr& A, const double* x, double* y) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < A.n; ++i) {
    double av = 0.;
    for (int64_t k = A.rowptr[i]; k < A.rowptr[i + 1]; ++k) av += A.nzval[k] * x[A.colind[k]];
    y[i] = av;
  }
}

double dot(int64_t n, const double* a, const double* b) {
  double s = 0.;
#pragma omp parallel for reduction(+ : s) schedule(static)
  for (int64_t i = 0; i < n; ++i) s += a[i] * b[i];
  return s;
}
double nrm2(int64_t n, const double* a) { return std::sqrt(dot(n, a, a)); }

// Symmetric eigensolver for the small Rayleigh-Ritz matrix (stands in for
// lapack::syev at lobpcgxx/rayleigh_ritz.hpp:70-77).  Cyclic Jacobi: A is
// k x k column-major (overwritten with the eigenvectors, ascending order),
// w receives the eigenvalues.
void jacobi_syev(int k, double* A, int lda, double* w) {
  std::vector<double> a((size_t)k * k), q((size_t)k * k, 0.);
  for (int j = 0; j < k; ++j)
    for (int i = 0; i < k; ++i) a[i + (size_t)k * j] = 0.5 * (A[i + (size_t)lda * j] + A[j + (size_t)lda * i]);
  for (int i = 0; i < k; ++i) q[i + (size_t)k * i] = 1.;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0., tot = 0.;
    for (int j = 0; j < k; ++j)
      for (int i = 0; i < k; ++i) {
        double v = a[i + (size_t)k * j] * a[i + (size_t)k * j];
        tot += v;
        if (i != j) off += v;
      }
    if (off <= 1e-32 * tot || off == 0.) break;
    for (int p = 0; p < k - 1; ++p)
      for (int r = p + 1; r < k; ++r) {
        double apq = a[p + (size_t)k * r];
        if (apq == 0.) continue;
        double app = a[p + (size_t)k * p], aqq = a[r + (size_t)k * r];
        double theta = (aqq - app) / (2. * apq);
        double t = (theta >= 0 ? 1. : -1.) / (std::abs(theta) + std::sqrt(theta * theta + 1.));
        double c = 1. / std::sqrt(t * t + 1.), s = t * c;
        for (int i = 0; i < k; ++i) {  // columns p, r
          double aip = a[i + (size_t)k * p], air = a[i + (size_t)k * r];
          a[i + (size_t)k * p] = c * aip - s * air;
          a[i + (size_t)k * r] = s * aip + c * air;
        }
        for (int i = 0; i < k; ++i) {  // rows p, r
          double api = a[p + (size_t)k * i], ari = a[r + (size_t)k * i];
          a[p + (size_t)k * i] = c * api - s * ari;
          a[r + (size_t)k * i] = s * api + c * ari;
        }
        for (int i = 0; i < k; ++i) {
          double qip = q[i + (size_t)k * p], qir = q[i + (size_t)k * r];
          q[i + (size_t)k * p] = c * qip - s * qir;
          q[i + (size_t)k * r] = s * qip + c * qir;
        }
      }
  }
  std::vector<int> ord(k);
  std::iota(ord.begin(), ord.end(), 0);
  std::sort(ord.begin(), ord.end(), [&](int x, int y) { return a[x + (size_t)k * x] < a[y + (size_t)k * y]; });
  for (int j = 0; j < k; ++j) {
    w[j] = a[ord[j] + (size_t)k * ord[j]];
    for (int i = 0; i < k; ++i) A[i + (size_t)lda * j] = q[i + (size_t)k * ord[j]];
  }
}

// gram_schmidt (include/macis/solvers/davidson.hpp:185-238): two classical
// Gram-Schmidt passes, then normalise; canonical-vector fallback.
void gram_schmidt(int64_t N, int64_t K, const double* Vold, double* Vnew, double min_norm = 1e-12) {
  if (K <= 0) {
    double nrm = nrm2(N, Vnew);
    if (nrm > min_norm)
      for (int64_t i = 0; i < N; ++i) Vnew[i] /= nrm;
    return;
  }
  std::vector<double> inner(K);
  auto pass = [&]() {
    for (int64_t k = 0; k < K; ++k) inner[k] = dot(N, Vold + k * N, Vnew);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < N; ++i) {
      double s = 0.;
      for (int64_t k = 0; k < K; ++k) s += Vold[i + k * N] * inner[k];
      Vnew[i] -= s;
    }
  };
  pass();
  pass();
  double nrm = nrm2(N, Vnew);
  if (nrm > min_norm) {
    double sc = 1. / nrm;
    for (int64_t i = 0; i < N; ++i) Vnew[i] *= sc;
    return;
  }
  for (int64_t idx = 0; idx < N; ++idx) {
    std::fill_n(Vnew, N, 0.);
    Vnew[idx] = 1.;
    pass();
    nrm = nrm2(N, Vnew);
    if (nrm > min_norm) {
      double sc = 1. / nrm;
      for (int64_t i = 0; i < N; ++i) Vnew[i] *= sc;
      return;
    }
  }
  throw std::runtime_error("gram_schmidt: Unable to find orthogonal vector");
}

// davidson (include/macis/solvers/davidson.hpp:259-372).  Returns 0 on
// convergence, 1 if max_m iterations passed without it.
int davidson(const Csr& A, int64_t max_m, const double* D, double tol, double* X, double* E_out, int64_t* iters_out,
             double min_abs_denominator = 1e-12) {
  const int64_t N = A.n;
  max_m = std::min<int64_t>(max_m, N);
  if (N == 1) {
    X[0] = 1.;
    double ax;
    spmv(A, X, &ax);
    *E_out = ax;
    *iters_out = 0;
    return 0;
  }
  std::vector<double> V((size_t)N * (max_m + 1)), AV((size_t)N * (max_m + 1)), C((size_t)(max_m + 1) * (max_m + 1)),
      LAM(max_m + 1);
  std::copy_n(X, N, V.begin());
  spmv(A, V.data(), AV.data());
  std::copy_n(AV.data(), N, V.data() + N);
  gram_schmidt(N, 1, V.data(), V.data() + N);
  bool converged = false;
  int64_t iter = 1;
  for (int64_t i = 1; i < max_m; ++i, ++iter) {
    const int64_t k = i + 1;
    spmv(A, V.data() + i * N, AV.data() + i * N);
    // rayleigh_ritz: C = V^T AV, then syev (lobpcgxx/rayleigh_ritz.hpp:70-77)
    for (int64_t c = 0; c < k; ++c)
      for (int64_t r = 0; r < k; ++r) C[r + k * c] = dot(N, V.data() + r * N, AV.data() + c * N);
    jacobi_syev((int)k, C.data(), (int)k, LAM.data());
    double* R = V.data() + (i + 1) * N;
#pragma omp parallel for schedule(static)
    for (int64_t j = 0; j < N; ++j) {
      double x = 0., ax = 0.;
      for (int64_t c = 0; c < k; ++c) {
        x += V[j + c * N] * C[c];
        ax += AV[j + c * N] * C[c];
      }
      X[j] = x;
      R[j] = ax - LAM[0] * x;
    }
    double res = nrm2(N, R);
    if (res < tol) {
      converged = true;
      break;
    }
    for (int64_t j = 0; j < N; ++j) {
      double denom = D[j] - LAM[0];
      if (std::abs(denom) < min_abs_denominator) denom = (denom >= 0) ? min_abs_denominator : -min_abs_denominator;
      R[j] = -R[j] / denom;
    }
    gram_schmidt(N, k, V.data(), R);
  }
  *E_out = LAM[0];
  *iters_out = iter;
  return converged ? 0 : 1;
}

// ---------------------------------------------------------------- RDMs
// Spin-resolved RDM contributions (include/macis/util/rdms.hpp:39-612), symm=true.
struct Rdms {
  int n;
  double *aa, *bb, *aaaa, *bbbb, *aabb;
  double& r4(double* t, uint32_t p, uint32_t q, uint32_t r, uint32_t s) const {
    return t[p + (size_t)n * (q + (size_t)n * (r + (size_t)n * s))];
  }
  double& r2(double* t, uint32_t p, uint32_t q) const { return t[p + (size_t)n * q]; }
};
inline void atomic_add(double& x, double v) {
#pragma omp atomic
  x += v;
}

// rdms.hpp:39-68
void rdm_4(const Rdms& R, double* trdm, uint64_t bra, uint64_t ket, uint64_t ex, double val) {
  if (!trdm) return;
  Double d = doubles_sign_indices(bra, ket, ex);
  val *= d.sign * 0.5;
  atomic_add(R.r4(trdm, d.v1, d.o1, d.v2, d.o2), val);
  atomic_add(R.r4(trdm, d.v2, d.o1, d.v1, d.o2), -val);
  atomic_add(R.r4(trdm, d.v1, d.o2, d.v2, d.o1), -val);
  atomic_add(R.r4(trdm, d.v2, d.o2, d.v1, d.o1), val);
  atomic_add(R.r4(trdm, d.o2, d.v2, d.o1, d.v1), val);
  atomic_add(R.r4(trdm, d.o2, d.v1, d.o1, d.v2), -val);
  atomic_add(R.r4(trdm, d.o1, d.v2, d.o2, d.v1), -val);
  atomic_add(R.r4(trdm, d.o1, d.v1, d.o2, d.v2), val);
}
// rdms.hpp:145-167
void rdm_22(const Rdms& R, uint64_t ba, uint64_t ka, uint64_t exa, uint64_t bb, uint64_t kb, uint64_t exb,
            double val) {
  if (!R.aabb) return;
  Single a = single_excitation_sign_indices(ba, ka, exa);  // (o2, v2)
  Single b = single_excitation_sign_indices(bb, kb, exb);  // (o1, v1)
  double sign = b.sign * a.sign;
  val *= sign * 0.5;
  atomic_add(R.r4(R.aabb, b.v, b.o, a.v, a.o), val);
  atomic_add(R.r4(R.aabb, b.o, b.v, a.o, a.v), val);
}
// rdms.hpp:282-368
void rdm_2(const Rdms& R, bool transpose, uint64_t bra, uint64_t ket, uint64_t ex, const std::vector<uint32_t>& occ_ss,
           const std::vector<uint32_t>& occ_os, double val, double* ordm_ss, double* trdm_ss, double* trdm_os) {
  Single s = single_excitation_sign_indices(bra, ket, ex);
  const uint32_t o1 = s.o, v1 = s.v;
  if (ordm_ss) {
    atomic_add(R.r2(ordm_ss, v1, o1), s.sign * val);
    atomic_add(R.r2(ordm_ss, o1, v1), s.sign * val);
  }
  val *= s.sign * 0.5;
  if (trdm_ss) {
    for (auto p : occ_ss) {
      atomic_add(R.r4(trdm_ss, v1, o1, p, p), val);
      atomic_add(R.r4(trdm_ss, p, p, v1, o1), val);
      atomic_add(R.r4(trdm_ss, v1, p, p, o1), -val);
      atomic_add(R.r4(trdm_ss, p, o1, v1, p), -val);
    }
    for (auto p : occ_ss) {
      atomic_add(R.r4(trdm_ss, p, p, o1, v1), val);
      atomic_add(R.r4(trdm_ss, o1, v1, p, p), val);
      atomic_add(R.r4(trdm_ss, o1, p, p, v1), -val);
      atomic_add(R.r4(trdm_ss, p, v1, o1, p), -val);
    }
  }
  if (trdm_os) {
    for (auto p : occ_os) {
      if (transpose)
        atomic_add(R.r4(trdm_os, v1, o1, p, p), val);
      else
        atomic_add(R.r4(trdm_os, p, p, v1, o1), val);
    }
    for (auto p : occ_os) {
      if (transpose)
        atomic_add(R.r4(trdm_os, o1, v1, p, p), val);
      else
        atomic_add(R.r4(trdm_os, p, p, o1, v1), val);
    }
  }
}
// rdms.hpp:439-516
void rdm_diag(const Rdms& R, const std::vector<uint32_t>& oa, const std::vector<uint32_t>& ob, double val) {
  if (R.aa)
    for (auto p : oa) atomic_add(R.r2(R.aa, p, p), val);
  if (R.bb)
    for (auto p : ob) atomic_add(R.r2(R.bb, p, p), val);
  val *= 0.5;
  if (R.aaaa)
    for (auto q : oa)
      for (auto p : oa) {
        atomic_add(R.r4(R.aaaa, p, p, q, q), val);
        atomic_add(R.r4(R.aaaa, p, q, q, p), -val);
      }
  if (R.bbbb)
    for (auto q : ob)
      for (auto p : ob) {
        atomic_add(R.r4(R.bbbb, p, p, q, q), val);
        atomic_add(R.r4(R.bbbb, p, q, q, p), -val);
      }
  if (R.aabb)
    for (auto q : ob)
      for (auto p : oa) atomic_add(R.r4(R.aabb, q, q, p, p), val);
}

// SortedDoubleLoopHamiltonianGenerator::form_rdms_spin_dep
// (sorted_double_loop.hpp:626-753) with rdm_contributions_spin_dep<true>
// (rdms.hpp:579-612).  Results are accumulated (+=).
void rdms_spin_dep(const uint64_t* alpha, const uint64_t* beta, int64_t nd, const double* C, const Rdms& R) {
  std::vector<uint64_t> ua;
  std::vector<int64_t> off;
  unique_alpha(alpha, nd, ua, off);
  const int64_t nu = (int64_t)ua.size();
#pragma omp parallel
  {
    std::vector<uint32_t> oa, ob;
#pragma omp for schedule(dynamic)
    for (int64_t ib = 0; ib < nu; ++ib) {
      if (!ua[ib]) continue;
      const uint64_t ba = ua[ib];
      for (int64_t ik = ib; ik < nu; ++ik) {
        if (!ua[ik]) continue;
        const uint64_t ka = ua[ik];
        const uint64_t exa = ba ^ ka;
        const int ca = popc(exa);
        if (ca > 4) continue;
        bits_to_indices(ba, oa);
        for (int64_t i = off[ib]; i < off[ib + 1]; ++i) {
          const uint64_t bb = beta[i];
          bits_to_indices(bb, ob);
          for (int64_t j = off[ik]; j < off[ik + 1]; ++j) {
            if (j < i) continue;
            const uint64_t kb = beta[j];
            const uint64_t exb = bb ^ kb;
            const int cb = popc(exb);
            if (ca + cb > 4) continue;
            const double val = C[i] * C[j];
            if (!(std::abs(val) > 1e-16)) continue;
            if (ca == 4)
              rdm_4(R, R.aaaa, ba, ka, exa, val);
            else if (cb == 4)
              rdm_4(R, R.bbbb, bb, kb, exb, val);
            else if (ca == 2 && cb == 2)
              rdm_22(R, ba, ka, exa, bb, kb, exb, val);
            else if (ca == 2)
              rdm_2(R, false, ba, ka, exa, oa, ob, val, R.aa, R.aaaa, R.aabb);
            else if (cb == 2)
              rdm_2(R, true, bb, kb, exb, ob, oa, val, R.bb, R.bbbb, R.aabb);
            else
              rdm_diag(R, oa, ob, val);
          }
        }
      }
    }
  }
}

// A bounded sample of the reference's symmetric SDL H build for timing on the
// host: the count and fill passes of build_csr_sdl (sorted_double_loop.hpp:
// 137-360) for the bra alpha groups ib = offset, offset + stride, ...
// (each against all ket groups >= ib, as the reference loops them).  The
// element values go to thread-local buffers (the per-row sort and the
// threshold compaction are not part of the sample).  Returns the number of
// elements the sampled groups produce (each upper-triangle pair counted for
// both (i,j) and (j,i), as the reference stores them).
int64_t sdl_sample(const Ham& H, const uint64_t* alpha, const uint64_t* beta, int64_t nd, double thresh,
                   int64_t stride, int64_t offset) {
  std::vector<uint64_t> ua;
  std::vector<int64_t> off;
  unique_alpha(alpha, nd, ua, off);
  const int64_t nu = (int64_t)ua.size();
  int64_t total = 0;
#pragma omp parallel reduction(+ : total)
  {
    std::vector<uint32_t> oa, ob;
    std::vector<double> vals;
    std::vector<int64_t> cols;
    int64_t counted = 0;
#pragma omp for schedule(dynamic)
    for (int64_t ib = offset; ib < nu; ib += stride) {
      if (!ua[ib]) continue;
      const uint64_t ba = ua[ib];
      bits_to_indices(ba, oa);
      // count pass
      for (int64_t ik = ib; ik < nu; ++ik) {
        const uint64_t ka = ua[ik];
        if (!ka) continue;
        const uint64_t exa = ba ^ ka;
        const int ca = popc(exa);
        if (ca > 4) continue;
        if (ca == 4 && std::abs(H.me_4(ba, ka, exa)) < thresh) continue;
        for (int64_t i = off[ib]; i < off[ib + 1]; ++i)
          for (int64_t j = off[ik]; j < off[ik + 1]; ++j) {
            if (j < i) continue;
            const uint64_t exb = beta[i] ^ beta[j];
            const int cb = popc(exb);
            if (ca + cb > 4) continue;
            if (cb == 4 && std::abs(H.me_4(beta[i], beta[j], exb)) < thresh) continue;
            counted += (i != j) ? 2 : 1;
          }
      }
      // fill pass
      for (int64_t ik = ib; ik < nu; ++ik) {
        const uint64_t ka = ua[ik];
        if (!ka) continue;
        const uint64_t exa = ba ^ ka;
        const int ca = popc(exa);
        if (ca > 4) continue;
        for (int64_t i = off[ib]; i < off[ib + 1]; ++i) {
          const uint64_t bb = beta[i];
          bits_to_indices(bb, ob);
          for (int64_t j = off[ik]; j < off[ik + 1]; ++j) {
            if (j < i) continue;
            const uint64_t kb = beta[j];
            const uint64_t exb = bb ^ kb;
            const int cb = popc(exb);
            if (ca + cb > 4) continue;
            double h;
            if (ca == 4) {
              h = H.me_4(ba, ka, exa);
              if (std::abs(h) < thresh) continue;
            } else if (cb == 4) {
              h = H.me_4(bb, kb, exb);
              if (std::abs(h) < thresh) continue;
            } else if (ca == 2) {
              h = (cb == 2) ? H.me_22(ba, ka, exa, bb, kb, exb) : H.me_2(ba, ka, exa, oa, ob);
            } else if (cb == 2) {
              h = H.me_2(bb, kb, exb, ob, oa);
            } else {
              h = H.me_diag(oa, ob);
            }
            vals.push_back(h);
            cols.push_back(j);
          }
        }
      }
      vals.clear();
      cols.clear();
    }
    total += counted;
  }
  return total;
}

// The rows [r0, r1) of the CSR (a whole number of alpha groups) against all
// kets, with the reference's non-symmetric SDL loop (is_symm == false):
// every ket group, every beta pair, values with the row determinant as bra,
// per-row sort, |h| > thresh.  Used to time a sample of the CPU sigma.
Csr* build_rows(const Ham& H, const uint64_t* alpha, const uint64_t* beta, int64_t nd, double thresh, int64_t r0,
                int64_t r1) {
  std::vector<uint64_t> ua;
  std::vector<int64_t> off;
  unique_alpha(alpha, nd, ua, off);
  const int64_t nu = (int64_t)ua.size();
  const int64_t nr = r1 - r0;
  std::vector<std::vector<std::pair<int64_t, double>>> rows(nr);
#pragma omp parallel
  {
    std::vector<uint32_t> oa, ob;
#pragma omp for schedule(dynamic)
    for (int64_t i = r0; i < r1; ++i) {
      const uint64_t ba = alpha[i], bb = beta[i];
      if (!ba) continue;
      bits_to_indices(ba, oa);
      bits_to_indices(bb, ob);
      auto& row = rows[i - r0];
      for (int64_t ik = 0; ik < nu; ++ik) {
        const uint64_t ka = ua[ik];
        if (!ka) continue;
        const uint64_t exa = ba ^ ka;
        const int ca = popc(exa);
        if (ca > 4) continue;
        for (int64_t j = off[ik]; j < off[ik + 1]; ++j) {
          const uint64_t kb = beta[j];
          const uint64_t exb = bb ^ kb;
          const int cb = popc(exb);
          if (ca + cb > 4) continue;
          double h;
          if (ca == 4)
            h = H.me_4(ba, ka, exa);
          else if (cb == 4)
            h = H.me_4(bb, kb, exb);
          else if (ca == 2)
            h = (cb == 2) ? H.me_22(ba, ka, exa, bb, kb, exb) : H.me_2(ba, ka, exa, oa, ob);
          else if (cb == 2)
            h = H.me_2(bb, kb, exb, ob, oa);
          else
            h = H.me_diag(oa, ob);
          if (thresh > 0 && !(std::abs(h) > thresh)) continue;
          row.push_back({j, h});
        }
      }
      std::sort(row.begin(), row.end());
    }
  }
  Csr* M = new Csr;
  M->n = nr;
  M->rowptr.assign(nr + 1, 0);
  for (int64_t i = 0; i < nr; ++i) M->rowptr[i + 1] = M->rowptr[i] + (int64_t)rows[i].size();
  M->colind.resize(M->rowptr[nr]);
  M->nzval.resize(M->rowptr[nr]);
  for (int64_t i = 0; i < nr; ++i)
    for (size_t k = 0; k < rows[i].size(); ++k) {
      M->colind[M->rowptr[i] + k] = rows[i][k].first;
      M->nzval[M->rowptr[i] + k] = rows[i][k].second;
    }
  return M;
}

thread_local char g_err[512];
template <class F>
int guard(F&& f) {
  try {
    f();
    return 0;
  } catch (const std::exception& e) {
    std::snprintf(g_err, sizeof(g_err), "%s", e.what());
    return -1;
  }
}

}  // namespace

extern "C" {

const char* orc_last_error() { return g_err; }

int orc_num_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

// generate_combs (include/macis/sd_operations.hpp:305-323): all nset-of-nbits
// strings in std::prev_permutation order starting from the lowest orbitals.
int64_t orc_combs(int nbits, int nset, uint64_t* out) {
  std::vector<char> v(nbits, 0);
  std::fill_n(v.begin(), nset, 1);
  int64_t cnt = 0;
  do {
    uint64_t s = 0;
    for (int i = 0; i < nbits; ++i)
      if (v[i]) s |= 1ull << i;
    if (out) out[cnt] = s;
    ++cnt;
  } while (std::prev_permutation(v.begin(), v.end()));
  return cnt;
}

void* orc_ham_create(int n, const double* T, const double* V) {
  Ham* h = new Ham;
  h->init(n, T, V);
  return h;
}
void orc_ham_destroy(void* h) { delete (Ham*)h; }
void orc_ham_intermediates(void* h, double* G_red, double* V_red, double* G2_red, double* V2_red) {
  Ham* H = (Ham*)h;
  std::copy(H->G_red.begin(), H->G_red.end(), G_red);
  std::copy(H->V_red.begin(), H->V_red.end(), V_red);
  std::copy(H->G2_red.begin(), H->G2_red.end(), G2_red);
  std::copy(H->V2_red.begin(), H->V2_red.end(), V2_red);
}
double orc_matrix_element(void* h, uint64_t ba, uint64_t bb, uint64_t ka, uint64_t kb) {
  return ((Ham*)h)->me(ba, bb, ka, kb);
}

void* orc_csr_build(void* h, const uint64_t* alpha, const uint64_t* beta, int64_t nd, double thresh) {
  Csr* M = nullptr;
  if (guard([&] { M = build_csr_sdl(*(Ham*)h, alpha, beta, nd, thresh); })) return nullptr;
  return M;
}
int64_t orc_csr_nnz(void* m) { return (int64_t)((Csr*)m)->colind.size(); }
void orc_csr_copy(void* m, int64_t* rowptr, int64_t* colind, double* nzval) {
  Csr* M = (Csr*)m;
  std::copy(M->rowptr.begin(), M->rowptr.end(), rowptr);
  std::copy(M->colind.begin(), M->colind.end(), colind);
  std::copy(M->nzval.begin(), M->nzval.end(), nzval);
}
void orc_csr_destroy(void* m) { delete (Csr*)m; }
void orc_csr_spmv(void* m, const double* x, double* y) { spmv(*(Csr*)m, x, y); }
// extract_diagonal_elements (sparsexx/util/submatrix.hpp:354-384)
void orc_csr_diag(void* m, double* D) {
  Csr* M = (Csr*)m;
  for (int64_t i = 0; i < M->n; ++i) {
    D[i] = 0.;
    for (int64_t k = M->rowptr[i]; k < M->rowptr[i + 1]; ++k)
      if (M->colind[k] == i) {
        D[i] = M->nzval[k];
        break;
      }
  }
}

// serial_selected_ci_diag (include/macis/solvers/selected_ci_diag.hpp:111-158):
// diagonal, guess (keep X when max|X| > 1/N, else one-hot at the first
// minimum of D, davidson.hpp:106-113), then davidson.  Returns 0 on
// convergence, 1 on "Davidson Did Not Converge!", -1 on other errors.
int orc_selected_ci_diag(void* m, int64_t max_m, double tol, double* X, double* E, int64_t* iters) {
  Csr* M = (Csr*)m;
  int rc = 0;
  int g = guard([&] {
    std::vector<double> D(M->n);
    orc_csr_diag(m, D.data());
    double maxc = 0.;
    for (int64_t i = 0; i < M->n; ++i) maxc = std::max(maxc, std::abs(X[i]));
    if (!(maxc > 1. / (double)M->n)) {
      int64_t imin = std::min_element(D.begin(), D.end()) - D.begin();
      X[imin] = 1.;
    }
    rc = davidson(*M, max_m, D.data(), tol, X, E, iters);
  });
  return g ? -1 : rc;
}

void orc_syev(int k, double* A, double* w) { jacobi_syev(k, A, k, w); }

int64_t orc_sdl_sample(void* h, const uint64_t* alpha, const uint64_t* beta, int64_t nd, double thresh, int64_t stride,
                       int64_t offset) {
  return sdl_sample(*(Ham*)h, alpha, beta, nd, thresh, stride, offset);
}
void* orc_csr_build_rows(void* h, const uint64_t* alpha, const uint64_t* beta, int64_t nd, double thresh, int64_t r0,
                         int64_t r1) {
  Csr* M = nullptr;
  if (guard([&] { M = build_rows(*(Ham*)h, alpha, beta, nd, thresh, r0, r1); })) return nullptr;
  return M;
}
// y[0:rows) = block * x (x over all columns)
void orc_csr_spmv_block(void* m, const double* x, double* y) { spmv(*(Csr*)m, x, y); }

void orc_rdms_spin_dep(int n, const uint64_t* alpha, const uint64_t* beta, int64_t nd, const double* C, double* aa,
                       double* bb, double* aaaa, double* bbbb, double* aabb) {
  Rdms R{n, aa, bb, aaaa, bbbb, aabb};
  rdms_spin_dep(alpha, beta, nd, C, R);
}

}  // extern "C"
