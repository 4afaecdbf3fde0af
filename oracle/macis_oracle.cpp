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
#include <limits>
#include <memory>
#include <numeric>
#include <stdexcept>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#include <parallel/algorithm>
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

// Summed over fixed blocks of 4096 elements, each in index order, and the
// block sums in block order: the result does not depend on the thread count
// or on the order in which threads finish (an OpenMP reduction combines its
// partial sums in no fixed order), so the Davidson steps repeat bit for bit.
double dot(int64_t n, const double* a, const double* b) {
  constexpr int64_t kBlk = 4096;
  const int64_t nb = (n + kBlk - 1) / kBlk;
  std::vector<double> part(nb);
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < nb; ++k) {
    double s = 0.;
    for (int64_t i = k * kBlk; i < std::min(n, (k + 1) * kBlk); ++i) s += a[i] * b[i];
    part[k] = s;
  }
  double s = 0.;
  for (int64_t k = 0; k < nb; ++k) s += part[k];
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
  std::stable_sort(ord.begin(), ord.end(),
                   [&](int x, int y) { return a[x + (size_t)k * x] < a[y + (size_t)k * y]; });
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
  // the 1-RDMs' fixed-point accumulators (see fx_add), when given
  unsigned long long *aa_fx = nullptr, *bb_fx = nullptr;
  double fx_inv = 1.;  // 1 / s
  double& r4(double* t, uint32_t p, uint32_t q, uint32_t r, uint32_t s) const {
    return t[p + (size_t)n * (q + (size_t)n * (r + (size_t)n * s))];
  }
  double& r2(double* t, uint32_t p, uint32_t q) const { return t[p + (size_t)n * q]; }
};
inline void atomic_add(double& x, double v) {
#pragma omp atomic
  x += v;
}
// The 1-RDM is summed in fixed point, two 64-bit words per element, in
// units of s = the power of two at or above max_I C_I^2: x / s = hi 2^-32 +
// lo 2^-76, hi = rint(x / s 2^32), lo the rest in units of 2^-76 (scaling and
// split are exact).  Integer sums do not depend on the
// order in which the threads' atomics land, so the 1-RDM - and the natural
// orbitals of the ASCI grow's rotation - repeat bit for bit, and equal the
// GPU's, which sums the same contributions the same way.
constexpr double kFxHi = 4294967296.0;               // 2^32
constexpr double kFxLo = 75557863725914323419136.0;  // 2^76
inline void fx_add(unsigned long long* t, size_t i, double v) {
  // v already divided by s
  const double hi = std::rint(v * kFxHi);
  const double lo = std::rint((v - hi * (1.0 / kFxHi)) * kFxLo);
  const unsigned long long uh = (unsigned long long)(long long)hi, ul = (unsigned long long)(long long)lo;
#pragma omp atomic
  t[2 * i] += uh;
#pragma omp atomic
  t[2 * i + 1] += ul;
}
inline void add_ordm(const Rdms& R, double* t, uint32_t p, uint32_t q, double v) {
  unsigned long long* fx = (t == R.aa) ? R.aa_fx : (t == R.bb) ? R.bb_fx : nullptr;
  if (fx)
    fx_add(fx, p + (size_t)R.n * q, v * R.fx_inv);
  else
    atomic_add(R.r2(t, p, q), v);
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
    add_ordm(R, ordm_ss, v1, o1, s.sign * val);
    add_ordm(R, ordm_ss, o1, v1, s.sign * val);
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
    for (auto p : oa) add_ordm(R, R.aa, p, p, val);
  if (R.bb)
    for (auto p : ob) add_ordm(R, R.bb, p, p, val);
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
void rdms_spin_dep(const uint64_t* alpha, const uint64_t* beta, int64_t nd, const double* C, const Rdms& R0) {
  std::vector<uint64_t> ua;
  std::vector<int64_t> off;
  unique_alpha(alpha, nd, ua, off);
  const int64_t nu = (int64_t)ua.size();
  const size_t n2 = (size_t)R0.n * R0.n;
  std::vector<unsigned long long> fa(R0.aa ? 2 * n2 : 0, 0ull), fb(R0.bb ? 2 * n2 : 0, 0ull);
  Rdms R = R0;
  R.aa_fx = R0.aa ? fa.data() : nullptr;
  R.bb_fx = R0.bb ? fb.data() : nullptr;
  double cmax = 0.;
  for (int64_t i = 0; i < nd; ++i) cmax = std::max(cmax, std::abs(C[i]));
  int e2 = 0;
  if (cmax > 0.) std::frexp(cmax * cmax, &e2);
  const double fx_s = std::ldexp(1.0, e2);
  R.fx_inv = std::ldexp(1.0, -e2);
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
  for (size_t i = 0; i < n2; ++i) {
    if (R0.aa)
      R0.aa[i] += ((double)(long long)fa[2 * i] * (1.0 / kFxHi) + (double)(long long)fa[2 * i + 1] * (1.0 / kFxLo)) * fx_s;
    if (R0.bb)
      R0.bb[i] += ((double)(long long)fb[2 * i] * (1.0 / kFxHi) + (double)(long long)fb[2 * i + 1] * (1.0 / kFxLo)) * fx_s;
  }
}

// ---------------------------------------------------------------- orbital entropies
// OrbitalRDMIntermediates and its contribution and assembly functions
// (include/macis/util/entropies.hpp) driven by the determinant-pair loop of
// SortedDoubleLoopHamiltonianGenerator::form_entropies
// (include/macis/hamiltonian_generator/sorted_double_loop.hpp:755-903).  The
// n x n intermediates are indexed M(i, j) = m[i * n + j]; names follow the
// reference's (a/b: alpha/beta; ii, ij, iijj ...: orbital pattern).
struct OrbInter {
  int n = 0;
  bool s2 = false;
  std::vector<double> a_ii, b_ii, ab_iiii;
  enum {
    A_IJ, B_IJ, AA_IIJJ, BB_IIJJ, AB_IIJJ, AB_IJJJ, AB_JIJJ, AB_JJIJ, AB_JJJI, AB_IJIJ, AB_IJJI, AAB_IIJJJJ,
    ABB_JJIIJJ, AAB_IIJJII, ABB_IIIIJJ, ABB_IJIIJJ, AAB_IIJJIJ, AABB_IIJJIIJJ, NMAT
  };
  std::vector<double> m[NMAT];
  void init(int norb, bool need_s2) {
    n = norb;
    s2 = need_s2;
    a_ii.assign(n, 0.);
    b_ii.assign(n, 0.);
    ab_iiii.assign(n, 0.);
    for (auto& x : m) x.assign(need_s2 ? (size_t)n * n : 0, 0.);
  }
  double& M(int k, uint32_t i, uint32_t j) { return m[k][(size_t)i * n + j]; }
  double M(int k, uint32_t i, uint32_t j) const { return m[k][(size_t)i * n + j]; }
  void add(const OrbInter& o) {
    for (int i = 0; i < n; ++i) {
      a_ii[i] += o.a_ii[i];
      b_ii[i] += o.b_ii[i];
      ab_iiii[i] += o.ab_iiii[i];
    }
    for (int k = 0; k < NMAT; ++k)
      for (size_t i = 0; i < m[k].size(); ++i) m[k][i] += o.m[k][i];
  }
};

// orbital_rdm_contrib_diag_s1 / orbital_rdm_contrib_diag (entropies.hpp:155-253)
void orb_diag(OrbInter& X, const std::vector<uint32_t>& oa, const std::vector<uint32_t>& ob, double val) {
  for (auto p : oa) X.a_ii[p] += val;
  for (auto p : ob) X.b_ii[p] += val;
  if (!X.s2) {
    for (auto q : ob)
      for (auto p : oa)
        if (p == q) X.ab_iiii[q] += val;
    return;
  }
  std::vector<char> isa(X.n, 0), isb(X.n, 0);
  for (auto p : oa) isa[p] = 1;
  for (auto p : ob) isb[p] = 1;
  for (auto q : oa)
    for (auto p : oa) {
      if (p == q) continue;
      X.M(OrbInter::AA_IIJJ, p, q) += val;
      if (isb[p]) {
        X.M(OrbInter::AAB_IIJJII, p, q) += val;
        if (isb[q]) X.M(OrbInter::AABB_IIJJIIJJ, p, q) += val;
      }
      if (isb[q]) X.M(OrbInter::AAB_IIJJJJ, p, q) += val;
    }
  for (auto q : ob)
    for (auto p : ob) {
      if (p == q) continue;
      X.M(OrbInter::BB_IIJJ, p, q) += val;
      if (isa[p]) X.M(OrbInter::ABB_JJIIJJ, q, p) += val;
      if (isa[q]) X.M(OrbInter::ABB_IIIIJJ, q, p) += val;
    }
  for (auto q : ob)
    for (auto p : oa) {
      if (p == q) X.ab_iiii[q] += val;
      X.M(OrbInter::AB_IIJJ, p, q) += val;
    }
}

// orbital_rdm_contrib_2<transpose> (entropies.hpp:255-313): a single
// excitation of one spin (beta when transposed); occ_os = the other spin's
// occupied orbitals of the bra
void orb_single(OrbInter& X, bool transpose, uint64_t bra, uint64_t ket, uint64_t ex,
                const std::vector<uint32_t>& occ_os, double val) {
  const Single s = single_excitation_sign_indices(bra, ket, ex);
  const uint32_t o1 = s.o, v1 = s.v;
  const double sv = s.sign * val;
  const int xij = transpose ? OrbInter::B_IJ : OrbInter::A_IJ;
  X.M(xij, v1, o1) += sv;
  X.M(xij, o1, v1) += sv;
  const int k1 = transpose ? OrbInter::AB_JJIJ : OrbInter::AB_IJJJ;
  const int k2 = transpose ? OrbInter::AB_JJJI : OrbInter::AB_JIJJ;
  bool o_in = false, v_in = false;
  for (auto p : occ_os) {
    if (o1 == p) {
      o_in = true;
      X.M(k1, v1, o1) += sv;
      X.M(k2, v1, o1) += sv;
    } else if (v1 == p) {
      v_in = true;
      X.M(k1, o1, v1) += sv;
      X.M(k2, o1, v1) += sv;
    }
  }
  if (o_in && v_in) {
    const int k3 = transpose ? OrbInter::AAB_IIJJIJ : OrbInter::ABB_IJIIJJ;
    X.M(k3, o1, v1) += sv;
    X.M(k3, v1, o1) += sv;
  }
}

// orbital_rdm_contrib_22 (entropies.hpp:315-340): one single per spin
void orb_double_os(OrbInter& X, uint64_t ba, uint64_t ka, uint64_t exa, uint64_t bb, uint64_t kb, uint64_t exb,
                   double val) {
  const Single sa = single_excitation_sign_indices(ba, ka, exa);  // (o2, v2)
  const Single sb = single_excitation_sign_indices(bb, kb, exb);  // (o1, v1)
  const double sv = sa.sign * sb.sign * val;
  const uint32_t o1 = sb.o, v1 = sb.v, o2 = sa.o, v2 = sa.v;
  if (o1 == o2 && v1 == v2) {
    X.M(OrbInter::AB_IJIJ, v1, o1) += sv;
    X.M(OrbInter::AB_IJIJ, o1, v1) += sv;
  } else if (o1 == v2 && v1 == o2) {
    X.M(OrbInter::AB_IJJI, v1, o1) += sv;
    X.M(OrbInter::AB_IJJI, o1, v1) += sv;
  }
}

void orb_entropy_pairs(OrbInter& X, const uint64_t* alpha, const uint64_t* beta, int64_t nd, const double* C) {
  std::vector<uint64_t> ua;
  std::vector<int64_t> off;
  unique_alpha(alpha, nd, ua, off);
  const int64_t nu = (int64_t)ua.size();
  const int lim = X.s2 ? 2 : 0;
  int nth = 1;
#ifdef _OPENMP
  nth = omp_get_max_threads();
#endif
  std::vector<OrbInter> part(nth);
  for (auto& p : part) p.init(X.n, X.s2);
#pragma omp parallel
  {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    OrbInter& Y = part[tid];
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
        if (ca > lim) continue;
        bits_to_indices(ba, oa);
        for (int64_t i = off[ib]; i < off[ib + 1]; ++i) {
          const uint64_t bb = beta[i];
          bits_to_indices(bb, ob);
          for (int64_t j = off[ik]; j < off[ik + 1]; ++j) {
            if (j < i) continue;
            const uint64_t kb = beta[j];
            const uint64_t exb = bb ^ kb;
            const int cb = popc(exb);
            if (cb > lim) continue;
            const double val = C[i] * C[j];
            if (!(std::abs(val) > 1e-16)) continue;
            // eval_ordm_intermediates (entropies.hpp:662-719)
            if (ca == 0 && cb == 0)
              orb_diag(Y, oa, ob, val);
            else if (!X.s2)
              continue;
            else if (ca == 2 && cb == 0)
              orb_single(Y, false, ba, ka, exa, ob, val);
            else if (ca == 0 && cb == 2)
              orb_single(Y, true, bb, kb, exb, oa, val);
            else
              orb_double_os(Y, ba, ka, exa, bb, kb, exb, val);
          }
        }
      }
    }
  }
  for (auto& p : part) X.add(p);
}

inline void add_ent(double& s, double v) {
  if (v > std::numeric_limits<double>::epsilon()) s -= v * std::log(v);
}

// build_s1_entropy (entropies.hpp:342-370)
void build_s1(const OrbInter& X, double* s1) {
  for (int i = 0; i < X.n; ++i) {
    double s = 0.;
    add_ent(s, 1 - X.a_ii[i] - X.b_ii[i] + X.ab_iiii[i]);
    add_ent(s, X.a_ii[i] - X.ab_iiii[i]);
    add_ent(s, X.b_ii[i] - X.ab_iiii[i]);
    add_ent(s, X.ab_iiii[i]);
    s1[i] = s;
  }
}

// build_s2_entropy (entropies.hpp:397-528): the two-orbital RDM of (i, j) in
// its symmetry blocks (1 + 2x2 + 2x2 + 1 + 1 + 4x4 + 2x2 + 2x2 + 1), the
// entropy of their eigenvalues
void build_s2(const OrbInter& X, double* s2) {
  using O = OrbInter;
  const int n = X.n;
  auto eig2 = [](double a, double b, double d, double& s) {
    const double hs = 0.5 * (a + d), hd = 0.5 * (a - d);
    const double w = std::sqrt(hd * hd + b * b);
    add_ent(s, hs - w);
    add_ent(s, hs + w);
  };
  for (int i = 0; i < n; ++i) {
    s2[(size_t)i * n + i] = 0.;
    for (int j = i + 1; j < n; ++j) {
      auto M = [&](int k, int p, int q) { return X.M(k, p, q); };
      const double aabb = M(O::AABB_IIJJIIJJ, i, j);
      double s = 0.;
      add_ent(s, 1 - X.a_ii[i] - X.b_ii[i] - X.a_ii[j] - X.b_ii[j] + X.ab_iiii[i] + X.ab_iiii[j] +
                     M(O::AA_IIJJ, i, j) + M(O::AB_IIJJ, i, j) + M(O::AB_IIJJ, j, i) + M(O::BB_IIJJ, i, j) -
                     M(O::AAB_IIJJJJ, i, j) - M(O::ABB_JJIIJJ, i, j) - M(O::AAB_IIJJII, i, j) -
                     M(O::ABB_IIIIJJ, i, j) + aabb);
      eig2(X.a_ii[j] - M(O::AB_IIJJ, j, i) - M(O::AA_IIJJ, i, j) - M(O::AB_IIJJ, j, j) + M(O::AAB_IIJJJJ, i, j) +
               M(O::AAB_IIJJII, i, j) + M(O::ABB_JJIIJJ, i, j) - aabb,
           M(O::A_IJ, i, j) - M(O::AB_JIJJ, j, i) - M(O::AB_IJJJ, i, j) + M(O::ABB_IJIIJJ, i, j),
           X.a_ii[i] - M(O::AB_IIJJ, i, j) - M(O::AA_IIJJ, i, j) - M(O::AB_IIJJ, i, i) + M(O::AAB_IIJJJJ, i, j) +
               M(O::AAB_IIJJII, i, j) + M(O::ABB_IIIIJJ, i, j) - aabb,
           s);
      eig2(X.b_ii[j] - M(O::AB_IIJJ, i, j) - M(O::BB_IIJJ, i, j) - M(O::AB_IIJJ, j, j) + M(O::ABB_IIIIJJ, i, j) +
               M(O::AAB_IIJJJJ, i, j) + M(O::ABB_JJIIJJ, i, j) - aabb,
           M(O::B_IJ, i, j) - M(O::AB_JJIJ, j, i) - M(O::AB_JJJI, i, j) + M(O::AAB_IIJJIJ, i, j),
           X.b_ii[i] - M(O::AB_IIJJ, j, i) - M(O::BB_IIJJ, i, j) - M(O::AB_IIJJ, i, i) + M(O::ABB_JJIIJJ, i, j) +
               M(O::AAB_IIJJII, i, j) + M(O::ABB_IIIIJJ, i, j) - aabb,
           s);
      add_ent(s, M(O::AA_IIJJ, i, j) - M(O::AAB_IIJJII, i, j) - M(O::AAB_IIJJJJ, i, j) + aabb);
      add_ent(s, M(O::BB_IIJJ, i, j) - M(O::ABB_IIIIJJ, i, j) - M(O::ABB_JJIIJJ, i, j) + aabb);
      double B[16];
      B[0] = M(O::AB_IIJJ, j, j) - M(O::AAB_IIJJJJ, i, j) - M(O::ABB_JJIIJJ, i, j) + aabb;
      B[1] = B[4] = M(O::AB_IJJJ, i, j) - M(O::ABB_IJIIJJ, i, j);
      B[2] = B[8] = -M(O::AB_JJIJ, i, j) + M(O::AAB_IIJJIJ, i, j);
      B[3] = B[12] = M(O::AB_IJIJ, i, j);
      B[5] = M(O::AB_IIJJ, i, j) - M(O::ABB_IIIIJJ, i, j) - M(O::AAB_IIJJJJ, i, j) + aabb;
      B[6] = B[9] = -M(O::AB_IJJI, j, i);
      B[7] = B[13] = M(O::AB_JJJI, j, i) - M(O::AAB_IIJJIJ, i, j);
      B[10] = M(O::AB_IIJJ, j, i) - M(O::AAB_IIJJII, i, j) - M(O::ABB_JJIIJJ, i, j) + aabb;
      B[11] = B[14] = -M(O::AB_JIJJ, j, i) + M(O::ABB_IJIIJJ, i, j);
      B[15] = X.ab_iiii[i] - M(O::AAB_IIJJII, i, j) - M(O::ABB_IIIIJJ, i, j) + aabb;
      double w4[4];
      jacobi_syev(4, B, 4, w4);
      for (double v : w4) add_ent(s, v);
      eig2(M(O::AAB_IIJJJJ, i, j) - aabb, -M(O::AAB_IIJJIJ, i, j), M(O::AAB_IIJJII, i, j) - aabb, s);
      eig2(M(O::ABB_JJIIJJ, i, j) - aabb, -M(O::ABB_IJIIJJ, i, j), M(O::ABB_IIIIJJ, i, j) - aabb, s);
      add_ent(s, aabb);
      s2[(size_t)i * n + j] = s2[(size_t)j * n + i] = s;
    }
  }
}

// form_entropies on a determinant list: s1 (n), s2 and mi (n x n, either may
// be null); mutual information I_ij = s1_i + s1_j - s2_ij (entropies.hpp:
// 638-651)
void form_entropies(int n, const uint64_t* alpha, const uint64_t* beta, int64_t nd, const double* C, double* s1,
                    double* s2, double* mi) {
  OrbInter X;
  X.init(n, s2 || mi);
  orb_entropy_pairs(X, alpha, beta, nd, C);
  build_s1(X, s1);
  if (!X.s2) return;
  std::vector<double> loc;
  double* t = s2;
  if (!t) {
    loc.assign((size_t)n * n, 0.);
    t = loc.data();
  }
  build_s2(X, t);
  if (mi)
    for (int i = 0; i < n; ++i) {
      mi[(size_t)i * n + i] = 0.;
      for (int j = i + 1; j < n; ++j) mi[(size_t)i * n + j] = mi[(size_t)j * n + i] = s1[i] + s1[j] - t[(size_t)i * n + j];
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

// ---------------------------------------------------------------- ASCI
// ASCISettings (include/macis/asci/determinant_search.hpp:95-199) subset
struct AsciSettings {
  int64_t ntdets_max = 100000, ntdets_min = 100, ncdets_max = 100;
  int core_fixed = 0;  // 0: Percentage, 1: Fixed
  double core_threshold = 0.95, h_el_tol = 1e-8, rv_prune_tol = 1e-8;
  double grow_factor = 8.0, min_grow_factor = 1.01, backoff = 0.5, recovery = 1.1;
  double taper_grow_factor = 0.;  // off
  int just_singles = 0;            // search: single excitations only
  int64_t max_refine_iter = 6;
  double refine_energy_tol = 1e-6;
  int warm_start = 1;
  double min_warm_start_overlap = 0.5;
  // MCSCFSettings (include/macis/mcscf/mcscf.hpp:22-52)
  double ci_res_tol = 1e-8;
  int64_t ci_max_subspace = 200;
  double ci_matel_tol = 2.220446049250313e-16;
  // natural-orbital rotation during the grow (determinant_search.hpp:179-181)
  int grow_with_rot = 0;
  int64_t rot_size_start = 1000;
};

struct Det {
  uint64_t a, b;
  bool operator==(const Det& o) const { return a == o.a && b == o.b; }
};
// spin_comparator (include/macis/wfn/raw_bitset.hpp:119-141)
inline bool spin_less(const Det& x, const Det& y) { return x.a != y.a ? x.a < y.a : x.b < y.b; }

struct Contrib {
  Det q;
  double c_h, h_diag;  // c * <Q|H|P>, E0 - H_QQ
  double rv() const { return c_h / h_diag; }
};

// single_orbital_ens (src/macis/hamiltonian_generator/fast_diagonals.ipp:30-50)
std::vector<double> orbital_ens(const Ham& H, const std::vector<uint32_t>& ss, const std::vector<uint32_t>& os) {
  const int n = H.n;
  std::vector<double> e(n);
  for (int i = 0; i < n; ++i) {
    double x = H.t(i, i);
    for (auto q : ss) x += H.G2_red[i + (size_t)n * q] + H.G2_red[q + (size_t)n * i];
    x -= H.G2_red[i + (size_t)n * i];
    for (auto q : os) x += H.V2_red[i + (size_t)n * q];
    e[i] = x;
  }
  return e;
}
inline double g2(const Ham& H, uint32_t p, uint32_t q) { return H.G2_red[p + (size_t)H.n * q]; }
inline double v2(const Ham& H, uint32_t p, uint32_t q) { return H.V2_red[p + (size_t)H.n * q]; }

// append_singles / append_ss_doubles / append_os_doubles_asci_contributions
// (include/macis/asci/determinant_contributions.hpp:93-297) with the fast
// diagonals (fast_diagonals.ipp:52-127), for one spin convention: `same` is
// the excited spin, `other` the spectator.
void singles_contribs(const Ham& H, double coeff, uint64_t same, uint64_t other, bool alpha,
                      const std::vector<uint32_t>& occ_s, const std::vector<uint32_t>& vir_s,
                      const std::vector<uint32_t>& occ_o, const std::vector<double>& eps, double hdiag, double E0,
                      double tol, std::vector<Contrib>& out) {
  const int n = H.n;
  for (auto i : occ_s)
    for (auto a : vir_s) {
      double h = H.t(a, i);
      const double* G = &H.G_red[(size_t)n * (a + (size_t)n * i)];
      const double* Vr = &H.V_red[(size_t)n * (a + (size_t)n * i)];
      for (auto p : occ_s) h += G[p];
      for (auto p : occ_o) h += Vr[p];
      if (std::abs(coeff * h) < tol) continue;
      const uint64_t ex = (same ^ (1ull << i)) | (1ull << a);
      h *= single_excitation_sign(same, a, i);
      const double hd = hdiag + eps[a] - eps[i] - g2(H, a, i) - g2(H, i, a);
      Det q = alpha ? Det{ex, other} : Det{other, ex};
      out.push_back({q, coeff * h, E0 - hd});
    }
}
void ss_doubles_contribs(const Ham& H, double coeff, uint64_t same, uint64_t other, bool alpha,
                         const std::vector<uint32_t>& occ, const std::vector<uint32_t>& vir,
                         const std::vector<double>& eps, double hdiag, double E0, double tol,
                         std::vector<Contrib>& out) {
  for (size_t ii = 0; ii < occ.size(); ++ii)
    for (size_t aa = 0; aa < vir.size(); ++aa) {
      const uint32_t i = occ[ii], a = vir[aa];
      for (size_t jj = ii + 1; jj < occ.size(); ++jj)
        for (size_t bb = aa + 1; bb < vir.size(); ++bb) {
          const uint32_t j = occ[jj], b = vir[bb];
          const double G = H.v(b, j, a, i) - H.v(b, i, a, j);
          if (std::abs(coeff * G) < tol) continue;
          const uint64_t full = (1ull << i) | (1ull << j) | (1ull << a) | (1ull << b);
          const uint64_t ex = same ^ full;
          const double sign = doubles_sign_indices(same, ex, full).sign;
          const double h = sign * G;
          const double hd = hdiag + eps[a] + eps[b] - eps[i] - eps[j] + g2(H, i, j) + g2(H, j, i) + g2(H, a, b) +
                            g2(H, b, a) - g2(H, a, i) - g2(H, i, a) - g2(H, b, i) - g2(H, i, b) - g2(H, a, j) -
                            g2(H, j, a) - g2(H, b, j) - g2(H, j, b);
          Det q = alpha ? Det{ex, other} : Det{other, ex};
          out.push_back({q, coeff * h, E0 - hd});
        }
    }
}
void os_doubles_contribs(const Ham& H, double coeff, uint64_t sa, uint64_t sb, const std::vector<uint32_t>& oa,
                         const std::vector<uint32_t>& va, const std::vector<uint32_t>& ob,
                         const std::vector<uint32_t>& vb, const std::vector<double>& ea,
                         const std::vector<double>& eb, double hdiag, double E0, double tol,
                         std::vector<Contrib>& out) {
  for (auto i : oa)
    for (auto a : va) {
      const double s_a = single_excitation_sign(sa, a, i);
      for (auto j : ob)
        for (auto b : vb) {
          const double V = H.v(a, i, b, j);
          if (std::abs(coeff * V) < tol) continue;
          const double s = s_a * single_excitation_sign(sb, b, j);
          const double hd = hdiag + ea[a] + eb[b] - ea[i] - eb[j] + v2(H, i, j) + v2(H, a, b) - g2(H, a, i) -
                            g2(H, i, a) - g2(H, b, j) - g2(H, j, b) - v2(H, a, j) - v2(H, i, b);
          Det q{(sa ^ (1ull << i)) | (1ull << a), (sb ^ (1ull << j)) | (1ull << b)};
          out.push_back({q, coeff * s * V, E0 - hd});
        }
    }
}

// Every contribution of one wavefunction determinant P (coefficient c): the
// singles and doubles of each spin and the opposite-spin doubles, in the
// order of the reference's per-determinant loop (determinant_search.hpp:
// 386-474, pt2.hpp:298-344), then P itself with an infinite score (it is in
// the wavefunction, so it drops out after accumulation).
// (just_singles: the search's option, determinant_search.hpp:274-296)
void contribs_of(const Ham& H, const Det& P, double c, double E0, double tol, std::vector<Contrib>& out,
                 bool just_singles = false) {
  const int n = H.n;
  std::vector<uint32_t> oa, va, ob, vb;
  for (int p = 0; p < n; ++p) {
    ((P.a >> p) & 1 ? oa : va).push_back(p);
    ((P.b >> p) & 1 ? ob : vb).push_back(p);
  }
  const double hdiag = H.me_diag(oa, ob);
  const std::vector<double> ea = orbital_ens(H, oa, ob), eb = orbital_ens(H, ob, oa);
  singles_contribs(H, c, P.a, P.b, true, oa, va, ob, ea, hdiag, E0, tol, out);
  if (!just_singles) {
    ss_doubles_contribs(H, c, P.a, P.b, true, oa, va, ea, hdiag, E0, tol, out);
    os_doubles_contribs(H, c, P.a, P.b, oa, va, ob, vb, ea, eb, hdiag, E0, tol, out);
  }
  singles_contribs(H, c, P.b, P.a, false, ob, vb, oa, eb, hdiag, E0, tol, out);
  if (!just_singles) ss_doubles_contribs(H, c, P.b, P.a, false, ob, vb, eb, hdiag, E0, tol, out);
  out.push_back({P, std::numeric_limits<double>::infinity(), 1.0});
}

// asci_search (include/macis/asci/determinant_search.hpp:808-1123) on the
// full contribution list: enumerate, sort by determinant and accumulate
// (determinant_sort.hpp:115-370), drop the core (infinite score), prune
// |rv| <= rv_prune_tol, keep the top ndets_max - ncore by |rv| with ties at
// the cutoff kept (:994-1080), append the core.  (The reference partitions the
// enumeration by alpha constraints for parallelism; every target determinant
// lies in one constraint, so the accumulated scores are the same.)
std::vector<Det> asci_search(const Ham& H, const AsciSettings& S, int64_t ndets_max, const std::vector<Det>& core,
                             const std::vector<double>& C, double E0) {
  const int n = H.n;
  const int64_t ncore = (int64_t)core.size();
  int nth = 1;
#ifdef _OPENMP
  nth = omp_get_max_threads();
#endif
  std::vector<std::vector<Contrib>> per(nth);
#pragma omp parallel
  {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    std::vector<Contrib>& out = per[tid];
    // static: thread t takes the t-th contiguous block of the core, so the
    // lists joined in thread order follow the core's order and the stable
    // sort below sums each determinant's contributions in a fixed order
#pragma omp for schedule(static)
    for (int64_t ip = 0; ip < ncore; ++ip) contribs_of(H, core[ip], C[ip], E0, S.h_el_tol, out, S.just_singles != 0);
  }
  (void)n;
  std::vector<Contrib> all;
  for (auto& v : per) all.insert(all.end(), v.begin(), v.end());
  std::stable_sort(all.begin(), all.end(), [](const Contrib& x, const Contrib& y) { return spin_less(x.q, y.q); });
  std::vector<Contrib> acc;
  for (size_t k = 0; k < all.size();) {
    size_t e = k + 1;
    Contrib c0 = all[k];
    for (; e < all.size() && all[e].q == all[k].q; ++e) c0.c_h += all[e].c_h;
    if (!std::isinf(c0.c_h) && std::abs(c0.rv()) > S.rv_prune_tol) acc.push_back(c0);
    k = e;
  }
  const int64_t topk = ndets_max - ncore;
  std::vector<Det> out;
  if ((int64_t)acc.size() > topk && topk >= 0) {
    std::vector<double> sc(acc.size());
    for (size_t i = 0; i < acc.size(); ++i) sc[i] = std::abs(acc[i].rv());
    std::vector<double> tmp = sc;
    double kth = 0.;
    if (topk > 0) {
      std::nth_element(tmp.begin(), tmp.begin() + (topk - 1), tmp.end(), std::greater<double>());
      kth = tmp[topk - 1];
    } else {
      kth = std::numeric_limits<double>::infinity();
    }
    for (size_t i = 0; i < acc.size(); ++i)
      if (sc[i] >= kth) out.push_back(acc[i].q);
  } else {
    for (auto& c : acc) out.push_back(c.q);
  }
  out.insert(out.end(), core.begin(), core.end());
  return out;
}

// asci_pt2_constraint (include/macis/asci/pt2.hpp:59-565): the second-order
// energy E_PT2 = sum over determinants Q outside the wavefunction of
// (sum_P c_P <Q|H|P>)^2 / (E0 - H_QQ) (asci_contrib::pt2, determinant_
// contributions.hpp:49-55), single contributions with |c_P <Q|H|P>| < pt2_tol
// dropped, H_QQ by the fast diagonals; the wavefunction must be sorted by
// spin_comparator (pt2.hpp:79-80).  The reference splits the Q space by alpha
// constraints to balance MPI ranks and threads and to bound the memory of its
// sort-and-accumulate; here Q is split by a hash into passes of at most
// `pass_max` contributions.  Every Q lies in one part of either split, so the
// accumulated sums are the same.
inline uint64_t det_mix(const Det& q) {
  uint64_t x = q.a * 0x9e3779b97f4a7c15ULL ^ (q.b + 0x632be59bd9b4e019ULL);
  x ^= x >> 31;
  x *= 0xd6e8feb86659fd93ULL;
  x ^= x >> 32;
  return x;
}
double asci_pt2(const Ham& H, const std::vector<Det>& dets, const std::vector<double>& C, double E0, double tol,
                int64_t* npt2, int64_t pass_max = (int64_t)1 << 25) {
  if (!std::is_sorted(dets.begin(), dets.end(), spin_less)) throw std::runtime_error("PT2 Only Works with Sorted Wfns");
  const int n = H.n;
  int64_t total = 0;
  for (const Det& P : dets) {
    const int ka = __builtin_popcountll(P.a), kb = __builtin_popcountll(P.b);
    const int64_t sa = (int64_t)ka * (n - ka), sb = (int64_t)kb * (n - kb);
    total += 1 + sa + sb + sa * sb + (int64_t)ka * (ka - 1) / 2 * ((n - ka) * (n - ka - 1) / 2) +
             (int64_t)kb * (kb - 1) / 2 * ((n - kb) * (n - kb - 1) / 2);
  }
  const uint64_t npass = (uint64_t)std::max<int64_t>(1, (total + pass_max - 1) / pass_max);
  int nth = 1;
#ifdef _OPENMP
  nth = omp_get_max_threads();
#endif
  double EPT2 = 0.;
  int64_t NPT2 = 0;
  for (uint64_t pass = 0; pass < npass; ++pass) {
    std::vector<std::vector<Contrib>> per(nth);
#pragma omp parallel
    {
      int tid = 0;
#ifdef _OPENMP
      tid = omp_get_thread_num();
#endif
      std::vector<Contrib> tmp;
#pragma omp for schedule(dynamic, 16)
      for (int64_t ip = 0; ip < (int64_t)dets.size(); ++ip) {
        tmp.clear();
        contribs_of(H, dets[ip], C[ip], E0, tol, tmp);
        for (const Contrib& x : tmp)
          if (npass == 1 || det_mix(x.q) % npass == pass) per[tid].push_back(x);
      }
    }
    std::vector<Contrib> all;
    size_t m = 0;
    for (auto& v : per) m += v.size();
    all.reserve(m);
    for (auto& v : per) {
      all.insert(all.end(), v.begin(), v.end());
      std::vector<Contrib>().swap(v);
    }
    auto less = [](const Contrib& x, const Contrib& y) { return spin_less(x.q, y.q); };
#ifdef _OPENMP
    __gnu_parallel::sort(all.begin(), all.end(), less);
#else
    std::sort(all.begin(), all.end(), less);
#endif
    for (size_t k = 0; k < all.size();) {
      size_t e = k + 1;
      Contrib c0 = all[k];
      for (; e < all.size() && all[e].q == all[k].q; ++e) c0.c_h += all[e].c_h;
      if (!std::isinf(c0.c_h)) {
        EPT2 += c0.c_h * c0.c_h / c0.h_diag;
        ++NPT2;
      }
      k = e;
    }
  }
  if (npt2) *npt2 = NPT2;
  return EPT2;
}

// ---------------------------------------------------------------- CASSCF
// casscf_diis / mcscf_impl (include/macis/mcscf/mcscf_impl.hpp:25-262) with
// inactive_fock_matrix, active_hamiltonian, inactive_energy,
// active_fock_matrix, aux_q_matrix, generalized_fock_matrix
// (src/macis/mcscf/fock_matrices.cxx:16-186), fock_to_linear_orb_grad and
// linear_orb_rot_to_matrix (orbital_rotation_utilities.cxx:16-118),
// approx_diag_hessian (orbital_hessian.cxx:16-62), precond_cg_orbital_step
// (orbital_steps.cxx:16-37), DIIS (include/macis/mcscf/diis.hpp),
// compute_orbital_rotation (orbital_gradient.cxx:17-28) and the two- and
// four-index transforms (src/macis/util/transform.cxx:17-60).  The CASCI of an
// iteration is compute_casci_rdms (include/macis/mcscf/cas.hpp:33-88): the
// complete active space, the SDL CSR, selected_ci_diag warm-started from the
// previous vector, the spin-traced RDMs.  Matrices column-major.
struct McscfSettings {
  int64_t max_macro_iter = 100;
  double max_orbital_step = 0.5, orb_grad_tol = 5e-6;
  int enable_diis = 1;
  int64_t diis_start_iter = 3, diis_nkeep = 10;
  double ci_res_tol = 1e-8;
  int64_t ci_max_subspace = 200;
  double ci_matel_tol = std::numeric_limits<double>::epsilon();
};

// exp(A) of a small square matrix: scaling and squaring of the Taylor series
std::vector<double> expm(int n, std::vector<double> A) {
  double nrm = 0.;
  for (int i = 0; i < n; ++i) {
    double r = 0.;
    for (int j = 0; j < n; ++j) r += std::abs(A[i + (size_t)n * j]);
    nrm = std::max(nrm, r);
  }
  int sq = 0;
  while (nrm > 0.125) {
    nrm /= 2.;
    ++sq;
  }
  for (double& x : A) x = std::ldexp(x, -sq);
  const size_t n2 = (size_t)n * n;
  std::vector<double> E(n2, 0.), P(n2, 0.), Q(n2);
  for (int i = 0; i < n; ++i) E[i * (n + 1)] = P[i * (n + 1)] = 1.;
  for (int k = 1; k < 40; ++k) {
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        double t = 0.;
        for (int l = 0; l < n; ++l) t += P[i + (size_t)n * l] * A[l + (size_t)n * j];
        Q[i + (size_t)n * j] = t / k;
      }
    P.swap(Q);
    double pm = 0.;
    for (size_t i = 0; i < n2; ++i) {
      E[i] += P[i];
      pm = std::max(pm, std::abs(P[i]));
    }
    if (pm < 1e-20) break;
  }
  for (int s = 0; s < sq; ++s) {
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        double t = 0.;
        for (int l = 0; l < n; ++l) t += E[i + (size_t)n * l] * E[l + (size_t)n * j];
        Q[i + (size_t)n * j] = t;
      }
    E.swap(Q);
  }
  return E;
}

// fock_matrices.cxx building blocks (n x n column-major; V n^4; active RDMs
// na^2 / na^4; active orbitals ni .. ni+na-1)
inline double v4(const double* V, int n, int p, int q, int r, int s) {
  return V[p + (size_t)n * (q + (size_t)n * (r + (size_t)n * s))];
}
// inactive_fock_matrix (:25-41): Fi = T + sum_i 2 (pq|ii) - (pi|iq)
void inactive_fock(int n, int ni, const double* T, const double* V, double* Fi) {
  for (int q = 0; q < n; ++q)
    for (int p = 0; p < n; ++p) {
      double t = 0.;
      for (int i = 0; i < ni; ++i) t += 2. * v4(V, n, p, q, i, i) - v4(V, n, p, i, i, q);
      Fi[p + (size_t)n * q] = T[p + (size_t)n * q] + t;
    }
}
// inactive_energy (:16-23): sum_i T_ii + Fi_ii
double inactive_energy(int n, int ni, const double* T, const double* Fi) {
  double E = 0.;
  for (int i = 0; i < ni; ++i) E += T[i * (n + 1)] + Fi[i * (n + 1)];
  return E;
}
// active_fock_matrix (:89-110): Fa = sum_vw g_vw [(pq|vw) - 1/2 (pw|vq)]
void active_fock(int n, int ni, int na, const double* V, const double* A1, double* Fa) {
  for (int q = 0; q < n; ++q)
    for (int p = 0; p < n; ++p) {
      double t = 0.;
      for (int w = 0; w < na; ++w)
        for (int v = 0; v < na; ++v)
          t += A1[v + (size_t)na * w] * (v4(V, n, p, q, v + ni, w + ni) - 0.5 * v4(V, n, p, w + ni, v + ni, q));
      Fa[p + (size_t)n * q] = t;
    }
}
// aux_q_matrix (:112-137): Q(v, p) = 2 sum_wxy G_vwxy (pw|xy)
void aux_q(int n, int ni, int na, const double* V, const double* A2, double* Q) {
  for (int p = 0; p < n; ++p)
    for (int v = 0; v < na; ++v) {
      double t = 0.;
      for (int y = 0; y < na; ++y)
        for (int x = 0; x < na; ++x)
          for (int w = 0; w < na; ++w)
            t += A2[v + na * (w + na * (x + (size_t)na * y))] * v4(V, n, p, w + ni, x + ni, y + ni);
      Q[v + (size_t)na * p] = 2. * t;
    }
}
// generalized_fock_matrix (:139-163): inactive rows 2 (Fi + Fa), active rows
// Fi g + Q, virtual rows zero
void generalized_fock(int n, int ni, int na, const double* Fi, const double* Fa, const double* A1, const double* Q,
                      double* F) {
  std::fill(F, F + (size_t)n * n, 0.);
  for (int p = 0; p < n; ++p) {
    for (int i = 0; i < ni; ++i) F[i + (size_t)n * p] = 2. * (Fi[p + (size_t)n * i] + Fa[p + (size_t)n * i]);
    for (int v = 0; v < na; ++v) {
      double t = 0.;
      for (int w = 0; w < na; ++w) t += Fi[p + (size_t)n * (w + ni)] * A1[w + (size_t)na * v];
      F[(v + ni) + (size_t)n * p] = t + Q[v + (size_t)na * p];
    }
  }
}
// energy_from_generalized_fock (:228-256)
double energy_from_generalized_fock(int n, int ni, int na, const double* T, const double* A1, const double* F) {
  double E = 0.;
  for (int i = 0; i < ni; ++i) E += 2. * T[i * (n + 1)];
  for (int y = 0; y < na; ++y)
    for (int x = 0; x < na; ++x) E += A1[x + (size_t)na * y] * T[(x + ni) + (size_t)n * (y + ni)];
  for (int p = 0; p < ni + na; ++p) E += F[p * (n + 1)];
  return 0.5 * E;
}

double casscf(const McscfSettings& S, int nalpha, int nbeta, int no, int ni, int na, double E_core, const double* T0,
              const double* V0, double* A1, double* A2, int64_t* iters_out, int* conv_out) {
  const int nv = no - ni - na;
  if (nv < 0 || na < 1 || ni < 0) throw std::runtime_error("bad orbital partition");
  const size_t no2 = (size_t)no * no, no4 = no2 * no2, na2 = (size_t)na * na, na4 = na2 * na2;
  const int rot = nv * (ni + na) + na * ni;
  auto VV = [&](const std::vector<double>& W, int p, int q, int r, int s4) { return v4(W.data(), no, p, q, r, s4); };
  std::vector<double> T(T0, T0 + no2), V(V0, V0 + no4);
  // complete active space (generate_hilbert_space order)
  auto strings = [](int n, int k) {
    std::vector<char> v(n, 0);
    std::fill_n(v.begin(), k, 1);
    std::vector<uint64_t> out;
    do {
      uint64_t x = 0;
      for (int i = 0; i < n; ++i)
        if (v[i]) x |= 1ull << i;
      out.push_back(x);
    } while (std::prev_permutation(v.begin(), v.end()));
    return out;
  };
  const std::vector<uint64_t> sa = strings(na, nalpha), sb = strings(na, nbeta);
  std::vector<uint64_t> da, db;
  for (uint64_t x : sa)
    for (uint64_t y : sb) {
      da.push_back(x);
      db.push_back(y);
    }
  const int64_t nd = (int64_t)da.size();
  std::vector<double> X(nd, 0.), Fi(no2), Fa(no2), F(no2), Q((size_t)na * no), Ta(na2), Va(na4);
  double E_inact = 0.;
  auto active_hamiltonian = [&]() {
    inactive_fock(no, ni, T.data(), V.data(), Fi.data());
    for (int y = 0; y < na; ++y)
      for (int x = 0; x < na; ++x) Ta[x + (size_t)na * y] = Fi[(x + ni) + (size_t)no * (y + ni)];
    for (int w = 0; w < na; ++w)
      for (int z = 0; z < na; ++z)
        for (int y = 0; y < na; ++y)
          for (int x = 0; x < na; ++x)
            Va[x + na * (y + na * (z + (size_t)na * w))] = VV(V, x + ni, y + ni, z + ni, w + ni);
    E_inact = E_core + inactive_energy(no, ni, T.data(), Fi.data());
  };
  auto casci = [&]() {
    Ham H;
    H.init(na, Ta.data(), Va.data());
    std::unique_ptr<Csr> M(build_csr_sdl(H, da.data(), db.data(), nd, S.ci_matel_tol));
    std::vector<double> D(nd, 0.);
    for (int64_t i = 0; i < nd; ++i)
      for (int64_t k = M->rowptr[i]; k < M->rowptr[i + 1]; ++k)
        if (M->colind[k] == i) D[i] = M->nzval[k];
    double mx = 0.;
    for (double x : X) mx = std::max(mx, std::abs(x));
    if (!(mx > 1. / (double)nd)) {
      std::fill(X.begin(), X.end(), 0.);
      X[std::min_element(D.begin(), D.end()) - D.begin()] = 1.;
    }
    double E = 0.;
    int64_t it = 0;
    if (nd == 1) {
      X[0] = 1.;
      E = M->nzval[0];
    } else if (davidson(*M, std::min<int64_t>(S.ci_max_subspace, nd), D.data(), S.ci_res_tol, X.data(), &E, &it)) {
      throw std::runtime_error("Davidson Did Not Converge!");
    }
    std::vector<double> aa(na2, 0.), bb(na2, 0.), aaaa(na4, 0.), bbbb(na4, 0.), aabb(na4, 0.);
    Rdms R{na, aa.data(), bb.data(), aaaa.data(), bbbb.data(), aabb.data()};
    rdms_spin_dep(da.data(), db.data(), nd, X.data(), R);
    for (size_t i = 0; i < na2; ++i) A1[i] = aa[i] + bb[i];
    for (int s4 = 0; s4 < na; ++s4)
      for (int r = 0; r < na; ++r)
        for (int q = 0; q < na; ++q)
          for (int p = 0; p < na; ++p) {
            const size_t i = p + na * (q + na * (r + (size_t)na * s4)), j = r + na * (s4 + na * (p + (size_t)na * q));
            A2[i] = aaaa[i] + bbbb[i] + aabb[i] + aabb[j];
          }
    return E;
  };
  std::vector<double> OG(rot), DH(rot);
  auto grad = [&]() {
    active_fock(no, ni, na, V.data(), A1, Fa.data());
    aux_q(no, ni, na, V.data(), A2, Q.data());
    generalized_fock(no, ni, na, Fi.data(), Fa.data(), A1, Q.data(), F.data());
    auto g = [&](int p, int q) { return 2. * (F[p + (size_t)no * q] - F[q + (size_t)no * p]); };
    int k = 0;
    for (int i = 0; i < ni; ++i)
      for (int a = 0; a < nv; ++a) OG[k++] = g(a + ni + na, i);
    for (int x = 0; x < na; ++x)
      for (int a = 0; a < nv; ++a) OG[k++] = g(a + ni + na, x + ni);
    for (int i = 0; i < ni; ++i)
      for (int x = 0; x < na; ++x) OG[k++] = g(x + ni, i);
    double n2 = 0.;
    for (double x : OG) n2 += x * x;
    return std::sqrt(n2);
  };
  auto hess = [&]() {
    auto f = [&](int p) { return Fi[p * (no + 1)] + Fa[p * (no + 1)]; };
    int k = 0;
    for (int i = 0; i < ni; ++i)
      for (int a = 0; a < nv; ++a) DH[k++] = 4. * (f(a + ni + na) - f(i));
    for (int x = 0; x < na; ++x)
      for (int a = 0; a < nv; ++a) DH[k++] = 2. * A1[x * (na + 1)] * f(a + ni + na) - 2. * F[(x + ni) * (no + 1)];
    for (int i = 0; i < ni; ++i)
      for (int x = 0; x < na; ++x)
        DH[k++] = 2. * A1[x * (na + 1)] * f(i) + 4. * (f(x + ni) - f(i)) - 2. * F[(x + ni) * (no + 1)];
  };
  auto to_mat = [&](const std::vector<double>& kl) {
    std::vector<double> K(no2, 0.);
    int t = 0;
    auto put = [&](int A, int I) {
      K[A + (size_t)no * I] = kl[t];
      K[I + (size_t)no * A] = -kl[t];
      ++t;
    };
    for (int i = 0; i < ni; ++i)
      for (int a = 0; a < nv; ++a) put(a + ni + na, i);
    for (int x = 0; x < na; ++x)
      for (int a = 0; a < nv; ++a) put(a + ni + na, x + ni);
    for (int i = 0; i < ni; ++i)
      for (int x = 0; x < na; ++x) put(x + ni, i);
    return K;
  };
  auto transform = [&](const std::vector<double>& U) {
    // T = U^T T0 U; V(pqrs) = sum U_ap U_bq U_cr U_ds V0(abcd), one index at a time
    std::vector<double> t1(no2);
    for (int q = 0; q < no; ++q)
      for (int a = 0; a < no; ++a) {
        double t = 0.;
        for (int b = 0; b < no; ++b) t += T0[a + (size_t)no * b] * U[b + (size_t)no * q];
        t1[a + (size_t)no * q] = t;
      }
    for (int q = 0; q < no; ++q)
      for (int p = 0; p < no; ++p) {
        double t = 0.;
        for (int a = 0; a < no; ++a) t += U[a + (size_t)no * p] * t1[a + (size_t)no * q];
        T[p + (size_t)no * q] = t;
      }
    std::vector<double> A(V0, V0 + no4), B(no4);
    for (int pass = 0; pass < 4; ++pass) {
      // B(j,k,l,p) = sum_a A(a,j,k,l) U(a,p): the contracted index moves last
      const int64_t n3 = (int64_t)no2 * no;
#pragma omp parallel for schedule(static)
      for (int64_t t = 0; t < n3 * no; ++t) {
        const int64_t rest = t % n3, p = t / n3;
        double acc = 0.;
        for (int a = 0; a < no; ++a) acc += A[a + no * rest] * U[a + (size_t)no * p];
        B[t] = acc;
      }
      A.swap(B);
    }
    V.swap(A);
  };

  active_hamiltonian();
  double tr = 0.;
  for (int i = 0; i < na; ++i) tr += A1[i * (na + 1)];
  if (std::abs(tr - nalpha - nbeta) > 1e-6) (void)casci();
  double E0 = E_inact;
  for (size_t i = 0; i < na2; ++i) E0 += A1[i] * Ta[i];
  for (size_t i = 0; i < na4; ++i) E0 += A2[i] * Va[i];
  double gn = grad();
  bool conv = gn < S.orb_grad_tol;
  std::vector<double> U(no2, 0.), K(no2, 0.);
  for (int i = 0; i < no; ++i) U[i * (no + 1)] = 1.;
  std::vector<std::pair<std::vector<double>, std::vector<double>>> hist;
  int64_t it = 0;
  for (; it < S.max_macro_iter && !conv; ++it) {
    const std::vector<double> Ksav = K;
    hess();
    std::vector<double> kl(rot);
    double amax = 0.;
    for (int p = 0; p < rot; ++p) {
      kl[p] = -OG[p] / DH[p];
      amax = std::max(amax, std::abs(kl[p]));
    }
    if (amax > S.max_orbital_step)
      for (double& x : kl) x *= S.max_orbital_step / amax;
    const std::vector<double> Ks = to_mat(kl);
    for (size_t i = 0; i < no2; ++i) K[i] += Ks[i];
    if (S.enable_diis && it >= S.diis_start_iter) {
      if ((int64_t)hist.size() == S.diis_nkeep) hist.erase(hist.begin());
      hist.emplace_back(K, OG);
      if (it >= S.diis_start_iter + 2) {
        // min |sum c_i e_i| with sum c_i = 1 (the bordered system, least squares)
        const int m = (int)hist.size(), mb = m + 1;
        std::vector<double> B((size_t)mb * mb, 0.), w(mb);
        for (int i = 0; i < m; ++i)
          for (int j = 0; j < m; ++j) {
            double d = 0.;
            for (int r = 0; r < rot; ++r) d += hist[i].second[r] * hist[j].second[r];
            B[i + (size_t)mb * j] = d;
          }
        for (int i = 0; i < m; ++i) B[i + (size_t)mb * m] = B[m + (size_t)mb * i] = 1.;
        jacobi_syev(mb, B.data(), mb, w.data());  // B: eigenvectors, w: eigenvalues
        double wmax = 0.;
        for (double x : w) wmax = std::max(wmax, std::abs(x));
        std::vector<double> c(mb, 0.);
        for (int k = 0; k < mb; ++k) {
          if (!(std::abs(w[k]) > std::numeric_limits<double>::epsilon() * wmax * mb)) continue;
          const double f = B[m + (size_t)mb * k] / w[k];
          for (int i = 0; i < mb; ++i) c[i] += B[i + (size_t)mb * k] * f;
        }
        std::fill(K.begin(), K.end(), 0.);
        for (int i = 0; i < m; ++i)
          for (size_t r = 0; r < no2; ++r) K[r] += c[i] * hist[i].first[r];
      }
    }
    std::vector<double> dK(no2);
    for (size_t i = 0; i < no2; ++i) dK[i] = -(it == 0 ? K[i] : K[i] - Ksav[i]);
    const std::vector<double> Us = expm(no, dK);
    std::vector<double> Un(no2);
    for (int j = 0; j < no; ++j)
      for (int i = 0; i < no; ++i) {
        double t = 0.;
        for (int l = 0; l < no; ++l) t += U[i + (size_t)no * l] * Us[l + (size_t)no * j];
        Un[i + (size_t)no * j] = t;
      }
    U.swap(Un);
    transform(U);
    active_hamiltonian();
    E0 = casci() + E_inact;
    gn = grad();
    conv = gn / std::sqrt((double)std::max(rot, 1)) < S.orb_grad_tol;
  }
  if (iters_out) *iters_out = it;
  if (conv_out) *conv_out = conv;
  return E0;
}

// selected_ci_diag (selected_ci_diag.hpp:111-158) on a sorted determinant list
double sci_diag(const Ham& H, const AsciSettings& S, const std::vector<Det>& dets, std::vector<double>& X) {
  std::vector<uint64_t> a(dets.size()), b(dets.size());
  for (size_t i = 0; i < dets.size(); ++i) {
    a[i] = dets[i].a;
    b[i] = dets[i].b;
  }
  std::unique_ptr<Csr> M(build_csr_sdl(H, a.data(), b.data(), (int64_t)dets.size(), S.ci_matel_tol));
  X.resize(dets.size(), 0.);
  std::vector<double> D(M->n);
  for (int64_t i = 0; i < M->n; ++i) {
    D[i] = 0.;
    for (int64_t k = M->rowptr[i]; k < M->rowptr[i + 1]; ++k)
      if (M->colind[k] == i) {
        D[i] = M->nzval[k];
        break;
      }
  }
  double maxc = 0.;
  for (double x : X) maxc = std::max(maxc, std::abs(x));
  if (!(maxc > 1. / (double)X.size())) {
    std::fill(X.begin(), X.end(), 0.);
    X[std::min_element(D.begin(), D.end()) - D.begin()] = 1.;
  }
  double E = 0.;
  int64_t it = 0;
  if (davidson(*M, S.ci_max_subspace, D.data(), S.ci_res_tol, X.data(), &E, &it))
    throw std::runtime_error("Davidson Did Not Converge!");
  return E;
}

// asci_iter (include/macis/asci/iteration.hpp:50-226)
double asci_iter(const Ham& H, const AsciSettings& S, int64_t ndets_max, double E0, std::vector<Det>& wfn,
                 std::vector<double>& X) {
  if (wfn.size() > 1) {  // reorder_ci_on_coeff (determinant_sort.hpp:45-64)
    std::vector<size_t> idx(wfn.size());
    std::iota(idx.begin(), idx.end(), 0);
    std::sort(idx.begin(), idx.end(), [&](size_t i, size_t j) { return std::abs(X[i]) > std::abs(X[j]); });
    std::vector<Det> w2(wfn.size());
    std::vector<double> x2(wfn.size());
    for (size_t i = 0; i < idx.size(); ++i) {
      w2[i] = wfn[idx[i]];
      x2[i] = X[idx[i]];
    }
    wfn.swap(w2);
    X.swap(x2);
  }
  size_t nkeep = 0;
  if (S.core_fixed) {
    nkeep = std::min<size_t>(S.ncdets_max, wfn.size());
  } else {
    double w = 0.;
    for (size_t i = 0; i < wfn.size(); ++i) {
      w += X[i] * X[i];
      nkeep++;
      if (w >= S.core_threshold) break;
    }
  }
  if (wfn.size() > 1) {  // reorder_ci_on_alpha of the core (determinant_sort.hpp:66-90)
    std::vector<size_t> idx(nkeep);
    std::iota(idx.begin(), idx.end(), 0);
    std::sort(idx.begin(), idx.end(), [&](size_t i, size_t j) { return spin_less(wfn[i], wfn[j]); });
    std::vector<Det> w2(nkeep);
    std::vector<double> x2(nkeep);
    for (size_t i = 0; i < nkeep; ++i) {
      w2[i] = wfn[idx[i]];
      x2[i] = X[idx[i]];
    }
    std::copy(w2.begin(), w2.end(), wfn.begin());
    std::copy(x2.begin(), x2.end(), X.begin());
  }
  std::vector<Det> old_wfn = wfn;
  std::vector<double> old_X = X;
  std::vector<Det> core(wfn.begin(), wfn.begin() + nkeep);
  std::vector<double> ccore(X.begin(), X.begin() + nkeep);
  wfn = asci_search(H, S, ndets_max, core, ccore, E0);
  std::sort(wfn.begin(), wfn.end(), spin_less);
  std::vector<double> Xl;
  if (S.warm_start) {
    std::vector<size_t> idx(old_wfn.size());
    std::iota(idx.begin(), idx.end(), 0);
    std::sort(idx.begin(), idx.end(), [&](size_t i, size_t j) { return spin_less(old_wfn[i], old_wfn[j]); });
    Xl.assign(wfn.size(), 0.);
    for (size_t i = 0; i < wfn.size(); ++i) {
      auto it = std::lower_bound(idx.begin(), idx.end(), wfn[i],
                                 [&](size_t k, const Det& d) { return spin_less(old_wfn[k], d); });
      if (it != idx.end() && old_wfn[*it] == wfn[i]) Xl[i] = old_X[*it];
    }
    double nrm = 0.;
    for (double x : Xl) nrm += x * x;
    nrm = std::sqrt(nrm);
    if (nrm < std::max(S.min_warm_start_overlap, 2.220446049250313e-16))
      Xl.clear();
    else
      for (double& x : Xl) x /= nrm;
  }
  const double E = sci_diag(H, S, wfn, Xl);
  X = Xl;
  return E;
}

// The natural-orbital rotation of asci_grow (grow.hpp:163-252): the
// spin-summed 1-RDM of (wfn, X), the eigenvectors of -RDM in ascending order
// (syev: occupations descending), T and V transformed by them
// (two_index_transform / four_index_transform, transform.cxx), intermediates
// rebuilt.  U (n x n) receives the rotation.
void rotate_to_natural_orbitals(Ham& H, const std::vector<Det>& wfn, const std::vector<double>& X,
                                std::vector<double>& U) {
  const int n = H.n;
  const size_t n2 = (size_t)n * n, n4 = n2 * n2;
  std::vector<uint64_t> a(wfn.size()), b(wfn.size());
  for (size_t i = 0; i < wfn.size(); ++i) {
    a[i] = wfn[i].a;
    b[i] = wfn[i].b;
  }
  std::vector<double> aa(n2, 0.), bb(n2, 0.);
  Rdms R{n, aa.data(), bb.data(), nullptr, nullptr, nullptr};
  rdms_spin_dep(a.data(), b.data(), (int64_t)wfn.size(), X.data(), R);
  U.assign(n2, 0.);
  for (size_t i = 0; i < n2; ++i) U[i] = -(aa[i] + bb[i]);
  std::vector<double> w(n);
  jacobi_syev(n, U.data(), n, w.data());
  std::vector<double> t1(n2), T(n2);
  for (int q = 0; q < n; ++q)
    for (int p = 0; p < n; ++p) {
      double t = 0.;
      for (int k = 0; k < n; ++k) t += H.T[p + (size_t)n * k] * U[k + (size_t)n * q];
      t1[p + (size_t)n * q] = t;
    }
  for (int q = 0; q < n; ++q)
    for (int p = 0; p < n; ++p) {
      double t = 0.;
      for (int k = 0; k < n; ++k) t += U[k + (size_t)n * p] * t1[k + (size_t)n * q];
      T[p + (size_t)n * q] = t;
    }
  std::vector<double> A(H.V), B(n4);
  const int64_t n3 = (int64_t)n2 * n;
  for (int pass = 0; pass < 4; ++pass) {
#pragma omp parallel for schedule(static)
    for (int64_t t = 0; t < n3 * n; ++t) {
      const int64_t rest = t % n3, p = t / n3;
      double acc = 0.;
      for (int k = 0; k < n; ++k) acc += A[k + n * rest] * U[k + (size_t)n * p];
      B[t] = acc;
    }
    A.swap(B);
  }
  H.init(n, T.data(), A.data());
}

// asci_grow (include/macis/asci/grow.hpp:45-268), natural-orbital rotation
// included when S.grow_with_rot (it rotates H; rot accumulates the
// rotations); steps, when given, receives for each asci_iter the size asked
// and the size reached
double asci_grow(Ham& H, const AsciSettings& S, double E0, std::vector<Det>& wfn, std::vector<double>& X,
                 std::vector<int64_t>* steps = nullptr, std::vector<double>* rot = nullptr) {
  size_t prev = wfn.size();
  double gf = S.grow_factor;
  while ((int64_t)wfn.size() < S.ntdets_max) {
    // taper (grow.hpp:97-107)
    double eff = gf;
    if (S.taper_grow_factor > 0. && (int64_t)std::ceil(wfn.size() * gf) > S.ntdets_max)
      eff = std::max(S.min_grow_factor, S.taper_grow_factor);
    int64_t nnew =
        std::min<int64_t>(std::max<int64_t>(S.ntdets_min, (int64_t)std::ceil(wfn.size() * eff)), S.ntdets_max);
    if (nnew <= (int64_t)wfn.size()) {
      nnew = std::min<int64_t>(wfn.size() + 1, S.ntdets_max);
      if (nnew <= (int64_t)wfn.size()) break;
    }
    const double E = asci_iter(H, S, nnew, E0, wfn, X);
    if (steps) {
      steps->push_back(nnew);
      steps->push_back((int64_t)wfn.size());
    }
    if ((int64_t)wfn.size() < nnew) {
      gf = std::max(S.min_grow_factor, gf * S.backoff);
      if (wfn.size() <= prev) break;
    } else {
      gf = std::min(S.grow_factor, gf * S.recovery);
    }
    prev = wfn.size();
    if (S.grow_with_rot && (int64_t)wfn.size() >= S.rot_size_start) {
      std::vector<double> U;
      rotate_to_natural_orbitals(H, wfn, X, U);
      if (rot) {
        const int n = H.n;
        if (rot->empty()) {
          *rot = U;
        } else {
          std::vector<double> Rr((size_t)n * n, 0.);
          for (int j = 0; j < n; ++j)
            for (int k = 0; k < n; ++k)
              for (int i = 0; i < n; ++i) Rr[i + (size_t)n * j] += (*rot)[i + (size_t)n * k] * U[k + (size_t)n * j];
          rot->swap(Rr);
        }
      }
      std::vector<double> Xr;  // rediagonalised from the diagonal guess; the iteration's energy is kept
      sci_diag(H, S, wfn, Xr);
      X.swap(Xr);
    }
    E0 = E;
  }
  return E0;
}

// asci_refine (include/macis/asci/refine.hpp:44-237), union stabilisation included
double asci_refine(const Ham& H, const AsciSettings& S, double E0, std::vector<Det>& wfn, std::vector<double>& X) {
  int64_t ndets = (int64_t)wfn.size();
  bool converged = false;
  double prev_dE = 0.;
  int osc = 0;
  int64_t max_iter = S.max_refine_iter, ext = 0;
  std::vector<Det> prev_wfn;
  for (int64_t iter = 0; iter < max_iter; ++iter) {
    const double E = asci_iter(H, S, ndets, E0, wfn, X);
    if ((int64_t)wfn.size() != ndets) {
      ndets = (int64_t)wfn.size();
      if (ndets < S.ntdets_min) break;
    }
    const double dE = E - E0;
    if (std::abs(dE) < S.refine_energy_tol) {
      E0 = E;
      converged = true;
      break;
    }
    if (iter > 0 && prev_dE * dE < 0 && std::abs(prev_dE + dE) < S.refine_energy_tol) {
      osc++;
      if (osc >= 2 && !prev_wfn.empty()) {
        std::vector<Det> uni;
        std::set_union(prev_wfn.begin(), prev_wfn.end(), wfn.begin(), wfn.end(), std::back_inserter(uni), spin_less);
        std::vector<double> Xu(uni.size(), 0.);
        for (size_t i = 0; i < wfn.size(); ++i) {
          auto it = std::lower_bound(uni.begin(), uni.end(), wfn[i], spin_less);
          if (it != uni.end() && *it == wfn[i]) Xu[it - uni.begin()] = X[i];
        }
        const double Eu = sci_diag(H, S, uni, Xu);
        const int64_t e = std::min<int64_t>(osc, S.max_refine_iter - ext);
        if (e > 0) {
          max_iter += e;
          ext += e;
        }
        wfn = uni;
        X = Xu;
        ndets = (int64_t)wfn.size();
        E0 = Eu;
        prev_wfn.clear();
        osc = 0;
        prev_dE = 0.;
        continue;
      }
    } else {
      osc = 0;
    }
    prev_dE = dE;
    prev_wfn = wfn;
    E0 = E;
  }
  if (!converged) throw std::runtime_error("ASCI Refine did not converge");
  return E0;
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
// a caller's CSR matrix (0-based), as davidson_solver receives it
// (python/src/pybind11/algorithms/davidson_solver.cpp:60-64)
void* orc_csr_from_arrays(int64_t n, const int64_t* rowptr, const int64_t* colind, const double* nzval) {
  Csr* M = new Csr;
  M->n = n;
  M->rowptr.assign(rowptr, rowptr + n + 1);
  M->colind.assign(colind, colind + rowptr[n]);
  M->nzval.assign(nzval, nzval + rowptr[n]);
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

// ASCI driver: settings as a flat double array (order of AsciSettings fields
// below), the initial wavefunction, and the phase ("grow", "refine" or both).
// Returns the number of determinants (<= cap) written to out_a/out_b/out_c,
// or -1 on error (orc_last_error).
}  // extern "C"

// the settings array of oracle.py (_ASCI_ORDER)
static AsciSettings asci_settings_from(const double* set) {
  AsciSettings S;
  S.ntdets_max = (int64_t)set[0];
  S.ntdets_min = (int64_t)set[1];
  S.ncdets_max = (int64_t)set[2];
  S.core_fixed = (int)set[3];
  S.core_threshold = set[4];
  S.h_el_tol = set[5];
  S.rv_prune_tol = set[6];
  S.grow_factor = set[7];
  S.min_grow_factor = set[8];
  S.backoff = set[9];
  S.recovery = set[10];
  S.max_refine_iter = (int64_t)set[11];
  S.refine_energy_tol = set[12];
  S.warm_start = (int)set[13];
  S.min_warm_start_overlap = set[14];
  S.ci_res_tol = set[15];
  S.ci_max_subspace = (int64_t)set[16];
  S.ci_matel_tol = set[17];
  S.taper_grow_factor = set[18];
  S.just_singles = (int)set[19];
  S.grow_with_rot = (int)set[20];
  S.rot_size_start = (int64_t)set[21];
  return S;
}

extern "C" {

int64_t orc_asci(void* h, const double* set, int64_t n0, const uint64_t* a0, const uint64_t* b0, const double* c0,
                 double E0, int do_grow, int do_refine, int64_t cap, uint64_t* out_a, uint64_t* out_b, double* out_c,
                 double* E_out, double* E_grow_out, double* rot_out) {
  const AsciSettings S = asci_settings_from(set);
  int64_t nret = -1;
  guard([&] {
    Ham H = *(Ham*)h;  // the grow's rotation changes this copy, which the refine then uses
    std::vector<Det> wfn(n0);
    std::vector<double> X(c0, c0 + n0);
    for (int64_t i = 0; i < n0; ++i) wfn[i] = {a0[i], b0[i]};
    double E = E0;
    std::vector<double> rot;
    if (do_grow) E = asci_grow(H, S, E, wfn, X, nullptr, &rot);
    if (rot_out)
      for (int j = 0; j < H.n; ++j)
        for (int i = 0; i < H.n; ++i)
          rot_out[i + (size_t)H.n * j] = rot.empty() ? (i == j ? 1. : 0.) : rot[i + (size_t)H.n * j];
    if (E_grow_out) *E_grow_out = E;
    if (do_refine) E = asci_refine(H, S, E, wfn, X);
    *E_out = E;
    nret = (int64_t)wfn.size();
    for (int64_t i = 0; i < std::min(nret, cap); ++i) {
      out_a[i] = wfn[i].a;
      out_b[i] = wfn[i].b;
      out_c[i] = X[i];
    }
  });
  return nret;
}

// asci_grow alone; req (up to cap entries) receives, per asci_iter, the size
// requested and the size reached; returns the number of entries, or -1
int64_t orc_asci_grow_requests(void* h, const double* set, int64_t n0, const uint64_t* a0, const uint64_t* b0,
                               const double* c0, double E0, int64_t cap, int64_t* req) {
  Ham H = *(Ham*)h;
  const AsciSettings S = asci_settings_from(set);
  int64_t nret = -1;
  guard([&] {
    std::vector<Det> wfn(n0);
    std::vector<double> X(c0, c0 + n0);
    for (int64_t i = 0; i < n0; ++i) wfn[i] = {a0[i], b0[i]};
    std::vector<int64_t> steps;
    asci_grow(H, S, E0, wfn, X, &steps);
    nret = (int64_t)steps.size();
    for (int64_t i = 0; i < std::min(nret, cap); ++i) req[i] = steps[i];
  });
  return nret;
}

// one asci_iter (include/macis/asci/iteration.hpp:50-226) towards ndets_max
int64_t orc_asci_iter(void* h, const double* set, int64_t n0, const uint64_t* a0, const uint64_t* b0,
                      const double* c0, double E0, int64_t ndets_max, int64_t cap, uint64_t* out_a, uint64_t* out_b,
                      double* out_c, double* E_out) {
  const Ham& H = *(Ham*)h;
  const AsciSettings S = asci_settings_from(set);
  int64_t nret = -1;
  guard([&] {
    std::vector<Det> wfn(n0);
    std::vector<double> X(c0, c0 + n0);
    for (int64_t i = 0; i < n0; ++i) wfn[i] = {a0[i], b0[i]};
    *E_out = asci_iter(H, S, ndets_max, E0, wfn, X);
    nret = (int64_t)wfn.size();
    for (int64_t i = 0; i < std::min(nret, cap); ++i) {
      out_a[i] = wfn[i].a;
      out_b[i] = wfn[i].b;
      out_c[i] = X[i];
    }
  });
  return nret;
}

// One asci_search call (the selection step alone), for parity of selected sets.
int64_t orc_asci_search(void* h, const double* set, int64_t ncore, const uint64_t* a, const uint64_t* b,
                        const double* c, double E0, int64_t ndets_max, int64_t cap, uint64_t* out_a,
                        uint64_t* out_b) {
  const Ham& H = *(Ham*)h;
  const AsciSettings S = asci_settings_from(set);
  int64_t nret = -1;
  guard([&] {
    std::vector<Det> core(ncore);
    for (int64_t i = 0; i < ncore; ++i) core[i] = {a[i], b[i]};
    std::vector<double> C(c, c + ncore);
    std::vector<Det> out = asci_search(H, S, ndets_max, core, C, E0);
    nret = (int64_t)out.size();
    for (int64_t i = 0; i < std::min(nret, cap); ++i) {
      out_a[i] = out[i].a;
      out_b[i] = out[i].b;
    }
  });
  return nret;
}

// asci_pt2 on a wavefunction (sorted by spin_comparator); 0 on success.
int orc_asci_pt2(void* h, int64_t nd, const uint64_t* a, const uint64_t* b, const double* c, double E0, double tol,
                 int64_t pass_max, double* ept2, int64_t* npt2) {
  const Ham& H = *(Ham*)h;
  return guard([&] {
    std::vector<Det> dets(nd);
    for (int64_t i = 0; i < nd; ++i) dets[i] = {a[i], b[i]};
    std::vector<double> C(c, c + nd);
    *ept2 = asci_pt2(H, dets, C, E0, tol, npt2, pass_max > 0 ? pass_max : (int64_t)1 << 25);
  });
}

// casscf_diis from full integrals; settings as a flat double array in the
// order of McscfSettings; 0 on success
int orc_casscf(const double* set, int nalpha, int nbeta, int norb, int ninact, int nact, double E_core,
               const double* T, const double* V, double* A1, double* A2, double* E, int64_t* iters, int* conv) {
  McscfSettings S;
  S.max_macro_iter = (int64_t)set[0];
  S.max_orbital_step = set[1];
  S.orb_grad_tol = set[2];
  S.enable_diis = (int)set[3];
  S.diis_start_iter = (int64_t)set[4];
  S.diis_nkeep = (int64_t)set[5];
  S.ci_res_tol = set[6];
  S.ci_max_subspace = (int64_t)set[7];
  S.ci_matel_tol = set[8];
  return guard([&] { *E = casscf(S, nalpha, nbeta, norb, ninact, nact, E_core, T, V, A1, A2, iters, conv); });
}

// the fock_matrices.cxx building blocks at one orbital partition: Fi, Fa
// (n^2), Q (na x n), F (n^2), the inactive energy and the energy from F
void orc_mcscf_fock(int n, int ni, int na, const double* T, const double* V, const double* A1, const double* A2,
                    double* Fi, double* Fa, double* Q, double* F, double* E_inact, double* E_fock) {
  inactive_fock(n, ni, T, V, Fi);
  *E_inact = inactive_energy(n, ni, T, Fi);
  if (na > 0) {
    active_fock(n, ni, na, V, A1, Fa);
    aux_q(n, ni, na, V, A2, Q);
    generalized_fock(n, ni, na, Fi, Fa, A1, Q, F);
    *E_fock = energy_from_generalized_fock(n, ni, na, T, A1, F);
  }
}

// orbital entropies of a CI vector; s2 / mi may be null; 0 on success
int orc_entropies(int n, const uint64_t* alpha, const uint64_t* beta, int64_t nd, const double* C, double* s1,
                  double* s2, double* mi) {
  return guard([&] { form_entropies(n, alpha, beta, nd, C, s1, s2, mi); });
}

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
