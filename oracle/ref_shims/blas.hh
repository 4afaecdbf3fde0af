// Stand-in for the subset of BLAS++ (namespace blas) that the reference's
// MACIS / lobpcgxx headers call, written as plain OpenMP loops for this shim:
// gemm, nrm2, dot, scal, axpy, copy, swap, iamax and the one trsm form that
// lobpcgxx's CholQR uses.  Column-major semantics as in reference BLAS.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <stdexcept>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace blas {
enum class Layout : char { ColMajor = 'C', RowMajor = 'R' };
enum class Op : char { NoTrans = 'N', Trans = 'T', ConjTrans = 'C' };
enum class Uplo : char { Upper = 'U', Lower = 'L', General = 'G' };
enum class Diag : char { NonUnit = 'N', Unit = 'U' };
enum class Side : char { Left = 'L', Right = 'R' };

namespace shim_detail {
inline int nthreads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
inline int thread_id() {
#ifdef _OPENMP
  return omp_get_thread_num();
#else
  return 0;
#endif
}

// C(m x n) = alpha * op(A) * op(B) + beta * C, column major.
template <typename T>
void gemm_cm(Op ta, Op tb, int64_t m, int64_t n, int64_t k, T alpha, const T* A, int64_t lda, const T* B,
             int64_t ldb, T beta, T* C, int64_t ldc) {
  const bool at = ta != Op::NoTrans, bt = tb != Op::NoTrans;
  auto bval = [&](int64_t p, int64_t j) { return bt ? B[j + p * ldb] : B[p + j * ldb]; };
  // scale C first (beta == 0 overwrites, as reference BLAS does)
#pragma omp parallel for schedule(static) if (m * n > 4096)
  for (int64_t j = 0; j < n; ++j)
    for (int64_t i = 0; i < m; ++i) C[i + j * ldc] = beta == T(0) ? T(0) : beta * C[i + j * ldc];
  if (k == 0 || alpha == T(0)) return;

  if (at && m * n <= 1 << 16 && k >= 4096) {
    // long inner dimension with op(A) = A^T (Gram-type products V^T W):
    // split k over threads, per-thread m x n partial sums, reduced in order
    const int nt = nthreads();
    std::vector<T> part((size_t)nt * m * n, T(0));
#pragma omp parallel
    {
      const int t = thread_id();
      const int64_t chunk = (k + nt - 1) / nt;
      const int64_t p0 = std::min<int64_t>(k, t * chunk), p1 = std::min<int64_t>(k, p0 + chunk);
      T* acc = part.data() + (size_t)t * m * n;
      constexpr int64_t tile = 256;
      for (int64_t q0 = p0; q0 < p1; q0 += tile) {
        const int64_t q1 = std::min(p1, q0 + tile);
        for (int64_t j = 0; j < n; ++j)
          for (int64_t i = 0; i < m; ++i) {
            const T* a = A + i * lda;
            T s = T(0);
            if (!bt) {
              const T* b = B + j * ldb;
              for (int64_t p = q0; p < q1; ++p) s += a[p] * b[p];
            } else {
              for (int64_t p = q0; p < q1; ++p) s += a[p] * B[j + p * ldb];
            }
            acc[i + j * m] += s;
          }
      }
    }
    for (int t = 0; t < nt; ++t)
      for (int64_t j = 0; j < n; ++j)
        for (int64_t i = 0; i < m; ++i) C[i + j * ldc] += alpha * part[(size_t)t * m * n + i + j * m];
    return;
  }
  if (!at) {
    // axpy form: column of C += A(:,p) * op(B)(p,j); rows split over threads
#pragma omp parallel for schedule(static) if (m * n * k > 1 << 16)
    for (int64_t i0 = 0; i0 < m; i0 += 512) {
      const int64_t i1 = std::min(m, i0 + 512);
      for (int64_t j = 0; j < n; ++j)
        for (int64_t p = 0; p < k; ++p) {
          const T bp = alpha * bval(p, j);
          const T* a = A + p * lda;
          T* c = C + j * ldc;
          for (int64_t i = i0; i < i1; ++i) c[i] += a[i] * bp;
        }
    }
    return;
  }
  // dot form: C(i,j) += A(:,i) . op(B)(:,j)
#pragma omp parallel for collapse(2) schedule(static) if (m * n * k > 1 << 16)
  for (int64_t j = 0; j < n; ++j)
    for (int64_t i = 0; i < m; ++i) {
      const T* a = A + i * lda;
      T s = T(0);
      for (int64_t p = 0; p < k; ++p) s += a[p] * bval(p, j);
      C[i + j * ldc] += alpha * s;
    }
}
}  // namespace shim_detail

template <typename T>
void gemm(Layout layout, Op ta, Op tb, int64_t m, int64_t n, int64_t k, T alpha, const T* A, int64_t lda,
          const T* B, int64_t ldb, T beta, T* C, int64_t ldc) {
  if (layout == Layout::ColMajor)
    shim_detail::gemm_cm(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
  else  // row major C = op(A) op(B)  <=>  column major C^T = op(B)^T op(A)^T
    shim_detail::gemm_cm(tb, ta, n, m, k, alpha, B, ldb, A, lda, beta, C, ldc);
}

template <typename T>
T nrm2(int64_t n, const T* x, int64_t incx) {
  T s = T(0);
#pragma omp parallel for reduction(+ : s) schedule(static) if (n > 1 << 15)
  for (int64_t i = 0; i < n; ++i) s += x[i * incx] * x[i * incx];
  return std::sqrt(s);
}
template <typename T>
T dot(int64_t n, const T* x, int64_t incx, const T* y, int64_t incy) {
  T s = T(0);
#pragma omp parallel for reduction(+ : s) schedule(static) if (n > 1 << 15)
  for (int64_t i = 0; i < n; ++i) s += x[i * incx] * y[i * incy];
  return s;
}
template <typename T>
void scal(int64_t n, T a, T* x, int64_t incx) {
#pragma omp parallel for schedule(static) if (n > 1 << 15)
  for (int64_t i = 0; i < n; ++i) x[i * incx] *= a;
}
template <typename T>
void axpy(int64_t n, T a, const T* x, int64_t incx, T* y, int64_t incy) {
#pragma omp parallel for schedule(static) if (n > 1 << 15)
  for (int64_t i = 0; i < n; ++i) y[i * incy] += a * x[i * incx];
}
template <typename T>
void copy(int64_t n, const T* x, int64_t incx, T* y, int64_t incy) {
  for (int64_t i = 0; i < n; ++i) y[i * incy] = x[i * incx];
}
template <typename T>
void swap(int64_t n, T* x, int64_t incx, T* y, int64_t incy) {
  for (int64_t i = 0; i < n; ++i) std::swap(x[i * incx], y[i * incy]);
}
template <typename T>
int64_t iamax(int64_t n, const T* x, int64_t incx) {
  int64_t best = 0;
  for (int64_t i = 1; i < n; ++i)
    if (std::abs(x[i * incx]) > std::abs(x[best * incx])) best = i;
  return best;
}

// Only the form lobpcgxx's CholQR calls: X op(L) = alpha B with L lower
// triangular on the right, op = transpose, i.e. X = alpha B L^{-T} row by row.
template <typename T>
void trsm(Layout layout, Side side, Uplo uplo, Op op, Diag diag, int64_t m, int64_t n, T alpha, const T* A,
          int64_t lda, T* B, int64_t ldb) {
  if (layout != Layout::ColMajor || side != Side::Right || uplo != Uplo::Lower || op == Op::NoTrans)
    throw std::runtime_error("blas shim: trsm form not provided");
#pragma omp parallel for schedule(static) if (m > 4096)
  for (int64_t r = 0; r < m; ++r) {
    for (int64_t j = 0; j < n; ++j) {
      T s = alpha * B[r + j * ldb];
      for (int64_t p = 0; p < j; ++p) s -= B[r + p * ldb] * A[j + p * lda];
      B[r + j * ldb] = diag == Diag::Unit ? s : s / A[j + j * lda];
    }
  }
}
}  // namespace blas
