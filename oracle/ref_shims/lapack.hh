// Stand-in for the subset of LAPACK++ (namespace lapack) that the reference's
// MACIS / lobpcgxx headers call, written for this shim:
//   syev  - symmetric eigensolver: cyclic Jacobi rotations (eigenvalues
//           ascending, orthonormal eigenvectors in the columns of A);
//   potrf - Cholesky (lower), returns the LAPACK info convention;
//   lacpy - general matrix copy;
//   gesvd, gelss - declared only (the fixtures never call them);
//   gelqf / ormlq - Householder LQ factorisation and Q^T applied from the
//           right, with LAPACK's reflector convention (H = I - tau v v^T,
//           v(i) = 1, beta = -sign(alpha) ||x||).
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <numeric>
#include <stdexcept>
#include <vector>

#include "blas.hh"

namespace lapack {
using blas::Op;
using blas::Side;
using blas::Uplo;
enum class Job : char { NoVec = 'N', Vec = 'V', UpdateVec = 'U', AllVec = 'A', SomeVec = 'S', OverwriteVec = 'O' };
enum class MatrixType : char { General = 'G', Lower = 'L', Upper = 'U' };

template <typename T>
void lacpy(MatrixType type, int64_t m, int64_t n, const T* A, int64_t lda, T* B, int64_t ldb) {
  for (int64_t j = 0; j < n; ++j)
    for (int64_t i = 0; i < m; ++i) {
      if (type == MatrixType::Lower && i < j) continue;
      if (type == MatrixType::Upper && i > j) continue;
      B[i + j * ldb] = A[i + j * lda];
    }
}

template <typename T>
int64_t syev(Job jobz, Uplo uplo, int64_t n, T* A, int64_t lda, T* W) {
  // full symmetric copy from the referenced triangle
  std::vector<T> a((size_t)n * n), v((size_t)n * n, T(0));
  for (int64_t j = 0; j < n; ++j)
    for (int64_t i = 0; i < n; ++i) {
      const int64_t hi = std::max(i, j), lo = std::min(i, j);
      a[i + j * n] = uplo == Uplo::Upper ? A[lo + hi * lda] : A[hi + lo * lda];
    }
  for (int64_t i = 0; i < n; ++i) v[i + i * n] = T(1);
  for (int sweep = 0; sweep < 100; ++sweep) {
    T off = 0, tot = 0;
    for (int64_t j = 0; j < n; ++j)
      for (int64_t i = 0; i < n; ++i) {
        tot += a[i + j * n] * a[i + j * n];
        if (i != j) off += a[i + j * n] * a[i + j * n];
      }
    if (off <= tot * 1e-34 || off == T(0)) break;
    for (int64_t p = 0; p < n - 1; ++p)
      for (int64_t q = p + 1; q < n; ++q) {
        const T apq = a[p + q * n];
        if (apq == T(0)) continue;
        const T app = a[p + p * n], aqq = a[q + q * n];
        const T theta = (aqq - app) / (2 * apq);
        const T t = (theta >= 0 ? T(1) : T(-1)) / (std::abs(theta) + std::sqrt(theta * theta + 1));
        const T c = 1 / std::sqrt(t * t + 1), s = t * c;
        for (int64_t k = 0; k < n; ++k) {  // columns p, q
          const T akp = a[k + p * n], akq = a[k + q * n];
          a[k + p * n] = c * akp - s * akq;
          a[k + q * n] = s * akp + c * akq;
        }
        for (int64_t k = 0; k < n; ++k) {  // rows p, q
          const T apk = a[p + k * n], aqk = a[q + k * n];
          a[p + k * n] = c * apk - s * aqk;
          a[q + k * n] = s * apk + c * aqk;
        }
        for (int64_t k = 0; k < n; ++k) {
          const T vkp = v[k + p * n], vkq = v[k + q * n];
          v[k + p * n] = c * vkp - s * vkq;
          v[k + q * n] = s * vkp + c * vkq;
        }
      }
  }
  std::vector<int64_t> ord(n);
  std::iota(ord.begin(), ord.end(), 0);
  std::stable_sort(ord.begin(), ord.end(), [&](int64_t x, int64_t y) { return a[x + x * n] < a[y + y * n]; });
  for (int64_t j = 0; j < n; ++j) {
    W[j] = a[ord[j] + ord[j] * n];
    if (jobz == Job::Vec)
      for (int64_t i = 0; i < n; ++i) A[i + j * lda] = v[i + ord[j] * n];
  }
  return 0;
}

template <typename T>
int64_t potrf(Uplo uplo, int64_t n, T* A, int64_t lda) {
  if (uplo != Uplo::Lower) throw std::runtime_error("lapack shim: potrf upper not provided");
  for (int64_t j = 0; j < n; ++j) {
    T d = A[j + j * lda];
    for (int64_t p = 0; p < j; ++p) d -= A[j + p * lda] * A[j + p * lda];
    if (!(d > T(0))) return j + 1;
    d = std::sqrt(d);
    A[j + j * lda] = d;
    for (int64_t i = j + 1; i < n; ++i) {
      T s = A[i + j * lda];
      for (int64_t p = 0; p < j; ++p) s -= A[i + p * lda] * A[j + p * lda];
      A[i + j * lda] = s / d;
    }
  }
  return 0;
}

// A (m x n, m <= n) = L Q; reflector i stored in A(i, i+1:n), tau[i].
template <typename T>
int64_t gelqf(int64_t m, int64_t n, T* A, int64_t lda, T* tau) {
  const int64_t k = std::min(m, n);
  for (int64_t i = 0; i < k; ++i) {
    T alpha = A[i + i * lda];
    T xn = 0;
    for (int64_t j = i + 1; j < n; ++j) xn += A[i + j * lda] * A[i + j * lda];
    if (xn == T(0)) {
      tau[i] = 0;
      continue;
    }
    const T beta = -std::copysign(std::sqrt(alpha * alpha + xn), alpha);
    tau[i] = (beta - alpha) / beta;
    const T scale = 1 / (alpha - beta);
    for (int64_t j = i + 1; j < n; ++j) A[i + j * lda] *= scale;
    A[i + i * lda] = beta;
    // rows below: A(r, i:n) <- A(r, i:n) (I - tau v v^T), v = (1, A(i, i+1:n))
    for (int64_t r = i + 1; r < m; ++r) {
      T w = A[r + i * lda];
      for (int64_t j = i + 1; j < n; ++j) w += A[r + j * lda] * A[i + j * lda];
      w *= tau[i];
      A[r + i * lda] -= w;
      for (int64_t j = i + 1; j < n; ++j) A[r + j * lda] -= w * A[i + j * lda];
    }
  }
  return 0;
}

// C (m x n) <- C op(Q) with Q = H(k-1) ... H(0) from gelqf; only the
// Side::Right forms are provided.
template <typename T>
int64_t ormlq(Side side, Op trans, int64_t m, int64_t n, int64_t k, const T* A, int64_t lda, const T* tau, T* C,
              int64_t ldc) {
  if (side != Side::Right) throw std::runtime_error("lapack shim: ormlq left not provided");
  auto apply = [&](int64_t i) {  // C <- C H(i)
    for (int64_t r = 0; r < m; ++r) {
      T w = C[r + i * ldc];
      for (int64_t j = i + 1; j < n; ++j) w += C[r + j * ldc] * A[i + j * lda];
      w *= tau[i];
      C[r + i * ldc] -= w;
      for (int64_t j = i + 1; j < n; ++j) C[r + j * ldc] -= w * A[i + j * lda];
    }
  };
  if (trans == Op::NoTrans)  // C Q = C H(k-1) ... H(0)
    for (int64_t i = k - 1; i >= 0; --i) apply(i);
  else  // C Q^T = C H(0) ... H(k-1)
    for (int64_t i = 0; i < k; ++i) apply(i);
  return 0;
}
// Present so that the reference's orbital-rotation helper compiles; the
// fixtures never rotate orbitals, and calling it is an error.
template <typename T, typename... Rest>
int64_t gesvd(Job, Job, int64_t, int64_t, T*, int64_t, Rest&&...) {
  throw std::runtime_error("lapack shim: gesvd not provided");
}
template <typename T>
int64_t gelss(int64_t, int64_t, int64_t, T*, int64_t, T*, int64_t, T*, T, int64_t*) {
  throw std::runtime_error("lapack shim: gelss not provided");
}
}  // namespace lapack
