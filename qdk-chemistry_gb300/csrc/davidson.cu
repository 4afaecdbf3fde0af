// Davidson eigensolver on the device (replaces macis::davidson,
// include/macis/solvers/davidson.hpp:259-372, with gram_schmidt :185-238 and
// lobpcgxx::rayleigh_ritz, lobpcgxx/rayleigh_ritz.hpp:70-77).
//
// Everything except the convergence test runs on the GPU in FP64: the
// subspace V and A*V (column-major, N x (max_m+1)), the projected matrix, its
// lowest eigenpair (one-CTA Householder tridiagonalisation + Sturm
// multisection + inverse iteration), the Ritz vector and
// residual, the diagonal preconditioner and classical Gram-Schmidt applied
// twice.  The host reads two scalars per iteration (residual norm, Ritz
// value) to decide convergence.
//
// Mixed precision (QDKGB_PREC_MIXED): new subspace directions are multiplied
// by H in FP32 (FP32 values, x, y and accumulation; half the bytes of the
// FP64 sigma).  Whenever the estimated residual has dropped by a factor
// `refresh_ratio` since the last full-precision check, or stagnates, the Ritz
// vector's sigma is recomputed in full precision (hi+lo values, FP64
// accumulation) and the subspace is thick-restarted on the lowest Ritz
// vectors with that exact column in front (defect correction).  Convergence
// is declared only on the full-precision residual, so the stopping rule is
// the same as the FP64 path's.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "internal.h"
#include "dfloat.cuh"
#include "small_eig.cuh"

namespace qdkgb {

constexpr int kMaxSubspace = 256;
// Row-parallel vector kernels: 256 threads, two rows per thread per step
// (rows i and i + 256 of a 512-row tile), grids of kVecBlocksPerSm blocks per
// SM striding over the tiles.  Every row sum runs over the columns in order,
// so a row's value does not depend on the launch shape.
constexpr int kVecThreads = 256;
constexpr int kVecTile = 2 * kVecThreads;
constexpr int kVecBlocksPerSm = 4;
constexpr int kDotCols = 8;  // columns per block of k_multidot (one per warp in its final sum)
constexpr int kDotChunks = (kMaxSubspace + 2 + kDotCols - 1) / kDotCols;

// Sum of v over the block, valid in thread 0 (red: kVecThreads/32 doubles).
__device__ __forceinline__ double block_sum_vec(double v, double* red) {
  v = warp_sum(v);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.;
  if (threadIdx.x < 32) {
    t = (threadIdx.x < (kVecThreads >> 5)) ? red[threadIdx.x] : 0.;
    t = warp_sum(t);
  }
  return t;
}

// Called by every thread after this block stored its partial sums: true in
// the block that finished last (count[slot] is then reset for the next
// launch).  Its reads of the other blocks' partials go through L2 (__ldcg).
__device__ __forceinline__ bool last_block_done(unsigned* count, int slot, unsigned nblocks) {
  __shared__ bool last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    last = atomicAdd(count + slot, 1u) == nblocks - 1;
    if (last) count[slot] = 0u;
  }
  __syncthreads();
  if (last) __threadfence();
  return last;
}

// out[j * out_stride] = A[:, j] . w for j < k.  Block (x, y) takes columns
// y*kDotCols .. +kDotCols over a grid-stride share of the rows, so w is read
// once per column block; partial sums go to partial[j * gridDim.x + x] and the
// block of column block y that finishes last adds them in block order (the
// result does not depend on the order in which blocks run).  self_out, when
// given, receives w . w as well (partial row k); a non-zero *skip makes the
// launch a no-op.
__global__ void __launch_bounds__(kVecThreads)
    k_multidot(const double* __restrict__ A, int64_t lda, int k, const double* __restrict__ w, int64_t n,
               double* __restrict__ partial, unsigned* __restrict__ count, double* __restrict__ out, int out_stride,
               double* __restrict__ self_out, const double* __restrict__ skip) {
  if (skip && *skip != 0.) return;
  __shared__ double red[kVecThreads / 32][kDotCols + 1];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int j0 = blockIdx.y * kDotCols;
  const int nc = min(kDotCols, k - j0);
  const double* a = A + (size_t)j0 * lda;
  const bool self = self_out && blockIdx.y == 0;
  double acc[kDotCols];
#pragma unroll
  for (int c = 0; c < kDotCols; ++c) acc[c] = 0.;
  double accw = 0.;
  const int64_t step = (int64_t)gridDim.x * kVecTile;
  for (int64_t i = (int64_t)blockIdx.x * kVecTile + threadIdx.x; i < n; i += step) {
    const int64_t i1 = i + kVecThreads;
    const bool has1 = i1 < n;
    const double w0 = w[i], w1 = has1 ? w[i1] : 0.;
    if (self) accw = fma(w1, w1, fma(w0, w0, accw));
#pragma unroll
    for (int c = 0; c < kDotCols; ++c) {
      if (c < nc) {
        const double a0 = a[i + (size_t)c * lda];
        const double a1 = has1 ? a[i1 + (size_t)c * lda] : 0.;
        acc[c] = fma(a0, w0, acc[c]);
        acc[c] = fma(a1, w1, acc[c]);
      }
    }
  }
#pragma unroll
  for (int c = 0; c < kDotCols; ++c) {
    if (c < nc) {
      const double t = warp_sum(acc[c]);
      if (lane == 0) red[wid][c] = t;
    }
  }
  if (self) {
    const double t = warp_sum(accw);
    if (lane == 0) red[wid][kDotCols] = t;
  }
  __syncthreads();
  if (threadIdx.x < nc) {
    double t = 0.;
    for (int q = 0; q < kVecThreads / 32; ++q) t += red[q][threadIdx.x];
    partial[(size_t)(j0 + threadIdx.x) * gridDim.x + blockIdx.x] = t;
  }
  if (self && threadIdx.x == kDotCols) {
    double t = 0.;
    for (int q = 0; q < kVecThreads / 32; ++q) t += red[q][kDotCols];
    partial[(size_t)k * gridDim.x + blockIdx.x] = t;
  }
  if (!last_block_done(count, blockIdx.y, gridDim.x)) return;
  if (wid < nc) {
    const double* p = partial + (size_t)(j0 + wid) * gridDim.x;
    double t = 0.;
    for (int b = lane; b < (int)gridDim.x; b += 32) t += __ldcg(p + b);
    t = warp_sum(t);
    if (lane == 0) out[(size_t)(j0 + wid) * out_stride] = t;
  }
  if (self && wid == kVecThreads / 32 - 1) {
    const double* p = partial + (size_t)k * gridDim.x;
    double t = 0.;
    for (int b = lane; b < (int)gridDim.x; b += 32) t += __ldcg(p + b);
    t = warp_sum(t);
    if (lane == 0) *self_out = t;
  }
}
// out[j * out_stride] = sum_b partial[j * nb + b], fixed order; one warp per j
__global__ void k_reduce_partials(const double* __restrict__ partial, int nb, int k, double* out, int out_stride) {
  const int j = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (j >= k) return;
  double s = 0.;
  for (int b = lane; b < nb; b += 32) s += partial[(size_t)j * nb + b];
  s = warp_sum(s);
  if (lane == 0) out[(size_t)j * out_stride] = s;
}
// y = A[:, 0:k] coef (SUB: y -= A[:, 0:k] coef), coef strided; each row sums
// over j in order, four columns' loads in flight per row.  A non-zero *skip
// makes the launch a no-op.  skip_out, when given, receives the selective
// reorthogonalisation test of a Gram-Schmidt pass (coef = V^T y for
// orthonormal V, *w2 = |y|^2 before it): 1 when |y - V coef|^2 = *w2 - |coef|^2
// keeps at least half of *w2 (a second pass is not needed), else 0.
template <bool SUB>
__global__ void __launch_bounds__(kVecThreads)
    k_gemv_rows(const double* __restrict__ A, int64_t lda, int k, const double* __restrict__ coef, int coef_stride,
                double* __restrict__ y, int64_t n, const double* __restrict__ skip = nullptr,
                const double* __restrict__ w2 = nullptr, double* __restrict__ skip_out = nullptr) {
  if (skip && *skip != 0.) return;
  __shared__ double c[kMaxSubspace + 2];
  for (int j = threadIdx.x; j < k; j += blockDim.x) c[j] = coef[(size_t)j * coef_stride];
  __syncthreads();
  if (skip_out && blockIdx.x == 0 && threadIdx.x == 0) {
    double cc = 0.;
    for (int j = 0; j < k; ++j) cc += c[j] * c[j];
    *skip_out = (*w2 - cc >= 0.5 * *w2) ? 1. : 0.;
  }
  const int64_t step = (int64_t)gridDim.x * kVecTile;
  for (int64_t i = (int64_t)blockIdx.x * kVecTile + threadIdx.x; i < n; i += step) {
    const int64_t i1 = i + kVecThreads;
    const bool has1 = i1 < n;
    double s0 = 0., s1 = 0.;
    int j = 0;
    for (; j + 4 <= k; j += 4) {
      double a0[4], a1[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        a0[q] = A[i + (size_t)(j + q) * lda];
        a1[q] = has1 ? A[i1 + (size_t)(j + q) * lda] : 0.;
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        s0 = fma(a0[q], c[j + q], s0);
        s1 = fma(a1[q], c[j + q], s1);
      }
    }
    for (; j < k; ++j) {
      s0 = fma(A[i + (size_t)j * lda], c[j], s0);
      if (has1) s1 = fma(A[i1 + (size_t)j * lda], c[j], s1);
    }
    if (SUB) {
      y[i] -= s0;
      if (has1) y[i1] -= s1;
    } else {
      y[i] = s0;
      if (has1) y[i1] = s1;
    }
  }
}
// Y[:, o] = A[:, 0:k] Q[:, o] for o < nout <= kMaxOut (Q column-major, ld k):
// the thick restart's new basis in one pass over A; each output's row sum runs
// over j in order (the same value as k_gemv_rows on that column of Q).
constexpr int kMaxOut = 8;
__global__ void __launch_bounds__(kVecThreads)
    k_gemv_multi(const double* __restrict__ A, int64_t lda, int k, const double* __restrict__ Q, int nout,
                 double* __restrict__ Y, int64_t ldy, int64_t n) {
  __shared__ double q[kMaxSubspace + 2][kMaxOut];
  for (int t = threadIdx.x; t < k * kMaxOut; t += blockDim.x) {
    const int j = t / kMaxOut, o = t % kMaxOut;
    q[j][o] = o < nout ? Q[(size_t)o * k + j] : 0.;
  }
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * kVecThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kVecThreads) {
    double acc[kMaxOut];
#pragma unroll
    for (int o = 0; o < kMaxOut; ++o) acc[o] = 0.;
    int j = 0;
    for (; j + 4 <= k; j += 4) {
      double a[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) a[u] = A[i + (size_t)(j + u) * lda];
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int o = 0; o < kMaxOut; ++o)
          if (o < nout) acc[o] = fma(a[u], q[j + u][o], acc[o]);
    }
    for (; j < k; ++j) {
      const double a = A[i + (size_t)j * lda];
#pragma unroll
      for (int o = 0; o < kMaxOut; ++o)
        if (o < nout) acc[o] = fma(a, q[j][o], acc[o]);
    }
#pragma unroll
    for (int o = 0; o < kMaxOut; ++o)
      if (o < nout) Y[i + (size_t)o * ldy] = acc[o];
  }
}
// w *= 1/sqrt(*nrm2) when sqrt(*nrm2) > min_norm, else raise *flag
__global__ void k_normalize(double* w, int64_t n, const double* nrm2, double min_norm, double* flag) {
  const double nrm = sqrt(*nrm2);
  if (!(nrm > min_norm)) {
    if (flag && blockIdx.x == 0 && threadIdx.x == 0) *flag = 1.;
    return;
  }
  const double sc = 1. / nrm;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    w[i] *= sc;
}
// diagonal preconditioner of one element: -r / (D - lam0) with |D - lam0|
// clamped to min_abs (davidson.hpp:352-361)
__device__ __forceinline__ double precondition_one(double r, double d, double min_abs) {
  if (fabs(d) < min_abs) d = (d >= 0) ? min_abs : -min_abs;
  return -r / d;
}
// X = V C0, R = AV C0 - lam0 X, *out = |R|^2 (partial sums per block, the
// last block adds them in block order).  With D, R is stored preconditioned
// (the residual itself is not needed again once its norm is known).
__global__ void __launch_bounds__(kVecThreads)
    k_ritz_residual(const double* __restrict__ V, const double* __restrict__ AV, int64_t ld, int k,
                    const double* __restrict__ C0, const double* __restrict__ lam, double* __restrict__ X,
                    double* __restrict__ R, int64_t n, const double* __restrict__ D, double min_abs,
                    double* __restrict__ partial, unsigned* __restrict__ count, double* __restrict__ out) {
  __shared__ double c[kMaxSubspace + 2];
  __shared__ double red[kVecThreads / 32];
  for (int j = threadIdx.x; j < k; j += blockDim.x) c[j] = C0[j];
  __syncthreads();
  const double l0 = lam[0];
  double s2 = 0.;
  const int64_t step = (int64_t)gridDim.x * kVecTile;
  for (int64_t i = (int64_t)blockIdx.x * kVecTile + threadIdx.x; i < n; i += step) {
    const int64_t i1 = i + kVecThreads;
    const bool has1 = i1 < n;
    double x0 = 0., ax0 = 0., x1 = 0., ax1 = 0.;
    int j = 0;
    for (; j + 4 <= k; j += 4) {
      double v0[4], v1[4], w0[4], w1[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const size_t o = (size_t)(j + q) * ld;
        v0[q] = V[i + o];
        w0[q] = AV[i + o];
        v1[q] = has1 ? V[i1 + o] : 0.;
        w1[q] = has1 ? AV[i1 + o] : 0.;
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        x0 = fma(v0[q], c[j + q], x0);
        ax0 = fma(w0[q], c[j + q], ax0);
        x1 = fma(v1[q], c[j + q], x1);
        ax1 = fma(w1[q], c[j + q], ax1);
      }
    }
    for (; j < k; ++j) {
      const size_t o = (size_t)j * ld;
      x0 = fma(V[i + o], c[j], x0);
      ax0 = fma(AV[i + o], c[j], ax0);
      if (has1) {
        x1 = fma(V[i1 + o], c[j], x1);
        ax1 = fma(AV[i1 + o], c[j], ax1);
      }
    }
    const double r0 = ax0 - l0 * x0;
    X[i] = x0;
    R[i] = D ? precondition_one(r0, D[i] - l0, min_abs) : r0;
    s2 += r0 * r0;
    if (has1) {
      const double r1 = ax1 - l0 * x1;
      X[i1] = x1;
      R[i1] = D ? precondition_one(r1, D[i1] - l0, min_abs) : r1;
      s2 += r1 * r1;
    }
  }
  const double t = block_sum_vec(s2, red);
  if (threadIdx.x == 0) partial[blockIdx.x] = t;
  if (!last_block_done(count, kDotChunks, gridDim.x)) return;
  double u = 0.;
  for (int b = threadIdx.x; b < (int)gridDim.x; b += kVecThreads) u += __ldcg(partial + b);
  __syncthreads();
  u = block_sum_vec(u, red);
  if (threadIdx.x == 0) *out = u;
}
// R = -R / (D - lam0) with |D - lam0| clamped to min_abs (davidson.hpp:352-361)
__global__ void k_precondition(double* R, const double* __restrict__ D, const double* lam, int64_t n,
                               double min_abs) {
  const double l0 = lam[0];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    R[i] = precondition_one(R[i], D[i] - l0, min_abs);
}
// r = s - e x, partial sums of r^2 (e = *eptr)
__global__ void k_axpy_residual(const double* __restrict__ s, const double* __restrict__ x, const double* eptr,
                                double* __restrict__ r, int64_t n, double* __restrict__ partial) {
  __shared__ double red[32];
  const double e = *eptr;
  double s2 = 0.;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double v = s[i] - e * x[i];
    r[i] = v;
    s2 += v * v;
  }
  s2 = warp_sum(s2);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s2;
  __syncthreads();
  if (threadIdx.x < 32) {
    double t = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.;
    t = warp_sum(t);
    if (threadIdx.x == 0) partial[blockIdx.x] = t;
  }
}
// index of the first minimum of D (diagonal_guess, davidson.hpp:106-113); one block
__global__ void k_argmin(const double* D, int64_t n, int64_t* out) {
  __shared__ double sv[1024];
  __shared__ int64_t si[1024];
  double best = INFINITY;
  int64_t bi = n;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    const double v = D[i];
    if (v < best) {
      best = v;
      bi = i;
    }
  }
  sv[threadIdx.x] = best;
  si[threadIdx.x] = bi;
  __syncthreads();
  for (int s = blockDim.x >> 1; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      const double v = sv[threadIdx.x + s];
      const int64_t j = si[threadIdx.x + s];
      if (v < sv[threadIdx.x] || (v == sv[threadIdx.x] && j < si[threadIdx.x])) {
        sv[threadIdx.x] = v;
        si[threadIdx.x] = j;
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = si[0] < n ? si[0] : 0;
}
__global__ void k_set_onehot(double* x, int64_t n, const int64_t* idx) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    x[i] = (i == *idx) ? 1. : 0.;
}
__global__ void k_set_value(double* p, double v) { *p = v; }
// x <- (x + s x^T) / 2 for x viewed as an n x n matrix (coefficients C[Ia, Ib]
// of a product space whose alpha and beta string lists coincide): projection
// on the spin-flip sector of parity s.  Block (J, I), I <= J, owns the 32 x 32
// tile pair P = x[I-tile, J-tile] and Q = x[J-tile, I-tile] (one tile when
// I == J), staged in shared memory so both are read and written row-wise.
constexpr int kFlipTile = 32;
__global__ void __launch_bounds__(kFlipTile * 8) k_flip_project(double* x, int64_t n, double s) {
  const int I = blockIdx.y, J = blockIdx.x;
  if (I > J) return;
  __shared__ double P[kFlipTile][kFlipTile + 1], Q[kFlipTile][kFlipTile + 1];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int64_t r0 = (int64_t)I * kFlipTile, c0 = (int64_t)J * kFlipTile;
  for (int r = ty; r < kFlipTile; r += 8) {
    const int64_t pr = r0 + r, pc = c0 + tx, qr = c0 + r, qc = r0 + tx;
    P[r][tx] = (pr < n && pc < n) ? x[pr * n + pc] : 0.;
    Q[r][tx] = (qr < n && qc < n) ? x[qr * n + qc] : 0.;
  }
  __syncthreads();
  for (int r = ty; r < kFlipTile; r += 8) {
    const int64_t pr = r0 + r, pc = c0 + tx, qr = c0 + r, qc = r0 + tx;
    if (I < J) {
      // element (pr, pc) has pr < pc: avg of it and its mirror Q[tx][r]
      if (pr < n && pc < n) x[pr * n + pc] = 0.5 * (P[r][tx] + s * Q[tx][r]);
      // element (qr, qc) = mirror of P[tx][r]: s * avg
      if (qr < n && qc < n) x[qr * n + qc] = s * (0.5 * (P[tx][r] + s * Q[r][tx]));
    } else if (pr < n && pc < n) {
      double v;
      if (r < tx)
        v = 0.5 * (P[r][tx] + s * P[tx][r]);
      else if (r > tx)
        v = s * (0.5 * (P[tx][r] + s * P[r][tx]));
      else
        v = s < 0 ? 0. : P[r][tx];
      x[pr * n + pc] = v;
    }
  }
}
// Hk(i, c) = Hk(c, i) = v[c], c <= i
__global__ void k_store_row(const double* v, int i, double* Hk, int ld) {
  for (int c = threadIdx.x; c <= i; c += blockDim.x) {
    Hk[i + (size_t)c * ld] = v[c];
    Hk[c + (size_t)i * ld] = v[c];
  }
}

// ---------------------------------------------------------------- double-float subspace
// The mixed-precision solver keeps V, A V, the Ritz vector and the new
// directions as double-float pairs (dfloat.cuh): the same bytes as FP64 but
// FP32-pipe arithmetic.  Each kernel mirrors its FP64 counterpart above (the
// same launch shapes, row split and fixed reduction order); per-block
// partial sums leave the block as doubles.

// out[j * out_stride] = A[:, j] . w for j < k (k_multidot in double-float)
__global__ void __launch_bounds__(kVecThreads)
    k_df_multidot(const float2* __restrict__ A, int64_t lda, int k, const float2* __restrict__ w, int64_t n,
                  double* __restrict__ partial, unsigned* __restrict__ count, double* __restrict__ out, int out_stride,
                  double* __restrict__ self_out, const double* __restrict__ skip) {
  if (skip && *skip != 0.) return;
  __shared__ double red[kVecThreads / 32][kDotCols + 1];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int j0 = blockIdx.y * kDotCols;
  const int nc = min(kDotCols, k - j0);
  const float2* a = A + (size_t)j0 * lda;
  const bool self = self_out && blockIdx.y == 0;
  float2 acc[kDotCols];
#pragma unroll
  for (int c = 0; c < kDotCols; ++c) acc[c] = make_float2(0.f, 0.f);
  float2 accw = make_float2(0.f, 0.f);
  const float2 zero = make_float2(0.f, 0.f);
  const int64_t step = (int64_t)gridDim.x * kVecTile;
  for (int64_t i = (int64_t)blockIdx.x * kVecTile + threadIdx.x; i < n; i += step) {
    const int64_t i1 = i + kVecThreads;
    const bool has1 = i1 < n;
    const float2 w0 = w[i], w1 = has1 ? w[i1] : zero;
    float2 a0[kDotCols], a1[kDotCols];
#pragma unroll
    for (int c = 0; c < kDotCols; ++c) {
      a0[c] = c < nc ? a[i + (size_t)c * lda] : zero;
      a1[c] = (c < nc && has1) ? a[i1 + (size_t)c * lda] : zero;
    }
    if (self) {
      df::mac(accw, w0, w0);
      df::mac(accw, w1, w1);
    }
#pragma unroll
    for (int c = 0; c < kDotCols; ++c) {
      if (c < nc) {
        df::mac(acc[c], a0[c], w0);
        df::mac(acc[c], a1[c], w1);
      }
    }
  }
#pragma unroll
  for (int c = 0; c < kDotCols; ++c) {
    if (c < nc) {
      const double t = warp_sum(df::to_double(acc[c]));
      if (lane == 0) red[wid][c] = t;
    }
  }
  if (self) {
    const double t = warp_sum(df::to_double(accw));
    if (lane == 0) red[wid][kDotCols] = t;
  }
  __syncthreads();
  if (threadIdx.x < nc) {
    double t = 0.;
    for (int q = 0; q < kVecThreads / 32; ++q) t += red[q][threadIdx.x];
    partial[(size_t)(j0 + threadIdx.x) * gridDim.x + blockIdx.x] = t;
  }
  if (self && threadIdx.x == kDotCols) {
    double t = 0.;
    for (int q = 0; q < kVecThreads / 32; ++q) t += red[q][kDotCols];
    partial[(size_t)k * gridDim.x + blockIdx.x] = t;
  }
  if (!last_block_done(count, blockIdx.y, gridDim.x)) return;
  if (wid < nc) {
    const double* p = partial + (size_t)(j0 + wid) * gridDim.x;
    double t = 0.;
    for (int b = lane; b < (int)gridDim.x; b += 32) t += __ldcg(p + b);
    t = warp_sum(t);
    if (lane == 0) out[(size_t)(j0 + wid) * out_stride] = t;
  }
  if (self && wid == kVecThreads / 32 - 1) {
    const double* p = partial + (size_t)k * gridDim.x;
    double t = 0.;
    for (int b = lane; b < (int)gridDim.x; b += 32) t += __ldcg(p + b);
    t = warp_sum(t);
    if (lane == 0) *self_out = t;
  }
}
// y -= A[:, 0:k] coef (k_gemv_rows<true> in double-float; the same skip and
// selective-reorthogonalisation outputs).  nrm_out, when given, receives
// |y|^2 of the result (Dot2 per thread, partial sums per block, the last
// block adds them in block order), so no separate norm pass follows.
__global__ void __launch_bounds__(kVecThreads)
    k_df_gemv_sub(const float2* __restrict__ A, int64_t lda, int k, const double* __restrict__ coef,
                  float2* __restrict__ y, int64_t n, const double* __restrict__ skip, const double* __restrict__ w2,
                  double* __restrict__ skip_out, double* __restrict__ partial, unsigned* __restrict__ count,
                  double* __restrict__ nrm_out) {
  if (skip && *skip != 0.) return;
  __shared__ double red[kVecThreads / 32];
  __shared__ float2 c[kMaxSubspace + 2];
  for (int j = threadIdx.x; j < k; j += blockDim.x) c[j] = df::split(coef[j]);
  if (skip_out && blockIdx.x == 0 && threadIdx.x == 0) {
    double cc = 0.;
    for (int j = 0; j < k; ++j) cc += coef[j] * coef[j];
    *skip_out = (*w2 - cc >= 0.5 * *w2) ? 1. : 0.;
  }
  __syncthreads();
  const float2 zero = make_float2(0.f, 0.f);
  float2 yy = zero;
  const int64_t step = (int64_t)gridDim.x * kVecTile;
  for (int64_t i = (int64_t)blockIdx.x * kVecTile + threadIdx.x; i < n; i += step) {
    const int64_t i1 = i + kVecThreads;
    const bool has1 = i1 < n;
    float2 s0 = zero, s1 = zero;
    int j = 0;
    for (; j + 4 <= k; j += 4) {
      float2 a0[4], a1[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        a0[q] = A[i + (size_t)(j + q) * lda];
        a1[q] = has1 ? A[i1 + (size_t)(j + q) * lda] : zero;
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        df::mac(s0, a0[q], c[j + q]);
        df::mac(s1, a1[q], c[j + q]);
      }
    }
    for (; j < k; ++j) {
      df::mac(s0, A[i + (size_t)j * lda], c[j]);
      if (has1) df::mac(s1, A[i1 + (size_t)j * lda], c[j]);
    }
    const float2 y0 = df::sub(y[i], df::normalise(s0));
    y[i] = y0;
    df::mac(yy, y0, y0);
    if (has1) {
      const float2 y1 = df::sub(y[i1], df::normalise(s1));
      y[i1] = y1;
      df::mac(yy, y1, y1);
    }
  }
  if (!nrm_out) return;
  const double t = block_sum_vec(df::to_double(yy), red);
  if (threadIdx.x == 0) partial[blockIdx.x] = t;
  if (!last_block_done(count, kDotChunks, gridDim.x)) return;
  double u = 0.;
  for (int b = threadIdx.x; b < (int)gridDim.x; b += kVecThreads) u += __ldcg(partial + b);
  __syncthreads();
  u = block_sum_vec(u, red);
  if (threadIdx.x == 0) *nrm_out = u;
}
// Y[:, o] = A[:, 0:k] Q[:, o] for o < nout (k_gemv_multi in double-float)
__global__ void __launch_bounds__(kVecThreads)
    k_df_gemv_multi(const float2* __restrict__ A, int64_t lda, int k, const double* __restrict__ Q, int nout,
                    float2* __restrict__ Y, int64_t ldy, int64_t n) {
  __shared__ float2 q[kMaxSubspace + 2][kMaxOut];
  for (int t = threadIdx.x; t < k * kMaxOut; t += blockDim.x) {
    const int j = t / kMaxOut, o = t % kMaxOut;
    q[j][o] = o < nout ? df::split(Q[(size_t)o * k + j]) : make_float2(0.f, 0.f);
  }
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * kVecThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kVecThreads) {
    float2 acc[kMaxOut];
#pragma unroll
    for (int o = 0; o < kMaxOut; ++o) acc[o] = make_float2(0.f, 0.f);
    for (int j = 0; j < k; ++j) {
      const float2 a = A[i + (size_t)j * lda];
#pragma unroll
      for (int o = 0; o < kMaxOut; ++o)
        if (o < nout) df::mac(acc[o], a, q[j][o]);
    }
#pragma unroll
    for (int o = 0; o < kMaxOut; ++o)
      if (o < nout) Y[i + (size_t)o * ldy] = df::normalise(acc[o]);
  }
}
// w *= 1/sqrt(*nrm2) when sqrt(*nrm2) > min_norm, else raise *flag; xf, when
// given, receives the FP32 copy of the result (the next FP32 sigma's input)
__global__ void k_df_normalize(float2* w, int64_t n, const double* nrm2, double min_norm, double* flag, float* xf) {
  __shared__ float2 sc;
  __shared__ bool ok;
  if (threadIdx.x == 0) {
    const double nrm = sqrt(*nrm2);
    ok = nrm > min_norm;
    sc = df::split(ok ? 1. / nrm : 0.);
    if (!ok && flag && blockIdx.x == 0) *flag = 1.;
  }
  __syncthreads();
  if (!ok) return;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float2 v = df::mul(w[i], sc);
    w[i] = v;
    if (xf) xf[i] = v.x;
  }
}
// X = V C0, R = AV C0 - lam0 X, *out = |R|^2 (k_ritz_residual in double-float;
// with Dd, R is stored preconditioned: -R / (D - lam0) with |D - lam0|
// clamped to min_abs, formed in FP32 - a search direction, orthogonalised
// afterwards)
__global__ void __launch_bounds__(kVecThreads)
    k_df_ritz_residual(const float2* __restrict__ V, const float2* __restrict__ AV, int64_t ld, int k,
                       const double* __restrict__ C0, const double* __restrict__ lam, float2* __restrict__ X,
                       float2* __restrict__ R, int64_t n, const float2* __restrict__ Dd, double min_abs,
                       double* __restrict__ partial, unsigned* __restrict__ count, double* __restrict__ out) {
  __shared__ float2 c[kMaxSubspace + 2];
  __shared__ double red[kVecThreads / 32];
  for (int j = threadIdx.x; j < k; j += blockDim.x) c[j] = df::split(C0[j]);
  __syncthreads();
  const float2 l0 = df::split(lam[0]);
  const float mina = (float)min_abs;
  const float2 zero = make_float2(0.f, 0.f);
  float s2 = 0.f;
  const int64_t step = (int64_t)gridDim.x * kVecTile;
  for (int64_t i = (int64_t)blockIdx.x * kVecTile + threadIdx.x; i < n; i += step) {
    const int64_t i1 = i + kVecThreads;
    const bool has1 = i1 < n;
    float2 x0 = zero, ax0 = zero, x1 = zero, ax1 = zero;
    int j = 0;
    for (; j + 4 <= k; j += 4) {
      float2 v0[4], v1[4], w0[4], w1[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const size_t o = (size_t)(j + q) * ld;
        v0[q] = V[i + o];
        w0[q] = AV[i + o];
        v1[q] = has1 ? V[i1 + o] : zero;
        w1[q] = has1 ? AV[i1 + o] : zero;
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        df::mac(x0, v0[q], c[j + q]);
        df::mac(ax0, w0[q], c[j + q]);
        df::mac(x1, v1[q], c[j + q]);
        df::mac(ax1, w1[q], c[j + q]);
      }
    }
    for (; j < k; ++j) {
      const size_t o = (size_t)j * ld;
      df::mac(x0, V[i + o], c[j]);
      df::mac(ax0, AV[i + o], c[j]);
      if (has1) {
        df::mac(x1, V[i1 + o], c[j]);
        df::mac(ax1, AV[i1 + o], c[j]);
      }
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      if (h == 1 && !has1) break;
      const int64_t r = h ? i1 : i;
      const float2 xv = df::normalise(h ? x1 : x0);
      const float2 rv = df::sub(df::normalise(h ? ax1 : ax0), df::mul(l0, xv));
      X[r] = xv;
      s2 = __fmaf_rn(rv.x, rv.x, s2);
      if (Dd) {
        const float2 dd = Dd[r];
        float d = __fadd_rn(__fsub_rn(dd.x, l0.x), __fsub_rn(dd.y, l0.y));
        if (fabsf(d) < mina) d = (d >= 0.f) ? mina : -mina;
        R[r] = make_float2(__fdiv_rn(-rv.x, d), 0.f);
      } else {
        R[r] = rv;
      }
    }
  }
  const double t = block_sum_vec((double)s2, red);
  if (threadIdx.x == 0) partial[blockIdx.x] = t;
  if (!last_block_done(count, kDotChunks, gridDim.x)) return;
  double u = 0.;
  for (int b = threadIdx.x; b < (int)gridDim.x; b += kVecThreads) u += __ldcg(partial + b);
  __syncthreads();
  u = block_sum_vec(u, red);
  if (threadIdx.x == 0) *out = u;
}
__global__ void k_df_from_f64(const double* __restrict__ x, float2* __restrict__ y, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = df::split(x[i]);
}
__global__ void k_df_from_f32(const float* __restrict__ x, float2* __restrict__ y, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = make_float2(x[i], 0.f);
}
__global__ void k_df_to_f64(const float2* __restrict__ x, double* __restrict__ y, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = df::to_double(x[i]);
}
// k_flip_project in double-float: x <- (x + s x^T) / 2 (s = +-1, so s x and
// the halving are exact)
__global__ void __launch_bounds__(kFlipTile * 8) k_df_flip_project(float2* x, int64_t n, float s) {
  const int I = blockIdx.y, J = blockIdx.x;
  if (I > J) return;
  __shared__ float2 P[kFlipTile][kFlipTile + 1], Q[kFlipTile][kFlipTile + 1];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int64_t r0 = (int64_t)I * kFlipTile, c0 = (int64_t)J * kFlipTile;
  const float2 zero = make_float2(0.f, 0.f);
  for (int r = ty; r < kFlipTile; r += 8) {
    const int64_t pr = r0 + r, pc = c0 + tx, qr = c0 + r, qc = r0 + tx;
    P[r][tx] = (pr < n && pc < n) ? x[pr * n + pc] : zero;
    Q[r][tx] = (qr < n && qc < n) ? x[qr * n + qc] : zero;
  }
  __syncthreads();
  // (a + s b) / 2, and s times it
  auto avg = [s](float2 a, float2 b) {
    const float2 t = df::add(a, make_float2(s * b.x, s * b.y));
    return make_float2(0.5f * t.x, 0.5f * t.y);
  };
  for (int r = ty; r < kFlipTile; r += 8) {
    const int64_t pr = r0 + r, pc = c0 + tx, qr = c0 + r, qc = r0 + tx;
    if (I < J) {
      if (pr < n && pc < n) x[pr * n + pc] = avg(P[r][tx], Q[tx][r]);
      if (qr < n && qc < n) {
        const float2 v = avg(P[tx][r], Q[r][tx]);
        x[qr * n + qc] = make_float2(s * v.x, s * v.y);
      }
    } else if (pr < n && pc < n) {
      float2 v;
      if (r < tx) {
        v = avg(P[r][tx], P[tx][r]);
      } else if (r > tx) {
        v = avg(P[tx][r], P[r][tx]);
        v = make_float2(s * v.x, s * v.y);
      } else {
        v = s < 0 ? zero : P[r][tx];
      }
      x[pr * n + pc] = v;
    }
  }
}

__global__ void __launch_bounds__(kEigThreads) k_lowest_eig(int k, const double* __restrict__ H, int ldh,
                                                            double* gA, int nev, double* eval, double* evec) {
  lowest_eig_cta(k, H, ldh, gA, nev, eval, evec);
}

// One CTA per instance of a batch: the lowest pair of the leading k x k block
// of Hs[b] (k = *kdev + kadd, matrices hstride apart, ld ldh); CTAs of
// inactive instances leave at once.
__global__ void __launch_bounds__(kEigThreads)
    k_lowest_eig_batch(const int* __restrict__ kdev, int kadd, const double* __restrict__ Hs, int ldh,
                       int64_t hstride, double* eval, double* evec, int64_t estride, const int* __restrict__ active) {
  const int b = blockIdx.x;
  if (active && !active[b]) return;
  const int k = *kdev + kadd;
  lowest_eig_cta(k, Hs + b * hstride, ldh, nullptr, 1, eval + b, evec + b * estride);
}

void lowest_eig_batch(cudaStream_t st, int B, const int* kdev, int kadd, int kmax, const double* Hs, int ldh,
                      int64_t hstride, double* eval, double* evec, int64_t estride, const int* active) {
  if (kmax > kEigSmemK) throw Error(QDKGB_ERR_INVALID, "batched subspace larger than the shared-memory eigensolver");
  set_max_dynamic_smem((const void*)k_lowest_eig_batch, (int)kEigDynSmemMax);
  k_lowest_eig_batch<<<B, kEigThreads, eig_dyn_smem(kmax), st>>>(kdev, kadd, Hs, ldh, hstride, eval, evec, estride,
                                                                 active);
  QDKGB_CHECK_LAUNCH();
}

// ---------------------------------------------------------------- driver
namespace {

// slots in the small scratch array
constexpr int kSlotRes = kMaxSubspace + 4;   // residual norm^2 (device reduce target)
constexpr int kSlotNrm = kMaxSubspace + 8;   // Gram-Schmidt norm^2
constexpr int kSlotE = kMaxSubspace + 12;    // full-precision Rayleigh quotient
constexpr int kSlotFlag = kMaxSubspace + 16; // Gram-Schmidt degeneracy flag
constexpr int kSlotW2 = kMaxSubspace + 20;   // |w|^2 before a Gram-Schmidt pass
constexpr int kSlotSkip = kMaxSubspace + 24; // selective second pass: 1 = not needed
constexpr int kSlotRoots = 2 * kMaxSubspace; // per-root residual norm^2 of the block Davidson (8)
constexpr int kSlotIdx = 3 * kMaxSubspace;   // argmin index (int64)
constexpr int kSlotCount = 3 * kMaxSubspace + 16;  // block-completion counters (unsigned, kDotChunks + 1)

struct Dav {
  Context* c;
  int64_t n;
  int64_t maxm;
  double *V, *AV, *D, *X, *Hk, *evec, *eval, *partial, *small, *work;
  int nb;  // blocks of the row-parallel kernels (partial sums per column)
  int sm_count;
  double* gA = nullptr;
  cudaStream_t st;

  unsigned* counts() { return (unsigned*)(small + kSlotCount); }

  double* col(double* base, int64_t j) { return base + (size_t)j * n; }

  // out[j * stride] = A[:, j] . w, j < k: column blocks of kDotCols on
  // grid.y, the row split on grid.x shrunk as column blocks are added (down to
  // one block per SM) so the grid stays near one resident wave
  void multidot(const double* A, int k, const double* w, double* out, int stride, double* self_out = nullptr,
                const double* skip = nullptr) {
    const int chunks = (k + kDotCols - 1) / kDotCols;
    const int bx = std::max(1, std::min(nb, std::max(sm_count, nb / chunks)));
    k_multidot<<<dim3(bx, chunks), kVecThreads, 0, st>>>(A, n, k, w, n, partial, counts(), out, stride, self_out,
                                                         skip);
    QDKGB_CHECK_LAUNCH();
  }
  void norm2(const double* w, double* out) { multidot(w, 1, w, out, 1); }

  void fetch(const double* a, double& va) {
    QDKGB_CUDA(cudaMemcpyAsync(c->pinned, a, sizeof(double), cudaMemcpyDeviceToHost, st));
    QDKGB_CUDA(cudaStreamSynchronize(st));
    va = c->pinned[0];
  }
  // residual norm^2, lowest Ritz value and the pending Gram-Schmidt flag in one sync
  void fetch3(const double* a, const double* b, double& va, double& vb, bool& flag) {
    QDKGB_CUDA(cudaMemcpyAsync(c->pinned, a, sizeof(double), cudaMemcpyDeviceToHost, st));
    QDKGB_CUDA(cudaMemcpyAsync(c->pinned + 1, b, sizeof(double), cudaMemcpyDeviceToHost, st));
    QDKGB_CUDA(cudaMemcpyAsync(c->pinned + 2, small + kSlotFlag, sizeof(double), cudaMemcpyDeviceToHost, st));
    QDKGB_CUDA(cudaStreamSynchronize(st));
    va = c->pinned[0];
    vb = c->pinned[1];
    flag = c->pinned[2] != 0.;
  }
  void clear_flag() { QDKGB_CUDA(cudaMemsetAsync(small + kSlotFlag, 0, sizeof(double), st)); }

  // Two CGS passes against V[:, 0:K].  selective: the second pass only when
  // the first removed more than half of |w|^2 (the Daniel-Gragg-Kaufman-
  // Stewart test, decided on the device; the mixed path's choice - the
  // reference always makes two passes).
  void orth_passes(int K, double* w, bool selective = false) {
    if (K <= 0) return;
    if (!selective) {
      for (int pass = 0; pass < 2; ++pass) {
        multidot(V, K, w, small, 1);
        k_gemv_rows<true><<<nb, kVecThreads, 0, st>>>(V, n, K, small, 1, w, n);
        QDKGB_CHECK_LAUNCH();
      }
      return;
    }
    multidot(V, K, w, small, 1, small + kSlotW2);
    k_gemv_rows<true><<<nb, kVecThreads, 0, st>>>(V, n, K, small, 1, w, n, nullptr, small + kSlotW2,
                                                  small + kSlotSkip);
    QDKGB_CHECK_LAUNCH();
    multidot(V, K, w, small, 1, nullptr, small + kSlotSkip);
    k_gemv_rows<true><<<nb, kVecThreads, 0, st>>>(V, n, K, small, 1, w, n, small + kSlotSkip);
    QDKGB_CHECK_LAUNCH();
  }
  // gram_schmidt (davidson.hpp:185-238): two CGS passes against V[:, 0:K],
  // normalise; a degenerate result raises the device flag (checked at the
  // next host sync, then repaired by fallback()).
  void gram_schmidt(int K, double* w, double min_norm = 1e-12, bool selective = false) {
    orth_passes(K, w, selective);
    norm2(w, small + kSlotNrm);
    k_normalize<<<nb, 256, 0, st>>>(w, n, small + kSlotNrm, min_norm, small + kSlotFlag);
    QDKGB_CHECK_LAUNCH();
  }
  // canonical-vector fallback of gram_schmidt (davidson.hpp:211-236)
  void fallback(int K, double* w, double min_norm = 1e-12) {
    for (int64_t idx = 0; idx < n; ++idx) {
      QDKGB_CUDA(cudaMemsetAsync(w, 0, n * sizeof(double), st));
      const double one = 1.0;
      QDKGB_CUDA(cudaMemcpyAsync(w + idx, &one, sizeof(double), cudaMemcpyHostToDevice, st));
      orth_passes(K, w);
      norm2(w, small + kSlotNrm);
      double nv;
      fetch(small + kSlotNrm, nv);
      if (std::sqrt(nv) > min_norm) {
        k_normalize<<<nb, 256, 0, st>>>(w, n, small + kSlotNrm, min_norm, nullptr);
        QDKGB_CHECK_LAUNCH();
        clear_flag();
        return;
      }
    }
    throw Error(QDKGB_ERR_INVALID, "gram_schmidt: Unable to find orthogonal vector");
  }

  // lowest `nev` eigenpairs of the leading k x k projected matrix
  void lowest(int k, int nev = 1) {
    const bool in_smem = k <= kEigSmemK;
    k_lowest_eig<<<1, kEigThreads, in_smem ? eig_dyn_smem(k) : 0, st>>>(
        k, Hk, (int)(maxm + 1), in_smem ? nullptr : gA, std::min(nev, k), eval, evec);
    QDKGB_CHECK_LAUNCH();
  }

  // new row i of the projected matrix, Hk(i, c) = V_i . AV_c for c <= i,
  // mirrored (syev reads the lower triangle, rayleigh_ritz.hpp:70-77)
  void projected_row(int i) {
    multidot(AV, i + 1, col(V, i), small, 1);
    k_store_row<<<1, 256, 0, st>>>(small, i, Hk, (int)(maxm + 1));
    QDKGB_CHECK_LAUNCH();
  }

  // X = V C0, R = AV C0 - lam0 X with |R|^2 into small[kSlotRes]; R is
  // stored preconditioned with the diagonal D (the next direction before
  // orthogonalisation)
  void ritz_residual(int k, double* R, double min_abs) {
    k_ritz_residual<<<nb, kVecThreads, 0, st>>>(V, AV, n, k, evec, eval, X, R, n, D, min_abs, partial, counts(),
                                                small + kSlotRes);
    QDKGB_CHECK_LAUNCH();
  }
  // ---- the double-float subspace of the mixed-precision solver
  float2 *Vf = nullptr, *AVf = nullptr;
  float* xf = nullptr;  // FP32 copy of the newest normalised direction (the FP32 sigma's input)
  float2* colf(float2* base, int64_t j) { return base + (size_t)j * n; }
  // grid as multidot's, sized by the blocks of k_df_multidot resident per SM
  // (its sixteen loads in flight per thread take more registers than four
  // blocks per SM allow)
  void df_multidot(const float2* A, int k, const float2* w, double* out, int stride, double* self_out = nullptr,
                   const double* skip = nullptr) {
    static const int per_sm = [] {
      int b = 0;
      QDKGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_df_multidot, kVecThreads, 0));
      return std::max(1, std::min(b, kVecBlocksPerSm));
    }();
    const int nbd = (int)std::max<int64_t>(1, std::min<int64_t>((n + kVecTile - 1) / kVecTile, (int64_t)sm_count * per_sm));
    const int chunks = (k + kDotCols - 1) / kDotCols;
    const int bx = std::max(1, std::min(nbd, std::max(sm_count, nbd / chunks)));
    k_df_multidot<<<dim3(bx, chunks), kVecThreads, 0, st>>>(A, n, k, w, n, partial, counts(), out, stride, self_out,
                                                            skip);
    QDKGB_CHECK_LAUNCH();
  }
  // the two CGS passes of df_gram_schmidt; every update that runs leaves
  // |w|^2 of its result in small[kSlotNrm] (the second, selective one only
  // when the test asks for it)
  void df_orth_passes(int K, float2* w, bool selective = false) {
    if (K <= 0) {
      df_multidot(w, 1, w, small + kSlotNrm, 1);
      return;
    }
    double* nrm = small + kSlotNrm;
    if (!selective) {
      for (int pass = 0; pass < 2; ++pass) {
        df_multidot(Vf, K, w, small, 1);
        k_df_gemv_sub<<<nb, kVecThreads, 0, st>>>(Vf, n, K, small, w, n, nullptr, nullptr, nullptr, partial, counts(),
                                                  nrm);
        QDKGB_CHECK_LAUNCH();
      }
      return;
    }
    df_multidot(Vf, K, w, small, 1, small + kSlotW2);
    k_df_gemv_sub<<<nb, kVecThreads, 0, st>>>(Vf, n, K, small, w, n, nullptr, small + kSlotW2, small + kSlotSkip,
                                              partial, counts(), nrm);
    QDKGB_CHECK_LAUNCH();
    df_multidot(Vf, K, w, small, 1, nullptr, small + kSlotSkip);
    k_df_gemv_sub<<<nb, kVecThreads, 0, st>>>(Vf, n, K, small, w, n, small + kSlotSkip, nullptr, nullptr, partial,
                                              counts(), nrm);
    QDKGB_CHECK_LAUNCH();
  }
  // gram_schmidt on the double-float basis; the normalised result's FP32
  // copy goes to xf
  void df_gram_schmidt(int K, float2* w, double min_norm, bool selective) {
    df_orth_passes(K, w, selective);
    k_df_normalize<<<nb, 256, 0, st>>>(w, n, small + kSlotNrm, min_norm, small + kSlotFlag, xf);
    QDKGB_CHECK_LAUNCH();
  }
  void df_fallback(int K, float2* w, double min_norm = 1e-12) {
    for (int64_t idx = 0; idx < n; ++idx) {
      QDKGB_CUDA(cudaMemsetAsync(w, 0, n * sizeof(float2), st));
      const float2 one = make_float2(1.f, 0.f);
      QDKGB_CUDA(cudaMemcpyAsync(w + idx, &one, sizeof(float2), cudaMemcpyHostToDevice, st));
      df_orth_passes(K, w);
      double nv;
      fetch(small + kSlotNrm, nv);
      if (std::sqrt(nv) > min_norm) {
        k_df_normalize<<<nb, 256, 0, st>>>(w, n, small + kSlotNrm, min_norm, nullptr, xf);
        QDKGB_CHECK_LAUNCH();
        clear_flag();
        return;
      }
    }
    throw Error(QDKGB_ERR_INVALID, "gram_schmidt: Unable to find orthogonal vector");
  }
  void df_projected_row(int i) {
    df_multidot(AVf, i + 1, colf(Vf, i), small, 1);
    k_store_row<<<1, 256, 0, st>>>(small, i, Hk, (int)(maxm + 1));
    QDKGB_CHECK_LAUNCH();
  }
  void df_ritz_residual(int k, float2* Xr, float2* R, const float2* Dd, double min_abs) {
    k_df_ritz_residual<<<nb, kVecThreads, 0, st>>>(Vf, AVf, n, k, evec, eval, Xr, R, n, Dd, min_abs, partial, counts(),
                                                   small + kSlotRes);
    QDKGB_CHECK_LAUNCH();
  }
  void df_from_f64(const double* x, float2* y) {
    k_df_from_f64<<<nb, 256, 0, st>>>(x, y, n);
    QDKGB_CHECK_LAUNCH();
  }
  void df_to_f64(const float2* x, double* y) {
    k_df_to_f64<<<nb, 256, 0, st>>>(x, y, n);
    QDKGB_CHECK_LAUNCH();
  }

  // the same for root r of the last Rayleigh-Ritz (eigenvector column r, ld
  // k): Ritz vector into Xr, preconditioned residual into Rr, |R|^2 into
  // small[kSlotRoots + r]
  void ritz_residual_root(int k, int r, double* Xr, double* Rr, double min_abs) {
    k_ritz_residual<<<nb, kVecThreads, 0, st>>>(V, AV, n, k, evec + (size_t)r * k, eval + r, Xr, Rr, n, D, min_abs,
                                                partial, counts(), small + kSlotRoots + r);
    QDKGB_CHECK_LAUNCH();
  }
};

}  // namespace

// ---------------------------------------------------------------- several roots
// Block Davidson for the `nroots` lowest eigenpairs (FP64).  The reference's
// davidson is single-root; its multi-root solver is lobpcgxx::lobpcg.  Here:
// a guess block of the nroots lowest diagonal elements (or the caller's
// vectors), the projected matrix grown one column at a time as in the
// single-root solver, Rayleigh-Ritz in FP64 (the Householder / Sturm /
// inverse-iteration solver with its matrix in global memory), and per
// iteration one new direction for every unconverged root: its residual
// preconditioned with (D - theta_r) clamped at min_abs_denominator, then two
// Gram-Schmidt passes.  When the next block would exceed max_m the basis
// restarts on the current Ritz vectors (and their sigmas, formed from the
// basis, so no extra operator application).  Converged when every root's
// residual 2-norm is below res_tol.
static void davidson_roots(Context* c, const qdkgb_davidson_settings* s, double* E, double* C,
                           qdkgb_davidson_info* info) {
  NvtxRange nvtx_range("qdkgb.davidson_roots");
  using clk = std::chrono::steady_clock;
  const auto t0 = clk::now();
  Hcsr& H = c->H;
  const int64_t N = H.n;
  const int R = s->nroots;
  if (s->precision != QDKGB_PREC_FP64) throw Error(QDKGB_ERR_UNSUPPORTED, "several roots: FP64 precision only");
  if (R > N) throw Error(QDKGB_ERR_INVALID, "nroots exceeds the number of determinants");
  if (R > kMaxOut) throw Error(QDKGB_ERR_UNSUPPORTED, "at most 8 roots");
  int64_t max_m = std::min<int64_t>(s->max_m, N);
  if (max_m > kMaxSubspace - 2) throw Error(QDKGB_ERR_INVALID, "max_m above 254 is not supported");
  if (max_m < 2 * R) throw Error(QDKGB_ERR_INVALID, "max_m must hold at least twice nroots vectors");
  qdkgb_davidson_info loc{};
  DavidsonWork& W = c->dav;
  Dav d;
  d.c = c;
  d.n = N;
  d.maxm = max_m;
  d.st = c->stream;
  d.sm_count = std::max(1, c->sm_count);
  d.nb = (int)std::max<int64_t>(1, std::min<int64_t>((N + kVecTile - 1) / kVecTile, (int64_t)d.sm_count * kVecBlocksPerSm));
  d.V = dev_array<double>(c, W.V, (size_t)N * (max_m + 1));
  d.AV = dev_array<double>(c, W.AV, (size_t)N * (max_m + 1));
  // Ritz vectors X_r, their sigmas AX_r and the preconditioned residuals
  d.X = dev_array<double>(c, W.scratch, (size_t)N * 3 * R);
  double* AX = d.X + (size_t)N * R;
  double* Rr = AX + (size_t)N * R;
  d.work = nullptr;
  d.Hk = dev_array<double>(c, W.Hk, (size_t)(max_m + 1) * (max_m + 1));
  d.evec = dev_array<double>(c, W.evec, (size_t)(max_m + 1) * (max_m + 1));
  d.eval = dev_array<double>(c, W.eval, (size_t)(max_m + 1));
  d.partial = dev_array<double>(c, W.partial, (size_t)d.nb * (kMaxSubspace + 2));
  d.small = dev_array<double>(c, W.small, 4 * kMaxSubspace);
  d.gA = dev_array<double>(c, W.yf, (size_t)(max_m + 1) * (max_m + 1));  // FP64 Rayleigh-Ritz (global matrix)
  d.D = (double*)H.diag.ptr;
  d.clear_flag();
  QDKGB_CUDA(cudaMemsetAsync(d.counts(), 0, (kDotChunks + 1) * sizeof(unsigned), c->stream));
  auto sigma = [&](const double* x, double* y) {
    spmv_fp64(c, x, y);
    loc.spmv_fp64++;
  };
  auto fetch_n = [&](const double* a, int cnt, std::vector<double>& out) {
    std::vector<double> h(cnt);
    QDKGB_CUDA(cudaMemcpyAsync(h.data(), a, cnt * sizeof(double), cudaMemcpyDeviceToHost, d.st));
    QDKGB_CUDA(cudaStreamSynchronize(d.st));
    out = h;
  };
  auto lowest_fp64 = [&](int k) {
    k_lowest_eig<<<1, kEigThreads, 0, d.st>>>(k, d.Hk, (int)(max_m + 1), d.gA, R, d.eval, d.evec);
    QDKGB_CHECK_LAUNCH();
  };
  // append w (already in V[:, k]) : orthonormalise, sigma, projected row
  int k = 0;
  auto append = [&](double* w) -> bool {
    double* vk = d.col(d.V, k);
    if (w != vk) QDKGB_CUDA(cudaMemcpyAsync(vk, w, N * sizeof(double), cudaMemcpyDeviceToDevice, d.st));
    d.gram_schmidt(k, vk);
    double flag = 0.;
    d.fetch(d.small + kSlotFlag, flag);
    if (flag != 0.) {  // linearly dependent: drop it
      d.clear_flag();
      return false;
    }
    sigma(vk, d.col(d.AV, k));
    d.projected_row(k);
    ++k;
    return true;
  };

  // guess block
  if (s->use_guess && C) {
    for (int r = 0; r < R; ++r) append(const_cast<double*>(C) + (size_t)r * N);
  }
  if (k < R) {
    std::vector<double> Dh(N);
    QDKGB_CUDA(cudaMemcpyAsync(Dh.data(), d.D, N * sizeof(double), cudaMemcpyDeviceToHost, d.st));
    QDKGB_CUDA(cudaStreamSynchronize(d.st));
    std::vector<int64_t> idx(N);
    for (int64_t i = 0; i < N; ++i) idx[i] = i;
    const int64_t m = std::min<int64_t>(N, 4 * R + 4);
    std::partial_sort(idx.begin(), idx.begin() + m, idx.end(),
                      [&](int64_t x, int64_t y) { return Dh[x] < Dh[y] || (Dh[x] == Dh[y] && x < y); });
    for (int64_t q = 0; q < m && k < R; ++q) {
      double* w = d.col(d.V, k);
      QDKGB_CUDA(cudaMemsetAsync(w, 0, N * sizeof(double), d.st));
      const double one = 1.0;
      QDKGB_CUDA(cudaMemcpyAsync(w + idx[q], &one, sizeof(double), cudaMemcpyHostToDevice, d.st));
      append(w);
    }
  }
  if (k < R) throw Error(QDKGB_ERR_INVALID, "several roots: no independent guess block");

  std::vector<double> theta(R), rn(R);
  bool converged = false;
  const int64_t max_iter = 50 * max_m;
  int64_t iter = 0;
  for (; iter < max_iter; ++iter) {
    lowest_fp64(k);
    for (int r = 0; r < R; ++r) {
      d.ritz_residual_root(k, r, d.col(d.X, r), d.col(Rr, r), s->min_abs_denominator);
      k_gemv_rows<false><<<d.nb, kVecThreads, 0, d.st>>>(d.AV, N, k, d.evec + (size_t)r * k, 1, AX + (size_t)r * N, N);
      QDKGB_CHECK_LAUNCH();
    }
    fetch_n(d.eval, R, theta);
    fetch_n(d.small + kSlotRoots, R, rn);
    double worst = 0.;
    for (int r = 0; r < R; ++r) worst = std::max(worst, std::sqrt(rn[r]));
    loc.iterations = iter + 1;
    loc.residual_norm = worst;
    if (worst < s->res_tol) {
      converged = true;
      break;
    }
    int pending = 0;
    for (int r = 0; r < R; ++r) pending += std::sqrt(rn[r]) >= s->res_tol;
    if (k + pending > max_m) {
      // restart on the Ritz vectors and their sigmas
      QDKGB_CUDA(cudaMemcpyAsync(d.V, d.X, (size_t)N * R * sizeof(double), cudaMemcpyDeviceToDevice, d.st));
      QDKGB_CUDA(cudaMemcpyAsync(d.AV, AX, (size_t)N * R * sizeof(double), cudaMemcpyDeviceToDevice, d.st));
      k = R;
      for (int i = 0; i < R; ++i) d.projected_row(i);
      loc.restarts++;
    }
    for (int r = 0; r < R; ++r)
      if (std::sqrt(rn[r]) >= s->res_tol && k < max_m) append(d.col(Rr, r));
  }
  fetch_n(d.eval, R, theta);
  for (int r = 0; r < R; ++r) E[r] = theta[r];
  if (C) QDKGB_CUDA(cudaMemcpyAsync(C, d.X, (size_t)N * R * sizeof(double), cudaMemcpyDeviceToHost, d.st));
  QDKGB_CUDA(cudaStreamSynchronize(d.st));
  loc.seconds = std::chrono::duration<double>(clk::now() - t0).count();
  if (info) *info = loc;
  if (!converged) throw Error(QDKGB_ERR_NOT_CONVERGED, "Davidson Did Not Converge!");
}

void davidson(Context* c, const qdkgb_davidson_settings* s, double* E, double* C, qdkgb_davidson_info* info) {
  if (s->nroots > 1) {
    if (!c->H.valid) throw Error(QDKGB_ERR_STATE, "Hamiltonian not built");
    davidson_roots(c, s, E, C, info);
    return;
  }
  NvtxRange nvtx_range("qdkgb.davidson");
  using clk = std::chrono::steady_clock;
  const auto t0 = clk::now();
  Hcsr& H = c->H;
  if (!H.valid) throw Error(QDKGB_ERR_STATE, "Hamiltonian not built");
  const int64_t N = H.n;
  const bool mixed = s->precision == QDKGB_PREC_MIXED;
  if (mixed && !c->op_direct && !c->fp32_direct && H.storage != QDKGB_H_SPLIT32)
    throw Error(QDKGB_ERR_STATE, "mixed precision needs the Hamiltonian built with QDKGB_H_SPLIT32 storage");
  if (s->precision != QDKGB_PREC_FP64 && !mixed) throw Error(QDKGB_ERR_INVALID, "unknown precision");
  if (s->max_m < 2 && N > 1) throw Error(QDKGB_ERR_INVALID, "max_m must be >= 2");
  int64_t max_m = std::min<int64_t>(s->max_m, N);
  if (max_m > kMaxSubspace - 2) throw Error(QDKGB_ERR_INVALID, "max_m above 254 is not supported");
  qdkgb_davidson_info loc{};
  DavidsonWork& W = c->dav;
  Dav d;
  d.c = c;
  d.n = N;
  d.maxm = max_m;
  d.st = c->stream;
  d.sm_count = std::max(1, c->sm_count);
  d.nb = (int)std::max<int64_t>(1, std::min<int64_t>((N + kVecTile - 1) / kVecTile, (int64_t)d.sm_count * kVecBlocksPerSm));
  d.V = dev_array<double>(c, W.V, (size_t)N * (max_m + 1));
  d.AV = dev_array<double>(c, W.AV, (size_t)N * (max_m + 1));
  constexpr int kKeep = 6;  // thick-restart size of the mixed path
  // X, then the mixed path's FP64 sig and Rt, kKeep + kKeep restart columns
  // and three double-float columns (Ritz vector, overflow direction, diagonal)
  d.X = dev_array<double>(c, W.scratch, (size_t)N * (6 + 2 * kKeep));
  d.work = d.X + N;
  d.Hk = dev_array<double>(c, W.Hk, (size_t)(max_m + 1) * (max_m + 1));
  d.evec = dev_array<double>(c, W.evec, (size_t)(max_m + 1) * (max_m + 1));
  d.eval = dev_array<double>(c, W.eval, (size_t)(max_m + 1));
  d.partial = dev_array<double>(c, W.partial, (size_t)d.nb * (kMaxSubspace + 2));
  d.small = dev_array<double>(c, W.small, 4 * kMaxSubspace);
  if (max_m + 1 > kEigSmemK) d.gA = dev_array<double>(c, W.yf, (size_t)(max_m + 1) * (max_m + 1));
  set_max_dynamic_smem((const void*)k_lowest_eig, (int)kEigDynSmemMax);
  d.D = (double*)H.diag.ptr;
  d.clear_flag();
  QDKGB_CUDA(cudaMemsetAsync(d.counts(), 0, (kDotChunks + 1) * sizeof(unsigned), c->stream));
  float* xf = nullptr;
  float* yf = nullptr;
  if (mixed) {
    xf = dev_array<float>(c, W.xf, (size_t)N * 2);
    yf = xf + N;
  }
  auto sigma_full = [&](const double* x, double* y) {
    spmv_fp64(c, x, y);
    loc.spmv_fp64++;
  };

  // guess (selected_ci_diag.hpp:130-140, diagonal_guess davidson.hpp:106-113);
  // the mixed path holds its basis in double-float form, so its FP64 guess
  // goes to the scratch column X
  double* V0 = mixed ? d.X : d.V;
  bool use_c = false;
  if (s->use_guess && C) {
    double mx = 0.;
    for (int64_t i = 0; i < N; ++i) mx = std::max(mx, std::fabs(C[i]));
    use_c = mx > 1. / (double)N;
  }
  if (use_c) {
    QDKGB_CUDA(cudaMemcpyAsync(V0, C, N * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  } else {
    int64_t* idx = (int64_t*)(d.small + kSlotIdx);
    k_argmin<<<1, 1024, 0, c->stream>>>(d.D, N, idx);
    QDKGB_CHECK_LAUNCH();
    k_set_onehot<<<d.nb, 256, 0, c->stream>>>(V0, N, idx);
    QDKGB_CHECK_LAUNCH();
  }

  if (N == 1) {
    // davidson.hpp:280-288: evaluate the 1x1 operator on X = [1]
    k_set_value<<<1, 1, 0, c->stream>>>(V0, 1.0);
    QDKGB_CHECK_LAUNCH();
    sigma_full(V0, d.AV);
    d.fetch(d.AV, *E);
    if (C) C[0] = 1.0;
    loc.residual_norm = 0.;
    loc.seconds = std::chrono::duration<double>(clk::now() - t0).count();
    if (info) *info = loc;
    return;
  }

  double lam0 = 0., res = 0.;
  bool converged = false;

  if (!mixed) {
    // ---------------- plain FP64 Davidson: the reference's algorithm
    // V1 = GS(A V0) (Krylov start, davidson.hpp:290-299)
    sigma_full(V0, d.AV);
    QDKGB_CUDA(cudaMemcpyAsync(d.col(d.V, 1), d.AV, N * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    d.gram_schmidt(1, d.col(d.V, 1));
    d.projected_row(0);
    int64_t iter = 1;
    for (int64_t i = 1; i < max_m; ++i, ++iter) {
      const int k = (int)i + 1;
      sigma_full(d.col(d.V, i), d.col(d.AV, i));
      d.projected_row((int)i);
      d.lowest(k);
      double* R = d.col(d.V, i + 1);
      d.ritz_residual(k, R, s->min_abs_denominator);
      double r2 = 0.;
      bool degenerate = false;
      d.fetch3(d.small + kSlotRes, d.eval, r2, lam0, degenerate);
      if (degenerate) {
        // V[:, i] was not normalisable: repair it and redo this iteration
        d.fallback((int)i, d.col(d.V, i));
        --i;
        --iter;
        continue;
      }
      res = std::sqrt(r2);
      loc.iterations = iter;
      if (res < s->res_tol) {
        converged = true;
        break;
      }
      d.gram_schmidt(k, R);
    }
  } else {
    // ---------------- mixed: FP32 sigma for new directions, full-precision refresh
    // The same Krylov-started Davidson runs with FP32 sigma columns until the
    // residual estimate stops improving (the FP32 noise floor) or has fallen by
    // `drop` since the last full-precision check.  Then the Ritz vector gets a
    // full-precision sigma; if its true residual is below res_tol the solve
    // is done, otherwise the subspace restarts on the kKeep lowest Ritz
    // vectors, the first carrying the exact sigma, and iterates on.
    const double drop = 1e-4;
    double* sig = d.work;       // exact (full-precision) sigma of the Ritz vector
    double* Rt = d.work + N;    // its exact residual
    float2* dfw = (float2*)(d.work + 2 * N);
    float2* tmpV = dfw;                       // restart columns (kKeep)
    float2* tmpAV = dfw + (size_t)kKeep * N;  // their sigmas (kKeep)
    float2* Xf = dfw + (size_t)2 * kKeep * N;  // Ritz vector
    float2* Rtf = Xf + N;                     // a direction that does not fit the basis
    float2* Df = Rtf + N;                     // the diagonal
    d.Vf = (float2*)d.V;
    d.AVf = (float2*)d.AV;
    d.xf = xf;
    double* Eptr = d.small + kSlotE;
    // The reference's FP64 iteration keeps the guess's spin-flip symmetry
    // (C[Ia, Ib] = +-C[Ib, Ia] when both spins share one string list): H and
    // the preconditioner commute with the flip.  FP32 sigma noise does not, and
    // can steer the solve into the other sector when that one holds a lower
    // state; new directions are therefore projected on the guess's sector.
    double flip = 0.;
    int64_t nstr = 0;
    {
      const DetSpace& S = c->dets;
      bool square = c->have_dets && S.ndets == N && S.ngroups == S.nbeta && S.ngroups * S.nbeta == N &&
                    S.h_galpha == S.h_ubeta;
      for (int64_t g = 0; g < S.ngroups && square; ++g) square = (S.h_gstart[g + 1] - S.h_gstart[g]) == S.nbeta;
      if (square) {
        nstr = S.nbeta;
        std::vector<double> g0(N);
        QDKGB_CUDA(cudaMemcpyAsync(g0.data(), V0, N * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        QDKGB_CUDA(cudaStreamSynchronize(c->stream));
        double dp = 0., dm = 0., nn = 0.;
        for (int64_t i = 0; i < nstr; ++i)
          for (int64_t j = 0; j < nstr; ++j) {
            const double x = g0[i * nstr + j], y = g0[j * nstr + i];
            dp += (x - y) * (x - y);
            dm += (x + y) * (x + y);
            nn += x * x;
          }
        if (dp <= 1e-24 * nn)
          flip = 1.;
        else if (dm <= 1e-24 * nn)
          flip = -1.;
      }
    }
    auto project = [&](float2* v) {
      if (flip == 0.) return;
      const unsigned nt = (unsigned)((nstr + kFlipTile - 1) / kFlipTile);
      k_df_flip_project<<<dim3(nt, nt), dim3(kFlipTile, 8), 0, c->stream>>>(v, nstr, (float)flip);
      QDKGB_CHECK_LAUNCH();
    };
    d.df_from_f64(d.D, Df);
    sigma_full(V0, sig);
    d.df_from_f64(V0, d.colf(d.Vf, 0));
    d.df_from_f64(sig, d.colf(d.AVf, 0));
    d.df_from_f64(sig, d.colf(d.Vf, 1));
    project(d.colf(d.Vf, 1));
    d.df_gram_schmidt(1, d.colf(d.Vf, 1), 1e-12, true);
    d.df_projected_row(0);
    // residual of the guess (exact): reference level for the first refresh
    d.multidot(sig, 1, V0, Eptr, 1);
    k_axpy_residual<<<d.nb, 256, 0, c->stream>>>(sig, V0, Eptr, Rt, N, d.partial);
    QDKGB_CHECK_LAUNCH();
    k_reduce_partials<<<1, 32, 0, c->stream>>>(d.partial, d.nb, 1, d.small + kSlotRes, 1);
    QDKGB_CHECK_LAUNCH();
    double last_true = 0.;
    d.fetch(d.small + kSlotRes, last_true);
    last_true = std::sqrt(last_true);
    int k = 1;  // valid columns; V[:, k] holds the next direction (its FP32 copy in xf)
    int64_t iter = 0;
    double best = 1e300;
    int since_best = 0;
    bool have_x64 = false;  // d.X holds the FP64 copy of the current Ritz vector
    while (iter < 4 * max_m) {
      spmv_fp32(c, xf, yf);
      loc.spmv_fp32++;
      k_df_from_f32<<<d.nb, 256, 0, c->stream>>>(yf, d.colf(d.AVf, k), N);
      QDKGB_CHECK_LAUNCH();
      d.df_projected_row(k);
      ++k;
      ++iter;
      d.lowest(k);
      float2* R = (k <= max_m - 1) ? d.colf(d.Vf, k) : Rtf;
      d.df_ritz_residual(k, Xf, R, Df, s->min_abs_denominator);
      have_x64 = false;
      double r2 = 0.;
      bool degenerate = false;
      d.fetch3(d.small + kSlotRes, d.eval, r2, lam0, degenerate);
      if (degenerate) {
        --k;
        --iter;
        d.df_fallback(k, d.colf(d.Vf, k));
        continue;
      }
      const double est = std::sqrt(r2);
      loc.iterations = iter;
      if (est < 0.9 * best) {
        best = est;
        since_best = 0;
      } else {
        ++since_best;
      }
      const bool refresh =
          est < 0.5 * s->res_tol || est < drop * last_true || since_best >= 6 || k >= max_m - 1;
      if (!refresh) {
        project(R);
        d.df_gram_schmidt(k, R, 1e-12, true);
        continue;
      }
      // full-precision sigma, Rayleigh quotient and residual of X (unit norm)
      d.df_to_f64(Xf, d.X);
      have_x64 = true;
      sigma_full(d.X, sig);
      d.multidot(sig, 1, d.X, Eptr, 1);
      k_axpy_residual<<<d.nb, 256, 0, c->stream>>>(sig, d.X, Eptr, Rt, N, d.partial);
      QDKGB_CHECK_LAUNCH();
      k_reduce_partials<<<1, 32, 0, c->stream>>>(d.partial, d.nb, 1, d.small + kSlotRes, 1);
      QDKGB_CHECK_LAUNCH();
      d.fetch3(d.small + kSlotRes, Eptr, r2, lam0, degenerate);
      last_true = std::sqrt(r2);
      res = last_true;
      loc.restarts++;
      if (res < s->res_tol) {
        converged = true;
        break;
      }
      // thick restart: V' = V Q[:, 0:kk], AV' = AV Q[:, 0:kk]; column 0 = X with its exact sigma
      const int kk = std::min(kKeep, k);
      d.lowest(k, kk);  // the kk lowest Ritz vectors (column 0 reproduces X)
      if (kk > 1) {
        static_assert(kKeep - 1 <= kMaxOut, "restart block wider than k_df_gemv_multi");
        k_df_gemv_multi<<<d.nb, kVecThreads, 0, c->stream>>>(d.Vf, N, k, d.evec + k, kk - 1, tmpV, N, N);
        QDKGB_CHECK_LAUNCH();
        k_df_gemv_multi<<<d.nb, kVecThreads, 0, c->stream>>>(d.AVf, N, k, d.evec + k, kk - 1, tmpAV, N, N);
        QDKGB_CHECK_LAUNCH();
      }
      QDKGB_CUDA(cudaMemcpyAsync(d.colf(d.Vf, 0), Xf, N * sizeof(float2), cudaMemcpyDeviceToDevice, c->stream));
      d.df_from_f64(sig, d.colf(d.AVf, 0));
      for (int j = 1; j < kk; ++j) {
        QDKGB_CUDA(cudaMemcpyAsync(d.colf(d.Vf, j), tmpV + (size_t)(j - 1) * N, N * sizeof(float2),
                                   cudaMemcpyDeviceToDevice, c->stream));
        QDKGB_CUDA(cudaMemcpyAsync(d.colf(d.AVf, j), tmpAV + (size_t)(j - 1) * N, N * sizeof(float2),
                                   cudaMemcpyDeviceToDevice, c->stream));
      }
      for (int j = 0; j < kk; ++j) d.df_projected_row(j);
      k = kk;
      // next direction: preconditioned true residual
      k_precondition<<<d.nb, 256, 0, c->stream>>>(Rt, d.D, Eptr, N, s->min_abs_denominator);
      QDKGB_CHECK_LAUNCH();
      d.df_from_f64(Rt, d.colf(d.Vf, k));
      project(d.colf(d.Vf, k));
      d.df_gram_schmidt(k, d.colf(d.Vf, k), 1e-12, true);
      best = 1e300;
      since_best = 0;
    }
    if (!have_x64) d.df_to_f64(Xf, d.X);
  }

  QDKGB_CUDA(cudaStreamSynchronize(c->stream));
  *E = lam0;
  if (C) {
    QDKGB_CUDA(cudaMemcpyAsync(C, d.X, N * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    QDKGB_CUDA(cudaStreamSynchronize(c->stream));
  }
  loc.residual_norm = res;
  loc.seconds = std::chrono::duration<double>(clk::now() - t0).count();
  if (info) *info = loc;
  if (!converged) throw Error(QDKGB_ERR_NOT_CONVERGED, "Davidson Did Not Converge!");
}

}  // namespace qdkgb
