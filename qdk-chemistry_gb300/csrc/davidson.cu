// Davidson eigensolver on the device (replaces macis::davidson,
// include/macis/solvers/davidson.hpp:259-372, with gram_schmidt :185-238 and
// lobpcgxx::rayleigh_ritz, lobpcgxx/rayleigh_ritz.hpp:70-77).
//
// Everything except the convergence test runs on the GPU in FP64: the
// subspace V and A*V (column-major, N x (max_m+1)), the projected matrix, its
// eigen-decomposition (one-CTA parallel cyclic Jacobi), the Ritz vector and
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

namespace qdkgb {

constexpr int kDotBlocksPerSm = 2;
constexpr int kMaxSubspace = 256;

// partial[j * nb + blk] = sum over this block's rows of A[:, j] . w
__global__ void k_multidot(const double* __restrict__ A, int64_t lda, int k, const double* __restrict__ w, int64_t n,
                           double* __restrict__ partial) {
  __shared__ double red[32];
  const int j = blockIdx.y;
  const double* a = A + (size_t)j * lda;
  double s = 0.;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    s += a[i] * w[i];
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    double t = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.;
    t = warp_sum(t);
    if (threadIdx.x == 0) partial[(size_t)j * gridDim.x + blockIdx.x] = t;
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
// w -= A[:, 0:k] * coef
__global__ void k_sub_gemv(const double* __restrict__ A, int64_t lda, int k, const double* __restrict__ coef,
                           double* __restrict__ w, int64_t n) {
  __shared__ double c[kMaxSubspace + 2];
  for (int j = threadIdx.x; j < k; j += blockDim.x) c[j] = coef[j];
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.;
    for (int j = 0; j < k; ++j) s += A[i + (size_t)j * lda] * c[j];
    w[i] -= s;
  }
}
// y = A[:, 0:k] * coef (coef strided)
__global__ void k_gemv(const double* __restrict__ A, int64_t lda, int k, const double* __restrict__ coef,
                       int coef_stride, double* __restrict__ y, int64_t n) {
  __shared__ double c[kMaxSubspace + 2];
  for (int j = threadIdx.x; j < k; j += blockDim.x) c[j] = coef[(size_t)j * coef_stride];
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.;
    for (int j = 0; j < k; ++j) s += A[i + (size_t)j * lda] * c[j];
    y[i] = s;
  }
}
// w *= 1/sqrt(*nrm2) when sqrt(*nrm2) > min_norm
__global__ void k_normalize(double* w, int64_t n, const double* nrm2, double min_norm) {
  const double nrm = sqrt(*nrm2);
  if (!(nrm > min_norm)) return;
  const double sc = 1. / nrm;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    w[i] *= sc;
}
// X = V C0, R = AV C0 - lam0 X; partial sums of R^2
__global__ void k_ritz_residual(const double* __restrict__ V, const double* __restrict__ AV, int64_t ld, int k,
                                const double* __restrict__ C0, const double* __restrict__ lam, double* __restrict__ X,
                                double* __restrict__ R, int64_t n, double* __restrict__ partial) {
  __shared__ double c[kMaxSubspace + 2];
  __shared__ double red[32];
  for (int j = threadIdx.x; j < k; j += blockDim.x) c[j] = C0[j];
  __syncthreads();
  const double l0 = lam[0];
  double s2 = 0.;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double x = 0., ax = 0.;
    for (int j = 0; j < k; ++j) {
      x += V[i + (size_t)j * ld] * c[j];
      ax += AV[i + (size_t)j * ld] * c[j];
    }
    const double r = ax - l0 * x;
    X[i] = x;
    R[i] = r;
    s2 += r * r;
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
// R = -R / (D - lam0) with |D - lam0| clamped to min_abs (davidson.hpp:352-361)
__global__ void k_precondition(double* R, const double* __restrict__ D, const double* lam, int64_t n,
                               double min_abs) {
  const double l0 = lam[0];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double d = D[i] - l0;
    if (fabs(d) < min_abs) d = (d >= 0) ? min_abs : -min_abs;
    R[i] = -R[i] / d;
  }
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
// Hk(i, c) = Hk(c, i) = v[c], c <= i
__global__ void k_store_row(const double* v, int i, double* Hk, int ld) {
  for (int c = threadIdx.x; c <= i; c += blockDim.x) {
    Hk[i + (size_t)c * ld] = v[c];
    Hk[c + (size_t)i * ld] = v[c];
  }
}

// ---------------------------------------------------------------- Jacobi
// One CTA: eigen-decomposition of the symmetric k x k matrix H (leading
// dimension ldh; the lower triangle, as syev(Uplo::Lower) reads it, is
// mirrored).  Parallel cyclic Jacobi in round-robin order: each round
// rotates k/2 disjoint (p,q) pairs at once (rows, then columns).  Eigenvalues
// ascending into eval, eigenvectors into evec (k x k, column-major, ld = k).
// The working matrices live in shared memory when they fit, otherwise in
// the global buffers gA / gQ.
__global__ void __launch_bounds__(1024) k_jacobi(int k, const double* __restrict__ H, int ldh, double* gA,
                                                 double* gQ, double* eval, double* evec, int max_sweeps) {
  extern __shared__ double dyn[];
  __shared__ double s_c[kMaxSubspace / 2 + 1], s_s[kMaxSubspace / 2 + 1];
  __shared__ int s_p[kMaxSubspace / 2 + 1], s_q[kMaxSubspace / 2 + 1];
  __shared__ double red[32];
  __shared__ int rank_of[kMaxSubspace];
  __shared__ int s_done;
  double* A = gA ? gA : dyn;
  double* Q = gA ? gQ : dyn + (size_t)k * k;
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int t = tid; t < k * k; t += nt) {
    const int i = t % k, j = t / k;
    const double lowv = (i >= j) ? H[i + (size_t)j * ldh] : H[j + (size_t)i * ldh];
    A[t] = lowv;
    Q[t] = (i == j) ? 1. : 0.;
  }
  __syncthreads();
  const int m = k + (k & 1);
  const int np = m / 2;
  for (int sweep = 0; sweep < max_sweeps; ++sweep) {
    double off = 0., tot = 0.;
    for (int t = tid; t < k * k; t += nt) {
      const double v = A[t] * A[t];
      tot += v;
      if (t % k != t / k) off += v;
    }
    off = warp_sum(off);
    tot = warp_sum(tot);
    if ((tid & 31) == 0) {
      red[tid >> 5] = off;
    }
    __syncthreads();
    if (tid == 0) {
      double o = 0.;
      for (int w = 0; w < (nt >> 5); ++w) o += red[w];
      red[31] = o;
    }
    __syncthreads();
    const double off_all = red[31];
    __syncthreads();
    if ((tid & 31) == 0) red[tid >> 5] = tot;
    __syncthreads();
    if (tid == 0) {
      double o = 0.;
      for (int w = 0; w < (nt >> 5); ++w) o += red[w];
      s_done = !(off_all > 1e-30 * o) ? 1 : 0;
    }
    __syncthreads();
    if (s_done) break;
    for (int round = 0; round < m - 1; ++round) {
      for (int i = tid; i < np; i += nt) {
        int p, q;
        if (i == 0) {
          p = round;
          q = m - 1;
        } else {
          p = (round + i) % (m - 1);
          q = (round - i + (m - 1)) % (m - 1);
        }
        if (p > q) {
          const int t = p;
          p = q;
          q = t;
        }
        double c = 1., s = 0.;
        if (q < k) {
          const double apq = A[p + (size_t)k * q];
          if (apq != 0.) {
            const double app = A[p + (size_t)k * p], aqq = A[q + (size_t)k * q];
            const double theta = (aqq - app) / (2. * apq);
            const double t = (theta >= 0 ? 1. : -1.) / (fabs(theta) + sqrt(theta * theta + 1.));
            c = 1. / sqrt(t * t + 1.);
            s = t * c;
          }
        }
        s_p[i] = p;
        s_q[i] = (q < k) ? q : -1;
        s_c[i] = c;
        s_s[i] = s;
      }
      __syncthreads();
      // rows p, q:  A[p][j] = c A[p][j] - s A[q][j];  A[q][j] = s A[p][j] + c A[q][j]
      for (int t = tid; t < np * k; t += nt) {
        const int i = t / k, j = t % k;
        const int q = s_q[i];
        if (q < 0 || s_s[i] == 0.) continue;
        const int p = s_p[i];
        const double c = s_c[i], s = s_s[i];
        const double apj = A[p + (size_t)k * j], aqj = A[q + (size_t)k * j];
        A[p + (size_t)k * j] = c * apj - s * aqj;
        A[q + (size_t)k * j] = s * apj + c * aqj;
      }
      __syncthreads();
      // columns p, q of A and Q
      for (int t = tid; t < np * k; t += nt) {
        const int i = t / k, j = t % k;
        const int q = s_q[i];
        if (q < 0 || s_s[i] == 0.) continue;
        const int p = s_p[i];
        const double c = s_c[i], s = s_s[i];
        const double ajp = A[j + (size_t)k * p], ajq = A[j + (size_t)k * q];
        A[j + (size_t)k * p] = c * ajp - s * ajq;
        A[j + (size_t)k * q] = s * ajp + c * ajq;
        const double qjp = Q[j + (size_t)k * p], qjq = Q[j + (size_t)k * q];
        Q[j + (size_t)k * p] = c * qjp - s * qjq;
        Q[j + (size_t)k * q] = s * qjp + c * qjq;
      }
      __syncthreads();
    }
  }
  // ascending order, ties by index
  for (int t = tid; t < k; t += nt) {
    const double lt = A[t + (size_t)k * t];
    int r = 0;
    for (int j = 0; j < k; ++j) {
      const double lj = A[j + (size_t)k * j];
      r += (lj < lt) || (lj == lt && j < t);
    }
    rank_of[t] = r;
  }
  __syncthreads();
  for (int t = tid; t < k; t += nt) eval[rank_of[t]] = A[t + (size_t)k * t];
  for (int t = tid; t < k * k; t += nt) {
    const int i = t % k, j = t / k;
    evec[i + (size_t)k * rank_of[j]] = Q[i + (size_t)k * j];
  }
}

// ---------------------------------------------------------------- driver
namespace {

struct Dav {
  Context* c;
  int64_t n;
  int64_t maxm;
  double *V, *AV, *D, *X, *Hk, *evec, *eval, *partial, *small, *work;
  float *xf, *yf;
  int nb;  // blocks for dot products / vector kernels
  double* gA = nullptr;
  double* gQ = nullptr;
  cudaStream_t st;

  double* col(double* base, int64_t j) { return base + (size_t)j * n; }

  // out[j*stride] = A[:, j] . w, j < k
  void multidot(const double* A, int k, const double* w, double* out, int stride) {
    dim3 g(nb, k);
    k_multidot<<<g, 256, 0, st>>>(A, n, k, w, n, partial);
    QDKGB_CHECK_LAUNCH();
    k_reduce_partials<<<(k + 7) / 8, 256, 0, st>>>(partial, nb, k, out, stride);
    QDKGB_CHECK_LAUNCH();
  }
  // squared norm of w into *out (device)
  void norm2(const double* w, double* out) { multidot(w, 1, w, out, 1); }

  double fetch(const double* dptr) {
    QDKGB_CUDA(cudaMemcpyAsync(c->pinned, dptr, sizeof(double), cudaMemcpyDeviceToHost, st));
    QDKGB_CUDA(cudaStreamSynchronize(st));
    return c->pinned[0];
  }
  void fetch2(const double* a, const double* b, double& va, double& vb) {
    QDKGB_CUDA(cudaMemcpyAsync(c->pinned, a, sizeof(double), cudaMemcpyDeviceToHost, st));
    QDKGB_CUDA(cudaMemcpyAsync(c->pinned + 1, b, sizeof(double), cudaMemcpyDeviceToHost, st));
    QDKGB_CUDA(cudaStreamSynchronize(st));
    va = c->pinned[0];
    vb = c->pinned[1];
  }

  // gram_schmidt (davidson.hpp:185-238): w against V[:, 0:K], twice; normalise.
  void gram_schmidt(int K, double* w, double min_norm = 1e-12) {
    double* inner = small;  // K doubles
    if (K > 0) {
      for (int pass = 0; pass < 2; ++pass) {
        multidot(V, K, w, inner, 1);
        k_sub_gemv<<<nb, 256, 0, st>>>(V, n, K, inner, w, n);
        QDKGB_CHECK_LAUNCH();
      }
    }
    double* nrm2 = small + kMaxSubspace + 8;
    norm2(w, nrm2);
    const double nv = std::sqrt(fetch(nrm2));
    if (nv > min_norm) {
      k_normalize<<<nb, 256, 0, st>>>(w, n, nrm2, min_norm);
      QDKGB_CHECK_LAUNCH();
      return;
    }
    // canonical-vector fallback
    for (int64_t idx = 0; idx < n; ++idx) {
      QDKGB_CUDA(cudaMemsetAsync(w, 0, n * sizeof(double), st));
      const double one = 1.0;
      QDKGB_CUDA(cudaMemcpyAsync(w + idx, &one, sizeof(double), cudaMemcpyHostToDevice, st));
      for (int pass = 0; pass < 2 && K > 0; ++pass) {
        multidot(V, K, w, inner, 1);
        k_sub_gemv<<<nb, 256, 0, st>>>(V, n, K, inner, w, n);
        QDKGB_CHECK_LAUNCH();
      }
      norm2(w, nrm2);
      if (std::sqrt(fetch(nrm2)) > min_norm) {
        k_normalize<<<nb, 256, 0, st>>>(w, n, nrm2, min_norm);
        QDKGB_CHECK_LAUNCH();
        return;
      }
    }
    throw Error(QDKGB_ERR_INVALID, "gram_schmidt: Unable to find orthogonal vector");
  }

  void jacobi(int k) {
    const size_t need = 2ull * k * k * sizeof(double);
    const bool in_smem = need <= 200 * 1024;
    const int threads = k <= 32 ? 256 : 1024;
    k_jacobi<<<1, threads, in_smem ? need : 0, st>>>(k, Hk, (int)(maxm + 1), in_smem ? nullptr : gA, gQ, eval, evec,
                                                     60);
    QDKGB_CHECK_LAUNCH();
  }

  // new row i of the projected matrix: Hk(i, c) = V_i . AV_c, c <= i (+ mirror)
  void projected_row(int i) {
    multidot(AV, i + 1, col(V, i), small, 1);
    k_store_row<<<1, 256, 0, st>>>(small, i, Hk, (int)(maxm + 1));
    QDKGB_CHECK_LAUNCH();
  }

  // X = V C0, R = AV C0 - lam0 X; returns |R|
  double ritz_residual(int k, double* R) {
    k_ritz_residual<<<nb, 256, 0, st>>>(V, AV, n, k, evec, eval, X, R, n, partial);
    QDKGB_CHECK_LAUNCH();
    k_reduce_partials<<<1, 32, 0, st>>>(partial, nb, 1, small + kMaxSubspace + 4, 1);
    QDKGB_CHECK_LAUNCH();
    return std::sqrt(fetch(small + kMaxSubspace + 4));
  }
};

}  // namespace

void davidson(Context* c, const qdkgb_davidson_settings* s, double* E, double* C, qdkgb_davidson_info* info) {
  using clk = std::chrono::steady_clock;
  const auto t0 = clk::now();
  Hcsr& H = c->H;
  if (!H.valid) throw Error(QDKGB_ERR_STATE, "Hamiltonian not built");
  const int64_t N = H.n;
  const bool mixed = s->precision == QDKGB_PREC_MIXED;
  if (mixed && H.storage != QDKGB_H_SPLIT32)
    throw Error(QDKGB_ERR_STATE, "mixed precision needs the Hamiltonian built with QDKGB_H_SPLIT32 storage");
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
  d.nb = std::min<int64_t>((N + 255) / 256, (int64_t)c->sm_count * kDotBlocksPerSm);
  d.nb = std::max(d.nb, 1);
  d.V = dev_array<double>(c, W.V, (size_t)N * (max_m + 1));
  d.AV = dev_array<double>(c, W.AV, (size_t)N * (max_m + 1));
  d.X = dev_array<double>(c, W.scratch, (size_t)N * 8);
  d.work = d.X + N;
  d.Hk = dev_array<double>(c, W.Hk, (size_t)(max_m + 1) * (max_m + 1));
  d.evec = dev_array<double>(c, W.evec, (size_t)(max_m + 1) * (max_m + 1));
  d.eval = dev_array<double>(c, W.eval, (size_t)(max_m + 1));
  d.partial = dev_array<double>(c, W.partial, (size_t)d.nb * (kMaxSubspace + 2));
  d.small = dev_array<double>(c, W.small, 4 * kMaxSubspace);
  if (2ull * (max_m + 1) * (max_m + 1) * 8 > 200 * 1024) {
    d.gA = dev_array<double>(c, W.yf, 2ull * (max_m + 1) * (max_m + 1));
    d.gQ = d.gA + (size_t)(max_m + 1) * (max_m + 1);
  }
  static bool attr_set = false;
  if (!attr_set) {
    QDKGB_CUDA(cudaFuncSetAttribute(k_jacobi, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    attr_set = true;
  }
  d.D = (double*)H.diag.ptr;
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
  auto sigma_sub = [&](const double* x, double* y) {
    if (!mixed) {
      sigma_full(x, y);
      return;
    }
    f64_to_f32(c, x, xf, N);
    spmv_fp32(c, xf, yf);
    f32_to_f64(c, yf, y, N);
    loc.spmv_fp32++;
  };

  // guess (selected_ci_diag.hpp:130-140)
  double* V0 = d.V;
  bool use_c = false;
  if (s->use_guess && C) {
    double mx = 0.;
    for (int64_t i = 0; i < N; ++i) mx = std::max(mx, std::fabs(C[i]));
    use_c = mx > 1. / (double)N;
  }
  if (use_c) {
    QDKGB_CUDA(cudaMemcpyAsync(V0, C, N * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  } else {
    int64_t* idx = (int64_t*)(d.small + 3 * kMaxSubspace);
    k_argmin<<<1, 1024, 0, c->stream>>>(d.D, N, idx);
    QDKGB_CHECK_LAUNCH();
    k_set_onehot<<<d.nb, 256, 0, c->stream>>>(V0, N, idx);
    QDKGB_CHECK_LAUNCH();
  }

  if (N == 1) {
    // davidson.hpp:280-288: evaluate the 1x1 operator on X = [1]
    k_set_value<<<1, 1, 0, c->stream>>>(V0, 1.0);
    sigma_full(V0, d.AV);
    *E = d.fetch(d.AV);
    if (C) C[0] = 1.0;
    loc.residual_norm = 0.;
    loc.seconds = std::chrono::duration<double>(clk::now() - t0).count();
    if (info) *info = loc;
    return;
  }

  double lam0 = 0., res = 0.;
  bool converged = false;
  double* nrm2 = d.small + kMaxSubspace + 8;

  if (!mixed) {
    // ---------------- plain FP64 Davidson, the reference's algorithm
    sigma_full(V0, d.AV);
    QDKGB_CUDA(cudaMemcpyAsync(d.col(d.V, 1), d.AV, N * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    d.gram_schmidt(1, d.col(d.V, 1));
    d.multidot(d.AV, 1, V0, d.Hk, 1);  // Hk(0,0)
    int64_t iter = 1;
    for (int64_t i = 1; i < max_m; ++i, ++iter) {
      const int k = (int)i + 1;
      sigma_full(d.col(d.V, i), d.col(d.AV, i));
      d.projected_row((int)i);
      d.jacobi(k);
      double* R = d.col(d.V, i + 1);
      res = d.ritz_residual(k, R);
      lam0 = d.fetch(d.eval);
      loc.iterations = iter;
      if (res < s->res_tol) {
        converged = true;
        break;
      }
      k_precondition<<<d.nb, 256, 0, c->stream>>>(R, d.D, d.eval, N, s->min_abs_denominator);
      QDKGB_CHECK_LAUNCH();
      d.gram_schmidt(k, R);
    }
  } else {
    // ---------------- mixed: FP32 sigma for new directions, full-precision refresh
    const double refresh_ratio = 1e-4;
    const int keep = 3;
    double* sig = d.work;         // full-precision sigma of the current Ritz vector
    double* Rt = d.work + N;      // full-precision residual
    double* tmpV = d.work + 2 * N;               // keep-1 rotated V columns
    double* tmpAV = d.work + (2 + keep - 1) * N; // keep-1 rotated AV columns
    double* Eptr = d.small + kMaxSubspace + 12;
    // column 0 = guess with its exact sigma
    sigma_full(V0, d.AV);
    d.multidot(d.AV, 1, V0, d.Hk, 1);
    k_axpy_residual<<<d.nb, 256, 0, c->stream>>>(d.AV, V0, d.Hk, Rt, N, d.partial);
    QDKGB_CHECK_LAUNCH();
    k_reduce_partials<<<1, 32, 0, c->stream>>>(d.partial, d.nb, 1, nrm2, 1);
    QDKGB_CHECK_LAUNCH();
    double last_true = std::sqrt(d.fetch(nrm2));
    lam0 = d.fetch(d.Hk);
    res = last_true;
    QDKGB_CUDA(cudaMemcpyAsync(d.X, V0, N * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    int k = 1;
    if (res < s->res_tol) converged = true;
    auto next_from_true_residual = [&]() {
      QDKGB_CUDA(cudaMemcpyAsync(d.col(d.V, k), Rt, N * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
      QDKGB_CUDA(cudaMemcpyAsync(d.eval, d.Hk, sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
      k_precondition<<<d.nb, 256, 0, c->stream>>>(d.col(d.V, k), d.D, Eptr, N, s->min_abs_denominator);
      QDKGB_CHECK_LAUNCH();
      d.gram_schmidt(k, d.col(d.V, k));
    };
    QDKGB_CUDA(cudaMemcpyAsync(Eptr, d.Hk, sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    if (!converged) next_from_true_residual();
    int64_t iter = 0;
    double prev_est = 1e300;
    int stall = 0;
    while (!converged && iter < 4 * max_m) {
      // expand with column k (orthonormal, already in V[:, k])
      sigma_sub(d.col(d.V, k), d.col(d.AV, k));
      d.projected_row(k);
      ++k;
      ++iter;
      d.jacobi(k);
      double* R = (k <= max_m - 1) ? d.col(d.V, k) : Rt;
      const double est = d.ritz_residual(k, R);
      lam0 = d.fetch(d.eval);
      loc.iterations = iter;
      stall = (est > 0.7 * prev_est) ? stall + 1 : 0;
      prev_est = std::min(prev_est, est);
      const bool refresh =
          est < refresh_ratio * last_true || est < 0.5 * s->res_tol || stall >= 4 || k >= max_m - 1;
      if (!refresh) {
        k_precondition<<<d.nb, 256, 0, c->stream>>>(R, d.D, d.eval, N, s->min_abs_denominator);
        QDKGB_CHECK_LAUNCH();
        d.gram_schmidt(k, R);
        continue;
      }
      // full-precision sigma, energy and residual of the Ritz vector X (unit norm)
      sigma_full(d.X, sig);
      d.multidot(sig, 1, d.X, Eptr, 1);
      k_axpy_residual<<<d.nb, 256, 0, c->stream>>>(sig, d.X, Eptr, Rt, N, d.partial);
      QDKGB_CHECK_LAUNCH();
      k_reduce_partials<<<1, 32, 0, c->stream>>>(d.partial, d.nb, 1, nrm2, 1);
      QDKGB_CHECK_LAUNCH();
      d.fetch2(nrm2, Eptr, last_true, lam0);
      last_true = std::sqrt(last_true);
      res = last_true;
      loc.restarts++;
      if (res < s->res_tol) {
        converged = true;
        break;
      }
      // thick restart on the `keep` lowest Ritz vectors: V' = V Q[:, 0:keep],
      // AV' = AV Q[:, 0:keep]; column 0 = X with its exact sigma.
      const int kk = std::min(keep, k);
      for (int j = 1; j < kk; ++j) {
        k_gemv<<<d.nb, 256, 0, c->stream>>>(d.V, N, k, d.evec + (size_t)j * k, 1, tmpV + (size_t)(j - 1) * N, N);
        QDKGB_CHECK_LAUNCH();
        k_gemv<<<d.nb, 256, 0, c->stream>>>(d.AV, N, k, d.evec + (size_t)j * k, 1, tmpAV + (size_t)(j - 1) * N, N);
        QDKGB_CHECK_LAUNCH();
      }
      QDKGB_CUDA(cudaMemcpyAsync(d.col(d.V, 0), d.X, N * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
      QDKGB_CUDA(cudaMemcpyAsync(d.col(d.AV, 0), sig, N * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
      for (int j = 1; j < kk; ++j) {
        QDKGB_CUDA(cudaMemcpyAsync(d.col(d.V, j), tmpV + (size_t)(j - 1) * N, N * sizeof(double),
                                   cudaMemcpyDeviceToDevice, c->stream));
        QDKGB_CUDA(cudaMemcpyAsync(d.col(d.AV, j), tmpAV + (size_t)(j - 1) * N, N * sizeof(double),
                                   cudaMemcpyDeviceToDevice, c->stream));
      }
      for (int j = 0; j < kk; ++j) d.projected_row(j);
      k = kk;
      next_from_true_residual();
      prev_est = 1e300;
      stall = 0;
    }
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
