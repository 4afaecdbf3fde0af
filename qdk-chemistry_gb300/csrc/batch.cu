// Batched CASCI: many independent complete active spaces solved together.
//
// The reference solves such a set one instance at a time (MacisCas::run per
// active space, qdk_chemistry/algorithms/microsoft/macis_cas.cpp:35-117).
// Here instances are grouped by shape (norb, n_alpha, n_beta); a shape's
// determinant space, string connectivity and slab tables are built once, and
// every step of the solve is one launch over all instances of the shape:
//   * per-instance integral intermediates and diagonals;
//   * the slab emission (grid.z = instance) of every instance's Hamiltonian;
//   * a mixed-precision Davidson in lockstep: FP32 sigma for new directions,
//     FP64 subspace, Gram-Schmidt (CGS2), Rayleigh-Ritz (one CTA per instance)
//     and residuals; each cycle starts from the Ritz vector with its sigma in
//     full precision (float-float from the split storage) and a convergence
//     test on the full-precision residual; an instance whose estimated
//     residual fell by 1e-4 since its last full-precision one (or whose
//     subspace is full) waits for the next cycle, a converged one drops out
//     of every launch;
//   * the inner iteration (a fixed launch sequence reading the subspace size
//     from device memory) is captured once as a CUDA graph and replayed;
//   * spin-summed 1-RDMs of the converged vectors.
// Sub-batches bound the device memory of the stored matrices.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <tuple>
#include <vector>

#include "batch_kernels.cuh"
#include "common.cuh"
#include "internal.h"

namespace qdkgb {

void build_integral_intermediates_into(Context* c, int n, const double* V, double* G, double* Vr, double* G2,
                                       double* V2);

namespace {

constexpr int kBT = 256;           // threads of the vector kernels
constexpr int kChunk = kBT * 8;    // elements per CTA in the reductions
constexpr int kMaxB = 1 << 16;     // instances per shape and sub-batch

__device__ double bsum(double v, double* red) {
  v = warp_sum(v);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) red[w] = v;
  __syncthreads();
  double t = 0.;
  if (threadIdx.x < 32) {
    t = (lane < (int)(blockDim.x >> 5)) ? red[lane] : 0.;
    t = warp_sum(t);
  }
  return t;  // valid in thread 0
}

// partial[b][chunk][j] = sum over the chunk of A[b][j][i] * w[b][i], j < kk,
// kk = *kdev + kadd (kdev may be null: kk = kadd).  w is offset by
// (*kdev) * wk_ld when wk_ld != 0 (the newest column of a stacked basis).
__global__ void __launch_bounds__(kBT)
    k_b_multidot(const double* __restrict__ A, int64_t astride, int64_t ld, const int* __restrict__ kdev, int kadd,
                 const double* __restrict__ w, int64_t wstride, int64_t wk_ld, int64_t n, int nchunk,
                 double* __restrict__ partial, int KM, const int* __restrict__ mask) {
  __shared__ double red[33];
  const int b = blockIdx.y;
  if (mask && !mask[b]) return;
  const int kk = (kdev ? *kdev : 0) + kadd;
  const int64_t i0 = (int64_t)blockIdx.x * kChunk;
  const double* Ab = A + b * astride;
  const double* wb = w + b * wstride + (wk_ld && kdev ? (int64_t)(*kdev) * wk_ld : 0);
  double wv[kChunk / kBT];
#pragma unroll
  for (int t = 0; t < kChunk / kBT; ++t) {
    const int64_t i = i0 + threadIdx.x + (int64_t)t * kBT;
    wv[t] = i < n ? wb[i] : 0.;
  }
  for (int j = 0; j < kk; ++j) {
    double acc = 0.;
#pragma unroll
    for (int t = 0; t < kChunk / kBT; ++t) {
      const int64_t i = i0 + threadIdx.x + (int64_t)t * kBT;
      if (i < n) acc += Ab[j * ld + i] * wv[t];
    }
    acc = bsum(acc, red);
    if (threadIdx.x == 0) partial[((int64_t)b * nchunk + blockIdx.x) * KM + j] = acc;
  }
}

// out[b][j] = sum over chunks in order (deterministic)
__global__ void k_b_reduce(const double* __restrict__ partial, int nchunk, int KM, const int* __restrict__ kdev,
                           int kadd, double* __restrict__ out, int64_t ostride, const int* __restrict__ mask) {
  const int b = blockIdx.x;
  if (mask && !mask[b]) return;
  const int kk = (kdev ? *kdev : 0) + kadd;
  for (int j = threadIdx.x; j < kk; j += blockDim.x) {
    double s = 0.;
    for (int c = 0; c < nchunk; ++c) s += partial[((int64_t)b * nchunk + c) * KM + j];
    out[b * ostride + j] = s;
  }
}

// y[b] = (w ? w[b] : 0) + alpha * sum_{j < kk} A[b][j] c[b][j]
__global__ void __launch_bounds__(kBT)
    k_b_gemv(const double* __restrict__ A, int64_t astride, int64_t ld, const int* __restrict__ kdev, int kadd,
             const double* __restrict__ c, int KM, double alpha, const double* w, double* y, int64_t vstride,
             int64_t n, const int* __restrict__ mask) {
  const int b = blockIdx.y;
  if (mask && !mask[b]) return;
  const int kk = (kdev ? *kdev : 0) + kadd;
  const double* Ab = A + b * astride;
  const double* cb = c + (int64_t)b * KM;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double acc = 0.;
    for (int j = 0; j < kk; ++j) acc += Ab[j * ld + i] * cb[j];
    y[b * vstride + i] = (w ? w[b * vstride + i] : 0.) + alpha * acc;
  }
}

// x = V y (the previous x kept in xprev), ax = AV y, r = ax - theta x;
// partial |r|^2 per chunk
__global__ void __launch_bounds__(kBT)
    k_b_ritz(const double* __restrict__ Vb, const double* __restrict__ AVb, int64_t astride, int64_t ld,
             const int* __restrict__ kdev, const double* __restrict__ yv, int KM, const double* __restrict__ theta,
             double* __restrict__ x, double* __restrict__ xprev, double* __restrict__ ax, double* __restrict__ r,
             int64_t n, int nchunk, double* __restrict__ partial, const int* __restrict__ mask) {
  __shared__ double red[33];
  const int b = blockIdx.y;
  if (mask && !mask[b]) return;
  const int kk = *kdev;
  const double th = theta[b];
  const double* yb = yv + (int64_t)b * KM;
  const int64_t i0 = (int64_t)blockIdx.x * kChunk;
  double acc = 0.;
  for (int t = 0; t < kChunk / kBT; ++t) {
    const int64_t i = i0 + threadIdx.x + (int64_t)t * kBT;
    if (i >= n) break;
    double sx = 0., sa = 0.;
    for (int j = 0; j < kk; ++j) {
      sx += Vb[b * astride + j * ld + i] * yb[j];
      sa += AVb[b * astride + j * ld + i] * yb[j];
    }
    const double rr = sa - th * sx;
    xprev[b * n + i] = x[b * n + i];
    x[b * n + i] = sx;
    ax[b * n + i] = sa;
    r[b * n + i] = rr;
    acc += rr * rr;
  }
  acc = bsum(acc, red);
  if (threadIdx.x == 0) partial[(int64_t)b * nchunk + blockIdx.x] = acc;
}

// t = -r / (D - theta), |D - theta| clamped below by min_abs (davidson.hpp:106-113)
__global__ void k_b_precond(const double* __restrict__ r, const double* __restrict__ D,
                            const double* __restrict__ theta, double* __restrict__ t, int64_t n, double min_abs,
                            const int* __restrict__ mask) {
  const int b = blockIdx.y;
  if (mask && !mask[b]) return;
  const double th = theta[b];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double d = D[b * n + i] - th;
    if (fabs(d) < min_abs) d = (d >= 0) ? min_abs : -min_abs;
    t[b * n + i] = -r[b * n + i] / d;
  }
}

// projection on the spin-flip sector flip[b] = +-1 (0: none) of an
// nstr x nstr coefficient matrix, pairwise in place
__global__ void k_b_flip(double* __restrict__ t, int64_t nstr, const double* __restrict__ flip,
                         const int* __restrict__ mask) {
  const int b = blockIdx.y;
  if (mask && !mask[b]) return;
  const double s = flip[b];
  if (s == 0.) return;
  double* x = t + b * nstr * nstr;
  const int64_t total = nstr * nstr;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = q / nstr, j = q % nstr;
    if (i < j) {
      const double avg = 0.5 * (x[i * nstr + j] + s * x[j * nstr + i]);
      x[i * nstr + j] = avg;
      x[j * nstr + i] = s * avg;
    } else if (i == j && s < 0) {
      x[q] = 0.;
    }
  }
}

// V[b][k] = t = t / |t|, t32 = float(t); |t| ~ 0 stops the instance's cycle
__global__ void k_b_store_dir(double* __restrict__ t, const double* __restrict__ nrm2, double* __restrict__ Vb,
                              int64_t astride, int64_t ld, const int* __restrict__ kdev, float* __restrict__ t32,
                              int64_t n, int* __restrict__ act, int* __restrict__ nsig) {
  const int b = blockIdx.y;
  if (!act[b]) return;
  const double nn = nrm2[(int64_t)b * 2];
  if (!(nn > 1e-28)) {
    if (blockIdx.x == 0 && threadIdx.x == 0) act[b] = 0;  // no new direction: wait for the cycle's end
    return;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) nsig[b] += 1;
  const double inv = 1. / sqrt(nn);
  double* v = Vb + b * astride + (int64_t)(*kdev) * ld;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double q = t[b * n + i] * inv;
    v[i] = q;
    t[b * n + i] = q;
    t32[b * n + i] = __double2float_rn(q);
  }
}

__global__ void k_b_f32_to_col(const float* __restrict__ s32, double* __restrict__ AVb, int64_t astride, int64_t ld,
                               const int* __restrict__ kdev, int64_t n, const int* __restrict__ mask) {
  const int b = blockIdx.y;
  if (mask && !mask[b]) return;
  double* a = AVb + b * astride + (int64_t)(*kdev) * ld;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    a[i] = (double)s32[b * n + i];
}

__global__ void k_b_f64_to_col(const double* __restrict__ y, double* __restrict__ AVb, int64_t astride, int64_t ld,
                               const int* __restrict__ kdev, int64_t n, const int* __restrict__ mask) {
  const int b = blockIdx.y;
  if (mask && !mask[b]) return;
  double* a = AVb + b * astride + (int64_t)(*kdev) * ld;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    a[i] = y[b * n + i];
}

// row k of the projected matrix, Hs(k, j) = coef[j], j <= k (lower triangle)
__global__ void k_b_hsrow(const double* __restrict__ coef, int KM, double* __restrict__ Hs, int m,
                          const int* __restrict__ kdev, const int* __restrict__ mask) {
  const int b = blockIdx.x;
  if (mask && !mask[b]) return;
  const int k = *kdev;
  for (int j = threadIdx.x; j <= k; j += blockDim.x) Hs[(int64_t)b * m * m + k + (int64_t)j * m] = coef[(int64_t)b * KM + j];
}

__global__ void k_b_kinc(int* kdev) { *kdev += 1; }

// second Gram-Schmidt pass where the first removed more than half of |t|^2
__global__ void k_b_need2(int B, const int* __restrict__ act, const double* __restrict__ nrm2,
                          const double* __restrict__ w0, int* __restrict__ need2) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < B) need2[b] = act[b] && !(nrm2[(int64_t)b * 2] > 0.5 * w0[b]);
}

// after the Ritz step: an instance waits for the next cycle when its
// estimated residual fell by `ratio` since its last full-precision one, or
// its subspace is full; nact = active instances (for the host)
__global__ void k_b_wait(int B, const double* __restrict__ est2, const double* __restrict__ last_true, double ratio,
                         const int* __restrict__ kdev, int m, int* __restrict__ act, int* __restrict__ nact) {
  __shared__ int cnt;
  if (threadIdx.x == 0) cnt = 0;
  __syncthreads();
  const bool full = *kdev >= m;
  int c = 0;
  for (int b = threadIdx.x; b < B; b += blockDim.x) {
    if (!act[b]) continue;
    if (full || sqrt(est2[(int64_t)b * 2]) < ratio * last_true[b]) act[b] = 0;
    else ++c;
  }
  atomicAdd(&cnt, c);
  __syncthreads();
  if (threadIdx.x == 0) *nact = cnt;
}

// refresh: x <- x / |x| into V[b][0] and the packed x; split pair (xh, xl)
__global__ void k_b_refresh_x(double* __restrict__ x, const double* __restrict__ nrm2, int ns,
                              double* __restrict__ Vb, int64_t astride, float* __restrict__ xh,
                              float* __restrict__ xl, int64_t n, const int* __restrict__ mask) {
  const int b = blockIdx.y;
  if (mask && !mask[b]) return;
  const double inv = 1. / sqrt(nrm2[(int64_t)b * ns]);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double q = x[b * n + i] * inv;
    x[b * n + i] = q;
    Vb[b * astride + i] = q;
    const float h = __double2float_rn(q);
    xh[b * n + i] = h;
    xl[b * n + i] = __double2float_rn(q - (double)h);
  }
}

// r = ax - theta x (theta = x.ax), AV[b][0] = ax; partial |r|^2
__global__ void __launch_bounds__(kBT)
    k_b_refresh_res(const double* __restrict__ x, const double* __restrict__ ax, const double* __restrict__ th2,
                    double* __restrict__ AVb, int64_t astride, double* __restrict__ r, int64_t n, int nchunk,
                    double* __restrict__ partial, const int* __restrict__ mask) {
  __shared__ double red[33];
  const int b = blockIdx.y;
  if (mask && !mask[b]) return;
  const double th = th2[(int64_t)b * 2];
  const int64_t i0 = (int64_t)blockIdx.x * kChunk;
  double acc = 0.;
  for (int t = 0; t < kChunk / kBT; ++t) {
    const int64_t i = i0 + threadIdx.x + (int64_t)t * kBT;
    if (i >= n) break;
    const double a = ax[b * n + i];
    AVb[b * astride + i] = a;
    const double rr = a - th * x[b * n + i];
    r[b * n + i] = rr;
    acc += rr * rr;
  }
  acc = bsum(acc, red);
  if (threadIdx.x == 0) partial[(int64_t)b * nchunk + blockIdx.x] = acc;
}

// GD+1 restart: partial sums of x.v and v.v for the candidates
// v = xprev, r, filler (six sums per chunk)
__global__ void __launch_bounds__(kBT)
    k_b_second_dots(const double* __restrict__ x, const double* __restrict__ xprev, const double* __restrict__ r,
                    int64_t n, int64_t nstr, const double* __restrict__ flip, int nchunk, double* __restrict__ partial,
                    const int* __restrict__ mask) {
  __shared__ double red[33];
  const int b = blockIdx.y;
  if (mask && !mask[b]) return;
  const double fs = flip ? flip[b] : 0.;
  const int64_t i0 = (int64_t)blockIdx.x * kChunk;
  double a[6] = {0., 0., 0., 0., 0., 0.};
  for (int t = 0; t < kChunk / kBT; ++t) {
    const int64_t i = i0 + threadIdx.x + (int64_t)t * kBT;
    if (i >= n) break;
    const double xi = x[b * n + i], p = xprev[b * n + i], q = r[b * n + i], z = filler(i, nstr, fs);
    a[0] += xi * p;
    a[1] += p * p;
    a[2] += xi * q;
    a[3] += q * q;
    a[4] += xi * z;
    a[5] += z * z;
  }
  for (int j = 0; j < 6; ++j) {
    const double v = bsum(a[j], red);
    if (threadIdx.x == 0) partial[((int64_t)b * nchunk + blockIdx.x) * 6 + j] = v;
  }
}

// V[b][1] = (v - (x.v) x) / |.| for the first candidate that keeps a 1e-4
// relative norm (x is unit); its split pair into (h2, l2)
__global__ void k_b_second_set(const double* __restrict__ x, const double* __restrict__ xprev,
                               const double* __restrict__ r, const double* __restrict__ dots, double* __restrict__ Vb,
                               int64_t astride, int64_t ld, float* __restrict__ h2, float* __restrict__ l2, int64_t n,
                               int64_t nstr, const double* __restrict__ flip, const int* __restrict__ mask) {
  const int b = blockIdx.y;
  if (mask && !mask[b]) return;
  const double fs = flip ? flip[b] : 0.;
  const double* d = dots + (int64_t)b * 6;
  int pick = 2;
  double nrm2 = d[5] - d[4] * d[4];
  if (d[1] - d[0] * d[0] > 1e-8 * d[1]) {
    pick = 0;
    nrm2 = d[1] - d[0] * d[0];
  } else if (d[3] - d[2] * d[2] > 1e-8 * d[3]) {
    pick = 1;
    nrm2 = d[3] - d[2] * d[2];
  }
  const double c = d[2 * pick], inv = 1. / sqrt(nrm2);
  double* v1 = Vb + b * astride + ld;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double v = pick == 0 ? xprev[b * n + i] : (pick == 1 ? r[b * n + i] : filler(i, nstr, fs));
    const double q = (v - c * x[b * n + i]) * inv;
    v1[i] = q;
    const float h = __double2float_rn(q);
    h2[b * n + i] = h;
    l2[b * n + i] = __double2float_rn(q - (double)h);
  }
}

__global__ void k_b_col_to_packed(const double* __restrict__ Vb, int64_t astride, int64_t ld, int col,
                                  double* __restrict__ y, int64_t n, const int* __restrict__ mask) {
  const int b = blockIdx.y;
  if (mask && !mask[b]) return;
  const double* v = Vb + b * astride + (int64_t)col * ld;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[b * n + i] = v[i];
}

__global__ void k_b_copy_col(const double* __restrict__ y, double* __restrict__ AVb, int64_t astride, int64_t ld,
                             int col, int64_t n, const int* __restrict__ mask) {
  const int b = blockIdx.y;
  if (mask && !mask[b]) return;
  double* a = AVb + b * astride + (int64_t)col * ld;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    a[i] = y[b * n + i];
}

// convergence test of the refreshed pair; restarts the subspace at k = 1
__global__ void k_b_check(int B, const double* __restrict__ th2, const double* __restrict__ res2, int rs, double tol,
                          int* __restrict__ notdone, int* __restrict__ act, int* __restrict__ nref,
                          double* __restrict__ last_true,
                          double* __restrict__ theta, double* __restrict__ energy, double* __restrict__ Hs, int m,
                          int* __restrict__ kdev, int* __restrict__ nact, double* __restrict__ resid) {
  __shared__ int cnt;
  if (threadIdx.x == 0) {
    cnt = 0;
    *kdev = 1;
  }
  __syncthreads();
  int c = 0;
  for (int b = threadIdx.x; b < B; b += blockDim.x) {
    act[b] = 0;
    if (!notdone[b]) continue;
    nref[b] += 1;
    const double th = th2[(int64_t)b * 2];
    const double rn = sqrt(res2[(int64_t)b * rs]);
    theta[b] = th;
    energy[b] = th;
    resid[b] = rn;
    if (rn < tol) {
      notdone[b] = 0;
      continue;
    }
    act[b] = 1;
    last_true[b] = rn;
    Hs[(int64_t)b * m * m] = th;
    ++c;
  }
  atomicAdd(&cnt, c);
  __syncthreads();
  if (threadIdx.x == 0) *nact = cnt;
}

// lowest diagonal element per instance (first on ties, diagonal_guess's
// std::min_element), one CTA per instance; x = the unit vector there
__global__ void k_b_guess(const double* __restrict__ D, int64_t n, double* __restrict__ x, int64_t* __restrict__ idx) {
  __shared__ double sv[kBT];
  __shared__ int64_t si[kBT];
  const int b = blockIdx.x;
  double best = INFINITY;
  int64_t bi = n;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    const double v = D[b * n + i];
    if (v < best || (v == best && i < bi)) {
      best = v;
      bi = i;
    }
  }
  sv[threadIdx.x] = best;
  si[threadIdx.x] = bi;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      const double v = sv[threadIdx.x + s];
      const int64_t i = si[threadIdx.x + s];
      if (v < sv[threadIdx.x] || (v == sv[threadIdx.x] && i < si[threadIdx.x])) {
        sv[threadIdx.x] = v;
        si[threadIdx.x] = i;
      }
    }
    __syncthreads();
  }
  const int64_t k = si[0];
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) x[b * n + i] = (i == k) ? 1. : 0.;
  if (threadIdx.x == 0) idx[b] = k;
}

// spin-summed 1-RDM of each instance's vector (rdm1_cta), one CTA per instance
__global__ void k_b_rdm1(const double* __restrict__ C, int G, int Nb, int norb, const uint64_t* __restrict__ galpha,
                         const uint64_t* __restrict__ ubeta, const int64_t* __restrict__ acon_ptr,
                         const int32_t* __restrict__ acon_idx, const int8_t* __restrict__ acon_lvl,
                         const int64_t* __restrict__ b1_ptr, const int32_t* __restrict__ b1_idx,
                         double* __restrict__ out, const int64_t* __restrict__ out_off) {
  extern __shared__ double gam[];
  const int b = blockIdx.x;
  rdm1_cta(C + (int64_t)b * G * Nb, G, Nb, norb, galpha, ubeta, acon_ptr, acon_idx, acon_lvl, b1_ptr, b1_idx,
           out + out_off[b], gam);
}

unsigned grid_x(int64_t n, int B) {
  const int64_t want = (n + kBT - 1) / kBT;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(want, std::max<int64_t>(1, 2048 / std::max(1, B))));
}

struct Shape {
  int norb, na, nb;
  bool operator<(const Shape& o) const { return std::tie(norb, na, nb) < std::tie(o.norb, o.na, o.nb); }
};

}  // namespace

// Solves every instance; energies[i] and (when rdm1 is not null) the
// spin-summed 1-RDM of instance i at rdm1 + sum_{j<i} norb_j^2.
void casci_batch(Context* ctx, int ninst, const qdkgb_cas_instance* inst, const qdkgb_batch_settings& st,
                 double* energies, double* rdm1, int* iters, qdkgb_batch_info* info) {
  NvtxRange nvtx_range("qdkgb.casci_batch");
  const auto t_start = std::chrono::steady_clock::now();
  if (ninst < 0) throw Error(QDKGB_ERR_INVALID, "negative instance count");
  if (st.max_subspace < 2 || st.max_subspace > 64) throw Error(QDKGB_ERR_INVALID, "max_subspace must be in [2, 64]");
  if (!(st.res_tol > 0.)) throw Error(QDKGB_ERR_INVALID, "res_tol must be positive");
  if (st.precision != QDKGB_PREC_FP64 && st.precision != QDKGB_PREC_MIXED)
    throw Error(QDKGB_ERR_INVALID, "unknown precision");
  std::map<Shape, std::vector<int>> shapes;
  std::vector<int64_t> rdm_off(ninst + 1, 0);
  for (int i = 0; i < ninst; ++i) {
    const qdkgb_cas_instance& q = inst[i];
    if (q.norb <= 0 || q.norb > 64 || q.nalpha <= 0 || q.nbeta <= 0 || q.nalpha > q.norb || q.nbeta > q.norb ||
        !q.T || !q.V)
      throw Error(QDKGB_ERR_INVALID, "instance " + std::to_string(i) + ": bad shape or null integrals");
    shapes[{q.norb, q.nalpha, q.nbeta}].push_back(i);
    rdm_off[i + 1] = rdm_off[i] + (int64_t)q.norb * q.norb;
  }
  const bool mixed = st.precision == QDKGB_PREC_MIXED;
  const int m = st.max_subspace;
  int max_it = 0, replays = 0;
  bool all_conv = true;
  cudaStream_t s0 = ctx->stream;
  for (auto& [shape, members] : shapes) {
    // the shape's space and tables, in a context of its own
    qdkgb_context* cc = new qdkgb_context();
    struct Owner {
      qdkgb_context* c;
      ~Owner() { qdkgb_destroy(c); }
    } own{cc};
    cc->device = ctx->device;
    cc->sm_count = ctx->sm_count;
    cc->stream = s0;
    cc->norb = shape.norb;
    int64_t N = 0;
    {
      int64_t nd = 0;
      qdkgb_fci_dets(shape.norb, shape.na, shape.nb, nullptr, nullptr, &nd);
      std::vector<uint64_t> a(nd), bb(nd);
      qdkgb_fci_dets(shape.norb, shape.na, shape.nb, a.data(), bb.data(), &nd);
      build_det_space(cc, nd, a.data(), bb.data());
      N = nd;
    }
    if (!cc->fci) throw Error(QDKGB_ERR_UNSUPPORTED, "batched CASCI: space too large for the slab tables");
    const DetSpace& S = cc->dets;
    const int64_t stored = struct_slab_elements(cc);
    const int n = shape.norb;
    const size_t n2 = (size_t)n * n, n3 = n2 * n, n4 = n3 * n;
    const int64_t slab_bytes = stored * 8;  // hi + lo, or FP64
    int64_t Bmax = std::max<int64_t>(1, st.max_slab_bytes / std::max<int64_t>(1, slab_bytes));
    Bmax = std::min<int64_t>(Bmax, kMaxB);
    const bool square = shape.na == shape.nb && S.ngroups == S.nbeta;
    for (size_t off = 0; off < members.size(); off += (size_t)Bmax) {
      const int B = (int)std::min<int64_t>(Bmax, (int64_t)(members.size() - off));
      // ---- integrals and intermediates
      // every device buffer of the sub-batch, freed on every exit
      struct BufSet {
        Context* c;
        DeviceBuffer b[40];
        ~BufSet() {
          for (DeviceBuffer& x : b) dev_free(c, x);
        }
      } bs{cc, {}};
      DeviceBuffer &dT = bs.b[0], &dV = bs.b[1], &dG = bs.b[2], &dVr = bs.b[3], &dG2 = bs.b[4], &dV2 = bs.b[5],
                   &dI = bs.b[6], &dD = bs.b[7], &dval = bs.b[8], &dhi = bs.b[9], &dlo = bs.b[10];
      std::vector<double> hT((size_t)B * n2), hV((size_t)B * n4);
      for (int q = 0; q < B; ++q) {
        const qdkgb_cas_instance& in = inst[members[off + q]];
        std::memcpy(&hT[q * n2], in.T, n2 * 8);
        std::memcpy(&hV[q * n4], in.V, n4 * 8);
      }
      double* T = dev_array<double>(cc, dT, B * n2);
      double* V = dev_array<double>(cc, dV, B * n4);
      double* G = dev_array<double>(cc, dG, B * n3);
      double* Vr = dev_array<double>(cc, dVr, B * n3);
      double* G2 = dev_array<double>(cc, dG2, B * n2);
      double* V2 = dev_array<double>(cc, dV2, B * n2);
      QDKGB_CUDA(cudaMemcpyAsync(T, hT.data(), B * n2 * 8, cudaMemcpyHostToDevice, s0));
      QDKGB_CUDA(cudaMemcpyAsync(V, hV.data(), B * n4 * 8, cudaMemcpyHostToDevice, s0));
      std::vector<Integrals> hI(B);
      for (int q = 0; q < B; ++q) {
        build_integral_intermediates_into(cc, n, V + q * n4, G + q * n3, Vr + q * n3, G2 + q * n2, V2 + q * n2);
        hI[q] = Integrals{T + q * n2, V + q * n4, G + q * n3, Vr + q * n3, G2 + q * n2, V2 + q * n2, n};
      }
      Integrals* I = dev_array<Integrals>(cc, dI, B);
      QDKGB_CUDA(cudaMemcpyAsync(I, hI.data(), B * sizeof(Integrals), cudaMemcpyHostToDevice, s0));
      // ---- diagonals and slabs
      double* D = dev_array<double>(cc, dD, (size_t)B * N);
      const unsigned tb = (unsigned)std::min<int64_t>((N + 255) / 256, (int64_t)cc->sm_count * 16);
      for (int q = 0; q < B; ++q) k_diag_launch(cc, hI[q], D + q * N, tb);
      const double thresh = st.matel_tol;
      double* val = nullptr;
      float *hi = nullptr, *lo = nullptr;
      if (mixed) {
        hi = dev_array<float>(cc, dhi, (size_t)B * stored);
        lo = dev_array<float>(cc, dlo, (size_t)B * stored);
        slab_emit_batch(cc, B, I, D, QDKGB_H_SPLIT32, nullptr, hi, lo, thresh);
      } else {
        val = dev_array<double>(cc, dval, (size_t)B * stored);
        slab_emit_batch(cc, B, I, D, QDKGB_H_FP64, val, nullptr, nullptr, thresh);
      }
      if (st.persistent) {
        // ---- one persistent launch over the sub-batch (batch_persist.cu)
        DeviceBuffer &pe = bs.b[11], &pr = bs.b[12], &pi = bs.b[13];
        BatchShapeJob job{};
        job.norb = n;
        job.na = shape.na;
        job.nb = shape.nb;
        job.B = B;
        job.m = m;
        job.max_cycles = st.max_cycles;
        job.cluster = st.cluster;
        job.mixed = mixed;
        job.square = square;
        job.N = N;
        job.nstr = S.nbeta;
        job.vstride = stored;
        job.tol = st.res_tol;
        job.min_abs = st.min_abs_denominator;
        job.hi = hi;
        job.lo = lo;
        job.val = val;
        job.D = D;
        job.energy = dev_array<double>(cc, pe, (size_t)2 * B);
        job.resid = job.energy + B;
        job.iters = dev_array<int>(cc, pi, (size_t)2 * B);
        job.notdone = job.iters + B;
        job.rdm = rdm1 ? dev_array<double>(cc, pr, (size_t)B * n2) : nullptr;
        batch_solve_persistent(cc, ctx, job);
        std::vector<double> hE(2 * (size_t)B);
        std::vector<int> hI(2 * (size_t)B);
        QDKGB_CUDA(cudaMemcpyAsync(hE.data(), job.energy, 2 * B * 8, cudaMemcpyDeviceToHost, s0));
        QDKGB_CUDA(cudaMemcpyAsync(hI.data(), job.iters, 2 * B * 4, cudaMemcpyDeviceToHost, s0));
        std::vector<double> hout(rdm1 ? (size_t)B * n2 : 0);
        if (rdm1) QDKGB_CUDA(cudaMemcpyAsync(hout.data(), job.rdm, B * n2 * 8, cudaMemcpyDeviceToHost, s0));
        QDKGB_CUDA(cudaStreamSynchronize(s0));
        for (int q = 0; q < B; ++q) {
          const int i = members[off + q];
          if (energies) energies[i] = hE[q];
          if (iters) iters[i] = hI[q];
          max_it = std::max(max_it, hI[q]);
          if (hI[B + q]) all_conv = false;
          if (rdm1) std::memcpy(rdm1 + rdm_off[i], &hout[q * n2], n2 * 8);
        }
        continue;
      }
      // mixed form: new directions through the direct contraction where it
      // applies (the stored hi / lo slab still serves the full-precision refresh)
      const bool dbatch = mixed && direct_batch_prepare(cc, B, T, V);
      // ---- Davidson state
      const int KM = m + 1;
      const int nchunk = (int)((N + kChunk - 1) / kChunk);
      DeviceBuffer &bV = bs.b[11], &bAV = bs.b[12], &bHs = bs.b[13], &bx = bs.b[14], &bax = bs.b[15], &br = bs.b[16],
                   &bt = bs.b[17], &bt32 = bs.b[18], &bs32 = bs.b[19], &bxh = bs.b[20], &bxl = bs.b[21],
                   &by = bs.b[22], &bev = bs.b[23], &bth = bs.b[24], &bco = bs.b[25], &bpart = bs.b[26],
                   &bsc = bs.b[27], &bsc2 = bs.b[28], &bflip = bs.b[29], &bint = bs.b[30], &bidx = bs.b[31],
                   &blt = bs.b[32], &ben = bs.b[33], &bres = bs.b[34], &bxp = bs.b[37], &bw0 = bs.b[38],
                   &bn2 = bs.b[39];
      const int64_t astride = (int64_t)m * N;
      double* Vb = dev_array<double>(cc, bV, (size_t)B * astride);
      double* AVb = dev_array<double>(cc, bAV, (size_t)B * astride);
      double* Hs = dev_array<double>(cc, bHs, (size_t)B * m * m);
      double* x = dev_array<double>(cc, bx, (size_t)B * N);
      double* xprev = dev_array<double>(cc, bxp, (size_t)B * N);
      double* ax = dev_array<double>(cc, bax, (size_t)B * N);
      double* r = dev_array<double>(cc, br, (size_t)B * N);
      double* t = dev_array<double>(cc, bt, (size_t)B * N);
      float* t32 = dev_array<float>(cc, bt32, (size_t)B * N);
      float* s32 = dev_array<float>(cc, bs32, (size_t)B * N);
      float* xh = dev_array<float>(cc, bxh, (size_t)B * N);
      float* xl = dev_array<float>(cc, bxl, (size_t)B * N);
      double* yfull = dev_array<double>(cc, by, (size_t)B * N);
      double* yv = dev_array<double>(cc, bev, (size_t)B * KM);
      double* theta = dev_array<double>(cc, bth, (size_t)B);
      double* coef = dev_array<double>(cc, bco, (size_t)B * KM);
      double* partial = dev_array<double>(cc, bpart, (size_t)B * nchunk * std::max(KM, 6));
      double* sc = dev_array<double>(cc, bsc, (size_t)B * 6);    // per-instance scalars
      double* sc2 = dev_array<double>(cc, bsc2, (size_t)B * 2);  // second scalar
      double* flip = dev_array<double>(cc, bflip, (size_t)B);
      double* last_true = dev_array<double>(cc, blt, (size_t)B);
      double* energy = dev_array<double>(cc, ben, (size_t)B);
      double* resid = dev_array<double>(cc, bres, (size_t)B);
      int* ints = dev_array<int>(cc, bint, (size_t)5 * B + 8);
      int* act = ints;
      int* notdone = ints + B;
      int* nsig = ints + 2 * B;
      int* nref = ints + 3 * B;
      int* kdev = ints + 4 * B;
      int* nact = ints + 4 * B + 1;
      int64_t* idx = dev_array<int64_t>(cc, bidx, (size_t)B);
      double* w0 = dev_array<double>(cc, bw0, (size_t)B);  // |t|^2 before the first Gram-Schmidt pass
      int* need2 = dev_array<int>(cc, bn2, (size_t)B);     // instances that take the second pass
      QDKGB_CUDA(cudaMemsetAsync(ints, 0, ((size_t)5 * B + 8) * sizeof(int), s0));
      QDKGB_CUDA(cudaMemsetAsync(Hs, 0, (size_t)B * m * m * 8, s0));
      // guess and its spin-flip sector (kept by the FP64 iteration; FP32
      // noise is projected out of new directions, as in the single solve)
      k_b_guess<<<B, kBT, 0, s0>>>(D, N, x, idx);
      QDKGB_CHECK_LAUNCH();
      {
        std::vector<int64_t> hidx(B);
        QDKGB_CUDA(cudaMemcpyAsync(hidx.data(), idx, B * 8, cudaMemcpyDeviceToHost, s0));
        QDKGB_CUDA(cudaStreamSynchronize(s0));
        std::vector<double> hf(B, 0.);
        std::vector<int> hnd(B, 1);
        if (square && mixed)
          for (int q = 0; q < B; ++q) hf[q] = (hidx[q] / S.nbeta == hidx[q] % S.nbeta) ? 1. : 0.;
        QDKGB_CUDA(cudaMemcpyAsync(flip, hf.data(), B * 8, cudaMemcpyHostToDevice, s0));
        QDKGB_CUDA(cudaMemcpyAsync(notdone, hnd.data(), B * 4, cudaMemcpyHostToDevice, s0));
      }
      const dim3 gv(grid_x(N, B), B), gc(nchunk, B);
      const int64_t ld = N;
      std::vector<int> hstat(2);
      auto read_nact = [&]() {
        QDKGB_CUDA(cudaMemcpyAsync(hstat.data(), nact, sizeof(int), cudaMemcpyDeviceToHost, s0));
        QDKGB_CUDA(cudaMemcpyAsync(hstat.data() + 1, kdev, sizeof(int), cudaMemcpyDeviceToHost, s0));
        QDKGB_CUDA(cudaStreamSynchronize(s0));
        return hstat[0];
      };
      // ---- refresh: full-precision sigma of the normalised Ritz vector; from
      // the second cycle on (gd) the subspace restarts on [x, x_prev] (GD+1:
      // the previous Ritz vector orthogonalised against x, also multiplied
      // in full precision) instead of x alone
      auto refresh = [&](bool gd) {
        k_b_multidot<<<gc, kBT, 0, s0>>>(x, N, N, nullptr, 1, x, N, 0, N, nchunk, partial, KM, notdone);
        QDKGB_CHECK_LAUNCH();
        k_b_reduce<<<B, 32, 0, s0>>>(partial, nchunk, KM, nullptr, 1, sc, 6, notdone);
        QDKGB_CHECK_LAUNCH();
        k_b_refresh_x<<<gv, kBT, 0, s0>>>(x, sc, 6, Vb, astride, xh, xl, N, notdone);
        QDKGB_CHECK_LAUNCH();
        if (gd) {
          // candidates kept in the guess's spin-flip sector: the estimated
          // residual carries the FP32 sigma's out-of-sector noise
          const double* fl = (square && mixed) ? flip : nullptr;
          if (fl) {
            k_b_flip<<<gv, kBT, 0, s0>>>(xprev, S.nbeta, flip, notdone);
            QDKGB_CHECK_LAUNCH();
            k_b_flip<<<gv, kBT, 0, s0>>>(r, S.nbeta, flip, notdone);
            QDKGB_CHECK_LAUNCH();
          }
          k_b_second_dots<<<gc, kBT, 0, s0>>>(x, xprev, r, N, S.nbeta, fl, nchunk, partial, notdone);
          QDKGB_CHECK_LAUNCH();
          k_b_reduce<<<B, 32, 0, s0>>>(partial, nchunk, 6, nullptr, 6, sc, 6, notdone);
          QDKGB_CHECK_LAUNCH();
          k_b_second_set<<<gv, kBT, 0, s0>>>(x, xprev, r, sc, Vb, astride, ld, t32, s32, N, S.nbeta, fl, notdone);
          QDKGB_CHECK_LAUNCH();
          if (mixed) {
            slab_sigma_batch(cc, 2, B, notdone, hi, lo, t32, s32, ax);
          } else {
            k_b_col_to_packed<<<gv, kBT, 0, s0>>>(Vb, astride, ld, 1, t, N, notdone);
            QDKGB_CHECK_LAUNCH();
            slab_sigma_batch(cc, 1, B, notdone, val, nullptr, t, nullptr, ax);
          }
        }
        if (mixed) slab_sigma_batch(cc, 2, B, notdone, hi, lo, xh, xl, yfull);
        else slab_sigma_batch(cc, 1, B, notdone, val, nullptr, x, nullptr, yfull);
        k_b_multidot<<<gc, kBT, 0, s0>>>(x, N, N, nullptr, 1, yfull, N, 0, N, nchunk, partial, KM, notdone);
        QDKGB_CHECK_LAUNCH();
        k_b_reduce<<<B, 32, 0, s0>>>(partial, nchunk, KM, nullptr, 1, sc2, 2, notdone);
        QDKGB_CHECK_LAUNCH();
        k_b_refresh_res<<<gc, kBT, 0, s0>>>(x, yfull, sc2, AVb, astride, r, N, nchunk, partial, notdone);
        QDKGB_CHECK_LAUNCH();
        k_b_reduce<<<B, 32, 0, s0>>>(partial, nchunk, 1, nullptr, 1, sc, 6, notdone);
        QDKGB_CHECK_LAUNCH();
        k_b_check<<<1, 1024, 0, s0>>>(B, sc2, sc, 6, st.res_tol, notdone, act, nref, last_true, theta, energy, Hs, m,
                                      kdev, nact, resid);
        QDKGB_CHECK_LAUNCH();
        if (gd) {
          k_b_copy_col<<<gv, kBT, 0, s0>>>(ax, AVb, astride, ld, 1, N, act);
          QDKGB_CHECK_LAUNCH();
          // row 1 of the projected matrix (kdev = 1 after the check), then k = 2
          k_b_multidot<<<gc, kBT, 0, s0>>>(AVb, astride, ld, kdev, 1, Vb, astride, ld, N, nchunk, partial, KM, act);
          QDKGB_CHECK_LAUNCH();
          k_b_reduce<<<B, 64, 0, s0>>>(partial, nchunk, KM, kdev, 1, coef, KM, act);
          QDKGB_CHECK_LAUNCH();
          k_b_hsrow<<<B, 64, 0, s0>>>(coef, KM, Hs, m, kdev, act);
          QDKGB_CHECK_LAUNCH();
          k_b_kinc<<<1, 1, 0, s0>>>(kdev);
          QDKGB_CHECK_LAUNCH();
          lowest_eig_batch(s0, B, kdev, 0, m, Hs, m, (int64_t)m * m, theta, yv, KM, act);
          k_b_ritz<<<gc, kBT, 0, s0>>>(Vb, AVb, astride, ld, kdev, yv, KM, theta, x, xprev, ax, r, N, nchunk, partial,
                                       act);
          QDKGB_CHECK_LAUNCH();
        }
      };
      // ---- one inner iteration (graph-captured): new direction from (r, theta)
      auto inner = [&]() {
        k_b_precond<<<gv, kBT, 0, s0>>>(r, D, theta, t, N, st.min_abs_denominator, act);
        QDKGB_CHECK_LAUNCH();
        if (square && mixed) {
          k_b_flip<<<gv, kBT, 0, s0>>>(t, S.nbeta, flip, act);
          QDKGB_CHECK_LAUNCH();
        }
        // Gram-Schmidt against V[0..k): the FP64 form always makes two passes
        // (the reference's CGS2); the mixed form makes the second only for the
        // instances whose first pass removed more than half of |t|^2 (the
        // Daniel-Gragg-Kaufman-Stewart test, as in the single solve)
        auto gs_pass = [&](const int* mask) {
          k_b_multidot<<<gc, kBT, 0, s0>>>(Vb, astride, ld, kdev, 0, t, N, 0, N, nchunk, partial, KM, mask);
          QDKGB_CHECK_LAUNCH();
          k_b_reduce<<<B, 64, 0, s0>>>(partial, nchunk, KM, kdev, 0, coef, KM, mask);
          QDKGB_CHECK_LAUNCH();
          k_b_gemv<<<gv, kBT, 0, s0>>>(Vb, astride, ld, kdev, 0, coef, KM, -1., t, t, N, N, mask);
          QDKGB_CHECK_LAUNCH();
        };
        auto norm2 = [&](double* out, int ostride, const int* mask) {
          k_b_multidot<<<gc, kBT, 0, s0>>>(t, N, N, nullptr, 1, t, N, 0, N, nchunk, partial, KM, mask);
          QDKGB_CHECK_LAUNCH();
          k_b_reduce<<<B, 32, 0, s0>>>(partial, nchunk, KM, nullptr, 1, out, ostride, mask);
          QDKGB_CHECK_LAUNCH();
        };
        if (mixed) {
          norm2(w0, 1, act);
          gs_pass(act);
          norm2(sc, 2, act);
          k_b_need2<<<(B + 255) / 256, 256, 0, s0>>>(B, act, sc, w0, need2);
          QDKGB_CHECK_LAUNCH();
          gs_pass(need2);
          norm2(sc, 2, need2);
        } else {
          gs_pass(act);
          gs_pass(act);
          norm2(sc, 2, act);
        }
        k_b_store_dir<<<gv, kBT, 0, s0>>>(t, sc, Vb, astride, ld, kdev, t32, N, act, nsig);
        QDKGB_CHECK_LAUNCH();
        if (mixed) {
          if (dbatch)
            direct_batch_sigma(cc, B, act, D, t32, s32);
          else
            slab_sigma_batch(cc, 0, B, act, hi, nullptr, t32, nullptr, s32);
          k_b_f32_to_col<<<gv, kBT, 0, s0>>>(s32, AVb, astride, ld, kdev, N, act);
        } else {
          slab_sigma_batch(cc, 1, B, act, val, nullptr, t, nullptr, yfull);
          k_b_f64_to_col<<<gv, kBT, 0, s0>>>(yfull, AVb, astride, ld, kdev, N, act);
        }
        QDKGB_CHECK_LAUNCH();
        // projected row k: Hs(k, j) = AV[j] . V[k], j <= k - the older (more
        // accurate) product of each pair: the exact AV[0] couples the new
        // direction to the refreshed vector
        k_b_multidot<<<gc, kBT, 0, s0>>>(AVb, astride, ld, kdev, 1, Vb, astride, ld, N, nchunk, partial, KM, act);
        QDKGB_CHECK_LAUNCH();
        k_b_reduce<<<B, 64, 0, s0>>>(partial, nchunk, KM, kdev, 1, coef, KM, act);
        QDKGB_CHECK_LAUNCH();
        k_b_hsrow<<<B, 64, 0, s0>>>(coef, KM, Hs, m, kdev, act);
        QDKGB_CHECK_LAUNCH();
        k_b_kinc<<<1, 1, 0, s0>>>(kdev);
        QDKGB_CHECK_LAUNCH();
        lowest_eig_batch(s0, B, kdev, 0, m, Hs, m, (int64_t)m * m, theta, yv, KM, act);
        k_b_ritz<<<gc, kBT, 0, s0>>>(Vb, AVb, astride, ld, kdev, yv, KM, theta, x, xprev, ax, r, N, nchunk, partial,
                                     act);
        QDKGB_CHECK_LAUNCH();
        k_b_reduce<<<B, 32, 0, s0>>>(partial, nchunk, 1, nullptr, 1, sc, 2, act);
        QDKGB_CHECK_LAUNCH();
        k_b_wait<<<1, 1024, 0, s0>>>(B, sc, last_true, 1e-4, kdev, m, act, nact);
        QDKGB_CHECK_LAUNCH();
      };
      // ---- cycles
      cudaGraph_t graph = nullptr;
      cudaGraphExec_t gexec = nullptr;
      struct GraphOwner {
        cudaGraph_t* g;
        cudaGraphExec_t* e;
        ~GraphOwner() {
          if (*e) cudaGraphExecDestroy(*e);
          if (*g) cudaGraphDestroy(*g);
        }
      } gown{&graph, &gexec};
      slab_reserve_batch(cc, B);
      refresh(false);
      int cycles = 0;
      bool warmed = false;  // one eager iteration first: it makes the allocations a capture may not
      while (read_nact() > 0) {
        if (++cycles > std::max(1, st.max_cycles)) break;
        for (int it = 1; it < m; ++it) {
          if (st.use_graph && warmed) {
            if (!gexec) {
              QDKGB_CUDA(cudaStreamBeginCapture(s0, cudaStreamCaptureModeThreadLocal));
              inner();
              QDKGB_CUDA(cudaStreamEndCapture(s0, &graph));
              QDKGB_CUDA(cudaGraphInstantiate(&gexec, graph, 0));
            }
            QDKGB_CUDA(cudaGraphLaunch(gexec, s0));
            ++replays;
          } else {
            inner();
            warmed = true;
          }
          if (read_nact() == 0 || hstat[1] >= m) break;
        }
        refresh(true);
      }
      // ---- results
      std::vector<double> hE(B), hR(B);
      std::vector<int> hnd(B), hns(B), hnr(B);
      QDKGB_CUDA(cudaMemcpyAsync(hnr.data(), nref, B * 4, cudaMemcpyDeviceToHost, s0));
      QDKGB_CUDA(cudaMemcpyAsync(hE.data(), energy, B * 8, cudaMemcpyDeviceToHost, s0));
      QDKGB_CUDA(cudaMemcpyAsync(hR.data(), resid, B * 8, cudaMemcpyDeviceToHost, s0));
      QDKGB_CUDA(cudaMemcpyAsync(hnd.data(), notdone, B * 4, cudaMemcpyDeviceToHost, s0));
      QDKGB_CUDA(cudaMemcpyAsync(hns.data(), nsig, B * 4, cudaMemcpyDeviceToHost, s0));
      QDKGB_CUDA(cudaStreamSynchronize(s0));
      for (int q = 0; q < B; ++q) {
        const int i = members[off + q];
        if (energies) energies[i] = hE[q];
        if (iters) iters[i] = hns[q] + hnr[q];
        max_it = std::max(max_it, hns[q] + hnr[q]);
        if (hnd[q]) all_conv = false;
      }
      if (rdm1) {
        DeviceBuffer &bo = bs.b[35], &boff = bs.b[36];
        double* dout = dev_array<double>(cc, bo, (size_t)B * n2);
        std::vector<int64_t> hoff(B);
        for (int q = 0; q < B; ++q) hoff[q] = (int64_t)q * n2;
        int64_t* doff = dev_array<int64_t>(cc, boff, B);
        QDKGB_CUDA(cudaMemcpyAsync(doff, hoff.data(), B * 8, cudaMemcpyHostToDevice, s0));
        k_b_rdm1<<<B, 256, n2 * sizeof(double), s0>>>(
            x, (int)S.ngroups, (int)S.nbeta, n, (const uint64_t*)S.galpha.ptr, (const uint64_t*)S.ubeta.ptr,
            (const int64_t*)S.acon_ptr.ptr, (const int32_t*)S.acon_idx.ptr, (const int8_t*)S.acon_lvl.ptr,
            (const int64_t*)S.b1_ptr.ptr, (const int32_t*)S.b1_idx.ptr, dout, doff);
        QDKGB_CHECK_LAUNCH();
        std::vector<double> hout((size_t)B * n2);
        QDKGB_CUDA(cudaMemcpyAsync(hout.data(), dout, B * n2 * 8, cudaMemcpyDeviceToHost, s0));
        QDKGB_CUDA(cudaStreamSynchronize(s0));
        for (int q = 0; q < B; ++q)
          std::memcpy(rdm1 + rdm_off[members[off + q]], &hout[q * n2], n2 * 8);
      }
    }
    cc->stream = cc->own_stream;  // the borrowed stream is not the shape context's to destroy
  }
  if (info) {
    info->iterations = max_it;
    info->graph_replays = replays;
    info->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
  }
  if (!all_conv) throw Error(QDKGB_ERR_NOT_CONVERGED, "batched CASCI: some instances did not converge");
}

}  // namespace qdkgb
