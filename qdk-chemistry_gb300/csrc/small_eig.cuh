// Small dense symmetric eigensolver, one CTA (Davidson's projected problem).
#pragma once
#include "common.cuh"

namespace qdkgb {

#ifndef QDKGB_EIG_MAX_SUBSPACE
#define QDKGB_EIG_MAX_SUBSPACE 256
#endif
constexpr int kEigMaxK = QDKGB_EIG_MAX_SUBSPACE;

// ---------------------------------------------------------------- lowest eigenpairs
// One CTA: the `nev` lowest eigenpairs of the symmetric k x k matrix H (lower
// triangle read, as syev(Uplo::Lower)).  Householder reduction to tridiagonal
// form (O(k^3) once, instead of Jacobi's O(k^3) per sweep - the FP64 pipe of
// one SM is the budget here), eigenvalues by multisection on the
// division-free Sturm sequence, eigenvectors by inverse iteration on the
// tridiagonal matrix (partial pivoting, re-orthogonalised against the lower
// ones), back-transformed through the reflectors.  Results: eval[0:nev)
// ascending, evec[:, 0:nev) with leading dimension k.
constexpr int kEigThreads = 256;
constexpr int kEigSmemK = 150;  // matrices up to this size live in shared memory

__device__ double block_sum_eig(double v, double* red) {
  v = warp_sum(v);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) red[w] = v;
  __syncthreads();
  double t = 0.;
  if (threadIdx.x < 32) {
    t = (lane < (int)(blockDim.x >> 5)) ? red[lane] : 0.;
    t = warp_sum(t);
    if (lane == 0) red[32] = t;
  }
  __syncthreads();
  return red[32];
}

// number of eigenvalues of tridiag(d, e) below x (division-free Sturm sequence
// of leading minors, rescaled by exact powers of two)
__device__ int sturm_count(int k, const double* d, const double* e2, double x) {
  double p0 = 1., p1 = d[0] - x;
  int cnt = (p1 < 0.) ? 1 : 0;
  int s_prev = (p1 < 0.) ? -1 : 1;
  for (int i = 1; i < k; ++i) {
    double p2 = (d[i] - x) * p1 - e2[i - 1] * p0;
    const double a2 = fabs(p2);
    if (a2 > 0x1p+600) {
      p2 *= 0x1p-600;
      p1 *= 0x1p-600;
    } else if (a2 < 0x1p-600 && a2 != 0. && fabs(p1) < 0x1p-600) {
      p2 *= 0x1p+600;
      p1 *= 0x1p+600;
    }
    int sg = (p2 < 0.) ? -1 : (p2 > 0. ? 1 : -s_prev);
    if (sg != s_prev) ++cnt;
    s_prev = sg;
    p0 = p1;
    p1 = p2;
  }
  return cnt;
}

__device__ bool lowest_eig_mixed_cta(int k, const double* __restrict__ H, int ldh, double* eval, double* evec,
                                     unsigned char* smem);
constexpr int kEigMixedMaxK = 128;

__device__ void lowest_eig_cta(int k, const double* __restrict__ H, int ldh, double* gA, int nev, double* eval,
                               double* evec) {
  extern __shared__ double dyn[];
  __shared__ double d[kEigMaxK], e[kEigMaxK], e2[kEigMaxK], beta[kEigMaxK];
  __shared__ double red[33];
  __shared__ double s_lo, s_hi;
  __shared__ double s_u[3 * kEigMaxK];
  if (nev == 1 && k >= 2 && k <= kEigMixedMaxK && !gA) {
    if (lowest_eig_mixed_cta(k, H, ldh, eval, evec, reinterpret_cast<unsigned char*>(dyn))) return;
    __syncthreads();
  }
  double* A = gA ? gA : dyn;  // k x k, column-major; reflector j kept in column j below the diagonal
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int t = tid; t < k * k; t += nt) {
    const int i = t % k, j = t / k;
    A[t] = (i >= j) ? H[i + (size_t)j * ldh] : H[j + (size_t)i * ldh];
  }
  __syncthreads();
  // ---- Householder tridiagonalisation
  for (int j = 0; j + 2 < k; ++j) {
    const int m0 = j + 1;
    double xx = 0.;
    for (int i = m0 + tid; i < k; i += nt) xx += A[i + (size_t)k * j] * A[i + (size_t)k * j];
    xx = block_sum_eig(xx, red);
    if (tid == 0) {
      const double x0 = A[m0 + (size_t)k * j];
      const double nrm = sqrt(xx);
      if (nrm == 0.) {
        beta[j] = 0.;
        e[j] = 0.;
      } else {
        const double alpha = (x0 >= 0.) ? -nrm : nrm;
        const double v0 = x0 - alpha;
        const double vv = xx - x0 * x0 + v0 * v0;
        beta[j] = (vv > 0.) ? 2. / vv : 0.;
        e[j] = alpha;
        A[m0 + (size_t)k * j] = v0;
      }
      d[j] = A[j + (size_t)k * j];
    }
    __syncthreads();
    const double b = beta[j];
    if (b == 0.) continue;
    const double* v = A + (size_t)k * j;  // v_i for i >= m0
    // p = b * A_sub v, kept in column j's upper part?  use the d/e-free scratch: A row j (i < j unused after)
    // p is stored transiently in e2[] (length k)
    for (int i = m0 + tid; i < k; i += nt) {
      double acc = 0.;
      for (int l = m0; l < k; ++l) acc += A[i + (size_t)k * l] * v[l];
      e2[i] = b * acc;
    }
    __syncthreads();
    double vp = 0.;
    for (int i = m0 + tid; i < k; i += nt) vp += v[i] * e2[i];
    vp = block_sum_eig(vp, red);
    const double K = 0.5 * b * vp;
    for (int i = m0 + tid; i < k; i += nt) e2[i] -= K * v[i];  // w
    __syncthreads();
    const int m = k - m0;
    for (int t = tid; t < m * m; t += nt) {
      const int i = m0 + t % m, l = m0 + t / m;
      A[i + (size_t)k * l] -= v[i] * e2[l] + e2[i] * v[l];
    }
    __syncthreads();
  }
  if (tid == 0) {
    if (k >= 2) {
      d[k - 2] = A[(k - 2) + (size_t)k * (k - 2)];
      e[k - 2] = A[(k - 1) + (size_t)k * (k - 2)];
      beta[k - 2] = 0.;
    }
    d[k - 1] = A[(k - 1) + (size_t)k * (k - 1)];
    if (k >= 1) beta[k - 1] = 0.;
  }
  __syncthreads();
  for (int i = tid; i < k - 1; i += nt) e2[i] = e[i] * e[i];
  __syncthreads();
  // ---- eigenvalues: multisection on the Sturm count (one warp: 32 points per round)
  for (int jv = 0; jv < nev; ++jv) {
    if (tid == 0) {
      double lo = 1e300, hi = -1e300;
      for (int i = 0; i < k; ++i) {
        const double r = (i > 0 ? fabs(e[i - 1]) : 0.) + (i + 1 < k ? fabs(e[i]) : 0.);
        lo = fmin(lo, d[i] - r);
        hi = fmax(hi, d[i] + r);
      }
      const double pad = 1e-12 * fmax(1., fmax(fabs(lo), fabs(hi)));
      s_lo = lo - pad;
      s_hi = hi + pad;
    }
    __syncthreads();
    if (tid < 32) {
      for (int round = 0; round < 80; ++round) {
        const double lo = s_lo, hi = s_hi;
        if (!(hi - lo > 4e-16 * fmax(fabs(lo), fabs(hi))) || hi - lo < 1e-300) break;
        const double x = lo + (hi - lo) * (double)(tid + 1) / 33.;
        const int cnt = sturm_count(k, d, e2, x);
        const unsigned above = __ballot_sync(QDKGB_FULL_MASK, cnt > jv);
        const int t = above ? (__ffs(above) - 1) : 32;  // first point with count > jv
        if (tid == 0) {
          s_lo = (t == 0) ? lo : lo + (hi - lo) * (double)t / 33.;
          s_hi = (t == 32) ? hi : lo + (hi - lo) * (double)(t + 1) / 33.;
        }
        __syncwarp();
      }
      if (tid == 0) eval[jv] = 0.5 * (s_lo + s_hi);
    }
    __syncthreads();
  }
  // ---- eigenvectors of T: inverse iteration with partial pivoting (thread 0)
  double* Y = evec;  // k x nev, ld k
  if (tid == 0) {
    double* Ua = s_u;
    double* Ub = s_u + kEigMaxK;
    double* Uc = s_u + 2 * kEigMaxK;
    for (int jv = 0; jv < nev; ++jv) {
      double* y = Y + (size_t)k * jv;
      const double lam0 = eval[jv];
      const double lam = lam0 + (jv % 2 ? 1. : -1.) * 1e-17 * fmax(1., fabs(lam0));
      for (int i = 0; i < k; ++i) y[i] = 1.0 + 0.01 * (double)((i * 7 + jv * 3) % 11);
      for (int it = 0; it < 3; ++it) {
        // forward elimination of T - lam I (rows i: [a b c] at columns i, i+1, i+2)
        double a_i = d[0] - lam, b_i = (k > 1) ? e[0] : 0., c_i = 0., yi = y[0];
        for (int i = 0; i < k - 1; ++i) {
          const double a1 = e[i], b1 = d[i + 1] - lam, c1 = (i + 2 < k) ? e[i + 1] : 0., y1 = y[i + 1];
          if (fabs(a_i) >= fabs(a1)) {
            const double f = (a_i != 0.) ? a1 / a_i : 0.;
            Ua[i] = a_i;
            Ub[i] = b_i;
            Uc[i] = c_i;
            y[i] = yi;
            a_i = b1 - f * b_i;
            b_i = c1 - f * c_i;
            yi = y1 - f * yi;
          } else {
            const double f = a_i / a1;
            Ua[i] = a1;
            Ub[i] = b1;
            Uc[i] = c1;
            y[i] = y1;
            const double na = b_i - f * b1, nb = c_i - f * c1;
            yi = yi - f * y1;
            a_i = na;
            b_i = nb;
          }
          c_i = 0.;
        }
        Ua[k - 1] = a_i;
        y[k - 1] = yi;
        double big = 0.;
        for (int i = k - 1; i >= 0; --i) {
          double r = y[i];
          if (i + 1 < k) r -= Ub[i] * y[i + 1];
          if (i + 2 < k) r -= Uc[i] * y[i + 2];
          const double piv = (Ua[i] != 0.) ? Ua[i] : 1e-300;
          y[i] = r / piv;
          big = fmax(big, fabs(y[i]));
        }
        // rescale to avoid overflow, orthogonalise against lower vectors, normalise
        for (int i = 0; i < k; ++i) y[i] /= big;
        for (int q = 0; q < jv; ++q) {
          const double* z = Y + (size_t)k * q;
          double dz = 0.;
          for (int i = 0; i < k; ++i) dz += z[i] * y[i];
          for (int i = 0; i < k; ++i) y[i] -= dz * z[i];
        }
        double nrm = 0.;
        for (int i = 0; i < k; ++i) nrm += y[i] * y[i];
        nrm = sqrt(nrm);
        for (int i = 0; i < k; ++i) y[i] /= nrm;
      }
    }
  }
  __syncthreads();
  // ---- back-transform: y <- H_0 H_1 ... H_{k-3} y
  for (int j = k - 3; j >= 0; --j) {
    const double b = beta[j];
    if (b == 0.) continue;
    const int m0 = j + 1;
    const double* v = A + (size_t)k * j;
    for (int jv = 0; jv < nev; ++jv) {
      double* y = Y + (size_t)k * jv;
      double dv = 0.;
      for (int i = m0 + tid; i < k; i += nt) dv += v[i] * y[i];
      dv = block_sum_eig(dv, red);
      for (int i = m0 + tid; i < k; i += nt) y[i] -= b * dv * v[i];
      __syncthreads();
    }
  }
}


}  // namespace qdkgb

namespace qdkgb {

// ---------------------------------------------------------------- mixed precision
// Lowest eigenpair of the symmetric k x k FP64 matrix H (lower triangle), k <=
// kEigMixedMaxK, with FP64 work only in a refinement: the full spectral
// decomposition H ~ Q L Q^T is computed in FP32 (Householder tridiagonal
// reduction, eigenvalues by bisection on the Sturm pivots one thread per
// eigenvalue, eigenvectors by inverse iteration one thread per eigenvalue,
// back-transformed through the reflectors), then the lowest pair is refined
// in FP64: theta = y.Hy, r = Hy - theta y, and y <- y - sum_{i>0} q_i
// (q_i.r) / (l_i - theta) (the correction equation solved on the FP32
// spectral basis), until |r| reaches rounding level.  One FP64 matrix-vector
// product per step instead of an FP64 O(k^3) reduction: GB300's FP64 pipe is
// narrow and a one-CTA FP64 reduction is latency bound.  Returns false (the
// caller takes the FP64 path) for a near-degenerate lowest pair or when the
// refinement does not reach rounding level.

__device__ float block_sum_f(float v, float* red) {
  v = warp_sum(v);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) red[w] = v;
  __syncthreads();
  float t = 0.f;
  if (threadIdx.x < 32) {
    t = (lane < (int)(blockDim.x >> 5)) ? red[lane] : 0.f;
    t = warp_sum(t);
    if (lane == 0) red[32] = t;
  }
  __syncthreads();
  return red[32];
}

// smem: doubles y, w (kEigMixedMaxK each), dred[34]; region R of k*k
// doubles (the FP32 matrix / reflectors first, the FP64 matrix in the
// refinement); floats Q[k*k] (row-major: Q[r*k + i] = component r of
// eigenvector i), d, e, e2, beta, lam (kEigMixedMaxK each), red[34]
__device__ bool lowest_eig_mixed_cta(int k, const double* __restrict__ H, int ldh, double* eval, double* evec,
                                     unsigned char* smem) {
  const int tid = threadIdx.x, nt = blockDim.x;
  const int wid = tid >> 5, lane = tid & 31, nw = nt >> 5;
  double* y = reinterpret_cast<double*>(smem);
  double* w = y + kEigMixedMaxK;
  double* dred = w + kEigMixedMaxK;
  double* R = dred + 34;
  float* A = reinterpret_cast<float*>(R);
  float* Q = reinterpret_cast<float*>(R + (size_t)k * k);
  float* d = Q + (size_t)k * k;
  float* e = d + kEigMixedMaxK;
  float* e2 = e + kEigMixedMaxK;
  float* beta = e2 + kEigMixedMaxK;
  float* lam = beta + kEigMixedMaxK;
  float* red = lam + kEigMixedMaxK;
  auto Hat = [&](int i, int j) { return i >= j ? H[i + (size_t)j * ldh] : H[j + (size_t)i * ldh]; };
  for (int t = tid; t < k * k; t += nt) {
    const int i = t % k, j = t / k;
    A[t] = (float)Hat(i, j);
  }
  __syncthreads();
  // ---- FP32 Householder tridiagonalisation (reflector j below A(j+1, j));
  // A stays symmetric, so rows are read as columns (conflict-free)
  for (int j = 0; j + 2 < k; ++j) {
    const int m0 = j + 1;
    float xx = 0.f;
    for (int i = m0 + tid; i < k; i += nt) xx += A[i + k * j] * A[i + k * j];
    xx = block_sum_f(xx, red);
    if (tid == 0) {
      const float x0 = A[m0 + k * j];
      const float nrm = sqrtf(xx);
      if (nrm == 0.f) {
        beta[j] = 0.f;
        e[j] = 0.f;
      } else {
        const float alpha = (x0 >= 0.f) ? -nrm : nrm;
        const float v0 = x0 - alpha;
        const float vv = xx - x0 * x0 + v0 * v0;
        beta[j] = (vv > 0.f) ? 2.f / vv : 0.f;
        e[j] = alpha;
        A[m0 + k * j] = v0;
      }
      d[j] = A[j + k * j];
    }
    __syncthreads();
    const float b = beta[j];
    if (b == 0.f) continue;
    const float* v = A + k * j;
    // p = b A_sub v (warp per row i, lanes over l reading column i)
    for (int i = m0 + wid; i < k; i += nw) {
      float acc = 0.f;
      for (int l = m0 + lane; l < k; l += 32) acc += A[l + k * i] * v[l];
      acc = warp_sum(acc);
      if (lane == 0) e2[i] = b * acc;
    }
    __syncthreads();
    float vp = 0.f;
    for (int i = m0 + tid; i < k; i += nt) vp += v[i] * e2[i];
    vp = block_sum_f(vp, red);
    const float K = 0.5f * b * vp;
    for (int i = m0 + tid; i < k; i += nt) e2[i] -= K * v[i];
    __syncthreads();
    const int m = k - m0;
    for (int t = tid; t < m * m; t += nt) {
      const int i = m0 + t % m, l = m0 + t / m;
      A[i + k * l] -= v[i] * e2[l] + e2[i] * v[l];
    }
    __syncthreads();
  }
  if (tid == 0) {
    if (k >= 2) {
      d[k - 2] = A[(k - 2) + k * (k - 2)];
      e[k - 2] = A[(k - 1) + k * (k - 2)];
      beta[k - 2] = 0.f;
    }
    d[k - 1] = A[(k - 1) + k * (k - 1)];
    beta[k - 1] = 0.f;
  }
  __syncthreads();
  for (int i = tid; i < k - 1; i += nt) e2[i] = e[i] * e[i];
  __syncthreads();
  // ---- all eigenvalues: thread i bisects for the i-th smallest (Sturm
  // pivots with the fast reciprocal: a count, not a value, is needed)
  float glo = 0.f, ghi = 0.f;
  for (int i = 0; i < k; ++i) {
    const float r = (i > 0 ? fabsf(e[i - 1]) : 0.f) + (i + 1 < k ? fabsf(e[i]) : 0.f);
    glo = (i == 0) ? d[i] - r : fminf(glo, d[i] - r);
    ghi = (i == 0) ? d[i] + r : fmaxf(ghi, d[i] + r);
  }
  const float scale = fmaxf(fabsf(glo), fabsf(ghi));
  const float tiny = 1e-30f + 1e-12f * scale;
  for (int i = tid; i < k; i += nt) {
    float lo = glo - 1e-6f * scale - tiny, hi = ghi + 1e-6f * scale + tiny;
    for (int it = 0; it < 64; ++it) {
      const float mid = 0.5f * (lo + hi);
      if (!(hi - lo > 2.4e-7f * fmaxf(fabsf(lo), fabsf(hi))) || mid == lo || mid == hi) break;
      int cnt = 0;
      float q = d[0] - mid;
      if (fabsf(q) < tiny) q = -tiny;
      cnt += q < 0.f;
      for (int r = 1; r < k; ++r) {
        q = (d[r] - mid) - __fdividef(e2[r - 1], q);
        if (fabsf(q) < tiny) q = -tiny;
        cnt += q < 0.f;
      }
      if (cnt > i) hi = mid;
      else lo = mid;
    }
    lam[i] = 0.5f * (lo + hi);
  }
  __syncthreads();
  // near-degenerate lowest pair: the FP32 basis cannot separate it
  if (k >= 2 && !(lam[1] - lam[0] > 1e-5f * (scale + 1e-30f))) return false;
  // ---- eigenvectors of T: thread i, inverse iteration (L D L^T of T - s I,
  // tiny pivots replaced), distinct start vectors; z_i in Q[:, i]
  for (int i = tid; i < k; i += nt) {
    const float s = lam[i] + 1e-7f * (scale + 1e-30f) * ((i & 1) ? 1.f : -1.f);
    float Dinv[kEigMixedMaxK];
    float Dp = d[0] - s;
    if (fabsf(Dp) < tiny) Dp = tiny;
    Dinv[0] = __fdividef(1.f, Dp);
    for (int r = 1; r < k; ++r) {
      float Dr = (d[r] - s) - e2[r - 1] * Dinv[r - 1];
      if (fabsf(Dr) < tiny) Dr = tiny;
      Dinv[r] = __fdividef(1.f, Dr);
    }
    for (int r = 0; r < k; ++r) Q[r * k + i] = 1.f + 0.37f * (float)(((r + 1) * (i + 3)) % 7) - 1.1f;
    for (int pass = 0; pass < 2; ++pass) {
      // L D L^T z_new = z: L_{r,r-1} = e_{r-1} / D_{r-1}
      float zp = Q[i];
      for (int r = 1; r < k; ++r) {
        const float zr = Q[r * k + i] - e[r - 1] * Dinv[r - 1] * zp;
        Q[r * k + i] = zr;
        zp = zr;
      }
      float mx = 0.f;
      float zn = Q[(k - 1) * k + i] * Dinv[k - 1];
      Q[(k - 1) * k + i] = zn;
      mx = fabsf(zn);
      for (int r = k - 2; r >= 0; --r) {
        const float zr = Q[r * k + i] * Dinv[r] - e[r] * Dinv[r] * zn;
        Q[r * k + i] = zr;
        zn = zr;
        mx = fmaxf(mx, fabsf(zr));
      }
      const float inv = mx > 0.f ? __fdividef(1.f, mx) : 1.f;
      for (int r = 0; r < k; ++r) Q[r * k + i] *= inv;
    }
    float nn = 0.f;
    for (int r = 0; r < k; ++r) nn += Q[r * k + i] * Q[r * k + i];
    const float inv = rsqrtf(nn);
    for (int r = 0; r < k; ++r) Q[r * k + i] *= inv;
  }
  __syncthreads();
  // ---- back-transform: Q <- H_0 ... H_{k-3} Q (thread per column, rows
  // contiguous across the threads)
  for (int j = k - 3; j >= 0; --j) {
    const float b = beta[j];
    if (b != 0.f) {
      const float* v = A + k * j;
      for (int c = tid; c < k; c += nt) {
        float dv = 0.f;
        for (int r = j + 1; r < k; ++r) dv += v[r] * Q[r * k + c];
        dv *= b;
        for (int r = j + 1; r < k; ++r) Q[r * k + c] -= dv * v[r];
      }
    }
    __syncthreads();
  }
  // ---- FP64 refinement of the lowest pair; the FP64 matrix replaces the
  // reflectors in shared memory (full, symmetric)
  for (int t = tid; t < k * k; t += nt) {
    const int i = t % k, j = t / k;
    R[t] = Hat(i, j);
  }
  for (int i = tid; i < k; i += nt) y[i] = (double)Q[i * k];
  __syncthreads();
  double nrm2 = 0.;
  {
    double sacc = 0.;
    for (int i = tid; i < k; i += nt) sacc += y[i] * y[i];
    nrm2 = block_sum_eig(sacc, dred);
  }
  {
    const double inv = 1. / sqrt(nrm2);
    for (int i = tid; i < k; i += nt) y[i] *= inv;
  }
  __syncthreads();
  // stop at rounding level or when a step no longer halves |r|; accept below
  // 4096 eps |H|
  const double eps = 1.1102230246251565e-16, hs = (double)scale + 1e-300;
  double theta = 0., rn = 1e300, rprev = 1e300;
  for (int it = 0; it < 8; ++it) {
    // w = H y (warp per row i, lanes over column i: conflict-free)
    for (int i = wid; i < k; i += nw) {
      double acc = 0.;
      for (int l = lane; l < k; l += 32) acc += R[l + (size_t)k * i] * y[l];
      acc = warp_sum(acc);
      if (lane == 0) w[i] = acc;
    }
    __syncthreads();
    double sacc = 0.;
    for (int i = tid; i < k; i += nt) sacc += y[i] * w[i];
    theta = block_sum_eig(sacc, dred);
    sacc = 0.;
    for (int i = tid; i < k; i += nt) {
      const double ri = w[i] - theta * y[i];
      w[i] = ri;
      sacc += ri * ri;
    }
    rn = sqrt(block_sum_eig(sacc, dred));
    if (rn <= 16. * eps * hs || (it >= 2 && rn > 0.5 * rprev)) break;
    rprev = rn;
    // c_i = q_i . r / (l_i - theta), i > 0 (FP32), into e2 as scratch
    for (int i = tid; i < k; i += nt) {
      float c = 0.f;
      if (i > 0) {
        for (int r = 0; r < k; ++r) c += Q[r * k + i] * (float)w[r];
        c = c / (lam[i] - (float)theta);
      }
      e2[i] = c;
    }
    __syncthreads();
    // y <- y - Q c (warp per row r, lanes over i), normalised
    for (int r = wid; r < k; r += nw) {
      float dlt = 0.f;
      for (int i = 1 + lane; i < k; i += 32) dlt += Q[r * k + i] * e2[i];
      dlt = warp_sum(dlt);
      if (lane == 0) y[r] -= (double)dlt;
    }
    __syncthreads();
    sacc = 0.;
    for (int i = tid; i < k; i += nt) sacc += y[i] * y[i];
    nrm2 = block_sum_eig(sacc, dred);
    const double inv = 1. / sqrt(nrm2);
    for (int i = tid; i < k; i += nt) y[i] *= inv;
    __syncthreads();
  }
  if (!(rn <= 4096. * eps * hs)) return false;
  for (int i = tid; i < k; i += nt) evec[i] = y[i];
  if (tid == 0) eval[0] = theta;
  __syncthreads();
  return true;
}

// shared-memory bytes of lowest_eig_mixed_cta for size k
__host__ __device__ constexpr size_t eig_mixed_smem(int k) {
  return (2 * (size_t)kEigMixedMaxK + 34 + (size_t)k * k) * sizeof(double) +
         ((size_t)k * k + 5 * kEigMixedMaxK + 34) * sizeof(float);
}

// dynamic shared memory of lowest_eig_cta for size k (matrix in shared memory)
__host__ __device__ constexpr size_t eig_dyn_smem(int k) {
  return (k <= kEigMixedMaxK && eig_mixed_smem(k) > (size_t)k * k * sizeof(double)) ? eig_mixed_smem(k)
                                                                                    : (size_t)k * k * sizeof(double);
}

// the largest dynamic shared memory lowest_eig_cta asks for (matrices up to
// kEigSmemK in shared memory)
constexpr size_t kEigDynSmemMax = eig_mixed_smem(kEigMixedMaxK) > (size_t)kEigSmemK * kEigSmemK * sizeof(double)
                                      ? eig_mixed_smem(kEigMixedMaxK)
                                      : (size_t)kEigSmemK * kEigSmemK * sizeof(double);

}  // namespace qdkgb
