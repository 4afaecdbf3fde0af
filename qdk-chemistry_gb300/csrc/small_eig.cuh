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

static __device__ double block_sum_eig(double v, double* red) {
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
static __device__ int sturm_count(int k, const double* d, const double* e2, double x) {
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

static __device__ bool lowest_eig_mixed_cta(int k, const double* __restrict__ H, int ldh, int nev, double* eval,
                                     double* evec, unsigned char* smem);
constexpr int kEigMixedMaxK = 128;

static __device__ void lowest_eig_cta(int k, const double* __restrict__ H, int ldh, double* gA, int nev, double* eval,
                               double* evec) {
  extern __shared__ double dyn[];
  __shared__ double d[kEigMaxK], e[kEigMaxK], e2[kEigMaxK], beta[kEigMaxK];
  __shared__ double red[33];
  __shared__ double s_lo, s_hi;
  __shared__ double s_u[3 * kEigMaxK];
  if (nev >= 1 && nev <= k && k >= 2 && k <= kEigMixedMaxK && !gA) {
    if (lowest_eig_mixed_cta(k, H, ldh, nev, eval, evec, reinterpret_cast<unsigned char*>(dyn))) return;
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
// reduction, eigenvalues by multisection on the Sturm pivots, eigenvectors by
// inverse iteration one thread per eigenvalue, back-transformed through the
// reflectors), then the lowest pair is refined in FP64: theta = y.Hy / y.y,
// r = Hy - theta y, and y <- y - sum_{i>0} q_i (q_i.r) / (l_i - theta) (the
// correction equation solved on the FP32 spectral basis), until |r| reaches
// rounding level.  One FP64 matrix-vector product per step instead of an FP64
// O(k^3) reduction: GB300's FP64 pipe is narrow and a one-CTA FP64 reduction
// is latency bound.  The phases are laid out for latency: a thread per row in
// the reduction (four barriers per reflector), 256/k threads per eigenvalue
// in the multisection, and aligned groups of g lanes per column or row (one
// warp each, no block barrier) in the back-transform and the refinement's
// products.  Returns false (the caller takes the FP64 path) for a
// near-degenerate lowest pair or when the refinement does not reach rounding
// level.

// sum over aligned groups of g lanes (g a power of two <= 32); every lane of
// the warp takes part
template <typename T>
__device__ __forceinline__ T group_sum(T v, int g) {
  for (int o = g >> 1; o > 0; o >>= 1) v += __shfl_xor_sync(QDKGB_FULL_MASK, v, o);
  return v;
}

// smem: doubles y, w (kEigMixedMaxK each); region R of k*k doubles (the FP32
// matrix / reflectors A[k*k] and the inverse-iteration pivots Dv[k*k] first,
// the FP64 matrix in the refinement); floats Q[k*ldq] (Q[r*ldq + i] =
// component r of eigenvector i, ldq = k | 1), d, e, e2, beta, lam, lamhi, vec
// (kEigMixedMaxK each), red[32]
static __device__ bool lowest_eig_mixed_cta(int k, const double* __restrict__ H, int ldh, int nev, double* eval,
                                     double* evec, unsigned char* smem) {
  const int tid = threadIdx.x, nt = blockDim.x;
  const int wid = tid >> 5, lane = tid & 31;
  const int ldq = k | 1;
  double* y = reinterpret_cast<double*>(smem);
  double* w = y + kEigMixedMaxK;
  double* R = w + kEigMixedMaxK;
  float* A = reinterpret_cast<float*>(R);
  float* Dv = A + (size_t)k * k;
  float* Q = reinterpret_cast<float*>(R + (size_t)k * k);
  float* d = Q + (size_t)k * ldq;
  float* e = d + kEigMixedMaxK;
  float* e2 = e + kEigMixedMaxK;
  float* beta = e2 + kEigMixedMaxK;
  float* lam = beta + kEigMixedMaxK;
  float* lamhi = lam + kEigMixedMaxK;
  float* vec = lamhi + kEigMixedMaxK;
  float* red = vec + kEigMixedMaxK;  // [0, 8): |x|^2 partials, [16, 24): v.p partials
  __shared__ int s_cnt[kEigThreads];
  __shared__ int s_ok;
  int g = 8;  // lanes per column / row in the grouped phases, g * k <= nt
  while (g > 1 && g * k > nt) g >>= 1;
  const int gc = tid / g, gs = tid - (tid / g) * g;
  auto Hat = [&](int i, int j) { return i >= j ? H[i + (size_t)j * ldh] : H[j + (size_t)i * ldh]; };
  for (int t = tid; t < k * k; t += nt) A[t] = (float)Hat(t % k, t / k);
  __syncthreads();
  // ---- FP32 Householder tridiagonalisation, thread per row (reflector j kept
  // below A(j+1, j); A stays symmetric)
  const int nwr = (k + 31) >> 5;
  for (int j = 0; j + 2 < k; ++j) {
    const int m0 = j + 1;
    const bool row = tid >= m0 && tid < k;
    const float xi = row ? A[tid + k * j] : 0.f;
    float sw = warp_sum(xi * xi);
    if (lane == 0 && wid < nwr) red[wid] = sw;
    __syncthreads();
    float xx = 0.f;
    for (int q = 0; q < nwr; ++q) xx += red[q];
    const float x0 = A[m0 + k * j];
    const float nrm = sqrtf(xx);
    float alpha = 0.f, v0 = x0, b = 0.f;
    if (nrm != 0.f) {
      alpha = (x0 >= 0.f) ? -nrm : nrm;
      v0 = x0 - alpha;
      const float vv = xx - x0 * x0 + v0 * v0;
      b = (vv > 0.f) ? 2.f / vv : 0.f;
    }
    if (tid == 0) {
      beta[j] = b;
      e[j] = alpha;
      d[j] = A[j + k * j];
    }
    if (b == 0.f) {  // the same in every thread
      __syncthreads();
      continue;
    }
    const float vi = row ? (tid == m0 ? v0 : xi) : 0.f;
    float p = 0.f;
    if (row) {
      p = A[tid + k * m0] * v0;
      for (int l = m0 + 1; l < k; ++l) p += A[tid + k * l] * A[l + k * j];
      p *= b;
    }
    sw = warp_sum(vi * p);
    if (lane == 0 && wid < nwr) red[16 + wid] = sw;
    __syncthreads();
    float vp = 0.f;
    for (int q = 0; q < nwr; ++q) vp += red[16 + q];
    const float wi = p - 0.5f * b * vp * vi;
    if (row) vec[tid] = wi;
    if (tid == m0) A[m0 + k * j] = v0;
    __syncthreads();
    if (row) {
      for (int l = m0; l < k; ++l) {
        const float vl = (l == m0) ? v0 : A[l + k * j];
        A[tid + k * l] -= vi * vec[l] + wi * vl;
      }
    }
    __syncthreads();
  }
  if (tid == 0) {
    d[k - 2] = A[(k - 2) + k * (k - 2)];
    e[k - 2] = A[(k - 1) + k * (k - 2)];
    beta[k - 2] = 0.f;
    d[k - 1] = A[(k - 1) + k * (k - 1)];
    beta[k - 1] = 0.f;
  }
  __syncthreads();
  for (int i = tid; i < k - 1; i += nt) e2[i] = e[i] * e[i];
  __syncthreads();
  // ---- all eigenvalues: multisection on the Sturm pivots (a count, not a
  // value, is needed: fast reciprocal), ps = nt / k points per eigenvalue and
  // round, to 2.4e-7 of the spectral scale
  float glo = 0.f, ghi = 0.f;
  for (int i = 0; i < k; ++i) {
    const float r = (i > 0 ? fabsf(e[i - 1]) : 0.f) + (i + 1 < k ? fabsf(e[i]) : 0.f);
    glo = (i == 0) ? d[i] - r : fminf(glo, d[i] - r);
    ghi = (i == 0) ? d[i] + r : fmaxf(ghi, d[i] + r);
  }
  const float scale = fmaxf(fabsf(glo), fabsf(ghi));
  const float tiny = 1e-30f + 1e-12f * scale;
  const float lo0 = glo - 1e-6f * scale - tiny, hi0 = ghi + 1e-6f * scale + tiny;
  const int ps = nt / k;
  const int ei = tid / ps, es = tid - (tid / ps) * ps;
  const float fden = (float)(ps + 1);
  int rounds = 0;
  for (float wd = hi0 - lo0; wd > 2.4e-7f * scale + tiny && rounds < 64; wd /= fden) ++rounds;
  for (int i = tid; i < k; i += nt) {
    lam[i] = lo0;
    lamhi[i] = hi0;
  }
  __syncthreads();
  for (int rd = 0; rd < rounds; ++rd) {
    if (ei < k) {
      const float lo = lam[ei], hi = lamhi[ei];
      const float x = lo + (hi - lo) * ((float)(es + 1) / fden);
      int cnt = 0;
      float q = d[0] - x;
      if (fabsf(q) < tiny) q = -tiny;
      cnt += q < 0.f;
      for (int r = 1; r < k; ++r) {
        q = (d[r] - x) - __fdividef(e2[r - 1], q);
        if (fabsf(q) < tiny) q = -tiny;
        cnt += q < 0.f;
      }
      s_cnt[tid] = cnt;
    }
    __syncthreads();
    if (ei < k && es == 0) {
      const float lo = lam[ei], hi = lamhi[ei];
      int t = ps;  // first point whose count exceeds ei
      for (int q = 0; q < ps; ++q) {
        if (s_cnt[tid + q] > ei) {
          t = q;
          break;
        }
      }
      lam[ei] = (t == 0) ? lo : lo + (hi - lo) * ((float)t / fden);
      lamhi[ei] = (t == ps) ? hi : lo + (hi - lo) * ((float)(t + 1) / fden);
    }
    __syncthreads();
  }
  for (int i = tid; i < k; i += nt) lam[i] = 0.5f * (lam[i] + lamhi[i]);
  __syncthreads();
  // near-degenerate lowest pair: the FP32 basis cannot separate it
  if (!(lam[1] - lam[0] > 1e-5f * (scale + 1e-30f))) return false;
  // ---- eigenvectors of T: thread i, inverse iteration (L D L^T of T - s I,
  // tiny pivots replaced, 1/D kept in Dv[r*k + i]), distinct start vectors
  for (int i = tid; i < k; i += nt) {
    const float s = lam[i] + 1e-7f * (scale + 1e-30f) * ((i & 1) ? 1.f : -1.f);
    float Dr = d[0] - s;
    if (fabsf(Dr) < tiny) Dr = tiny;
    float di = __fdividef(1.f, Dr);
    Dv[i] = di;
    for (int r = 1; r < k; ++r) {
      Dr = (d[r] - s) - e2[r - 1] * di;
      if (fabsf(Dr) < tiny) Dr = tiny;
      di = __fdividef(1.f, Dr);
      Dv[r * k + i] = di;
    }
    for (int r = 0; r < k; ++r) Q[r * ldq + i] = 1.f + 0.37f * (float)(((r + 1) * (i + 3)) % 7) - 1.1f;
    for (int pass = 0; pass < 2; ++pass) {
      // L D L^T z_new = z: L_{r,r-1} = e_{r-1} / D_{r-1}
      float zp = Q[i];
      for (int r = 1; r < k; ++r) {
        const float zr = Q[r * ldq + i] - e[r - 1] * Dv[(r - 1) * k + i] * zp;
        Q[r * ldq + i] = zr;
        zp = zr;
      }
      float zn = Q[(k - 1) * ldq + i] * Dv[(k - 1) * k + i];
      Q[(k - 1) * ldq + i] = zn;
      float mx = fabsf(zn);
      for (int r = k - 2; r >= 0; --r) {
        const float dr = Dv[r * k + i];
        const float zr = Q[r * ldq + i] * dr - e[r] * dr * zn;
        Q[r * ldq + i] = zr;
        zn = zr;
        mx = fmaxf(mx, fabsf(zr));
      }
      const float inv = mx > 0.f ? __fdividef(1.f, mx) : 1.f;
      for (int r = 0; r < k; ++r) Q[r * ldq + i] *= inv;
    }
    float nn = 0.f;
    for (int r = 0; r < k; ++r) nn += Q[r * ldq + i] * Q[r * ldq + i];
    const float inv = rsqrtf(nn);
    for (int r = 0; r < k; ++r) Q[r * ldq + i] *= inv;
  }
  __syncthreads();
  // ---- back-transform Q <- H_0 ... H_{k-3} Q: column gc by its g lanes
  for (int j = k - 3; j >= 0; --j) {
    const float b = beta[j];
    if (b != 0.f) {
      const float* v = A + k * j;
      float dv = 0.f;
      if (gc < k)
        for (int r = j + 1 + gs; r < k; r += g) dv += v[r] * Q[r * ldq + gc];
      dv = group_sum(dv, g) * b;
      if (gc < k)
        for (int r = j + 1 + gs; r < k; r += g) Q[r * ldq + gc] -= dv * v[r];
    }
    __syncwarp();
  }
  __syncthreads();
  // ---- FP64 refinement of the lowest pair; the FP64 matrix replaces the
  // reflectors in shared memory (full, symmetric).  y is kept unnormalised:
  // theta = y.w / y.y, |r| / |y|.  Every warp forms the same sums in the same
  // order, so theta and |r| are known everywhere without a barrier.
  for (int t = tid; t < k * k; t += nt) R[t] = Hat(t % k, t / k);
  for (int i = tid; i < k; i += nt) y[i] = (double)Q[i * ldq];
  __syncthreads();
  const double eps = 1.1102230246251565e-16, hs = (double)scale + 1e-300;
  double theta = 0., rn = 1e300, rprev = 1e300;
  for (int it = 0; it < 8; ++it) {
    double acc = 0.;
    if (gc < k)
      for (int l = gs; l < k; l += g) acc += R[l + (size_t)k * gc] * y[l];
    acc = group_sum(acc, g);
    if (gc < k && gs == 0) w[gc] = acc;
    __syncthreads();
    double yy = 0., yw = 0.;
    for (int i = lane; i < k; i += 32) {
      yy += y[i] * y[i];
      yw += y[i] * w[i];
    }
    yy = warp_sum(yy);
    yw = warp_sum(yw);
    theta = yw / yy;
    double rr = 0.;
    for (int i = lane; i < k; i += 32) {
      const double ri = w[i] - theta * y[i];
      rr += ri * ri;
    }
    rn = sqrt(warp_sum(rr) / yy);
    if (rn <= 16. * eps * hs || (it >= 2 && rn > 0.5 * rprev)) break;
    rprev = rn;
    // c_i = q_i . r / (l_i - theta), i > 0 (FP32), group gc = i
    float c = 0.f;
    if (gc > 0 && gc < k)
      for (int r = gs; r < k; r += g) c += Q[r * ldq + gc] * (float)(w[r] - theta * y[r]);
    c = group_sum(c, g);
    if (gc < k && gs == 0) vec[gc] = (gc > 0) ? c / (lam[gc] - (float)theta) : 0.f;
    __syncthreads();
    // y_r -= sum_{i>0} Q[r, i] c_i, group gc = r
    float dl = 0.f;
    if (gc < k)
      for (int i = 1 + gs; i < k; i += g) dl += Q[gc * ldq + i] * vec[i];
    dl = group_sum(dl, g);
    if (gc < k && gs == 0) y[gc] -= (double)dl;
    __syncthreads();
  }
  if (!(rn <= 4096. * eps * hs)) return false;
  {
    double yy = 0.;
    for (int i = lane; i < k; i += 32) yy += y[i] * y[i];
    const double inv = 1. / sqrt(warp_sum(yy));
    for (int i = tid; i < k; i += nt) evec[i] = y[i] * inv;
  }
  if (tid == 0) eval[0] = theta;
  __syncthreads();
  if (nev == 1) return true;
  // Further columns (a thick-restart basis): the FP32 eigenvectors 1..nev-1,
  // orthonormalised in FP64 against the columns before them (classical
  // Gram-Schmidt twice, one warp); eval[j] = the FP32 eigenvalue.  A vector
  // that loses most of its norm there sends the caller to the FP64 path.
  if (wid == 0) {
    bool ok = true;
    for (int jv = 1; jv < nev && ok; ++jv) {
      double* z = evec + (size_t)jv * k;
      for (int i = lane; i < k; i += 32) w[i] = (double)Q[i * ldq + jv];
      for (int pass = 0; pass < 2; ++pass) {
        for (int q = 0; q < jv; ++q) {
          const double* u = evec + (size_t)q * k;
          double dz = 0.;
          for (int i = lane; i < k; i += 32) dz += u[i] * w[i];
          dz = warp_sum(dz);
          for (int i = lane; i < k; i += 32) w[i] -= dz * u[i];
        }
      }
      double nn = 0.;
      for (int i = lane; i < k; i += 32) nn += w[i] * w[i];
      nn = warp_sum(nn);
      ok = nn > 1e-4;
      const double inv = ok ? 1. / sqrt(nn) : 0.;
      for (int i = lane; i < k; i += 32) z[i] = w[i] * inv;
      if (lane == 0) eval[jv] = (double)lam[jv];
      __syncwarp();
    }
    if (lane == 0) s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// shared-memory bytes of lowest_eig_mixed_cta for size k
__host__ __device__ constexpr size_t eig_mixed_smem(int k) {
  return (2 * (size_t)kEigMixedMaxK + (size_t)k * k) * sizeof(double) +
         ((size_t)k * (k | 1) + 7 * (size_t)kEigMixedMaxK + 32) * sizeof(float);
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
