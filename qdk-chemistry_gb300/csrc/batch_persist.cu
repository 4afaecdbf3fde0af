// Persistent batched CASCI: one launch solves every instance of a shape.
//
// The reference solves a set of active spaces one MacisCas::run at a time
// (qdk_chemistry/algorithms/microsoft/macis_cas.cpp:35-117).  Here a shape's
// instances (emitted slabs in HBM) are solved by a grid of thread-block
// clusters that stays resident for the whole batch: each cluster takes the
// next instance from a device counter and runs its whole mixed-precision
// Davidson (the algorithm of the lockstep path in batch.cu, instance by
// instance) before taking another, so an instance that converges early frees
// its SMs at once and a slow one holds only its own cluster.
//   * bra block: CTA r of a cluster of CL owns the rows [r N/CL, (r+1) N/CL)
//     for every vector operation (preconditioner, Gram-Schmidt, Ritz vector,
//     residual) and takes every CL-th sigma tile;
//   * ket window: a sigma tile is (alpha group, row segment, beta part) with
//     the segment's x slices staged in shared memory (slab_sigma_tile);
//   * reductions: per CTA in warp order, then over the cluster's CTAs in rank
//     order through distributed shared memory - every CTA holds the same
//     totals, so the control flow (convergence, restarts) is uniform;
//   * the projected eigenproblem is solved by the cluster's first CTA and
//     its eigenpair copied to the others through distributed shared memory;
//   * the only waits are cluster barriers (hardware; the CTAs of a cluster are
//     co-scheduled) - no CTA waits on another cluster.
// The cluster size is chosen per shape by a measured autotuner (every
// candidate runs a few iterations of every instance; the fastest is kept and
// recorded on the context).
#include <cooperative_groups.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <vector>

#include "batch_kernels.cuh"
#include "common.cuh"
#include "internal.h"
#include "slab_sigma.cuh"
#include "small_eig.cuh"

namespace qdkgb {

namespace cg = cooperative_groups;

namespace {

constexpr int kPT = 256;       // threads per CTA (the projected eigensolver's CTA size)
constexpr int kPW = kPT / 32;  // warps per CTA
constexpr int kPMaxK = 72;     // values per cluster reduction (subspace + 1, or six restart dots)
constexpr int kSG = 4;         // FP32 sigma: tile groups per CTA, kPT / kSG threads each
constexpr int kSGT = kPT / kSG;
constexpr int kRing = 8;       // FP32 sigma: positions in flight per thread (async copies)

struct BPArgs {
  SlabArgs A;
  PlanArgs P0, P1;  // FP32 plan (4-byte staged x), 8-byte plan (FP64 and float-float)
  int64_t N, nstr;  // determinants; strings per spin of a square space (flip projection)
  int B, m, max_cycles, mixed, square, probe_iters;
  int pipe32;           // FP32 sigma through the async-copy tiles (beta strings a multiple of 4)
  int64_t stage_bytes;  // per tile group: staged x slices + segment record (pipelined tiles)
  double tol, min_abs;
  int64_t vstride;  // slab elements per instance
  const float* hi;
  const float* lo;
  const double* val;
  const double* D;  // [B][N] diagonals
  int* next;        // instance counter
  // per instance
  double* energy;
  double* resid;
  int* iters;
  int* notdone;
  // spin-summed 1-RDMs (norb > 0): [B][norb^2]
  int norb;
  double* rdm;
  const uint64_t* galpha;
  const uint64_t* ubeta;
  const int64_t* acon_ptr;
  const int32_t* acon_idx;
  const int8_t* acon_lvl;
  const int64_t* b1_ptr;
  const int32_t* b1_idx;
  // per cluster: V, AV [m][N]; vec [6][N] (x, xprev, ax, r, t, y); fvec
  // [4][N] (t32, s32, xh, xl); part (sigma partial sums); Hs [m][m] (the
  // projected matrix, lower triangle, kept by the first CTA)
  double* V;
  double* AV;
  double* vec;
  float* fvec;
  unsigned char* part;
  int64_t part_bytes;
  double* Hs;
};

struct Red {
  double w[kPW][kPMaxK];  // warp partials
  double c[kPMaxK];       // this CTA's sums (read by the cluster)
  double t[kPMaxK];       // cluster totals
  double eg[kPMaxK + 1];  // lowest eigenvalue, then its eigenvector
  double minv;
  int64_t mini;
  int inst;
};

// Adds v (this thread's part of value j) into the warp partial of j.
__device__ __forceinline__ void stash(Red& R, double v, int j) {
  v = warp_sum(v);
  if ((threadIdx.x & 31) == 0) R.w[threadIdx.x >> 5][j] = v;
}

// Cluster totals of values 0..nv-1 into R.t: warps in order, then CTAs in
// rank order (every CTA computes the same sums in the same order).
__device__ __forceinline__ void cluster_total(cg::cluster_group& cl, Red& R, int nv) {
  __syncthreads();
  for (int j = threadIdx.x; j < nv; j += kPT) {
    double s = 0.;
    for (int w = 0; w < kPW; ++w) s += R.w[w][j];
    R.c[j] = s;
  }
  cl.sync();
  const int CL = (int)cl.num_blocks();
  for (int j = threadIdx.x; j < nv; j += kPT) {
    double s = 0.;
    for (int r = 0; r < CL; ++r) s += cl.map_shared_rank(R.c, r)[j];
    R.t[j] = s;
  }
  cl.sync();
}

__device__ __forceinline__ double cluster_dot(cg::cluster_group& cl, Red& R, const double* a, const double* b,
                                              int64_t lo, int64_t hi) {
  double acc = 0.;
  for (int64_t i = lo + threadIdx.x; i < hi; i += kPT) acc += a[i] * b[i];
  stash(R, acc, 0);
  cluster_total(cl, R, 1);
  return R.t[0];
}

// this CTA's partial dots A[j] . w over its rows for j < nj (A: columns N
// apart), stashed as values j0 + j; four columns per pass over the rows so
// that each thread keeps five loads in flight.  w is read through L2 when
// other CTAs may have written it (WCG).
template <bool WCG>
__device__ __forceinline__ void slice_multidot(Red& R, const double* __restrict__ A, int64_t N, int nj,
                                               const double* __restrict__ w, int64_t lo, int64_t hi, int j0) {
  for (int jb = 0; jb < nj; jb += 4) {
    const int nb = nj - jb < 4 ? nj - jb : 4;
    const double* a0 = A + (int64_t)jb * N;
    double s0 = 0., s1 = 0., s2 = 0., s3 = 0.;
    if (nb == 4) {
      for (int64_t i = lo + threadIdx.x; i < hi; i += kPT) {
        const double wi = WCG ? __ldcg(w + i) : w[i];
        s0 += a0[i] * wi;
        s1 += a0[N + i] * wi;
        s2 += a0[2 * N + i] * wi;
        s3 += a0[3 * N + i] * wi;
      }
    } else {
      for (int64_t i = lo + threadIdx.x; i < hi; i += kPT) {
        const double wi = WCG ? __ldcg(w + i) : w[i];
        s0 += a0[i] * wi;
        if (nb > 1) s1 += a0[N + i] * wi;
        if (nb > 2) s2 += a0[2 * N + i] * wi;
      }
    }
    stash(R, s0, j0 + jb);
    if (nb > 1) stash(R, s1, j0 + jb + 1);
    if (nb > 2) stash(R, s2, j0 + jb + 2);
    if (nb > 3) stash(R, s3, j0 + jb + 3);
  }
}

// projection on the spin-flip sector s of an nstr x nstr coefficient matrix;
// the pair (i, j), i < j, belongs to the slice holding i * nstr + j, whose
// mirror may lie in another CTA's slice (read and written through L2)
__device__ __forceinline__ void flip_slice(double* t, int64_t nstr, double s, int64_t lo, int64_t hi) {
  for (int64_t q = lo + threadIdx.x; q < hi; q += kPT) {
    const int64_t i = q / nstr, j = q - i * nstr;
    if (i < j) {
      const int64_t mq = j * nstr + i;
      const double avg = 0.5 * (__ldcg(t + q) + s * __ldcg(t + mq));
      __stcg(t + q, avg);
      __stcg(t + mq, s * avg);
    } else if (i == j && s < 0) {
      __stcg(t + q, 0.);
    }
  }
}


__device__ __forceinline__ void cp16_cg(void* dst, const void* src) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}
__device__ __forceinline__ void group_bar(int id) { asm volatile("bar.sync %0, %1;\n" ::"r"(id), "r"(kSGT) : "memory"); }

// One FP32 sigma tile (group g, segment s, part z) by a tile group of kSGT
// threads, four adjacent beta strings per thread: the row values stream into
// a per-thread ring of kRing positions through 16-byte async copies (L2 ->
// shared, no registers held while in flight), each with its beta-list entries
// (own-group and alpha-single blocks) or the alpha double's x (through L2:
// x was written by other CTAs of the kernel).  Per row the products are
// summed in the order of k_slab_sigma32v<4> (own block, then the
// alpha-single blocks level-1 entry by entry, then the alpha doubles), so the
// result is that kernel's bit for bit.
__device__ void pipe_tile32(const SlabArgs& A, const PlanArgs& P, const float* __restrict__ vals,
                            const float* __restrict__ x, float* __restrict__ out, int64_t part_stride, int g, int s,
                            int z, float* xs, int32_t* rec, unsigned char* ring, int bar_id, int lt) {
  const int Nb = A.Nb, nvec = Nb / 4;
  const int32_t* rg = P.rec + ((int64_t)g * P.S + s) * P.R;
  for (int i = lt; i < P.R; i += kSGT) rec[i] = __ldg(rg + i);
  const int32_t* sh = P.segh + ((int64_t)g * P.S + s) * P.M;
  const int q4 = P.M * nvec;
  float4* xs4 = reinterpret_cast<float4*>(xs);
  const float4* x4 = reinterpret_cast<const float4*>(x);
#pragma unroll 4
  for (int q = lt; q < q4; q += kSGT) {
    const int j = q / nvec, i = q - j * nvec;
    const int h = __ldg(sh + j);
    if (h >= 0) xs4[q] = __ldcg(x4 + (int64_t)h * nvec + i);
  }
  group_bar(bar_id);
  const int t = z * kSGT + lt;
  if (t < nvec) {
    const int has0 = rec[0], off0 = rec[1], sb0 = rec[2], n1b = rec[3];
    const int32_t* e1 = rec + 4;
    const int nd = rec[4 + 2 * n1b];
    const int32_t* e2 = rec + 6 + 2 * n1b;
    const int n_own = has0 ? A.n2 : 0, n_sing = A.n1 * n1b;
    const int L = n_own + n_sing + nd;
    const int b0 = t * 4;
    const float* vg = vals + (int64_t)g * A.rowlen * Nb + b0;
    float4* rv = reinterpret_cast<float4*>(ring);
    uint4* ra = reinterpret_cast<uint4*>(ring + kRing * 16);
    auto issue = [&](int q) {
      const int slot = q & (kRing - 1);
      int64_t voff;
      const void* asrc;
      if (q < n_own) {
        voff = off0 + (int64_t)q * Nb;
        asrc = A.blT + (int64_t)q * Nb + b0;
      } else if (q < n_own + n_sing) {
        const int u = q - n_own, k = u / n1b, e = u - k * n1b;
        voff = e1[2 * e] + (int64_t)k * Nb;
        asrc = A.blT + (int64_t)(A.n2 + k) * Nb + b0;
      } else {
        const int j = q - n_own - n_sing;
        voff = e2[2 * j];
        asrc = x + e2[2 * j + 1] + b0;
      }
      cp16_cg(rv + slot, vg + voff);
      cp16_cg(ra + slot, asrc);
    };
#pragma unroll
    for (int q = 0; q < kRing; ++q) {
      if (q < L) issue(q);
      cp_commit();
    }
    float c0 = 0.f, c1 = 0.f, c2 = 0.f, c3 = 0.f;
    for (int q = 0; q < L; ++q) {
      cp_wait<kRing - 1>();
      const int slot = q & (kRing - 1);
      const float4 v = rv[slot];
      const uint4 au = ra[slot];
      if (q < n_own + n_sing) {
        const int sb = q < n_own ? sb0 : e1[2 * ((q - n_own) % n1b) + 1];
        c0 = fmaf(v.x, xs[sb + (int)au.x], c0);
        c1 = fmaf(v.y, xs[sb + (int)au.y], c1);
        c2 = fmaf(v.z, xs[sb + (int)au.z], c2);
        c3 = fmaf(v.w, xs[sb + (int)au.w], c3);
      } else {
        c0 = fmaf(v.x, __uint_as_float(au.x), c0);
        c1 = fmaf(v.y, __uint_as_float(au.y), c1);
        c2 = fmaf(v.z, __uint_as_float(au.z), c2);
        c3 = fmaf(v.w, __uint_as_float(au.w), c3);
      }
      if (q + kRing < L) issue(q + kRing);
      cp_commit();
    }
    cp_wait<0>();
    *reinterpret_cast<float4*>(out + s * part_stride + (int64_t)g * Nb + b0) = make_float4(c0, c1, c2, c3);
  }
  group_bar(bar_id);
}

// y = H x for the cluster's instance: sigma tiles round-robin over the CTAs
// into the partial buffer, then each CTA sums its own rows' segments (in
// order) into y (so y's slice is written by its owner).
template <int MODE>
__device__ void cluster_sigma(const BPArgs& a, cg::cluster_group& cl, const void* vals, const float* vlo,
                              const void* x, const float* xlo, void* y, unsigned char* part, unsigned char* smem,
                              int64_t lo, int64_t hi) {
  using Out = typename SlabPol<MODE>::Out;
  const PlanArgs& P = MODE == 0 ? a.P0 : a.P1;
  const int rank = (int)cl.block_rank(), CL = (int)cl.num_blocks();
  if (MODE == 0 && a.pipe32) {
    // tile groups of kSGT threads, each on its own tiles and staging
    const int sg = threadIdx.x / kSGT, lt = threadIdx.x - sg * kSGT;
    const int Zp = (a.A.Nb / 4 + kSGT - 1) / kSGT;
    const int64_t tiles = (int64_t)a.A.G * P.S * Zp;
    float* xs = reinterpret_cast<float*>(smem + sg * a.stage_bytes);
    int32_t* rec = reinterpret_cast<int32_t*>(smem + sg * a.stage_bytes + (int64_t)P.M * a.A.Nb * 4);
    unsigned char* ring = smem + kSG * a.stage_bytes + (int64_t)threadIdx.x * (2 * kRing * 16);
    for (int64_t t = (int64_t)rank * kSG + sg; t < tiles; t += (int64_t)CL * kSG) {
      const int z = (int)(t % Zp);
      const int64_t gs = t / Zp;
      const int s = (int)(gs % P.S), g = (int)(gs / P.S);
      pipe_tile32(a.A, P, (const float*)vals, (const float*)x, (float*)part, a.N, g, s, z, xs, rec, ring, 1 + sg, lt);
    }
    __syncthreads();
  } else {
    const int Z = (a.A.Nb + kPT - 1) / kPT;
    const int64_t tiles = (int64_t)a.A.G * P.S * Z;
    for (int64_t t = rank; t < tiles; t += CL) {
      const int z = (int)(t % Z);
      const int64_t gs = t / Z;
      const int s = (int)(gs % P.S), g = (int)(gs / P.S);
      slab_sigma_tile<MODE, true>(a.A, P, vals, vlo, x, xlo, part, a.N, g, s, z, smem);
      __syncthreads();
    }
  }
  cl.sync();
  const Out* pp = (const Out*)part;
  for (int64_t i = lo + threadIdx.x; i < hi; i += kPT) {
    Out acc = __ldcg(pp + i);
    for (int s = 1; s < P.S; ++s) acc += __ldcg(pp + (int64_t)s * a.N + i);
    ((Out*)y)[i] = acc;
  }
}

__global__ void __launch_bounds__(kPT) k_bp_solve(BPArgs a) {
  extern __shared__ __align__(16) unsigned char dsm[];
  __shared__ Red R;
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank(), CL = (int)cl.num_blocks();
  const int64_t cid = blockIdx.x / CL;
  const int64_t N = a.N, m = a.m;
  const int64_t sl = (N + CL - 1) / CL;
  const int64_t lo = rank * sl < N ? rank * sl : N, hi = lo + sl < N ? lo + sl : N;
  const int tid = threadIdx.x;
  double* V = a.V + cid * m * N;
  double* AV = a.AV + cid * m * N;
  double* x = a.vec + cid * 6 * N;
  double* xprev = x + N;
  double* ax = x + 2 * N;
  double* r = x + 3 * N;
  double* t = x + 4 * N;
  double* y = x + 5 * N;
  float* t32 = a.fvec + cid * 4 * N;
  float* s32 = t32 + N;
  float* xh = t32 + 2 * N;
  float* xl = t32 + 3 * N;
  unsigned char* part = a.part + cid * a.part_bytes;
  double* Hs = a.Hs + cid * m * m;
  for (;;) {
    if (rank == 0 && tid == 0) R.inst = atomicAdd(a.next, 1);
    cl.sync();
    const int inst = *cl.map_shared_rank(&R.inst, 0);
    cl.sync();
    if (inst >= a.B) break;
    const double* D = a.D + (int64_t)inst * N;
    const float* hi32 = a.hi ? a.hi + (int64_t)inst * a.vstride : nullptr;
    const float* lo32 = a.lo ? a.lo + (int64_t)inst * a.vstride : nullptr;
    const double* v64 = a.val ? a.val + (int64_t)inst * a.vstride : nullptr;
    // ---- guess: the lowest diagonal element (first on ties)
    int64_t gmin = N;
    {
      double best = INFINITY;
      int64_t bi = N;
      for (int64_t i = lo + tid; i < hi; i += kPT) {
        const double v = __ldg(D + i);
        if (v < best || (v == best && i < bi)) {
          best = v;
          bi = i;
        }
      }
      for (int d = 16; d > 0; d >>= 1) {
        const double ov = __shfl_xor_sync(QDKGB_FULL_MASK, best, d);
        const int64_t oi = __shfl_xor_sync(QDKGB_FULL_MASK, bi, d);
        if (ov < best || (ov == best && oi < bi)) {
          best = ov;
          bi = oi;
        }
      }
      if ((tid & 31) == 0) {
        R.w[tid >> 5][0] = best;
        R.w[tid >> 5][1] = (double)bi;
      }
      __syncthreads();
      if (tid == 0) {
        double bv = INFINITY;
        int64_t bix = N;
        for (int w = 0; w < kPW; ++w) {
          const double v = R.w[w][0];
          const int64_t i = (int64_t)R.w[w][1];
          if (v < bv || (v == bv && i < bix)) {
            bv = v;
            bix = i;
          }
        }
        R.minv = bv;
        R.mini = bix;
      }
      cl.sync();
      double bv = INFINITY;
      int64_t bix = N;
      for (int q = 0; q < CL; ++q) {
        const double v = *cl.map_shared_rank(&R.minv, q);
        const int64_t i = *cl.map_shared_rank(&R.mini, q);
        if (v < bv || (v == bv && i < bix)) {
          bv = v;
          bix = i;
        }
      }
      cl.sync();
      for (int64_t i = lo + tid; i < hi; i += kPT) x[i] = (i == bix) ? 1. : 0.;
      gmin = bix;
    }
    // the guess's spin-flip sector (kept by the FP64 iteration; FP32 noise is
    // projected out of new directions, as in the single solve)
    const double flip = (a.square && a.mixed) ? ((gmin / a.nstr == gmin % a.nstr) ? 1. : 0.) : 0.;
    int k = 0, act = 0, done = 0, nsig = 0, nref = 0;
    double theta = 0., last_true = 0., energy = 0., resn = 0.;
    // projected row k of Hs from the values R.t[0..k] (first CTA)
    auto set_row = [&](int kk) {
      if (rank == 0)
        for (int j = tid; j <= kk; j += kPT) Hs[kk + (int64_t)j * m] = R.t[j];
      __syncthreads();
    };
    // lowest pair of the leading k x k block (first CTA, then copied to the
    // others), the Ritz vector x = V y, ax = AV y, r = ax - theta x (previous
    // x kept); returns |r|^2
    auto ritz = [&]() -> double {
      if (rank == 0) lowest_eig_cta(k, Hs, (int)m, nullptr, 1, R.eg, R.eg + 1);
      cl.sync();
      if (rank != 0) {
        const double* src = cl.map_shared_rank(R.eg, 0);
        for (int j = tid; j <= k; j += kPT) R.eg[j] = src[j];
      }
      cl.sync();
      theta = R.eg[0];
      double acc = 0.;
      for (int64_t i = lo + tid; i < hi; i += kPT) {
        double sx = 0., sa = 0.;
#pragma unroll 4
        for (int j = 0; j < k; ++j) {
          const double c = R.eg[1 + j];
          sx += V[j * N + i] * c;
          sa += AV[j * N + i] * c;
        }
        const double rr = sa - theta * sx;
        xprev[i] = x[i];
        x[i] = sx;
        ax[i] = sa;
        r[i] = rr;
        acc += rr * rr;
      }
      stash(R, acc, 0);
      cluster_total(cl, R, 1);
      return R.t[0];
    };
    // refresh: normalised x, its full-precision sigma and residual; the
    // convergence test; from the second cycle on (gd) the subspace restarts
    // on [x, second vector] (GD+1)
    auto refresh = [&](bool gd) {
      const double nrm = cluster_dot(cl, R, x, x, lo, hi);
      const double inv = 1. / sqrt(nrm);
      for (int64_t i = lo + tid; i < hi; i += kPT) {
        const double q = x[i] * inv;
        x[i] = q;
        V[i] = q;
        const float h = __double2float_rn(q);
        xh[i] = h;
        xl[i] = __double2float_rn(q - (double)h);
      }
      if (gd) {
        if (flip != 0.) {
          cl.sync();
          flip_slice(xprev, a.nstr, flip, lo, hi);
          flip_slice(r, a.nstr, flip, lo, hi);
          cl.sync();
        }
        double d6[6] = {0., 0., 0., 0., 0., 0.};
        for (int64_t i = lo + tid; i < hi; i += kPT) {
          const double xi = x[i], p = __ldcg(xprev + i), q = __ldcg(r + i), z = filler(i, a.nstr, flip);
          d6[0] += xi * p;
          d6[1] += p * p;
          d6[2] += xi * q;
          d6[3] += q * q;
          d6[4] += xi * z;
          d6[5] += z * z;
        }
        for (int j = 0; j < 6; ++j) stash(R, d6[j], j);
        cluster_total(cl, R, 6);
        const double* d = R.t;
        int pick = 2;
        double nrm2 = d[5] - d[4] * d[4];
        if (d[1] - d[0] * d[0] > 1e-8 * d[1]) {
          pick = 0;
          nrm2 = d[1] - d[0] * d[0];
        } else if (d[3] - d[2] * d[2] > 1e-8 * d[3]) {
          pick = 1;
          nrm2 = d[3] - d[2] * d[2];
        }
        const double c = d[2 * pick], inv2 = 1. / sqrt(nrm2);
        for (int64_t i = lo + tid; i < hi; i += kPT) {
          const double v = pick == 0 ? __ldcg(xprev + i) : (pick == 1 ? __ldcg(r + i) : filler(i, a.nstr, flip));
          const double q = (v - c * x[i]) * inv2;
          V[N + i] = q;
          if (a.mixed) {
            const float h = __double2float_rn(q);
            t32[i] = h;
            s32[i] = __double2float_rn(q - (double)h);
          } else {
            t[i] = q;
          }
        }
        cl.sync();
        if (a.mixed)
          cluster_sigma<2>(a, cl, hi32, lo32, t32, s32, ax, part, dsm, lo, hi);
        else
          cluster_sigma<1>(a, cl, v64, nullptr, t, nullptr, ax, part, dsm, lo, hi);
      }
      cl.sync();
      if (a.mixed)
        cluster_sigma<2>(a, cl, hi32, lo32, xh, xl, y, part, dsm, lo, hi);
      else
        cluster_sigma<1>(a, cl, v64, nullptr, x, nullptr, y, part, dsm, lo, hi);
      const double th = cluster_dot(cl, R, x, y, lo, hi);
      double acc = 0.;
      for (int64_t i = lo + tid; i < hi; i += kPT) {
        const double yy = y[i];
        AV[i] = yy;
        const double rr = yy - th * x[i];
        r[i] = rr;
        acc += rr * rr;
      }
      stash(R, acc, 0);
      cluster_total(cl, R, 1);
      ++nref;
      theta = th;
      energy = th;
      resn = sqrt(R.t[0]);
      if (resn < a.tol) {
        done = 1;
        act = 0;
        return;
      }
      act = 1;
      last_true = resn;
      if (rank == 0 && tid == 0) Hs[0] = th;
      __syncthreads();
      k = 1;
      if (gd) {
        for (int64_t i = lo + tid; i < hi; i += kPT) AV[N + i] = ax[i];
        for (int j = 0; j < 2; ++j) {
          double s = 0.;
          for (int64_t i = lo + tid; i < hi; i += kPT) s += AV[j * N + i] * V[N + i];
          stash(R, s, j);
        }
        cluster_total(cl, R, 2);
        set_row(1);
        k = 2;
        ritz();
      }
    };
    // one inner iteration: new direction from (r, theta), its FP32 sigma, the
    // projected row, the Ritz pair; the instance waits for the next refresh
    // when its estimated residual fell by 1e-4 or the subspace is full
    auto inner = [&]() {
      for (int64_t i = lo + tid; i < hi; i += kPT) {
        double d = __ldg(D + i) - theta;
        if (fabs(d) < a.min_abs) d = (d >= 0) ? a.min_abs : -a.min_abs;
        t[i] = -r[i] / d;
      }
      if (flip != 0.) {
        cl.sync();
        flip_slice(t, a.nstr, flip, lo, hi);
        cl.sync();
      }
      // Gram-Schmidt against V[0..k): two passes in the FP64 form; in the
      // mixed form the second only when the first removed more than half of
      // |t|^2 (as the lockstep path)
      auto tnorm2 = [&]() -> double {
        double q2 = 0.;
        for (int64_t i = lo + tid; i < hi; i += kPT) {
          const double q = __ldcg(t + i);
          q2 += q * q;
        }
        stash(R, q2, 0);
        cluster_total(cl, R, 1);
        return R.t[0];
      };
      const double w0 = a.mixed ? tnorm2() : 0.;
      double nn = -1.;
      for (int pass = 0; pass < 2; ++pass) {
        slice_multidot<true>(R, V, N, k, t, lo, hi, 0);
        cluster_total(cl, R, k);
        for (int64_t i = lo + tid; i < hi; i += kPT) {
          double acc = 0.;
#pragma unroll 4
          for (int j = 0; j < k; ++j) acc += V[j * N + i] * R.t[j];
          __stcg(t + i, __ldcg(t + i) - acc);
        }
        if (pass == 0 && a.mixed) {
          nn = tnorm2();
          if (nn > 0.5 * w0) break;
          nn = -1.;
        }
      }
      if (nn < 0.) nn = tnorm2();
      if (!(nn > 1e-28)) {  // no new direction: wait for the cycle's end
        act = 0;
        return;
      }
      ++nsig;
      const double inv = 1. / sqrt(nn);
      for (int64_t i = lo + tid; i < hi; i += kPT) {
        const double q = __ldcg(t + i) * inv;
        V[k * N + i] = q;
        __stcg(t + i, q);
        t32[i] = __double2float_rn(q);
      }
      cl.sync();
      if (a.mixed) {
        cluster_sigma<0>(a, cl, hi32, nullptr, t32, nullptr, s32, part, dsm, lo, hi);
        for (int64_t i = lo + tid; i < hi; i += kPT) AV[k * N + i] = (double)s32[i];
      } else {
        cluster_sigma<1>(a, cl, v64, nullptr, t, nullptr, y, part, dsm, lo, hi);
        for (int64_t i = lo + tid; i < hi; i += kPT) AV[k * N + i] = y[i];
      }
      // projected row k: Hs(k, j) = AV[j] . V[k], j <= k
      slice_multidot<false>(R, AV, N, k + 1, V + k * N, lo, hi, 0);
      cluster_total(cl, R, k + 1);
      set_row(k);
      ++k;
      const double est2 = ritz();
      if (k >= m || sqrt(est2) < 1e-4 * last_true) act = 0;
    };
    refresh(false);
    int cycles = 0;
    while (!done) {
      if (++cycles > max(1, a.max_cycles)) break;
      for (int it = 1; it < m && act; ++it) {
        inner();
        if (a.probe_iters > 0 && nsig >= a.probe_iters) break;
      }
      if (a.probe_iters > 0 && nsig >= a.probe_iters) break;
      refresh(true);
    }
    if (rank == 0 && tid == 0) {
      a.energy[inst] = energy;
      a.resid[inst] = resn;
      a.iters[inst] = nsig + nref;
      a.notdone[inst] = done ? 0 : 1;
    }
    if (a.norb > 0) {
      cl.sync();
      if (rank == 0)
        rdm1_cta(x, a.A.G, a.A.Nb, a.norb, a.galpha, a.ubeta, a.acon_ptr, a.acon_idx, a.acon_lvl, a.b1_ptr,
                 a.b1_idx, a.rdm + (int64_t)inst * a.norb * a.norb, reinterpret_cast<double*>(dsm));
    }
    cl.sync();
  }
}

constexpr int kProbeIters = 4;  // inner iterations per instance in one tuning run

struct Launch {
  cudaLaunchConfig_t cfg{};
  cudaLaunchAttribute attr[1];
  Launch(int CL, int ncl, size_t smem, cudaStream_t s) {
    cfg.gridDim = dim3((unsigned)(CL * ncl));
    cfg.blockDim = dim3(kPT);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)CL;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
  }
};

// clusters of CL CTAs resident at once (0: the kernel does not fit, or the
// device refuses the cluster shape)
int resident_clusters(int CL, size_t smem, cudaStream_t s) {
  Launch L(CL, 1, smem, s);
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, (const void*)k_bp_solve, &L.cfg) != cudaSuccess) {
    (void)cudaGetLastError();
    return 0;
  }
  return n;
}

}  // namespace

void batch_solve_persistent(Context* cc, Context* owner, const BatchShapeJob& job) {
  NvtxRange nvtx_range("qdkgb.casci_batch_persistent");
  const int64_t N = job.N;
  const int m = job.m;
  const int n2 = job.norb * job.norb;
  BPArgs a{};
  a.A = slab_args(cc);
  a.P0 = slab_plan_args(cc, 0);
  a.P1 = slab_plan_args(cc, 1);
  a.N = N;
  a.nstr = job.nstr;
  a.B = job.B;
  a.m = m;
  a.max_cycles = job.max_cycles;
  a.mixed = job.mixed ? 1 : 0;
  a.square = job.square ? 1 : 0;
  a.tol = job.tol;
  a.min_abs = job.min_abs;
  a.vstride = job.vstride;
  a.hi = job.hi;
  a.lo = job.lo;
  a.val = job.val;
  a.D = job.D;
  a.energy = job.energy;
  a.resid = job.resid;
  a.iters = job.iters;
  a.notdone = job.notdone;
  a.norb = job.rdm ? job.norb : 0;
  a.rdm = job.rdm;
  const DetSpace& S = cc->dets;
  a.galpha = (const uint64_t*)S.galpha.ptr;
  a.ubeta = (const uint64_t*)S.ubeta.ptr;
  a.acon_ptr = (const int64_t*)S.acon_ptr.ptr;
  a.acon_idx = (const int32_t*)S.acon_idx.ptr;
  a.acon_lvl = (const int8_t*)S.acon_lvl.ptr;
  a.b1_ptr = (const int64_t*)S.b1_ptr.ptr;
  a.b1_idx = (const int32_t*)S.b1_idx.ptr;
  size_t smem = std::max(slab_plan_smem(cc, 0, 4), slab_plan_smem(cc, 1, 8));
  // the FP32 sigma's async-copy tiles: four beta strings per thread in
  // 16-byte copies (beta strings a multiple of 4), kSG staging areas and the
  // per-thread rings within the shared-memory budget
  {
    const int64_t stage = ((int64_t)a.P0.M * a.A.Nb * 4 + (int64_t)a.P0.R * 4 + 15) / 16 * 16;
    const int64_t pipe = kSG * stage + (int64_t)kPT * 2 * kRing * 16;
    a.pipe32 = (a.A.Nb % 4 == 0 && pipe + 32 * 1024 <= 227 * 1024) ? 1 : 0;
    a.stage_bytes = stage;
    if (a.pipe32) smem = std::max(smem, (size_t)pipe);
  }
  smem = std::max(smem, eig_dyn_smem(m));
  smem = std::max(smem, (size_t)n2 * sizeof(double));
  smem = (smem + 15) / 16 * 16;
  set_max_dynamic_smem((const void*)k_bp_solve, (int)smem);
  cudaStream_t st = cc->stream;
  // candidates: CTAs per instance; each CTA keeps at least 2048 rows
  std::vector<int> cand;
  if (job.cluster > 0) {
    cand.push_back(job.cluster);
  } else {
    for (int CL : {1, 2, 4, 8})
      if (CL == 1 || N / CL >= 2048) cand.push_back(CL);
  }
  std::vector<int> ncl;
  {
    std::vector<int> fit;
    for (int CL : cand) {
      const int n = std::min(job.B, resident_clusters(CL, smem, st));
      if (n >= 1) {
        fit.push_back(CL);
        ncl.push_back(n);
      }
    }
    if (fit.empty())
      throw Error(QDKGB_ERR_UNSUPPORTED, "batched CASCI: no cluster shape of the persistent solver fits the device");
    cand.swap(fit);
  }
  int max_ncl = 0;
  for (int n : ncl) max_ncl = std::max(max_ncl, n);
  // per-cluster workspace for the largest cluster count among the candidates
  const int64_t part_bytes = (std::max<int64_t>((int64_t)a.P0.S * N * 4, (int64_t)a.P1.S * N * 8) + 255) / 256 * 256;
  ScopedBuffers<7> ws(cc);
  a.V = dev_array<double>(cc, ws.b[0], (size_t)max_ncl * m * N);
  a.AV = dev_array<double>(cc, ws.b[1], (size_t)max_ncl * m * N);
  a.vec = dev_array<double>(cc, ws.b[2], (size_t)max_ncl * 6 * N);
  a.fvec = dev_array<float>(cc, ws.b[3], (size_t)max_ncl * 4 * N);
  a.part = dev_array<unsigned char>(cc, ws.b[4], (size_t)max_ncl * part_bytes);
  a.part_bytes = part_bytes;
  a.Hs = dev_array<double>(cc, ws.b[5], (size_t)max_ncl * m * m);
  a.next = dev_array<int>(cc, ws.b[6], 1);
  auto run = [&](size_t i, int probe) {
    a.probe_iters = probe;
    QDKGB_CUDA(cudaMemsetAsync(a.next, 0, sizeof(int), st));
    Launch L(cand[i], ncl[i], smem, st);
    QDKGB_CUDA(cudaLaunchKernelEx(&L.cfg, k_bp_solve, a));
    QDKGB_CHECK_LAUNCH();
  };
  // the shape's tuned cluster size, measured on first use
  BatchTune* rec = nullptr;
  for (BatchTune& t : owner->batch_tune)
    if (t.norb == job.norb && t.na == job.na && t.nb == job.nb && t.m == m && t.mixed == a.mixed) rec = &t;
  size_t pick = 0;
  if (cand.size() > 1) {
    if (!rec) {
      owner->batch_tune.push_back(BatchTune{job.norb, job.na, job.nb, m, a.mixed, 0, {}});
      rec = &owner->batch_tune.back();
      cudaEvent_t e0, e1;
      QDKGB_CUDA(cudaEventCreate(&e0));
      QDKGB_CUDA(cudaEventCreate(&e1));
      double best = 1e300;
      for (size_t i = 0; i < cand.size(); ++i) {
        QDKGB_CUDA(cudaEventRecord(e0, st));
        run(i, kProbeIters);
        QDKGB_CUDA(cudaEventRecord(e1, st));
        QDKGB_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        QDKGB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        rec->cand_ms.push_back({cand[i], (double)ms});
        if (ms < best) {
          best = ms;
          rec->cluster = cand[i];
        }
      }
      QDKGB_CUDA(cudaEventDestroy(e0));
      QDKGB_CUDA(cudaEventDestroy(e1));
    }
    for (size_t i = 0; i < cand.size(); ++i)
      if (cand[i] == rec->cluster) pick = i;
  }
  run(pick, 0);
  QDKGB_CUDA(cudaStreamSynchronize(st));
}

}  // namespace qdkgb
