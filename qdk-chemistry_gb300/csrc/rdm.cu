// Spin-resolved 1-/2-RDMs (replaces SortedDoubleLoopHamiltonianGenerator::
// form_rdms_spin_dep, include/macis/hamiltonian_generator/
// sorted_double_loop.hpp:626-753, with rdm_contributions_spin_dep<true>,
// include/macis/util/rdms.hpp:39-612).
//
// The pair walk is the CSR build's (no connectivity is stored): one warp per
// bra determinant visits its connected kets, and every unordered pair is
// handled once with the lower-index determinant as bra, as the reference
// does.  Contributions are accumulated in a per-CTA shared-memory tile of one
// spin block (aaaa with aa, bbbb with bb, or aabb), split over ranges of the
// last index when n^4 does not fit, then flushed once to global memory with
// atomics.  For large orbital counts (where the tile would need many passes
// and the targets rarely collide) the kernel accumulates straight into
// global memory.
#include <algorithm>
#include <vector>

#include "common.cuh"
#include "internal.h"
#include "rowwalk.cuh"

namespace qdkgb {

constexpr int kRdmWarps = 16;

struct RdmTarget {
  int block;       // 0: aaaa (+aa), 1: bbbb (+bb), 2: aabb
  int n;
  int s_lo, s_hi;  // last-index range held by the tile
  double* t4;      // tile or global n^4 block
  double* t2;      // tile or global n^2 block (blocks 0, 1)
  bool shared;
  bool with_ordm;  // accumulate the 1-RDM (first last-index slice only)
};

__device__ __forceinline__ void add4(const RdmTarget& T, int blk, uint32_t p, uint32_t q, uint32_t r, uint32_t s,
                                     double v) {
  if (blk != T.block || (int)s < T.s_lo || (int)s >= T.s_hi) return;
  const size_t n = (size_t)T.n;
  atomicAdd(T.t4 + p + n * (q + n * (r + n * (s - T.s_lo))), v);
}
__device__ __forceinline__ void add2(const RdmTarget& T, int blk, uint32_t p, uint32_t q, double v) {
  if (blk != T.block || !T.t2) return;
  atomicAdd(T.t2 + p + (size_t)T.n * q, v);
}

// rdm_contributions_4 (rdms.hpp:39-68), symm
__device__ void rdm_same_spin_double(const RdmTarget& T, int blk, uint64_t bra, uint64_t ket, uint64_t ex, double val) {
  SingleEx a = single_ex(bra, ket, ex);
  const uint64_t flip = (1ull << a.o) | (1ull << a.v);
  SingleEx b = single_ex(bra, ket ^ flip, ex ^ flip);
  const uint32_t o1 = a.o, v1 = a.v, o2 = b.o, v2 = b.v;
  val *= ((a.neg != b.neg) ? -1. : 1.) * 0.5;
  add4(T, blk, v1, o1, v2, o2, val);
  add4(T, blk, v2, o1, v1, o2, -val);
  add4(T, blk, v1, o2, v2, o1, -val);
  add4(T, blk, v2, o2, v1, o1, val);
  add4(T, blk, o2, v2, o1, v1, val);
  add4(T, blk, o2, v1, o1, v2, -val);
  add4(T, blk, o1, v2, o2, v1, -val);
  add4(T, blk, o1, v1, o2, v2, val);
}
// rdm_contributions_22_spin_dep (rdms.hpp:145-167), symm
__device__ void rdm_opposite_spin_double(const RdmTarget& T, uint64_t ba, uint64_t ka, uint64_t exa, uint64_t bb,
                                         uint64_t kb, uint64_t exb, double val) {
  SingleEx a = single_ex(ba, ka, exa);  // (o2, v2): alpha
  SingleEx b = single_ex(bb, kb, exb);  // (o1, v1): beta
  val *= ((a.neg != b.neg) ? -1. : 1.) * 0.5;
  add4(T, 2, b.v, b.o, a.v, a.o, val);
  add4(T, 2, b.o, b.v, a.o, a.v, val);
}
// rdm_contributions_2_spin_dep (rdms.hpp:282-368), symm; transpose for a beta single
__device__ void rdm_single(const RdmTarget& T, int blk_ss, bool transpose, uint64_t bra, uint64_t ket, uint64_t ex,
                           uint64_t occ_os, double val) {
  SingleEx s = single_ex(bra, ket, ex);
  const uint32_t o1 = s.o, v1 = s.v;
  const double sg = s.neg ? -1. : 1.;
  add2(T, blk_ss, v1, o1, sg * val);
  add2(T, blk_ss, o1, v1, sg * val);
  val *= sg * 0.5;
  if (T.block == blk_ss) {
    for (uint64_t m = bra; m; m &= m - 1) {
      const uint32_t p = low_bit(m);
      add4(T, blk_ss, v1, o1, p, p, val);
      add4(T, blk_ss, p, p, v1, o1, val);
      add4(T, blk_ss, v1, p, p, o1, -val);
      add4(T, blk_ss, p, o1, v1, p, -val);
      add4(T, blk_ss, p, p, o1, v1, val);
      add4(T, blk_ss, o1, v1, p, p, val);
      add4(T, blk_ss, o1, p, p, v1, -val);
      add4(T, blk_ss, p, v1, o1, p, -val);
    }
  }
  if (T.block == 2) {
    for (uint64_t m = occ_os; m; m &= m - 1) {
      const uint32_t p = low_bit(m);
      if (transpose) {
        add4(T, 2, v1, o1, p, p, val);
        add4(T, 2, o1, v1, p, p, val);
      } else {
        add4(T, 2, p, p, v1, o1, val);
        add4(T, 2, p, p, o1, v1, val);
      }
    }
  }
}
// rdm_contributions_diag_spin_dep (rdms.hpp:439-516)
__device__ void rdm_diag(const RdmTarget& T, uint64_t oa, uint64_t ob, double val) {
  if (T.block == 0)
    for (uint64_t m = oa; m; m &= m - 1) add2(T, 0, low_bit(m), low_bit(m), val);
  if (T.block == 1)
    for (uint64_t m = ob; m; m &= m - 1) add2(T, 1, low_bit(m), low_bit(m), val);
  val *= 0.5;
  if (T.block == 0 || T.block == 1) {
    const uint64_t o = T.block == 0 ? oa : ob;
    for (uint64_t mq = o; mq; mq &= mq - 1)
      for (uint64_t mp = o; mp; mp &= mp - 1) {
        const uint32_t q = low_bit(mq), p = low_bit(mp);
        add4(T, T.block, p, p, q, q, val);
        add4(T, T.block, p, q, q, p, -val);
      }
  } else {
    for (uint64_t mq = ob; mq; mq &= mq - 1)
      for (uint64_t mp = oa; mp; mp &= mp - 1) add4(T, 2, low_bit(mq), low_bit(mq), low_bit(mp), low_bit(mp), val);
  }
}

__device__ __forceinline__ void rdm_pair(const RdmTarget& T, uint64_t ba, uint64_t bb, uint64_t ka, uint64_t kb,
                                         double val) {
  const uint64_t exa = ba ^ ka, exb = bb ^ kb;
  const int ca = popc64(exa), cb = popc64(exb);
  if (ca == 4) {
    if (T.block == 0) rdm_same_spin_double(T, 0, ba, ka, exa, val);
  } else if (cb == 4) {
    if (T.block == 1) rdm_same_spin_double(T, 1, bb, kb, exb, val);
  } else if (ca == 2 && cb == 2) {
    if (T.block == 2) rdm_opposite_spin_double(T, ba, ka, exa, bb, kb, exb, val);
  } else if (ca == 2) {
    if (T.block != 1) rdm_single(T, 0, false, ba, ka, exa, bb, val);
  } else if (cb == 2) {
    if (T.block != 0) rdm_single(T, 1, true, bb, kb, exb, ba, val);
  } else {
    rdm_diag(T, ba, bb, val);
  }
}

__global__ void __launch_bounds__(kRdmWarps * 32)
    k_rdm(RowArgs a, const double* __restrict__ C, RdmTarget T, double* g4, double* g2) {
  extern __shared__ double tile[];
  __shared__ RowWalkSmemT<kRdmWarps> sm;
  const int n = T.n;
  const size_t n4 = (size_t)n * n * n * (T.s_hi - T.s_lo), n2 = (size_t)n * n;
  if (T.shared) {
    T.t4 = tile;
    T.t2 = (T.block < 2 && T.with_ordm) ? tile + n4 : nullptr;
    for (size_t i = threadIdx.x; i < n4 + (T.t2 ? n2 : 0); i += blockDim.x) tile[i] = 0.;
    __syncthreads();
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int64_t r = (int64_t)blockIdx.x * kRdmWarps + w; r < a.ndets; r += (int64_t)gridDim.x * kRdmWarps) {
    const double cr = C[r];
    walk_row(a, r, w, lane, sm, [&](int64_t ket, int64_t row, uint64_t ra, uint64_t rb, uint64_t ka, uint64_t kb) {
      if (ket < row) return;  // every unordered pair once, lower index as bra
      const double val = cr * C[ket];
      if (!(fabs(val) > 1e-16)) return;
      rdm_pair(T, ra, rb, ka, kb, val);
    });
  }
  if (T.shared) {
    __syncthreads();
    for (size_t i = threadIdx.x; i < n4; i += blockDim.x) {
      const double v = tile[i];
      if (v != 0.) atomicAdd(g4 + (size_t)T.s_lo * n * n * n + i, v);
    }
    if (T.t2)
      for (size_t i = threadIdx.x; i < n2; i += blockDim.x) {
        const double v = tile[n4 + i];
        if (v != 0.) atomicAdd(g2 + i, v);
      }
  }
}

void rdms_spin_dep(Context* c, const double* C, double* aa, double* bb, double* aaaa, double* bbbb, double* aabb) {
  if (!c->have_ints) throw Error(QDKGB_ERR_STATE, "integrals not set (needed for the orbital count)");
  const int n = c->norb;
  const int64_t N = c->dets.ndets;
  const size_t n2 = (size_t)n * n, n4 = n2 * n2;
  DeviceBuffer bC, b4, b2;
  double* dC = dev_array<double>(c, bC, N);
  QDKGB_CUDA(cudaMemcpyAsync(dC, C, N * 8, cudaMemcpyHostToDevice, c->stream));
  double* d4 = dev_array<double>(c, b4, n4);
  double* d2 = dev_array<double>(c, b2, n2);
  RowArgs a = row_args(c, 0.);
  const size_t smem_cap = 200 * 1024;
  const size_t slice = (size_t)n * n * n * 8;
  const bool use_shared = n <= 16;
  int s_step = use_shared ? (int)std::min<size_t>((size_t)n, (smem_cap - n2 * 8) / slice) : n;
  if (s_step < 1) s_step = 1;
  set_max_dynamic_smem((const void*)k_rdm, (int)smem_cap);
  const int64_t blocks = std::min<int64_t>((N + kRdmWarps - 1) / kRdmWarps, (int64_t)c->sm_count * (use_shared ? 1 : 4));
  double* outs4[3] = {aaaa, bbbb, aabb};
  double* outs2[3] = {aa, bb, nullptr};
  std::vector<double> h4(n4), h2(n2);
  for (int blk = 0; blk < 3; ++blk) {
    if (!outs4[blk] && !outs2[blk]) continue;
    QDKGB_CUDA(cudaMemsetAsync(d4, 0, n4 * 8, c->stream));
    QDKGB_CUDA(cudaMemsetAsync(d2, 0, n2 * 8, c->stream));
    for (int s0 = 0; s0 < n; s0 += s_step) {
      RdmTarget T;
      T.block = blk;
      T.n = n;
      T.s_lo = s0;
      T.s_hi = use_shared ? std::min(n, s0 + s_step) : n;
      T.shared = use_shared;
      T.with_ordm = (s0 == 0);
      T.t4 = use_shared ? nullptr : d4;
      T.t2 = (!use_shared && blk < 2) ? d2 : nullptr;
      const size_t tile =
          use_shared ? (n2 * n * (T.s_hi - T.s_lo) + ((blk < 2 && T.with_ordm) ? n2 : 0)) * 8 : 0;
      k_rdm<<<(unsigned)blocks, kRdmWarps * 32, tile, c->stream>>>(a, dC, T, d4, d2);
      QDKGB_CHECK_LAUNCH();
      if (!use_shared) break;
    }
    QDKGB_CUDA(cudaStreamSynchronize(c->stream));
    if (outs4[blk]) {
      QDKGB_CUDA(cudaMemcpy(h4.data(), d4, n4 * 8, cudaMemcpyDeviceToHost));
      for (size_t i = 0; i < n4; ++i) outs4[blk][i] += h4[i];
    }
    if (outs2[blk]) {
      QDKGB_CUDA(cudaMemcpy(h2.data(), d2, n2 * 8, cudaMemcpyDeviceToHost));
      for (size_t i = 0; i < n2; ++i) outs2[blk][i] += h2[i];
    }
  }
  dev_free(c, bC);
  dev_free(c, b4);
  dev_free(c, b2);
}

}  // namespace qdkgb
