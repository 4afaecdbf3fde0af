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
#include <cmath>
#include <limits>
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
  NvtxRange nvtx_range("qdkgb.rdms");
  if (!c->have_ints) throw Error(QDKGB_ERR_STATE, "integrals not set (needed for the orbital count)");
  check_dets_in_orbitals(c);
  const int n = c->norb;
  const int64_t N = c->dets.ndets;
  const size_t n2 = (size_t)n * n, n4 = n2 * n2;
  ScopedBuffers<3> scratch(c);
  DeviceBuffer &bC = scratch.b[0], &b4 = scratch.b[1], &b2 = scratch.b[2];
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
}

// ---------------------------------------------------------------- orbital entropies
// SortedDoubleLoopHamiltonianGenerator::form_entropies (sorted_double_loop.hpp:
// 755-903) with the OrbitalRDMIntermediates contributions of
// include/macis/util/entropies.hpp:155-340: the RDM pair walk above (every
// unordered pair with at most one excitation per spin, lower index as bra)
// accumulates a_ii, b_ii, ab_iiii and the n x n intermediates in a per-CTA
// shared-memory tile (global atomics when the tile would not fit); the one-
// and two-orbital RDM blocks and their entropies are assembled on the host
// (entropies.hpp:342-651).  Without the pair terms only the diagonal pairs
// contribute.
namespace {

// intermediate matrices, M(k, i, j) at 3n + k n^2 + i n + j (after a_ii, b_ii, ab_iiii)
enum : int {
  E_A_IJ, E_B_IJ, E_AA_IIJJ, E_BB_IIJJ, E_AB_IIJJ, E_AB_IJJJ, E_AB_JIJJ, E_AB_JJIJ, E_AB_JJJI, E_AB_IJIJ, E_AB_IJJI,
  E_AAB_IIJJJJ, E_ABB_JJIIJJ, E_AAB_IIJJII, E_ABB_IIIIJJ, E_ABB_IJIIJJ, E_AAB_IIJJIJ, E_AABB_IIJJIIJJ, E_NMAT
};

struct EntTarget {
  double* t;
  int n;
  bool s2;
};
__device__ __forceinline__ void e_vec(const EntTarget& T, int v, uint32_t i, double x) { atomicAdd(T.t + v * T.n + i, x); }
__device__ __forceinline__ void e_mat(const EntTarget& T, int k, uint32_t i, uint32_t j, double x) {
  atomicAdd(T.t + 3 * T.n + ((size_t)k * T.n + i) * T.n + j, x);
}

// orbital_rdm_contrib_diag_s1 / orbital_rdm_contrib_diag (entropies.hpp:155-253)
__device__ void ent_diag(const EntTarget& T, uint64_t oa, uint64_t ob, double val) {
  for (uint64_t m = oa; m; m &= m - 1) e_vec(T, 0, low_bit(m), val);
  for (uint64_t m = ob; m; m &= m - 1) e_vec(T, 1, low_bit(m), val);
  for (uint64_t m = oa & ob; m; m &= m - 1) e_vec(T, 2, low_bit(m), val);
  if (!T.s2) return;
  for (uint64_t mq = oa; mq; mq &= mq - 1) {
    const uint32_t q = low_bit(mq);
    for (uint64_t mp = oa & ~(1ull << q); mp; mp &= mp - 1) {
      const uint32_t p = low_bit(mp);
      e_mat(T, E_AA_IIJJ, p, q, val);
      if ((ob >> p) & 1) {
        e_mat(T, E_AAB_IIJJII, p, q, val);
        if ((ob >> q) & 1) e_mat(T, E_AABB_IIJJIIJJ, p, q, val);
      }
      if ((ob >> q) & 1) e_mat(T, E_AAB_IIJJJJ, p, q, val);
    }
  }
  for (uint64_t mq = ob; mq; mq &= mq - 1) {
    const uint32_t q = low_bit(mq);
    for (uint64_t mp = ob & ~(1ull << q); mp; mp &= mp - 1) {
      const uint32_t p = low_bit(mp);
      e_mat(T, E_BB_IIJJ, p, q, val);
      if ((oa >> p) & 1) e_mat(T, E_ABB_JJIIJJ, q, p, val);
      if ((oa >> q) & 1) e_mat(T, E_ABB_IIIIJJ, q, p, val);
    }
  }
  for (uint64_t mq = ob; mq; mq &= mq - 1)
    for (uint64_t mp = oa; mp; mp &= mp - 1) e_mat(T, E_AB_IIJJ, low_bit(mp), low_bit(mq), val);
}

// orbital_rdm_contrib_2<transpose> (entropies.hpp:255-313); occ_os = the bra's
// other-spin string
__device__ void ent_single(const EntTarget& T, bool transpose, uint64_t bra, uint64_t ket, uint64_t ex,
                           uint64_t occ_os, double val) {
  const SingleEx s = single_ex(bra, ket, ex);
  const uint32_t o1 = s.o, v1 = s.v;
  const double sv = s.neg ? -val : val;
  const int xij = transpose ? E_B_IJ : E_A_IJ;
  e_mat(T, xij, v1, o1, sv);
  e_mat(T, xij, o1, v1, sv);
  const int k1 = transpose ? E_AB_JJIJ : E_AB_IJJJ, k2 = transpose ? E_AB_JJJI : E_AB_JIJJ;
  const bool o_in = (occ_os >> o1) & 1, v_in = (occ_os >> v1) & 1;
  if (o_in) {
    e_mat(T, k1, v1, o1, sv);
    e_mat(T, k2, v1, o1, sv);
  }
  if (v_in) {
    e_mat(T, k1, o1, v1, sv);
    e_mat(T, k2, o1, v1, sv);
  }
  if (o_in && v_in) {
    const int k3 = transpose ? E_AAB_IIJJIJ : E_ABB_IJIIJJ;
    e_mat(T, k3, o1, v1, sv);
    e_mat(T, k3, v1, o1, sv);
  }
}

// orbital_rdm_contrib_22 (entropies.hpp:315-340)
__device__ void ent_double_os(const EntTarget& T, uint64_t ba, uint64_t ka, uint64_t exa, uint64_t bb, uint64_t kb,
                              uint64_t exb, double val) {
  const SingleEx a = single_ex(ba, ka, exa);  // (o2, v2)
  const SingleEx b = single_ex(bb, kb, exb);  // (o1, v1)
  const double sv = (a.neg != b.neg) ? -val : val;
  if (b.o == a.o && b.v == a.v) {
    e_mat(T, E_AB_IJIJ, b.v, b.o, sv);
    e_mat(T, E_AB_IJIJ, b.o, b.v, sv);
  } else if (b.o == a.v && b.v == a.o) {
    e_mat(T, E_AB_IJJI, b.v, b.o, sv);
    e_mat(T, E_AB_IJJI, b.o, b.v, sv);
  }
}

__global__ void __launch_bounds__(kRdmWarps * 32)
    k_entropy(RowArgs a, const double* __restrict__ C, int n, bool s2, bool shared, double* __restrict__ g) {
  extern __shared__ double tile[];
  __shared__ RowWalkSmemT<kRdmWarps> sm;
  const size_t total = 3 * (size_t)n + (s2 ? (size_t)E_NMAT * n * n : 0);
  const EntTarget T{shared ? tile : g, n, s2};
  if (shared) {
    for (size_t i = threadIdx.x; i < total; i += blockDim.x) tile[i] = 0.;
    __syncthreads();
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int64_t r = (int64_t)blockIdx.x * kRdmWarps + w; r < a.ndets; r += (int64_t)gridDim.x * kRdmWarps) {
    const double cr = C[r];
    if (!s2) {
      const uint64_t ra = a.galpha[a.det_group[r]], rb = a.ubeta[a.brank[r]];
      const double val = cr * cr;
      if (lane == 0 && ra != 0 && fabs(val) > 1e-16) ent_diag(T, ra, rb, val);
      continue;
    }
    walk_row(a, r, w, lane, sm, [&](int64_t ket, int64_t row, uint64_t ra, uint64_t rb, uint64_t ka, uint64_t kb) {
      if (ket < row) return;  // every unordered pair once, lower index as bra
      const uint64_t exa = ra ^ ka, exb = rb ^ kb;
      const int ca = popc64(exa), cb = popc64(exb);
      if (ca > 2 || cb > 2) return;
      const double val = cr * C[ket];
      if (!(fabs(val) > 1e-16)) return;
      if (ca == 0 && cb == 0)
        ent_diag(T, ra, rb, val);
      else if (cb == 0)
        ent_single(T, false, ra, ka, exa, rb, val);
      else if (ca == 0)
        ent_single(T, true, rb, kb, exb, ra, val);
      else
        ent_double_os(T, ra, ka, exa, rb, kb, exb, val);
    });
  }
  if (shared) {
    __syncthreads();
    for (size_t i = threadIdx.x; i < total; i += blockDim.x) {
      const double v = tile[i];
      if (v != 0.) atomicAdd(g + i, v);
    }
  }
}

// eigenvalues of a symmetric 4 x 4 matrix by cyclic Jacobi rotations
void sym4_eigenvalues(double A[4][4], double w[4]) {
  for (int sweep = 0; sweep < 64; ++sweep) {
    double off = 0., dia = 0.;
    for (int p = 0; p < 4; ++p) {
      dia += A[p][p] * A[p][p];
      for (int q = p + 1; q < 4; ++q) off += A[p][q] * A[p][q];
    }
    if (!(off > 1e-34 * dia) || off == 0.) break;
    for (int p = 0; p < 4; ++p)
      for (int q = p + 1; q < 4; ++q) {
        if (A[p][q] == 0.) continue;
        const double th = (A[q][q] - A[p][p]) / (2. * A[p][q]);
        const double t = (th >= 0. ? 1. : -1.) / (std::fabs(th) + std::sqrt(th * th + 1.));
        const double cs = 1. / std::sqrt(t * t + 1.), sn = t * cs;
        for (int r = 0; r < 4; ++r) {
          const double x = A[r][p], y = A[r][q];
          A[r][p] = cs * x - sn * y;
          A[r][q] = sn * x + cs * y;
        }
        for (int r = 0; r < 4; ++r) {
          const double x = A[p][r], y = A[q][r];
          A[p][r] = cs * x - sn * y;
          A[q][r] = sn * x + cs * y;
        }
      }
  }
  for (int i = 0; i < 4; ++i) w[i] = A[i][i];
}

inline void add_entropy(double& s, double v) {
  if (v > std::numeric_limits<double>::epsilon()) s -= v * std::log(v);
}
inline void add_entropy_2x2(double& s, double a, double b, double d) {
  const double hs = 0.5 * (a + d), hd = 0.5 * (a - d), r = std::sqrt(hd * hd + b * b);
  add_entropy(s, hs - r);
  add_entropy(s, hs + r);
}

}  // namespace

void orbital_entropies(Context* c, const double* C, double* s1, double* s2, double* mi) {
  NvtxRange nvtx_range("qdkgb.orbital_entropies");
  if (!c->have_ints) throw Error(QDKGB_ERR_STATE, "integrals not set (needed for the orbital count)");
  if (!c->have_dets) throw Error(QDKGB_ERR_STATE, "determinants not set");
  check_dets_in_orbitals(c);
  const int n = c->norb;
  const int64_t N = c->dets.ndets;
  const bool need_s2 = s2 || mi;
  const size_t nn = (size_t)n * n, total = 3 * (size_t)n + (need_s2 ? E_NMAT * nn : 0);
  ScopedBuffers<2> scratch(c);
  DeviceBuffer &bC = scratch.b[0], &bg = scratch.b[1];
  double* dC = dev_array<double>(c, bC, N);
  double* g = dev_array<double>(c, bg, total);
  QDKGB_CUDA(cudaMemcpyAsync(dC, C, N * 8, cudaMemcpyHostToDevice, c->stream));
  QDKGB_CUDA(cudaMemsetAsync(g, 0, total * 8, c->stream));
  const size_t smem_cap = 200 * 1024;
  const bool shared = total * 8 <= smem_cap;
  set_max_dynamic_smem((const void*)k_entropy, (int)smem_cap);
  const int64_t blocks = std::min<int64_t>((N + kRdmWarps - 1) / kRdmWarps, (int64_t)c->sm_count * (shared ? 1 : 4));
  k_entropy<<<(unsigned)std::max<int64_t>(blocks, 1), kRdmWarps * 32, shared ? total * 8 : 0, c->stream>>>(
      row_args(c, 0.), dC, n, need_s2, shared, g);
  QDKGB_CHECK_LAUNCH();
  std::vector<double> h(total);
  QDKGB_CUDA(cudaMemcpyAsync(h.data(), g, total * 8, cudaMemcpyDeviceToHost, c->stream));
  QDKGB_CUDA(cudaStreamSynchronize(c->stream));
  const double *a_ii = h.data(), *b_ii = a_ii + n, *ab_ii = b_ii + n;
  // build_s1_entropy (entropies.hpp:342-370): the diagonal one-orbital RDM
  // (empty, alpha, beta, double)
  for (int i = 0; i < n; ++i) {
    double s = 0.;
    add_entropy(s, 1. - a_ii[i] - b_ii[i] + ab_ii[i]);
    add_entropy(s, a_ii[i] - ab_ii[i]);
    add_entropy(s, b_ii[i] - ab_ii[i]);
    add_entropy(s, ab_ii[i]);
    s1[i] = s;
  }
  if (!need_s2) return;
  auto M = [&](int k, int i, int j) { return h[3 * (size_t)n + ((size_t)k * n + i) * n + j]; };
  std::vector<double> t(nn, 0.);
  // build_s2_entropy (entropies.hpp:397-528): the two-orbital RDM of (i, j)
  // block by block (particle-number and spin sectors), entropy of the
  // eigenvalues
  for (int i = 0; i < n; ++i)
    for (int j = i + 1; j < n; ++j) {
      const double q4 = M(E_AABB_IIJJIIJJ, i, j);
      const double a3j = M(E_AAB_IIJJJJ, i, j), a3i = M(E_AAB_IIJJII, i, j);
      const double b3j = M(E_ABB_JJIIJJ, i, j), b3i = M(E_ABB_IIIIJJ, i, j);
      double s = 0.;
      add_entropy(s, 1. - a_ii[i] - b_ii[i] - a_ii[j] - b_ii[j] + ab_ii[i] + ab_ii[j] + M(E_AA_IIJJ, i, j) +
                         M(E_AB_IIJJ, i, j) + M(E_AB_IIJJ, j, i) + M(E_BB_IIJJ, i, j) - a3j - b3j - a3i - b3i + q4);
      add_entropy_2x2(s,
                      a_ii[j] - M(E_AB_IIJJ, j, i) - M(E_AA_IIJJ, i, j) - M(E_AB_IIJJ, j, j) + a3j + a3i + b3j - q4,
                      M(E_A_IJ, i, j) - M(E_AB_JIJJ, j, i) - M(E_AB_IJJJ, i, j) + M(E_ABB_IJIIJJ, i, j),
                      a_ii[i] - M(E_AB_IIJJ, i, j) - M(E_AA_IIJJ, i, j) - M(E_AB_IIJJ, i, i) + a3j + a3i + b3i - q4);
      add_entropy_2x2(s,
                      b_ii[j] - M(E_AB_IIJJ, i, j) - M(E_BB_IIJJ, i, j) - M(E_AB_IIJJ, j, j) + b3i + a3j + b3j - q4,
                      M(E_B_IJ, i, j) - M(E_AB_JJIJ, j, i) - M(E_AB_JJJI, i, j) + M(E_AAB_IIJJIJ, i, j),
                      b_ii[i] - M(E_AB_IIJJ, j, i) - M(E_BB_IIJJ, i, j) - M(E_AB_IIJJ, i, i) + b3j + a3i + b3i - q4);
      add_entropy(s, M(E_AA_IIJJ, i, j) - a3i - a3j + q4);
      add_entropy(s, M(E_BB_IIJJ, i, j) - b3i - b3j + q4);
      double B[4][4];
      B[0][0] = M(E_AB_IIJJ, j, j) - a3j - b3j + q4;
      B[0][1] = B[1][0] = M(E_AB_IJJJ, i, j) - M(E_ABB_IJIIJJ, i, j);
      B[0][2] = B[2][0] = -M(E_AB_JJIJ, i, j) + M(E_AAB_IIJJIJ, i, j);
      B[0][3] = B[3][0] = M(E_AB_IJIJ, i, j);
      B[1][1] = M(E_AB_IIJJ, i, j) - b3i - a3j + q4;
      B[1][2] = B[2][1] = -M(E_AB_IJJI, j, i);
      B[1][3] = B[3][1] = M(E_AB_JJJI, j, i) - M(E_AAB_IIJJIJ, i, j);
      B[2][2] = M(E_AB_IIJJ, j, i) - a3i - b3j + q4;
      B[2][3] = B[3][2] = -M(E_AB_JIJJ, j, i) + M(E_ABB_IJIIJJ, i, j);
      B[3][3] = ab_ii[i] - a3i - b3i + q4;
      double w4[4];
      sym4_eigenvalues(B, w4);
      for (double v : w4) add_entropy(s, v);
      add_entropy_2x2(s, a3j - q4, -M(E_AAB_IIJJIJ, i, j), a3i - q4);
      add_entropy_2x2(s, b3j - q4, -M(E_ABB_IJIIJJ, i, j), b3i - q4);
      add_entropy(s, q4);
      t[(size_t)i * n + j] = t[(size_t)j * n + i] = s;
    }
  if (s2) std::copy(t.begin(), t.end(), s2);
  // build_mutual_information (entropies.hpp:638-651)
  if (mi)
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) mi[(size_t)i * n + j] = (i == j) ? 0. : s1[i] + s1[j] - t[(size_t)i * n + j];
}

}  // namespace qdkgb
