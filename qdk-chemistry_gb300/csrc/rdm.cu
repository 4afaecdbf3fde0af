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
#include <cstdlib>
#include <cmath>
#include <limits>
#include <vector>

#include "common.cuh"
#include "internal.h"
#include "rowwalk.cuh"

namespace qdkgb {

constexpr int kRdmWarps = 16;

// The pair walk's 1-RDM is summed in fixed point, two 64-bit words per
// element, in units of s = the power of two at or above max_I C_I^2 (so every
// contribution x / s lies in [-1, 1]): x / s = hi 2^-32 + lo 2^-76 with
// hi = rint(x / s 2^32) and lo the rest in units of 2^-76 (scaling by s and
// the split of each contribution are exact).  Integer
// additions are exact and associative, so the 1-RDM does not depend on the
// order in which the atomics land (FP64 atomics would): the natural orbitals
// of the ASCI grow's rotation, and every 1-RDM of a selected space, repeat
// bit for bit.  |x| < 2^20 per contribution and up to ~2^19 contributions
// per element keep the words in range.
constexpr double kRdmFixHi = 4294967296.0;               // 2^32
constexpr double kRdmFixLo = 75557863725914323419136.0;  // 2^76

struct RdmTarget {
  int block;       // 0: aaaa (+aa), 1: bbbb (+bb), 2: aabb
  int n;
  int s_lo, s_hi;  // last-index range held by the tile
  double* t4;      // tile or global n^4 block
  double* t2;      // tile or global n^2 block (blocks 0, 1) when not fixed point
  unsigned long long* t2fx = nullptr;  // global fixed-point n^2 block (2 words per element), when given
  double fx_inv = 1.;                  // 1 / s of the fixed point
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
  if (blk != T.block) return;
  if (T.t2fx) {
    v *= T.fx_inv;
    const double hi = rint(v * kRdmFixHi);
    const double lo = rint((v - hi * (1.0 / kRdmFixHi)) * kRdmFixLo);
    unsigned long long* e = T.t2fx + 2 * (p + (size_t)T.n * q);
    atomicAdd(e, (unsigned long long)(long long)hi);
    atomicAdd(e + 1, (unsigned long long)(long long)lo);
    return;
  }
  if (!T.t2) return;
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
    T.t2 = (T.block < 2 && T.with_ordm && !T.t2fx) ? tile + n4 : nullptr;
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

// ---------------------------------------------------------------- complete spaces
// For a complete (n_alpha, n_beta) product space the CI vector is a matrix
// C[g, b] (determinant g * N_b + b) and the same contributions as above are
// regrouped by spin, with no pair walk and no atomics on the opposite-spin
// block:
//
//   aabb: every ordered pair (I <- J) with at most one excitation per spin
//     adds 1/2 s_a s_b C_I C_J to G[i, j, k, l], (i, j) the beta and (k, l)
//     the alpha orbitals (created in the bra, annihilated in the ket; a
//     string-diagonal term has i = j or k = l occupied).  For each alpha
//     transition (gJ -> gI, class (k, l)) the kernel sums over every beta
//     transition of class (i, j):
//         t_ij = sum_{(bJ -> bI) in class (i, j)} s_b C[gI, bI] C[gJ, bJ]
//     with one thread per beta class (its list of (bI, bJ, s_b) streamed
//     from L2) and the two rows of C staged in shared memory, accumulating
//     s_a t_ij in registers over a chunk of transitions of one alpha class.
//     Chunks write partial sums that a second kernel adds in a fixed order
//     (deterministic).  The reversed alpha transition gives the same value
//     at G[j, i, l, k], so only classes k >= l are swept.
//   aaaa + aa: the pairs with equal beta strings, i.e. alpha string pairs
//     (gI, gJ) within a double excitation weighted by the string overlap
//     S_a = sum_b C[gI, b] C[gJ, b], then the same-spin formulas above
//     (rdm_same_spin_double / rdm_single / rdm_diag, block 0); bbbb + bb the
//     same with S_b over the columns.
//
// The reference drops a pair when |C_I C_J| <= 1e-16 (rdms.hpp skip rule,
// k_rdm above); the same rule is applied to every product here: in the sweep
// by the exponents of the two factors (one DFMA when the product is surely
// above or below the bound, the product formed and tested in the narrow band
// between), in the overlaps by forming each product.

namespace {

constexpr int kCasThreads = 320;  // beta work items per CTA (one per thread)
constexpr int kCasChunk = 48;     // alpha transitions per CTA

struct CasItem {
  int32_t cls;    // beta class i + n j
  int32_t begin;  // into the packed list
  int32_t len;
};

// |a b| > 1e-16 decided from the biased exponents where the answer is certain
// (sum >= 2046 - 53: |ab| >= 2^-53 > 1e-16; sum <= 2046 - 56: |ab| < 2^-54),
// by the rounded product itself in between.
__device__ __forceinline__ double cas_acc(double acc, double a, double b, bool neg) {
  const int ea = (int)((__double_as_longlong(a) >> 52) & 0x7ff);
  const int eb = (int)((__double_as_longlong(b) >> 52) & 0x7ff);
  const int es = ea + eb;
  if (es >= 2046 - 53) return fma(flip_if(a, neg), b, acc);
  if (es <= 2046 - 56) return acc;
  const double p = a * b;
  return fabs(p) > 1e-16 ? acc + flip_if(p, neg) : acc;
}

__global__ void __launch_bounds__(kCasThreads)
    k_rdm_cas_ab(int64_t nb, const double* __restrict__ C, const uint32_t* __restrict__ atr,
                 const int4* __restrict__ chunks, const CasItem* __restrict__ items, int nitems,
                 const uint32_t* __restrict__ blist, double* __restrict__ partial) {
  extern __shared__ double rows[];  // rowI | rowJ
  double* rowI = rows;
  double* rowJ = rows + nb;
  const int4 ch = chunks[blockIdx.x];  // (alpha class, first transition, count, unused)
  const int it = threadIdx.x;
  CasItem item = {0, 0, 0};
  if (it < nitems) item = items[it];
  const uint32_t* lst = blist + item.begin;
  double acc = 0.;
  for (int t = 0; t < ch.z; ++t) {
    const uint32_t w = __ldg(atr + ch.y + t);
    const int64_t gI = w & 0x7fff, gJ = (w >> 15) & 0x7fff;
    const bool na = (w >> 31) != 0;
    __syncthreads();
    for (int64_t b = threadIdx.x; b < nb; b += blockDim.x) {
      rowI[b] = C[gI * nb + b];
      rowJ[b] = C[gJ * nb + b];
    }
    __syncthreads();
    double s0 = 0., s1 = 0., s2 = 0., s3 = 0.;
    int e = 0;
    for (; e + 4 <= item.len; e += 4) {
      const uint32_t x0 = __ldg(lst + e), x1 = __ldg(lst + e + 1), x2 = __ldg(lst + e + 2), x3 = __ldg(lst + e + 3);
      s0 = cas_acc(s0, rowI[x0 & 0x7fff], rowJ[(x0 >> 15) & 0x7fff], (x0 >> 31) != 0);
      s1 = cas_acc(s1, rowI[x1 & 0x7fff], rowJ[(x1 >> 15) & 0x7fff], (x1 >> 31) != 0);
      s2 = cas_acc(s2, rowI[x2 & 0x7fff], rowJ[(x2 >> 15) & 0x7fff], (x2 >> 31) != 0);
      s3 = cas_acc(s3, rowI[x3 & 0x7fff], rowJ[(x3 >> 15) & 0x7fff], (x3 >> 31) != 0);
    }
    for (; e < item.len; ++e) {
      const uint32_t x0 = __ldg(lst + e);
      s0 = cas_acc(s0, rowI[x0 & 0x7fff], rowJ[(x0 >> 15) & 0x7fff], (x0 >> 31) != 0);
    }
    acc += flip_if((s0 + s1) + (s2 + s3), na);
  }
  if (it < nitems) partial[(int64_t)blockIdx.x * nitems + it] = acc;
}

// G[i, j, k, l] (and G[j, i, l, k] for k > l) = 1/2 sum over the class's
// chunks and the beta class's items, in a fixed order.  One thread per
// (alpha class, beta class).
__global__ void k_rdm_cas_ab_reduce(int n, int nacls, const int2* __restrict__ acls, const int2* __restrict__ acls_chunks,
                                    const int2* __restrict__ bcls_items, int nitems,
                                    const double* __restrict__ partial, double* __restrict__ G) {
  const int n2 = n * n;
  const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (tid >= (int64_t)nacls * n2) return;
  const int ac = (int)(tid / n2), bc = (int)(tid % n2);
  const int2 kl = acls[ac];
  const int2 chr = acls_chunks[ac];
  const int2 itr = bcls_items[bc];
  double v = 0.;
  for (int q = chr.x; q < chr.y; ++q)
    for (int m = itr.x; m < itr.y; ++m) v += partial[(int64_t)q * nitems + m];
  v *= 0.5;
  const int i = bc % n, j = bc / n, k = kl.x, l = kl.y;
  G[i + (size_t)n * (j + (size_t)n * (k + (size_t)n * l))] = v;
  if (k != l) G[j + (size_t)n * (i + (size_t)n * (l + (size_t)n * k))] = v;
}

// S[p] = sum_b X[r1, b] X[r2, b] over the pair list (rows of X with ld cols),
// each product kept when |product| > 1e-16.  One warp per pair.
__global__ void k_pair_overlap(int64_t npairs, const int2* __restrict__ pairs, const double* __restrict__ X,
                               int64_t cols, double* __restrict__ S) {
  const int lane = threadIdx.x & 31;
  for (int64_t p = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; p < npairs;
       p += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const int2 pr = pairs[p];
    const double* x = X + pr.x * cols;
    const double* y = X + pr.y * cols;
    double s = 0.;
    for (int64_t b = lane; b < cols; b += 32) {
      const double v = __ldg(x + b) * __ldg(y + b);
      if (fabs(v) > 1e-16) s += v;
    }
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) S[p] = s;
  }
}

// same-spin blocks of one spin from the string overlaps (block 0: aaaa + aa,
// block 1: bbbb + bb); the bra is the lower-ranked string, as the
// determinant order puts it first.
__global__ void k_rdm_cas_same_spin(int64_t npairs, const int2* __restrict__ pairs, const uint64_t* __restrict__ str,
                                    const double* __restrict__ S, RdmTarget T) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < npairs; p += (int64_t)gridDim.x * blockDim.x) {
    const double val = S[p];
    if (val == 0.) continue;
    const int2 pr = pairs[p];
    const uint64_t bra = str[pr.x], ket = str[pr.y];
    const uint64_t ex = bra ^ ket;
    const int c = popc64(ex);
    if (c == 4)
      rdm_same_spin_double(T, T.block, bra, ket, ex, val);
    else if (c == 2)
      rdm_single(T, T.block, false, bra, ket, ex, 0, val);
    else
      rdm_diag(T, bra, bra, val);
  }
}

inline bool cas_sign_odd(uint64_t state, uint32_t p, uint32_t q) {
  const uint32_t lo = p < q ? p : q, hi = p < q ? q : p;
  const uint64_t m = ((hi >= 64 ? ~0ull : ((1ull << hi) - 1ull))) ^ ((1ull << (lo + 1)) - 1ull);
  return __builtin_popcountll(state & m) & 1;
}

}  // namespace

// True when the determinants form a complete product space this path serves.
static bool cas_rdm_eligible(const Context* c) {
  const DetSpace& S = c->dets;
  if (!S.product || c->norb > 16 || S.ngroups < 1 || S.nbeta < 1) return false;
  if (S.ngroups > 32767 || S.nbeta > 32767) return false;
  if ((size_t)2 * S.nbeta * 8 > 220 * 1024) return false;  // the two staged rows of C
  for (int64_t g = 0; g < S.ngroups; ++g)
    if (S.h_gstart[g] != g * S.nbeta) return false;
  return true;
}

// transitions (ket -> bra) of class (v, o) among strs: bra = ket - o + v
static void cas_string_maps(const std::vector<uint64_t>& strs, std::vector<int32_t>& rank_of, int n) {
  rank_of.assign((size_t)1 << n, -1);
  for (size_t i = 0; i < strs.size(); ++i) rank_of[strs[i]] = (int32_t)i;
}

// Returns false (nothing accumulated) when the space has more beta classes
// than the kernel's CTA holds; the pair walk serves it then.
static bool rdms_cas(Context* c, const double* dC, double* aa, double* bb, double* aaaa, double* bbbb, double* aabb) {
  const DetSpace& S = c->dets;
  const int n = c->norb;
  const int64_t na = S.ngroups, nb = S.nbeta, N = na * nb;
  const size_t n2 = (size_t)n * n, n4 = n2 * n2;
  std::vector<int32_t> ra, rb;
  cas_string_maps(S.h_galpha, ra, n);
  cas_string_maps(S.h_ubeta, rb, n);
  ScopedBuffers<12> buf(c);
  std::vector<double> h4(n4), h2(n2);

  // ---------------- opposite spin (aabb)
  if (aabb) {
    // beta lists per class (i, j): (bI, bJ, s_b) packed bI | bJ << 15 | s << 31
    std::vector<uint32_t> blist;
    std::vector<int32_t> bbeg(n2 + 1, 0);
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        const int cls = i + n * j;
        bbeg[cls] = (int32_t)blist.size();
        for (int64_t x = 0; x < nb; ++x) {
          const uint64_t ket = S.h_ubeta[x];
          if (!((ket >> j) & 1)) continue;
          if (i == j) {
            blist.push_back((uint32_t)x | ((uint32_t)x << 15));
            continue;
          }
          if ((ket >> i) & 1) continue;
          const uint64_t bra = ket ^ (1ull << i) ^ (1ull << j);
          const int32_t y = rb[bra];
          if (y < 0) throw Error(QDKGB_ERR_UNSUPPORTED, "RDM: beta strings are not a complete set");
          const bool neg = cas_sign_odd(ket, (uint32_t)i, (uint32_t)j);
          blist.push_back((uint32_t)y | ((uint32_t)x << 15) | ((uint32_t)neg << 31));
        }
      }
    bbeg[n2] = (int32_t)blist.size();
    // work items: lists split to at most the longest off-diagonal length
    int32_t lmax = 1;
    for (size_t cl = 0; cl < n2; ++cl)
      if ((int)(cl % n) != (int)(cl / n)) lmax = std::max(lmax, bbeg[cl + 1] - bbeg[cl]);
    for (size_t cl = 0; cl < n2; ++cl)
      if ((int)(cl % n) == (int)(cl / n) && lmax == 1) lmax = std::max(lmax, bbeg[cl + 1] - bbeg[cl]);
    std::vector<CasItem> items;
    std::vector<int2> bitems(n2);
    for (size_t cl = 0; cl < n2; ++cl) {
      const int32_t len = bbeg[cl + 1] - bbeg[cl];
      const int parts = std::max(1, (len + lmax - 1) / lmax);
      bitems[cl].x = (int)items.size();
      for (int q = 0; q < parts; ++q) {
        const int32_t b0 = (int32_t)((int64_t)len * q / parts), b1 = (int32_t)((int64_t)len * (q + 1) / parts);
        items.push_back({(int32_t)cl, bbeg[cl] + b0, b1 - b0});
      }
      bitems[cl].y = (int)items.size();
    }
    const int nitems = (int)items.size();
    if (nitems > kCasThreads) return false;
    // alpha transitions per class (k, l), k >= l: (gI, gJ, s_a)
    std::vector<uint32_t> atr;
    std::vector<int2> acls, acls_chunks;
    std::vector<int4> chunks;
    for (int k = 0; k < n; ++k)
      for (int l = 0; l <= k; ++l) {
        const size_t t0 = atr.size();
        for (int64_t x = 0; x < na; ++x) {
          const uint64_t ket = S.h_galpha[x];
          if (!((ket >> l) & 1)) continue;
          if (k == l) {
            atr.push_back((uint32_t)x | ((uint32_t)x << 15));
            continue;
          }
          if ((ket >> k) & 1) continue;
          const uint64_t bra = ket ^ (1ull << k) ^ (1ull << l);
          const int32_t y = ra[bra];
          if (y < 0) throw Error(QDKGB_ERR_UNSUPPORTED, "RDM: alpha strings are not a complete set");
          const bool neg = cas_sign_odd(ket, (uint32_t)k, (uint32_t)l);
          atr.push_back((uint32_t)y | ((uint32_t)x << 15) | ((uint32_t)neg << 31));
        }
        const size_t t1 = atr.size();
        if (t1 == t0) continue;
        acls.push_back({k, l});
        const int c0 = (int)chunks.size();
        for (size_t q = t0; q < t1; q += kCasChunk)
          chunks.push_back({(int)acls.size() - 1, (int)q, (int)std::min<size_t>(kCasChunk, t1 - q), 0});
        acls_chunks.push_back({c0, (int)chunks.size()});
      }
    double* dG = dev_array<double>(c, buf.b[0], n4);
    QDKGB_CUDA(cudaMemsetAsync(dG, 0, n4 * 8, c->stream));
    if (!chunks.empty()) {
      auto up = [&](DeviceBuffer& b, const void* src, size_t bytes) {
        void* p = dev_alloc(c, b, bytes + 16);
        QDKGB_CUDA(cudaMemcpyAsync(p, src, bytes, cudaMemcpyHostToDevice, c->stream));
        return p;
      };
      const uint32_t* d_bl = (const uint32_t*)up(buf.b[1], blist.data(), blist.size() * 4);
      const CasItem* d_it = (const CasItem*)up(buf.b[2], items.data(), items.size() * sizeof(CasItem));
      const uint32_t* d_at = (const uint32_t*)up(buf.b[3], atr.data(), atr.size() * 4);
      const int4* d_ch = (const int4*)up(buf.b[4], chunks.data(), chunks.size() * sizeof(int4));
      const int2* d_ac = (const int2*)up(buf.b[5], acls.data(), acls.size() * sizeof(int2));
      const int2* d_acc = (const int2*)up(buf.b[6], acls_chunks.data(), acls_chunks.size() * sizeof(int2));
      const int2* d_bi = (const int2*)up(buf.b[7], bitems.data(), bitems.size() * sizeof(int2));
      double* d_part = dev_array<double>(c, buf.b[8], chunks.size() * nitems);
      const size_t smem = (size_t)2 * nb * 8;
      set_max_dynamic_smem((const void*)k_rdm_cas_ab, (int)std::max<size_t>(smem, 48 * 1024));
      k_rdm_cas_ab<<<(unsigned)chunks.size(), kCasThreads, smem, c->stream>>>(nb, dC, d_at, d_ch, d_it, nitems, d_bl,
                                                                               d_part);
      QDKGB_CHECK_LAUNCH();
      const int64_t nred = (int64_t)acls.size() * n2;
      k_rdm_cas_ab_reduce<<<(unsigned)((nred + 127) / 128), 128, 0, c->stream>>>(n, (int)acls.size(), d_ac, d_acc,
                                                                                   d_bi, nitems, d_part, dG);
      QDKGB_CHECK_LAUNCH();
    }
    QDKGB_CUDA(cudaMemcpyAsync(h4.data(), dG, n4 * 8, cudaMemcpyDeviceToHost, c->stream));
    QDKGB_CUDA(cudaStreamSynchronize(c->stream));
    for (size_t i = 0; i < n4; ++i) aabb[i] += h4[i];
  }

  // ---------------- same spin (aaaa + aa from alpha pairs, bbbb + bb from beta pairs)
  for (int blk = 0; blk < 2; ++blk) {
    double* o4 = blk == 0 ? aaaa : bbbb;
    double* o2 = blk == 0 ? aa : bb;
    if (!o4 && !o2) continue;
    const std::vector<uint64_t>& strs = blk == 0 ? S.h_galpha : S.h_ubeta;
    const std::vector<int32_t>& rk = blk == 0 ? ra : rb;
    // unordered string pairs within a double excitation, lower rank first
    std::vector<int2> pairs;
    const int64_t ns = (int64_t)strs.size();
    for (int64_t x = 0; x < ns; ++x) {
      const uint64_t s0 = strs[x];
      pairs.push_back({(int)x, (int)x});
      std::vector<int> occ, vir;
      for (int p = 0; p < n; ++p) ((s0 >> p) & 1 ? occ : vir).push_back(p);
      auto add = [&](uint64_t t) {
        const int32_t y = rk[t];
        if (y < 0) throw Error(QDKGB_ERR_UNSUPPORTED, "RDM: strings are not a complete set");
        if (y > x) pairs.push_back({(int)x, (int)y});
      };
      for (int o : occ)
        for (int v : vir) add(s0 ^ (1ull << o) ^ (1ull << v));
      for (size_t a = 0; a < occ.size(); ++a)
        for (size_t b2 = a + 1; b2 < occ.size(); ++b2)
          for (size_t u = 0; u < vir.size(); ++u)
            for (size_t w = u + 1; w < vir.size(); ++w)
              add(s0 ^ (1ull << occ[a]) ^ (1ull << occ[b2]) ^ (1ull << vir[u]) ^ (1ull << vir[w]));
    }
    const int64_t np = (int64_t)pairs.size();
    int2* d_pairs = (int2*)dev_alloc(c, buf.b[9], np * sizeof(int2) + 16);
    QDKGB_CUDA(cudaMemcpyAsync(d_pairs, pairs.data(), np * sizeof(int2), cudaMemcpyHostToDevice, c->stream));
    double* d_S = dev_array<double>(c, buf.b[10], np);
    const double* X = dC;
    int64_t cols = nb;
    if (blk == 1) {  // columns of C as rows
      double* Ct = dev_array<double>(c, buf.b[11], N);
      transpose_f64(c, dC, Ct, na, nb);
      X = Ct;
      cols = na;
    }
    k_pair_overlap<<<(unsigned)std::min<int64_t>((np * 32 + 255) / 256, (int64_t)c->sm_count * 64), 256, 0,
                     c->stream>>>(np, d_pairs, X, cols, d_S);
    QDKGB_CHECK_LAUNCH();
    uint64_t* d_str = (uint64_t*)dev_alloc(c, buf.b[1], strs.size() * 8 + 16);
    QDKGB_CUDA(cudaMemcpyAsync(d_str, strs.data(), strs.size() * 8, cudaMemcpyHostToDevice, c->stream));
    double* d4 = dev_array<double>(c, buf.b[2], n4);
    double* d2 = dev_array<double>(c, buf.b[3], n2);
    QDKGB_CUDA(cudaMemsetAsync(d4, 0, n4 * 8, c->stream));
    QDKGB_CUDA(cudaMemsetAsync(d2, 0, n2 * 8, c->stream));
    RdmTarget T;
    T.block = blk;
    T.n = n;
    T.s_lo = 0;
    T.s_hi = n;
    T.t4 = d4;
    T.t2 = d2;
    T.shared = false;
    T.with_ordm = true;
    k_rdm_cas_same_spin<<<(unsigned)std::min<int64_t>((np + 255) / 256, (int64_t)c->sm_count * 16), 256, 0,
                          c->stream>>>(np, d_pairs, d_str, d_S, T);
    QDKGB_CHECK_LAUNCH();
    QDKGB_CUDA(cudaStreamSynchronize(c->stream));
    if (o4) {
      QDKGB_CUDA(cudaMemcpy(h4.data(), d4, n4 * 8, cudaMemcpyDeviceToHost));
      for (size_t i = 0; i < n4; ++i) o4[i] += h4[i];
    }
    if (o2) {
      QDKGB_CUDA(cudaMemcpy(h2.data(), d2, n2 * 8, cudaMemcpyDeviceToHost));
      for (size_t i = 0; i < n2; ++i) o2[i] += h2[i];
    }
  }
  return true;
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
  // QDKGB_RDM_PAIR_WALK=1 keeps complete spaces on the pair walk (a test
  // compares the two paths)
  const char* walk = getenv("QDKGB_RDM_PAIR_WALK");
  const bool force_walk = walk && walk[0] == '1';
  if (!force_walk && cas_rdm_eligible(c) && rdms_cas(c, dC, aa, bb, aaaa, bbbb, aabb)) return;
  double* d4 = dev_array<double>(c, b4, n4);
  unsigned long long* d2 = dev_array<unsigned long long>(c, b2, 2 * n2);
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
  std::vector<double> h4(n4);
  std::vector<long long> h2(2 * n2);
  // the fixed point's unit: the power of two at or above max C^2
  double cmax = 0.;
  for (int64_t i = 0; i < N; ++i) cmax = std::max(cmax, std::fabs(C[i]));
  int e2 = 0;
  if (cmax > 0.) std::frexp(cmax * cmax, &e2);
  const double fx_s = std::ldexp(1.0, e2), fx_inv = std::ldexp(1.0, -e2);
  for (int blk = 0; blk < 3; ++blk) {
    if (!outs4[blk] && !outs2[blk]) continue;
    QDKGB_CUDA(cudaMemsetAsync(d4, 0, n4 * 8, c->stream));
    QDKGB_CUDA(cudaMemsetAsync(d2, 0, 2 * n2 * 8, c->stream));
    for (int s0 = 0; s0 < n; s0 += s_step) {
      RdmTarget T;
      T.block = blk;
      T.n = n;
      T.s_lo = s0;
      T.s_hi = use_shared ? std::min(n, s0 + s_step) : n;
      T.shared = use_shared;
      T.with_ordm = (s0 == 0);
      T.t4 = use_shared ? nullptr : d4;
      T.t2 = nullptr;
      T.t2fx = (blk < 2 && T.with_ordm) ? d2 : nullptr;
      T.fx_inv = fx_inv;
      const size_t tile = use_shared ? n2 * n * (T.s_hi - T.s_lo) * 8 : 0;  // the 1-RDM goes to t2fx
      k_rdm<<<(unsigned)blocks, kRdmWarps * 32, tile, c->stream>>>(a, dC, T, d4, nullptr);
      QDKGB_CHECK_LAUNCH();
      if (!use_shared) break;
    }
    QDKGB_CUDA(cudaStreamSynchronize(c->stream));
    if (outs4[blk]) {
      QDKGB_CUDA(cudaMemcpy(h4.data(), d4, n4 * 8, cudaMemcpyDeviceToHost));
      for (size_t i = 0; i < n4; ++i) outs4[blk][i] += h4[i];
    }
    if (outs2[blk]) {
      QDKGB_CUDA(cudaMemcpy(h2.data(), d2, 2 * n2 * 8, cudaMemcpyDeviceToHost));
      for (size_t i = 0; i < n2; ++i)
        outs2[blk][i] +=
            ((double)h2[2 * i] * (1.0 / kRdmFixHi) + (double)h2[2 * i + 1] * (1.0 / kRdmFixLo)) * fx_s;
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
