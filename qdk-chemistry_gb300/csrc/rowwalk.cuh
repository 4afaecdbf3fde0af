// Row walk over the connected determinants of one determinant (shared by the
// CSR build, the RDM kernels and the direct sigma).  See hbuild.cu for the
// design.
#pragma once
#include "common.cuh"
#include "internal.h"

namespace qdkgb {

struct RowArgs {
  Integrals I;
  int64_t ndets;
  const uint64_t* galpha;
  const int64_t* gstart;
  const int32_t* det_group;
  const int32_t* brank;
  const uint64_t* ubeta;
  const uint8_t* gcomplete;
  const int64_t* acon_ptr;
  const int32_t* acon_idx;
  const int8_t* acon_lvl;
  const int64_t* b2_ptr;
  const int32_t* b2_idx;
  const int64_t* b1_ptr;
  const int32_t* b1_idx;
  double thresh;
};

enum : int { kIdent = 0, kSearch = 1, kScan = 2 };
constexpr int kRowWarps = 8;

// Position of rank `cval` inside the sorted rank list [lo, hi); -1 if absent.
__device__ __forceinline__ int64_t find_rank(const int32_t* __restrict__ br, int64_t lo, int64_t hi, int32_t cval) {
  const int64_t end = hi;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    const int32_t v = __ldg(br + mid);
    if (v < cval)
      lo = mid + 1;
    else
      hi = mid;
  }
  return (lo < end && __ldg(br + lo) == cval) ? lo : -1;
}

// Walks the connected columns of row r in ascending order and calls
// visit(col, value) for every kept element.  Shared by the count and emit
// passes, and (with a different visitor) by the direct-sigma and RDM kernels.
template <int W>
struct RowWalkSmemT {
  int off[W][33];
  int h[W][32];
  int8_t lvl[W][32];
  int8_t mode[W][32];
};
using RowWalkSmem = RowWalkSmemT<kRowWarps>;

template <typename Smem, typename Visit>
__device__ __forceinline__ void walk_row(const RowArgs& a, int64_t r, int w, int lane, Smem& sm,
                                         Visit&& visit) {
  const int32_t g = a.det_group[r];
  const int32_t b = a.brank[r];
  const uint64_t ra = a.galpha[g], rb = a.ubeta[b];
  if (ra == 0) return;  // the reference skips alpha-empty groups
  const int64_t b1 = a.b1_ptr[b], n1 = a.b1_ptr[b + 1] - b1;
  const int64_t b2 = a.b2_ptr[b], n2 = a.b2_ptr[b + 1] - b2;
  const int64_t e_end = a.acon_ptr[g + 1];
  for (int64_t e0 = a.acon_ptr[g]; e0 < e_end; e0 += 32) {
    const int64_t e = e0 + lane;
    int my = 0, h = 0, lvl = 0, mode = kIdent;
    if (e < e_end) {
      h = a.acon_idx[e];
      lvl = a.acon_lvl[e];
      const int64_t gs = a.gstart[h + 1] - a.gstart[h];
      const int64_t cand = lvl == 0 ? n2 : (lvl == 1 ? n1 : 1);
      if (a.gcomplete[h]) {
        mode = kIdent;
        my = (int)cand;
      } else if (gs <= cand) {
        mode = kScan;
        my = (int)gs;
      } else {
        mode = kSearch;
        my = (int)cand;
      }
    }
    const int incl = warp_inclusive_scan(my, lane);
    const int total = __shfl_sync(QDKGB_FULL_MASK, incl, 31);
    sm.off[w][lane + 1] = incl;
    if (lane == 0) sm.off[w][0] = 0;
    sm.h[w][lane] = h;
    sm.lvl[w][lane] = (int8_t)lvl;
    sm.mode[w][lane] = (int8_t)mode;
    __syncwarp();
    for (int base = 0; base < total; base += 32) {
      const int f = base + lane;
      int64_t ket = -1;
      uint64_t ka = 0, kb = 0;
      if (f < total) {
        int lo = 0, hi = 31;
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (sm.off[w][mid] <= f)
            lo = mid;
          else
            hi = mid - 1;
        }
        const int k = f - sm.off[w][lo];
        const int hh = sm.h[w][lo], ll = sm.lvl[w][lo], md = sm.mode[w][lo];
        const int64_t g0 = a.gstart[hh];
        ka = a.galpha[hh];
        if (md == kScan) {
          const int64_t d = g0 + k;
          kb = a.ubeta[a.brank[d]];
          if (popc64(rb ^ kb) <= 2 * (2 - ll)) ket = d;
        } else {
          const int32_t cr = ll == 0 ? a.b2_idx[b2 + k] : (ll == 1 ? a.b1_idx[b1 + k] : b);
          kb = a.ubeta[cr];
          if (md == kIdent)
            ket = g0 + cr;
          else
            ket = find_rank(a.brank, g0, a.gstart[hh + 1], cr);
        }
      }
      visit(ket, r, ra, rb, ka, kb);
    }
    __syncwarp();
  }
}

// Matrix element of the (row, ket) pair with the lower-index determinant as
// bra, as the reference's mirrored fill does (sorted_double_loop.hpp:325-355).
__device__ __forceinline__ double pair_value(const Integrals& I, int64_t r, int64_t ket, uint64_t ra, uint64_t rb,
                                             uint64_t ka, uint64_t kb) {
  return (ket >= r) ? matrix_element(I, ra, rb, ka, kb) : matrix_element(I, ka, kb, ra, rb);
}


RowArgs row_args(Context* c, double thresh);

}  // namespace qdkgb
