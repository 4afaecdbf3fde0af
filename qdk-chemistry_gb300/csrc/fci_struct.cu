// Structured kernels for complete (CAS) determinant spaces.
//
// In a full (n_alpha, n_beta) product space every row has the same shape: the
// row of determinant r = g * N_b + b (alpha group g, beta string b) holds, in
// ascending column order, one block per alpha group h within a double
// excitation of g - the beta strings within level 2 of b for h = g, within
// level 1 for an alpha single, b alone for an alpha double.  The position of
// every element inside its row is therefore known from (g, entry, k) alone:
// per alpha group three short tables (the level-1 and level-2 groups with the
// offset of their block in the row, and the offset of the own-group block)
// replace the per-element search of the general row walk.
//
// Two uses:
//  * emission: each element is written at its fixed slot (columns and values),
//    elements that fail |h| > thresh are marked and removed by a compaction
//    pass only when any exist;
//  * sigma without column indices: when no element was removed, the CSR
//    columns of row r are implied by these tables, so the sigma streams only
//    the values (4 B per nonzero in FP32, 8 B in FP64) and regenerates the
//    columns from tables that stay in L1/L2.
#include <algorithm>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "internal.h"

namespace qdkgb {

struct FciStruct {
  int64_t G = 0, Nb = 0;
  int n1 = 0, n2 = 0;  // beta list lengths (level <= 1, level <= 2), uniform
  int c1 = 0, c2 = 0;  // alpha singles / doubles per group, uniform
  int64_t rowlen = 0;  // n2 + c1 * n1 + c2
  DeviceBuffer l0_off, l1_h, l1_off, l2_h, l2_off;
};

void free_struct(Context* c) {
  if (!c->fci) return;
  for (DeviceBuffer* b : {&c->fci->l0_off, &c->fci->l1_h, &c->fci->l1_off, &c->fci->l2_h, &c->fci->l2_off})
    dev_free(c, *b);
  delete c->fci;
  c->fci = nullptr;
}

// Called at the end of build_det_space: keeps the tables when the space is a
// full product with uniform list lengths, else leaves c->fci null.
void build_struct(Context* c) {
  free_struct(c);
  DetSpace& D = c->dets;
  const int64_t G = D.ngroups, Nb = D.nbeta;
  if (G * Nb != D.ndets || G < 1) return;
  for (int64_t g = 0; g < G; ++g) {
    if (D.h_gstart[g + 1] - D.h_gstart[g] != Nb) return;
    if (D.h_galpha[g] == 0) return;
  }
  if (D.ndets >= (int64_t)INT32_MAX) return;
  // beta list lengths
  std::vector<int64_t> b1p(Nb + 1), b2p(Nb + 1);
  QDKGB_CUDA(cudaMemcpy(b1p.data(), D.b1_ptr.ptr, (Nb + 1) * 8, cudaMemcpyDeviceToHost));
  QDKGB_CUDA(cudaMemcpy(b2p.data(), D.b2_ptr.ptr, (Nb + 1) * 8, cudaMemcpyDeviceToHost));
  const int64_t n1 = b1p[1] - b1p[0], n2 = b2p[1] - b2p[0];
  for (int64_t b = 0; b < Nb; ++b)
    if (b1p[b + 1] - b1p[b] != n1 || b2p[b + 1] - b2p[b] != n2) return;
  // alpha connectivity, split by level with each block's offset in the row
  std::vector<int64_t> ap(G + 1);
  QDKGB_CUDA(cudaMemcpy(ap.data(), D.acon_ptr.ptr, (G + 1) * 8, cudaMemcpyDeviceToHost));
  std::vector<int32_t> aidx(ap[G]);
  std::vector<int8_t> alvl(ap[G]);
  if (ap[G]) {
    QDKGB_CUDA(cudaMemcpy(aidx.data(), D.acon_idx.ptr, ap[G] * 4, cudaMemcpyDeviceToHost));
    QDKGB_CUDA(cudaMemcpy(alvl.data(), D.acon_lvl.ptr, ap[G], cudaMemcpyDeviceToHost));
  }
  int c1 = -1, c2 = -1;
  std::vector<int32_t> l0(G), l1h, l1o, l2h, l2o;
  for (int64_t g = 0; g < G; ++g) {
    int64_t off = 0;
    int k1 = 0, k2 = 0, k0 = 0;
    for (int64_t e = ap[g]; e < ap[g + 1]; ++e) {
      const int lv = alvl[e];
      if (lv == 0) {
        if (aidx[e] != g) return;  // repeated alpha string
        l0[g] = (int32_t)off;
        off += n2;
        ++k0;
      } else if (lv == 1) {
        l1h.push_back(aidx[e]);
        l1o.push_back((int32_t)off);
        off += n1;
        ++k1;
      } else {
        l2h.push_back(aidx[e]);
        l2o.push_back((int32_t)off);
        off += 1;
        ++k2;
      }
    }
    if (k0 != 1) return;
    if (c1 < 0) {
      c1 = k1;
      c2 = k2;
    }
    if (k1 != c1 || k2 != c2) return;
  }
  FciStruct* F = new FciStruct();
  F->G = G;
  F->Nb = Nb;
  F->n1 = (int)n1;
  F->n2 = (int)n2;
  F->c1 = c1;
  F->c2 = c2;
  F->rowlen = n2 + (int64_t)c1 * n1 + c2;
  auto up = [&](DeviceBuffer& b, const std::vector<int32_t>& v) {
    void* p = dev_alloc(c, b, std::max<size_t>(v.size(), 1) * 4 + 16);
    if (!v.empty()) QDKGB_CUDA(cudaMemcpy(p, v.data(), v.size() * 4, cudaMemcpyHostToDevice));
  };
  up(F->l0_off, l0);
  up(F->l1_h, l1h);
  up(F->l1_off, l1o);
  up(F->l2_h, l2h);
  up(F->l2_off, l2o);
  c->fci = F;
}

namespace {

struct SArgs {
  int64_t G, Nb;
  int n1, n2, c1, c2;
  int64_t rowlen;
  const int32_t* l0_off;
  const int32_t* l1_h;
  const int32_t* l1_off;
  const int32_t* l2_h;
  const int32_t* l2_off;
  const int32_t* b1_idx;  // [Nb][n1]
  const int32_t* b2_idx;  // [Nb][n2]
};

SArgs sargs(Context* c) {
  FciStruct* F = c->fci;
  SArgs s;
  s.G = F->G;
  s.Nb = F->Nb;
  s.n1 = F->n1;
  s.n2 = F->n2;
  s.c1 = F->c1;
  s.c2 = F->c2;
  s.rowlen = F->rowlen;
  s.l0_off = (const int32_t*)F->l0_off.ptr;
  s.l1_h = (const int32_t*)F->l1_h.ptr;
  s.l1_off = (const int32_t*)F->l1_off.ptr;
  s.l2_h = (const int32_t*)F->l2_h.ptr;
  s.l2_off = (const int32_t*)F->l2_off.ptr;
  s.b1_idx = (const int32_t*)c->dets.b1_idx.ptr;
  s.b2_idx = (const int32_t*)c->dets.b2_idx.ptr;
  return s;
}

// Calls f(pos_in_row, col) for every element of row r (g = r / Nb, b = r % Nb),
// lanes striding three flat ranges; the order is free, positions are exact.
template <typename F>
__device__ __forceinline__ void for_each_struct(const SArgs& s, int64_t g, int64_t b, int lane, F&& f) {
  const int64_t gb = g * s.Nb;
  const int32_t o0 = __ldg(s.l0_off + g);
  const int32_t* b2 = s.b2_idx + b * s.n2;
  for (int k = lane; k < s.n2; k += 32) f((int64_t)o0 + k, gb + __ldg(b2 + k));
  const int32_t* b1 = s.b1_idx + b * s.n1;
  const int64_t t1 = (int64_t)s.c1 * s.n1;
  for (int64_t t = lane; t < t1; t += 32) {
    const int e = (int)(t / s.n1), k = (int)(t - (int64_t)e * s.n1);
    const int64_t ge = g * s.c1 + e;
    f((int64_t)__ldg(s.l1_off + ge) + k, (int64_t)__ldg(s.l1_h + ge) * s.Nb + __ldg(b1 + k));
  }
  for (int t = lane; t < s.c2; t += 32) {
    const int64_t ge = g * s.c2 + t;
    f((int64_t)__ldg(s.l2_off + ge), (int64_t)__ldg(s.l2_h + ge) * s.Nb + b);
  }
}

template <int STORAGE>
__global__ void __launch_bounds__(256)
    k_struct_emit(SArgs s, Integrals I, const uint64_t* __restrict__ galpha, const uint64_t* __restrict__ ubeta,
                  long long tbits, const double* __restrict__ diag_raw, int32_t* __restrict__ colind,
                  double* __restrict__ val, float* __restrict__ hi, float* __restrict__ lo,
                  double* __restrict__ diag, int64_t* __restrict__ kept) {
  const int lane = threadIdx.x & 31;
  const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t n = s.G * s.Nb;
  for (int64_t r = w0; r < n; r += nw) {
    const int64_t g = r / s.Nb, b = r - g * s.Nb;
    const uint64_t ra = galpha[g], rb = ubeta[b];
    const int64_t base = r * s.rowlen;
    int cnt = 0;
    for_each_struct(s, g, b, lane, [&](int64_t pos, int64_t col) {
      double v;
      bool keep;
      if (col == r) {
        v = diag_raw[r];
        keep = above_thresh(v, tbits);
        diag[r] = keep ? v : 0.;
      } else {
        const int64_t h = col / s.Nb, cb = col - h * s.Nb;
        const uint64_t ka = galpha[h], kb = ubeta[cb];
        v = (col > r) ? offdiag_element(I, ra, rb, ka, kb) : offdiag_element(I, ka, kb, ra, rb);
        keep = above_thresh(v, tbits);
      }
      const int64_t p = base + pos;
      colind[p] = keep ? (int32_t)col : -1;
      if (STORAGE == QDKGB_H_FP64) {
        val[p] = v;
      } else {
        const float h32 = __double2float_rn(v);
        hi[p] = h32;
        lo[p] = __double2float_rn(v - (double)h32);
      }
      cnt += keep;
    });
    cnt = warp_sum(cnt);
    if (lane == 0) kept[r] = cnt;
  }
}

// compaction of the marked slots into the final CSR (threshold_parallel's
// rule, csr_matrix.hpp:317-372): warp per row, ballot packing in order
template <int STORAGE>
__global__ void k_struct_compact(int64_t n, int64_t rowlen, const int64_t* __restrict__ new_ptr,
                                 const int32_t* __restrict__ ci, const double* __restrict__ v,
                                 const float* __restrict__ h, const float* __restrict__ l, int32_t* __restrict__ ci2,
                                 double* __restrict__ v2, float* __restrict__ h2, float* __restrict__ l2) {
  const int lane = threadIdx.x & 31;
  const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = w0; r < n; r += nw) {
    const int64_t src = r * rowlen;
    int64_t dst = new_ptr[r];
    for (int64_t k0 = 0; k0 < rowlen; k0 += 32) {
      const int64_t k = k0 + lane;
      const bool keep = k < rowlen && ci[src + k] >= 0;
      const unsigned m = __ballot_sync(QDKGB_FULL_MASK, keep);
      if (keep) {
        const int64_t p = dst + __popc(m & ((1u << lane) - 1u));
        ci2[p] = ci[src + k];
        if (STORAGE == QDKGB_H_FP64) {
          v2[p] = v[src + k];
        } else {
          h2[p] = h[src + k];
          l2[p] = l[src + k];
        }
      }
      dst += __popc(m);
    }
  }
}

template <typename Acc, typename X, typename Val>
__global__ void __launch_bounds__(256)
    k_struct_spmv(SArgs s, Val val, const X* __restrict__ x, X* __restrict__ y) {
  const int lane = threadIdx.x & 31;
  const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t n = s.G * s.Nb;
  for (int64_t r = w0; r < n; r += nw) {
    const int64_t g = r / s.Nb, b = r - g * s.Nb;
    const int64_t base = r * s.rowlen;
    Acc acc = 0;
    for_each_struct(s, g, b, lane, [&](int64_t pos, int64_t col) { acc += val(base + pos) * (Acc)__ldg(x + col); });
    acc = warp_sum(acc);
    if (lane == 0) y[r] = (X)acc;
  }
}

struct SValF64 {
  const double* v;
  __device__ __forceinline__ double operator()(int64_t k) const { return __ldcs(v + k); }
};
struct SValF32 {
  const float* v;
  __device__ __forceinline__ float operator()(int64_t k) const { return __ldcs(v + k); }
};

}  // namespace

bool struct_ready(Context* c) { return c->fci && c->H.valid && !c->op_direct && c->H.structured; }

unsigned struct_blocks(Context* c, int64_t n) {
  return (unsigned)std::min<int64_t>((n + 7) / 8, (int64_t)c->sm_count * 32);
}

void struct_spmv_fp64(Context* c, const double* x, double* y) {
  SArgs s = sargs(c);
  k_struct_spmv<double, double><<<struct_blocks(c, c->H.n), 256, 0, c->stream>>>(
      s, SValF64{(const double*)c->H.val.ptr}, x, y);
  QDKGB_CHECK_LAUNCH();
}
void struct_spmv_fp32(Context* c, const float* x, float* y) {
  SArgs s = sargs(c);
  k_struct_spmv<float, float><<<struct_blocks(c, c->H.n), 256, 0, c->stream>>>(
      s, SValF32{(const float*)c->H.hi.ptr}, x, y);
  QDKGB_CHECK_LAUNCH();
}

// Structured build for complete spaces (build_hamiltonian dispatches here).
void build_hamiltonian_struct(Context* c, double thresh, int storage) {
  Hcsr& H = c->H;
  DetSpace& D = c->dets;
  FciStruct* F = c->fci;
  const int64_t n = D.ndets;
  const int64_t nnz_pre = n * F->rowlen;
  long long tbits = -1;
  if (thresh > 0.) std::memcpy(&tbits, &thresh, sizeof(double));
  Integrals I = integrals_view(c);
  double* diag_raw = dev_array<double>(c, H.diag_raw, n);
  double* diag = dev_array<double>(c, H.diag, n);
  int64_t* kept = dev_array<int64_t>(c, H.row_nnz, n + 1);
  const unsigned tb = (unsigned)std::min<int64_t>((n + 255) / 256, (int64_t)c->sm_count * 16);
  k_diag_launch(c, I, diag_raw, tb);
  if (storage == QDKGB_H_FP64) {
    dev_free(c, H.hi);
    dev_free(c, H.lo);
  } else {
    dev_free(c, H.val);
  }
  int32_t* colind = dev_array<int32_t>(c, H.colind, nnz_pre);
  double* val = storage == QDKGB_H_FP64 ? dev_array<double>(c, H.val, nnz_pre) : nullptr;
  float* hi = storage == QDKGB_H_SPLIT32 ? dev_array<float>(c, H.hi, nnz_pre) : nullptr;
  float* lo = storage == QDKGB_H_SPLIT32 ? dev_array<float>(c, H.lo, nnz_pre) : nullptr;
  QDKGB_CUDA(cudaMemsetAsync(diag, 0, n * sizeof(double), c->stream));
  SArgs s = sargs(c);
  const unsigned eb = struct_blocks(c, n);
  const uint64_t* ga = (const uint64_t*)D.galpha.ptr;
  const uint64_t* ub = (const uint64_t*)D.ubeta.ptr;
  if (storage == QDKGB_H_FP64)
    k_struct_emit<QDKGB_H_FP64><<<eb, 256, 0, c->stream>>>(s, I, ga, ub, tbits, diag_raw, colind, val, hi, lo, diag,
                                                            kept);
  else
    k_struct_emit<QDKGB_H_SPLIT32><<<eb, 256, 0, c->stream>>>(s, I, ga, ub, tbits, diag_raw, colind, val, hi, lo,
                                                               diag, kept);
  QDKGB_CHECK_LAUNCH();
  int64_t* rowptr = dev_array<int64_t>(c, H.rowptr, n + 1);
  exclusive_scan_i64(c, kept, rowptr, n, H.scan_tmp);
  int64_t nnz = 0;
  QDKGB_CUDA(cudaMemcpyAsync(&nnz, rowptr + n, sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
  QDKGB_CUDA(cudaStreamSynchronize(c->stream));
  H.structured = (nnz == nnz_pre);
  if (!H.structured) {
    DeviceBuffer ci2b, v2b, h2b, l2b;
    const int64_t cap2 = std::max<int64_t>(nnz, 1);
    int32_t* ci2 = dev_array<int32_t>(c, ci2b, cap2);
    double* v2 = storage == QDKGB_H_FP64 ? dev_array<double>(c, v2b, cap2) : nullptr;
    float* h2 = storage == QDKGB_H_SPLIT32 ? dev_array<float>(c, h2b, cap2) : nullptr;
    float* l2 = storage == QDKGB_H_SPLIT32 ? dev_array<float>(c, l2b, cap2) : nullptr;
    if (storage == QDKGB_H_FP64)
      k_struct_compact<QDKGB_H_FP64>
          <<<eb, 256, 0, c->stream>>>(n, F->rowlen, rowptr, colind, val, hi, lo, ci2, v2, h2, l2);
    else
      k_struct_compact<QDKGB_H_SPLIT32>
          <<<eb, 256, 0, c->stream>>>(n, F->rowlen, rowptr, colind, val, hi, lo, ci2, v2, h2, l2);
    QDKGB_CHECK_LAUNCH();
    QDKGB_CUDA(cudaStreamSynchronize(c->stream));
    std::swap(H.colind, ci2b);
    dev_free(c, ci2b);
    if (storage == QDKGB_H_FP64) {
      std::swap(H.val, v2b);
      dev_free(c, v2b);
    } else {
      std::swap(H.hi, h2b);
      std::swap(H.lo, l2b);
      dev_free(c, h2b);
      dev_free(c, l2b);
    }
  }
  H.n = n;
  H.nnz = nnz;
  H.storage = storage;
  H.thresh = thresh;
  H.valid = true;
}

}  // namespace qdkgb
