// Direct (recompute-on-the-fly) sigma for complete active spaces.
//
// For CASCI spaces whose CSR would not fit in HBM (CAS(14e,14o): 11.8M
// determinants, 3.98e10 nonzeros, ~478 GB as CSR) the Hamiltonian is never
// stored.  A full (n_alpha, n_beta) product space is a matrix C[I_a, I_b]
// (determinant I_a * N_b + I_b, the reference's alpha-major order), and
//   sigma = diag(D) C + S_aa(C) + S_bb(C) + S_ab(C)
// where, with MACIS's matrix elements (matrix_elements.hpp:65-230):
//   S_aa(C)[Ia, Ib] = sum_{Ja: alpha double of Ia} V_aa(Ia,Ja) C[Ja, Ib]
//                   + sum_{Ja: alpha single of Ia, (v,o)} s (A(Ia,Ja) + W_b[(v,o), Ib]) C[Ja, Ib]
//     A(Ia, Ja)   = T(v,o) + sum_{p in Ia} G_red(p,v,o)      (string-only part)
//     W_b[(v,o), Ib] = sum_{p in Ib} V_red(p,v,o)             (the other spin's part)
//   S_bb: the same with the spins exchanged (applied to C^T);
//   S_ab(C)[Ia, Ib] = sum_{k: alpha single of Ia} sum_{l: beta single of Ib}
//                     s_k s_l V(v_k, o_k, v_l, o_l) C[Ja_k, Jb_l].
// The string tables (singles and doubles of every string, with their values)
// are built once per space; they are kilobytes to tens of megabytes.  The
// opposite-spin term, the dominant cost (49 x 49 terms per determinant at
// CAS(14,14)), runs one CTA per alpha string with chunks of the alpha
// singles' rows C[Ja_k, :] staged in shared memory and the signed slices
// s_k V(v_k, o_k, :, :) beside them; each thread owns a set of beta strings
// and walks their singles list once per chunk.
// Element values equal the CSR build's up to the rounding of the single
// excitation's sum (A + W is summed in two parts here).
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <unordered_map>
#include <vector>

#include "common.cuh"
#include "internal.h"

namespace qdkgb {

namespace {

constexpr int kDsThreads = 256;
constexpr int kDsMaxCols = 16 * kDsThreads;  // up to 4096 strings of the other spin

// host copies of the reference's sign / index logic (sd_operations.hpp:27-50,394-425)
inline int hpopc(uint64_t x) { return __builtin_popcountll(x); }
inline uint32_t hlow(uint64_t x) { return (uint32_t)__builtin_ctzll(x); }
inline uint64_t hmask(uint32_t i) { return i >= 64 ? ~0ull : ((1ull << i) - 1ull); }
inline bool hsign_odd(uint64_t state, uint32_t p, uint32_t q) {
  const uint64_t m = (p > q) ? (hmask(p) ^ hmask(q + 1)) : (hmask(q) ^ hmask(p + 1));
  return hpopc(state & m) & 1;
}
struct HSingle {
  uint32_t o, v;
  bool neg;
};
inline HSingle hsingle(uint64_t bra, uint64_t ket, uint64_t ex) {
  HSingle s;
  s.o = hlow(ket & ex);
  s.v = hlow(bra & ex);
  s.neg = hsign_odd(ket, s.v, s.o);
  return s;
}

}  // namespace

// FP32 contraction form (k_ds_opposite_mm): beta strings J_b in chunks of
// kMmCols; E rows 16 per warp, each thread 4 rows x 8 columns.
constexpr int kMmCols = 64;
constexpr int kMmEStride = kMmCols + 4;  // row stride of E in shared memory (16-byte rows)
constexpr int kMmMaxWarps = 16;

struct SpinTables {
  int64_t nstr = 0;
  int ns = 0, nd = 0;
  DeviceBuffer sJ, svo, sA64, sA32, dJ, dval64, dval32, W64, W32;  // W over THIS spin's strings
  DeviceBuffer packed;  // singles packed as Jb | rs << 16 | neg << 31 (opposite-spin walk)
  std::vector<uint32_t> h_packed;  // host copy of `packed` while the contraction tables are built
};

struct DirectSigma {
  int n = 0;
  SpinTables a, b;
  bool same = false;  // beta tables alias alpha's (same string set)
  DeviceBuffer V32, tmp64, tmp32, ct64, ct32;
  // contraction form of the FP32 sigma (k_ds_opposite_mm).  Rows r of E:
  //   r < mr          pair (v, o), v != o, by ascending v + n o (mr = n (n - 1))
  //   mr + p, p < n   the other spin's occupied orbital p (single excitations' W part)
  //   mr + n          the string-only part of the alpha singles
  // mrows = mr + n + 1 rounded up to 16 is mrp (one warp per 16 rows).
  // V2mm[pq][r]: V(pq, rs_r) for r < mr, V(p p | pq) for r = mr + p, else 0.
  // lists: per chunk of kMmCols beta strings, the (nb + 1) uint16 offsets of
  // each beta string's entries (padded to 16 bytes) then the entries
  // jl | r << 8 | neg << 31 (jl = J_b - chunk start), each string's sorted by
  // (J_b, r); seg[c] = the chunk's first 4-byte word (16-byte aligned)
  bool mm = false;
  int mr = 0, mrp = 0, mm_threads = 0, mm_jpt = 0, seg_max = 0, off_words = 0;
  size_t mm_smem = 0;
  DeviceBuffer V2mm, rs_of, lists, seg;
};

void free_direct(Context* c) {
  if (!c->direct) return;
  DirectSigma* d = c->direct;
  for (SpinTables* t : {&d->a, &d->b})
    for (DeviceBuffer* b : {&t->sJ, &t->svo, &t->sA64, &t->sA32, &t->dJ, &t->dval64, &t->dval32, &t->W64, &t->W32,
                            &t->packed})
      dev_free(c, *b);
  for (DeviceBuffer* b : {&d->V32, &d->tmp64, &d->tmp32, &d->ct64, &d->ct32, &d->V2mm, &d->rs_of, &d->lists, &d->seg})
    dev_free(c, *b);
  delete d;
  c->direct = nullptr;
}

static void build_spin_tables(Context* c, const std::vector<uint64_t>& strs, SpinTables& t) {
  const int n = c->norb;
  const size_t nn = (size_t)n;
  const std::vector<double>& T = c->h_T;
  const std::vector<double>& V = c->h_V;
  auto Vat = [&](uint32_t p, uint32_t q, uint32_t r, uint32_t s) { return V[p + nn * (q + nn * (r + nn * s))]; };
  auto Gred = [&](uint32_t k, uint32_t i, uint32_t j) { return Vat(k, k, i, j) - Vat(k, j, i, k); };
  auto Vred = [&](uint32_t k, uint32_t i, uint32_t j) { return Vat(k, k, i, j); };
  const int64_t N = (int64_t)strs.size();
  std::unordered_map<uint64_t, int32_t> rank;
  for (int64_t i = 0; i < N; ++i) rank[strs[i]] = (int32_t)i;
  const int k = hpopc(strs[0]);
  const int ns = k * (n - k), nd = (k * (k - 1) / 2) * ((n - k) * (n - k - 1) / 2);
  t.nstr = N;
  t.ns = ns;
  t.nd = nd;
  std::vector<int32_t> sJ((size_t)N * ns), svo((size_t)N * ns), dJ((size_t)N * std::max(nd, 1));
  std::vector<double> sA((size_t)N * ns), dval((size_t)N * std::max(nd, 1));
  std::vector<uint32_t> packed((size_t)N * ns);
  std::vector<double> W(nn * nn * N);
  const uint64_t full = (n == 64) ? ~0ull : ((1ull << n) - 1ull);
  for (int64_t i = 0; i < N; ++i) {
    const uint64_t I = strs[i];
    std::vector<uint32_t> occ, vir;
    for (int p = 0; p < n; ++p) ((I >> p) & 1 ? occ : vir).push_back(p);
    int m = 0;
    for (uint32_t v : occ)
      for (uint32_t o : vir) {
        const uint64_t J = I ^ (1ull << v) ^ (1ull << o);
        auto it = rank.find(J);
        if (it == rank.end()) throw Error(QDKGB_ERR_UNSUPPORTED, "direct sigma needs a complete string set");
        HSingle s = hsingle(I, J, I ^ J);  // bra I, ket J: v in I, o in J
        double a = T[s.v + nn * s.o];
        for (uint32_t p : occ) a += Gred(p, s.v, s.o);
        sJ[(size_t)i * ns + m] = it->second;
        svo[(size_t)i * ns + m] = (int32_t)(s.v | (s.o << 8) | ((uint32_t)s.neg << 16));
        sA[(size_t)i * ns + m] = a;
        packed[(size_t)i * ns + m] =
            (uint32_t)it->second | ((uint32_t)(s.v + nn * s.o) << 16) | ((uint32_t)s.neg << 31);
        ++m;
      }
    m = 0;
    for (size_t x = 0; x < occ.size(); ++x)
      for (size_t y = x + 1; y < occ.size(); ++y)
        for (size_t u = 0; u < vir.size(); ++u)
          for (size_t w = u + 1; w < vir.size(); ++w) {
            const uint64_t J = I ^ (1ull << occ[x]) ^ (1ull << occ[y]) ^ (1ull << vir[u]) ^ (1ull << vir[w]);
            auto it = rank.find(J);
            if (it == rank.end()) throw Error(QDKGB_ERR_UNSUPPORTED, "direct sigma needs a complete string set");
            // matrix_element_4 with doubles_sign_indices (bra I, ket J)
            uint64_t ket = J, ex = I ^ J;
            HSingle s1 = hsingle(I, ket, ex);
            ket ^= (1ull << s1.o) | (1ull << s1.v);
            ex ^= (1ull << s1.o) | (1ull << s1.v);
            HSingle s2 = hsingle(I, ket, ex);
            const double g = Vat(s1.v, s1.o, s2.v, s2.o) - Vat(s1.v, s2.o, s2.v, s1.o);
            dJ[(size_t)i * nd + m] = it->second;
            dval[(size_t)i * nd + m] = (s1.neg != s2.neg) ? -g : g;
            ++m;
          }
    // W[(v,o)][i] = sum_{p in I} V_red(p, v, o)
    for (uint32_t o = 0; o < (uint32_t)n; ++o)
      for (uint32_t v = 0; v < (uint32_t)n; ++v) {
        double w = 0.;
        for (uint32_t p : occ) w += Vred(p, v, o);
        W[(v + nn * o) * N + i] = w;
      }
    (void)full;
  }
  auto up = [&](DeviceBuffer& b, const void* src, size_t bytes) {
    void* p = dev_alloc(c, b, bytes + 16);
    QDKGB_CUDA(cudaMemcpyAsync(p, src, bytes, cudaMemcpyHostToDevice, c->stream));
  };
  auto to32 = [](const std::vector<double>& x) {
    std::vector<float> y(x.size());
    for (size_t i = 0; i < x.size(); ++i) y[i] = (float)x[i];
    return y;
  };
  up(t.sJ, sJ.data(), sJ.size() * 4);
  up(t.svo, svo.data(), svo.size() * 4);
  up(t.sA64, sA.data(), sA.size() * 8);
  std::vector<float> sA32 = to32(sA), dval32 = to32(dval), W32 = to32(W);
  up(t.sA32, sA32.data(), sA32.size() * 4);
  up(t.dJ, dJ.data(), dJ.size() * 4);
  up(t.dval64, dval.data(), dval.size() * 8);
  up(t.dval32, dval32.data(), dval32.size() * 4);
  up(t.W64, W.data(), W.size() * 8);
  up(t.W32, W32.data(), W32.size() * 4);
  up(t.packed, packed.data(), packed.size() * 4);
  t.h_packed = std::move(packed);
  QDKGB_CUDA(cudaStreamSynchronize(c->stream));
}

// out[I, col] (+)= sum over same-spin doubles and singles of row string I
// (rows: strings of this spin; cols: strings of the other spin; W over the
// other spin's strings; W null: the singles' string-only part A alone).
template <typename T>
__global__ void __launch_bounds__(kDsThreads)
    k_ds_same_spin(int64_t nrow, int64_t ncol, int ns, int nd, const int32_t* __restrict__ sJ,
                   const int32_t* __restrict__ svo, const T* __restrict__ sA, const int32_t* __restrict__ dJ,
                   const T* __restrict__ dval, const T* __restrict__ W, int n, const T* __restrict__ C,
                   T* __restrict__ out) {
  const int64_t I = blockIdx.x;
  if (I >= nrow) return;
  for (int64_t col = threadIdx.x; col < ncol; col += blockDim.x) {
    T acc = 0;
    for (int m = 0; m < nd; ++m) acc += __ldg(dval + I * nd + m) * __ldg(C + (int64_t)__ldg(dJ + I * nd + m) * ncol + col);
    for (int m = 0; m < ns; ++m) {
      const int32_t vo = __ldg(svo + I * ns + m);
      const int v = vo & 0xff, o = (vo >> 8) & 0xff;
      T coef = __ldg(sA + I * ns + m);
      if (W) coef += __ldg(W + (int64_t)(v + n * o) * ncol + col);
      if (vo >> 16) coef = -coef;
      acc += coef * __ldg(C + (int64_t)__ldg(sJ + I * ns + m) * ncol + col);
    }
    out[I * ncol + col] = acc;
  }
}

template <typename T>
__device__ __forceinline__ T negate_if(T v, bool neg);
template <>
__device__ __forceinline__ double negate_if<double>(double v, bool neg) {
  return flip_if(v, neg);
}
template <>
__device__ __forceinline__ float negate_if<float>(float v, bool neg) {
  return __int_as_float(__float_as_int(v) ^ ((int)neg << 31));
}

// sigma[Ia, Ib] += D C + opposite-spin term (see the file comment).
template <typename T, int KC>
__global__ void __launch_bounds__(kDsThreads)
    k_ds_opposite(int64_t na, int64_t nb, int nsa, int nsb, const int32_t* __restrict__ a_sJ,
                  const int32_t* __restrict__ a_svo, const uint32_t* __restrict__ b_packed,
                  const T* __restrict__ Vt, int n, const double* __restrict__ D, const T* __restrict__ C,
                  T* __restrict__ sigma) {
  extern __shared__ unsigned char smem_raw[];
  T* rows = (T*)smem_raw;                          // KC x nb
  T* vsl = rows + (size_t)KC * nb;                 // KC x n^2 signed slices
  const int64_t Ia = blockIdx.x;
  if (Ia >= na) return;
  const int n2 = n * n;
  constexpr int JPT = kDsMaxCols / kDsThreads;
  T acc[JPT];
#pragma unroll
  for (int j = 0; j < JPT; ++j) {
    const int64_t col = threadIdx.x + (int64_t)j * kDsThreads;
    acc[j] = (col < nb) ? sigma[Ia * nb + col] + (T)D[Ia * nb + col] * C[Ia * nb + col] : (T)0;
  }
  for (int k0 = 0; k0 < nsa; k0 += KC) {
    const int kc = min(KC, nsa - k0);
    __syncthreads();
    for (int kk = 0; kk < kc; ++kk) {
      const int32_t Ja = __ldg(a_sJ + Ia * nsa + k0 + kk);
      const int32_t vo = __ldg(a_svo + Ia * nsa + k0 + kk);
      const int pq = (vo & 0xff) + n * ((vo >> 8) & 0xff);
      const bool neg = (vo >> 16) != 0;
      for (int64_t col = threadIdx.x; col < nb; col += blockDim.x) rows[kk * nb + col] = C[(int64_t)Ja * nb + col];
      for (int rs = threadIdx.x; rs < n2; rs += blockDim.x)
        vsl[kk * n2 + rs] = negate_if<T>(Vt[pq + (int64_t)n2 * rs], neg);
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < JPT; ++j) {
      const int64_t col = threadIdx.x + (int64_t)j * kDsThreads;
      if (col >= nb) break;
      const uint32_t* lst = b_packed + col * nsb;
      T a = acc[j];
      for (int l = 0; l < nsb; ++l) {
        const uint32_t w = __ldg(lst + l);
        const int Jb = w & 0xffff;
        const int rs = (w >> 16) & 0x7fff;
        const bool neg = (w >> 31) != 0;
#pragma unroll
        for (int kk = 0; kk < KC; ++kk)
          if (kk < kc) a += negate_if<T>(vsl[kk * n2 + rs], neg) * rows[kk * nb + Jb];
      }
      acc[j] = a;
    }
  }
#pragma unroll
  for (int j = 0; j < JPT; ++j) {
    const int64_t col = threadIdx.x + (int64_t)j * kDsThreads;
    if (col < nb) sigma[Ia * nb + col] = acc[j];
  }
}

__device__ __forceinline__ void cp_async4_zfill(void* dst, const void* src, bool valid) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(sa), "l"(src), "r"(valid ? 4 : 0) : "memory");
}

__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(src) : "memory");
}

// FP32 sigma terms that couple the two spins, as one contraction per alpha
// string (the Knowles-Handy factorisation restricted to the string's own
// singles).  For alpha string Ia with singles k = (Ja_k, pq_k, s_k), and
// k = own (Ja = Ia):
//   E[r][Jb] = sum_k Vp[k][r] C[Ja_k, Jb]                 (register-tiled FMAs)
//     Vp[k][r]      = s_k V(pq_k, rs_r)         pair rows
//     Vp[k][mr + p] = s_k V(p p | pq_k)         W rows
//     Vp[k][mr + n] = s_k A(Ia, Ja_k)           string-only singles row
//     Vp[own][r]    = W_a[rs_r](Ia)             (beta singles' W part)
//   sigma[Ia, Ib] += sum_{l: beta single of Ib} s_l E[r_l][Jb_l]       opposite spin + beta W part
//                  + sum_{p in Ib} E[mr + p][Ib] + E[mr + n][Ib]       alpha singles
// so one kernel applies the opposite-spin doubles and every single
// excitation except the beta singles' string-only part.  E is formed for
// every (r, Jb), n^2 / (k_b (n - k_b)) times the opposite-spin element count
// (3.7x at CAS(14,14)), as FMAs with three shared-memory wavefronts per 32 of
// them, where the element-wise walk spends two shared-memory gathers per
// element.  J_b runs in chunks of kMmCols: the chunk's C rows and walk lists
// are copied (cp.async) while the previous chunk is formed; every warp forms
// 16 rows of E; then each thread walks its beta strings' entries of the
// chunk in the lists' fixed order, so the sums are reproducible.
// sigma[Ia, :] += diag * C[Ia, :] + the terms; JPT beta strings per thread.
template <int JPT>
__global__ void __launch_bounds__(kMmMaxWarps * 32)
    k_ds_opposite_mm(int na, int nb, int nsa, int mr, int mrp, int off_words, int seg_max,
                     const int32_t* __restrict__ a_sJ, const int32_t* __restrict__ a_svo,
                     const float* __restrict__ a_sA, const float* __restrict__ a_W, const int32_t* __restrict__ rs_of,
                     const uint32_t* __restrict__ lists, const int32_t* __restrict__ seg,
                     const float* __restrict__ V2, int n, const double* __restrict__ D, const float* __restrict__ C,
                     float* __restrict__ sigma) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int K = nsa + 1;
  float* Vp = (float*)smem_raw;                          // [K][mrp]
  float* G = Vp + (size_t)K * mrp;                       // [2][K][kMmCols]
  float* E = G + (size_t)2 * K * kMmCols;                // [mrp][kMmEStride]
  uint32_t* L = (uint32_t*)(E + (size_t)mrp * kMmEStride);  // [2][seg_max]
  int32_t* Jrow = (int32_t*)(L + (size_t)2 * seg_max);   // [K]
  const int64_t Ia = blockIdx.x;
  const int tid = threadIdx.x, nthr = blockDim.x, lane = tid & 31, warp = tid >> 5;
  const int ty = lane >> 3, tx = lane & 7;
  for (int i = tid; i < K * mrp; i += nthr) {
    const int k = i / mrp, r = i - k * mrp;
    float v = 0.f;
    if (k < nsa) {
      const int32_t vo = __ldg(a_svo + Ia * nsa + k);
      const int pq = (vo & 0xff) + n * ((vo >> 8) & 0xff);
      v = (r == mr + n) ? __ldg(a_sA + Ia * nsa + k) : __ldg(V2 + (size_t)pq * mrp + r);
      v = negate_if<float>(v, (vo >> 16) != 0);
    } else if (r < mr) {
      v = __ldg(a_W + (int64_t)__ldg(rs_of + r) * na + Ia);
    }
    Vp[i] = v;
  }
  for (int k = tid; k < K; k += nthr) Jrow[k] = k < nsa ? __ldg(a_sJ + Ia * nsa + k) : (int32_t)Ia;
  __syncthreads();
  auto stage = [&](int chunk, int buf) {
    const int j0 = chunk * kMmCols;
    float* g = G + (size_t)buf * K * kMmCols;
    for (int i = tid; i < K * kMmCols; i += nthr) {
      const int k = i / kMmCols, j = i - k * kMmCols;
      const bool ok = j0 + j < nb;
      cp_async4_zfill(g + i, C + (int64_t)Jrow[k] * nb + (ok ? j0 + j : 0), ok);
    }
    const int w0 = __ldg(seg + chunk), nv = (__ldg(seg + chunk + 1) - w0) >> 2;
    uint32_t* l = L + (size_t)buf * seg_max;
    for (int i = tid; i < nv; i += nthr) cp_async16(l + 4 * i, lists + w0 + 4 * i);
    asm volatile("cp.async.commit_group;\n" ::: "memory");
  };
  float acc[JPT];
#pragma unroll
  for (int j = 0; j < JPT; ++j) {
    const int Ib = tid + j * nthr;
    acc[j] = Ib < nb ? sigma[Ia * nb + Ib] + (float)D[Ia * nb + Ib] * C[Ia * nb + Ib] : 0.f;
  }
  const int nchunk = (nb + kMmCols - 1) / kMmCols;
  stage(0, 0);
  for (int c = 0; c < nchunk; ++c) {
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    __syncthreads();  // chunk c staged by every thread; E and buffer (c + 1) & 1 free
    if (c + 1 < nchunk) stage(c + 1, (c + 1) & 1);
    {
      const float* vrow = Vp + warp * 16 + ty * 4;
      const float* grow = G + (size_t)(c & 1) * K * kMmCols + tx * 4;
      float a4[4][8];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int jj = 0; jj < 8; ++jj) a4[i][jj] = 0.f;
#pragma unroll 4
      for (int k = 0; k < K; ++k) {
        const float4 va = *(const float4*)(vrow + (size_t)k * mrp);
        const float4 b0 = *(const float4*)(grow + k * kMmCols);
        const float4 b1 = *(const float4*)(grow + k * kMmCols + 32);
        const float av[4] = {va.x, va.y, va.z, va.w};
        const float bv[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int jj = 0; jj < 8; ++jj) a4[i][jj] = fmaf(av[i], bv[jj], a4[i][jj]);
      }
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        float* e = E + (size_t)(warp * 16 + ty * 4 + i) * kMmEStride + tx * 4;
        *(float4*)e = make_float4(a4[i][0], a4[i][1], a4[i][2], a4[i][3]);
        *(float4*)(e + 32) = make_float4(a4[i][4], a4[i][5], a4[i][6], a4[i][7]);
      }
    }
    __syncthreads();
    const uint32_t* l = L + (size_t)(c & 1) * seg_max;
    const uint16_t* off = (const uint16_t*)l;
    const uint32_t* ent = l + off_words;
#pragma unroll
    for (int j = 0; j < JPT; ++j) {
      const int Ib = tid + j * nthr;
      if (Ib < nb) {
        const int e1 = off[Ib + 1];
        float a = acc[j];
        for (int e = off[Ib]; e < e1; ++e) {
          const uint32_t w = ent[e];
          a += negate_if<float>(E[((w >> 8) & 0x7fff) * kMmEStride + (w & 0xff)], (w >> 31) != 0);
        }
        acc[j] = a;
      }
    }
  }
#pragma unroll
  for (int j = 0; j < JPT; ++j) {
    const int Ib = tid + j * nthr;
    if (Ib < nb) sigma[Ia * nb + Ib] = acc[j];
  }
}

// out (nc x nr) = in^T (in: nr x nc); add != 0: out += in^T
template <typename T>
__global__ void k_transpose(const T* __restrict__ in, T* __restrict__ out, int64_t nr, int64_t nc, int add) {
  __shared__ T tile[32][33];
  const int64_t r0 = (int64_t)blockIdx.y * 32, c0 = (int64_t)blockIdx.x * 32;
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    const int64_t r = r0 + i, cc = c0 + threadIdx.x;
    if (r < nr && cc < nc) tile[i][threadIdx.x] = in[r * nc + cc];
  }
  __syncthreads();
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    const int64_t cc = c0 + i, r = r0 + threadIdx.x;
    if (cc < nc && r < nr) {
      if (add)
        out[cc * nr + r] += tile[threadIdx.x][i];
      else
        out[cc * nr + r] = tile[threadIdx.x][i];
    }
  }
}

template <typename T>
static void transpose(Context* c, const T* in, T* out, int64_t nr, int64_t nc, bool add) {
  dim3 g((unsigned)((nc + 31) / 32), (unsigned)((nr + 31) / 32));
  k_transpose<T><<<g, dim3(32, 8), 0, c->stream>>>(in, out, nr, nc, add ? 1 : 0);
  QDKGB_CHECK_LAUNCH();
}

void transpose_f64(Context* c, const double* in, double* out, int64_t nr, int64_t nc) {
  transpose<double>(c, in, out, nr, nc, false);
}

template <typename T>
static void direct_sigma_t(Context* c, const T* x, T* y) {
  DirectSigma* d = c->direct;
  const SpinTables& A = d->a;
  const SpinTables& B = d->same ? d->a : d->b;
  const int64_t na = A.nstr, nb = B.nstr, N = na * nb;
  const bool f64 = sizeof(T) == 8;
  // the contraction form applies every single excitation but the beta
  // singles' string-only part, so the same-spin kernels then take the
  // doubles (alpha) and the doubles plus string-only singles (beta)
  const bool mm = !f64 && d->mm;
  auto P = [&](const DeviceBuffer& b64, const DeviceBuffer& b32) { return (const T*)(f64 ? b64.ptr : b32.ptr); };
  T* ct = (T*)dev_alloc(c, f64 ? d->ct64 : d->ct32, N * sizeof(T));
  T* tmp = (T*)dev_alloc(c, f64 ? d->tmp64 : d->tmp32, N * sizeof(T));
  // alpha-alpha into y
  k_ds_same_spin<T><<<(unsigned)na, kDsThreads, 0, c->stream>>>(
      na, nb, mm ? 0 : A.ns, A.nd, (const int32_t*)A.sJ.ptr, (const int32_t*)A.svo.ptr, P(A.sA64, A.sA32),
      (const int32_t*)A.dJ.ptr, P(A.dval64, A.dval32), P(B.W64, B.W32), d->n, x, y);
  QDKGB_CHECK_LAUNCH();
  // beta-beta on C^T, added back transposed
  transpose<T>(c, x, ct, na, nb, false);
  k_ds_same_spin<T><<<(unsigned)nb, kDsThreads, 0, c->stream>>>(
      nb, na, B.ns, B.nd, (const int32_t*)B.sJ.ptr, (const int32_t*)B.svo.ptr, P(B.sA64, B.sA32),
      (const int32_t*)B.dJ.ptr, P(B.dval64, B.dval32), mm ? nullptr : P(A.W64, A.W32), d->n, ct, tmp);
  QDKGB_CHECK_LAUNCH();
  transpose<T>(c, tmp, y, nb, na, true);
  // opposite spin + diagonal (+ the singles, contraction form)
  if constexpr (sizeof(T) == 4) {
    if (mm) {
      auto go = [&](auto kern) {
        kern<<<(unsigned)na, d->mm_threads, d->mm_smem, c->stream>>>(
            (int)na, (int)nb, A.ns, d->mr, d->mrp, d->off_words, d->seg_max, (const int32_t*)A.sJ.ptr,
            (const int32_t*)A.svo.ptr, (const float*)A.sA32.ptr, (const float*)A.W32.ptr, (const int32_t*)d->rs_of.ptr,
            (const uint32_t*)d->lists.ptr, (const int32_t*)d->seg.ptr, (const float*)d->V2mm.ptr, d->n,
            (const double*)c->H.diag.ptr, (const float*)x, (float*)y);
      };
      switch (d->mm_jpt) {
        case 1: go(k_ds_opposite_mm<1>); break;
        case 2: go(k_ds_opposite_mm<2>); break;
        case 4: go(k_ds_opposite_mm<4>); break;
        case 8: go(k_ds_opposite_mm<8>); break;
        case 12: go(k_ds_opposite_mm<12>); break;
        default: go(k_ds_opposite_mm<16>); break;
      }
      QDKGB_CHECK_LAUNCH();
      return;
    }
  }
  const T* Vt = f64 ? (const T*)c->V.ptr : (const T*)d->V32.ptr;
  constexpr int KC = f64 ? 4 : 8;
  const size_t smem = ((size_t)KC * nb + (size_t)KC * d->n * d->n) * sizeof(T);
  k_ds_opposite<T, KC><<<(unsigned)na, kDsThreads, smem, c->stream>>>(
      na, nb, A.ns, B.ns, (const int32_t*)A.sJ.ptr, (const int32_t*)A.svo.ptr, (const uint32_t*)B.packed.ptr, Vt,
      d->n, (const double*)c->H.diag.ptr, x, y);
  QDKGB_CHECK_LAUNCH();
}

void direct_sigma_fp64(Context* c, const double* x, double* y) { direct_sigma_t<double>(c, x, y); }
void direct_sigma_fp32(Context* c, const float* x, float* y) { direct_sigma_t<float>(c, x, y); }

__global__ void k_diag_product(Integrals I, int64_t na, int64_t nb, const uint64_t* __restrict__ sa,
                               const uint64_t* __restrict__ sb, double* __restrict__ D) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < na * nb; r += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t a = sa[r / nb];
    D[r] = a ? me_diag(I, a, sb[r % nb]) : 0.;
  }
}

// Tables of the contraction form (k_ds_opposite_mm); leaves d->mm false
// where they do not apply.
static void build_mm_tables(Context* c, DirectSigma* d) {
  d->mm = false;
  const char* env = std::getenv("QDKGB_DIRECT_MM");
  if (env && env[0] == '0') return;
  const SpinTables& A = d->a;
  const SpinTables& B = d->same ? d->a : d->b;
  const int n = d->n, n2 = n * n;
  const int64_t nb = B.nstr;
  if (A.ns <= 0 || B.ns <= 0 || B.h_packed.size() != (size_t)nb * B.ns) return;
  const int mr = n * (n - 1), mrows = mr + n + 1, mrp = (mrows + 15) / 16 * 16;
  const int warps = mrp / 16;
  if (warps > kMmMaxWarps || mrows >= (1 << 15)) return;
  const int threads = warps * 32;
  int jpt = (int)((nb + threads - 1) / threads);
  for (int cand : {1, 2, 4, 8, 12, 16})
    if (jpt <= cand) {
      jpt = cand;
      break;
    }
  if ((int64_t)jpt * threads < nb) return;
  // pair index of each (v, o), v != o
  std::vector<int32_t> rmap(n2, -1), rs_of(mr);
  for (int rs = 0, r = 0; rs < n2; ++rs)
    if (rs % n != rs / n) {
      rmap[rs] = r;
      rs_of[r++] = rs;
    }
  // per chunk: offsets (uint16) and entries of every beta string
  const int nchunk = (int)((nb + kMmCols - 1) / kMmCols);
  const int off_words = (int)(((nb + 1) + 1) / 2 + 3) / 4 * 4;
  std::vector<std::vector<std::pair<uint32_t, uint32_t>>> per(nb);  // (sort key, entry) by string
  for (int64_t ib = 0; ib < nb; ++ib) {
    auto& v = per[ib];
    for (int l = 0; l < B.ns; ++l) {
      const uint32_t w = B.h_packed[(size_t)ib * B.ns + l];
      const uint32_t Jb = w & 0xffff, r = (uint32_t)rmap[(w >> 16) & 0x7fff];
      v.push_back({(Jb << 16) | r, Jb | (r << 16) | (w & 0x80000000u)});
    }
    const uint64_t bits = c->dets.h_ubeta[ib];
    for (int p = 0; p < n; ++p)
      if ((bits >> p) & 1) v.push_back({((uint32_t)ib << 16) | (uint32_t)(mr + p), (uint32_t)ib | ((uint32_t)(mr + p) << 16)});
    v.push_back({((uint32_t)ib << 16) | (uint32_t)(mr + n), (uint32_t)ib | ((uint32_t)(mr + n) << 16)});
    std::sort(v.begin(), v.end());
  }
  std::vector<uint32_t> lists;
  std::vector<int32_t> seg(nchunk + 1);
  std::vector<size_t> cur(nb, 0);
  int seg_max = 0;
  for (int ch = 0; ch < nchunk; ++ch) {
    const uint32_t j0 = (uint32_t)ch * kMmCols, j1 = j0 + kMmCols;
    seg[ch] = (int32_t)lists.size();
    std::vector<uint16_t> off(nb + 1);
    std::vector<uint32_t> ent;
    for (int64_t ib = 0; ib < nb; ++ib) {
      off[ib] = (uint16_t)ent.size();
      auto& v = per[ib];
      while (cur[ib] < v.size() && (v[cur[ib]].second & 0xffff) < j1) {
        const uint32_t w = v[cur[ib]++].second;
        const uint32_t jl = (w & 0xffff) - j0, r = (w >> 16) & 0x7fff;
        ent.push_back(jl | (r << 8) | (w & 0x80000000u));
      }
      if (ent.size() > 65535) return;
    }
    off[nb] = (uint16_t)ent.size();
    std::vector<uint32_t> words(off_words, 0);
    std::memcpy(words.data(), off.data(), off.size() * 2);
    lists.insert(lists.end(), words.begin(), words.end());
    lists.insert(lists.end(), ent.begin(), ent.end());
    while (lists.size() % 4) lists.push_back(0);
    seg_max = std::max(seg_max, (int)(lists.size() - seg[ch]));
  }
  seg[nchunk] = (int32_t)lists.size();
  if (lists.size() >= (size_t)INT32_MAX) return;
  const int K = A.ns + 1;
  const size_t smem = ((size_t)K * mrp + (size_t)2 * K * kMmCols + (size_t)mrp * kMmEStride) * 4 +
                      (size_t)2 * seg_max * 4 + (size_t)K * 4;
  if (smem > 220 * 1024) return;
  // V2mm[pq][r]
  std::vector<float> v2((size_t)n2 * mrp, 0.f);
  const std::vector<double>& V = c->h_V;
  for (int pq = 0; pq < n2; ++pq) {
    for (int r = 0; r < mr; ++r) v2[(size_t)pq * mrp + r] = (float)V[pq + (size_t)n2 * rs_of[r]];
    for (int p = 0; p < n; ++p) v2[(size_t)pq * mrp + mr + p] = (float)V[p + (size_t)n * p + (size_t)n2 * pq];
  }
  auto up = [&](DeviceBuffer& b, const void* src, size_t bytes) {
    void* ptr = dev_alloc(c, b, bytes + 16);
    QDKGB_CUDA(cudaMemcpyAsync(ptr, src, bytes, cudaMemcpyHostToDevice, c->stream));
  };
  up(d->V2mm, v2.data(), v2.size() * 4);
  up(d->rs_of, rs_of.data(), rs_of.size() * 4);
  up(d->lists, lists.data(), lists.size() * 4);
  up(d->seg, seg.data(), seg.size() * 4);
  for (const void* f : {(const void*)k_ds_opposite_mm<1>, (const void*)k_ds_opposite_mm<2>,
                        (const void*)k_ds_opposite_mm<4>, (const void*)k_ds_opposite_mm<8>,
                        (const void*)k_ds_opposite_mm<12>, (const void*)k_ds_opposite_mm<16>})
    set_max_dynamic_smem(f, 220 * 1024);
  d->mr = mr;
  d->mrp = mrp;
  d->mm_threads = threads;
  d->mm_jpt = jpt;
  d->seg_max = seg_max;
  d->off_words = off_words;
  d->mm_smem = smem;
  QDKGB_CUDA(cudaStreamSynchronize(c->stream));
  d->mm = true;
}

void build_direct_sigma(Context* c) {
  NvtxRange nvtx_range("qdkgb.build_direct_sigma");
  if (!c->have_ints) throw Error(QDKGB_ERR_STATE, "integrals not set");
  if (!c->have_dets) throw Error(QDKGB_ERR_STATE, "determinants not set");
  DetSpace& S = c->dets;
  for (int64_t g = 0; g < S.ngroups; ++g)
    if (S.h_gstart[g + 1] - S.h_gstart[g] != S.nbeta)
      throw Error(QDKGB_ERR_UNSUPPORTED, "direct sigma needs a complete (CAS) determinant space");
  if (S.nbeta > kDsMaxCols || S.ngroups > kDsMaxCols)
    throw Error(QDKGB_ERR_UNSUPPORTED, "direct sigma supports up to 4096 strings per spin");
  if (c->norb > 20) throw Error(QDKGB_ERR_UNSUPPORTED, "direct sigma supports up to 20 orbitals");
  if (S.h_galpha.empty() || S.h_galpha[0] == 0 || S.h_ubeta.empty() || S.h_ubeta[0] == 0)
    throw Error(QDKGB_ERR_UNSUPPORTED, "direct sigma needs at least one electron of each spin");
  free_direct(c);
  c->direct = new DirectSigma();
  DirectSigma* d = c->direct;
  d->n = c->norb;
  build_spin_tables(c, S.h_galpha, d->a);
  d->same = (S.h_galpha == S.h_ubeta);
  if (!d->same) build_spin_tables(c, S.h_ubeta, d->b);
  const size_t n4 = (size_t)d->n * d->n * d->n * d->n;
  std::vector<float> v32(n4);
  for (size_t i = 0; i < n4; ++i) v32[i] = (float)c->h_V[i];
  float* V32 = dev_array<float>(c, d->V32, n4);
  QDKGB_CUDA(cudaMemcpyAsync(V32, v32.data(), n4 * 4, cudaMemcpyHostToDevice, c->stream));
  // diagonal and operator state
  Hcsr& H = c->H;
  H.valid = false;
  const int64_t N = S.ndets;
  double* D = dev_array<double>(c, H.diag, N);
  const unsigned blocks = (unsigned)std::min<int64_t>((N + 255) / 256, (int64_t)c->sm_count * 16);
  k_diag_product<<<blocks, 256, 0, c->stream>>>(integrals_view(c), S.ngroups, S.nbeta,
                                               (const uint64_t*)S.galpha.ptr, (const uint64_t*)S.ubeta.ptr, D);
  QDKGB_CHECK_LAUNCH();
  set_max_dynamic_smem((const void*)k_ds_opposite<double, 4>, 200 * 1024);
  set_max_dynamic_smem((const void*)k_ds_opposite<float, 8>, 200 * 1024);
  // contraction form of the FP32 sigma, where its tables and shared memory
  // fit (QDKGB_DIRECT_MM=0 keeps the element-wise walk)
  build_mm_tables(c, d);
  d->a.h_packed.clear();
  d->b.h_packed.clear();
  QDKGB_CUDA(cudaStreamSynchronize(c->stream));
  H.n = N;
  H.nnz = 0;
  H.valid = true;
  c->op_direct = true;
}

}  // namespace qdkgb
