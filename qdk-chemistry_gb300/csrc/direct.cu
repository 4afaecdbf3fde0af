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
#include "tcgen05.cuh"

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
// kMmCols; E rows 16 per warp, each thread 4 rows x 8 columns; E rows
// kMmEStride floats apart in shared memory (16-byte rows that start four
// banks apart).
constexpr int kMmCols = 64;
constexpr int kMmEStride = kMmCols + 4;

// Instance strides of the contraction kernels (grid axis y = instance; a
// single space has one instance and zero strides): the value tables sA, W
// and V2mm, and the vectors (diagonal, C, sigma); act, when given, skips the
// instances whose entry is zero.
struct DsInst {
  const int* act;
  int64_t sA, W, V2, vec;
};
// the same for the dense same-spin products (grid axis z = instance)
struct GmInst {
  const int* act;
  int64_t A1, B1, A2, B2, out;
};
constexpr int kMmMaxWarps = 16;

// One spin's string tables.  Structure (built once per determinant space):
// sJ / svo the singles (target string; v | o << 8 | neg << 16), dJ / dvo the
// doubles (target; v1 | o1 << 5 | v2 << 10 | o2 << 15 | neg << 20), packed
// the singles as Jb | rs << 16 | neg << 31, str the strings.  Values
// (recomputed from the integrals by every build, k_ds_values): sA the
// singles' string-only part, dval the doubles, W over THIS spin's strings.
struct SpinTables {
  int64_t nstr = 0;
  int ns = 0, nd = 0;
  DeviceBuffer sJ, svo, dJ, dvo, packed, str;
  DeviceBuffer sA64, sA32, dval64, dval32, W64, W32;
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
  // lists (uint16): per chunk of kMmCols beta strings, the (nb + 1) offsets
  // of each beta string's entries (padded to 16 bytes) then the entries
  // (r kMmEStride + jl) | neg << 15 (jl = J_b - chunk start: the entry's place
  // in E), each string's sorted by (J_b, r); seg[c] = the chunk's first
  // element (16-byte aligned); off_u16 = the padded offset count
  bool mm = false;
  int mr = 0, mrp = 0, mm_threads = 0, mm_jpt = 0, seg_max = 0, off_u16 = 0;
  bool mm_vec = false;  // C rows 16-byte aligned (nb % 4 == 0): 16-byte staging copies
  size_t mm_smem = 0;
  DeviceBuffer V2mm, rs_of, lists, seg;
  // same-spin string-only parts as dense FP32 matrices for the contraction
  // form: Haa[Ia][Ja] the alpha doubles, HbbT[Jb][Ib] the beta doubles and
  // the beta singles' string-only part; dense_state -1 until the first FP32
  // sigma times the dense products against the element-wise same-spin
  // kernels (0 element-wise, 1 dense)
  int dense_state = -1;
  double dense_ms[2] = {0., 0.};
  char mm_env = 0, dense_env = 0;  // QDKGB_DIRECT_MM / QDKGB_DIRECT_DENSE when built
  bool tc = false;                 // tensor cores (k_tc_gemm2b, k_ds_opposite_tc; QDKGB_DIRECT_TC=0: FMA pipe)
  // the contraction's E on the tensor cores (k_ds_opposite_tc): K padded to
  // kpad, its shared memory, beta strings per thread
  // otc_state: -1 until the first FP32 sigma times the FMA and tensor-core
  // contractions (0 FMA kept, 1 tensor cores kept); otc_ms their times
  bool otc = false;
  int kpad = 0, otc_jpt = 0, otc_state = -1;
  double otc_ms[2] = {0., 0.};
  size_t otc_smem = 0;
  DeviceBuffer Haa, HbbT;
  // the dense products' operands split into TF32 parts in the blocked layout
  // (k_tc_split): H_aa (A form), H_bb^T (B form) per build, x in both forms
  // per sigma; nkb1 / nkb2 the K blocks of the two products
  DeviceBuffer HaaS, HbbS, XA, XB;
  int nkb1 = 0, nkb2 = 0;
  int64_t szA1 = 0, szB1 = 0, szA2 = 0, szB2 = 0;  // floats per split part
  // batched CASCI over instances of this space (direct_batch_*): per-instance
  // FP32 value tables and their dense same-spin matrices; bform -1 until the
  // first call fixes the contraction form (0 FMA pipe, 1 tensor cores)
  int bcap = 0, bform = -1;
  DeviceBuffer bsAa, bWa, bdva, bsAb, bWb, bdvb, bV2, bHaa, bHbbT, bHaaS, bHbbS, bXA, bXB;
};

void free_direct(Context* c) {
  if (!c->direct) return;
  DirectSigma* d = c->direct;
  for (SpinTables* t : {&d->a, &d->b})
    for (DeviceBuffer* b : {&t->sJ, &t->svo, &t->dJ, &t->dvo, &t->packed, &t->str, &t->sA64, &t->sA32, &t->dval64,
                            &t->dval32, &t->W64, &t->W32})
      dev_free(c, *b);
  for (DeviceBuffer* b : {&d->V32, &d->tmp64, &d->tmp32, &d->ct64, &d->ct32, &d->V2mm, &d->rs_of, &d->lists, &d->seg,
                          &d->Haa, &d->HbbT, &d->bsAa, &d->bWa, &d->bdva, &d->bsAb, &d->bWb, &d->bdvb, &d->bV2,
                          &d->bHaa, &d->bHbbT, &d->HaaS, &d->HbbS, &d->XA, &d->XB, &d->bHaaS, &d->bHbbS,
                          &d->bXA, &d->bXB})
    dev_free(c, *b);
  delete d;
  c->direct = nullptr;
}

// Structure of one spin's tables (host, once per determinant space).
static void build_spin_tables(Context* c, const std::vector<uint64_t>& strs, SpinTables& t) {
  const int n = c->norb;
  const size_t nn = (size_t)n;
  const int64_t N = (int64_t)strs.size();
  std::unordered_map<uint64_t, int32_t> rank;
  for (int64_t i = 0; i < N; ++i) rank[strs[i]] = (int32_t)i;
  const int k = hpopc(strs[0]);
  const int ns = k * (n - k), nd = (k * (k - 1) / 2) * ((n - k) * (n - k - 1) / 2);
  t.nstr = N;
  t.ns = ns;
  t.nd = nd;
  std::vector<int32_t> sJ((size_t)N * ns), svo((size_t)N * ns), dJ((size_t)N * std::max(nd, 1));
  std::vector<uint32_t> dvo((size_t)N * std::max(nd, 1)), packed((size_t)N * ns);
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
        sJ[(size_t)i * ns + m] = it->second;
        svo[(size_t)i * ns + m] = (int32_t)(s.v | (s.o << 8) | ((uint32_t)s.neg << 16));
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
            dJ[(size_t)i * nd + m] = it->second;
            dvo[(size_t)i * nd + m] = s1.v | (s1.o << 5) | (s2.v << 10) | (s2.o << 15) |
                                      ((uint32_t)(s1.neg != s2.neg) << 20);
            ++m;
          }
  }
  auto up = [&](DeviceBuffer& b, const void* src, size_t bytes) {
    void* p = dev_alloc(c, b, bytes + 16);
    QDKGB_CUDA(cudaMemcpyAsync(p, src, bytes, cudaMemcpyHostToDevice, c->stream));
  };
  up(t.sJ, sJ.data(), sJ.size() * 4);
  up(t.svo, svo.data(), svo.size() * 4);
  up(t.dJ, dJ.data(), dJ.size() * 4);
  up(t.dvo, dvo.data(), dvo.size() * 4);
  up(t.packed, packed.data(), packed.size() * 4);
  up(t.str, strs.data(), strs.size() * 8);
  QDKGB_CUDA(cudaStreamSynchronize(c->stream));
  t.h_packed = std::move(packed);
}

// Values of one spin's tables from the integrals, in the order of the
// reference's matrix elements (matrix_elements.hpp:65-230): the singles'
// string-only part A = T(v, o) + sum_{p in I} G_red(p, v, o) (ascending p),
// the doubles V(v1 o1 | v2 o2) - V(v1 o2 | v2 o1) with the sign pair's
// parity, and W[(v, o)][I] = sum_{p in I} V(p p | v o); FP64 and its FP32
// rounding.  One thread per entry.
__global__ void k_ds_values(int64_t N, int ns, int nd, int n, const uint64_t* __restrict__ strs,
                            const int32_t* __restrict__ svo, const uint32_t* __restrict__ dvo,
                            const double* __restrict__ T, const double* __restrict__ V, double* __restrict__ sA64,
                            float* __restrict__ sA32, double* __restrict__ dval64, float* __restrict__ dval32,
                            double* __restrict__ W64, float* __restrict__ W32) {
  const int64_t nn = n, ts = N * ns, td = N * nd, tw = nn * nn * N;
  auto Vat = [&](int64_t p, int64_t q, int64_t r, int64_t s) { return __ldg(V + p + nn * (q + nn * (r + nn * s))); };
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < ts + td + tw;
       t += (int64_t)gridDim.x * blockDim.x) {
    if (t < ts) {
      const uint64_t I = __ldg(strs + t / ns);
      const int32_t vo = __ldg(svo + t);
      const int v = vo & 0xff, o = (vo >> 8) & 0xff;
      double a = __ldg(T + v + nn * o);
      for (int p = 0; p < n; ++p)
        if ((I >> p) & 1) a += Vat(p, p, v, o) - Vat(p, o, v, p);
      if (sA64) sA64[t] = a;
      sA32[t] = (float)a;
    } else if (t < ts + td) {
      const int64_t u = t - ts;
      const uint32_t w = __ldg(dvo + u);
      const int v1 = w & 31, o1 = (w >> 5) & 31, v2 = (w >> 10) & 31, o2 = (w >> 15) & 31;
      const double g = Vat(v1, o1, v2, o2) - Vat(v1, o2, v2, o1);
      const double d = ((w >> 20) & 1) ? -g : g;
      if (dval64) dval64[u] = d;
      dval32[u] = (float)d;
    } else {
      const int64_t u = t - ts - td, vo = u / N;
      const uint64_t I = __ldg(strs + (u - vo * N));
      const int v = (int)(vo % nn), o = (int)(vo / nn);
      double w = 0.;
      for (int p = 0; p < n; ++p)
        if ((I >> p) & 1) w += Vat(p, p, v, o);
      if (W64) W64[u] = w;
      W32[u] = (float)w;
    }
  }
}

static void spin_values(Context* c, SpinTables& t) {
  const int64_t N = t.nstr, n = c->norb;
  dev_array<double>(c, t.sA64, (size_t)N * t.ns + 1);
  dev_array<float>(c, t.sA32, (size_t)N * t.ns + 1);
  dev_array<double>(c, t.dval64, (size_t)N * std::max(t.nd, 1));
  dev_array<float>(c, t.dval32, (size_t)N * std::max(t.nd, 1));
  dev_array<double>(c, t.W64, (size_t)(n * n * N));
  dev_array<float>(c, t.W32, (size_t)(n * n * N));
  const int64_t tot = N * t.ns + N * t.nd + n * n * N;
  const unsigned blocks = (unsigned)std::min<int64_t>((tot + 255) / 256, (int64_t)c->sm_count * 16);
  k_ds_values<<<blocks, 256, 0, c->stream>>>(N, t.ns, t.nd, (int)n, (const uint64_t*)t.str.ptr,
                                             (const int32_t*)t.svo.ptr, (const uint32_t*)t.dvo.ptr,
                                             (const double*)c->T.ptr, (const double*)c->V.ptr, (double*)t.sA64.ptr,
                                             (float*)t.sA32.ptr, (double*)t.dval64.ptr, (float*)t.dval32.ptr,
                                             (double*)t.W64.ptr, (float*)t.W32.ptr);
  QDKGB_CHECK_LAUNCH();
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
template <int JPT, bool BIG>
__global__ void __launch_bounds__(BIG ? kMmMaxWarps * 32 : 320, BIG ? 1 : 2)
    k_ds_opposite_mm(int na, int nb, int nsa, int mr, int mrp, int off_u16, int seg_max, int vec,
                     const int32_t* __restrict__ a_sJ, const int32_t* __restrict__ a_svo,
                     const float* __restrict__ a_sA, const float* __restrict__ a_W, const int32_t* __restrict__ rs_of,
                     const uint16_t* __restrict__ lists, const int32_t* __restrict__ seg,
                     const float* __restrict__ V2, int n, const double* __restrict__ D, const float* __restrict__ C,
                     float* __restrict__ sigma, DsInst bi) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  {
    const int inst = blockIdx.y;
    if (bi.act && !bi.act[inst]) return;
    a_sA += inst * bi.sA;
    a_W += inst * bi.W;
    V2 += inst * bi.V2;
    D += inst * bi.vec;
    C += inst * bi.vec;
    sigma += inst * bi.vec;
  }
  const int K = nsa + 1;
  float* Vp = (float*)smem_raw;                           // [K][mrp]
  float* G = Vp + (size_t)K * mrp;                        // [2][K][kMmCols]
  float* E = G + (size_t)2 * K * kMmCols;                 // [mrp][kMmEStride]
  uint16_t* L = (uint16_t*)(E + (size_t)mrp * kMmEStride);  // [2][seg_max]
  int32_t* Jrow = (int32_t*)(L + (size_t)2 * seg_max);    // [K]
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
    if (vec) {
      for (int i = tid; i < K * (kMmCols / 4); i += nthr) {
        const int k = i / (kMmCols / 4), j = 4 * (i - k * (kMmCols / 4));
        const bool ok = j0 + j < nb;
        const unsigned sa = (unsigned)__cvta_generic_to_shared(g + k * kMmCols + j);
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(sa),
                     "l"(C + (int64_t)Jrow[k] * nb + (ok ? j0 + j : 0)), "r"(ok ? 16 : 0)
                     : "memory");
      }
    } else {
      for (int i = tid; i < K * kMmCols; i += nthr) {
        const int k = i / kMmCols, j = i - k * kMmCols;
        const bool ok = j0 + j < nb;
        cp_async4_zfill(g + i, C + (int64_t)Jrow[k] * nb + (ok ? j0 + j : 0), ok);
      }
    }
    const int u0 = __ldg(seg + chunk), nv = (__ldg(seg + chunk + 1) - u0) >> 3;
    uint16_t* l = L + (size_t)buf * seg_max;
    for (int i = tid; i < nv; i += nthr) cp_async16(l + 8 * i, lists + u0 + 8 * i);
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
      const float* v0 = Vp + warp * 16 + ty * 4;
      const float* g0 = G + (size_t)(c & 1) * K * kMmCols + tx * 4;
      float a[4][8];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int jj = 0; jj < 8; ++jj) a[i][jj] = 0.f;
#pragma unroll 4
      for (int k = 0; k < K; ++k) {
        const float4 va = *(const float4*)(v0 + (size_t)k * mrp);
        const float4 b0 = *(const float4*)(g0 + k * kMmCols);
        const float4 b1 = *(const float4*)(g0 + k * kMmCols + 32);
        const float av[4] = {va.x, va.y, va.z, va.w};
        const float bv[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int jj = 0; jj < 8; ++jj) a[i][jj] = fmaf(av[i], bv[jj], a[i][jj]);
      }
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        float* e = E + (size_t)(warp * 16 + ty * 4 + i) * kMmEStride + tx * 4;
        *(float4*)e = make_float4(a[i][0], a[i][1], a[i][2], a[i][3]);
        *(float4*)(e + 32) = make_float4(a[i][4], a[i][5], a[i][6], a[i][7]);
      }
    }
    __syncthreads();
    const uint16_t* off = L + (size_t)(c & 1) * seg_max;
    const uint16_t* ent = off + off_u16;
#pragma unroll
    for (int j = 0; j < JPT; ++j) {
      const int Ib = tid + j * nthr;
      if (Ib < nb) {
        const int e1 = off[Ib + 1];
        float s = acc[j];
        for (int e = off[Ib]; e < e1; ++e) {
          const uint32_t w = ent[e];
          s += negate_if<float>(E[w & 0x7fff], (w >> 15) != 0);
        }
        acc[j] = s;
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

__global__ void k_ds_v32(const double* __restrict__ V, float* __restrict__ V32, int64_t n4) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n4; i += (int64_t)gridDim.x * blockDim.x)
    V32[i] = (float)V[i];
}

// V2mm[pq][r] (see DirectSigma)
__global__ void k_ds_v2mm(const double* __restrict__ V, const int32_t* __restrict__ rs_of, int n, int mr, int mrp,
                          float* __restrict__ V2) {
  const int64_t n2 = (int64_t)n * n, tot = n2 * mrp;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < tot; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t pq = i / mrp;
    const int r = (int)(i - pq * mrp);
    float v = 0.f;
    if (r < mr)
      v = (float)V[pq + n2 * rs_of[r]];
    else if (r < mr + n)
      v = (float)V[(r - mr) * (int64_t)(n + 1) + n2 * pq];
    V2[i] = v;
  }
}

// Dense same-spin matrices of the contraction form (Haa, HbbT zeroed first):
// Haa[i][dJ] = dval_a; HbbT[dJ_b][j] = dval_b; HbbT[sJ_b][j] = s A_b.
__global__ void k_ds_dense_fill(int64_t na, int nda, const int32_t* __restrict__ adJ,
                                const float* __restrict__ adval, int64_t nb, int ndb, int nsb,
                                const int32_t* __restrict__ bdJ, const float* __restrict__ bdval,
                                const int32_t* __restrict__ bsJ, const int32_t* __restrict__ bsvo,
                                const float* __restrict__ bsA, float* __restrict__ Haa, float* __restrict__ HbbT) {
  const int64_t t1 = na * nda, t2 = nb * ndb, t3 = nb * nsb;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < t1 + t2 + t3;
       t += (int64_t)gridDim.x * blockDim.x) {
    if (t < t1) {
      Haa[(t / nda) * na + adJ[t]] = adval[t];
    } else if (t < t1 + t2) {
      const int64_t u = t - t1;
      HbbT[(int64_t)bdJ[u] * nb + u / ndb] = bdval[u];
    } else {
      const int64_t u = t - t1 - t2;
      HbbT[(int64_t)bsJ[u] * nb + u / nsb] = negate_if<float>(bsA[u], (bsvo[u] >> 16) != 0);
    }
  }
}

// out (M x N) = A1 (M x K1) B1 (K1 x N) + A2 (M x K2) B2 (K2 x N), row-major
// FP32: 64 x 64 tiles, 256 threads of 4 x 4, K in steps of 16 through
// register-staged double-buffered shared memory.
constexpr int kGmT = 64, kGmK = 16;
__global__ void __launch_bounds__(256) k_ds_gemm2(int M, int N, int K1, int K2, const float* __restrict__ A1,
                                                  const float* __restrict__ B1, const float* __restrict__ A2,
                                                  const float* __restrict__ B2, float* __restrict__ out, GmInst bi) {
  {
    const int inst = blockIdx.z;
    if (bi.act && !bi.act[inst]) return;
    A1 += inst * bi.A1;
    B1 += inst * bi.B1;
    A2 += inst * bi.A2;
    B2 += inst * bi.B2;
    out += inst * bi.out;
  }
  __shared__ __align__(16) float As[2][kGmK][kGmT + 4];
  __shared__ __align__(16) float Bs[2][kGmK][kGmT];
  const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;
  const int m0 = blockIdx.y * kGmT, n0 = blockIdx.x * kGmT;
  const int am = tid >> 2, ak = (tid & 3) * 4;   // A loader: row am, k ak..ak+3
  const int bk = tid >> 4, bn = (tid & 15) * 4;  // B loader: k bk, cols bn..bn+3
  float acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
  float ra[4], rb[4];
  for (int phase = 0; phase < 2; ++phase) {
    const float* A = phase ? A2 : A1;
    const float* B = phase ? B2 : B1;
    const int K = phase ? K2 : K1;
    const int ntile = (K + kGmK - 1) / kGmK;
    auto load = [&](int t) {
      const int k0 = t * kGmK;
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int m = m0 + am, k = k0 + ak + i;
        ra[i] = (m < M && k < K) ? __ldg(A + (int64_t)m * K + k) : 0.f;
        const int kb = k0 + bk, nn = n0 + bn + i;
        rb[i] = (kb < K && nn < N) ? __ldg(B + (int64_t)kb * N + nn) : 0.f;
      }
    };
    auto store = [&](int buf) {
#pragma unroll
      for (int i = 0; i < 4; ++i) As[buf][ak + i][am] = ra[i];
      *(float4*)&Bs[buf][bk][bn] = make_float4(rb[0], rb[1], rb[2], rb[3]);
    };
    load(0);
    store(0);
    __syncthreads();
    for (int t = 0; t < ntile; ++t) {
      const int buf = t & 1;
      if (t + 1 < ntile) load(t + 1);
#pragma unroll
      for (int kk = 0; kk < kGmK; ++kk) {
        const float4 a = *(const float4*)&As[buf][kk][ty * 4];
        const float4 b = *(const float4*)&Bs[buf][kk][tx * 4];
        const float av[4] = {a.x, a.y, a.z, a.w}, bv[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
      }
      if (t + 1 < ntile) store(buf ^ 1);
      __syncthreads();
    }
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int m = m0 + ty * 4 + i;
    if (m >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int nn = n0 + tx * 4 + j;
      if (nn < N) out[(int64_t)m * N + nn] = acc[i][j];
    }
  }
}

// Tensor-core tiles (tcgen05, TF32 x 3: each FP32 operand split into a TF32
// high part and the TF32 rounding of the remainder; hi hi + hi lo + lo hi
// accumulated in FP32 in TMEM, about FP32 accuracy): 128 x 64 output tiles
// (TMEM columns 0..63, lane = row), K in blocks of 32.
constexpr int kTcM = 128, kTcN = 64, kTcBK = 32;
constexpr int kTcABytes = kTcM * kTcBK * 4, kTcBBytes = kTcN * kTcBK * 4;
constexpr uint32_t kTcSpin = 1u << 22;
__device__ unsigned int g_tc_fault;  // set by a CTA whose wait timed out (its tile is NaN)

// Operands of the dense same-spin products, split once into TF32 high and
// low parts in the tensor core's blocked K-major layout, so that a K block
// of a tile is one contiguous 16 KB (A: 128 rows x 32 K) or 8 KB (B: 64
// rows x 32 K) run per part that one bulk copy (TMA) moves into shared
// memory.  Block (rb, kb) of an operand with nkb K blocks starts at float
// (rb nkb + kb) rows 32; inside it the 16-byte chunk c holds rows
// rb rows + (c / 64) 8 + c % 8, K kb 32 + ((c / 8) % 8) 4 .. + 3.  Source
// element (r, k): S[r ld + k] (A form) or S[k ld + r] (B form, the second
// product's C H^T and the first's C read as K x N).
constexpr int kSpRowsA = 128, kSpRowsB = 64, kSpK = 32;
__global__ void k_tc_split(const float* __restrict__ S, int R, int K, int64_t ld, int bform, int rows, int nkb,
                           int64_t nblk, float* __restrict__ hi, float* __restrict__ lo, int64_t sstride,
                           int64_t dstride, const int* __restrict__ act) {
  // grid axis y = instance (source and destination strides; act skips)
  if (act && !act[blockIdx.y]) return;
  S += blockIdx.y * sstride;
  hi += blockIdx.y * dstride;
  lo += blockIdx.y * dstride;
  const int64_t per = (int64_t)rows * 8, tot = nblk * per;
  for (int64_t id = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; id < tot; id += (int64_t)gridDim.x * blockDim.x) {
    const int64_t blk = id / per;
    const int c = (int)(id - blk * per);
    const int rb = (int)(blk / nkb), kb = (int)(blk - (int64_t)rb * nkb);
    const int cm = c >> 3, r = rb * rows + (cm >> 3) * 8 + (c & 7), k0 = kb * kSpK + (cm & 7) * 4;
    float h[4], l[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int k = k0 + q;
      const float v = (r < R && k < K) ? (bform ? S[(int64_t)k * ld + r] : S[(int64_t)r * ld + k]) : 0.f;
      h[q] = tc::to_tf32(v);
      l[q] = tc::to_tf32(v - h[q]);
    }
    *(float4*)(hi + blk * rows * kSpK + (int64_t)c * 4) = make_float4(h[0], h[1], h[2], h[3]);
    *(float4*)(lo + blk * rows * kSpK + (int64_t)c * 4) = make_float4(l[0], l[1], l[2], l[3]);
  }
}

// Pre-split operands of one product pair and their instance strides.
struct GmSplit {
  const float *a1h, *a1l, *b1h, *b1l, *a2h, *a2l, *b2h, *b2l;
  int nkb1, nkb2;
  const int* act;
  int64_t sa1, sb1, sa2, sb2, sout;  // per-instance strides (floats)
};

// out (M x N) = A1 B1 + A2 B2 on tcgen05 (TF32 x 3) from pre-split operands:
// warp 0 lane 0 fills a ring of kTmStages shared-memory stages with four
// bulk copies per K block (A hi / lo 16 KB, B hi / lo 8 KB, one mbarrier
// with the byte count), warp 1 lane 0 issues the twelve MMAs per block and
// commits each stage back to its producer, warps 2-5 (one per TMEM lane
// quadrant) read the 128 x 64 FP32 tile out after the last commit.  Every
// wait is bounded; a timeout sets g_tc_fault and the tile is NaN.
constexpr int kTmStages = 2, kTmThreads = 192;
constexpr int kTmStage = 2 * kTcABytes + 2 * kTcBBytes;
__global__ void __launch_bounds__(kTmThreads) k_tc_gemm2b(int M, int N, GmSplit g, float* __restrict__ out) {
  extern __shared__ __align__(128) unsigned char tm_smem[];
  __shared__ __align__(8) uint64_t full[kTmStages], empty[kTmStages], done;
  __shared__ uint32_t tslot;
  __shared__ int fail;
  const int inst = blockIdx.z;
  if (g.act && !g.act[inst]) return;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int rb = blockIdx.y, nbk = blockIdx.x;
  if (warp == 0) tc::tmem_alloc(&tslot, kTcN);
  if (tid == 0) {
    for (int s = 0; s < kTmStages; ++s) {
      tc::mbar_init(&full[s], 1);
      tc::mbar_init(&empty[s], 1);
    }
    tc::mbar_init(&done, 1);
    tc::mbar_init_fence();
    fail = 0;
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = tslot;
  const int nblk = g.nkb1 + g.nkb2;
  if (warp == 0 && lane == 0) {
    // producer
    for (int b = 0; b < nblk; ++b) {
      const int s = b % kTmStages;
      if (b >= kTmStages && !tc::mbar_wait(&empty[s], (uint32_t)((b / kTmStages - 1) & 1), kTcSpin)) {
        fail = 1;
        break;
      }
      const bool p2 = b >= g.nkb1;
      const int kb = p2 ? b - g.nkb1 : b, nkb = p2 ? g.nkb2 : g.nkb1;
      const int64_t ao = (int64_t)inst * (p2 ? g.sa2 : g.sa1) + ((int64_t)rb * nkb + kb) * (kSpRowsA * kSpK);
      const int64_t bo = (int64_t)inst * (p2 ? g.sb2 : g.sb1) + ((int64_t)nbk * nkb + kb) * (kSpRowsB * kSpK);
      unsigned char* st = tm_smem + s * kTmStage;
      tc::mbar_expect_tx(&full[s], (uint32_t)kTmStage);
      tc::bulk_g2s(st, (p2 ? g.a2h : g.a1h) + ao, kTcABytes, &full[s]);
      tc::bulk_g2s(st + kTcABytes, (p2 ? g.a2l : g.a1l) + ao, kTcABytes, &full[s]);
      tc::bulk_g2s(st + 2 * kTcABytes, (p2 ? g.b2h : g.b1h) + bo, kTcBBytes, &full[s]);
      tc::bulk_g2s(st + 2 * kTcABytes + kTcBBytes, (p2 ? g.b2l : g.b1l) + bo, kTcBBytes, &full[s]);
    }
  } else if (warp == 1 && lane == 0) {
    // MMA issue
    constexpr uint32_t idesc = tc::idesc_tf32(kTcM, kTcN);
    constexpr uint32_t sbo = (kTcBK / 4) * 128;
    bool ok = true;
    for (int b = 0; b < nblk; ++b) {
      const int s = b % kTmStages;
      if (!tc::mbar_wait(&full[s], (uint32_t)((b / kTmStages) & 1), kTcSpin)) {
        ok = false;
        break;
      }
      tc::fence_after();
      unsigned char* st = tm_smem + s * kTmStage;
      const uint32_t ah = tc::smem_addr(st), al = ah + kTcABytes, bh = ah + 2 * kTcABytes, bl = bh + kTcBBytes;
#pragma unroll
      for (int ks = 0; ks < kTcBK / 8; ++ks) {
        const uint32_t ko = ks * 256;
        tc::mma_tf32(tmem, tc::desc(ah + ko, 128, sbo), tc::desc(bh + ko, 128, sbo), idesc, (b | ks) ? 1u : 0u);
        tc::mma_tf32(tmem, tc::desc(ah + ko, 128, sbo), tc::desc(bl + ko, 128, sbo), idesc, 1u);
        tc::mma_tf32(tmem, tc::desc(al + ko, 128, sbo), tc::desc(bh + ko, 128, sbo), idesc, 1u);
      }
      tc::commit(&empty[s]);
    }
    if (!ok) fail = 1;
    tc::commit(&done);  // completes when every MMA issued above has
  } else if (warp >= 2) {
    // epilogue: warp w reads TMEM lanes 32 (w % 4) ..
    const int q = warp & 3;
    const bool ok = __all_sync(0xffffffffu, tc::mbar_wait(&done, 0u, kTcSpin) && !fail);
    tc::fence_after();
    const int row = rb * kTcM + q * 32 + lane;
    float* o = out + (int64_t)inst * g.sout;
#pragma unroll 1
    for (int cb = 0; cb < kTcN; cb += 16) {
      float v[16];
      if (ok) {
        tc::tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)cb, v);
      } else {
#pragma unroll
        for (int j = 0; j < 16; ++j) v[j] = __int_as_float(0x7fc00000);
      }
      if (row < M)
#pragma unroll
        for (int j = 0; j < 16; ++j)
          if (nbk * kTcN + cb + j < N) o[(int64_t)row * N + nbk * kTcN + cb + j] = v[j];
    }
    if (!ok && lane == 0) atomicOr(&g_tc_fault, 1u);
  }
  tc::fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_free(tmem, kTcN);
}

// K blocks and split-part sizes (floats) of the dense products' operands
static void tm_sizes(DirectSigma* d, int64_t na, int64_t nb) {
  d->nkb1 = (int)((na + kSpK - 1) / kSpK);
  d->nkb2 = (int)((nb + kSpK - 1) / kSpK);
  const int64_t nrb = (na + kSpRowsA - 1) / kSpRowsA, nnb = (nb + kSpRowsB - 1) / kSpRowsB;
  d->szA1 = nrb * d->nkb1 * kSpRowsA * kSpK;  // H_aa, A form
  d->szB1 = nnb * d->nkb1 * kSpRowsB * kSpK;  // x as K x N, B form
  d->szA2 = nrb * d->nkb2 * kSpRowsA * kSpK;  // x, A form
  d->szB2 = nnb * d->nkb2 * kSpRowsB * kSpK;  // H_bb^T as K x N, B form
}
// split of B instances (hi at dst, lo at dst + part; instance strides)
static void tm_split(Context* c, const float* S, int R, int K, int64_t ld, int bform, int nkb, float* dst,
                     int64_t part, int B, int64_t sstride, int64_t dstride, const int* act) {
  const int rows = bform ? kSpRowsB : kSpRowsA;
  const int64_t nblk = (int64_t)((R + rows - 1) / rows) * nkb, tot = nblk * rows * 8;
  const unsigned bx = (unsigned)std::max<int64_t>(1, std::min<int64_t>((tot + 255) / 256, (int64_t)c->sm_count * 8));
  k_tc_split<<<dim3(bx, (unsigned)B), 256, 0, c->stream>>>(S, R, K, ld, bform, rows, nkb, nblk, dst, dst + part,
                                                          sstride, dstride, act);
  QDKGB_CHECK_LAUNCH();
}
// y = H_aa x + x H_bb^T for B instances from the pre-split matrices (hs:
// H_aa parts, bs: H_bb^T parts, instance strides of the matrices' parts)
static void tm_products(Context* c, DirectSigma* d, int64_t na, int64_t nb, int B, const int* act,
                        const float* haa, const float* hbb, int64_t mstride_a, int64_t mstride_b, float* xa,
                        float* xb, const float* x, float* y) {
  const int64_t N = na * nb;
  tm_split(c, x, (int)na, (int)nb, nb, 0, d->nkb2, xa, d->szA2, B, N, 2 * d->szA2, act);  // x as A2
  tm_split(c, x, (int)nb, (int)na, nb, 1, d->nkb1, xb, d->szB1, B, N, 2 * d->szB1, act);  // x as B1
  GmSplit g{haa, haa + d->szA1, xb, xb + d->szB1, xa, xa + d->szA2, hbb, hbb + d->szB2, d->nkb1, d->nkb2,
            act, mstride_a, 2 * d->szB1, 2 * d->szA2, mstride_b, N};
  dim3 grid((unsigned)((nb + kTcN - 1) / kTcN), (unsigned)((na + kTcM - 1) / kTcM), (unsigned)B);
  k_tc_gemm2b<<<grid, kTmThreads, kTmStages * kTmStage, c->stream>>>((int)na, (int)nb, g, y);
  QDKGB_CHECK_LAUNCH();
}

// The contraction form with E formed on the tensor cores (tcgen05, TF32 x 3;
// the same terms and walk as k_ds_opposite_mm).  Per alpha string: the A
// operand Vp^T (rows r, K = the singles and the own row, zero-padded to kpad)
// is split once into TF32 high and low parts in the canonical K-major layout,
// two M tiles of 128 rows (the second holds the rows past 128; its MMA reads
// on into the following shared memory for the lanes that are never read).
// Per chunk of 64 beta strings: the C rows are copied in (cp.async), split
// into the B operand, one thread issues the 2 tiles x kpad / 8 steps x 3
// products into TMEM (128 columns: tile t at column 64 t) and commits to an
// mbarrier; the eight warps read E out of TMEM (warp w: lanes 32 (w % 4)..,
// tile w / 4) into shared memory and walk it as the FMA kernel does.
constexpr int kOtThreads = 512;

template <int JPT>
__global__ void __launch_bounds__(kOtThreads + 32, 1)
    k_ds_opposite_tc(int na, int nb, int nsa, int mr, int mrows, int kpad, int off_u16, int seg_max, int vec,
                     const int32_t* __restrict__ a_sJ, const int32_t* __restrict__ a_svo,
                     const float* __restrict__ a_sA, const float* __restrict__ a_W, const int32_t* __restrict__ rs_of,
                     const uint16_t* __restrict__ lists, const int32_t* __restrict__ seg,
                     const float* __restrict__ V2, int mrp, int n, const double* __restrict__ D,
                     const float* __restrict__ C, float* __restrict__ sigma, DsInst bi) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  {
    const int inst = blockIdx.y;
    if (bi.act && !bi.act[inst]) return;  // the whole CTA, before any TMEM or barrier
    a_sA += inst * bi.sA;
    a_W += inst * bi.W;
    V2 += inst * bi.V2;
    D += inst * bi.vec;
    C += inst * bi.vec;
    sigma += inst * bi.vec;
  }
  __shared__ __align__(8) uint64_t mbar[2];
  __shared__ uint32_t tslot;
  const int K = nsa + 1, kq4 = kpad >> 2;
  const int rows1 = (mrows > 128 ? ((mrows - 128 + 7) & ~7) : 0);  // rows held for tile 1
  const int abytes = (128 + rows1) * kpad * 4, bbytes = 64 * kpad * 4;
  unsigned char* Ahi = smem_raw;
  unsigned char* Alo = Ahi + abytes;
  unsigned char* Bhi = Alo + abytes;
  unsigned char* Blo = Bhi + bbytes;
  float* G = (float*)(Blo + bbytes);                              // [2][K][kMmCols]
  float* E = G + (size_t)2 * K * kMmCols;                         // [mrows][kMmEStride]
  uint16_t* L = (uint16_t*)(E + (size_t)((mrows + 3) & ~3) * kMmEStride);  // [2][seg_max]
  int32_t* Jrow = (int32_t*)(L + (size_t)2 * seg_max);            // [K]
  const int64_t Ia = blockIdx.x;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (warp == 0) tc::tmem_alloc(&tslot, 256);
  if (tid == 0) {
    tc::mbar_init(&mbar[0], 1);
    tc::mbar_init(&mbar[1], 1);
    tc::mbar_init_fence();
  }
  // A operand: element (r, k) of tile t = r / 128 at byte 16 c of the tile,
  // c = ((r % 128) / 8 * kq4 + k / 4) * 8 + r % 8
  const int nA = (128 + rows1) * kq4;  // 16-byte chunks, both tiles (tile 1 only its held rows)
  const bool issuer = tid >= kOtThreads;  // the last warp issues the MMAs; the others work
  for (int ci = issuer ? nA : tid; ci < nA; ci += kOtThreads) {
    const int t = ci >= 128 * kq4 ? 1 : 0;
    const int c = ci - t * 128 * kq4;
    const int cm = c >> 3, rr = c & 7;
    const int r = t * 128 + (cm / kq4) * 8 + rr, k0 = (cm % kq4) * 4;
    float h[4], l[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int k = k0 + q;
      float v = 0.f;
      if (r < mrows) {
        if (k < nsa) {
          const int32_t vo = __ldg(a_svo + Ia * nsa + k);
          const int pq = (vo & 0xff) + n * ((vo >> 8) & 0xff);
          v = (r == mr + n) ? __ldg(a_sA + Ia * nsa + k) : __ldg(V2 + (size_t)pq * mrp + r);
          v = negate_if<float>(v, (vo >> 16) != 0);
        } else if (k == nsa && r < mr) {
          v = __ldg(a_W + (int64_t)__ldg(rs_of + r) * na + Ia);
        }
      }
      h[q] = tc::to_tf32(v);
      l[q] = tc::to_tf32(v - h[q]);
    }
    const int off = t * 128 * kpad * 4 + 16 * c;
    *(float4*)(Ahi + off) = make_float4(h[0], h[1], h[2], h[3]);
    *(float4*)(Alo + off) = make_float4(l[0], l[1], l[2], l[3]);
  }
  for (int k = issuer ? K : tid; k < K; k += kOtThreads) Jrow[k] = k < nsa ? __ldg(a_sJ + Ia * nsa + k) : (int32_t)Ia;
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = tslot;
  // copies in (cp.async, one commit group each): the chunk's C rows (G) and
  // its walk lists (L)
  auto stage_g = [&](int chunk, int buf) {
    const int j0 = chunk * kMmCols;
    float* g = G + (size_t)buf * K * kMmCols;
    if (vec) {
      for (int i = tid; i < K * (kMmCols / 4); i += kOtThreads) {
        const int k = i / (kMmCols / 4), j = 4 * (i - k * (kMmCols / 4));
        const bool ok = j0 + j < nb;
        const unsigned sa = (unsigned)__cvta_generic_to_shared(g + k * kMmCols + j);
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(sa),
                     "l"(C + (int64_t)Jrow[k] * nb + (ok ? j0 + j : 0)), "r"(ok ? 16 : 0)
                     : "memory");
      }
    } else {
      for (int i = tid; i < K * kMmCols; i += kOtThreads) {
        const int k = i / kMmCols, j = i - k * kMmCols;
        const bool ok = j0 + j < nb;
        cp_async4_zfill(g + i, C + (int64_t)Jrow[k] * nb + (ok ? j0 + j : 0), ok);
      }
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
  };
  auto stage_l = [&](int chunk, int buf) {
    const int u0 = __ldg(seg + chunk), nv = (__ldg(seg + chunk + 1) - u0) >> 3;
    uint16_t* l = L + (size_t)buf * seg_max;
    for (int i = tid; i < nv; i += kOtThreads) cp_async16(l + 8 * i, lists + u0 + 8 * i);
    asm volatile("cp.async.commit_group;\n" ::: "memory");
  };
  float acc[JPT];
#pragma unroll
  for (int j = 0; j < JPT; ++j) {
    const int Ib = tid + j * kOtThreads;
    acc[j] = (!issuer && Ib < nb) ? sigma[Ia * nb + Ib] + (float)D[Ia * nb + Ib] * C[Ia * nb + Ib] : 0.f;
  }
  constexpr uint32_t idesc = tc::idesc_tf32(128, kMmCols);
  const uint32_t sbo = (uint32_t)kq4 * 128;
  const int nchunk = (nb + kMmCols - 1) / kMmCols;
  const int ntile = mrows > 128 ? 2 : 1;
  // descriptors of K step 0; a K step moves the start by 256 bytes (16 in
  // the descriptor's address field), a tile by 128 kpad 4 bytes
  const uint64_t dah = tc::desc(tc::smem_addr(Ahi), 128, sbo), dal = tc::desc(tc::smem_addr(Alo), 128, sbo);
  const uint64_t dbh = tc::desc(tc::smem_addr(Bhi), 128, sbo), dbl = tc::desc(tc::smem_addr(Blo), 128, sbo);
  const uint64_t tstep = (uint64_t)((128 * kpad * 4) >> 4);
  uint32_t par0 = 0u, par1 = 0u;
  bool ok = true;
  // B operand of chunk cc (G buffer cc & 1): element (j, k) at byte 16 ci of
  // Bhi / Blo, ci = (j / 8 kq4 + k / 4) 8 + j % 8
  auto split = [&](int cc) {
    const float* g = G + (size_t)(cc & 1) * K * kMmCols;
    for (int ci = tid; ci < kMmCols * kq4; ci += kOtThreads) {
      const int cm = ci >> 3, j = (cm / kq4) * 8 + (ci & 7), k0 = (cm % kq4) * 4;
      float h[4], l[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const float v = k0 + q < K ? g[(k0 + q) * kMmCols + j] : 0.f;
        h[q] = tc::to_tf32(v);
        l[q] = tc::to_tf32(v - h[q]);
      }
      *(float4*)(Bhi + 16 * ci) = make_float4(h[0], h[1], h[2], h[3]);
      *(float4*)(Blo + 16 * ci) = make_float4(l[0], l[1], l[2], l[3]);
    }
    tc::fence_proxy_async();
  };
  // MMAs of chunk cc into TMEM set cc & 1 (columns 128 (cc & 1) + 64 t)
  auto issue = [&](int cc) {
    {
      tc::fence_after();
      const uint32_t dset = tmem + (uint32_t)((cc & 1) * 128);
      for (int t = 0; t < ntile; ++t) {
        const uint32_t dt = dset + (uint32_t)(t * kMmCols);
        for (int ks = 0; ks < kpad / 8; ++ks) {
          const uint64_t ko = (uint64_t)ks * 16, ah = dah + t * tstep + ko, al = dal + t * tstep + ko;
          tc::mma_tf32(dt, ah, dbh + ko, idesc, ks ? 1u : 0u);
          tc::mma_tf32(dt, ah, dbl + ko, idesc, 1u);
          tc::mma_tf32(dt, al, dbh + ko, idesc, 1u);
        }
      }
      tc::commit(&mbar[cc & 1]);
    }
  };
  // Named barriers: 1 the 512 workers; 2 "B operand of the next chunk
  // written and TMEM set free" (workers arrive, the issuer warp waits).
  // Copy schedule: G(c + 2) leaves at the start of iteration c (its buffer's
  // chunk c was split in iteration c - 1), L(c + 2) at its end (after walk
  // c); "all but the newest group" before split(c + 1) covers G(c + 1),
  // L(c + 1) and L(c).  A worker reaches arrive(c + 1) only after it has
  // seen MMA(c) complete, which the issuer started after its wait for c, so
  // barrier 2 never holds two workers' rounds at once.  After a timed-out
  // wait the workers keep the barrier rounds (no more waits) so the issuer
  // finishes, and the output is NaN.
  auto bar_sync = [](int id, int cnt) { asm volatile("bar.sync %0, %1;\n" ::"r"(id), "r"(cnt) : "memory"); };
  auto bar_arrive = [](int id, int cnt) { asm volatile("bar.arrive %0, %1;\n" ::"r"(id), "r"(cnt) : "memory"); };
  constexpr int kAll = kOtThreads + 32;
  if (issuer) {
    for (int cc = 0; cc < nchunk; ++cc) {
      bar_sync(2, kAll);
      if (lane == 0) issue(cc);
      __syncwarp();
    }
  } else {
    stage_g(0, 0);
    stage_l(0, 0);
    if (nchunk > 1) {
      stage_g(1, 1);
      stage_l(1, 1);
    }
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    bar_sync(1, kOtThreads);
    split(0);
    tc::fence_before();
    bar_arrive(2, kAll);
    for (int c = 0; c < nchunk; ++c) {
      if (c + 2 < nchunk) stage_g(c + 2, c & 1);
      // MMA(c) done: the B operand is free and TMEM set c & 1 holds chunk c's E
      if (ok) ok = tc::mbar_wait(&mbar[c & 1], (c & 1) ? par1 : par0, kTcSpin);
      if (c & 1)
        par1 ^= 1u;
      else
        par0 ^= 1u;
      if (c + 2 < nchunk)
        asm volatile("cp.async.wait_group 1;\n" ::: "memory");
      else
        asm volatile("cp.async.wait_group 0;\n" ::: "memory");
      if (c + 1 < nchunk) {  // chunk c + 1's products run while chunk c is read out and walked
        bar_sync(1, kOtThreads);
        split(c + 1);
        tc::fence_before();
        bar_arrive(2, kAll);
      }
      tc::fence_after();
      if (ok) {
        // warp w: lanes 32 (w % 4).., tile (w / 4) % 2, columns 32 (w / 8)..
        const int q = warp & 3, t = (warp >> 2) & 1, half = warp >> 3;
        const int row = t * 128 + q * 32 + lane;
        if (t * 128 < mrows) {
#pragma unroll 1
          for (int cb = half * 32; cb < half * 32 + 32; cb += 16) {
            float v[16];
            tc::tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)((c & 1) * 128 + t * kMmCols + cb), v);
            if (row < mrows) {
              float* e = E + (size_t)row * kMmEStride + cb;
#pragma unroll
              for (int i = 0; i < 16; i += 4) *(float4*)(e + i) = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
            }
          }
        }
      }
      tc::fence_before();
      bar_sync(1, kOtThreads);
      const uint16_t* off = L + (size_t)(c & 1) * seg_max;
      const uint16_t* ent = off + off_u16;
#pragma unroll
      for (int j = 0; j < JPT; ++j) {
        const int Ib = tid + j * kOtThreads;
        if (Ib < nb) {
          const int e1 = off[Ib + 1];
          float s = acc[j];
#pragma unroll 4
          for (int e = off[Ib]; e < e1; ++e) {
            const uint32_t w = ent[e];
            s += negate_if<float>(E[w & 0x7fff], (w >> 15) != 0);
          }
          acc[j] = s;
        }
      }
      bar_sync(1, kOtThreads);  // E and L buffer c & 1 free
      if (c + 2 < nchunk) stage_l(c + 2, c & 1);
    }
  }
  if (!ok) {
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
#pragma unroll
    for (int j = 0; j < JPT; ++j) acc[j] = __int_as_float(0x7fc00000);
    if (tid == 0) atomicOr(&g_tc_fault, 1u);
  }
  if (!issuer) {
#pragma unroll
    for (int j = 0; j < JPT; ++j) {
      const int Ib = tid + j * kOtThreads;
      if (Ib < nb) sigma[Ia * nb + Ib] = acc[j];
    }
  }
  tc::fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_free(tmem, 256);
}

// the timed forms of this space's shape on the context (see Context::direct_tune)
static void tune_record(Context* c, const DirectSigma* d) {
  const int64_t na = d->a.nstr, nb = (d->same ? d->a : d->b).nstr;
  for (Context::DirectTune& t : c->direct_tune)
    if (t.n == d->n && t.na == na && t.nb == nb && t.tc == d->tc) {
      t.dense = d->dense_state;
      t.otc = d->otc_state;
      return;
    }
  c->direct_tune.push_back({d->n, na, nb, d->tc, d->dense_state, d->otc_state});
}
static void tune_recall(Context* c, DirectSigma* d) {
  const int64_t na = d->a.nstr, nb = (d->same ? d->a : d->b).nstr;
  for (const Context::DirectTune& t : c->direct_tune)
    if (t.n == d->n && t.na == na && t.nb == nb && t.tc == d->tc) {
      if (d->dense_state < 0) d->dense_state = t.dense;
      if (d->otc_state < 0) d->otc_state = t.otc;
      return;
    }
}

template <typename T>
static void direct_sigma_t(Context* c, const T* x, T* y) {
  DirectSigma* d = c->direct;
  const SpinTables& A = d->a;
  const SpinTables& B = d->same ? d->a : d->b;
  const int64_t na = A.nstr, nb = B.nstr, N = na * nb;
  const bool f64 = sizeof(T) == 8;
  // the contraction form applies every single excitation but the beta
  // singles' string-only part, so the same-spin part is then the alpha
  // doubles and the beta doubles plus string-only singles
  const bool mm = !f64 && d->mm;
  auto P = [&](const DeviceBuffer& b64, const DeviceBuffer& b32) { return (const T*)(f64 ? b64.ptr : b32.ptr); };
  auto same_spin = [&]() {
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
  };
  if constexpr (sizeof(T) == 4) {
    if (mm) {
      // y = Haa x + x HbbT
      auto dense = [&]() {
        if (d->tc) {
          tm_products(c, d, na, nb, 1, nullptr, (const float*)d->HaaS.ptr, (const float*)d->HbbS.ptr, 0, 0,
                      (float*)d->XA.ptr, (float*)d->XB.ptr, (const float*)x, (float*)y);
        } else {
          dim3 g((unsigned)((nb + kGmT - 1) / kGmT), (unsigned)((na + kGmT - 1) / kGmT));
          k_ds_gemm2<<<g, 256, 0, c->stream>>>((int)na, (int)nb, (int)na, (int)nb, (const float*)d->Haa.ptr,
                                                (const float*)x, (const float*)x, (const float*)d->HbbT.ptr,
                                                (float*)y, GmInst{});
        }
        QDKGB_CHECK_LAUNCH();
      };
      if (d->dense_state < 0) {
        // first FP32 sigma of this space: time both forms of the same-spin part
        cudaEvent_t e[3];
        for (cudaEvent_t& ev : e) QDKGB_CUDA(cudaEventCreate(&ev));
        for (int form = 0; form < 2; ++form) {
          form ? dense() : same_spin();  // warm
          QDKGB_CUDA(cudaEventRecord(e[0], c->stream));
          for (int r = 0; r < 3; ++r) form ? dense() : same_spin();
          QDKGB_CUDA(cudaEventRecord(e[1], c->stream));
          QDKGB_CUDA(cudaEventSynchronize(e[1]));
          float ms = 0.f;
          QDKGB_CUDA(cudaEventElapsedTime(&ms, e[0], e[1]));
          d->dense_ms[form] = ms / 3.0;
        }
        for (cudaEvent_t& ev : e) QDKGB_CUDA(cudaEventDestroy(ev));
        d->dense_state = d->dense_ms[1] < d->dense_ms[0] ? 1 : 0;
        tune_record(c, d);
      }
      if (d->dense_state == 1)
        dense();
      else
        same_spin();
      // opposite spin + diagonal + the singles
      auto go = [&](auto kern) {
        kern<<<(unsigned)na, d->mm_threads, d->mm_smem, c->stream>>>(
            (int)na, (int)nb, A.ns, d->mr, d->mrp, d->off_u16, d->seg_max, d->mm_vec ? 1 : 0,
            (const int32_t*)A.sJ.ptr, (const int32_t*)A.svo.ptr, (const float*)A.sA32.ptr, (const float*)A.W32.ptr,
            (const int32_t*)d->rs_of.ptr, (const uint16_t*)d->lists.ptr, (const int32_t*)d->seg.ptr,
            (const float*)d->V2mm.ptr, d->n, (const double*)c->H.diag.ptr, (const float*)x, (float*)y);
      };
      // the contraction into yo (which reads yo as its start value): the
      // FMA-pipe kernel (0) or the tensor-core one (1)
      auto contract = [&](float* yo, int form) {
        if (form == 1) {
          auto gt = [&](auto kern) {
            kern<<<(unsigned)na, kOtThreads + 32, d->otc_smem, c->stream>>>(
                (int)na, (int)nb, A.ns, d->mr, d->mr + d->n + 1, d->kpad, d->off_u16, d->seg_max,
                d->mm_vec ? 1 : 0, (const int32_t*)A.sJ.ptr, (const int32_t*)A.svo.ptr, (const float*)A.sA32.ptr,
                (const float*)A.W32.ptr, (const int32_t*)d->rs_of.ptr, (const uint16_t*)d->lists.ptr,
                (const int32_t*)d->seg.ptr, (const float*)d->V2mm.ptr, d->mrp, d->n, (const double*)c->H.diag.ptr,
                (const float*)x, yo, DsInst{});
          };
          switch (d->otc_jpt) {
            case 2: gt(k_ds_opposite_tc<2>); break;
            case 4: gt(k_ds_opposite_tc<4>); break;
            default: gt(k_ds_opposite_tc<8>); break;
          }
          QDKGB_CHECK_LAUNCH();
          return;
        }
        auto go = [&](auto kern) {
          kern<<<(unsigned)na, d->mm_threads, d->mm_smem, c->stream>>>(
              (int)na, (int)nb, A.ns, d->mr, d->mrp, d->off_u16, d->seg_max, d->mm_vec ? 1 : 0,
              (const int32_t*)A.sJ.ptr, (const int32_t*)A.svo.ptr, (const float*)A.sA32.ptr, (const float*)A.W32.ptr,
              (const int32_t*)d->rs_of.ptr, (const uint16_t*)d->lists.ptr, (const int32_t*)d->seg.ptr,
              (const float*)d->V2mm.ptr, d->n, (const double*)c->H.diag.ptr, (const float*)x, yo, DsInst{});
        };
        if (d->mm_threads <= 320) {
          switch (d->mm_jpt) {
            case 2: go(k_ds_opposite_mm<2, false>); break;
            case 4: go(k_ds_opposite_mm<4, false>); break;
            case 6: go(k_ds_opposite_mm<6, false>); break;
            case 8: go(k_ds_opposite_mm<8, false>); break;
            case 12: go(k_ds_opposite_mm<12, false>); break;
            case 16: go(k_ds_opposite_mm<16, false>); break;
            default: go(k_ds_opposite_mm<24, false>); break;
          }
        } else {
          switch (d->mm_jpt) {
            case 2: go(k_ds_opposite_mm<2, true>); break;
            case 4: go(k_ds_opposite_mm<4, true>); break;
            case 6: go(k_ds_opposite_mm<6, true>); break;
            case 8: go(k_ds_opposite_mm<8, true>); break;
            case 12: go(k_ds_opposite_mm<12, true>); break;
            default: go(k_ds_opposite_mm<16, true>); break;
          }
        }
        QDKGB_CHECK_LAUNCH();
      };
      if (d->otc && d->otc_state < 0) {
        // first FP32 sigma of this space: time both contractions on a copy
        // of the same-spin result and keep the faster
        float* sc = (float*)dev_alloc(c, d->tmp32, N * sizeof(float));
        cudaEvent_t e0, e1;
        QDKGB_CUDA(cudaEventCreate(&e0));
        QDKGB_CUDA(cudaEventCreate(&e1));
        for (int form = 0; form < 2; ++form) {
          double tot = 0.;
          for (int r = 0; r < 4; ++r) {
            QDKGB_CUDA(cudaMemcpyAsync(sc, y, N * sizeof(float), cudaMemcpyDeviceToDevice, c->stream));
            QDKGB_CUDA(cudaEventRecord(e0, c->stream));
            contract(sc, form);
            QDKGB_CUDA(cudaEventRecord(e1, c->stream));
            QDKGB_CUDA(cudaEventSynchronize(e1));
            float ms = 0.f;
            QDKGB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            if (r > 0) tot += ms;
          }
          d->otc_ms[form] = tot / 3.0;
        }
        QDKGB_CUDA(cudaEventDestroy(e0));
        QDKGB_CUDA(cudaEventDestroy(e1));
        d->otc_state = d->otc_ms[1] < d->otc_ms[0] ? 1 : 0;
        tune_record(c, d);
      }
      contract((float*)y, d->otc && d->otc_state == 1 ? 1 : 0);
      QDKGB_CHECK_LAUNCH();
      return;
    }
  }
  same_spin();
  // opposite spin + diagonal
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

// Values of every table from the current integrals (GPU).
static void direct_values(Context* c, DirectSigma* d) {
  spin_values(c, d->a);
  if (!d->same) spin_values(c, d->b);
  const int n = d->n;
  const int64_t n4 = (int64_t)n * n * n * n;
  float* V32 = dev_array<float>(c, d->V32, (size_t)n4);
  const unsigned b4 = (unsigned)std::min<int64_t>((n4 + 255) / 256, (int64_t)c->sm_count * 8);
  k_ds_v32<<<b4, 256, 0, c->stream>>>((const double*)c->V.ptr, V32, n4);
  QDKGB_CHECK_LAUNCH();
  if (!d->mm) return;
  const int64_t tot = (int64_t)n * n * d->mrp;
  k_ds_v2mm<<<(unsigned)std::min<int64_t>((tot + 255) / 256, (int64_t)c->sm_count * 8), 256, 0, c->stream>>>(
      (const double*)c->V.ptr, (const int32_t*)d->rs_of.ptr, n, d->mr, d->mrp, (float*)d->V2mm.ptr);
  QDKGB_CHECK_LAUNCH();
  const SpinTables& A = d->a;
  const SpinTables& B = d->same ? d->a : d->b;
  const int64_t na = A.nstr, nb = B.nstr;
  const char* env = std::getenv("QDKGB_DIRECT_DENSE");
  if (env && env[0] == '0') {
    d->dense_state = 0;
    return;
  }
  float* Haa = dev_array<float>(c, d->Haa, (size_t)(na * na));
  float* HbbT = dev_array<float>(c, d->HbbT, (size_t)(nb * nb));
  QDKGB_CUDA(cudaMemsetAsync(Haa, 0, (size_t)(na * na) * 4, c->stream));
  QDKGB_CUDA(cudaMemsetAsync(HbbT, 0, (size_t)(nb * nb) * 4, c->stream));
  const int64_t fill = na * A.nd + nb * B.nd + nb * B.ns;
  k_ds_dense_fill<<<(unsigned)std::min<int64_t>((fill + 255) / 256, (int64_t)c->sm_count * 8), 256, 0, c->stream>>>(
      na, A.nd, (const int32_t*)A.dJ.ptr, (const float*)A.dval32.ptr, nb, B.nd, B.ns, (const int32_t*)B.dJ.ptr,
      (const float*)B.dval32.ptr, (const int32_t*)B.sJ.ptr, (const int32_t*)B.svo.ptr, (const float*)B.sA32.ptr, Haa,
      HbbT);
  QDKGB_CHECK_LAUNCH();
  if (d->tc) {
    tm_sizes(d, na, nb);
    float* hs = dev_array<float>(c, d->HaaS, (size_t)(2 * d->szA1));
    float* bs = dev_array<float>(c, d->HbbS, (size_t)(2 * d->szB2));
    dev_array<float>(c, d->XA, (size_t)(2 * d->szA2));
    dev_array<float>(c, d->XB, (size_t)(2 * d->szB1));
    tm_split(c, Haa, (int)na, (int)na, na, 0, d->nkb1, hs, d->szA1, 1, 0, 0, nullptr);
    tm_split(c, HbbT, (int)nb, (int)nb, nb, 1, d->nkb2, bs, d->szB2, 1, 0, 0, nullptr);
    set_max_dynamic_smem((const void*)k_tc_gemm2b, kTmStages * kTmStage);
  }
  if (env && env[0] == '1') d->dense_state = 1;
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
  if (warps > kMmMaxWarps || mrp * kMmEStride > (1 << 15)) return;
  const int threads = warps * 32;
  int jpt = (int)((nb + threads - 1) / threads);
  for (int cand : {2, 4, 6, 8, 12, 16, 24})
    if (jpt <= cand) {
      jpt = cand;
      break;
    }
  if ((int64_t)jpt * threads < nb || (threads > 320 && jpt > 16)) return;
  // pair index of each (v, o), v != o
  std::vector<int32_t> rmap(n2, -1), rs_of(mr);
  for (int rs = 0, r = 0; rs < n2; ++rs)
    if (rs % n != rs / n) {
      rmap[rs] = r;
      rs_of[r++] = rs;
    }
  // per chunk: offsets (uint16) and entries of every beta string
  const int nchunk = (int)((nb + kMmCols - 1) / kMmCols);
  const int off_u16 = (int)((nb + 1 + 7) / 8 * 8);
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
      if ((bits >> p) & 1)
        v.push_back({((uint32_t)ib << 16) | (uint32_t)(mr + p), (uint32_t)ib | ((uint32_t)(mr + p) << 16)});
    v.push_back({((uint32_t)ib << 16) | (uint32_t)(mr + n), (uint32_t)ib | ((uint32_t)(mr + n) << 16)});
    std::sort(v.begin(), v.end());
  }
  std::vector<uint16_t> lists;
  std::vector<int32_t> seg(nchunk + 1);
  std::vector<size_t> cur(nb, 0);
  int seg_max = 0;
  for (int ch = 0; ch < nchunk; ++ch) {
    const uint32_t j0 = (uint32_t)ch * kMmCols, j1 = j0 + kMmCols;
    seg[ch] = (int32_t)lists.size();
    std::vector<uint16_t> off(off_u16, 0);
    std::vector<uint16_t> ent;
    for (int64_t ib = 0; ib < nb; ++ib) {
      off[ib] = (uint16_t)ent.size();
      auto& v = per[ib];
      while (cur[ib] < v.size() && (v[cur[ib]].second & 0xffff) < j1) {
        const uint32_t w = v[cur[ib]++].second;
        const uint32_t jl = (w & 0xffff) - j0, r = (w >> 16) & 0x7fff;
        ent.push_back((uint16_t)((r * kMmEStride + jl) | ((w >> 31) << 15)));
      }
      if (ent.size() > 65535) return;
    }
    off[nb] = (uint16_t)ent.size();
    lists.insert(lists.end(), off.begin(), off.end());
    lists.insert(lists.end(), ent.begin(), ent.end());
    while (lists.size() % 8) lists.push_back(0);
    seg_max = std::max(seg_max, (int)(lists.size() - seg[ch]));
  }
  seg[nchunk] = (int32_t)lists.size();
  if (lists.size() >= (size_t)INT32_MAX) return;
  const int K = A.ns + 1;
  const size_t smem = ((size_t)K * mrp + (size_t)2 * K * kMmCols + (size_t)mrp * kMmEStride) * 4 +
                      (size_t)2 * seg_max * 2 + (size_t)K * 4;
  if (smem > 220 * 1024) return;
  auto up = [&](DeviceBuffer& b, const void* src, size_t bytes) {
    void* ptr = dev_alloc(c, b, bytes + 16);
    QDKGB_CUDA(cudaMemcpyAsync(ptr, src, bytes, cudaMemcpyHostToDevice, c->stream));
  };
  dev_array<float>(c, d->V2mm, (size_t)n2 * mrp);
  up(d->rs_of, rs_of.data(), rs_of.size() * 4);
  up(d->lists, lists.data(), lists.size() * 2);
  up(d->seg, seg.data(), seg.size() * 4);
  for (const void* f :
       {(const void*)k_ds_opposite_mm<2, false>, (const void*)k_ds_opposite_mm<4, false>,
        (const void*)k_ds_opposite_mm<6, false>, (const void*)k_ds_opposite_mm<8, false>,
        (const void*)k_ds_opposite_mm<12, false>, (const void*)k_ds_opposite_mm<16, false>,
        (const void*)k_ds_opposite_mm<24, false>, (const void*)k_ds_opposite_mm<2, true>,
        (const void*)k_ds_opposite_mm<4, true>, (const void*)k_ds_opposite_mm<6, true>,
        (const void*)k_ds_opposite_mm<8, true>, (const void*)k_ds_opposite_mm<12, true>,
        (const void*)k_ds_opposite_mm<16, true>})
    set_max_dynamic_smem(f, 220 * 1024);
  d->mr = mr;
  d->mrp = mrp;
  d->mm_threads = threads;
  d->mm_jpt = jpt;
  d->seg_max = seg_max;
  d->off_u16 = off_u16;
  d->mm_vec = nb % 4 == 0;
  d->mm_smem = smem;
  QDKGB_CUDA(cudaStreamSynchronize(c->stream));
  d->mm = true;
}

// The direct sigma's structure for the context's space (built once per
// space; set_dets frees it) and its per-build settings from the environment.
static DirectSigma* direct_structure(Context* c) {
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
  // structure once per determinant space (set_dets frees it), values from
  // the current integrals on every build
  auto env0 = [](const char* name) {
    const char* e = std::getenv(name);
    return e ? e[0] : (char)0;
  };
  const char mm_env = env0("QDKGB_DIRECT_MM"), dense_env = env0("QDKGB_DIRECT_DENSE");
  const bool tc = env0("QDKGB_DIRECT_TC") != '0';
  if (c->direct && (c->direct->n != c->norb || c->direct->mm_env != mm_env)) free_direct(c);
  if (c->direct && c->direct->dense_env != dense_env) c->direct->dense_state = -1;
  if (!c->direct) {
    c->direct = new DirectSigma();
    DirectSigma* d = c->direct;
    d->n = c->norb;
    d->mm_env = mm_env;
    build_spin_tables(c, S.h_galpha, d->a);
    d->same = (S.h_galpha == S.h_ubeta);
    if (!d->same) build_spin_tables(c, S.h_ubeta, d->b);
    set_max_dynamic_smem((const void*)k_ds_opposite<double, 4>, 200 * 1024);
    set_max_dynamic_smem((const void*)k_ds_opposite<float, 8>, 200 * 1024);
    // contraction form of the FP32 sigma, where its tables and shared memory
    // fit (QDKGB_DIRECT_MM=0 keeps the element-wise walk)
    build_mm_tables(c, d);
    d->a.h_packed.clear();
    d->b.h_packed.clear();
  }
  DirectSigma* d = c->direct;
  d->dense_env = dense_env;
  if (tc != d->tc) {
    d->dense_state = dense_env ? d->dense_state : -1;
    d->otc_state = -1;
  }
  d->tc = tc;
  d->otc = false;
  if (tc && d->mm) {
    const int K = d->a.ns + 1, mrows = d->mr + d->n + 1;
    const int kpad = (K + 7) / 8 * 8;
    const int rows1 = mrows > 128 ? ((mrows - 128 + 7) & ~7) : 0;
    const size_t smem = (size_t)2 * (128 + rows1) * kpad * 4 + (size_t)2 * 64 * kpad * 4 +
                        (size_t)2 * K * kMmCols * 4 + (size_t)((mrows + 3) & ~3) * kMmEStride * 4 +
                        (size_t)2 * d->seg_max * 2 + (size_t)K * 4;
    const int64_t nbs = (d->same ? d->a : d->b).nstr;
    int jpt = (int)((nbs + kOtThreads - 1) / kOtThreads);
    jpt = jpt <= 2 ? 2 : jpt <= 4 ? 4 : 8;
    if (mrows <= 256 && smem <= 226 * 1024 && (int64_t)jpt * kOtThreads >= nbs) {
      d->otc = true;
      d->kpad = kpad;
      d->otc_jpt = jpt;
      d->otc_smem = smem;
      for (const void* f : {(const void*)k_ds_opposite_tc<2>, (const void*)k_ds_opposite_tc<4>,
                            (const void*)k_ds_opposite_tc<8>})
        set_max_dynamic_smem(f, (int)smem);
    }
  }
  if (!dense_env) tune_recall(c, d);  // forms timed before for this shape
  return d;
}

static DirectSigma* direct_prepare(Context* c) {
  if (!c->have_ints) throw Error(QDKGB_ERR_STATE, "integrals not set");
  DirectSigma* d = direct_structure(c);
  direct_values(c, d);
  return d;
}

void direct_plan(const Context* c, int* mm, int* dense, double* ms) {
  const DirectSigma* d = c->direct;
  if (mm) *mm = !(d && d->mm) ? 0 : (d->otc && d->otc_state == 1) ? 2 : 1;
  if (dense) *dense = d ? d->dense_state : -1;
  if (ms) {
    ms[0] = d ? d->dense_ms[0] : 0.;
    ms[1] = d ? d->dense_ms[1] : 0.;
    ms[2] = d ? d->otc_ms[0] : 0.;
    ms[3] = d ? d->otc_ms[1] : 0.;
  }
}

bool attach_direct_fp32(Context* c) {
  NvtxRange nvtx_range("qdkgb.attach_direct_fp32");
  const char* env = std::getenv("QDKGB_MIXED_FP32");
  if (env && env[0] == 's') return false;  // "slab": the stored FP32 copy
  DirectSigma* d = nullptr;
  try {
    d = direct_prepare(c);
  } catch (const Error&) {
    return false;
  }
  return d->mm;
}

void build_direct_sigma(Context* c) {
  NvtxRange nvtx_range("qdkgb.build_direct_sigma");
  c->fp32_direct = false;
  direct_prepare(c);
  DetSpace& S = c->dets;
  // diagonal and operator state
  Hcsr& H = c->H;
  H.valid = false;
  const int64_t N = S.ndets;
  double* D = dev_array<double>(c, H.diag, N);
  const unsigned blocks = (unsigned)std::min<int64_t>((N + 255) / 256, (int64_t)c->sm_count * 16);
  k_diag_product<<<blocks, 256, 0, c->stream>>>(integrals_view(c), S.ngroups, S.nbeta,
                                               (const uint64_t*)S.galpha.ptr, (const uint64_t*)S.ubeta.ptr, D);
  QDKGB_CHECK_LAUNCH();
  QDKGB_CUDA(cudaStreamSynchronize(c->stream));
  H.n = N;
  H.nnz = 0;
  H.valid = true;
  c->op_direct = true;
}

// ---------------------------------------------------------------- batched CASCI
// FP32 sigma of a sub-batch of instances of one complete space (the batched
// solver's new directions): the structure of the context's space, the value
// tables per instance from the instances' integrals (T: [B][n^2], V:
// [B][n^4] on the device).  False where the contraction form does not apply
// (the caller keeps the stored FP32 slab).
bool direct_batch_prepare(Context* c, int B, const double* T, const double* V) {
  const char* env = std::getenv("QDKGB_BATCH_DIRECT");
  if (env && env[0] == '0') return false;
  DirectSigma* d = nullptr;
  try {
    d = direct_structure(c);
  } catch (const Error&) {
    return false;
  }
  if (!d->mm || !d->tc) return false;
  const SpinTables& A = d->a;
  const SpinTables& Bt = d->same ? d->a : d->b;
  const int n = d->n;
  const int64_t n2 = (int64_t)n * n, n4 = n2 * n2, na = A.nstr, nb = Bt.nstr;
  const int64_t sa = na * A.ns, wa = n2 * na, da = na * std::max(A.nd, 1);
  const int64_t sb = nb * Bt.ns, wb = n2 * nb, db = nb * std::max(Bt.nd, 1);
  float* sAa = dev_array<float>(c, d->bsAa, (size_t)(B * sa + 1));
  float* Wa = dev_array<float>(c, d->bWa, (size_t)(B * wa));
  float* dva = dev_array<float>(c, d->bdva, (size_t)(B * da));
  float* sAb = d->same ? sAa : dev_array<float>(c, d->bsAb, (size_t)(B * sb + 1));
  float* Wb = d->same ? Wa : dev_array<float>(c, d->bWb, (size_t)(B * wb));
  float* dvb = d->same ? dva : dev_array<float>(c, d->bdvb, (size_t)(B * db));
  float* V2 = dev_array<float>(c, d->bV2, (size_t)(B * n2 * d->mrp));
  float* Haa = dev_array<float>(c, d->bHaa, (size_t)(B * na * na));
  float* HbbT = dev_array<float>(c, d->bHbbT, (size_t)(B * nb * nb));
  QDKGB_CUDA(cudaMemsetAsync(Haa, 0, (size_t)(B * na * na) * 4, c->stream));
  QDKGB_CUDA(cudaMemsetAsync(HbbT, 0, (size_t)(B * nb * nb) * 4, c->stream));
  auto vals = [&](const SpinTables& t, int q, float* sA, float* W, float* dv) {
    const int64_t tot = t.nstr * t.ns + t.nstr * t.nd + n2 * t.nstr;
    const unsigned blocks = (unsigned)std::min<int64_t>((tot + 255) / 256, (int64_t)c->sm_count * 4);
    k_ds_values<<<blocks, 256, 0, c->stream>>>(t.nstr, t.ns, t.nd, n, (const uint64_t*)t.str.ptr,
                                               (const int32_t*)t.svo.ptr, (const uint32_t*)t.dvo.ptr, T + q * n2,
                                               V + q * n4, nullptr, sA, nullptr, dv, nullptr, W);
    QDKGB_CHECK_LAUNCH();
  };
  for (int q = 0; q < B; ++q) {
    vals(A, q, sAa + q * sa, Wa + q * wa, dva + q * da);
    if (!d->same) vals(Bt, q, sAb + q * sb, Wb + q * wb, dvb + q * db);
    const int64_t tot = n2 * d->mrp;
    k_ds_v2mm<<<(unsigned)std::min<int64_t>((tot + 255) / 256, (int64_t)c->sm_count * 4), 256, 0, c->stream>>>(
        V + q * n4, (const int32_t*)d->rs_of.ptr, n, d->mr, d->mrp, V2 + q * n2 * d->mrp);
    QDKGB_CHECK_LAUNCH();
    const int64_t fill = na * A.nd + nb * Bt.nd + nb * Bt.ns;
    k_ds_dense_fill<<<(unsigned)std::min<int64_t>((fill + 255) / 256, (int64_t)c->sm_count * 4), 256, 0,
                      c->stream>>>(na, A.nd, (const int32_t*)A.dJ.ptr, dva + q * da, nb, Bt.nd, Bt.ns,
                                   (const int32_t*)Bt.dJ.ptr, dvb + q * db, (const int32_t*)Bt.sJ.ptr,
                                   (const int32_t*)Bt.svo.ptr, sAb + q * sb, Haa + q * na * na, HbbT + q * nb * nb);
    QDKGB_CHECK_LAUNCH();
  }
  tm_sizes(d, na, nb);
  float* hs = dev_array<float>(c, d->bHaaS, (size_t)(B * 2 * d->szA1));
  float* bs = dev_array<float>(c, d->bHbbS, (size_t)(B * 2 * d->szB2));
  dev_array<float>(c, d->bXA, (size_t)(B * 2 * d->szA2));
  dev_array<float>(c, d->bXB, (size_t)(B * 2 * d->szB1));
  tm_split(c, Haa, (int)na, (int)na, na, 0, d->nkb1, hs, d->szA1, B, na * na, 2 * d->szA1, nullptr);
  tm_split(c, HbbT, (int)nb, (int)nb, nb, 1, d->nkb2, bs, d->szB2, B, nb * nb, 2 * d->szB2, nullptr);
  set_max_dynamic_smem((const void*)k_tc_gemm2b, kTmStages * kTmStage);
  d->bcap = B;
  return true;
}

// y = sigma(x) in FP32 for the instances with act[q] != 0 (x, y: [B][N];
// D: [B][N] the FP64 diagonals): the dense same-spin products, then the
// contraction (tensor cores or FMA pipe by a fixed rule).
void direct_batch_sigma(Context* c, int B, const int* act, const double* D, const float* x, float* y) {
  DirectSigma* d = c->direct;
  const SpinTables& A = d->a;
  const SpinTables& Bt = d->same ? d->a : d->b;
  const int n = d->n;
  const int64_t n2 = (int64_t)n * n, na = A.nstr, nb = Bt.nstr, N = na * nb;
  const float* sAa = (const float*)d->bsAa.ptr;
  const float* Wa = (const float*)d->bWa.ptr;
  tm_products(c, d, na, nb, B, act, (const float*)d->bHaaS.ptr, (const float*)d->bHbbS.ptr, 2 * d->szA1,
              2 * d->szB2, (float*)d->bXA.ptr, (float*)d->bXB.ptr, x, y);
  const DsInst bi{act, na * A.ns, n2 * na, n2 * d->mrp, N};
  auto contract = [&](float* yo, int form) {
    if (form == 1) {
      auto gt = [&](auto kern) {
        kern<<<dim3((unsigned)na, (unsigned)B), kOtThreads + 32, d->otc_smem, c->stream>>>(
            (int)na, (int)nb, A.ns, d->mr, d->mr + d->n + 1, d->kpad, d->off_u16, d->seg_max, d->mm_vec ? 1 : 0,
            (const int32_t*)A.sJ.ptr, (const int32_t*)A.svo.ptr, sAa, Wa, (const int32_t*)d->rs_of.ptr,
            (const uint16_t*)d->lists.ptr, (const int32_t*)d->seg.ptr, (const float*)d->bV2.ptr, d->mrp, d->n, D, x,
            yo, bi);
      };
      switch (d->otc_jpt) {
        case 2: gt(k_ds_opposite_tc<2>); break;
        case 4: gt(k_ds_opposite_tc<4>); break;
        default: gt(k_ds_opposite_tc<8>); break;
      }
    } else {
      auto go = [&](auto kern) {
        kern<<<dim3((unsigned)na, (unsigned)B), d->mm_threads, d->mm_smem, c->stream>>>(
            (int)na, (int)nb, A.ns, d->mr, d->mrp, d->off_u16, d->seg_max, d->mm_vec ? 1 : 0,
            (const int32_t*)A.sJ.ptr, (const int32_t*)A.svo.ptr, sAa, Wa, (const int32_t*)d->rs_of.ptr,
            (const uint16_t*)d->lists.ptr, (const int32_t*)d->seg.ptr, (const float*)d->bV2.ptr, d->n, D, x, yo,
            bi);
      };
      if (d->mm_threads <= 320) {
        switch (d->mm_jpt) {
          case 2: go(k_ds_opposite_mm<2, false>); break;
          case 4: go(k_ds_opposite_mm<4, false>); break;
          case 6: go(k_ds_opposite_mm<6, false>); break;
          case 8: go(k_ds_opposite_mm<8, false>); break;
          case 12: go(k_ds_opposite_mm<12, false>); break;
          case 16: go(k_ds_opposite_mm<16, false>); break;
          default: go(k_ds_opposite_mm<24, false>); break;
        }
      } else {
        switch (d->mm_jpt) {
          case 2: go(k_ds_opposite_mm<2, true>); break;
          case 4: go(k_ds_opposite_mm<4, true>); break;
          case 6: go(k_ds_opposite_mm<6, true>); break;
          case 8: go(k_ds_opposite_mm<8, true>); break;
          case 12: go(k_ds_opposite_mm<12, true>); break;
          default: go(k_ds_opposite_mm<16, true>); break;
        }
      }
    }
    QDKGB_CHECK_LAUNCH();
  };
  if (d->bform < 0) {
    // a fixed rule, so that repeated calls (eager or graph-replayed) take the
    // same form and give the same sums: the tensor cores when E has more than
    // one 128-row tile, else the FMA pipe (QDKGB_BATCH_CONTRACTION=tc|fma)
    const char* env = std::getenv("QDKGB_BATCH_CONTRACTION");
    const int mrows = d->mr + d->n + 1;
    d->bform = (d->otc && (env ? env[0] == 't' : mrows > 128)) ? 1 : 0;
  }
  contract(y, d->bform);
}

}  // namespace qdkgb
