// The slab sigma tile shared by the sigma kernels (fci_struct.cu) and the
// persistent batched solver (batch_persist.cu): one CTA applies the rows of
// one alpha group (a part of its beta strings) over one segment of the row
// positions, with the segment's staged x slices in shared memory.
#pragma once
#include "common.cuh"

namespace qdkgb {

struct Context;

constexpr int kSlabUnroll = 8;  // independent value loads in flight per thread

// the row-shape tables of a complete space (slab layout)
struct SlabArgs {
  int G, Nb, rowlen, n1, n2;
  int seglen;  // emission / export position range per CTA
  const int32_t* blT;
  const uint32_t* gdesc;
};

// one sigma plan: S segments per group, at most M staged x slices per
// segment, R ints of segment record per (group, segment)
struct PlanArgs {
  int S, M, R;
  const int32_t* rec;
  const int32_t* segh;
};

SlabArgs slab_args(Context* c);
// plan 0: 4-byte staged x (FP32 sigma); plan 1: 8-byte staged x (FP64 and
// float-float sigmas)
PlanArgs slab_plan_args(Context* c, int pl);
// shared-memory bytes of one tile of plan pl with x_bytes per staged element
size_t slab_plan_smem(Context* c, int pl, size_t x_bytes);

//   MODE 0: FP32 values, FP32 x, FP32 accumulation
//   MODE 1: FP64 values, FP64 x, FP64 accumulation
//   MODE 2: split values (hi, lo) with split x (xh, xl), float-float sums
// gx reads x through the read-only path; gx_l2 through L2 (for an x written
// by other CTAs of the same kernel).
template <int MODE>
struct SlabPol;
template <>
struct SlabPol<0> {
  using Xs = float;
  using Acc = float;
  using Out = float;
  struct Val {
    float h;
  };
  static __device__ __forceinline__ Val load(const void* v, const float*, int64_t q) {
    return {__ldcs((const float*)v + q)};
  }
  static __device__ __forceinline__ Xs gx(const void* x, const float*, int64_t i) { return __ldg((const float*)x + i); }
  static __device__ __forceinline__ Xs gx_l2(const void* x, const float*, int64_t i) {
    return __ldcg((const float*)x + i);
  }
  static __device__ __forceinline__ void add(Acc& a, Val v, Xs x) { a = fmaf(v.h, x, a); }
  static __device__ __forceinline__ Acc zero() { return 0.f; }
  static __device__ __forceinline__ Acc merge(Acc a, Acc b) { return a + b; }
  static __device__ __forceinline__ Out fin(Acc a) { return a; }
};
template <>
struct SlabPol<1> {
  using Xs = double;
  using Acc = double;
  using Out = double;
  struct Val {
    double h;
  };
  static __device__ __forceinline__ Val load(const void* v, const float*, int64_t q) {
    return {__ldcs((const double*)v + q)};
  }
  static __device__ __forceinline__ Xs gx(const void* x, const float*, int64_t i) {
    return __ldg((const double*)x + i);
  }
  static __device__ __forceinline__ Xs gx_l2(const void* x, const float*, int64_t i) {
    return __ldcg((const double*)x + i);
  }
  static __device__ __forceinline__ void add(Acc& a, Val v, Xs x) { a = fma(v.h, x, a); }
  static __device__ __forceinline__ Acc zero() { return 0.; }
  static __device__ __forceinline__ Acc merge(Acc a, Acc b) { return a + b; }
  static __device__ __forceinline__ Out fin(Acc a) { return a; }
};
template <>
struct SlabPol<2> {
  using Xs = float2;
  using Acc = FF;
  using Out = double;
  struct Val {
    float h, l;
  };
  static __device__ __forceinline__ Val load(const void* v, const float* vlo, int64_t q) {
    return {__ldcs((const float*)v + q), __ldcs(vlo + q)};
  }
  static __device__ __forceinline__ Xs gx(const void* x, const float* xlo, int64_t i) {
    return make_float2(__ldg((const float*)x + i), __ldg(xlo + i));
  }
  static __device__ __forceinline__ Xs gx_l2(const void* x, const float* xlo, int64_t i) {
    return make_float2(__ldcg((const float*)x + i), __ldcg(xlo + i));
  }
  static __device__ __forceinline__ void add(Acc& a, Val v, Xs x) {
    float p, e;
    ff_prod(v.h, v.l, x.x, x.y, p, e);
    ff_add(a, p, e);
  }
  static __device__ __forceinline__ Acc zero() { return FF{0.f, 0.f}; }
  static __device__ __forceinline__ Acc merge(Acc a, Acc b) { return ff_merge(a, b); }
  static __device__ __forceinline__ Out fin(Acc a) { return (double)a.s + (double)a.c; }
};

__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}

// One tile: rows (g, b) for the beta strings b of part z (blockDim.x strings
// per part) over segment s.  The x slices of the segment's staged blocks are
// copied to shared memory; the own-group block runs over b's level-2 list,
// the alpha-single blocks share b's level-1 list (each list entry is loaded
// once and used for every block of the segment), the alpha doubles read
// x[h * Nb + b] (coalesced).  Row (g, b) of segment s goes to
// y[s * part_stride + g * Nb + b].  L2X: x was written by other CTAs of the
// running kernel, so it is read through L2 (plain staging loads, ld.global.cg)
// instead of the read-only path and cp.async.ca.  Ends with the staged slices
// still in use by other threads: a caller that runs another tile on the same
// shared memory synchronises the CTA first.
template <int MODE, bool L2X>
__device__ __forceinline__ void slab_sigma_tile(const SlabArgs& A, const PlanArgs& P, const void* __restrict__ vals,
                                                const float* __restrict__ vlo, const void* __restrict__ xv,
                                                const float* __restrict__ xlo, void* __restrict__ yv,
                                                int64_t part_stride, int g, int s, int z, unsigned char* smem_raw) {
  using Pol = SlabPol<MODE>;
  using Xs = typename Pol::Xs;
  using Acc = typename Pol::Acc;
  using Val = typename Pol::Val;
  constexpr int U = MODE == 2 ? kSlabUnroll / 2 : kSlabUnroll;  // loads in flight per thread
  const int Nb = A.Nb;
  Xs* xs = reinterpret_cast<Xs*>(smem_raw);
  int32_t* rec = reinterpret_cast<int32_t*>(xs + (size_t)P.M * Nb);
  const int32_t* rg = P.rec + ((int64_t)g * P.S + s) * P.R;
  for (int i = threadIdx.x; i < P.R; i += blockDim.x) rec[i] = __ldg(rg + i);
  const int32_t* sh = P.segh + ((int64_t)g * P.S + s) * P.M;
  if constexpr (L2X) {
    for (int j = 0; j < P.M; ++j) {
      const int h = __ldg(sh + j);
      if (h < 0) continue;
      for (int i = threadIdx.x; i < Nb; i += blockDim.x)
        xs[(size_t)j * Nb + i] = Pol::gx_l2(xv, xlo, (int64_t)h * Nb + i);
    }
  } else {
    // staging: every slice copy in flight at once (cp.async), then one wait
    for (int j = 0; j < P.M; ++j) {
      const int h = __ldg(sh + j);
      if (h < 0) continue;
      for (int i = threadIdx.x; i < Nb; i += blockDim.x) {
        const int64_t src = (int64_t)h * Nb + i;
        Xs* dst = xs + (size_t)j * Nb + i;
        if constexpr (MODE == 0) {
          cp_async4(dst, (const float*)xv + src);
        } else if constexpr (MODE == 1) {
          cp_async8(dst, (const double*)xv + src);
        } else {
          cp_async4(&dst->x, (const float*)xv + src);
          cp_async4(&dst->y, xlo + src);
        }
      }
    }
    cp_async_wait_all();
  }
  __syncthreads();
  const int has0 = rec[0], off0 = rec[1], sb0 = rec[2], n1b = rec[3];
  const int32_t* e1 = rec + 4;
  const int nd = rec[4 + 2 * n1b];
  const int32_t* e2 = rec + 6 + 2 * n1b;
  const int bend = min(Nb, (z + 1) * (int)blockDim.x);
  for (int b = z * blockDim.x + threadIdx.x; b < bend; b += blockDim.x) {
    const int64_t gbase = (int64_t)g * A.rowlen * Nb + b;  // slab index of (g, p = 0, b)
    const int32_t* lst = A.blT + b;
    Acc acc[U];
#pragma unroll
    for (int j = 0; j < U; ++j) acc[j] = Pol::zero();
    // own-group block over b's level-2 list
    if (has0) {
      int k = 0;
      for (; k + U <= A.n2; k += U) {
        Val v[U];
        int l[U];
#pragma unroll
        for (int j = 0; j < U; ++j) {
          l[j] = __ldg(lst + (k + j) * Nb);
          v[j] = Pol::load(vals, vlo, gbase + off0 + (k + j) * Nb);
        }
#pragma unroll
        for (int j = 0; j < U; ++j) Pol::add(acc[j], v[j], xs[sb0 + l[j]]);
      }
      for (; k < A.n2; ++k)
        Pol::add(acc[0], Pol::load(vals, vlo, gbase + off0 + k * Nb), xs[sb0 + __ldg(lst + k * Nb)]);
    }
    // alpha-single blocks: each entry of b's level-1 list is loaded once and
    // used for every block of the segment
    for (int k = 0; k < A.n1; ++k) {
      const int l = __ldg(lst + (A.n2 + k) * Nb);
      const int kk = k * Nb;
      int e = 0;
      for (; e + U <= n1b; e += U) {
        Val v[U];
#pragma unroll
        for (int j = 0; j < U; ++j) v[j] = Pol::load(vals, vlo, gbase + e1[2 * (e + j)] + kk);
#pragma unroll
        for (int j = 0; j < U; ++j) Pol::add(acc[j], v[j], xs[e1[2 * (e + j) + 1] + l]);
      }
      for (; e < n1b; ++e) Pol::add(acc[0], Pol::load(vals, vlo, gbase + e1[2 * e] + kk), xs[e1[2 * e + 1] + l]);
    }
    // alpha doubles: x of the same beta string in group h
    {
      int j0 = 0;
      for (; j0 + U <= nd; j0 += U) {
        Val v[U];
        Xs xx[U];
#pragma unroll
        for (int j = 0; j < U; ++j) {
          v[j] = Pol::load(vals, vlo, gbase + e2[2 * (j0 + j)]);
          xx[j] = L2X ? Pol::gx_l2(xv, xlo, (int64_t)e2[2 * (j0 + j) + 1] + b)
                      : Pol::gx(xv, xlo, (int64_t)e2[2 * (j0 + j) + 1] + b);
        }
#pragma unroll
        for (int j = 0; j < U; ++j) Pol::add(acc[j], v[j], xx[j]);
      }
      for (; j0 < nd; ++j0)
        Pol::add(acc[0], Pol::load(vals, vlo, gbase + e2[2 * j0]),
                 L2X ? Pol::gx_l2(xv, xlo, (int64_t)e2[2 * j0 + 1] + b)
                     : Pol::gx(xv, xlo, (int64_t)e2[2 * j0 + 1] + b));
    }
#pragma unroll
    for (int j = 1; j < U; ++j) acc[0] = Pol::merge(acc[0], acc[j]);
    ((typename Pol::Out*)yv)[s * part_stride + (int64_t)g * Nb + b] = Pol::fin(acc[0]);
  }
}

}  // namespace qdkgb
