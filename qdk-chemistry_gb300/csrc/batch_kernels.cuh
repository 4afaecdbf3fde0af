// Device pieces shared by the batched CASCI solvers (batch.cu: the lockstep
// launch sequence; batch_persist.cu: the persistent cluster solver).
#pragma once
#include "common.cuh"

namespace qdkgb {

// deterministic filler in [-1, 1): the last-resort second restart vector,
// inside the spin-flip sector s of an nstr x nstr coefficient matrix when
// s != 0 (f(i, j) = s f(j, i))
__device__ __forceinline__ double filler(int64_t i, int64_t nstr, double s) {
  int64_t key = i;
  double sg = 1.;
  if (s != 0.) {
    const int64_t g = i / nstr, b = i - g * nstr;
    if (g == b && s < 0.) return 0.;
    key = g < b ? g * nstr + b : b * nstr + g;
    sg = (g > b) ? s : 1.;
  }
  uint64_t h = (uint64_t)key * 0x9E3779B97F4A7C15ull;
  h ^= h >> 31;
  h *= 0xBF58476D1CE4E5B9ull;
  h ^= h >> 29;
  return sg * ((double)(h >> 11) * 0x1p-52 - 1.0);
}

// spin-summed 1-RDM gamma_pq = <C| a+_p a_q |C> (alpha + beta) of a complete
// space by one CTA: diagonal from the row / column weights, off-diagonal from
// one dot product per single excitation of an alpha group (rows) or a beta
// string (columns) - form_rdms_spin_dep's one-body part
// (sorted_double_loop.hpp:626-753) on the product structure.  X is read
// through L2 (it may have been written by other CTAs of the running kernel);
// gam: norb^2 doubles of shared memory; out: norb^2 doubles.
__device__ __forceinline__ void rdm1_cta(const double* __restrict__ X, int G, int Nb, int norb,
                                         const uint64_t* __restrict__ galpha, const uint64_t* __restrict__ ubeta,
                                         const int64_t* __restrict__ acon_ptr, const int32_t* __restrict__ acon_idx,
                                         const int8_t* __restrict__ acon_lvl, const int64_t* __restrict__ b1_ptr,
                                         const int32_t* __restrict__ b1_idx, double* __restrict__ out, double* gam) {
  const int nn = norb * norb;
  for (int i = threadIdx.x; i < nn; i += blockDim.x) gam[i] = 0.;
  __syncthreads();
  // diagonal
  for (int g = threadIdx.x; g < G; g += blockDim.x) {
    double w = 0.;
    for (int j = 0; j < Nb; ++j) {
      const double c = __ldcg(X + (int64_t)g * Nb + j);
      w += c * c;
    }
    for (uint64_t s = galpha[g]; s; s &= s - 1) atomicAdd(&gam[low_bit(s) * (norb + 1)], w);
  }
  for (int j = threadIdx.x; j < Nb; j += blockDim.x) {
    double w = 0.;
    for (int g = 0; g < G; ++g) {
      const double c = __ldcg(X + (int64_t)g * Nb + j);
      w += c * c;
    }
    for (uint64_t s = ubeta[j]; s; s &= s - 1) atomicAdd(&gam[low_bit(s) * (norb + 1)], w);
  }
  // alpha singles: pairs (g, h > g)
  for (int g = threadIdx.x; g < G; g += blockDim.x) {
    const uint64_t ket = galpha[g];
    for (int64_t e = acon_ptr[g]; e < acon_ptr[g + 1]; ++e) {
      const int h = acon_idx[e];
      if (acon_lvl[e] != 1 || h <= g) continue;
      const uint64_t bra = galpha[h];
      double dot = 0.;
      for (int j = 0; j < Nb; ++j) dot += __ldcg(X + (int64_t)h * Nb + j) * __ldcg(X + (int64_t)g * Nb + j);
      const SingleEx sx = single_ex(bra, ket, bra ^ ket);
      const double v = sx.neg ? -dot : dot;
      atomicAdd(&gam[sx.v * norb + sx.o], v);
      atomicAdd(&gam[sx.o * norb + sx.v], v);
    }
  }
  // beta singles: pairs (j, j2 > j)
  for (int j = threadIdx.x; j < Nb; j += blockDim.x) {
    const uint64_t ket = ubeta[j];
    for (int64_t e = b1_ptr[j]; e < b1_ptr[j + 1]; ++e) {
      const int j2 = b1_idx[e];
      if (j2 <= j) continue;
      const uint64_t bra = ubeta[j2];
      double dot = 0.;
      for (int g = 0; g < G; ++g) dot += __ldcg(X + (int64_t)g * Nb + j2) * __ldcg(X + (int64_t)g * Nb + j);
      const SingleEx sx = single_ex(bra, ket, bra ^ ket);
      const double v = sx.neg ? -dot : dot;
      atomicAdd(&gam[sx.v * norb + sx.o], v);
      atomicAdd(&gam[sx.o * norb + sx.v], v);
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nn; i += blockDim.x) out[i] = gam[i];
  __syncthreads();
}

}  // namespace qdkgb
