// Device-side bit algebra and Slater-Condon matrix elements on uint64 spin strings.
//
// Every function here reproduces the operation order of the MACIS routine it
// cites, so that FP64 matrix elements are bitwise identical to the reference
// (sums of integrals in ascending orbital order, sign applied last; no
// multiply-add pattern exists in these formulas, so FMA contraction cannot
// change a result).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#define QDKGB_FULL_MASK 0xffffffffu

namespace qdkgb {

__device__ __forceinline__ int popc64(uint64_t x) { return __popcll(x); }
// 0-based index of the lowest set bit (macis::ffs(x) - 1, bitset_operations.hpp:240-263).
__device__ __forceinline__ uint32_t low_bit(uint64_t x) { return (uint32_t)(__ffsll((long long)x) - 1); }
// macis::full_mask(i): bits [0, i) (bitset_operations.hpp:230-238).
__device__ __forceinline__ uint64_t full_mask(uint32_t i) { return i >= 64 ? ~0ull : ((1ull << i) - 1ull); }

// single_excitation_sign (sd_operations.hpp:40-50): true when the number of
// occupied orbitals of `state` strictly between p and q is odd.
__device__ __forceinline__ bool excitation_sign_odd(uint64_t state, uint32_t p, uint32_t q) {
  const uint64_t m = (p > q) ? (full_mask(p) ^ full_mask(q + 1)) : (full_mask(q) ^ full_mask(p + 1));
  return popc64(state & m) & 1;
}

struct Integrals {
  const double* T;     // n x n
  const double* V;     // n^4
  const double* G_red; // n^3: G_red(p, i, j) at p + n i + n^2 j
  const double* V_red; // n^3
  const double* G2;    // n^2
  const double* V2;    // n^2
  int n;
};

__device__ __forceinline__ double ld(const double* p) { return __ldg(p); }

// Sign flip and |v| > t on the integer pipes.  GB300's FP64 pipe is narrow;
// flipping the sign bit is bit-identical to multiplying by -1.0, and for
// finite values |a| > |b| orders like the magnitude bit patterns.
__device__ __forceinline__ double flip_if(double v, bool neg) {
  return __longlong_as_double(__double_as_longlong(v) ^ ((long long)neg << 63));
}
// tbits < 0 means "keep everything" (threshold <= 0)
__device__ __forceinline__ bool above_thresh(double v, long long tbits) {
  return tbits < 0 || (__double_as_longlong(v) & 0x7fffffffffffffffLL) > tbits;
}

__device__ __forceinline__ double Vat(const Integrals& I, uint32_t p, uint32_t q, uint32_t r, uint32_t s) {
  const size_t n = (size_t)I.n;
  return ld(I.V + p + n * (q + n * (r + n * s)));
}

// single_excitation_sign_indices (sd_operations.hpp:394-402)
struct SingleEx {
  uint32_t o, v;
  bool neg;
};
__device__ __forceinline__ SingleEx single_ex(uint64_t bra, uint64_t ket, uint64_t ex) {
  SingleEx s;
  s.o = low_bit(ket & ex);
  s.v = low_bit(bra & ex);
  s.neg = excitation_sign_odd(ket, s.v, s.o);
  return s;
}

// matrix_element_4 with doubles_sign_indices (matrix_elements.hpp:113-121,
// sd_operations.hpp:413-425)
__device__ __forceinline__ double me_same_spin_double(const Integrals& I, uint64_t bra, uint64_t ket, uint64_t ex) {
  SingleEx a = single_ex(bra, ket, ex);
  const uint64_t flip = (1ull << a.o) | (1ull << a.v);
  ket ^= flip;
  ex ^= flip;
  SingleEx b = single_ex(bra, ket, ex);
  const double g = Vat(I, a.v, a.o, b.v, b.o) - Vat(I, a.v, b.o, b.v, a.o);
  return flip_if(g, a.neg != b.neg);
}

// matrix_element_22 (matrix_elements.hpp:140-151)
__device__ __forceinline__ double me_opposite_spin_double(const Integrals& I, uint64_t bra_a, uint64_t ket_a,
                                                          uint64_t ex_a, uint64_t bra_b, uint64_t ket_b,
                                                          uint64_t ex_b) {
  SingleEx a = single_ex(bra_a, ket_a, ex_a);
  SingleEx b = single_ex(bra_b, ket_b, ex_b);
  const double v = Vat(I, a.v, a.o, b.v, b.o);
  return flip_if(v, a.neg != b.neg);
}

// matrix_element_2 (matrix_elements.hpp:169-189): T(v,o) + sum over the bra's
// same-spin occupations of G_red(p,v,o) + sum over its other-spin occupations
// of V_red(p,v,o), ascending p.
__device__ __forceinline__ double me_single(const Integrals& I, uint64_t bra, uint64_t ket, uint64_t ex,
                                            uint64_t bra_other) {
  SingleEx s = single_ex(bra, ket, ex);
  const size_t n = (size_t)I.n;
  double h = ld(I.T + s.v + n * s.o);
  const double* g = I.G_red + n * (s.v + n * s.o);
  for (uint64_t m = bra; m; m &= m - 1) h += ld(g + low_bit(m));
  const double* vr = I.V_red + n * (s.v + n * s.o);
  for (uint64_t m = bra_other; m; m &= m - 1) h += ld(vr + low_bit(m));
  return flip_if(h, s.neg);
}

// matrix_element_diag (matrix_elements.hpp:203-230)
__device__ __forceinline__ double me_diag(const Integrals& I, uint64_t a, uint64_t b) {
  const size_t n = (size_t)I.n;
  double h = 0.;
  for (uint64_t m = a; m; m &= m - 1) {
    const uint32_t p = low_bit(m);
    h += ld(I.T + p + n * p);
  }
  for (uint64_t m = b; m; m &= m - 1) {
    const uint32_t p = low_bit(m);
    h += ld(I.T + p + n * p);
  }
  for (uint64_t mq = a; mq; mq &= mq - 1) {
    const double* col = I.G2 + n * low_bit(mq);
    for (uint64_t mp = a; mp; mp &= mp - 1) h += ld(col + low_bit(mp));
  }
  for (uint64_t mq = b; mq; mq &= mq - 1) {
    const double* col = I.G2 + n * low_bit(mq);
    for (uint64_t mp = b; mp; mp &= mp - 1) h += ld(col + low_bit(mp));
  }
  for (uint64_t mq = b; mq; mq &= mq - 1) {
    const double* col = I.V2 + n * low_bit(mq);
    for (uint64_t mp = a; mp; mp &= mp - 1) h += ld(col + low_bit(mp));
  }
  return h;
}

// matrix_element dispatch (matrix_elements.hpp:65-97) for a pair already
// known to be within a double excitation.
__device__ __forceinline__ double matrix_element(const Integrals& I, uint64_t bra_a, uint64_t bra_b, uint64_t ket_a,
                                                 uint64_t ket_b) {
  const uint64_t exa = bra_a ^ ket_a, exb = bra_b ^ ket_b;
  const int ca = popc64(exa), cb = popc64(exb);
  if (ca == 4) return me_same_spin_double(I, bra_a, ket_a, exa);
  if (cb == 4) return me_same_spin_double(I, bra_b, ket_b, exb);
  if (ca == 2 && cb == 2) return me_opposite_spin_double(I, bra_a, ket_a, exa, bra_b, ket_b, exb);
  if (ca == 2) return me_single(I, bra_a, ket_a, exa, bra_b);
  if (cb == 2) return me_single(I, bra_b, ket_b, exb, bra_a);
  return me_diag(I, bra_a, bra_b);
}

// Off-diagonal element (the pair differs), as matrix_element.
__device__ __forceinline__ double offdiag_element(const Integrals& I, uint64_t bra_a, uint64_t bra_b, uint64_t ket_a,
                                                  uint64_t ket_b) {
  const uint64_t exa = bra_a ^ ket_a, exb = bra_b ^ ket_b;
  const int ca = popc64(exa), cb = popc64(exb);
  if (ca == 4) return me_same_spin_double(I, bra_a, ket_a, exa);
  if (cb == 4) return me_same_spin_double(I, bra_b, ket_b, exb);
  if (ca == 2 && cb == 2) return me_opposite_spin_double(I, bra_a, ket_a, exa, bra_b, ket_b, exb);
  if (ca == 2) return me_single(I, bra_a, ket_a, exa, bra_b);
  return me_single(I, bra_b, ket_b, exb, bra_a);
}

// Warp-wide inclusive scan of an int.
__device__ __forceinline__ int warp_inclusive_scan(int v, int lane) {
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    int t = __shfl_up_sync(QDKGB_FULL_MASK, v, d);
    if (lane >= d) v += t;
  }
  return v;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(QDKGB_FULL_MASK, v, d);
  return v;
}

// Unevaluated float-float sum (two-sum), used by the full-precision sigma
// from split storage: a.s + a.c carries ~2^-44 relative accuracy on the FP32
// pipe.
struct FF {
  float s, c;
};
__device__ __forceinline__ void ff_add(FF& a, float p, float e) {
  const float t = a.s + p;
  const float bv = t - a.s;
  const float err = (a.s - (t - bv)) + (p - bv);
  a.s = t;
  a.c += err + e;
}
__device__ __forceinline__ FF ff_merge(FF a, FF b) {
  FF r = a;
  ff_add(r, b.s, b.c);
  return r;
}
// (h + l)(x + y) as p + e with p = fl(h x) and e its rounding error plus the
// cross terms (the l*y term is below the pair's resolution)
__device__ __forceinline__ void ff_prod(float h, float l, float x, float y, float& p, float& e) {
  p = h * x;
  e = fmaf(h, x, -p);
  e = fmaf(h, y, fmaf(l, x, e));
}

// (hi, lo) = (fl32(v), fl32(v - fl32(v))), both round-to-nearest-even: the
// split storage of an FP64 value.  On the integer pipes for |v| in
// [2^-74, 2^127) (the FP64 pipe is narrow on GB300): the 53-bit significand is
// rounded to 24 bits by hand, and the exact remainder (at most 29 bits) is
// converted and scaled by a power of two.  Zeros, tiny and huge values, NaN
// and Inf take the FP64 conversions.  Bit-identical to the FP64 form.
__device__ __forceinline__ void split_f64(double v, float& hi, float& lo) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(v);
  const unsigned int sign = (unsigned int)(u >> 32) & 0x80000000u;
  const int e = (int)((u >> 52) & 0x7ff) - 1023;
  if ((u << 1) == 0) {
    hi = __uint_as_float(sign);
    lo = 0.f;
    return;
  }
  if (e < -74 || e > 126) {
    const float h = __double2float_rn(v);
    hi = h;
    lo = __double2float_rn(v - (double)h);
    return;
  }
  const unsigned long long M = (u & 0xFFFFFFFFFFFFFull) | (1ull << 52);
  unsigned int q = (unsigned int)(M >> 29);
  const unsigned int r = (unsigned int)(M & 0x1FFFFFFFu);
  const bool up = r > 0x10000000u || (r == 0x10000000u && (q & 1u));
  const int res = up ? (int)r - (1 << 29) : (int)r;  // v - hi in units of 2^(e - 52)
  q += up ? 1u : 0u;
  int eh = e;
  if (q == (1u << 24)) {
    q >>= 1;
    ++eh;
  }
  hi = __uint_as_float(sign | ((unsigned int)(eh + 127) << 23) | (q & 0x7FFFFFu));
  const float lf = __int2float_rn(res) * __uint_as_float((unsigned int)(e - 52 + 127) << 23);
  lo = res == 0 ? 0.f : (sign ? -lf : lf);
}

}  // namespace qdkgb
