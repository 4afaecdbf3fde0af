// ASCI determinant search on the device (replaces asci_search /
// asci_contributions_constraint, include/macis/asci/determinant_search.hpp:
// 349-1123, with the contribution formulas of determinant_contributions.hpp:
// 93-297 and the fast diagonals of src/macis/hamiltonian_generator/
// fast_diagonals.ipp:52-127).
//
// GPU design: one warp per core determinant P enumerates every single and
// double excitation Q of P as one flat index space (alpha singles, beta
// singles, alpha-alpha, beta-beta, alpha-beta doubles), evaluates c_P <Q|H|P>
// and the fast diagonal E0 - H_QQ exactly as the reference does, drops
// |c h| < h_el_tol, and accumulates into an open-addressing hash table keyed by
// the full (alpha, beta) pair (128-bit atomicCAS, then exact fixed-point
// integer atomics of c h; see Table below).  That replaces the reference's
// constraint partitioning plus sort-and-accumulate: every Q's contributions
// meet in one slot.  The core itself is marked and drops out.  Then |rv| =
// |sum / (E0 - H_QQ)| is pruned (|rv| > rv_prune_tol), the k-th largest |rv|
// is found by a radix select on the bit patterns (four 16-bit digits), and
// every candidate with |rv| >= that value is kept - the reference's
// tie-inclusive top-k.  Sums and diagonals do not depend on the order of the
// atomics, so a search repeated on the same input selects the same set with
// the same scores; they agree with the reference's (whose unstable sort
// fixes its own order) to rounding, and the selected sets are identical
// unless two scores tie to the last bits at the cutoff.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <vector>

#include "common.cuh"
#include "host_parallel.h"
#include "internal.h"

namespace qdkgb {

namespace {

typedef unsigned __int128 u128;
constexpr u128 kEmpty = ~(u128)0;
constexpr int kAsciWarps = 8;
constexpr int kMaxOrb = 64;

__device__ __forceinline__ uint64_t mix64(uint64_t x) {
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdULL;
  x ^= x >> 33;
  x *= 0xc4ceb9fe1a85ec53ULL;
  x ^= x >> 33;
  return x;
}

// A target's accumulated c <Q|H|P> is kept in fixed point, two 64-bit words
// per slot: x = hi 2^-32 + lo 2^-76 with hi = rint(x 2^32) and lo the rest
// in units of 2^-76 (the split is exact).  Integer additions are exact and
// associative, so the sum - and the selection made from it - does not depend
// on the order in which the atomics land (FP64 atomics would).  |x| < 2^20
// and up to 2^19 contributions per target keep both words in range.  The
// slot's diagonal E0 - H_QQ (the fast diagonal, computed from each
// contributing P, equal up to rounding) is the largest bit pattern among its
// contributors (atomicMax on the bits: order-independent as well); core
// determinants set it to kCoreMark and drop out of the candidates.
constexpr long long kCoreMark = 0x7fffffffffffffffLL;
constexpr long long kHdEmpty = (long long)0x8000000000000000ULL;
constexpr double kFixHi = 4294967296.0;               // 2^32
constexpr double kFixLo = 75557863725914323419136.0;  // 2^76

struct Table {
  u128* keys;
  long long* acc;  // 2 words per slot (hi, lo)
  long long* hd;   // bit pattern of E0 - H_QQ, or kCoreMark
  uint64_t mask;
  int* err;  // set when a probe sequence runs past kMaxProbe (the table is too full): the pass is redone larger
};
constexpr uint64_t kMaxProbe = 4096;

__device__ __forceinline__ double table_sum(const Table& t, uint64_t i) {
  return (double)t.acc[2 * i] * (1.0 / kFixHi) + (double)t.acc[2 * i + 1] * (1.0 / kFixLo);
}
__device__ __forceinline__ bool table_core(const Table& t, uint64_t i) { return t.hd[i] == kCoreMark; }

// slot of (qa, qb), inserting the key; -1 when the probe limit is reached
__device__ __forceinline__ int64_t table_slot(const Table& t, uint64_t qa, uint64_t qb) {
  const u128 key = ((u128)qb << 64) | (u128)qa;
  uint64_t h = mix64(qa * 0x9e3779b97f4a7c15ULL ^ mix64(qb)) & t.mask;
  for (uint64_t probe = 0; probe <= t.mask && probe < kMaxProbe; ++probe) {
    const u128 old = atomicCAS(t.keys + h, kEmpty, key);
    if (old == kEmpty || old == key) return (int64_t)h;
    h = (h + 1) & t.mask;
  }
  *t.err = 1;
  return -1;
}

__device__ __forceinline__ void table_add(const Table& t, uint64_t qa, uint64_t qb, double ch, double hd) {
  const int64_t h = table_slot(t, qa, qb);
  if (h < 0) return;
  if (!(fabs(ch) < 1048576.0)) {  // outside the fixed-point range (or not finite)
    *t.err = 2;
    return;
  }
  const double hi = rint(ch * kFixHi);
  const double lo = rint((ch - hi * (1.0 / kFixHi)) * kFixLo);
  atomicAdd((unsigned long long*)t.acc + 2 * h, (unsigned long long)(long long)hi);
  atomicAdd((unsigned long long*)t.acc + 2 * h + 1, (unsigned long long)(long long)lo);
  atomicMax(t.hd + h, (long long)__double_as_longlong(hd));
}

__device__ __forceinline__ void table_add_core(const Table& t, uint64_t qa, uint64_t qb) {
  const int64_t h = table_slot(t, qa, qb);
  if (h >= 0) atomicMax(t.hd + h, kCoreMark);
}

struct CoreArgs {
  Integrals I;
  int n;
  int64_t ncore;
  const uint64_t* ca;
  const uint64_t* cb;
  const double* cc;
  double E0;
  double h_el_tol;
  Table T;
  uint32_t npass = 1, pass = 0;  // targets whose part_of() == pass are inserted (npass > 1: PT2 passes)
  bool just_singles = false;     // the search's just_singles: single excitations only
};

// part of the target space of a determinant in a split into npass passes (a
// hash independent of the table slot)
__device__ __forceinline__ uint32_t part_of(uint64_t qa, uint64_t qb, uint32_t npass) {
  return (uint32_t)(mix64(qb * 0x9e3779b97f4a7c15ULL ^ mix64(qa + 0x632be59bd9b4e019ULL)) % npass);
}

// (i, j) with i < j from a pair index p = j (j - 1) / 2 + i
__device__ __forceinline__ void pair_of(int p, int& i, int& j) {
  int jj = (int)((1.0f + sqrtf(1.0f + 8.0f * (float)p)) * 0.5f);
  while (jj * (jj - 1) / 2 > p) --jj;
  while ((jj + 1) * jj / 2 <= p) ++jj;
  j = jj;
  i = p - jj * (jj - 1) / 2;
}

struct WarpSm {
  double ea[kMaxOrb], eb[kMaxOrb];
  uint8_t oa[kMaxOrb], va[kMaxOrb], ob[kMaxOrb], vb[kMaxOrb];
};

__device__ __forceinline__ double G2at(const Integrals& I, uint32_t p, uint32_t q) {
  return ld(I.G2 + p + (size_t)I.n * q);
}
__device__ __forceinline__ double V2at(const Integrals& I, uint32_t p, uint32_t q) {
  return ld(I.V2 + p + (size_t)I.n * q);
}
// single_excitation_sign(state, a, i) as a double (+1 / -1)
__device__ __forceinline__ double sgn(uint64_t state, uint32_t a, uint32_t i) {
  return excitation_sign_odd(state, a, i) ? -1. : 1.;
}

__global__ void __launch_bounds__(kAsciWarps * 32) k_asci_enum(CoreArgs A) {
  __shared__ WarpSm wsm[kAsciWarps];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  WarpSm& s = wsm[w];
  const Integrals& I = A.I;
  const int n = A.n;
  const uint64_t full = (n == 64) ? ~0ull : ((1ull << n) - 1ull);
  for (int64_t ip = (int64_t)blockIdx.x * kAsciWarps + w; ip < A.ncore; ip += (int64_t)gridDim.x * kAsciWarps) {
    const uint64_t Pa = A.ca[ip], Pb = A.cb[ip];
    const double c = A.cc[ip];
    const int ka = popc64(Pa), kb = popc64(Pb), na_v = n - ka, nb_v = n - kb;
    // occupied / virtual lists and orbital energies (single_orbital_ens, fast_diagonals.ipp:30-50)
    if (lane == 0) {
      int x = 0, y = 0, u = 0, v = 0;
      for (int p = 0; p < n; ++p) {
        if ((Pa >> p) & 1)
          s.oa[x++] = p;
        else
          s.va[y++] = p;
        if ((Pb >> p) & 1)
          s.ob[u++] = p;
        else
          s.vb[v++] = p;
      }
    }
    for (int i = lane; i < n; i += 32) {
      double e = ld(I.T + i + (size_t)n * i);
      for (uint64_t m = Pa; m; m &= m - 1) {
        const uint32_t q = low_bit(m);
        e += G2at(I, i, q) + G2at(I, q, i);
      }
      e -= G2at(I, i, i);
      for (uint64_t m = Pb; m; m &= m - 1) e += V2at(I, i, low_bit(m));
      s.ea[i] = e;
      double f = ld(I.T + i + (size_t)n * i);
      for (uint64_t m = Pb; m; m &= m - 1) {
        const uint32_t q = low_bit(m);
        f += G2at(I, i, q) + G2at(I, q, i);
      }
      f -= G2at(I, i, i);
      for (uint64_t m = Pa; m; m &= m - 1) f += V2at(I, i, low_bit(m));
      s.eb[i] = f;
    }
    double hdiag = 0.;
    if (lane == 0) hdiag = me_diag(I, Pa, Pb);
    hdiag = __shfl_sync(QDKGB_FULL_MASK, hdiag, 0);
    __syncwarp();
    // the core determinant itself: infinite score (removed later)
    if (lane == 0 && (A.npass == 1 || part_of(Pa, Pb, A.npass) == A.pass)) table_add_core(A.T, Pa, Pb);
    const int64_t nsa = (int64_t)ka * na_v, nsb = (int64_t)kb * nb_v;
    const int64_t pa_o = (int64_t)ka * (ka - 1) / 2, pa_v = (int64_t)na_v * (na_v - 1) / 2;
    const int64_t pb_o = (int64_t)kb * (kb - 1) / 2, pb_v = (int64_t)nb_v * (nb_v - 1) / 2;
    const int64_t nda = pa_o * pa_v, ndb = pb_o * pb_v, nab = nsa * nsb;
    const int64_t total = A.just_singles ? nsa + nsb : nsa + nsb + nda + ndb + nab;
    for (int64_t e = lane; e < total; e += 32) {
      double ch = 0., hd = 0.;
      uint64_t qa = Pa, qb = Pb;
      bool ok = false;
      int64_t x = e;
      if (x < nsa + nsb) {
        // append_singles_asci_contributions (determinant_contributions.hpp:93-133)
        const bool alpha = x < nsa;
        if (!alpha) x -= nsa;
        const int nv = alpha ? na_v : nb_v;
        const uint32_t i = alpha ? s.oa[x / nv] : s.ob[x / nv];
        const uint32_t a = alpha ? s.va[x % nv] : s.vb[x % nv];
        const uint64_t same = alpha ? Pa : Pb, other = alpha ? Pb : Pa;
        const size_t nn = (size_t)n;
        double h = ld(I.T + a + nn * i);
        const double* G = I.G_red + nn * (a + nn * i);
        const double* Vr = I.V_red + nn * (a + nn * i);
        for (uint64_t m = same; m; m &= m - 1) h += ld(G + low_bit(m));
        for (uint64_t m = other; m; m &= m - 1) h += ld(Vr + low_bit(m));
        if (fabs(c * h) >= A.h_el_tol) {
          h *= sgn(same, a, i);
          const double* eps = alpha ? s.ea : s.eb;
          const double hdq = hdiag + eps[a] - eps[i] - G2at(I, a, i) - G2at(I, i, a);
          const uint64_t ex = (same ^ (1ull << i)) | (1ull << a);
          if (alpha)
            qa = ex;
          else
            qb = ex;
          ch = c * h;
          hd = A.E0 - hdq;
          ok = true;
        }
      } else if ((x -= nsa + nsb) < nda + ndb) {
        // append_ss_doubles_asci_contributions (determinant_contributions.hpp:149-210)
        const bool alpha = x < nda;
        if (!alpha) x -= nda;
        const int64_t pv = alpha ? pa_v : pb_v;
        int ii, jj, aa, bb;
        pair_of((int)(x / pv), ii, jj);
        pair_of((int)(x % pv), aa, bb);
        const uint8_t* occ = alpha ? s.oa : s.ob;
        const uint8_t* vir = alpha ? s.va : s.vb;
        const uint32_t i = occ[ii], j = occ[jj], a = vir[aa], b = vir[bb];
        const double Gv = Vat(I, b, j, a, i) - Vat(I, b, i, a, j);
        if (fabs(c * Gv) >= A.h_el_tol) {
          const uint64_t same = alpha ? Pa : Pb;
          const uint64_t fullex = (1ull << i) | (1ull << j) | (1ull << a) | (1ull << b);
          const uint64_t ex = same ^ fullex;
          // doubles_sign(state_same, ex_det, full_ex): bra = P, ket = Q
          SingleEx s1 = single_ex(same, ex, fullex);
          const uint64_t f1 = (1ull << s1.o) | (1ull << s1.v);
          SingleEx s2 = single_ex(same, ex ^ f1, fullex ^ f1);
          const double h = (s1.neg != s2.neg) ? -Gv : Gv;
          const double* eps = alpha ? s.ea : s.eb;
          const double hdq = hdiag + eps[a] + eps[b] - eps[i] - eps[j] + G2at(I, i, j) + G2at(I, j, i) +
                             G2at(I, a, b) + G2at(I, b, a) - G2at(I, a, i) - G2at(I, i, a) - G2at(I, b, i) -
                             G2at(I, i, b) - G2at(I, a, j) - G2at(I, j, a) - G2at(I, b, j) - G2at(I, j, b);
          if (alpha)
            qa = ex;
          else
            qb = ex;
          ch = c * h;
          hd = A.E0 - hdq;
          ok = true;
        }
      } else {
        // append_os_doubles_asci_contributions (determinant_contributions.hpp:226-297)
        x -= nda + ndb;
        const int64_t xa = x / nsb, xb = x % nsb;
        const uint32_t i = s.oa[xa / na_v], a = s.va[xa % na_v];
        const uint32_t j = s.ob[xb / nb_v], b = s.vb[xb % nb_v];
        const double V = Vat(I, a, i, b, j);
        if (fabs(c * V) >= A.h_el_tol) {
          const double sg = sgn(Pa, a, i) * sgn(Pb, b, j);
          const double hdq = hdiag + s.ea[a] + s.eb[b] - s.ea[i] - s.eb[j] + V2at(I, i, j) + V2at(I, a, b) -
                             G2at(I, a, i) - G2at(I, i, a) - G2at(I, b, j) - G2at(I, j, b) - V2at(I, a, j) -
                             V2at(I, i, b);
          qa = (Pa ^ (1ull << i)) | (1ull << a);
          qb = (Pb ^ (1ull << j)) | (1ull << b);
          ch = c * sg * V;
          hd = A.E0 - hdq;
          ok = true;
        }
      }
      if (ok && (A.npass == 1 || part_of(qa, qb, A.npass) == A.pass)) table_add(A.T, qa, qb, ch, hd);
    }
    __syncwarp();
    (void)full;
  }
}

// Number of distinct target determinants of an enumeration (every single
// and double of every core determinant, and the core itself) as a
// HyperLogLog sketch: 2^kHllBits registers hold the largest leading-zero rank
// of a 64-bit hash per bucket (block-local in shared memory, merged with
// atomicMax).  Sizes the hash table to the targets instead of the
// contributions (relative error ~1.04 / 2^(kHllBits/2)).
constexpr int kHllBits = 12, kHllRegs = 1 << kHllBits;
__device__ __forceinline__ void hll_add(unsigned* reg, uint64_t qa, uint64_t qb) {
  const uint64_t h = mix64(qb * 0xbf58476d1ce4e5b9ULL ^ mix64(qa + 0x94d049bb133111ebULL));
  const unsigned idx = (unsigned)(h >> (64 - kHllBits));
  const uint64_t w = h << kHllBits;
  const unsigned rank = w ? (unsigned)__clzll(w) + 1u : (unsigned)(64 - kHllBits + 1);
  if (reg[idx] < rank) atomicMax(reg + idx, rank);
}
__global__ void __launch_bounds__(kAsciWarps * 32) k_target_sketch(CoreArgs A, unsigned* __restrict__ regs) {
  __shared__ unsigned sreg[kHllRegs];
  __shared__ WarpSm wsm[kAsciWarps];
  for (int i = threadIdx.x; i < kHllRegs; i += blockDim.x) sreg[i] = 0u;
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  WarpSm& s = wsm[w];
  const int n = A.n;
  for (int64_t ip = (int64_t)blockIdx.x * kAsciWarps + w; ip < A.ncore; ip += (int64_t)gridDim.x * kAsciWarps) {
    const uint64_t Pa = A.ca[ip], Pb = A.cb[ip];
    const int ka = popc64(Pa), kb = popc64(Pb), na_v = n - ka, nb_v = n - kb;
    if (lane == 0) {
      int x = 0, y = 0, u = 0, v = 0;
      for (int p = 0; p < n; ++p) {
        if ((Pa >> p) & 1)
          s.oa[x++] = p;
        else
          s.va[y++] = p;
        if ((Pb >> p) & 1)
          s.ob[u++] = p;
        else
          s.vb[v++] = p;
      }
      hll_add(sreg, Pa, Pb);
    }
    __syncwarp();
    const int64_t nsa = (int64_t)ka * na_v, nsb = (int64_t)kb * nb_v;
    const int64_t pa_v = (int64_t)na_v * (na_v - 1) / 2, pb_v = (int64_t)nb_v * (nb_v - 1) / 2;
    const int64_t nda = (int64_t)ka * (ka - 1) / 2 * pa_v, ndb = (int64_t)kb * (kb - 1) / 2 * pb_v;
    const int64_t total = A.just_singles ? nsa + nsb : nsa + nsb + nda + ndb + nsa * nsb;
    for (int64_t e = lane; e < total; e += 32) {
      uint64_t qa = Pa, qb = Pb;
      int64_t x = e;
      if (x < nsa + nsb) {
        const bool alpha = x < nsa;
        if (!alpha) x -= nsa;
        const int nv = alpha ? na_v : nb_v;
        const uint32_t i = alpha ? s.oa[x / nv] : s.ob[x / nv];
        const uint32_t a = alpha ? s.va[x % nv] : s.vb[x % nv];
        if (alpha)
          qa = (Pa ^ (1ull << i)) | (1ull << a);
        else
          qb = (Pb ^ (1ull << i)) | (1ull << a);
      } else if ((x -= nsa + nsb) < nda + ndb) {
        const bool alpha = x < nda;
        if (!alpha) x -= nda;
        const int64_t pv = alpha ? pa_v : pb_v;
        int ii, jj, aa, bb;
        pair_of((int)(x / pv), ii, jj);
        pair_of((int)(x % pv), aa, bb);
        const uint8_t* occ = alpha ? s.oa : s.ob;
        const uint8_t* vir = alpha ? s.va : s.vb;
        const uint64_t full = (1ull << occ[ii]) | (1ull << occ[jj]) | (1ull << vir[aa]) | (1ull << vir[bb]);
        if (alpha)
          qa = Pa ^ full;
        else
          qb = Pb ^ full;
      } else {
        x -= nda + ndb;
        const int64_t xa = x / nsb, xb = x % nsb;
        qa = (Pa ^ (1ull << s.oa[xa / na_v])) | (1ull << s.va[xa % na_v]);
        qb = (Pb ^ (1ull << s.ob[xb / nb_v])) | (1ull << s.vb[xb % nb_v]);
      }
      hll_add(sreg, qa, qb);
    }
    __syncwarp();
  }
  __syncthreads();
  for (int i = threadIdx.x; i < kHllRegs; i += blockDim.x)
    if (sreg[i]) atomicMax(regs + i, sreg[i]);
}

// candidates: finite score with |rv| > prune; key = bit pattern of |rv|
__global__ void k_asci_extract(Table T, uint64_t cap, double prune, uint64_t* __restrict__ keys,
                               uint64_t* __restrict__ slots, unsigned long long* __restrict__ count) {
  const int lane = threadIdx.x & 31;
  for (uint64_t i0 = (uint64_t)blockIdx.x * blockDim.x; i0 < cap; i0 += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t i = i0 + threadIdx.x;
    bool take = false;
    double arv = 0.;
    if (i < cap && T.keys[i] != kEmpty && !table_core(T, i)) {
      arv = fabs(table_sum(T, i) / __longlong_as_double(T.hd[i]));
      take = arv > prune;
    }
    const unsigned m = __ballot_sync(QDKGB_FULL_MASK, take);
    unsigned long long base = 0;
    if (lane == 0 && m) base = atomicAdd(count, (unsigned long long)__popc(m));
    base = __shfl_sync(QDKGB_FULL_MASK, base, 0);
    if (take) {
      const unsigned long long p = base + __popc(m & ((1u << lane) - 1u));
      keys[p] = (uint64_t)__double_as_longlong(arv);
      slots[p] = i;
    }
  }
}

// histogram (2^width bins, block-local in shared memory) of the digit at
// `shift` among keys whose higher digits equal `prefix`
constexpr int kRadixBits = 11;
__global__ void k_radix_hist(const uint64_t* __restrict__ keys, uint64_t n, int shift, int width, uint64_t prefix,
                             uint64_t hi_mask, unsigned long long* __restrict__ hist) {
  __shared__ unsigned int sh[1 << kRadixBits];
  const int nb = 1 << width;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) sh[i] = 0;
  __syncthreads();
  const uint64_t dm = (uint64_t)nb - 1;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t k = keys[i];
    if ((k & hi_mask) == prefix) atomicAdd(sh + ((k >> shift) & dm), 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nb; i += blockDim.x)
    if (sh[i]) atomicAdd(hist + i, (unsigned long long)sh[i]);
}

__global__ void k_asci_select(const uint64_t* __restrict__ keys, const uint64_t* __restrict__ slots, uint64_t n,
                              uint64_t kth, Table T, uint64_t* __restrict__ oa, uint64_t* __restrict__ ob,
                              unsigned long long* __restrict__ count) {
  const int lane = threadIdx.x & 31;
  for (uint64_t i0 = (uint64_t)blockIdx.x * blockDim.x; i0 < n; i0 += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t i = i0 + threadIdx.x;
    const bool take = i < n && keys[i] >= kth;
    const unsigned m = __ballot_sync(QDKGB_FULL_MASK, take);
    unsigned long long base = 0;
    if (lane == 0 && m) base = atomicAdd(count, (unsigned long long)__popc(m));
    base = __shfl_sync(QDKGB_FULL_MASK, base, 0);
    if (take) {
      const unsigned long long p = base + __popc(m & ((1u << lane) - 1u));
      const u128 key = T.keys[slots[i]];
      oa[p] = (uint64_t)key;
      ob[p] = (uint64_t)(key >> 64);
    }
  }
}

// PT2 terms of the filled slots: sum^2 / (E0 - H_QQ) over finite sums (the
// wavefunction's own determinants carry an infinite sum), per block
__global__ void __launch_bounds__(256) k_pt2_sum(Table T, uint64_t cap, double* __restrict__ partial,
                                                 unsigned long long* __restrict__ count) {
  __shared__ double rs[8];
  __shared__ unsigned long long rc[8];
  double s = 0.;
  unsigned long long m = 0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < cap; i += (uint64_t)gridDim.x * blockDim.x) {
    if (T.keys[i] != kEmpty && !table_core(T, i)) {
      const double v = table_sum(T, i);
      s += v * v / __longlong_as_double(T.hd[i]);
      ++m;
    }
  }
  s = warp_sum(s);
  for (int d = 16; d > 0; d >>= 1) m += __shfl_xor_sync(QDKGB_FULL_MASK, m, d);
  if ((threadIdx.x & 31) == 0) {
    rs[threadIdx.x >> 5] = s;
    rc[threadIdx.x >> 5] = m;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.;
    unsigned long long u = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      t += rs[w];
      u += rc[w];
    }
    partial[blockIdx.x] = t;
    count[blockIdx.x] = u;
  }
}

__global__ void k_fill_empty(Table T, uint64_t cap) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < cap; i += (uint64_t)gridDim.x * blockDim.x) {
    T.keys[i] = kEmpty;
    T.acc[2 * i] = 0;
    T.acc[2 * i + 1] = 0;
    T.hd[i] = kHdEmpty;
  }
}

int64_t binom64(int n, int k) {
  if (k < 0 || k > n) return 0;
  long double r = 1;
  for (int i = 1; i <= k; ++i) r = r * (n - k + i) / i;
  return (int64_t)std::llround(r);
}

// HyperLogLog estimate of the distinct targets of an enumeration over the
// core list already on the device in A (small-range correction by linear
// counting); `regs` is kHllRegs device words of scratch
double distinct_targets(Context* c, const CoreArgs& A, unsigned* regs) {
  QDKGB_CUDA(cudaMemsetAsync(regs, 0, kHllRegs * sizeof(unsigned), c->stream));
  const unsigned eb = (unsigned)std::min<int64_t>((A.ncore + kAsciWarps - 1) / kAsciWarps, (int64_t)c->sm_count * 8);
  k_target_sketch<<<eb, kAsciWarps * 32, 0, c->stream>>>(A, regs);
  QDKGB_CHECK_LAUNCH();
  std::vector<unsigned> h(kHllRegs);
  QDKGB_CUDA(cudaMemcpyAsync(h.data(), regs, kHllRegs * sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
  QDKGB_CUDA(cudaStreamSynchronize(c->stream));
  const double m = kHllRegs;
  double z = 0.;
  int zeros = 0;
  for (unsigned r : h) {
    z += std::ldexp(1., -(int)r);
    zeros += r == 0;
  }
  double e = 0.7213 / (1. + 1.079 / m) * m * m / z;
  if (e <= 2.5 * m && zeros > 0) e = m * std::log(m / zeros);
  return e;
}

}  // namespace

// Returns the new determinant list (top-k candidates followed by the core).
void asci_search_gpu(Context* c, int64_t ncore, const uint64_t* ca, const uint64_t* cb, const double* cc, double E0,
                     int64_t ndets_max, double h_el_tol, double rv_prune_tol, std::vector<uint64_t>& out_a,
                     std::vector<uint64_t>& out_b, int64_t* n_candidates, bool just_singles) {
  NvtxRange nvtx_range("qdkgb.asci_search");
  if (!c->have_ints) throw Error(QDKGB_ERR_STATE, "integrals not set");
  if (ncore <= 0) throw Error(QDKGB_ERR_INVALID, "empty core");
  const int n = c->norb;
  {
    uint64_t u = 0;
    for (int64_t i = 0; i < ncore; ++i) u |= ca[i] | cb[i];
    if (n < 64 && (u >> n)) throw Error(QDKGB_ERR_INVALID, "a determinant occupies an orbital beyond the integrals' norb");
  }
  // table capacity from the number of contributions (a bound on distinct targets)
  int64_t total = ncore;
  for (int64_t i = 0; i < ncore; ++i) {
    const int ka = __builtin_popcountll(ca[i]), kb = __builtin_popcountll(cb[i]);
    const int64_t sa = (int64_t)ka * (n - ka), sb = (int64_t)kb * (n - kb);
    total += sa + sb + sa * sb + binom64(ka, 2) * binom64(n - ka, 2) + binom64(kb, 2) * binom64(n - kb, 2);
  }
  ScopedBuffers<11> scratch(c);
  DeviceBuffer &bkeys = scratch.b[0], &bsum = scratch.b[1], &bhd = scratch.b[2], &bck = scratch.b[3],
               &bcs = scratch.b[4], &bcnt = scratch.b[5], &berr = scratch.b[6], &bcore = scratch.b[7],
               &bout = scratch.b[8], &bhist = scratch.b[9], &bhll = scratch.b[10];
  uint64_t* dcore = dev_array<uint64_t>(c, bcore, 3 * ncore);
  QDKGB_CUDA(cudaMemcpyAsync(dcore, ca, ncore * 8, cudaMemcpyHostToDevice, c->stream));
  QDKGB_CUDA(cudaMemcpyAsync(dcore + ncore, cb, ncore * 8, cudaMemcpyHostToDevice, c->stream));
  QDKGB_CUDA(cudaMemcpyAsync(dcore + 2 * ncore, cc, ncore * 8, cudaMemcpyHostToDevice, c->stream));
  int* err = dev_array<int>(c, berr, 1);
  unsigned long long* cnt = dev_array<unsigned long long>(c, bcnt, 2);
  QDKGB_CUDA(cudaMemsetAsync(cnt, 0, 2 * sizeof(unsigned long long), c->stream));
  CoreArgs A;
  A.I = integrals_view(c);
  A.n = n;
  A.ncore = ncore;
  A.ca = dcore;
  A.cb = dcore + ncore;
  A.cc = (const double*)(dcore + 2 * ncore);
  A.E0 = E0;
  A.h_el_tol = h_el_tol;
  A.just_singles = just_singles;
  // table: 2.5 x the estimated distinct targets (at most 1.5 x the
  // contributions); an overflowing enumeration is redone with twice the slots
  const double est = distinct_targets(c, A, dev_array<unsigned>(c, bhll, kHllRegs));
  const double want = std::min((double)(total + total / 2), 2.5 * est + 2. * (double)ncore) + 1024.;
  uint64_t cap = 1024;
  while ((double)cap < want) cap <<= 1;
  size_t freeb = 0, totb = 0;
  QDKGB_CUDA(cudaMemGetInfo(&freeb, &totb));
  const size_t slot_bytes = 16 + 16 + 8 + 16;  // key, fixed-point sum, hd, candidate key + slot
  if (cap * slot_bytes > freeb / 2) throw Error(QDKGB_ERR_OOM, "ASCI search: hash table does not fit in device memory");
  const unsigned eb = (unsigned)std::min<int64_t>((ncore + kAsciWarps - 1) / kAsciWarps, (int64_t)c->sm_count * 16);
  for (;;) {
    u128* keys = (u128*)dev_alloc(c, bkeys, cap * 16 + 256);
    keys = (u128*)(((uintptr_t)keys + 15) & ~(uintptr_t)15);
    A.T = Table{keys, dev_array<long long>(c, bsum, 2 * cap), dev_array<long long>(c, bhd, cap), cap - 1, err};
    const unsigned fb = (unsigned)std::min<uint64_t>((cap + 255) / 256, (uint64_t)c->sm_count * 64);
    QDKGB_CUDA(cudaMemsetAsync(err, 0, sizeof(int), c->stream));
    k_fill_empty<<<fb, 256, 0, c->stream>>>(A.T, cap);
    QDKGB_CHECK_LAUNCH();
    k_asci_enum<<<eb, kAsciWarps * 32, 0, c->stream>>>(A);
    QDKGB_CHECK_LAUNCH();
    int herr = 0;
    QDKGB_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    QDKGB_CUDA(cudaStreamSynchronize(c->stream));
    if (herr == 2) throw Error(QDKGB_ERR_UNSUPPORTED, "ASCI: a contribution |c H| >= 2^20 is outside the accumulator range");
    if (!herr) break;
    if ((cap << 1) * slot_bytes > freeb / 2) throw Error(QDKGB_ERR_OOM, "ASCI search: hash table overflow");
    cap <<= 1;
  }
  const unsigned fb = (unsigned)std::min<uint64_t>((cap + 255) / 256, (uint64_t)c->sm_count * 64);
  uint64_t* ckeys = dev_array<uint64_t>(c, bck, cap);
  uint64_t* cslots = dev_array<uint64_t>(c, bcs, cap);
  k_asci_extract<<<fb, 256, 0, c->stream>>>(A.T, cap, rv_prune_tol, ckeys, cslots, cnt);
  QDKGB_CHECK_LAUNCH();
  int herr = 0;
  unsigned long long ncand = 0;
  QDKGB_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  QDKGB_CUDA(cudaMemcpyAsync(&ncand, cnt, sizeof(ncand), cudaMemcpyDeviceToHost, c->stream));
  QDKGB_CUDA(cudaStreamSynchronize(c->stream));
  if (herr == 2) throw Error(QDKGB_ERR_UNSUPPORTED, "ASCI: a contribution |c H| >= 2^20 is outside the accumulator range");
  if (herr) throw Error(QDKGB_ERR_OOM, "ASCI search: hash table overflow");
  if (n_candidates) *n_candidates = (int64_t)ncand;
  const int64_t topk = ndets_max - ncore;
  uint64_t kth = 0;  // keep everything
  if (topk <= 0) {
    kth = ~0ull;  // keep nothing but the core
  } else if ((int64_t)ncand > topk) {
    // radix select of the topk-th largest key, digits from the top
    unsigned long long* hist = dev_array<unsigned long long>(c, bhist, 1 << kRadixBits);
    uint64_t prefix = 0, hi_mask = 0;
    int64_t k = topk;
    std::vector<unsigned long long> h(1 << kRadixBits);
    const unsigned hb = (unsigned)std::min<uint64_t>((ncand + 255) / 256, (uint64_t)c->sm_count * 32);
    for (int top = 64; top > 0;) {
      const int width = std::min(kRadixBits, top);
      const int shift = top - width;
      const int nb = 1 << width;
      QDKGB_CUDA(cudaMemsetAsync(hist, 0, nb * 8, c->stream));
      k_radix_hist<<<hb, 256, 0, c->stream>>>(ckeys, ncand, shift, width, prefix, hi_mask, hist);
      QDKGB_CHECK_LAUNCH();
      QDKGB_CUDA(cudaMemcpyAsync(h.data(), hist, nb * 8, cudaMemcpyDeviceToHost, c->stream));
      QDKGB_CUDA(cudaStreamSynchronize(c->stream));
      int64_t acc = 0;
      int d = nb - 1;
      for (; d >= 0; --d) {
        if (acc + (int64_t)h[d] >= k) break;
        acc += (int64_t)h[d];
      }
      if (d < 0) d = 0;
      k -= acc;
      prefix |= (uint64_t)d << shift;
      hi_mask |= ((uint64_t)nb - 1) << shift;
      top = shift;
    }
    kth = prefix;
  }
  uint64_t* dout = dev_array<uint64_t>(c, bout, 2 * std::max<uint64_t>(ncand, 1));
  QDKGB_CUDA(cudaMemsetAsync(cnt + 1, 0, sizeof(unsigned long long), c->stream));
  unsigned long long nsel = 0;
  if (ncand > 0 && kth != ~0ull) {
    const unsigned sb = (unsigned)std::min<uint64_t>((ncand + 255) / 256, (uint64_t)c->sm_count * 32);
    k_asci_select<<<sb, 256, 0, c->stream>>>(ckeys, cslots, ncand, kth, A.T, dout, dout + ncand, cnt + 1);
    QDKGB_CHECK_LAUNCH();
    QDKGB_CUDA(cudaMemcpyAsync(&nsel, cnt + 1, sizeof(nsel), cudaMemcpyDeviceToHost, c->stream));
    QDKGB_CUDA(cudaStreamSynchronize(c->stream));
  }
  out_a.resize(nsel + ncore);
  out_b.resize(nsel + ncore);
  if (nsel) {
    QDKGB_CUDA(cudaMemcpyAsync(out_a.data(), dout, nsel * 8, cudaMemcpyDeviceToHost, c->stream));
    QDKGB_CUDA(cudaMemcpyAsync(out_b.data(), dout + ncand, nsel * 8, cudaMemcpyDeviceToHost, c->stream));
  }
  QDKGB_CUDA(cudaStreamSynchronize(c->stream));
  std::copy(ca, ca + ncore, out_a.begin() + nsel);
  std::copy(cb, cb + ncore, out_b.begin() + nsel);
}

// asci_pt2_constraint (include/macis/asci/pt2.hpp:59-565) on the device:
// E_PT2 = sum over the determinants Q outside the wavefunction of
// (sum_P c_P <Q|H|P>)^2 / (E0 - H_QQ), single contributions with
// |c_P <Q|H|P>| < pt2_tol dropped (determinant_contributions.hpp:49-55,
// mask_constraints.hpp:400-670).  The enumeration of the search runs over the
// whole wavefunction (each determinant inserted with an infinite score, so
// that it drops out), into the hash table; the reference's constraint split
// (there for MPI / OpenMP balance and memory) becomes a split of the target
// space by a hash into passes when the table for every contribution would
// not fit in half of the free device memory.  Every Q lies in one part of
// either split, so the sums are the same.
double asci_pt2_gpu(Context* c, int64_t nd, const uint64_t* a, const uint64_t* b, const double* C, double E0,
                    double pt2_tol, int64_t max_slots, int64_t* npt2) {
  NvtxRange nvtx_range("qdkgb.asci_pt2");
  if (!c->have_ints) throw Error(QDKGB_ERR_STATE, "integrals not set");
  if (nd <= 0) throw Error(QDKGB_ERR_INVALID, "empty wavefunction");
  for (int64_t i = 1; i < nd; ++i)
    if (a[i] < a[i - 1] || (a[i] == a[i - 1] && b[i] < b[i - 1]))
      throw Error(QDKGB_ERR_INVALID, "PT2 Only Works with Sorted Wfns");
  const int n = c->norb;
  {
    uint64_t u = 0;
    for (int64_t i = 0; i < nd; ++i) u |= a[i] | b[i];
    if (n < 64 && (u >> n)) throw Error(QDKGB_ERR_INVALID, "a determinant occupies an orbital beyond the integrals' norb");
  }
  int64_t total = nd;
  for (int64_t i = 0; i < nd; ++i) {
    const int ka = __builtin_popcountll(a[i]), kb = __builtin_popcountll(b[i]);
    const int64_t sa = (int64_t)ka * (n - ka), sb = (int64_t)kb * (n - kb);
    total += sa + sb + sa * sb + binom64(ka, 2) * binom64(n - ka, 2) + binom64(kb, 2) * binom64(n - kb, 2);
  }
  ScopedBuffers<7> scratch(c);
  DeviceBuffer &bkeys = scratch.b[0], &bsum = scratch.b[1], &bhd = scratch.b[2], &berr = scratch.b[3],
               &bcore = scratch.b[4], &bpart = scratch.b[5], &bhll = scratch.b[6];
  uint64_t* dcore = dev_array<uint64_t>(c, bcore, 3 * nd);
  QDKGB_CUDA(cudaMemcpyAsync(dcore, a, nd * 8, cudaMemcpyHostToDevice, c->stream));
  QDKGB_CUDA(cudaMemcpyAsync(dcore + nd, b, nd * 8, cudaMemcpyHostToDevice, c->stream));
  QDKGB_CUDA(cudaMemcpyAsync(dcore + 2 * nd, C, nd * 8, cudaMemcpyHostToDevice, c->stream));
  int* err = dev_array<int>(c, berr, 1);
  CoreArgs A;
  A.I = integrals_view(c);
  A.n = n;
  A.ncore = nd;
  A.ca = dcore;
  A.cb = dcore + nd;
  A.cc = (const double*)(dcore + 2 * nd);
  A.E0 = E0;
  A.h_el_tol = pt2_tol;
  // table: 2.5 x the estimated distinct targets (at most 1.5 x the
  // contributions), split into passes when it exceeds half the free memory or
  // max_slots; a pass whose probing overflows is redone with twice the slots
  const double est = distinct_targets(c, A, dev_array<unsigned>(c, bhll, kHllRegs));
  const double want = std::min((double)(total + total / 2), 2.5 * est + 2. * (double)nd) + 1024.;
  uint64_t need = 1024;
  while ((double)need < want) need <<= 1;
  size_t freeb = 0, totb = 0;
  QDKGB_CUDA(cudaMemGetInfo(&freeb, &totb));
  const size_t slot_bytes = 16 + 16 + 8;  // key, fixed-point sum, E0 - H_QQ
  const size_t budget = freeb / 2;
  const uint64_t slot_max = max_slots > 0 ? std::max<uint64_t>((uint64_t)max_slots, 1024) : ~0ull;
  auto fits = [&](uint64_t cp) { return cp * slot_bytes <= budget && cp <= slot_max; };
  uint64_t cap = 1024;
  while (cap < need && fits(cap << 1)) cap <<= 1;
  const uint64_t npass = std::max<uint64_t>(1, (need + cap - 1) / cap);
  if (npass > 0xffffffffull) throw Error(QDKGB_ERR_OOM, "ASCI PT2: too many passes for the device memory");
  A.npass = (uint32_t)npass;
  const unsigned sb = (unsigned)std::min<uint64_t>((need + 255) / 256, (uint64_t)c->sm_count * 8);
  double* partial = (double*)dev_alloc(c, bpart, (size_t)sb * 16 + 64);
  unsigned long long* pcount = (unsigned long long*)(partial + sb);
  const unsigned eb = (unsigned)std::min<int64_t>((nd + kAsciWarps - 1) / kAsciWarps, (int64_t)c->sm_count * 16);
  std::vector<double> hp(sb);
  std::vector<unsigned long long> hc(sb);
  double ept2 = 0.;
  int64_t count = 0;
  for (uint64_t pass = 0; pass < npass; ++pass) {
    A.pass = (uint32_t)pass;
    for (;;) {
      u128* keys = (u128*)dev_alloc(c, bkeys, cap * 16 + 256);
      keys = (u128*)(((uintptr_t)keys + 15) & ~(uintptr_t)15);
      A.T = Table{keys, dev_array<long long>(c, bsum, 2 * cap), dev_array<long long>(c, bhd, cap), cap - 1, err};
      const unsigned fb = (unsigned)std::min<uint64_t>((cap + 255) / 256, (uint64_t)c->sm_count * 64);
      QDKGB_CUDA(cudaMemsetAsync(err, 0, sizeof(int), c->stream));
      k_fill_empty<<<fb, 256, 0, c->stream>>>(A.T, cap);
      QDKGB_CHECK_LAUNCH();
      k_asci_enum<<<eb, kAsciWarps * 32, 0, c->stream>>>(A);
      QDKGB_CHECK_LAUNCH();
      k_pt2_sum<<<sb, 256, 0, c->stream>>>(A.T, cap, partial, pcount);
      QDKGB_CHECK_LAUNCH();
      int herr = 0;
      QDKGB_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
      QDKGB_CUDA(cudaMemcpyAsync(hp.data(), partial, sb * 8, cudaMemcpyDeviceToHost, c->stream));
      QDKGB_CUDA(cudaMemcpyAsync(hc.data(), pcount, sb * 8, cudaMemcpyDeviceToHost, c->stream));
      QDKGB_CUDA(cudaStreamSynchronize(c->stream));
      if (herr == 2) throw Error(QDKGB_ERR_UNSUPPORTED, "ASCI: a contribution |c H| >= 2^20 is outside the accumulator range");
    if (!herr) break;
      if (!fits(cap << 1)) throw Error(QDKGB_ERR_OOM, "ASCI PT2: hash table overflow");
      cap <<= 1;
    }
    for (unsigned i = 0; i < sb; ++i) {
      ept2 += hp[i];
      count += (int64_t)hc[i];
    }
  }
  if (npt2) *npt2 = count;
  return ept2;
}

}  // namespace qdkgb

// ---------------------------------------------------------------- drivers
namespace qdkgb {

namespace {

struct HDet {
  uint64_t a, b;
};
inline bool hspin_less(const HDet& x, const HDet& y) { return x.a != y.a ? x.a < y.a : x.b < y.b; }
inline bool hdet_eq(const HDet& x, const HDet& y) { return x.a == y.a && x.b == y.b; }



// Wall time of the ASCI phases (synchronised: each phase ends in a host
// sync anyway), accumulated into Context::asci_phase_s.
struct PhaseClock {
  Context* c;
  std::chrono::steady_clock::time_point t;
  explicit PhaseClock(Context* ctx) : c(ctx) {
    QDKGB_CUDA(cudaStreamSynchronize(c->stream));
    t = std::chrono::steady_clock::now();
  }
  void lap(int phase) {
    QDKGB_CUDA(cudaStreamSynchronize(c->stream));
    const auto now = std::chrono::steady_clock::now();
    c->asci_phase_s[phase] += std::chrono::duration<double>(now - t).count();
    t = now;
  }
};

// The list the context's FP64 CSR was last built for, so that the next
// iteration patches that matrix instead of rebuilding it (asci_iter's
// incremental build, include/macis/solvers/incremental_h_build.hpp:38-356).
struct HPatchCache {
  std::vector<uint64_t> a, b;
  double thresh = 0.;
  bool valid = false;
};

bool patch_disabled() {
  const char* e = std::getenv("QDKGB_ASCI_FULL_BUILD");
  return e && e[0] && e[0] != '0';
}

// selected_ci_diag (selected_ci_diag.hpp:111-158) on the device for a list
// sorted by spin_comparator; X is the guess (empty: diagonal guess) and the
// eigenvector on return.  With a cache holding the previous list, the FP64
// CSR is patched from the previous one (bit-identical to a rebuild).
double sci_diag_gpu(Context* c, const qdkgb_asci_settings& S, const qdkgb_davidson_settings& ci, double matel_tol,
                    const std::vector<HDet>& dets, std::vector<double>& X, HPatchCache* cache) {
  const int64_t n = (int64_t)dets.size();
  std::vector<uint64_t> a(n), b(n);
  for (int64_t i = 0; i < n; ++i) {
    a[i] = dets[i].a;
    b[i] = dets[i].b;
  }
  const bool mixed = ci.precision == QDKGB_PREC_MIXED;
  // the previous CSR leaves the context before the determinant space is reset
  ScopedBuffers<3> old(c);
  const bool have_old = cache && cache->valid && !mixed && !patch_disabled() && c->H.valid && !c->op_direct &&
                        !c->H.structured && c->H.storage == QDKGB_H_FP64 && c->H.thresh == matel_tol &&
                        c->H.n == (int64_t)cache->a.size() && cache->thresh == matel_tol;
  if (have_old) {
    std::swap(old.b[0], c->H.rowptr);
    std::swap(old.b[1], c->H.colind);
    std::swap(old.b[2], c->H.val);
  }
  if (cache) cache->valid = false;
  PhaseClock clock(c);
  build_det_space(c, n, a.data(), b.data());
  clock.lap(1);
  bool patched = false;
  if (have_old && !c->fci)
    patched = build_hamiltonian_patched(c, matel_tol, cache->a, cache->b, old.b[0], old.b[1], old.b[2],
                                        S.min_patch_overlap);
  for (DeviceBuffer& x : old.b) dev_free(c, x);
  if (patched)
    ++c->asci_patches;
  else
    build_hamiltonian(c, matel_tol, mixed ? QDKGB_H_SPLIT32 : QDKGB_H_FP64);
  clock.lap(2);
  if (cache && !mixed) {
    cache->a.swap(a);
    cache->b.swap(b);
    cache->thresh = matel_tol;
    cache->valid = true;
  }
  qdkgb_davidson_settings s = ci;
  s.nroots = 1;  // the ASCI iterations solve for the lowest root, as the reference's do
  s.use_guess = X.empty() ? 0 : 1;
  X.resize(n, 0.);
  if (!s.use_guess) std::fill(X.begin(), X.end(), 0.);
  double E = 0.;
  davidson(c, &s, &E, X.data(), nullptr);
  clock.lap(3);
  return E;
}

// asci_iter (include/macis/asci/iteration.hpp:50-226)
double asci_iter_gpu(Context* c, const qdkgb_asci_settings& S, const qdkgb_davidson_settings& ci, double matel_tol,
                     int64_t ndets_max, double E0, std::vector<HDet>& wfn, std::vector<double>& X, int64_t* ncand,
                     HPatchCache* cache) {
  NvtxRange nvtx_range("qdkgb.asci_iter");
  ++c->asci_iters;
  // the list and vector in spin order, for the warm start's merge scan (the
  // list arrives in that order from the previous iteration)
  std::vector<HDet> sorted_wfn;
  std::vector<double> sorted_X;
  if (S.warm_start) {
    if (std::is_sorted(wfn.begin(), wfn.end(), hspin_less)) {
      sorted_wfn = wfn;
      sorted_X = X;
    } else {
      struct DC {
        HDet d;
        double c;
      };
      std::vector<DC> v(wfn.size());
      for (size_t i = 0; i < v.size(); ++i) v[i] = {wfn[i], X[i]};
      parallel_sort(v, [](const DC& x, const DC& y) { return hspin_less(x.d, y.d); });
      sorted_wfn.resize(v.size());
      sorted_X.resize(v.size());
      for (size_t i = 0; i < v.size(); ++i) {
        sorted_wfn[i] = v[i].d;
        sorted_X[i] = v[i].c;
      }
    }
  }
  if (wfn.size() > 1) {
    // reorder_ci_on_coeff (determinant_sort.hpp:45-64): std::sort of the
    // indices by |C| descending.  The (|C|, index) pairs go through the same
    // std::sort with the same comparisons, so ties come out in the
    // reference's order; the pairs sit together in memory.
    struct KI {
      double k;
      size_t i;
    };
    std::vector<KI> idx(wfn.size());
    for (size_t i = 0; i < idx.size(); ++i) idx[i] = {std::fabs(X[i]), i};
    std::sort(idx.begin(), idx.end(), [](const KI& x, const KI& y) { return x.k > y.k; });
    std::vector<HDet> w2(wfn.size());
    std::vector<double> x2(wfn.size());
    for (size_t i = 0; i < idx.size(); ++i) {
      w2[i] = wfn[idx[i].i];
      x2[i] = X[idx[i].i];
    }
    wfn.swap(w2);
    X.swap(x2);
  }
  size_t nkeep = 0;
  if (S.core_selection_fixed) {
    nkeep = std::min<size_t>((size_t)S.ncdets_max, wfn.size());
  } else {
    if (!(S.core_selection_threshold >= 2.220446049250313e-16 && S.core_selection_threshold <= 1.0))
      throw Error(QDKGB_ERR_INVALID, "core_selection_threshold must be in [epsilon, 1.0]");
    double w = 0.;
    for (size_t i = 0; i < wfn.size(); ++i) {
      w += X[i] * X[i];
      nkeep++;
      if (w >= S.core_selection_threshold) break;
    }
  }
  if (wfn.size() > 1) {  // reorder_ci_on_alpha of the core (determinant_sort.hpp:66-90)
    std::vector<size_t> idx(nkeep);
    for (size_t i = 0; i < nkeep; ++i) idx[i] = i;
    std::sort(idx.begin(), idx.end(), [&](size_t i, size_t j) { return hspin_less(wfn[i], wfn[j]); });
    std::vector<HDet> w2(nkeep);
    std::vector<double> x2(nkeep);
    for (size_t i = 0; i < nkeep; ++i) {
      w2[i] = wfn[idx[i]];
      x2[i] = X[idx[i]];
    }
    std::copy(w2.begin(), w2.end(), wfn.begin());
    std::copy(x2.begin(), x2.end(), X.begin());
  }
  std::vector<uint64_t> ca(nkeep), cb(nkeep);
  for (size_t i = 0; i < nkeep; ++i) {
    ca[i] = wfn[i].a;
    cb[i] = wfn[i].b;
  }
  std::vector<uint64_t> na, nb;
  {
    PhaseClock clock(c);
    asci_search_gpu(c, (int64_t)nkeep, ca.data(), cb.data(), X.data(), E0, ndets_max, S.h_el_tol, S.rv_prune_tol,
                    na, nb, ncand, S.just_singles != 0);
    clock.lap(0);
  }
  wfn.resize(na.size());
  for (size_t i = 0; i < na.size(); ++i) wfn[i] = {na[i], nb[i]};
  parallel_sort(wfn, hspin_less);
  std::vector<double> Xl;
  if (S.warm_start) {
    Xl.assign(wfn.size(), 0.);
    for (size_t i = 0, k = 0; i < wfn.size() && k < sorted_wfn.size();) {
      if (hspin_less(sorted_wfn[k], wfn[i])) {
        ++k;
      } else if (hspin_less(wfn[i], sorted_wfn[k])) {
        ++i;
      } else {
        Xl[i++] = sorted_X[k++];
      }
    }
    double nrm = 0.;
    for (double x : Xl) nrm += x * x;
    nrm = std::sqrt(nrm);
    if (nrm < std::max(S.min_warm_start_overlap, 2.220446049250313e-16))
      Xl.clear();
    else
      for (double& x : Xl) x /= nrm;
  }
  const double E = sci_diag_gpu(c, S, ci, matel_tol, wfn, Xl, cache);
  X = Xl;
  return E;
}

}  // namespace

void asci_run(Context* c, const qdkgb_asci_settings& S, const qdkgb_davidson_settings& ci, double matel_tol,
              std::vector<uint64_t>& a, std::vector<uint64_t>& b, std::vector<double>& X, double& E0, bool grow,
              bool refine, double* E_grow) {
  // the growth settings as get_asci_settings_ checks them
  // (cpp/src/qdk/chemistry/algorithms/microsoft/macis_base.cpp:101-124)
  if (!(S.grow_factor > 1.0)) throw Error(QDKGB_ERR_INVALID, "grow_factor must be > 1.0");
  if (!(S.min_grow_factor > 1.0)) throw Error(QDKGB_ERR_INVALID, "min_grow_factor must be > 1.0");
  if (S.min_grow_factor > S.grow_factor) throw Error(QDKGB_ERR_INVALID, "min_grow_factor must be <= grow_factor");
  if (!(S.growth_backoff_rate > 0.0 && S.growth_backoff_rate < 1.0))
    throw Error(QDKGB_ERR_INVALID, "growth_backoff_rate must be in (0, 1)");
  if (!(S.growth_recovery_rate > 1.0)) throw Error(QDKGB_ERR_INVALID, "growth_recovery_rate must be > 1.0");
  for (double& t : c->asci_phase_s) t = 0.;
  c->asci_iters = 0;
  c->asci_patches = 0;
  c->asci_rot.clear();
  HPatchCache cache;
  std::vector<HDet> wfn(a.size());
  for (size_t i = 0; i < a.size(); ++i) wfn[i] = {a[i], b[i]};
  int64_t ncand = 0;
  if (grow) {
    // asci_grow (include/macis/asci/grow.hpp:45-268), without rotations
    size_t prev = wfn.size();
    double gf = S.grow_factor;
    while ((int64_t)wfn.size() < S.ntdets_max) {
      // taper (grow.hpp:97-107): a step that would pass ntdets_max at the
      // current factor uses max(min_grow_factor, taper_grow_factor) instead
      double eff = gf;
      if (S.taper_grow_factor > 0. && (int64_t)std::ceil((double)wfn.size() * gf) > S.ntdets_max)
        eff = std::max(S.min_grow_factor, S.taper_grow_factor);
      int64_t nnew = std::min<int64_t>(
          std::max<int64_t>(S.ntdets_min, (int64_t)std::ceil((double)wfn.size() * eff)), S.ntdets_max);
      if (nnew <= (int64_t)wfn.size()) {
        nnew = std::min<int64_t>((int64_t)wfn.size() + 1, S.ntdets_max);
        if (nnew <= (int64_t)wfn.size()) break;
      }
      const double E = asci_iter_gpu(c, S, ci, matel_tol, nnew, E0, wfn, X, &ncand, &cache);
      if ((int64_t)wfn.size() < nnew) {
        gf = std::max(S.min_grow_factor, gf * S.growth_backoff_rate);
        if (wfn.size() <= prev) break;
      } else {
        gf = std::min(S.grow_factor, gf * S.growth_recovery_rate);
      }
      prev = wfn.size();
      if (S.grow_with_rot && (int64_t)wfn.size() >= S.rot_size_start) {
        // natural-orbital rotation (grow.hpp:163-252): the spin-summed 1-RDM
        // of the current wavefunction (the context holds its list), its
        // natural orbitals, the integrals rotated to them, and the list
        // rediagonalised from the diagonal guess in the new orbitals (the
        // iteration's energy is kept, as the reference keeps it)
        const int n = c->norb;
        std::vector<double> aa((size_t)n * n, 0.), bb((size_t)n * n, 0.), ordm((size_t)n * n), U;
        rdms_spin_dep(c, X.data(), aa.data(), bb.data(), nullptr, nullptr, nullptr);
        for (size_t i = 0; i < ordm.size(); ++i) ordm[i] = aa[i] + bb[i];
        natural_orbitals(n, ordm, U);
        rotate_integrals(c, U);
        if (c->asci_rot.empty()) {
          c->asci_rot = U;
        } else {
          std::vector<double> R((size_t)n * n, 0.);
          for (int j = 0; j < n; ++j)
            for (int k = 0; k < n; ++k) {
              const double u = U[k + (size_t)n * j];
              for (int i = 0; i < n; ++i) R[i + (size_t)n * j] += c->asci_rot[i + (size_t)n * k] * u;
            }
          c->asci_rot.swap(R);
        }
        cache.valid = false;  // the integrals changed
        std::vector<double> Xr;
        sci_diag_gpu(c, S, ci, matel_tol, wfn, Xr, nullptr);
        X.swap(Xr);
      }
      E0 = E;
    }
  }
  if (E_grow) *E_grow = E0;
  if (refine) {
    // asci_refine (include/macis/asci/refine.hpp:44-237)
    int64_t ndets = (int64_t)wfn.size();
    bool converged = false;
    double prev_dE = 0.;
    int osc = 0;
    int64_t max_iter = S.max_refine_iter, ext = 0;
    std::vector<HDet> prev_wfn;
    for (int64_t iter = 0; iter < max_iter; ++iter) {
      const double E = asci_iter_gpu(c, S, ci, matel_tol, ndets, E0, wfn, X, &ncand, &cache);
      if ((int64_t)wfn.size() != ndets) {
        ndets = (int64_t)wfn.size();
        if (ndets < S.ntdets_min) break;
      }
      const double dE = E - E0;
      if (std::fabs(dE) < S.refine_energy_tol) {
        E0 = E;
        converged = true;
        break;
      }
      if (iter > 0 && prev_dE * dE < 0 && std::fabs(prev_dE + dE) < S.refine_energy_tol) {
        osc++;
        if (osc >= 2 && !prev_wfn.empty()) {
          std::vector<HDet> uni;
          std::set_union(prev_wfn.begin(), prev_wfn.end(), wfn.begin(), wfn.end(), std::back_inserter(uni),
                         hspin_less);
          std::vector<double> Xu(uni.size(), 0.);
          for (size_t i = 0; i < wfn.size(); ++i) {
            auto it = std::lower_bound(uni.begin(), uni.end(), wfn[i], hspin_less);
            if (it != uni.end() && hdet_eq(*it, wfn[i])) Xu[it - uni.begin()] = X[i];
          }
          const double Eu = sci_diag_gpu(c, S, ci, matel_tol, uni, Xu, &cache);
          const int64_t e = std::min<int64_t>(osc, S.max_refine_iter - ext);
          if (e > 0) {
            max_iter += e;
            ext += e;
          }
          wfn = uni;
          X = Xu;
          ndets = (int64_t)wfn.size();
          E0 = Eu;
          prev_wfn.clear();
          osc = 0;
          prev_dE = 0.;
          continue;
        }
      } else {
        osc = 0;
      }
      prev_dE = dE;
      prev_wfn = wfn;
      E0 = E;
    }
    if (!converged) throw Error(QDKGB_ERR_NOT_CONVERGED, "ASCI Refine did not converge");
  }
  a.resize(wfn.size());
  b.resize(wfn.size());
  for (size_t i = 0; i < wfn.size(); ++i) {
    a[i] = wfn[i].a;
    b[i] = wfn[i].b;
  }
}

}  // namespace qdkgb
