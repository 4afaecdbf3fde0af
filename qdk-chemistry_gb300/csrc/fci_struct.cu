// Slab kernels for complete (CAS) determinant spaces.
//
// In a full (n_alpha, n_beta) product space every row has the same shape: the
// row of determinant r = g * N_b + b (alpha group g, beta string b) holds, in
// ascending column order, one block per alpha group h within a double
// excitation of g - the beta strings within level 2 of b for h = g, within
// level 1 for an alpha single, b alone for an alpha double.  The sequence of
// blocks depends on g only, so a row position p names the same (h, beta-list
// entry) for every b of the group.
//
// Slab layout: the Hamiltonian of such a space is stored values-only as
//     value(g, p, b) at ((g * rowlen + p) * N_b + b),
// beta string fastest.  A thread owns one row (one b) of a group and walks the
// positions: the per-position descriptor is warp-uniform, the value and
// beta-list loads are coalesced, and the x of the own group and of the alpha
// singles (the blocks of the position range a CTA covers) is staged in shared
// memory, so each element costs one streamed value, one cached list entry, one
// shared-memory gather and an FMA.  Elements dropped by the threshold are
// stored as zero (the operator is unchanged); the CSR arrays the reference
// defines are produced from the slab on request (export), or in place of it
// when most elements are dropped.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <type_traits>
#include <vector>

#include "common.cuh"
#include "internal.h"
#include "slab_sigma.cuh"

namespace qdkgb {

constexpr int kListAlphaDouble = 2047;       // beta-list index meaning "b itself"
constexpr size_t kSlabSmemMax = 110 * 1024;  // staged x + segment record per CTA (two CTAs per SM)
constexpr size_t kSlabPlanMax[2] = {32 * 1024, kSlabSmemMax};  // per plan: 4-byte (FP32) x, 8-byte x
constexpr int kSlabVecThreads = 256;         // vectorised FP32 sigma: CTA size at most
constexpr int kSlabThreads = 512;            // sigma CTA size at most; a group's beta strings are split
                                             // over ceil(Nb / 512) CTAs (grid.z)
constexpr int kEmitSegments = 4;             // position ranges per group in emission / export
constexpr int kSigma32Kernels = 4;           // FP32 sigma kernels the autotuner chooses from

// Sigma work split for one staged-x element size: CTA per (group, segment);
// a segment is a run of whole row items (the own-group block, alpha-single
// blocks, alpha-double elements).  Per (g, s) a record of R int32:
//   [0] own-group block present, [1] its offset p * Nb, [2] its slot * Nb,
//   [3] n1b, then n1b pairs (p_e * Nb, slot_e * Nb) of alpha-single blocks,
//   then nd and one pad word, then nd pairs (p_j * Nb, h_j * Nb) of alpha
//   doubles,
// and segh[g][s][0..M) the alpha group whose x slice each slot holds.
struct SlabPlan {
  int S = 0, M = 0, R = 0;
  DeviceBuffer rec, segh;
};

struct PlanHost {
  int S = 0, M = 0, R = 0;
  std::vector<int32_t> rec, segh;
};

struct FciStruct {
  int64_t G = 0, Nb = 0;
  int n1 = 0, n2 = 0;  // beta list lengths (level <= 1, level <= 2), uniform
  int rowlen = 0;      // n2 + c1 * n1 + c2
  DeviceBuffer blT;    // [n2 + n1][Nb] int32: entry k of b's level-2 list, then of its level-1 list
  DeviceBuffer gdesc;  // [G][rowlen] h << 11 | list entry (kListAlphaDouble: b itself)
  SlabPlan plan[2];    // staged x of 4 bytes (FP32) / 8 bytes (FP64, split pair)
  DeviceBuffer ypart;  // [S][n] partial sums (S > 1)
  // segment-count autotuner: candidate plans (host) until the first
  // single-instance sigma of each plan times them and keeps the fastest;
  // then the record of that choice: (S, mean ms) per candidate
  std::vector<PlanHost> cand[2];
  bool tuned[2] = {false, false};
  std::vector<std::pair<int, double>> tune_ms[2];
  // FP32 sigma kernel in use: 0 register-fed (k_slab_sigma32v, four
  // positions in flight per thread), 1 TMA-fed (k_slab_sigma32t), 2 and 3
  // register-fed with eight and sixteen positions in flight; the autotuner
  // times them per candidate plan (tune_kernel_ms[k][i]: kernel k, plan i,
  // NaN where not eligible)
  int kernel32 = 0;
  std::vector<double> tune_kernel_ms[kSigma32Kernels];
  // spin-pair tables of the table-driven emission (rebuilt with every build)
  DeviceBuffer tab_b, tab_bm, tab_a, tab_am;
};

void free_struct(Context* c) {
  if (!c->fci) return;
  for (DeviceBuffer* b : {&c->fci->blT, &c->fci->gdesc, &c->fci->plan[0].rec, &c->fci->plan[0].segh,
                          &c->fci->plan[1].rec, &c->fci->plan[1].segh, &c->fci->ypart, &c->fci->tab_b,
                          &c->fci->tab_bm, &c->fci->tab_a, &c->fci->tab_am})
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
  if (G * Nb != D.ndets || G < 1 || G >= (1 << 20)) return;
  for (int64_t g = 0; g < G; ++g) {
    if (D.h_gstart[g + 1] - D.h_gstart[g] != Nb) return;
    if (D.h_galpha[g] == 0) return;
  }
  std::vector<int64_t> b1p(Nb + 1), b2p(Nb + 1);
  QDKGB_CUDA(cudaMemcpy(b1p.data(), D.b1_ptr.ptr, (Nb + 1) * 8, cudaMemcpyDeviceToHost));
  QDKGB_CUDA(cudaMemcpy(b2p.data(), D.b2_ptr.ptr, (Nb + 1) * 8, cudaMemcpyDeviceToHost));
  const int64_t n1 = b1p[1] - b1p[0], n2 = b2p[1] - b2p[0];
  if (n1 + n2 >= kListAlphaDouble) return;
  for (int64_t b = 0; b < Nb; ++b)
    if (b1p[b + 1] - b1p[b] != n1 || b2p[b + 1] - b2p[b] != n2) return;
  // one staged block must fit the shared-memory budget
  if ((size_t)Nb * 8 > kSlabSmemMax / 2) return;
  std::vector<int64_t> ap(G + 1);
  QDKGB_CUDA(cudaMemcpy(ap.data(), D.acon_ptr.ptr, (G + 1) * 8, cudaMemcpyDeviceToHost));
  std::vector<int32_t> aidx(ap[G]);
  std::vector<int8_t> alvl(ap[G]);
  if (ap[G]) {
    QDKGB_CUDA(cudaMemcpy(aidx.data(), D.acon_idx.ptr, ap[G] * 4, cudaMemcpyDeviceToHost));
    QDKGB_CUDA(cudaMemcpy(alvl.data(), D.acon_lvl.ptr, ap[G], cudaMemcpyDeviceToHost));
  }
  // descriptors in row order; per position the staged block it belongs to
  // (index of the own-group / alpha-single block in the row, -1 for an
  // alpha double)
  int rowlen = -1, c1 = -1, c2 = -1;
  PlanHost plan_tmp[2];
  std::vector<PlanHost> cand_tmp[2];
  std::vector<uint32_t> gdesc;
  std::vector<int32_t> pblock;  // [G][rowlen]
  {
    const size_t guess = (size_t)G * (size_t)(n2 + (ap[1] - ap[0]) * std::max<int64_t>(n1, 1));
    if (guess < ((size_t)1 << 31)) {
      gdesc.reserve(guess);
      pblock.reserve(guess);
    }
  }
  for (int64_t g = 0; g < G; ++g) {
    const size_t row0 = gdesc.size();
    int k0 = 0, k1 = 0, k2 = 0, nb = 0;
    for (int64_t e = ap[g]; e < ap[g + 1]; ++e) {
      const uint32_t h = (uint32_t)aidx[e];
      if (alvl[e] == 0) {
        if (aidx[e] != g) return;  // repeated alpha string
        for (int64_t k = 0; k < n2; ++k) {
          gdesc.push_back((h << 11) | (uint32_t)k);
          pblock.push_back(nb);
        }
        ++nb;
        ++k0;
      } else if (alvl[e] == 1) {
        for (int64_t k = 0; k < n1; ++k) {
          gdesc.push_back((h << 11) | (uint32_t)(n2 + k));
          pblock.push_back(nb);
        }
        ++nb;
        ++k1;
      } else {
        gdesc.push_back((h << 11) | (uint32_t)kListAlphaDouble);
        pblock.push_back(-1);
        ++k2;
      }
    }
    if (k0 != 1) return;
    if (rowlen < 0) {
      rowlen = (int)(gdesc.size() - row0);
      c1 = k1;
      c2 = k2;
      if ((int64_t)rowlen * G * 4 > ((int64_t)1 << 30)) return;  // tables above 1 GiB
    }
    if (k1 != c1 || k2 != c2 || (int)(gdesc.size() - row0) != rowlen) return;
  }
  if (n2 + (int64_t)c1 * n1 + c2 != rowlen) return;
  if ((int64_t)rowlen * Nb >= INT32_MAX) return;  // int32 slab offsets within a group
  // row items of every group: (first position, length, alpha group)
  struct Item {
    int p, len, h;
  };
  std::vector<Item> items;
  std::vector<int> item0(G + 1, 0);
  for (int64_t g = 0; g < G; ++g) {
    int p = 0;
    while (p < rowlen) {
      const size_t i = (size_t)g * rowlen + p;
      const int bk = pblock[i];
      int len = 1;
      if (bk >= 0)
        while (p + len < rowlen && pblock[i + len] == bk) ++len;
      items.push_back({p, bk >= 0 ? len : 0, (int)(gdesc[i] >> 11)});  // len 0: alpha double
      p += len;
    }
    item0[g + 1] = (int)items.size();
  }
  auto seg_of = [&](const Item& it, int S) {
    const int len = std::max(it.len, 1);
    return std::min(S - 1, (int)(((int64_t)(2 * it.p + len) * S) / (2 * (int64_t)rowlen)));
  };
  // staged blocks (M) and record length (R) per segment count; segments are
  // runs of items in row order, so one pass per group counts them
  constexpr int kMaxS = 16;
  int shapeM[kMaxS + 1], shapeR[kMaxS + 1];
  for (int S = 1; S <= kMaxS && S <= rowlen; ++S) {
    int M = 1, R = 6;
    for (int64_t g = 0; g < G; ++g) {
      int cur = -1, nb = 0, ndd = 0;
      for (int i = item0[g]; i <= item0[g + 1]; ++i) {
        const int sg = i < item0[g + 1] ? seg_of(items[i], S) : S;
        if (sg != cur) {
          M = std::max(M, nb);
          R = std::max(R, 6 + 2 * (nb + ndd));
          cur = sg;
          nb = ndd = 0;
        }
        if (i < item0[g + 1]) (items[i].len ? nb : ndd) += 1;
      }
    }
    shapeM[S] = M;
    shapeR[S] = R;
  }
  // per plan: the segment count that fits the budget and fills the SMs best
  std::vector<int32_t> dd;
  for (int pl = 0; pl < 2; ++pl) {
    const size_t xsize = pl == 0 ? 4 : 8;
    auto smem_of = [&](int M, int R) { return (size_t)M * Nb * xsize + ((size_t)R * 4 + 15) / 16 * 16; };
    int best_S = -1;
    double best = -1.;
    // CTA shape of the sigma that uses the plan (the FP32 one is vectorised
    // over 4 or 2 beta strings when Nb allows)
    const int vec = pl == 0 ? (Nb % 4 == 0 ? 4 : (Nb % 2 == 0 ? 2 : 1)) : 1;
    int bz, threads;
    if (vec > 1) {
      const int nvec = (int)(Nb / vec);
      threads = std::min(kSlabVecThreads, (nvec + 31) / 32 * 32);
      bz = (nvec + threads - 1) / threads;
    } else {
      bz = (int)((Nb + kSlabThreads - 1) / kSlabThreads);
      threads = (int)(((Nb + bz - 1) / bz + 31) / 32 * 32);
    }
    std::vector<int> feasible;
    for (int S = 1; S <= kMaxS && S <= rowlen; ++S) {
      const int M = shapeM[S], R = shapeR[S];
      const size_t sm = smem_of(M, R);
      if (sm > kSlabPlanMax[pl]) continue;
      feasible.push_back(S);
      // resident CTAs per SM: threads, 64 registers per thread, shared memory
      const int64_t per_sm = std::max<int64_t>(
          1, std::min<int64_t>(std::min<int64_t>(2048 / threads, 65536 / (64 * threads)), (227 * 1024) / (int64_t)sm));
      const int64_t slots = per_sm * c->sm_count, n_items = G * S * bz;
      const double eff = (double)n_items / (double)(((n_items + slots - 1) / slots) * slots);
      const double score = eff - 0.01 * S;
      if (score > best) {
        best = score;
        best_S = S;
      }
    }
    if (best_S < 0) return;
    // the occupancy model's choice first, then the other feasible counts of
    // at least 4 segments (fewer leave most SMs idle for these row counts)
    std::vector<int> cands{best_S};
    for (int S : feasible)
      if (S != best_S && S >= std::min(4, best_S)) cands.push_back(S);
    for (int S : cands) {
      const int M = shapeM[S], R = shapeR[S];
      std::vector<int32_t> rec((size_t)G * S * R, 0), segh((size_t)G * S * M, -1);
      for (int64_t g = 0; g < G; ++g) {
        int cur = -1, nslot = 0, nb1 = 0;
        int32_t* r = nullptr;
        auto close = [&]() {
          if (!r) return;
          r[3] = nb1;
          r[4 + 2 * nb1] = (int32_t)(dd.size() / 2);
          std::copy(dd.begin(), dd.end(), r + 6 + 2 * nb1);
        };
        for (int i = item0[g]; i < item0[g + 1]; ++i) {
          const Item& it = items[i];
          const int sg = seg_of(it, S);
          if (sg != cur) {
            close();
            cur = sg;
            r = &rec[((size_t)g * S + sg) * R];
            nslot = nb1 = 0;
            dd.clear();
          }
          if (it.len == 0) {
            dd.push_back((int32_t)(it.p * Nb));
            dd.push_back((int32_t)(it.h * Nb));
            continue;
          }
          const int slot = nslot++;
          segh[((size_t)g * S + sg) * M + slot] = it.h;
          if (it.h == g) {
            r[0] = 1;
            r[1] = (int32_t)(it.p * Nb);
            r[2] = (int32_t)(slot * Nb);
          } else {
            r[4 + 2 * nb1] = (int32_t)(it.p * Nb);
            r[5 + 2 * nb1] = (int32_t)(slot * Nb);
            ++nb1;
          }
        }
        close();
      }
      PlanHost ph;
      ph.S = S;
      ph.M = M;
      ph.R = R;
      ph.rec = std::move(rec);
      ph.segh = std::move(segh);
      if (S == best_S) plan_tmp[pl] = ph;
      cand_tmp[pl].push_back(std::move(ph));
    }
  }
  // transposed beta lists
  std::vector<int32_t> b1(Nb * n1), b2(Nb * n2), blT((n1 + n2) * Nb);
  QDKGB_CUDA(cudaMemcpy(b1.data(), D.b1_idx.ptr, b1.size() * 4, cudaMemcpyDeviceToHost));
  QDKGB_CUDA(cudaMemcpy(b2.data(), D.b2_idx.ptr, b2.size() * 4, cudaMemcpyDeviceToHost));
  for (int64_t b = 0; b < Nb; ++b) {
    for (int64_t k = 0; k < n2; ++k) blT[k * Nb + b] = b2[b * n2 + k];
    for (int64_t k = 0; k < n1; ++k) blT[(n2 + k) * Nb + b] = b1[b * n1 + k];
  }
  FciStruct* F = new FciStruct();
  F->G = G;
  F->Nb = Nb;
  F->n1 = (int)n1;
  F->n2 = (int)n2;
  F->rowlen = rowlen;
  auto up = [&](DeviceBuffer& buf, const void* src, size_t bytes) {
    void* p = dev_alloc(c, buf, std::max<size_t>(bytes, 4) + 16);
    if (bytes) QDKGB_CUDA(cudaMemcpy(p, src, bytes, cudaMemcpyHostToDevice));
  };
  up(F->blT, blT.data(), blT.size() * 4);
  up(F->gdesc, gdesc.data(), gdesc.size() * 4);
  for (int pl = 0; pl < 2; ++pl) {
    F->plan[pl].S = plan_tmp[pl].S;
    F->plan[pl].M = plan_tmp[pl].M;
    F->plan[pl].R = plan_tmp[pl].R;
    up(F->plan[pl].rec, plan_tmp[pl].rec.data(), plan_tmp[pl].rec.size() * 4);
    up(F->plan[pl].segh, plan_tmp[pl].segh.data(), plan_tmp[pl].segh.size() * 4);
    F->cand[pl] = std::move(cand_tmp[pl]);
    F->tuned[pl] = F->cand[pl].size() <= 1;
  }
  c->fci = F;
}

SlabArgs slab_args(Context* c) {
  FciStruct* F = c->fci;
  SlabArgs a;
  a.G = (int)F->G;
  a.Nb = (int)F->Nb;
  a.rowlen = F->rowlen;
  a.n1 = F->n1;
  a.n2 = F->n2;
  a.seglen = (F->rowlen + kEmitSegments - 1) / kEmitSegments;
  a.blT = (const int32_t*)F->blT.ptr;
  a.gdesc = (const uint32_t*)F->gdesc.ptr;
  return a;
}

PlanArgs slab_plan_args(Context* c, int pl) {
  const SlabPlan& PL = c->fci->plan[pl];
  return PlanArgs{PL.S, PL.M, PL.R, (const int32_t*)PL.rec.ptr, (const int32_t*)PL.segh.ptr};
}

size_t slab_plan_smem(Context* c, int pl, size_t x_bytes) {
  const SlabPlan& PL = c->fci->plan[pl];
  return (size_t)PL.M * c->fci->Nb * x_bytes + ((size_t)PL.R * 4 + 15) / 16 * 16;
}

namespace {

// CTA size and beta-range split of a group: bz CTAs of slab_threads each
unsigned slab_bz(int Nb) { return (unsigned)((Nb + kSlabThreads - 1) / kSlabThreads); }
unsigned slab_threads(int Nb) {
  const int bz = (int)slab_bz(Nb);
  return (unsigned)(((Nb + bz - 1) / bz + 31) / 32 * 32);
}

// ------------------------------------------------------------------ emission
// CTA per (group, segment), a thread per beta string, positions in order
// (k_slab_emit_tab below).  Every element is written (zero when dropped);
// kept counts go to kept[r].  kSlabF64F32: the single-instance layout of
// QDKGB_H_SPLIT32 storage (FP64 values and their FP32 rounding, one FP64-pipe
// conversion per element instead of the four of the hi/lo split; the
// full-precision sigma then runs on the FP64 values).
constexpr int kEmitThreads = 256;
constexpr int kSlabF64F32 = 2;

// ------------------------------------------------------------------ emission from spin-pair tables
// The build (single instance or a batch) emits the reference's values bit for
// bit with few FP64 operations per element, by evaluating once per string
// pair what the reference's element formulas compute from one spin's strings
// alone, in the same summation order:
//   * a single excitation of one spin (matrix_element_2,
//     matrix_elements.hpp:169-189) is h = T(v,o) + sum_{p in bra, same spin}
//     G_red(p,v,o) + sum_{p in bra, other spin} V_red(p,v,o); its first two
//     terms depend only on the excited spin's (bra, ket) pair, so the table
//     holds that partial sum and the element adds the other spin's terms
//     (6 additions at CAS(12,12) instead of 13);
//   * a same-spin double (matrix_element_4, :113-121) depends only on that
//     spin's pair: the table holds the value;
//   * an opposite-spin double (matrix_element_22, :140-151) is a signed
//     integral gather, done from the tables' orbital indices and signs.
// Which determinant is the bra follows the CSR build (the lower index), so
// the tables are oriented per pair.  Tables: per (beta list entry k, beta
// string b) for the beta pairs, per (alpha group g, row position p) for the
// alpha pairs; metadata v | o << 8 | neg << 16 | kind << 24.
namespace {
constexpr uint32_t kPairSingle = 1u << 24, kPairDouble = 2u << 24;

__device__ __forceinline__ double single_partial(const Integrals& I, uint64_t bra, const SingleEx& s) {
  const size_t n = (size_t)I.n;
  double h = ld(I.T + s.v + n * s.o);
  const double* g = I.G_red + n * (s.v + n * s.o);
  for (uint64_t m = bra; m; m &= m - 1) h += ld(g + low_bit(m));
  return h;
}

// beta pairs: own-group entries (k < n2) oriented by the beta index (the
// same group); level-1 entries (alpha-single blocks) unoriented: the orbital
// only in b, the one only in bc, and the sign (equal in both orientations).
// Batches: instance blockIdx.y with the integrals Iinst[blockIdx.y] and its
// own table (tot entries apart).
__global__ void k_emit_beta_table(SlabArgs A, Integrals I0, const Integrals* __restrict__ Iinst,
                                  const uint64_t* __restrict__ ubeta, double* __restrict__ bt,
                                  uint32_t* __restrict__ bm) {
  const int64_t tot = (int64_t)(A.n2 + A.n1) * A.Nb;
  const Integrals I = Iinst ? Iinst[blockIdx.y] : I0;
  bt += blockIdx.y * tot;
  bm += blockIdx.y * tot;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < tot; t += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(t / A.Nb), b = (int)(t - (int64_t)k * A.Nb);
    const int bc = __ldg(A.blT + t);
    uint32_t meta = 0;
    double val = 0.;
    if (bc != b) {
      const uint64_t rb = ubeta[b], rc = ubeta[bc];
      const uint64_t ex = rb ^ rc;
      if (k < A.n2) {
        const uint64_t bra = bc > b ? rb : rc, ket = bc > b ? rc : rb;
        if (popc64(ex) == 2) {
          const SingleEx sx = single_ex(bra, ket, ex);
          val = single_partial(I, bra, sx);
          meta = sx.v | (sx.o << 8) | ((uint32_t)sx.neg << 16) | kPairSingle;
        } else {
          val = me_same_spin_double(I, bra, ket, ex);
          meta = kPairDouble;
        }
      } else {
        const SingleEx sx = single_ex(rb, rc, ex);
        meta = sx.v | (sx.o << 8) | ((uint32_t)sx.neg << 16) | kPairSingle;
      }
    }
    bt[t] = val;
    bm[t] = meta;
  }
}

// alpha pairs per row position (alpha-single blocks and alpha doubles),
// oriented by the group index
__global__ void k_emit_alpha_table(SlabArgs A, Integrals I0, const Integrals* __restrict__ Iinst,
                                   const uint64_t* __restrict__ galpha, double* __restrict__ at,
                                   uint32_t* __restrict__ am) {
  const int64_t tot = (int64_t)A.G * A.rowlen;
  const Integrals I = Iinst ? Iinst[blockIdx.y] : I0;
  at += blockIdx.y * tot;
  am += blockIdx.y * tot;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < tot; t += (int64_t)gridDim.x * blockDim.x) {
    const int g = (int)(t / A.rowlen);
    const uint32_t d = __ldg(A.gdesc + t);
    const int h = (int)(d >> 11), k = (int)(d & 2047u);
    uint32_t meta = 0;
    double val = 0.;
    if (h != g) {
      const uint64_t ra = galpha[g], rh = galpha[h];
      const uint64_t bra = h > g ? ra : rh, ket = h > g ? rh : ra;
      const uint64_t ex = ra ^ rh;
      if (k == kListAlphaDouble) {
        val = me_same_spin_double(I, bra, ket, ex);
        meta = kPairDouble;
      } else {
        const SingleEx sx = single_ex(bra, ket, ex);
        val = single_partial(I, bra, sx);
        meta = sx.v | (sx.o << 8) | ((uint32_t)sx.neg << 16) | kPairSingle;
      }
    }
    at[t] = val;
    am[t] = meta;
  }
}

// STORAGE: QDKGB_H_FP64 (val), kSlabF64F32 (val and its FP32 rounding in
// hi), QDKGB_H_SPLIT32 (the batched layout: hi and lo only).  Batches:
// instance blockIdx.z with the integrals Iinst[blockIdx.z]; tables, diagonal
// and slab of an instance tb_stride / ta_stride, nstride and vstride apart.
template <int STORAGE>
__global__ void __launch_bounds__(kEmitThreads)
    k_slab_emit_tab(SlabArgs A, Integrals I0, const Integrals* __restrict__ Iinst, const uint64_t* __restrict__ galpha,
                    const uint64_t* __restrict__ ubeta, const double* __restrict__ bt,
                    const uint32_t* __restrict__ bm, const double* __restrict__ at, const uint32_t* __restrict__ am,
                    long long tbits, const double* __restrict__ diag_raw, double* __restrict__ val,
                    float* __restrict__ hi, float* __restrict__ lo, double* __restrict__ diag,
                    unsigned long long* __restrict__ kept, int64_t tb_stride, int64_t ta_stride, int64_t nstride,
                    int64_t vstride) {
  const int g = blockIdx.x / kEmitSegments, s = blockIdx.x - g * kEmitSegments;
  const int p0 = s * A.seglen, p1 = min(A.rowlen, p0 + A.seglen);
  const int Nb = A.Nb;
  const int b = blockIdx.y * blockDim.x + threadIdx.x;
  if (b >= Nb) return;
  const int64_t inst = blockIdx.z;
  const Integrals I = Iinst ? Iinst[inst] : I0;
  const size_t n = (size_t)I.n;
  bt += inst * tb_stride;
  bm += inst * tb_stride;
  at += inst * ta_stride;
  am += inst * ta_stride;
  diag_raw += inst * nstride;
  if (val) val += inst * vstride;
  if (hi) hi += inst * vstride;
  if (lo) lo += inst * vstride;
  const int64_t r = (int64_t)g * Nb + b;
  const uint64_t ra = galpha[g], rb = ubeta[b];
  unsigned cnt = 0;
  for (int p = p0; p < p1; ++p) {
    const int64_t gp = (int64_t)g * A.rowlen + p;
    const uint32_t d = __ldg(A.gdesc + gp);
    const int h = (int)(d >> 11), k = (int)(d & 2047u);
    double v;
    bool is_diag = false;
    if (k == kListAlphaDouble) {
      v = __ldg(at + gp);  // alpha double: one value for the whole group row
    } else {
      const int64_t kb = (int64_t)k * Nb + b;
      const int bc = __ldg(A.blT + kb);
      if (h == g) {
        if (bc == b) {
          is_diag = true;
          v = diag_raw[r];
        } else {
          const uint32_t m = __ldg(bm + kb);
          if (m & kPairDouble) {
            v = __ldg(bt + kb);
          } else {  // beta single: the alpha string's V_red terms
            double x = __ldg(bt + kb);
            const double* vr = I.V_red + n * ((m & 255u) + n * ((m >> 8) & 255u));
            for (uint64_t q = ra; q; q &= q - 1) x += ld(vr + low_bit(q));
            v = flip_if(x, (m >> 16) & 1u);
          }
        }
      } else {
        const uint32_t ma = __ldg(am + gp);
        const uint32_t av = ma & 255u, ao = (ma >> 8) & 255u;
        if (bc == b) {  // alpha single: the beta string's V_red terms
          double x = __ldg(at + gp);
          const double* vr = I.V_red + n * (av + n * ao);
          for (uint64_t q = rb; q; q &= q - 1) x += ld(vr + low_bit(q));
          v = flip_if(x, (ma >> 16) & 1u);
        } else {  // opposite-spin double, oriented like the alpha pair
          const uint32_t mb = __ldg(bm + kb);
          const uint32_t xb = mb & 255u, xc = (mb >> 8) & 255u;
          const uint32_t bv = h > g ? xb : xc, bo = h > g ? xc : xb;
          v = flip_if(Vat(I, av, ao, bv, bo), ((ma >> 16) & 1u) != ((mb >> 16) & 1u));
        }
      }
    }
    const bool keep = above_thresh(v, tbits);
    if (is_diag && diag) diag[r] = keep ? v : 0.;
    if (!keep) v = 0.;
    cnt += keep;
    const int64_t q = gp * Nb + b;
    if (STORAGE == QDKGB_H_SPLIT32) {
      const float h = __double2float_rn(v);
      hi[q] = h;
      lo[q] = __double2float_rn(v - (double)h);
    } else {
      val[q] = v;
      if (STORAGE == kSlabF64F32) hi[q] = __double2float_rn(v);
    }
  }
  if (kept) atomicAdd(kept + r, (unsigned long long)cnt);
}
}  // namespace

// ------------------------------------------------------------------ export
// Slab -> CSR (rowptr given): a thread per row writes it in column order.
// Kept rule: every position when thresh <= 0, else the nonzero stored values
// (a kept element exceeds thresh > 0, a dropped one is stored as zero).
template <int STORAGE>
__global__ void __launch_bounds__(256)
    k_slab_export(SlabArgs A, bool keep_all, const double* __restrict__ val, const float* __restrict__ hi,
                  const float* __restrict__ lo, const int64_t* __restrict__ rowptr, int32_t* __restrict__ ci,
                  double* __restrict__ v64, float* __restrict__ h32, float* __restrict__ l32) {
  const int64_t n = (int64_t)A.G * A.Nb;
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const int Nb = A.Nb;
  const int g = (int)(r / Nb), b = (int)(r - (int64_t)g * Nb);
  int64_t o = rowptr[r];
  const int64_t oend = rowptr[r + 1];
  for (int p = 0; p < A.rowlen && o < oend; ++p) {
    const uint32_t d = __ldg(A.gdesc + (int64_t)g * A.rowlen + p);
    const int h = (int)(d >> 11), k = (int)(d & 2047u);
    const int bc = k == kListAlphaDouble ? b : __ldg(A.blT + (int64_t)k * Nb + b);
    const int64_t q = ((int64_t)g * A.rowlen + p) * Nb + b;
    if (STORAGE == QDKGB_H_FP64) {
      const double v = val[q];
      if (keep_all || v != 0.) {
        ci[o] = (int32_t)((int64_t)h * Nb + bc);
        v64[o] = v;
        ++o;
      }
    } else if (STORAGE == kSlabF64F32) {
      // split on the way out: the same (hi, lo) pair the split layout stores
      const double v = val[q];
      if (keep_all || v != 0.) {
        ci[o] = (int32_t)((int64_t)h * Nb + bc);
        const float vh = __double2float_rn(v), vl = __double2float_rn(v - (double)vh);
        if (v64) {
          v64[o] = (double)vh + (double)vl;
        } else {
          h32[o] = vh;
          l32[o] = vl;
        }
        ++o;
      }
    } else {
      const float vh = hi[q], vl = lo[q];
      if (keep_all || vh != 0.f || vl != 0.f) {
        ci[o] = (int32_t)((int64_t)h * Nb + bc);
        if (v64) {
          v64[o] = (double)vh + (double)vl;
        } else {
          h32[o] = vh;
          l32[o] = vl;
        }
        ++o;
      }
    }
  }
}

// ------------------------------------------------------------------ sigma
// CTA per (group g, segment s, part z of the beta strings), instance
// blockIdx.y of a batch (slab vstride apart, vectors n apart); the CTAs of an
// inactive instance leave at once.  The tile itself is slab_sigma_tile.
template <int MODE>
__global__ void __launch_bounds__(kSlabThreads, 2)
    k_slab_sigma(SlabArgs A, PlanArgs P, const void* __restrict__ vals, const float* __restrict__ vlo,
                 const void* __restrict__ xv, const float* __restrict__ xlo, void* __restrict__ yv,
                 int64_t part_stride, int64_t vstride, const int* __restrict__ active) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int g = blockIdx.x / P.S, s = blockIdx.x - g * P.S;
  const int inst = blockIdx.y;
  if (active && !active[inst]) return;
  const int64_t n = (int64_t)A.G * A.Nb;
  if constexpr (MODE == 0) {
    vals = (const float*)vals + inst * vstride;
    xv = (const float*)xv + inst * n;
    yv = (float*)yv + inst * n;
  } else if constexpr (MODE == 1) {
    vals = (const double*)vals + inst * vstride;
    xv = (const double*)xv + inst * n;
    yv = (double*)yv + inst * n;
  } else {
    vals = (const float*)vals + inst * vstride;
    vlo += inst * vstride;
    xv = (const float*)xv + inst * n;
    xlo += inst * n;
    yv = (double*)yv + inst * n;
  }
  slab_sigma_tile<MODE, false>(A, P, vals, vlo, xv, xlo, yv, part_stride, g, s, (int)blockIdx.z, smem_raw);
}

// FP32 sigma, VEC adjacent beta strings per thread (Nb % VEC == 0): float4 /
// float2 value loads (one 16- or 8-byte load per position covers VEC rows, a
// warp reads 32 * 4 * VEC contiguous bytes of a position row), the beta-list
// entries of the VEC rows in one vector load, the alpha doubles' x likewise.
// Same work split, staging and summation structure as k_slab_sigma<0>.
template <int VEC>
struct VecT;
template <>
struct VecT<4> {
  using F = float4;
  using I = int4;
  static __device__ __forceinline__ float at(const float4& v, int c) {
    return c == 0 ? v.x : (c == 1 ? v.y : (c == 2 ? v.z : v.w));
  }
  static __device__ __forceinline__ int at(const int4& v, int c) {
    return c == 0 ? v.x : (c == 1 ? v.y : (c == 2 ? v.z : v.w));
  }
};
template <>
struct VecT<2> {
  using F = float2;
  using I = int2;
  static __device__ __forceinline__ float at(const float2& v, int c) { return c == 0 ? v.x : v.y; }
  static __device__ __forceinline__ int at(const int2& v, int c) { return c == 0 ? v.x : v.y; }
};

// U positions in flight per thread (U * VEC values); the per-row sums keep
// one accumulator per row in position order, so every U gives the same result.
template <int VEC, int U = 4>
__global__ void __launch_bounds__(kSlabVecThreads)
    k_slab_sigma32v(SlabArgs A, PlanArgs P, const float* __restrict__ vals, const float* __restrict__ xv,
                    float* __restrict__ yv, int64_t part_stride, int64_t vstride, const int* __restrict__ active) {
  using VT = VecT<VEC>;
  using F = typename VT::F;
  using I = typename VT::I;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int Nb = A.Nb;
  const int g = blockIdx.x / P.S, s = blockIdx.x - g * P.S;
  const int inst = blockIdx.y;
  if (active && !active[inst]) return;
  const int64_t n = (int64_t)A.G * Nb;
  vals += inst * vstride;
  xv += inst * n;
  yv += inst * n;
  float* xs = reinterpret_cast<float*>(smem_raw);
  int32_t* rec = reinterpret_cast<int32_t*>(xs + (size_t)P.M * Nb);
  const int32_t* rg = P.rec + ((int64_t)g * P.S + s) * P.R;
  for (int i = threadIdx.x; i < P.R; i += blockDim.x) rec[i] = __ldg(rg + i);
  const int32_t* sh = P.segh + ((int64_t)g * P.S + s) * P.M;
  for (int j = 0; j < P.M; ++j) {
    const int h = __ldg(sh + j);
    if (h < 0) continue;
    for (int i = threadIdx.x; i < Nb; i += blockDim.x) cp_async4(xs + (size_t)j * Nb + i, xv + (int64_t)h * Nb + i);
  }
  cp_async_wait_all();
  __syncthreads();
  const int has0 = rec[0], off0 = rec[1], sb0 = rec[2], n1b = rec[3];
  const int32_t* e1 = rec + 4;
  const int nd = rec[4 + 2 * n1b];
  const int32_t* e2 = rec + 6 + 2 * n1b;
  const int nvec = Nb / VEC;
  for (int t = blockIdx.z * blockDim.x + threadIdx.x; t < nvec; t += gridDim.z * blockDim.x) {
    const int b0 = t * VEC;
    // row (g, b0 .. b0+VEC-1): vector index of (p = 0) and the beta-list base
    const F* vb = reinterpret_cast<const F*>(vals + (int64_t)g * A.rowlen * Nb + b0);
    const I* lb = reinterpret_cast<const I*>(A.blT + b0);
    const int nv = Nb / VEC;  // vector stride of one position row / list row
    float acc[VEC];
#pragma unroll
    for (int c = 0; c < VEC; ++c) acc[c] = 0.f;
    if (has0) {
      const int ov = off0 / VEC;
      int k = 0;
      for (; k + U <= A.n2; k += U) {
        F v[U];
        I l[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          v[u] = __ldcs(vb + ov + (k + u) * nv);
          l[u] = __ldg(lb + (k + u) * nv);
        }
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll
          for (int c = 0; c < VEC; ++c) acc[c] = fmaf(VT::at(v[u], c), xs[sb0 + VT::at(l[u], c)], acc[c]);
      }
      for (; k < A.n2; ++k) {
        const F v = __ldcs(vb + ov + k * nv);
        const I l = __ldg(lb + k * nv);
#pragma unroll
        for (int c = 0; c < VEC; ++c) acc[c] = fmaf(VT::at(v, c), xs[sb0 + VT::at(l, c)], acc[c]);
      }
    }
    for (int k = 0; k < A.n1; ++k) {
      const I l = __ldg(lb + (A.n2 + k) * nv);
      const int kk = k * nv;
      int e = 0;
      for (; e + U <= n1b; e += U) {
        F v[U];
#pragma unroll
        for (int u = 0; u < U; ++u) v[u] = __ldcs(vb + e1[2 * (e + u)] / VEC + kk);
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int sb = e1[2 * (e + u) + 1];
#pragma unroll
          for (int c = 0; c < VEC; ++c) acc[c] = fmaf(VT::at(v[u], c), xs[sb + VT::at(l, c)], acc[c]);
        }
      }
      for (; e < n1b; ++e) {
        const F v = __ldcs(vb + e1[2 * e] / VEC + kk);
        const int sb = e1[2 * e + 1];
#pragma unroll
        for (int c = 0; c < VEC; ++c) acc[c] = fmaf(VT::at(v, c), xs[sb + VT::at(l, c)], acc[c]);
      }
    }
    {
      const F* xvv = reinterpret_cast<const F*>(xv + b0);
      int j0 = 0;
      for (; j0 + U <= nd; j0 += U) {
        F v[U], xx[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          v[u] = __ldcs(vb + e2[2 * (j0 + u)] / VEC);
          xx[u] = __ldg(xvv + e2[2 * (j0 + u) + 1] / VEC);
        }
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll
          for (int c = 0; c < VEC; ++c) acc[c] = fmaf(VT::at(v[u], c), VT::at(xx[u], c), acc[c]);
      }
      for (; j0 < nd; ++j0) {
        const F v = __ldcs(vb + e2[2 * j0] / VEC);
        const F xx = __ldg(xvv + e2[2 * j0 + 1] / VEC);
#pragma unroll
        for (int c = 0; c < VEC; ++c) acc[c] = fmaf(VT::at(v, c), VT::at(xx, c), acc[c]);
      }
    }
#pragma unroll
    for (int c = 0; c < VEC; ++c) yv[s * part_stride + (int64_t)g * Nb + b0 + c] = acc[c];
  }
}

// ------------------------------------------------------------------ FP32 sigma, TMA-fed
// The vectorised FP32 sigma (four beta strings per thread) with the slab
// values brought in by the Tensor Memory Accelerator: a producer warp issues
// one 1D bulk copy (cp.async.bulk, global -> shared, completion counted on an
// mbarrier) per position row of the tile (N_b contiguous FP32 values) into a
// ring of kTmaStages stages of up to kTmaRows rows, and eight consumer warps
// read the values from shared memory, so a CTA keeps up to 12 rows in flight
// without registers held for them.  Stages follow the consumption order of
// k_slab_sigma32v<4> (own block; level-1 entry by entry over the segment's
// alpha-single blocks; alpha doubles) and every row is summed in that order:
// the results are that kernel's bit for bit.  Every wait is bounded
// (kTmaSpin tries): on a timeout the CTA records it in g_sigma_fault, writes
// NaN to its rows, waits (bounded) for its own copies still in flight and
// returns.
constexpr int kTmaStages = 3;
constexpr int kTmaRows = 4;
constexpr int kTmaConsumers = 256;  // eight consumer warps; warp 8 issues the copies
constexpr uint32_t kTmaSpin = 1u << 24;

__device__ unsigned int g_sigma_fault;  // set by a CTA whose wait timed out

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* b, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(smem_u32(b)) : "memory");
}
// true once the phase of the given parity has completed; false after kTmaSpin tries
__device__ __forceinline__ bool mbar_wait(uint64_t* b, uint32_t parity) {
  for (uint32_t it = 0; it < kTmaSpin; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(smem_u32(b)), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* b) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(b))
               : "memory");
}

// stage i of a tile: kind 0 own block (rows k0 .. k0+cnt-1), 1 alpha-single
// blocks e0 .. e0+cnt-1 at level-1 entry k, 2 alpha doubles j0 .. j0+cnt-1
struct TmaStage {
  int kind, k, first, cnt;
};
__device__ __forceinline__ TmaStage tma_stage(int i, int n_os, int n_sk, int n_ss, int n2, int n1b, int nd) {
  TmaStage t;
  if (i < n_os) {
    t.kind = 0;
    t.k = 0;
    t.first = i * kTmaRows;
    t.cnt = min(kTmaRows, n2 - t.first);
  } else if (i < n_os + n_ss) {
    const int u = i - n_os;
    t.kind = 1;
    t.k = u / n_sk;
    t.first = (u - t.k * n_sk) * kTmaRows;
    t.cnt = min(kTmaRows, n1b - t.first);
  } else {
    t.kind = 2;
    t.k = 0;
    t.first = (i - n_os - n_ss) * kTmaRows;
    t.cnt = min(kTmaRows, nd - t.first);
  }
  return t;
}

__global__ void __launch_bounds__(kTmaConsumers + 32)
    k_slab_sigma32t(SlabArgs A, PlanArgs P, const float* __restrict__ vals, const float* __restrict__ xv,
                    float* __restrict__ yv, int64_t part_stride, int64_t vstride, const int* __restrict__ active) {
  __shared__ __align__(8) uint64_t full[kTmaStages], empty[kTmaStages];
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int Nb = A.Nb;
  const int g = blockIdx.x / P.S, s = blockIdx.x - g * P.S;
  const int inst = blockIdx.y;
  if (active && !active[inst]) return;
  const int64_t n = (int64_t)A.G * Nb;
  vals += inst * vstride;
  xv += inst * n;
  yv += inst * n;
  float* xs = reinterpret_cast<float*>(smem_raw);
  int32_t* rec = reinterpret_cast<int32_t*>(xs + (size_t)P.M * Nb);
  float* ring = reinterpret_cast<float*>(smem_raw + (((size_t)P.M * Nb * 4 + (size_t)P.R * 4 + 15) / 16 * 16));
  const int tid = threadIdx.x;
  const int32_t* rg = P.rec + ((int64_t)g * P.S + s) * P.R;
  for (int i = tid; i < P.R; i += blockDim.x) rec[i] = __ldg(rg + i);
  if (tid == 0) {
    for (int i = 0; i < kTmaStages; ++i) {
      mbar_init(&full[i], 1);
      mbar_init(&empty[i], kTmaConsumers / 32);
    }
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  __syncthreads();
  const int has0 = rec[0], off0 = rec[1], sb0 = rec[2], n1b = rec[3];
  const int32_t* e1 = rec + 4;
  const int nd = rec[4 + 2 * n1b];
  const int32_t* e2 = rec + 6 + 2 * n1b;
  const int n_os = has0 ? (A.n2 + kTmaRows - 1) / kTmaRows : 0;
  const int n_sk = (n1b + kTmaRows - 1) / kTmaRows;
  const int n_ss = A.n1 * n_sk;
  const int n_st = n_os + n_ss + (nd + kTmaRows - 1) / kTmaRows;
  const float* vg = vals + (int64_t)g * A.rowlen * Nb;
  const uint32_t row_bytes = (uint32_t)Nb * 4u;
  if (tid >= kTmaConsumers) {
    // producer: one elected thread issues the copies
    if (tid != kTmaConsumers) return;
    bool ok = true;
    int issued = 0;
    for (int i = 0; i < n_st; ++i) {
      const int slot = i % kTmaStages, round = i / kTmaStages;
      if (round > 0 && !mbar_wait(&empty[slot], (uint32_t)((round - 1) & 1))) {
        ok = false;
        break;
      }
      const TmaStage t = tma_stage(i, n_os, n_sk, n_ss, A.n2, n1b, nd);
      float* dst = ring + (size_t)slot * kTmaRows * Nb;
      mbar_expect_tx(&full[slot], row_bytes * (uint32_t)t.cnt);
      for (int r = 0; r < t.cnt; ++r) {
        int64_t off;
        if (t.kind == 0)
          off = off0 + (int64_t)(t.first + r) * Nb;
        else if (t.kind == 1)
          off = e1[2 * (t.first + r)] + (int64_t)t.k * Nb;
        else
          off = e2[2 * (t.first + r)];
        bulk_g2s(dst + (size_t)r * Nb, vg + off, row_bytes, &full[slot]);
      }
      ++issued;
    }
    if (!ok) {
      atomicOr(&g_sigma_fault, 1u);
      // the copies still in flight land before this thread (and the CTA) ends
      for (int i = issued - 1; i >= 0 && i >= issued - kTmaStages; --i)
        (void)mbar_wait(&full[i % kTmaStages], (uint32_t)((i / kTmaStages) & 1));
    }
    return;
  }
  // consumers: the staged x slices, then the stages in order
  const int32_t* sh = P.segh + ((int64_t)g * P.S + s) * P.M;
  for (int j = 0; j < P.M; ++j) {
    const int h = __ldg(sh + j);
    if (h < 0) continue;
    for (int i = tid; i < Nb; i += kTmaConsumers) cp_async4(xs + (size_t)j * Nb + i, xv + (int64_t)h * Nb + i);
  }
  cp_async_wait_all();
  asm volatile("bar.sync 1, %0;\n" ::"r"(kTmaConsumers) : "memory");
  const int nvec = Nb / 4;
  const bool live = tid < nvec;
  const int b0 = tid * 4;
  float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
  bool ok = true;
  for (int i = 0; i < n_st; ++i) {
    const int slot = i % kTmaStages;
    if (!mbar_wait(&full[slot], (uint32_t)((i / kTmaStages) & 1))) {
      ok = false;
      break;
    }
    if (live) {
      const TmaStage t = tma_stage(i, n_os, n_sk, n_ss, A.n2, n1b, nd);
      const float* src = ring + (size_t)slot * kTmaRows * Nb + b0;
      if (t.kind == 0) {
        for (int r = 0; r < t.cnt; ++r) {
          const float4 v = *reinterpret_cast<const float4*>(src + (size_t)r * Nb);
          const int4 l = __ldg(reinterpret_cast<const int4*>(A.blT + (int64_t)(t.first + r) * Nb + b0));
          a0 = fmaf(v.x, xs[sb0 + l.x], a0);
          a1 = fmaf(v.y, xs[sb0 + l.y], a1);
          a2 = fmaf(v.z, xs[sb0 + l.z], a2);
          a3 = fmaf(v.w, xs[sb0 + l.w], a3);
        }
      } else if (t.kind == 1) {
        const int4 l = __ldg(reinterpret_cast<const int4*>(A.blT + (int64_t)(A.n2 + t.k) * Nb + b0));
        for (int r = 0; r < t.cnt; ++r) {
          const float4 v = *reinterpret_cast<const float4*>(src + (size_t)r * Nb);
          const int sb = e1[2 * (t.first + r) + 1];
          a0 = fmaf(v.x, xs[sb + l.x], a0);
          a1 = fmaf(v.y, xs[sb + l.y], a1);
          a2 = fmaf(v.z, xs[sb + l.z], a2);
          a3 = fmaf(v.w, xs[sb + l.w], a3);
        }
      } else {
        for (int r = 0; r < t.cnt; ++r) {
          const float4 v = *reinterpret_cast<const float4*>(src + (size_t)r * Nb);
          const float4 x = __ldg(reinterpret_cast<const float4*>(xv + e2[2 * (t.first + r) + 1] + b0));
          a0 = fmaf(v.x, x.x, a0);
          a1 = fmaf(v.y, x.y, a1);
          a2 = fmaf(v.z, x.z, a2);
          a3 = fmaf(v.w, x.w, a3);
        }
      }
    }
    __syncwarp();
    if ((tid & 31) == 0) mbar_arrive(&empty[slot]);
  }
  if (!ok) {
    atomicOr(&g_sigma_fault, 1u);
    a0 = a1 = a2 = a3 = __int_as_float(0x7fc00000);
  }
  if (live)
    *reinterpret_cast<float4*>(yv + s * part_stride + (int64_t)g * Nb + b0) = make_float4(a0, a1, a2, a3);
}

template <typename T>
__global__ void k_slab_combine(int64_t n, int S, const T* __restrict__ part, T* __restrict__ y) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    T a = part[i];
    for (int s = 1; s < S; ++s) a += part[s * n + i];
    y[i] = a;
  }
}

template <int MODE>
void slab_sigma_launch(Context* c, int B, const int* active, const void* vals, const float* vlo, const void* x,
                       const float* xlo, void* y);

// the TMA-fed FP32 sigma needs whole 16-byte rows (N_b a multiple of 4, the
// slab and x 16-byte aligned) and at most kTmaConsumers threads' worth of
// beta strings per group
bool sigma32t_eligible(Context* c, const void* vals, const void* x) {
  FciStruct* F = c->fci;
  return F->Nb % 4 == 0 && F->Nb / 4 <= kTmaConsumers && ((uintptr_t)vals & 15) == 0 && ((uintptr_t)x & 15) == 0 &&
         ((uintptr_t)F->blT.ptr & 15) == 0;
}

// Times every candidate segment count of the plan on this call's inputs
// (one untimed and three timed sigmas each, CUDA events on the context's
// stream) and keeps the fastest; single-instance sigmas only, never inside a
// stream capture.
template <int MODE>
void slab_sigma_tune(Context* c, const void* vals, const float* vlo, const void* x, const float* xlo, void* y) {
  FciStruct* F = c->fci;
  const int pl = MODE == 0 ? 0 : 1;
  SlabPlan& PL = F->plan[pl];
  cudaEvent_t e0, e1;
  QDKGB_CUDA(cudaEventCreate(&e0));
  QDKGB_CUDA(cudaEventCreate(&e1));
  auto load = [&](const PlanHost& ph) {
    PL.S = ph.S;
    PL.M = ph.M;
    PL.R = ph.R;
    void* r = dev_alloc(c, PL.rec, ph.rec.size() * 4 + 16);
    void* g = dev_alloc(c, PL.segh, ph.segh.size() * 4 + 16);
    QDKGB_CUDA(cudaMemcpyAsync(r, ph.rec.data(), ph.rec.size() * 4, cudaMemcpyHostToDevice, c->stream));
    QDKGB_CUDA(cudaMemcpyAsync(g, ph.segh.data(), ph.segh.size() * 4, cudaMemcpyHostToDevice, c->stream));
  };
  auto time3 = [&]() {
    slab_sigma_launch<MODE>(c, 1, nullptr, vals, vlo, x, xlo, y);
    QDKGB_CUDA(cudaEventRecord(e0, c->stream));
    for (int r = 0; r < 3; ++r) slab_sigma_launch<MODE>(c, 1, nullptr, vals, vlo, x, xlo, y);
    QDKGB_CUDA(cudaEventRecord(e1, c->stream));
    QDKGB_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    QDKGB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    return ms / 3.0;
  };
  // QDKGB_SIGMA32_KERNEL=register / tma / register8 / register16: no timing,
  // the planner's default plan with that FP32 kernel (all of them then sum
  // every row alike)
  const char* names[kSigma32Kernels] = {"register", "tma", "register8", "register16"};
  const char* force = MODE == 0 ? std::getenv("QDKGB_SIGMA32_KERNEL") : nullptr;
  auto eligible = [&](int k) {
    if (MODE != 0) return k == 0;
    if (k == 1) return sigma32t_eligible(c, vals, x);
    if (k >= 2) return F->Nb % 4 == 0 && ((uintptr_t)vals & 15) == 0 && ((uintptr_t)x & 15) == 0;
    return true;
  };
  if (force) {
    for (int k = 0; k < kSigma32Kernels; ++k)
      if (std::strcmp(force, names[k]) == 0) {
        F->kernel32 = eligible(k) ? k : 0;
        QDKGB_CUDA(cudaEventDestroy(e0));
        QDKGB_CUDA(cudaEventDestroy(e1));
        F->cand[pl].clear();
        F->cand[pl].shrink_to_fit();
        F->tuned[pl] = true;
        return;
      }
  }
  int best = 0, best_kernel = 0;
  double best_ms = 1e300;
  F->tune_ms[pl].clear();
  if (MODE == 0)
    for (std::vector<double>& v : F->tune_kernel_ms) v.clear();
  for (size_t i = 0; i < F->cand[pl].size(); ++i) {
    load(F->cand[pl][i]);
    for (int k = 0; k < (MODE == 0 ? kSigma32Kernels : 1); ++k) {
      if (!eligible(k)) {
        F->tune_kernel_ms[k].push_back(std::nan(""));
        continue;
      }
      if (MODE == 0) F->kernel32 = k;
      const double ms = time3();
      if (k == 0) F->tune_ms[pl].push_back({F->cand[pl][i].S, ms});
      if (MODE == 0) F->tune_kernel_ms[k].push_back(ms);
      if (ms < best_ms) {
        best_ms = ms;
        best = (int)i;
        best_kernel = k;
      }
    }
  }
  load(F->cand[pl][best]);
  if (MODE == 0) F->kernel32 = best_kernel;
  QDKGB_CUDA(cudaStreamSynchronize(c->stream));
  QDKGB_CUDA(cudaEventDestroy(e0));
  QDKGB_CUDA(cudaEventDestroy(e1));
  F->cand[pl].clear();
  F->cand[pl].shrink_to_fit();
  F->tuned[pl] = true;
}

template <int MODE>
void slab_sigma(Context* c, int B, const int* active, const void* vals, const float* vlo, const void* x,
                const float* xlo, void* y, bool may_tune = false) {
  FciStruct* F = c->fci;
  const int pl = MODE == 0 ? 0 : 1;
  if (may_tune && B == 1 && !F->tuned[pl]) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    QDKGB_CUDA(cudaStreamIsCapturing(c->stream, &cs));
    if (cs == cudaStreamCaptureStatusNone) slab_sigma_tune<MODE>(c, vals, vlo, x, xlo, y);
  }
  slab_sigma_launch<MODE>(c, B, active, vals, vlo, x, xlo, y);
}

template <int MODE>
void slab_sigma_launch(Context* c, int B, const int* active, const void* vals, const float* vlo, const void* x,
                       const float* xlo, void* y) {
  FciStruct* F = c->fci;
  SlabPlan& PL = F->plan[MODE == 0 ? 0 : 1];
  PlanArgs P{PL.S, PL.M, PL.R, (const int32_t*)PL.rec.ptr, (const int32_t*)PL.segh.ptr};
  using Pol = SlabPol<MODE>;
  using Out = typename Pol::Out;
  const size_t smem = (size_t)PL.M * F->Nb * sizeof(typename Pol::Xs) + ((size_t)PL.R * 4 + 15) / 16 * 16;
  set_max_dynamic_smem((const void*)k_slab_sigma<MODE>, (int)kSlabSmemMax);
  if (MODE == 0) {
    set_max_dynamic_smem((const void*)k_slab_sigma32v<4>, (int)kSlabSmemMax);
    set_max_dynamic_smem((const void*)k_slab_sigma32v<4, 8>, (int)kSlabSmemMax);
    set_max_dynamic_smem((const void*)k_slab_sigma32v<4, 16>, (int)kSlabSmemMax);
    set_max_dynamic_smem((const void*)k_slab_sigma32v<2>, (int)kSlabSmemMax);
  }
  const int64_t n = F->G * F->Nb;
  const int64_t vstride = n * F->rowlen;
  void* out = y;
  // partial sums [S][B][n], combined in segment order (deterministic)
  if (PL.S > 1) out = dev_alloc(c, F->ypart, (size_t)PL.S * B * n * sizeof(Out));
  const int Nb = (int)F->Nb;
  const int vec = (MODE == 0 && ((uintptr_t)vals & 15) == 0 && ((uintptr_t)x & 15) == 0 &&
                   ((uintptr_t)F->blT.ptr & 15) == 0)
                      ? (Nb % 4 == 0 ? 4 : (Nb % 2 == 0 ? 2 : 1))
                      : 1;
  if (MODE == 0 && F->kernel32 == 1 && B == 1 && sigma32t_eligible(c, vals, x)) {
    // TMA-fed FP32 sigma: eight consumer warps and one producer warp per CTA
    const size_t tsm = ((size_t)PL.M * Nb * 4 + (size_t)PL.R * 4 + 15) / 16 * 16 + (size_t)kTmaStages * kTmaRows * Nb * 4;
    set_max_dynamic_smem((const void*)k_slab_sigma32t, (int)tsm);
    const dim3 grid((unsigned)(F->G * PL.S), (unsigned)B);
    k_slab_sigma32t<<<grid, kTmaConsumers + 32, tsm, c->stream>>>(slab_args(c), P, (const float*)vals,
                                                                   (const float*)x, (float*)out, (int64_t)B * n,
                                                                   vstride, active);
  } else if (vec > 1) {
    // vectorised FP32 sigma: VEC beta strings per thread
    const int nvec = Nb / vec;
    const unsigned thr = (unsigned)std::min(kSlabVecThreads, (nvec + 31) / 32 * 32);
    const unsigned bz = (unsigned)((nvec + thr - 1) / thr);
    const dim3 grid((unsigned)(F->G * PL.S), (unsigned)B, bz);
    if (vec == 4 && F->kernel32 == 2)
      k_slab_sigma32v<4, 8><<<grid, thr, smem, c->stream>>>(slab_args(c), P, (const float*)vals, (const float*)x,
                                                            (float*)out, (int64_t)B * n, vstride, active);
    else if (vec == 4 && F->kernel32 == 3)
      k_slab_sigma32v<4, 16><<<grid, thr, smem, c->stream>>>(slab_args(c), P, (const float*)vals, (const float*)x,
                                                             (float*)out, (int64_t)B * n, vstride, active);
    else if (vec == 4)
      k_slab_sigma32v<4><<<grid, thr, smem, c->stream>>>(slab_args(c), P, (const float*)vals, (const float*)x,
                                                         (float*)out, (int64_t)B * n, vstride, active);
    else
      k_slab_sigma32v<2><<<grid, thr, smem, c->stream>>>(slab_args(c), P, (const float*)vals, (const float*)x,
                                                         (float*)out, (int64_t)B * n, vstride, active);
  } else {
    const dim3 grid((unsigned)(F->G * PL.S), (unsigned)B, slab_bz(Nb));
    k_slab_sigma<MODE><<<grid, slab_threads(Nb), smem, c->stream>>>(slab_args(c), P, vals, vlo, x, xlo, out,
                                                                    (int64_t)B * n, vstride, active);
  }
  QDKGB_CHECK_LAUNCH();
  if (PL.S > 1) {
    const int64_t tot = (int64_t)B * n;
    const unsigned cb = (unsigned)std::min<int64_t>((tot + 255) / 256, (int64_t)c->sm_count * 8);
    k_slab_combine<Out><<<cb, 256, 0, c->stream>>>(tot, PL.S, (const Out*)out, (Out*)y);
    QDKGB_CHECK_LAUNCH();
  }
}

}  // namespace

// the sigma plan of a precision (0: FP32, 1: FP64): segments in use and the
// autotuner's record (S, ms) per candidate (empty before the first sigma)
int struct_sigma_plan(Context* c, int pl, std::vector<std::pair<int, double>>* record, int* kernel,
                      std::vector<std::vector<double>>* kernel_ms) {
  if (kernel) *kernel = 0;
  if (kernel_ms) kernel_ms->clear();
  if (!c->fci || pl < 0 || pl > 1) return 0;
  if (record) *record = c->fci->tune_ms[pl];
  if (kernel && pl == 0) *kernel = c->fci->kernel32;
  if (kernel_ms && pl == 0) kernel_ms->assign(c->fci->tune_kernel_ms, c->fci->tune_kernel_ms + kSigma32Kernels);
  return c->fci->plan[pl].S;
}

int64_t struct_slab_elements(Context* c) { return c->fci ? c->fci->G * c->fci->Nb * c->fci->rowlen : 0; }

bool struct_ready(Context* c) { return c->fci && c->H.valid && !c->op_direct && c->H.structured; }

// Both storages keep the FP64 values of a single-instance slab (val).
void struct_spmv_fp64(Context* c, const double* x, double* y) {
  slab_sigma<1>(c, 1, nullptr, c->H.val.ptr, nullptr, x, nullptr, y, true);
}

void struct_spmv_fp32(Context* c, const float* x, float* y) {
  Hcsr& H = c->H;
  if (H.storage != QDKGB_H_SPLIT32)
    throw Error(QDKGB_ERR_STATE, "FP32 sigma needs the Hamiltonian built with QDKGB_H_SPLIT32 storage");
  slab_sigma<0>(c, 1, nullptr, H.hi.ptr, nullptr, x, nullptr, y, true);
}

// ------------------------------------------------------------------ batches
// Instances sharing this context's complete space, each with its own
// integrals: slabs [B][stored], per-determinant arrays [B][n].
void slab_emit_batch(Context* c, int B, const Integrals* d_ints, const double* diag_raw, int storage, double* val,
                     float* hi, float* lo, double thresh) {
  FciStruct* F = c->fci;
  const int64_t n = F->G * F->Nb;
  long long tbits = -1;
  if (thresh > 0.) std::memcpy(&tbits, &thresh, sizeof(double));
  SlabArgs A = slab_args(c);
  const uint64_t* ga = (const uint64_t*)c->dets.galpha.ptr;
  const uint64_t* ub = (const uint64_t*)c->dets.ubeta.ptr;
  Integrals none{};
  // every instance's spin-pair tables, then the emission from them
  const int64_t nbt = (int64_t)(F->n2 + F->n1) * F->Nb, nat = F->G * F->rowlen;
  ScopedBuffers<4> tb(c);
  double* bt = dev_array<double>(c, tb.b[0], (size_t)B * nbt);
  uint32_t* bm = dev_array<uint32_t>(c, tb.b[1], (size_t)B * nbt);
  double* at = dev_array<double>(c, tb.b[2], (size_t)B * nat);
  uint32_t* am = dev_array<uint32_t>(c, tb.b[3], (size_t)B * nat);
  const dim3 gb((unsigned)std::max<int64_t>(1, std::min<int64_t>((nbt + 255) / 256, (int64_t)c->sm_count * 8 / B)),
                (unsigned)B);
  k_emit_beta_table<<<gb, 256, 0, c->stream>>>(A, none, d_ints, ub, bt, bm);
  QDKGB_CHECK_LAUNCH();
  const dim3 ga2((unsigned)std::max<int64_t>(1, std::min<int64_t>((nat + 255) / 256, (int64_t)c->sm_count * 8 / B)),
                 (unsigned)B);
  k_emit_alpha_table<<<ga2, 256, 0, c->stream>>>(A, none, d_ints, ga, at, am);
  QDKGB_CHECK_LAUNCH();
  const dim3 grid((unsigned)(F->G * kEmitSegments), (unsigned)((F->Nb + kEmitThreads - 1) / kEmitThreads),
                  (unsigned)B);
  const unsigned thr = (unsigned)std::min<int64_t>(kEmitThreads, (F->Nb + 31) / 32 * 32);
  const int64_t vstride = n * F->rowlen;
  if (storage == QDKGB_H_FP64)
    k_slab_emit_tab<QDKGB_H_FP64><<<grid, thr, 0, c->stream>>>(A, none, d_ints, ga, ub, bt, bm, at, am, tbits,
                                                                diag_raw, val, nullptr, nullptr, nullptr, nullptr,
                                                                nbt, nat, n, vstride);
  else
    k_slab_emit_tab<QDKGB_H_SPLIT32><<<grid, thr, 0, c->stream>>>(A, none, d_ints, ga, ub, bt, bm, at, am, tbits,
                                                                   diag_raw, nullptr, hi, lo, nullptr, nullptr, nbt,
                                                                   nat, n, vstride);
  QDKGB_CHECK_LAUNCH();
  QDKGB_CUDA(cudaStreamSynchronize(c->stream));  // the tables are freed on return
}

// Sizes the partial-sum scratch for B instances in every mode, so that no
// later sigma reallocates it (a captured graph keeps its address).
void slab_reserve_batch(Context* c, int B) {
  FciStruct* F = c->fci;
  const int64_t n = F->G * F->Nb;
  const size_t need = std::max<size_t>((size_t)F->plan[0].S * 4, (size_t)F->plan[1].S * 8) * B * n;
  dev_alloc(c, F->ypart, need);
  // the batched FP32 sigma is not autotuned: the four-deep register-fed
  // kernel unless QDKGB_SIGMA32_KERNEL pins a register-fed depth
  const char* force = std::getenv("QDKGB_SIGMA32_KERNEL");
  F->kernel32 = 0;
  if (force && F->Nb % 4 == 0) {
    if (std::strcmp(force, "register8") == 0) F->kernel32 = 2;
    if (std::strcmp(force, "register16") == 0) F->kernel32 = 3;
  }
}

// mode 0: FP32 (vals = hi, x/y float); 1: FP64; 2: float-float from (hi, lo)
// with split x (x = xh, xlo = xl) into FP64 y.  active[B] masks instances.
void slab_sigma_batch(Context* c, int mode, int B, const int* active, const void* vals, const float* vlo,
                      const void* x, const float* xlo, void* y) {
  if (mode == 0) slab_sigma<0>(c, B, active, vals, nullptr, x, nullptr, y);
  else if (mode == 1) slab_sigma<1>(c, B, active, vals, nullptr, x, nullptr, y);
  else slab_sigma<2>(c, B, active, vals, vlo, x, xlo, y);
}

// CSR arrays of a slab Hamiltonian into device buffers of nnz entries: the
// columns, and the values as FP64 (v64) or as the split pair (h32, l32).
void struct_export(Context* c, int32_t* ci, double* v64, float* h32, float* l32) {
  Hcsr& H = c->H;
  SlabArgs A = slab_args(c);
  const unsigned nb = (unsigned)((H.n + 255) / 256);
  const bool keep_all = !(H.thresh > 0.);
  if (H.storage == QDKGB_H_FP64)
    k_slab_export<QDKGB_H_FP64><<<nb, 256, 0, c->stream>>>(A, keep_all, (const double*)H.val.ptr, nullptr, nullptr,
                                                           (const int64_t*)H.rowptr.ptr, ci, v64, h32, l32);
  else
    k_slab_export<kSlabF64F32><<<nb, 256, 0, c->stream>>>(A, keep_all, (const double*)H.val.ptr, nullptr, nullptr,
                                                          (const int64_t*)H.rowptr.ptr, ci, v64, h32, l32);
  QDKGB_CHECK_LAUNCH();
}

// Slab build for complete spaces (build_hamiltonian dispatches here).  When
// fewer than half of the elements survive the threshold the slab is turned
// into the reference's CSR arrays and freed.
void build_hamiltonian_struct(Context* c, double thresh, int storage) {
  Hcsr& H = c->H;
  DetSpace& D = c->dets;
  FciStruct* F = c->fci;
  const int64_t n = D.ndets;
  const int64_t nslab = n * F->rowlen;
  long long tbits = -1;
  if (thresh > 0.) std::memcpy(&tbits, &thresh, sizeof(double));
  Integrals I = integrals_view(c);
  double* diag_raw = dev_array<double>(c, H.diag_raw, n);
  double* diag = dev_array<double>(c, H.diag, n);
  int64_t* kept = dev_array<int64_t>(c, H.row_nnz, n + 1);
  const unsigned tb = (unsigned)std::min<int64_t>((n + 255) / 256, (int64_t)c->sm_count * 16);
  k_diag_launch(c, I, diag_raw, tb);
  dev_free(c, H.colind);
  dev_free(c, H.lo);
  if (storage == QDKGB_H_FP64) dev_free(c, H.hi);
  double* val = dev_array<double>(c, H.val, nslab);
  float* hi = storage == QDKGB_H_SPLIT32 ? dev_array<float>(c, H.hi, nslab) : nullptr;
  QDKGB_CUDA(cudaMemsetAsync(diag, 0, n * sizeof(double), c->stream));
  QDKGB_CUDA(cudaMemsetAsync(kept, 0, (n + 1) * sizeof(int64_t), c->stream));
  SlabArgs A = slab_args(c);
  const dim3 grid((unsigned)(F->G * kEmitSegments), (unsigned)((F->Nb + kEmitThreads - 1) / kEmitThreads));
  const unsigned thr = kEmitThreads;
  const uint64_t* ga = (const uint64_t*)D.galpha.ptr;
  const uint64_t* ub = (const uint64_t*)D.ubeta.ptr;
  unsigned long long* kc = (unsigned long long*)kept;
  // spin-pair tables, then the emission from them
  const int64_t nbt = (int64_t)(F->n2 + F->n1) * F->Nb, nat = F->G * F->rowlen;
  double* bt = dev_array<double>(c, F->tab_b, nbt);
  uint32_t* bm = dev_array<uint32_t>(c, F->tab_bm, nbt);
  double* at = dev_array<double>(c, F->tab_a, nat);
  uint32_t* am = dev_array<uint32_t>(c, F->tab_am, nat);
  k_emit_beta_table<<<(unsigned)std::min<int64_t>((nbt + 255) / 256, (int64_t)c->sm_count * 8), 256, 0, c->stream>>>(
      A, I, nullptr, ub, bt, bm);
  QDKGB_CHECK_LAUNCH();
  k_emit_alpha_table<<<(unsigned)std::min<int64_t>((nat + 255) / 256, (int64_t)c->sm_count * 8), 256, 0,
                       c->stream>>>(A, I, nullptr, ga, at, am);
  QDKGB_CHECK_LAUNCH();
  if (storage == QDKGB_H_FP64)
    k_slab_emit_tab<QDKGB_H_FP64><<<grid, thr, 0, c->stream>>>(A, I, nullptr, ga, ub, bt, bm, at, am, tbits, diag_raw,
                                                                val, nullptr, nullptr, diag, kc, 0, 0, 0, 0);
  else
    k_slab_emit_tab<kSlabF64F32><<<grid, thr, 0, c->stream>>>(A, I, nullptr, ga, ub, bt, bm, at, am, tbits, diag_raw,
                                                               val, hi, nullptr, diag, kc, 0, 0, 0, 0);
  QDKGB_CHECK_LAUNCH();
  int64_t* rowptr = dev_array<int64_t>(c, H.rowptr, n + 1);
  exclusive_scan_i64(c, kept, rowptr, n, H.scan_tmp);
  int64_t nnz = 0;
  QDKGB_CUDA(cudaMemcpyAsync(&nnz, rowptr + n, sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
  QDKGB_CUDA(cudaStreamSynchronize(c->stream));
  H.n = n;
  H.nnz = nnz;
  H.storage = storage;
  H.thresh = thresh;
  H.structured = true;
  H.valid = true;
  if (2 * nnz < nslab) {
    // mostly thresholded away: the CSR arrays are smaller than the slab
    DeviceBuffer cib, vb, hb, lb;
    const int64_t cap = std::max<int64_t>(nnz, 1);
    int32_t* ci = dev_array<int32_t>(c, cib, cap);
    double* v64 = storage == QDKGB_H_FP64 ? dev_array<double>(c, vb, cap) : nullptr;
    float* h32 = storage == QDKGB_H_SPLIT32 ? dev_array<float>(c, hb, cap) : nullptr;
    float* l32 = storage == QDKGB_H_SPLIT32 ? dev_array<float>(c, lb, cap) : nullptr;
    struct_export(c, ci, v64, h32, l32);
    QDKGB_CUDA(cudaStreamSynchronize(c->stream));
    std::swap(H.colind, cib);
    dev_free(c, cib);
    if (storage == QDKGB_H_FP64) {
      std::swap(H.val, vb);
      dev_free(c, vb);
    } else {
      std::swap(H.hi, hb);
      std::swap(H.lo, lb);
      dev_free(c, hb);
      dev_free(c, lb);
      dev_free(c, H.val);
    }
    H.structured = false;
  }
}

}  // namespace qdkgb
