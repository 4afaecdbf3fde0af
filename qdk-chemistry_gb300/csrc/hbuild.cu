// Determinant-space preparation and the CSR Hamiltonian build.
//
// Replaces SortedDoubleLoopHamiltonianGenerator::make_csr_hamiltonian_block_
// (include/macis/hamiltonian_generator/sorted_double_loop.hpp:86-451).
//
// GPU design (not a translation of the reference's loops): the reference
// visits alpha-group pairs and then all beta x beta pairs of the two groups,
// testing each with a popcount, fills with atomic slot capture and sorts each
// row afterwards.  Here one warp owns one CSR row and generates only the
// connected columns, already in ascending order:
//   * alpha groups connected to the row's group (<= 4 differing bits) come
//     from a precomputed, sorted alpha-connectivity list, tagged with their
//     excitation level e_a in {0,1,2};
//   * inside a connected group the admissible beta strings are those within
//     level 2 - e_a of the row's beta string; they come from precomputed,
//     sorted beta-connectivity lists (level <= 1 and level <= 2) and are
//     located in the group by identity (groups holding every beta string),
//     by binary search, or by a direct scan of small groups;
//   * the row's candidate list is the concatenation of these per-group lists;
//     the 32 lanes walk it as one flat index space (load-balanced across the
//     uneven per-group sizes), evaluate the Slater-Condon element, apply the
//     strict |h| > thresh rule, and compact survivors with a ballot.
// A count pass and an emit pass run the same code; an exclusive scan between
// them gives the row pointers.  No sort and no atomics are needed, and the
// result is deterministic.
#include <algorithm>
#include <cstring>
#include <functional>
#include <numeric>
#include <queue>
#include <unordered_map>

#include "common.cuh"
#include "host_parallel.h"
#include "internal.h"
#include "rowwalk.cuh"

namespace qdkgb {

// ------------------------------------------------------------------ integrals
// generate_integral_intermediates_ (src/macis/hamiltonian_generator/base.ipp:38-77)
__global__ void k_intermediates(int n, const double* __restrict__ V, double* G_red, double* V_red, double* G2,
                                double* V2) {
  const size_t nn = (size_t)n;
  const int64_t total = (int64_t)n * n * n;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(t % n), i = (int)((t / n) % n), j = (int)(t / (nn * nn));
    auto v = [&](int p, int q, int r, int s) { return V[p + nn * (q + nn * (r + nn * s))]; };
    G_red[t] = v(k, k, i, j) - v(k, j, i, k);
    V_red[t] = v(k, k, i, j);
    if (k == 0) {
      G2[i + nn * j] = 0.5 * (v(i, i, j, j) - v(i, j, j, i));
      V2[i + nn * j] = v(i, i, j, j);
    }
  }
}

// intermediates of integrals already on the device (batched instances)
void build_integral_intermediates_into(Context* c, int n, const double* V, double* G, double* Vr, double* G2,
                                       double* V2) {
  const int64_t n3 = (int64_t)n * n * n;
  const int blocks = (int)std::min<int64_t>((n3 + 255) / 256, 4096);
  k_intermediates<<<blocks, 256, 0, c->stream>>>(n, V, G, Vr, G2, V2);
  QDKGB_CHECK_LAUNCH();
}

void build_integral_intermediates(Context* c) {
  const int n = c->norb;
  const size_t n2 = (size_t)n * n, n3 = n2 * n, n4 = n3 * n;
  double* T = dev_array<double>(c, c->T, n2);
  double* V = dev_array<double>(c, c->V, n4);
  double* G = dev_array<double>(c, c->G_red, n3);
  double* Vr = dev_array<double>(c, c->V_red, n3);
  double* G2 = dev_array<double>(c, c->G2, n2);
  double* V2 = dev_array<double>(c, c->V2, n2);
  QDKGB_CUDA(cudaMemcpyAsync(T, c->h_T.data(), n2 * 8, cudaMemcpyHostToDevice, c->stream));
  QDKGB_CUDA(cudaMemcpyAsync(V, c->h_V.data(), n4 * 8, cudaMemcpyHostToDevice, c->stream));
  int blocks = (int)std::min<int64_t>((n3 + 255) / 256, 4096);
  k_intermediates<<<blocks, 256, 0, c->stream>>>(n, V, G, Vr, G2, V2);
  QDKGB_CHECK_LAUNCH();
  QDKGB_CUDA(cudaStreamSynchronize(c->stream));
}

Integrals integrals_view(Context* c) {
  Integrals I;
  I.T = (const double*)c->T.ptr;
  I.V = (const double*)c->V.ptr;
  I.G_red = (const double*)c->G_red.ptr;
  I.V_red = (const double*)c->V_red.ptr;
  I.G2 = (const double*)c->G2.ptr;
  I.V2 = (const double*)c->V2.ptr;
  I.n = c->norb;
  return I;
}

// ------------------------------------------------------------------ scan
__global__ void k_scan_block_sums(const int64_t* in, int64_t n, int64_t* sums) {
  __shared__ int64_t s[32];
  const int64_t base = (int64_t)blockIdx.x * 1024;
  int64_t v = 0;
  for (int k = threadIdx.x; k < 1024; k += blockDim.x)
    if (base + k < n) v += in[base + k];
  v = warp_sum(v);
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    int64_t w = (threadIdx.x < (blockDim.x >> 5)) ? s[threadIdx.x] : 0;
    w = warp_sum(w);
    if (threadIdx.x == 0) sums[blockIdx.x] = w;
  }
}
// single block: exclusive scan of the block sums, in place; total at sums[nb]
__global__ void k_scan_sums(int64_t* sums, int64_t nb) {
  __shared__ int64_t carry;
  __shared__ int64_t warp_tot[32];
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int64_t base = 0; base < nb; base += blockDim.x) {
    const int64_t i = base + threadIdx.x;
    int64_t v = (i < nb) ? sums[i] : 0, incl = v;
    for (int d = 1; d < 32; d <<= 1) {
      int64_t t = __shfl_up_sync(QDKGB_FULL_MASK, incl, d);
      if (lane >= d) incl += t;
    }
    if (lane == 31) warp_tot[w] = incl;
    __syncthreads();
    if (w == 0) {
      int64_t t = (lane < (int)(blockDim.x >> 5)) ? warp_tot[lane] : 0, ti = t;
      for (int d = 1; d < 32; d <<= 1) {
        int64_t u = __shfl_up_sync(QDKGB_FULL_MASK, ti, d);
        if (lane >= d) ti += u;
      }
      warp_tot[lane] = ti - t;
    }
    __syncthreads();
    const int64_t excl = carry + warp_tot[w] + incl - v;
    __syncthreads();
    if (i < nb) sums[i] = excl;
    if (threadIdx.x == blockDim.x - 1) carry = excl + v;
    __syncthreads();
  }
  if (threadIdx.x == 0) sums[nb] = carry;
}
__global__ void k_scan_apply(const int64_t* in, int64_t n, const int64_t* sums, int64_t* out) {
  // one block of 1024 threads per 1024 elements
  __shared__ int64_t warp_tot[32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t i = (int64_t)blockIdx.x * 1024 + threadIdx.x;
  int64_t v = (i < n) ? in[i] : 0, incl = v;
  for (int d = 1; d < 32; d <<= 1) {
    int64_t t = __shfl_up_sync(QDKGB_FULL_MASK, incl, d);
    if (lane >= d) incl += t;
  }
  if (lane == 31) warp_tot[w] = incl;
  __syncthreads();
  if (w == 0) {
    int64_t t = warp_tot[lane], ti = t;
    for (int d = 1; d < 32; d <<= 1) {
      int64_t u = __shfl_up_sync(QDKGB_FULL_MASK, ti, d);
      if (lane >= d) ti += u;
    }
    warp_tot[lane] = ti - t;
  }
  __syncthreads();
  if (i < n) out[i] = sums[blockIdx.x] + warp_tot[w] + incl - v;
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) out[n] = sums[gridDim.x];
}

// out[0..n] = exclusive scan of in[0..n), out[n] = total.
void exclusive_scan_i64(Context* c, const int64_t* in, int64_t* out, int64_t n, DeviceBuffer& tmp) {
  const int64_t nb = std::max<int64_t>(1, (n + 1023) / 1024);
  int64_t* sums = dev_array<int64_t>(c, tmp, nb + 1);
  k_scan_block_sums<<<(unsigned)nb, 256, 0, c->stream>>>(in, n, sums);
  QDKGB_CHECK_LAUNCH();
  k_scan_sums<<<1, 1024, 0, c->stream>>>(sums, nb);
  QDKGB_CHECK_LAUNCH();
  k_scan_apply<<<(unsigned)nb, 1024, 0, c->stream>>>(in, n, sums, out);
  QDKGB_CHECK_LAUNCH();
}

// ------------------------------------------------------------------ string connectivity
// For every string i, the sorted list of strings j with popc(s_i ^ s_j) <=
// maxbits.  skip_zero drops the empty string on both sides (the reference
// skips alpha groups whose string has no electrons,
// sorted_double_loop.hpp:145,153).  Warp per i, ballot compaction.
template <bool EMIT>
__global__ void k_conn(const uint64_t* __restrict__ s, int64_t m, int maxbits, bool skip_zero, int64_t* cnt,
                       const int64_t* ptr, int32_t* idx, int8_t* lvl) {
  const int lane = threadIdx.x & 31;
  const int64_t wid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t i = wid; i < m; i += nw) {
    const uint64_t si = s[i];
    int64_t out = EMIT ? ptr[i] : 0;
    int64_t c = 0;
    const bool dead = skip_zero && si == 0;
    for (int64_t j0 = 0; j0 < m && !dead; j0 += 32) {
      const int64_t j = j0 + lane;
      bool hit = false;
      int d = 0;
      if (j < m) {
        const uint64_t sj = s[j];
        d = popc64(si ^ sj);
        hit = d <= maxbits && !(skip_zero && sj == 0);
      }
      const unsigned b = __ballot_sync(QDKGB_FULL_MASK, hit);
      if (EMIT && hit) {
        const int64_t pos = out + c + __popc(b & ((1u << lane) - 1u));
        idx[pos] = (int32_t)j;
        if (lvl) lvl[pos] = (int8_t)(d >> 1);
      }
      c += __popc(b);
    }
    if (!EMIT && lane == 0) cnt[i] = c;
  }
}

static void build_conn(Context* c, const uint64_t* d_s, int64_t m, int maxbits, bool skip_zero, DeviceBuffer& ptr,
                       DeviceBuffer& idx, DeviceBuffer* lvl, int64_t& total) {
  DeviceBuffer cnt, tmp;
  int64_t* d_cnt = dev_array<int64_t>(c, cnt, m + 1);
  int64_t* d_ptr = dev_array<int64_t>(c, ptr, m + 1);
  const int threads = 256;
  const int64_t blocks = std::min<int64_t>((m * 32 + threads - 1) / threads, (int64_t)c->sm_count * 64);
  k_conn<false><<<(unsigned)blocks, threads, 0, c->stream>>>(d_s, m, maxbits, skip_zero, d_cnt, nullptr, nullptr,
                                                             nullptr);
  QDKGB_CHECK_LAUNCH();
  exclusive_scan_i64(c, d_cnt, d_ptr, m, tmp);
  QDKGB_CUDA(cudaMemcpyAsync(&total, d_ptr + m, sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
  QDKGB_CUDA(cudaStreamSynchronize(c->stream));
  int32_t* d_idx = dev_array<int32_t>(c, idx, std::max<int64_t>(total, 1));
  int8_t* d_lvl = lvl ? dev_array<int8_t>(c, *lvl, std::max<int64_t>(total, 1)) : nullptr;
  k_conn<true><<<(unsigned)blocks, threads, 0, c->stream>>>(d_s, m, maxbits, skip_zero, nullptr, d_ptr, d_idx, d_lvl);
  QDKGB_CHECK_LAUNCH();
  QDKGB_CUDA(cudaStreamSynchronize(c->stream));
  dev_free(c, cnt);
  dev_free(c, tmp);
}

// ------------------------------------------------------------------ determinant space
// Host part: alpha runs (get_unique_alpha, sd_operations.hpp:449-468) and a
// single order on the distinct beta strings that every group's beta sequence
// follows.  Tried in turn: ascending integer order (lists sorted by
// spin_comparator), the common sequence of a full product space
// (generate_hilbert_space), and a topological order of the per-group
// successions.
void build_det_space(Context* c, int64_t nd, const uint64_t* alpha, const uint64_t* beta) {
  NvtxRange nvtx_range("qdkgb.set_dets");
  DetSpace& D = c->dets;
  for (DeviceBuffer* b : {&D.galpha, &D.gstart, &D.det_group, &D.brank, &D.ubeta, &D.gcomplete, &D.acon_ptr,
                          &D.acon_idx, &D.acon_lvl, &D.b2_ptr, &D.b2_idx, &D.b1_ptr, &D.b1_idx})
    dev_free(c, *b);
  D = DetSpace();
  c->have_dets = false;
  c->fci_shape[0] = c->fci_shape[1] = c->fci_shape[2] = -1;
  c->H.valid = false;
  free_direct(c);
  free_struct(c);
  c->op_direct = false;
  c->fp32_direct = false;
  if (nd <= 0) throw Error(QDKGB_ERR_INVALID, "empty determinant list");
  if (nd >= (int64_t)INT32_MAX) throw Error(QDKGB_ERR_UNSUPPORTED, "more than 2^31-1 determinants");
  D.ndets = nd;
  D.h_alpha.assign(alpha, alpha + nd);
  D.h_beta.assign(beta, beta + nd);
  for (int64_t i = 0; i < nd; ++i) D.occ_union |= alpha[i] | beta[i];
  D.h_gstart.push_back(0);
  D.h_galpha.push_back(alpha[0]);
  for (int64_t i = 1; i < nd; ++i)
    if (alpha[i] != alpha[i - 1]) {
      D.h_galpha.push_back(alpha[i]);
      D.h_gstart.push_back(i);
    }
  D.h_gstart.push_back(nd);
  D.ngroups = (int64_t)D.h_galpha.size();
  const int64_t G = D.ngroups;

  std::vector<uint64_t> ubeta;
  std::vector<int32_t> brank(nd);
  // product space (generate_hilbert_space): every group repeats group 0's beta
  // sequence - ranks by position, O(n)
  bool product0 = G >= 1 && nd % D.h_gstart[1] == 0 && G * D.h_gstart[1] == nd;
  {
    const int64_t s0 = D.h_gstart[1];
    for (int64_t g = 1; g < G && product0; ++g) {
      if (D.h_gstart[g + 1] - D.h_gstart[g] != s0) product0 = false;
      else product0 = std::memcmp(beta + D.h_gstart[g], beta, s0 * sizeof(uint64_t)) == 0;
    }
    for (int64_t k = 1; k < s0 && product0; ++k) product0 = beta[k - 1] < beta[k];
  }
  bool ascending = !product0;
  if (product0) {
    const int64_t s0 = D.h_gstart[1];
    ubeta.assign(beta, beta + s0);
    for (int64_t i = 0; i < nd; ++i) brank[i] = (int32_t)(i % s0);
    D.product = true;
  }
  for (int64_t g = 0; g < G && ascending; ++g)
    for (int64_t i = D.h_gstart[g] + 1; i < D.h_gstart[g + 1]; ++i)
      if (!(beta[i - 1] < beta[i])) {
        ascending = false;
        break;
      }
  if (product0) {
    // ranks set above
  } else if (ascending) {
    ubeta.assign(beta, beta + nd);
    parallel_sort(ubeta, std::less<uint64_t>());
    ubeta.erase(std::unique(ubeta.begin(), ubeta.end()), ubeta.end());
    parallel_ranges(nd, [&](int64_t i0, int64_t i1) {
      for (int64_t i = i0; i < i1; ++i)
        brank[i] = (int32_t)(std::lower_bound(ubeta.begin(), ubeta.end(), beta[i]) - ubeta.begin());
    });
  } else {
    // product space: every group repeats group 0's beta sequence
    const int64_t s0 = D.h_gstart[1];
    bool product = (nd % s0) == 0 && G * s0 == nd;
    for (int64_t g = 1; g < G && product; ++g) {
      if (D.h_gstart[g + 1] - D.h_gstart[g] != s0) product = false;
      for (int64_t k = 0; k < s0 && product; ++k)
        if (beta[D.h_gstart[g] + k] != beta[k]) product = false;
    }
    std::unordered_map<uint64_t, int32_t> rank;
    if (product) {
      ubeta.assign(beta, beta + s0);
      for (int64_t k = 0; k < s0; ++k)
        if (!rank.emplace(beta[k], (int32_t)k).second)
          throw Error(QDKGB_ERR_UNSUPPORTED, "repeated determinant in the list");
    } else {
      // topological order of "b precedes b'" edges from consecutive dets of each group
      std::unordered_map<uint64_t, int32_t> id;
      std::vector<uint64_t> strs;
      for (int64_t i = 0; i < nd; ++i)
        if (id.emplace(beta[i], (int32_t)strs.size()).second) strs.push_back(beta[i]);
      const int64_t U = (int64_t)strs.size();
      std::vector<std::vector<int32_t>> succ(U);
      std::vector<int32_t> indeg(U, 0);
      for (int64_t g = 0; g < G; ++g)
        for (int64_t i = D.h_gstart[g] + 1; i < D.h_gstart[g + 1]; ++i) {
          const int32_t a = id[beta[i - 1]], b = id[beta[i]];
          succ[a].push_back(b);
          indeg[b]++;
        }
      std::priority_queue<std::pair<uint64_t, int32_t>, std::vector<std::pair<uint64_t, int32_t>>,
                          std::greater<std::pair<uint64_t, int32_t>>>
          pq;
      for (int64_t u = 0; u < U; ++u)
        if (!indeg[u]) pq.push({strs[u], (int32_t)u});
      while (!pq.empty()) {
        auto [s, u] = pq.top();
        pq.pop();
        rank[s] = (int32_t)ubeta.size();
        ubeta.push_back(s);
        for (int32_t v : succ[u])
          if (--indeg[v] == 0) pq.push({strs[v], v});
      }
      if ((int64_t)ubeta.size() != U)
        throw Error(QDKGB_ERR_UNSUPPORTED,
                    "determinant list is not alpha-grouped with one common beta order (sort it by spin_comparator)");
    }
    for (int64_t i = 0; i < nd; ++i) brank[i] = rank[beta[i]];
    D.product = product;
  }
  // strict increase inside every group (no repeated determinant)
  for (int64_t g = 0; g < G; ++g)
    for (int64_t i = D.h_gstart[g] + 1; i < D.h_gstart[g + 1]; ++i)
      if (!(brank[i - 1] < brank[i]))
        throw Error(QDKGB_ERR_UNSUPPORTED, "repeated determinant or inconsistent beta order in an alpha group");
  D.nbeta = (int64_t)ubeta.size();
  D.h_ubeta = ubeta;

  std::vector<int32_t> det_group(nd);
  std::vector<uint8_t> complete(G);
  for (int64_t g = 0; g < G; ++g) {
    for (int64_t i = D.h_gstart[g]; i < D.h_gstart[g + 1]; ++i) det_group[i] = (int32_t)g;
    complete[g] = (D.h_gstart[g + 1] - D.h_gstart[g]) == D.nbeta;
  }

  auto up = [&](DeviceBuffer& b, const void* src, size_t bytes) {
    void* p = dev_alloc(c, b, bytes + 16);
    QDKGB_CUDA(cudaMemcpyAsync(p, src, bytes, cudaMemcpyHostToDevice, c->stream));
  };
  up(D.galpha, D.h_galpha.data(), G * 8);
  up(D.gstart, D.h_gstart.data(), (G + 1) * 8);
  up(D.det_group, det_group.data(), nd * 4);
  up(D.brank, brank.data(), nd * 4);
  up(D.ubeta, ubeta.data(), D.nbeta * 8);
  up(D.gcomplete, complete.data(), G);
  QDKGB_CUDA(cudaStreamSynchronize(c->stream));

  build_conn(c, (const uint64_t*)D.galpha.ptr, G, 4, true, D.acon_ptr, D.acon_idx, &D.acon_lvl, D.acon_total);
  build_conn(c, (const uint64_t*)D.ubeta.ptr, D.nbeta, 4, false, D.b2_ptr, D.b2_idx, nullptr, D.b2_total);
  build_conn(c, (const uint64_t*)D.ubeta.ptr, D.nbeta, 2, false, D.b1_ptr, D.b1_idx, nullptr, D.b1_total);
  build_struct(c);
  c->have_dets = true;
}

// ------------------------------------------------------------------ CSR rows
// Diagonal elements, one thread per determinant (matrix_element_diag in the
// reference's order); alpha-empty determinants get 0 (the reference skips
// their rows).
__global__ void k_diag(Integrals I, int64_t n, const int32_t* __restrict__ det_group,
                       const int32_t* __restrict__ brank, const uint64_t* __restrict__ galpha,
                       const uint64_t* __restrict__ ubeta, double* __restrict__ D) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t a = galpha[det_group[r]];
    D[r] = a ? me_diag(I, a, ubeta[brank[r]]) : 0.;
  }
}

void k_diag_launch(Context* c, const Integrals& I, double* D, unsigned blocks) {
  const DetSpace& S = c->dets;
  k_diag<<<blocks, 256, 0, c->stream>>>(I, S.ndets, (const int32_t*)S.det_group.ptr, (const int32_t*)S.brank.ptr,
                                        (const uint64_t*)S.galpha.ptr, (const uint64_t*)S.ubeta.ptr, D);
  QDKGB_CHECK_LAUNCH();
}

// Pre-threshold row lengths: the number of connected determinants present in
// the list.  Integer work only: groups holding every beta string contribute
// their candidate-list length directly; the others are checked candidate by
// candidate (binary search or scan).
// rows: the rows to count (row i of the output is row rows[i]); null: all
__global__ void __launch_bounds__(kRowWarps * 32)
    k_row_count(RowArgs a, const int32_t* __restrict__ rows, int64_t nrows, int64_t* __restrict__ row_nnz) {
  __shared__ RowWalkSmem sm;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int64_t i = (int64_t)blockIdx.x * kRowWarps + w; i < nrows; i += (int64_t)gridDim.x * kRowWarps) {
    const int64_t r = rows ? (int64_t)rows[i] : i;
    const int32_t g = a.det_group[r];
    const int32_t b = a.brank[r];
    const uint64_t rb = a.ubeta[b];
    int64_t cnt = 0;
    if (a.galpha[g] != 0) {
      const int64_t b1 = a.b1_ptr[b], n1 = a.b1_ptr[b + 1] - b1;
      const int64_t b2 = a.b2_ptr[b], n2 = a.b2_ptr[b + 1] - b2;
      const int64_t e_end = a.acon_ptr[g + 1];
      for (int64_t e0 = a.acon_ptr[g]; e0 < e_end; e0 += 32) {
        const int64_t e = e0 + lane;
        int my = 0, h = 0, lvl = 0, mode = kIdent;
        int64_t direct = 0;
        if (e < e_end) {
          h = a.acon_idx[e];
          lvl = a.acon_lvl[e];
          const int64_t gs = a.gstart[h + 1] - a.gstart[h];
          const int64_t cand = lvl == 0 ? n2 : (lvl == 1 ? n1 : 1);
          if (a.gcomplete[h]) {
            direct = cand;
          } else if (gs <= cand) {
            mode = kScan;
            my = (int)gs;
          } else {
            mode = kSearch;
            my = (int)cand;
          }
        }
        int64_t dsum = direct;
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) dsum += __shfl_xor_sync(QDKGB_FULL_MASK, dsum, d);
        cnt += dsum;
        const int incl = warp_inclusive_scan(my, lane);
        const int total = __shfl_sync(QDKGB_FULL_MASK, incl, 31);
        if (total == 0) continue;
        sm.off[w][lane + 1] = incl;
        if (lane == 0) sm.off[w][0] = 0;
        sm.h[w][lane] = h;
        sm.lvl[w][lane] = (int8_t)lvl;
        sm.mode[w][lane] = (int8_t)mode;
        __syncwarp();
        for (int base = 0; base < total; base += 32) {
          const int f = base + lane;
          bool hit = false;
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
            const int hh = sm.h[w][lo], ll = sm.lvl[w][lo];
            const int64_t g0 = a.gstart[hh];
            if (sm.mode[w][lo] == kScan) {
              hit = popc64(rb ^ a.ubeta[a.brank[g0 + k]]) <= 2 * (2 - ll);
            } else {
              const int32_t cr = ll == 0 ? a.b2_idx[b2 + k] : (ll == 1 ? a.b1_idx[b1 + k] : b);
              hit = find_rank(a.brank, g0, a.gstart[hh + 1], cr) >= 0;
            }
          }
          cnt += __popc(__ballot_sync(QDKGB_FULL_MASK, hit));
        }
        __syncwarp();
      }
    }
    if (lane == 0) row_nnz[i] = cnt;
  }
}

// Emission into the pre-threshold slots: each row's kept elements are packed
// at the start of its slot range (ballot compaction), the kept count is
// recorded.  Values: the precomputed diagonal, or the off-diagonal element with
// the lower-index determinant as bra (sorted_double_loop.hpp:325-355).
template <int STORAGE>
__global__ void __launch_bounds__(kRowWarps * 32)
    k_row_emit(RowArgs a, const int32_t* __restrict__ rows, int64_t nrows, long long tbits,
               const double* __restrict__ diag_raw, const int64_t* __restrict__ rowptr, int64_t* __restrict__ kept,
               int32_t* __restrict__ colind, double* __restrict__ val, float* __restrict__ hi,
               float* __restrict__ lo, double* __restrict__ diag) {
  __shared__ RowWalkSmem sm;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int64_t i = (int64_t)blockIdx.x * kRowWarps + w; i < nrows; i += (int64_t)gridDim.x * kRowWarps) {
    const int64_t r = rows ? (int64_t)rows[i] : i;
    const int64_t start = rowptr[i];
    int64_t pos0 = start;
    walk_row(a, r, w, lane, sm, [&](int64_t ket, int64_t row, uint64_t ra, uint64_t rb, uint64_t ka, uint64_t kb) {
      bool keep = false;
      double v = 0.;
      if (ket >= 0) {
        if (ket == row) {
          v = diag_raw[row];
          keep = above_thresh(v, tbits);
          diag[row] = keep ? v : 0.;
        } else {
          v = (ket > row) ? offdiag_element(a.I, ra, rb, ka, kb) : offdiag_element(a.I, ka, kb, ra, rb);
          keep = above_thresh(v, tbits);
        }
      }
      const unsigned m = __ballot_sync(QDKGB_FULL_MASK, keep);
      if (keep) {
        const int64_t p = pos0 + __popc(m & ((1u << lane) - 1u));
        colind[p] = (int32_t)ket;
        if (STORAGE == QDKGB_H_FP64) {
          val[p] = v;
        } else {
          const float h = __double2float_rn(v);
          hi[p] = h;
          lo[p] = __double2float_rn(v - (double)h);
        }
      }
      pos0 += __popc(m);
    });
    if (lane == 0) kept[i] = pos0 - start;
  }
}

// Moves each row's kept prefix from its pre-threshold slot range to the final
// compact position (only when the threshold removed elements).
template <int STORAGE>
__global__ void k_row_compact(int64_t n, const int64_t* __restrict__ pre_ptr, const int64_t* __restrict__ new_ptr,
                              const int32_t* __restrict__ ci, const double* __restrict__ v,
                              const float* __restrict__ h, const float* __restrict__ l, int32_t* __restrict__ ci2,
                              double* __restrict__ v2, float* __restrict__ h2, float* __restrict__ l2) {
  const int lane = threadIdx.x & 31;
  const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = w0; r < n; r += nw) {
    const int64_t src = pre_ptr[r], dst = new_ptr[r], len = new_ptr[r + 1] - dst;
    for (int64_t k = lane; k < len; k += 32) {
      ci2[dst + k] = ci[src + k];
      if (STORAGE == QDKGB_H_FP64) {
        v2[dst + k] = v[src + k];
      } else {
        h2[dst + k] = h[src + k];
        l2[dst + k] = l[src + k];
      }
    }
  }
}

// extract_diagonal_elements (sparsexx/util/submatrix.hpp:354-384): first
// stored (i, i) element of each row, 0 when absent.  Warp per row.
__global__ void k_extract_diag(int64_t n, const int64_t* __restrict__ rowptr, const int32_t* __restrict__ colind,
                               const double* __restrict__ val, double* __restrict__ D) {
  const int lane = threadIdx.x & 31;
  const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = w0; r < n; r += nw) {
    const int64_t st = rowptr[r], en = rowptr[r + 1];
    int64_t found = -1;
    for (int64_t k0 = st; k0 < en && found < 0; k0 += 32) {
      const int64_t k = k0 + lane;
      const unsigned m = __ballot_sync(QDKGB_FULL_MASK, k < en && colind[k] == r);
      if (m) found = k0 + __ffs(m) - 1;
    }
    if (lane == 0) D[r] = (found >= 0) ? val[found] : 0.;
  }
}

// A caller's CSR matrix (0-based) becomes the device operator, FP64 storage
// (the matrix davidson_solver receives, pybind11/algorithms/davidson_solver.cpp:60-107).
void set_csr(Context* c, int64_t n, const int64_t* rowptr, const int64_t* colind, const double* values) {
  if (n <= 0) throw Error(QDKGB_ERR_INVALID, "empty matrix");
  if (n >= (int64_t)INT32_MAX) throw Error(QDKGB_ERR_UNSUPPORTED, "more than 2^31-1 rows");
  Hcsr& H = c->H;
  H.valid = false;
  H.structured = false;
  c->op_direct = false;
  c->fp32_direct = false;
  const int64_t nnz = rowptr[n] - rowptr[0];
  if (rowptr[0] != 0 || nnz < 0) throw Error(QDKGB_ERR_INVALID, "row pointers must start at 0 and not decrease");
  std::vector<int32_t> ci(std::max<int64_t>(nnz, 1));
  for (int64_t k = 0; k < nnz; ++k) {
    if (colind[k] < 0 || colind[k] >= n) throw Error(QDKGB_ERR_INVALID, "column index out of range");
    ci[k] = (int32_t)colind[k];
  }
  for (int64_t i = 0; i < n; ++i)
    if (rowptr[i + 1] < rowptr[i]) throw Error(QDKGB_ERR_INVALID, "row pointers must not decrease");
  dev_free(c, H.hi);
  dev_free(c, H.lo);
  int64_t* rp = dev_array<int64_t>(c, H.rowptr, n + 1);
  int32_t* dci = dev_array<int32_t>(c, H.colind, std::max<int64_t>(nnz, 1));
  double* dv = dev_array<double>(c, H.val, std::max<int64_t>(nnz, 1));
  double* D = dev_array<double>(c, H.diag, n);
  QDKGB_CUDA(cudaMemcpyAsync(rp, rowptr, (n + 1) * 8, cudaMemcpyHostToDevice, c->stream));
  if (nnz) {
    QDKGB_CUDA(cudaMemcpyAsync(dci, ci.data(), nnz * 4, cudaMemcpyHostToDevice, c->stream));
    QDKGB_CUDA(cudaMemcpyAsync(dv, values, nnz * 8, cudaMemcpyHostToDevice, c->stream));
  }
  const unsigned blocks = (unsigned)std::min<int64_t>((n + 7) / 8, (int64_t)c->sm_count * 32);
  k_extract_diag<<<blocks, 256, 0, c->stream>>>(n, rp, dci, dv, D);
  QDKGB_CHECK_LAUNCH();
  QDKGB_CUDA(cudaStreamSynchronize(c->stream));
  H.n = n;
  H.nnz = nnz;
  H.storage = QDKGB_H_FP64;
  H.thresh = 0.;
  H.valid = true;
}

RowArgs row_args(Context* c, double thresh) {
  DetSpace& D = c->dets;
  RowArgs a;
  a.I = integrals_view(c);
  a.ndets = D.ndets;
  a.galpha = (const uint64_t*)D.galpha.ptr;
  a.gstart = (const int64_t*)D.gstart.ptr;
  a.det_group = (const int32_t*)D.det_group.ptr;
  a.brank = (const int32_t*)D.brank.ptr;
  a.ubeta = (const uint64_t*)D.ubeta.ptr;
  a.gcomplete = (const uint8_t*)D.gcomplete.ptr;
  a.acon_ptr = (const int64_t*)D.acon_ptr.ptr;
  a.acon_idx = (const int32_t*)D.acon_idx.ptr;
  a.acon_lvl = (const int8_t*)D.acon_lvl.ptr;
  a.b2_ptr = (const int64_t*)D.b2_ptr.ptr;
  a.b2_idx = (const int32_t*)D.b2_idx.ptr;
  a.b1_ptr = (const int64_t*)D.b1_ptr.ptr;
  a.b1_idx = (const int32_t*)D.b1_idx.ptr;
  a.thresh = thresh;
  return a;
}

void check_dets_in_orbitals(const Context* c) {
  if (c->norb < 64 && (c->dets.occ_union >> c->norb))
    throw Error(QDKGB_ERR_INVALID, "a determinant occupies an orbital beyond the integrals' norb");
}

void build_hamiltonian(Context* c, double thresh, int storage) {
  NvtxRange nvtx_range("qdkgb.build_hamiltonian");
  if (!c->have_ints) throw Error(QDKGB_ERR_STATE, "integrals not set");
  if (!c->have_dets) throw Error(QDKGB_ERR_STATE, "determinants not set");
  check_dets_in_orbitals(c);
  if (storage != QDKGB_H_FP64 && storage != QDKGB_H_SPLIT32) throw Error(QDKGB_ERR_INVALID, "unknown storage");
  Hcsr& H = c->H;
  H.valid = false;
  H.structured = false;
  c->op_direct = false;
  c->fp32_direct = false;
  // slab layout for complete spaces; its kept rule (nonzero stored value)
  // needs every kept element to stay nonzero in the split pair
  if (c->fci && (!(thresh > 0.) || thresh >= 1e-30)) {
    // mixed form: the FP64 slab for the full-precision sigma and the direct
    // contraction for the FP32 one, where it applies (no FP32 copy stored)
    if (storage == QDKGB_H_SPLIT32) {
      build_hamiltonian_struct(c, thresh, QDKGB_H_FP64);
      if (H.structured && attach_direct_fp32(c)) {
        c->fp32_direct = true;
        return;
      }
    }
    build_hamiltonian_struct(c, thresh, storage);
    return;
  }
  DetSpace& D = c->dets;
  const int64_t n = D.ndets;
  RowArgs a = row_args(c, thresh);
  long long tbits = -1;
  if (thresh > 0.) {
    std::memcpy(&tbits, &thresh, sizeof(double));
  }
  int64_t* row_nnz = dev_array<int64_t>(c, H.row_nnz, n + 1);
  int64_t* rowptr = dev_array<int64_t>(c, H.rowptr, n + 1);
  double* diag_raw = dev_array<double>(c, H.diag_raw, n);
  double* diag = dev_array<double>(c, H.diag, n);
  const unsigned tblocks = (unsigned)std::min<int64_t>((n + 255) / 256, (int64_t)c->sm_count * 16);
  k_diag<<<tblocks, 256, 0, c->stream>>>(a.I, n, a.det_group, a.brank, a.galpha, a.ubeta, diag_raw);
  QDKGB_CHECK_LAUNCH();
  const int64_t blocks = std::min<int64_t>((n + kRowWarps - 1) / kRowWarps, (int64_t)c->sm_count * 64);
  k_row_count<<<(unsigned)blocks, kRowWarps * 32, 0, c->stream>>>(a, nullptr, n, row_nnz);
  QDKGB_CHECK_LAUNCH();
  exclusive_scan_i64(c, row_nnz, rowptr, n, H.scan_tmp);
  int64_t nnz_pre = 0;
  QDKGB_CUDA(cudaMemcpyAsync(&nnz_pre, rowptr + n, sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
  QDKGB_CUDA(cudaStreamSynchronize(c->stream));
  // release the other storage's arrays before allocating this one
  if (storage == QDKGB_H_FP64) {
    dev_free(c, H.hi);
    dev_free(c, H.lo);
  } else {
    dev_free(c, H.val);
  }
  const int64_t cap = std::max<int64_t>(nnz_pre, 1);
  int32_t* colind = dev_array<int32_t>(c, H.colind, cap);
  double* val = nullptr;
  float *hi = nullptr, *lo = nullptr;
  if (storage == QDKGB_H_FP64)
    val = dev_array<double>(c, H.val, cap);
  else {
    hi = dev_array<float>(c, H.hi, cap);
    lo = dev_array<float>(c, H.lo, cap);
  }
  QDKGB_CUDA(cudaMemsetAsync(diag, 0, n * sizeof(double), c->stream));
  // row_nnz now receives the kept counts
  if (storage == QDKGB_H_FP64)
    k_row_emit<QDKGB_H_FP64><<<(unsigned)blocks, kRowWarps * 32, 0, c->stream>>>(
        a, nullptr, n, tbits, diag_raw, rowptr, row_nnz, colind, val, hi, lo, diag);
  else
    k_row_emit<QDKGB_H_SPLIT32><<<(unsigned)blocks, kRowWarps * 32, 0, c->stream>>>(
        a, nullptr, n, tbits, diag_raw, rowptr, row_nnz, colind, val, hi, lo, diag);
  QDKGB_CHECK_LAUNCH();
  // kept total
  DeviceBuffer newptr_b, tmp;
  int64_t* newptr = dev_array<int64_t>(c, newptr_b, n + 1);
  exclusive_scan_i64(c, row_nnz, newptr, n, H.scan_tmp);
  int64_t nnz = 0;
  QDKGB_CUDA(cudaMemcpyAsync(&nnz, newptr + n, sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
  QDKGB_CUDA(cudaStreamSynchronize(c->stream));
  if (nnz != nnz_pre) {
    // threshold_parallel's compaction (csr_matrix.hpp:317-372), into fresh arrays
    DeviceBuffer ci2b, v2b, h2b, l2b;
    const int64_t cap2 = std::max<int64_t>(nnz, 1);
    int32_t* ci2 = dev_array<int32_t>(c, ci2b, cap2);
    double* v2 = storage == QDKGB_H_FP64 ? dev_array<double>(c, v2b, cap2) : nullptr;
    float* h2 = storage == QDKGB_H_SPLIT32 ? dev_array<float>(c, h2b, cap2) : nullptr;
    float* l2 = storage == QDKGB_H_SPLIT32 ? dev_array<float>(c, l2b, cap2) : nullptr;
    const unsigned cblocks = (unsigned)std::min<int64_t>((n + 7) / 8, (int64_t)c->sm_count * 32);
    if (storage == QDKGB_H_FP64)
      k_row_compact<QDKGB_H_FP64>
          <<<cblocks, 256, 0, c->stream>>>(n, rowptr, newptr, colind, val, hi, lo, ci2, v2, h2, l2);
    else
      k_row_compact<QDKGB_H_SPLIT32>
          <<<cblocks, 256, 0, c->stream>>>(n, rowptr, newptr, colind, val, hi, lo, ci2, v2, h2, l2);
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
  std::swap(H.rowptr, newptr_b);
  dev_free(c, newptr_b);
  dev_free(c, tmp);
  H.n = n;
  H.nnz = nnz;
  H.storage = storage;
  H.thresh = thresh;
  H.valid = true;
}


// ---------------------------------------------------------------- incremental build
// The reference's asci_iter patches the previous Hamiltonian instead of
// rebuilding it (PatchedSparseOperator / build_patched_operator,
// include/macis/solvers/incremental_h_build.hpp:38-356): kept x kept
// elements come from the old matrix, added rows and kept x added elements are
// computed.  Here the patch produces the full CSR of the new list, bit
// identical to a rebuild (the kept determinants keep their relative order,
// so every kept x kept element has the same bra and value; the new elements
// are computed with the lower-index determinant as bra, as a rebuild does):
//   1. the rows of added determinants are walked as in a full build;
//   2. their elements in kept columns are transposed into the kept rows
//      (counted, scattered, each row's list sorted by column);
//   3. every kept row is the merge of its old row (columns renumbered,
//      dropped determinants skipped) with its transposed list.
namespace {

constexpr int kSortCap = 1024;  // transposed list length sorted in shared memory

// transposed entries into the kept rows: counts
__global__ void k_patch_tcount(int64_t nw, const int64_t* __restrict__ rpA, const int32_t* __restrict__ ciA,
                               const uint8_t* __restrict__ walk, unsigned long long* __restrict__ tcnt) {
  const int lane = threadIdx.x & 31;
  for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < nw;
       i += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    for (int64_t e = rpA[i] + lane; e < rpA[i + 1]; e += 32) {
      const int32_t col = ciA[e];
      if (!walk[col]) atomicAdd(tcnt + col, 1ull);
    }
  }
}

// ... scattered (the order within a row is fixed afterwards by the sort)
__global__ void k_patch_tscatter(int64_t nw, const int32_t* __restrict__ rows, const int64_t* __restrict__ rpA,
                                 const int32_t* __restrict__ ciA, const double* __restrict__ vA,
                                 const uint8_t* __restrict__ walk, const int64_t* __restrict__ toff,
                                 unsigned long long* __restrict__ tcur, int32_t* __restrict__ tcol,
                                 double* __restrict__ tval) {
  const int lane = threadIdx.x & 31;
  for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < nw;
       i += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const int32_t w = rows[i];
    for (int64_t e = rpA[i] + lane; e < rpA[i + 1]; e += 32) {
      const int32_t col = ciA[e];
      if (walk[col]) continue;
      const int64_t p = toff[col] + (int64_t)atomicAdd(tcur + col, 1ull);
      tcol[p] = w;
      tval[p] = vA[e];
    }
  }
}

// sorts each kept row's transposed list by column (columns are distinct) with
// a bitonic sort in shared memory; a list above kSortCap goes to the long
// list (k_patch_tsort_long)
__global__ void __launch_bounds__(256) k_patch_tsort(int64_t n, const uint8_t* __restrict__ walk,
                                                     const int64_t* __restrict__ toff, int32_t* __restrict__ tcol,
                                                     double* __restrict__ tval, int32_t* __restrict__ long_rows,
                                                     unsigned* __restrict__ nlong) {
  __shared__ int32_t key[kSortCap];
  __shared__ int32_t src[kSortCap];
  __shared__ double vbuf[kSortCap];
  for (int64_t r = blockIdx.x; r < n; r += gridDim.x) {
    const int64_t b = toff[r], len = toff[r + 1] - b;
    if (walk[r] || len < 2) continue;
    if (len > kSortCap) {
      if (threadIdx.x == 0) long_rows[atomicAdd(nlong, 1u)] = (int32_t)r;
      continue;
    }
    int m = 1;
    while (m < len) m <<= 1;
    for (int t = threadIdx.x; t < m; t += blockDim.x) {
      key[t] = t < len ? tcol[b + t] : INT32_MAX;
      src[t] = t;
    }
    __syncthreads();
    for (int k = 2; k <= m; k <<= 1)
      for (int j = k >> 1; j > 0; j >>= 1) {
        for (int t = threadIdx.x; t < m; t += blockDim.x) {
          const int u = t ^ j;
          if (u > t) {
            const bool up = (t & k) == 0;
            if ((key[t] > key[u]) == up) {
              const int32_t kk = key[t];
              key[t] = key[u];
              key[u] = kk;
              const int32_t ss = src[t];
              src[t] = src[u];
              src[u] = ss;
            }
          }
        }
        __syncthreads();
      }
    for (int t = threadIdx.x; t < len; t += blockDim.x) vbuf[t] = tval[b + src[t]];
    __syncthreads();
    for (int t = threadIdx.x; t < len; t += blockDim.x) {
      tcol[b + t] = key[t];
      tval[b + t] = vbuf[t];
    }
    __syncthreads();
  }
}

// the long lists: a list's columns are added rows, so their walked-row
// indices widx (increasing with the column) mark a bitmap of nw bits; a
// column's place is the count of marks before it.  Each block owns one
// bitmap (words words) and its word prefix (words + 1).
__global__ void __launch_bounds__(256)
    k_patch_tsort_long(const int32_t* __restrict__ long_rows, const unsigned* __restrict__ nlong,
                       const int64_t* __restrict__ toff, const int32_t* __restrict__ widx, int64_t words,
                       unsigned* __restrict__ bitmaps, int64_t* __restrict__ prefixes, int32_t* __restrict__ tcol,
                       double* __restrict__ tval, int32_t* __restrict__ scol, double* __restrict__ sval) {
  __shared__ int64_t part[256];
  unsigned* bm = bitmaps + (int64_t)blockIdx.x * words;
  int64_t* pre = prefixes + (int64_t)blockIdx.x * (words + 1);
  const int64_t chunk = (words + blockDim.x - 1) / blockDim.x;
  const int64_t w0 = (int64_t)threadIdx.x * chunk < words ? (int64_t)threadIdx.x * chunk : words;
  const int64_t w1 = w0 + chunk < words ? w0 + chunk : words;
  for (unsigned q = blockIdx.x; q < *nlong; q += gridDim.x) {
    const int32_t r = long_rows[q];
    const int64_t b = toff[r], len = toff[r + 1] - b;
    for (int64_t w = threadIdx.x; w < words; w += blockDim.x) bm[w] = 0u;
    __syncthreads();
    for (int64_t e = threadIdx.x; e < len; e += blockDim.x) {
      const int32_t i = widx[tcol[b + e]];
      atomicOr(bm + (i >> 5), 1u << (i & 31));
    }
    __syncthreads();
    int64_t sum = 0;
    for (int64_t w = w0; w < w1; ++w) sum += __popc(bm[w]);
    part[threadIdx.x] = sum;
    __syncthreads();
    if (threadIdx.x == 0) {
      int64_t run = 0;
      for (int t = 0; t < (int)blockDim.x; ++t) {
        const int64_t x = part[t];
        part[t] = run;
        run += x;
      }
    }
    __syncthreads();
    int64_t run = part[threadIdx.x];
    for (int64_t w = w0; w < w1; ++w) {
      pre[w] = run;
      run += __popc(bm[w]);
    }
    __syncthreads();
    for (int64_t e = threadIdx.x; e < len; e += blockDim.x) {
      const int32_t col = tcol[b + e];
      const int32_t i = widx[col];
      const int64_t rank = pre[i >> 5] + __popc(bm[i >> 5] & ((1u << (i & 31)) - 1u));
      scol[b + rank] = col;
      sval[b + rank] = tval[b + e];
    }
    __syncthreads();
    for (int64_t e = threadIdx.x; e < len; e += blockDim.x) {
      tcol[b + e] = scol[b + e];
      tval[b + e] = sval[b + e];
    }
    __syncthreads();
  }
}

// kept entries of each merged row's old row
__global__ void k_patch_kcount(int64_t n, const uint8_t* __restrict__ walk, const int32_t* __restrict__ n2o,
                               const int64_t* __restrict__ rpO, const int32_t* __restrict__ ciO,
                               const int32_t* __restrict__ o2n, int64_t* __restrict__ kcnt) {
  const int lane = threadIdx.x & 31;
  for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < n;
       r += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    int64_t cnt = 0;
    if (!walk[r]) {
      const int32_t o = n2o[r];
      for (int64_t e = rpO[o] + lane; e < rpO[o + 1]; e += 32) cnt += o2n[ciO[e]] >= 0;
      for (int d = 16; d > 0; d >>= 1) cnt += __shfl_xor_sync(QDKGB_FULL_MASK, cnt, d);
    }
    if (lane == 0) kcnt[r] = cnt;
  }
}

// row lengths of the new matrix
__global__ void k_patch_rowlen(int64_t n, const uint8_t* __restrict__ walk, const int32_t* __restrict__ widx,
                               const int64_t* __restrict__ rpA, const int64_t* __restrict__ kcnt,
                               const unsigned long long* __restrict__ tcnt, int64_t* __restrict__ len) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    if (walk[r]) {
      const int32_t i = widx[r];
      len[r] = rpA[i + 1] - rpA[i];
    } else {
      len[r] = kcnt[r] + (int64_t)tcnt[r];
    }
  }
}

__device__ __forceinline__ int64_t lower_bound_i32(const int32_t* a, int64_t n, int32_t x) {
  int64_t lo = 0, hi = n;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (a[mid] < x)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo;
}

// the new rows: walked rows copied, kept rows merged (a warp per row; the
// kept entries' renumbered columns go to kcol, where the transposed entries
// find their places)
__global__ void k_patch_write(int64_t n, const uint8_t* __restrict__ walk, const int32_t* __restrict__ widx,
                              const int32_t* __restrict__ n2o, const int32_t* __restrict__ o2n,
                              const int64_t* __restrict__ rpO, const int32_t* __restrict__ ciO,
                              const double* __restrict__ vO, const int64_t* __restrict__ rpA,
                              const int32_t* __restrict__ ciA, const double* __restrict__ vA,
                              const int64_t* __restrict__ toff, const int32_t* __restrict__ tcol,
                              const double* __restrict__ tval, const int64_t* __restrict__ koff,
                              int32_t* __restrict__ kcol, const int64_t* __restrict__ rp, int32_t* __restrict__ ci,
                              double* __restrict__ v) {
  const int lane = threadIdx.x & 31;
  for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < n;
       r += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const int64_t base = rp[r];
    if (walk[r]) {
      const int32_t i = widx[r];
      const int64_t a0 = rpA[i], len = rpA[i + 1] - a0;
      for (int64_t e = lane; e < len; e += 32) {
        ci[base + e] = ciA[a0 + e];
        v[base + e] = vA[a0 + e];
      }
      continue;
    }
    const int32_t o = n2o[r];
    const int64_t e0 = rpO[o], e1 = rpO[o + 1];
    const int64_t t0 = toff[r], tl = toff[r + 1] - t0;
    int32_t* kr = kcol + koff[r];
    // kept entries, in order, after the transposed entries of smaller columns
    int64_t K = 0;
    for (int64_t c0 = e0; c0 < e1; c0 += 32) {
      const int64_t e = c0 + lane;
      const int32_t nc = e < e1 ? o2n[ciO[e]] : -1;
      const unsigned m = __ballot_sync(QDKGB_FULL_MASK, nc >= 0);
      if (nc >= 0) {
        const int64_t q = K + __popc(m & ((1u << lane) - 1u));
        kr[q] = nc;
        const int64_t pos = base + q + lower_bound_i32(tcol + t0, tl, nc);
        ci[pos] = nc;
        v[pos] = vO[e];
      }
      K += __popc(m);
    }
    __syncwarp();
    // transposed entries after the kept entries of smaller columns
    for (int64_t t = lane; t < tl; t += 32) {
      const int32_t j = tcol[t0 + t];
      const int64_t pos = base + t + lower_bound_i32(kr, K, j);
      ci[pos] = j;
      v[pos] = tval[t0 + t];
    }
    __syncwarp();
  }
}

}  // namespace

bool build_hamiltonian_patched(Context* c, double thresh, const std::vector<uint64_t>& oa,
                               const std::vector<uint64_t>& ob, DeviceBuffer& old_rowptr, DeviceBuffer& old_colind,
                               DeviceBuffer& old_val, double min_overlap) {
  NvtxRange nvtx_range("qdkgb.build_hamiltonian_patched");
  DetSpace& D = c->dets;
  const int64_t n = D.ndets, n_old = (int64_t)oa.size();
  if (n == 0 || n_old == 0 || n >= INT32_MAX || n_old >= INT32_MAX) return false;
  // classify by a merge scan of the two lists (both sorted by spin_comparator)
  std::vector<int32_t> o2n(n_old, -1), n2o(n, -1);
  int64_t kept = 0;
  for (int64_t io = 0, in = 0; io < n_old && in < n;) {
    const uint64_t xa = oa[io], xb = ob[io], ya = D.h_alpha[in], yb = D.h_beta[in];
    if (xa < ya || (xa == ya && xb < yb)) {
      ++io;
    } else if (ya < xa || (ya == xa && yb < xb)) {
      ++in;
    } else {
      o2n[io] = (int32_t)in;
      n2o[in] = (int32_t)io;
      ++kept;
      ++io;
      ++in;
    }
  }
  if ((double)kept / (double)n < min_overlap) return false;
  // walked rows: the added determinants
  std::vector<uint8_t> walk(n, 0);
  std::vector<int32_t> rows, widx(n, -1);
  for (int64_t r = 0; r < n; ++r)
    if (n2o[r] < 0) {
      walk[r] = 1;
      widx[r] = (int32_t)rows.size();
      rows.push_back((int32_t)r);
    }
  const int64_t nw = (int64_t)rows.size();
  ScopedBuffers<23> sb(c);
  auto up = [&](DeviceBuffer& b, const void* src, size_t bytes) {
    void* p = dev_alloc(c, b, std::max<size_t>(bytes, 8) + 16);
    if (bytes) QDKGB_CUDA(cudaMemcpyAsync(p, src, bytes, cudaMemcpyHostToDevice, c->stream));
    return p;
  };
  const int32_t* d_o2n = (const int32_t*)up(sb.b[0], o2n.data(), n_old * 4);
  const int32_t* d_n2o = (const int32_t*)up(sb.b[1], n2o.data(), n * 4);
  const uint8_t* d_walk = (const uint8_t*)up(sb.b[2], walk.data(), n);
  const int32_t* d_widx = (const int32_t*)up(sb.b[3], widx.data(), n * 4);
  const int32_t* d_rows = (const int32_t*)up(sb.b[4], rows.data(), nw * 4);
  Hcsr& H = c->H;
  RowArgs a = row_args(c, thresh);
  long long tbits = -1;
  if (thresh > 0.) std::memcpy(&tbits, &thresh, sizeof(double));
  double* diag_raw = dev_array<double>(c, H.diag_raw, n);
  double* diag = dev_array<double>(c, H.diag, n);
  const unsigned tblocks = (unsigned)std::min<int64_t>((n + 255) / 256, (int64_t)c->sm_count * 16);
  k_diag<<<tblocks, 256, 0, c->stream>>>(a.I, n, a.det_group, a.brank, a.galpha, a.ubeta, diag_raw);
  QDKGB_CHECK_LAUNCH();
  QDKGB_CUDA(cudaMemsetAsync(diag, 0, n * sizeof(double), c->stream));
  // 1. walked rows into A (pre-threshold slots, then compacted)
  int64_t* cntA = dev_array<int64_t>(c, sb.b[5], std::max<int64_t>(nw, n) + 1);
  int64_t* rpA0 = dev_array<int64_t>(c, sb.b[6], nw + 1);
  const int64_t wblocks =
      std::max<int64_t>(1, std::min<int64_t>((nw + kRowWarps - 1) / kRowWarps, (int64_t)c->sm_count * 64));
  int64_t nA0 = 0;
  if (nw) {
    k_row_count<<<(unsigned)wblocks, kRowWarps * 32, 0, c->stream>>>(a, d_rows, nw, cntA);
    QDKGB_CHECK_LAUNCH();
    exclusive_scan_i64(c, cntA, rpA0, nw, H.scan_tmp);
    QDKGB_CUDA(cudaMemcpyAsync(&nA0, rpA0 + nw, 8, cudaMemcpyDeviceToHost, c->stream));
    QDKGB_CUDA(cudaStreamSynchronize(c->stream));
  } else {
    QDKGB_CUDA(cudaMemsetAsync(rpA0, 0, 8, c->stream));
  }
  int32_t* ciA0 = dev_array<int32_t>(c, sb.b[7], std::max<int64_t>(nA0, 1));
  double* vA0 = dev_array<double>(c, sb.b[8], std::max<int64_t>(nA0, 1));
  int64_t* rpA = dev_array<int64_t>(c, sb.b[9], nw + 1);
  int64_t nA = 0;
  int32_t* ciA = ciA0;
  double* vA = vA0;
  if (nw) {
    k_row_emit<QDKGB_H_FP64><<<(unsigned)wblocks, kRowWarps * 32, 0, c->stream>>>(
        a, d_rows, nw, tbits, diag_raw, rpA0, cntA, ciA0, vA0, nullptr, nullptr, diag);
    QDKGB_CHECK_LAUNCH();
    exclusive_scan_i64(c, cntA, rpA, nw, H.scan_tmp);
    QDKGB_CUDA(cudaMemcpyAsync(&nA, rpA + nw, 8, cudaMemcpyDeviceToHost, c->stream));
    QDKGB_CUDA(cudaStreamSynchronize(c->stream));
    if (nA != nA0) {
      ciA = dev_array<int32_t>(c, sb.b[10], std::max<int64_t>(nA, 1));
      vA = dev_array<double>(c, sb.b[11], std::max<int64_t>(nA, 1));
      const unsigned cblocks = (unsigned)std::min<int64_t>((nw + 7) / 8, (int64_t)c->sm_count * 32);
      k_row_compact<QDKGB_H_FP64><<<cblocks, 256, 0, c->stream>>>(nw, rpA0, rpA, ciA0, vA0, nullptr, nullptr, ciA,
                                                                   vA, nullptr, nullptr);
      QDKGB_CHECK_LAUNCH();
    }
  } else {
    QDKGB_CUDA(cudaMemsetAsync(rpA, 0, 8, c->stream));
  }
  // 2. transposed entries into the merged rows
  unsigned long long* tcnt = dev_array<unsigned long long>(c, sb.b[12], 2 * (n + 1));
  unsigned long long* tcur = tcnt + n + 1;
  QDKGB_CUDA(cudaMemsetAsync(tcnt, 0, 2 * (n + 1) * 8, c->stream));
  const unsigned eblocks = (unsigned)std::max<int64_t>(1, std::min<int64_t>((nw + 7) / 8, (int64_t)c->sm_count * 32));
  if (nw) {
    k_patch_tcount<<<eblocks, 256, 0, c->stream>>>(nw, rpA, ciA, d_walk, tcnt);
    QDKGB_CHECK_LAUNCH();
  }
  int64_t* toff = dev_array<int64_t>(c, sb.b[13], n + 1);
  exclusive_scan_i64(c, (const int64_t*)tcnt, toff, n, H.scan_tmp);
  int64_t nT = 0;
  QDKGB_CUDA(cudaMemcpyAsync(&nT, toff + n, 8, cudaMemcpyDeviceToHost, c->stream));
  QDKGB_CUDA(cudaStreamSynchronize(c->stream));
  int32_t* tcol = dev_array<int32_t>(c, sb.b[14], std::max<int64_t>(nT, 1));
  double* tval = dev_array<double>(c, sb.b[15], std::max<int64_t>(nT, 1));
  if (nw) {
    k_patch_tscatter<<<eblocks, 256, 0, c->stream>>>(nw, d_rows, rpA, ciA, vA, d_walk, toff, tcur, tcol, tval);
    QDKGB_CHECK_LAUNCH();
  }
  // short lists sorted in shared memory; the long ones by the walked-row bitmap
  int32_t* long_rows = dev_array<int32_t>(c, sb.b[18], n + 2);
  unsigned* nlong = reinterpret_cast<unsigned*>(long_rows + n);
  QDKGB_CUDA(cudaMemsetAsync(nlong, 0, sizeof(unsigned), c->stream));
  k_patch_tsort<<<(unsigned)std::min<int64_t>(n, (int64_t)c->sm_count * 8), 256, 0, c->stream>>>(
      n, d_walk, toff, tcol, tval, long_rows, nlong);
  QDKGB_CHECK_LAUNCH();
  unsigned nlong_h = 0;
  QDKGB_CUDA(cudaMemcpyAsync(&nlong_h, nlong, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
  QDKGB_CUDA(cudaStreamSynchronize(c->stream));
  if (nlong_h) {
    const int64_t words = (nw + 31) / 32;
    const unsigned lblocks = (unsigned)std::min<int64_t>(nlong_h, c->sm_count);
    unsigned* bitmaps = dev_array<unsigned>(c, sb.b[19], (size_t)lblocks * words);
    int64_t* prefixes = dev_array<int64_t>(c, sb.b[20], (size_t)lblocks * (words + 1));
    int32_t* scol = dev_array<int32_t>(c, sb.b[21], nT);
    double* sval = dev_array<double>(c, sb.b[22], nT);
    k_patch_tsort_long<<<lblocks, 256, 0, c->stream>>>(long_rows, nlong, toff, d_widx, words, bitmaps, prefixes,
                                                       tcol, tval, scol, sval);
    QDKGB_CHECK_LAUNCH();
  }
  // 3. row lengths and the merged matrix
  int64_t* kcnt = cntA;  // the walked rows' counts are no longer needed
  const unsigned rblocks = (unsigned)std::min<int64_t>((n + 7) / 8, (int64_t)c->sm_count * 32);
  k_patch_kcount<<<rblocks, 256, 0, c->stream>>>(n, d_walk, d_n2o, (const int64_t*)old_rowptr.ptr,
                                                 (const int32_t*)old_colind.ptr, d_o2n, kcnt);
  QDKGB_CHECK_LAUNCH();
  int64_t* len = dev_array<int64_t>(c, H.row_nnz, n + 1);
  k_patch_rowlen<<<tblocks, 256, 0, c->stream>>>(n, d_walk, d_widx, rpA, kcnt, tcnt, len);
  QDKGB_CHECK_LAUNCH();
  int64_t* koff = dev_array<int64_t>(c, sb.b[16], n + 1);
  exclusive_scan_i64(c, kcnt, koff, n, H.scan_tmp);
  int64_t nK = 0;
  QDKGB_CUDA(cudaMemcpyAsync(&nK, koff + n, 8, cudaMemcpyDeviceToHost, c->stream));
  QDKGB_CUDA(cudaStreamSynchronize(c->stream));
  int32_t* kcol = dev_array<int32_t>(c, sb.b[17], std::max<int64_t>(nK, 1));
  DeviceBuffer rpb;
  int64_t* rp = dev_array<int64_t>(c, rpb, n + 1);
  exclusive_scan_i64(c, len, rp, n, H.scan_tmp);
  int64_t nnz = 0;
  QDKGB_CUDA(cudaMemcpyAsync(&nnz, rp + n, 8, cudaMemcpyDeviceToHost, c->stream));
  QDKGB_CUDA(cudaStreamSynchronize(c->stream));
  DeviceBuffer cib, vb;
  int32_t* ci = dev_array<int32_t>(c, cib, std::max<int64_t>(nnz, 1));
  double* v = dev_array<double>(c, vb, std::max<int64_t>(nnz, 1));
  k_patch_write<<<rblocks, 256, 0, c->stream>>>(n, d_walk, d_widx, d_n2o, d_o2n, (const int64_t*)old_rowptr.ptr,
                                                (const int32_t*)old_colind.ptr, (const double*)old_val.ptr, rpA, ciA,
                                                vA, toff, tcol, tval, koff, kcol, rp, ci, v);
  QDKGB_CHECK_LAUNCH();
  // the Davidson diagonal: first stored (i, i) element, 0 when thresholded away
  k_extract_diag<<<rblocks, 256, 0, c->stream>>>(n, rp, ci, v, diag);
  QDKGB_CHECK_LAUNCH();
  QDKGB_CUDA(cudaStreamSynchronize(c->stream));
  dev_free(c, H.hi);
  dev_free(c, H.lo);
  std::swap(H.rowptr, rpb);
  std::swap(H.colind, cib);
  std::swap(H.val, vb);
  dev_free(c, rpb);
  dev_free(c, cib);
  dev_free(c, vb);
  H.n = n;
  H.nnz = nnz;
  H.storage = QDKGB_H_FP64;
  H.thresh = thresh;
  H.structured = false;
  H.valid = true;
  c->op_direct = false;
  c->fp32_direct = false;
  return true;
}

}  // namespace qdkgb
