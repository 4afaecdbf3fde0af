// C ABI entry points (include/qdkgb.h).  Every function converts internal
// exceptions into a status code plus a message kept in the context.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <map>
#include <mutex>
#include <vector>

#include "internal.h"

#include <atomic>

namespace qdkgb {

static std::atomic<int64_t> g_launches{0};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

static thread_local std::string g_context_free_err;
void set_context_free_error(const std::string& msg) { g_context_free_err = msg; }

void set_max_dynamic_smem(const void* func, int bytes) {
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, int> done;
  int dev = 0;
  QDKGB_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(mu);
  const auto key = std::make_pair(func, dev);
  const auto it = done.find(key);
  if (it != done.end() && it->second >= bytes) return;
  QDKGB_CUDA(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  done[key] = bytes;
}

void* dev_alloc(Context* c, DeviceBuffer& b, size_t bytes) {
  if (b.ptr && b.bytes >= bytes) return b.ptr;
  dev_free(c, b);
  if (c->dev_limit > 0 && c->dev_bytes + (int64_t)bytes > c->dev_limit)
    throw Error(QDKGB_ERR_OOM, "device memory limit of " + std::to_string(c->dev_limit) + " bytes reached (" +
                                   std::to_string(c->dev_bytes) + " held, " + std::to_string(bytes) + " asked)");
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, std::max<size_t>(bytes, 16));
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    throw Error(QDKGB_ERR_OOM, "cudaMalloc of " + std::to_string(bytes) + " bytes failed: " + cudaGetErrorString(e));
  }
  b.ptr = p;
  b.bytes = bytes;
  c->dev_bytes += (int64_t)bytes;
  return p;
}

void dev_free(Context* c, DeviceBuffer& b) {
  if (b.ptr) {
    cudaFree(b.ptr);
    c->dev_bytes -= (int64_t)b.bytes;
  }
  b.ptr = nullptr;
  b.bytes = 0;
}

// generate_combs (sd_operations.hpp:305-323): std::prev_permutation order,
// i.e. combinations of occupied positions in lexicographic order.
static std::vector<uint64_t> combs(int nbits, int nset) {
  std::vector<uint64_t> out;
  std::vector<int> pos(nset);
  for (int i = 0; i < nset; ++i) pos[i] = i;
  while (true) {
    uint64_t s = 0;
    for (int p : pos) s |= 1ull << p;
    out.push_back(s);
    int i = nset - 1;
    while (i >= 0 && pos[i] == nbits - nset + i) --i;
    if (i < 0) break;
    pos[i]++;
    for (int j = i + 1; j < nset; ++j) pos[j] = pos[j - 1] + 1;
  }
  return out;
}

static int64_t binom(int n, int k) {
  if (k < 0 || k > n) return 0;
  long double r = 1;
  for (int i = 1; i <= k; ++i) r = r * (n - k + i) / i;
  return (int64_t)std::llround(r);
}

}  // namespace qdkgb

using namespace qdkgb;

template <class F>
static int guarded(qdkgb_context* ctx, F&& f) {
  try {
    f();
    if (ctx) ctx->err.clear();
    return QDKGB_OK;
  } catch (const Error& e) {
    if (ctx) ctx->err = e.what();
    return e.code;
  } catch (const std::bad_alloc&) {
    if (ctx) ctx->err = "host allocation failed";
    return QDKGB_ERR_OOM;
  } catch (const std::exception& e) {
    if (ctx) ctx->err = e.what();
    return QDKGB_ERR_INVALID;
  }
}

template <typename I>
static void get_csr(Context* c, I* rowptr, I* colind, double* values) {
  Hcsr& H = c->H;
  if (!H.valid || c->op_direct) throw Error(QDKGB_ERR_STATE, "no CSR Hamiltonian built");
  if (sizeof(I) == 4 && H.nnz > INT32_MAX) throw Error(QDKGB_ERR_UNSUPPORTED, "nnz exceeds int32");
  std::vector<int64_t> rp(H.n + 1);
  QDKGB_CUDA(cudaMemcpyAsync(rp.data(), H.rowptr.ptr, (H.n + 1) * 8, cudaMemcpyDeviceToHost, c->stream));
  std::vector<int32_t> ci;
  if (H.structured) {
    // slab layout: produce the CSR arrays on the device
    DeviceBuffer cib, vb;
    const int64_t cap = std::max<int64_t>(H.nnz, 1);
    int32_t* dci = dev_array<int32_t>(c, cib, cap);
    double* dv = dev_array<double>(c, vb, cap);
    struct_export(c, dci, dv, nullptr, nullptr);
    if (colind) {
      ci.resize(H.nnz);
      QDKGB_CUDA(cudaMemcpyAsync(ci.data(), dci, H.nnz * 4, cudaMemcpyDeviceToHost, c->stream));
    }
    if (values) QDKGB_CUDA(cudaMemcpyAsync(values, dv, H.nnz * 8, cudaMemcpyDeviceToHost, c->stream));
    QDKGB_CUDA(cudaStreamSynchronize(c->stream));
    dev_free(c, cib);
    dev_free(c, vb);
    values = nullptr;
  } else if (colind) {
    ci.resize(H.nnz);
    QDKGB_CUDA(cudaMemcpyAsync(ci.data(), H.colind.ptr, H.nnz * 4, cudaMemcpyDeviceToHost, c->stream));
  }
  if (values) {
    if (H.storage == QDKGB_H_FP64) {
      QDKGB_CUDA(cudaMemcpyAsync(values, H.val.ptr, H.nnz * 8, cudaMemcpyDeviceToHost, c->stream));
    } else {
      DeviceBuffer tmp;
      double* d = dev_array<double>(c, tmp, H.nnz);
      csr_values_to_double(c, d);
      QDKGB_CUDA(cudaMemcpyAsync(values, d, H.nnz * 8, cudaMemcpyDeviceToHost, c->stream));
      QDKGB_CUDA(cudaStreamSynchronize(c->stream));
      dev_free(c, tmp);
    }
  }
  QDKGB_CUDA(cudaStreamSynchronize(c->stream));
  if (rowptr)
    for (int64_t i = 0; i <= H.n; ++i) rowptr[i] = (I)rp[i];
  if (colind)
    for (int64_t i = 0; i < H.nnz; ++i) colind[i] = (I)ci[i];
}

// Stored elements of a complete (n, k_a, k_b) space: every row holds the
// diagonal, the singles and doubles of each spin and the alpha x beta singles.
static int64_t cas_row_elements(int n, int ka, int kb) {
  auto C2 = [](int64_t x) { return x * (x - 1) / 2; };
  const int64_t sa = (int64_t)ka * (n - ka), sb = (int64_t)kb * (n - kb);
  return 1 + sa + sb + C2(ka) * C2(n - ka) + C2(kb) * C2(n - kb) + sa * sb;
}

// Complete spaces from this many determinants up take the direct sigma for
// mixed-precision solves (QDKGB_H_SPLIT32): their FP32 sigma is the direct
// contraction whatever is stored, so a stored FP64 matrix would serve only the
// few full-precision refreshes of the solve, and emitting it costs more than
// recomputing them (853,776 determinants: 9.3 ms of emission, refreshes of
// 2.8 ms from the stored matrix against 3.75 ms recomputed, four refreshes).
constexpr int64_t kMixedDirectMinDets = (int64_t)1 << 17;

// The stored Hamiltonian when it fits in the device memory available to this
// context (free memory, and the cap of qdkgb_set_device_limit, counting what
// the current operator holds) beside the Davidson workspace of max_m
// vectors; otherwise, for a complete space the direct sigma serves.  A large
// complete space with QDKGB_H_SPLIT32 storage takes the direct sigma as well
// (kMixedDirectMinDets; QDKGB_MIXED_FP32=slab keeps the stored operator).
// Returns true when the direct sigma was built.
bool qdkgb::build_operator(Context* c, double thresh, int storage, int max_m) {
  const DetSpace& S = c->dets;
  if (!c->have_dets) throw Error(QDKGB_ERR_STATE, "determinants not set");
  bool complete = S.product && S.ngroups > 0;
  for (int64_t g = 0; complete && g < S.ngroups; ++g) complete = S.h_gstart[g] == g * S.nbeta;
  if (complete && !S.h_galpha.empty() && !S.h_ubeta.empty()) {
    const int n = c->norb;
    const int ka = __builtin_popcountll(S.h_galpha[0]), kb = __builtin_popcountll(S.h_ubeta[0]);
    const double N = (double)S.ndets;
    const double stored = N * (double)cas_row_elements(n, ka, kb) * (storage == QDKGB_H_SPLIT32 ? 12.0 : 8.0);
    const double work = N * 8.0 * (2.0 * (std::max(max_m, 2) + 1) + 16.0);
    size_t fr = 0, tot = 0;
    QDKGB_CUDA(cudaMemGetInfo(&fr, &tot));
    double held = 0;
    for (const DeviceBuffer* b : {&c->H.rowptr, &c->H.colind, &c->H.val, &c->H.hi, &c->H.lo})
      held += (double)b->bytes;
    double avail = (double)fr + held;
    if (c->dev_limit > 0) avail = std::min(avail, (double)(c->dev_limit - c->dev_bytes) + held);
    const bool direct_ok = n <= 20 && S.ngroups <= 4096 && S.nbeta <= 4096 && ka > 0 && kb > 0;
    const char* keep = std::getenv("QDKGB_MIXED_FP32");
    const bool mixed_direct = storage == QDKGB_H_SPLIT32 && S.ndets >= kMixedDirectMinDets &&
                              !(keep && std::string(keep) == "slab");
    if (direct_ok && (mixed_direct || stored + work > 0.92 * avail)) {
      build_direct_sigma(c);
      return true;
    }
  }
  build_hamiltonian(c, thresh, storage);
  return false;
}

// Rows [r0, r1) of the device CSR: rowptr (r1 - r0 + 1 entries) relative to
// the block's first element, as a bra block of make_csr_hamiltonian_block_
// returns it; colind are global columns.
template <typename I>
static void get_csr_rows(Context* c, int64_t r0, int64_t r1, I* rowptr, I* colind, double* values) {
  Hcsr& H = c->H;
  if (!H.valid || c->op_direct) throw Error(QDKGB_ERR_STATE, "no CSR Hamiltonian built");
  if (r0 < 0 || r1 < r0 || r1 > H.n) throw Error(QDKGB_ERR_INVALID, "row range outside [0, ndets]");
  std::vector<int64_t> rp(r1 - r0 + 1);
  QDKGB_CUDA(cudaMemcpyAsync(rp.data(), (const int64_t*)H.rowptr.ptr + r0, (r1 - r0 + 1) * 8,
                             cudaMemcpyDeviceToHost, c->stream));
  QDKGB_CUDA(cudaStreamSynchronize(c->stream));
  const int64_t e0 = rp.front(), cnt = rp.back() - rp.front();
  if (sizeof(I) == 4 && cnt > INT32_MAX) throw Error(QDKGB_ERR_UNSUPPORTED, "block nnz exceeds int32");
  std::vector<int32_t> ci(colind ? cnt : 0);
  DeviceBuffer cib, vb;
  const int32_t* dci = (const int32_t*)H.colind.ptr;
  const double* dv = (H.storage == QDKGB_H_FP64 && !H.structured) ? (const double*)H.val.ptr : nullptr;
  if (H.structured) {
    // slab layout: the CSR arrays are produced on the device, then sliced
    const int64_t cap = std::max<int64_t>(H.nnz, 1);
    int32_t* tci = dev_array<int32_t>(c, cib, cap);
    double* tv = dev_array<double>(c, vb, cap);
    struct_export(c, tci, tv, nullptr, nullptr);
    dci = tci;
    dv = tv;
  } else if (!dv && values) {
    double* tv = dev_array<double>(c, vb, std::max<int64_t>(H.nnz, 1));
    csr_values_to_double(c, tv);
    dv = tv;
  }
  if (colind && cnt)
    QDKGB_CUDA(cudaMemcpyAsync(ci.data(), dci + e0, cnt * 4, cudaMemcpyDeviceToHost, c->stream));
  if (values && cnt)
    QDKGB_CUDA(cudaMemcpyAsync(values, dv + e0, cnt * 8, cudaMemcpyDeviceToHost, c->stream));
  QDKGB_CUDA(cudaStreamSynchronize(c->stream));
  dev_free(c, cib);
  dev_free(c, vb);
  if (rowptr)
    for (int64_t i = 0; i <= r1 - r0; ++i) rowptr[i] = (I)(rp[i] - e0);
  if (colind)
    for (int64_t i = 0; i < cnt; ++i) colind[i] = (I)ci[i];
}

extern "C" {

const char* qdkgb_version(void) { return "qdkgb 0.1 (sm_103a)"; }

int64_t qdkgb_kernel_launches(void) { return g_launches.load(); }

int qdkgb_create(qdkgb_context** out, int device) {
  if (!out) return QDKGB_ERR_INVALID;
  *out = nullptr;
  qdkgb_context* c = new (std::nothrow) qdkgb_context();
  if (!c) return QDKGB_ERR_OOM;
  int rc = guarded(c, [&] {
    int ndev = 0;
    QDKGB_CUDA(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) throw Error(QDKGB_ERR_INVALID, "no such CUDA device");
    QDKGB_CUDA(cudaSetDevice(device));
    c->device = device;
    QDKGB_CUDA(cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device));
    QDKGB_CUDA(cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking));
    c->stream = c->own_stream;
    QDKGB_CUDA(cudaMallocHost((void**)&c->pinned, 64 * sizeof(double)));
  });
  if (rc != QDKGB_OK) {
    delete c;
    return rc;
  }
  *out = c;
  return QDKGB_OK;
}

int qdkgb_destroy(qdkgb_context* c) {
  if (!c) return QDKGB_OK;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  for (DeviceBuffer* b : {&c->T, &c->V, &c->G_red, &c->V_red, &c->G2, &c->V2, &c->dets.galpha, &c->dets.gstart,
                          &c->dets.det_group, &c->dets.brank, &c->dets.ubeta, &c->dets.gcomplete, &c->dets.acon_ptr,
                          &c->dets.acon_idx, &c->dets.acon_lvl, &c->dets.b2_ptr, &c->dets.b2_idx, &c->dets.b1_ptr,
                          &c->dets.b1_idx, &c->H.rowptr, &c->H.colind, &c->H.val, &c->H.hi, &c->H.lo, &c->H.diag, &c->H.diag_raw,
                          &c->H.row_nnz, &c->H.scan_tmp, &c->H.xsplit, &c->dav.V, &c->dav.AV, &c->dav.xf, &c->dav.yf, &c->dav.Hk,
                          &c->dav.evec, &c->dav.eval, &c->dav.scratch, &c->dav.partial, &c->dav.small})
    dev_free(c, *b);
  free_direct(c);
  free_struct(c);
  if (c->pinned) cudaFreeHost(c->pinned);
  if (c->own_stream) cudaStreamDestroy(c->own_stream);
  delete c;
  return QDKGB_OK;
}

const char* qdkgb_last_error(const qdkgb_context* c) { return c ? c->err.c_str() : g_context_free_err.c_str(); }

int qdkgb_set_stream(qdkgb_context* c, void* stream) {
  if (!c) return QDKGB_ERR_INVALID;
  return guarded(c, [&] {
    QDKGB_CUDA(cudaStreamSynchronize(c->stream));
    c->stream = stream ? (cudaStream_t)stream : c->own_stream;
  });
}

int qdkgb_set_device_limit(qdkgb_context* c, int64_t bytes) {
  if (!c || bytes < 0) return QDKGB_ERR_INVALID;
  c->dev_limit = bytes;
  return QDKGB_OK;
}

int qdkgb_device_bytes(const qdkgb_context* c, int64_t* bytes) {
  if (!c || !bytes) return QDKGB_ERR_INVALID;
  *bytes = c->dev_bytes;
  return QDKGB_OK;
}

int qdkgb_problem_size(const qdkgb_context* c, int64_t* ndets, int64_t* nnz) {
  if (!c) return QDKGB_ERR_INVALID;
  if (ndets) *ndets = c->H.valid ? c->H.n : (c->have_dets ? c->dets.ndets : 0);
  if (nnz) *nnz = (c->H.valid && !c->op_direct) ? c->H.nnz : 0;
  return QDKGB_OK;
}

int qdkgb_direct_plan(const qdkgb_context* c, int* contraction, int* dense, double* form_ms) {
  if (!c) return QDKGB_ERR_INVALID;
  direct_plan(c, contraction, dense, form_ms);
  return QDKGB_OK;
}

int qdkgb_operator_layout(const qdkgb_context* c, int* layout, int64_t* stored) {
  if (!c || !layout) return QDKGB_ERR_INVALID;
  const Hcsr& H = c->H;
  int64_t st = 0;
  if (!H.valid) {
    *layout = QDKGB_LAYOUT_NONE;
  } else if (c->op_direct) {
    *layout = QDKGB_LAYOUT_DIRECT;
  } else if (H.structured) {
    *layout = c->fp32_direct ? QDKGB_LAYOUT_SLAB_DIRECT32 : QDKGB_LAYOUT_SLAB;
    st = struct_slab_elements(const_cast<qdkgb_context*>(c));
  } else {
    *layout = QDKGB_LAYOUT_CSR;
    st = H.nnz;
  }
  if (stored) *stored = st;
  return QDKGB_OK;
}

int qdkgb_set_integrals(qdkgb_context* c, int norb, const double* T, const double* V, int layout) {
  if (!c) return QDKGB_ERR_INVALID;
  return guarded(c, [&] {
    if (norb <= 0 || norb > 64) throw Error(QDKGB_ERR_INVALID, "norb must be in [1, 64]");
    if (!T || !V) throw Error(QDKGB_ERR_INVALID, "null integral buffer");
    if (layout != QDKGB_LAYOUT_COLMAJOR && layout != QDKGB_LAYOUT_ROWMAJOR)
      throw Error(QDKGB_ERR_INVALID, "unknown integral layout");
    QDKGB_CUDA(cudaSetDevice(c->device));
    const size_t n = norb, n2 = n * n, n4 = n2 * n2;
    c->h_T.resize(n2);
    c->h_V.resize(n4);
    if (layout == QDKGB_LAYOUT_COLMAJOR) {
      std::memcpy(c->h_T.data(), T, n2 * 8);
      std::memcpy(c->h_V.data(), V, n4 * 8);
    } else {
      // qdk's row-major i*n^3 + j*n^2 + k*n + l buffer -> column-major
      for (size_t p = 0; p < n; ++p)
        for (size_t q = 0; q < n; ++q) c->h_T[p + n * q] = T[p * n + q];
      for (size_t p = 0; p < n; ++p)
        for (size_t q = 0; q < n; ++q)
          for (size_t r = 0; r < n; ++r)
            for (size_t s = 0; s < n; ++s) c->h_V[p + n * (q + n * (r + n * s))] = V[((p * n + q) * n + r) * n + s];
    }
    c->norb = norb;
    build_integral_intermediates(c);
    c->have_ints = true;
    c->H.valid = false;
  });
}

int qdkgb_fci_dets(int norb, int nalpha, int nbeta, uint64_t* alpha, uint64_t* beta, int64_t* ndets) {
  if (norb <= 0 || norb > 64 || nalpha < 0 || nbeta < 0 || nalpha > norb || nbeta > norb || !ndets)
    return QDKGB_ERR_INVALID;
  const int64_t na = binom(norb, nalpha), nb = binom(norb, nbeta);
  *ndets = na * nb;
  if (!alpha) return QDKGB_OK;
  if (!beta) return QDKGB_ERR_INVALID;
  try {
    std::vector<uint64_t> A = combs(norb, nalpha), B = combs(norb, nbeta);
    for (int64_t i = 0; i < na; ++i)
      for (int64_t j = 0; j < nb; ++j) {
        alpha[i * nb + j] = A[i];
        beta[i * nb + j] = B[j];
      }
  } catch (...) {
    return QDKGB_ERR_OOM;
  }
  return QDKGB_OK;
}

int qdkgb_set_dets(qdkgb_context* c, int64_t ndets, const uint64_t* alpha, const uint64_t* beta) {
  if (!c) return QDKGB_ERR_INVALID;
  return guarded(c, [&] {
    if (!alpha || !beta) throw Error(QDKGB_ERR_INVALID, "null determinant buffer");
    QDKGB_CUDA(cudaSetDevice(c->device));
    build_det_space(c, ndets, alpha, beta);
  });
}

int qdkgb_build_hamiltonian(qdkgb_context* c, double thresh, int storage, int64_t* nnz) {
  if (!c) return QDKGB_ERR_INVALID;
  return guarded(c, [&] {
    QDKGB_CUDA(cudaSetDevice(c->device));
    build_hamiltonian(c, thresh, storage);
    if (nnz) *nnz = c->H.nnz;
  });
}

int qdkgb_get_csr32(qdkgb_context* c, int32_t* rowptr, int32_t* colind, double* values) {
  if (!c) return QDKGB_ERR_INVALID;
  return guarded(c, [&] { get_csr<int32_t>(c, rowptr, colind, values); });
}
int qdkgb_get_csr64(qdkgb_context* c, int64_t* rowptr, int64_t* colind, double* values) {
  if (!c) return QDKGB_ERR_INVALID;
  return guarded(c, [&] { get_csr<int64_t>(c, rowptr, colind, values); });
}

int qdkgb_get_csr32_rows(qdkgb_context* c, int64_t r0, int64_t r1, int32_t* rowptr, int32_t* colind,
                         double* values) {
  if (!c) return QDKGB_ERR_INVALID;
  return guarded(c, [&] { get_csr_rows<int32_t>(c, r0, r1, rowptr, colind, values); });
}
int qdkgb_get_csr64_rows(qdkgb_context* c, int64_t r0, int64_t r1, int64_t* rowptr, int64_t* colind,
                         double* values) {
  if (!c) return QDKGB_ERR_INVALID;
  return guarded(c, [&] { get_csr_rows<int64_t>(c, r0, r1, rowptr, colind, values); });
}

int qdkgb_set_csr(qdkgb_context* c, int64_t n, const int64_t* rowptr, const int64_t* colind, const double* values) {
  if (!c) return QDKGB_ERR_INVALID;
  return guarded(c, [&] {
    if (!rowptr || (!colind && n > 0) || (!values && n > 0)) throw Error(QDKGB_ERR_INVALID, "null CSR buffer");
    QDKGB_CUDA(cudaSetDevice(c->device));
    set_csr(c, n, rowptr, colind, values);
  });
}

int qdkgb_build_direct_sigma(qdkgb_context* c) {
  if (!c) return QDKGB_ERR_INVALID;
  return guarded(c, [&] {
    QDKGB_CUDA(cudaSetDevice(c->device));
    build_direct_sigma(c);
  });
}

int qdkgb_diagonal(qdkgb_context* c, double* D) {
  if (!c) return QDKGB_ERR_INVALID;
  return guarded(c, [&] {
    if (!c->H.valid) throw Error(QDKGB_ERR_STATE, "Hamiltonian not built");
    QDKGB_CUDA(cudaMemcpyAsync(D, c->H.diag.ptr, c->H.n * 8, cudaMemcpyDeviceToHost, c->stream));
    QDKGB_CUDA(cudaStreamSynchronize(c->stream));
  });
}

int qdkgb_spmv_device(qdkgb_context* c, int precision, const void* x, void* y) {
  if (!c) return QDKGB_ERR_INVALID;
  return guarded(c, [&] {
    if (precision == QDKGB_PREC_FP64)
      spmv_fp64(c, (const double*)x, (double*)y);
    else if (precision == QDKGB_PREC_MIXED)
      spmv_fp32(c, (const float*)x, (float*)y);
    else
      throw Error(QDKGB_ERR_INVALID, "unknown precision");
  });
}

int qdkgb_spmv(qdkgb_context* c, int precision, const double* x, double* y) {
  if (!c) return QDKGB_ERR_INVALID;
  return guarded(c, [&] {
    Hcsr& H = c->H;
    if (!H.valid) throw Error(QDKGB_ERR_STATE, "Hamiltonian not built");
    DeviceBuffer bx, by;
    const int64_t n = H.n;
    double* dx = dev_array<double>(c, bx, n);
    double* dy = dev_array<double>(c, by, n);
    QDKGB_CUDA(cudaMemcpyAsync(dx, x, n * 8, cudaMemcpyHostToDevice, c->stream));
    if (precision == QDKGB_PREC_FP64) {
      spmv_fp64(c, dx, dy);
    } else if (precision == QDKGB_PREC_MIXED) {
      DeviceBuffer bf;
      float* xf = dev_array<float>(c, bf, 2 * n);
      f64_to_f32(c, dx, xf, n);
      spmv_fp32(c, xf, xf + n);
      f32_to_f64(c, xf + n, dy, n);
      QDKGB_CUDA(cudaStreamSynchronize(c->stream));
      dev_free(c, bf);
    } else {
      throw Error(QDKGB_ERR_INVALID, "unknown precision");
    }
    QDKGB_CUDA(cudaMemcpyAsync(y, dy, n * 8, cudaMemcpyDeviceToHost, c->stream));
    QDKGB_CUDA(cudaStreamSynchronize(c->stream));
    dev_free(c, bx);
    dev_free(c, by);
  });
}

void qdkgb_davidson_default_settings(qdkgb_davidson_settings* s) {
  if (!s) return;
  s->max_m = 200;
  s->res_tol = 1e-8;
  s->precision = QDKGB_PREC_FP64;
  s->use_guess = 0;
  s->min_abs_denominator = 1e-12;
  s->nroots = 1;
}

int qdkgb_davidson(qdkgb_context* c, const qdkgb_davidson_settings* s, double* E, double* C,
                   qdkgb_davidson_info* info) {
  if (!c) return QDKGB_ERR_INVALID;
  return guarded(c, [&] {
    if (!E) throw Error(QDKGB_ERR_INVALID, "null energy pointer");
    qdkgb_davidson_settings def;
    qdkgb_davidson_default_settings(&def);
    QDKGB_CUDA(cudaSetDevice(c->device));
    davidson(c, s ? s : &def, E, C, info);
  });
}

int qdkgb_operator_action(qdkgb_context* c, int64_t m, double alpha, const double* V, int64_t ldv, double beta,
                          double* AV, int64_t ldav) {
  if (!c) return QDKGB_ERR_INVALID;
  return guarded(c, [&] {
    Hcsr& H = c->H;
    if (!H.valid) throw Error(QDKGB_ERR_STATE, "Hamiltonian not built");
    const int64_t n = H.n;
    if (m < 0 || (m > 0 && (!V || !AV || ldv < n || ldav < n))) throw Error(QDKGB_ERR_INVALID, "bad block shape");
    if (m == 0) return;
    QDKGB_CUDA(cudaSetDevice(c->device));
    ScopedBuffers<2> buf(c);
    double* dx = dev_array<double>(c, buf.b[0], n);
    double* dy = dev_array<double>(c, buf.b[1], n);
    std::vector<double> y(n);
    for (int64_t j = 0; j < m; ++j) {
      QDKGB_CUDA(cudaMemcpyAsync(dx, V + j * ldv, n * 8, cudaMemcpyHostToDevice, c->stream));
      spmv_fp64(c, dx, dy);
      QDKGB_CUDA(cudaMemcpyAsync(y.data(), dy, n * 8, cudaMemcpyDeviceToHost, c->stream));
      QDKGB_CUDA(cudaStreamSynchronize(c->stream));
      double* out = AV + j * ldav;
      if (beta == 0.)
        for (int64_t i = 0; i < n; ++i) out[i] = alpha * y[i];
      else
        for (int64_t i = 0; i < n; ++i) out[i] = alpha * y[i] + beta * out[i];
    }
  });
}

int qdkgb_rdms(qdkgb_context* c, const double* C, double* ordm, double* trdm) {
  if (!c) return QDKGB_ERR_INVALID;
  return guarded(c, [&] {
    if (!C) throw Error(QDKGB_ERR_INVALID, "null CI vector");
    if (!c->have_dets) throw Error(QDKGB_ERR_STATE, "determinants not set");
    if (!c->have_ints) throw Error(QDKGB_ERR_STATE, "integrals not set (needed for the orbital count)");
    if (!ordm && !trdm) return;
    QDKGB_CUDA(cudaSetDevice(c->device));
    const size_t n = (size_t)c->norb, n2 = n * n, n4 = n2 * n2;
    std::vector<double> aa(ordm ? n2 : 0), bb(ordm ? n2 : 0), aaaa(trdm ? n4 : 0), bbbb(trdm ? n4 : 0),
        aabb(trdm ? n4 : 0);
    rdms_spin_dep(c, C, ordm ? aa.data() : nullptr, ordm ? bb.data() : nullptr, trdm ? aaaa.data() : nullptr,
                  trdm ? bbbb.data() : nullptr, trdm ? aabb.data() : nullptr);
    if (ordm)
      for (size_t i = 0; i < n2; ++i) ordm[i] += aa[i] + bb[i];
    if (trdm)
      for (size_t pq = 0; pq < n2; ++pq)
        for (size_t rs = 0; rs < n2; ++rs) {
          const size_t i = pq + n2 * rs;
          trdm[i] += aaaa[i] + bbbb[i] + aabb[i] + aabb[rs + n2 * pq];
        }
  });
}

int qdkgb_rdms_spin_dep(qdkgb_context* c, const double* C, double* aa, double* bb, double* aaaa, double* bbbb,
                        double* aabb) {
  if (!c) return QDKGB_ERR_INVALID;
  return guarded(c, [&] {
    if (!C) throw Error(QDKGB_ERR_INVALID, "null CI vector");
    if (!c->have_dets) throw Error(QDKGB_ERR_STATE, "determinants not set");
    QDKGB_CUDA(cudaSetDevice(c->device));
    rdms_spin_dep(c, C, aa, bb, aaaa, bbbb, aabb);
  });
}

int qdkgb_orbital_entropies(qdkgb_context* c, const double* C, double* s1, double* s2, double* mi) {
  if (!c) return QDKGB_ERR_INVALID;
  return guarded(c, [&] {
    if (!C || !s1) throw Error(QDKGB_ERR_INVALID, "null argument");
    if (!c->have_dets) throw Error(QDKGB_ERR_STATE, "determinants not set");
    QDKGB_CUDA(cudaSetDevice(c->device));
    orbital_entropies(c, C, s1, s2, mi);
  });
}

void qdkgb_mcscf_default_settings(qdkgb_mcscf_settings* s) {
  if (!s) return;
  s->max_macro_iter = 100;
  s->max_orbital_step = 0.5;
  s->orb_grad_tol = 5e-6;
  s->enable_diis = 1;
  s->diis_start_iter = 3;
  s->diis_nkeep = 10;
  s->ci_res_tol = 1e-8;
  s->ci_max_subspace = 200;
  s->ci_matel_tol = std::numeric_limits<double>::epsilon();
}

int qdkgb_casscf(qdkgb_context* c, const qdkgb_mcscf_settings* s, int nalpha, int nbeta, int norb, int ninact,
                 int nact, double E_core, const double* T, const double* V, double* A1, double* A2, double* E,
                 double* U, int64_t* iterations, int* converged) {
  if (!c) return QDKGB_ERR_INVALID;
  return guarded(c, [&] {
    if (!T || !V || !A1 || !A2 || !E) throw Error(QDKGB_ERR_INVALID, "null argument");
    qdkgb_mcscf_settings def;
    qdkgb_mcscf_default_settings(&def);
    QDKGB_CUDA(cudaSetDevice(c->device));
    *E = casscf(c, s ? *s : def, nalpha, nbeta, norb, ninact, nact, E_core, T, V, A1, A2, U, iterations, converged);
  });
}

void qdkgb_asci_default_settings(qdkgb_asci_settings* s) {
  if (!s) return;
  s->ntdets_max = 100000;
  s->ntdets_min = 100;
  s->ncdets_max = 100;
  s->core_selection_fixed = 0;
  s->core_selection_threshold = 0.95;
  s->h_el_tol = 1e-8;
  s->rv_prune_tol = 1e-8;
  s->grow_factor = 8.0;
  s->min_grow_factor = 1.01;
  s->growth_backoff_rate = 0.5;
  s->growth_recovery_rate = 1.1;
  s->max_refine_iter = 6;
  s->refine_energy_tol = 1e-6;
  s->warm_start = 1;
  s->min_warm_start_overlap = 0.5;
  s->taper_grow_factor = 0.0;
  s->just_singles = 0;
  s->min_patch_overlap = 0.3;
  s->grow_with_rot = 0;
  s->rot_size_start = 1000;
}

int qdkgb_asci_rotation(const qdkgb_context* c, double* U) {
  if (!c || !U) return QDKGB_ERR_INVALID;
  const int n = c->norb;
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i)
      U[i + (size_t)n * j] = c->asci_rot.empty() ? (i == j ? 1. : 0.) : c->asci_rot[i + (size_t)n * j];
  return QDKGB_OK;
}

int qdkgb_asci_search(qdkgb_context* c, const qdkgb_asci_settings* s, int64_t ncore, const uint64_t* ca,
                      const uint64_t* cb, const double* cc, double E0, int64_t ndets_max, int64_t cap, uint64_t* out_a,
                      uint64_t* out_b, int64_t* n_out) {
  if (!c) return QDKGB_ERR_INVALID;
  return guarded(c, [&] {
    if (!s || !ca || !cb || !cc || !n_out) throw Error(QDKGB_ERR_INVALID, "null argument");
    QDKGB_CUDA(cudaSetDevice(c->device));
    std::vector<uint64_t> a, b;
    asci_search_gpu(c, ncore, ca, cb, cc, E0, ndets_max, s->h_el_tol, s->rv_prune_tol, a, b, nullptr,
                    s->just_singles != 0);
    *n_out = (int64_t)a.size();
    for (int64_t i = 0; i < std::min<int64_t>((int64_t)a.size(), cap); ++i) {
      if (out_a) out_a[i] = a[i];
      if (out_b) out_b[i] = b[i];
    }
  });
}

int qdkgb_asci_pt2(qdkgb_context* c, int64_t ndets, const uint64_t* alpha, const uint64_t* beta, const double* C,
                   double E0, double pt2_tol, int64_t max_slots, double* ept2, int64_t* n_external) {
  if (!c) return QDKGB_ERR_INVALID;
  return guarded(c, [&] {
    if (!alpha || !beta || !C || !ept2 || ndets <= 0) throw Error(QDKGB_ERR_INVALID, "null argument");
    if (!(pt2_tol >= 0.)) throw Error(QDKGB_ERR_INVALID, "pt2_tol must be >= 0");
    QDKGB_CUDA(cudaSetDevice(c->device));
    if (max_slots < 0) throw Error(QDKGB_ERR_INVALID, "max_slots must be >= 0");
    *ept2 = asci_pt2_gpu(c, ndets, alpha, beta, C, E0, pt2_tol, max_slots, n_external);
  });
}

int qdkgb_asci(qdkgb_context* c, const qdkgb_asci_settings* s, const qdkgb_davidson_settings* ci, double matel_tol,
               int64_t n0, const uint64_t* a0, const uint64_t* b0, const double* c0, double E0, int do_grow,
               int do_refine, int64_t cap, uint64_t* out_a, uint64_t* out_b, double* out_c, int64_t* n_out,
               double* E_out, double* E_grow_out) {
  if (!c) return QDKGB_ERR_INVALID;
  return guarded(c, [&] {
    if (!s || !a0 || !b0 || !c0 || n0 <= 0 || !n_out || !E_out) throw Error(QDKGB_ERR_INVALID, "null argument");
    if (!c->have_ints) throw Error(QDKGB_ERR_STATE, "integrals not set");
    QDKGB_CUDA(cudaSetDevice(c->device));
    qdkgb_davidson_settings def;
    qdkgb_davidson_default_settings(&def);
    std::vector<uint64_t> a(a0, a0 + n0), b(b0, b0 + n0);
    std::vector<double> X(c0, c0 + n0);
    double E = E0;
    asci_run(c, *s, ci ? *ci : def, matel_tol, a, b, X, E, do_grow != 0, do_refine != 0, E_grow_out);
    *n_out = (int64_t)a.size();
    *E_out = E;
    for (int64_t i = 0; i < std::min<int64_t>((int64_t)a.size(), cap); ++i) {
      if (out_a) out_a[i] = a[i];
      if (out_b) out_b[i] = b[i];
      if (out_c) out_c[i] = X[i];
    }
  });
}

int qdkgb_sigma_plan(qdkgb_context* c, int precision, int* segments, int* ncand, int* cand_segments,
                     double* cand_ms, int* kernel, double* kernel_ms) {
  if (!c || !segments) return QDKGB_ERR_INVALID;
  std::vector<std::pair<int, double>> rec;
  std::vector<std::vector<double>> kms;
  *segments = struct_sigma_plan(c, precision == QDKGB_PREC_MIXED ? 0 : 1, &rec, kernel, &kms);
  const int cap = ncand ? *ncand : 0;
  if (ncand) *ncand = (int)rec.size();
  for (int i = 0; i < std::min(cap, (int)rec.size()); ++i) {
    if (cand_segments) cand_segments[i] = rec[i].first;
    if (cand_ms) cand_ms[i] = rec[i].second;
    if (kernel_ms)
      for (int k = 0; k < QDKGB_SIGMA32_KERNELS; ++k)
        kernel_ms[(size_t)k * cap + i] =
            (k < (int)kms.size() && i < (int)kms[k].size()) ? kms[k][i] : std::nan("");
  }
  return QDKGB_OK;
}

int qdkgb_asci_phase_times(const qdkgb_context* c, double* seconds, int64_t* iterations, int64_t* patched) {
  if (!c || !seconds) return QDKGB_ERR_INVALID;
  for (int i = 0; i < 4; ++i) seconds[i] = c->asci_phase_s[i];
  if (iterations) *iterations = c->asci_iters;
  if (patched) *patched = c->asci_patches;
  return QDKGB_OK;
}

int qdkgb_build_operator(qdkgb_context* c, double thresh, int storage, int max_m, int* layout, int64_t* nnz) {
  if (!c) return QDKGB_ERR_INVALID;
  return guarded(c, [&] {
    QDKGB_CUDA(cudaSetDevice(c->device));
    const bool direct = build_operator(c, thresh, storage, max_m);
    if (layout) *layout = direct ? QDKGB_LAYOUT_DIRECT : (c->H.structured ? QDKGB_LAYOUT_SLAB : QDKGB_LAYOUT_CSR);
    if (nnz) *nnz = direct ? 0 : c->H.nnz;
  });
}

int qdkgb_casci(qdkgb_context* c, int norb, int nalpha, int nbeta, const double* T, const double* V, int layout,
                const qdkgb_davidson_settings* s, double matel_tol, double* E, double* C,
                qdkgb_davidson_info* info) {
  if (!c) return QDKGB_ERR_INVALID;
  int rc = qdkgb_set_integrals(c, norb, T, V, layout);
  if (rc) return rc;
  int64_t nd = 0;
  rc = qdkgb_fci_dets(norb, nalpha, nbeta, nullptr, nullptr, &nd);
  if (rc) return rc;
  return guarded(c, [&] {
    // the complete space of this shape is reused when the context holds it
    if (!(c->have_dets && c->fci_shape[0] == norb && c->fci_shape[1] == nalpha && c->fci_shape[2] == nbeta)) {
      std::vector<uint64_t> a(nd), b(nd);
      if (qdkgb_fci_dets(norb, nalpha, nbeta, a.data(), b.data(), &nd)) throw Error(QDKGB_ERR_INVALID, "fci dets");
      build_det_space(c, nd, a.data(), b.data());
      c->fci_shape[0] = norb;
      c->fci_shape[1] = nalpha;
      c->fci_shape[2] = nbeta;
    }
    qdkgb_davidson_settings def;
    qdkgb_davidson_default_settings(&def);
    const qdkgb_davidson_settings* ss = s ? s : &def;
    build_operator(c, matel_tol, ss->precision == QDKGB_PREC_MIXED ? QDKGB_H_SPLIT32 : QDKGB_H_FP64,
                   (int)ss->max_m);
    davidson(c, ss, E, C, info);
  });
}

int qdkgb_batch_default_settings(qdkgb_batch_settings* s) {
  if (!s) return QDKGB_ERR_INVALID;
  s->res_tol = 1e-8;
  s->precision = QDKGB_PREC_MIXED;
  s->max_subspace = 24;
  s->max_cycles = 200;
  s->matel_tol = std::numeric_limits<double>::epsilon();
  s->min_abs_denominator = 1e-12;
  s->use_graph = 1;
  s->max_slab_bytes = (int64_t)96 << 30;
  s->persistent = 0;
  s->cluster = 0;
  return QDKGB_OK;
}

int qdkgb_batch_plan(const qdkgb_context* c, int cap, int* nshapes, int* shape, int* cluster, int* ncand,
                     int* cand_cluster, double* cand_ms) {
  if (!c || cap < 0) return QDKGB_ERR_INVALID;
  const int n = (int)c->batch_tune.size();
  if (nshapes) *nshapes = n;
  for (int i = 0; i < std::min(n, cap); ++i) {
    const BatchTune& t = c->batch_tune[i];
    if (shape) {
      shape[3 * i] = t.norb;
      shape[3 * i + 1] = t.na;
      shape[3 * i + 2] = t.nb;
    }
    if (cluster) cluster[i] = t.cluster;
    const int nc = std::min<int>(4, (int)t.cand_ms.size());
    if (ncand) ncand[i] = nc;
    for (int j = 0; j < nc; ++j) {
      if (cand_cluster) cand_cluster[4 * i + j] = t.cand_ms[j].first;
      if (cand_ms) cand_ms[4 * i + j] = t.cand_ms[j].second;
    }
  }
  return QDKGB_OK;
}

int qdkgb_casci_batch(qdkgb_context* c, int ninst, const qdkgb_cas_instance* inst, const qdkgb_batch_settings* s,
                      double* energies, double* rdm1, int* iterations, qdkgb_batch_info* info) {
  if (!c) return QDKGB_ERR_INVALID;
  return guarded(c, [&] {
    if (ninst > 0 && !inst) throw Error(QDKGB_ERR_INVALID, "null instance array");
    QDKGB_CUDA(cudaSetDevice(c->device));
    qdkgb_batch_settings def;
    qdkgb_batch_default_settings(&def);
    casci_batch(c, ninst, inst, s ? *s : def, energies, rdm1, iterations, info);
  });
}

}  // extern "C"
