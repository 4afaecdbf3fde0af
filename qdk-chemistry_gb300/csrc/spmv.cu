// Sigma = H x on the device CSR (replaces sparsexx::spblas::gespmbv,
// sparsexx/spblas/spmbv.hpp:49-85, as driven by SparseMatrixOperator,
// include/macis/solvers/davidson.hpp:79-90).
//
// HBM-bound: a sigma streams nnz * (value + 4 B column) once; x (<= a few MB)
// stays L2-resident.  One warp per row (FCI rows hold ~10^2..10^3 elements),
// lanes stride the row with coalesced loads, several loads in flight per lane,
// and a fixed-order shuffle reduction (deterministic results).
//   fp64  : FP64 values, FP64 x/y, FP64 FMA
//   fp32  : FP32 values (the high part of the split storage), FP32 x/y/accumulation
//   split : hi + lo values with float-float products and sums (FP32 pipe),
//           FP64 x/y - the full-precision sigma of the mixed-precision path
#include <mutex>

#include "common.cuh"
#include "internal.h"

namespace qdkgb {

constexpr int kSpmvWarps = 8;

struct ValF64 {
  const double* v;
  __device__ __forceinline__ double operator()(int64_t k) const { return __ldcs(v + k); }
};
struct ValF32 {
  const float* v;
  __device__ __forceinline__ float operator()(int64_t k) const { return __ldcs(v + k); }
};

template <typename Acc, typename X, typename Val>
__global__ void __launch_bounds__(kSpmvWarps * 32)
    k_spmv_csr(int64_t n, const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col, Val val,
               const X* __restrict__ x, X* __restrict__ y) {
  const int lane = threadIdx.x & 31;
  const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = w0; r < n; r += nw) {
    const int64_t st = rowptr[r], en = rowptr[r + 1];
    Acc acc0 = 0, acc1 = 0, acc2 = 0, acc3 = 0;
    int64_t k = st + lane;
    for (; k + 96 < en; k += 128) {
      const int32_t c0 = __ldcs(col + k), c1 = __ldcs(col + k + 32), c2 = __ldcs(col + k + 64),
                    c3 = __ldcs(col + k + 96);
      const Acc v0 = val(k), v1 = val(k + 32), v2 = val(k + 64), v3 = val(k + 96);
      acc0 += v0 * (Acc)__ldg(x + c0);
      acc1 += v1 * (Acc)__ldg(x + c1);
      acc2 += v2 * (Acc)__ldg(x + c2);
      acc3 += v3 * (Acc)__ldg(x + c3);
    }
    for (; k < en; k += 32) acc0 += val(k) * (Acc)__ldg(x + __ldcs(col + k));
    Acc acc = (acc0 + acc1) + (acc2 + acc3);
    acc = warp_sum(acc);
    if (lane == 0) y[r] = (X)acc;
  }
}

// Full-precision sigma from the split storage without the FP64 pipe (slow on
// GB300): h = hi + lo and x = xh + xl are float pairs, each product
// (hi + lo)(xh + xl) is formed with an error-free FP32 product of hi*xh plus
// the cross terms, and the row sum is kept as an unevaluated float-float pair
// (two-sum).  Relative accuracy ~2^-44 per product, far below what the
// defect correction needs; the row result is rounded to FP64 once.
__global__ void __launch_bounds__(kSpmvWarps * 32)
    k_spmv_split_ff(int64_t n, const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                    const float* __restrict__ hi, const float* __restrict__ lo, const float* __restrict__ xh,
                    const float* __restrict__ xl, double* __restrict__ y) {
  const int lane = threadIdx.x & 31;
  const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = w0; r < n; r += nw) {
    const int64_t st = rowptr[r], en = rowptr[r + 1];
    FF a0{0.f, 0.f}, a1{0.f, 0.f};
    int64_t k = st + lane;
    for (; k + 32 < en; k += 64) {
      const int32_t c0 = __ldcs(col + k), c1 = __ldcs(col + k + 32);
      const float h0 = __ldcs(hi + k), h1 = __ldcs(hi + k + 32);
      const float l0 = __ldcs(lo + k), l1 = __ldcs(lo + k + 32);
      const float x0 = __ldg(xh + c0), x1 = __ldg(xh + c1);
      const float y0 = __ldg(xl + c0), y1 = __ldg(xl + c1);
      float p0 = h0 * x0, p1 = h1 * x1;
      float e0 = fmaf(h0, x0, -p0), e1 = fmaf(h1, x1, -p1);
      e0 = fmaf(h0, y0, fmaf(l0, x0, e0));
      e1 = fmaf(h1, y1, fmaf(l1, x1, e1));
      ff_add(a0, p0, e0);
      ff_add(a1, p1, e1);
    }
    for (; k < en; k += 32) {
      const int32_t c0 = __ldcs(col + k);
      const float h0 = __ldcs(hi + k), l0 = __ldcs(lo + k);
      const float x0 = __ldg(xh + c0), y0 = __ldg(xl + c0);
      const float p0 = h0 * x0;
      float e0 = fmaf(h0, x0, -p0);
      e0 = fmaf(h0, y0, fmaf(l0, x0, e0));
      ff_add(a0, p0, e0);
    }
    FF a = ff_merge(a0, a1);
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
      FF o;
      o.s = __shfl_xor_sync(QDKGB_FULL_MASK, a.s, d);
      o.c = __shfl_xor_sync(QDKGB_FULL_MASK, a.c, d);
      a = (lane & d) ? ff_merge(o, a) : ff_merge(a, o);
    }
    if (lane == 0) y[r] = (double)a.s + (double)a.c;
  }
}
__global__ void k_split_x(const double* __restrict__ x, float* __restrict__ xh, float* __restrict__ xl, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float h, l;
    split_f64(x[i], h, l);
    xh[i] = h;
    xl[i] = l;
  }
}

// x -> (xh, xl) float pair in the context's scratch, xh at [0, n), xl at [n, 2n)
float* split_x(Context* c, const double* x) {
  const int64_t n = c->H.n;
  float* xs = dev_array<float>(c, c->H.xsplit, 2 * (size_t)n);
  k_split_x<<<c->sm_count * 4, 256, 0, c->stream>>>(x, xs, xs + n, n);
  QDKGB_CHECK_LAUNCH();
  return xs;
}

static unsigned spmv_blocks(Context* c, int64_t n) {
  const int64_t want = (n + kSpmvWarps - 1) / kSpmvWarps;
  return (unsigned)std::min<int64_t>(want, (int64_t)c->sm_count * 32);
}

void spmv_fp64(Context* c, const double* x, double* y) {
  Hcsr& H = c->H;
  if (!H.valid) throw Error(QDKGB_ERR_STATE, "Hamiltonian not built");
  if (c->op_direct) {
    direct_sigma_fp64(c, x, y);
    return;
  }
  if (struct_ready(c)) {
    struct_spmv_fp64(c, x, y);
    return;
  }
  const int64_t* rp = (const int64_t*)H.rowptr.ptr;
  const int32_t* ci = (const int32_t*)H.colind.ptr;
  if (H.storage == QDKGB_H_FP64)
    k_spmv_csr<double, double><<<spmv_blocks(c, H.n), kSpmvWarps * 32, 0, c->stream>>>(
        H.n, rp, ci, ValF64{(const double*)H.val.ptr}, x, y);
  else {
    float* xs = split_x(c, x);
    k_spmv_split_ff<<<spmv_blocks(c, H.n), kSpmvWarps * 32, 0, c->stream>>>(
        H.n, rp, ci, (const float*)H.hi.ptr, (const float*)H.lo.ptr, xs, xs + H.n, y);
  }
  QDKGB_CHECK_LAUNCH();
}

void spmv_fp32(Context* c, const float* x, float* y) {
  Hcsr& H = c->H;
  if (!H.valid) throw Error(QDKGB_ERR_STATE, "Hamiltonian not built");
  if (c->op_direct || c->fp32_direct) {
    direct_sigma_fp32(c, x, y);
    return;
  }
  if (struct_ready(c) && H.storage == QDKGB_H_SPLIT32) {
    struct_spmv_fp32(c, x, y);
    return;
  }
  if (H.storage != QDKGB_H_SPLIT32)
    throw Error(QDKGB_ERR_STATE, "FP32 sigma needs the Hamiltonian built with QDKGB_H_SPLIT32 storage");
  k_spmv_csr<float, float><<<spmv_blocks(c, H.n), kSpmvWarps * 32, 0, c->stream>>>(
      H.n, (const int64_t*)H.rowptr.ptr, (const int32_t*)H.colind.ptr, ValF32{(const float*)H.hi.ptr}, x, y);
  QDKGB_CHECK_LAUNCH();
}

__global__ void k_split_to_double(int64_t nnz, const float* hi, const float* lo, double* out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nnz; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (double)hi[i] + (double)lo[i];
}
void csr_values_to_double(Context* c, double* out) {
  Hcsr& H = c->H;
  if (H.storage == QDKGB_H_FP64) {
    QDKGB_CUDA(cudaMemcpyAsync(out, H.val.ptr, H.nnz * 8, cudaMemcpyDeviceToDevice, c->stream));
  } else {
    k_split_to_double<<<c->sm_count * 8, 256, 0, c->stream>>>(H.nnz, (const float*)H.hi.ptr,
                                                              (const float*)H.lo.ptr, out);
    QDKGB_CHECK_LAUNCH();
  }
}

__global__ void k_f64_to_f32(const double* x, float* y, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = __double2float_rn(x[i]);
}
__global__ void k_f32_to_f64(const float* x, double* y, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = (double)x[i];
}
void f64_to_f32(Context* c, const double* x, float* y, int64_t n) {
  k_f64_to_f32<<<c->sm_count * 4, 256, 0, c->stream>>>(x, y, n);
  QDKGB_CHECK_LAUNCH();
}
void f32_to_f64(Context* c, const float* x, double* y, int64_t n) {
  k_f32_to_f64<<<c->sm_count * 4, 256, 0, c->stream>>>(x, y, n);
  QDKGB_CHECK_LAUNCH();
}

// ------------------------------------------------------------------ allocation-free sigma
// Scratch of qdkgb_sigma_split_noalloc: the x vector split into FP32 high and
// low halves.  A file-scope device array, so the entry point never allocates;
// every GPU that loads the library holds it (8 MiB) until the process exits.
constexpr int64_t kNoAllocMaxRows = QDKGB_NOALLOC_MAX_ROWS;
static __device__ __align__(256) float g_noalloc_split_x[2 * kNoAllocMaxRows];

namespace {
struct NoAllocDevice {
  bool ready = false;
  float* scratch = nullptr;  // device address of g_noalloc_split_x on this device
  int sm_count = 0;
};
constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
NoAllocDevice g_noalloc_dev[kNoAllocMaxDevices];
}  // namespace

}  // namespace qdkgb

extern "C" int qdkgb_sigma_split_noalloc(int64_t n, const int64_t* rowptr, const int32_t* colind, const float* hi,
                                         const float* lo, const double* x, double* y, void* stream) {
  using namespace qdkgb;
  if (n < 0 || n > kNoAllocMaxRows) {
    set_context_free_error("qdkgb_sigma_split_noalloc: " + std::to_string(n) +
                           " rows is outside [0, QDKGB_NOALLOC_MAX_ROWS = " + std::to_string(kNoAllocMaxRows) + "]");
    return QDKGB_ERR_INVALID;
  }
  if (n == 0) return QDKGB_OK;
  if (!rowptr || !colind || !hi || !lo || !x || !y) {
    set_context_free_error("qdkgb_sigma_split_noalloc: null pointer");
    return QDKGB_ERR_INVALID;
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kNoAllocMaxDevices) {
    set_context_free_error(std::string("qdkgb_sigma_split_noalloc: no current CUDA device: ") +
                           cudaGetErrorString(e));
    return QDKGB_ERR_CUDA;
  }
  NoAllocDevice st;
  {
    // one-time set-up per device, with that device current: the host-side
    // symbol is only a stand-in, the kernels need the device address
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    NoAllocDevice& d = g_noalloc_dev[dev];
    if (!d.ready) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_noalloc_split_x);
      if (e != cudaSuccess) {
        set_context_free_error(std::string("qdkgb_sigma_split_noalloc: cudaGetSymbolAddress failed: ") +
                               cudaGetErrorString(e));
        return QDKGB_ERR_CUDA;
      }
      e = cudaDeviceGetAttribute(&d.sm_count, cudaDevAttrMultiProcessorCount, dev);
      if (e != cudaSuccess) {
        set_context_free_error(std::string("qdkgb_sigma_split_noalloc: ") + cudaGetErrorString(e));
        return QDKGB_ERR_CUDA;
      }
      d.scratch = (float*)p;
      d.ready = true;
    }
    st = d;
  }
  // An error left pending by the caller's own earlier CUDA work stays the
  // caller's: report it without launching and without clearing it.
  e = cudaPeekAtLastError();
  if (e != cudaSuccess) {
    set_context_free_error(std::string("qdkgb_sigma_split_noalloc: a CUDA error was already pending before "
                                       "this call (not cleared): ") + cudaGetErrorString(e));
    return QDKGB_ERR_CUDA;
  }
  cudaStream_t s = (cudaStream_t)stream;
  float* xh = st.scratch;
  float* xl = st.scratch + kNoAllocMaxRows;
  k_split_x<<<st.sm_count * 4, 256, 0, s>>>(x, xh, xl, n);
  count_launch();
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_context_free_error(std::string("qdkgb_sigma_split_noalloc: launch of the x split failed: ") +
                           cudaGetErrorString(e));
    return QDKGB_ERR_CUDA;
  }
  const unsigned blocks = (unsigned)std::min<int64_t>((n + kSpmvWarps - 1) / kSpmvWarps, (int64_t)st.sm_count * 32);
  k_spmv_split_ff<<<blocks, kSpmvWarps * 32, 0, s>>>(n, rowptr, colind, hi, lo, xh, xl, y);
  count_launch();
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_context_free_error(std::string("qdkgb_sigma_split_noalloc: launch of the sigma failed: ") +
                           cudaGetErrorString(e));
    return QDKGB_ERR_CUDA;
  }
  return QDKGB_OK;
}

