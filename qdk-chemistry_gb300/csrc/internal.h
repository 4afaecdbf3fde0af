// Internal declarations shared by the library's translation units.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "../../include/qdkgb.h"

namespace qdkgb {

// A named NVTX range over a scope: the library's phases (determinant space,
// H build, Davidson, RDMs, ASCI steps, PT2, CASSCF iterations) appear on the
// Nsight timelines; without an attached tool the calls return at once.
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

// Thrown inside the library, converted to a status code at the C ABI.
struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define QDKGB_CUDA(call)                                                                              \
  do {                                                                                                \
    cudaError_t e_ = (call);                                                                          \
    if (e_ != cudaSuccess)                                                                            \
      throw ::qdkgb::Error(e_ == cudaErrorMemoryAllocation ? QDKGB_ERR_OOM : QDKGB_ERR_CUDA,          \
                           std::string(#call) + ": " + cudaGetErrorString(e_));                      \
  } while (0)

// Every kernel launch site ends with this check; it also counts the launch.
#define QDKGB_CHECK_LAUNCH()        \
  do {                              \
    ::qdkgb::count_launch();        \
    QDKGB_CUDA(cudaGetLastError()); \
  } while (0)

// Device allocation owned by a context (tracked so the context can report and
// release what it holds).
struct DeviceBuffer {
  void* ptr = nullptr;
  size_t bytes = 0;
};

struct Context;
struct Integrals;
struct DirectSigma;
struct FciStruct;

void count_launch();
// cudaFuncAttributeMaxDynamicSharedMemorySize of a kernel on the current
// device, raised to at least `bytes` (idempotent, thread-safe)
void set_max_dynamic_smem(const void* func, int bytes);
// message of the last failed call that takes no context (qdkgb_last_error(NULL))
void set_context_free_error(const std::string& msg);

void* dev_alloc(Context* c, DeviceBuffer& b, size_t bytes);  // (re)allocates when too small
void dev_free(Context* c, DeviceBuffer& b);

template <typename T>
T* dev_array(Context* c, DeviceBuffer& b, size_t n) {
  return (T*)dev_alloc(c, b, n * sizeof(T) + 16);
}

// Scratch device buffers released on every exit of a scope (exceptions included).
template <int N>
struct ScopedBuffers {
  Context* c;
  DeviceBuffer b[N];
  explicit ScopedBuffers(Context* ctx) : c(ctx) {}
  ~ScopedBuffers() {
    for (DeviceBuffer& x : b) dev_free(c, x);
  }
  ScopedBuffers(const ScopedBuffers&) = delete;
  ScopedBuffers& operator=(const ScopedBuffers&) = delete;
};

// Determinant list prepared for the kernels.
struct DetSpace {
  int64_t ndets = 0;
  int64_t ngroups = 0;  // alpha groups (runs of equal alpha strings)
  int64_t nbeta = 0;    // distinct beta strings
  bool product = false; // every group holds every beta string (FCI-like)
  uint64_t occ_union = 0;  // OR of every alpha and beta string (orbitals in use)
  std::vector<uint64_t> h_alpha, h_beta;
  std::vector<uint64_t> h_galpha;
  std::vector<uint64_t> h_ubeta;  // distinct beta strings in rank order
  std::vector<int64_t> h_gstart;
  // device
  DeviceBuffer galpha, gstart, det_group, brank, ubeta, gcomplete;
  DeviceBuffer acon_ptr, acon_idx, acon_lvl;  // alpha-group connectivity (<= double)
  DeviceBuffer b2_ptr, b2_idx;                // beta-string connectivity, level <= 2 (<= 4 differing bits)
  DeviceBuffer b1_ptr, b1_idx;                // beta-string connectivity, level <= 1
  int64_t acon_total = 0, b2_total = 0, b1_total = 0;
};

struct Hcsr {
  int64_t n = 0, nnz = 0;
  int storage = QDKGB_H_FP64;
  double thresh = 0.;
  DeviceBuffer rowptr, colind, val, hi, lo, diag, diag_raw, row_nnz, scan_tmp, xsplit;
  bool valid = false;
  bool structured = false;  // complete space in the slab layout (values only, columns implied by the row tables)
};

struct DavidsonWork {
  DeviceBuffer V, AV, xf, yf, Hk, evec, eval, scratch, partial, small;
  int64_t n = 0, maxm = 0;
};

// The batched solver's measured choice for one shape: CTAs per instance
// (cluster) and the timed candidates (cluster size, ms of a tuning run).
struct BatchTune {
  int norb, na, nb, m, mixed;
  int cluster;
  std::vector<std::pair<int, double>> cand_ms;
};

struct Context {
  int device = 0;
  cudaStream_t own_stream = nullptr, stream = nullptr;
  std::string err;
  int64_t dev_bytes = 0;
  int64_t dev_limit = 0;  // cap on dev_bytes (0: none), set by qdkgb_set_device_limit
  int sm_count = 0;
  // integrals
  int norb = 0;
  DeviceBuffer T, V, G_red, V_red, G2, V2;
  std::vector<double> h_T, h_V;  // column-major host copies
  bool have_ints = false;
  DetSpace dets;
  bool have_dets = false;
  int fci_shape[3] = {-1, -1, -1};  // (norb, n_alpha, n_beta) when the dets are that complete space
  Hcsr H;
  DavidsonWork dav;
  DirectSigma* direct = nullptr;  // recompute-on-the-fly operator (complete spaces)
  FciStruct* fci = nullptr;       // row-shape tables of a complete space (structured kernels)
  bool op_direct = false;         // Davidson / spmv use the direct sigma instead of the CSR
  bool fp32_direct = false;       // complete space, mixed form: FP32 sigma by the direct contraction,
                                  // full-precision sigma by the stored (FP64) slab
  // seconds spent by the last qdkgb_asci call in its phases: the determinant
  // search, the determinant-space set-up, the Hamiltonian build, Davidson;
  // and its asci_iter count
  double asci_phase_s[4] = {0., 0., 0., 0.};
  int64_t asci_iters = 0;
  int64_t asci_patches = 0;  // Hamiltonians of the last qdkgb_asci call built by patching the previous one
  std::vector<BatchTune> batch_tune;  // persistent batched solver: cluster size per shape
  // the direct sigma's timed FP32 forms per space shape (n, n_alpha strings,
  // n_beta strings, tensor cores on): same-spin form and contraction form,
  // kept across rebuilds so that a context's FP32 sigma repeats bit for bit
  struct DirectTune {
    int n;
    int64_t na, nb;
    bool tc;
    int dense, otc;
  };
  std::vector<DirectTune> direct_tune;
  std::vector<double> asci_rot;       // accumulated natural-orbital rotation of the last qdkgb_asci (empty: none)
  DeviceBuffer host_pinned_dummy;
  double* pinned = nullptr;  // small pinned host staging (64 doubles)
};

Integrals integrals_view(Context* c);
// throws QDKGB_ERR_INVALID when a determinant occupies an orbital >= norb
// (the integral and RDM indices of the kernels stop at norb)
void check_dets_in_orbitals(const Context* c);

// hbuild.cu
void build_integral_intermediates(Context* c);
void build_det_space(Context* c, int64_t ndets, const uint64_t* alpha, const uint64_t* beta);
void build_hamiltonian(Context* c, double thresh, int storage);
bool build_operator(Context* c, double thresh, int storage, int max_m);  // true: direct sigma
// The CSR of the current list from the previous list's CSR (old host lists
// sorted by spin_comparator, old FP64 CSR buffers, the same threshold); false
// when the kept share of the new determinants is below min_overlap
// (incremental_h_build.hpp:263-282).
bool build_hamiltonian_patched(Context* c, double thresh, const std::vector<uint64_t>& oa,
                               const std::vector<uint64_t>& ob, DeviceBuffer& old_rowptr, DeviceBuffer& old_colind,
                               DeviceBuffer& old_val, double min_overlap);
void set_csr(Context* c, int64_t n, const int64_t* rowptr, const int64_t* colind, const double* values);
void exclusive_scan_i64(Context* c, const int64_t* in, int64_t* out, int64_t n, DeviceBuffer& tmp);

// spmv.cu
void spmv_fp64(Context* c, const double* x, double* y);
void spmv_fp32(Context* c, const float* x, float* y);
void csr_values_to_double(Context* c, double* out);
void f64_to_f32(Context* c, const double* x, float* y, int64_t n);
void f32_to_f64(Context* c, const float* x, double* y, int64_t n);

// fci_struct.cu
void build_struct(Context* c);
void free_struct(Context* c);
bool struct_ready(Context* c);
void struct_spmv_fp64(Context* c, const double* x, double* y);
void struct_spmv_fp32(Context* c, const float* x, float* y);
void struct_export(Context* c, int32_t* ci, double* v64, float* h32, float* l32);
int64_t struct_slab_elements(Context* c);
// segments in use and the autotuner's record (segments, ms) per candidate; for
// the FP32 plan also the kernel in use (0 register-fed, 1 TMA-fed, 2 / 3
// register-fed eight / sixteen positions deep) and every kernel's timing per
// candidate
int struct_sigma_plan(Context* c, int plan, std::vector<std::pair<int, double>>* record, int* kernel = nullptr,
                      std::vector<std::vector<double>>* kernel_ms = nullptr);
// batch.cu
void casci_batch(Context* ctx, int ninst, const qdkgb_cas_instance* inst, const qdkgb_batch_settings& st,
                 double* energies, double* rdm1, int* iters, qdkgb_batch_info* info);
// davidson.cu: lowest eigenpair of B small matrices, one CTA each
// batch_persist.cu: one shape's sub-batch (slabs emitted, diagonals set) solved
// by the persistent cluster kernel; results in the job's device arrays.
// cc: the shape's context (space, tables, plans); owner: the caller's
// context, which keeps the tuned cluster size per shape.
struct BatchShapeJob {
  int norb, na, nb, B, m, max_cycles, cluster;
  bool mixed, square;
  int64_t N, nstr, vstride;
  double tol, min_abs;
  const float* hi;
  const float* lo;
  const double* val;
  const double* D;
  double* energy;
  double* resid;
  int* iters;
  int* notdone;
  double* rdm;  // [B][norb^2] or null
};
void batch_solve_persistent(Context* cc, Context* owner, const BatchShapeJob& job);
// mcscf.cu: the natural orbitals of a spin-summed 1-RDM (columns, occupations
// descending: syev of -ordm, grow.hpp:181-188) and the rotation of the
// context's integrals to them (two_index_transform / four_index_transform,
// grow.hpp:196-199), intermediates rebuilt
void natural_orbitals(int n, const std::vector<double>& ordm, std::vector<double>& C);
void rotate_integrals(Context* c, const std::vector<double>& C);
void lowest_eig_batch(cudaStream_t st, int B, const int* kdev, int kadd, int kmax, const double* Hs, int ldh,
                      int64_t hstride, double* eval, double* evec, int64_t estride, const int* active);
void slab_emit_batch(Context* c, int B, const Integrals* d_ints, const double* diag_raw, int storage, double* val,
                     float* hi, float* lo, double thresh);
void slab_reserve_batch(Context* c, int B);
void slab_sigma_batch(Context* c, int mode, int B, const int* active, const void* vals, const float* vlo,
                      const void* x, const float* xlo, void* y);
float* split_x(Context* c, const double* x);
void build_hamiltonian_struct(Context* c, double thresh, int storage);
void k_diag_launch(Context* c, const Integrals& I, double* D, unsigned blocks);

// direct.cu
void build_direct_sigma(Context* c);
// The FP32 sigma of a complete space through the direct contraction beside
// the stored FP64 slab (mixed form); false where the contraction form does
// not apply.
bool attach_direct_fp32(Context* c);
// Batched CASCI's FP32 sigma through the direct contraction: per-instance
// value tables of a sub-batch (T: [B][n^2], V: [B][n^4] on the device; false
// where the form does not apply), then y = sigma(x) for the active instances
// (x, y: [B][N] FP32; D: [B][N] the diagonals).
bool direct_batch_prepare(Context* c, int B, const double* T, const double* V);
void direct_batch_sigma(Context* c, int B, const int* act, const double* D, const float* x, float* y);
// The direct sigma's FP32 form: contraction in use (0 element-wise walk,
// 1 FMA pipe, 2 tensor cores), same-spin form (-1 not yet timed, 0
// element-wise, 1 dense) and the times (ms) of the same-spin forms
// (element-wise, dense) and of the contractions (FMA, tensor cores).
void direct_plan(const Context* c, int* mm, int* dense, double* ms);
void free_direct(Context* c);
void direct_sigma_fp64(Context* c, const double* x, double* y);
void direct_sigma_fp32(Context* c, const float* x, float* y);
// out (nc x nr) = in^T for a row-major in (nr x nc)
void transpose_f64(Context* c, const double* in, double* out, int64_t nr, int64_t nc);

// asci.cu
void asci_search_gpu(Context* c, int64_t ncore, const uint64_t* ca, const uint64_t* cb, const double* cc, double E0,
                     int64_t ndets_max, double h_el_tol, double rv_prune_tol, std::vector<uint64_t>& out_a,
                     std::vector<uint64_t>& out_b, int64_t* n_candidates, bool just_singles = false);
double asci_pt2_gpu(Context* c, int64_t nd, const uint64_t* a, const uint64_t* b, const double* C, double E0,
                    double pt2_tol, int64_t max_slots, int64_t* npt2);
void asci_run(Context* c, const qdkgb_asci_settings& S, const qdkgb_davidson_settings& ci, double matel_tol,
              std::vector<uint64_t>& a, std::vector<uint64_t>& b, std::vector<double>& X, double& E0, bool grow,
              bool refine, double* E_grow);

// davidson.cu
void davidson(Context* c, const qdkgb_davidson_settings* s, double* E, double* C, qdkgb_davidson_info* info);

// rdm.cu
void rdms_spin_dep(Context* c, const double* C, double* aa, double* bb, double* aaaa, double* bbbb, double* aabb);
void orbital_entropies(Context* c, const double* C, double* s1, double* s2, double* mi);

// mcscf.cu
double casscf(Context* c, const qdkgb_mcscf_settings& S, int nalpha, int nbeta, int norb, int ninact, int nact,
              double E_core, const double* T0, const double* V0, double* A1, double* A2, double* U_out,
              int64_t* iterations, int* converged_out);

}  // namespace qdkgb

struct qdkgb_context : qdkgb::Context {};
