/*
 * qdkgb.h — C ABI of the GB300-native selected-CI / CASCI core.
 *
 * This is the drop-in boundary for the hot path that qdk-chemistry runs
 * through MACIS: determinant-driven Hamiltonian build, Davidson eigensolve,
 * spin-resolved 1-/2-RDMs and the ASCI determinant search.  All compute runs
 * in hand-written sm_103a CUDA kernels; there is no CPU fallback.
 *
 * Conventions
 *   - Every call returns an int status (QDKGB_OK == 0).  On failure the
 *     message is available from qdkgb_last_error(ctx).  No C++ exception
 *     crosses this boundary.
 *   - Buffers passed as plain pointers are caller-owned HOST memory unless a
 *     function name ends in _device, in which case they are device pointers on
 *     the context's GPU.
 *   - Integrals are MACIS's column-major spans: T(p,q) = T[p + n q],
 *     V(p,q,r,s) = V[p + n q + n^2 r + n^3 s] (layout QDKGB_LAYOUT_COLMAJOR),
 *     or qdk's row-major dense buffer (QDKGB_LAYOUT_ROWMAJOR).
 *   - A determinant is a pair of uint64 spin strings (bit i = spatial orbital
 *     i occupied), alpha and beta in separate arrays.  This covers MACIS's
 *     wfn_t<N> for N <= 128 (alpha = low N/2 bits, beta = high N/2 bits of the
 *     std::bitset<N>).
 *   - One context per host thread; a context owns device memory and a CUDA
 *     stream (the caller may substitute its own with qdkgb_set_stream).
 */
#ifndef QDKGB_H
#define QDKGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define QDKGB_OK 0
#define QDKGB_ERR_INVALID 1       /* bad argument (maps to std::invalid_argument / runtime_error) */
#define QDKGB_ERR_CUDA 2          /* CUDA runtime error */
#define QDKGB_ERR_OOM 3           /* device allocation failed */
#define QDKGB_ERR_NOT_CONVERGED 4 /* "Davidson Did Not Converge!" (davidson.hpp:368) */
#define QDKGB_ERR_UNSUPPORTED 5   /* input outside what the GPU path handles */
#define QDKGB_ERR_STATE 6         /* call made before its prerequisites */

#define QDKGB_LAYOUT_COLMAJOR 0
#define QDKGB_LAYOUT_ROWMAJOR 1

/* Storage of the Hamiltonian values on the device. */
#define QDKGB_H_FP64 0    /* FP64 values: 8 B/nnz + int32 column */
#define QDKGB_H_SPLIT32 1 /* FP32 high part + FP32 low part (h ~= hi + lo to 2^-48 |h|) */

/* Davidson precision modes. */
#define QDKGB_PREC_FP64 0  /* plain FP64 SpMV and vectors */
#define QDKGB_PREC_MIXED 1 /* FP32 SpMV (FP32 values, x, y, accumulation) + FP64 defect-correction restarts */

typedef struct qdkgb_context qdkgb_context;

/* ------------------------------------------------------------ context */
int qdkgb_create(qdkgb_context** ctx, int device);
int qdkgb_destroy(qdkgb_context* ctx);
/* Message of the last failure; NULL asks for the last failed context-free call. */
const char* qdkgb_last_error(const qdkgb_context* ctx);
/* cudaStream_t passed as void*; NULL restores the context's own stream. */
int qdkgb_set_stream(qdkgb_context* ctx, void* stream);
/* Bytes of device memory currently held by the context. */
int qdkgb_device_bytes(const qdkgb_context* ctx, int64_t* bytes);
/* Caps the device memory the context may hold (0: no cap): an allocation that
 * would pass it fails with QDKGB_ERR_OOM before reaching the device, and the
 * context stays usable.  The capped allocator behind the out-of-memory tests. */
int qdkgb_set_device_limit(qdkgb_context* ctx, int64_t bytes);

/* Storage of the operator the last build produced (no counterpart in the
 * reference, whose operator is always a sparsexx::csr_matrix):
 *   QDKGB_LAYOUT_CSR     the reference's CSR arrays (rowptr, colind, values);
 *   QDKGB_LAYOUT_SLAB    complete (CAS) space: values only, stored
 *                        group-major with beta strings fastest, columns
 *                        implied by the space; qdkgb_get_csr* exports CSR;
 *   QDKGB_LAYOUT_DIRECT  no stored matrix (qdkgb_build_direct_sigma);
 *   QDKGB_LAYOUT_SLAB_DIRECT32  complete space built with QDKGB_H_SPLIT32
 *                        storage: the FP64 slab (full-precision sigma and
 *                        exports) and, for the mixed form's FP32 sigma, the
 *                        direct contraction instead of a stored FP32 copy
 *                        (environment QDKGB_MIXED_FP32=slab keeps the copy).
 * stored_elements = matrix elements held on the device (slab: every
 * position, zeros for thresholded elements); NULL to skip. */
#define QDKGB_LAYOUT_NONE 0
#define QDKGB_LAYOUT_CSR 1
#define QDKGB_LAYOUT_SLAB 2
#define QDKGB_LAYOUT_DIRECT 3
#define QDKGB_LAYOUT_SLAB_DIRECT32 4
int qdkgb_operator_layout(const qdkgb_context* ctx, int* layout, int64_t* stored_elements);

/* The direct sigma's FP32 form (layouts QDKGB_LAYOUT_DIRECT and
 * QDKGB_LAYOUT_SLAB_DIRECT32; no counterpart in the reference):
 * *contraction 0 the element-wise walk, 1 the opposite-spin doubles and the
 * single excitations as one FP32 contraction per alpha string on the FMA
 * pipe, 2 the same with the contraction on the tensor cores (tcgen05, TF32
 * x 3); *dense the same-spin part's form, -1 until the first FP32 sigma
 * times the forms, 0 element-wise kernels, 1 two dense products (tensor
 * cores unless QDKGB_DIRECT_TC=0); form_ms[4] the times (ms) of the
 * same-spin forms (element-wise, dense) and of the contractions (FMA pipe,
 * tensor cores), 0 where not timed.  Any pointer may be NULL. */
int qdkgb_direct_plan(const qdkgb_context* ctx, int* contraction, int* dense, double* form_ms);

/* The sizes the getters write (no counterpart; the reference's sparsexx
 * matrix carries its own m() and nnz()): *ndets the dimension of the
 * operator (the rows of a caller's CSR after qdkgb_set_csr, else the
 * determinant count of the context's current list; 0 before either), *nnz
 * the CSR element count of the built operator as qdkgb_get_csr* exports it
 * (0 when none is built or the operator is the direct sigma).  Either
 * pointer may be NULL.
 * qdkgb_asci leaves its final list and that list's Hamiltonian in the
 * context, so the sizes change across that call. */
int qdkgb_problem_size(const qdkgb_context* ctx, int64_t* ndets, int64_t* nnz);

/* ------------------------------------------------------------ integrals
 * Replaces the HamiltonianGeneratorBase constructor and
 * generate_integral_intermediates_ (external/macis/src/macis/
 * hamiltonian_generator/base.ipp:27-77): uploads T, V and builds
 * G_red, V_red, G2_red, V2_red on the device.  norb <= 64. */
int qdkgb_set_integrals(qdkgb_context* ctx, int norb, const double* T, const double* V, int layout);

/* ------------------------------------------------------------ determinants
 * generate_combs / generate_hilbert_space
 * (external/macis/include/macis/sd_operations.hpp:305-351): all
 * (nalpha, nbeta) determinants over norb orbitals in MACIS order (alpha
 * major, strings in std::prev_permutation order).  Call with alpha == NULL to
 * query *ndets only. */
int qdkgb_fci_dets(int norb, int nalpha, int nbeta, uint64_t* alpha, uint64_t* beta, int64_t* ndets);

/* Uploads a determinant list and builds its alpha grouping
 * (get_unique_alpha, sd_operations.hpp:449-468) and the alpha/beta string
 * connectivity used by every kernel.  The list must be alpha-grouped (equal
 * alpha strings contiguous) with the beta strings of every group in one
 * common order, as both MACIS producers give it (generate_hilbert_space and
 * std::sort by spin_comparator, raw_bitset.hpp:119-141); otherwise
 * QDKGB_ERR_UNSUPPORTED. */
int qdkgb_set_dets(qdkgb_context* ctx, int64_t ndets, const uint64_t* alpha, const uint64_t* beta);

/* ------------------------------------------------------------ Hamiltonian
 * Replaces SortedDoubleLoopHamiltonianGenerator::make_csr_hamiltonian_block_
 * (include/macis/hamiltonian_generator/sorted_double_loop.hpp:86-451) for the
 * symmetric case, including threshold_parallel
 * (sparsexx/matrix_types/csr_matrix.hpp:317-372): keeps |h| > thresh (all
 * entries when thresh <= 0), columns sorted per row, values of the mirrored
 * entry computed with the lower-index determinant as bra.  The CSR stays on
 * the device (int64 row pointers, int32 columns); *nnz receives its size. */
int qdkgb_build_hamiltonian(qdkgb_context* ctx, double thresh, int storage, int64_t* nnz);
/* Direct (recompute-on-the-fly) sigma for complete active spaces whose CSR
 * would not fit in HBM: replaces the stored H of make_csr_hamiltonian_block_ +
 * SparseMatrixOperator (davidson.hpp:79-90) by sigma = diag C + S_aa(C) +
 * S_bb(C) + S_ab(C) evaluated from per-spin string tables on every
 * application, in FP64 (qdkgb_spmv / Davidson FP64) or FP32 (mixed mode).
 * Needs a full (n_alpha, n_beta) product space (qdkgb_fci_dets order or any
 * complete alpha-grouped list), at most 20 orbitals and 4096 strings per spin.
 * After this call qdkgb_spmv, qdkgb_davidson and qdkgb_diagonal use it; a later
 * qdkgb_build_hamiltonian switches back to the CSR. */
int qdkgb_build_direct_sigma(qdkgb_context* ctx);

/* The Davidson operator of the current determinants, chosen by memory: the
 * stored Hamiltonian (exactly qdkgb_build_hamiltonian(ctx, thresh, storage))
 * when it fits in the device memory available to the context (free memory
 * and the qdkgb_set_device_limit cap, counting what the current operator
 * holds) together with a Davidson workspace of max_m vectors; otherwise, for
 * a complete (n_alpha, n_beta) space within the direct sigma's limits, the
 * direct sigma (qdkgb_build_direct_sigma).  A complete space of 131,072
 * (2^17) or more determinants with storage QDKGB_H_SPLIT32 (a mixed-precision
 * solve) takes the direct sigma even when the matrix would fit: its FP32
 * sigma is the direct contraction either way, and recomputing the solve's few
 * full-precision refreshes costs less than emitting an FP64 matrix for them
 * (environment QDKGB_MIXED_FP32=slab keeps the stored form).  *layout (may be NULL) receives
 * QDKGB_LAYOUT_SLAB, QDKGB_LAYOUT_CSR or QDKGB_LAYOUT_DIRECT, *nnz (may be
 * NULL) the element count of the stored matrix's CSR (0 for the direct sigma).  The reference
 * always stores the matrix (make_csr_hamiltonian_block_ in
 * selected_ci_diag / compute_casci_rdms, include/macis/mcscf/cas.hpp:52-55);
 * at CAS(14e,14o) that matrix (3.98e10 elements) exceeds HBM, and this is how
 * the drop-in calculators reach that size.  qdkgb_casci uses it. */
int qdkgb_build_operator(qdkgb_context* ctx, double thresh, int storage, int max_m, int* layout, int64_t* nnz);

/* Introspection of the complete-space sigma's work split (no counterpart):
 * each CTA takes one segment of an alpha group's row.  The number of
 * segments is chosen by a measured autotuner: the first sigma of each
 * precision on a new space (outside any stream capture) times every
 * candidate count, one untimed and three timed sigmas each, and keeps the
 * fastest.  *segments receives the count in use (0: no complete-space
 * sigma); with ncand (in: capacity, out: candidates tried) the candidates'
 * counts and mean milliseconds, empty before the first sigma.  For the FP32
 * sigma the tuner also times the TMA-fed kernel (slab rows streamed into
 * shared memory by bulk copies) and the register-fed kernel with eight and
 * with sixteen positions in flight per thread on every candidate: *kernel
 * (may be NULL) receives the kernel in use (0 register-fed four deep, 1
 * TMA-fed, 2 / 3 register-fed eight / sixteen deep); kernel_ms (may be NULL,
 * QDKGB_SIGMA32_KERNELS rows of the ncand capacity) each kernel's
 * milliseconds per candidate (NaN where not timed).  All of them sum every
 * row in the same order: the same FP32 sigma bit for bit on the same plan. */
#define QDKGB_SIGMA32_KERNELS 4
int qdkgb_sigma_plan(qdkgb_context* ctx, int precision, int* segments, int* ncand, int* cand_segments,
                     double* cand_ms, int* kernel, double* kernel_ms);

/* Copies the device CSR to host buffers (rowptr: ndets+1, colind/values: nnz).
 * For QDKGB_H_SPLIT32 storage, values receive (double)hi + (double)lo.
 * The 32-bit and 64-bit variants mirror make_csr_hamiltonian_block_32bit_ /
 * _64bit_ (include/macis/hamiltonian_generator.hpp:32-294). */
int qdkgb_get_csr32(qdkgb_context* ctx, int32_t* rowptr, int32_t* colind, double* values);
int qdkgb_get_csr64(qdkgb_context* ctx, int64_t* rowptr, int64_t* colind, double* values);
/* A bra block: rows [row_begin, row_end) against every ket, as
 * make_csr_hamiltonian_block_{32,64}bit_(bra_begin, bra_end, ket_begin,
 * ket_end, thresh) returns it for a sub-range of bras and the full ket range
 * (include/macis/hamiltonian_generator.hpp:240-293; the distributed build,
 * include/macis/csr_hamiltonian.hpp:102-136).  rowptr (row_end - row_begin + 1
 * entries) starts at 0, colind holds global column indices; the element count
 * of the block is rowptr[row_end - row_begin].  Any buffer may be NULL (not
 * copied); call with NULL colind/values first to learn the count. */
int qdkgb_get_csr32_rows(qdkgb_context* ctx, int64_t row_begin, int64_t row_end, int32_t* rowptr,
                         int32_t* colind, double* values);
int qdkgb_get_csr64_rows(qdkgb_context* ctx, int64_t row_begin, int64_t row_end, int64_t* rowptr,
                         int64_t* colind, double* values);
/* A caller's symmetric CSR matrix (0-based, n rows, host buffers) becomes the
 * device operator for qdkgb_spmv / qdkgb_davidson, FP64 storage.  This is the
 * entry of davidson_solver(csr, tol, max_m) (python/src/pybind11/algorithms/
 * davidson_solver.cpp:60-107), which feeds a scipy CSR to macis::davidson. */
int qdkgb_set_csr(qdkgb_context* ctx, int64_t n, const int64_t* rowptr, const int64_t* colind, const double* values);
/* extract_diagonal_elements (sparsexx/util/submatrix.hpp:354-384). */
int qdkgb_diagonal(qdkgb_context* ctx, double* D);

/* y = H x with the device CSR (gespmbv, sparsexx/spblas/spmbv.hpp:49-85).
 * precision QDKGB_PREC_FP64 uses the full-precision values with FP64
 * accumulation; QDKGB_PREC_MIXED uses FP32 values, x and accumulation. */
int qdkgb_spmv(qdkgb_context* ctx, int precision, const double* x, double* y);
/* Same on device vectors: FP64 mode takes double*, MIXED mode float*. */
int qdkgb_spmv_device(qdkgb_context* ctx, int precision, const void* x, void* y);
/* The Davidson operator seam of the reference,
 * SparseMatrixOperator::operator_action(m, alpha, V, LDV, beta, AV, LDAV)
 * (include/macis/solvers/davidson.hpp:79-90, gespmbv): AV = alpha H V + beta AV
 * for m column-major host vectors of ndets (leading dimensions LDV, LDAV >=
 * ndets), FP64, with whichever operator is built (stored or direct sigma).
 * beta == 0 overwrites AV without reading it, as BLAS does. */
int qdkgb_operator_action(qdkgb_context* ctx, int64_t m, double alpha, const double* V, int64_t ldv, double beta,
                          double* AV, int64_t ldav);

/* ------------------------------------------------------------ eigensolver */
typedef struct qdkgb_davidson_settings {
  int64_t max_m;      /* ci_max_subspace / max_solver_iterations (default 200) */
  double res_tol;     /* ci_res_tol: residual 2-norm (default 1e-8) */
  int precision;      /* QDKGB_PREC_FP64 or QDKGB_PREC_MIXED */
  int use_guess;      /* 1: C holds a guess (used when max|C| > 1/N, selected_ci_diag.hpp:130-140) */
  double min_abs_denominator; /* preconditioner clamp (default 1e-12) */
  int nroots;         /* lowest roots wanted (default 1).  1: the reference's
                       * single-root davidson (davidson.hpp:259-372).  > 1: a
                       * block Davidson (no counterpart in MACIS, whose
                       * multi-root solver is lobpcgxx::lobpcg,
                       * src/lobpcgxx/include/lobpcgxx/simplified_interface.hpp:37-72):
                       * FP64 only, E receives nroots energies and C (if not
                       * NULL) nroots column-major vectors of ndets, converged
                       * when every root's residual is below res_tol; max_m
                       * bounds the subspace, which restarts on the Ritz
                       * vectors of the roots. */
} qdkgb_davidson_settings;

typedef struct qdkgb_davidson_info {
  int64_t iterations;       /* Davidson iterations (all precisions) */
  int64_t spmv_fp64;        /* full-precision sigma applications */
  int64_t spmv_fp32;        /* FP32 sigma applications (mixed mode) */
  int64_t restarts;         /* defect-correction restarts (mixed mode) */
  double residual_norm;     /* final full-precision residual 2-norm */
  double seconds;           /* wall time of the eigensolve */
} qdkgb_davidson_info;

void qdkgb_davidson_default_settings(qdkgb_davidson_settings* s);
/* serial_selected_ci_diag + davidson (include/macis/solvers/
 * selected_ci_diag.hpp:111-158, davidson.hpp:259-372) on the device CSR:
 * lowest eigenpair.  C (host, ndets) is the guess on input when use_guess,
 * and the eigenvector on output; *E the eigenvalue (electronic). */
int qdkgb_davidson(qdkgb_context* ctx, const qdkgb_davidson_settings* s, double* E, double* C,
                   qdkgb_davidson_info* info);

/* ------------------------------------------------------------ RDMs
 * SortedDoubleLoopHamiltonianGenerator::form_rdms (sorted_double_loop.hpp:
 * 512-624): the spin-traced 1-RDM (n x n) and 2-RDM (n^4), ACCUMULATED (+=);
 * NULL skips.  ordm = aa + bb and trdm(p,q,r,s) = aaaa + bbbb + aabb(p,q,r,s)
 * + aabb(r,s,p,q) of the spin-resolved blocks below, the identity the
 * reference's two routines satisfy. */
int qdkgb_rdms(qdkgb_context* ctx, const double* C, double* ordm, double* trdm);
/*
 * SortedDoubleLoopHamiltonianGenerator::form_rdms_spin_dep
 * (sorted_double_loop.hpp:626-753, contributions util/rdms.hpp:39-612):
 * spin-resolved 1-RDMs (n x n) and 2-RDMs (n^4), column-major, MACIS index
 * convention, ACCUMULATED into the caller's buffers (+=).  A NULL buffer
 * skips that block.  C is the host CI vector of the current determinants. */
int qdkgb_rdms_spin_dep(qdkgb_context* ctx, const double* C, double* ordm_aa, double* ordm_bb, double* trdm_aaaa,
                        double* trdm_bbbb, double* trdm_aabb);

/* Orbital entropies of the CI vector C over the context's determinants
 * (SortedDoubleLoopHamiltonianGenerator::form_entropies, external/macis/
 * include/macis/hamiltonian_generator/sorted_double_loop.hpp:755-903, with
 * the orbital-RDM intermediates of include/macis/util/entropies.hpp):
 * s1[norb] the single-orbital entropies; s2[norb*norb] the two-orbital
 * entropies and mi[norb*norb] the mutual information s1_i + s1_j - s2_ij
 * (symmetric, zero diagonal).  s2 and mi may be NULL (both NULL: only the
 * one-orbital terms are accumulated).  Integrals must be set (orbital count). */
int qdkgb_orbital_entropies(qdkgb_context* ctx, const double* C, double* s1, double* s2, double* mi);

/* ------------------------------------------------------------ ASCI
 * ASCISettings (external/macis/include/macis/asci/determinant_search.hpp:95-199),
 * the fields the search, grow and refine steps read. */
typedef struct qdkgb_asci_settings {
  int64_t ntdets_max;              /* default 100000 */
  int64_t ntdets_min;              /* default 100 */
  int64_t ncdets_max;              /* default 100 */
  int core_selection_fixed;        /* 0: Percentage (default), 1: Fixed */
  double core_selection_threshold; /* default 0.95 */
  double h_el_tol;                 /* default 1e-8 */
  double rv_prune_tol;             /* default 1e-8 */
  double grow_factor;              /* default 8 */
  double min_grow_factor;          /* default 1.01 */
  double growth_backoff_rate;      /* default 0.5 */
  double growth_recovery_rate;     /* default 1.1 */
  int64_t max_refine_iter;         /* default 6 */
  double refine_energy_tol;        /* default 1e-6 */
  int warm_start;                  /* default 1 */
  double min_warm_start_overlap;   /* default 0.5 */
  double taper_grow_factor;        /* default 0 (off): the growth factor of a step that would pass ntdets_max */
  int just_singles;                /* default 0: 1 = the search enumerates single excitations only */
  double min_patch_overlap;        /* default 0.3: patch the previous Hamiltonian when kept/new >= this */
  int grow_with_rot;               /* default 0: 1 = natural-orbital rotation after each grow step from
                                      rot_size_start determinants on (grow.hpp:163-252) */
  int64_t rot_size_start;          /* default 1000 */
} qdkgb_asci_settings;

void qdkgb_asci_default_settings(qdkgb_asci_settings* s);

/* One determinant search (asci_search, determinant_search.hpp:808-1123) from a
 * core list (alpha-major sorted) with coefficients: returns in out_a/out_b the
 * selected targets (tie-inclusive top ndets_max - ncore by |rv|) followed by
 * the core; *n_out receives the count (written only up to cap). */
int qdkgb_asci_search(qdkgb_context* ctx, const qdkgb_asci_settings* s, int64_t ncore, const uint64_t* core_alpha,
                      const uint64_t* core_beta, const double* core_coeff, double E0, int64_t ndets_max, int64_t cap,
                      uint64_t* out_a, uint64_t* out_b, int64_t* n_out);

/* asci_grow then asci_refine (grow.hpp:45-268, refine.hpp:44-237, iteration
 * asci_iter, iteration.hpp:50-226) with the search, the H build and the
 * Davidson on the device.  Starts from (n0 determinants, coefficients, E0 =
 * electronic energy of the start); returns the final list sorted by
 * spin_comparator with its eigenvector, the electronic energy and the energy
 * after the grow phase.  Integrals must be set. */
int qdkgb_asci(qdkgb_context* ctx, const qdkgb_asci_settings* s, const qdkgb_davidson_settings* ci, double matel_tol,
               int64_t n0, const uint64_t* a0, const uint64_t* b0, const double* c0, double E0, int do_grow,
               int do_refine, int64_t cap, uint64_t* out_a, uint64_t* out_b, double* out_c, int64_t* n_out,
               double* E_out, double* E_grow_out);
/* The orbital rotation of the last qdkgb_asci call with grow_with_rot (no
 * counterpart: the reference rotates its generator's integrals in place):
 * U (norb x norb, column-major) holds the final orbitals as columns over the
 * orbitals the integrals were given in; the identity when no rotation took
 * place.  After such a call the context's integrals are the rotated ones and
 * the returned determinants and coefficients refer to the rotated orbitals,
 * as the reference's generator does after asci_grow. */
int qdkgb_asci_rotation(const qdkgb_context* ctx, double* U);

/* Where the last qdkgb_asci call on this context spent its time (no
 * counterpart; the reference logs the same phases through its asci_search /
 * h_build / davidson loggers): seconds[0] the determinant searches,
 * seconds[1] the determinant-space set-ups, seconds[2] the Hamiltonian
 * builds, seconds[3] the Davidson solves; *iterations (may be NULL) the
 * asci_iter count; *patched (may be NULL) how many of its Hamiltonians were
 * patched from the previous iteration's instead of built from scratch (the
 * role of the reference's incremental build, incremental_h_build.hpp:38-356;
 * the patched CSR is bit-identical to a rebuild; FP64 storage only, and off
 * when the environment sets QDKGB_ASCI_FULL_BUILD=1). */
int qdkgb_asci_phase_times(const qdkgb_context* ctx, double* seconds, int64_t* iterations, int64_t* patched);

/* ASCI-PT2 (asci_pt2_constraint, external/macis/include/macis/asci/pt2.hpp:
 * 59-565): E_PT2 = sum over the determinants Q outside the wavefunction of
 * (sum_P C_P <Q|H|P>)^2 / (E0 - H_QQ), single contributions with
 * |C_P <Q|H|P>| < pt2_tol dropped (the reference default is 1e-16), H_QQ by
 * the fast diagonals.  The wavefunction (alpha[i], beta[i], C[i]) must be
 * sorted by spin_comparator (alpha string, then beta; QDKGB_ERR_INVALID
 * "PT2 Only Works with Sorted Wfns" otherwise); E0 is its electronic energy.
 * Integrals must be set.  max_slots bounds the hash table of target
 * determinants (the memory role of the reference's pt2_reserve_count; 0: half
 * of the free device memory): when every contribution would not fit, the
 * target space is split by a hash into passes.  *ept2 receives E_PT2,
 * *n_external (may be NULL) the number of distinct external determinants. */
int qdkgb_asci_pt2(qdkgb_context* ctx, int64_t ndets, const uint64_t* alpha, const uint64_t* beta, const double* C,
                   double E0, double pt2_tol, int64_t max_slots, double* ept2, int64_t* n_external);

/* ------------------------------------------------------------ CASSCF
 * MCSCFSettings (external/macis/include/macis/mcscf/mcscf.hpp:22-52). */
typedef struct qdkgb_mcscf_settings {
  int64_t max_macro_iter;  /* default 100 */
  double max_orbital_step; /* default 0.5 */
  double orb_grad_tol;     /* orb_grad_tol_mcscf, RMS of the orbital gradient (default 5e-6) */
  int enable_diis;         /* default 1 */
  int64_t diis_start_iter; /* default 3 */
  int64_t diis_nkeep;      /* default 10 */
  double ci_res_tol;       /* default 1e-8 */
  int64_t ci_max_subspace; /* default 200 (at most 254 here) */
  double ci_matel_tol;     /* default machine epsilon */
} qdkgb_mcscf_settings;

void qdkgb_mcscf_default_settings(qdkgb_mcscf_settings* s);

/* CASSCF (casscf_diis, external/macis/include/macis/mcscf/mcscf.hpp:54-60,
 * mcscf_impl.hpp:25-262): orbital optimisation of a CAS(nalpha + nbeta
 * electrons, nact orbitals) wavefunction over norb molecular orbitals (ninact
 * doubly occupied below the active ones, the rest virtual), from the
 * column-major full integrals T (norb^2) and V (norb^4) and the core energy;
 * the CASCI and RDMs of every macro iteration and the integral transform run
 * on the device.  A1 (nact^2) / A2 (nact^4) are the spin-traced active RDMs:
 * used as the start when trace(A1) = nalpha + nbeta, overwritten with the
 * final ones.  *E receives the total energy (also when not converged, as the
 * reference returns it); U (norb^2, may be NULL) the total orbital rotation;
 * *iterations and *converged (may be NULL) the macro iterations and the
 * convergence flag. */
int qdkgb_casscf(qdkgb_context* ctx, const qdkgb_mcscf_settings* s, int nalpha, int nbeta, int norb, int ninact,
                 int nact, double E_core, const double* T, const double* V, double* A1, double* A2, double* E,
                 double* U, int64_t* iterations, int* converged);

/* ------------------------------------------------------------ CASCI driver
 * cas_helper::impl / compute_casci_rdms (cpp/src/qdk/chemistry/algorithms/
 * microsoft/macis_cas.cpp:35-117, include/macis/mcscf/cas.hpp:33-64): FCI
 * space, the operator of qdkgb_build_operator (stored, or the direct sigma
 * when the stored matrix would not fit or the solve is mixed precision on a
 * space of 2^17 or more determinants), Davidson.  E receives the electronic energy (the caller
 * adds the core energy, macis_cas.cpp:113); C (may be NULL) the CI vector in
 * MACIS determinant order. */
int qdkgb_casci(qdkgb_context* ctx, int norb, int nalpha, int nbeta, const double* T, const double* V, int layout,
                const qdkgb_davidson_settings* s, double matel_tol, double* E, double* C, qdkgb_davidson_info* info);

/* ------------------------------------------------------------ batched CASCI
 * Many independent complete active spaces in one call.  The reference solves
 * them one at a time (MultiConfigurationCalculator::run -> cas_helper::impl,
 * cpp/src/qdk/chemistry/algorithms/microsoft/macis_cas.cpp:35-117, per
 * instance); here instances of one shape share their determinant space and
 * every solver step is one launch over all of them (inner iteration replayed
 * from a CUDA graph).  Energies are electronic (add each core energy);
 * the spin-summed 1-RDM of instance i (alpha + beta, norb_i x norb_i) lands at
 * rdm1 + sum_{j<i} norb_j^2 (rdm1 may be NULL).  QDKGB_ERR_NOT_CONVERGED when
 * an instance did not reach res_tol within max_cycles restarts (its energy is
 * still written). */
typedef struct {
  int norb, nalpha, nbeta;
  const double* T; /* norb x norb, column-major, host */
  const double* V; /* norb^4, column-major, host */
} qdkgb_cas_instance;

typedef struct {
  double res_tol;             /* full-precision residual norm per instance (1e-8) */
  int precision;              /* QDKGB_PREC_MIXED (default) or QDKGB_PREC_FP64 */
  int max_subspace;           /* subspace size of one cycle, 2..64 (24) */
  int max_cycles;             /* restarts before giving up (200) */
  double matel_tol;           /* Hamiltonian threshold (machine epsilon) */
  double min_abs_denominator; /* preconditioner clamp (1e-12) */
  int use_graph;              /* lockstep path: replay the inner iteration from a CUDA graph (1) */
  int64_t max_slab_bytes;     /* stored-matrix bytes per sub-batch (96 GiB) */
  int persistent;             /* 0 (default): the lockstep launch sequence over all instances;
                                 1: one persistent cluster launch per shape solves every instance */
  int cluster;                /* persistent: CTAs per instance, 1, 2, 4 or 8; 0 (default): measured
                                 per shape on first use and kept on the context (qdkgb_batch_plan) */
} qdkgb_batch_settings;

typedef struct {
  int iterations;    /* sigma applications, maximum over instances */
  int graph_replays; /* inner iterations launched from the graph */
  double seconds;    /* wall time of the call */
} qdkgb_batch_info;

int qdkgb_batch_default_settings(qdkgb_batch_settings* s);
/* The persistent batched solver's tuning record on this context (no
 * counterpart in the reference): for each shape tuned so far, in tuning
 * order, shape[3 i .. 3 i + 2] = (norb, nalpha, nbeta), cluster[i] = CTAs
 * per instance in use, ncand[i] timed candidates with their cluster sizes
 * cand_cluster[4 i + j] and milliseconds cand_ms[4 i + j] (a tuning run: a
 * few inner iterations of every instance).  Records up to cap are written;
 * *nshapes receives the number of records.  Any array may be NULL. */
int qdkgb_batch_plan(const qdkgb_context* ctx, int cap, int* nshapes, int* shape, int* cluster, int* ncand,
                     int* cand_cluster, double* cand_ms);
int qdkgb_casci_batch(qdkgb_context* ctx, int ninst, const qdkgb_cas_instance* inst, const qdkgb_batch_settings* s,
                      double* energies, double* rdm1, int* iterations, qdkgb_batch_info* info);

/* ------------------------------------------------------------ allocation-free sigma
 * No counterpart in the reference.  For callers that cannot call cudaMalloc
 * while they run: code being captured into a CUDA graph (allocation is not
 * allowed during stream capture), applications whose device memory is owned
 * by another allocator (a framework's caching pool, a fixed arena), and
 * latency-critical loops that must not synchronise.  It is the full-precision
 * sigma of the split storage (y = (hi + lo) x, float-float products and sums,
 * FP64 result) on caller-owned device arrays, with its scratch (x split into
 * two FP32 halves) in a fixed file-scope device array instead of an
 * allocation.
 *   - n <= QDKGB_NOALLOC_MAX_ROWS (1,048,576 rows; 8 MiB of scratch that every
 *     GPU loading the library holds until exit); larger n returns
 *     QDKGB_ERR_INVALID with the reason in qdkgb_last_error(NULL).
 *   - rowptr (n+1, int64), colind (int32), hi/lo (FP32, as QDKGB_H_SPLIT32
 *     stores them), x and y (FP64, n) are device pointers on the current
 *     device; stream is a cudaStream_t (NULL = legacy default stream).
 *   - The first call on a device looks up the scratch's device address (once
 *     per device, with that device current); make that first call before any
 *     stream capture.  The address is kept for the life of the process: a
 *     cudaDeviceReset (which destroys the primary context and the array with
 *     it) invalidates it, so do not call this entry point on a device after
 *     resetting that device.
 *   - A CUDA error already pending on the calling thread is reported
 *     (QDKGB_ERR_CUDA) without launching and is not cleared.
 *   - The scratch is overwritten completely by every call, so nothing has to
 *     be cleared; all calls share it, so calls that overlap on the GPU (two
 *     streams at once) race.
 *   - No cudaMalloc, cudaFree or allocating library routine is called. */
#define QDKGB_NOALLOC_MAX_ROWS (1 << 20)
int qdkgb_sigma_split_noalloc(int64_t n, const int64_t* rowptr, const int32_t* colind, const float* hi,
                              const float* lo, const double* x, double* y, void* stream);

/* ------------------------------------------------------------ version, counters */
const char* qdkgb_version(void);
/* Number of kernel launches this library has issued in this process. */
int64_t qdkgb_kernel_launches(void);

#ifdef __cplusplus
}
#endif
#endif /* QDKGB_H */
