// C++ adapter of MACIS's interfaces over the qdkgb C ABI (header only).
//
// A maintainer of the reference adds this header and links libqdkgb.so; it
// needs the reference's MACIS headers on the include path.  It provides:
//
//   qdkgb_macis::GpuHamiltonianGenerator<WfnType>
//       a macis::HamiltonianGenerator<WfnType>
//       (include/macis/hamiltonian_generator.hpp:32-294) implementing every
//       pure virtual on the GPU: make_csr_hamiltonian_block_{32,64}bit_,
//       form_rdms, form_rdms_spin_dep, form_entropies.  Its non-virtual
//       helpers (matrix_element, fast diagonals, the integral intermediates)
//       stay the base class's CPU code.
//   qdkgb_macis::GpuSparseOperator
//       the Davidson operator seam, operator_action(m, alpha, V, LDV, beta,
//       AV, LDAV) (include/macis/solvers/davidson.hpp:79-90), on the
//       operator built on the device.
//
// Determinants cross the ABI as two uint64 arrays (alpha = low N/2 bits of
// the bitset, raw_bitset.hpp:55-106), so WfnType is wfn_t<N> with N <= 128.
// Lists must be alpha-grouped with one common beta order, which
// generate_hilbert_space and any spin_comparator-sorted list are.
// Errors are thrown as std::runtime_error with the library's message
// (non-convergence as "Davidson Did Not Converge!", as the reference throws).
#pragma once

#include <cstdint>
#include <iterator>
#include <stdexcept>
#include <string>
#include <vector>

#include <macis/hamiltonian_generator.hpp>
#include <macis/wfn/raw_bitset.hpp>

#include "qdkgb.h"

namespace qdkgb_macis {

inline void check(qdkgb_context* c, int rc) {
  if (rc == QDKGB_OK) return;
  if (rc == QDKGB_ERR_NOT_CONVERGED) throw std::runtime_error("Davidson Did Not Converge!");
  throw std::runtime_error(std::string("qdkgb: ") + qdkgb_last_error(c));
}

template <typename WfnType>
class GpuHamiltonianGenerator : public macis::HamiltonianGenerator<WfnType> {
 public:
  using base = macis::HamiltonianGenerator<WfnType>;
  using full_det_iterator = typename base::full_det_iterator;
  using matrix_span_t = typename base::matrix_span_t;
  using rank4_span_t = typename base::rank4_span_t;
  template <typename index_t>
  using csr_t = sparsexx::csr_matrix<double, index_t>;

  // T (n x n) and V (n^4) column-major, as the base class reads them
  GpuHamiltonianGenerator(matrix_span_t T, rank4_span_t V, int device = 0) : base(T, V) {
    check(nullptr, qdkgb_create(&ctx_, device));
    norb_ = (int)T.extent(0);
    const int rc = qdkgb_set_integrals(ctx_, norb_, T.data_handle(), V.data_handle(), QDKGB_LAYOUT_COLMAJOR);
    if (rc) {
      const std::string msg = qdkgb_last_error(ctx_);
      qdkgb_destroy(ctx_);
      throw std::runtime_error("qdkgb: " + msg);
    }
  }
  ~GpuHamiltonianGenerator() noexcept override { qdkgb_destroy(ctx_); }
  GpuHamiltonianGenerator(const GpuHamiltonianGenerator&) = delete;
  GpuHamiltonianGenerator& operator=(const GpuHamiltonianGenerator&) = delete;

  qdkgb_context* context() const { return ctx_; }

 protected:
  csr_t<int32_t> make_csr_hamiltonian_block_32bit_(full_det_iterator bb, full_det_iterator be, full_det_iterator kb,
                                                   full_det_iterator ke, double thresh) override {
    return block<int32_t>(bb, be, kb, ke, thresh);
  }
  csr_t<int64_t> make_csr_hamiltonian_block_64bit_(full_det_iterator bb, full_det_iterator be, full_det_iterator kb,
                                                   full_det_iterator ke, double thresh) override {
    return block<int64_t>(bb, be, kb, ke, thresh);
  }

 public:
  // accumulates (+=); a null data_handle skips the block (the reference's contract)
  void form_rdms(full_det_iterator bb, full_det_iterator be, full_det_iterator kb, full_det_iterator ke, double* C,
                 matrix_span_t ordm, rank4_span_t trdm) override {
    same_list(bb, be, kb, ke, "form_rdms");
    upload(bb, be);
    check(ctx_, qdkgb_rdms(ctx_, C, ordm.data_handle(), trdm.data_handle()));
  }
  void form_rdms_spin_dep(full_det_iterator bb, full_det_iterator be, full_det_iterator kb, full_det_iterator ke,
                          double* C, matrix_span_t ordm_aa, matrix_span_t ordm_bb, rank4_span_t trdm_aaaa,
                          rank4_span_t trdm_bbbb, rank4_span_t trdm_aabb) override {
    same_list(bb, be, kb, ke, "form_rdms_spin_dep");
    upload(bb, be);
    check(ctx_, qdkgb_rdms_spin_dep(ctx_, C, ordm_aa.data_handle(), ordm_bb.data_handle(), trdm_aaaa.data_handle(),
                                    trdm_bbbb.data_handle(), trdm_aabb.data_handle()));
  }
  void form_entropies(full_det_iterator bb, full_det_iterator be, full_det_iterator kb, full_det_iterator ke,
                      double* C, std::vector<double>& single_orbital_entropies, matrix_span_t s2_entropy,
                      matrix_span_t mutual_information) override {
    same_list(bb, be, kb, ke, "form_entropies");
    upload(bb, be);
    single_orbital_entropies.resize(norb_);
    check(ctx_, qdkgb_orbital_entropies(ctx_, C, single_orbital_entropies.data(), s2_entropy.data_handle(),
                                        mutual_information.data_handle()));
  }

 private:
  qdkgb_context* ctx_ = nullptr;
  int norb_ = 0;
  std::vector<uint64_t> la_, lb_;  // the list on the device

  static void same_list(full_det_iterator bb, full_det_iterator be, full_det_iterator kb, full_det_iterator ke,
                        const char* what) {
    if (bb != kb || be != ke)
      throw std::runtime_error(std::string("GPU generator: ") + what + " needs the bra and ket lists to be the same");
  }

  void upload(full_det_iterator b, full_det_iterator e) {
    using traits = macis::wavefunction_traits<WfnType>;
    std::vector<uint64_t> a, bt;
    a.reserve(std::distance(b, e));
    bt.reserve(std::distance(b, e));
    for (auto it = b; it != e; ++it) {
      a.push_back((uint64_t)macis::fast_to_ullong(traits::alpha_string(*it)));
      bt.push_back((uint64_t)macis::fast_to_ullong(traits::beta_string(*it)));
    }
    if (a == la_ && bt == lb_) return;  // the device already holds this list
    check(ctx_, qdkgb_set_dets(ctx_, (int64_t)a.size(), a.data(), bt.data()));
    la_.swap(a);
    lb_.swap(bt);
  }

  // The symmetric block (bra list == ket list), or a bra sub-range of the
  // ket list: the rows [bra_begin, bra_end) of the ket list's Hamiltonian
  // against every ket, columns relative to ket_begin.  In the sub-range case
  // the elements above the diagonal are the symmetric build's (bra = the
  // lower-index determinant), equal to the reference's general block up to
  // the rounding of the single-excitation sums.
  template <typename index_t>
  csr_t<index_t> block(full_det_iterator bb, full_det_iterator be, full_det_iterator kb, full_det_iterator ke,
                       double thresh) {
    const int64_t off = std::distance(kb, bb), rows = std::distance(bb, be), nk = std::distance(kb, ke);
    if (off < 0 || off + rows > nk)
      throw std::runtime_error("GPU generator: the bra range must lie within the ket range");
    upload(kb, ke);
    int64_t nnz = 0;
    check(ctx_, qdkgb_build_hamiltonian(ctx_, thresh, QDKGB_H_FP64, &nnz));
    std::vector<index_t> rp(rows + 1);
    auto get = [&](index_t* r, index_t* c, double* v) {
      if constexpr (sizeof(index_t) == 4)
        return qdkgb_get_csr32_rows(ctx_, off, off + rows, (int32_t*)r, (int32_t*)c, v);
      else
        return qdkgb_get_csr64_rows(ctx_, off, off + rows, (int64_t*)r, (int64_t*)c, v);
    };
    check(ctx_, get(rp.data(), nullptr, nullptr));
    std::vector<index_t> ci(rp[rows]);
    std::vector<double> nz(rp[rows]);
    check(ctx_, get(rp.data(), ci.data(), nz.data()));
    return csr_t<index_t>(rows, nk, std::move(rp), std::move(ci), std::move(nz));
  }
};

// The operator of macis::davidson (davidson.hpp:79-90) on the device: build
// the operator on the context first (qdkgb_build_operator or
// qdkgb_build_hamiltonian), then pass this to macis::davidson(N, max_m, op,
// D, tol, X) in place of SparseMatrixOperator.
struct GpuSparseOperator {
  qdkgb_context* ctx;
  void operator_action(size_t m, double alpha, const double* V, size_t LDV, double beta, double* AV,
                       size_t LDAV) const {
    check(ctx, qdkgb_operator_action(ctx, (int64_t)m, alpha, V, (int64_t)LDV, beta, AV, (int64_t)LDAV));
  }
};

}  // namespace qdkgb_macis
