// Compiled by tests/test_macis_adapter_cpu.py against the reference's MACIS
// headers: the adapter's generator must be concrete (every pure virtual of
// macis::HamiltonianGenerator overridden) for both bitset widths, and its
// operator must satisfy macis::davidson's functor contract.  Run without a
// GPU, constructing the generator reports the library's error; with one, it
// builds a CAS(4e,4o) block and solves it with the reference's davidson on
// the device operator.
#include <cstdio>
#include <type_traits>

#include "qdkgb_macis_generator.hpp"

#include <macis/csr_hamiltonian.hpp>
#include <macis/sd_operations.hpp>
#include <macis/solvers/davidson.hpp>

int main() {
  using gen64 = qdkgb_macis::GpuHamiltonianGenerator<macis::wfn_t<64>>;
  using gen128 = qdkgb_macis::GpuHamiltonianGenerator<macis::wfn_t<128>>;
  static_assert(!std::is_abstract_v<gen64> && !std::is_abstract_v<gen128>, "generator must implement every virtual");
  std::vector<double> T(16, 0.0), V(256, 0.0);
  for (int p = 0; p < 4; ++p) T[p + 4 * p] = -1.0 + 0.25 * p;
  for (int p = 0; p < 4; ++p)
    for (int q = 0; q < 4; ++q) V[p + 4 * (p + 4 * (q + 4 * q))] = 0.1;
  try {
    gen64 g(macis::matrix_span<double>(T.data(), 4, 4), macis::rank4_span<double>(V.data(), 4, 4, 4, 4));
    auto dets = macis::generate_hilbert_space<macis::wfn_t<64>>(4, 2, 2);
    auto H = g.make_csr_hamiltonian_block<int64_t>(dets.begin(), dets.end(), dets.begin(), dets.end(), 1e-16);
    qdkgb_davidson_settings s;
    qdkgb_davidson_default_settings(&s);
    std::vector<double> D(dets.size()), X(dets.size(), 0.0);
    qdkgb_macis::check(g.context(), qdkgb_diagonal(g.context(), D.data()));
    X[0] = 1.0;
    qdkgb_macis::GpuSparseOperator op{g.context()};
    auto [it, E] = macis::davidson((int64_t)dets.size(), 20, op, D.data(), 1e-8, X.data());
    std::printf("device: nnz %zu E %.12f iterations %zu\n", (size_t)H.nnz(), E, (size_t)it);
  } catch (const std::runtime_error& e) {
    std::printf("no device: %s\n", e.what());
  }
  return 0;
}
