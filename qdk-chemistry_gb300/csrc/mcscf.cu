// CASSCF (replaces macis::casscf_diis / mcscf_impl, external/macis/include/
// macis/mcscf/mcscf_impl.hpp:25-262, with the pieces of src/macis/mcscf/
// fock_matrices.cxx, orbital_gradient.cxx, orbital_hessian.cxx,
// orbital_steps.cxx, orbital_rotation_utilities.cxx, include/macis/mcscf/
// diis.hpp and src/macis/util/transform.cxx).
//
// One macro iteration: the active-space Hamiltonian in the current orbitals
// (inactive Fock matrix, active blocks), the CASCI and its spin-traced RDMs on
// the device (the library's own H build, Davidson warm-started from the
// previous CI vector and RDM pair walk, on an internal context holding the
// active space), the generalized Fock matrix and the orbital gradient, the
// step -g / (approximate diagonal Hessian) capped at max_orbital_step, DIIS on
// the accumulated rotation with the gradient as error, U = exp(-K), and the
// integrals transformed from the original ones by U on the device (four
// one-index quarter transforms, n^5 FMAs each).  The remaining work is O(n^2)
// to O(n^3 n_act) host arithmetic on n <= 64 orbitals.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "common.cuh"
#include "internal.h"

namespace qdkgb {
namespace {

// Y[j + n k + n^2 l + n^3 p] = sum_a X[a + n (j + n k + n^2 l)] C[a + n p]:
// contracts the leading index of a column-major n^4 tensor with C and appends
// the new index last; four passes give Y(p,q,r,s) = sum C_ap C_bq C_cr C_ds X(abcd)
__global__ void k_quarter_transform(const double* __restrict__ X, const double* __restrict__ C,
                                    double* __restrict__ Y, int n) {
  const int64_t n3 = (int64_t)n * n * n, total = n3 * n;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t rest = t % n3, p = t / n3;
    const double* x = X + rest * n;
    const double* c = C + p * n;
    double s = 0.;
    for (int a = 0; a < n; ++a) s = fma(x[a], c[a], s);
    Y[t] = s;
  }
}

using Mat = std::vector<double>;  // column-major n x n

// C = A^T B (transA) or A B, n x n
void matmul(int n, const double* A, bool transA, const double* B, double* C) {
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) {
      double s = 0.;
      for (int k = 0; k < n; ++k) s += (transA ? A[k + (size_t)n * i] : A[i + (size_t)n * k]) * B[k + (size_t)n * j];
      C[i + (size_t)n * j] = s;
    }
}

// exp(-alpha K) for antisymmetric K (compute_orbital_rotation,
// orbital_gradient.cxx): scaling and squaring of the Taylor series
Mat orbital_rotation(int n, double alpha, const Mat& K) {
  const size_t n2 = (size_t)n * n;
  Mat A(n2);
  double nrm = 0.;
  for (int i = 0; i < n; ++i) {
    double row = 0.;
    for (int j = 0; j < n; ++j) row += std::fabs(K[i + (size_t)n * j]);
    nrm = std::max(nrm, std::fabs(alpha) * row);
  }
  int sq = 0;
  while (nrm > 0.25 && sq < 60) {
    nrm *= 0.5;
    ++sq;
  }
  const double sc = -alpha * std::ldexp(1., -sq);
  for (size_t i = 0; i < n2; ++i) A[i] = sc * K[i];
  Mat E(n2, 0.), term(n2, 0.), tmp(n2);
  for (int i = 0; i < n; ++i) E[i + (size_t)n * i] = term[i + (size_t)n * i] = 1.;
  for (int k = 1; k <= 30; ++k) {
    matmul(n, term.data(), false, A.data(), tmp.data());
    double tm = 0.;
    for (size_t i = 0; i < n2; ++i) {
      term[i] = tmp[i] / k;
      E[i] += term[i];
      tm = std::max(tm, std::fabs(term[i]));
    }
    if (tm < 1e-18) break;
  }
  for (int s = 0; s < sq; ++s) {
    matmul(n, E.data(), false, E.data(), tmp.data());
    E.swap(tmp);
  }
  return E;
}

// eigen-decomposition of a small symmetric matrix (cyclic Jacobi): A is
// overwritten by its eigenvalues on the diagonal, Z receives the eigenvectors
void sym_eigen(int m, std::vector<double>& A, std::vector<double>& Z) {
  Z.assign((size_t)m * m, 0.);
  for (int i = 0; i < m; ++i) Z[i + (size_t)m * i] = 1.;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0., tot = 0.;
    for (int p = 0; p < m; ++p)
      for (int q = 0; q < m; ++q) {
        const double v = A[p + (size_t)m * q] * A[p + (size_t)m * q];
        tot += v;
        if (p != q) off += v;
      }
    if (!(off > 1e-32 * tot)) break;
    for (int p = 0; p < m; ++p)
      for (int q = p + 1; q < m; ++q) {
        const double apq = A[p + (size_t)m * q];
        if (apq == 0.) continue;
        const double th = (A[q + (size_t)m * q] - A[p + (size_t)m * p]) / (2. * apq);
        const double t = (th >= 0. ? 1. : -1.) / (std::fabs(th) + std::sqrt(th * th + 1.));
        const double c = 1. / std::sqrt(t * t + 1.), s = t * c;
        for (int r = 0; r < m; ++r) {
          const double x = A[r + (size_t)m * p], y = A[r + (size_t)m * q];
          A[r + (size_t)m * p] = c * x - s * y;
          A[r + (size_t)m * q] = s * x + c * y;
        }
        for (int r = 0; r < m; ++r) {
          const double x = A[p + (size_t)m * r], y = A[q + (size_t)m * r];
          A[p + (size_t)m * r] = c * x - s * y;
          A[q + (size_t)m * r] = s * x + c * y;
        }
        for (int r = 0; r < m; ++r) {
          const double x = Z[r + (size_t)m * p], y = Z[r + (size_t)m * q];
          Z[r + (size_t)m * p] = c * x - s * y;
          Z[r + (size_t)m * q] = s * x + c * y;
        }
      }
  }
}

// DIIS (diis.hpp): keeps the last nkeep (vector, error) pairs; the
// extrapolation solves the bordered error-overlap system in the least-squares
// sense (pseudo-inverse through its eigen-decomposition, cut at machine
// precision relative to the largest eigenvalue)
struct Diis {
  size_t nkeep;
  std::vector<std::pair<std::vector<double>, std::vector<double>>> pairs;
  void add(const std::vector<double>& v, const std::vector<double>& e) {
    if (pairs.size() == nkeep) pairs.erase(pairs.begin());
    pairs.emplace_back(v, e);
  }
  std::vector<double> extrapolate() const {
    const int m = (int)pairs.size(), mb = m + 1;
    std::vector<double> B((size_t)mb * mb, 0.), Z;
    for (int i = 0; i < m; ++i)
      for (int j = i; j < m; ++j) {
        double d = 0.;
        const auto &ei = pairs[i].second, &ej = pairs[j].second;
        for (size_t k = 0; k < ei.size(); ++k) d += ei[k] * ej[k];
        B[i + (size_t)mb * j] = B[j + (size_t)mb * i] = d;
      }
    for (int i = 0; i < m; ++i) B[i + (size_t)mb * m] = B[m + (size_t)mb * i] = 1.;
    sym_eigen(mb, B, Z);
    double lmax = 0.;
    for (int i = 0; i < mb; ++i) lmax = std::max(lmax, std::fabs(B[i + (size_t)mb * i]));
    const double cut = 2.220446049250313e-16 * lmax * mb;
    std::vector<double> c(mb, 0.);  // c = B^+ (0, ..., 0, 1)
    for (int k = 0; k < mb; ++k) {
      const double l = B[k + (size_t)mb * k];
      if (!(std::fabs(l) > cut)) continue;
      const double w = Z[m + (size_t)mb * k] / l;
      for (int i = 0; i < mb; ++i) c[i] += Z[i + (size_t)mb * k] * w;
    }
    std::vector<double> x(pairs[0].first.size(), 0.);
    for (int i = 0; i < m; ++i)
      for (size_t k = 0; k < x.size(); ++k) x[k] += c[i] * pairs[i].first[k];
    return x;
  }
};

void check_rc(qdkgb_context* sub, int rc) {
  if (rc) throw Error(rc, std::string("CASSCF active-space CASCI: ") + qdkgb_last_error(sub));
}

struct SubContext {
  qdkgb_context* h = nullptr;
  ~SubContext() {
    if (h) qdkgb_destroy(h);
  }
};

}  // namespace

double casscf(Context* c, const qdkgb_mcscf_settings& S, int nalpha, int nbeta, int norb, int ninact, int nact,
              double E_core, const double* T0, const double* V0, double* A1, double* A2, double* U_out,
              int64_t* iterations, int* converged_out) {
  NvtxRange nvtx_range("qdkgb.casscf");
  const int no = norb, ni = ninact, na = nact, nv = norb - ninact - nact;
  if (no < 1 || no > 64 || ni < 0 || na < 1 || nv < 0) throw Error(QDKGB_ERR_INVALID, "bad orbital partition");
  if (nalpha < 0 || nbeta < 0 || nalpha > na || nbeta > na) throw Error(QDKGB_ERR_INVALID, "bad active electron count");
  const size_t no2 = (size_t)no * no, no4 = no2 * no2, na2 = (size_t)na * na, na4 = na2 * na2;
  const int rot = nv * (ni + na) + na * ni;
  const double rms = std::sqrt((double)std::max(rot, 1));
  auto Vat = [&](const double* V, int p, int q, int r, int s) {
    return V[p + (size_t)no * (q + (size_t)no * (r + (size_t)no * s))];
  };
  // ---- device buffers for the transform (released on every exit)
  ScopedBuffers<4> bufs(c);
  double* dV0 = dev_array<double>(c, bufs.b[0], no4);
  double* dV1 = dev_array<double>(c, bufs.b[1], no4);
  double* dV2 = dev_array<double>(c, bufs.b[2], no4);
  double* dU = dev_array<double>(c, bufs.b[3], no2);
  QDKGB_CUDA(cudaMemcpyAsync(dV0, V0, no4 * 8, cudaMemcpyHostToDevice, c->stream));
  Mat T(T0, T0 + no2), V(V0, V0 + no4);
  // ---- active-space CASCI on an internal context
  SubContext sub;
  check_rc(nullptr, qdkgb_create(&sub.h, c->device));
  int64_t ndets = 0;
  check_rc(sub.h, qdkgb_fci_dets(na, nalpha, nbeta, nullptr, nullptr, &ndets));
  std::vector<uint64_t> da(ndets), db(ndets);
  check_rc(sub.h, qdkgb_fci_dets(na, nalpha, nbeta, da.data(), db.data(), &ndets));
  std::vector<double> X(ndets, 0.);
  bool have_x = false;
  Mat Fi(no2), Fa(no2), F(no2), Q((size_t)na * no), Ta(na2), Va(na4);
  std::vector<double> aa(na2), bb(na2), aaaa(na4), bbbb(na4), aabb(na4);
  // active_hamiltonian + inactive_energy (fock_matrices.cxx)
  auto active_hamiltonian = [&](double& E_inact) {
    for (int p = 0; p < no; ++p)
      for (int q = 0; q < no; ++q) {
        double t = 0.;
        for (int i = 0; i < ni; ++i) t += 2. * Vat(V.data(), p, q, i, i) - Vat(V.data(), p, i, i, q);
        Fi[p + (size_t)no * q] = T[p + (size_t)no * q] + t;
      }
    for (int x = 0; x < na; ++x)
      for (int y = 0; y < na; ++y) Ta[x + (size_t)na * y] = Fi[(x + ni) + (size_t)no * (y + ni)];
    for (int x = 0; x < na; ++x)
      for (int y = 0; y < na; ++y)
        for (int z = 0; z < na; ++z)
          for (int w = 0; w < na; ++w)
            Va[x + na * (y + na * (z + (size_t)na * w))] = Vat(V.data(), x + ni, y + ni, z + ni, w + ni);
    E_inact = E_core;
    for (int i = 0; i < ni; ++i) E_inact += T[i + (size_t)no * i] + Fi[i + (size_t)no * i];
  };
  // CASCI of the active Hamiltonian: electronic energy, spin-traced RDMs
  // (E = sum g T + sum G V; compute_casci_rdms, cas.hpp:33-64)
  auto casci_rdms = [&]() {
    check_rc(sub.h, qdkgb_set_integrals(sub.h, na, Ta.data(), Va.data(), QDKGB_LAYOUT_COLMAJOR));
    if (!have_x) check_rc(sub.h, qdkgb_set_dets(sub.h, ndets, da.data(), db.data()));
    check_rc(sub.h, qdkgb_build_hamiltonian(sub.h, S.ci_matel_tol, QDKGB_H_FP64, nullptr));
    qdkgb_davidson_settings ds;
    qdkgb_davidson_default_settings(&ds);
    ds.max_m = std::min<int64_t>(S.ci_max_subspace, 254);
    ds.res_tol = S.ci_res_tol;
    ds.use_guess = have_x ? 1 : 0;
    double E = 0.;
    check_rc(sub.h, qdkgb_davidson(sub.h, &ds, &E, X.data(), nullptr));
    have_x = true;
    std::fill(aa.begin(), aa.end(), 0.);
    std::fill(bb.begin(), bb.end(), 0.);
    std::fill(aaaa.begin(), aaaa.end(), 0.);
    std::fill(bbbb.begin(), bbbb.end(), 0.);
    std::fill(aabb.begin(), aabb.end(), 0.);
    check_rc(sub.h, qdkgb_rdms_spin_dep(sub.h, X.data(), aa.data(), bb.data(), aaaa.data(), bbbb.data(), aabb.data()));
    for (size_t i = 0; i < na2; ++i) A1[i] = aa[i] + bb[i];
    for (int p = 0; p < na; ++p)
      for (int q = 0; q < na; ++q)
        for (int r = 0; r < na; ++r)
          for (int s = 0; s < na; ++s) {
            const size_t i = p + na * (q + na * (r + (size_t)na * s)), j = r + na * (s + na * (p + (size_t)na * q));
            A2[i] = aaaa[i] + bbbb[i] + aabb[i] + aabb[j];
          }
    return E;
  };
  // generalized Fock matrix (active_fock_matrix, aux_q_matrix,
  // generalized_fock_matrix) and the linear orbital gradient
  // (fock_to_linear_orb_grad): blocks virtual-inactive, virtual-active,
  // active-inactive
  std::vector<double> OG(rot), DH(rot);
  auto gradient = [&]() {
    for (int p = 0; p < no; ++p)
      for (int q = 0; q < no; ++q) {
        double t = 0.;
        for (int v = 0; v < na; ++v)
          for (int w = 0; w < na; ++w)
            t += A1[v + (size_t)na * w] *
                 (Vat(V.data(), p, q, v + ni, w + ni) - 0.5 * Vat(V.data(), p, w + ni, v + ni, q));
        Fa[p + (size_t)no * q] = t;
      }
    for (int v = 0; v < na; ++v)
      for (int p = 0; p < no; ++p) {
        double t = 0.;
        for (int w = 0; w < na; ++w)
          for (int x = 0; x < na; ++x)
            for (int y = 0; y < na; ++y)
              t += A2[v + na * (w + na * (x + (size_t)na * y))] * Vat(V.data(), p, w + ni, x + ni, y + ni);
        Q[v + (size_t)na * p] = 2. * t;
      }
    std::fill(F.begin(), F.end(), 0.);
    for (int i = 0; i < ni; ++i)
      for (int p = 0; p < no; ++p) F[i + (size_t)no * p] = 2. * (Fi[p + (size_t)no * i] + Fa[p + (size_t)no * i]);
    for (int v = 0; v < na; ++v)
      for (int p = 0; p < no; ++p) {
        double t = 0.;
        for (int w = 0; w < na; ++w) t += Fi[p + (size_t)no * (w + ni)] * A1[w + (size_t)na * v];
        F[(v + ni) + (size_t)no * p] = t + Q[v + (size_t)na * p];
      }
    auto FF = [&](int p, int q) { return F[p + (size_t)no * q]; };
    int k = 0;
    for (int i = 0; i < ni; ++i)
      for (int a = 0; a < nv; ++a) {
        const int A = a + ni + na;
        OG[k++] = 2. * (FF(A, i) - FF(i, A));
      }
    for (int x = 0; x < na; ++x)
      for (int a = 0; a < nv; ++a) {
        const int A = a + ni + na, Xo = x + ni;
        OG[k++] = 2. * (FF(A, Xo) - FF(Xo, A));
      }
    for (int i = 0; i < ni; ++i)
      for (int x = 0; x < na; ++x) {
        const int Xo = x + ni;
        OG[k++] = 2. * (FF(Xo, i) - FF(i, Xo));
      }
    double g = 0.;
    for (double v : OG) g += v * v;
    return std::sqrt(g);
  };
  // approx_diag_hessian (orbital_hessian.cxx) in the same block order
  auto diag_hessian = [&]() {
    auto FI = [&](int p) { return Fi[p + (size_t)no * p] + Fa[p + (size_t)no * p]; };
    int k = 0;
    for (int i = 0; i < ni; ++i)
      for (int a = 0; a < nv; ++a) DH[k++] = 4. * (FI(a + ni + na) - FI(i));
    for (int x = 0; x < na; ++x)
      for (int a = 0; a < nv; ++a)
        DH[k++] = 2. * A1[x + (size_t)na * x] * FI(a + ni + na) - 2. * F[(x + ni) + (size_t)no * (x + ni)];
    for (int i = 0; i < ni; ++i)
      for (int x = 0; x < na; ++x)
        DH[k++] = 2. * A1[x + (size_t)na * x] * FI(i) + 4. * (FI(x + ni) - FI(i)) -
                  2. * F[(x + ni) + (size_t)no * (x + ni)];
  };
  // linear_orb_rot_to_matrix
  auto to_matrix = [&](const std::vector<double>& k, Mat& K) {
    std::fill(K.begin(), K.end(), 0.);
    int t = 0;
    auto put = [&](int A, int I) {
      K[A + (size_t)no * I] = k[t];
      K[I + (size_t)no * A] = -k[t];
      ++t;
    };
    for (int i = 0; i < ni; ++i)
      for (int a = 0; a < nv; ++a) put(a + ni + na, i);
    for (int x = 0; x < na; ++x)
      for (int a = 0; a < nv; ++a) put(a + ni + na, x + ni);
    for (int i = 0; i < ni; ++i)
      for (int x = 0; x < na; ++x) put(x + ni, i);
  };
  // two_index_transform / four_index_transform (transform.cxx) of the
  // original integrals by U
  auto transform = [&](const Mat& U) {
    Mat tmp(no2);
    matmul(no, T0, false, U.data(), tmp.data());  // T0 U
    matmul(no, U.data(), true, tmp.data(), T.data());  // U^T T0 U
    QDKGB_CUDA(cudaMemcpyAsync(dU, U.data(), no2 * 8, cudaMemcpyHostToDevice, c->stream));
    const unsigned nb = (unsigned)std::min<int64_t>(((int64_t)no4 + 255) / 256, (int64_t)c->sm_count * 16);
    const double* src = dV0;
    double* bufs[2] = {dV1, dV2};
    for (int qpass = 0; qpass < 4; ++qpass) {
      k_quarter_transform<<<nb, 256, 0, c->stream>>>(src, dU, bufs[qpass & 1], no);
      QDKGB_CHECK_LAUNCH();
      src = bufs[qpass & 1];
    }
    QDKGB_CUDA(cudaMemcpyAsync(V.data(), src, no4 * 8, cudaMemcpyDeviceToHost, c->stream));
    QDKGB_CUDA(cudaStreamSynchronize(c->stream));
  };

  double E_inact = 0., E0 = 0.;
  active_hamiltonian(E_inact);
  double tr = 0.;
  for (int i = 0; i < na; ++i) tr += A1[i + (size_t)na * i];
  if (std::fabs(tr - nalpha - nbeta) > 1e-6) {
    std::fill(A1, A1 + na2, 0.);
    std::fill(A2, A2 + na4, 0.);
    (void)casci_rdms();
  }
  {
    double e1 = 0., e2 = 0.;
    for (size_t i = 0; i < na2; ++i) e1 += A1[i] * Ta[i];
    for (size_t i = 0; i < na4; ++i) e2 += A2[i] * Va[i];
    E0 = e1 + e2 + E_inact;
  }
  double gn = gradient();
  bool converged = gn < S.orb_grad_tol;
  Mat U_total(no2, 0.), K_total(no2, 0.), K_step(no2);
  for (int i = 0; i < no; ++i) U_total[i + (size_t)no * i] = 1.;
  Diis diis{(size_t)std::max<int64_t>(1, S.diis_nkeep), {}};
  int64_t it = 0;
  for (; it < S.max_macro_iter && !converged; ++it) {
    const Mat K_sav = K_total;
    // precond_cg_orbital_step (orbital_steps.cxx): -g / diagonal Hessian
    diag_hessian();
    std::vector<double> kl(rot);
    double amax = 0.;
    for (int p = 0; p < rot; ++p) {
      kl[p] = -OG[p] / DH[p];
      amax = std::max(amax, std::fabs(kl[p]));
    }
    if (amax > S.max_orbital_step)
      for (double& v : kl) v *= S.max_orbital_step / amax;
    to_matrix(kl, K_step);
    for (size_t i = 0; i < no2; ++i) K_total[i] += K_step[i];
    if (S.enable_diis && it >= S.diis_start_iter) {
      diis.add(K_total, OG);
      if (it >= S.diis_start_iter + 2) K_total = diis.extrapolate();
    }
    if (it == 0) {
      U_total = orbital_rotation(no, 1., K_total);
    } else {
      Mat dK(no2), tmp(no2);
      for (size_t i = 0; i < no2; ++i) dK[i] = K_total[i] - K_sav[i];
      const Mat Us = orbital_rotation(no, 1., dK);
      matmul(no, U_total.data(), false, Us.data(), tmp.data());
      U_total.swap(tmp);
    }
    transform(U_total);
    active_hamiltonian(E_inact);
    std::fill(A1, A1 + na2, 0.);
    std::fill(A2, A2 + na4, 0.);
    E0 = casci_rdms() + E_inact;
    gn = gradient();
    converged = gn / rms < S.orb_grad_tol;
  }
  if (U_out) std::copy(U_total.begin(), U_total.end(), U_out);
  if (iterations) *iterations = it;
  if (converged_out) *converged_out = converged ? 1 : 0;
  return E0;  // the last energy also without convergence, as the reference returns it
}


// eigenvectors of -ordm (symmetrised) by cyclic Jacobi, ascending eigenvalues,
// ties in index order: the eigensolver the oracle uses in place of syev, so
// that both rotate to the same orbitals
void natural_orbitals(int n, const std::vector<double>& ordm, std::vector<double>& C) {
  const size_t k = (size_t)n;
  std::vector<double> a(k * k), q(k * k, 0.);
  for (size_t j = 0; j < k; ++j)
    for (size_t i = 0; i < k; ++i) a[i + k * j] = -0.5 * (ordm[i + k * j] + ordm[j + k * i]);
  for (size_t i = 0; i < k; ++i) q[i + k * i] = 1.;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0., tot = 0.;
    for (size_t j = 0; j < k; ++j)
      for (size_t i = 0; i < k; ++i) {
        const double v = a[i + k * j] * a[i + k * j];
        tot += v;
        if (i != j) off += v;
      }
    if (off <= 1e-32 * tot || off == 0.) break;
    for (size_t p = 0; p + 1 < k; ++p)
      for (size_t r = p + 1; r < k; ++r) {
        const double apq = a[p + k * r];
        if (apq == 0.) continue;
        const double app = a[p + k * p], aqq = a[r + k * r];
        const double theta = (aqq - app) / (2. * apq);
        const double t = (theta >= 0 ? 1. : -1.) / (std::fabs(theta) + std::sqrt(theta * theta + 1.));
        const double c = 1. / std::sqrt(t * t + 1.), s = t * c;
        for (size_t i = 0; i < k; ++i) {
          const double aip = a[i + k * p], air = a[i + k * r];
          a[i + k * p] = c * aip - s * air;
          a[i + k * r] = s * aip + c * air;
        }
        for (size_t i = 0; i < k; ++i) {
          const double api = a[p + k * i], ari = a[r + k * i];
          a[p + k * i] = c * api - s * ari;
          a[r + k * i] = s * api + c * ari;
        }
        for (size_t i = 0; i < k; ++i) {
          const double qip = q[i + k * p], qir = q[i + k * r];
          q[i + k * p] = c * qip - s * qir;
          q[i + k * r] = s * qip + c * qir;
        }
      }
  }
  std::vector<int> ord(n);
  for (int i = 0; i < n; ++i) ord[i] = i;
  std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return a[x + k * x] < a[y + k * y]; });
  C.assign(k * k, 0.);
  for (size_t j = 0; j < k; ++j)
    for (size_t i = 0; i < k; ++i) C[i + k * j] = q[i + k * ord[j]];
}

void rotate_integrals(Context* c, const std::vector<double>& C) {
  const int n = c->norb;
  const size_t n2 = (size_t)n * n, n4 = n2 * n2;
  Mat tmp(n2), T(n2);
  matmul(n, c->h_T.data(), false, C.data(), tmp.data());  // T C
  matmul(n, C.data(), true, tmp.data(), T.data());        // C^T T C
  ScopedBuffers<4> sb(c);
  double* dC = dev_array<double>(c, sb.b[0], n2);
  double* d0 = dev_array<double>(c, sb.b[1], n4);
  double* d1 = dev_array<double>(c, sb.b[2], n4);
  QDKGB_CUDA(cudaMemcpyAsync(dC, C.data(), n2 * 8, cudaMemcpyHostToDevice, c->stream));
  QDKGB_CUDA(cudaMemcpyAsync(d0, c->h_V.data(), n4 * 8, cudaMemcpyHostToDevice, c->stream));
  const unsigned nb = (unsigned)std::min<int64_t>(((int64_t)n4 + 255) / 256, (int64_t)c->sm_count * 16);
  double* bufs[2] = {d1, d0};
  const double* src = d0;
  for (int q = 0; q < 4; ++q) {
    k_quarter_transform<<<nb, 256, 0, c->stream>>>(src, dC, bufs[q & 1], n);
    QDKGB_CHECK_LAUNCH();
    src = bufs[q & 1];
  }
  QDKGB_CUDA(cudaMemcpyAsync(c->h_V.data(), src, n4 * 8, cudaMemcpyDeviceToHost, c->stream));
  QDKGB_CUDA(cudaStreamSynchronize(c->stream));
  c->h_T = T;
  build_integral_intermediates(c);
}

}  // namespace qdkgb
