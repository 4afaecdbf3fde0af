// Host-side helpers that spread list handling over the host's threads.
#pragma once
#include <algorithm>
#include <thread>
#include <vector>

namespace qdkgb {

// Sorts v on the host threads: chunks sorted in parallel, then merged pairwise
// in parallel rounds.  The result is the sorted sequence std::sort gives
// (elements that compare equal are indistinguishable for the keys used here:
// distinct determinants, or plain integers).
template <class T, class Cmp>
void parallel_sort(std::vector<T>& v, Cmp cmp) {
  const size_t n = v.size();
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  if (n < ((size_t)1 << 16) || hw < 2) {
    std::sort(v.begin(), v.end(), cmp);
    return;
  }
  unsigned nc = 1;
  while (nc * 2 <= std::min(hw, 64u)) nc *= 2;
  std::vector<size_t> bnd(nc + 1);
  for (unsigned i = 0; i <= nc; ++i) bnd[i] = n * i / nc;
  {
    std::vector<std::thread> th;
    for (unsigned i = 0; i < nc; ++i)
      th.emplace_back([&v, &bnd, cmp, i] { std::sort(v.begin() + bnd[i], v.begin() + bnd[i + 1], cmp); });
    for (std::thread& t : th) t.join();
  }
  std::vector<T> buf(n);
  std::vector<T>* src = &v;
  std::vector<T>* dst = &buf;
  for (unsigned w = 1; w < nc; w *= 2) {
    std::vector<std::thread> th;
    for (unsigned i = 0; i < nc; i += 2 * w)
      th.emplace_back([src, dst, &bnd, cmp, i, w] {
        std::merge(src->begin() + bnd[i], src->begin() + bnd[i + w], src->begin() + bnd[i + w],
                   src->begin() + bnd[i + 2 * w], dst->begin() + bnd[i], cmp);
      });
    for (std::thread& t : th) t.join();
    std::swap(src, dst);
  }
  if (src != &v) v.swap(*src);
}

// f(i0, i1) over [0, n) split into contiguous ranges, one per host thread
template <class F>
void parallel_ranges(int64_t n, F f) {
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const int64_t nt = std::min<int64_t>(std::min(hw, 64u), std::max<int64_t>(1, n >> 15));
  if (nt <= 1) {
    f((int64_t)0, n);
    return;
  }
  std::vector<std::thread> th;
  for (int64_t t = 0; t < nt; ++t) th.emplace_back([&f, n, nt, t] { f(n * t / nt, n * (t + 1) / nt); });
  for (std::thread& x : th) x.join();
}

}  // namespace qdkgb
