// Connect graph shared by the host-side graph algorithms (Sloan renumbering,
// node-set blocks): TPZRenumbering::ConvertGraph of the element graph that
// TPZCompMesh::ComputeElGraph lists (Mesh/pzcmesh.cpp:1214-1262).
#pragma once
#include <algorithm>
#include <cstdint>
#include <exception>
#include <thread>
#include <vector>

namespace gpz_graph {

struct Graph {
  int64_t n = 0;
  std::vector<int64_t> ptr, adj;  // sorted neighbours of each node, self excluded
  int64_t degree(int64_t v) const { return ptr[v + 1] - ptr[v]; }
};

// TPZRenumbering::ConvertGraph (External/TPZRenumbering.cpp:76-105): every
// node's list is built on its own (a count pass and a fill pass over node
// ranges on the host threads), so the result does not depend on the threads.
// Allocation failures throw std::bad_alloc into the caller's thread.
inline bool convert_graph(int64_t nnodes, int64_t nel, const int64_t *eptr, const int64_t *eg, Graph &g) {
  std::vector<int64_t> cnt(nnodes + 1, 0);
  for (int64_t e = 0; e < nel; e++)
    for (int64_t k = eptr[e]; k < eptr[e + 1]; k++) {
      if (eg[k] < 0 || eg[k] >= nnodes) return false;
      cnt[eg[k] + 1]++;
    }
  for (int64_t i = 0; i < nnodes; i++) cnt[i + 1] += cnt[i];
  std::vector<int64_t> n2e(cnt[nnodes]), fill(cnt.begin(), cnt.end() - 1);
  for (int64_t e = 0; e < nel; e++)
    for (int64_t k = eptr[e]; k < eptr[e + 1]; k++) n2e[fill[eg[k]]++] = e;
  g.n = nnodes;
  g.ptr.assign(nnodes + 1, 0);
  unsigned nt = std::thread::hardware_concurrency();
  nt = std::max(1u, std::min(nt, 16u));
  if (nnodes < 65536) nt = 1;
  // one node's neighbours (self removed), unsorted, with a per-thread marker
  auto neighbours = [&](int64_t v, std::vector<int64_t> &mark, std::vector<int64_t> &nb) {
    nb.clear();
    mark[v] = v;
    for (int64_t k = cnt[v]; k < cnt[v + 1]; k++) {
      const int64_t e = n2e[k];
      for (int64_t j = eptr[e]; j < eptr[e + 1]; j++)
        if (mark[eg[j]] != v) {
          mark[eg[j]] = v;
          nb.push_back(eg[j]);
        }
    }
  };
  // the per-thread markers are allocated here, in the calling thread, so an
  // allocation failure reaches the caller's handler; anything a worker still
  // throws (its neighbour list growing) is carried out and rethrown after join
  std::vector<std::vector<int64_t>> marks(nt, std::vector<int64_t>(nnodes, -1));
  auto run = [&](auto &&body) {
    for (auto &m : marks) std::fill(m.begin(), m.end(), -1);
    std::vector<std::exception_ptr> err(nt);
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nt; t++)
      th.emplace_back([&, t]() {
        try {
          std::vector<int64_t> nb;
          const int64_t b = nnodes * t / nt, e = nnodes * (t + 1) / nt;
          for (int64_t v = b; v < e; v++) body(v, marks[t], nb);
        } catch (...) {
          err[t] = std::current_exception();
        }
      });
    for (auto &x : th) x.join();
    for (auto &x : err)
      if (x) std::rethrow_exception(x);
  };
  run([&](int64_t v, std::vector<int64_t> &mark, std::vector<int64_t> &nb) {
    neighbours(v, mark, nb);
    g.ptr[v + 1] = (int64_t)nb.size();
  });
  for (int64_t v = 0; v < nnodes; v++) g.ptr[v + 1] += g.ptr[v];
  g.adj.assign(g.ptr[nnodes], 0);
  run([&](int64_t v, std::vector<int64_t> &mark, std::vector<int64_t> &nb) {
    neighbours(v, mark, nb);
    std::sort(nb.begin(), nb.end());
    std::copy(nb.begin(), nb.end(), g.adj.begin() + g.ptr[v]);
  });
  return true;
}

}  // namespace gpz_graph
