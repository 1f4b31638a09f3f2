// Sloan profile / wavefront reduction of the connect graph: the renumbering
// TPZAnalysis::OptimizeBandwidth applies before assembling
// (Analysis/TPZAnalysis.cpp:228-300 with RENUMBER = TPZSloanRenumbering,
// External/TPZSloanRenumbering.cpp:23-175).
//
// The algorithm is one sequential greedy front, so it runs on the host.  It
// gives the reference's permutation exactly -- the same node graph
// (TPZRenumbering::ConvertGraph: sorted neighbours, self removed), the same
// pseudo-peripheral pair (TPZCutHillMcKee::SGraph::PseudoPeripheralNodes,
// External/TPZCutHillMcKee.cpp:165-260) and the same tie-breaks -- but the
// queue's "first node of highest priority" (FindHighestPriority, a scan of the
// whole queue per numbered node) is a leftmost-maximum query on a segment tree
// over the queue's slots, O(log n) instead of O(queue length), and the level
// structures use one visited array instead of a fresh history per level.
#include <algorithm>
#include <climits>
#include <cstdint>
#include <map>
#include <thread>
#include <vector>

#include "../../include/gpz.h"

#include "gpz_graph.h"

namespace {

using gpz_graph::Graph;
using gpz_graph::convert_graph;

// TPZCutHillMcKee::SGraph::RootedLevelStructure (External/TPZCutHillMcKee.cpp:93-119):
// levels in breadth-first order, each level's nodes in the order their first
// parent (in the previous level's order) lists them
void rooted_levels(const Graph &g, int64_t root, std::vector<int64_t> &order, std::vector<int64_t> &lstart,
                   std::vector<char> &seen) {
  order.clear();
  lstart.clear();
  std::fill(seen.begin(), seen.end(), 0);
  order.push_back(root);
  seen[root] = 1;
  int64_t b = 0;
  while (b < (int64_t)order.size()) {
    lstart.push_back(b);
    const int64_t e = (int64_t)order.size();
    for (int64_t i = b; i < e; i++) {
      const int64_t v = order[i];
      for (int64_t k = g.ptr[v]; k < g.ptr[v + 1]; k++)
        if (!seen[g.adj[k]]) {
          seen[g.adj[k]] = 1;
          order.push_back(g.adj[k]);
        }
    }
    b = e;
  }
  lstart.push_back((int64_t)order.size());
}

// TPZCutHillMcKee::SGraph::PseudoPeripheralNodes (External/TPZCutHillMcKee.cpp:165-260)
// with SmallestDegree, SortNodes and ShrinkLastLevel (:16-30, :121-163)
void pseudo_peripheral(const Graph &g, int64_t &start, int64_t &end) {
  int64_t mindeg = 1000000;
  start = -1;
  for (int64_t v = 0; v < g.n; v++)
    if (g.degree(v) < mindeg) {
      mindeg = g.degree(v);
      start = v;
    }
  end = -1;
  std::vector<char> seen(g.n);
  std::vector<int64_t> order, lstart, lorder, llstart;
  rooted_levels(g, start, order, lstart, seen);
  for (int count = 0; count < 10 || end == -1;) {
    count++;
    const int64_t s0 = start, e0 = end;
    const int64_t nlev = (int64_t)lstart.size() - 1;
    if (nlev == 0) break;
    std::vector<int64_t> last(order.begin() + lstart[nlev - 1], order.begin() + lstart[nlev]);
    const int64_t norig = (int64_t)last.size();
    std::stable_sort(last.begin(), last.end(), [&](int64_t a, int64_t b) { return g.degree(a) < g.degree(b); });
    std::map<int64_t, int64_t> bydeg;  // one node per degree: the last one of that degree
    for (int64_t v : last) bydeg[g.degree(v)] = v;
    last.clear();
    for (auto &kv : bydeg) last.push_back(kv.second);
    const int64_t keep = (norig + 2) / 2;
    if (keep < (int64_t)last.size()) last.resize(keep);
    int64_t we = 1000000000L;
    const int64_t hs = nlev;
    for (int64_t q : last) {
      rooted_levels(g, q, lorder, llstart, seen);
      const int64_t h = (int64_t)llstart.size() - 1;
      int64_t w = 0;
      for (int64_t j = 0; j < h; j++) w = std::max(w, llstart[j + 1] - llstart[j]);
      if (h > hs && w < we) {
        start = q;
        order.swap(lorder);
        lstart.swap(llstart);
        break;
      } else if (w < we) {
        end = q;
        we = w;
      }
    }
    if (s0 == start && e0 == end) break;
  }
}

// leftmost maximum over the queue's slots (empty slots hold INT64_MIN)
struct LeftMax {
  int64_t size = 1;
  std::vector<int64_t> val;
  std::vector<int64_t> arg;
  explicit LeftMax(int64_t n) {
    while (size < std::max<int64_t>(n, 1)) size <<= 1;
    val.assign(2 * size, INT64_MIN);
    arg.assign(2 * size, 0);
    for (int64_t i = 0; i < size; i++) arg[size + i] = i;
    for (int64_t i = size - 1; i >= 1; i--) pull(i);
  }
  void pull(int64_t i) {
    const int64_t l = 2 * i, r = 2 * i + 1;
    if (val[r] > val[l]) {  // strictly greater: ties keep the left slot
      val[i] = val[r];
      arg[i] = arg[r];
    } else {
      val[i] = val[l];
      arg[i] = arg[l];
    }
  }
  // an increase of one slot's value: walk up only while this slot wins
  void raise(int64_t slot, int64_t v) {
    int64_t i = size + slot;
    val[i] = v;
    for (i >>= 1; i >= 1; i >>= 1) {
      if (arg[i] == slot || v > val[i] || (v == val[i] && slot < arg[i])) {
        val[i] = v;
        arg[i] = slot;
      } else {
        break;  // this subtree's winner is unchanged, so is everything above it
      }
    }
  }
  void set(int64_t slot, int64_t v) {
    int64_t i = size + slot;
    val[i] = v;
    for (i >>= 1; i >= 1; i >>= 1) pull(i);
  }
};

}  // namespace

extern "C" int gpz_sloan_resequence(int64_t nnodes, int64_t nel, const int64_t *elgraphindex, const int64_t *elgraph,
                                    int64_t *perm_gather, int64_t *perm_scatter) {
  if (nnodes < 0 || nel < 0 || (nel > 0 && !elgraphindex) || !perm_gather || !perm_scatter) return GPZ_E_INVALID;
  if (nnodes == 0) return GPZ_OK;  // TPZAnalysis::OptimizeBandwidth returns when there are no connects
  if (nel > 0 && elgraphindex[0] < 0) return GPZ_E_INVALID;
  for (int64_t e = 0; e < nel; e++)
    if (elgraphindex[e + 1] < elgraphindex[e]) return GPZ_E_INVALID;
  if (nel > 0 && elgraphindex[nel] > 0 && !elgraph) return GPZ_E_INVALID;
  try {
    Graph g;
    if (!convert_graph(nnodes, nel, elgraphindex, elgraph, g)) return GPZ_E_INVALID;
    int64_t start, end;
    pseudo_peripheral(g, start, end);
    if (start < 0 || end < 0) return GPZ_E_INVALID;
    // distances to the end node (TPZSloanRenumbering.cpp:51-62)
    std::vector<int64_t> order, lstart, dist(nnodes, -1);
    std::vector<char> seen(nnodes);
    rooted_levels(g, end, order, lstart, seen);
    for (int64_t l = 0; l + 1 < (int64_t)lstart.size(); l++)
      for (int64_t i = lstart[l]; i < lstart[l + 1]; i++) dist[order[i]] = l;
    for (int64_t v = 0; v < nnodes; v++)
      if (dist[v] < 0) return GPZ_E_INVALID;  // more than one connected component
    const int64_t W1 = 1, W2 = 2;
    std::vector<int64_t> prio(nnodes);
    for (int64_t v = 0; v < nnodes; v++) prio[v] = W1 * dist[v] - W2 * (g.degree(v) + 1);
    enum : char { kInactive = 0, kPreActive = 1, kActive = 2, kPostActive = 3 };
    std::vector<char> status(nnodes, kInactive), hist(nnodes, 0);
    std::vector<int64_t> slot_node(nnodes), slot_of(nnodes, -1);
    int64_t qsize = 0, numbered = 0;
    LeftMax tree(nnodes);
    auto push = [&](int64_t v) {  // SList::push_back: a node enters the queue once ever
      if (hist[v]) return false;
      hist[v] = 1;
      slot_node[qsize] = v;
      slot_of[v] = qsize;
      tree.raise(qsize, prio[v]);  // from the empty value
      qsize++;
      return true;
    };
    auto bump = [&](int64_t v, int64_t by) {
      prio[v] += by;
      if (slot_of[v] >= 0) tree.raise(slot_of[v], prio[v]);  // priorities only grow
    };
    status[start] = kPreActive;
    push(start);
    while (qsize) {
      const int64_t slot = tree.arg[1];
      const int64_t cur = slot_node[slot];
      // SList::remove: the last slot's node moves into the freed slot
      const int64_t lastn = slot_node[qsize - 1];
      qsize--;
      slot_of[cur] = -1;
      if (slot != qsize) {
        slot_node[slot] = lastn;
        slot_of[lastn] = slot;
        tree.set(slot, prio[lastn]);
      }
      tree.set(qsize, INT64_MIN);
      if (status[cur] == kPreActive) {
        for (int64_t k = g.ptr[cur]; k < g.ptr[cur + 1]; k++) {
          const int64_t a = g.adj[k];
          bump(a, W2);
          if (push(a) && status[a] == kInactive) status[a] = kPreActive;
        }
      }
      perm_scatter[numbered++] = cur;
      status[cur] = kPostActive;
      for (int64_t k = g.ptr[cur]; k < g.ptr[cur + 1]; k++) {
        const int64_t a = g.adj[k];
        if (status[a] != kPreActive) continue;
        status[a] = kActive;
        bump(a, W2);
        for (int64_t j = g.ptr[a]; j < g.ptr[a + 1]; j++) {
          const int64_t q = g.adj[j];
          if (status[q] != kPostActive) bump(q, W2);
          if (push(q) && status[q] == kInactive) status[q] = kPreActive;
        }
      }
    }
    if (numbered != nnodes) return GPZ_E_INVALID;
    for (int64_t i = 0; i < nnodes; i++) perm_gather[perm_scatter[i]] = i;
  } catch (...) {
    return GPZ_E_NOMEM;
  }
  return GPZ_OK;
}
