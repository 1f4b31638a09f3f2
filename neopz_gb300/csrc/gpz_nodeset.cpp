// Node-set blocks of the block-Jacobi preconditioner that
// TPZAnalysis::BuildPreconditioner(EBlockJacobi, overlap = false) builds
// (Analysis/TPZAnalysis.cpp:1008-1085): TPZNodesetCompute::AnalyseGraph,
// BuildNodeGraph, ExpandGraph and ColorGraph (External/tpznodesetcompute.cpp:
// 47-209, 528-607) over the connect graph of TPZRenumbering::ConvertGraph.
//
// A connect's "node set" is its closed neighbourhood in the connect graph (the
// connects it shares an element with, itself included).  Connects are visited
// in increasing order; before a connect is numbered, every neighbour whose set
// is a proper subset of its own is numbered first (depth first, neighbours in
// increasing order), its level is one more than the largest level of those
// subsets, and the neighbours with an identical set join its block.  Blocks are
// the sequence numbers in order, each listing its connects in increasing order,
// then expanded to equations through the connects' block positions and sizes
// (empty blocks dropped), then coloured so that no two blocks of one colour
// share an equation.
//
// The reference tests every inclusion on std::set copies of the neighbourhoods
// while it recurses.  Here the relation of each connect to each of its
// neighbours (proper subset, identical, neither) is one byte beside the
// adjacency entry, computed for all connects at once on the host threads (a
// marker array per thread, a size test first, the subset walk stopping at the
// first foreign connect); the numbering pass then only follows the marked
// entries.  Neither the relation nor the visiting order depends on the threads,
// so the blocks, levels and sequence numbers are the reference's.
#include <algorithm>
#include <cstdint>
#include <thread>
#include <vector>

#include "../../include/gpz.h"
#include "gpz_graph.h"

namespace {

using gpz_graph::Graph;

enum : char { kNone = 0, kSubset = 1, kEqual = 2 };

// rel[k] for the adjacency entry k = (v, o): kSubset when the closed
// neighbourhood of o is a proper subset of v's, kEqual when they are equal
void relations(const Graph &g, std::vector<char> &rel) {
  const int64_t n = g.n;
  rel.assign(g.adj.size(), kNone);
  unsigned nt = std::thread::hardware_concurrency();
  nt = std::max(1u, std::min(nt, 16u));
  if (n < 65536) nt = 1;
  // markers allocated in the calling thread: an allocation failure reaches the caller's handler
  std::vector<std::vector<int64_t>> marks(nt, std::vector<int64_t>(n, -1));
  std::vector<std::thread> th;
  for (unsigned t = 0; t < nt; t++)
    th.emplace_back([&, t]() {
      std::vector<int64_t> &mark = marks[t];
      const int64_t b = n * t / nt, e = n * (t + 1) / nt;
      for (int64_t v = b; v < e; v++) {
        mark[v] = v;
        for (int64_t k = g.ptr[v]; k < g.ptr[v + 1]; k++) mark[g.adj[k]] = v;
        const int64_t dv = g.degree(v);
        for (int64_t k = g.ptr[v]; k < g.ptr[v + 1]; k++) {
          const int64_t o = g.adj[k];
          const int64_t dn = g.degree(o);
          if (dn > dv) continue;  // a larger set is neither contained nor equal
          bool inside = true;     // o itself is in v's set: it is v's neighbour
          for (int64_t j = g.ptr[o]; j < g.ptr[o + 1] && inside; j++) inside = mark[g.adj[j]] == v;
          if (inside) rel[k] = dn < dv ? kSubset : kEqual;
        }
      }
    });
  for (auto &x : th) x.join();
}

struct Analysis {
  const Graph &g;
  const std::vector<char> &rel;
  std::vector<int64_t> seq;
  std::vector<int> level;
  std::vector<int64_t> card;  // fSeqCard: connects per sequence number
  bool ok = true;

  Analysis(const Graph &graph, const std::vector<char> &r)
      : g(graph), rel(r), seq(graph.n, -1), level(graph.n, 0) {}

  // TPZNodesetCompute::AnalyseNode (External/tpznodesetcompute.cpp:77-188).
  // Depth is bounded by the largest neighbourhood: each call goes to a
  // strictly smaller set.
  void analyse(int64_t v) {
    if (seq[v] != -1) return;
    int minlevel = 0;
    for (int64_t k = g.ptr[v]; k < g.ptr[v + 1]; k++) {
      const int64_t o = g.adj[k];
      if (rel[k] == kSubset) {
        analyse(o);
        minlevel = std::max(minlevel, level[o] + 1);
      } else if (rel[k] == kEqual && seq[o] != -1) {
        ok = false;  // the reference's DebugStop: an identical set numbered apart
      }
    }
    const int64_t s = (int64_t)card.size();
    card.push_back(1);
    seq[v] = s;
    level[v] = minlevel;
    for (int64_t k = g.ptr[v]; k < g.ptr[v + 1]; k++)
      if (rel[k] == kEqual) {
        seq[g.adj[k]] = s;
        level[g.adj[k]] = minlevel;
        card[s]++;
      }
  }
};

}  // namespace

extern "C" int gpz_nodeset_blocks(int64_t nnodes, int64_t nel, const int64_t *elgraphindex, const int64_t *elgraph,
                                  const int64_t *block_position, const int64_t *block_size, int64_t neq,
                                  int64_t *blockindex, int64_t *blockeqs, int64_t *nblocks, int *colors,
                                  int *ncolors, int64_t *seqnum, int *level) {
  if (nnodes < 0 || nel < 0 || neq < 0 || !nblocks || (nel && (!elgraphindex || !elgraph)) ||
      (nnodes && (!block_position || !block_size || !blockindex || !blockeqs)))
    return GPZ_E_INVALID;
  for (int64_t e = 0; e < nel; e++)
    if (elgraphindex[e] < 0 || elgraphindex[e + 1] < elgraphindex[e]) return GPZ_E_INVALID;
  for (int64_t v = 0; v < nnodes; v++)
    if (block_size[v] < 0 || block_position[v] < 0 || block_position[v] + block_size[v] > neq) return GPZ_E_INVALID;
  if (nnodes == 0) {  // no blocks; ColorGraph still reports one colour
    *nblocks = 0;
    if (ncolors) *ncolors = 1;
    return GPZ_OK;
  }
  try {
    Graph g;
    if (!gpz_graph::convert_graph(nnodes, nel, elgraphindex, elgraph, g)) return GPZ_E_INVALID;
    std::vector<char> rel;
    relations(g, rel);
    Analysis an(g, rel);
    for (int64_t v = 0; v < nnodes; v++) an.analyse(v);  // AnalyseGraph (:47-71)
    if (!an.ok) return GPZ_E_INVALID;
    // BuildNodeGraph (:190-209): the connects of each sequence number, increasing
    const int64_t nseq = (int64_t)an.card.size();
    std::vector<int64_t> bptr(nseq + 1, 0), bnode(nnodes);
    for (int64_t s = 0; s < nseq; s++) bptr[s + 1] = bptr[s] + an.card[s];
    {
      std::vector<int64_t> fill(bptr.begin(), bptr.end() - 1);
      for (int64_t v = 0; v < nnodes; v++) bnode[fill[an.seq[v]]++] = v;
    }
    // ExpandGraph (:528-562): equations of each block; blocks without any dropped
    int64_t cnt = 0, nb = 0;
    blockindex[0] = 0;
    for (int64_t s = 0; s < nseq; s++) {
      for (int64_t k = bptr[s]; k < bptr[s + 1]; k++) {
        const int64_t v = bnode[k];
        for (int64_t b = 0; b < block_size[v]; b++) blockeqs[cnt++] = block_position[v] + b;
      }
      if (blockindex[nb] != cnt) blockindex[++nb] = cnt;
    }
    *nblocks = nb;
    // ColorGraph (:567-607): greedy colours, a block taking the current colour
    // when none of its equations already has it
    if (colors || ncolors) {
      std::vector<int> col(nb, -1), eqcolor(neq, -1);
      int color = 0;
      bool uncolored = true;
      while (uncolored) {
        uncolored = false;
        std::fill(eqcolor.begin(), eqcolor.end(), -1);
        for (int64_t b = 0; b < nb; b++) {
          if (col[b] != -1) continue;
          bool clash = false;
          for (int64_t k = blockindex[b]; k < blockindex[b + 1] && !clash; k++) clash = eqcolor[blockeqs[k]] == color;
          if (clash) {
            uncolored = true;
          } else {
            col[b] = color;
            for (int64_t k = blockindex[b]; k < blockindex[b + 1]; k++) eqcolor[blockeqs[k]] = color;
          }
        }
        color++;
      }
      if (colors) std::copy(col.begin(), col.end(), colors);
      if (ncolors) *ncolors = color;
    }
    if (seqnum) std::copy(an.seq.begin(), an.seq.end(), seqnum);
    if (level) std::copy(an.level.begin(), an.level.end(), level);
  } catch (...) {
    return GPZ_E_NOMEM;
  }
  return GPZ_OK;
}
