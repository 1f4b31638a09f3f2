// Element colouring of the atomic-free scatter (gpz_element_colours): greedy
// first fit over the elements in order, an element taking the smallest colour
// that no earlier element sharing one of its non-empty connects holds -- the
// idea of TPZStructMatrix::ComputeElementColors (StrMatrix/TPZStructMatrix.cpp:
// 104-161), over the element graph of TPZCompMesh::ComputeElGraph.  Elements
// of one colour share no connect, hence write disjoint rows and CSR slots, so
// one launch per colour needs no atomics.  Host code; gpz_mesh_upload colours
// its buckets with the same loop, reading the connects of its descriptor.
#include <cstdint>
#include <vector>

#include "gpz_internal.h"

namespace gpz {
namespace {

// connects(e, f): calls f(cn) for each connect of element e (false: a connect out of range)
template <class Connects>
int greedy_colours(int64_t nel, int64_t nconnects, Connects &&connects, const int64_t *bsz64, const int32_t *bsz32,
                   int32_t *colours, int32_t *ncolours) {
  std::vector<uint64_t> used(nconnects, 0);
  auto nonempty = [&](int64_t cn) { return bsz64 ? bsz64[cn] > 0 : bsz32[cn] > 0; };
  int ncol = 0;
  for (int64_t e = 0; e < nel; e++) {
    uint64_t mask = 0;
    bool ok = connects(e, [&](int64_t cn) {
      if (cn < 0 || cn >= nconnects) return false;
      if (nonempty(cn)) mask |= used[cn];
      return true;
    });
    if (!ok) return GPZ_E_INVALID;
    if (~mask == 0) return GPZ_E_INVALID;  // more than 64 colours
    const int col = __builtin_ctzll(~mask);
    colours[e] = col;
    if (col + 1 > ncol) ncol = col + 1;
    connects(e, [&](int64_t cn) {
      if (nonempty(cn)) used[cn] |= (1ull << col);
      return true;
    });
  }
  *ncolours = ncol;
  return GPZ_OK;
}

}  // namespace

int colour_mesh_elements(const gpz_mesh_desc &d, const int *nsides_of_type, int32_t *colours, int32_t *ncolours) {
  return greedy_colours(
      d.nel, d.nconnects,
      [&](int64_t e, auto &&f) {
        const int64_t *cn = d.el_conn + e * 27;
        const int ns = nsides_of_type[d.el_type[e]];
        for (int s = 0; s < ns; s++)
          if (!f(cn[s])) return false;
        return true;
      },
      nullptr, d.block_size, colours, ncolours);
}

}  // namespace gpz

extern "C" int gpz_element_colours(int64_t nel, const int64_t *elgraphindex, const int64_t *elgraph,
                                   int64_t nconnects, const int64_t *block_size, int32_t *colours,
                                   int32_t *ncolours) {
  if (nel < 0 || nconnects < 0 || !ncolours || (nel > 0 && (!elgraphindex || !elgraph || !colours)) ||
      (nconnects > 0 && !block_size))
    return GPZ_E_INVALID;
  try {
    return gpz::greedy_colours(
        nel, nconnects,
        [&](int64_t e, auto &&f) {
          const int64_t k0 = elgraphindex[e], k1 = elgraphindex[e + 1];
          if (k0 < 0 || k1 < k0) return false;
          for (int64_t k = k0; k < k1; k++)
            if (!f(elgraph[k])) return false;
          return true;
        },
        block_size, nullptr, colours, ncolours);
  } catch (...) {
    return GPZ_E_NOMEM;
  }
}
