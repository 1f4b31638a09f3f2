// Element colouring of the atomic-free scatter (gpz_element_colours): greedy
// first fit over the elements in order, an element taking the smallest colour
// that no earlier element sharing one of its non-empty connects holds -- the
// idea of TPZStructMatrix::ComputeElementColors (StrMatrix/TPZStructMatrix.cpp:
// 104-161), over the element graph of TPZCompMesh::ComputeElGraph.  Elements
// of one colour share no connect, hence write disjoint rows and CSR slots, so
// one launch per colour needs no atomics.  Host code; gpz_mesh_upload colours
// its buckets with it.
#include <cstdint>
#include <vector>

#include "../../include/gpz.h"

extern "C" int gpz_element_colours(int64_t nel, const int64_t *elgraphindex, const int64_t *elgraph,
                                   int64_t nconnects, const int64_t *block_size, int32_t *colours,
                                   int32_t *ncolours) {
  if (nel < 0 || nconnects < 0 || !ncolours || (nel > 0 && (!elgraphindex || !elgraph || !colours)) ||
      (nconnects > 0 && !block_size))
    return GPZ_E_INVALID;
  try {
    std::vector<uint64_t> used(nconnects, 0);
    int ncol = 0;
    for (int64_t e = 0; e < nel; e++) {
      const int64_t k0 = elgraphindex[e], k1 = elgraphindex[e + 1];
      if (k0 < 0 || k1 < k0) return GPZ_E_INVALID;
      uint64_t mask = 0;
      for (int64_t k = k0; k < k1; k++) {
        const int64_t cn = elgraph[k];
        if (cn < 0 || cn >= nconnects) return GPZ_E_INVALID;
        if (block_size[cn] > 0) mask |= used[cn];
      }
      if (~mask == 0) return GPZ_E_INVALID;  // more than 64 colours
      const int col = __builtin_ctzll(~mask);
      colours[e] = col;
      if (col + 1 > ncol) ncol = col + 1;
      for (int64_t k = k0; k < k1; k++)
        if (block_size[elgraph[k]] > 0) used[elgraph[k]] |= (1ull << col);
    }
    *ncolours = ncol;
    return GPZ_OK;
  } catch (...) {
    return GPZ_E_NOMEM;
  }
}
