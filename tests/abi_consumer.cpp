// A C++ program that uses the library through include/gpz.h alone, as the
// reference's C++ host code would: the host-only entry points on a
// three-connect chain (connects 0-1 and 1-2 share an element), then a context
// on device 0, which reports GPZ_E_NO_DEVICE on a machine without a GPU.
#include <cstdio>
#include <vector>

#include "gpz.h"

int main() {
  std::vector<int64_t> elgraphindex{0, 2, 4}, elgraph{0, 1, 1, 2}, pos{0, 1, 2}, size{1, 1, 1};
  std::vector<int64_t> blockindex(4), blockeqs(3), seq(3), gather(3), scatter(3);
  std::vector<int> colors(3), level(3);
  int64_t nblocks = 0;
  int ncolors = 0;
  int rc = gpz_nodeset_blocks(3, 2, elgraphindex.data(), elgraph.data(), pos.data(), size.data(), 3,
                              blockindex.data(), blockeqs.data(), &nblocks, colors.data(), &ncolors, seq.data(),
                              level.data());
  std::printf("nodeset %d %lld %d %lld %lld %lld\n", rc, (long long)nblocks, ncolors, (long long)blockeqs[0],
              (long long)blockeqs[1], (long long)blockeqs[2]);
  rc = gpz_sloan_resequence(3, 2, elgraphindex.data(), elgraph.data(), gather.data(), scatter.data());
  std::printf("sloan %d %lld %lld %lld\n", rc, (long long)scatter[0], (long long)scatter[1], (long long)scatter[2]);
  gpz_ctx *ctx = nullptr;
  rc = gpz_ctx_create(&ctx, 0);
  std::printf("context %d\n", rc);
  if (rc == GPZ_OK) gpz_ctx_destroy(ctx);
  return 0;
}
