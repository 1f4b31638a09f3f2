// Exclusive prefix sums on the device (int64), used by the pattern builder.
#include "gpz_internal.h"

namespace gpz {

namespace {
constexpr int kScanThreads = 512;
constexpr int kScanTile = 2 * kScanThreads;

// Block-local exclusive scan of a tile of kScanTile values (Blelloch up/down sweep).
__global__ void k_scan_tiles(const int64_t *__restrict__ in, int64_t *__restrict__ out, int64_t *__restrict__ sums,
                             int64_t n) {
  __shared__ int64_t s[kScanTile];
  int64_t base = (int64_t)blockIdx.x * kScanTile;
  int t = threadIdx.x;
  int64_t i0 = base + 2 * t, i1 = base + 2 * t + 1;
  s[2 * t] = i0 < n ? in[i0] : 0;
  s[2 * t + 1] = i1 < n ? in[i1] : 0;
  int off = 1;
  for (int d = kScanTile >> 1; d > 0; d >>= 1) {
    __syncthreads();
    if (t < d) {
      int ai = off * (2 * t + 1) - 1, bi = off * (2 * t + 2) - 1;
      s[bi] += s[ai];
    }
    off <<= 1;
  }
  if (t == 0) {
    if (sums) sums[blockIdx.x] = s[kScanTile - 1];
    s[kScanTile - 1] = 0;
  }
  for (int d = 1; d < kScanTile; d <<= 1) {
    off >>= 1;
    __syncthreads();
    if (t < d) {
      int ai = off * (2 * t + 1) - 1, bi = off * (2 * t + 2) - 1;
      int64_t v = s[ai];
      s[ai] = s[bi];
      s[bi] += v;
    }
  }
  __syncthreads();
  if (i0 < n) out[i0] = s[2 * t];
  if (i1 < n) out[i1] = s[2 * t + 1];
}

__global__ void k_add_tile_offsets(int64_t *__restrict__ out, const int64_t *__restrict__ offs, int64_t n) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] += offs[i / kScanTile];
}
}  // namespace

void exclusive_scan_i64(const int64_t *in, int64_t *out, int64_t n, cudaStream_t s, Ctx &c) {
  if (n <= 0) return;
  int64_t ntiles = (n + kScanTile - 1) / kScanTile;
  if (ntiles == 1) {
    k_scan_tiles<<<1, kScanThreads, 0, s>>>(in, out, nullptr, n);
    c.launches++;
    GPZ_CUDA_TRY(cudaGetLastError());
    return;
  }
  DBuf<int64_t> sums, sums_scan;
  sums.alloc(ntiles);
  sums_scan.alloc(ntiles);
  k_scan_tiles<<<(unsigned)ntiles, kScanThreads, 0, s>>>(in, out, sums.p, n);
  c.launches++;
  GPZ_CUDA_TRY(cudaGetLastError());
  exclusive_scan_i64(sums.p, sums_scan.p, ntiles, s, c);
  k_add_tile_offsets<<<grid_for(n, 256), 256, 0, s>>>(out, sums_scan.p, n);
  c.launches++;
  GPZ_CUDA_TRY(cudaGetLastError());
  // the temporaries are freed when this returns: order the stream first
  GPZ_CUDA_TRY(cudaStreamSynchronize(s));
}

void check_device_flag(Ctx &c, const char *where) {
  int h = 0;
  GPZ_CUDA_TRY(cudaMemcpyAsync(&h, c.d_err.p, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
  GPZ_CUDA_TRY(cudaStreamSynchronize(c.stream));
  if (h) {
    int z = 0;
    cudaMemcpy(c.d_err.p, &z, sizeof(int), cudaMemcpyHostToDevice);
    throw Error{GPZ_E_DEVICE_CHECK, std::string("device-side check failed in ") + where + " (code " +
                                        std::to_string(h) + ")"};
  }
}

}  // namespace gpz
