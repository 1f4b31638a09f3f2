// tcgen05 helpers shared by the tensor-core kernels (sm_103a): shared-memory
// operand descriptors of the K-major no-swizzle layout, the TF32 hi / lo split,
// the MMA issue and commit, bounded mbarrier waits and TMEM loads.
//
// Operand layout: 8-row x 16-byte core matrices, K direction fastest inside a
// row of core matrices (LBO 128 B between core matrices along K, SBO = K/4 x
// 128 B between 8-row groups).  kmaj(r, k, K) is the byte offset of element
// (r, k) of an operand with K columns (K a multiple of 4).
#pragma once
#include <stdint.h>

namespace gpz {
namespace {

constexpr int kTcWaitTries = 1 << 22;

__device__ __forceinline__ uint32_t tc_smem(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
__host__ __device__ __forceinline__ uint32_t kmaj(int r, int k, int kcols) {
  return ((uint32_t)(r >> 3) * (uint32_t)(kcols >> 2) + (uint32_t)(k >> 2)) * 128u + (uint32_t)(r & 7) * 16u +
         (uint32_t)(k & 3) * 4u;
}
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t sbo) {
  return (uint64_t)((saddr >> 4) & 0x3FFF) | ((uint64_t)((128u >> 4) & 0x3FFF) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | ((uint64_t)1 << 46);
}
__device__ __forceinline__ float tf32_rna(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}
__device__ __forceinline__ void st_split(unsigned char *hi, unsigned char *lo, uint32_t off, float v) {
  const float h = tf32_rna(v);
  *(float *)(hi + off) = h;
  *(float *)(lo + off) = tf32_rna(v - h);
}
__device__ __forceinline__ void tc_mma(uint32_t tm, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile("{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\ntcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tm),
               "l"(a), "l"(b), "r"(idesc), "r"(acc));
}
__device__ __forceinline__ void tc_commit(uint64_t *mb) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(tc_smem(mb)));
}
// non-blocking test of an mbarrier phase: the waits below poll it with a short
// sleep instead of the potentially-suspending try_wait, so a waiting thread is
// never parked for a system-dependent time after the phase has completed
__device__ __forceinline__ bool mb_test(uint64_t *mb, uint32_t parity) {
  uint32_t done;
  asm volatile("{\n.reg .pred p;\nmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
               : "=r"(done)
               : "r"(tc_smem(mb)), "r"(parity)
               : "memory");
  return done != 0;
}
// bounded wait (kTcWaitTries polls of at most ~0.1 us apart)
__device__ __forceinline__ bool tc_wait(uint64_t *mb, uint32_t parity) {
  for (int it = 0; it < kTcWaitTries; it++) {
    if (mb_test(mb, parity)) return true;
    if (it > 16) __nanosleep(64);
  }
  return false;
}
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float *v) {
  uint32_t r[16];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                 "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
               : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
  for (int j = 0; j < 16; j++) v[j] = __uint_as_float(r[j]);
}

}  // namespace
}  // namespace gpz
