// tcgen05 building blocks of the tensor-core trailing updates (sm_103a):
// tile and k-chunk geometry, mbarriers with bounded waits, 2-D TMA loads,
// shared-memory matrix descriptors for K-major swizzled FP32 operands, the
// TF32 MMA with its instruction descriptor (M = 128, N = 256), commits and
// TMEM loads.  Used by the bulk update kernels (gemm_tc.cu) and by the
// diagonal-block kernel's own update (lu.cu).
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace bem {
namespace tc {

constexpr int BM = 128;
constexpr int BN = 256;
#define BEM_TC_BK 16
// k chunk: one swizzle atom of FP32, 128-byte swizzle for 32, 64-byte for
// 16, 32-byte for 8
constexpr int BK = BEM_TC_BK;
static_assert(BK == 32 || BK == 16 || BK == 8, "BK must be 8, 16 or 32");
constexpr int SW_BYTES = BK * 4;           // swizzle span (bytes per row)
constexpr int SW_SBO = 8 * SW_BYTES;       // 8-row group stride in shared memory
constexpr uint64_t SW_LAYOUT = BK == 32 ? 2 : (BK == 16 ? 4 : 6);  // descriptor: 128B / 64B / 32B swizzle
constexpr int A_BYTES = BM * BK * 4;  // 8 KB at BK = 16
constexpr int B_BYTES = BN * BK * 4;  // 16 KB at BK = 16
constexpr int STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;  // hi + lo

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}
// bounded wait for the given phase parity; false on timeout
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  uint32_t done = 0;
  for (int it = 0; it < (1 << 20); ++it) {
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y,
                                            uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          dst),
      "l"((uint64_t)map), "r"(x), "r"(y), "r"(bar)
      : "memory");
}

// shared-memory matrix descriptor: K-major, swizzled rows of SW_BYTES, 8-row
// groups SW_SBO bytes apart (SBO), leading offset unused for this layout (1).
__device__ __forceinline__ uint64_t sdesc(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFF) >> 4);
  d |= (uint64_t)1 << 16;
  d |= (uint64_t)(SW_SBO >> 4) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version for tcgen05
  d |= SW_LAYOUT << 61;
  return d;
}

// instruction descriptor: D f32, A/B tf32, both K-major, M=128, N=256
constexpr uint32_t IDESC = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(BN >> 3) << 17) |
                           ((uint32_t)(BM >> 4) << 24);

__device__ __forceinline__ void mma_tf32(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t accum,
                                         uint32_t idesc = IDESC) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(
          dtmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accum)
      : "memory");
}
// the same with N = 128
constexpr uint32_t IDESC_N128 = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(128 >> 3) << 17) |
                                ((uint32_t)(BM >> 4) << 24);

__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
               : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t* v) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, "
      "%12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, "
      "%30, %31}, [%32];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
        "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
        "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]),
        "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]),
        "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

}  // namespace tc
}  // namespace bem
