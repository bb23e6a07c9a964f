// Trailing-update GEMM of the blocked LU on the 5th-generation tensor cores
// (sm_103a): C (M x N) = beta C + alpha A (M x 128) B (128 x N) in FP32 with
// the 3xTF32 split  A B ~ A_hi B_hi + A_hi B_lo + A_lo B_hi.
//
// One CTA computes a 128 x 256 tile:
//   warp 0, one lane : TMA producer.  Per 32-wide k chunk it loads A_hi, A_lo
//                      (128 x 32) and B_hi, B_lo (256 x 32), K-major with the
//                      128-byte swizzle, into a STAGES-deep ring.
//   warp 1, one lane : MMA issuer.  tcgen05.mma.kind::tf32, M=128, N=256,
//                      K=8 per instruction, accumulator in TMEM (256 columns).
//                      tcgen05.commit frees a stage / signals the epilogue.
//   all WARPS warps  : epilogue.  tcgen05.ld 32x32b: thread = row, 32
//                      columns per load, WARPS/4 warps per TMEM lane quadrant
//                      (column ranges); C read/modify/write coalesced per
//                      column (a warp covers 32 consecutive rows), its first
//                      columns loaded before the roles start.
// The default (16-wide k chunks with the 64-byte swizzle, two 48 KB stages,
// 4 warps, 120 registers) keeps two CTAs on each SM (2 x 256 TMEM columns),
// so that one tile's epilogue traffic overlaps the other's loads and MMAs;
// measured alone on a 8064^2 update it beats the 32-wide 2-stage / 8-warp
// single-CTA form by 12 % and the whole solve by 4 %.
// The tensor core reads the top 19 bits of an FP32 operand (TF32), so the
// FP32 matrix itself is the "hi" operand; the "lo" operands x - tf32(x) and
// the transposed L panel are written by the panel kernel of the look-ahead
// LU (by k_split_lo in the plain blocked LU).  Every mbarrier wait is
// bounded: on timeout
// the CTA records an error, leaves the tile unwritten and frees its TMEM.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "bem_lu.h"
#include "bem_prof.h"
#include "bem_tc.cuh"

namespace bem {

namespace tc {

#define BEM_TC_STAGES 2
#define BEM_TC_WARPS 4
constexpr int STAGES = BEM_TC_STAGES;
constexpr int WARPS = BEM_TC_WARPS;  // epilogue warps: 4 (all columns each) or 8 (column halves)
constexpr int THREADS = 32 * WARPS;
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 + 256;
static_assert(8 * (2 * STAGES + 1) + 16 <= 256, "barrier area");
// two CTAs per SM when their shared memory fits (registers capped at 128)
constexpr int MIN_BLOCKS = (SMEM_BYTES <= 110 * 1024 && WARPS <= 8) ? 2 : 1;
constexpr uint32_t TMEM_COLS = 256;

struct TcArgs {
  float* C;
  int64_t ldc;
  int M, N;       // valid extent of C (M multiple of 128)
  int ay0;        // row (m) coordinate of the first A row in the A maps
  int bx0, by0;   // B maps: k coordinate and n coordinate of B(0, 0)
  int blx0, bly0; // B lo map: same for the lo copy
  float alpha, beta;
  int* err;
  int cx0, cy0;   // C map (persistent kernel): row and column of C(0, 0)
  int* ctr;       // persistent kernel: {next tile, CTAs done} (zero at launch),
                  // or null for the static order t = blockIdx.x + i gridDim.x
};

__global__ void __launch_bounds__(THREADS, MIN_BLOCKS) k_gemm_tc(const __grid_constant__ CUtensorMap mA,
                                                    const __grid_constant__ CUtensorMap mAlo,
                                                    const __grid_constant__ CUtensorMap mB,
                                                    const __grid_constant__ CUtensorMap mBlo,
                                                    TcArgs a) {
  extern __shared__ __align__(1024) uint8_t dsm[];
  // 1024-byte aligned tile area
  const uint32_t base_u = smem_u32(dsm);
  const uint32_t tiles = (base_u + 1023u) & ~1023u;
  uint8_t* misc = dsm + (tiles - base_u) + STAGES * STAGE_BYTES;
  uint64_t* bars = (uint64_t*)misc;  // full[STAGES], empty[STAGES], done
  uint32_t* s_tmem = (uint32_t*)(misc + 8 * (2 * STAGES + 1));
  int* s_fail = (int*)(misc + 8 * (2 * STAGES + 1) + 8);
  const uint32_t full0 = smem_u32(&bars[0]);
  const uint32_t empty0 = smem_u32(&bars[STAGES]);
  const uint32_t done = smem_u32(&bars[2 * STAGES]);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;

  if (threadIdx.x == 0) {
    for (int i = 0; i < STAGES; ++i) {
      mbar_init(full0 + 8 * i, 1);
      mbar_init(empty0 + 8 * i, 1);
    }
    mbar_init(done, 1);
    *s_fail = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(s_tmem)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *s_tmem;
  constexpr int NCH = LU_NB / BK;  // k chunks

  // epilogue geometry: warp w owns TMEM lanes 32 (w % 4) .. +31 (its rows)
  // and SPAN columns starting at (w / 4) SPAN.  Its first PRE columns of C
  // are loaded now, before the producer and MMA roles start, so that they
  // arrive while the operands load and the MMAs run (all of its columns
  // when they fit in registers).
  constexpr int SPAN = BN * 4 / WARPS;
  constexpr int PRE = SPAN <= 64 ? SPAN : 32;
  const int quad = warp & 3, half = warp >> 2;
  const int row = m0 + quad * 32 + lane;
  const bool rowok = row < a.M;
  const bool useC = a.beta != 0.f;
  float* Crow = a.C + row;
  const int cb0 = half * SPAN;
  float cpre[PRE];
  if (rowok && useC) {
#pragma unroll
    for (int q = 0; q < PRE; ++q) {
      const int col = n0 + cb0 + q;
      cpre[q] = (col < a.N) ? __ldcs(Crow + (size_t)col * a.ldc) : 0.f;
    }
  }

  if (warp == 0 && lane == 0) {
    // producer
    for (int c = 0; c < NCH; ++c) {
      const int s = c % STAGES;
      if (c >= STAGES) {
        if (!mbar_wait(empty0 + 8 * s, ((c / STAGES) - 1) & 1)) { atomicExch(s_fail, 1); break; }
      }
      const uint32_t st = tiles + s * STAGE_BYTES;
      mbar_expect_tx(full0 + 8 * s, STAGE_BYTES);
      tma_load_2d(st, &mA, c * BK, a.ay0 + m0, full0 + 8 * s);
      tma_load_2d(st + A_BYTES, &mAlo, c * BK, a.ay0 + m0, full0 + 8 * s);
      tma_load_2d(st + 2 * A_BYTES, &mB, a.bx0 + c * BK, a.by0 + n0, full0 + 8 * s);
      tma_load_2d(st + 2 * A_BYTES + B_BYTES, &mBlo, a.blx0 + c * BK, a.bly0 + n0, full0 + 8 * s);
    }
  } else if (warp == 1 && lane == 0) {
    // MMA issuer
    bool ok = true;
    for (int c = 0; c < NCH && ok; ++c) {
      const int s = c % STAGES;
      if (!mbar_wait(full0 + 8 * s, (c / STAGES) & 1)) { atomicExch(s_fail, 1); ok = false; break; }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t st = tiles + s * STAGE_BYTES;
      const uint64_t dah = sdesc(st), dal = sdesc(st + A_BYTES);
      const uint64_t dbh = sdesc(st + 2 * A_BYTES), dbl = sdesc(st + 2 * A_BYTES + B_BYTES);
#pragma unroll
      for (int ks = 0; ks < BK / 8; ++ks) {
        const uint64_t off = (uint64_t)((ks * 32) >> 4);  // 32 bytes per k step
        const uint32_t acc0 = (c > 0 || ks > 0) ? 1u : 0u;
        mma_tf32(tmem, dal + off, dbh + off, acc0);
        mma_tf32(tmem, dah + off, dbl + off, 1u);
        mma_tf32(tmem, dah + off, dbh + off, 1u);
      }
      mma_commit(empty0 + 8 * s);
    }
    mma_commit(done);
  }
  __syncwarp();
  // epilogue.  When a warp's columns do not all fit in registers, C is
  // software-pipelined: each 32-column block's loads are issued before the
  // previous block is processed.
  // the go/no-go decision is block-uniform
  const bool got = mbar_wait(done, 0);
  const int all_ok = __syncthreads_and(got ? 1 : 0);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const int fail = *((volatile int*)s_fail);
  if (all_ok && !fail && PRE == SPAN) {
    const uint32_t lane_addr = tmem + ((uint32_t)(quad * 32) << 16);
#pragma unroll
    for (int b = 0; b < PRE / 32; ++b) {
      uint32_t v[32];
      tmem_ld32(lane_addr + cb0 + 32 * b, v);
      if (rowok) {
#pragma unroll
        for (int q = 0; q < 32; ++q) {
          const int col = n0 + cb0 + 32 * b + q;
          if (col < a.N) {
            const float accv = __uint_as_float(v[q]);
            const float r = useC ? a.beta * cpre[32 * b + q] + a.alpha * accv : a.alpha * accv;
            __stcs(Crow + (size_t)col * a.ldc, r);
          }
        }
      }
    }
  } else if (all_ok && !fail) {
    float cnext[32];
#pragma unroll
    for (int q = 0; q < 32; ++q) cnext[q] = cpre[q % PRE];
    const uint32_t lane_addr = tmem + ((uint32_t)(quad * 32) << 16);
#pragma unroll 1
    for (int cb = cb0; cb < cb0 + SPAN; cb += 32) {
      float cv[32];
#pragma unroll
      for (int q = 0; q < 32; ++q) cv[q] = cnext[q];
      if (rowok && useC && cb + 32 < cb0 + SPAN) {
#pragma unroll
        for (int q = 0; q < 32; ++q) {
          const int col = n0 + cb + 32 + q;
          cnext[q] = (col < a.N) ? __ldcs(Crow + (size_t)col * a.ldc) : 0.f;
        }
      }
      uint32_t v[32];
      tmem_ld32(lane_addr + cb, v);
      if (rowok) {
#pragma unroll
        for (int q = 0; q < 32; ++q) {
          const int col = n0 + cb + q;
          if (col < a.N) {
            const float accv = __uint_as_float(v[q]);
            const float r = useC ? a.beta * cv[q] + a.alpha * accv : a.alpha * accv;
            __stcs(Crow + (size_t)col * a.ldc, r);
          }
        }
      }
    }
  } else {
    if (threadIdx.x == 0) atomicExch(a.err, 1);
    // let any MMA still in flight finish before the accumulator is freed
    if (!all_ok) mbar_wait(done, 0);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS)
                 : "memory");
  }
}

// ---------------------------------------------------------------------------
// Persistent variant.  One CTA per SM it runs on (the grid may leave SMs to
// the look-ahead's diagonal and panel kernels) loops over 128 x 256 tiles in
// column-major tile order (the B panel of a tile column stays in L2):
//   warp 0, one lane : TMA producer of the operand chunks (P_STAGES ring).
//   warp 1, one lane : MMA issuer into one of two 256-column TMEM
//                      accumulators, so that tile t+1's MMAs run while the
//                      epilogue drains tile t.
//   warp 2, one lane : TMA producer of C in 128 x 64 chunks (two buffers).
//   warps 4..7       : epilogue (TMEM lane quadrant = warp % 4): C chunk from
//                      shared memory, r = beta C + alpha acc written back in
//                      place, a TMA store of the chunk.
// C thus moves in 32 KB asynchronous copies instead of per-thread loads, and
// neither producer waits on the other.  Every wait is bounded and also stops
// when another role has failed (s_fail), so a failure ends the kernel within
// one wait; the CTA then lets its issued copies and MMAs land before freeing
// TMEM and exiting.  C's tensor map covers the whole matrix, so a tile that
// reaches past the region's last column may only be used where that column
// is the matrix's last (the store clips there); the host checks this.
// Measured alone on 8064^2 updates: 3 operand stages with five 128 x 32 C
// buffers (16 KB each) run at 101 us; 64-column chunks in two buffers at
// 163 us, two operand stages with eight C buffers at 114 us, four stages with
// two C buffers at 201 us: the C ring is the latency the kernel hides.
#ifndef BEM_TCP_STAGES
#define BEM_TCP_STAGES 3
#endif
#ifndef BEM_TCP_CW
#define BEM_TCP_CW 32
#endif
#ifndef BEM_TCP_CBUF
#define BEM_TCP_CBUF 5
#endif
constexpr int P_STAGES = BEM_TCP_STAGES;       // operand ring depth
constexpr int P_CW = BEM_TCP_CW;               // C chunk width (columns)
constexpr int P_CBUF = BEM_TCP_CBUF;           // C chunk buffers
constexpr int P_CBYTES = BM * P_CW * 4;
constexpr int P_NCHUNK = BN / P_CW;            // C chunks per tile
static_assert(P_CW % 32 == 0 && BN % P_CW == 0 && P_CBUF >= 2 && P_CBUF <= 8, "C chunking");
constexpr int P_THREADS = 256;
constexpr int P_SMEM = P_STAGES * STAGE_BYTES + P_CBUF * P_CBYTES + 1024 + 512;
static_assert(P_SMEM <= 227 * 1024, "persistent kernel shared memory");
constexpr uint32_t P_TMEM_COLS = 512;

// bounded wait (one thread) for the phase of `bar` with parity `parity`;
// false on timeout (which sets *fail) or once another role has failed
__device__ __forceinline__ bool pwait(uint32_t bar, uint32_t parity, volatile int* fail) {
  for (int it = 0; it < (1 << 20); ++it) {
    uint32_t done = 0;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
    if ((it & 63) == 63 && *fail) return false;
  }
  *fail = 1;
  return false;
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void tma_store_2d(const CUtensorMap* map, int x, int y, uint32_t src) {
  asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%1, %2}], [%3];" ::"l"(
                   (uint64_t)map),
               "r"(x), "r"(y), "r"(src)
               : "memory");
}

// drain wait used on the exit path only (short bound, no failure check)
__device__ __forceinline__ void pdrain(uint32_t bar, uint32_t parity) {
  for (int i = 0; i < (1 << 16); ++i) {
    uint32_t done = 0;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return;
  }
}

// the same for a whole warp: lane 0 waits, the warp follows its answer, and
// after a completed phase every lane observes it itself (returns at once), so
// that each lane's reads of what the phase published are ordered after it
__device__ __forceinline__ int pwait_warp(uint32_t bar, uint32_t parity, volatile int* fail, int lane) {
  int ok = 0;
  if (lane == 0) ok = pwait(bar, parity, fail) ? 1 : 0;
  ok = __shfl_sync(0xffffffffu, ok, 0);
  if (ok) pdrain(bar, parity);
  return ok;
}

// one consumer thread's next tile from the CTA's tile ring (P_TRING slots
// written by the operand producer): the tile, or -1 at the end or after a
// failure; the slot is released at once
constexpr int P_TRING = 4;
__device__ __forceinline__ int take_tile(uint32_t tile_full, uint32_t tile_empty, volatile int* s_tile, int it,
                                         volatile int* fail) {
  const int slot = it % P_TRING;
  if (!pwait(tile_full + 8 * slot, (it / P_TRING) & 1, fail)) return -1;
  const int t = s_tile[slot];
  mbar_arrive(tile_empty + 8 * slot);
  return t;
}

__global__ void __launch_bounds__(P_THREADS, 1) k_gemm_tc_p(const __grid_constant__ CUtensorMap mA,
                                                          const __grid_constant__ CUtensorMap mAlo,
                                                          const __grid_constant__ CUtensorMap mB,
                                                          const __grid_constant__ CUtensorMap mBlo,
                                                          const __grid_constant__ CUtensorMap mC, TcArgs a) {
  extern __shared__ __align__(1024) uint8_t dsm[];
  const uint32_t base_u = smem_u32(dsm);
  const uint32_t tiles = (base_u + 1023u) & ~1023u;
  const uint32_t cbuf0 = tiles + P_STAGES * STAGE_BYTES;
  uint8_t* misc = dsm + (tiles - base_u) + P_STAGES * STAGE_BYTES + P_CBUF * P_CBYTES;
  // barriers: op_full[P_STAGES], op_empty[P_STAGES], acc_full[2],
  // acc_empty[2], c_full[P_CBUF], c_empty[P_CBUF], fin, tile_full[P_TRING],
  // tile_empty[P_TRING]
  constexpr int NBAR = 2 * P_STAGES + 4 + 2 * P_CBUF + 1 + 2 * P_TRING;
  uint64_t* bars = (uint64_t*)misc;
  const uint32_t op_full = smem_u32(&bars[0]), op_empty = smem_u32(&bars[P_STAGES]);
  const uint32_t acc_full = smem_u32(&bars[2 * P_STAGES]), acc_empty = acc_full + 16;
  const uint32_t c_full = acc_empty + 16, c_empty = c_full + 8 * P_CBUF, fin = c_empty + 8 * P_CBUF;
  const uint32_t tile_full = fin + 8, tile_empty = tile_full + 8 * P_TRING;
  uint32_t* s_tmem = (uint32_t*)(misc + 8 * NBAR);
  volatile int* s_fail = (volatile int*)(misc + 8 * NBAR + 4);
  // [0] operand chunks issued, [1] C chunks issued, [2] operand chunks
  // consumed, [3] C chunks consumed (for the exit path)
  volatile int* s_cnt = (volatile int*)(misc + 8 * NBAR + 8);
  // the tile ring and the epilogue's current tile
  volatile int* s_tile = (volatile int*)(misc + 8 * NBAR + 24);
  volatile int* s_etile = (volatile int*)(misc + 8 * NBAR + 24 + 4 * P_TRING);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int MT = a.M / BM, NT = (a.N + BN - 1) / BN, T = MT * NT;

  if (threadIdx.x == 0) {
    for (int i = 0; i < P_STAGES; ++i) {
      mbar_init(op_full + 8 * i, 1);
      mbar_init(op_empty + 8 * i, 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(acc_full + 8 * i, 1);
      mbar_init(acc_empty + 8 * i, 4);  // one arrival per epilogue warp
    }
    for (int i = 0; i < P_CBUF; ++i) {
      mbar_init(c_full + 8 * i, 1);
      mbar_init(c_empty + 8 * i, 1);
    }
    mbar_init(fin, 1);
    for (int i = 0; i < P_TRING; ++i) {
      mbar_init(tile_full + 8 * i, 1);
      mbar_init(tile_empty + 8 * i, 3);  // MMA issuer, C producer, epilogue
    }
    *s_fail = 0;
    for (int i = 0; i < 4; ++i) s_cnt[i] = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(s_tmem)),
                 "r"(P_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *s_tmem;
  constexpr int NCH = LU_NB / BK;

  if (warp == 0 && lane == 0) {
    // operand producer; it also claims the tiles (from the global counter
    // when there is one, so that CTAs that start late take fewer tiles)
    // and hands them to the other roles through the tile ring
    int opc = 0;
    for (int it = 0;; ++it) {
      int t = a.ctr ? atomicAdd(a.ctr, 1) : (int)blockIdx.x + it * (int)gridDim.x;
      if (t >= T || *s_fail) t = -1;
      const int slot = it % P_TRING;
      if (it >= P_TRING && !pwait(tile_empty + 8 * slot, ((it / P_TRING) - 1) & 1, s_fail)) break;
      s_tile[slot] = t;
      mbar_arrive(tile_full + 8 * slot);
      if (t < 0) break;
      const int m0 = (t % MT) * BM, n0 = (t / MT) * BN;
      for (int c = 0; c < NCH && !*s_fail; ++c, ++opc) {
        const int s = opc % P_STAGES;
        if (opc >= P_STAGES && !pwait(op_empty + 8 * s, ((opc / P_STAGES) - 1) & 1, s_fail)) break;
        const uint32_t st = tiles + s * STAGE_BYTES;
        mbar_expect_tx(op_full + 8 * s, STAGE_BYTES);
        tma_load_2d(st, &mA, c * BK, a.ay0 + m0, op_full + 8 * s);
        tma_load_2d(st + A_BYTES, &mAlo, c * BK, a.ay0 + m0, op_full + 8 * s);
        tma_load_2d(st + 2 * A_BYTES, &mB, a.bx0 + c * BK, a.by0 + n0, op_full + 8 * s);
        tma_load_2d(st + 2 * A_BYTES + B_BYTES, &mBlo, a.blx0 + c * BK, a.bly0 + n0, op_full + 8 * s);
        s_cnt[0] = opc + 1;
      }
    }
  } else if (warp == 2 && lane == 0) {
    // C producer
    int cc = 0;
    for (int it = 0;; ++it) {
      const int t = take_tile(tile_full, tile_empty, s_tile, it, s_fail);
      if (t < 0) break;
      const int m0 = (t % MT) * BM, n0 = (t / MT) * BN;
      const int nch = min(P_NCHUNK, (a.N - n0 + P_CW - 1) / P_CW);
      for (int ch = 0; ch < nch && !*s_fail; ++ch, ++cc) {
        const int b = cc % P_CBUF;
        if (cc >= P_CBUF && !pwait(c_empty + 8 * b, ((cc / P_CBUF) - 1) & 1, s_fail)) break;
        mbar_expect_tx(c_full + 8 * b, P_CBYTES);
        tma_load_2d(cbuf0 + b * P_CBYTES, &mC, a.cx0 + m0, a.cy0 + n0 + ch * P_CW, c_full + 8 * b);
        s_cnt[1] = cc + 1;
      }
      if (*s_fail) break;
    }
  } else if (warp == 1 && lane == 0) {
    // MMA issuer
    int opc = 0;
    for (int it = 0;; ++it) {
      if (take_tile(tile_full, tile_empty, s_tile, it, s_fail) < 0) break;
      const int b = it & 1;
      if (it >= 2 && !pwait(acc_empty + 8 * b, ((it >> 1) - 1) & 1, s_fail)) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t acc = tmem + (uint32_t)(b * BN);
      bool ok = true;
      for (int c = 0; c < NCH; ++c, ++opc) {
        const int s = opc % P_STAGES;
        if (!pwait(op_full + 8 * s, (opc / P_STAGES) & 1, s_fail)) { ok = false; break; }
        s_cnt[2] = opc + 1;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t st = tiles + s * STAGE_BYTES;
        const uint64_t dah = sdesc(st), dal = sdesc(st + A_BYTES);
        const uint64_t dbh = sdesc(st + 2 * A_BYTES), dbl = sdesc(st + 2 * A_BYTES + B_BYTES);
#pragma unroll
        for (int ks = 0; ks < BK / 8; ++ks) {
          const uint64_t off = (uint64_t)((ks * 32) >> 4);
          const uint32_t acc0 = (c > 0 || ks > 0) ? 1u : 0u;
          mma_tf32(acc, dal + off, dbh + off, acc0);
          mma_tf32(acc, dah + off, dbl + off, 1u);
          mma_tf32(acc, dah + off, dbh + off, 1u);
        }
        mma_commit(op_empty + 8 * s);
      }
      if (!ok) break;
      mma_commit(acc_full + 8 * b);
    }
  } else if (warp >= 4) {
    // epilogue: warp w owns TMEM lanes 32 (w % 4) .. + 31 (the tile's rows).
    // All four warps run the same sequence of waits and named barriers over
    // every tile; lane 0 waits and the warp follows its answer, so a failure
    // only skips work and no warp is left at a barrier.
    const int quad = warp & 3;
    const int rloc = quad * 32 + lane;
    int cc = 0;
    for (int it = 0;; ++it) {
      // thread 128 takes the tile for the four warps
      if (threadIdx.x == 128) *s_etile = take_tile(tile_full, tile_empty, s_tile, it, s_fail);
      asm volatile("bar.sync 1, 128;" ::: "memory");
      const int t = *s_etile;
      if (t < 0) break;
      const int m0 = (t % MT) * BM, n0 = (t / MT) * BN;
      const int b = it & 1;
      const int okt = pwait_warp(acc_full + 8 * b, (it >> 1) & 1, s_fail, lane);
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t lane_addr = tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(b * BN);
      const int nch = min(P_NCHUNK, (a.N - n0 + P_CW - 1) / P_CW);
      for (int ch = 0; ch < nch; ++ch, ++cc) {
        const int cb = cc % P_CBUF;
        const int okc = pwait_warp(c_full + 8 * cb, (cc / P_CBUF) & 1, s_fail, lane);
        if (okc && threadIdx.x == 128) s_cnt[3] = cc + 1;
        if (okt && okc) {
          float* cs = (float*)(dsm + (cbuf0 - base_u) + cb * P_CBYTES);
#pragma unroll
          for (int q = 0; q < P_CW / 32; ++q) {
            uint32_t v[32];
            tmem_ld32(lane_addr + ch * P_CW + q * 32, v);
#pragma unroll
            for (int j = 0; j < 32; ++j) {
              float* cp = cs + (q * 32 + j) * BM + rloc;
              *cp = a.beta * *cp + a.alpha * __uint_as_float(v[j]);
            }
          }
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("bar.sync 1, 128;" ::: "memory");
        if (threadIdx.x == 128) {
          // the buffer of the previous chunk is released once its store has
          // read it; this chunk's store stays in flight meanwhile
          if (okt && okc && !*s_fail) {
            tma_store_2d(&mC, a.cx0 + m0, a.cy0 + n0 + ch * P_CW, cbuf0 + cb * P_CBYTES);
            asm volatile("cp.async.bulk.commit_group;" ::: "memory");
            asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory");
          } else {
            asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
          }
          if (cc > 0) mbar_arrive(c_empty + 8 * ((cc - 1) % P_CBUF));
        }
      }
      // the accumulator may be overwritten once every epilogue warp read it
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(acc_empty + 8 * b);
    }
    if (threadIdx.x == 128) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
  }
  __syncwarp();
  __syncthreads();
  if (threadIdx.x == 0 && a.ctr) {
    // the last CTA to finish (every claim made) rearms the counter
    __threadfence();
    if (atomicAdd(a.ctr + 1, 1) == (int)gridDim.x - 1) {
      atomicExch(a.ctr, 0);
      atomicExch(a.ctr + 1, 0);
    }
  }
  if (*s_fail) {
    if (threadIdx.x == 0) {
      atomicExch(a.err, 1);
      // copies issued and not consumed land before the shared memory goes away
      for (int k = s_cnt[2]; k < s_cnt[0]; ++k) pdrain(op_full + 8 * (k % P_STAGES), (k / P_STAGES) & 1);
      for (int k = s_cnt[3]; k < s_cnt[1]; ++k) pdrain(c_full + 8 * (k % P_CBUF), (k / P_CBUF) & 1);
    }
    __syncthreads();
  }
  if (warp == 1) {
    // every MMA issued by this warp's lane 0 completes before TMEM is freed
    if (lane == 0) {
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(fin)
                   : "memory");
      pdrain(fin, 0);
    }
    __syncwarp();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(P_TMEM_COLS)
                 : "memory");
  }
}

}  // namespace tc

// ---------------------------------------------------------------------------
// lo parts and the transposed L panel
// ---------------------------------------------------------------------------
__device__ __forceinline__ float tf32_trunc(float x) {
  return __uint_as_float(__float_as_uint(x) & 0xFFFFE000u);
}

// Lt[m][k] = L21[m][k] (K-major copy), Ltlo = Lt - tf32(Lt);
// U12lo[k][n] = U12 - tf32(U12)  (same K-major layout as U12 in the matrix)
__global__ void k_split_lo(const float* __restrict__ A, int64_t ld, int kk, int rem,
                           float* __restrict__ Lt, float* __restrict__ Ltlo, float* __restrict__ Ulo) {
  __shared__ float tile[32][33];
  // L21: rows kk+128 .., columns kk..kk+127 -> Lt (rem x 128)
  const int mt = blockIdx.x * 32, kt = blockIdx.y * 32;
  if (mt < rem) {
    const float* L = A + (size_t)(kk + LU_NB) + (size_t)kk * ld;
    for (int i = threadIdx.y; i < 32; i += blockDim.y)
      tile[i][threadIdx.x] = L[(size_t)(mt + threadIdx.x) + (size_t)(kt + i) * ld];
    __syncthreads();
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
      const float v = tile[threadIdx.x][i];
      const size_t o = (size_t)(mt + i) * LU_NB + kt + threadIdx.x;
      Lt[o] = v;
      Ltlo[o] = v - tf32_trunc(v);
    }
    // U12: rows kk..kk+127, columns kk+128+mt.. (reuse the m index as n)
    const float* U = A + (size_t)kk + (size_t)(kk + LU_NB) * ld;
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
      const size_t n = (size_t)(mt + i);
      const float v = U[(size_t)(kt + threadIdx.x) + n * ld];
      Ulo[(size_t)(kt + threadIdx.x) + n * LU_NB] = v - tf32_trunc(v);
    }
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
typedef CUresult (*EncodeTiled)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                const cuuint64_t*, const cuuint32_t*, const cuuint32_t*,
                                CUtensorMapInterleave, CUtensorMapSwizzle, CUtensorMapL2promotion,
                                CUtensorMapFloatOOBfill);

static EncodeTiled encode_fn() {
  static EncodeTiled fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiled)p;
  });
  return fn;
}

// 2-D FP32 map: inner dimension `inner` (contiguous), outer `outer`, row
// pitch `pitch` elements, box BK x box_outer, swizzle of BK * 4 bytes.
static bool make_map(CUtensorMap* m, const float* base, uint64_t inner, uint64_t outer, uint64_t pitch,
                     uint32_t box_outer) {
  EncodeTiled fn = encode_fn();
  if (!fn) return false;
  cuuint64_t dims[2] = {inner, outer};
  cuuint64_t strides[1] = {pitch * 4};
  cuuint32_t box[2] = {(cuuint32_t)tc::BK, box_outer};
  cuuint32_t es[2] = {1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void*)base, dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE,
            tc::BK == 32 ? CU_TENSOR_MAP_SWIZZLE_128B
                         : (tc::BK == 16 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_32B),
            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// the matrix as the C operand of the persistent kernel: rows inner, box of
// 128 rows x 64 columns, no swizzle (thread = row reads shared memory
// conflict-free)
static bool make_map_c(CUtensorMap* m, const float* base, uint64_t Npad, uint64_t pitch) {
  EncodeTiled fn = encode_fn();
  if (!fn) return false;
  cuuint64_t dims[2] = {Npad, Npad};
  cuuint64_t strides[1] = {pitch * 4};
  cuuint32_t box[2] = {(cuuint32_t)tc::BM, (cuuint32_t)tc::P_CW};
  cuuint32_t es[2] = {1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void*)base, dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

bool tc_plan(TcPlan& p, float* A, int64_t ld, int Npad, float* Lt, float* Ltlo, float* Ulo, int variant,
             int reserve) {
  p.A = A;
  p.ld = ld;
  p.Npad = Npad;
  p.Lt = Lt;
  p.Ltlo = Ltlo;
  p.Ulo = Ulo;
  p.ok = make_map((CUtensorMap*)p.mA, Lt, LU_NB, (uint64_t)Npad, LU_NB, tc::BM) &&
         make_map((CUtensorMap*)p.mAlo, Ltlo, LU_NB, (uint64_t)Npad, LU_NB, tc::BM) &&
         make_map((CUtensorMap*)p.mB, A, (uint64_t)Npad, (uint64_t)Npad, (uint64_t)ld, tc::BN) &&
         make_map((CUtensorMap*)p.mBlo, Ulo, LU_NB, (uint64_t)Npad, LU_NB, tc::BN) &&
         make_map((CUtensorMap*)p.mB128, A, (uint64_t)Npad, (uint64_t)Npad, (uint64_t)ld, LU_NB) &&
         make_map((CUtensorMap*)p.mBlo128, Ulo, LU_NB, (uint64_t)Npad, LU_NB, LU_NB);
  if (p.ok) {
    cudaFuncSetAttribute(tc::k_gemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, tc::SMEM_BYTES);
  }
  p.variant = 1;
  if (p.ok && variant == 2 && (ld % 4) == 0 && make_map_c((CUtensorMap*)p.mC, A, (uint64_t)Npad, (uint64_t)ld)) {
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    p.grid = nsm - (reserve < 0 ? 0 : reserve);
    if (p.grid >= 1 &&
        cudaFuncSetAttribute(tc::k_gemm_tc_p, cudaFuncAttributeMaxDynamicSharedMemorySize, tc::P_SMEM) ==
            cudaSuccess)
      p.variant = 2;
  }
  return p.ok;
}

void tc_split(const TcPlan& p, int k, cudaStream_t st) {
  const int kk = k * LU_NB;
  const int rem = p.Npad - kk - LU_NB;
  if (rem <= 0) return;
  dim3 sg(rem / 32, LU_NB / 32);
  k_split_lo<<<sg, dim3(32, 8), 0, st>>>(p.A, p.ld, kk, rem, p.Lt, p.Ltlo, p.Ulo);
  count_launches(1);
}

int tc_gemm_sub(const TcPlan& p, int k, int ro, int co, int M, int N, int* err, cudaStream_t st, int* ctr) {
  if (M <= 0 || N <= 0) return 0;
  const int kk = k * LU_NB;
  tc::TcArgs a{};
  a.C = p.A + (size_t)(kk + LU_NB + ro) + (size_t)(kk + LU_NB + co) * p.ld;
  a.ldc = p.ld;
  a.M = M;
  a.N = N;
  a.ay0 = ro;
  a.bx0 = kk;
  a.by0 = kk + LU_NB + co;
  a.blx0 = 0;
  a.bly0 = co;
  a.alpha = -1.f;
  a.beta = 1.f;
  a.err = err;
  count_launches(1);
  // the persistent kernel's C tiles end at a 64-column chunk or at the
  // matrix's last column
  const int cy0 = kk + LU_NB + co;
  if (p.variant == 2 && (N % tc::P_CW == 0 || cy0 + N == p.Npad)) {
    a.cx0 = kk + LU_NB + ro;
    a.cy0 = cy0;
    a.ctr = ctr;
    const int T = (M / tc::BM) * ((N + tc::BN - 1) / tc::BN);
    tc::k_gemm_tc_p<<<T < p.grid ? T : p.grid, tc::P_THREADS, tc::P_SMEM, st>>>(
        *(const CUtensorMap*)p.mA, *(const CUtensorMap*)p.mAlo, *(const CUtensorMap*)p.mB,
        *(const CUtensorMap*)p.mBlo, *(const CUtensorMap*)p.mC, a);
    return (int)cudaGetLastError();
  }
  dim3 grid(M / tc::BM, (N + tc::BN - 1) / tc::BN);
  tc::k_gemm_tc<<<grid, tc::THREADS, tc::SMEM_BYTES, st>>>(*(const CUtensorMap*)p.mA, *(const CUtensorMap*)p.mAlo,
                                                    *(const CUtensorMap*)p.mB, *(const CUtensorMap*)p.mBlo,
                                                    a);
  return (int)cudaGetLastError();
}

}  // namespace bem
