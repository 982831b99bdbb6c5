// BF16 tensor-core GEMM for sm_103a: TMA + mbarrier ring + tcgen05.mma (TMEM accumulator).
//
//   D (M x Ncol, fp32, column-major, ldd = M) (=|+=) A (M x K, bf16, row-major) * B (K x Ncol)
// with B stored column-major (each column's K values contiguous), i.e. both operands
// K-major.  One CTA computes a 128 x 128 tile; warp 0 lane 0 issues TMA loads into a
// 4-stage ring, warp 1 lane 0 issues tcgen05.mma (M=128, N=128, K=16 per instruction),
// all four warps drain the TMEM accumulator with tcgen05.ld.  Every mbarrier wait is
// bounded: on timeout the kernel raises err[0], stops issuing, and still frees TMEM.
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace wg {
namespace tc {

// 3 stages: 97 KiB of shared memory, so two CTAs (2 x 128 TMEM columns) share an SM and
// one CTA's loads and epilogue overlap the other's MMAs
constexpr int BM = 128, BN = 128, BK = 64, STAGES = 3;
constexpr int A_STAGE = BM * BK * 2;         // 16 KiB
constexpr int B_STAGE = BN * BK * 2;         // 16 KiB
constexpr int STAGE_BYTES = A_STAGE + B_STAGE;
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 + 256;
constexpr long long kSpinLimit = 1ll << 22;  // bounded try_wait polling (well under a second normally)

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait; returns false (and raises err) when the limit is reached.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* err) {
  for (long long i = 0; i < kSpinLimit; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((i & 1023) == 1023 && *(volatile int*)err) return false;
  }
  atomicExch(err, 1);
  return false;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int c0, int c1, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// 32 lanes x 32 consecutive fp32 columns of TMEM into 32 registers per thread.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// Shared-memory matrix descriptor: K-major operand, 128-byte swizzle, rows of
// 128 B, 8-row core groups 1024 B apart (stride byte offset), sm_100 version bits.
__device__ __forceinline__ uint64_t sdesc_sw128(const void* p) {
  const uint64_t addr = smem_u32(p);
  uint64_t d = 0;
  d |= (addr >> 4) & 0x3FFFull;
  d |= 1ull << 16;                    // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;   // stride byte offset
  d |= 1ull << 46;                    // descriptor version
  d |= 2ull << 61;                    // 128-byte swizzle
  return d;
}

// Instruction descriptor of kind::f16: D f32, A/B bf16, both K-major, M = 128, N = 128.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) |
                            ((uint32_t)(BM >> 4) << 24);

// EPI 0: D = A B.  EPI 1: D += A B.
template <int EPI>
__global__ void __launch_bounds__(128, 2) gemm_bf16_kernel(const __grid_constant__ CUtensorMap tmA,
                                                           const __grid_constant__ CUtensorMap tmB,
                                                           float* __restrict__ D, int M, long long Ncol, int K,
                                                           int* __restrict__ err, const int* __restrict__ mask,
                                                           int cols_per_problem) {
  // a column tile whose problems are all inactive (mask[b] == 0) has nothing to compute
  if (mask) {
    const long long c0 = (long long)blockIdx.y * BN, c1 = min(Ncol, c0 + BN) - 1;
    bool any = false;
    for (long long b = c0 / cols_per_problem; b <= c1 / cols_per_problem; ++b) any |= mask[b] != 0;
    if (!any) return;
  }
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + STAGES * STAGE_BYTES);
  uint64_t* empty = full + STAGES;
  uint64_t* done = empty + STAGES;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * BM;
  const long long n0 = (long long)blockIdx.y * BN;
  const int nkb = (K + BK - 1) / BK;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) tmem_alloc(tmem_slot, BN);
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0 && lane == 0) {
    // TMA producer
    for (int kb = 0; kb < nkb; ++kb) {
      const int s = kb % STAGES;
      if (kb >= STAGES && !mbar_wait(&empty[s], ((kb / STAGES) + 1) & 1, err)) break;
      uint8_t* a = smem + s * STAGE_BYTES;
      uint8_t* b = a + A_STAGE;
      mbar_expect_tx(&full[s], STAGE_BYTES);
      tma_load_2d(a, &tmA, kb * BK, m0, &full[s]);
      tma_load_2d(b, &tmB, kb * BK, (int)n0, &full[s]);
    }
  } else if (warp == 1 && lane == 0) {
    // MMA issuer
    int issued = 0;
    for (int kb = 0; kb < nkb; ++kb) {
      const int s = kb % STAGES;
      if (!mbar_wait(&full[s], (kb / STAGES) & 1, err)) break;
      fence_after();
      const uint8_t* a = smem + s * STAGE_BYTES;
      const uint8_t* b = a + A_STAGE;
#pragma unroll
      for (int kk = 0; kk < BK / 16; ++kk) {
        mma_bf16(tmem, sdesc_sw128(a + kk * 32), sdesc_sw128(b + kk * 32), kIdesc, (kb | kk) != 0);
        ++issued;
      }
      mma_commit(&empty[s]);
    }
    mma_commit(done);
    (void)issued;
  }
  __syncwarp();
  // epilogue: every warp drains its 32 TMEM lanes (rows 32w .. 32w+31)
  const bool ok = mbar_wait(done, 0, err);
  fence_after();
  if (ok && !*(volatile int*)err) {
    const int row = m0 + warp * 32 + lane;
#pragma unroll 1
    for (int cb = 0; cb < BN / 32; ++cb) {
      float v[32];
      tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + cb * 32, v);
      if (row < M) {
        float* dst = D + (n0 + cb * 32) * (long long)M + row;
        const int ncb = (int)min((long long)32, Ncol - (n0 + cb * 32));
        if (EPI == 1) {
          // issue all loads before any store so they overlap
          float old[32];
#pragma unroll
          for (int i = 0; i < 32; ++i) old[i] = i < ncb ? dst[(long long)i * M] : 0.f;
#pragma unroll
          for (int i = 0; i < 32; ++i) v[i] += old[i];
        }
#pragma unroll
        for (int i = 0; i < 32; ++i)
          if (i < ncb) dst[(long long)i * M] = v[i];
      }
    }
  }
  fence_before();
  __syncthreads();
  if (warp == 0) {
    fence_after();
    tmem_dealloc(tmem, BN);
  }
}

}  // namespace tc
}  // namespace wg
