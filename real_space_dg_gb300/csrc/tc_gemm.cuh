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

// Bounded wait; returns false (and raises err) when the limit of polls is reached, or when
// another thread has raised err already.
__device__ __forceinline__ bool mbar_wait_limit(uint64_t* bar, uint32_t parity, int* err, long long limit) {
  for (long long i = 0; i < limit; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((i & 1023) == 1023 && *(volatile int*)err) return false;
  }
  atomicExch(err, 1);
  return false;
}
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* err) {
  return mbar_wait_limit(bar, parity, err, kSpinLimit);
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

// 32 lanes x 4 consecutive fp32 columns of TMEM.
__device__ __forceinline__ void tmem_ld4(uint32_t taddr, float* v) {
  uint32_t r[4];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 4; ++i) v[i] = __uint_as_float(r[i]);
}

// 16-byte asynchronous global -> shared copy (zero-filled when !valid); many in flight per thread.
__device__ __forceinline__ void cp_async16(void* dst, const void* src, bool valid) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_u32(dst)), "l"(src), "r"(valid ? 16 : 0)
               : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}

// 32 lanes x 2 consecutive fp32 columns of TMEM.
__device__ __forceinline__ void tmem_ld2(uint32_t taddr, float* v) {
  uint32_t r[2];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x2.b32 {%0,%1}, [%2];\n" : "=r"(r[0]), "=r"(r[1]) : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
  v[0] = __uint_as_float(r[0]);
  v[1] = __uint_as_float(r[1]);
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

// The FP32 upwind flux of the mixed form as the epilogue of GEMM 2 (EPI 2): D = A B + flux(x),
// x laid out like D (column-major, M = 2 Nk rows interleaving re/im of k, one column per DG
// node (element e, node a) of a problem of n_el elements with NK nodes each):
//   flux(x)[n][r] = qd_b k_j (sum_c K(a,c) x[e,c][r] + K3c(a) x[e-1,NK-1][r] (k_j > 0) or
//                   K5c(a) x[e+1,0][r] (k_j < 0)) + shift x[e,a][r],  j = r / 2,
// with K = K1 + K2 for k_j > 0 and K1 - K2 for k_j < 0 (the single-node upwind coupling).
struct FluxEpi {
  const float* x;
  const float* kvec;   // [M / 2]
  const float* qd;     // [problems]
  float kp[16], km[16], k3c[4], k5c[4];
  int n_el;
  float shift;
};

// EPI 0: D = A B.  EPI 1: D += A B.  EPI 2: D = A B + flux(x) (NK nodes per element).
// THREADS / 128 warps share each TMEM lane quarter in the epilogue and split its column chunks.
template <int EPI, int NK = 0, int THREADS = 128>
__global__ void __launch_bounds__(THREADS, 2) gemm_bf16_kernel(const __grid_constant__ CUtensorMap tmA,
                                                           const __grid_constant__ CUtensorMap tmB,
                                                           float* __restrict__ D, int M, long long Ncol, int K,
                                                           int* __restrict__ err, const int* __restrict__ mask,
                                                           int cols_per_problem, const FluxEpi ep = FluxEpi{}) {
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
  // EPI 2: the x columns the tile's flux reads (n0 - NK .. n0 + BN + NK - 1, rows m0 .. m0 + BM - 1)
  // staged in the (now idle) operand ring, coalesced: one 512-byte column per warp access
  float* xs = reinterpret_cast<float*>(smem);
  if constexpr (EPI == 2) {
    static_assert(NK == 0 || (BN + 2 * NK) * BM * 4 <= STAGES * STAGE_BYTES, "x tile must fit the stage ring");
    __syncthreads();
    if (ok) {
      // 16-byte asynchronous copies, all issued before any is waited for (M % 128 == 0 here)
      constexpr int NC = BN + 2 * (NK > 0 ? NK : 1);
      constexpr int CH = BM / 4;                       // 16-byte chunks per column
      for (int idx = threadIdx.x; idx < NC * CH; idx += blockDim.x) {
        const int cl = idx / CH, ch = idx - cl * CH;
        const long long n = n0 - NK + cl;
        const bool v = n >= 0 && n < Ncol;
        cp_async16(xs + cl * BM + ch * 4, ep.x + (v ? n : 0) * (long long)M + m0 + ch * 4, v);
      }
      cp_async_wait_all();
    }
    __syncthreads();
  }
  if (ok && !*(volatile int*)err) {
    const int wq = warp & 3, cg = warp >> 2;
    const int row = m0 + wq * 32 + lane;
#pragma unroll 1
    for (int cb = cg; cb < BN / 32; cb += THREADS / 128) {
      float v[32];
      tmem_ld32(tmem + ((uint32_t)(wq * 32) << 16) + cb * 32, v);
      if (EPI == 2 && row < M) {
        // k_j > 0 for j < Nk / 2: the branch is warp-uniform when Nk is a multiple of 32
        const float kj = ep.kvec[row >> 1];
        const bool pos = kj > 0.f;
        const int cpp = cols_per_problem;
        const long long nb = n0 + cb * 32;
        const int ncb = (int)min((long long)32, Ncol - nb);
        const int rl = row - m0;
#pragma unroll
        for (int i = 0; i < 32; ++i) {
          if (i >= ncb) continue;
          const long long n = nb + i;
          const int b = (int)n / cpp;                  // 32-bit: a handle's columns fit an int
          const int rem = (int)n - b * cpp;
          const int e = rem / NK, a = rem - e * NK;
          // column n - a + c of x is staged at xs[(n - a + c - (n0 - NK)) * BM + rl]
          const float* xc = xs + (int)(n - a - (n0 - NK)) * BM + rl;   // node 0 of element e
          float acc = 0.f;
#pragma unroll
          for (int c = 0; c < NK; ++c) acc = fmaf(pos ? ep.kp[a * NK + c] : ep.km[a * NK + c], xc[c * BM], acc);
          if (pos && e > 0) acc = fmaf(ep.k3c[a], xc[-BM], acc);
          else if (!pos && e < ep.n_el - 1) acc = fmaf(ep.k5c[a], xc[NK * BM], acc);
          v[i] += fmaf(ep.qd[b] * kj, acc, ep.shift * xc[a * BM]);
        }
      }
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

// ---------------------------------------------------------------------------------------------
// GEMM 1 with the xi stencil of the mixed form in its epilogue:
//   X^ = Phi' x (all 2 N_xi rows of a tile of BN2 state columns, MT = 2 N_xi / 128 accumulators
//   of 128 x BN2 in TMEM), then per element e of the tile, node a, cell s:
//   Y_a(s) = sum_c beta_ac(s) (X_c(s) + X_c(s-1)) + beta_ac(s+1) (X_c(s) + X_c(s+1)),
//   beta = betar (pairs a <= c stored) + i betai, written as the BF16 B operand of GEMM 2.
// A tile holds EPT = BN2 / NK whole elements (columns n0 = tile * EPT * NK ..); its B box of BN2
// columns may reach into the next tile, those columns are computed and not used.  TMEM lane r of
// accumulator mt holds row 128 mt + r (row 2 s + o: o = 0 real, 1 imaginary part of cell s); warp
// w reads lanes 32 w .. 32 w + 31, i.e. cells 16 consecutive cells; the cells at a warp's edges
// come from the neighbouring warp through shared memory (first pass), the interior ones by
// shuffles (second pass).  No X^ round trip through global memory.
// ---------------------------------------------------------------------------------------------
constexpr int BN2 = 64;
constexpr int ST_STAGES = 3;
constexpr int B2_STAGE = BN2 * BK * 2;       // 8 KiB
constexpr int ST_STAGE_BYTES = A_STAGE + B2_STAGE;
constexpr int ST_MAX_MT = 8;                  // 2 N_xi <= 1024
constexpr int ST_EDGE_BYTES = 2 * 4 * ST_MAX_MT * BN2 * 8;
constexpr int ST_SMEM_BYTES = ST_STAGES * ST_STAGE_BYTES + ST_EDGE_BYTES + 1024 + 256;
constexpr uint32_t kIdescN64 = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN2 >> 3) << 17) |
                               ((uint32_t)(BM >> 4) << 24);

__host__ __device__ constexpr int st_pair_index(int nk, int a, int c) { return a * nk - a * (a - 1) / 2 + (c - a); }

constexpr int ST_THREADS = 512;   // 16 warps: TMEM lane quarter w % 4, element group w / 4

template <int NK>
__global__ void __launch_bounds__(ST_THREADS, 2) gemm_stencil_kernel(const __grid_constant__ CUtensorMap tmA,
                                                              const __grid_constant__ CUtensorMap tmB,
                                                              __nv_bfloat162* __restrict__ Yh,
                                                              const float* __restrict__ betar,
                                                              const float* __restrict__ betai, int nxi, int ne4,
                                                              long long n_elements, int n_el, int K,
                                                              int* __restrict__ err, const int* __restrict__ mask) {
  constexpr int EPT = BN2 / NK;
  constexpr int NP = NK * (NK + 1) / 2;
  const int MT = (2 * nxi) / BM;
  const long long be0 = (long long)blockIdx.x * EPT;
  if (mask) {
    const long long be1 = min(n_elements, be0 + EPT) - 1;
    bool any = false;
    for (long long b = be0 / n_el; b <= be1 / n_el; ++b) any |= mask[b] != 0;
    if (!any) return;
  }
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  float2* edge_first = reinterpret_cast<float2*>(smem + ST_STAGES * ST_STAGE_BYTES);   // [4 MT][BN2]
  float2* edge_last = edge_first + 4 * ST_MAX_MT * BN2;
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + ST_STAGES * ST_STAGE_BYTES + ST_EDGE_BYTES);
  uint64_t* empty = full + ST_STAGES;
  uint64_t* done = empty + ST_STAGES;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wq = warp & 3, eg = warp >> 2;            // TMEM lane quarter, element group
  constexpr int NEG = ST_THREADS / 128;               // element groups
  const int n0 = (int)(be0 * NK);
  const int nkb = K / BK;
  const int iters = MT * nkb;
  const uint32_t ncols_tmem = (uint32_t)(MT * BN2);   // 128, 256 or 512

  if (threadIdx.x == 0) {
    for (int s = 0; s < ST_STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) tmem_alloc(tmem_slot, ncols_tmem);
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0 && lane == 0) {
    // TMA producer: for every accumulator mt the A rows 128 mt .. and the B tile, k block by k block
    for (int it = 0; it < iters; ++it) {
      const int s = it % ST_STAGES, mt = it / nkb, kb = it - mt * nkb;
      if (it >= ST_STAGES && !mbar_wait(&empty[s], ((it / ST_STAGES) + 1) & 1, err)) break;
      uint8_t* a = smem + s * ST_STAGE_BYTES;
      uint8_t* b = a + A_STAGE;
      mbar_expect_tx(&full[s], ST_STAGE_BYTES);
      tma_load_2d(a, &tmA, kb * BK, mt * BM, &full[s]);
      tma_load_2d(b, &tmB, kb * BK, n0, &full[s]);
    }
  } else if (warp == 1 && lane == 0) {
    // MMA issuer: accumulator mt occupies TMEM columns mt * BN2 ..
    for (int it = 0; it < iters; ++it) {
      const int s = it % ST_STAGES, mt = it / nkb, kb = it - mt * nkb;
      if (!mbar_wait(&full[s], (it / ST_STAGES) & 1, err)) break;
      fence_after();
      const uint8_t* a = smem + s * ST_STAGE_BYTES;
      const uint8_t* b = a + A_STAGE;
#pragma unroll
      for (int kk = 0; kk < BK / 16; ++kk)
        mma_bf16(tmem + (uint32_t)(mt * BN2), sdesc_sw128(a + kk * 32), sdesc_sw128(b + kk * 32), kIdescN64,
                 (kb | kk) != 0);
      mma_commit(&empty[s]);
    }
    mma_commit(done);
  }
  __syncwarp();
  const bool ok = mbar_wait(done, 0, err);
  fence_after();
  // block-uniform, since the epilogue synchronises the block between its passes
  const bool go = __syncthreads_and(ok && !*(volatile int*)err) != 0;
  const uint32_t lane_base = (uint32_t)(wq * 32) << 16;
  if (go && eg == 0) {
    // pass 1: the first and the last cell of every lane quarter's 16 cells, every column
    for (int mt = 0; mt < MT; ++mt) {
      const int q = 4 * mt + wq;
#pragma unroll 1
      for (int half = 0; half < BN2 / 32; ++half) {
        float v[32];
        tmem_ld32(tmem + lane_base + mt * BN2 + half * 32, v);
        if (lane < 2 || lane >= 30) {
          float2* dst = (lane < 2 ? edge_first : edge_last) + q * BN2 + half * 32;
          const int comp = lane & 1;
#pragma unroll
          for (int c = 0; c < 32; ++c) reinterpret_cast<float*>(dst + c)[comp] = v[c];
        }
      }
    }
  }
  __syncthreads();
  // the weights of one accumulator's 64 cells (+1) for the tile's elements, staged in the idle
  // operand ring: sbr[et][pair][65], sbi[a NK + c][65]
  constexpr int SW = BM / 2 + 4;   // 65 weights (cells s_lo .. s_lo + 64) in 16-byte rows
  static_assert((EPT * NP + NK * NK) * SW * 4 <= ST_STAGES * ST_STAGE_BYTES, "weights must fit the stage ring");
  float* sbr = reinterpret_cast<float*>(smem);
  float* sbi = sbr + EPT * NP * SW;
  if (go) {
    const int comp = lane & 1;
    for (int mt = 0; mt < MT; ++mt) {
      const int s_lo = mt * (BM / 2);
      // rows of ne4 floats (ne4 % 4 == 0, s_lo % 64 == 0, s_lo + SW <= ne4): 16-byte aligned chunks,
      // asynchronous copies all in flight before the wait
      constexpr int CH = SW / 4;
      for (int idx = threadIdx.x; idx < (EPT * NP + NK * NK) * CH; idx += blockDim.x) {
        const int row = idx / CH, ch = idx - row * CH;
        const float* src;
        bool v = true;
        if (row < EPT * NP) {
          const int et = row / NP, p = row - et * NP;
          const long long be = be0 + et;
          v = be < n_elements;
          src = betar + ((v ? be : 0) * NP + p) * (long long)ne4 + s_lo + ch * 4;
        } else {
          src = betai + (row - EPT * NP) * (long long)ne4 + s_lo + ch * 4;
        }
        cp_async16(sbr + row * SW + ch * 4, src, v);
      }
      cp_async_wait_all();
      __syncthreads();
      const int q = 4 * mt + wq;
      const int s = (mt * BM + wq * 32 + lane) >> 1;          // this thread's cell
      const int sl = s - s_lo;
      const bool first_cell = lane < 2, last_cell = lane >= 30;
#pragma unroll 1
      for (int et = eg; et < EPT; et += NEG) {
        const long long be = be0 + et;
        const bool valid = be < n_elements && (!mask || mask[be / n_el]);
        // X^ of this element's NK columns (a 4-column load for NK = 3 stays inside the tile:
        // its last element ends at column 62)
        float v[4];
        if constexpr (NK == 2) tmem_ld2(tmem + lane_base + mt * BN2 + et * NK, v);
        else tmem_ld4(tmem + lane_base + mt * BN2 + et * NK, v);
        float yr[NK], yi[NK];
#pragma unroll
        for (int a = 0; a < NK; ++a) yr[a] = yi[a] = 0.f;
        const float* br = sbr + et * NP * SW + sl;
        const float* bi = sbi + sl;
#pragma unroll
        for (int c = 0; c < NK; ++c) {
          const int col = et * NK + c;
          const float own = v[c];
          const float other = __shfl_xor_sync(0xffffffffu, own, 1);
          const float xr = comp ? other : own, xi = comp ? own : other;
          float mr = __shfl_up_sync(0xffffffffu, xr, 2), mi = __shfl_up_sync(0xffffffffu, xi, 2);
          float pr = __shfl_down_sync(0xffffffffu, xr, 2), pi = __shfl_down_sync(0xffffffffu, xi, 2);
          if (first_cell) {
            const float2 t = q > 0 ? edge_last[(q - 1) * BN2 + col] : make_float2(0.f, 0.f);
            mr = t.x;
            mi = t.y;
          }
          if (last_cell) {
            const float2 t = q + 1 < 4 * MT ? edge_first[(q + 1) * BN2 + col] : make_float2(0.f, 0.f);
            pr = t.x;
            pi = t.y;
          }
          const float smr = xr + mr, smi = xi + mi, spr = xr + pr, spi = xi + pi;
          if (valid) {
#pragma unroll
            for (int a = 0; a < NK; ++a) {
              const float* rr = br + st_pair_index(NK, a < c ? a : c, a < c ? c : a) * SW;
              const float* ri = bi + (a * NK + c) * SW;
              const float b0r = rr[0], b1r = rr[1], b0i = ri[0], b1i = ri[1];
              yr[a] += b0r * smr - b0i * smi + b1r * spr - b1i * spi;
              yi[a] += b0r * smi + b0i * smr + b1r * spi + b1i * spr;
            }
          }
        }
        if (valid && comp == 0) {
#pragma unroll
          for (int a = 0; a < NK; ++a) Yh[(be * NK + a) * nxi + s] = __floats2bfloat162_rn(yr[a], yi[a]);
        }
      }
      __syncthreads();   // the next accumulator restages the weights
    }
  }
  fence_before();
  __syncthreads();
  if (warp == 0) {
    fence_after();
    tmem_dealloc(tmem, ncols_tmem);
  }
}

}  // namespace tc
}  // namespace wg
