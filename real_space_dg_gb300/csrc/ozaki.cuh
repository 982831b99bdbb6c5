// FP64 GEMM emulated on the BF16 tensor cores (Ozaki splitting), sm_103a.
//
//   C (M x Ncol, fp64, column-major)  (=|+=)  A (M x K, fp64)  *  B (K x Ncol, fp64, column-major)
//
// Each row of A and each column of B is scaled by a power of two and rounded to
// an integer F with |F| <= 2^(6S-1), which is written in S balanced base-64
// digits: a = 2^e sum_p t_p 2^(-6(p+1)), |t_p| <= 32 (|t_0| <= 33).  The digits
// are exact in BF16 and a digit product summed over K <= 1024 stays below
// 33^2 * 1024 < 2^21, so every product A^(p) B^(q) is EXACT in the FP32 tensor-core
// accumulator.  Products of equal weight p+q (at most 8 of them) share one TMEM
// accumulator (< 8 * 33^2 * 1024 < 2^24, still exact); the S groups of a 128 x 64 output tile use 8 x 64 = 512
// TMEM columns.  Products of weight p+q >= S are dropped.  The B digit slices lie
// one after the other in shared memory, so the products of one A slice p with the
// slices q = q0 .. q0+n-1 are ONE instruction of N = 64 n (n <= 4) whose accumulator
// starts at group p+q0: 12 MMAs per k step instead of 36, and the A tile is read
// from shared memory 12 times instead of 36.  The epilogue adds the groups as
// integers in a 64-bit fixed point (unit 2^-50), rounds once to FP64 and applies
// the row and column exponents, all with integer instructions.  Error: a few
// 2^(-6S) (S = 8: ~1e-14) relative to |A| |B|, unbiased (rounded split).
#pragma once
#include "tc_gemm.cuh"

namespace wg {
namespace oz {

constexpr int S = 8;              // digits per operand
constexpr int BETA = 6;           // bits per digit
// k blocks of 32 (64-byte rows, 64-byte swizzle).  A stage holds the nd A and nd B slices
// the launch uses, so the 192 KiB ring has two stages at 7 or 8 digits and more with fewer
// digits (three at 5, four at 4): the TMA loads run further ahead of the MMAs
constexpr int BM = 128, BN = 64, BK = 32, STAGES = 2, MAX_STAGES = 8;
constexpr int THREADS = 512;      // warp 0 TMA, warp 1 MMA, all 16 drain TMEM (four warps per lane quarter)
constexpr int EPI_COLS = BN / (THREADS / 128);   // 16 output columns per epilogue warp
static_assert(EPI_COLS == 16, "the epilogue drains 16 TMEM columns per warp");
constexpr int NGROUP = S;         // weights p+q = 2 .. S+1
constexpr int A_SLICE = BM * BK * 2;      // 8 KiB
constexpr int B_SLICE = BN * BK * 2;      // 4 KiB
constexpr int STAGE = S * (A_SLICE + B_SLICE);   // 96 KiB (all 8 digits)
constexpr int RING = STAGES * STAGE;              // 192 KiB
constexpr int SMEM_BYTES = RING + 1024 + 256;
__host__ __device__ constexpr int stages_for(int nd) {
  return RING / (nd * (A_SLICE + B_SLICE)) < MAX_STAGES ? RING / (nd * (A_SLICE + B_SLICE)) : MAX_STAGES;
}
constexpr int MAX_K = 1024;       // exactness bound of the grouped accumulation (8 * 33^2 * K < 2^24)

// Instruction descriptor: D f32, A/B bf16, K-major, M = 128, N = n (16 <= n <= 256, n % 16 == 0).
constexpr uint32_t kIdescM128 = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BM >> 4) << 24);
__device__ __forceinline__ uint32_t idesc_n(int n) { return kIdescM128 | ((uint32_t)(n >> 3) << 17); }
constexpr int kSlicesPerMma = 256 / BN;   // B slices one instruction covers (N <= 256)

// K-major operand tile with 64-byte rows and the 64-byte swizzle (8-row atoms of 512 bytes).
__device__ __forceinline__ uint64_t sdesc_sw64(const void* p) {
  const uint64_t addr = tc::smem_u32(p);
  uint64_t d = 0;
  d |= (addr >> 4) & 0x3FFFull;
  d |= 1ull << 16;                    // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(512 >> 4) << 32;    // stride byte offset: 8 rows x 64 bytes
  d |= 1ull << 46;                    // descriptor version
  d |= 4ull << 61;                    // 64-byte swizzle
  return d;
}

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int c0, int c1, int c2,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::
          "r"(tc::smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(tc::smem_u32(bar))
      : "memory");
}

// 32 lanes x 16 consecutive fp32 columns of TMEM into 16 registers per thread.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// Fixed-point unit of the epilogue: 2^-50.  Group g (weight 2^(-6(g+2))) enters
// shifted left by 38 - 6g; the last group (g = 7) is rounded by 4 bits.  |sum| <
// 33^2 * 1024 * 2^38 + ... < 2^59 for K <= 1024.
constexpr int kFixBits = 50;
__device__ __forceinline__ long long group_fixed(float v, int g) {
  const long long t = (long long)__float2int_rn(v);   // exact: an integer below 2^24
  const int sh = kFixBits - BETA * (g + 2);
  return sh >= 0 ? (t << sh) : ((t + (1ll << (-sh - 1))) >> -sh);
}

// a * 2^e as the nearest double (ties to even), integer instructions only; results
// below the normal range flush to zero.
__device__ __forceinline__ double fixed_to_double(long long a, int e) {
  if (a == 0) return 0.0;
  const unsigned long long sign = a < 0 ? 1ull << 63 : 0ull;
  unsigned long long u = a < 0 ? 0ull - (unsigned long long)a : (unsigned long long)a;
  int msb = 63 - __clzll((long long)u);
  unsigned long long mant;
  if (msb <= 52) {
    mant = u << (52 - msb);
  } else {
    const int sh = msb - 52;
    mant = u >> sh;
    const unsigned long long rem = u & ((1ull << sh) - 1), half = 1ull << (sh - 1);
    if (rem > half || (rem == half && (mant & 1ull))) ++mant;
    if (mant >> 53) {
      mant >>= 1;
      ++msb;
    }
  }
  const int ex = msb + e + 1023;
  if (ex <= 0) return sign ? -0.0 : 0.0;
  if (ex >= 0x7FF) return __longlong_as_double((long long)(sign | (0x7FFull << 52)));
  return __longlong_as_double((long long)(sign | ((unsigned long long)ex << 52) | (mant & 0xFFFFFFFFFFFFFull)));
}

// EPI 0: C = A B.  EPI 1: C += A B.   ea[row], eb[col]: power-of-two exponents of A's rows and B's columns.
template <int EPI>
__global__ void __launch_bounds__(THREADS, 1) gemm_ozaki_kernel(const __grid_constant__ CUtensorMap tmA,
                                                            const __grid_constant__ CUtensorMap tmB,
                                                            const int* __restrict__ ea, const int* __restrict__ eb,
                                                            double* __restrict__ C, int M, long long Ncol, int K,
                                                            int* __restrict__ err, const int* __restrict__ mask,
                                                            int cols_per_problem, int nd,
                                                            const int* __restrict__ nd_pp) {
  // nd (1 .. S): leading digits used of each operand (products of weight < nd); the error grows
  // to ~2^(-6 nd) of |A||B|.  nd_pp (optional): digits per problem, the tile takes the largest of
  // its problems.  A column tile whose problems are all inactive has nothing to compute.
  if (mask || nd_pp) {
    const long long c0 = (long long)blockIdx.y * BN, c1 = min(Ncol, c0 + BN) - 1;
    bool any = false;
    int ndt = 1;
    for (long long b = c0 / cols_per_problem; b <= c1 / cols_per_problem; ++b) {
      const bool on = !mask || mask[b] != 0;
      any |= on;
      if (nd_pp && on) ndt = max(ndt, min(S, max(1, nd_pp[b])));
    }
    if (!any) return;
    if (nd_pp) nd = ndt;
  }
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  // stage s: [nd][BM][BK] bf16 A slices, then [nd][BN][BK] bf16 B slices
  const int ns = stages_for(nd);
  const int stage = nd * (A_SLICE + B_SLICE);
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + RING);
  uint64_t* empty = full + MAX_STAGES;
  uint64_t* done = empty + MAX_STAGES;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * BM;
  const long long n0 = (long long)blockIdx.y * BN;
  const int nkb = (K + BK - 1) / BK;

  if (threadIdx.x == 0) {
    for (int st = 0; st < ns; ++st) {
      tc::mbar_init(&full[st], 1);
      tc::mbar_init(&empty[st], 1);
    }
    tc::mbar_init(done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) tc::tmem_alloc(tmem_slot, 512);
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0 && lane == 0) {
    for (int kb = 0; kb < nkb; ++kb) {
      const int st = kb % ns;
      if (kb >= ns && !tc::mbar_wait(&empty[st], ((kb / ns) + 1) & 1, err)) break;
      uint8_t* sa = smem + st * stage;
      uint8_t* sb = sa + nd * A_SLICE;
      tc::mbar_expect_tx(&full[st], (uint32_t)(nd * (A_SLICE + B_SLICE)));
      for (int p = 0; p < nd; ++p) {
        tma_load_3d(sa + p * A_SLICE, &tmA, kb * BK, m0, p, &full[st]);
        tma_load_3d(sb + p * B_SLICE, &tmB, kb * BK, (int)n0, p, &full[st]);
      }
    }
  } else if (warp == 1 && lane == 0) {
    for (int kb = 0; kb < nkb; ++kb) {
      const int st = kb % ns;
      if (!tc::mbar_wait(&full[st], (kb / ns) & 1, err)) break;
      tc::fence_after();
      const uint8_t* sa = smem + st * stage;
      const uint8_t* sb = sa + nd * A_SLICE;
#pragma unroll
      for (int kk = 0; kk < BK / 16; ++kk)
        for (int p = 0; p < nd; ++p)
          for (int q0 = 0; q0 + p < nd; q0 += kSlicesPerMma) {   // weights p+q (0-based) <= nd-1
            const int n = min(kSlicesPerMma, nd - p - q0);
            // slices q0 .. q0+n-1 are consecutive 64-row blocks: their accumulators, groups
            // p+q0 .. p+q0+n-1, are consecutive 64-column blocks of TMEM
            const uint32_t d = tmem + (uint32_t)((p + q0) * BN);
            // every group is first reached with p == 0: the p == 0 products of the first k block
            // and k step initialise the accumulators, every other one accumulates
            const uint32_t acc = (kb > 0 || kk > 0 || p > 0) ? 1u : 0u;
            tc::mma_bf16(d, sdesc_sw64(sa + p * A_SLICE + kk * 32), sdesc_sw64(sb + q0 * B_SLICE + kk * 32),
                         idesc_n(n * BN), acc);
          }
      tc::mma_commit(&empty[st]);
    }
    tc::mma_commit(done);
  }
  __syncwarp();
  const bool ok = tc::mbar_wait(done, 0, err);
  tc::fence_after();
  if (ok && !*(volatile int*)err) {
    // warp w reads TMEM lanes 32 (w % 4) .. +31 (rows) and the 16-column block w / 4
    constexpr int EC = EPI_COLS;
    const int wq = warp & 3, cb = warp >> 2;
    const int row = m0 + wq * 32 + lane;
    const int er = row < M ? ea[row] : 0;
    {
      long long fx[EC];
#pragma unroll
      for (int i = 0; i < EC; ++i) fx[i] = 0;
#pragma unroll 1
      for (int g = 0; g < nd; ++g) {
        float v[EC];
        tmem_ld16(tmem + ((uint32_t)(wq * 32) << 16) + (uint32_t)(g * BN + cb * EC), v);
#pragma unroll
        for (int i = 0; i < EC; ++i) fx[i] += group_fixed(v[i], g);
      }
      if (row < M) {
        const long long c0 = n0 + cb * EC;
        const int ncb = (int)max(0ll, min((long long)EC, Ncol - c0));
        double* dst = C + c0 * (long long)M + row;
        double old[EC];
        if (EPI == 1) {
#pragma unroll
          for (int i = 0; i < EC; ++i) old[i] = i < ncb ? dst[(long long)i * M] : 0.0;
        }
#pragma unroll
        for (int i = 0; i < EC; ++i) {
          if (i < ncb) {
            const double val = fixed_to_double(fx[i], er + eb[c0 + i] - kFixBits);
            dst[(long long)i * M] = EPI == 1 ? old[i] + val : val;
          }
        }
      }
    }
  }
  tc::fence_before();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after();
    tc::tmem_dealloc(tmem, 512);
  }
}

// Digits of the columns of a K x Ncol column-major FP64 matrix: for column c with
// max|x| < 2^m, F = round(x 2^(6S-1-m)) (|F| <= 2^(6S-1)) is split into balanced
// base-64 digits t_p (p = 0 most significant), x = 2^e sum_p t_p 2^(-6(p+1)) with
// e = m + 1 written to e_out[c]; t_p goes as bf16 to slices[p][c][k] (K-major).
// Integer arithmetic on the FP64 bit patterns only.
constexpr int kSliceColsPerBlock = 8;   // one warp per column

__device__ __forceinline__ long long round_scaled(long long bits, int m, bool nonzero) {
  const int ex = (int)((bits >> 52) & 0x7FF);
  long long F = 0;   // round(|x| 2^(6S-1-m)) <= 2^(6S-1)
  if (ex != 0 && nonzero) {
    const unsigned long long mant = ((unsigned long long)bits & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    const int rs = m - (ex - 1023 - 52) - (BETA * S - 1);   // >= 6 since |x| < 2^m
    if (rs < 64) F = (long long)((mant + (1ull << (rs - 1))) >> rs);
  }
  return bits < 0 ? -F : F;
}

// One warp per column, two consecutive k per lane (K is even): 4-byte stores per slice.
__global__ void __launch_bounds__(32 * kSliceColsPerBlock) slice_columns_kernel(const double* __restrict__ X, int K,
                                                                               long long Ncol,
                                                                               __nv_bfloat16* __restrict__ slices,
                                                                               int* __restrict__ e_out,
                                                                               const int* __restrict__ mask = nullptr,
                                                                               int cols_per_problem = 1,
                                                                               int Kout = 0, int nd = S,
                                                                               const int* __restrict__ nd_pp = nullptr) {
  // Kout: row length of the slices (>= K, zero-padded; 0: K), for 16-byte TMA rows.
  // nd, nd_pp: the digits gemm_ozaki_kernel reads for the column's 64-column tile (the same
  // rule: nd_pp's largest over the tile's active problems, else nd); only those are written
  const int lane = threadIdx.x & 31;
  const long long c = (long long)blockIdx.x * kSliceColsPerBlock + (threadIdx.x >> 5);
  if (c >= Ncol || (mask && !mask[c / cols_per_problem])) return;
  int ndt = nd < 1 ? 1 : (nd > S ? S : nd);
  if (nd_pp) {
    const long long c0 = c / BN * BN, c1 = min(Ncol, c0 + BN) - 1;
    ndt = 1;
    for (long long b = c0 / cols_per_problem; b <= c1 / cols_per_problem; ++b)
      if (!mask || mask[b] != 0) ndt = max(ndt, min(S, max(1, nd_pp[b])));
  }
  const int Ko = Kout > K ? Kout : K;
  const double2* x = reinterpret_cast<const double2*>(X + c * (long long)K);
  const int K2 = K / 2;
  unsigned long long mx = 0;
  for (int k = lane; k < K2; k += 32) {
    const double2 v = x[k];
    const unsigned long long a = (unsigned long long)__double_as_longlong(v.x) & 0x7FFFFFFFFFFFFFFFull;
    const unsigned long long b = (unsigned long long)__double_as_longlong(v.y) & 0x7FFFFFFFFFFFFFFFull;
    mx = a > mx ? a : mx;
    mx = b > mx ? b : mx;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long t = __shfl_xor_sync(0xffffffffu, mx, o);
    mx = t > mx ? t : mx;
  }
  const int emax = (int)((mx >> 52) & 0x7FF);
  const int m = mx == 0 ? 0 : emax - 1023 + 1;   // max|x| < 2^m
  if (lane == 0) e_out[c] = m + 1;
  const long long slice_stride = Ncol * (long long)Ko;
  __nv_bfloat162* out = reinterpret_cast<__nv_bfloat162*>(slices + c * (long long)Ko);
  for (int k = K2 + lane; k < Ko / 2; k += 32)
#pragma unroll
    for (int p = 0; p < S; ++p) out[p * (slice_stride / 2) + k] = __floats2bfloat162_rn(0.f, 0.f);
  for (int k = lane; k < K2; k += 32) {
    const double2 v = x[k];
    long long F0 = round_scaled(__double_as_longlong(v.x), m, mx != 0);
    long long F1 = round_scaled(__double_as_longlong(v.y), m, mx != 0);
#pragma unroll
    for (int p = S - 1; p > 0; --p) {
      const int d0 = (int)(((F0 + 32) & 63) - 32), d1 = (int)(((F1 + 32) & 63) - 32);
      if (p < ndt) out[p * (slice_stride / 2) + k] = __floats2bfloat162_rn((float)d0, (float)d1);
      F0 = (F0 - d0) >> BETA;
      F1 = (F1 - d1) >> BETA;
    }
    out[k] = __floats2bfloat162_rn((float)F0, (float)F1);
  }
}

}  // namespace oz
}  // namespace wg
