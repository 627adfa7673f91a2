// Split-BF16 GEMM on the fifth-generation tensor cores (tcgen05).
//
// C[m][n] = sum_k A[m][k] B[n][k] with A and B each given as NP BF16 pieces
// (K contiguous, K padded to a multiple of 64 with zeros):
//   NP = 2:  C ~= A0 B0 + A0 B1 + A1 B0                        (~2^-16 relative)
//   NP = 3:  C ~= A0 B0 + A0 B1 + A1 B0 + A1 B1 + A0 B2 + A2 B0 (~2^-24 relative)
// with FP32 accumulation in tensor memory.
//
// One CTA computes one 128 x 128 tile of C with four warps:
//   warp 0 lane 0  TMA producer: per 64-wide K step, the 2 NP operand tiles
//                  (128 x 64 BF16, 16 KB each) into a ring of 128-byte-swizzled
//                  shared-memory stages (3 stages for NP = 2, 2 for NP = 3);
//   warp 1 lane 0  MMA issuer: 4 x (products) tcgen05.mma (M 128, N 128, K 16)
//                  per step into a 128-column FP32 accumulator in tensor memory;
//                  each step's tcgen05.commit releases its stage;
//   all 4 warps    epilogue: tcgen05.ld of their 32 accumulator lanes (rows),
//                  FP32 or split-BF16 stores with optional grouped row / column
//                  remaps.
// Every wait on an mbarrier is bounded; a wait that runs out sets *err and the
// CTA skips to its clean-up (TMEM is always released).
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstring>
#include <mutex>

#include "kernels.cuh"

namespace lgb {
namespace {

constexpr int kBM = 128, kBN = 128, kBK = 64;
constexpr int kTileBytes = 128 * kBK * 2;               // one operand tile, 16 KB
constexpr int kTmemCols = 128;                          // FP32 accumulator columns (= kBN)
constexpr uint32_t kSpinLimit = 1u << 22;

template <int NP>
struct GemmCfg {
  static constexpr int kStages = NP == 2 ? 3 : 2;
  static constexpr int kStageBytes = 2 * NP * kTileBytes;
  static constexpr int kSmemBytes = kStages * kStageBytes + 1024 /*alignment*/ + 256 /*barriers*/;
  static constexpr int kProducts = NP == 2 ? 3 : 6;
};
// (A piece, B piece) of product t, in issue order: (0,0) (0,1) (1,0) (1,1) (0,2) (2,0)
__host__ __device__ constexpr int prod_a(int t) { return t == 2 || t == 3 ? 1 : (t == 5 ? 2 : 0); }
__host__ __device__ constexpr int prod_b(int t) { return t == 1 || t == 3 ? 1 : (t == 4 ? 2 : 0); }

struct TmapSet {
  CUtensorMap a[kMaxPieces], b[kMaxPieces];
};

struct GemmArgs {
  int M, N, Kp;
  int a_batch_rows, b_batch_rows;   // row offset of batch z in the A / B tensors
  long long c_batch;                // element offset of batch z in C
  float *C;                         // FP32 output, or
  __nv_bfloat16 *Cp[kMaxPieces];    // split output
  long long ldc;
  long long grp_rows, grp_stride, row0;   // out row = (m / grp_rows) * grp_stride + m % grp_rows + row0
  long long grp_cols, gcol_stride, col0;  // out column = (n / grp_cols) * gcol_stride + n % grp_cols + col0
  int *err;
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
  const uint32_t a = smem_u32(bar);
  for (uint32_t it = 0; it < kSpinLimit; ++it) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.b32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, uint64_t *bar, int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
          smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(x), "r"(y)
      : "memory");
}

// shared-memory matrix descriptor: K-major operand tile, 128-byte swizzle,
// 8-row core-matrix groups 1024 bytes apart
__device__ __forceinline__ uint64_t smem_desc(const void *tile) {
  const uint32_t a = smem_u32(tile);
  uint64_t d = (uint64_t)((a >> 4) & 0x3FFFu);   // start address
  d |= (uint64_t)1 << 16;                        // leading byte offset (unused with this swizzle)
  d |= (uint64_t)(1024 >> 4) << 32;              // stride byte offset
  d |= (uint64_t)1 << 46;                        // descriptor version
  d |= (uint64_t)2 << 61;                        // 128-byte swizzle
  return d;
}

// instruction descriptor, kind::f16: FP32 accumulator, BF16 A and B, both K-major
constexpr uint32_t make_idesc(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(da), "l"(db), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void umma_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

template <int NP>
__global__ void __launch_bounds__(128, 1) gemm_split_kernel(const __grid_constant__ TmapSet maps, GemmArgs g) {
  using Cfg = GemmCfg<NP>;
  constexpr int kStages = Cfg::kStages, kStageBytes = Cfg::kStageBytes;
  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t *full = reinterpret_cast<uint64_t *>(smem + kStages * kStageBytes);
  uint64_t *empty = full + kStages;
  uint64_t *done = empty + kStages;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(done + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int n0 = blockIdx.x * kBN, m0 = blockIdx.y * kBM, z = blockIdx.z;
  const int nk = g.Kp / kBK;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    __syncwarp();   // tcgen05.alloc is warp-collective
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0 && lane == 0) {
    // producer: stage s holds A pieces 0..NP-1 then B pieces 0..NP-1
    int issued = 0;
    for (int k = 0; k < nk; ++k) {
      const int s = k % kStages;
      const uint32_t ph = (uint32_t)(k / kStages) & 1u;
      if (!mbar_wait(&empty[s], ph ^ 1u)) {
        atomicExch(g.err, 1);
        break;
      }
      uint8_t *st = smem + s * kStageBytes;
      mbar_expect_tx(&full[s], kStageBytes);
      const int ya = z * g.a_batch_rows + m0, yb = z * g.b_batch_rows + n0;
#pragma unroll
      for (int q = 0; q < NP; ++q) {
        tma_load_2d(st + q * kTileBytes, &maps.a[q], &full[s], k * kBK, ya);
        tma_load_2d(st + (NP + q) * kTileBytes, &maps.b[q], &full[s], k * kBK, yb);
      }
      ++issued;
    }
    // loads still in flight land before the CTA releases its shared memory:
    // wait (bounded) for the full barrier of the last issued step of each stage
    for (int k = issued - kStages; k < issued; ++k) {
      if (k < 0) continue;
      mbar_wait(&full[k % kStages], (uint32_t)(k / kStages) & 1u);
    }
  } else if (warp == 1 && lane == 0) {
    // MMA issuer
    constexpr uint32_t idesc = make_idesc(kBM, kBN);
    for (int k = 0; k < nk; ++k) {
      const int s = k % kStages;
      const uint32_t ph = (uint32_t)(k / kStages) & 1u;
      if (!mbar_wait(&full[s], ph)) {
        atomicExch(g.err, 2);
        break;
      }
      tc_fence_after();
      const uint8_t *st = smem + s * kStageBytes;
      uint64_t da[NP], db[NP];
#pragma unroll
      for (int q = 0; q < NP; ++q) {
        da[q] = smem_desc(st + q * kTileBytes);
        db[q] = smem_desc(st + (NP + q) * kTileBytes);
      }
#pragma unroll
      for (int kk = 0; kk < kBK / 16; ++kk) {
        const uint64_t off = (uint64_t)(kk * 16 * 2) >> 4;   // K step of 16 BF16 = 32 bytes
#pragma unroll
        for (int t = 0; t < Cfg::kProducts; ++t)
          umma_bf16(tmem, da[prod_a(t)] + off, db[prod_b(t)] + off, idesc, (k | kk | t) != 0);
      }
      umma_commit(&empty[s]);
    }
    umma_commit(done);
  }
  __syncwarp();

  // epilogue: warp w owns accumulator lanes (tile rows) 32w .. 32w + 31
  const bool ready = mbar_wait(done, 0);
  if (!ready && lane == 0) atomicExch(g.err, 3);
  tc_fence_after();
  const int row = m0 + warp * 32 + lane;
  long long orow = 0;
  if (row < g.M) orow = (long long)(row / g.grp_rows) * g.grp_stride + row % g.grp_rows + g.row0;
  const long long cbase = (long long)z * g.c_batch + orow * g.ldc;
#pragma unroll 1
  for (int c0 = 0; c0 < kBN; c0 += 32) {
    uint32_t r[32];
    __syncwarp();   // tcgen05.ld is warp-collective
    tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, r);
    if (!ready || row >= g.M) continue;
    const int ncol = min(32, g.N - (n0 + c0));
    if (ncol <= 0) continue;
#pragma unroll
    for (int j = 0; j < 32; ++j)
      if (j < ncol) {
        const long long nn = n0 + c0 + j;
        const long long oc =
            cbase + (g.grp_cols ? (nn / g.grp_cols) * g.gcol_stride + nn % g.grp_cols + g.col0 : nn);
        const float x = __uint_as_float(r[j]);
        if (g.C) {
          g.C[oc] = x;
        } else {
          __nv_bfloat16 pc[kMaxPieces];
          bf16_pieces(x, NP, pc);
#pragma unroll
          for (int q = 0; q < NP; ++q) g.Cp[q][oc] = pc[q];
        }
      }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
}

// ------------------------------------------------------------ precise mode --
// Expected loss of one tensor-core FP32 result (a 16-wide slab sum), in units
// of half its last place, with its sign, added back to the slab sums.  Measured
// on this part from the mean relative error of 128 x 4096 x K products of
// uniform positive operands (K = 640 and 1216): -1.29e-8 with no
// compensation, +9.2e-9 at 0.5, linear in between, zero at 0.29 (a pure
// truncation of the exact sum would lose 1.0).
constexpr float kPTruncComp = 0.29f;
// half a unit in the last place of FP32 value `bits`, with its sign: 2^-24
// times its leading power of two (0 for zero and subnormals)
__device__ __forceinline__ float half_ulp_signed(uint32_t bits) {
  return __uint_as_float(bits & 0xff800000u) * 5.9604644775390625e-8f;
}

// Three pieces per operand, eight products (p0q0 + p0q1 + p1q0 + p1q1 + p0q2
// + p2q0 + p1q2 + p2q1), and no long FP32 running sum in the tensor cores:
// the p0q0 product of every 16-wide K slab (one MMA) goes to a fresh
// tensor-memory accumulator, the seven smaller products of a 64-wide K step
// to one more; after every step the accumulator warps add the four slab sums
// in FP32 and enter the step total into a compensated FP32 pair (hi + lo,
// Knuth's error-free TwoSum), the corrections into the low part.  The tensor
// cores round each slab's main sum once, toward zero, instead of carrying a
// 640-term FP32 running sum, which is what limits a plain FP32-accumulated
// product on inputs with strong cancellation.  That rounding loses on average
// a fixed fraction of a unit in the last place of the result (with its sign,
// kPTruncComp): the accumulator warps add it back into the low part, which
// removes the systematic shrinkage that squared quantities (MP2 pair
// energies) would otherwise accumulate.  The FP32 pipe (64x the FP64 rate on
// this part) keeps up with the tensor cores.
// Warps: 0 TMA producer, 1 MMA issuer, 2-9 accumulators / epilogue (warp w
// reads tensor-memory lanes 32 (w % 4) .. + 31, columns 24 ((w - 2) / 4) ..
// + 23 of each accumulator).  Tiles 128 x 48; persistent CTAs walk the N
// tiles; accumulator buffers are double-buffered across steps.
constexpr int kPBN = 48, kPStages = 3, kPAccWarps = 8, kPColsPerWarp = kPBN / 2;
constexpr int kPTileA = 128 * kBK * 2, kPTileB = kPBN * kBK * 2;
constexpr int kPStageBytes = 3 * kPTileA + 3 * kPTileB;
constexpr int kPBufCols = 5 * kPBN;                 // 4 slab accumulators + 1 correction accumulator
constexpr int kPTmemCols = 512;
constexpr int kPThreads = 32 * (2 + kPAccWarps);
constexpr int kPSmemBytes = kPStages * kPStageBytes + 1024 + 256;

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t *r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}

__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t *r) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
}

// hi + lo += x without rounding error in the sum (TwoSum), the error kept in lo
__device__ __forceinline__ void two_sum_acc(float &hi, float &lo, float x) {
  const float s = hi + x;
  const float bb = s - hi;
  const float e = (hi - (s - bb)) + (x - bb);
  hi = s;
  lo += e;
}

__global__ void __launch_bounds__(kPThreads, 1) gemm_precise_kernel(const __grid_constant__ TmapSet maps, GemmArgs g) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t *full = reinterpret_cast<uint64_t *>(smem + kPStages * kPStageBytes);
  uint64_t *empty = full + kPStages;
  uint64_t *acc_full = empty + kPStages;
  uint64_t *acc_free = acc_full + 2;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(acc_free + 2);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.y * kBM, z = blockIdx.z;
  const int nk = g.Kp / kBK;
  const int ntiles = (g.N + kPBN - 1) / kPBN;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kPStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&acc_full[b], 1);
      mbar_init(&acc_free[b], kPAccWarps);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    __syncwarp();
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(kPTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      long long gs = 0, issued = 0;
      bool ok = true;
      for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
        const int n0 = t * kPBN;
        for (int k = 0; k < nk; ++k, ++gs) {
          const int s = (int)(gs % kPStages);
          if (!mbar_wait(&empty[s], (uint32_t)((gs / kPStages) & 1) ^ 1u)) {
            atomicExch(g.err, 11);
            ok = false;
            break;
          }
          uint8_t *st = smem + s * kPStageBytes;
          mbar_expect_tx(&full[s], kPStageBytes);
          const int ya = z * g.a_batch_rows + m0, yb = z * g.b_batch_rows + n0;
#pragma unroll
          for (int q = 0; q < 3; ++q) {
            tma_load_2d(st + q * kPTileA, &maps.a[q], &full[s], k * kBK, ya);
            tma_load_2d(st + 3 * kPTileA + q * kPTileB, &maps.b[q], &full[s], k * kBK, yb);
          }
          ++issued;
        }
      }
      for (long long k = issued - kPStages; k < issued; ++k) {
        if (k < 0) continue;
        mbar_wait(&full[k % kPStages], (uint32_t)((k / kPStages) & 1));
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      constexpr uint32_t idesc = make_idesc(kBM, kPBN);
      long long gs = 0;
      bool ok = true;
      for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
        for (int k = 0; k < nk; ++k, ++gs) {
          const int s = (int)(gs % kPStages), b = (int)(gs & 1);
          if (gs >= 2 && !mbar_wait(&acc_free[b], (uint32_t)(((gs - 2) >> 1) & 1))) {
            atomicExch(g.err, 12);
            ok = false;
            break;
          }
          if (!mbar_wait(&full[s], (uint32_t)((gs / kPStages) & 1))) {
            atomicExch(g.err, 13);
            ok = false;
            break;
          }
          tc_fence_after();
          const uint8_t *st = smem + s * kPStageBytes;
          uint64_t da[3], db[3];
#pragma unroll
          for (int q = 0; q < 3; ++q) {
            da[q] = smem_desc(st + q * kPTileA);
            db[q] = smem_desc(st + 3 * kPTileA + q * kPTileB);
          }
          const uint32_t tb = tmem + (uint32_t)(b * kPBufCols);
#pragma unroll
          for (int kk = 0; kk < kBK / 16; ++kk) {
            const uint64_t off = (uint64_t)(kk * 16 * 2) >> 4;
            // main product: a fresh accumulator per 16-wide slab
            umma_bf16(tb + (uint32_t)(kk * kPBN), da[0] + off, db[0] + off, idesc, 0u);
#pragma unroll
            for (int p = 1; p < 8; ++p) {
              const int qa = p == 2 || p == 3 || p == 7 ? 1 : (p == 5 || p == 6 ? 2 : 0);
              const int qb = p == 1 || p == 3 || p == 6 ? 1 : (p == 4 || p == 7 ? 2 : 0);
              umma_bf16(tb + (uint32_t)(4 * kPBN), da[qa] + off, db[qb] + off, idesc, (kk | (p - 1)) != 0);
            }
          }
          umma_commit(&empty[s]);
          umma_commit(&acc_full[b]);
        }
      }
    }
  } else {
    // accumulator warps: lane quarter wq, columns c0 .. c0 + 23 of every accumulator
    const int wq = warp & 3, c0 = ((warp - 2) >> 2) * kPColsPerWarp;
    const int row = m0 + wq * 32 + lane;
    long long orow = 0;
    if (row < g.M) orow = (long long)(row / g.grp_rows) * g.grp_stride + row % g.grp_rows + g.row0;
    const long long cbase = (long long)z * g.c_batch + orow * g.ldc;
    long long gs = 0;
    bool ok = true;
    for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
      const int n0 = t * kPBN;
      float hi[kPColsPerWarp], lo[kPColsPerWarp];
#pragma unroll
      for (int j = 0; j < kPColsPerWarp; ++j) hi[j] = lo[j] = 0.f;
      for (int k = 0; k < nk; ++k, ++gs) {
        const int b = (int)(gs & 1);
        const bool got = mbar_wait(&acc_full[b], (uint32_t)((gs >> 1) & 1));
        if (!got) {
          if (lane == 0) atomicExch(g.err, 14);
          ok = false;
          break;
        }
        tc_fence_after();
        __syncwarp();
        const uint32_t ta = tmem + ((uint32_t)(wq * 32) << 16) + (uint32_t)(b * kPBufCols + c0);
        // the step's four slab sums (each truncated once by the tensor cores)
        // add in FP32, round to nearest; the step total enters the running
        // pair by TwoSum; the correction products and the expected
        // truncation losses of the slab sums go to the low part
        float stepsum[kPColsPerWarp], trunc[kPColsPerWarp];
        uint32_t r[kPColsPerWarp];
#pragma unroll
        for (int c = 0; c < 5; ++c) {
          // loads at column offsets aligned to their width
          if (c0 == 0) {
            tmem_ld16(ta + (uint32_t)(c * kPBN), r);
            tmem_ld8(ta + (uint32_t)(c * kPBN + 16), r + 16);
          } else {
            tmem_ld8(ta + (uint32_t)(c * kPBN), r);
            tmem_ld16(ta + (uint32_t)(c * kPBN + 8), r + 8);
          }
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
          if (c == 0) {
#pragma unroll
            for (int j = 0; j < kPColsPerWarp; ++j) {
              stepsum[j] = __uint_as_float(r[j]);
              trunc[j] = half_ulp_signed(r[j]);
            }
          } else if (c < 4) {
#pragma unroll
            for (int j = 0; j < kPColsPerWarp; ++j) {
              stepsum[j] += __uint_as_float(r[j]);
              trunc[j] += half_ulp_signed(r[j]);
            }
          } else {
#pragma unroll
            for (int j = 0; j < kPColsPerWarp; ++j) {
              two_sum_acc(hi[j], lo[j], stepsum[j]);
              lo[j] += __uint_as_float(r[j]) + kPTruncComp * trunc[j];
            }
          }
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&acc_free[b]);
      }
      if (!ok || row >= g.M) continue;
#pragma unroll
      for (int j = 0; j < kPColsPerWarp; ++j) {
        const long long nn = n0 + c0 + j;
        if (nn >= g.N) continue;
        const long long oc =
            cbase + (g.grp_cols ? (nn / g.grp_cols) * g.gcol_stride + nn % g.grp_cols + g.col0 : nn);
        // FP32 arithmetic only (the FP64 pipe of this part is 1/64 of the FP32 one)
        if (g.C) {
          g.C[oc] = hi[j] + lo[j];
        } else {
          __nv_bfloat16 pc[kMaxPieces];
          bf16_pieces_pair(hi[j], lo[j], 3, pc);
#pragma unroll
          for (int q = 0; q < 3; ++q) g.Cp[q][oc] = pc[q];
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    __syncwarp();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kPTmemCols) : "memory");
  }
}

// FP32 / FP64 row-major [rows][cols] -> np BF16 pieces [rows][ldo] (columns
// >= cols are left as they are: the caller clears the padding once)
template <typename T>
__global__ void split_bf16_kernel(const T *__restrict__ src, long long rows, int cols, long long lds, int np,
                                  __nv_bfloat16 *o0, __nv_bfloat16 *o1, __nv_bfloat16 *o2, long long ldo) {
  const long long tot = rows * cols;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < tot; t += (long long)gridDim.x * blockDim.x) {
    const long long r = t / cols;
    const int c = (int)(t % cols);
    __nv_bfloat16 pc[kMaxPieces] = {};
    bf16_pieces((double)src[r * lds + c], np, pc);
    o0[r * ldo + c] = pc[0];
    o1[r * ldo + c] = pc[1];
    if (np > 2) o2[r * ldo + c] = pc[2];
  }
}

std::once_flag g_encode_once;
PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

bool tensor_map(CUtensorMap *m, const void *base, long long rows, int Kp, int box_rows = 128) {
  std::call_once(g_encode_once, [] {
    cudaDriverEntryPointQueryResult q;
    void *fn = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  });
  if (!g_encode) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)Kp, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)Kp * 2};
  const cuuint32_t box[2] = {(cuuint32_t)kBK, (cuuint32_t)box_rows};
  const cuuint32_t estr[2] = {1u, 1u};
  return g_encode(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int NP>
cudaError_t launch_gemm_np(const TmapSet &maps, const GemmArgs &g, unsigned nt, unsigned mt, unsigned batch,
                           cudaStream_t s) {
  static PerDeviceLevel attr;
  const cudaError_t e = attr.raise(1, [] {
    return cudaFuncSetAttribute(gemm_split_kernel<NP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                GemmCfg<NP>::kSmemBytes);
  });
  if (e != cudaSuccess) return e;
  gemm_split_kernel<NP><<<dim3(nt, mt, batch), 128, GemmCfg<NP>::kSmemBytes, s>>>(maps, g);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_gemm_split(const Bf16Split &A, long long a_rows, const Bf16Split &B, long long b_rows, int Kp,
                              int M, int N, int batch, int a_batch_rows, int b_batch_rows, int np,
                              const GemmOut &out, int *derr, cudaStream_t s) {
  if (Kp <= 0 || Kp % kBK || M <= 0 || N <= 0 || batch <= 0 || np < 2 || np > kMaxPieces)
    return cudaErrorInvalidValue;
  uintptr_t bits = 0;
  for (int q = 0; q < np; ++q) {
    if (!A.p[q] || !B.p[q] || (!out.C && !out.Cp[q])) return cudaErrorInvalidValue;
    bits |= reinterpret_cast<uintptr_t>(A.p[q]) | reinterpret_cast<uintptr_t>(B.p[q]);
  }
  if (bits & 15u) return cudaErrorMisalignedAddress;
  const long long nt = (N + kBN - 1) / kBN, mt = (M + kBM - 1) / kBM;
  if (nt > 0x7fffffffLL || mt > 65535 || batch > 65535) return cudaErrorInvalidConfiguration;
  TmapSet maps;
  memset(&maps, 0, sizeof(maps));
  for (int q = 0; q < np; ++q)
    if (!tensor_map(&maps.a[q], A.p[q], a_rows, Kp) || !tensor_map(&maps.b[q], B.p[q], b_rows, Kp))
      return cudaErrorInvalidValue;
  GemmArgs g{};
  g.M = M;
  g.N = N;
  g.Kp = Kp;
  g.a_batch_rows = a_batch_rows;
  g.b_batch_rows = b_batch_rows;
  g.c_batch = out.c_batch;
  g.C = out.C;
  for (int q = 0; q < kMaxPieces; ++q) g.Cp[q] = out.Cp[q];
  g.ldc = out.ldc;
  g.grp_rows = out.grp_rows > 0 ? out.grp_rows : (long long)M;
  g.grp_stride = out.grp_rows > 0 ? out.grp_stride : 0;
  g.row0 = out.row0;
  g.grp_cols = out.grp_cols;
  g.gcol_stride = out.gcol_stride;
  g.col0 = out.col0;
  g.err = derr;
  const cudaError_t e = np == 2 ? launch_gemm_np<2>(maps, g, (unsigned)nt, (unsigned)mt, (unsigned)batch, s)
                                : launch_gemm_np<3>(maps, g, (unsigned)nt, (unsigned)mt, (unsigned)batch, s);
  count_launches(1);
  return e;
}

cudaError_t launch_gemm_precise(const Bf16Split &A, long long a_rows, const Bf16Split &B, long long b_rows, int Kp,
                                int M, int N, int batch, int a_batch_rows, int b_batch_rows, const GemmOut &out,
                                int *derr, cudaStream_t s) {
  if (Kp <= 0 || Kp % kBK || M <= 0 || N <= 0 || batch <= 0) return cudaErrorInvalidValue;
  uintptr_t bits = 0;
  for (int q = 0; q < 3; ++q) {
    if (!A.p[q] || !B.p[q] || (!out.C && !out.Cp[q])) return cudaErrorInvalidValue;
    bits |= reinterpret_cast<uintptr_t>(A.p[q]) | reinterpret_cast<uintptr_t>(B.p[q]);
  }
  if (bits & 15u) return cudaErrorMisalignedAddress;
  const long long nt = (N + kPBN - 1) / kPBN, mt = (M + kBM - 1) / kBM;
  if (mt > 65535 || batch > 65535) return cudaErrorInvalidConfiguration;
  TmapSet maps;
  memset(&maps, 0, sizeof(maps));
  for (int q = 0; q < 3; ++q)
    if (!tensor_map(&maps.a[q], A.p[q], a_rows, Kp, 128) || !tensor_map(&maps.b[q], B.p[q], b_rows, Kp, kPBN))
      return cudaErrorInvalidValue;
  GemmArgs g{};
  g.M = M;
  g.N = N;
  g.Kp = Kp;
  g.a_batch_rows = a_batch_rows;
  g.b_batch_rows = b_batch_rows;
  g.c_batch = out.c_batch;
  g.C = out.C;
  for (int q = 0; q < kMaxPieces; ++q) g.Cp[q] = out.Cp[q];
  g.ldc = out.ldc;
  g.grp_rows = out.grp_rows > 0 ? out.grp_rows : (long long)M;
  g.grp_stride = out.grp_rows > 0 ? out.grp_stride : 0;
  g.row0 = out.row0;
  g.grp_cols = out.grp_cols;
  g.gcol_stride = out.gcol_stride;
  g.col0 = out.col0;
  g.err = derr;
  static PerDeviceLevel attr;
  const cudaError_t e = attr.raise(1, [] {
    return cudaFuncSetAttribute(gemm_precise_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kPSmemBytes);
  });
  if (e != cudaSuccess) return e;
  // persistent CTAs: one wave over the SMs (one CTA fits an SM), split over (M tiles x batches)
  long long per = (152LL + mt * batch - 1) / (mt * batch);
  const unsigned gx = (unsigned)std::max<long long>(1, std::min<long long>(nt, per));
  gemm_precise_kernel<<<dim3(gx, (unsigned)mt, (unsigned)batch), kPThreads, kPSmemBytes, s>>>(maps, g);
  count_launches(1);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_split_bf16(const T *src, long long rows, int cols, long long lds, int np, __nv_bfloat16 *const *out,
                              long long ldo, cudaStream_t s) {
  const long long tot = rows * cols;
  if (tot <= 0) return cudaSuccess;
  if (np < 2 || np > kMaxPieces) return cudaErrorInvalidValue;
  const long long blocks = std::min<long long>((tot + 255) / 256, 152LL * 32);
  split_bf16_kernel<T><<<(unsigned)blocks, 256, 0, s>>>(src, rows, cols, lds, np, out[0], out[1],
                                                        np > 2 ? out[2] : nullptr, ldo);
  count_launches(1);
  return cudaGetLastError();
}

template cudaError_t launch_split_bf16<float>(const float *, long long, int, long long, int, __nv_bfloat16 *const *,
                                              long long, cudaStream_t);
template cudaError_t launch_split_bf16<double>(const double *, long long, int, long long, int,
                                               __nv_bfloat16 *const *, long long, cudaStream_t);

}  // namespace lgb
