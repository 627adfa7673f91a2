// 3-term split-BF16 GEMM on the fifth-generation tensor cores (tcgen05).
//
// C[m][n] = sum_k A[m][k] B[n][k] with A = Ah + Al and B = Bh + Bl, each term a
// BF16 array (K contiguous, K padded to a multiple of 64 with zeros):
//   C ~= Ah Bh + Ah Bl + Al Bh,    FP32 accumulation in tensor memory.
// The dropped Al Bl term and the two-term representation leave a relative
// error of about 2^-16 per product.
//
// One CTA computes one 128 x 128 tile of C with four warps:
//   warp 0 lane 0  TMA producer: per 64-wide K step, the four operand tiles
//                  (Ah, Al: 128 x 64; Bh, Bl: 128 x 64, 16 KB each) into a
//                  3-stage ring of 128-byte-swizzled shared-memory buffers;
//   warp 1 lane 0  MMA issuer: 3 x 4 tcgen05.mma (M 128, N 128, K 16) per step
//                  into a 128-column FP32 accumulator in tensor memory; each
//                  step's tcgen05.commit releases its ring slot;
//   all 4 warps    epilogue: tcgen05.ld of their 32 accumulator lanes (rows),
//                  FP32 or split-BF16 (hi, lo) stores with an optional grouped
//                  row remap.
// Every wait on an mbarrier is bounded; a wait that runs out sets *err and the
// CTA skips to its clean-up (TMEM is always released).
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <mutex>

#include "kernels.cuh"

namespace lgb {
namespace {

constexpr int kBM = 128, kBN = 128, kBK = 64, kStages = 3;
constexpr int kTileBytes = 128 * kBK * 2;               // one operand tile, 16 KB
constexpr int kStageBytes = 4 * kTileBytes;             // Ah, Al, Bh, Bl
constexpr int kTmemCols = 128;                          // FP32 accumulator columns (= kBN)
constexpr int kSmemBytes = kStages * kStageBytes + 1024 /*alignment*/ + 256 /*barriers*/;
constexpr uint32_t kSpinLimit = 1u << 22;

struct GemmArgs {
  int M, N, Kp;
  int a_batch_rows, b_batch_rows;   // row offset of batch z in the A / B tensors
  long long c_batch;                // element offset of batch z in C
  float *C;                         // FP32 output, or
  __nv_bfloat16 *Ch, *Cl;           // split output (hi, lo)
  long long ldc;
  long long grp_rows, grp_stride, row0;   // out row = (m / grp_rows) * grp_stride + m % grp_rows + row0
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

__global__ void __launch_bounds__(128, 1)
    gemm_bf16x3_kernel(const __grid_constant__ CUtensorMap tAh, const __grid_constant__ CUtensorMap tAl,
                       const __grid_constant__ CUtensorMap tBh, const __grid_constant__ CUtensorMap tBl,
                       GemmArgs g) {
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
    // producer
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
      tma_load_2d(st, &tAh, &full[s], k * kBK, ya);
      tma_load_2d(st + kTileBytes, &tAl, &full[s], k * kBK, ya);
      tma_load_2d(st + 2 * kTileBytes, &tBh, &full[s], k * kBK, yb);
      tma_load_2d(st + 3 * kTileBytes, &tBl, &full[s], k * kBK, yb);
      ++issued;
    }
    // loads still in flight land before the CTA releases its shared memory:
    // wait (bounded) for the full barrier of the last issued step of each slot
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
      const uint64_t dAh = smem_desc(st), dAl = smem_desc(st + kTileBytes);
      const uint64_t dBh = smem_desc(st + 2 * kTileBytes), dBl = smem_desc(st + 3 * kTileBytes);
#pragma unroll
      for (int kk = 0; kk < kBK / 16; ++kk) {
        const uint64_t off = (uint64_t)(kk * 16 * 2) >> 4;   // K step of 16 BF16 = 32 bytes
        umma_bf16(tmem, dAh + off, dBh + off, idesc, (k | kk) != 0);
        umma_bf16(tmem, dAh + off, dBl + off, idesc, 1u);
        umma_bf16(tmem, dAl + off, dBh + off, idesc, 1u);
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
    if (g.C) {
      float *dst = g.C + cbase + n0 + c0;
#pragma unroll
      for (int j = 0; j < 32; ++j)
        if (j < ncol) dst[j] = __uint_as_float(r[j]);
    } else {
      __nv_bfloat16 *dh = g.Ch + cbase + n0 + c0, *dl = g.Cl + cbase + n0 + c0;
#pragma unroll
      for (int j = 0; j < 32; ++j)
        if (j < ncol) {
          const float x = __uint_as_float(r[j]);
          const __nv_bfloat16 h = __float2bfloat16_rn(x);
          dh[j] = h;
          dl[j] = __float2bfloat16_rn(x - __bfloat162float(h));
        }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
}

// FP32 / FP64 row-major [rows][cols] -> BF16 hi / lo [rows][ldo] (columns
// >= cols are left as they are: the caller clears the padding once)
template <typename T>
__global__ void split_bf16_kernel(const T *__restrict__ src, long long rows, int cols, long long lds,
                                  __nv_bfloat16 *hi, __nv_bfloat16 *lo, long long ldo) {
  const long long tot = rows * cols;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < tot; t += (long long)gridDim.x * blockDim.x) {
    const long long r = t / cols;
    const int c = (int)(t % cols);
    const double x = (double)src[r * lds + c];
    const __nv_bfloat16 h = __float2bfloat16_rn((float)x);
    hi[r * ldo + c] = h;
    lo[r * ldo + c] = __float2bfloat16_rn((float)(x - (double)__bfloat162float(h)));
  }
}

std::once_flag g_encode_once;
PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

bool tensor_map(CUtensorMap *m, const void *base, long long rows, int Kp) {
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
  const cuuint32_t box[2] = {(cuuint32_t)kBK, 128u};
  const cuuint32_t estr[2] = {1u, 1u};
  return g_encode(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

cudaError_t launch_gemm_bf16x3(const Bf16Split &A, long long a_rows, const Bf16Split &B, long long b_rows, int Kp,
                               int M, int N, int batch, int a_batch_rows, int b_batch_rows, const GemmOut &out,
                               int *derr, cudaStream_t s) {
  if (Kp <= 0 || Kp % kBK || M <= 0 || N <= 0 || batch <= 0) return cudaErrorInvalidValue;
  if ((reinterpret_cast<uintptr_t>(A.hi) | reinterpret_cast<uintptr_t>(A.lo) | reinterpret_cast<uintptr_t>(B.hi) |
       reinterpret_cast<uintptr_t>(B.lo)) & 15u)
    return cudaErrorMisalignedAddress;
  const long long nt = (N + kBN - 1) / kBN, mt = (M + kBM - 1) / kBM;
  if (nt > 0x7fffffffLL || mt > 65535 || batch > 65535) return cudaErrorInvalidConfiguration;
  CUtensorMap tAh, tAl, tBh, tBl;
  if (!tensor_map(&tAh, A.hi, a_rows, Kp) || !tensor_map(&tAl, A.lo, a_rows, Kp) ||
      !tensor_map(&tBh, B.hi, b_rows, Kp) || !tensor_map(&tBl, B.lo, b_rows, Kp))
    return cudaErrorInvalidValue;
  static bool attr = false;
  if (!attr) {
    const cudaError_t e = cudaFuncSetAttribute(gemm_bf16x3_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               kSmemBytes);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  GemmArgs g{};
  g.M = M;
  g.N = N;
  g.Kp = Kp;
  g.a_batch_rows = a_batch_rows;
  g.b_batch_rows = b_batch_rows;
  g.c_batch = out.c_batch;
  g.C = out.C;
  g.Ch = out.Ch;
  g.Cl = out.Cl;
  g.ldc = out.ldc;
  g.grp_rows = out.grp_rows > 0 ? out.grp_rows : (long long)M;
  g.grp_stride = out.grp_rows > 0 ? out.grp_stride : 0;
  g.row0 = out.row0;
  g.err = derr;
  gemm_bf16x3_kernel<<<dim3((unsigned)nt, (unsigned)mt, (unsigned)batch), 128, kSmemBytes, s>>>(tAh, tAl, tBh, tBl,
                                                                                             g);
  count_launches(1);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_split_bf16(const T *src, long long rows, int cols, long long lds, __nv_bfloat16 *hi,
                              __nv_bfloat16 *lo, long long ldo, cudaStream_t s) {
  const long long tot = rows * cols;
  if (tot <= 0) return cudaSuccess;
  const long long blocks = std::min<long long>((tot + 255) / 256, 152LL * 32);
  split_bf16_kernel<T><<<(unsigned)blocks, 256, 0, s>>>(src, rows, cols, lds, hi, lo, ldo);
  count_launches(1);
  return cudaGetLastError();
}

template cudaError_t launch_split_bf16<float>(const float *, long long, int, long long, __nv_bfloat16 *,
                                              __nv_bfloat16 *, long long, cudaStream_t);
template cudaError_t launch_split_bf16<double>(const double *, long long, int, long long, __nv_bfloat16 *,
                                               __nv_bfloat16 *, long long, cudaStream_t);

}  // namespace lgb
