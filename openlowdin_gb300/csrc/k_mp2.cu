// MP2 transform helpers: coefficient preparation, unpacking of the packed
// ket-pair columns into a full (lam, sig) square, and the pair-energy sum.
#include <type_traits>
#include <algorithm>

#include "kernels.cuh"

namespace lgb {
namespace {

__global__ void mp2_coeffs_kernel(const double *__restrict__ C, const double *__restrict__ norma, int n, int n_frozen,
                                  int n_occ, double *Co, double *Cv, float *Co32, float *Cv32) {
  const int o = n_occ - n_frozen, v = n - n_occ;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)n * n) return;
  const int mu = (int)(t / n), p = (int)(t % n);   // output row mu, orbital column p
  if (p < n_frozen) return;
  const double x = C[(size_t)p * n + mu] * norma[mu];
  if (p < n_occ) {
    const size_t k = (size_t)mu * o + (p - n_frozen);
    if (Co) Co[k] = x;
    if (Co32) Co32[k] = (float)x;
  } else {
    const size_t k = (size_t)mu * v + (p - n_occ);
    if (Cv) Cv[k] = x;
    if (Cv32) Cv32[k] = (float)x;
  }
}

template <typename T>
__global__ void mp2_unpack_kernel(const T *__restrict__ Y, const unsigned *__restrict__ colpair, long long ncols,
                                  int n, int v, T *Z) {
  for (long long col = blockIdx.x; col < ncols; col += gridDim.x) {
    const unsigned cp = __ldg(colpair + col);
    const int lam = cp & 0xffff, sig = (cp >> 16) & 0x7fff;
    const bool two = cp >> 31;
    const T *y = Y + col * v;
    T *z1 = Z + ((size_t)lam * n + sig) * v;
    T *z2 = Z + ((size_t)sig * n + lam) * v;
    for (int a = threadIdx.x; a < v; a += blockDim.x) {
      const T x = y[a];
      z1[a] = x;
      if (two) z2[a] = x;
    }
  }
}

// 32 x 32 (b, a) tiles of one j; the transposed tile comes through shared memory
template <typename T>
__global__ void __launch_bounds__(256) mp2_energy_kernel(const T *__restrict__ M, int v, double ei,
                                                         const double *__restrict__ eo,
                                                         const double *__restrict__ ev, double cut, double *e2) {
  __shared__ T tr[32][33];
  __shared__ double red[8];
  const int j = blockIdx.z;
  const int a0 = blockIdx.x * 32, b0 = blockIdx.y * 32;
  const T *Mj = M + (size_t)j * v * v;
  // tr[x][y] = M[j][a0 + y][b0 + x]
  for (int y = threadIdx.y; y < 32; y += 8) {
    const int a = a0 + y, b = b0 + threadIdx.x;
    tr[threadIdx.x][y] = (a < v && b < v) ? Mj[(size_t)a * v + b] : T(0);
  }
  __syncthreads();
  const double eij = ei + eo[j];
  double acc = 0.0;
  if constexpr (std::is_same<T, float>::value) {
    // split-BF16 path: M is FP32, so each term is formed in FP32 (no FP64
    // division per element, which dominated this kernel on the FP64 pipe);
    // a thread's four terms are summed in FP32 and everything after in FP64
    const float eijf = (float)eij, cutf = (float)cut;
    float part = 0.f;
    for (int y = threadIdx.y; y < 32; y += 8) {
      const int b = b0 + y, a = a0 + threadIdx.x;
      if (a < v && b < v) {
        float x = Mj[(size_t)b * v + a];
        float t = tr[y][threadIdx.x];
        if (!(fabsf(x) > cutf)) x = 0.f;
        if (!(fabsf(t) > cutf)) t = 0.f;
        part += x * (2.f * x - t) / (eijf - (float)ev[a] - (float)ev[b]);
      }
    }
    acc = part;
  } else {
    for (int y = threadIdx.y; y < 32; y += 8) {
      const int b = b0 + y, a = a0 + threadIdx.x;
      if (a < v && b < v) {
        double x = (double)Mj[(size_t)b * v + a];      // (ia|jb)
        double t = (double)tr[y][threadIdx.x];          // (ib|ja) = M[j][a][b]
        if (!(fabs(x) > cut)) x = 0.0;
        if (!(fabs(t) > cut)) t = 0.0;
        acc += x * (2.0 * x - t) / (eij - ev[a] - ev[b]);
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (threadIdx.x == 0) red[threadIdx.y] = acc;
  __syncthreads();
  if (threadIdx.y == 0 && threadIdx.x == 0) {
    double s = 0;
    for (int k = 0; k < 8; ++k) s += red[k];
    atomicAdd(e2, s);
  }
}

__global__ void mp2_coeffs_bf16_kernel(const double *__restrict__ C, const double *__restrict__ norma, int n,
                                       int n_frozen, int n_occ, int Kp, int np, __nv_bfloat16 *CoT0,
                                       __nv_bfloat16 *CoT1, __nv_bfloat16 *CoT2, __nv_bfloat16 *CvT0,
                                       __nv_bfloat16 *CvT1, __nv_bfloat16 *CvT2) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)n * n) return;
  const int p = (int)(t / n), mu = (int)(t % n);   // orbital row p, function mu
  if (p < n_frozen) return;
  __nv_bfloat16 pc[kMaxPieces];
  bf16_pieces(C[t] * norma[mu], np, pc);
  const bool occ = p < n_occ;
  const size_t k = (size_t)(occ ? p - n_frozen : p - n_occ) * Kp + mu;
  __nv_bfloat16 *dst[kMaxPieces] = {occ ? CoT0 : CvT0, occ ? CoT1 : CvT1, occ ? CoT2 : CvT2};
  for (int q = 0; q < np; ++q) dst[q][k] = pc[q];
}

// block (sig chunk of 16 rows, a): gather the chunk's entries into a shared
// FP32 tile [16][Kp], then write its rows as split BF16 with 16-byte stores
constexpr int kUnpackRows = 16;
__global__ void __launch_bounds__(256) mp2_unpack_csr_kernel(const float *__restrict__ Yp, long long ystride,
                                                             const int *__restrict__ rowptr,
                                                             const int2 *__restrict__ ent, int n, int Kp, int np,
                                                             __nv_bfloat16 *Z0, __nv_bfloat16 *Z1,
                                                             __nv_bfloat16 *Z2) {
  extern __shared__ float tile[];
  const int s0 = blockIdx.x * kUnpackRows, a = blockIdx.y;
  const int s1 = min(s0 + kUnpackRows, n);
  for (int k = threadIdx.x; k < kUnpackRows * Kp; k += blockDim.x) tile[k] = 0.f;
  __syncthreads();
  const float *y = Yp + (size_t)a * ystride;
  for (int e = __ldg(rowptr + s0) + threadIdx.x; e < __ldg(rowptr + s1); e += blockDim.x) {
    const int2 t = __ldg(ent + e);
    const int lam = t.x & 0xffff, sig = t.x >> 16;
    tile[(sig - s0) * Kp + lam] = __ldg(y + t.y);
  }
  __syncthreads();
  __nv_bfloat16 *Z[kMaxPieces] = {Z0, Z1, Z2};
  const int nvec = (s1 - s0) * Kp / 8;   // Kp is a multiple of 64
  for (int k = threadIdx.x; k < nvec; k += blockDim.x) {
    const int r = (k * 8) / Kp, c = (k * 8) % Kp;
    const float *src = tile + r * Kp + c;
    __align__(16) __nv_bfloat16 pv[kMaxPieces][8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      __nv_bfloat16 pc[kMaxPieces] = {};
      bf16_pieces(src[q], np, pc);
#pragma unroll
      for (int j = 0; j < kMaxPieces; ++j) pv[j][q] = pc[j];
    }
    const size_t o = ((size_t)a * Kp + s0 + r) * Kp + c;
    for (int j = 0; j < np; ++j) *reinterpret_cast<uint4 *>(Z[j] + o) = *reinterpret_cast<const uint4 *>(pv[j]);
  }
}

template <typename T>
__global__ void __launch_bounds__(256) mp2_energy_coupling_kernel(const T *__restrict__ M, int vB, int vA, double ei,
                                                                  const double *__restrict__ eo,
                                                                  const double *__restrict__ evA,
                                                                  const double *__restrict__ evB, double cut,
                                                                  double factor, double *e2) {
  __shared__ double red[8];
  const int j = blockIdx.y;
  const T *Mj = M + (size_t)j * vB * vA;
  const double eij = ei + eo[j];
  double acc = 0.0;
  if constexpr (std::is_same<T, float>::value) {
    // FP32 terms (FP32 M), FP64 sums of each thread's short FP32 partials
    const float eijf = (float)eij, cutf = (float)cut;
    float part = 0.f;
    int k = 0;
    for (long long t = (long long)blockIdx.x * 256 + threadIdx.x; t < (long long)vB * vA;
         t += (long long)gridDim.x * 256) {
      const int b = (int)(t / vA), a = (int)(t % vA);
      float x = Mj[t];
      if (!(fabsf(x) > cutf)) x = 0.f;
      part += x * x / (eijf - (float)evA[a] - (float)evB[b]);
      if (++k == 16) {
        acc += part;
        part = 0.f;
        k = 0;
      }
    }
    acc += part;
  } else {
    for (long long t = (long long)blockIdx.x * 256 + threadIdx.x; t < (long long)vB * vA;
         t += (long long)gridDim.x * 256) {
      const int b = (int)(t / vA), a = (int)(t % vA);
      double x = (double)Mj[t];
      if (!(fabs(x) > cut)) x = 0.0;
      acc += x * x / (eij - evA[a] - evB[b]);
    }
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0;
    for (int k = 0; k < 8; ++k) s += red[k];
    atomicAdd(e2, s * factor);
  }
}

__global__ void fill_hash_kernel(float *x, long long n, unsigned seed) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    unsigned h = (unsigned)i * 2654435761u ^ seed;
    h ^= h >> 16;
    h *= 2246822519u;
    h ^= h >> 13;
    x[i] = (float)(h & 0xFFFFFF) * (2.0f / 16777216.0f) - 1.0f;
  }
}

}  // namespace

cudaError_t launch_fill_hash(float *x, long long n, unsigned seed, cudaStream_t s) {
  fill_hash_kernel<<<152 * 8, 256, 0, s>>>(x, n, seed);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_mp2_coeffs_bf16(const double *C, const double *norma, int n, int n_frozen, int n_occ, int Kp,
                                   int np, __nv_bfloat16 *const *CoT, __nv_bfloat16 *const *CvT, cudaStream_t s) {
  if (np < 2 || np > kMaxPieces) return cudaErrorInvalidValue;
  const long long tot = (long long)n * n;
  mp2_coeffs_bf16_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(
      C, norma, n, n_frozen, n_occ, Kp, np, CoT[0], CoT[1], np > 2 ? CoT[2] : nullptr, CvT[0], CvT[1],
      np > 2 ? CvT[2] : nullptr);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_mp2_unpack_csr(const float *Yp, long long ystride, const int *rowptr, const int2 *ent, int n,
                                  int Kp, int v, int np, __nv_bfloat16 *const *Z, cudaStream_t s) {
  if (Kp % 64 || v <= 0 || v > 65535 || np < 2 || np > kMaxPieces) return cudaErrorInvalidValue;
  const size_t smem = (size_t)kUnpackRows * Kp * sizeof(float);
  static PerDeviceLevel attr;   // per device: the largest Kp set up so far
  if (smem > 48 * 1024) {
    const cudaError_t e = attr.raise(Kp, [smem] {
      return cudaFuncSetAttribute(mp2_unpack_csr_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    });
    if (e != cudaSuccess) return e;
  }
  const dim3 grid((unsigned)((n + kUnpackRows - 1) / kUnpackRows), (unsigned)v);
  mp2_unpack_csr_kernel<<<grid, 256, smem, s>>>(Yp, ystride, rowptr, ent, n, Kp, np, Z[0], Z[1],
                                                 np > 2 ? Z[2] : nullptr);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_mp2_coeffs(const double *C, const double *norma, int n, int n_frozen, int n_occ, double *Co,
                              double *Cv, float *Co32, float *Cv32, cudaStream_t s) {
  const long long tot = (long long)n * n;
  mp2_coeffs_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(C, norma, n, n_frozen, n_occ, Co, Cv, Co32, Cv32);
  count_launches(1);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_mp2_unpack(const T *Y, const unsigned *colpair, long long ncols, int n, int v, T *Z,
                              cudaStream_t s) {
  if (ncols <= 0) return cudaSuccess;
  const unsigned blocks = (unsigned)(ncols < 152LL * 64 ? ncols : 152LL * 64);
  mp2_unpack_kernel<T><<<blocks, 128, 0, s>>>(Y, colpair, ncols, n, v, Z);
  count_launches(1);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_mp2_energy(const T *M, int o, int v, double ei, const double *eo, const double *ev, double cut,
                              double *e2, cudaStream_t s) {
  if (o <= 0 || v <= 0) return cudaSuccess;
  const dim3 grid((unsigned)((v + 31) / 32), (unsigned)((v + 31) / 32), (unsigned)o);
  mp2_energy_kernel<T><<<grid, dim3(32, 8), 0, s>>>(M, v, ei, eo, ev, cut, e2);
  count_launches(1);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_mp2_energy_coupling(const T *M, int o, int vB, int vA, double ei, const double *eo,
                                       const double *evA, const double *evB, double cut, double factor, double *e2,
                                       cudaStream_t s) {
  if (o <= 0 || vA <= 0 || vB <= 0) return cudaSuccess;
  const long long per = (long long)vB * vA;
  const unsigned gx = (unsigned)std::min<long long>((per + 255) / 256, 64);
  mp2_energy_coupling_kernel<T><<<dim3(gx, (unsigned)o), 256, 0, s>>>(M, vB, vA, ei, eo, evA, evB, cut, factor, e2);
  count_launches(1);
  return cudaGetLastError();
}

template cudaError_t launch_mp2_energy_coupling<double>(const double *, int, int, int, double, const double *,
                                                        const double *, const double *, double, double, double *,
                                                        cudaStream_t);
template cudaError_t launch_mp2_energy_coupling<float>(const float *, int, int, int, double, const double *,
                                                       const double *, const double *, double, double, double *,
                                                       cudaStream_t);
template cudaError_t launch_mp2_unpack<double>(const double *, const unsigned *, long long, int, int, double *,
                                               cudaStream_t);
template cudaError_t launch_mp2_unpack<float>(const float *, const unsigned *, long long, int, int, float *,
                                              cudaStream_t);
template cudaError_t launch_mp2_energy<double>(const double *, int, int, double, const double *, const double *,
                                               double, double *, cudaStream_t);
template cudaError_t launch_mp2_energy<float>(const float *, int, int, double, const double *, const double *,
                                              double, double *, cudaStream_t);

}  // namespace lgb
