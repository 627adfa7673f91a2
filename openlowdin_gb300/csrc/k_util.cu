// Element-wise helpers around the integral kernels: density preparation,
// symmetrisation and output scaling.  All are HBM-streaming O(n^2) / O(n^3)
// kernels with grid-stride loops.
#include <atomic>

#include "kernels.cuh"

namespace lgb {

namespace {

int grid_for(size_t n, int block) {
  size_t g = (n + block - 1) / block;
  return (int)(g > 152 * 16 ? 152 * 16 : (g == 0 ? 1 : g));
}

// max of non-negative values through their bit patterns (IEEE order == integer
// order for x >= 0), exact
__device__ __forceinline__ void atomic_max_nonneg(double *p, double v) {
  atomicMax(reinterpret_cast<unsigned long long *>(p), (unsigned long long)__double_as_longlong(v));
}
__device__ __forceinline__ void atomic_max_nonneg(float *p, float v) {
  atomicMax(reinterpret_cast<unsigned int *>(p), (unsigned int)__float_as_int(v));
}

// Ds = N D N (FP64 and FP32 copies) and Dn[s1][s2] = max |D| over the shell
// block (unscaled D)
__global__ void prepare_density_kernel(const double *__restrict__ D, const double *__restrict__ norma,
                                       const int *__restrict__ shell_of, int n, int nsh, double *__restrict__ Ds,
                                       float *__restrict__ Ds32, double *__restrict__ Dn, float *__restrict__ Dn32) {
  const size_t nn = (size_t)n * n;
  for (size_t x = blockIdx.x * (size_t)blockDim.x + threadIdx.x; x < nn; x += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(x / n), j = (int)(x % n);
    const double d = D[x];
    const double s = d * norma[i] * norma[j];
    Ds[x] = s;
    if (Ds32) Ds32[x] = (float)s;
    const int b = shell_of[i] * nsh + shell_of[j];
    atomic_max_nonneg(Dn + b, fabs(d));
    if (Dn32) atomic_max_nonneg(Dn32 + b, (float)fabs(d));
  }
}

__global__ void scale_density_kernel(const double *__restrict__ D, const double *__restrict__ norma, int n,
                                     double *__restrict__ Ds, float *__restrict__ Ds32) {
  const size_t nn = (size_t)n * n;
  for (size_t x = blockIdx.x * (size_t)blockDim.x + threadIdx.x; x < nn; x += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(x / n), j = (int)(x % n);
    const double s = D[x] * norma[i] * norma[j];
    Ds[x] = s;
    if (Ds32) Ds32[x] = (float)s;
  }
}

// G = scale * N_i N_j (Gacc + Gacc^T) (+ the FP32 accumulator when present)
__global__ void symmetrize_kernel(const double *__restrict__ Gacc, const float *__restrict__ Gacc32,
                                  const double *__restrict__ norma, int n, double scale, double *__restrict__ G) {
  const size_t nn = (size_t)n * n;
  for (size_t x = blockIdx.x * (size_t)blockDim.x + threadIdx.x; x < nn; x += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(x / n), j = (int)(x % n);
    const size_t y = (size_t)j * n + i;
    double g = Gacc[x] + Gacc[y];
    if (Gacc32) g += (double)Gacc32[x] + (double)Gacc32[y];
    G[x] = scale * norma[i] * norma[j] * g;
  }
}

// out = scale * N_i N_j J (row >= col only when lower_only, zero above)
__global__ void coupling_extract_kernel(const double *__restrict__ J, const float *__restrict__ J32,
                                        const double *__restrict__ norma, int n, double scale, int lower_only,
                                        double *__restrict__ out) {
  const size_t nn = (size_t)n * n;
  for (size_t x = blockIdx.x * (size_t)blockDim.x + threadIdx.x; x < nn; x += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(x / n), j = (int)(x % n);
    const double v = J[x] + (J32 ? (double)J32[x] : 0.0);
    out[x] = (lower_only && j > i) ? 0.0 : scale * norma[i] * norma[j] * v;
  }
}

__global__ void scale_cube_kernel(double *__restrict__ A, const double *__restrict__ normA,
                                  const double *__restrict__ normB, int nA, int nB) {
  const size_t total = (size_t)nA * nB * nB;
  for (size_t x = blockIdx.x * (size_t)blockDim.x + threadIdx.x; x < total; x += (size_t)gridDim.x * blockDim.x) {
    const int s = (int)(x % nB);
    const int l = (int)((x / nB) % nB);
    const int nu = (int)(x / ((size_t)nB * nB));
    A[x] *= normA[nu] * normB[l] * normB[s];
  }
}

// 8 independent FMA chains per thread; the result is stored so nothing is
// removed by the compiler.
template <typename T>
__global__ void __launch_bounds__(256) fma_probe_kernel(T *out, int iters, T a, T b) {
  T x0 = T(threadIdx.x) * T(1e-3), x1 = x0 + T(1), x2 = x0 + T(2), x3 = x0 + T(3);
  T x4 = x0 + T(4), x5 = x0 + T(5), x6 = x0 + T(6), x7 = x0 + T(7);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b;
      x4 = x4 * a + b; x5 = x5 * a + b; x6 = x6 * a + b; x7 = x7 * a + b;
    }
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

std::atomic<long long> g_launches{0};

__device__ __forceinline__ int find_slot(const SpeciesSlot *__restrict__ slots, int nslots, long long x) {
  int lo = 0, hi = nslots - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (slots[mid].off <= x) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// every species of a batch: Ds = N P N (FP64 and FP32), Dn = shell-block max
// |P| (when used) and zeroed accumulators
__global__ void prepare_batch_kernel(const SpeciesSlot *__restrict__ slots, int nslots, long long total) {
  for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < total;
       x += (long long)gridDim.x * blockDim.x) {
    const SpeciesSlot &S = slots[find_slot(slots, nslots, x)];
    if (S.active && __ldg(S.active) == 0) continue;
    const long long e = x - S.off;
    const int i = (int)(e / S.n), j = (int)(e % S.n);
    const double p = S.P[(long long)i * S.ld + j];
    const double s = p * S.norma[i] * S.norma[j];
    S.Ds[e] = s;
    S.Ds32[e] = (float)s;
    if (S.Gacc) {
      S.Gacc[e] = 0.0;
      S.Gacc32[e] = 0.0f;
    }
    S.Jacc[e] = 0.0;
    S.Jacc32[e] = 0.0f;
    if (S.Dn) {
      const int b = S.shell_of[i] * S.nsh + S.shell_of[j];
      atomic_max_nonneg(S.Dn + b, fabs(p));
      atomic_max_nonneg(S.Dn32 + b, (float)fabs(p));
    }
  }
}

// maximum over the block (valid in thread 0)
__device__ __forceinline__ float block_max(float m) {
  __shared__ float part[32];
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    m = threadIdx.x < (blockDim.x >> 5) ? part[threadIdx.x] : 0.f;
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  }
  return m;   // valid in thread 0
}

// largest of Dn32: block x takes columns [256 x, 256 x + 256) of the nsh x nsh
// norms (a thread walks its column, coalesced across the block), its maximum
// goes to *out (non-negative floats order as their bit patterns)
__device__ __forceinline__ void dn_max_block(const float *__restrict__ Dn32, int nsh, float *__restrict__ out) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  float m = 0.f;
  if (s < nsh)
    for (int t = 0; t < nsh; ++t) m = fmaxf(m, Dn32[(size_t)t * nsh + s]);
  m = block_max(m);
  if (threadIdx.x == 0) atomicMax(reinterpret_cast<int *>(out), __float_as_int(m));
}

__global__ void dn_max_batch_kernel(const SpeciesSlot *__restrict__ slots) {
  const SpeciesSlot &S = slots[blockIdx.y];
  if (!S.Dn32 || !S.Dnmax32 || blockIdx.x * blockDim.x >= (unsigned)S.nsh) return;
  if (S.active && __ldg(S.active) == 0) return;
  dn_max_block(S.Dn32, S.nsh, S.Dnmax32);
}

__global__ void dn_max_kernel(const float *__restrict__ Dn32, int nsh, float *__restrict__ out) {
  dn_max_block(Dn32, nsh, out);
}

// G = gscale N (Gacc + Gacc^T) N (0 when the species builds none), J = N Jacc N,
// FP32 accumulators added in
__global__ void finalize_batch_kernel(const SpeciesSlot *__restrict__ slots, int nslots, long long total) {
  for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < total;
       x += (long long)gridDim.x * blockDim.x) {
    const SpeciesSlot &S = slots[find_slot(slots, nslots, x)];
    if (S.active && __ldg(S.active) == 0) continue;   // switched-off system: outputs kept
    const long long e = x - S.off;
    const int i = (int)(e / S.n), j = (int)(e % S.n);
    const double nn = S.norma[i] * S.norma[j];
    const long long o = (long long)i * S.ld + j;   // outputs may be rows of a wider (padded) matrix
    if (S.G) {
      if (S.Gacc) {
        const long long y = (long long)j * S.n + i;
        const double g = S.Gacc[e] + S.Gacc[y] + (double)S.Gacc32[e] + (double)S.Gacc32[y];
        S.G[o] = S.gscale * nn * g;
      } else {
        S.G[o] = 0.0;
      }
    }
    S.J[o] = nn * (S.Jacc[e] + (double)S.Jacc32[e]);
  }
}

__device__ __forceinline__ int find_pair_slot(const PairSlot *__restrict__ slots, int nslots, long long x) {
  int lo = 0, hi = nslots - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (slots[mid].poff <= x) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// class of pair record `idx` of a slot and its position in the class
__device__ __forceinline__ int pair_class_of(const PairSlot &S, int idx, int *pos) {
  int c = 0;
  while (c + 1 < kNumPairClasses && S.start[c + 1] <= idx) ++c;
  *pos = idx - S.start[c];
  return c;
}

// one thread per (slot, pair): its D block, norm, and a cleared accumulator
__global__ void pair_gather_kernel(const PairSlot *__restrict__ slots, int nslots, long long total) {
  for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < total;
       x += (long long)gridDim.x * blockDim.x) {
    const PairSlot &S = slots[find_pair_slot(slots, nslots, x)];
    if (S.active && __ldg(S.active) == 0) continue;
    const int idx = (int)(x - S.poff);
    int k;
    const int c = pair_class_of(S, idx, &k);
    const int cnt = S.start[c + 1] - S.start[c];
    const PairRec32 r = S.pairs[idx];
    const int nb = ncart(r.lb), ne = ncart(r.la) * nb;
    const long long base = S.pe_base[c] + k;
    for (int e = 0; e < ne; ++e) {
      S.Dp32[base + (long long)e * cnt] = S.Ds32[(size_t)(r.fa + e / nb) * S.n + r.fb + e % nb];
      S.Jp32[base + (long long)e * cnt] = 0.f;
    }
    if (S.Dn32) S.DnP32[idx] = S.Dn32[(size_t)r.sa * S.nsh + r.sb];
  }
}

__global__ void pair_scatter_kernel(const PairSlot *__restrict__ slots, int nslots, long long total) {
  for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < total;
       x += (long long)gridDim.x * blockDim.x) {
    const PairSlot &S = slots[find_pair_slot(slots, nslots, x)];
    if (S.active && __ldg(S.active) == 0) continue;
    const int idx = (int)(x - S.poff);
    int k;
    const int c = pair_class_of(S, idx, &k);
    const int cnt = S.start[c + 1] - S.start[c];
    const PairRec32 r = S.pairs[idx];
    const int nb = ncart(r.lb), ne = ncart(r.la) * nb;
    const long long base = S.pe_base[c] + k;
    // each pair owns its block of Gacc32 (distinct shell pairs, canonical order)
    for (int e = 0; e < ne; ++e) {
      const float v = S.Jp32[base + (long long)e * cnt];
      if (v != 0.f) S.Gacc32[(size_t)(r.fa + e / nb) * S.n + r.fb + e % nb] += v;
    }
  }
}

}  // namespace

long long pair_elements(const int *start, long long *pe_base) {
  long long tot = 0;
  for (int c = 0; c < kNumPairClasses; ++c) {
    pe_base[c] = tot;
    tot += (long long)(start[c + 1] - start[c]) * ncart(pc_la(c)) * ncart(pc_lb(c));
  }
  return tot;
}

cudaError_t launch_pair_gather(const PairSlot *slots, int nslots, long long total_pairs, cudaStream_t s) {
  if (total_pairs <= 0) return cudaSuccess;
  pair_gather_kernel<<<grid_for((size_t)total_pairs, 256), 256, 0, s>>>(slots, nslots, total_pairs);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_pair_scatter(const PairSlot *slots, int nslots, long long total_pairs, cudaStream_t s) {
  if (total_pairs <= 0) return cudaSuccess;
  pair_scatter_kernel<<<grid_for((size_t)total_pairs, 256), 256, 0, s>>>(slots, nslots, total_pairs);
  count_launches(1);
  return cudaGetLastError();
}

void count_launches(long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
long long launch_count() { return g_launches.load(std::memory_order_relaxed); }

cudaError_t launch_prepare_batch(const SpeciesSlot *slots, int nslots, long long total, cudaStream_t s) {
  if (total <= 0) return cudaSuccess;
  prepare_batch_kernel<<<grid_for((size_t)total, 256), 256, 0, s>>>(slots, nslots, total);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_dn_max_batch(const SpeciesSlot *slots, int nslots, int max_nsh, cudaStream_t s) {
  if (nslots <= 0 || max_nsh <= 0) return cudaSuccess;
  dn_max_batch_kernel<<<dim3((unsigned)((max_nsh + 255) / 256), (unsigned)nslots), 256, 0, s>>>(slots);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_dn_max(const float *Dn32, int nsh, float *out, cudaStream_t s) {
  const cudaError_t e = cudaMemsetAsync(out, 0, sizeof(float), s);
  if (e != cudaSuccess) return e;
  dn_max_kernel<<<(nsh + 255) / 256, 256, 0, s>>>(Dn32, nsh, out);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_finalize_batch(const SpeciesSlot *slots, int nslots, long long total, cudaStream_t s) {
  if (total <= 0) return cudaSuccess;
  finalize_batch_kernel<<<grid_for((size_t)total, 256), 256, 0, s>>>(slots, nslots, total);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t measure_fma_tflops(bool fp64, double *tflops) {
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  const int blocks = sms * 8, threads = 256;
  const int iters = fp64 ? 512 : 4096;
  void *buf = nullptr;
  e = cudaMalloc(&buf, (size_t)blocks * threads * 8);
  if (e != cudaSuccess) return e;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  float best = 1e30f;
  for (int rep = 0; rep < 4; ++rep) {
    cudaEventRecord(a);
    if (fp64) fma_probe_kernel<double><<<blocks, threads>>>((double *)buf, iters, 0.999999, 1e-7);
    else fma_probe_kernel<float><<<blocks, threads>>>((float *)buf, iters, 0.999999f, 1e-7f);
    cudaEventRecord(b);
    cudaEventSynchronize(b);
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    if (rep > 0 && ms < best) best = ms;
  }
  e = cudaGetLastError();
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(buf);
  const double flops = 2.0 * 8 * 16 * (double)iters * blocks * threads;
  *tflops = flops / (best * 1e-3) / 1e12;
  return e;
}

cudaError_t launch_prepare_density(const double *D, const double *norma, const int *shell_of, int n, int nsh,
                                   double *Ds, float *Ds32, double *Dn, float *Dn32, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(Dn, 0, sizeof(double) * nsh * nsh, s);
  if (e != cudaSuccess) return e;
  if (Dn32) {
    e = cudaMemsetAsync(Dn32, 0, sizeof(float) * nsh * nsh, s);
    if (e != cudaSuccess) return e;
  }
  prepare_density_kernel<<<grid_for((size_t)n * n, 256), 256, 0, s>>>(D, norma, shell_of, n, nsh, Ds, Ds32, Dn,
                                                                      Dn32);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_scale_density(const double *D, const double *norma, int n, double *Ds, float *Ds32,
                                 cudaStream_t s) {
  scale_density_kernel<<<grid_for((size_t)n * n, 256), 256, 0, s>>>(D, norma, n, Ds, Ds32);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_symmetrize(const double *Gacc, const float *Gacc32, const double *norma, int n, double scale,
                              double *G, cudaStream_t s) {
  symmetrize_kernel<<<grid_for((size_t)n * n, 256), 256, 0, s>>>(Gacc, Gacc32, norma, n, scale, G);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_coupling_extract(const double *J, const float *J32, const double *norma, int n, double scale,
                                    int lower_only, double *out, cudaStream_t s) {
  coupling_extract_kernel<<<grid_for((size_t)n * n, 256), 256, 0, s>>>(J, J32, norma, n, scale, lower_only, out);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_scale_cube(double *A, const double *normA, const double *normB, int nA, int nB,
                              cudaStream_t s) {
  scale_cube_kernel<<<grid_for((size_t)nA * nB * nB, 256), 256, 0, s>>>(A, normA, normB, nA, nB);
  count_launches(1);
  return cudaGetLastError();
}

}  // namespace lgb
