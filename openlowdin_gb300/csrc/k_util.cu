// Element-wise helpers around the integral kernels: density preparation,
// symmetrisation and output scaling.  All are HBM-streaming O(n^2) / O(n^3)
// kernels with grid-stride loops.
#include "kernels.cuh"

namespace lgb {

namespace {

int grid_for(size_t n, int block) {
  size_t g = (n + block - 1) / block;
  return (int)(g > 152 * 16 ? 152 * 16 : (g == 0 ? 1 : g));
}

// Ds = N D N and Dn[s1][s2] = max |D| over the shell block (unscaled D)
__global__ void prepare_density_kernel(const double *__restrict__ D, const double *__restrict__ norma,
                                       const int *__restrict__ shell_of, int n, int nsh, double *__restrict__ Ds,
                                       double *__restrict__ Dn) {
  const size_t nn = (size_t)n * n;
  for (size_t x = blockIdx.x * (size_t)blockDim.x + threadIdx.x; x < nn; x += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(x / n), j = (int)(x % n);
    const double d = D[x];
    Ds[x] = d * norma[i] * norma[j];
    // |d| >= 0, so the IEEE bit pattern orders like the value: integer max is exact
    atomicMax(reinterpret_cast<unsigned long long *>(Dn) + shell_of[i] * nsh + shell_of[j],
              (unsigned long long)__double_as_longlong(fabs(d)));
  }
}

__global__ void scale_density_kernel(const double *__restrict__ D, const double *__restrict__ norma, int n,
                                     double *__restrict__ Ds) {
  const size_t nn = (size_t)n * n;
  for (size_t x = blockIdx.x * (size_t)blockDim.x + threadIdx.x; x < nn; x += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(x / n), j = (int)(x % n);
    Ds[x] = D[x] * norma[i] * norma[j];
  }
}

// G = scale * N_i N_j (Gacc + Gacc^T)
__global__ void symmetrize_kernel(const double *__restrict__ Gacc, const double *__restrict__ norma, int n,
                                  double scale, double *__restrict__ G) {
  const size_t nn = (size_t)n * n;
  for (size_t x = blockIdx.x * (size_t)blockDim.x + threadIdx.x; x < nn; x += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(x / n), j = (int)(x % n);
    G[x] = scale * norma[i] * norma[j] * (Gacc[x] + Gacc[(size_t)j * n + i]);
  }
}

// out = scale * N_i N_j J (row >= col only when lower_only, zero above)
__global__ void coupling_extract_kernel(const double *__restrict__ J, const double *__restrict__ norma, int n,
                                        double scale, int lower_only, double *__restrict__ out) {
  const size_t nn = (size_t)n * n;
  for (size_t x = blockIdx.x * (size_t)blockDim.x + threadIdx.x; x < nn; x += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(x / n), j = (int)(x % n);
    out[x] = (lower_only && j > i) ? 0.0 : scale * norma[i] * norma[j] * J[x];
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

}  // namespace

cudaError_t launch_prepare_density(const double *D, const double *norma, const int *shell_of, int n, int nsh,
                                   double *Ds, double *Dn, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(Dn, 0, sizeof(double) * nsh * nsh, s);
  if (e != cudaSuccess) return e;
  prepare_density_kernel<<<grid_for((size_t)n * n, 256), 256, 0, s>>>(D, norma, shell_of, n, nsh, Ds, Dn);
  return cudaGetLastError();
}

cudaError_t launch_scale_density(const double *D, const double *norma, int n, double *Ds, cudaStream_t s) {
  scale_density_kernel<<<grid_for((size_t)n * n, 256), 256, 0, s>>>(D, norma, n, Ds);
  return cudaGetLastError();
}

cudaError_t launch_symmetrize(const double *Gacc, const double *norma, int n, double scale, double *G,
                              cudaStream_t s) {
  symmetrize_kernel<<<grid_for((size_t)n * n, 256), 256, 0, s>>>(Gacc, norma, n, scale, G);
  return cudaGetLastError();
}

cudaError_t launch_coupling_extract(const double *J, const double *norma, int n, double scale, int lower_only,
                                    double *out, cudaStream_t s) {
  coupling_extract_kernel<<<grid_for((size_t)n * n, 256), 256, 0, s>>>(J, norma, n, scale, lower_only, out);
  return cudaGetLastError();
}

cudaError_t launch_scale_cube(double *A, const double *normA, const double *normB, int nA, int nB,
                              cudaStream_t s) {
  scale_cube_kernel<<<grid_for((size_t)nA * nB * nB, 256), 256, 0, s>>>(A, normA, normB, nA, nB);
  return cudaGetLastError();
}

}  // namespace lgb
