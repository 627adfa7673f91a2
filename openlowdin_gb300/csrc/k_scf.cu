// Device-side pieces of the SCF driver (caller side of the integral path).
//
// Pulay DIIS coefficients (openLOWDIN src/scf/Convergence.f90:543-633): for
// each system the error-product matrix E[i][j] = <e_i, e_j> of its last h
// error vectors gives the bordered system
//     [ E   -1 ] [c]   [ 0]
//     [-1^T  0 ] [l] = [-1],
// solved here by a pseudo-inverse.  The reference takes an SVD of the bordered
// matrix and inverts the singular values above 1e-4.  An SCF history has
// errors over many orders of magnitude, so this kernel first scales E to unit
// diagonal (E' = D^-1 E D^-1, D = diag(sqrt(E_ii)), c = D^-1 c') with the
// border w_i = 1/sqrt(E_ii) brought to at most 1 in magnitude, diagonalises
// the symmetric bordered matrix by cyclic Jacobi rotations in FP64 (one
// thread per system, h <= 20) and inverts the eigenvalues above 1e-12 of the
// largest in magnitude (the rest are dropped): the minimum-norm least-squares
// solution of the extrapolation, with no host round trip.
#include "lint_host.cuh"

namespace lgb {
namespace {

constexpr int kDiisMax = 20;   // history length limit (h)

__global__ void diis_solve_kernel(const double *__restrict__ E, int h, int nsys, const int *__restrict__ first,
                                  double *__restrict__ coef, int *__restrict__ status) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nsys) return;
  constexpr int M = kDiisMax + 1;
  double A[M][M], V[M][M];
  const int m = h + 1;
  const double *e = E + (size_t)s * h * h;
  // unit-diagonal scaling: dinv[i] = 1/sqrt(E_ii) (a zero error keeps a
  // floor), border -alpha dinv[i] with alpha = 1 / max dinv
  // entries before first[s] are left out of the extrapolation (a decoupled
  // unit row: coefficient 0)
  const int f0 = first ? min(max(first[s], 0), h - 1) : 0;
  double dinv[kDiisMax], wmax = 0.0;
  for (int i = 0; i < h; ++i) {
    dinv[i] = i < f0 ? 0.0 : 1.0 / sqrt(fmax(e[i * h + i], 1e-300));
    wmax = fmax(wmax, dinv[i]);
  }
  const double alpha = 1.0 / wmax;
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < m; ++j) {
      double v;
      if (i < h && j < h) v = (i < f0 || j < f0) ? (i == j ? 1.0 : 0.0)
                                                 : 0.5 * (e[i * h + j] + e[j * h + i]) * dinv[i] * dinv[j];
      else if (i == h && j == h) v = 0.0;
      else v = -alpha * dinv[i < h ? i : j];
      A[i][j] = v;
      V[i][j] = i == j ? 1.0 : 0.0;
    }
  // cyclic Jacobi: rotate away every off-diagonal element, sweep until the
  // off-diagonal norm is at FP64 rounding of the diagonal
  int sweep = 0;
  for (; sweep < 60; ++sweep) {
    double off = 0.0, dia = 0.0;
    for (int i = 0; i < m; ++i) {
      dia += A[i][i] * A[i][i];
      for (int j = i + 1; j < m; ++j) off += A[i][j] * A[i][j];
    }
    if (off <= 1e-30 * dia || off == 0.0) break;
    for (int p = 0; p < m - 1; ++p)
      for (int q = p + 1; q < m; ++q) {
        const double apq = A[p][q];
        if (apq == 0.0) continue;
        // tan of the rotation angle from cot(2 theta) = (a_qq - a_pp) / (2 a_pq)
        const double th = (A[q][q] - A[p][p]) / (2.0 * apq);
        const double t = (th >= 0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
        const double c = 1.0 / sqrt(t * t + 1.0), sn = t * c;
        for (int k = 0; k < m; ++k) {
          const double akp = A[k][p], akq = A[k][q];
          A[k][p] = c * akp - sn * akq;
          A[k][q] = sn * akp + c * akq;
        }
        for (int k = 0; k < m; ++k) {
          const double apk = A[p][k], aqk = A[q][k];
          A[p][k] = c * apk - sn * aqk;
          A[q][k] = sn * apk + c * aqk;
        }
        for (int k = 0; k < m; ++k) {
          const double vkp = V[k][p], vkq = V[k][q];
          V[k][p] = c * vkp - sn * vkq;
          V[k][q] = sn * vkp + c * vkq;
        }
      }
  }
  double amax = 0.0;
  for (int i = 0; i < m; ++i) amax = fmax(amax, fabs(A[i][i]));
  // c' = V diag(1/lambda) V^T r with r = (0, ..., 0, -alpha); c = D^-1 c'
  for (int i = 0; i < h; ++i) {
    double x = 0.0;
    for (int k = 0; k < m; ++k) {
      const double lam = A[k][k];
      if (fabs(lam) > 1e-12 * amax) x += V[i][k] * (-alpha * V[h][k]) / lam;
    }
    coef[(size_t)s * h + i] = x * dinv[i];
  }
  if (status) status[s] = sweep;
}

}  // namespace
}  // namespace lgb

extern "C" int LowdinGB300_diis_coefficients(const double *dE, int h, int nsys, const int *dfirst, double *dcoef,
                                             void *stream) {
  if (h < 1 || h > lgb::kDiisMax || nsys < 0 || (nsys > 0 && (!dE || !dcoef))) {
    lgb::set_error("diis_coefficients: history length %d outside 1..%d or null arrays", h, lgb::kDiisMax);
    return -1;
  }
  if (nsys == 0) return 0;
  lgb::diis_solve_kernel<<<(nsys + 31) / 32, 32, 0, (cudaStream_t)stream>>>(dE, h, nsys, dfirst, dcoef, nullptr);
  lgb::count_launches(1);
  if (cudaGetLastError() != cudaSuccess) {
    lgb::set_error("diis_coefficients: launch failed");
    return -1;
  }
  return 0;
}

// ------------------------------------------------------------ Boys check --
// Evaluation of the device Boys functions at given arguments, for the tests
// (FP32: the arithmetic form of the FP32 kernels; FP64: the tabulated Taylor
// form of the FP64 kernels).
namespace lgb {
namespace {

template <int L>
__global__ void boys_eval_kernel(int fp32, const double *T, int n, double *out, BoysTables tabs) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (fp32) {
    float F[L + 1];
    boys_f32<L>((float)T[i], F, tabs.f32);
    for (int m = 0; m <= L; ++m) out[(size_t)i * (L + 1) + m] = F[m];
  } else {
    double F[L + 1];
    boys_f64<L>(T[i], F, tabs.f64);
    for (int m = 0; m <= L; ++m) out[(size_t)i * (L + 1) + m] = F[m];
  }
}

}  // namespace
}  // namespace lgb

extern "C" int LowdinGB300_boys_eval(int fp32, int L, const double *T, int n, double *out) {
  using namespace lgb;
  if (L < 0 || L > 4 || n < 0 || (n > 0 && (!T || !out))) {
    set_error("boys_eval: order %d outside 0..4 or null arrays", L);
    return -1;
  }
  if (n == 0) return 0;
  BoysTables tabs{};
  if (!device_boys(tabs)) return -1;
  double *dT = nullptr, *dF = nullptr;
  if (cudaMalloc(&dT, sizeof(double) * n) != cudaSuccess ||
      cudaMalloc(&dF, sizeof(double) * n * (L + 1)) != cudaSuccess) {
    if (dT) cudaFree(dT);
    set_error("boys_eval: allocation failed");
    return -1;
  }
  cudaMemcpy(dT, T, sizeof(double) * n, cudaMemcpyHostToDevice);
  const int nb = (n + 127) / 128;
  switch (L) {
    case 0: boys_eval_kernel<0><<<nb, 128>>>(fp32, dT, n, dF, tabs); break;
    case 1: boys_eval_kernel<1><<<nb, 128>>>(fp32, dT, n, dF, tabs); break;
    case 2: boys_eval_kernel<2><<<nb, 128>>>(fp32, dT, n, dF, tabs); break;
    case 3: boys_eval_kernel<3><<<nb, 128>>>(fp32, dT, n, dF, tabs); break;
    default: boys_eval_kernel<4><<<nb, 128>>>(fp32, dT, n, dF, tabs); break;
  }
  count_launches(1);
  const cudaError_t e = cudaMemcpy(out, dF, sizeof(double) * n * (L + 1), cudaMemcpyDeviceToHost);
  cudaFree(dT);
  cudaFree(dF);
  if (e != cudaSuccess) {
    set_error("boys_eval: kernel or copy failed (%s)", cudaGetErrorString(e));
    return -1;
  }
  return 0;
}
