// One-electron matrices on the device: overlap S, kinetic T and the
// point-charge potential V = sum_C Z_C <a|1/|r - C||b> of one species, one
// thread per unordered shell pair, Obara-Saika recursions (1-D overlap tables
// for S and T; the vertical recursion with Boys values and a horizontal
// transfer for V), written normalised (norma_i norma_j) to both (i, j) and
// (j, i).  Same formulas as the host blocks the library's
// LibintInterface_compute_1body_ints uses (ContractedGaussian / Overlap /
// Kinetic / Attraction integrals of the reference, src/ints/*.f90).
#include "eri_generic.cuh"
#include "kernels.cuh"

namespace lgb {
namespace {

constexpr int kOneMaxL = kMaxL + 2;   // kinetic needs j + 2

__device__ void ovl1d_dev(int li, int lj, double PA, double PB, double o2p, double s[kMaxL + 1][kOneMaxL + 1]) {
  for (int i = 0; i <= li; ++i)
    for (int j = 0; j <= lj; ++j) {
      double v;
      if (!i && !j) {
        v = 1.0;
      } else if (i > 0) {
        v = PA * s[i - 1][j];
        if (i > 1) v += (i - 1) * o2p * s[i - 2][j];
        if (j > 0) v += j * o2p * s[i - 1][j - 1];
      } else {
        v = PB * s[0][j - 1];
        if (j > 1) v += (j - 1) * o2p * s[0][j - 2];
      }
      s[i][j] = v;
    }
}

__global__ void __launch_bounds__(128) one_body_kernel(OneBodyParams P) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int npair = P.nsh * (P.nsh + 1) / 2;
  if (t >= npair) return;
  // t -> (s1 >= s2)
  int s1 = (int)((sqrt(8.0 * t + 1.0) - 1.0) * 0.5);
  while (s1 * (s1 + 1) / 2 > t) --s1;
  while ((s1 + 1) * (s1 + 2) / 2 <= t) ++s1;
  const int s2 = t - s1 * (s1 + 1) / 2;
  const DevShell A = P.shells[s1], B = P.shells[s2];
  const CartInfo *ct = kCartTable.e;
  const int la = A.l, lb = B.l, n1 = ncart(la), n2 = ncart(lb);
  constexpr int kNC2 = ncart(kMaxL) * ncart(kMaxL);
  double S[kNC2], T[kNC2], V[kNC2];
  for (int k = 0; k < n1 * n2; ++k) S[k] = T[k] = V[k] = 0.0;
  double AB[3], AB2 = 0;
  for (int d = 0; d < 3; ++d) {
    AB[d] = A.O[d] - B.O[d];
    AB2 += AB[d] * AB[d];
  }
  // potential: vertical recursion on the bra up to la + lb, then transfer
  const int L = la + lb, NE = coff(L + 1), E0 = coff(la), M = L + 1;
  double W[coff(2 * kMaxL + 1) * (2 * kMaxL + 1)], X[coff(2 * kMaxL + 1)];
  for (int e = 0; e < NE - E0; ++e) X[e] = 0.0;
  for (int pa = 0; pa < A.nprim; ++pa)
    for (int pb = 0; pb < B.nprim; ++pb) {
      const double a = P.alpha[A.p0 + pa], b = P.alpha[B.p0 + pb], p = a + b, o2p = 0.5 / p;
      const double cab = P.cn[A.p0 + pa] * P.cn[B.p0 + pb] * exp(-a * b / p * AB2);
      double Pc[3], PA[3];
      for (int d = 0; d < 3; ++d) {
        Pc[d] = (a * A.O[d] + b * B.O[d]) / p;
        PA[d] = Pc[d] - A.O[d];
      }
      if (P.S || P.T) {
        const double pref = cab * pow(3.14159265358979323846 / p, 1.5);
        double s[3][kMaxL + 1][kOneMaxL + 1];
        for (int d = 0; d < 3; ++d) ovl1d_dev(la, lb + 2, PA[d], Pc[d] - B.O[d], o2p, s[d]);
        for (int f1 = 0; f1 < n1; ++f1) {
          const CartInfo &c1 = ct[coff(la) + f1];
          for (int f2 = 0; f2 < n2; ++f2) {
            const CartInfo &c2 = ct[coff(lb) + f2];
            const double sx = s[0][c1.xyz[0]][c2.xyz[0]], sy = s[1][c1.xyz[1]][c2.xyz[1]],
                         sz = s[2][c1.xyz[2]][c2.xyz[2]];
            S[f1 * n2 + f2] += pref * sx * sy * sz;
            double tk[3];
            for (int d = 0; d < 3; ++d) {
              const int i = c1.xyz[d], j = c2.xyz[d];
              double v = -2.0 * b * (2 * j + 1) * s[d][i][j] + 4.0 * b * b * s[d][i][j + 2];
              if (j >= 2) v += j * (j - 1) * s[d][i][j - 2];
              tk[d] = -0.5 * v;
            }
            T[f1 * n2 + f2] += pref * (tk[0] * sy * sz + sx * tk[1] * sz + sx * sy * tk[2]);
          }
        }
      }
      if (P.V) {
        const double w = cab * 2.0 * 3.14159265358979323846 / p;
        for (int c = 0; c < P.ncharge; ++c) {
          double PC[3], PC2 = 0, F[kGenMaxL + 1];
          for (int d = 0; d < 3; ++d) {
            PC[d] = Pc[d] - P.R[3 * c + d];
            PC2 += PC[d] * PC[d];
          }
          boys_f64_rt(L, p * PC2, F, P.boys.f64);
          for (int m = 0; m <= L; ++m) W[m] = F[m];
          for (int e = 1; e < NE; ++e) {
            const CartInfo &ce = ct[e];
            const int d = ce.dir, em = ce.m[d], ei = ce.xyz[d] - 1;
            for (int m = 0; m <= L - ce.lev; ++m) {
              double v = PA[d] * W[em * M + m] - PC[d] * W[em * M + m + 1];
              if (ei > 0) {
                const int emm = ct[em].m[d];
                v += ei * o2p * (W[emm * M + m] - W[emm * M + m + 1]);
              }
              W[e * M + m] = v;
            }
          }
          const double zw = P.Z[c] * w;
          for (int e = E0; e < NE; ++e) X[e - E0] += zw * W[e * M];
        }
      }
    }
  if (P.V) {
    // horizontal transfer (a, b+1_i| = (a+1_i, b| + AB_i (a, b| over lb
    // levels: level j has rows over totals la .. la + lb - j (the last level
    // only la) and ncart(j) columns; it reads level j - 1 (X for j = 1)
    constexpr int kHRows = coff(2 * kMaxL), kHCols = ncart(kMaxL);
    double Hb[2][kHRows * kHCols];
    if (lb == 0) {
      for (int f1 = 0; f1 < n1; ++f1) V[f1] = X[f1];
    } else {
      for (int j = 1; j <= lb; ++j) {
        const int na = j == lb ? n1 : coff(la + lb - j + 1) - E0, nb = ncart(j), pnb = j == 1 ? 1 : ncart(j - 1);
        const double *src = j == 1 ? X : Hb[j & 1];
        double *dst = j == lb ? V : Hb[(j - 1) & 1];
        for (int bi = 0; bi < nb; ++bi) {
          const int bc = coff(j) + bi, d = ct[bc].dir, bm = ct[bc].m[d] - coff(j - 1);
          for (int ar = 0; ar < na; ++ar) {
            const int apr = ct[E0 + ar].p[d] - E0;
            dst[ar * nb + bi] = src[apr * pnb + bm] + AB[d] * src[ar * pnb + bm];
          }
        }
      }
    }
  }
  const int fa = P.first[s1], fb = P.first[s2];
  const size_t n = P.n;
  for (int f1 = 0; f1 < n1; ++f1)
    for (int f2 = 0; f2 < n2; ++f2) {
      const int i = fa + f1, j = fb + f2;
      const double nn = P.norma[i] * P.norma[j];
      const int k = f1 * n2 + f2;
      if (P.S) P.S[i * n + j] = P.S[j * n + i] = S[k] * nn;
      if (P.T) P.T[i * n + j] = P.T[j * n + i] = T[k] * nn;
      if (P.V) P.V[i * n + j] = P.V[j * n + i] = V[k] * nn;
    }
}

}  // namespace

cudaError_t launch_one_body(const OneBodyParams &p, cudaStream_t s) {
  const int npair = p.nsh * (p.nsh + 1) / 2;
  if (npair <= 0) return cudaSuccess;
  one_body_kernel<<<(npair + 127) / 128, 128, 0, s>>>(p);
  count_launches(1);
  return cudaGetLastError();
}

}  // namespace lgb
