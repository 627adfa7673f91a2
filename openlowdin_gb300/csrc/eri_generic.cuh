// Runtime-class electron-repulsion integrals for the heaviest quartet classes
// (total angular momentum 7 and 8: (dd|dp), (dp|dd), (dd|dd)).  Same recursion
// as eri.cuh -- Obara-Saika vertical recursion on the bra then on the ket,
// contraction, horizontal transfer on bra and ket -- with runtime loops.  The
// work arrays of a class this size (~8k doubles) do not fit in registers, so
// each thread keeps them in an explicit global scratch buffer, interleaved
// across the threads of the grid (element i of thread t at i * stride + t) so
// that the lanes of a warp touch consecutive addresses.
#pragma once
#include "common.cuh"

namespace lgb {

constexpr int kGenMaxL1 = 2 * kMaxL;                 // bra (or ket) total
constexpr int kGenNcum = (kGenMaxL1 + 1) * (kGenMaxL1 + 2) * (kGenMaxL1 + 3) / 6;  // 35
constexpr int kGenMaxL = 4 * kMaxL;                  // 8
// scratch doubles per thread (regions below)
constexpr int kGenVb = kGenNcum * (kGenMaxL + 1);             // 315
constexpr int kGenVk = kGenNcum * 70;                          // 2450 >= sum_f (L2-|f|+1)
constexpr int kGenX = 31 * 31;                                 // nE * nF for (dd|dd)
constexpr int kGenH = 2 * 1600;                                // two HRR level buffers
constexpr int kGenY = 36 * 31;                                 // after the bra transfer
constexpr int kGenOut = 36 * 36;                               // (dd|dd)
constexpr int kGenScratch = kGenVb + kGenVk + kGenX + kGenH + kGenY + kGenOut;

__device__ __forceinline__ int g_cx(int c) { return cx(c); }
__device__ __forceinline__ int g_comp(int c, int d) { return ccomp(c, d); }

// strided view of a thread's scratch region
struct Strided {
  double *p;
  size_t s;
  __device__ __forceinline__ double &operator[](int i) const { return p[(size_t)i * s]; }
};

__device__ inline void boys_f64_rt(int L, double T, double *F, const double *__restrict__ tab) {
  if (T < kBoysTMax) {
    const int i = __double2int_rn(T * (1.0 / kBoysH));
    const double mdT = i * kBoysH - T;
    const double *t = tab + i * kBoysOrders + L;
    double s = __ldg(t + kBoysTaylor - 1);
    for (int k = kBoysTaylor - 1; k >= 1; --k) s = fma(mdT * (1.0 / k), s, __ldg(t + k - 1));
    F[L] = s;
    const double e = exp(-T);
    for (int m = L - 1; m >= 0; --m) F[m] = fma(2.0 * T, F[m + 1], e) / (2 * m + 1);
  } else {
    const double e = exp(-T);
    F[0] = 0.88622692545275801365 / sqrt(T);
    const double o2T = 0.5 / T;
    for (int m = 0; m < L; ++m) F[m + 1] = ((2 * m + 1) * F[m] - e) * o2T;
  }
}

// offset of ket level-node (f, m) blocks: nodes with |f| >= 1 are stored as
// [f][e][m], m <= L2 - |f|; returns the start of f's block
__device__ __forceinline__ int ket_block(int f, int L2, int NE) {
  int off = 0;
  for (int g = 1; g < f; ++g) off += NE * (L2 - clevel(g) + 1);
  return off;
}

// Raw contracted integrals of one quartet of runtime class (la lb|lc ld) into
// out (strided), row-major (a, b, c, d).
__device__ inline void eri_generic(int la, int lb, int lc, int ld, const PairRec &bra, const PrimRec *__restrict__ pbra,
                                   const PairRec &ket, const PrimRec *__restrict__ pket, const double *boys64,
                                   double *scratch, size_t stride, int nint_out) {
  const int L1 = la + lb, L2 = lc + ld, L = L1 + L2, M = L + 1;
  const int NE = coff(L1 + 1), NF = coff(L2 + 1), E0 = coff(la), F0 = coff(lc);
  const int nE = NE - E0, nF = NF - F0;
  Strided Vb{scratch, stride};
  Strided Vk{scratch + (size_t)kGenVb * stride, stride};
  Strided X{scratch + (size_t)(kGenVb + kGenVk) * stride, stride};
  Strided H0{scratch + (size_t)(kGenVb + kGenVk + kGenX) * stride, stride};
  Strided H1{scratch + (size_t)(kGenVb + kGenVk + kGenX + kGenH / 2) * stride, stride};
  Strided Y{scratch + (size_t)(kGenVb + kGenVk + kGenX + kGenH) * stride, stride};
  Strided out{scratch + (size_t)(kGenVb + kGenVk + kGenX + kGenH + kGenY) * stride, stride};
  (void)nint_out;
  for (int i = 0; i < nE * nF; ++i) X[i] = 0.0;
  double F[kGenMaxL + 1];
  for (int ib = 0; ib < bra.nprim; ++ib) {
    const PrimRec pb = pbra[bra.prim0 + ib];
    for (int ik = 0; ik < ket.nprim; ++ik) {
      const PrimRec pk = pket[ket.prim0 + ik];
      const double p = pb.p, q = pk.p;
      const double opq = 1.0 / (p + q);
      const double rp = q * opq, rq = p * opq, rho = p * rp;
      double PA[3], WP[3], QC[3], WQ[3], PQ2 = 0;
      for (int d = 0; d < 3; ++d) {
        const double PQ = pb.P[d] - pk.P[d];
        PA[d] = pb.PA[d];
        QC[d] = pk.PA[d];
        WP[d] = -rp * PQ;
        WQ[d] = rq * PQ;
        PQ2 += PQ * PQ;
      }
      boys_f64_rt(L, rho * PQ2, F, boys64);
      const double pref = pb.Kt * pk.Kt * sqrt(opq);
      const double o2p = 0.5 * pb.inv_p, o2q = 0.5 * pk.inv_p, o2pq = 0.5 * opq;
      for (int m = 0; m <= L; ++m) Vb[m] = pref * F[m];
      for (int e = 1; e < NE; ++e) {
        const int d = cdir(e), em = cminus(e, d), ei = ccomp(e, d) - 1;
        const int emm = ei > 0 ? cminus(em, d) : 0;
        const int mmax = L - clevel(e);
        for (int m = 0; m <= mmax; ++m) {
          double v = PA[d] * Vb[em * M + m] + WP[d] * Vb[em * M + m + 1];
          if (ei > 0) v += ei * o2p * (Vb[emm * M + m] - rp * Vb[emm * M + m + 1]);
          Vb[e * M + m] = v;
        }
      }
      if (NF == 1) {
        for (int e = E0; e < NE; ++e) X[e - E0] += Vb[e * M];
        continue;
      }
      // ket nodes: block of f holds [e][m], m <= L2 - |f|
      int fblock = 0;
      for (int f = 1; f < NF; ++f) {
        const int d = cdir(f), fm = cminus(f, d), fi = ccomp(f, d) - 1;
        const int fmm = fi > 0 ? cminus(fm, d) : 0;
        const int mf = L2 - clevel(f) + 1;                  // m count of level f
        const int bm = fm > 0 ? ket_block(fm, L2, NE) : 0, mm_ = fm > 0 ? L2 - clevel(fm) + 1 : 0;
        const int bmm = fmm > 0 ? ket_block(fmm, L2, NE) : 0, mmm = fmm > 0 ? L2 - clevel(fmm) + 1 : 0;
        for (int e = 0; e < NE; ++e) {
          const int ed = ccomp(e, d);
          const int em = ed > 0 ? cminus(e, d) : 0;
          for (int m = 0; m < mf; ++m) {
            // get(e', f', m') = f' == 0 ? Vb[e' M + m'] : Vk[block(f') + e' * mcount(f') + m']
            const double x0 = fm == 0 ? Vb[e * M + m] : Vk[bm + e * mm_ + m];
            const double x1 = fm == 0 ? Vb[e * M + m + 1] : Vk[bm + e * mm_ + m + 1];
            double v = QC[d] * x0 + WQ[d] * x1;
            if (fi > 0) {
              const double y0 = fmm == 0 ? Vb[e * M + m] : Vk[bmm + e * mmm + m];
              const double y1 = fmm == 0 ? Vb[e * M + m + 1] : Vk[bmm + e * mmm + m + 1];
              v += fi * o2q * (y0 - rq * y1);
            }
            if (ed > 0) v += ed * o2pq * (fm == 0 ? Vb[em * M + m + 1] : Vk[bm + em * mm_ + m + 1]);
            Vk[fblock + e * mf + m] = v;
          }
        }
        fblock += NE * mf;
      }
      for (int f = F0; f < NF; ++f) {
        const int blk = ket_block(f, L2, NE), mf = L2 - clevel(f) + 1;
        for (int e = E0; e < NE; ++e) X[(e - E0) * nF + (f - F0)] += Vk[blk + e * mf];
      }
    }
  }
  // bra transfer: X [a over totals la..la+lb][nF] -> Y [NA][NB][nF]
  const int NA = ncart(la), NB = ncart(lb), NC = ncart(lc), ND = ncart(ld);
  if (lb == 0) {
    for (int i = 0; i < NA * nF; ++i) Y[i] = X[i];
  } else {
    Strided prev = X, cur = H0;
    int prev_nb = 1;
    for (int j = 1; j <= lb; ++j) {
      const int na = coff(la + lb - j + 1) - E0, nb = ncart(j);
      Strided dst = (j == lb) ? Y : cur;
      for (int bi = 0; bi < nb; ++bi) {
        const int b = coff(j) + bi, d = cdir(b), bm = cminus(b, d) - coff(j - 1);
        const double AB = bra.AB[d];
        for (int ar = 0; ar < (j == lb ? NA : na); ++ar) {
          const int apr = cplus(E0 + ar, d) - E0;
          for (int k = 0; k < nF; ++k)
            dst[(ar * nb + bi) * nF + k] = prev[(apr * prev_nb + bm) * nF + k] + AB * prev[(ar * prev_nb + bm) * nF + k];
        }
      }
      prev = dst;
      prev_nb = nb;
      cur = (cur.p == H0.p) ? H1 : H0;
    }
  }
  // ket transfer per (a, b) row
  for (int r = 0; r < NA * NB; ++r) {
    if (ld == 0) {
      for (int c = 0; c < NC; ++c) out[r * NC + c] = Y[r * nF + c];
      continue;
    }
    // level j writes [c over totals lc..lc+ld-j][d of level j] into H0 (odd j)
    // or H1 (even j) and reads level j-1 (level 0 is the row of Y)
    int prev_nd = 1;
    for (int j = 1; j <= ld; ++j) {
      const int nc = coff(lc + ld - j + 1) - F0, nd = ncart(j);
      const Strided dst = (j & 1) ? H0 : H1;
      const Strided src = (j & 1) ? H1 : H0;
      for (int di = 0; di < nd; ++di) {
        const int dd = coff(j) + di, d = cdir(dd), dm = cminus(dd, d) - coff(j - 1);
        const double CD = ket.AB[d];
        for (int cr = 0; cr < (j == ld ? NC : nc); ++cr) {
          const int cpr = cplus(F0 + cr, d) - F0;
          const double v1 = j == 1 ? Y[r * nF + cpr] : src[cpr * prev_nd + dm];
          const double v0 = j == 1 ? Y[r * nF + cr] : src[cr * prev_nd + dm];
          const double v = v1 + CD * v0;
          if (j == ld) out[(r * NC + cr) * ND + di] = v;
          else dst[cr * nd + di] = v;
        }
      }
      prev_nd = nd;
    }
  }
}

}  // namespace lgb
