// Class-templated electron-repulsion integrals over contracted Cartesian
// Gaussians, one shell quartet per thread.
//
// Scheme (published recursions, written for this library):
//   [00|00]^(m) = 2 pi^{5/2} / (p q sqrt(p+q)) K_ab K_cd F_m(rho |PQ|^2)
//   Obara-Saika vertical recursion, first on the bra
//     [e+1_i,0|00]^(m) = PA_i [e0|00]^(m) + WP_i [e0|00]^(m+1)
//                       + e_i/(2p) ([e-1_i,0|00]^(m) - rho/p [e-1_i,0|00]^(m+1))
//   then on the ket
//     [e0|f+1_i,0]^(m) = QC_i [e0|f0]^(m) + WQ_i [e0|f0]^(m+1)
//                       + f_i/(2q) ([e0|f-1_i,0]^(m) - rho/q [e0|f-1_i,0]^(m+1))
//                       + e_i/(2(p+q)) [e-1_i,0|f0]^(m+1)
//   contraction over primitive pairs of [e0|f0]^(0), |e| in [la, la+lb],
//   |f| in [lc, lc+ld], then the horizontal transfer
//     (a, b+1_i| = (a+1_i, b| + AB_i (a, b|   on the bra and the same on the ket.
// Every index is a compile-time constant (sfor), so the arrays below are
// scalarised into registers by the compiler.  The integrals are "raw": the
// contraction coefficients carry the primitive normalisation of the x^l
// component, the per-component renormalisation is applied by the callers.
#pragma once
#include "common.cuh"

namespace lgb {

template <int LA, int LB, int LC, int LD>
struct QClass {
  static constexpr int L1 = LA + LB, L2 = LC + LD, L = L1 + L2;
  static constexpr int NA = ncart(LA), NB = ncart(LB), NC = ncart(LC), ND = ncart(LD);
  static constexpr int NE = coff(L1 + 1), NF = coff(L2 + 1);
  static constexpr int E0 = coff(LA), F0 = coff(LC);
  static constexpr int nE = NE - E0, nF = NF - F0;
  static constexpr int NINT = NA * NB * NC * ND;
};

// Accumulate one primitive quartet into X[(e-E0)*nF + (f-F0)].
template <typename R, int LA, int LB, int LC, int LD>
__device__ __forceinline__ void vrr_prim(R (&X)[QClass<LA, LB, LC, LD>::nE * QClass<LA, LB, LC, LD>::nF],
                                         const PrimT<R> &pb, const PrimT<R> &pk, const double *boys64,
                                         const float *boys32) {
  using QC_ = QClass<LA, LB, LC, LD>;
  constexpr int L = QC_::L, L2 = QC_::L2, NE = QC_::NE, NF = QC_::NF, E0 = QC_::E0, F0 = QC_::F0,
                nF = QC_::nF;
  const R p = pb.p, q = pk.p;
  const R rs = rsqrt_r(p + q);    // 1 / sqrt(p + q)
  const R opq = rs * rs;
  const R rp = q * opq;          // rho / p
  const R rq = p * opq;          // rho / q
  const R rho = p * rp;          // p q / (p + q)
  R PQ2 = 0, PA[3], WP[3], QCv[3], WQ[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const R PQ = pb.P[d] - pk.P[d];
    PA[d] = pb.PA[d];
    QCv[d] = pk.PA[d];
    WP[d] = -rp * PQ;            // W - P = q (Q - P) / (p + q)
    WQ[d] = rq * PQ;             // W - Q = p (P - Q) / (p + q)
    PQ2 += PQ * PQ;
  }
  R F[L + 1];
  BoysTab<R>::template eval<L>(rho * PQ2, F, boys64, boys32);
  // 2 pi^{5/2} K_ab K_cd / (p q sqrt(p + q)) with the constants folded into Kt
  const R pref = pb.Kt * pk.Kt * rs;
  const R o2p = R(0.5) * pb.inv_p, o2q = R(0.5) * pk.inv_p, o2pq = R(0.5) * opq;

  // bra nodes Vb[e][m], m <= L - |e|
  R Vb[NE][L + 1];
#pragma unroll
  for (int m = 0; m <= L; ++m) Vb[0][m] = pref * F[m];
  sfor<1, NE>([&](auto ec) {
    constexpr int e = decltype(ec)::value;
    constexpr int d = cdir(e), em = cminus(e, d), ei = ccomp(e, d) - 1;
    constexpr int emm = ei > 0 ? cminus(em, d) : 0;
    constexpr int mmax = L - clevel(e);
#pragma unroll
    for (int m = 0; m <= mmax; ++m) {
      R v = PA[d] * Vb[em][m] + WP[d] * Vb[em][m + 1];
      if constexpr (ei > 0) v += R(ei) * o2p * (Vb[emm][m] - rp * Vb[emm][m + 1]);
      Vb[e][m] = v;
    }
  });
  if constexpr (NF == 1) {
    sfor<E0, NE>([&](auto ec) {
      constexpr int e = decltype(ec)::value;
      X[e - E0] += Vb[e][0];
    });
  } else {
    // ket nodes Vk[e][f][m], |f| >= 1, m <= L2 - |f|
    R Vk[NE][NF][L2 + 1];
    auto get = [&](auto ec, auto fc, int m) -> R {
      constexpr int e = decltype(ec)::value, f = decltype(fc)::value;
      if constexpr (f == 0) return Vb[e][m];
      else return Vk[e][f][m];
    };
    sfor<1, NF>([&](auto fc) {
      constexpr int f = decltype(fc)::value;
      constexpr int d = cdir(f), fm = cminus(f, d), fi = ccomp(f, d) - 1;
      constexpr int fmm = fi > 0 ? cminus(fm, d) : 0;
      constexpr int mmax = L2 - clevel(f);
      sfor<0, NE>([&](auto ec) {
        constexpr int e = decltype(ec)::value;
        constexpr int ed = ccomp(e, d);
        constexpr int em = ed > 0 ? cminus(e, d) : 0;
#pragma unroll
        for (int m = 0; m <= mmax; ++m) {
          R v = QCv[d] * get(ec, std::integral_constant<int, fm>{}, m) +
                WQ[d] * get(ec, std::integral_constant<int, fm>{}, m + 1);
          if constexpr (fi > 0)
            v += R(fi) * o2q *
                 (get(ec, std::integral_constant<int, fmm>{}, m) - rq * get(ec, std::integral_constant<int, fmm>{}, m + 1));
          if constexpr (ed > 0)
            v += R(ed) * o2pq * get(std::integral_constant<int, em>{}, std::integral_constant<int, fm>{}, m + 1);
          Vk[e][f][m] = v;
        }
      });
    });
    sfor<E0, NE>([&](auto ec) {
      constexpr int e = decltype(ec)::value;
      sfor<F0, NF>([&](auto fc) {
        constexpr int f = decltype(fc)::value;
        X[(e - E0) * nF + (f - F0)] += Vk[e][f][0];
      });
    });
  }
}

// Horizontal transfer on the leading (bra) index.
//   in : [cumulative index over totals LA..LA+LB, offset by coff(LA)][NK]
//   out: [ncart(LA)][ncart(LB)][NK]
template <typename R, int LA, int LB, int NK>
__device__ __forceinline__ void hrr(const R *in, const R (&AB)[3], R *out) {
  constexpr int A0 = coff(LA);
  constexpr int nA = coff(LA + LB + 1) - A0;
  if constexpr (LB == 0) {
#pragma unroll
    for (int i = 0; i < ncart(LA) * NK; ++i) out[i] = in[i];
  } else {
    // level buffers H[j][a][b][k]
    R H[LB + 1][nA][ncart(LB)][NK];
#pragma unroll
    for (int a = 0; a < nA; ++a)
#pragma unroll
      for (int k = 0; k < NK; ++k) H[0][a][0][k] = in[a * NK + k];
    sfor<1, LB + 1>([&](auto jc) {
      constexpr int j = decltype(jc)::value;
      constexpr int na = coff(LA + LB - j + 1) - A0;
      sfor<0, ncart(j)>([&](auto bc) {
        constexpr int bi = decltype(bc)::value;
        constexpr int b = coff(j) + bi;
        constexpr int d = cdir(b);
        constexpr int bm = cminus(b, d) - coff(j - 1);
        sfor<0, na>([&](auto ac) {
          constexpr int ar = decltype(ac)::value;
          constexpr int apr = cplus(A0 + ar, d) - A0;
#pragma unroll
          for (int k = 0; k < NK; ++k) H[j][ar][bi][k] = H[j - 1][apr][bm][k] + AB[d] * H[j - 1][ar][bm][k];
        });
      });
    });
#pragma unroll
    for (int a = 0; a < ncart(LA); ++a)
#pragma unroll
      for (int b = 0; b < ncart(LB); ++b)
#pragma unroll
        for (int k = 0; k < NK; ++k) out[(a * ncart(LB) + b) * NK + k] = H[LB][a][b][k];
  }
}

// Horizontal transfer on the trailing (ket) index of rows [NROW][...].
template <typename R, int LC, int LD, int NROW>
__device__ __forceinline__ void hrr_ket(const R *in, const R (&CD)[3], R *out) {
  constexpr int C0 = coff(LC);
  constexpr int nC = coff(LC + LD + 1) - C0;
  if constexpr (LD == 0) {
#pragma unroll
    for (int i = 0; i < NROW * ncart(LC); ++i) out[i] = in[i];
  } else {
    R H[LD + 1][NROW][nC][ncart(LD)];
#pragma unroll
    for (int r = 0; r < NROW; ++r)
#pragma unroll
      for (int c = 0; c < nC; ++c) H[0][r][c][0] = in[r * nC + c];
    sfor<1, LD + 1>([&](auto jc) {
      constexpr int j = decltype(jc)::value;
      constexpr int nc = coff(LC + LD - j + 1) - C0;
      sfor<0, ncart(j)>([&](auto dc) {
        constexpr int di = decltype(dc)::value;
        constexpr int dd = coff(j) + di;
        constexpr int d = cdir(dd);
        constexpr int dm = cminus(dd, d) - coff(j - 1);
        sfor<0, nc>([&](auto cc) {
          constexpr int cr = decltype(cc)::value;
          constexpr int cpr = cplus(C0 + cr, d) - C0;
#pragma unroll
          for (int r = 0; r < NROW; ++r) H[j][r][cr][di] = H[j - 1][r][cpr][dm] + CD[d] * H[j - 1][r][cr][dm];
        });
      });
    });
#pragma unroll
    for (int r = 0; r < NROW; ++r)
#pragma unroll
      for (int c = 0; c < ncart(LC); ++c)
#pragma unroll
        for (int d = 0; d < ncart(LD); ++d) out[(r * ncart(LC) + c) * ncart(LD) + d] = H[LD][r][c][d];
  }
}

// Full contracted quartet: out[NA*NB*NC*ND] row-major (a, b, c, d).  pbra and
// pket point at the first primitive pair of the bra and of the ket pair (they
// may come from different species, and from global or shared memory).
template <typename R, int LA, int LB, int LC, int LD>
__device__ __forceinline__ void eri_quartet(const PairT<R> &bra, const PrimT<R> *pbra, const PairT<R> &ket,
                                            const PrimT<R> *pket,
                                            const double *boys64, const float *boys32,
                                            R (&out)[QClass<LA, LB, LC, LD>::NINT]) {
  using QC_ = QClass<LA, LB, LC, LD>;
  R X[QC_::nE * QC_::nF];
#pragma unroll
  for (int i = 0; i < QC_::nE * QC_::nF; ++i) X[i] = R(0);
  for (int ib = 0; ib < bra.nprim; ++ib) {
    const PrimT<R> pb = pbra[ib];
    for (int ik = 0; ik < ket.nprim; ++ik) {
      const PrimT<R> pk = pket[ik];
      vrr_prim<R, LA, LB, LC, LD>(X, pb, pk, boys64, boys32);
    }
  }
  const R AB[3] = {bra.AB[0], bra.AB[1], bra.AB[2]};
  const R CD[3] = {ket.AB[0], ket.AB[1], ket.AB[2]};
  R Y[QC_::NA * QC_::NB * QC_::nF];
  hrr<R, LA, LB, QC_::nF>(X, AB, Y);
  hrr_ket<R, LC, LD, QC_::NA * QC_::NB>(Y, CD, out);
}

// The same with a one-primitive ket pair whose primitive is passed by value
// (the FP32 row kernels assemble it in registers from structure-of-arrays
// fields).
template <typename R, int LA, int LB, int LC, int LD>
__device__ __forceinline__ void eri_quartet_k1(const PairT<R> &bra, const PrimT<R> *pbra, const PairT<R> &ket,
                                               const PrimT<R> &pk, const double *boys64, const float *boys32,
                                               R (&out)[QClass<LA, LB, LC, LD>::NINT]) {
  using QC_ = QClass<LA, LB, LC, LD>;
  R X[QC_::nE * QC_::nF];
#pragma unroll
  for (int i = 0; i < QC_::nE * QC_::nF; ++i) X[i] = R(0);
  for (int ib = 0; ib < bra.nprim; ++ib) {
    const PrimT<R> pb = pbra[ib];
    vrr_prim<R, LA, LB, LC, LD>(X, pb, pk, boys64, boys32);
  }
  const R AB[3] = {bra.AB[0], bra.AB[1], bra.AB[2]};
  const R CD[3] = {ket.AB[0], ket.AB[1], ket.AB[2]};
  R Y[QC_::NA * QC_::NB * QC_::nF];
  hrr<R, LA, LB, QC_::nF>(X, AB, Y);
  hrr_ket<R, LC, LD, QC_::NA * QC_::NB>(Y, CD, out);
}

}  // namespace lgb
