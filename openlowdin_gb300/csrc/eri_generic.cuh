// Cooperative electron-repulsion integrals for the heavy quartet classes
// (total angular momentum above kTemplatedMaxL).  Same recursion as eri.cuh --
// Obara-Saika vertical recursion on the bra then on the ket, contraction,
// horizontal transfer on bra and ket -- with runtime loops: the threads of a
// group (a warp) evaluate one quartet together, every recursion level split
// across the threads, the work arrays in shared memory.
#pragma once
#include "common.cuh"

namespace lgb {

constexpr int kGenMaxL = 4 * kMaxL;   // largest total angular momentum of a quartet

// Cartesian index table (cumulative index c through total 2 kMaxL, the largest
// pair total): total, exponents, recursion axis, c - 1_d and c + 1_d (below
// the top total).  The cooperative kernels copy it to shared memory; the
// runtime forms of clevel / cx / cminus ... loop.
struct CartInfo {
  unsigned char lev, xyz[3], dir, m[3], p[3], pad;
};
constexpr int kCartTop = 2 * kMaxL;          // largest total of the table
constexpr int kCartN = coff(kCartTop + 1);
struct CartTable {
  CartInfo e[kCartN];
};
__host__ __device__ constexpr CartTable make_cart_table() {
  CartTable t{};
  for (int c = 0; c < kCartN; ++c) {
    CartInfo &q = t.e[c];
    q.lev = (unsigned char)clevel(c);
    q.xyz[0] = (unsigned char)cx(c);
    q.xyz[1] = (unsigned char)cy(c);
    q.xyz[2] = (unsigned char)cz(c);
    q.dir = (unsigned char)cdir(c);
    for (int d = 0; d < 3; ++d) {
      q.m[d] = (unsigned char)(ccomp(c, d) > 0 ? cminus(c, d) : 0);
      q.p[d] = (unsigned char)(clevel(c) < kCartTop ? cplus(c, d) : 0);
    }
    q.pad = 0;
  }
  return t;
}
__device__ const CartTable kCartTable = make_cart_table();

// copy of the table in shared memory, filled by the whole block
__device__ __forceinline__ const CartInfo *cart_shared(CartInfo *dst) {
  for (int i = threadIdx.x; i < kCartN; i += blockDim.x) dst[i] = kCartTable.e[i];
  __syncthreads();
  return dst;
}
// Work arrays of one quartet evaluation, sized for its class (offsets in
// doubles): bra nodes Vb[e][m], ket nodes Vk (blocks [f][e][m]), the
// contracted X[e][f], two buffers H0 / H1 for the intermediate
// horizontal-transfer levels (level j writes H[(j - 1) & 1], reads
// H[j & 1] of level j - 1), Y after the bra transfer, the integrals, scalars
// of the primitive quartet, ket block offsets (ints).
struct CoLayout {
  int vb, vk, x, h0, h1, y, out, misc, kb, total;
};
constexpr int kCoMiscN = 32;
constexpr int kCoKbN = (kCartN + 2) / 2;   // doubles holding kCartN + 1 ints

__host__ __device__ inline CoLayout co_layout(int la, int lb, int lc, int ld) {
  const int L1 = la + lb, L2 = lc + ld, L = L1 + L2;
  const int NE = coff(L1 + 1), NF = coff(L2 + 1), nE = NE - coff(la), nF = NF - coff(lc);
  const int NA = ncart(la), NB = ncart(lb), NC = ncart(lc), ND = ncart(ld);
  int nvk = 0;
  for (int f = 1; f < NF; ++f) nvk += NE * (L2 - clevel(f) + 1);
  // intermediate transfer levels j < lb (bra) and j < ld (ket)
  int hmax = 0;
  for (int j = 1; j < lb; ++j) {
    const int s = (coff(la + lb - j + 1) - coff(la)) * ncart(j) * nF;
    hmax = s > hmax ? s : hmax;
  }
  for (int j = 1; j < ld; ++j) {
    const int s = NA * NB * (coff(lc + ld - j + 1) - coff(lc)) * ncart(j);
    hmax = s > hmax ? s : hmax;
  }
  CoLayout o;
  o.vb = 0;
  o.vk = o.vb + NE * (L + 1);
  o.x = o.vk + nvk;
  o.h0 = o.x + nE * nF;
  o.h1 = o.h0 + hmax;
  o.y = o.h1 + hmax;
  o.out = o.y + NA * NB * nF;
  o.misc = o.out + NA * NB * NC * ND;
  o.kb = o.misc + kCoMiscN;
  o.total = (o.kb + kCoKbN + 1) & ~1;   // keep 16-byte alignment between groups
  return o;
}

// cooperating threads: a warp (one quartet per warp) or a whole CTA
struct WarpGroup {
  __device__ __forceinline__ int tid() const { return threadIdx.x & 31; }
  __device__ __forceinline__ int nt() const { return 32; }
  __device__ __forceinline__ void sync() const { __syncwarp(); }
};

__device__ inline void boys_f64_rt(int L, double T, double *F, const double *__restrict__ tab) {
  if (T < kBoysTMax) {
    const int i = __double2int_rn(T * (1.0 / kBoysH));
    const double mdT = i * kBoysH - T;
    const double *t = tab + kBoysScaledOff + (L * kBoysPoints + i) * kBoysSRow;
    double s = __ldg(t + kBoysTaylor - 1);
    for (int k = kBoysTaylor - 1; k >= 1; --k) s = fma(s, mdT, __ldg(t + k - 1));
    F[L] = s;
    const double e = __ldg(t + kBoysTaylor) * exp_small(mdT);
    for (int m = L - 1; m >= 0; --m) F[m] = fma(2.0 * T, F[m + 1], e) / (2 * m + 1);
  } else {
    const double e = T < 46.0 ? exp(-T) : 0.0;   // below 1.1e-20 above T = 46
    const double r = rsqrt(T);
    F[0] = 0.88622692545275801365 * r;
    const double o2T = 0.5 * r * r;
    for (int m = 0; m < L; ++m) F[m + 1] = ((2 * m + 1) * F[m] - e) * o2T;
  }
}

// Auxiliary integrals of the contracted Gaussian geminal sum_k c_k exp(-g_k r12^2)
// in the units of the Coulomb ones: with the Coulomb prefactor
// 2 pi^{5/2} K_ab K_cd / (p q sqrt(p+q)) outside,
//   F[m] = sqrt(pi)/2 sum_k c_k rho (rho+g_k)^{-3/2} (g_k/(rho+g_k))^m exp(-g_k T/(rho+g_k)),
// the m-th (-d/dT) derivative of the Gaussian product integral at
// T = rho |PQ|^2, which the Obara-Saika recursion consumes unchanged for any
// operator of r12.  gem = {count, g_0..g_{n-1}, c_0..c_{n-1}}.
__device__ inline void geminal_aux(int L, double rho, double T, const double *__restrict__ gem, double *F) {
  const int n = (int)gem[0];
  for (int m = 0; m <= L; ++m) F[m] = 0.0;
  for (int k = 0; k < n; ++k) {
    const double gk = gem[1 + k], ck = gem[1 + n + k];
    const double t = 1.0 / (rho + gk);
    const double r = gk * t;
    double v = 0.88622692545275801365 * ck * rho * t * sqrt(t) * exp(-gk * t * T);
    for (int m = 0; m <= L; ++m) {
      F[m] += v;
      v *= r;
    }
  }
}

// Raw contracted integrals of one quartet of runtime class (la lb|lc ld),
// evaluated by the threads of group g together; result in sm[Lo.out ...],
// row-major (a, b, c, d).  Every thread of the group must call it (it
// synchronises the group); the result is valid after the call returns.
// GEM: the operator is the geminal `gem` (geminal_aux) instead of 1/r12.
template <typename G, bool GEM = false>
__device__ inline void eri_coop(G g, const CartInfo *__restrict__ ct, const CoLayout &Lo, int la, int lb, int lc,
                                int ld, const PairRec &bra, const PrimRec *__restrict__ pbra, const PairRec &ket,
                                const PrimRec *__restrict__ pket, const double *boys64, double *sm,
                                const double *gem = nullptr) {
  const int tid = g.tid(), nt = g.nt();
  const int L1 = la + lb, L2 = lc + ld, L = L1 + L2, M = L + 1;
  const int NE = coff(L1 + 1), NF = coff(L2 + 1), E0 = coff(la), F0 = coff(lc);
  const int nE = NE - E0, nF = NF - F0;
  double *Vb = sm + Lo.vb, *Vk = sm + Lo.vk, *X = sm + Lo.x, *Y = sm + Lo.y, *out = sm + Lo.out;
  double *Hb[2] = {sm + Lo.h0, sm + Lo.h1};
  double *misc = sm + Lo.misc;
  int *kb = reinterpret_cast<int *>(sm + Lo.kb);
  g.sync();   // the previous quartet's readers of the work arrays are done
  for (int i = tid; i < nE * nF; i += nt) X[i] = 0.0;
  if (tid == 0) {
    // first Vk entry of ket node f (nodes with |f| >= 1, blocks [e][m], m <= L2 - |f|)
    int off = 0;
    for (int f = 1; f < NF; ++f) {
      kb[f] = off;
      off += NE * (L2 - ct[f].lev + 1);
    }
  }
  for (int ib = 0; ib < bra.nprim; ++ib)
    for (int ik = 0; ik < ket.nprim; ++ik) {
      g.sync();
      if (tid == 0) {
        const PrimRec pb = pbra[bra.prim0 + ib];
        const PrimRec pk = pket[ket.prim0 + ik];
        const double p = pb.p, q = pk.p;
        const double opq = 1.0 / (p + q);
        const double rp = q * opq, rq = p * opq, rho = p * rp;
        double PQ2 = 0;
        for (int d = 0; d < 3; ++d) {
          const double PQ = pb.P[d] - pk.P[d];
          misc[d] = pb.PA[d];          // PA
          misc[3 + d] = -rp * PQ;      // WP
          misc[6 + d] = pk.PA[d];      // QC
          misc[9 + d] = rq * PQ;       // WQ
          PQ2 += PQ * PQ;
        }
        misc[12] = rp;
        misc[13] = rq;
        misc[14] = 0.5 * pb.inv_p;
        misc[15] = 0.5 * pk.inv_p;
        misc[16] = 0.5 * opq;
        double F[kGenMaxL + 1];
        if constexpr (GEM) geminal_aux(L, rho, rho * PQ2, gem, F);
        else boys_f64_rt(L, rho * PQ2, F, boys64);
        const double pref = pb.Kt * pk.Kt * sqrt(opq);
        for (int m = 0; m <= L; ++m) Vb[m] = pref * F[m];
      }
      g.sync();
      const double rp = misc[12], rq = misc[13], o2p = misc[14], o2q = misc[15], o2pq = misc[16];
      // bra vertical recursion, one angular-momentum level at a time
      for (int lev = 1; lev <= L1; ++lev) {
        const int e0 = coff(lev), mm = L - lev + 1;
        for (int idx = tid; idx < ncart(lev) * mm; idx += nt) {
          const int e = e0 + idx / mm, m = idx % mm;
          const int d = ct[e].dir, em = ct[e].m[d], ei = ct[e].xyz[d] - 1;
          double v = misc[d] * Vb[em * M + m] + misc[3 + d] * Vb[em * M + m + 1];
          if (ei > 0) {
            const int emm = ct[em].m[d];
            v += ei * o2p * (Vb[emm * M + m] - rp * Vb[emm * M + m + 1]);
          }
          Vb[e * M + m] = v;
        }
        g.sync();
      }
      if (NF == 1) {
        for (int i = tid; i < nE; i += nt) X[i] += Vb[(E0 + i) * M];
        continue;
      }
      // ket vertical recursion by level
      for (int lev = 1; lev <= L2; ++lev) {
        const int f0 = coff(lev), mf = L2 - lev + 1, per = NE * mf;
        for (int idx = tid; idx < ncart(lev) * per; idx += nt) {
          const int f = f0 + idx / per, rem = idx % per, e = rem / mf, m = rem % mf;
          const int d = ct[f].dir, fm = ct[f].m[d], fi = ct[f].xyz[d] - 1;
          const int mfm = L2 - ct[fm].lev + 1;
          const double x0 = fm == 0 ? Vb[e * M + m] : Vk[kb[fm] + e * mfm + m];
          const double x1 = fm == 0 ? Vb[e * M + m + 1] : Vk[kb[fm] + e * mfm + m + 1];
          double v = misc[6 + d] * x0 + misc[9 + d] * x1;
          if (fi > 0) {
            const int fmm = ct[fm].m[d], mfmm = L2 - ct[fmm].lev + 1;
            const double y0 = fmm == 0 ? Vb[e * M + m] : Vk[kb[fmm] + e * mfmm + m];
            const double y1 = fmm == 0 ? Vb[e * M + m + 1] : Vk[kb[fmm] + e * mfmm + m + 1];
            v += fi * o2q * (y0 - rq * y1);
          }
          const int ed = ct[e].xyz[d];
          if (ed > 0) {
            const int em = ct[e].m[d];
            v += ed * o2pq * (fm == 0 ? Vb[em * M + m + 1] : Vk[kb[fm] + em * mfm + m + 1]);
          }
          Vk[kb[f] + e * mf + m] = v;
        }
        g.sync();
      }
      for (int i = tid; i < nE * nF; i += nt) {
        const int e = E0 + i / nF, f = F0 + i % nF;
        X[i] += Vk[kb[f] + e * (L2 - ct[f].lev + 1)];
      }
    }
  g.sync();
  // bra transfer: X [a over totals la..la+lb][nF] -> Y [NA][NB][nF]
  const int NA = ncart(la), NB = ncart(lb), NC = ncart(lc), ND = ncart(ld);
  if (lb == 0) {
    for (int i = tid; i < NA * nF; i += nt) Y[i] = X[i];
    g.sync();
  } else {
    for (int j = 1; j <= lb; ++j) {
      const int na = (j == lb) ? NA : coff(la + lb - j + 1) - E0, nb = ncart(j), pnb = j == 1 ? 1 : ncart(j - 1);
      // level j reads level j - 1 (X, or the other H buffer) and writes H or Y
      const double *src = j == 1 ? X : Hb[j & 1];
      double *dst = j == lb ? Y : Hb[(j - 1) & 1];
      for (int idx = tid; idx < na * nb * nF; idx += nt) {
        const int ar = idx / (nb * nF), rem = idx % (nb * nF), bi = rem / nF, k = rem % nF;
        const int b = coff(j) + bi, d = ct[b].dir, bm = ct[b].m[d] - coff(j - 1);
        const int apr = ct[E0 + ar].p[d] - E0;
        dst[(ar * nb + bi) * nF + k] = src[(apr * pnb + bm) * nF + k] + bra.AB[d] * src[(ar * pnb + bm) * nF + k];
      }
      g.sync();
    }
  }
  // ket transfer for every (a, b) row: Y [row][nF] -> out [row][NC][ND]
  const int R = NA * NB;
  if (ld == 0) {
    for (int i = tid; i < R * NC; i += nt) out[i] = Y[(i / NC) * nF + i % NC];
    g.sync();
  } else {
    for (int j = 1; j <= ld; ++j) {
      const int nc = (j == ld) ? NC : coff(lc + ld - j + 1) - F0, nd = ncart(j), pnd = j == 1 ? 1 : ncart(j - 1);
      for (int idx = tid; idx < R * nc * nd; idx += nt) {
        const int r = idx / (nc * nd), rem = idx % (nc * nd), cr = rem / nd, di = rem % nd;
        const int dd = coff(j) + di, d = ct[dd].dir, dm = ct[dd].m[d] - coff(j - 1);
        const int cpr = ct[F0 + cr].p[d] - F0;
        double v1, v0;
        if (j == 1) {
          v1 = Y[r * nF + cpr];
          v0 = Y[r * nF + cr];
        } else {
          // level j - 1 lives in Hb[j & 1] as [r][c][d'] with c over totals lc..lc+ld-j+1
          const double *Hp = Hb[j & 1];
          const int pnc = coff(lc + ld - (j - 1) + 1) - F0;
          v1 = Hp[(r * pnc + cpr) * pnd + dm];
          v0 = Hp[(r * pnc + cr) * pnd + dm];
        }
        const double v = v1 + ket.AB[d] * v0;
        if (j == ld) out[(r * NC + cr) * ND + di] = v;
        else Hb[(j - 1) & 1][(r * nc + cr) * nd + di] = v;
      }
      g.sync();
    }
  }
}

}  // namespace lgb
