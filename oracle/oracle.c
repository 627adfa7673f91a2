/*
 * oracle.c -- CPU FP64 restatement of openLOWDIN's direct two-particle path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the GPU library: it is
 * linked by tests/, by __graft_entry__.smoke() and by the CPU-baseline leg of
 * bench.py, never by the product path (openlowdin_gb300/).
 *
 * What it restates (reference paths are relative to the openLOWDIN tree):
 *   - primitive normalisation of a shell and per-Cartesian renormalisation
 *       src/ints/Libint2Iface.cpp:79-128 (add_shell, `norma`),
 *       src/core/ContractedGaussian.f90:353-411, Cartesian order :786-812
 *   - significant shell-pair list        src/ints/Libint2Iface.cpp:3248-3342
 *   - Schwarz factors Q(s1,s2)           src/ints/Libint2Iface.cpp:3345-3412
 *   - shell-block infinity norms of D    src/ints/Libint2Iface.cpp:143-161
 *   - direct intra-species G matrix      src/ints/Libint2Iface.cpp:418-618
 *   - direct first-quarter transform     src/ints/Libint2Iface.cpp:620-921,
 *                                        src/ints/Iterators.cpp:13-181
 *   - direct inter-species coupling      src/ints/Libint2Iface.cpp:1111-1294, 3566-3589
 *   - coupling first-quarter transform   src/ints/Libint2Iface.cpp:1296-1622, 3591-3620
 *   - direct geminal (G12) matrices      src/ints/Libint2Iface.cpp:2193-2540, 3687-3734
 *     (intra-species and inter-species, operator sum_k c_k exp(-g_k r12^2))
 * The ERI arithmetic itself lives in libint2 in the reference (third party, not
 * vendored; pinned at commit 668b10c4bdca5876984058742d4212675eb93f3f by the
 * reference's CI).  It is restated here from the published Obara-Saika recursion
 * (Obara & Saika, J. Chem. Phys. 84, 3963 (1986)) with the horizontal transfer of
 * Head-Gordon & Pople (J. Chem. Phys. 89, 5777 (1988)); the Boys function is
 * evaluated from its series definition and the large-argument closed form.
 * One-electron integrals (overlap, kinetic, point-charge attraction) follow the
 * same Obara-Saika recursions (the reference computes them in
 * src/ints/{Overlap,Kinetic,Attraction}Integrals.f90).
 *
 * Not restated: libint2's primitive-quartet truncation (engine precision
 * min(eps/max|D|, eps)/nprim^4, Libint2Iface.cpp:443-454); it changes integrals
 * only below 1e-16 relative.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <float.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OR_MAXL 4            /* per-shell angular momentum (g) */
#define OR_MAXPRIM 32
#define OR_MAXLT (4 * OR_MAXL) /* total L of a quartet */

typedef struct {
  int l, nprim;
  double O[3];
  double alpha[OR_MAXPRIM];
  double cn[OR_MAXPRIM]; /* contraction coefficient x primitive norm of x^l */
} or_shell;

typedef struct {
  int nshell, nbf, max_l, max_nprim;
  or_shell *sh;
  int *first; /* shell -> first basis function */
  double *norma;
} or_basis;

static int ncart(int l) { return (l + 1) * (l + 2) / 2; }
static int cart_off(int k) { return k * (k + 1) * (k + 2) / 6; }
/* cumulative index of x^a y^b z^c over all totals; lowdin order within a total:
   for i=0..k: x=k-i, for j=0..i: y=i-j, z=j  (ContractedGaussian.f90:800-809) */
static int cidx(int x, int y, int z) {
  int k = x + y + z, i = y + z;
  return cart_off(k) + i * (i + 1) / 2 + z;
}

#define NCUM_MAX 165 /* cart_off(9): all Cartesians with total <= 8 */
static int g_cx[NCUM_MAX], g_cy[NCUM_MAX], g_cz[NCUM_MAX];
static int g_tables_ready = 0;
static void init_tables(void) {
  if (g_tables_ready) return;
  for (int k = 0; k <= 8; ++k)
    for (int i = 0; i <= k; ++i)
      for (int j = 0; j <= i; ++j) {
        int x = k - i, y = i - j, z = j, c = cidx(x, y, z);
        g_cx[c] = x; g_cy[c] = y; g_cz[c] = z;
      }
  g_tables_ready = 1;
}

/* ---------------------------------------------------------------- Boys ---- */
/* F_m(T) = int_0^1 t^{2m} exp(-T t^2) dt, m = 0..mmax.
   T < 40: series F_M(T) = e^{-T} sum_k (2T)^k / ((2M+1)(2M+3)...(2M+2k+1)),
           then downward recursion F_m = (2T F_{m+1} + e^{-T}) / (2m+1).
   T >= 40: F_0 = sqrt(pi/T)/2 * erf(sqrt(T)), upward F_{m+1} = ((2m+1)F_m - e^{-T})/(2T). */
void or_boys(int mmax, double T, double *F) {
  if (T < 40.0) {
    double e = exp(-T);
    double term = 1.0 / (2 * mmax + 1), sum = term;
    for (int k = 1; k < 400; ++k) {
      term *= 2.0 * T / (2 * mmax + 2 * k + 1);
      sum += term;
      if (term < 1e-18 * sum) break;
    }
    F[mmax] = e * sum;
    for (int m = mmax - 1; m >= 0; --m) F[m] = (2.0 * T * F[m + 1] + e) / (2 * m + 1);
  } else {
    double e = exp(-T);
    F[0] = 0.5 * sqrt(M_PI / T) * erf(sqrt(T));
    for (int m = 0; m < mmax; ++m) F[m + 1] = ((2 * m + 1) * F[m] - e) / (2.0 * T);
  }
}

/* primitive normalisation of the x^l component:
   N = sqrt(2^l (2a)^{l+3/2} / (pi^{3/2} (2l-1)!!)) */
static double prim_norm(double a, int l) {
  double df = 1.0;
  for (int k = 2 * l - 1; k > 1; k -= 2) df *= k;
  return sqrt(pow(2.0, l) * pow(2.0 * a, l + 1.5) / (pow(M_PI, 1.5) * df));
}

/* ------------------------------------------------------------- overlap ---- */
/* 1-D overlap table s[i][j] for i<=li, j<=lj (Obara-Saika), without exp/pi factor */
static void ovl1d(int li, int lj, double PA, double PB, double o2p, double s[][OR_MAXL + 4]) {
  s[0][0] = 1.0;
  for (int i = 0; i <= li; ++i)
    for (int j = 0; j <= lj; ++j) {
      if (i == 0 && j == 0) continue;
      if (i > 0) {
        double v = PA * s[i - 1][j];
        if (i > 1) v += (i - 1) * o2p * s[i - 2][j];
        if (j > 0) v += j * o2p * s[i - 1][j - 1];
        s[i][j] = v;
      } else {
        double v = PB * s[i][j - 1];
        if (j > 1) v += (j - 1) * o2p * s[i][j - 2];
        s[i][j] = v;
      }
    }
}

/* raw (norma-free) contracted overlap block of two shells, out[n1*n2] row-major;
   if kin != NULL the kinetic-energy block is written there too */
static void shell_overlap_kinetic(const or_shell *A, const or_shell *B, double *out, double *kin) {
  int n1 = ncart(A->l), n2 = ncart(B->l);
  memset(out, 0, sizeof(double) * n1 * n2);
  if (kin) memset(kin, 0, sizeof(double) * n1 * n2);
  double AB2 = 0;
  for (int d = 0; d < 3; ++d) AB2 += (A->O[d] - B->O[d]) * (A->O[d] - B->O[d]);
  for (int pa = 0; pa < A->nprim; ++pa)
    for (int pb = 0; pb < B->nprim; ++pb) {
      double a = A->alpha[pa], b = B->alpha[pb], p = a + b, o2p = 0.5 / p;
      double pref = pow(M_PI / p, 1.5) * exp(-a * b / p * AB2) * A->cn[pa] * B->cn[pb];
      double s[3][OR_MAXL + 4][OR_MAXL + 4];
      for (int d = 0; d < 3; ++d) {
        double P = (a * A->O[d] + b * B->O[d]) / p;
        ovl1d(A->l, B->l + 2, P - A->O[d], P - B->O[d], o2p, s[d]);
      }
      int f1 = 0;
      for (int i1 = 0; i1 <= A->l; ++i1)
        for (int j1 = 0; j1 <= i1; ++j1, ++f1) {
          int ax = A->l - i1, ay = i1 - j1, az = j1, f2 = 0;
          for (int i2 = 0; i2 <= B->l; ++i2)
            for (int j2 = 0; j2 <= i2; ++j2, ++f2) {
              int bx = B->l - i2, by = i2 - j2, bz = j2;
              double sx = s[0][ax][bx], sy = s[1][ay][by], sz = s[2][az][bz];
              out[f1 * n2 + f2] += pref * sx * sy * sz;
              if (kin) {
                int bb[3] = {bx, by, bz}, aa[3] = {ax, ay, az};
                double t1[3];
                for (int d = 0; d < 3; ++d) {
                  int j = bb[d];
                  double v = -2.0 * b * (2 * j + 1) * s[d][aa[d]][j] + 4.0 * b * b * s[d][aa[d]][j + 2];
                  if (j >= 2) v += j * (j - 1) * s[d][aa[d]][j - 2];
                  t1[d] = -0.5 * v;
                }
                kin[f1 * n2 + f2] += pref * (t1[0] * sy * sz + sx * t1[1] * sz + sx * sy * t1[2]);
              }
            }
        }
    }
}

/* ----------------------------------------------------------------- HRR ---- */
/* Horizontal transfer (a,b+1_i| = (a+1_i,b| + AB_i (a,b|.
   in : rows over the cumulative Cartesian index of totals la..la+lb (row r holds
        index cart_off(la)+r), each row nk wide.
   out: [ncart(la)][ncart(lb)][nk]. */
static void hrr(int la, int lb, const double AB[3], const double *in, int nk, double *out, double *tmp) {
  if (lb == 0) {
    memcpy(out, in, sizeof(double) * ncart(la) * nk);
    return;
  }
  int off0 = cart_off(la);
  /* level j buffer: [a over cumulative totals la..la+lb-j][b over level j][nk] */
  const double *prev = in;
  int prev_nb = 1;
  double *bufs[2] = {tmp, tmp + (size_t)NCUM_MAX * 15 * nk};
  for (int j = 1; j <= lb; ++j) {
    int na = cart_off(la + lb - j + 1) - off0, nb = ncart(j);
    double *cur = (j == lb) ? out : bufs[j & 1];
    /* the final level writes only totals == la, i.e. the first ncart(la) rows */
    for (int bi = 0; bi < nb; ++bi) {
      int bc = cart_off(j) + bi;
      int bx = g_cx[bc], by = g_cy[bc], bz = g_cz[bc];
      int dir = bx > 0 ? 0 : (by > 0 ? 1 : 2);
      int bmx = bx - (dir == 0), bmy = by - (dir == 1), bmz = bz - (dir == 2);
      int bm = cidx(bmx, bmy, bmz) - cart_off(j - 1);
      for (int ar = 0; ar < na; ++ar) {
        int ac = off0 + ar;
        int apx = g_cx[ac] + (dir == 0), apy = g_cy[ac] + (dir == 1), apz = g_cz[ac] + (dir == 2);
        int apr = cidx(apx, apy, apz) - off0;
        const double *x1 = prev + ((size_t)apr * prev_nb + bm) * nk;
        const double *x0 = prev + ((size_t)ar * prev_nb + bm) * nk;
        if (j == lb && ar >= ncart(la)) continue;
        double *y = cur + ((size_t)ar * nb + bi) * nk;
        for (int k = 0; k < nk; ++k) y[k] = x1[k] + AB[dir] * x0[k];
      }
    }
    prev = cur;
    prev_nb = nb;
  }
}

/* ----------------------------------------------------------------- ERI ---- */
typedef struct {
  double *V;    /* VRR [e][f][m] */
  double *X;    /* contracted [e][f] */
  double *Y;    /* after bra HRR */
  double *tmp;  /* HRR scratch */
  double *raw;  /* shell quartet buffer */
  /* two-particle operator: Coulomb 1/r12 when gem_n == 0, else the contracted
     Gaussian geminal sum_k gem_c[k] exp(-gem_g[k] r12^2) */
  int gem_n;
  const double *gem_c, *gem_g;
} or_work;

static or_work *work_new(void) {
  or_work *w = (or_work *)calloc(1, sizeof(or_work));
  w->V = (double *)malloc(sizeof(double) * NCUM_MAX * NCUM_MAX * (OR_MAXLT + 1));
  w->X = (double *)malloc(sizeof(double) * NCUM_MAX * NCUM_MAX);
  w->Y = (double *)malloc(sizeof(double) * 225 * NCUM_MAX);
  w->tmp = (double *)malloc(sizeof(double) * 2 * NCUM_MAX * 15 * NCUM_MAX);
  w->raw = (double *)malloc(sizeof(double) * 15 * 15 * 15 * 15);
  return w;
}
static void work_free(or_work *w) {
  free(w->V); free(w->X); free(w->Y); free(w->tmp); free(w->raw); free(w);
}

/* Raw contracted Cartesian ERIs (ab|cd) of four shells (norma not applied).
   out[n1*n2*n3*n4], row-major in (f1,f2,f3,f4).
   Obara-Saika VRR builds [e0|f0]^(m): first on the bra, then on the ket;
   HRR then moves angular momentum to b and d. */
static void eri_shells(const or_shell *A, const or_shell *B, const or_shell *C, const or_shell *D,
                       double *out, or_work *w) {
  const int la = A->l, lb = B->l, lc = C->l, ld = D->l;
  const int L1 = la + lb, L2 = lc + ld, L = L1 + L2, M = L + 1;
  const int NE = cart_off(L1 + 1), NF = cart_off(L2 + 1);
  const int e0 = cart_off(la), f0 = cart_off(lc);
  const int nE = NE - e0, nF = NF - f0;
  double AB[3], CD[3], AB2 = 0, CD2 = 0;
  for (int d = 0; d < 3; ++d) {
    AB[d] = A->O[d] - B->O[d]; CD[d] = C->O[d] - D->O[d];
    AB2 += AB[d] * AB[d]; CD2 += CD[d] * CD[d];
  }
  double *X = w->X, *V = w->V;
  memset(X, 0, sizeof(double) * nE * nF);
  double F[OR_MAXLT + 1];
  for (int pa = 0; pa < A->nprim; ++pa)
    for (int pb = 0; pb < B->nprim; ++pb) {
      double a = A->alpha[pa], b = B->alpha[pb], p = a + b;
      double Kab = exp(-a * b / p * AB2);
      double P[3];
      for (int d = 0; d < 3; ++d) P[d] = (a * A->O[d] + b * B->O[d]) / p;
      for (int pc = 0; pc < C->nprim; ++pc)
        for (int pd = 0; pd < D->nprim; ++pd) {
          double c = C->alpha[pc], dd = D->alpha[pd], q = c + dd;
          double Kcd = exp(-c * dd / q * CD2);
          double Q[3], W[3], PA[3], WP[3], QC[3], WQ[3], PQ2 = 0;
          for (int d = 0; d < 3; ++d) {
            Q[d] = (c * C->O[d] + dd * D->O[d]) / q;
            W[d] = (p * P[d] + q * Q[d]) / (p + q);
            PA[d] = P[d] - A->O[d]; WP[d] = W[d] - P[d];
            QC[d] = Q[d] - C->O[d]; WQ[d] = W[d] - Q[d];
            PQ2 += (P[d] - Q[d]) * (P[d] - Q[d]);
          }
          double rho = p * q / (p + q);
          double wgt = A->cn[pa] * B->cn[pb] * C->cn[pc] * D->cn[pd];
          if (w->gem_n > 0) {
            /* [0|0]^(m) of exp(-g r12^2): the Gaussian product integral
               Kab Kcd (pi^2 / ((p+q)(rho+g)))^{3/2} exp(-rho g/(rho+g) |PQ|^2)
               times (g/(rho+g))^m, the m-th (-d/dT) derivative at T = rho|PQ|^2,
               which is what the Obara-Saika recursion below consumes for any
               operator of r12 (Ahlrichs, Phys. Chem. Chem. Phys. 8, 3072 (2006)) */
            for (int m = 0; m <= L; ++m) V[m] = 0.0;
            for (int k = 0; k < w->gem_n; ++k) {
              double g = w->gem_g[k], rg = rho + g;
              double base = w->gem_c[k] * Kab * Kcd * pow(M_PI * M_PI / ((p + q) * rg), 1.5) *
                            exp(-rho * g / rg * PQ2);
              double r = g / rg, t = 1.0;
              for (int m = 0; m <= L; ++m) {
                V[m] += base * t;
                t *= r;
              }
            }
          } else {
            double pref = 2.0 * pow(M_PI, 2.5) / (p * q * sqrt(p + q)) * Kab * Kcd;
            or_boys(L, rho * PQ2, F);
            /* [0|0]^(m) */
            for (int m = 0; m <= L; ++m) V[m] = pref * F[m];
          }
          double o2p = 0.5 / p, o2q = 0.5 / q, o2pq = 0.5 / (p + q), rp = rho / p, rq = rho / q;
          /* bra VRR: [e|0]^(m), m <= L-|e| */
          for (int e = 1; e < NE; ++e) {
            int ex = g_cx[e], ey = g_cy[e], ez = g_cz[e], ke = ex + ey + ez;
            int dir = ex > 0 ? 0 : (ey > 0 ? 1 : 2);
            int ei = (dir == 0 ? ex : dir == 1 ? ey : ez) - 1; /* component of e-1_dir */
            int em = cidx(ex - (dir == 0), ey - (dir == 1), ez - (dir == 2));
            int emm = ei > 0 ? cidx(ex - 2 * (dir == 0), ey - 2 * (dir == 1), ez - 2 * (dir == 2)) : 0;
            for (int m = 0; m <= L - ke; ++m) {
              double v = PA[dir] * V[(em * NF) * M + m] + WP[dir] * V[(em * NF) * M + m + 1];
              if (ei > 0)
                v += ei * o2p * (V[(emm * NF) * M + m] - rp * V[(emm * NF) * M + m + 1]);
              V[(e * NF) * M + m] = v;
            }
          }
          /* ket VRR: [e|f]^(m), m <= L-|e|-|f| */
          for (int f = 1; f < NF; ++f) {
            int fx = g_cx[f], fy = g_cy[f], fz = g_cz[f], kf = fx + fy + fz;
            int dir = fx > 0 ? 0 : (fy > 0 ? 1 : 2);
            int fi = (dir == 0 ? fx : dir == 1 ? fy : fz) - 1;
            int fm = cidx(fx - (dir == 0), fy - (dir == 1), fz - (dir == 2));
            int fmm = fi > 0 ? cidx(fx - 2 * (dir == 0), fy - 2 * (dir == 1), fz - 2 * (dir == 2)) : 0;
            for (int e = 0; e < NE; ++e) {
              int ex = g_cx[e], ey = g_cy[e], ez = g_cz[e], ke = ex + ey + ez;
              if (ke + kf > L) continue;
              int edir = (dir == 0 ? ex : dir == 1 ? ey : ez);
              int eminus = edir > 0 ? cidx(ex - (dir == 0), ey - (dir == 1), ez - (dir == 2)) : 0;
              for (int m = 0; m <= L - ke - kf; ++m) {
                double v = QC[dir] * V[(e * NF + fm) * M + m] + WQ[dir] * V[(e * NF + fm) * M + m + 1];
                if (fi > 0)
                  v += fi * o2q * (V[(e * NF + fmm) * M + m] - rq * V[(e * NF + fmm) * M + m + 1]);
                if (edir > 0) v += edir * o2pq * V[(eminus * NF + fm) * M + m + 1];
                V[(e * NF + f) * M + m] = v;
              }
            }
          }
          for (int e = e0; e < NE; ++e)
            for (int f = f0; f < NF; ++f) X[(e - e0) * nF + (f - f0)] += wgt * V[(e * NF + f) * M];
        }
    }
  /* bra HRR: X[e][f] -> Y[a][b][f] */
  int n1 = ncart(la), n2 = ncart(lb), n3 = ncart(lc), n4 = ncart(ld);
  hrr(la, lb, AB, X, nF, w->Y, w->tmp);
  /* ket HRR per (a,b) row */
  for (int ab = 0; ab < n1 * n2; ++ab) hrr(lc, ld, CD, w->Y + (size_t)ab * nF, 1, out + (size_t)ab * n3 * n4, w->tmp);
}

/* --------------------------------------------------------- basis build ---- */
/* Builds a basis from flat arrays: shell s has angular momentum ls[s], nprim[s]
   primitives starting at poff = sum nprim[<s], exponents alpha[poff..], raw file
   coefficients coef[poff..], origin origin[3s..3s+2]. Normalisation as
   Libint2Iface.cpp:79-128: primitive norm of x^l times coefficient, then
   norma[i] = 1/sqrt(S_ii) of the shell's own overlap. */
static or_basis *basis_new(int nsh, const int *ls, const int *nprim, const double *origin,
                           const double *alpha, const double *coef) {
  init_tables();
  or_basis *b = (or_basis *)calloc(1, sizeof(or_basis));
  b->nshell = nsh;
  b->sh = (or_shell *)calloc(nsh, sizeof(or_shell));
  b->first = (int *)calloc(nsh + 1, sizeof(int));
  int poff = 0, nbf = 0;
  for (int s = 0; s < nsh; ++s) {
    or_shell *S = &b->sh[s];
    S->l = ls[s]; S->nprim = nprim[s];
    for (int d = 0; d < 3; ++d) S->O[d] = origin[3 * s + d];
    for (int p = 0; p < nprim[s]; ++p) {
      S->alpha[p] = alpha[poff + p];
      S->cn[p] = coef[poff + p] * prim_norm(alpha[poff + p], ls[s]);
    }
    poff += nprim[s];
    b->first[s] = nbf;
    nbf += ncart(ls[s]);
    if (ls[s] > b->max_l) b->max_l = ls[s];
    if (nprim[s] > b->max_nprim) b->max_nprim = nprim[s];
  }
  b->first[nsh] = nbf;
  b->nbf = nbf;
  b->norma = (double *)calloc(nbf, sizeof(double));
  double buf[15 * 15];
  for (int s = 0; s < nsh; ++s) {
    int n = ncart(ls[s]);
    shell_overlap_kinetic(&b->sh[s], &b->sh[s], buf, NULL);
    for (int i = 0; i < n; ++i) b->norma[b->first[s] + i] = 1.0 / sqrt(buf[i * n + i]);
  }
  return b;
}
static void basis_free(or_basis *b) {
  free(b->sh); free(b->first); free(b->norma); free(b);
}

#define BASIS_ARGS int nsh, const int *ls, const int *nprim, const double *origin, const double *alpha, const double *coef
#define BASIS_PASS nsh, ls, nprim, origin, alpha, coef

/* ------------------------------------------------------------- exports ---- */
int or_nbasis(BASIS_ARGS) {
  or_basis *b = basis_new(BASIS_PASS);
  int n = b->nbf;
  basis_free(b);
  return n;
}

void or_norma(BASIS_ARGS, double *norma) {
  or_basis *b = basis_new(BASIS_PASS);
  memcpy(norma, b->norma, sizeof(double) * b->nbf);
  basis_free(b);
}

/* Raw ERIs of one shell quartet (shells i,j,k,l of the given basis). */
void or_eri_quartet(BASIS_ARGS, int s1, int s2, int s3, int s4, double *out) {
  or_basis *b = basis_new(BASIS_PASS);
  or_work *w = work_new();
  eri_shells(&b->sh[s1], &b->sh[s2], &b->sh[s3], &b->sh[s4], out, w);
  work_free(w);
  basis_free(b);
}

/* Primitive raw ERI set with unit coefficients and NO primitive normalisation:
   (la lb|lc ld) over one exponent per centre; used against the reference's own
   Rys code (src/ints/RysQInts.cpp coul_rep_), which returns unnormalised values. */
void or_eri_primitive(const int *l4, const double *alpha4, const double *origin12, double *out) {
  init_tables();
  or_shell S[4];
  for (int i = 0; i < 4; ++i) {
    S[i].l = l4[i]; S[i].nprim = 1; S[i].alpha[0] = alpha4[i]; S[i].cn[0] = 1.0;
    for (int d = 0; d < 3; ++d) S[i].O[d] = origin12[3 * i + d];
  }
  or_work *w = work_new();
  eri_shells(&S[0], &S[1], &S[2], &S[3], out, w);
  work_free(w);
}

/* The same primitive set for the geminal operator sum_k coef[k] exp(-expo[k] r12^2). */
void or_g12_primitive(const int *l4, const double *alpha4, const double *origin12, int npot, const double *coef,
                      const double *expo, double *out) {
  init_tables();
  or_shell S[4];
  for (int i = 0; i < 4; ++i) {
    S[i].l = l4[i]; S[i].nprim = 1; S[i].alpha[0] = alpha4[i]; S[i].cn[0] = 1.0;
    for (int d = 0; d < 3; ++d) S[i].O[d] = origin12[3 * i + d];
  }
  or_work *w = work_new();
  w->gem_n = npot;
  w->gem_c = coef;
  w->gem_g = expo;
  eri_shells(&S[0], &S[1], &S[2], &S[3], out, w);
  work_free(w);
}

/* Significant-pair mask, Libint2Iface.cpp:3248-3342: mask[s1*nsh+s2] (s2<=s1)
   is 1 when both shells sit on the same centre or the Frobenius norm of the raw
   overlap block is >= 1e-12. */
static void pair_mask(const or_basis *b, unsigned char *mask) {
  int nsh = b->nshell;

  memset(mask, 0, (size_t)nsh * nsh);
  double buf[15 * 15];
  for (int s1 = 0; s1 < nsh; ++s1)
    for (int s2 = 0; s2 <= s1; ++s2) {
      const or_shell *A = &b->sh[s1], *B = &b->sh[s2];
      int same = A->O[0] == B->O[0] && A->O[1] == B->O[1] && A->O[2] == B->O[2];
      int sig = same;
      if (!same) {
        shell_overlap_kinetic(A, B, buf, NULL);
        double nrm = 0;
        for (int i = 0; i < ncart(A->l) * ncart(B->l); ++i) nrm += buf[i] * buf[i];
        sig = sqrt(nrm) >= 1e-12;
      }
      mask[s1 * nsh + s2] = (unsigned char)sig;
    }
}

void or_pair_mask(BASIS_ARGS, unsigned char *mask) {
  or_basis *b = basis_new(BASIS_PASS);
  pair_mask(b, mask);
  basis_free(b);
}

/* Schwarz factors Q(s1,s2) = sqrt(max_i |(ab|ab)_ii|) over raw integrals,
   Libint2Iface.cpp:3345-3412 (symmetric, nsh x nsh). */
static void schwarz(const or_basis *b, double *Q, int nthreads) {
  int nsh = b->nshell;

#pragma omp parallel num_threads(nthreads)
  {
    or_work *w = work_new();
#pragma omp for schedule(dynamic)
    for (int s1 = 0; s1 < nsh; ++s1)
      for (int s2 = 0; s2 <= s1; ++s2) {
        eri_shells(&b->sh[s1], &b->sh[s2], &b->sh[s1], &b->sh[s2], w->raw, w);
        int n12 = ncart(b->sh[s1].l) * ncart(b->sh[s2].l);
        double mx = 0;
        for (int i = 0; i < n12; ++i) {
          double v = fabs(w->raw[(size_t)i * n12 + i]);
          if (v > mx) mx = v;
        }
        Q[s1 * nsh + s2] = Q[s2 * nsh + s1] = sqrt(mx);
      }
    work_free(w);
  }
}

void or_schwarz(BASIS_ARGS, double *Q, int nthreads) {
  or_basis *b = basis_new(BASIS_PASS);
  schwarz(b, Q, nthreads);
  basis_free(b);
}

/* max |D| over each shell block, Libint2Iface.cpp:143-161 */
static void shellblock_norm(const or_basis *b, const double *D, double *Dn) {
  int nsh = b->nshell;
  int n = b->nbf;
  for (int s1 = 0; s1 < nsh; ++s1)
    for (int s2 = 0; s2 < nsh; ++s2) {
      double mx = 0;
      for (int i = b->first[s1]; i < b->first[s1 + 1]; ++i)
        for (int j = b->first[s2]; j < b->first[s2 + 1]; ++j) {
          double v = fabs(D[(size_t)i * n + j]);
          if (v > mx) mx = v;
        }
      Dn[s1 * nsh + s2] = mx;
    }
}

static double dmax(double a, double b) { return a > b ? a : b; }

/* Counters of the last or_2body_direct call (quartets evaluated per class). */
static long long g_last_quartets = 0;
long long or_last_quartet_count(void) { return g_last_quartets; }

/* Direct intra-species two-particle matrix, Libint2Iface.cpp:418-618 with the
   wrapper at :3510-3526 (Schwarz recomputed per call, shell pairs from
   init_2body_ints :54-67).  G = 0.25 (Gacc + Gacc^T); with factor f this is
   J[D] + f K[D].  D and G are row-major n x n. */
static void twobody_loops(BASIS_ARGS, int is_electron, const double *D, double factor, double *Gout,
                          int nthreads, int gem_n, const double *gem_c, const double *gem_g) {
  or_basis *b = basis_new(BASIS_PASS);
  int n = b->nbf;
  unsigned char *mask = (unsigned char *)malloc((size_t)nsh * nsh);
  pair_mask(b, mask);
  /* the geminal build screens nothing (Libint2Iface.cpp:2255-2330) */
  int screen = is_electron && gem_n == 0;
  double *Q = (double *)malloc(sizeof(double) * nsh * nsh);
  if (screen) schwarz(b, Q, nthreads);
  double *Dn = (double *)malloc(sizeof(double) * nsh * nsh);
  if (screen) shellblock_norm(b, D, Dn);
  const double eps = DBL_EPSILON;
  double *Gall = (double *)calloc((size_t)nthreads * n * n, sizeof(double));
  long long count = 0;
#pragma omp parallel num_threads(nthreads) reduction(+ : count)
  {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    double *g = Gall + (size_t)tid * n * n;
    or_work *w = work_new();
    w->gem_n = gem_n;
    w->gem_c = gem_c;
    w->gem_g = gem_g;
    long long s1234 = 0;
    for (int s1 = 0; s1 < nsh; ++s1) {
      int bf1f = b->first[s1], n1 = ncart(b->sh[s1].l);
      for (int s2 = 0; s2 <= s1; ++s2) {
        if (!mask[s1 * nsh + s2]) continue;
        int bf2f = b->first[s2], n2 = ncart(b->sh[s2].l);
        double Dn12 = screen ? Dn[s1 * nsh + s2] : 0.;
        for (int s3 = 0; s3 <= s1; ++s3) {
          int bf3f = b->first[s3], n3 = ncart(b->sh[s3].l);
          double Dn123 = screen ? dmax(Dn[s1 * nsh + s3], dmax(Dn[s2 * nsh + s3], Dn12)) : 0.;
          int s4max = (s1 == s3) ? s2 : s3;
          for (int s4 = 0; s4 <= s4max; ++s4) {
            if (!mask[s3 * nsh + s4]) continue;
            if ((s1234++) % nthreads != tid) continue;
            double Dn1234 = screen ? dmax(Dn[s1 * nsh + s4], dmax(Dn[s2 * nsh + s4], dmax(Dn[s3 * nsh + s4], Dn123))) : 0.;
            if (screen && Dn1234 * Q[s1 * nsh + s2] * Q[s3 * nsh + s4] < eps) continue;
            int bf4f = b->first[s4], n4 = ncart(b->sh[s4].l);
            ++count;
            double deg = (s1 == s2 ? 1.0 : 2.0) * (s3 == s4 ? 1.0 : 2.0) *
                         ((s1 == s3) ? (s2 == s4 ? 1.0 : 2.0) : 2.0);
            eri_shells(&b->sh[s1], &b->sh[s2], &b->sh[s3], &b->sh[s4], w->raw, w);
            int f1234 = 0;
            for (int f1 = 0; f1 < n1; ++f1) {
              int i = bf1f + f1;
              for (int f2 = 0; f2 < n2; ++f2) {
                int j = bf2f + f2;
                for (int f3 = 0; f3 < n3; ++f3) {
                  int k = bf3f + f3;
                  for (int f4 = 0; f4 < n4; ++f4, ++f1234) {
                    int l = bf4f + f4;
                    double v = w->raw[f1234] * deg * b->norma[i] * b->norma[j] * b->norma[k] * b->norma[l];
                    g[(size_t)i * n + j] += D[(size_t)k * n + l] * v;
                    g[(size_t)k * n + l] += D[(size_t)i * n + j] * v;
                    g[(size_t)i * n + k] += 0.5 * factor * D[(size_t)j * n + l] * v;
                    g[(size_t)j * n + l] += 0.5 * factor * D[(size_t)i * n + k] * v;
                    g[(size_t)i * n + l] += 0.5 * factor * D[(size_t)j * n + k] * v;
                    g[(size_t)j * n + k] += 0.5 * factor * D[(size_t)i * n + l] * v;
                  }
                }
              }
            }
          }
        }
      }
    }
    work_free(w);
  }
  g_last_quartets = count;
  for (int t = 1; t < nthreads; ++t)
    for (size_t x = 0; x < (size_t)n * n; ++x) Gall[x] += Gall[(size_t)t * n * n + x];
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) Gout[(size_t)i * n + j] = 0.25 * (Gall[(size_t)i * n + j] + Gall[(size_t)j * n + i]);
  free(Gall); free(Dn); free(Q); free(mask);
  basis_free(b);
}

void or_2body_direct(BASIS_ARGS, int is_electron, const double *D, double factor, double *Gout,
                     int nthreads) {
  twobody_loops(BASIS_PASS, is_electron, D, factor, Gout, nthreads, 0, NULL, NULL);
}

/* Direct intra-species geminal matrix, Libint2Iface.cpp:2193-2365 with the
   wrapper at :3687-3706: the loops, degeneracies, six updates and 0.25 (G+G^T)
   of the Coulomb build, the operator sum_k c_k exp(-g_k r12^2) (libint2's
   contracted Gaussian geminal, parameters {g_k, c_k}), no screening of any kind. */
void or_g12_direct(BASIS_ARGS, const double *D, double factor, int npot, const double *pot_coef,
                   const double *pot_expo, double *Gout, int nthreads) {
  twobody_loops(BASIS_PASS, 0, D, factor, Gout, nthreads, npot, pot_coef, pot_expo);
}

/* Direct inter-species coupling, Libint2Iface.cpp:1111-1294 and wrapper
   :3566-3589.  `this_` is the species whose matrix is built (lint), `other` the
   species whose density D (n_o x n_o) is contracted (olint).  When
   id_this > id_other the reference loops with the other species as the bra
   (permuted).  Only the lower triangle (row >= col) of the row-major result is
   written, the rest is zero; |raw| < 1e-10 integrals are skipped. */
static void coupling_loops(int nsh_a, const int *ls_a, const int *np_a, const double *or_a,
                           const double *al_a, const double *co_a, int id_a,
                           int nsh_b, const int *ls_b, const int *np_b, const double *or_b,
                           const double *al_b, const double *co_b, int id_b,
                           const double *D, double *Bout, int nthreads,
                           int gem_n, const double *gem_c, const double *gem_g) {
  or_basis *ba = basis_new(nsh_a, ls_a, np_a, or_a, al_a, co_a);
  or_basis *bo = basis_new(nsh_b, ls_b, np_b, or_b, al_b, co_b);
  int permuted = id_a > id_b;
  or_basis *self = permuted ? bo : ba, *oth = permuted ? ba : bo;
  int n = ba->nbf, nD = bo->nbf;
  double *Ball = (double *)calloc((size_t)nthreads * n * n, sizeof(double));
#pragma omp parallel num_threads(nthreads)
  {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    double *B = Ball + (size_t)tid * n * n;
    or_work *w = work_new();
    w->gem_n = gem_n;
    w->gem_c = gem_c;
    w->gem_g = gem_g;
    long long s1234 = 0;
    for (int s1 = 0; s1 < self->nshell; ++s1)
      for (int s2 = s1; s2 < self->nshell; ++s2)
        for (int o1 = 0; o1 < oth->nshell; ++o1)
          for (int o2 = o1; o2 < oth->nshell; ++o2) {
            if ((s1234++) % nthreads != tid) continue;
            eri_shells(&self->sh[s1], &self->sh[s2], &oth->sh[o1], &oth->sh[o2], w->raw, w);
            int n1 = ncart(self->sh[s1].l), n2 = ncart(self->sh[s2].l);
            int m1 = ncart(oth->sh[o1].l), m2 = ncart(oth->sh[o2].l);
            int idx = 0;
            for (int f1 = 0; f1 < n1; ++f1)
              for (int f2 = 0; f2 < n2; ++f2)
                for (int g1 = 0; g1 < m1; ++g1)
                  for (int g2 = 0; g2 < m2; ++g2, ++idx) {
                    int i = self->first[s1] + f1, j = self->first[s2] + f2;
                    int k = oth->first[o1] + g1, l = oth->first[o2] + g2;
                    if (!(i <= j && k <= l)) continue;
                    double raw = w->raw[idx];
                    if (fabs(raw) < 1e-10) continue;
                    double nrm = raw * self->norma[i] * self->norma[j] * oth->norma[k] * oth->norma[l];
                    if (permuted) {
                      double c = D[(size_t)i * nD + j] * nrm;
                      B[(size_t)l * n + k] += c;
                      if (i != j) B[(size_t)l * n + k] += c;
                    } else {
                      double c = D[(size_t)k * nD + l] * nrm;
                      B[(size_t)j * n + i] += c;
                      if (k != l) B[(size_t)j * n + i] += c;
                    }
                  }
          }
    work_free(w);
  }
  for (size_t x = 0; x < (size_t)n * n; ++x) {
    double s = 0;
    for (int t = 0; t < nthreads; ++t) s += Ball[(size_t)t * n * n + x];
    Bout[x] = s;
  }
  free(Ball);
  basis_free(ba); basis_free(bo);
}

void or_coupling_direct(int nsh_a, const int *ls_a, const int *np_a, const double *or_a,
                        const double *al_a, const double *co_a, int id_a,
                        int nsh_b, const int *ls_b, const int *np_b, const double *or_b,
                        const double *al_b, const double *co_b, int id_b,
                        const double *D, double *Bout, int nthreads) {
  coupling_loops(nsh_a, ls_a, np_a, or_a, al_a, co_a, id_a, nsh_b, ls_b, np_b, or_b, al_b, co_b, id_b, D, Bout,
                 nthreads, 0, NULL, NULL);
}

/* Direct inter-species geminal matrix, Libint2Iface.cpp:2367-2540 with the
   wrapper at :3708-3734: the loops, triangle rule, |raw| < 1e-10 cut and
   lower-triangle result of the Coulomb coupling, with the operator
   sum_k c_k exp(-g_k r12^2). */
void or_g12inter_direct(int nsh_a, const int *ls_a, const int *np_a, const double *or_a,
                        const double *al_a, const double *co_a, int id_a,
                        int nsh_b, const int *ls_b, const int *np_b, const double *or_b,
                        const double *al_b, const double *co_b, int id_b,
                        const double *D, int npot, const double *coef, const double *expo, double *Bout,
                        int nthreads) {
  coupling_loops(nsh_a, ls_a, np_a, or_a, al_a, co_a, id_a, nsh_b, ls_b, np_b, or_b, al_b, co_b, id_b, D, Bout,
                 nthreads, npot, coef, expo);
}

/* Enumeration of permutation-unique integrals inside one shell quartet, as
   IntraIntsIt (src/ints/Iterators.cpp:13-181): visits buffer positions
   (ii,jj,kk,ll) of the quartet and returns canonical labels (i>=j, k>=l,
   (ij)>=(kl)) as used by the first-quarter accumulation. */
typedef void (*it_visit)(void *ctx, int i, int j, int k, int l, int index);
static void intra_ints_iterate(int n1, int n2, int n3, int n4, int f1, int f2, int f3, int f4,
                               it_visit visit, void *ctx) {
  int case1 = (f1 == f2 && f3 == f4 && f1 == f3);
  int case2 = !case1 && (f1 == f3 && f2 == f4);
  for (int ii = 0; ii < n1; ++ii) {
    int jmax = case1 ? ii : case2 ? n2 - 1 : (f1 == f2 ? ii : n2 - 1);
    for (int jj = 0; jj <= jmax; ++jj) {
      int kmax = (case1 || case2) ? ii : n3 - 1;
      for (int kk = 0; kk <= kmax; ++kk) {
        int lmax;
        if (case1) lmax = (kk == ii) ? jj : kk;
        else if (case2) lmax = (kk == ii) ? jj : n4 - 1;
        else lmax = (f3 == f4) ? kk : n4 - 1;
        for (int ll = 0; ll <= lmax; ++ll) {
          int i = ii + f1, j = jj + f2, k = kk + f3, l = ll + f4, t;
          int index = ll + n4 * (kk + n3 * (jj + n2 * ii));
          if (case1) {
          } else if (case2) {
            if (i < j) { t = i; i = j; j = t; t = k; k = l; l = t; }
            if (i < k) { t = i; i = k; k = t; t = j; j = l; l = t; }
          } else {
            if (i < j) { t = i; i = j; j = t; }
            if (k < l) { t = k; k = l; l = t; }
            if (i < k || (i == k && j < l)) { t = i; i = k; k = t; t = j; j = l; l = t; }
          }
          visit(ctx, i, j, k, l, index);
        }
      }
    }
  }
}

typedef struct {
  const double *raw, *norma, *Cp;
  double *GG;
  int n;
} it_ctx;

static void it_accumulate(void *vctx, int i, int j, int k, int l, int index) {
  it_ctx *c = (it_ctx *)vctx;
  double raw = c->raw[index];
  if (!(fabs(raw) > 1.0e-10)) return;
  size_t n = c->n;
  double v = raw * c->norma[i] * c->norma[j] * c->norma[k] * c->norma[l];
  int kl0 = k < l ? k : l, kl1 = k < l ? l : k, ij0 = i < j ? i : j, ij1 = i < j ? j : i;
  c->GG[((size_t)j * n + kl0) * n + kl1] += v * c->Cp[i];
  if (i != j) c->GG[((size_t)i * n + kl0) * n + kl1] += v * c->Cp[j];
  if (i != k || j != l) {
    c->GG[((size_t)l * n + ij0) * n + ij1] += v * c->Cp[k];
    if (k != l) c->GG[((size_t)k * n + ij0) * n + ij1] += v * c->Cp[l];
  }
}

/* First-quarter transform for one orbital p, Libint2Iface.cpp:620-921 with the
   wrapper :3528-3549: A[nu][lam][sig] = sum_mu C(p,mu) (mu nu|lam sig) over the
   screened quartets of the direct build, |raw| > 1e-10, symmetric in lam/sig.
   C is row-major n x n (C[p*n + mu]); A has n^3 entries. */
void or_2body_directIT(BASIS_ARGS, int is_electron, const double *D, const double *C, int p,
                       double *A) {
  or_basis *b = basis_new(BASIS_PASS);
  int n = b->nbf;
  unsigned char *mask = (unsigned char *)malloc((size_t)nsh * nsh);
  pair_mask(b, mask);
  double *Q = (double *)malloc(sizeof(double) * nsh * nsh);
  schwarz(b, Q, 1);
  double *Dn = (double *)malloc(sizeof(double) * nsh * nsh);
  int screen = is_electron;
  if (screen) shellblock_norm(b, D, Dn);
  memset(A, 0, sizeof(double) * (size_t)n * n * n);
  or_work *w = work_new();
  it_ctx ctx = {w->raw, b->norma, C + (size_t)p * n, A, n};
  for (int s1 = 0; s1 < nsh; ++s1)
    for (int s2 = 0; s2 <= s1; ++s2) {
      if (!mask[s1 * nsh + s2]) continue;
      double Dn12 = screen ? Dn[s1 * nsh + s2] : 0.;
      for (int s3 = 0; s3 <= s1; ++s3) {
        double Dn123 = screen ? dmax(Dn[s1 * nsh + s3], dmax(Dn[s2 * nsh + s3], Dn12)) : 0.;
        int s4max = (s1 == s3) ? s2 : s3;
        for (int s4 = 0; s4 <= s4max; ++s4) {
          if (!mask[s3 * nsh + s4]) continue;
          double Dn1234 = screen ? dmax(Dn[s1 * nsh + s4], dmax(Dn[s2 * nsh + s4], dmax(Dn[s3 * nsh + s4], Dn123))) : 0.;
          if (screen && Dn1234 * Q[s1 * nsh + s2] * Q[s3 * nsh + s4] < DBL_EPSILON) continue;
          eri_shells(&b->sh[s1], &b->sh[s2], &b->sh[s3], &b->sh[s4], w->raw, w);
          intra_ints_iterate(ncart(b->sh[s1].l), ncart(b->sh[s2].l), ncart(b->sh[s3].l), ncart(b->sh[s4].l),
                             b->first[s1], b->first[s2], b->first[s3], b->first[s4], it_accumulate, &ctx);
        }
      }
    }
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j)
      for (int k = j; k < n; ++k) A[((size_t)i * n + k) * n + j] = A[((size_t)i * n + j) * n + k];
  work_free(w);
  free(Dn); free(Q); free(mask);
  basis_free(b);
}

/* Coupling first-quarter transform, Libint2Iface.cpp:1296-1622 and wrapper
   :3591-3620: A[nu][lam][sig] = sum_mu C(p,mu) (mu nu|lam sig), mu,nu of species
   a (lint, whose coefficients C are n_a x n_a row-major), lam,sig of species b;
   no Schwarz screening, |raw| < 1e-10 skipped; A has n_a*n_b*n_b entries. */
void or_coupling_directIT(int nsh_a, const int *ls_a, const int *np_a, const double *or_a,
                          const double *al_a, const double *co_a, int id_a,
                          int nsh_b, const int *ls_b, const int *np_b, const double *or_b,
                          const double *al_b, const double *co_b, int id_b,
                          const double *C, int p, double *A) {
  or_basis *ba = basis_new(nsh_a, ls_a, np_a, or_a, al_a, co_a);
  or_basis *bo = basis_new(nsh_b, ls_b, np_b, or_b, al_b, co_b);
  int permuted = id_a > id_b;
  or_basis *self = permuted ? bo : ba, *oth = permuted ? ba : bo;
  size_t n = ba->nbf, on = bo->nbf;
  const double *Cp = C + (size_t)p * n;
  memset(A, 0, sizeof(double) * n * on * on);
  or_work *w = work_new();
  for (int s1 = 0; s1 < self->nshell; ++s1)
    for (int s2 = s1; s2 < self->nshell; ++s2)
      for (int o1 = 0; o1 < oth->nshell; ++o1)
        for (int o2 = o1; o2 < oth->nshell; ++o2) {
          eri_shells(&self->sh[s1], &self->sh[s2], &oth->sh[o1], &oth->sh[o2], w->raw, w);
          int n1 = ncart(self->sh[s1].l), n2 = ncart(self->sh[s2].l);
          int m1 = ncart(oth->sh[o1].l), m2 = ncart(oth->sh[o2].l);
          int idx = 0;
          for (int f1 = 0; f1 < n1; ++f1)
            for (int f2 = 0; f2 < n2; ++f2)
              for (int g1 = 0; g1 < m1; ++g1)
                for (int g2 = 0; g2 < m2; ++g2, ++idx) {
                  int i = self->first[s1] + f1, j = self->first[s2] + f2;
                  int k = oth->first[o1] + g1, l = oth->first[o2] + g2;
                  if (!(i <= j && k <= l)) continue;
                  double raw = w->raw[idx];
                  if (fabs(raw) < 1e-10) continue;
                  double c = raw * self->norma[i] * self->norma[j] * oth->norma[k] * oth->norma[l];
                  if (permuted) {
                    /* bra = species b (i,j), ket = species a (k,l) */
                    A[((size_t)l * on + i) * on + j] += c * Cp[k];
                    if (k != l) A[((size_t)k * on + i) * on + j] += c * Cp[l];
                  } else {
                    A[((size_t)j * on + k) * on + l] += c * Cp[i];
                    if (i != j) A[((size_t)i * on + k) * on + l] += c * Cp[j];
                  }
                }
        }
  for (size_t i = 0; i < n; ++i)
    for (size_t j = 0; j < on; ++j)
      for (size_t k = j; k < on; ++k) A[(i * on + k) * on + j] = A[(i * on + j) * on + k];
  work_free(w);
  basis_free(ba); basis_free(bo);
}

/* ----------------------------------------------------- one-body blocks ---- */
/* Overlap S and kinetic T (norma applied), row-major n x n. */
void or_overlap_kinetic(BASIS_ARGS, double *S, double *T) {
  or_basis *b = basis_new(BASIS_PASS);
  int n = b->nbf;
  double s[15 * 15], t[15 * 15];
  for (int s1 = 0; s1 < b->nshell; ++s1)
    for (int s2 = 0; s2 < b->nshell; ++s2) {
      shell_overlap_kinetic(&b->sh[s1], &b->sh[s2], s, t);
      int n1 = ncart(b->sh[s1].l), n2 = ncart(b->sh[s2].l);
      for (int f1 = 0; f1 < n1; ++f1)
        for (int f2 = 0; f2 < n2; ++f2) {
          int i = b->first[s1] + f1, j = b->first[s2] + f2;
          double nn = b->norma[i] * b->norma[j];
          S[(size_t)i * n + j] = s[f1 * n2 + f2] * nn;
          T[(size_t)i * n + j] = t[f1 * n2 + f2] * nn;
        }
    }
  basis_free(b);
}

/* Point-charge potential V_ij = sum_C Z_C <i| 1/|r-R_C| |j> (positive for a
   positive charge; the caller scales by the particle charge). */
void or_potential(BASIS_ARGS, int ncharge, const double *Z, const double *R, double *V) {
  or_basis *b = basis_new(BASIS_PASS);
  int n = b->nbf;
  memset(V, 0, sizeof(double) * (size_t)n * n);
  /* [e|C|0]^(m) via OS, then HRR on the bra */
  double *W = (double *)malloc(sizeof(double) * NCUM_MAX * (2 * OR_MAXL + 1));
  double *X = (double *)malloc(sizeof(double) * NCUM_MAX);
  double *out = (double *)malloc(sizeof(double) * 225);
  double *tmp = (double *)malloc(sizeof(double) * 2 * NCUM_MAX * 15);
  for (int s1 = 0; s1 < b->nshell; ++s1)
    for (int s2 = 0; s2 < b->nshell; ++s2) {
      const or_shell *A = &b->sh[s1], *B = &b->sh[s2];
      int la = A->l, lb = B->l, L = la + lb, M = L + 1, NE = cart_off(L + 1), e0 = cart_off(la);
      double AB[3], AB2 = 0;
      for (int d = 0; d < 3; ++d) { AB[d] = A->O[d] - B->O[d]; AB2 += AB[d] * AB[d]; }
      memset(X, 0, sizeof(double) * NE);
      for (int pa = 0; pa < A->nprim; ++pa)
        for (int pb = 0; pb < B->nprim; ++pb) {
          double a = A->alpha[pa], bb = B->alpha[pb], p = a + bb, o2p = 0.5 / p;
          double P[3];
          for (int d = 0; d < 3; ++d) P[d] = (a * A->O[d] + bb * B->O[d]) / p;
          double wgt = A->cn[pa] * B->cn[pb] * 2.0 * M_PI / p * exp(-a * bb / p * AB2);
          for (int c = 0; c < ncharge; ++c) {
            double PC[3], PA[3], PC2 = 0, F[2 * OR_MAXL + 1];
            for (int d = 0; d < 3; ++d) {
              PC[d] = P[d] - R[3 * c + d]; PA[d] = P[d] - A->O[d]; PC2 += PC[d] * PC[d];
            }
            or_boys(L, p * PC2, F);
            for (int m = 0; m <= L; ++m) W[m] = F[m];
            for (int e = 1; e < NE; ++e) {
              int ex = g_cx[e], ey = g_cy[e], ez = g_cz[e], ke = ex + ey + ez;
              int dir = ex > 0 ? 0 : (ey > 0 ? 1 : 2);
              int ei = (dir == 0 ? ex : dir == 1 ? ey : ez) - 1;
              int em = cidx(ex - (dir == 0), ey - (dir == 1), ez - (dir == 2));
              int emm = ei > 0 ? cidx(ex - 2 * (dir == 0), ey - 2 * (dir == 1), ez - 2 * (dir == 2)) : 0;
              for (int m = 0; m <= L - ke; ++m) {
                double v = PA[dir] * W[em * M + m] - PC[dir] * W[em * M + m + 1];
                if (ei > 0) v += ei * o2p * (W[emm * M + m] - W[emm * M + m + 1]);
                W[e * M + m] = v;
              }
            }
            for (int e = e0; e < NE; ++e) X[e - e0] += Z[c] * wgt * W[e * M];
          }
        }
      hrr(la, lb, AB, X, 1, out, tmp);
      int n1 = ncart(la), n2 = ncart(lb);
      for (int f1 = 0; f1 < n1; ++f1)
        for (int f2 = 0; f2 < n2; ++f2) {
          int i = b->first[s1] + f1, j = b->first[s2] + f2;
          V[(size_t)i * n + j] = out[f1 * n2 + f2] * b->norma[i] * b->norma[j];
        }
    }
  free(W); free(X); free(out); free(tmp);
  basis_free(b);
}

/* Full normalised AO ERI tensor (ij|kl), n^4 row-major, no screening (small
   systems only: used for MP2 energies in the oracle). */
void or_eri_full(BASIS_ARGS, double *out, int nthreads) {
  or_basis *b = basis_new(BASIS_PASS);
  size_t n = b->nbf;

#pragma omp parallel num_threads(nthreads)
  {
    or_work *w = work_new();
#pragma omp for schedule(dynamic) collapse(2)
    for (int s1 = 0; s1 < nsh; ++s1)
      for (int s2 = 0; s2 < nsh; ++s2)
        for (int s3 = 0; s3 < nsh; ++s3)
          for (int s4 = 0; s4 < nsh; ++s4) {
            eri_shells(&b->sh[s1], &b->sh[s2], &b->sh[s3], &b->sh[s4], w->raw, w);
            int n1 = ncart(b->sh[s1].l), n2 = ncart(b->sh[s2].l), n3 = ncart(b->sh[s3].l), n4 = ncart(b->sh[s4].l);
            int idx = 0;
            for (int f1 = 0; f1 < n1; ++f1)
              for (int f2 = 0; f2 < n2; ++f2)
                for (int f3 = 0; f3 < n3; ++f3)
                  for (int f4 = 0; f4 < n4; ++f4, ++idx) {
                    size_t i = b->first[s1] + f1, j = b->first[s2] + f2, k = b->first[s3] + f3, l = b->first[s4] + f4;
                    out[((i * n + j) * n + k) * n + l] =
                        w->raw[idx] * b->norma[i] * b->norma[j] * b->norma[k] * b->norma[l];
                  }
          }
    work_free(w);
  }
  basis_free(b);
}
