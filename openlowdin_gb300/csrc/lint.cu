// Host side of liblowdin_gb300.so, part 1: error reporting, the Boys tables,
// the host one-electron blocks, the coupling and first-quarter builds, the
// LibintInterface_* C ABI with the device-resident entry points, and the
// allocation-free two-particle build.  The per-species handle itself is in
// lint_host.cuh, batched builds in batch.cu, MP2 in mp2.cu.
#include "lint_host.cuh"

namespace lgb {

// ------------------------------------------------------------------ errors --
std::mutex g_err_mu;
std::string g_err;

void set_error(const char *fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  {
    std::lock_guard<std::mutex> lk(g_err_mu);
    g_err = buf;
  }
  fprintf(stderr, "lowdin_gb300: %s\n", buf);
  const char *strict = getenv("LOWDIN_GB300_STRICT");
  if (strict && strict[0] == '1') abort();
}

// ------------------------------------------------------------- Boys table --
// F_n(T_i), T_i = i h, from the series F_n(T) = e^{-T} sum_k (2T)^k /
// ((2n+1)(2n+3)...(2n+2k+1)) in long double.
struct BoysHost {
  std::vector<double> f64;
  std::vector<float> f32;
  BoysHost() : f64((size_t)kBoysF64Size), f32((size_t)kBoysPoints * kBoysStride) {
    for (int i = 0; i < kBoysPoints; ++i) {
      const long double T = (long double)i * (long double)kBoysH;
      f64[(size_t)i * kBoysStride + kBoysOrders] = (double)expl(-T);
      f32[(size_t)i * kBoysStride + kBoysOrders] = (float)expl(-T);
      for (int n = 0; n < kBoysOrders; ++n) {
        long double term = 1.0L / (2 * n + 1), sum = term;
        for (int k = 1; k < 2000; ++k) {
          term *= 2.0L * T / (2 * n + 2 * k + 1);
          sum += term;
          if (term < 1e-24L * sum) break;
        }
        const double v = (double)(expl(-T) * sum);
        f64[(size_t)i * kBoysStride + n] = v;
        f32[(size_t)i * kBoysStride + n] = (float)v;
      }
    }
    // per-order Taylor coefficients F_{L+k}(T_i) / k! and e^{-T_i}
    for (int L = 0; L <= kMaxLQuartet; ++L)
      for (int i = 0; i < kBoysPoints; ++i) {
        double *row = &f64[kBoysScaledOff + ((size_t)L * kBoysPoints + i) * kBoysSRow];
        double fact = 1.0;
        for (int k = 0; k < kBoysTaylor; ++k) {
          if (k > 0) fact *= k;
          row[k] = f64[(size_t)i * kBoysStride + L + k] / fact;
        }
        row[kBoysTaylor] = f64[(size_t)i * kBoysStride + kBoysOrders];
      }
  }
  // F_m(T), m = 0..mmax (host; Taylor + downward recursion like the device)
  void eval(int mmax, double T, double *F) const {
    if (T < kBoysTMax) {
      const int i = (int)std::lround(T / kBoysH);
      const double mdT = i * kBoysH - T;
      const double *t = &f64[(size_t)i * kBoysStride + mmax];
      double s = t[kBoysTaylor - 1];
      for (int k = kBoysTaylor - 1; k >= 1; --k) s = std::fma(mdT / k, s, t[k - 1]);
      F[mmax] = s;
      const double e = std::exp(-T);
      for (int m = mmax - 1; m >= 0; --m) F[m] = (2.0 * T * F[m + 1] + e) / (2 * m + 1);
    } else {
      const double e = std::exp(-T);
      F[0] = 0.88622692545275801365 / std::sqrt(T);
      for (int m = 0; m < mmax; ++m) F[m + 1] = ((2 * m + 1) * F[m] - e) / (2.0 * T);
    }
  }
};
const BoysHost &boys_host() {
  static BoysHost b;
  return b;
}

// device copies of the Boys tables, one per device
struct DeviceBoys {
  int device = -1;
  double *f64 = nullptr;
  float *f32 = nullptr;
};
std::mutex g_boys_mu;
std::vector<DeviceBoys> g_boys;

bool device_boys(BoysTables &out) {
  int dev = 0;
  CK(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_boys_mu);
  for (auto &b : g_boys)
    if (b.device == dev) {
      out.f64 = b.f64;
      out.f32 = b.f32;
      return true;
    }
  const BoysHost &h = boys_host();
  DeviceBoys b;
  b.device = dev;
  CK(cudaMalloc(&b.f64, h.f64.size() * sizeof(double)));
  CK(cudaMalloc(&b.f32, h.f32.size() * sizeof(float)));
  CK(cudaMemcpy(b.f64, h.f64.data(), h.f64.size() * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(b.f32, h.f32.data(), h.f32.size() * sizeof(float), cudaMemcpyHostToDevice));
  g_boys.push_back(b);
  out.f64 = b.f64;
  out.f32 = b.f32;
  return true;
}

// ------------------------------------------------------------ host shells --

double prim_norm(double a, int l) {
  double df = 1.0;
  for (int k = 2 * l - 1; k > 1; k -= 2) df *= k;
  return std::sqrt(std::pow(2.0, l) * std::pow(2.0 * a, l + 1.5) / (std::pow(M_PI, 1.5) * df));
}

// 1-D Obara-Saika overlap table s[i][j], i <= li, j <= lj
void ovl1d(int li, int lj, double PA, double PB, double o2p, double s[8][8]) {
  s[0][0] = 1.0;
  for (int i = 0; i <= li; ++i)
    for (int j = 0; j <= lj; ++j) {
      if (!i && !j) continue;
      double v;
      if (i > 0) {
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

// raw overlap (and optionally kinetic) block, row-major [ncart(la)][ncart(lb)]
void overlap_block(const HostShell &A, const HostShell &B, double *S, double *T) {
  const int n1 = ncart(A.l), n2 = ncart(B.l);
  std::fill(S, S + n1 * n2, 0.0);
  if (T) std::fill(T, T + n1 * n2, 0.0);
  double AB2 = 0;
  for (int d = 0; d < 3; ++d) AB2 += (A.O[d] - B.O[d]) * (A.O[d] - B.O[d]);
  for (int pa = 0; pa < A.nprim; ++pa)
    for (int pb = 0; pb < B.nprim; ++pb) {
      const double a = A.alpha[pa], b = B.alpha[pb], p = a + b, o2p = 0.5 / p;
      const double pref = std::pow(M_PI / p, 1.5) * std::exp(-a * b / p * AB2) * A.cn[pa] * B.cn[pb];
      double s[3][8][8];
      for (int d = 0; d < 3; ++d) {
        const double P = (a * A.O[d] + b * B.O[d]) / p;
        ovl1d(A.l, B.l + 2, P - A.O[d], P - B.O[d], o2p, s[d]);
      }
      for (int f1 = 0; f1 < n1; ++f1) {
        const int c1 = coff(A.l) + f1;
        const int ax[3] = {cx(c1), cy(c1), cz(c1)};
        for (int f2 = 0; f2 < n2; ++f2) {
          const int c2 = coff(B.l) + f2;
          const int bx[3] = {cx(c2), cy(c2), cz(c2)};
          const double sx = s[0][ax[0]][bx[0]], sy = s[1][ax[1]][bx[1]], sz = s[2][ax[2]][bx[2]];
          S[f1 * n2 + f2] += pref * sx * sy * sz;
          if (T) {
            double t[3];
            for (int d = 0; d < 3; ++d) {
              const int j = bx[d];
              double v = -2.0 * b * (2 * j + 1) * s[d][ax[d]][j] + 4.0 * b * b * s[d][ax[d]][j + 2];
              if (j >= 2) v += j * (j - 1) * s[d][ax[d]][j - 2];
              t[d] = -0.5 * v;
            }
            T[f1 * n2 + f2] += pref * (t[0] * sy * sz + sx * t[1] * sz + sx * sy * t[2]);
          }
        }
      }
    }
}

// raw external-potential block sum_k c_k <a| exp(-g_k |r - C_k|^2) |b>: the
// three Gaussians multiply to exp(-p |r - P|^2) with p = a + b + g and
// P = (a A + b B + g C) / p, times exp(-(a b AB^2 + a g AC^2 + b g BC^2) / p),
// so each component is an ordinary overlap recursion about that P
void gaussian_potential_block(const HostShell &A, const HostShell &B, int ncomp, const double *coef,
                              const double *expo, const double *C, double *V) {
  const int n1 = ncart(A.l), n2 = ncart(B.l);
  std::fill(V, V + n1 * n2, 0.0);
  for (int pa = 0; pa < A.nprim; ++pa)
    for (int pb = 0; pb < B.nprim; ++pb)
      for (int k = 0; k < ncomp; ++k) {
        const double a = A.alpha[pa], b = B.alpha[pb], g = expo[k], p = a + b + g, o2p = 0.5 / p;
        double e = 0, s[3][8][8];
        for (int d = 0; d < 3; ++d) {
          const double ab = A.O[d] - B.O[d], ac = A.O[d] - C[3 * k + d], bc = B.O[d] - C[3 * k + d];
          e += a * b * ab * ab + a * g * ac * ac + b * g * bc * bc;
          const double P = (a * A.O[d] + b * B.O[d] + g * C[3 * k + d]) / p;
          ovl1d(A.l, B.l, P - A.O[d], P - B.O[d], o2p, s[d]);
        }
        const double pref = coef[k] * std::pow(M_PI / p, 1.5) * std::exp(-e / p) * A.cn[pa] * B.cn[pb];
        for (int f1 = 0; f1 < n1; ++f1) {
          const int c1 = coff(A.l) + f1;
          for (int f2 = 0; f2 < n2; ++f2) {
            const int c2 = coff(B.l) + f2;
            V[f1 * n2 + f2] += pref * s[0][cx(c1)][cx(c2)] * s[1][cy(c1)][cy(c2)] * s[2][cz(c1)][cz(c2)];
          }
        }
      }
}

// raw point-charge potential block sum_C Z_C <a|1/|r-C||b> via Obara-Saika on
// the bra and horizontal transfer to b
void potential_block(const HostShell &A, const HostShell &B, int nc, const double *Z, const double *R, double *V) {
  const int la = A.l, lb = B.l, L = la + lb, NE = coff(L + 1), E0 = coff(la), M = L + 1;
  std::vector<double> W((size_t)NE * M), X(NE - E0, 0.0);
  double AB[3], AB2 = 0;
  for (int d = 0; d < 3; ++d) {
    AB[d] = A.O[d] - B.O[d];
    AB2 += AB[d] * AB[d];
  }
  const BoysHost &bh = boys_host();
  for (int pa = 0; pa < A.nprim; ++pa)
    for (int pb = 0; pb < B.nprim; ++pb) {
      const double a = A.alpha[pa], b = B.alpha[pb], p = a + b, o2p = 0.5 / p;
      double P[3], PA[3];
      for (int d = 0; d < 3; ++d) {
        P[d] = (a * A.O[d] + b * B.O[d]) / p;
        PA[d] = P[d] - A.O[d];
      }
      const double w = A.cn[pa] * B.cn[pb] * 2.0 * M_PI / p * std::exp(-a * b / p * AB2);
      for (int c = 0; c < nc; ++c) {
        double PC[3], PC2 = 0, F[kMaxLQuartet + 1];
        for (int d = 0; d < 3; ++d) {
          PC[d] = P[d] - R[3 * c + d];
          PC2 += PC[d] * PC[d];
        }
        bh.eval(L, p * PC2, F);
        for (int m = 0; m <= L; ++m) W[m] = F[m];
        for (int e = 1; e < NE; ++e) {
          const int d = cdir(e), em = cminus(e, d), ei = ccomp(e, d) - 1;
          for (int m = 0; m <= L - clevel(e); ++m) {
            double v = PA[d] * W[em * M + m] - PC[d] * W[em * M + m + 1];
            if (ei > 0) {
              const int emm = cminus(em, d);
              v += ei * o2p * (W[emm * M + m] - W[emm * M + m + 1]);
            }
            W[e * M + m] = v;
          }
        }
        for (int e = E0; e < NE; ++e) X[e - E0] += Z[c] * w * W[e * M];
      }
    }
  // horizontal transfer (a, b+1_i| = (a+1_i, b| + AB_i (a, b|
  const int nA = NE - E0;
  std::vector<std::vector<double>> lev(lb + 1);
  lev[0] = X;  // [a rows][1]
  for (int j = 1; j <= lb; ++j) {
    const int na = coff(la + lb - j + 1) - E0, nb = ncart(j), nbm = ncart(j - 1);
    lev[j].assign((size_t)na * nb, 0.0);
    for (int bi = 0; bi < nb; ++bi) {
      const int bc = coff(j) + bi, d = cdir(bc), bm = cminus(bc, d) - coff(j - 1);
      for (int ar = 0; ar < na; ++ar) {
        const int apr = cplus(E0 + ar, d) - E0;
        lev[j][(size_t)ar * nb + bi] = lev[j - 1][(size_t)apr * nbm + bm] + AB[d] * lev[j - 1][(size_t)ar * nbm + bm];
      }
    }
  }
  (void)nA;
  const int n1 = ncart(la), n2 = ncart(lb);
  for (int f1 = 0; f1 < n1; ++f1)
    for (int f2 = 0; f2 < n2; ++f2) V[f1 * n2 + f2] = lev[lb][(size_t)f1 * n2 + f2];
}

// coupling tasks of species pair (A bra, B ket) into ts
bool add_cp_tasks(TaskSet<CPTask> &ts, LibintInterface *A, LibintInterface *B, const SpeciesBufs &ba,
                  const SpeciesBufs &bb, bool want_a, bool want_b, double scale,
                  unsigned long long *counters) {
  // JA (from D_B) accumulates into ba.G / ba.G32, JB (from D_A) into bb.G / bb.G32
  double *JA = want_a ? ba.G : nullptr, *JB = want_b ? bb.G : nullptr;
  if (!A->ensure_all() || !B->ensure_all()) return false;
  for (int cb = 0; cb < kNumPairClasses; ++cb)
    for (int ck = 0; ck < kNumPairClasses; ++ck) {
      if (!A->all.count(cb) || !B->all.count(ck)) continue;
      if (!class_supported(cb, ck)) {
        set_error("coupling class (%d,%d|%d,%d) is not built into this library", pc_la(cb), pc_lb(cb), pc_la(ck),
                  pc_lb(ck));
        return false;
      }
      CPTask t{};
      t.pa = A->all.d;
      t.pra = A->all.dp;
      t.pb = B->all.d;
      t.prb = B->all.dp;
      t.pa32 = A->all.d32;
      t.pra32 = A->all.dp32;
      t.pb32 = B->all.d32;
      t.prb32 = B->all.dp32;
      t.DsA = JB ? ba.Ds : nullptr;
      t.DsA32 = JB ? ba.Ds32 : nullptr;
      t.DsB = JA ? bb.Ds : nullptr;
      t.DsB32 = JA ? bb.Ds32 : nullptr;
      t.JA = JA;
      t.JA32 = JA ? ba.G32 : nullptr;
      t.JB = JB;
      t.JB32 = JB ? bb.G32 : nullptr;
      t.DnA32 = ba.Dn32;
      t.DnB32 = bb.Dn32;
      t.count = counters ? counters + cb * kNumPairClasses + ck : nullptr;
      t.nshA = A->nshell();
      t.nshB = B->nshell();
      t.scale = scale;
      t.scale32 = (float)scale;
      t.bra0 = A->all.start[cb];
      t.nbra = A->all.count(cb);
      t.ket0 = B->all.start[ck];
      t.nket = B->all.count(ck);
      t.nA = A->nbasis;
      t.nB = B->nbasis;
      ts.add(cb, ck, t);
    }
  return true;
}

// mode 0: FP64, 1: FP32 throughout, 2: split at `split` (FP64 above, FP32 below)
bool launch_cp_groups(const TaskSet<CPTask> &ts, int mode, double split, BoysTables boys, cudaStream_t s,
                      double skip) {
  for (int c = 0; c < kNQC; ++c) {
    if (!ts.cnt[c]) continue;
    TaskLaunch tl{};
    tl.ntasks = ts.cnt[c];
    tl.nblocks = ts.nblk[c];
    tl.eps = DBL_EPSILON;
    tl.cut = 1e-10;
    tl.skip = (float)skip;
    tl.boys = boys;
    const int cb = c / kNumPairClasses, ck = c % kNumPairClasses;
    if (mode == 2) {
      tl.split = split;
      set_fp32_copies(tl);
      tl.lower = 0;
      CK(launch_cp_tasks(cb, ck, false, ts.d + ts.off[c], tl, s));
      tl.lower = 1;
      CK(launch_cp_tasks(cb, ck, true, ts.d + ts.off[c], tl, s));
    } else {
      set_fp32_copies(tl);
      CK(launch_cp_tasks(cb, ck, mode == 1, ts.d + ts.off[c], tl, s));
    }
  }
  return true;
}


bool coupling(LibintInterface *A, LibintInterface *B, const double *dDa, const double *dDb, double *dJa,
              double *dJb, bool fp32, cudaStream_t s) {
  if (!A->ensure_all() || !B->ensure_all()) return false;
  const int nA = A->nbasis, nB = B->nbasis;
  // scaled densities in each handle's dDsC(32), accumulators in dJacc(32)
  auto bufs = [](LibintInterface *X, int n) {
    return X->dDsC.ensure((size_t)n * n) && X->dDsC32.ensure((size_t)n * n) && X->dJacc.ensure((size_t)n * n) &&
           X->dJacc32.ensure((size_t)n * n);
  };
  if (!bufs(A, nA) || !bufs(B, nB)) return false;
  if (dJa) {
    CK(launch_scale_density(dDb, B->d_norma, nB, B->dDsC.p, B->dDsC32.p, s));
    CK(cudaMemsetAsync(A->dJacc.p, 0, sizeof(double) * nA * nA, s));
    CK(cudaMemsetAsync(A->dJacc32.p, 0, sizeof(float) * nA * nA, s));
  }
  if (dJb) {
    CK(launch_scale_density(dDa, A->d_norma, nA, A->dDsC.p, A->dDsC32.p, s));
    CK(cudaMemsetAsync(B->dJacc.p, 0, sizeof(double) * nB * nB, s));
    CK(cudaMemsetAsync(B->dJacc32.p, 0, sizeof(float) * nB * nB, s));
  }
  A->cp.clear();
  SpeciesBufs ba{A->dDsC.p, A->dDsC32.p, nullptr, nullptr, A->dJacc.p, A->dJacc32.p};
  SpeciesBufs bb{B->dDsC.p, B->dDsC32.p, nullptr, nullptr, B->dJacc.p, B->dJacc32.p};
  if (!add_cp_tasks(A->cp, A, B, ba, bb, dJa != nullptr, dJb != nullptr, 1.0)) return false;
  if (!A->cp.upload(s)) return false;
  if (!launch_cp_groups(A->cp, fp32 ? 1 : 0, 0.0, A->boys, s)) return false;
  if (dJa) CK(launch_coupling_extract(A->dJacc.p, A->dJacc32.p, A->d_norma, nA, 1.0, 0, dJa, s));
  if (dJb) CK(launch_coupling_extract(B->dJacc.p, B->dJacc32.p, B->d_norma, nB, 1.0, 0, dJb, s));
  return true;
}

bool first_quarter(LibintInterface *A, LibintInterface *B, const double *hD, const double *hC, int p,
                   double *hOut) {
  // B == nullptr: intra-species (screened like the direct build); else coupling
  const bool intra = B == nullptr;
  if (intra ? !A->ensure_sig() : (!A->ensure_all() || !B->ensure_all())) return false;
  LibintInterface *K = intra ? A : B;
  const int nA = A->nbasis, nB = K->nbasis, nsh = A->nshell();
  cudaStream_t s = A->stream;
  if (p < 0 || p >= nA) {
    set_error("orbital index p=%d out of range [0,%d)", p, nA);
    return false;
  }
  std::vector<double> Cs(nA);
  for (int mu = 0; mu < nA; ++mu) Cs[mu] = hC[(size_t)p * nA + mu] * A->norma[mu];
  const size_t cube = (size_t)nA * nB * nB;
  if (!A->dA.ensure(cube) || !A->dC.ensure(nA)) return false;
  CK(cudaMemcpyAsync(A->dC.p, Cs.data(), nA * sizeof(double), cudaMemcpyHostToDevice, s));
  CK(cudaMemsetAsync(A->dA.p, 0, cube * sizeof(double), s));
  ITParams q{};
  q.intra = intra;
  q.Cs = A->dC.p;
  q.nA = nA;
  q.nB = nB;
  q.A = A->dA.p;
  q.boys = A->boys;
  q.cut = 1e-10;
  q.eps = DBL_EPSILON;
  q.nsh = nsh;
  if (intra) {
    if (!A->dD.ensure((size_t)nA * nA) || !A->dDs.ensure((size_t)nA * nA) || !A->dDn.ensure((size_t)nsh * nsh))
      return false;
    CK(cudaMemcpyAsync(A->dD.p, hD, sizeof(double) * nA * nA, cudaMemcpyHostToDevice, s));
    CK(launch_prepare_density(A->dD.p, A->d_norma, A->d_shell_of, nA, nsh, A->dDs.p, nullptr, A->dDn.p, nullptr,
                              s));
    q.Dn = A->dDn.p;
    q.screen = A->is_electron ? 1 : 0;
    q.pa = q.pb = A->sig.d;
    q.pra = q.prb = A->sig.dp;
    for (int cb = 0; cb < kNumPairClasses; ++cb)
      for (int ck = 0; ck <= cb; ++ck) {
        if (!A->sig.count(cb) || !A->sig.count(ck)) continue;
        if (!class_supported(cb, ck)) {
          set_error("quartet class not built into this library");
          return false;
        }
        q.bra0 = A->sig.start[cb];
        q.nbra = A->sig.count(cb);
        q.ket0 = A->sig.start[ck];
        q.nket = A->sig.count(ck);
        q.triangle = cb == ck;
        CK(launch_it(cb, ck, q, s));
      }
  } else {
    q.screen = 0;
    q.pa = A->all.d;
    q.pra = A->all.dp;
    q.pb = B->all.d;
    q.prb = B->all.dp;
    for (int cb = 0; cb < kNumPairClasses; ++cb)
      for (int ck = 0; ck < kNumPairClasses; ++ck) {
        if (!A->all.count(cb) || !B->all.count(ck)) continue;
        if (!class_supported(cb, ck)) {
          set_error("quartet class not built into this library");
          return false;
        }
        q.bra0 = A->all.start[cb];
        q.nbra = A->all.count(cb);
        q.ket0 = B->all.start[ck];
        q.nket = B->all.count(ck);
        q.triangle = 0;
        CK(launch_it(cb, ck, q, s));
      }
  }
  CK(launch_scale_cube(A->dA.p, A->d_norma, K->d_norma, nA, nB, s));
  CK(cudaMemcpyAsync(hOut, A->dA.p, cube * sizeof(double), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  return true;
}

// geminal parameters {count, exponents, coefficients} into A->dGem (stream of A)
bool upload_geminal(LibintInterface *A, const double *coefficients, const double *exponents, int pot_size,
                    const char *fn) {
  if (pot_size <= 0 || !coefficients || !exponents) {
    set_error("%s: the geminal needs pot_size > 0 coefficients and exponents (got %d)", fn, pot_size);
    return false;
  }
  std::vector<double> h(1 + 2 * (size_t)pot_size);
  h[0] = pot_size;
  for (int k = 0; k < pot_size; ++k) {
    if (!(exponents[k] >= 0.0) || !std::isfinite(exponents[k]) || !std::isfinite(coefficients[k])) {
      set_error("%s: geminal term %d has exponent %g, coefficient %g (exponents must be finite and >= 0)", fn, k,
                exponents[k], coefficients[k]);
      return false;
    }
    h[1 + k] = exponents[k];
    h[1 + pot_size + k] = coefficients[k];
  }
  if (!A->dGem.ensure(h.size())) return false;
  // synchronous: the host vector is freed on return
  CK(cudaMemcpyAsync(A->dGem.p, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice, A->stream));
  CK(cudaStreamSynchronize(A->stream));
  return true;
}

// Geminal matrix on the device, ordered on s.  B == nullptr: intra-species
// G = 0.25 (Gacc + Gacc^T) of A's significant pairs with exchange factor
// `factor`, from A's density dD (n x n), into dOut.  Else: J of A's species from
// B's density dD (nB x nB) over every pair of both species, lower triangle of
// dOut (row >= col), zero above.  The geminal is A->dGem.
bool g12_build(LibintInterface *A, LibintInterface *B, const double *dD, double factor, double *dOut,
               cudaStream_t s) {
  const int n = A->nbasis;
  G12Params P{};
  P.gem = A->dGem.p;
  P.n = n;
  if (!B) {
    CK(launch_scale_density(dD, A->d_norma, n, A->dDs.p, A->dDs32.p, s));
    CK(cudaMemsetAsync(A->dGacc.p, 0, sizeof(double) * n * n, s));
    P.pa = P.pb = A->sig.d;
    P.pra = P.prb = A->sig.dp;
    P.intra = 1;
    P.Ds = A->dDs.p;
    P.Gacc = A->dGacc.p;
    P.hf = 0.5 * factor;
    for (int cb = 0; cb < kNumPairClasses; ++cb)
      for (int ck = 0; ck <= cb; ++ck) {
        if (!A->sig.count(cb) || !A->sig.count(ck)) continue;
        P.bra0 = A->sig.start[cb];
        P.nbra = A->sig.count(cb);
        P.ket0 = A->sig.start[ck];
        P.nket = A->sig.count(ck);
        P.triangle = cb == ck;
        CK(launch_g12(cb, ck, P, s));
      }
    CK(launch_symmetrize(A->dGacc.p, nullptr, A->d_norma, n, 0.25, dOut, s));
    return true;
  }
  const int nB = B->nbasis;
  CK(launch_scale_density(dD, B->d_norma, nB, B->dDsC.p, B->dDsC32.p, s));
  CK(cudaMemsetAsync(A->dJacc.p, 0, sizeof(double) * n * n, s));
  P.pa = A->all.d;
  P.pra = A->all.dp;
  P.pb = B->all.d;
  P.prb = B->all.dp;
  P.intra = 0;
  P.Ds = B->dDsC.p;
  P.Gacc = A->dJacc.p;
  P.nB = nB;
  P.cut = 1e-10;
  for (int cb = 0; cb < kNumPairClasses; ++cb)
    for (int ck = 0; ck < kNumPairClasses; ++ck) {
      if (!A->all.count(cb) || !B->all.count(ck)) continue;
      P.bra0 = A->all.start[cb];
      P.nbra = A->all.count(cb);
      P.ket0 = B->all.start[ck];
      P.nket = B->all.count(ck);
      CK(launch_g12(cb, ck, P, s));
    }
  CK(launch_coupling_extract(A->dJacc.p, nullptr, A->d_norma, n, 1.0, 1, dOut, s));
  return true;
}

bool check_handle(LibintInterface *l, const char *fn) {
  if (!l) {
    set_error("%s: null handle", fn);
    return false;
  }
  return true;
}

void unsupported(const char *fn) { set_error("%s is not provided by this library (direct Coulomb path only)", fn); }

}  // namespace lgb

// ====================================================================== C ABI
extern "C" {

LibintInterface *LibintInterface_new(const int stack_size, const int id, const bool el, const bool parallel) {
  (void)parallel;
  LibintInterface *l = new LibintInterface();
  l->stack_size = stack_size;
  l->id = id;
  l->is_electron = el;
  return l;
}

void LibintInterface_del(LibintInterface *lint) { delete lint; }

void LibintInterface_add_particle(LibintInterface *lint, const int z, const double *center) {
  if (!check_handle(lint, __func__)) return;
  lint->atoms.push_back({z, {center[0], center[1], center[2]}});
}

void LibintInterface_add_shell(LibintInterface *lint, double *alpha, double *coeff, double *origin, int l,
                               int nprim) {
  if (!check_handle(lint, __func__)) return;
  if (l < 0 || nprim <= 0) {
    set_error("add_shell: invalid l=%d nprim=%d", l, nprim);
    return;
  }
  HostShell s;
  s.l = l;
  s.nprim = nprim;
  for (int d = 0; d < 3; ++d) s.O[d] = origin[d];
  for (int k = 0; k < nprim; ++k) {
    s.alpha.push_back(alpha[k]);
    s.cn.push_back(coeff[k] * prim_norm(alpha[k], l));
  }
  lint->first.push_back(lint->nbasis);
  lint->nbasis += ncart(l);
  // renormalise every Cartesian component to unit self-overlap
  const int n = ncart(l);
  std::vector<double> S((size_t)n * n);
  overlap_block(s, s, S.data(), nullptr);
  for (int i = 0; i < n; ++i) lint->norma.push_back(1.0 / std::sqrt(S[(size_t)i * n + i]));
  lint->shells.push_back(std::move(s));
  lint->dirty = true;
}

int LibintInterface_get_nbasis(LibintInterface *lint) { return lint ? lint->nbasis : 0; }

void LibintInterface_compute_1body_ints(LibintInterface *lint, int integral_kind, double *result) {
  if (!check_handle(lint, __func__)) return;
  const int n = lint->nbasis, nsh = lint->nshell();
  std::vector<double> Z, R;
  for (auto &a : lint->atoms) {
    Z.push_back((double)a.first);
    R.insert(R.end(), a.second.begin(), a.second.end());
  }
  double S[225], T[225];
  for (int s1 = 0; s1 < nsh; ++s1)
    for (int s2 = 0; s2 < nsh; ++s2) {
      const HostShell &A = lint->shells[s1], &B = lint->shells[s2];
      const int n1 = ncart(A.l), n2 = ncart(B.l);
      if (integral_kind == 3) potential_block(A, B, (int)Z.size(), Z.data(), R.data(), S);
      else overlap_block(A, B, S, integral_kind == 2 ? T : nullptr);
      const double *src = integral_kind == 2 ? T : S;
      for (int f1 = 0; f1 < n1; ++f1)
        for (int f2 = 0; f2 < n2; ++f2) {
          const int i = lint->first[s1] + f1, j = lint->first[s2] + f2;
          result[(size_t)i * n + j] = src[f1 * n2 + f2] * lint->norma[i] * lint->norma[j];
        }
    }
}

void LibintInterface_init_2body_ints(LibintInterface *lint) {
  if (!check_handle(lint, __func__)) return;
  lint->ensure_sig();
}

void LibintInterface_compute_2body_direct(LibintInterface *lint, double *dens, double *result, double &factor) {
  if (!check_handle(lint, __func__)) return;
  if (!lint->ensure_sig()) return;
  const int n = lint->nbasis;
  cudaStream_t s = lint->stream;
  if (!lint->dD.ensure((size_t)n * n) || !lint->dG.ensure((size_t)n * n)) return;
  if (cudaMemcpyAsync(lint->dD.p, dens, sizeof(double) * n * n, cudaMemcpyHostToDevice, s) != cudaSuccess) {
    set_error("compute_2body_direct: density upload failed");
    return;
  }
  if (!lint->twobody(lint->dD.p, lint->dG.p, factor, lint->abi_precision, lint->abi_split, s)) return;
  if (cudaMemcpyAsync(result, lint->dG.p, sizeof(double) * n * n, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    set_error("compute_2body_direct: result download failed");
}

void LibintInterface_compute_2body_directIT(LibintInterface *lint, double *dens, double *coeff, double *result,
                                            int &p) {
  if (!check_handle(lint, __func__)) return;
  first_quarter(lint, nullptr, dens, coeff, p, result);
}

void LibintInterface_compute_2body_disk(LibintInterface *, const char *, double *) { unsupported(__func__); }

void LibintInterface_compute_coupling_direct(LibintInterface *lint, LibintInterface *olint, double *dens,
                                             double *result) {
  if (!check_handle(lint, __func__) || !check_handle(olint, __func__)) return;
  if (!lint->ensure_all() || !olint->ensure_all()) return;
  const int n = lint->nbasis, no = olint->nbasis;
  cudaStream_t s = lint->stream;
  if (!olint->dD.ensure((size_t)no * no) || !lint->dG.ensure((size_t)n * n)) return;
  if (cudaMemcpyAsync(olint->dD.p, dens, sizeof(double) * no * no, cudaMemcpyHostToDevice, s) != cudaSuccess) {
    set_error("compute_coupling_direct: density upload failed");
    return;
  }
  // J of lint's species from olint's density, then keep the lower triangle
  if (!coupling(lint, olint, nullptr, olint->dD.p, lint->dG.p, nullptr, false, s)) return;
  std::vector<double> tmp((size_t)n * n);
  if (cudaMemcpyAsync(tmp.data(), lint->dG.p, sizeof(double) * n * n, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess) {
    set_error("compute_coupling_direct: result download failed");
    return;
  }
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) result[(size_t)i * n + j] = j > i ? 0.0 : tmp[(size_t)i * n + j];
}

void LibintInterface_compute_coupling_directIT(LibintInterface *lint, LibintInterface *olint, double *dens,
                                               double *coeff, double *result, int &p) {
  (void)dens;
  if (!check_handle(lint, __func__) || !check_handle(olint, __func__)) return;
  first_quarter(lint, olint, nullptr, coeff, p, result);
}

void LibintInterface_compute_alphabeta_direct(LibintInterface *lint, LibintInterface *olint, double *dens,
                                              double *otherdens, double *result) {
  if (!check_handle(lint, __func__) || !check_handle(olint, __func__)) return;
  if (!dens || !otherdens || !result) {
    set_error("%s: null argument", __func__);
    return;
  }
  if (!lint->ensure_all() || !olint->ensure_all()) return;
  const int n = lint->nbasis, no = olint->nbasis;
  cudaStream_t s = lint->stream;
  if (!olint->dD.ensure((size_t)no * no) || !lint->dG.ensure((size_t)n * n)) return;
  if (cudaMemcpyAsync(olint->dD.p, otherdens, sizeof(double) * no * no, cudaMemcpyHostToDevice, s) != cudaSuccess) {
    set_error("compute_alphabeta_direct: density upload failed");
    return;
  }
  // sum_{ij kl} D(ij) (ij|kl) D_other(kl) over the coupling integral set (raw
  // |v| < 1e-10 dropped, no screening) = sum_ij D(ij) J[D_other](ij)
  if (!coupling(lint, olint, nullptr, olint->dD.p, lint->dG.p, nullptr, false, s)) return;
  std::vector<double> J((size_t)n * n);
  if (cudaMemcpyAsync(J.data(), lint->dG.p, sizeof(double) * n * n, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess) {
    set_error("compute_alphabeta_direct: result download failed");
    return;
  }
  double e = 0.0;
  for (size_t k = 0; k < J.size(); ++k) e += dens[k] * J[k];
  result[0] = e;
}
void LibintInterface_compute_coupling_disk(LibintInterface *, LibintInterface *, const char *) {
  unsupported(__func__);
}
void libintinterface_compute_g12_disk(LibintInterface *, const char *, const double *, const double *, const int) {
  unsupported(__func__);
}
void libintinterface_compute_g12inter_disk(LibintInterface *, LibintInterface *, const char *, const double *,
                                           const double *, const int) {
  unsupported(__func__);
}
void libintinterface_compute_g12_direct(LibintInterface *lint, double *dens, double *result, double &factor,
                                        const double *coefficients, const double *exponents, const int pot_size) {
  if (!check_handle(lint, __func__)) return;
  if (!dens || !result) {
    set_error("%s: null argument", __func__);
    return;
  }
  if (!lint->ensure_sig()) return;
  const int n = lint->nbasis;
  cudaStream_t s = lint->stream;
  if (!upload_geminal(lint, coefficients, exponents, pot_size, __func__)) return;
  if (!lint->dD.ensure((size_t)n * n) || !lint->dDs.ensure((size_t)n * n) || !lint->dDs32.ensure((size_t)n * n) ||
      !lint->dGacc.ensure((size_t)n * n) || !lint->dG.ensure((size_t)n * n))
    return;
  if (cudaMemcpyAsync(lint->dD.p, dens, sizeof(double) * n * n, cudaMemcpyHostToDevice, s) != cudaSuccess) {
    set_error("%s: density upload failed", __func__);
    return;
  }
  if (!g12_build(lint, nullptr, lint->dD.p, factor, lint->dG.p, s)) return;
  if (cudaMemcpyAsync(result, lint->dG.p, sizeof(double) * n * n, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    set_error("%s: result download failed", __func__);
}

void libintinterface_compute_g12inter_direct(LibintInterface *lint, LibintInterface *olint, double *dens,
                                             double *result, const double *coefficients, const double *exponents,
                                             const int pot_size) {
  if (!check_handle(lint, __func__) || !check_handle(olint, __func__)) return;
  if (!dens || !result) {
    set_error("%s: null argument", __func__);
    return;
  }
  if (!lint->ensure_all() || !olint->ensure_all()) return;
  const int n = lint->nbasis, no = olint->nbasis;
  cudaStream_t s = lint->stream;
  if (!upload_geminal(lint, coefficients, exponents, pot_size, __func__)) return;
  if (!olint->dD.ensure((size_t)no * no) || !olint->dDsC.ensure((size_t)no * no) ||
      !olint->dDsC32.ensure((size_t)no * no) || !lint->dJacc.ensure((size_t)n * n) || !lint->dG.ensure((size_t)n * n))
    return;
  if (cudaMemcpyAsync(olint->dD.p, dens, sizeof(double) * no * no, cudaMemcpyHostToDevice, s) != cudaSuccess) {
    set_error("%s: density upload failed", __func__);
    return;
  }
  if (!g12_build(lint, olint, olint->dD.p, 0.0, lint->dG.p, s)) return;
  if (cudaMemcpyAsync(result, lint->dG.p, sizeof(double) * n * n, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    set_error("%s: result download failed", __func__);
}
void LibintInterface_compute_2body_directAll(LibintInterface *, double *, double *) { unsupported(__func__); }
void LibintInterface_compute_coupling_directAll(LibintInterface *, LibintInterface *, double *, double *) {
  unsupported(__func__);
}
void libintinterface_compute_g12_directAll(LibintInterface *, double *, double *, const double *, const double *,
                                           const int) {
  unsupported(__func__);
}
void libintinterface_compute_g12inter_directAll(LibintInterface *, LibintInterface *, double *, double *,
                                                const double *, const double *, const int) {
  unsupported(__func__);
}

const char *LowdinGB300_last_error(void) {
  std::lock_guard<std::mutex> lk(g_err_mu);
  static thread_local std::string copy;
  copy = g_err;
  return copy.c_str();
}

void LowdinGB300_clear_error(void) {
  std::lock_guard<std::mutex> lk(g_err_mu);
  g_err.clear();
}

void LowdinGB300_potential(LibintInterface *lint, int ncharge, const double *Z, const double *R, double *result) {
  if (!check_handle(lint, __func__)) return;
  const int n = lint->nbasis, nsh = lint->nshell();
  double V[225];
  for (int s1 = 0; s1 < nsh; ++s1)
    for (int s2 = 0; s2 < nsh; ++s2) {
      const HostShell &A = lint->shells[s1], &B = lint->shells[s2];
      potential_block(A, B, ncharge, Z, R, V);
      const int n1 = ncart(A.l), n2 = ncart(B.l);
      for (int f1 = 0; f1 < n1; ++f1)
        for (int f2 = 0; f2 < n2; ++f2) {
          const int i = lint->first[s1] + f1, j = lint->first[s2] + f2;
          result[(size_t)i * n + j] = V[f1 * n2 + f2] * lint->norma[i] * lint->norma[j];
        }
    }
}

// the external Gaussian-fit potential of a species, the matrix the reference
// builds in src/ints/DirectIntegralManager.f90:848-949 (each basis contraction
// times each potential component, then an overlap with the other contraction)
void LowdinGB300_gaussian_potential(LibintInterface *lint, int ncomp, const double *coefficients,
                                    const double *exponents, const double *origins, double *result) {
  if (!check_handle(lint, __func__)) return;
  if (ncomp < 0 || (ncomp > 0 && (!coefficients || !exponents || !origins)) || !result) {
    set_error("gaussian_potential: invalid components (ncomp=%d)", ncomp);
    return;
  }
  const int n = lint->nbasis, nsh = lint->nshell();
  double V[225];
  for (int s1 = 0; s1 < nsh; ++s1)
    for (int s2 = 0; s2 < nsh; ++s2) {
      const HostShell &A = lint->shells[s1], &B = lint->shells[s2];
      gaussian_potential_block(A, B, ncomp, coefficients, exponents, origins, V);
      const int n1 = ncart(A.l), n2 = ncart(B.l);
      for (int f1 = 0; f1 < n1; ++f1)
        for (int f2 = 0; f2 < n2; ++f2) {
          const int i = lint->first[s1] + f1, j = lint->first[s2] + f2;
          result[(size_t)i * n + j] = V[f1 * n2 + f2] * lint->norma[i] * lint->norma[j];
        }
    }
}

int LowdinGB300_one_body_device(LibintInterface *lint, int ncharge, const double *Z, const double *R, double *dS,
                                double *dT, double *dV, void *stream) {
  if (!check_handle(lint, __func__)) return -1;
  if (!lint->ensure_base()) return -1;
  cudaStream_t s = (cudaStream_t)stream;
  OneBodyParams p{};
  p.shells = lint->d_shells;
  p.alpha = lint->d_alpha;
  p.cn = lint->d_cn;
  p.first = lint->d_first;
  p.norma = lint->d_norma;
  p.nsh = lint->nshell();
  p.n = lint->nbasis;
  p.ncharge = dV ? ncharge : 0;
  p.S = dS;
  p.T = dT;
  p.V = dV;
  p.boys = lint->boys;
  if (p.ncharge > 0) {
    if (!lint->dZR.ensure((size_t)4 * ncharge)) return -1;
    if (cudaMemcpyAsync(lint->dZR.p, Z, ncharge * sizeof(double), cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(lint->dZR.p + ncharge, R, 3 * ncharge * sizeof(double), cudaMemcpyHostToDevice, s) !=
            cudaSuccess) {
      set_error("%s: charge upload failed", __func__);
      return -1;
    }
    p.Z = lint->dZR.p;
    p.R = lint->dZR.p + ncharge;
  } else if (dV) {
    if (cudaMemsetAsync(dV, 0, sizeof(double) * lint->nbasis * lint->nbasis, s) != cudaSuccess) return -1;
  }
  const cudaError_t e = launch_one_body(p, s);
  if (e != cudaSuccess) {
    set_error("%s: %s", __func__, cudaGetErrorString(e));
    return -1;
  }
  return 0;
}

int LowdinGB300_set_precision(LibintInterface *lint, int precision, double split) {
  if (!check_handle(lint, __func__)) return -1;
  if (precision != 0 && precision != 1) {
    set_error("%s: precision must be 0 (FP64) or 1 (FP32/FP64 split), got %d", __func__, precision);
    return -1;
  }
  if (precision == 1 && !(split > 0.0 && split < 1.0)) {
    set_error("%s: split bound %g outside (0, 1)", __func__, split);
    return -1;
  }
  lint->abi_precision = precision;
  lint->abi_split = precision ? split : 0.0;
  return 0;
}

int LowdinGB300_twobody_device(LibintInterface *lint, const double *dD, double *dG, double factor, int precision,
                               double split, void *stream) {
  if (!check_handle(lint, __func__)) return -1;
  return lint->twobody(dD, dG, factor, precision, split, (cudaStream_t)stream) ? 0 : -1;
}

int LowdinGB300_coupling_device(LibintInterface *a, LibintInterface *b, const double *dDa, const double *dDb,
                                double *dJa, double *dJb, int fp32, void *stream) {
  if (!check_handle(a, __func__) || !check_handle(b, __func__)) return -1;
  return coupling(a, b, dDa, dDb, dJa, dJb, fp32 != 0, (cudaStream_t)stream) ? 0 : -1;
}

long long LowdinGB300_last_quartets(LibintInterface *lint) {
  if (!lint) return -1;
  lint->collect_counts();
  return lint->last_quartets;
}

long long LowdinGB300_launch_count(void) { return lgb::launch_count(); }

int LowdinGB300_last_class_quartets(LibintInterface *lint, long long *out) {
  if (!check_handle(lint, __func__)) return -1;
  lint->collect_counts();
  for (int c = 0; c < kNumPairClasses * kNumPairClasses; ++c) out[c] = lint->class_quartets[c];
  return kNumPairClasses * kNumPairClasses;
}

int LowdinGB300_pair_class_counts(LibintInterface *lint, int all_pairs, int *out) {
  if (!check_handle(lint, __func__)) return -1;
  if (!(all_pairs ? lint->ensure_all() : lint->ensure_sig())) return -1;
  const PairList &L = all_pairs ? lint->all : lint->sig;
  for (int c = 0; c < kNumPairClasses; ++c) out[c] = L.count(c);
  return kNumPairClasses;
}

double LowdinGB300_measure_fma_tflops(int fp64) {
  double t = 0;
  if (lgb::measure_fma_tflops(fp64 != 0, &t) != cudaSuccess) {
    set_error("FMA throughput probe failed");
    return -1.0;
  }
  return t;
}

const char *LowdinGB300_version(void) { return "lowdin_gb300 0.1 (sm_103a, FP64/FP32 Obara-Saika, s p d f shells)"; }

}  // extern "C"

// ====================================================== allocation-free build
// LowdinGB300_twobody_device_noalloc: the device two-particle build for
// callers that must not allocate device memory once they are running -- a host
// program that owns every device byte through its own pool, or a serving loop
// that forbids allocations after warm-up.  Its work buffers (scaled densities, shell-block norms, accumulators,
// task list, counters) live in one file-scope device array instead of
// cudaMalloc'd memory; the handle's shell-pair data must already exist
// (LibintInterface_init_2body_ints, which does allocate, is called at set-up).
namespace {

constexpr int kNoAllocMaxBasis = 512;   // largest species (Cartesian functions)
constexpr int kNoAllocMaxShells = 512;  // largest species (shells)
constexpr int kNoAllocMaxTasks = 64;
constexpr size_t kNaN2 = (size_t)kNoAllocMaxBasis * kNoAllocMaxBasis;
constexpr size_t kNaS2 = (size_t)kNoAllocMaxShells * kNoAllocMaxShells;
constexpr size_t na_align(size_t x) { return (x + 255) / 256 * 256; }
constexpr size_t kNaOffDs = 0;
constexpr size_t kNaOffGacc = na_align(kNaOffDs + 8 * kNaN2);
constexpr size_t kNaOffDn = na_align(kNaOffGacc + 8 * kNaN2);
constexpr size_t kNaOffDs32 = na_align(kNaOffDn + 8 * kNaS2);
constexpr size_t kNaOffGacc32 = na_align(kNaOffDs32 + 4 * kNaN2);
constexpr size_t kNaOffDn32 = na_align(kNaOffGacc32 + 4 * kNaN2);
constexpr size_t kNaOffCnt = na_align(kNaOffDn32 + 4 * kNaS2);
constexpr size_t kNaOffTasks = na_align(kNaOffCnt + 8 * kNQC);
constexpr size_t kNaBytes = na_align(kNaOffTasks + sizeof(JKTask) * kNoAllocMaxTasks);  // ~9.5 MB

// Every GPU that loads the library holds this array until the process exits.
// In host code the name is only a host-side stand-in: the device address comes
// from cudaGetSymbolAddress, once per device.
__device__ __align__(256) unsigned char g_twobody_scratch[kNaBytes];

std::mutex g_na_mu;
std::vector<std::pair<int, unsigned char *>> g_na_addr;

// device address of the scratch array on the current device (set-up on the
// first call per device, with that device current)
bool noalloc_scratch(unsigned char **out) {
  int dev = 0;
  CK(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_na_mu);
  for (auto &e : g_na_addr)
    if (e.first == dev) {
      *out = e.second;
      return true;
    }
  unsigned char *p = nullptr;
  CK(cudaGetSymbolAddress((void **)&p, g_twobody_scratch));
  g_na_addr.push_back({dev, p});
  *out = p;
  return true;
}

}  // namespace

extern "C" {

size_t LowdinGB300_noalloc_scratch_bytes(void) { return kNaBytes; }

int LowdinGB300_twobody_device_noalloc(LibintInterface *lint, const double *dD, double *dG, double factor,
                                       int precision, double split, void *stream) {
  if (!check_handle(lint, __func__)) return -1;
  if (lint->dirty || !lint->have_sig || !lint->stream) {
    set_error("%s: call LibintInterface_init_2body_ints on this handle first (set-up allocates the shell-pair "
              "data; this entry point allocates nothing)",
              __func__);
    return -1;
  }
  const int n = lint->nbasis, nsh = lint->nshell();
  if (n > kNoAllocMaxBasis || nsh > kNoAllocMaxShells) {
    set_error("%s: species with %d functions / %d shells exceeds the allocation-free limit of %d functions and "
              "%d shells; use LowdinGB300_twobody_device",
              __func__, n, nsh, kNoAllocMaxBasis, kNoAllocMaxShells);
    return -1;
  }
  for (const auto &sh : lint->shells)
    if (sh.l > 2) {
      // quartet classes of two f shells against f or d need work arrays in
      // global memory beyond a CTA's shared memory, which only the allocating
      // entry point provides
      set_error("%s: shells above d (l=%d) are not supported by the allocation-free build; use "
                "LowdinGB300_twobody_device",
                __func__, sh.l);
      return -1;
    }
  unsigned char *base = nullptr;
  if (!noalloc_scratch(&base)) return -1;
  cudaStream_t s = (cudaStream_t)stream;
  double *Ds = (double *)(base + kNaOffDs), *Gacc = (double *)(base + kNaOffGacc), *Dn = (double *)(base + kNaOffDn);
  float *Ds32 = (float *)(base + kNaOffDs32), *Gacc32 = (float *)(base + kNaOffGacc32);
  float *Dn32 = (float *)(base + kNaOffDn32);
  unsigned long long *cnt = (unsigned long long *)(base + kNaOffCnt);
  JKTask *dtasks = (JKTask *)(base + kNaOffTasks);
  // task list on the host, flattened into the scratch array
  TaskSet<JKTask> ts;
  SpeciesBufs bf{Ds, Ds32, Dn, Dn32, Gacc, Gacc32};
  if (!lint->add_jk_tasks(ts, bf, 0.5 * factor, cnt)) return -1;
  std::vector<JKTask> flat;
  for (int c = 0; c < kNQC; ++c) {
    ts.off[c] = (int)flat.size();
    ts.cnt[c] = (int)ts.group[c].size();
    int b = 0;
    for (JKTask t : ts.group[c]) {
      ts.place(c, t, b);
      flat.push_back(t);
    }
    ts.nblk[c] = b;
  }
  if ((int)flat.size() > kNoAllocMaxTasks) {
    set_error("%s: %d tasks exceed the allocation-free limit of %d", __func__, (int)flat.size(), kNoAllocMaxTasks);
    return -1;
  }
  if (!flat.empty() &&
      cudaMemcpyAsync(dtasks, flat.data(), flat.size() * sizeof(JKTask), cudaMemcpyHostToDevice, s) != cudaSuccess) {
    set_error("%s: task upload failed", __func__);
    return -1;
  }
  ts.d = dtasks;
  // the array keeps the previous call's contents: clear what accumulates
  if (launch_prepare_density(dD, lint->d_norma, lint->d_shell_of, n, nsh, Ds, Ds32, Dn, Dn32, s) != cudaSuccess ||
      cudaMemsetAsync(Gacc, 0, sizeof(double) * n * n, s) != cudaSuccess ||
      cudaMemsetAsync(Gacc32, 0, sizeof(float) * n * n, s) != cudaSuccess ||
      cudaMemsetAsync(cnt, 0, sizeof(unsigned long long) * kNQC, s) != cudaSuccess) {
    set_error("%s: preparation failed", __func__);
    return -1;
  }
  if (!LibintInterface::launch_jk_groups(ts, precision, split, lint->boys, s)) return -1;
  if (launch_symmetrize(Gacc, Gacc32, lint->d_norma, n, 0.25, dG, s) != cudaSuccess) {
    set_error("%s: symmetrisation failed", __func__);
    return -1;
  }
  return 0;
}

}  // extern "C"
