// Host side of liblowdin_gb300.so: the per-species handle behind the
// LibintInterface_* C ABI, device data of a species (class-binned shell pairs
// sorted by Schwarz factor), and the builds that queue the integral kernels.
#include <algorithm>
#include <array>
#include <cfloat>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include <cublas_v2.h>

#include "../../include/lowdin_gb300.h"
#include "kernels.cuh"

using namespace lgb;

// ------------------------------------------------------------------ errors --
namespace {
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

#define CK(call)                                                                          \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess) {                                                              \
      set_error("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
      return false;                                                                       \
    }                                                                                     \
  } while (0)

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
struct HostShell {
  int l = 0, nprim = 0;
  double O[3] = {0, 0, 0};
  std::vector<double> alpha, cn;  // cn = coefficient * primitive norm of x^l
};

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

// --------------------------------------------------------- device species --
template <typename T>
bool dev_upload(T *&dst, const std::vector<T> &src) {
  if (dst) cudaFree(dst);
  dst = nullptr;
  if (src.empty()) return true;
  CK(cudaMalloc(&dst, src.size() * sizeof(T)));
  CK(cudaMemcpy(dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice));
  return true;
}

struct PairList {
  std::vector<PairRec> h;
  std::vector<PrimRec> hp;
  int start[kNumPairClasses + 1] = {0};
  PairRec *d = nullptr;
  PrimRec *dp = nullptr;
  PairRec32 *d32 = nullptr;   // FP32 copies for the FP32 kernels
  PrimRec32 *dp32 = nullptr;
  void release() {
    if (d) cudaFree(d);
    if (dp) cudaFree(dp);
    if (d32) cudaFree(d32);
    if (dp32) cudaFree(dp32);
    d = nullptr;
    dp = nullptr;
    d32 = nullptr;
    dp32 = nullptr;
  }
  int count(int pc) const { return start[pc + 1] - start[pc]; }
  // uploads the FP64 records and their FP32 copies
  bool upload() {
    release();
    std::vector<PairRec32> h32(h.size());
    std::vector<PrimRec32> hp32(hp.size());
    for (size_t i = 0; i < h.size(); ++i) {
      const PairRec &a = h[i];
      PairRec32 &b = h32[i];
      b.sa = a.sa; b.sb = a.sb; b.fa = a.fa; b.fb = a.fb; b.prim0 = a.prim0; b.nprim = a.nprim;
      b.la = a.la; b.lb = a.lb;
      for (int k = 0; k < 3; ++k) {
        b.A[k] = (float)a.A[k];
        b.AB[k] = (float)a.AB[k];
      }
      b.Q = (float)a.Q;
      b.pad = 0.f;
    }
    for (size_t i = 0; i < hp.size(); ++i) {
      const PrimRec &a = hp[i];
      PrimRec32 &b = hp32[i];
      b.p = (float)a.p; b.inv_p = (float)a.inv_p; b.Kt = (float)a.Kt; b.pad = 0.f;
      for (int k = 0; k < 3; ++k) {
        b.P[k] = (float)a.P[k];
        b.PA[k] = (float)a.PA[k];
      }
    }
    return dev_upload(d, h) && dev_upload(dp, hp) && dev_upload(d32, h32) && dev_upload(dp32, hp32);
  }
};

template <typename T>
struct DevBuf {
  T *p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  ~DevBuf() { release(); }
  bool ensure(size_t want) {
    if (want <= n && p) return true;
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
    CK(cudaMalloc(&p, want * sizeof(T) + 16));
    n = want;
    return true;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
};

constexpr int kNQC = kNumPairClasses * kNumPairClasses;

// device buffers of one species in one build: scaled density (FP64 + FP32),
// shell-block norms (FP64 + FP32) and the output accumulators (FP64 + FP32)
struct SpeciesBufs {
  const double *Ds;
  const float *Ds32;
  const double *Dn;
  const float *Dn32;
  double *G;
  float *G32;
};

// Tasks grouped by quartet class (bra pair class * 6 + ket pair class); one
// device array holds every group, each group is one launch.
template <typename T>
struct TaskSet {
  std::vector<T> group[kNQC];
  T *d = nullptr;
  size_t cap = 0;
  int off[kNQC] = {0}, cnt[kNQC] = {0}, nblk[kNQC] = {0};
  void clear() {
    for (auto &g : group) g.clear();
  }
  void add(int cb, int ck, const T &t) { group[cb * kNumPairClasses + ck].push_back(t); }
  // assigns blk0 / nbx and copies all groups to the device, ordered on stream s;
  // with `on`, a task whose flag (t.active - flag_base) is off in `on` is left
  // out, so the launches of switched-off systems carry no blocks at all
  bool upload(cudaStream_t s, const int *flag_base = nullptr, const std::vector<int> *on = nullptr) {
    std::vector<T> flat;
    for (int c = 0; c < kNQC; ++c) {
      off[c] = (int)flat.size();
      int b = 0;
      for (T t : group[c]) {
        if (on && t.active && !(*on)[t.active - flag_base]) continue;
        t.nbx = task_nbx(t.nket);
        t.blk0 = b;
        b += t.nbx * task_nby(t.nbra);
        flat.push_back(t);
      }
      cnt[c] = (int)flat.size() - off[c];
      nblk[c] = b;
    }
    if (flat.empty()) return true;
    if (flat.size() > cap) {
      if (d) cudaFree(d);
      d = nullptr;
      cap = 0;
      CK(cudaMalloc(&d, flat.size() * sizeof(T)));
      cap = flat.size();
    }
    // pageable source: the call returns once the data is staged, the copy is
    // ordered on s after the kernels that read the previous contents
    CK(cudaMemcpyAsync(d, flat.data(), flat.size() * sizeof(T), cudaMemcpyHostToDevice, s));
    return true;
  }
  void release() {
    if (d) cudaFree(d);
    d = nullptr;
    cap = 0;
  }
};


}  // namespace

struct LibintInterface {
  int id = 0;
  bool is_electron = true;
  int stack_size = 0;
  std::vector<HostShell> shells;
  std::vector<int> first;  // shell -> first basis function
  std::vector<double> norma;
  std::vector<std::pair<int, std::array<double, 3>>> atoms;
  int nbasis = 0;

  // device state (valid while !dirty)
  bool dirty = true;
  int device = -1;
  cudaStream_t stream = nullptr;
  BoysTables boys{nullptr, nullptr};
  PairList sig;   // significant pairs (pair-list test), sorted by Schwarz factor inside a class
  PairList all;   // every unordered pair (coupling)
  bool have_sig = false, have_all = false;
  double *d_norma = nullptr;
  int *d_shell_of = nullptr;
  DevShell *d_shells = nullptr;
  double *d_alpha = nullptr, *d_cn = nullptr;
  int *d_first = nullptr;
  DevBuf<double> dZR;          // point charges and positions of the last one-body call
  DevBuf<double> dD, dDs, dDn, dGacc, dG, dA, dC, dDsC, dJacc;
  DevBuf<float> dDs32, dDn32, dGacc32, dDsC32, dJacc32;
  DevBuf<unsigned long long> dcount;
  unsigned long long *hcount = nullptr;   // pinned copy of dcount, read once its stream is done
  cudaStream_t count_stream = nullptr;
  bool count_pending = false;
  long long last_quartets = -1;
  long long class_quartets[kNQC] = {0};
  TaskSet<JKTask> jk;        // cached J/K tasks of the handle's own buffers
  double jk_hf = 0.0;
  bool jk_ready = false;
  TaskSet<CPTask> cp;        // coupling tasks of the last coupling call (this handle as bra)

  ~LibintInterface() { release_device(); }

  void release_device() {
    sig.release();
    all.release();
    if (d_norma) cudaFree(d_norma);
    if (d_shell_of) cudaFree(d_shell_of);
    for (void *q : {(void *)d_shells, (void *)d_alpha, (void *)d_cn, (void *)d_first})
      if (q) cudaFree(q);
    d_norma = nullptr;
    d_shell_of = nullptr;
    d_shells = nullptr;
    d_alpha = d_cn = nullptr;
    d_first = nullptr;
    dZR.release();
    dD.release(); dDs.release(); dDn.release(); dGacc.release(); dG.release(); dA.release(); dC.release();
    dDsC.release(); dJacc.release();
    dDs32.release(); dDn32.release(); dGacc32.release(); dDsC32.release(); dJacc32.release();
    dcount.release();
    if (hcount) cudaFreeHost(hcount);
    hcount = nullptr;
    count_pending = false;
    jk.release();
    cp.release();
    jk_ready = false;
    if (stream) cudaStreamDestroy(stream);
    stream = nullptr;
    have_sig = have_all = false;
    dirty = true;
  }
  int nshell() const { return (int)shells.size(); }

  bool ensure_base() {
    if (!dirty && stream) return true;
    int dev = 0;
    CK(cudaGetDevice(&dev));
    if (stream && dev != device) release_device();
    device = dev;
    if (!stream) CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    if (!device_boys(boys)) return false;
    for (const auto &s : shells)
      if (s.l > kMaxL) {
        set_error("shell with l=%d: this build handles l <= %d", s.l, kMaxL);
        return false;
      }
    std::vector<int> shell_of(nbasis);
    for (int s = 0; s < nshell(); ++s)
      for (int i = first[s]; i < first[s] + ncart(shells[s].l); ++i) shell_of[i] = s;
    if (d_norma) cudaFree(d_norma);
    if (d_shell_of) cudaFree(d_shell_of);
    d_norma = nullptr;
    d_shell_of = nullptr;
    if (!dev_upload(d_norma, norma)) return false;
    if (!dev_upload(d_shell_of, shell_of)) return false;
    // shells for the one-electron kernels
    std::vector<DevShell> ds(nshell());
    std::vector<double> al, cn;
    for (int k = 0; k < nshell(); ++k) {
      const HostShell &h = shells[k];
      ds[k].l = h.l;
      ds[k].nprim = h.nprim;
      ds[k].p0 = (int)al.size();
      ds[k].pad = 0;
      for (int d = 0; d < 3; ++d) ds[k].O[d] = h.O[d];
      al.insert(al.end(), h.alpha.begin(), h.alpha.end());
      cn.insert(cn.end(), h.cn.begin(), h.cn.end());
    }
    if (!dev_upload(d_shells, ds) || !dev_upload(d_alpha, al) || !dev_upload(d_cn, cn) ||
        !dev_upload(d_first, first))
      return false;
    have_sig = have_all = false;
    jk_ready = false;
    dirty = false;
    return true;
  }

  PairRec make_pair(int s1, int s2, std::vector<PrimRec> &prims) const {
    // canonical order: larger l first; equal l keeps (s1, s2)
    int a = s1, b = s2;
    if (shells[b].l > shells[a].l) std::swap(a, b);
    const HostShell &A = shells[a], &B = shells[b];
    PairRec r{};
    r.sa = a;
    r.sb = b;
    r.fa = first[a];
    r.fb = first[b];
    r.la = A.l;
    r.lb = B.l;
    r.prim0 = (int)prims.size();
    r.nprim = A.nprim * B.nprim;
    double AB2 = 0;
    for (int d = 0; d < 3; ++d) {
      r.A[d] = A.O[d];
      r.AB[d] = A.O[d] - B.O[d];
      AB2 += r.AB[d] * r.AB[d];
    }
    r.Q = 0;
    for (int i = 0; i < A.nprim; ++i)
      for (int j = 0; j < B.nprim; ++j) {
        const double x = A.alpha[i], y = B.alpha[j], p = x + y;
        PrimRec q{};
        q.p = p;
        q.inv_p = 1.0 / p;
        for (int d = 0; d < 3; ++d) {
          q.P[d] = (x * A.O[d] + y * B.O[d]) / p;
          q.PA[d] = q.P[d] - A.O[d];
        }
        q.Kt = kSqrt2Pi52 * std::exp(-x * y / p * AB2) * A.cn[i] * B.cn[j] / p;
        prims.push_back(q);
      }
    return r;
  }

  // Bins pairs by class (stable), rebuilding the primitive array in the new order.
  static void bin_pairs(PairList &L, std::vector<PairRec> &raw, const std::vector<PrimRec> &rawp, bool by_q) {
    std::stable_sort(raw.begin(), raw.end(), [&](const PairRec &x, const PairRec &y) {
      const int cx_ = pair_class(x.la, x.lb), cy_ = pair_class(y.la, y.lb);
      if (cx_ != cy_) return cx_ < cy_;
      if (by_q && x.Q != y.Q) return x.Q > y.Q;
      return false;
    });
    L.h.clear();
    L.hp.clear();
    for (int c = 0; c <= kNumPairClasses; ++c) L.start[c] = 0;
    for (auto r : raw) {
      const int n0 = (int)L.hp.size();
      for (int k = 0; k < r.nprim; ++k) L.hp.push_back(rawp[r.prim0 + k]);
      r.prim0 = n0;
      L.h.push_back(r);
      L.start[pair_class(r.la, r.lb) + 1]++;
    }
    for (int c = 0; c < kNumPairClasses; ++c) L.start[c + 1] += L.start[c];
  }

  bool compute_schwarz(PairList &L) {
    DevBuf<double> dq;
    if (!dq.ensure(L.h.size())) return false;
    for (int pc = 0; pc < kNumPairClasses; ++pc) {
      if (!L.count(pc)) continue;
      SchwarzParams sp{L.d, L.dp, L.start[pc], L.count(pc), dq.p, boys};
      CK(launch_schwarz(pc, sp, stream));
    }
    std::vector<double> q(L.h.size());
    CK(cudaMemcpyAsync(q.data(), dq.p, q.size() * sizeof(double), cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    dq.release();
    for (size_t i = 0; i < q.size(); ++i) L.h[i].Q = q[i];
    return true;
  }

  // significant pairs of init_2body_ints (Libint2Iface.cpp:3248-3342): same
  // centre, or Frobenius norm of the raw overlap block >= 1e-12
  bool ensure_sig() {
    if (!ensure_base()) return false;
    if (have_sig) return true;
    std::vector<PairRec> raw;
    std::vector<PrimRec> rawp;
    double S[225];
    for (int s1 = 0; s1 < nshell(); ++s1)
      for (int s2 = 0; s2 <= s1; ++s2) {
        const HostShell &A = shells[s1], &B = shells[s2];
        bool sigf = A.O[0] == B.O[0] && A.O[1] == B.O[1] && A.O[2] == B.O[2];
        if (!sigf) {
          overlap_block(A, B, S, nullptr);
          double nrm = 0;
          for (int i = 0; i < ncart(A.l) * ncart(B.l); ++i) nrm += S[i] * S[i];
          sigf = std::sqrt(nrm) >= 1e-12;
        }
        if (sigf) raw.push_back(make_pair(s1, s2, rawp));
      }
    bin_pairs(sig, raw, rawp, false);
    if (!sig.upload()) return false;
    if (!compute_schwarz(sig)) return false;
    // sort by decreasing Schwarz factor inside each class
    std::vector<PairRec> tmp = sig.h;
    std::vector<PrimRec> tmpp = sig.hp;
    bin_pairs(sig, tmp, tmpp, true);
    if (!sig.upload()) return false;
    have_sig = true;
    return true;
  }

  bool ensure_all() {
    if (!ensure_base()) return false;
    if (have_all) return true;
    std::vector<PairRec> raw;
    std::vector<PrimRec> rawp;
    for (int s1 = 0; s1 < nshell(); ++s1)
      for (int s2 = 0; s2 <= s1; ++s2) raw.push_back(make_pair(s1, s2, rawp));
    bin_pairs(all, raw, rawp, false);
    if (!all.upload()) return false;
    // Schwarz factors of every pair: exact skip of quartets whose bound is
    // below the coupling cut, and the mixed-precision split; sorted by Q inside
    // a class so skipped quartets cluster into whole warps
    if (!compute_schwarz(all)) return false;
    std::vector<PairRec> tmp = all.h;
    std::vector<PrimRec> tmpp = all.hp;
    bin_pairs(all, tmp, tmpp, true);
    if (!all.upload()) return false;
    have_all = true;
    return true;
  }

  // dG = J[dD] + factor K[dD]; dD, dG device n x n
  bool twobody(const double *dDin, double *dGout, double factor, int precision, double split, cudaStream_t s) {
    if (!ensure_sig()) return false;
    const int n = nbasis, nsh = nshell();
    if (!dDs.ensure((size_t)n * n) || !dDn.ensure((size_t)nsh * nsh) || !dGacc.ensure((size_t)n * n) ||
        !dDs32.ensure((size_t)n * n) || !dDn32.ensure((size_t)nsh * nsh) || !dGacc32.ensure((size_t)n * n) ||
        !dcount.ensure(kNQC))
      return false;
    if (!jk_ready || jk_hf != 0.5 * factor) {
      jk.clear();
      SpeciesBufs b{dDs.p, dDs32.p, dDn.p, dDn32.p, dGacc.p, dGacc32.p};
      if (!add_jk_tasks(jk, b, 0.5 * factor, dcount.p)) return false;
      if (!jk.upload(s)) return false;
      jk_hf = 0.5 * factor;
      jk_ready = true;
    }
    CK(launch_prepare_density(dDin, d_norma, d_shell_of, n, nsh, dDs.p, dDs32.p, dDn.p, dDn32.p, s));
    CK(cudaMemsetAsync(dGacc.p, 0, sizeof(double) * n * n, s));
    CK(cudaMemsetAsync(dGacc32.p, 0, sizeof(float) * n * n, s));
    CK(cudaMemsetAsync(dcount.p, 0, sizeof(unsigned long long) * kNQC, s));
    if (!launch_jk_groups(jk, precision, split, boys, s)) return false;
    CK(launch_symmetrize(dGacc.p, dGacc32.p, d_norma, n, 0.25, dGout, s));
    // the quartet counts travel with the result; they are summed when asked for
    if (!hcount) CK(cudaHostAlloc((void **)&hcount, kNQC * sizeof(unsigned long long), cudaHostAllocDefault));
    CK(cudaMemcpyAsync(hcount, dcount.p, kNQC * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    count_stream = s;
    count_pending = true;
    return true;
  }

  void collect_counts() {
    if (!count_pending) return;
    if (cudaStreamSynchronize(count_stream) != cudaSuccess) {
      set_error("quartet counts: stream synchronisation failed");
      return;
    }
    count_pending = false;
    last_quartets = 0;
    for (int c = 0; c < kNQC; ++c) {
      class_quartets[c] = (long long)hcount[c];
      last_quartets += (long long)hcount[c];
    }
  }

  // J/K tasks of this species into ts: one task per (bra class >= ket class)
  bool add_jk_tasks(TaskSet<JKTask> &ts, const SpeciesBufs &bf, double hf, unsigned long long *counters) {
    if (!ensure_sig()) return false;
    for (int cb = 0; cb < kNumPairClasses; ++cb)
      for (int ck = 0; ck <= cb; ++ck) {
        if (!sig.count(cb) || !sig.count(ck)) continue;
        if (!class_supported(cb, ck)) {
          set_error("quartet class (%d,%d|%d,%d) is not built into this library", pc_la(cb), pc_lb(cb), pc_la(ck),
                    pc_lb(ck));
          return false;
        }
        JKTask t{};
        t.pairs = sig.d;
        t.prims = sig.dp;
        t.pairs32 = sig.d32;
        t.prims32 = sig.dp32;
        t.Ds = bf.Ds;
        t.Ds32 = bf.Ds32;
        t.Dn = bf.Dn;
        t.Dn32 = bf.Dn32;
        t.Gacc = bf.G;
        t.Gacc32 = bf.G32;
        t.count = counters ? counters + cb * kNumPairClasses + ck : nullptr;
        t.hf = hf;
        t.bra0 = sig.start[cb];
        t.nbra = sig.count(cb);
        t.ket0 = sig.start[ck];
        t.nket = sig.count(ck);
        t.n = nbasis;
        t.nsh = nshell();
        t.triangle = cb == ck;
        t.screen = is_electron ? 1 : 0;
        ts.add(cb, ck, t);
      }
    return true;
  }

  static bool launch_jk_groups(const TaskSet<JKTask> &ts, int precision, double split, BoysTables boys,
                               cudaStream_t s, double skip = 0.0) {
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
      if (precision == 0) {
        tl.split = 0.0;
        CK(launch_jk_tasks(cb, ck, false, ts.d + ts.off[c], tl, s));
      } else {
        tl.split = split;
        tl.lower = 0;
        CK(launch_jk_tasks(cb, ck, false, ts.d + ts.off[c], tl, s));
        tl.lower = 1;
        CK(launch_jk_tasks(cb, ck, true, ts.d + ts.off[c], tl, s));
      }
    }
    return true;
  }
};

// coupling tasks of species pair (A bra, B ket) into ts
bool add_cp_tasks(TaskSet<CPTask> &ts, LibintInterface *A, LibintInterface *B, const SpeciesBufs &ba,
                  const SpeciesBufs &bb, bool want_a, bool want_b, double scale,
                  unsigned long long *counters = nullptr) {
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
                      double skip = 0.0) {
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
      tl.lower = 0;
      CK(launch_cp_tasks(cb, ck, false, ts.d + ts.off[c], tl, s));
      tl.lower = 1;
      CK(launch_cp_tasks(cb, ck, true, ts.d + ts.off[c], tl, s));
    } else {
      CK(launch_cp_tasks(cb, ck, mode == 1, ts.d + ts.off[c], tl, s));
    }
  }
  return true;
}

namespace {

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

bool check_handle(LibintInterface *l, const char *fn) {
  if (!l) {
    set_error("%s: null handle", fn);
    return false;
  }
  return true;
}

void unsupported(const char *fn) { set_error("%s is not provided by this library (direct Coulomb path only)", fn); }

}  // namespace

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
  if (!lint->twobody(lint->dD.p, lint->dG.p, factor, 0, 0.0, s)) return;
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

void LibintInterface_compute_alphabeta_direct(LibintInterface *, LibintInterface *, double *, double *, double *) {
  unsupported(__func__);
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
void libintinterface_compute_g12_direct(LibintInterface *, double *, double *, double &, const double *,
                                        const double *, const int) {
  unsupported(__func__);
}
void libintinterface_compute_g12inter_direct(LibintInterface *, LibintInterface *, double *, double *,
                                             const double *, const double *, const int) {
  unsupported(__func__);
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

const char *LowdinGB300_version(void) { return "lowdin_gb300 0.1 (sm_103a, FP64/FP32 Obara-Saika, s p d shells)"; }

}  // extern "C"

// ================================================================== batches
// A batch holds many molecular systems (each a list of species handles) whose
// two-particle and coupling builds run together: every species' density
// preparation in one kernel, every J/K task of a quartet class in one launch,
// every coupling task of a class in one launch, every output in one kernel.
// Nothing in LowdinGB300_batch_fock waits on the host, so the sequence can be
// captured in a CUDA graph once the batch is finalised.
struct LowdinGB300_Batch {
  struct Spec {
    LibintInterface *h;
    double q, factor;
    int two_body;
    const double *P;
    double *G, *J;
    int sys;
    int ld;            // row stride of P, G, J
  };
  DevBuf<int> active;  // per system: built while non-zero (LowdinGB300_batch_set_active)
  std::vector<Spec> sp;
  std::vector<int> sys_first;
  bool finalized = false;
  DevBuf<double> Ds, Dn, Gacc, Jacc;
  DevBuf<float> Ds32, Dn32, Gacc32, Jacc32;
  DevBuf<unsigned long long> cnt;
  DevBuf<SpeciesSlot> slots;
  long long total = 0;
  int nslots = 0;
  TaskSet<JKTask> jk;
  TaskSet<CPTask> cp;
  BoysTables boys{nullptr, nullptr};
  long long class_quartets[kNQC] = {0};

  // The launch sequence of one build, captured once per precision mode into
  // a CUDA graph and replayed (every pointer and task list is fixed once the
  // batch is finalised).  The first build runs eagerly: it performs the
  // one-time kernel set-up that must not happen inside a capture.
  struct Graph {
    cudaGraphExec_t exec = nullptr;
    double split = 0.0, skip = 0.0;
    long long launches = 0;
  };
  double skip = 0.0;   // mixed builds: density-weighted bound below which quartets are dropped
  std::vector<int> on; // host copy of the per-system flags
  bool tasks_dirty = false;
  Graph graphs[4];
  cudaStream_t capture = nullptr;
  bool use_graph = true;
  long long calls = 0;

  ~LowdinGB300_Batch() {
    drop_graphs();
    if (capture) cudaStreamDestroy(capture);
    Ds.release(); Dn.release(); Gacc.release(); Jacc.release(); cnt.release(); slots.release();
    Ds32.release(); Dn32.release(); Gacc32.release(); Jacc32.release();
    active.release();
    jk.release(); cp.release();
  }

  void drop_graphs() {
    for (auto &g : graphs) {
      if (g.exec) cudaGraphExecDestroy(g.exec);
      g = Graph{};
    }
  }

  bool finalize(cudaStream_t s) {
    if (sp.empty()) {
      set_error("batch_finalize: empty batch");
      return false;
    }
    drop_graphs();
    calls = 0;
    if (!device_boys(boys)) return false;
    // device buffers of the handles
    for (auto &x : sp) {
      if (!x.h->ensure_all()) return false;
      if (x.two_body && !x.h->ensure_sig()) return false;
    }
    // arena layout
    std::vector<long long> off(sp.size()), dnoff(sp.size(), -1);
    long long tot = 0, dtot = 0;
    for (size_t k = 0; k < sp.size(); ++k) {
      off[k] = tot;
      tot += (long long)sp[k].h->nbasis * sp[k].h->nbasis;
      // shell-block norms of every species: J/K screening (electrons) and the
      // mixed-precision split of J/K and couplings
      dnoff[k] = dtot;
      dtot += (long long)sp[k].h->nshell() * sp[k].h->nshell();
    }
    total = tot;
    const long long dsz = dtot > 0 ? dtot : 1;
    if (!Ds.ensure(tot) || !Gacc.ensure(tot) || !Jacc.ensure(tot) || !Dn.ensure(dsz) || !Ds32.ensure(tot) ||
        !Gacc32.ensure(tot) || !Jacc32.ensure(tot) || !Dn32.ensure(dsz) || !cnt.ensure(2 * kNQC))
      return false;
    std::vector<SpeciesSlot> hs(sp.size());
    std::vector<SpeciesBufs> bf(sp.size());
    jk.clear();
    cp.clear();
    const int nsys = (int)sys_first.size();
    if (!active.ensure(std::max(1, nsys))) return false;
    {
      std::vector<int> ones(std::max(1, nsys), 1);
      CK(cudaMemcpyAsync(active.p, ones.data(), ones.size() * sizeof(int), cudaMemcpyHostToDevice, s));
      CK(cudaStreamSynchronize(s));
    }
    // tasks added since `before` belong to system `sys`: they read its active flag
    auto mark = [&](auto &ts, const std::vector<size_t> &before, int sys) {
      for (int c = 0; c < kNQC; ++c)
        for (size_t i = before[c]; i < ts.group[c].size(); ++i) ts.group[c][i].active = active.p + sys;
    };
    auto sizes = [](const auto &ts) {
      std::vector<size_t> v(kNQC);
      for (int c = 0; c < kNQC; ++c) v[c] = ts.group[c].size();
      return v;
    };
    for (size_t k = 0; k < sp.size(); ++k) {
      const Spec &x = sp[k];
      SpeciesSlot &S = hs[k];
      S.P = x.P;
      S.Ds = Ds.p + off[k];
      S.Ds32 = Ds32.p + off[k];
      S.Dn = dnoff[k] >= 0 ? Dn.p + dnoff[k] : nullptr;
      S.Dn32 = dnoff[k] >= 0 ? Dn32.p + dnoff[k] : nullptr;
      S.norma = x.h->d_norma;
      S.shell_of = x.h->d_shell_of;
      S.Gacc = x.two_body ? Gacc.p + off[k] : nullptr;
      S.Gacc32 = x.two_body ? Gacc32.p + off[k] : nullptr;
      S.Jacc = Jacc.p + off[k];
      S.Jacc32 = Jacc32.p + off[k];
      S.G = x.G;
      S.J = x.J;
      S.gscale = 0.25 * x.q * x.q;
      S.n = x.h->nbasis;
      S.nsh = x.h->nshell();
      S.off = off[k];
      S.ld = x.ld > 0 ? x.ld : S.n;
      S.active = active.p + x.sys;
      if (x.two_body) {
        // non-electron species are not screened: their norm pointers are never read
        SpeciesBufs b{S.Ds, S.Ds32, S.Dn ? S.Dn : Dn.p, S.Dn32 ? S.Dn32 : Dn32.p, S.Gacc, S.Gacc32};
        const auto before = sizes(jk);
        if (!x.h->add_jk_tasks(jk, b, 0.5 * x.factor, cnt.p)) return false;
        mark(jk, before, x.sys);
      }
      bf[k] = SpeciesBufs{S.Ds, S.Ds32, S.Dn, S.Dn32, S.Jacc, S.Jacc32};
    }
    // coupling tasks: every species pair of a system
    for (size_t a = 0; a < sp.size(); ++a)
      for (size_t b = a + 1; b < sp.size(); ++b) {
        if (sp[a].sys != sp[b].sys) continue;
        const auto before = sizes(cp);
        if (!add_cp_tasks(cp, sp[a].h, sp[b].h, bf[a], bf[b], true, true, sp[a].q * sp[b].q, cnt.p + kNQC))
          return false;
        mark(cp, before, sp[a].sys);
      }
    on.assign(std::max(1, nsys), 1);
    tasks_dirty = false;
    nslots = (int)hs.size();
    if (!slots.ensure(hs.size())) return false;
    CK(cudaMemcpyAsync(slots.p, hs.data(), hs.size() * sizeof(SpeciesSlot), cudaMemcpyHostToDevice, s));
    if (!jk.upload(s) || !cp.upload(s)) return false;
    CK(cudaStreamSynchronize(s));
    finalized = true;
    return true;
  }

  bool fock(int precision, double split, cudaStream_t s) {
    if (!finalized) {
      set_error("batch_fock: batch not finalised");
      return false;
    }
    if (tasks_dirty) {
      // systems were switched off or on: launch only the active systems' tasks
      if (!jk.upload(s, active.p, &on) || !cp.upload(s, active.p, &on)) return false;
      drop_graphs();
      tasks_dirty = false;
    }
    if (!use_graph || calls++ == 0) return fock_sequence(precision, split, s);
    Graph &g = graphs[precision & 3];
    if (!g.exec || g.split != split || g.skip != skip) {
      if (g.exec) cudaGraphExecDestroy(g.exec);
      g = Graph{};
      if (!capture) CK(cudaStreamCreateWithFlags(&capture, cudaStreamNonBlocking));
      const long long l0 = launch_count();
      CK(cudaStreamBeginCapture(capture, cudaStreamCaptureModeThreadLocal));
      const bool ok = fock_sequence(precision, split, capture);
      cudaGraph_t graph = nullptr;
      const cudaError_t e = cudaStreamEndCapture(capture, &graph);
      const long long captured = launch_count() - l0;
      count_launches(-captured);   // nothing ran during the capture
      if (!ok || e != cudaSuccess || !graph) {
        if (graph) cudaGraphDestroy(graph);
        set_error("batch_fock: graph capture failed (%s)", cudaGetErrorString(e));
        return false;
      }
      const cudaError_t ei = cudaGraphInstantiate(&g.exec, graph, 0);
      cudaGraphDestroy(graph);
      if (ei != cudaSuccess) {
        g = Graph{};
        set_error("batch_fock: graph instantiation failed (%s)", cudaGetErrorString(ei));
        return false;
      }
      g.split = split;
      g.skip = skip;
      g.launches = captured;
    }
    CK(cudaGraphLaunch(g.exec, s));
    count_launches(g.launches);
    return true;
  }

  // every launch of one build, in stream order
  bool fock_sequence(int precision, double split, cudaStream_t s) {
    CK(cudaMemsetAsync(Dn.p, 0, Dn.n * sizeof(double), s));
    CK(cudaMemsetAsync(Dn32.p, 0, Dn32.n * sizeof(float), s));
    CK(cudaMemsetAsync(cnt.p, 0, 2 * kNQC * sizeof(unsigned long long), s));
    CK(launch_prepare_batch(slots.p, nslots, total, s));
    const int jk_mixed = precision & 1;
    if (!LibintInterface::launch_jk_groups(jk, jk_mixed, jk_mixed ? split : 0.0, boys, s, skip)) return false;
    if (!launch_cp_groups(cp, (precision & 2) ? 2 : 0, split, boys, s, skip)) return false;
    CK(launch_finalize_batch(slots.p, nslots, total, s));
    return true;
  }
};

extern "C" {

LowdinGB300_Batch *LowdinGB300_batch_new(void) { return new LowdinGB300_Batch(); }

void LowdinGB300_batch_del(LowdinGB300_Batch *b) { delete b; }

int LowdinGB300_batch_add_system(LowdinGB300_Batch *b, LibintInterface **species, int nspecies,
                                 const double *charges, const double *factors, const int *two_body,
                                 const double **dP, double **dG, double **dJ) {
  return LowdinGB300_batch_add_system_ld(b, species, nspecies, charges, factors, two_body, dP, dG, dJ, nullptr);
}

int LowdinGB300_batch_set_skip(LowdinGB300_Batch *b, double skip) {
  if (!b || !(skip >= 0.0)) return -1;
  b->skip = skip;
  return 0;
}

int LowdinGB300_batch_set_active(LowdinGB300_Batch *b, const int *flags, void *stream) {
  if (!b || !b->finalized || !flags) return -1;
  const size_t nsys = b->sys_first.size();
  if (cudaMemcpyAsync(b->active.p, flags, nsys * sizeof(int), cudaMemcpyHostToDevice, (cudaStream_t)stream) !=
      cudaSuccess) {
    set_error("batch_set_active: copy failed");
    return -1;
  }
  for (size_t i = 0; i < nsys; ++i) {
    const int f = flags[i] != 0;
    if (b->on[i] != f) b->tasks_dirty = true;
    b->on[i] = f;
  }
  return 0;
}

int LowdinGB300_batch_add_system_ld(LowdinGB300_Batch *b, LibintInterface **species, int nspecies,
                                    const double *charges, const double *factors, const int *two_body,
                                    const double **dP, double **dG, double **dJ, const int *ld) {
  if (!b || !species || nspecies <= 0) {
    set_error("batch_add_system: invalid arguments");
    return -1;
  }
  const int sys = (int)b->sys_first.size();
  const int first = (int)b->sp.size();
  b->sys_first.push_back(first);
  for (int k = 0; k < nspecies; ++k) {
    if (!check_handle(species[k], __func__)) return -1;
    if (ld && ld[k] < species[k]->nbasis) {
      set_error("batch_add_system: row stride %d below the species' %d functions", ld[k], species[k]->nbasis);
      return -1;
    }
    LowdinGB300_Batch::Spec x{species[k], charges[k], factors[k], two_body[k], dP[k], dG ? dG[k] : nullptr,
                              dJ[k], sys, ld ? ld[k] : species[k]->nbasis};
    b->sp.push_back(x);
  }
  b->finalized = false;
  return first;
}

int LowdinGB300_batch_finalize(LowdinGB300_Batch *b, void *stream) {
  if (!b) return -1;
  return b->finalize((cudaStream_t)stream) ? 0 : -1;
}

int LowdinGB300_batch_fock(LowdinGB300_Batch *b, int precision, double split, void *stream) {
  if (!b) return -1;
  return b->fock(precision, split, (cudaStream_t)stream) ? 0 : -1;
}

int LowdinGB300_batch_use_graph(LowdinGB300_Batch *b, int on) {
  if (!b) return -1;
  b->use_graph = on != 0;
  if (!b->use_graph) b->drop_graphs();
  return 0;
}

int LowdinGB300_batch_quartets(LowdinGB300_Batch *b, long long *out, void *stream) {
  if (!b || !b->finalized) return -1;
  unsigned long long c[kNQC];
  if (cudaMemcpyAsync(c, b->cnt.p, sizeof(c), cudaMemcpyDeviceToHost, (cudaStream_t)stream) != cudaSuccess ||
      cudaStreamSynchronize((cudaStream_t)stream) != cudaSuccess) {
    set_error("batch_quartets: copy failed");
    return -1;
  }
  for (int k = 0; k < kNQC; ++k) out[k] = (long long)c[k];
  return kNQC;
}

int LowdinGB300_batch_coupling_quartets(LowdinGB300_Batch *b, long long *out, void *stream) {
  if (!b || !b->finalized) return -1;
  unsigned long long c[kNQC];
  if (cudaMemcpyAsync(c, b->cnt.p + kNQC, sizeof(c), cudaMemcpyDeviceToHost, (cudaStream_t)stream) !=
          cudaSuccess ||
      cudaStreamSynchronize((cudaStream_t)stream) != cudaSuccess) {
    set_error("batch_coupling_quartets: copy failed");
    return -1;
  }
  for (int k = 0; k < kNQC; ++k) out[k] = (long long)c[k];
  return kNQC;
}

}  // extern "C"

// ====================================================== allocation-free build
// LowdinGB300_twobody_device_noalloc: the device two-particle build for
// callers that must not allocate device memory once they are running -- a host
// program that owns every device byte through its own pool, a serving loop that
// forbids allocations after warm-up, or code queuing work into a captured
// stream.  Its work buffers (scaled densities, shell-block norms, accumulators,
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
      t.nbx = task_nbx(t.nket);
      t.blk0 = b;
      b += t.nbx * task_nby(t.nbra);
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

// ========================================================= MP2 transform
// LowdinGB300_mp2_direct: closed-shell MP2 of one electron species with the
// four-index transform on the device.  Same integral set as the reference's
// DIRECT transform (TransformIntegralsC.f90:472-665 over
// LibintInterface_compute_2body_directIT, Libint2Iface.cpp:620-921):
// significant shell pairs only, quartets dropped by the density screening,
// raw |v| <= 1e-10 dropped; MO integrals with |(ia|jb)| <= 1e-10 read as zero
// in the energy (only larger ones are stored, :634).  The first quarter is not
// recomputed per occupied orbital: the integrals of every bra pair against a
// batch of ket pairs are written once into X[mu][col][nu] and contracted by
// GEMMs:
//   T1[i][col][nu] = sum_mu Co[mu][i] X[mu][col][nu]          (o x N^2 P)
//   Y[i][col][a]   = sum_nu T1[i][col][nu] Cv[nu][a]          (o v N P)
// then for every i: Z[lam][sig][a] (unpacked Y[i]),
//   W[j][sig][a]   = sum_lam Co[lam][j] Z[lam][sig][a]        (o^2 v N^2)
//   M[j][b][a]     = sum_sig Cv[sig][b] W[j][sig][a] = (ia|jb) (o^2 v^2 N)
// and the pair energies.  A column is one Cartesian component pair (c, d) of
// a significant ket shell pair (all nc^2 of a diagonal pair).
namespace {

std::mutex g_blas_mu;
std::vector<std::pair<int, cublasHandle_t>> g_blas;

bool blas_handle(cublasHandle_t *out) {
  int dev = 0;
  CK(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_blas_mu);
  for (auto &e : g_blas)
    if (e.first == dev) {
      *out = e.second;
      return true;
    }
  cublasHandle_t h = nullptr;
  if (cublasCreate(&h) != CUBLAS_STATUS_SUCCESS) {
    set_error("cublasCreate failed");
    return false;
  }
  g_blas.push_back({dev, h});
  *out = h;
  return true;
}

// row-major C_b = op(A_b) op(B_b), b < batch, with element strides between batches
bool dgemm_rm(cublasHandle_t h, bool ta, bool tb, int m, int n, int k, const double *A, int lda, long long sA,
              const double *B, int ldb, long long sB, double *C, int ldc, long long sC, int batch) {
  const double one = 1.0, zero = 0.0;
  const cublasStatus_t st =
      cublasDgemmStridedBatched(h, tb ? CUBLAS_OP_T : CUBLAS_OP_N, ta ? CUBLAS_OP_T : CUBLAS_OP_N, n, m, k, &one, B,
                                ldb, sB, A, lda, sA, &zero, C, ldc, sC, batch);
  if (st != CUBLAS_STATUS_SUCCESS) {
    set_error("cublasDgemmStridedBatched failed (status %d, m=%d n=%d k=%d batch=%d)", (int)st, m, n, k, batch);
    return false;
  }
  return true;
}

struct MP2Stats {
  long long ncols = 0;
  int batches = 0;
};
MP2Stats g_mp2_last;

// Columns of the significant ket pairs (colbase per pair record; colpair =
// lam | sig << 16 | offdiag << 31) and batches of whole ket pairs with at most
// colB columns (bfirst: first pair of each batch, then npairs).
struct MP2Columns {
  std::vector<int> colbase;
  std::vector<unsigned> colpair;
  std::vector<int> bfirst;
  long long ncols = 0;
};

void mp2_columns(const PairList &P, long long colB, MP2Columns &mc) {
  const int npairs = (int)P.h.size();
  mc.colbase.assign(npairs, 0);
  mc.colpair.clear();
  for (int k = 0; k < npairs; ++k) {
    const PairRec &r = P.h[k];
    mc.colbase[k] = (int)mc.colpair.size();
    const int nc = ncart(r.la), nd = ncart(r.lb);
    for (int c = 0; c < nc; ++c)
      for (int d = 0; d < nd; ++d)
        mc.colpair.push_back((unsigned)(r.fa + c) | (unsigned)(r.fb + d) << 16 | (r.sa != r.sb ? 1u << 31 : 0u));
  }
  mc.ncols = (long long)mc.colpair.size();
  mc.bfirst.clear();
  for (int k = 0; k < npairs;) {
    mc.bfirst.push_back(k);
    const int c0 = mc.colbase[k];
    while (k < npairs && mc.colbase[k] - c0 + ncart(P.h[k].la) * ncart(P.h[k].lb) <= colB) ++k;
  }
  mc.bfirst.push_back(npairs);
}

// integrals of every bra pair of PA against the ket pairs [k0, k1) of PB
bool mp2_batch_ints(const PairList &PA, const PairList &PB, MXParams q, int k0, int k1, cudaStream_t s) {
  for (int ck = 0; ck < kNumPairClasses; ++ck) {
    const int ka = std::max(k0, PB.start[ck]), kb = std::min(k1, PB.start[ck + 1]);
    if (ka >= kb) continue;
    for (int cb = 0; cb < kNumPairClasses; ++cb)
      for (int b0 = PA.start[cb]; b0 < PA.start[cb + 1]; b0 += 65535 * kWarpsPerBlock) {  // grid y limit
        q.bra0 = b0;
        q.nbra = std::min(PA.start[cb + 1] - b0, 65535 * kWarpsPerBlock);
        q.ket0 = ka;
        q.nket = kb - ka;
        CK(launch_mp2x(cb, ck, q, s));
      }
  }
  return true;
}

// Writer of the reference's transformed-integral file `<species>moint.dat`
// (TransformIntegralsC.f90:531-654, read by ReadTransformedIntegrals.f90:225-233):
// a Fortran sequential unformatted file whose records each hold four int32
// index arrays p, q, r, s and one FP64 value array, all of the stack size
// (30000 by default), framed by the record length in bytes (int32) before and
// after, as gfortran writes them.  Entries fill a stack in the order they
// come; a full stack is written as one record and cleared; the last record
// marks the end with p = -1 after its last entry (zeros beyond).
struct MointWriter {
  FILE *f = nullptr;
  int stack = 0, m = 0;
  long long written = 0;
  std::vector<int32_t> pp, qq, rr, ss;
  std::vector<double> val;
  bool open(const char *path, int stack_size) {
    stack = stack_size;
    pp.assign(stack, 0); qq.assign(stack, 0); rr.assign(stack, 0); ss.assign(stack, 0);
    val.assign(stack, 0.0);
    f = std::fopen(path, "wb");
    if (!f) {
      set_error("moint: cannot open %s for writing", path);
      return false;
    }
    return true;
  }
  bool record() {
    const int32_t len = (int32_t)((size_t)stack * (4 * sizeof(int32_t) + sizeof(double)));
    bool ok = std::fwrite(&len, 4, 1, f) == 1;
    for (auto *a : {&pp, &qq, &rr, &ss}) ok = ok && std::fwrite(a->data(), 4, stack, f) == (size_t)stack;
    ok = ok && std::fwrite(val.data(), 8, stack, f) == (size_t)stack && std::fwrite(&len, 4, 1, f) == 1;
    if (!ok) set_error("moint: write failed");
    for (auto *a : {&pp, &qq, &rr, &ss}) std::fill(a->begin(), a->end(), 0);
    std::fill(val.begin(), val.end(), 0.0);
    return ok;
  }
  bool put(int p, int q, int r, int s_, double v) {
    pp[m] = p; qq[m] = q; rr[m] = r; ss[m] = s_; val[m] = v;
    ++written;
    if (++m == stack) {
      m = 0;
      return record();
    }
    return true;
  }
  bool finish() {
    pp[m] = -1;
    const bool ok = record();
    std::fclose(f);
    f = nullptr;
    return ok;
  }
  ~MointWriter() {
    if (f) std::fclose(f);
  }
};

// One MP2 term: intra-species (A == B, closed shell: (ia|jb)[2(ia|jb) -
// (ib|ja)]/D) or inter-species (A != B: factor (ia|jb)^2 / D, factor = (q_A
// q_B)^2 lambda_A lambda_B).  The bra index pairs (mu nu) belong to A, the ket
// columns (lam sig) to B.
struct MP2Setup {
  LibintInterface *A, *B;
  const PairList *PA, *PB;
  bool coupling;
  double factor;
  int nA, nB, oA, vA, oB, vB, noccA, nfA, noccB, nfB;
  const double *dCA, *dCB, *epsA, *epsB;
  MXParams q;      // common integral parameters
  MointWriter *moint = nullptr;   // FP64 intra-species path: also write every (ia|jb) to the file
};

// (ia|jb) of occupied i (M[j][b][a], device) into the file in the reference's
// loop order: a, then j >= i, then b (b >= a when j == i), |v| > 1e-10
// (TransformIntegralsC.f90:570-640 with the MP2 bounds of :1489-1501)
bool moint_block(const MP2Setup &S, int i, const double *dM, std::vector<double> &h, cudaStream_t s) {
  const int oB = S.oB, vB = S.vB, vA = S.vA;
  h.resize((size_t)oB * vB * vA);
  CK(cudaMemcpyAsync(h.data(), dM, h.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  const int p = S.nfA + i + 1;
  for (int a = 0; a < vA; ++a)
    for (int j = i; j < oB; ++j)
      for (int b = (j == i ? a : 0); b < vB; ++b) {
        const double v = h[((size_t)j * vB + b) * vA + a];
        if (std::fabs(v) > 1e-10 && !S.moint->put(p, S.noccA + a + 1, S.nfB + j + 1, S.noccB + b + 1, v))
          return false;
      }
  return true;
}

bool mp2_need(size_t bytes) {
  size_t freeb = 0, totb = 0;
  CK(cudaMemGetInfo(&freeb, &totb));
  if (bytes > freeb) {
    set_error("mp2: needs %.1f GB of device memory, %.1f GB free", bytes / 1e9, freeb / 1e9);
    return false;
  }
  return true;
}

long long mp2_max_batch(const MP2Columns &mc, const PairList &P) {
  long long colB = 0;
  for (size_t b = 0; b + 1 < mc.bfirst.size(); ++b) {
    const int k1 = mc.bfirst[b + 1];
    colB = std::max<long long>(colB, (k1 < (int)P.h.size() ? mc.colbase[k1] : mc.ncols) - mc.colbase[mc.bfirst[b]]);
  }
  return colB;
}

// FP64 back end: cuBLAS DGEMM for the four quarters
bool mp2_fp64(MP2Setup &S, size_t budget, double *e2out, cudaStream_t s) {
  const int nA = S.nA, nB = S.nB, oA = S.oA, vA = S.vA, oB = S.oB, vB = S.vB;
  cublasHandle_t blas;
  if (!blas_handle(&blas)) return false;
  if (cublasSetStream(blas, s) != CUBLAS_STATUS_SUCCESS) {
    set_error("cublasSetStream failed");
    return false;
  }
  const PairList &PB = *S.PB;
  const size_t per_col = (size_t)nA * nA * sizeof(double) + (size_t)oA * nA * sizeof(double);
  MP2Columns mc;
  mp2_columns(PB, std::max<long long>(36, (long long)(budget / per_col)), mc);
  const long long ncols = mc.ncols;
  const long long colB = mp2_max_batch(mc, PB);
  if (!mp2_need((size_t)oA * ncols * vA * 8 + (size_t)nB * nB * vA * 8 + (size_t)colB * per_col +
                (size_t)oB * nB * vA * 8 + (size_t)oB * vB * vA * 8))
    return false;
  DevBuf<double> CoA, CvA, CoB, CvB, EoB, EvA, EvB, Y, X, T1, Z, W, M, e2;
  DevBuf<int> dcolbase;
  DevBuf<unsigned> dcolpair;
  if (!CoA.ensure((size_t)nA * oA) || !CvA.ensure((size_t)nA * vA) || !CoB.ensure((size_t)nB * oB) ||
      !CvB.ensure((size_t)nB * vB) || !EoB.ensure(oB) || !EvA.ensure(vA) || !EvB.ensure(vB) ||
      !Y.ensure((size_t)oA * ncols * vA) || !X.ensure((size_t)nA * colB * nA) || !T1.ensure((size_t)oA * colB * nA) ||
      !Z.ensure((size_t)nB * nB * vA) || !W.ensure((size_t)oB * nB * vA) || !M.ensure((size_t)oB * vB * vA) ||
      !e2.ensure(1) || !dcolbase.ensure(PB.h.size()) || !dcolpair.ensure(ncols))
    return false;
  CK(cudaMemcpyAsync(dcolbase.p, mc.colbase.data(), PB.h.size() * sizeof(int), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(dcolpair.p, mc.colpair.data(), ncols * sizeof(unsigned), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(EoB.p, S.epsB + S.nfB, oB * sizeof(double), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(EvA.p, S.epsA + S.noccA, vA * sizeof(double), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(EvB.p, S.epsB + S.noccB, vB * sizeof(double), cudaMemcpyHostToDevice, s));
  CK(cudaMemsetAsync(e2.p, 0, sizeof(double), s));
  CK(launch_mp2_coeffs(S.dCA, S.A->d_norma, nA, S.nfA, S.noccA, CoA.p, CvA.p, nullptr, nullptr, s));
  CK(launch_mp2_coeffs(S.dCB, S.B->d_norma, nB, S.nfB, S.noccB, CoB.p, CvB.p, nullptr, nullptr, s));
  MXParams q = S.q;
  q.colbase = dcolbase.p;
  q.X = X.p;
  std::vector<double> hM;
  const int nbatch = (int)mc.bfirst.size() - 1;
  for (int bt = 0; bt < nbatch; ++bt) {
    const int k0 = mc.bfirst[bt], k1 = mc.bfirst[bt + 1];
    const int c0 = mc.colbase[k0];
    const int nb = (int)((k1 < (int)PB.h.size() ? mc.colbase[k1] : ncols) - c0);
    q.col_first = c0;
    q.ncol = nb;
    CK(cudaMemsetAsync(X.p, 0, (size_t)nA * nb * nA * sizeof(double), s));
    if (!mp2_batch_ints(*S.PA, PB, q, k0, k1, s)) return false;
    // T1 (oA x nb*nA) = CoA^T X ; Y[i][c0 + col][a] = T1[i] (nb x nA) CvA
    if (!dgemm_rm(blas, true, false, oA, nb * nA, nA, CoA.p, oA, 0, X.p, nb * nA, 0, T1.p, nb * nA, 0, 1))
      return false;
    if (!dgemm_rm(blas, false, false, nb, vA, nA, T1.p, nA, (long long)nb * nA, CvA.p, vA, 0, Y.p + (size_t)c0 * vA,
                  vA, ncols * vA, oA))
      return false;
  }
  CK(cudaMemsetAsync(Z.p, 0, (size_t)nB * nB * vA * sizeof(double), s));
  for (int i = 0; i < oA; ++i) {
    CK(launch_mp2_unpack<double>(Y.p + (size_t)i * ncols * vA, dcolpair.p, ncols, nB, vA, Z.p, s));
    // W (oB x nB*vA) = CoB^T Z ; M_j (vB x vA) = CvB^T W_j
    if (!dgemm_rm(blas, true, false, oB, nB * vA, nB, CoB.p, oB, 0, Z.p, nB * vA, 0, W.p, nB * vA, 0, 1))
      return false;
    if (!dgemm_rm(blas, true, false, vB, vA, nB, CvB.p, vB, 0, W.p, vA, (long long)nB * vA, M.p, vA,
                  (long long)vB * vA, oB))
      return false;
    const double ei = S.epsA[S.nfA + i];
    if (S.coupling)
      CK(launch_mp2_energy_coupling<double>(M.p, oB, vB, vA, ei, EoB.p, EvA.p, EvB.p, 1e-10, S.factor, e2.p, s));
    else
      CK(launch_mp2_energy<double>(M.p, oB, vB, ei, EoB.p, EvB.p, 1e-10, e2.p, s));
    if (S.moint && !moint_block(S, i, M.p, hM, s)) return false;
  }
  double e = 0;
  CK(cudaMemcpyAsync(&e, e2.p, sizeof(double), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  *e2out = e;
  g_mp2_last.ncols = ncols;
  g_mp2_last.batches = nbatch;
  return true;  // the buffers are freed on return
}

// Split-BF16 back end: the same quarters on the tensor cores (np BF16 pieces
// per operand, FP32 accumulation), operands written K-major by their producers:
//   Xt[col][nu][mu]   (integral kernel)          GEMM1: T1[i][col nu] = CoT_A Xt^T
//   Y'[a][i][col]     (GEMM2 = CvT_A T1^T, FP32) per i: Zt[a][sig][lam] (gather)
//   GEMM3: Wt[j][a sig] = CoT_B Zt^T             GEMM4: M_j[b][a] = CvT_B Wt_j^T
struct SplitBuf {
  DevBuf<__nv_bfloat16> p[kMaxPieces];
  bool ensure(int np, size_t n) {
    for (int q = 0; q < np; ++q)
      if (!p[q].ensure(n)) return false;
    return true;
  }
  Bf16Split in() const { return Bf16Split{{p[0].p, p[1].p, p[2].p}}; }
  void out(GemmOut &o) const {
    for (int q = 0; q < kMaxPieces; ++q) o.Cp[q] = p[q].p;
  }
  __nv_bfloat16 *const *ptrs(__nv_bfloat16 *(&tmp)[kMaxPieces]) const {
    for (int q = 0; q < kMaxPieces; ++q) tmp[q] = p[q].p;
    return tmp;
  }
};

bool mp2_split(MP2Setup &S, int np, size_t budget, double *e2out, cudaStream_t s) {
  using bf = __nv_bfloat16;
  const int nA = S.nA, nB = S.nB, oA = S.oA, vA = S.vA, oB = S.oB, vB = S.vB;
  const int KA = (nA + 63) / 64 * 64, KB = (nB + 63) / 64 * 64;
  const PairList &PB = *S.PB;
  const size_t per_col = (size_t)KA * KA * 2 * np + (size_t)oA * KA * 2 * np;   // Xt and T1 pieces
  MP2Columns mc;
  mp2_columns(PB, std::max<long long>(36, (long long)(budget / per_col)), mc);
  const long long ncols = mc.ncols;
  const long long colB = mp2_max_batch(mc, PB);
  // gather lists over B's functions: row sig -> (lam, col) with Z[lam][sig] = Y[col]
  std::vector<int> rowptr(nB + 1, 0);
  for (long long c = 0; c < ncols; ++c) {
    const unsigned cp = mc.colpair[c];
    rowptr[((cp >> 16) & 0x7fff) + 1]++;
    if (cp >> 31) rowptr[(cp & 0xffff) + 1]++;
  }
  for (int r = 0; r < nB; ++r) rowptr[r + 1] += rowptr[r];
  std::vector<int2> ent(rowptr[nB]);
  {
    std::vector<int> fill(rowptr.begin(), rowptr.end() - 1);
    for (long long c = 0; c < ncols; ++c) {
      const unsigned cp = mc.colpair[c];
      const int lam = cp & 0xffff, sig = (cp >> 16) & 0x7fff;
      ent[fill[sig]++] = make_int2(lam | sig << 16, (int)c);
      if (cp >> 31) ent[fill[lam]++] = make_int2(sig | lam << 16, (int)c);
    }
  }
  const size_t need = (size_t)vA * oA * ncols * 4 + (size_t)colB * per_col +
                      ((size_t)vA * KB * KB + (size_t)oB * vA * KB + (size_t)(oA + vA) * KA + (size_t)(oB + vB) * KB) *
                          2 * np +
                      (size_t)oB * vB * vA * 4 + ent.size() * 8;
  if (!mp2_need(need)) return false;
  SplitBuf CoTA, CvTA, CoTB, CvTB, X, T1, Z, W;
  DevBuf<float> Y, M;
  DevBuf<double> EoB, EvA, EvB, e2;
  DevBuf<int> dcolbase, drowptr, err;
  DevBuf<int2> dent;
  const size_t xsz = (size_t)colB * KA * KA, t1sz = (size_t)oA * colB * KA, zsz = (size_t)vA * KB * KB,
               wsz = (size_t)oB * vA * KB;
  if (!CoTA.ensure(np, (size_t)oA * KA) || !CvTA.ensure(np, (size_t)vA * KA) || !CoTB.ensure(np, (size_t)oB * KB) ||
      !CvTB.ensure(np, (size_t)vB * KB) || !X.ensure(np, xsz) || !T1.ensure(np, t1sz) || !Z.ensure(np, zsz) ||
      !W.ensure(np, wsz) || !Y.ensure((size_t)vA * oA * ncols) || !M.ensure((size_t)oB * vB * vA) ||
      !EoB.ensure(oB) || !EvA.ensure(vA) || !EvB.ensure(vB) || !e2.ensure(1) || !dcolbase.ensure(PB.h.size()) ||
      !drowptr.ensure(nB + 1) || !err.ensure(1) || !dent.ensure(std::max<size_t>(1, ent.size())))
    return false;
  CK(cudaMemcpyAsync(dcolbase.p, mc.colbase.data(), PB.h.size() * sizeof(int), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(drowptr.p, rowptr.data(), (nB + 1) * sizeof(int), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(dent.p, ent.data(), ent.size() * sizeof(int2), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(EoB.p, S.epsB + S.nfB, oB * sizeof(double), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(EvA.p, S.epsA + S.noccA, vA * sizeof(double), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(EvB.p, S.epsB + S.noccB, vB * sizeof(double), cudaMemcpyHostToDevice, s));
  CK(cudaMemsetAsync(e2.p, 0, sizeof(double), s));
  CK(cudaMemsetAsync(err.p, 0, sizeof(int), s));
  for (const SplitBuf *b : {&CoTA, &CvTA, &CoTB, &CvTB, &Z})
    for (int k = 0; k < np; ++k) CK(cudaMemsetAsync(b->p[k].p, 0, b->p[k].n * sizeof(bf), s));
  bf *t0[kMaxPieces], *t1[kMaxPieces];
  CK(launch_mp2_coeffs_bf16(S.dCA, S.A->d_norma, nA, S.nfA, S.noccA, KA, np, CoTA.ptrs(t0), CvTA.ptrs(t1), s));
  CK(launch_mp2_coeffs_bf16(S.dCB, S.B->d_norma, nB, S.nfB, S.noccB, KB, np, CoTB.ptrs(t0), CvTB.ptrs(t1), s));
  // np 3: every quarter on the precise engine (the tensor cores round their
  // FP32 running sums toward zero; over a long contraction that bias, not
  // the BF16 pieces, dominated the energy error); np 2: the split engine
  auto gemm = [&](const Bf16Split &Am, long long ar, const Bf16Split &Bm, long long br, int Kp, int Mr, int Nc,
                  int batch, int abr, int bbr, const GemmOut &out) {
    return np == 3 ? launch_gemm_precise(Am, ar, Bm, br, Kp, Mr, Nc, batch, abr, bbr, out, err.p, s)
                   : launch_gemm_split(Am, ar, Bm, br, Kp, Mr, Nc, batch, abr, bbr, np, out, err.p, s);
  };
  MXParams q = S.q;
  q.colbase = dcolbase.p;
  q.X = nullptr;
  for (int k = 0; k < kMaxPieces; ++k) q.Xp[k] = X.p[k].p;
  q.np = np;
  q.Kp = KA;
  const int nbatch = (int)mc.bfirst.size() - 1;
  for (int bt = 0; bt < nbatch; ++bt) {
    const int k0 = mc.bfirst[bt], k1 = mc.bfirst[bt + 1];
    const int c0 = mc.colbase[k0];
    const int nb = (int)((k1 < (int)PB.h.size() ? mc.colbase[k1] : ncols) - c0);
    q.col_first = c0;
    q.ncol = nb;
    for (int k = 0; k < np; ++k) CK(cudaMemsetAsync(X.p[k].p, 0, (size_t)nb * KA * KA * sizeof(bf), s));
    if (!mp2_batch_ints(*S.PA, PB, q, k0, k1, s)) return false;
    GemmOut o1{};
    T1.out(o1);
    o1.ldc = (long long)nb * KA;
    CK(gemm(CoTA.in(), oA, X.in(), (long long)nb * KA, KA, oA, nb * KA, 1, 0, 0, o1));
    GemmOut o2{};
    o2.C = Y.p;
    o2.ldc = (long long)oA * ncols;
    o2.grp_cols = nb;
    o2.gcol_stride = ncols;
    o2.col0 = c0;
    CK(gemm(CvTA.in(), vA, T1.in(), (long long)oA * nb, KA, vA, oA * nb, 1, 0, 0, o2));
  }
  bf *tz[kMaxPieces];
  for (int i = 0; i < oA; ++i) {
    CK(launch_mp2_unpack_csr(Y.p + (size_t)i * ncols, (long long)oA * ncols, drowptr.p, dent.p, nB, KB, vA, np,
                             Z.ptrs(tz), s));
    GemmOut o3{};
    W.out(o3);
    o3.ldc = (long long)vA * KB;
    CK(gemm(CoTB.in(), oB, Z.in(), (long long)vA * KB, KB, oB, vA * KB, 1, 0, 0, o3));
    GemmOut o4{};
    o4.C = M.p;
    o4.ldc = vA;
    o4.c_batch = (long long)vB * vA;
    CK(gemm(CvTB.in(), vB, W.in(), (long long)oB * vA, KB, vB, vA, oB, 0, vA, o4));
    const double ei = S.epsA[S.nfA + i];
    if (S.coupling)
      CK(launch_mp2_energy_coupling<float>(M.p, oB, vB, vA, ei, EoB.p, EvA.p, EvB.p, 1e-10, S.factor, e2.p, s));
    else
      CK(launch_mp2_energy<float>(M.p, oB, vB, ei, EoB.p, EvB.p, 1e-10, e2.p, s));
  }
  double e = 0;
  int herr = 0;
  CK(cudaMemcpyAsync(&e, e2.p, sizeof(double), cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (herr) {
    set_error("mp2: a tensor-core GEMM pipeline wait ran out (code %d)", herr);
    return false;
  }
  *e2out = e;
  g_mp2_last.ncols = ncols;
  g_mp2_last.batches = nbatch;
  return true;
}

bool mp2_run(MP2Setup &S, int precision, size_t budget, double *e2out, cudaStream_t s) {
  if (precision < 0 || precision > 2) {
    set_error("mp2: precision %d is not available (0: FP64, 1 / 2: split BF16 in 2 / 3 pieces)", precision);
    return false;
  }
  if (S.nA >= 32768 || S.nB >= 32768) {
    set_error("mp2: more than 32767 basis functions exceed the column encoding");
    return false;
  }
  return precision == 0 ? mp2_fp64(S, budget, e2out, s) : mp2_split(S, precision + 1, budget, e2out, s);
}

bool mp2_direct(LibintInterface *L, const double *dD, const double *dC, const double *eps, int n_occ, int n_frozen,
                int precision, size_t x_budget_bytes, double *e2out, cudaStream_t s, MointWriter *moint = nullptr) {
  if (!L->is_electron) {
    set_error("mp2_direct: closed-shell MP2 is defined here for an electron species");
    return false;
  }
  if (!L->ensure_sig()) return false;
  const int n = L->nbasis, nsh = L->nshell();
  if (!(0 <= n_frozen && n_frozen < n_occ && n_occ < n)) {
    set_error("mp2_direct: need 0 <= n_frozen < n_occ < nbasis (got %d, %d, %d)", n_frozen, n_occ, n);
    return false;
  }
  MP2Setup S{};
  S.A = S.B = L;
  S.PA = S.PB = &L->sig;
  S.coupling = false;
  S.factor = 1.0;
  S.nA = S.nB = n;
  S.noccA = S.noccB = n_occ;
  S.nfA = S.nfB = n_frozen;
  S.oA = S.oB = n_occ - n_frozen;
  S.vA = S.vB = n - n_occ;
  S.dCA = S.dCB = dC;
  S.epsA = S.epsB = eps;
  // shell-block norms of D for the screening
  if (!L->dDs.ensure((size_t)n * n) || !L->dDn.ensure((size_t)nsh * nsh)) return false;
  CK(launch_prepare_density(dD, L->d_norma, L->d_shell_of, n, nsh, L->dDs.p, nullptr, L->dDn.p, nullptr, s));
  MXParams &q = S.q;
  q.pairs = q.kpairs = L->sig.d;
  q.prims = q.kprims = L->sig.dp;
  q.Dn = L->dDn.p;
  q.nsh = nsh;
  q.screen = 1;
  q.eps = DBL_EPSILON;
  q.cut = 1e-10;
  q.n = n;
  q.boys = L->boys;
  S.moint = moint;
  return mp2_run(S, precision, x_budget_bytes, e2out, s);
}

bool mp2_coupling(LibintInterface *A, LibintInterface *B, const double *dCA, const double *dCB, const double *epsA,
                  const double *epsB, int noccA, int nfA, int noccB, int nfB, double factor, int precision,
                  size_t budget, double *e2out, cudaStream_t s) {
  if (A == B) {
    set_error("mp2_coupling: the two handles must be different species");
    return false;
  }
  if (!A->ensure_all() || !B->ensure_all()) return false;
  const int nA = A->nbasis, nB = B->nbasis;
  if (!(0 <= nfA && nfA < noccA && noccA < nA && 0 <= nfB && nfB < noccB && noccB < nB)) {
    set_error("mp2_coupling: need 0 <= n_frozen < n_occ < nbasis for both species");
    return false;
  }
  MP2Setup S{};
  S.A = A;
  S.B = B;
  S.PA = &A->all;
  S.PB = &B->all;
  S.coupling = true;
  S.factor = factor;
  S.nA = nA;
  S.nB = nB;
  S.noccA = noccA;
  S.nfA = nfA;
  S.noccB = noccB;
  S.nfB = nfB;
  S.oA = noccA - nfA;
  S.vA = nA - noccA;
  S.oB = noccB - nfB;
  S.vB = nB - noccB;
  S.dCA = dCA;
  S.dCB = dCB;
  S.epsA = epsA;
  S.epsB = epsB;
  // coupling integrals: no density screening (Libint2Iface.cpp:1296-1622),
  // quartets whose Schwarz bound is below the raw cut contribute nothing
  MXParams &q = S.q;
  q.pairs = A->all.d;
  q.prims = A->all.dp;
  q.kpairs = B->all.d;
  q.kprims = B->all.dp;
  q.screen = 0;
  q.eps = 0.0;
  q.cut = 1e-10;
  q.n = nA;
  q.boys = A->boys;
  return mp2_run(S, precision, budget, e2out, s);
}

}  // namespace

extern "C" {

int LowdinGB300_mp2_direct(LibintInterface *lint, const double *dD, const double *dC, const double *eps, int n_occ,
                           int n_frozen, int precision, double x_budget_gb, double *e2, void *stream) {
  if (!check_handle(lint, __func__)) return -1;
  if (!dD || !dC || !eps || !e2) {
    set_error("%s: null argument", __func__);
    return -1;
  }
  const size_t budget = x_budget_gb > 0 ? (size_t)(x_budget_gb * 1e9) : (size_t)8e9;
  return mp2_direct(lint, dD, dC, eps, n_occ, n_frozen, precision, budget, e2, (cudaStream_t)stream) ? 0 : -1;
}

int LowdinGB300_mp2_coupling(LibintInterface *a, LibintInterface *b, const double *dCa, const double *dCb,
                             const double *eps_a, const double *eps_b, int n_occ_a, int n_frozen_a, int n_occ_b,
                             int n_frozen_b, double factor, int precision, double x_budget_gb, double *e2,
                             void *stream) {
  if (!check_handle(a, __func__) || !check_handle(b, __func__)) return -1;
  if (!dCa || !dCb || !eps_a || !eps_b || !e2) {
    set_error("%s: null argument", __func__);
    return -1;
  }
  const size_t budget = x_budget_gb > 0 ? (size_t)(x_budget_gb * 1e9) : (size_t)8e9;
  return mp2_coupling(a, b, dCa, dCb, eps_a, eps_b, n_occ_a, n_frozen_a, n_occ_b, n_frozen_b, factor, precision,
                      budget, e2, (cudaStream_t)stream)
             ? 0
             : -1;
}

long long LowdinGB300_mp2_last_columns(void) { return g_mp2_last.ncols; }

int LowdinGB300_mp2_moint(LibintInterface *lint, const double *dD, const double *dC, const double *eps, int n_occ,
                          int n_frozen, const char *path, int stack_size, double x_budget_gb, double *e2,
                          long long *n_written, void *stream) {
  if (!check_handle(lint, __func__)) return -1;
  if (!dD || !dC || !eps || !e2 || !path || stack_size < 1) {
    set_error("%s: invalid argument", __func__);
    return -1;
  }
  MointWriter w;
  if (!w.open(path, stack_size)) return -1;
  const size_t budget = x_budget_gb > 0 ? (size_t)(x_budget_gb * 1e9) : (size_t)8e9;
  if (!mp2_direct(lint, dD, dC, eps, n_occ, n_frozen, 0, budget, e2, (cudaStream_t)stream, &w)) return -1;
  if (!w.finish()) return -1;
  if (n_written) *n_written = w.written;
  return 0;
}

int LowdinGB300_moint_write(const char *path, int stack_size, const int *p, const int *q, const int *r,
                            const int *s, const double *v, long long count) {
  if (!path || stack_size < 1 || count < 0 || (count > 0 && (!p || !q || !r || !s || !v))) {
    set_error("%s: invalid argument", __func__);
    return -1;
  }
  MointWriter w;
  if (!w.open(path, stack_size)) return -1;
  for (long long k = 0; k < count; ++k)
    if (!w.put(p[k], q[k], r[k], s[k], v[k])) return -1;
  return w.finish() ? 0 : -1;
}

}  // extern "C"

// ============================================== split-BF16 tensor-core GEMM
namespace {
int gemm_entry(const char *fn, const float *dA, const float *dB, float *dC, int M, int N, int K, int pieces,
               bool precise, void *stream) {
  if (!dA || !dB || !dC || M <= 0 || N <= 0 || K <= 0 || pieces < 2 || pieces > kMaxPieces) {
    set_error("%s: invalid arguments", fn);
    return -1;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const int Kp = (K + 63) / 64 * 64;
  SplitBuf A, B;
  DevBuf<int> err;
  if (!A.ensure(pieces, (size_t)M * Kp) || !B.ensure(pieces, (size_t)N * Kp) || !err.ensure(1)) return -1;
  auto fail = [&](const char *what, cudaError_t e) {
    set_error("%s: %s (%s)", fn, what, cudaGetErrorString(e));
    return -1;
  };
  cudaError_t e;
  for (int q = 0; q < pieces; ++q)
    if ((e = cudaMemsetAsync(A.p[q].p, 0, (size_t)M * Kp * 2, s)) != cudaSuccess ||
        (e = cudaMemsetAsync(B.p[q].p, 0, (size_t)N * Kp * 2, s)) != cudaSuccess)
      return fail("clear", e);
  if ((e = cudaMemsetAsync(err.p, 0, sizeof(int), s)) != cudaSuccess) return fail("clear", e);
  __nv_bfloat16 *ta[kMaxPieces], *tb[kMaxPieces];
  if ((e = launch_split_bf16<float>(dA, M, K, K, pieces, A.ptrs(ta), Kp, s)) != cudaSuccess ||
      (e = launch_split_bf16<float>(dB, N, K, K, pieces, B.ptrs(tb), Kp, s)) != cudaSuccess)
    return fail("split", e);
  GemmOut out{};
  out.C = dC;
  out.ldc = N;
  e = precise ? launch_gemm_precise(A.in(), M, B.in(), N, Kp, M, N, 1, 0, 0, out, err.p, s)
              : launch_gemm_split(A.in(), M, B.in(), N, Kp, M, N, 1, 0, 0, pieces, out, err.p, s);
  if (e != cudaSuccess) return fail("gemm launch", e);
  int herr = 0;
  if ((e = cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
      (e = cudaStreamSynchronize(s)) != cudaSuccess)
    return fail("gemm", e);
  if (herr) {
    set_error("%s: a pipeline wait ran out (code %d)", fn, herr);
    return -1;
  }
  return 0;
}
}  // namespace

extern "C" {


int LowdinGB300_gemm_bf16_split(const float *dA, const float *dB, float *dC, int M, int N, int K, int pieces,
                                void *stream) {
  return gemm_entry(__func__, dA, dB, dC, M, N, K, pieces, false, stream);
}

int LowdinGB300_gemm_bf16_precise(const float *dA, const float *dB, float *dC, int M, int N, int K, void *stream) {
  return gemm_entry(__func__, dA, dB, dC, M, N, K, 3, true, stream);
}

double LowdinGB300_gemm_bench(int M, int N, int K, int mode, int reps, void *stream) {
  const int pieces = mode == 2 ? 2 : 3;
  if (M <= 0 || N <= 0 || K <= 0 || reps <= 0 || (mode != 2 && mode != 3 && mode != 8)) {
    set_error("%s: invalid arguments (mode 2, 3 or 8)", __func__);
    return -1.0;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const int Kp = (K + 63) / 64 * 64;
  SplitBuf A, B;
  DevBuf<float> src, C;
  DevBuf<int> err;
  if (!A.ensure(pieces, (size_t)M * Kp) || !B.ensure(pieces, (size_t)N * Kp) ||
      !src.ensure((size_t)std::max(M, N) * K) || !C.ensure((size_t)M * N) || !err.ensure(1))
    return -1.0;
  __nv_bfloat16 *ta[kMaxPieces], *tb[kMaxPieces];
  cudaEvent_t e0, e1;
  bool ok = cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess;
  for (int q = 0; ok && q < pieces; ++q)
    ok = cudaMemsetAsync(A.p[q].p, 0, (size_t)M * Kp * 2, s) == cudaSuccess &&
         cudaMemsetAsync(B.p[q].p, 0, (size_t)N * Kp * 2, s) == cudaSuccess;
  ok = ok && cudaMemsetAsync(err.p, 0, sizeof(int), s) == cudaSuccess &&
       launch_fill_hash(src.p, (long long)M * K, 1u, s) == cudaSuccess &&
       launch_split_bf16<float>(src.p, M, K, K, pieces, A.ptrs(ta), Kp, s) == cudaSuccess &&
       launch_fill_hash(src.p, (long long)N * K, 2u, s) == cudaSuccess &&
       launch_split_bf16<float>(src.p, N, K, K, pieces, B.ptrs(tb), Kp, s) == cudaSuccess;
  GemmOut out{};
  out.C = C.p;
  out.ldc = N;
  auto run = [&]() {
    return mode == 8 ? launch_gemm_precise(A.in(), M, B.in(), N, Kp, M, N, 1, 0, 0, out, err.p, s)
                     : launch_gemm_split(A.in(), M, B.in(), N, Kp, M, N, 1, 0, 0, pieces, out, err.p, s);
  };
  ok = ok && run() == cudaSuccess && cudaEventRecord(e0, s) == cudaSuccess;
  for (int r = 0; ok && r < reps; ++r) ok = run() == cudaSuccess;
  float ms = 0.f;
  int herr = 0;
  ok = ok && cudaEventRecord(e1, s) == cudaSuccess && cudaEventSynchronize(e1) == cudaSuccess &&
       cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess &&
       cudaMemcpy(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (!ok || herr) {
    set_error("%s: failed (%s, pipeline code %d)", __func__, cudaGetErrorString(cudaGetLastError()), herr);
    return -1.0;
  }
  return (double)ms / reps;
}

}  // extern "C"
