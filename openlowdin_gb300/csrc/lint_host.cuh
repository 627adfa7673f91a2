// Host-side internals shared by the library's translation units (lint.cu,
// batch.cu, mp2.cu): error reporting, device buffers, shell-pair lists, task
// lists and the per-species handle behind the LibintInterface_* C ABI.
#pragma once
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
#include <type_traits>
#include <vector>

#include <cublas_v2.h>

#include "../../include/lowdin_gb300.h"
#include "kernels.cuh"

namespace lgb {

// records the message for LowdinGB300_last_error (and prints it)
void set_error(const char *fmt, ...);

#define CK(call)                                                                          \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess) {                                                              \
      set_error("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
      return false;                                                                       \
    }                                                                                     \
  } while (0)

// device copies of the Boys tables of the current device
bool device_boys(BoysTables &out);

struct HostShell {
  int l = 0, nprim = 0;
  double O[3] = {0, 0, 0};
  std::vector<double> alpha, cn;  // cn = coefficient * primitive norm of x^l
};

double prim_norm(double a, int l);
void overlap_block(const HostShell &A, const HostShell &B, double *S, double *T);
void potential_block(const HostShell &A, const HostShell &B, int nc, const double *Z, const double *R, double *V);

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
  // the FP32 records of one-primitive pairs as structure of arrays
  // (kSoaFields arrays of size(); null when a pair has several primitives),
  // read by the FP32 row kernels one coalesced field at a time
  float *soa32 = nullptr;
  void release() {
    if (d) cudaFree(d);
    if (dp) cudaFree(dp);
    if (d32) cudaFree(d32);
    if (dp32) cudaFree(dp32);
    if (soa32) cudaFree(soa32);
    d = nullptr;
    dp = nullptr;
    d32 = nullptr;
    dp32 = nullptr;
    soa32 = nullptr;
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
    if (!(dev_upload(d, h) && dev_upload(dp, hp) && dev_upload(d32, h32) && dev_upload(dp32, hp32))) return false;
    bool one = !h.empty();
    for (const auto &r : h) one = one && r.nprim == 1;
    if (one) {
      const size_t np = h.size();
      std::vector<float> soa(kSoaFields * np);
      for (size_t i = 0; i < np; ++i) {
        const PairRec32 &r = h32[i];
        const PrimRec32 &q = hp32[r.prim0];
        float *c = soa.data() + i;
        c[kSoaQ * np] = r.Q;
        c[kSoaShells * np] = __int_as_float_host(r.sa | r.sb << 16);
        c[kSoaFuncs * np] = __int_as_float_host(r.fa | r.fb << 16);
        c[kSoaP * np] = q.p;
        c[kSoaInvP * np] = q.inv_p;
        c[kSoaKt * np] = q.Kt;
        for (int k = 0; k < 3; ++k) {
          c[(kSoaPx + k) * np] = q.P[k];
          c[(kSoaPAx + k) * np] = q.PA[k];
          c[(kSoaABx + k) * np] = r.AB[k];
        }
      }
      if (!dev_upload(soa32, soa)) return false;
    }
    return true;
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
  // pair-indexed arrays of the FP32 row kernels (PairSlot), or null
  float *Dp32 = nullptr;
  float *Jp32 = nullptr;
  float *DnP32 = nullptr;
  const float *Dnmax32 = nullptr;   // largest element of Dn32, or null
};

// Tasks grouped by quartet class (bra pair class * 6 + ket pair class); one
// device array holds every group, each group is one launch.
template <typename T>
struct TaskSet {
  std::vector<T> group[kNQC];
  T *d = nullptr;
  size_t cap = 0;
  int off[kNQC] = {0}, cnt[kNQC] = {0}, nblk[kNQC] = {0};
  int nrblk[kNQC] = {0}, rn[kNQC] = {0}, rnsh[kNQC] = {0};   // bra-row launches (J/K tasks)
  // block offsets of task t of group c (b: blocks so far in the group)
  void place(int c, T &t, int &b) {
    t.nbx = task_nbx(t.nket);
    t.blk0 = b;
    b += t.nbx * task_nby(t.nbra);
    if constexpr (std::is_same<T, JKTask>::value) {
      t.rblk0 = nrblk[c];
      nrblk[c] += t.nbra;
      rn[c] = std::max(rn[c], t.n);
      rnsh[c] = std::max(rnsh[c], t.nsh);
    }
  }
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
      nrblk[c] = rn[c] = rnsh[c] = 0;
      for (T t : group[c]) {
        if (on && t.active && !(*on)[t.active - flag_base]) continue;
        place(c, t, b);
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


}  // namespace lgb

using namespace lgb;

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
  DevBuf<double> dGem;         // geminal parameters of the last G12 call {count, exponents, coefficients}
  // precision of LibintInterface_compute_2body_direct (LowdinGB300_set_precision):
  // 0 = FP64 (the reference's behaviour), 1 = FP32/FP64 split at abi_split
  int abi_precision = 0;
  double abi_split = 1e-5;
  DevBuf<double> dD, dDs, dDn, dGacc, dG, dA, dC, dDsC, dJacc;
  DevBuf<float> dDs32, dDn32, dGacc32, dDsC32, dJacc32;
  DevBuf<float> dDp32, dJp32, dDnP32;   // pair-indexed arrays of the FP32 row kernels
  DevBuf<float> dDnmax32;               // largest shell-block norm of the last density
  DevBuf<PairSlot> dpslot;
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
    dGem.release();
    dD.release(); dDs.release(); dDn.release(); dGacc.release(); dG.release(); dA.release(); dC.release();
    dDsC.release(); dJacc.release();
    dDs32.release(); dDn32.release(); dGacc32.release(); dDsC32.release(); dJacc32.release();
    dDp32.release(); dJp32.release(); dDnP32.release(); dpslot.release(); dDnmax32.release();
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
        set_error("shell with l=%d: the library handles l <= %d", s.l, kMaxL);
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
      // pair-indexed arrays of the FP32 row kernels and their slot
      long long pe_base[kNumPairClasses];
      const long long pe = pair_elements(sig.start, pe_base);
      const int npairs = (int)sig.h.size();
      if (!dDp32.ensure(std::max(1LL, pe)) || !dJp32.ensure(std::max(1LL, pe)) ||
          !dDnP32.ensure(std::max(1, npairs)) || !dpslot.ensure(1) || !dDnmax32.ensure(1))
        return false;
      PairSlot ps{};
      ps.pairs = sig.d32;
      ps.npairs = npairs;
      ps.poff = 0;
      for (int c = 0; c <= kNumPairClasses; ++c) ps.start[c] = sig.start[c];
      for (int c = 0; c < kNumPairClasses; ++c) ps.pe_base[c] = pe_base[c];
      ps.Ds32 = dDs32.p;
      ps.Dn32 = is_electron ? dDn32.p : nullptr;
      ps.Gacc32 = dGacc32.p;
      ps.n = n;
      ps.nsh = nsh;
      ps.Dp32 = dDp32.p;
      ps.Jp32 = dJp32.p;
      ps.DnP32 = dDnP32.p;
      ps.active = nullptr;
      CK(cudaMemcpyAsync(dpslot.p, &ps, sizeof(ps), cudaMemcpyHostToDevice, s));
      jk.clear();
      SpeciesBufs b{dDs.p, dDs32.p, dDn.p, dDn32.p, dGacc.p, dGacc32.p, dDp32.p, dJp32.p, dDnP32.p, dDnmax32.p};
      if (!add_jk_tasks(jk, b, 0.5 * factor, dcount.p)) return false;
      if (!jk.upload(s)) return false;
      jk_hf = 0.5 * factor;
      jk_ready = true;
    }
    CK(launch_prepare_density(dDin, d_norma, d_shell_of, n, nsh, dDs.p, dDs32.p, dDn.p, dDn32.p, s));
    if (precision != 0 && is_electron) CK(launch_dn_max(dDn32.p, nsh, dDnmax32.p, s));
    CK(cudaMemsetAsync(dGacc.p, 0, sizeof(double) * n * n, s));
    CK(cudaMemsetAsync(dGacc32.p, 0, sizeof(float) * n * n, s));
    CK(cudaMemsetAsync(dcount.p, 0, sizeof(unsigned long long) * kNQC, s));
    if (precision != 0) CK(launch_pair_gather(dpslot.p, 1, (long long)sig.h.size(), s));
    if (!launch_jk_groups(jk, precision, split, boys, s)) return false;
    if (precision != 0) CK(launch_pair_scatter(dpslot.p, 1, (long long)sig.h.size(), s));
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
        t.hf32 = (float)hf;
        t.bra0 = sig.start[cb];
        t.nbra = sig.count(cb);
        t.ket0 = sig.start[ck];
        t.nket = sig.count(ck);
        t.n = nbasis;
        t.nsh = nshell();
        t.triangle = cb == ck;
        t.screen = is_electron ? 1 : 0;
        t.soa32 = sig.soa32;
        t.npairs = (int)sig.h.size();
        t.Dnmax32 = is_electron ? bf.Dnmax32 : nullptr;
        if (bf.Dp32) {
          long long pe_base[kNumPairClasses];
          pair_elements(sig.start, pe_base);
          t.Dp32 = bf.Dp32 + pe_base[ck];
          t.Jp32 = bf.Jp32 + pe_base[ck];
          t.DnP32 = is_electron ? bf.DnP32 : nullptr;
        }
        ts.add(cb, ck, t);
      }
    return true;
  }

  // rows: per quartet class the FP32 kernel of mixed launches (-1 size rule,
  // 0 jk_tasks_kernel, 1 bra-row kernel; null: size rule); only: a single
  // class (-1: all) and, with lower_only, only its FP32 launch (autotuning)
  static bool launch_jk_groups(const TaskSet<JKTask> &ts, int precision, double split, BoysTables boys,
                               cudaStream_t s, double skip = 0.0, const signed char *rows = nullptr,
                               int only = -1, bool lower_only = false) {
    for (int c = 0; c < kNQC; ++c) {
      if (!ts.cnt[c] || (only >= 0 && c != only)) continue;
      TaskLaunch tl{};
      tl.rows_pref = rows ? rows[c] : -1;
      tl.ntasks = ts.cnt[c];
      tl.nblocks = ts.nblk[c];
      tl.nrblocks = ts.nrblk[c];
      tl.rows_n = ts.rn[c];
      tl.rows_nsh = ts.rnsh[c];
      tl.eps = DBL_EPSILON;
      tl.cut = 1e-10;
      tl.skip = (float)skip;
      tl.boys = boys;
      const int cb = c / kNumPairClasses, ck = c % kNumPairClasses;
      if (precision == 0) {
        tl.split = 0.0;
        set_fp32_copies(tl);
        CK(launch_jk_tasks(cb, ck, false, ts.d + ts.off[c], tl, s));
      } else {
        tl.split = split;
        set_fp32_copies(tl);
        tl.lower = 0;
        if (!lower_only) CK(launch_jk_tasks(cb, ck, false, ts.d + ts.off[c], tl, s));
        tl.lower = 1;
        CK(launch_jk_tasks(cb, ck, true, ts.d + ts.off[c], tl, s));
      }
    }
    return true;
  }
};

namespace lgb {

// coupling tasks of species pair (A bra, B ket) into ts
bool add_cp_tasks(TaskSet<CPTask> &ts, LibintInterface *A, LibintInterface *B, const SpeciesBufs &ba,
                  const SpeciesBufs &bb, bool want_a, bool want_b, double scale,
                  unsigned long long *counters = nullptr);
// mode 0: FP64, 1: FP32 throughout, 2: split at `split` (FP64 above, FP32 below)
bool launch_cp_groups(const TaskSet<CPTask> &ts, int mode, double split, BoysTables boys, cudaStream_t s,
                      double skip = 0.0);
bool coupling(LibintInterface *A, LibintInterface *B, const double *dDa, const double *dDb, double *dJa,
              double *dJb, bool fp32, cudaStream_t s);
bool first_quarter(LibintInterface *A, LibintInterface *B, const double *hD, const double *hC, int p,
                   double *hOut);
bool check_handle(LibintInterface *l, const char *fn);
void unsupported(const char *fn);

}  // namespace lgb
