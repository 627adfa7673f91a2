// Batched builds (LowdinGB300_Batch): many systems' two-particle and coupling
// matrices from one fixed sequence of launches, replayed from a CUDA graph.
#include "lint_host.cuh"

#include <map>
#include <tuple>

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
  // pair-indexed arrays of the FP32 row kernels, one PairSlot per two-body species
  DevBuf<float> Dp32, Jp32, DnP32;
  DevBuf<float> Dnmax32;   // per slot: largest shell-block norm of the build's input
  int max_nsh = 0;
  DevBuf<PairSlot> pslots;
  int npslots = 0;
  long long ptotal = 0;
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
  // FP32 kernel of the mixed launches per quartet class (autotune): -1 size
  // rule, 0 jk_tasks_kernel, 1 bra-row kernel; the timings behind the choice
  signed char rows_choice[kNQC];
  float tune_ms[kNQC][2];
  LowdinGB300_Batch() {
    for (int c = 0; c < kNQC; ++c) {
      rows_choice[c] = -1;
      tune_ms[c][0] = tune_ms[c][1] = -1.f;
    }
  }

  ~LowdinGB300_Batch() {
    drop_graphs();
    if (capture) cudaStreamDestroy(capture);
    Ds.release(); Dn.release(); Gacc.release(); Jacc.release(); cnt.release(); slots.release();
    Dp32.release(); Jp32.release(); DnP32.release(); pslots.release();
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
    // pair-indexed arenas of the two-body species
    std::vector<long long> peoff(sp.size(), -1), pairoff(sp.size(), -1);
    long long petot = 0, pptot = 0;
    for (size_t k = 0; k < sp.size(); ++k) {
      if (!sp[k].two_body) continue;
      long long pb[kNumPairClasses];
      peoff[k] = petot;
      pairoff[k] = pptot;
      petot += pair_elements(sp[k].h->sig.start, pb);
      pptot += (long long)sp[k].h->sig.h.size();
    }
    if (!Dp32.ensure(std::max(1LL, petot)) || !Jp32.ensure(std::max(1LL, petot)) ||
        !DnP32.ensure(std::max(1LL, pptot)))
      return false;
    max_nsh = 0;
    for (size_t k = 0; k < sp.size(); ++k) max_nsh = std::max(max_nsh, sp[k].h->nshell());
    if (!Dnmax32.ensure(std::max<size_t>(1, sp.size()))) return false;
    std::vector<PairSlot> hps;
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
      S.Dnmax32 = S.Dn32 ? Dnmax32.p + k : nullptr;
      if (x.two_body) {
        // non-electron species are not screened: their norm pointers are never read
        SpeciesBufs b{S.Ds, S.Ds32, S.Dn ? S.Dn : Dn.p, S.Dn32 ? S.Dn32 : Dn32.p, S.Gacc, S.Gacc32,
                      Dp32.p + peoff[k], Jp32.p + peoff[k], DnP32.p + pairoff[k], S.Dnmax32};
        const auto before = sizes(jk);
        if (!x.h->add_jk_tasks(jk, b, 0.5 * x.factor, cnt.p)) return false;
        mark(jk, before, x.sys);
        PairSlot ps{};
        const PairList &L = x.h->sig;
        ps.pairs = L.d32;
        ps.npairs = (int)L.h.size();
        ps.poff = pairoff[k];
        for (int c = 0; c <= kNumPairClasses; ++c) ps.start[c] = L.start[c];
        pair_elements(L.start, ps.pe_base);
        ps.Ds32 = S.Ds32;
        ps.Dn32 = x.h->is_electron ? S.Dn32 : nullptr;
        ps.Gacc32 = S.Gacc32;
        ps.n = S.n;
        ps.nsh = S.nsh;
        ps.Dp32 = Dp32.p + peoff[k];
        ps.Jp32 = Jp32.p + peoff[k];
        ps.DnP32 = DnP32.p + pairoff[k];
        ps.active = S.active;
        hps.push_back(ps);
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
    npslots = (int)hps.size();
    ptotal = pptot;
    if (npslots > 0) {
      if (!pslots.ensure(hps.size())) return false;
      CK(cudaMemcpyAsync(pslots.p, hps.data(), hps.size() * sizeof(PairSlot), cudaMemcpyHostToDevice, s));
    }
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

  // Autotuner: for every quartet class whose FP32 half can run on either
  // FP32 kernel, time both on this batch's current densities (the FP32
  // launch alone, after one untimed launch) and keep the faster.  Choices are
  // cached process-wide by (class, log2 of the class's bra x ket pairs, log2
  // of the largest species), so batches of similar molecules reuse them;
  // `force` re-times.  Both kernels take the same quartets, so the choice
  // changes only the order of FP32 additions.
  bool autotune(double split, bool force, cudaStream_t s) {
    if (!finalized) {
      set_error("batch_autotune: batch not finalised");
      return false;
    }
    if (tasks_dirty) {
      if (!jk.upload(s, active.p, &on) || !cp.upload(s, active.p, &on)) return false;
      drop_graphs();
      tasks_dirty = false;
    }
    CK(cudaMemsetAsync(Dn.p, 0, Dn.n * sizeof(double), s));
    CK(cudaMemsetAsync(Dn32.p, 0, Dn32.n * sizeof(float), s));
    CK(launch_prepare_batch(slots.p, nslots, total, s));
    CK(cudaMemsetAsync(Dnmax32.p, 0, Dnmax32.n * sizeof(float), s));
    CK(launch_dn_max_batch(slots.p, nslots, max_nsh, s));
    if (npslots) CK(launch_pair_gather(pslots.p, npslots, ptotal, s));
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    bool ok = true;
    for (int c = 0; c < kNQC && ok; ++c) {
      const int cb = c / kNumPairClasses, ck = c % kNumPairClasses;
      if (!jk.cnt[c] || !jk_rows_used(cb, ck, jk.rn[c], jk.rnsh[c])) continue;
      double work = 0;
      for (const auto &t : jk.group[c]) work += (double)t.nbra * t.nket;
      const auto key = std::make_tuple(c, (int)std::log2(std::max(1.0, work)), (int)std::log2(std::max(1, jk.rn[c])));
      if (!force) {
        std::lock_guard<std::mutex> lk(tune_mu());
        auto it = tune_cache().find(key);
        if (it != tune_cache().end()) {
          rows_choice[c] = it->second;
          continue;
        }
      }
      float ms[2] = {0.f, 0.f};
      for (int v = 1; v >= 0 && ok; --v) {
        signed char pref[kNQC];
        for (int k = 0; k < kNQC; ++k) pref[k] = (signed char)v;
        ok = LibintInterface::launch_jk_groups(jk, 1, split, boys, s, skip, pref, c, true);
        if (!ok) break;
        if (cudaEventRecord(e0, s) != cudaSuccess) ok = false;
        for (int r = 0; r < 2 && ok; ++r) ok = LibintInterface::launch_jk_groups(jk, 1, split, boys, s, skip, pref, c, true);
        if (ok && (cudaEventRecord(e1, s) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
                   cudaEventElapsedTime(&ms[v], e0, e1) != cudaSuccess))
          ok = false;
      }
      if (!ok) break;
      tune_ms[c][1] = ms[1] / 2;
      tune_ms[c][0] = ms[0] / 2;
      rows_choice[c] = ms[1] <= ms[0] ? 1 : 0;
      std::lock_guard<std::mutex> lk(tune_mu());
      tune_cache()[key] = rows_choice[c];
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (!ok) {
      set_error("batch_autotune: a timed launch failed");
      return false;
    }
    drop_graphs();
    return true;
  }
  static std::mutex &tune_mu() {
    static std::mutex m;
    return m;
  }
  static std::map<std::tuple<int, int, int>, signed char> &tune_cache() {
    static std::map<std::tuple<int, int, int>, signed char> m;
    return m;
  }

  // every launch of one build, in stream order
  bool fock_sequence(int precision, double split, cudaStream_t s) {
    CK(cudaMemsetAsync(Dn.p, 0, Dn.n * sizeof(double), s));
    CK(cudaMemsetAsync(Dn32.p, 0, Dn32.n * sizeof(float), s));
    CK(cudaMemsetAsync(cnt.p, 0, 2 * kNQC * sizeof(unsigned long long), s));
    CK(launch_prepare_batch(slots.p, nslots, total, s));
    const int jk_mixed = precision & 1;
    if (jk_mixed) {
      CK(cudaMemsetAsync(Dnmax32.p, 0, Dnmax32.n * sizeof(float), s));
      CK(launch_dn_max_batch(slots.p, nslots, max_nsh, s));
    }
    if (jk_mixed && npslots) CK(launch_pair_gather(pslots.p, npslots, ptotal, s));
    if (!LibintInterface::launch_jk_groups(jk, jk_mixed, jk_mixed ? split : 0.0, boys, s, skip, rows_choice))
      return false;
    if (jk_mixed && npslots) CK(launch_pair_scatter(pslots.p, npslots, ptotal, s));
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
  // every species is checked before the batch changes: a rejected system
  // leaves no trace
  for (int k = 0; k < nspecies; ++k) {
    if (!check_handle(species[k], __func__)) return -1;
    if (ld && ld[k] < species[k]->nbasis) {
      set_error("batch_add_system: row stride %d below the species' %d functions", ld[k], species[k]->nbasis);
      return -1;
    }
  }
  const int sys = (int)b->sys_first.size();
  const int first = (int)b->sp.size();
  b->sys_first.push_back(first);
  for (int k = 0; k < nspecies; ++k) {
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

int LowdinGB300_batch_autotune(LowdinGB300_Batch *b, double split, int force, void *stream) {
  if (!b) return -1;
  return b->autotune(split, force != 0, (cudaStream_t)stream) ? 0 : -1;
}

int LowdinGB300_batch_tuning(LowdinGB300_Batch *b, int *choice, float *ms_rows, float *ms_tiles) {
  if (!b) return -1;
  for (int c = 0; c < kNQC; ++c) {
    if (choice) choice[c] = b->rows_choice[c];
    if (ms_rows) ms_rows[c] = b->tune_ms[c][1];
    if (ms_tiles) ms_tiles[c] = b->tune_ms[c][0];
  }
  return kNQC;
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
