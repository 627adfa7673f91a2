// Block-cooperative kernels for the quartet classes of total angular momentum
// above kTemplatedMaxL, the Schwarz kernels, and the dispatch of every class
// to its templated or cooperative kernel.
//
// In a cooperative kernel every warp is a worker with its own class-sized
// shared work arrays (up to 4 warps per CTA, a persistent grid); a warp takes
// work units -- a bra pair and 8 ket pairs of a task's 4 x 32 tile, or one
// quartet -- and evaluates their quartets one after another, its 32 lanes
// together on each (eri_coop), then digests the quartet's integrals with the
// lanes split over the output elements.  They compute in
// FP64 (also when a mixed launch asks for the FP32 half: the split decides
// which quartets a launch takes, the quartets are evaluated in FP64 and
// accumulated into the FP64 arrays).
#include "eri_generic.cuh"
#include "fock_kernels.cuh"

#include <algorithm>
#include <cstdlib>

namespace lgb {

constexpr int NPC = kNumPairClasses;
extern const JKFn kJK64_0[NPC], kJK64_1[NPC], kJK64_2[NPC], kJK64_3[NPC], kJK64_4[NPC], kJK64_5[NPC];
extern const JKFn kJK32_0[NPC], kJK32_1[NPC], kJK32_2[NPC], kJK32_3[NPC], kJK32_4[NPC], kJK32_5[NPC];
extern const JKFn kJKR_0[NPC], kJKR_1[NPC], kJKR_2[NPC], kJKR_3[NPC], kJKR_4[NPC], kJKR_5[NPC];
extern const CPFn kCP64_0[NPC], kCP64_1[NPC], kCP64_2[NPC], kCP64_3[NPC], kCP64_4[NPC], kCP64_5[NPC];
extern const CPFn kCP32_0[NPC], kCP32_1[NPC], kCP32_2[NPC], kCP32_3[NPC], kCP32_4[NPC], kCP32_5[NPC];
extern const ITFn kIT_0[NPC], kIT_1[NPC], kIT_2[NPC], kIT_3[NPC], kIT_4[NPC], kIT_5[NPC];
extern const MXFn kMX_0[NPC], kMX_1[NPC], kMX_2[NPC], kMX_3[NPC], kMX_4[NPC], kMX_5[NPC];

namespace {

// bra pair classes with an f shell have no templated kernels: every entry null
const JKFn kJKnone[NPC] = {};
const CPFn kCPnone[NPC] = {};
const ITFn kITnone[NPC] = {};
const MXFn kMXnone[NPC] = {};
#define LGB_F_ROWS(X) X, X, X, X
const JKFn *const kJK64[NPC] = {kJK64_0, kJK64_1, kJK64_2, kJK64_3, kJK64_4, kJK64_5, LGB_F_ROWS(kJKnone)};
const JKFn *const kJK32[NPC] = {kJK32_0, kJK32_1, kJK32_2, kJK32_3, kJK32_4, kJK32_5, LGB_F_ROWS(kJKnone)};
const JKFn *const kJKR[NPC] = {kJKR_0, kJKR_1, kJKR_2, kJKR_3, kJKR_4, kJKR_5, LGB_F_ROWS(kJKnone)};
const CPFn *const kCP64[NPC] = {kCP64_0, kCP64_1, kCP64_2, kCP64_3, kCP64_4, kCP64_5, LGB_F_ROWS(kCPnone)};
const CPFn *const kCP32[NPC] = {kCP32_0, kCP32_1, kCP32_2, kCP32_3, kCP32_4, kCP32_5, LGB_F_ROWS(kCPnone)};
const ITFn *const kIT[NPC] = {kIT_0, kIT_1, kIT_2, kIT_3, kIT_4, kIT_5, LGB_F_ROWS(kITnone)};
const MXFn *const kMX[NPC] = {kMX_0, kMX_1, kMX_2, kMX_3, kMX_4, kMX_5, LGB_F_ROWS(kMXnone)};
#undef LGB_F_ROWS

const dim3 kBlock(32, kWarpsPerBlock);
// LOWDIN_GB300_ROWS=0 keeps the FP32 half of mixed builds on jk_tasks_kernel
// (read at every launch, so a process can compare both kernels)
bool row_rows_off() {
  const char *e = std::getenv("LOWDIN_GB300_ROWS");
  return e && e[0] == '0';
}
constexpr int kCoUnitsPerTile = kWarpsPerBlock * 4;   // (bra row, group of 8 kets)
constexpr int kCoMaxSmem = 200 * 1024;                 // dynamic shared memory of a cooperative CTA

struct GenClass {
  int la, lb, lc, ld;
};

// work unit u of a task-tiled launch -> task, bra position, first ket position
template <typename Task>
__device__ __forceinline__ const Task &coop_unit(const Task *tasks, int ntasks, int u, int *bpos, int *kpos0) {
  const int blk = u / kCoUnitsPerTile, sub = u % kCoUnitsPerTile;
  const Task &T = tasks[find_task(tasks, ntasks, blk)];
  const int local = blk - T.blk0;
  const int tx = local % T.nbx, ty = local / T.nbx;
  *bpos = ty * kWarpsPerBlock + sub / 4;
  *kpos0 = tx * 32 + (sub % 4) * 8;
  return T;
}

// every warp of a cooperative CTA is an independent worker with its own work
// arrays: in shared memory, or, for classes whose arrays exceed a CTA's shared
// memory (a pair of f shells against f or d), in the launch's global scratch
// `gscr` (one slice per warp of the grid, cached by L2)
#define LGB_COOP_PROLOGUE(K)                                              \
  extern __shared__ double smem[];                                        \
  __shared__ CartInfo cart_sm[kCartN];                                    \
  const CartInfo *ct = cart_shared(cart_sm);                              \
  const CoLayout Lo = co_layout(K.la, K.lb, K.lc, K.ld);                  \
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;             \
  const int nwarps = blockDim.x >> 5;                                     \
  double *sm = gscr ? gscr + ((size_t)blockIdx.x * nwarps + warp) * Lo.total \
                    : smem + (size_t)warp * Lo.total;                     \
  const double *I = sm + Lo.out;                                          \
  const WarpGroup g;                                                      \
  const long long w0 = (long long)blockIdx.x * nwarps + warp, wstep = (long long)gridDim.x * nwarps;

// ------------------------------------------------------------------ J/K --
__global__ void __launch_bounds__(128) jk_coop_kernel(const JKTask *__restrict__ tasks, TaskLaunch TL, GenClass K, double *gscr) {
  LGB_COOP_PROLOGUE(K)
  const int NA = ncart(K.la), NB = ncart(K.lb), NC = ncart(K.lc), ND = ncart(K.ld);
  for (long long u = w0; u < (long long)TL.nblocks * kCoUnitsPerTile; u += wstep) {
    int bpos, kpos0;
    const JKTask &T = coop_unit(tasks, TL.ntasks, (int)u, &bpos, &kpos0);
    const int act = system_flag(T.active);
    if (bpos >= T.nbra || act == kSysOff || (act == kSysFP64 && TL.mixed && TL.lower)) continue;
    for (int kpos = kpos0; kpos < kpos0 + 8 && kpos < T.nket; ++kpos) {
      if (T.triangle && kpos > bpos) break;
      const int bi = T.bra0 + bpos, ki = T.ket0 + kpos;
      const PairRec &bra = T.pairs[bi];
      const PairRec &ket = T.pairs[ki];
      bool active = true;
      if (TL.mixed) {
        float b = T.pairs32[bi].Q * T.pairs32[ki].Q;
        if (T.screen) {
          b *= dnorm6(T.Dn32, T.nsh, bra.sa, bra.sb, ket.sa, ket.sb);
          if (b < fmaxf(TL.eps32, act == kSysFP64 ? 0.f : TL.skip)) active = false;
        }
        if (act != kSysFP64 && (TL.lower ? !(b < TL.split32) : (b < TL.split32))) active = false;
      } else if (T.screen) {
        if (abs_below(bra.Q * ket.Q * dnorm6(T.Dn, T.nsh, bra.sa, bra.sb, ket.sa, ket.sb), TL.eps)) active = false;
      }
      if (!active) continue;   // uniform across the warp
      if (T.count && lane == 0) atomicAdd(T.count, 1ull);
      eri_coop(g, ct, Lo, K.la, K.lb, K.lc, K.ld, bra, T.prims, ket, T.prims, TL.boys.f64, sm);
      const double deg = (bra.sa == bra.sb ? 1 : 2) * (ket.sa == ket.sb ? 1 : 2) * (bi == ki ? 1 : 2);
      const double hdeg = deg * T.hf;
      const double *__restrict__ D = T.Ds;
      const int n = T.n, fa = bra.fa, fb = bra.fb, fc = ket.fa, fd = ket.fb;
      auto Iat = [&](int a, int b, int c, int d) { return I[((a * NB + b) * NC + c) * ND + d]; };
      // the six updates, lanes over their output elements
      const int n12 = NA * NB, n34 = NC * ND, n13 = NA * NC, n24 = NB * ND, n14 = NA * ND, n23 = NB * NC;
      for (int t = lane; t < n12 + n34 + n13 + n24 + n14 + n23; t += 32) {
        int x = t;
        double s = 0;
        if (x < n12) {
          const int a = x / NB, b = x % NB;
          for (int c = 0; c < NC; ++c)
            for (int d = 0; d < ND; ++d) s += __ldg(D + (fc + c) * n + fd + d) * Iat(a, b, c, d);
          atomicAdd(T.Gacc + (size_t)(fa + a) * n + fb + b, s * deg);
          continue;
        }
        x -= n12;
        if (x < n34) {
          const int c = x / ND, d = x % ND;
          for (int a = 0; a < NA; ++a)
            for (int b = 0; b < NB; ++b) s += __ldg(D + (fa + a) * n + fb + b) * Iat(a, b, c, d);
          atomicAdd(T.Gacc + (size_t)(fc + c) * n + fd + d, s * deg);
          continue;
        }
        x -= n34;
        if (x < n13) {
          const int a = x / NC, c = x % NC;
          for (int b = 0; b < NB; ++b)
            for (int d = 0; d < ND; ++d) s += __ldg(D + (fb + b) * n + fd + d) * Iat(a, b, c, d);
          atomicAdd(T.Gacc + (size_t)(fa + a) * n + fc + c, s * hdeg);
          continue;
        }
        x -= n13;
        if (x < n24) {
          const int b = x / ND, d = x % ND;
          for (int a = 0; a < NA; ++a)
            for (int c = 0; c < NC; ++c) s += __ldg(D + (fa + a) * n + fc + c) * Iat(a, b, c, d);
          atomicAdd(T.Gacc + (size_t)(fb + b) * n + fd + d, s * hdeg);
          continue;
        }
        x -= n24;
        if (x < n14) {
          const int a = x / ND, d = x % ND;
          for (int b = 0; b < NB; ++b)
            for (int c = 0; c < NC; ++c) s += __ldg(D + (fb + b) * n + fc + c) * Iat(a, b, c, d);
          atomicAdd(T.Gacc + (size_t)(fa + a) * n + fd + d, s * hdeg);
          continue;
        }
        x -= n14;
        {
          const int b = x / NC, c = x % NC;
          for (int a = 0; a < NA; ++a)
            for (int d = 0; d < ND; ++d) s += __ldg(D + (fa + a) * n + fd + d) * Iat(a, b, c, d);
          atomicAdd(T.Gacc + (size_t)(fb + b) * n + fc + c, s * hdeg);
        }
      }
    }
  }
}

// ------------------------------------------------------------- coupling --
__global__ void __launch_bounds__(128) cp_coop_kernel(const CPTask *__restrict__ tasks, TaskLaunch TL, GenClass K, double *gscr) {
  LGB_COOP_PROLOGUE(K)
  const int NA = ncart(K.la), NB = ncart(K.lb), NC = ncart(K.lc), ND = ncart(K.ld);
  for (long long u = w0; u < (long long)TL.nblocks * kCoUnitsPerTile; u += wstep) {
    int bpos, kpos0;
    const CPTask &T = coop_unit(tasks, TL.ntasks, (int)u, &bpos, &kpos0);
    const int act = system_flag(T.active);
    if (bpos >= T.nbra || act == kSysOff || (act == kSysFP64 && TL.mixed && TL.lower)) continue;
    for (int kpos = kpos0; kpos < kpos0 + 8 && kpos < T.nket; ++kpos) {
      const int bi = T.bra0 + bpos, ki = T.ket0 + kpos;
      const bool tiny = TL.mixed ? T.pa32[bi].Q * T.pb32[ki].Q * 0.999f < TL.cut32
                                       : T.pa[bi].Q * T.pb[ki].Q * (1.0 - 1e-9) < TL.cut;
      if (tiny) continue;
      if (TL.mixed) {
        const PairRec32 &b32 = T.pa32[bi];
        const PairRec32 &k32 = T.pb32[ki];
        float dm = 0.f;
        if (T.DnA32) dm = __ldg(T.DnA32 + b32.sa * T.nshA + b32.sb);
        if (T.DnB32) dm = fmaxf(dm, __ldg(T.DnB32 + k32.sa * T.nshB + k32.sb));
        const float b = b32.Q * k32.Q * dm;
        if (act != kSysFP64 && (TL.lower ? !(b < TL.split32) : (b < TL.split32))) continue;
        if ((T.DnA32 || T.DnB32) && act != kSysFP64 && b < TL.skip) continue;
      }
      if (T.count && lane == 0) atomicAdd(T.count, 1ull);
      const PairRec &bra = T.pa[bi];
      const PairRec &ket = T.pb[ki];
      eri_coop(g, ct, Lo, K.la, K.lb, K.lc, K.ld, bra, T.pra, ket, T.prb, TL.boys.f64, sm);
      auto Iat = [&](int a, int b, int c, int d) {
        const double v = I[((a * NB + b) * NC + c) * ND + d];
        return abs_below(v, TL.cut) ? 0.0 : v;
      };
      const int fa = bra.fa, fb = bra.fb, fc = ket.fa, fd = ket.fb;
      const bool abdiff = bra.sa != bra.sb, cddiff = ket.sa != ket.sb;
      const int nja = T.JA ? NA * NB : 0, njb = T.JB ? NC * ND : 0;
      for (int t = lane; t < nja + njb; t += 32) {
        double s = 0;
        if (t < nja) {
          const int a = t / NB, b = t % NB;
          for (int c = 0; c < NC; ++c)
            for (int d = 0; d < ND; ++d) s += __ldg(T.DsB + (fc + c) * T.nB + fd + d) * Iat(a, b, c, d);
          s *= (cddiff ? 2.0 : 1.0) * T.scale;
          atomicAdd(T.JA + (size_t)(fa + a) * T.nA + fb + b, s);
          if (abdiff) atomicAdd(T.JA + (size_t)(fb + b) * T.nA + fa + a, s);
        } else {
          const int x = t - nja, c = x / ND, d = x % ND;
          for (int a = 0; a < NA; ++a)
            for (int b = 0; b < NB; ++b) s += __ldg(T.DsA + (fa + a) * T.nA + fb + b) * Iat(a, b, c, d);
          s *= (abdiff ? 2.0 : 1.0) * T.scale;
          atomicAdd(T.JB + (size_t)(fc + c) * T.nB + fd + d, s);
          if (cddiff) atomicAdd(T.JB + (size_t)(fd + d) * T.nB + fc + c, s);
        }
      }
    }
  }
}

// ---------------------------------------------------------- geminal (G12) --
// Every class runs here (the geminal matrices are not a hot path): one quartet
// per warp, all quartets of the launch's bra x ket pair ranges, no screening.
__global__ void __launch_bounds__(128) g12_coop_kernel(G12Params P, GenClass K, double *gscr) {
  LGB_COOP_PROLOGUE(K)
  const int NA = ncart(K.la), NB = ncart(K.lb), NC = ncart(K.lc), ND = ncart(K.ld);
  const long long nq = (long long)P.nbra * P.nket;
  for (long long q = w0; q < nq; q += wstep) {
    const int bpos = (int)(q / P.nket), kpos = (int)(q % P.nket);
    if (P.triangle && kpos > bpos) continue;
    const int bi = P.bra0 + bpos, ki = P.ket0 + kpos;
    const PairRec &bra = P.pa[bi];
    const PairRec &ket = P.pb[ki];
    eri_coop<WarpGroup, true>(g, ct, Lo, K.la, K.lb, K.lc, K.ld, bra, P.pra, ket, P.prb, nullptr, sm, P.gem);
    auto Iat = [&](int a, int b, int c, int d) { return I[((a * NB + b) * NC + c) * ND + d]; };
    const int fa = bra.fa, fb = bra.fb, fc = ket.fa, fd = ket.fb;
    const double *__restrict__ D = P.Ds;
    if (P.intra) {
      const double deg = (bra.sa == bra.sb ? 1 : 2) * (ket.sa == ket.sb ? 1 : 2) * (bi == ki ? 1 : 2);
      const double hdeg = deg * P.hf;
      const int n = P.n;
      const int n12 = NA * NB, n34 = NC * ND, n13 = NA * NC, n24 = NB * ND, n14 = NA * ND, n23 = NB * NC;
      // the six updates, lanes over their output elements
      for (int t = lane; t < n12 + n34 + n13 + n24 + n14 + n23; t += 32) {
        int x = t;
        double s = 0;
        if (x < n12) {
          const int a = x / NB, b = x % NB;
          for (int c = 0; c < NC; ++c)
            for (int d = 0; d < ND; ++d) s += D[(fc + c) * n + fd + d] * Iat(a, b, c, d);
          atomicAdd(P.Gacc + (size_t)(fa + a) * n + fb + b, s * deg);
          continue;
        }
        x -= n12;
        if (x < n34) {
          const int c = x / ND, d = x % ND;
          for (int a = 0; a < NA; ++a)
            for (int b = 0; b < NB; ++b) s += D[(fa + a) * n + fb + b] * Iat(a, b, c, d);
          atomicAdd(P.Gacc + (size_t)(fc + c) * n + fd + d, s * deg);
          continue;
        }
        x -= n34;
        if (x < n13) {
          const int a = x / NC, c = x % NC;
          for (int b = 0; b < NB; ++b)
            for (int d = 0; d < ND; ++d) s += D[(fb + b) * n + fd + d] * Iat(a, b, c, d);
          atomicAdd(P.Gacc + (size_t)(fa + a) * n + fc + c, s * hdeg);
          continue;
        }
        x -= n13;
        if (x < n24) {
          const int b = x / ND, d = x % ND;
          for (int a = 0; a < NA; ++a)
            for (int c = 0; c < NC; ++c) s += D[(fa + a) * n + fc + c] * Iat(a, b, c, d);
          atomicAdd(P.Gacc + (size_t)(fb + b) * n + fd + d, s * hdeg);
          continue;
        }
        x -= n24;
        if (x < n14) {
          const int a = x / ND, d = x % ND;
          for (int b = 0; b < NB; ++b)
            for (int c = 0; c < NC; ++c) s += D[(fb + b) * n + fc + c] * Iat(a, b, c, d);
          atomicAdd(P.Gacc + (size_t)(fa + a) * n + fd + d, s * hdeg);
          continue;
        }
        x -= n14;
        {
          const int b = x / NC, c = x % NC;
          for (int a = 0; a < NA; ++a)
            for (int d = 0; d < ND; ++d) s += D[(fa + a) * n + fd + d] * Iat(a, b, c, d);
          atomicAdd(P.Gacc + (size_t)(fb + b) * n + fc + c, s * hdeg);
        }
      }
    } else {
      // J of the bra species: both orientations of a two-shell bra pair, the
      // ket pair's density over its components (x2 for a two-shell ket pair)
      const bool abdiff = bra.sa != bra.sb, cddiff = ket.sa != ket.sb;
      for (int t = lane; t < NA * NB; t += 32) {
        const int a = t / NB, b = t % NB;
        double s = 0;
        for (int c = 0; c < NC; ++c)
          for (int d = 0; d < ND; ++d) {
            const double v = Iat(a, b, c, d);
            if (!abs_below(v, P.cut)) s += D[(size_t)(fc + c) * P.nB + fd + d] * v;
          }
        if (cddiff) s *= 2.0;
        atomicAdd(P.Gacc + (size_t)(fa + a) * P.n + fb + b, s);
        if (abdiff) atomicAdd(P.Gacc + (size_t)(fb + b) * P.n + fa + a, s);
      }
    }
  }
}

// -------------------------------------------------------- first quarter --
// role r of the permutational orbit: (mu, nu, l, s) -> quartet indices (a, b, c, d)
__device__ __forceinline__ void it_map(int r, int mu, int nu, int l, int s, int *a, int *b, int *c, int *d) {
  switch (r) {
    case 0: *a = mu; *b = nu; *c = l; *d = s; break;   // (a b|c d)
    case 1: *a = nu; *b = mu; *c = l; *d = s; break;   // (b a|c d)
    case 2: *a = mu; *b = nu; *c = s; *d = l; break;   // (a b|d c)
    case 3: *a = nu; *b = mu; *c = s; *d = l; break;   // (b a|d c)
    case 4: *a = l; *b = s; *c = mu; *d = nu; break;   // (c d|a b)
    case 5: *a = l; *b = s; *c = nu; *d = mu; break;   // (d c|a b)
    case 6: *a = s; *b = l; *c = mu; *d = nu; break;   // (c d|b a)
    default: *a = s; *b = l; *c = nu; *d = mu; break;  // (d c|b a)
  }
}

__global__ void __launch_bounds__(128) it_coop_kernel(ITParams P, GenClass K, double *gscr) {
  LGB_COOP_PROLOGUE(K)
  const int NA = ncart(K.la), NB = ncart(K.lb), NC = ncart(K.lc), ND = ncart(K.ld);
  const long long nq = (long long)P.nbra * P.nket;
  for (long long q = w0; q < nq; q += wstep) {
    const int bpos = (int)(q / P.nket), kpos = (int)(q % P.nket);
    if (P.triangle && kpos > bpos) continue;
    const int bi = P.bra0 + bpos, ki = P.ket0 + kpos;
    const PairRec &bra = P.pa[bi];
    const PairRec &ket = P.pb[ki];
    if (!abs_above(bra.Q * ket.Q * (1.0 - 1e-9), P.cut)) continue;
    if (P.screen && abs_below(bra.Q * ket.Q * dnorm6(P.Dn, P.nsh, bra.sa, bra.sb, ket.sa, ket.sb), P.eps)) continue;
    eri_coop(g, ct, Lo, K.la, K.lb, K.lc, K.ld, bra, P.pra, ket, P.prb, P.boys.f64, sm);
    const bool ab = bra.sa != bra.sb, cd = ket.sa != ket.sb;
    const bool mirror = P.intra && bi != ki;
    const int f[4] = {bra.fa, bra.fb, ket.fa, ket.fb};
    const int nn[4] = {NA, NB, NC, ND};
    for (int r = 0; r < 8; ++r) {
      if ((r & 1) && !ab && r < 4) continue;
      if ((r >= 2 && r < 4) && !cd) continue;
      if (r >= 4 && !mirror) continue;
      if ((r == 5 || r == 7) && !cd) continue;
      if ((r == 6 || r == 7) && !ab) continue;
      int qa, qb, qc, qd;
      it_map(r, 0, 1, 2, 3, &qa, &qb, &qc, &qd);   // role index at quartet positions a, b, c, d
      int pos[4];                                    // role index -> quartet position
      pos[qa] = 0;
      pos[qb] = 1;
      pos[qc] = 2;
      pos[qd] = 3;
      const int nmu = nn[pos[0]], nnu = nn[pos[1]], nl = nn[pos[2]], ns = nn[pos[3]];
      const int fmu = f[pos[0]], fnu = f[pos[1]], fl = f[pos[2]], fs = f[pos[3]];
      for (int t = lane; t < nnu * nl * ns; t += 32) {
        const int nu = t / (nl * ns), l = (t / ns) % nl, s = t % ns;
        double acc = 0;
        for (int mu = 0; mu < nmu; ++mu) {
          int a, b, c, d;
          it_map(r, mu, nu, l, s, &a, &b, &c, &d);
          const double v = I[((a * NB + b) * NC + c) * ND + d];
          if (abs_above(v, P.cut)) acc += __ldg(P.Cs + fmu + mu) * v;
        }
        atomicAdd(P.A + ((size_t)(fnu + nu) * P.nB + fl + l) * P.nB + fs + s, acc);
      }
    }
  }
}

// ------------------------------------------------------ MP2 transform input --
__global__ void __launch_bounds__(128) mp2x_coop_kernel(MXParams P, GenClass K, double *gscr) {
  LGB_COOP_PROLOGUE(K)
  const int NB = ncart(K.lb), NC = ncart(K.lc), ND = ncart(K.ld), NA = ncart(K.la);
  const long long nq = (long long)P.nbra * P.nket;
  for (long long q = w0; q < nq; q += wstep) {
    const int bi = P.bra0 + (int)(q / P.nket), ki = P.ket0 + (int)(q % P.nket);
    const PairRec &bra = P.pairs[bi];
    const PairRec &ket = P.kpairs[ki];
    if (!abs_above(bra.Q * ket.Q * (1.0 - 1e-9), P.cut)) continue;
    if (P.screen && abs_below(bra.Q * ket.Q * dnorm6(P.Dn, P.nsh, bra.sa, bra.sb, ket.sa, ket.sb), P.eps)) continue;
    eri_coop(g, ct, Lo, K.la, K.lb, K.lc, K.ld, bra, P.prims, ket, P.kprims, P.boys.f64, sm);
    const int col0 = __ldg(P.colbase + ki) - P.col_first;
    const bool two = bra.sa != bra.sb;
    const size_t n = P.n, ncol = P.ncol;
    for (int t = lane; t < NA * NB * NC * ND; t += 32) {
      const int a = t / (NB * NC * ND), b = (t / (NC * ND)) % NB, c = (t / ND) % NC, d = t % ND;
      const double v = I[t];
      if (!abs_above(v, P.cut)) continue;
      const size_t col = col0 + c * ND + d;
      if (P.X) {
        P.X[((bra.fa + a) * ncol + col) * n + bra.fb + b] = v;
        if (two) P.X[((bra.fb + b) * ncol + col) * n + bra.fa + a] = v;
      } else {
        // Xt[col * Kp + nu][mu] and the mirrored bra orientation
        __nv_bfloat16 pc[kMaxPieces];
        bf16_pieces((float)v, P.np, pc);   // three pieces hold the FP32 value exactly
        const size_t kp = P.Kp;
        const size_t j1 = (col * kp + bra.fb + b) * kp + bra.fa + a;
        const size_t j2 = (col * kp + bra.fa + a) * kp + bra.fb + b;
        for (int k = 0; k < P.np; ++k) {
          P.Xp[k][j1] = pc[k];
          if (two) P.Xp[k][j2] = pc[k];
        }
      }
    }
  }
}

// ----------------------------------------------------------------- Schwarz --
__global__ void __launch_bounds__(128) schwarz_coop_kernel(SchwarzParams P, GenClass K, double *gscr) {
  LGB_COOP_PROLOGUE(K)
  const int N = ncart(K.la) * ncart(K.lb);
  for (long long t = w0; t < P.np; t += wstep) {
    const PairRec &pr = P.pairs[P.p0 + t];
    eri_coop(g, ct, Lo, K.la, K.lb, K.la, K.lb, pr, P.prims, pr, P.prims, P.boys.f64, sm);
    if (lane == 0) {
      double m = 0;
      for (int i = 0; i < N; ++i) m = fmax(m, fabs(I[i * N + i]));
      P.Q[P.p0 + t] = sqrt(m);
    }
  }
}

using SZFn = void (*)(SchwarzParams);
const SZFn kSZ[5] = {&schwarz_kernel<0, 0>, &schwarz_kernel<1, 0>, &schwarz_kernel<1, 1>, &schwarz_kernel<2, 0>,
                     &schwarz_kernel<2, 1>};

GenClass gen_class(int pcb, int pck) { return GenClass{pc_la(pcb), pc_lb(pcb), pc_la(pck), pc_lb(pck)}; }

template <typename F>
cudaError_t coop_attr(F *fn) {
  return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, kCoMaxSmem);
}

bool coop_ready() {
  static PerDeviceLevel done;
  return done.raise(1, [] {
           cudaError_t e = coop_attr(jk_coop_kernel);
           if (e == cudaSuccess) e = coop_attr(cp_coop_kernel);
           if (e == cudaSuccess) e = coop_attr(it_coop_kernel);
           if (e == cudaSuccess) e = coop_attr(mp2x_coop_kernel);
           if (e == cudaSuccess) e = coop_attr(schwarz_coop_kernel);
           if (e == cudaSuccess) e = coop_attr(g12_coop_kernel);
           return e;
         }) == cudaSuccess;
}

// launch shape of a cooperative kernel for class K: warps per CTA (each with
// its class-sized work arrays), dynamic shared memory, grid over `units`; a
// class whose arrays exceed kCoMaxSmem runs one warp per CTA on global
// scratch (`scratch` doubles, allocated on the stream for the launch)
struct CoopShape {
  dim3 grid, block;
  size_t smem;
  size_t scratch;
};
CoopShape coop_shape(const GenClass &K, long long units) {
  const size_t per = (size_t)co_layout(K.la, K.lb, K.lc, K.ld).total * sizeof(double);
  if (per > (size_t)kCoMaxSmem) {
    const long long ctas = std::max<long long>(1, std::min<long long>(units, 152LL * 4));
    return CoopShape{dim3((unsigned)ctas), dim3(32u), 0, (size_t)ctas * per / sizeof(double)};
  }
  int w = (int)std::min<size_t>(4, kCoMaxSmem / per);
  if (w < 1) w = 1;
  const long long ctas = std::max<long long>(1, std::min<long long>((units + w - 1) / w, 152LL * 16));
  return CoopShape{dim3((unsigned)ctas), dim3((unsigned)(32 * w)), per * w, 0};
}

// launches kernel `f` with shape c on stream s, with its global scratch when
// the shape asks for one (stream-ordered allocation, freed after the launch)
template <typename F, typename... Args>
cudaError_t coop_launch(F f, const CoopShape &c, cudaStream_t s, Args... args) {
  double *scr = nullptr;
  if (c.scratch) {
    const cudaError_t e = cudaMallocAsync((void **)&scr, c.scratch * sizeof(double), s);
    if (e != cudaSuccess) return e;
  }
  f<<<c.grid, c.block, c.smem, s>>>(args..., scr);
  cudaError_t e = cudaGetLastError();
  if (scr) {
    const cudaError_t e2 = cudaFreeAsync(scr, s);
    if (e == cudaSuccess) e = e2;
  }
  return e;
}

}  // namespace

bool class_supported(int pcb, int pck) {
  return pcb >= 0 && pck >= 0 && pcb < kNumPairClasses && pck < kNumPairClasses;
}

bool jk_rows_used(int pcb, int pck, int n, int nsh) {
  if (!class_supported(pcb, pck) || !kJKR[pcb][pck]) return false;
  if (row_rows_off()) return false;
  return row_smem_bytes(ncart(pc_la(pcb)) + ncart(pc_lb(pcb)), n, nsh) <= (size_t)kRowMaxSmem;
}

cudaError_t launch_jk_tasks(int pcb, int pck, bool fp32, const JKTask *dtasks, const TaskLaunch &tl,
                            cudaStream_t s) {
  if (!class_supported(pcb, pck)) return cudaErrorNotSupported;
  if (tl.ntasks <= 0 || tl.nblocks <= 0) return cudaSuccess;
  if (fp32 && tl.mixed && tl.lower && tl.rows_pref != 0 && jk_rows_used(pcb, pck, tl.rows_n, tl.rows_nsh)) {
    // the FP32 half of a mixed build: bra-row kernel
    const JKFn r = kJKR[pcb][pck];
    const size_t smem = row_smem_bytes(ncart(pc_la(pcb)) + ncart(pc_lb(pcb)), tl.rows_n, tl.rows_nsh);
    static PerDeviceLevel attr[kNumPairClasses][kNumPairClasses];
    if (smem > 48 * 1024) {
      const cudaError_t e = attr[pcb][pck].raise((long long)smem, [r, smem] {
        return cudaFuncSetAttribute(r, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      });
      if (e != cudaSuccess) return e;
    }
    if (tl.nrblocks > 0) r<<<tl.nrblocks, 32 * kRowWarps, smem, s>>>(dtasks, tl);
    count_launches(1);
    return cudaGetLastError();
  }
  const JKFn f = fp32 ? kJK32[pcb][pck] : kJK64[pcb][pck];
  if (f) {
    f<<<tl.nblocks, kBlock, 0, s>>>(dtasks, tl);
  } else {
    if (!coop_ready()) return cudaErrorInvalidValue;
    const GenClass K = gen_class(pcb, pck);
    const CoopShape c = coop_shape(K, (long long)tl.nblocks * kCoUnitsPerTile);
    const cudaError_t e = coop_launch(jk_coop_kernel, c, s, dtasks, tl, K);
    if (e != cudaSuccess) return e;
  }
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_cp_tasks(int pcb, int pck, bool fp32, const CPTask *dtasks, const TaskLaunch &tl,
                            cudaStream_t s) {
  if (!class_supported(pcb, pck)) return cudaErrorNotSupported;
  if (tl.ntasks <= 0 || tl.nblocks <= 0) return cudaSuccess;
  const CPFn f = fp32 ? kCP32[pcb][pck] : kCP64[pcb][pck];
  if (f) {
    f<<<tl.nblocks, kBlock, 0, s>>>(dtasks, tl);
  } else {
    if (!coop_ready()) return cudaErrorInvalidValue;
    const GenClass K = gen_class(pcb, pck);
    const CoopShape c = coop_shape(K, (long long)tl.nblocks * kCoUnitsPerTile);
    const cudaError_t e = coop_launch(cp_coop_kernel, c, s, dtasks, tl, K);
    if (e != cudaSuccess) return e;
  }
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_it(int pcb, int pck, const ITParams &p, cudaStream_t s) {
  if (!class_supported(pcb, pck)) return cudaErrorNotSupported;
  if (p.nbra <= 0 || p.nket <= 0) return cudaSuccess;
  const ITFn f = kIT[pcb][pck];
  if (f) {
    const dim3 grid((unsigned)((p.nket + 31) / 32), (unsigned)((p.nbra + kWarpsPerBlock - 1) / kWarpsPerBlock));
    f<<<grid, kBlock, 0, s>>>(p);
  } else {
    if (!coop_ready()) return cudaErrorInvalidValue;
    const GenClass K = gen_class(pcb, pck);
    const CoopShape c = coop_shape(K, (long long)p.nbra * p.nket);
    const cudaError_t e = coop_launch(it_coop_kernel, c, s, p, K);
    if (e != cudaSuccess) return e;
  }
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_mp2x(int pcb, int pck, const MXParams &p, cudaStream_t s) {
  if (!class_supported(pcb, pck)) return cudaErrorNotSupported;
  if (p.nbra <= 0 || p.nket <= 0) return cudaSuccess;
  const MXFn f = kMX[pcb][pck];
  if (f) {
    const dim3 grid((unsigned)((p.nket + 31) / 32), (unsigned)((p.nbra + kWarpsPerBlock - 1) / kWarpsPerBlock));
    f<<<grid, kBlock, 0, s>>>(p);
  } else {
    if (!coop_ready()) return cudaErrorInvalidValue;
    const GenClass K = gen_class(pcb, pck);
    const CoopShape c = coop_shape(K, (long long)p.nbra * p.nket);
    const cudaError_t e = coop_launch(mp2x_coop_kernel, c, s, p, K);
    if (e != cudaSuccess) return e;
  }
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_g12(int pcb, int pck, const G12Params &p, cudaStream_t s) {
  if (!class_supported(pcb, pck) || !p.gem) return cudaErrorNotSupported;
  if (p.nbra <= 0 || p.nket <= 0) return cudaSuccess;
  if (!coop_ready()) return cudaErrorInvalidValue;
  const GenClass K = gen_class(pcb, pck);
  const CoopShape c = coop_shape(K, (long long)p.nbra * p.nket);
  const cudaError_t e = coop_launch(g12_coop_kernel, c, s, p, K);
  if (e != cudaSuccess) return e;
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_schwarz(int pc, const SchwarzParams &p, cudaStream_t s) {
  if (pc < 0 || pc >= kNumPairClasses) return cudaErrorNotSupported;
  if (p.np <= 0) return cudaSuccess;
  if (2 * pc_L(pc) <= kTemplatedMaxL) {
    kSZ[pc]<<<(p.np + 127) / 128, 128, 0, s>>>(p);
  } else {
    if (!coop_ready()) return cudaErrorInvalidValue;
    const GenClass K{pc_la(pc), pc_lb(pc), pc_la(pc), pc_lb(pc)};
    const CoopShape c = coop_shape(K, p.np);
    const cudaError_t e = coop_launch(schwarz_coop_kernel, c, s, p, K);
    if (e != cudaSuccess) return e;
  }
  count_launches(1);
  return cudaGetLastError();
}

}  // namespace lgb
