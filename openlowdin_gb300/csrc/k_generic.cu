// Generic (runtime-class) kernels for the quartet classes of total angular
// momentum 7 and 8, the Schwarz kernels, and the dispatch of every class to its
// templated or generic kernel.
//
// The generic kernels run a fixed grid of kGenericBlocks persistent blocks;
// block g owns scratch slots g*128 .. g*128+127 and walks the tiles g,
// g + kGenericBlocks, ... of the task list, so every running thread has its own
// work arrays.  They compute in FP64 (also when a mixed launch asks for the FP32
// half: the split decides which quartets a launch takes, the generic kernel
// evaluates them in FP64 and accumulates into the FP64 arrays).
#include "eri_generic.cuh"
#include "fock_kernels.cuh"

namespace lgb {

extern const JKFn kJK64_0[6], kJK64_1[6], kJK64_2[6], kJK64_3[6], kJK64_4[6], kJK64_5[6];
extern const JKFn kJK32_0[6], kJK32_1[6], kJK32_2[6], kJK32_3[6], kJK32_4[6], kJK32_5[6];
extern const CPFn kCP64_0[6], kCP64_1[6], kCP64_2[6], kCP64_3[6], kCP64_4[6], kCP64_5[6];
extern const CPFn kCP32_0[6], kCP32_1[6], kCP32_2[6], kCP32_3[6], kCP32_4[6], kCP32_5[6];
extern const ITFn kIT_0[6], kIT_1[6], kIT_2[6], kIT_3[6], kIT_4[6], kIT_5[6];
extern const MXFn kMX_0[6], kMX_1[6], kMX_2[6], kMX_3[6], kMX_4[6], kMX_5[6];

namespace {

const JKFn *const kJK64[6] = {kJK64_0, kJK64_1, kJK64_2, kJK64_3, kJK64_4, kJK64_5};
const JKFn *const kJK32[6] = {kJK32_0, kJK32_1, kJK32_2, kJK32_3, kJK32_4, kJK32_5};
const CPFn *const kCP64[6] = {kCP64_0, kCP64_1, kCP64_2, kCP64_3, kCP64_4, kCP64_5};
const CPFn *const kCP32[6] = {kCP32_0, kCP32_1, kCP32_2, kCP32_3, kCP32_4, kCP32_5};
const ITFn *const kIT[6] = {kIT_0, kIT_1, kIT_2, kIT_3, kIT_4, kIT_5};
const MXFn *const kMX[6] = {kMX_0, kMX_1, kMX_2, kMX_3, kMX_4, kMX_5};

const dim3 kBlock(32, kWarpsPerBlock);

struct GenClass {
  int la, lb, lc, ld;
};

__device__ __forceinline__ double *thread_scratch(double *scratch, size_t *stride) {
  *stride = (size_t)gridDim.x * kGenericThreads;
  return scratch + (size_t)blockIdx.x * kGenericThreads + threadIdx.y * 32 + threadIdx.x;
}

// ------------------------------------------------------------------ J/K --
__global__ void __launch_bounds__(128) jk_generic_kernel(const JKTask *__restrict__ tasks, TaskLaunch TL, GenClass K) {
  size_t stride;
  double *scr = thread_scratch(TL.scratch, &stride);
  const int NA = ncart(K.la), NB = ncart(K.lb), NC = ncart(K.lc), ND = ncart(K.ld);
  const Strided I{scr + (size_t)(kGenScratch - kGenOut) * stride, stride};
  for (int blk = blockIdx.x; blk < TL.nblocks; blk += gridDim.x) {
    const int t = find_task(tasks, TL.ntasks, blk);
    const JKTask &T = tasks[t];
    const int local = blk - T.blk0;
    const int tx = local % T.nbx, ty = local / T.nbx;
    if (T.triangle && tx * 32 > ty * kWarpsPerBlock + kWarpsPerBlock - 1) continue;
    const int kpos = tx * 32 + threadIdx.x;
    const int bpos = ty * kWarpsPerBlock + threadIdx.y;
    if (bpos >= T.nbra) continue;  // warp-uniform
    bool active = kpos < T.nket && (!T.triangle || kpos <= bpos);
    const int bi = T.bra0 + bpos;
    const int ki = T.ket0 + min(kpos, T.nket - 1);
    const PairRec &bra = T.pairs[bi];
    const PairRec ket = T.pairs[ki];
    if (TL.split > 0.0) {
      float b = T.pairs32[bi].Q * T.pairs32[ki].Q;
      if (T.screen) {
        b *= dnorm6(T.Dn32, T.nsh, bra.sa, bra.sb, ket.sa, ket.sb);
        if (b < (float)TL.eps) active = false;
      }
      if (TL.lower ? !(b < (float)TL.split) : (b < (float)TL.split)) active = false;
    } else if (T.screen) {
      const double b = bra.Q * ket.Q * dnorm6(T.Dn, T.nsh, bra.sa, bra.sb, ket.sa, ket.sb);
      if (b < TL.eps) active = false;
    }
    if (__all_sync(0xffffffffu, !active)) continue;
    if (T.count) {
      const unsigned cnt = __popc(__ballot_sync(0xffffffffu, active));
      if (threadIdx.x == 0) atomicAdd(T.count, (unsigned long long)cnt);
    }
    if (active) eri_generic(K.la, K.lb, K.lc, K.ld, bra, T.prims, ket, T.prims, TL.boys.f64, scr, stride, 0);
    const double deg = active ? (bra.sa == bra.sb ? 1 : 2) * (ket.sa == ket.sb ? 1 : 2) * (bi == ki ? 1 : 2) : 0.0;
    const double hdeg = deg * T.hf;
    const double *__restrict__ D = T.Ds;
    const int n = T.n;
    double *G = T.Gacc;
    const int fa = bra.fa, fb = bra.fb, fc = ket.fa, fd = ket.fb;
    auto Iat = [&](int a, int b, int c, int d) -> double { return active ? I[((a * NB + b) * NC + c) * ND + d] : 0.0; };
    for (int a = 0; a < NA; ++a)
      for (int b = 0; b < NB; ++b) {
        double s = 0;
        for (int c = 0; c < NC; ++c)
          for (int d = 0; d < ND; ++d) s += __ldg(D + (fc + c) * n + fd + d) * Iat(a, b, c, d);
        s = warp_sum(s * deg);
        if (threadIdx.x == 0) atomicAdd(G + (size_t)(fa + a) * n + fb + b, s);
      }
    if (!active) continue;
    for (int c = 0; c < NC; ++c)
      for (int d = 0; d < ND; ++d) {
        double s = 0;
        for (int a = 0; a < NA; ++a)
          for (int b = 0; b < NB; ++b) s += __ldg(D + (fa + a) * n + fb + b) * Iat(a, b, c, d);
        atomicAdd(G + (size_t)(fc + c) * n + fd + d, s * deg);
      }
    for (int a = 0; a < NA; ++a)
      for (int c = 0; c < NC; ++c) {
        double s = 0;
        for (int b = 0; b < NB; ++b)
          for (int d = 0; d < ND; ++d) s += __ldg(D + (fb + b) * n + fd + d) * Iat(a, b, c, d);
        atomicAdd(G + (size_t)(fa + a) * n + fc + c, s * hdeg);
      }
    for (int b = 0; b < NB; ++b)
      for (int d = 0; d < ND; ++d) {
        double s = 0;
        for (int a = 0; a < NA; ++a)
          for (int c = 0; c < NC; ++c) s += __ldg(D + (fa + a) * n + fc + c) * Iat(a, b, c, d);
        atomicAdd(G + (size_t)(fb + b) * n + fd + d, s * hdeg);
      }
    for (int a = 0; a < NA; ++a)
      for (int d = 0; d < ND; ++d) {
        double s = 0;
        for (int b = 0; b < NB; ++b)
          for (int c = 0; c < NC; ++c) s += __ldg(D + (fb + b) * n + fc + c) * Iat(a, b, c, d);
        atomicAdd(G + (size_t)(fa + a) * n + fd + d, s * hdeg);
      }
    for (int b = 0; b < NB; ++b)
      for (int c = 0; c < NC; ++c) {
        double s = 0;
        for (int a = 0; a < NA; ++a)
          for (int d = 0; d < ND; ++d) s += __ldg(D + (fa + a) * n + fd + d) * Iat(a, b, c, d);
        atomicAdd(G + (size_t)(fb + b) * n + fc + c, s * hdeg);
      }
  }
}

// ------------------------------------------------------------- coupling --
__global__ void __launch_bounds__(128) cp_generic_kernel(const CPTask *__restrict__ tasks, TaskLaunch TL, GenClass K) {
  size_t stride;
  double *scr = thread_scratch(TL.scratch, &stride);
  const int NA = ncart(K.la), NB = ncart(K.lb), NC = ncart(K.lc), ND = ncart(K.ld);
  const Strided I{scr + (size_t)(kGenScratch - kGenOut) * stride, stride};
  for (int blk = blockIdx.x; blk < TL.nblocks; blk += gridDim.x) {
    const int t = find_task(tasks, TL.ntasks, blk);
    const CPTask &T = tasks[t];
    const int local = blk - T.blk0;
    const int tx = local % T.nbx, ty = local / T.nbx;
    const int kpos = tx * 32 + threadIdx.x;
    const int bpos = ty * kWarpsPerBlock + threadIdx.y;
    if (bpos >= T.nbra) continue;
    bool active = kpos < T.nket;
    const int bi = T.bra0 + bpos, ki = T.ket0 + min(kpos, T.nket - 1);
    const bool tiny = TL.split > 0.0 ? T.pa32[bi].Q * T.pb32[ki].Q * 0.999f < (float)TL.cut
                                     : T.pa[bi].Q * T.pb[ki].Q * (1.0 - 1e-9) < TL.cut;
    if (tiny) active = false;
    if (TL.split > 0.0) {
      const PairRec32 &b32 = T.pa32[bi];
      const PairRec32 &k32 = T.pb32[ki];
      float dm = 0.f;
      if (T.DnA32) dm = __ldg(T.DnA32 + b32.sa * T.nshA + b32.sb);
      if (T.DnB32) dm = fmaxf(dm, __ldg(T.DnB32 + k32.sa * T.nshB + k32.sb));
      const float b = b32.Q * k32.Q * dm;
      if (TL.lower ? !(b < (float)TL.split) : (b < (float)TL.split)) active = false;
    }
    if (__all_sync(0xffffffffu, !active)) continue;
    if (T.count) {
      const unsigned cnt = __popc(__ballot_sync(0xffffffffu, active));
      if (threadIdx.x == 0) atomicAdd(T.count, (unsigned long long)cnt);
    }
    const PairRec &bra = T.pa[bi];
    const PairRec ket = T.pb[ki];
    if (active) eri_generic(K.la, K.lb, K.lc, K.ld, bra, T.pra, ket, T.prb, TL.boys.f64, scr, stride, 0);
    auto Iat = [&](int a, int b, int c, int d) -> double {
      if (!active) return 0.0;
      const double v = I[((a * NB + b) * NC + c) * ND + d];
      return fabs(v) >= TL.cut ? v : 0.0;
    };
    const int fa = bra.fa, fb = bra.fb, fc = ket.fa, fd = ket.fb;
    const bool abdiff = bra.sa != bra.sb, cddiff = ket.sa != ket.sb;
    if (T.JA) {
      const double wk = active ? (cddiff ? 2.0 : 1.0) * T.scale : 0.0;
      for (int a = 0; a < NA; ++a)
        for (int b = 0; b < NB; ++b) {
          double s = 0;
          for (int c = 0; c < NC; ++c)
            for (int d = 0; d < ND; ++d) s += __ldg(T.DsB + (fc + c) * T.nB + fd + d) * Iat(a, b, c, d);
          s = warp_sum(s * wk);
          if (threadIdx.x == 0) {
            atomicAdd(T.JA + (size_t)(fa + a) * T.nA + fb + b, s);
            if (abdiff) atomicAdd(T.JA + (size_t)(fb + b) * T.nA + fa + a, s);
          }
        }
    }
    if (T.JB && active) {
      const double wb = (abdiff ? 2.0 : 1.0) * T.scale;
      for (int c = 0; c < NC; ++c)
        for (int d = 0; d < ND; ++d) {
          double s = 0;
          for (int a = 0; a < NA; ++a)
            for (int b = 0; b < NB; ++b) s += __ldg(T.DsA + (fa + a) * T.nA + fb + b) * Iat(a, b, c, d);
          s *= wb;
          atomicAdd(T.JB + (size_t)(fc + c) * T.nB + fd + d, s);
          if (cddiff) atomicAdd(T.JB + (size_t)(fd + d) * T.nB + fc + c, s);
        }
    }
  }
}

// -------------------------------------------------------- first quarter --
__device__ __forceinline__ void it_role_rt(const Strided &I, int NA, int NB, int NC, int ND, int roleperm,
                                           const double *__restrict__ Cs, int fmu, int fnu, int fl, int fs, int nmu,
                                           int nnu, int nl, int ns, double *A, int nB, double cut) {
  // roleperm selects how (mu, nu, l, s) map onto the quartet's (a, b, c, d)
  for (int nu = 0; nu < nnu; ++nu)
    for (int l = 0; l < nl; ++l)
      for (int s = 0; s < ns; ++s) {
        double acc = 0;
        for (int mu = 0; mu < nmu; ++mu) {
          int a, b, c, d;
          switch (roleperm) {
            case 0: a = mu; b = nu; c = l; d = s; break;   // (a b|c d)
            case 1: a = nu; b = mu; c = l; d = s; break;   // (b a|c d)
            case 2: a = mu; b = nu; c = s; d = l; break;   // (a b|d c)
            case 3: a = nu; b = mu; c = s; d = l; break;   // (b a|d c)
            case 4: a = l; b = s; c = mu; d = nu; break;   // (c d|a b)
            case 5: a = l; b = s; c = nu; d = mu; break;   // (d c|a b)
            case 6: a = s; b = l; c = mu; d = nu; break;   // (c d|b a)
            default: a = s; b = l; c = nu; d = mu; break;  // (d c|b a)
          }
          const double v = I[((a * NB + b) * NC + c) * ND + d];
          if (fabs(v) > cut) acc += __ldg(Cs + fmu + mu) * v;
        }
        atomicAdd(A + ((size_t)(fnu + nu) * nB + fl + l) * nB + fs + s, acc);
      }
}

__global__ void __launch_bounds__(128) it_generic_kernel(ITParams P, GenClass K) {
  size_t stride;
  double *scr = thread_scratch(P.scratch, &stride);
  const int NA = ncart(K.la), NB = ncart(K.lb), NC = ncart(K.lc), ND = ncart(K.ld);
  const Strided I{scr + (size_t)(kGenScratch - kGenOut) * stride, stride};
  const int nbx = (P.nket + 31) / 32, nby = (P.nbra + kWarpsPerBlock - 1) / kWarpsPerBlock;
  for (int blk = blockIdx.x; blk < nbx * nby; blk += gridDim.x) {
    const int tx = blk % nbx, ty = blk / nbx;
    const int kpos = tx * 32 + threadIdx.x;
    const int bpos = ty * kWarpsPerBlock + threadIdx.y;
    if (bpos >= P.nbra || kpos >= P.nket) continue;
    if (P.triangle && kpos > bpos) continue;
    const int bi = P.bra0 + bpos, ki = P.ket0 + kpos;
    const PairRec bra = P.pa[bi];
    const PairRec ket = P.pb[ki];
    if (bra.Q * ket.Q * (1.0 - 1e-9) <= P.cut) continue;
    if (P.screen && bra.Q * ket.Q * dnorm6(P.Dn, P.nsh, bra.sa, bra.sb, ket.sa, ket.sb) < P.eps) continue;
    eri_generic(K.la, K.lb, K.lc, K.ld, bra, P.pra, ket, P.prb, P.boys.f64, scr, stride, 0);
    const bool ab = bra.sa != bra.sb, cd = ket.sa != ket.sb;
    const int fa = bra.fa, fb = bra.fb, fc = ket.fa, fd = ket.fb;
    it_role_rt(I, NA, NB, NC, ND, 0, P.Cs, fa, fb, fc, fd, NA, NB, NC, ND, P.A, P.nB, P.cut);
    if (ab) it_role_rt(I, NA, NB, NC, ND, 1, P.Cs, fb, fa, fc, fd, NB, NA, NC, ND, P.A, P.nB, P.cut);
    if (cd) it_role_rt(I, NA, NB, NC, ND, 2, P.Cs, fa, fb, fd, fc, NA, NB, ND, NC, P.A, P.nB, P.cut);
    if (ab && cd) it_role_rt(I, NA, NB, NC, ND, 3, P.Cs, fb, fa, fd, fc, NB, NA, ND, NC, P.A, P.nB, P.cut);
    if (P.intra && bi != ki) {
      it_role_rt(I, NA, NB, NC, ND, 4, P.Cs, fc, fd, fa, fb, NC, ND, NA, NB, P.A, P.nB, P.cut);
      if (cd) it_role_rt(I, NA, NB, NC, ND, 5, P.Cs, fd, fc, fa, fb, ND, NC, NA, NB, P.A, P.nB, P.cut);
      if (ab) it_role_rt(I, NA, NB, NC, ND, 6, P.Cs, fc, fd, fb, fa, NC, ND, NB, NA, P.A, P.nB, P.cut);
      if (ab && cd) it_role_rt(I, NA, NB, NC, ND, 7, P.Cs, fd, fc, fb, fa, ND, NC, NB, NA, P.A, P.nB, P.cut);
    }
  }
}

// ------------------------------------------------------ MP2 transform input --
__global__ void __launch_bounds__(128) mp2x_generic_kernel(MXParams P, GenClass K) {
  size_t stride;
  double *scr = thread_scratch(P.scratch, &stride);
  const int NB = ncart(K.lb), NC = ncart(K.lc), ND = ncart(K.ld), NA = ncart(K.la);
  const Strided I{scr + (size_t)(kGenScratch - kGenOut) * stride, stride};
  const int nbx = (P.nket + 31) / 32, nby = (P.nbra + kWarpsPerBlock - 1) / kWarpsPerBlock;
  for (int blk = blockIdx.x; blk < nbx * nby; blk += gridDim.x) {
    const int tx = blk % nbx, ty = blk / nbx;
    const int kpos = tx * 32 + threadIdx.x;
    const int bpos = ty * kWarpsPerBlock + threadIdx.y;
    if (bpos >= P.nbra || kpos >= P.nket) continue;
    const int bi = P.bra0 + bpos, ki = P.ket0 + kpos;
    const PairRec bra = P.pairs[bi];
    const PairRec ket = P.pairs[ki];
    if (bra.Q * ket.Q * (1.0 - 1e-9) <= P.cut) continue;
    if (P.screen && bra.Q * ket.Q * dnorm6(P.Dn, P.nsh, bra.sa, bra.sb, ket.sa, ket.sb) < P.eps) continue;
    eri_generic(K.la, K.lb, K.lc, K.ld, bra, P.prims, ket, P.prims, P.boys.f64, scr, stride, 0);
    const int col0 = __ldg(P.colbase + ki) - P.col_first;
    const bool two = bra.sa != bra.sb;
    const size_t n = P.n, ncol = P.ncol;
    for (int a = 0; a < NA; ++a)
      for (int b = 0; b < NB; ++b)
        for (int c = 0; c < NC; ++c)
          for (int d = 0; d < ND; ++d) {
            const double v = I[((a * NB + b) * NC + c) * ND + d];
            if (!(fabs(v) > P.cut)) continue;
            const size_t col = col0 + c * ND + d;
            const size_t i1 = ((bra.fa + a) * ncol + col) * n + bra.fb + b;
            const size_t i2 = ((bra.fb + b) * ncol + col) * n + bra.fa + a;
            if (P.X) {
              P.X[i1] = v;
              if (two) P.X[i2] = v;
            } else {
              // Xt[col * Kp + nu][mu] and the mirrored bra orientation
              __nv_bfloat16 pc[kMaxPieces];
              bf16_pieces(v, P.np, pc);
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
__global__ void __launch_bounds__(128) schwarz_generic_kernel(SchwarzParams P, int la, int lb) {
  size_t stride;
  double *scr = thread_scratch(P.scratch, &stride);
  const Strided I{scr + (size_t)(kGenScratch - kGenOut) * stride, stride};
  const int N = ncart(la) * ncart(lb);
  for (int t = blockIdx.x * kGenericThreads + threadIdx.y * 32 + threadIdx.x; t < P.np;
       t += gridDim.x * kGenericThreads) {
    const PairRec pr = P.pairs[P.p0 + t];
    eri_generic(la, lb, la, lb, pr, P.prims, pr, P.prims, P.boys.f64, scr, stride, 0);
    double m = 0;
    for (int i = 0; i < N; ++i) m = fmax(m, fabs(I[i * N + i]));
    P.Q[P.p0 + t] = sqrt(m);
  }
}

using SZFn = void (*)(SchwarzParams);
const SZFn kSZ[5] = {&schwarz_kernel<0, 0>, &schwarz_kernel<1, 0>, &schwarz_kernel<1, 1>, &schwarz_kernel<2, 0>,
                     &schwarz_kernel<2, 1>};

GenClass gen_class(int pcb, int pck) { return GenClass{pc_la(pcb), pc_lb(pcb), pc_la(pck), pc_lb(pck)}; }

}  // namespace

int generic_scratch_doubles() { return kGenScratch; }

bool class_supported(int pcb, int pck) {
  return pcb >= 0 && pck >= 0 && pcb < kNumPairClasses && pck < kNumPairClasses;
}

cudaError_t launch_jk_tasks(int pcb, int pck, bool fp32, const JKTask *dtasks, const TaskLaunch &tl,
                            cudaStream_t s) {
  if (!class_supported(pcb, pck)) return cudaErrorNotSupported;
  if (tl.ntasks <= 0 || tl.nblocks <= 0) return cudaSuccess;
  const JKFn f = fp32 ? kJK32[pcb][pck] : kJK64[pcb][pck];
  if (f) {
    f<<<tl.nblocks, kBlock, 0, s>>>(dtasks, tl);
  } else {
    if (!tl.scratch) return cudaErrorInvalidValue;
    jk_generic_kernel<<<kGenericBlocks, kBlock, 0, s>>>(dtasks, tl, gen_class(pcb, pck));
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
    if (!tl.scratch) return cudaErrorInvalidValue;
    cp_generic_kernel<<<kGenericBlocks, kBlock, 0, s>>>(dtasks, tl, gen_class(pcb, pck));
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
    if (!p.scratch) return cudaErrorInvalidValue;
    it_generic_kernel<<<kGenericBlocks, kBlock, 0, s>>>(p, gen_class(pcb, pck));
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
    if (!p.scratch) return cudaErrorInvalidValue;
    mp2x_generic_kernel<<<kGenericBlocks, kBlock, 0, s>>>(p, gen_class(pcb, pck));
  }
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_schwarz(int pc, const SchwarzParams &p, cudaStream_t s) {
  if (pc < 0 || pc >= kNumPairClasses) return cudaErrorNotSupported;
  if (p.np <= 0) return cudaSuccess;
  if (pc < 5) {
    kSZ[pc]<<<(p.np + 127) / 128, 128, 0, s>>>(p);
  } else {
    if (!p.scratch) return cudaErrorInvalidValue;
    schwarz_generic_kernel<<<kGenericBlocks, kBlock, 0, s>>>(p, pc_la(pc), pc_lb(pc));
  }
  count_launches(1);
  return cudaGetLastError();
}

}  // namespace lgb
