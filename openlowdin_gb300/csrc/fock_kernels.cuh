// Kernel templates: Schwarz factors, intra-species J/K, fused inter-species
// coupling and first-quarter transforms.  Included by the translation units
// that instantiate them for a set of quartet classes.
#pragma once
#include "eri.cuh"
#include "kernels.cuh"

namespace lgb {

template <typename R>
__device__ __forceinline__ R warp_sum(R v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ double dnorm6(const double *__restrict__ Dn, int nsh, int a, int b, int c, int d) {
  double m = __ldg(Dn + a * nsh + b);
  m = fmax(m, __ldg(Dn + a * nsh + c));
  m = fmax(m, __ldg(Dn + b * nsh + c));
  m = fmax(m, __ldg(Dn + a * nsh + d));
  m = fmax(m, __ldg(Dn + b * nsh + d));
  m = fmax(m, __ldg(Dn + c * nsh + d));
  return m;
}

// task owning flattened block b: last task with blk0 <= b (tasks sorted by blk0)
template <typename T>
__device__ __forceinline__ int find_task(const T *__restrict__ tasks, int ntasks, int b) {
  int lo = 0, hi = ntasks - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(&tasks[mid].blk0) <= b) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// ----------------------------------------------------------------- Schwarz --
template <int LA, int LB>
__global__ void __launch_bounds__(128) schwarz_kernel(SchwarzParams P) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= P.np) return;
  const PairRec pr = P.pairs[P.p0 + t];
  constexpr int N = ncart(LA) * ncart(LB);
  double I[N * N];
  eri_quartet<double, LA, LB, LA, LB>(pr, P.prims, pr, P.prims, P.boys.f64, P.boys.f32, I);
  double m = 0;
#pragma unroll
  for (int i = 0; i < N; ++i) m = fmax(m, fabs(I[i * N + i]));
  P.Q[P.p0 + t] = sqrt(m);
}

// --------------------------------------------------------------------- J/K --
// Lane x of warp y in a block evaluates quartet (bra = tile_y*4 + y, ket =
// tile_x*32 + x) of its task.  The 32 lanes of a warp share the bra pair, so the
// bra-block Coulomb term is reduced across the warp before its atomics.
// Digestion follows the six updates of a permutation-unique quartet
// (g12 += D34 v, g34 += D12 v, g13/g24/g14/g23 += 0.5 f D v, all x degeneracy);
// with G = (Gacc + Gacc^T)/4 this is J[D] + f K[D].
template <typename R, int LA, int LB, int LC, int LD>
__global__ void __launch_bounds__(128) jk_tasks_kernel(const JKTask *__restrict__ tasks, TaskLaunch TL) {
  using Q = QClass<LA, LB, LC, LD>;
  constexpr int NA = Q::NA, NB = Q::NB, NC = Q::NC, ND = Q::ND;
  const int t = find_task(tasks, TL.ntasks, blockIdx.x);
  const JKTask &T = tasks[t];
  const int local = blockIdx.x - T.blk0;
  const int tx = local % T.nbx, ty = local / T.nbx;
  if (T.triangle && tx * 32 > ty * kWarpsPerBlock + kWarpsPerBlock - 1) return;
  const int kpos = tx * 32 + threadIdx.x;
  const int bpos = ty * kWarpsPerBlock + threadIdx.y;
  if (bpos >= T.nbra) return;  // warp-uniform
  bool active = kpos < T.nket && (!T.triangle || kpos <= bpos);
  const int bi = T.bra0 + bpos;
  const int ki = T.ket0 + min(kpos, T.nket - 1);
  const PairRec &bra = T.pairs[bi];
  const PairRec ket = T.pairs[ki];
  double bound = bra.Q * ket.Q;
  if (T.screen) {
    bound *= dnorm6(T.Dn, T.nsh, bra.sa, bra.sb, ket.sa, ket.sb);
    if (bound < TL.eps) active = false;
  }
  if (TL.split > 0.0) {
    if (TL.lower ? !(bound < TL.split) : (bound < TL.split)) active = false;
  }
  if (__all_sync(0xffffffffu, !active)) return;
  if (T.count) {
    const unsigned cnt = __popc(__ballot_sync(0xffffffffu, active));
    if (threadIdx.x == 0) atomicAdd(T.count, (unsigned long long)cnt);
  }
  R I[Q::NINT];
  if (active) {
    eri_quartet<R, LA, LB, LC, LD>(bra, T.prims, ket, T.prims, TL.boys.f64, TL.boys.f32, I);
  } else {
#pragma unroll
    for (int x = 0; x < Q::NINT; ++x) I[x] = R(0);
  }
  const R deg = active ? R((bra.sa == bra.sb ? 1 : 2) * (ket.sa == ket.sb ? 1 : 2) * (bi == ki ? 1 : 2)) : R(0);
  const R hdeg = deg * R(T.hf);
  const double *__restrict__ D = T.Ds;
  const int n = T.n;
  double *G = T.Gacc;
  const int fa = bra.fa, fb = bra.fb, fc = ket.fa, fd = ket.fb;
  auto Iat = [&](int a, int b, int c, int d) -> R { return I[((a * NB + b) * NC + c) * ND + d]; };
  // J12: bra block, warp-reduced
#pragma unroll
  for (int a = 0; a < NA; ++a)
#pragma unroll
    for (int b = 0; b < NB; ++b) {
      R s = 0;
#pragma unroll
      for (int c = 0; c < NC; ++c)
#pragma unroll
        for (int d = 0; d < ND; ++d) s += R(__ldg(D + (fc + c) * n + fd + d)) * Iat(a, b, c, d);
      s = warp_sum(s * deg);
      if (threadIdx.x == 0) atomicAdd(G + (fa + a) * n + fb + b, double(s));
    }
  if (!active) return;
  // J34
#pragma unroll
  for (int c = 0; c < NC; ++c)
#pragma unroll
    for (int d = 0; d < ND; ++d) {
      R s = 0;
#pragma unroll
      for (int a = 0; a < NA; ++a)
#pragma unroll
        for (int b = 0; b < NB; ++b) s += R(__ldg(D + (fa + a) * n + fb + b)) * Iat(a, b, c, d);
      atomicAdd(G + (fc + c) * n + fd + d, double(s * deg));
    }
  // K13 (i,k) += D(j,l)
#pragma unroll
  for (int a = 0; a < NA; ++a)
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      R s = 0;
#pragma unroll
      for (int b = 0; b < NB; ++b)
#pragma unroll
        for (int d = 0; d < ND; ++d) s += R(__ldg(D + (fb + b) * n + fd + d)) * Iat(a, b, c, d);
      atomicAdd(G + (fa + a) * n + fc + c, double(s * hdeg));
    }
  // K24 (j,l) += D(i,k)
#pragma unroll
  for (int b = 0; b < NB; ++b)
#pragma unroll
    for (int d = 0; d < ND; ++d) {
      R s = 0;
#pragma unroll
      for (int a = 0; a < NA; ++a)
#pragma unroll
        for (int c = 0; c < NC; ++c) s += R(__ldg(D + (fa + a) * n + fc + c)) * Iat(a, b, c, d);
      atomicAdd(G + (fb + b) * n + fd + d, double(s * hdeg));
    }
  // K14 (i,l) += D(j,k)
#pragma unroll
  for (int a = 0; a < NA; ++a)
#pragma unroll
    for (int d = 0; d < ND; ++d) {
      R s = 0;
#pragma unroll
      for (int b = 0; b < NB; ++b)
#pragma unroll
        for (int c = 0; c < NC; ++c) s += R(__ldg(D + (fb + b) * n + fc + c)) * Iat(a, b, c, d);
      atomicAdd(G + (fa + a) * n + fd + d, double(s * hdeg));
    }
  // K23 (j,k) += D(i,l)
#pragma unroll
  for (int b = 0; b < NB; ++b)
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      R s = 0;
#pragma unroll
      for (int a = 0; a < NA; ++a)
#pragma unroll
        for (int d = 0; d < ND; ++d) s += R(__ldg(D + (fa + a) * n + fd + d)) * Iat(a, b, c, d);
      atomicAdd(G + (fb + b) * n + fc + c, double(s * hdeg));
    }
}

// ---------------------------------------------------------------- coupling --
// Bra pairs of species A (every unordered shell pair), ket pairs of species B.
// J_A[i][j] += scale sum_{kl} D_B[k][l] (ij|kl), J_B[k][l] += scale
// sum_{ij} D_A[i][j] (ij|kl), both as full symmetric matrices; raw |v| < cut is
// dropped (the reference's 1e-10 test on each integral).
template <typename R, int LA, int LB, int LC, int LD>
__global__ void __launch_bounds__(128) cp_tasks_kernel(const CPTask *__restrict__ tasks, TaskLaunch TL) {
  using Q = QClass<LA, LB, LC, LD>;
  constexpr int NA = Q::NA, NB = Q::NB, NC = Q::NC, ND = Q::ND;
  const int t = find_task(tasks, TL.ntasks, blockIdx.x);
  const CPTask &T = tasks[t];
  const int local = blockIdx.x - T.blk0;
  const int tx = local % T.nbx, ty = local / T.nbx;
  const int kpos = tx * 32 + threadIdx.x;
  const int bpos = ty * kWarpsPerBlock + threadIdx.y;
  if (bpos >= T.nbra) return;
  const bool active = kpos < T.nket;
  const PairRec &bra = T.pa[T.bra0 + bpos];
  const PairRec ket = T.pb[T.ket0 + min(kpos, T.nket - 1)];
  R I[Q::NINT];
  if (active) {
    eri_quartet<R, LA, LB, LC, LD>(bra, T.pra, ket, T.prb, TL.boys.f64, TL.boys.f32, I);
  } else {
#pragma unroll
    for (int x = 0; x < Q::NINT; ++x) I[x] = R(0);
  }
  const R cut = R(TL.cut);
#pragma unroll
  for (int x = 0; x < Q::NINT; ++x)
    if (!(fabs(I[x]) >= cut)) I[x] = R(0);
  auto Iat = [&](int a, int b, int c, int d) -> R { return I[((a * NB + b) * NC + c) * ND + d]; };
  const int fa = bra.fa, fb = bra.fb, fc = ket.fa, fd = ket.fb;
  const bool abdiff = bra.sa != bra.sb, cddiff = ket.sa != ket.sb;
  const R scale = R(T.scale);
  if (T.JA) {
    const R wk = active ? R(cddiff ? 2 : 1) * scale : R(0);
    const double *__restrict__ D = T.DsB;
    const int nB = T.nB, nA = T.nA;
#pragma unroll
    for (int a = 0; a < NA; ++a)
#pragma unroll
      for (int b = 0; b < NB; ++b) {
        R s = 0;
#pragma unroll
        for (int c = 0; c < NC; ++c)
#pragma unroll
          for (int d = 0; d < ND; ++d) s += R(__ldg(D + (fc + c) * nB + fd + d)) * Iat(a, b, c, d);
        s = warp_sum(s * wk);
        if (threadIdx.x == 0) {
          atomicAdd(T.JA + (fa + a) * nA + fb + b, double(s));
          if (abdiff) atomicAdd(T.JA + (fb + b) * nA + fa + a, double(s));
        }
      }
  }
  if (T.JB && active) {
    const R wb = R(abdiff ? 2 : 1) * scale;
    const double *__restrict__ D = T.DsA;
    const int nA = T.nA, nB = T.nB;
#pragma unroll
    for (int c = 0; c < NC; ++c)
#pragma unroll
      for (int d = 0; d < ND; ++d) {
        R s = 0;
#pragma unroll
        for (int a = 0; a < NA; ++a)
#pragma unroll
          for (int b = 0; b < NB; ++b) s += R(__ldg(D + (fa + a) * nA + fb + b)) * Iat(a, b, c, d);
        s *= wb;
        atomicAdd(T.JB + (fc + c) * nB + fd + d, double(s));
        if (cddiff) atomicAdd(T.JB + (fd + d) * nB + fc + c, double(s));
      }
  }
}

// ------------------------------------------------------- first quarter (IT) --
// Output A[nu][lam][sig] accumulates sum_mu Cs(mu) v(mu nu|lam sig) over every
// distinct member of the quartet's permutational orbit (intra) or of the
// (bra swap) x (ket swap) orbit (coupling); v are raw integrals with |v| > cut.
template <int NMU, int NNU, int NL, int NS, typename F>
__device__ __forceinline__ void it_role(F &&val, const double *__restrict__ Cs, int fmu, int fnu, int fl, int fs,
                                        double *A, int nB) {
#pragma unroll
  for (int nu = 0; nu < NNU; ++nu)
#pragma unroll
    for (int l = 0; l < NL; ++l)
#pragma unroll
      for (int s = 0; s < NS; ++s) {
        double acc = 0;
#pragma unroll
        for (int mu = 0; mu < NMU; ++mu) acc += __ldg(Cs + fmu + mu) * val(mu, nu, l, s);
        atomicAdd(A + ((size_t)(fnu + nu) * nB + fl + l) * nB + fs + s, acc);
      }
}

template <int LA, int LB, int LC, int LD>
__global__ void __launch_bounds__(128) it_kernel(ITParams P) {
  using Q = QClass<LA, LB, LC, LD>;
  constexpr int NA = Q::NA, NB = Q::NB, NC = Q::NC, ND = Q::ND;
  if (P.triangle && blockIdx.x * 32 > blockIdx.y * kWarpsPerBlock + kWarpsPerBlock - 1) return;
  const int kpos = blockIdx.x * 32 + threadIdx.x;
  const int bpos = blockIdx.y * kWarpsPerBlock + threadIdx.y;
  if (bpos >= P.nbra || kpos >= P.nket) return;
  if (P.triangle && kpos > bpos) return;
  const int bi = P.bra0 + bpos, ki = P.ket0 + kpos;
  const PairRec bra = P.pa[bi];
  const PairRec ket = P.pb[ki];
  if (P.screen) {
    const double b = bra.Q * ket.Q * dnorm6(P.Dn, P.nsh, bra.sa, bra.sb, ket.sa, ket.sb);
    if (b < P.eps) return;
  }
  double I[Q::NINT];
  eri_quartet<double, LA, LB, LC, LD>(bra, P.pra, ket, P.prb, P.boys.f64, P.boys.f32, I);
#pragma unroll
  for (int x = 0; x < Q::NINT; ++x)
    if (!(fabs(I[x]) > P.cut)) I[x] = 0.0;
  auto I4 = [&](int a, int b, int c, int d) -> double { return I[((a * NB + b) * NC + c) * ND + d]; };
  const bool ab = bra.sa != bra.sb, cd = ket.sa != ket.sb;
  const int fa = bra.fa, fb = bra.fb, fc = ket.fa, fd = ket.fb, nB = P.nB;
  const double *Cs = P.Cs;
  // (a b|c d): mu=a nu=b
  it_role<NA, NB, NC, ND>([&](int mu, int nu, int l, int s) { return I4(mu, nu, l, s); }, Cs, fa, fb, fc, fd, P.A, nB);
  if (ab)
    it_role<NB, NA, NC, ND>([&](int mu, int nu, int l, int s) { return I4(nu, mu, l, s); }, Cs, fb, fa, fc, fd, P.A, nB);
  if (cd)
    it_role<NA, NB, ND, NC>([&](int mu, int nu, int l, int s) { return I4(mu, nu, s, l); }, Cs, fa, fb, fd, fc, P.A, nB);
  if (ab && cd)
    it_role<NB, NA, ND, NC>([&](int mu, int nu, int l, int s) { return I4(nu, mu, s, l); }, Cs, fb, fa, fd, fc, P.A, nB);
  if (P.intra && bi != ki) {
    // (c d|a b) and its swaps: mu in the ket pair
    it_role<NC, ND, NA, NB>([&](int mu, int nu, int l, int s) { return I4(l, s, mu, nu); }, Cs, fc, fd, fa, fb, P.A, nB);
    if (cd)
      it_role<ND, NC, NA, NB>([&](int mu, int nu, int l, int s) { return I4(l, s, nu, mu); }, Cs, fd, fc, fa, fb, P.A, nB);
    if (ab)
      it_role<NC, ND, NB, NA>([&](int mu, int nu, int l, int s) { return I4(s, l, mu, nu); }, Cs, fc, fd, fb, fa, P.A, nB);
    if (ab && cd)
      it_role<ND, NC, NB, NA>([&](int mu, int nu, int l, int s) { return I4(s, l, nu, mu); }, Cs, fd, fc, fb, fa, P.A, nB);
  }
}

}  // namespace lgb
