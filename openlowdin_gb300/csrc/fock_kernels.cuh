// Kernel templates: Schwarz factors, intra-species J/K, fused inter-species
// coupling and first-quarter transforms.  Included by the translation units
// that instantiate them for a set of quartet classes.
#pragma once
#include <type_traits>

#include "eri.cuh"
#include "kernels.cuh"

namespace lgb {

template <typename R>
__device__ __forceinline__ R warp_sum(R v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// The FP64 pipe of this GPU issues at 1/64 of the FP32 rate, so comparisons
// and maxima of non-negative doubles are done on their bit patterns (IEEE
// order of non-negative values = unsigned integer order of their bits):
// integer instructions, identical decisions.
__device__ __forceinline__ unsigned long long abs_bits(double v) {
  return (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
}
__device__ __forceinline__ unsigned abs_bits(float v) { return __float_as_uint(v) & 0x7fffffffu; }
// |v| < t and |v| > t for a non-negative threshold t
template <typename R>
__device__ __forceinline__ bool abs_below(R v, R t) { return abs_bits(v) < abs_bits(t); }
template <typename R>
__device__ __forceinline__ bool abs_above(R v, R t) { return abs_bits(v) > abs_bits(t); }
// 2^k, k = 0..3 (quartet degeneracies), from the exponent field alone
template <typename R>
__device__ __forceinline__ R pow2(int k) {
  if constexpr (std::is_same<R, double>::value) return __longlong_as_double((long long)(1023 + k) << 52);
  else return __int_as_float((127 + k) << 23);
}

// largest shell-block maximum |D| over the six index pairs of a quartet
template <typename T>
__device__ __forceinline__ T dnorm6(const T *__restrict__ Dn, int nsh, int a, int b, int c, int d) {
  T m = __ldg(Dn + a * nsh + b);
  m = max(m, __ldg(Dn + a * nsh + c));
  m = max(m, __ldg(Dn + b * nsh + c));
  m = max(m, __ldg(Dn + a * nsh + d));
  m = max(m, __ldg(Dn + b * nsh + d));
  m = max(m, __ldg(Dn + c * nsh + d));
  return m;
}
template <>
__device__ __forceinline__ double dnorm6(const double *__restrict__ Dn, int nsh, int a, int b, int c, int d) {
  const unsigned long long *u = reinterpret_cast<const unsigned long long *>(Dn);   // entries are >= 0
  unsigned long long m = __ldg(u + a * nsh + b);
  m = max(m, __ldg(u + a * nsh + c));
  m = max(m, __ldg(u + b * nsh + c));
  m = max(m, __ldg(u + a * nsh + d));
  m = max(m, __ldg(u + b * nsh + d));
  m = max(m, __ldg(u + c * nsh + d));
  return __longlong_as_double((long long)m);
}

// Per-system build flag of a batch (LowdinGB300_batch_set_active): off
// (converged, nothing built), on, or held in FP64 (mixed builds evaluate all
// of the system's quartets in their FP64 launches).  Tasks without a flag are on.
constexpr int kSysOff = 0, kSysOn = 1, kSysFP64 = 2;
__device__ __forceinline__ int system_flag(const int *f) { return f ? __ldg(f) : kSysOn; }

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

template <typename R>
__device__ __forceinline__ void atomic_acc(double *g64, float *g32, size_t i, R v) {
  if constexpr (std::is_same<R, double>::value) atomicAdd(g64 + i, v);
  else atomicAdd(g32 + i, v);
}

// ----------------------------------------------------------------- Schwarz --
template <int LA, int LB>
__global__ void __launch_bounds__(128) schwarz_kernel(SchwarzParams P) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= P.np) return;
  const PairRec pr = P.pairs[P.p0 + t];
  constexpr int N = ncart(LA) * ncart(LB);
  double I[N * N];
  eri_quartet<double, LA, LB, LA, LB>(pr, P.prims + pr.prim0, pr, P.prims + pr.prim0, P.boys.f64, P.boys.f32, I);
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
// Screening bound: plain launches (split = 0) use the FP64 product
// Q_ab Q_cd max|D| as the reference does; mixed launches compute it in FP32
// from the FP32 records in both kernels, so each quartet lands in exactly one
// of the FP64 (bound >= split) and FP32 (bound < split) launches.
template <typename R, int LA, int LB, int LC, int LD>
__global__ void __launch_bounds__(128) jk_tasks_kernel(const JKTask *__restrict__ tasks, TaskLaunch TL) {
  using Q = QClass<LA, LB, LC, LD>;
  constexpr bool F64 = std::is_same<R, double>::value;
  constexpr int NA = Q::NA, NB = Q::NB, NC = Q::NC, ND = Q::ND;
  const int t = find_task(tasks, TL.ntasks, blockIdx.x);
  const JKTask &T = tasks[t];
  const int act = system_flag(T.active);
  if (act == kSysOff) return;   // converged system: nothing to build
  if (act == kSysFP64 && TL.mixed && TL.lower) return;   // system held in FP64: the FP64 launch takes it all
  const int local = blockIdx.x - T.blk0;
  const int tx = local % T.nbx, ty = local / T.nbx;
  if (T.triangle && tx * 32 > ty * kWarpsPerBlock + kWarpsPerBlock - 1) return;
  if (TL.mixed && act != kSysFP64 && ty * kWarpsPerBlock < T.nbra && (T.Dnmax32 || !T.screen)) {
    // The tile's first bra and first ket carry its largest Schwarz factors and
    // Dnmax32 bounds the six norms, so in FP32 (rounding is monotonic, same
    // order of products) ub >= every quartet bound b of the tile: a tile the
    // launch cannot take leaves before staging its records.
    float ub = T.pairs32[T.bra0 + ty * kWarpsPerBlock].Q * T.pairs32[T.ket0 + tx * 32].Q;
    if (T.screen) ub *= __ldg(T.Dnmax32);
    if (TL.lower ? (T.screen && ub < fmaxf(TL.eps32, TL.skip)) : ub < TL.split32) return;
  }
  const PairT<R> *pairs;
  const PrimT<R> *prims;
  const R *D;
  if constexpr (F64) {
    pairs = T.pairs; prims = T.prims; D = T.Ds;
  } else {
    pairs = T.pairs32; prims = T.prims32; D = T.Ds32;
  }
  // The block's 32 ket pairs (shared by its bra warps) and the first primitive
  // pair of each, staged once in shared memory by coalesced 16-byte copies.
  // Strides 80 / 112 B (pairs) and 48 / 80 B (primitives) keep the per-lane
  // 16-byte reads free of bank conflicts.
  struct alignas(16) SPair {
    PairT<R> p;
    int4 pad;
  };
  __shared__ SPair sk[32];
  __shared__ PrimT<R> skp[32];
  {
    constexpr int WP = sizeof(PairT<R>) / 16, WQ = sizeof(PrimT<R>) / 16;
    const int tid = threadIdx.y * 32 + threadIdx.x;
    for (int w = tid; w < 32 * WP; w += 32 * kWarpsPerBlock) {
      const int r = w / WP, k = w % WP;
      const int kr = T.ket0 + min(tx * 32 + r, T.nket - 1);
      reinterpret_cast<int4 *>(&sk[r].p)[k] = __ldg(reinterpret_cast<const int4 *>(pairs + kr) + k);
    }
    __syncthreads();
    for (int w = tid; w < 32 * WQ; w += 32 * kWarpsPerBlock) {
      const int r = w / WQ, k = w % WQ;
      reinterpret_cast<int4 *>(skp + r)[k] = __ldg(reinterpret_cast<const int4 *>(prims + sk[r].p.prim0) + k);
    }
    __syncthreads();
  }
  const int kpos = tx * 32 + threadIdx.x;
  const int bpos = ty * kWarpsPerBlock + threadIdx.y;
  if (bpos >= T.nbra) return;  // warp-uniform
  bool active = kpos < T.nket && (!T.triangle || kpos <= bpos);
  const int bi = T.bra0 + bpos;
  const int ki = T.ket0 + min(kpos, T.nket - 1);
  const PairT<R> &bra = pairs[bi];
  const PairT<R> &ket = sk[threadIdx.x].p;
  if (TL.mixed) {
    // FP32 bound from the FP32 Schwarz factors (the FP64 records hold the
    // same values before rounding), identical in both launches
    float b = T.pairs32[bi].Q * (float)ket.Q;
    if (T.screen) {
      b *= dnorm6(T.Dn32, T.nsh, bra.sa, bra.sb, ket.sa, ket.sb);
      if (b < fmaxf(TL.eps32, act == kSysFP64 ? 0.f : TL.skip)) active = false;   // no skip in an FP64 check
    }
    if (act != kSysFP64 && (TL.lower ? !(b < TL.split32) : (b < TL.split32))) active = false;
  } else if (T.screen) {
    const double b = T.pairs[bi].Q * (F64 ? (double)ket.Q : T.pairs[ki].Q) *
                     dnorm6(T.Dn, T.nsh, bra.sa, bra.sb, ket.sa, ket.sb);
    if (abs_below(b, TL.eps)) active = false;
  }
  if (__all_sync(0xffffffffu, !active)) return;
  if (T.count) {
    const unsigned cnt = __popc(__ballot_sync(0xffffffffu, active));
    if (threadIdx.x == 0) atomicAdd(T.count, (unsigned long long)cnt);
  }
  R I[Q::NINT];
  if (active) {
    const PrimT<R> *kp = ket.nprim == 1 ? skp + threadIdx.x : prims + ket.prim0;
    eri_quartet<R, LA, LB, LC, LD>(bra, prims + bra.prim0, ket, kp, TL.boys.f64, TL.boys.f32, I);
  } else {
#pragma unroll
    for (int x = 0; x < Q::NINT; ++x) I[x] = R(0);
  }
  const R deg = active ? pow2<R>((bra.sa != bra.sb) + (ket.sa != ket.sb) + (bi != ki)) : R(0);
  R hf;
  if constexpr (F64) hf = T.hf;
  else hf = T.hf32;
  const R hdeg = deg * hf;
  const int n = T.n;
  double *G = T.Gacc;
  float *G32 = T.Gacc32;
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
        for (int d = 0; d < ND; ++d) s += __ldg(D + (fc + c) * n + fd + d) * Iat(a, b, c, d);
      s = warp_sum(s * deg);
      if (threadIdx.x == 0) atomic_acc<R>(G, G32, (size_t)(fa + a) * n + fb + b, s);
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
        for (int b = 0; b < NB; ++b) s += __ldg(D + (fa + a) * n + fb + b) * Iat(a, b, c, d);
      atomic_acc<R>(G, G32, (size_t)(fc + c) * n + fd + d, s * deg);
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
        for (int d = 0; d < ND; ++d) s += __ldg(D + (fb + b) * n + fd + d) * Iat(a, b, c, d);
      atomic_acc<R>(G, G32, (size_t)(fa + a) * n + fc + c, s * hdeg);
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
        for (int c = 0; c < NC; ++c) s += __ldg(D + (fa + a) * n + fc + c) * Iat(a, b, c, d);
      atomic_acc<R>(G, G32, (size_t)(fb + b) * n + fd + d, s * hdeg);
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
        for (int c = 0; c < NC; ++c) s += __ldg(D + (fb + b) * n + fc + c) * Iat(a, b, c, d);
      atomic_acc<R>(G, G32, (size_t)(fa + a) * n + fd + d, s * hdeg);
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
        for (int d = 0; d < ND; ++d) s += __ldg(D + (fa + a) * n + fd + d) * Iat(a, b, c, d);
      atomic_acc<R>(G, G32, (size_t)(fb + b) * n + fc + c, s * hdeg);
    }
}

// ------------------------------------------------------- J/K, FP32 bra rows --
// FP32 half of a mixed J/K build, one block per bra pair (a b| of a task; its
// kRowWarps warps take the task's ket pairs 32 at a time).  The exchange
// updates of a quartet touch only rows fa.. and fb.. of the output (K13, K14
// on the rows of shell a, K23, K24 on those of shell b) and read only those
// rows of D, so the block keeps both in shared memory, interleaved by column
// (Drow[col][r], Krow[col][r], r < NA + NB, padded to an odd pitch so that
// random columns spread over the banks), together with the largest
// shell-block norm of shells a and b against every shell (Dnab[s] =
// max(|D|_{a s}, |D|_{b s})), which gives four of the six screening norms in
// two reads.  The ket side is read from pair-indexed arrays when the build
// provides them (JKTask::Dp32 / DnP32 / Jp32: per ket pair its D block, its
// shell-block norm and its Coulomb accumulator, element-major inside the ket
// class, so a warp's 32 kets are one coalesced line per element), else from
// the n x n matrices.  The bra Coulomb block (J12) is summed in registers
// over every ket of the warp before one warp reduction.  At the end the
// exchange rows go to the global accumulator (non-zero entries only).
// Quartet selection, bound and arithmetic are those of jk_tasks_kernel's FP32
// launch (same FP32 bound, same screening and split), so the quartets taken
// and the integrals are the same; only the order of the FP32 additions differs.
template <typename T>
__device__ __forceinline__ int find_task_rows(const T *__restrict__ tasks, int ntasks, int b) {
  int lo = 0, hi = ntasks - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(&tasks[mid].rblk0) <= b) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

template <int LA, int LB, int LC, int LD>
__global__ void __launch_bounds__(32 * kRowWarps) jk32_row_kernel(const JKTask *__restrict__ tasks, TaskLaunch TL) {
  using Q = QClass<LA, LB, LC, LD>;
  constexpr int NA = Q::NA, NB = Q::NB, NC = Q::NC, ND = Q::ND, NR = NA + NB, NRP = row_pitch(NA + NB);
  extern __shared__ float rsm[];
  const int t = find_task_rows(tasks, TL.ntasks, blockIdx.x);
  const JKTask &T = tasks[t];
  if (system_flag(T.active) != kSysOn) return;   // converged, or held in FP64
  const int bpos = blockIdx.x - T.rblk0;
  if (bpos >= T.nbra) return;
  const int bi = T.bra0 + bpos;
  const int nk = T.triangle ? bpos + 1 : T.nket;  // ket positions [0, nk)
  const int n = T.n, nsh = T.nsh;
  const PairRec32 bra = T.pairs32[bi];
  const PrimRec32 *__restrict__ prims = T.prims32;
  const float cutoff = fmaxf(TL.eps32, TL.skip);
  // kets are sorted by decreasing Schwarz factor: bra.Q Q(ket k0) Dnmax32 bounds
  // every quartet bound from ket position k0 on (same FP32 product order)
  const float dmax = (T.screen && T.Dnmax32) ? __ldg(T.Dnmax32) : -1.f;
  auto below_from = [&](int k0) {
    const float qk = T.soa32 ? T.soa32[kSoaQ * T.npairs + T.ket0 + k0] : T.pairs32[T.ket0 + k0].Q;
    return dmax >= 0.f && bra.Q * qk * dmax < cutoff;
  };
  if (below_from(0)) return;   // nothing of this bra row reaches the cutoff
  float *Drow = rsm;                 // [n][NRP]: D(fa + r, col) for r < NA, D(fb + r - NA, col) after
  float *Krow = rsm + NRP * n;       // [n][NRP]: exchange accumulators of the same rows
  float *Dnab = Krow + NRP * n;      // [nsh]
  for (int i = threadIdx.x; i < NRP * n; i += blockDim.x) {
    const int c = i / NRP, r = i - c * NRP;
    float v = 0.f;
    if (r < NR) v = __ldg(T.Ds32 + (size_t)(r < NA ? bra.fa + r : bra.fb + (r - NA)) * n + c);
    Drow[i] = v;
    Krow[i] = 0.f;
  }
  if (T.screen)
    for (int i = threadIdx.x; i < nsh; i += blockDim.x)
      Dnab[i] = fmaxf(__ldg(T.Dn32 + (size_t)bra.sa * nsh + i), __ldg(T.Dn32 + (size_t)bra.sb * nsh + i));
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const float hf = T.hf32;
  const float *__restrict__ D = T.Ds32;
  float *G32 = T.Gacc32;
  float j12[NA * NB];
#pragma unroll
  for (int x = 0; x < NA * NB; ++x) j12[x] = 0.f;
  const float dn_ab = T.screen ? __ldg(T.Dn32 + (size_t)bra.sa * nsh + bra.sb) : 0.f;
  const float *__restrict__ soa = T.soa32;
  const int np = T.npairs;
  const float *__restrict__ Dp = T.Dp32;          // pair-indexed ket data (null: n x n matrices)
  const float *__restrict__ DnP = T.DnP32;
  float *Jp = T.Jp32;
  const int kstride = T.nket;                     // element stride of the pair-indexed arrays
  unsigned cnt = 0;
  for (int k0 = warp * 32; k0 < nk; k0 += 32 * kRowWarps) {
    if (below_from(k0)) break;   // warp-uniform; every later ket chunk is below too
    const int kpos = k0 + lane;
    bool active = kpos < nk;
    const int kq = min(kpos, nk - 1);
    const int ki = T.ket0 + kq;
    PairRec32 ket;
    PrimRec32 kprim;
    if (soa) {
      // one coalesced 128-byte line per field and warp; only the fields the
      // class reads are loaded
      const float *f = soa + ki;
      ket.Q = f[kSoaQ * np];
      const int sh = __float_as_int(f[kSoaShells * np]), fn = __float_as_int(f[kSoaFuncs * np]);
      ket.sa = sh & 0xffff;
      ket.sb = sh >> 16;
      ket.fa = fn & 0xffff;
      ket.fb = fn >> 16;
      ket.nprim = 1;
      ket.prim0 = 0;
      if constexpr (LD > 0) {
        ket.AB[0] = f[kSoaABx * np];
        ket.AB[1] = f[kSoaABy * np];
        ket.AB[2] = f[kSoaABz * np];
      }
      kprim.p = f[kSoaP * np];
      kprim.Kt = f[kSoaKt * np];
      kprim.P[0] = f[kSoaPx * np];
      kprim.P[1] = f[kSoaPy * np];
      kprim.P[2] = f[kSoaPz * np];
      if constexpr (LC + LD > 0) {
        kprim.inv_p = f[kSoaInvP * np];
        kprim.PA[0] = f[kSoaPAx * np];
        kprim.PA[1] = f[kSoaPAy * np];
        kprim.PA[2] = f[kSoaPAz * np];
      }
    } else {
      ket = T.pairs32[ki];
    }
    float bound = bra.Q * ket.Q;
    if (T.screen) {
      float m = fmaxf(dn_ab, fmaxf(Dnab[ket.sa], Dnab[ket.sb]));
      m = fmaxf(m, DnP ? DnP[ki] : __ldg(T.Dn32 + (size_t)ket.sa * nsh + ket.sb));
      bound *= m;
      if (bound < cutoff) active = false;
    }
    if (!(bound < TL.split32)) active = false;   // the FP64 launch takes these
    const unsigned live = __ballot_sync(0xffffffffu, active);
    if (!live) continue;
    cnt += __popc(live);
    float I[Q::NINT];
    if (active) {
      if (soa)
        eri_quartet_k1<float, LA, LB, LC, LD>(bra, prims + bra.prim0, ket, kprim, TL.boys.f64, TL.boys.f32, I);
      else
        eri_quartet<float, LA, LB, LC, LD>(bra, prims + bra.prim0, ket, prims + ket.prim0, TL.boys.f64,
                                           TL.boys.f32, I);
    } else {
#pragma unroll
      for (int x = 0; x < Q::NINT; ++x) I[x] = 0.f;
    }
    const float deg = active ? pow2<float>((bra.sa != bra.sb) + (ket.sa != ket.sb) + (bi != ki)) : 0.f;
    const float hdeg = deg * hf;
    const int fc = ket.fa, fd = ket.fb;
    auto Iat = [&](int a, int b, int c, int d) -> float { return I[((a * NB + b) * NC + c) * ND + d]; };
    // J12 (bra block): D of the ket block, summed over this warp's kets
#pragma unroll
    for (int c = 0; c < NC; ++c)
#pragma unroll
      for (int d = 0; d < ND; ++d) {
        float dcd = 0.f;
        if (active) dcd = (Dp ? Dp[(size_t)(c * ND + d) * kstride + kq] : __ldg(D + (size_t)(fc + c) * n + fd + d)) * deg;
#pragma unroll
        for (int a = 0; a < NA; ++a)
#pragma unroll
          for (int b = 0; b < NB; ++b) j12[a * NB + b] = fmaf(dcd, Iat(a, b, c, d), j12[a * NB + b]);
      }
    if (!active) continue;
    // the D rows of the bra shells at the ket's columns
    float dc[NC][NR], dd[ND][NR];
#pragma unroll
    for (int c = 0; c < NC; ++c)
#pragma unroll
      for (int r = 0; r < NR; ++r) dc[c][r] = Drow[(fc + c) * NRP + r];
#pragma unroll
    for (int d = 0; d < ND; ++d)
#pragma unroll
      for (int r = 0; r < NR; ++r) dd[d][r] = Drow[(fd + d) * NRP + r];
    // J34 (ket block): D of the bra block
#pragma unroll
    for (int c = 0; c < NC; ++c)
#pragma unroll
      for (int d = 0; d < ND; ++d) {
        float s = 0.f;
#pragma unroll
        for (int a = 0; a < NA; ++a)
#pragma unroll
          for (int b = 0; b < NB; ++b) s = fmaf(Drow[(bra.fb + b) * NRP + a], Iat(a, b, c, d), s);
        if (Jp) atomicAdd(Jp + (size_t)(c * ND + d) * kstride + kq, s * deg);
        else atomicAdd(G32 + (size_t)(fc + c) * n + fd + d, s * deg);
      }
    // K13 (a,c) += D(b,d), K14 (a,d) += D(b,c): rows of shell a
#pragma unroll
    for (int a = 0; a < NA; ++a) {
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        float s = 0.f;
#pragma unroll
        for (int b = 0; b < NB; ++b)
#pragma unroll
          for (int d = 0; d < ND; ++d) s = fmaf(dd[d][NA + b], Iat(a, b, c, d), s);
        atomicAdd(Krow + (fc + c) * NRP + a, s * hdeg);
      }
#pragma unroll
      for (int d = 0; d < ND; ++d) {
        float s = 0.f;
#pragma unroll
        for (int b = 0; b < NB; ++b)
#pragma unroll
          for (int c = 0; c < NC; ++c) s = fmaf(dc[c][NA + b], Iat(a, b, c, d), s);
        atomicAdd(Krow + (fd + d) * NRP + a, s * hdeg);
      }
    }
    // K24 (b,d) += D(a,c), K23 (b,c) += D(a,d): rows of shell b
#pragma unroll
    for (int b = 0; b < NB; ++b) {
#pragma unroll
      for (int d = 0; d < ND; ++d) {
        float s = 0.f;
#pragma unroll
        for (int a = 0; a < NA; ++a)
#pragma unroll
          for (int c = 0; c < NC; ++c) s = fmaf(dc[c][a], Iat(a, b, c, d), s);
        atomicAdd(Krow + (fd + d) * NRP + NA + b, s * hdeg);
      }
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        float s = 0.f;
#pragma unroll
        for (int a = 0; a < NA; ++a)
#pragma unroll
          for (int d = 0; d < ND; ++d) s = fmaf(dd[d][a], Iat(a, b, c, d), s);
        atomicAdd(Krow + (fc + c) * NRP + NA + b, s * hdeg);
      }
    }
  }
  if (T.count && lane == 0 && cnt) atomicAdd(T.count, (unsigned long long)cnt);
  // J12: one reduction per warp
#pragma unroll
  for (int x = 0; x < NA * NB; ++x) {
    const float v = warp_sum(j12[x]);
    if (lane == 0 && v != 0.f) atomicAdd(G32 + (size_t)(bra.fa + x / NB) * n + bra.fb + x % NB, v);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < NRP * n; i += blockDim.x) {
    const float v = Krow[i];
    const int c = i / NRP, r = i - c * NRP;
    if (v != 0.f && r < NR) atomicAdd(G32 + (size_t)(r < NA ? bra.fa + r : bra.fb + (r - NA)) * n + c, v);
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
  constexpr bool F64 = std::is_same<R, double>::value;
  constexpr int NA = Q::NA, NB = Q::NB, NC = Q::NC, ND = Q::ND;
  const int t = find_task(tasks, TL.ntasks, blockIdx.x);
  const CPTask &T = tasks[t];
  const int act = system_flag(T.active);
  if (act == kSysOff) return;   // converged system: nothing to build
  if (act == kSysFP64 && TL.mixed && TL.lower) return;   // system held in FP64: the FP64 launch takes it all
  const int local = blockIdx.x - T.blk0;
  const int tx = local % T.nbx, ty = local / T.nbx;
  const int kpos = tx * 32 + threadIdx.x;
  const int bpos = ty * kWarpsPerBlock + threadIdx.y;
  if (bpos >= T.nbra) return;
  bool active = kpos < T.nket;
  {
    // |(ij|kl)| <= Q_ab Q_cd for every component (Schwarz), and raw values
    // below the cut are dropped, so such a quartet contributes nothing; the
    // test is done in FP32 in mixed launches so both launches agree
    const int bi = T.bra0 + bpos, ki = T.ket0 + min(kpos, T.nket - 1);
    const bool tiny = TL.mixed ? T.pa32[bi].Q * T.pb32[ki].Q * 0.999f < TL.cut32
                                     : abs_below(T.pa[bi].Q * T.pb[ki].Q * (1.0 - 1e-9), TL.cut);
    if (tiny) active = false;
  }
  if (TL.mixed) {
    // mixed precision: FP32 for quartets whose Q_ab Q_cd max(|D_A|, |D_B|)
    // bound (FP32, identical in both launches) is below the split
    const int bi = T.bra0 + bpos, ki = T.ket0 + min(kpos, T.nket - 1);
    const PairRec32 &b32 = T.pa32[bi];
    const PairRec32 &k32 = T.pb32[ki];
    float dm = 0.f;
    if (T.DnA32) dm = __ldg(T.DnA32 + b32.sa * T.nshA + b32.sb);
    if (T.DnB32) dm = fmaxf(dm, __ldg(T.DnB32 + k32.sa * T.nshB + k32.sb));
    const float b = b32.Q * k32.Q * dm;
    if (act != kSysFP64 && (TL.lower ? !(b < TL.split32) : (b < TL.split32))) active = false;
    if ((T.DnA32 || T.DnB32) && act != kSysFP64 && b < TL.skip) active = false;
  }
  if (__all_sync(0xffffffffu, !active)) return;
  if (T.count) {
    const unsigned cnt = __popc(__ballot_sync(0xffffffffu, active));
    if (threadIdx.x == 0) atomicAdd(T.count, (unsigned long long)cnt);
  }
  const PairT<R> *pa, *pb;
  const PrimT<R> *pra, *prb;
  const R *DA, *DB;
  if constexpr (F64) {
    pa = T.pa; pb = T.pb; pra = T.pra; prb = T.prb; DA = T.DsA; DB = T.DsB;
  } else {
    pa = T.pa32; pb = T.pb32; pra = T.pra32; prb = T.prb32; DA = T.DsA32; DB = T.DsB32;
  }
  const PairT<R> &bra = pa[T.bra0 + bpos];
  const PairT<R> ket = pb[T.ket0 + min(kpos, T.nket - 1)];
  R I[Q::NINT];
  if (active) {
    eri_quartet<R, LA, LB, LC, LD>(bra, pra + bra.prim0, ket, prb + ket.prim0, TL.boys.f64, TL.boys.f32, I);
  } else {
#pragma unroll
    for (int x = 0; x < Q::NINT; ++x) I[x] = R(0);
  }
  R cut, scale;
  if constexpr (F64) {
    cut = TL.cut;
    scale = T.scale;
  } else {
    cut = TL.cut32;
    scale = T.scale32;
  }
#pragma unroll
  for (int x = 0; x < Q::NINT; ++x)
    if (abs_below(I[x], cut)) I[x] = R(0);
  auto Iat = [&](int a, int b, int c, int d) -> R { return I[((a * NB + b) * NC + c) * ND + d]; };
  const int fa = bra.fa, fb = bra.fb, fc = ket.fa, fd = ket.fb;
  const bool abdiff = bra.sa != bra.sb, cddiff = ket.sa != ket.sb;
  if (T.JA) {
    const R wk = active ? R(cddiff ? 2 : 1) * scale : R(0);
    const int nB = T.nB, nA = T.nA;
#pragma unroll
    for (int a = 0; a < NA; ++a)
#pragma unroll
      for (int b = 0; b < NB; ++b) {
        R s = 0;
#pragma unroll
        for (int c = 0; c < NC; ++c)
#pragma unroll
          for (int d = 0; d < ND; ++d) s += __ldg(DB + (fc + c) * nB + fd + d) * Iat(a, b, c, d);
        s = warp_sum(s * wk);
        if (threadIdx.x == 0) {
          atomic_acc<R>(T.JA, T.JA32, (size_t)(fa + a) * nA + fb + b, s);
          if (abdiff) atomic_acc<R>(T.JA, T.JA32, (size_t)(fb + b) * nA + fa + a, s);
        }
      }
  }
  if (T.JB && active) {
    const R wb = R(abdiff ? 2 : 1) * scale;
    const int nA = T.nA, nB = T.nB;
#pragma unroll
    for (int c = 0; c < NC; ++c)
#pragma unroll
      for (int d = 0; d < ND; ++d) {
        R s = 0;
#pragma unroll
        for (int a = 0; a < NA; ++a)
#pragma unroll
          for (int b = 0; b < NB; ++b) s += __ldg(DA + (fa + a) * nA + fb + b) * Iat(a, b, c, d);
        s *= wb;
        atomic_acc<R>(T.JB, T.JB32, (size_t)(fc + c) * nB + fd + d, s);
        if (cddiff) atomic_acc<R>(T.JB, T.JB32, (size_t)(fd + d) * nB + fc + c, s);
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
  // every raw integral is bounded by Q_ab Q_cd (Schwarz) and only |v| > cut is used
  if (!abs_above(bra.Q * ket.Q * (1.0 - 1e-9), P.cut)) return;
  if (P.screen) {
    const double b = bra.Q * ket.Q * dnorm6(P.Dn, P.nsh, bra.sa, bra.sb, ket.sa, ket.sb);
    if (abs_below(b, P.eps)) return;
  }
  double I[Q::NINT];
  eri_quartet<double, LA, LB, LC, LD>(bra, P.pra + bra.prim0, ket, P.prb + ket.prim0, P.boys.f64, P.boys.f32, I);
#pragma unroll
  for (int x = 0; x < Q::NINT; ++x)
    if (!abs_above(I[x], P.cut)) I[x] = 0.0;
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

// ------------------------------------------------------ MP2 transform input --
// Lane x of warp y: bra pair tile_y*4 + y, ket pair tile_x*32 + x of the batch.
template <int LA, int LB, int LC, int LD>
__global__ void __launch_bounds__(128) mp2x_kernel(MXParams P) {
  using Q = QClass<LA, LB, LC, LD>;
  constexpr int NA = Q::NA, NB = Q::NB, NC = Q::NC, ND = Q::ND;
  const int kpos = blockIdx.x * 32 + threadIdx.x;
  const int bpos = blockIdx.y * kWarpsPerBlock + threadIdx.y;
  if (bpos >= P.nbra || kpos >= P.nket) return;
  const int bi = P.bra0 + bpos, ki = P.ket0 + kpos;
  const PairRec bra = P.pairs[bi];
  const PairRec ket = P.kpairs[ki];
  if (!abs_above(bra.Q * ket.Q * (1.0 - 1e-9), P.cut)) return;
  if (P.screen && abs_below(bra.Q * ket.Q * dnorm6(P.Dn, P.nsh, bra.sa, bra.sb, ket.sa, ket.sb), P.eps)) return;
  double I[Q::NINT];
  eri_quartet<double, LA, LB, LC, LD>(bra, P.prims + bra.prim0, ket, P.kprims + ket.prim0, P.boys.f64, P.boys.f32,
                                      I);
  const int col0 = __ldg(P.colbase + ki) - P.col_first;
  const bool two = bra.sa != bra.sb;
  const size_t n = P.n, ncol = P.ncol;
#pragma unroll
  for (int a = 0; a < NA; ++a)
#pragma unroll
    for (int b = 0; b < NB; ++b)
#pragma unroll
      for (int c = 0; c < NC; ++c)
#pragma unroll
        for (int d = 0; d < ND; ++d) {
          const double v = I[((a * NB + b) * NC + c) * ND + d];
          if (!abs_above(v, P.cut)) continue;
          const size_t col = col0 + c * ND + d;
          const size_t i1 = ((bra.fa + a) * ncol + col) * n + bra.fb + b;
          const size_t i2 = ((bra.fb + b) * ncol + col) * n + bra.fa + a;
          if (P.X) {
            P.X[i1] = v;
            if (two) P.X[i2] = v;
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

}  // namespace lgb
