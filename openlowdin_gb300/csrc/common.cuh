// Shared device definitions: Cartesian index tables, compile-time loops,
// device-side records of shells / shell pairs and the Boys function.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <type_traits>

namespace lgb {

constexpr int kMaxL = 3;               // per-shell angular momentum handled by the kernels (f)
constexpr int kMaxLQuartet = 4 * kMaxL;

// ---- Cartesian components -------------------------------------------------
// Order inside a shell of angular momentum l (lowdin order, also libint2's
// default): for i = 0..l: x = l - i, for j = 0..i: y = i - j, z = j,
// i.e. xx, xy, xz, yy, yz, zz for d.  A "cumulative" index enumerates every
// component of every total 0, 1, 2, ... in that order.
__host__ __device__ constexpr int ncart(int l) { return (l + 1) * (l + 2) / 2; }
__host__ __device__ constexpr int coff(int k) { return k * (k + 1) * (k + 2) / 6; }
__host__ __device__ constexpr int cidx(int x, int y, int z) {
  return coff(x + y + z) + (y + z) * (y + z + 1) / 2 + z;
}
__host__ __device__ constexpr int clevel(int c) {
  int k = 0;
  while (coff(k + 1) <= c) ++k;
  return k;
}
__host__ __device__ constexpr int crow(int c) {
  int r = c - coff(clevel(c)), i = 0;
  while ((i + 1) * (i + 2) / 2 <= r) ++i;
  return i;
}
__host__ __device__ constexpr int cx(int c) { return clevel(c) - crow(c); }
__host__ __device__ constexpr int cz(int c) { return c - coff(clevel(c)) - crow(c) * (crow(c) + 1) / 2; }
__host__ __device__ constexpr int cy(int c) { return clevel(c) - cx(c) - cz(c); }
__host__ __device__ constexpr int ccomp(int c, int d) { return d == 0 ? cx(c) : (d == 1 ? cy(c) : cz(c)); }
// recursion axis: first axis with a non-zero exponent
__host__ __device__ constexpr int cdir(int c) { return cx(c) > 0 ? 0 : (cy(c) > 0 ? 1 : 2); }
__host__ __device__ constexpr int cminus(int c, int d) {
  return cidx(cx(c) - (d == 0), cy(c) - (d == 1), cz(c) - (d == 2));
}
__host__ __device__ constexpr int cplus(int c, int d) {
  return cidx(cx(c) + (d == 0), cy(c) + (d == 1), cz(c) + (d == 2));
}

// compile-time loop: f(std::integral_constant<int, I>) for I in [B, E)
template <int B, int E, typename F>
__device__ __forceinline__ void sfor(F &&f) {
  if constexpr (B < E) {
    f(std::integral_constant<int, B>{});
    sfor<B + 1, E>(f);
  }
}

// ---- device records ---------------------------------------------------------
// One shell pair of a species, stored in canonical order (la >= lb).  Pairs are
// grouped by class (la, lb) and, inside a class, sorted by decreasing Schwarz
// factor so that a contiguous range is one class.  R = double for the FP64
// kernels, float for the FP32 kernels (a separate copy, so the FP32 kernels
// issue no FP64 conversions).
template <typename R>
struct alignas(16) PairT {
  int sa, sb;      // shell indices inside the species
  int fa, fb;      // first basis function of each shell
  int prim0, nprim;// primitive-pair range
  int la, lb;
  R A[3];          // centre of shell a
  R AB[3];         // A - B
  R Q;             // Schwarz factor sqrt(max |(ab|ab)|) of raw integrals
  R pad;
};
using PairRec = PairT<double>;
using PairRec32 = PairT<float>;

// One primitive pair: exponent sum p, its reciprocal, the Gaussian-product
// centre P, P - A, and Kt = sqrt(2 pi^{5/2}) exp(-ab/p |AB|^2) c_a N_a c_b N_b / p
// (coefficients times the primitive norm of the x^l component), so that the
// quartet prefactor is Kt_ab Kt_cd / sqrt(p + q).
template <typename R>
struct alignas(16) PrimT {
  R p, inv_p, Kt, pad;
  R P[3];
  R PA[3];
};
using PrimRec = PrimT<double>;
using PrimRec32 = PrimT<float>;

constexpr double kSqrt2Pi52 = 5.914967172795612;  // sqrt(2 pi^{5/2})

// ---- Boys function ----------------------------------------------------------
// F_m(T) = int_0^1 t^{2m} exp(-T t^2) dt.
// T < kBoysTMax: Taylor series about the nearest grid point T_i = i h of a table
// of F_n(T_i) (n = 0 .. kBoysOrders-1), giving F_L, then the downward recursion
// F_m = (2T F_{m+1} + e^{-T}) / (2m+1).
// T >= kBoysTMax: F_0 = sqrt(pi/T)/2 (erfc(6) < 3e-17), upward recursion
// F_{m+1} = ((2m+1) F_m - e^{-T}) / (2T).
constexpr double kBoysH = 0.1;
constexpr double kBoysTMax = 36.0;
constexpr int kBoysPoints = 361;          // T_i = 0, 0.1, ..., 36.0
constexpr int kBoysTaylor = 9;            // terms k = 0..8 (|dT| <= 0.05: error < 6e-18)
constexpr int kBoysOrders = kMaxLQuartet + kBoysTaylor + 1;
constexpr int kBoysStride = kBoysOrders + 1;  // row i: F_0..F_{kBoysOrders-1}(T_i), then e^{-T_i}
// After that table, one table per order L = 0..kMaxLQuartet of the Taylor
// coefficients of F_L about T_i, c_k = F_{L+k}(T_i) / k! (k < kBoysTaylor),
// followed by e^{-T_i}: rows of kBoysSRow doubles, so the series is a plain
// Horner chain of FMAs in (T_i - T).
constexpr int kBoysSRow = kBoysTaylor + 1;
constexpr int kBoysScaledOff = kBoysPoints * kBoysStride;
constexpr int kBoysF64Size = kBoysScaledOff + (kMaxLQuartet + 1) * kBoysPoints * kBoysSRow;

// e^x for |x| <= h/2 = 0.05: Taylor polynomial of degree 9 (remainder below
// 0.05^10 / 10! = 2.7e-20 relative), so e^{-T} = e^{-T_i} e^{T_i - T} costs
// nine FMAs and one table read
__host__ __device__ __forceinline__ double exp_small(double x) {
  double s = 1.0 / 362880.0;  // 1/9!
  s = fma(s, x, 1.0 / 40320.0);
  s = fma(s, x, 1.0 / 5040.0);
  s = fma(s, x, 1.0 / 720.0);
  s = fma(s, x, 1.0 / 120.0);
  s = fma(s, x, 1.0 / 24.0);
  s = fma(s, x, 1.0 / 6.0);
  s = fma(s, x, 0.5);
  s = fma(s, x, 1.0);
  return fma(s, x, 1.0);
}

__device__ __forceinline__ double rsqrt_r(double x) { return rsqrt(x); }
__device__ __forceinline__ float rsqrt_r(float x) { return rsqrtf(x); }

template <int L>
__device__ __forceinline__ void boys_f64(double T, double (&F)[L + 1], const double *__restrict__ tab) {
  if (T < kBoysTMax) {
    const int i = __double2int_rn(T * (1.0 / kBoysH));
    const double mdT = i * kBoysH - T;  // -(T - T_i)
    const double *t = tab + kBoysScaledOff + (L * kBoysPoints + i) * kBoysSRow;
    double s = __ldg(t + kBoysTaylor - 1);
#pragma unroll
    for (int k = kBoysTaylor - 1; k >= 1; --k) s = fma(s, mdT, __ldg(t + k - 1));
    F[L] = s;
    if constexpr (L > 0) {
      const double e = __ldg(t + kBoysTaylor) * exp_small(mdT);
      const double twoT = 2.0 * T;
#pragma unroll
      for (int m = L - 1; m >= 0; --m) F[m] = fma(twoT, F[m + 1], e) * (1.0 / (2 * m + 1));
    }
  } else {
    const double r = rsqrt(T);
    F[0] = 0.88622692545275801365 * r;  // sqrt(pi/T)/2
    if constexpr (L > 0) {
      // e^{-T} < 1.1e-20 above T = 46: its share of every F_m (m <= 8) there is
      // below 1e-11 relative and 1e-21 absolute, so it is left out
      const double e = T < 46.0 ? exp(-T) : 0.0;
      const double o2T = 0.5 * r * r;
#pragma unroll
      for (int m = 0; m < L; ++m) F[m + 1] = ((2 * m + 1) * F[m] - e) * o2T;
    }
  }
}

// FP32 Boys function by arithmetic alone (no table reads: a warp's 32
// table rows are 32 scattered cache sectors, which bound the FP32 kernels on
// the L1 pipe while their FMA pipe idled).
//   L = 0: F_0(T) = sqrt(pi/T)/2 erf(sqrt(T)) (erff), F_0(0) = 1.
//   L > 0, T < 4: F_L(T) = e^{-T} sum_k (2T)^k / ((2L+1)(2L+3)...(2L+2k+1))
//     (a series of positive terms; kBoysSeries(L) terms leave < 1e-7 of the
//     sum at T = 4), then the downward recursion
//     F_m = (2T F_{m+1} + e^{-T}) / (2m+1).
//   L > 0, T >= 4: F_0 as above, then the upward recursion
//     F_{m+1} = ((2m+1) F_m - e^{-T}) / (2T) (stable there for m < 4).
// Relative error below 8e-7 for every m <= L <= 4 and T >= 0 (checked against
// the incomplete gamma function); FP32 evaluates only quartets whose
// contribution is bounded by the mixed-precision split.
__host__ __device__ constexpr int kBoysSeries(int L) { return L <= 1 ? 16 : (L == 2 ? 15 : 14); }
constexpr float kBoysSplitT = 4.0f;

__device__ __forceinline__ float boys0_f32(float T) {
  return T < 1e-8f ? 1.0f - T * (1.0f / 3.0f) : 0.886226925f * erff(sqrtf(T)) * rsqrtf(T);
}

template <int L>
__device__ __forceinline__ void boys_f32(float T, float (&F)[L + 1], const float *__restrict__) {
  if constexpr (L == 0) {
    F[0] = boys0_f32(T);
  } else {
    const float e = __expf(-T);
    if (T < kBoysSplitT) {
      const float twoT = 2.0f * T;
      float term = 1.0f / (2 * L + 1), sum = term;
#pragma unroll
      for (int k = 1; k <= kBoysSeries(L); ++k) {
        term *= twoT * (1.0f / (2 * L + 2 * k + 1));
        sum += term;
      }
      F[L] = e * sum;
#pragma unroll
      for (int m = L - 1; m >= 0; --m) F[m] = fmaf(twoT, F[m + 1], e) * (1.0f / (2 * m + 1));
    } else {
      F[0] = boys0_f32(T);
      const float o2T = 0.5f / T;
#pragma unroll
      for (int m = 0; m < L; ++m) F[m + 1] = fmaf((float)(2 * m + 1), F[m], -e) * o2T;
    }
  }
}

template <typename R>
struct BoysTab;
template <>
struct BoysTab<double> {
  template <int L>
  __device__ __forceinline__ static void eval(double T, double (&F)[L + 1], const double *t64, const float *) {
    boys_f64<L>(T, F, t64);
  }
};
template <>
struct BoysTab<float> {
  template <int L>
  __device__ __forceinline__ static void eval(float T, float (&F)[L + 1], const double *, const float *t32) {
    boys_f32<L>(T, F, t32);
  }
};

}  // namespace lgb
