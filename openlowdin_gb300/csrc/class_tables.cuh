// Launch-table entries of the class-templated kernels.  Each k_<kind>_c<B>.cu
// translation unit instantiates the kernels of one kind for bra pair class B
// and every ket pair class, so the classes compile in parallel.  Entries are
// null where the generic runtime-class kernels take over (total angular
// momentum above kTemplatedMaxL) or where a kernel is never used (J/K with the
// ket class above the bra class).
#pragma once
#include "fock_kernels.cuh"

namespace lgb {

// the pair classes of s, p and d shells with total angular momentum up to
// kTemplatedMaxL; classes with an f shell run on the cooperative kernels
constexpr int kTemplatedPairClasses = 6;
template <int B, int K>
constexpr bool templated_class() {
  return B < kTemplatedPairClasses && K < kTemplatedPairClasses && pc_L(B) + pc_L(K) <= kTemplatedMaxL;
}

template <typename R, int B, int K>
constexpr JKFn jk_entry() {
  if constexpr (templated_class<B, K>() && B >= K) return &jk_tasks_kernel<R, pc_la(B), pc_lb(B), pc_la(K), pc_lb(K)>;
  else return nullptr;
}
template <int B, int K>
constexpr JKFn jkr_entry() {
  if constexpr (templated_class<B, K>() && B >= K) return &jk32_row_kernel<pc_la(B), pc_lb(B), pc_la(K), pc_lb(K)>;
  else return nullptr;
}
template <typename R, int B, int K>
constexpr CPFn cp_entry() {
  if constexpr (templated_class<B, K>()) return &cp_tasks_kernel<R, pc_la(B), pc_lb(B), pc_la(K), pc_lb(K)>;
  else return nullptr;
}
template <int B, int K>
constexpr ITFn it_entry() {
  if constexpr (templated_class<B, K>()) return &it_kernel<pc_la(B), pc_lb(B), pc_la(K), pc_lb(K)>;
  else return nullptr;
}

template <int B, int K>
constexpr MXFn mx_entry() {
  if constexpr (templated_class<B, K>()) return &mp2x_kernel<pc_la(B), pc_lb(B), pc_la(K), pc_lb(K)>;
  else return nullptr;
}

static_assert(kNumPairClasses == 10, "launch-table rows list every pair class");
#define LGB_ROW(F, ...)                                                                                   \
  { F<__VA_ARGS__, 0>(), F<__VA_ARGS__, 1>(), F<__VA_ARGS__, 2>(), F<__VA_ARGS__, 3>(), F<__VA_ARGS__, 4>(), \
    F<__VA_ARGS__, 5>(), F<__VA_ARGS__, 6>(), F<__VA_ARGS__, 7>(), F<__VA_ARGS__, 8>(), F<__VA_ARGS__, 9>() }

#define LGB_JK_TABLES(B)                                   \
  extern const JKFn kJK64_##B[kNumPairClasses];                          \
  extern const JKFn kJK32_##B[kNumPairClasses];                          \
  extern const JKFn kJKR_##B[kNumPairClasses];                           \
  const JKFn kJK64_##B[kNumPairClasses] = LGB_ROW(jk_entry, double, B); \
  const JKFn kJK32_##B[kNumPairClasses] = LGB_ROW(jk_entry, float, B);  \
  const JKFn kJKR_##B[kNumPairClasses] = LGB_ROW(jkr_entry, B);

#define LGB_CP_TABLES(B)                                   \
  extern const CPFn kCP64_##B[kNumPairClasses];                          \
  extern const CPFn kCP32_##B[kNumPairClasses];                          \
  const CPFn kCP64_##B[kNumPairClasses] = LGB_ROW(cp_entry, double, B); \
  const CPFn kCP32_##B[kNumPairClasses] = LGB_ROW(cp_entry, float, B);

#define LGB_IT_TABLE(B)                      \
  extern const ITFn kIT_##B[kNumPairClasses];              \
  extern const MXFn kMX_##B[kNumPairClasses];              \
  const ITFn kIT_##B[kNumPairClasses] = LGB_ROW(it_entry, B); \
  const MXFn kMX_##B[kNumPairClasses] = LGB_ROW(mx_entry, B);

}  // namespace lgb
