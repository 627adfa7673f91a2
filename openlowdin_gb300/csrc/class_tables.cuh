// Launch-table entries of the class-templated kernels.  Each k_<kind>_c<B>.cu
// translation unit instantiates the kernels of one kind for bra pair class B
// and every ket pair class, so the classes compile in parallel.  Entries are
// null where the generic runtime-class kernels take over (total angular
// momentum above kTemplatedMaxL) or where a kernel is never used (J/K with the
// ket class above the bra class).
#pragma once
#include "fock_kernels.cuh"

namespace lgb {

template <int B, int K>
constexpr bool templated_class() { return pc_L(B) + pc_L(K) <= kTemplatedMaxL; }

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

#define LGB_ROW6(F, ...) \
  { F<__VA_ARGS__, 0>(), F<__VA_ARGS__, 1>(), F<__VA_ARGS__, 2>(), F<__VA_ARGS__, 3>(), F<__VA_ARGS__, 4>(), F<__VA_ARGS__, 5>() }

#define LGB_JK_TABLES(B)                                   \
  extern const JKFn kJK64_##B[6];                          \
  extern const JKFn kJK32_##B[6];                          \
  extern const JKFn kJKR_##B[6];                           \
  const JKFn kJK64_##B[6] = LGB_ROW6(jk_entry, double, B); \
  const JKFn kJK32_##B[6] = LGB_ROW6(jk_entry, float, B);  \
  const JKFn kJKR_##B[6] = LGB_ROW6(jkr_entry, B);

#define LGB_CP_TABLES(B)                                   \
  extern const CPFn kCP64_##B[6];                          \
  extern const CPFn kCP32_##B[6];                          \
  const CPFn kCP64_##B[6] = LGB_ROW6(cp_entry, double, B); \
  const CPFn kCP32_##B[6] = LGB_ROW6(cp_entry, float, B);

#define LGB_IT_TABLE(B)                      \
  extern const ITFn kIT_##B[6];              \
  extern const MXFn kMX_##B[6];              \
  const ITFn kIT_##B[6] = LGB_ROW6(it_entry, B); \
  const MXFn kMX_##B[6] = LGB_ROW6(mx_entry, B);

}  // namespace lgb
