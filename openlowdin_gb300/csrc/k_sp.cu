// Instantiations and launchers of the class-templated kernels for s and p
// shells (every quartet class built from the pair classes ss, ps, pp).
#include "fock_kernels.cuh"

namespace lgb {

namespace {

constexpr int kSPClasses = 3;  // pair classes handled here: 0 (ss), 1 (ps), 2 (pp)

using JKFn = void (*)(const JKTask *, TaskLaunch);
using CPFn = void (*)(const CPTask *, TaskLaunch);
using ITFn = void (*)(ITParams);
using SZFn = void (*)(SchwarzParams);

template <typename R, int B, int K>
constexpr JKFn jkf() { return &jk_tasks_kernel<R, pc_la(B), pc_lb(B), pc_la(K), pc_lb(K)>; }
template <typename R, int B, int K>
constexpr CPFn cpf() { return &cp_tasks_kernel<R, pc_la(B), pc_lb(B), pc_la(K), pc_lb(K)>; }
template <int B, int K>
constexpr ITFn itf() { return &it_kernel<pc_la(B), pc_lb(B), pc_la(K), pc_lb(K)>; }

#define ROW3(F, R, B) {F<R, B, 0>(), F<R, B, 1>(), F<R, B, 2>()}
const JKFn kJK64[3][3] = {ROW3(jkf, double, 0), ROW3(jkf, double, 1), ROW3(jkf, double, 2)};
const JKFn kJK32[3][3] = {ROW3(jkf, float, 0), ROW3(jkf, float, 1), ROW3(jkf, float, 2)};
const CPFn kCP64[3][3] = {ROW3(cpf, double, 0), ROW3(cpf, double, 1), ROW3(cpf, double, 2)};
const CPFn kCP32[3][3] = {ROW3(cpf, float, 0), ROW3(cpf, float, 1), ROW3(cpf, float, 2)};
#undef ROW3
const ITFn kIT[3][3] = {{itf<0, 0>(), itf<0, 1>(), itf<0, 2>()},
                        {itf<1, 0>(), itf<1, 1>(), itf<1, 2>()},
                        {itf<2, 0>(), itf<2, 1>(), itf<2, 2>()}};
const SZFn kSZ[3] = {&schwarz_kernel<0, 0>, &schwarz_kernel<1, 0>, &schwarz_kernel<1, 1>};

const dim3 kBlock(32, kWarpsPerBlock);

}  // namespace

bool class_supported(int pcb, int pck) { return pcb >= 0 && pck >= 0 && pcb < kSPClasses && pck < kSPClasses; }

cudaError_t launch_jk_tasks(int pcb, int pck, bool fp32, const JKTask *dtasks, const TaskLaunch &tl,
                            cudaStream_t s) {
  if (!class_supported(pcb, pck)) return cudaErrorNotSupported;
  if (tl.ntasks <= 0 || tl.nblocks <= 0) return cudaSuccess;
  JKFn f = fp32 ? kJK32[pcb][pck] : kJK64[pcb][pck];
  f<<<tl.nblocks, kBlock, 0, s>>>(dtasks, tl);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_cp_tasks(int pcb, int pck, bool fp32, const CPTask *dtasks, const TaskLaunch &tl,
                            cudaStream_t s) {
  if (!class_supported(pcb, pck)) return cudaErrorNotSupported;
  if (tl.ntasks <= 0 || tl.nblocks <= 0) return cudaSuccess;
  CPFn f = fp32 ? kCP32[pcb][pck] : kCP64[pcb][pck];
  f<<<tl.nblocks, kBlock, 0, s>>>(dtasks, tl);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_it(int pcb, int pck, const ITParams &p, cudaStream_t s) {
  if (!class_supported(pcb, pck)) return cudaErrorNotSupported;
  if (p.nbra <= 0 || p.nket <= 0) return cudaSuccess;
  const dim3 grid((unsigned)((p.nket + 31) / 32), (unsigned)((p.nbra + kWarpsPerBlock - 1) / kWarpsPerBlock));
  kIT[pcb][pck]<<<grid, kBlock, 0, s>>>(p);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_schwarz(int pc, const SchwarzParams &p, cudaStream_t s) {
  if (pc < 0 || pc >= kSPClasses) return cudaErrorNotSupported;
  if (p.np <= 0) return cudaSuccess;
  kSZ[pc]<<<(p.np + 127) / 128, 128, 0, s>>>(p);
  count_launches(1);
  return cudaGetLastError();
}

}  // namespace lgb
