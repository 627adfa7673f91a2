// Launch parameters and host-side launchers of the integral kernels.
//
// The two-particle (J/K) and inter-species coupling builds run from task
// lists: a task is one (bra pair-class range) x (ket pair-class range) block of
// quartets of one species (J/K) or of one species pair (coupling).  All tasks of
// the same quartet class -- across species, species pairs and molecules of a
// batch -- go into one launch; block b of the flattened grid finds its task by
// binary search on the tasks' first-block offsets.
#pragma once
#include <cuda_bf16.h>

#include <cstring>
#include <mutex>
#include <utility>
#include <vector>

#include "common.cuh"

namespace lgb {

// Per-device set-up (kernel attributes such as the dynamic shared-memory
// limit are properties of a device): raise(level) runs f() on the current
// device when that device has not yet been set up to at least `level`, under
// a lock, so host threads calling the library at once and processes using
// several devices are both served.
class PerDeviceLevel {
 public:
  template <typename F>
  cudaError_t raise(long long level, F &&f) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lk(mu_);
    for (auto &d : done_)
      if (d.first == dev) {
        if (d.second >= level) return cudaSuccess;
        e = f();
        if (e == cudaSuccess) d.second = level;
        return e;
      }
    e = f();
    if (e == cudaSuccess) done_.push_back({dev, level});
    return e;
  }

 private:
  std::mutex mu_;
  std::vector<std::pair<int, long long>> done_;
};

// pair class id of a canonical pair (la >= lb): (0,0)=0 (1,0)=1 (1,1)=2 (2,0)=3 (2,1)=4 (2,2)=5
__host__ __device__ constexpr int pair_class(int la, int lb) { return la * (la + 1) / 2 + lb; }
constexpr int kNumPairClasses = (kMaxL + 1) * (kMaxL + 2) / 2;
__host__ __device__ constexpr int pc_la(int pc) { return pc >= 6 ? 3 : (pc >= 3 ? 2 : (pc >= 1 ? 1 : 0)); }
__host__ __device__ constexpr int pc_lb(int pc) { return pc - pc_la(pc) * (pc_la(pc) + 1) / 2; }

constexpr int kWarpsPerBlock = 4;  // bra pairs per block (one per warp); 32 kets per warp

struct BoysTables {
  const double *f64;
  const float *f32;
};

// Fields of the structure-of-arrays copy of a pair list's FP32 records
// (one-primitive pairs): field k of pair i at soa[k * npairs + i].  Shell and
// function indices are packed as a | b << 16 in the bits of a float.
enum SoaField {
  kSoaQ, kSoaShells, kSoaFuncs, kSoaP, kSoaInvP, kSoaKt, kSoaPx, kSoaPy, kSoaPz,
  kSoaPAx, kSoaPAy, kSoaPAz, kSoaABx, kSoaABy, kSoaABz, kSoaFields
};
inline float __int_as_float_host(int v) {
  float f;
  static_assert(sizeof(f) == sizeof(v), "32-bit float");
  memcpy(&f, &v, sizeof(f));
  return f;
}

// One J/K task: quartets (bra in [bra0, bra0+nbra), ket in [ket0, ket0+nket))
// of one species' significant pairs.
// Every array exists in FP64 (used by the FP64 kernels) and FP32 (used by the
// FP32 kernels of the mixed-precision path).
struct JKTask {
  const PairRec *pairs;
  const PrimRec *prims;
  const PairRec32 *pairs32;
  const PrimRec32 *prims32;
  const double *Ds;       // norma-scaled density N D N, n x n row-major
  const float *Ds32;
  const double *Dn;       // max |D| of each shell block, nsh x nsh
  const float *Dn32;
  double *Gacc;           // n x n accumulator (symmetrised by the finaliser)
  float *Gacc32;          // FP32 kernels accumulate here (added by the finaliser)
  unsigned long long *count;  // quartets evaluated (may be null)
  const int *active;      // the task's system is built while *active != 0 (null: always)
  double hf;              // 0.5 * exchange factor
  float hf32;             // the same in FP32
  int bra0, nbra, ket0, nket;
  int n, nsh;
  int triangle;           // same pair class: only ket position <= bra position
  int screen;             // Schwarz x density screening (electrons only)
  int blk0;               // first flattened block of the task
  int nbx;                // blocks along the ket axis
  int rblk0;              // first block of the task in a bra-row launch (one block per bra pair)
  const float *soa32;     // structure-of-arrays FP32 pair records (null: use pairs32 / prims32)
  int npairs;             // pairs in the species' list (the field stride of soa32)
  // pair-indexed ket data of the FP32 row kernels (null: read the n x n
  // matrices), element e of the ket at class position k at [e * nket + k]:
  // the ket's block of Ds32, its Coulomb (J34) accumulator, and (indexed by
  // pair record) its shell-block norm
  const float *Dp32;
  float *Jp32;
  const float *DnP32;
  // largest element of Dn32 (null: unknown).  Pair records are sorted by
  // decreasing Schwarz factor inside a class, so Q(first bra) Q(first ket)
  // Dnmax32 bounds every quartet bound of a tile or of a ket range after it:
  // the mixed launches leave ranges that bound cannot reach at once
  const float *Dnmax32;
};

// One coupling task: quartets (A pair | B pair) of two species; accumulates
// JA += scale * sum D_B (..) and JB += scale * sum D_A (..).
struct CPTask {
  const PairRec *pa;
  const PrimRec *pra;
  const PairRec *pb;
  const PrimRec *prb;
  const PairRec32 *pa32;
  const PrimRec32 *pra32;
  const PairRec32 *pb32;
  const PrimRec32 *prb32;
  const double *DsA;      // norma-scaled density of A (feeds JB), null if JB is null
  const double *DsB;      // norma-scaled density of B (feeds JA), null if JA is null
  const float *DsA32;
  const float *DsB32;
  double *JA;             // nA x nA full symmetric accumulator (or null)
  double *JB;             // nB x nB (or null)
  float *JA32;            // FP32 accumulators of the FP32 kernels
  float *JB32;
  const float *DnA32;     // shell-block max |D| of A and B (mixed-precision split)
  const float *DnB32;
  unsigned long long *count;  // quartets evaluated (may be null)
  const int *active;      // the task's system is built while *active != 0 (null: always)
  int nshA, nshB;
  double scale;           // q_A q_B (1 for the reference-shaped calls)
  float scale32;          // the same in FP32
  int bra0, nbra, ket0, nket;
  int nA, nB;
  int blk0, nbx;
};

struct TaskLaunch {
  int ntasks;
  int nblocks;            // total flattened blocks
  int nrblocks;           // bra-row launches: total bra pairs of the tasks
  int rows_n, rows_nsh;   // bra-row launches: largest basis and shell count of the tasks
  int rows_pref;          // FP32 half of a mixed launch: -1 size rule, 0 jk_tasks_kernel, 1 bra-row kernel
  double eps;             // screening threshold
  double split;           // mixed precision: quartets with bound >= split run in FP64
  int lower;              // 1: this launch takes the quartets below split
  double cut;             // coupling: |raw| < cut is dropped
  float skip;             // mixed launches: quartets whose density-weighted bound is below skip are dropped
  // FP32 copies of the thresholds and the mixed flag (split > 0), so that the
  // kernels issue no FP64 conversion or comparison for them
  int mixed;
  float eps32, split32, cut32;
  BoysTables boys;
};
inline void set_fp32_copies(TaskLaunch &tl) {
  tl.mixed = tl.split > 0.0;
  tl.eps32 = (float)tl.eps;
  tl.split32 = (float)tl.split;
  tl.cut32 = (float)tl.cut;
}

// Kernel entry types of the class-templated launch tables (class_tables.cuh);
// null entries are served by the block-cooperative kernels (classes of total
// angular momentum above kTemplatedMaxL).
using JKFn = void (*)(const JKTask *, TaskLaunch);
// FP32 J/K kernels that keep the bra pair's rows of D and of the exchange
// output in shared memory (jk32_row_kernel), one block per bra pair
constexpr int kRowWarps = 4;
constexpr int kRowMaxSmem = 200 * 1024;
// shared rows per column: the bra shells' NA + NB rows padded to an odd count
// (an odd column pitch spreads random columns over all 32 banks)
__host__ __device__ constexpr int row_pitch(int nrows) { return nrows | 1; }
__host__ __device__ constexpr size_t row_smem_bytes(int nrows, int n, int nsh) {
  return (size_t)(2 * row_pitch(nrows) * n + nsh) * sizeof(float);
}
using CPFn = void (*)(const CPTask *, TaskLaunch);
struct ITParams;
using ITFn = void (*)(ITParams);
__host__ __device__ constexpr int pc_L(int pc) { return pc_la(pc) + pc_lb(pc); }
// classes above this total angular momentum use the block-cooperative kernels
// (the fully unrolled one-thread-per-quartet kernels of heavier classes spill)
constexpr int kTemplatedMaxL = 4;

// First-quarter transform A[nu][lam][sig] += sum_mu C_p(mu) (mu nu|lam sig).
struct ITParams {
  const PairRec *pa;
  const PrimRec *pra;
  int bra0, nbra;
  const PairRec *pb;
  const PrimRec *prb;
  int ket0, nket;
  int intra;              // 1: one species (triangle + permutational orbit), 0: coupling
  int triangle;
  const double *Dn;       // screening (intra electrons only)
  int nsh;
  int screen;
  double eps;
  const double *Cs;       // norma-scaled coefficient row of orbital p (bra species)
  int nA, nB;             // output dims [nA][nB][nB]
  double *A;
  BoysTables boys;
  double cut;             // raw values with |v| <= cut are dropped (1e-10)
};

// Geminal (G12) two-particle matrices for the operator sum_k c_k exp(-g_k r12^2):
// intra-species (six-update digestion of one species, every quartet of the
// significant pairs, no screening) or inter-species (J of the bra species from
// the ket species' density, raw |v| < cut dropped, no quartet skipped).
struct G12Params {
  const PairRec *pa;
  const PrimRec *pra;
  int bra0, nbra;
  const PairRec *pb;
  const PrimRec *prb;
  int ket0, nket;
  int intra;              // 1: one species, 0: coupling
  int triangle;           // ket position <= bra position only
  const double *Ds;       // norma-scaled density: intra n x n, coupling nB x nB (ket species)
  double *Gacc;           // accumulator of the bra species (n x n)
  int n, nB;
  double hf;              // 0.5 * exchange factor (intra)
  double cut;             // coupling: raw values with |v| < cut are dropped (1e-10)
  const double *gem;      // {count, exponents..., coefficients...} in device memory
};
cudaError_t launch_g12(int pcb, int pck, const G12Params &p, cudaStream_t s);

struct SchwarzParams {
  const PairRec *pairs;
  const PrimRec *prims;
  int p0, np;
  double *Q;              // per pair record
  BoysTables boys;
};

// MP2 transform input: raw integrals (mu nu|lam sig) of every significant bra
// pair and the ket pairs of one column batch, written to
// X[mu][col][nu] (both bra orientations), col = colbase[ket pair] + c * ND + d
// for ket components (c, d); quartets that the screening drops and raw values
// with |v| <= cut stay at the zero the caller cleared X to.
struct MXParams {
  const PairRec *pairs;   // bra pairs (species A)
  const PrimRec *prims;
  const PairRec *kpairs;  // ket pairs (species B; A's own list for one species)
  const PrimRec *kprims;
  int bra0, nbra;
  int ket0, nket;
  const int *colbase;     // per pair record: first column of its components
  int col_first;          // first column of the batch
  const double *Dn;       // density screening (electrons)
  int nsh;
  int screen;
  double eps;
  double cut;
  int n;                  // basis functions
  int ncol;               // columns of the batch
  double *X;              // FP64 output X[mu][col][nu], or (X null)
  __nv_bfloat16 *Xp[3];   // split-BF16 output Xt[col * Kp + nu][mu] (K-major for the tensor cores)
  int np;                 // pieces of the split output
  int Kp;                 // padded function count of the split layout
  BoysTables boys;
};
using MXFn = void (*)(MXParams);

// blocks of one task (grid tile of 32 kets x kWarpsPerBlock bras)
inline int task_nbx(int nket) { return (nket + 31) / 32; }
inline int task_nby(int nbra) { return (nbra + kWarpsPerBlock - 1) / kWarpsPerBlock; }

// launchers (every class with l <= kMaxL)
cudaError_t launch_jk_tasks(int pcb, int pck, bool fp32, const JKTask *dtasks, const TaskLaunch &tl,
                            cudaStream_t s);
// whether the FP32 launch of class (pcb, pck) over species of up to n
// functions / nsh shells runs on the bra-row kernel
bool jk_rows_used(int pcb, int pck, int n, int nsh);
cudaError_t launch_cp_tasks(int pcb, int pck, bool fp32, const CPTask *dtasks, const TaskLaunch &tl,
                            cudaStream_t s);
cudaError_t launch_it(int pcb, int pck, const ITParams &p, cudaStream_t s);
cudaError_t launch_schwarz(int pc, const SchwarzParams &p, cudaStream_t s);
cudaError_t launch_mp2x(int pcb, int pck, const MXParams &p, cudaStream_t s);
// MP2 transform helpers (k_mp2.cu).  Coefficients: C[p][mu] rows are
// orbitals; Co[mu][i] = norma[mu] C[n_frozen + i][mu] (n x o), Cv[mu][a] =
// norma[mu] C[n_occ + a][mu] (n x v); the *32 outputs may be null.
cudaError_t launch_mp2_coeffs(const double *C, const double *norma, int n, int n_frozen, int n_occ, double *Co,
                              double *Cv, float *Co32, float *Cv32, cudaStream_t s);
// Z[lam][sig][a] = Y[col][a] for col's (lam, sig) and, when the column's shell
// pair is off-diagonal, Z[sig][lam][a] too; colpair[col] = lam | sig << 16 |
// offdiag << 31 (n < 32768)
template <typename T>
cudaError_t launch_mp2_unpack(const T *Y, const unsigned *colpair, long long ncols, int n, int v, T *Z,
                              cudaStream_t s);
// e2 += sum_{j,a,b} M[j][b][a] (2 M[j][b][a] - M[j][a][b]) / (ei + e_j - e_a - e_b)
// with |M| <= cut read as zero; M[j][b][a] = (ia|jb)
// split-BF16 coefficients (np pieces), K-major and padded to Kp (padding
// cleared by the caller): CoT[i][mu] = norma[mu] C[n_frozen + i][mu], CvT[a][mu] = norma[mu] C[n_occ + a][mu]
cudaError_t launch_mp2_coeffs_bf16(const double *C, const double *norma, int n, int n_frozen, int n_occ, int Kp,
                                   int np, __nv_bfloat16 *const *CoT, __nv_bfloat16 *const *CvT, cudaStream_t s);
// Zt[a][sig][lam] (split BF16, rows of Kp) = Y'[a][lam sig column] for every
// entry of the sig-row lists: rowptr[sig] .. rowptr[sig+1] hold (lam | sig << 16, col);
// Yp points at Y'[0][i][0], a-rows ystride apart
cudaError_t launch_mp2_unpack_csr(const float *Yp, long long ystride, const int *rowptr, const int2 *ent, int n,
                                  int Kp, int v, int np, __nv_bfloat16 *const *Z, cudaStream_t s);
// coupling pair energies: e2 += factor sum_{j,b,a} M[j][b][a]^2 / (ei + eo[j] - evA[a] - evB[b]),
// M [o][vB][vA], |M| <= cut read as zero
template <typename T>
cudaError_t launch_mp2_energy_coupling(const T *M, int o, int vB, int vA, double ei, const double *eo,
                                       const double *evA, const double *evB, double cut, double factor, double *e2,
                                       cudaStream_t s);
template <typename T>
cudaError_t launch_mp2_energy(const T *M, int o, int v, double ei, const double *eo, const double *ev, double cut,
                              double *e2, cudaStream_t s);
bool class_supported(int pcb, int pck);
inline bool class_generic(int pcb, int pck) { return pc_L(pcb) + pc_L(pck) > kTemplatedMaxL; }

// small kernels (the *32 arguments may be null)
cudaError_t launch_prepare_density(const double *D, const double *norma, const int *shell_of, int n, int nsh,
                                   double *Ds, float *Ds32, double *Dn, float *Dn32, cudaStream_t s);
cudaError_t launch_scale_density(const double *D, const double *norma, int n, double *Ds, float *Ds32,
                                 cudaStream_t s);
cudaError_t launch_symmetrize(const double *Gacc, const float *Gacc32, const double *norma, int n, double scale,
                              double *G, cudaStream_t s);
cudaError_t launch_coupling_extract(const double *J, const float *J32, const double *norma, int n, double scale,
                                    int lower_only, double *out, cudaStream_t s);

// batched element-wise work over many species of a batch
struct SpeciesSlot {
  const double *P;        // density (input)
  double *Ds;             // N P N
  float *Ds32;
  double *Dn;             // shell-block max |P| (null: not needed)
  float *Dn32;
  const double *norma;
  const int *shell_of;
  double *Gacc, *Jacc;    // accumulators
  float *Gacc32, *Jacc32;
  double *G, *J;          // outputs (G may be null)
  double gscale;          // 0.25 q^2 for the two-particle matrix
  int n, nsh;
  int ld;                 // row stride of P, G and J (>= n; the arenas are n x n)
  long long off;          // prefix of n*n over the slots
  const int *active;      // the slot's system is built while *active != 0 (null: always)
  float *Dnmax32;         // largest element of Dn32 (null: not computed)
};
cudaError_t launch_prepare_batch(const SpeciesSlot *slots, int nslots, long long total, cudaStream_t s);
// Dnmax32 of every slot that has Dn32 (after launch_prepare_batch; the
// Dnmax32 values must be zero beforehand); max_nsh: largest nsh of a slot
cudaError_t launch_dn_max_batch(const SpeciesSlot *slots, int nslots, int max_nsh, cudaStream_t s);
// *out = max of Dn32[0 .. nsh * nsh) (set to zero here first)
cudaError_t launch_dn_max(const float *Dn32, int nsh, float *out, cudaStream_t s);

// pair-indexed copies of a species' FP32 density for the FP32 row kernels:
// for every significant pair (class c, position k in its class) and element e
// of its block, Dp32[pe_base[c] + e * count_c + k] = Ds32 at the block's
// element, Jp32 there = 0, and DnP32[pair] = Dn32 of its shell block;
// pair_scatter adds the Jp32 accumulators into Gacc32 after the build
struct PairSlot {
  const PairRec32 *pairs;
  int npairs;
  long long poff;         // prefix of npairs over the slots
  int start[kNumPairClasses + 1];
  long long pe_base[kNumPairClasses];
  const float *Ds32, *Dn32;
  float *Gacc32;
  int n, nsh;
  float *Dp32, *Jp32, *DnP32;
  const int *active;      // slot's system flag (null: always built)
};
cudaError_t launch_pair_gather(const PairSlot *slots, int nslots, long long total_pairs, cudaStream_t s);
cudaError_t launch_pair_scatter(const PairSlot *slots, int nslots, long long total_pairs, cudaStream_t s);
// elements of the pair-indexed arrays of a pair list (class starts `start`),
// and the per-class bases
long long pair_elements(const int *start, long long *pe_base);
cudaError_t launch_finalize_batch(const SpeciesSlot *slots, int nslots, long long total, cudaStream_t s);

// Split-BF16 operands: x ~= p[0] + p[1] (+ p[2]), each piece the BF16
// rounding of what the previous pieces leave.  Two pieces keep ~16 bits of x,
// three ~24 bits.
constexpr int kMaxPieces = 3;
template <typename T>
__device__ __forceinline__ void bf16_pieces(T x, int np, __nv_bfloat16 *p) {
#pragma unroll
  for (int k = 0; k < kMaxPieces; ++k)
    if (k < np) {
      p[k] = __float2bfloat16_rn((float)x);
      x -= (T)__bfloat162float(p[k]);
    }
}
// pieces of hi + lo (an FP32 pair) without FP64 arithmetic: hi - p0 is exact,
// so the residual carries the pair to ~2^-32 relative
__device__ __forceinline__ void bf16_pieces_pair(float hi, float lo, int np, __nv_bfloat16 *p) {
  p[0] = __float2bfloat16_rn(hi + lo);
  float r = (hi - __bfloat162float(p[0])) + lo;
#pragma unroll
  for (int k = 1; k < kMaxPieces; ++k)
    if (k < np) {
      p[k] = __float2bfloat16_rn(r);
      r -= __bfloat162float(p[k]);
    }
}
struct Bf16Split {
  const __nv_bfloat16 *p[kMaxPieces];
};

// Split-BF16 tensor-core GEMM (k_gemm.cu):
//   C_z[m][n] = sum_k A[z * a_batch_rows + m][k] B[z * b_batch_rows + n][k]
// A and B in np pieces (rows of Kp BF16, Kp a multiple of 64, zero beyond the
// true K); a_rows / b_rows: rows of the whole arrays (loads past them read
// zeros).  np = 2: products p0q0 + p0q1 + p1q0 (3 per K step, ~2^-16
// relative per product); np = 3: adds p1q1 + p0q2 + p2q0 (6, ~2^-24).  FP32
// accumulation.
struct GemmOut {
  float *C;                   // FP32 output, or (C null)
  __nv_bfloat16 *Cp[kMaxPieces];  // split output in np pieces
  long long ldc;              // row stride of the output
  long long c_batch;          // element offset of batch z
  long long grp_rows, grp_stride, row0;  // output row of m: (m / grp_rows) * grp_stride + m % grp_rows + row0
                                          // (grp_rows 0: row m + row0)
  long long grp_cols, gcol_stride, col0; // output column of n: (n / grp_cols) * gcol_stride + n % grp_cols + col0
                                          // (grp_cols 0: column n)
};
cudaError_t launch_gemm_split(const Bf16Split &A, long long a_rows, const Bf16Split &B, long long b_rows, int Kp,
                              int M, int N, int batch, int a_batch_rows, int b_batch_rows, int np,
                              const GemmOut &out, int *derr, cudaStream_t s);
// Same product with three pieces per operand, eight products and per-slab
// FP64 accumulation (about FP64-level error on the kept ~24 bits per
// operand): for contractions with strong cancellation.  Output in three pieces
// or FP32.
cudaError_t launch_gemm_precise(const Bf16Split &A, long long a_rows, const Bf16Split &B, long long b_rows, int Kp,
                                int M, int N, int batch, int a_batch_rows, int b_batch_rows, const GemmOut &out,
                                int *derr, cudaStream_t s);
// src [rows][cols] (row stride lds) -> np pieces [rows][ldo]
template <typename T>
cudaError_t launch_split_bf16(const T *src, long long rows, int cols, long long lds, int np, __nv_bfloat16 *const *out,
                              long long ldo, cudaStream_t s);

// one-electron matrices of one species (k_onebody.cu)
struct DevShell {
  int l, nprim, p0, pad;
  double O[3];
};
struct OneBodyParams {
  const DevShell *shells;
  const double *alpha, *cn;   // per primitive: exponent, coefficient x primitive norm
  const int *first;           // first function of each shell
  const double *norma;
  int nsh, n;
  int ncharge;
  const double *Z, *R;        // device point charges and positions (3 per charge)
  double *S, *T, *V;          // n x n outputs (any may be null)
  BoysTables boys;
};
cudaError_t launch_one_body(const OneBodyParams &p, cudaStream_t s);

// x[i] = deterministic pseudo-random values in [-1, 1) (benchmark operands)
cudaError_t launch_fill_hash(float *x, long long n, unsigned seed, cudaStream_t s);

// number of kernels this library has launched (process-wide)
void count_launches(long long n);
long long launch_count();

// FMA throughput of the GPU (independent FMA chains on every SM), TFLOP/s
cudaError_t measure_fma_tflops(bool fp64, double *tflops);
cudaError_t launch_scale_cube(double *A, const double *normA, const double *normB, int nA, int nB,
                              cudaStream_t s);

}  // namespace lgb
