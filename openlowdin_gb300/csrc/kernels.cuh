// Launch parameters and host-side launchers of the integral kernels.
#pragma once
#include "common.cuh"

namespace lgb {

// pair class id of a canonical pair (la >= lb): (0,0)=0 (1,0)=1 (1,1)=2 (2,0)=3 (2,1)=4 (2,2)=5
__host__ __device__ constexpr int pair_class(int la, int lb) { return la * (la + 1) / 2 + lb; }
constexpr int kNumPairClasses = (kMaxL + 1) * (kMaxL + 2) / 2;
__host__ __device__ constexpr int pc_la(int pc) { return pc >= 3 ? 2 : (pc >= 1 ? 1 : 0); }
__host__ __device__ constexpr int pc_lb(int pc) { return pc - pc_la(pc) * (pc_la(pc) + 1) / 2; }

struct BoysTables {
  const double *f64;
  const float *f32;
};

// Intra-species J/K build over the quartets (bra pair, ket pair) of one class.
struct JKParams {
  const PairRec *pairs;
  const PrimRec *prims;
  int bra0, nbra, ket0, nket;
  int triangle;           // same pair class: only ket position <= bra position
  const double *Ds;       // norma-scaled density N D N, n x n row-major
  int n;
  const double *Dn;       // max |D| of each shell block, nsh x nsh
  int nsh;
  int screen;             // Schwarz x density screening (electrons only)
  double eps;             // screening threshold
  double hf;              // 0.5 * exchange factor
  double *Gacc;           // n x n accumulator (raw-weighted; symmetrised later)
  BoysTables boys;
  unsigned long long *nquartets;  // quartets evaluated (may be null)
  // mixed precision: quartets with bound >= split go to FP64, the rest to FP32;
  // split <= 0 sends every quartet to the precision of the kernel.
  double split;
  int lower;              // 1: this launch takes the quartets below split
};

// Fused inter-species Coulomb coupling over (A pair | B pair) quartets:
// J_A += D_B contraction and/or J_B += D_A contraction in one pass.
struct CouplingParams {
  const PairRec *pa;
  const PrimRec *pra;
  int bra0, nbra;
  const PairRec *pb;
  const PrimRec *prb;
  int ket0, nket;
  const double *DsA;      // norma-scaled density of A (feeds J_B), may be null
  const double *DsB;      // norma-scaled density of B (feeds J_A), may be null
  int nA, nB;
  double *JA;             // nA x nA full symmetric accumulator (or null)
  double *JB;             // nB x nB (or null)
  BoysTables boys;
  double cut;             // |raw| < cut is dropped (1e-10)
};

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

struct SchwarzParams {
  const PairRec *pairs;
  const PrimRec *prims;
  int p0, np;
  double *Q;              // per pair record
  BoysTables boys;
};

// launchers (return cudaError_t of the launch; the kernels exist for every
// class with la, lb, lc, ld <= kMaxL)
cudaError_t launch_jk(int pcb, int pck, bool fp32, const JKParams &p, cudaStream_t s);
cudaError_t launch_coupling(int pcb, int pck, bool fp32, const CouplingParams &p, cudaStream_t s);
cudaError_t launch_it(int pcb, int pck, const ITParams &p, cudaStream_t s);
cudaError_t launch_schwarz(int pc, const SchwarzParams &p, cudaStream_t s);
bool class_supported(int pcb, int pck);

// small kernels
cudaError_t launch_prepare_density(const double *D, const double *norma, const int *shell_of, int n, int nsh,
                                   double *Ds, double *Dn, cudaStream_t s);
cudaError_t launch_scale_density(const double *D, const double *norma, int n, double *Ds, cudaStream_t s);
cudaError_t launch_symmetrize(const double *Gacc, const double *norma, int n, double scale, double *G,
                              cudaStream_t s);
cudaError_t launch_coupling_extract(const double *J, const double *norma, int n, double scale, int lower_only,
                                    double *out, cudaStream_t s);
// number of kernels this library has launched (process-wide)
void count_launches(long long n);
long long launch_count();

// FMA throughput of the GPU (independent FMA chains on every SM), TFLOP/s
cudaError_t measure_fma_tflops(bool fp64, double *tflops);
cudaError_t launch_scale_cube(double *A, const double *normA, const double *normB, int nA, int nB,
                              cudaStream_t s);

}  // namespace lgb
