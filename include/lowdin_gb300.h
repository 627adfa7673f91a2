/*
 * lowdin_gb300.h -- C ABI of liblowdin_gb300.so, a GB300 (sm_103a) drop-in for
 * openLOWDIN's direct two-particle integral interface.
 *
 * Part 1 repeats the reference's extern "C" interface (src/ints/Libint2Iface.h,
 * lines 357-449; the Fortran binding is src/ints/Libint2Interface.f90:165-373)
 * with the same names, argument order, passing convention and layouts:
 *   - handles are created by LibintInterface_new and destroyed by _del;
 *   - shells are added in basis order; coefficients are the raw basis-file
 *     contraction coefficients (the library applies the primitive norm of the
 *     x^l component and renormalises every Cartesian component to unit
 *     self-overlap, src/ints/Libint2Iface.cpp:79-128);
 *   - matrices are n x n, read and written row-major (the Fortran caller
 *     passes column-major arrays; densities and two-particle matrices are
 *     symmetric so the transposition is harmless);
 *   - `factor` and `p` are passed by reference (C++ double& / int&): in C they
 *     are pointers, in C++ references; the ABI is the same;
 *   - results are fully overwritten; calls are synchronous with respect to the
 *     host buffers.
 * All reference functions return void as in the reference.  Errors (CUDA
 * failures, unsupported requests) are reported through LowdinGB300_last_error()
 * and printed on stderr; with LOWDIN_GB300_STRICT=1 in the environment the
 * process aborts on the first error, as the reference aborts in libint.
 *
 * Part 2 adds device-resident entry points (pointers are device pointers) used
 * by batched and served SCF drivers that keep densities and Fock matrices in
 * HBM between iterations.
 */
#ifndef LOWDIN_GB300_H
#define LOWDIN_GB300_H

#ifdef __cplusplus
#include <cstddef>
#define LGB_REF(T) T &
extern "C" {
#else
#include <stdbool.h>
#include <stddef.h>
#define LGB_REF(T) T *
#endif

typedef struct LibintInterface LibintInterface;

/* ---------------------------------------------------------------- Part 1 --
 * Reference interface, src/ints/Libint2Iface.h:357-449.                      */

/* Libint2Iface.h:364 -- one handle per species; stack_size and parallel are
   accepted and ignored (one CUDA stream per handle replaces the OpenMP pool). */
LibintInterface *LibintInterface_new(const int stack_size, const int id, const bool el, const bool parallel);

/* Libint2Iface.h:367 */
void LibintInterface_del(LibintInterface *lint);

/* Libint2Iface.h:369 -- point charge z at center[3] (used by kind 3 of
   LibintInterface_compute_1body_ints). */
void LibintInterface_add_particle(LibintInterface *lint, const int z, const double *center);

/* Libint2Iface.h:372 */
void LibintInterface_add_shell(LibintInterface *lint, double *alpha, double *coeff, double *origin, int l, int nprim);

/* Libint2Iface.h:375 */
int LibintInterface_get_nbasis(LibintInterface *lint);

/* Libint2Iface.h:377 -- kind 1 overlap, 2 kinetic, 3 attraction to the added
   particles (sum_C z_C <i|1/|r-C||j>); row-major n x n; host computed. */
void LibintInterface_compute_1body_ints(LibintInterface *lint, int integral_kind, double *result);

/* Libint2Iface.h:380 -- builds the significant shell-pair list; the library
   also caches Schwarz factors on the device (they depend on the shells only). */
void LibintInterface_init_2body_ints(LibintInterface *lint);

/* Libint2Iface.h:382 (Libint2Iface.cpp:3510-3526, :418-618) -- two-particle
   matrix G = J[D] + factor K[D] of one species from its density. */
void LibintInterface_compute_2body_direct(LibintInterface *lint, double *dens, double *result, LGB_REF(double) factor);

/* Libint2Iface.h:385 (Libint2Iface.cpp:3528-3549, :620-921) -- first-quarter
   transform of orbital p: result[nu][lam][sig] = sum_mu C(p,mu)(mu nu|lam sig),
   n^3 entries; coeff is n x n row-major, dens is used for screening. */
void LibintInterface_compute_2body_directIT(LibintInterface *lint, double *dens, double *coeff, double *result,
                                            LGB_REF(int) p);

/* Libint2Iface.h:388 -- disk integrals: not provided (reports an error). */
void LibintInterface_compute_2body_disk(LibintInterface *lint, const char *filename, double *dens);

/* Libint2Iface.h:391 (Libint2Iface.cpp:3566-3589, :1111-1294) -- inter-species
   Coulomb matrix of lint's species from olint's density dens (n_o x n_o):
   lower triangle (row >= col) of the row-major n x n result, zero above. */
void LibintInterface_compute_coupling_direct(LibintInterface *lint, LibintInterface *olint, double *dens,
                                             double *result);

/* Libint2Iface.h:395 (Libint2Iface.cpp:3591-3620, :1296-1622) --
   result[nu][lam][sig] = sum_mu C(p,mu)(mu nu|lam sig), mu,nu of lint's
   species (coeff n x n), lam,sig of olint's; n * n_o * n_o entries. */
void LibintInterface_compute_coupling_directIT(LibintInterface *lint, LibintInterface *olint, double *dens,
                                               double *coeff, double *result, LGB_REF(int) p);

/* Libint2Iface.h:399 (Libint2Iface.cpp:1626-1825, wrapper :3625-3658) -- UHF
   alpha/beta Coulomb energy: result[0] = sum_{ij in lint, kl in olint}
   dens(ij) (ij|kl) otherdens(kl) over the coupling integral set (raw
   |v| < 1e-10 dropped, no screening); the two species share one basis in the
   reference's use (E-ALPHA / E-BETA). */
void LibintInterface_compute_alphabeta_direct(LibintInterface *lint, LibintInterface *olint, double *dens,
                                              double *otherdens, double *result);

/* Libint2Iface.h:403 -- not provided. */
void LibintInterface_compute_coupling_disk(LibintInterface *lint, LibintInterface *olint, const char *filename);

/* Libint2Iface.h:407-415 -- G12 (inter-particle potential) integrals on disk:
   not provided. */
void libintinterface_compute_g12_disk(LibintInterface *lint, const char *filename, const double *coefficients,
                                      const double *exponents, const int pot_size);
void libintinterface_compute_g12inter_disk(LibintInterface *lint, LibintInterface *olint, const char *filename,
                                           const double *coefficients, const double *exponents, const int pot_size);

/* Libint2Iface.h:411 (Libint2Iface.cpp:2193-2365, wrapper :3687-3706) --
   direct intra-species matrix of the inter-particle potential
   V(r12) = sum_k coefficients[k] exp(-exponents[k] r12^2) (libint2's
   contracted Gaussian geminal, pot_size terms, exponents >= 0): the loops,
   degeneracies, six updates and 0.25 (G + G^T) of compute_2body_direct over
   every quartet of the significant pairs (no screening); result n x n. */
void libintinterface_compute_g12_direct(LibintInterface *lint, double *dens, double *result, LGB_REF(double) factor,
                                        const double *coefficients, const double *exponents, const int pot_size);

/* Libint2Iface.h:418 (Libint2Iface.cpp:2367-2540, wrapper :3708-3734) --
   inter-species matrix of the same potential: J of lint's species from
   olint's density `dens` (n_o x n_o) over every pair of both species, raw
   |v| < 1e-10 dropped; row >= col triangle of the n x n result, zero above,
   as compute_coupling_direct. */
void libintinterface_compute_g12inter_direct(LibintInterface *lint, LibintInterface *olint, double *dens,
                                             double *result, const double *coefficients, const double *exponents,
                                             const int pot_size);

/* Libint2Iface.h:439-446 -- in-memory all-integral tensors: not provided. */
void LibintInterface_compute_2body_directAll(LibintInterface *lint, double *dens, double *result);
void LibintInterface_compute_coupling_directAll(LibintInterface *lint, LibintInterface *olint, double *dens,
                                                double *result);
void libintinterface_compute_g12_directAll(LibintInterface *lint, double *dens, double *result,
                                           const double *coefficients, const double *exponents, const int pot_size);
void libintinterface_compute_g12inter_directAll(LibintInterface *lint, LibintInterface *olint, double *dens,
                                                double *result, const double *coefficients, const double *exponents,
                                                const int pot_size);

/* ---------------------------------------------------------------- Part 2 --
 * Device-resident extensions (no counterpart in the reference).             */

/* Text of the last error in this process ("" when none); cleared by the call
   of LowdinGB300_clear_error. */
const char *LowdinGB300_last_error(void);
void LowdinGB300_clear_error(void);

/* Point-charge potential V_ij = sum_C Z_C <i|1/|r-R_C||j> (norma applied),
   row-major n x n, host memory. */
void LowdinGB300_potential(LibintInterface *lint, int ncharge, const double *Z, const double *R, double *result);

/* External Gaussian-fit potential of a species (EXTERPOTENTIAL):
   V_ij = sum_k c_k <i| exp(-g_k |r - C_k|^2) |j> (norma applied) for ncomp
   s-type components with coefficients c, exponents g and origins C (3 ncomp,
   bohr); row-major n x n, host memory, computed on the host.  Replaces
   DirectIntegralManager_getExternalPotentialIntegrals
   (src/ints/DirectIntegralManager.f90:848-949), which the reference computes
   in Fortran outside the Libint interface. */
void LowdinGB300_gaussian_potential(LibintInterface *lint, int ncomp, const double *coefficients,
                                    const double *exponents, const double *origins, double *result);

/* Precision of this handle's LibintInterface_compute_2body_direct (host
   buffers, the reference's own call): 0 = FP64 (default, the reference's
   behaviour); 1 = quartets whose Schwarz bound times the density's shell-block
   maximum is below `split` run in FP32, the rest in FP64 (a caller that passes
   density changes gets the incremental mixed-precision build of the
   batched SCF).  The coupling and first-quarter calls stay FP64.  Returns 0, or
   -1 for an unknown precision or a split outside (0, 1). */
int LowdinGB300_set_precision(LibintInterface *lint, int precision, double split);

/* Device-resident two-particle matrix: dG = J[dD] + factor K[dD] (n x n device
   buffers, full symmetric).  precision: 0 = FP64, 1 = mixed (quartets whose
   Schwarz-density bound is below `split` run in FP32, the rest in FP64).
   Work is queued on `stream` (a cudaStream_t, 0 = legacy default); returns 0
   on success, -1 on error (see LowdinGB300_last_error). */
int LowdinGB300_twobody_device(LibintInterface *lint, const double *dD, double *dG, double factor, int precision,
                               double split, void *stream);

/* Device-resident fused coupling of species a and b in one pass over the
   (a pair | b pair) quartets: dJa = J_a[dDb] and dJb = J_b[dDa] (full
   symmetric, either output may be NULL).  fp32 selects FP32 integrals. */
int LowdinGB300_coupling_device(LibintInterface *a, LibintInterface *b, const double *dDa, const double *dDb,
                                double *dJa, double *dJb, int fp32, void *stream);

/* Number of shell quartets evaluated by the last two-particle build of the
   handle (after screening), or -1. */
long long LowdinGB300_last_quartets(LibintInterface *lint);

/* Shell quartets per (bra pair class, ket pair class) of the last two-particle
   build, 100 entries (pair classes ss, ps, pp, ds, dp, dd, fs, fp, fd, ff;
   class (la >= lb) at la (la + 1) / 2 + lb); returns 100 or -1. */
int LowdinGB300_last_class_quartets(LibintInterface *lint, long long *out);

/* Number of shell pairs per pair class (10 entries): significant pairs when
   all_pairs = 0, every unordered pair when 1.  Returns 10 or -1. */
int LowdinGB300_pair_class_counts(LibintInterface *lint, int all_pairs, int *out);

/* Measured FMA throughput of the current GPU in TFLOP/s (fp64 = 1: FP64,
   0: FP32), from independent FMA chains on every SM; -1 on error. */
double LowdinGB300_measure_fma_tflops(int fp64);

/* Batches: many molecular systems, each a list of species handles, built
   together.  For every species k of a system the caller gives device buffers
   dP[k] (density, input), dG[k] (two-particle matrix q^2 (J + f K)[P], may be
   NULL when two_body[k] = 0) and dJ[k] (sum over the other species j of the
   system of q_k q_j J_k[P_j]); charges[k] = q_k, factors[k] = kappa/eta.
   batch_fock queues the whole build on `stream` without waiting on the host
   (a fixed sequence of launches that can be captured in a CUDA graph). */
typedef struct LowdinGB300_Batch LowdinGB300_Batch;
LowdinGB300_Batch *LowdinGB300_batch_new(void);
void LowdinGB300_batch_del(LowdinGB300_Batch *b);
/* returns the index of the system's first species in the batch, -1 on error */
int LowdinGB300_batch_add_system(LowdinGB300_Batch *b, LibintInterface **species, int nspecies,
                                 const double *charges, const double *factors, const int *two_body,
                                 const double **dP, double **dG, double **dJ);
/* Same with a row stride per species: P, G and J of species k are n_k x n_k
   blocks of an ld[k] x ld[k] row-major array (ld[k] >= n_k), so molecules of
   different sizes can share one padded stacked array. ld = NULL: ld[k] = n_k. */
int LowdinGB300_batch_add_system_ld(LowdinGB300_Batch *b, LibintInterface **species, int nspecies,
                                    const double *charges, const double *factors, const int *two_body,
                                    const double **dP, double **dG, double **dJ, const int *ld);
/* builds pair data, task lists and work arenas (synchronises `stream`) */
int LowdinGB300_batch_finalize(LowdinGB300_Batch *b, void *stream);
/* One flag per system (host array, in add order; copied on `stream`): the
   integral launches of a system whose flag is 0 return at once, leaving its
   G and J unwritten (a converged molecule of the batch costs no quartets);
   1 = built; 2 = built, and in mixed builds every quartet of the system is
   evaluated in FP64 (a system whose mixed-precision solution failed its FP64
   check continues in FP64 inside the same batch).  All systems are 1 after
   finalize. */
int LowdinGB300_batch_set_active(LowdinGB300_Batch *b, const int *flags, void *stream);
/* precision bits: 1 = two-particle quartets whose Schwarz-density bound
   Q_ab Q_cd max|D block| is below `split` run in FP32 (the rest FP64); 2 = the
   same split for coupling quartets (bound Q_ab Q_cd max(|D_A|, |D_B|)).
   0 = FP64 throughout. */
int LowdinGB300_batch_fock(LowdinGB300_Batch *b, int precision, double split, void *stream);
/* Mixed builds (precision != 0) also drop the quartets whose density-weighted
   bound (the FP32 bound of the split) is below `skip`: with incremental
   builds from a density change, late iterations then evaluate only the
   quartets the change can move by more than `skip`.  Default 0 (only the
   screening of the plain build). */
int LowdinGB300_batch_set_skip(LowdinGB300_Batch *b, double skip);
/* Autotuner of the mixed builds (no counterpart in the reference): for every
   quartet class whose FP32 half can run on either FP32 kernel (one bra pair
   per block with its exchange rows in shared memory, or one quartet per
   thread), times both on the batch's current densities and keeps the faster
   for the following batch_fock calls (split: the mixed build's split).
   Choices are cached in the process by (class, size bucket); force = 1
   re-times.  Both kernels take the same quartets.  Synchronises `stream`.
   batch_tuning reports the 100 per-class choices (-1 not tuned, 0 one quartet
   per thread, 1 bra rows) and the two timings (ms, -1 where not timed). */
int LowdinGB300_batch_autotune(LowdinGB300_Batch *b, double split, int force, void *stream);
int LowdinGB300_batch_tuning(LowdinGB300_Batch *b, int *choice, float *ms_rows, float *ms_tiles);
/* batch_fock replays a CUDA graph of its launch sequence (captured once per
   precision mode after a first eager build; default on); 0 launches eagerly. */
int LowdinGB300_batch_use_graph(LowdinGB300_Batch *b, int on);
/* quartets evaluated per (bra pair class, ket pair class) by the last J/K
   build and by the last coupling build of the batch (100 entries each;
   synchronise `stream`) */
int LowdinGB300_batch_quartets(LowdinGB300_Batch *b, long long *out, void *stream);
int LowdinGB300_batch_coupling_quartets(LowdinGB300_Batch *b, long long *out, void *stream);

/* Allocation-free two-particle build (no counterpart in the reference).
   Same result as LowdinGB300_twobody_device, for callers that cannot allocate
   device memory once running: a host program whose device memory is owned by
   its own pool, or a serving loop that forbids allocations after warm-up.
   Work buffers live in one static device
   array (LowdinGB300_noalloc_scratch_bytes() bytes, ~9.5 MB, held by every GPU
   that loads the library until the process exits); species are limited to 512
   Cartesian functions, 512 shells and shells up to d (f shells need global
   work arrays for some classes); others are rejected with an error.
   The handle must have been set up with LibintInterface_init_2body_ints (which
   does allocate).  The call uploads its task list from host memory that
   lives only for the call, so it must not be recorded into a CUDA graph
   (stream capture); it queues ordinary work on `stream`.  Every call shares
   the array and clears what it accumulates; calls
   whose work overlaps on the GPU (other streams, other handles) race.
   Returns 0, or -1 with LowdinGB300_last_error() set. */
size_t LowdinGB300_noalloc_scratch_bytes(void);
int LowdinGB300_twobody_device_noalloc(LibintInterface *lint, const double *dD, double *dG, double factor,
                                       int precision, double split, void *stream);

/* Closed-shell MP2 of one electron species with the four-index transform on
   the device (replaces the DIRECT branch of TransformIntegralsC.f90:472-665,
   which calls LibintInterface_compute_2body_directIT once per occupied orbital
   (Libint2Iface.cpp:620-921), and the energy sum of MPFunctions.f90:514-662).
   Same integral set as that path: significant shell pairs, quartets dropped by
   the density screening with dD, raw |v| <= 1e-10 dropped, MO integrals with
   |(ia|jb)| <= 1e-10 read as zero.  dD: device n x n density; dC: device n x n
   coefficients, row p = orbital p (the layout LibintInterface_compute_2body_directIT
   reads); eps: host orbital energies (n); orbitals [n_frozen, n_occ) are the
   active occupied ones, [n_occ, n) the virtual ones.  precision 0: FP64
   throughout (cuBLAS DGEMM for the dense contractions); 1 / 2: the four dense
   contractions as split-BF16 tensor-core products, operands in 2 / 3 BF16
   pieces (LowdinGB300_gemm_bf16_split's engine; with 3 pieces the first
   quarter uses LowdinGB300_gemm_bf16_precise's), integrals and the energy sum
   in FP64.  x_budget_gb bounds the per-batch integral array (0: 8 GB).  Writes E_MP2 to *e2 (host) and
   synchronises `stream`.  Returns 0, or -1 with LowdinGB300_last_error() set. */
int LowdinGB300_mp2_direct(LibintInterface *lint, const double *dD, const double *dC, const double *eps,
                           int n_occ, int n_frozen, int precision, double x_budget_gb, double *e2, void *stream);
/* Inter-species MP2 term of species a and b (APMO; replaces the two-species
   branch of TransformIntegralsC.f90 over LibintInterface_compute_coupling_directIT,
   Libint2Iface.cpp:1296-1622, and the coupling sum of MPFunctions.f90:682-886):
   e2 = factor * sum_{i,a in A; j,b in B} (ia|jb)^2 / (e_i + e_j - e_a - e_b)
   with factor = (q_A q_B)^2 lambda_A lambda_B.  Same integral set as that path
   (no density screening, raw |v| <= 1e-10 dropped, |(ia|jb)| <= 1e-10 read as
   zero).  dCa / dCb: device coefficients (row p = orbital p); eps_a / eps_b:
   host orbital energies; precision as for LowdinGB300_mp2_direct.  Writes
   *e2 and synchronises `stream`.  Returns 0, or -1 with the error set. */
int LowdinGB300_mp2_coupling(LibintInterface *a, LibintInterface *b, const double *dCa, const double *dCb,
                             const double *eps_a, const double *eps_b, int n_occ_a, int n_frozen_a, int n_occ_b,
                             int n_frozen_b, double factor, int precision, double x_budget_gb, double *e2,
                             void *stream);
/* ket-component columns of the last LowdinGB300_mp2_direct / _mp2_coupling call */
long long LowdinGB300_mp2_last_columns(void);
/* LowdinGB300_mp2_direct in FP64 that also writes the transformed integrals
   to `path` in the reference's moint.dat layout (replaces the DIRECT branch of
   TransformIntegralsC_atomicToMolecularOfOneSpecie, TransformIntegralsC.f90:472-665,
   with partialTransform = "MP2", :1489-1501): every (ia|jb) with i <= j
   (b >= a when i == j), |value| > 1e-10, as Fortran sequential unformatted
   records of `stack_size` (the reference's INTEGRAL_STACK_SIZE, 30000) int32
   p, q, r, s (1-based orbital numbers) and FP64 values, the last record ending
   with p = -1 (ReadTransformedIntegrals.f90:225-233 reads it).  *n_written =
   integrals written.  Returns 0, or -1 with the error set. */
int LowdinGB300_mp2_moint(LibintInterface *lint, const double *dD, const double *dC, const double *eps, int n_occ,
                          int n_frozen, const char *path, int stack_size, double x_budget_gb, double *e2,
                          long long *n_written, void *stream);
/* LowdinGB300_mp2_coupling in FP64 that also writes the inter-species
   (ia|jb), i, a of species a and j, b of species b, to `path`
   ("<species a>.<species b>moint.dat" in the reference; two-species DIRECT
   branch of TransformIntegralsC.f90:1170-1374 with the MP2 bounds of
   :1687-1697): every i, a, j, b in that loop order, |value| > 1e-10, same
   record layout as LowdinGB300_mp2_moint. */
int LowdinGB300_mp2_coupling_moint(LibintInterface *a, LibintInterface *b, const double *dCa, const double *dCb,
                                   const double *eps_a, const double *eps_b, int n_occ_a, int n_frozen_a,
                                   int n_occ_b, int n_frozen_b, double factor, const char *path, int stack_size,
                                   double x_budget_gb, double *e2, long long *n_written, void *stream);
/* The record writer alone (host only): `count` entries in the given order. */
int LowdinGB300_moint_write(const char *path, int stack_size, const int *p, const int *q, const int *r,
                            const int *s, const double *v, long long count);

/* Split-BF16 GEMM on the tensor cores (no counterpart in the reference; the
   engine of the mixed-precision MP2 transform): C (M x N) = A (M x K) B^T with
   B given as N x K, all row-major FP32 device arrays.  Each operand is split
   into `pieces` BF16 parts (2 or 3); C accumulates, in FP32, the products
   p0q0 + p0q1 + p1q0 (pieces 2, relative error ~2^-16 per product) or those
   plus p1q1 + p0q2 + p2q0 (pieces 3, ~2^-24).  Synchronises `stream`.
   Returns 0, or -1 with LowdinGB300_last_error() set. */
int LowdinGB300_gemm_bf16_split(const float *dA, const float *dB, float *dC, int M, int N, int K, int pieces,
                                void *stream);
/* Same product, three pieces per operand, eight products (adds p1q2 + p2q1)
   and no long FP32 running sums: every 16-wide K slab's main product is
   rounded once by the tensor cores, its mean rounding loss added back, and
   the partial results enter a compensated FP32 sum (hi + lo).  For
   contractions with strong cancellation and for squared results (every
   quarter of the MP2 transform at precision 2). */
int LowdinGB300_gemm_bf16_precise(const float *dA, const float *dB, float *dC, int M, int N, int K, void *stream);
/* Benchmark of the tensor-core GEMM engines (no counterpart in the reference):
   operands of M x K and N x K pseudo-random values split once, then `reps`
   launches timed with CUDA events on `stream`; mode 2 / 3: split engine with
   2 / 3 pieces, 8: precise engine.  Returns milliseconds per launch, or -1. */
double LowdinGB300_gemm_bench(int M, int N, int K, int mode, int reps, void *stream);

/* One-electron matrices of a species on the device (no counterpart in the
   reference's C ABI; computes what LibintInterface_compute_1body_ints kinds 1
   and 2 and LowdinGB300_potential return): dS overlap, dT kinetic, dV
   sum_C Z_C <a|1/|r-C||b> for the host point charges Z (ncharge) at R
   (3 ncharge, bohr); device n x n row-major outputs, any may be null.
   Queued on `stream`.  Returns 0, or -1 with the error set. */
int LowdinGB300_one_body_device(LibintInterface *lint, int ncharge, const double *Z, const double *R, double *dS,
                                double *dT, double *dV, void *stream);

/* Pulay DIIS coefficients of nsys systems on the device (caller side of the
   integral path; replaces the host solve of src/scf/Convergence.f90:543-633).
   dE: [nsys][h][h] error products <e_i, e_j> (device, FP64), 1 <= h <= 20;
   dfirst: per system the first history entry to use (device ints, entries
   before it get coefficient 0), or NULL for all; dcoef: [nsys][h]
   coefficients c minimising |sum_i c_i e_i| under sum_i c_i = 1
   (pseudo-inverse of the bordered Pulay matrix scaled to unit diagonal,
   eigenvalues below 1e-12 of the largest dropped).  Queued on `stream`;
   returns 0, or -1 with the error set. */
int LowdinGB300_diis_coefficients(const double *dE, int h, int nsys, const int *dfirst, double *dcoef,
                                  void *stream);

/* The device Boys functions F_0..F_L(T) (L <= 4) at the n host arguments T,
   into host out[n][L+1]: fp32 = 1 the arithmetic FP32 form of the FP32
   kernels, 0 the tabulated FP64 form (a check of the integral kernels'
   building block; no counterpart in the reference).  Returns 0 or -1. */
int LowdinGB300_boys_eval(int fp32, int L, const double *T, int n, double *out);

/* Number of CUDA kernels this library has launched in the process. */
long long LowdinGB300_launch_count(void);

/* Library and device description (static string). */
const char *LowdinGB300_version(void);

#ifdef __cplusplus
}
#endif
#undef LGB_REF
#endif /* LOWDIN_GB300_H */
