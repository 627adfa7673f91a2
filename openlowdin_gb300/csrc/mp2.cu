// MP2 on the device (LowdinGB300_mp2_direct / _mp2_coupling / _mp2_moint) and
// the entries of the split-BF16 tensor-core GEMM engines.
#include "lint_host.cuh"

// ========================================================= MP2 transform
// LowdinGB300_mp2_direct: closed-shell MP2 of one electron species with the
// four-index transform on the device.  Same integral set as the reference's
// DIRECT transform (TransformIntegralsC.f90:472-665 over
// LibintInterface_compute_2body_directIT, Libint2Iface.cpp:620-921):
// significant shell pairs only, quartets dropped by the density screening,
// raw |v| <= 1e-10 dropped; MO integrals with |(ia|jb)| <= 1e-10 read as zero
// in the energy (only larger ones are stored, :634).  The first quarter is not
// recomputed per occupied orbital: the integrals of every bra pair against a
// batch of ket pairs are written once into X[mu][col][nu] and contracted by
// GEMMs:
//   T1[i][col][nu] = sum_mu Co[mu][i] X[mu][col][nu]          (o x N^2 P)
//   Y[i][col][a]   = sum_nu T1[i][col][nu] Cv[nu][a]          (o v N P)
// then for every i: Z[lam][sig][a] (unpacked Y[i]),
//   W[j][sig][a]   = sum_lam Co[lam][j] Z[lam][sig][a]        (o^2 v N^2)
//   M[j][b][a]     = sum_sig Cv[sig][b] W[j][sig][a] = (ia|jb) (o^2 v^2 N)
// and the pair energies.  A column is one Cartesian component pair (c, d) of
// a significant ket shell pair (all nc^2 of a diagonal pair).
namespace {

std::mutex g_blas_mu;
std::vector<std::pair<int, cublasHandle_t>> g_blas;

bool blas_handle(cublasHandle_t *out) {
  int dev = 0;
  CK(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_blas_mu);
  for (auto &e : g_blas)
    if (e.first == dev) {
      *out = e.second;
      return true;
    }
  cublasHandle_t h = nullptr;
  if (cublasCreate(&h) != CUBLAS_STATUS_SUCCESS) {
    set_error("cublasCreate failed");
    return false;
  }
  g_blas.push_back({dev, h});
  *out = h;
  return true;
}

// row-major C_b = op(A_b) op(B_b), b < batch, with element strides between batches
bool dgemm_rm(cublasHandle_t h, bool ta, bool tb, int m, int n, int k, const double *A, int lda, long long sA,
              const double *B, int ldb, long long sB, double *C, int ldc, long long sC, int batch) {
  const double one = 1.0, zero = 0.0;
  const cublasStatus_t st =
      cublasDgemmStridedBatched(h, tb ? CUBLAS_OP_T : CUBLAS_OP_N, ta ? CUBLAS_OP_T : CUBLAS_OP_N, n, m, k, &one, B,
                                ldb, sB, A, lda, sA, &zero, C, ldc, sC, batch);
  if (st != CUBLAS_STATUS_SUCCESS) {
    set_error("cublasDgemmStridedBatched failed (status %d, m=%d n=%d k=%d batch=%d)", (int)st, m, n, k, batch);
    return false;
  }
  return true;
}

struct MP2Stats {
  long long ncols = 0;
  int batches = 0;
};
MP2Stats g_mp2_last;

// Columns of the significant ket pairs (colbase per pair record; colpair =
// lam | sig << 16 | offdiag << 31) and batches of whole ket pairs with at most
// colB columns (bfirst: first pair of each batch, then npairs).
struct MP2Columns {
  std::vector<int> colbase;
  std::vector<unsigned> colpair;
  std::vector<int> bfirst;
  long long ncols = 0;
};

void mp2_columns(const PairList &P, long long colB, MP2Columns &mc) {
  const int npairs = (int)P.h.size();
  mc.colbase.assign(npairs, 0);
  mc.colpair.clear();
  for (int k = 0; k < npairs; ++k) {
    const PairRec &r = P.h[k];
    mc.colbase[k] = (int)mc.colpair.size();
    const int nc = ncart(r.la), nd = ncart(r.lb);
    for (int c = 0; c < nc; ++c)
      for (int d = 0; d < nd; ++d)
        mc.colpair.push_back((unsigned)(r.fa + c) | (unsigned)(r.fb + d) << 16 | (r.sa != r.sb ? 1u << 31 : 0u));
  }
  mc.ncols = (long long)mc.colpair.size();
  mc.bfirst.clear();
  for (int k = 0; k < npairs;) {
    mc.bfirst.push_back(k);
    const int c0 = mc.colbase[k];
    while (k < npairs && mc.colbase[k] - c0 + ncart(P.h[k].la) * ncart(P.h[k].lb) <= colB) ++k;
  }
  mc.bfirst.push_back(npairs);
}

// integrals of every bra pair of PA against the ket pairs [k0, k1) of PB
bool mp2_batch_ints(const PairList &PA, const PairList &PB, MXParams q, int k0, int k1, cudaStream_t s) {
  for (int ck = 0; ck < kNumPairClasses; ++ck) {
    const int ka = std::max(k0, PB.start[ck]), kb = std::min(k1, PB.start[ck + 1]);
    if (ka >= kb) continue;
    for (int cb = 0; cb < kNumPairClasses; ++cb)
      for (int b0 = PA.start[cb]; b0 < PA.start[cb + 1]; b0 += 65535 * kWarpsPerBlock) {  // grid y limit
        q.bra0 = b0;
        q.nbra = std::min(PA.start[cb + 1] - b0, 65535 * kWarpsPerBlock);
        q.ket0 = ka;
        q.nket = kb - ka;
        CK(launch_mp2x(cb, ck, q, s));
      }
  }
  return true;
}

// Writer of the reference's transformed-integral file `<species>moint.dat`
// (TransformIntegralsC.f90:531-654, read by ReadTransformedIntegrals.f90:225-233):
// a Fortran sequential unformatted file whose records each hold four int32
// index arrays p, q, r, s and one FP64 value array, all of the stack size
// (30000 by default), framed by the record length in bytes (int32) before and
// after, as gfortran writes them.  Entries fill a stack in the order they
// come; a full stack is written as one record and cleared; the last record
// marks the end with p = -1 after its last entry (zeros beyond).
struct MointWriter {
  FILE *f = nullptr;
  int stack = 0, m = 0;
  long long written = 0;
  std::vector<int32_t> pp, qq, rr, ss;
  std::vector<double> val;
  bool open(const char *path, int stack_size) {
    stack = stack_size;
    pp.assign(stack, 0); qq.assign(stack, 0); rr.assign(stack, 0); ss.assign(stack, 0);
    val.assign(stack, 0.0);
    f = std::fopen(path, "wb");
    if (!f) {
      set_error("moint: cannot open %s for writing", path);
      return false;
    }
    return true;
  }
  bool record() {
    const int32_t len = (int32_t)((size_t)stack * (4 * sizeof(int32_t) + sizeof(double)));
    bool ok = std::fwrite(&len, 4, 1, f) == 1;
    for (auto *a : {&pp, &qq, &rr, &ss}) ok = ok && std::fwrite(a->data(), 4, stack, f) == (size_t)stack;
    ok = ok && std::fwrite(val.data(), 8, stack, f) == (size_t)stack && std::fwrite(&len, 4, 1, f) == 1;
    if (!ok) set_error("moint: write failed");
    for (auto *a : {&pp, &qq, &rr, &ss}) std::fill(a->begin(), a->end(), 0);
    std::fill(val.begin(), val.end(), 0.0);
    return ok;
  }
  bool put(int p, int q, int r, int s_, double v) {
    pp[m] = p; qq[m] = q; rr[m] = r; ss[m] = s_; val[m] = v;
    ++written;
    if (++m == stack) {
      m = 0;
      return record();
    }
    return true;
  }
  bool finish() {
    pp[m] = -1;
    const bool ok = record();
    std::fclose(f);
    f = nullptr;
    return ok;
  }
  ~MointWriter() {
    if (f) std::fclose(f);
  }
};

// One MP2 term: intra-species (A == B, closed shell: (ia|jb)[2(ia|jb) -
// (ib|ja)]/D) or inter-species (A != B: factor (ia|jb)^2 / D, factor = (q_A
// q_B)^2 lambda_A lambda_B).  The bra index pairs (mu nu) belong to A, the ket
// columns (lam sig) to B.
struct MP2Setup {
  LibintInterface *A, *B;
  const PairList *PA, *PB;
  bool coupling;
  double factor;
  int nA, nB, oA, vA, oB, vB, noccA, nfA, noccB, nfB;
  const double *dCA, *dCB, *epsA, *epsB;
  MXParams q;      // common integral parameters
  MointWriter *moint = nullptr;   // FP64 intra-species path: also write every (ia|jb) to the file
};

// (ia|jb) of occupied i (M[j][b][a], device) into the file in the reference's
// loop order: a, then j, then b, |v| > 1e-10.  One species
// (TransformIntegralsC.f90:570-640 with the MP2 bounds of :1489-1501): j >= i,
// b >= a when j == i.  Two species (:1255-1350 with the bounds of :1687-1697):
// every j and b of the other species.
bool moint_block(const MP2Setup &S, int i, const double *dM, std::vector<double> &h, cudaStream_t s) {
  const int oB = S.oB, vB = S.vB, vA = S.vA;
  h.resize((size_t)oB * vB * vA);
  CK(cudaMemcpyAsync(h.data(), dM, h.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  const int p = S.nfA + i + 1;
  const bool sym = !S.coupling;
  for (int a = 0; a < vA; ++a)
    for (int j = sym ? i : 0; j < oB; ++j)
      for (int b = (sym && j == i ? a : 0); b < vB; ++b) {
        const double v = h[((size_t)j * vB + b) * vA + a];
        if (std::fabs(v) > 1e-10 && !S.moint->put(p, S.noccA + a + 1, S.nfB + j + 1, S.noccB + b + 1, v))
          return false;
      }
  return true;
}

bool mp2_need(size_t bytes) {
  size_t freeb = 0, totb = 0;
  CK(cudaMemGetInfo(&freeb, &totb));
  if (bytes > freeb) {
    set_error("mp2: needs %.1f GB of device memory, %.1f GB free", bytes / 1e9, freeb / 1e9);
    return false;
  }
  return true;
}

long long mp2_max_batch(const MP2Columns &mc, const PairList &P) {
  long long colB = 0;
  for (size_t b = 0; b + 1 < mc.bfirst.size(); ++b) {
    const int k1 = mc.bfirst[b + 1];
    colB = std::max<long long>(colB, (k1 < (int)P.h.size() ? mc.colbase[k1] : mc.ncols) - mc.colbase[mc.bfirst[b]]);
  }
  return colB;
}

// FP64 back end: cuBLAS DGEMM for the four quarters
bool mp2_fp64(MP2Setup &S, size_t budget, double *e2out, cudaStream_t s) {
  const int nA = S.nA, nB = S.nB, oA = S.oA, vA = S.vA, oB = S.oB, vB = S.vB;
  cublasHandle_t blas;
  if (!blas_handle(&blas)) return false;
  if (cublasSetStream(blas, s) != CUBLAS_STATUS_SUCCESS) {
    set_error("cublasSetStream failed");
    return false;
  }
  const PairList &PB = *S.PB;
  const size_t per_col = (size_t)nA * nA * sizeof(double) + (size_t)oA * nA * sizeof(double);
  MP2Columns mc;
  mp2_columns(PB, std::max<long long>(36, (long long)(budget / per_col)), mc);
  const long long ncols = mc.ncols;
  const long long colB = mp2_max_batch(mc, PB);
  if (!mp2_need((size_t)oA * ncols * vA * 8 + (size_t)nB * nB * vA * 8 + (size_t)colB * per_col +
                (size_t)oB * nB * vA * 8 + (size_t)oB * vB * vA * 8))
    return false;
  DevBuf<double> CoA, CvA, CoB, CvB, EoB, EvA, EvB, Y, X, T1, Z, W, M, e2;
  DevBuf<int> dcolbase;
  DevBuf<unsigned> dcolpair;
  if (!CoA.ensure((size_t)nA * oA) || !CvA.ensure((size_t)nA * vA) || !CoB.ensure((size_t)nB * oB) ||
      !CvB.ensure((size_t)nB * vB) || !EoB.ensure(oB) || !EvA.ensure(vA) || !EvB.ensure(vB) ||
      !Y.ensure((size_t)oA * ncols * vA) || !X.ensure((size_t)nA * colB * nA) || !T1.ensure((size_t)oA * colB * nA) ||
      !Z.ensure((size_t)nB * nB * vA) || !W.ensure((size_t)oB * nB * vA) || !M.ensure((size_t)oB * vB * vA) ||
      !e2.ensure(1) || !dcolbase.ensure(PB.h.size()) || !dcolpair.ensure(ncols))
    return false;
  CK(cudaMemcpyAsync(dcolbase.p, mc.colbase.data(), PB.h.size() * sizeof(int), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(dcolpair.p, mc.colpair.data(), ncols * sizeof(unsigned), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(EoB.p, S.epsB + S.nfB, oB * sizeof(double), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(EvA.p, S.epsA + S.noccA, vA * sizeof(double), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(EvB.p, S.epsB + S.noccB, vB * sizeof(double), cudaMemcpyHostToDevice, s));
  CK(cudaMemsetAsync(e2.p, 0, sizeof(double), s));
  CK(launch_mp2_coeffs(S.dCA, S.A->d_norma, nA, S.nfA, S.noccA, CoA.p, CvA.p, nullptr, nullptr, s));
  CK(launch_mp2_coeffs(S.dCB, S.B->d_norma, nB, S.nfB, S.noccB, CoB.p, CvB.p, nullptr, nullptr, s));
  MXParams q = S.q;
  q.colbase = dcolbase.p;
  q.X = X.p;
  std::vector<double> hM;
  const int nbatch = (int)mc.bfirst.size() - 1;
  for (int bt = 0; bt < nbatch; ++bt) {
    const int k0 = mc.bfirst[bt], k1 = mc.bfirst[bt + 1];
    const int c0 = mc.colbase[k0];
    const int nb = (int)((k1 < (int)PB.h.size() ? mc.colbase[k1] : ncols) - c0);
    q.col_first = c0;
    q.ncol = nb;
    CK(cudaMemsetAsync(X.p, 0, (size_t)nA * nb * nA * sizeof(double), s));
    if (!mp2_batch_ints(*S.PA, PB, q, k0, k1, s)) return false;
    // T1 (oA x nb*nA) = CoA^T X ; Y[i][c0 + col][a] = T1[i] (nb x nA) CvA
    if (!dgemm_rm(blas, true, false, oA, nb * nA, nA, CoA.p, oA, 0, X.p, nb * nA, 0, T1.p, nb * nA, 0, 1))
      return false;
    if (!dgemm_rm(blas, false, false, nb, vA, nA, T1.p, nA, (long long)nb * nA, CvA.p, vA, 0, Y.p + (size_t)c0 * vA,
                  vA, ncols * vA, oA))
      return false;
  }
  CK(cudaMemsetAsync(Z.p, 0, (size_t)nB * nB * vA * sizeof(double), s));
  for (int i = 0; i < oA; ++i) {
    CK(launch_mp2_unpack<double>(Y.p + (size_t)i * ncols * vA, dcolpair.p, ncols, nB, vA, Z.p, s));
    // W (oB x nB*vA) = CoB^T Z ; M_j (vB x vA) = CvB^T W_j
    if (!dgemm_rm(blas, true, false, oB, nB * vA, nB, CoB.p, oB, 0, Z.p, nB * vA, 0, W.p, nB * vA, 0, 1))
      return false;
    if (!dgemm_rm(blas, true, false, vB, vA, nB, CvB.p, vB, 0, W.p, vA, (long long)nB * vA, M.p, vA,
                  (long long)vB * vA, oB))
      return false;
    const double ei = S.epsA[S.nfA + i];
    if (S.coupling)
      CK(launch_mp2_energy_coupling<double>(M.p, oB, vB, vA, ei, EoB.p, EvA.p, EvB.p, 1e-10, S.factor, e2.p, s));
    else
      CK(launch_mp2_energy<double>(M.p, oB, vB, ei, EoB.p, EvB.p, 1e-10, e2.p, s));
    if (S.moint && !moint_block(S, i, M.p, hM, s)) return false;
  }
  double e = 0;
  CK(cudaMemcpyAsync(&e, e2.p, sizeof(double), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  *e2out = e;
  g_mp2_last.ncols = ncols;
  g_mp2_last.batches = nbatch;
  return true;  // the buffers are freed on return
}

// Split-BF16 back end: the same quarters on the tensor cores (np BF16 pieces
// per operand, FP32 accumulation), operands written K-major by their producers:
//   Xt[col][nu][mu]   (integral kernel)          GEMM1: T1[i][col nu] = CoT_A Xt^T
//   Y'[a][i][col]     (GEMM2 = CvT_A T1^T, FP32) per i: Zt[a][sig][lam] (gather)
//   GEMM3: Wt[j][a sig] = CoT_B Zt^T             GEMM4: M_j[b][a] = CvT_B Wt_j^T
struct SplitBuf {
  DevBuf<__nv_bfloat16> p[kMaxPieces];
  bool ensure(int np, size_t n) {
    for (int q = 0; q < np; ++q)
      if (!p[q].ensure(n)) return false;
    return true;
  }
  Bf16Split in() const { return Bf16Split{{p[0].p, p[1].p, p[2].p}}; }
  void out(GemmOut &o) const {
    for (int q = 0; q < kMaxPieces; ++q) o.Cp[q] = p[q].p;
  }
  __nv_bfloat16 *const *ptrs(__nv_bfloat16 *(&tmp)[kMaxPieces]) const {
    for (int q = 0; q < kMaxPieces; ++q) tmp[q] = p[q].p;
    return tmp;
  }
};

bool mp2_split(MP2Setup &S, int np, size_t budget, double *e2out, cudaStream_t s) {
  using bf = __nv_bfloat16;
  const int nA = S.nA, nB = S.nB, oA = S.oA, vA = S.vA, oB = S.oB, vB = S.vB;
  const int KA = (nA + 63) / 64 * 64, KB = (nB + 63) / 64 * 64;
  const PairList &PB = *S.PB;
  const size_t per_col = (size_t)KA * KA * 2 * np + (size_t)oA * KA * 2 * np;   // Xt and T1 pieces
  MP2Columns mc;
  mp2_columns(PB, std::max<long long>(36, (long long)(budget / per_col)), mc);
  const long long ncols = mc.ncols;
  const long long colB = mp2_max_batch(mc, PB);
  // gather lists over B's functions: row sig -> (lam, col) with Z[lam][sig] = Y[col]
  std::vector<int> rowptr(nB + 1, 0);
  for (long long c = 0; c < ncols; ++c) {
    const unsigned cp = mc.colpair[c];
    rowptr[((cp >> 16) & 0x7fff) + 1]++;
    if (cp >> 31) rowptr[(cp & 0xffff) + 1]++;
  }
  for (int r = 0; r < nB; ++r) rowptr[r + 1] += rowptr[r];
  std::vector<int2> ent(rowptr[nB]);
  {
    std::vector<int> fill(rowptr.begin(), rowptr.end() - 1);
    for (long long c = 0; c < ncols; ++c) {
      const unsigned cp = mc.colpair[c];
      const int lam = cp & 0xffff, sig = (cp >> 16) & 0x7fff;
      ent[fill[sig]++] = make_int2(lam | sig << 16, (int)c);
      if (cp >> 31) ent[fill[lam]++] = make_int2(sig | lam << 16, (int)c);
    }
  }
  const size_t need = (size_t)vA * oA * ncols * 4 + (size_t)colB * per_col +
                      ((size_t)vA * KB * KB + (size_t)oB * vA * KB + (size_t)(oA + vA) * KA + (size_t)(oB + vB) * KB) *
                          2 * np +
                      (size_t)oB * vB * vA * 4 + ent.size() * 8;
  if (!mp2_need(need)) return false;
  SplitBuf CoTA, CvTA, CoTB, CvTB, X, T1, Z, W;
  DevBuf<float> Y, M;
  DevBuf<double> EoB, EvA, EvB, e2;
  DevBuf<int> dcolbase, drowptr, err;
  DevBuf<int2> dent;
  const size_t xsz = (size_t)colB * KA * KA, t1sz = (size_t)oA * colB * KA, zsz = (size_t)vA * KB * KB,
               wsz = (size_t)oB * vA * KB;
  if (!CoTA.ensure(np, (size_t)oA * KA) || !CvTA.ensure(np, (size_t)vA * KA) || !CoTB.ensure(np, (size_t)oB * KB) ||
      !CvTB.ensure(np, (size_t)vB * KB) || !X.ensure(np, xsz) || !T1.ensure(np, t1sz) || !Z.ensure(np, zsz) ||
      !W.ensure(np, wsz) || !Y.ensure((size_t)vA * oA * ncols) || !M.ensure((size_t)oB * vB * vA) ||
      !EoB.ensure(oB) || !EvA.ensure(vA) || !EvB.ensure(vB) || !e2.ensure(1) || !dcolbase.ensure(PB.h.size()) ||
      !drowptr.ensure(nB + 1) || !err.ensure(1) || !dent.ensure(std::max<size_t>(1, ent.size())))
    return false;
  CK(cudaMemcpyAsync(dcolbase.p, mc.colbase.data(), PB.h.size() * sizeof(int), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(drowptr.p, rowptr.data(), (nB + 1) * sizeof(int), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(dent.p, ent.data(), ent.size() * sizeof(int2), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(EoB.p, S.epsB + S.nfB, oB * sizeof(double), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(EvA.p, S.epsA + S.noccA, vA * sizeof(double), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(EvB.p, S.epsB + S.noccB, vB * sizeof(double), cudaMemcpyHostToDevice, s));
  CK(cudaMemsetAsync(e2.p, 0, sizeof(double), s));
  CK(cudaMemsetAsync(err.p, 0, sizeof(int), s));
  for (const SplitBuf *b : {&CoTA, &CvTA, &CoTB, &CvTB, &Z})
    for (int k = 0; k < np; ++k) CK(cudaMemsetAsync(b->p[k].p, 0, b->p[k].n * sizeof(bf), s));
  bf *t0[kMaxPieces], *t1[kMaxPieces];
  CK(launch_mp2_coeffs_bf16(S.dCA, S.A->d_norma, nA, S.nfA, S.noccA, KA, np, CoTA.ptrs(t0), CvTA.ptrs(t1), s));
  CK(launch_mp2_coeffs_bf16(S.dCB, S.B->d_norma, nB, S.nfB, S.noccB, KB, np, CoTB.ptrs(t0), CvTB.ptrs(t1), s));
  // np 3: every quarter on the precise engine (the tensor cores round their
  // FP32 running sums toward zero; over a long contraction that bias, not
  // the BF16 pieces, dominated the energy error); np 2: the split engine
  auto gemm = [&](const Bf16Split &Am, long long ar, const Bf16Split &Bm, long long br, int Kp, int Mr, int Nc,
                  int batch, int abr, int bbr, const GemmOut &out) {
    return np == 3 ? launch_gemm_precise(Am, ar, Bm, br, Kp, Mr, Nc, batch, abr, bbr, out, err.p, s)
                   : launch_gemm_split(Am, ar, Bm, br, Kp, Mr, Nc, batch, abr, bbr, np, out, err.p, s);
  };
  MXParams q = S.q;
  q.colbase = dcolbase.p;
  q.X = nullptr;
  for (int k = 0; k < kMaxPieces; ++k) q.Xp[k] = X.p[k].p;
  q.np = np;
  q.Kp = KA;
  const int nbatch = (int)mc.bfirst.size() - 1;
  for (int bt = 0; bt < nbatch; ++bt) {
    const int k0 = mc.bfirst[bt], k1 = mc.bfirst[bt + 1];
    const int c0 = mc.colbase[k0];
    const int nb = (int)((k1 < (int)PB.h.size() ? mc.colbase[k1] : ncols) - c0);
    q.col_first = c0;
    q.ncol = nb;
    for (int k = 0; k < np; ++k) CK(cudaMemsetAsync(X.p[k].p, 0, (size_t)nb * KA * KA * sizeof(bf), s));
    if (!mp2_batch_ints(*S.PA, PB, q, k0, k1, s)) return false;
    GemmOut o1{};
    T1.out(o1);
    o1.ldc = (long long)nb * KA;
    CK(gemm(CoTA.in(), oA, X.in(), (long long)nb * KA, KA, oA, nb * KA, 1, 0, 0, o1));
    GemmOut o2{};
    o2.C = Y.p;
    o2.ldc = (long long)oA * ncols;
    o2.grp_cols = nb;
    o2.gcol_stride = ncols;
    o2.col0 = c0;
    CK(gemm(CvTA.in(), vA, T1.in(), (long long)oA * nb, KA, vA, oA * nb, 1, 0, 0, o2));
  }
  bf *tz[kMaxPieces];
  for (int i = 0; i < oA; ++i) {
    CK(launch_mp2_unpack_csr(Y.p + (size_t)i * ncols, (long long)oA * ncols, drowptr.p, dent.p, nB, KB, vA, np,
                             Z.ptrs(tz), s));
    GemmOut o3{};
    W.out(o3);
    o3.ldc = (long long)vA * KB;
    CK(gemm(CoTB.in(), oB, Z.in(), (long long)vA * KB, KB, oB, vA * KB, 1, 0, 0, o3));
    GemmOut o4{};
    o4.C = M.p;
    o4.ldc = vA;
    o4.c_batch = (long long)vB * vA;
    CK(gemm(CvTB.in(), vB, W.in(), (long long)oB * vA, KB, vB, vA, oB, 0, vA, o4));
    const double ei = S.epsA[S.nfA + i];
    if (S.coupling)
      CK(launch_mp2_energy_coupling<float>(M.p, oB, vB, vA, ei, EoB.p, EvA.p, EvB.p, 1e-10, S.factor, e2.p, s));
    else
      CK(launch_mp2_energy<float>(M.p, oB, vB, ei, EoB.p, EvB.p, 1e-10, e2.p, s));
  }
  double e = 0;
  int herr = 0;
  CK(cudaMemcpyAsync(&e, e2.p, sizeof(double), cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (herr) {
    set_error("mp2: a tensor-core GEMM pipeline wait ran out (code %d)", herr);
    return false;
  }
  *e2out = e;
  g_mp2_last.ncols = ncols;
  g_mp2_last.batches = nbatch;
  return true;
}

bool mp2_run(MP2Setup &S, int precision, size_t budget, double *e2out, cudaStream_t s) {
  if (precision < 0 || precision > 2) {
    set_error("mp2: precision %d is not available (0: FP64, 1 / 2: split BF16 in 2 / 3 pieces)", precision);
    return false;
  }
  if (S.nA >= 32768 || S.nB >= 32768) {
    set_error("mp2: more than 32767 basis functions exceed the column encoding");
    return false;
  }
  return precision == 0 ? mp2_fp64(S, budget, e2out, s) : mp2_split(S, precision + 1, budget, e2out, s);
}

bool mp2_direct(LibintInterface *L, const double *dD, const double *dC, const double *eps, int n_occ, int n_frozen,
                int precision, size_t x_budget_bytes, double *e2out, cudaStream_t s, MointWriter *moint = nullptr) {
  if (!L->is_electron) {
    set_error("mp2_direct: closed-shell MP2 is defined here for an electron species");
    return false;
  }
  if (!L->ensure_sig()) return false;
  const int n = L->nbasis, nsh = L->nshell();
  if (!(0 <= n_frozen && n_frozen < n_occ && n_occ < n)) {
    set_error("mp2_direct: need 0 <= n_frozen < n_occ < nbasis (got %d, %d, %d)", n_frozen, n_occ, n);
    return false;
  }
  MP2Setup S{};
  S.A = S.B = L;
  S.PA = S.PB = &L->sig;
  S.coupling = false;
  S.factor = 1.0;
  S.nA = S.nB = n;
  S.noccA = S.noccB = n_occ;
  S.nfA = S.nfB = n_frozen;
  S.oA = S.oB = n_occ - n_frozen;
  S.vA = S.vB = n - n_occ;
  S.dCA = S.dCB = dC;
  S.epsA = S.epsB = eps;
  // shell-block norms of D for the screening
  if (!L->dDs.ensure((size_t)n * n) || !L->dDn.ensure((size_t)nsh * nsh)) return false;
  CK(launch_prepare_density(dD, L->d_norma, L->d_shell_of, n, nsh, L->dDs.p, nullptr, L->dDn.p, nullptr, s));
  MXParams &q = S.q;
  q.pairs = q.kpairs = L->sig.d;
  q.prims = q.kprims = L->sig.dp;
  q.Dn = L->dDn.p;
  q.nsh = nsh;
  q.screen = 1;
  q.eps = DBL_EPSILON;
  q.cut = 1e-10;
  q.n = n;
  q.boys = L->boys;
  S.moint = moint;
  return mp2_run(S, precision, x_budget_bytes, e2out, s);
}

bool mp2_coupling(LibintInterface *A, LibintInterface *B, const double *dCA, const double *dCB, const double *epsA,
                  const double *epsB, int noccA, int nfA, int noccB, int nfB, double factor, int precision,
                  size_t budget, double *e2out, cudaStream_t s, MointWriter *moint = nullptr) {
  if (A == B) {
    set_error("mp2_coupling: the two handles must be different species");
    return false;
  }
  if (!A->ensure_all() || !B->ensure_all()) return false;
  const int nA = A->nbasis, nB = B->nbasis;
  if (!(0 <= nfA && nfA < noccA && noccA < nA && 0 <= nfB && nfB < noccB && noccB < nB)) {
    set_error("mp2_coupling: need 0 <= n_frozen < n_occ < nbasis for both species");
    return false;
  }
  MP2Setup S{};
  S.A = A;
  S.B = B;
  S.PA = &A->all;
  S.PB = &B->all;
  S.coupling = true;
  S.factor = factor;
  S.nA = nA;
  S.nB = nB;
  S.noccA = noccA;
  S.nfA = nfA;
  S.noccB = noccB;
  S.nfB = nfB;
  S.oA = noccA - nfA;
  S.vA = nA - noccA;
  S.oB = noccB - nfB;
  S.vB = nB - noccB;
  S.dCA = dCA;
  S.dCB = dCB;
  S.epsA = epsA;
  S.epsB = epsB;
  // coupling integrals: no density screening (Libint2Iface.cpp:1296-1622),
  // quartets whose Schwarz bound is below the raw cut contribute nothing
  MXParams &q = S.q;
  q.pairs = A->all.d;
  q.prims = A->all.dp;
  q.kpairs = B->all.d;
  q.kprims = B->all.dp;
  q.screen = 0;
  q.eps = 0.0;
  q.cut = 1e-10;
  q.n = nA;
  q.boys = A->boys;
  S.moint = moint;
  return mp2_run(S, precision, budget, e2out, s);
}

}  // namespace

extern "C" {

int LowdinGB300_mp2_direct(LibintInterface *lint, const double *dD, const double *dC, const double *eps, int n_occ,
                           int n_frozen, int precision, double x_budget_gb, double *e2, void *stream) {
  if (!check_handle(lint, __func__)) return -1;
  if (!dD || !dC || !eps || !e2) {
    set_error("%s: null argument", __func__);
    return -1;
  }
  const size_t budget = x_budget_gb > 0 ? (size_t)(x_budget_gb * 1e9) : (size_t)8e9;
  return mp2_direct(lint, dD, dC, eps, n_occ, n_frozen, precision, budget, e2, (cudaStream_t)stream) ? 0 : -1;
}

int LowdinGB300_mp2_coupling(LibintInterface *a, LibintInterface *b, const double *dCa, const double *dCb,
                             const double *eps_a, const double *eps_b, int n_occ_a, int n_frozen_a, int n_occ_b,
                             int n_frozen_b, double factor, int precision, double x_budget_gb, double *e2,
                             void *stream) {
  if (!check_handle(a, __func__) || !check_handle(b, __func__)) return -1;
  if (!dCa || !dCb || !eps_a || !eps_b || !e2) {
    set_error("%s: null argument", __func__);
    return -1;
  }
  const size_t budget = x_budget_gb > 0 ? (size_t)(x_budget_gb * 1e9) : (size_t)8e9;
  return mp2_coupling(a, b, dCa, dCb, eps_a, eps_b, n_occ_a, n_frozen_a, n_occ_b, n_frozen_b, factor, precision,
                      budget, e2, (cudaStream_t)stream)
             ? 0
             : -1;
}

long long LowdinGB300_mp2_last_columns(void) { return g_mp2_last.ncols; }

int LowdinGB300_mp2_moint(LibintInterface *lint, const double *dD, const double *dC, const double *eps, int n_occ,
                          int n_frozen, const char *path, int stack_size, double x_budget_gb, double *e2,
                          long long *n_written, void *stream) {
  if (!check_handle(lint, __func__)) return -1;
  if (!dD || !dC || !eps || !e2 || !path || stack_size < 1) {
    set_error("%s: invalid argument", __func__);
    return -1;
  }
  MointWriter w;
  if (!w.open(path, stack_size)) return -1;
  const size_t budget = x_budget_gb > 0 ? (size_t)(x_budget_gb * 1e9) : (size_t)8e9;
  if (!mp2_direct(lint, dD, dC, eps, n_occ, n_frozen, 0, budget, e2, (cudaStream_t)stream, &w)) return -1;
  if (!w.finish()) return -1;
  if (n_written) *n_written = w.written;
  return 0;
}

int LowdinGB300_mp2_coupling_moint(LibintInterface *a, LibintInterface *b, const double *dCa, const double *dCb,
                                   const double *eps_a, const double *eps_b, int n_occ_a, int n_frozen_a,
                                   int n_occ_b, int n_frozen_b, double factor, const char *path, int stack_size,
                                   double x_budget_gb, double *e2, long long *n_written, void *stream) {
  if (!check_handle(a, __func__) || !check_handle(b, __func__)) return -1;
  if (!dCa || !dCb || !eps_a || !eps_b || !e2 || !path || stack_size < 1) {
    set_error("%s: invalid argument", __func__);
    return -1;
  }
  MointWriter w;
  if (!w.open(path, stack_size)) return -1;
  const size_t budget = x_budget_gb > 0 ? (size_t)(x_budget_gb * 1e9) : (size_t)8e9;
  if (!mp2_coupling(a, b, dCa, dCb, eps_a, eps_b, n_occ_a, n_frozen_a, n_occ_b, n_frozen_b, factor, 0, budget, e2,
                    (cudaStream_t)stream, &w))
    return -1;
  if (!w.finish()) return -1;
  if (n_written) *n_written = w.written;
  return 0;
}

int LowdinGB300_moint_write(const char *path, int stack_size, const int *p, const int *q, const int *r,
                            const int *s, const double *v, long long count) {
  if (!path || stack_size < 1 || count < 0 || (count > 0 && (!p || !q || !r || !s || !v))) {
    set_error("%s: invalid argument", __func__);
    return -1;
  }
  MointWriter w;
  if (!w.open(path, stack_size)) return -1;
  for (long long k = 0; k < count; ++k)
    if (!w.put(p[k], q[k], r[k], s[k], v[k])) return -1;
  return w.finish() ? 0 : -1;
}

}  // extern "C"

// ============================================== split-BF16 tensor-core GEMM
namespace {
int gemm_entry(const char *fn, const float *dA, const float *dB, float *dC, int M, int N, int K, int pieces,
               bool precise, void *stream) {
  if (!dA || !dB || !dC || M <= 0 || N <= 0 || K <= 0 || pieces < 2 || pieces > kMaxPieces) {
    set_error("%s: invalid arguments", fn);
    return -1;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const int Kp = (K + 63) / 64 * 64;
  SplitBuf A, B;
  DevBuf<int> err;
  if (!A.ensure(pieces, (size_t)M * Kp) || !B.ensure(pieces, (size_t)N * Kp) || !err.ensure(1)) return -1;
  auto fail = [&](const char *what, cudaError_t e) {
    set_error("%s: %s (%s)", fn, what, cudaGetErrorString(e));
    return -1;
  };
  cudaError_t e;
  for (int q = 0; q < pieces; ++q)
    if ((e = cudaMemsetAsync(A.p[q].p, 0, (size_t)M * Kp * 2, s)) != cudaSuccess ||
        (e = cudaMemsetAsync(B.p[q].p, 0, (size_t)N * Kp * 2, s)) != cudaSuccess)
      return fail("clear", e);
  if ((e = cudaMemsetAsync(err.p, 0, sizeof(int), s)) != cudaSuccess) return fail("clear", e);
  __nv_bfloat16 *ta[kMaxPieces], *tb[kMaxPieces];
  if ((e = launch_split_bf16<float>(dA, M, K, K, pieces, A.ptrs(ta), Kp, s)) != cudaSuccess ||
      (e = launch_split_bf16<float>(dB, N, K, K, pieces, B.ptrs(tb), Kp, s)) != cudaSuccess)
    return fail("split", e);
  GemmOut out{};
  out.C = dC;
  out.ldc = N;
  e = precise ? launch_gemm_precise(A.in(), M, B.in(), N, Kp, M, N, 1, 0, 0, out, err.p, s)
              : launch_gemm_split(A.in(), M, B.in(), N, Kp, M, N, 1, 0, 0, pieces, out, err.p, s);
  if (e != cudaSuccess) return fail("gemm launch", e);
  int herr = 0;
  if ((e = cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
      (e = cudaStreamSynchronize(s)) != cudaSuccess)
    return fail("gemm", e);
  if (herr) {
    set_error("%s: a pipeline wait ran out (code %d)", fn, herr);
    return -1;
  }
  return 0;
}
}  // namespace

extern "C" {


int LowdinGB300_gemm_bf16_split(const float *dA, const float *dB, float *dC, int M, int N, int K, int pieces,
                                void *stream) {
  return gemm_entry(__func__, dA, dB, dC, M, N, K, pieces, false, stream);
}

int LowdinGB300_gemm_bf16_precise(const float *dA, const float *dB, float *dC, int M, int N, int K, void *stream) {
  return gemm_entry(__func__, dA, dB, dC, M, N, K, 3, true, stream);
}

double LowdinGB300_gemm_bench(int M, int N, int K, int mode, int reps, void *stream) {
  const int pieces = mode == 2 ? 2 : 3;
  if (M <= 0 || N <= 0 || K <= 0 || reps <= 0 || (mode != 2 && mode != 3 && mode != 8)) {
    set_error("%s: invalid arguments (mode 2, 3 or 8)", __func__);
    return -1.0;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const int Kp = (K + 63) / 64 * 64;
  SplitBuf A, B;
  DevBuf<float> src, C;
  DevBuf<int> err;
  if (!A.ensure(pieces, (size_t)M * Kp) || !B.ensure(pieces, (size_t)N * Kp) ||
      !src.ensure((size_t)std::max(M, N) * K) || !C.ensure((size_t)M * N) || !err.ensure(1))
    return -1.0;
  __nv_bfloat16 *ta[kMaxPieces], *tb[kMaxPieces];
  cudaEvent_t e0, e1;
  bool ok = cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess;
  for (int q = 0; ok && q < pieces; ++q)
    ok = cudaMemsetAsync(A.p[q].p, 0, (size_t)M * Kp * 2, s) == cudaSuccess &&
         cudaMemsetAsync(B.p[q].p, 0, (size_t)N * Kp * 2, s) == cudaSuccess;
  ok = ok && cudaMemsetAsync(err.p, 0, sizeof(int), s) == cudaSuccess &&
       launch_fill_hash(src.p, (long long)M * K, 1u, s) == cudaSuccess &&
       launch_split_bf16<float>(src.p, M, K, K, pieces, A.ptrs(ta), Kp, s) == cudaSuccess &&
       launch_fill_hash(src.p, (long long)N * K, 2u, s) == cudaSuccess &&
       launch_split_bf16<float>(src.p, N, K, K, pieces, B.ptrs(tb), Kp, s) == cudaSuccess;
  GemmOut out{};
  out.C = C.p;
  out.ldc = N;
  auto run = [&]() {
    return mode == 8 ? launch_gemm_precise(A.in(), M, B.in(), N, Kp, M, N, 1, 0, 0, out, err.p, s)
                     : launch_gemm_split(A.in(), M, B.in(), N, Kp, M, N, 1, 0, 0, pieces, out, err.p, s);
  };
  ok = ok && run() == cudaSuccess && cudaEventRecord(e0, s) == cudaSuccess;
  for (int r = 0; ok && r < reps; ++r) ok = run() == cudaSuccess;
  float ms = 0.f;
  int herr = 0;
  ok = ok && cudaEventRecord(e1, s) == cudaSuccess && cudaEventSynchronize(e1) == cudaSuccess &&
       cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess &&
       cudaMemcpy(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (!ok || herr) {
    set_error("%s: failed (%s, pipeline code %d)", __func__, cudaGetErrorString(cudaGetLastError()), herr);
    return -1.0;
  }
  return (double)ms / reps;
}

}  // extern "C"
