#!/usr/bin/env python
"""Benchmark: served SCF(+MP2) solves/s of the mixed-precision engine on GB300.

Headline workload (one "step" = one request of the stream): the serving
stream of the batched, served SCF -- Poisson arrivals (default 50
req/s), H/C/N/O chain molecules of the batched-RHF generator grown to a size
drawn log-uniformly from 30-1200 Cartesian functions, 70 % RHF and 30 % RHF +
frozen-core MP2, admitted under a 150 GB HBM budget -- served by the
continuous-batching engine (openlowdin_gb300.serve) in mixed precision (FP32
integrals below the 1e-5 Schwarz-density bound, incremental builds, FP64
check of every converged job, split-BF16 tensor-core MP2 transform).  The
same requests are served by the plain FP64 engine; every job's energy is
compared with its plain result (the plain path is pinned to the oracle).  K
steps = K requests drawn from the 10,000-request stream's generator (seed
fixed); W warm-up requests (a different seed, up to 300 functions) are
served before timing.  Synthetic inputs stand in for any dataset.

Sections of the JSON line:
  value / variants  -- mixed and plain served solves/s (converged jobs only),
                       p50/p99 latency, offered and served rates, per-job
                       errors.
  e2e               -- the same requests through the reference-facing C ABI
                       (LibintInterface_compute_2body_direct with host buffers,
                       the reference program's calling pattern, FP64), the
                       MP2 of MP2 requests through LowdinGB300_mp2_direct with
                       host-resident orbitals copied in.
  roofline          -- the FP64 J/K kernels (one plain build of the stream's
                       largest molecule, CUDA events) against the FP64 FMA
                       peak measured in the run; the FP32 row kernels beside.
  cpu_baseline      -- the oracle port (C/OpenMP, all host threads) on every
                       request of the stream: setup + one SCF iteration,
                       scaled by the request's plain iteration count.
  c1_apmo_batch, c2_mp2, c3_random_batch -- the other workloads (4-water APMO
                       batch; 16-water d-shell RMP2 transform FP64 vs
                       split-BF16; random-molecule batch).
  --impl reference  -- the oracle port on the host cores, same stream: per
                       step one request, setup + one timed SCF iteration,
                       scaled to a solve.
Multi-GPU: replicas (each rank serves its own stream, no collective in the
data path); rank 0 prints the JSON line.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

# one BLAS thread per host eigensolver worker (set before numpy is imported)
os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "SCF(+MP2) solves/s and p50/p99 latency, mixed vs plain FP64 GPU at 1e-6 Eh"
UNIT = "solves/s"
STREAM_LO, STREAM_HI, MP2_FRACTION = 30, 1200, 0.3
WORKLOAD = ("serving stream: Poisson arrivals, H/C/N/O chain molecules log-uniform 30-1200 Cartesian functions, "
            "70% RHF / 30% RHF+frozen-core MP2, 150 GB HBM budget; SCF to dE<1e-8 Eh, rms dP<1e-6 (MP2 jobs "
            "dE<1e-10, rms dP<1e-8)")
APMO_WORKLOAD = ("APMO HF, 4-water cluster: e- 136 Cartesian fn (40 e-) + 8 one-proton species "
                 "(7 fn each, s 4/8/16/24 + p 16), classical O; dE<1e-8 Eh, rms dP<1e-6")
# mean SCF iterations of a plain solve of the stream's requests (GB300 runs of
# this benchmark); the reference arm scales its one-iteration samples by it
STREAM_ITERATIONS = 32.0


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--serve-rate", type=float, default=50.0, help="Poisson arrival rate of the stream (req/s)")
    ap.add_argument("--seed", type=int, default=0, help="stream seed (rank r serves seed + r)")
    ap.add_argument("--batch", type=int, default=8, help="molecules of the APMO batch section (0: off)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer C ABI leg")
    ap.add_argument("--e2e-plain", action="store_true", help="also run the host-buffer C ABI leg in plain FP64")
    ap.add_argument("--no-mp2", action="store_true", help="skip the d-shell MP2 transform section")
    ap.add_argument("--mp2-waters", type=int, default=16)
    ap.add_argument("--random-molecules", type=int, default=16,
                    help="batched-RHF section over this many random chain molecules (0: off)")
    ap.add_argument("--profile-fock", type=int, default=0,
                    help="profiling case: N batched Fock builds of the step's molecules at the "
                         "core-Hamiltonian-guess densities, then exit")
    ap.add_argument("--profile-precision", type=int, default=0,
                    help="precision bits of the profiled builds (0 FP64, 3 mixed split)")
    ap.add_argument("--profile-split", type=float, default=1e-5,
                    help="with --profile-fock: FP32/FP64 split bound of the mixed build")
    ap.add_argument("--profile-random", type=int, default=0,
                    help="with --profile-fock: this many random chain molecules (batched-RHF generator)")
    ap.add_argument("--profile-chain", type=int, default=0,
                    help="with --profile-fock: one chain molecule of the serving generator with at least this "
                         "many functions instead of the APMO batch")
    ap.add_argument("--profile-d-waters", type=int, default=0,
                    help="with --profile-fock: one cluster of this many waters with a d shell on O "
                         "instead of the APMO batch")
    ap.add_argument("--profile-gemm", type=int, default=0,
                    help="profiling case: tensor-core GEMM engine (2 / 3 pieces, 8 precise) on the MP2 "
                         "first-quarter shape M=128 N=65536 K=640, three launches, then exit")
    ap.add_argument("--profile-mp2", type=int, default=-1,
                    help="profiling case: one MP2 of the d-shell water cluster (--mp2-waters) at this "
                         "precision (0 FP64, 1 / 2 split BF16), then exit")
    return ap.parse_args()


def profile_fock(args):
    """Small, self-contained case for ncu: setup + N batched builds."""
    import torch
    from openlowdin_gb300.batch_scf import BatchSCF
    torch.cuda.set_device(0)
    from openlowdin_gb300 import flops as FL
    from openlowdin_gb300 import systems as S
    if args.profile_chain:
        mols = [S.chain_for_basis(10_007, args.profile_chain)]
    elif args.profile_d_waters:
        mols = [S.water_cluster(args.profile_d_waters, seed=0, o_d=True)]
    elif args.profile_random:
        mols = [S.chain_molecule(20_000 + i) for i in range(args.profile_random)]
    else:
        mols = systems_for(0, args.batch)
    s = BatchSCF(mols)
    s.batch.use_graph(False)          # profiling case: every launch eager
    st = torch.cuda.current_stream().cuda_stream
    for g in s.groups.values():
        g.Pin.copy_(s._density(g, g.H) if g.ragged else s._purify(g, g.H))
    torch.cuda.synchronize()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(args.profile_fock):
        s.batch.fock(args.profile_precision, args.profile_split, st)
    b.record()
    torch.cuda.synchronize()
    ms = a.elapsed_time(b) / max(1, args.profile_fock)
    q, qc = s.batch.quartets(st), s.batch.coupling_quartets(st)
    fl = FL.class_table_flops(q, "jk") + FL.class_table_flops(qc, "coupling")
    print(json.dumps({"profile_fock_builds": args.profile_fock, "molecules": len(mols), "ms_per_build": ms,
                      "quartets": int(q.sum() + qc.sum()), "quartets_by_class": q.tolist(),
                      "tflops": fl / (ms * 1e-3) / 1e12}))
    s.close()
    return 0


def replica_seeds(rank, batch):
    """Molecule seeds of one rank: replicas solve disjoint molecules, so the
    multi-GPU form has no collective in the data path."""
    return [rank * batch + i for i in range(batch)]


def reduce_step_times(values, dist, device):
    """Max over ranks of this rank's timed totals (the slowest rank sets the
    whole job's time); returns floats."""
    import torch
    t = torch.tensor(values, dtype=torch.float64, device=device)
    if dist is not None:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t]


def whole_job_rate(units_per_rank, world, total_ms):
    """Units of all ranks per second of the max-over-ranks time."""
    return units_per_rank * world / (total_ms * 1e-3)


def systems_for(rank, batch):
    from openlowdin_gb300 import systems as S
    return [S.water_cluster(4, seed=sd, quantum_protons=True) for sd in replica_seeds(rank, batch)]


# ------------------------------------------------------------------ clocks --
class ClockSampler:
    """nvidia-smi clock / throttle-reason sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------- serving --
def serving_requests(n, rate, seed=0, lo=STREAM_LO, hi=STREAM_HI, mp2_frac=MP2_FRACTION):
    """Seeded open-loop stream: Poisson arrivals, chain molecules with sizes
    log-uniform in [lo, hi] functions, mp2_frac of the requests SCF+MP2."""
    import numpy as np
    from openlowdin_gb300 import serve, systems as S
    rng = np.random.Generator(np.random.PCG64(seed))
    t, reqs = 0.0, []
    for i in range(n):
        t += rng.exponential(1.0 / rate)
        nbf = int(np.exp(rng.uniform(np.log(lo), np.log(hi))))
        kind = "scf+mp2" if rng.random() < mp2_frac else "scf"
        reqs.append(serve.Request(S.chain_for_basis(10_000 + seed * 100_000 + i, nbf), kind, t, i))
    return reqs


def serve_stream(reqs, precision, flush=None, engines=None):
    """Serve `reqs` in real time with one engine; returns (results, seconds,
    CUDA-event milliseconds, kernels launched)."""
    import torch
    from openlowdin_gb300 import lint, serve
    eng = serve.ServingEngine(precision=precision)
    if engines is not None:
        engines.append(eng)
    if flush is not None:
        flush.fill_(1.0)              # L2 flush before the timed stream
    torch.cuda.synchronize()
    l0 = lint.launch_count()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    a.record()
    r = eng.run(reqs)
    b.record()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    return r, wall, a.elapsed_time(b), lint.launch_count() - l0


def stream_summary(res, wall, reqs, rate):
    """Converged solves/s, latency and rates of one served stream."""
    from openlowdin_gb300 import serve
    conv = [x for x in res if x.converged]
    lat = serve.latency_stats(conv)
    span = max(r.arrival for r in reqs) if reqs else 0.0
    return {"solves_per_s": len(conv) / wall, "converged": len(conv), "requests": len(res), "wall_s": wall,
            "p50_s": lat["p50_s"], "p99_s": lat["p99_s"], "offered_rate_req_s": rate,
            "arrival_span_s": span, "served_rate_req_s": len(conv) / wall,
            "iterations_mean": float(sum(x.iterations for x in res) / max(1, len(res)))}


def tuning_summary(tuning):
    """Per quartet class of the mixed builds: how often the autotuner kept the
    bra-row FP32 kernel or the one-quartet-per-thread one, and the median
    timings (ms) of both where they were timed."""
    import numpy as np
    names = ["ss", "ps", "pp", "ds", "dp", "dd", "fs", "fp", "fd", "ff"]
    out = {}
    for b in range(len(names)):
        for k in range(b + 1):
            ch = [int(t[0][b, k]) for t in tuning if t[0][b, k] >= 0]
            if not ch:
                continue
            ra = [float(t[1][b, k]) for t in tuning if t[1][b, k] > 0]
            tl = [float(t[2][b, k]) for t in tuning if t[2][b, k] > 0]
            out[f"({names[b]}|{names[k]})"] = {
                "rows_kernel": ch.count(1), "tile_kernel": ch.count(0),
                "median_ms_rows": float(np.median(ra)) if ra else None,
                "median_ms_tiles": float(np.median(tl)) if tl else None}
    return {"batches": len(tuning), "classes": out}


def per_job_table(reqs, plain, mixed):
    """Every job: size, kind, iterations, plain energy, |E_mixed - E_plain|,
    the mixed job's own FP64-check error, |dE2|."""
    rows = []
    for q in reqs:
        p, m = plain.get(q.rid), mixed.get(q.rid)
        row = {"rid": q.rid, "nbasis": p.nbasis if p else None, "kind": q.kind,
               "iterations_plain": p.iterations if p else None, "iterations_mixed": m.iterations if m else None,
               "converged_plain": bool(p and p.converged), "converged_mixed": bool(m and m.converged),
               "E_plain_Eh": p.energy if p else None}
        if p and m:
            row["abs_dE_mixed_vs_plain_Eh"] = abs(m.energy - p.energy)
            row["err_vs_fp64_check_Eh"] = m.err_vs_fp64
            row["guard_hit"] = m.guard_hit
            if p.e2 is not None and m.e2 is not None:
                row["abs_dE2_mixed_vs_plain_Eh"] = abs(m.e2 - p.e2)
        rows.append(row)
    return rows


# ------------------------------------------------ e2e: reference-facing ABI --
def e2e_stream(reqs, precision="mixed", workers=16):
    """The stream's requests through the reference-facing C ABI with host
    buffers: HostSCF calls LibintInterface_compute_2body_direct every
    iteration (host density in, host matrix out, the copies inside), host
    linear algebra as the Fortran caller does; MP2 requests then run
    LowdinGB300_mp2_direct on orbitals copied in from the host.  "mixed": the
    handles' FP32/FP64 split (LowdinGB300_set_precision), density changes
    passed in after the first build, an FP64 build at the converged density
    for the stated error, split-BF16 MP2.  Requests are solved concurrently
    (one host thread each, up to `workers`)."""
    import concurrent.futures as cf
    import numpy as np
    import torch
    from openlowdin_gb300 import lint, scf, systems as S

    def one(q):
        hs = scf.HostSCF(q.system, precision=precision)
        r = hs.solve(tol_energy=1e-10, tol_density=1e-8) if q.kind == "scf+mp2" else \
            hs.solve(tol_energy=1e-8, tol_density=1e-6)
        n = hs.handles[0].nbasis
        up = down = r.iterations * 8 * n * n       # D up, G down per iteration
        e2 = None
        if q.kind == "scf+mp2" and r.converged:
            sp = q.system["species"][0]
            st = torch.cuda.Stream()
            with torch.cuda.stream(st):
                dD = torch.from_numpy(np.ascontiguousarray(r.densities[0])).pin_memory().to("cuda", non_blocking=True)
                dC = torch.from_numpy(np.ascontiguousarray(r.coefficients[0].T)).pin_memory().to(
                    "cuda", non_blocking=True)
                e2 = hs.handles[0].mp2_direct(dD.data_ptr(), dC.data_ptr(), r.orbital_energies[0],
                                              sp["n_particles"] // 2, S.n_core(q.system),
                                              2 if precision == "mixed" else 0, 8.0, stream=st.cuda_stream)
            up += 2 * 8 * n * n
            down += 8
        hs.close()
        return r, e2, up, down

    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(max_workers=min(workers, len(reqs))) as ex:
        out = list(ex.map(one, reqs))
    wall = time.perf_counter() - t0
    return out, wall


# ------------------------------------------------------------- CPU oracle --
def oracle_request_sample(sysd, nthreads):
    """Oracle port on the host cores for one request: (seconds of its set-up
    -- one-electron matrices, S^-1/2, core-Hamiltonian guess --, seconds of
    one complete SCF iteration: Fock build, energy, DIIS, eigensolve,
    density).  The iteration is the difference of a one-iteration SCF run and
    the set-up timed on its own."""
    import numpy as np
    from oracle import lowdin_oracle as O
    sysO = O.from_plain(sysd)
    t0 = time.perf_counter()
    for s in sysO.species:
        Sm, T = O.overlap_kinetic(s.basis)
        V = O.potential(s.basis, sysO.point_charges, sysO.point_positions)
        H = T / s.mass + s.charge * V
        w, U = np.linalg.eigh(Sm)
        X = (U * w ** -0.5) @ U.T
        e, Cp = np.linalg.eigh(X.T @ H @ X)
    setup = time.perf_counter() - t0
    t0 = time.perf_counter()
    O.scf(sysO, max_iter=1, nthreads=nthreads)
    t1 = time.perf_counter() - t0
    return setup, max(t1 - setup, 1e-9)


def random_batch_section(args):
    """Batched RHF over independent random chain molecules (H/C/N/O, 3-30
    atoms, the generator of the batched-RHF workload): padded size buckets,
    converged molecules switched off, plain FP64 and mixed, one solve of the
    whole batch each (a bounded sample of the 512-molecule batch)."""
    import numpy as np
    import torch
    from openlowdin_gb300 import systems as S
    from openlowdin_gb300.batch_scf import PipelinedSCF
    mols = [S.chain_molecule(20_000 + i) for i in range(args.random_molecules)]
    nbf = [S.nbasis(m["species"][0]) for m in mols]
    out = {"molecules": len(mols), "functions_min": int(min(nbf)), "functions_max": int(max(nbf)),
           "functions_total": int(sum(nbf)),
           "note": "bounded sample of the 512-molecule batch; one SCF of every molecule per precision"}
    res = {}
    for prec in ("fp64", "mixed"):
        s = PipelinedSCF(mols, precision=prec)
        out["buckets"] = sum(len(h.groups) for h in s.halves)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = s.solve()
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        s.close()
        res[prec] = r
        out["plain" if prec == "fp64" else "mixed"] = {
            "solves_per_s": len(r) / wall, "wall_s": wall, "converged": int(sum(x.converged for x in r)),
            "max_iterations": int(max(x.iterations for x in r))}
    both = [i for i in range(len(mols)) if res["fp64"][i].converged and res["mixed"][i].converged]
    de = [abs(res["mixed"][i].energy - res["fp64"][i].energy) for i in both]
    out["jobs_converged_in_both"] = len(both)
    out["max_abs_dE_mixed_vs_plain_Eh"] = float(max(de)) if de else None
    out["throughput_ratio_mixed_over_plain"] = out["mixed"]["solves_per_s"] / out["plain"]["solves_per_s"]
    return out


def mp2_profile_case(args):
    import numpy as np
    import torch
    from openlowdin_gb300 import lint, systems as S
    from openlowdin_gb300.batch_scf import BatchSCF
    nw = args.mp2_waters
    sysd = S.water_cluster(nw, seed=0, o_d=True)
    s = BatchSCF([sysd])
    r = s.solve(tol_energy=1e-9, tol_density=1e-7)[0]
    s.close()
    h = lint.Libint2Interface(sysd["species"][0], 1)
    dD = torch.tensor(r.densities[0], device="cuda")
    dC = torch.tensor(np.ascontiguousarray(r.coefficients[0].T), device="cuda")
    t0 = time.perf_counter()
    e2 = h.mp2_direct(dD.data_ptr(), dC.data_ptr(), r.orbital_energies[0], 5 * nw, nw, args.profile_mp2, 0.0,
                      stream=torch.cuda.current_stream().cuda_stream)
    h.close()
    return {"profile_mp2_precision": args.profile_mp2, "waters": nw, "e2": e2, "seconds": time.perf_counter() - t0}


def mp2_section(args):
    """MP2 four-index transform of a d-shell water cluster: FP64 (cuBLAS
    DGEMM) vs split-BF16 tensor cores (3 pieces, 8 products), same SCF
    orbitals; plus the tensor-core GEMM engine alone on the transform's
    first-quarter shape."""
    import numpy as np
    import torch
    from openlowdin_gb300 import lint, systems as S
    from openlowdin_gb300.batch_scf import BatchSCF
    nw = args.mp2_waters
    sysd = S.water_cluster(nw, seed=0, o_d=True)
    sp = sysd["species"][0]
    s = BatchSCF([sysd])
    r = s.solve(tol_energy=1e-9, tol_density=1e-7)[0]
    s.close()
    h = lint.Libint2Interface(sp, 1)
    dD = torch.tensor(r.densities[0], device="cuda")
    dC = torch.tensor(np.ascontiguousarray(r.coefficients[0].T), device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    nocc, nfz = 5 * nw, nw
    out = {"system": f"{nw} waters, one Cartesian d (1.2) on O: {h.nbasis} functions, {nocc - nfz} active "
                     f"occupied, {h.nbasis - nocc} virtual, frozen core {nfz}"}
    e2 = {}
    for prec, name in ((2, "split_bf16_tensor_cores"), (0, "fp64_dgemm")):
        h.mp2_direct(dD.data_ptr(), dC.data_ptr(), r.orbital_energies[0], nocc, nfz, prec, 0.0, stream=st)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2[prec] = h.mp2_direct(dD.data_ptr(), dC.data_ptr(), r.orbital_energies[0], nocc, nfz, prec, 0.0,
                                stream=st)
        out[name] = {"seconds": time.perf_counter() - t0, "e2_Eh": e2[prec]}
    h.close()
    out["abs_dE2_split_vs_fp64_Eh"] = abs(e2[2] - e2[0])
    out["speedup_split_over_fp64"] = out["fp64_dgemm"]["seconds"] / out["split_bf16_tensor_cores"]["seconds"]
    # the GEMM engines alone (kernel time, CUDA events): first-quarter shape
    M, N, K = 128, 1 << 17, 640
    peak = None
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peak = json.load(f)["bf16_tflops"]
    except (OSError, KeyError, ValueError):
        peak = None   # no measured peak on this machine: the fraction is left out
    gemms = {}
    for name, mode, products in (("split2_3products", 2, 3), ("split3_6products", 3, 6),
                                 ("precise_8products", 8, 8)):
        ms = lint.gemm_bench(M, N, K, mode, 5, st)
        useful = 2.0 * M * N * K / (ms * 1e-3) / 1e12
        gemms[name] = {"ms_per_launch": ms, "useful_tflops": useful, "tensor_tflops": useful * products,
                       "tensor_frac_of_measured_bf16": (useful * products / peak) if peak else None}
    out["gemm_engines"] = {"shape": f"M={M} N={N} K={K}, FP32 out", **gemms}
    return out


# ----------------------------------------------------------- reference arm --
def run_reference(args):
    """The oracle port (C/OpenMP, every host thread) on the same stream: step
    k = request k, timed as its set-up and one complete SCF iteration, a solve
    = set-up + STREAM_ITERATIONS iterations; requests in stream order until
    about 4 minutes of CPU work.  A complete CPU solve of a 1200-function
    request takes many minutes, so requests are sampled this way; MP2 requests
    count as their SCF (the oracle's per-orbital direct MP2 transform is not
    sampled)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    from oracle import lowdin_oracle as O
    from openlowdin_gb300 import systems as S
    O.build()
    nthreads = O.nthreads_default()
    warm = serving_requests(max(1, args.warmup), 1000.0, seed=9, hi=120)
    for q in warm:
        oracle_request_sample(q.system, nthreads)   # untimed warm-up requests
    reqs = serving_requests(args.steps, args.serve_rate, seed=args.seed)
    t_solves, t_meas, sizes = [], 0.0, []
    for q in reqs:                    # stream order (random sizes), at most ~4 min of CPU work
        t0 = time.perf_counter()
        setup, it = oracle_request_sample(q.system, nthreads)
        t_meas += time.perf_counter() - t0
        t_solves.append(setup + STREAM_ITERATIONS * it)
        sizes.append(S.nbasis(q.system["species"][0]))
        if t_meas > 240.0:
            break
    value = len(t_solves) / sum(t_solves)
    sample = (f"oracle port (C/OpenMP, {nthreads} threads) on the first {len(t_solves)} of the {len(reqs)} "
              f"requests of the stream ({min(sizes)}-{max(sizes)} functions): per request its set-up and one "
              f"complete SCF iteration (a one-iteration run minus the set-up timed alone), a solve = set-up + "
              f"{STREAM_ITERATIONS:g} iterations (mean plain iteration count of the stream on GB300); MP2 "
              f"requests sampled as their SCF; {t_meas:.0f} s of CPU sampling")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(t_solves) / len(reqs),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "requests": len(reqs), "seed": args.seed,
                       "step": "one request of the stream (bounded CPU sample, scaled to a solve)",
                       "parallelism": "rank 0 only"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# ------------------------------------------------------------ APMO batch --
def apmo_batch_section(args, dev):
    """The 4-water APMO batch (8 molecules, two alternating halves), one
    solve per precision, plain and mixed (FP64 check of every converged
    molecule in mixed)."""
    import torch
    from openlowdin_gb300.batch_scf import BatchSCF, PipelinedSCF
    mols = systems_for(0, args.batch)
    out = {"workload": APMO_WORKLOAD, "molecules": len(mols)}
    res = {}
    for prec in ("fp64", "mixed"):
        make = (lambda: PipelinedSCF(mols, precision=prec)) if len(mols) >= 2 else \
            (lambda: BatchSCF(mols, precision=prec))
        s = make()
        s.solve()                     # warm-up solve (graph capture, allocator)
        s.close()
        s = make()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = s.solve(tol_energy=1e-8, tol_density=1e-6)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        s.close()
        res[prec] = r
        out["plain" if prec == "fp64" else "mixed"] = {
            "solves_per_s": sum(x.converged for x in r) / wall, "wall_s": wall,
            "converged": int(sum(x.converged for x in r)),
            "iterations_mean": float(sum(x.iterations for x in r) / len(r))}
    out["max_abs_dE_mixed_vs_plain_Eh"] = float(max(abs(a.energy - b.energy)
                                                   for a, b in zip(res["fp64"], res["mixed"])))
    out["throughput_ratio_mixed_over_plain"] = out["mixed"]["solves_per_s"] / out["plain"]["solves_per_s"]
    return out


# --------------------------------------------------------------- roofline --
def roofline_section(sysd):
    """FP64 J/K kernels: one plain Fock build of `sysd` at its core-guess
    density (CUDA events on the launching stream, 3 builds), FLOPs from the
    frozen per-class model over the quartets the build evaluated, against the
    FP64 FMA throughput measured in this run.  Beside it the FP32 row kernels:
    the same build with every quartet in FP32 (split above every bound)."""
    import torch
    from openlowdin_gb300 import flops as FL, lint, systems as S
    from openlowdin_gb300.batch_scf import BatchSCF
    s = BatchSCF([sysd])
    g = list(s.groups.values())[0]
    g.Pin.copy_(s._density(g, g.H))
    st = torch.cuda.current_stream().cuda_stream
    out = {}
    for name, prec, split in (("fp64", 0, 0.0), ("fp32_rows", 1, 1e30)):
        s.batch.fock(prec, split, st)
        s.batch.fock(prec, split, st)
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        reps = 3
        a.record()
        for _ in range(reps):
            s.batch.fock(prec, split, st)
        b.record()
        torch.cuda.synchronize()
        ms = a.elapsed_time(b) / reps
        q = s.batch.quartets(st)
        fl = FL.class_table_flops(q, "jk")
        out[name] = {"ms_per_build": ms, "quartets": int(q.sum()), "flop_per_build": fl,
                     "achieved_tflops": fl / (ms * 1e-3) / 1e12}
    s.close()
    # the FMA-chain peaks, with the clocks seen while they ran
    clk = ClockSampler(torch.cuda.current_device())
    clk.start()
    peak64 = max(lint.measure_fma_tflops(True) for _ in range(3))
    peak32 = max(lint.measure_fma_tflops(False) for _ in range(3))
    peak_clocks = clk.stop()
    f64, f32 = out["fp64"], out["fp32_rows"]
    traffic = None
    prof = os.path.join(ROOT, "profiles", "roofline_traffic.json")
    if os.path.exists(prof):
        try:
            with open(prof) as f:
                tr = json.load(f)
            traffic = tr.get("bytes_per_build_at", {}).get(str(S.nbasis(sysd["species"][0])))
        except (OSError, ValueError):
            traffic = None
    return {"bound": "fp64", "achieved": f64["achieved_tflops"], "peak": peak64, "unit": "TFLOP/s",
            "frac": f64["achieved_tflops"] / peak64 if peak64 > 0 else None, "traffic": traffic,
            "kernel": "jk_tasks_kernel<double> (every J/K class launch of one plain FP64 Fock build)",
            "system": f"chain molecule, {S.nbasis(sysd['species'][0])} functions (largest request of the stream)",
            "ms_per_build": f64["ms_per_build"], "quartets": f64["quartets"], "flop_per_build": f64["flop_per_build"],
            "peak_source": "FP64 FMA throughput measured on this GPU in this run (LowdinGB300_measure_fma_tflops: "
                           "8 independent FMA chains per thread, 8 CTAs of 256 threads per SM, best of 3; "
                           "MEASURED_PEAKS.json has no FP64 entry)",
            "peak_clocks": peak_clocks,
            "fp32_rows": {"kernel": "jk32_row_kernel (all quartets in FP32)", "ms_per_build": f32["ms_per_build"],
                          "achieved": f32["achieved_tflops"], "peak": peak32,
                          "frac": f32["achieved_tflops"] / peak32 if peak32 > 0 else None}}


# ----------------------------------------------------------------- GPU arm --
def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.profile_fock:
        return profile_fock(args)
    if args.profile_gemm:
        import torch
        from openlowdin_gb300 import lint
        torch.cuda.set_device(0)
        ms = lint.gemm_bench(128, 1 << 16, 640, args.profile_gemm, 2)
        print(json.dumps({"profile_gemm_mode": args.profile_gemm, "ms_per_launch": ms}))
        return 0
    if args.profile_mp2 >= 0:
        import torch
        torch.cuda.set_device(0)
        print(json.dumps(mp2_profile_case(args)))
        return 0
    import numpy as np
    import torch
    from openlowdin_gb300 import lint, systems as S

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    reqs = serving_requests(args.steps, args.serve_rate, seed=args.seed + rank)
    warm = serving_requests(max(1, args.warmup), 1000.0, seed=9, hi=300)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    from openlowdin_gb300 import serve
    serve.warm_up()                   # GPU eigensolver set-up in its worker threads
    for prec in ("mixed", "fp64"):
        serve_stream(warm, prec)      # untimed warm-up requests

    # headline: the mixed engine on the stream
    barrier()
    clk = ClockSampler(local)
    clk.start()
    engs = []
    res_m, wall_m, ms_m, launches = serve_stream(reqs, "mixed", flush, engs)
    clocks = clk.stop()
    barrier()
    # the plain FP64 engine on the same requests
    res_p, wall_p, ms_p, _ = serve_stream(reqs, "fp64", flush)
    barrier()
    conv_m = sum(x.converged for x in res_m)
    conv_p = sum(x.converged for x in res_p)
    ms_m, ms_p = reduce_step_times([ms_m, ms_p], dist, dev)
    tot = torch.tensor([float(conv_m), float(conv_p)], dtype=torch.float64, device=dev)
    if dist is not None:
        dist.all_reduce(tot)
    value = float(tot[0]) / (ms_m * 1e-3)
    value_plain = float(tot[1]) / (ms_p * 1e-3)
    mixed = {x.rid: x for x in res_m}
    plain = {x.rid: x for x in res_p}
    table = per_job_table(reqs, plain, mixed)
    both = [r for r in table if r["converged_plain"] and r["converged_mixed"]]
    de = [r["abs_dE_mixed_vs_plain_Eh"] for r in both]
    de2 = [r["abs_dE2_mixed_vs_plain_Eh"] for r in both if "abs_dE2_mixed_vs_plain_Eh" in r]
    chk = [r["err_vs_fp64_check_Eh"] for r in both if r.get("err_vs_fp64_check_Eh") is not None]
    sizes = [S.nbasis(q.system["species"][0]) for q in reqs]
    sm = stream_summary(res_m, ms_m * 1e-3, reqs, args.serve_rate)
    sp_ = stream_summary(res_p, ms_p * 1e-3, reqs, args.serve_rate)

    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms_m / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64 (ERIs), bf16x3 split (MP2 GEMMs)",
           "data": "synthetic",
           "config": {"workload": WORKLOAD, "requests_per_step": 1, "requests": len(reqs), "seed": args.seed,
                      "arrivals": f"Poisson, {args.serve_rate:g} req/s offered",
                      "functions": [int(min(sizes)), int(max(sizes))], "functions_total": int(sum(sizes)),
                      "mp2_requests": int(sum(q.kind == "scf+mp2" for q in reqs)),
                      "precision": "mixed: FP32 ERIs below the 1e-5 Schwarz-density bound, incremental builds, "
                                   "FP64 check of every converged job; MP2 split-BF16 tensor cores",
                      "l2": "flushed before each timed stream (256 MiB write); a job's matrices exceed L2",
                      "parallelism": "replicas" if world > 1 else "single GPU",
                      "note": "bounded sample of the 10,000-request stream: `steps` requests of its generator"},
           "variants": {"mixed": sm, "plain_fp64": sp_,
                        "throughput_ratio_mixed_over_plain": value / value_plain if value_plain > 0 else None},
           "serving": {"jobs_converged_in_both": len(both),
                       "unconverged_plain": [r["rid"] for r in table if not r["converged_plain"]],
                       "unconverged_mixed": [r["rid"] for r in table if not r["converged_mixed"]],
                       "max_abs_dE_mixed_vs_plain_Eh": max(de) if de else None,
                       "max_err_vs_fp64_check_Eh": max(chk) if chk else None,
                       "max_abs_dE2_mixed_vs_plain_Eh": max(de2) if de2 else None,
                       "guard_hits": int(sum(bool(r.get("guard_hit")) for r in table)),
                       "autotune": tuning_summary(engs[0].tuning),
                       "per_job": table},
           "clocks": clocks, "gpu_launches": int(launches)}

    if rank == 0:
        if not args.no_e2e:
            for prec in (("mixed", "fp64") if args.e2e_plain else ("mixed",)):
                e2e_res, e2e_wall = e2e_stream(reqs, prec)
                up = sum(x[2] for x in e2e_res)
                down = sum(x[3] for x in e2e_res)
                conv = sum(x[0].converged for x in e2e_res)
                de_e2e = [abs(x[0].energy - plain[q.rid].energy) for x, q in zip(e2e_res, reqs)
                          if x[0].converged and plain[q.rid].converged]
                chk = [x[0].err_vs_fp64 for x in e2e_res if x[0].err_vs_fp64 is not None]
                line = {"value": conv / e2e_wall, "unit": UNIT, "h2d_bytes_per_step": up // len(reqs),
                        "d2h_bytes_per_step": down // len(reqs), "wall_s": e2e_wall, "converged": int(conv),
                        "precision": prec,
                        "max_abs_dE_vs_plain_engine_Eh": max(de_e2e) if de_e2e else None,
                        "max_err_vs_fp64_check_Eh": max(chk) if chk else None,
                        "guard_hits": int(sum(bool(x[0].guard_hit) for x in e2e_res)),
                        "path": "HostSCF: LibintInterface_compute_2body_direct with host buffers every "
                                "iteration (the reference program's calling pattern; host linear algebra), "
                                + ("the handles' FP32/FP64 split set once by LowdinGB300_set_precision, density "
                                   "changes after the first build, an FP64 build at the converged density, "
                                   if prec == "mixed" else "FP64, ")
                                + "MP2 via LowdinGB300_mp2_direct on orbitals copied from the host; requests "
                                  "solved concurrently, one host thread each"}
                out["e2e" if prec == "mixed" else "e2e_plain_fp64"] = line
        big = reqs[int(np.argmax(sizes))].system
        out["roofline"] = roofline_section(big)
        if not args.no_cpu_baseline:
            from oracle import lowdin_oracle as O
            O.build()
            nth = O.nthreads_default()
            t_est, t_meas = [], 0.0
            for q in reqs:            # stream order (random sizes), about 30 s of CPU work
                t0 = time.perf_counter()
                setup, it = oracle_request_sample(q.system, nth)
                t_meas += time.perf_counter() - t0
                t_est.append(setup + it * max(1, plain[q.rid].iterations))
                if t_meas > 30.0 and len(t_est) >= 3:
                    break
            out["cpu_baseline"] = {
                "value": len(t_est) / sum(t_est), "unit": UNIT, "cores": nth, "kind": "port",
                "sample": f"oracle port on {nth} host threads, the first {len(t_est)} requests of the stream: "
                          f"set-up and one complete SCF iteration each ({t_meas:.0f} s of CPU), a solve = set-up "
                          f"+ the request's plain iteration count x iteration; MP2 requests counted as their SCF"}
        if args.batch > 0:
            out["c1_apmo_batch"] = apmo_batch_section(args, dev)
        if not args.no_mp2:
            out["c2_mp2"] = mp2_section(args)
        if args.random_molecules > 0:
            out["c3_random_batch"] = random_batch_section(args)
        print(json.dumps(out))
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
