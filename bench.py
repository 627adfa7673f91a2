#!/usr/bin/env python
"""Benchmark: SCF solves/s of the APMO workload on GB300.

Workload (one "step"): B independent APMO Hartree-Fock solves of seeded
4-water clusters (electrons: 136 Cartesian functions, 40 e-; quantum protons:
8 one-particle species of 7 functions each), each from the core-Hamiltonian guess
to |dE| < 1e-8 Eh and rms(dP) < 1e-6, including the per-molecule setup (one-
electron integrals, pair lists, Schwarz factors).  Synthetic inputs generated
by openlowdin_gb300.systems (seeds rank*B + i).

Arms:
  default        -- GPU, device-resident SCF driver (plain FP64 integrals);
                    `value` is solves/s over all ranks.  Also reports the mixed
                    FP32/FP64 variant, the end-to-end number through the host-
                    buffer C ABI (`e2e`), the roofline of the dominant kernel
                    and a CPU baseline of the oracle port on the host cores.
  --impl reference -- the CPU restatement of the reference's direct path
                    (oracle/, C + OpenMP, all host threads) on the same
                    workload; no GPU work.
Multi-GPU: replicas (each rank solves its own molecules, no collective in the
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
WORKLOAD = ("APMO HF, 4-water cluster: e- 136 Cartesian fn (40 e-) + 8 one-proton species "
            "(7 fn each, s 4/8/16/24 + p 16), classical O; dE<1e-8 Eh, rms dP<1e-6")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--batch", type=int, default=8, help="molecules per step")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving-stream section")
    ap.add_argument("--no-mp2", action="store_true", help="skip the MP2 transform section")
    ap.add_argument("--serve-requests", type=int, default=40)
    ap.add_argument("--serve-rate", type=float, default=100.0, help="Poisson arrival rate (req/s)")
    ap.add_argument("--mp2-waters", type=int, default=8)
    ap.add_argument("--random-molecules", type=int, default=32,
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
def serving_requests(n, rate, seed=0, lo=30, hi=300, mp2_frac=0.3):
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


def serving_section(args):
    """The continuous-batching engine on a bounded sample of the serving
    stream, plain FP64 and mixed, same requests."""
    import numpy as np
    from openlowdin_gb300 import serve
    warm = serving_requests(6, 1000.0, seed=9)
    for prec in ("fp64", "mixed"):
        serve.ServingEngine(precision=prec).run(warm, realtime=False)
    reqs = serving_requests(args.serve_requests, args.serve_rate)
    out = {"requests": len(reqs), "arrivals": f"Poisson, {args.serve_rate:g} req/s",
           "sizes": "chain molecules (H/C/N/O generator), 30-300 functions log-uniform", "mp2_fraction": 0.3,
           "hbm_budget_gb": 150, "note": "bounded sample of the 10,000-request stream (30-1200 functions) "
                                         "so the benchmark finishes in minutes"}
    res = {}
    for prec in ("fp64", "mixed"):
        eng = serve.ServingEngine(precision=prec)
        t0 = time.perf_counter()
        r = eng.run(reqs)
        wall = time.perf_counter() - t0
        res[prec] = {x.rid: x for x in r}
        lat = serve.latency_stats(r)
        out["plain" if prec == "fp64" else "mixed"] = {
            "solves_per_s": len(r) / wall, "p50_s": lat["p50_s"], "p99_s": lat["p99_s"], "wall_s": wall,
            "converged": int(sum(x.converged for x in r))}
    both = [i for i in res["fp64"] if res["fp64"][i].converged and res["mixed"][i].converged]
    de = [abs(res["mixed"][i].energy - res["fp64"][i].energy) for i in both]
    de2 = [abs(res["mixed"][i].e2 - res["fp64"][i].e2) for i in both if res["fp64"][i].e2 is not None]
    out["jobs_converged_in_both"] = len(both)
    out["unconverged_jobs"] = sorted(set(res["fp64"]) - set(both))
    out["max_abs_dE_mixed_vs_plain_Eh"] = float(max(de)) if de else None
    out["max_abs_dE_mp2_mixed_vs_plain_Eh"] = float(max(de2)) if de2 else None
    out["throughput_ratio_mixed_over_plain"] = out["mixed"]["solves_per_s"] / out["plain"]["solves_per_s"]
    return out


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


# ------------------------------------------------------------- CPU oracle --
def cpu_iteration_sample(sysd, nthreads):
    """One APMO Fock-build iteration of the oracle (all intra and coupling
    matrices from the core-Hamiltonian-guess densities) on host cores."""
    import numpy as np
    from oracle import lowdin_oracle as O
    O.build()
    sysO = O.from_plain(sysd)
    sp = sysO.species
    P = []
    for s in sp:
        Sm, T = O.overlap_kinetic(s.basis)
        V = O.potential(s.basis, sysO.point_charges, sysO.point_positions)
        H = T / s.mass + s.charge * V
        w, U = np.linalg.eigh(Sm)
        X = (U * w ** -0.5) @ U.T
        e, Cp = np.linalg.eigh(X.T @ H @ X)
        C = X @ Cp
        P.append(s.eta * C[:, :s.n_occ] @ C[:, :s.n_occ].T)
    t0 = time.perf_counter()
    for i, s in enumerate(sp):
        if s.n_particles > 1:
            O.two_body_direct(s.basis, s.is_electron, P[i], s.exchange_factor, nthreads)
        for j, o in enumerate(sp):
            if j != i:
                O.coupling_direct(s.basis, i + 1, o.basis, j + 1, P[j], nthreads)
    return time.perf_counter() - t0


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    from oracle import lowdin_oracle as O
    O.build()
    nthreads = O.nthreads_default()
    sysd = systems_for(0, 1)[0]
    # warm-up: one complete oracle SCF (gives the iteration count of a solve)
    t0 = time.perf_counter()
    res = O.scf(O.from_plain(sysd), tol_energy=1e-8, tol_density=1e-6, nthreads=nthreads)
    full = time.perf_counter() - t0
    iters = res.iterations
    for _ in range(max(0, args.warmup - 1)):
        cpu_iteration_sample(sysd, nthreads)
    times = [cpu_iteration_sample(sysd, nthreads) for _ in range(args.steps)]
    t_it = sum(times) / len(times)
    value = 1.0 / (t_it * iters)
    sample = (f"oracle port (C/OpenMP, {nthreads} threads): {args.steps} timed Fock-build iterations of the "
              f"4-water APMO system (G_e, G_p, both couplings); solve = {iters} iterations "
              f"(full oracle solve in warm-up took {full:.1f} s)")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_it * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "step": "one Fock-build iteration (bounded CPU sample)",
                       "parallelism": "rank 0 only"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


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
    from openlowdin_gb300 import flops as FL
    from openlowdin_gb300 import lint, scf

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

    mols = systems_for(rank, args.batch)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    from openlowdin_gb300.batch_scf import BatchSCF, PipelinedSCF

    def step(precision):
        s = PipelinedSCF(mols, precision=precision) if len(mols) >= 2 else BatchSCF(mols, precision=precision)
        res = s.solve(tol_energy=1e-8, tol_density=1e-6)
        s.close()
        return res

    def timed(precision, steps, warmup):
        for _ in range(warmup):
            step(precision)
        barrier()
        total_ms, results = 0.0, []
        st = torch.cuda.current_stream()
        for _ in range(steps):
            flush.fill_(1.0)               # L2 flush (256 MiB write) between timed steps
            torch.cuda.synchronize()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(st)
            results += step(precision)
            b.record(st)
            torch.cuda.synchronize()
            total_ms += a.elapsed_time(b)
        barrier()
        return total_ms, results

    # plain FP64: the headline
    launches0 = lint.launch_count()
    clk = ClockSampler(local)
    clk.start()
    ms_plain, res_plain = timed("fp64", args.steps, args.warmup)
    clocks = clk.stop()
    launches = lint.launch_count() - launches0
    # mixed FP32/FP64 integrals
    ms_mixed, res_mixed = timed("mixed", args.steps, max(1, args.warmup // 2))
    ms_plain, ms_mixed = reduce_step_times([ms_plain, ms_mixed], dist, dev)
    value = whole_job_rate(args.batch * args.steps, world, ms_plain)
    value_mixed = whole_job_rate(args.batch * args.steps, world, ms_mixed)
    mixed_err = max(abs(a.energy - b.energy) for a, b in zip(res_plain, res_mixed))
    iters = float(np.mean([r.iterations for r in res_plain]))

    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms_plain / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": WORKLOAD, "molecules_per_step_per_gpu": args.batch,
                      "iterations_per_solve": iters, "l2": "flushed between timed steps (256 MiB write)",
                      "parallelism": "replicas" if world > 1 else "single GPU",
                      "driver": "device-resident batched SCF in two alternating halves (host eigensolves of "
                                "one half overlap the other half's GPU Fock build)"},
           "variants": {"mixed_fp32_fp64": {"value": value_mixed, "unit": UNIT,
                                            "max_energy_diff_vs_plain_Eh": mixed_err,
                                            "ms_per_step": ms_mixed / args.steps},
                        "plain_energies_Eh": [r.energy for r in res_plain[:args.batch]]},
           "clocks": clocks, "gpu_launches": int(launches)}

    if rank == 0:
        # ---- e2e: the reference-shaped C ABI with host buffers every iteration,
        # the step's molecules solved concurrently (one host thread and one set
        # of handles, hence one CUDA stream per handle, per molecule)
        import concurrent.futures as cf

        def e2e_solve(m):
            hs = scf.HostSCF(m)
            r = hs.solve(tol_energy=1e-8, tol_density=1e-6)
            nb = [h.nbasis for h in hs.handles]
            sps = m["species"]
            up = down = 0
            # per iteration: each two-particle call moves D up and G down; each
            # coupling call (i <- j) moves D_j up and the n_i x n_i result down
            for i, sp in enumerate(sps):
                if sp["n_particles"] > 1:
                    up += r.iterations * 8 * nb[i] ** 2
                    down += r.iterations * 8 * nb[i] ** 2
                for j in range(len(sps)):
                    if j != i:
                        up += r.iterations * 8 * nb[j] ** 2
                        down += r.iterations * 8 * nb[i] ** 2
            hs.close()
            return up, down

        e2e_steps = max(1, min(2, args.steps))
        h2d = d2h = 0
        t0 = time.perf_counter()
        with cf.ThreadPoolExecutor(max_workers=len(mols)) as ex:
            for _ in range(e2e_steps):
                for up, down in ex.map(e2e_solve, mols):
                    h2d += up
                    d2h += down
        e2e_s = time.perf_counter() - t0
        out["e2e"] = {"value": args.batch * e2e_steps / e2e_s, "unit": UNIT,
                      "h2d_bytes_per_step": h2d // e2e_steps, "d2h_bytes_per_step": d2h // e2e_steps,
                      "path": "HostSCF: LibintInterface_compute_2body_direct / _compute_coupling_direct with "
                              "host buffers each iteration (numpy linear algebra on the host); the step's "
                              f"{len(mols)} molecules solved concurrently, one host thread each"}

        # ---- roofline of the integral kernels: one batched Fock build (all
        # J/K and coupling launches of the step's molecules) at converged densities
        s = BatchSCF(mols, precision="fp64")
        s.solve(tol_energy=1e-8, tol_density=1e-6)
        stv = torch.cuda.current_stream().cuda_stream
        s.batch.set_active([1] * len(mols), stv)   # the solve switched converged molecules off
        for _ in range(3):
            s.batch.fock(0, 0.0, stv)
        reps = 20
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(reps):
            s.batch.fock(0, 0.0, stv)
        b.record()
        torch.cuda.synchronize()
        ms = a.elapsed_time(b) / reps
        counts = s.batch.quartets(stv)
        cpc = s.batch.coupling_quartets(stv)
        fl = FL.class_table_flops(counts, "jk") + FL.class_table_flops(cpc, "coupling")
        peak64 = lint.measure_fma_tflops(True)
        peak32 = lint.measure_fma_tflops(False)
        achieved = fl / (ms * 1e-3) / 1e12
        traffic = None
        prof = os.path.join(ROOT, "profiles", "roofline_traffic.json")
        if os.path.exists(prof):
            try:
                with open(prof) as f:
                    traffic = json.load(f).get("bytes_per_build")
            except (OSError, ValueError):
                traffic = None
        out["roofline"] = {"bound": "fp64", "achieved": achieved, "peak": peak64, "unit": "TFLOP/s",
                           "frac": achieved / peak64 if peak64 > 0 else None, "traffic": traffic,
                           "kernel": "jk_tasks_kernel + cp_tasks_kernel (one batched Fock build of the step's "
                                     "molecules, FP64, converged densities)",
                           "ms_per_build": ms, "quartets_jk": int(counts.sum()),
                           "quartets_coupling": int(cpc.sum()), "flop_per_build": fl,
                           "peak_source": "measured FP64 FMA throughput of this GPU in this run "
                                          "(MEASURED_PEAKS.json has no FP64 entry)",
                           "fp32_peak_tflops": peak32}
        s.close()

        # ---- CPU baseline (oracle port on the host cores), bounded sample
        if not args.no_cpu_baseline:
            from oracle import lowdin_oracle as O
            nth = O.nthreads_default()
            t_it = cpu_iteration_sample(mols[0], nth)
            out["cpu_baseline"] = {"value": 1.0 / (t_it * iters), "unit": UNIT, "cores": nth, "kind": "port",
                                   "sample": f"one APMO Fock-build iteration (G_e, G_p, both couplings) of the "
                                             f"oracle on {nth} host threads: {t_it:.2f} s; solves/s = "
                                             f"1/(t_iter x {iters:.1f} iterations)"}
        if not args.no_serving:
            out["serving"] = serving_section(args)
        if not args.no_mp2:
            out["mp2"] = mp2_section(args)
        if args.random_molecules > 0:
            out["random_batch"] = random_batch_section(args)
        print(json.dumps(out))
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
