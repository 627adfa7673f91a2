"""Continuous-batching SCF / SCF+MP2 serving on one GPU.

Requests (a molecular system, "scf" or "scf+mp2") arrive over time.  The
engine loop

  1. admits waiting requests in arrival order while their estimated device
     footprint fits the HBM budget and the active set has room,
  2. (re)builds the library batch when the active set changed -- every active
     job's species in one LowdinGB300_Batch, so one batch_fock call per
     iteration builds the two-particle and coupling matrices of all of them,
  3. runs one SCF iteration of every active job (openLOWDIN's scheme 3,
     src/scf/MultiSCF.f90:276-440: each species updated from the previous
     densities, Pulay DIIS over all species of a job),
  4. retires converged jobs: "scf" jobs finish, "scf+mp2" jobs hand their
     orbitals to an MP2 worker thread that runs LowdinGB300_mp2_direct on its
     own CUDA stream, so their transforms overlap the next SCF iterations.

Densities, Fock matrices, DIIS histories and the handles' Schwarz tables stay
on the device for a job's whole life.  A job's result does not depend on the
other jobs in the mix: its J/K and coupling tasks touch only its own buffers.
"""
from __future__ import annotations

import queue
import threading
import time
from dataclasses import dataclass, field

import numpy as np

from . import lint
from .batch_scf import MIXED_SKIP
from .scf import _one_body_device, _orthogonaliser, coulomb_only, n_occ, nuclear_repulsion, occupied_subspace
from .systems import n_core

HOST_EIGH_MAX = 384


@dataclass
class Request:
    system: dict
    kind: str = "scf"            # "scf" or "scf+mp2"
    arrival: float = 0.0         # seconds after the start of the stream
    rid: int = 0


@dataclass
class Result:
    rid: int
    kind: str
    energy: float
    e2: float | None
    iterations: int
    converged: bool
    arrival: float
    admitted: float
    finished: float
    nbasis: int
    # mixed precision: |E_mixed - E_FP64| at the converged density (the FP64
    # check's rebuild), and whether the check sent the job on in FP64
    err_vs_fp64: float | None = None
    guard_hit: bool = False

    @property
    def latency(self) -> float:
        return self.finished - self.arrival


@dataclass
class _Species:
    n: int
    occ: int
    eta: float
    H: object
    S: object
    X: object
    P: object
    G: object
    J: object
    Pin: object
    Gb: object
    Jb: object
    Pref: object
    Flast: object = None


@dataclass
class _Job:
    req: Request
    handles: list
    sp: list
    enuc: float
    footprint: float
    admitted: float
    it: int = 0
    e_old: float = float("nan")
    energy: float = float("nan")
    hist_F: list = field(default_factory=list)
    hist_E: list = field(default_factory=list)
    hist_B: list = field(default_factory=list)
    # FP64 check of a mixed-precision solution (ServingEngine.guard): flag is
    # the job's batch flag (1 mixed, 2 every quartet in FP64), verify marks the
    # iteration that rebuilds its matrices in FP64 at the converged density
    flag: int = 1
    verify: bool = False
    e_mixed: float = float("nan")
    err_vs_fp64: float | None = None
    commutator: float | None = None
    guard_hit: bool = False


_POOLS = None
_TLS = threading.local()
_POOL_LOCK = threading.Lock()


def _pools():
    """(host LAPACK pool, GPU eigensolver pool), shared by every engine of the
    process: one BLAS thread per host worker; the GPU workers each use their
    own CUDA stream."""
    global _POOLS
    with _POOL_LOCK:
        if _POOLS is None:
            import concurrent.futures as cf
            import os
            _POOLS = (cf.ThreadPoolExecutor(max_workers=max(1, min(16, os.cpu_count() or 1))),
                      cf.ThreadPoolExecutor(max_workers=2))
    return _POOLS


def _side_stream(dev):
    if not hasattr(_TLS, "stream"):
        import torch
        _TLS.stream = torch.cuda.Stream(dev)
    return _TLS.stream


_LINALG_READY = False


def _load_linalg(dev):
    """torch loads its CUDA linear-algebra library on the first eigensolve,
    and that first call must not happen in two threads at once: make it
    once, here, under a lock."""
    global _LINALG_READY
    with _POOL_LOCK:
        if not _LINALG_READY:
            import torch
            torch.linalg.eigh(torch.eye(4, dtype=torch.float64, device=dev))
            torch.cuda.synchronize(dev)
            _LINALG_READY = True


def warm_up(device="cuda"):
    """Runs the GPU eigensolver once in every GPU worker thread (its library
    set-up and first-use kernel loading happen here, not in a served job)."""
    import torch
    dev = torch.device(device)
    _load_linalg(dev)

    def one():
        s = _side_stream(dev)
        with torch.cuda.stream(s):
            for n in (400, 800, 1200):
                a = torch.eye(n, dtype=torch.float64, device=dev) + 1e-3
                torch.linalg.eigh(a)
                torch.linalg.eigh(a.float())
        s.synchronize()
        return True

    one()

    pool = _pools()[1]
    futs = [pool.submit(one) for _ in range(4)]
    for f in futs:
        f.result()


def footprint_bytes(sysd, kind: str, diis_size: int = 10, mp2_budget_gb: float = 8.0) -> float:
    """Device bytes a job holds while active: per species 11 n^2 matrices plus
    2 * diis_size history matrices (FP64), the handle's pair data, and for
    MP2 jobs the transform's arrays (split-BF16 path: Y' in FP32, the integral
    batch, the per-orbital square)."""
    tot = 0.0
    for sp in sysd["species"]:
        n = sum((l + 1) * (l + 2) // 2 for l, _, _, _ in sp["shells"])
        ns = len(sp["shells"])
        tot += (11 + 2 * diis_size) * n * n * 8 + ns * ns * 300
    if kind == "scf+mp2":
        sp = sysd["species"][0]
        n = sum((l + 1) * (l + 2) // 2 for l, _, _, _ in sp["shells"])
        o = n_occ(sp)
        v = n - o
        ncols = n * (n + 1) / 2 * 1.2
        kp = (n + 63) // 64 * 64
        tot += v * o * ncols * 4 + mp2_budget_gb * 1e9 + v * kp * kp * 6 + o * v * v * 4
    return tot


class ServingEngine:
    def __init__(self, device="cuda", precision="fp64", split=1e-5, hbm_budget_gb=150.0, max_active=256,
                 diis_size=10, tol_energy=1e-8, tol_density=1e-6, max_iter=100, mp2_precision=None,
                 mp2_budget_gb=8.0, skip=None, guard=True, guard_energy=1e-6, guard_commutator=1e-4,
                 tol_energy_mp2=1e-10, tol_density_mp2=1e-8, refine_eigh=None, autotune=True):
        """guard (mixed precision): when a job converges, its matrices are
        rebuilt once in FP64 at the converged density; the FP64 energy is the
        job's result and |E_mixed - E_FP64| its stated error.  If that error
        exceeds guard_energy, or the largest element of the FP64 commutator
        X^T (FPS - SPF) X exceeds guard_commutator, the job continues in FP64
        (every quartet in the FP64 launches, full builds) until it converges.
        SCF+MP2 jobs converge to tol_energy_mp2 / tol_density_mp2: the MP2
        energy moves with the orbitals, and at rms(dP) < 1e-6 two converged
        solutions of one molecule can differ by 1e-6 Eh in E2.
        refine_eigh (default: mixed precision): densities of species of at
        least HOST_EIGH_MAX functions from an FP32 eigensolve whose occupied
        subspace is refined in FP64 (scf.occupied_subspace) instead of the
        FP64 eigensolver; the job's final orbitals always come from the FP64
        eigensolver.  autotune (mixed): each new cohort batch picks its FP32
        kernel per quartet class by timing (LowdinGB300_batch_autotune)."""
        import torch
        self.torch = torch
        self.dev = torch.device(device)
        self.precision = precision
        self.split = split
        self.skip = (MIXED_SKIP if skip is None else skip) if precision == "mixed" else 0.0
        self.budget = hbm_budget_gb * 1e9
        self.max_active = max_active
        self.diis_size = diis_size
        self.tol_energy = tol_energy
        self.tol_density = tol_density
        self.tol_energy_mp2 = tol_energy_mp2
        self.tol_density_mp2 = tol_density_mp2
        self.max_iter = max_iter
        self.mp2_precision = (2 if precision == "mixed" else 0) if mp2_precision is None else mp2_precision
        self.mp2_budget_gb = mp2_budget_gb
        self.guard = guard and precision == "mixed"
        self.refine_eigh = (precision == "mixed") if refine_eigh is None else bool(refine_eigh)
        self.autotune = autotune
        self.tuning = []     # (choice, ms rows, ms tiles) of every autotuned cohort batch
        self.guard_energy = guard_energy
        self.guard_commutator = guard_commutator
        self.stream = torch.cuda.current_stream(self.dev)
        _load_linalg(self.dev)
        self.mp2_stream = torch.cuda.Stream(self.dev)
        # optional phase timing (set to {} before run): synchronises the device
        # at each phase boundary, so only for diagnostics
        self.trace = None
        self._last = 0.0

    def _tick(self, name):
        if self.trace is None:
            return
        self.torch.cuda.synchronize(self.dev)
        now = time.perf_counter()
        self.trace[name] = self.trace.get(name, 0.0) + (now - self._last)
        self._last = now

    # ------------------------------------------------------------ helpers --
    def _host_pool(self):
        return _pools()[0]

    def _new_job(self, req: Request, now: float, footprint: float) -> _Job:
        torch = self.torch
        sysd = req.system
        handles = [lint.Libint2Interface(sp, k + 1) for k, sp in enumerate(sysd["species"])]
        H, S = _one_body_device(handles, sysd, self.dev, self.stream.cuda_stream)
        sps = []
        for k, sp in enumerate(sysd["species"]):
            n = handles[k].nbasis
            Xt = _orthogonaliser(S[k], host_max=HOST_EIGH_MAX)
            z = lambda: torch.zeros((n, n), dtype=torch.float64, device=self.dev)  # noqa: E731
            sps.append(_Species(n, n_occ(sp), float(sp["eta"]), H[k], S[k], Xt, z(), z(), z(), z(), z(), z(), z()))
        job = _Job(req, handles, sps, nuclear_repulsion(sysd), footprint, now)
        for s, P in zip(job.sp, self._densities([(s, s.H) for s in job.sp])):
            s.P.copy_(P)                                  # core-Hamiltonian guess
            s.Flast = s.H.clone()
        return job

    def _densities(self, items):
        return self._density_collect(self._density_submit(items))

    def _density_submit(self, items):
        """Start eta C_occ C_occ^T for a list of (species, F) without waiting
        for the GPU: X^T F X is queued on the engine's stream; matrices below
        HOST_EIGH_MAX functions go to the host pool as one pinned copy (a pool
        thread waits for the copy's event, then runs LAPACK), larger ones to a
        GPU worker thread that runs the FP64 eigensolver and the density on its
        own stream after an event of the engine's stream.  The caller can queue
        the other cohort's Fock build at once: it overlaps these eigensolves."""
        torch = self.torch
        main = self.stream
        out = [None] * len(items)
        host_idx, host_mats, gpu_futs = [], [], {}
        for i, (s, F) in enumerate(items):
            Fp = s.X.T @ F @ s.X
            if s.n >= HOST_EIGH_MAX:
                ev = torch.cuda.Event()
                ev.record(main)
                gpu_futs[i] = self._gpu_pool().submit(self._gpu_density, s, Fp, ev)
            else:
                host_idx.append(i)
                host_mats.append(Fp)
        futs = []
        if host_idx:
            sizes = [m.numel() for m in host_mats]
            flat = torch.cat([m.reshape(-1) for m in host_mats])
            pinned = torch.empty(flat.shape, dtype=flat.dtype, pin_memory=True)
            pinned.copy_(flat, non_blocking=True)
            ready = torch.cuda.Event()
            ready.record(main)
            offs = np.cumsum([0] + sizes)

            def work(j):
                ready.synchronize()
                i = host_idx[j]
                n = items[i][0].n
                w, V = np.linalg.eigh(pinned.numpy()[offs[j]:offs[j + 1]].reshape(n, n))
                return np.ascontiguousarray(V[:, :items[i][0].occ])

            futs = [self._host_pool().submit(work, j) for j in range(len(host_idx))]
        return items, out, host_idx, futs, gpu_futs

    def _gpu_density(self, s, Fp, ev):
        """eta C_occ C_occ^T of one large species on a worker stream (FP64
        eigensolver), after event ev of the engine's stream."""
        torch = self.torch
        side = self._side_stream()
        with torch.cuda.stream(side):
            side.wait_event(ev)
            Fp.record_stream(side)
            if self.refine_eigh:
                # mixed precision: FP32 eigensolve, FP64 refinement of the
                # occupied subspace (scf.occupied_subspace)
                Co = s.X @ occupied_subspace(Fp, s.occ)
            else:
                e, Cp = torch.linalg.eigh(Fp)
                Co = s.X @ Cp[:, :s.occ]
            P = s.eta * Co @ Co.T
            done = torch.cuda.Event()
            done.record(side)
        return P, done

    def _side_stream(self):
        return _side_stream(self.dev)

    def _gpu_pool(self):
        return _pools()[1]

    def _density_collect(self, pending):
        torch = self.torch
        items, out, host_idx, futs, gpu_futs = pending
        for i, f in gpu_futs.items():
            P, done = f.result()
            self.stream.wait_event(done)
            P.record_stream(self.stream)
            out[i] = P
        if host_idx:
            vecs = [f.result() for f in futs]
            allv = torch.from_numpy(np.concatenate([v.reshape(-1) for v in vecs])).to(self.dev, non_blocking=True)
            o = 0
            for j, i in enumerate(host_idx):
                s = items[i][0]
                Cp = allv[o:o + s.n * s.occ].reshape(s.n, s.occ)
                o += s.n * s.occ
                Co = s.X @ Cp
                out[i] = s.eta * Co @ Co.T
        return out

    def _build_batch(self, jobs):
        b = lint.Batch()
        for job in jobs:
            sps = job.req.system["species"]
            b.add_system(job.handles, [sp["charge"] for sp in sps], [sp["kappa"] / sp["eta"] for sp in sps],
                         [1 if sp["n_particles"] > 1 else 0 for sp in sps],
                         [s.Pin for s in job.sp], [s.Gb for s in job.sp], [s.Jb for s in job.sp])
        b.finalize(self.stream.cuda_stream)
        b.set_skip(self.skip)
        b.flags = [1] * len(jobs)
        b.tuned = False
        return b

    def _apply_flags(self, jobs, batch):
        """Batch flags of the jobs (2: every quartet of the job in FP64)."""
        flags = [job.flag for job in jobs]
        if flags != batch.flags:
            batch.set_active(flags, self.stream.cuda_stream)
            batch.flags = flags

    # --------------------------------------------------------- SCF step --
    def _iterate(self, jobs, batch):
        """One SCF iteration of every job of the list; returns the jobs that
        converged (or ran out of iterations)."""
        return self._iter_finish(self._iter_start(jobs, batch))

    def _iter_start(self, jobs, batch):
        """Fock build, assembly and DIIS of an SCF iteration; the eigensolves are
        left running on the host pool."""
        torch = self.torch
        mixed = self.precision == "mixed"
        # full builds: plain mode, a job's first iteration, and jobs in FP64
        # (the guard's check and what follows a failed check)
        fulls = [(not mixed) or job.it == 0 or job.flag == 2 for job in jobs]
        for job, full in zip(jobs, fulls):
            for s in job.sp:
                if full:
                    s.Pin.copy_(s.P)
                else:
                    torch.sub(s.P, s.Pref, out=s.Pin)
        if mixed:
            self._apply_flags(jobs, batch)
            if self.autotune and not batch.tuned:
                # FP32 kernel per quartet class, timed on this cohort's densities
                # (cached by class and size, so mostly a look-up)
                batch.autotune(self.split, stream=self.stream.cuda_stream)
                batch.tuned = True
                self.tuning.append(batch.tuning())
        self._tick("other")
        batch.fock(3 if mixed else 0, self.split, self.stream.cuda_stream)
        self._tick("fock")
        stats = []
        dmats = []
        for job, full in zip(jobs, fulls):
            Fs, Es = [], []
            energy = torch.tensor(job.enuc, dtype=torch.float64, device=self.dev)
            for s in job.sp:
                if full:
                    s.G.copy_(s.Gb)
                    s.J.copy_(s.Jb)
                else:
                    s.G += s.Gb
                    s.J += s.Jb
                s.Pref.copy_(s.P)
                F = s.H + s.G + s.J
                energy = energy + torch.sum(s.P * (s.H + 0.5 * s.G + 0.5 * s.J))
                FPS = F @ s.P @ s.S
                Fs.append(F)
                Es.append(s.X.T @ (FPS - FPS.T) @ s.X)
            job.hist_F.append(Fs)
            job.hist_E.append(Es)
            if len(job.hist_F) > self.diis_size:
                job.hist_F.pop(0)
                job.hist_E.pop(0)
                job.hist_B.pop(0)
                job.hist_B = [b[1:] for b in job.hist_B]
            h = len(job.hist_F)
            row = torch.stack([sum(torch.sum(e * f) for e, f in zip(Es, job.hist_E[j])) for j in range(h)])
            job.hist_B.append(row)
            if job.verify:
                comm = torch.stack([e.abs().max() for e in Es]).max()
                stats.append(torch.stack([energy, comm]))
            else:
                stats.append(torch.stack([energy, torch.zeros_like(energy)]))
        self._tick("assemble")
        # DIIS coefficients of all jobs on the device (LowdinGB300_diis_coefficients,
        # one launch per history length): no host round trip
        byh = {}
        for q, job in enumerate(jobs):
            byh.setdefault(len(job.hist_F), []).append(q)
        coefs = [None] * len(jobs)
        for h, qs in byh.items():
            if h < 2:
                continue
            E = torch.empty((len(qs), h, h), dtype=torch.float64, device=self.dev)
            for r, q in enumerate(qs):
                hb = jobs[q].hist_B
                for i in range(h):
                    E[r, i, :i + 1] = hb[i][:i + 1]
                    E[r, :i + 1, i] = hb[i][:i + 1]
            c = torch.empty((len(qs), h), dtype=torch.float64, device=self.dev)
            lint.diis_coefficients(E.data_ptr(), h, len(qs), c.data_ptr(), self.stream.cuda_stream)
            for r, q in enumerate(qs):
                coefs[q] = c[r]
        for job, c in zip(jobs, coefs):
            h = len(job.hist_F)
            for k, s in enumerate(job.sp):
                Fx = job.hist_F[-1][k] if c is None else sum(c[j] * job.hist_F[j][k] for j in range(h))
                dmats.append((s, Fx))
        self._tick("diis")
        return jobs, stats, self._density_submit(dmats)

    def _iter_finish(self, started):
        """Collect the eigensolves of an iteration started by _iter_start: new
        densities, convergence test."""
        torch = self.torch
        jobs, stats, pending = started
        newP = self._density_collect(pending)
        self._tick("density")
        dP = []
        k = 0
        for job in jobs:
            d = torch.zeros((), dtype=torch.float64, device=self.dev)
            for s in job.sp:
                Pn = newP[k]
                k += 1
                d = torch.maximum(d, torch.sqrt(torch.mean((Pn - s.P) ** 2)))
                s.Flast = job.hist_F[-1][job.sp.index(s)]
                s.P.copy_(Pn)
            dP.append(d)
        st = torch.stack(stats)
        vals = torch.stack([st[:, 0], torch.stack(dP), st[:, 1]]).cpu().numpy()
        self._tick("convergence")
        done = []
        for q, job in enumerate(jobs):
            job.it += 1
            e, d = float(vals[0, q]), float(vals[1, q])
            if job.req.kind == "scf+mp2":
                conv = abs(e - job.e_old) < self.tol_energy_mp2 and d < self.tol_density_mp2
            else:
                conv = abs(e - job.e_old) < self.tol_energy and d < self.tol_density
            job.e_old = e
            job.energy = e
            if job.verify:
                # the FP64 check: this iteration's matrices were rebuilt in FP64
                # at the density the mixed iterations converged to
                job.verify = False
                job.err_vs_fp64 = abs(e - job.e_mixed)
                job.commutator = float(vals[2, q])
                if job.err_vs_fp64 <= self.guard_energy and job.commutator <= self.guard_commutator:
                    job.converged = True
                    done.append(job)
                    continue
                # continue in FP64 (flag stays 2): full FP64 builds and a
                # fresh DIIS history (the mixed-precision Fock matrices leave it)
                job.guard_hit = True
                job.e_old = float("nan")
                job.hist_F, job.hist_E, job.hist_B = [], [], []
                continue
            if conv and self.guard and job.flag == 1 and job.it < self.max_iter:
                job.verify = True         # next iteration: FP64 rebuild at this density
                job.flag = 2
                job.e_mixed = e
                continue
            if conv and job.guard_hit:
                job.err_vs_fp64 = 0.0     # finished in FP64 after a failed check
            job.converged = conv
            if conv or job.it >= self.max_iter:
                done.append(job)
        return done

    # --------------------------------------------------------------- MP2 --
    def _mp2_worker(self, inbox, results, start):
        torch = self.torch
        while True:
            item = inbox.get()
            if item is None:
                return
            job, Fp, Pd, ev = item
            try:
                ev.synchronize()
                eps, V = np.linalg.eigh(Fp.cpu().numpy())
                C = job.sp[0].X.cpu().numpy() @ V
                self._mp2_one(job, C, eps, Pd.cpu().numpy(), results, start)
            finally:
                with self._lock:
                    self._used -= job.footprint

    def _mp2_one(self, job, C, eps, P, results, start):
        torch = self.torch
        sysd = job.req.system
        sp = sysd["species"][0]
        with torch.cuda.stream(self.mp2_stream):
            dC = torch.tensor(np.ascontiguousarray(C.T), device=self.dev)
            dD = torch.tensor(P, device=self.dev)
            e2 = job.handles[0].mp2_direct(dD.data_ptr(), dC.data_ptr(), eps, n_occ(sp), n_core(sysd),
                                           self.mp2_precision, self.mp2_budget_gb,
                                           stream=self.mp2_stream.cuda_stream)
        results.append(self._finish(job, e2, start))

    def _finish(self, job, e2, start):
        now = time.perf_counter() - start
        for h in job.handles:
            h.close()
        return Result(job.req.rid, job.req.kind, job.energy, e2, job.it, bool(getattr(job, "converged", False)),
                      job.req.arrival, job.admitted, now, job.sp[0].n, job.err_vs_fp64, job.guard_hit)

    # -------------------------------------------------------------- loop --
    def run(self, requests, realtime=True, on_iteration=None):
        """Serve `requests` (sorted by arrival).  realtime: requests become
        visible at start + arrival; otherwise all are visible at once.
        Returns the results in completion order.

        Active jobs form two cohorts, each with its own library batch, worked
        alternately: while one cohort's eigensolves run on the host pool, the
        other cohort's Fock build runs on the GPU."""
        torch = self.torch
        for r in requests:
            coulomb_only(r.system, "ServingEngine")
        pending = sorted(requests, key=lambda r: r.arrival)
        results = []
        cohorts = [[], []]
        batches = [None, None]
        dirty = [True, True]
        inflight = [None, None]
        self._used = 0.0
        self._lock = threading.Lock()
        inbox = queue.Queue()
        start = time.perf_counter()
        worker = threading.Thread(target=self._mp2_worker, args=(inbox, results, start), daemon=True)
        worker.start()
        pi = 0
        step = 0

        def retire(done):
            for job in done:
                for c in (0, 1):
                    if job in cohorts[c]:
                        cohorts[c].remove(job)
                        dirty[c] = True
                if job.req.kind == "scf+mp2":
                    # the final orbitals are computed by the MP2 worker: the
                    # loop only queues the transformed Fock matrix and an event
                    sp0 = job.sp[0]
                    Fp = sp0.X.T @ sp0.Flast @ sp0.X
                    ev = torch.cuda.Event()
                    ev.record(self.stream)
                    inbox.put((job, Fp, sp0.P.clone(), ev))
                else:
                    results.append(self._finish(job, None, start))
                    with self._lock:
                        self._used -= job.footprint

        try:
            while pi < len(pending) or cohorts[0] or cohorts[1] or inflight[0] or inflight[1]:
                c = step % 2
                step += 1
                # finish this cohort's previous iteration (its eigensolves ran
                # while the other cohort used the GPU)
                if inflight[c] is not None:
                    retire(self._iter_finish(inflight[c]))
                    inflight[c] = None
                # admission in arrival order under the HBM budget
                now = time.perf_counter() - start
                nact = len(cohorts[0]) + len(cohorts[1])
                while pi < len(pending) and (not realtime or pending[pi].arrival <= now) and nact < self.max_active:
                    req = pending[pi]
                    fp = footprint_bytes(req.system, req.kind, self.diis_size, self.mp2_budget_gb)
                    with self._lock:
                        if (nact or self._used > 0) and self._used + fp > self.budget:
                            break
                        self._used += fp
                    self._tick("other")
                    job = self._new_job(req, now, fp)
                    # the cohort with less work (sum of n^3) takes the job, so
                    # both cohorts have GPU work to overlap the other's eigensolves
                    work = [sum(sum(x.n ** 3 for x in j.sp) for j in cohorts[k]) for k in (0, 1)]
                    k = 0 if work[0] <= work[1] else 1
                    cohorts[k].append(job)
                    self._tick("admit")
                    dirty[k] = True
                    nact += 1
                    pi += 1
                if not cohorts[c]:
                    if not cohorts[1 - c] and inflight[1 - c] is None and pi < len(pending):
                        # idle: next arrival, or memory held by MP2 transforms still running
                        time.sleep(max(0.001, min(0.05, pending[pi].arrival - (time.perf_counter() - start))))
                    continue
                if dirty[c]:
                    if batches[c] is not None:
                        batches[c].close()
                    self._tick("other")
                    batches[c] = self._build_batch(cohorts[c])
                    self._tick("batch_build")
                    dirty[c] = False
                inflight[c] = self._iter_start(list(cohorts[c]), batches[c])
                if on_iteration is not None:
                    on_iteration(len(cohorts[0]) + len(cohorts[1]))
        finally:
            inbox.put(None)
            worker.join()
            for b in batches:
                if b is not None:
                    b.close()
        return results


def latency_stats(results):
    lat = np.array([r.latency for r in results])
    if not len(lat):
        return {"p50_s": None, "p99_s": None}
    return {"p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99))}
