"""Batched, device-resident multi-species Hartree-Fock.

Every matrix of every species of every molecule stays in HBM.  Species are
grouped by (basis size, occupied count, eta) into stacked tensors [m, n, n], so
one SCF iteration over any number of molecules is

  1 library build (LowdinGB300_batch_fock: all J/K and coupling work, ~20
    kernel launches whatever the batch size),
  a fixed number of batched tensor ops per size group (Fock assembly, energy,
    commutator error, orthogonal transform, batched eigh, densities),
  one small host read (energies and density changes) for convergence,

which follows openLOWDIN's iteration scheme 3 (src/scf/MultiSCF.f90:276-440):
every species of a molecule is updated once per global iteration from the
previous densities, with Pulay DIIS over all species of the molecule.

Molecules of many different sizes (a batch of random molecules) share padded
size buckets: a member of n_i < n functions occupies the top-left n_i x n_i
block of its n x n slot (the library reads and writes it with row stride n),
its padding has S = 1, X = 1 and H = PAD on the diagonal (so the padded
orbitals sit far above every real one and are never occupied), and its own
occupation count.  Host eigensolves run on the n_i x n_i block only.  A
molecule that has converged leaves the iteration: the library drops its tasks
from the launches (LowdinGB300_batch_set_active), and its members leave the
group tensors and the DIIS history (_compact) after their final density and
Fock matrix are stored, so it costs nothing while the rest of the batch
iterates.
"""
from __future__ import annotations

import time
from dataclasses import dataclass

import numpy as np

from . import lint
from .scf import (SCFResult, _one_body_device, _orthogonaliser, _orthogonaliser_np, coulomb_only, n_occ,
                  nuclear_repulsion)

HOST_EIGH_MAX = 384   # matrices below this size are diagonalised on the host (single-threaded LAPACK beats the GPU solver up to ~350 functions)
PAD = 1.0e4           # diagonal of H on padded rows (far above every occupied orbital energy)
EXACT_GROUPS_MAX = 8  # bucket="auto": exact (n, occ, eta) groups up to this many, padded buckets beyond
# mixed builds drop quartets whose density-weighted bound (from the density
# change, in incremental builds) is below this threshold.  Without a check,
# 1e-12 once summed to 1.3e-6 Eh on one molecule of a 512-molecule batch; every
# mixed solution now ends with an FP64 rebuild at its converged density
# (the guard), which states the error and continues in FP64 above 1e-6 Eh.
# On 8 requests of the serving stream: 8 % less time, largest error 1.6e-8 Eh.
MIXED_SKIP = 1e-12


def bucket_size(n: int) -> int:
    """Padded size of the bucket holding n functions: multiples of 16 up to
    128, of 32 up to 256, of 64 above (at most ~25% padding past 64)."""
    step = 16 if n <= 128 else 32 if n <= 256 else 64
    return -(-n // step) * step


@dataclass
class _Full:
    """Every member of a group (the view the final orbitals are computed on)."""
    H: object
    S: object
    X: object
    nsq: object
    occ_mask: object
    sys_index: object
    sys_np: object
    ns: object
    occs: object
    members: list
    n: int
    occ: int
    eta: float
    ragged: bool


_COMPACT = ("H", "S", "X", "nsq", "occ_mask", "sys_index")   # device tensors sliced by _compact


@dataclass
class _Group:
    n: int
    occ: int
    eta: float
    members: list        # (system index, species index)
    ns: object = None    # per member: its own size n_i <= n (ragged groups)
    occs: object = None  # per member: its own occupied count
    ragged: bool = False
    H: object = None
    S: object = None
    X: object = None
    P: object = None
    G: object = None
    J: object = None
    C: object = None
    eps: object = None


class BatchSCF:
    """SCF of many independent systems at once on one GPU."""

    def __init__(self, systems, device="cuda", precision="fp64", split=1e-5, diis_size=10, rebuild_every=1000,
                 bucket="auto", skip=MIXED_SKIP, guard=True, guard_energy=1e-6, guard_commutator=1e-4):
        """bucket: False = one group per exact (n, occ, eta); True = padded
        size buckets (bucket_size) with per-member sizes and occupations;
        "auto" = exact groups when they are at most EXACT_GROUPS_MAX.
        skip (mixed only): quartets whose density-weighted bound (from the
        density change of an incremental build) is below skip are dropped.
        guard (mixed only): a system that converges is rebuilt once in FP64
        at its converged density; that FP64 energy is its result and
        |E_mixed - E_FP64| its stated error (SCFResult.err_vs_fp64).  Above
        guard_energy, or with an FP64 commutator element above
        guard_commutator, the system continues in FP64 until it converges."""
        import torch
        for sysd in systems:
            coulomb_only(sysd, "BatchSCF")
        self.torch = torch
        self.guard = guard and precision == "mixed"
        self.guard_energy = guard_energy
        self.guard_commutator = guard_commutator
        self.rebuild_every = rebuild_every
        self.trace = None
        self.dev = torch.device(device)
        self.systems = systems
        self.precision = precision
        self.split = split
        self.diis_size = diis_size
        self.handles = []       # per system: list of handles
        groups = {}
        self.where = []         # per system: list of (group key, slot)
        devmats = {}
        for sysd in systems:
            self.handles.append([lint.Libint2Interface(sp, k + 1) for k, sp in enumerate(sysd["species"])])
        # one-electron matrices on the device (LowdinGB300_one_body_device)
        stream = torch.cuda.current_stream(self.dev).cuda_stream
        exact = {(h.nbasis, n_occ(sp), float(sp["eta"]))
                 for sysd, hs in zip(systems, self.handles) for h, sp in zip(hs, sysd["species"])}
        padded = bool(bucket) if bucket != "auto" else len(exact) > EXACT_GROUPS_MAX
        for si, sysd in enumerate(systems):
            hs = self.handles[si]
            H, S = _one_body_device(hs, sysd, self.dev, stream)
            w = []
            for k, sp in enumerate(sysd["species"]):
                n_k, occ_k, eta = hs[k].nbasis, n_occ(sp), float(sp["eta"])
                key = (bucket_size(n_k), eta) if padded else (n_k, occ_k, eta)
                g = groups.setdefault(key, _Group(key[0], occ_k, eta, [], [], []))
                w.append((key, len(g.members)))
                g.members.append((si, k))
                g.ns.append(n_k)
                g.occs.append(occ_k)
                devmats.setdefault(key, []).append((H[k], S[k]))
            self.where.append(w)
        self.groups = groups
        for key, g in groups.items():
            g.ns = np.asarray(g.ns)
            g.occs = np.asarray(g.occs)
            g.occ = int(g.occs.max())
            g.ragged = bool((g.ns != g.n).any() or (g.occs != g.occ).any())
            if g.ragged:
                self._pad_members(g, devmats[key])
            else:
                g.H = torch.stack([h for h, _ in devmats[key]])
                g.S = torch.stack([s for _, s in devmats[key]])
            # S^-1/2 of every member: host LAPACK pool (one transfer) or the GPU solver
            if g.n < HOST_EIGH_MAX or g.ragged:
                Sh = g.S.cpu().numpy()
                Xs = list(self._host_pool().map(_orthogonaliser_np, [Sh[i, :k, :k] for i, k in enumerate(g.ns)]))
                Xp = np.zeros((len(Xs), g.n, g.n))
                for i, (x, k) in enumerate(zip(Xs, g.ns)):
                    if x.shape != (k, k):
                        raise ValueError(f"member {g.members[i]}: overlap of {k} functions is rank-deficient")
                    Xp[i, :k, :k] = x
                    Xp[i, range(k, g.n), range(k, g.n)] = 1.0
                g.X = torch.from_numpy(Xp).to(self.dev)
            else:
                g.X = torch.stack([_orthogonaliser(x) for x in g.S])
            g.sys_np = np.array([s for s, _ in g.members])
            g.nsq = torch.tensor((g.ns.astype(np.float64)) ** 2, device=self.dev)
            g.occ_mask = None
            if g.ragged:
                occ_mask = (np.arange(g.occ)[None, :] < g.occs[:, None]).astype(np.float64)
                g.occ_mask = torch.from_numpy(occ_mask).to(self.dev)[:, None, :]
            m = len(g.members)
            # library build buffers (fixed addresses, every member): input
            # density (P or P - P_ref) and outputs
            g.Pin = torch.zeros((m, g.n, g.n), dtype=torch.float64, device=self.dev)
            g.Gb = torch.zeros_like(g.Pin)
            g.Jb = torch.zeros_like(g.Pin)
        self.enuc = torch.tensor([nuclear_repulsion(s) for s in systems], dtype=torch.float64, device=self.dev)
        self.nsys = len(systems)
        # library batch: species buffers are slices of the stacked tensors
        self.batch = lint.Batch()
        for si, sysd in enumerate(systems):
            sps = sysd["species"]
            P, G, J, ld = [], [], [], []
            for k, sp in enumerate(sps):
                key, slot = self.where[si][k]
                g = groups[key]
                P.append(g.Pin[slot]); G.append(g.Gb[slot]); J.append(g.Jb[slot])
                ld.append(g.n)
            self.batch.add_system(self.handles[si], [sp["charge"] for sp in sps],
                                  [sp["kappa"] / sp["eta"] for sp in sps],
                                  [1 if sp["n_particles"] > 1 else 0 for sp in sps], P, G, J, ld=ld)
        self.batch.finalize(torch.cuda.current_stream(self.dev).cuda_stream)
        self.batch.set_skip(skip if precision == "mixed" else 0.0)
        for key, g in groups.items():
            g.sys_index = torch.tensor([s for s, _ in g.members], device=self.dev)
            # the whole group; the iteration works on the members still running
            # (_reset, _compact)
            g.full = _Full(H=g.H, S=g.S, X=g.X, nsq=g.nsq, occ_mask=g.occ_mask, sys_index=g.sys_index,
                           sys_np=g.sys_np, ns=g.ns, occs=g.occs, members=list(g.members), n=g.n, occ=g.occ,
                           eta=g.eta, ragged=g.ragged)

    def _pad_members(self, g, mats):
        """Stacked H and S of a ragged group: member i in the top-left
        n_i x n_i block, PAD / 1 on the diagonal of its padding."""
        torch = self.torch
        m = len(mats)
        g.H = torch.zeros((m, g.n, g.n), dtype=torch.float64, device=self.dev)
        g.S = torch.zeros_like(g.H)
        for i, (h, s_) in enumerate(mats):
            k = int(g.ns[i])
            g.H[i, :k, :k] = h
            g.S[i, :k, :k] = s_
            d = torch.arange(k, g.n, device=self.dev)
            g.H[i, d, d] = PAD
            g.S[i, d, d] = 1.0

    def close(self):
        self.batch.close()
        for hs in self.handles:
            for h in hs:
                h.close()

    # --------------------------------------------------------------- pieces --
    def _purify(self, g, F, max_iter=200, tol=1e-11):
        """Density of the n_occ lowest orbitals of F (all species of the group
        at once) by trace-conserving canonical purification (Palser and
        Manolopoulos, Phys. Rev. B 58, 12704 (1998)): batched GEMMs and traces
        only, no eigensolver.  Returns eta X P' X^T (exact groups only)."""
        torch = self.torch
        if g.ragged:
            raise ValueError("purification needs one occupation count per group")
        Fp = g.X.transpose(1, 2) @ F @ g.X
        m, n = Fp.shape[0], Fp.shape[-1]
        N = float(g.occ)
        I = torch.eye(n, dtype=Fp.dtype, device=Fp.device).expand(m, n, n)
        d = torch.diagonal(Fp, dim1=1, dim2=2)
        r = Fp.abs().sum(-1) - d.abs()
        fmin = (d - r).min(-1).values
        fmax = (d + r).max(-1).values
        mu = d.mean(-1)
        lam = torch.minimum(N / (fmax - mu), (n - N) / (mu - fmin))
        P = (lam / n)[:, None, None] * (mu[:, None, None] * I - Fp) + (N / n) * I
        for it in range(max_iter):
            P2 = P @ P
            P3 = P2 @ P
            t1 = torch.diagonal(P - P2, dim1=1, dim2=2).sum(-1)
            t2 = torch.diagonal(P2 - P3, dim1=1, dim2=2).sum(-1)
            c = torch.where(t1.abs() > 1e-300, t2 / t1, torch.full_like(t1, 0.5))
            up = ((1 + c)[:, None, None] * P2 - P3) / c[:, None, None]
            lo = ((1 - 2 * c)[:, None, None] * P + (1 + c)[:, None, None] * P2 - P3) / (1 - c)[:, None, None]
            P = torch.where((c >= 0.5)[:, None, None], up, lo)
            if it % 8 == 7 and float(t1.abs().max()) < tol:
                break
        P = 0.5 * (P + P.transpose(1, 2))
        return g.eta * (g.X @ P @ g.X.transpose(1, 2))

    _pool = None

    @staticmethod
    def _host_pool():
        import concurrent.futures as cf
        import os
        if BatchSCF._pool is None:
            BatchSCF._pool = cf.ThreadPoolExecutor(max_workers=max(1, min(16, os.cpu_count() or 1)))
        return BatchSCF._pool

    def _eigh_host(self, g, Fp, idx, occ_only):
        """LAPACK eigensolves of the members `idx` of group g on the host pool,
        each on its own n_i x n_i block.  Returns (w, V) with V[j] the member's
        n x occ (occ_only) or n x n eigenvectors, zero past its own size and
        occupation; w[j] its eigenvalues, PAD past its size."""
        host = Fp[idx].cpu().numpy() if len(idx) != len(g.members) else Fp.cpu().numpy()
        ncol = g.occ if occ_only else g.n
        V = np.zeros((host.shape[0], g.n, ncol))
        w = np.full((host.shape[0], g.n), PAD)

        def work(j0, j1):
            for j in range(j0, j1):
                i = idx[j]
                k, o = int(g.ns[i]), int(g.occs[i])
                e, U = np.linalg.eigh(host[j, :k, :k])
                w[j, :k] = e
                if occ_only:
                    V[j, :k, :o] = U[:, :o]
                else:
                    V[j, :k, :k] = U
                    V[j, range(k, g.n), range(k, g.n)] = 1.0

        m = host.shape[0]
        nchunk = max(1, min(m, 16))
        bounds = [(m * c // nchunk, m * (c + 1) // nchunk) for c in range(nchunk)]
        return w, V, [self._host_pool().submit(work, a, b) for a, b in bounds]

    def _on_host(self, g):
        return g.n < HOST_EIGH_MAX or g.ragged

    def _density(self, g, F):
        """eta C_occ C_occ^T of the Roothaan problem F C = S C e.  Matrices
        below HOST_EIGH_MAX functions (and every member of a ragged group) are
        diagonalised by LAPACK on a host thread pool (a 136 x 136 FP64
        eigensolve takes ~2 ms there against ~5 ms for the GPU solver, whose
        cost is latency, not arithmetic); larger ones use the GPU solver.  The
        orthogonal transforms and the density product stay on the GPU."""
        return self._density_collect(g, self._density_submit(g, F))

    def _diag(self, g, F):
        torch = self.torch
        Fp = g.X.transpose(1, 2) @ F @ g.X
        if not self._on_host(g):
            e, Cp = torch.linalg.eigh(Fp)
        else:
            w, V, futs = self._eigh_host(g, Fp, np.arange(len(g.members)), False)
            for f in futs:
                f.result()
            e = torch.from_numpy(w).to(self.dev)
            Cp = torch.from_numpy(V).to(self.dev)
        C = g.X @ Cp
        Co = C[:, :, :g.occ]
        if g.ragged:
            Co = Co * g.occ_mask
        return e, C, g.eta * Co @ Co.transpose(1, 2)

    # ------------------------------------------------ asynchronous densities --
    def _density_submit(self, g, F, skip=None):
        """Start eta C_occ C_occ^T of F C = S C e for every species of group g
        (members with skip[i] set are left out: their result is zero): host
        eigensolves go to the pool and return futures (the GPU stays free for
        other work meanwhile); large exact groups are solved on the GPU at once."""
        torch = self.torch
        Fp = g.X.transpose(1, 2) @ F @ g.X
        if not self._on_host(g):
            e, Cp = torch.linalg.eigh(Fp)
            Co = g.X @ Cp[:, :, :g.occ]
            return ("done", g.eta * Co @ Co.transpose(1, 2))
        idx = np.arange(len(g.members)) if skip is None else np.flatnonzero(~skip)
        if len(idx) == 0:
            return ("done", torch.zeros_like(F))
        _, V, futs = self._eigh_host(g, Fp, idx, True)
        return ("host", idx, V, futs)

    def _density_collect(self, g, pending):
        torch = self.torch
        if pending[0] == "done":
            return pending[1]
        _, idx, V, futs = pending
        for f in futs:
            f.result()
        Cp = torch.from_numpy(V).to(self.dev, non_blocking=True)
        if len(idx) != len(g.members):
            full = torch.zeros((len(g.members), g.n, g.occ), dtype=torch.float64, device=self.dev)
            full[torch.from_numpy(idx).to(self.dev)] = Cp
            Cp = full
        Co = g.X @ Cp
        return g.eta * Co @ Co.transpose(1, 2)

    # ---------------------------------------------------------- iteration --
    class _State:
        pass

    def _reset(self, g):
        """Iterate over every member of g again (start of a solve)."""
        torch = self.torch
        f = g.full
        for a in _COMPACT:
            setattr(g, a, getattr(f, a))
        g.sys_np, g.ns, g.occs, g.members = f.sys_np, f.ns, f.occs, list(f.members)
        m = len(f.members)
        g.alive_np = np.arange(m)
        g.alive = torch.arange(m, device=self.dev)
        g.compact = False
        g.P = torch.zeros((m, g.n, g.n), dtype=torch.float64, device=self.dev)
        g.G = torch.zeros_like(g.P)
        g.J = torch.zeros_like(g.P)
        g.Pref = torch.zeros_like(g.P)
        g.Pfinal = torch.zeros_like(g.P)
        g.Ffinal = torch.zeros_like(g.P)

    def _compact(self, st, gi, g, keep):
        """Drop the members of g whose systems converged (keep[i] False): their
        final density and Fock matrix are stored, and every per-member tensor
        of the iteration (matrices, DIIS history) shrinks to the members still
        running, so converged molecules cost no batched GEMMs either."""
        torch = self.torch
        idx = np.flatnonzero(keep)
        drop = np.flatnonzero(~keep)
        dl = torch.from_numpy(drop).to(self.dev)
        dpos = torch.from_numpy(g.alive_np[drop]).to(self.dev)
        g.Pfinal.index_copy_(0, dpos, g.P.index_select(0, dl))
        g.Ffinal.index_copy_(0, dpos, g.Flast.index_select(0, dl))
        il = torch.from_numpy(idx).to(self.dev)
        for a in _COMPACT + ("P", "G", "J", "Pref", "Flast"):
            v = getattr(g, a)
            if v is not None:
                setattr(g, a, v.index_select(0, il))
        for hist in (st.hist_F, st.hist_E):
            for h in hist:
                if h[gi] is not None:
                    h[gi] = h[gi].index_select(0, il)
        g.sys_np, g.ns, g.occs = g.sys_np[idx], g.ns[idx], g.occs[idx]
        g.members = [g.members[i] for i in idx]
        g.alive_np = g.alive_np[idx]
        g.alive = torch.from_numpy(g.alive_np).to(self.dev)
        g.compact = True

    def _state(self, tol_energy, tol_density, max_iter):
        torch = self.torch
        st = BatchSCF._State()
        st.t0 = time.perf_counter()
        st.stream = torch.cuda.current_stream(self.dev).cuda_stream
        st.groups = list(self.groups.values())
        for g in st.groups:
            self._reset(g)
            g.P.copy_(self._density(g, g.H))      # core-Hamiltonian guess
            g.Flast = g.H.clone()
        st.hist_F, st.hist_E, st.hist_B = [], [], []
        st.e_old = np.full(self.nsys, np.nan)
        st.final_e = np.zeros(self.nsys)
        st.conv = np.zeros(self.nsys, bool)
        st.iters = np.zeros(self.nsys, int)
        # FP64 check of mixed solutions: fp64[s] = the system's quartets all in
        # FP64 (batch flag 2) and full builds; verify[s] = this iteration is
        # the check; diis_first[s] = first DIIS entry used (set past the
        # mixed entries when a check fails)
        st.fp64 = np.zeros(self.nsys, bool)
        st.verify = np.zeros(self.nsys, bool)
        st.e_mixed = np.full(self.nsys, np.nan)
        st.err_fp64 = np.full(self.nsys, np.nan)
        st.guard_hit = np.zeros(self.nsys, bool)
        st.diis_first = np.zeros(self.nsys, np.int32)
        self.batch.set_active(np.ones(self.nsys, np.int32), st.stream)
        st.it = 0
        st.done = False
        st.tol_energy, st.tol_density, st.max_iter = tol_energy, tol_density, max_iter
        st.trace = self.trace
        st.last = [time.perf_counter()]
        return st

    def _tick(self, st, name):
        if st.trace is None:
            return
        self.torch.cuda.synchronize(self.dev)
        now = time.perf_counter()
        st.trace[name] = st.trace.get(name, 0.0) + (now - st.last[0])
        st.last[0] = now

    def _start(self, st):
        """Fock build, assembly and DIIS of one iteration; the eigensolves of
        the new densities are left running (see _finish)."""
        torch = self.torch
        st.it += 1
        it = st.it
        groups = st.groups
        mixed = self.precision == "mixed"
        # plain: full build from P every iteration (the reference's scheme).
        # mixed: incremental build from dP = P - P_ref on top of the previous
        # matrices, a full build (FP64 couplings) on the first and every
        # rebuild_every-th iteration; two-particle quartets whose Schwarz x
        # |dP| bound is below the split run in FP32, the rest in FP64, and
        # incremental couplings run in FP32 (their size scales with |dP|).
        full = (not mixed) or (it - 1) % self.rebuild_every == 0
        # systems in FP64 (an FP64 check, or after a failed one): full builds
        fmask = {}
        if not full and st.fp64.any():
            for gi, g in enumerate(groups):
                if g.members:
                    m = st.fp64[g.sys_np]
                    if m.any():
                        fmask[gi] = torch.from_numpy(m).to(self.dev)[:, None, None]
        for gi, g in enumerate(groups):
            if not g.members:
                continue
            src = g.P if full else g.P - g.Pref
            if gi in fmask:
                src = torch.where(fmask[gi], g.P, src)
            if g.compact:
                g.Pin.index_copy_(0, g.alive, src)
            else:
                g.Pin.copy_(src)
        if mixed and not getattr(self, "_tuned", False):
            # FP32 kernel per quartet class, timed on these densities
            self.batch.autotune(self.split, stream=st.stream)
            self._tuned = True
        # precision bits: 1 = two-particle FP32/FP64 split, 2 = coupling split
        self.batch.fock(3 if mixed else 0, self.split, st.stream)
        self._tick(st, "fock")
        for gi, g in enumerate(groups):
            if not g.members:
                continue
            Gb = g.Gb.index_select(0, g.alive) if g.compact else g.Gb
            Jb = g.Jb.index_select(0, g.alive) if g.compact else g.Jb
            if full:
                g.G.copy_(Gb)
                g.J.copy_(Jb)
            elif gi in fmask:
                g.G.copy_(torch.where(fmask[gi], Gb, g.G + Gb))
                g.J.copy_(torch.where(fmask[gi], Jb, g.J + Jb))
            else:
                g.G += Gb
                g.J += Jb
            g.Pref.copy_(g.P)
        energy = self.enuc.clone()
        comm = torch.zeros(self.nsys, dtype=torch.float64, device=self.dev)
        Fs, Es = [], []
        for g in groups:
            if not g.members:
                Fs.append(None)
                Es.append(None)
                continue
            F = g.H + g.G + g.J
            e_sp = torch.sum(g.P * (g.H + 0.5 * g.G + 0.5 * g.J), dim=(1, 2))
            energy.index_add_(0, g.sys_index, e_sp)
            FPS = F @ g.P @ g.S
            err = g.X.transpose(1, 2) @ (FPS - FPS.transpose(1, 2)) @ g.X
            if st.verify.any():
                comm.scatter_reduce_(0, g.sys_index, err.abs().amax(dim=(1, 2)), reduce="amax")
            Fs.append(F)
            Es.append(err)
        self._tick(st, "assemble")
        # Pulay DIIS per system over all of its species
        st.hist_F.append(Fs)
        st.hist_E.append(Es)
        if len(st.hist_F) > self.diis_size:
            st.hist_F.pop(0); st.hist_E.pop(0); st.hist_B.pop(0)
            st.hist_B = [b[:, 1:] for b in st.hist_B]
            st.diis_first = np.maximum(st.diis_first - 1, 0).astype(np.int32)
        h = len(st.hist_F)
        row = torch.zeros((self.nsys, h), dtype=torch.float64, device=self.dev)
        for gi, g in enumerate(groups):
            if not g.members:
                continue
            cur = Es[gi].reshape(len(g.members), -1)
            for j in range(h):
                d = torch.sum(cur * st.hist_E[j][gi].reshape(len(g.members), -1), dim=1)
                row[:, j].index_add_(0, g.sys_index, d)
        st.hist_B.append(row)
        if h >= 2:
            # error products of every system, solved on the device
            # (LowdinGB300_diis_coefficients): no host round trip
            E = torch.empty((self.nsys, h, h), dtype=torch.float64, device=self.dev)
            for i in range(h):
                E[:, i, :i + 1] = st.hist_B[i][:, :i + 1]
                E[:, :i + 1, i] = st.hist_B[i][:, :i + 1]
            coef = torch.empty((self.nsys, h), dtype=torch.float64, device=self.dev)
            first = torch.from_numpy(st.diis_first).to(self.dev) if st.diis_first.any() else None
            lint.diis_coefficients(E.data_ptr(), h, self.nsys, coef.data_ptr(), st.stream,
                                   first.data_ptr() if first is not None else 0)
        else:
            coef = None
        self._tick(st, "diis")
        st.pending = []
        for gi, g in enumerate(groups):
            if not g.members:
                st.pending.append(None)
                continue
            if coef is None:
                Fx = Fs[gi]
            else:
                c = coef[g.sys_index]                               # [m, h]
                Fx = sum(c[:, j, None, None] * st.hist_F[j][gi] for j in range(h))
            st.pending.append(self._density_submit(g, Fx))
        st.Fs = Fs
        st.energy = energy
        st.comm = comm

    def _finish(self, st):
        """Collect the eigensolves started by _start: new densities and the
        convergence test; sets st.done.  Converged systems leave the batch."""
        torch = self.torch
        dP = torch.zeros(self.nsys, dtype=torch.float64, device=self.dev)
        for gi, g in enumerate(st.groups):
            if not g.members:
                continue
            Pn = self._density_collect(g, st.pending[gi])
            d = torch.sqrt(torch.sum((Pn - g.P) ** 2, dim=(1, 2)) / g.nsq)
            dP = torch.maximum(dP, torch.zeros_like(dP).scatter_reduce_(0, g.sys_index, d, reduce="amax"))
            g.Flast = st.Fs[gi]
            g.P.copy_(Pn)
        self._tick(st, "density")
        stats = torch.stack([st.energy, dP, st.comm]).cpu().numpy()
        self._tick(st, "convergence")
        en, dpn, cmm = stats[0], stats[1], stats[2]
        active = ~st.conv
        st.final_e[active] = en[active]
        st.iters[active] = st.it
        newly = active & (np.abs(en - st.e_old) < st.tol_energy) & (dpn < st.tol_density)
        st.e_old[active] = en[active]
        flags_changed = False
        if self.guard:
            # systems whose FP64 check ran in this iteration
            chk = active & st.verify
            st.verify[:] = False
            if chk.any():
                err = np.abs(en - st.e_mixed)
                ok = chk & (err <= self.guard_energy) & (cmm <= self.guard_commutator)
                bad = chk & ~ok
                st.err_fp64[chk] = err[chk]
                newly = (newly & ~chk) | ok
                st.guard_hit |= bad
                st.e_old[bad] = np.nan
                st.diis_first[bad] = len(st.hist_F)      # entries from here on only
            # newly converged mixed systems: FP64 check next iteration
            start = newly & ~st.fp64
            if start.any() and st.it < st.max_iter:
                st.verify |= start
                st.fp64 |= start
                st.e_mixed[start] = en[start]
                newly &= ~start
                flags_changed = True
            st.err_fp64[newly & st.guard_hit] = 0.0
        st.conv |= newly
        st.done = bool(st.conv.all()) or st.it >= st.max_iter
        if (newly.any() or flags_changed) and not st.done:
            # a converged system keeps its energy, density and Fock matrix from
            # here on: its integral work is switched off and its members leave
            # the iteration's tensors; systems in FP64 get flag 2
            self.batch.set_active(np.where(st.conv, 0, np.where(st.fp64, 2, 1)).astype(np.int32), st.stream)
            for gi, g in enumerate(st.groups):
                if g.members:
                    keep = ~st.conv[g.sys_np]
                    if not keep.all():
                        self._compact(st, gi, g, keep)

    def _results(self, st):
        torch = self.torch
        # Roothaan orbitals of the last Fock matrix of every species (one eigh)
        for g in st.groups:
            if g.members:
                g.Pfinal.index_copy_(0, g.alive, g.P)
                g.Ffinal.index_copy_(0, g.alive, g.Flast)
            g.eps, g.C, _ = self._diag(g.full, g.Ffinal)
        q = self.batch.quartets(st.stream)
        quartets = int(q.sum())
        self.last_class_quartets = q
        out = []
        for si in range(self.nsys):
            eps, C, P = [], [], []
            for key, slot in self.where[si]:
                g = self.groups[key]
                k = int(g.full.ns[slot])
                eps.append(g.eps[slot, :k].cpu().numpy())
                C.append(g.C[slot, :k, :k].cpu().numpy())
                P.append(g.Pfinal[slot, :k, :k].cpu().numpy())
            r = SCFResult(float(st.final_e[si]), int(st.iters[si]), bool(st.conv[si]),
                          time.perf_counter() - st.t0, eps, C, P, quartets)
            if self.guard:
                r.err_vs_fp64 = None if np.isnan(st.err_fp64[si]) else float(st.err_fp64[si])
                r.guard_hit = bool(st.guard_hit[si])
            out.append(r)
        return out

    def solve(self, tol_energy=1e-8, tol_density=1e-6, max_iter=100):
        st = self._state(tol_energy, tol_density, max_iter)
        while not st.done:
            self._start(st)
            self._finish(st)
        return self._results(st)


class PipelinedSCF:
    """Two BatchSCF halves iterated alternately: while one half's host
    eigensolves run, the other half's Fock build, assembly and DIIS run on the
    GPU.  Same iteration scheme and results as BatchSCF (each system's
    arithmetic is unchanged; only the order of work across systems differs)."""

    def __init__(self, systems, **kw):
        if len(systems) < 2:
            raise ValueError("PipelinedSCF needs at least two systems")
        h = (len(systems) + 1) // 2
        self.halves = [BatchSCF(systems[:h], **kw), BatchSCF(systems[h:], **kw)]

    def close(self):
        for b in self.halves:
            b.close()

    def solve(self, tol_energy=1e-8, tol_density=1e-6, max_iter=100):
        a, b = self.halves
        sa = a._state(tol_energy, tol_density, max_iter)
        sb = b._state(tol_energy, tol_density, max_iter)
        a._start(sa)
        while not (sa.done and sb.done):
            if not sb.done:
                b._start(sb)        # half b on the GPU while half a's eigensolves run
            if not sa.done:
                a._finish(sa)
                if not sa.done:
                    a._start(sa)    # half a on the GPU while half b's eigensolves run
            if not sb.done:
                b._finish(sb)
        if not sa.done:
            a._finish(sa)
        return a._results(sa) + b._results(sb)
