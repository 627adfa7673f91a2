"""Multi-species Hartree-Fock drivers over the GPU two-particle library.

These are the caller side of the integral boundary, restated from openLOWDIN's
src/scf (MultiSCF.f90:276-440 iteration scheme 3, WaveFunction.f90):

  H_i = T_i / m_i + q_i V_i                          (WaveFunction.f90:471-570)
  X_i = S_i^{-1/2} (eigenvalues below 1e-8 dropped)  (WaveFunction.f90:394-467)
  P_i from the core-Hamiltonian guess
  every iteration, for every species i:
    G_i = q_i^2 (J[P_i] + kappa_i/eta_i K[P_i])  when the species has > 1 particle
                                                     (WaveFunction.f90:817-1159)
    J_i = sum_{j != i} q_i q_j J_i[P_j]              (WaveFunction.f90:1432-1505)
    F_i = H_i + G_i + J_i                            (WaveFunction.f90:1768-1826)
  E = E_nuc + sum_i tr P_i (H_i + G_i / 2) + sum_{i<j} tr P_i J_ij
  Gaussian-fit potentials (HostSCF): an external potential of species i is
  added to H_i (DirectIntegralManager.f90:848-949); with interpotentials
  every G_i and J_ij is a G12 matrix of the pair's potential instead of
  Coulomb, without charge factors, and pairs without one do not interact
  (WaveFunction.f90:1097-1135, 1439-1477)
  Pulay DIIS over all species (one coefficient set), F' = X^T F X, C = X C',
  P_i = eta_i C_occ C_occ^T; converged when |dE| < tol and rms(dP) < tol_p.

HostSCF keeps matrices in host memory and calls the reference-shaped C ABI
(LibintInterface_compute_2body_direct / _compute_coupling_direct) with host
buffers each iteration, the way the Fortran program does.  DeviceSCF keeps every
matrix in HBM (torch FP64 tensors), calls the device entry points, fuses both
coupling directions into one pass per species pair, and synchronises once per
iteration for the convergence test.
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field

import numpy as np

from . import lint


def nuclear_repulsion(sysd) -> float:
    Z = np.asarray(sysd["point_charges"], float)
    R = np.asarray(sysd["point_positions"], float).reshape(-1, 3)
    e = 0.0
    for a in range(len(Z)):
        for b in range(a):
            e += Z[a] * Z[b] / float(np.linalg.norm(R[a] - R[b]))
    return e


def n_occ(sp) -> int:
    return int(round(sp["n_particles"] * sp["particles_fraction"]))


@dataclass
class SCFResult:
    energy: float
    iterations: int
    converged: bool
    seconds: float
    orbital_energies: list = field(default_factory=list)
    coefficients: list = field(default_factory=list)
    densities: list = field(default_factory=list)
    quartets: int = 0
    # mixed precision: |E_mixed - E_FP64| of the FP64 check at the converged
    # density, and whether the check sent the system on in FP64
    err_vs_fp64: float | None = None
    guard_hit: bool = False


def _one_body(handles, sysd):
    H, S = [], []
    for h, sp in zip(handles, sysd["species"]):
        Sm = h.one_body(1)
        T = h.one_body(2)
        V = h.potential(sysd["point_charges"], sysd["point_positions"])
        H.append(T / sp["mass"] + sp["charge"] * V)
        S.append(Sm)
    return H, S


def _one_body_device(handles, sysd, device, stream):
    """H = T / mass + q V and S of every species, computed on the device."""
    import torch
    H, S = [], []
    for h, sp in zip(handles, sysd["species"]):
        n = h.nbasis
        Sm = torch.empty((n, n), dtype=torch.float64, device=device)
        T = torch.empty_like(Sm)
        V = torch.empty_like(Sm)
        h.one_body_device(sysd["point_charges"], sysd["point_positions"], Sm.data_ptr(), T.data_ptr(),
                          V.data_ptr(), stream)
        H.append(T / sp["mass"] + sp["charge"] * V)
        S.append(Sm)
    return H, S


def interpotentials(sysd) -> dict:
    """{(i, j), i <= j: (coefficients, exponents)} of sysd["interpotentials"],
    a list of {"species": [i, j], "coefficients": [...], "exponents": [...]}."""
    out = {}
    for e in sysd.get("interpotentials", []):
        i, j = sorted(int(x) for x in e["species"])
        if len(e["coefficients"]) != len(e["exponents"]):
            raise ValueError(f"interpotential {i},{j}: coefficients and exponents differ in length")
        out[(i, j)] = (list(e["coefficients"]), list(e["exponents"]))
    return out


DOUBLE_ZERO = 1e-12


def damped_fock(F, P, kept):
    """The reference's default convergence method (CONVERGENCE_METHOD 1,
    src/scf/Convergence.f90:444-511) for one species: the kept pair
    (F0, P0) starts as the first Fock matrix and density; with
    dE = -tr(F0 (P - P0)) / 2 and dEF = tr((F - F0)(P - P0)), the step is
    undamped (the pair becomes (F, P)) when dEF <= dE or |dEF| < 1e-12,
    otherwise F0 and P0 move by dE / dEF towards F and P and F0 is the matrix
    diagonalised.  Returns (matrix to diagonalise, new kept pair)."""
    F0, P0 = kept
    dP = P - P0
    dE = -0.5 * float(np.vdot(F0, dP.T))
    dEF = float(np.vdot(F - F0, dP.T))
    if dEF <= dE or abs(dEF) < DOUBLE_ZERO:
        return F, (F.copy(), P.copy())
    w = dE / dEF
    F0 = F0 + w * (F - F0)
    return F0, (F0, P0 + w * (P - P0))


def coulomb_only(sysd, who: str) -> None:
    """Raise unless the system has only Coulomb interactions: drivers that keep
    no Gaussian-fit potential path must not drop one silently."""
    if sysd.get("interpotentials") or sysd.get("external_potentials"):
        raise ValueError(f"{who}: Gaussian-fit potentials (interpotentials / external_potentials) "
                         "are supported by HostSCF only")


def _orthogonaliser(S, cut=1e-8, host_max=384):
    """S^-1/2 (symmetric, or canonical when eigenvalues fall below cut) of a
    device matrix: host LAPACK below host_max functions, the GPU solver above."""
    import torch
    if S.shape[0] < host_max:
        return torch.from_numpy(_orthogonaliser_np(S.cpu().numpy(), cut)).to(S.device)
    w, U = torch.linalg.eigh(S)
    keep = w > cut
    if bool(keep.all()):
        return (U * w.rsqrt()) @ U.T
    return U[:, keep] / torch.sqrt(w[keep])


def occupied_subspace(Fp, occ, passes=2):
    """Orthonormal basis of the occupied subspace (the occ lowest eigenvectors)
    of a symmetric FP64 matrix Fp, from an FP32 eigensolve refined in FP64:
    each pass re-orthonormalises the occupied and virtual blocks (Cholesky of
    their overlaps), forms A_ov = C_o^T Fp C_v and the diagonals of the two
    blocks in FP64, and rotates by the first-order occupied-virtual mixing
    X_ia = A_ia / (d_a - d_i) (Rayleigh-Ritz / Jacobi correction of an
    invariant subspace).  The error of the subspace falls quadratically: two
    passes from FP32 vectors reach the FP64 eigensolver's occupied projector
    to ~1e-14 for Fock matrices whose occupied-virtual gap is > ~1e-3 of
    their spectral range.  Degeneracies inside the occupied or the virtual
    block need no resolution (the projector does not depend on them).
    Returns C_o (n x occ, FP64)."""
    import torch
    _, V32 = torch.linalg.eigh(Fp.to(torch.float32))
    V = V32.to(torch.float64)
    Vo, Vv = V[:, :occ], V[:, occ:]
    for _ in range(passes):
        Lo = torch.linalg.cholesky(Vo.T @ Vo)
        Vo = torch.linalg.solve_triangular(Lo, Vo.T, upper=False).T
        Vv = Vv - Vo @ (Vo.T @ Vv)
        Lv = torch.linalg.cholesky(Vv.T @ Vv)
        Vv = torch.linalg.solve_triangular(Lv, Vv.T, upper=False).T
        FVo, FVv = Fp @ Vo, Fp @ Vv
        do = torch.sum(Vo * FVo, dim=0)
        dv = torch.sum(Vv * FVv, dim=0)
        Xm = (Vo.T @ FVv) / (dv[None, :] - do[:, None])
        Vo, Vv = Vo - Vv @ Xm.T, Vv + Vo @ Xm
    Lo = torch.linalg.cholesky(Vo.T @ Vo)
    return torch.linalg.solve_triangular(Lo, Vo.T, upper=False).T


def _orthogonaliser_np(S, cut=1e-8):
    w, U = np.linalg.eigh(S)
    keep = w > cut
    if keep.all():
        return (U * w ** -0.5) @ U.T
    return U[:, keep] / np.sqrt(w[keep])


class _DIIS:
    def __init__(self, xp, size=10):
        self.xp, self.size = xp, size
        self.F, self.E = [], []

    def __call__(self, Fs, errs):
        xp = self.xp
        self.F.append([f.clone() if hasattr(f, "clone") else f.copy() for f in Fs])
        self.E.append(errs)
        if len(self.F) > self.size:
            self.F.pop(0)
            self.E.pop(0)
        m = len(self.F)
        if m < 2:
            return Fs
        B = np.zeros((m + 1, m + 1))
        B[m, :] = B[:, m] = -1.0
        B[m, m] = 0.0
        if xp is np:
            for i in range(m):
                for j in range(i + 1):
                    B[i, j] = B[j, i] = sum(float(np.vdot(a, b)) for a, b in zip(self.E[i], self.E[j]))
        else:
            flat = xp.stack([xp.cat([e.reshape(-1) for e in E]) for E in self.E])
            G = (flat @ flat.T).cpu().numpy()
            B[:m, :m] = G
        rhs = np.zeros(m + 1)
        rhs[m] = -1.0
        c = np.linalg.lstsq(B, rhs, rcond=1e-14)[0]
        return [sum(float(c[i]) * self.F[i][k] for i in range(m)) for k in range(len(Fs))]


class HostSCF:
    """SCF whose integral work goes through the host-buffer C ABI each
    iteration (the reference program's calling pattern).

    precision "mixed": the handles' compute_2body_direct runs the FP32/FP64
    split (LowdinGB300_set_precision) and the caller passes density changes:
    a full build on the first iteration, then G += G[P - P_ref]; when the
    energy and density converge, one full FP64 build at the converged density
    gives the result's energy and its stated error |E_mixed - E_FP64|; above
    guard_energy, or with an FP64 commutator element above guard_commutator,
    the solve continues in FP64 with a fresh DIIS history.  Couplings stay
    FP64 full builds.

    convergence: "diis" (Pulay over all species, the reference's method 2) or
    "damping" (its default method 1, damped_fock); damping is slower but
    follows the reference to its stationary point where DIIS can jump to
    another one (species of several protons, for instance).

    Gaussian-fit potentials: sysd["external_potentials"], a list of
    {"species": i, "coefficients", "exponents", "origins"}, are added to H_i
    (LowdinGB300_gaussian_potential); sysd["interpotentials"] switches every
    species pair to G12 matrices (libintinterface_compute_g12_direct /
    _g12inter_direct, FP64 full builds)."""

    def __init__(self, sysd, precision="fp64", split=1e-5, guard_energy=1e-6, guard_commutator=1e-4,
                 convergence="diis"):
        if precision not in ("fp64", "mixed"):
            raise ValueError(f"precision must be 'fp64' or 'mixed', not {precision!r}")
        if convergence not in ("diis", "damping"):
            raise ValueError(f"convergence must be 'diis' or 'damping', not {convergence!r}")
        self.convergence = convergence
        self.sysd = sysd
        self.species = sysd["species"]
        self.precision, self.split = precision, split
        self.guard_energy, self.guard_commutator = guard_energy, guard_commutator
        self.handles = [lint.Libint2Interface(sp, i + 1) for i, sp in enumerate(self.species)]
        for h in self.handles:
            h.init_2body_ints()
        self.H, self.S = _one_body(self.handles, sysd)
        for e in sysd.get("external_potentials", []):
            i = int(e["species"])
            self.H[i] = self.H[i] + self.handles[i].gaussian_potential(e["coefficients"], e["exponents"],
                                                                       e["origins"])
        self.g12 = interpotentials(sysd)
        if self.g12 and precision != "fp64":
            raise ValueError("mixed precision applies to Coulomb builds; G12 systems run in FP64")
        self.X = [_orthogonaliser_np(S) for S in self.S]
        self.enuc = nuclear_repulsion(sysd)

    def close(self):
        for h in self.handles:
            h.close()

    def _set_split(self, on: bool):
        for h in self.handles:
            h.set_precision(1 if on else 0, self.split)

    def _full_G(self, i, Pi):
        """FP64 two-particle (or G12) matrix of species i from density Pi."""
        sp = self.species[i]
        if sp["n_particles"] <= 1:
            return np.zeros_like(self.H[i])
        f = sp["kappa"] / sp["eta"]
        if self.g12:
            pot = self.g12.get((i, i))
            return self.handles[i].compute_g12_direct(Pi, f, *pot) if pot else np.zeros_like(self.H[i])
        return self.handles[i].compute_2body_direct(Pi, f) * sp["charge"] ** 2

    def solve(self, tol_energy=1e-8, tol_density=1e-6, max_iter=100, density_sum=False, scheme=3,
              sub_max=(50, 50), sub_tolerances=(1e-8, 1e-6)) -> SCFResult:
        """Converged when |dE| < tol_energy and the density change is below
        tol_density (either alone with the other tolerance set to inf): the
        largest rms change over the species, or with density_sum their sum,
        the reference's measure (MultiSCF.f90:350-425, 776-830).

        scheme: the reference's iteration scheme (MultiSCF.f90:150-185): 3 =
        every species once per global iteration; 0 / 1 / 2 = the
        non-electronic species / the electrons / every species iterate on
        their own inside a global iteration, up to sub_max = (electronic,
        non-electronic) times, while their energy tr P (H + G/2 + J) changes
        by more than sub_tolerances[0] or their density by more than
        sub_tolerances[1]; each such step rebuilds the species' two-particle
        matrix, the couplings stay those of the global build.  The
        reference's criteria set the unused quantity's tolerances to 1.0
        (CONTROL.f90:3174-3190): ENERGY gives (1e-8, 1.0), DENSITY (1.0,
        1e-6), BOTH (1e-8, 1e-6).  Schemes 0-2 need convergence "damping"
        and FP64."""
        if scheme not in (0, 1, 2, 3):
            raise ValueError(f"iteration scheme must be 0-3, not {scheme!r}")
        if scheme != 3 and (self.convergence != "damping" or self.precision != "fp64"):
            raise ValueError("iteration schemes 0-2 run with convergence 'damping' in FP64")
        t0 = time.perf_counter()
        sp, H, S, X = self.species, self.H, self.S, self.X
        ns = len(sp)
        sub = []
        for s_ in sp:
            el = s_["is_electron"]
            sub.append({0: 1 if el else sub_max[1], 1: sub_max[0] if el else 1,
                        2: sub_max[0] if el else sub_max[1], 3: 1}[scheme])
        mixed = self.precision == "mixed"
        fp64 = not mixed          # builds in FP64 (plain, the FP64 check, after a failed check)
        checking = False          # this iteration's build is the FP64 check
        e_mixed, err_vs_fp64, guard_hit = None, None, False
        self._set_split(mixed)
        P, C, eps = [], [], []
        for i in range(ns):
            e, Cp = np.linalg.eigh(X[i].T @ H[i] @ X[i])
            Ci = X[i] @ Cp
            C.append(Ci); eps.append(e)
            o = n_occ(sp[i])
            P.append(sp[i]["eta"] * Ci[:, :o] @ Ci[:, :o].T)
        Pref, Gprev = [None] * ns, [None] * ns
        diis = _DIIS(np)
        kept = None
        e_old, converged, it, quartets = None, False, 0, 0
        energy = 0.0
        for it in range(1, max_iter + 1):
            full = fp64 or it == 1
            G, J = [], [[None] * ns for _ in range(ns)]
            for i in range(ns):
                if self.g12:
                    pot = self.g12.get((i, i))
                    if sp[i]["n_particles"] > 1 and pot:
                        G.append(self.handles[i].compute_g12_direct(P[i], sp[i]["kappa"] / sp[i]["eta"], *pot))
                    else:
                        G.append(np.zeros_like(H[i]))
                    for j in range(ns):
                        pot = self.g12.get((min(i, j), max(i, j)))
                        if j == i:
                            continue
                        if pot:
                            B = self.handles[i].compute_g12inter_direct(self.handles[j], P[j], *pot)
                            J[i][j] = np.tril(B) + np.tril(B, -1).T
                        else:
                            J[i][j] = np.zeros_like(H[i])
                    continue
                if sp[i]["n_particles"] > 1:
                    f = sp[i]["kappa"] / sp[i]["eta"]
                    q2 = sp[i]["charge"] ** 2
                    if full:
                        G.append(self.handles[i].compute_2body_direct(P[i], f) * q2)
                    else:
                        G.append(Gprev[i] + self.handles[i].compute_2body_direct(P[i] - Pref[i], f) * q2)
                    quartets += max(0, self.handles[i].last_quartets())
                else:
                    G.append(np.zeros_like(H[i]))
                for j in range(ns):
                    if j == i:
                        continue
                    B = self.handles[i].compute_coupling_direct(self.handles[j], P[j])
                    B = (np.tril(B) + np.tril(B, -1).T) * sp[i]["charge"] * sp[j]["charge"]
                    J[i][j] = B
            Pref, Gprev = [p.copy() for p in P], G
            F = [H[i] + G[i] + sum(J[i][j] for j in range(ns) if j != i) for i in range(ns)]
            energy = self.enuc
            for i in range(ns):
                energy += float(np.sum(P[i] * (H[i] + 0.5 * G[i])))
                for j in range(i + 1, ns):
                    energy += float(np.sum(P[i] * J[i][j]))
            errs = [X[i].T @ (F[i] @ P[i] @ S[i] - S[i] @ P[i] @ F[i]) @ X[i] for i in range(ns)]
            if checking:
                checking = False
                err_vs_fp64 = abs(e_mixed - energy)
                comm = max(float(np.max(np.abs(e))) for e in errs)
                if err_vs_fp64 <= self.guard_energy and comm <= self.guard_commutator:
                    # the FP64 energy is the result; orbitals of the FP64 Fock matrix
                    for i in range(ns):
                        e, Cp = np.linalg.eigh(X[i].T @ F[i] @ X[i])
                        C[i], eps[i] = X[i] @ Cp, e
                    converged = True
                    break
                guard_hit = True                  # continue in FP64 from this Fock build
                diis, e_old, kept = _DIIS(np), None, None
            def density(i, Fi):
                e, Cp = np.linalg.eigh(X[i].T @ Fi @ X[i])
                Ci = X[i] @ Cp
                C[i], eps[i] = Ci, e
                o = n_occ(sp[i])
                return sp[i]["eta"] * Ci[:, :o] @ Ci[:, :o].T

            if self.convergence == "damping" and kept is None:
                kept = [(F[i].copy(), P[i].copy()) for i in range(ns)]
            dmax = 0.0
            newP = []
            if max(sub) > 1:
                # nested scheme: each species in turn, on its own
                for i in range(ns):
                    Ji = sum(J[i][j] for j in range(ns) if j != i)
                    Fi, Gi, Pi = F[i], G[i], P[i]
                    e_i = float(np.sum(Pi * (H[i] + 0.5 * Gi + Ji)))
                    d_e, rms, k = 1e16, math.inf, 0
                    while (abs(d_e) > sub_tolerances[0] or rms > sub_tolerances[1]) and k < sub[i]:
                        k += 1
                        Fd, kept[i] = damped_fock(Fi, Pi, kept[i])
                        Pn = density(i, Fd)
                        rms = float(np.sqrt(np.mean((Pn - Pi) ** 2)))
                        Pi = Pn
                        e_new = float(np.sum(Pi * (H[i] + 0.5 * Gi + Ji)))
                        if sub[i] > 1:
                            Gi = self._full_G(i, Pi)
                            Fi = H[i] + Gi + Ji
                            d_e, e_i = e_i - e_new, e_new
                    newP.append(Pi)
                    dmax = dmax + rms if density_sum else max(dmax, rms)
            else:
                if self.convergence == "diis":
                    Fx = diis(F, errs)
                else:
                    Fx = []
                    for i in range(ns):
                        Fd, kept[i] = damped_fock(F[i], P[i], kept[i])
                        Fx.append(Fd)
                for i in range(ns):
                    Pn = density(i, Fx[i])
                    rms = float(np.sqrt(np.mean((Pn - P[i]) ** 2)))
                    dmax = dmax + rms if density_sum else max(dmax, rms)
                    newP.append(Pn)
            if e_old is not None and abs(energy - e_old) < tol_energy and dmax < tol_density:
                if not fp64:
                    # FP64 check: a full FP64 build at this iteration's density
                    fp64, checking, e_mixed = True, True, energy
                    self._set_split(False)
                    continue
                converged = True
                break
            e_old = energy
            P = newP
        self._set_split(False)
        return SCFResult(energy, it, converged, time.perf_counter() - t0, eps, C, P, quartets,
                         err_vs_fp64=err_vs_fp64, guard_hit=guard_hit)


class DeviceSCF:
    """SCF of one system with every matrix resident in HBM: a one-system
    BatchSCF (the library's batched build and batched tensor algebra)."""

    def __init__(self, sysd, device="cuda", precision="fp64", split=1e-5):
        from .batch_scf import BatchSCF
        self.sysd = sysd
        self.inner = BatchSCF([sysd], device=device, precision=precision, split=split)
        self.handles = self.inner.handles[0]

    def close(self):
        self.inner.close()

    def solve(self, tol_energy=1e-8, tol_density=1e-6, max_iter=100) -> SCFResult:
        return self.inner.solve(tol_energy, tol_density, max_iter)[0]
