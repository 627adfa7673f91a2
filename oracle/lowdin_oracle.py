"""CPU FP64 oracle for the openLOWDIN direct-SCF / MP2 hot path.

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()`` and
by the CPU-baseline leg of ``bench.py``; the product package never imports it.

The integral work is done by ``liboracle.so`` (``oracle.c``, a C restatement of
``src/ints/Libint2Iface.cpp``'s direct loops).  This module adds the caller side
restated from the Fortran program:

* Hcore: kinetic / mass + charge x point-charge potential
  (``src/scf/WaveFunction.f90:471-570``),
* symmetric orthogonalisation S^-1/2 with the 1e-8 eigenvalue cut
  (``WaveFunction.f90:394-467``), HCORE guess
  (``src/scf/DensityMatrixSCFGuess.f90:183-215``),
* two-particle matrix x q^2 and only for species with more than one particle
  (``WaveFunction.f90:817-1159``), coupling x q_i q_j symmetrised from the upper
  triangle (``WaveFunction.f90:1432-1505``), F = H + G + sum_j J_ij
  (``WaveFunction.f90:1768-1826``), P = eta C_occ C_occ^T (``:1830-1878``),
* total energy E_nuc + sum_i tr P_i (H_i + G_i/2) + sum_{i<j} tr P_i J_ij
  (``WaveFunction.f90:1882-2003``),
* iteration scheme 3 -- every species once per global iteration
  (``src/scf/MultiSCF.f90:276-440``) with Pulay DIIS (``src/scf/Convergence.f90``),
* closed-shell MP2 from (ia|jb) (``src/MBPT/MPFunctions.f90:514-662``).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
_RYS = None

_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")


def reference_available() -> bool:
    """Whether the openLOWDIN source tree the Makefile points at (environment
    variable LOWDIN_REFERENCE, else the Makefile's default) is present."""
    return subprocess.run(["make", "-s", "-C", _HERE, "have-reference"], capture_output=True).returncode == 0


def build(ref: bool = False) -> None:
    """Compile liboracle.so (and the reference's Rys code when ``ref``)."""
    subprocess.check_call(["make", "-s", "-C", _HERE, "liboracle.so"])
    if ref:
        subprocess.check_call(["make", "-s", "-C", _HERE, "ref"])


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        B = [ctypes.c_int, _i32p, _i32p, _f64p, _f64p, _f64p]
        L.or_nbasis.argtypes = B
        L.or_nbasis.restype = ctypes.c_int
        L.or_norma.argtypes = B + [_f64p]
        L.or_eri_quartet.argtypes = B + [ctypes.c_int] * 4 + [_f64p]
        L.or_eri_primitive.argtypes = [_i32p, _f64p, _f64p, _f64p]
        L.or_pair_mask.argtypes = B + [_u8p]
        L.or_schwarz.argtypes = B + [_f64p, ctypes.c_int]
        L.or_2body_direct.argtypes = B + [ctypes.c_int, _f64p, ctypes.c_double, _f64p, ctypes.c_int]
        L.or_coupling_direct.argtypes = B + [ctypes.c_int] + B + [ctypes.c_int, _f64p, _f64p, ctypes.c_int]
        L.or_2body_directIT.argtypes = B + [ctypes.c_int, _f64p, _f64p, ctypes.c_int, _f64p]
        L.or_coupling_directIT.argtypes = B + [ctypes.c_int] + B + [ctypes.c_int, _f64p, ctypes.c_int, _f64p]
        L.or_overlap_kinetic.argtypes = B + [_f64p, _f64p]
        L.or_potential.argtypes = B + [ctypes.c_int, _f64p, _f64p, _f64p]
        L.or_eri_full.argtypes = B + [_f64p, ctypes.c_int]
        L.or_boys.argtypes = [ctypes.c_int, ctypes.c_double, _f64p]
        G = [ctypes.c_int, _f64p, _f64p]   # geminal: count, coefficients, exponents
        L.or_g12_direct.argtypes = B + [_f64p, ctypes.c_double] + G + [_f64p, ctypes.c_int]
        L.or_g12inter_direct.argtypes = B + [ctypes.c_int] + B + [ctypes.c_int, _f64p] + G + [_f64p, ctypes.c_int]
        L.or_g12_primitive.argtypes = [_i32p, _f64p, _f64p] + G + [_f64p]
        L.or_last_quartet_count.restype = ctypes.c_longlong
        _LIB = L
    return _LIB


def rys_lib():
    """The reference's own src/ints/RysQInts.cpp, built into _ref/ (or None)."""
    global _RYS
    if _RYS is None:
        path = os.path.join(_HERE, "_ref", "librys.so")
        if not os.path.exists(path):
            return None
        _RYS = ctypes.CDLL(path)
    return _RYS


def nthreads_default() -> int:
    return max(1, len(os.sched_getaffinity(0)))


# --------------------------------------------------------------------- basis --
@dataclass
class Basis:
    """Shells of one species in insertion order (the reference's `shells`)."""

    l: np.ndarray        # int32 [nsh]
    nprim: np.ndarray    # int32 [nsh]
    origin: np.ndarray   # f64 [nsh*3]
    alpha: np.ndarray    # f64 [sum nprim]
    coef: np.ndarray     # f64 [sum nprim] raw file coefficients

    @staticmethod
    def from_shells(shells):
        """shells: iterable of (l, alphas, coefs, origin3)."""
        ls, nps, org, al, co = [], [], [], [], []
        for l, a, c, o in shells:
            ls.append(int(l)); nps.append(len(a)); org.extend(o); al.extend(a); co.extend(c)
        return Basis(np.array(ls, np.int32), np.array(nps, np.int32), np.array(org, np.float64),
                     np.array(al, np.float64), np.array(co, np.float64))

    def args(self):
        return (len(self.l), self.l, self.nprim, self.origin, self.alpha, self.coef)

    @property
    def nshell(self):
        return len(self.l)

    @property
    def nbf(self):
        return int(sum((l + 1) * (l + 2) // 2 for l in self.l))


def norma(b: Basis) -> np.ndarray:
    out = np.zeros(b.nbf)
    lib().or_norma(*b.args(), out)
    return out


def eri_quartet(b: Basis, s1, s2, s3, s4) -> np.ndarray:
    n = [(int(b.l[s]) + 1) * (int(b.l[s]) + 2) // 2 for s in (s1, s2, s3, s4)]
    out = np.zeros(int(np.prod(n)))
    lib().or_eri_quartet(*b.args(), s1, s2, s3, s4, out)
    return out.reshape(n)


def eri_full(b: Basis, nthreads=None) -> np.ndarray:
    n = b.nbf
    out = np.zeros(n ** 4)
    lib().or_eri_full(*b.args(), out, nthreads or nthreads_default())
    return out.reshape(n, n, n, n)


def schwarz(b: Basis, nthreads=None) -> np.ndarray:
    Q = np.zeros(b.nshell * b.nshell)
    lib().or_schwarz(*b.args(), Q, nthreads or nthreads_default())
    return Q.reshape(b.nshell, b.nshell)


def pair_mask(b: Basis) -> np.ndarray:
    m = np.zeros(b.nshell * b.nshell, np.uint8)
    lib().or_pair_mask(*b.args(), m)
    return m.reshape(b.nshell, b.nshell)


def two_body_direct(b: Basis, is_electron: bool, D: np.ndarray, factor: float, nthreads=None):
    """LibintInterface_compute_2body_direct (row-major D -> G)."""
    n = b.nbf
    G = np.zeros(n * n)
    lib().or_2body_direct(*b.args(), int(is_electron), np.ascontiguousarray(D, np.float64).ravel(),
                          float(factor), G, nthreads or nthreads_default())
    return G.reshape(n, n)


def last_quartet_count() -> int:
    return int(lib().or_last_quartet_count())


def coupling_direct(b: Basis, sid: int, ob: Basis, osid: int, Dother: np.ndarray, nthreads=None):
    """LibintInterface_compute_coupling_direct(lint=b, olint=ob, D_other)."""
    n = b.nbf
    B = np.zeros(n * n)
    lib().or_coupling_direct(*b.args(), sid, *ob.args(), osid,
                             np.ascontiguousarray(Dother, np.float64).ravel(), B,
                             nthreads or nthreads_default())
    return B.reshape(n, n)


def alphabeta_direct(b: Basis, sid: int, ob: Basis, osid: int, D, Dother) -> float:
    """LibintInterface_compute_alphabeta_direct (src/ints/Libint2Iface.cpp:1626-1825,
    wrapper :3625-3658): sum_{ij kl} D(ij) (ij|kl) D_other(kl) over the
    coupling integral set, i.e. D contracted with the full symmetric J[D_other]
    of coupling_direct."""
    B = coupling_direct(b, sid, ob, osid, Dother)
    J = np.tril(B) + np.tril(B, -1).T
    return float(np.sum(np.asarray(D, np.float64) * J))


def _geminal(coefficients, exponents):
    c = np.ascontiguousarray(coefficients, np.float64).ravel()
    g = np.ascontiguousarray(exponents, np.float64).ravel()
    if c.shape != g.shape:
        raise ValueError("geminal coefficients and exponents differ in length")
    return len(c), c, g


def g12_direct(b: Basis, D: np.ndarray, factor: float, coefficients, exponents, nthreads=None):
    """libintinterface_compute_g12_direct (row-major D -> G) for the operator
    sum_k c_k exp(-g_k r12^2)."""
    n = b.nbf
    G = np.zeros(n * n)
    lib().or_g12_direct(*b.args(), np.ascontiguousarray(D, np.float64).ravel(), float(factor),
                        *_geminal(coefficients, exponents), G, nthreads or nthreads_default())
    return G.reshape(n, n)


def g12inter_direct(b: Basis, sid: int, ob: Basis, osid: int, Dother: np.ndarray, coefficients, exponents,
                    nthreads=None):
    """libintinterface_compute_g12inter_direct(lint=b, olint=ob, D_other)."""
    n = b.nbf
    B = np.zeros(n * n)
    lib().or_g12inter_direct(*b.args(), sid, *ob.args(), osid, np.ascontiguousarray(Dother, np.float64).ravel(),
                             *_geminal(coefficients, exponents), B, nthreads or nthreads_default())
    return B.reshape(n, n)


def g12_primitive(l4, alpha4, origins, coefficients, exponents) -> np.ndarray:
    """Unnormalised primitive geminal integrals (la lb|g|lc ld), row-major."""
    from math import prod
    l4 = np.ascontiguousarray(l4, np.int32)
    out = np.zeros(prod((l + 1) * (l + 2) // 2 for l in l4))
    lib().or_g12_primitive(l4, np.ascontiguousarray(alpha4, np.float64),
                           np.ascontiguousarray(origins, np.float64).ravel(), *_geminal(coefficients, exponents), out)
    return out


def two_body_directIT(b: Basis, is_electron: bool, D, C, p: int):
    n = b.nbf
    A = np.zeros(n ** 3)
    lib().or_2body_directIT(*b.args(), int(is_electron), np.ascontiguousarray(D, np.float64).ravel(),
                            np.ascontiguousarray(C, np.float64).ravel(), int(p), A)
    return A.reshape(n, n, n)


def coupling_directIT(b: Basis, sid: int, ob: Basis, osid: int, C, p: int):
    n, on = b.nbf, ob.nbf
    A = np.zeros(n * on * on)
    lib().or_coupling_directIT(*b.args(), sid, *ob.args(), osid,
                               np.ascontiguousarray(C, np.float64).ravel(), int(p), A)
    return A.reshape(n, on, on)


def overlap_kinetic(b: Basis):
    n = b.nbf
    S = np.zeros(n * n)
    T = np.zeros(n * n)
    lib().or_overlap_kinetic(*b.args(), S, T)
    return S.reshape(n, n), T.reshape(n, n)


def potential(b: Basis, charges, positions):
    n = b.nbf
    V = np.zeros(n * n)
    Z = np.ascontiguousarray(charges, np.float64)
    R = np.ascontiguousarray(positions, np.float64).ravel()
    lib().or_potential(*b.args(), len(Z), Z, R, V)
    return V.reshape(n, n)


def boys(mmax: int, T: float) -> np.ndarray:
    F = np.zeros(mmax + 1)
    lib().or_boys(mmax, T, F)
    return F


# ------------------------------------------------------------------- system --
@dataclass
class Species:
    """One quantum species (src/core/Species.f90:81-165)."""

    name: str
    basis: Basis
    charge: float
    mass: float
    n_particles: int
    kappa: float = -1.0
    eta: float = 2.0
    particles_fraction: float = 0.5
    is_electron: bool = True

    @property
    def n_occ(self) -> int:
        return int(round(self.n_particles * self.particles_fraction))

    @property
    def exchange_factor(self) -> float:
        """kappa / eta (src/core/MolecularSystem.f90:1398-1413)."""
        return self.kappa / self.eta


@dataclass
class System:
    species: list
    point_charges: np.ndarray = field(default_factory=lambda: np.zeros(0))
    point_positions: np.ndarray = field(default_factory=lambda: np.zeros((0, 3)))

    def nuclear_repulsion(self) -> float:
        Z, R = self.point_charges, self.point_positions
        e = 0.0
        for a in range(len(Z)):
            for b in range(a):
                e += Z[a] * Z[b] / np.linalg.norm(R[a] - R[b])
        return e


def from_plain(desc) -> System:
    """System from the plain-data description used by the product's generators."""
    sp = []
    for s in desc["species"]:
        sp.append(Species(s["name"], Basis.from_shells(s["shells"]), s["charge"], s["mass"],
                          s["n_particles"], s["kappa"], s["eta"], s["particles_fraction"],
                          s["is_electron"]))
    return System(sp, np.array(desc["point_charges"], float),
                  np.array(desc["point_positions"], float).reshape(-1, 3))


# ---------------------------------------------------------------------- SCF --
@dataclass
class SCFResult:
    energy: float
    iterations: int
    converged: bool
    densities: list
    coefficients: list
    orbital_energies: list
    fock: list
    hcore: list
    two_particle: list
    coupling: list


def _orthogonaliser(S, cut=1e-8):
    w, U = np.linalg.eigh(S)
    keep = w > cut
    return U[:, keep] @ np.diag(w[keep] ** -0.5) @ U[:, keep].T if keep.all() else U[:, keep] / np.sqrt(w[keep])


class DIIS:
    """Pulay extrapolation shared by all species: one set of coefficients from
    the concatenated commutator errors X^T(FPS - SPF)X of every species."""

    def __init__(self, size=10):
        self.size = size
        self.F, self.E = [], []

    def __call__(self, Fs, errs):
        self.F.append([f.copy() for f in Fs]); self.E.append([e.copy() for e in errs])
        if len(self.F) > self.size:
            self.F.pop(0); self.E.pop(0)
        m = len(self.F)
        if m < 2:
            return Fs
        B = -np.ones((m + 1, m + 1))
        B[m, m] = 0
        for i in range(m):
            for j in range(m):
                B[i, j] = sum(np.vdot(a, b) for a, b in zip(self.E[i], self.E[j]))
        rhs = np.zeros(m + 1)
        rhs[m] = -1
        c = np.linalg.lstsq(B, rhs, rcond=1e-14)[0]
        return [sum(c[i] * self.F[i][k] for i in range(m)) for k in range(len(Fs))]


def scf(system: System, tol_energy=1e-10, tol_density=1e-8, max_iter=200, nthreads=None,
        diis=True, verbose=False) -> SCFResult:
    """Multi-species Hartree-Fock, iteration scheme 3, restated from src/scf."""
    sp = system.species
    ns = len(sp)
    H, X, S = [], [], []
    for s in sp:
        Sm, T = overlap_kinetic(s.basis)
        V = potential(s.basis, system.point_charges, system.point_positions)
        # T / mass + (q) * V  -- puntual interaction scaled by the particle charge
        H.append(T / s.mass + s.charge * V)
        S.append(Sm)
        X.append(_orthogonaliser(Sm))
    # HCORE guess
    P, C, eps = [], [], []
    for i, s in enumerate(sp):
        Fp = X[i].T @ H[i] @ X[i]
        e, Cp = np.linalg.eigh(Fp)
        Ci = X[i] @ Cp
        C.append(Ci); eps.append(e)
        P.append(s.eta * Ci[:, :s.n_occ] @ Ci[:, :s.n_occ].T)
    enuc = system.nuclear_repulsion()
    diis_obj = DIIS()
    e_old = None
    converged = False
    it = 0
    for it in range(1, max_iter + 1):
        G, J = [], []
        for i, s in enumerate(sp):
            if s.n_particles > 1:
                G.append(two_body_direct(s.basis, s.is_electron, P[i], s.exchange_factor, nthreads) * s.charge ** 2)
            else:
                G.append(np.zeros_like(H[i]))
            Ji = np.zeros_like(H[i])
            Jparts = {}
            for j, o in enumerate(sp):
                if j == i:
                    continue
                B = coupling_direct(s.basis, i + 1, o.basis, j + 1, P[j], nthreads) * s.charge * o.charge
                B = np.tril(B) + np.tril(B, -1).T  # row-major lower == Fortran upper
                Jparts[j] = B
                Ji += B
            J.append((Ji, Jparts))
        F = [H[i] + G[i] + J[i][0] for i in range(ns)]
        energy = enuc
        for i in range(ns):
            energy += np.sum(P[i] * (H[i] + 0.5 * G[i]))
            for j, B in J[i][1].items():
                if j > i:
                    energy += np.sum(P[i] * B)
        newP = []
        dmax = 0.0
        Fx = F
        if diis:
            errs = [X[i].T @ (F[i] @ P[i] @ S[i] - S[i] @ P[i] @ F[i]) @ X[i] for i in range(ns)]
            Fx = diis_obj(F, errs)
        for i, s in enumerate(sp):
            Fi = Fx[i]
            e, Cp = np.linalg.eigh(X[i].T @ Fi @ X[i])
            Ci = X[i] @ Cp
            C[i] = Ci; eps[i] = e
            Pn = s.eta * Ci[:, :s.n_occ] @ Ci[:, :s.n_occ].T
            dmax = max(dmax, float(np.sqrt(np.mean((Pn - P[i]) ** 2))))
            newP.append(Pn)
        if verbose:
            print(f"iter {it:3d}  E = {energy:.12f}  dP = {dmax:.2e}")
        if e_old is not None and abs(energy - e_old) < tol_energy and dmax < tol_density:
            converged = True
            break
        e_old = energy
        P = newP
    return SCFResult(energy, it, converged, P, C, eps, F, H, G, J)


MO_CUT = 1e-10


def rmp2_direct(b: Basis, D: np.ndarray, C: np.ndarray, eps: np.ndarray, n_occ: int, n_frozen: int = 0) -> float:
    """Closed-shell MP2 through the reference's DIRECT transform.

    TransformIntegralsC.f90:472-665: for every active occupied i the first
    quarter A_i[nu][lam][sig] = sum_mu C(mu,i) (mu nu|lam sig) comes from
    LibintInterface_compute_2body_directIT (density-screened, |raw| > 1e-10),
    quarters 2-4 are dense sums, and only MO integrals with |(ia|jb)| > 1e-10
    are stored (:634).  MPFunctions.f90:514-662 then sums, for closed-shell
    electrons (lambda = 2, q^4 / (2 * particlesFraction) = 1),
    (ia|jb) [2 (ia|jb) - (ib|ja)] / (e_i + e_j - e_a - e_b), with integrals
    absent from the file read as zero.  C: columns are orbitals (n x n)."""
    Co = C[:, n_frozen:n_occ]
    Cv = C[:, n_occ:]
    eo, ev = eps[n_frozen:n_occ], eps[n_occ:]
    Crow = np.ascontiguousarray(C.T)
    e2 = 0.0
    for k, i in enumerate(range(n_frozen, n_occ)):
        A = two_body_directIT(b, True, D, Crow, i)
        M = np.einsum("nls,na,lj,sb->jab", A, Cv, Co, Cv, optimize=True)   # M[j][a][b] = (ia|jb)
        M[np.abs(M) <= MO_CUT] = 0.0
        den = eo[k] + eo[:, None, None] - ev[None, :, None] - ev[None, None, :]
        e2 += float(np.sum(M * (2.0 * M - M.transpose(0, 2, 1)) / den))
    return e2


def mp2_coupling_direct(bA: Basis, sidA: int, CA, epsA, noccA: int, nfA: int,
                        bB: Basis, sidB: int, CB, epsB, noccB: int, nfB: int, qAqB: float) -> float:
    """Inter-species MP2 of species A and B through the reference's DIRECT
    path: first quarter A_i[nu][lam][sig] = sum_mu C_A(mu,i) (mu nu|lam sig)
    from LibintInterface_compute_coupling_directIT (|raw| > 1e-10,
    Libint2Iface.cpp:1296-1622), quarters 2-4 dense, MO integrals with
    |(ia|jb)| <= 1e-10 dropped (TransformIntegralsC.f90), then
    MPFunctions.f90:682-886: sum (q_A q_B (ia|jb))^2 / (e_i + e_j - e_a - e_b)
    (the caller multiplies by lambda_A lambda_B, :878-879).
    C: columns are orbitals."""
    CoB, CvB = CB[:, nfB:noccB], CB[:, noccB:]
    CvA = CA[:, noccA:]
    eoB, evB, evA = epsB[nfB:noccB], epsB[noccB:], epsA[noccA:]
    Crow = np.ascontiguousarray(CA.T)
    e2 = 0.0
    for i in range(nfA, noccA):
        A = coupling_directIT(bA, sidA, bB, sidB, Crow, i)            # [nu in A][lam in B][sig in B]
        M = np.einsum("nls,na,lj,sb->ajb", A, CvA, CoB, CvB, optimize=True)   # (ia|jb)
        M[np.abs(M) <= MO_CUT] = 0.0
        den = epsA[i] + eoB[None, :, None] - evA[:, None, None] - evB[None, None, :]
        e2 += float(np.sum((qAqB * M) ** 2 / den))
    return e2


def apmo_mp2(system, res) -> dict:
    """Second-order correction of an APMO Hartree-Fock solution (no frozen
    core): the closed-shell intra-species term of every electron species and
    the inter-species term of every species pair.  One-particle species
    (lambda = 1) have no intra-species term.  Returns the parts and the total
    corrected energy."""
    sp = system.species
    parts = {}
    for k, s in enumerate(sp):
        if s.is_electron and s.n_particles > 1:
            parts[(k,)] = rmp2_direct(s.basis, res.densities[k], res.coefficients[k], res.orbital_energies[k],
                                      s.n_occ)
    for a in range(len(sp)):
        for b in range(a + 1, len(sp)):
            A, B = sp[a], sp[b]
            # lambda_A lambda_B x the pair sum (MPFunctions.f90:878-879); lambda = eta for
            # electrons (2) and one-particle protons (1)
            parts[(a, b)] = A.eta * B.eta * mp2_coupling_direct(
                A.basis, a + 1, res.coefficients[a], res.orbital_energies[a], A.n_occ, 0, B.basis, b + 1,
                res.coefficients[b], res.orbital_energies[b], B.n_occ, 0, A.charge * B.charge)
    return {"parts": parts, "e2": sum(parts.values()), "total": res.energy + sum(parts.values())}


def rmp2(eri_ao: np.ndarray, C: np.ndarray, eps: np.ndarray, n_occ: int, n_frozen: int = 0) -> float:
    """Closed-shell MP2 correlation energy, sum (ia|jb)[2(ia|jb)-(ib|ja)]/D."""
    o = C[:, n_frozen:n_occ]
    v = C[:, n_occ:]
    ovov = np.einsum("pqrs,pi,qa,rj,sb->iajb", eri_ao, o, v, o, v, optimize=True)
    eo, ev = eps[n_frozen:n_occ], eps[n_occ:]
    den = eo[:, None, None, None] - ev[None, :, None, None] + eo[None, None, :, None] - ev[None, None, None, :]
    return float(np.sum(ovov * (2 * ovov - ovov.transpose(0, 3, 2, 1)) / den))
