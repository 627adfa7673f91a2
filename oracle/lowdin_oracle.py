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
* Gaussian-fit potentials: INTERPOTENTIAL replaces every Coulomb term by G12
  matrices without charge factors (``WaveFunction.f90:1097-1135, 1439-1477``),
  EXTERPOTENTIAL adds sum_k c_k exp(-g_k |r - C_k|^2) to H
  (``src/ints/DirectIntegralManager.f90:848-949``),
* iteration scheme 3 -- every species once per global iteration
  (``src/scf/MultiSCF.f90:276-440``) with Pulay DIIS or the reference's
  default damping (``src/scf/Convergence.f90:382-511``),
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


def _prim_norm(a: float, l: int) -> float:
    """Norm of the x^l component of a primitive (src/ints/Libint2Iface.cpp:79-128)."""
    df = 1.0
    for k in range(2 * l - 1, 1, -2):
        df *= k
    return float(np.sqrt(2.0 ** l * (2.0 * a) ** (l + 1.5) / (np.pi ** 1.5 * df)))


def _cart_exponents(l: int):
    return [(l - i, i - j, j) for i in range(l + 1) for j in range(i + 1)]


def gaussian_potential(b: Basis, coefficients, exponents, origins) -> np.ndarray:
    """External Gaussian-fit potential V_ij = sum_k c_k <i|exp(-g_k |r - C_k|^2)|j>
    (src/ints/DirectIntegralManager.f90:848-949: each contraction times each
    potential component, then an overlap with the other contraction), each
    Cartesian function normalised to one like ``norma``.

    Computed by Gauss-Hermite quadrature in each direction after completing the
    square of the three Gaussians (8 nodes: exact for the polynomial degree
    <= 15 that shells up to l = 7 give), not by the recursion the library uses."""
    xg, wg = np.polynomial.hermite.hermgauss(8)
    cs = np.asarray(coefficients, float)
    gs = np.asarray(exponents, float)
    Cs = np.asarray(origins, float).reshape(-1, 3)
    n = b.nbf
    V, S = np.zeros((n, n)), np.zeros((n, n))
    shells, off, first = [], 0, 0
    for s in range(b.nshell):
        l, k = int(b.l[s]), int(b.nprim[s])
        al = b.alpha[off:off + k]
        cn = np.array([b.coef[off + p] * _prim_norm(al[p], l) for p in range(k)])
        shells.append((l, al, cn, b.origin[3 * s:3 * s + 3], first))
        off += k
        first += (l + 1) * (l + 2) // 2

    def tables(a, A, la, bb, B, lb, g, C):
        # T[k, d, i, j] = int (x-A_d)^i (x-B_d)^j exp(-(p (x-x0)^2)) dx, and the
        # remaining factor exp(-c0_k) p_k^-1.5 of each component k
        p = a + bb + g
        x0 = (a * A[None, :] + bb * B[None, :] + g[:, None] * C) / p[:, None]
        c0 = np.sum(a * A ** 2 + bb * B ** 2 + g[:, None] * C ** 2 - p[:, None] * x0 ** 2, axis=1)
        x = x0[:, :, None] + xg[None, None, :] / np.sqrt(p)[:, None, None]
        pa = (x - A[None, :, None])[..., None] ** np.arange(la + 1)
        pb = (x - B[None, :, None])[..., None] ** np.arange(lb + 1)
        T = np.einsum("q,kdqi,kdqj->kdij", wg, pa, pb)
        return T, np.exp(-c0) / p ** 1.5

    one, zero = np.ones(1), np.zeros((1, 3))
    for la, aa, ca, A, fa in shells:
        for lb, ab, cb, B, fb in shells:
            ea, eb = _cart_exponents(la), _cart_exponents(lb)
            for pa_ in range(len(aa)):
                for pb_ in range(len(ab)):
                    w = ca[pa_] * cb[pb_]
                    for M, c, g, C in ((V, cs, gs, Cs), (S, one, np.zeros(1), zero)):
                        if len(c) == 0:
                            continue
                        T, f = tables(aa[pa_], A, la, ab[pb_], B, lb, g, C)
                        fk = w * c * f
                        for i, (ix, iy, iz) in enumerate(ea):
                            for j, (jx, jy, jz) in enumerate(eb):
                                M[fa + i, fb + j] += float(np.sum(fk * T[:, 0, ix, jx] * T[:, 1, iy, jy]
                                                                  * T[:, 2, iz, jz]))
    nrm = 1.0 / np.sqrt(np.diag(S))
    return V * np.outer(nrm, nrm)


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
    """Species, fixed point charges and, optionally, Gaussian-fit potentials:
    ``interpotentials`` {(i, j), i <= j: (coefficients, exponents)} (INTERPOTENTIAL:
    when present, every species pair interacts through G12 integrals instead of
    Coulomb, without charge factors, and pairs without a potential not at all --
    src/scf/WaveFunction.f90:1097-1135, 1439-1477) and ``external``
    {i: (coefficients, exponents, origins)} (EXTERPOTENTIAL, added to H_i)."""
    species: list
    point_charges: np.ndarray = field(default_factory=lambda: np.zeros(0))
    point_positions: np.ndarray = field(default_factory=lambda: np.zeros((0, 3)))
    interpotentials: dict = field(default_factory=dict)
    external: dict = field(default_factory=dict)

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
    inter = {}
    for e in desc.get("interpotentials", []):
        i, j = sorted(int(x) for x in e["species"])
        inter[(i, j)] = (list(e["coefficients"]), list(e["exponents"]))
    ext = {int(e["species"]): (list(e["coefficients"]), list(e["exponents"]), list(e["origins"]))
           for e in desc.get("external_potentials", [])}
    return System(sp, np.array(desc["point_charges"], float),
                  np.array(desc["point_positions"], float).reshape(-1, 3), inter, ext)


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


DOUBLE_ZERO_THRESHOLD = 1e-12   # src/core/CONTROL.f90:1592


def damping_step(F, P, F0, P0):
    """One species' step of the reference's default convergence method
    (CONVERGENCE_METHOD 1, Convergence_dampingMethod,
    src/scf/Convergence.f90:444-511): with the kept pair (F0, P0),
    d = -tr(F0 (P - P0)) / 2 and f = tr((F - F0)(P - P0)); when f <= d or
    |f| < 1e-12 the pair becomes (F, P) and F is used undamped, otherwise
    lambda = d / f moves F0 and P0 by lambda towards F and P and the damped F0
    is diagonalised.  Returns (Fock to diagonalise, F0, P0)."""
    dP = P - P0
    d = -0.5 * float(np.sum(F0 * dP.T))
    f = float(np.sum((F - F0) * dP.T))
    if f <= d or abs(f) < DOUBLE_ZERO_THRESHOLD:
        return F, F.copy(), P.copy()
    lam = d / f
    F0 = F0 + lam * (F - F0)
    return F0.copy(), F0, P0 + lam * (P - P0)


def reference_tolerances(criterion="ENERGY", total_energy=1e-8, total_density=1e-6, species_energy=1e-8,
                         species_density=1e-6) -> dict:
    """tol_energy, tol_density and sub_tolerances of scf() for the reference's
    scfConvergenceCriterium: the global test uses the chosen quantities
    (src/scf/MultiSCF.f90:813-830), and the reference switches the other
    quantity's tolerances off by setting them, per species and total, to 1.0
    (src/core/CONTROL.f90:3174-3190), which the single-species loops see."""
    c = criterion.upper()
    if c == "ENERGY":
        return {"tol_energy": total_energy, "tol_density": float("inf"), "sub_tolerances": (species_energy, 1.0)}
    if c == "DENSITY":
        return {"tol_energy": float("inf"), "tol_density": total_density, "sub_tolerances": (1.0, species_density)}
    if c == "BOTH":
        return {"tol_energy": total_energy, "tol_density": total_density,
                "sub_tolerances": (species_energy, species_density)}
    raise ValueError(f"unknown convergence criterion {criterion!r}")


def scheme_iterations(system: System, scheme: int, electronic_max=50, nonelectronic_max=50) -> list:
    """Single-species sub-iterations per global iteration of the reference's
    iteration schemes (src/scf/MultiSCF.f90:150-185): 0 = non-electronic
    species iterate up to nonelectronic_max times, 1 = electrons up to
    electronic_max, 2 = both, 3 = every species once (SCF_*_MAX_ITERATIONS
    default to 50, src/core/CONTROL.f90:1474-1475)."""
    out = []
    for s in system.species:
        el = s.is_electron
        out.append({0: 1 if el else nonelectronic_max, 1: electronic_max if el else 1,
                    2: electronic_max if el else nonelectronic_max, 3: 1}[scheme])
    return out


def scf(system: System, tol_energy=1e-10, tol_density=1e-8, max_iter=200, nthreads=None,
        convergence="diis", density_sum=False, sub_iterations=None, sub_tolerances=(1e-8, 1e-6),
        verbose=False) -> SCFResult:
    """Multi-species Hartree-Fock restated from src/scf: every global
    iteration builds every species' two-particle and coupling matrices, Fock
    matrix and the total energy from the current densities, then updates the
    species one after the other (src/scf/MultiSCF.f90:276-440).

    convergence: "diis" (Pulay, CONVERGENCE_METHOD 2), "damping" (the
    reference's default, CONVERGENCE_METHOD 1; the kept pair starts from the
    first Fock build, src/scf/MultiSCF.f90:330-336) or "none".  Converged
    when |dE| < tol_energy and the density change < tol_density (either
    criterion alone with the other tolerance set to inf): the largest rms
    change over the species, or with density_sum their sum, the reference's
    measure (src/scf/MultiSCF.f90:350-425, 776-830).

    sub_iterations (scheme_iterations; default one per species, scheme 3):
    a species with more than one iterates on its own inside the global
    iteration -- diagonalise, new density, its energy tr P (H + G/2 + J) with
    the matrices so far, rebuild its two-particle matrix (the couplings stay
    those of the global build) -- while its energy change or its density
    change exceeds sub_tolerances (1e-8 / 1e-6 by default, CONTROL.f90:
    1461-1464; reference_tolerances gives the values the reference's
    criteria leave), up to that many times (MultiSCF.f90:350-425).  Not
    with DIIS, which the drivers here run over all species at once."""
    if convergence not in ("diis", "damping", "none"):
        raise ValueError(f"unknown convergence method {convergence!r}")
    if sub_iterations is not None and max(sub_iterations) > 1 and convergence == "diis":
        raise ValueError("single-species sub-iterations need damping or no convergence method")
    sp = system.species
    ns = len(sp)
    H, X, S = [], [], []
    for s in sp:
        Sm, T = overlap_kinetic(s.basis)
        V = potential(s.basis, system.point_charges, system.point_positions)
        # T / mass + (q) * V  -- puntual interaction scaled by the particle charge
        H.append(T / s.mass + s.charge * V)
        if len(H) - 1 in system.external:
            H[-1] = H[-1] + gaussian_potential(s.basis, *system.external[len(H) - 1])
        S.append(Sm)
        X.append(_orthogonaliser(Sm))
    g12 = bool(system.interpotentials)
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
    kept = None
    e_old = None
    converged = False
    it = 0
    sub = list(sub_iterations) if sub_iterations is not None else [1] * ns

    def build_G(i, Pi):
        s = sp[i]
        if s.n_particles > 1 and not g12:
            return two_body_direct(s.basis, s.is_electron, Pi, s.exchange_factor, nthreads) * s.charge ** 2
        if s.n_particles > 1 and (i, i) in system.interpotentials:
            return g12_direct(s.basis, Pi, s.exchange_factor, *system.interpotentials[(i, i)], nthreads)
        return np.zeros_like(H[i])

    def diagonalise(i, Fi):
        e, Cp = np.linalg.eigh(X[i].T @ Fi @ X[i])
        Ci = X[i] @ Cp
        C[i] = Ci; eps[i] = e
        return sp[i].eta * Ci[:, :sp[i].n_occ] @ Ci[:, :sp[i].n_occ].T

    for it in range(1, max_iter + 1):
        G, J = [], []
        for i, s in enumerate(sp):
            G.append(build_G(i, P[i]))
            Ji = np.zeros_like(H[i])
            Jparts = {}
            for j, o in enumerate(sp):
                if j == i:
                    continue
                if not g12:
                    B = coupling_direct(s.basis, i + 1, o.basis, j + 1, P[j], nthreads) * s.charge * o.charge
                elif (min(i, j), max(i, j)) in system.interpotentials:
                    B = g12inter_direct(s.basis, i + 1, o.basis, j + 1, P[j],
                                        *system.interpotentials[(min(i, j), max(i, j))], nthreads)
                else:
                    B = np.zeros((s.basis.nbf, s.basis.nbf))
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
        if kept is None and convergence == "damping":
            kept = [(F[i].copy(), P[i].copy()) for i in range(ns)]
        if max(sub) > 1:
            newP, dmax = [], 0.0
            for i in range(ns):
                Fi, Gi, Pi, Ji = F[i], G[i], P[i], J[i][0]
                e_i = float(np.sum(Pi * (H[i] + 0.5 * Gi + Ji)))
                d_e, rms, k = 1e16, np.inf, 0
                while (abs(d_e) > sub_tolerances[0] or rms > sub_tolerances[1]) and k < sub[i]:
                    k += 1
                    Fd = Fi
                    if convergence == "damping":
                        Fd, F0, P0 = damping_step(Fi, Pi, *kept[i])
                        kept[i] = (F0, P0)
                    Pn = diagonalise(i, Fd)
                    rms = float(np.sqrt(np.mean((Pn - Pi) ** 2)))
                    Pi = Pn
                    e_new = float(np.sum(Pi * (H[i] + 0.5 * Gi + Ji)))
                    if sub[i] > 1:
                        Gi = build_G(i, Pi)
                        Fi = H[i] + Gi + Ji
                        d_e, e_i = e_i - e_new, e_new
                newP.append(Pi)
                dmax = dmax + rms if density_sum else max(dmax, rms)
            if verbose:
                print(f"iter {it:3d}  E = {energy:.12f}  dP = {dmax:.2e}")
            if e_old is not None and abs(energy - e_old) < tol_energy and dmax < tol_density:
                converged = True
                break
            e_old = energy
            P = newP
            continue
        newP = []
        dmax = 0.0
        Fx = F
        if convergence == "diis":
            errs = [X[i].T @ (F[i] @ P[i] @ S[i] - S[i] @ P[i] @ F[i]) @ X[i] for i in range(ns)]
            Fx = diis_obj(F, errs)
        elif convergence == "damping":
            Fx = []
            for i in range(ns):
                Fd, F0, P0 = damping_step(F[i], P[i], *kept[i])
                kept[i] = (F0, P0)
                Fx.append(Fd)
        for i, s in enumerate(sp):
            Pn = diagonalise(i, Fx[i])
            rms = float(np.sqrt(np.mean((Pn - P[i]) ** 2)))
            dmax = dmax + rms if density_sum else max(dmax, rms)
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
