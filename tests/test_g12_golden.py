"""The G12 path pinned to the reference's own golden values, on the CPU.

test/TIP4P-dimer-{singlet,triplet}-direct put the two protons of a TIP4P water
dimer in Gaussian-fit potentials: the external O-H potential VOH-CCSDT on each
proton (EXTERPOTENTIAL), the H-H potential VHH-CCSDT between them
(INTERPOTENTIAL, G12 integrals in place of Coulomb), and the charges of the
second water as fixed point charges.  Singlet: two species with one proton
each, coupled by the inter-species G12 matrix.  Triplet: one species with both
protons, UHF, G = G12 Coulomb - G12 exchange.  The checkers assert the HF
energy to 1e-8 and the energy components to 1e-4.

test/He.POTENTIALS does the same for the two electrons of He: the fitted
potential HEE is their nucleus and the fitted EE their interaction; and
test/He{2,3}-C60potential-NOCI for helium atoms in a C60 cage fitted as 1500
off-centre Gaussian terms.

The external-potential matrix is checked twice: the oracle's quadrature against
the identity exp(-0 r^2) = 1 (the overlap) and the library's host recursion
(LowdinGB300_gaussian_potential, no GPU work) against the oracle.
"""
import numpy as np
import pytest

from openlowdin_gb300 import systems as S
from tests import golden_systems as GS

TESTS = ("TIP4P-dimer-singlet-direct", "TIP4P-dimer-triplet-direct")


@pytest.fixture(scope="module")
def built():
    from openlowdin_gb300 import build, lint
    build.build()
    return lint


def _mixed_shells():
    # contracted and uncontracted s, p, d, f shells on three centres
    A, B, C = [0.0, 0.0, 0.0], [0.3, -0.8, 1.1], [-1.0, 0.4, 0.2]
    return [(0, [5.0, 1.2, 0.3], [0.2, 0.5, 0.4], A), (1, [2.0, 0.5], [0.6, 0.5], A), (2, [1.1], [1.0], B),
            (3, [0.9], [1.0], C), (0, [0.7], [1.0], C), (2, [3.0, 0.8], [0.3, 0.8], A)]


def test_gaussian_potential_of_a_constant_is_the_overlap(oracle):
    b = oracle.Basis.from_shells(_mixed_shells())
    Sm, _ = oracle.overlap_kinetic(b)
    V = oracle.gaussian_potential(b, [2.5], [0.0], [[0.3, 0.2, -0.1]])
    assert np.max(np.abs(V - 2.5 * Sm)) < 1e-12


def test_gaussian_potential_factorises(oracle):
    """exp(-g |r-C|^2) exp(-h |r-C|^2) = exp(-(g+h) |r-C|^2) and linearity in
    the components."""
    b = oracle.Basis.from_shells(_mixed_shells())
    C = [[0.1, -0.2, 0.5]]
    V1 = oracle.gaussian_potential(b, [1.0], [0.7], C)
    V2 = oracle.gaussian_potential(b, [-3.0], [2.2], C)
    V12 = oracle.gaussian_potential(b, [1.0, -3.0], [0.7, 2.2], C + C)
    assert np.max(np.abs(V12 - V1 - V2)) < 1e-13
    assert np.max(np.abs(V1 - V1.T)) < 1e-13


def test_library_gaussian_potential_matches_oracle(built, oracle):
    sh = _mixed_shells()
    b = oracle.Basis.from_shells(sh)
    h = built.Libint2Interface(S.electron_species(sh, 2), 1)
    coef, expo = [0.7, -1.3, 2.0], [0.4, 1.7, 0.05]
    origins = [[0.0, 0.0, 0.0], [0.5, -0.5, 0.9], [-1.2, 0.3, 0.4]]
    ref = oracle.gaussian_potential(b, coef, expo, origins)
    assert np.max(np.abs(h.gaussian_potential(coef, expo, origins) - ref)) < 1e-12
    assert np.max(np.abs(h.gaussian_potential([], [], []))) == 0.0
    h.close()


@pytest.mark.parametrize("test", TESTS)
def test_library_external_potential_of_tip4p(built, oracle, golden, test):
    sysd = GS.g12_system(golden, test)
    for e in sysd["external_potentials"]:
        sp = sysd["species"][e["species"]]
        h = built.Libint2Interface(sp, 1)
        ref = oracle.gaussian_potential(oracle.Basis.from_shells(sp["shells"]), e["coefficients"],
                                        e["exponents"], e["origins"])
        assert np.max(np.abs(h.gaussian_potential(e["coefficients"], e["exponents"], e["origins"]) - ref)) < 1e-12
        h.close()


def _components(oracle, sysd, res):
    sy = oracle.from_plain(sysd)
    names = [s["name"] for s in sysd["species"]]
    Vext, Vfix, GJ, Gintra, Ginter = [], [], [], [], {}
    for i, s in enumerate(sy.species):
        e = sy.external.get(i)
        Vext.append(oracle.gaussian_potential(s.basis, *e) if e else np.zeros_like(res.densities[i]))
        Vfix.append(s.charge * oracle.potential(s.basis, sy.point_charges, sy.point_positions))
        pot = sy.interpotentials.get((i, i))
        if s.n_particles > 1 and pot:
            GJ.append(oracle.g12_direct(s.basis, res.densities[i], 0.0, *pot))
            Gintra.append(oracle.g12_direct(s.basis, res.densities[i], s.exchange_factor, *pot))
        else:
            GJ.append(None); Gintra.append(None)
        for j in range(i + 1, len(sy.species)):
            if (i, j) in sy.interpotentials:
                Ginter[(i, j)] = res.coupling[i][1][j]
    return GS.g12_components(res.densities, names, sysd, Vext, Vfix, Ginter, GJ, Gintra)


@pytest.mark.parametrize("test", TESTS)
def test_oracle_reproduces_tip4p_golden(oracle, golden, test):
    """The oracle SCF (G12 pair potentials, external Gaussian potential, fixed
    charges) against the checker's HF energy (1e-8) and components (1e-4).
    The triplet converges slowly along a nearly flat direction (the energy
    moves by < 1e-10 while the density still moves), so it runs to a fixed
    200 iterations with the checker's own energy criterion met."""
    sysd = GS.g12_system(golden, test)
    singlet = "singlet" in test
    res = oracle.scf(oracle.from_plain(sysd), tol_energy=1e-12, tol_density=1e-9 if singlet else 0.0,
                     max_iter=60 if singlet else 200)
    if singlet:
        assert res.converged
    ref = golden["values"][test]
    assert abs(res.energy - ref["HF energy"][0]) <= ref["HF energy"][1], res.energy
    comps = _components(oracle, sysd, res)
    for key, (val, tol) in ref.items():
        if key == "HF energy":
            continue
        assert abs(comps[key] - val) <= tol, (key, comps[key], val)
    if singlet:
        # the singlet's components agree far inside the checker's tolerance
        for key, (val, _) in ref.items():
            if key != "HF energy":
                assert abs(comps[key] - val) < 2e-8, (key, comps[key], val)


def test_oracle_reproduces_he_potentials(oracle, golden):
    """test/He.POTENTIALS: the He electrons (UHF) with the fitted nucleus
    potential HEE and the fitted electron-electron potential EE in place of
    Coulomb (both from the reference's lib/potentials); HF energy 1e-8."""
    res = oracle.scf(oracle.from_plain(GS.he_potentials(golden)), tol_energy=1e-11, tol_density=1e-9)
    ref = golden["values"]["He.POTENTIALS"]["HF energy"]
    assert res.converged and abs(res.energy - ref[0]) <= ref[1], res.energy


C60_TESTS = ("He2-C60potential-NOCI", "He3-C60potential-NOCI")


@pytest.mark.parametrize("test", C60_TESTS)
def test_oracle_reproduces_c60_cage(oracle, golden, test):
    """test/He2-C60potential-NOCI and He3-: helium atoms (one s function each;
    in He3 two of them form one species) in a C60 cage given as 1500 Gaussian
    terms at the 60 carbon centres, interacting through a fitted He-He
    potential; HF energy 1e-8 (the checkers' NOCI values are not used)."""
    res = oracle.scf(oracle.from_plain(GS.c60_system(golden, test)), tol_energy=1e-12, tol_density=1e-10)
    ref = golden["values"][test]["HF energy"]
    assert res.converged and abs(res.energy - ref[0]) <= ref[1], res.energy


def test_library_c60_cage_potential(built, oracle, golden):
    """The library's host recursion on 1500 off-centre components against the
    oracle's quadrature."""
    sysd = GS.c60_system(golden, "He3-C60potential-NOCI")
    for e in sysd["external_potentials"]:
        sp = sysd["species"][e["species"]]
        h = built.Libint2Interface(sp, 1)
        ref = oracle.gaussian_potential(oracle.Basis.from_shells(sp["shells"]), e["coefficients"],
                                        e["exponents"], e["origins"])
        got = h.gaussian_potential(e["coefficients"], e["exponents"], e["origins"])
        assert np.max(np.abs(got - ref)) < 1e-12 * max(1.0, np.max(np.abs(ref)))
        h.close()


def test_library_gaussian_potential_random_cases(built, oracle):
    """Random contracted shells up to f on random centres and random
    off-centre components: the library's recursion against the oracle's
    quadrature, relative 1e-11."""
    rng = np.random.default_rng(11)
    for case in range(6):
        sh = []
        for _ in range(int(rng.integers(2, 6))):
            l = int(rng.integers(0, 4))
            k = int(rng.integers(1, 4))
            sh.append((l, list(rng.uniform(0.2, 6.0, k)), list(rng.uniform(0.1, 1.0, k)),
                       list(rng.uniform(-1.5, 1.5, 3))))
        m = int(rng.integers(1, 8))
        coef, expo = rng.normal(size=m), rng.uniform(0.0, 4.0, m)
        origins = rng.uniform(-2.0, 2.0, (m, 3))
        h = built.Libint2Interface(S.electron_species(sh, 2), 1)
        ref = oracle.gaussian_potential(oracle.Basis.from_shells(sh), coef, expo, origins)
        got = h.gaussian_potential(coef, expo, origins)
        assert np.max(np.abs(got - ref)) <= 1e-11 * max(1.0, np.max(np.abs(ref))), case
        h.close()
