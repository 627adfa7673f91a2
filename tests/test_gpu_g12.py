"""GPU parity of the geminal (G12) direct matrices against the oracle.

libintinterface_compute_g12_direct / _g12inter_direct (reference
src/ints/Libint2Iface.cpp:2193-2540, wrappers :3687-3734) through the C ABI,
element-wise against the oracle's restatement (itself pinned by Gauss-Hermite
quadrature and by the constant-potential identity, tests/test_g12_oracle.py).
Tolerance: 1e-10 absolute per element, as the Coulomb matrices.
"""
import numpy as np
import pytest

from openlowdin_gb300 import systems as S

pytestmark = pytest.mark.gpu

TOL = 1e-10
# a synthetic potential: a constant, a long-range and two short-range terms
COEF = [0.085, 1.3, -4.3, 7.5]
EXPO = [0.0, 0.1, 0.75, 5.6]


@pytest.fixture(scope="module")
def L():
    from openlowdin_gb300 import build, lint
    build.build()
    return lint


def _sym(rng, n, scale=0.2):
    X = rng.normal(size=(n, n)) * scale
    return X + X.T


@pytest.mark.parametrize("d_shell", [False, True])
def test_g12_intra_matches_oracle(L, oracle, d_shell):
    """Every class up to (dd|dd) when the oxygen carries a d shell."""
    sp = S.water(d_shell=d_shell)["species"][0]
    b = oracle.Basis.from_shells(sp["shells"])
    D = _sym(np.random.default_rng(1), b.nbf)
    h = L.Libint2Interface(sp, 1)
    G = h.compute_g12_direct(D, -0.5, COEF, EXPO)
    ref = oracle.g12_direct(b, D, -0.5, COEF, EXPO)
    assert np.max(np.abs(G - ref)) < TOL
    assert np.max(np.abs(G - G.T)) == 0.0
    h.close()


def test_g12_intra_protons_and_repeated_calls(L, oracle):
    """A non-electron species (factor -1), then a second potential on the same handle."""
    sp = S.water_cluster(2, seed=1, quantum_protons=True, proton_species_mode="single")["species"][1]
    b = oracle.Basis.from_shells(sp["shells"])
    D = _sym(np.random.default_rng(2), b.nbf, 0.05)
    h = L.Libint2Interface(sp, 2)
    for coef, expo in ((COEF, EXPO), ([2.0, -0.7], [1.5, 12.0])):
        G = h.compute_g12_direct(D, -1.0, coef, expo)
        ref = oracle.g12_direct(b, D, -1.0, coef, expo)
        assert np.max(np.abs(G - ref)) < TOL
    h.close()


def test_g12_constant_potential_is_overlap_products(L, oracle):
    sp = S.water(d_shell=True)["species"][0]
    b = oracle.Basis.from_shells(sp["shells"])
    Sm, _ = oracle.overlap_kinetic(b)
    D = _sym(np.random.default_rng(3), b.nbf)
    h = L.Libint2Interface(sp, 1)
    G = h.compute_g12_direct(D, -0.5, [0.37], [0.0])
    ref = 0.37 * (Sm * np.sum(D * Sm) - 0.5 * Sm @ D @ Sm)
    assert np.max(np.abs(G - ref)) < TOL
    h.close()


def test_g12_inter_matches_oracle_both_orders(L, oracle):
    sysd = S.water_cluster(2, seed=0, quantum_protons=True, proton_species_mode="single")
    ea, pr = sysd["species"][0], sysd["species"][1]
    be, bp = oracle.Basis.from_shells(ea["shells"]), oracle.Basis.from_shells(pr["shells"])
    rng = np.random.default_rng(4)
    De, Dp = _sym(rng, be.nbf, 0.1), _sym(rng, bp.nbf, 0.05)
    he, hp = L.Libint2Interface(ea, 1), L.Libint2Interface(pr, 2)
    # electrons from the protons' density (id 1 < 2: not permuted) ...
    B = he.compute_g12inter_direct(hp, Dp, COEF, EXPO)
    ref = oracle.g12inter_direct(be, 1, bp, 2, Dp, COEF, EXPO)
    assert np.max(np.abs(B - ref)) < TOL
    assert np.all(np.triu(B, 1) == 0.0)
    # ... and the protons from the electrons' density (permuted loops)
    B = hp.compute_g12inter_direct(he, De, COEF, EXPO)
    ref = oracle.g12inter_direct(bp, 2, be, 1, De, COEF, EXPO)
    assert np.max(np.abs(B - ref)) < TOL
    he.close()
    hp.close()


def test_g12_rejects_bad_potentials(L):
    sp = S.water()["species"][0]
    h = L.Libint2Interface(sp, 1)
    D = np.eye(S.nbasis(sp))
    with pytest.raises(L.LowdinGB300Error, match="pot_size"):
        h.compute_g12_direct(D, -0.5, [], [])
    with pytest.raises(L.LowdinGB300Error, match="exponent"):
        h.compute_g12_direct(D, -0.5, [1.0], [-0.5])
    # the handle stays usable
    G = h.compute_g12_direct(D, -0.5, [1.0], [0.5])
    assert np.all(np.isfinite(G))
    h.close()


@pytest.mark.parametrize("test", ["TIP4P-dimer-singlet-direct", "TIP4P-dimer-triplet-direct"])
def test_tip4p_golden_through_host_scf(L, oracle, golden, test):
    """test/TIP4P-dimer-*-direct end to end through the reference-shaped host
    calls (HostSCF: external potential, G12 intra- and inter-species matrices
    on the device each iteration): the checker's HF energy (1e-8) and energy
    components (1e-4), the G12 matrices at the converged densities against the
    oracle (1e-10), and the energy against the oracle SCF.  The triplet runs a
    fixed 200 iterations (its energy is flat to 1e-10 long before its density
    settles); the singlet converges."""
    from openlowdin_gb300 import scf
    from tests import golden_systems as GS
    from tests.test_g12_golden import _components
    sysd = GS.g12_system(golden, test)
    singlet = "singlet" in test
    s = scf.HostSCF(sysd)
    r = s.solve(tol_energy=1e-12, tol_density=1e-9 if singlet else 0.0, max_iter=60 if singlet else 200)
    sy = oracle.from_plain(sysd)
    for i, (h, sp) in enumerate(zip(s.handles, sy.species)):
        pot = sy.interpotentials.get((i, i))
        if sp.n_particles > 1 and pot:
            G = h.compute_g12_direct(r.densities[i], sp.exchange_factor, *pot)
            assert np.max(np.abs(G - oracle.g12_direct(sp.basis, r.densities[i], sp.exchange_factor, *pot))) < TOL
        for j, o in enumerate(sy.species):
            pot = sy.interpotentials.get((min(i, j), max(i, j)))
            if j != i and pot:
                B = h.compute_g12inter_direct(s.handles[j], r.densities[j], *pot)
                ref = oracle.g12inter_direct(sp.basis, i + 1, o.basis, j + 1, r.densities[j], *pot)
                assert np.max(np.abs(np.tril(B) - np.tril(ref))) < TOL
    s.close()
    if singlet:
        assert r.converged
    ref = golden["values"][test]
    assert abs(r.energy - ref["HF energy"][0]) <= ref["HF energy"][1], r.energy
    res = oracle.scf(sy, tol_energy=1e-12, tol_density=1e-9 if singlet else 0.0, max_iter=60 if singlet else 200)
    assert abs(r.energy - res.energy) < 1e-10
    res.densities = r.densities
    for j in range(len(sy.species)):
        for k in list(res.coupling[j][1]):
            b = sy.species[j].basis
            pot = sy.interpotentials.get((min(j, k), max(j, k)))
            B = oracle.g12inter_direct(b, j + 1, sy.species[k].basis, k + 1, r.densities[k], *pot)
            res.coupling[j][1][k] = np.tril(B) + np.tril(B, -1).T
    comps = _components(oracle, sysd, res)
    for key, (val, tol) in ref.items():
        if key != "HF energy":
            assert abs(comps[key] - val) <= tol, (key, comps[key], val)
