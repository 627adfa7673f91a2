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
