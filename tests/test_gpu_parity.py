"""GPU parity: the C-ABI library against the oracle, element-wise.

Tolerance: 1e-10 absolute on every element of the two-particle / coupling
matrices (plain FP64); 1e-9 on first-quarter tensors (they sum n raw products
with coefficients of order 1-10).
"""
import numpy as np
import pytest

from openlowdin_gb300 import systems as S
from tests import golden_systems as GS

pytestmark = pytest.mark.gpu

TOL_FOCK = 1e-10
TOL_IT = 1e-9


@pytest.fixture(scope="module")
def L():
    from openlowdin_gb300 import build, lint
    build.build()
    return lint


def _sym(rng, n, scale=0.3):
    X = rng.normal(size=(n, n)) * scale
    return X + X.T


def _scf_density(oracle, sysd, species=0):
    res = oracle.scf(oracle.from_plain(sysd), tol_energy=1e-9, tol_density=1e-6)
    return res.densities[species]


def test_twobody_water_scf_density(L, oracle):
    """c0 workload, converged density: screening active, factor -1/2."""
    sysd = S.water()
    sp = sysd["species"][0]
    D = _scf_density(oracle, sysd)
    h = L.Libint2Interface(sp, 1)
    G = h.compute_2body_direct(D, -0.5)
    ref = oracle.two_body_direct(oracle.Basis.from_shells(sp["shells"]), True, D, -0.5)
    assert np.max(np.abs(G - ref)) < TOL_FOCK
    assert np.max(np.abs(G - G.T)) == 0.0
    h.close()


def test_twobody_contracted_golden_basis(L, oracle, golden):
    """6-311G (contracted s/p shells) of test/H2O.BOA.DIRECT."""
    sysd = GS.h2o_boa(golden)
    sp = sysd["species"][0]
    rng = np.random.default_rng(11)
    D = _sym(rng, S.nbasis(sp))
    h = L.Libint2Interface(sp, 1)
    G = h.compute_2body_direct(D, -0.5)
    ref = oracle.two_body_direct(oracle.Basis.from_shells(sp["shells"]), True, D, -0.5)
    assert np.max(np.abs(G - ref)) < TOL_FOCK
    h.close()


def test_twobody_protons_unscreened(L, oracle):
    """Non-electron species: no Schwarz screening, factor kappa/eta = -1."""
    sysd = S.water_cluster(2, seed=1, quantum_protons=True, proton_species_mode="single")
    sp = sysd["species"][1]
    rng = np.random.default_rng(5)
    D = _sym(rng, S.nbasis(sp), 0.05)
    h = L.Libint2Interface(sp, 2)
    G = h.compute_2body_direct(D, -1.0)
    ref = oracle.two_body_direct(oracle.Basis.from_shells(sp["shells"]), False, D, -1.0)
    assert np.max(np.abs(G - ref)) < TOL_FOCK
    h.close()


def test_twobody_apmo_cluster_electrons(L, oracle):
    """Electrons of the 4-water APMO cluster (136 functions)."""
    sysd = S.water_cluster(4, seed=0, quantum_protons=True)
    sp = sysd["species"][0]
    rng = np.random.default_rng(3)
    D = _sym(rng, S.nbasis(sp), 0.1)
    h = L.Libint2Interface(sp, 1)
    G = h.compute_2body_direct(D, -0.5)
    ref = oracle.two_body_direct(oracle.Basis.from_shells(sp["shells"]), True, D, -0.5)
    assert np.max(np.abs(G - ref)) < TOL_FOCK
    assert h.last_quartets() == oracle.last_quartet_count()
    h.close()


@pytest.mark.parametrize("ids", [(1, 2), (2, 1)])
def test_coupling_both_orders(L, oracle, ids):
    sysd = S.water_cluster(1, seed=0, quantum_protons=True, place=False, proton_species_mode="single")
    e, p = sysd["species"]
    rng = np.random.default_rng(4)
    Dp = _sym(rng, S.nbasis(p), 0.2)
    he = L.Libint2Interface(e, ids[0])
    hp = L.Libint2Interface(p, ids[1])
    B = he.compute_coupling_direct(hp, Dp)
    ref = oracle.coupling_direct(oracle.Basis.from_shells(e["shells"]), ids[0],
                                 oracle.Basis.from_shells(p["shells"]), ids[1], Dp)
    assert np.max(np.abs(B - ref)) < TOL_FOCK
    assert np.all(np.triu(B, 1) == 0.0)
    he.close(); hp.close()


@pytest.mark.parametrize("ids", [(1, 2), (2, 1)])
def test_alphabeta_energy(L, oracle, ids):
    """LibintInterface_compute_alphabeta_direct: alpha and beta electrons of
    the water basis (two species, one basis), random densities; both handle
    orders give sum D_a (ij|kl) D_b."""
    sp = S.water()["species"][0]
    n = S.nbasis(sp)
    rng = np.random.default_rng(12)
    Da, Db = _sym(rng, n, 0.2), _sym(rng, n, 0.2)
    ha = L.Libint2Interface(sp, ids[0])
    hb = L.Libint2Interface(sp, ids[1])
    b = oracle.Basis.from_shells(sp["shells"])
    ref = oracle.alphabeta_direct(b, ids[0], b, ids[1], Da, Db)
    e_ab = ha.compute_alphabeta_direct(hb, Da, Db)
    e_ba = hb.compute_alphabeta_direct(ha, Db, Da)
    assert abs(e_ab - ref) < 1e-10 * max(1.0, abs(ref))
    assert abs(e_ba - ref) < 1e-10 * max(1.0, abs(ref))
    ha.close(); hb.close()


def test_alphabeta_golden_apmo_water(L, oracle, golden):
    """test/H2O.APMO.UHF.DIRECT.py: E-ALPHA/E-BETA Hartree energy from the
    library (closed-shell solution: P_alpha = P_beta = P_e / 2)."""
    sysd = GS.h2o_apmo(golden)
    res = oracle.scf(oracle.from_plain(sysd))
    sp = sysd["species"][0]
    Ph = res.densities[0] / 2.0
    ha, hb = L.Libint2Interface(sp, 1), L.Libint2Interface(sp, 2)
    e = ha.compute_alphabeta_direct(hb, Ph, Ph)
    ha.close(); hb.close()
    b = oracle.Basis.from_shells(sp["shells"])
    assert abs(e - oracle.alphabeta_direct(b, 1, b, 2, Ph, Ph)) < 1e-9
    ref = golden["values"]["H2O.APMO.UHF.DIRECT"]["e-AlphaBetaRepulsion"]
    assert abs(e - ref[0]) <= ref[1]


def test_first_quarter_intra(L, oracle):
    sysd = S.water()
    sp = sysd["species"][0]
    n = S.nbasis(sp)
    rng = np.random.default_rng(6)
    C = rng.normal(size=(n, n))
    D = _scf_density(oracle, sysd)
    h = L.Libint2Interface(sp, 1)
    for p in (0, 4):
        A = h.compute_2body_directIT(D, C, p)
        ref = oracle.two_body_directIT(oracle.Basis.from_shells(sp["shells"]), True, D, C, p)
        assert np.max(np.abs(A - ref)) < TOL_IT
    h.close()


def test_first_quarter_coupling(L, oracle):
    sysd = S.water_cluster(1, seed=0, quantum_protons=True, place=False, proton_species_mode="single")
    e, p = sysd["species"]
    ne = S.nbasis(e)
    rng = np.random.default_rng(8)
    C = rng.normal(size=(ne, ne))
    he = L.Libint2Interface(e, 1)
    hp = L.Libint2Interface(p, 2)
    A = he.compute_coupling_directIT(hp, C, 2)
    ref = oracle.coupling_directIT(oracle.Basis.from_shells(e["shells"]), 1,
                                   oracle.Basis.from_shells(p["shells"]), 2, C, 2)
    assert np.max(np.abs(A - ref)) < TOL_IT
    he.close(); hp.close()


def test_device_entry_points_match_host_calls(L, oracle):
    torch = pytest.importorskip("torch")
    sysd = S.water_cluster(1, seed=0, quantum_protons=True, place=False, proton_species_mode="single")
    e, p = sysd["species"]
    rng = np.random.default_rng(9)
    De, Dp = _sym(rng, S.nbasis(e), 0.2), _sym(rng, S.nbasis(p), 0.2)
    he = L.Libint2Interface(e, 1)
    hp = L.Libint2Interface(p, 2)
    dDe = torch.tensor(De, device="cuda")
    dDp = torch.tensor(Dp, device="cuda")
    dG = torch.empty_like(dDe)
    dJe = torch.empty_like(dDe)
    dJp = torch.empty_like(dDp)
    stream = torch.cuda.current_stream().cuda_stream
    he.twobody_device(dDe.data_ptr(), dG.data_ptr(), -0.5, stream=stream)
    L.coupling_device(he, hp, dDe.data_ptr(), dDp.data_ptr(), dJe.data_ptr(), dJp.data_ptr(), stream=stream)
    torch.cuda.synchronize()
    G = he.compute_2body_direct(De, -0.5)
    assert np.max(np.abs(dG.cpu().numpy() - G)) < 1e-12
    Be = he.compute_coupling_direct(hp, Dp)
    Bp = hp.compute_coupling_direct(he, De)
    Je, Jp = dJe.cpu().numpy(), dJp.cpu().numpy()
    assert np.max(np.abs(np.tril(Je) - Be)) < TOL_FOCK
    assert np.max(np.abs(np.tril(Jp) - Bp)) < TOL_FOCK
    assert np.max(np.abs(Je - Je.T)) < 1e-14
    he.close(); hp.close()


@pytest.mark.parametrize("which", ["water_d", "apmo_proton", "golden_6311g"])
def test_one_body_device_matches_host(L, golden, which):
    """LowdinGB300_one_body_device against the host one-electron blocks."""
    torch = pytest.importorskip("torch")
    if which == "water_d":
        sysd = S.water(d_shell=True); k = 0
    elif which == "apmo_proton":
        sysd = S.water_cluster(2, seed=1, quantum_protons=True); k = 1
    else:
        sysd = GS.h2o_boa(golden); k = 0
    sp = sysd["species"][k]
    h = L.Libint2Interface(sp, k + 1)
    n = h.nbasis
    dS, dT, dV = (torch.empty((n, n), dtype=torch.float64, device="cuda") for _ in range(3))
    h.one_body_device(sysd["point_charges"], sysd["point_positions"], dS.data_ptr(), dT.data_ptr(), dV.data_ptr(),
                      torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert np.max(np.abs(dS.cpu().numpy() - h.one_body(1))) < 1e-12
    assert np.max(np.abs(dT.cpu().numpy() - h.one_body(2))) < 1e-10
    Vh = h.potential(sysd["point_charges"], sysd["point_positions"])
    assert np.max(np.abs(dV.cpu().numpy() - Vh)) < 1e-10 * max(1.0, np.max(np.abs(Vh)))
    h.close()
