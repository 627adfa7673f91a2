"""GPU parity with f shells (l = 3): the quartet classes with an f shell run on
the block-cooperative kernels, the largest ones ((ff|fd), (ff|ff)) with their
work arrays in global scratch.  Checked element-wise against the oracle (whose
primitive integrals reach l = 4 and are pinned to the reference's own Rys
code) and against the golden energies of the reference's test/HF.APMO
(cc-pVTZ electrons with an f shell on F, DZSPDN quantum proton).

Tolerances: 1e-10 absolute on two-particle / coupling / geminal matrices and
one-electron matrices, 1e-9 on first-quarter tensors; the checker's 1e-7 Eh
on the HF energy and 1e-5 Eh on the MP2 energy.
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


def _sym(rng, n, scale=0.2):
    X = rng.normal(size=(n, n)) * scale
    return X + X.T


def _two_f_centres():
    # two centres with s, p, d and f shells: every class up to (ff|ff),
    # (ff|ff) and (ff|fd) on global scratch, both same-centre and two-centre
    A, B = [0.0, 0.0, 0.0], [0.0, 0.9, 1.3]
    sh = []
    for c in (A, B):
        sh += [(0, [3.0, 0.6], [0.4, 0.7], c), (1, [1.1], [1.0], c), (2, [0.9], [1.0], c), (3, [1.3], [1.0], c)]
    return S.electron_species(sh, 6)


def test_twobody_f_shells_every_class(L, oracle):
    sp = _two_f_centres()
    D = _sym(np.random.default_rng(51), S.nbasis(sp))
    h = L.Libint2Interface(sp, 1)
    assert h.pair_class_counts(all_pairs=False)[9] > 0          # ff pairs present
    G = h.compute_2body_direct(D, -0.5)
    ref = oracle.two_body_direct(oracle.Basis.from_shells(sp["shells"]), True, D, -0.5)
    assert np.max(np.abs(G - ref)) < TOL_FOCK
    assert h.last_quartets() == oracle.last_quartet_count()
    cq = np.array(h.last_class_quartets()).reshape(L.NPC, L.NPC)
    assert cq[9, 9] > 0 and cq[9, 8] > 0
    h.close()


def test_golden_hf_apmo_matrices(L, oracle, golden):
    """test/HF.APMO species: cc-pVTZ electrons (contracted, f on F) and the
    DZSPDN proton: two-particle, both coupling directions, one-electron."""
    sysd = GS.hf_apmo(golden)
    e, p = sysd["species"]
    be, bp = oracle.Basis.from_shells(e["shells"]), oracle.Basis.from_shells(p["shells"])
    rng = np.random.default_rng(52)
    De, Dp = _sym(rng, be.nbf, 0.1), _sym(rng, bp.nbf, 0.1)
    he, hp = L.Libint2Interface(e, 1), L.Libint2Interface(p, 2)
    G = he.compute_2body_direct(De, -0.5)
    assert np.max(np.abs(G - oracle.two_body_direct(be, True, De, -0.5))) < TOL_FOCK
    B = he.compute_coupling_direct(hp, Dp)
    assert np.max(np.abs(B - oracle.coupling_direct(be, 1, bp, 2, Dp))) < TOL_FOCK
    B = hp.compute_coupling_direct(he, De)
    assert np.max(np.abs(B - oracle.coupling_direct(bp, 2, be, 1, De))) < TOL_FOCK
    Sm, T = oracle.overlap_kinetic(be)
    assert np.max(np.abs(he.one_body(1) - Sm)) < TOL_FOCK
    assert np.max(np.abs(he.one_body(2) - T)) < TOL_FOCK
    V = oracle.potential(be, sysd["point_charges"], sysd["point_positions"])
    assert np.max(np.abs(he.potential(sysd["point_charges"], sysd["point_positions"]) - V)) < TOL_FOCK
    he.close(); hp.close()


def test_one_body_device_f_shells(L, oracle):
    torch = pytest.importorskip("torch")
    sp = _two_f_centres()
    b = oracle.Basis.from_shells(sp["shells"])
    Z, R = [3.0, 1.0], [[0.0, 0.0, 0.2], [0.5, 0.4, 1.0]]
    h = L.Libint2Interface(sp, 1)
    n = h.nbasis
    dS, dT, dV = (torch.empty((n, n), dtype=torch.float64, device="cuda") for _ in range(3))
    h.one_body_device(Z, R, dS.data_ptr(), dT.data_ptr(), dV.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    Sm, T = oracle.overlap_kinetic(b)
    V = oracle.potential(b, Z, R)
    for got, ref in ((dS, Sm), (dT, T), (dV, V)):
        assert np.max(np.abs(got.cpu().numpy() - ref)) < TOL_FOCK
    h.close()


def test_first_quarter_f_shells(L, oracle):
    sp = _two_f_centres()
    n = S.nbasis(sp)
    rng = np.random.default_rng(53)
    C = rng.normal(size=(n, n))
    D = np.ones((n, n))
    h = L.Libint2Interface(sp, 1)
    A = h.compute_2body_directIT(D, C, 2)
    ref = oracle.two_body_directIT(oracle.Basis.from_shells(sp["shells"]), True, D, C, 2)
    assert np.max(np.abs(A - ref)) < TOL_IT
    h.close()


def test_geminal_f_shells(L, oracle):
    sp = _two_f_centres()
    b = oracle.Basis.from_shells(sp["shells"])
    D = _sym(np.random.default_rng(54), b.nbf)
    coef, expo = [0.3, -1.1, 2.0], [0.0, 0.5, 3.0]
    h = L.Libint2Interface(sp, 1)
    G = h.compute_g12_direct(D, -1.0, coef, expo)
    assert np.max(np.abs(G - oracle.g12_direct(b, D, -1.0, coef, expo))) < TOL_FOCK
    h.close()


def test_noalloc_rejects_f_shells(L):
    torch = pytest.importorskip("torch")
    sp = _two_f_centres()
    h = L.Libint2Interface(sp, 1)
    h.init_2body_ints()
    dD = torch.zeros((h.nbasis, h.nbasis), dtype=torch.float64, device="cuda")
    dG = torch.zeros_like(dD)
    rc = L.lib().LowdinGB300_twobody_device_noalloc(h.h, dD.data_ptr(), dG.data_ptr(), -0.5, 0, 0.0,
                                                    torch.cuda.current_stream().cuda_stream)
    assert rc == -1 and "above d" in L.last_error()
    L.lib().LowdinGB300_clear_error()
    h.close()


def test_golden_hf_apmo_energies(L, oracle, golden):
    """test/HF.APMO: RHF-APMO energy (checker tolerance 1e-7 Eh) through the
    reference-shaped host calls and the device SCF, and the APMO-MP2 energy
    (1e-5 Eh) through the device transform on the device SCF's orbitals."""
    from openlowdin_gb300 import scf
    from tests.test_gpu_mp2 import _apmo_device_mp2
    sysd = GS.hf_apmo(golden)
    ref = golden["values"]["HF.APMO"]
    for cls in (scf.HostSCF, scf.DeviceSCF):
        s = cls(sysd)
        r = s.solve(tol_energy=1e-10, tol_density=1e-8)
        s.close()
        assert r.converged, cls.__name__
        assert abs(r.energy - ref["HF energy"][0]) <= 1e-7, (cls.__name__, r.energy)
    res = oracle.scf(oracle.from_plain(sysd), tol_energy=1e-11, tol_density=1e-9)
    total = res.energy + sum(_apmo_device_mp2(L, sysd, res, 0).values())
    assert abs(total - ref["MP2 energy"][0]) <= ref["MP2 energy"][1], total
