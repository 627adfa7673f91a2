"""GPU parity with d shells: every quartet class up to (dd|dd), including the
block-cooperative kernels (total angular momentum 5 to 8), against the
oracle element-wise, and the golden APMO energy whose proton basis
(NAKAI-5-SPD) carries d shells.

Tolerances as in test_gpu_parity: 1e-10 absolute on two-particle / coupling
matrices, 1e-9 on first-quarter tensors; mixed precision 1e-6 Eh on energies.
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


def _dwater2():
    # two waters, a d shell on each oxygen: (dd|dd), (dd|dp), (dp|dd) quartets
    return S.water_cluster(2, seed=3, quantum_protons=False, o_d=True)


def _pair_classes(L, h):
    return h.pair_class_counts(all_pairs=False)


def test_twobody_d_shells_random_density(L, oracle):
    sysd = _dwater2()
    sp = sysd["species"][0]
    rng = np.random.default_rng(31)
    D = _sym(rng, S.nbasis(sp), 0.1)
    h = L.Libint2Interface(sp, 1)
    assert _pair_classes(L, h)[5] > 0          # dd pairs present
    G = h.compute_2body_direct(D, -0.5)
    ref = oracle.two_body_direct(oracle.Basis.from_shells(sp["shells"]), True, D, -0.5)
    assert np.max(np.abs(G - ref)) < TOL_FOCK
    assert h.last_quartets() == oracle.last_quartet_count()
    cq = np.array(h.last_class_quartets()).reshape(L.NPC, L.NPC)
    assert cq[5, 5] > 0 and cq[5, 4] > 0       # cooperative classes evaluated
    h.close()


def test_twobody_d_shells_scf_density(L, oracle):
    sysd = S.water(d_shell=True)
    sp = sysd["species"][0]
    D = oracle.scf(oracle.from_plain(sysd), tol_energy=1e-9, tol_density=1e-6).densities[0]
    h = L.Libint2Interface(sp, 1)
    G = h.compute_2body_direct(D, -0.5)
    ref = oracle.two_body_direct(oracle.Basis.from_shells(sp["shells"]), True, D, -0.5)
    assert np.max(np.abs(G - ref)) < TOL_FOCK
    h.close()


def test_golden_apmo_proton_d_shells(L, oracle, golden):
    """NAKAI-5-SPD protons: two-particle (unscreened) and coupling builds."""
    sysd = GS.h2o_apmo(golden)
    e, p = sysd["species"][0], sysd["species"][1]
    rng = np.random.default_rng(32)
    Dp = _sym(rng, S.nbasis(p), 0.2)
    he = L.Libint2Interface(e, 1)
    hp = L.Libint2Interface(p, 2)
    Gp = hp.compute_2body_direct(Dp, -1.0)
    ref = oracle.two_body_direct(oracle.Basis.from_shells(p["shells"]), False, Dp, -1.0)
    assert np.max(np.abs(Gp - ref)) < TOL_FOCK
    B = he.compute_coupling_direct(hp, Dp)
    ref = oracle.coupling_direct(oracle.Basis.from_shells(e["shells"]), 1,
                                 oracle.Basis.from_shells(p["shells"]), 2, Dp)
    assert np.max(np.abs(B - ref)) < TOL_FOCK
    he.close(); hp.close()


def test_coupling_generic_classes(L, oracle):
    """(dd|dd) coupling quartets: d-shell electrons against NAKAI-5-SPD-like
    proton shells (the d shells of both species meet in the cooperative kernel)."""
    sysd = S.water(d_shell=True)
    e = sysd["species"][0]
    O = e["shells"][0][3]
    pshells = [(2, [1.5], [1.0], list(O)), (1, [3.0], [1.0], list(O)), (0, [8.0], [1.0], list(O))]
    p = S.proton_species(pshells, 1, name="H-D_1")
    rng = np.random.default_rng(33)
    Dp = _sym(rng, S.nbasis(p), 0.2)
    De = _sym(rng, S.nbasis(e), 0.2)
    he = L.Libint2Interface(e, 1)
    hp = L.Libint2Interface(p, 2)
    for A, idA, B_, idB, D in ((he, 1, hp, 2, Dp), (hp, 2, he, 1, De)):
        got = A.compute_coupling_direct(B_, D)
        sa = e if A is he else p
        sb = p if A is he else e
        ref = oracle.coupling_direct(oracle.Basis.from_shells(sa["shells"]), idA,
                                     oracle.Basis.from_shells(sb["shells"]), idB, D)
        assert np.max(np.abs(got - ref)) < TOL_FOCK
    he.close(); hp.close()


def test_first_quarter_d_shells(L, oracle):
    sysd = S.water(d_shell=True)
    sp = sysd["species"][0]
    n = S.nbasis(sp)
    rng = np.random.default_rng(34)
    C = rng.normal(size=(n, n))
    D = np.ones((n, n))
    h = L.Libint2Interface(sp, 1)
    for pidx in (0, n - 1):
        A = h.compute_2body_directIT(D, C, pidx)
        ref = oracle.two_body_directIT(oracle.Basis.from_shells(sp["shells"]), True, D, C, pidx)
        assert np.max(np.abs(A - ref)) < TOL_IT
    h.close()


def test_first_quarter_coupling_d_shells(L, oracle, golden):
    sysd = GS.h2o_apmo(golden)
    e, p = sysd["species"][0], sysd["species"][1]
    ne = S.nbasis(e)
    rng = np.random.default_rng(35)
    C = rng.normal(size=(ne, ne))
    he = L.Libint2Interface(e, 1)
    hp = L.Libint2Interface(p, 2)
    A = he.compute_coupling_directIT(hp, C, 3)
    ref = oracle.coupling_directIT(oracle.Basis.from_shells(e["shells"]), 1,
                                   oracle.Basis.from_shells(p["shells"]), 2, C, 3)
    assert np.max(np.abs(A - ref)) < TOL_IT
    he.close(); hp.close()


def test_mixed_precision_d_shells_close_to_fp64(L):
    """FP32 templated classes + FP64 cooperative classes under the split."""
    torch = pytest.importorskip("torch")
    sysd = _dwater2()
    sp = sysd["species"][0]
    rng = np.random.default_rng(36)
    D = _sym(rng, S.nbasis(sp), 0.02)
    h = L.Libint2Interface(sp, 1)
    dD = torch.tensor(D, device="cuda")
    G64 = torch.empty_like(dD)
    G32 = torch.empty_like(dD)
    st = torch.cuda.current_stream().cuda_stream
    h.twobody_device(dD.data_ptr(), G64.data_ptr(), -0.5, stream=st)
    h.twobody_device(dD.data_ptr(), G32.data_ptr(), -0.5, precision=1, split=1e-4, stream=st)
    torch.cuda.synchronize()
    a, b = G64.cpu().numpy(), G32.cpu().numpy()
    assert np.max(np.abs(a - b)) < 1e-5 * max(1.0, np.max(np.abs(a)))
    h.close()


def test_noalloc_d_shells_match(L):
    """The allocation-free entry serves d-shell species too (the cooperative
    kernels keep their work arrays in shared memory)."""
    torch = pytest.importorskip("torch")
    sp = _dwater2()["species"][0]
    h = L.Libint2Interface(sp, 1)
    h.init_2body_ints()
    n = h.nbasis
    rng = np.random.default_rng(37)
    dD = torch.tensor(_sym(rng, n, 0.1), device="cuda")
    dG = torch.zeros_like(dD)
    dG2 = torch.zeros_like(dD)
    st = torch.cuda.current_stream().cuda_stream
    rc = L.lib().LowdinGB300_twobody_device_noalloc(h.h, dD.data_ptr(), dG.data_ptr(), -0.5, 0, 0.0, st)
    assert rc == 0, L.last_error()
    h.twobody_device(dD.data_ptr(), dG2.data_ptr(), -0.5, stream=st)
    torch.cuda.synchronize()
    assert float((dG - dG2).abs().max()) < 1e-12
    h.close()


def test_golden_apmo_energy_on_gpu(golden):
    """test/H2O.APMO.MP2 RHF-APMO energy through the device SCF (NAKAI-5-SPD)."""
    from openlowdin_gb300 import scf
    sysd = GS.h2o_apmo(golden)
    ref = golden["values"]["H2O.APMO.MP2"]["HF energy"]
    s = scf.DeviceSCF(sysd)
    r = s.solve(tol_energy=1e-10, tol_density=1e-8)
    s.close()
    assert r.converged
    assert abs(r.energy - ref[0]) <= ref[1], r.energy


def test_batched_scf_d_shells_matches_oracle(oracle):
    from openlowdin_gb300.batch_scf import BatchSCF
    mols = [S.water(d_shell=True), S.water()]
    s = BatchSCF(mols)
    res = s.solve(tol_energy=1e-10, tol_density=1e-8)
    s.close()
    for m, r in zip(mols, res):
        ro = oracle.scf(oracle.from_plain(m), tol_energy=1e-10, tol_density=1e-8)
        assert r.converged
        assert abs(r.energy - ro.energy) < 1e-8
