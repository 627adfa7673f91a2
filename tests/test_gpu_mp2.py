"""Device MP2 (four-index transform + pair energies) against the oracle's
restatement of the reference's DIRECT transform, on the same SCF inputs.

Tolerance: 1e-10 Eh on E_MP2 for the FP64 path (the plain path's MP2 bar is
1e-8 Eh); the golden MP2 total energy within its test tolerance; the
split-BF16 tensor-core path within 1e-6 Eh of the oracle (the per-job bar of
the mixed-precision forms).
"""
import numpy as np
import pytest

from openlowdin_gb300 import systems as S
from tests import golden_systems as GS

pytestmark = pytest.mark.gpu

TOL_E2 = 1e-10
TOL_MIXED = 1e-6


@pytest.fixture(scope="module")
def L():
    from openlowdin_gb300 import build, lint
    build.build()
    return lint


def _device_mp2(L, sp, res, n_occ, n_frozen, precision=0, x_budget_gb=0.0):
    torch = pytest.importorskip("torch")
    h = L.Libint2Interface(sp, 1)
    dD = torch.tensor(res.densities[0], device="cuda")
    dC = torch.tensor(np.ascontiguousarray(res.coefficients[0].T), device="cuda")   # row p = orbital p
    st = torch.cuda.current_stream().cuda_stream
    e2 = h.mp2_direct(dD.data_ptr(), dC.data_ptr(), res.orbital_energies[0], n_occ, n_frozen, precision,
                      x_budget_gb, stream=st)
    h.close()
    return e2


def test_mp2_golden_h2o(L, oracle, golden):
    """test/H2O.BOA.MP2.DIRECT: 6-311G water, MP2 total energy."""
    sysd = GS.h2o_boa(golden)
    res = oracle.scf(oracle.from_plain(sysd))
    sp = sysd["species"][0]
    e2 = _device_mp2(L, sp, res, 5, 0)
    b = oracle.Basis.from_shells(sp["shells"])
    ref = oracle.rmp2_direct(b, res.densities[0], res.coefficients[0], res.orbital_energies[0], 5)
    assert abs(e2 - ref) < TOL_E2
    g = golden["values"]["H2O.BOA.MP2.DIRECT"]["MP2 energy"]
    assert abs(res.energy + e2 - g[0]) <= g[1]


@pytest.mark.parametrize("budget", [0.0, 2e-4])
def test_mp2_d_shells_frozen_core(L, oracle, budget):
    """Water with a d shell on O, frozen O 1s; a tiny budget forces many
    column batches."""
    sysd = S.water(d_shell=True)
    res = oracle.scf(oracle.from_plain(sysd))
    sp = sysd["species"][0]
    e2 = _device_mp2(L, sp, res, 5, 1, x_budget_gb=budget)
    b = oracle.Basis.from_shells(sp["shells"])
    ref = oracle.rmp2_direct(b, res.densities[0], res.coefficients[0], res.orbital_energies[0], 5, 1)
    assert abs(e2 - ref) < TOL_E2
    if budget:
        assert L.lib().LowdinGB300_mp2_last_columns() > 0


def test_mp2_two_waters_d(L, oracle):
    sysd = S.water_cluster(2, seed=3, o_d=True)
    res = oracle.scf(oracle.from_plain(sysd))
    sp = sysd["species"][0]
    e2 = _device_mp2(L, sp, res, 10, 2)
    b = oracle.Basis.from_shells(sp["shells"])
    ref = oracle.rmp2_direct(b, res.densities[0], res.coefficients[0], res.orbital_energies[0], 10, 2)
    assert abs(e2 - ref) < TOL_E2


@pytest.mark.parametrize("budget", [0.0, 2e-4])
def test_mp2_split_bf16_tensor_cores(L, oracle, budget):
    """precision 2: the four contractions on the tensor cores, 3 BF16 pieces
    per operand (6 products) -- within the 1e-6 Eh bar; precision 1 (2
    pieces, 3 products) is reported, its error is ~1e-5 relative."""
    sysd = S.water_cluster(2, seed=3, o_d=True)
    res = oracle.scf(oracle.from_plain(sysd))
    sp = sysd["species"][0]
    b = oracle.Basis.from_shells(sp["shells"])
    ref = oracle.rmp2_direct(b, res.densities[0], res.coefficients[0], res.orbital_energies[0], 10, 2)
    e2 = _device_mp2(L, sp, res, 10, 2, precision=2, x_budget_gb=budget)
    assert abs(e2 - ref) < TOL_MIXED, (e2, ref)
    e2_3term = _device_mp2(L, sp, res, 10, 2, precision=1, x_budget_gb=budget)
    assert abs(e2_3term - ref) < 5e-5 * abs(ref), (e2_3term, ref)


def test_mp2_split_bf16_golden_h2o(L, oracle, golden):
    sysd = GS.h2o_boa(golden)
    res = oracle.scf(oracle.from_plain(sysd))
    sp = sysd["species"][0]
    b = oracle.Basis.from_shells(sp["shells"])
    ref = oracle.rmp2_direct(b, res.densities[0], res.coefficients[0], res.orbital_energies[0], 5)
    e2 = _device_mp2(L, sp, res, 5, 0, precision=2)
    assert abs(e2 - ref) < TOL_MIXED, (e2, ref)


def _apmo_device_mp2(L, sysd, res, precision):
    torch = pytest.importorskip("torch")
    sps = sysd["species"]
    hs = [L.Libint2Interface(sp, k + 1) for k, sp in enumerate(sps)]
    dC = [torch.tensor(np.ascontiguousarray(C.T), device="cuda") for C in res.coefficients]
    st = torch.cuda.current_stream().cuda_stream
    occ = [int(round(sp["n_particles"] * sp["particles_fraction"])) for sp in sps]
    parts = {}
    dD = torch.tensor(res.densities[0], device="cuda")
    parts[(0,)] = hs[0].mp2_direct(dD.data_ptr(), dC[0].data_ptr(), res.orbital_energies[0], occ[0], 0, precision,
                                   stream=st)
    for a in range(len(sps)):
        for b in range(a + 1, len(sps)):
            f = (sps[a]["charge"] * sps[b]["charge"]) ** 2 * sps[a]["eta"] * sps[b]["eta"]
            parts[(a, b)] = hs[a].mp2_coupling(hs[b], dC[a].data_ptr(), dC[b].data_ptr(), res.orbital_energies[a],
                                               res.orbital_energies[b], occ[a], 0, occ[b], 0, f, precision,
                                               stream=st)
    for h in hs:
        h.close()
    return parts


def test_apmo_mp2_golden_and_parts(L, oracle, golden):
    """test/H2O.APMO.MP2: every term against the oracle (FP64 1e-10 Eh, split
    BF16 1e-6 Eh) and the total against the golden MP2 energy."""
    sysd = GS.h2o_apmo(golden)
    sysO = oracle.from_plain(sysd)
    res = oracle.scf(sysO)
    ref = oracle.apmo_mp2(sysO, res)
    for precision, tol in ((0, TOL_E2), (2, TOL_MIXED)):
        parts = _apmo_device_mp2(L, sysd, res, precision)
        for k, v in ref["parts"].items():
            assert abs(parts[k] - v) < tol, (precision, k, parts[k], v)
    total = res.energy + sum(_apmo_device_mp2(L, sysd, res, 0).values())
    for name in ("H2O.APMO.MP2", "H2O.APMO.UMP2.DIRECT"):   # closed-shell UHF: UMP2 = this sum
        g = golden["values"][name]["MP2 energy"]
        assert abs(total - g[0]) <= g[1], name


def test_mp2_coupling_d_shell_species(L, oracle):
    """Coupling MP2 between d-shell electrons and a multi-shell proton species."""
    torch = pytest.importorskip("torch")
    sysd = S.water(d_shell=True)
    e = sysd["species"][0]
    O = e["shells"][0][3]
    p = S.proton_species([(2, [1.5], [1.0], list(O)), (1, [3.0], [1.0], list(O)), (0, [8.0], [1.0], list(O))],
                         1, name="H-D_1")
    rng = np.random.default_rng(41)
    ne, npn = S.nbasis(e), S.nbasis(p)
    Ce = np.linalg.qr(rng.normal(size=(ne, ne)))[0]
    Cp = np.linalg.qr(rng.normal(size=(npn, npn)))[0]
    ee = np.sort(rng.normal(size=ne)) - np.arange(ne)[::-1] * 0.05
    ep = np.sort(rng.normal(size=npn)) + 0.0
    ep[0] -= 5.0
    he, hp = L.Libint2Interface(e, 1), L.Libint2Interface(p, 2)
    dCe = torch.tensor(np.ascontiguousarray(Ce.T), device="cuda")
    dCp = torch.tensor(np.ascontiguousarray(Cp.T), device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    got = he.mp2_coupling(hp, dCe.data_ptr(), dCp.data_ptr(), ee, ep, 5, 1, 1, 0, 2.0, 0, stream=st)
    ref = 2.0 * oracle.mp2_coupling_direct(oracle.Basis.from_shells(e["shells"]), 1, Ce, ee, 5, 1,
                                           oracle.Basis.from_shells(p["shells"]), 2, Cp, ep, 1, 0, -1.0)
    assert abs(got - ref) < 1e-10 * max(1.0, abs(ref))
    he.close(); hp.close()


def test_moint_file_matches_oracle(L, oracle, golden, tmp_path):
    """LowdinGB300_mp2_moint on the golden water: the file holds the oracle's
    (ia|jb) entries in the transform's order (same indices, values within
    1e-10), and its MP2 energy is the device one and the golden one."""
    torch = pytest.importorskip("torch")
    from openlowdin_gb300 import moint as M
    sysd = GS.h2o_boa(golden)
    res = oracle.scf(oracle.from_plain(sysd))
    sp = sysd["species"][0]
    b = oracle.Basis.from_shells(sp["shells"])
    C, eps = res.coefficients[0], res.orbital_energies[0]
    nocc, n = 5, b.nbf
    eri = oracle.eri_full(b)
    iajb = np.einsum("pqrs,pi,qa,rj,sb->iajb", eri, C[:, :nocc], C[:, nocc:], C[:, :nocc], C[:, nocc:],
                     optimize=True)
    ref = M.mp2_entries(iajb, 0, nocc)
    h = L.Libint2Interface(sp, 1)
    dD = torch.tensor(res.densities[0], device="cuda")
    dC = torch.tensor(np.ascontiguousarray(C.T), device="cuda")
    path = str(tmp_path / "Emoint.dat")
    e2, nw = h.mp2_moint(dD.data_ptr(), dC.data_ptr(), eps, nocc, 0, path, stack_size=1000,
                         stream=torch.cuda.current_stream().cuda_stream)
    h.close()
    got = M.read_moint(path, 1000)
    assert nw == len(got[4])
    # entries within 1e-13 relative of the cut may fall on either side of it
    near = lambda v: np.abs(np.abs(v) - 1e-10) < 1e-13
    kg = {tuple(k): v for k, v in zip(np.stack(got[:4], 1).tolist(), got[4])}
    kr = {tuple(k): v for k, v in zip(np.stack(ref[:4], 1).tolist(), ref[4])}
    assert all(near(kr[k]) for k in set(kr) - set(kg))
    assert all(near(kg[k]) for k in set(kg) - set(kr))
    common = [k for k in kr if k in kg]
    assert max(abs(kg[k] - kr[k]) for k in common) < 1e-10
    order = np.lexsort(np.stack(got[:4], 1).astype(np.int64)[:, ::-1].T)
    assert np.array_equal(order, np.arange(len(order)))
    assert abs(M.mp2_energy(got, eps, nocc, 0, n) - e2) < 1e-10
    g = golden["values"]["H2O.BOA.MP2.DIRECT"]["MP2 energy"]
    assert abs(res.energy + e2 - g[0]) <= g[1]


def test_coupling_moint_file_matches_oracle(L, oracle, golden, tmp_path):
    """LowdinGB300_mp2_coupling_moint on the golden APMO water (electrons x
    first proton species): the file holds the oracle's inter-species (ia|jb)
    in the transform's order, and its energy is the device term."""
    torch = pytest.importorskip("torch")
    from openlowdin_gb300 import moint as M
    sysd = GS.h2o_apmo(golden)
    sysO = oracle.from_plain(sysd)
    res = oracle.scf(sysO)
    A, B = sysO.species[0], sysO.species[1]
    CA, CB = res.coefficients[0], res.coefficients[1]
    eA, eB = res.orbital_energies[0], res.orbital_energies[1]
    oA, oB = A.n_occ, B.n_occ
    ref = {}
    for i in range(oA):
        Ai = oracle.coupling_directIT(A.basis, 1, B.basis, 2, np.ascontiguousarray(CA.T), i)
        Mi = np.einsum("nls,na,lj,sb->ajb", Ai, CA[:, oA:], CB[:, :oB], CB[:, oB:], optimize=True)
        for a, j, b in zip(*np.nonzero(np.abs(Mi) > 1e-10)):
            ref[(i + 1, oA + a + 1, j + 1, oB + b + 1)] = Mi[a, j, b]
    factor = A.eta * B.eta * (A.charge * B.charge) ** 2
    he = L.Libint2Interface(sysd["species"][0], 1)
    hp = L.Libint2Interface(sysd["species"][1], 2)
    dCA = torch.tensor(np.ascontiguousarray(CA.T), device="cuda")
    dCB = torch.tensor(np.ascontiguousarray(CB.T), device="cuda")
    path = str(tmp_path / "E-.H_1moint.dat")
    e2, nw = he.mp2_coupling_moint(hp, dCA.data_ptr(), dCB.data_ptr(), eA, eB, oA, 0, oB, 0, factor, path,
                                   stack_size=500, stream=torch.cuda.current_stream().cuda_stream)
    he.close(); hp.close()
    p, q, r, s, v = M.read_moint(path, 500)
    assert nw == len(v)
    key = np.stack([p, q, r, s], 1).astype(np.int64)
    order = np.lexsort(key[:, ::-1].T)
    assert np.array_equal(order, np.arange(len(order)))
    got = {tuple(k): x for k, x in zip(key.tolist(), v)}
    near = lambda x: abs(abs(x) - 1e-10) < 1e-13
    assert all(near(ref[k]) for k in set(ref) - set(got))
    assert all(near(got[k]) for k in set(got) - set(ref))
    assert max(abs(got[k] - ref[k]) for k in got if k in ref) < 1e-10
    den = eA[p - 1] + eB[r - 1] - eA[q - 1] - eB[s - 1]
    assert abs(factor * float(np.sum(v ** 2 / den)) - e2) < 1e-10 * max(1.0, abs(e2))
