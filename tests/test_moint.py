"""The moint.dat layout (TransformIntegralsC.f90:531-654 writer,
ReadTransformedIntegrals.f90:225-233 reader): the library's record writer on
the host, and the MP2 entries restated from the oracle against the golden
MP2 energy."""
import os

import numpy as np
import pytest

from openlowdin_gb300 import lint
from openlowdin_gb300 import moint as M
from tests import golden_systems as GS


@pytest.fixture(scope="module")
def built():
    from openlowdin_gb300 import build
    build.build()
    return lint.lib()


def _entries(n, seed=0):
    rng = np.random.default_rng(seed)
    return [rng.integers(1, 60, n).astype(np.int32) for _ in range(4)] + [rng.normal(size=n)]


@pytest.mark.parametrize("count", [0, 3, 7, 14, 17])
def test_record_layout_and_reader(built, tmp_path, count):
    """Stacks of 7: full stacks are records of their own, the last record
    carries p = -1 after its entries (a record of the marker alone when the
    entries fill whole stacks), every record framed by its byte length."""
    stack = 7
    e = _entries(count, seed=count)
    path = str(tmp_path / "Emoint.dat")
    lint.moint_write(path, *e, stack_size=stack)
    raw = open(path, "rb").read()
    nrec = count // stack + 1
    rec = stack * 24
    assert len(raw) == nrec * (rec + 8)
    for k in range(nrec):
        base = k * (rec + 8)
        assert np.frombuffer(raw, np.int32, 1, base)[0] == rec
        assert np.frombuffer(raw, np.int32, 1, base + 4 + rec)[0] == rec
    last = (nrec - 1) * (rec + 8) + 4
    p_last = np.frombuffer(raw, np.int32, stack, last)
    assert p_last[count % stack] == -1
    assert np.all(p_last[count % stack + 1:] == 0)
    got = M.read_moint(path, stack)
    for x, y in zip(got, e):
        assert np.array_equal(x, y)


def test_reader_rejects_a_file_without_end_marker(built, tmp_path):
    path = str(tmp_path / "Emoint.dat")
    lint.moint_write(path, *_entries(7), stack_size=7)
    raw = open(path, "rb").read()
    open(path, "wb").write(raw[:7 * 24 + 8])   # drop the marker record
    with pytest.raises(ValueError):
        M.read_moint(path, 7)


def test_mp2_entries_reproduce_golden_energy(oracle, golden):
    """(ia|jb) of the golden water from the oracle's full tensor, written in
    the transform's order with the 1e-10 cut, give the oracle's MP2 energy
    and the golden MP2 total energy."""
    sysd = GS.h2o_boa(golden)
    res = oracle.scf(oracle.from_plain(sysd))
    b = oracle.Basis.from_shells(sysd["species"][0]["shells"])
    C, eps = res.coefficients[0], res.orbital_energies[0]
    eri = oracle.eri_full(b)
    nocc, n = 5, b.nbf
    Co, Cv = C[:, :nocc], C[:, nocc:]
    iajb = np.einsum("pqrs,pi,qa,rj,sb->iajb", eri, Co, Cv, Co, Cv, optimize=True)
    ent = M.mp2_entries(iajb, 0, nocc)
    # the order: p, then q, then r >= p, then s (s >= q when r == p)
    key = np.stack(ent[:4], 1).astype(np.int64)
    assert np.all(key[:, 2] >= key[:, 0])
    assert np.all((key[:, 2] > key[:, 0]) | (key[:, 3] >= key[:, 1]))
    order = np.lexsort(key[:, ::-1].T)
    assert np.array_equal(order, np.arange(len(order)))
    e2 = M.mp2_energy(ent, eps, nocc, 0, n)
    assert abs(e2 - oracle.rmp2(eri, C, eps, nocc)) < 1e-12
    g = golden["values"]["H2O.BOA.MP2.DIRECT"]["MP2 energy"]
    assert abs(res.energy + e2 - g[0]) <= g[1]


def test_writer_reports_bad_arguments(built, tmp_path):
    e = _entries(3)
    with pytest.raises(lint.LowdinGB300Error):
        lint.moint_write(str(tmp_path / "x.dat"), *e, stack_size=0)
    with pytest.raises(lint.LowdinGB300Error):
        lint.moint_write(str(tmp_path / "no_such_dir" / "x.dat"), *e, stack_size=7)
    lint.lib().LowdinGB300_clear_error()


def test_two_species_entries_reproduce_coupling_mp2(oracle, golden, built, tmp_path):
    """Inter-species (ia|jb) of the golden APMO water (electrons x first proton
    species) from the oracle's restated first quarter, written through the
    library's record writer and read back, give the oracle's inter-species
    MP2 term."""
    sysd = GS.h2o_apmo(golden)
    sysO = oracle.from_plain(sysd)
    res = oracle.scf(sysO)
    A, B = sysO.species[0], sysO.species[1]
    CA, CB = res.coefficients[0], res.coefficients[1]
    oA, oB = A.n_occ, B.n_occ
    P, Q, R, S_, V = [], [], [], [], []
    for i in range(oA):
        Ai = oracle.coupling_directIT(A.basis, 1, B.basis, 2, np.ascontiguousarray(CA.T), i)
        Mi = np.einsum("nls,na,lj,sb->ajb", Ai, CA[:, oA:], CB[:, :oB], CB[:, oB:], optimize=True)
        for a, j, b in zip(*np.nonzero(np.abs(Mi) > 1e-10)):
            P.append(i + 1); Q.append(oA + a + 1); R.append(j + 1); S_.append(oB + b + 1); V.append(Mi[a, j, b])
    path = str(tmp_path / "E-.H_1moint.dat")
    lint.moint_write(path, P, Q, R, S_, V, stack_size=300)
    ent = M.read_moint(path, 300)
    factor = A.eta * B.eta * (A.charge * B.charge) ** 2
    e = M.mp2_coupling_energy(ent, res.orbital_energies[0], res.orbital_energies[1], factor)
    ref = A.eta * B.eta * oracle.mp2_coupling_direct(A.basis, 1, CA, res.orbital_energies[0], oA, 0, B.basis, 2, CB,
                                                     res.orbital_energies[1], oB, 0, A.charge * B.charge)
    assert abs(e - ref) < 1e-12 * max(1.0, abs(ref))
