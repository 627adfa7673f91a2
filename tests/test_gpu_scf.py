"""SCF drivers on the GPU library against the oracle and the golden values."""
import numpy as np
import pytest

from openlowdin_gb300 import systems as S
from tests import golden_systems as GS

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scf():
    from openlowdin_gb300 import build, scf
    build.build()
    return scf


def test_host_and_device_scf_golden_h2o(scf, golden):
    """test/H2O.BOA.DIRECT.py: -76.008843007734 Eh within 1e-8."""
    sysd = GS.h2o_boa(golden)
    ref = golden["values"]["H2O.BOA.DIRECT"]["HF energy"]
    for cls in (scf.HostSCF, scf.DeviceSCF):
        s = cls(sysd)
        r = s.solve(tol_energy=1e-10, tol_density=1e-8)
        s.close()
        assert r.converged
        assert abs(r.energy - ref[0]) <= ref[1], (cls.__name__, r.energy)


def test_device_scf_water_matches_oracle(scf, oracle):
    sysd = S.water()
    ro = oracle.scf(oracle.from_plain(sysd), tol_energy=1e-10, tol_density=1e-8)
    s = scf.DeviceSCF(sysd)
    r = s.solve(tol_energy=1e-10, tol_density=1e-8)
    s.close()
    assert abs(r.energy - ro.energy) < 1e-8


def test_apmo_water_plain_and_mixed(scf, oracle):
    """Coupled electron / quantum-proton SCF: plain matches the oracle to 1e-8,
    mixed FP32/FP64 integrals stay within 1e-6 Eh."""
    sysd = S.water_cluster(1, seed=0, quantum_protons=True, place=False)
    ro = oracle.scf(oracle.from_plain(sysd), tol_energy=1e-10, tol_density=1e-8)
    s = scf.DeviceSCF(sysd)
    r = s.solve(tol_energy=1e-10, tol_density=1e-8)
    s.close()
    assert abs(r.energy - ro.energy) < 1e-8
    s = scf.DeviceSCF(sysd, precision="mixed")
    rm = s.solve(tol_energy=1e-10, tol_density=1e-8)
    s.close()
    assert abs(rm.energy - ro.energy) < 1e-6


def test_batch_fock_matches_handle_calls(scf):
    """One batched build == the per-species reference-shaped calls."""
    torch = pytest.importorskip("torch")
    from openlowdin_gb300 import lint
    sysd = S.water_cluster(1, seed=0, quantum_protons=True, place=False)   # e- + 2 proton species
    sps = sysd["species"]
    hs = [lint.Libint2Interface(sp, k + 1) for k, sp in enumerate(sps)]
    rng = np.random.default_rng(21)
    Ph, P, G, J = [], [], [], []
    for h in hs:
        X = rng.normal(size=(h.nbasis, h.nbasis)) * 0.2
        Ph.append(X + X.T)
        P.append(torch.tensor(Ph[-1], device="cuda"))
        G.append(torch.zeros_like(P[-1]))
        J.append(torch.zeros_like(P[-1]))
    two = [1, 1, 1]   # exercise the proton two-particle path too
    b = lint.Batch()
    b.add_system(hs, [sp["charge"] for sp in sps], [sp["kappa"] / sp["eta"] for sp in sps], two, P, G, J)
    st = torch.cuda.current_stream().cuda_stream
    b.finalize(st)
    b.fock(0, 0.0, st)
    torch.cuda.synchronize()
    for k, sp in enumerate(sps):
        ref = hs[k].compute_2body_direct(Ph[k], sp["kappa"] / sp["eta"]) * sp["charge"] ** 2
        assert np.max(np.abs(G[k].cpu().numpy() - ref)) < 1e-10
        Jref = np.zeros_like(Ph[k])
        for j, o in enumerate(sps):
            if j != k:
                B = hs[k].compute_coupling_direct(hs[j], Ph[j])
                Jref += (np.tril(B) + np.tril(B, -1).T) * sp["charge"] * o["charge"]
        assert np.max(np.abs(J[k].cpu().numpy() - Jref)) < 1e-10
    b.close()
    for h in hs:
        h.close()


def test_batched_scf_matches_oracle_per_molecule(oracle):
    from openlowdin_gb300.batch_scf import BatchSCF
    mols = [S.water(), S.water_cluster(1, seed=0, quantum_protons=True, place=False)]
    s = BatchSCF(mols)
    res = s.solve(tol_energy=1e-10, tol_density=1e-8)
    s.close()
    for m, r in zip(mols, res):
        ro = oracle.scf(oracle.from_plain(m), tol_energy=1e-10, tol_density=1e-8)
        assert r.converged
        assert abs(r.energy - ro.energy) < 1e-8


def test_pipelined_halves_match_single_batch():
    """Two halves iterated alternately give the same solves as one batch."""
    from openlowdin_gb300.batch_scf import BatchSCF, PipelinedSCF
    mols = [S.water_cluster(2, seed=i, quantum_protons=True) for i in range(3)] + [S.water()]
    a = BatchSCF(mols)
    ra = a.solve(tol_energy=1e-10, tol_density=1e-8)
    a.close()
    for prec in ("fp64", "mixed"):
        b = PipelinedSCF(mols, precision=prec)
        rb = b.solve(tol_energy=1e-10, tol_density=1e-8)
        b.close()
        for x, y in zip(ra, rb):
            assert y.converged
            assert abs(x.energy - y.energy) < (1e-9 if prec == "fp64" else 1e-6)


def test_batch_fock_graph_replay_matches_eager(scf):
    """The captured CUDA graph of a batched build gives the eager launches' results."""
    torch = pytest.importorskip("torch")
    from openlowdin_gb300 import lint
    sysd = S.water_cluster(2, seed=4, quantum_protons=True)
    sps = sysd["species"]
    rng = np.random.default_rng(51)
    out = {}
    for graph in (True, False):
        hs = [lint.Libint2Interface(sp, k + 1) for k, sp in enumerate(sps)]
        P = [torch.zeros((h.nbasis, h.nbasis), dtype=torch.float64, device="cuda") for h in hs]
        G = [torch.zeros_like(p) for p in P]
        J = [torch.zeros_like(p) for p in P]
        b = lint.Batch()
        b.use_graph(graph)
        b.add_system(hs, [sp["charge"] for sp in sps], [sp["kappa"] / sp["eta"] for sp in sps],
                     [1] * len(sps), P, G, J)
        st = torch.cuda.current_stream().cuda_stream
        b.finalize(st)
        res = []
        rr = np.random.default_rng(52)
        for it in range(4):
            for p in P:
                X = rr.normal(size=p.shape) * 0.1
                p.copy_(torch.tensor(X + X.T))
            for prec in (0, 3):
                b.fock(prec, 1e-5, st)
                torch.cuda.synchronize()
                res.append((prec, [g.cpu().numpy().copy() for g in G] + [j.cpu().numpy().copy() for j in J]))
        out[graph] = res
        b.close()
        for h in hs:
            h.close()
    # FP64 builds: same up to the order of FP64 atomics; mixed builds also
    # accumulate FP32 atomics, whose order changes their rounding
    for (prec, a), (_, c) in zip(out[True], out[False]):
        for x, y in zip(a, c):
            assert np.max(np.abs(x - y)) < (1e-10 if prec == 0 else 1e-5)


def test_batch_row_stride_and_active_flags(scf):
    """Species matrices inside larger padded arrays (row stride ld > n) give
    the unpadded build and leave the padding untouched; a system switched off
    with set_active launches no quartets and keeps its outputs."""
    torch = pytest.importorskip("torch")
    from openlowdin_gb300 import lint
    mols = [S.water_cluster(1, seed=0, quantum_protons=True, place=False), S.water()]
    rng = np.random.default_rng(61)
    st = torch.cuda.current_stream().cuda_stream
    runs = {}
    for padded in (False, True):
        b = lint.Batch()
        keep, outs = [], []
        for m in mols:
            sps = m["species"]
            hs = [lint.Libint2Interface(sp, k + 1) for k, sp in enumerate(sps)]
            P, G, J, ld = [], [], [], []
            for h in hs:
                n = h.nbasis
                L = n + 7 if padded else n
                X = np.random.default_rng(n).normal(size=(n, n)) * 0.2
                Pf = torch.full((L, L), 3.0, dtype=torch.float64, device="cuda")
                Pf[:n, :n] = torch.tensor(X + X.T)
                P.append(Pf)
                G.append(torch.full((L, L), -5.0, dtype=torch.float64, device="cuda"))
                J.append(torch.full((L, L), -5.0, dtype=torch.float64, device="cuda"))
                ld.append(L)
            b.add_system(hs, [sp["charge"] for sp in sps], [sp["kappa"] / sp["eta"] for sp in sps],
                         [1 if sp["n_particles"] > 1 else 0 for sp in sps], P, G, J, ld=ld)
            keep.append(hs)
            outs.append((hs, G, J))
        b.finalize(st)
        b.fock(0, 0.0, st)
        q_all = b.quartets(st).sum()
        torch.cuda.synchronize()
        res = [[(g[:h.nbasis, :h.nbasis].cpu().numpy().copy(), j[:h.nbasis, :h.nbasis].cpu().numpy().copy())
                for h, g, j in zip(*o)] for o in outs]
        if padded:
            for hs, G, J in outs:
                for h, g, j in zip(hs, G, J):
                    n = h.nbasis
                    assert torch.all(g[n:, :] == -5.0) and torch.all(g[:, n:] == -5.0)
                    assert torch.all(j[n:, :] == -5.0) and torch.all(j[:, n:] == -5.0)
            # switch the second system off: its outputs stay, its quartets go
            for g in outs[1][1]:
                g.fill_(7.0)
            b.set_active([1, 0], st)
            b.fock(0, 0.0, st)
            q_one = b.quartets(st).sum()
            torch.cuda.synchronize()
            assert all(torch.all(g == 7.0) for g in outs[1][1])
            assert 0 < q_one < q_all
            for (h, g, j), (g0, j0) in zip(zip(*outs[0]), res[0]):
                n = h.nbasis
                assert np.max(np.abs(g[:n, :n].cpu().numpy() - g0)) < 1e-12
            b.set_active([1, 1], st)
            b.fock(0, 0.0, st)
            assert b.quartets(st).sum() == q_all
        runs[padded] = res
        b.close()
        for hs in keep:
            for h in hs:
                h.close()
    for a, c in zip(runs[False], runs[True]):
        for (g0, j0), (g1, j1) in zip(a, c):
            assert np.max(np.abs(g0 - g1)) < 1e-11
            assert np.max(np.abs(j0 - j1)) < 1e-11


def test_padded_buckets_match_exact_groups():
    """Molecules of different sizes in padded buckets (per-member sizes and
    occupations, converged members switched off) converge to the energies and
    orbitals of exact-size groups."""
    from openlowdin_gb300.batch_scf import BatchSCF
    mols = [S.chain_molecule(700 + i, n_atoms=3 + i % 4) for i in range(6)]
    mols.append(S.water_cluster(1, seed=0, quantum_protons=True, place=False))
    out = {}
    for bucket in (False, True):
        s = BatchSCF(mols, bucket=bucket)
        if bucket:
            assert any(g.ragged for g in s.groups.values())
        out[bucket] = s.solve(tol_energy=1e-10, tol_density=1e-8)
        s.close()
    for a, b in zip(out[False], out[True]):
        assert a.converged and b.converged
        assert abs(a.energy - b.energy) < 1e-9
        for ea, eb in zip(a.orbital_energies, b.orbital_energies):
            assert ea.shape == eb.shape
            assert np.max(np.abs(ea - eb)) < 1e-6


def test_batch_mixed_fp64_check_and_guard():
    """BatchSCF in mixed precision: every converged system gets an FP64 check
    (its stated error <= 1e-6 Eh, energy within 1e-6 of plain); with every
    quartet forced into FP32 the check fails and the system finishes in FP64
    on the plain energy (the check bar is lowered to 1e-9 Eh so that it fails
    for every molecule, whatever its size)."""
    from openlowdin_gb300 import systems as S
    from openlowdin_gb300.batch_scf import BatchSCF
    mols = [S.chain_for_basis(500 + i, nbf) for i, nbf in enumerate((50, 80, 120))]
    b = BatchSCF(mols, precision="fp64")
    plain = b.solve()
    b.close()
    b = BatchSCF(mols, precision="mixed")
    mixed = b.solve()
    b.close()
    for p, m in zip(plain, mixed):
        assert p.converged and m.converged and not m.guard_hit
        assert m.err_vs_fp64 is not None and m.err_vs_fp64 <= 1e-6
        assert abs(m.energy - p.energy) < 1e-6
    # every quartet in FP32 and a check bar (1e-9 Eh) far below its error
    b = BatchSCF(mols, precision="mixed", split=1e30, guard_energy=1e-9)
    forced = b.solve()
    b.close()
    for p, f in zip(plain, forced):
        assert f.converged and f.guard_hit and f.err_vs_fp64 == 0.0
        assert abs(f.energy - p.energy) < 1e-8


def test_host_abi_mixed_precision_matches_plain(scf):
    """The reference-shaped host-buffer calls with the handle's FP32/FP64 split
    (LowdinGB300_set_precision) and incremental builds: within 1e-6 Eh of the
    plain FP64 solve, with the FP64 check's stated error."""
    sysd = S.chain_for_basis(10_003, 120)
    s = scf.HostSCF(sysd)
    rp = s.solve(tol_energy=1e-10, tol_density=1e-8)
    s.close()
    s = scf.HostSCF(sysd, precision="mixed")
    rm = s.solve(tol_energy=1e-10, tol_density=1e-8)
    s.close()
    assert rp.converged and rm.converged
    assert rm.err_vs_fp64 is not None and rm.err_vs_fp64 <= 1e-6
    assert not rm.guard_hit
    assert abs(rm.energy - rp.energy) <= 1e-6


def test_host_abi_mixed_guard_continues_in_fp64(scf):
    """A guard bar no mixed build meets: the check fires and the solve ends in
    FP64 on the plain energy."""
    sysd = S.water()
    s = scf.HostSCF(sysd)
    rp = s.solve(tol_energy=1e-10, tol_density=1e-8)
    s.close()
    s = scf.HostSCF(sysd, precision="mixed", split=0.5, guard_energy=1e-15)
    rm = s.solve(tol_energy=1e-10, tol_density=1e-8)
    s.close()
    assert rm.converged and rm.guard_hit
    assert abs(rm.energy - rp.energy) <= 1e-8


def test_set_precision_rejects_bad_arguments(scf):
    from openlowdin_gb300 import lint
    h = lint.Libint2Interface(S.water()["species"][0], 1)
    with pytest.raises(lint.LowdinGB300Error, match="precision"):
        h.set_precision(3)
    with pytest.raises(lint.LowdinGB300Error, match="split"):
        h.set_precision(1, 2.0)
    h.close()
