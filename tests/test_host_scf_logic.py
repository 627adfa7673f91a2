"""HostSCF's control flow on the CPU.

HostSCF calls the library every iteration: host-side one-body matrices
(overlap, kinetic, point-charge and Gaussian-fit potentials, which run here
without a GPU) and device-side two-particle, coupling and G12 builds.  These
tests keep the host-side calls real and replace the device-side calls of the
handles with the oracle's restatements (which the GPU tests compare the device
builds against), so the driver's own logic -- damping and DIIS, the reference's
stopping rules, G12 wiring, external potentials, the mixed-precision
bookkeeping and its FP64 check -- is exercised and pinned to the reference's
golden values without a GPU.
"""
import numpy as np
import pytest

from tests import golden_systems as GS
from tests.test_oracle import DAMPING_CASES, SCHEME_CASES, scheme_tolerances


@pytest.fixture
def scf(monkeypatch, oracle):
    from openlowdin_gb300 import build, lint, scf
    build.build()
    L = lint.Libint2Interface
    init = L.__init__
    calls = {"precision": []}

    def fake_init(self, sp, sid, *a, **k):
        init(self, sp, sid, *a, **k)
        self._basis, self._sid, self._el = oracle.Basis.from_shells(sp["shells"]), sid, sp["is_electron"]

    monkeypatch.setattr(L, "__init__", fake_init)
    monkeypatch.setattr(L, "init_2body_ints", lambda self: None)
    monkeypatch.setattr(L, "compute_2body_direct",
                        lambda self, D, f: oracle.two_body_direct(self._basis, self._el, D, f))
    monkeypatch.setattr(L, "compute_coupling_direct",
                        lambda self, o, D: oracle.coupling_direct(self._basis, self._sid, o._basis, o._sid, D))
    monkeypatch.setattr(L, "compute_g12_direct",
                        lambda self, D, f, c, g: oracle.g12_direct(self._basis, D, f, c, g))
    monkeypatch.setattr(L, "compute_g12inter_direct",
                        lambda self, o, D, c, g: oracle.g12inter_direct(self._basis, self._sid, o._basis, o._sid,
                                                                        D, c, g))
    monkeypatch.setattr(L, "last_quartets", lambda self: oracle.last_quartet_count())
    monkeypatch.setattr(L, "set_precision", lambda self, p, split: calls["precision"].append(p))
    scf.calls = calls
    return scf


@pytest.mark.parametrize("case", DAMPING_CASES, ids=[c[1] for c in DAMPING_CASES])
def test_damping_stops_where_the_reference_did(scf, golden, case):
    build, test, te, td = case
    s = scf.HostSCF(getattr(GS, build)(golden), convergence="damping")
    r = s.solve(tol_energy=te, tol_density=td, max_iter=3000, density_sum=True)
    s.close()
    ref = golden["values"][test]
    assert r.converged and abs(r.energy - ref["HF energy"][0]) < 1e-9
    assert abs(r.iterations - ref["Iterations"][0]) <= 5


@pytest.mark.parametrize("case", SCHEME_CASES, ids=[c[1] for c in SCHEME_CASES])
def test_nested_schemes_stop_where_the_reference_did(scf, oracle, golden, case):
    build, test, scheme, emax, nmax, criterion, total = case
    s = scf.HostSCF(getattr(GS, build)(golden), convergence="damping")
    r = s.solve(max_iter=3000, density_sum=True, scheme=scheme, sub_max=(emax, nmax),
                **scheme_tolerances(oracle, criterion, total))
    s.close()
    ref = golden["values"][test]
    assert r.converged and abs(r.energy - ref["HF energy"][0]) <= ref["HF energy"][1]
    assert abs(r.iterations - ref["Iterations"][0]) <= 2, r.iterations


@pytest.mark.parametrize("test", ["TIP4P-dimer-singlet-direct", "He.POTENTIALS", "He3-C60potential-NOCI"])
def test_fitted_potentials(scf, golden, test):
    if test == "He.POTENTIALS":
        sysd = GS.he_potentials(golden)
    elif "C60" in test:
        sysd = GS.c60_system(golden, test)
    else:
        sysd = GS.g12_system(golden, test)
    s = scf.HostSCF(sysd)
    r = s.solve(tol_energy=1e-11, tol_density=1e-9)
    s.close()
    ref = golden["values"][test]["HF energy"]
    assert r.converged and abs(r.energy - ref[0]) <= ref[1], r.energy


def test_positron_and_uhf_electrons(scf, golden):
    s = scf.HostSCF(GS.psh(golden))
    r = s.solve(tol_energy=1e-11, tol_density=1e-9)
    s.close()
    ref = golden["values"]["PsH.P3"]["HF energy"]
    assert r.converged and abs(r.energy - ref[0]) <= ref[1]


def test_mixed_bookkeeping_and_fp64_check(scf, golden):
    """precision "mixed": the split is switched on for the solve and off for
    the FP64 check; incremental builds G += G[P - P_ref] reproduce the full
    builds, so with exact builds the check agrees to round-off."""
    sysd = GS.h2o_apmo(golden)
    s = scf.HostSCF(sysd, precision="mixed")
    r = s.solve(tol_energy=1e-10, tol_density=1e-8)
    s.close()
    assert r.converged and not r.guard_hit
    assert r.err_vs_fp64 is not None and r.err_vs_fp64 < 1e-9
    assert abs(r.energy - golden["values"]["H2O.APMO.MP2"]["HF energy"][0]) <= 1e-8
    assert scf.calls["precision"][0] == 1 and scf.calls["precision"][-1] == 0


def test_guard_continues_in_fp64(scf, golden):
    """A check that fails the guard sends the solve on in FP64 with a fresh
    history; it still converges to the reference's energy."""
    s = scf.HostSCF(GS.h2o_boa(golden), precision="mixed", guard_energy=-1.0)
    r = s.solve(tol_energy=1e-10, tol_density=1e-8)
    s.close()
    assert r.converged and r.guard_hit
    ref = golden["values"]["H2O.BOA.DIRECT"]["HF energy"]
    assert abs(r.energy - ref[0]) <= ref[1]


def test_invalid_requests_raise(scf, golden):
    tip4p = GS.g12_system(golden, "TIP4P-dimer-singlet-direct")
    with pytest.raises(ValueError, match="G12 systems run in FP64"):
        scf.HostSCF(tip4p, precision="mixed")
    with pytest.raises(ValueError, match="convergence"):
        scf.HostSCF(GS.h2o_boa(golden), convergence="levelshift")
    with pytest.raises(ValueError, match="schemes 0-2"):
        scf.HostSCF(GS.h2o_boa(golden)).solve(scheme=0)
    from openlowdin_gb300.batch_scf import BatchSCF
    with pytest.raises(ValueError, match="HostSCF only"):
        BatchSCF([tip4p])


def test_damped_fock_rules():
    """The damping step: undamped when the predicted change does not call for
    it, otherwise both kept matrices move by dE / dEF."""
    from openlowdin_gb300.scf import damped_fock
    rng = np.random.default_rng(3)
    sym = lambda: (lambda a: a + a.T)(rng.normal(size=(4, 4)))
    F0, P0, F, P = sym(), sym(), sym(), sym()
    Fd, (F1, P1) = damped_fock(F, P, (F0, P0))
    dP = P - P0
    dE, dEF = -0.5 * np.sum(F0 * dP), np.sum((F - F0) * dP)
    if dEF <= dE:
        assert Fd is F and np.array_equal(F1, F) and np.array_equal(P1, P)
    else:
        w = dE / dEF
        assert np.allclose(Fd, F0 + w * (F - F0)) and np.allclose(P1, P0 + w * (P - P0))
    # no change of the density: undamped
    Fd, (F1, P1) = damped_fock(F, P0.copy(), (F0, P0))
    assert Fd is F
