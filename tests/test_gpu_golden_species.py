"""GPU runs of the reference's golden inputs with species beyond electrons and
single protons: one species of two or three protons (test/H2O.APMO.iter3,
test/NH3.APMO.convBoth), a
positron species (test/PsH.P3) and electrons interacting only through fitted
Gaussian potentials (test/He.POTENTIALS), through the reference-shaped host
calls (HostSCF) and, for PsH.P3, the device-resident driver too.  Energies
against the checkers' HF values (1e-8 Eh) and against the oracle."""
import pytest

from tests import golden_systems as GS
from tests.test_oracle import DAMPING_CASES, SCHEME_CASES, scheme_tolerances

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scf():
    from openlowdin_gb300 import build, scf
    build.build()
    return scf


@pytest.mark.parametrize("case", DAMPING_CASES, ids=[c[1] for c in DAMPING_CASES])
def test_multi_proton_species_with_the_reference_damping(scf, golden, case):
    """Damping (the reference's default method) under each input's own
    criteria: every iteration's two-particle matrices of the electrons and of
    the proton species and both couplings come from the library; the solve
    stops where the reference's did (its recorded iteration count) at its
    energy."""
    build, test, te, td = case
    sysd = getattr(GS, build)(golden)
    s = scf.HostSCF(sysd, convergence="damping")
    r = s.solve(tol_energy=te, tol_density=td, max_iter=3000, density_sum=True)
    s.close()
    ref = golden["values"][test]
    assert r.converged
    assert abs(r.energy - ref["HF energy"][0]) <= ref["HF energy"][1], r.energy
    assert abs(r.iterations - ref["Iterations"][0]) <= ref["Iterations"][1], r.iterations


def test_positron_species(scf, oracle, golden):
    sysd = GS.psh(golden)
    ref = golden["values"]["PsH.P3"]["HF energy"]
    res = oracle.scf(oracle.from_plain(sysd), tol_energy=1e-11, tol_density=1e-9)
    for cls in (scf.HostSCF, scf.DeviceSCF):
        s = cls(sysd)
        r = s.solve(tol_energy=1e-11, tol_density=1e-9)
        s.close()
        assert r.converged, cls.__name__
        assert abs(r.energy - ref[0]) <= ref[1], (cls.__name__, r.energy)
        assert abs(r.energy - res.energy) < 1e-10, cls.__name__


def test_he_fitted_potentials(scf, oracle, golden):
    sysd = GS.he_potentials(golden)
    s = scf.HostSCF(sysd)
    r = s.solve(tol_energy=1e-11, tol_density=1e-9)
    s.close()
    ref = golden["values"]["He.POTENTIALS"]["HF energy"]
    assert r.converged and abs(r.energy - ref[0]) <= ref[1], r.energy
    res = oracle.scf(oracle.from_plain(sysd), tol_energy=1e-11, tol_density=1e-9)
    assert abs(r.energy - res.energy) < 1e-10


@pytest.mark.parametrize("case", SCHEME_CASES, ids=[c[1] for c in SCHEME_CASES])
def test_nested_iteration_schemes(scf, oracle, golden, case):
    """The reference's iteration schemes 0 and 2 (species iterating on their
    own inside a global iteration, damping, each input's criterion) through
    the library: the checkers' energies (1e-8) and iteration counts (their
    tolerances)."""
    build, test, scheme, emax, nmax, criterion, total = case
    s = scf.HostSCF(getattr(GS, build)(golden), convergence="damping")
    r = s.solve(max_iter=3000, density_sum=True, scheme=scheme, sub_max=(emax, nmax),
                **scheme_tolerances(oracle, criterion, total))
    s.close()
    ref = golden["values"][test]
    assert r.converged
    assert abs(r.energy - ref["HF energy"][0]) <= ref["HF energy"][1], r.energy
    assert abs(r.iterations - ref["Iterations"][0]) <= ref["Iterations"][1], r.iterations
