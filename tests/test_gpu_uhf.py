"""Open-shell UHF on the GPU library: E-ALPHA / E-BETA species (exchange factor
-1 each) coupled by the inter-species Coulomb matrix, as the reference runs UHF,
against the reference's golden energies (tests/golden/golden.json)."""
import pytest

from tests import golden_systems as GS
from tests.test_oracle import UEN_CASES, UHF_CASES, closed_shell_twin

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scf():
    from openlowdin_gb300 import build, scf
    build.build()
    return scf


@pytest.mark.parametrize("case", UHF_CASES, ids=[c[0] for c in UHF_CASES])
def test_uhf_golden_host_and_device(scf, golden, case):
    test, ebas, pbas, tol = case
    sysd = GS.uhf_system(golden, test, ebas, pbas)
    ref = golden["values"][test]["HF energy"][0]
    for cls in (scf.HostSCF, scf.DeviceSCF):
        s = cls(sysd)
        r = s.solve(tol_energy=1e-11, tol_density=1e-9, max_iter=300)
        s.close()
        assert r.converged, cls.__name__
        assert abs(r.energy - ref) <= tol, (cls.__name__, r.energy, ref)


def test_h2o_apmo_uhf_golden_plain_and_mixed(scf, golden):
    """test/H2O.APMO.UHF.DIRECT within 1e-8 (plain FP64); the mixed FP32/FP64
    build within 1e-6 Eh of it."""
    sysd = GS.h2o_apmo_uhf(golden)
    ref = golden["values"]["H2O.APMO.UHF.DIRECT"]["HF energy"]
    s = scf.DeviceSCF(sysd)
    r = s.solve(tol_energy=1e-11, tol_density=1e-9)
    s.close()
    assert r.converged and abs(r.energy - ref[0]) <= ref[1]
    s = scf.DeviceSCF(sysd, precision="mixed")
    rm = s.solve(tol_energy=1e-11, tol_density=1e-9)
    s.close()
    assert rm.converged and abs(rm.energy - r.energy) <= 1e-6


@pytest.mark.parametrize("case", UEN_CASES, ids=[c[0] for c in UEN_CASES])
def test_uen_mp2_golden(scf, oracle, golden, case):
    """test/H2.APMO.UEN and test/H2O.BOA.UEN: closed-shell UHF solutions, so
    the checkers' UMP2 energies are the closed-shell (APMO-)MP2 totals: the
    device SCF of the merged electron species, then the device transform
    (intra-species and every species pair) against the golden MP2 (1e-5)."""
    from openlowdin_gb300 import lint
    from tests.test_gpu_mp2 import _apmo_device_mp2
    test, ebas, pbas = case
    sysd = closed_shell_twin(GS.uhf_system(golden, test, ebas, pbas))
    s = scf.DeviceSCF(sysd)
    r = s.solve(tol_energy=1e-11, tol_density=1e-9)
    s.close()
    res = oracle.scf(oracle.from_plain(sysd), tol_energy=1e-11, tol_density=1e-9)
    assert r.converged and abs(r.energy - res.energy) < 1e-9
    assert abs(r.energy - golden["values"][test]["HF energy"][0]) <= 1e-8
    total = res.energy + sum(_apmo_device_mp2(lint, sysd, res, 0).values())
    ref = golden["values"][test]["MP2 energy"]
    assert abs(total - ref[0]) <= ref[1], total
