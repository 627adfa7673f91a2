"""Open-shell UHF on the GPU library: E-ALPHA / E-BETA species (exchange factor
-1 each) coupled by the inter-species Coulomb matrix, as the reference runs UHF,
against the reference's golden energies (tests/golden/golden.json)."""
import pytest

from tests import golden_systems as GS
from tests.test_oracle import UHF_CASES

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
