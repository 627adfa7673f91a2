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
