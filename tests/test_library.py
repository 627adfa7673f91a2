"""CPU-side checks of the C-ABI library: it loads and exports every symbol the
public header declares (no GPU call is made)."""
import ctypes
import os
import re

import pytest

from openlowdin_gb300 import lint

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_symbols():
    txt = open(os.path.join(ROOT, "include", "lowdin_gb300.h")).read()
    return sorted(set(re.findall(r"\b((?:LibintInterface|libintinterface|LowdinGB300)_\w+)\s*\(", txt)))


@pytest.fixture(scope="module")
def built():
    from openlowdin_gb300 import build
    build.build()
    return lint.lib()


def test_header_and_binding_agree():
    assert sorted(lint.EXPORTED_SYMBOLS) == _declared_symbols()


def test_library_exports_every_declared_symbol(built):
    for name in _declared_symbols():
        assert hasattr(built, name), name
        assert isinstance(getattr(built, name), ctypes._CFuncPtr)


def test_handle_lifecycle_without_gpu(built):
    """Creating a handle and adding shells is host-only work."""
    from openlowdin_gb300 import systems
    h = lint.Libint2Interface(systems.water()["species"][0], 1)
    assert h.nbasis == 34
    h.close()


def test_one_body_host_integrals_match_oracle(built, oracle):
    import numpy as np
    from openlowdin_gb300 import systems
    sysd = systems.water(d_shell=True)
    sp = sysd["species"][0]
    h = lint.Libint2Interface(sp, 1)
    b = oracle.Basis.from_shells(sp["shells"])
    S0, T0 = oracle.overlap_kinetic(b)
    V0 = oracle.potential(b, sysd["point_charges"], sysd["point_positions"])
    assert np.max(np.abs(h.one_body(1) - S0)) < 1e-13
    assert np.max(np.abs(h.one_body(2) - T0)) < 1e-11
    assert np.max(np.abs(h.potential(sysd["point_charges"], sysd["point_positions"]) - V0)) < 1e-11
    h.close()


def test_one_body_host_integrals_f_shells_and_contractions(built, oracle):
    """The host one-body matrices (overlap, kinetic, point-charge potential)
    on contracted s, p, d and f shells over two centres, against the oracle."""
    import numpy as np
    from openlowdin_gb300 import systems
    A, B = [0.0, 0.0, 0.0], [0.0, 0.9, 1.3]
    sh = []
    for c in (A, B):
        sh += [(0, [3.0, 0.6], [0.4, 0.7], c), (1, [1.1, 0.3], [0.5, 0.6], c), (2, [0.9], [1.0], c),
               (3, [1.3, 0.4], [0.3, 0.8], c)]
    h = lint.Libint2Interface(systems.electron_species(sh, 6), 1)
    b = oracle.Basis.from_shells(sh)
    S0, T0 = oracle.overlap_kinetic(b)
    Z, R = [3.0, 1.0], [[0.0, 0.0, 0.2], [0.5, 0.4, 1.0]]
    V0 = oracle.potential(b, Z, R)
    assert np.max(np.abs(h.one_body(1) - S0)) < 1e-13
    assert np.max(np.abs(h.one_body(2) - T0)) < 1e-11
    assert np.max(np.abs(h.potential(Z, R) - V0)) < 1e-11
    h.close()
