"""The allocation-free two-particle build, through the C ABI.

Some callers cannot allocate device memory while they run (a host program that
owns all device memory through its own pool, a serving loop that forbids
allocations after warm-up).  For them
LowdinGB300_twobody_device_noalloc keeps its work buffers in one static device
array.  This file is collected last so that a failure here, in a run that stops
at the first failure, comes after every other test has run.
"""
import ctypes

import numpy as np
import pytest

from openlowdin_gb300 import systems as S

pytestmark = pytest.mark.gpu

TOL = 1e-10  # same element-wise tolerance as the other two-particle parity tests


@pytest.fixture(scope="module")
def L():
    from openlowdin_gb300 import build, lint
    build.build()
    return lint


def _call_noalloc(L, h, D, G, factor, stream, precision=0, split=0.0):
    return L.lib().LowdinGB300_twobody_device_noalloc(h.h, D.data_ptr(), G.data_ptr(), float(factor), precision,
                                                      float(split), stream)


def _system(which):
    return S.water() if which == "water" else S.water_cluster(4, seed=0, quantum_protons=True)


# precision 1 splits at 1e-5: the FP32 work arrays of the scratch array are in
# use; it is compared with the allocating entry point's mixed build, whose
# FP32 additions may run in another order (1e-7 of the largest element)
@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("which", ["water", "apmo_electrons"])
def test_noalloc_matches_allocating_entry_point_twice(L, which, precision):
    torch = pytest.importorskip("torch")
    sp = _system(which)["species"][0]
    h = L.Libint2Interface(sp, 1)
    h.init_2body_ints()
    n = h.nbasis
    rng = np.random.default_rng(31)
    st = torch.cuda.current_stream().cuda_stream
    X = rng.normal(size=(n, n)) * 0.1
    D = torch.tensor(X + X.T, device="cuda")
    split = 1e-5 if precision else 0.0
    Gref = torch.empty_like(D)
    h.twobody_device(D.data_ptr(), Gref.data_ptr(), -0.5, precision, split, st)
    torch.cuda.synchronize()
    tol = TOL if precision == 0 else 1e-7 * max(1.0, float(Gref.abs().max()))
    for call in range(2):
        G = torch.full_like(D, float("nan"))
        assert _call_noalloc(L, h, D, G, -0.5, st, precision, split) == 0, L.last_error()
        torch.cuda.synchronize()
        err = float((G - Gref).abs().max())
        assert err < tol, (call, err)
    h.close()


def test_noalloc_alternating_species_share_the_array(L):
    """Two species of different sizes take turns in the shared array on one
    stream: what one call leaves behind must not leak into the next."""
    torch = pytest.importorskip("torch")
    st = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(32)
    cases = []
    for which in ("apmo_electrons", "water"):
        h = L.Libint2Interface(_system(which)["species"][0], 1)
        h.init_2body_ints()
        n = h.nbasis
        X = rng.normal(size=(n, n)) * 0.1
        D = torch.tensor(X + X.T, device="cuda")
        Gref = torch.empty_like(D)
        h.twobody_device(D.data_ptr(), Gref.data_ptr(), -0.5, 0, 0.0, st)
        cases.append((h, D, Gref))
    torch.cuda.synchronize()
    for rnd in range(2):
        for h, D, Gref in cases:
            G = torch.full_like(D, float("nan"))
            assert _call_noalloc(L, h, D, G, -0.5, st) == 0, L.last_error()
            torch.cuda.synchronize()
            assert float((G - Gref).abs().max()) < TOL, rnd
    for h, _, _ in cases:
        h.close()


def test_noalloc_rejects_species_above_the_limit(L):
    torch = pytest.importorskip("torch")
    sysd = S.water_cluster(16, seed=0)            # 544 Cartesian functions > 512
    sp = sysd["species"][0]
    h = L.Libint2Interface(sp, 1)
    h.init_2body_ints()
    n = h.nbasis
    assert n > 512
    D = torch.zeros((n, n), dtype=torch.float64, device="cuda")
    G = torch.zeros_like(D)
    rc = _call_noalloc(L, h, D, G, -0.5, torch.cuda.current_stream().cuda_stream)
    assert rc == -1
    msg = L.last_error()
    L.lib().LowdinGB300_clear_error()
    assert "512" in msg
    h.close()


def test_noalloc_scratch_is_modest(L):
    assert L.lib().LowdinGB300_noalloc_scratch_bytes() < 16 * 1024 * 1024
