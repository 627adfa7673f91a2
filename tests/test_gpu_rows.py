"""FP32 half of the mixed J/K build on the bra-row kernel (jk32_row_kernel).

The row kernel keeps a bra pair's rows of D and of the exchange output in
shared memory; it must take exactly the quartets the one-quartet-per-thread
FP32 kernel (jk_tasks_kernel) takes -- same FP32 bound, screening and split,
so the same quartet counts -- and give the same matrix up to the order of the
FP32 additions (1e-6 of the largest element here).  Against the FP64 build the
split keeps the error at the FP32 rounding of the small quartets.
"""
import os

import numpy as np
import pytest

from openlowdin_gb300 import systems as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def L():
    from openlowdin_gb300 import build, lint
    build.build()
    return lint


def _cases():
    return {
        "chain": S.chain_for_basis(10_011, 180)["species"][0],
        "water4": S.water_cluster(4, seed=0)["species"][0],
        "water2_d": S.water_cluster(2, seed=1, o_d=True)["species"][0],
        "protons": S.water_cluster(2, seed=0, quantum_protons=True, proton_species_mode="single")["species"][1],
    }


@pytest.mark.parametrize("name", ["chain", "water4", "water2_d", "protons"])
@pytest.mark.parametrize("split", [1e-5, 1.0])
def test_row_kernel_matches_tile_kernel(L, name, split, monkeypatch):
    torch = pytest.importorskip("torch")
    sp = _cases()[name]
    factor = -0.5 if sp["is_electron"] else -1.0
    h = L.Libint2Interface(sp, 1)
    n = h.nbasis
    rng = np.random.default_rng(41)
    X = rng.normal(size=(n, n)) * 0.05
    dD = torch.tensor(X + X.T, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    out = {}
    for rows in ("1", "0"):
        monkeypatch.setenv("LOWDIN_GB300_ROWS", rows)
        G = torch.full_like(dD, float("nan"))
        h.twobody_device(dD.data_ptr(), G.data_ptr(), factor, precision=1, split=split, stream=st)
        torch.cuda.synchronize()
        out[rows] = (G.cpu().numpy(), h.last_quartets(), h.last_class_quartets().copy())
    G64 = torch.empty_like(dD)
    h.twobody_device(dD.data_ptr(), G64.data_ptr(), factor, stream=st)
    torch.cuda.synchronize()
    g64 = G64.cpu().numpy()
    h.close()
    (gr, qr, cr), (go, qo, co) = out["1"], out["0"]
    assert qr == qo and np.array_equal(cr, co), (qr, qo)
    scale = max(1.0, float(np.max(np.abs(go))))
    assert np.all(np.isfinite(gr))
    # split 1e-5: only quartets bounded by 1e-5 are in FP32, so both FP32
    # kernels sit within 1e-6 of each other and of the FP64 build; split 1.0
    # puts large quartets in FP32 too (FP32 rounding of O(1) contributions)
    tol = 1e-6 if split < 1e-3 else 2e-5
    assert float(np.max(np.abs(gr - go))) < tol * scale
    assert float(np.max(np.abs(gr - g64))) < 10 * tol * scale


def test_autotune_keeps_the_quartets_and_the_matrices(L):
    """The autotuner only chooses which FP32 kernel runs each class: a mixed
    batch build before and after forced tuning evaluates the same quartets per
    class and gives the same matrices up to the order of FP32 additions."""
    torch = pytest.importorskip("torch")
    mols = [S.chain_for_basis(10_021, 150), S.water_cluster(2, seed=3)]
    st = torch.cuda.current_stream().cuda_stream
    hs, bufs = [], []
    b = L.Batch()
    rng = np.random.default_rng(5)
    for m in mols:
        sp = m["species"][0]
        h = L.Libint2Interface(sp, 1)
        n = h.nbasis
        X = rng.normal(size=(n, n)) * 0.03
        P = torch.tensor(X + X.T, device="cuda")
        G = torch.zeros_like(P)
        J = torch.zeros_like(P)
        b.add_system([h], [-1.0], [-0.5], [1], [P], [G], [J])
        hs.append(h)
        bufs.append((P, G, J))
    b.finalize(st)
    b.fock(3, 1e-5, st)
    q0 = b.quartets(st).copy()
    G0 = [g.clone() for _, g, _ in bufs]
    b.autotune(1e-5, force=True, stream=st)
    choice, ms_rows, ms_tiles = b.tuning()
    assert (choice >= 0).any()
    b.fock(3, 1e-5, st)
    q1 = b.quartets(st)
    assert np.array_equal(q0, q1)
    for g0, (_, g1, _) in zip(G0, bufs):
        scale = max(1.0, float(g0.abs().max()))
        assert float((g1 - g0).abs().max()) < 1e-6 * scale
    b.close()
    for h in hs:
        h.close()
