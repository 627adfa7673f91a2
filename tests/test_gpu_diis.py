"""Device DIIS coefficients (LowdinGB300_diis_coefficients) against the exact
minimiser of the extrapolated error under sum(c) = 1 on the host
(src/scf/Convergence.f90:543-633 solves the same bordered system through an
SVD), for histories whose errors fall by orders of magnitude as an SCF's do;
and the device Boys functions against their definition."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _host(E):
    """Exact minimiser of c^T E c under sum(c) = 1: c ~ E^-1 1, solved on the
    unit-diagonal form of E (well conditioned for independent vectors)."""
    d = 1.0 / np.sqrt(np.diag(E))
    y = d * np.linalg.solve(E * d[:, None] * d[None, :], d)
    return y / y.sum()


@pytest.mark.parametrize("h", [2, 3, 7, 10, 20])
def test_diis_coefficients_match_host_least_squares(h):
    torch = pytest.importorskip("torch")
    from openlowdin_gb300 import build, lint
    build.build()
    rng = np.random.default_rng(h)
    nsys = 37
    Es = []
    for s in range(nsys):
        # error vectors shrinking like an SCF history (condition grows with h)
        V = rng.normal(size=(h, 200)) * (0.3 ** np.arange(h))[:, None]
        Es.append(V @ V.T)
    E = np.stack(Es)
    dE = torch.tensor(E, device="cuda")
    dc = torch.empty((nsys, h), dtype=torch.float64, device="cuda")
    lint.diis_coefficients(dE.data_ptr(), h, nsys, dc.data_ptr(), torch.cuda.current_stream().cuda_stream)
    c = dc.cpu().numpy()
    for s in range(nsys):
        ref = _host(E[s])
        assert abs(c[s].sum() - 1.0) < 1e-10
        # the extrapolated error |sum c_i e_i|^2 = c^T E c is what DIIS
        # minimises: no worse than the host solution (up to rounding)
        got, want = c[s] @ E[s] @ c[s], ref @ E[s] @ ref
        assert got <= want * (1 + 1e-6)
        assert np.max(np.abs(c[s] - ref)) < 1e-6 * max(1.0, np.max(np.abs(ref)))


def test_diis_rejects_long_histories():
    torch = pytest.importorskip("torch")
    from openlowdin_gb300 import lint
    dE = torch.zeros((1, 21, 21), dtype=torch.float64, device="cuda")
    dc = torch.zeros((1, 21), dtype=torch.float64, device="cuda")
    with pytest.raises(lint.LowdinGB300Error):
        lint.diis_coefficients(dE.data_ptr(), 21, 1, dc.data_ptr())


@pytest.mark.parametrize("L", [0, 1, 2, 3, 4])
def test_device_boys_functions_against_incomplete_gamma(L):
    """The FP32 kernels' arithmetic Boys function within 1e-6 relative of the
    incomplete-gamma definition for T in [0, 60]; the FP64 tabulated one within
    1e-13 (every order m <= L)."""
    from scipy.special import gamma, gammainc
    from openlowdin_gb300 import build, lint
    build.build()
    T = np.concatenate([[0.0, 1e-10, 1e-6], np.linspace(1e-4, 1.0, 500), np.linspace(1.0, 60.0, 6000)])
    for fp32, tol in ((True, 1e-6), (False, 1e-13)):
        F = lint.boys_eval(T, L, fp32)
        for m in range(L + 1):
            ex = np.where(T < 1e-12, 1.0 / (2 * m + 1),
                          gamma(m + 0.5) * gammainc(m + 0.5, np.maximum(T, 1e-300)) /
                          (2 * np.maximum(T, 1e-300) ** (m + 0.5)))
            rel = np.max(np.abs(F[:, m] - ex) / ex)
            assert rel < tol, (fp32, m, rel)


@pytest.mark.parametrize("n,occ", [(200, 60), (600, 150)])
def test_occupied_subspace_matches_fp64_eigensolver(n, occ):
    """FP32 eigensolve + FP64 refinement of the occupied subspace gives the
    FP64 eigensolver's density projector (a Fock-like spectrum: degenerate
    core levels, a 0.05 Eh gap, virtuals up to 300 Eh)."""
    torch = pytest.importorskip("torch")
    from openlowdin_gb300.scf import occupied_subspace
    rng = np.random.default_rng(n)
    ev = np.concatenate([np.full(10, -20.0) + rng.normal(size=10) * 1e-3,
                         -np.sort(rng.uniform(0.3, 1.5, occ - 10)),
                         -0.25 + np.zeros(0), np.sort(rng.uniform(-0.2, 300, n - occ))])
    Q, _ = np.linalg.qr(rng.normal(size=(n, n)))
    F = torch.tensor((Q * ev) @ Q.T, device="cuda")
    Co = occupied_subspace(F, occ)
    w, V = torch.linalg.eigh(F)
    P, Pe = Co @ Co.T, V[:, :occ] @ V[:, :occ].T
    assert float((P - Pe).abs().max()) < 1e-11
    assert float((Co.T @ Co - torch.eye(occ, dtype=Co.dtype, device="cuda")).abs().max()) < 1e-12
