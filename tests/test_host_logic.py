"""Host-side logic of the drivers and the benchmark (no GPU): size buckets of
the batched SCF, the serving engine's admission footprint and latency
statistics, the Poisson request stream, and the frozen FLOP model."""
import numpy as np
import pytest

from openlowdin_gb300 import flops as FL
from openlowdin_gb300 import systems as S


def test_bucket_sizes_cover_and_bound_padding():
    from openlowdin_gb300.batch_scf import bucket_size
    prev = 0
    for n in range(1, 1300):
        b = bucket_size(n)
        assert b >= n and b >= prev
        step = 16 if n <= 128 else 32 if n <= 256 else 64
        assert b % step == 0
        if n >= 64:
            assert (b - n) / n <= 0.25
        prev = b
    # the batched-RHF workload's 512 molecules fall into few buckets
    sizes = {bucket_size(S.nbasis(S.chain_molecule(20_000 + i)["species"][0])) for i in range(64)}
    assert len(sizes) <= 24


def test_footprint_grows_with_size_and_mp2():
    from openlowdin_gb300.serve import footprint_bytes
    small, big = S.chain_for_basis(1, 60), S.chain_for_basis(1, 240)
    f_small, f_big = footprint_bytes(small, "scf"), footprint_bytes(big, "scf")
    assert 0 < f_small < f_big
    n = S.nbasis(big["species"][0])
    assert f_big >= 31 * n * n * 8        # 11 matrices + 2 x 10 DIIS history, FP64
    assert footprint_bytes(big, "scf+mp2") > f_big + 8e9 - 1


def test_latency_percentiles():
    from openlowdin_gb300.serve import latency_stats

    class R:
        def __init__(self, t):
            self.latency = t
    st = latency_stats([R(float(t)) for t in range(1, 101)])
    assert abs(st["p50_s"] - 50.5) < 1e-12
    assert abs(st["p99_s"] - 99.01) < 1e-9
    assert latency_stats([]) == {"p50_s": None, "p99_s": None}


def test_serving_stream_is_seeded_poisson():
    import bench
    a = bench.serving_requests(200, 100.0, seed=3)
    b = bench.serving_requests(200, 100.0, seed=3)
    assert [r.arrival for r in a] == [r.arrival for r in b]
    t = np.array([r.arrival for r in a])
    assert np.all(np.diff(t) >= 0)
    gaps = np.diff(t)
    assert 0.006 < gaps.mean() < 0.014          # 1 / (100 req/s), 200 samples
    kinds = [r.kind for r in a]
    assert 0.15 < kinds.count("scf+mp2") / len(kinds) < 0.45


def test_flop_model_is_additive():
    c = np.zeros((10, 10), np.int64)
    c[0, 0], c[1, 0], c[1, 1] = 10, 7, 3
    tot = FL.class_table_flops(c, "jk")
    parts = 10 * FL.quartet_flops(0, 0, 0, 0, "jk") + 7 * FL.quartet_flops(1, 0, 0, 0, "jk") + \
        3 * FL.quartet_flops(1, 0, 1, 0, "jk")
    assert tot == pytest.approx(parts)
    # more angular momentum, more work
    assert FL.quartet_flops(0, 0, 0, 0) < FL.quartet_flops(1, 0, 0, 0) < FL.quartet_flops(1, 1, 1, 1) \
        < FL.quartet_flops(2, 2, 2, 2)


def test_chain_generator_properties():
    """Batched-RHF workload generator: seeded, closed shell, atoms at least
    2 bohr apart, 3-30 atoms (one H more or less for the electron count)."""
    for seed in range(40):
        m = S.chain_molecule(20_000 + seed)
        m2 = S.chain_molecule(20_000 + seed)
        assert m["point_positions"] == m2["point_positions"]
        Z = m["point_charges"]
        assert int(sum(Z)) % 2 == 0
        assert 3 <= len(Z) <= 31
        R = np.array(m["point_positions"])
        d = np.linalg.norm(R[:, None] - R[None], axis=-1) + np.eye(len(R)) * 1e9
        assert d.min() >= 2.0 - 1e-12
        assert m["species"][0]["n_particles"] == int(sum(Z))


def test_canonical_orthogonaliser_drops_dependent_functions():
    from openlowdin_gb300.scf import _orthogonaliser_np
    rng = np.random.default_rng(5)
    A = rng.normal(size=(6, 6))
    S_full = A @ A.T + 6 * np.eye(6)
    X = _orthogonaliser_np(S_full)
    assert np.allclose(X.T @ S_full @ X, np.eye(6), atol=1e-12)
    B = rng.normal(size=(6, 4))
    S_def = B @ B.T                              # rank 4
    X = _orthogonaliser_np(S_def)
    assert X.shape == (6, 4)
    assert np.allclose(X.T @ S_def @ X, np.eye(4), atol=1e-10)


def test_batch_arguments_checked_on_the_host():
    """Row strides below a species' size and flag arrays of the wrong length
    are rejected before any device work."""
    from openlowdin_gb300 import build, lint
    build.build()
    sp = S.water()["species"][0]
    h = lint.Libint2Interface(sp, 1)
    b = lint.Batch()
    with pytest.raises(lint.LowdinGB300Error):
        b.add_system([h], [-1.0], [-0.5], [1], [1], [1], [1], ld=[h.nbasis - 1])
    lint.lib().LowdinGB300_clear_error()
    b.add_system([h], [-1.0], [-0.5], [1], [1], [1], [1], ld=[h.nbasis + 8])
    with pytest.raises(ValueError):
        b.set_active([1, 1])
    with pytest.raises(lint.LowdinGB300Error):
        b.set_active([1])                        # not finalised yet
    b.close()
    h.close()


def test_serving_stream_sizes_span_the_configured_range():
    """The headline stream draws sizes log-uniformly from 30-1200 functions:
    the generated chains reach at least the drawn size and stay within the
    range plus one atom's functions."""
    import bench
    from openlowdin_gb300 import systems as S
    reqs = bench.serving_requests(40, 50.0, seed=1)
    n = np.array([S.nbasis(r.system["species"][0]) for r in reqs])
    assert n.min() >= bench.STREAM_LO and n.max() <= bench.STREAM_HI + 20
    # log-uniform: about half of the draws below the geometric mean (190)
    assert 0.25 < np.mean(n < np.sqrt(bench.STREAM_LO * bench.STREAM_HI)) < 0.75


def test_bench_per_job_table_and_tuning_summary():
    """The per-job error table pairs mixed and plain results by request and
    the autotuner summary counts the kernels kept per class."""
    import bench
    from types import SimpleNamespace as NS
    reqs = [NS(rid=0, kind="scf"), NS(rid=1, kind="scf+mp2")]
    plain = {0: NS(nbasis=40, iterations=20, converged=True, energy=-76.0, e2=None),
             1: NS(nbasis=80, iterations=30, converged=True, energy=-150.0, e2=-0.5)}
    mixed = {0: NS(nbasis=40, iterations=21, converged=True, energy=-76.0 + 3e-9, e2=None, err_vs_fp64=1e-9,
                   guard_hit=False),
             1: NS(nbasis=80, iterations=31, converged=False, energy=-150.1, e2=-0.6, err_vs_fp64=None,
                   guard_hit=False)}
    rows = bench.per_job_table(reqs, plain, mixed)
    assert abs(rows[0]["abs_dE_mixed_vs_plain_Eh"] - 3e-9) < 1e-12
    assert rows[1]["converged_mixed"] is False and abs(rows[1]["abs_dE2_mixed_vs_plain_Eh"] - 0.1) < 1e-12
    ch = np.full((10, 10), -1)
    ch[0, 0], ch[1, 0] = 1, 0
    ms = np.where(ch >= 0, 1.0, -1.0).astype(np.float32)
    s = bench.tuning_summary([(ch, ms, 2 * ms)])
    assert s["batches"] == 1
    assert s["classes"]["(ss|ss)"]["rows_kernel"] == 1 and s["classes"]["(ps|ss)"]["tile_kernel"] == 1


def test_uhf_electron_species_counts():
    from openlowdin_gb300 import systems as S
    shells = [(0, [1.0], [1.0], [0.0, 0.0, 0.0])]
    a, b = S.uhf_electron_species(shells, 16, 3)
    assert (a["name"], a["n_particles"], b["name"], b["n_particles"]) == ("E-ALPHA", 9, "E-BETA", 7)
    for sp in (a, b):
        assert sp["eta"] == 1.0 and sp["kappa"] / sp["eta"] == -1.0 and sp["particles_fraction"] == 1.0
    a, b = S.uhf_electron_species(shells, 1, 2)
    assert (a["n_particles"], b["n_particles"]) == (1, 0)
    import pytest
    with pytest.raises(ValueError):
        S.uhf_electron_species(shells, 2, 2)
