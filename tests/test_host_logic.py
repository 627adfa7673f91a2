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
    c = np.zeros((6, 6), np.int64)
    c[0, 0], c[1, 0], c[1, 1] = 10, 7, 3
    tot = FL.class_table_flops(c, "jk")
    parts = 10 * FL.quartet_flops(0, 0, 0, 0, "jk") + 7 * FL.quartet_flops(1, 0, 0, 0, "jk") + \
        3 * FL.quartet_flops(1, 0, 1, 0, "jk")
    assert tot == pytest.approx(parts)
    # more angular momentum, more work
    assert FL.quartet_flops(0, 0, 0, 0) < FL.quartet_flops(1, 0, 0, 0) < FL.quartet_flops(1, 1, 1, 1) \
        < FL.quartet_flops(2, 2, 2, 2)
