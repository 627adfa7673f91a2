"""Continuous-batching serving engine: a job's result is the same alone and in
a mix of other jobs (arriving before and after it), plain FP64 and mixed;
plain results match the oracle; admission respects the HBM budget.

Tolerances: alone vs mix 1e-10 Eh plain, 1e-8 Eh mixed (the job's arithmetic
does not depend on the mix; only the order of floating-point atomics differs,
which the FP32 accumulators of the mixed path feel more); plain vs oracle
1e-8 Eh.
"""
import numpy as np
import pytest

from openlowdin_gb300 import systems as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def serve():
    from openlowdin_gb300 import build, serve
    build.build()
    return serve


def _mix(serve, target):
    others = [serve.Request(S.chain_for_basis(200 + i, nbf), kind, 0.0, 100 + i)
              for i, (nbf, kind) in enumerate([(40, "scf"), (90, "scf+mp2"), (60, "scf"), (120, "scf")])]
    t = serve.Request(target.system, target.kind, 0.0, 1)
    return others[:2] + [t] + others[2:]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_same_alone_and_in_mix(serve, precision):
    target = serve.Request(S.chain_for_basis(7, 70), "scf+mp2", 0.0, 1)
    alone = serve.ServingEngine(precision=precision).run([target], realtime=False)
    assert len(alone) == 1 and alone[0].converged
    mixres = serve.ServingEngine(precision=precision).run(_mix(serve, target), realtime=False)
    assert len(mixres) == 5 and all(r.converged for r in mixres)
    m = [r for r in mixres if r.rid == 1][0]
    tol = 1e-10 if precision == "fp64" else 1e-8
    assert abs(m.energy - alone[0].energy) < tol
    assert abs(m.e2 - alone[0].e2) < tol


def test_plain_serving_matches_oracle(serve, oracle):
    sysd = S.chain_for_basis(11, 50)
    res = serve.ServingEngine(precision="fp64", tol_energy=1e-10, tol_density=1e-8).run(
        [serve.Request(sysd, "scf+mp2", 0.0, 0)], realtime=False)[0]
    ro = oracle.scf(oracle.from_plain(sysd), tol_energy=1e-10, tol_density=1e-8)
    assert abs(res.energy - ro.energy) < 1e-8
    b = oracle.Basis.from_shells(sysd["species"][0]["shells"])
    e2 = oracle.rmp2_direct(b, ro.densities[0], ro.coefficients[0], ro.orbital_energies[0],
                            sysd["species"][0]["n_particles"] // 2, S.n_core(sysd))
    assert abs(res.e2 - e2) < 1e-8


def test_admission_respects_budget(serve):
    reqs = [serve.Request(S.chain_for_basis(300 + i, 40), "scf", 0.0, i) for i in range(4)]
    fp = serve.footprint_bytes(reqs[0].system, "scf")
    seen = []
    eng = serve.ServingEngine(precision="fp64", hbm_budget_gb=1.5 * fp / 1e9)
    res = eng.run(reqs, realtime=False, on_iteration=seen.append)
    assert len(res) == 4 and all(r.converged for r in res)
    assert max(seen) == 1


def test_mixed_jobs_state_their_fp64_error(serve):
    """Every mixed job ends with an FP64 rebuild at its converged density:
    its energy is the FP64 energy there and |E_mixed - E_FP64| is reported,
    within the 1e-6 Eh bar; the plain run of the same job agrees to 1e-6."""
    reqs = [serve.Request(S.chain_for_basis(400 + i, nbf), "scf", 0.0, i) for i, nbf in enumerate((60, 110))]
    plain = {r.rid: r for r in serve.ServingEngine(precision="fp64").run(reqs, realtime=False)}
    mixed = serve.ServingEngine(precision="mixed").run(reqs, realtime=False)
    for r in mixed:
        assert r.converged and not r.guard_hit
        assert r.err_vs_fp64 is not None and r.err_vs_fp64 <= 1e-6
        assert abs(r.energy - plain[r.rid].energy) < 1e-6


def test_guard_sends_a_failed_job_on_in_fp64(serve):
    """With every quartet forced into FP32 (split far above every bound) and
    the check's bar at 1e-9 Eh the mixed solution fails its FP64 check: the
    job continues in FP64 and ends on the plain result."""
    req = serve.Request(S.chain_for_basis(421, 90), "scf", 0.0, 0)
    plain = serve.ServingEngine(precision="fp64").run([req], realtime=False)[0]
    forced = serve.ServingEngine(precision="mixed", split=1e30, guard_energy=1e-9).run([req], realtime=False)[0]
    assert forced.converged and forced.guard_hit
    assert forced.err_vs_fp64 == 0.0
    assert abs(forced.energy - plain.energy) < 1e-8
