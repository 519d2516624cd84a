"""Serving loop: admission by slots and memory budget (CPU, with a fake
context), and on the GPU that every job's result is the same alone and in
a mix of concurrently resident jobs."""
import numpy as np
import pytest

from mdynamix_gb300 import serve
from mdynamix_gb300 import system as S
from mdynamix_gb300.abi import MDX_FP64, MDX_MIXED


class _Params:
    lmdee = 0


class _Packed:
    def __init__(self):
        self.params = _Params()


class _Thermo:
    temp = 298.0
    tke = 1.0


class FakeContext:
    """Stands in for ForcePath: a queued segment finishes after a fixed
    number of polls; records what the server asked for."""
    live = 0
    max_live = 0

    def __init__(self, system, precision):
        self.system = system
        self.packed = _Packed()
        self.pending = 0
        self.lambdas = []
        self.segments = []
        FakeContext.live += 1
        FakeContext.max_live = max(FakeContext.max_live, FakeContext.live)

    def set_params(self, p):
        assert p.lmdee == 1

    def set_state(self, *st):
        pass

    def set_lambda(self, ec, pw1, pw2, bee):
        self.lambdas.append(ec)

    def enqueue_double(self, nsteps, mstep0, prologue=False):
        assert prologue
        self.segments.append((nsteps, mstep0))
        self.pending = 3

    def poll(self):
        self.pending -= 1
        return self.pending <= 0

    def get_state(self):
        n = self.system.nstot
        return tuple(np.zeros(n) for _ in range(6)), _Thermo()

    def close(self):
        FakeContext.live -= 1


def _jobs(n, rate, steps=5):
    return [serve.prepare(j) for j in serve.solvation_stream(n, rate, seed=3,
                                                             steps_per_state=steps,
                                                             nwater=(200, 400))]


def test_solvation_jobs_follow_the_workload_shape():
    jobs = serve.solvation_stream(50, rate=100.0, seed=1)
    arr = [j.arrival for j in jobs]
    assert arr == sorted(arr) and arr[0] > 0
    for j in jobs:
        (sol, one), (water, nw) = j.spec.molecules
        assert sol in S.SOLUTES and one == 1 and water == "H2O"
        assert 200 <= nw <= 2000
        assert j.spec.iee_type == 1 and j.spec.rcut == 9.0 and j.spec.nfreq == 10
        assert tuple(j.lambdas) == (1.0, 0.75, 0.5, 0.25, 0.0)


def test_admission_respects_slots_and_budget():
    preps = _jobs(12, rate=0.0)          # all arrive at once
    est = [serve.estimate_bytes(p.system, MDX_MIXED) for p in preps]
    budget = int(sum(sorted(est)[-3:]) + 1)  # room for about three jobs
    FakeContext.live = FakeContext.max_live = 0
    srv = serve.Server(precision=MDX_MIXED, budget=budget, slots=4,
                       open_context=FakeContext)
    res = srv.run(preps)
    assert len(res) == 12
    assert FakeContext.live == 0
    assert 1 <= srv.peak_resident <= 4
    assert srv.peak_bytes <= budget
    # first come, first served
    assert srv.admit_order == [p.job.name for p in preps]
    for r in res:
        assert [st["lambda"] for st in r.states] == [1.0, 0.75, 0.5, 0.25, 0.0]
        assert r.latency >= 0 and r.admitted >= r.arrival - 1e-9
    st = serve.latency_stats(res, wall=1.0)
    assert st["p50_s"] <= st["p99_s"] <= st["max_s"]


def test_a_job_larger_than_the_budget_still_runs_alone():
    preps = _jobs(3, rate=0.0)
    srv = serve.Server(precision=MDX_MIXED, budget=1, slots=8, open_context=FakeContext)
    res = srv.run(preps)
    assert len(res) == 3 and srv.peak_resident == 1


def _final(res):
    return {r.name: np.stack(r.states[-1]["state"][:3]) for r in res}


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [(MDX_MIXED, 0.0), (MDX_FP64, 1e-8)])
def test_same_result_alone_and_in_the_mix(precision, tol):
    # tol: mixed is bit-exact (integer force sums, ordered reductions);
    # FP64 pair forces use atomics, so the last bits may differ run to run:
    # relative position difference after 5 x 4 long steps
    preps = _jobs(4, rate=0.0, steps=4)
    alone = {}
    for p in preps:
        srv = serve.Server(precision=precision, budget=8 << 30, slots=1, keep_states=True)
        alone.update(_final(srv.run([p])))
    srv = serve.Server(precision=precision, budget=8 << 30, slots=8, keep_states=True)
    mix = srv.run(preps)
    assert srv.peak_resident == 4
    together = _final(mix)
    for name, x in alone.items():
        y = together[name]
        err = np.abs(x - y).max() / np.abs(x).max()
        assert err <= tol, (name, err)
