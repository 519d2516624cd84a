"""Continuous-batching serving loop: many independent MD jobs on one GPU.

A job is one system (e.g. a solute in water, ``system.solvation_job``) run
through a sequence of fixed expanded-ensemble coupling states (RECINT,
mdee.f:86-140: ``set_lambda`` then a DOUBLE segment of ``steps_per_state``
long steps, mdstep.f:281-530).  The reference runs one system per process;
here a single host loop keeps many systems resident on the device:

- requests arrive over time (``JobSpec.arrival``, seconds after start);
- a request is admitted as soon as a slot and enough of the HBM budget are
  free (first come, first served; its device footprint is estimated from
  its sizes before it is opened);
- every admitted job owns a library context (its own CUDA stream); its
  segments are queued without waiting (``enqueue_double``, graph-replayed
  long steps), so the kernels of all resident jobs overlap on the GPU;
- the loop polls the streams; a finished segment moves its job to the next
  coupling state, a finished job is downloaded, its context closed (device
  memory is stream-ordered, so closing does not stall the other jobs) and
  its slot and memory go to the next request.

A job may instead walk between its coupling states (``walk_ncee`` > 0):
segments of NCEE long steps, each followed by a CHENS move (mdee.f:142-262;
``mdee.MdeeWalk``: energy differences on the GPU, Metropolis on the host)
that keeps or changes the coupling, ``walk_moves`` moves in all -- the
reference's MDEE walk rather than fixed-coupling segments.

Results are per job: the state (positions, momenta, thermostat) after each
coupling state or segment, and the latency from arrival to completion.  Contexts are
independent and the mixed path is deterministic, so a job's results are the
same alone and in any mix.
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field
from typing import Callable, List, Optional, Sequence

import numpy as np

from . import system as S
from .abi import MDX_MIXED
from .mdx import ForcePath, device_memory


@dataclass
class JobSpec:
    name: str
    spec: S.RunSpec
    lambdas: Sequence[float] = (1.0, 0.75, 0.5, 0.25, 0.0)   # EC per state
    steps_per_state: int = 500
    seed: int = 1
    arrival: float = 0.0
    pw1: float = 1.0            # input.f:152-156 defaults
    pw2: float = 1.0 / 3.0
    bee: float = 3.0
    walk_ncee: int = 0          # > 0: CHENS walk, a move every NCEE long steps
    walk_moves: int = 0
    walk_wl: float = 0.0        # Wang-Landau decrement of EE(ME) per move

    def segments(self) -> int:
        return self.walk_moves + 1 if self.walk_ncee else len(self.lambdas)


@dataclass
class JobResult:
    name: str
    atoms: int
    arrival: float
    admitted: float
    finished: float
    est_bytes: int
    states: List[dict] = field(default_factory=list)

    @property
    def latency(self) -> float:
        return self.finished - self.arrival

    @property
    def atom_steps(self) -> int:
        return self.atoms * sum(st["steps"] for st in self.states)


@dataclass
class Prepared:
    """Host-side preprocessing of a request (topology, start state)."""
    job: JobSpec
    system: S.System
    state: tuple


def prepare(job: JobSpec) -> Prepared:
    s = S.System(job.spec)
    st = S.make_configuration(s, seed=job.seed, jitter=0.05)
    return Prepared(job, s, st)


def estimate_bytes(s: S.System, precision: int) -> int:
    """Upper estimate of a context's device footprint from its sizes."""
    from .abi import default_caps
    n = s.nstot
    cs, cl = default_caps(s)
    if precision == MDX_MIXED:
        cs, cl = 2 * cs, 2 * cl
    nkv = max(1, s.kvector_count())
    kmax = int(math.ceil((nkv * 3.0 / (2.0 * math.pi)) ** (1.0 / 3.0))) + 2
    rows = 4 * kmax + 3
    per_atom = 1024 + 4 * (cs + cl) + 16 * rows + 4 * s.nbdmax
    slices = max(1, -(-n // 128))
    per_k = 256 + 16 * slices
    return int(n * per_atom + nkv * per_k + (24 << 20))


class _Running:
    def __init__(self, prep: Prepared, g: ForcePath, res: JobResult, nbytes: int):
        self.prep, self.g, self.res, self.bytes = prep, g, res, nbytes
        self.k = 0          # coupling state (or walk segment) in flight
        self.mstep = 0
        self.walk = None


class Server:
    """One GPU, many resident jobs.  ``budget`` is the device memory the
    jobs may hold (bytes); ``slots`` caps how many run at once."""

    def __init__(self, precision: int = MDX_MIXED, budget: Optional[int] = None,
                 slots: int = 64, keep_states: bool = False,
                 clock: Callable[[], float] = time.perf_counter,
                 open_context: Callable = ForcePath):
        self.precision = precision
        self.open_context = open_context
        if budget is None:
            free, _ = device_memory()
            budget = int(0.8 * free)
        self.budget = budget
        self.slots = slots
        self.keep_states = keep_states
        self.clock = clock
        self.peak_resident = 0
        self.peak_bytes = 0
        self.admit_order: List[str] = []

    # one coupling state: RECINT scaling, then DOUBLE's prologue + segment
    def _start_state(self, r: _Running):
        j = r.prep.job
        if j.walk_ncee:
            if r.walk is None:
                from .mdee import MdeeWalk
                r.walk = MdeeWalk(r.prep.system, ec=list(j.lambdas), me=1, pw1=j.pw1,
                                  pw2=j.pw2, bee=j.bee, wl_corr=j.walk_wl, seed=j.seed)
                r.walk.apply(r.g)
                r.g.enqueue_double(j.walk_ncee, r.mstep, prologue=True)
            else:
                r.walk.attempt(r.g)   # the previous segment has finished (polled)
                r.g.enqueue_double(j.walk_ncee, r.mstep, prologue=False)
            return
        r.g.set_lambda(j.lambdas[r.k], j.pw1, j.pw2, j.bee)
        r.g.enqueue_double(j.steps_per_state, r.mstep, prologue=True)

    def _finish_state(self, r: _Running):
        j = r.prep.job
        (x, y, z, vx, vy, vz), th = r.g.get_state()
        if j.walk_ncee:
            rec = {"lambda": r.walk.ec[r.walk.me - 1], "me": r.walk.me, "steps": j.walk_ncee,
                   "temp": th.temp, "tke": th.tke, "accepted": r.walk.accepted}
            if self.keep_states:
                rec["state"] = (x, y, z, vx, vy, vz)
            r.res.states.append(rec)
            r.mstep += j.walk_ncee
            r.k += 1
            return
        rec = {"lambda": j.lambdas[r.k], "steps": j.steps_per_state, "temp": th.temp,
               "tke": th.tke}
        if self.keep_states:
            rec["state"] = (x, y, z, vx, vy, vz)
        r.res.states.append(rec)
        r.mstep += j.steps_per_state
        r.k += 1

    def run(self, preps: Sequence[Prepared]) -> List[JobResult]:
        pending = sorted(preps, key=lambda p: p.job.arrival)
        active: List[_Running] = []
        done: List[JobResult] = []
        used = 0
        t0 = self.clock()
        while pending or active:
            now = self.clock() - t0
            progressed = False
            # admission: first come, first served, by slot and memory budget
            while pending and pending[0].job.arrival <= now and len(active) < self.slots:
                p = pending[0]
                est = estimate_bytes(p.system, self.precision)
                if used + est > self.budget and active:
                    break
                pending.pop(0)
                g = self.open_context(p.system, precision=self.precision)
                g.packed.params.lmdee = 1
                g.set_params(g.packed.params)
                g.set_state(*p.state)
                res = JobResult(p.job.name, p.system.nstot, p.job.arrival, self.clock() - t0,
                                0.0, est)
                r = _Running(p, g, res, est)
                self.admit_order.append(p.job.name)
                self._start_state(r)
                active.append(r)
                used += est
                self.peak_resident = max(self.peak_resident, len(active))
                self.peak_bytes = max(self.peak_bytes, used)
                progressed = True
            # progress: finished segments move on, finished jobs leave
            for r in list(active):
                if not r.g.poll():
                    continue
                progressed = True
                self._finish_state(r)
                if r.k < r.prep.job.segments():
                    self._start_state(r)
                    continue
                r.res.finished = self.clock() - t0
                r.g.close()
                used -= r.bytes
                active.remove(r)
                done.append(r.res)
            if not progressed:
                if active or (pending and pending[0].job.arrival <= now):
                    time.sleep(50e-6)
                elif pending:
                    time.sleep(min(1e-3, max(0.0, pending[0].job.arrival - now)))
        return done


def solvation_stream(n_jobs: int, rate: float, seed: int = 7, steps_per_state: int = 500,
                     nwater: Sequence[int] = (200, 2000),
                     lambdas: Sequence[float] = (1.0, 0.75, 0.5, 0.25, 0.0)) -> List[JobSpec]:
    """Poisson arrivals at ``rate`` jobs/s; solute uniform over
    ``system.SOLUTES``, water count uniform in [nwater[0], nwater[1]]."""
    rng = np.random.default_rng(seed)
    t = 0.0
    jobs = []
    for i in range(n_jobs):
        t += rng.exponential(1.0 / rate) if rate > 0 else 0.0
        sol = S.SOLUTES[int(rng.integers(len(S.SOLUTES)))]
        nw = int(rng.integers(nwater[0], nwater[1] + 1))
        jobs.append(JobSpec(f"job{i:03d}-{sol}-{nw}", S.solvation_job(sol, nw),
                            lambdas=tuple(lambdas), steps_per_state=steps_per_state,
                            seed=seed * 1000 + i, arrival=t))
    return jobs


def latency_stats(results: Sequence[JobResult], wall: float) -> dict:
    lat = np.array([r.latency for r in results])
    steps = sum(r.atom_steps for r in results)
    return {"jobs": len(results), "p50_s": float(np.percentile(lat, 50)),
            "p99_s": float(np.percentile(lat, 99)), "max_s": float(lat.max()),
            "atom_steps": int(steps), "wall_s": wall, "atom_steps_per_s": steps / wall}
