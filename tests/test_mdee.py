"""Expanded-ensemble moves: DIFFUR / DIFEN (mdee.f:265-536) on the GPU against
the oracle's restatement, the restatement's own consistency, DIFF_LRCOR, and
a CHENS walk over the device state."""
import numpy as np
import pytest

import oracle
from mdynamix_gb300 import mdee
from mdynamix_gb300 import system as S
from mdynamix_gb300.abi import MDX_FP64, MDX_MIXED

PW1, PW2, BEE = 1.0, 1.0 / 3.0, 3.0


def job(solute="CH3OH", nwater=300):
    spec = S.solvation_job(solute, nwater)
    s = S.System(spec)
    return s, S.make_configuration(s, seed=4, jitter=0.05)


def _oracle(s, st, ec):
    o = oracle.Oracle(s)
    p = o.packed.params
    p.lmdee = 1
    o.L.ox_set_params(o.h, p)
    o.set_state(*st)
    o.set_lambda(ec, PW1, PW2, BEE)
    o.chcnb()
    o.allforce()
    return o


def test_oracle_ee_delta_is_consistent_between_states():
    """DIFFUR/DIFEN from a to b give, as the 'new' energies, what the same
    routines give as the 'old' energies once the system sits at b."""
    s, st = job()
    a, b = 0.75, 0.5
    o = _oracle(s, st, a)
    efn, efo, een, eeo = o.ee_delta(a, b, PW1, PW2, BEE)
    o.set_lambda(b, PW1, PW2, BEE)
    efn2, efo2, een2, eeo2 = o.ee_delta(b, a, PW1, PW2, BEE)
    for x, y in ((efo2, efn), (eeo2, een), (efn2, efo), (een2, eeo)):
        assert abs(x - y) <= 1e-11 * max(abs(x), abs(y))
    assert efn != efo and een != eeo


def test_ee_lrc_is_a_quarter_of_elrclj_at_full_coupling():
    """DIFF_LRCOR takes EP = A6^2 / (4 B12) where ELRCLJ takes A6^2 / B12
    (mdee.f:580 against forces.f:1717); at EC = 1 the two sums differ by
    exactly that factor."""
    s, _ = job()
    pel, _ = S.lrc_per_pair(s)
    e = mdee.ee_lrc(s, [1.0, 0.5], 1, PW1, PW2, BEE)
    assert abs(e[0] - 0.25 * pel.sum()) <= 1e-12 * abs(e[0])
    assert e[1] != e[0]


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [MDX_FP64, MDX_MIXED])
def test_ee_delta_matches_oracle(precision):
    from mdynamix_gb300.mdx import ForcePath
    s, st = job()
    tol = 1e-10 if precision == MDX_FP64 else 1e-5
    for a, b in ((1.0, 0.75), (0.5, 0.25), (0.25, 0.0)):
        o = _oracle(s, st, a)
        g = ForcePath(s, precision=precision)
        p = g.packed.params
        p.lmdee = 1
        g.set_params(p)
        g.set_state(*st)
        g.set_lambda(a, PW1, PW2, BEE)
        g.chcnb()
        g.allforce()
        rg = g.ee_delta(a, b, PW1, PW2, BEE)
        ro = o.ee_delta(a, b, PW1, PW2, BEE)
        for x, y in zip(rg, ro):
            assert abs(x - y) <= tol * abs(y), (a, b, rg, ro)
        # the differences the Metropolis rule uses
        assert abs((rg[0] - rg[1]) - (ro[0] - ro[1])) <= tol * abs(ro[1])
        assert abs((rg[2] - rg[3]) - (ro[2] - ro[3])) <= tol * abs(ro[3])
        g.close()


@pytest.mark.gpu
def test_mdee_walk_moves_between_subensembles():
    """A CHENS walk over 5 couplings (EC 1 .. 0), a move every 2 long steps;
    after a move the device interactions are those of the new subensemble."""
    from mdynamix_gb300.mdx import ForcePath
    s, st = job(nwater=200)
    g = ForcePath(s)
    p = g.packed.params
    p.lmdee = 1
    g.set_params(p)
    g.set_state(*st)
    walk = mdee.MdeeWalk(s, ec=[1.0, 0.75, 0.5, 0.25, 0.0], me=3, seed=2, wl_corr=0.5)
    walk.apply(g)
    g.double(2, records=False)
    for k in range(20):
        walk.attempt(g)
        g.double_steps(2, 2 + 2 * k, records=False)
    assert walk.attempts == 20 and walk.accepted > 0
    assert 1 <= walk.me <= 5 and sum(walk.visits) == 20
    # the interactions now in use are RECINT's at the walk's coupling
    g.chcnb()
    g.allforce()
    o = _oracle(s, g.get_state()[0], walk.ec[walk.me - 1])
    assert np.abs(g.forces(3) - o.forces(3)).max() <= 1e-10 * np.abs(o.forces(3)).max()


@pytest.mark.gpu
def test_walk_jobs_same_alone_and_in_the_mix():
    """Serving jobs that walk between couplings (CHENS every 2 long steps):
    on the mixed path (deterministic) a job's walk and final state are the
    same run alone and among other jobs."""
    import dataclasses
    from mdynamix_gb300 import serve
    jobs = serve.solvation_stream(3, rate=0.0, seed=5, steps_per_state=2, nwater=(150, 260))
    jobs = [dataclasses.replace(j, walk_ncee=2, walk_moves=6) for j in jobs]
    preps = [serve.prepare(j) for j in jobs]
    mix = serve.Server(precision=MDX_MIXED, slots=8, keep_states=True).run(preps)
    alone = serve.Server(precision=MDX_MIXED, slots=1, keep_states=True).run(preps[1:2])
    a = next(r for r in mix if r.name == jobs[1].name)
    b = alone[0]
    assert [s["me"] for s in a.states] == [s["me"] for s in b.states]
    assert len(a.states) == 7
    for x, y in zip(a.states[-1]["state"], b.states[-1]["state"]):
        assert np.array_equal(x, y)


@pytest.mark.gpu
@pytest.mark.parametrize("icell", [1, 2])
def test_ee_delta_cell_shapes(icell):
    """DIFFUR / DIFEN in the truncated octahedron and the hexagonal cell:
    the cell's k-set (octahedral columns of one nz parity, the hexagonal
    RYV) and minimum image (mdee.f:351, 432, 502), FP64 against the
    oracle."""
    import dataclasses
    from mdynamix_gb300.mdx import ForcePath
    spec = dataclasses.replace(S.solvation_job("CH3OH", 300), icell=icell)
    s = S.System(spec)
    st = S.make_configuration(s, seed=4, jitter=0.05)
    a, b = 0.75, 0.5
    o = _oracle(s, st, a)
    g = ForcePath(s, precision=MDX_FP64)
    p = g.packed.params
    p.lmdee = 1
    g.set_params(p)
    g.set_state(*st)
    g.set_lambda(a, PW1, PW2, BEE)
    g.chcnb()
    g.allforce()
    rg = g.ee_delta(a, b, PW1, PW2, BEE)
    ro = o.ee_delta(a, b, PW1, PW2, BEE)
    for x, y in zip(rg, ro):
        assert abs(x - y) <= 1e-10 * abs(y), (rg, ro)
    g.close()
