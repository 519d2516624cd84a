"""Path-integral MD over bead replicas (pimd.f): the oracle's ring-polymer
dynamics conserve the ring-polymer energy when the bead thermostats are off
(CPU), and the GPU bead coupling matches the oracle (GPU)."""
import os

import numpy as np
import pytest

import oracle
from mdynamix_gb300 import system as S
from mdynamix_gb300.abi import MDX_FP64, MDX_MIXED

FP64_TOL = 1e-10     # relative, bead positions / records after a few steps
MIXED_TOL = 1e-5     # relative RMS, bead forces of the mixed path


def small(nbeads=4, nwater=32, dt=0.25):
    spec = S.pimd_water(nwater=nwater, nbeads=nbeads)
    spec.rcut = 4.9          # 9.9 A box
    spec.rshort = 3.5
    spec.dt_fs = dt
    s = S.System(spec)
    return s, S.pimd_beads(s, seed=3)


def ring_energy(r, P):
    # sum over beads of KE + PE / P, plus the spring energy QEK
    return r.tke + r.pe / P + r.qek


def test_bead_masses_and_coupling_constants():
    s1 = S.System(S.pimd_water(nwater=8, nbeads=1))
    s4 = S.System(S.pimd_water(nwater=8, nbeads=4))
    np.testing.assert_allclose(s4.massdi, 4 * s1.massdi, rtol=1e-14)   # MASS / NBEADS
    p = S.pimd_params(s4)
    assert p.nbeads == 4 and p.jnh == 4
    assert p.fnh == pytest.approx(p.dqqt / 12.0)
    assert p.conveq == pytest.approx(s4.enerf * s4.tempf / 4)


def test_oracle_ring_polymer_conserves_energy():
    s, states = small()
    op = oracle.OraclePimd(s, states)
    op.pp.dqqt = 0.0           # bead thermostats off: Hamiltonian dynamics
    op.pp.fnh = 0.0
    recs = op.run(40)
    P = s.spec.nbeads
    e = np.array([ring_energy(r, P) for r in recs])
    ke = np.array([r.tke for r in recs])
    assert np.all(np.array([r.qek for r in recs]) > 0)
    assert e.std() < 0.02 * ke.std()
    assert abs(e[-5:].mean() - e[:5].mean()) < 0.02 * ke.std()


def test_oracle_bead_thermostat_pulls_toward_trtemp():
    s, states = small()
    op = oracle.OraclePimd(s, states)
    recs = op.run(30)
    assert np.all(np.isfinite(op.thermo))
    assert np.abs(op.thermo).max() > 0


# ------------------------------------------------------------------- GPU
def _gpu(s, states, precision=MDX_FP64):
    from mdynamix_gb300.mdx import PimdPath
    return PimdPath(s, states, precision=precision)


def relmax(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.gpu
def test_pimd_fp64_forces_match_oracle():
    # the preparation (pimd.f:48-72): CHCNB, GETCOM, SLFORCES, FFORCES,
    # forces / NBEADS, PIFORCES, on identical bead coordinates
    s, states = small()
    op = oracle.OraclePimd(s, states)
    op.run(0)
    gp = _gpu(s, states)
    gp.run(0)
    for g, o in zip(gp.beads, op.beads):
        assert relmax(g.forces(1), o.forces(1)) < FP64_TOL   # H: fast / P + springs
        assert relmax(g.forces(2), o.forces(2)) < FP64_TOL   # G: slow / P


# Bead coordinates cross between beads as REAL*4 (pimd.f:450-486): a
# last-bit difference of the FP64 paths can move a rounded coordinate by one
# single-precision ulp (~1e-7 relative), so trajectories agree to that level.
TRAJ_TOL = 1e-5


@pytest.mark.gpu
def test_pimd_fp64_trajectory_tracks_oracle():
    s, states = small()
    op = oracle.OraclePimd(s, states)
    ro = op.run(5)
    gp = _gpu(s, states)
    rg = gp.run(5)
    for a, b in zip(gp.states(), op.states()):
        assert relmax(np.stack(a), np.stack(b)) < TRAJ_TOL
    for x, y in zip(rg, ro):
        assert x.mstep == y.mstep
        for f in ("qek", "pe", "tke", "temp"):
            assert abs(getattr(x, f) - getattr(y, f)) <= TRAJ_TOL * abs(getattr(y, f)), f
    assert relmax(gp.thermo(), op.thermo) < TRAJ_TOL
    ro2 = op.steps(3, 5)
    rg2 = gp.steps(3, 5)
    assert [r.mstep for r in rg2] == [r.mstep for r in ro2] == [6, 7, 8]
    for a, b in zip(gp.states(), op.states()):
        assert relmax(np.stack(a), np.stack(b)) < TRAJ_TOL


@pytest.mark.gpu
def test_pimd_mixed_force_error():
    s, states = small()
    g64 = _gpu(s, states, MDX_FP64)
    g32 = _gpu(s, states, MDX_MIXED)
    g64.run(0)
    g32.run(0)
    num = den = 0.0
    for a, b in zip(g32.beads, g64.beads):
        fa = a.forces(1) + a.forces(2)
        fb = b.forces(1) + b.forces(2)
        num += ((fa - fb) ** 2).sum()
        den += (fb ** 2).sum()
    assert np.sqrt(num / den) < MIXED_TOL


@pytest.mark.gpu
def test_pimd_graph_replay_matches_eager(monkeypatch):
    s, states = small()
    a = _gpu(s, states, MDX_MIXED)
    ra = a.run(4)
    monkeypatch.setenv("MDX_GRAPHS", "0")
    b = _gpu(s, states, MDX_MIXED)
    rb = b.run(4)
    for x, y in zip(a.states(), b.states()):
        assert np.array_equal(np.stack(x), np.stack(y))
    assert [r.qek for r in ra] == [r.qek for r in rb]
