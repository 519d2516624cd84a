"""Verlet-skin list mode (a list mode of this library, not of the reference):
rows reach RCUT + skin, the long-row sweeps skip pairs beyond RCUT, and the
lists are rebuilt once an atom has moved half the skin.

At the configuration of a build, skin mode and the reference's list mode
evaluate the same pairs, so their forces agree; along a trajectory the GPU
follows the oracle's restatement of the same mode."""
import dataclasses

import numpy as np
import pytest

import oracle
from mdynamix_gb300 import system as S
from mdynamix_gb300.abi import MDX_FP64, MDX_MIXED
from tests import systems

FP64_TOL = 1e-10
MIXED_TOL = 1e-5


def _spec(rskin, n=512):
    # 512 SPC-FW waters + ions: a 24.8 A box, so RCUT 9 + skin 1.5 stays
    # within half the box
    return dataclasses.replace(systems.spcfw(n=n, rcut=9.0), rskin=rskin)


def _pairs(l1, l2):
    return set(zip(np.abs(l1).tolist(), l2.tolist()))


def relmax(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def test_oracle_skin_forces_equal_reference_mode():
    """The oracle's skin mode: same short list, a long list that holds the
    reference's, and the same forces and energies at the build
    configuration."""
    s0, st = systems.build(_spec(0.0))
    s1 = S.System(_spec(1.5))
    out = []
    for s in (s0, s1):
        o = oracle.Oracle(s)
        o.set_state(*st)
        o.chcnb()
        o.getcom()
        sc = o.allforce()
        out.append((o.lists(), o.forces(3), sc))
    (rs, rl), f0, a = out[0]
    (ss, sl), f1, b = out[1]
    assert np.array_equal(rs[0], ss[0]) and np.array_equal(rs[1], ss[1])
    assert _pairs(*rl) < _pairs(*sl)
    assert relmax(f1, f0) < 1e-12
    for n in ("pe1", "pels1", "vir1", "virx", "wirs"):
        assert abs(getattr(a, n) - getattr(b, n)) <= 1e-12 * abs(getattr(a, n)), n


@pytest.mark.gpu
def test_skin_lists_and_forces_match_reference_mode():
    from mdynamix_gb300.mdx import ForcePath
    s0, st = systems.build(_spec(0.0))
    s1 = S.System(_spec(1.5))
    g0, g1, g1m = ForcePath(s0), ForcePath(s1), ForcePath(s1, precision=MDX_MIXED)
    res = []
    for g in (g0, g1, g1m):
        g.set_state(*st)
        g.chcnb()
        g.getcom()
        res.append((g.lists(), g.allforce(), g.forces(3)))
    (rs, rl), a, f0 = res[0]
    (ss, sl), b, f1 = res[1]
    assert np.array_equal(rs[0], ss[0]) and np.array_equal(rs[1], ss[1])
    assert _pairs(*rl) < _pairs(*sl)  # the skin adds pairs out to RCUT + 1.5
    assert relmax(f1, f0) < FP64_TOL
    for n in ("pe1", "pels1", "vir1", "virx", "viry", "virz", "wirs"):
        assert abs(getattr(a, n) - getattr(b, n)) <= FP64_TOL * abs(getattr(a, n)), n
    # skin lists of the mixed path (full rows) hold the same pairs
    (ms, ml), c, fm = res[2]
    assert _pairs(*sl) == _pairs(*ml)
    rms = np.sqrt(((fm - f0) ** 2).sum() / (f0 ** 2).sum())
    assert rms < MIXED_TOL, rms


@pytest.mark.gpu
@pytest.mark.parametrize("graphs", ["1", "0"])
def test_skin_double_tracks_oracle(graphs, monkeypatch):
    """DOUBLE in skin mode (0.3 A skin: rebuilds inside the run, decided on
    the device) against the oracle's skin mode; the same number of builds."""
    from mdynamix_gb300.mdx import ForcePath
    monkeypatch.setenv("MDX_GRAPHS", graphs)
    s, st = systems.build(_spec(0.3, n=512))
    g = ForcePath(s)
    o = oracle.Oracle(s)
    g.set_state(*st)
    o.set_state(*st)
    rg, ro = g.double(8), o.double(8)
    (gx, gy, gz, *_), tg = g.get_state()
    (ox, oy, oz, *_), to = o.get_state()
    dpos = max(np.abs(gx - ox).max(), np.abs(gy - oy).max(), np.abs(gz - oz).max())
    assert dpos < 1e-9
    assert tg.list_builds == to.list_builds and to.list_builds >= 2
    for a, b in zip(rg, ro):
        for n in ("pe1", "pels1", "pe2", "pels2", "pint", "tke"):
            assert abs(getattr(a, n) - getattr(b, n)) <= 1e-8 * max(abs(getattr(b, n)), 1e-12), n


@pytest.mark.gpu
def test_skin_mixed_tracks_fp64():
    from mdynamix_gb300.mdx import ForcePath
    s, st = systems.build(_spec(0.3, n=512))
    out = []
    for prec in (MDX_FP64, MDX_MIXED):
        g = ForcePath(s, precision=prec)
        g.set_state(*st)
        g.double(8, records=False)
        (x, y, z, *_), th = g.get_state()
        out.append((np.stack([x, y, z]), th.list_builds))
        g.close()
    assert np.abs(out[0][0] - out[1][0]).max() < 1e-5
    assert out[0][1] >= 2


@pytest.mark.gpu
def test_skin_refuses_npt_and_oversized_radius():
    from mdynamix_gb300.mdx import ForcePath, MdxError
    spec = dataclasses.replace(_spec(1.0), npt=(1.0, 500.0))
    with pytest.raises(MdxError) as e:
        ForcePath(S.System(spec))
    assert e.value.code == 10
    with pytest.raises(MdxError) as e:
        ForcePath(S.System(_spec(4.0)))  # 9 + 4 A is above half of the 24.8 A box
    assert e.value.code == 1
