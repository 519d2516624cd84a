"""The reference's own example run as the parity pin.

sample/4nacl.in (256 flexible SPC waters + 4 Na+_SD + 4 Cl-_SD), the restart
file its run wrote (sample/NaCl.dmp, 776 atoms with momenta) and the numbers
its output prints (sample/4nacl.out) are committed as fixtures under
tests/golden/ (made by tests/golden/make_nacl_fixture.py).

- CPU: the numbers 4nacl.out prints that follow from the input alone (box
  from the density, k-vector count of INIFUR, degrees of freedom, LJ tail
  corrections per type pair) against this build's setup; the restart-file
  reader and writer.
- GPU: from the reference's own configuration, lists bit for bit, FP64
  forces / energies / virials at 1e-10 with SCLFRC armed (and cutting), the
  bonded statistics, the mixed error, DOUBLE steps against the oracle.
- GPU, statistics: a 24 ps continuation of the reference's run (from its
  restart file) in FP64 and in mixed precision; the averages agree with the
  final averages the reference printed, within the error bars.
"""
import math
import os

import numpy as np
import pytest

import oracle
from mdynamix_gb300 import restart
from mdynamix_gb300 import system as S
from mdynamix_gb300.abi import MDX_FP64, MDX_MIXED
from tests.nacl776 import (AGREE, REF, agrees, load_sample, reference_averages,
                           sample_run_averages)

FP64_TOL = 1e-10

# ------------------------------------------------------------------- CPU --
def test_sample_setup_matches_reference_output():
    """Box from Density 1.02, INIFUR's k-vector count, the degrees of
    freedom and the tail corrections as 4nacl.out prints them."""
    s_dens = S.System(S.nacl_sample())
    assert s_dens.nstot == REF["nstot"] and s_dens.nop == REF["nop"]
    # printed as 0.199064D+02; the restart file holds 19.906419..
    assert abs(s_dens.boxl - REF["dmp"]["box"][0]) < 2e-7 * REF["dmp"]["box"][0]
    assert round(s_dens.boxl, 4) == REF["box"][0]
    s, _, _ = load_sample()
    assert s.kvector_count() == REF["nkv"]
    assert (s.fnst, s.fttr, s.fnstr, s.fnsti) == (REF["fnst"], REF["fttr"], REF["fnstr"],
                                                 REF["fnsti"])
    pel, vrl = S.lrc_per_pair(s)
    # "PE LRC 1" (F12.8) and "PR LRC 1" (F12.4): the water-water pair
    assert abs(pel[0] * s.permol - REF["pe_lrc_kj_mol"]) <= 1e-8
    assert abs(vrl[0] * s.unitp / (3.0 * s.vol) - REF["pr_lrc_atm"]) <= 1e-4
    # "Out cutoff corr" per molecule-type pair: PELRC * TOKJ / min(NSPEC)
    # (aver.f:136-141), printed with 4 decimals
    names = [t["name"] for t in s.types]
    for it in range(s.ntypes):
        for jt in range(it, s.ntypes):
            key = f"{names[it]}-{names[jt]}"
            mt = s.mdx[it, jt] - 1
            v = pel[mt] * s.enerf * 1e-3 / min(s.nspec[it], s.nspec[jt])
            assert abs(v - REF["inter"][key]["lrc"]) <= 0.5e-4 + 1e-9, key


def test_restart_file_round_trip(tmp_path):
    s, st, th = load_sample()
    th.scl = 0.25
    r = restart.restart_from_state(s, st, th, nstep=10000, nsttot=10000, tim=2e-11)
    p = str(tmp_path / "x.dmp")
    restart.write_dmp(p, r)
    q = restart.read_dmp(p)
    assert (q.nop, q.ntypes, q.nstot, q.nsttot, q.label) == (264, 3, 776, 10000, "MDYN_v5.3")
    for a, b in zip(q.positions + q.momenta, st):
        assert np.array_equal(a, b)
    assert (q.sc, q.scl, q.boxl) == (th.sc, 0.25, th.boxl)
    # the records RESTRT writes: 7 framed records, coordinates interleaved
    raw = open(p, "rb").read()
    recs = restart._records(raw)
    assert [len(x) for x in recs] == [24, 24, 60, 8 * (10 + 3 + 1), 88, 18624, 18624]
    xyz = np.frombuffer(recs[5], "<f8").reshape(-1, 3)
    assert np.array_equal(xyz[:, 0], st[0]) and np.array_equal(xyz[:, 2], st[2])


def test_trace_xmol_format(tmp_path):
    s, st, th = load_sample()
    w = restart.TraceWriter(s, str(tmp_path / "NaCl"), itrek=2, ltrek=2)
    for k in range(3):
        w.add(st, 2e-11 + k * 2e-13, (th.boxl, th.boyl, th.bozl))
    w.close()
    assert [os.path.basename(f) for f in w.files] == ["NaCl.001", "NaCl.002"]
    lines = open(w.files[0]).read().splitlines()
    assert int(lines[0]) == 776 and len(lines) == 2 * 778
    assert lines[1].startswith(" after        20000.00 fs, BOX:")
    assert lines[2].split()[0] == "O" and abs(float(lines[2].split()[1]) - st[0][0]) < 6e-4


# ------------------------------------------------------------------- GPU --
def _pair(precision=MDX_FP64):
    from mdynamix_gb300.mdx import ForcePath
    s, st, th = load_sample()
    g = ForcePath(s, precision=precision)
    g.set_state(*st, thermo=th)
    o = oracle.Oracle(s)
    o.set_state(*st, thermo=th)
    return s, st, th, g, o


def relmax(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


SCAL = ["pe1", "pels1", "pe2", "pels2", "spe", "pint", "qpe", "vir1", "vir2", "virb",
        "virx", "viry", "virz", "virfx", "virfy", "virfz", "wirs", "wirss"]


@pytest.mark.gpu
def test_sample_lists_bit_exact():
    s, st, th, g, o = _pair()
    assert g.chcnb() == o.chcnb()
    (gs1, gs2), (gl1, gl2) = g.lists()
    (os1, os2), (ol1, ol2) = o.lists()
    assert np.array_equal(gs1, os1) and np.array_equal(gs2, os2)
    assert np.array_equal(gl1, ol1) and np.array_equal(gl2, ol2)


@pytest.mark.gpu
@pytest.mark.parametrize("routine", ["fforces", "slforces", "allforce"])
def test_sample_forces_fp64(routine):
    s, st, th, g, o = _pair()
    g.chcnb(); o.chcnb()
    g.getcom(); o.getcom()
    a = getattr(g, routine)()
    b = getattr(o, routine)()
    which = {"fforces": 1, "slforces": 2, "allforce": 3}[routine]
    assert relmax(g.forces(which), o.forces(which)) < FP64_TOL
    scale = max(abs(getattr(b, n)) for n in ("pe1", "pels1", "pe2", "pels2", "pint"))
    for n in SCAL:
        x, y = getattr(a, n), getattr(b, n)
        assert abs(x - y) <= FP64_TOL * max(abs(y), 1e-6 * scale), (n, x, y)
    if routine != "fforces":
        assert a.nkv == REF["nkv"]
    assert a.lscfl == b.lscfl


@pytest.mark.gpu
def test_sample_sclfrc_cuts_like_oracle():
    """Cut_forces 1: an H pushed to 0.6 A of a neighbouring O makes SCLFRC
    scale forces (service.f:182-287) on the GPU as in the oracle."""
    s, st, th = load_sample()
    st = [a.copy() for a in st]
    o_idx, h_idx = 0, 3 * 37 + 1
    d = np.array([st[0][h_idx] - st[0][o_idx], st[1][h_idx] - st[1][o_idx],
                  st[2][h_idx] - st[2][o_idx]])
    d -= np.round(d / s.boxl) * s.boxl
    for k in range(3):
        st[k][h_idx] = st[k][o_idx] + 0.6 * d[k] / np.linalg.norm(d)
    from mdynamix_gb300.mdx import ForcePath
    g, o = ForcePath(s), oracle.Oracle(s)
    for x in (g, o):
        x.set_state(*st, thermo=th)
        x.chcnb()
        x.getcom()
    a, b = g.allforce(), o.allforce()
    assert b.lscfl == 1 and a.lscfl == 1
    assert relmax(g.forces(3), o.forces(3)) < FP64_TOL


@pytest.mark.gpu
def test_sample_bonded_averages_match_oracle():
    s, st, th, g, o = _pair()
    g.chcnb(); o.chcnb()
    g.fforces(True); o.fforces(True)
    ag, ao = g.bonded_averages(), o.bonded_averages()
    for k in ("br", "be"):
        assert relmax(ag[k], ao[k]) < FP64_TOL, k
    # flexible SPC: O-H, O-H, H-H
    assert np.all(np.abs(ag["br"] - np.array([1.02, 1.02, 1.62])) < 0.02)


@pytest.mark.gpu
def test_sample_mixed_force_error():
    from mdynamix_gb300.mdx import ForcePath
    s, st, th = load_sample()
    f = {}
    for prec in (MDX_FP64, MDX_MIXED):
        g = ForcePath(s, precision=prec)
        g.set_state(*st, thermo=th)
        g.chcnb()
        g.getcom()
        g.allforce()
        f[prec] = g.forces(3)
    rms = np.sqrt(((f[MDX_MIXED] - f[MDX_FP64]) ** 2).sum() / (f[MDX_FP64] ** 2).sum())
    assert rms < 1e-5, rms


@pytest.mark.gpu
def test_sample_double_tracks_oracle():
    """Three DOUBLE long steps continuing the reference's run (NVT, NFREQ
    10, SCLFRC armed) against the oracle."""
    s, st, th, g, o = _pair()
    rg, ro = g.double(3, nsttot=10000), o.double(3, nsttot=10000)
    (gx, gy, gz, *_), tg = g.get_state()
    (ox, oy, oz, *_), to = o.get_state()
    assert max(np.abs(gx - ox).max(), np.abs(gy - oy).max(), np.abs(gz - oz).max()) < 1e-9
    for a, b in zip(rg, ro):
        for n in ("pe1", "pels1", "pe2", "pels2", "pint", "tke", "temp", "tryck", "sc"):
            assert abs(getattr(a, n) - getattr(b, n)) <= 1e-8 * max(abs(getattr(b, n)), 1e-12), n


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [MDX_FP64, MDX_MIXED])
def test_sample_run_averages_agree_with_reference(precision):
    """24 ps continuing the reference's run from its restart file: the
    averages agree with those the reference printed (bars in
    tests/nacl776.py: statistical for temperature and pressure, absolute for
    the energies and bond statistics, whose reference values still drift or
    hang on slow ion-pair moves).  Statistical agreement is the bar the
    reference's sample/Sample sets itself: its trajectory is v5.0 built with
    -ffast-math and is not reproducible bit for bit."""
    ours = sample_run_averages(precision)
    ref = reference_averages()
    for k in AGREE:
        assert agrees(k, ours[k], ref[k]), (k, ours[k], ref[k])


@pytest.mark.gpu
def test_snapshot_dumper_writes_device_state(tmp_path):
    """Restart file and XMOL frames written from device snapshots while the
    step loop goes on: the restart file read back equals the state after the
    last block, each frame the positions at its request."""
    from mdynamix_gb300.mdx import ForcePath
    s, st, th = load_sample()
    g = ForcePath(s)
    g.set_state(*st, thermo=th)
    g.double(0)
    tw = restart.TraceWriter(s, str(tmp_path / "NaCl"), itrek=2, ltrek=100)
    d = restart.SnapshotDumper(g, trace=tw)
    frames = []
    for b in range(3):
        g.double_steps(5, 5 * b, records=False)
        d.request("trace", time_s=(b + 1) * 5 * 2e-15)
        frames.append(g.get_state()[0])
    path = str(tmp_path / "NaCl.dmp")
    d.request("restart", path=path, nstep=15, nsttot=10015, tim=2.003e-11)
    d.close()
    (x, y, z, vx, vy, vz), th_end = g.get_state()
    r = restart.read_dmp(path)
    assert np.array_equal(r.sx, x) and np.array_equal(r.vz, vz)
    assert r.nsttot == 10015 and r.sc == th_end.sc
    lines = open(tw.files[0]).read().splitlines()
    assert len(lines) == 3 * 778
    for b in range(3):
        first = lines[b * 778 + 2].split()
        assert abs(float(first[1]) - frames[b][0][0]) < 6e-4
