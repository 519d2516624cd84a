"""GPU path against the CPU oracle, through the C ABI (FP64 and mixed)."""
import numpy as np
import pytest

import oracle
from mdynamix_gb300.abi import MDX_FP64, MDX_MIXED
from mdynamix_gb300.mdx import ForcePath, MdxError
from tests import systems

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10      # relative, forces / energies / virials (FP64 drop-in bar)
MIXED_TOL = 1e-5      # relative RMS force error of the mixed path

def _short_beyond_cut():
    # R_short above R_cutoff: CHCNB still files every pair within SHORT in
    # the short list (forces.f:1964-1976)
    spec = systems.spcfw(n=125, ions=0, rcut=5.5)
    spec.rshort = 6.0
    return systems.build(spec)


def _bilayer_patch():
    # one DMPC per leaflet (118 atoms: bonds, angles, torsions, 1-4 pairs,
    # SHAKE on a 118-atom molecule) in SPC water
    from mdynamix_gb300 import system as S
    spec = S.dmpc_bilayer(nside=1, nwater=500, box=(20.0, 20.0, 60.0), rcut=9.0,
                          alpha=2.8, fexp=9.0)
    s = S.System(spec)
    return s, S.bilayer_configuration(s, seed=2)


CASES = {
    "spce_ions": lambda: systems.build(systems.spce_ions()),
    "bilayer_patch": _bilayer_patch,
    "short_beyond_cut": _short_beyond_cut,
    "spcfw": lambda: systems.build(systems.spcfw()),
    "organics": lambda: systems.build(systems.organics()),
}


def pair(name, precision=MDX_FP64):
    s, st = CASES[name]()
    g = ForcePath(s, precision=precision)
    o = oracle.Oracle(s)
    g.set_state(*st)
    o.set_state(*st)
    return s, st, g, o


def relmax(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("name", list(CASES))
def test_lists_bit_exact(name):
    s, st, g, o = pair(name)
    assert g.chcnb() == o.chcnb()
    (gs1, gs2), (gl1, gl2) = g.lists()
    o.chcnb_counts = o.chcnb()
    (os1, os2), (ol1, ol2) = o.lists()
    assert np.array_equal(gs1, os1) and np.array_equal(gs2, os2)
    assert np.array_equal(gl1, ol1) and np.array_equal(gl2, ol2)
    assert (gs1 < 0).sum() == (os1 < 0).sum()


SCAL = ["pe1", "pels1", "pe2", "pels2", "spe", "pint", "qpe", "vir1", "vir2", "virb",
        "virx", "viry", "virz", "virfx", "virfy", "virfz", "wirs", "wirss"]


def check_scalars(a, b, names, tol, scale):
    for n in names:
        x, y = getattr(a, n), getattr(b, n)
        assert abs(x - y) <= tol * max(abs(y), scale), (n, x, y)


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("routine", ["fforces", "slforces", "allforce"])
def test_forces_fp64(name, routine):
    s, st, g, o = pair(name)
    g.chcnb(); o.chcnb()
    g.getcom(); o.getcom()
    a = getattr(g, routine)()
    b = getattr(o, routine)()
    which = {"fforces": 1, "slforces": 2, "allforce": 3}[routine]
    assert relmax(g.forces(which), o.forces(which)) < FP64_TOL
    scale = max(abs(getattr(b, n)) for n in ("pe1", "pels1", "pe2", "pels2", "pint"))
    check_scalars(a, b, SCAL, FP64_TOL, 1e-6 * scale)
    for n in ("pote1", "potl1", "pes141", "psr141", "spee"):
        x, y = np.array(getattr(a, n)), np.array(getattr(b, n))
        assert np.abs(x - y).max() <= FP64_TOL * max(np.abs(y).max(), 1e-6 * scale), n


@pytest.mark.parametrize("name", ["spcfw", "organics"])
def test_double_fp64(name):
    s, st, g, o = pair(name)
    rg = g.double(3)
    ro = o.double(3)
    (gx, gy, gz, vx, vy, vz), tg = g.get_state()
    (ox, oy, oz, wx, wy, wz), to = o.get_state()
    dpos = max(np.abs(gx - ox).max(), np.abs(gy - oy).max(), np.abs(gz - oz).max())
    assert dpos < 1e-9
    assert relmax(np.stack([vx, vy, vz]), np.stack([wx, wy, wz])) < 1e-8
    for a, b in zip(rg, ro):
        for n in ("pe1", "pels1", "pe2", "pels2", "pint", "tke", "temp", "tryck", "sc"):
            assert abs(getattr(a, n) - getattr(b, n)) <= 1e-8 * max(abs(getattr(b, n)), 1e-12), n


def test_double_mixed_tracks_fp64():
    """Mixed DOUBLE long steps stay on the FP64 trajectory: methanol and
    ethanol (more than four atoms: the per-molecule update) and water (the
    register path), a list rebuild inside the run (ICHNB 10); positions
    within 1e-5 A after 11 long steps, energies within 1e-4."""
    s, st = CASES["organics"]()
    out = {}
    for prec in (MDX_FP64, MDX_MIXED):
        g = ForcePath(s, precision=prec)
        g.set_state(*st)
        rec = g.double(11)
        (x, y, z, *_), _ = g.get_state()
        out[prec] = (np.stack([x, y, z]), rec)
        g.close()
    dpos = np.abs(out[MDX_MIXED][0] - out[MDX_FP64][0]).max()
    assert dpos < 1e-5, dpos
    for a, b in zip(out[MDX_MIXED][1], out[MDX_FP64][1]):
        for n in ("pe1", "pels1", "pe2", "pels2", "pint", "tke"):
            assert abs(getattr(a, n) - getattr(b, n)) <= 1e-4 * max(abs(getattr(b, n)), 1e-9), n


@pytest.mark.parametrize("name", ["organics", "spce_ions"])
def test_getkin_chkmom_match_oracle(name):
    """GETKIN (molecules of 1 to 9 sites: the singular-tensor and
    single-atom branches too) and CHKMOM against the oracle."""
    s, st, g, o = pair(name)
    for x in (g, o):
        x.getcom()
    kg = g.getkin()
    ko = o.getkin()
    for n, v in zip(("ektr", "ekrot", "ekint", "tke", "ttr", "trot", "tint"), ko):
        assert abs(getattr(kg, n) - v) <= 1e-10 * max(abs(v), abs(ko[3])), n
    # a start with a net momentum (the seeded configuration has none)
    v = [st[3] + 0.3 * np.abs(st[3]).mean(), st[4] - 0.2 * np.abs(st[4]).mean(), st[5]]
    for x in (g, o):
        x.set_state(*st[:3], *v)
    dg, do = np.array(g.chkmom()), np.array(o.chkmom())
    assert np.abs(dg - do).max() <= 1e-10 * np.abs(do).max()
    (_, _, _, gx, gy, gz), tg = g.get_state()
    (_, _, _, ox, oy, oz), to = o.get_state()
    assert relmax(np.stack([gx, gy, gz]), np.stack([ox, oy, oz])) < 1e-12
    assert abs(tg.temp - to.temp) <= 1e-10 * to.temp


def test_sultan_shake_fp64():
    s, st, g, o = pair("spce_ions")
    rg = g.sultan(3)
    ro = o.sultan(3)
    (gx, gy, gz, *_), tg = g.get_state()
    (ox, oy, oz, *_), to = o.get_state()
    dpos = max(np.abs(gx - ox).max(), np.abs(gy - oy).max(), np.abs(gz - oz).max())
    assert dpos < 1e-9
    for a, b in zip(rg, ro):
        assert abs(a.temp - b.temp) <= 1e-8 * b.temp
        assert abs(a.pels1 - b.pels1) <= 1e-8 * abs(b.pels1)


def _npt_pair(spec):
    s, st = systems.build(spec)
    g = ForcePath(s)
    o = oracle.Oracle(s)
    g.set_state(*st)
    o.set_state(*st)
    return g, o


def _check_npt(g, o, rg, ro):
    (gx, gy, gz, *_), tg = g.get_state()
    (ox, oy, oz, *_), to = o.get_state()
    dpos = max(np.abs(gx - ox).max(), np.abs(gy - oy).max(), np.abs(gz - oz).max())
    assert dpos < 1e-9
    for a, b in zip(rg, ro):
        for n in ("boxl", "boyl", "bozl", "vol", "scl", "sc", "tryck", "temp", "pels1"):
            assert abs(getattr(a, n) - getattr(b, n)) <= 1e-8 * max(abs(getattr(b, n)), 1e-12), n
    assert ro[-1].vol != ro[0].vol  # the barostat moved the box


@pytest.mark.parametrize("aniso", [False, True])
def test_sultan_npt_fp64(aniso):
    """SULTAN + SHEJK with SCALING(3): Nose-Hoover NPT, isotropic or per axis
    (mdstep.f:534-1093)."""
    spec = systems.spce_ions()
    spec.nvt = (300.0, 30.0)
    spec.npt = (1.0, 500.0)
    spec.anisotropic = aniso
    g, o = _npt_pair(spec)
    rg, ro = g.sultan(5), o.sultan(5)
    _check_npt(g, o, rg, ro)


def test_sultan_npt_bilayer_fp64():
    """Lipid bilayer patch: SULTAN + SHEJK (118-atom molecule) with the
    anisotropic barostat."""
    s, st = _bilayer_patch()
    g = ForcePath(s)
    o = oracle.Oracle(s)
    g.set_state(*st)
    o.set_state(*st)
    rg, ro = g.sultan(3), o.sultan(3)
    _check_npt(g, o, rg, ro)
    assert [r.shake_iter for r in rg] == [r.shake_iter for r in ro]


@pytest.mark.parametrize("aniso", [False, True])
def test_double_npt_fp64(aniso):
    """DOUBLE with SCALING(1)/(2) in NPT (box rescaled every long step)."""
    spec = systems.spcfw()
    spec.npt = (1.0, 500.0)
    spec.anisotropic = aniso
    g, o = _npt_pair(spec)
    rg, ro = g.double(3), o.double(3)
    _check_npt(g, o, rg, ro)


@pytest.mark.parametrize("name", list(CASES))
def test_mixed_force_error(name):
    s, st = CASES[name]()
    g64 = ForcePath(s, precision=MDX_FP64)
    g32 = ForcePath(s, precision=MDX_MIXED)
    for g in (g64, g32):
        g.set_state(*st)
        g.chcnb()
        g.getcom()
    a = g64.allforce(); b = g32.allforce()
    for which in (1, 2, 3):
        f64, f32 = g64.forces(which), g32.forces(which)
        rms = np.sqrt(((f32 - f64) ** 2).sum() / (f64 ** 2).sum())
        assert rms < MIXED_TOL, (which, rms)
    for n in ("pe1", "pels1", "pe2", "pels2", "pint", "spe"):
        assert abs(getattr(a, n) - getattr(b, n)) <= 1e-4 * abs(getattr(a, n)) + 1e-9, n


@pytest.mark.parametrize("name", ["spce_ions", "spcfw", "bilayer_patch"])
def test_mixed_ewald_tensor_core_passes(name, monkeypatch):
    """Tensor-core reciprocal passes (3 x TF32 products) against the CUDA-core
    FP32 passes and the FP64 path: MDX_EWALD_TC=1 (force pass, the default)
    and 2 (force pass and S(k)) keep the forces within the mixed bar and
    within 2e-6 of the FP32 passes; the default keeps the reciprocal energy
    of the FP32 passes (S(k) is the same kernel); the tensor-core S(k) keeps
    it within 1e-4."""
    s, st = CASES[name]()
    out, en = {}, {}
    for tc in ("0", "1", "2"):
        monkeypatch.setenv("MDX_EWALD_TC", tc)
        g = ForcePath(s, precision=MDX_MIXED)
        g.set_state(*st)
        g.chcnb()
        g.getcom()
        en[tc] = g.allforce().pels1
        out[tc] = g.forces(3)
        g.close()
    g64 = ForcePath(s, precision=MDX_FP64)
    g64.set_state(*st)
    g64.chcnb()
    g64.getcom()
    e64 = g64.allforce().pels1
    f64 = g64.forces(3)
    nrm = np.sqrt((f64 ** 2).sum())
    for tc, f in out.items():
        assert np.sqrt(((f - f64) ** 2).sum()) / nrm < MIXED_TOL, tc
    for tc in ("1", "2"):
        assert np.sqrt(((out[tc] - out["0"]) ** 2).sum()) / nrm < 2e-6, tc
    assert en["1"] == en["0"]
    assert abs(en["2"] - e64) <= 1e-4 * abs(e64)


def test_mixed_deterministic():
    s, st = CASES["spcfw"]()
    outs = []
    for _ in range(2):
        g = ForcePath(s, precision=MDX_MIXED)
        g.set_state(*st)
        g.double(2, records=False)
        (x, y, z, *_), _ = g.get_state()
        outs.append(np.stack([x, y, z]))
    assert np.array_equal(outs[0], outs[1])


def test_list_overflow_is_an_error():
    s, st = CASES["spcfw"]()
    g = ForcePath(s, cap_short=4, cap_long=16)
    g.set_state(*st)
    with pytest.raises(MdxError) as e:
        g.chcnb()
    assert e.value.code == 3 and "overfilled" in str(e.value)


def test_call_order_is_an_error():
    s, st = CASES["spcfw"]()
    g = ForcePath(s)
    with pytest.raises(MdxError) as e:
        g.chcnb()
    assert e.value.code == 7


def test_set_lambda_matches_oracle():
    s, st = systems.build(systems.__dict__["organics"]().__class__(
        molecules=[("SPC-FW", 100), ("CH3OH", 1)], density=1.0, dt_fs=2.0, nfreq=10,
        rcut=7.0, rshort=5.0, alpha=2.0, fexp=9.0, ichnb=10, nvt=(298.0, 30.0),
        iee_type=2))
    g = ForcePath(s)
    o = oracle.Oracle(s)
    g.packed.params.lmdee = 1
    o_params = o.packed.params
    o_params.lmdee = 1
    g.set_params(g.packed.params)
    o.L.ox_set_params(o.h, o_params)
    g.set_state(*st); o.set_state(*st)
    g.set_lambda(0.5); o.set_lambda(0.5)
    g.chcnb(); o.chcnb()
    g.allforce(); o.allforce()
    assert relmax(g.forces(3), o.forces(3)) < FP64_TOL
    # a later state upload keeps the scaled charges (they go up only once)
    g.set_state(*st); o.set_state(*st)
    g.chcnb(); o.chcnb()
    g.allforce(); o.allforce()
    assert relmax(g.forces(3), o.forces(3)) < FP64_TOL


def test_graph_replay_matches_eager(monkeypatch):
    """Long steps replayed from captured CUDA graphs give the same state and
    records as eager launches (mixed path: bit for bit)."""
    s, st = CASES["spcfw"]()
    runs = []
    for graphs in ("1", "0"):
        monkeypatch.setenv("MDX_GRAPHS", graphs)
        g = ForcePath(s, precision=MDX_MIXED)
        g.set_state(*st)
        rec = g.double(12)
        (x, y, z, *_), th = g.get_state()
        runs.append((np.stack([x, y, z]), [r.temp for r in rec], [r.mstep for r in rec]))
    assert np.array_equal(runs[0][0], runs[1][0])
    assert runs[0][1] == runs[1][1]
    assert runs[0][2] == list(range(1, 13))


def _bilayer_patch_hbonds():
    from mdynamix_gb300 import system as S
    spec = S.dmpc_bilayer(nside=1, nwater=500, box=(20.0, 20.0, 60.0), rcut=9.0,
                          alpha=2.8, fexp=9.0, shake_hbonds=True)
    s = S.System(spec)
    return s, S.bilayer_configuration(s, seed=2)


@pytest.mark.parametrize("npt", [False, True])
def test_sultan_shake_hbonds_bilayer_fp64(npt):
    """SHAKE on the bonds to hydrogen only (a per-record constraint flag the
    reference cannot express; its ID != 2 rule constrains every bond of a
    type): the lipid's constraints fall into small independent clusters,
    each iterated on its own on the GPU; positions, SHAKE iteration counts
    and the NPT box follow the oracle's molecule-wide sweeps."""
    s, st = _bilayer_patch_hbonds()
    if not npt:
        import dataclasses
        from mdynamix_gb300 import system as S
        s = S.System(dataclasses.replace(s.spec, npt=None, anisotropic=False))
    g = ForcePath(s)
    o = oracle.Oracle(s)
    g.set_state(*st)
    o.set_state(*st)
    rg, ro = g.sultan(3), o.sultan(3)
    (gx, gy, gz, *_), tg = g.get_state()
    (ox, oy, oz, *_), to = o.get_state()
    assert max(np.abs(gx - ox).max(), np.abs(gy - oy).max(), np.abs(gz - oz).max()) < 1e-9
    assert [r.shake_iter for r in rg] == [r.shake_iter for r in ro]
    for a, b in zip(rg, ro):
        for n in ("temp", "pels1", "boxl", "tryck"):
            assert abs(getattr(a, n) - getattr(b, n)) <= 1e-8 * max(abs(getattr(b, n)), 1e-12), n


def test_mixed_sweep_splits():
    """Every work split of the mixed pair sweeps (threads per owner atom):
    forces within the mixed bar of FP64 and within 1e-6 of the default
    split, the same split twice bit for bit (also through the step graphs,
    which a change of split recaptures), and the table's choice restored by
    set_tuning()."""
    s, st = CASES["spcfw"]()
    g64 = ForcePath(s, precision=MDX_FP64)
    g64.set_state(*st)
    g64.chcnb()
    g64.getcom()
    g64.allforce()
    f64 = g64.forces(3)
    nrm = np.sqrt((f64 ** 2).sum())
    g = ForcePath(s, precision=MDX_MIXED)
    g.set_state(*st)
    g.chcnb()
    g.getcom()
    g.allforce()
    t0 = g.tuning()
    assert t0["source"] == 1 and t0["tpo_short"] in (2, 4, 8) and t0["tpo_long"] in (4, 8, 16, 32)
    f0 = g.forces(3)
    for ts, tl in ((2, 8), (8, 16), (4, 32), (8, 32)):
        g.set_tuning(ts, tl)
        assert g.tuning() == {"tpo_short": ts, "tpo_long": tl, "source": 2}
        g.allforce()
        f = g.forces(3)
        assert np.sqrt(((f - f64) ** 2).sum()) / nrm < MIXED_TOL, (ts, tl)
        assert np.sqrt(((f - f0) ** 2).sum()) / nrm < 1e-6, (ts, tl)
        g.allforce()
        assert np.array_equal(g.forces(3), f), (ts, tl)
    with pytest.raises(MdxError):
        g.set_tuning(3, 32)
    g.set_tuning()
    assert g.tuning() == t0
    outs = []
    for split in ((2, 16), (2, 16), None):
        h = ForcePath(s, precision=MDX_MIXED)
        h.set_state(*st)
        if split:
            h.set_tuning(*split)
        h.double(3, records=False)
        (x, y, z, *_), _ = h.get_state()
        outs.append(np.stack([x, y, z]))
        h.close()
    assert np.array_equal(outs[0], outs[1])
    assert np.abs(outs[0] - outs[2]).max() < 1e-6


@pytest.mark.parametrize("icell", [1, 2])
def test_npt_cell_shapes_fp64(icell):
    """NPT in the truncated octahedron and the hexagonal cell: RECLEN keeps
    the cell's shape (service.f:576-585) and the octahedron's half-cube
    volume; SULTAN + SHEJK and DOUBLE against the oracle."""
    import dataclasses
    spec = dataclasses.replace(systems.spce_ions(n=200, toler=1e-6), icell=icell,
                               nvt=(300.0, 30.0), npt=(1.0, 500.0))
    g, o = _npt_pair(spec)
    rg, ro = g.sultan(5), o.sultan(5)
    _check_npt(g, o, rg, ro)
    if icell == 2:
        assert abs(rg[-1].boyl - rg[-1].boxl * 0.8660254037844386) < 1e-6 * rg[-1].boxl
    else:
        assert rg[-1].boxl == rg[-1].boyl == rg[-1].bozl
        assert abs(rg[-1].vol - 0.5 * rg[-1].boxl ** 3) < 1e-9 * rg[-1].vol
    spec2 = dataclasses.replace(systems.spcfw(n=256, ions=2, rcut=8.0), icell=icell,
                                npt=(1.0, 500.0))
    g2, o2 = _npt_pair(spec2)
    rg2, ro2 = g2.double(3), o2.double(3)
    _check_npt(g2, o2, rg2, ro2)
