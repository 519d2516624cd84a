"""GPU against the oracle on the named configurations and on the torsion
forms no moldb molecule uses.

- The plain-method case as specified: 512 rigid SPC/E + 4 Na+ + 4 Cl-
  (1,544 atoms, 25.04 A box), R_cutoff 10, Ewald 2.8 / 9.84, SULTAN + SHEJK
  with TOLER 1e-8 taken literally (SHEJK squares it, mdstep.f:1119, so the
  bond lengths must meet 1e-16 relative: MAXIT is reached) and with TOLER
  1.4e-4 (about 1e-8 in length), NVE.
- GETTRS's MM3 (ITORS 1, forces.f:401-414), cosine-power (ITORS 5,
  forces.f:415-434) and improper (ITORS -1, forces.f:435-440) branches on a
  copy of ethanol whose dihedrals are switched to those forms.
"""
import copy
import dataclasses

import numpy as np
import pytest

import oracle
from mdynamix_gb300 import system as S
from mdynamix_gb300.abi import MDX_FP64, MDX_MIXED
from tests import systems

pytestmark = pytest.mark.gpu
FP64_TOL = 1e-10


def relmax(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def cfg1(toler=1e-8):
    s = S.System(dataclasses.replace(S.spce_nacl_nve(), toler=toler))
    return s, S.make_configuration(s, seed=1, jitter=0.05)


def _pair(s, st):
    from mdynamix_gb300.mdx import ForcePath
    g, o = ForcePath(s), oracle.Oracle(s, threads=4)
    g.set_state(*st)
    o.set_state(*st)
    return g, o


def test_cfg1_lists_and_forces():
    s, st = cfg1()
    assert s.nstot == 1544
    g, o = _pair(s, st)
    assert g.chcnb() == o.chcnb()
    (gs1, gs2), (gl1, gl2) = g.lists()
    (os1, os2), (ol1, ol2) = o.lists()
    assert np.array_equal(gs1, os1) and np.array_equal(gl1, ol1)
    assert np.array_equal(gs2, os2) and np.array_equal(gl2, ol2)
    g.getcom(); o.getcom()
    a, b = g.allforce(), o.allforce()
    assert relmax(g.forces(3), o.forces(3)) < FP64_TOL
    for n in ("pe1", "pels1", "pe2", "pels2", "spe", "vir1", "vir2", "virx", "wirs", "wirss"):
        assert abs(getattr(a, n) - getattr(b, n)) <= FP64_TOL * abs(getattr(b, n)), n


@pytest.mark.parametrize("toler", [1e-8, 1.4e-4])
def test_cfg1_sultan_shake_tracks_oracle(toler):
    """Three SULTAN steps: positions to 1e-9 A; the same SHAKE iteration
    counts (MAXIT + 1 = 2001 for the literal tolerance, every molecule
    reported as not converged, as mdstep.f:1264-1269 prints)."""
    s, st = cfg1(toler)
    g, o = _pair(s, st)
    rg, ro = g.sultan(3), o.sultan(3)
    (gx, gy, gz, *_), tg = g.get_state()
    (ox, oy, oz, *_), to = o.get_state()
    assert max(np.abs(gx - ox).max(), np.abs(gy - oy).max(), np.abs(gz - oz).max()) < 1e-9
    assert [r.shake_iter for r in rg] == [r.shake_iter for r in ro]
    if toler == 1e-8:
        assert all(r.shake_iter == 2001 for r in rg)
    else:
        assert all(r.shake_iter < 200 for r in rg)
    for a, b in zip(rg, ro):
        assert abs(a.temp - b.temp) <= 1e-8 * b.temp
        assert abs(a.pels1 - b.pels1) <= 1e-8 * abs(b.pels1)


def test_cfg1_nve_conserves_energy_like_fp64():
    """Rigid SPC/E, SHEJK at TOLER 1.4e-4: after 400 NVT steps from the
    lattice start, 300 NVE steps; the total energy's RMS stays a small
    fraction of the kinetic energy's on both paths, and the mixed path
    conserves it like the FP64 path."""
    from mdynamix_gb300.mdx import ForcePath
    s = S.System(dataclasses.replace(S.spce_nacl_nve(), toler=1.4e-4, nvt=(300.0, 30.0)))
    st = S.make_configuration(s, seed=1, jitter=0.05)
    g = ForcePath(s)
    g.set_state(*st)
    g.sultan(400, records=False)
    state, th = g.get_state()
    g.close()
    out = {}
    for prec in (MDX_FP64, MDX_MIXED):
        g = ForcePath(s, precision=prec)
        p = g.packed.params
        p.lnvt = 0
        g.set_params(p)
        th.sc = 0.0
        g.set_state(*state, thermo=th)
        rec = g.sultan(300, 400)
        e = np.array([r.pe1 + r.pe2 + r.pels1 + r.pels2 + r.spe + r.pint + r.tke for r in rec])
        ke = np.array([r.tke for r in rec])
        out[prec] = float(e.std() / ke.std())
        assert max(r.shake_iter for r in rec) < 2001
        g.close()
    assert out[MDX_FP64] < 0.2, out
    assert out[MDX_MIXED] < 2.0 * out[MDX_FP64] + 0.02, out


# ------------------------------------------------------------ torsions --
def torsion_db():
    """moldb with "C2H5OH" whose twelve dihedrals cycle through ITORS 0, 1,
    5 and -1 (parameters in kJ/mol and degrees, as .mmol files give them)."""
    db = copy.deepcopy(S.load_moldb())
    forms = [
        dict(itors=0, nmul=3, ft=0.67, rt=0.0),
        dict(itors=1, ft1=1.3, ft2=-0.45, ft3=0.8),
        dict(itors=5, ft=0.4, ft1=1.1, ft2=-0.7, ft3=0.35, ft4=0.2, ft5=-0.12, rt=15.0),
        dict(itors=-1, ft=0.02, rt=60.0),
    ]
    for k, t in enumerate(db["C2H5OH"]["tors"]):
        base = dict(ft=0.0, ft1=0.0, ft2=0.0, ft3=0.0, ft4=0.0, ft5=0.0, rt=0.0, nmul=0)
        base.update(forms[k % 4])
        t.update(base)
    return db


def torsion_system():
    db = torsion_db()
    spec = S.RunSpec(molecules=[("H2O", 100), ("CH3OH", 3), ("C2H5OH", 2)], density=1.0,
                     dt_fs=2.0, nfreq=10, rcut=7.0, rshort=5.0, alpha=2.0, fexp=9.0, ichnb=10,
                     nvt=(298.0, 30.0), trtemp=298.0)
    s = S.System(spec, moldb=db)
    assert set(s.t_itors.tolist()) == {0, 1, 5, -1}
    return s, S.make_configuration(s, seed=11, jitter=0.05)


def test_torsion_forms_match_oracle():
    s, st = torsion_system()
    g, o = _pair(s, st)
    g.chcnb(); o.chcnb()
    g.getcom(); o.getcom()
    a, b = g.fforces(True), o.fforces(True)
    assert relmax(g.forces(1), o.forces(1)) < FP64_TOL
    assert abs(a.pint - b.pint) <= FP64_TOL * abs(b.pint)
    ag, ao = g.bonded_averages(), o.bonded_averages()
    for k in ("te", "br", "be", "ar", "ae"):
        assert relmax(ag[k], ao[k]) < FP64_TOL, k
    # dihedrals near 180 degrees: acos amplifies the last bits of the cosine
    # (d acos / d co -> infinity at co = -1), so the angles agree to 1e-8
    assert relmax(ag["tr"], ao["tr"]) < 1e-8
    # and along three DOUBLE long steps
    g2, o2 = _pair(s, st)
    g2.double(3), o2.double(3)
    (gx, *_), _ = g2.get_state()
    (ox, *_), _ = o2.get_state()
    assert np.abs(gx - ox).max() < 1e-9


def test_torsion_forms_mixed_error():
    from mdynamix_gb300.mdx import ForcePath
    s, st = torsion_system()
    f = {}
    for prec in (MDX_FP64, MDX_MIXED):
        g = ForcePath(s, precision=prec)
        g.set_state(*st)
        g.chcnb()
        g.getcom()
        g.fforces(True)
        f[prec] = g.forces(1)
    rms = np.sqrt(((f[MDX_MIXED] - f[MDX_FP64]) ** 2).sum() / (f[MDX_FP64] ** 2).sum())
    assert rms < 1e-5, rms


# ------------------------------------------------------ reaction field --
def rf_system(diel=78.0, debye=0.0, rigid=True):
    """Electrostatics ALPHA <= 0 (main.f:740-793): reaction field of
    dielectric constant -ALPHA (FEXP the Debye length), molecular cutoff
    lists; DIEL = 1 is a plain cutoff."""
    base = systems.spce_ions(n=216, ions=2) if rigid else systems.organics(nw=150)
    spec = dataclasses.replace(base, alpha=-diel, fexp=debye, rcut=9.0)
    s = S.System(spec)
    assert s.lmnbl and s.alphad == 0.0
    return s, S.make_configuration(s, seed=3, jitter=0.05)


@pytest.mark.parametrize("diel,debye,rigid", [(78.0, 0.0, True), (1.0, 0.0, True),
                                              (60.0, 8.0, False)])
def test_reaction_field_lists_and_forces(diel, debye, rigid):
    """The molecular cutoff list (small molecules whole, by centre of mass,
    forces.f:1882-1936) bit for bit, and the reaction-field forces and
    energies at 1e-10, against the oracle."""
    s, st = rf_system(diel, debye, rigid)
    g, o = _pair(s, st)
    assert g.chcnb() == o.chcnb()
    (gs1, gs2), (gl1, gl2) = g.lists()
    (os1, os2), (ol1, ol2) = o.lists()
    assert np.array_equal(gs1, os1) and np.array_equal(gs2, os2)
    assert np.array_equal(gl1, ol1) and np.array_equal(gl2, ol2)
    g.getcom(); o.getcom()
    a, b = g.allforce(), o.allforce()
    assert relmax(g.forces(3), o.forces(3)) < FP64_TOL
    for n in ("pe1", "pels1", "pe2", "pels2", "vir1", "vir2", "wirs", "wirss"):
        assert abs(getattr(a, n) - getattr(b, n)) <= FP64_TOL * max(abs(getattr(b, n)), 1e-12), n


def test_reaction_field_dynamics_and_mixed():
    s, st = rf_system()
    g, o = _pair(s, st)
    rg, ro = g.sultan(3), o.sultan(3)
    (gx, gy, gz, *_), _ = g.get_state()
    (ox, oy, oz, *_), _ = o.get_state()
    assert max(np.abs(gx - ox).max(), np.abs(gy - oy).max(), np.abs(gz - oz).max()) < 1e-9
    from mdynamix_gb300.mdx import ForcePath
    f = {}
    for prec in (MDX_FP64, MDX_MIXED):
        x = ForcePath(s, precision=prec)
        x.set_state(*st)
        x.chcnb()
        x.getcom()
        x.allforce()
        f[prec] = x.forces(3)
    rms = np.sqrt(((f[MDX_MIXED] - f[MDX_FP64]) ** 2).sum() / (f[MDX_FP64] ** 2).sum())
    assert rms < 1e-5, rms


# ---------------------------------------------------------- PULLBACK --
def pullback_case():
    from mdynamix_gb300.abi import pullback
    s, st = systems.build(systems.spcfw(n=216, ions=2))
    rng = np.random.default_rng(8)
    atoms = rng.choice(s.nstot, 6, replace=False) + 1
    ref = [st[k][atoms - 1] + rng.normal(scale=0.3, size=6) for k in range(3)]
    # 10^15 m/s^2 drags, 0.5 A wells, a 5 MV/cm field at 40 THz
    pb = pullback(s, drag={2: 1.0e3, 3: -8.0e2}, wells=(atoms, *ref), rlr=0.5,
                  field=(5.0e6, 4.0e13), tim=1.0e-12)
    return s, st, pb


def test_pullback_matches_oracle():
    """PULLBACK (forces.f:1756-1799): drag on the ion types, wells on six
    atoms, an oscillating field along z -- on G after the slow forces, and
    along DOUBLE steps whose field follows the step count."""
    s, st, pb = pullback_case()
    g, o = _pair(s, st)
    g.set_pullback(pb)
    o.set_pullback(pb)
    g.chcnb(); o.chcnb()
    g.getcom(); o.getcom()
    g.slforces(); o.slforces()
    assert relmax(g.forces(2), o.forces(2)) < FP64_TOL
    g.allforce(); o.allforce()
    assert relmax(g.forces(2), o.forces(2)) < FP64_TOL
    assert relmax(g.forces(3), o.forces(3)) < FP64_TOL
    g2, o2 = _pair(s, st)
    g2.set_pullback(pb)
    o2.set_pullback(pb)
    g2.double(3), o2.double(3)
    (gx, gy, gz, *_), _ = g2.get_state()
    (ox, oy, oz, *_), _ = o2.get_state()
    assert max(np.abs(gx - ox).max(), np.abs(gz - oz).max()) < 1e-9


# --------------------------------------------------- FP64 sweep math --
def test_pair_math_against_library():
    """The FP64 pair sweeps' exp(-y) (Tang's table method) and 1/d (FP32
    seed + two Newton steps) against the CUDA library's exp and division on
    the device: within 4 units in the last place over the sweeps' ranges
    (y = (alpha r)^2 up to 40 and beyond to the 700 clamp, d = 1 + p alpha r
    in [1, 4])."""
    from mdynamix_gb300.mdx import probe_pair_math
    rng = np.random.default_rng(3)
    y = np.concatenate([np.linspace(0.0, 40.0, 200001), rng.uniform(0, 700, 20000),
                        [0.0, 5e-324, 1e-300, 1e-17, 1e-9, 700.0, 699.999]])
    d = np.concatenate([np.linspace(1.0, 4.0, 200001), rng.uniform(1, 1e6, 20000),
                        [1.0, 1.0 + 2.0 ** -52, 2.0, 2.0 - 2.0 ** -52, 3.0, 1e6, 7.0]])
    own_e, lib_e, own_r, lib_r = probe_pair_math(y, d)
    ulp = 2.0 ** -52
    assert np.all(np.abs(own_e - lib_e) <= 4 * ulp * lib_e)
    assert np.all(np.abs(own_r - lib_r) <= 4 * ulp * lib_r)
    # and against numpy's exp / division (the host's libm)
    assert np.all(np.abs(own_e - np.exp(-y)) <= 4 * ulp * np.exp(-y))
    assert np.all(np.abs(own_r - 1.0 / d) <= 4 * ulp / d)


# ------------------------------------------- non-rectangular cells ---
def cell_system(icell, rigid=False):
    """Water + ions in a truncated octahedron (ICELL 1) or a hexagonal cell
    (ICELL 2): flexible SPC-FW with DOUBLE, or rigid SPC/E with SULTAN +
    SHEJK."""
    base = systems.spce_ions(n=200, ions=2, toler=1e-6) if rigid else systems.spcfw(
        n=256, ions=2, rcut=8.0)
    return systems.build(dataclasses.replace(base, icell=icell))


@pytest.mark.parametrize("icell", [1, 2])
def test_cell_shapes_match_oracle(icell):
    """PBC of the truncated octahedron and the hexagonal cell (service.f:
    953-990, inlined in LOCALF, FORCES, ETERMS, CHCNB) and INIFUR's k-sets
    for them (forces.f:1392-1406): lists bit for bit, SLFORCES / FFORCES /
    ALLFORCE forces and scalars at 1e-10, and three DOUBLE steps."""
    s, st = cell_system(icell)
    g, o = _pair(s, st)
    assert g.inifur() == o.inifur() == s.kvector_count()
    assert g.chcnb() == o.chcnb()
    (gs1, gs2), (gl1, gl2) = g.lists()
    (os1, os2), (ol1, ol2) = o.lists()
    assert np.array_equal(gs1, os1) and np.array_equal(gs2, os2)
    assert np.array_equal(gl1, ol1) and np.array_equal(gl2, ol2)
    g.getcom(); o.getcom()
    for routine in ("slforces", "fforces", "allforce"):
        a, b = getattr(g, routine)(), getattr(o, routine)()
        which = {"slforces": 2, "fforces": 1, "allforce": 3}[routine]
        assert relmax(g.forces(which), o.forces(which)) < FP64_TOL, routine
        names = {"slforces": ("pels1", "pe1", "spe", "vir1", "virx", "viry", "virz", "wirs"),
                 "fforces": ("pels2", "pe2", "vir2", "pint", "wirss"),
                 "allforce": ("pe1", "pels1", "pe2", "pels2", "spe", "vir1", "vir2", "wirs")}
        for n in names[routine]:
            assert abs(getattr(a, n) - getattr(b, n)) <= FP64_TOL * max(abs(getattr(b, n)),
                                                                        1e-12), (routine, n)
    g2, o2 = _pair(s, st)
    g2.double(3), o2.double(3)
    (gx, gy, gz, *_), _ = g2.get_state()
    (ox, oy, oz, *_), _ = o2.get_state()
    assert max(np.abs(gx - ox).max(), np.abs(gy - oy).max(), np.abs(gz - oz).max()) < 1e-9


@pytest.mark.parametrize("icell", [1, 2])
def test_cell_shapes_sultan_shake(icell):
    """Rigid water under SULTAN + SHEJK in the two cells: the constraint
    vectors take the cell's minimum image (mdstep.f:1175, 1186); three steps
    against the oracle."""
    s, st = cell_system(icell, rigid=True)
    g, o = _pair(s, st)
    g.sultan(3), o.sultan(3)
    (gx, gy, gz, *_), _ = g.get_state()
    (ox, oy, oz, *_), _ = o.get_state()
    assert max(np.abs(gx - ox).max(), np.abs(gy - oy).max(), np.abs(gz - oz).max()) < 1e-9


@pytest.mark.parametrize("icell", [1, 2])
def test_cell_shapes_mixed(icell):
    """The mixed path in the two cells.  Hexagonal: fixed-point y words of
    period 2 BOYL, the cell's fold in FP32 after the integer differences, the
    X phase of the Ewald tables as the sum of the x and y words.  Truncated
    octahedron: the corner fold in FP32, the k-set's columns grouped by the
    parity of their nz and read every other z by the CUDA-core S(k) and force
    passes.  Against the FP64 path: force RMS error under 1e-5 in SLFORCES /
    FFORCES / ALLFORCE, energies and virials to 1e-4, eleven DOUBLE steps
    tracking it to 1e-5 A."""
    from mdynamix_gb300.mdx import ForcePath
    s, st = cell_system(icell)
    g64 = ForcePath(s, precision=MDX_FP64)
    g32 = ForcePath(s, precision=MDX_MIXED)
    for g in (g64, g32):
        g.set_state(*st)
        assert g.inifur() == s.kvector_count()
        g.chcnb()
        g.getcom()
    for routine in ("slforces", "fforces", "allforce"):
        a, b = getattr(g64, routine)(), getattr(g32, routine)()
        which = {"slforces": 2, "fforces": 1, "allforce": 3}[routine]
        f64, f32 = g64.forces(which), g32.forces(which)
        rms = np.sqrt(((f32 - f64) ** 2).sum() / (f64 ** 2).sum())
        assert rms < 1e-5, (routine, rms)
        for n in ("pe1", "pels1", "pe2", "pels2", "vir1", "vir2"):
            assert abs(getattr(a, n) - getattr(b, n)) <= 1e-4 * max(abs(getattr(a, n)), 1e-9), \
                (routine, n)
    h64 = ForcePath(s, precision=MDX_FP64)
    h32 = ForcePath(s, precision=MDX_MIXED)
    for h in (h64, h32):
        h.set_state(*st)
    r64, r32 = h64.double(11), h32.double(11)
    (ax, ay, az, *_), _ = h64.get_state()
    (bx, by, bz, *_), _ = h32.get_state()
    dpos = max(np.abs(ax - bx).max(), np.abs(ay - by).max(), np.abs(az - bz).max())
    assert dpos < 1e-5, dpos
    for a, b in zip(r64, r32):
        for n in ("pe1", "pels1", "temp"):
            assert abs(getattr(a, n) - getattr(b, n)) <= 1e-4 * max(abs(getattr(a, n)), 1e-9), n


def test_cell_shapes_refused_where_not_built():
    """Non-rectangular cells with a Verlet skin are refused (the skin's
    displacement check and rectangular-grid build are not written for
    them)."""
    from mdynamix_gb300.mdx import ForcePath, MdxError
    base = systems.spcfw(n=256, ions=2, rcut=8.0)
    for prec in (MDX_FP64, MDX_MIXED):
        s = systems.build(dataclasses.replace(base, icell=1, rskin=1.0))[0]
        with pytest.raises(MdxError):
            ForcePath(s, precision=prec)
