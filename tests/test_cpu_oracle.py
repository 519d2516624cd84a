"""CPU tests: the oracle against physical invariants and an independent
numpy restatement of the pair classification; the system builder; the C ABI
layout and exported symbols (no GPU needed)."""
import ctypes
import math
import os
import re
import subprocess

import numpy as np
import pytest

import oracle
from mdynamix_gb300 import abi, system as S
from tests import systems

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def etot(sc):
    return sc.pe1 + sc.pe2 + sc.pels1 + sc.pels2 + sc.spe + sc.pint


# ------------------------------------------------------------- builder ----
def test_named_workloads_sizes():
    s1 = S.System(S.spce_nacl_nve())
    assert s1.nstot == 1544 and abs(s1.boxl - 25.042) < 1e-3
    assert abs(s1.alphad - 0.28) < 1e-12
    assert s1.fnst == 3 * 1544 - 3 * 512 - 3
    s2 = S.System(S.spcfw_water())
    assert s2.nstot == 98304 and abs(s2.boxl - 99.336) < 1e-3
    assert abs(s2.alphad - 0.25) < 1e-12
    assert s2.kvector_count() == 16700


def test_units_literals():
    s = S.System(systems.spcfw())
    # UNITP carries the REAL*4 literal 1.e-5 of setup.f:103
    assert s.unitp == s.unite * float(np.float32(1e-5)) / s.unitl ** 3
    assert abs(s.tstep - 1.0) < 1e-12


def test_lj_types_spce():
    s = S.System(S.spce_nacl_nve())
    assert s.nnbt == 4 and list(s.inbt) == [1, 2, 2, 3, 4]
    a6, b12 = S.comb_rules(3.166, 3.166, 0.6507 * s.efact, 0.6507 * s.efact, 16, 16)
    assert abs(s.a6lj[0, 0] - a6) < 1e-20 and abs(s.b12lj[0, 0] - b12) < 1e-16


def test_exclusions_water_and_methanol():
    s = S.System(systems.organics())
    # fSPC water: O-H1, O-H2 bonded (1-2), H1-H2 via the H-H bond record
    assert s.nnbb[0] == 2
    # methanol has 1-4 pairs (H on C to H on O)
    off = s.isaddr[1]
    rows = [s.inbb[:s.nnbb[off + k], off + k] for k in range(6)]
    assert any((r < 0).any() for r in rows)


MOLDB_DIR = os.environ.get("MDX_REFERENCE_MOLDB", "")


@pytest.mark.skipif(not os.path.isdir(MOLDB_DIR),
                    reason="set MDX_REFERENCE_MOLDB to the reference's moldb directory")
def test_moldb_fixture_matches_mmol_files():
    db = S.load_moldb()
    for name in ("SPC_E", "SPC-FW", "H2O", "CH3OH", "dmpc", "Na+_SD", "Cl-_SD"):
        with open(os.path.join(MOLDB_DIR, f"{name}.mmol"), encoding="latin-1") as fh:
            parsed = S.parse_mmol(fh.read(), name)
        assert parsed == db[name]


# -------------------------------------------------------------- oracle ----
def brute_lists(s, st):
    """Independent restatement of CHCNB's pair set with numpy."""
    x, y, z = st[0], st[1], st[2]
    n = s.nstot
    L = np.array([s.boxl, s.boyl, s.bozl])
    short, long_, s14 = set(), set(), set()
    excl = {}
    for i in range(n):
        excl[i + 1] = {int(v) for v in s.inbb[: s.nnbb[i], i]}
    for I in range(1, n + 1):
        J = np.arange(1, n + 1)
        own = np.where(((I - J) % 2) == 0, J < I, J > I)
        d = np.stack([x[I - 1] - x, y[I - 1] - y, z[I - 1] - z], axis=1)
        for k in range(3):
            m = np.abs(d[:, k]) > L[k] / 2
            d[m, k] -= np.copysign(L[k], d[m, k])
        rr = (d ** 2).sum(1)
        for j in np.nonzero(own)[0]:
            Jv = j + 1
            if s.nnum[I - 1] == s.nnum[j] and rr[j] <= 64.0:
                if Jv in excl[I]:
                    continue
                if -Jv in excl[I]:
                    s14.add((I, Jv))
                    continue
            if rr[j] <= s.short2:
                short.add((max(I, Jv), min(I, Jv)))
            elif rr[j] <= s.rssq:
                long_.add((max(I, Jv), min(I, Jv)))
    return short, long_, s14


@pytest.mark.parametrize("spec", [systems.spce_ions(n=64, ions=1), systems.organics(nw=40)])
def test_oracle_lists_against_numpy(spec):
    s = S.System(spec)
    st = S.make_configuration(s, seed=5, jitter=0.05)
    o = oracle.Oracle(s)
    o.set_state(*st)
    (a1, a2), (b1, b2) = o.chcnb_lists()
    short, long_, s14 = brute_lists(s, st)
    got_short = {(int(p), int(q)) for p, q in zip(a1, a2) if p > 0}
    got_14 = {(-int(p), int(q)) for p, q in zip(a1, a2) if p < 0}
    got_long = {(int(p), int(q)) for p, q in zip(b1, b2)}
    assert got_short == short and got_long == long_ and got_14 == s14


def _rf(spec, diel=78.0, debye=0.0):
    import dataclasses
    return dataclasses.replace(spec, alpha=-diel, fexp=debye)


@pytest.mark.parametrize("spec", [systems.spce_ions(n=64, ions=1), systems.organics(nw=40),
                                  systems.spcfw(n=64, rcut=6.0),
                                  _rf(systems.spce_ions(n=64, ions=1)),
                                  _rf(systems.organics(nw=40), diel=60.0, debye=8.0)])
def test_oracle_newton_and_finite_difference(spec):
    s = S.System(spec)
    st = S.make_configuration(s, seed=3, jitter=0.05)
    o = oracle.Oracle(s)
    o.set_state(*st)
    o.chcnb()
    o.allforce()
    F = o.forces(3)
    assert np.abs(F.sum(0)).max() < 1e-10 * np.abs(F).max() * s.nstot
    rng = np.random.default_rng(0)
    fscale = np.sqrt((F ** 2).mean())
    for _ in range(4):
        i = int(rng.integers(s.nstot)); k = int(rng.integers(3)); h = 1e-5
        arr = [st[0].copy(), st[1].copy(), st[2].copy()]
        arr[k][i] += h
        o.set_state(*arr, *st[3:]); ep = etot(o.allforce())
        arr[k][i] -= 2 * h
        o.set_state(*arr, *st[3:]); em = etot(o.allforce())
        fd = -(ep - em) / (2 * h)
        # the A&S erfc of the reference is not the antiderivative of its force
        # (max error 1.5e-7), hence the 1e-4 bound relative to the force scale
        assert abs(F[i, k] - fd) < 1e-4 * fscale


def test_oracle_ewald_alpha_independence():
    base = dict(molecules=[("SPC_E", 64), ("Na+", 1), ("Cl-", 1)], density=1.0, rcut=6.0,
                rshort=5.0, ichnb=5)
    es = []
    # converged real space (erfc(A) < 1e-6) and reciprocal space (e^-B < 1e-6)
    for a, b in ((3.5, 14.0), (4.0, 20.0)):
        s = S.System(S.RunSpec(alpha=a, fexp=b, **base))
        st = S.make_configuration(s, seed=9, jitter=0.05)
        o = oracle.Oracle(s)
        o.set_state(*st)
        o.chcnb()
        sc = o.allforce()
        es.append(sc.pels1 + sc.pels2 + sc.spe)
    assert abs(es[0] - es[1]) < 1e-3 * abs(es[0])


def test_oracle_nve_conservation_double():
    """Equilibrate 300 NVT long steps, then 200 NVE steps: the total energy
    drift stays a small fraction of the kinetic-energy fluctuation."""
    spec = S.RunSpec(molecules=[("SPC-FW", 64)], density=1.0, dt_fs=2.0, nfreq=10, rcut=6.0,
                     rshort=5.0, alpha=2.6, fexp=12.0, ichnb=5, nvt=(300.0, 30.0))
    s = S.System(spec)
    st = S.make_configuration(s, seed=2, jitter=0.05)
    o = oracle.Oracle(s)
    o.set_state(*st)
    o.double(300)
    (x, y, z, vx, vy, vz), th = o.get_state()
    p = o.packed.params
    p.lnvt = 0
    o.L.ox_set_params(o.h, p)
    th.sc = 0.0
    o.set_state(x, y, z, vx, vy, vz, th)
    rec = o.double(200, 300)
    e = np.array([etot_rec(r) for r in rec])
    ke = np.array([r.tke for r in rec])
    assert abs(e[-20:].mean() - e[:20].mean()) < 0.15 * ke.std()
    assert e.std() < 0.3 * ke.std()


def etot_rec(r):
    return r.pe1 + r.pe2 + r.pels1 + r.pels2 + r.spe + r.pint + r.tke


def test_oracle_shake_constraints_hold():
    s = S.System(systems.spce_ions(n=64, ions=1, toler=1e-6))
    st = S.make_configuration(s, seed=4, jitter=0.05)
    o = oracle.Oracle(s)
    o.set_state(*st)
    o.sultan(5)
    (x, y, z, *_), th = o.get_state()
    for m in range(64):
        i = 3 * m
        d = math.dist((x[i], y[i], z[i]), (x[i + 1], y[i + 1], z[i + 1]))
        assert abs(d - 1.0) < 1e-5


# ------------------------------------------------------------------ ABI ---
def test_abi_struct_sizes_match_c():
    src = r'''
#include <stdio.h>
#include <stddef.h>
#include "mdx_gpu.h"
int main(void){printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\n", sizeof(mdx_dims), sizeof(mdx_topo),
 sizeof(mdx_params), sizeof(mdx_scalars), sizeof(mdx_thermo), sizeof(mdx_step_record),
 sizeof(mdx_kin), sizeof(mdx_pimd_params), sizeof(mdx_pimd_record), sizeof(mdx_path_info),
 sizeof(mdx_tuning));
 return 0;}
'''
    tmp = os.path.join(ROOT, "_build")
    os.makedirs(tmp, exist_ok=True)
    c = os.path.join(tmp, "abi_sizes.c")
    exe = os.path.join(tmp, "abi_sizes")
    with open(c, "w") as fh:
        fh.write(src)
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe], check=True)
    got = [int(v) for v in subprocess.run([exe], capture_output=True, text=True).stdout.split()]
    want = [ctypes.sizeof(t) for t in (abi.MdxDims, abi.MdxTopo, abi.MdxParams,
                                       abi.MdxScalars, abi.MdxThermo, abi.MdxStepRecord,
                                       abi.MdxKin, abi.MdxPimdParams, abi.MdxPimdRecord,
                                       abi.MdxPathInfo, abi.MdxTuning)]
    assert got == want


def header_functions():
    txt = open(os.path.join(ROOT, "include", "mdx_gpu.h")).read()
    return sorted(set(re.findall(r"\b(mdx_[a-z_0-9]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    from mdynamix_gb300.build import LIB, build
    if not os.path.exists(LIB):
        build()
    lib = ctypes.CDLL(LIB)
    for name in header_functions():
        assert hasattr(lib, name), name
    lib.mdx_strerror.restype = ctypes.c_char_p
    assert lib.mdx_strerror(3) == b"neighbour list overflow"
    assert lib.mdx_version() >= 1


# ---------------------------------------------------- GETKIN / CHKMOM ----
def _kin_setup(seed=4):
    s, st = systems.build(systems.organics(nw=30))
    m = 1.0 / s.massdi                    # internal masses per atom
    mol = s.nnum - 1
    x = np.stack(st[:3], axis=1)
    mm = np.zeros(s.nop)
    np.add.at(mm, mol, m)
    com = np.zeros((s.nop, 3))
    for k in range(3):
        np.add.at(com[:, k], mol, m * x[:, k])
    com /= mm[:, None]
    return s, st, m, mol, x - com[mol], np.random.default_rng(seed)


def test_getkin_splits_translation_and_rotation():
    """GETKIN (service.f:611-735) in the oracle: momenta that translate each
    molecule rigidly are all translational energy; momenta that rotate each
    (non-linear) molecule rigidly about its centre are all rotational."""
    s, st, m, mol, w, rng = _kin_setup()
    o = oracle.Oracle(s)
    V = rng.normal(size=(s.nop, 3))
    p = m[:, None] * V[mol]
    o.set_state(*st[:3], p[:, 0], p[:, 1], p[:, 2])
    o.getcom()
    ektr, ekrot, ekint, tke = o.getkin()[:4]
    assert abs(ektr - tke) < 1e-10 * tke and abs(ekrot) < 1e-10 * tke
    om = rng.normal(size=(s.nop, 3))
    p = m[:, None] * np.cross(om[mol], w)
    o.set_state(*st[:3], p[:, 0], p[:, 1], p[:, 2])
    o.getcom()
    ektr, ekrot, ekint, tke, ttr, trot, tint = o.getkin()
    assert abs(ektr) < 1e-10 * tke
    assert abs(ekrot - tke) < 1e-8 * tke and abs(ekint) < 1e-8 * tke
    assert abs(trot - 3.0 * ekrot * s.enerf * s.tempf / s.fnstr) < 1e-12 * trot


def test_chkmom_removes_total_momentum():
    s, st, m, mol, w, rng = _kin_setup()
    o = oracle.Oracle(s)
    v = rng.normal(size=(s.nstot, 3))
    o.set_state(*st[:3], v[:, 0], v[:, 1], v[:, 2])
    dv = o.chkmom()
    (_, _, _, vx, vy, vz), _ = o.get_state()
    tot = np.array([vx.sum(), vy.sum(), vz.sum()])
    assert np.abs(tot).max() < 1e-10 * np.abs(v).sum()
    assert np.allclose(np.array(dv) * S.kin_sumasd(s), v.sum(axis=0), rtol=1e-12, atol=1e-12)


def test_fixed_point_phase_split():
    """The mixed phase tables' arithmetic (ewald.cu k_tables): k times a
    32-bit fixed-point coordinate is the phase modulo one turn exactly
    (integer wrap-around); its top 24 bits are exact in FP32 and the low 8
    bits rotate the result to first order.  Restated in numpy (FP32 where
    the kernel rounds), it stays within 2e-7 of exp(2 pi i k x / L)."""
    rng = np.random.default_rng(7)
    u = rng.integers(0, 2 ** 32, size=4000, dtype=np.uint64)
    for k in (1, 2, 7, 21):
        ph = ((u * k) % 2 ** 32).astype(np.int64)
        ph = np.where(ph >= 2 ** 31, ph - 2 ** 32, ph)          # signed fraction of half a turn
        hi = ph & ~0xff
        lo = ph - hi
        x = np.float32(hi) * np.float32(2.0 ** -31)               # exact in FP32
        s = np.sin(np.pi * x.astype(np.float64)).astype(np.float32)
        c = np.cos(np.pi * x.astype(np.float64)).astype(np.float32)
        d = np.float32(lo) * np.float32(np.pi * 2.0 ** -31)
        re = c - s * d
        im = s + c * d
        exact = np.exp(2j * np.pi * ((u * k) % 2 ** 32).astype(np.float64) / 2 ** 32)
        err = np.abs((re.astype(np.float64) + 1j * im.astype(np.float64)) - exact).max()
        assert err < 2e-7, (k, err)


# --------------------------------------------- fixed-point rounding ----
def _f2ll_rn(y):
    """mdx_internal.cuh f2ll_rn on the bits of a float32, in Python ints."""
    b = int(np.float32(y).view(np.uint32))
    e = min(((b >> 23) & 0xFF) - 150, 39)
    m = (b & 0x7FFFFF) | 0x800000
    r = 0
    if e >= 0:
        r = m << e
    elif e >= -24:
        s = -e
        q, rem, half = m >> s, m & ((1 << s) - 1), 1 << (s - 1)
        r = q + (1 if (rem > half or (rem == half and q & 1)) else 0)
    return -r if b >> 31 else r


def test_float_to_int64_rounding_is_exact():
    """f2ll_rn (the mixed path's rounding of FP32 partial sums to 64-bit
    fixed point, integer operations on the float's bits) equals
    round-half-even of the float, i.e. __float2ll_rn."""
    rng = np.random.default_rng(3)
    ys = np.concatenate([rng.normal(size=20000) * 10.0 ** rng.integers(-3, 18, 20000),
                         [0.0, 0.5, 1.5, 2.5, -0.5, -2.5, 1e-30, 4294967296.0, 2.0 ** 40 + 1e5,
                          8388608.5, 16777215.0]]).astype(np.float32)
    for y in ys:
        assert _f2ll_rn(y) == int(np.rint(np.float64(y))), y


def test_shake_on_bonds_to_hydrogen_counts_constraints():
    """SHAKE on bonds to hydrogen: fewer constraints per lipid than the
    reference's ID != 2 rule, and the degrees of freedom grow by the
    difference (main.f:297-350 counts NRCON per type)."""
    from mdynamix_gb300 import system as S
    kw = dict(nside=1, nwater=100, box=(20.0, 20.0, 60.0), rcut=9.0, alpha=2.8, fexp=9.0)
    a = S.System(S.dmpc_bilayer(**kw))
    b = S.System(S.dmpc_bilayer(shake_hbonds=True, **kw))
    assert b.nrcon[0] < a.nrcon[0] and b.nrcon[1] == a.nrcon[1] == 3
    assert b.fnst - a.fnst == (a.nrcon[0] - b.nrcon[0]) * a.nspec[0]
    lip = a.types[0]
    heavy = [i for i, st in enumerate(lip["sites"]) if st["mass"] > 1.5]
    cons = [bd for bd, f in zip(lip["bonds"], b.b_lcon[:a.nrb[0]]) if f]
    assert all(bd["i"] - 1 not in heavy or bd["j"] - 1 not in heavy for bd in cons)


def test_oracle_pullback_field_and_wells():
    """The oracle's PULLBACK: the field adds Q E along z with E at
    TIM + NSTEP DT, a well pulls its atom back to the well's centre."""
    from mdynamix_gb300.abi import pullback
    s, st = systems.build(systems.spcfw(n=64, ions=1, rcut=6.0))
    o = oracle.Oracle(s)
    o.set_state(*st)
    o.chcnb()
    o.getcom()
    o.slforces()
    g0 = o.forces(2)
    E0, w, t0 = 5.0e6, 3.0e13, 5.0e-13     # V/cm, Hz, s
    atom = 7
    ref = (st[0][atom - 1] + 0.2, st[1][atom - 1], st[2][atom - 1] - 0.1)
    pb = pullback(s, field=(E0, w), tim=t0, nstep=4,
                  wells=(np.array([atom]), *[np.array([r]) for r in ref]), rlr=0.5)
    # setup.f:113 and setup.f:263 conversions
    k = 1.0 / (s.unite / (S.BOLTZ * s.trtemp) * 0.25)
    assert abs(pb.rlr - k) <= 1e-15 * k
    assert abs(pb.exampl - E0 * 1e-8 * S.ELECHG / s.unite) <= 1e-15 * pb.exampl
    o.set_pullback(pb)
    o.slforces()
    d = o.forces(2) - g0
    E = pb.exampl * np.cos(w * (t0 + 4 * s.unitt) * 0.5 / S.PI)
    qz = s.q * E
    qz[atom - 1] += -k * (st[2][atom - 1] - ref[2])
    assert np.abs(qz).max() > 0.05 * np.abs(g0).max()
    assert np.allclose(d[:, 2], qz, rtol=1e-9, atol=1e-12 * np.abs(g0).max())
    assert abs(d[atom - 1, 0] - (-k * (st[0][atom - 1] - ref[0]))) < 1e-12 * np.abs(g0).max()


@pytest.mark.parametrize("icell", [1, 2])
def test_cell_shapes_oracle_ewald_consistent(icell):
    """The oracle's truncated octahedron (ICELL 1) and hexagonal cell
    (ICELL 2): INIFUR's k-set count equals the host's count of the same rule
    (forces.f:1392-1406), and the Ewald total (reciprocal + real-space + self
    terms) barely moves between two splittings (alpha 3.0 / Rc and 3.6 / Rc
    with B = A^2), as a correct lattice sum must (the rectangular cell moves
    as much)."""
    import dataclasses
    base = dataclasses.replace(systems.spcfw(n=256, ions=2, rcut=8.0), icell=icell)
    s, st = systems.build(base)
    out = []
    for A in (3.0, 3.6):
        s2 = S.System(dataclasses.replace(base, alpha=A, fexp=A * A))
        o = oracle.Oracle(s2)
        o.set_state(*st)
        assert o.inifur() == s2.kvector_count()
        o.chcnb()
        o.getcom()
        r = o.allforce()
        out.append((r.pels1 + r.pels2 + r.spe, r.pels1, o.forces(3)))
    assert abs(out[0][0] - out[1][0]) < 2e-3 * abs(out[0][1])
    f0, f1 = out[0][2], out[1][2]
    assert np.abs(f0 - f1).max() < 1e-4 * np.abs(f0).max()


def test_autotune_table_from_timings():
    """The tuning table's construction: size classes between the measured
    systems, the fastest split of each class's largest measured system, and
    the lookup that a context makes with its sizes."""
    from mdynamix_gb300 import autotune
    res = [
        dict(n=768, row_short=52.0, row_long=254.0, short={2: 3.0, 4: 2.0, 8: 1.0},
             long={8: 3.0, 16: 2.0, 32: 1.0}),
        dict(n=24000, row_short=52.0, row_long=254.0, short={2: 3.0, 4: 1.0, 8: 2.0},
             long={8: 2.0, 16: 1.0, 32: 3.0}),
        dict(n=24000, row_short=52.0, row_long=673.0, short={2: 3.0, 4: 1.0, 8: 2.0},
             long={8: 3.0, 16: 2.0, 32: 1.0}),
    ]
    sc = autotune.table(res, "row_short", "short")
    lc = autotune.table(res, "row_long", "long")

    def pick(cells, n, row):
        for mx, mr, t in cells:
            if n <= mx and row <= mr:
                return t

    assert pick(sc, 768, 52.0) == 8 and pick(sc, 24000, 52.0) == 4
    assert pick(lc, 768, 254.0) == 32
    assert pick(lc, 24000, 254.0) == 16 and pick(lc, 24000, 673.0) == 32
    assert pick(lc, 10 ** 9, 1e9) is not None  # the last class is open


def _pbc_hex64(x, y, boxl, boyl):
    """The reference's PBC for the hexagonal cell (service.f:953-990, LHEX),
    elementwise in FP64: x folded to +-BOXL/2, then its four tests."""
    cos30 = float(np.float32(0.8660254037844386))
    boxyc = float(np.float32(0.5) / np.float32(cos30))  # REAL parameter (common_inc.f:33)
    boxy3 = 0.66666666666666666667 * boyl               # RECLEN (service.f:579)
    hbx = 0.5 * boxl
    x = np.where(np.abs(x) > hbx, x - np.copysign(boxl, x), x)
    xy = boxyc * x
    m = (y > boxy3 - xy) & ((x > 0) | (y > 2 * boxy3 - xy))
    y = np.where(m, y - boyl, y); x = np.where(m, x - hbx, x); xy = boxyc * x
    m = (y < -boxy3 - xy) & ((x < 0) | (y < -2 * boxy3 - xy))
    y = np.where(m, y + boyl, y); x = np.where(m, x + hbx, x); xy = boxyc * x
    m = y > boxy3 + xy
    y = np.where(m, y - boyl, y); x = np.where(m, x + hbx, x); xy = boxyc * x
    m = y < -boxy3 + xy
    y = np.where(m, y + boyl, y); x = np.where(m, x - hbx, x)
    return x, y


def test_hexagonal_fixed_point_images():
    """The mixed path's hexagonal cell, restated in numpy: 32-bit words
    x / BOXL and y / (2 BOYL) (2 BOYL is a lattice period, BOYL alone is
    not), their wrapped integer differences in FP32 folded by the same four
    tests in FP32 (pbc_hexf) give the FP64 minimum image of every pair
    within 0.4 BOXL to FP32 rounding; the sum of the two words is the Ewald
    X phase x / BOXL + y / (2 BOYL) (forces.f:1402) modulo one turn."""
    rng = np.random.default_rng(7)
    boxl = 41.3
    boyl = boxl * float(np.float32(0.8660254037844386))
    # positions inside the cell: raw points folded by the cell's PBC
    x, y = _pbc_hex64(rng.uniform(-boxl, boxl, 3000), rng.uniform(-boyl, boyl, 3000), boxl, boyl)
    two32 = 4294967296.0
    xw = (np.rint(x / boxl * two32).astype(np.int64) & 0xffffffff).astype(np.uint32)
    yw = (np.rint(y / (2 * boyl) * two32).astype(np.int64) & 0xffffffff).astype(np.uint32)
    i, j = rng.integers(0, len(x), (2, 20000))
    mx, my = _pbc_hex64(x[i] - x[j], y[i] - y[j], boxl, boyl)
    near = np.hypot(mx, my) < 0.4 * boxl
    dxw = (xw[i] - xw[j]).view(np.int32).astype(np.float32) * np.float32(boxl / two32)
    dyw = (yw[i] - yw[j]).view(np.int32).astype(np.float32) * np.float32(2 * boyl / two32)
    f32 = np.float32
    hbx, by = f32(0.5 * boxl), f32(boyl)
    boxy3 = f32(0.66666666666666666667 * boyl)
    boxyc = f32(0.5) / f32(0.8660254037844386)
    X, Y = dxw.copy(), dyw.copy()
    for k in range(len(X)):  # the FP32 fold, one vector at a time as the kernel does
        xx, yy = X[k], Y[k]
        xy = boxyc * xx
        if yy > boxy3 - xy and (xx > 0 or yy > f32(2) * boxy3 - xy):
            yy = yy - by; xx = xx - hbx; xy = boxyc * xx
        if yy < -boxy3 - xy and (xx < 0 or yy < -f32(2) * boxy3 - xy):
            yy = yy + by; xx = xx + hbx; xy = boxyc * xx
        if yy > boxy3 + xy:
            yy = yy - by; xx = xx + hbx; xy = boxyc * xx
        if yy < -boxy3 + xy:
            yy = yy + by; xx = xx - hbx
        X[k], Y[k] = xx, yy
    assert near.sum() > 1000
    assert np.abs(X[near] - mx[near]).max() < 1e-5 and np.abs(Y[near] - my[near]).max() < 1e-5
    # X phase: the sum of the words against the FP64 fraction
    ph = ((xw.astype(np.uint64) + yw) & 0xffffffff).astype(np.float64) / two32
    ref = np.mod(x / boxl + y / (2 * boyl), 1.0)
    d = np.abs(ph - ref)
    assert np.minimum(d, 1.0 - d).max() < 2.0 ** -30
