"""ctypes mirror of include/mdx_gpu.h and packing of a System into it.

The structures below match the C declarations field for field; the
``pack`` function fills them from a ``system.System`` exactly as the
Fortran driver would from its COMMON blocks.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass
from typing import List

import numpy as np

from .system import BOLTZ, F32_1EM5, NTPP, NTPS, System

I32P = C.POINTER(C.c_int32)
F64P = C.POINTER(C.c_double)

MDX_FP64 = 0
MDX_MIXED = 1

ERRORS = {0: "MDX_OK", 1: "MDX_ERR_ARG", 2: "MDX_ERR_CUDA", 3: "MDX_ERR_LIST_OVERFLOW",
          4: "MDX_ERR_SHAKE", 5: "MDX_ERR_NAN", 6: "MDX_ERR_TIMEOUT", 7: "MDX_ERR_STATE",
          8: "MDX_ERR_NOMEM", 9: "MDX_ERR_KVEC", 10: "MDX_ERR_UNSUPPORTED"}


class MdxDims(C.Structure):
    _fields_ = [(n, C.c_int32) for n in (
        "nstot", "nop", "ntypes", "nsites", "nnbt", "nrbb", "nraa", "nrtt", "nrbt",
        "nrat", "nrrt", "nbdmax", "cap_short", "cap_long", "nkv_max", "precision")]


_TOPO_FIELDS = [
    ("itype", I32P), ("nnum", I32P), ("nsite", I32P), ("massdi", F64P), ("q", F64P),
    ("charge", F64P), ("mass", F64P), ("inbt", I32P),
    ("nspec", I32P), ("nsits", I32P), ("isadr", I32P), ("isaddr", I32P), ("iaddr", I32P),
    ("ipot", I32P), ("nrb", I32P), ("iadb", I32P), ("ishejk", I32P), ("iee", I32P),
    ("lmove", I32P), ("c14el", F64P), ("c14lj", F64P), ("summas", F64P),
    ("a6lj", F64P), ("b12lj", F64P), ("a6lj0", F64P), ("b12lj0", F64P), ("a6_14", F64P),
    ("b12_14", F64P), ("ld_lj", C.c_int32),
    ("mdx", I32P), ("ld_mdx", C.c_int32),
    ("nnbb", I32P), ("inbb", I32P), ("ld_inbb", C.c_int32),
    ("ib", I32P), ("jb", I32P), ("id", I32P), ("rb", F64P), ("fb", F64P), ("db", F64P),
    ("ro", F64P),
    ("ibi", I32P), ("jbj", I32P), ("ibuk", I32P),
    ("ra", F64P), ("fa", F64P), ("iai", I32P), ("jaj", I32P), ("kak", I32P), ("iauk", I32P),
    ("itors", I32P), ("nmul", I32P), ("ft", F64P), ("rt", F64P), ("ft1", F64P), ("ft2", F64P),
    ("ft3", F64P), ("ft4", F64P), ("ft5", F64P),
    ("iti", I32P), ("jtj", I32P), ("ktk", I32P), ("ltl", I32P), ("ituk", I32P),
    ("lcon", I32P),
]


class MdxTopo(C.Structure):
    _fields_ = _TOPO_FIELDS


class MdxParams(C.Structure):
    _fields_ = [
        ("boxl", C.c_double), ("boyl", C.c_double), ("bozl", C.c_double),
        ("icell", C.c_int32), ("lmnbl", C.c_int32),
        ("coulf", C.c_double), ("alphad", C.c_double), ("fexp", C.c_double),
        ("rcut", C.c_double), ("rshort", C.c_double), ("rskin", C.c_double),
        ("rff", C.c_double), ("rff2", C.c_double),
        ("tstep", C.c_double), ("tsteb", C.c_double),
        ("nfreq", C.c_int32), ("ichnb", C.c_int32),
        ("lshejk", C.c_int32), ("maxit", C.c_int32),
        ("toler", C.c_double), ("bdtol", C.c_double),
        ("lnvt", C.c_int32), ("lnpt", C.c_int32), ("lsep", C.c_int32), ("lsctd", C.c_int32),
        ("lp_xy", C.c_int32), ("lsclt", C.c_int32), ("lscft", C.c_int32),
        ("trtemp", C.c_double), ("tdelt", C.c_double),
        ("trpres", C.c_double), ("trpresx", C.c_double), ("trpresy", C.c_double),
        ("trpresz", C.c_double),
        ("dqt", C.c_double), ("dqp", C.c_double), ("rtp", C.c_double),
        ("fnst", C.c_double), ("fnop", C.c_double),
        ("ftscl", C.c_double), ("ftimes", C.c_double),
        ("convet", C.c_double), ("unitp", C.c_double), ("efact", C.c_double),
        ("tfact", C.c_double * NTPS),
        ("tridm_coef", C.c_double), ("tridee_coef", C.c_double),
        ("epd", C.c_double), ("vird", C.c_double), ("chktf", C.c_double),
        ("lmdee", C.c_int32), ("raex", C.c_double), ("ec_me", C.c_double),
        ("ntyp1", C.c_int32), ("molint", C.c_int32),
    ]


class MdxScalars(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "pe1", "pels1", "pe2", "pels2", "spe", "pint", "qpe", "vir1", "vir2", "virb",
        "virx", "viry", "virz", "virfx", "virfy", "virfz", "wirs", "wirss")] + [
        ("pote1", C.c_double * NTPP), ("potl1", C.c_double * NTPP),
        ("pes141", C.c_double * NTPS), ("psr141", C.c_double * NTPS),
        ("spee", C.c_double * NTPS),
        ("mbsh", C.c_int32), ("mbln", C.c_int32), ("nkv", C.c_int32), ("lscfl", C.c_int32)]

    def as_dict(self) -> dict:
        d = {}
        for name, typ in self._fields_:
            v = getattr(self, name)
            d[name] = list(v) if hasattr(v, "__len__") else v
        return d


class MdxThermo(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("sc", "scl", "sclx", "scly", "sclz")] + [
        ("scm", C.c_double * NTPS), ("eabs", C.c_double),
        ("boxl", C.c_double), ("boyl", C.c_double), ("bozl", C.c_double), ("vol", C.c_double),
        ("tke", C.c_double), ("temp", C.c_double),
        ("tempr", C.c_double * (NTPS + 4)), ("ekin", C.c_double * (NTPS + 4)),
        ("virkx", C.c_double), ("virky", C.c_double), ("virkz", C.c_double),
        ("vira", C.c_double * 3), ("viran", C.c_double * 3),
        ("tryck", C.c_double), ("tryckm", C.c_double), ("tryckx", C.c_double),
        ("trycky", C.c_double), ("tryckz", C.c_double),
        ("shake_iter_max", C.c_int32), ("shake_fail", C.c_int32), ("nscale", C.c_int32),
        ("npt_fail", C.c_int32), ("list_builds", C.c_int32), ("reserved", C.c_int32)]


class MdxStepRecord(C.Structure):
    _fields_ = [("mstep", C.c_int32), ("mbsh", C.c_int32), ("mbln", C.c_int32),
                ("shake_iter", C.c_int32)] + [(n, C.c_double) for n in (
        "pe1", "pels1", "pe2", "pels2", "spe", "pint", "vir1", "vir2", "virb", "virx",
        "viry", "virz", "virfx", "virfy", "virfz", "wirs", "wirss", "tke", "temp", "sc",
        "scl", "tryck", "tryckm", "boxl", "boyl", "bozl", "vol", "eabs")]

    def as_dict(self) -> dict:
        return {n: getattr(self, n) for n, _ in self._fields_}


class MdxPathInfo(C.Structure):
    """mdx_path_info: which passes a context runs."""
    _fields_ = [(n, C.c_int32) for n in ("precision", "ewald_force_pass", "ewald_sfac_pass",
                                         "sfac_slices", "sfac_ordered", "list_mode", "graphs",
                                         "nkv")]

    def as_dict(self) -> dict:
        return {n: getattr(self, n) for n, _ in self._fields_}


class MdxTuning(C.Structure):
    """mdx_tuning: threads per owner atom of the mixed pair sweeps."""
    _fields_ = [(n, C.c_int32) for n in ("tpo_short", "tpo_long", "source", "reserved")]

    def as_dict(self) -> dict:
        return {n: getattr(self, n) for n, _ in self._fields_[:3]}


class MdxPullback(C.Structure):
    """mdx_pullback: PULLBACK's drag, wells and external field."""
    _fields_ = [("ldrag", C.c_int32), ("ldragt", C.c_int32 * NTPS), ("fdrag", C.c_double * NTPS),
                ("npull", C.c_int32), ("inpl", I32P), ("xpl", F64P), ("ypl", F64P),
                ("zpl", F64P), ("rlr", C.c_double), ("iext", C.c_int32),
                ("exampl", C.c_double), ("exfreq", C.c_double), ("tim", C.c_double),
                ("dt", C.c_double), ("nstep", C.c_int32)]


def pullback(s: System, drag=None, wells=None, rlr=0.0, field=None, tim=0.0, nstep=0):
    """An MdxPullback (and the arrays it points to) for a System, from the
    values in the reference's input units, converted as setup.f does:

    drag  = {type (1-based): FDRAG in 10^12 m/s^2}  (x 1e12 UNITT^2/UNITL,
            setup.f:250)
    wells = (atoms 1-based, x, y, z in A), rlr = the allowed deviation in A
            (RLR = 1/(BETA RLR^2), setup.f:113)
    field = (EXAMPL in V/cm, EXFREQ in Hz)  (EXAMPL x UNITL 1e2 ELECHG/UNITE,
            setup.f:263)
    tim   = TIM in s, nstep = NSTEP (the field's time is TIM + NSTEP DT)."""
    from .system import BOLTZ, ELECHG
    pb = MdxPullback()
    keep = []
    if drag:
        pb.ldrag = 1
        for t, f in drag.items():
            pb.ldragt[t - 1] = 1
            pb.fdrag[t - 1] = f * (1.0e12 * s.unitt ** 2 / s.unitl)
    if wells is not None:
        atoms, x, y, z = (np.ascontiguousarray(a) for a in wells)
        atoms = atoms.astype(np.int32)
        x, y, z = (a.astype(np.float64) for a in (x, y, z))
        keep += [atoms, x, y, z]
        pb.npull = len(atoms)
        pb.inpl = atoms.ctypes.data_as(I32P)
        pb.xpl, pb.ypl, pb.zpl = (a.ctypes.data_as(F64P) for a in (x, y, z))
        beta = s.unite / (BOLTZ * s.trtemp)
        pb.rlr = 1.0 / (beta * rlr ** 2)
    if field is not None:
        pb.iext = 1
        pb.exampl = field[0] * s.unitl * 1.0e2 * ELECHG / s.unite
        pb.exfreq = field[1]
    pb.tim = tim
    pb.dt = s.unitt
    pb.nstep = nstep
    pb._keep = keep
    return pb


class MdxKin(C.Structure):
    """mdx_kin: GETKIN's kinetic energies and temperatures."""
    _fields_ = [(n, C.c_double) for n in ("ektr", "ekrot", "ekint", "tke", "ttr", "trot",
                                          "tint")]


class MdxPimdParams(C.Structure):
    _fields_ = [("nbeads", C.c_int32), ("jnh", C.c_int32), ("beadfac", C.c_double),
                ("conveq", C.c_double), ("dqqt", C.c_double), ("fnh", C.c_double)]


class MdxPimdRecord(C.Structure):
    _fields_ = [("mstep", C.c_int32)] + [(n, C.c_double) for n in (
        "qek", "virpi", "pe", "tke", "temp")]

    def as_dict(self) -> dict:
        return {n: getattr(self, n) for n, _ in self._fields_}


def records_to_dicts(recs) -> List[dict]:
    return [r.as_dict() for r in recs]


@dataclass
class Packed:
    dims: MdxDims
    topo: MdxTopo
    params: MdxParams
    keep: list


def _i32(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.int32))


def _f64(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64))


def default_caps(s: System):
    """Per-atom capacities of the owned short and long lists."""
    rho = s.nstot / (s.boxl * s.boyl * s.bozl)
    rl = s.spec.rcut + s.spec.rskin
    mean_long = (2.0 / 3.0) * math.pi * rl ** 3 * rho
    mean_short = (2.0 / 3.0) * math.pi * s.spec.rshort ** 3 * rho
    cap_long = int(math.ceil(1.6 * mean_long + 96))
    cap_short = int(math.ceil(2.0 * mean_short + 16 + s.nbdmax))
    return cap_short, cap_long


def pack(s: System, precision: int = MDX_FP64, cap_short: int = 0, cap_long: int = 0,
         nkv_max: int = 0) -> Packed:
    keep = []

    def p(arr, kind):
        a = _i32(arr) if kind == "i" else _f64(arr)
        keep.append(a)
        return a.ctypes.data_as(I32P if kind == "i" else F64P)

    cs, cl = default_caps(s)
    dims = MdxDims(nstot=s.nstot, nop=s.nop, ntypes=s.ntypes, nsites=s.nsites, nnbt=s.nnbt,
                   nrbb=s.nrbb, nraa=s.nraa, nrtt=s.nrtt, nrbt=s.nrbt, nrat=s.nrat,
                   nrrt=s.nrrt, nbdmax=s.nbdmax, cap_short=cap_short or cs,
                   cap_long=cap_long or cl,
                   nkv_max=nkv_max or max(100000, int(1.3 * s.kvector_count()) + 64),
                   precision=precision)
    nt = s.ntypes
    t = MdxTopo()
    t.itype = p(s.itype, "i"); t.nnum = p(s.nnum, "i"); t.nsite = p(s.nsite, "i")
    t.massdi = p(s.massdi, "f"); t.q = p(s.q, "f")
    t.charge = p(s.site_charge, "f"); t.mass = p(s.site_mass, "f"); t.inbt = p(s.inbt, "i")
    t.nspec = p(s.nspec, "i"); t.nsits = p(s.nsits, "i")
    t.isadr = p(s.isadr[:nt], "i"); t.isaddr = p(s.isaddr[:nt], "i"); t.iaddr = p(s.iaddr[:nt], "i")
    t.ipot = p(s.ipot, "i"); t.nrb = p(s.nrb, "i"); t.iadb = p(s.iadb, "i")
    t.ishejk = p(s.ishejk, "i"); t.iee = p(s.iee, "i"); t.lmove = p(s.lmove, "i")
    t.c14el = p(s.c14el, "f"); t.c14lj = p(s.c14lj, "f"); t.summas = p(s.summas, "f")
    # LJ tables: numpy [i, j] row-major; Fortran column-major (i,j) at i + j*ld,
    # i.e. the transposed C array.  The tables are symmetric anyway.
    for name in ("a6lj", "b12lj", "a6lj0", "b12lj0", "a6_14", "b12_14"):
        setattr(t, name, p(np.asarray(getattr(s, name)).T.copy(), "f"))
    t.ld_lj = s.nnbt
    t.mdx = p(s.mdx.T.copy(), "i"); t.ld_mdx = NTPS
    t.nnbb = p(s.nnbb, "i"); t.inbb = p(s.inbb, "i"); t.ld_inbb = s.ld_inbb
    t.ib = p(s.b_ib, "i"); t.jb = p(s.b_jb, "i"); t.id = p(s.b_id, "i")
    t.rb = p(s.b_rb, "f"); t.fb = p(s.b_fb, "f"); t.db = p(s.b_db, "f"); t.ro = p(s.b_ro, "f")
    t.ibi = p(s.ibi, "i"); t.jbj = p(s.jbj, "i"); t.ibuk = p(s.ibuk, "i")
    t.ra = p(s.a_ra, "f"); t.fa = p(s.a_fa, "f")
    t.iai = p(s.iai, "i"); t.jaj = p(s.jaj, "i"); t.kak = p(s.kak, "i"); t.iauk = p(s.iauk, "i")
    t.itors = p(s.t_itors, "i"); t.nmul = p(s.t_nmul, "i")
    for name, src in (("ft", s.t_ft), ("rt", s.t_rt), ("ft1", s.t_ft1), ("ft2", s.t_ft2),
                      ("ft3", s.t_ft3), ("ft4", s.t_ft4), ("ft5", s.t_ft5)):
        setattr(t, name, p(src, "f"))
    t.iti = p(s.iti, "i"); t.jtj = p(s.jtj, "i"); t.ktk = p(s.ktk, "i"); t.ltl = p(s.ltl, "i")
    t.ituk = p(s.ituk, "i")
    t.lcon = p(s.b_lcon, "i")
    par = params_of(s)
    return Packed(dims, t, par, keep)


def params_of(s: System) -> MdxParams:
    sp = s.spec
    par = MdxParams()
    par.boxl, par.boyl, par.bozl = s.boxl, s.boyl, s.bozl
    par.icell = int(sp.icell)
    par.lmnbl = int(s.lmnbl)
    par.rff = s.rff
    par.rff2 = s.rff2
    par.coulf = s.coulf
    par.alphad = s.alphad
    par.fexp = s.fexp
    par.rcut = s.rcutt
    par.rshort = sp.rshort
    par.rskin = sp.rskin
    par.tstep = s.tstep
    par.tsteb = s.tsteb
    par.nfreq = sp.nfreq
    par.ichnb = sp.ichnb
    par.lshejk = int(s.lshejk)
    par.maxit = 2000
    par.toler = sp.toler
    par.bdtol = float(np.float32(0.0001))
    par.lnvt = int(s.lnvt)
    par.lnpt = int(s.lnpt)
    par.lsep = int(sp.anisotropic)
    par.lsctd = 0
    par.lp_xy = 0
    par.lsclt = 0
    par.lscft = int(sp.cut_forces is not None)
    par.trtemp = s.trtemp
    par.tdelt = 0.0
    par.trpres = s.trpres
    par.trpresx = s.trpres if s.lnpt else 1.0
    par.trpresy = s.trpres if s.lnpt else 1.0
    par.trpresz = s.trpres if s.lnpt else 1.0
    par.dqt = s.dqt
    par.dqp = s.dqp
    par.rtp = s.rtp
    par.fnst = s.fnst
    par.fnop = s.fnop
    par.ftscl = 1.0 / sp.cut_forces if sp.cut_forces else 0.0  # FTSCL=1./FTSCL, main.f:850
    par.ftimes = s.ftimes
    par.convet = s.convet
    par.unitp = s.unitp
    par.efact = s.efact
    for i in range(NTPS):
        par.tfact[i] = s.tfact[i]
    par.tridm_coef = s.nop * BOLTZ * 1.0e-5 / s.unitl ** 3  # 1.d-5, mdstep.f:608
    par.tridee_coef = 0.0
    par.epd = s.epd
    par.vird = s.vird
    par.chktf = 0.0
    par.lmdee = 0
    par.raex = 0.0
    par.ec_me = 1.0
    par.ntyp1 = s.ntypes + 1
    par.molint = s.molint
    return par


def thermo_init(s: System) -> MdxThermo:
    th = MdxThermo()
    th.boxl, th.boyl, th.bozl = s.boxl, s.boyl, s.bozl
    th.vol = s.boxl * s.boyl * s.bozl
    return th
