"""Host-side set-up of an MDynaMix system: topology, internal units, tables.

In a real drop-in the Fortran driver does all of this (READMOL, IUNITS,
BNDLST, ELRCLJ) and passes its COMMON-block arrays through the C ABI.  This
module restates that set-up in Python so that tests, the benchmark and the
oracle can produce exactly the arrays the Fortran would hand over:

* ``parse_mmol``          READMOL            input.f:936-1340
* ``System.__init__``     main.f:229-450 (counts, degrees of freedom,
                          thermostat constants) and IUNITS setup.f:27-702
* ``_lj_types``           IUNITS 1.8         setup.f:433-569
* ``comb_rules``          COMB_RULES         setup.f:709-747
* ``_bndlst``             BNDLST/BNDREG      setup.f:753-939
* ``elrclj``              ELRCLJ             forces.f:1684-1746
* ``ewald_alpha``         main.f:795-812
* ``make_configuration``  seeded start: jittered lattice, random
                          orientations, Maxwell momenta rescaled as in
                          main.f:679-714 (the reference's own lattices and
                          LCG generator are not reproduced)

All arrays use the reference's 1-based index values.  Fortran REAL*4
literals that feed double-precision results (``1.e-5`` in UNITP,
setup.f:103) are reproduced through ``np.float32``.
"""
from __future__ import annotations

import json
import math
import os
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

# common_inc.f:22-33
AVSNO = 6.02252e23
BOLTZ = 1.38054e-23
FKCALJ = 4.1868
ELECHG = 1.602e-19
EPS0 = 8.854e-12
HPLANK = 1.0545e-34
PI = 3.1415926536
TOTPI = 1.128379169
TODGR = 180.0 / PI
COS30 = float(np.float32(0.8660254037844386))  # REAL*4 literal, common_inc.f:33
NTPS = 10
NTPP = NTPS * (NTPS + 1) // 2 + 1
F32_1EM5 = float(np.float32(1.0e-5))           # UNITP literal, setup.f:103
COS30 = float(np.float32(0.8660254037844386))  # cos30, a REAL*4 literal (common_inc.f:33)
BDTOL_DEFAULT = float(np.float32(0.0001))       # main.f:124

DATA_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data")


# ---------------------------------------------------------------- .mmol ----
def _num_tokens(line: str, n: int) -> List[str]:
    """First n whitespace tokens of a list-directed read line."""
    toks = line.split()
    return toks[:n]


def _is_number(tok: str) -> bool:
    try:
        float(tok.replace("d", "e").replace("D", "e"))
        return True
    except ValueError:
        return False


def _f(tok: str) -> float:
    return float(tok.replace("d", "e").replace("D", "e"))


def parse_mmol(text: str, name: str = "") -> dict:
    """Parse a ``.mmol`` topology the way READMOL (input.f:936-1340) does.

    Lines whose first character is '#' are skipped (TAKESTR, input.f:1361).
    Bond lines take 7 values when present, else 5 (input.f:1063-1071); a
    negative bond length is taken from the coordinates (input.f:1074-1076);
    angles with RA <= 0 are taken from the coordinates (input.f:1102).
    Optional sections: Tors1/Tors5/Impro torsions, sel14/slj14 scaling,
    'Speci' special 1-4 LJ, fSPC flexible water (input.f:1140-1318).
    """
    lines = [ln.rstrip("\n") for ln in text.splitlines()]
    it = iter([ln for ln in lines if not ln.startswith("#")])

    def take() -> str:
        return next(it)

    nsts = int(_num_tokens(take(), 1)[0])
    sites = []
    for _ in range(nsts):
        t = take().split()
        sites.append(dict(name=t[0], r=[_f(t[1]), _f(t[2]), _f(t[3])],
                          mass=_f(t[4]), charge=_f(t[5]), sigma=_f(t[6]),
                          eps=_f(t[7])))
    # COM shift (input.f:983-1013)
    mass = np.array([s["mass"] for s in sites])
    r = np.array([s["r"] for s in sites], dtype=np.float64)
    summ = float(np.sum(mass))
    cm = [0.0, 0.0, 0.0]
    for k in range(3):
        acc = 0.0
        for i in range(nsts):
            acc = acc + r[i, k] * mass[i]
        cm[k] = acc / summ
    for k in range(3):
        for i in range(nsts):
            r[i, k] = r[i, k] - cm[k]
    nsr = int(_num_tokens(take(), 1)[0])
    for _ in range(nsr):
        take()
    nbd = int(_num_tokens(take(), 1)[0])
    bonds = []
    for _ in range(nbd):
        t = take().split()
        vals = []
        for tok in t:
            if not _is_number(tok):
                break
            vals.append(tok)
        if len(vals) >= 7:
            idb, ib, jb = int(vals[0]), int(vals[1]), int(vals[2])
            rb, fb, db, ro = _f(vals[3]), _f(vals[4]), _f(vals[5]), _f(vals[6])
        else:
            idb, ib, jb = int(vals[0]), int(vals[1]), int(vals[2])
            rb, fb, db, ro = _f(vals[3]), _f(vals[4]), 0.0, 0.0
        if rb < 0.0:
            d = r[ib - 1] - r[jb - 1]
            rb = math.sqrt(d[0] ** 2 + d[1] ** 2 + d[2] ** 2)
        bonds.append(dict(id=idb, i=ib, j=jb, rb=rb, fb=fb, db=db, ro=ro))
    nan = int(_num_tokens(take(), 1)[0])
    angles = []
    for _ in range(nan):
        t = take().split()
        ia, ja, ka = int(t[0]), int(t[1]), int(t[2])
        ra, fa = _f(t[3]), _f(t[4])
        if ra <= 0:
            a = r[ia - 1] - r[ja - 1]
            b = r[ka - 1] - r[ja - 1]
            ra = math.acos(float(a @ b) / math.sqrt(float(a @ a) * float(b @ b))) * TODGR
        angles.append(dict(i=ia, j=ja, k=ka, ra=ra, fa=fa))
    ntt = int(_num_tokens(take(), 1)[0])
    tors = []
    for _ in range(ntt):
        t = take().split()
        tors.append(dict(itors=0, i=int(t[0]), j=int(t[1]), k=int(t[2]),
                         l=int(t[3]), rt=_f(t[4]), ft=_f(t[5]), nmul=int(t[6]),
                         ft1=0.0, ft2=0.0, ft3=0.0, ft4=0.0, ft5=0.0))
    mol = dict(name=name, sites=sites, r=r.tolist(), summas=summ, bonds=bonds,
               angles=angles, tors=tors, c14el=1.0, c14lj=1.0, ipot=0,
               special14=[], par14=[])
    # optional sections (input.f:1140-1318)
    while True:
        try:
            s = take()
        except StopIteration:
            break
        st = s.strip()
        if not st:
            continue
        nmf = st[:5]
        low = nmf.lower()
        if low == "tors1":
            n = int(_num_tokens(take(), 1)[0])
            for _ in range(n):
                t = take().split()
                tors.append(dict(itors=1, i=int(t[0]), j=int(t[1]), k=int(t[2]),
                                 l=int(t[3]), rt=0.0, ft=0.0, nmul=0,
                                 ft1=_f(t[4]), ft2=_f(t[5]), ft3=_f(t[6]),
                                 ft4=0.0, ft5=0.0))
        elif low == "tors5":
            n = int(_num_tokens(take(), 1)[0])
            for _ in range(n):
                t = take().split()
                f1, f2, f3, f4, f5 = (_f(x) for x in t[4:9])
                tors.append(dict(itors=5, i=int(t[0]), j=int(t[1]), k=int(t[2]),
                                 l=int(t[3]), rt=180.0, ft=-(f1 + f2 + f3 + f4 + f5),
                                 nmul=0, ft1=f1, ft2=f2, ft3=f3, ft4=f4, ft5=f5))
        elif low == "impro":
            n = int(_num_tokens(take(), 1)[0])
            for _ in range(n):
                t = take().split()
                tors.append(dict(itors=-1, i=int(t[0]), j=int(t[1]), k=int(t[2]),
                                 l=int(t[3]), rt=_f(t[4]), ft=_f(t[5]), nmul=0,
                                 ft1=0.0, ft2=0.0, ft3=0.0, ft4=0.0, ft5=0.0))
        elif low == "sel14":
            mol["c14el"] = _f(st.split()[1])
        elif low == "slj14":
            mol["c14lj"] = _f(st.split()[1])
        elif low == "speci":
            n = int(_num_tokens(take(), 1)[0])
            for _ in range(n):
                t = take().split()
                mol["special14"].append(dict(site=int(t[0]), sigma=_f(t[1]),
                                             eps=_f(t[2])))
        elif low == "par14":
            n = int(_num_tokens(take(), 1)[0])
            for _ in range(n):
                t = take().split()
                mol["par14"].append(dict(i=int(t[0]), j=int(t[1]), sigma=_f(t[2]),
                                         eps=_f(t[3])))
        elif st[:4] == "fSPC":
            if nsts != 3:
                raise ValueError("fSPC needs a 3-site molecule")
            mol["ipot"] = 2
        elif st[:3].lower() == "end":
            break
    return mol


def load_moldb(path: Optional[str] = None) -> Dict[str, dict]:
    """Parsed topologies committed with the package (see data/make_moldb.py)."""
    path = path or os.path.join(DATA_DIR, "moldb.json")
    with open(path) as fh:
        return json.load(fh)


# --------------------------------------------------------- combination ----
def comb_rules(s1, s2, e1, e2, m1, m2, icr=0):
    """COMB_RULES, setup.f:709-747.  Returns (A6, B12)."""
    if icr == 1:
        a6 = -4.0 * math.sqrt(e1 * e2) * (s1 * s2) ** 3
        b12 = 4.0 * math.sqrt(e1 * e2) * (s1 * s2) ** 6
    elif icr == 2:
        a6 = -math.sqrt(e1 * e2) * (s1 * s2) ** 3
        if e1 * s1 ** 12 == 0.0:
            b12 = 0.0
        else:
            b12 = (e1 * s1 ** 12 / 2.0 ** 13) * (1 + (e2 * s2 ** 12 / (e1 * s1 ** 12)) ** (1.0 / 13.0)) ** 13
    elif icr == 3:
        a6 = -8.0 * (e1 * e2) * (0.5 * (s1 + s2)) ** 6 / (e1 + e2) if e1 + e2 != 0 else 0.0
        b12 = 8.0 * (e1 * e2) * (0.5 * (s1 + s2)) ** 12 / (e1 + e2) if e1 + e2 != 0 else 0.0
    elif icr in (4, 5) and not (icr == 5 and (m1 < 2.5 or m2 < 2.5)):
        sip6 = (s1 ** 6 + s2 ** 6) / 2
        ep = 2 * math.sqrt(e1 * e2) * (s1 ** 3 * s2 ** 3 / (s1 ** 6 + s2 ** 6)) if sip6 else 0.0
        a6 = -4.0 * ep * sip6
        b12 = 4.0 * ep * sip6 ** 2
    else:
        a6 = -4.0 * math.sqrt(e1 * e2) * (0.5 * (s1 + s2)) ** 6
        b12 = 4.0 * math.sqrt(e1 * e2) * (0.5 * (s1 + s2)) ** 12
    return a6, b12


def ewald_alpha(alpha_in: float, rcut: float, box_min: float) -> float:
    """ALPHAD from the input ALPHA (main.f:803-810)."""
    if rcut <= 0.5 * box_min:
        return alpha_in / rcut
    return 2.0 * alpha_in / box_min


def kvector_count(alphad: float, fexp: float, boxl: float, boyl: float,
                  bozl: float, icell: int = 0) -> int:
    """Number of k-vectors INIFUR (forces.f:1356-1412) keeps."""
    twopi = 2.0 * PI
    cutk2 = 4.0 * alphad ** 2 * fexp
    cutk = math.sqrt(cutk2)
    kmax = int(cutk * boxl / twopi + 1)
    kmay = int(cutk * boyl / twopi + 1)
    kmaz = int(cutk * bozl / twopi + 1)
    n = 0
    for ikz in range(-kmaz, kmaz + 1):
        for ikx in range(0, kmax + 1):
            if ikx == 0:
                ky1 = 0 if ikz > 0 else 1
            else:
                ky1 = -kmay
            for iky in range(ky1, kmay + 1):
                if icell == 1:
                    rxv, ryv, rzv = twopi * ikx, twopi * iky, twopi * (-ikx + iky + 2 * ikz)
                elif icell == 2:
                    rxv, ryv, rzv = twopi * ikx, twopi * iky + PI * ikx, twopi * ikz
                else:
                    rxv, ryv, rzv = twopi * ikx, twopi * iky, twopi * ikz
                rk2 = (rxv / boxl) ** 2 + (ryv / boyl) ** 2 + (rzv / bozl) ** 2
                if rk2 <= cutk2:
                    n += 1
    return n


def kin_summd(s) -> List[float]:
    """GETKIN's molecular masses in internal units, SUMMAS / (AVSNO 1000
    UNITM NBEADS) per type (service.f:619)."""
    return [s.summas[t] / (AVSNO * 1000.0 * s.unitm * s.spec.nbeads) for t in range(s.ntypes)]


def kin_sumasd(s) -> float:
    """CHKMOM's total mass, TOTMAS / UNITM (service.f:1096)."""
    return s.totmas / s.unitm


def kcolumn_counts(alphad: float, fexp: float, boxl: float, boyl: float,
                   bozl: float) -> Tuple[int, int, int]:
    """(columns, paired records, table rows) of the rectangular-cell k-set
    INIFUR keeps (forces.f:1356-1412) as the GPU passes walk it: a column is
    one (nx, ny) with its contiguous nz range, a paired record one p = 0..m,
    m = max |nz|, covering nz = +p and -p; rows = (KMAX+1) + (KMAY+1) +
    (KMAZ+1) phase-table rows per atom."""
    twopi = 2.0 * PI
    cutk2 = 4.0 * alphad ** 2 * fexp
    cutk = math.sqrt(cutk2)
    kmax = int(cutk * boxl / twopi + 1)
    kmay = int(cutk * boyl / twopi + 1)
    kmaz = int(cutk * bozl / twopi + 1)
    cols = {}
    for ikz in range(-kmaz, kmaz + 1):
        for ikx in range(0, kmax + 1):
            ky1 = (0 if ikz > 0 else 1) if ikx == 0 else -kmay
            for iky in range(ky1, kmay + 1):
                rk2 = ((twopi * ikx / boxl) ** 2 + (twopi * iky / boyl) ** 2
                       + (twopi * ikz / bozl) ** 2)
                if rk2 <= cutk2:
                    m = cols.get((ikx, iky), 0)
                    cols[(ikx, iky)] = max(m, abs(ikz))
    npair = sum(m + 1 for m in cols.values())
    return len(cols), npair, kmax + kmay + kmaz + 3


# ---------------------------------------------------------------- spec ----
@dataclass
class RunSpec:
    """The md.input keywords this path needs (input.f:166-674 defaults)."""
    molecules: List[Tuple[str, int]]
    density: float = 1.0                 # Density (g/cm3); ignored if box set
    box: Optional[Tuple[float, float, float]] = None
    dt_fs: float = 2.0                   # Time_step
    nfreq: int = 1                       # Double_timestep
    rcut: float = 12.0                   # R_cutoff
    rshort: float = 5.0                  # R_short
    alpha: float = 2.8                   # Electrostatics Ewald A B
    fexp: float = 9.0
    ichnb: int = 10                      # Neighbour_list
    shake: bool = False                  # Constrain TOLER [ISHEJK..]
    toler: float = 1e-5
    ishejk: Optional[List[int]] = None
    nvt: Optional[Tuple[float, float]] = None     # Nose_thermostat T QT
    npt: Optional[Tuple[float, float]] = None     # Barostate_NH P QPR
    anisotropic: bool = False                     # Barostate_anisotropic
    trtemp: float = 298.0
    lmove: Optional[List[int]] = None
    icr: int = 0                                   # combination rule
    cut_forces: Optional[float] = None             # Cut_forces FTSCL
    shake_hbonds: bool = False                     # constrain bonds to H only (not in the reference)
    rskin: float = 0.0                             # list skin (build mode)
    iee_type: Optional[int] = None                 # EE_type (1-based)
    nbeads: int = 1                                # PIMD NBEADS (bead masses MASS/NBEADS)
    pi_thermo: Optional[Tuple[float, int]] = None  # PI_thermo BTAU (fs), JNH (TRTEMP: trtemp)
    icell: int = 0                                 # PBC: 0 rectangular, 1 truncated octahedron, 2 hexagonal


class System:
    """Everything IUNITS/BNDLST would leave in the COMMON blocks."""

    def __init__(self, spec: RunSpec, moldb: Optional[Dict[str, dict]] = None):
        db = moldb if moldb is not None else load_moldb()
        self.spec = spec
        self.types = [db[name] for name, _ in spec.molecules]
        self.nspec = np.array([n for _, n in spec.molecules], dtype=np.int32)
        self.ntypes = len(self.types)
        if self.ntypes > NTPS:
            raise ValueError("more molecule types than NTPS")
        self.nsits = np.array([len(t["sites"]) for t in self.types], dtype=np.int32)
        self.nop = int(self.nspec.sum())
        self.nsites = int(self.nsits.sum())
        self.nstot = int((self.nspec * self.nsits).sum())
        self.lmove = np.array(spec.lmove if spec.lmove else [1] * self.ntypes, dtype=np.int32)
        self.ipot = np.array([t["ipot"] for t in self.types], dtype=np.int32)
        self.iee = np.ones(self.ntypes, dtype=np.int32)
        if spec.iee_type is not None:
            self.iee[spec.iee_type - 1] = 0
        self.c14el = np.array([t["c14el"] for t in self.types])
        self.c14lj = np.array([t["c14lj"] for t in self.types])
        self.summas = np.array([t["summas"] for t in self.types])
        self.lshejk = bool(spec.shake)
        self.ishejk = np.array(spec.ishejk if spec.ishejk else [1] * self.ntypes, dtype=np.int32)
        # per-type bond/angle/torsion records (READMOL appends type by type)
        self.nrb = np.array([len(t["bonds"]) for t in self.types], dtype=np.int32)
        self.nra = np.array([len(t["angles"]) for t in self.types], dtype=np.int32)
        self.nrt = np.array([len(t["tors"]) for t in self.types], dtype=np.int32)
        # SHAKE constraints per bond record: the reference's ID != 2
        # (mdstep.f:1135), or with shake_hbonds only those of them that
        # bind a hydrogen (a site lighter than 1.5 amu)
        def con(t, b):
            if b["id"] == 2:
                return 0
            if not spec.shake_hbonds:
                return 1
            m = [t["sites"][b["i"] - 1]["mass"], t["sites"][b["j"] - 1]["mass"]]
            return int(min(m) < 1.5)
        self.b_lcon = np.array([con(t, b) for t in self.types for b in t["bonds"]],
                               dtype=np.int32)
        self.nrcon = np.array([sum(con(t, b) for b in t["bonds"]) for t in self.types],
                              dtype=np.int32)
        self.iadb = (np.concatenate([[0], np.cumsum(self.nrb)[:-1]]) + 1).astype(np.int32)
        self.iada = (np.concatenate([[0], np.cumsum(self.nra)[:-1]]) + 1).astype(np.int32)
        self.iadt = (np.concatenate([[0], np.cumsum(self.nrt)[:-1]]) + 1).astype(np.int32)
        self._degrees_of_freedom()
        self._units()
        self._addresses()
        self._bonded_tables()
        self._lj_types()
        self._bonded_instances()
        self._bndlst()
        self._params()

    # main.f:289-350
    def _degrees_of_freedom(self):
        """FNST (total), FTTR (translational), FNSTR (rotational) and FNSTI
        (internal) degrees of freedom, main.f:297-350."""
        fnst = fttr = fnstr = 0.0
        lma = True
        for t in range(self.ntypes):
            if self.lmove[t]:
                fnst += 3 * self.nspec[t] * self.nsits[t]
                fttr += 3 * self.nspec[t]
                if self.lshejk and self.ishejk[t] > 0:
                    fnst -= self.nrcon[t] * self.nspec[t]
                if self.nsits[t] == 2:
                    fnstr += 2.0 * self.nspec[t]
                if self.nsits[t] >= 3:
                    fnstr += 3.0 * self.nspec[t]
            else:
                lma = False
        self.fnsti = float(fnst - fttr - fnstr)
        if lma and self.nop > 1 and self.spec.nbeads <= 1:
            fnst -= 3.0
            fttr -= 3.0
        self.fnst = float(fnst)
        self.fttr = float(fttr)
        self.fnstr = float(fnstr)

    # setup.f:27-113
    def _units(self):
        sp = self.spec
        totmas_amu = 0.0
        for t in range(self.ntypes):
            totmas_amu = totmas_amu + self.summas[t] * self.nspec[t]
        self.totmas_amu = totmas_amu
        factm = AVSNO * 1000.0
        totmas = totmas_amu / factm
        self.totmas = totmas
        fnop = float(self.nop)
        self.fnop = fnop
        avofnr = AVSNO / fnop
        if sp.box is None:  # setup.f:38-60
            volm = avofnr * (totmas / (sp.density * 1000.0))
            vol = volm * fnop * 1.0e30 / AVSNO
            if sp.icell == 1:
                vol = 2.0 * vol
            elif sp.icell == 2:
                vol = vol / COS30
            cl = vol ** (1.0 / 3.0)
            self.boxl = self.boyl = self.bozl = cl
            if sp.icell == 2:
                self.boyl = self.boxl * COS30
        else:
            self.boxl, self.boyl, self.bozl = (float(x) for x in sp.box)
            if sp.icell == 2:  # RECLEN (service.f:576-579)
                self.boyl = self.boxl * COS30
            elif sp.icell == 1:
                self.boyl = self.bozl = self.boxl
        self.vol = self.boxl * self.boyl * self.bozl
        if sp.icell == 1:  # the truncated octahedron is half its cube (service.f:602)
            self.vol = 0.5 * self.vol
        self.rcutt = sp.rcut
        if sp.alpha <= 0.0:  # reaction field: a spherical cutoff within L/2 (main.f:745-749)
            self.rcutt = min(self.rcutt, 0.5 * min(self.boxl, self.boyl, self.bozl))
        self.rssq = self.rcutt ** 2
        dt = sp.dt_fs * 1.0e-15
        self.unitl = 1.0e-10
        self.unitm = totmas
        self.unitt = dt
        self.unite = self.unitm * (self.unitl / self.unitt) ** 2
        self.unitp = self.unite * F32_1EM5 / self.unitl ** 3
        self.ftimes = 1.0 / float(sp.nfreq)
        self.tstep = self.unitt / math.sqrt((self.unitm / self.unite) * self.unitl ** 2)
        self.htstep = 0.5 * self.tstep
        self.tsteb = self.tstep * self.ftimes
        self.htsteb = 0.5 * self.tsteb
        self.trtemp = sp.nvt[0] if sp.nvt else sp.trtemp
        self.enerf = AVSNO * self.unite
        self.tempf = 2.0 / (3.0 * AVSNO * BOLTZ)
        self.coulf = (ELECHG / EPS0) * (ELECHG / self.unite) / (4.0 * PI * self.unitl)
        self.permol = self.enerf * 1.0e-3 / fnop
        self.short2 = sp.rshort ** 2
        self.convet = 3.0 * self.enerf * self.tempf / self.fnst
        self.tfact = np.zeros(NTPS)
        for t in range(self.ntypes):
            fnss3 = 3.0 * float(self.nsits[t])
            fnss1 = self.nstot / (self.nstot - 1.0)
            tf = self.enerf * self.tempf * fnss1 / (self.nsits[t] * self.nspec[t])
            if self.lshejk and self.ishejk[t] != 0:
                tf = tf * fnss3 / (fnss3 - self.nrcon[t])
            self.tfact[t] = tf
        self.factm = factm
        self.efact = 1.0e3 / AVSNO / self.unite

    # setup.f:131-250, 533-569 (Q, MASSDI, addresses, MDX)
    def _addresses(self):
        nt = self.ntypes
        self.iaddr = np.zeros(nt + 1, dtype=np.int32)
        self.isadr = np.zeros(nt + 1, dtype=np.int32)
        self.isaddr = np.zeros(nt + 1, dtype=np.int32)
        for t in range(nt):
            self.iaddr[t + 1] = self.iaddr[t] + self.nspec[t]
            self.isadr[t + 1] = self.isadr[t] + self.nsits[t]
            self.isaddr[t + 1] = self.isaddr[t] + self.nsits[t] * self.nspec[t]
        self.site_mass = np.concatenate([[s["mass"] for s in t["sites"]] for t in self.types])
        self.site_charge = np.concatenate([[s["charge"] for s in t["sites"]] for t in self.types])
        self.site_sigma = np.concatenate([[s["sigma"] for s in t["sites"]] for t in self.types])
        self.site_eps = np.concatenate([[s["eps"] for s in t["sites"]] for t in self.types])
        self.site_r = np.concatenate([np.array(t["r"]) for t in self.types], axis=0)
        self.site_type = np.concatenate([[i + 1] * len(t["sites"]) for i, t in enumerate(self.types)]).astype(np.int32)
        nb = self.spec.nbeads  # NBEADS (setup.f:149)
        self.massd_site = self.site_mass / (nb * self.factm * self.unitm)
        n = self.nstot
        self.itype = np.zeros(n, dtype=np.int32)
        self.nnum = np.zeros(n, dtype=np.int32)
        self.nsite = np.zeros(n, dtype=np.int32)
        self.itm = np.zeros(self.nop, dtype=np.int32)
        iatom = 0
        imol = 0
        ist = 0
        for t in range(nt):
            for _ in range(self.nspec[t]):
                imol += 1
                for i in range(self.nsits[t]):
                    self.nnum[iatom] = imol
                    self.nsite[iatom] = ist + i + 1
                    self.itype[iatom] = t + 1
                    iatom += 1
                self.itm[imol - 1] = t + 1
            ist += self.nsits[t]
        self.massdi = 1.0 / self.massd_site[self.nsite - 1]
        self.charge_atom = self.site_charge[self.nsite - 1].copy()
        self.q = self.charge_atom.copy()
        self.mdx = np.zeros((NTPS, NTPS), dtype=np.int32)  # [ityp-1, jtyp-1]
        mt = 0
        for i in range(nt):
            for j in range(i, nt):
                mt += 1
                self.mdx[i, j] = mt
                self.mdx[j, i] = mt
        self.molint = mt + 1

    # setup.f:397-429 unit conversion of bonded parameters
    def _bonded_tables(self):
        ef = self.efact
        b = [bd for t in self.types for bd in t["bonds"]]
        self.nrbb = len(b)
        self.b_id = np.array([x["id"] for x in b], dtype=np.int32)
        self.b_ib = np.array([x["i"] for x in b], dtype=np.int32)
        self.b_jb = np.array([x["j"] for x in b], dtype=np.int32)
        self.b_rb = np.array([x["rb"] for x in b], dtype=np.float64)
        self.b_fb = np.array([x["fb"] * ef for x in b], dtype=np.float64)
        self.b_db = np.array([x["db"] * ef for x in b], dtype=np.float64)
        self.b_ro = np.array([x["ro"] for x in b], dtype=np.float64)
        a = [ag for t in self.types for ag in t["angles"]]
        self.nraa = len(a)
        self.a_ra = np.array([x["ra"] / TODGR for x in a], dtype=np.float64)
        self.a_fa = np.array([x["fa"] * ef for x in a], dtype=np.float64)
        self.a_ia = np.array([x["i"] for x in a], dtype=np.int32)
        self.a_ja = np.array([x["j"] for x in a], dtype=np.int32)
        self.a_ka = np.array([x["k"] for x in a], dtype=np.int32)
        tr = [tt for t in self.types for tt in t["tors"]]
        self.nrtt = len(tr)
        self.t_itors = np.array([x["itors"] for x in tr], dtype=np.int32)
        self.t_nmul = np.array([x["nmul"] for x in tr], dtype=np.int32)
        self.t_rt = np.array([x["rt"] / TODGR for x in tr], dtype=np.float64)
        self.t_ft = np.array([x["ft"] * ef for x in tr], dtype=np.float64)
        self.t_ft1 = np.array([x["ft1"] * ef for x in tr], dtype=np.float64)
        self.t_ft2 = np.array([x["ft2"] * ef for x in tr], dtype=np.float64)
        self.t_ft3 = np.array([x["ft3"] * ef for x in tr], dtype=np.float64)
        self.t_ft4 = np.array([x["ft4"] * ef for x in tr], dtype=np.float64)
        self.t_ft5 = np.array([x["ft5"] * ef for x in tr], dtype=np.float64)
        self.t_i = np.array([x["i"] for x in tr], dtype=np.int32)
        self.t_j = np.array([x["j"] for x in tr], dtype=np.int32)
        self.t_k = np.array([x["k"] for x in tr], dtype=np.int32)
        self.t_l = np.array([x["l"] for x in tr], dtype=np.int32)

    # setup.f:433-569 non-bonded types and LJ tables
    def _lj_types(self):
        ns = self.nsites
        sig, eps = self.site_sigma, self.site_eps
        # special 1-4 site parameters (ILJ/SIGAD/EPAD), input.f:1280-1292
        ilj, sigad, epad = [], [], []
        for t, mol in enumerate(self.types):
            for sp in mol["special14"]:
                ilj.append(sp["site"] + self.isadr[t])
                sigad.append(sp["sigma"])
                epad.append(sp["eps"])
        nnad = len(ilj)
        ilip, jlip, sigap, epap = [], [], [], []
        for t, mol in enumerate(self.types):
            for pp in mol.get("par14", []):
                ilip.append(pp["i"] + self.isadr[t]); jlip.append(pp["j"] + self.isadr[t])
                sigap.append(pp["sigma"]); epap.append(pp["eps"])
        if ilip:
            # LPAIRS/NNADP > 0: one LJ type per site (setup.f:441-449); SIGAT
            # takes SIGAD by record number, as the reference does.
            self._lj_tables(list(sig), list(eps),
                            [sigad[i] if i < nnad else 0.0 for i in range(ns)],
                            [epad[i] if i < nnad else 0.0 for i in range(ns)],
                            np.arange(1, ns + 1, dtype=np.int32))
            ef = self.efact
            for k in range(len(ilip)):
                a6 = -4.0 * ef * epap[k] * sigap[k] ** 6
                b12 = 4.0 * ef * epap[k] * sigap[k] ** 12
                i, j = ilip[k] - 1, jlip[k] - 1
                self.a6_14[i, j] = a6; self.b12_14[i, j] = b12
                self.a6_14[j, i] = a6; self.b12_14[j, i] = b12
            return
        inbt = np.zeros(ns, dtype=np.int32)
        sigt, epst, sigat, epsat = [sig[0]], [eps[0]], [], []
        found = False
        for j in range(nnad):
            if ilj[j] == 1:
                sigat.append(sigad[j]); epsat.append(epad[j]); found = True
                break
        if not found:
            sigat.append(sig[0]); epsat.append(eps[0])
        inbt[0] = 1
        nnbt = 1
        its = self.site_type
        for is_ in range(2, ns + 1):
            ityp = its[is_ - 1]
            assigned = False
            for js in range(1, nnbt + 1):
                if abs(sig[is_ - 1] - sigt[js - 1]) < 1e-12 and abs(eps[is_ - 1] - epst[js - 1]) < 1e-12:
                    reject = False
                    if self.iee[ityp - 1] == 0:
                        for j in range(1, is_):
                            if inbt[j - 1] == js and self.iee[its[j - 1] - 1] != 0:
                                reject = True
                                break
                    if not reject and self.iee[ityp - 1] == 1:
                        for j in range(1, is_):
                            if inbt[j - 1] == js and self.iee[its[j - 1] - 1] == 0:
                                reject = True
                                break
                    if reject:
                        break  # goto 183: new type
                    jspec = None
                    for j in range(nnad):
                        if ilj[j] == is_:
                            jspec = j
                            break
                    if jspec is None:
                        if abs(sig[is_ - 1] - sigat[js - 1]) < 1e-12 and abs(eps[is_ - 1] - epsat[js - 1]) < 1e-12:
                            inbt[is_ - 1] = js
                            assigned = True
                        break  # goto 186 or 183
                    else:
                        if abs(sigad[jspec] - sigat[js - 1]) < 1e-12 and abs(epad[jspec] - epsat[js - 1]) < 1e-12:
                            inbt[is_ - 1] = js
                            assigned = True
                            break
                        # else continue the js loop (label 182 falls through)
            if assigned:
                continue
            nnbt += 1
            inbt[is_ - 1] = nnbt
            sigt.append(sig[is_ - 1]); epst.append(eps[is_ - 1])
            jspec = None
            for j in range(nnad):
                if ilj[j] == is_:
                    jspec = j
                    break
            if jspec is not None:
                sigat.append(sigad[jspec]); epsat.append(epad[jspec])
            else:
                sigat.append(sigt[-1]); epsat.append(epst[-1])
        self._lj_tables(sigt, epst, sigat, epsat, inbt)

    def _lj_tables(self, sigt, epst, sigat, epsat, inbt):
        """LJ cross tables A6LJ/B12LJ/A6_14/B12_14 (setup.f:519-543)."""
        ns = self.nsites
        nnbt = len(sigt)
        self.nnbt = nnbt
        self.inbt = np.asarray(inbt, dtype=np.int32)
        ef = self.efact
        epst = [e * ef for e in epst]
        epsat = [e * ef for e in epsat]
        n = nnbt
        self.a6lj = np.zeros((n, n)); self.b12lj = np.zeros((n, n))
        self.a6_14 = np.zeros((n, n)); self.b12_14 = np.zeros((n, n))
        for i in range(n):
            for j in range(n):
                # AM1/AM2 are MASS(IS)/MASS(JS) indexed by type number, as in setup.f:537-538
                am1 = self.site_mass[i] if i < ns else 0.0
                am2 = self.site_mass[j] if j < ns else 0.0
                a6, b12 = comb_rules(sigt[i], sigt[j], epst[i], epst[j], am1, am2, self.spec.icr)
                self.a6lj[i, j] = a6; self.b12lj[i, j] = b12
                a6, b12 = comb_rules(sigat[i], sigat[j], epsat[i], epsat[j], am1, am2, self.spec.icr)
                self.a6_14[i, j] = a6; self.b12_14[i, j] = b12
        self.a6lj0 = self.a6lj.copy()
        self.b12lj0 = self.b12lj.copy()

    # setup.f:283-388 bond/angle/torsion instances (serial: NUMTASK=1)
    def _bonded_instances(self):
        ibi, jbj, ibuk = [], [], []
        iai, jaj, kak, iauk = [], [], [], []
        iti, jtj, ktk, ltl, ituk = [], [], [], [], []
        for t in range(self.ntypes):
            if self.ipot[t] != 0:
                continue
            for i in range(self.nspec[t]):
                iml = self.isaddr[t] + i * self.nsits[t]
                for j in range(self.nrb[t]):
                    is_ = self.iadb[t] - 1 + j
                    ibi.append(self.b_ib[is_] + iml); jbj.append(self.b_jb[is_] + iml); ibuk.append(is_ + 1)
                for j in range(self.nra[t]):
                    is_ = self.iada[t] - 1 + j
                    iai.append(self.a_ia[is_] + iml); jaj.append(self.a_ja[is_] + iml)
                    kak.append(self.a_ka[is_] + iml); iauk.append(is_ + 1)
                for j in range(self.nrt[t]):
                    is_ = self.iadt[t] - 1 + j
                    iti.append(self.t_i[is_] + iml); jtj.append(self.t_j[is_] + iml)
                    ktk.append(self.t_k[is_] + iml); ltl.append(self.t_l[is_] + iml); ituk.append(is_ + 1)
        a32 = lambda v: np.array(v, dtype=np.int32)
        self.ibi, self.jbj, self.ibuk = a32(ibi), a32(jbj), a32(ibuk)
        self.iai, self.jaj, self.kak, self.iauk = a32(iai), a32(jaj), a32(kak), a32(iauk)
        self.iti, self.jtj, self.ktk, self.ltl, self.ituk = a32(iti), a32(jtj), a32(ktk), a32(ltl), a32(ituk)
        self.nrbt, self.nrat, self.nrrt = len(ibi), len(iai), len(iti)

    # setup.f:753-939
    def _bndlst(self):
        n = self.nstot
        lists = [[] for _ in range(n)]

        def bndreg(ibb, jbb, isig):
            if ibb == jbb:
                return
            ityp = self.site_type[ibb - 1]
            nsp = self.nsits[ityp - 1]
            isg = 1 if isig >= 0 else -1
            if ityp != self.site_type[jbb - 1]:
                raise RuntimeError("different types in BNDREG")
            isha = self.isaddr[ityp - 1] - self.isadr[ityp - 1]
            for im in range(1, self.nspec[ityp - 1] + 1):
                ibs = ibb + isha + (im - 1) * nsp
                jbs = jbb + isha + (im - 1) * nsp
                if not any(abs(x) == jbs for x in lists[ibs - 1]):
                    lists[ibs - 1].append(isg * jbs)
                if not any(abs(x) == ibs for x in lists[jbs - 1]):
                    lists[jbs - 1].append(isg * ibs)

        for t in range(self.ntypes):
            nbbeg = self.iadb[t] - 1
            nbend = nbbeg + self.nrb[t]
            isbeg = self.isadr[t] + 1
            isend = self.isadr[t + 1]
            ishf = self.isadr[t]
            IB, JB, ID = self.b_ib, self.b_jb, self.b_id
            for i in range(nbbeg, nbend):
                if ID[i] != 2:
                    bndreg(IB[i] + ishf, JB[i] + ishf, 1)
            for is_ in range(isbeg, isend + 1):
                for j in range(nbbeg, nbend):
                    ibb, jbb = IB[j] + ishf, JB[j] + ishf
                    if is_ == ibb and ID[j] != 2:
                        for k in range(j + 1, nbend):
                            ibk, jbk = IB[k] + ishf, JB[k] + ishf
                            if is_ == ibk and ID[k] != 2:
                                bndreg(jbb, jbk, 1)
                            elif is_ == jbk and ID[k] != 2:
                                bndreg(jbb, ibk, 1)
                    elif is_ == jbb and ID[j] != 2:
                        for k in range(j + 1, nbend):
                            ibk, jbk = IB[k] + ishf, JB[k] + ishf
                            if is_ == ibk and ID[k] != 2:
                                bndreg(ibb, jbk, 1)
                            elif is_ == jbk and ID[k] != 2:
                                bndreg(ibb, ibk, 1)
            for i in range(nbbeg, nbend):
                is_, js = IB[i], JB[i]
                if ID[i] == 2:
                    continue
                for j in range(nbbeg, nbend):
                    if is_ == JB[j] and ID[j] != 2:
                        for k in range(nbbeg, nbend):
                            if js == IB[k] and ID[k] != 2:
                                bndreg(IB[j] + ishf, JB[k] + ishf, -1)
                            elif js == JB[k] and ID[k] != 2:
                                bndreg(IB[j] + ishf, IB[k] + ishf, -1)
                    elif is_ == IB[j] and ID[j] != 2:
                        for k in range(nbbeg, nbend):
                            if js == IB[k] and ID[k] != 2:
                                bndreg(JB[j] + ishf, JB[k] + ishf, -1)
                            elif js == JB[k] and ID[k] != 2:
                                bndreg(JB[j] + ishf, IB[k] + ishf, -1)
        self.nbdmax = max(1, max((len(l) for l in lists), default=1))
        self.nnbb = np.array([len(l) for l in lists], dtype=np.int32)
        # INBB(NTOT, NBDMAX) column-major: element (i,k) at i + k*ld
        self.ld_inbb = n
        inbb = np.zeros((self.nbdmax, n), dtype=np.int32)
        for i, l in enumerate(lists):
            for k, v in enumerate(l):
                inbb[k, i] = v
        self.inbb = inbb  # shape (nbdmax, nstot); flat C order == Fortran column-major

    # main.f:380-450, 729-812 and derived run parameters
    def _params(self):
        sp = self.spec
        cl = min(self.boxl, self.boyl, self.bozl)
        self.alphad = ewald_alpha(sp.alpha, self.rcutt, cl) if sp.alpha > 0 else 0.0
        self.fexp = sp.fexp
        # Electrostatics with ALPHA <= 0: reaction field of dielectric
        # constant DIEL = -ALPHA, FEXP the Debye length (0: no salt), with the
        # molecular cutoff list (LMNBL); DIEL <= 1 is a plain cutoff
        # (main.f:740-793)
        self.lmnbl = sp.alpha <= 0.0
        self.rff = self.rff2 = 0.0
        if self.lmnbl:
            diel = -sp.alpha
            rdeb = sp.fexp
            rck = self.rcutt / rdeb if rdeb > 1e-3 else 0.0
            self.rff2 = -((2.0 * (diel - 1.0) * (rck + 1.0) + diel * rck ** 2)
                          / (((2.0 * diel + 1.0) * (rck + 1.0) + diel * rck ** 2) * self.rcutt ** 3))
            self.rff = (1.0 / (diel * (1.0 + rck)) - 1.0) / self.rcutt
            if diel <= 1.0000001:
                self.rff = self.rff2 = 0.0
        self.lnvt = sp.nvt is not None
        self.lnpt = sp.npt is not None
        self.dqt = (self.unitt * 1e15 / sp.nvt[1]) ** 2 if self.lnvt else 0.0
        if self.lnpt:
            trpres, qpr = sp.npt
            qt = sp.nvt[1]
            self.dqt = (self.unitt * 1e15 / qt) ** 2
            self.dqp = 3.0 * self.unite * self.unitt ** 2 / (
                self.unitp * (self.fnst + 3) * BOLTZ * self.trtemp * (qpr * 1e-15) ** 2)
            self.rtp = (qpr / qt) ** 2 * (self.fnst + 3.0) / self.fnst
            self.trpres = trpres
        else:
            self.dqp = 0.0
            self.rtp = 0.0
            self.trpres = 1.0
        self.epd, self.vird = elrclj(self)

    # --------------------------------------------------------- helpers ---
    def kvector_count(self) -> int:
        return kvector_count(self.alphad, self.fexp, self.boxl, self.boyl, self.bozl,
                             self.spec.icell)

    def kcolumn_counts(self) -> Tuple[int, int, int]:
        return kcolumn_counts(self.alphad, self.fexp, self.boxl, self.boyl, self.bozl)

    def summary(self) -> dict:
        return dict(nstot=self.nstot, nop=self.nop, ntypes=self.ntypes, nnbt=self.nnbt,
                    box=(self.boxl, self.boyl, self.bozl), alphad=self.alphad,
                    nkv=self.kvector_count(), fnst=self.fnst)


def elrclj(s: System) -> Tuple[float, float]:
    """LJ tail corrections EPD and VIRD at the current volume (ELRCLJ,
    forces.f:1684-1746).  Host constants; returned to the driver."""
    pel = np.zeros(NTPP)
    vrl = np.zeros(NTPP)
    rc0 = math.sqrt(s.rssq)
    for it in range(s.ntypes):
        for is_ in range(s.isadr[it] + 1, s.isadr[it + 1] + 1):
            ist = s.inbt[is_ - 1] - 1
            for jt in range(it, s.ntypes):
                rc = rc0 + (0.0 if s.iee[it] * s.iee[jt] != 0 else 0.0)
                mt = s.mdx[it, jt]
                fnopij = float(s.nspec[it] * s.nspec[jt])
                if it == jt:
                    fnopij = 0.5 * fnopij
                for js in range(s.isadr[jt] + 1, s.isadr[jt + 1] + 1):
                    jst = s.inbt[js - 1] - 1
                    b12 = s.b12lj[ist, jst]
                    a6 = s.a6lj[ist, jst]
                    if b12 > 1e-50 and a6 < -1e-50:
                        ep = a6 ** 2 / b12
                        si3 = math.sqrt(-b12 / a6)
                        x = si3 / rc ** 3
                        pel[mt - 1] += ep * si3 * ((1.0 / 9.0) * x ** 3 - (1.0 / 3.0) * x) * fnopij
                        vrl[mt - 1] += ep * si3 * ((-4.0 / 3.0) * x ** 3 + 2.0 * x) * fnopij
    epd = 0.0
    vird = 0.0
    for i in range(s.molint):
        epd += 4.0 * PI * pel[i] / s.vol
        vird += -4.0 * PI * vrl[i] / s.vol
    return epd, vird


# ------------------------------------------------------- configuration ----
def _random_rotation(rng: np.random.Generator) -> np.ndarray:
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    a, b, c, d = q
    return np.array([
        [a * a + b * b - c * c - d * d, 2 * (b * c - a * d), 2 * (b * d + a * c)],
        [2 * (b * c + a * d), a * a - b * b + c * c - d * d, 2 * (c * d - a * b)],
        [2 * (b * d - a * c), 2 * (c * d + a * b), a * a - b * b - c * c + d * d]])


def _lattice_with_room(rng, nside: int, nop: int, big: List[int]) -> np.ndarray:
    """Lattice cell per molecule, leaving the neighbour cells of molecules
    with more than three sites empty as far as the spare cells allow (first
    the 6 face neighbours of every such molecule, then the other 20), so a
    solute does not start inside its neighbours."""
    ncell = nside ** 3
    spare = ncell - nop
    order = rng.permutation(ncell)
    taken = np.zeros(ncell, dtype=bool)
    blocked = np.zeros(ncell, dtype=bool)
    cell_of = np.full(nop, -1, dtype=np.int64)

    def idx(i, j, k):
        return ((i % nside) * nside + (j % nside)) * nside + (k % nside)

    faces = [(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)]
    rest = [(a, b, c) for a in (-1, 0, 1) for b in (-1, 0, 1) for c in (-1, 0, 1)
            if (a, b, c) != (0, 0, 0) and (a, b, c) not in faces]
    pos = 0
    for m in big:
        while taken[order[pos]] or blocked[order[pos]]:
            pos += 1
        c = order[pos]
        taken[c] = True
        cell_of[m] = c
    for shell in (faces, rest):
        for m in big:
            c = cell_of[m]
            i, j, k = c // (nside * nside), (c // nside) % nside, c % nside
            for d in shell:
                nb = idx(i + d[0], j + d[1], k + d[2])
                if not taken[nb] and not blocked[nb] and blocked.sum() < spare:
                    blocked[nb] = True
    free = [c for c in order if not taken[c] and not blocked[c]]
    others = [m for m in range(nop) if cell_of[m] < 0]
    cell_of[others] = free[:len(others)]
    return cell_of


def _cell_lattice(s: System, rng):
    """Molecular centres for the non-rectangular cells: a point set that the
    cell's lattice maps onto itself, one point of each lattice class (each
    brought into the cell by the cell's minimum image), in random order,
    shifted off the cell's faces.  Truncated octahedron (ICELL 1): a
    body-centred grid of the cube, n^3 classes, nearest points sqrt(3)/2 of
    the grid spacing apart (n even: the half-diagonal (L/2)(1, 1, 1) is a
    grid vector).  Hexagonal (ICELL 2): the grid of the L x L cos30 x Lz
    rectangle with an even count along x (the lattice vector
    (L/2, L cos30, 0) is then a grid vector)."""
    nop = s.nop
    box = np.array([s.boxl, s.boyl, s.bozl])
    if s.spec.icell == 1:
        L = s.boxl
        n = 2
        while n ** 3 < nop:
            n += 2
        a = L / n
        g = np.arange(n) * a - 0.5 * L
        cube = np.array([(x, y, z) for x in g for y in g for z in g])
        pts = np.concatenate([cube, cube + 0.5 * a]) + np.array([0.11, 0.23, 0.37]) * a
        pts = pts - L * np.round(pts / L)  # cube wrap, then the octahedral fold
        corss = 0.5 * L * np.floor((4.0 / 3.0) * np.abs(pts).sum(axis=1) / L)
        pts = pts - np.sign(pts) * corss[:, None]
        key = np.round(pts / (1e-6 * L)).astype(np.int64)
        _, first = np.unique(key, axis=0, return_index=True)
        pts = pts[np.sort(first)]
        a = np.full(3, a)
    else:
        # the counts with the largest smallest spacing that hold nop points
        best = None
        for nx in range(2, 2 * int(s.boxl) + 3, 2):
            for ny in range(1, int(s.boyl) + 2):
                nz = max(1, -(-nop // (nx * ny)))
                gap = min(s.boxl / nx, s.boyl / ny, s.bozl / nz)
                if best is None or gap > best[0]:
                    best = (gap, nx, ny, nz)
        _, nx, ny, nz = best
        a = box / np.array([nx, ny, nz])
        pts = np.array([((i + 0.5) * a[0], (j + 0.5) * a[1], (k + 0.5) * a[2])
                        for i in range(nx) for j in range(ny) for k in range(nz)]) - 0.5 * box
    if len(pts) < nop:
        raise ValueError("cell lattice too small")
    return pts[rng.permutation(len(pts))[:nop]], a


def make_configuration(s: System, seed: int = 1, jitter: float = 0.3,
                       order: Optional[np.ndarray] = None):
    """Seeded start: molecular centres on a jittered simple-cubic lattice
    spanning the box (centred on 0, as after GETCOM's PBC, service.f:537),
    random orientations, Maxwell momenta rescaled to TRTEMP with the
    reference's formula (main.f:689-714).  Returns sx, sy, sz, vx, vy, vz."""
    rng = np.random.default_rng(seed)
    nop = s.nop
    box = np.array([s.boxl, s.boyl, s.bozl])
    if s.spec.icell != 0:
        com, a = _cell_lattice(s, rng)
    else:
        nside = int(math.ceil(nop ** (1.0 / 3.0) - 1e-9))
        cells = np.array([(i, j, k) for i in range(nside) for j in range(nside)
                          for k in range(nside)], dtype=np.float64)
        mtype = np.repeat(np.arange(s.ntypes), s.nspec[:s.ntypes])
        big = [int(m) for m in np.nonzero(s.nsits[mtype] > 3)[0]]
        if big and len(cells) > nop:
            cells = cells[_lattice_with_room(rng, nside, nop, big)]
        else:
            perm = rng.permutation(len(cells))[:nop]
            cells = cells[perm]
        a = box / nside
        com = (cells + 0.5) * a - 0.5 * box
    com += rng.uniform(-jitter, jitter, size=com.shape) * a
    sx = np.zeros(s.nstot); sy = np.zeros(s.nstot); sz = np.zeros(s.nstot)
    n = 0
    imol = 0
    for t in range(s.ntypes):
        r = np.array(s.types[t]["r"])
        for _ in range(s.nspec[t]):
            rot = _random_rotation(rng)
            pos = r @ rot.T + com[imol]
            for i in range(s.nsits[t]):
                sx[n], sy[n], sz[n] = pos[i]
                n += 1
            imol += 1
    # momenta: COMVEL (service.f:128-157) then rescale (main.f:689-714)
    m = s.site_mass[s.nsite - 1]
    rt = np.sqrt(200.0 * m / s.trtemp)
    g = rng.normal(size=(3, s.nstot))
    vx, vy, vz = rt * g[0], rt * g[1], rt * g[2]
    vx -= vx.sum() / s.nstot; vy -= vy.sum() / s.nstot; vz -= vz.sum() / s.nstot
    lm = s.lmove[s.itype - 1].astype(bool)
    vsq = float(np.sum(((vx ** 2 + vy ** 2 + vz ** 2) * s.massdi)[lm]))
    temp = 1.50 * vsq * s.enerf * s.tempf / s.fnst
    ftmp = math.sqrt(s.trtemp / temp)
    vx = np.where(lm, vx * ftmp, 0.0); vy = np.where(lm, vy * ftmp, 0.0); vz = np.where(lm, vz * ftmp, 0.0)
    return sx, sy, sz, vx, vy, vz


# ------------------------------------------------------- named workloads --
def spce_nacl_nve(nwater: int = 512, nion: int = 4, steps_shake: bool = True) -> RunSpec:
    """Rigid SPC/E water + Na+/Cl-, SHAKE, NVE, Rcut 10, Ewald A=2.8 (alpha
    0.28/A), |n|<=7 per axis: the 1544-atom plain-method case."""
    L = None
    spec = RunSpec(molecules=[("SPC_E", nwater), ("Na+", nion), ("Cl-", nion)],
                   density=1.0, dt_fs=2.0, nfreq=1, rcut=10.0, rshort=5.0,
                   alpha=2.8, fexp=9.84, ichnb=10, shake=steps_shake, toler=1e-8,
                   nvt=None, trtemp=300.0)
    return spec


def spcfw_water(nwater: int = 32768, nmax: int = 20, alpha_per_a: float = 0.25,
                rcut: float = 12.0, steps_nfreq: int = 10) -> RunSpec:
    """Flexible SPC-FW water, double time step 0.2/2 fs, NVT 300 K, Rcut 12,
    Ewald alpha 0.25/A with |n|<=nmax per axis inside INIFUR's sphere."""
    # box at 1.0 g/cm3 fixes L; B = (2 pi nmax / L)^2 / (4 alpha^2)
    mw = 15.9994 + 2 * 1.008
    vol = nwater * mw / (AVSNO * 1000.0) / (1.0 * 1000.0) * 1e30
    L = vol ** (1.0 / 3.0)
    fexp = (2 * PI * nmax / L) ** 2 / (4 * alpha_per_a ** 2)
    fexp = float(math.ceil(fexp * 100.0) / 100.0)
    return RunSpec(molecules=[("SPC-FW", nwater)], density=1.0, dt_fs=2.0,
                   nfreq=steps_nfreq, rcut=rcut, rshort=5.0,
                   alpha=alpha_per_a * rcut, fexp=fexp, ichnb=10, shake=False,
                   nvt=(300.0, 30.0), trtemp=300.0)


def nacl_sample(box=None) -> RunSpec:
    """The reference's own example, sample/4nacl.in: 256 flexible SPC
    waters (H2O, fSPC) + 4 Na+_SD + 4 Cl-_SD at 1.02 g/cm3, double time step
    0.2/2 fs, Nose-Hoover 298 K / 30 fs, R_cutoff 10, R_short 5, Ewald A = 3,
    B = 9, Neighbour_list 10, Cut_forces 1.  ``box``: the box of a restart
    file (the reference takes BOXL.. from the restart, restart.f:167)."""
    return RunSpec(molecules=[("H2O", 256), ("Na+_SD", 4), ("Cl-_SD", 4)], density=1.02,
                   box=None if box is None else tuple(float(x) for x in box), dt_fs=2.0,
                   nfreq=10, rcut=10.0, rshort=5.0, alpha=3.0, fexp=9.0, ichnb=10,
                   nvt=(298.0, 30.0), trtemp=298.0, cut_forces=1.0)


def lrc_per_pair(s: System):
    """PELRC and VRLRC per molecule-type pair (ELRCLJ, forces.f:1684-1736),
    at the current volume, indexed by MDX - 1."""
    pel = np.zeros(NTPP)
    vrl = np.zeros(NTPP)
    rc = math.sqrt(s.rssq)
    for it in range(s.ntypes):
        for is_ in range(s.isadr[it] + 1, s.isadr[it + 1] + 1):
            ist = s.inbt[is_ - 1] - 1
            for jt in range(it, s.ntypes):
                mt = s.mdx[it, jt]
                f = float(s.nspec[it] * s.nspec[jt])
                if it == jt:
                    f = 0.5 * f
                for js in range(s.isadr[jt] + 1, s.isadr[jt + 1] + 1):
                    jst = s.inbt[js - 1] - 1
                    b12, a6 = s.b12lj[ist, jst], s.a6lj[ist, jst]
                    if b12 > 1e-50 and a6 < -1e-50:
                        ep = a6 ** 2 / b12
                        si3 = math.sqrt(-b12 / a6)
                        x = si3 / rc ** 3
                        pel[mt - 1] += ep * si3 * ((1.0 / 9.0) * x ** 3 - (1.0 / 3.0) * x) * f
                        vrl[mt - 1] += ep * si3 * ((-4.0 / 3.0) * x ** 3 + 2.0 * x) * f
    return 4.0 * PI * pel / s.vol, -4.0 * PI * vrl / s.vol


SOLUTES = ("CH3OH", "C2H5OH", "CH3CN", "dmso", "Li+", "Na+", "Cl-")


def solvation_job(solute: str, nwater: int, rcut: float = 9.0) -> RunSpec:
    """One solute (the expanded-ensemble type, EE_type 1) in flexible SPC
    water (H2O, fSPC) at 1.0 g/cm3: Rcut 9, Ewald A = 2.8, B = 9 (input.f
    defaults), double time step 0.2/2 fs, Nose-Hoover 298 K / 30 fs."""
    return RunSpec(molecules=[(solute, 1), ("H2O", nwater)], density=1.0, dt_fs=2.0,
                   nfreq=10, rcut=rcut, rshort=5.0, alpha=2.8, fexp=9.0, ichnb=10,
                   nvt=(298.0, 30.0), trtemp=298.0, iee_type=1)


def pimd_params(s: System):
    """BEADFAC, CONVEQ (setup.f:696-700), DQQT, FNH (main.f:413-415) of a
    spec with nbeads > 1 and pi_thermo = (BTAU fs, JNH)."""
    from .abi import MdxPimdParams
    sp = s.spec
    P = sp.nbeads
    btau, jnh = sp.pi_thermo
    beadfac = 0.5e-3 * P * (BOLTZ * sp.trtemp / HPLANK) ** 2 * s.unitl ** 2 / (s.unite * AVSNO)
    dqqt = (s.unitt * 1.0e15 / btau) ** 2
    return MdxPimdParams(nbeads=P, jnh=int(jnh), beadfac=beadfac,
                         conveq=s.enerf * s.tempf / P, dqqt=dqqt, fnh=dqqt / (3.0 * P))


def pimd_beads(s: System, seed: int = 1, sigma_h: float = 0.1):
    """Bead starts: the classical start of make_configuration, each bead
    displaced by a seeded Gaussian of width sigma_h * sqrt(m_H / m) A per
    axis, with its own Maxwell momenta (bead masses) at TRTEMP."""
    P = s.spec.nbeads
    base = make_configuration(s, seed=seed, jitter=0.05)
    rng = np.random.default_rng(seed + 7777)
    m = s.site_mass[s.nsite - 1]
    sig = sigma_h * np.sqrt(1.008 / m)
    states = []
    for b in range(P):
        mom = make_configuration(s, seed=seed + 1 + b, jitter=0.05)[3:]
        d = rng.normal(size=(3, s.nstot)) * sig
        states.append((base[0] + d[0], base[1] + d[1], base[2] + d[2]) + tuple(mom))
    return states


def pimd_water(nwater: int = 256, nbeads: int = 32) -> RunSpec:
    """Flexible SPC-FW water as bead replicas: 300 K, Rcut 9, Ewald A 3.15,
    B 13.27 (alpha 0.35/A, |n| <= 8), dt 0.25 fs without double time step,
    PI_thermo 300 K, 5 fs, chains of 4."""
    return RunSpec(molecules=[("SPC-FW", nwater)], density=1.0, dt_fs=0.25, nfreq=1,
                   rcut=9.0, rshort=5.0, alpha=3.15, fexp=13.27, ichnb=10, nvt=None,
                   trtemp=300.0, nbeads=nbeads, pi_thermo=(5.0, 4))


def dmpc_bilayer(nside: int = 7, nwater: int = 3655, box=(62.0, 62.0, 76.0),
                 rcut: float = 12.0, alpha: float = 3.12, fexp: float = 9.72,
                 shake_hbonds: bool = False) -> RunSpec:
    """DMPC bilayer (2 x nside^2 lipids, tails along z) in SPC water.  The
    all-atom, fully extended dmpc.mmol conformation needs 76 A of box height
    to leave room for 3655 waters at 1.0 g/cm3, and packs without overlaps
    (every intermolecular distance >= 1.5 A) at 7 x 7 lipids per leaflet in
    62 x 62 A; 8 x 8 would start with atoms 0.9 A apart.  Then
    anisotropic Nose-Hoover NPT at 303 K / 1 bar, SHAKE on every constrained
    bond (the reference's per-type rule: ID != 2; with shake_hbonds only
    the bonds to hydrogen), dt 2 fs, Ewald A, B."""
    return RunSpec(molecules=[("dmpc", 2 * nside * nside), ("SPC", nwater)], box=tuple(box),
                   dt_fs=2.0, nfreq=1, rcut=rcut, rshort=5.0, alpha=alpha, fexp=fexp,
                   ichnb=10, shake=True, toler=1e-5, nvt=(303.0, 50.0), npt=(1.0, 1000.0),
                   anisotropic=True, trtemp=303.0, shake_hbonds=shake_hbonds)


def bilayer_configuration(s: System, seed: int = 1, clearance: float = 2.3,
                          tilt_gap: float = 0.5):
    """Seeded bilayer start: lipids on an nside x nside grid per leaflet with
    their long axis along z (upper leaflet head up, lower leaflet head down
    and shifted by half a grid cell), each rotated about z by the sampled
    angle that keeps it farthest from the lipids already placed, tail tips
    ``tilt_gap`` from z = 0 (interdigitated when negative); waters on a
    cubic lattice at 1.0 g/cm3 spacing, keeping the sites farthest from the
    bilayer centre that are at least ``clearance`` from every lipid atom.
    Momenta as make_configuration.  Molecule types: lipid first, water
    second."""
    from scipy.spatial import cKDTree
    rng = np.random.default_rng(seed)
    box = np.array([s.boxl, s.boyl, s.bozl])
    nlip, nw = int(s.nspec[0]), int(s.nspec[1])
    nside = int(round(math.sqrt(nlip / 2)))
    r = np.array(s.types[0]["r"])
    r = r - r.mean(axis=0)
    tail = r[:, 2].min()
    a = box[:2] / nside
    angles = np.linspace(0.0, 2 * math.pi, 24, endpoint=False)

    def wrap(x):  # into [0, box) for the periodic tree
        return np.mod(x + 0.5 * box, box)

    pos = []
    for leaf in (1, -1):
        for ix in range(nside):
            for iy in range(nside):
                zc = leaf * (-tail + tilt_gap)
                sh = 0.5 if leaf < 0 else 0.0
                ctr = np.array([(ix + 0.5 + sh) * a[0] - 0.5 * box[0],
                                (iy + 0.5 + sh) * a[1] - 0.5 * box[1], zc])
                tree = cKDTree(wrap(np.concatenate(pos)), boxsize=box) if pos else None
                best, best_d = None, -1.0
                phase = rng.uniform(0, 2 * math.pi)
                for th in angles + phase:
                    c, sn = math.cos(th), math.sin(th)
                    x = r @ np.array([[c, -sn, 0], [sn, c, 0], [0, 0, 1]]).T
                    if leaf < 0:
                        x = x * np.array([1, -1, -1])    # 180 degrees about x
                    x = x + ctr
                    if tree is None:
                        best = x
                        break
                    m = float(tree.query(wrap(x), k=1)[0].min())
                    if m > best_d:
                        best, best_d = x, m
                pos.append(best)
    lip = np.concatenate(pos, axis=0)
    sp = (18.015 / AVSNO * 1e24) ** (1.0 / 3.0)
    n = np.maximum(1, np.floor(box / sp).astype(int))
    g = np.stack(np.meshgrid(*[(np.arange(k) + 0.5) * box[d] / k - 0.5 * box[d]
                               for d, k in enumerate(n)], indexing="ij"), -1).reshape(-1, 3)
    dist = cKDTree(wrap(lip), boxsize=box).query(wrap(g), k=1)[0]
    g = g[dist >= clearance]
    g = g[np.argsort(-np.abs(g[:, 2]), kind="stable")][:nw]
    if len(g) < nw:
        raise ValueError(f"only {len(g)} water sites clear of the bilayer; need {nw}")
    rw = np.array(s.types[1]["r"])
    rw = rw - rw.mean(axis=0)
    wat = [rw @ _random_rotation(rng).T + g[k] for k in range(nw)]
    xyz = np.concatenate([lip] + wat, axis=0)
    mom = make_configuration(s, seed=seed + 1, jitter=0.05)[3:]
    return (xyz[:, 0].copy(), xyz[:, 1].copy(), xyz[:, 2].copy()) + tuple(mom)
