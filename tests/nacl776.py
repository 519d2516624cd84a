"""The reference's sample run (sample/4nacl.in, its restart file NaCl.dmp
and the averages its output 4nacl.out prints) as fixtures, and the
continuation run whose averages are compared with the printed ones.  No
oracle here: the benchmark's evidence leg imports this module too."""
import json
import math
import os

import numpy as np

from mdynamix_gb300 import system as S
from mdynamix_gb300.abi import thermo_init

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
REF = json.load(open(os.path.join(GOLD, "nacl776_reference.json")))


def load_sample():
    """System, state (positions, momenta) and thermostat state of NaCl.dmp."""
    z = np.load(os.path.join(GOLD, "nacl776_state.npz"))
    s = S.System(S.nacl_sample(box=z["box"]))
    st = tuple(z[k].copy() for k in ("sx", "sy", "sz", "vx", "vy", "vz"))
    th = thermo_init(s)
    th.sc = float(z["sc"])
    return s, st, th


def sample_run_averages(precision, nequil=2000, nrun=10000, nblock=10):
    """Continue the reference's run from its restart file: nequil long steps,
    then nrun long steps averaged in nblock blocks (GETAVR's quantities,
    aver.f:157-176: TEMP, PE TOKJ/NOP, PINT PERMOL, TRYCK, TRYCKM; the bond
    statistics BR, BE TOKJ from the device sums).  Returns {name: (mean,
    standard error of the block means)}."""
    from mdynamix_gb300.mdx import ForcePath
    s, st, th = load_sample()
    g = ForcePath(s, precision=precision)
    g.set_state(*st, thermo=th)
    g.double(nequil, nsttot=10000, records=False)
    g.set_averaging(True)
    g.bonded_sums(clear=True)
    epd, _ = S.elrclj(s)
    tokj = s.enerf * 1e-3
    per = nrun // nblock
    blocks = {k: [] for k in ("temp", "ep_nonbond", "ep_bonded", "p_atomic", "p_molecular",
                              "r_oh", "r_hh", "e_bond")}
    for b in range(nblock):
        rec = g.double_steps(per, 10000 + nequil + b * per)
        pe = np.array([r.pe1 + r.pe2 + r.pels1 + r.pels2 + r.spe + epd for r in rec])
        blocks["temp"].append(np.mean([r.temp for r in rec]))
        blocks["ep_nonbond"].append(np.mean(pe) * s.permol)
        blocks["ep_bonded"].append(np.mean([r.pint for r in rec]) * s.permol)
        blocks["p_atomic"].append(np.mean([r.tryck for r in rec]))
        blocks["p_molecular"].append(np.mean([r.tryckm for r in rec]))
        n, sums, _ = g.bonded_sums(clear=True)
        br, be = sums["br"] / n, sums["be"] / n * tokj
        blocks["r_oh"].append(0.5 * (br[0] + br[1]))
        blocks["r_hh"].append(br[2])
        blocks["e_bond"].append(be[:3].sum())
    g.close()
    return {k: (float(np.mean(v)), float(np.std(v, ddof=1) / math.sqrt(len(v))))
            for k, v in blocks.items()}


def reference_averages():
    """The reference run's averages the continuation is compared with.

    4nacl.out's final averages cover 4-24 ps of a run that started from an
    FCC lattice with cold internal modes; its history shows the internal
    temperature rising until about 18 ps (198 K in the 4-6 ps block, 285-296
    K from 16 ps on) and the intramolecular energy with it.  So the
    thermodynamic averages are taken from its blocks after 16 ps (9-12,
    16-24 ps; the spread of the block means over the root of their number as
    the error), the bond statistics, which it prints only as 4-24 ps
    averages, from the final table."""
    f, b = REF["final"], {x["pair"]: x for x in REF["bonds_h2o"]}
    late = [h for h in REF["history"] if h["t_ps"] > 16.0]

    def blk(key):
        v = np.array([h[key] for h in late])
        return float(v.mean()), float(v.std(ddof=1) / math.sqrt(len(v)))
    return {"temp": blk("temp"), "ep_nonbond": blk("ep_nonbond"),
            "ep_bonded": blk("ep_intra"), "p_atomic": blk("p_atomic"),
            "p_molecular": blk("p_molecular"),
            "r_oh": (0.5 * (b["O-H1"]["r"] + b["O-H2"]["r"]),
                     max(b["O-H1"]["r_err"], b["O-H2"]["r_err"])),
            "r_hh": (b["H1-H2"]["r"], b["H1-H2"]["r_err"]),
            "e_bond": (REF["bond_energy_h2o"],
                       math.sqrt(sum(x["e_err"] ** 2 for x in REF["bonds_h2o"])))}


# Agreement bars of the continuation: statistical (a few combined standard
# errors) where the quantity equilibrates within the run, and an absolute
# bar where the reference's own average still drifts (intramolecular terms:
# its 4-24 ps bond statistics include the cold-internal-mode period) or
# depends on slow ion-pair rearrangements (non-bonded energy).
AGREE = {"temp": ("sigma", 4.0), "p_atomic": ("sigma", 4.0), "p_molecular": ("sigma", 4.0),
         "ep_nonbond": ("abs", 1.5), "ep_bonded": ("abs", 0.6), "e_bond": ("abs", 1.0),
         "r_oh": ("abs", 0.003), "r_hh": ("abs", 0.004)}


def agrees(key, ours, ref):
    (v, e), (rv, re_) = ours, ref
    kind, bar = AGREE[key]
    return abs(v - rv) <= (bar * math.hypot(e, re_) if kind == "sigma" else bar)
