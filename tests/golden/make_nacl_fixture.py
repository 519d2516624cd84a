"""Generates the fixtures of the reference's own sample run (run here, where
the reference tree is; the GPU tests read only the generated files).

The reference ships one complete example: sample/4nacl.in (256 flexible SPC
waters + 4 Na+_SD + 4 Cl-_SD, 776 atoms), the restart file its run left,
sample/NaCl.dmp (written by RESTRT, restart.f:390-420, in the v5.0 layout),
and the run's printed output, sample/4nacl.out.

Writes
  nacl776_state.npz       positions (A) and momenta (the reference's VX) of
                          NaCl.dmp, its box and time step, read with
                          mdynamix_gb300.restart.read_dmp
  nacl776_reference.json  numbers 4nacl.out prints that depend only on the
                          input (box, k-vector count, degrees of freedom,
                          long-range corrections) and the run's final
                          averages with their error bars

Usage: python tests/golden/make_nacl_fixture.py [reference tree]
"""
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from mdynamix_gb300.restart import read_dmp  # noqa: E402


def _num(s):
    return float(s.replace("D", "E").replace("d", "e"))


def parse_out(text):
    ref = {}
    g = lambda pat: re.search(pat, text, re.M)  # noqa: E731
    ref["nstot"] = int(g(r"NR OF SITES/TOT \(NSTOT\)\s+(\d+)").group(1))
    ref["nop"] = int(g(r"NR OF PARTICLES \(NOP\)\s+(\d+)").group(1))
    ref["fnst"] = float(g(r"NR of DEGREES of FREEDOM\s+([\d.]+)").group(1))
    ref["fttr"] = float(g(r"translationalnal:\s+([\d.]+)").group(1))
    ref["fnstr"] = float(g(r"rotational:\s+([\d.]+)").group(1))
    ref["fnsti"] = float(g(r"internal:\s+([\d.]+)").group(1))
    ref["pe_lrc_kj_mol"] = float(g(r"PE  LRC  1:\s+(\S+) kJ/mol").group(1))
    ref["pr_lrc_atm"] = float(g(r"PR  LRC  1:\s+(\S+) atm").group(1))
    ref["box"] = [_num(x) for x in g(r"BOX LENGTHS\s+(\S+) A\s+(\S+) A\s+(\S+) A").groups()]
    ref["volume"] = _num(g(r"BOX VOLUME\s+(\S+) A").group(1))
    ref["nkv"] = int(g(r"Num. of k-vectors\s+(\d+)").group(1))
    # final averages (after "FINAL AVERAGE QUANTITIES")
    fin = text[text.index("FINAL AVERAGE QUANTITIES"):]
    bonds = []
    for m in re.finditer(r"^(\S+(?: \d)?)\s*-\s*(\S+(?: \d)?)\s+([\d.]+)\+/-\s+([\d.]+)\s+"
                         r"([\d.]+)\+/-\s+([\d.]+)",
                         fin[:fin.index("Total bond energy")], re.M):
        bonds.append({"pair": f"{m.group(1).replace(' ', '')}-{m.group(2).replace(' ', '')}",
                      "r": float(m.group(3)), "r_err": float(m.group(4)),
                      "e": float(m.group(5)), "e_err": float(m.group(6))})
    ref["bonds_h2o"] = bonds
    ref["bond_energy_h2o"] = float(re.search(r"Total bond energy for H2O\s+(\S+)", fin).group(1))
    inter = {}
    for m in re.finditer(r"INTERMOLECULAR ENERGIES: (\S+)\s+- (\S+)\s+\*\*\*\s*\n"
                         r"\s+Electrostatic\s+:\s+(\S+) kj/mol\s+\+/-\s+(\S+)\s*\n"
                         r"\s+Lennard-Jones\s+:\s+(\S+) kj/mol\s+\+/-\s+(\S+)\s*\n"
                         r"\s+Out cutoff corr:\s+(\S+)", fin):
        inter[f"{m.group(1)}-{m.group(2)}"] = {
            "el": float(m.group(3)), "el_err": float(m.group(4)),
            "lj": float(m.group(5)), "lj_err": float(m.group(6)), "lrc": float(m.group(7))}
    ref["inter"] = inter
    th = fin[fin.index("FINAL thermodynamics properties"):]
    def av(label):
        m = re.search(re.escape(label) + r"\s*:?\s+(\S+)\s+\S+\s+\+/-\s+(\S+)", th)
        return {"v": float(m.group(1)), "err": float(m.group(2))}
    ref["final"] = {k: av(lab) for k, lab in (
        ("temp", "TEMP    "), ("ep_nonbond", "EPnon-bd"), ("ep_bonded", "EPbonded"),
        ("ep_total", "EPtotal "), ("p_atomic", "PRES(At)"), ("p_molecular", "PRES(Ml)"),
        ("temp_h2o", "Temp (H2O   )"))}
    hist = []
    blk = fin[fin.index("History of global thermodynamic properties"):]
    for m in re.finditer(r"^\s*(\d+)\s+([\d.]+)\s+(\d+)\.\s+([\d.]+)\s+(\S+)\s+(\S+)\s+(\S+)"
                         r"\s+(\S+)\s+(\S+)\s*$", blk[:blk.index("Pressure - Density")], re.M):
        hist.append({"block": int(m.group(1)), "t_ps": float(m.group(2)),
                     "temp": float(m.group(4)), "ep_nonbond": float(m.group(5)),
                     "ep_intra": float(m.group(6)), "ep_total": float(m.group(7)),
                     "p_atomic": float(m.group(8)), "p_molecular": float(m.group(9))})
    ref["history"] = hist
    ref["source"] = "sample/4nacl.out (MDYN_v5.0, 18.02.06), sample/4nacl.in"
    return ref


def main(tree):
    sample = os.path.join(tree, "sample")
    r = read_dmp(os.path.join(sample, "NaCl.dmp"))
    np.savez(os.path.join(HERE, "nacl776_state.npz"), sx=r.sx, sy=r.sy, sz=r.sz, vx=r.vx,
             vy=r.vy, vz=r.vz, box=np.array([r.boxl, r.boyl, r.bozl]), dt=r.dt,
             sc=r.sc, nsttot=r.nsttot, tim=r.tim, label=r.label)
    with open(os.path.join(sample, "4nacl.out"), encoding="latin-1") as f:
        ref = parse_out(f.read())
    ref["dmp"] = {"label": r.label, "nop": r.nop, "ntypes": r.ntypes, "nstot": r.nstot,
                  "nnav": r.nnav, "dt": r.dt, "nstep": r.nstep, "nsttot": r.nsttot,
                  "tim": r.tim, "box": [r.boxl, r.boyl, r.bozl], "sc": r.sc}
    with open(os.path.join(HERE, "nacl776_reference.json"), "w") as f:
        json.dump(ref, f, indent=1)
    print(f"wrote nacl776_state.npz ({r.nstot} atoms) and nacl776_reference.json")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
