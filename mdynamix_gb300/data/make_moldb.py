"""Regenerate moldb.json from an MDynaMix ``moldb`` directory.

Usage:  python make_moldb.py <moldb-dir> [out.json]

Parses each topology this package uses with ``system.parse_mmol`` (the
READMOL restatement) and stores the parsed records, so that the package
runs where the original ``.mmol`` files are not present.
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from mdynamix_gb300.system import parse_mmol  # noqa: E402

MOLECULES = ["SPC_E", "SPC-FW", "SPC", "H2O", "Na+", "Cl-", "Li+", "CH3OH",
             "C2H5OH", "CH3CN", "dmso", "dmpc", "Na+_SD", "Cl-_SD"]


def main(argv):
    src = argv[1]
    out = argv[2] if len(argv) > 2 else os.path.join(HERE, "moldb.json")
    db = {}
    for name in MOLECULES:
        path = os.path.join(src, name + ".mmol")
        with open(path, encoding="latin-1") as fh:
            db[name] = parse_mmol(fh.read(), name)
    with open(out, "w") as fh:
        json.dump(db, fh, indent=0, sort_keys=True)
    print("wrote", out, "with", len(db), "molecules")


if __name__ == "__main__":
    main(sys.argv)
