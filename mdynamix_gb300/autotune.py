"""Tuning of the mixed pair sweeps' work split (threads per owner atom).

For a set of water systems spanning the sizes this library serves (PIMD
beads of 768 atoms, solvation jobs of 1-6 k atoms, the 98,304-atom box) and
the cutoffs they use, each split of the short sweep (2, 4, 8 threads per
owner) and of the long sweep (4, 8, 16, 32) is timed on the GPU with the
library's device timers over DOUBLE long steps, and the fastest is kept.
The result is written as ``csrc/tune_table.cuh`` (compiled into the
library, so a context's choice depends on its sizes alone and equal systems
always run the same split) and as a Markdown record of the timings.

Usage (on a GPU): python -m mdynamix_gb300.autotune OUT_DIR [--quick]
then copy OUT_DIR/tune_table.cuh to mdynamix_gb300/csrc/ and rebuild.
"""
from __future__ import annotations

import argparse
import math
import os
import time
from typing import List, Tuple

import numpy as np

from . import system as S
from .abi import MDX_MIXED
from .mdx import ForcePath

SHORT_SPLITS = (2, 4, 8)
LONG_SPLITS = (4, 8, 16, 32)
# (waters, cutoff A): beads and small jobs at 9 A, the named water box at 12 A
SYSTEMS = ((256, 9.0), (700, 9.0), (2000, 9.0), (2000, 12.0), (8000, 9.0), (8000, 12.0),
           (32768, 12.0))


def mean_rows(path: ForcePath) -> Tuple[float, float]:
    """The library's estimate of the mean full-row lengths (short, long):
    rho (4/3) pi r^3 with the list radius RCUT + skin."""
    s = path.system
    rho = s.nstot / (s.boxl * s.boyl * s.bozl)
    c = 4.0 / 3.0 * math.pi
    rs, rl = s.spec.rshort, s.rcutt + s.spec.rskin
    return rho * c * rs ** 3, rho * c * (rl ** 3 - rs ** 3)


def time_split(g: ForcePath, ts: int, tl: int, steps: int, mstep: int, reps: int = 2):
    """Best of ``reps`` per-long-step device times (ms) of the short and long
    sweeps with this split."""
    g.set_tuning(ts, tl)
    g.double_steps(1, mstep, records=False)  # capture the graphs of this split
    best_s = best_l = float("inf")
    for r in range(reps):
        g.set_timers(True)
        g.timers()
        g.double_steps(steps, mstep + 1 + r * steps, records=False)
        tm = g.timers()
        g.set_timers(False)
        best_s = min(best_s, tm["pair_short"][0] / steps)
        best_l = min(best_l, tm["pair_long"][0] / steps)
    return best_s, best_l


def measure(nwater: int, rcut: float, steps: int):
    spec = S.spcfw_water(nwater=nwater, nmax=8 if nwater < 4000 else 20, rcut=rcut)
    s = S.System(spec)
    st = S.make_configuration(s, seed=1, jitter=0.05)
    g = ForcePath(s, precision=MDX_MIXED)
    g.set_state(*st)
    g.double(0)
    g.double_steps(2, 0, records=False)
    rs, rl = mean_rows(g)
    short = {ts: time_split(g, ts, 32, steps, 10)[0] for ts in SHORT_SPLITS}
    long_ = {tl: time_split(g, 4, tl, steps, 40)[1] for tl in LONG_SPLITS}
    g.close()
    return dict(n=s.nstot, rcut=rcut, row_short=rs, row_long=rl, short=short, long=long_)


def classes(points: List[float]) -> List[float]:
    """Upper class bounds between sorted distinct points (geometric
    midpoints), the last one open."""
    p = sorted(set(points))
    return [math.sqrt(a * b) for a, b in zip(p, p[1:])] + [float("inf")]


def table(results, key_row: str, key_t: str):
    """Cells (max_atoms, max_row, tpo): by atom-count class, then by row
    class within it, the fastest split of the measured system in that cell."""
    cells = []
    nb = classes([r["n"] for r in results])
    lo = 0.0
    for hi in nb:
        group = [r for r in results if lo < r["n"] <= hi]
        rb = classes([r[key_row] for r in group])
        rlo = 0.0
        for rhi in rb:
            sub = [r for r in group if rlo < r[key_row] <= rhi]
            # the largest measured system of the cell decides
            best = max(sub, key=lambda r: r["n"])
            tpo = min(best[key_t], key=best[key_t].get)
            cells.append((hi, rhi, tpo))
            rlo = rhi
        lo = hi
    return cells


def write_header(path: str, short_cells, long_cells, device: str):
    def fmt(cells):
        out = []
        for n, r, t in cells:
            ns = "2147483647" if math.isinf(n) else str(int(n))
            rs = "1e30" if math.isinf(r) else f"{r:.1f}"
            out.append(f"{{{ns}, {rs}, {t}}}")
        return "{" + ", ".join(out) + "}"
    text = f"""// tune_table.cuh -- written by mdynamix_gb300/autotune.py; do not edit.
// Threads per owner atom of the mixed pair sweeps, by system size (atoms)
// and mean full-row length (entries): the first cell with n <= max_atoms
// and row <= max_row wins.  Measured on {device}.
#pragma once

struct TuneCell {{
  int max_atoms;
  double max_row;
  int tpo;
}};

constexpr TuneCell TUNE_SHORT[] = {fmt(short_cells)};
constexpr TuneCell TUNE_LONG[] = {fmt(long_cells)};
"""
    with open(path, "w") as f:
        f.write(text)


def write_record(path: str, results, short_cells, long_cells, device: str, cmd: str):
    lines = [f"# Tuning of the mixed pair sweeps' work split ({device})", "",
             "Device time per long step (ms, best of two passes of the library's timers) of the",
             "short sweep (10 per long step) by threads per owner atom (long split 32), and of the",
             "long sweep by threads per owner (short split 4).  SPC-FW water at 1 g/cm3, Rshort 5 A.",
             "", f"Command: `{cmd}`", "",
             "| atoms | Rcut | mean row short / long | short 2 / 4 / 8 | long 4 / 8 / 16 / 32 | chosen |",
             "|---|---|---|---|---|---|"]
    for r in results:
        sh = " / ".join(f"{r['short'][k]:.4f}" for k in SHORT_SPLITS)
        lg = " / ".join(f"{r['long'][k]:.4f}" for k in LONG_SPLITS)
        cs = min(r["short"], key=r["short"].get)
        cl = min(r["long"], key=r["long"].get)
        lines.append(f"| {r['n']} | {r['rcut']:.0f} | {r['row_short']:.0f} / {r['row_long']:.0f} "
                     f"| {sh} | {lg} | {cs} / {cl} |")
    lines += ["", "Table cells (max atoms, max mean row, threads per owner):", "",
              f"- short: {short_cells}", f"- long: {long_cells}", ""]
    with open(path, "w") as f:
        f.write("\n".join(lines))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("out")
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--quick", action="store_true", help="three systems only")
    a = ap.parse_args()
    import torch
    os.makedirs(a.out, exist_ok=True)
    device = torch.cuda.get_device_name(0)
    systems = SYSTEMS if not a.quick else (SYSTEMS[0], SYSTEMS[3], SYSTEMS[-1])
    results = []
    for nw, rc in systems:
        t0 = time.perf_counter()
        r = measure(nw, rc, a.steps)
        results.append(r)
        print(r, f"{time.perf_counter() - t0:.1f} s", flush=True)
    sc = table(results, "row_short", "short")
    lc = table(results, "row_long", "long")
    write_header(os.path.join(a.out, "tune_table.cuh"), sc, lc, device)
    cmd = "python -m mdynamix_gb300.autotune OUT" + (" --quick" if a.quick else "")
    write_record(os.path.join(a.out, "autotune_pair32.md"), results, sc, lc, device, cmd)
    print("short", sc)
    print("long", lc)


if __name__ == "__main__":
    main()
