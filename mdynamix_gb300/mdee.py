"""Expanded-ensemble (MDEE) moves over the device state.

The reference's walk between subensembles ME = 1..NE (mdee.f): every NCEE
long steps CHENS (mdee.f:142-262) proposes ME +- 1, computes the energy
change of the EE molecules' coupling -- DIFFUR (reciprocal Ewald), DIFEN
(pair terms over the lists), both on the GPU through ``mdx_ee_delta``, and
the LJ tail corrections EELRC of DIFF_LRCOR (mdee.f:541-600, host) -- and
accepts by the Metropolis rule, then rescales the interactions (RECINT,
``mdx_set_lambda``).  Balancing factors EE(ME) may be adapted by the
Wang-Landau scheme of the same routine.  The random stream is this module's
own (seeded), not the reference's ``rand()``.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from .system import BOLTZ, PI, System


def ee_lrc(s: System, ec: List[float], me: int, pw1: float, pw2: float, bee: float) -> np.ndarray:
    """EELRC(I) for every subensemble I (DIFF_LRCOR, mdee.f:541-600), with
    the cutoff shift taken at the current subensemble ME (1-based) for all
    I, as the reference does."""
    rc0 = math.sqrt(s.rssq)
    eeal3 = ec[me - 1] ** pw2
    out = np.zeros(len(ec))
    for I, eci in enumerate(ec):
        tot = 0.0
        for it in range(s.ntypes):
            esci = eci ** pw1 if s.iee[it] == 0 else 1.0
            for jt in range(it, s.ntypes):
                f = float(s.nspec[it] * s.nspec[jt])
                if it == jt:
                    f = 0.5 * f
                rc = rc0 + bee * (1.0 - eeal3) if s.iee[it] * s.iee[jt] == 0 else rc0
                escl = esci
                if s.iee[jt] == 0:
                    escl = eci ** pw1
                for isb in range(s.isadr[it], s.isadr[it + 1]):
                    ist = s.inbt[isb] - 1
                    for jsb in range(s.isadr[jt], s.isadr[jt + 1]):
                        jst = s.inbt[jsb] - 1
                        a6 = escl * s.a6lj0[ist, jst]
                        b12 = escl * s.b12lj0[ist, jst]
                        if abs(a6) >= 1e-50 and abs(b12) > 1e-50:
                            si3 = math.sqrt(-b12 / a6)
                            ep = 0.25 * a6 ** 2 / b12
                        else:
                            si3 = ep = 0.0
                        x = si3 / rc ** 3
                        elr = ep * si3 * ((1.0 / 9.0) * x ** 3 - (1.0 / 3.0) * x) * f
                        tot += 4.0 * PI * elr / s.vol
        out[I] = tot
    return out


@dataclass
class MdeeWalk:
    """CHENS over a ForcePath: NE couplings EC (EC[ME-1] is the current one),
    balancing factors EE, the MDEE keywords PW1, PW2, BEE, and the optional
    Wang-Landau adaptation (wl_corr > 0: EE(ME) -= wl_corr after every
    attempt)."""
    system: System
    ec: List[float]
    me: int = 1
    pw1: float = 1.0
    pw2: float = 1.0 / 3.0
    bee: float = 3.0
    ee: Optional[List[float]] = None
    wl_corr: float = 0.0
    seed: int = 1
    attempts: int = 0
    accepted: int = 0
    visits: List[int] = field(default_factory=list)

    def __post_init__(self):
        self.rng = np.random.default_rng(self.seed)
        if self.ee is None:
            self.ee = [0.0] * len(self.ec)
        self.visits = [0] * len(self.ec)
        s = self.system
        self.beta = s.unite / (BOLTZ * s.trtemp)  # setup.f:105
        self.eelrc = ee_lrc(s, self.ec, self.me, self.pw1, self.pw2, self.bee)

    def apply(self, path):
        """RECINT for the current subensemble on a ForcePath."""
        path.set_lambda(self.ec[self.me - 1], self.pw1, self.pw2, self.bee)

    def attempt(self, path) -> bool:
        """One CHENS move on the path's current state; True if accepted."""
        me1 = self.me - 1 if self.rng.random() < 0.5 else self.me + 1
        self.attempts += 1
        ok = False
        if 1 <= me1 <= len(self.ec):
            efn, efo, een, eeo = path.ee_delta(self.ec[self.me - 1], self.ec[me1 - 1],
                                               self.pw1, self.pw2, self.bee)
            de = ((een - eeo + efn - efo + self.eelrc[me1 - 1] - self.eelrc[self.me - 1])
                  * self.beta - self.ee[me1 - 1] + self.ee[self.me - 1])
            r = self.rng.random()
            # reject when exp(-DE) < rand() (mdee.f:193-197)
            if de <= 0.0 or not math.exp(-de) < r:
                self.me = me1
                self.accepted += 1
                self.apply(path)
                ok = True
        if self.wl_corr:
            self.ee[self.me - 1] -= self.wl_corr
        self.visits[self.me - 1] += 1
        return ok
