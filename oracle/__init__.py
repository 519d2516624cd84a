"""Python loader of the CPU oracle (test infrastructure only).

``Oracle`` exposes the restated reference routines under the reference's
names (chcnb, fforces, slforces, allforce, double, sultan, ...) over the
same packed inputs the GPU library takes.  Only tests, the smoke check and
the benchmark's CPU-baseline leg import this package.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "libmdx_oracle.so")

_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with oracle/Makefile (gcc, a few seconds; make
    skips it when the library is newer than its sources)."""
    subprocess.run(["make", "-s", "-C", HERE] + (["-B"] if force else []), check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIB)
        from mdynamix_gb300.abi import (F64P, I32P, MdxDims, MdxParams, MdxScalars,
                                        MdxStepRecord, MdxThermo, MdxTopo)
        P = C.c_void_p
        L = _lib
        L.ox_open.argtypes = [C.POINTER(MdxDims), C.POINTER(MdxTopo), C.POINTER(MdxParams),
                              C.POINTER(P)]
        L.ox_close.argtypes = [P]
        L.ox_last_error.argtypes = [P]
        L.ox_last_error.restype = C.c_char_p
        L.ox_set_threads.argtypes = [P, C.c_int]
        L.ox_set_params.argtypes = [P, C.POINTER(MdxParams)]
        L.ox_set_state.argtypes = [P, F64P, F64P, F64P, F64P, F64P, F64P, C.POINTER(MdxThermo)]
        L.ox_get_state.argtypes = [P, F64P, F64P, F64P, F64P, F64P, F64P, C.POINTER(MdxThermo)]
        L.ox_get_forces.argtypes = [P, C.c_int, F64P, F64P, F64P]
        L.ox_get_bonded_averages.argtypes = [P, F64P, F64P, F64P, F64P, F64P, F64P]
        L.ox_inifur.argtypes = [P, I32P]
        L.ox_chcnb.argtypes = [P, I32P, I32P]
        L.ox_get_lists.argtypes = [P, I32P, I32P, C.c_int32, I32P, I32P, C.c_int32]
        L.ox_getcom.argtypes = [P]
        L.ox_getkin.argtypes = [P, C.POINTER(C.c_double), C.c_double, C.c_double, C.c_double,
                                C.c_double, C.POINTER(C.c_double)]
        L.ox_chkmom.argtypes = [P, C.c_double, C.POINTER(C.c_double)]
        L.ox_fforces.argtypes = [P, C.c_int, C.POINTER(MdxScalars)]
        L.ox_slforces.argtypes = [P, C.POINTER(MdxScalars)]
        L.ox_allforce.argtypes = [P, C.POINTER(MdxScalars)]
        for n in ("ox_double", "ox_double_steps", "ox_sultan", "ox_sultan_steps"):
            getattr(L, n).argtypes = [P, C.c_int32, C.c_int32, C.POINTER(MdxStepRecord)]
        L.ox_set_lambda.argtypes = [P, C.c_double, C.c_double, C.c_double, C.c_double]
        from mdynamix_gb300.abi import MdxPullback
        L.ox_set_pullback.argtypes = [P, C.POINTER(MdxPullback)]
        L.ox_ee_delta.argtypes = [P, C.c_double, C.c_double, C.c_double, C.c_double,
                                  C.c_double, F64P]
        from mdynamix_gb300.abi import MdxPimdParams, MdxPimdRecord
        L.ox_pimd_steps.argtypes = [C.POINTER(P), C.POINTER(MdxPimdParams), F64P, C.c_int32,
                                    C.c_int32, C.c_int, C.POINTER(MdxPimdRecord)]
    return _lib


def _fp(a):
    from mdynamix_gb300.abi import F64P
    return a.ctypes.data_as(F64P)


class OracleError(RuntimeError):
    pass


class Oracle:
    """The restated reference routines on one system (CPU)."""

    def __init__(self, system, threads: int = 1, packed=None):
        from mdynamix_gb300.abi import pack
        self.system = system
        self.packed = packed or pack(system)
        self.L = lib()
        h = C.c_void_p()
        self._check(self.L.ox_open(C.byref(self.packed.dims), C.byref(self.packed.topo),
                                   C.byref(self.packed.params), C.byref(h)), None)
        self.h = h
        self.L.ox_set_threads(self.h, threads)
        self.n = system.nstot

    def _check(self, rc, h=True):
        if rc != 0:
            msg = self.L.ox_last_error(self.h).decode() if h is not None and getattr(self, "h", None) else ""
            from mdynamix_gb300.abi import ERRORS
            raise OracleError(f"{ERRORS.get(rc, rc)}: {msg}")

    def close(self):
        if getattr(self, "h", None):
            self.L.ox_close(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_threads(self, n):
        self.L.ox_set_threads(self.h, n)

    def set_state(self, sx, sy, sz, vx, vy, vz, thermo=None):
        from mdynamix_gb300.abi import thermo_init
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (sx, sy, sz, vx, vy, vz)]
        th = thermo if thermo is not None else thermo_init(self.system)
        self._check(self.L.ox_set_state(self.h, *[_fp(a) for a in arrs], C.byref(th)))

    def get_state(self):
        from mdynamix_gb300.abi import MdxThermo
        out = [np.zeros(self.n) for _ in range(6)]
        th = MdxThermo()
        self._check(self.L.ox_get_state(self.h, *[_fp(a) for a in out], C.byref(th)))
        return out, th

    def forces(self, which=3):
        out = [np.zeros(self.n) for _ in range(3)]
        self._check(self.L.ox_get_forces(self.h, which, *[_fp(a) for a in out]))
        return np.stack(out, axis=1)

    def inifur(self):
        n = C.c_int32()
        self._check(self.L.ox_inifur(self.h, C.byref(n)))
        return n.value

    def chcnb(self):
        a, b = C.c_int32(), C.c_int32()
        self._check(self.L.ox_chcnb(self.h, C.byref(a), C.byref(b)))
        self.chcnb_counts = (a.value, b.value)
        return self.chcnb_counts

    def lists(self):
        from mdynamix_gb300.abi import I32P
        ms, ml = self.chcnb_counts
        a1, a2 = np.zeros(ms, np.int32), np.zeros(ms, np.int32)
        b1, b2 = np.zeros(ml, np.int32), np.zeros(ml, np.int32)
        self._check(self.L.ox_get_lists(self.h, a1.ctypes.data_as(I32P), a2.ctypes.data_as(I32P),
                                        ms, b1.ctypes.data_as(I32P), b2.ctypes.data_as(I32P), ml))
        return (a1, a2), (b1, b2)

    def chcnb_lists(self):
        self.chcnb_counts = self.chcnb()
        return self.lists()

    def getcom(self):
        self._check(self.L.ox_getcom(self.h))

    def bonded_averages(self):
        s = self.system
        out = {k: np.zeros(max(1, n)) for k, n in (("br", s.nrbb), ("be", s.nrbb),
                                                    ("ar", s.nraa), ("ae", s.nraa),
                                                    ("tr", s.nrtt), ("te", s.nrtt))}
        self._check(self.L.ox_get_bonded_averages(self.h, *[_fp(out[k]) for k in
                                                           ("br", "be", "ar", "ae", "tr", "te")]))
        n = {"br": s.nrbb, "be": s.nrbb, "ar": s.nraa, "ae": s.nraa, "tr": s.nrtt, "te": s.nrtt}
        return {k: v[:n[k]] for k, v in out.items()}

    def getkin(self):
        """GETKIN: [EKTR, EKROT, EKINT, TKE, TTR, TROT, TINT]."""
        from mdynamix_gb300.system import kin_summd
        s = self.system
        summd = (C.c_double * max(1, s.ntypes))(*kin_summd(s))
        out = (C.c_double * 7)()
        self._check(self.L.ox_getkin(self.h, summd, s.enerf * s.tempf, s.fnop, s.fnstr,
                                     s.fnsti, out))
        return list(out)

    def chkmom(self):
        from mdynamix_gb300.system import kin_sumasd
        dv = (C.c_double * 3)()
        self._check(self.L.ox_chkmom(self.h, kin_sumasd(self.system), dv))
        return tuple(dv)

    def fforces(self, laver=True):
        from mdynamix_gb300.abi import MdxScalars
        s = MdxScalars()
        self._check(self.L.ox_fforces(self.h, int(laver), C.byref(s)))
        return s

    def slforces(self):
        from mdynamix_gb300.abi import MdxScalars
        s = MdxScalars()
        self._check(self.L.ox_slforces(self.h, C.byref(s)))
        return s

    def allforce(self):
        from mdynamix_gb300.abi import MdxScalars
        s = MdxScalars()
        self._check(self.L.ox_allforce(self.h, C.byref(s)))
        return s

    def _run(self, fn, nsteps, start):
        from mdynamix_gb300.abi import MdxStepRecord
        recs = (MdxStepRecord * max(1, nsteps))()
        self._check(getattr(self.L, fn)(self.h, nsteps, start, recs))
        return [recs[i] for i in range(nsteps)]

    def double(self, nsteps, nsttot=0):
        return self._run("ox_double", nsteps, nsttot)

    def double_steps(self, nsteps, mstep0):
        return self._run("ox_double_steps", nsteps, mstep0)

    def sultan(self, nsteps, nsttot=0):
        return self._run("ox_sultan", nsteps, nsttot)

    def sultan_steps(self, nsteps, mstep0):
        return self._run("ox_sultan_steps", nsteps, mstep0)

    def set_pullback(self, pb=None):
        self._check(self.L.ox_set_pullback(self.h, C.byref(pb) if pb is not None else None))

    def ee_delta(self, ec_old, ec_new, pw1=1.0, pw2=1.0 / 3.0, bee=3.0):
        out = np.zeros(4)
        self._check(self.L.ox_ee_delta(self.h, ec_old, ec_new, pw1, pw2, bee, _fp(out)))
        return tuple(float(x) for x in out)

    def set_lambda(self, ec, pw1=1.0, pw2=1.0 / 3.0, bee=3.0):
        self._check(self.L.ox_set_lambda(self.h, ec, pw1, pw2, bee))


class OraclePimd:
    """PIMD over bead replicas with the restated pimd.f (PIFORCES, BEADNOSE,
    the PIMD loop); one Oracle per bead."""

    def __init__(self, system, states, threads: int = 1):
        from mdynamix_gb300.system import pimd_params
        self.system = system
        self.pp = pimd_params(system)
        self.beads = []
        for st in states:
            o = Oracle(system, threads=threads)
            o.set_state(*st)
            self.beads.append(o)
        self.thermo = np.zeros(system.nstot * self.pp.jnh)
        self.L = lib()

    def _steps(self, nsteps, mstep0, prologue):
        from mdynamix_gb300.abi import MdxPimdRecord
        hs = (C.c_void_p * len(self.beads))(*[b.h.value for b in self.beads])
        recs = (MdxPimdRecord * max(1, nsteps))()
        rc = self.L.ox_pimd_steps(hs, C.byref(self.pp), _fp(self.thermo), nsteps, mstep0,
                                  int(prologue), recs)
        if rc != 0:
            self.beads[0]._check(rc)
        return [recs[i] for i in range(nsteps)]

    def run(self, nsteps, nsttot=0):
        return self._steps(nsteps, nsttot, True)

    def steps(self, nsteps, mstep0):
        return self._steps(nsteps, mstep0, False)

    def states(self):
        return [b.get_state()[0] for b in self.beads]
