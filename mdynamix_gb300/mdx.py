"""Python binding of the GB300 force path (libmdxgpu.so, C ABI).

``ForcePath`` exposes the reference's routines under their own names:

    chcnb()        CHCNB     forces.f:1813   neighbour lists
    fforces(laver) FFORCES   forces.f:36     fast forces H
    slforces()     SLFORCES  forces.f:55     slow forces G
    allforce()     ALLFORCE  forces.f:77     F = G + H
    getcom()       GETCOM    service.f:463
    double(n)      DOUBLE    mdstep.f:281    double time step loop
    sultan(n)      SULTAN    mdstep.f:29     leap-frog + SHAKE loop
    set_lambda()   RECINT    mdee.f:86

Errors come back as ``MdxError`` carrying the library's code and message,
where the reference would print and stop.  There is no CPU fallback: if the
CUDA library is missing or no GPU is present, construction fails.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .abi import (ERRORS, F64P, I32P, MDX_FP64, MDX_MIXED, MdxDims, MdxParams,
                  MdxScalars, MdxStepRecord, MdxThermo, MdxTopo, Packed, pack,
                  thermo_init)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libmdxgpu.so")

_lib = None

TIMER_NAMES = ["list", "pair_short", "pair_long", "ew_tables", "ew_sfac", "ew_kterms",
               "ew_force", "eterms", "bonded", "move", "other"]


def probe_fma_peak(fp64: bool) -> float:
    """Measured FMA throughput (TFLOP/s) of the current GPU."""
    L = load()
    v = C.c_double()
    rc = L.mdx_probe_fma_peak(int(fp64), C.byref(v))
    if rc != 0:
        raise MdxError(rc, "probe failed")
    return v.value


def probe_pair_math(y, d):
    """The FP64 pair sweeps' exp(-y) and 1/d beside the CUDA library's, on
    the current GPU: (own_exp, lib_exp, own_rcp, lib_rcp)."""
    L = load()
    y = np.ascontiguousarray(y, np.float64)
    d = np.ascontiguousarray(d, np.float64)
    n = len(y)
    assert len(d) == n
    out = [np.zeros(n) for _ in range(4)]
    rc = L.mdx_probe_pair_math(n, _fp(y), _fp(d), *[_fp(a) for a in out])
    if rc != 0:
        raise MdxError(rc, "probe failed")
    return tuple(out)


class MdxError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


def load():
    """Load libmdxgpu.so and declare its C signatures."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is not built; run __graft_entry__.build()")
    L = C.CDLL(LIB_PATH)
    P = C.c_void_p
    L.mdx_open.argtypes = [C.POINTER(MdxDims), C.POINTER(P)]
    L.mdx_close.argtypes = [P]
    L.mdx_last_error.argtypes = [P]
    L.mdx_last_error.restype = C.c_char_p
    L.mdx_strerror.argtypes = [C.c_int]
    L.mdx_strerror.restype = C.c_char_p
    L.mdx_upload_topology.argtypes = [P, C.POINTER(MdxTopo)]
    L.mdx_set_params.argtypes = [P, C.POINTER(MdxParams)]
    L.mdx_upload_state.argtypes = [P, F64P, F64P, F64P, F64P, F64P, F64P, C.POINTER(MdxThermo)]
    L.mdx_download_state.argtypes = [P, F64P, F64P, F64P, F64P, F64P, F64P, C.POINTER(MdxThermo)]
    L.mdx_download_forces.argtypes = [P, C.c_int, F64P, F64P, F64P]
    L.mdx_snapshot.argtypes = [P, C.c_int32, F64P, F64P, F64P, F64P, F64P, F64P,
                               C.POINTER(MdxThermo)]
    L.mdx_snapshot_wait.argtypes = [P, C.c_int32]
    L.mdx_get_bonded_averages.argtypes = [P, F64P, F64P, F64P, F64P, F64P, F64P]
    L.mdx_set_averaging.argtypes = [P, C.c_int]
    from mdynamix_gb300.abi import MdxPullback
    L.mdx_set_pullback.argtypes = [P, C.POINTER(MdxPullback)]
    L.mdx_get_bonded_sums.argtypes = [P, F64P, C.c_int32]
    L.mdx_inifur.argtypes = [P, I32P]
    L.mdx_chcnb.argtypes = [P, I32P, I32P]
    L.mdx_get_lists.argtypes = [P, I32P, I32P, C.c_int32, I32P, I32P, C.c_int32]
    L.mdx_getcom.argtypes = [P]
    L.mdx_getkin.argtypes = [P, C.POINTER(C.c_double), C.c_double, C.c_double, C.c_double,
                             C.c_double, C.c_void_p]
    L.mdx_chkmom.argtypes = [P, C.c_double, C.POINTER(C.c_double)]
    L.mdx_fforces.argtypes = [P, C.c_int, C.POINTER(MdxScalars)]
    L.mdx_slforces.argtypes = [P, C.POINTER(MdxScalars)]
    L.mdx_allforce.argtypes = [P, C.POINTER(MdxScalars)]
    L.mdx_slforces_static.argtypes = [P, C.POINTER(MdxScalars)]
    L.mdx_double_enqueue.argtypes = [P, C.c_int32, C.c_int32, C.c_int32]
    L.mdx_poll.argtypes = [P, I32P]
    L.mdx_device_memory.argtypes = [C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]
    L.mdx_pool_usage.argtypes = [C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]
    from mdynamix_gb300.abi import MdxPathInfo, MdxTuning
    L.mdx_get_path_info.argtypes = [P, C.POINTER(MdxPathInfo)]
    L.mdx_set_tuning.argtypes = [P, C.POINTER(MdxTuning)]
    L.mdx_get_tuning.argtypes = [P, C.POINTER(MdxTuning)]
    for n in ("mdx_double", "mdx_double_steps", "mdx_sultan", "mdx_sultan_steps"):
        getattr(L, n).argtypes = [P, C.c_int32, C.c_int32, C.POINTER(MdxStepRecord)]
    L.mdx_set_lambda.argtypes = [P, C.c_double, C.c_double, C.c_double, C.c_double]
    L.mdx_ee_delta.argtypes = [P, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                               F64P]
    L.mdx_stream.argtypes = [P]
    L.mdx_stream.restype = C.c_void_p
    L.mdx_launch_count.argtypes = [P]
    L.mdx_launch_count.restype = C.c_int64
    L.mdx_sync.argtypes = [P]
    L.mdx_version.restype = C.c_int
    L.mdx_set_timers.argtypes = [P, C.c_int]
    L.mdx_get_timers.argtypes = [P, F64P, C.POINTER(C.c_int64)]
    L.mdx_probe_fma_peak.argtypes = [C.c_int, F64P]
    L.mdx_probe_pair_math.argtypes = [C.c_int, F64P, F64P, F64P, F64P, F64P, F64P]
    from .abi import MdxPimdParams, MdxPimdRecord
    L.mdx_pimd_open.argtypes = [C.POINTER(P), C.POINTER(MdxPimdParams), C.POINTER(P)]
    L.mdx_pimd_close.argtypes = [P]
    L.mdx_pimd_run.argtypes = [P, C.c_int32, C.c_int32, C.POINTER(MdxPimdRecord)]
    L.mdx_pimd_steps.argtypes = [P, C.c_int32, C.c_int32, C.POINTER(MdxPimdRecord)]
    L.mdx_pimd_get_thermo.argtypes = [P, F64P]
    L.mdx_pimd_stream.argtypes = [P]
    L.mdx_pimd_stream.restype = P
    L.mdx_pimd_set_thermo.argtypes = [P, F64P]
    _lib = L
    return L


def device_memory():
    """(free, total) bytes of the current device."""
    L = load()
    f, t = C.c_size_t(), C.c_size_t()
    if L.mdx_device_memory(C.byref(f), C.byref(t)) != 0:
        raise MdxError(2, "cudaMemGetInfo failed")
    return f.value, t.value


def _fp(a):
    return a.ctypes.data_as(F64P)


class ForcePath:
    """One system resident on the GPU behind the C ABI."""

    def __init__(self, system, precision: int = MDX_FP64, packed: Packed = None, **caps):
        self.L = load()
        self.system = system
        self.packed = packed or pack(system, precision=precision, **caps)
        self.n = system.nstot
        h = C.c_void_p()
        rc = self.L.mdx_open(C.byref(self.packed.dims), C.byref(h))
        if rc != 0:
            raise MdxError(rc, "mdx_open failed (no GPU or bad sizes)")
        self.h = h
        self._check(self.L.mdx_upload_topology(self.h, C.byref(self.packed.topo)))
        self._check(self.L.mdx_set_params(self.h, C.byref(self.packed.params)))

    # ---------------------------------------------------------------- util
    def _check(self, rc):
        if rc != 0:
            raise MdxError(rc, self.L.mdx_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.L.mdx_close(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self) -> int:
        return self.L.mdx_stream(self.h)

    @property
    def launches(self) -> int:
        return self.L.mdx_launch_count(self.h)

    def sync(self):
        self._check(self.L.mdx_sync(self.h))

    def set_timers(self, on: bool = True):
        self._check(self.L.mdx_set_timers(self.h, int(on)))

    def timers(self) -> dict:
        """Accumulated device milliseconds and launch counts per routine group
        since the last call (the GPU counterpart of the reference's CPU time
        table); clears them."""
        ms = np.zeros(len(TIMER_NAMES))
        cnt = np.zeros(len(TIMER_NAMES), dtype=np.int64)
        self._check(self.L.mdx_get_timers(self.h, _fp(ms), cnt.ctypes.data_as(C.POINTER(C.c_int64))))
        return {n: (float(ms[i]), int(cnt[i])) for i, n in enumerate(TIMER_NAMES)}

    # ---------------------------------------------------------------- data
    def set_params(self, params: MdxParams):
        self._check(self.L.mdx_set_params(self.h, C.byref(params)))

    def set_state(self, sx, sy, sz, vx, vy, vz, thermo: MdxThermo = None):
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (sx, sy, sz, vx, vy, vz)]
        th = thermo if thermo is not None else thermo_init(self.system)
        self._check(self.L.mdx_upload_state(self.h, *[_fp(a) for a in arrs], C.byref(th)))

    def get_state(self, out=None):
        """(sx, sy, sz, vx, vy, vz), thermo; ``out``: six contiguous float64
        arrays to download into (e.g. page-locked host buffers)."""
        if out is None:
            out = [np.zeros(self.n) for _ in range(6)]
        else:
            assert len(out) == 6 and all(a.dtype == np.float64 and a.flags.c_contiguous
                                         and a.size == self.n for a in out)
        th = MdxThermo()
        self._check(self.L.mdx_download_state(self.h, *[_fp(a) for a in out], C.byref(th)))
        return out, th

    def forces(self, which: int = 3) -> np.ndarray:
        out = [np.zeros(self.n) for _ in range(3)]
        self._check(self.L.mdx_download_forces(self.h, which, *[_fp(a) for a in out]))
        return np.stack(out, axis=1)

    # ------------------------------------------------------------ routines
    def inifur(self) -> int:
        n = C.c_int32()
        self._check(self.L.mdx_inifur(self.h, C.byref(n)))
        return n.value

    def chcnb(self):
        a, b = C.c_int32(), C.c_int32()
        self._check(self.L.mdx_chcnb(self.h, C.byref(a), C.byref(b)))
        self.counts = (a.value, b.value)
        return self.counts

    def lists(self):
        ms, ml = self.counts
        a1, a2 = np.zeros(ms, np.int32), np.zeros(ms, np.int32)
        b1, b2 = np.zeros(ml, np.int32), np.zeros(ml, np.int32)
        self._check(self.L.mdx_get_lists(self.h, a1.ctypes.data_as(I32P), a2.ctypes.data_as(I32P),
                                         ms, b1.ctypes.data_as(I32P), b2.ctypes.data_as(I32P), ml))
        return (a1, a2), (b1, b2)

    def getcom(self):
        self._check(self.L.mdx_getcom(self.h))

    def getkin(self):
        """GETKIN (service.f:611-735): EKTR, EKROT, EKINT, TKE, TTR, TROT, TINT
        with the system's unit and degree-of-freedom constants."""
        from mdynamix_gb300.abi import MdxKin
        from mdynamix_gb300.system import kin_summd
        s = self.system
        summd = (C.c_double * max(1, s.ntypes))(*kin_summd(s))
        k = MdxKin()
        self._check(self.L.mdx_getkin(self.h, summd, s.enerf * s.tempf, s.fnop, s.fnstr,
                                      s.fnsti, C.byref(k)))
        return k

    def chkmom(self):
        """CHKMOM (service.f:1081-1125): removes the total momentum; returns
        the removed (DVX, DVY, DVZ)."""
        from mdynamix_gb300.system import kin_sumasd
        dv = (C.c_double * 3)()
        self._check(self.L.mdx_chkmom(self.h, kin_sumasd(self.system), dv))
        return tuple(dv)

    def fforces(self, laver: bool = True) -> MdxScalars:
        s = MdxScalars()
        self._check(self.L.mdx_fforces(self.h, int(laver), C.byref(s)))
        return s

    def slforces(self) -> MdxScalars:
        s = MdxScalars()
        self._check(self.L.mdx_slforces(self.h, C.byref(s)))
        return s

    def allforce(self) -> MdxScalars:
        s = MdxScalars()
        self._check(self.L.mdx_allforce(self.h, C.byref(s)))
        return s

    def path_info(self) -> dict:
        """Which Ewald passes, list mode and graph replay the context uses."""
        from mdynamix_gb300.abi import MdxPathInfo
        info = MdxPathInfo()
        self._check(self.L.mdx_get_path_info(self.h, C.byref(info)))
        return info.as_dict()

    def tuning(self) -> dict:
        """Threads per owner atom of the mixed pair sweeps and where the
        choice came from (1 the tuning table, 2 set_tuning)."""
        from mdynamix_gb300.abi import MdxTuning
        t = MdxTuning()
        self._check(self.L.mdx_get_tuning(self.h, C.byref(t)))
        return t.as_dict()

    def set_tuning(self, tpo_short: int = None, tpo_long: int = None):
        """Override the split (both None: back to the tuning table)."""
        from mdynamix_gb300.abi import MdxTuning
        if tpo_short is None and tpo_long is None:
            self._check(self.L.mdx_set_tuning(self.h, None))
            return
        cur = self.tuning()
        t = MdxTuning(tpo_short if tpo_short is not None else cur["tpo_short"],
                      tpo_long if tpo_long is not None else cur["tpo_long"], 2, 0)
        self._check(self.L.mdx_set_tuning(self.h, C.byref(t)))

    def bonded_averages(self) -> dict:
        """BR, BE, AR, AE, TR, TE of the last FFORCES with LAVER: per bond,
        angle and torsion record, its length (angle) and energy averaged over
        the type's molecules (forces.f:181-182, 272-273, 446-447)."""
        s = self.system
        out = {k: np.zeros(max(1, n)) for k, n in (("br", s.nrbb), ("be", s.nrbb),
                                                    ("ar", s.nraa), ("ae", s.nraa),
                                                    ("tr", s.nrtt), ("te", s.nrtt))}
        self._check(self.L.mdx_get_bonded_averages(self.h, *[_fp(out[k]) for k in
                                                             ("br", "be", "ar", "ae", "tr", "te")]))
        n = {"br": s.nrbb, "be": s.nrbb, "ar": s.nraa, "ae": s.nraa, "tr": s.nrtt, "te": s.nrtt}
        return {k: v[:n[k]] for k, v in out.items()}

    def set_pullback(self, pb=None):
        """PULLBACK's drag, wells and external field (abi.pullback builds
        pb); None switches them off."""
        self._check(self.L.mdx_set_pullback(self.h, C.byref(pb) if pb is not None else None))

    def set_averaging(self, on: bool = True):
        """Keep GETAVR's bonded statistics on the device, one sample per long
        step (mdx_set_averaging)."""
        self._check(self.L.mdx_set_averaging(self.h, int(on)))

    def bonded_sums(self, clear: bool = False):
        """(samples, sums, sums of squares) of BR, BE, AR, AE, TR, TE, each a
        dict of arrays per record."""
        s = self.system
        lens = [("br", s.nrbb), ("be", s.nrbb), ("ar", s.nraa), ("ae", s.nraa),
                ("tr", s.nrtt), ("te", s.nrtt)]
        L = sum(n for _, n in lens)
        buf = np.zeros(1 + 2 * L)
        self._check(self.L.mdx_get_bonded_sums(self.h, _fp(buf), int(clear)))
        sums, sq, off = {}, {}, 1
        for k, n in lens:
            sums[k] = buf[off:off + n].copy()
            sq[k] = buf[1 + L + off - 1:1 + L + off - 1 + n].copy()
            off += n
        return int(buf[0]), sums, sq

    def _run(self, fn, nsteps, start, records=True):
        recs = (MdxStepRecord * max(1, nsteps))() if records else None
        self._check(getattr(self.L, fn)(self.h, nsteps, start, recs))
        return [recs[i] for i in range(nsteps)] if records else None

    def double(self, nsteps: int, nsttot: int = 0, records: bool = True):
        return self._run("mdx_double", nsteps, nsttot, records)

    def double_steps(self, nsteps: int, mstep0: int, records: bool = True):
        return self._run("mdx_double_steps", nsteps, mstep0, records)

    def sultan(self, nsteps: int, nsttot: int = 0, records: bool = True):
        return self._run("mdx_sultan", nsteps, nsttot, records)

    def sultan_steps(self, nsteps: int, mstep0: int, records: bool = True):
        return self._run("mdx_sultan_steps", nsteps, mstep0, records)

    def enqueue_double(self, nsteps: int, mstep0: int = 0, prologue: bool = False):
        """Queue nsteps DOUBLE long steps (and the prologue) without waiting."""
        self._check(self.L.mdx_double_enqueue(self.h, nsteps, mstep0, int(prologue)))

    def poll(self) -> bool:
        """True once the queued work has finished (errors raise MdxError)."""
        d = C.c_int32()
        self._check(self.L.mdx_poll(self.h, C.byref(d)))
        return bool(d.value)

    def ee_delta(self, ec_old: float, ec_new: float, pw1: float = 1.0, pw2: float = 1.0 / 3.0,
                 bee: float = 3.0):
        """DIFFUR and DIFEN for a move from coupling ec_old to ec_new:
        (EFN, EFO, EEN, EEO) in internal energy units."""
        out = np.zeros(4)
        self._check(self.L.mdx_ee_delta(self.h, ec_old, ec_new, pw1, pw2, bee, _fp(out)))
        return tuple(float(x) for x in out)

    def set_lambda(self, ec: float, pw1: float = 1.0, pw2: float = 1.0 / 3.0, bee: float = 3.0):
        self._check(self.L.mdx_set_lambda(self.h, ec, pw1, pw2, bee))


__all__ = ["ForcePath", "MdxError", "load", "MDX_FP64", "MDX_MIXED"]


class PimdPath:
    """Path-integral MD: one ForcePath per bead replica, advanced together
    (PIMD, pimd.f:18-316) by the library's bead coupling."""

    def __init__(self, system, states, precision: int = MDX_FP64, **caps):
        from .system import pimd_params
        from .abi import MdxPimdRecord
        self.L = load()
        self.system = system
        self.pp = pimd_params(system)
        self.beads = []
        for st in states:
            g = ForcePath(system, precision=precision, **caps)
            g.set_state(*st)
            self.beads.append(g)
        hs = (C.c_void_p * len(self.beads))(*[b.h.value for b in self.beads])
        h = C.c_void_p()
        rc = self.L.mdx_pimd_open(hs, C.byref(self.pp), C.byref(h))
        if rc != 0:
            raise MdxError(rc, self.L.mdx_last_error(self.beads[0].h).decode())
        self.h = h
        self._Rec = MdxPimdRecord

    def _run(self, fn, nsteps, start):
        recs = (self._Rec * max(1, nsteps))()
        rc = getattr(self.L, fn)(self.h, nsteps, start, recs)
        if rc != 0:
            raise MdxError(rc, "PIMD: " + " / ".join(
                self.L.mdx_last_error(b.h).decode() for b in self.beads[:1]))
        return [recs[i] for i in range(nsteps)]

    @property
    def stream(self) -> int:
        return self.L.mdx_pimd_stream(self.h)

    def run(self, nsteps: int, nsttot: int = 0):
        return self._run("mdx_pimd_run", nsteps, nsttot)

    def steps(self, nsteps: int, mstep0: int):
        return self._run("mdx_pimd_steps", nsteps, mstep0)

    def thermo(self) -> np.ndarray:
        t = np.zeros(self.system.nstot * self.pp.jnh)
        if self.L.mdx_pimd_get_thermo(self.h, _fp(t)) != 0:
            raise MdxError(2, "PIMD thermo download")
        return t

    def states(self):
        return [b.get_state()[0] for b in self.beads]

    def close(self):
        if getattr(self, "h", None):
            self.L.mdx_pimd_close(self.h)
            self.h = None
        for b in self.beads:
            b.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
