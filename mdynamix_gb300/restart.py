"""Restart files and trajectories in the reference's formats, fed from device
state.

- ``read_dmp`` / ``write_dmp``: the unformatted restart file of RESTRT
  (restart.f:133-238 reads it, restart.f:390-420 writes it): Fortran
  sequential records, each framed by its byte length as a 4-byte integer.
  Both the v5.0 layout (the third record without ME, NEOLD, I3, I4, as the
  reference's own ``sample/NaCl.dmp``) and the v5.3 layout are read; the
  v5.3 layout is written.
- ``TraceWriter``: TRACE's trajectory files (restart.f:425-598), XMOL text
  (ITREK even) or the binary form (ITREK odd), a new numbered file after
  LTREK configurations.
- ``SnapshotDumper``: the device half -- ``mdx_snapshot`` queues the copy of
  positions, momenta and thermostat state into pinned host buffers on the
  context's stream and returns; a host thread waits for that copy and does
  the formatted write, so the next steps are already queued while the file
  is written (the reference stops its step loop for both).
"""
from __future__ import annotations

import ctypes as C
import os
import queue
import struct
import threading
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

LABEL = "MDYN_v5.3"


# ------------------------------------------------------ Fortran records --
def _records(data: bytes) -> List[bytes]:
    """Split a Fortran unformatted sequential file into its records."""
    out, off = [], 0
    while off < len(data):
        if off + 4 > len(data):
            raise ValueError("truncated record marker")
        n = struct.unpack_from("<i", data, off)[0]
        if n < 0 or off + 8 + n > len(data):
            raise ValueError(f"bad record length {n} at byte {off}")
        rec = data[off + 4:off + 4 + n]
        if struct.unpack_from("<i", data, off + 4 + n)[0] != n:
            raise ValueError(f"record markers differ at byte {off}")
        out.append(rec)
        off += 8 + n
    return out


def _frame(payload: bytes) -> bytes:
    return struct.pack("<i", len(payload)) + payload + struct.pack("<i", len(payload))


# ------------------------------------------------------------- .dmp file --
@dataclass
class RestartFile:
    """The contents of an unformatted restart file (plain MD, no MDEE/PIMD
    blocks unless present)."""
    label: str
    nop: int
    ntypes: int
    nstot: int
    nnav: int
    dt: float                       # DT (s)
    nstep: int = 0                  # MSTEP of the run that wrote it
    nsttot: int = 0                 # NSTTOT: steps since the very start
    nstepa: int = 0
    navt: int = 0
    nhist: int = 0
    tim: float = 0.0                # TIM (s)
    tima: float = 0.0
    ntrkf: int = 0
    ntrkz: int = 0
    me: int = 0
    neold: int = 0
    sc: float = 0.0                 # thermostat / barostat state
    scl: float = 0.0
    boxl: float = 0.0
    vol: float = 0.0
    rdfcut: float = 0.0
    boyl: float = 0.0
    bozl: float = 0.0
    sclx: float = 0.0
    scly: float = 0.0
    sclz: float = 0.0
    scm: List[float] = field(default_factory=list)
    box_extra: List[float] = field(default_factory=list)  # SHUTA and anything after SCM
    times: List[float] = field(default_factory=list)      # the 11 CPU-time counters
    sx: np.ndarray = None
    sy: np.ndarray = None
    sz: np.ndarray = None
    vx: np.ndarray = None           # momenta, the reference's VX
    vy: np.ndarray = None
    vz: np.ndarray = None
    av: np.ndarray = None           # averages of the current window (AV, AW)
    aw: np.ndarray = None
    hist: List[np.ndarray] = field(default_factory=list)
    tail: List[bytes] = field(default_factory=list)       # records not decoded (MDEE/PIMD)

    @property
    def positions(self):
        return self.sx, self.sy, self.sz

    @property
    def momenta(self):
        return self.vx, self.vy, self.vz


def read_dmp(path: str, ntypes: Optional[int] = None) -> RestartFile:
    """Read an unformatted restart file (restart.f:133-238).  ``ntypes``
    (the input's number of molecule types) splits SCM from the values that
    follow it in the fourth record; by default the file's own NTYPES."""
    with open(path, "rb") as f:
        recs = _records(f.read())
    if len(recs) < 7:
        raise ValueError(f"{path}: {len(recs)} records, a restart file has at least 7")
    label = recs[0].decode("latin-1").rstrip()
    nop, nt, nstot, nnav = struct.unpack_from("<4i", recs[1])
    (dt,) = struct.unpack_from("<d", recs[1], 16)
    r = RestartFile(label=label, nop=nop, ntypes=nt, nstot=nstot, nnav=nnav, dt=dt)
    h = recs[2]
    r.nstep, r.nsttot, r.nstepa, r.navt, r.nhist = struct.unpack_from("<5i", h)
    r.tim, r.tima = struct.unpack_from("<2d", h, 20)
    r.ntrkf, r.ntrkz = struct.unpack_from("<2i", h, 36)
    if len(h) >= 52:  # v5.3: ME, NEOLD (and I3, I4)
        r.me, r.neold = struct.unpack_from("<2i", h, 44)
    b = np.frombuffer(recs[3], "<f8")
    (r.sc, r.scl, r.boxl, r.vol, r.rdfcut, r.boyl, r.bozl, r.sclx, r.scly, r.sclz) = (
        float(x) for x in b[:10])
    k = ntypes if ntypes is not None else nt
    r.scm = [float(x) for x in b[10:10 + k]]
    r.box_extra = [float(x) for x in b[10 + k:]]
    r.times = [float(x) for x in np.frombuffer(recs[4], "<f8")]
    xyz = np.frombuffer(recs[5], "<f8")
    vel = np.frombuffer(recs[6], "<f8")
    if xyz.size != 3 * nstot or vel.size != 3 * nstot:
        raise ValueError(f"{path}: coordinate records do not hold {nstot} atoms")
    # WRITE (SX(I),SY(I),SZ(I),I=1,NSTOT): interleaved per atom
    xyz = xyz.reshape(nstot, 3)
    vel = vel.reshape(nstot, 3)
    r.sx, r.sy, r.sz = (xyz[:, 0].copy(), xyz[:, 1].copy(), xyz[:, 2].copy())
    r.vx, r.vy, r.vz = (vel[:, 0].copy(), vel[:, 1].copy(), vel[:, 2].copy())
    rest = recs[7:]
    if r.neold == 0 and rest and len(rest[0]) == 16 * nnav:
        avw = np.frombuffer(rest[0], "<f8").reshape(nnav, 2)
        r.av, r.aw = avw[:, 0].copy(), avw[:, 1].copy()
        rest = rest[1:]
        nh = min(r.nhist, len(rest))
        r.hist = [np.frombuffer(rest[j], "<f8").copy() for j in range(nh)]
        rest = rest[nh:]
    r.tail = list(rest)
    return r


def write_dmp(path: str, r: RestartFile) -> None:
    """Write an unformatted restart file in the layout of restart.f:390-420
    (v5.3: the third record carries ME, NEOLD, I3, I4)."""
    n = r.nstot
    lab = (r.label or LABEL).encode("latin-1")[:24].ljust(24)
    recs = [lab,
            struct.pack("<4id", r.nop, r.ntypes, n, r.nnav, r.dt),
            struct.pack("<5i2d6i", r.nstep, r.nsttot, r.nstepa, r.navt, r.nhist, r.tim, r.tima,
                        r.ntrkf, r.ntrkz, r.me, r.neold, 0, 0),
            np.array([r.sc, r.scl, r.boxl, r.vol, r.rdfcut, r.boyl, r.bozl, r.sclx, r.scly,
                      r.sclz] + list(r.scm) + list(r.box_extra), "<f8").tobytes(),
            np.array(list(r.times) + [0.0] * (11 - len(r.times)), "<f8").tobytes(),
            np.stack([r.sx, r.sy, r.sz], axis=1).astype("<f8").tobytes(),
            np.stack([r.vx, r.vy, r.vz], axis=1).astype("<f8").tobytes()]
    if r.av is not None:
        recs.append(np.stack([r.av, r.aw], axis=1).astype("<f8").tobytes())
        recs.extend(np.asarray(h, "<f8").tobytes() for h in r.hist)
    recs.extend(r.tail)
    tmp = path + ".part"
    with open(tmp, "wb") as f:
        for p in recs:
            f.write(_frame(p))
    os.replace(tmp, path)


def restart_from_state(system, state, thermo, nstep: int = 0, nsttot: int = 0,
                       tim: float = 0.0, times=None, av=None, aw=None, hist=None,
                       label: str = LABEL) -> RestartFile:
    """A restart record of a System and a state (positions, momenta) and
    mdx_thermo as the library returns them."""
    sx, sy, sz, vx, vy, vz = state
    nt = system.ntypes
    nnav = len(av) if av is not None else 0
    return RestartFile(
        label=label, nop=system.nop, ntypes=nt, nstot=system.nstot, nnav=nnav,
        dt=system.unitt, nstep=nstep, nsttot=nsttot, nstepa=nsttot, navt=0,
        nhist=len(hist) if hist else 0, tim=tim, tima=tim,
        sc=thermo.sc, scl=thermo.scl, boxl=thermo.boxl, vol=thermo.vol, rdfcut=0.0,
        boyl=thermo.boyl, bozl=thermo.bozl, sclx=thermo.sclx, scly=thermo.scly,
        sclz=thermo.sclz, scm=[thermo.scm[t] for t in range(nt)], box_extra=[0.0],
        times=list(times) if times is not None else [0.0] * 11,
        sx=np.asarray(sx), sy=np.asarray(sy), sz=np.asarray(sz),
        vx=np.asarray(vx), vy=np.asarray(vy), vz=np.asarray(vz),
        av=None if av is None else np.asarray(av), aw=None if aw is None else np.asarray(aw),
        hist=list(hist or []))


def thermo_of(r: RestartFile, system):
    """mdx_thermo with the thermostat and box state of a restart file."""
    from .abi import MdxThermo
    th = MdxThermo()
    th.sc, th.scl, th.sclx, th.scly, th.sclz = r.sc, r.scl, r.sclx, r.scly, r.sclz
    for t, v in enumerate(r.scm[:system.ntypes]):
        th.scm[t] = v
    th.boxl, th.boyl, th.bozl = r.boxl, r.boyl, r.bozl
    th.vol = r.boxl * r.boyl * r.bozl
    return th


# ------------------------------------------------------------ trajectory --
class TraceWriter:
    """TRACE (restart.f:425-598).  itrek 2: XMOL coordinates; 4: with
    velocities (A/fs); 6: with forces (kJ/mol/A); 8: both; odd itrek: the
    binary form (coordinates, and velocities when itrek > 2).  A new file
    (name + 3-digit number, as the reference's FTRK) after ltrek
    configurations."""

    def __init__(self, system, base: str, itrek: int = 2, ltrek: int = 1000,
                 listed=None):
        self.s = system
        self.base = base
        self.itrek = itrek
        self.ltrek = ltrek
        self.listed = list(listed) if listed is not None else [1] * system.ntypes
        self.ntrkf = 0
        self.ntrkz = 0
        self.f = None
        self.names = [n[:2] for t in system.types for n in (st["name"] for st in t["sites"])]
        self.files: List[str] = []

    def _open(self):
        if self.f:
            self.f.close()
        self.ntrkf += 1
        self.ntrkz = 0
        name = f"{self.base}.{self.ntrkf:03d}"
        self.files.append(name)
        if self.itrek % 2:
            self.f = open(name, "wb")
            s = self.s
            ivel = 0 if self.itrek <= 2 or self.itrek == 5 else 1
            head = struct.pack("<id3ddi", ivel, s.unitt, s.boxl, s.boyl, s.bozl, s.unitl,
                               s.ntypes)
            for t in range(s.ntypes):
                head += struct.pack("<3i", int(s.nspec[t]), int(s.nsits[t]), 1)
            self.f.write(_frame(head))
            for t in range(s.ntypes):
                m = np.array([st["mass"] for st in s.types[t]["sites"]], "<f8")
                self.f.write(_frame(m.tobytes() + struct.pack("<i", self.listed[t])))
        else:
            self.f = open(name, "w")

    def add(self, state, time_s: float, box, forces=None, temp=0.0, tryck=0.0, poten=0.0,
            cumtim=0.0):
        """One configuration.  state = (sx, sy, sz, vx, vy, vz) with the
        reference's momenta; forces (N x 3, internal units) for itrek 6/8."""
        if self.f is None or self.ntrkz >= self.ltrek:
            self._open()
        self.ntrkz += 1
        s = self.s
        sx, sy, sz, vx, vy, vz = state
        sel = np.repeat(np.array(self.listed, bool)[:s.ntypes], s.nspec * s.nsits)
        vfac = s.massdi * 1.0e-15 / s.unitt  # momenta -> A/fs
        if self.itrek % 2 == 0:
            out = [f"{int(sel.sum()):12d}\n",
                   " after %15.2f fs, BOX: %12.4f%12.4f%12.4f\n" % (time_s * 1e15, *box)]
            tokj = s.enerf * 1.0e-3 if hasattr(s, "enerf") else 1.0
            for i in np.nonzero(sel)[0]:
                nm = self.names[s.nsite[i] - 1].ljust(2)
                line = "%s %8.3f %8.3f %8.3f" % (nm, sx[i], sy[i], sz[i])
                if self.itrek in (4, 8):
                    v = (vx[i] * vfac[i], vy[i] * vfac[i], vz[i] * vfac[i])
                if self.itrek == 4:
                    line += " %11.5f %11.5f %11.5f" % v
                elif self.itrek == 6:
                    line += "%14.6E%14.6E%14.6E" % tuple(tokj * forces[i])
                elif self.itrek == 8:
                    line += "%14.6E%14.6E%14.6E" % v
                    line += " %11.5f %11.5f %11.5f" % tuple(tokj * forces[i])
                out.append(line + "\n")
            self.f.write("".join(out))
        else:
            rec = struct.pack("<i2d3d3d", 0, time_s, cumtim, temp, tryck, poten, *box)
            rec += struct.pack(f"<{s.ntypes}i", *self.listed[:s.ntypes])
            self.f.write(_frame(rec))
            ivel = 0 if self.itrek <= 2 or self.itrek == 5 else 1
            for t in range(s.ntypes):
                if not self.listed[t]:
                    continue
                a, b = int(s.isaddr[t]), int(s.isaddr[t + 1])
                self.f.write(_frame(np.concatenate([sx[a:b], sy[a:b], sz[a:b]]).astype("<f4")
                                    .tobytes()))
                if ivel:
                    v = [vx[a:b] * vfac[a:b], vy[a:b] * vfac[a:b], vz[a:b] * vfac[a:b]]
                    self.f.write(_frame(np.concatenate(v).astype("<f4").tobytes()))

    def close(self):
        if self.f:
            self.f.close()
            self.f = None


# ---------------------------------------------------- device snapshots --
class SnapshotDumper:
    """Restart dumps and trajectory frames written from device state off the
    step loop.  ``request(kind, **meta)`` queues ``mdx_snapshot`` on the
    context's stream (an asynchronous copy into pinned buffers, ordered after
    the steps already queued) and returns; a writer thread waits for that
    copy (``mdx_snapshot_wait``) and writes the file.  kind is "restart"
    (meta: path, nstep, nsttot, tim) or "trace" (meta: time_s), with a
    TraceWriter given at construction for the latter.  Buffers rotate over
    ``depth`` slots; a request waits only when every slot is still being
    written."""

    def __init__(self, path, trace: Optional[TraceWriter] = None, depth: int = 2):
        import torch  # pinned host memory
        from .abi import MdxThermo
        self.p = path
        self.L = path.L
        self.n = path.n
        self.trace = trace
        self.depth = depth
        self.bufs = [[torch.empty(self.n, dtype=torch.float64, pin_memory=True)
                      for _ in range(6)] for _ in range(depth)]
        # thermostat state lands in page-locked memory too (a copy into
        # pageable memory would wait for the stream)
        self.thbuf = [torch.empty(C.sizeof(MdxThermo), dtype=torch.uint8, pin_memory=True)
                      for _ in range(depth)]
        self.th = [MdxThermo.from_address(b.data_ptr()) for b in self.thbuf]
        self.free = queue.Queue()
        for k in range(depth):
            self.free.put(k)
        self.work = queue.Queue()
        self.errors: List[BaseException] = []
        self.written: List[str] = []
        self.t = threading.Thread(target=self._run, daemon=True)
        self.t.start()

    def _ptrs(self, k):
        from .abi import F64P
        return [C.cast(C.c_void_p(b.data_ptr()), F64P) for b in self.bufs[k]]

    def request(self, kind: str, **meta):
        k = self.free.get()
        rc = self.L.mdx_snapshot(self.p.h, k, *self._ptrs(k), C.byref(self.th[k]))
        if rc:
            self.free.put(k)
            self.p._check(rc)
        self.work.put((k, kind, meta))

    def _run(self):
        while True:
            item = self.work.get()
            if item is None:
                return
            k, kind, meta = item
            try:
                rc = self.L.mdx_snapshot_wait(self.p.h, k)
                if rc:
                    raise RuntimeError(f"mdx_snapshot_wait: {rc}")
                st = [b.numpy().copy() for b in self.bufs[k]]
                th = self.th[k]
                if kind == "restart":
                    r = restart_from_state(self.p.system, st, th, nstep=meta.get("nstep", 0),
                                           nsttot=meta.get("nsttot", 0),
                                           tim=meta.get("tim", 0.0))
                    write_dmp(meta["path"], r)
                    self.written.append(meta["path"])
                else:
                    self.trace.add(st, meta.get("time_s", 0.0), (th.boxl, th.boyl, th.bozl),
                                   temp=th.temp, tryck=th.tryck)
            except BaseException as e:  # reported by close()
                self.errors.append(e)
            finally:
                self.free.put(k)

    def close(self):
        self.work.put(None)
        self.t.join()
        if self.trace:
            self.trace.close()
        if self.errors:
            raise self.errors[0]
