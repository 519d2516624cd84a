"""Benchmark of the MDynaMix step on GB300.

Workload (one GPU): 32,768 flexible SPC-FW waters, 98,304 atoms, cubic box
99.336 A at 1.0 g/cm3, double time step 0.2/2 fs (NFREQ 10), Nose-Hoover NVT
300 K, R_cutoff 12 A, R_short 5 A, Ewald alpha 0.25/A with |n| <= 20 per axis
(16,700 k-vectors), neighbour lists refreshed every 10 long steps, seeded
jittered lattice start.  A step is one long step (DOUBLE, mdstep.f:324-436).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Our arm: the FP64 drop-in (value) and the mixed-precision path (``mixed``)
run the same workload; both numbers go on one JSON line with the mixed path's
force error against FP64.  ``e2e`` drives the C ABI with pinned host buffers:
every step uploads positions and momenta and downloads them again.
Reference arm (--impl reference): the CPU restatement of the reference's
routines (oracle/), all host threads, timed on the same workload.
Under torchrun each rank runs its own replica (the path does not shard).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "atom-steps/s mixed vs FP64 on GB300 at ≤1e-5 force err; p50/p99 job latency"
UNIT = "atom-steps/s"
WORKLOAD = dict(workload="SPC-FW water 32768 molecules (98304 atoms), DOUBLE 0.2/2 fs, "
                         "NVT 300 K, Rc 12 A, Ewald alpha 0.25/A |n|<=20",
                atoms=98304, nkv=16700, nfreq=10, ichnb=10, rcut=12.0, rshort=5.0,
                l2="working set > L2 (long rows 266 MB, phase tables 98 MB per step)",
                list_mode="reference (list at Rc, refresh every 10 long steps)")

# Algorithmic work per unit of each kernel group (frozen constants; an add,
# sub or mul counts 1, an FMA 2, sqrt / reciprocal / exp / sin / cos 1 each).
OPS_PAIR = 80            # per listed pair evaluated (forces.f:1071-1198)
# Reciprocal Ewald (forces.f:1286-1331) as the GPU passes walk the k-set:
# columns of fixed (nx, ny), each nz = +p and -p taken together.
OPS_EW_PAIR = 24         # per (paired record, atom): S(k) 4 FMA + forces 8 FMA
OPS_EW_COL = 23          # per (column, atom): X Y twice, Im(T U), Im(T V), F
OPS_EW_ROW = 8           # per (phase-table row, atom): recurrence step + charge
OPS_EW_K = 20            # per k-vector (energy, virial, W)
# The same work in the scope table's frozen per-(k, atom) count (a per-k
# loop: phase 5, sin + cos 2, q x 2, S accumulate 2, force 10) + 20 per k;
# the paired-record passes above do about half the multiply-adds of that
# loop, so this count reads higher for the same time.
OPS_EW_FROZEN_KATOM = 21

# DRAM bytes per long step of each group, from ncu captures of
# `python bench.py --only {fp64,mixed} --steps 2 --warmup 3`
# (dram__bytes_read.sum + dram__bytes_write.sum of every launch of the
# group's kernels in one long step, MB).
# fp64 ewald: k_tables 43.4 + k_sfac 126.0 + k_sfac_sum 51.3 + k_kterms 1.0
#             + k_wpairs 0.6 + k_rforce64 102.9
# mixed ewald: k_tables 4.7 + k_zimages 18.0 + k_sfac32 53.7 + k_sfac_sum 32.4
#              + k_kterms 1.0 + k_wtiles 0.6 + k_rforce_tc 75.4
# fp64 pair: 9 x 30.7 (short, forces) + 30.7 (short, energies) + 153.1 (long)
# mixed pair: 9 x 25.9 (short, forces) + 25.9 (short, energies) + 283.2 (long)
TRAFFIC_MB = {
    ("fp64", "ewald"): 325.2, ("mixed", "ewald"): 185.8,
    ("fp64", "pair"): 459.9, ("mixed", "pair"): 542.1,
}


def env_rank():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


class Clocks:
    """nvidia-smi samples during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        fd, self.path = tempfile.mkstemp(prefix="mdx_clocks_", suffix=".csv")
        os.close(fd)

    def __enter__(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}",
                 "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.fh, stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        try:
            rows = [r.split(",") for r in open(self.path).read().strip().splitlines()]
            os.unlink(self.path)
        except OSError:
            rows = []
        rows = [[c.strip() for c in r] for r in rows if len(r) >= 8]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[0]) for r in rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[4 + k] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons, "samples": len(rows)}


def make_system():
    from mdynamix_gb300 import system as S
    s = S.System(S.spcfw_water())
    st = S.make_configuration(s, seed=1, jitter=0.05)
    return s, st


def roofline_of(timers, mbsh, mbln, nfreq, kset, n, peak64, peak32, prec, nsteps):
    """Roofline of the dominant kernel group of one long step: reciprocal
    Ewald (phase tables, S(k), per-k terms, forces) or the real-space pair
    loops (NFREQ short-list passes + one long-list pass).  Ops per long step
    from the frozen per-unit constants; time from the device timers (CUDA
    events on the launching stream) of the instrumented pass, per long
    step; peak = measured FMA throughput of the pipe the path computes on."""
    ms = {k: v[0] / nsteps for k, v in timers.items()}
    nkv, ncol, npair, rows = kset
    ew_kernels = ("k_tables + k_zimages + k_sfac32 + k_sfac_sum + k_kterms + k_wtiles + "
                  "k_rforce_tc (TF32 tensor cores)" if prec == "mixed" else
                  "k_tables + k_sfac + k_sfac_sum + k_kterms + k_wpairs + k_rforce64")
    groups = {
        "ewald": (ms["ew_tables"] + ms["ew_sfac"] + ms["ew_kterms"] + ms["ew_force"],
                  (OPS_EW_PAIR * npair + OPS_EW_COL * ncol + OPS_EW_ROW * rows) * n
                  + OPS_EW_K * nkv, ew_kernels),
        "pair": (ms["pair_short"] + ms["pair_long"], OPS_PAIR * (nfreq * mbsh + mbln),
                 "k_pair (short list x NFREQ, long list x 1)"),
    }
    top = max(groups, key=lambda g: groups[g][0])
    t_ms, ops, kernels = groups[top]
    achieved = ops / (t_ms * 1e-3) / 1e12
    peak = peak64 if prec == "fp64" else peak32
    tr = TRAFFIC_MB.get((prec, top))
    share = t_ms / sum(ms.values())
    other = {g: {"ms_per_long_step": v[0], "ops_per_long_step": v[1],
                 "achieved_tflops": v[1] / (v[0] * 1e-3) / 1e12,
                 "traffic": (TRAFFIC_MB.get((prec, g)) or 0) * 1e6, "kernels": v[2]}
             for g, v in groups.items()}
    frozen = OPS_EW_FROZEN_KATOM * nkv * n + OPS_EW_K * nkv if top == "ewald" else ops
    return {"bound": "fp64" if prec == "fp64" else "fp32", "achieved": achieved, "peak": peak,
            "unit": "TFLOP/s", "frac": achieved / peak if peak else None,
            "traffic": tr * 1e6 if tr is not None else None,
            "kernel": f"{top}: {kernels}", "ms_per_long_step": t_ms, "share_of_step": share,
            "ops_per_long_step": ops,
            "frozen": {"ops_per_long_step": frozen,
                       "achieved": frozen / (t_ms * 1e-3) / 1e12,
                       "frac": frozen / (t_ms * 1e-3) / 1e12 / peak if peak else None},
            "groups": other,
            "peak_source": "measured in-run FMA probe (mdx_probe_fma_peak, of measured)"}


def max_over_ranks(value: float, dist, device) -> float:
    """The largest of the ranks' values (each replica's timed region: the job
    takes as long as its slowest rank); the value itself on one rank."""
    if not dist:
        return float(value)
    import torch
    t = torch.tensor([float(value)], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_rate(world: int, atoms: int, steps: int, ms: float) -> float:
    """Whole-job atom-steps/s of ``world`` replicas of ``atoms`` atoms, each
    running ``steps`` long steps, the slowest taking ``ms``."""
    return world * atoms * steps / (ms * 1e-3)


def run_gpu(args, rank, world, local):
    import torch
    from mdynamix_gb300.abi import MDX_FP64, MDX_MIXED
    from mdynamix_gb300.mdx import ForcePath, probe_fma_peak

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist:
            dist.barrier()

    if args.only == "pimd":
        from mdynamix_gb300 import system as S
        from mdynamix_gb300.mdx import PimdPath
        sp = S.System(S.pimd_water(nwater=256, nbeads=32))
        pp = PimdPath(sp, S.pimd_beads(sp, seed=5), precision=MDX_MIXED)
        pp.run(args.warmup)
        pp.steps(args.steps, args.warmup)
        pp.close()
        return None
    s, st = make_system()
    n = s.nstot
    out = {}
    if args.only:
        g = ForcePath(s, precision=MDX_FP64 if args.only == "fp64" else MDX_MIXED)
        g.set_state(*st)
        g.double(0)
        g.double_steps(args.warmup + args.steps, 0, records=False)
        g.sync()
        return None
    for prec in ("fp64", "mixed"):
        g = ForcePath(s, precision=MDX_FP64 if prec == "fp64" else MDX_MIXED)
        g.set_state(*st)
        g.double(0)                       # prologue: CHCNB, GETCOM, SLFORCES, FFORCES
        g.double_steps(args.warmup, 0, records=False)
        stream = torch.cuda.ExternalStream(g.stream)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        barrier()
        torch.cuda.synchronize()
        l0 = g.launches
        with Clocks(local) as clk:
            e0.record(stream)
            g.double_steps(args.steps, args.warmup, records=False)
            e1.record(stream)
            torch.cuda.synchronize()
        barrier()
        ms = max_over_ranks(e0.elapsed_time(e1), dist, "cuda")
        launches = g.launches - l0
        # instrumented pass: per-group device time (CUDA events on the same stream)
        g.set_timers(True)
        g.timers()
        g.double_steps(args.steps, args.warmup + args.steps, records=False)
        tm = g.timers()
        g.set_timers(False)
        out[prec] = dict(ms=ms, launches=launches, timers=tm, clocks=clk.summary(), ctx=g,
                         path=g.path_info())
    # the same workload with the 1.5 A Verlet skin (rows to 13.5 A, pairs
    # beyond 12 A skipped, rebuilt after 0.75 A of travel)
    skin = {}
    if args.skin:
        from mdynamix_gb300 import system as S
        import dataclasses
        s_skin = S.System(dataclasses.replace(s.spec, rskin=1.5))
        for prec in ("fp64", "mixed"):
            g = ForcePath(s_skin, precision=MDX_FP64 if prec == "fp64" else MDX_MIXED)
            g.set_state(*st)
            g.double(0)
            g.double_steps(args.warmup, 0, records=False)
            stream = torch.cuda.ExternalStream(g.stream)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            _, th0 = g.get_state()
            e0.record(stream)
            g.double_steps(args.steps, args.warmup, records=False)
            e1.record(stream)
            torch.cuda.synchronize()
            _, th1 = g.get_state()
            skin[prec] = dict(ms=max_over_ranks(e0.elapsed_time(e1), dist, "cuda"),
                              builds=th1.list_builds - th0.list_builds)
            g.close()
    # list sizes and force error at the shared start state
    g64 = ForcePath(s, precision=MDX_FP64)
    g32 = ForcePath(s, precision=MDX_MIXED)
    for g in (g64, g32):
        g.set_state(*st)
        mbsh, mbln = g.chcnb()
        g.getcom()
        g.last_allforce = g.allforce()
    f64, f32 = g64.forces(3), g32.forces(3)
    g32.close()
    ferr = float(np.sqrt(((f32 - f64) ** 2).sum() / (f64 ** 2).sum()))
    ferr_max = float(np.abs(f32 - f64).max() / np.abs(f64).max())
    # e2e through the C ABI with pinned host buffers
    g = out["fp64"]["ctx"]
    pinned = [torch.empty(n, dtype=torch.float64, pin_memory=True).numpy() for _ in range(6)]
    (x, y, z, vx, vy, vz), th = g.get_state()
    for a, b in zip(pinned, (x, y, z, vx, vy, vz)):
        a[:] = b
    ke = max(2, min(args.steps, 10))
    mstep = 2 * args.steps + args.warmup

    def e2e_step(k):
        # upload positions and momenta, one long step with its record, and
        # download them again, host buffers page-locked
        nonlocal th
        g.set_state(*pinned, thermo=th)
        g.double_steps(1, mstep + k, records=True)
        _, th = g.get_state(out=pinned)

    e2e_step(0)  # warm-up: the step graph with records is captured here
    barrier()
    t0 = time.perf_counter()
    for k in range(ke):
        e2e_step(1 + k)
    e2e_s = max_over_ranks((time.perf_counter() - t0) / ke, dist, "cuda")
    peak64 = probe_fma_peak(True)
    peak32 = probe_fma_peak(False)
    from mdynamix_gb300.abi import MdxStepRecord
    import ctypes
    for prec in ("fp64", "mixed"):
        out[prec]["ctx"].close()
    return dict(rec_bytes=ctypes.sizeof(MdxStepRecord), out=out, n=n, mbsh=mbsh, mbln=mbln, ferr=ferr, ferr_max=ferr_max,
                e2e_s=e2e_s, e2e_steps=ke, peak64=peak64, peak32=peak32, dist=dist,
                kset=(s.kvector_count(),) + s.kcolumn_counts(), nfreq=s.spec.nfreq, skin=skin,
                g64=g64)


def serving_leg(args):
    """Continuous batching of solvation jobs (a bounded sample of the
    256-job stream): Poisson arrivals, 5 coupling states per job, admission
    by slots and HBM budget, p50/p99 latency from arrival to completion."""
    from mdynamix_gb300 import serve
    from mdynamix_gb300.abi import MDX_FP64, MDX_MIXED
    out = {}
    jobs = serve.solvation_stream(args.serve_jobs, rate=args.serve_rate, seed=11,
                                  steps_per_state=args.serve_steps)
    preps = [serve.prepare(j) for j in jobs]          # request preprocessing (host)
    warm = serve.Server(precision=MDX_MIXED, slots=4)  # first-use costs (module load)
    warm.run([serve.prepare(serve.JobSpec("warm", jobs[0].spec, steps_per_state=2))])
    for name, prec in (("mixed", MDX_MIXED), ("fp64", MDX_FP64)):
        srv = serve.Server(precision=prec, slots=args.serve_slots)
        t0 = time.perf_counter()
        res = srv.run(preps)
        wall = time.perf_counter() - t0
        st = serve.latency_stats(res, wall)
        st["peak_resident_jobs"] = srv.peak_resident
        out[name] = st
    atoms = [p.system.nstot for p in preps]
    out["sample"] = (f"{len(preps)} jobs of {min(atoms)}-{max(atoms)} atoms (one solute in water), "
                     f"Poisson arrivals at {args.serve_rate}/s, 5 coupling states x "
                     f"{args.serve_steps} DOUBLE long steps per job, up to {args.serve_slots} "
                     f"resident; latency = completion - arrival")
    out["speedup_mixed_vs_fp64"] = out["mixed"]["atom_steps_per_s"] / out["fp64"]["atom_steps_per_s"]
    return out


def pimd_leg(args):
    """Path-integral water: 256 SPC-FW x 32 bead replicas (24,576 bead
    atoms), dt 0.25 fs, bead thermostats; a bounded sample of long steps per
    precision, and the mixed path's force error against FP64 after the
    preparation."""
    import torch
    from mdynamix_gb300 import system as S
    from mdynamix_gb300.abi import MDX_FP64, MDX_MIXED
    from mdynamix_gb300.mdx import PimdPath
    s = S.System(S.pimd_water(nwater=256, nbeads=32))
    states = S.pimd_beads(s, seed=5)
    out = {}
    paths = {}
    for name, prec in (("mixed", MDX_MIXED), ("fp64", MDX_FP64)):
        pp = PimdPath(s, states, precision=prec)
        pp.run(args.pimd_warmup)
        torch.cuda.synchronize()
        stream = torch.cuda.ExternalStream(pp.stream)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        recs = pp.steps(args.pimd_steps, args.pimd_warmup)
        e1.record(stream)
        torch.cuda.synchronize()
        dt = e0.elapsed_time(e1) * 1e-3
        atoms = s.nstot * s.spec.nbeads
        out[name] = {"atom_steps_per_s": atoms * args.pimd_steps / dt,
                     "ms_per_step": dt / args.pimd_steps * 1e3,
                     "temp_last": recs[-1].temp, "qek_last": recs[-1].qek}
        paths[name] = pp
    # force error of the mixed path on identical bead coordinates
    g64 = PimdPath(s, states, precision=MDX_FP64)
    g32 = PimdPath(s, states, precision=MDX_MIXED)
    g64.run(0)
    g32.run(0)
    num = den = 0.0
    for a, b in zip(g32.beads, g64.beads):
        fa = a.forces(1) + a.forces(2)
        fb = b.forces(1) + b.forces(2)
        num += float(((fa - fb) ** 2).sum())
        den += float((fb ** 2).sum())
    out["force_err_rms_mixed_vs_fp64"] = math.sqrt(num / den)
    out["speedup_mixed_vs_fp64"] = out["mixed"]["atom_steps_per_s"] / out["fp64"]["atom_steps_per_s"]
    out["sample"] = (f"256 SPC-FW waters x 32 beads (24576 bead atoms), Rc 9 A, alpha 0.35/A, "
                     f"dt 0.25 fs, PI_thermo 300 K / 5 fs / chains of 4; {args.pimd_warmup} "
                     f"steps with the preparation, then {args.pimd_steps} timed long steps "
                     f"(CUDA events on the bead ensemble's stream)")
    for pp in list(paths.values()) + [g64, g32]:
        pp.close()
    return out


def bilayer_leg(args):
    """DMPC bilayer in SPC water (98 lipids, 3655 waters), anisotropic NPT
    with SHAKE (SULTAN): mixed-path force, energy and virial errors against
    FP64 on the same configuration, and a bounded sample of long steps per
    precision."""
    import torch
    from mdynamix_gb300 import system as S
    from mdynamix_gb300.abi import MDX_FP64, MDX_MIXED
    from mdynamix_gb300.mdx import ForcePath
    s = S.System(S.dmpc_bilayer(shake_hbonds=True))
    st = S.bilayer_configuration(s, seed=1)
    out = {}
    sc = {}
    f = {}
    for name, prec in (("fp64", MDX_FP64), ("mixed", MDX_MIXED)):
        g = ForcePath(s, precision=prec)
        g.set_state(*st)
        g.chcnb()
        g.getcom()
        sc[name] = g.allforce()
        f[name] = g.forces(3)
        g.sultan(args.bilayer_warmup)
        torch.cuda.synchronize()
        stream = torch.cuda.ExternalStream(g.stream)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        g.sultan_steps(args.bilayer_steps, args.bilayer_warmup, records=False)
        e1.record(stream)
        torch.cuda.synchronize()
        dt = e0.elapsed_time(e1) * 1e-3
        out[name] = {"atom_steps_per_s": s.nstot * args.bilayer_steps / dt,
                     "ms_per_step": dt / args.bilayer_steps * 1e3}
        g.close()
    a, b = f["mixed"], f["fp64"]
    err = {"force_rms": float(np.sqrt(((a - b) ** 2).sum() / (b ** 2).sum()))}
    for n in ("pe1", "pe2", "pels1", "pels2", "spe", "pint"):
        x, y = getattr(sc["mixed"], n), getattr(sc["fp64"], n)
        err[n] = abs(x - y) / max(abs(y), 1e-300)
    vm = sc["mixed"].vir1 + sc["mixed"].vir2 + sc["mixed"].virb
    vf = sc["fp64"].vir1 + sc["fp64"].vir2 + sc["fp64"].virb
    err["virial"] = abs(vm - vf) / abs(vf)
    out["mixed_vs_fp64_rel_err"] = err
    out["speedup_mixed_vs_fp64"] = out["mixed"]["atom_steps_per_s"] / out["fp64"]["atom_steps_per_s"]
    out["sample"] = (f"{s.nspec[0]} DMPC + {s.nspec[1]} SPC ({s.nstot} atoms), box "
                     f"{s.boxl:.0f}x{s.boyl:.0f}x{s.bozl:.0f} A, Rc 12, Ewald 3.12/9.72, SHAKE on "
                     f"bonds to H, "
                     f"anisotropic NPT 303 K / 1 bar, dt 2 fs; {args.bilayer_warmup} + "
                     f"{args.bilayer_steps} timed SULTAN steps (CUDA events on the stream)")
    return out


def nve_run(prec, s, st, th, nsteps, mstep0):
    """NVE DOUBLE long steps from a given state: per-step total energy
    (PE1 + PE2 + PELS1 + PELS2 + SPE + PINT + TKE, as the reference's
    output sums them) and kinetic energy."""
    from mdynamix_gb300.mdx import ForcePath
    g = ForcePath(s, precision=prec)
    p = g.packed.params
    p.lnvt = 0
    g.set_params(p)
    th.sc = 0.0
    g.set_state(*st, thermo=th)
    rec = g.double(nsteps, mstep0)
    g.close()
    e = np.array([r.pe1 + r.pe2 + r.pels1 + r.pels2 + r.spe + r.pint + r.tke for r in rec])
    ke = np.array([r.tke for r in rec])
    return e, ke


NVE_SEEDS = (3, 7, 11)


def nve_leg(args):
    """NVE energy conservation of both paths, each pair of runs from the same
    equilibrated state (1000 SPC-FW waters, DOUBLE 0.2/2 fs, Rc 9 A), three
    starts: linear drift of the total energy and its RMS fluctuation over
    the run, per start and averaged.  (The FP64 equilibration sums forces
    with atomics, so a start differs from run to run in its last bits, and
    the drift of a single 1 ps run moves with it.)"""
    from mdynamix_gb300 import system as S
    from mdynamix_gb300.abi import MDX_FP64, MDX_MIXED
    from mdynamix_gb300.mdx import ForcePath
    spec = S.RunSpec(molecules=[("SPC-FW", 1000)], density=1.0, dt_fs=2.0, nfreq=10,
                     rcut=9.0, rshort=5.0, alpha=2.8, fexp=12.0, ichnb=10, nvt=(300.0, 30.0))
    s = S.System(spec)
    t = np.arange(args.nve_steps) * s.spec.dt_fs * 1e-3  # ps
    per = {"fp64": [], "mixed": []}
    for seed in NVE_SEEDS:
        st = S.make_configuration(s, seed=seed, jitter=0.05)
        g = ForcePath(s, precision=MDX_FP64)
        g.set_state(*st)
        g.double(args.nve_equil, records=False)
        state, th = g.get_state()
        g.close()
        for name, prec in (("fp64", MDX_FP64), ("mixed", MDX_MIXED)):
            e, ke = nve_run(prec, s, state, th, args.nve_steps, args.nve_equil)
            slope = float(np.polyfit(t, e, 1)[0])
            per[name].append((slope / float(ke.std()), float(e.std() / ke.std())))
    out = {}
    for name, v in per.items():
        out[name] = {"drift_per_ps_over_ke_rms": float(np.mean([a for a, _ in v])),
                     "etot_rms_over_ke_rms": float(np.mean([b for _, b in v])),
                     "per_start": [[round(a, 4), round(b, 4)] for a, b in v]}
    out["units"] = ("linear drift of the total energy per ps and its RMS fluctuation, "
                    "both divided by the RMS fluctuation of the kinetic energy")
    out["sample"] = (f"{s.nstot} atoms, starts from seeds {list(NVE_SEEDS)}: "
                     f"{args.nve_equil} NVT long steps, then {args.nve_steps} NVE long steps "
                     f"(2 fs) per path from each start")
    return out


def cpu_baseline_and_parity(s, st, threads, g64):
    """The oracle (restated reference routines) on the same workload: one
    CHCNB and one long step, the list build amortised over ICHNB steps; and,
    on the way, the parity check of the FP64 GPU path at this size: lists
    bit for bit, ALLFORCE forces, energies and virials at the start state."""
    import oracle
    o = oracle.Oracle(s, threads=threads)
    o.set_state(*st)
    t0 = time.perf_counter(); counts = o.chcnb(); t_list = time.perf_counter() - t0
    par = {"lists_bit_exact": None}
    if g64 is not None:
        (gs1, gs2), (gl1, gl2) = g64.lists()
        (os1, os2), (ol1, ol2) = o.lists()
        par["lists_bit_exact"] = bool(
            g64.counts == counts and np.array_equal(gs1, os1) and np.array_equal(gs2, os2)
            and np.array_equal(gl1, ol1) and np.array_equal(gl2, ol2))
        del gs1, gs2, gl1, gl2, os1, os2, ol1, ol2
    o.getcom()
    b = o.allforce()
    if g64 is not None:
        fo = o.forces(3)
        fg = g64.forces(3)
        a = g64.last_allforce
        par["force_rel_max"] = float(np.abs(fg - fo).max() / np.abs(fo).max())
        par["scalar_rel_max"] = float(max(
            abs(getattr(a, n) - getattr(b, n)) / abs(getattr(b, n))
            for n in ("pe1", "pels1", "pe2", "pels2", "spe", "pint", "vir1", "vir2", "virb",
                      "virx", "viry", "virz", "wirs", "wirss") if getattr(b, n) != 0.0))
        par["pairs"] = {"short": int(counts[0]), "long": int(counts[1])}
        par["tolerance"] = 1e-10
    t0 = time.perf_counter(); o.double_steps(1, 0); t_step = time.perf_counter() - t0
    per = t_step + t_list / s.spec.ichnb
    cpu = {"value": s.nstot / per, "unit": UNIT, "cores": threads, "kind": "port",
           "sample": f"1 long step ({t_step:.1f} s) + CHCNB ({t_list:.1f} s)/ICHNB, full "
                     f"98304-atom workload, C restatement -O2 OpenMP"}
    return cpu, par


def reference_arm(args, rank, world):
    if rank != 0:
        return
    import oracle
    s, st = make_system()
    threads = os.cpu_count() or 1
    o = oracle.Oracle(s, threads=threads)
    o.set_state(*st)
    t0 = time.perf_counter(); o.chcnb(); t_list = time.perf_counter() - t0
    o.getcom(); o.slforces(); o.fforces()
    w = min(args.warmup, 3)  # warm-up long steps (2-3 s each on the CPU), at most three
    if w:
        o.double_steps(w, 0)
    # bounded sample: at most ~3 minutes of timed CPU work
    t0 = time.perf_counter(); o.double_steps(1, w); t1 = time.perf_counter() - t0
    k = max(1, min(args.steps - 1, int(150.0 / max(t1, 1e-3))))
    t0 = time.perf_counter(); o.double_steps(k, w + 1); tk = time.perf_counter() - t0
    steps = k + 1
    per = (t1 + tk) / steps + t_list / s.spec.ichnb
    v = s.nstot / per
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": steps,
            "warmup": w, "ms_per_step": per * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": dict(WORKLOAD, parallelism="cpu threads"), "impl": "reference",
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{steps} DOUBLE long steps of the full workload + "
                                       f"CHCNB ({t_list:.1f} s) amortised over ICHNB=10; "
                                       f"C restatement of the reference routines, OpenMP"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _r(x, sig=4):
    """Round floats (recursively) to sig significant digits for the line."""
    if isinstance(x, float):
        return float(f"{x:.{sig}g}") if math.isfinite(x) else x
    if isinstance(x, dict):
        return {k: _r(v, sig) for k, v in x.items()}
    if isinstance(x, (list, tuple)):
        return [_r(v, sig) for v in x]
    return x


def extra_legs(args):
    """Evidence runs printed as their own JSON lines (not part of the
    default run): the plain-method case's NVE run and the reference
    sample's statistics."""
    import torch  # noqa: F401  (CUDA context first)
    if "cfg1" in args.leg:
        print(json.dumps({"leg": "cfg1_nve", **_r(cfg1_nve_leg(args))}), flush=True)
    if "serving" in args.leg:
        a = argparse.Namespace(**vars(args))
        a.serve_jobs, a.serve_steps, a.serve_slots = 256, 500, 256
        out = serving_leg(a)
        print(json.dumps({"leg": "serving_256x5x500", **_r(out)}), flush=True)
    if "sample" in args.leg:
        from tests.nacl776 import reference_averages, sample_run_averages
        from mdynamix_gb300.abi import MDX_FP64, MDX_MIXED
        out = {"reference_4nacl_out": reference_averages()}
        for name, prec in (("fp64", MDX_FP64), ("mixed", MDX_MIXED)):
            t0 = time.perf_counter()
            out[name] = sample_run_averages(prec)
            out[name + "_wall_s"] = time.perf_counter() - t0
        print(json.dumps({"leg": "sample_4nacl", **_r(out, 6)}), flush=True)


def cfg1_nve_leg(args):
    """512 rigid SPC/E + 4 Na+ + 4 Cl- (1544 atoms), SULTAN + SHEJK: SHAKE
    iterations at TOLER 1e-8 taken literally and at 1.4e-4; energy
    conservation over 1000 NVE steps (2 fs) after 1000 NVT steps from the
    lattice start, FP64 and mixed."""
    import dataclasses
    from mdynamix_gb300 import system as S
    from mdynamix_gb300.abi import MDX_FP64, MDX_MIXED
    from mdynamix_gb300.mdx import ForcePath
    out = {}
    for toler in (1e-8, 1.4e-4):
        s = S.System(dataclasses.replace(S.spce_nacl_nve(), toler=toler, nvt=(300.0, 30.0)))
        st = S.make_configuration(s, seed=1, jitter=0.05)
        g = ForcePath(s)
        g.set_state(*st)
        g.sultan(args.cfg1_equil, records=False)
        state, th = g.get_state()
        g.close()
        for name, prec in (("fp64", MDX_FP64), ("mixed", MDX_MIXED)):
            g = ForcePath(s, precision=prec)
            p = g.packed.params
            p.lnvt = 0
            g.set_params(p)
            th.sc = 0.0
            g.set_state(*state, thermo=th)
            t0 = time.perf_counter()
            rec = g.sultan(args.cfg1_steps, args.cfg1_equil)
            wall = time.perf_counter() - t0
            _, th_end = g.get_state()
            g.close()
            e = np.array([r.pe1 + r.pe2 + r.pels1 + r.pels2 + r.spe + r.pint + r.tke for r in rec])
            ke = np.array([r.tke for r in rec])
            t = np.arange(len(rec)) * 2e-3
            its = [r.shake_iter for r in rec]
            out[f"toler_{toler:g}_{name}"] = {
                "drift_per_ps_over_ke_rms": float(np.polyfit(t, e, 1)[0] / ke.std()),
                "etot_rms_over_ke_rms": float(e.std() / ke.std()),
                "shake_iter_mean": float(np.mean(its)), "shake_iter_max": int(max(its)),
                "molecules_past_maxit": int(th_end.shake_fail),
                "temp_mean": float(np.mean([r.temp for r in rec])),
                "atom_steps_per_s": s.nstot * len(rec) / wall}
    out["sample"] = (f"{args.cfg1_equil} NVT (300 K, 30 fs) steps from the seeded lattice, "
                     f"then {args.cfg1_steps} NVE steps per path; TOLER is squared by SHEJK")
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline and parity leg")
    ap.add_argument("--no-skin", dest="skin", action="store_false", help="skip the skin-mode leg")
    ap.add_argument("--serve-jobs", type=int, default=32, help="serving leg sample (0 = off)")
    ap.add_argument("--serve-steps", type=int, default=20, help="long steps per coupling state")
    ap.add_argument("--serve-rate", type=float, default=100.0, help="arrivals per second")
    ap.add_argument("--serve-slots", type=int, default=64)
    ap.add_argument("--pimd-steps", type=int, default=2000,
                    help="PIMD leg timed steps (config 5: 2000; 0 = off)")
    ap.add_argument("--pimd-warmup", type=int, default=3)
    ap.add_argument("--bilayer-steps", type=int, default=100, help="bilayer leg timed steps (0 = off)")
    ap.add_argument("--bilayer-warmup", type=int, default=3)
    ap.add_argument("--nve-steps", type=int, default=500, help="NVE leg long steps (0 = off)")
    ap.add_argument("--nve-equil", type=int, default=100)
    ap.add_argument("--leg", nargs="*", default=[], choices=["cfg1", "sample", "serving"],
                    help="evidence runs only (their own JSON lines, no headline line)")
    ap.add_argument("--cfg1-steps", type=int, default=1000)
    ap.add_argument("--cfg1-equil", type=int, default=1000)
    ap.add_argument("--detail", default=None, help="also write the full results to this file")
    ap.add_argument("--only", choices=["fp64", "mixed", "pimd"], default=None,
                    help="profiling runs: one precision (or the mixed PIMD ensemble of "
                         "the pimd leg), warm-up + steps only, no JSON line")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    rank, world, local = env_rank()
    if args.impl == "reference":
        reference_arm(args, rank, world)
        return
    if args.leg:
        if rank == 0:
            extra_legs(args)
        return
    r = run_gpu(args, rank, world, local)
    if r is None:
        return
    if rank != 0:
        if r["dist"]:
            r["dist"].destroy_process_group()
        return
    n = r["n"]
    o64, o32 = r["out"]["fp64"], r["out"]["mixed"]
    v64 = replica_rate(world, n, args.steps, o64["ms"])
    v32 = replica_rate(world, n, args.steps, o32["ms"])
    nfreq = r["nfreq"]
    roof = roofline_of(o64["timers"], r["mbsh"], r["mbln"], nfreq, r["kset"], n,
                       r["peak64"], r["peak32"], "fp64", args.steps)
    roof32 = roofline_of(o32["timers"], r["mbsh"], r["mbln"], nfreq, r["kset"], n,
                         r["peak64"], r["peak32"], "mixed", args.steps)
    serving = serving_leg(args) if args.serve_jobs > 0 else None
    pimd = pimd_leg(args) if args.pimd_steps > 0 else None
    bilayer = bilayer_leg(args) if args.bilayer_steps > 0 else None
    nve = nve_leg(args) if args.nve_steps > 0 else None
    cpu = parity = None
    if world == 1 and not args.no_cpu:
        s, st = make_system()
        cpu, parity = cpu_baseline_and_parity(s, st, os.cpu_count() or 1, r["g64"])
    r["g64"].close()
    dt_fs = 2.0
    full = {"roofline": roof, "mixed_roofline": roof32, "serving": serving, "pimd": pimd,
            "bilayer": bilayer, "nve": nve, "cpu_baseline": cpu, "parity": parity,
            "timers_ms_fp64": {k: v[0] / args.steps for k, v in o64["timers"].items()},
            "timers_ms_mixed": {k: v[0] / args.steps for k, v in o32["timers"].items()},
            "skin": r["skin"]}
    if args.detail:
        with open(args.detail, "w") as fh:
            json.dump(full, fh, indent=1)

    def roof_short(x):
        return {"bound": x["bound"], "achieved": x["achieved"], "peak": x["peak"],
                "unit": x["unit"], "frac": x["frac"], "traffic": x["traffic"],
                "kernel": x["kernel"].split(":")[0] + " group",
                "frac_frozen_ops": x["frozen"]["frac"], "ms_per_step": x["ms_per_long_step"],
                "share": x["share_of_step"]}

    skin = None
    if r["skin"]:
        k64, k32 = r["skin"]["fp64"], r["skin"]["mixed"]
        skin = {"rskin_A": 1.5,
                "fp64": replica_rate(world, n, args.steps, k64["ms"]),
                "mixed": replica_rate(world, n, args.steps, k32["ms"]),
                "list_builds": [k64["builds"], k32["builds"]]}
    line = {
        "metric": METRIC, "value": v64, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": o64["ms"] / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": dict(WORKLOAD, parallelism=f"replicas x{world}" if world > 1 else "single GPU"),
        "ns_per_day": v64 / n * dt_fs * 1e-6 * 86400,
        "mixed": {"value": v32, "ms_per_step": o32["ms"] / args.steps,
                  "speedup_vs_fp64": v32 / v64, "force_err_rms": r["ferr"],
                  "force_err_max_rel": r["ferr_max"],
                  "dtype": "f32 pair/bonded/Ewald products; S(k) f32 per slice, f64 across "
                           "slices; i64 fixed-point forces; f64 reductions and update",
                  "path": o32["path"], "roofline": roof_short(roof32),
                  "gpu_launches": o32["launches"], "clocks": o32["clocks"]},
        "roofline": roof_short(roof),
        "e2e": {"value": world * n / r["e2e_s"], "unit": UNIT,
                "h2d_bytes_per_step": 6 * n * 8,
                "d2h_bytes_per_step": 6 * n * 8 + r["rec_bytes"]},
        "gpu_launches": o64["launches"],
        "clocks": o64["clocks"],
        "parity": parity,
        "skin": skin,
        "cpu_baseline": cpu,
    }
    if serving:
        line["serving"] = {k: {"value": serving[k]["atom_steps_per_s"],
                               "p50_s": serving[k]["p50_s"], "p99_s": serving[k]["p99_s"]}
                           for k in ("mixed", "fp64")}
        line["serving"]["speedup"] = serving["speedup_mixed_vs_fp64"]
    if pimd:
        line["pimd"] = {"mixed": pimd["mixed"]["atom_steps_per_s"],
                        "fp64": pimd["fp64"]["atom_steps_per_s"],
                        "speedup": pimd["speedup_mixed_vs_fp64"],
                        "force_err_rms": pimd["force_err_rms_mixed_vs_fp64"]}
    if bilayer:
        line["bilayer"] = {"mixed": bilayer["mixed"]["atom_steps_per_s"],
                           "fp64": bilayer["fp64"]["atom_steps_per_s"],
                           "speedup": bilayer["speedup_mixed_vs_fp64"],
                           "force_err_rms": bilayer["mixed_vs_fp64_rel_err"]["force_rms"]}
    if nve:
        line["nve"] = {k: nve[k]["drift_per_ps_over_ke_rms"] for k in ("fp64", "mixed")}
    print(json.dumps(_r(line)), flush=True)
    if r["dist"]:
        r["dist"].destroy_process_group()


if __name__ == "__main__":
    main()
