"""mdx_slforces_static (no device allocation) against mdx_slforces, through
the C ABI.  Collected last so that it also runs after every other GPU test
in the same process (the static scratch is per process and per device)."""
import ctypes as C

import numpy as np
import pytest

from mdynamix_gb300.abi import MDX_FP64, MDX_MIXED, MdxScalars, thermo_init
from mdynamix_gb300.mdx import ForcePath
from mdynamix_gb300 import system as S
from tests import systems

pytestmark = pytest.mark.gpu

# Same kernels, same summation order, only the S(k) scratch lives elsewhere:
# the results agree to rounding (they are in fact bit-identical).
TOL = 1e-12          # relative to the largest |value| of each quantity
MDX_ERR_STATE = 7
MDX_ERR_UNSUPPORTED = 10
SCALARS = ("pe1", "pels1", "spe", "qpe", "vir1", "virx", "viry", "virz", "wirs")


def close(a, b):
    scale = max(np.abs(b).max(), 1e-300)
    return np.abs(np.asarray(a) - np.asarray(b)).max() <= TOL * scale


def memory(L):
    """(bytes in use, bytes reserved) of the device's default memory pool,
    which every context allocates from, and the device's free bytes."""
    used, res, free, tot = (C.c_size_t() for _ in range(4))
    assert L.mdx_pool_usage(C.byref(used), C.byref(res)) == 0
    assert L.mdx_device_memory(C.byref(free), C.byref(tot)) == 0
    return used.value, res.value, free.value


@pytest.mark.parametrize("precision", [MDX_FP64, MDX_MIXED])
def test_static_matches_slforces_twice(precision):
    s, st = systems.build(systems.spcfw(n=216))
    g = ForcePath(s, precision=precision)
    g.set_state(*st)
    g.chcnb()
    g.getcom()
    ref = g.slforces()                       # builds the k-set (allocates)
    g_ref = g.forces(2).copy()
    out = MdxScalars()                       # first call per device: module set-up
    assert g.L.mdx_slforces_static(g.h, C.byref(out)) == 0, g.L.mdx_last_error(g.h).decode()
    g.sync()
    before = memory(g.L)
    for call in range(2):                    # two calls in a row
        out = MdxScalars()
        rc = g.L.mdx_slforces_static(g.h, C.byref(out))
        assert rc == 0, g.L.mdx_last_error(g.h).decode()
        assert close(g.forces(2), g_ref), f"G differs on call {call}"
        for name in SCALARS:
            assert close(getattr(out, name), getattr(ref, name)), f"{name} on call {call}"
        assert out.nkv == ref.nkv
    g.sync()
    assert memory(g.L) == before             # nothing allocated by the two calls


def test_static_refuses_a_box_outside_the_kset_window():
    """A box 6 % larger than the one the k-set was built for needs a new
    k-set (device memory): refused, and the k-set is left as it was."""
    s, st = systems.build(systems.spcfw(n=216, ions=0))
    g = ForcePath(s, precision=MDX_FP64)
    g.set_state(*st)
    g.chcnb()
    nkv = g.inifur()
    th = thermo_init(s)
    th.boxl, th.boyl, th.bozl = 1.06 * s.boxl, 1.06 * s.boyl, 1.06 * s.bozl
    th.vol = th.boxl * th.boyl * th.bozl
    g.set_state(*st, thermo=th)
    out = MdxScalars()
    assert g.L.mdx_slforces_static(g.h, C.byref(out)) == MDX_ERR_STATE
    assert "5 %" in g.L.mdx_last_error(g.h).decode()
    th.boxl, th.boyl, th.bozl = s.boxl, s.boyl, s.bozl   # back inside the window
    th.vol = s.boxl * s.boyl * s.bozl
    g.set_state(*st, thermo=th)
    assert g.L.mdx_slforces_static(g.h, C.byref(out)) == 0
    assert out.nkv == nkv


def test_static_refuses_with_timers_on():
    s, st = systems.build(systems.spcfw(n=216, ions=0))
    g = ForcePath(s, precision=MDX_FP64)
    g.set_state(*st)
    g.chcnb()
    g.inifur()
    g.set_timers(True)
    out = MdxScalars()
    assert g.L.mdx_slforces_static(g.h, C.byref(out)) == MDX_ERR_STATE
    assert "timers" in g.L.mdx_last_error(g.h).decode()
    g.set_timers(False)
    assert g.L.mdx_slforces_static(g.h, C.byref(out)) == 0


def test_static_needs_a_kset_first():
    s, st = systems.build(systems.spcfw(n=216, ions=0))
    g = ForcePath(s, precision=MDX_FP64)
    g.set_state(*st)
    g.chcnb()
    out = MdxScalars()
    rc = g.L.mdx_slforces_static(g.h, C.byref(out))
    assert rc == MDX_ERR_STATE
    assert "k-set" in g.L.mdx_last_error(g.h).decode()
    g.inifur()                               # now the k-set exists
    assert g.L.mdx_slforces_static(g.h, C.byref(out)) == 0


def test_static_rejects_scratch_beyond_its_size():
    # 1,536 waters (4,608 atoms, 9 slices of 512) with a k-set of about
    # 40,000 vectors: 9 x 40,000 x 16 B is above the 4 MiB static scratch
    spec = S.RunSpec(molecules=[("SPC-FW", 1536)], density=1.0, dt_fs=2.0, nfreq=1,
                     rcut=9.0, rshort=5.0, alpha=0.35 * 9.0, fexp=40.0, ichnb=10)
    s, st = systems.build(spec)
    g = ForcePath(s, precision=MDX_FP64, nkv_max=200000)
    g.set_state(*st)
    g.chcnb()
    nkv = g.inifur()
    slices = -(-s.nstot // 512)
    assert slices * nkv * 16 > 4 << 20
    out = MdxScalars()
    rc = g.L.mdx_slforces_static(g.h, C.byref(out))
    assert rc == MDX_ERR_UNSUPPORTED
    assert "MDX_SK_STATIC_BYTES" in g.L.mdx_last_error(g.h).decode()
