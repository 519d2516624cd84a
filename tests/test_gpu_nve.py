"""NVE energy conservation of the mixed path against the FP64 path (DOUBLE,
flexible SPC-FW water), from the same equilibrated state."""
import numpy as np
import pytest

from mdynamix_gb300 import system as S
from mdynamix_gb300.abi import MDX_FP64, MDX_MIXED
from mdynamix_gb300.mdx import ForcePath

pytestmark = pytest.mark.gpu


def _nve(prec, s, state, th, nsteps, mstep0):
    g = ForcePath(s, precision=prec)
    p = g.packed.params
    p.lnvt = 0
    g.set_params(p)
    th.sc = 0.0
    g.set_state(*state, thermo=th)
    rec = g.double(nsteps, mstep0)
    g.close()
    e = np.array([r.pe1 + r.pe2 + r.pels1 + r.pels2 + r.spe + r.pint + r.tke for r in rec])
    ke = np.array([r.tke for r in rec])
    return e, ke


def test_mixed_nve_drift_matches_fp64():
    spec = S.RunSpec(molecules=[("SPC-FW", 216)], density=1.0, dt_fs=2.0, nfreq=10, rcut=8.0,
                     rshort=5.0, alpha=2.8, fexp=12.0, ichnb=10, nvt=(300.0, 30.0))
    s = S.System(spec)
    st = S.make_configuration(s, seed=5, jitter=0.05)
    g = ForcePath(s, precision=MDX_FP64)
    g.set_state(*st)
    g.double(100, records=False)
    state, th = g.get_state()
    g.close()
    nsteps = 300
    t = np.arange(nsteps) * spec.dt_fs * 1e-3
    res = {}
    for name, prec in (("fp64", MDX_FP64), ("mixed", MDX_MIXED)):
        e, ke = _nve(prec, s, state, th, nsteps, 100)
        drift = abs(np.polyfit(t, e, 1)[0]) * t[-1]  # over the run
        res[name] = (drift / ke.std(), e.std() / ke.std())
    for name, (d, r) in res.items():
        assert d < 0.05 and r < 0.05, (name, d, r)
    assert res["mixed"][0] < 2.0 * res["fp64"][0] + 0.01, res
    assert res["mixed"][1] < 1.5 * res["fp64"][1] + 0.005, res
