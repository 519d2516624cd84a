"""Small seeded systems shared by the tests (sizes the oracle finishes fast)."""
from mdynamix_gb300 import system as S


def spce_ions(n=128, ions=2, shake=True, toler=1e-8):
    """Rigid SPC/E + Na+/Cl-, SHAKE, NVE (the plain-method case, scaled down)."""
    return S.RunSpec(molecules=[("SPC_E", n), ("Na+", ions), ("Cl-", ions)], density=1.0,
                     dt_fs=2.0, nfreq=1, rcut=7.0, rshort=5.0, alpha=1.96, fexp=9.0,
                     ichnb=5, shake=shake, toler=toler, trtemp=300.0)


def spcfw(n=216, ions=2, rcut=9.0, nvt=True):
    """Flexible SPC-FW water (+ ions), double time step 0.2/2 fs."""
    mols = [("SPC-FW", n)] + ([("Na+", ions), ("Cl-", ions)] if ions else [])
    return S.RunSpec(molecules=mols, density=1.0, dt_fs=2.0, nfreq=10, rcut=rcut,
                     rshort=5.0, alpha=0.28 * rcut, fexp=9.0, ichnb=10,
                     nvt=(300.0, 30.0) if nvt else None, trtemp=300.0)


def organics(nw=100):
    """Morse flexible water (IPOT 2) with methanol and ethanol: angles,
    torsions, 1-4 pairs with scaled Coulomb, special 1-4 LJ."""
    return S.RunSpec(molecules=[("H2O", nw), ("CH3OH", 3), ("C2H5OH", 2)], density=1.0,
                     dt_fs=2.0, nfreq=10, rcut=7.0, rshort=5.0, alpha=2.0, fexp=9.0,
                     ichnb=10, nvt=(298.0, 30.0), trtemp=298.0)


def build(spec, seed=11, jitter=0.05):
    s = S.System(spec)
    st = S.make_configuration(s, seed=seed, jitter=jitter)
    return s, st
