"""Regenerate the golden vectors of tests/golden/ from the FP64 oracle.

    python tests/golden/make_golden.py

cavity16_oldroydb_10steps.npz: 16x16 lid-driven cavity, Oldroyd-B-Log,
Wi=0.5, beta=0.5, Re=0.01, dt=1e-3, 10 steps (fields U, p, theta, tau, phi).
cavity16_fenecr_5steps.npz, cavity16_roliepoly_5steps.npz: the same cavity
with FENE-CR-Log (L2 = 20) and Rolie-Poly-Log (lambdaR 0.2, beta 0.5,
delta -0.5, chiMax 5), Wi=0.5, dt=5e-3, 5 steps.
cavity16_xpompom_5steps.npz, cavity16_whitemetznercy_5steps.npz: the same
cavity with XPomPom-Log (lambdaB = Wi = 0.5, lambdaS 0.2, q 2, alpha 0.15,
n 0) and WhiteMetznerCY-Log (K 1, a 2, n 0.5), dt=5e-3, 5 steps.
periodicchannel_ptt_3steps.npz: 8x8x4 channel periodic in x and z, PTT-Log
(epsilon 0.25), Wi=2, laminar profile and the seeded lognormal conformation
(sigma 0.1, seed 20261203), nInIter 2, 3 steps.
The oracle is compiled with -ffp-contract=off, so x86_64 and aarch64 give the
same bits.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle.pyoracle import Oracle  # noqa: E402
from rheotool_gb300.case import cavity_case  # noqa: E402


def save(name, o):
    np.savez_compressed(os.path.join(HERE, name), U=o.f.U, p=o.f.p, theta=o.f.theta, tau=o.f.tau, phi=o.f.phi)


def golden_cases():
    """(file name, case, initial fields or None, steps) of every golden vector."""
    from rheotool_gb300.case import periodic_channel_case, periodic_channel_state
    from rheotool_gb300.mesh import periodic_channel_mesh
    out = [("cavity16_oldroydb_10steps.npz", cavity_case(16), None, 10),
           ("cavity16_fenecr_5steps.npz", cavity_case(16, model="FENE-CRLog", Wi=0.5, dt=5e-3, L2=20.0), None, 5)]
    rp = cavity_case(16, model="Rolie-PolyLog", Wi=0.5, dt=5e-3, lambdaR=0.2, delta=-0.5, chiMax=5.0)
    rp.model.beta = 0.5
    out.append(("cavity16_roliepoly_5steps.npz", rp, None, 5))
    xp = cavity_case(16, model="XPomPomLog", Wi=0.5, dt=5e-3, lambdaS=0.2, q=2.0, alpha=0.15)
    out.append(("cavity16_xpompom_5steps.npz", xp, None, 5))
    wm = cavity_case(16, model="WhiteMetznerCYLog", Wi=0.5, dt=5e-3, K=1.0, a=2.0)
    wm.model.n = 0.5    # cavity_case's own n is the mesh size
    out.append(("cavity16_whitemetznercy_5steps.npz", wm, None, 5))
    ch = periodic_channel_case(periodic_channel_mesh(8, 8, 4, L=2.0, depth=1.0), Wi=2.0)
    ch.nInIter = 2
    out.append(("periodicchannel_ptt_3steps.npz", ch, periodic_channel_state(ch, 0.1, 20261203), 3))
    return out


def main():
    for name, case, f0, steps in golden_cases():
        o = Oracle(case, None if f0 is None else f0.copy())
        o.step(steps)
        save(name, o)


if __name__ == "__main__":
    main()
