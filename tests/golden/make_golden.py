"""Regenerate the golden vectors of tests/golden/ from the FP64 oracle.

    python tests/golden/make_golden.py

cavity16_oldroydb_10steps.npz: 16x16 lid-driven cavity, Oldroyd-B-Log,
Wi=0.5, beta=0.5, Re=0.01, dt=1e-3, 10 steps (fields U, p, theta, tau, phi).
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


def main():
    o = Oracle(cavity_case(16))
    o.step(10)
    np.savez_compressed(os.path.join(HERE, "cavity16_oldroydb_10steps.npz"),
                        U=o.f.U, p=o.f.p, theta=o.f.theta, tau=o.f.tau, phi=o.f.phi)


if __name__ == "__main__":
    main()
