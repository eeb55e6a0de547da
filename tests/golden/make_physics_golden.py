"""Copy the reference's physics curves used as loose pins into a small fixture.

Run once in a container that has the SPECTRAX source tree:

    python tests/golden/make_physics_golden.py <path to the SPECTRAX source tree>

Reads Examples/damping_rate_1836.csv (Landau damping rate against k for
mi/me = 1836, the physics behind the 1D1V Landau workload) and
Examples/growth_rate.csv (two-stream growth rate against k) and writes
physics_curves.npz with their (k, rate) columns.  Nothing on the test path
reads the reference: only this fixture travels.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref_root: str) -> None:
    ex = os.path.join(ref_root, "Examples")
    damp = np.loadtxt(os.path.join(ex, "damping_rate_1836.csv"), delimiter=",")
    grow = np.loadtxt(os.path.join(ex, "growth_rate.csv"), delimiter=",")
    np.savez(os.path.join(HERE, "physics_curves.npz"), damping_k=damp[:, 0], damping_rate=damp[:, 1],
             growth_k=grow[:, 0], growth_rate=grow[:, 1])


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit("usage: make_physics_golden.py <path to the SPECTRAX source tree>")
    main(sys.argv[1])
