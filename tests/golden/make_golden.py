"""Regenerate tests/golden/oracle_midpoint_gas.npz.

Input: a seeded uniform gas with minimum separation 0.9 (numpy rejection),
600 atoms in a 14 x 15 x 16 periodic box, rc = 2.5.  Output: the CPU oracle's
forces (restated exaMD_forces_midpoint_all), candidate/accepted counts, and
the extension's energy and virial.  The fixture pins the oracle against
regressions; it is not a reference golden vector (the reference ships none).

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as O  # noqa: E402


def gas(n, L, dmin, seed):
    rng = np.random.default_rng(seed)
    pos = np.zeros((0, 3))
    while len(pos) < n:
        p = rng.uniform(0, 1, 3) * L
        if len(pos):
            d = pos - p
            d -= np.round(d / L) * L
            if (d * d).sum(1).min() < dmin * dmin:
                continue
        pos = np.vstack([pos, p])
    return pos


def main():
    L = np.array([14.0, 15.0, 16.0])
    pos = gas(600, L, 0.9, 20261203)
    f, c = O.forces_midpoint_all(pos, L, 2.5)
    t = O.forces_typed(pos, L, 2.5)
    np.savez(os.path.join(HERE, "oracle_midpoint_gas.npz"), pos=pos, box=L, cutoff=2.5, forces=f,
             candidates=c.candidates, accepted=c.accepted, epot=t["epot"], virial=t["virial"])
    print("wrote", len(pos), "atoms", c.candidates, c.accepted)


if __name__ == "__main__":
    main()
