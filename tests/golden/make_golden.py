"""Regenerate tests/golden/oracle_midpoint_gas.npz and oracle_typed_mixture.npz.

oracle_midpoint_gas: a seeded uniform gas with minimum separation 0.9 (numpy
rejection), 600 atoms in a 14 x 15 x 16 periodic box, rc = 2.5.  Output: the
CPU oracle's forces (restated exaMD_forces_midpoint_all), candidate/accepted
counts, and the extension's energy and virial.

oracle_typed_mixture: 500 atoms, 80:20 of two types with the
Kob-Andersen-type table of the binary-mixture workload (eps AB 1.5, BB 0.5;
sigma AB 0.8, BB 0.88; rc = 2.5 sigma per type pair), minimum separation
0.75, in a 12 x 12.5 x 13 box.  Output: the oracle's typed forces, energy,
virial, and candidate/accepted counts.

The fixtures pin the oracle against regressions; they are not reference
golden vectors (the reference ships none).

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

    Lm = np.array([12.0, 12.5, 13.0])
    pm = gas(500, Lm, 0.75, 20261204)
    types = (np.random.default_rng(20261205).uniform(0, 1, len(pm)) < 0.2).astype(np.int32)
    eps = np.array([[1.0, 1.5], [1.5, 0.5]])
    sigma = np.array([[1.0, 0.8], [0.8, 0.88]])
    rc = 2.5 * sigma
    t = O.forces_typed(pm, Lm, rc, eps, sigma, types, 2)
    np.savez(os.path.join(HERE, "oracle_typed_mixture.npz"), pos=pm, box=Lm, types=types, eps=eps, sigma=sigma,
             rc=rc, forces=t["forces"], epot=t["epot"], virial=t["virial"], candidates=t["counts"].candidates,
             accepted=t["counts"].accepted)
    print("wrote", len(pm), "atoms of 2 types", t["counts"].candidates, t["counts"].accepted)


if __name__ == "__main__":
    main()
