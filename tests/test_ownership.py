"""Ownership logic of the pair kernel, checked on the CPU.

The library derives, from the reference's 63-entry midpoint table
(SRC/exaMD_module.f90:276-346), 13 x-rows and per-position-class masks that
tell a CTA tile which cell pairs it owns.  Replaying the kernel's enumeration
over every tile of a periodic grid must cover each unordered cell pair with
separation in {-2..2}^3 exactly once, and each pair must be computed by the
tile that contains its home block as the table assigns it.
"""
import itertools

import numpy as np
import pytest


def slot_off(s):
    s -= 1
    return np.array([s % 3 - 1, (s // 3) % 3 - 1, s // 9 - 1])


def pos_class(l, t):
    return 0 if l < 0 else (1 if l == 0 else (2 if l < t - 1 else (3 if l == t - 1 else 4)))


def tiles_1d(gpulib, nb, T, width=1.0, balance=0):
    st = gpulib.tile_split(nb, width, T, balance)  # the library's split of an axis
    return [(int(st[k]), int(st[k + 1] - st[k])) for k in range(len(st) - 1)]


def test_rows_and_table_shape(gpulib, oracle):
    rows, lut = gpulib.own_table()
    assert tuple(rows[12]) == (0, 0)
    assert len({tuple(r) for r in rows}) == 13
    tab = oracle.midpoint_table()
    seps = set()
    for a, b in tab[1:]:
        d = tuple(slot_off(b) - slot_off(a))
        seps.add(d)
        assert tuple(-x for x in d) not in seps or d == (0, 0, 0)
    assert len(seps) == 62
    # every non-self separation lies in one of the 12 full rows or the half self row
    for d in seps:
        assert (d[1], d[2]) in {tuple(r) for r in rows}
    # interior class owns everything
    assert all(lut[2 * 25 + 2 * 5 + 2, r] == 0b11111 for r in range(12))
    assert lut[2 * 25 + 2 * 5 + 2, 12] == 0b11100


@pytest.mark.parametrize("nb,T,width,balance", [
    ((5, 5, 5), (2, 2, 2), (1.0,) * 3, 0), ((7, 8, 9), (2, 3, 4), (1.0,) * 3, 0),
    ((9, 6, 11), (3, 2, 5), (1.0,) * 3, 0), ((6, 7, 5), (6, 7, 5), (1.0,) * 3, 0),
    ((10, 10, 10), (4, 4, 4), (1.0,) * 3, 0),
    # split by width: wide last cells on two axes shorten the tiles that hold them
    ((11, 9, 13), (4, 3, 5), (1.7, 1.2, 1.9), 1), ((7, 8, 9), (3, 3, 3), (1.6, 1.6, 1.6), 1)])
def test_each_cell_pair_owned_once(gpulib, oracle, nb, T, width, balance):
    rows, lut = gpulib.own_table()
    nb = np.array(nb)
    tab = oracle.midpoint_table()
    # home offset of separation d from the table: home = A - slot_a
    home_of = {}
    for a, b in tab[1:]:
        d = tuple(slot_off(b) - slot_off(a))
        home_of[d] = -slot_off(a)
    cover = {}
    ax = [tiles_1d(gpulib, nb[a], T[a], width[a], balance) for a in range(3)]
    tiles = [(x, y, z) for z in ax[2] for y in ax[1] for x in ax[0]]
    lin = lambda c: int(c[0] + nb[0] * (c[1] + nb[1] * c[2]))
    for (x0, tx), (y0, ty), (z0, tz) in tiles:
        org = np.array([x0, y0, z0])
        t = np.array([tx, ty, tz])
        for l in itertools.product(range(-1, tx + 1), range(-1, ty + 1), range(-1, tz + 1)):
            l = np.array(l)
            cls = pos_class(l[0], tx) * 25 + pos_class(l[1], ty) * 5 + pos_class(l[2], tz)
            A = (org + l) % nb
            for r in range(13):
                m = int(lut[cls, r])
                for bit in range(5):
                    if not (m >> bit) & 1:
                        continue
                    d = np.array([bit - 2, rows[r][0], rows[r][1]])
                    if r == 12 and bit == 2:
                        key = ("self", lin(A))
                    else:
                        B = (org + l + d) % nb
                        # home of the pair per the table must be inside this tile
                        h = l + home_of[tuple(d)]
                        assert np.all(h >= 0) and np.all(h < t), (l, d, h)
                        key = ("pair",) + tuple(sorted((lin(A), lin(B))))
                    cover[key] = cover.get(key, 0) + 1
    ncell = int(np.prod(nb))
    assert all(v == 1 for v in cover.values())
    assert sum(1 for k in cover if k[0] == "self") == ncell
    assert sum(1 for k in cover if k[0] == "pair") == 62 * ncell
