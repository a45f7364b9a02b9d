"""The reference's particle file, exaMD_particles.dat (SRC/exaMD_input_formats.f90:128-235):
list-directed records natms_tot / globalbox(3) / x y z per atom.  Host code only (no GPU)."""
import numpy as np
import pytest


def test_round_trip_is_exact(gpulib, tmp_path):
    rng = np.random.default_rng(3)
    L = np.array([33.59205, 40.0, 1.0 / 3.0])
    pos = rng.uniform(0, 1, (257, 3)) * L
    pos[0] = [0.0, np.nextafter(L[1], 0), 1e-300]
    p = tmp_path / "exaMD_particles.dat"
    gpulib.write_particles(p, pos, L)
    q, Lq = gpulib.read_particles(p)
    assert np.array_equal(q, pos) and np.array_equal(Lq, L)
    lines = p.read_text().splitlines()
    assert int(lines[0]) == 257 and len(lines) == 2 + 257


def test_reads_fortran_list_directed_text(gpulib, tmp_path):
    """What a Fortran compiler writes and reads: blanks or commas, D exponents,
    repeat counts, items continued onto the next record, the rest of a record skipped."""
    text = ("           4  extra items after the count are skipped\n"
            "   10.000000000000000        1.2D+01,  8.0e0  \n"
            "   1.0000000000000000        2.0000000000000000        3.0000000000000000\n"
            " 0.5D0, 0.25d0, 0.125\n"
            " 3*2.5\n"
            " 9.0\n"
            " 8.5 7.5   skipped\n")
    p = tmp_path / "exaMD_particles.dat"
    p.write_text(text)
    pos, L = gpulib.read_particles(p)
    assert np.array_equal(L, [10.0, 12.0, 8.0])
    assert np.array_equal(pos, [[1, 2, 3], [0.5, 0.25, 0.125], [2.5, 2.5, 2.5], [9.0, 8.5, 7.5]])


@pytest.mark.parametrize("text", ["", "3\n1 2 3\n0 0 0\n1 1 1\n", "x\n1 2 3\n", "1\n1 2 3\n0 0 zz\n",
                                  "2\n1 2\n"])
def test_malformed_files_are_refused(gpulib, tmp_path, text):
    from examd_gb300 import _lib
    p = tmp_path / "exaMD_particles.dat"
    p.write_text(text)
    with pytest.raises(_lib.ExamdError) as e:
        gpulib.read_particles(p)
    assert e.value.code == _lib.ERR_IO


def test_missing_file(gpulib, tmp_path):
    from examd_gb300 import _lib
    with pytest.raises(_lib.ExamdError) as e:
        gpulib.read_particles(tmp_path / "nope.dat")
    assert e.value.code == _lib.ERR_IO
