"""What the drivers and the file layer do on the host alone.

The jamming drivers' argument handling runs before any device call: invalid numbers
and unreadable data files end the driver with status 1 and a message, and a missing
argument is prompted for and read from standard input, as the reference's drivers do
(src/cuda/main_2point_findjam.cpp:17-58).  Position files are written from host
arrays without a handle, and the configuration maker (src/cuda/main_configmaker.cpp)
runs without a GPU."""
from __future__ import annotations

import os
import subprocess

import pytest

from conftest import ROOT

BIN = os.path.join(ROOT, "spherocyls_gb300", "bin")


def _run(name, args, stdin=subprocess.DEVNULL):
    return subprocess.run([os.path.join(BIN, name)] + [str(a) for a in args], stdin=stdin,
                          capture_output=True, text=True, timeout=60)


@pytest.mark.parametrize("name", ["spherocyl_find_jam", "spherocyl_y_compress"])
def test_zero_resize_step_is_refused(library, tmp_path, name):
    r = _run(name, ["r", tmp_path, 64, 0, 0.01, 1e-6, 0.01, 0.01, 0.1, 0.8, 1.0, 1.4])
    assert r.returncode == 1 and "non-zero resize step" in r.stderr


def test_qs_compress_needs_a_positive_packing(library, tmp_path):
    r = _run("spherocyl_qs_compress", ["r", tmp_path, 64, 5e-3, 0.01, 0, 0.01, 0.01, 0.1])
    assert r.returncode == 1 and "final packing fraction" in r.stderr


@pytest.mark.parametrize("name", ["spherocyl_find_jam", "spherocyl_qs_compress",
                                  "spherocyl_y_compress"])
def test_unreadable_data_file_fails_before_the_device(library, tmp_path, name):
    r = _run(name, [tmp_path / "sd0000000000.dat", tmp_path, 64, 1e-3, 0.01, 0.9, 0.01, 0.01,
                    0.1])
    assert r.returncode != 0 and "read" in (r.stdout + r.stderr)


def test_missing_arguments_are_read_from_stdin(library, tmp_path):
    """Arguments past argv come from standard input, one per line; here the resize step
    (0) arrives that way and is refused, and an exhausted input ends the driver."""
    r = _run("spherocyl_find_jam", ["r", tmp_path, 64])
    assert r.returncode == 1 and "missing input" in r.stderr
    r = subprocess.run([os.path.join(BIN, "spherocyl_find_jam"), "r", str(tmp_path), "64"],
                       input="0\n0.01\n1e-6\n0.01\n0.01\n0.1\n", capture_output=True, text=True,
                       timeout=60)
    assert r.returncode == 1 and "Resize rate (epsilon): " in r.stdout
    assert "non-zero resize step" in r.stderr


@pytest.mark.parametrize("fmt", ["sp", "sd", "bin"])
def test_write_positions_round_trip(library, tmp_path, fmt):
    """Host arrays to a position file and back without a handle: the binary layout
    and the %.17g rows of sd files are exact, sp files carry 14 digits, and sd files
    carry R with two digits as the reference writes it (%.2g)."""
    import numpy as np

    from spherocyls_gb300 import read_positions, write_positions

    rng = np.random.default_rng(5)
    n = 9
    x, y = rng.uniform(0, 7, (2, n))
    p = rng.uniform(-1.5, 1.5, n)
    R = np.where(np.arange(n) % 2, 0.5, 0.7)
    A = R * 1.25
    hdr = dict(Lx=7.0, Ly=7.5 if fmt != "sp" else 7.0, packing=0.8125, gamma=0.125,
               gamma_total=2.5, rate=1e-3, dt=0.02)
    path = str(tmp_path / f"sd0000000003.{'bin' if fmt == 'bin' else 'dat'}")
    write_positions(path, hdr, x, y, p, R, A, fmt=fmt)
    h, xx, yy, pp, RR, AA = read_positions(path)
    tol = 0 if fmt != "sp" else 1e-13
    for a, b in ((xx, x), (yy, y), (pp, p), (AA, A), (RR, R)):
        assert np.allclose(a, b, rtol=tol, atol=0)
    assert h["Lx"] == hdr["Lx"] and h["Ly"] == hdr["Ly"] and h["gamma_total"] == 2.5


def test_configmaker_writes_zero_energy_configurations(library, oracle_built, tmp_path):
    """main_configmaker.cpp's run on the host alone: configuration i in sd%010d.dat,
    each contact-free (zero energy in the oracle's calc_se), angles in [-pi/2, pi/2],
    the seeds giving different configurations."""
    import numpy as np

    from spherocyls_gb300 import read_positions

    r = _run("spherocyl_configmaker", [tmp_path, 64, 3, 0.5, 1.0, 1.4])
    assert r.returncode == 0, r.stderr
    states = []
    for i in range(3):
        h, x, y, p, R, A = read_positions(str(tmp_path / f"sd{i:010d}.dat"))
        assert len(x) == 64 and h["Lx"] == h["Ly"] and h["packing"] == 0.5
        assert h["rate"] == 1e-3 and h["dt"] == 1.0
        assert np.all(p >= -np.pi / 2) and np.all(p <= np.pi / 2)
        ob = oracle_built.OracleBox(h["Lx"], x, y, p, A, R, 0.1)
        ob.calc_se()
        assert ob.se()[0] == 0.0
        states.append(x)
    assert not np.array_equal(states[0], states[1])
